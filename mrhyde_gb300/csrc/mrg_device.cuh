// Device helpers shared by the Krylov solvers: structured row layout, row products, deterministic
// block reductions with the "last block sums the partials" pattern.
#pragma once

#include "mrg_internal.h"

namespace mrgdev {

__device__ __forceinline__ void decompose(const Grid& g, int64_t n, int& ix, int& iy, int& iz) {
  // 32-bit arithmetic: n_dofs <= INT32_MAX is enforced by mrg_problem_create
  const unsigned un = (unsigned)n, nx = (unsigned)g.nn[0], ny = (unsigned)g.nn[1];
  const unsigned t = un / nx;
  ix = (int)(un - t * nx);
  iy = (int)(t % ny);
  iz = (int)(t / ny);
}

struct RowInfo {
  int lx, ly, lz, cx, cy, cz;
  int64_t rp;
};

// PC > 0: the polynomial order is a compile-time constant (the axis divisions fold away)
template <int PC = 0>
__device__ __forceinline__ RowInfo row_info(const Grid& g, int ix, int iy, int iz) {
  RowInfo R;
  const int p = PC > 0 ? PC : g.p;
  axis_range(ix, g.nn[0], p, R.lx, R.cx);
  axis_range(iy, g.nn[1], p, R.ly, R.cy);
  if (g.dim == 3) axis_range(iz, g.nn[2], p, R.lz, R.cz); else { R.lz = 0; R.cz = 1; }
  R.rp = g.P[2][iz] * g.T[1] * g.T[0] + (int64_t)R.cz * (g.P[1][iy] * g.T[0] + (int64_t)R.cy * g.P[0][ix]);
  return R;
}

__device__ __forceinline__ int64_t diag_pos(const RowInfo& R, int ix, int iy, int iz) {
  return R.rp + ((int64_t)(iz - R.lz) * R.cy + (iy - R.ly)) * R.cx + (ix - R.lx);
}

// y_i = sum_j J_ij x_j over the row (values contiguous at vals), accumulated in AT
template <int P, typename JT, typename XT, typename AT>
__device__ __forceinline__ AT row_dot(const Grid& g, const RowInfo& R, const JT* __restrict__ vals,
                                      const XT* __restrict__ x) {
  constexpr int MC = 2 * P + 1;
  const int64_t NX = g.nn[0], plane = (int64_t)g.nn[0] * g.nn[1];
  if (P == 1 && R.cx == 3 && R.cy == 3 && R.cz == 3) {
    const XT* xb = x + R.lx + NX * R.ly + plane * R.lz;
    AT xv[27];
#pragma unroll
    for (int k = 0; k < 27; ++k) xv[k] = (AT)__ldg(xb + (k % 3) + NX * ((k / 3) % 3) + plane * (k / 9));
    AT acc = AT(0);
#pragma unroll
    for (int k = 0; k < 27; ++k) acc = fma((AT)vals[k], xv[k], acc);
    return acc;
  }
  AT acc = AT(0);
  int pos = 0;
#pragma unroll
  for (int z = 0; z < MC; ++z) {
    if (z < R.cz) {
#pragma unroll
      for (int y = 0; y < MC; ++y) {
        if (y < R.cy) {
          const int64_t base = R.lx + NX * (R.ly + y) + plane * (R.lz + z);
#pragma unroll
          for (int xo = 0; xo < MC; ++xo)
            if (xo < R.cx) {
              acc = fma((AT)vals[pos], (AT)__ldg(x + base + xo), acc);
              ++pos;
            }
        }
      }
    }
  }
  return acc;
}

// sum over the block; result valid in thread 0
__device__ __forceinline__ double block_sum(double v) {
  __shared__ double sh[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += sh[i];
  __syncthreads();
  return s;
}

// Each block publishes K partials; the block that arrives last (counter) returns true.
template <int K>
__device__ __forceinline__ bool last_block(double* parts, const double (&mine)[K], unsigned int* counter) {
  __shared__ bool amlast;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) parts[(size_t)k * gridDim.x + blockIdx.x] = mine[k];
    __threadfence();
    const unsigned int prev = atomicAdd(counter, 1u);
    amlast = (prev == gridDim.x - 1);
  }
  __syncthreads();
  return amlast;
}

// Sums the partials in a fixed order (deterministic); resets the counter.  Results valid in thread 0.
template <int K>
__device__ __forceinline__ void sum_parts(const double* parts, double (&out)[K], unsigned int* counter) {
  for (int k = 0; k < K; ++k) {
    const double* pk = parts + (size_t)k * gridDim.x;
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    unsigned int i = threadIdx.x;
    const unsigned int st = blockDim.x;
    for (; i + 3 * st < gridDim.x; i += 4 * st) {
      s0 += __ldcg(pk + i);
      s1 += __ldcg(pk + i + st);
      s2 += __ldcg(pk + i + 2 * st);
      s3 += __ldcg(pk + i + 3 * st);
    }
    for (; i < gridDim.x; i += st) s0 += __ldcg(pk + i);
    out[k] = block_sum((s0 + s1) + (s2 + s3));
  }
  if (threadIdx.x == 0) *counter = 0u;
}

}  // namespace mrgdev
