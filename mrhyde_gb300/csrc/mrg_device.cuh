// Device helpers shared by the Krylov solvers and the multigrid levels: structured row layout, row
// products, the per-warp bulk-staged row loop, deterministic block reductions with the "last block sums
// the partials" pattern.
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

__device__ __forceinline__ int64_t row_ptr_of(const Grid& g, int64_t n, int64_t nrows) {
  if (n >= nrows) return g.T[0] * g.T[1] * g.T[2];
  int ix, iy, iz;
  decompose(g, n, ix, iy, iz);
  int lo, cx, cy, cz;
  axis_range(ix, g.nn[0], g.p, lo, cx);
  axis_range(iy, g.nn[1], g.p, lo, cy);
  if (g.dim == 3) axis_range(iz, g.nn[2], g.p, lo, cz); else cz = 1;
  return g.P[2][iz] * g.T[1] * g.T[0] + (int64_t)cz * (g.P[1][iy] * g.T[0] + (int64_t)cy * g.P[0][ix]);
}

// Copy (or add) a contiguous segment from shared memory to global memory.  src[k] <-> dst[k]; both
// pointers have the same address phase modulo 16 bytes, so the body uses aligned 16-byte accesses.
template <typename T, bool ADD>
__device__ __forceinline__ void seg_store(T* __restrict__ dst, const T* __restrict__ src, int64_t len) {
  constexpr int V = 16 / sizeof(T);
  int head = (int)(((16 - ((uintptr_t)dst & 15)) & 15) / sizeof(T));
  if (head > len) head = (int)len;
  for (int k = threadIdx.x; k < head; k += blockDim.x) {
    if (ADD) dst[k] += src[k]; else dst[k] = src[k];
  }
  int64_t body = (len - head) / V;
  if constexpr (sizeof(T) == 8) {
    const double2* s2 = reinterpret_cast<const double2*>(src + head);
    double2* d2 = reinterpret_cast<double2*>(dst + head);
    for (int64_t v = threadIdx.x; v < body; v += blockDim.x) {
      double2 x = s2[v];
      if (ADD) { double2 y = d2[v]; x.x += y.x; x.y += y.y; d2[v] = x; } else __stcs(d2 + v, x);
    }
  } else {
    const float4* s4 = reinterpret_cast<const float4*>(src + head);
    float4* d4 = reinterpret_cast<float4*>(dst + head);
    for (int64_t v = threadIdx.x; v < body; v += blockDim.x) {
      float4 x = s4[v];
      if (ADD) { float4 y = d4[v]; x.x += y.x; x.y += y.y; x.z += y.z; x.w += y.w; d4[v] = x; } else __stcs(d4 + v, x);
    }
  }
  for (int64_t k = head + body * V + threadIdx.x; k < len; k += blockDim.x) {
    if (ADD) dst[k] += src[k]; else dst[k] = src[k];
  }
}

// Make this thread's shared-memory writes visible to the bulk-copy (async) proxy; every writing thread
// executes it before the barrier that precedes seg_store_bulk.
__device__ __forceinline__ void fence_to_bulk() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Copy a contiguous segment from shared to global memory (overwrite): the 16-byte aligned body with one
// bulk copy through the copy engine, the ragged ends (at most one 16-byte unit each) with plain stores.
// src[k] <-> dst[k] share the address phase modulo 16 bytes.  Called by every thread of the CTA after
// fence_to_bulk and a CTA barrier; thread 0 issues the copy and waits until it has read the shared
// memory, which must outlive the read (the wait ends as the copy proceeds: it depends on no other CTA).
template <typename T>
__device__ __forceinline__ void seg_store_bulk(T* __restrict__ dst, const T* __restrict__ src, int64_t len) {
  constexpr int V = 16 / sizeof(T);
  int head = (int)(((16 - ((uintptr_t)dst & 15)) & 15) / sizeof(T));
  if (head > len) head = (int)len;
  const int64_t body = (len - head) / V;
  for (int k = threadIdx.x; k < head; k += blockDim.x) dst[k] = src[k];
  for (int64_t k = head + body * V + threadIdx.x; k < len; k += blockDim.x) dst[k] = src[k];
  if (threadIdx.x == 0 && body > 0) {
    const uint32_t saddr = (uint32_t)__cvta_generic_to_shared(src + head);
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst + head), "r"(saddr),
                 "r"((uint32_t)(body * 16))
                 : "memory");
    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
    asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
  }
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

// CSR row start of row n (nnz for n = nrows); PC > 0: compile-time polynomial order
template <int PC = 0>
__device__ __forceinline__ int64_t row_ptr_at(const Grid& g, int64_t n, int64_t nrows) {
  if (n >= nrows) return g.T[0] * g.T[1] * g.T[2];
  int ix, iy, iz;
  decompose(g, n, ix, iy, iz);
  return row_info<PC>(g, ix, iy, iz).rp;
}

// ---- row products: y_i = sum_j J_ij x_j over the row of node i --------------------------------
template <int P, typename JT, typename XT>
__device__ __forceinline__ double row_apply(const Grid& g, const RowInfo& R, const JT* __restrict__ vals,
                                            const XT* __restrict__ x) {
  constexpr int MC = 2 * P + 1;
  const int64_t NX = g.nn[0], plane = (int64_t)g.nn[0] * g.nn[1];
  if (P == 1 && R.cx == 3 && R.cy == 3 && R.cz == 3) {
    // interior row: all 27 couplings, no predicates, so all loads issue before the FMAs
    const XT* xb = x + R.lx + NX * R.ly + plane * R.lz;
    double xv[27];
#pragma unroll
    for (int k = 0; k < 27; ++k) xv[k] = (double)__ldg(xb + (k % 3) + NX * ((k / 3) % 3) + plane * (k / 9));
    double acc = 0.0;
#pragma unroll
    for (int k = 0; k < 27; ++k) acc = fma((double)vals[k], xv[k], acc);
    return acc;
  }
  double acc = 0.0;
  int pos = 0;
#pragma unroll
  for (int z = 0; z < (P == 1 ? 3 : MC); ++z) {
    if (z < R.cz) {
#pragma unroll
      for (int y = 0; y < MC; ++y) {
        if (y < R.cy) {
          const int64_t base = (R.lx) + NX * (R.ly + y) + plane * (R.lz + z);
#pragma unroll
          for (int xo = 0; xo < MC; ++xo)
            if (xo < R.cx) {
              acc = fma((double)vals[pos], (double)__ldg(x + base + xo), acc);
              ++pos;
            }
        }
      }
    }
  }
  return acc;
}

// FP32 variant accumulating in FP32 (inner solve of the mixed path)
template <int P>
__device__ __forceinline__ float row_apply_f(const Grid& g, const RowInfo& R, const float* __restrict__ vals,
                                             const float* __restrict__ x) {
  constexpr int MC = 2 * P + 1;
  const int64_t NX = g.nn[0], plane = (int64_t)g.nn[0] * g.nn[1];
  if (P == 1 && R.cx == 3 && R.cy == 3 && R.cz == 3) {
    const float* xb = x + R.lx + NX * R.ly + plane * R.lz;
    float xv[27];
#pragma unroll
    for (int k = 0; k < 27; ++k) xv[k] = __ldg(xb + (k % 3) + NX * ((k / 3) % 3) + plane * (k / 9));
    float acc = 0.0f;
#pragma unroll
    for (int k = 0; k < 27; ++k) acc = fmaf(vals[k], xv[k], acc);
    return acc;
  }
  float acc = 0.0f;
  int pos = 0;
#pragma unroll
  for (int z = 0; z < MC; ++z) {
    if (z < R.cz) {
#pragma unroll
      for (int y = 0; y < MC; ++y) {
        if (y < R.cy) {
          const int64_t base = (R.lx) + NX * (R.ly + y) + plane * (R.lz + z);
#pragma unroll
          for (int xo = 0; xo < MC; ++xo)
            if (xo < R.cx) {
              acc = fmaf(vals[pos], __ldg(x + base + xo), acc);
              ++pos;
            }
        }
      }
    }
  }
  return acc;
}

constexpr int WST = 128;  // threads per CTA of the kernels that use the per-warp staged row loop

// ---- per-warp staged rows (P = 1) --------------------------------------------------------------
// A warp owns tiles of 32 consecutive rows.  Their CSR values form one contiguous segment, which lane 0
// copies into the warp's own shared buffer with a 1-D bulk copy (cp.async.bulk, completion counted on
// the warp's mbarrier) while the warp multiplies its previous tile; the unaligned ends of the segment
// are copied with plain loads.  No CTA-wide barrier is involved, so warps never wait for each other.
constexpr int WROWS = 32;
template <typename JT>
__host__ __device__ constexpr int wbuf_elems() { return WROWS * 27 + 2 * (16 / (int)sizeof(JT)); }
template <typename JT>
constexpr int wspmv_smem() { return (WST / 32) * 2 * wbuf_elems<JT>() * (int)sizeof(JT); }

constexpr unsigned long long WAIT_NS = 1000000000ull;  // default bound on one tile's copy: 1 s

__device__ __forceinline__ bool wbar_try(uint32_t mbar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(mbar), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ uint64_t wtimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
  return t;
}

// bounded wait by every lane of the warp (limit in ns); the result is warp-uniform
__device__ __forceinline__ bool wbar_wait(uint32_t mbar, uint32_t parity, unsigned long long limit) {
  int ok = 1;
  if (!wbar_try(mbar, parity)) {
    const uint64_t t0 = wtimer();
    while (!wbar_try(mbar, parity))
      if (wtimer() - t0 > limit) { ok = 0; break; }
  }
  return __all_sync(0xffffffffu, ok) != 0;
}

// Issues the copy of warp tile `tile` into buf; returns the global byte address mapped to buf[0].  R is
// the set-up of the lane's row of the tile (kept until the tile is processed); the tile's CSR segment runs
// from lane 0's row start to the end of its last row.
template <typename JT>
__device__ __forceinline__ uintptr_t wtile_issue(const Grid& g, int64_t nrows, const JT* __restrict__ J, int64_t tile,
                                                 JT* buf, uint32_t mbar, int lane, RowInfo& R) {
  const int64_t n0 = tile * WROWS;
  const int64_t n1 = (n0 + WROWS < nrows) ? n0 + WROWS : nrows;
  const int64_t nnz = g.T[0] * g.T[1] * g.T[2];
  int64_t rend = 0;
  R = RowInfo{0, 0, 0, 1, 1, 1, 0};
  if (n0 + lane < nrows) {
    int ix, iy, iz;
    decompose(g, n0 + lane, ix, iy, iz);
    R = row_info<1>(g, ix, iy, iz);
    rend = R.rp + (int64_t)R.cx * R.cy * R.cz;
  }
  const int64_t seg0 = __shfl_sync(0xffffffffu, R.rp, 0);
  const int64_t seg1 = __shfl_sync(0xffffffffu, rend, (int)(n1 - n0) - 1);
  const uintptr_t lo = (uintptr_t)(J + seg0), hi = (uintptr_t)(J + seg1);
  const uintptr_t base = lo & ~(uintptr_t)15;
  const uintptr_t jb = ((uintptr_t)J + 15) & ~(uintptr_t)15, je = (uintptr_t)(J + nnz) & ~(uintptr_t)15;
  uintptr_t b0 = base < jb ? jb : base;
  uintptr_t b1 = (hi + 15) & ~(uintptr_t)15;
  if (b1 > je) b1 = je;
  if (b0 > hi) b0 = hi;
  if (b1 < b0) b1 = b0;
  unsigned char* sb = reinterpret_cast<unsigned char*>(buf);
  // plain loads: head [lo, b0) and tail [max(b1, lo), hi) -- a few elements at most
  constexpr int E = (int)sizeof(JT);
  const int nhead = (int)((b0 - lo) / E);
  const uintptr_t t0 = b1 > lo ? b1 : lo;
  const int ntail = (int)((hi - t0) / E);
  if (lane < nhead) *reinterpret_cast<JT*>(sb + (lo - base) + lane * E) = __ldcs(reinterpret_cast<const JT*>(lo) + lane);
  if (lane >= 8 && lane - 8 < ntail)
    *reinterpret_cast<JT*>(sb + (t0 - base) + (lane - 8) * E) = __ldcs(reinterpret_cast<const JT*>(t0) + (lane - 8));
  // g.withhold (testing): the copy of tile 0 is never issued, so the wait for it runs out
  if (lane == 0 && !(g.withhold && tile == 0)) {
    const uint32_t bytes = (uint32_t)(b1 - b0);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(mbar), "r"(bytes) : "memory");
    if (bytes)
      asm volatile(
          "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
              (uint32_t)__cvta_generic_to_shared(sb + (b0 - base))),
          "l"(b0), "r"(bytes), "r"(mbar)
          : "memory");
  }
  return base;
}

// Runs f(n, R, vals) for every row n (vals = the row's values in shared memory), warp-tiled and
// double-buffered.  Returns false if a copy did not complete within the time bound.
template <typename JT, typename F>
__device__ __forceinline__ bool warp_staged_rows(const Grid& g, int64_t nrows, const JT* __restrict__ J,
                                                 unsigned char* smem_raw, uint64_t* mbar_base, F&& f) {
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  JT* const buf0 = reinterpret_cast<JT*>(smem_raw) + (2 * w) * wbuf_elems<JT>();
  JT* const buf1 = buf0 + wbuf_elems<JT>();
  const uint32_t mb0 = (uint32_t)__cvta_generic_to_shared(mbar_base + 2 * w), mb1 = mb0 + 8u;
  if (lane == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(mb0) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(mb1) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  __syncwarp();
  const int64_t ntiles = (nrows + WROWS - 1) / WROWS;
  const int64_t W = (int64_t)gridDim.x * (WST / 32);
  const unsigned long long limit = g.wait_ns ? g.wait_ns : WAIT_NS;
  int64_t tile = (int64_t)blockIdx.x * (WST / 32) + w;
  // buffer b of the current tile; the other buffer receives the next tile
  uintptr_t base0 = 0, base1 = 0;
  uint32_t ph0 = 0u, ph1 = 0u;
  bool armed0 = false, armed1 = false, ok = true;
  int b = 0;
  RowInfo Rc, Rn;  // the lane's row of the current tile / of the next tile
  if (tile < ntiles) {
    base0 = wtile_issue<JT>(g, nrows, J, tile, buf0, mb0, lane, Rc);
    armed0 = true;
  }
  for (; tile < ntiles; tile += W) {
    const int64_t nxt = tile + W;
    if (nxt < ntiles) {
      if (b == 0) { base1 = wtile_issue<JT>(g, nrows, J, nxt, buf1, mb1, lane, Rn); armed1 = true; }
      else        { base0 = wtile_issue<JT>(g, nrows, J, nxt, buf0, mb0, lane, Rn); armed0 = true; }
    }
    const bool got = (b == 0) ? wbar_wait(mb0, ph0, limit) : wbar_wait(mb1, ph1, limit);
    if (!got) { ok = false; break; }
    if (b == 0) { ph0 ^= 1u; armed0 = false; } else { ph1 ^= 1u; armed1 = false; }
    __syncwarp();
    const int64_t n = tile * WROWS + lane;
    if (n < nrows) {
      const unsigned char* cb = reinterpret_cast<const unsigned char*>(b == 0 ? buf0 : buf1);
      const JT* vals = reinterpret_cast<const JT*>(cb + ((uintptr_t)(J + Rc.rp) - (b == 0 ? base0 : base1)));
      f(n, Rc, vals);
    }
    __syncwarp();
    Rc = Rn;
    b ^= 1;
  }
  if (!ok) {  // let copies still in flight land before the CTA exits (bounded)
    if (armed0) wbar_wait(mb0, ph0, limit);
    if (armed1) wbar_wait(mb1, ph1, limit);
  }
  return ok;
}

__device__ __forceinline__ double block_max(double v) {
  __shared__ double sh[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s = fmax(s, sh[i]);
  __syncthreads();
  return s;
}

}  // namespace mrgdev
