// Batched multiscale-subgrid solves (configuration C4): thousands of independent steady-thermal Q1
// hexahedral problems of uneven size, assembled and solved in one persistent launch.
//
// Reference: the multiscale manager solves each macro element's local problem one at a time on the
// host (src/managers/multiscale/multiscaleManager.cpp:866 -> src/subgrid/subgridDtN.cpp:985 ->
// src/subgrid/subgridDtN_solver.cpp:136, assembly :681, nonlinear solve :903), each with its own
// workset assembly and linear solve.  Here one CTA owns one local problem at a time, taken from an
// atomic work queue ordered largest-first; everything a problem needs happens inside that CTA:
//
//   1. u = Dirichlet data on the boundary, 0 inside (setDirichlet);
//   2. FP32 Jacobian of the problem written to its canonical CSR (factored form kappa_c * K_ref of
//      identical box cells, consistent diagonal), Jacobi diagonal kept in registers;
//   3. FP64 residual r = b - A(u) (matrix-free factored form, FP64 kappa);
//   4. refinement loop: FP32 Jacobi-PCG on J32 d = r to the inner tolerance, u += d (FP64),
//      FP64 residual again, until ||r||_inf / ||r_0||_inf <= tol (the reference's Newton test).
//
// Each thread owns a fixed set of rows and keeps their x, r, z and 1/diag in registers; only the
// search direction p lives in shared memory (the SpMV needs neighbours).  Reductions are block
// reductions in a fixed order, so a problem's result does not depend on which CTA ran it or on what
// else was running: the same bits alone or in the mix.  No grid-wide synchronisation, no spinning.
#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

#include "mrg_internal.h"

struct BatchProb {
  int nx, ny, nz, pad;
  int64_t cell_off, node_off, nnz_off;
  double Kp[8];
  float Kp32[8];
  double load;  // f * vol / 8
};

struct mrg_batch {
  int nprob = 0;
  int64_t ncell = 0, nnode = 0, nnz = 0;
  int max_nodes = 0;
  BatchProb* d_probs = nullptr;
  int32_t* d_order = nullptr;
  double* d_kappa = nullptr;
  float* d_kappa32 = nullptr;
  double* d_g = nullptr;
  int* d_counter = nullptr;
  mrg_batch_stat* d_stats = nullptr;
  std::vector<BatchProb> probs;
  // tuned launch configuration
  int threads = 256;
  int ctas_per_sm = 2;
  double f = 1.0;
  cudaGraphExec_t graph = nullptr;
  const void* graph_key[4] = {nullptr, nullptr, nullptr, nullptr};
  int graph_threads = 0, graph_ctas = 0;
  cudaStream_t graph_stream = nullptr;
  double graph_tol[2] = {0, 0};
  int graph_iters[2] = {0, 0};
};

namespace {

struct BatchArgs {
  const BatchProb* probs;
  const int32_t* order;
  int nprob;
  const double* kappa;
  const float* kappa32;
  const double* g;
  double* u;
  float* J;
  int* counter;
  mrg_batch_stat* stats;
  double tol, inner_tol;
  int max_outer, max_inner;
  int max_nodes;  // nodes of the largest problem: length of each shared-memory array
};

// Block sums of FP32 per-thread partials (the inner solve is FP32): warp tree, one partial per warp in
// shared memory, one barrier, then every thread adds the warp partials in the same fixed order (same
// value everywhere, independent of scheduling).  The partial buffers alternate between two halves, so a
// reduction never overwrites partials that a slower thread may still be reading from the previous one:
// between a write to a half and the previous reads of that half lies the barrier of the reduction in
// between.
template <int T>
__device__ __forceinline__ float2 bsum2(float a, float b, float* red, int& half) {
  constexpr int NW = T / 32;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
  }
  float* buf = red + half * (2 * NW);
  if ((threadIdx.x & 31) == 0) {
    buf[threadIdx.x >> 5] = a;
    buf[NW + (threadIdx.x >> 5)] = b;
  }
  __syncthreads();
  float sa = 0.0f, sb = 0.0f;
#pragma unroll
  for (int w = 0; w < NW; ++w) {
    sa += buf[w];
    sb += buf[NW + w];
  }
  half ^= 1;
  return make_float2(sa, sb);
}

template <int T>
__device__ __forceinline__ double bmax(double v, double* sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < T / 32; ++i) s = fmax(s, sh[i]);
  return s;
}

__device__ __forceinline__ int axis_count(int i, int N) { return (i == 0 || i == N - 1) ? 2 : 3; }
__device__ __forceinline__ int64_t axis_prefix(int i, int N) { return i == 0 ? 0 : (i >= N ? 3LL * N - 2 : 3LL * i - 1); }

__device__ __forceinline__ void nstep_add(float& sum, float& comp, float v) {
  const float t = sum + v;
  comp += (fabsf(sum) >= fabsf(v)) ? (sum - t) + v : (v - t) + sum;
  sum = t;
}

// R = max rows per thread.  Registers hold only the residual r and the SpMV result q of the thread's
// rows; the correction x, the Jacobi inverse, the CSR row offsets and the search direction p live in
// shared memory (4 floats per node of the largest problem), which leaves room for several CTAs per SM.
template <int T, int R>
__global__ void __launch_bounds__(T) k_batch(const BatchArgs A) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float* p_sh = reinterpret_cast<float*>(smem_raw);
  float* x_sh = p_sh + A.max_nodes;
  float* mi_sh = x_sh + A.max_nodes;
  int* rp_sh = reinterpret_cast<int*>(mi_sh + A.max_nodes);
  __shared__ float red[2 * 2 * (T / 32)];
  __shared__ double redd[T / 32];
  __shared__ int s_idx;
  int half = 0;
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) s_idx = atomicAdd(A.counter, 1);
    __syncthreads();
    const int idx = s_idx;
    if (idx >= A.nprob) break;
    const int pid = A.order[idx];
    const BatchProb P = A.probs[pid];
    const int NX = P.nx + 1, NY = P.ny + 1, NZ = P.nz + 1;
    const int nn = NX * NY * NZ;
    const double* kap = A.kappa + P.cell_off;
    const float* kap32 = A.kappa32 + P.cell_off;
    double* u = A.u + P.node_off;
    float* J = A.J + P.nnz_off;
    const double* gv = A.g + P.node_off;
    const int64_t Tx = 3LL * NX - 2, Ty = 3LL * NY - 2;
    // rows of this thread: i = threadIdx.x + k T for k < kn
    const int kn = nn > (int)threadIdx.x ? (nn - (int)threadIdx.x + T - 1) / T : 0;
    // ---- 1. Dirichlet data; 2. FP32 Jacobian (+ Jacobi inverse); p = 0 ----
    unsigned interior = 0u;  // bit k: row k of this thread is a free (interior) row
#pragma unroll
    for (int k = 0; k < R; ++k) {
      if (k >= kn) break;
      const int i = threadIdx.x + k * T;
      const int ix = i % NX, iy = (i / NX) % NY, iz = i / (NX * NY);
      const bool inside = ix > 0 && ix < NX - 1 && iy > 0 && iy < NY - 1 && iz > 0 && iz < NZ - 1;
      interior |= (inside ? 1u : 0u) << k;
      u[i] = inside ? 0.0 : gv[i];
      p_sh[i] = 0.0f;
      const int cxn = axis_count(ix, NX), cyn = axis_count(iy, NY), czn = axis_count(iz, NZ);
      const int64_t rp = axis_prefix(iz, NZ) * Ty * Tx + (int64_t)czn * (axis_prefix(iy, NY) * Tx + (int64_t)cyn * axis_prefix(ix, NX));
      rp_sh[i] = (int)rp;
      mi_sh[i] = 0.0f;
      if (!inside) {
        // Dirichlet row: identity (never scattered, J(d,d) = 1)
        const int lx = ix > 0 ? ix - 1 : 0, ly = iy > 0 ? iy - 1 : 0, lz = iz > 0 ? iz - 1 : 0;
        const int len = cxn * cyn * czn;
        const int dpos = ((iz - lz) * cyn + (iy - ly)) * cxn + (ix - lx);
        for (int e = 0; e < len; ++e) J[rp + e] = (e == dpos) ? 1.0f : 0.0f;
        continue;
      }
      float k32[2][2][2];
#pragma unroll
      for (int c = 0; c < 2; ++c)
#pragma unroll
        for (int b = 0; b < 2; ++b)
#pragma unroll
          for (int a = 0; a < 2; ++a)
            k32[c][b][a] = kap32[(ix - 1 + a) + P.nx * ((iy - 1 + b) + P.ny * (iz - 1 + c))];
      float osum = 0.0f, ocomp = 0.0f;
#pragma unroll
      for (int dz = -1; dz <= 1; ++dz)
#pragma unroll
        for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
          for (int dx = -1; dx <= 1; ++dx) {
            float s = 0.0f;
#pragma unroll
            for (int c = 0; c < 2; ++c)
#pragma unroll
              for (int b = 0; b < 2; ++b)
#pragma unroll
                for (int a = 0; a < 2; ++a) {
                  const bool incl = (dx == 0 || dx == 2 * a - 1) && (dy == 0 || dy == 2 * b - 1) && (dz == 0 || dz == 2 * c - 1);
                  if (incl) s += k32[c][b][a];
                }
            const int cls = (dx != 0) + 2 * (dy != 0) + 4 * (dz != 0);
            const int pos = (dz + 1) * 9 + (dy + 1) * 3 + (dx + 1);
            if (cls != 0) {
              const float v = P.Kp32[cls] * s;
              J[rp + pos] = v;
              nstep_add(osum, ocomp, v);
            }
          }
      const float dg = -(osum + ocomp);
      J[rp + 13] = dg;
      mi_sh[i] = 1.0f / dg;
    }
    __syncthreads();
    // ---- 3./4. refinement loop ----
    double r0 = 0.0, rnorm = 0.0;
    int outer = 0, inner_tot = 0, status = MRG_OK;
    for (;;) {
      // FP64 residual at u (matrix-free factored form): per offset class c, t_c = sum S(off) u(i+off),
      // then r = b - sum_c K_c t_c (35 FP64 FMAs a row instead of 54 multiplies and FMAs)
      float r[R];
      double amax = 0.0;
#pragma unroll
      for (int k = 0; k < R; ++k) r[k] = 0.0f;
#pragma unroll
      for (int k = 0; k < R; ++k) {
        if (k >= kn) break;
        if (!((interior >> k) & 1u)) continue;
        const int i = threadIdx.x + k * T;
        const int ix = i % NX, iy = (i / NX) % NY, iz = i / (NX * NY);
        double kk[2][2][2];
#pragma unroll
        for (int c = 0; c < 2; ++c)
#pragma unroll
          for (int b = 0; b < 2; ++b)
#pragma unroll
            for (int a = 0; a < 2; ++a)
              kk[c][b][a] = kap[(ix - 1 + a) + P.nx * ((iy - 1 + b) + P.ny * (iz - 1 + c))];
        double sx[2][2][3], sxy[2][3][3];
#pragma unroll
        for (int c = 0; c < 2; ++c)
#pragma unroll
          for (int b = 0; b < 2; ++b) {
            sx[c][b][0] = kk[c][b][0];
            sx[c][b][1] = kk[c][b][0] + kk[c][b][1];
            sx[c][b][2] = kk[c][b][1];
          }
#pragma unroll
        for (int c = 0; c < 2; ++c)
#pragma unroll
          for (int x = 0; x < 3; ++x) {
            sxy[c][0][x] = sx[c][0][x];
            sxy[c][1][x] = sx[c][0][x] + sx[c][1][x];
            sxy[c][2][x] = sx[c][1][x];
          }
        double t[8];
#pragma unroll
        for (int c = 0; c < 8; ++c) t[c] = 0.0;
#pragma unroll
        for (int dz = 0; dz < 3; ++dz)
#pragma unroll
          for (int dy = 0; dy < 3; ++dy)
#pragma unroll
            for (int dx = 0; dx < 3; ++dx) {
              const double s = (dz == 0) ? sxy[0][dy][dx] : (dz == 2 ? sxy[1][dy][dx] : sxy[0][dy][dx] + sxy[1][dy][dx]);
              const int cls = (dx != 1) + 2 * (dy != 1) + 4 * (dz != 1);
              t[cls] = fma(s, u[i + (dx - 1) + NX * ((dy - 1) + NY * (dz - 1))], t[cls]);
            }
        double acc = P.load * 8.0;
#pragma unroll
        for (int c = 0; c < 8; ++c) acc = fma(-P.Kp[c], t[c], acc);
        r[k] = (float)acc;  // scaled below, once the max is known
        amax = fmax(amax, fabs(acc));
      }
      rnorm = bmax<T>(amax, redd);
      if (outer == 0) r0 = rnorm;
      if (!isfinite(rnorm)) { status = MRG_ENUMERIC; break; }
      if (rnorm == 0.0 || rnorm <= A.tol * r0 || outer >= A.max_outer) break;
      // FP32 Jacobi PCG on J32 d = r / ||r||_inf (x0 = 0): the scaled residual is O(1), so FP32 squares and
      // dot products stay far from the FP32 range limits whatever the refinement level (r itself is held
      // in FP32 from here on, as the inner solve is)
      const float sc = (float)(1.0 / rnorm);
      float rrf = 0.0f, rzf = 0.0f;
#pragma unroll
      for (int k = 0; k < R; ++k) {
        if (k >= kn) break;
        const int i = threadIdx.x + k * T;
        r[k] *= sc;
        const float z = r[k] * mi_sh[i];
        x_sh[i] = 0.0f;
        p_sh[i] = z;
        rrf = fmaf(r[k], r[k], rrf);
        rzf = fmaf(r[k], z, rzf);
      }
      float2 d2 = bsum2<T>(rrf, rzf, red, half);
      float rr = d2.x, rho = d2.y;
      const float stop2 = (float)A.inner_tol * (float)A.inner_tol * rr;  // ||r||^2 threshold of the inner solve
      int it = 0;
      while (it < A.max_inner && rr > stop2 && stop2 > 0.0f) {
        // q = J p  (stored FP32 Jacobian rows, p from shared memory)
        float q[R];
        float pqf = 0.0f;
#pragma unroll
        for (int k = 0; k < R; ++k) {
          q[k] = 0.0f;
          if (k >= kn) break;
          if (!((interior >> k) & 1u)) continue;
          const int i = threadIdx.x + k * T;
          const float* row = J + rp_sh[i];
          float acc = 0.0f;
#pragma unroll
          for (int dz = -1; dz <= 1; ++dz)
#pragma unroll
            for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
              for (int dx = -1; dx <= 1; ++dx)
                acc = fmaf(row[(dz + 1) * 9 + (dy + 1) * 3 + (dx + 1)], p_sh[i + dx + NX * (dy + NY * dz)], acc);
          q[k] = acc;
          pqf = fmaf(acc, p_sh[i], pqf);
        }
        const float pq = bsum2<T>(pqf, 0.0f, red, half).x;
        if (!(pq > 0.0f)) { status = MRG_ENUMERIC; break; }
        const float alpha = rho / pq;
        rrf = 0.0f;
        rzf = 0.0f;
#pragma unroll
        for (int k = 0; k < R; ++k) {
          if (k >= kn) break;
          const int i = threadIdx.x + k * T;
          x_sh[i] = fmaf(alpha, p_sh[i], x_sh[i]);
          r[k] = fmaf(-alpha, q[k], r[k]);
          const float z = r[k] * mi_sh[i];
          rrf = fmaf(r[k], r[k], rrf);
          rzf = fmaf(r[k], z, rzf);
        }
        d2 = bsum2<T>(rrf, rzf, red, half);
        rr = d2.x;
        const float beta = d2.y / rho;
        rho = d2.y;
#pragma unroll
        for (int k = 0; k < R; ++k) {
          if (k >= kn) break;
          const int i = threadIdx.x + k * T;
          p_sh[i] = fmaf(beta, p_sh[i], r[k] * mi_sh[i]);
        }
        __syncthreads();
        ++it;
      }
      if (status != MRG_OK) break;
      inner_tot += it;
      // u += ||r|| x  (FP64); Dirichlet rows have r = 0 -> x = 0
#pragma unroll
      for (int k = 0; k < R; ++k) {
        if (k >= kn) break;
        const int i = threadIdx.x + k * T;
        if ((interior >> k) & 1u) u[i] = fma((double)x_sh[i], rnorm, u[i]);
      }
      __syncthreads();
      ++outer;
    }
    if (threadIdx.x == 0) {
      mrg_batch_stat st;
      st.outer_iterations = outer;
      st.inner_iterations = inner_tot;
      st.rel_residual = (r0 > 0.0) ? rnorm / r0 : 0.0;
      st.status = (status == MRG_OK && !(rnorm <= A.tol * r0 || rnorm == 0.0)) ? MRG_ENOCONV : status;
      A.stats[pid] = st;
    }
  }
}

// box-cell stiffness classes K(|dx|,|dy|,|dz|) (exact integration of the trilinear element):
// K = kx (x) my (x) mz + mx (x) ky (x) mz + mx (x) my (x) kz with 1-D k = [1,-1]/h, m = h [1/3, 1/6]
void box_classes(double hx, double hy, double hz, double* Kp) {
  const double k1[2] = {1.0, -1.0}, m1[2] = {1.0 / 3.0, 1.0 / 6.0};
  for (int c = 0; c < 8; ++c) {
    const int a = c & 1, b = (c >> 1) & 1, d = (c >> 2) & 1;
    Kp[c] = (k1[a] / hx) * (hy * m1[b]) * (hz * m1[d]) + (hx * m1[a]) * (k1[b] / hy) * (hz * m1[d]) +
            (hx * m1[a]) * (hy * m1[b]) * (k1[d] / hz);
  }
}

typedef void (*BatchKernel)(const BatchArgs);

struct KCfg {
  int threads, rows;
  BatchKernel k;
};

// rows per thread must cover the largest problem (4913 nodes for 16^3 cells)
const KCfg kCfgs[] = {
    {256, 20, k_batch<256, 20>},
    {512, 10, k_batch<512, 10>},
    {1024, 5, k_batch<1024, 5>},
};

}  // namespace

extern "C" int mrg_batch_create(const mrg_batch_desc* d, mrg_batch** out) {
  if (!d || !out || !d->sizes || !d->kappa || !d->dirichlet) return mrg_fail(MRG_EINVAL, "mrg_batch_create: null argument");
  *out = nullptr;
  if (d->n_problems < 1) return mrg_fail(MRG_EINVAL, "mrg_batch_create: n_problems must be >= 1");
  mrg_batch* B = new mrg_batch();
  B->nprob = d->n_problems;
  B->f = d->source;
  B->probs.resize(B->nprob);
  for (int k = 0; k < B->nprob; ++k) {
    BatchProb& P = B->probs[k];
    P.nx = d->sizes[3 * k];
    P.ny = d->sizes[3 * k + 1];
    P.nz = d->sizes[3 * k + 2];
    P.pad = 0;
    if (P.nx < 2 || P.ny < 2 || P.nz < 2 || P.nx > 16 || P.ny > 16 || P.nz > 16) {
      delete B;
      return mrg_fail(MRG_EINVAL, "mrg_batch_create: local problem cells per axis must be in [2, 16]");
    }
    const int64_t nc = (int64_t)P.nx * P.ny * P.nz, nnode = (int64_t)(P.nx + 1) * (P.ny + 1) * (P.nz + 1);
    P.cell_off = B->ncell;
    P.node_off = B->nnode;
    P.nnz_off = B->nnz;
    B->ncell += nc;
    B->nnode += nnode;
    B->nnz += (3LL * (P.nx + 1) - 2) * (3LL * (P.ny + 1) - 2) * (3LL * (P.nz + 1) - 2);
    B->max_nodes = std::max<int>(B->max_nodes, (int)nnode);
    const double hx = 1.0 / P.nx, hy = 1.0 / P.ny, hz = 1.0 / P.nz;
    box_classes(hx, hy, hz, P.Kp);
    for (int c = 0; c < 8; ++c) P.Kp32[c] = (float)P.Kp[c];
    P.load = d->source * hx * hy * hz / 8.0;
  }
  for (int64_t c = 0; c < B->ncell; ++c)
    if (!std::isfinite(d->kappa[c])) {
      delete B;
      return mrg_fail(MRG_ENUMERIC, "mrg_batch_create: kappa contains NaN or Inf");
    }
  // largest problems first (longest-processing-time order for the work queue)
  std::vector<int32_t> order(B->nprob);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    const BatchProb &A = B->probs[a], &C = B->probs[b];
    return (int64_t)A.nx * A.ny * A.nz > (int64_t)C.nx * C.ny * C.nz;
  });
  std::vector<float> k32(B->ncell);
  for (int64_t c = 0; c < B->ncell; ++c) k32[c] = (float)d->kappa[c];
  auto fail = [&](cudaError_t e, const char* w) {
    int st = mrg_cuda_check(e, w);
    mrg_batch_destroy(B);
    return st;
  };
  cudaError_t e;
  if ((e = cudaMalloc(&B->d_probs, B->nprob * sizeof(BatchProb))) != cudaSuccess) return fail(e, "cudaMalloc probs");
  if ((e = cudaMalloc(&B->d_order, B->nprob * sizeof(int32_t))) != cudaSuccess) return fail(e, "cudaMalloc order");
  if ((e = cudaMalloc(&B->d_kappa, B->ncell * sizeof(double))) != cudaSuccess) return fail(e, "cudaMalloc kappa");
  if ((e = cudaMalloc(&B->d_kappa32, B->ncell * sizeof(float))) != cudaSuccess) return fail(e, "cudaMalloc kappa32");
  if ((e = cudaMalloc(&B->d_g, B->nnode * sizeof(double))) != cudaSuccess) return fail(e, "cudaMalloc dirichlet");
  if ((e = cudaMalloc(&B->d_counter, sizeof(int))) != cudaSuccess) return fail(e, "cudaMalloc counter");
  if ((e = cudaMalloc(&B->d_stats, B->nprob * sizeof(mrg_batch_stat))) != cudaSuccess) return fail(e, "cudaMalloc stats");
  if ((e = cudaMemcpy(B->d_probs, B->probs.data(), B->nprob * sizeof(BatchProb), cudaMemcpyHostToDevice)) != cudaSuccess)
    return fail(e, "upload probs");
  if ((e = cudaMemcpy(B->d_order, order.data(), B->nprob * sizeof(int32_t), cudaMemcpyHostToDevice)) != cudaSuccess)
    return fail(e, "upload order");
  if ((e = cudaMemcpy(B->d_kappa, d->kappa, B->ncell * sizeof(double), cudaMemcpyHostToDevice)) != cudaSuccess)
    return fail(e, "upload kappa");
  if ((e = cudaMemcpy(B->d_kappa32, k32.data(), B->ncell * sizeof(float), cudaMemcpyHostToDevice)) != cudaSuccess)
    return fail(e, "upload kappa32");
  if ((e = cudaMemcpy(B->d_g, d->dirichlet, B->nnode * sizeof(double), cudaMemcpyHostToDevice)) != cudaSuccess)
    return fail(e, "upload dirichlet");
  // four shared-memory arrays of max_nodes words per CTA (78.6 KB for 16^3-cell problems)
  const int smem = 4 * B->max_nodes * (int)sizeof(float);
  for (const KCfg& c : kCfgs)
    if ((e = cudaFuncSetAttribute(c.k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)) != cudaSuccess)
      return fail(e, "batch kernel shared memory");
  *out = B;
  return MRG_OK;
}

extern "C" int mrg_batch_destroy(mrg_batch* B) {
  if (!B) return MRG_EINVAL;
  if (B->graph) cudaGraphExecDestroy(B->graph);
  cudaFree(B->d_probs);
  cudaFree(B->d_order);
  cudaFree(B->d_kappa);
  cudaFree(B->d_kappa32);
  cudaFree(B->d_g);
  cudaFree(B->d_counter);
  cudaFree(B->d_stats);
  delete B;
  return MRG_OK;
}

extern "C" int mrg_batch_get_info(const mrg_batch* B, mrg_batch_info* info, int64_t* node_off, int64_t* nnz_off) {
  if (!B || !info) return mrg_fail(MRG_EINVAL, "mrg_batch_get_info: null argument");
  info->n_problems = B->nprob;
  info->n_cells = B->ncell;
  info->n_nodes = B->nnode;
  info->nnz = B->nnz;
  info->threads = B->threads;
  info->ctas_per_sm = B->ctas_per_sm;
  for (int k = 0; k < B->nprob; ++k) {
    if (node_off) node_off[k] = B->probs[k].node_off;
    if (nnz_off) nnz_off[k] = B->probs[k].nnz_off;
  }
  return MRG_OK;
}

static int launch_batch(mrg_batch* B, double* u, float* J, const mrg_batch_opts* o, int threads, int ctas_per_sm,
                        cudaStream_t s) {
  int dev = 0, nsm = 0;
  MRG_CUDA(cudaGetDevice(&dev));
  MRG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const KCfg* cfg = nullptr;
  for (const KCfg& c : kCfgs)
    if (c.threads == threads) cfg = &c;
  if (!cfg) return mrg_fail(MRG_EINVAL, "mrg_batch: unsupported thread count");
  if (B->max_nodes > cfg->threads * cfg->rows) return mrg_fail(MRG_EINVAL, "mrg_batch: problem too large for config");
  BatchArgs A{B->d_probs, B->d_order, B->nprob, B->d_kappa, B->d_kappa32, B->d_g, u, J, B->d_counter, B->d_stats,
              o->tol, o->inner_tol, o->max_outer, o->max_inner, B->max_nodes};
  const int smem = 4 * B->max_nodes * (int)sizeof(float);  // p, x, 1/diag, row offsets
  const int grid = std::max(1, std::min(B->nprob, nsm * ctas_per_sm));
  MRG_CUDA(cudaMemsetAsync(B->d_counter, 0, sizeof(int), s));
  cfg->k<<<grid, cfg->threads, smem, s>>>(A);
  MRG_CUDA(cudaGetLastError());
  return MRG_OK;
}

extern "C" int mrg_batch_solve(mrg_batch* B, double* u, float* J, const mrg_batch_opts* o, mrg_batch_stat* stats,
                               mrg_stream_t stream) {
  if (!B || !u || !J || !o) return mrg_fail(MRG_EINVAL, "mrg_batch_solve: null argument");
  if (!(o->tol > 0.0) || !(o->inner_tol > 0.0) || o->max_outer < 1 || o->max_inner < 1)
    return mrg_fail(MRG_EINVAL, "mrg_batch_solve: bad options");
  cudaStream_t s = (cudaStream_t)stream;
  // one captured graph per (buffers, options, configuration, stream): counter reset + persistent launch
  const bool same = B->graph && B->graph_key[0] == u && B->graph_key[1] == J && B->graph_threads == B->threads &&
                    B->graph_ctas == B->ctas_per_sm && B->graph_stream == s && B->graph_tol[0] == o->tol &&
                    B->graph_tol[1] == o->inner_tol && B->graph_iters[0] == o->max_outer &&
                    B->graph_iters[1] == o->max_inner;
  if (!same) {
    if (B->graph) cudaGraphExecDestroy(B->graph);
    B->graph = nullptr;
    cudaStream_t cs = s;
    bool own = false;
    if (!s) {
      MRG_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
      own = true;
    }
    cudaGraph_t gph;
    MRG_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
    int rc = launch_batch(B, u, J, o, B->threads, B->ctas_per_sm, cs);
    cudaError_t e = cudaStreamEndCapture(cs, &gph);
    if (own) cudaStreamDestroy(cs);
    if (rc) return rc;
    if (e != cudaSuccess) return mrg_cuda_check(e, "capture batch solve");
    e = cudaGraphInstantiate(&B->graph, gph, 0);
    cudaGraphDestroy(gph);
    if (e != cudaSuccess) return mrg_cuda_check(e, "instantiate batch solve");
    B->graph_key[0] = u;
    B->graph_key[1] = J;
    B->graph_threads = B->threads;
    B->graph_ctas = B->ctas_per_sm;
    B->graph_stream = s;
    B->graph_tol[0] = o->tol;
    B->graph_tol[1] = o->inner_tol;
    B->graph_iters[0] = o->max_outer;
    B->graph_iters[1] = o->max_inner;
  }
  MRG_CUDA(cudaGraphLaunch(B->graph, s));
  if (stats) {
    MRG_CUDA(cudaMemcpyAsync(stats, B->d_stats, B->nprob * sizeof(mrg_batch_stat), cudaMemcpyDeviceToHost, s));
    MRG_CUDA(cudaStreamSynchronize(s));
    for (int k = 0; k < B->nprob; ++k)
      if (stats[k].status != MRG_OK) return mrg_fail(stats[k].status, "mrg_batch_solve: a local problem did not converge");
  }
  return MRG_OK;
}

// Autotuner: times the whole batch for each (threads, CTAs per SM) configuration that fits and keeps
// the fastest.  The buffers are scratch for the trials (their contents are overwritten).
extern "C" int mrg_batch_autotune(mrg_batch* B, double* u, float* J, const mrg_batch_opts* o, mrg_stream_t stream) {
  if (!B || !u || !J || !o) return mrg_fail(MRG_EINVAL, "mrg_batch_autotune: null argument");
  cudaStream_t s = (cudaStream_t)stream;
  cudaEvent_t e0, e1;
  MRG_CUDA(cudaEventCreate(&e0));
  MRG_CUDA(cudaEventCreate(&e1));
  float best = 1e30f;
  int bt = B->threads, bc = B->ctas_per_sm;
  for (const KCfg& c : kCfgs) {
    if (B->max_nodes > c.threads * c.rows) continue;
    for (int cps : {1, 2, 4, 8}) {
      if (c.threads * cps > 2048) continue;
      int rc = launch_batch(B, u, J, o, c.threads, cps, s);  // warm
      if (rc) continue;
      MRG_CUDA(cudaEventRecord(e0, s));
      rc = launch_batch(B, u, J, o, c.threads, cps, s);
      MRG_CUDA(cudaEventRecord(e1, s));
      MRG_CUDA(cudaEventSynchronize(e1));
      float ms = 0.f;
      MRG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      if (rc == MRG_OK && ms < best) {
        best = ms;
        bt = c.threads;
        bc = cps;
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  B->threads = bt;
  B->ctas_per_sm = bc;
  return MRG_OK;
}

extern "C" int mrg_batch_set_config(mrg_batch* B, int32_t threads, int32_t ctas_per_sm) {
  if (!B) return mrg_fail(MRG_EINVAL, "mrg_batch_set_config: null batch");
  bool ok = false;
  for (const KCfg& c : kCfgs)
    if (c.threads == threads && B->max_nodes <= c.threads * c.rows) ok = true;
  if (!ok || ctas_per_sm < 1 || ctas_per_sm > 16) return mrg_fail(MRG_EINVAL, "mrg_batch_set_config: unsupported");
  B->threads = threads;
  B->ctas_per_sm = ctas_per_sm;
  return MRG_OK;
}
