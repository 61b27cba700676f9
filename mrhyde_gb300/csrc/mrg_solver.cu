// Linear algebra on the assembled system and the Newton driver.
//
//   mrg_spmv       y = J x on the canonical structured graph (Tpetra CrsMatrix::apply)
//   mrg_solve_pcg  Jacobi PCG, the iteration of SolverManager::PCG
//                  (src/managers/solver/solverManager_solvers.hpp:812-901)
//   mrg_newton     SolverManager::nonlinearSolver (src/managers/solver/solverManager_solvers.hpp:290-643)
//
// Design: the column indices of the canonical graph are implied by the structured layout, so the
// SpMV reads only the values (8 or 4 bytes per nonzero) and the source vector.  For Q1 rows a warp
// stages the CSR values of its 32 rows in shared memory with one bulk copy (cp.async.bulk on a
// per-warp mbarrier), double-buffered, with no CTA-wide barrier.  An FP64 PCG iteration is three
// kernels (SpMV+dot, vector update+dots, direction update); the FP32 inner PCG keeps q = J p by
// recurrence and folds the direction update into its SpMV (two kernels).  Each dot product is reduced
// deterministically by the "last block finishes the sum" pattern (partials written per block, a
// counter incremented after a fence, the last block sums the partials in index order) -- no extra
// launch, no spinning, and bit-identical results from run to run and independent of what else runs
// on the GPU.  The scalars (alpha, beta, rho, norms, iteration count, done flag) live in device
// memory, so a chunk of iterations is captured once as a CUDA graph and replayed; the host reads the
// done flag once per chunk.  After convergence every kernel returns at entry.
//
// Mixed precision: the Jacobian values and the inner PCG vectors are FP32 (half the bytes per
// iteration), dot products are accumulated in FP64 per block; the Newton residual, the update of u
// and the stopping test stay FP64, so Newton / iterative refinement recovers the FP64 solution.
#include <cmath>
#include <mutex>
#include <string>
#include <vector>

#include "mrg_device.cuh"
#include "mrg_internal.h"

namespace {

using namespace mrgdev;

constexpr int ST = WST;          // rows per CTA
constexpr int CHUNK = 16;        // PCG iterations per captured graph

// device scalars of one PCG instance
struct PcgScal {
  double rho, rho_old, pq, alpha, beta, r0, rnorm, tol;
  int iter, maxiter, done, status;
  unsigned int counter;
  int pad;
};

// y = J x (FP64 accumulation); Q1 rows through the per-warp staged loop.  err (may be null) is set to
// 1 if a staging copy did not complete within its time bound.
template <int P, typename JT>
__global__ void __launch_bounds__(ST) k_spmv(Grid g, int64_t nrows, const JT* __restrict__ J, const double* __restrict__ x,
                                             double* __restrict__ y, int* err) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t mbar[2 * (ST / 32)];
  if constexpr (P == 1) {
    const bool ok = warp_staged_rows<JT>(g, nrows, J, smem_raw, mbar, [&](int64_t n, const RowInfo& R, const JT* vals) {
      y[n] = row_apply<1, JT, double>(g, R, vals, x);
    });
    if (!ok && err) atomicExch(err, 1);
  } else {
    for (int64_t n = (int64_t)blockIdx.x * ST + threadIdx.x; n < nrows; n += (int64_t)gridDim.x * ST) {
      int ix, iy, iz;
      decompose(g, n, ix, iy, iz);
      const RowInfo R = row_info<P>(g, ix, iy, iz);
      y[n] = row_apply<P, JT, double>(g, R, J + R.rp, x);
    }
  }
}

// ---- FP64 PCG kernels ---------------------------------------------------------------------------
// All PCG kernels are grid-stride loops over a fixed grid of at most 16 CTAs per SM, so that each
// deterministic reduction has at most a few thousand per-CTA partials and counter increments.
struct PcgVec64 {
  double *x, *r, *z, *p, *q, *minv, *parts;
  const double* b;
  const double* J;
  PcgScal* s;
};

// r = b - J x, minv = 1/diag, z = minv r, p = z; partial r.r, r.z
template <int P>
__global__ void __launch_bounds__(ST) k_pcg64_init(Grid g, int64_t nrows, PcgVec64 V) {
  double rr = 0.0, rz = 0.0;
  for (int64_t n = (int64_t)blockIdx.x * ST + threadIdx.x; n < nrows; n += (int64_t)gridDim.x * ST) {
    int ix, iy, iz;
    decompose(g, n, ix, iy, iz);
    RowInfo R = row_info<P>(g, ix, iy, iz);
    double ax = row_apply<P, double, double>(g, R, V.J + R.rp, V.x);
    double d = V.J[R.rp + ((int64_t)(iz - R.lz) * R.cy + (iy - R.ly)) * R.cx + (ix - R.lx)];
    double mi = 1.0 / d;
    double r = V.b[n] - ax;
    double z = r * mi;
    V.minv[n] = mi;
    V.r[n] = r;
    V.z[n] = z;
    V.p[n] = z;
    rr = fma(r, r, rr);
    rz = fma(r, z, rz);
  }
  double m[2] = {block_sum(rr), block_sum(rz)};
  if (last_block<2>(V.parts, m, &V.s->counter)) {
    double t[2];
    sum_parts<2>(V.parts, t, &V.s->counter);
    if (threadIdx.x == 0) {
      PcgScal* s = V.s;
      s->r0 = sqrt(t[0]);
      s->rnorm = s->r0;
      s->rho = t[1];
      s->iter = 0;
      s->status = MRG_OK;
      s->done = (s->r0 == 0.0 || !(s->r0 / s->r0 > s->tol) || s->maxiter <= 0) ? 1 : 0;
      if (!isfinite(s->r0)) { s->done = 1; s->status = MRG_ENUMERIC; }
    }
  }
}

// q = J p ; pq partial ; last block: alpha = rho / pq
template <int P>
__global__ void __launch_bounds__(ST) k_pcg64_spmv(Grid g, int64_t nrows, PcgVec64 V) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t mbar[2 * (ST / 32)];
  if (((volatile PcgScal*)V.s)->done) return;
  double pq = 0.0;
  if constexpr (P == 1) {
    const bool ok = warp_staged_rows<double>(g, nrows, V.J, smem_raw, mbar, [&](int64_t n, const RowInfo& R,
                                                                                  const double* vals) {
      const double q = row_apply<1, double, double>(g, R, vals, V.p);
      V.q[n] = q;
      pq = fma(V.p[n], q, pq);
    });
    if (!ok) { V.s->status = MRG_ETIMEOUT; V.s->done = 1; }
  } else {
    for (int64_t n = (int64_t)blockIdx.x * ST + threadIdx.x; n < nrows; n += (int64_t)gridDim.x * ST) {
      int ix, iy, iz;
      decompose(g, n, ix, iy, iz);
      const RowInfo R = row_info<P>(g, ix, iy, iz);
      const double q = row_apply<P, double, double>(g, R, V.J + R.rp, V.p);
      V.q[n] = q;
      pq = fma(V.p[n], q, pq);
    }
  }
  double m[1] = {block_sum(pq)};
  if (last_block<1>(V.parts, m, &V.s->counter)) {
    double t[1];
    sum_parts<1>(V.parts, t, &V.s->counter);
    if (threadIdx.x == 0) {
      PcgScal* s = V.s;
      s->pq = t[0];
      s->alpha = s->rho / t[0];
      if (!(t[0] > 0.0) || !isfinite(s->alpha)) {
        if (s->status == MRG_OK) s->status = MRG_ENUMERIC;
        s->done = 1;
      }
    }
  }
}

// x += alpha p ; r -= alpha q ; z = minv r ; partial r.r, r.z ; last block: beta, stopping test
__global__ void __launch_bounds__(ST) k_pcg64_update(int64_t nrows, PcgVec64 V) {
  if (((volatile PcgScal*)V.s)->done) return;
  const double alpha = V.s->alpha;
  double rr = 0.0, rz = 0.0;
  const int64_t st = (int64_t)gridDim.x * ST;
  int64_t n = (int64_t)blockIdx.x * ST + threadIdx.x;
  for (; n + 3 * st < nrows; n += 4 * st) {
    double p[4], q[4], r[4], x[4], mi[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      p[k] = V.p[n + k * st]; q[k] = V.q[n + k * st]; r[k] = V.r[n + k * st];
      x[k] = V.x[n + k * st]; mi[k] = V.minv[n + k * st];
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      V.x[n + k * st] = fma(alpha, p[k], x[k]);
      const double rn = fma(-alpha, q[k], r[k]);
      const double z = rn * mi[k];
      V.r[n + k * st] = rn;
      V.z[n + k * st] = z;
      rr = fma(rn, rn, rr);
      rz = fma(rn, z, rz);
    }
  }
  for (; n < nrows; n += st) {
    V.x[n] = fma(alpha, V.p[n], V.x[n]);
    double r = fma(-alpha, V.q[n], V.r[n]);
    double z = r * V.minv[n];
    V.r[n] = r;
    V.z[n] = z;
    rr = fma(r, r, rr);
    rz = fma(r, z, rz);
  }
  double m[2] = {block_sum(rr), block_sum(rz)};
  if (last_block<2>(V.parts, m, &V.s->counter)) {
    double t[2];
    sum_parts<2>(V.parts, t, &V.s->counter);
    if (threadIdx.x == 0) {
      PcgScal* s = V.s;
      s->rnorm = sqrt(t[0]);
      s->rho_old = s->rho;
      s->rho = t[1];
      s->beta = s->rho / s->rho_old;
      s->iter += 1;
      if (!(s->rnorm / s->r0 > s->tol) || s->iter >= s->maxiter) s->done = 1;
      if (!isfinite(s->rnorm)) {
        s->done = 1;
        if (s->status == MRG_OK) s->status = MRG_ENUMERIC;
      }
    }
  }
}

// p = z + beta p
__global__ void __launch_bounds__(ST) k_pcg64_dir(int64_t nrows, PcgVec64 V) {
  if (((volatile PcgScal*)V.s)->done) return;
  const double beta = V.s->beta;
  const int64_t st = (int64_t)gridDim.x * ST;
  int64_t n = (int64_t)blockIdx.x * ST + threadIdx.x;
  for (; n + 3 * st < nrows; n += 4 * st) {
    double p[4], z[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) { p[k] = V.p[n + k * st]; z[k] = V.z[n + k * st]; }
#pragma unroll
    for (int k = 0; k < 4; ++k) V.p[n + k * st] = fma(beta, p[k], z[k]);
  }
  for (; n < nrows; n += st) V.p[n] = fma(beta, V.p[n], V.z[n]);
}

// ---- FP32 inner PCG kernels (mixed path) ---------------------------------------------------------
struct PcgVec32 {
  float *x, *r, *z, *p, *q, *minv;
  double* parts;
  const double* b;   // FP64 right-hand side (converted on the fly)
  const float* J;
  PcgScal* s;
};

template <int P>
__global__ void __launch_bounds__(ST) k_pcg32_init(Grid g, int64_t nrows, PcgVec32 V) {
  double rr = 0.0, rz = 0.0;
  for (int64_t n = (int64_t)blockIdx.x * ST + threadIdx.x; n < nrows; n += (int64_t)gridDim.x * ST) {
    int ix, iy, iz;
    decompose(g, n, ix, iy, iz);
    RowInfo R = row_info<P>(g, ix, iy, iz);
    float d = V.J[R.rp + ((int64_t)(iz - R.lz) * R.cy + (iy - R.ly)) * R.cx + (ix - R.lx)];
    float mi = 1.0f / d;
    float r = (float)V.b[n];   // x0 = 0
    float z = r * mi;
    V.x[n] = 0.0f;
    V.minv[n] = mi;
    V.r[n] = r;
    V.z[n] = z;
    V.p[n] = z;
    V.q[n] = 0.0f;
    rr += (double)(r * r);
    rz += (double)(r * z);
  }
  double m[2] = {block_sum(rr), block_sum(rz)};
  if (last_block<2>(V.parts, m, &V.s->counter)) {
    double t[2];
    sum_parts<2>(V.parts, t, &V.s->counter);
    if (threadIdx.x == 0) {
      PcgScal* s = V.s;
      s->beta = 0.0;
      s->r0 = sqrt(t[0]);
      s->rnorm = s->r0;
      s->rho = t[1];
      s->iter = 0;
      s->status = MRG_OK;
      s->done = (s->r0 == 0.0 || s->maxiter <= 0) ? 1 : 0;
      if (!isfinite(s->r0)) { s->done = 1; s->status = MRG_ENUMERIC; }
    }
  }
}

// FP32 PCG, direction and product in one pass.  With q = J p maintained by recurrence,
//   p <- z + beta p,   q <- J z + beta q   (= J p by linearity),
// so the SpMV reads z and the separate direction update of the classic loop disappears: one
// iteration is this kernel plus k_pcg32_update.  Partial p.q; last block: alpha = rho / (p.q).
// Before the first iteration p = z, q = 0 and beta = 0.
template <int P>
__global__ void __launch_bounds__(ST) k_pcg32_spmv(Grid g, int64_t nrows, PcgVec32 V) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t mbar[2 * (ST / 32)];
  if (((volatile PcgScal*)V.s)->done) return;
  const float beta = (float)V.s->beta;
  float pq = 0.0f;
  auto fin = [&](int64_t n, float w) {
    const float pn = fmaf(beta, V.p[n], V.z[n]);
    const float qn = fmaf(beta, V.q[n], w);
    V.p[n] = pn;
    V.q[n] = qn;
    pq = fmaf(pn, qn, pq);
  };
  if constexpr (P == 1) {
    const bool ok = warp_staged_rows<float>(g, nrows, V.J, smem_raw, mbar, [&](int64_t n, const RowInfo& R,
                                                                                const float* vals) {
      fin(n, row_apply_f<1>(g, R, vals, V.z));
    });
    if (!ok) { V.s->status = MRG_ETIMEOUT; V.s->done = 1; }
  } else {
    for (int64_t n = (int64_t)blockIdx.x * ST + threadIdx.x; n < nrows; n += (int64_t)gridDim.x * ST) {
      int ix, iy, iz;
      decompose(g, n, ix, iy, iz);
      const RowInfo R = row_info<P>(g, ix, iy, iz);
      fin(n, row_apply_f<P>(g, R, V.J + R.rp, V.z));
    }
  }
  double m[1] = {block_sum((double)pq)};
  if (last_block<1>(V.parts, m, &V.s->counter)) {
    double t[1];
    sum_parts<1>(V.parts, t, &V.s->counter);
    if (threadIdx.x == 0) {
      PcgScal* s = V.s;
      s->pq = t[0];
      s->alpha = s->rho / t[0];
      if (!(t[0] > 0.0) || !isfinite(s->alpha)) {
        if (s->status == MRG_OK) s->status = MRG_ENUMERIC;
        s->done = 1;
      }
    }
  }
}

__global__ void __launch_bounds__(ST) k_pcg32_update(int64_t nrows, PcgVec32 V) {
  if (((volatile PcgScal*)V.s)->done) return;
  const float alpha = (float)V.s->alpha;
  float rr = 0.0f, rz = 0.0f;
  const int64_t st = (int64_t)gridDim.x * ST;
  int64_t n = (int64_t)blockIdx.x * ST + threadIdx.x;
  for (; n + 3 * st < nrows; n += 4 * st) {
    float p[4], q[4], r[4], x[4], mi[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      p[k] = V.p[n + k * st]; q[k] = V.q[n + k * st]; r[k] = V.r[n + k * st];
      x[k] = V.x[n + k * st]; mi[k] = V.minv[n + k * st];
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      V.x[n + k * st] = fmaf(alpha, p[k], x[k]);
      const float rn = fmaf(-alpha, q[k], r[k]);
      const float z = rn * mi[k];
      V.r[n + k * st] = rn;
      V.z[n + k * st] = z;
      rr = fmaf(rn, rn, rr);
      rz = fmaf(rn, z, rz);
    }
  }
  for (; n < nrows; n += st) {
    V.x[n] = fmaf(alpha, V.p[n], V.x[n]);
    float r = fmaf(-alpha, V.q[n], V.r[n]);
    float z = r * V.minv[n];
    V.r[n] = r;
    V.z[n] = z;
    rr = fmaf(r, r, rr);
    rz = fmaf(r, z, rz);
  }
  double m[2] = {block_sum((double)rr), block_sum((double)rz)};
  if (last_block<2>(V.parts, m, &V.s->counter)) {
    double t[2];
    sum_parts<2>(V.parts, t, &V.s->counter);
    if (threadIdx.x == 0) {
      PcgScal* s = V.s;
      s->rnorm = sqrt(t[0]);
      s->rho_old = s->rho;
      s->rho = t[1];
      s->beta = s->rho / s->rho_old;
      s->iter += 1;
      if (!(s->rnorm / s->r0 > s->tol) || s->iter >= s->maxiter) s->done = 1;
      if (!isfinite(s->rnorm)) {
        s->done = 1;
        if (s->status == MRG_OK) s->status = MRG_ENUMERIC;
      }
    }
  }
}

// u += (double) du32   (mixed path update; Dirichlet rows have du = 0 because r = 0 there)
__global__ void k_add_f32(int64_t n, const float* __restrict__ du, double* __restrict__ u) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) u[i] += (double)du[i];
}
__global__ void k_axpy(int64_t n, double a, const double* __restrict__ x, double* __restrict__ y) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = fma(a, x[i], y[i]);
}
__global__ void k_f32_to_f64(int64_t n, const float* __restrict__ a, double* __restrict__ b) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = (double)a[i];
}

// inf-norm with the last-block pattern; result in s->rnorm
__global__ void __launch_bounds__(ST) k_norminf(int64_t n, const double* __restrict__ v, double* parts, PcgScal* s) {
  double a = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * ST + threadIdx.x; i < n; i += (int64_t)gridDim.x * ST) {
    const double x = v[i];
    a = isfinite(x) ? fmax(a, fabs(x)) : INFINITY;
  }
  double m[1] = {block_max(a)};
  if (last_block<1>(parts, m, &s->counter)) {
    double mx = 0.0;
    for (unsigned int k = threadIdx.x; k < gridDim.x; k += blockDim.x) mx = fmax(mx, __ldcg(parts + k));
    mx = block_max(mx);
    if (threadIdx.x == 0) {
      s->rnorm = mx;
      s->counter = 0u;
    }
  }
}

inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

// host message for a failed PCG, chosen from the device status word
inline std::string pcg_status_text(const char* who, int status) {
  switch (status) {
    case MRG_ETIMEOUT:
      return std::string(who) + ": a CSR staging copy of the SpMV did not complete within its time bound";
    case MRG_ENUMERIC:
      return std::string(who) + ": non-positive or non-finite curvature (matrix not SPD?) or non-finite residual";
    default:
      return std::string(who) + ": failed with status " + std::to_string(status);
  }
}

// grid of the PCG kernels: one CTA per 128-row tile, at most per_sm CTAs per SM of the current device
inline unsigned pcg_grid(const mrg_problem* p, int per_sm = 16) {
  const unsigned tiles = nblk(p->ndof, ST);
  const unsigned cap = (unsigned)(per_sm * mrg_device_sms());
  return tiles < cap ? tiles : cap;
}

// dynamic shared memory of the PCG SpMV: two staging buffers for P = 1
template <int P, typename JT>
constexpr int spmv_smem() { return P == 1 ? wspmv_smem<JT>() : 0; }
// CTAs per SM the SpMV grid is sized for (shared-memory bound for P = 1)
template <int P, typename JT>
constexpr int spmv_per_sm() { return P == 1 ? (sizeof(JT) == 8 ? 4 : 7) : 16; }

}  // namespace

// ------------------------------------------------------------------------------------------------
// workspace
// ------------------------------------------------------------------------------------------------
struct SolverWork {
  int64_t n = 0, nnz = 0;
  double *r = nullptr, *z = nullptr, *p = nullptr, *q = nullptr, *minv = nullptr, *parts = nullptr;
  float *x32 = nullptr, *r32 = nullptr, *z32 = nullptr, *p32 = nullptr, *q32 = nullptr, *minv32 = nullptr;
  PcgScal* s = nullptr;
  PcgScal* h_s = nullptr;       // pinned host mirror
  // Newton buffers
  double *F = nullptr, *du = nullptr, *J64 = nullptr;
  float* J32 = nullptr;
  // captured iteration chunks
  cudaGraphExec_t g64 = nullptr, g32 = nullptr;
  const void* g64_key[3] = {nullptr, nullptr, nullptr};
  const void* g32_key[3] = {nullptr, nullptr, nullptr};
  cudaStream_t g64_stream = nullptr, g32_stream = nullptr;
};

void mrg_solver_free(mrg_problem* p) {
  SolverWork* w = p->work;
  if (!w) return;
  if (w->g64) cudaGraphExecDestroy(w->g64);
  if (w->g32) cudaGraphExecDestroy(w->g32);
  cudaStream_t s = p->stream;
  for (void* ptr : {(void*)w->r, (void*)w->z, (void*)w->p, (void*)w->q, (void*)w->minv, (void*)w->parts,
                    (void*)w->x32, (void*)w->r32, (void*)w->z32, (void*)w->p32, (void*)w->q32, (void*)w->minv32,
                    (void*)w->s, (void*)w->F, (void*)w->du, (void*)w->J64, (void*)w->J32})
    if (ptr) cudaFreeAsync(ptr, s);
  mrg_pinned_release(w->h_s);
  delete w;
  p->work = nullptr;
}

void mrg_solver_drop_graphs(mrg_problem* p) {
  SolverWork* w = p->work;
  if (!w) return;
  if (w->g64) cudaGraphExecDestroy(w->g64);
  if (w->g32) cudaGraphExecDestroy(w->g32);
  w->g64 = w->g32 = nullptr;
}

static int ensure_work(mrg_problem* p, bool need64, bool need32, cudaStream_t st) {
  if (!p->work) {
    p->work = new SolverWork();
    p->work->n = p->ndof;
    p->work->nnz = p->nnz;
  }
  SolverWork* w = p->work;
  const int64_t n = p->ndof;
  static bool attrs = false;  // opt in to more than 48 KB of dynamic shared memory (once per process)
  if (!attrs) {
    MRG_CUDA(cudaFuncSetAttribute(k_pcg64_spmv<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, spmv_smem<1, double>()));
    MRG_CUDA(cudaFuncSetAttribute(k_pcg32_spmv<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, spmv_smem<1, float>()));
    attrs = true;
  }
  const size_t nparts = 3 * (size_t)nblk(n, ST) + 64;
  if (!w->parts) MRG_CUDA(cudaMallocAsync(&w->parts, nparts * sizeof(double), st));
  if (!w->s) {
    MRG_CUDA(cudaMallocAsync(&w->s, sizeof(PcgScal), st));
    MRG_CUDA(cudaMemsetAsync(w->s, 0, sizeof(PcgScal), st));
    static_assert(sizeof(PcgScal) <= 256, "pinned slot size");
    w->h_s = (PcgScal*)mrg_pinned_slot();
    if (!w->h_s) return mrg_fail(MRG_ENOMEM, "solver pinned scalars");
  }
  if (need64 && !w->r) {
    MRG_CUDA(cudaMallocAsync(&w->r, n * sizeof(double), st));
    MRG_CUDA(cudaMallocAsync(&w->z, n * sizeof(double), st));
    MRG_CUDA(cudaMallocAsync(&w->p, n * sizeof(double), st));
    MRG_CUDA(cudaMallocAsync(&w->q, n * sizeof(double), st));
    MRG_CUDA(cudaMallocAsync(&w->minv, n * sizeof(double), st));
  }
  if (need32 && !w->r32) {
    MRG_CUDA(cudaMallocAsync(&w->x32, n * sizeof(float), st));
    MRG_CUDA(cudaMallocAsync(&w->r32, n * sizeof(float), st));
    MRG_CUDA(cudaMallocAsync(&w->z32, n * sizeof(float), st));
    MRG_CUDA(cudaMallocAsync(&w->p32, n * sizeof(float), st));
    MRG_CUDA(cudaMallocAsync(&w->q32, n * sizeof(float), st));
    MRG_CUDA(cudaMallocAsync(&w->minv32, n * sizeof(float), st));
  }
  return MRG_OK;
}

template <int P>
static void enqueue_chunk64(const mrg_problem* p, const PcgVec64& V, cudaStream_t s) {
  const unsigned nb = pcg_grid(p);
  const unsigned nbs = pcg_grid(p, spmv_per_sm<P, double>());
  for (int it = 0; it < CHUNK; ++it) {
    k_pcg64_spmv<P><<<nbs, ST, spmv_smem<P, double>(), s>>>(p->g, p->ndof, V);
    k_pcg64_update<<<nb, ST, 0, s>>>(p->ndof, V);
    k_pcg64_dir<<<nb, ST, 0, s>>>(p->ndof, V);
  }
}
template <int P>
static void enqueue_chunk32(const mrg_problem* p, const PcgVec32& V, cudaStream_t s) {
  const unsigned nb = pcg_grid(p);
  const unsigned nbs = pcg_grid(p, spmv_per_sm<P, float>());
  for (int it = 0; it < CHUNK; ++it) {
    k_pcg32_spmv<P><<<nbs, ST, spmv_smem<P, float>(), s>>>(p->g, p->ndof, V);
    k_pcg32_update<<<nb, ST, 0, s>>>(p->ndof, V);
  }
}

// Capture one chunk of iterations as a graph (re-captured when the buffers or stream change).
static int chunk_graph(cudaGraphExec_t* exec, const void** key, cudaStream_t* kstream, const void* a, const void* b,
                       const void* c, cudaStream_t s, void (*enqueue)(const mrg_problem*, const void*, cudaStream_t),
                       const mrg_problem* p, const void* V) {
  if (*exec && key[0] == a && key[1] == b && key[2] == c && *kstream == s) return MRG_OK;
  if (*exec) {
    cudaGraphExecDestroy(*exec);
    *exec = nullptr;
  }
  cudaStream_t cs = s;
  bool own = false;
  if (s == nullptr) {  // the legacy default stream cannot be captured: capture on a private stream
    MRG_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    own = true;
  }
  cudaGraph_t graph;
  MRG_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
  enqueue(p, V, cs);
  cudaError_t e = cudaStreamEndCapture(cs, &graph);
  if (own) cudaStreamDestroy(cs);
  if (e != cudaSuccess) return mrg_cuda_check(e, "capture PCG chunk");
  e = cudaGraphInstantiate(exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return mrg_cuda_check(e, "instantiate PCG chunk");
  key[0] = a; key[1] = b; key[2] = c;
  *kstream = s;
  return MRG_OK;
}

static void enq64_p1(const mrg_problem* p, const void* V, cudaStream_t s) { enqueue_chunk64<1>(p, *(const PcgVec64*)V, s); }
static void enq64_p2(const mrg_problem* p, const void* V, cudaStream_t s) { enqueue_chunk64<2>(p, *(const PcgVec64*)V, s); }
static void enq32_p1(const mrg_problem* p, const void* V, cudaStream_t s) { enqueue_chunk32<1>(p, *(const PcgVec32*)V, s); }
static void enq32_p2(const mrg_problem* p, const void* V, cudaStream_t s) { enqueue_chunk32<2>(p, *(const PcgVec32*)V, s); }

// Runs the chunk graph until the device done flag is set.  Reads the scalars back (one sync per chunk).
static int run_chunks(mrg_problem* p, cudaGraphExec_t exec, cudaStream_t s, int maxiter) {
  SolverWork* w = p->work;
  const int max_chunks = maxiter / CHUNK + 2;
  for (int c = 0; c < max_chunks; ++c) {
    MRG_CUDA(cudaGraphLaunch(exec, s));
    MRG_CUDA(cudaMemcpyAsync(w->h_s, w->s, sizeof(PcgScal), cudaMemcpyDeviceToHost, s));
    MRG_CUDA(cudaStreamSynchronize(s));
    if (w->h_s->done) return MRG_OK;
  }
  return MRG_OK;
}

static int pcg64(mrg_problem* p, const double* J, const double* b, double* x, double rtol, int maxiter,
                 mrg_solve_stats* st, cudaStream_t s) {
  int rc = ensure_work(p, true, false, s);
  if (rc) return rc;
  SolverWork* w = p->work;
  PcgVec64 V{x, w->r, w->z, w->p, w->q, w->minv, w->parts, b, J, w->s};
  PcgScal init{};
  init.tol = rtol;
  init.maxiter = maxiter;
  MRG_CUDA(cudaMemcpyAsync(w->s, &init, sizeof(PcgScal), cudaMemcpyHostToDevice, s));
  const unsigned nb = pcg_grid(p);
  if (p->g.p == 1) k_pcg64_init<1><<<nb, ST, 0, s>>>(p->g, p->ndof, V);
  else k_pcg64_init<2><<<nb, ST, 0, s>>>(p->g, p->ndof, V);
  MRG_CUDA(cudaGetLastError());
  rc = chunk_graph(&w->g64, w->g64_key, &w->g64_stream, J, b, x, s, p->g.p == 1 ? enq64_p1 : enq64_p2, p, &V);
  if (rc) return rc;
  rc = run_chunks(p, w->g64, s, maxiter);
  if (rc) return rc;
  PcgScal* h = w->h_s;
  if (st) {
    st->iterations = h->iter;
    st->outer_iterations = 0;
    st->rel_residual = (h->r0 > 0) ? h->rnorm / h->r0 : 0.0;
    st->abs_residual = h->rnorm;
    st->status = h->status;
  }
  if (h->status != MRG_OK) return mrg_fail(h->status, pcg_status_text("PCG", h->status));
  if (h->r0 > 0 && h->rnorm / h->r0 > rtol) {
    if (st) st->status = MRG_ENOCONV;
    return mrg_fail(MRG_ENOCONV, "PCG: maximum iterations reached before the tolerance");
  }
  return MRG_OK;
}

// FP32 PCG on J32 dx = b (x0 = 0); result in w->x32
static int pcg32(mrg_problem* p, const float* J, const double* b, double rtol, int maxiter, mrg_solve_stats* st,
                 cudaStream_t s) {
  int rc = ensure_work(p, false, true, s);
  if (rc) return rc;
  SolverWork* w = p->work;
  PcgVec32 V{w->x32, w->r32, w->z32, w->p32, w->q32, w->minv32, w->parts, b, J, w->s};
  PcgScal init{};
  init.tol = rtol;
  init.maxiter = maxiter;
  MRG_CUDA(cudaMemcpyAsync(w->s, &init, sizeof(PcgScal), cudaMemcpyHostToDevice, s));
  const unsigned nb = pcg_grid(p);
  if (p->g.p == 1) k_pcg32_init<1><<<nb, ST, 0, s>>>(p->g, p->ndof, V);
  else k_pcg32_init<2><<<nb, ST, 0, s>>>(p->g, p->ndof, V);
  MRG_CUDA(cudaGetLastError());
  rc = chunk_graph(&w->g32, w->g32_key, &w->g32_stream, J, b, w->x32, s, p->g.p == 1 ? enq32_p1 : enq32_p2, p, &V);
  if (rc) return rc;
  rc = run_chunks(p, w->g32, s, maxiter);
  if (rc) return rc;
  PcgScal* h = w->h_s;
  if (st) {
    st->iterations = h->iter;
    st->rel_residual = (h->r0 > 0) ? h->rnorm / h->r0 : 0.0;
    st->abs_residual = h->rnorm;
    st->status = h->status;
  }
  if (h->status != MRG_OK) return mrg_fail(h->status, pcg_status_text("PCG (FP32)", h->status));
  return MRG_OK;
}

extern "C" int mrg_spmv(const mrg_problem* p, const void* J, int32_t fp32, const double* x, double* y,
                        mrg_stream_t stream) {
  if (!p || !J || !x || !y) return mrg_fail(MRG_EINVAL, "mrg_spmv: null argument");
  cudaStream_t s = (cudaStream_t)stream;
  static std::once_flag attr_once;
  static cudaError_t attr_err = cudaSuccess;
  std::call_once(attr_once, [] {
    attr_err = cudaFuncSetAttribute(k_spmv<1, double>, cudaFuncAttributeMaxDynamicSharedMemorySize, spmv_smem<1, double>());
    if (attr_err == cudaSuccess)
      attr_err = cudaFuncSetAttribute(k_spmv<1, float>, cudaFuncAttributeMaxDynamicSharedMemorySize, spmv_smem<1, float>());
  });
  MRG_CUDA(attr_err);
  if (p->g.p == 1) {
    if (fp32) k_spmv<1, float><<<pcg_grid(p, spmv_per_sm<1, float>()), ST, spmv_smem<1, float>(), s>>>(p->g, p->ndof, (const float*)J, x, y, nullptr);
    else k_spmv<1, double><<<pcg_grid(p, spmv_per_sm<1, double>()), ST, spmv_smem<1, double>(), s>>>(p->g, p->ndof, (const double*)J, x, y, nullptr);
  } else {
    if (fp32) k_spmv<2, float><<<pcg_grid(p), ST, 0, s>>>(p->g, p->ndof, (const float*)J, x, y, nullptr);
    else k_spmv<2, double><<<pcg_grid(p), ST, 0, s>>>(p->g, p->ndof, (const double*)J, x, y, nullptr);
  }
  MRG_CUDA(cudaGetLastError());
  return MRG_OK;
}

// res = b - res
__global__ void k_b_minus(int64_t n, const double* __restrict__ b, double* __restrict__ res) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) res[i] = b[i] - res[i];
}

extern "C" int mrg_solve_pcg(mrg_problem* p, const void* J, int32_t fp32, const double* b, double* x, double rtol,
                             int32_t maxiter, mrg_solve_stats* st, mrg_stream_t stream) {
  if (!p || !J || !b || !x) return mrg_fail(MRG_EINVAL, "mrg_solve_pcg: null argument");
  if (!(rtol >= 0.0) || maxiter < 0) return mrg_fail(MRG_EINVAL, "mrg_solve_pcg: bad tolerance or iteration limit");
  cudaStream_t s = (cudaStream_t)stream;
  p->last_stream = s;
  if (mrg_gmg_kind(p) == MRG_PREC_GMG) {
    // multigrid CG on the correction: dx solves J dx = b - J x0, then x = x0 + dx
    int rc = ensure_work(p, true, false, s);
    if (rc) return rc;
    SolverWork* w = p->work;
    rc = mrg_spmv(p, J, fp32, x, w->r, stream);
    if (rc) return rc;
    k_b_minus<<<nblk(p->ndof, 256), 256, 0, s>>>(p->ndof, b, w->r);
    MRG_CUDA(cudaGetLastError());
    rc = mrg_gmg_solve(p, J, fp32 != 0, w->r, w->z, rtol, maxiter, st, false, s);
    if (rc && rc != MRG_ENOCONV) return rc;
    k_axpy<<<nblk(p->ndof, 256), 256, 0, s>>>(p->ndof, 1.0, w->z, x);
    MRG_CUDA(cudaGetLastError());
    MRG_CUDA(cudaStreamSynchronize(s));
    return rc;
  }
  if (!fp32) return pcg64(p, (const double*)J, b, x, rtol, maxiter, st, s);
  // FP32 matrix: solve J dx = b - J x0 in FP32, then x = x0 + dx
  int rc = ensure_work(p, true, true, s);
  if (rc) return rc;
  SolverWork* w = p->work;
  double* res = w->r;  // b - J x0
  rc = mrg_spmv(p, J, 1, x, res, stream);
  if (rc) return rc;
  const unsigned nb = nblk(p->ndof, 256);
  // z = b - J x0
  MRG_CUDA(cudaMemcpyAsync(w->z, b, p->ndof * sizeof(double), cudaMemcpyDeviceToDevice, s));
  k_axpy<<<nb, 256, 0, s>>>(p->ndof, -1.0, res, w->z);
  MRG_CUDA(cudaGetLastError());
  rc = pcg32(p, (const float*)J, w->z, rtol, maxiter, st, s);
  if (rc) return rc;
  k_add_f32<<<nb, 256, 0, s>>>(p->ndof, w->x32, x);
  MRG_CUDA(cudaGetLastError());
  MRG_CUDA(cudaStreamSynchronize(s));
  return MRG_OK;
}


int mrg_residual_from(mrg_problem* p, const double* b, double* res, cudaStream_t s) {
  k_b_minus<<<nblk(p->ndof, 256), 256, 0, s>>>(p->ndof, b, res);
  MRG_CUDA(cudaGetLastError());
  return MRG_OK;
}

static int norm_inf(mrg_problem* p, const double* v, double* out, cudaStream_t s) {
  SolverWork* w = p->work;
  k_norminf<<<pcg_grid(p), ST, 0, s>>>(p->ndof, v, w->parts, w->s);
  MRG_CUDA(cudaGetLastError());
  MRG_CUDA(cudaMemcpyAsync(w->h_s, w->s, sizeof(PcgScal), cudaMemcpyDeviceToHost, s));
  MRG_CUDA(cudaStreamSynchronize(s));
  *out = w->h_s->rnorm;
  return MRG_OK;
}

extern "C" int mrg_newton(mrg_problem* p, double* u, const mrg_newton_opts* o, mrg_solve_stats* st,
                          mrg_stream_t stream) {
  if (!p || !u || !o) return mrg_fail(MRG_EINVAL, "mrg_newton: null argument");
  if (o->max_iters < 1 || !(o->nl_tol > 0.0)) return mrg_fail(MRG_EINVAL, "mrg_newton: bad options");
  cudaStream_t s = (cudaStream_t)stream;
  p->last_stream = s;
  const bool mixed = o->mixed != 0;
  int rc = ensure_work(p, true, mixed, s);
  if (rc) return rc;
  SolverWork* w = p->work;
  if (!w->F) {
    MRG_CUDA(cudaMallocAsync(&w->F, p->ndof * sizeof(double), s));
    MRG_CUDA(cudaMallocAsync(&w->du, p->ndof * sizeof(double), s));
  }
  if (mixed && !w->J32) MRG_CUDA(cudaMallocAsync(&w->J32, p->nnz * sizeof(float), s));
  if (!mixed && !w->J64) MRG_CUDA(cudaMallocAsync(&w->J64, p->nnz * sizeof(double), s));
  void* J = mixed ? (void*)w->J32 : (void*)w->J64;
  const uint32_t jflags = MRG_ASM_JAC | MRG_ASM_OVERWRITE | (mixed ? MRG_ASM_J_FP32 : 0u);
  rc = mrg_set_dirichlet(p, u, stream);
  if (rc) return rc;
  double first = 0.0, scaled = 1.0, nrm = 0.0, alpha = 1.0;
  int it = 0, cgtot = 0;
  int full_iters = -1, last_iters = 0;  // Krylov iterations after the last full multigrid setup / last solve
  bool proceed = true, have_J = false, have_du = false;
  int status = MRG_OK;
  while (proceed) {
    // residual (assembleRes, FP64), inf norm (solverManager_solvers.hpp:380-390)
    rc = mrg_assemble(p, u, w->F, nullptr, MRG_ASM_RES | MRG_ASM_OVERWRITE, stream);
    if (rc) return rc;
    rc = norm_inf(p, w->F, &nrm, s);
    if (rc) return rc;
    if (!std::isfinite(nrm)) { status = MRG_ENUMERIC; break; }
    bool solve = true;
    if (it == 0) { first = nrm; scaled = 1.0; } else scaled = (first > 0.0) ? nrm / first : 0.0;
    if (it > 0 && scaled > 1.1 && have_du) {
      // backtracking (solverManager_solvers.hpp:416-429): u -= alpha*du, alpha halves
      alpha *= 0.5;
      k_axpy<<<nblk(p->ndof, 256), 256, 0, s>>>(p->ndof, -alpha, w->du, u);
      MRG_CUDA(cudaGetLastError());
      solve = false;
    } else if (scaled < o->nl_tol || nrm < 1.0e-100) {
      solve = false;
      proceed = false;
    }
    if (solve) {
      // The thermal form is linear in u (kappa and any weak-Dirichlet face terms do not depend on u), so
      // its Jacobian is the same at every Newton step of this call: assemble it once.  The 1+u^2 form is
      // re-assembled every step unless reuse_jacobian asks otherwise.
      const bool fresh = !have_J || (!o->reuse_jacobian && p->kind != MRG_THERMAL);
      if (fresh) {
        rc = mrg_assemble(p, u, nullptr, J, jflags, stream);
        if (rc) return rc;
        have_J = true;
      }
      mrg_solve_stats ls{};
      // the 1+u^2 Jacobian is nonsymmetric (2 u phi_j grad u . grad phi_i): BiCGStab; CG otherwise
      const bool bicg = (o->krylov == MRG_KRYLOV_BICGSTAB) || (o->krylov == MRG_KRYLOV_AUTO && p->kind != MRG_THERMAL);
      if (mrg_gmg_kind(p) == MRG_PREC_GMG) {
        // A re-assembled J gets a full multigrid setup at the first solve and whenever the previous solve
        // needed more Krylov iterations than the one right after the last full setup; otherwise only level 0
        // follows J and the coarse Galerkin operators are kept (their setup costs more than a Krylov
        // iteration; late Newton steps change J little).  opts.gmg_full_setup forces a full setup.
        int setup = MRG_GMG_SETUP_REUSE;
        if (fresh)
          setup = (o->gmg_full_setup || full_iters < 0 || last_iters > full_iters) ? MRG_GMG_SETUP_FULL
                                                                                     : MRG_GMG_SETUP_LEVEL0;
        rc = bicg ? mrg_gmg_bicgstab(p, J, mixed, w->F, w->du, o->lin_tol, o->lin_maxiter, &ls, setup, s)
                  : mrg_gmg_solve(p, J, mixed, w->F, w->du, o->lin_tol, o->lin_maxiter, &ls, setup, s);
        if (rc && rc != MRG_ENOCONV && !(bicg && rc == MRG_ENUMERIC)) return rc;
        if (setup == MRG_GMG_SETUP_FULL) full_iters = ls.iterations;
        last_iters = ls.iterations;
      } else if (!mixed) {
        MRG_CUDA(cudaMemsetAsync(w->du, 0, p->ndof * sizeof(double), s));
        rc = bicg ? mrg_bicg_solve64(p, w->J64, w->F, w->du, o->lin_tol, o->lin_maxiter, &ls, s)
                  : pcg64(p, w->J64, w->F, w->du, o->lin_tol, o->lin_maxiter, &ls, s);
        if (rc && rc != MRG_ENOCONV && !(bicg && rc == MRG_ENUMERIC)) return rc;
      } else if (bicg) {
        const float* d = nullptr;
        rc = mrg_bicg_solve32(p, w->J32, w->F, o->lin_tol, o->lin_maxiter, &ls, &d, s);
        if (rc && rc != MRG_ENOCONV && rc != MRG_ENUMERIC) return rc;
        k_f32_to_f64<<<nblk(p->ndof, 256), 256, 0, s>>>(p->ndof, d, w->du);
        MRG_CUDA(cudaGetLastError());
      } else {
        rc = pcg32(p, w->J32, w->F, o->lin_tol, o->lin_maxiter, &ls, s);
        if (rc) return rc;
        k_f32_to_f64<<<nblk(p->ndof, 256), 256, 0, s>>>(p->ndof, w->x32, w->du);
        MRG_CUDA(cudaGetLastError());
      }
      cgtot += ls.iterations;
      alpha = 1.0;
      k_axpy<<<nblk(p->ndof, 256), 256, 0, s>>>(p->ndof, 1.0, w->du, u);
      MRG_CUDA(cudaGetLastError());
      have_du = true;
    }
    it++;
    if (it >= o->max_iters) proceed = false;
  }
  MRG_CUDA(cudaStreamSynchronize(s));
  if (st) {
    st->iterations = cgtot;
    st->outer_iterations = it;
    st->rel_residual = scaled;
    st->abs_residual = nrm;
    st->status = status;
  }
  if (status != MRG_OK) return mrg_fail(status, "Newton: non-finite residual");
  if (!(scaled < o->nl_tol) && nrm >= 1.0e-100) {
    if (st) st->status = MRG_ENOCONV;
    return mrg_fail(MRG_ENOCONV, "Newton: not converged within max_iters");
  }
  return MRG_OK;
}

// ------------------------------------------------------------------------------------------------
// PCG that allocates nothing (mrg_solve_pcg_noalloc).
//
// Some callers cannot call cudaMalloc: a runtime that owns all device memory and admits work
// against a fixed HBM budget, a host framework whose pool allocator must be the only one, or a
// latency-critical loop where an allocation (and the implicit synchronisation cudaMalloc/cudaFree
// may bring) is not acceptable.  This entry point runs the same Jacobi PCG iteration as
// mrg_solve_pcg on an FP64 Jacobian, but keeps every work vector, the per-block partial sums and the
// device scalars in one file-scope __device__ array of fixed size instead of library-allocated
// workspace, and reads the scalars back into a host stack variable instead of pinned memory.
//
// Limits and sharing rules:
//   * at most MRG_NOALLOC_MAX_DOFS unknowns; larger problems are rejected with MRG_EINVAL;
//   * the array (about 10.5 MB) is part of the module image: every GPU that loads the library
//     holds it until the process exits;
//   * all calls share the one array and it keeps the last call's contents; the scalars (including
//     the reduction counter) are re-initialised by every call, the vectors are fully rewritten;
//   * calls whose GPU work overlaps (different streams, or different host threads) race on the
//     array: serialise them;
//   * the first call on a device looks up the array's device address (cudaGetSymbolAddress) with
//     that device current; make that first call before any stream capture on the device.
// ------------------------------------------------------------------------------------------------

namespace {
constexpr int64_t NA_N = MRG_NOALLOC_MAX_DOFS;
constexpr int64_t NA_PARTS = 3 * ((NA_N + ST - 1) / ST) + 64;
struct NoAllocScratch {
  double vec[5][NA_N];  // r, z, p, q, 1/diag
  double parts[NA_PARTS];
  PcgScal scal;
};

__global__ void k_na_init_scal(PcgScal* s, double tol, int maxiter) {
  PcgScal z{};
  z.tol = tol;
  z.maxiter = maxiter;
  *s = z;  // also clears the last-block counter left by the previous call
}
}  // namespace

static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

static std::mutex g_na_mutex;
static NoAllocScratch* g_na_addr[256] = {nullptr};

static int noalloc_scratch(NoAllocScratch** out) {
  int dev = 0;
  MRG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 256) return mrg_fail(MRG_EINVAL, "mrg_solve_pcg_noalloc: device ordinal out of range");
  std::lock_guard<std::mutex> lk(g_na_mutex);
  if (!g_na_addr[dev]) {
    void* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess) return mrg_cuda_check(e, "cudaGetSymbolAddress(no-alloc PCG scratch)");
    g_na_addr[dev] = static_cast<NoAllocScratch*>(ptr);
  }
  *out = g_na_addr[dev];
  return MRG_OK;
}

extern "C" int mrg_solve_pcg_noalloc(mrg_problem* p, const double* J, const double* b, double* x, double rtol,
                                     int32_t maxiter, mrg_solve_stats* st, mrg_stream_t stream) {
  if (!p || !J || !b || !x) return mrg_fail(MRG_EINVAL, "mrg_solve_pcg_noalloc: null argument");
  if (!(rtol >= 0.0) || maxiter < 0)
    return mrg_fail(MRG_EINVAL, "mrg_solve_pcg_noalloc: bad tolerance or iteration limit");
  if (p->ndof > NA_N)
    return mrg_fail(MRG_EINVAL, "mrg_solve_pcg_noalloc: problem has " + std::to_string(p->ndof) +
                                    " DOFs, above the fixed scratch limit MRG_NOALLOC_MAX_DOFS = " +
                                    std::to_string((long long)NA_N));
  NoAllocScratch* S = nullptr;
  int rc = noalloc_scratch(&S);
  if (rc) return rc;
  // the SpMV stages two CSR tiles in more than 48 KB of dynamic shared memory
  MRG_CUDA(cudaFuncSetAttribute(k_pcg64_spmv<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, spmv_smem<1, double>()));
  cudaStream_t s = (cudaStream_t)stream;
  PcgVec64 V{x, S->vec[0], S->vec[1], S->vec[2], S->vec[3], S->vec[4], S->parts, b, J, &S->scal};
  k_na_init_scal<<<1, 1, 0, s>>>(&S->scal, rtol, maxiter);
  const unsigned nb = pcg_grid(p);
  if (p->g.p == 1) k_pcg64_init<1><<<nb, ST, 0, s>>>(p->g, p->ndof, V);
  else k_pcg64_init<2><<<nb, ST, 0, s>>>(p->g, p->ndof, V);
  MRG_CUDA(cudaGetLastError());
  PcgScal h{};
  const int max_chunks = maxiter / CHUNK + 2;
  for (int c = 0; c < max_chunks; ++c) {
    if (p->g.p == 1) enqueue_chunk64<1>(p, V, s);
    else enqueue_chunk64<2>(p, V, s);
    MRG_CUDA(cudaGetLastError());
    MRG_CUDA(cudaMemcpyAsync(&h, &S->scal, sizeof(PcgScal), cudaMemcpyDeviceToHost, s));
    MRG_CUDA(cudaStreamSynchronize(s));
    if (h.done) break;
  }
  if (st) {
    st->iterations = h.iter;
    st->outer_iterations = 0;
    st->rel_residual = (h.r0 > 0) ? h.rnorm / h.r0 : 0.0;
    st->abs_residual = h.rnorm;
    st->status = h.status;
  }
  if (h.status != MRG_OK) return mrg_fail(h.status, pcg_status_text("PCG (no-alloc)", h.status));
  if (h.r0 > 0 && h.rnorm / h.r0 > rtol) {
    if (st) st->status = MRG_ENOCONV;
    return mrg_fail(MRG_ENOCONV, "PCG (no-alloc): maximum iterations reached before the tolerance");
  }
  return MRG_OK;
}
