// Jacobi-preconditioned BiCGStab on the assembled system, for the nonsymmetric Jacobians of the
// nonlinear form -div((1+u^2) grad u) (the 2 u phi_j grad u . grad phi_i term makes J nonsymmetric,
// where CG is not guaranteed to converge).  The reference reaches the same method through Belos
// ("Belos solver: BiCGStab", src/interfaces/linear_algebra/linearAlgebraInterface_solvers.hpp:108-110).
//
// Right-preconditioned BiCGStab (van der Vorst), M = diag(J):
//   p = r + beta (p - omega v);  ph = M^-1 p;  v = J ph;  alpha = rho / (rh . v)
//   s = r - alpha v;  sh = M^-1 s;  t = J sh;  omega = (t . s) / (t . t)
//   x += alpha ph + omega sh;  r = s - omega t;  rho' = rh . r;  beta = (rho'/rho)(alpha/omega)
// Five kernels per iteration (two SpMVs); every dot product is reduced deterministically by the
// last-block pattern; the scalars live on the device and a chunk of iterations is replayed as a CUDA
// graph, exactly like the PCG.  FP64 vectors for an FP64 Jacobian; FP32 vectors (FP64 block sums of
// the dots) for the FP32 Jacobian of the mixed-precision Newton.
#include <cmath>

#include "mrg_device.cuh"

using namespace mrgdev;

namespace {

constexpr int BT = 128;
constexpr int BCHUNK = 8;

struct BScal {
  double rho, rho_old, alpha, omega, beta, r0, rnorm, tol;
  double rv, ts, tt;
  int iter, maxiter, done, status;
  unsigned int counter;
  int pad;
};

template <typename VT, typename JT>
struct BVec {
  VT *x, *r, *rh, *p, *v, *ph, *s, *sh, *t, *minv;
  double* parts;
  const double* b;
  const JT* J;
  BScal* S;
};

#define BDONE(V) (((volatile BScal*)(V).S)->done)
#define GSTRIDE(n) for (int64_t n = (int64_t)blockIdx.x * BT + threadIdx.x; n < nrows; n += (int64_t)gridDim.x * BT)

template <int P, typename VT, typename JT>
__global__ void __launch_bounds__(BT) k_b_init(Grid g, int64_t nrows, BVec<VT, JT> V, int x0_zero) {
  double rr = 0.0;
  GSTRIDE(n) {
    int ix, iy, iz;
    decompose(g, n, ix, iy, iz);
    const RowInfo R = row_info<P>(g, ix, iy, iz);
    const VT d = (VT)V.J[diag_pos(R, ix, iy, iz)];
    const VT ax = x0_zero ? VT(0) : row_dot<P, JT, VT, VT>(g, R, V.J + R.rp, V.x);
    if (x0_zero) V.x[n] = VT(0);
    const VT r = (VT)V.b[n] - ax;
    V.r[n] = r;
    V.rh[n] = r;
    V.p[n] = VT(0);
    V.v[n] = VT(0);
    V.minv[n] = VT(1) / d;
    rr += (double)(r * r);
  }
  double m[1] = {block_sum(rr)};
  if (last_block<1>(V.parts, m, &V.S->counter)) {
    double t[1];
    sum_parts<1>(V.parts, t, &V.S->counter);
    if (threadIdx.x == 0) {
      BScal* S = V.S;
      S->r0 = sqrt(t[0]);
      S->rnorm = S->r0;
      S->rho = t[0];
      S->alpha = 1.0;
      S->omega = 1.0;
      S->beta = 0.0;
      S->iter = 0;
      S->status = MRG_OK;
      S->done = (S->r0 == 0.0 || S->maxiter <= 0) ? 1 : 0;
      if (!isfinite(S->r0)) { S->done = 1; S->status = MRG_ENUMERIC; }
    }
  }
}

// p = r + beta (p - omega v); ph = M^-1 p
template <typename VT, typename JT>
__global__ void __launch_bounds__(BT) k_b_dir(int64_t nrows, BVec<VT, JT> V) {
  if (BDONE(V)) return;
  const VT beta = (VT)V.S->beta, omega = (VT)V.S->omega;
  GSTRIDE(n) {
    const VT p = V.r[n] + beta * (V.p[n] - omega * V.v[n]);
    V.p[n] = p;
    V.ph[n] = V.minv[n] * p;
  }
}

// out = J in ; partial (a . out) [and (out . out)] ; last block runs the scalar step
template <int P, int STEP, typename VT, typename JT>
__global__ void __launch_bounds__(BT) k_b_spmv(Grid g, int64_t nrows, BVec<VT, JT> V) {
  if (BDONE(V)) return;
  const VT* in = (STEP == 0) ? V.ph : V.sh;
  VT* out = (STEP == 0) ? V.v : V.t;
  VT d0 = VT(0), d1 = VT(0);  // per-thread partials in the vector precision, block sums in FP64
  GSTRIDE(n) {
    int ix, iy, iz;
    decompose(g, n, ix, iy, iz);
    const RowInfo R = row_info<P>(g, ix, iy, iz);
    const VT y = row_dot<P, JT, VT, VT>(g, R, V.J + R.rp, in);
    out[n] = y;
    if (STEP == 0) {
      d0 = fma(V.rh[n], y, d0);
    } else {
      d0 = fma(y, V.s[n], d0);
      d1 = fma(y, y, d1);
    }
  }
  double m[2] = {block_sum((double)d0), block_sum((double)d1)};
  if (last_block<2>(V.parts, m, &V.S->counter)) {
    double t[2];
    sum_parts<2>(V.parts, t, &V.S->counter);
    if (threadIdx.x == 0) {
      BScal* S = V.S;
      if (STEP == 0) {
        S->rv = t[0];
        S->alpha = S->rho / t[0];
        if (!(t[0] != 0.0) || !isfinite(S->alpha)) { S->status = MRG_ENUMERIC; S->done = 1; }
      } else {
        S->ts = t[0];
        S->tt = t[1];
        S->omega = (t[1] > 0.0) ? t[0] / t[1] : 0.0;
      }
    }
  }
}

// s = r - alpha v; sh = M^-1 s
template <typename VT, typename JT>
__global__ void __launch_bounds__(BT) k_b_s(int64_t nrows, BVec<VT, JT> V) {
  if (BDONE(V)) return;
  const VT alpha = (VT)V.S->alpha;
  GSTRIDE(n) {
    const VT s = V.r[n] - alpha * V.v[n];
    V.s[n] = s;
    V.sh[n] = V.minv[n] * s;
  }
}

// x += alpha ph + omega sh; r = s - omega t; partial r.r, rh.r; last block: rho, beta, stopping test
template <typename VT, typename JT>
__global__ void __launch_bounds__(BT) k_b_update(int64_t nrows, BVec<VT, JT> V) {
  if (BDONE(V)) return;
  const VT alpha = (VT)V.S->alpha, omega = (VT)V.S->omega;
  VT rr = VT(0), rhr = VT(0);
  GSTRIDE(n) {
    V.x[n] += alpha * V.ph[n] + omega * V.sh[n];
    const VT r = V.s[n] - omega * V.t[n];
    V.r[n] = r;
    rr = fma(r, r, rr);
    rhr = fma(V.rh[n], r, rhr);
  }
  double m[2] = {block_sum((double)rr), block_sum((double)rhr)};
  if (last_block<2>(V.parts, m, &V.S->counter)) {
    double t[2];
    sum_parts<2>(V.parts, t, &V.S->counter);
    if (threadIdx.x == 0) {
      BScal* S = V.S;
      S->rnorm = sqrt(t[0]);
      S->rho_old = S->rho;
      S->rho = t[1];
      S->iter += 1;
      if (!isfinite(S->rnorm)) {
        S->done = 1;
        S->status = MRG_ENUMERIC;
      } else if (!(S->rnorm / S->r0 > S->tol) || S->iter >= S->maxiter) {
        S->done = 1;
      } else if (S->rho == 0.0 || S->omega == 0.0) {
        S->done = 1;  // breakdown before convergence
        S->status = MRG_ENUMERIC;
      } else {
        S->beta = (S->rho / S->rho_old) * (S->alpha / S->omega);
      }
    }
  }
}

inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

unsigned b_grid(const mrg_problem* p) {
  const unsigned tiles = nblk(p->ndof, BT), cap = (unsigned)(16 * mrg_device_sms());
  return tiles < cap ? tiles : cap;
}

template <int P, typename VT, typename JT>
void enqueue_iters(const mrg_problem* p, const BVec<VT, JT>& V, cudaStream_t s) {
  const unsigned nb = b_grid(p);
  for (int it = 0; it < BCHUNK; ++it) {
    k_b_dir<VT, JT><<<nb, BT, 0, s>>>(p->ndof, V);
    k_b_spmv<P, 0, VT, JT><<<nb, BT, 0, s>>>(p->g, p->ndof, V);
    k_b_s<VT, JT><<<nb, BT, 0, s>>>(p->ndof, V);
    k_b_spmv<P, 1, VT, JT><<<nb, BT, 0, s>>>(p->g, p->ndof, V);
    k_b_update<VT, JT><<<nb, BT, 0, s>>>(p->ndof, V);
  }
}

}  // namespace

struct BicgWork {
  void* v64[9] = {};   // r, rh, p, v, ph, s, sh, t, minv (FP64)
  void* v32[10] = {};  // x + the nine above (FP32)
  double* parts = nullptr;
  BScal* S = nullptr;
  cudaGraphExec_t g[2] = {nullptr, nullptr};
  const void* key[2][3] = {{nullptr, nullptr, nullptr}, {nullptr, nullptr, nullptr}};
  cudaStream_t gs[2] = {nullptr, nullptr};
};

void mrg_bicg_drop_graphs(mrg_problem* p) {
  BicgWork* w = reinterpret_cast<BicgWork*>(p->bicg);
  if (!w) return;
  for (int k = 0; k < 2; ++k) {
    if (w->g[k]) cudaGraphExecDestroy(w->g[k]);
    w->g[k] = nullptr;
  }
}

void mrg_bicg_free(mrg_problem* p) {
  BicgWork* w = reinterpret_cast<BicgWork*>(p->bicg);
  if (!w) return;
  for (int k = 0; k < 2; ++k)
    if (w->g[k]) cudaGraphExecDestroy(w->g[k]);
  for (void* ptr : w->v64)
    if (ptr) cudaFreeAsync(ptr, p->stream);
  for (void* ptr : w->v32)
    if (ptr) cudaFreeAsync(ptr, p->stream);
  if (w->parts) cudaFreeAsync(w->parts, p->stream);
  if (w->S) cudaFreeAsync(w->S, p->stream);
  delete w;
  p->bicg = nullptr;
}

static int bicg_ensure(mrg_problem* p, bool fp32, cudaStream_t s) {
  if (!p->bicg) p->bicg = new BicgWork();
  BicgWork* w = reinterpret_cast<BicgWork*>(p->bicg);
  const int64_t n = p->ndof;
  if (!w->parts) MRG_CUDA(cudaMallocAsync(&w->parts, (2 * (size_t)nblk(n, BT) + 64) * sizeof(double), s));
  if (!w->S) MRG_CUDA(cudaMallocAsync(&w->S, sizeof(BScal), s));
  if (!fp32 && !w->v64[0])
    for (auto& ptr : w->v64) MRG_CUDA(cudaMallocAsync(&ptr, n * sizeof(double), s));
  if (fp32 && !w->v32[0])
    for (auto& ptr : w->v32) MRG_CUDA(cudaMallocAsync(&ptr, n * sizeof(float), s));
  return MRG_OK;
}

template <typename VT, typename JT>
static int bicg_run(mrg_problem* p, const JT* J, const double* b, VT* x, bool x0_zero, double rtol, int maxiter,
                    mrg_solve_stats* st, cudaStream_t s) {
  const bool fp32 = sizeof(VT) == 4;
  int rc = bicg_ensure(p, fp32, s);
  if (rc) return rc;
  BicgWork* w = reinterpret_cast<BicgWork*>(p->bicg);
  VT* const* v = fp32 ? reinterpret_cast<VT* const*>(w->v32 + 1) : reinterpret_cast<VT* const*>(w->v64);
  BVec<VT, JT> V{x, v[0], v[1], v[2], v[3], v[4], v[5], v[6], v[7], v[8], w->parts, b, J, w->S};
  BScal init{};
  init.tol = rtol;
  init.maxiter = maxiter;
  MRG_CUDA(cudaMemcpyAsync(w->S, &init, sizeof(BScal), cudaMemcpyHostToDevice, s));
  const unsigned nb = b_grid(p);
  if (p->g.p == 1) k_b_init<1, VT, JT><<<nb, BT, 0, s>>>(p->g, p->ndof, V, x0_zero ? 1 : 0);
  else k_b_init<2, VT, JT><<<nb, BT, 0, s>>>(p->g, p->ndof, V, x0_zero ? 1 : 0);
  MRG_CUDA(cudaGetLastError());
  // chunk graph (captured once per buffers / stream)
  const int gi = fp32 ? 1 : 0;
  if (!(w->g[gi] && w->key[gi][0] == J && w->key[gi][1] == b && w->key[gi][2] == x && w->gs[gi] == s)) {
    if (w->g[gi]) cudaGraphExecDestroy(w->g[gi]);
    w->g[gi] = nullptr;
    cudaStream_t cs = s;
    bool own = false;
    if (!s) {
      MRG_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
      own = true;
    }
    cudaGraph_t graph;
    MRG_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
    if (p->g.p == 1) enqueue_iters<1, VT, JT>(p, V, cs);
    else enqueue_iters<2, VT, JT>(p, V, cs);
    cudaError_t e = cudaStreamEndCapture(cs, &graph);
    if (own) cudaStreamDestroy(cs);
    if (e != cudaSuccess) return mrg_cuda_check(e, "capture BiCGStab chunk");
    e = cudaGraphInstantiate(&w->g[gi], graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return mrg_cuda_check(e, "instantiate BiCGStab chunk");
    w->key[gi][0] = J;
    w->key[gi][1] = b;
    w->key[gi][2] = x;
    w->gs[gi] = s;
  }
  BScal h{};
  const int max_chunks = maxiter / BCHUNK + 2;
  for (int c = 0; c < max_chunks; ++c) {
    MRG_CUDA(cudaGraphLaunch(w->g[gi], s));
    MRG_CUDA(cudaMemcpyAsync(&h, w->S, sizeof(BScal), cudaMemcpyDeviceToHost, s));
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
  if (h.status != MRG_OK && !(h.r0 > 0 && h.rnorm / h.r0 <= rtol))
    return mrg_fail(h.status, "BiCGStab: breakdown (rho or omega or (rh . v) vanished) before convergence");
  if (h.r0 > 0 && h.rnorm / h.r0 > rtol) {
    if (st) st->status = MRG_ENOCONV;
    return mrg_fail(MRG_ENOCONV, "BiCGStab: maximum iterations reached before the tolerance");
  }
  if (st) st->status = MRG_OK;
  return MRG_OK;
}

// FP32 solve J32 d = b with d0 = 0; the correction is left in the work vector returned by *d.
int mrg_bicg_solve32(mrg_problem* p, const float* J32, const double* b, double rtol, int maxiter,
                     mrg_solve_stats* st, const float** d, cudaStream_t s) {
  int rc = bicg_ensure(p, true, s);
  if (rc) return rc;
  BicgWork* w = reinterpret_cast<BicgWork*>(p->bicg);
  float* x32 = reinterpret_cast<float*>(w->v32[0]);
  *d = x32;
  return bicg_run<float, float>(p, J32, b, x32, true, rtol, maxiter, st, s);
}

int mrg_bicg_solve64(mrg_problem* p, const double* J, const double* b, double* x, double rtol, int maxiter,
                     mrg_solve_stats* st, cudaStream_t s) {
  return bicg_run<double, double>(p, J, b, x, false, rtol, maxiter, st, s);
}

__global__ void k_b_add(int64_t n, const double* __restrict__ d, double* __restrict__ x) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] += d[i];
}

__global__ void k_b_addf(int64_t n, const float* __restrict__ d, double* __restrict__ x) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] += (double)d[i];
}

extern "C" int mrg_solve_bicgstab(mrg_problem* p, const void* J, int32_t fp32, const double* b, double* x,
                                  double rtol, int32_t maxiter, mrg_solve_stats* st, mrg_stream_t stream) {
  if (!p || !J || !b || !x) return mrg_fail(MRG_EINVAL, "mrg_solve_bicgstab: null argument");
  if (!(rtol >= 0.0) || maxiter < 0) return mrg_fail(MRG_EINVAL, "mrg_solve_bicgstab: bad tolerance or iteration limit");
  cudaStream_t s = (cudaStream_t)stream;
  p->last_stream = s;
  if (mrg_gmg_kind(p) == MRG_PREC_GMG) {
    // multigrid-preconditioned BiCGStab on the correction: J dx = b - J x, x += dx
    double *res = nullptr, *dx = nullptr;
    MRG_CUDA(cudaMallocAsync(&res, p->ndof * sizeof(double), s));
    MRG_CUDA(cudaMallocAsync(&dx, p->ndof * sizeof(double), s));
    int rc = mrg_spmv(p, J, fp32, x, res, stream);
    if (rc == MRG_OK) rc = mrg_residual_from(p, b, res, s);
    if (rc == MRG_OK) rc = mrg_gmg_bicgstab(p, J, fp32 != 0, res, dx, rtol, maxiter, st, false, s);
    if (rc == MRG_OK || rc == MRG_ENOCONV) {
      k_b_add<<<nblk(p->ndof, 256), 256, 0, s>>>(p->ndof, dx, x);
      cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess && rc == MRG_OK) rc = mrg_cuda_check(e, "BiCGStab update");
    }
    cudaFreeAsync(res, s);
    cudaFreeAsync(dx, s);
    cudaStreamSynchronize(s);
    return rc;
  }
  if (!fp32) return mrg_bicg_solve64(p, (const double*)J, b, x, rtol, maxiter, st, s);
  // FP32 matrix: the correction of x from J32 d = b - J32 x (residual formed in FP64 by the SpMV)
  double* res = nullptr;
  MRG_CUDA(cudaMallocAsync(&res, p->ndof * sizeof(double), s));
  int rc = mrg_spmv(p, J, 1, x, res, stream);
  if (rc == MRG_OK) {
    rc = mrg_residual_from(p, b, res, s);  // res = b - res
  }
  const float* d = nullptr;
  if (rc == MRG_OK) rc = mrg_bicg_solve32(p, (const float*)J, res, rtol, maxiter, st, &d, s);
  if (rc == MRG_OK || rc == MRG_ENOCONV) {
    k_b_addf<<<nblk(p->ndof, 256), 256, 0, s>>>(p->ndof, d, x);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess && rc == MRG_OK) rc = mrg_cuda_check(e, "BiCGStab update");
  }
  cudaFreeAsync(res, s);
  cudaStreamSynchronize(s);
  return rc;
}
