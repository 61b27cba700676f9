// Problem lifetime, structure queries, coefficients, Dirichlet data and the assembly dispatcher
// of the C ABI declared in include/mrhyde_gb300.h.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "mrg_internal.h"

// ------------------------------------------------------------------------------------------------
// errors
// ------------------------------------------------------------------------------------------------
static thread_local std::string g_last_error;

void mrg_set_error(const std::string& msg) { g_last_error = msg; }
int mrg_fail(int status, const std::string& msg) {
  g_last_error = msg;
  return status;
}
int mrg_cuda_check(cudaError_t e, const char* what) {
  g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
  return (e == cudaErrorMemoryAllocation) ? MRG_ENOMEM : MRG_ECUDA;
}

// ------------------------------------------------------------------------------------------------
// pinned slot pool
// ------------------------------------------------------------------------------------------------
namespace {
constexpr size_t PIN_SLOT = 256, PIN_CHUNK = 64 * 1024;
std::mutex g_pin_mu;
std::vector<void*> g_pin_free;
}  // namespace

void* mrg_pinned_slot() {
  std::lock_guard<std::mutex> lk(g_pin_mu);
  if (g_pin_free.empty()) {
    void* chunk = nullptr;
    if (cudaMallocHost(&chunk, PIN_CHUNK) != cudaSuccess) return nullptr;
    for (size_t off = 0; off < PIN_CHUNK; off += PIN_SLOT) g_pin_free.push_back((char*)chunk + off);
  }
  void* p = g_pin_free.back();
  g_pin_free.pop_back();
  std::memset(p, 0, PIN_SLOT);
  return p;
}

void mrg_pinned_release(void* p) {
  if (!p) return;
  std::lock_guard<std::mutex> lk(g_pin_mu);
  g_pin_free.push_back(p);
}

// ------------------------------------------------------------------------------------------------
// SM count of the current device, looked up once per device ordinal (safe from any host thread)
// ------------------------------------------------------------------------------------------------
namespace {
constexpr int SM_CACHE = 256;
std::atomic<int> g_sm_count[SM_CACHE];
}  // namespace

int mrg_device_sms() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) dev = -1;
  if (dev >= 0 && dev < SM_CACHE) {
    const int c = g_sm_count[dev].load(std::memory_order_relaxed);
    if (c > 0) return c;
  }
  int nsm = 0;
  if (dev < 0 || cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || nsm <= 0)
    return 148;  // conservative grid sizing when the query fails; not cached
  if (dev < SM_CACHE) g_sm_count[dev].store(nsm, std::memory_order_relaxed);
  return nsm;
}

extern "C" int mrg_last_error(char* buf, size_t len) {
  if (!buf || len == 0) return MRG_EINVAL;
  size_t n = g_last_error.size() < len - 1 ? g_last_error.size() : len - 1;
  std::memcpy(buf, g_last_error.data(), n);
  buf[n] = '\0';
  return MRG_OK;
}

extern "C" const char* mrg_version(void) { return "mrhyde_gb300 0.1 (sm_103a)"; }

// ------------------------------------------------------------------------------------------------
// host helpers: Gauss rule and Lagrange basis (same published algorithms as the reference's
// Intrepid2 DefaultCubatureFactory / HGRAD_*_Cn with equispaced nodes)
// ------------------------------------------------------------------------------------------------
static void gauss_rule(int order, std::vector<double>& x, std::vector<double>& w) {
  int n = order / 2 + 1;
  x.assign(n, 0.0);
  w.assign(n, 0.0);
  const double pi = 3.14159265358979323846;
  for (int i = 0; i < n; ++i) {
    double z = std::cos(pi * (i + 0.75) / (n + 0.5));
    double dp = 1.0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = z;
      for (int k = 2; k <= n; ++k) {
        double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      double pn = (n == 1) ? z : p1, pm = (n == 1) ? 1.0 : p0;
      dp = n * (z * pn - pm) / (z * z - 1.0);
      double dz = pn / dp;
      z -= dz;
      if (std::fabs(dz) < 1e-17) break;
    }
    double p0 = 1.0, p1 = z;
    for (int k = 2; k <= n; ++k) {
      double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
      p0 = p1;
      p1 = p2;
    }
    double pn = (n == 1) ? z : p1, pm = (n == 1) ? 1.0 : p0;
    dp = n * (z * pn - pm) / (z * z - 1.0);
    x[n - 1 - i] = z;
    w[n - 1 - i] = 2.0 / ((1.0 - z * z) * dp * dp);
  }
}

static void lagrange(int p, double xi, double* l, double* dl) {
  double nodes[8];
  for (int a = 0; a <= p; ++a) nodes[a] = -1.0 + 2.0 * a / p;
  for (int a = 0; a <= p; ++a) {
    double v = 1.0;
    for (int b = 0; b <= p; ++b)
      if (b != a) v *= (xi - nodes[b]) / (nodes[a] - nodes[b]);
    l[a] = v;
    double dv = 0.0;
    for (int k = 0; k <= p; ++k) {
      if (k == a) continue;
      double t = 1.0 / (nodes[a] - nodes[k]);
      for (int b = 0; b <= p; ++b)
        if (b != a && b != k) t *= (xi - nodes[b]) / (nodes[a] - nodes[b]);
      dv += t;
    }
    dl[a] = dv;
  }
}

void mrg_lagrange_1d(int p, double xi, double* l, double* dl) { lagrange(p, xi, l, dl); }

// ------------------------------------------------------------------------------------------------
// small kernels
// ------------------------------------------------------------------------------------------------
__device__ inline int64_t grid_row_ptr(const Grid& g, int ix, int iy, int iz) {
  int lo, cx, cy, cz;
  axis_range(ix, g.nn[0], g.p, lo, cx);
  axis_range(iy, g.nn[1], g.p, lo, cy);
  if (g.dim == 3) axis_range(iz, g.nn[2], g.p, lo, cz); else cz = 1;
  (void)lo;
  return g.P[2][iz] * g.T[1] * g.T[0] + (int64_t)cz * (g.P[1][iy] * g.T[0] + (int64_t)cy * g.P[0][ix]);
}

__global__ void k_graph(Grid g, int64_t nrows, int64_t* __restrict__ row_ptr, int32_t* __restrict__ col_idx) {
  int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n > nrows) return;
  if (n == nrows) {
    row_ptr[nrows] = g.T[0] * g.T[1] * g.T[2];
    return;
  }
  int ix = (int)(n % g.nn[0]);
  int64_t t = n / g.nn[0];
  int iy = (int)(t % g.nn[1]);
  int iz = (int)(t / g.nn[1]);
  int lx, ly, lz, cx, cy, cz;
  axis_range(ix, g.nn[0], g.p, lx, cx);
  axis_range(iy, g.nn[1], g.p, ly, cy);
  if (g.dim == 3) axis_range(iz, g.nn[2], g.p, lz, cz); else { lz = 0; cz = 1; }
  int64_t rp = grid_row_ptr(g, ix, iy, iz);
  row_ptr[n] = rp;
  int64_t k = rp;
  for (int z = lz; z < lz + cz; ++z)
    for (int y = ly; y < ly + cy; ++y)
      for (int x = lx; x < lx + cx; ++x) col_idx[k++] = x + g.nn[0] * (y + g.nn[1] * z);
}

__global__ void k_dof_map(Grid g, int64_t ncell, int npe, int32_t* __restrict__ lids) {
  int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ncell * npe) return;
  int64_t c = e / npe;
  int i = (int)(e % npe);
  int q = g.p + 1;
  int a = i % q, b = (i / q) % q, cc = (g.dim == 3) ? i / (q * q) : 0;
  int cx = (int)(c % g.nc[0]);
  int64_t t = c / g.nc[0];
  int cy = (int)(t % g.nc[1]);
  int cz = (int)(t / g.nc[1]);
  lids[e] = (g.p * cx + a) + g.nn[0] * ((g.p * cy + b) + g.nn[1] * (g.p * cz + cc));
}

__global__ void k_fill(double* __restrict__ a, int64_t n, double v) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) a[i] = v;
}

__global__ void k_set_dirichlet(const int32_t* __restrict__ dofs, const double* __restrict__ vals, int64_t n,
                                double* __restrict__ u) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) u[dofs[k]] = vals[k];
}

__global__ void k_copy_fixed(const int32_t* __restrict__ src, const double* __restrict__ sv, int64_t n,
                             int32_t* __restrict__ dofs, double* __restrict__ vals) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) {
    dofs[k] = src[k];
    if (vals) vals[k] = sv[k];
  }
}

static inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

// ------------------------------------------------------------------------------------------------
// create / destroy
// ------------------------------------------------------------------------------------------------
// Frees the handle's device memory in stream order on its creation stream, after the last stream the
// handle's work was enqueued on has drained (no device-wide synchronisation, so concurrent solves on
// other streams keep running).
static void free_problem(mrg_problem* p) {
  if (!p) return;
  cudaStream_t s = p->stream;
  if (p->last_stream != s) cudaStreamSynchronize(p->last_stream);
  mrg_solver_free(p);
  mrg_bicg_free(p);
  mrg_q2_free(p);
  mrg_boundary_free(p);
  mrg_gmg_free(p);
  cudaFreeAsync(p->d_prefix, s);
  cudaFreeAsync(p->d_kappa, s);
  cudaFreeAsync(p->d_kappa32, s);
  cudaFreeAsync(p->d_kappa_s, s);
  cudaFreeAsync(p->d_fixed, s);
  cudaFreeAsync(p->d_fixed_vals, s);
  cudaFreeAsync(p->d_vcoord, s);
  cudaFreeAsync(p->d_srcB, s);
  cudaFreeAsync(p->d_qtab, s);
  cudaFreeAsync(p->d_khat, s);
  cudaFreeAsync(p->d_khat32, s);
  cudaFreeAsync(p->d_bload, s);
  cudaStreamSynchronize(s);
  delete p;
}

static int create_impl(const mrg_mesh_desc* m, const mrg_physics_desc* ph, cudaStream_t cs, mrg_problem** out) {
  if (!m || !ph || !out) return mrg_fail(MRG_EINVAL, "mrg_problem_create: null argument");
  *out = nullptr;
  if (m->dim != 2 && m->dim != 3) return mrg_fail(MRG_EINVAL, "dim must be 2 or 3");
  if (m->order < 1 || m->order > 2) return mrg_fail(MRG_EINVAL, "order must be 1 or 2");
  if (m->nx < 1 || m->ny < 1 || (m->dim == 3 && m->nz < 1)) return mrg_fail(MRG_EINVAL, "cell counts must be >= 1");
  if (ph->kind != MRG_THERMAL && ph->kind != MRG_DIFFUSION_1PU2) return mrg_fail(MRG_EINVAL, "unknown physics kind");
  if (ph->source_kind != MRG_SRC_CONST && ph->source_kind != MRG_SRC_SINPROD)
    return mrg_fail(MRG_EINVAL, "unknown source kind");
  if (ph->dirichlet_kind == MRG_DBC_NODE && !ph->dirichlet_node)
    return mrg_fail(MRG_EINVAL, "dirichlet_node is null");
  for (int k = 0; k < m->dim; ++k)
    if (!(m->hi[k] > m->lo[k])) return mrg_fail(MRG_EINVAL, "box must have hi > lo on every axis");
  const int p = m->order;
  int64_t nn[3] = {(int64_t)p * m->nx + 1, (int64_t)p * m->ny + 1, m->dim == 3 ? (int64_t)p * m->nz + 1 : 1};
  int64_t ndof = nn[0] * nn[1] * nn[2];
  if (ndof > (int64_t)INT32_MAX) return mrg_fail(MRG_EINVAL, "mesh too large for 32-bit local ordinals");
  int qo = ph->quad_order > 0 ? ph->quad_order : 2 * p;
  if (qo > 14) return mrg_fail(MRG_EINVAL, "quadrature order above 14 not supported");

  mrg_problem* P = new mrg_problem();
  P->stream = cs;
  P->last_stream = cs;
  Grid& g = P->g;
  g.dim = m->dim;
  g.p = p;
  g.nc[0] = m->nx; g.nc[1] = m->ny; g.nc[2] = (m->dim == 3) ? m->nz : 1;
  for (int k = 0; k < 3; ++k) g.nn[k] = (int)nn[k];
  g.faces = ph->dirichlet_faces & (m->dim == 3 ? 63u : 15u);
  // per-axis prefix tables of coupling counts
  std::vector<int64_t> pref;
  int64_t offs[3];
  for (int k = 0; k < 3; ++k) {
    offs[k] = (int64_t)pref.size();
    int64_t acc = 0;
    pref.push_back(0);
    for (int i = 0; i < g.nn[k]; ++i) {
      int lo, cnt;
      if (k < m->dim) axis_range(i, g.nn[k], p, lo, cnt); else cnt = 1;
      acc += cnt;
      pref.push_back(acc);
    }
    g.T[k] = acc;
  }
  P->ndof = ndof;
  P->ncell = (int64_t)g.nc[0] * g.nc[1] * g.nc[2];
  P->nnz = g.T[0] * g.T[1] * g.T[2];
  P->npe = 1;
  for (int k = 0; k < m->dim; ++k) P->npe *= (p + 1);
  std::vector<double> gx, gw;
  gauss_rule(qo, gx, gw);
  int n1 = (int)gx.size();
  P->nq = 1;
  for (int k = 0; k < m->dim; ++k) P->nq *= n1;
  P->quad_order = qo;
  P->kind = ph->kind;
  P->source_kind = ph->source_kind;
  P->source_amp = ph->source_amp;
  P->source_freq = ph->source_freq;
  for (int k = 0; k < 3; ++k) {
    P->lo[k] = (k < m->dim) ? m->lo[k] : 0.0;
    P->hi[k] = (k < m->dim) ? m->hi[k] : 1.0;
    P->h[k] = (k < m->dim) ? (P->hi[k] - P->lo[k]) / g.nc[k] : 1.0;
  }
  P->gx1 = gx;
  P->gw1 = gw;
  P->affine = (m->vertex_coords == nullptr);
  if (P->affine && p == 1 && ph->kind == MRG_THERMAL && qo >= 2)
    P->path = MRG_PATH_FACTORED;
  else if (P->affine && m->dim == 3 && n1 == p + 1 && ph->source_kind == MRG_SRC_CONST &&
           (p == 2 || ph->kind == MRG_DIFFUSION_1PU2))
    P->path = MRG_PATH_TENSOR;
  else if (mrg_stored_eligible(m->dim, p, ph->kind, n1, P->affine))
    P->path = MRG_PATH_STORED;
  else
    P->path = MRG_PATH_CELL;

  auto fail_cuda = [&](cudaError_t e, const char* what) {
    int st = mrg_cuda_check(e, what);
    free_problem(P);
    return st;
  };
  cudaError_t e;
  // prefix tables
  if ((e = cudaMallocAsync(&P->d_prefix, pref.size() * sizeof(int64_t), cs)) != cudaSuccess) return fail_cuda(e, "cudaMalloc prefix");
  if ((e = cudaMemcpyAsync(P->d_prefix, pref.data(), pref.size() * sizeof(int64_t), cudaMemcpyHostToDevice, cs)) != cudaSuccess)
    return fail_cuda(e, "upload prefix");
  for (int k = 0; k < 3; ++k) g.P[k] = P->d_prefix + offs[k];
  // coefficients
  if (ph->kappa_cell) {
    for (int64_t c = 0; c < P->ncell; ++c)
      if (!std::isfinite(ph->kappa_cell[c])) {
        free_problem(P);
        return mrg_fail(MRG_ENUMERIC, "kappa contains NaN or Inf");
      }
  } else if (!std::isfinite(ph->kappa_const)) {
    free_problem(P);
    return mrg_fail(MRG_ENUMERIC, "kappa contains NaN or Inf");
  }
  if ((e = cudaMallocAsync(&P->d_kappa, P->ncell * sizeof(double), cs)) != cudaSuccess) return fail_cuda(e, "cudaMalloc kappa");
  if ((e = cudaMallocAsync(&P->d_kappa32, P->ncell * sizeof(float), cs)) != cudaSuccess) return fail_cuda(e, "cudaMalloc kappa32");
  if (ph->kappa_cell) {
    if ((e = cudaMemcpyAsync(P->d_kappa, ph->kappa_cell, P->ncell * sizeof(double), cudaMemcpyHostToDevice, cs)) != cudaSuccess)
      return fail_cuda(e, "upload kappa");
  } else {
    k_fill<<<nblk(P->ncell, 256), 256, 0, cs>>>(P->d_kappa, P->ncell, ph->kappa_const);
    if ((e = cudaGetLastError()) != cudaSuccess) return fail_cuda(e, "fill kappa");
  }
  // Dirichlet DOFs in increasing order; only boundary rows of the node grid are visited
  std::vector<int32_t> fixed;
  std::vector<double> fvals;
  auto add_fixed = [&](int ix, int iy, int iz) {
    int32_t n = ix + g.nn[0] * (iy + g.nn[1] * iz);
    fixed.push_back(n);
    fvals.push_back(ph->dirichlet_kind == MRG_DBC_NODE ? ph->dirichlet_node[n] : ph->dirichlet_const);
  };
  for (int iz = 0; iz < g.nn[2]; ++iz)
    for (int iy = 0; iy < g.nn[1]; ++iy) {
      if (node_fixed(g, 1 % g.nn[0], iy, iz) && g.nn[0] > 2) {
        // an interior x position is fixed: the whole x-line lies on a y or z face
        for (int ix = 0; ix < g.nn[0]; ++ix) add_fixed(ix, iy, iz);
      } else {
        for (int ix = 0; ix < g.nn[0]; ++ix) {
          if (ix > 0 && ix < g.nn[0] - 1) ix = g.nn[0] - 1;  // interior x positions are free on this line
          if (node_fixed(g, ix, iy, iz)) add_fixed(ix, iy, iz);
        }
      }
    }
  P->nfixed = (int64_t)fixed.size();
  if (P->nfixed > 0) {
    if ((e = cudaMallocAsync(&P->d_fixed, P->nfixed * sizeof(int32_t), cs)) != cudaSuccess) return fail_cuda(e, "cudaMalloc fixed");
    if ((e = cudaMallocAsync(&P->d_fixed_vals, P->nfixed * sizeof(double), cs)) != cudaSuccess)
      return fail_cuda(e, "cudaMalloc fixed vals");
    if ((e = cudaMemcpyAsync(P->d_fixed, fixed.data(), P->nfixed * sizeof(int32_t), cudaMemcpyHostToDevice, cs)) != cudaSuccess)
      return fail_cuda(e, "upload fixed");
    if ((e = cudaMemcpyAsync(P->d_fixed_vals, fvals.data(), P->nfixed * sizeof(double), cudaMemcpyHostToDevice, cs)) !=
        cudaSuccess)
      return fail_cuda(e, "upload fixed vals");
  }
  // reference tables at the quadrature points (phi: order p; psi: the bilinear/trilinear geometry map)
  const int d = m->dim, npe = P->npe, nq = P->nq, nvpe = (d == 3) ? 8 : 4;
  std::vector<double> tab(nq + npe * nq + npe * nq * d + nvpe * nq + nvpe * nq * d, 0.0);
  double* tw = tab.data();
  double* tphi = tw + nq;
  double* tdphi = tphi + npe * nq;
  double* tpsi = tdphi + npe * nq * d;
  double* tdpsi = tpsi + nvpe * nq;
  for (int q = 0; q < nq; ++q) {
    int qi[3] = {q % n1, (q / n1) % n1, (d == 3) ? q / (n1 * n1) : 0};
    double L[3][8], DL[3][8], G[3][2], DG[3][2];
    double w = 1.0;
    for (int k = 0; k < d; ++k) {
      lagrange(p, gx[qi[k]], L[k], DL[k]);
      lagrange(1, gx[qi[k]], G[k], DG[k]);
      w *= gw[qi[k]];
    }
    tw[q] = w;
    for (int i = 0; i < npe; ++i) {
      int a[3] = {i % (p + 1), (i / (p + 1)) % (p + 1), (d == 3) ? i / ((p + 1) * (p + 1)) : 0};
      double v = 1.0;
      for (int k = 0; k < d; ++k) v *= L[k][a[k]];
      tphi[i * nq + q] = v;
      for (int gg = 0; gg < d; ++gg) {
        double gv = 1.0;
        for (int k = 0; k < d; ++k) gv *= (k == gg) ? DL[k][a[k]] : L[k][a[k]];
        tdphi[(i * nq + q) * d + gg] = gv;
      }
    }
    for (int i = 0; i < nvpe; ++i) {
      int a[3] = {i % 2, (i / 2) % 2, (d == 3) ? i / 4 : 0};
      double v = 1.0;
      for (int k = 0; k < d; ++k) v *= G[k][a[k]];
      tpsi[i * nq + q] = v;
      for (int gg = 0; gg < d; ++gg) {
        double gv = 1.0;
        for (int k = 0; k < d; ++k) gv *= (k == gg) ? DG[k][a[k]] : G[k][a[k]];
        tdpsi[(i * nq + q) * d + gg] = gv;
      }
    }
  }
  P->qtab_host = tab;
  if ((e = cudaMallocAsync(&P->d_qtab, tab.size() * sizeof(double), cs)) != cudaSuccess) return fail_cuda(e, "cudaMalloc qtab");
  if ((e = cudaMemcpyAsync(P->d_qtab, tab.data(), tab.size() * sizeof(double), cudaMemcpyHostToDevice, cs)) != cudaSuccess)
    return fail_cuda(e, "upload qtab");
  // factored path: K(|dx|,|dy|,|dz|) of one box cell with kappa = 1 and the load of one node
  if (P->path == MRG_PATH_FACTORED) {
    double detJ = 1.0, gs[3];
    for (int k = 0; k < d; ++k) {
      detJ *= 0.5 * P->h[k];
      gs[k] = 2.0 / P->h[k];
    }
    for (int j = 0; j < 8; ++j) P->Kp[j] = 0.0;
    for (int j = 0; j < nvpe; ++j) {
      double s = 0.0;
      for (int q = 0; q < nq; ++q) {
        double dot = 0.0;
        for (int k = 0; k < d; ++k) dot += (tdphi[(0 * nq + q) * d + k] * gs[k]) * (tdphi[(j * nq + q) * d + k] * gs[k]);
        s += dot * tw[q] * detJ;
      }
      P->Kp[j] = s;
    }
    // Classes whose coefficient cancels in exact arithmetic (the axis neighbours of cubic cells:
    // -h/9 + h/18 + h/18) come out of the quadrature as rounding residue, ~1e-17 of the largest; a
    // coefficient within 64 ulps of the largest is that residue and is set to the exact zero.
    double kmax = 0.0;
    for (int j = 0; j < nvpe; ++j) kmax = std::max(kmax, std::fabs(P->Kp[j]));
    for (int j = 0; j < nvpe; ++j)
      if (std::fabs(P->Kp[j]) <= 64.0 * 2.220446049250313e-16 * kmax) P->Kp[j] = 0.0;
    // cubic cells: classes 3, 5, 6 and 7 are -h/12 and the diagonal h/3 in exact arithmetic; their
    // quadrature values agree to rounding.  The factored kernel then sums scaled conductances
    // |K7| kappa_c (k_kappa_scale) instead of multiplying every kappa sum by its class coefficient.
    if (d == 3) {
      const double k7 = P->Kp[7];
      auto near = [&](double a, double b) { return std::fabs(a - b) <= 64.0 * 2.220446049250313e-16 * std::fabs(b); };
      const bool axis0 = P->Kp[1] == 0.0 && P->Kp[2] == 0.0 && P->Kp[4] == 0.0 && !std::signbit(P->Kp[1]) &&
                         !std::signbit(P->Kp[2]) && !std::signbit(P->Kp[4]);
      if (axis0 && k7 < 0.0 && std::isnormal(k7) && near(P->Kp[3], k7) && near(P->Kp[5], k7) && near(P->Kp[6], k7) &&
          near(P->Kp[0], -4.0 * k7)) {
        P->cubic = 1;
        P->kscale = -k7;
        if ((e = cudaMallocAsync(&P->d_kappa_s, P->ncell * sizeof(double), cs)) != cudaSuccess)
          return fail_cuda(e, "cudaMalloc scaled kappa");
      }
    }
    double ld = 0.0;
    for (int q = 0; q < nq; ++q) ld += tphi[0 * nq + q] * tw[q] * detJ;
    P->cell_load = ld;
    if (P->source_kind == MRG_SRC_SINPROD) {
      // per-axis factor B_k[i] = sum over adjacent cells and 1-D Gauss points of
      // sin(freq x) * l_a(xi) * w * h/2   (the load vector is amp * prod_k B_k[i_k])
      std::vector<double> B;
      int64_t total = 0;
      for (int k = 0; k < d; ++k) total += g.nn[k];
      B.assign(total + (d == 2 ? 1 : 0), 1.0);
      int64_t off = 0;
      for (int k = 0; k < d; ++k) {
        for (int i = 0; i < g.nn[k]; ++i) {
          int cf, ncl;
          axis_cells(i, g.nn[k], 1, cf, ncl);
          double s = 0.0;
          for (int c = cf; c < cf + ncl; ++c) {
            int a = i - c;  // local node along the axis (0 or 1)
            for (int q = 0; q < n1; ++q) {
              double l[2], dl[2];
              lagrange(1, gx[q], l, dl);
              double x = P->lo[k] + P->h[k] * (c + 0.5 * (1.0 + gx[q]));
              s += std::sin(P->source_freq * x) * l[a] * gw[q] * 0.5 * P->h[k];
            }
          }
          B[off + i] = s;
        }
        off += g.nn[k];
      }
      if ((e = cudaMallocAsync(&P->d_srcB, B.size() * sizeof(double), cs)) != cudaSuccess) return fail_cuda(e, "cudaMalloc srcB");
      if ((e = cudaMemcpyAsync(P->d_srcB, B.data(), B.size() * sizeof(double), cudaMemcpyHostToDevice, cs)) != cudaSuccess)
        return fail_cuda(e, "upload srcB");
    }
  }
  // vertex coordinates for the general path (uniform boxes: computed in the kernel from lo and h)
  int64_t nvert = (int64_t)(g.nc[0] + 1) * (g.nc[1] + 1) * (d == 3 ? g.nc[2] + 1 : 1);
  if (m->vertex_coords) {
    std::vector<double> vc(nvert * d);
    for (int64_t v = 0; v < nvert; ++v) {
      int iv[3] = {(int)(v % (g.nc[0] + 1)), (int)((v / (g.nc[0] + 1)) % (g.nc[1] + 1)),
                   (int)(v / ((int64_t)(g.nc[0] + 1) * (g.nc[1] + 1)))};
      for (int k = 0; k < d; ++k)
        vc[v * d + k] = m->vertex_coords ? m->vertex_coords[v * d + k]
                                         : P->lo[k] + (P->hi[k] - P->lo[k]) * iv[k] / g.nc[k];
    }
    if ((e = cudaMallocAsync(&P->d_vcoord, vc.size() * sizeof(double), cs)) != cudaSuccess) return fail_cuda(e, "cudaMalloc vcoord");
    if ((e = cudaMemcpyAsync(P->d_vcoord, vc.data(), vc.size() * sizeof(double), cudaMemcpyHostToDevice, cs)) != cudaSuccess)
      return fail_cuda(e, "upload vcoord");
  }
  int st = mrg_launch_kappa32(P, cs);
  if (st == MRG_OK && P->path == MRG_PATH_TENSOR) st = mrg_q2_setup(P);
  if (st == MRG_OK && P->path == MRG_PATH_STORED) st = mrg_stored_setup(P, cs);
  if (st != MRG_OK) {
    free_problem(P);
    return st;
  }
  if ((e = cudaStreamSynchronize(cs)) != cudaSuccess) return fail_cuda(e, "problem setup");
  *out = P;
  return MRG_OK;
}

extern "C" int mrg_problem_create(const mrg_mesh_desc* m, const mrg_physics_desc* ph, mrg_problem** out) {
  return create_impl(m, ph, (cudaStream_t)0, out);
}

extern "C" int mrg_problem_create_on_stream(const mrg_mesh_desc* m, const mrg_physics_desc* ph, mrg_stream_t stream,
                                            mrg_problem** out) {
  return create_impl(m, ph, (cudaStream_t)stream, out);
}

extern "C" int mrg_problem_destroy(mrg_problem* p) {
  if (!p) return MRG_EINVAL;
  free_problem(p);
  return MRG_OK;
}

extern "C" int mrg_set_wait_policy(mrg_problem* p, uint64_t limit_ns, int32_t withhold_copy) {
  if (!p) return mrg_fail(MRG_EINVAL, "mrg_set_wait_policy: null problem");
  if (limit_ns > MRG_WAIT_LIMIT_MAX_NS)
    return mrg_fail(MRG_EINVAL, "mrg_set_wait_policy: limit above MRG_WAIT_LIMIT_MAX_NS");
  // captured graphs and multigrid levels hold copies of the grid description: let the work in flight
  // finish, then drop them so that the next solve records the new policy
  MRG_CUDA(cudaStreamSynchronize(p->last_stream));
  p->g.wait_ns = (unsigned long long)limit_ns;
  p->g.withhold = withhold_copy ? 1 : 0;
  mrg_solver_drop_graphs(p);
  mrg_bicg_drop_graphs(p);
  mrg_gmg_drop_hierarchy(p);
  return MRG_OK;
}

extern "C" int mrg_problem_get_info(const mrg_problem* p, mrg_problem_info* info) {
  if (!p || !info) return mrg_fail(MRG_EINVAL, "mrg_problem_get_info: null argument");
  info->n_dofs = p->ndof;
  info->n_cells = p->ncell;
  info->nnz = p->nnz;
  info->n_fixed = p->nfixed;
  info->nodes_per_cell = p->npe;
  info->qp_per_cell = p->nq;
  info->path = p->path;
  info->reserved = 0;
  return MRG_OK;
}

extern "C" int mrg_get_graph(const mrg_problem* p, int64_t* row_ptr, int32_t* col_idx, mrg_stream_t stream) {
  if (!p || !row_ptr || !col_idx) return mrg_fail(MRG_EINVAL, "mrg_get_graph: null argument");
  k_graph<<<nblk(p->ndof + 1, 256), 256, 0, (cudaStream_t)stream>>>(p->g, p->ndof, row_ptr, col_idx);
  MRG_CUDA(cudaGetLastError());
  return MRG_OK;
}

extern "C" int mrg_get_dof_map(const mrg_problem* p, int32_t* lids, mrg_stream_t stream) {
  if (!p || !lids) return mrg_fail(MRG_EINVAL, "mrg_get_dof_map: null argument");
  k_dof_map<<<nblk(p->ncell * p->npe, 256), 256, 0, (cudaStream_t)stream>>>(p->g, p->ncell, p->npe, lids);
  MRG_CUDA(cudaGetLastError());
  return MRG_OK;
}

extern "C" int mrg_get_fixed_dofs(const mrg_problem* p, int32_t* dofs, double* values, mrg_stream_t stream) {
  if (!p || !dofs) return mrg_fail(MRG_EINVAL, "mrg_get_fixed_dofs: null argument");
  if (p->nfixed == 0) return MRG_OK;
  k_copy_fixed<<<nblk(p->nfixed, 256), 256, 0, (cudaStream_t)stream>>>(p->d_fixed, p->d_fixed_vals, p->nfixed, dofs,
                                                                          values);
  MRG_CUDA(cudaGetLastError());
  return MRG_OK;
}

extern "C" int mrg_set_kappa(mrg_problem* p, const double* kappa_dev, mrg_stream_t stream) {
  if (!p || !kappa_dev) return mrg_fail(MRG_EINVAL, "mrg_set_kappa: null argument");
  MRG_CUDA(cudaMemcpyAsync(p->d_kappa, kappa_dev, p->ncell * sizeof(double), cudaMemcpyDeviceToDevice,
                           (cudaStream_t)stream));
  return mrg_launch_kappa32(p, (cudaStream_t)stream);
}

extern "C" int mrg_set_dirichlet(const mrg_problem* p, double* u, mrg_stream_t stream) {
  if (!p || !u) return mrg_fail(MRG_EINVAL, "mrg_set_dirichlet: null argument");
  if (p->nfixed == 0) return MRG_OK;
  k_set_dirichlet<<<nblk(p->nfixed, 256), 256, 0, (cudaStream_t)stream>>>(p->d_fixed, p->d_fixed_vals, p->nfixed, u);
  MRG_CUDA(cudaGetLastError());
  return MRG_OK;
}

// ------------------------------------------------------------------------------------------------
// assembly dispatcher: AssemblyManager::assembleJacRes / assembleRes
// ------------------------------------------------------------------------------------------------
extern "C" int mrg_assemble(mrg_problem* p, const double* u, double* r, void* J, uint32_t flags, mrg_stream_t stream) {
  if (!p || !u) return mrg_fail(MRG_EINVAL, "mrg_assemble: null problem or u");
  if (flags & (MRG_ASM_ADJOINT | MRG_ASM_SENS))
    return mrg_fail(MRG_ENOTSUP, "adjoint and sensitivity assembly are not built");
  const bool doJ = flags & MRG_ASM_JAC, doR = flags & MRG_ASM_RES;
  if (!doJ && !doR) return mrg_fail(MRG_EINVAL, "mrg_assemble: neither MRG_ASM_RES nor MRG_ASM_JAC");
  if (doJ && !J) return mrg_fail(MRG_EINVAL, "mrg_assemble: Jacobian requested but J_vals is null");
  if (doR && !r) return mrg_fail(MRG_EINVAL, "mrg_assemble: residual requested but r is null");
  cudaStream_t s = (cudaStream_t)stream;
  p->last_stream = s;
  const bool fp32 = flags & MRG_ASM_J_FP32;
  int st;
  if (p->path == MRG_PATH_FACTORED && !(flags & MRG_ASM_FORCE_CELL)) {
    st = mrg_launch_factored(p, u, r, J, flags, s);
    if (st != MRG_OK) return st;
  } else if (p->path == MRG_PATH_TENSOR && !(flags & MRG_ASM_FORCE_CELL)) {
    st = mrg_launch_q2(p, u, r, J, flags, s);
    if (st != MRG_OK) return st;
  } else if (p->path == MRG_PATH_STORED && !(flags & (MRG_ASM_FORCE_CELL | MRG_ASM_ATOMIC))) {
    st = mrg_launch_stored(p, u, r, J, flags, s);
    if (st != MRG_OK) return st;
  } else {
    if (flags & MRG_ASM_OVERWRITE) {
      if (doJ) MRG_CUDA(cudaMemsetAsync(J, 0, p->nnz * (fp32 ? sizeof(float) : sizeof(double)), s));
      if (doR) MRG_CUDA(cudaMemsetAsync(r, 0, p->ndof * sizeof(double), s));
    }
    st = mrg_launch_cell(p, u, doR ? r : nullptr, doJ ? J : nullptr, flags, s);
    if (st != MRG_OK) return st;
    if (doJ) {
      st = mrg_launch_constraints(p, J, fp32, s);
      if (st != MRG_OK) return st;
    }
  }
  // boundary workset loop (jacres:485-603): Neumann / weak-Dirichlet faces, after the volume terms
  if (mrg_boundary_active(p)) {
    st = mrg_launch_boundary(p, u, doR ? r : nullptr, doJ ? J : nullptr, fp32, s);
    if (st != MRG_OK) return st;
  }
  if (doJ && (flags & MRG_ASM_FIX_ZERO_ROWS)) return mrg_launch_fix_zero_rows(p, J, fp32, s);
  return MRG_OK;
}

extern "C" int mrg_assemble_residual(mrg_problem* p, const double* u, double* r, uint32_t flags, mrg_stream_t stream) {
  return mrg_assemble(p, u, r, nullptr, (flags & ~(uint32_t)(MRG_ASM_JAC | MRG_ASM_J_FP32)) | MRG_ASM_RES, stream);
}
