// Boundary terms on mesh faces: Neumann data and weakly imposed (Nitsche) Dirichlet data.
//
// Reference: thermal::boundaryResidual (src/physics/thermal.cpp:170-260), called by the boundary
// workset loop of AssemblyManager::assembleJacRes (src/managers/assembly/assemblyManager_jacres.hpp:
// 485-603) on every side whose boundary condition is "Neumann" or "weak Dirichlet"; side element size
// Workset::getSideElementSize (src/tools/workset.cpp:2719-2733).  Per side point q with weight w_q:
//     Neumann         res_i += -g_q w_q phi_i
//     weak Dirichlet  res_i += 10/h kappa (T - g) w phi_i - kappa (grad T . n) w phi_i
//                              - kappa (T - g) w (grad phi_i . n)            (form_param = 1)
// with h = (sum_q w_q)^(1/(dim-1)), kappa the cell's diffusion (kappa_c, or 1 + T^2) and the same
// scatter as the volume terms (r -= res, J += d res / du, strong-Dirichlet rows skipped).
//
// Data: the caller gives g at the side points of a face (mrg_get_side_points order: face cells with
// the first tangential cell index fastest, then the side points of the cell with the first
// tangential axis fastest).  Box cells are identical, so per face the side tables (phi_i, grad phi_i . n
// at the side points, weights, h) are the same for every face cell and are computed once on the host.
// General (non-affine) cells: phi_i at the side points is still the reference table, while the weights,
// grad phi_i . n and h differ per face cell; they are computed once per face on the host when the
// condition is set, from the trilinear map of the cell's vertices (geometric Jacobian J at the side
// point, side measure |dx/dxi_t| in 2-D or |dx/dxi_t1 x dx/dxi_t2| in 3-D, outward unit normal
// +-J^{-T} e_a normalised, physical gradients J^{-T} grad_xi phi_i -- the CellTools quantities of the
// reference's side workset, src/tools/workset.cpp), and the kernel reads them per cell.
//
// Kernel: one thread per row node in the p+1 node layers next to the face (every node of a boundary
// cell).  The thread walks the row's boundary cells in a fixed order, forms the cell's T and grad T . n
// at the side points from u, and adds the row's residual value and Jacobian entries.  Each row is
// owned by one thread and faces are processed one launch after another, so there are no atomics and
// the result is deterministic.
#include <cmath>
#include <vector>

#include "mrg_device.cuh"
#include "mrg_internal.h"

namespace {

constexpr int MAXSP = 16;   // side points per cell (1-D rule of up to 4 points, squared)
constexpr int MAXPE = 27;   // nodes per cell

struct FaceDev {
  int face, kind, nsp, dim, p;
  double h;
  const double* g;     // [nfc][nsp]
  const double* tab;   // phi [npe][nsp], gn [npe][nsp], w [nsp]
  const double* ctab;  // general cells: per face cell gn [npe][nsp], w [nsp], 10 / h (null for box cells)
  int cstride;         // doubles per face cell in ctab
};

template <typename JT>
__global__ void k_face(Grid g, FaceDev F, int phys, const double* __restrict__ kap, const double* __restrict__ u,
                       double* __restrict__ r, JT* __restrict__ J, int64_t nthreads) {
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= nthreads) return;
  const int dim = F.dim, p = F.p, a = F.face >> 1, hi_side = F.face & 1;
  int t0 = -1, t1 = -1;
  for (int k = 0, m = 0; k < dim; ++k)
    if (k != a) { if (m == 0) t0 = k; else t1 = k; ++m; }
  // thread -> (layer, i_t0, i_t1)
  const int nt0 = g.nn[t0], nt1 = (dim == 3) ? g.nn[t1] : 1;
  const int layer = (int)(tid / ((int64_t)nt0 * nt1));
  const int64_t rem = tid - (int64_t)layer * nt0 * nt1;
  const int it0 = (int)(rem % nt0), it1 = (int)(rem / nt0);
  int node[3] = {0, 0, 0};
  node[a] = hi_side ? g.nn[a] - 1 - layer : layer;
  node[t0] = it0;
  if (dim == 3) node[t1] = it1;
  if (node_fixed(g, node[0], node[1], node[2])) return;
  const int ca = hi_side ? g.nc[a] - 1 : 0;  // boundary cell index along the normal axis
  int f0, n0, f1 = 0, n1 = 1;
  axis_cells(it0, nt0, p, f0, n0);
  if (dim == 3) axis_cells(it1, nt1, p, f1, n1);
  const mrgdev::RowInfo R = mrgdev::row_info(g, node[0], node[1], node[2]);
  const int n1d = p + 1, npe = (dim == 3) ? n1d * n1d * n1d : n1d * n1d, nsp = F.nsp;
  const double* phi = F.tab;
  const double* gn_box = F.tab + npe * nsp;
  const double* w_box = F.tab + 2 * npe * nsp;
  const double epen_box = 10.0 / F.h;
  double res = 0.0;
  for (int c1 = f1; c1 < f1 + n1; ++c1)
    for (int c0 = f0; c0 < f0 + n0; ++c0) {
      int cc[3] = {0, 0, 0};
      cc[a] = ca;
      cc[t0] = c0;
      if (dim == 3) cc[t1] = c1;
      const int64_t cell = cc[0] + (int64_t)g.nc[0] * (cc[1] + (int64_t)g.nc[1] * cc[2]);
      const int64_t fcell = c0 + (int64_t)g.nc[t0] * c1;  // index in face order
      int lc[3];
      for (int k = 0; k < 3; ++k) lc[k] = (k < dim) ? node[k] - p * cc[k] : 0;
      const int l = lc[0] + n1d * (lc[1] + n1d * lc[2]);
      const double* gq = F.g + fcell * nsp;
      // this face cell's weights, normal derivatives and penalty (the shared tables on box cells)
      const double* gn = gn_box;
      const double* w = w_box;
      double epen_h = epen_box;
      if (F.ctab) {
        gn = F.ctab + fcell * F.cstride;
        w = gn + npe * nsp;
        epen_h = w[nsp];
      }
      if (F.kind == MRG_BC_NEUMANN) {
        for (int q = 0; q < nsp; ++q) res += -gq[q] * w[q] * phi[l * nsp + q];
        continue;
      }
      // weak Dirichlet: T and grad T . n at the side points
      double uc[MAXPE];
      for (int j = 0; j < npe; ++j) {
        const int jx = j % n1d, jy = (j / n1d) % n1d, jz = j / (n1d * n1d);
        const int nx = p * cc[0] + jx, ny = p * cc[1] + jy, nz = (dim == 3) ? p * cc[2] + jz : 0;
        uc[j] = __ldg(u + nx + (int64_t)g.nn[0] * (ny + (int64_t)g.nn[1] * nz));
      }
      double T[MAXSP], dTn[MAXSP], kq[MAXSP], dk[MAXSP], jump[MAXSP];
      for (int q = 0; q < nsp; ++q) {
        double t = 0.0, d = 0.0;
        for (int j = 0; j < npe; ++j) {
          t = fma(uc[j], phi[j * nsp + q], t);
          d = fma(uc[j], gn[j * nsp + q], d);
        }
        T[q] = t;
        dTn[q] = d;
        kq[q] = (phys == MRG_THERMAL) ? __ldg(kap + cell) : 1.0 + t * t;
        dk[q] = (phys == MRG_THERMAL) ? 0.0 : 2.0 * t;
        jump[q] = t - gq[q];
        res += w[q] * (epen_h * kq[q] * jump[q] * phi[l * nsp + q] - kq[q] * dTn[q] * phi[l * nsp + q] -
                       kq[q] * jump[q] * gn[l * nsp + q]);
      }
      if (J) {
        for (int j = 0; j < npe; ++j) {
          double dj = 0.0;
          for (int q = 0; q < nsp; ++q) {
            const double pj = phi[j * nsp + q], gj = gn[j * nsp + q];
            const double dkj = dk[q] * pj;                       // d kappa / d u_j
            const double djump = pj, ddtn = gj;                  // d (T - g) / d u_j, d (grad T . n) / d u_j
            dj += w[q] * (epen_h * (dkj * jump[q] + kq[q] * djump) * phi[l * nsp + q] -
                          (dkj * dTn[q] + kq[q] * ddtn) * phi[l * nsp + q] -
                          (dkj * jump[q] + kq[q] * djump) * gn[l * nsp + q]);
          }
          const int jx = j % n1d, jy = (j / n1d) % n1d, jz = j / (n1d * n1d);
          const int cxn = p * cc[0] + jx, cyn = p * cc[1] + jy, czn = (dim == 3) ? p * cc[2] + jz : 0;
          const int64_t pos = ((int64_t)(czn - R.lz) * R.cy + (cyn - R.ly)) * R.cx + (cxn - R.lx);
          J[R.rp + pos] += (JT)dj;
        }
      }
    }
  if (r) r[node[0] + (int64_t)g.nn[0] * (node[1] + (int64_t)g.nn[1] * node[2])] -= res;
}

struct FaceBC {
  int kind = MRG_BC_NONE;
  int nsp = 0;
  int64_t nfc = 0;
  double h = 0.0;
  double* d_g = nullptr;
  double* d_tab = nullptr;
  double* d_ctab = nullptr;  // general cells
  int cstride = 0;
};

struct BoundaryData {
  FaceBC f[6];
  std::vector<double> vc;  // general cells: host copy of the vertex coordinates, fetched on first use
};

// Side rule of one face on the problem's 1-D Gauss rule, box cells: reference coordinates of the side
// points (first tangential axis fastest), weights w_ref * prod_t h_t / 2, and per node phi_i and
// grad phi_i . n at the points.
void side_tables(const mrg_problem* p, int face, std::vector<double>& tab, int& nsp, double& h) {
  const int dim = p->g.dim, P = p->g.p, a = face / 2, n1d = P + 1;
  const int npe = (dim == 3) ? n1d * n1d * n1d : n1d * n1d;
  const std::vector<double>& gx = p->gx1;
  const std::vector<double>& gw = p->gw1;
  const int nq1 = (int)gx.size();
  int t[2] = {-1, -1}, nt = 0;
  for (int k = 0; k < dim; ++k)
    if (k != a) t[nt++] = k;
  nsp = (dim == 3) ? nq1 * nq1 : nq1;
  tab.assign((size_t)2 * npe * nsp + nsp, 0.0);
  double meas = 1.0;
  for (int m = 0; m < nt; ++m) meas *= 0.5 * p->h[t[m]];
  const double sgn = (face & 1) ? 1.0 : -1.0;
  double wsum = 0.0;
  for (int q = 0; q < nsp; ++q) {
    double xi[3] = {0.0, 0.0, 0.0}, wq = meas;
    xi[a] = sgn;
    xi[t[0]] = gx[q % nq1];
    wq *= gw[q % nq1];
    if (dim == 3) {
      xi[t[1]] = gx[q / nq1];
      wq *= gw[q / nq1];
    }
    tab[(size_t)2 * npe * nsp + q] = wq;
    wsum += wq;
    double L[3][3], DL[3][3];
    for (int k = 0; k < dim; ++k) mrg_lagrange_1d(P, xi[k], L[k], DL[k]);
    for (int i = 0; i < npe; ++i) {
      const int ai[3] = {i % n1d, (i / n1d) % n1d, (dim == 3) ? i / (n1d * n1d) : 0};
      double v = 1.0, dn = 1.0;
      for (int k = 0; k < dim; ++k) {
        v *= L[k][ai[k]];
        dn *= (k == a) ? DL[k][ai[k]] : L[k][ai[k]];
      }
      tab[(size_t)i * nsp + q] = v;
      tab[(size_t)npe * nsp + (size_t)i * nsp + q] = sgn * (2.0 / p->h[a]) * dn;  // grad phi . n, n = sgn e_a
    }
  }
  h = (dim == 2) ? wsum : std::pow(wsum, 1.0 / (dim - 1.0));
}

// General cells: the geometry of face cell k of `face` at its side points.  Fills, when non-null,
// ct [npe*nsp + nsp + 1] = grad phi_i . n [npe][nsp], w [nsp], 10 / h and xyz [nsp][3] (physical
// coordinates of the side points).
void side_cell_general(const mrg_problem* p, int face, int64_t k, const std::vector<double>& vc, double* ct,
                       double* xyz) {
  const int dim = p->g.dim, P = p->g.p, a = face / 2, n1d = P + 1;
  const int npe = (dim == 3) ? n1d * n1d * n1d : n1d * n1d;
  const std::vector<double>& gx = p->gx1;
  const std::vector<double>& gw = p->gw1;
  const int nq1 = (int)gx.size(), nsp = (dim == 3) ? nq1 * nq1 : nq1;
  int t[2] = {-1, -1}, nt = 0;
  for (int m = 0; m < dim; ++m)
    if (m != a) t[nt++] = m;
  const int n0 = p->g.nc[t[0]];
  int cc[3] = {0, 0, 0};
  cc[a] = (face & 1) ? p->g.nc[a] - 1 : 0;
  cc[t[0]] = (int)(k % n0);
  if (dim == 3) cc[t[1]] = (int)(k / n0);
  const int nvx = p->g.nc[0] + 1, nvy = p->g.nc[1] + 1;
  double xv[8][3] = {};
  for (int v = 0; v < (1 << dim); ++v) {
    const int64_t vid = (cc[0] + (v & 1)) + (int64_t)nvx * ((cc[1] + ((v >> 1) & 1)) + (int64_t)nvy * (dim == 3 ? cc[2] + (v >> 2) : 0));
    for (int m = 0; m < dim; ++m) xv[v][m] = vc[(size_t)vid * dim + m];
  }
  const double sgn = (face & 1) ? 1.0 : -1.0;
  double wsum = 0.0;
  for (int q = 0; q < nsp; ++q) {
    double xi[3] = {0.0, 0.0, 0.0}, wref = gw[q % nq1];
    xi[a] = sgn;
    xi[t[0]] = gx[q % nq1];
    if (dim == 3) {
      xi[t[1]] = gx[q / nq1];
      wref *= gw[q / nq1];
    }
    double L[3][3], DL[3][3], G[3][2], DG[3][2];
    for (int m = 0; m < dim; ++m) {
      mrg_lagrange_1d(P, xi[m], L[m], DL[m]);
      mrg_lagrange_1d(1, xi[m], G[m], DG[m]);
    }
    double Jm[3][3] = {}, x[3] = {};
    for (int v = 0; v < (1 << dim); ++v) {
      const int av[3] = {v & 1, (v >> 1) & 1, v >> 2};
      double ps = 1.0;
      for (int m = 0; m < dim; ++m) ps *= G[m][av[m]];
      for (int m = 0; m < dim; ++m) {
        x[m] += xv[v][m] * ps;
        for (int e = 0; e < dim; ++e) {
          double dp = 1.0;
          for (int f = 0; f < dim; ++f) dp *= (f == e) ? DG[f][av[f]] : G[f][av[f]];
          Jm[m][e] += xv[v][m] * dp;
        }
      }
    }
    // inverse from the cofactors: Ji[e][m] = C[m][e] / det
    double Ji[3][3] = {};
    if (dim == 2) {
      const double det = Jm[0][0] * Jm[1][1] - Jm[0][1] * Jm[1][0];
      Ji[0][0] = Jm[1][1] / det; Ji[0][1] = -Jm[0][1] / det;
      Ji[1][0] = -Jm[1][0] / det; Ji[1][1] = Jm[0][0] / det;
    } else {
      double C[3][3];
      for (int m = 0; m < 3; ++m)
        for (int e = 0; e < 3; ++e) {
          const int m1 = (m + 1) % 3, m2 = (m + 2) % 3, e1 = (e + 1) % 3, e2 = (e + 2) % 3;
          C[m][e] = Jm[m1][e1] * Jm[m2][e2] - Jm[m1][e2] * Jm[m2][e1];
        }
      const double det = Jm[0][0] * C[0][0] + Jm[0][1] * C[0][1] + Jm[0][2] * C[0][2];
      for (int m = 0; m < 3; ++m)
        for (int e = 0; e < 3; ++e) Ji[e][m] = C[m][e] / det;
    }
    double meas;
    if (dim == 2) {
      meas = std::sqrt(Jm[0][t[0]] * Jm[0][t[0]] + Jm[1][t[0]] * Jm[1][t[0]]);
    } else {
      const double u0[3] = {Jm[0][t[0]], Jm[1][t[0]], Jm[2][t[0]]}, u1[3] = {Jm[0][t[1]], Jm[1][t[1]], Jm[2][t[1]]};
      const double cr[3] = {u0[1] * u1[2] - u0[2] * u1[1], u0[2] * u1[0] - u0[0] * u1[2], u0[0] * u1[1] - u0[1] * u1[0]};
      meas = std::sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
    }
    double nv[3] = {}, nn2 = 0.0;
    for (int m = 0; m < dim; ++m) {
      nv[m] = Ji[a][m];
      nn2 += nv[m] * nv[m];
    }
    const double inv = sgn / std::sqrt(nn2);
    for (int m = 0; m < dim; ++m) nv[m] *= inv;
    if (xyz)
      for (int m = 0; m < 3; ++m) xyz[q * 3 + m] = (m < dim) ? x[m] : 0.0;
    if (!ct) continue;
    const double wq = wref * meas;
    ct[(size_t)npe * nsp + q] = wq;
    wsum += wq;
    for (int i = 0; i < npe; ++i) {
      const int ai[3] = {i % n1d, (i / n1d) % n1d, (dim == 3) ? i / (n1d * n1d) : 0};
      double dr[3];
      for (int e = 0; e < dim; ++e) {
        double gv = 1.0;
        for (int m = 0; m < dim; ++m) gv *= (m == e) ? DL[m][ai[m]] : L[m][ai[m]];
        dr[e] = gv;
      }
      double gnv = 0.0;
      for (int m = 0; m < dim; ++m) {
        double gm = 0.0;
        for (int e = 0; e < dim; ++e) gm += Ji[e][m] * dr[e];
        gnv += gm * nv[m];
      }
      ct[(size_t)i * nsp + q] = gnv;
    }
  }
  if (ct) ct[(size_t)npe * nsp + nsp] = 10.0 / ((dim == 2) ? wsum : std::pow(wsum, 1.0 / (dim - 1.0)));
}

// The host copy of the vertex coordinates (general cells), fetched from the device once
const std::vector<double>& host_vertices(const mrg_problem* p, BoundaryData* B) {
  if (B->vc.empty()) {
    const int64_t nvert = (int64_t)(p->g.nc[0] + 1) * (p->g.nc[1] + 1) * (p->g.dim == 3 ? p->g.nc[2] + 1 : 1);
    B->vc.resize((size_t)nvert * p->g.dim);
    cudaMemcpyAsync(B->vc.data(), p->d_vcoord, B->vc.size() * sizeof(double), cudaMemcpyDeviceToHost, p->stream);
    cudaStreamSynchronize(p->stream);
  }
  return B->vc;
}

int64_t face_cell_count(const mrg_problem* p, int face) {
  const int a = face / 2;
  int64_t n = 1;
  for (int k = 0; k < p->g.dim; ++k)
    if (k != a) n *= p->g.nc[k];
  return n;
}

}  // namespace

void mrg_boundary_free(mrg_problem* p) {
  BoundaryData* B = reinterpret_cast<BoundaryData*>(p->bnd);
  if (!B) return;
  for (FaceBC& f : B->f) {
    if (f.d_g) cudaFreeAsync(f.d_g, p->stream);
    if (f.d_tab) cudaFreeAsync(f.d_tab, p->stream);
    if (f.d_ctab) cudaFreeAsync(f.d_ctab, p->stream);
  }
  delete B;
  p->bnd = nullptr;
}

bool mrg_boundary_active(const mrg_problem* p) {
  const BoundaryData* B = reinterpret_cast<const BoundaryData*>(p->bnd);
  if (!B) return false;
  for (const FaceBC& f : B->f)
    if (f.kind != MRG_BC_NONE) return true;
  return false;
}

int mrg_launch_boundary(mrg_problem* p, const double* u, double* r, void* J, bool fp32, cudaStream_t s) {
  BoundaryData* B = reinterpret_cast<BoundaryData*>(p->bnd);
  if (!B) return MRG_OK;
  for (int face = 0; face < 2 * p->g.dim; ++face) {
    const FaceBC& f = B->f[face];
    if (f.kind == MRG_BC_NONE) continue;
    if (f.kind == MRG_BC_NEUMANN && !r) continue;  // Neumann data does not depend on u
    FaceDev F{face, f.kind, f.nsp, p->g.dim, p->g.p, f.h, f.d_g, f.d_tab, f.d_ctab, f.cstride};
    const int a = face / 2;
    int64_t n = (int64_t)(p->g.p + 1);
    for (int k = 0; k < p->g.dim; ++k)
      if (k != a) n *= p->g.nn[k];
    const unsigned nb = (unsigned)((n + 127) / 128);
    if (fp32)
      k_face<float><<<nb, 128, 0, s>>>(p->g, F, p->kind, p->d_kappa, u, r, (float*)J, n);
    else
      k_face<double><<<nb, 128, 0, s>>>(p->g, F, p->kind, p->d_kappa, u, r, (double*)J, n);
    MRG_CUDA(cudaGetLastError());
  }
  return MRG_OK;
}

extern "C" int mrg_get_side_points(const mrg_problem* p, int32_t face, int64_t* npts, double* xyz) {
  if (!p || !npts) return mrg_fail(MRG_EINVAL, "mrg_get_side_points: null argument");
  if (face < 0 || face >= 2 * p->g.dim) return mrg_fail(MRG_EINVAL, "mrg_get_side_points: face out of range");
  const int dim = p->g.dim, a = face / 2;
  const int nq1 = (int)p->gx1.size(), nsp = (dim == 3) ? nq1 * nq1 : nq1;
  int t[2] = {-1, -1}, nt = 0;
  for (int k = 0; k < dim; ++k)
    if (k != a) t[nt++] = k;
  const int64_t nfc = face_cell_count(p, face);
  *npts = nfc * nsp;
  if (!xyz) return MRG_OK;
  if (!p->affine) {
    if (nq1 > 4) return mrg_fail(MRG_ENOTSUP, "face rule: at most 4 points per axis");
    mrg_problem* pm = const_cast<mrg_problem*>(p);  // the vertex cache only
    if (!pm->bnd) pm->bnd = new BoundaryData();
    const std::vector<double>& vc = host_vertices(p, reinterpret_cast<BoundaryData*>(pm->bnd));
    for (int64_t k = 0; k < nfc; ++k) side_cell_general(p, face, k, vc, nullptr, xyz + k * nsp * 3);
    return MRG_OK;
  }
  const int n0 = p->g.nc[t[0]];
  for (int64_t k = 0; k < nfc; ++k) {
    const int c0 = (int)(k % n0), c1 = (int)(k / n0);
    for (int q = 0; q < nsp; ++q) {
      double* x = xyz + (k * nsp + q) * 3;
      x[0] = x[1] = x[2] = 0.0;
      x[a] = (face & 1) ? p->hi[a] : p->lo[a];
      x[t[0]] = p->lo[t[0]] + p->h[t[0]] * (c0 + 0.5 * (1.0 + p->gx1[q % nq1]));
      if (dim == 3) x[t[1]] = p->lo[t[1]] + p->h[t[1]] * (c1 + 0.5 * (1.0 + p->gx1[q / nq1]));
    }
  }
  return MRG_OK;
}

extern "C" int mrg_set_face_bc(mrg_problem* p, int32_t face, int32_t kind, const double* g) {
  if (!p) return mrg_fail(MRG_EINVAL, "mrg_set_face_bc: null problem");
  if (face < 0 || face >= 2 * p->g.dim) return mrg_fail(MRG_EINVAL, "mrg_set_face_bc: face out of range");
  if (kind != MRG_BC_NONE && kind != MRG_BC_NEUMANN && kind != MRG_BC_WEAK_DIRICHLET)
    return mrg_fail(MRG_EINVAL, "mrg_set_face_bc: unknown boundary-condition kind");
  if (kind != MRG_BC_NONE && (p->g.faces >> face) & 1u)
    return mrg_fail(MRG_EINVAL, "mrg_set_face_bc: the face carries a strong Dirichlet condition");
  if (kind != MRG_BC_NONE && p->gx1.size() > 4) return mrg_fail(MRG_ENOTSUP, "face rule: at most 4 points per axis");
  if (!p->bnd) p->bnd = new BoundaryData();
  BoundaryData* B = reinterpret_cast<BoundaryData*>(p->bnd);
  FaceBC& f = B->f[face];
  cudaStream_t s = p->stream;
  if (f.d_g) { cudaFreeAsync(f.d_g, s); f.d_g = nullptr; }
  if (f.d_tab) { cudaFreeAsync(f.d_tab, s); f.d_tab = nullptr; }
  if (f.d_ctab) { cudaFreeAsync(f.d_ctab, s); f.d_ctab = nullptr; }
  f.cstride = 0;
  f.kind = MRG_BC_NONE;
  if (kind == MRG_BC_NONE) return MRG_OK;
  std::vector<double> tab;
  side_tables(p, face, tab, f.nsp, f.h);
  f.nfc = face_cell_count(p, face);
  const size_t ng = (size_t)f.nfc * f.nsp;
  std::vector<double> gh(ng, 0.0);
  if (g)
    for (size_t i = 0; i < ng; ++i) gh[i] = g[i];
  MRG_CUDA(cudaMallocAsync(&f.d_g, ng * sizeof(double), s));
  MRG_CUDA(cudaMallocAsync(&f.d_tab, tab.size() * sizeof(double), s));
  MRG_CUDA(cudaMemcpyAsync(f.d_g, gh.data(), ng * sizeof(double), cudaMemcpyHostToDevice, s));
  MRG_CUDA(cudaMemcpyAsync(f.d_tab, tab.data(), tab.size() * sizeof(double), cudaMemcpyHostToDevice, s));
  std::vector<double> ctab;
  if (!p->affine) {
    // per face cell: grad phi . n, weights and 10 / h of its own geometry
    const int n1d = p->g.p + 1, npe = (p->g.dim == 3) ? n1d * n1d * n1d : n1d * n1d;
    f.cstride = npe * f.nsp + f.nsp + 1;
    ctab.assign((size_t)f.nfc * f.cstride, 0.0);
    const std::vector<double>& vc = host_vertices(p, B);
    for (int64_t k = 0; k < f.nfc; ++k) side_cell_general(p, face, k, vc, ctab.data() + k * f.cstride, nullptr);
    MRG_CUDA(cudaMallocAsync(&f.d_ctab, ctab.size() * sizeof(double), s));
    MRG_CUDA(cudaMemcpyAsync(f.d_ctab, ctab.data(), ctab.size() * sizeof(double), cudaMemcpyHostToDevice, s));
  }
  MRG_CUDA(cudaStreamSynchronize(s));
  f.kind = kind;
  return MRG_OK;
}
