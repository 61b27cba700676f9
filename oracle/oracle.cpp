// Oracle: CPU restatement of MrHyDE's workset finite-element assembly path.
//
// TEST INFRASTRUCTURE ONLY.  Nothing in the product (mrhyde_gb300/) links, loads or calls this
// file.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it, and only
// as the checker or as the timed CPU baseline, never as the thing measured on the GPU.
//
// It restates, in plain FP64 C++ (serial, or OpenMP with atomic scatter), the algorithm of the
// reference path (all paths relative to the MrHyDE source tree):
//   * workset loop            src/managers/assembly/assemblyManager_jacres.hpp:121-630
//                             (sequential groups :336, gather :346, updateWorkset :380,
//                              volumeResidual :381, scatter :409-414, constraints :606)
//   * gather                  src/managers/assembly/assemblyManager_gather.hpp:183-232
//   * AD seeding (SFad e_dof) src/tools/workset.cpp:865-901 (seed at :884)
//   * solution fields at ip   src/tools/workset.cpp:1093-1105
//   * thermal residual        src/physics/thermal.cpp:71-165 (kernel :125-163)
//   * scatter (-val, +dx)     src/managers/assembly/assemblyManager_scatter.hpp:164-278
//   * strong Dirichlet rows   src/managers/assembly/assemblyManager_constraints.hpp:125-138
//   * residual-only assembly  src/managers/assembly/assemblyManager_jacres.hpp:669-880
//   * fix zero rows           src/managers/assembly/assemblyManager_jacres.hpp:609-628
//   * setDirichlet            src/managers/solver/solverManager_util.hpp:60-140
//   * boundary L2 projection  src/managers/solver/solverManager_util.hpp:14-54
//   * Newton                  src/managers/solver/solverManager_solvers.hpp:290-643
//   * Jacobi PCG              src/managers/solver/solverManager_solvers.hpp:812-901
//   * CRS graph               src/interfaces/linear_algebra/linearAlgebraInterface_construct.hpp:214-265
//   * L2 / H1-semi error      src/managers/postprocess/postprocessManager_error_estimation.hpp:173-330
//   * Gauss rule of order 2p  src/interfaces/discretization/discretizationInterface_construct.hpp:111
//                             src/interfaces/discretization/discretizationInterface_integration.hpp:91-104
//   * Lagrange HGRAD bases    src/interfaces/discretization/discretizationInterface_basis.hpp:219-260
//   * boundary terms          src/physics/thermal.cpp:170-260 (Neumann, weak Dirichlet), side element
//                             size src/tools/workset.cpp:2719-2733, boundary workset loop
//                             src/managers/assembly/assemblyManager_jacres.hpp:485-603
//
// Third-party arithmetic the reference delegates (not vendored in the reference tree, versions
// unpinned beyond Trilinos >= 14): Intrepid2 HGRAD_{QUAD,HEX}_{C1,Cn} Lagrange bases, Gauss-Legendre
// cubature, CellTools Jacobian/inverse/determinant; Sacado SFad forward AD; Tpetra sumIntoValues.
// Their published algorithms are restated here: tensor-product Lagrange polynomials on [-1,1]^d with
// equispaced nodes, Gauss-Legendre points by Newton iteration on P_n, the trilinear (bilinear)
// geometric map of the 2^d cell vertices, and value+N-tangent dual numbers.
//
// Canonical numbering (the reference's Panzer/STK numbering is not in its tree, so the structured
// numbering below is the contract; the GPU library produces the same one):
//   node (ix,iy,iz) of the (p*nx+1) x (p*ny+1) x (p*nz+1) grid -> ix + NX*(iy + NY*iz)
//   cell (cx,cy,cz) -> cx + nx*(cy + ny*cz)
//   local node (a,b,c), a,b,c in [0,p], lexicographic x fastest -> a + (p+1)*(b + (p+1)*c)
//   CSR columns sorted ascending (Tpetra fillComplete order).

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <cstdio>
#include <type_traits>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ------------------------------------------------------------------------------------------
// Forward-mode dual number with N tangents (Sacado SFad semantics: value + fixed-width dx()).
// ------------------------------------------------------------------------------------------
template <int N>
struct Dual {
  double v;
  double d[N];
  Dual() : v(0.0) { for (int i = 0; i < N; ++i) d[i] = 0.0; }
  explicit Dual(double x) : v(x) { for (int i = 0; i < N; ++i) d[i] = 0.0; }
  // SFad(N, i, x): value x, tangent e_i (workset.cpp:884)
  Dual(double x, int seed) : v(x) { for (int i = 0; i < N; ++i) d[i] = (i == seed) ? 1.0 : 0.0; }
};
template <int N> inline Dual<N> operator+(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r; r.v = a.v + b.v; for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + b.d[i]; return r; }
template <int N> inline Dual<N> operator-(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r; r.v = a.v - b.v; for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - b.d[i]; return r; }
template <int N> inline Dual<N> operator*(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r; r.v = a.v * b.v; for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i]; return r; }
template <int N> inline Dual<N> operator*(const Dual<N>& a, double s) {
  Dual<N> r; r.v = a.v * s; for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * s; return r; }
template <int N> inline Dual<N> operator*(double s, const Dual<N>& a) {
  Dual<N> r; r.v = s * a.v; for (int i = 0; i < N; ++i) r.d[i] = s * a.d[i]; return r; }
template <int N> inline Dual<N>& operator+=(Dual<N>& a, const Dual<N>& b) {
  a.v += b.v; for (int i = 0; i < N; ++i) a.d[i] += b.d[i]; return a; }
inline double val(double x) { return x; }
template <int N> inline double val(const Dual<N>& x) { return x.v; }

// ------------------------------------------------------------------------------------------
// 1-D building blocks.
// ------------------------------------------------------------------------------------------
// Gauss-Legendre rule on [-1,1] exact to polynomial degree `order` (Intrepid2 DefaultCubatureFactory
// picks the Gauss rule of the requested degree): n = floor(order/2)+1 points.
void gauss_legendre(int order, std::vector<double>& x, std::vector<double>& w) {
  int n = order / 2 + 1;
  x.assign(n, 0.0);
  w.assign(n, 0.0);
  const double pi = 3.14159265358979323846;
  for (int i = 0; i < n; ++i) {
    double z = std::cos(pi * (i + 0.75) / (n + 0.5));
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = z;
      for (int k = 2; k <= n; ++k) {
        double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
        p0 = p1; p1 = p2;
      }
      double pn = (n == 1) ? z : p1;
      double pnm1 = (n == 1) ? 1.0 : p0;
      double dp = n * (z * pn - pnm1) / (z * z - 1.0);
      double dz = pn / dp;
      z -= dz;
      if (std::fabs(dz) < 1e-17) break;
    }
    double p0 = 1.0, p1 = z;
    for (int k = 2; k <= n; ++k) { double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k; p0 = p1; p1 = p2; }
    double pn = (n == 1) ? z : p1, pnm1 = (n == 1) ? 1.0 : p0;
    double dp = n * (z * pn - pnm1) / (z * z - 1.0);
    x[n - 1 - i] = z;                 // ascending order
    w[n - 1 - i] = 2.0 / ((1.0 - z * z) * dp * dp);
  }
}

// 1-D Lagrange basis of degree p on equispaced nodes of [-1,1] (POINTTYPE_EQUISPACED); node a at -1+2a/p.
void lagrange1d(int p, double xi, double* phi, double* dphi) {
  std::vector<double> nodes(p + 1);
  for (int a = 0; a <= p; ++a) nodes[a] = -1.0 + 2.0 * a / p;
  for (int a = 0; a <= p; ++a) {
    double v = 1.0;
    for (int b = 0; b <= p; ++b) if (b != a) v *= (xi - nodes[b]) / (nodes[a] - nodes[b]);
    phi[a] = v;
    double dv = 0.0;
    for (int k = 0; k <= p; ++k) {
      if (k == a) continue;
      double t = 1.0 / (nodes[a] - nodes[k]);
      for (int b = 0; b <= p; ++b) if (b != a && b != k) t *= (xi - nodes[b]) / (nodes[a] - nodes[b]);
      dv += t;
    }
    dphi[a] = dv;
  }
}

inline double sinprod(double amp, double freq, int dim, const double* x) {
  double f = amp;
  for (int k = 0; k < dim; ++k) f *= std::sin(freq * x[k]);
  return f;
}

}  // namespace

// ------------------------------------------------------------------------------------------
// Problem description (mirrors the GPU library's mrg_mesh_desc + mrg_physics_desc).
// ------------------------------------------------------------------------------------------
extern "C" {

typedef struct orc_desc {
  int32_t dim, order, nx, ny, nz;
  double lo[3], hi[3];
  const double* vertex_coords;   // optional [(nx+1)(ny+1)(nz+1)*dim]
  int32_t kind;                  // 0 thermal (kappa per cell), 1 diffusion kappa = 1 + u^2
  int32_t source_kind;           // 0 const, 1 amp*prod sin(freq*x_d)
  double source_amp, source_freq;
  double kappa_const;
  const double* kappa_cell;      // optional [ncell]
  uint32_t dirichlet_faces;      // bit k: face k (x-,x+,y-,y+,z-,z+)
  int32_t dirichlet_kind;        // 0 const, 1 per-node array, 2 sinprod nodal, 3 sinprod boundary L2 projection
  double dirichlet_const;
  const double* dirichlet_node;  // [ndof] values (kind 1)
  double dirichlet_amp, dirichlet_freq;
  int32_t quad_order;            // 0 -> 2*order
  int32_t workset_size;          // 0 -> 100 (groups.hpp:83 default)
} orc_desc;

}  // extern "C"

struct orc_problem {
  int dim, p, nx, ny, nz;
  int NX, NY, NZ;             // node grid
  int64_t ndof, ncell, nnz;
  int npe, nvpe, nq;          // nodes / vertices / quadrature points per cell
  std::vector<double> vcoord; // vertex coords [nvert*dim]
  int VX, VY, VZ;             // vertex grid
  std::vector<int32_t> lids;  // [ncell*npe]
  std::vector<int32_t> cverts;// [ncell*nvpe]
  int kind, source_kind;
  double samp, sfreq;
  std::vector<double> kappa;  // [ncell]
  std::vector<uint8_t> fixed; // [ndof]
  std::vector<int32_t> fixed_list;
  std::vector<double> fixed_vals; // [ndof]
  std::vector<int64_t> row_ptr;
  std::vector<int32_t> col_idx;
  // reference tables at quadrature points
  std::vector<double> qw;        // [nq]
  std::vector<double> phi;       // [npe*nq]
  std::vector<double> dphi;      // [npe*nq*dim] reference gradient
  std::vector<double> psi;       // [nvpe*nq] geometric basis
  std::vector<double> dpsi;      // [nvpe*nq*dim]
  std::vector<double> qxi;       // [nq*dim]
  int ws;
  int qorder;                    // 1-D Gauss order of the volume rule (the side rule uses the same)
  int bc_kind[6] = {0, 0, 0, 0, 0, 0};  // per face: 0 none, 1 Neumann, 2 weak Dirichlet
  std::vector<double> bc_g[6];          // per face: boundary data at the side points (face order)
};

namespace {

int node_id(const orc_problem* P, int ix, int iy, int iz) { return ix + P->NX * (iy + P->NY * iz); }

void build_tables(orc_problem* P, int quad_order) {
  std::vector<double> gx, gw;
  gauss_legendre(quad_order, gx, gw);
  int n1 = (int)gx.size();
  int d = P->dim, p = P->p;
  P->nq = 1; for (int k = 0; k < d; ++k) P->nq *= n1;
  P->qw.assign(P->nq, 0.0);
  P->qxi.assign(P->nq * d, 0.0);
  P->phi.assign(P->npe * P->nq, 0.0);
  P->dphi.assign(P->npe * P->nq * d, 0.0);
  P->psi.assign(P->nvpe * P->nq, 0.0);
  P->dpsi.assign(P->nvpe * P->nq * d, 0.0);
  std::vector<double> l(p + 1), dl(p + 1), l1(2), dl1(2);
  for (int q = 0; q < P->nq; ++q) {
    int qi[3] = {q % n1, (q / n1) % n1, (d == 3) ? q / (n1 * n1) : 0};
    double w = 1.0;
    for (int k = 0; k < d; ++k) { P->qxi[q * d + k] = gx[qi[k]]; w *= gw[qi[k]]; }
    P->qw[q] = w;
    // per-axis 1-D values
    double L[3][8], DL[3][8], G[3][2], DG[3][2];
    for (int k = 0; k < d; ++k) {
      lagrange1d(p, gx[qi[k]], l.data(), dl.data());
      for (int a = 0; a <= p; ++a) { L[k][a] = l[a]; DL[k][a] = dl[a]; }
      lagrange1d(1, gx[qi[k]], l1.data(), dl1.data());
      for (int a = 0; a < 2; ++a) { G[k][a] = l1[a]; DG[k][a] = dl1[a]; }
    }
    for (int i = 0; i < P->npe; ++i) {
      int a[3] = {i % (p + 1), (i / (p + 1)) % (p + 1), (d == 3) ? i / ((p + 1) * (p + 1)) : 0};
      double v = 1.0;
      for (int k = 0; k < d; ++k) v *= L[k][a[k]];
      P->phi[i * P->nq + q] = v;
      for (int g = 0; g < d; ++g) {
        double gv = 1.0;
        for (int k = 0; k < d; ++k) gv *= (k == g) ? DL[k][a[k]] : L[k][a[k]];
        P->dphi[(i * P->nq + q) * d + g] = gv;
      }
    }
    for (int i = 0; i < P->nvpe; ++i) {
      int a[3] = {i % 2, (i / 2) % 2, (d == 3) ? i / 4 : 0};
      double v = 1.0;
      for (int k = 0; k < d; ++k) v *= G[k][a[k]];
      P->psi[i * P->nq + q] = v;
      for (int g = 0; g < d; ++g) {
        double gv = 1.0;
        for (int k = 0; k < d; ++k) gv *= (k == g) ? DG[k][a[k]] : G[k][a[k]];
        P->dpsi[(i * P->nq + q) * d + g] = gv;
      }
    }
  }
}

// Geometry of one cell at all quadrature points: physical gradients, weights w*|detJ|, coordinates.
// (CellTools::setJacobian/Inv/Det, HGRADtransformGRAD, computeCellMeasure; basis.hpp:407-455,
//  integration.hpp:248-262)
void cell_geometry(const orc_problem* P, int64_t c, double* gphys /*npe*nq*dim*/, double* wdet /*nq*/,
                   double* xq /*nq*dim*/) {
  const int d = P->dim;
  double xv[8][3];
  for (int v = 0; v < P->nvpe; ++v) {
    int vid = P->cverts[c * P->nvpe + v];
    for (int k = 0; k < d; ++k) xv[v][k] = P->vcoord[(int64_t)vid * d + k];
  }
  for (int q = 0; q < P->nq; ++q) {
    double J[3][3] = {{0}};
    for (int k = 0; k < d; ++k) xq[q * d + k] = 0.0;
    for (int v = 0; v < P->nvpe; ++v) {
      double ps = P->psi[v * P->nq + q];
      for (int k = 0; k < d; ++k) {
        xq[q * d + k] += xv[v][k] * ps;
        for (int g = 0; g < d; ++g) J[k][g] += xv[v][k] * P->dpsi[(v * P->nq + q) * d + g];
      }
    }
    double det, Ji[3][3];
    if (d == 2) {
      det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
      Ji[0][0] = J[1][1] / det; Ji[0][1] = -J[0][1] / det;
      Ji[1][0] = -J[1][0] / det; Ji[1][1] = J[0][0] / det;
    } else {
      det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) - J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
            J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
      Ji[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / det;
      Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
      Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
      Ji[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) / det;
      Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
      Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
      Ji[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / det;
      Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
      Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
    }
    wdet[q] = P->qw[q] * std::fabs(det);
    // grad_phys_k = sum_g Jinv[g][k] * dref_g   (J^{-T} applied to the reference gradient)
    for (int i = 0; i < P->npe; ++i) {
      const double* dr = &P->dphi[(i * P->nq + q) * d];
      for (int k = 0; k < d; ++k) {
        double s = 0.0;
        for (int g = 0; g < d; ++g) s += Ji[g][k] * dr[g];
        gphys[(i * P->nq + q) * d + k] = s;
      }
    }
  }
}

inline void atomic_add(double* a, double v, bool atomic) {
  if (atomic) {
#ifdef _OPENMP
#pragma omp atomic
#endif
    *a += v;
  } else {
    *a += v;
  }
}

int64_t find_slot(const orc_problem* P, int64_t row, int32_t col) {
  // Tpetra sumIntoValues(isSorted=false): search the row for the column (scatter.hpp:271)
  for (int64_t k = P->row_ptr[row]; k < P->row_ptr[row + 1]; ++k)
    if (P->col_idx[k] == col) return k;
  return -1;
}

// One cell: gather, seed, fields at ip, thermal residual, scatter.  EvalT = Dual<N> or double.
template <class EvalT, int N>
void assemble_cell(const orc_problem* P, int64_t c, const double* u, double* r, double* Jv, bool jac, bool atomic,
                   double* gphys, double* wdet, double* xq) {
  const int d = P->dim, nq = P->nq, npe = P->npe;
  cell_geometry(P, c, gphys, wdet, xq);
  // gather (gather.hpp:224-232) + seed (workset.cpp:884)
  EvalT uad[N];
  for (int i = 0; i < npe; ++i) {
    double uv = u[P->lids[c * npe + i]];
    if constexpr (std::is_same<EvalT, double>::value) uad[i] = uv; else uad[i] = EvalT(uv, i);
  }
  // solution fields at ip (workset.cpp:1093-1105)
  EvalT T[64], dT[64][3];
  for (int q = 0; q < nq; ++q) {
    T[q] = uad[0] * P->phi[0 * nq + q];
    for (int k = 0; k < d; ++k) dT[q][k] = uad[0] * gphys[(0 * nq + q) * d + k];
    for (int i = 1; i < npe; ++i) {
      T[q] += uad[i] * P->phi[i * nq + q];
      for (int k = 0; k < d; ++k) dT[q][k] += uad[i] * gphys[(i * nq + q) * d + k];
    }
  }
  // coefficients at ip ("thermal source", "thermal diffusion"; thermal.cpp:81-84)
  double src[64];
  EvalT diff[64];
  for (int q = 0; q < nq; ++q) {
    src[q] = (P->source_kind == 0) ? P->samp : sinprod(P->samp, P->sfreq, d, &xq[q * d]);
    if (P->kind == 0) diff[q] = EvalT(P->kappa[c]);
    else diff[q] = EvalT(1.0) + T[q] * T[q];
  }
  // residual (thermal.cpp:125-137): res(e,i) += (-f)*w*phi + diff*dT/dx_k*w*dphi_k
  EvalT res[N];
  for (int i = 0; i < npe; ++i) {
    res[i] = EvalT(0.0);
    for (int q = 0; q < nq; ++q) {
      double w = wdet[q];
      res[i] += EvalT((0.0 - src[q]) * w * P->phi[i * nq + q]);
      for (int k = 0; k < d; ++k) res[i] += diff[q] * dT[q][k] * w * gphys[(i * nq + q) * d + k];
    }
  }
  // scatter (scatter.hpp:196-277): r[row] += -res.val, J(row, LIDs) += res.dx, fixed rows skipped
  for (int i = 0; i < npe; ++i) {
    int32_t row = P->lids[c * npe + i];
    if (P->fixed[row]) continue;
    if (r) atomic_add(&r[row], -val(res[i]), atomic);
    if constexpr (!std::is_same<EvalT, double>::value) {
      if (jac) {
        for (int j = 0; j < npe; ++j) {
          int64_t s = find_slot(P, row, P->lids[c * npe + j]);
          atomic_add(&Jv[s], res[i].d[j], atomic);
        }
      }
    }
  }
}

// ------------------------------------------------------------------------------------------
// Boundary terms (thermal.cpp:170-260).  Face f = 2a + s: a = normal axis, s = 0 (low) / 1 (high).
// Side points: the volume rule's 1-D Gauss points on the tangential axes (first tangential axis
// fastest), xi_a = -1 or +1.  Face cells are ordered by their tangential cell coordinates (first
// tangential axis fastest); the boundary data of a face is one value per (face cell, side point).
// ------------------------------------------------------------------------------------------
void side_rule(const orc_problem* P, int face, std::vector<double>& xi, std::vector<double>& wr) {
  std::vector<double> gx, gw;
  gauss_legendre(P->qorder, gx, gw);
  const int n1 = (int)gx.size(), d = P->dim, a = face / 2;
  int t[2] = {-1, -1}, nt = 0;
  for (int k = 0; k < d; ++k)
    if (k != a) t[nt++] = k;
  const int npts = (d == 3) ? n1 * n1 : n1;
  xi.assign((size_t)npts * d, 0.0);
  wr.assign(npts, 1.0);
  for (int q = 0; q < npts; ++q) {
    const int i0 = q % n1, i1 = q / n1;
    xi[(size_t)q * d + a] = (face % 2) ? 1.0 : -1.0;
    xi[(size_t)q * d + t[0]] = gx[i0];
    wr[q] = gw[i0];
    if (d == 3) {
      xi[(size_t)q * d + t[1]] = gx[i1];
      wr[q] *= gw[i1];
    }
  }
}

std::vector<int64_t> face_cells(const orc_problem* P, int face) {
  const int d = P->dim, a = face / 2;
  const int nc[3] = {P->nx, P->ny, P->nz};
  int t[2] = {-1, -1}, nt = 0;
  for (int k = 0; k < d; ++k)
    if (k != a) t[nt++] = k;
  const int n0 = nc[t[0]], n1 = (d == 3) ? nc[t[1]] : 1;
  std::vector<int64_t> out;
  out.reserve((size_t)n0 * n1);
  for (int j = 0; j < n1; ++j)
    for (int i = 0; i < n0; ++i) {
      int cc[3] = {0, 0, 0};
      cc[a] = (face % 2) ? nc[a] - 1 : 0;
      cc[t[0]] = i;
      if (d == 3) cc[t[1]] = j;
      out.push_back(cc[0] + (int64_t)P->nx * (cc[1] + (int64_t)P->ny * cc[2]));
    }
  return out;
}

// Cell c at the side points of `face`: coordinates x, basis values phi [npe][npts], physical gradients
// gphys [npe][npts][dim], weights w = w_ref * side measure, outward unit normal nrm [npts][dim].
// (CellTools Jacobian; side measure |dx/dxi_t| (2-D) or |dx/dxi_t1 x dx/dxi_t2| (3-D); normal
// +-J^{-T} e_a normalised.)
void side_geometry(const orc_problem* P, int64_t c, int face, const std::vector<double>& xi,
                   const std::vector<double>& wr, double* x, double* phi, double* gphys, double* w, double* nrm) {
  const int d = P->dim, p = P->p, a = face / 2;
  const int npts = (int)wr.size();
  double xv[8][3];
  for (int v = 0; v < P->nvpe; ++v) {
    const int vid = P->cverts[c * P->nvpe + v];
    for (int k = 0; k < d; ++k) xv[v][k] = P->vcoord[(int64_t)vid * d + k];
  }
  std::vector<double> l(p + 1), dl(p + 1);
  for (int q = 0; q < npts; ++q) {
    const double* e = &xi[(size_t)q * d];
    double L[3][8], DL[3][8], G[3][2], DG[3][2];
    double l1[2], dl1[2];
    for (int k = 0; k < d; ++k) {
      lagrange1d(p, e[k], l.data(), dl.data());
      for (int b = 0; b <= p; ++b) { L[k][b] = l[b]; DL[k][b] = dl[b]; }
      lagrange1d(1, e[k], l1, dl1);
      for (int b = 0; b < 2; ++b) { G[k][b] = l1[b]; DG[k][b] = dl1[b]; }
    }
    double J[3][3] = {{0}};
    for (int k = 0; k < d; ++k) x[q * d + k] = 0.0;
    for (int v = 0; v < P->nvpe; ++v) {
      const int av[3] = {v % 2, (v / 2) % 2, v / 4};
      double ps = 1.0;
      for (int k = 0; k < d; ++k) ps *= G[k][av[k]];
      for (int k = 0; k < d; ++k) {
        x[q * d + k] += xv[v][k] * ps;
        for (int gg = 0; gg < d; ++gg) {
          double dp = 1.0;
          for (int m = 0; m < d; ++m) dp *= (m == gg) ? DG[m][av[m]] : G[m][av[m]];
          J[k][gg] += xv[v][k] * dp;
        }
      }
    }
    double det, Ji[3][3];
    if (d == 2) {
      det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
      Ji[0][0] = J[1][1] / det; Ji[0][1] = -J[0][1] / det;
      Ji[1][0] = -J[1][0] / det; Ji[1][1] = J[0][0] / det;
    } else {
      det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) - J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
            J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
      Ji[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / det;
      Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
      Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
      Ji[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) / det;
      Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
      Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
      Ji[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / det;
      Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
      Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
    }
    // side measure from the tangential columns of J
    int t[2] = {-1, -1}, nt = 0;
    for (int k = 0; k < d; ++k)
      if (k != a) t[nt++] = k;
    double meas;
    if (d == 2) {
      meas = std::sqrt(J[0][t[0]] * J[0][t[0]] + J[1][t[0]] * J[1][t[0]]);
    } else {
      const double u0[3] = {J[0][t[0]], J[1][t[0]], J[2][t[0]]}, u1[3] = {J[0][t[1]], J[1][t[1]], J[2][t[1]]};
      const double cr[3] = {u0[1] * u1[2] - u0[2] * u1[1], u0[2] * u1[0] - u0[0] * u1[2], u0[0] * u1[1] - u0[1] * u1[0]};
      meas = std::sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
    }
    w[q] = wr[q] * meas;
    double nv[3], nn2 = 0.0;
    for (int k = 0; k < d; ++k) { nv[k] = Ji[a][k]; nn2 += nv[k] * nv[k]; }
    const double sgn = (face % 2) ? 1.0 : -1.0, inv = sgn / std::sqrt(nn2);
    for (int k = 0; k < d; ++k) nrm[q * d + k] = nv[k] * inv;
    for (int i = 0; i < P->npe; ++i) {
      const int ai[3] = {i % (p + 1), (i / (p + 1)) % (p + 1), (d == 3) ? i / ((p + 1) * (p + 1)) : 0};
      double v = 1.0, dr[3];
      for (int k = 0; k < d; ++k) v *= L[k][ai[k]];
      for (int gg = 0; gg < d; ++gg) {
        double gv = 1.0;
        for (int k = 0; k < d; ++k) gv *= (k == gg) ? DL[k][ai[k]] : L[k][ai[k]];
        dr[gg] = gv;
      }
      phi[i * npts + q] = v;
      for (int k = 0; k < d; ++k) {
        double sg = 0.0;
        for (int gg = 0; gg < d; ++gg) sg += Ji[gg][k] * dr[gg];
        gphys[((size_t)i * npts + q) * d + k] = sg;
      }
    }
  }
}

// One boundary cell side: thermal boundaryResidual (thermal.cpp:209-260) and the same scatter as the
// volume terms.  Neumann: res_i += -g w phi_i.  Weak Dirichlet (Nitsche, epen = 10, form_param = 1):
// res_i += epen/h kappa (T - g) w phi_i - kappa (grad T . n) w phi_i - kappa (T - g) w (grad phi_i . n),
// h = (sum of the side weights)^(1/(dim-1)) (workset.cpp:2719-2733).
template <class EvalT, int N>
void boundary_cell(const orc_problem* P, int64_t c, int face, int64_t k, const std::vector<double>& xi,
                   const std::vector<double>& wr, const double* u, double* r, double* Jv, bool jac, bool atomic) {
  const int d = P->dim, npe = P->npe, npts = (int)wr.size();
  std::vector<double> x((size_t)npts * d), phi((size_t)npe * npts), gphys((size_t)npe * npts * d), w(npts),
      nrm((size_t)npts * d);
  side_geometry(P, c, face, xi, wr, x.data(), phi.data(), gphys.data(), w.data(), nrm.data());
  EvalT uad[N];
  for (int i = 0; i < npe; ++i) {
    const double uv = u[P->lids[c * npe + i]];
    if constexpr (std::is_same<EvalT, double>::value) uad[i] = uv; else uad[i] = EvalT(uv, i);
  }
  const double* g = P->bc_g[face].data() + (size_t)k * npts;
  double hs = 0.0;
  for (int q = 0; q < npts; ++q) hs += w[q];
  const double h = (d == 2) ? hs : std::pow(hs, 1.0 / (d - 1.0));
  const double epen = 10.0, sf = 1.0;
  EvalT res[N];
  for (int i = 0; i < npe; ++i) res[i] = EvalT(0.0);
  for (int q = 0; q < npts; ++q) {
    if (P->bc_kind[face] == 1) {
      for (int i = 0; i < npe; ++i) res[i] += EvalT(-g[q] * w[q] * phi[i * npts + q]);
      continue;
    }
    EvalT T = uad[0] * phi[0 * npts + q], dTn = EvalT(0.0);
    for (int i = 1; i < npe; ++i) T += uad[i] * phi[i * npts + q];
    for (int i = 0; i < npe; ++i) {
      double gn = 0.0;
      for (int m = 0; m < d; ++m) gn += gphys[((size_t)i * npts + q) * d + m] * nrm[q * d + m];
      dTn += uad[i] * gn;
    }
    const EvalT diff = (P->kind == 0) ? EvalT(P->kappa[c]) : EvalT(1.0) + T * T;
    const EvalT jump = T - EvalT(g[q]);
    for (int i = 0; i < npe; ++i) {
      double gin = 0.0;
      for (int m = 0; m < d; ++m) gin += gphys[((size_t)i * npts + q) * d + m] * nrm[q * d + m];
      res[i] += (epen / h) * diff * jump * (w[q] * phi[i * npts + q]);
      res[i] += (-1.0) * diff * dTn * (w[q] * phi[i * npts + q]);
      res[i] += (-sf) * diff * jump * (w[q] * gin);
    }
  }
  for (int i = 0; i < npe; ++i) {
    const int32_t row = P->lids[c * npe + i];
    if (P->fixed[row]) continue;
    if (r) atomic_add(&r[row], -val(res[i]), atomic);
    if constexpr (!std::is_same<EvalT, double>::value) {
      if (jac)
        for (int j = 0; j < npe; ++j) atomic_add(&Jv[find_slot(P, row, P->lids[c * npe + j])], res[i].d[j], atomic);
    }
  }
}

template <int N>
void assemble_boundary(orc_problem* P, const double* u, double* r, double* Jv, bool jac, int nthreads) {
  const bool atomic = nthreads > 1;
  for (int face = 0; face < 2 * P->dim; ++face) {
    if (!P->bc_kind[face]) continue;
    std::vector<double> xi, wr;
    side_rule(P, face, xi, wr);
    const std::vector<int64_t> cells = face_cells(P, face);
    const int64_t nfc = (int64_t)cells.size();
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads) if (nthreads > 1) schedule(static)
#endif
    for (int64_t k = 0; k < nfc; ++k) {
      if (jac) boundary_cell<Dual<N>, N>(P, cells[k], face, k, xi, wr, u, r, Jv, true, atomic);
      else boundary_cell<double, N>(P, cells[k], face, k, xi, wr, u, r, Jv, false, atomic);
    }
  }
}

template <int N>
void assemble_all(orc_problem* P, const double* u, double* r, double* Jv, int flags, int nthreads) {
  bool jac = (flags & 2) && Jv;
  bool atomic = nthreads > 1;
  const int npe = P->npe, nq = P->nq, d = P->dim;
  // sequential groups of `ws` cells (jacres:336); the cells of one group run in parallel
  for (int64_t g0 = 0; g0 < P->ncell; g0 += P->ws) {
    int64_t g1 = std::min<int64_t>(P->ncell, g0 + P->ws);
#ifdef _OPENMP
#pragma omp parallel num_threads(nthreads) if (nthreads > 1)
#endif
    {
      std::vector<double> gphys(npe * nq * d), wdet(nq), xq(nq * d);
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
      for (int64_t c = g0; c < g1; ++c) {
        if (jac) assemble_cell<Dual<N>, N>(P, c, u, r, Jv, true, atomic, gphys.data(), wdet.data(), xq.data());
        else assemble_cell<double, N>(P, c, u, r, Jv, false, atomic, gphys.data(), wdet.data(), xq.data());
      }
    }
  }
  // boundary workset loop (jacres:485-603)
  assemble_boundary<N>(P, u, r, Jv, jac, nthreads);
  // dofConstraints -> setJacobianConstraints: J(d,d) = 1 (constraints.hpp:125-138)
  if (jac) {
    for (int32_t dd : P->fixed_list) Jv[find_slot(P, dd, dd)] = 1.0;
    if (flags & 16) {  // fix zero rows (jacres:609-628)
      for (int64_t row = 0; row < P->ndof; ++row) {
        double s = 0.0;
        for (int64_t k = P->row_ptr[row]; k < P->row_ptr[row + 1]; ++k) s += std::fabs(Jv[k]);
        if (s < 1.0e-14) Jv[find_slot(P, row, (int32_t)row)] = 1.0;
      }
    }
  }
}

void spmv(const orc_problem* P, const double* Jv, const double* x, double* y, int nthreads) {
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads) if (nthreads > 1) schedule(static)
#endif
  for (int64_t i = 0; i < P->ndof; ++i) {
    double s = 0.0;
    for (int64_t k = P->row_ptr[i]; k < P->row_ptr[i + 1]; ++k) s += Jv[k] * x[P->col_idx[k]];
    y[i] = s;
  }
}

double dot(const double* a, const double* b, int64_t n, int nthreads) {
  double s = 0.0;
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads) if (nthreads > 1) reduction(+ : s) schedule(static)
#endif
  for (int64_t i = 0; i < n; ++i) s += a[i] * b[i];
  return s;
}

}  // namespace

extern "C" {

void orc_destroy(orc_problem* P) { delete P; }

// Builds mesh, DOF map, CRS graph, reference tables, Dirichlet data.  Returns nullptr on bad input.
orc_problem* orc_create(const orc_desc* D) {
  if (!D || (D->dim != 2 && D->dim != 3) || D->order < 1 || D->order > 4 || D->nx < 1 || D->ny < 1 ||
      (D->dim == 3 && D->nz < 1))
    return nullptr;
  if (D->dim == 3 && D->order > 2) return nullptr;
  orc_problem* P = new orc_problem();
  P->dim = D->dim; P->p = D->order; P->nx = D->nx; P->ny = D->ny; P->nz = (D->dim == 3) ? D->nz : 1;
  P->NX = P->p * P->nx + 1; P->NY = P->p * P->ny + 1; P->NZ = (P->dim == 3) ? P->p * P->nz + 1 : 1;
  P->VX = P->nx + 1; P->VY = P->ny + 1; P->VZ = (P->dim == 3) ? P->nz + 1 : 1;
  P->ndof = (int64_t)P->NX * P->NY * P->NZ;
  P->ncell = (int64_t)P->nx * P->ny * P->nz;
  P->npe = 1; P->nvpe = 1;
  for (int k = 0; k < P->dim; ++k) { P->npe *= (P->p + 1); P->nvpe *= 2; }
  P->ws = D->workset_size > 0 ? D->workset_size : 100;
  // vertices
  int64_t nvert = (int64_t)P->VX * P->VY * P->VZ;
  P->vcoord.assign(nvert * P->dim, 0.0);
  for (int64_t v = 0; v < nvert; ++v) {
    int iv[3] = {(int)(v % P->VX), (int)((v / P->VX) % P->VY), (int)(v / ((int64_t)P->VX * P->VY))};
    int nn[3] = {P->nx, P->ny, P->nz};
    for (int k = 0; k < P->dim; ++k) {
      if (D->vertex_coords) P->vcoord[v * P->dim + k] = D->vertex_coords[v * P->dim + k];
      else P->vcoord[v * P->dim + k] = D->lo[k] + (D->hi[k] - D->lo[k]) * iv[k] / nn[k];
    }
  }
  // connectivity
  P->lids.assign(P->ncell * P->npe, 0);
  P->cverts.assign(P->ncell * P->nvpe, 0);
  for (int64_t c = 0; c < P->ncell; ++c) {
    int cx = (int)(c % P->nx), cy = (int)((c / P->nx) % P->ny), cz = (int)(c / ((int64_t)P->nx * P->ny));
    for (int i = 0; i < P->npe; ++i) {
      int a = i % (P->p + 1), b = (i / (P->p + 1)) % (P->p + 1), e = (P->dim == 3) ? i / ((P->p + 1) * (P->p + 1)) : 0;
      P->lids[c * P->npe + i] = node_id(P, P->p * cx + a, P->p * cy + b, (P->dim == 3) ? P->p * cz + e : 0);
    }
    for (int i = 0; i < P->nvpe; ++i) {
      int a = i % 2, b = (i / 2) % 2, e = (P->dim == 3) ? i / 4 : 0;
      P->cverts[c * P->nvpe + i] = (cx + a) + P->VX * ((cy + b) + P->VY * (cz + e));
    }
  }
  // coefficients
  P->kind = D->kind; P->source_kind = D->source_kind; P->samp = D->source_amp; P->sfreq = D->source_freq;
  P->kappa.assign(P->ncell, D->kappa_const);
  if (D->kappa_cell) for (int64_t c = 0; c < P->ncell; ++c) P->kappa[c] = D->kappa_cell[c];
  // CRS graph: union of element couplings, sorted columns (LA construct.hpp:214-265)
  {
    std::vector<int64_t> cnt(P->ndof + 1, 0);
    // structured: row couplings are a product of per-axis ranges; build generically by marking
    std::vector<std::vector<int32_t>> rows(P->ndof);
    for (int64_t c = 0; c < P->ncell; ++c)
      for (int i = 0; i < P->npe; ++i) {
        auto& R = rows[P->lids[c * P->npe + i]];
        for (int j = 0; j < P->npe; ++j) R.push_back(P->lids[c * P->npe + j]);
      }
    P->row_ptr.assign(P->ndof + 1, 0);
    for (int64_t i = 0; i < P->ndof; ++i) {
      auto& R = rows[i];
      std::sort(R.begin(), R.end());
      R.erase(std::unique(R.begin(), R.end()), R.end());
      P->row_ptr[i + 1] = P->row_ptr[i] + (int64_t)R.size();
    }
    P->nnz = P->row_ptr[P->ndof];
    P->col_idx.resize(P->nnz);
    for (int64_t i = 0; i < P->ndof; ++i) {
      std::copy(rows[i].begin(), rows[i].end(), P->col_idx.begin() + P->row_ptr[i]);
      std::vector<int32_t>().swap(rows[i]);
    }
  }
  // tables
  P->qorder = D->quad_order > 0 ? D->quad_order : 2 * P->p;
  build_tables(P, P->qorder);
  // Dirichlet DOFs: nodes on the selected faces, in increasing DOF order
  P->fixed.assign(P->ndof, 0);
  P->fixed_vals.assign(P->ndof, 0.0);
  for (int64_t n = 0; n < P->ndof; ++n) {
    int ix = (int)(n % P->NX), iy = (int)((n / P->NX) % P->NY), iz = (int)(n / ((int64_t)P->NX * P->NY));
    uint32_t f = D->dirichlet_faces;
    bool on = ((f & 1) && ix == 0) || ((f & 2) && ix == P->NX - 1) || ((f & 4) && iy == 0) ||
              ((f & 8) && iy == P->NY - 1) ||
              (P->dim == 3 && (((f & 16) && iz == 0) || ((f & 32) && iz == P->NZ - 1)));
    if (on) { P->fixed[n] = 1; P->fixed_list.push_back((int32_t)n); }
  }
  // node coordinates (vertex grid interpolated for p>1 through the geometric map)
  auto node_x = [&](int64_t n, double* x) {
    int ix = (int)(n % P->NX), iy = (int)((n / P->NX) % P->NY), iz = (int)(n / ((int64_t)P->NX * P->NY));
    int ii[3] = {ix, iy, iz};
    int cc[3], nn[3] = {P->nx, P->ny, P->nz};
    double xi[3];
    for (int k = 0; k < P->dim; ++k) {
      cc[k] = std::min(ii[k] / P->p, nn[k] - 1);
      xi[k] = -1.0 + 2.0 * (double)(ii[k] - P->p * cc[k]) / P->p;
    }
    for (int k = 0; k < P->dim; ++k) x[k] = 0.0;
    for (int v = 0; v < P->nvpe; ++v) {
      int a[3] = {v % 2, (v / 2) % 2, v / 4};
      double w = 1.0;
      for (int k = 0; k < P->dim; ++k) w *= a[k] ? 0.5 * (1.0 + xi[k]) : 0.5 * (1.0 - xi[k]);
      int64_t vid = (cc[0] + a[0]) + (int64_t)P->VX * ((cc[1] + a[1]) + (int64_t)P->VY * ((P->dim == 3 ? cc[2] : 0) + (P->dim == 3 ? a[2] : 0)));
      for (int k = 0; k < P->dim; ++k) x[k] += w * P->vcoord[vid * P->dim + k];
    }
  };
  for (int32_t n : P->fixed_list) {
    double v = D->dirichlet_const;
    if (D->dirichlet_kind == 1 && D->dirichlet_node) v = D->dirichlet_node[n];
    if (D->dirichlet_kind == 2 || D->dirichlet_kind == 3) {
      double x[3];
      node_x(n, x);
      v = sinprod(D->dirichlet_amp, D->dirichlet_freq, P->dim, x);
    }
    P->fixed_vals[n] = v;
  }
  if (D->dirichlet_kind == 3) {
    // Boundary L2 projection of g = amp*prod sin(freq x) onto the trace space on the Dirichlet faces
    // (projectDirichlet, solverManager_util.hpp:14-54): M_b x = int_{dOmega_D} g phi, solved for the
    // boundary DOFs by CG.  Side quadrature uses the volume rule's 1-D points.
    std::vector<double> gx, gw;
    gauss_legendre(D->quad_order > 0 ? D->quad_order : 2 * P->p, gx, gw);
    int n1 = (int)gx.size();
    std::vector<double> rhs(P->ndof, 0.0);
    std::vector<std::vector<std::pair<int32_t, double>>> M(P->ndof);
    int p = P->p, d = P->dim;
    std::vector<double> l(p + 1), dl(p + 1);
    for (int face = 0; face < 2 * d; ++face) {
      if (!(D->dirichlet_faces & (1u << face))) continue;
      int ax = face / 2, hiside = face % 2;
      int nn[3] = {P->nx, P->ny, P->nz};
      // iterate cells touching this face
      for (int64_t c = 0; c < P->ncell; ++c) {
        int cc[3] = {(int)(c % P->nx), (int)((c / P->nx) % P->ny), (int)(c / ((int64_t)P->nx * P->ny))};
        if (cc[ax] != (hiside ? nn[ax] - 1 : 0)) continue;
        int tang[2], nt = 0;
        for (int k = 0; k < d; ++k) if (k != ax) tang[nt++] = k;
        int nsq = (nt == 1) ? n1 : n1 * n1;
        // face-local nodes: local index with coordinate along ax fixed
        std::vector<int> fnodes;
        for (int i = 0; i < P->npe; ++i) {
          int a[3] = {i % (p + 1), (i / (p + 1)) % (p + 1), i / ((p + 1) * (p + 1))};
          if (a[ax] == (hiside ? p : 0)) fnodes.push_back(i);
        }
        for (int sq = 0; sq < nsq; ++sq) {
          int si[2] = {sq % n1, sq / n1};
          double xi[3];
          xi[ax] = hiside ? 1.0 : -1.0;
          double w = 1.0;
          for (int t = 0; t < nt; ++t) { xi[tang[t]] = gx[si[t]]; w *= gw[si[t]]; }
          // geometric map and surface measure
          double x[3] = {0, 0, 0}, dx[3][3] = {{0}};
          for (int v = 0; v < P->nvpe; ++v) {
            int a[3] = {v % 2, (v / 2) % 2, v / 4};
            int vid = P->cverts[c * P->nvpe + v];
            double g1[3], dg1[3];
            for (int k = 0; k < d; ++k) { g1[k] = a[k] ? 0.5 * (1 + xi[k]) : 0.5 * (1 - xi[k]); dg1[k] = a[k] ? 0.5 : -0.5; }
            double val = 1.0;
            for (int k = 0; k < d; ++k) val *= g1[k];
            for (int k = 0; k < d; ++k) x[k] += val * P->vcoord[(int64_t)vid * d + k];
            for (int t = 0; t < nt; ++t) {
              double dv = 1.0;
              for (int k = 0; k < d; ++k) dv *= (k == tang[t]) ? dg1[k] : g1[k];
              for (int k = 0; k < d; ++k) dx[t][k] += dv * P->vcoord[(int64_t)vid * d + k];
            }
          }
          double meas;
          if (nt == 1) meas = std::sqrt(dx[0][0] * dx[0][0] + dx[0][1] * dx[0][1]);
          else {
            double cr[3] = {dx[0][1] * dx[1][2] - dx[0][2] * dx[1][1], dx[0][2] * dx[1][0] - dx[0][0] * dx[1][2],
                            dx[0][0] * dx[1][1] - dx[0][1] * dx[1][0]};
            meas = std::sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
          }
          double gval = sinprod(D->dirichlet_amp, D->dirichlet_freq, d, x);
          // basis values on the face
          std::vector<double> phv(fnodes.size());
          for (size_t fi = 0; fi < fnodes.size(); ++fi) {
            int i = fnodes[fi];
            int a[3] = {i % (p + 1), (i / (p + 1)) % (p + 1), i / ((p + 1) * (p + 1))};
            double v = 1.0;
            for (int k = 0; k < d; ++k) { lagrange1d(p, xi[k], l.data(), dl.data()); v *= l[a[k]]; }
            phv[fi] = v;
          }
          for (size_t fi = 0; fi < fnodes.size(); ++fi) {
            int32_t row = P->lids[c * P->npe + fnodes[fi]];
            rhs[row] += gval * phv[fi] * w * meas;
            for (size_t fj = 0; fj < fnodes.size(); ++fj) {
              int32_t col = P->lids[c * P->npe + fnodes[fj]];
              double mv = phv[fi] * phv[fj] * w * meas;
              bool found = false;
              for (auto& e : M[row]) if (e.first == col) { e.second += mv; found = true; break; }
              if (!found) M[row].push_back({col, mv});
            }
          }
        }
      }
    }
    // CG on the boundary mass system (restricted to DOFs that appear)
    std::vector<double> x(P->ndof, 0.0), r(rhs), pp(P->ndof, 0.0), Ap(P->ndof, 0.0);
    auto apply = [&](const std::vector<double>& in, std::vector<double>& out) {
      for (int64_t i = 0; i < P->ndof; ++i) { double s = 0; for (auto& e : M[i]) s += e.second * in[e.first]; out[i] = s; }
    };
    double rr = 0; for (double v : r) rr += v * v;
    double rr0 = rr;
    pp = r;
    for (int it = 0; it < 10000 && rr > 1e-32 * rr0 && rr > 0; ++it) {
      apply(pp, Ap);
      double pAp = 0; for (int64_t i = 0; i < P->ndof; ++i) pAp += pp[i] * Ap[i];
      double a = rr / pAp;
      for (int64_t i = 0; i < P->ndof; ++i) { x[i] += a * pp[i]; r[i] -= a * Ap[i]; }
      double rn = 0; for (double v : r) rn += v * v;
      double b = rn / rr; rr = rn;
      for (int64_t i = 0; i < P->ndof; ++i) pp[i] = r[i] + b * pp[i];
    }
    for (int32_t n : P->fixed_list) P->fixed_vals[n] = x[n];
  }
  return P;
}

void orc_sizes(const orc_problem* P, int64_t* out /* ndof, ncell, nnz, nfixed, npe, nq */) {
  out[0] = P->ndof; out[1] = P->ncell; out[2] = P->nnz; out[3] = (int64_t)P->fixed_list.size();
  out[4] = P->npe; out[5] = P->nq;
}
void orc_graph(const orc_problem* P, int64_t* row_ptr, int32_t* col_idx) {
  std::memcpy(row_ptr, P->row_ptr.data(), sizeof(int64_t) * (P->ndof + 1));
  std::memcpy(col_idx, P->col_idx.data(), sizeof(int32_t) * P->nnz);
}
void orc_dof_map(const orc_problem* P, int32_t* lids) {
  std::memcpy(lids, P->lids.data(), sizeof(int32_t) * P->ncell * P->npe);
}
void orc_fixed(const orc_problem* P, int32_t* dofs, double* vals) {
  for (size_t i = 0; i < P->fixed_list.size(); ++i) {
    dofs[i] = P->fixed_list[i];
    if (vals) vals[i] = P->fixed_vals[P->fixed_list[i]];
  }
}
void orc_set_kappa(orc_problem* P, const double* kappa) {
  for (int64_t c = 0; c < P->ncell; ++c) P->kappa[c] = kappa[c];
}

// u[fixed] = g (setDirichlet, solverManager_util.hpp:86-118)
void orc_set_dirichlet(const orc_problem* P, double* u) {
  for (int32_t n : P->fixed_list) u[n] = P->fixed_vals[n];
}

// Sum-into assembly.  flags: 1 residual, 2 Jacobian (AD), 16 fix zero rows.
// Caller zeroes r and J first, as SolverManager::nonlinearSolver does (putScalar(0)/setAllToScalar(0)).
int orc_assemble(orc_problem* P, const double* u, double* r, double* Jv, int flags, int nthreads) {
  if (!(flags & 1)) r = nullptr;
  switch (P->npe) {
    case 4: assemble_all<4>(P, u, r, Jv, flags, nthreads); break;
    case 8: assemble_all<8>(P, u, r, Jv, flags, nthreads); break;
    case 9: assemble_all<9>(P, u, r, Jv, flags, nthreads); break;
    case 16: assemble_all<16>(P, u, r, Jv, flags, nthreads); break;
    case 25: assemble_all<25>(P, u, r, Jv, flags, nthreads); break;
    case 27: assemble_all<27>(P, u, r, Jv, flags, nthreads); break;
    default: return 1;
  }
  return 0;
}

// Time-limited assembly of the first `ncell_sample` cells only (CPU baseline sampling).
int orc_assemble_sample(orc_problem* P, const double* u, double* r, double* Jv, int flags, int nthreads,
                        int64_t ncell_sample) {
  int64_t keep = P->ncell;
  P->ncell = std::min<int64_t>(keep, ncell_sample);
  int rc = orc_assemble(P, u, r, Jv, flags, nthreads);
  P->ncell = keep;
  return rc;
}

void orc_spmv(const orc_problem* P, const double* Jv, const double* x, double* y, int nthreads) {
  spmv(P, Jv, x, y, nthreads);
}

// Jacobi PCG exactly as SolverManager::PCG (solverManager_solvers.hpp:812-901); M = diag(J).
// Returns iterations; *relres = ||r||/||r0||.
int orc_pcg(const orc_problem* P, const double* Jv, const double* b, double* x, double tol, int maxiter,
            int nthreads, double* relres) {
  int64_t n = P->ndof;
  std::vector<double> p(n, 0.0), q(n, 0.0), r(n, 0.0), z(n, 0.0), M(n, 1.0);
  for (int64_t i = 0; i < n; ++i) {
    int64_t s = find_slot(P, i, (int32_t)i);
    M[i] = (s >= 0) ? Jv[s] : 1.0;
  }
  spmv(P, Jv, x, q.data(), nthreads);
  for (int64_t i = 0; i < n; ++i) r[i] = b[i] - q[i];
  double rnorm = std::sqrt(dot(r.data(), r.data(), n, nthreads));
  double r0 = rnorm;
  double rho = 1.0, rho1, beta, alpha, pq;
  int iter = 0;
  if (r0 == 0.0) { if (relres) *relres = 0.0; return 0; }
  while (iter < maxiter && rnorm / r0 > tol) {
    for (int64_t k = 0; k < n; ++k) z[k] = r[k] / M[k];
    rho1 = rho;
    rho = dot(r.data(), z.data(), n, nthreads);
    if (iter == 0) p = z;
    else { beta = rho / rho1; for (int64_t k = 0; k < n; ++k) p[k] = z[k] + beta * p[k]; }
    spmv(P, Jv, p.data(), q.data(), nthreads);
    pq = dot(p.data(), q.data(), n, nthreads);
    alpha = rho / pq;
    for (int64_t k = 0; k < n; ++k) { x[k] += alpha * p[k]; r[k] -= alpha * q[k]; }
    rnorm = std::sqrt(dot(r.data(), r.data(), n, nthreads));
    iter++;
  }
  if (relres) *relres = rnorm / r0;
  return iter;
}

// Newton (solverManager_solvers.hpp:290-643, relative inf-norm test, autotune path: residual-only
// assembly, then Jacobian+residual assembly when a solve is needed) with Jacobi PCG as the linear
// solver.  u must already hold the Dirichlet values.  stats: [iters, final scaled norm, total cg its]
int orc_newton(orc_problem* P, double* u, double nltol, int maxiter, double lintol, int linmaxiter, int nthreads,
               double* stats) {
  int64_t n = P->ndof;
  std::vector<double> r(n), Jv(P->nnz), du(n);
  double first = 0.0, scaled = 1.0;
  int it = 0, cgtot = 0;
  bool proceed = true;
  while (proceed) {
    std::fill(r.begin(), r.end(), 0.0);
    orc_assemble(P, u, r.data(), nullptr, 1, nthreads);
    double nrm = 0.0;
    for (double v : r) nrm = std::max(nrm, std::fabs(v));
    if (it == 0) { first = nrm; scaled = 1.0; } else scaled = nrm / first;
    bool solve = true;
    if (scaled < nltol || nrm < 1.0e-100) { solve = false; proceed = false; }
    if (solve) {
      std::fill(Jv.begin(), Jv.end(), 0.0);
      std::fill(r.begin(), r.end(), 0.0);
      orc_assemble(P, u, r.data(), Jv.data(), 3, nthreads);
      std::fill(du.begin(), du.end(), 0.0);
      double rr;
      cgtot += orc_pcg(P, Jv.data(), r.data(), du.data(), lintol, linmaxiter, nthreads, &rr);
      for (int64_t i = 0; i < n; ++i) u[i] += du[i];
    }
    it++;
    if (it >= maxiter) proceed = false;
  }
  if (stats) { stats[0] = it; stats[1] = scaled; stats[2] = cgtot; }
  return (scaled < nltol) ? 0 : 1;
}

// L2 error of u_h against amp*prod sin(freq x) and H1-seminorm error against its gradient, at the
// volume quadrature points (computeError, postprocessManager_error_estimation.hpp:252-330).
void orc_errors(const orc_problem* P, const double* u, double amp, double freq, double* l2, double* h1) {
  const int d = P->dim, nq = P->nq, npe = P->npe;
  std::vector<double> gphys(npe * nq * d), wdet(nq), xq(nq * d);
  double e2 = 0.0, g2 = 0.0;
  for (int64_t c = 0; c < P->ncell; ++c) {
    cell_geometry(P, c, gphys.data(), wdet.data(), xq.data());
    for (int q = 0; q < nq; ++q) {
      double uh = 0.0, gh[3] = {0, 0, 0};
      for (int i = 0; i < npe; ++i) {
        double ui = u[P->lids[c * npe + i]];
        uh += ui * P->phi[i * nq + q];
        for (int k = 0; k < d; ++k) gh[k] += ui * gphys[(i * nq + q) * d + k];
      }
      const double* x = &xq[q * d];
      double ue = sinprod(amp, freq, d, x);
      double diff = uh - ue;
      e2 += diff * diff * wdet[q];
      for (int k = 0; k < d; ++k) {
        double ge = amp * freq;
        for (int m = 0; m < d; ++m) ge *= (m == k) ? std::cos(freq * x[m]) : std::sin(freq * x[m]);
        double dg = gh[k] - ge;
        g2 += dg * dg * wdet[q];
      }
    }
  }
  if (l2) *l2 = std::sqrt(e2);
  if (h1) *h1 = std::sqrt(g2);
}

// Reference tables (for tests of the GPU library's basis/quadrature setup).
void orc_tables(const orc_problem* P, double* qw, double* phi, double* dphi) {
  if (qw) std::memcpy(qw, P->qw.data(), sizeof(double) * P->nq);
  if (phi) std::memcpy(phi, P->phi.data(), sizeof(double) * P->npe * P->nq);
  if (dphi) std::memcpy(dphi, P->dphi.data(), sizeof(double) * P->npe * P->nq * P->dim);
}

// Side points of one face (face order, see side_rule / face_cells): returns the count; fills xyz
// [count][3] (z = 0 in 2-D) when xyz is not null.  -1 for a bad face.
int64_t orc_side_points(const orc_problem* P, int face, double* xyz) {
  if (face < 0 || face >= 2 * P->dim) return -1;
  std::vector<double> xi, wr;
  side_rule(P, face, xi, wr);
  const std::vector<int64_t> cells = face_cells(P, face);
  const int npts = (int)wr.size(), d = P->dim;
  if (xyz) {
    std::vector<double> x((size_t)npts * d), phi((size_t)P->npe * npts), gp((size_t)P->npe * npts * d), w(npts),
        nrm((size_t)npts * d);
    for (size_t k = 0; k < cells.size(); ++k) {
      side_geometry(P, cells[k], face, xi, wr, x.data(), phi.data(), gp.data(), w.data(), nrm.data());
      for (int q = 0; q < npts; ++q)
        for (int m = 0; m < 3; ++m) xyz[((k * npts) + q) * 3 + m] = (m < d) ? x[q * d + m] : 0.0;
    }
  }
  return (int64_t)cells.size() * npts;
}

// Boundary condition of one face: kind 0 none, 1 Neumann, 2 weak Dirichlet; g has one value per side
// point (orc_side_points order), null means zero.  Returns 0, or -1 on bad input.
int orc_set_face_bc(orc_problem* P, int face, int kind, const double* g) {
  if (face < 0 || face >= 2 * P->dim || kind < 0 || kind > 2) return -1;
  const int64_t n = orc_side_points(P, face, nullptr);
  P->bc_kind[face] = kind;
  P->bc_g[face].assign(n, 0.0);
  if (g) for (int64_t i = 0; i < n; ++i) P->bc_g[face][i] = g[i];
  return 0;
}

int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"
