// Internal declarations shared by the translation units of libmrhyde_gb.so.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/mrhyde_gb300.h"

// ------------------------------------------------------------------------------------------------
// Error plumbing: every C entry point returns an mrg_status; the message is kept per host thread.
// ------------------------------------------------------------------------------------------------
void mrg_set_error(const std::string& msg);
int mrg_fail(int status, const std::string& msg);
int mrg_cuda_check(cudaError_t e, const char* what);

// Small pinned host slots (<= 256 bytes: device scalars read back by the host) from a process-wide pool.
// cudaMallocHost / cudaFreeHost per problem cost driver round trips and can synchronise the device,
// stalling every other stream in flight; the pool's chunks are pinned once and kept.
void* mrg_pinned_slot();
void mrg_pinned_release(void* p);

// Number of SMs of the current device, cached per device ordinal (any host thread).
int mrg_device_sms();

#define MRG_CUDA(call)                                          \
  do {                                                          \
    cudaError_t e__ = (call);                                   \
    if (e__ != cudaSuccess) return mrg_cuda_check(e__, #call);  \
  } while (0)

// ------------------------------------------------------------------------------------------------
// Structured grid description passed by value to kernels.
//
// Nodes of the (p*nx+1) x (p*ny+1) x (p*nz+1) grid are numbered ix + NX*(iy + NY*iz); cells
// cx + nx*(cy + ny*cz); local node (a,b,c) -> a + (p+1)*(b + (p+1)*c).  The CSR graph is the union
// of element couplings with sorted columns, so along every axis a row couples to a contiguous node
// range [lo, lo+cnt) and the row length is the product of the three per-axis counts.  Rows are
// ordered (iz, iy, ix), which gives
//     row_ptr(ix,iy,iz) = Pz[iz]*Ty*Tx + cz(iz)*(Py[iy]*Tx + cy(iy)*Px[ix])
// with P*[i] the per-axis prefix sums of the counts and T* their totals.
// ------------------------------------------------------------------------------------------------
struct Grid {
  int dim, p;
  int nc[3];       // cells per axis (nc[2] = 1 in 2-D)
  int nn[3];       // nodes per axis (nn[2] = 1 in 2-D)
  uint32_t faces;  // Dirichlet face mask
  int64_t T[3];    // per-axis totals of the coupling counts
  const int64_t* P[3];  // device per-axis prefix tables, length nn[k]+1
  // bounded device waits (mrg_set_wait_policy): limit in ns (0 = the kernel's default) and the testing
  // switch that withholds the first staged copy so that its wait runs out
  unsigned long long wait_ns;
  int withhold;
  int reserved;
};

// Coupled node range along one axis for node index i (host + device).
__host__ __device__ inline void axis_range(int i, int nnodes, int p, int& lo, int& cnt) {
  int ncell = (nnodes - 1) / p;
  int cf, cl;
  if (i % p == 0) { cf = i / p - 1; cl = i / p; } else { cf = cl = i / p; }
  if (cf < 0) cf = 0;
  if (cl > ncell - 1) cl = ncell - 1;
  lo = p * cf;
  cnt = p * (cl - cf) + p + 1;
}

// Number of cells adjacent to node i along one axis (1 or 2) and the first one.
__host__ __device__ inline void axis_cells(int i, int nnodes, int p, int& cf, int& ncells) {
  int ncell = (nnodes - 1) / p;
  int cl;
  if (i % p == 0) { cf = i / p - 1; cl = i / p; } else { cf = cl = i / p; }
  if (cf < 0) cf = 0;
  if (cl > ncell - 1) cl = ncell - 1;
  ncells = cl - cf + 1;
}

__host__ __device__ inline bool node_fixed(const Grid& g, int ix, int iy, int iz) {
  uint32_t f = g.faces;
  bool on = ((f & 1u) && ix == 0) || ((f & 2u) && ix == g.nn[0] - 1) || ((f & 4u) && iy == 0) ||
            ((f & 8u) && iy == g.nn[1] - 1);
  if (g.dim == 3) on = on || ((f & 16u) && iz == 0) || ((f & 32u) && iz == g.nn[2] - 1);
  return on;
}

// ------------------------------------------------------------------------------------------------
// Problem handle.
// ------------------------------------------------------------------------------------------------
struct SolverWork;  // mrg_solver.cu

struct mrg_problem {
  Grid g;
  int npe, nq, quad_order;
  int64_t ndof, ncell, nnz, nfixed;
  int path;
  int kind, source_kind;
  double source_amp, source_freq;
  double lo[3], hi[3], h[3];
  bool affine;                 // uniform box cells (no vertex_coords)
  // device data owned by the handle
  int64_t* d_prefix = nullptr;  // concatenated per-axis prefix tables
  double* d_kappa = nullptr;    // [ncell]
  float* d_kappa32 = nullptr;   // [ncell] FP32 copy for the mixed-precision Jacobian
  int32_t* d_fixed = nullptr;   // [nfixed] fixed DOFs, increasing
  double* d_fixed_vals = nullptr;
  double* d_vcoord = nullptr;   // [nvert*dim] (general geometry) or null
  double* d_srcB = nullptr;     // per-axis source tables (factored path, sinprod source)
  double* d_qtab = nullptr;     // reference tables for the per-cell path: w, phi, dphi (+ geometric psi, dpsi)
  double* d_khat = nullptr;     // stored-geometry path: [36][ncell] kappa-free symmetric cell stiffness
  float* d_khat32 = nullptr;    // [36][ncell] FP32 copy (mixed-precision Jacobian)
  double* d_bload = nullptr;    // [ndof] load vector b_i = sum over the node's cells of int f phi_i
  // host copies of small tables
  double Kp[8];                 // factored path: K(|dx|,|dy|,|dz|) of one cell, kappa = 1
  // cubic cells of the factored path: the axis classes are +0 and the other off-diagonal classes share
  // one coefficient -|K| (diagonal 4 |K|); d_kappa_s holds |K| kappa_c, formed per assembly
  int cubic = 0;
  double kscale = 0.0;
  double* d_kappa_s = nullptr;
  double cell_load;             // factored path: int_cell phi_l for one node (vol / 2^dim)
  std::vector<double> qtab_host;
  std::vector<double> gx1, gw1;  // 1-D Gauss rule of the problem
  void* q2 = nullptr;            // Q2 tensor-product data (mrg_assemble_q2.cu)
  void* bicg = nullptr;          // BiCGStab workspace (mrg_bicgstab.cu)
  void* bnd = nullptr;           // face boundary conditions (mrg_boundary.cu)
  void* gmg = nullptr;           // multigrid hierarchy and preconditioner choice (mrg_gmg.cu)
  cudaStream_t stream = nullptr;       // creation stream: the handle's memory is allocated/freed in its order
  cudaStream_t last_stream = nullptr;  // last stream work was enqueued on (drained before destroy)
  SolverWork* work = nullptr;
};

// Layout of d_qtab for the per-cell path: [nq] weights, [npe*nq] phi, [npe*nq*dim] dphi,
// [nvpe*nq] psi, [nvpe*nq*dim] dpsi.
struct QTab {
  const double* w;
  const double* phi;
  const double* dphi;
  const double* psi;
  const double* dpsi;
};

// Launchers (mrg_assemble_q1.cu)
int mrg_launch_factored(mrg_problem* p, const double* u, double* r, void* J, uint32_t flags, cudaStream_t s);
int mrg_launch_cell(mrg_problem* p, const double* u, double* r, void* J, uint32_t flags, cudaStream_t s);
int mrg_launch_constraints(mrg_problem* p, void* J, bool fp32, cudaStream_t s);
int mrg_launch_fix_zero_rows(mrg_problem* p, void* J, bool fp32, cudaStream_t s);
int mrg_launch_kappa32(mrg_problem* p, cudaStream_t s);
// Q2 hexahedra on identical affine cells (mrg_assemble_q2.cu)
int mrg_q2_setup(mrg_problem* p);
void mrg_q2_free(mrg_problem* p);
int mrg_launch_q2(mrg_problem* p, const double* u, double* r, void* J, uint32_t flags, cudaStream_t s);
// Q2 element matrices on tcgen05 tensor cores and their row gather (mrg_tc_q2.cu)
struct Q2Tc;
int mrg_q2tc_create(mrg_problem* p, const double* tab, const double s[3], Q2Tc** out, cudaStream_t st);
void mrg_q2tc_free(Q2Tc* T, cudaStream_t st);
float* mrg_q2tc_w_image(Q2Tc* T);  // [tile][hi, lo][K chunk 28][cell 128][4] TF32 operand image
int mrg_q2tc_launch(const mrg_problem* p, Q2Tc* T, float* J, bool ovw, int* err, cudaStream_t s);
// Thermal Q1 hexahedra on general geometry from per-cell data stored at setup (mrg_stored.cu)
bool mrg_stored_eligible(int dim, int order, int kind, int points_per_axis, bool affine);
int mrg_stored_setup(mrg_problem* p, cudaStream_t s);
int mrg_launch_stored(mrg_problem* p, const double* u, double* r, void* J, uint32_t flags, cudaStream_t s);
// Face boundary terms (mrg_boundary.cu)
void mrg_boundary_free(mrg_problem* p);
bool mrg_boundary_active(const mrg_problem* p);
int mrg_launch_boundary(mrg_problem* p, const double* u, double* r, void* J, bool fp32, cudaStream_t s);
// 1-D Lagrange basis of degree p on equispaced nodes of [-1,1]: values l[0..p], derivatives dl[0..p]
void mrg_lagrange_1d(int p, double xi, double* l, double* dl);
// Multigrid preconditioned CG (mrg_gmg.cu)
int mrg_gmg_kind(const mrg_problem* p);
void mrg_gmg_free(mrg_problem* p);
// setup: how the hierarchy follows J.  FULL rebuilds every level; REUSE keeps everything (J unchanged
// since the last setup); LEVEL0 refreshes level 0 (J itself, its diagonal and Chebyshev bound) and keeps
// the coarse Galerkin operators of the last full setup (a lagged preconditioner; the Krylov operator is
// always the current J).
enum { MRG_GMG_SETUP_FULL = 0, MRG_GMG_SETUP_REUSE = 1, MRG_GMG_SETUP_LEVEL0 = 2 };
int mrg_gmg_solve(mrg_problem* p, const void* J, bool fp32, const double* b, double* x, double rtol, int maxiter,
                  mrg_solve_stats* st, int setup, cudaStream_t s);
int mrg_gmg_bicgstab(mrg_problem* p, const void* J, bool fp32, const double* b, double* x, double rtol, int maxiter,
                     mrg_solve_stats* st, int setup, cudaStream_t s);
// Solver (mrg_solver.cu)
void mrg_solver_free(mrg_problem* p);
void mrg_solver_drop_graphs(mrg_problem* p);  // captured PCG chunks (recaptured on next use)
void mrg_bicg_drop_graphs(mrg_problem* p);    // captured BiCGStab chunks
void mrg_gmg_drop_hierarchy(mrg_problem* p);  // multigrid levels and graphs (rebuilt on next use)
int mrg_residual_from(mrg_problem* p, const double* b, double* res, cudaStream_t s);  // res = b - res
// BiCGStab (mrg_bicgstab.cu)
void mrg_bicg_free(mrg_problem* p);
int mrg_bicg_solve32(mrg_problem* p, const float* J32, const double* b, double rtol, int maxiter,
                     mrg_solve_stats* st, const float** d, cudaStream_t s);
int mrg_bicg_solve64(mrg_problem* p, const double* J, const double* b, double* x, double rtol, int maxiter,
                     mrg_solve_stats* st, cudaStream_t s);
