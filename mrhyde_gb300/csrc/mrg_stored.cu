// Thermal assembly on general (non-affine) Q1 hexahedra and quadrilaterals from per-cell geometry stored
// at setup.
//
// The reference keeps, for every cell, its physical basis values, gradients and quadrature weights
// computed once at setup: AssemblyManager::allocateGroupStorage -> Group::computeBasis for every group
// below the "storage proportion" (default 1.0, i.e. all cells;
// src/managers/assembly/assemblyManager_groups.hpp:20, :396-398, :476-513), which updateWorkset then
// binds instead of recomputing the geometry (src/managers/assembly/assemblyManager_workset.hpp:990-995).
// The thermal residual (src/physics/thermal.cpp:125-137) needs of the geometry only
//     Khat_c[i][j] = sum_q w_q |det J_q| grad phi_i(x_q) . grad phi_j(x_q)   (symmetric, kappa-free)
//     b_c[i]       = sum_q w_q |det J_q| f(x_q) phi_i(x_q)
// so those are what is stored here: Khat in FP64 and FP32 (36 values each: 432 bytes a cell) and the
// load summed per node, b_i = sum_c b_c[l_i] (8 bytes a node), computed once per problem by k_geo_hex
// and k_node_load.  Each assembly then needs no geometry at all:
//     J(i, col) = sum over the row's cells c that contain col, in a fixed order, of kappa_c Khat_c[l_i][l_col]
//     r_i       = b_i - sum_c kappa_c sum_j Khat_c[l_i][j] u_j   (= the reference's -sum_c res_c(l_i))
// k_stored_hex writes one CSR row per thread (no atomics, no zero-fill pass, deterministic), with the row
// held in registers at compile-time positions.  FP64 is the bound (1/64 of the FP32 rate on this GPU),
// so each pass takes the cheaper of two exact-arithmetic-equal residual forms: with the FP64 Jacobian
// row in registers, r_i = b_i - sum_col J(i, col) u_col (27 FMAs after the row's 64); without it (the
// residual-only pass, which the mixed pass also runs for its residual) the per-cell form above (72
// FMAs).  The two agree to rounding; each pass is deterministic.
//
// Quadrilaterals store 10 values a cell, FP64 only (80 bytes a cell; k_geo_quad, k_node_load_quad), and
// take one thread per 9-entry row (k_stored_quad), whose Jacobian passes, the mixed one included, form
// the row in FP64 and take the residual from it.
//
// Geometry in k_geo_hex: with C the cofactor matrix of the geometric Jacobian J_q (J[k][m] = dx_k/dxi_m),
// J^{-T} = C / det, so grad phi_i . grad phi_j w |det| = ghat_i^T (C^T C) ghat_j * w / |det| for the
// reference gradients ghat: one symmetric 3 x 3 metric per quadrature point instead of eight physical
// gradients.
#include <type_traits>

#include "mrg_device.cuh"
#include "mrg_fixmul.cuh"
#include "mrg_internal.h"

namespace {

using namespace mrgdev;

constexpr int GEO_CPB = 16;   // cells per CTA of the setup kernel (8 threads each)
constexpr int ST_T = 256;     // rows per CTA of the assembly kernel

// Rows staged in shared memory (see k_stored_hex) in every Jacobian pass except the FP64 Jacobian +
// residual, which is bound by the FP64 pipe and measured faster with direct row stores
template <typename JT, bool DOJ, bool DOR>
constexpr bool stored_stage() {
  return DOJ && !(sizeof(JT) == 8 && DOR);
}
// CTAs per SM each instance of the assembly kernel is compiled for (by measurement on 128^3): the FP64
// Jacobian row keeps its registers (2), the single-product passes run at 3
template <typename JT, bool DOJ, bool DOR>
constexpr int stored_minb() {
  return (DOJ && (sizeof(JT) == 8 || DOR)) ? 2 : 3;
}

// index of (i, j), i <= j, in the row-major upper triangle of an 8 x 8 symmetric matrix
__host__ __device__ constexpr int sym8(int i, int j) {
  return i <= j ? i * 8 - (i * (i - 1)) / 2 + (j - i) : j * 8 - (j * (j - 1)) / 2 + (i - j);
}
static_assert(sym8(7, 7) == 35 && sym8(0, 7) == 7 && sym8(1, 1) == 8, "triangle layout");

struct GeoArgs {
  Grid g;
  QTab tab;
  const double* vcoord;  // [nvert][dim], x fastest
  int src_sin;
  double amp, freq;
  int64_t ncell;
  double* khat;          // [36][ncell] (hexahedra) or [10][ncell] (quadrilaterals)
  float* khat32;         // [36][ncell], hexahedra only
  double* bload;         // [8 or 4][ncell] cell loads (summed per node by k_node_load / k_node_load_quad)
};

// 8 threads per cell: thread t first evaluates the geometry at quadrature point t, then row t of Khat.
__global__ void __launch_bounds__(GEO_CPB * 8) k_geo_hex(const GeoArgs A) {
  __shared__ double s_x[GEO_CPB][8][3];
  __shared__ double s_m[GEO_CPB][8][6];  // w / |det| * C^T C at each point: xx, yy, zz, xy, xz, yz
  __shared__ double s_fw[GEO_CPB][8];    // f(x_q) w_q |det J_q|
  const int slot = threadIdx.x >> 3, t = threadIdx.x & 7;
  const int64_t c = (int64_t)blockIdx.x * GEO_CPB + slot;
  const bool active = c < A.ncell;
  const Grid& g = A.g;
  if (active) {
    const int cx = (int)(c % g.nc[0]);
    const int64_t rest = c / g.nc[0];
    const int cy = (int)(rest % g.nc[1]), cz = (int)(rest / g.nc[1]);
    const int64_t vid = (cx + (t & 1)) + (int64_t)(g.nc[0] + 1) * ((cy + ((t >> 1) & 1)) + (int64_t)(g.nc[1] + 1) * (cz + (t >> 2)));
#pragma unroll
    for (int k = 0; k < 3; ++k) s_x[slot][t][k] = __ldg(A.vcoord + vid * 3 + k);
  }
  __syncthreads();
  if (active) {
    const int q = t;
    double Jm[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, xq[3] = {0, 0, 0};
#pragma unroll
    for (int v = 0; v < 8; ++v) {
      const double ps = A.tab.psi[v * 8 + q];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const double xv = s_x[slot][v][k];
        xq[k] = fma(xv, ps, xq[k]);
#pragma unroll
        for (int m = 0; m < 3; ++m) Jm[k][m] = fma(xv, A.tab.dpsi[(v * 8 + q) * 3 + m], Jm[k][m]);
      }
    }
    double C[3][3];  // cofactors: C[k][m] = (-1)^(k+m) minor(k, m)
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
      for (int m = 0; m < 3; ++m) {
        const int k1 = (k + 1) % 3, k2 = (k + 2) % 3, m1 = (m + 1) % 3, m2 = (m + 2) % 3;
        C[k][m] = Jm[k1][m1] * Jm[k2][m2] - Jm[k1][m2] * Jm[k2][m1];
      }
    const double det = Jm[0][0] * C[0][0] + Jm[0][1] * C[0][1] + Jm[0][2] * C[0][2];
    const double ad = fabs(det), w = A.tab.w[q];
    const double sc = w / ad;
#pragma unroll
    for (int e = 0; e < 6; ++e) {
      const int mi = e < 3 ? e : (e == 5 ? 1 : 0), ni = e < 3 ? e : (e == 3 ? 1 : 2);
      double s = 0.0;
#pragma unroll
      for (int k = 0; k < 3; ++k) s = fma(C[k][mi], C[k][ni], s);
      s_m[slot][q][e] = s * sc;
    }
    double f = A.amp;
    if (A.src_sin) {
#pragma unroll
      for (int k = 0; k < 3; ++k) f *= sin(A.freq * xq[k]);
    }
    s_fw[slot][q] = f * w * ad;
  }
  __syncthreads();
  if (!active) return;
  const int i = t;
  double kr[8] = {0, 0, 0, 0, 0, 0, 0, 0}, bl = 0.0;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const double* M = s_m[slot][q];
    const double g0 = A.tab.dphi[(i * 8 + q) * 3 + 0], g1 = A.tab.dphi[(i * 8 + q) * 3 + 1],
                 g2 = A.tab.dphi[(i * 8 + q) * 3 + 2];
    const double v0 = M[0] * g0 + M[3] * g1 + M[4] * g2;
    const double v1 = M[3] * g0 + M[1] * g1 + M[5] * g2;
    const double v2 = M[4] * g0 + M[5] * g1 + M[2] * g2;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const double* gj = A.tab.dphi + (j * 8 + q) * 3;
      kr[j] = fma(v0, gj[0], fma(v1, gj[1], fma(v2, gj[2], kr[j])));
    }
    bl = fma(A.tab.phi[i * 8 + q], s_fw[slot][q], bl);
  }
#pragma unroll
  for (int j = 0; j < 8; ++j)
    if (j >= i) {
      const int e = sym8(i, j);
      A.khat[(int64_t)e * A.ncell + c] = kr[j];
      A.khat32[(int64_t)e * A.ncell + c] = (float)kr[j];
    }
  A.bload[(int64_t)i * A.ncell + c] = bl;
}

// b_i = sum over the node's cells (fixed order: cz, cy, cx) of the cell loads b_c[l_i]
__global__ void k_node_load(Grid g, int64_t nrows, int64_t ncell, const double* __restrict__ bload,
                            double* __restrict__ b) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nrows) return;
  int ix, iy, iz;
  decompose(g, n, ix, iy, iz);
  double s = 0.0;
  for (int bz = 0; bz < 2; ++bz)
    for (int by = 0; by < 2; ++by)
      for (int bx = 0; bx < 2; ++bx) {
        const int cx = ix - 1 + bx, cy = iy - 1 + by, cz = iz - 1 + bz;
        if (cx < 0 || cy < 0 || cz < 0 || cx >= g.nc[0] || cy >= g.nc[1] || cz >= g.nc[2]) continue;
        const int l = (1 - bx) | ((1 - by) << 1) | ((1 - bz) << 2);
        s += bload[l * ncell + cx + (int64_t)g.nc[0] * (cy + (int64_t)g.nc[1] * cz)];
      }
  b[n] = s;
}

struct StoredArgs {
  Grid g;
  const double* khat;
  const float* khat32;
  const double* bnode;
  const double* kap;
  const float* kap32;
  int64_t nrows, ncell;
};

// The row of node n, written into the CTA's staged segment sv (CSR offset seg0) or straight into J, and
// into r.  Dirichlet rows are never scattered: zeros (J(d,d) = 1 in overwrite mode).  Row slots are the
// 3 x 3 x 3 node neighbourhood (dz, dy, dx) at compile-time positions; the row's cells (offsets
// (ox, oy, oz) in {-1, 0}^3) are visited in a fixed order.  The cells below the node (oz = -1) contribute
// to the dz = -1 and dz = 0 planes of the row, the cells above (oz = 0) to dz = 0 and dz = +1, so after
// the lower four cells the dz = -1 plane is final: it is stored then, and at most 18 of the 27 slots are
// live at a time.  Cells outside the mesh (boundary rows) are read at a clamped index with their
// coefficient selected to 0, which adds exact zeros: the loads carry no branches.
template <typename JT, bool DOJ, bool DOR, bool OVW, bool STAGE>
__device__ __forceinline__ void row_body(const StoredArgs& A, const Grid& g, int64_t n, const double* __restrict__ u,
                                         double* __restrict__ r, JT* sv, int64_t seg0, JT* __restrict__ J,
                                         bool& fixed, int64_t& dglob) {
  constexpr bool F32 = sizeof(JT) == 4;
  constexpr bool ROW64 = DOJ && !F32;      // FP64 Jacobian row (its residual: b - J u)
  constexpr bool ROW32 = DOJ && F32;       // FP32 Jacobian row from FP32 products
  constexpr bool CELLRES = DOR && !ROW64;  // residual in the per-cell form
  int ix, iy, iz;
  decompose(g, n, ix, iy, iz);
  const RowInfo R = row_info<1>(g, ix, iy, iz);
  const int64_t loc = R.rp - seg0;
  if (node_fixed(g, ix, iy, iz)) {
    fixed = true;
    if (DOJ) {
      const int len = R.cx * R.cy * R.cz;
      const int dp = (int)(diag_pos(R, ix, iy, iz) - R.rp);
      dglob = R.rp + dp;
      if (STAGE) {
        for (int k = 0; k < len; ++k) sv[loc + k] = (OVW && k == dp) ? JT(1) : JT(0);
      } else if (OVW) {
        for (int k = 0; k < len; ++k) J[R.rp + k] = (k == dp) ? JT(1) : JT(0);
      } else {
        J[dglob] = JT(1);
      }
    }
    if (DOR && OVW) r[n] = 0.0;
    return;
  }
  const int64_t nc = A.ncell;
  const int64_t NX = g.nn[0], PL = (int64_t)g.nn[0] * g.nn[1];
  // the row's slots: dx in [xlo, xlo + R.cx) etc. (xlo = -1, or 0 on the first node of an axis)
  const int xlo = R.lx - ix, ylo = R.ly - iy, zlo = R.lz - iz;
  // the node's cells per axis: index 0 = below the node, 1 = above; outside the mesh, a clamped index
  // whose coefficient is selected to 0 (its products add exact zeros, and only to slots outside the row)
  int cc[3][2];
  bool ok[3][2];
  {
    const int iv[3] = {ix, iy, iz};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      ok[k][0] = iv[k] >= 1;
      ok[k][1] = iv[k] < g.nc[k];
      cc[k][0] = ok[k][0] ? iv[k] - 1 : 0;
      cc[k][1] = ok[k][1] ? iv[k] : g.nc[k] - 1;
    }
  }
  double res = CELLRES ? __ldg(A.bnode + n) : 0.0, ju = 0.0;
  // per-cell residual: u of the row's node neighbourhood, one plane (dz) of 9 slots at a time, read at
  // indices clamped into the mesh (a clamped slot only meets cells whose coefficient is 0)
  auto load_u = [&](int dz, double* up) {
    const int z = min(max(iz + dz, 0), g.nn[2] - 1);
#pragma unroll
    for (int s = 0; s < 9; ++s) {
      const int x = min(max(ix + s % 3 - 1, 0), g.nn[0] - 1), y = min(max(iy + s / 3 - 1, 0), g.nn[1] - 1);
      up[s] = __ldg(u + x + NX * y + PL * z);
    }
  };
  double uA[9], uB[9];
  if (CELLRES) {
    load_u(-1, uA);
    load_u(0, uB);
  }
  double lo64[9], mid64[9], hi64[9];
  float lo32[9], mid32[9], hi32[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    lo64[k] = mid64[k] = hi64[k] = 0.0;
    lo32[k] = mid32[k] = hi32[k] = 0.0f;
  }
  // the cell at offset (bx - 1, by - 1, bz - 1): its products on the two row planes it touches
  auto cell = [&](auto BX, auto BY, auto BZ, double* p0, double* p1, float* q0, float* q1, const double* u0,
                  const double* u1) {
    constexpr int bx = decltype(BX)::value, by = decltype(BY)::value, bz = decltype(BZ)::value;
    const bool valid = ok[0][bx] && ok[1][by] && ok[2][bz];
    const int64_t c = cc[0][bx] + (int64_t)g.nc[0] * (cc[1][by] + (int64_t)g.nc[1] * cc[2][bz]);
    constexpr int l = (1 - bx) | ((1 - by) << 1) | ((1 - bz) << 2);  // this node's local index in the cell
    const double k64 = (ROW64 || CELLRES) ? (valid ? __ldg(A.kap + c) : 0.0) : 0.0;
    const float k32 = ROW32 ? (valid ? __ldg(A.kap32 + c) : 0.0f) : 0.0f;
    double dot = 0.0;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int jx = j & 1, jy = (j >> 1) & 1, jz = j >> 2;
      const int s = (by + jy) * 3 + (bx + jx);  // slot within the plane: (dy + 1) * 3 + (dx + 1), dx = bx - 1 + jx
      const int e = sym8(l, j);
      if (ROW64 || CELLRES) {
        const double kh = __ldg(A.khat + e * nc + c);
        if (ROW64) {
          double* pl = jz ? p1 : p0;
          pl[s] = fma(k64, kh, pl[s]);
        }
        if (CELLRES) dot = fma(kh, (jz ? u1 : u0)[s], dot);
      }
      if (ROW32) {
        float* ql = jz ? q1 : q0;
        ql[s] = fmaf(k32, __ldg(A.khat32 + e * nc + c), ql[s]);
      }
    }
    if (CELLRES) res = fma(-k64, dot, res);
  };
  // stores one final plane (dz) of the row; with the FP64 row, adds its part of sum_col J u
  auto finish = [&](int dz, const double* p64, const float* p32) {
    if (dz < zlo || dz >= zlo + R.cz) return;
#pragma unroll
    for (int s = 0; s < 9; ++s) {
      const int dx = s % 3 - 1, dy = s / 3 - 1;
      if (dx >= xlo && dx < xlo + R.cx && dy >= ylo && dy < ylo + R.cy) {
        if (ROW64 && DOR) ju = fma(p64[s], __ldg(u + n + dx + NX * dy + PL * dz), ju);
        if (DOJ) {
          const int k = ((dz - zlo) * R.cy + (dy - ylo)) * R.cx + (dx - xlo);
          const JT v = F32 ? (JT)p32[s] : (JT)p64[s];
          if (STAGE) sv[loc + k] = v;
          else if (OVW) J[R.rp + k] = v;
          else J[R.rp + k] += v;
        }
      }
    }
  };
  using I0 = std::integral_constant<int, 0>;
  using I1 = std::integral_constant<int, 1>;
  // cells below the node (bz = 0): planes dz = -1 (jz = 0) and dz = 0 (jz = 1)
  cell(I0{}, I0{}, I0{}, lo64, mid64, lo32, mid32, uA, uB);
  cell(I1{}, I0{}, I0{}, lo64, mid64, lo32, mid32, uA, uB);
  cell(I0{}, I1{}, I0{}, lo64, mid64, lo32, mid32, uA, uB);
  cell(I1{}, I1{}, I0{}, lo64, mid64, lo32, mid32, uA, uB);
  finish(-1, lo64, lo32);
  if (CELLRES) load_u(1, uA);  // planes dz = 0 (uB) and dz = +1 (uA) for the cells above
  // cells above (bz = 1): planes dz = 0 (jz = 0) and dz = +1 (jz = 1)
  cell(I0{}, I0{}, I1{}, mid64, hi64, mid32, hi32, uB, uA);
  cell(I1{}, I0{}, I1{}, mid64, hi64, mid32, hi32, uB, uA);
  cell(I0{}, I1{}, I1{}, mid64, hi64, mid32, hi32, uB, uA);
  cell(I1{}, I1{}, I1{}, mid64, hi64, mid32, hi32, uB, uA);
  finish(0, mid64, mid32);
  finish(1, hi64, hi32);
  if (DOR) {
    const double rv = CELLRES ? res : __ldg(A.bnode + n) - ju;
    if (OVW) r[n] = rv; else r[n] += rv;
  }
}

// One CSR row per thread.  The CTA's rows are contiguous in CSR: where stores bind (see stored_stage)
// they are staged in shared memory (same 16-byte phase as global) and written once with 16-byte stores
// (one row per thread touches ~27 lines per store instruction).
template <typename JT, bool DOJ, bool DOR, bool OVW>
__global__ void __launch_bounds__(ST_T, stored_minb<JT, DOJ, DOR>())
    k_stored_hex(const StoredArgs A, const double* __restrict__ u, double* __restrict__ r, JT* __restrict__ J) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr bool STAGE = stored_stage<JT, DOJ, DOR>();
  const Grid& g = A.g;
  const int64_t n0 = (int64_t)blockIdx.x * ST_T, n = n0 + threadIdx.x;
  const int64_t nend = (n0 + ST_T < A.nrows) ? n0 + ST_T : A.nrows;
  int64_t seg0 = 0, seg1 = 0;
  JT* sv = nullptr;
  if (STAGE) {
    seg0 = row_ptr_of(g, n0, A.nrows);
    seg1 = row_ptr_of(g, nend, A.nrows);
    sv = reinterpret_cast<JT*>(smem_raw) + (int)(((uintptr_t)(J + seg0) & 15) / sizeof(JT));
  }
  const bool active = n < A.nrows;
  bool fixed = false;
  int64_t dglob = 0;
  if (active) row_body<JT, DOJ, DOR, OVW, STAGE>(A, g, n, u, r, sv, seg0, J, fixed, dglob);
  if (STAGE) {
    if (OVW) {  // the staged segment leaves through the copy engine
      fence_to_bulk();
      __syncthreads();
      seg_store_bulk<JT>(J + seg0, sv, seg1 - seg0);
    } else {
      __syncthreads();
      seg_store<JT, true>(J + seg0, sv, seg1 - seg0);
      __syncthreads();  // a Dirichlet row's diagonal is replaced, not added to (setJacobianConstraints)
      if (active && fixed) J[dglob] = JT(1);
    }
  }
}

// ---- quadrilaterals (2-D): 4 nodes and 4 Gauss points a cell, 10 symmetric stiffness values, 9-entry rows

// index of (i, j), i <= j, in the row-major upper triangle of a 4 x 4 symmetric matrix
__host__ __device__ constexpr int sym4(int i, int j) {
  return i <= j ? i * 4 - (i * (i - 1)) / 2 + (j - i) : j * 4 - (j * (j - 1)) / 2 + (i - j);
}
static_assert(sym4(3, 3) == 9 && sym4(0, 3) == 3 && sym4(1, 1) == 4, "triangle layout");

constexpr int GEO2_CPB = 32;  // cells per CTA of the 2-D setup kernel (4 threads each)

// 4 threads per cell: thread t evaluates the geometry at Gauss point t, then row t of Khat.  With C the
// cofactor matrix of the 2 x 2 geometric Jacobian, grad phi_i . grad phi_j w |det| = ghat_i^T C^T C ghat_j
// w / |det|.
__global__ void __launch_bounds__(GEO2_CPB * 4) k_geo_quad(const GeoArgs A) {
  __shared__ double s_x[GEO2_CPB][4][2];
  __shared__ double s_m[GEO2_CPB][4][3];  // w / |det| * C^T C: xx, yy, xy
  __shared__ double s_fw[GEO2_CPB][4];
  const int slot = threadIdx.x >> 2, t = threadIdx.x & 3;
  const int64_t c = (int64_t)blockIdx.x * GEO2_CPB + slot;
  const bool active = c < A.ncell;
  const Grid& g = A.g;
  if (active) {
    const int cx = (int)(c % g.nc[0]), cy = (int)(c / g.nc[0]);
    const int64_t vid = (cx + (t & 1)) + (int64_t)(g.nc[0] + 1) * (cy + (t >> 1));
    s_x[slot][t][0] = __ldg(A.vcoord + vid * 2);
    s_x[slot][t][1] = __ldg(A.vcoord + vid * 2 + 1);
  }
  __syncthreads();
  if (active) {
    const int q = t;
    double Jm[2][2] = {{0, 0}, {0, 0}}, xq[2] = {0, 0};
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const double ps = A.tab.psi[v * 4 + q];
#pragma unroll
      for (int k = 0; k < 2; ++k) {
        const double xv = s_x[slot][v][k];
        xq[k] = fma(xv, ps, xq[k]);
#pragma unroll
        for (int m = 0; m < 2; ++m) Jm[k][m] = fma(xv, A.tab.dpsi[(v * 4 + q) * 2 + m], Jm[k][m]);
      }
    }
    // cofactors C[k][m] = (-1)^(k+m) minor(k, m)
    const double C00 = Jm[1][1], C01 = -Jm[1][0], C10 = -Jm[0][1], C11 = Jm[0][0];
    const double det = Jm[0][0] * Jm[1][1] - Jm[0][1] * Jm[1][0];
    const double ad = fabs(det), w = A.tab.w[q];
    const double sc = w / ad;
    s_m[slot][q][0] = (C00 * C00 + C10 * C10) * sc;
    s_m[slot][q][1] = (C01 * C01 + C11 * C11) * sc;
    s_m[slot][q][2] = (C00 * C01 + C10 * C11) * sc;
    double f = A.amp;
    if (A.src_sin) f *= sin(A.freq * xq[0]) * sin(A.freq * xq[1]);
    s_fw[slot][q] = f * w * ad;
  }
  __syncthreads();
  if (!active) return;
  const int i = t;
  double kr[4] = {0, 0, 0, 0}, bl = 0.0;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const double* M = s_m[slot][q];
    const double g0 = A.tab.dphi[(i * 4 + q) * 2], g1 = A.tab.dphi[(i * 4 + q) * 2 + 1];
    const double v0 = M[0] * g0 + M[2] * g1, v1 = M[2] * g0 + M[1] * g1;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const double* gj = A.tab.dphi + (j * 4 + q) * 2;
      kr[j] = fma(v0, gj[0], fma(v1, gj[1], kr[j]));
    }
    bl = fma(A.tab.phi[i * 4 + q], s_fw[slot][q], bl);
  }
#pragma unroll
  for (int j = 0; j < 4; ++j)
    if (j >= i) A.khat[(int64_t)sym4(i, j) * A.ncell + c] = kr[j];
  A.bload[(int64_t)i * A.ncell + c] = bl;
}

__global__ void k_node_load_quad(Grid g, int64_t nrows, int64_t ncell, const double* __restrict__ bload,
                                 double* __restrict__ b) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nrows) return;
  const int ix = (int)(n % g.nn[0]), iy = (int)(n / g.nn[0]);
  double s = 0.0;
  for (int by = 0; by < 2; ++by)
    for (int bx = 0; bx < 2; ++bx) {
      const int cx = ix - 1 + bx, cy = iy - 1 + by;
      if (cx < 0 || cy < 0 || cx >= g.nc[0] || cy >= g.nc[1]) continue;
      s += bload[((1 - bx) | ((1 - by) << 1)) * ncell + cx + (int64_t)g.nc[0] * cy];
    }
  b[n] = s;
}

// One CSR row (at most 9 entries) per thread.  The row is formed in FP64 for both Jacobian types and
// rounded once when stored (an FP32 row would carry its rounding relative to the row's terms, which cancel
// across the two cells sharing an edge of a distorted mesh), so every Jacobian pass, the mixed one
// included, takes its residual from the FP64 row, r = b - J u (16 + 9 FMAs a row), and the residual-only
// pass the per-cell form (20 FMAs).  Both are bound by FP64 issue.
template <typename JT, bool DOJ, bool DOR, bool OVW>
__global__ void __launch_bounds__(ST_T) k_stored_quad(const StoredArgs A, const double* __restrict__ u,
                                                      double* __restrict__ r, JT* __restrict__ J) {
  constexpr bool ROW64 = DOJ, CELLRES = DOR && !DOJ;
  const int64_t n = (int64_t)blockIdx.x * ST_T + threadIdx.x;
  if (n >= A.nrows) return;
  const Grid& g = A.g;
  const int NX = g.nn[0];
  const int ix = (int)(n % NX), iy = (int)(n / NX);
  const RowInfo R = row_info<1>(g, ix, iy, 0);
  if (node_fixed(g, ix, iy, 0)) {
    if (DOJ) {
      const int len = R.cx * R.cy;
      const int dp = (iy - R.ly) * R.cx + (ix - R.lx);
      if (OVW) for (int k = 0; k < len; ++k) J[R.rp + k] = (k == dp) ? JT(1) : JT(0);
      else J[R.rp + dp] = JT(1);
    }
    if (DOR && OVW) r[n] = 0.0;
    return;
  }
  const int64_t nc = A.ncell;
  const int xlo = R.lx - ix, ylo = R.ly - iy;
  double a64[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) a64[k] = 0.0;
  double res = CELLRES ? __ldg(A.bnode + n) : 0.0;
#pragma unroll
  for (int co = 0; co < 4; ++co) {
    const int bx = co & 1, by = co >> 1;
    const int cx = ix - 1 + bx, cy = iy - 1 + by;
    const bool valid = cx >= 0 && cy >= 0 && cx < g.nc[0] && cy < g.nc[1];
    const int64_t c = (valid ? cx : 0) + (int64_t)g.nc[0] * (valid ? cy : 0);
    const int l = (1 - bx) | ((1 - by) << 1);
    const double k64 = valid ? __ldg(A.kap + c) : 0.0;
    double dot = 0.0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int jx = j & 1, jy = j >> 1;
      const int s = (by + jy) * 3 + (bx + jx);  // (dy + 1) * 3 + (dx + 1)
      const double kh = __ldg(A.khat + sym4(l, j) * nc + c);
      if (ROW64) a64[s] = fma(k64, kh, a64[s]);
      if (CELLRES && valid) dot = fma(kh, __ldg(u + (cx + jx) + (int64_t)NX * (cy + jy)), dot);
    }
    if (CELLRES) res = fma(-k64, dot, res);
  }
  double ju = 0.0;
#pragma unroll
  for (int s = 0; s < 9; ++s) {
    const int dx = s % 3 - 1, dy = s / 3 - 1;
    if (dx >= xlo && dx < xlo + R.cx && dy >= ylo && dy < ylo + R.cy) {
      if (ROW64 && DOR) ju = fma(a64[s], __ldg(u + n + dx + (int64_t)NX * dy), ju);
      if (DOJ) {
        const int64_t pos = R.rp + (dy - ylo) * R.cx + (dx - xlo);
        // FP32: rounded on the integer pipes (the conversion instruction issues at the FP64 rate)
        const JT v = sizeof(JT) == 4 ? (JT)mrgfix::f64_to_f32_rn(a64[s]) : (JT)a64[s];
        if (OVW) J[pos] = v; else J[pos] += v;
      }
    }
  }
  if (DOR) {
    const double rv = CELLRES ? res : __ldg(A.bnode + n) - ju;
    if (OVW) r[n] = rv; else r[n] += rv;
  }
}

inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

template <typename JT, bool DOJ, bool DOR, bool OVW>
cudaError_t launch_stored_quad(const mrg_problem* p, const StoredArgs& A, const double* u, double* r, JT* J,
                               cudaStream_t s) {
  k_stored_quad<JT, DOJ, DOR, OVW><<<nblk(p->ndof, ST_T), ST_T, 0, s>>>(A, u, r, J);
  return cudaGetLastError();
}

template <typename JT, bool DOJ, bool DOR, bool OVW>
cudaError_t launch_stored(const mrg_problem* p, const StoredArgs& A, const double* u, double* r, JT* J,
                          cudaStream_t s) {
  const int smem = stored_stage<JT, DOJ, DOR>() ? (ST_T * 27 + 16 / (int)sizeof(JT)) * (int)sizeof(JT) : 0;
  auto kern = k_stored_hex<JT, DOJ, DOR, OVW>;
  if (smem > 48 * 1024) {
    const cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
  }
  kern<<<nblk(p->ndof, ST_T), ST_T, smem, s>>>(A, u, r, J);
  return cudaGetLastError();
}

}  // namespace

bool mrg_stored_eligible(int dim, int order, int kind, int points_per_axis, bool affine) {
  return !affine && (dim == 2 || dim == 3) && order == 1 && kind == MRG_THERMAL && points_per_axis == 2;
}

int mrg_stored_setup(mrg_problem* p, cudaStream_t s) {
  const int64_t nc = p->ncell;
  const int d = p->g.dim, npe = p->npe, nq = p->nq, nsym = npe * (npe + 1) / 2;  // 36 (hexahedra) or 10
  double* cell_load = nullptr;
  MRG_CUDA(cudaMallocAsync(&p->d_khat, (size_t)nsym * nc * sizeof(double), s));
  if (d == 3) MRG_CUDA(cudaMallocAsync(&p->d_khat32, (size_t)nsym * nc * sizeof(float), s));  // 2-D: FP64 only
  MRG_CUDA(cudaMallocAsync(&p->d_bload, (size_t)p->ndof * sizeof(double), s));
  MRG_CUDA(cudaMallocAsync(&cell_load, (size_t)npe * nc * sizeof(double), s));
  GeoArgs A;
  A.g = p->g;
  A.tab.w = p->d_qtab;
  A.tab.phi = A.tab.w + nq;
  A.tab.dphi = A.tab.phi + npe * nq;
  A.tab.psi = A.tab.dphi + npe * nq * d;
  A.tab.dpsi = A.tab.psi + npe * nq;
  A.vcoord = p->d_vcoord;
  A.src_sin = (p->source_kind == MRG_SRC_SINPROD);
  A.amp = p->source_amp;
  A.freq = p->source_freq;
  A.ncell = nc;
  A.khat = p->d_khat;
  A.khat32 = p->d_khat32;
  A.bload = cell_load;
  if (d == 3) k_geo_hex<<<nblk(nc, GEO_CPB), GEO_CPB * 8, 0, s>>>(A);
  else k_geo_quad<<<nblk(nc, GEO2_CPB), GEO2_CPB * 4, 0, s>>>(A);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) {
    if (d == 3) k_node_load<<<nblk(p->ndof, 256), 256, 0, s>>>(p->g, p->ndof, nc, cell_load, p->d_bload);
    else k_node_load_quad<<<nblk(p->ndof, 256), 256, 0, s>>>(p->g, p->ndof, nc, cell_load, p->d_bload);
    e = cudaGetLastError();
  }
  cudaFreeAsync(cell_load, s);
  if (e != cudaSuccess) return mrg_cuda_check(e, "stored-geometry setup launch");
  return MRG_OK;
}

int mrg_launch_stored(mrg_problem* p, const double* u, double* r, void* J, uint32_t flags, cudaStream_t s) {
  StoredArgs A;
  A.g = p->g;
  A.khat = p->d_khat;
  A.khat32 = p->d_khat32;
  A.bnode = p->d_bload;
  A.kap = p->d_kappa;
  A.kap32 = p->d_kappa32;
  A.nrows = p->ndof;
  A.ncell = p->ncell;
  const bool doJ = (flags & MRG_ASM_JAC) && J, doR = (flags & MRG_ASM_RES) && r, ovw = flags & MRG_ASM_OVERWRITE;
  cudaError_t e = cudaSuccess;
  if (p->g.dim == 2) {
    // quadrilaterals: one launch per pass (k_stored_quad)
    if (doJ && (flags & MRG_ASM_J_FP32)) {
      float* J32 = (float*)J;
      e = doR ? (ovw ? launch_stored_quad<float, true, true, true>(p, A, u, r, J32, s)
                     : launch_stored_quad<float, true, true, false>(p, A, u, r, J32, s))
              : (ovw ? launch_stored_quad<float, true, false, true>(p, A, u, nullptr, J32, s)
                     : launch_stored_quad<float, true, false, false>(p, A, u, nullptr, J32, s));
    } else if (doJ) {
      double* J64 = (double*)J;
      e = doR ? (ovw ? launch_stored_quad<double, true, true, true>(p, A, u, r, J64, s)
                     : launch_stored_quad<double, true, true, false>(p, A, u, r, J64, s))
              : (ovw ? launch_stored_quad<double, true, false, true>(p, A, u, nullptr, J64, s)
                     : launch_stored_quad<double, true, false, false>(p, A, u, nullptr, J64, s));
    } else if (doR) {
      e = ovw ? launch_stored_quad<double, false, true, true>(p, A, u, r, nullptr, s)
              : launch_stored_quad<double, false, true, false>(p, A, u, r, nullptr, s);
    }
    if (e != cudaSuccess) return mrg_cuda_check(e, "stored-geometry assembly launch");
    return MRG_OK;
  }
  if (doJ && (flags & MRG_ASM_J_FP32)) {
    // mixed: the FP32 Jacobian pass, then (below) the FP64 residual pass: one fused launch holds both rows
    // and both copies of the stored stiffness and measured slower than the two
    e = ovw ? launch_stored<float, true, false, true>(p, A, u, nullptr, (float*)J, s)
            : launch_stored<float, true, false, false>(p, A, u, nullptr, (float*)J, s);
  } else if (doJ) {
    if (doR)
      e = ovw ? launch_stored<double, true, true, true>(p, A, u, r, (double*)J, s)
              : launch_stored<double, true, true, false>(p, A, u, r, (double*)J, s);
    else
      e = ovw ? launch_stored<double, true, false, true>(p, A, u, nullptr, (double*)J, s)
              : launch_stored<double, true, false, false>(p, A, u, nullptr, (double*)J, s);
    if (e != cudaSuccess) return mrg_cuda_check(e, "stored-geometry assembly launch");
    return MRG_OK;
  }
  if (e == cudaSuccess && doR)
    e = ovw ? launch_stored<double, false, true, true>(p, A, u, r, nullptr, s)
            : launch_stored<double, false, true, false>(p, A, u, r, nullptr, s);
  if (e != cudaSuccess) return mrg_cuda_check(e, "stored-geometry assembly launch");
  return MRG_OK;
}
