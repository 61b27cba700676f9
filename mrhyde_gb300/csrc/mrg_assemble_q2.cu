// Tensor-product (sum-factorised) assembly on identical affine hexahedra, Q1 and Q2, any of the two
// physics forms.  Used for Q2 (configuration C3: -div((1+u^2) grad u) = f, 27 nodes and 3x3x3 Gauss
// points per cell) and for nonlinear Q1 (the nonlinear requests of the serving loop), where the
// coefficient varies inside the cell so the kappa_c * K_ref factorisation does not apply.
// Reference: src/physics/thermal.cpp:71-165 (residual form), src/managers/assembly/
// assemblyManager_jacres.hpp:121-630 (workset loop), assemblyManager_scatter.hpp:164-278 (scatter).
//
// Residual (FP64).  NL = (P+1)^3 lanes per cell (27 for Q2: one cell per warp; 8 for Q1: four cells
// per warp), lane = one tensor-product index.  Values and reference gradients at the Gauss points come
// from sum factorisation (three 1-D contractions with the (P+1)x(P+1) Lagrange value / derivative
// tables); the flux F_d = W diff s_d^2 g_d is formed pointwise and contracted back the same way.  For
// Q2 that is ~60 FP64 operations per lane instead of ~216 for dense 27x27 contractions -- the FP64 pipe
// is the binding roof on GB300.  Cells run in 8 colours (no shared nodes within a launch), so the
// scatter is a plain deterministic read-modify-write.  The kernel optionally stores, per cell and
// point, cw_q = W diff_q and ew_{q,d} = W 2 u_q s_d^2 g_d(q) for the Jacobian pass.
//
// Jacobian.  K[l][j] = sum_{d,q} G_d[q][l] (s_d^2 cw_q G_d[q][j]) + sum_q (sum_d G_d[q][l] ew_{q,d}) Phi[q][j]
// where G_d / Phi are the reference gradient / value tables.  Row gather: one thread per CSR row loops
// over the row's cells in a fixed order, forms the coefficient vector (alpha, beta) of its (row, cell)
// pair and multiplies it by the constant table [G; Phi] held in shared memory.  The CTA's rows are
// contiguous in CSR: they are staged in shared memory and written once with 16-byte stores.  Every
// (row, cell) pair is one row of a GEMM with a constant right operand.
#include <cmath>
#include <cstdio>
#include <vector>

#include "mrg_fixmul.cuh"
#include "mrg_internal.h"

namespace {

struct TPTabs {
  double phi1[3][3];  // [gauss point][node] 1-D Lagrange values
  double dph1[3][3];  // 1-D derivatives (reference coordinate in [-1,1])
  double W[27];       // w_q * |detJ|
  double s[3];        // 2 / h_d
  double load[27];    // f * sum_q W_q phi_l(q)
  float phi1f[3][3], dph1f[3][3], Wf[27], sf[3];  // FP32 copies for the FP32 coefficient pass
};

// table access in the pass's arithmetic type
template <typename CT>
__device__ __forceinline__ CT tp_phi(const TPTabs& T, int q, int a) {
  if constexpr (sizeof(CT) == 4) return T.phi1f[q][a]; else return T.phi1[q][a];
}
template <typename CT>
__device__ __forceinline__ CT tp_dph(const TPTabs& T, int q, int a) {
  if constexpr (sizeof(CT) == 4) return T.dph1f[q][a]; else return T.dph1[q][a];
}
template <typename CT>
__device__ __forceinline__ CT tp_w(const TPTabs& T, int q) {
  if constexpr (sizeof(CT) == 4) return T.Wf[q]; else return T.W[q];
}
template <typename CT>
__device__ __forceinline__ CT tp_s(const TPTabs& T, int d) {
  if constexpr (sizeof(CT) == 4) return T.sf[d]; else return T.s[d];
}

template <int P>
struct TP {
  static constexpr int N1 = P + 1;           // nodes = Gauss points per axis
  static constexpr int NL = N1 * N1 * N1;    // nodes = points per cell
  static constexpr int CPW = 32 / NL;        // cells per warp
  static constexpr int NQB = 4 * NL;         // per-cell coefficient block: cw (NL) + ew (3 NL)
  static constexpr int TS = (NL + 3) / 4 * 4;  // table row stride (16-byte rows)
  static constexpr int RMAX = (2 * P + 1) * (2 * P + 1) * (2 * P + 1);  // max row length
};

__device__ __forceinline__ void split3(int l, int n1, int& i0, int& i1, int& i2) {
  i0 = l % n1;
  i1 = (l / n1) % n1;
  i2 = l / (n1 * n1);
}

constexpr int RW = 8;  // warps per CTA in the residual kernel

// round to the nearest TF32 value (10 explicit mantissa bits, ties away from zero)
__device__ __forceinline__ float tf32_rn(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;\n" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// FP32 value of an interpolated quantity: FP32 stages pass it through, FP64 stages round it to nearest
// on the integer pipes (the conversion instruction issues at the FP64 rate)
__device__ __forceinline__ float to_f32(float v) { return v; }
__device__ __forceinline__ float to_f32(double v) { return mrgfix::f64_to_f32_rn(v); }

// mode bits: 1 = scatter residual, 2 = store qp coefficients (QT precision).  CT = arithmetic type of
// the interpolation stages: double for every pass that scatters the residual; float for the pass that
// only stores the FP32 coefficients of the FP32 Jacobian (1 + u^2 and 2 u grad u at the Gauss points),
// which the FP64 stages made FP64-pipe bound (~1,000 FP64 operations a cell).
template <int P, typename QT, typename CT = double>
__global__ void __launch_bounds__(RW * 32) k_tp_res(const TPTabs T, Grid g, int color, int cc0, int cc1, int64_t ncl,
                                                    int kind, const double* __restrict__ u,
                                                    const double* __restrict__ kap, double* __restrict__ r,
                                                    QT* __restrict__ qbuf, int tc_image, int mode) {
  using K = TP<P>;
  constexpr int N1 = K::N1, NL = K::NL;
  __shared__ CT sm[RW][K::CPW][6][NL];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int sub = lane / NL, l = lane % NL;
  const int64_t cl = ((int64_t)blockIdx.x * RW + w) * K::CPW + sub;
  const bool on = (sub < K::CPW) && (cl < ncl);
  int cx = 0, cy = 0, cz = 0;
  if (on) {
    if (color < 0) {
      cx = (int)(cl % g.nc[0]);
      int64_t t = cl / g.nc[0];
      cy = (int)(t % g.nc[1]);
      cz = (int)(t / g.nc[1]);
    } else {
      int kx = (int)(cl % cc0);
      int64_t t = cl / cc0;
      int ky = (int)(t % cc1);
      int kz = (int)(t / cc1);
      cx = 2 * kx + (color & 1);
      cy = 2 * ky + ((color >> 1) & 1);
      cz = 2 * kz + ((color >> 2) & 1);
    }
  }
  const int64_t cid = cx + (int64_t)g.nc[0] * (cy + (int64_t)g.nc[1] * cz);
  int i0 = 0, i1 = 0, i2 = 0;
  split3(l, N1, i0, i1, i2);
  const int sc = on ? sub : 0;
  CT* U = sm[w][sc][0];
  CT* X0 = sm[w][sc][1];
  CT* X1 = sm[w][sc][2];
  CT* Y0 = sm[w][sc][3];
  CT* Y1 = sm[w][sc][4];
  CT* Y2 = sm[w][sc][5];
  const int NX = g.nn[0], NY = g.nn[1];
  int64_t node = 0;
  if (on) {
    node = (P * cx + i0) + (int64_t)NX * ((P * cy + i1) + (int64_t)NY * (P * cz + i2));
    U[l] = (CT)__ldg(u + node);
  }
  __syncwarp();
  // stage x: lane (qx,b,c)
  if (on) {
    CT a0 = CT(0), a1 = CT(0);
#pragma unroll
    for (int a = 0; a < N1; ++a) {
      const CT v = U[a + N1 * i1 + N1 * N1 * i2];
      a0 = fma(tp_phi<CT>(T, i0, a), v, a0);
      a1 = fma(tp_dph<CT>(T, i0, a), v, a1);
    }
    X0[l] = a0;
    X1[l] = a1;
  }
  __syncwarp();
  // stage y: lane (qx,qy,c)
  if (on) {
    CT b0 = CT(0), b1 = CT(0), b2 = CT(0);
#pragma unroll
    for (int b = 0; b < N1; ++b) {
      const CT ux = X0[i0 + N1 * b + N1 * N1 * i2], dx = X1[i0 + N1 * b + N1 * N1 * i2];
      b0 = fma(tp_phi<CT>(T, i1, b), ux, b0);
      b1 = fma(tp_phi<CT>(T, i1, b), dx, b1);
      b2 = fma(tp_dph<CT>(T, i1, b), ux, b2);
    }
    Y0[l] = b0;
    Y1[l] = b1;
    Y2[l] = b2;
  }
  __syncwarp();
  // stage z: lane = Gauss point q; pointwise flux
  CT Fx = CT(0), Fy = CT(0), Fz = CT(0);
  if (on) {
    CT uq = CT(0), gx = CT(0), gy = CT(0), gz = CT(0);
#pragma unroll
    for (int c = 0; c < N1; ++c) {
      const int k = i0 + N1 * i1 + N1 * N1 * c;
      uq = fma(tp_phi<CT>(T, i2, c), Y0[k], uq);
      gx = fma(tp_phi<CT>(T, i2, c), Y1[k], gx);
      gy = fma(tp_phi<CT>(T, i2, c), Y2[k], gy);
      gz = fma(tp_dph<CT>(T, i2, c), Y0[k], gz);
    }
    const CT Wq = tp_w<CT>(T, l);
    const CT diff = (kind == MRG_THERMAL) ? (CT)__ldg(kap + cid) : CT(1) + uq * uq;
    const CT cw = Wq * diff;
    Fx = cw * tp_s<CT>(T, 0) * tp_s<CT>(T, 0) * gx;
    Fy = cw * tp_s<CT>(T, 1) * tp_s<CT>(T, 1) * gy;
    Fz = cw * tp_s<CT>(T, 2) * tp_s<CT>(T, 2) * gz;
    if (mode & 2) {
      QT* qb = qbuf + cid * K::NQB;
      // tc_image (FP32 only): split x = hi + lo (hi = x rounded to TF32, lo = the FP32 remainder rounded to
      // TF32) and store both into the tensor-core operand image [tile][hi, lo][K chunk][cell][4] with
      // 128-cell tiles and 112 K slots; otherwise plain QT values [cell][4 NL]
      auto put = [&](int k, CT v) {
        if constexpr (sizeof(QT) == 4) {
          if (tc_image) {
            // split of the FP32 value (the remainder is exact in FP32; 3xTF32 keeps ~22 bits anyway):
            // one FP64 -> FP32 rounding per value, on the integer pipes, the rest on the FP32 pipe
            const float f = to_f32(v);
            const float hi = tf32_rn(f);
            float* t = qbuf + (cid >> 7) * (2 * 128 * 112) + (k >> 2) * 512 + (cid & 127) * 4 + (k & 3);
            t[0] = hi;
            t[128 * 112] = tf32_rn(f - hi);
            return;
          }
        }
        if constexpr (sizeof(QT) == 4) qb[k] = to_f32(v);
        else qb[k] = (QT)v;
      };
      put(l, cw);
      if (kind != MRG_THERMAL) {
        const CT e = Wq * CT(2) * uq;
        put(NL + l, e * tp_s<CT>(T, 0) * tp_s<CT>(T, 0) * gx);
        put(2 * NL + l, e * tp_s<CT>(T, 1) * tp_s<CT>(T, 1) * gy);
        put(3 * NL + l, e * tp_s<CT>(T, 2) * tp_s<CT>(T, 2) * gz);
      }
    }
  }
  if (!(mode & 1)) return;
  __syncwarp();
  if (on) {
    X0[l] = Fx;
    X1[l] = Fy;
    Y0[l] = Fz;
  }
  __syncwarp();
  // transpose z: lane (qx,qy,c)
  CT Ax = CT(0), Ay = CT(0), Az = CT(0);
  if (on) {
#pragma unroll
    for (int qz = 0; qz < N1; ++qz) {
      const int k = i0 + N1 * i1 + N1 * N1 * qz;
      Ax = fma(tp_phi<CT>(T, qz, i2), X0[k], Ax);
      Ay = fma(tp_phi<CT>(T, qz, i2), X1[k], Ay);
      Az = fma(tp_dph<CT>(T, qz, i2), Y0[k], Az);
    }
  }
  __syncwarp();
  if (on) {
    Y1[l] = Ax;
    Y2[l] = Ay;
    U[l] = Az;
  }
  __syncwarp();
  // transpose y: lane (qx,b,c)
  CT Bx = CT(0), Byz = CT(0);
  if (on) {
#pragma unroll
    for (int qy = 0; qy < N1; ++qy) {
      const int k = i0 + N1 * qy + N1 * N1 * i2;
      Bx = fma(tp_phi<CT>(T, qy, i1), Y1[k], Bx);
      Byz = fma(tp_dph<CT>(T, qy, i1), Y2[k], Byz);
      Byz = fma(tp_phi<CT>(T, qy, i1), U[k], Byz);
    }
  }
  __syncwarp();
  if (on) {
    X0[l] = Bx;
    X1[l] = Byz;
  }
  __syncwarp();
  // transpose x: lane (a,b,c) = element row
  if (on) {
    CT res = (CT)(-T.load[l]);
#pragma unroll
    for (int qx = 0; qx < N1; ++qx) {
      const int k = qx + N1 * i1 + N1 * N1 * i2;
      res = fma(tp_dph<CT>(T, qx, i0), X0[k], res);
      res = fma(tp_phi<CT>(T, qx, i0), X1[k], res);
    }
    if (!node_fixed(g, P * cx + i0, P * cy + i1, P * cz + i2)) r[node] -= res;  // r += -res.val()
  }
}

// ---- Jacobian row gather --------------------------------------------------------------------------
constexpr int JR = 64;  // rows per CTA

template <typename T>
__device__ __forceinline__ void seg_store_tp(T* __restrict__ dst, const T* __restrict__ src, int64_t len, bool add) {
  constexpr int V = 16 / sizeof(T);
  int head = (int)(((16 - ((uintptr_t)dst & 15)) & 15) / sizeof(T));
  if (head > len) head = (int)len;
  for (int k = threadIdx.x; k < head; k += blockDim.x) dst[k] = add ? dst[k] + src[k] : src[k];
  const int64_t body = (len - head) / V;
  if constexpr (sizeof(T) == 8) {
    const double2* s2 = reinterpret_cast<const double2*>(src + head);
    double2* d2 = reinterpret_cast<double2*>(dst + head);
    for (int64_t v = threadIdx.x; v < body; v += blockDim.x) {
      double2 x = s2[v];
      if (add) { double2 y = d2[v]; x.x += y.x; x.y += y.y; d2[v] = x; } else __stcs(d2 + v, x);
    }
  } else {
    const float4* s4 = reinterpret_cast<const float4*>(src + head);
    float4* d4 = reinterpret_cast<float4*>(dst + head);
    for (int64_t v = threadIdx.x; v < body; v += blockDim.x) {
      float4 x = s4[v];
      if (add) { float4 y = d4[v]; x.x += y.x; x.y += y.y; x.z += y.z; x.w += y.w; d4[v] = x; } else __stcs(d4 + v, x);
    }
  }
  for (int64_t k = head + body * V + threadIdx.x; k < len; k += blockDim.x) dst[k] = add ? dst[k] + src[k] : src[k];
}

__device__ __forceinline__ void decompose32(const Grid& g, int64_t n, int& ix, int& iy, int& iz) {
  const unsigned un = (unsigned)n, nx = (unsigned)g.nn[0], ny = (unsigned)g.nn[1];
  const unsigned t = un / nx;
  ix = (int)(un - t * nx);
  iy = (int)(t % ny);
  iz = (int)(t / ny);
}

__device__ __forceinline__ int64_t rowptr_tp(const Grid& g, int ix, int iy, int iz, int& lx, int& ly, int& lz,
                                             int& cx, int& cy, int& cz) {
  axis_range(ix, g.nn[0], g.p, lx, cx);
  axis_range(iy, g.nn[1], g.p, ly, cy);
  axis_range(iz, g.nn[2], g.p, lz, cz);
  return g.P[2][iz] * g.T[1] * g.T[0] + (int64_t)cz * (g.P[1][iy] * g.T[0] + (int64_t)cy * g.P[0][ix]);
}

__device__ __forceinline__ int64_t rowptr_at(const Grid& g, int64_t n, int64_t nrows) {
  if (n >= nrows) return g.T[0] * g.T[1] * g.T[2];
  int ix, iy, iz, a, b, c, d, e, f;
  decompose32(g, n, ix, iy, iz);
  return rowptr_tp(g, ix, iy, iz, a, b, c, d, e, f);
}

// tab: [G_x | G_y | G_z | Phi] as [q][j] blocks, tab[(d*NL + q)*TS + j], d = 3 for Phi.
// Q1 1-D tables for the Jacobian: l[q][a] = phi_a(xi_q) at the 2 Gauss points, d[a] = phi_a' (constant)
struct Tab1 {
  double l[2][2];
  double d[2];
};

// Row l of one Q1 cell's Jacobian, added to acc[0..7] (node and Gauss-point indices x fastest).  The
// reference gradient of a linear node along its own axis is the constant d[.], so with
// C(q_b, q_c) = sum over q_a of cw_q the stiffness part along axis a is
//     s_a^2 d[l_a] d[j_a] sum_{q_b, q_c} C l[q_b][l_b] l[q_c][l_c] l[q_b][j_b] l[q_c][j_c]
// (two 2 x 2 contractions), and the advective part sum_q b_q phi_j(q) factorises axis by axis: ~200
// operations per row and cell where the general loop takes ~330.
template <typename JT>
__device__ __forceinline__ void q1_cell_row(const Tab1& t1, const JT sq[3], int l, int kind, const JT* __restrict__ tab,
                                            const JT* __restrict__ qb, JT acc[8]) {
  constexpr int NL = 8, TS = 8;
  JT L[2][2], D[2];
#pragma unroll
  for (int q = 0; q < 2; ++q)
#pragma unroll
    for (int a = 0; a < 2; ++a) L[q][a] = (JT)t1.l[q][a];
  D[0] = (JT)t1.d[0];
  D[1] = (JT)t1.d[1];
  JT cw[NL];
#pragma unroll
  for (int q = 0; q < NL; ++q) cw[q] = qb[q];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const int b = (a == 0) ? 1 : 0, c = (a == 2) ? 1 : 2;
    JT C[2][2] = {{JT(0), JT(0)}, {JT(0), JT(0)}};
#pragma unroll
    for (int q = 0; q < NL; ++q) C[(q >> b) & 1][(q >> c) & 1] += cw[q];
    const int lb = (l >> b) & 1, lc = (l >> c) & 1;
    JT W[2][2], U[2][2], T[2][2];
#pragma unroll
    for (int pb = 0; pb < 2; ++pb)
#pragma unroll
      for (int pc = 0; pc < 2; ++pc) W[pb][pc] = C[pb][pc] * L[pb][lb] * L[pc][lc];
#pragma unroll
    for (int pb = 0; pb < 2; ++pb)
#pragma unroll
      for (int jc = 0; jc < 2; ++jc) U[pb][jc] = W[pb][0] * L[0][jc] + W[pb][1] * L[1][jc];
#pragma unroll
    for (int jb = 0; jb < 2; ++jb)
#pragma unroll
      for (int jc = 0; jc < 2; ++jc) T[jb][jc] = U[0][jc] * L[0][jb] + U[1][jc] * L[1][jb];
    const JT f = sq[a] * D[(l >> a) & 1];
    const JT fd[2] = {f * D[0], f * D[1]};
#pragma unroll
    for (int j = 0; j < NL; ++j) acc[j] += fd[(j >> a) & 1] * T[(j >> b) & 1][(j >> c) & 1];
  }
  if (kind != MRG_THERMAL) {
    // b_q = sum_d G_d[q][l] ew_{q,d}, then sum_q b_q phi_j(q) one axis at a time (z, y, then x into acc)
    JT bq[NL];
#pragma unroll
    for (int q = 0; q < NL; ++q)
      bq[q] = tab[(0 * NL + q) * TS + l] * qb[NL + q] + tab[(1 * NL + q) * TS + l] * qb[2 * NL + q] +
              tab[(2 * NL + q) * TS + l] * qb[3 * NL + q];
    JT V1[2][2][2], V2[2][2][2];  // [qx][qy][jz], then [qx][jy][jz]
#pragma unroll
    for (int qx = 0; qx < 2; ++qx)
#pragma unroll
      for (int qy = 0; qy < 2; ++qy)
#pragma unroll
        for (int jz = 0; jz < 2; ++jz)
          V1[qx][qy][jz] = bq[qx + 2 * qy] * L[0][jz] + bq[qx + 2 * qy + 4] * L[1][jz];
#pragma unroll
    for (int qx = 0; qx < 2; ++qx)
#pragma unroll
      for (int jy = 0; jy < 2; ++jy)
#pragma unroll
        for (int jz = 0; jz < 2; ++jz) V2[qx][jy][jz] = V1[qx][0][jz] * L[0][jy] + V1[qx][1][jz] * L[1][jy];
#pragma unroll
    for (int j = 0; j < NL; ++j) {
      const int jx = j & 1, jy = (j >> 1) & 1, jz = j >> 2;
      acc[j] += V2[0][jy][jz] * L[0][jx] + V2[1][jy][jz] * L[1][jx];
    }
  }
}

template <int P, typename JT>
__global__ void __launch_bounds__(JR) k_tp_jac(Grid g, int64_t nrows, int kind, const double s0, const double s1,
                                               const double s2, const JT* __restrict__ tab_g,
                                               const JT* __restrict__ qbuf, JT* __restrict__ J, int ovw,
                                               const Tab1 t1) {
  using K = TP<P>;
  constexpr int N1 = K::N1, NL = K::NL, TS = K::TS;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  JT* tab = reinterpret_cast<JT*>(smem_raw);  // 4*NL*TS
  JT* sv_base = tab + 4 * NL * TS;             // staged segment (JR*RMAX + pad)
  for (int k = threadIdx.x; k < 4 * NL * TS; k += blockDim.x) tab[k] = tab_g[k];
  const int64_t n0 = (int64_t)blockIdx.x * JR;
  const int64_t n1 = (n0 + JR < nrows) ? n0 + JR : nrows;
  const int64_t seg0 = rowptr_at(g, n0, nrows), seg1 = rowptr_at(g, n1, nrows);
  const int phase = (int)(((uintptr_t)(J + seg0) & 15) / sizeof(JT));
  JT* sv = sv_base + phase;
  for (int64_t k = threadIdx.x; k < seg1 - seg0; k += blockDim.x) sv[k] = JT(0);
  __syncthreads();
  const int64_t n = n0 + threadIdx.x;
  const JT sq[3] = {(JT)(s0 * s0), (JT)(s1 * s1), (JT)(s2 * s2)};
  bool fixed = false;
  int64_t rp = 0, diag = 0;
  if (n < nrows) {
    int ix, iy, iz, lx, ly, lz, cxn, cyn, czn;
    decompose32(g, n, ix, iy, iz);
    rp = rowptr_tp(g, ix, iy, iz, lx, ly, lz, cxn, cyn, czn);
    JT* row = sv + (rp - seg0);
    diag = ((int64_t)(iz - lz) * cyn + (iy - ly)) * cxn + (ix - lx);
    fixed = node_fixed(g, ix, iy, iz);
    if (fixed) {
      if (ovw) row[diag] = JT(1);
    } else {
      int fx, fy, fz, nxc, nyc, nzc;
      axis_cells(ix, g.nn[0], P, fx, nxc);
      axis_cells(iy, g.nn[1], P, fy, nyc);
      axis_cells(iz, g.nn[2], P, fz, nzc);
      for (int ccz = fz; ccz < fz + nzc; ++ccz)
        for (int ccy = fy; ccy < fy + nyc; ++ccy)
          for (int ccx = fx; ccx < fx + nxc; ++ccx) {
            const int l = (ix - P * ccx) + N1 * (iy - P * ccy) + N1 * N1 * (iz - P * ccz);
            const int64_t cid = ccx + (int64_t)g.nc[0] * (ccy + (int64_t)g.nc[1] * ccz);
            const JT* qb = qbuf + cid * K::NQB;
            JT acc[NL];
#pragma unroll
            for (int j = 0; j < NL; ++j) acc[j] = JT(0);
            if constexpr (P == 1) {
              q1_cell_row<JT>(t1, sq, l, kind, tab, qb, acc);
            } else {
            // stiffness part: alpha_{d,q} = G_d[q][l] s_d^2 cw_q against G_d[q][:]
            for (int q = 0; q < NL; ++q) {
              const JT cw = qb[q];
#pragma unroll
              for (int d = 0; d < 3; ++d) {
                const JT* trow = tab + (d * NL + q) * TS;
                const JT a = trow[l] * sq[d] * cw;
#pragma unroll
                for (int j = 0; j < NL; ++j) acc[j] += a * trow[j];
              }
            }
            if (kind != MRG_THERMAL) {
              // advective part: beta_q = sum_d G_d[q][l] ew_{q,d} against Phi[q][:]
              for (int q = 0; q < NL; ++q) {
                const JT b = tab[(0 * NL + q) * TS + l] * qb[NL + q] + tab[(1 * NL + q) * TS + l] * qb[2 * NL + q] +
                             tab[(2 * NL + q) * TS + l] * qb[3 * NL + q];
                const JT* prow = tab + (3 * NL + q) * TS;
#pragma unroll
                for (int j = 0; j < NL; ++j) acc[j] += b * prow[j];
              }
            }
            }
            // add into the row: column of local node j of this cell
#pragma unroll
            for (int j = 0; j < NL; ++j) {
              const int jx = P * ccx + j % N1, jy = P * ccy + (j / N1) % N1, jz = P * ccz + j / (N1 * N1);
              row[((int64_t)(jz - lz) * cyn + (jy - ly)) * cxn + (jx - lx)] += acc[j];
            }
          }
    }
  }
  __syncthreads();
  seg_store_tp<JT>(J + seg0, sv, seg1 - seg0, !ovw);
  if (!ovw) {
    __syncthreads();
    if (n < nrows && fixed) J[rp + diag] = JT(1);
  }
}

inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

// ------------------------------------------------------------------------------------------------
// host side
// ------------------------------------------------------------------------------------------------
struct TPData {
  TPTabs T;
  int P = 2;
  double* d_tab64 = nullptr;
  float* d_tab32 = nullptr;
  void* d_qbuf = nullptr;  // ncell * 4 NL (FP64 or FP32, by the last Jacobian request)
  size_t qbuf_bytes = 0;
  int* d_err = nullptr;    // tensor-core kernel status (bounded waits), sticky until reported
  int* h_err = nullptr;    // pinned mirror, refreshed asynchronously after every tensor-core launch
  cudaEvent_t err_ev = nullptr;  // recorded after the refresh
  bool err_pending = false;
  std::vector<double> tab_host;  // [G_x | G_y | G_z | Phi] rows of TS doubles
  Q2Tc* tc = nullptr;      // tensor-core element-matrix plan (Q2, FP32 Jacobian), built on first use
};

static TPData* tpdata(mrg_problem* p) { return reinterpret_cast<TPData*>(p->q2); }

int mrg_q2_setup(mrg_problem* p) {
  TPData* Q = new TPData();
  p->q2 = Q;
  const int P = p->g.p, N1 = P + 1, NL = N1 * N1 * N1;
  const int TS = (NL + 3) / 4 * 4;
  Q->P = P;
  const int nq = p->nq, npe = p->npe;  // == NL
  const double* tw = p->qtab_host.data();
  const double* tphi = tw + nq;
  const double* tdphi = tphi + npe * nq;
  for (int q = 0; q < 3; ++q)
    for (int a = 0; a < 3; ++a) {
      Q->T.phi1[q][a] = 0.0;
      Q->T.dph1[q][a] = 0.0;
    }
  for (int q = 0; q < N1; ++q) {
    const double x = p->gx1[q];
    if (P == 2) {
      const double l[3] = {0.5 * x * (x - 1.0), 1.0 - x * x, 0.5 * x * (x + 1.0)};
      const double dl[3] = {x - 0.5, -2.0 * x, x + 0.5};
      for (int a = 0; a < 3; ++a) {
        Q->T.phi1[q][a] = l[a];
        Q->T.dph1[q][a] = dl[a];
      }
    } else {
      const double l[2] = {0.5 * (1.0 - x), 0.5 * (1.0 + x)};
      const double dl[2] = {-0.5, 0.5};
      for (int a = 0; a < 2; ++a) {
        Q->T.phi1[q][a] = l[a];
        Q->T.dph1[q][a] = dl[a];
      }
    }
  }
  double detJ = 1.0;
  for (int d = 0; d < 3; ++d) {
    detJ *= 0.5 * p->h[d];
    Q->T.s[d] = 2.0 / p->h[d];
  }
  for (int q = 0; q < 27; ++q) Q->T.W[q] = (q < nq) ? tw[q] * detJ : 0.0;
  for (int q = 0; q < 3; ++q)
    for (int a = 0; a < 3; ++a) {
      Q->T.phi1f[q][a] = (float)Q->T.phi1[q][a];
      Q->T.dph1f[q][a] = (float)Q->T.dph1[q][a];
    }
  for (int q = 0; q < 27; ++q) Q->T.Wf[q] = (float)Q->T.W[q];
  for (int d = 0; d < 3; ++d) Q->T.sf[d] = (float)Q->T.s[d];
  for (int l = 0; l < 27; ++l) {
    double s = 0.0;
    if (l < npe)
      for (int q = 0; q < nq; ++q) s += Q->T.W[q] * tphi[l * nq + q];
    Q->T.load[l] = p->source_amp * s;
  }
  std::vector<double> tab(4 * NL * TS, 0.0);
  std::vector<float> tab32(4 * NL * TS, 0.0f);
  for (int d = 0; d < 4; ++d)
    for (int q = 0; q < NL; ++q)
      for (int j = 0; j < NL; ++j)
        tab[(d * NL + q) * TS + j] = (d < 3) ? tdphi[(j * nq + q) * 3 + d] : tphi[j * nq + q];
  for (size_t k = 0; k < tab.size(); ++k) tab32[k] = (float)tab[k];
  Q->tab_host = tab;
  cudaStream_t s = p->stream;
  MRG_CUDA(cudaMallocAsync(&Q->d_err, sizeof(int), s));
  MRG_CUDA(cudaMemsetAsync(Q->d_err, 0, sizeof(int), s));
  MRG_CUDA(cudaMallocAsync(&Q->d_tab64, tab.size() * sizeof(double), s));
  MRG_CUDA(cudaMallocAsync(&Q->d_tab32, tab.size() * sizeof(float), s));
  MRG_CUDA(cudaMemcpyAsync(Q->d_tab64, tab.data(), tab.size() * sizeof(double), cudaMemcpyHostToDevice, s));
  MRG_CUDA(cudaMemcpyAsync(Q->d_tab32, tab32.data(), tab32.size() * sizeof(float), cudaMemcpyHostToDevice, s));
  MRG_CUDA(cudaStreamSynchronize(s));
  return MRG_OK;
}

void mrg_q2_free(mrg_problem* p) {
  TPData* Q = tpdata(p);
  if (!Q) return;
  cudaFreeAsync(Q->d_tab64, p->stream);
  cudaFreeAsync(Q->d_tab32, p->stream);
  cudaFreeAsync(Q->d_err, p->stream);
  if (Q->err_ev) cudaEventDestroy(Q->err_ev);
  mrg_pinned_release(Q->h_err);
  if (Q->d_qbuf) cudaFreeAsync(Q->d_qbuf, p->stream);
  mrg_q2tc_free(Q->tc, p->stream);
  delete Q;
  p->q2 = nullptr;
}

template <int P>
static int launch_res_t(mrg_problem* p, const double* u, double* r, void* qbuf, bool tc_image, bool fp32q, int mode,
                        cudaStream_t s) {
  TPData* Q = tpdata(p);
  const Grid& g = p->g;
  constexpr int CPB = RW * TP<P>::CPW;  // cells per CTA
  auto launch = [&](int color, int cc0, int cc1, int64_t tot) {
    if (fp32q && !(mode & 1))
      k_tp_res<P, float, float><<<nblk(tot, CPB), RW * 32, 0, s>>>(Q->T, g, color, cc0, cc1, tot, p->kind, u,
                                                                    p->d_kappa, r, (float*)qbuf, tc_image ? 1 : 0, mode);
    else if (fp32q)
      k_tp_res<P, float><<<nblk(tot, CPB), RW * 32, 0, s>>>(Q->T, g, color, cc0, cc1, tot, p->kind, u, p->d_kappa, r,
                                                             (float*)qbuf, tc_image ? 1 : 0, mode);
    else
      k_tp_res<P, double><<<nblk(tot, CPB), RW * 32, 0, s>>>(Q->T, g, color, cc0, cc1, tot, p->kind, u, p->d_kappa, r,
                                                              (double*)qbuf, 0, mode);
    return cudaGetLastError();
  };
  if (mode & 1) {
    // 8 colours: no two cells of one launch share a node
    for (int c = 0; c < 8; ++c) {
      int cc[3];
      int64_t tot = 1;
      for (int k = 0; k < 3; ++k) {
        int bit = (c >> k) & 1;
        cc[k] = (g.nc[k] - bit + 1) / 2;
        tot *= cc[k];
      }
      if (tot == 0) continue;
      cudaError_t e = launch(c, cc[0], cc[1], tot);
      if (e != cudaSuccess) return mrg_cuda_check(e, "tensor-product residual launch");
    }
  } else {
    cudaError_t e = launch(-1, 1, 1, p->ncell);
    if (e != cudaSuccess) return mrg_cuda_check(e, "tensor-product qp-coefficient launch");
  }
  return MRG_OK;
}

template <int P, typename JT>
static cudaError_t launch_jac_t(mrg_problem* p, const JT* tab, const void* qbuf, JT* J, bool ovw, cudaStream_t s) {
  using K = TP<P>;
  TPData* Q = tpdata(p);
  const int smem = (4 * K::NL * K::TS + JR * K::RMAX + 16 / (int)sizeof(JT)) * (int)sizeof(JT);
  auto kern = k_tp_jac<P, JT>;
  if (smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  Tab1 t1;
  for (int q = 0; q < 2; ++q)
    for (int a = 0; a < 2; ++a) t1.l[q][a] = Q->T.phi1[q][a];
  for (int a = 0; a < 2; ++a) t1.d[a] = Q->T.dph1[0][a];
  kern<<<nblk(p->ndof, JR), JR, smem, s>>>(p->g, p->ndof, p->kind, Q->T.s[0], Q->T.s[1], Q->T.s[2], tab,
                                           (const JT*)qbuf, J, ovw ? 1 : 0, t1);
  return cudaGetLastError();
}

int mrg_launch_q2(mrg_problem* p, const double* u, double* r, void* J, uint32_t flags, cudaStream_t s) {
  TPData* Q = tpdata(p);
  const int P = Q->P, NL = (P + 1) * (P + 1) * (P + 1);
  const bool doJ = flags & MRG_ASM_JAC, doR = flags & MRG_ASM_RES, ovw = flags & MRG_ASM_OVERWRITE;
  const bool fp32 = flags & MRG_ASM_J_FP32;
  void* qbuf = nullptr;
  const bool tc = doJ && P == 2 && fp32 && !(flags & MRG_ASM_CUDA_CORES);
  if (tc) {
    // A time-out inside a previous tensor-core launch is reported here, without synchronising: the
    // status word is copied to pinned memory behind an event after every launch and read once that
    // event has completed, so the assembly stays free of host synchronisation (graph-capturable once
    // the workspace exists).
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    MRG_CUDA(cudaStreamIsCapturing(s, &cap));
    const bool capturing = cap != cudaStreamCaptureStatusNone;
    if (!capturing && Q->err_pending && cudaEventQuery(Q->err_ev) == cudaSuccess) {
      Q->err_pending = false;
      if (*Q->h_err) {
        *Q->h_err = 0;
        MRG_CUDA(cudaMemsetAsync(Q->d_err, 0, sizeof(int), s));
        return mrg_fail(MRG_ETIMEOUT, "tensor-core element kernel: an mbarrier wait timed out in a previous launch");
      }
    }
    // tensor cores: the residual pass writes the TF32 hi/lo planes of W straight into the plan's buffer.
    // The first call allocates the workspace (element matrices, operand images) and uploads the
    // constant operand: make it outside stream capture.
    if (!Q->tc) {
      int st = mrg_q2tc_create(p, Q->tab_host.data(), Q->T.s, &Q->tc, s);
      if (st) return st;
      Q->h_err = (int*)mrg_pinned_slot();
      if (!Q->h_err) return mrg_fail(MRG_ENOMEM, "pinned error word");
      *Q->h_err = 0;
      MRG_CUDA(cudaEventCreateWithFlags(&Q->err_ev, cudaEventDisableTiming));
    }
    if (doR && ovw) MRG_CUDA(cudaMemsetAsync(r, 0, p->ndof * sizeof(double), s));
    int st = launch_res_t<2>(p, u, doR ? r : nullptr, mrg_q2tc_w_image(Q->tc), true, true, (doR ? 1 : 0) | 2, s);
    if (st) return st;
    st = mrg_q2tc_launch(p, Q->tc, (float*)J, ovw, Q->d_err, s);
    if (st) return st;
    MRG_CUDA(cudaMemcpyAsync(Q->h_err, Q->d_err, sizeof(int), cudaMemcpyDeviceToHost, s));
    if (!capturing) {
      MRG_CUDA(cudaEventRecord(Q->err_ev, s));
      Q->err_pending = true;
    }
    return MRG_OK;
  }
  if (doJ) {
    const size_t need = (size_t)p->ncell * 4 * NL * (fp32 ? sizeof(float) : sizeof(double));
    if (Q->qbuf_bytes < need) {
      if (Q->d_qbuf) cudaFreeAsync(Q->d_qbuf, s);
      Q->d_qbuf = nullptr;
      Q->qbuf_bytes = 0;
      MRG_CUDA(cudaMallocAsync(&Q->d_qbuf, need, s));
      Q->qbuf_bytes = need;
    }
    qbuf = Q->d_qbuf;
  }
  if (doR && ovw) MRG_CUDA(cudaMemsetAsync(r, 0, p->ndof * sizeof(double), s));
  const int mode = (doR ? 1 : 0) | (doJ ? 2 : 0);
  int st = (P == 2) ? launch_res_t<2>(p, u, doR ? r : nullptr, qbuf, false, fp32, mode, s)
                    : launch_res_t<1>(p, u, doR ? r : nullptr, qbuf, false, fp32, mode, s);
  if (st) return st;
  if (doJ) {
    cudaError_t e;
    if (P == 2)
      e = fp32 ? launch_jac_t<2, float>(p, Q->d_tab32, qbuf, (float*)J, ovw, s)
               : launch_jac_t<2, double>(p, Q->d_tab64, qbuf, (double*)J, ovw, s);
    else
      e = fp32 ? launch_jac_t<1, float>(p, Q->d_tab32, qbuf, (float*)J, ovw, s)
               : launch_jac_t<1, double>(p, Q->d_tab64, qbuf, (double*)J, ovw, s);
    if (e != cudaSuccess) return mrg_cuda_check(e, "tensor-product Jacobian launch");
  }
  return MRG_OK;
}
