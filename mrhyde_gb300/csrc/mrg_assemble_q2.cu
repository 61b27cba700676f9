// Q2 hexahedra on identical affine cells (configuration C3: -div((1+u^2) grad u) = f, 27 nodes and
// 3x3x3 Gauss points per cell).  Reference: src/physics/thermal.cpp:71-165 (residual form),
// src/managers/assembly/assemblyManager_jacres.hpp:121-630 (workset loop), scatter.hpp:164-278.
//
// Residual (FP64).  One warp per cell, lane = one of 27 tensor-product indices.  Values and reference
// gradients at the 27 points come from sum factorisation (three 1-D contractions with the 3x3 Lagrange
// value / derivative tables), the flux F_d = W (1+u^2) s_d^2 g_d is formed pointwise and contracted
// back the same way: ~60 FP64 operations per lane instead of ~216 for dense 27x27 contractions -- the
// FP64 pipe is the binding roof on GB300.  Cells run in 8 colours (no shared nodes within a launch),
// so the scatter is a plain deterministic read-modify-write.  The kernel optionally stores, per cell and
// point, cw_q = W (1+u_q^2) and ew_{q,d} = W 2 u_q s_d^2 g_d(q) for the Jacobian pass.
//
// Jacobian.  K[l][j] = sum_{d,q} G_d[q][l] (s_d^2 cw_q G_d[q][j]) + sum_q (sum_d G_d[q][l] ew_{q,d}) Phi[q][j]
// where G_d / Phi are the reference gradient / value tables.  Row gather: one thread per CSR row loops
// over the row's cells in a fixed order, forms the 108-long coefficient vector (alpha, beta) of its
// (row, cell) pair and multiplies it by the constant 108x27 table [G; Phi] held in shared memory.  The
// CTA's rows are contiguous in CSR: they are staged in shared memory and written once with 16-byte
// stores.  Every (row, cell) pair is one row of a GEMM with a constant right operand.
#include <cmath>
#include <cstdio>
#include <vector>

#include "mrg_internal.h"

namespace {

struct Q2Tabs {
  double phi1[3][3];  // [gauss point][node] 1-D Lagrange values
  double dph1[3][3];  // 1-D derivatives (reference coordinate in [-1,1])
  double W[27];       // w_q * |detJ|
  double s[3];        // 2 / h_d
  double load[27];    // f * sum_q W_q phi_l(q)
};

__device__ __forceinline__ void lane3(int l, int& i0, int& i1, int& i2) {
  i0 = l % 3;
  i1 = (l / 3) % 3;
  i2 = l / 9;
}

constexpr int RW = 8;  // warps (cells) per CTA in the residual kernel

// mode bits: 1 = scatter residual, 2 = store qp coefficients (JT precision)
template <typename QT>
__global__ void __launch_bounds__(RW * 32) k_q2_res(const Q2Tabs T, Grid g, int color, int cc0, int cc1, int64_t ncl,
                                                    int kind, const double* __restrict__ u,
                                                    const double* __restrict__ kap, double* __restrict__ r,
                                                    QT* __restrict__ qbuf, int mode) {
  __shared__ double sm[RW][6][27];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t cl = (int64_t)blockIdx.x * RW + w;
  if (cl >= ncl) return;  // whole warp leaves together
  int cx, cy, cz;
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
  const int64_t cid = cx + (int64_t)g.nc[0] * (cy + (int64_t)g.nc[1] * cz);
  const bool on = lane < 27;
  int i0 = 0, i1 = 0, i2 = 0;
  if (on) lane3(lane, i0, i1, i2);
  double* U = sm[w][0];
  double* X0 = sm[w][1];
  double* X1 = sm[w][2];
  double* Y0 = sm[w][3];
  double* Y1 = sm[w][4];
  double* Y2 = sm[w][5];
  const int NX = g.nn[0], NY = g.nn[1];
  int64_t node = 0;
  if (on) {
    node = (2 * cx + i0) + (int64_t)NX * ((2 * cy + i1) + (int64_t)NY * (2 * cz + i2));
    U[lane] = __ldg(u + node);
  }
  __syncwarp();
  // stage x: lane (qx,b,c)
  if (on) {
    double a0 = 0.0, a1 = 0.0;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const double v = U[a + 3 * i1 + 9 * i2];
      a0 = fma(T.phi1[i0][a], v, a0);
      a1 = fma(T.dph1[i0][a], v, a1);
    }
    X0[lane] = a0;  // Ux
    X1[lane] = a1;  // Dx
  }
  __syncwarp();
  // stage y: lane (qx,qy,c)
  if (on) {
    double b0 = 0.0, b1 = 0.0, b2 = 0.0;
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      const double ux = X0[i0 + 3 * b + 9 * i2], dx = X1[i0 + 3 * b + 9 * i2];
      b0 = fma(T.phi1[i1][b], ux, b0);  // Uxy
      b1 = fma(T.phi1[i1][b], dx, b1);  // DxY
      b2 = fma(T.dph1[i1][b], ux, b2);  // DyY
    }
    Y0[lane] = b0;
    Y1[lane] = b1;
    Y2[lane] = b2;
  }
  __syncwarp();
  // stage z: lane = quadrature point q (qx,qy,qz); pointwise flux
  double Fx = 0.0, Fy = 0.0, Fz = 0.0;
  if (on) {
    double uq = 0.0, gx = 0.0, gy = 0.0, gz = 0.0;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const int k = i0 + 3 * i1 + 9 * c;
      uq = fma(T.phi1[i2][c], Y0[k], uq);
      gx = fma(T.phi1[i2][c], Y1[k], gx);
      gy = fma(T.phi1[i2][c], Y2[k], gy);
      gz = fma(T.dph1[i2][c], Y0[k], gz);
    }
    const double Wq = T.W[lane];
    const double diff = (kind == MRG_THERMAL) ? __ldg(kap + cid) : 1.0 + uq * uq;
    const double cw = Wq * diff;
    Fx = cw * T.s[0] * T.s[0] * gx;
    Fy = cw * T.s[1] * T.s[1] * gy;
    Fz = cw * T.s[2] * T.s[2] * gz;
    if (mode & 2) {
      QT* qb = qbuf + cid * 108;
      qb[lane] = (QT)cw;
      if (kind != MRG_THERMAL) {
        const double e = Wq * 2.0 * uq;
        qb[27 + lane] = (QT)(e * T.s[0] * T.s[0] * gx);
        qb[54 + lane] = (QT)(e * T.s[1] * T.s[1] * gy);
        qb[81 + lane] = (QT)(e * T.s[2] * T.s[2] * gz);
      }
    }
  }
  if (!(mode & 1)) return;
  __syncwarp();
  if (on) {
    X0[lane] = Fx;
    X1[lane] = Fy;
    Y0[lane] = Fz;
  }
  __syncwarp();
  // transpose z: lane (qx,qy,c)
  double Ax = 0.0, Ay = 0.0, Az = 0.0;
  if (on) {
#pragma unroll
    for (int qz = 0; qz < 3; ++qz) {
      const int k = i0 + 3 * i1 + 9 * qz;
      Ax = fma(T.phi1[qz][i2], X0[k], Ax);
      Ay = fma(T.phi1[qz][i2], X1[k], Ay);
      Az = fma(T.dph1[qz][i2], Y0[k], Az);
    }
  }
  __syncwarp();
  if (on) {
    Y1[lane] = Ax;
    Y2[lane] = Ay;
    U[lane] = Az;
  }
  __syncwarp();
  // transpose y: lane (qx,b,c)
  double Bx = 0.0, Byz = 0.0;
  if (on) {
#pragma unroll
    for (int qy = 0; qy < 3; ++qy) {
      const int k = i0 + 3 * qy + 9 * i2;
      Bx = fma(T.phi1[qy][i1], Y1[k], Bx);
      Byz = fma(T.dph1[qy][i1], Y2[k], Byz);
      Byz = fma(T.phi1[qy][i1], U[k], Byz);
    }
  }
  __syncwarp();
  if (on) {
    X0[lane] = Bx;
    X1[lane] = Byz;
  }
  __syncwarp();
  // transpose x: lane (a,b,c) = element row
  if (on) {
    double res = -T.load[lane];
#pragma unroll
    for (int qx = 0; qx < 3; ++qx) {
      const int k = qx + 3 * i1 + 9 * i2;
      res = fma(T.dph1[qx][i0], X0[k], res);
      res = fma(T.phi1[qx][i0], X1[k], res);
    }
    if (!node_fixed(g, 2 * cx + i0, 2 * cy + i1, 2 * cz + i2)) r[node] -= res;  // r += -res.val()
  }
}

// ---- Jacobian row gather --------------------------------------------------------------------------
constexpr int JR = 64;  // rows per CTA
constexpr int TS = 28;  // padded table row (16-byte aligned rows for vector shared loads)

template <typename T>
__device__ __forceinline__ void seg_store_q2(T* __restrict__ dst, const T* __restrict__ src, int64_t len, bool add) {
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

__device__ __forceinline__ int64_t rowptr2(const Grid& g, int ix, int iy, int iz, int& lx, int& ly, int& lz, int& cx,
                                           int& cy, int& cz) {
  axis_range(ix, g.nn[0], 2, lx, cx);
  axis_range(iy, g.nn[1], 2, ly, cy);
  axis_range(iz, g.nn[2], 2, lz, cz);
  return g.P[2][iz] * g.T[1] * g.T[0] + (int64_t)cz * (g.P[1][iy] * g.T[0] + (int64_t)cy * g.P[0][ix]);
}

// tab: [G_x (27x27) | G_y | G_z | Phi] as [q][j] blocks, i.e. tab[(d*27 + q)*TS + j], d = 3 for Phi.
template <typename JT>
__global__ void __launch_bounds__(JR) k_q2_jac(Grid g, int64_t nrows, int kind, const double s0, const double s1,
                                               const double s2, const JT* __restrict__ tab_g,
                                               const JT* __restrict__ qbuf, JT* __restrict__ J, int ovw) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  JT* tab = reinterpret_cast<JT*>(smem_raw);                   // 108*TS
  JT* sv_base = tab + 108 * TS;                                 // staged segment (JR*125 + pad)
  for (int k = threadIdx.x; k < 108 * TS; k += blockDim.x) tab[k] = tab_g[k];
  const int64_t n0 = (int64_t)blockIdx.x * JR;
  const int64_t n1 = (n0 + JR < nrows) ? n0 + JR : nrows;
  int dummy[6];
  int64_t seg0, seg1;
  {
    int ax, ay, az;
    decompose32(g, n0, ax, ay, az);
    seg0 = rowptr2(g, ax, ay, az, dummy[0], dummy[1], dummy[2], dummy[3], dummy[4], dummy[5]);
    if (n1 >= nrows) seg1 = g.T[0] * g.T[1] * g.T[2];
    else {
      decompose32(g, n1, ax, ay, az);
      seg1 = rowptr2(g, ax, ay, az, dummy[0], dummy[1], dummy[2], dummy[3], dummy[4], dummy[5]);
    }
  }
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
    rp = rowptr2(g, ix, iy, iz, lx, ly, lz, cxn, cyn, czn);
    JT* row = sv + (rp - seg0);
    diag = ((int64_t)(iz - lz) * cyn + (iy - ly)) * cxn + (ix - lx);
    fixed = node_fixed(g, ix, iy, iz);
    if (fixed) {
      if (ovw) row[diag] = JT(1);
    } else {
      int fx, fy, fz, nxc, nyc, nzc;
      axis_cells(ix, g.nn[0], 2, fx, nxc);
      axis_cells(iy, g.nn[1], 2, fy, nyc);
      axis_cells(iz, g.nn[2], 2, fz, nzc);
      for (int ccz = fz; ccz < fz + nzc; ++ccz)
        for (int ccy = fy; ccy < fy + nyc; ++ccy)
          for (int ccx = fx; ccx < fx + nxc; ++ccx) {
            const int l = (ix - 2 * ccx) + 3 * (iy - 2 * ccy) + 9 * (iz - 2 * ccz);
            const int64_t cid = ccx + (int64_t)g.nc[0] * (ccy + (int64_t)g.nc[1] * ccz);
            const JT* qb = qbuf + cid * 108;
            JT acc[27];
#pragma unroll
            for (int j = 0; j < 27; ++j) acc[j] = JT(0);
            // stiffness part: alpha_{d,q} = G_d[q][l] s_d^2 cw_q against G_d[q][:]
            for (int q = 0; q < 27; ++q) {
              const JT cw = qb[q];
#pragma unroll
              for (int d = 0; d < 3; ++d) {
                const JT* trow = tab + (d * 27 + q) * TS;
                const JT a = trow[l] * sq[d] * cw;
#pragma unroll
                for (int j = 0; j < 27; ++j) acc[j] += a * trow[j];
              }
            }
            if (kind != MRG_THERMAL) {
              // advective part: beta_q = sum_d G_d[q][l] ew_{q,d} against Phi[q][:]
              for (int q = 0; q < 27; ++q) {
                const JT b = tab[(0 * 27 + q) * TS + l] * qb[27 + q] + tab[(1 * 27 + q) * TS + l] * qb[54 + q] +
                             tab[(2 * 27 + q) * TS + l] * qb[81 + q];
                const JT* prow = tab + (3 * 27 + q) * TS;
#pragma unroll
                for (int j = 0; j < 27; ++j) acc[j] += b * prow[j];
              }
            }
            // add into the row: column of local node j of this cell
#pragma unroll
            for (int j = 0; j < 27; ++j) {
              const int jx = 2 * ccx + j % 3, jy = 2 * ccy + (j / 3) % 3, jz = 2 * ccz + j / 9;
              row[((int64_t)(jz - lz) * cyn + (jy - ly)) * cxn + (jx - lx)] += acc[j];
            }
          }
    }
  }
  __syncthreads();
  seg_store_q2<JT>(J + seg0, sv, seg1 - seg0, !ovw);
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
struct Q2Data {
  Q2Tabs T;
  double* d_tab64 = nullptr;  // 108*27
  float* d_tab32 = nullptr;
  void* d_qbuf = nullptr;     // ncell*108 (FP64 or FP32, by the last Jacobian request)
  size_t qbuf_bytes = 0;
};

static Q2Data* q2data(mrg_problem* p) { return reinterpret_cast<Q2Data*>(p->q2); }

int mrg_q2_setup(mrg_problem* p) {
  Q2Data* Q = new Q2Data();
  p->q2 = Q;
  const int nq = 27, npe = 27;
  const double* tw = p->qtab_host.data();
  const double* tphi = tw + nq;
  const double* tdphi = tphi + npe * nq;
  for (int q = 0; q < 3; ++q) {
    const double x = p->gx1[q];
    const double l[3] = {0.5 * x * (x - 1.0), 1.0 - x * x, 0.5 * x * (x + 1.0)};
    const double dl[3] = {x - 0.5, -2.0 * x, x + 0.5};
    for (int a = 0; a < 3; ++a) {
      Q->T.phi1[q][a] = l[a];
      Q->T.dph1[q][a] = dl[a];
    }
  }
  double detJ = 1.0;
  for (int d = 0; d < 3; ++d) {
    detJ *= 0.5 * p->h[d];
    Q->T.s[d] = 2.0 / p->h[d];
  }
  for (int q = 0; q < 27; ++q) Q->T.W[q] = tw[q] * detJ;
  for (int l = 0; l < 27; ++l) {
    double s = 0.0;
    for (int q = 0; q < 27; ++q) s += Q->T.W[q] * tphi[l * nq + q];
    Q->T.load[l] = p->source_amp * s;
  }
  // [G_x | G_y | G_z | Phi] as tab[(d*27 + q)*TS + j], rows padded to TS = 28 entries (16-byte rows)
  std::vector<double> tab(108 * TS, 0.0);
  std::vector<float> tab32(108 * TS, 0.0f);
  for (int d = 0; d < 4; ++d)
    for (int q = 0; q < 27; ++q)
      for (int j = 0; j < 27; ++j)
        tab[(d * 27 + q) * TS + j] = (d < 3) ? tdphi[(j * nq + q) * 3 + d] : tphi[j * nq + q];
  for (size_t k = 0; k < tab.size(); ++k) tab32[k] = (float)tab[k];
  MRG_CUDA(cudaMalloc(&Q->d_tab64, tab.size() * sizeof(double)));
  MRG_CUDA(cudaMalloc(&Q->d_tab32, tab.size() * sizeof(float)));
  MRG_CUDA(cudaMemcpy(Q->d_tab64, tab.data(), tab.size() * sizeof(double), cudaMemcpyHostToDevice));
  MRG_CUDA(cudaMemcpy(Q->d_tab32, tab32.data(), tab32.size() * sizeof(float), cudaMemcpyHostToDevice));
  return MRG_OK;
}

void mrg_q2_free(mrg_problem* p) {
  Q2Data* Q = q2data(p);
  if (!Q) return;
  cudaFree(Q->d_tab64);
  cudaFree(Q->d_tab32);
  cudaFree(Q->d_qbuf);
  delete Q;
  p->q2 = nullptr;
}

static int launch_res(mrg_problem* p, const double* u, double* r, void* qbuf, bool fp32q, int mode, cudaStream_t s) {
  Q2Data* Q = q2data(p);
  const Grid& g = p->g;
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
      if (fp32q)
        k_q2_res<float><<<nblk(tot, RW), RW * 32, 0, s>>>(Q->T, g, c, cc[0], cc[1], tot, p->kind, u, p->d_kappa, r,
                                                          (float*)qbuf, mode);
      else
        k_q2_res<double><<<nblk(tot, RW), RW * 32, 0, s>>>(Q->T, g, c, cc[0], cc[1], tot, p->kind, u, p->d_kappa, r,
                                                           (double*)qbuf, mode);
      cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) return mrg_cuda_check(e, "Q2 residual launch");
    }
  } else {
    if (fp32q)
      k_q2_res<float><<<nblk(p->ncell, RW), RW * 32, 0, s>>>(Q->T, g, -1, 1, 1, p->ncell, p->kind, u, p->d_kappa, r,
                                                              (float*)qbuf, mode);
    else
      k_q2_res<double><<<nblk(p->ncell, RW), RW * 32, 0, s>>>(Q->T, g, -1, 1, 1, p->ncell, p->kind, u, p->d_kappa, r,
                                                               (double*)qbuf, mode);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return mrg_cuda_check(e, "Q2 qp-coefficient launch");
  }
  return MRG_OK;
}

int mrg_launch_q2(mrg_problem* p, const double* u, double* r, void* J, uint32_t flags, cudaStream_t s) {
  Q2Data* Q = q2data(p);
  const bool doJ = flags & MRG_ASM_JAC, doR = flags & MRG_ASM_RES, ovw = flags & MRG_ASM_OVERWRITE;
  const bool fp32 = flags & MRG_ASM_J_FP32;
  void* qbuf = nullptr;
  if (doJ) {
    const size_t need = (size_t)p->ncell * 108 * (fp32 ? sizeof(float) : sizeof(double));
    if (Q->qbuf_bytes < need) {
      cudaFree(Q->d_qbuf);
      Q->d_qbuf = nullptr;
      Q->qbuf_bytes = 0;
      MRG_CUDA(cudaMalloc(&Q->d_qbuf, need));
      Q->qbuf_bytes = need;
    }
    qbuf = Q->d_qbuf;
  }
  if (doR && ovw) MRG_CUDA(cudaMemsetAsync(r, 0, p->ndof * sizeof(double), s));
  int st = launch_res(p, u, doR ? r : nullptr, qbuf, fp32, (doR ? 1 : 0) | (doJ ? 2 : 0), s);
  if (st) return st;
  if (doJ) {
    const unsigned grid = nblk(p->ndof, JR);
    if (fp32) {
      const int smem = (108 * TS + JR * 125 + 4) * (int)sizeof(float);
      auto kern = k_q2_jac<float>;
      if (smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
      kern<<<grid, JR, smem, s>>>(p->g, p->ndof, p->kind, Q->T.s[0], Q->T.s[1], Q->T.s[2], Q->d_tab32,
                                  (const float*)qbuf, (float*)J, ovw ? 1 : 0);
    } else {
      const int smem = (108 * TS + JR * 125 + 2) * (int)sizeof(double);
      auto kern = k_q2_jac<double>;
      if (smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
      kern<<<grid, JR, smem, s>>>(p->g, p->ndof, p->kind, Q->T.s[0], Q->T.s[1], Q->T.s[2], Q->d_tab64,
                                  (const double*)qbuf, (double*)J, ovw ? 1 : 0);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return mrg_cuda_check(e, "Q2 Jacobian launch");
  }
  return MRG_OK;
}
