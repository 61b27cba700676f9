// Geometric multigrid preconditioner for Q1 problems on the structured graph, and the CG that uses it.
//
// The reference's linear solver is Belos with an algebraic multigrid preconditioner (MueLu) or its own
// Jacobi PCG (src/managers/solver/solverManager_solvers.hpp:812-901; Belos/MueLu options in
// src/interfaces/linear_algebra/linearAlgebraInterface_solvers.hpp:15-160).  On the structured box the
// multigrid hierarchy is known in closed form, so it is built geometrically and Galerkin-exactly:
//
//   * levels: vertex coarsening by 2 along the axes that still have >= 3 cells and whose cells are at
//     most twice as long as the shortest (semi-coarsening on stretched grids); a fine node with an
//     even index is a coarse node, and when the cell count is odd the last fine node is kept as a coarse
//     node too (the last coarse cell is one fine cell wide).  Every level has the canonical 27-point
//     (9-point in 2-D) layout of a p = 1 grid, so the level operators use the same CSR layout, row
//     formulas and staged SpMV as the fine one.
//   * interpolation P: tensor product of 1-D linear interpolation (weights 1 or 1/2); rows of fixed
//     (strong Dirichlet) fine nodes and columns of fixed coarse nodes are zero, so the hierarchy acts on
//     the free unknowns only, where J is symmetric.
//   * coarse operators A_c = P^T A_f P (restricted to free nodes; fixed coarse rows are identity rows),
//     computed as one 1-D Galerkin sweep per coarsened axis (the masked P is a tensor product).
//   * smoother: Chebyshev polynomial of degree 2 in D^{-1} A on [0.25 L, L], L the Gershgorin bound
//     max_i sum_j |a_ij| / a_ii of the level (computed on the device; no host synchronisation);
//   * coarsest level (at most 27 unknowns): dense inverse, Gauss-Jordan on the device.
//   * V(2,2) cycle, symmetric, so it preconditions CG.
//
// The CG keeps q = A p by recurrence (p <- z + beta p, q <- A z + beta q) so the SpMV reads z and no
// separate direction update is needed; dot products reduce deterministically (per-block partials,
// last block sums in index order).  The hierarchy and the CG run in the precision of the Jacobian
// (FP64, or FP32 for the inner solve of the mixed path).  Chunks of iterations are captured as CUDA
// graphs; the host reads the done flag once per chunk.
#include <algorithm>
#include <cmath>
#include <mutex>
#include <string>
#include <vector>

#include "mrg_device.cuh"
#include "mrg_internal.h"

namespace {

using namespace mrgdev;

constexpr int NT = WST;            // threads per CTA
constexpr int NU = 2;              // Chebyshev degree (pre and post smoothing)
constexpr double CHEB_LO = 0.25;   // lower end of the smoothed interval, fraction of the bound
constexpr int GCHUNK = 2;          // Krylov iterations per captured graph (2: fewer nodes to instantiate and fewer iterations past convergence than 4; measured on small and large problems)
constexpr int MAXC = 32;           // largest coarsest level solved densely
constexpr int MAXLEV = 16;
constexpr int64_t RAP_WARP_ROWS = 24576;  // Galerkin sweeps with fewer output rows: one warp per row

// ---- 1-D transfer along one axis ----------------------------------------------------------------
// Parents of fine node i (fine nodes 0..nnf-1, coarse nodes 0..nnc-1) with interpolation weights.
__host__ __device__ inline int axis_parents(int i, int nnf, int nnc, int coarsen, int* pc, float* pw) {
  if (!coarsen) { pc[0] = i; pw[0] = 1.0f; return 1; }
  if ((i & 1) == 0) { pc[0] = i >> 1; pw[0] = 1.0f; return 1; }
  if (i == nnf - 1) { pc[0] = nnc - 1; pw[0] = 1.0f; return 1; }  // odd last node is kept
  pc[0] = (i - 1) >> 1; pw[0] = 0.5f;
  pc[1] = (i + 1) >> 1; pw[1] = 0.5f;
  return 2;
}

// Children of coarse node c with their weights (the transpose of axis_parents).
__device__ inline int axis_children(int c, int nnf, int nnc, int coarsen, int* ci, float* cw) {
  if (!coarsen) { ci[0] = c; cw[0] = 1.0f; return 1; }
  int n = 0;
  for (int i = 2 * c - 1; i <= 2 * c + 1; ++i) {
    if (i < 0 || i >= nnf) continue;
    int pc[2];
    float pw[2];
    const int np = axis_parents(i, nnf, nnc, 1, pc, pw);
    for (int k = 0; k < np; ++k)
      if (pc[k] == c) { ci[n] = i; cw[n] = pw[k]; ++n; }
  }
  return n;
}

struct Xfer {
  int co[3];  // axis coarsened from the finer level
};

template <typename T>
struct LevDev {
  Grid g;
  int64_t n;
  const T* A;
  T* minv;
  T *xa, *xb, *d, *b, *r;
};

struct GScal {
  double rho, pq, alpha, beta, r0, rnorm, tol;
  double omega, rv;  // BiCGStab
  int iter, maxiter, done, status;
  unsigned int counter;
  int err;
};

template <int P, typename T>
__device__ __forceinline__ auto row_prod(const Grid& g, const RowInfo& R, const T* vals, const T* x) {
  if constexpr (sizeof(T) == 4) return row_apply_f<P>(g, R, vals, x);
  else return row_apply<P, double, double>(g, R, vals, x);
}

// f(n, R, vals) for every row: Q1 rows through the per-warp staged loop, Q2 rows (125-point) read directly.
template <int P, typename T, typename F>
__device__ __forceinline__ bool level_rows(const Grid& g, int64_t n, const T* __restrict__ A, unsigned char* smem_raw,
                                           uint64_t* mbar, F&& f) {
  if constexpr (P == 1) {
    return warp_staged_rows<T>(g, n, A, smem_raw, mbar, f);
  } else {
    for (int64_t i = (int64_t)blockIdx.x * NT + threadIdx.x; i < n; i += (int64_t)gridDim.x * NT) {
      int ix, iy, iz;
      decompose(g, i, ix, iy, iz);
      const RowInfo R = row_info<P>(g, ix, iy, iz);
      f(i, R, A + R.rp);
    }
    return true;
  }
}

// Per-axis polynomial order of a grid's coupling ranges (an intermediate grid of the Q2 -> Q1 Galerkin
// sweeps couples +-1 along the swept axes and +-2 along the others).
struct P3 {
  int p[3];
};

__device__ __forceinline__ RowInfo row_info_p3(const Grid& g, const P3& pp, int ix, int iy, int iz) {
  RowInfo R;
  axis_range(ix, g.nn[0], pp.p[0], R.lx, R.cx);
  axis_range(iy, g.nn[1], pp.p[1], R.ly, R.cy);
  if (g.dim == 3) axis_range(iz, g.nn[2], pp.p[2], R.lz, R.cz); else { R.lz = 0; R.cz = 1; }
  R.rp = g.P[2][iz] * g.T[1] * g.T[0] + (int64_t)R.cz * (g.P[1][iy] * g.T[0] + (int64_t)R.cy * g.P[0][ix]);
  return R;
}

__device__ __forceinline__ bool is_done(const GScal* S) { return ((volatile const GScal*)S)->done != 0; }

// ---- setup kernels ------------------------------------------------------------------------------
// One axis of the Galerkin product, one thread per row of the output grid gc (gc = gf coarsened along
// `axis` only).  The free nodes form a Cartesian product (Dirichlet faces are axis-aligned), so the
// masked interpolation is a tensor product and P^T A P is three such sweeps (x, then y, then z),
// each keeping the 27-point layout on an intermediate grid: ~160 multiply-adds per output row instead
// of ~5,800 for the direct triple product.
//
// Rows away from the faces take a fast path: every fine column and coarse parent there is free and has the
// standard weights (1/2, 1, 1/2), and every row has its full width, so the loops unroll with
// compile-time accumulator positions (registers instead of a local-memory array).  Row widths along an
// axis: 3 on a p = 1 axis; on a p = 2 axis 5 at even (vertex) nodes and 3 at odd (mid-edge) nodes.  The
// swept axis A goes from p = QA ? 2 : 1 to p = 1; the other two axes keep their widths WB, WC (B < C).
// The fast path adds the same products in the same order as the general loop (children ascending, then
// the row's entries in storage order, then the lower and upper parent), so the result is bit-identical.
template <typename T, int A, bool QA, int WB, int WC, int DC>
__device__ __forceinline__ void rap_child(const Grid& gf, const P3& pf, const int I[3], const T* __restrict__ Af,
                                          T* acc) {
  constexpr int B = (A == 0) ? 1 : 0;  // the lower of the two other axes (C is the remaining one)
  constexpr int WA = (QA && DC == 0) ? 5 : 3;  // child 2I is a vertex node, 2I +- 1 mid-edge nodes
  constexpr int W0 = (A == 0) ? WA : (B == 0 ? WB : WC);
  constexpr int W1 = (A == 1) ? WA : (B == 1 ? WB : WC);
  constexpr int W2 = (A == 2) ? WA : (B == 2 ? WB : WC);
  constexpr int O0 = (A == 0) ? 3 : W0, O1 = (A == 1) ? 3 : W1, O2 = (A == 2) ? 3 : W2;  // output widths
  int f[3] = {I[0], I[1], I[2]};
  f[A] = 2 * I[A] + DC;
  const T* vals = Af + row_info_p3(gf, pf, f[0], f[1], f[2]).rp;
  const T wc = (DC == 0) ? T(1) : T(0.5);
#pragma unroll
  for (int ez = -(W2 - 1) / 2; ez <= (W2 - 1) / 2; ++ez)
#pragma unroll
    for (int ey = -(W1 - 1) / 2; ey <= (W1 - 1) / 2; ++ey)
#pragma unroll
      for (int ex = -(W0 - 1) / 2; ex <= (W0 - 1) / 2; ++ex) {
        const T a = vals[((ez + (W2 - 1) / 2) * W1 + (ey + (W1 - 1) / 2)) * W0 + (ex + (W0 - 1) / 2)] * wc;
        const int e[3] = {ex, ey, ez};
        const int sft = DC + e[A];  // fine column along A relative to 2I: -2..2
        int o[3] = {ex, ey, ez};
        if ((sft & 1) == 0) {
          o[A] = sft / 2;
          T& t = acc[((o[2] + (O2 - 1) / 2) * O1 + (o[1] + (O1 - 1) / 2)) * O0 + (o[0] + (O0 - 1) / 2)];
          t += a * T(1);
        } else {
          o[A] = (sft - 1) / 2;
          T& t0 = acc[((o[2] + (O2 - 1) / 2) * O1 + (o[1] + (O1 - 1) / 2)) * O0 + (o[0] + (O0 - 1) / 2)];
          t0 += a * T(0.5);
          o[A] = (sft + 1) / 2;
          T& t1 = acc[((o[2] + (O2 - 1) / 2) * O1 + (o[1] + (O1 - 1) / 2)) * O0 + (o[0] + (O0 - 1) / 2)];
          t1 += a * T(0.5);
        }
      }
}

template <typename T, int A, bool QA, int WB, int WC>
__device__ __forceinline__ void rap_interior(const Grid& gf, const P3& pf, const int I[3], const T* __restrict__ Af,
                                             T* __restrict__ out) {
  constexpr int LEN = 3 * WB * WC;
  T acc[LEN];
#pragma unroll
  for (int k = 0; k < LEN; ++k) acc[k] = T(0);
  rap_child<T, A, QA, WB, WC, -1>(gf, pf, I, Af, acc);
  rap_child<T, A, QA, WB, WC, 0>(gf, pf, I, Af, acc);
  rap_child<T, A, QA, WB, WC, 1>(gf, pf, I, Af, acc);
#pragma unroll
  for (int k = 0; k < LEN; ++k) out[k] = acc[k];
}

template <typename T>
__global__ void __launch_bounds__(NT) k_rap_axis(Grid gf, P3 pf, Grid gc, P3 pc, int axis, const T* __restrict__ Af,
                                                 T* __restrict__ Ac, int* __restrict__ err) {
  const int64_t n = (int64_t)blockIdx.x * NT + threadIdx.x;
  const int64_t nrows = (int64_t)gc.nn[0] * gc.nn[1] * gc.nn[2];
  if (n >= nrows) return;
  int I[3];
  decompose(gc, n, I[0], I[1], I[2]);
  const RowInfo Rc = row_info_p3(gc, pc, I[0], I[1], I[2]);
  const int lenc = Rc.cx * Rc.cy * Rc.cz;
  T* out = Ac + Rc.rp;
  if (node_fixed(gc, I[0], I[1], I[2])) {
    const int dg = (int)(diag_pos(Rc, I[0], I[1], I[2]) - Rc.rp);
    for (int e = 0; e < lenc; ++e) out[e] = (e == dg) ? T(1) : T(0);
    return;
  }
  // fast path: 3-D, order 1 throughout (the h-levels).  The same template covers order-2 rows, but
  // instantiating those variants in this kernel raised it from 64 to 128 (FP32) / 254 (FP64) registers
  // and slowed every sweep; on the Q2 -> Q1 sweeps it was no faster than the loop below (1.66 vs 1.40 ms
  // for the first sweep of a 64^3 Q2 grid).
  if (gf.dim == 3 && pf.p[0] == 1 && pf.p[1] == 1 && pf.p[2] == 1 && pc.p[0] == 1 && pc.p[1] == 1 && pc.p[2] == 1) {
    bool inner = I[axis] >= 2 && 2 * I[axis] + 2 <= gf.nn[axis] - 2;
#pragma unroll
    for (int b = 0; b < 3; ++b)
      if (b != axis) inner = inner && I[b] >= 2 && I[b] <= gf.nn[b] - 3;
    if (inner) {
      if (axis == 0) rap_interior<T, 0, false, 3, 3>(gf, pf, I, Af, out);
      else if (axis == 1) rap_interior<T, 1, false, 3, 3>(gf, pf, I, Af, out);
      else rap_interior<T, 2, false, 3, 3>(gf, pf, I, Af, out);
      return;
    }
  }
  constexpr int MAXROW = 75;  // 3 x 5 x 5: the widest output row (one axis swept from a Q2 grid)
  if (lenc > MAXROW) { atomicExch(err, 1); return; }
  T acc[MAXROW];
  for (int e = 0; e < lenc; ++e) acc[e] = T(0);
  int ci[3];
  float cw[3];
  const int nci = axis_children(I[axis], gf.nn[axis], gc.nn[axis], 1, ci, cw);
  for (int c = 0; c < nci; ++c) {
    int f[3] = {I[0], I[1], I[2]};
    f[axis] = ci[c];
    if (node_fixed(gf, f[0], f[1], f[2])) continue;
    const RowInfo Rf = row_info_p3(gf, pf, f[0], f[1], f[2]);
    const T* vals = Af + Rf.rp;
    int e = 0;
    for (int jz = Rf.lz; jz < Rf.lz + Rf.cz; ++jz)
      for (int jy = Rf.ly; jy < Rf.ly + Rf.cy; ++jy)
        for (int jx = Rf.lx; jx < Rf.lx + Rf.cx; ++jx, ++e) {
          if (node_fixed(gf, jx, jy, jz)) continue;
          const T a = vals[e] * (T)cw[c];
          int jj[3] = {jx, jy, jz};
          int pc[2];
          float pw[2];
          const int np = axis_parents(jj[axis], gf.nn[axis], gc.nn[axis], 1, pc, pw);
          for (int k = 0; k < np; ++k) {
            jj[axis] = pc[k];
            if (node_fixed(gc, jj[0], jj[1], jj[2])) continue;
            const int pos = ((jj[2] - Rc.lz) * Rc.cy + (jj[1] - Rc.ly)) * Rc.cx + (jj[0] - Rc.lx);
            if (pos < 0 || pos >= lenc) { atomicExch(err, 1); continue; }
            acc[pos] += a * (T)pw[k];
          }
        }
  }
  for (int e = 0; e < lenc; ++e) out[e] = acc[e];
}

// The same sweep with one warp per output row and the lanes over the row's entries: an entry sums, over
// the children c of the row and the fine columns j whose parent is the entry's column, a_c(j) w_c w_j --
// the row loop above adds exactly these products, in the same order (children ascending, then fine
// columns ascending), so the result is bit-identical.  Used on small levels (below ~25k output rows),
// where one thread's serial walk over a row set the duration of the thread-per-row loop (42 µs for a
// 128-row level against 8 µs here); above that the thread-per-row fast path is faster.
// Children of coarse node c along a coarsened axis in three fixed slots (fine 2c-1, 2c, 2c+1): the
// same set, order and weights as axis_children, without its run-time slot index.
__device__ __forceinline__ void children3(int c, int nnf, int nnc, int ci[3], float cw[3], bool ok[3]) {
  ci[0] = 2 * c - 1;
  ci[1] = 2 * c;
  ci[2] = 2 * c + 1;
  // 2c-1 (odd): parents (i-1)/2, (i+1)/2 = c with weight 1/2, or the kept odd last node (parent nnc-1, 1)
  ok[0] = c >= 1 && ci[0] <= nnf - 1 && (ci[0] != nnf - 1 || c == nnc - 1);
  cw[0] = (ci[0] == nnf - 1) ? 1.0f : 0.5f;
  ok[1] = ci[1] <= nnf - 1;  // even: parent c, weight 1
  cw[1] = 1.0f;
  ok[2] = ci[2] <= nnf - 2;  // odd, not the last node: parents c and c+1, weight 1/2
  cw[2] = 0.5f;
}

template <typename T, int A>
__global__ void __launch_bounds__(NT) k_rap_axis_w(Grid gf, P3 pf, Grid gc, P3 pc, const T* __restrict__ Af,
                                                   T* __restrict__ Ac) {
  const int lane = threadIdx.x & 31;
  const int64_t n = ((int64_t)blockIdx.x * NT + threadIdx.x) >> 5;
  const int64_t nrows = (int64_t)gc.nn[0] * gc.nn[1] * gc.nn[2];
  if (n >= nrows) return;  // uniform over the warp
  int I[3];
  decompose(gc, n, I[0], I[1], I[2]);
  const RowInfo Rc = row_info_p3(gc, pc, I[0], I[1], I[2]);
  const int lenc = Rc.cx * Rc.cy * Rc.cz;
  T* out = Ac + Rc.rp;
  if (node_fixed(gc, I[0], I[1], I[2])) {
    const int dg = (int)(diag_pos(Rc, I[0], I[1], I[2]) - Rc.rp);
    for (int e = lane; e < lenc; e += 32) out[e] = (e == dg) ? T(1) : T(0);
    return;
  }
  const int nnf = gf.nn[A], nnc = gc.nn[A];
  int ci[3];
  float cw[3];
  bool cok[3];
  children3(I[A], nnf, nnc, ci, cw, cok);
  RowInfo Rf[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    int f[3] = {I[0], I[1], I[2]};
    f[A] = ci[c];
    cok[c] = cok[c] && !node_fixed(gf, f[0], f[1], f[2]);
    if (cok[c]) Rf[c] = row_info_p3(gf, pf, f[0], f[1], f[2]);
  }
  for (int e = lane; e < lenc; e += 32) {
    int o[3];
    o[0] = Rc.lx + e % Rc.cx;
    o[1] = Rc.ly + (e / Rc.cx) % Rc.cy;
    o[2] = Rc.lz + e / (Rc.cx * Rc.cy);
    T acc = T(0);
    if (!node_fixed(gc, o[0], o[1], o[2])) {
      int cj[3];
      float wj[3];
      bool jok[3];
      children3(o[A], nnf, nnc, cj, wj, jok);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        if (!cok[c]) continue;
        const RowInfo& R = Rf[c];
        const T* vals = Af + R.rp;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          if (!jok[k]) continue;
          int j[3] = {o[0], o[1], o[2]};
          j[A] = cj[k];
          if (j[0] < R.lx || j[0] >= R.lx + R.cx || j[1] < R.ly || j[1] >= R.ly + R.cy || j[2] < R.lz ||
              j[2] >= R.lz + R.cz)
            continue;
          if (node_fixed(gf, j[0], j[1], j[2])) continue;
          const T a = vals[((j[2] - R.lz) * R.cy + (j[1] - R.ly)) * R.cx + (j[0] - R.lx)] * (T)cw[c];
          acc += a * (T)wj[k];
        }
      }
    }
    out[e] = acc;
  }
}

// minv = 1 / diag; Gershgorin bound max_i sum_j |a_ij| / |a_ii| into lmax (as float bits, atomicMax)
template <int P, typename T>
__global__ void __launch_bounds__(NT) k_diag(Grid g, const T* __restrict__ A, T* __restrict__ minv,
                                             unsigned int* __restrict__ lmax_bits) {
  const int64_t n = (int64_t)blockIdx.x * NT + threadIdx.x;
  const int64_t nrows = (int64_t)g.nn[0] * g.nn[1] * g.nn[2];
  float v = 0.0f;
  if (n < nrows) {
    int ix, iy, iz;
    decompose(g, n, ix, iy, iz);
    const RowInfo R = row_info<P>(g, ix, iy, iz);
    const T* vals = A + R.rp;
    const int len = R.cx * R.cy * R.cz;
    const T dgv = vals[diag_pos(R, ix, iy, iz) - R.rp];
    T s = T(0);  // a bound: the level's precision is enough
    for (int e = 0; e < len; ++e) s += fabs(vals[e]);
    minv[n] = T(1) / dgv;
    v = (float)(s / fabs(dgv));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_down_sync(0xffffffffu, v, o));
  if ((threadIdx.x & 31) == 0 && v > 0.0f) atomicMax(lmax_bits, __float_as_uint(v));
}

// Dense inverse of the coarsest operator (n <= MAXC), Gauss-Jordan with partial pivoting, one CTA, in
// the hierarchy's precision (FP32 for the inner solve's hierarchy: FP64 arithmetic there cost the FP64
// pipe's latency on every step for a preconditioner that is FP32 anyway).  The pivot is the first row
// of largest magnitude, found by warp 0 with shuffles.
template <typename T>
__global__ void __launch_bounds__(NT) k_coarse_inv(Grid g, const T* __restrict__ A, T* __restrict__ inv,
                                                   int* __restrict__ err) {
  __shared__ T M[MAXC][2 * MAXC];
  __shared__ int piv;
  const int n = g.nn[0] * g.nn[1] * g.nn[2];
  for (int k = threadIdx.x; k < MAXC * 2 * MAXC; k += NT) (&M[0][0])[k] = T(0);
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += NT) {
    int ix, iy, iz;
    decompose(g, i, ix, iy, iz);
    const RowInfo R = row_info<1>(g, ix, iy, iz);
    int e = 0;
    for (int jz = R.lz; jz < R.lz + R.cz; ++jz)
      for (int jy = R.ly; jy < R.ly + R.cy; ++jy)
        for (int jx = R.lx; jx < R.lx + R.cx; ++jx, ++e)
          M[i][jx + g.nn[0] * (jy + g.nn[1] * jz)] = A[R.rp + e];
    M[i][n + i] = T(1);
  }
  __syncthreads();
  for (int c = 0; c < n; ++c) {
    if (threadIdx.x < 32) {
      const int r = threadIdx.x;
      T v = (r >= c && r < n) ? fabs(M[r][c]) : T(-1);
      int bi = r;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const T ov = __shfl_down_sync(0xffffffffu, v, o);
        const int oi = __shfl_down_sync(0xffffffffu, bi, o);
        if (ov > v || (ov == v && oi < bi)) {
          v = ov;
          bi = oi;
        }
      }
      if (threadIdx.x == 0) {
        piv = bi;
        if (!(v > T(0))) atomicExch(err, 2);
      }
    }
    __syncthreads();
    const int pr = piv;
    if (pr != c)
      for (int k = threadIdx.x; k < 2 * n; k += NT) {
        const T t = M[c][k];
        M[c][k] = M[pr][k];
        M[pr][k] = t;
      }
    __syncthreads();
    const T inv_p = T(1) / M[c][c];
    __syncthreads();
    for (int k = threadIdx.x; k < 2 * n; k += NT) M[c][k] *= inv_p;
    __syncthreads();
    for (int idx = threadIdx.x; idx < n * 2 * n; idx += NT) {
      const int r = idx / (2 * n), k = idx % (2 * n);
      if (r != c && k != c) M[r][k] -= M[r][c] * M[c][k];
    }
    __syncthreads();
    for (int r = threadIdx.x; r < n; r += NT)
      if (r != c) M[r][c] = T(0);
    __syncthreads();
  }
  for (int idx = threadIdx.x; idx < n * n; idx += NT) inv[idx] = M[idx / n][n + idx % n];
}

// ---- cycle kernels --------------------------------------------------------------------------------
// Chebyshev step `k` (0..NU-1): d = rho_k rho_{k-1} d + (2 rho_k / delta) D^{-1}(b - A x)  (k = 0:
// d = D^{-1}(b - A x) / theta); xout = x + d.  zero_x: x = 0 (no SpMV).
// Chebyshev coefficients of every level and step (one thread per level, at setup): coef[(l NU + k) 3 + m]
// = {1/theta, rho_k rho_{k-1}, 2 rho_k / delta} on [CHEB_LO L, L], L the level's Gershgorin bound.
__global__ void k_cheb_coef(const unsigned int* __restrict__ lmax_bits, int nlev, double* __restrict__ coef) {
  const int l = threadIdx.x;
  if (l >= nlev) return;
  const double hi = (double)__uint_as_float(lmax_bits[l]), lo = CHEB_LO * hi;
  const double theta = 0.5 * (hi + lo), delta = 0.5 * (hi - lo), sigma = theta / delta;
  double rho_prev = 1.0 / sigma, rho = rho_prev;
  for (int k = 0; k < NU; ++k) {
    if (k > 0) {
      const double rn = 1.0 / (2.0 * sigma - rho);
      rho_prev = rho;
      rho = rn;
    }
    double* c = coef + ((size_t)l * NU + k) * 3;
    c[0] = 1.0 / theta;
    c[1] = rho * rho_prev;
    c[2] = 2.0 * rho / delta;
  }
}

// Rounded operations that the compiler does not contract: the row updates shared by the per-step kernels
// and k_vcycle_tail must round the same way in both.
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }

// Chebyshev-Jacobi step k for row n given ax = (A x_in)_n: d = c_first z (k = 0) or c_old d + c_new z with
// z = D^{-1} (b - ax); x_out = x_in + d (x_in = 0 when zero_x).  Shared by k_cheb and k_vcycle_tail.
template <typename T>
__device__ __forceinline__ void cheb_row(const LevDev<T>& L, int64_t n, T ax, const T* __restrict__ xin,
                                         T* __restrict__ xout, int k, int zero_x, T c_first, T c_old, T c_new) {
  const T z = mul_rn(L.minv[n], sub_rn(L.b[n], ax));
  const T d = (k == 0) ? mul_rn(c_first, z) : fma(c_old, L.d[n], mul_rn(c_new, z));
  L.d[n] = d;
  xout[n] = add_rn(zero_x ? T(0) : xin[n], d);
}

// r = b - A x, row n
template <typename T>
__device__ __forceinline__ void resid_row(const LevDev<T>& L, int64_t n, T ax) {
  L.r[n] = sub_rn(L.b[n], ax);
}

template <int P, typename T>
__global__ void __launch_bounds__(NT) k_cheb(LevDev<T> L, const T* __restrict__ xin, T* __restrict__ xout, int k,
                                             int zero_x, const double* __restrict__ coef,
                                             const GScal* __restrict__ S, int* __restrict__ err) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t mbar[2 * (NT / 32)];
  if (is_done(S)) return;
  const T c_first = (T)coef[3 * k], c_old = (T)coef[3 * k + 1], c_new = (T)coef[3 * k + 2];
  auto fin = [&](int64_t n, T ax) { cheb_row<T>(L, n, ax, xin, xout, k, zero_x, c_first, c_old, c_new); };
  if (zero_x) {
    for (int64_t n = (int64_t)blockIdx.x * NT + threadIdx.x; n < L.n; n += (int64_t)gridDim.x * NT) fin(n, T(0));
    return;
  }
  const bool ok = level_rows<P, T>(L.g, L.n, L.A, smem_raw, mbar, [&](int64_t n, const RowInfo& R, const T* vals) {
    fin(n, (T)row_prod<P, T>(L.g, R, vals, xin));
  });
  if (!ok) atomicExch(err, 3);
}

// r = b - A x
template <int P, typename T>
__global__ void __launch_bounds__(NT) k_resid(LevDev<T> L, const T* __restrict__ x, const GScal* __restrict__ S,
                                              int* __restrict__ err) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t mbar[2 * (NT / 32)];
  if (is_done(S)) return;
  const bool ok = level_rows<P, T>(L.g, L.n, L.A, smem_raw, mbar, [&](int64_t n, const RowInfo& R, const T* vals) {
    resid_row<T>(L, n, (T)row_prod<P, T>(L.g, R, vals, x));
  });
  if (!ok) atomicExch(err, 3);
}

// b_c = P^T r_f
// Per-axis transfer slots with validity flags (registers, no run-time indexed arrays): children of a
// coarse node (fine 2c-1, 2c, 2c+1 on a coarsened axis, the node itself otherwise) and parents of a
// fine node (1 or 2).  Same sets, order and weights as axis_children / axis_parents.
__device__ __forceinline__ void child_slots(int c, int nnf, int nnc, int co, bool in_dim, int ci[3], float cw[3],
                                            bool ok[3]) {
  if (!in_dim) {
    ci[0] = ci[1] = ci[2] = 0;
    cw[0] = cw[1] = cw[2] = 1.0f;
    ok[0] = ok[2] = false;
    ok[1] = true;
    return;
  }
  if (!co) {
    ci[0] = ci[1] = ci[2] = c;
    cw[0] = cw[1] = cw[2] = 1.0f;
    ok[0] = ok[2] = false;
    ok[1] = true;
    return;
  }
  children3(c, nnf, nnc, ci, cw, ok);
}

__device__ __forceinline__ void parent_slots(int i, int nnf, int nnc, int co, bool in_dim, int pc[2], float pw[2],
                                             bool ok[2]) {
  if (!in_dim) {
    pc[0] = pc[1] = 0;
    pw[0] = pw[1] = 1.0f;
    ok[0] = true;
    ok[1] = false;
    return;
  }
  const int np = axis_parents(i, nnf, nnc, co, pc, pw);
  ok[0] = true;
  ok[1] = np == 2;
  if (np < 2) {
    pc[1] = pc[0];
    pw[1] = 0.0f;
  }
}

// b_c = P^T r_f, coarse row n (shared by k_restrict and k_vcycle_tail)
template <typename T>
__device__ __forceinline__ void restrict_row(const Grid& gf, const Grid& gc, const Xfer& X, const T* __restrict__ rf,
                                             T* __restrict__ bc, int64_t n) {
  int I[3];
  decompose(gc, n, I[0], I[1], I[2]);
  if (node_fixed(gc, I[0], I[1], I[2])) { bc[n] = T(0); return; }
  int c0[3], c1[3], c2[3];
  float w0[3], w1[3], w2[3];
  bool k0[3], k1[3], k2[3];
  child_slots(I[0], gf.nn[0], gc.nn[0], X.co[0], gf.dim > 0, c0, w0, k0);
  child_slots(I[1], gf.nn[1], gc.nn[1], X.co[1], gf.dim > 1, c1, w1, k1);
  child_slots(I[2], gf.nn[2], gc.nn[2], X.co[2], gf.dim > 2, c2, w2, k2);
  T s = T(0);
#pragma unroll
  for (int a2 = 0; a2 < 3; ++a2)
#pragma unroll
    for (int a1 = 0; a1 < 3; ++a1)
#pragma unroll
      for (int a0 = 0; a0 < 3; ++a0) {
        if (!(k2[a2] && k1[a1] && k0[a0])) continue;
        const int ix = c0[a0], iy = c1[a1], iz = c2[a2];
        if (node_fixed(gf, ix, iy, iz)) continue;
        s = fma((T)(w0[a0] * w1[a1] * w2[a2]), rf[ix + (int64_t)gf.nn[0] * (iy + (int64_t)gf.nn[1] * iz)], s);
      }
  bc[n] = s;
}

template <typename T>
__global__ void __launch_bounds__(NT) k_restrict(Grid gf, Grid gc, Xfer X, const T* __restrict__ rf, T* __restrict__ bc,
                                                 const GScal* __restrict__ S) {
  if (is_done(S)) return;
  const int64_t nc = (int64_t)gc.nn[0] * gc.nn[1] * gc.nn[2];
  for (int64_t n = (int64_t)blockIdx.x * NT + threadIdx.x; n < nc; n += (int64_t)gridDim.x * NT)
    restrict_row<T>(gf, gc, X, rf, bc, n);
}

// x_f += P x_c, fine row n (shared by k_prolong and k_vcycle_tail)
template <typename T>
__device__ __forceinline__ void prolong_row(const Grid& gf, const Grid& gc, const Xfer& X, const T* __restrict__ xc,
                                            T* __restrict__ xf, int64_t n) {
  int i[3];
  decompose(gf, n, i[0], i[1], i[2]);
  if (node_fixed(gf, i[0], i[1], i[2])) return;
  int p0[2], p1[2], p2[2];
  float w0[2], w1[2], w2[2];
  bool k0[2], k1[2], k2[2];
  parent_slots(i[0], gf.nn[0], gc.nn[0], X.co[0], gf.dim > 0, p0, w0, k0);
  parent_slots(i[1], gf.nn[1], gc.nn[1], X.co[1], gf.dim > 1, p1, w1, k1);
  parent_slots(i[2], gf.nn[2], gc.nn[2], X.co[2], gf.dim > 2, p2, w2, k2);
  T s = T(0);
#pragma unroll
  for (int b2 = 0; b2 < 2; ++b2)
#pragma unroll
    for (int b1 = 0; b1 < 2; ++b1)
#pragma unroll
      for (int b0 = 0; b0 < 2; ++b0) {
        if (!(k2[b2] && k1[b1] && k0[b0])) continue;
        if (node_fixed(gc, p0[b0], p1[b1], p2[b2])) continue;
        s = fma((T)(w0[b0] * w1[b1] * w2[b2]), xc[p0[b0] + (int64_t)gc.nn[0] * (p1[b1] + (int64_t)gc.nn[1] * p2[b2])], s);
      }
  xf[n] = add_rn(xf[n], s);
}

template <typename T>
__global__ void __launch_bounds__(NT) k_prolong(Grid gf, Grid gc, Xfer X, const T* __restrict__ xc, T* __restrict__ xf,
                                                const GScal* __restrict__ S) {
  if (is_done(S)) return;
  const int64_t nf = (int64_t)gf.nn[0] * gf.nn[1] * gf.nn[2];
  for (int64_t n = (int64_t)blockIdx.x * NT + threadIdx.x; n < nf; n += (int64_t)gridDim.x * NT)
    prolong_row<T>(gf, gc, X, xc, xf, n);
}

// x = inv b on the coarsest level, row i (shared by k_coarse_apply and k_vcycle_tail)
template <typename T>
__device__ __forceinline__ void coarse_row(int n, const T* __restrict__ inv, const T* __restrict__ b, T* __restrict__ x,
                                           int i) {
  T s = T(0);
  for (int j = 0; j < n; ++j) s = fma(inv[i * n + j], b[j], s);
  x[i] = s;
}

template <typename T>
__global__ void __launch_bounds__(NT) k_coarse_apply(int n, const T* __restrict__ inv, const T* __restrict__ b,
                                                     T* __restrict__ x, const GScal* __restrict__ S) {
  if (is_done(S)) return;
  for (int i = threadIdx.x; i < n; i += NT) coarse_row<T>(n, inv, b, x, i);
}

// ---- the coarse end of the V-cycle in one CTA ---------------------------------------------------------
// The smallest levels take a microsecond of work per step but a launch each (seven per level and cycle).
// k_vcycle_tail runs the whole cycle below the first such level -- pre-smoothing, residual and restriction
// down to the coarsest level, the dense coarsest solve, prolongation and post-smoothing back up -- in one
// CTA, with a CTA barrier between steps.  Every row is computed by the same device functions, in the same
// order, as by the per-step kernels, so the result is bit-identical (MRG_PREC_GMG_SPLIT keeps the per-step
// launches for comparison).
constexpr int TT = 1024;               // threads of the tail CTA
constexpr int MAXTAIL = 8;             // levels the tail can hold
constexpr int64_t TAIL_ROWS32 = 1024;  // FP32: first level taken into the tail has at most this many rows
// A level's sweep in one SM must cost less than the launches it replaces.  Measured on the C2 mixed
// multigrid Newton solve (128^3): FP32 tail from 9^3 nodes 9.62 ms, none 9.83 ms, from 17^3 nodes
// 10.66 ms.  FP64 takes none: its pipe (1/64 of the FP32 rate) makes a single-SM sweep of a 729-row
// level as long as a launch, and from 17^3 nodes the FP64 solve went 26.4 -> 31.9 ms.
template <typename T>
constexpr int64_t tail_rows() { return sizeof(T) == 4 ? TAIL_ROWS32 : 0; }

template <typename T>
struct TailArgs {
  int nlev = 0;                  // levels in the tail; the last is the coarsest
  LevDev<T> L[MAXTAIL];
  Xfer X[MAXTAIL];               // X[j]: how tail level j was coarsened from level j - 1
  const double* coef[MAXTAIL];   // Chebyshev coefficients of each level
  const T* cinv = nullptr;       // dense inverse of the coarsest operator
};

template <typename T>
__device__ __forceinline__ void tail_cheb(const LevDev<T>& D, const T* xin, T* xout, int k, int zero_x,
                                          const double* __restrict__ coef) {
  const T c_first = (T)coef[3 * k], c_old = (T)coef[3 * k + 1], c_new = (T)coef[3 * k + 2];
  for (int64_t n = threadIdx.x; n < D.n; n += TT) {
    T ax = T(0);
    if (!zero_x) {
      int ix, iy, iz;
      decompose(D.g, n, ix, iy, iz);
      const RowInfo R = row_info<1>(D.g, ix, iy, iz);
      ax = (T)row_prod<1, T>(D.g, R, D.A + R.rp, xin);
    }
    cheb_row<T>(D, n, ax, xin, xout, k, zero_x, c_first, c_old, c_new);
  }
  __syncthreads();
}

template <typename T>
__global__ void __launch_bounds__(TT) k_vcycle_tail(const TailArgs<T> A, const GScal* __restrict__ S) {
  if (is_done(S)) return;
  const int nl = A.nlev;
  for (int j = 0; j < nl - 1; ++j) {
    const LevDev<T>& D = A.L[j];
    tail_cheb<T>(D, D.xa, D.xa, 0, 1, A.coef[j]);
    tail_cheb<T>(D, D.xa, D.xb, 1, 0, A.coef[j]);
    for (int64_t n = threadIdx.x; n < D.n; n += TT) {
      int ix, iy, iz;
      decompose(D.g, n, ix, iy, iz);
      const RowInfo R = row_info<1>(D.g, ix, iy, iz);
      resid_row<T>(D, n, (T)row_prod<1, T>(D.g, R, D.A + R.rp, D.xb));
    }
    __syncthreads();
    const LevDev<T>& C = A.L[j + 1];
    for (int64_t n = threadIdx.x; n < C.n; n += TT) restrict_row<T>(D.g, C.g, A.X[j + 1], D.r, C.b, n);
    __syncthreads();
  }
  const LevDev<T>& Lc = A.L[nl - 1];
  for (int i = threadIdx.x; i < (int)Lc.n; i += TT) coarse_row<T>((int)Lc.n, A.cinv, Lc.b, Lc.xb, i);
  __syncthreads();
  for (int j = nl - 2; j >= 0; --j) {
    const LevDev<T>& D = A.L[j];
    const LevDev<T>& C = A.L[j + 1];
    for (int64_t n = threadIdx.x; n < D.n; n += TT) prolong_row<T>(D.g, C.g, A.X[j + 1], C.xb, D.xb, n);
    __syncthreads();
    tail_cheb<T>(D, D.xb, D.xa, 0, 0, A.coef[j]);
    tail_cheb<T>(D, D.xa, D.xb, 1, 0, A.coef[j]);
  }
}

// ---- CG kernels -----------------------------------------------------------------------------------
template <typename T>
struct CgVec {
  T *x, *r, *p, *q;
  const T* z;
  double* parts;
  GScal* S;
};

// x = 0, r = b (FP64 in, T out), p = q = 0; r0 = |r|
template <typename T>
__global__ void __launch_bounds__(NT) k_cg_init(int64_t n, const double* __restrict__ b, CgVec<T> V) {
  T rr = T(0);  // per-thread partials in the vector precision (no per-element FP64 work for FP32)
  for (int64_t i = (int64_t)blockIdx.x * NT + threadIdx.x; i < n; i += (int64_t)gridDim.x * NT) {
    const T r = (T)b[i];
    V.x[i] = T(0);
    V.r[i] = r;
    V.p[i] = T(0);
    V.q[i] = T(0);
    rr = fma(r, r, rr);
  }
  double m[1] = {block_sum((double)rr)};
  if (last_block<1>(V.parts, m, &V.S->counter)) {
    double t[1];
    sum_parts<1>(V.parts, t, &V.S->counter);
    if (threadIdx.x == 0) {
      GScal* S = V.S;
      S->r0 = sqrt(t[0]);
      S->rnorm = S->r0;
      S->iter = 0;
      S->status = MRG_OK;
      S->beta = 0.0;
      S->rho = 0.0;
      S->done = (S->r0 == 0.0 || S->maxiter <= 0) ? 1 : 0;
      if (!isfinite(S->r0)) { S->done = 1; S->status = MRG_ENUMERIC; }
    }
  }
}

// rho_new = r . z ; beta = rho_new / rho (0 on the first call)
template <typename T>
__global__ void __launch_bounds__(NT) k_cg_rz(int64_t n, CgVec<T> V, int first) {
  if (is_done(V.S)) return;
  T rz = T(0);
  for (int64_t i = (int64_t)blockIdx.x * NT + threadIdx.x; i < n; i += (int64_t)gridDim.x * NT)
    rz = fma(V.r[i], V.z[i], rz);
  double m[1] = {block_sum((double)rz)};
  if (last_block<1>(V.parts, m, &V.S->counter)) {
    double t[1];
    sum_parts<1>(V.parts, t, &V.S->counter);
    if (threadIdx.x == 0) {
      GScal* S = V.S;
      S->beta = first ? 0.0 : t[0] / S->rho;
      S->rho = t[0];
      if (!(t[0] > 0.0) || !isfinite(t[0])) { S->status = MRG_ENUMERIC; S->done = 1; }
    }
  }
}

// w = A z ; p = z + beta p ; q = w + beta q ; partial p.q ; alpha = rho / p.q
template <int P, typename T>
__global__ void __launch_bounds__(NT) k_cg_spmv(Grid g, int64_t n, const T* __restrict__ A, CgVec<T> V) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t mbar[2 * (NT / 32)];
  if (is_done(V.S)) return;
  const T beta = (T)V.S->beta;
  T pq = T(0);
  const bool ok = level_rows<P, T>(g, n, A, smem_raw, mbar, [&](int64_t i, const RowInfo& R, const T* vals) {
    const T w = (T)row_prod<P, T>(g, R, vals, V.z);
    const T pn = V.z[i] + beta * V.p[i];
    const T qn = w + beta * V.q[i];
    V.p[i] = pn;
    V.q[i] = qn;
    pq = fma(pn, qn, pq);
  });
  if (!ok) atomicExch(&V.S->err, 3);
  double m[1] = {block_sum((double)pq)};
  if (last_block<1>(V.parts, m, &V.S->counter)) {
    double t[1];
    sum_parts<1>(V.parts, t, &V.S->counter);
    if (threadIdx.x == 0) {
      GScal* S = V.S;
      S->pq = t[0];
      S->alpha = S->rho / t[0];
      if (!(t[0] > 0.0) || !isfinite(S->alpha)) { S->status = MRG_ENUMERIC; S->done = 1; }
      if (S->err) { S->status = MRG_ETIMEOUT; S->done = 1; }
    }
  }
}

// x += alpha p ; r -= alpha q ; |r| ; stopping test
template <typename T>
__global__ void __launch_bounds__(NT) k_cg_update(int64_t n, CgVec<T> V) {
  if (is_done(V.S)) return;
  const T alpha = (T)V.S->alpha;
  T rr = T(0);
  for (int64_t i = (int64_t)blockIdx.x * NT + threadIdx.x; i < n; i += (int64_t)gridDim.x * NT) {
    V.x[i] += alpha * V.p[i];
    const T r = V.r[i] - alpha * V.q[i];
    V.r[i] = r;
    rr = fma(r, r, rr);
  }
  double m[1] = {block_sum((double)rr)};
  if (last_block<1>(V.parts, m, &V.S->counter)) {
    double t[1];
    sum_parts<1>(V.parts, t, &V.S->counter);
    if (threadIdx.x == 0) {
      GScal* S = V.S;
      S->rnorm = sqrt(t[0]);
      S->iter += 1;
      if (!(S->rnorm / S->r0 > S->tol) || S->iter >= S->maxiter) S->done = 1;
      if (!isfinite(S->rnorm)) { S->done = 1; S->status = MRG_ENUMERIC; }
    }
  }
}

template <typename T>
__global__ void k_to_f64(int64_t n, const T* __restrict__ a, double* __restrict__ b) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = (double)a[i];
}

// ---- BiCGStab kernels (right preconditioning by the same V-cycle) ------------------------------
template <typename T>
struct BgVec {
  T *x, *r, *rh, *p, *v, *s, *t, *ph, *sh;
  double* parts;
  GScal* S;
};

// x = 0, r = rh = b, p = v = 0; rho = (rh . r), alpha = omega = 1, beta = 0
template <typename T>
__global__ void __launch_bounds__(NT) k_bg_init(int64_t n, const double* __restrict__ b, BgVec<T> V) {
  T rr = T(0);
  for (int64_t i = (int64_t)blockIdx.x * NT + threadIdx.x; i < n; i += (int64_t)gridDim.x * NT) {
    const T r = (T)b[i];
    V.x[i] = T(0);
    V.r[i] = r;
    V.rh[i] = r;
    V.p[i] = T(0);
    V.v[i] = T(0);
    rr = fma(r, r, rr);
  }
  double m[1] = {block_sum((double)rr)};
  if (last_block<1>(V.parts, m, &V.S->counter)) {
    double t[1];
    sum_parts<1>(V.parts, t, &V.S->counter);
    if (threadIdx.x == 0) {
      GScal* S = V.S;
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

// p = r + beta (p - omega v)
template <typename T>
__global__ void __launch_bounds__(NT) k_bg_p(int64_t n, BgVec<T> V) {
  if (is_done(V.S)) return;
  const T beta = (T)V.S->beta, omega = (T)V.S->omega;
  for (int64_t i = (int64_t)blockIdx.x * NT + threadIdx.x; i < n; i += (int64_t)gridDim.x * NT)
    V.p[i] = V.r[i] + beta * (V.p[i] - omega * V.v[i]);
}

// STEP 0: v = A ph, rv = rh . v, alpha = rho / rv.   STEP 1: t = A sh, omega = (t . s) / (t . t).
template <int P, typename T, int STEP>
__global__ void __launch_bounds__(NT) k_bg_spmv(Grid g, int64_t n, const T* __restrict__ A, BgVec<T> V) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t mbar[2 * (NT / 32)];
  if (is_done(V.S)) return;
  const T* in = STEP == 0 ? V.ph : V.sh;
  T* out = STEP == 0 ? V.v : V.t;
  T d0 = T(0), d1 = T(0);
  const bool ok = level_rows<P, T>(g, n, A, smem_raw, mbar, [&](int64_t i, const RowInfo& R, const T* vals) {
    const T y = (T)row_prod<P, T>(g, R, vals, in);
    out[i] = y;
    if (STEP == 0) {
      d0 = fma(V.rh[i], y, d0);
    } else {
      d0 = fma(y, V.s[i], d0);
      d1 = fma(y, y, d1);
    }
  });
  if (!ok) atomicExch(&V.S->err, 3);
  double m[2] = {block_sum((double)d0), block_sum((double)d1)};
  if (last_block<2>(V.parts, m, &V.S->counter)) {
    double t[2];
    sum_parts<2>(V.parts, t, &V.S->counter);
    if (threadIdx.x == 0) {
      GScal* S = V.S;
      if (STEP == 0) {
        S->rv = t[0];
        S->alpha = S->rho / t[0];
        if (!(t[0] != 0.0) || !isfinite(S->alpha)) { S->status = MRG_ENUMERIC; S->done = 1; }
      } else {
        S->omega = (t[1] > 0.0) ? t[0] / t[1] : 0.0;
      }
      if (S->err) { S->status = MRG_ETIMEOUT; S->done = 1; }
    }
  }
}

// s = r - alpha v
template <typename T>
__global__ void __launch_bounds__(NT) k_bg_s(int64_t n, BgVec<T> V) {
  if (is_done(V.S)) return;
  const T alpha = (T)V.S->alpha;
  for (int64_t i = (int64_t)blockIdx.x * NT + threadIdx.x; i < n; i += (int64_t)gridDim.x * NT)
    V.s[i] = V.r[i] - alpha * V.v[i];
}

// x += alpha ph + omega sh ; r = s - omega t ; |r|, rh . r -> beta for the next direction; stopping test
template <typename T>
__global__ void __launch_bounds__(NT) k_bg_update(int64_t n, BgVec<T> V) {
  if (is_done(V.S)) return;
  const T alpha = (T)V.S->alpha, omega = (T)V.S->omega;
  T rr = T(0), rhr = T(0);
  for (int64_t i = (int64_t)blockIdx.x * NT + threadIdx.x; i < n; i += (int64_t)gridDim.x * NT) {
    V.x[i] += alpha * V.ph[i] + omega * V.sh[i];
    const T r = V.s[i] - omega * V.t[i];
    V.r[i] = r;
    rr = fma(r, r, rr);
    rhr = fma(V.rh[i], r, rhr);
  }
  double m[2] = {block_sum((double)rr), block_sum((double)rhr)};
  if (last_block<2>(V.parts, m, &V.S->counter)) {
    double t[2];
    sum_parts<2>(V.parts, t, &V.S->counter);
    if (threadIdx.x == 0) {
      GScal* S = V.S;
      S->rnorm = sqrt(t[0]);
      S->iter += 1;
      S->beta = (t[1] / S->rho) * (S->alpha / S->omega);
      S->rho = t[1];
      if (!(S->rnorm / S->r0 > S->tol) || S->iter >= S->maxiter) S->done = 1;
      if (!isfinite(S->rnorm)) { S->done = 1; S->status = MRG_ENUMERIC; }
      else if (!S->done && (!(t[1] != 0.0) || !(S->omega != 0.0))) { S->done = 1; S->status = MRG_ENUMERIC; }
    }
  }
}

inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

int num_sms() { return mrg_device_sms(); }

unsigned grid_for(int64_t n, int per_sm) {
  const unsigned need = nblk(n, NT), cap = (unsigned)(per_sm * num_sms());
  return need < cap ? need : cap;
}

template <typename T>
constexpr int staged_per_sm() { return sizeof(T) == 8 ? 4 : 7; }

// ---- hierarchy ------------------------------------------------------------------------------------
struct HLevel {
  Grid g;
  int64_t n = 0, nnz = 0;
  Xfer X{{0, 0, 0}};          // how this level was coarsened from the finer one
  P3 pp{{1, 1, 1}};           // per-axis coupling order of this level (2 only on a Q2 level 0)
  int nsweep = 0;             // Galerkin sweeps from the finer level (one per coarsened axis)
  int sweep_axis[3] = {0, 0, 0};
  Grid mid[2];                // intermediate grids after all but the last sweep
  P3 mid_pp[2];
  int64_t* d_mid_pref[2] = {nullptr, nullptr};
  int64_t* d_pref = nullptr;  // prefix tables (coarse levels)
  void* A = nullptr;          // coarse levels: owned; level 0: the caller's Jacobian
  void *minv = nullptr, *xa = nullptr, *xb = nullptr, *d = nullptr, *b = nullptr, *r = nullptr;
};

template <typename T>
struct Hier {
  std::vector<HLevel> L;
  T* cinv = nullptr;
  T* mid[2] = {nullptr, nullptr};  // intermediate operators of the Galerkin sweeps
  unsigned int* lmax = nullptr;   // [nlev] float bits
  double* coef = nullptr;         // [nlev][NU][3] Chebyshev coefficients
  int* err = nullptr;             // setup / cycle error word
  T *x = nullptr, *r = nullptr, *p = nullptr, *q = nullptr;  // CG vectors (level-0 size)
  double* parts = nullptr;
  GScal* S = nullptr;
  GScal* h_S = nullptr;           // pinned mirror
  cudaGraphExec_t graph = nullptr;
  const void* graph_A = nullptr;
  cudaStream_t graph_stream = nullptr;
  // BiCGStab vectors (allocated on first use) and its captured chunk
  T *rh = nullptr, *v = nullptr, *sv = nullptr, *t = nullptr, *ph = nullptr, *sh = nullptr;
  cudaGraphExec_t bgraph = nullptr;
  const void* bgraph_A = nullptr;
  cudaStream_t bgraph_stream = nullptr;
  const void* setup_J = nullptr;  // Jacobian of the last setup
  // levels >= tail run in k_vcycle_tail (tail == number of levels: every step its own launch)
  int tail = -1;
  int graph_tail = -1, bgraph_tail = -1;  // the tail the captured chunks were recorded with
  TailArgs<T> targs;
};

struct GmgData {
  int kind = MRG_PREC_JACOBI;
  bool split = false;  // MRG_PREC_GMG_SPLIT: no fused coarse-level tail
  Hier<double>* h64 = nullptr;
  Hier<float>* h32 = nullptr;
};

GmgData* gdata(mrg_problem* p) {
  if (!p->gmg) p->gmg = new GmgData();
  return reinterpret_cast<GmgData*>(p->gmg);
}

// Host grid of a p = 1 level with nn nodes per axis (prefix tables uploaded to d_pref).
int make_level_grid(const Grid& fine, const int nn[3], const P3& pp, cudaStream_t s, Grid& g, int64_t*& d_pref) {
  g = fine;
  g.p = std::max(pp.p[0], std::max(pp.p[1], pp.p[2]));
  for (int k = 0; k < 3; ++k) {
    g.nn[k] = nn[k];
    g.nc[k] = (k < fine.dim) ? (nn[k] - 1) / pp.p[k] : 1;
  }
  std::vector<int64_t> pref;
  int64_t offs[3];
  for (int k = 0; k < 3; ++k) {
    offs[k] = (int64_t)pref.size();
    int64_t acc = 0;
    pref.push_back(0);
    for (int i = 0; i < g.nn[k]; ++i) {
      int lo, cnt;
      if (k < g.dim) axis_range(i, g.nn[k], pp.p[k], lo, cnt); else cnt = 1;
      acc += cnt;
      pref.push_back(acc);
    }
    g.T[k] = acc;
  }
  MRG_CUDA(cudaMallocAsync(&d_pref, pref.size() * sizeof(int64_t), s));
  MRG_CUDA(cudaMemcpyAsync(d_pref, pref.data(), pref.size() * sizeof(int64_t), cudaMemcpyHostToDevice, s));
  for (int k = 0; k < 3; ++k) g.P[k] = d_pref + offs[k];
  return MRG_OK;
}

template <typename T>
void free_hier(Hier<T>* H, cudaStream_t s) {
  if (!H) return;
  if (H->graph) cudaGraphExecDestroy(H->graph);
  if (H->bgraph) cudaGraphExecDestroy(H->bgraph);
  for (void* ptr : {(void*)H->rh, (void*)H->v, (void*)H->sv, (void*)H->t, (void*)H->ph, (void*)H->sh})
    if (ptr) cudaFreeAsync(ptr, s);
  for (size_t l = 0; l < H->L.size(); ++l) {
    HLevel& L = H->L[l];
    if (l > 0) {
      if (L.A) cudaFreeAsync(L.A, s);
      if (L.d_pref) cudaFreeAsync(L.d_pref, s);
      for (int k = 0; k < 2; ++k)
        if (L.d_mid_pref[k]) cudaFreeAsync(L.d_mid_pref[k], s);
    }
    for (void* ptr : {L.minv, L.xa, L.xb, L.d, L.b, L.r})
      if (ptr) cudaFreeAsync(ptr, s);
  }
  for (void* ptr : {(void*)H->mid[0], (void*)H->mid[1]})
    if (ptr) cudaFreeAsync(ptr, s);
  for (void* ptr : {(void*)H->cinv, (void*)H->lmax, (void*)H->coef, (void*)H->err, (void*)H->x, (void*)H->r, (void*)H->p,
                    (void*)H->q, (void*)H->parts, (void*)H->S})
    if (ptr) cudaFreeAsync(ptr, s);
  mrg_pinned_release(H->h_S);
  delete H;
}

// Builds the level structure (sizes, grids, buffers).  Values are computed by setup_values.
template <typename T>
int build_hier(const mrg_problem* p, Hier<T>*& out, cudaStream_t s) {
  Hier<T>* H = new Hier<T>();
  auto fail = [&](int rc) {
    free_hier(H, s);
    return rc;
  };
  HLevel L0;
  L0.g = p->g;
  L0.n = p->ndof;
  L0.nnz = p->nnz;
  for (int k = 0; k < 3; ++k) L0.pp.p[k] = (k < p->g.dim) ? p->g.p : 1;
  H->L.push_back(L0);
  // cell size per axis (box estimate); an axis is coarsened only while its cells are at most twice as
  // long as the shortest ones (semi-coarsening keeps point smoothing effective on stretched grids)
  double h[3] = {p->h[0], p->h[1], p->h[2]};
  while ((int)H->L.size() < MAXLEV) {
    const Grid& gf = H->L.back().g;
    const P3 pf = H->L.back().pp;
    const bool ptransfer = pf.p[0] == 2;  // Q2 level 0 -> Q1 on the same cells: every axis, h unchanged
    int nn[3], co[3] = {0, 0, 0}, any = 0;
    double hmin = 1e300;
    for (int k = 0; k < gf.dim; ++k) hmin = std::fmin(hmin, h[k]);
    for (int pass = 0; pass < 2 && !any; ++pass)
      for (int k = 0; k < gf.dim; ++k)
        if (ptransfer || (gf.nn[k] - 1 >= 3 && (pass == 1 || h[k] <= 2.0 * hmin * (1.0 + 1e-9)))) {
          co[k] = 1;
          any = 1;
        }
    for (int k = 0; k < 3; ++k) {
      nn[k] = gf.nn[k];
      if (co[k]) {
        nn[k] = (gf.nn[k] - 1 + 1) / 2 + 1;
        if (!ptransfer) h[k] *= 2.0;
      }
    }
    const int64_t nfine = H->L.back().n;
    if (!any || (nfine <= MAXC && !ptransfer)) break;
    HLevel Lc;
    int rc = make_level_grid(gf, nn, Lc.pp, s, Lc.g, Lc.d_pref);
    if (rc) { H->L.push_back(Lc); return fail(rc); }
    for (int k = 0; k < 3; ++k) Lc.X.co[k] = co[k];
    // sweep plan: coarsen the axes one at a time; intermediate grids for all but the last sweep (a
    // swept axis couples at order 1, the others keep the finer level's order)
    int cur[3] = {gf.nn[0], gf.nn[1], gf.nn[2]};
    P3 cp = pf;
    for (int k = 0; k < 3; ++k)
      if (co[k]) Lc.sweep_axis[Lc.nsweep++] = k;
    for (int w = 0; w + 1 < Lc.nsweep; ++w) {
      cur[Lc.sweep_axis[w]] = nn[Lc.sweep_axis[w]];
      cp.p[Lc.sweep_axis[w]] = 1;
      Lc.mid_pp[w] = cp;
      rc = make_level_grid(gf, cur, cp, s, Lc.mid[w], Lc.d_mid_pref[w]);
      if (rc) { H->L.push_back(Lc); return fail(rc); }
    }
    Lc.n = (int64_t)nn[0] * nn[1] * nn[2];
    Lc.nnz = Lc.g.T[0] * Lc.g.T[1] * Lc.g.T[2];
    H->L.push_back(Lc);
  }
  if (H->L.back().n > MAXC) return fail(mrg_fail(MRG_ENOTSUP, "multigrid: coarsest level too large"));
  for (size_t l = 0; l < H->L.size(); ++l) {
    HLevel& L = H->L[l];
    const size_t vb = (size_t)L.n * sizeof(T);
    if (l > 0 && cudaMallocAsync(&L.A, (size_t)L.nnz * sizeof(T), s) != cudaSuccess) return fail(mrg_fail(MRG_ENOMEM, "multigrid level matrix"));
    for (void** ptr : {&L.minv, &L.xa, &L.xb, &L.d, &L.b, &L.r})
      if (cudaMallocAsync(ptr, vb, s) != cudaSuccess) return fail(mrg_fail(MRG_ENOMEM, "multigrid level vectors"));
  }
  // scratch for the intermediate operators (largest over all levels)
  size_t midmax[2] = {0, 0};
  for (size_t l = 1; l < H->L.size(); ++l)
    for (int w = 0; w + 1 < H->L[l].nsweep; ++w) {
      const Grid& gm = H->L[l].mid[w];
      midmax[w] = std::max(midmax[w], (size_t)(gm.T[0] * gm.T[1] * gm.T[2]));
    }
  for (int w = 0; w < 2; ++w)
    if (midmax[w] && cudaMallocAsync(&H->mid[w], midmax[w] * sizeof(T), s) != cudaSuccess)
      return fail(mrg_fail(MRG_ENOMEM, "multigrid Galerkin scratch"));
  const int64_t n0 = p->ndof, nc = H->L.back().n;
  const size_t nparts = (size_t)2 * grid_for(n0, 16) + 64;
  if (cudaMallocAsync(&H->cinv, (size_t)nc * nc * sizeof(T), s) != cudaSuccess ||
      cudaMallocAsync(&H->lmax, MAXLEV * sizeof(unsigned int), s) != cudaSuccess ||
      cudaMallocAsync(&H->coef, (size_t)MAXLEV * NU * 3 * sizeof(double), s) != cudaSuccess ||
      cudaMallocAsync(&H->err, sizeof(int), s) != cudaSuccess ||
      cudaMallocAsync(&H->x, n0 * sizeof(T), s) != cudaSuccess || cudaMallocAsync(&H->r, n0 * sizeof(T), s) != cudaSuccess ||
      cudaMallocAsync(&H->p, n0 * sizeof(T), s) != cudaSuccess || cudaMallocAsync(&H->q, n0 * sizeof(T), s) != cudaSuccess ||
      cudaMallocAsync(&H->parts, nparts * sizeof(double), s) != cudaSuccess ||
      cudaMallocAsync(&H->S, sizeof(GScal), s) != cudaSuccess)
    return fail(mrg_fail(MRG_ENOMEM, "multigrid workspace"));
  static_assert(sizeof(GScal) <= 256, "pinned slot size");
  H->h_S = (GScal*)mrg_pinned_slot();
  if (!H->h_S) return fail(mrg_fail(MRG_ENOMEM, "multigrid pinned scalars"));
  MRG_CUDA(cudaMemsetAsync(H->S, 0, sizeof(GScal), s));
  MRG_CUDA(cudaMemsetAsync(H->parts, 0, nparts * sizeof(double), s));
  out = H;
  return MRG_OK;
}

template <typename T>
LevDev<T> levdev(const HLevel& L) {
  return LevDev<T>{L.g, L.n, (const T*)L.A, (T*)L.minv, (T*)L.xa, (T*)L.xb, (T*)L.d, (T*)L.b, (T*)L.r};
}

// First level of the fused tail: the first level below the finest with at most tail_rows<T>() rows (all
// levels below the finest are Q1), unless the caller asked for the split cycle or the tail would be too
// deep.  Fills the tail's kernel arguments.
template <typename T>
void set_tail(Hier<T>* H, bool split) {
  const int nl = (int)H->L.size();
  int t = nl;
  if (!split) {
    for (int l = 1; l < nl; ++l)
      if (H->L[l].n <= tail_rows<T>()) { t = l; break; }
    if (nl - t > MAXTAIL) t = nl;
    for (int l = t; l < nl; ++l)
      if (H->L[l].pp.p[0] != 1 || H->L[l].pp.p[1] != 1 || H->L[l].pp.p[2] != 1) t = nl;
  }
  H->tail = t;
  TailArgs<T>& A = H->targs;
  A.nlev = nl - t;
  for (int j = 0; j < A.nlev; ++j) {
    A.L[j] = levdev<T>(H->L[t + j]);
    A.X[j] = H->L[t + j].X;
    A.coef[j] = H->coef + (size_t)(t + j) * NU * 3;
  }
  A.cinv = H->cinv;
}

template <typename T>
int set_staged_attr() {
  static std::once_flag once;
  static cudaError_t e = cudaSuccess;
  std::call_once(once, [] {
    const int smem = (NT / 32) * 2 * wbuf_elems<T>() * (int)sizeof(T);
    e = cudaFuncSetAttribute(k_cheb<1, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_resid<1, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_cg_spmv<1, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_bg_spmv<1, T, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_bg_spmv<1, T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  });
  return e == cudaSuccess ? MRG_OK : mrg_cuda_check(e, "multigrid smem attribute");
}

template <typename T>
constexpr int staged_smem() { return (NT / 32) * 2 * wbuf_elems<T>() * (int)sizeof(T); }

// Level operators, diagonals, Gershgorin bounds and the coarsest inverse for the Jacobian J.
// Level 0 only: the new J, its Jacobi inverse and Chebyshev bound; the coarse levels stay as they are.
template <typename T>
int setup_level0(Hier<T>* H, const T* J, cudaStream_t s) {
  HLevel& L = H->L[0];
  L.A = const_cast<T*>(J);
  MRG_CUDA(cudaMemsetAsync(H->lmax, 0, sizeof(unsigned int), s));
  if (L.pp.p[0] == 2) k_diag<2, T><<<nblk(L.n, NT), NT, 0, s>>>(L.g, (const T*)L.A, (T*)L.minv, H->lmax);
  else k_diag<1, T><<<nblk(L.n, NT), NT, 0, s>>>(L.g, (const T*)L.A, (T*)L.minv, H->lmax);
  k_cheb_coef<<<1, 32, 0, s>>>(H->lmax, (int)H->L.size(), H->coef);
  MRG_CUDA(cudaGetLastError());
  return MRG_OK;
}

template <typename T>
int setup_values(Hier<T>* H, const T* J, cudaStream_t s) {
  H->L[0].A = const_cast<T*>(J);
  MRG_CUDA(cudaMemsetAsync(H->lmax, 0, MAXLEV * sizeof(unsigned int), s));
  MRG_CUDA(cudaMemsetAsync(H->err, 0, sizeof(int), s));
  const int nl = (int)H->L.size();
  for (int l = 0; l < nl; ++l) {
    HLevel& L = H->L[l];
    if (l > 0) {
      const HLevel& F = H->L[l - 1];
      const Grid* gin = &F.g;
      P3 pin = F.pp;
      const T* ain = (const T*)F.A;
      for (int w = 0; w < L.nsweep; ++w) {
        const bool last = (w + 1 == L.nsweep);
        const Grid& gout = last ? L.g : L.mid[w];
        const P3 pout = last ? L.pp : L.mid_pp[w];
        T* aout = last ? (T*)L.A : H->mid[w];
        const int64_t nout = (int64_t)gout.nn[0] * gout.nn[1] * gout.nn[2];
        if (nout < RAP_WARP_ROWS) {
          const unsigned nb = nblk(nout * 32, NT);
          if (L.sweep_axis[w] == 0) k_rap_axis_w<T, 0><<<nb, NT, 0, s>>>(*gin, pin, gout, pout, ain, aout);
          else if (L.sweep_axis[w] == 1) k_rap_axis_w<T, 1><<<nb, NT, 0, s>>>(*gin, pin, gout, pout, ain, aout);
          else k_rap_axis_w<T, 2><<<nb, NT, 0, s>>>(*gin, pin, gout, pout, ain, aout);
        } else
          k_rap_axis<T><<<nblk(nout, NT), NT, 0, s>>>(*gin, pin, gout, pout, L.sweep_axis[w], ain, aout, H->err);
        MRG_CUDA(cudaGetLastError());
        gin = &gout;
        pin = pout;
        ain = aout;
      }
    }
    if (L.pp.p[0] == 2) k_diag<2, T><<<nblk(L.n, NT), NT, 0, s>>>(L.g, (const T*)L.A, (T*)L.minv, H->lmax + l);
    else k_diag<1, T><<<nblk(L.n, NT), NT, 0, s>>>(L.g, (const T*)L.A, (T*)L.minv, H->lmax + l);
    MRG_CUDA(cudaGetLastError());
  }
  k_coarse_inv<T><<<1, NT, 0, s>>>(H->L.back().g, (const T*)H->L.back().A, H->cinv, H->err);
  k_cheb_coef<<<1, 32, 0, s>>>(H->lmax, nl, H->coef);
  MRG_CUDA(cudaGetLastError());
  return MRG_OK;
}

// Launches of the row kernels for a level: Q1 levels use the staged loop (dynamic shared memory, fewer
// CTAs per SM), a Q2 level 0 the direct row loop.
template <typename T>
void launch_cheb(const HLevel& L, const LevDev<T>& D, const T* xin, T* xout, int k, int zero_x,
                 const double* coef, const GScal* S, int* err, cudaStream_t s) {
  if (zero_x)
    k_cheb<1, T><<<grid_for(D.n, 16), NT, 0, s>>>(D, xin, xout, k, 1, coef, S, err);
  else if (L.pp.p[0] == 2)
    k_cheb<2, T><<<grid_for(D.n, 16), NT, 0, s>>>(D, xin, xout, k, 0, coef, S, err);
  else
    k_cheb<1, T><<<grid_for(D.n, staged_per_sm<T>()), NT, staged_smem<T>(), s>>>(D, xin, xout, k, 0, coef, S, err);
}

template <typename T>
void launch_resid(const HLevel& L, const LevDev<T>& D, const T* x, const GScal* S, int* err, cudaStream_t s) {
  if (L.pp.p[0] == 2) k_resid<2, T><<<grid_for(D.n, 16), NT, 0, s>>>(D, x, S, err);
  else k_resid<1, T><<<grid_for(D.n, staged_per_sm<T>()), NT, staged_smem<T>(), s>>>(D, x, S, err);
}

// One V(NU, NU) cycle: out = M^{-1} in on level 0 (in, out: level-0 vectors not used by the cycle).
template <typename T>
void enqueue_vcycle(Hier<T>* H, const T* in, T* out, cudaStream_t s) {
  const int nl = (int)H->L.size();
  const int tail = H->tail < 1 ? nl : H->tail;  // levels >= tail: k_vcycle_tail
  const GScal* S = H->S;
  for (int l = 0; l < nl - 1 && l < tail; ++l) {
    LevDev<T> D = levdev<T>(H->L[l]);
    if (l == 0) D.b = const_cast<T*>(in);
    // pre-smoothing from x = 0: xa <- step 0, xb <- step 1
    launch_cheb<T>(H->L[l], D, D.xa, D.xa, 0, 1, H->coef + (size_t)l * NU * 3, S, H->err, s);
    launch_cheb<T>(H->L[l], D, D.xa, D.xb, 1, 0, H->coef + (size_t)l * NU * 3, S, H->err, s);
    launch_resid<T>(H->L[l], D, D.xb, S, H->err, s);
    const HLevel& C = H->L[l + 1];
    k_restrict<T><<<grid_for(C.n, 16), NT, 0, s>>>(D.g, C.g, C.X, D.r, (T*)C.b, S);
  }
  if (tail < nl) {
    k_vcycle_tail<T><<<1, TT, 0, s>>>(H->targs, S);
  } else {
    const HLevel& Lc = H->L[nl - 1];
    k_coarse_apply<T><<<1, NT, 0, s>>>((int)Lc.n, H->cinv, (const T*)Lc.b, (T*)Lc.xb, S);
  }
  for (int l = std::min(tail, nl - 1) - 1; l >= 0; --l) {
    LevDev<T> D = levdev<T>(H->L[l]);
    if (l == 0) D.b = const_cast<T*>(in);
    const HLevel& C = H->L[l + 1];
    k_prolong<T><<<grid_for(D.n, 16), NT, 0, s>>>(D.g, C.g, C.X, (const T*)C.xb, D.xb, S);
    // post-smoothing: xb -> xa (step 0), xa -> xb (step 1; level 0: -> out)
    launch_cheb<T>(H->L[l], D, D.xb, D.xa, 0, 0, H->coef + (size_t)l * NU * 3, S, H->err, s);
    launch_cheb<T>(H->L[l], D, D.xa, l == 0 ? out : D.xb, 1, 0, H->coef + (size_t)l * NU * 3, S, H->err, s);
  }
}

template <typename T>
CgVec<T> cgvec(Hier<T>* H) {
  return CgVec<T>{H->x, H->r, H->p, H->q, (const T*)H->L[0].xb, H->parts, H->S};
}

template <typename T>
void enqueue_iters(Hier<T>* H, int count, cudaStream_t s) {
  const HLevel& L0 = H->L[0];
  CgVec<T> V = cgvec(H);
  const unsigned ge = grid_for(L0.n, 16), gs = grid_for(L0.n, staged_per_sm<T>());
  for (int it = 0; it < count; ++it) {
    if (L0.pp.p[0] == 2) k_cg_spmv<2, T><<<ge, NT, 0, s>>>(L0.g, L0.n, (const T*)L0.A, V);
    else k_cg_spmv<1, T><<<gs, NT, staged_smem<T>(), s>>>(L0.g, L0.n, (const T*)L0.A, V);
    k_cg_update<T><<<ge, NT, 0, s>>>(L0.n, V);
    enqueue_vcycle(H, H->r, (T*)H->L[0].xb, s);
    k_cg_rz<T><<<ge, NT, 0, s>>>(L0.n, V, 0);
  }
}

template <typename T>
int finish_solve(mrg_problem* p, Hier<T>* H, cudaGraphExec_t graph, double* x, double rtol, int maxiter,
                 mrg_solve_stats* st, cudaStream_t s, const char* what) {
  const int64_t n = p->ndof;
  const int max_chunks = maxiter / GCHUNK + 2;
  for (int c = 0; c < max_chunks; ++c) {
    MRG_CUDA(cudaGraphLaunch(graph, s));
    MRG_CUDA(cudaMemcpyAsync(H->h_S, H->S, sizeof(GScal), cudaMemcpyDeviceToHost, s));
    MRG_CUDA(cudaStreamSynchronize(s));
    if (H->h_S->done) break;
  }
  int herr = 0;
  MRG_CUDA(cudaMemcpyAsync(&herr, H->err, sizeof(int), cudaMemcpyDeviceToHost, s));
  k_to_f64<T><<<nblk(n, 256), 256, 0, s>>>(n, H->x, x);
  MRG_CUDA(cudaGetLastError());
  MRG_CUDA(cudaStreamSynchronize(s));
  const GScal* h = H->h_S;
  if (st) {
    st->iterations = h->iter;
    st->outer_iterations = 0;
    st->rel_residual = (h->r0 > 0) ? h->rnorm / h->r0 : 0.0;
    st->abs_residual = h->rnorm;
    st->status = h->status;
  }
  if (herr == 3 || h->status == MRG_ETIMEOUT) return mrg_fail(MRG_ETIMEOUT, std::string(what) + ": a staging copy timed out");
  if (herr) return mrg_fail(MRG_ENUMERIC, "multigrid setup: singular coarse operator or transfer out of range");
  if (h->status != MRG_OK) return mrg_fail(h->status, std::string(what) + ": breakdown or non-finite values");
  if (h->r0 > 0 && h->rnorm / h->r0 > rtol) {
    if (st) st->status = MRG_ENOCONV;
    return mrg_fail(MRG_ENOCONV, std::string(what) + ": not converged within maxiter");
  }
  return MRG_OK;
}

// Brings the hierarchy up to date with J as the caller asks (MRG_GMG_SETUP_*); a J other than the one of
// the last setup always gets a full setup.
template <typename T>
int follow_j(Hier<T>* H, const T* J, int setup, cudaStream_t s) {
  if (setup == MRG_GMG_SETUP_FULL || H->setup_J != (const void*)J) {
    const int rc = setup_values(H, J, s);
    if (rc) return rc;
    H->setup_J = J;
  } else if (setup == MRG_GMG_SETUP_LEVEL0) {
    return setup_level0(H, J, s);
  }
  return MRG_OK;
}

template <typename T>
int gmg_cg(mrg_problem* p, Hier<T>* H, const T* J, const double* b, double* x, double rtol, int maxiter,
           mrg_solve_stats* st, int setup, cudaStream_t s) {
  int rc = set_staged_attr<T>();
  if (rc) return rc;
  rc = follow_j(H, J, setup, s);
  if (rc) return rc;
  set_tail(H, gdata(p)->split);
  GScal init{};
  init.tol = rtol;
  init.maxiter = maxiter;
  MRG_CUDA(cudaMemcpyAsync(H->S, &init, sizeof(GScal), cudaMemcpyHostToDevice, s));
  const int64_t n = p->ndof;
  CgVec<T> V = cgvec(H);
  k_cg_init<T><<<grid_for(n, 16), NT, 0, s>>>(n, b, V);
  MRG_CUDA(cudaGetLastError());
  enqueue_vcycle(H, H->r, (T*)H->L[0].xb, s);
  k_cg_rz<T><<<grid_for(n, 16), NT, 0, s>>>(n, V, 1);
  MRG_CUDA(cudaGetLastError());
  // captured chunk of iterations (re-captured when the Jacobian pointer or the stream changes)
  if (!H->graph || H->graph_A != (const void*)J || H->graph_stream != s || H->graph_tail != H->tail) {
    if (H->graph) {
      cudaGraphExecDestroy(H->graph);
      H->graph = nullptr;
    }
    cudaStream_t cs = nullptr;
    MRG_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      enqueue_iters(H, GCHUNK, cs);
      e = cudaStreamEndCapture(cs, &graph);
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&H->graph, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    cudaStreamDestroy(cs);
    if (e != cudaSuccess) return mrg_cuda_check(e, "multigrid CG graph capture");
    H->graph_A = J;
    H->graph_stream = s;
    H->graph_tail = H->tail;
  }
  return finish_solve(p, H, H->graph, x, rtol, maxiter, st, s, "multigrid CG");
}

template <typename T>
BgVec<T> bgvec(Hier<T>* H) {
  return BgVec<T>{H->x, H->r, H->rh, H->p, H->v, H->sv, H->t, H->ph, H->sh, H->parts, H->S};
}

template <typename T>
void enqueue_bg_iters(Hier<T>* H, int count, cudaStream_t s) {
  const HLevel& L0 = H->L[0];
  BgVec<T> V = bgvec(H);
  const unsigned ge = grid_for(L0.n, 16), gs = grid_for(L0.n, staged_per_sm<T>());
  for (int it = 0; it < count; ++it) {
    k_bg_p<T><<<ge, NT, 0, s>>>(L0.n, V);
    enqueue_vcycle(H, H->p, H->ph, s);
    if (L0.pp.p[0] == 2) k_bg_spmv<2, T, 0><<<ge, NT, 0, s>>>(L0.g, L0.n, (const T*)L0.A, V);
    else k_bg_spmv<1, T, 0><<<gs, NT, staged_smem<T>(), s>>>(L0.g, L0.n, (const T*)L0.A, V);
    k_bg_s<T><<<ge, NT, 0, s>>>(L0.n, V);
    enqueue_vcycle(H, H->sv, H->sh, s);
    if (L0.pp.p[0] == 2) k_bg_spmv<2, T, 1><<<ge, NT, 0, s>>>(L0.g, L0.n, (const T*)L0.A, V);
    else k_bg_spmv<1, T, 1><<<gs, NT, staged_smem<T>(), s>>>(L0.g, L0.n, (const T*)L0.A, V);
    k_bg_update<T><<<ge, NT, 0, s>>>(L0.n, V);
  }
}

template <typename T>
int gmg_bicgstab(mrg_problem* p, Hier<T>* H, const T* J, const double* b, double* x, double rtol, int maxiter,
                 mrg_solve_stats* st, int setup, cudaStream_t s) {
  int rc = set_staged_attr<T>();
  if (rc) return rc;
  const int64_t n = p->ndof;
  if (!H->rh)
    for (T** ptr : {&H->rh, &H->v, &H->sv, &H->t, &H->ph, &H->sh})
      if (cudaMallocAsync(ptr, n * sizeof(T), s) != cudaSuccess) return mrg_fail(MRG_ENOMEM, "multigrid BiCGStab vectors");
  rc = follow_j(H, J, setup, s);
  if (rc) return rc;
  set_tail(H, gdata(p)->split);
  GScal init{};
  init.tol = rtol;
  init.maxiter = maxiter;
  MRG_CUDA(cudaMemcpyAsync(H->S, &init, sizeof(GScal), cudaMemcpyHostToDevice, s));
  k_bg_init<T><<<grid_for(n, 16), NT, 0, s>>>(n, b, bgvec(H));
  MRG_CUDA(cudaGetLastError());
  if (!H->bgraph || H->bgraph_A != (const void*)J || H->bgraph_stream != s || H->bgraph_tail != H->tail) {
    if (H->bgraph) {
      cudaGraphExecDestroy(H->bgraph);
      H->bgraph = nullptr;
    }
    cudaStream_t cs = nullptr;
    MRG_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      enqueue_bg_iters(H, GCHUNK, cs);
      e = cudaStreamEndCapture(cs, &graph);
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&H->bgraph, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    cudaStreamDestroy(cs);
    if (e != cudaSuccess) return mrg_cuda_check(e, "multigrid BiCGStab graph capture");
    H->bgraph_A = J;
    H->bgraph_stream = s;
    H->bgraph_tail = H->tail;
  }
  return finish_solve(p, H, H->bgraph, x, rtol, maxiter, st, s, "multigrid BiCGStab");
}

}  // namespace

int mrg_gmg_kind(const mrg_problem* p) {
  return p->gmg ? reinterpret_cast<const GmgData*>(p->gmg)->kind : MRG_PREC_JACOBI;
}

void mrg_gmg_drop_hierarchy(mrg_problem* p) {
  GmgData* G = reinterpret_cast<GmgData*>(p->gmg);
  if (!G) return;
  free_hier(G->h64, p->stream);
  free_hier(G->h32, p->stream);
  G->h64 = nullptr;
  G->h32 = nullptr;
}

void mrg_gmg_free(mrg_problem* p) {
  GmgData* G = reinterpret_cast<GmgData*>(p->gmg);
  if (!G) return;
  free_hier(G->h64, p->stream);
  free_hier(G->h32, p->stream);
  delete G;
  p->gmg = nullptr;
}

// Solves J x = b (x0 = 0) with multigrid-preconditioned CG in the precision of J; x receives the FP64
// solution.
int mrg_gmg_solve(mrg_problem* p, const void* J, bool fp32, const double* b, double* x, double rtol, int maxiter,
                  mrg_solve_stats* st, int setup, cudaStream_t s) {
  if (p->g.p > 2) return mrg_fail(MRG_ENOTSUP, "multigrid: Q1 and Q2 problems only");
  GmgData* G = gdata(p);
  int rc;
  if (fp32) {
    if (!G->h32 && (rc = build_hier<float>(p, G->h32, s))) return rc;
    return gmg_cg<float>(p, G->h32, (const float*)J, b, x, rtol, maxiter, st, setup, s);
  }
  if (!G->h64 && (rc = build_hier<double>(p, G->h64, s))) return rc;
  return gmg_cg<double>(p, G->h64, (const double*)J, b, x, rtol, maxiter, st, setup, s);
}

// Same for a nonsymmetric J: right-preconditioned BiCGStab with the multigrid V-cycle.
int mrg_gmg_bicgstab(mrg_problem* p, const void* J, bool fp32, const double* b, double* x, double rtol, int maxiter,
                     mrg_solve_stats* st, int setup, cudaStream_t s) {
  if (p->g.p > 2) return mrg_fail(MRG_ENOTSUP, "multigrid: Q1 and Q2 problems only");
  GmgData* G = gdata(p);
  int rc;
  if (fp32) {
    if (!G->h32 && (rc = build_hier<float>(p, G->h32, s))) return rc;
    return gmg_bicgstab<float>(p, G->h32, (const float*)J, b, x, rtol, maxiter, st, setup, s);
  }
  if (!G->h64 && (rc = build_hier<double>(p, G->h64, s))) return rc;
  return gmg_bicgstab<double>(p, G->h64, (const double*)J, b, x, rtol, maxiter, st, setup, s);
}

extern "C" int mrg_set_preconditioner(mrg_problem* p, int32_t kind) {
  if (!p) return mrg_fail(MRG_EINVAL, "mrg_set_preconditioner: null problem");
  if (kind != MRG_PREC_JACOBI && kind != MRG_PREC_GMG && kind != MRG_PREC_GMG_SPLIT)
    return mrg_fail(MRG_EINVAL, "mrg_set_preconditioner: unknown preconditioner");
  if (kind != MRG_PREC_JACOBI && p->g.p > 2)
    return mrg_fail(MRG_ENOTSUP, "multigrid preconditioner: Q1 and Q2 problems only");
  gdata(p)->kind = (kind == MRG_PREC_GMG_SPLIT) ? MRG_PREC_GMG : kind;
  gdata(p)->split = (kind == MRG_PREC_GMG_SPLIT);
  return MRG_OK;
}
