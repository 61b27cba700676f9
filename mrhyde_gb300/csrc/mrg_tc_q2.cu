// Q2 Jacobian element contractions on the 5th-generation tensor cores (tcgen05, kind::tf32, 3xTF32).
//
// The row-gather Jacobian of the tensor-product path (mrg_assemble_q2.cu) is, for every (CSR row, cell)
// pair m, one row of the product  D = A * B  with
//     A[m][k]  = alpha_{d,q} = G_d[q][l] s_d^2 cw_q        (k = 27 d + q < 81)
//              = beta_q      = sum_d G_d[q][l] ew_{q,d}      (k = 81 + q)
//     B[k][j]  = [G_x; G_y; G_z; Phi][k][j]                  (constant, 108 x 27)
// (l = local index of the row's node in the cell).  A CTA owns 32 consecutive CSR rows, enumerates their
// (row, cell) pairs in a fixed order, builds A for up to 128 pairs at a time in shared memory, and one
// thread issues tcgen05.mma (M = 128, N = 32, K = 8 per instruction, 14 K steps) into a 32-column TMEM
// accumulator.  Each operand is split x = hi + lo with hi = x rounded to TF32, and D accumulates
// A_hi B_hi + A_hi B_lo + A_lo B_hi in FP32 (3xTF32: ~2^-21 relative per product, i.e. FP32-class).
// The accumulator rows are read back with tcgen05.ld (warp w owns TMEM lanes 32w..32w+31 = pairs),
// parked in shared memory, and each row's pairs are summed in a fixed order into the CTA's staged CSR
// segment, which is written once with 16-byte stores.  The wait on the MMA completion mbarrier is
// bounded; on time-out the kernel records an error, frees its TMEM and returns.
//
// Operand layout: K-major, no swizzle.  A "core matrix" is 8 rows x 16 bytes (4 TF32 values); core
// matrix (row group i, K chunk c) lives at byte (i * 28 + c) * 128, so the leading-dimension byte offset
// (next core matrix along K) is 128 and the stride-dimension byte offset (next 8-row group) is 28 * 128.
#include <cstdio>

#include "mrg_internal.h"

namespace {

constexpr int TCR = 32;                // CSR rows per work item
constexpr int TCT = 128;               // threads per CTA (= M of one MMA tile)
constexpr int KP = 112;                // K padded to a multiple of 8 (108 used)
constexpr int NP = 32;                 // N padded (27 used)
constexpr int KC = KP / 4;             // core-matrix columns along K
constexpr int A_BYTES = TCT * KP * 4;  // 57344
constexpr int B_BYTES = NP * KP * 4;   // 14336
constexpr int TS = 28;                 // row stride of the plain FP32 table
constexpr int MAXP = 8 * TCR;          // pairs per work item (8 cells per row at most)

// shared-memory layout (bytes)
constexpr int OFF_AHI = 0;
constexpr int OFF_ALO = OFF_AHI + A_BYTES;
constexpr int OFF_BHI = OFF_ALO + A_BYTES;
constexpr int OFF_BLO = OFF_BHI + B_BYTES;
constexpr int OFF_D = OFF_BLO + B_BYTES;              // float [128][28]
constexpr int OFF_TAB = OFF_D + TCT * TS * 4;         // float [108][28]
constexpr int OFF_SEG = OFF_TAB + 108 * TS * 4;       // float [TCR*125 + 4]
constexpr int OFF_PAIR = OFF_SEG + (TCR * 125 + 4) * 4;  // int4 [MAXP]
constexpr int OFF_MISC = OFF_PAIR + MAXP * 16;        // mbarrier (8) + tmem addr (4) + flags
constexpr int TC_SMEM = OFF_MISC + 64;

__device__ __forceinline__ uint32_t su32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// byte offset of (row, k) in the K-major no-swizzle core-matrix tile
__device__ __forceinline__ uint32_t cm_off(int row, int k) {
  return (uint32_t)(((row >> 3) * KC + (k >> 2)) * 128 + (row & 7) * 16 + (k & 3) * 4);
}

__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version for tcgen05; base offset 0, relative LBO, no swizzle
  return d;
}

// kind::tf32 instruction descriptor: D = F32, A = B = TF32, both K-major, N = 32, M = 128
constexpr uint32_t IDESC = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(NP >> 3) << 17) | ((uint32_t)(TCT >> 4) << 24);

// round to the nearest TF32 value (10 explicit mantissa bits); the remainder x - hi is exact in FP32
__device__ __forceinline__ float tf32_hi(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;\n" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

__device__ __forceinline__ void mma_tf32(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(IDESC), "r"(accumulate));
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t mbar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(mbar), "r"(parity)
      : "memory");
  return ok != 0;
}

// bounded wait: ~2^22 polls (well above the few microseconds an MMA batch takes)
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t mbar, uint32_t parity) {
  for (int i = 0; i < (1 << 22); ++i)
    if (mbar_try_wait(mbar, parity)) return true;
  return false;
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

__device__ __forceinline__ int64_t rowptr_at2(const Grid& g, int64_t n, int64_t nrows) {
  if (n >= nrows) return g.T[0] * g.T[1] * g.T[2];
  int ix, iy, iz, a, b, c, d, e, f;
  decompose32(g, n, ix, iy, iz);
  return rowptr2(g, ix, iy, iz, a, b, c, d, e, f);
}

__global__ void __launch_bounds__(TCT, 1) k_q2_jac_tc(Grid g, int64_t nrows, int kind, float sq0, float sq1, float sq2,
                                                      const float* __restrict__ tab_g, const float* __restrict__ qbuf,
                                                      float* __restrict__ J, int ovw, int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char sm[];
  float* Dsm = reinterpret_cast<float*>(sm + OFF_D);
  float* tab = reinterpret_cast<float*>(sm + OFF_TAB);
  float* segbuf = reinterpret_cast<float*>(sm + OFF_SEG);
  int4* pairs = reinterpret_cast<int4*>(sm + OFF_PAIR);
  uint64_t* mbar = reinterpret_cast<uint64_t*>(sm + OFF_MISC);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(sm + OFF_MISC + 8);
  int* s_flag = reinterpret_cast<int*>(sm + OFF_MISC + 12);
  __shared__ int s_off[TCR + 1];
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const float sq[3] = {sq0, sq1, sq2};

  // ---- one-time set-up: tables, B operand (hi/lo), mbarrier, TMEM ----
  for (int k = t; k < 108 * TS; k += TCT) tab[k] = tab_g[k];
  __syncthreads();
  for (int e = t; e < NP * KP; e += TCT) {
    const int j = e / KP, k = e % KP;
    const float v = (j < 27 && k < 108) ? tab[k * TS + j] : 0.0f;
    const float hi = tf32_hi(v);
    *reinterpret_cast<float*>(sm + OFF_BHI + cm_off(j, k)) = hi;
    *reinterpret_cast<float*>(sm + OFF_BLO + cm_off(j, k)) = v - hi;
  }
  if (t == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(su32(mbar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    *s_flag = 0;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 32;\n" ::"r"(su32(tmem_slot))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t dtmem = *tmem_slot;
  uint32_t phase = 0;
  bool failed = false;

  const int64_t nchunks = (nrows + TCR - 1) / TCR;
  for (int64_t ch = blockIdx.x; ch < nchunks && !failed; ch += gridDim.x) {
    const int64_t n0 = ch * TCR;
    const int64_t n1 = (n0 + TCR < nrows) ? n0 + TCR : nrows;
    const int64_t seg0 = rowptr_at2(g, n0, nrows), seg1 = rowptr_at2(g, n1, nrows);
    const int phs = (int)(((uintptr_t)(J + seg0) & 15) / sizeof(float));
    float* sv = segbuf + phs;
    for (int64_t k = t; k < seg1 - seg0; k += TCT) sv[k] = 0.0f;
    // row descriptors (threads 0..TCR-1)
    int64_t rp = 0, diag = 0;
    int lx = 0, ly = 0, lz = 0, cxn = 0, cyn = 0, czn = 0, fx = 0, fy = 0, fz = 0, nxc = 0, nyc = 0, nzc = 0;
    int ix = 0, iy = 0, iz = 0, npair = 0;
    bool fixed = false, act = false;
    if (t < TCR) {
      const int64_t n = n0 + t;
      act = n < nrows;
      if (act) {
        decompose32(g, n, ix, iy, iz);
        rp = rowptr2(g, ix, iy, iz, lx, ly, lz, cxn, cyn, czn);
        diag = ((int64_t)(iz - lz) * cyn + (iy - ly)) * cxn + (ix - lx);
        fixed = node_fixed(g, ix, iy, iz);
        if (!fixed) {
          axis_cells(ix, g.nn[0], 2, fx, nxc);
          axis_cells(iy, g.nn[1], 2, fy, nyc);
          axis_cells(iz, g.nn[2], 2, fz, nzc);
          npair = nxc * nyc * nzc;
        }
      }
      // exclusive scan of the pair counts over warp 0
      int incl = npair;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
      }
      s_off[t] = incl - npair;
      if (t == TCR - 1) s_off[TCR] = incl;
    }
    __syncthreads();
    if (t < TCR && npair) {
      int m = s_off[t];
      for (int ccz = fz; ccz < fz + nzc; ++ccz)
        for (int ccy = fy; ccy < fy + nyc; ++ccy)
          for (int ccx = fx; ccx < fx + nxc; ++ccx) {
            const int l = (ix - 2 * ccx) + 3 * (iy - 2 * ccy) + 9 * (iz - 2 * ccz);
            const int cid = ccx + g.nc[0] * (ccy + g.nc[1] * ccz);
            pairs[m++] = make_int4(t, cid, l, ccx | (ccy << 10) | (ccz << 20));
          }
    }
    __syncthreads();
    const int ptotal = s_off[TCR];
    for (int base = 0; base < ptotal; base += TCT) {
      // ---- build A rows (hi/lo) for pairs base..base+127 ----
      const int m = base + t;
      if (m < ptotal) {
        const int4 pr = pairs[m];
        const int l = pr.z;
        const float* qb = qbuf + (int64_t)pr.y * 108;
        for (int k = 0; k < KP; ++k) {
          float v = 0.0f;
          if (k < 81) {
            const int d = k / 27, q = k % 27;
            v = tab[k * TS + l] * sq[d] * __ldg(qb + q);
          } else if (k < 108 && kind != MRG_THERMAL) {
            const int q = k - 81;
            v = tab[q * TS + l] * __ldg(qb + 27 + q) + tab[(27 + q) * TS + l] * __ldg(qb + 54 + q) +
                tab[(54 + q) * TS + l] * __ldg(qb + 81 + q);
          }
          const float hi = tf32_hi(v);
          *reinterpret_cast<float*>(sm + OFF_AHI + cm_off(t, k)) = hi;
          *reinterpret_cast<float*>(sm + OFF_ALO + cm_off(t, k)) = v - hi;
        }
      } else {
        for (int k = 0; k < KP; ++k) {
          *reinterpret_cast<float*>(sm + OFF_AHI + cm_off(t, k)) = 0.0f;
          *reinterpret_cast<float*>(sm + OFF_ALO + cm_off(t, k)) = 0.0f;
        }
      }
      asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
      __syncthreads();
      // ---- one thread issues the 3xTF32 MMAs ----
      if (t == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        const uint32_t ahi = su32(sm + OFF_AHI), alo = su32(sm + OFF_ALO);
        const uint32_t bhi = su32(sm + OFF_BHI), blo = su32(sm + OFF_BLO);
        for (int ks = 0; ks < KP / 8; ++ks) {
          const uint32_t koff = (uint32_t)ks * 256u;  // two core-matrix columns per K step
          const uint64_t dAh = smem_desc(ahi + koff, 128, KC * 128), dAl = smem_desc(alo + koff, 128, KC * 128);
          const uint64_t dBh = smem_desc(bhi + koff, 128, KC * 128), dBl = smem_desc(blo + koff, 128, KC * 128);
          mma_tf32(dtmem, dAh, dBh, ks > 0 ? 1u : 0u);
          mma_tf32(dtmem, dAh, dBl, 1u);
          mma_tf32(dtmem, dAl, dBh, 1u);
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(su32(mbar))
                     : "memory");
      }
      if (!mbar_wait_bounded(su32(mbar), phase)) atomicExch(s_flag, 1);
      phase ^= 1u;
      __syncthreads();
      if (*s_flag) {
        failed = true;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      // ---- accumulator rows back to registers (warp w: TMEM lanes 32w..32w+31) ----
      uint32_t r[32];
      const uint32_t taddr = dtmem + ((uint32_t)(warp * 32) << 16);
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
          "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
            "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
            "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
          : "r"(taddr)
          : "memory");
      asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
      for (int j = 0; j < 27; ++j) Dsm[t * TS + j] = __uint_as_float(r[j]);
      asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
      __syncthreads();
      // ---- each row sums its pairs of this tile in order into its staged CSR row ----
      if (t < TCR && act && !fixed) {
        const int p0 = max(s_off[t], base), p1 = min(s_off[t + 1], base + TCT);
        float* row = sv + (rp - seg0);
        for (int pm = p0; pm < p1; ++pm) {
          const int4 pr = pairs[pm];
          const int ccx = pr.w & 1023, ccy = (pr.w >> 10) & 1023, ccz = pr.w >> 20;
          const float* dr = Dsm + (pm - base) * TS;
#pragma unroll
          for (int j = 0; j < 27; ++j) {
            const int jx = 2 * ccx + j % 3, jy = 2 * ccy + (j / 3) % 3, jz = 2 * ccz + j / 9;
            row[((int64_t)(jz - lz) * cyn + (jy - ly)) * cxn + (jx - lx)] += dr[j];
          }
        }
      }
      __syncthreads();
    }
    if (failed) break;
    if (t < TCR && act && fixed && ovw) sv[(rp - seg0) + diag] = 1.0f;
    __syncthreads();
    // ---- write the segment once (16-byte stores), or add into it ----
    {
      float* dst = J + seg0;
      const int64_t len = seg1 - seg0;
      int head = (int)(((16 - ((uintptr_t)dst & 15)) & 15) / 4);
      if (head > len) head = (int)len;
      for (int k = t; k < head; k += TCT) dst[k] = ovw ? sv[k] : dst[k] + sv[k];
      const int64_t body = (len - head) / 4;
      const float4* s4 = reinterpret_cast<const float4*>(sv + head);
      float4* d4 = reinterpret_cast<float4*>(dst + head);
      for (int64_t v = t; v < body; v += TCT) {
        float4 x = s4[v];
        if (!ovw) {
          const float4 y = d4[v];
          x.x += y.x; x.y += y.y; x.z += y.z; x.w += y.w;
        }
        __stcs(d4 + v, x);
      }
      for (int64_t k = head + body * 4 + t; k < len; k += TCT) dst[k] = ovw ? sv[k] : dst[k] + sv[k];
    }
    if (!ovw) {
      __syncthreads();
      if (t < TCR && act && fixed) J[rp + diag] = 1.0f;
    }
    __syncthreads();
  }
  if (failed && t == 0) atomicExch(err, 1);
  // ---- release TMEM ----
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 32;\n" ::"r"(dtmem) : "memory");
  }
}

}  // namespace

// Launches the tensor-core Jacobian for a Q2 problem.  tab32 = [G_x | G_y | G_z | Phi] rows of 28 floats,
// qbuf = per-cell FP32 coefficients (cw, ew) written by the residual pass, err = device int (0 on entry).
int mrg_launch_q2_jac_tc(const mrg_problem* p, const float* tab32, const float* qbuf, float* J, bool ovw, int* err,
                         double s0, double s1, double s2, cudaStream_t s) {
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k_q2_jac_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM);
    if (e != cudaSuccess) return mrg_cuda_check(e, "tensor-core Jacobian smem attribute");
    attr = true;
  }
  int dev = 0, nsm = 0;
  MRG_CUDA(cudaGetDevice(&dev));
  MRG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const int64_t nchunks = (p->ndof + TCR - 1) / TCR;
  const int grid = (int)((nchunks < nsm) ? nchunks : nsm);
  k_q2_jac_tc<<<grid, TCT, TC_SMEM, s>>>(p->g, p->ndof, p->kind, (float)(s0 * s0), (float)(s1 * s1), (float)(s2 * s2),
                                         tab32, qbuf, J, ovw ? 1 : 0, err);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? MRG_OK : mrg_cuda_check(e, "tensor-core Jacobian launch");
}

int mrg_tc_smem_bytes() { return TC_SMEM; }
