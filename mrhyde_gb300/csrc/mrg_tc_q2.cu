// Q2 element matrices on the 5th-generation tensor cores (tcgen05.mma kind::tf32, 3xTF32, operands
// brought in by TMA, accumulators in TMEM, results written by TMA), then their deterministic row-gather
// assembly into the CSR Jacobian.
//
// For one cell c of the tensor-product Q2 form (reference: src/physics/thermal.cpp:71-165 volume
// residual, differentiated by the workset AD types of assemblyManager_jacres.hpp:121-630) the element
// Jacobian is
//     K_c[l][j] = sum_q cw_q sum_d s_d^2 G_d[q][l] G_d[q][j]  +  sum_{d,q} ew_{q,d} G_d[q][l] Phi[q][j]
// with per-point coefficients W_c = (cw_q | ew_{q,x} | ew_{q,y} | ew_{q,z}) (108 values, written by the
// residual pass; the ew block is zero for the linear thermal form) and the constant reference tables G_d
// (gradients) and Phi (values).  All element matrices together are ONE GEMM with a constant right operand:
//     E (ncell x 768) = W (ncell x K) * H (K x 768),   H[k][28 l + j] = the products above,
// K = 108 (nonlinear) or 27 (thermal), the 27 x 27 element matrix stored with rows padded to 28 so that
// each row starts on 16 bytes.  The GEMM runs in FP32-class precision as 3xTF32: every operand is split
// x = hi + lo (hi = x rounded to TF32, lo = the rounded remainder) and E = Wh Hh + Wh Hl + Wl Hh.
//
// k_q2_elem_tc is a persistent warp-specialised kernel (one CTA per SM, 6 warps):
//   warp 0  producer: 1-D bulk copies (cp.async.bulk) of the 128-cell W tile (hi and lo planes) and of
//           256-column slices of H in a 5-stage ring (K = 8 per stage).  Both operands are kept in global
//           memory as the exact shared-memory image of the K-major no-swizzle core-matrix layout (the
//           residual pass writes W that way; H is a constant built on the host), so each copy is one
//           contiguous transfer instead of hundreds of 16-byte rows;
//   warp 1  owns TMEM (512 columns = two 128 x 256 FP32 accumulators) and issues tcgen05.mma from one
//           thread: per 256-column slice, K/8 steps x 3 products, then tcgen05.commit to the mbarriers
//           that release the H stage, hand the accumulator to the epilogue and release the W tile;
//   warps 2-5 epilogue: tcgen05.ld (warp w reads TMEM lanes 32 (w % 4) ..), stage 32 x 32 values in a
//           128-byte-swizzled shared buffer (conflict-free) and write them with a TMA tensor store.
// Every mbarrier wait is bounded by the global timer; on time-out the kernel raises a shared abort flag,
// every role leaves its loop, waits (bounded) for its own copies and MMAs in flight, TMEM is freed and the
// status word is set, so the host reports MRG_ETIMEOUT instead of hanging.
//
// k_q2_gather: one warp per CSR row, one lane per local column, 32 consecutive rows per warp with the row
// set-up computed lane-parallel: J(i,j) = sum over the cells that contain both nodes (fixed order cz, cy,
// cx) of E_c[l_i][l_j].  Every element-matrix value is read exactly once and
// every Jacobian value is written exactly once, coalesced; no atomics, so the result is deterministic.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "mrg_device.cuh"
#include "mrg_internal.h"

namespace {

constexpr int TM = 128;           // cells per tile = MMA M
constexpr int NE = 768;           // element-matrix columns (27 rows x 28 + 12 zero columns)
constexpr int NCH = 256;          // columns per accumulator = MMA N
constexpr int NNCH = NE / NCH;    // 3 accumulator slices per tile
constexpr int KH = 112;           // H^T row length (K padded to a multiple of 8)
constexpr int KW = 108;           // W row length in global memory
// H stages (K = 8 each) and epilogue staging buffers per epilogue warp
#ifndef MRG_TC_NBS
#define MRG_TC_NBS 6
#endif
#ifndef MRG_TC_EBUFS
#define MRG_TC_EBUFS 1
#endif
constexpr int NBS = MRG_TC_NBS;
constexpr int EBUFS = MRG_TC_EBUFS;
constexpr int A_PLANE = TM * KH * 4;          // 57344 bytes per W plane (hi or lo)
constexpr int B_PLANE = NCH * 8 * 4;          // 8192 bytes per H plane per stage
constexpr int B_STAGE = 2 * B_PLANE;          // hi + lo
constexpr int E_BUF = 32 * 32 * 4;            // one epilogue staging buffer (32 cells x 32 columns)
constexpr int THREADS = 192;
constexpr int KSTEPS_MAX = KH / 8;            // 14
constexpr int W_TILE_FLOATS = 2 * TM * KH;    // hi plane then lo plane of one 128-cell tile
constexpr int H_STAGE_FLOATS = B_STAGE / 4;   // one (slice, K step) stage of H: hi chunks 0,1 then lo

constexpr int OFF_AH = 0;
constexpr int OFF_AL = OFF_AH + A_PLANE;
constexpr int OFF_B = OFF_AL + A_PLANE;                 // NBS stages of [hi | lo]
constexpr int OFF_E = OFF_B + NBS * B_STAGE;            // 4 warps x EBUFS buffers (1024-byte aligned)
constexpr int OFF_BAR = OFF_E + 4 * EBUFS * E_BUF;
// barriers: a_full[K steps], a_empty[K steps] (one per 8-wide K chunk of the W tile, so the next tile's W
// streams in while the last slice of the current tile still uses the later chunks), b_full[NBS],
// b_empty[NBS], t_full[2], t_empty[2], spare
constexpr int KS = KH / 8;
constexpr int BAR_A_FULL = 0, BAR_A_EMPTY = KS, BAR_B_FULL = 2 * KS, BAR_B_EMPTY = 2 * KS + NBS,
              BAR_T_FULL = 2 * KS + 2 * NBS, BAR_T_EMPTY = 2 * KS + 2 * NBS + 2, BAR_SPARE = 2 * KS + 2 * NBS + 4,
              NBAR = 2 * KS + 2 * NBS + 5;
constexpr int A_CHUNK = 2 * TM * 16;          // bytes of one K step (8 values) of one W plane
constexpr int OFF_MISC = OFF_BAR + NBAR * 8;            // tmem address (4) + abort flag (4)
constexpr int SMEM_USED = OFF_MISC + 16;
constexpr int SMEM_BYTES = SMEM_USED + 1024;            // slack for aligning the base to 1024 bytes
static_assert(OFF_E % 1024 == 0, "swizzled staging buffers need 1024-byte alignment");
static_assert(SMEM_BYTES <= 232448, "shared memory budget");

// kind::tf32 instruction descriptor: D = F32, A = B = TF32, both K-major, N = 256, M = 128
constexpr uint32_t IDESC = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(NCH >> 3) << 17) | ((uint32_t)(TM >> 4) << 24);

constexpr unsigned long long WAIT_NS = 2000000000ull;  // default wait bound, 2 s: far above any legitimate wait

__device__ __forceinline__ uint64_t gtimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
  return t;
}

__device__ __forceinline__ bool mbar_try(uint32_t mbar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(mbar), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait (limit in ns) on an mbarrier phase.  Returns false (and raises the CTA abort flag) on
// time-out, or false when another role has already aborted.
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity, volatile int* abort_flag,
                                          unsigned long long limit) {
  if (mbar_try(mbar, parity)) return true;
  const uint64_t t0 = gtimer();
  for (uint32_t i = 1;; ++i) {
    if (mbar_try(mbar, parity)) return true;
    if ((i & 63u) == 0) {
      if (*abort_flag) return false;
      if (gtimer() - t0 > limit) {
        *abort_flag = 1;
        return false;
      }
    }
  }
}

// wait with a limit only, used while cleaning up after an abort
__device__ __forceinline__ void mbar_wait_cleanup(uint32_t mbar, uint32_t parity) {
  const uint64_t t0 = gtimer();
  while (!mbar_try(mbar, parity))
    if (gtimer() - t0 > 200000000ull) return;
}

__device__ __forceinline__ void mbar_init(uint32_t mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(mbar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t mbar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(mbar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t mbar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(mbar) : "memory");
}

__device__ __forceinline__ void bulk_load(uint32_t dst, const void* src, uint32_t bytes, uint32_t mbar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(dst),
               "l"(reinterpret_cast<uint64_t>(src)), "r"(bytes), "r"(mbar)
               : "memory");
}

__device__ __forceinline__ void tma_store_2d(const CUtensorMap* map, int x, int y, uint32_t src) {
  asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%1, %2}], [%3];\n" ::"l"(
                   reinterpret_cast<uint64_t>(map)),
               "r"(x), "r"(y), "r"(src)
               : "memory");
}

__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;  // tcgen05 descriptor version; base offset 0, relative LBO, no swizzle
  return d;
}

__device__ __forceinline__ void mma_tf32(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(IDESC), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mbar)
               : "memory");
}

__global__ void __launch_bounds__(THREADS, 1)
    k_q2_elem_tc(const float* __restrict__ wimg, const float* __restrict__ himg, const __grid_constant__ CUtensorMap mE,
                 int ntiles, int ksteps, int* __restrict__ err, unsigned long long wait_ns, int withhold) {
  extern __shared__ unsigned char sm_raw[];
  const uint32_t raw = (uint32_t)__cvta_generic_to_shared(sm_raw);
  const uint32_t base = (raw + 1023u) & ~1023u;
  unsigned char* sm = sm_raw + (base - raw);
  const uint32_t sAh = base + OFF_AH, sAl = base + OFF_AL, sB = base + OFF_B, sE = base + OFF_E;
  const uint32_t bar0 = base + OFF_BAR;
  auto bar = [&](int i) { return bar0 + 8u * (uint32_t)i; };
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(sm + OFF_MISC);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(sm + OFF_MISC + 4);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int k = 0; k < KS; ++k) {
      mbar_init(bar(BAR_A_FULL + k), 1);
      mbar_init(bar(BAR_A_EMPTY + k), 1);
    }
    for (int s = 0; s < NBS; ++s) {
      mbar_init(bar(BAR_B_FULL + s), 1);
      mbar_init(bar(BAR_B_EMPTY + s), 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(bar(BAR_T_FULL + b), 1);
      mbar_init(bar(BAR_T_EMPTY + b), 4);
    }
    mbar_init(bar(BAR_SPARE), 1);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    *abort_flag = 0;
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;\n" ::"r"(
                     (uint32_t)__cvta_generic_to_shared(tmem_slot))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  const unsigned long long lim = wait_ns ? wait_ns : WAIT_NS;

  if (warp == 0) {
    // ------------------------------ TMA producer ------------------------------
    if (lane == 0) {
      bool ok = true;
      uint32_t bit = 0, ta = 0;
      int a_armed[KS];
      int b_armed[NBS];
      for (int k = 0; k < KS; ++k) a_armed[k] = -1;
      for (int s = 0; s < NBS; ++s) b_armed[s] = -1;
      for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x, ++ta) {
        const float* wt = wimg + (size_t)tile * W_TILE_FLOATS;
        for (int n = 0; n < NNCH && ok; ++n)
          for (int ks = 0; ks < ksteps; ++ks, ++bit) {
            if (n == 0) {
              // K chunk ks of the tile's W (hi and lo planes), once its previous contents are consumed
              if (!mbar_wait(bar(BAR_A_EMPTY + ks), (ta & 1u) ^ 1u, abort_flag, lim)) { ok = false; break; }
              // withhold (testing): the W copies of tile 0 are never issued, so the MMA thread's wait for
              // them runs out and the abort path is taken with no copy in flight on those barriers
              if (!(withhold && tile == 0)) {
                mbar_expect_tx(bar(BAR_A_FULL + ks), 2u * A_CHUNK);
                a_armed[ks] = (int)(ta & 1u);
                const size_t ko = (size_t)ks * (A_CHUNK / 4);
                bulk_load(sAh + ks * A_CHUNK, wt + ko, A_CHUNK, bar(BAR_A_FULL + ks));
                bulk_load(sAl + ks * A_CHUNK, wt + TM * KH + ko, A_CHUNK, bar(BAR_A_FULL + ks));
              }
            }
            const uint32_t st = bit % NBS, ph = (bit / NBS) & 1u;
            if (!mbar_wait(bar(BAR_B_EMPTY + st), ph ^ 1u, abort_flag, lim)) { ok = false; break; }
            mbar_expect_tx(bar(BAR_B_FULL + st), (uint32_t)B_STAGE);
            b_armed[st] = (int)ph;
            bulk_load(sB + st * B_STAGE, himg + (size_t)(n * KSTEPS_MAX + ks) * H_STAGE_FLOATS, (uint32_t)B_STAGE,
                      bar(BAR_B_FULL + st));
          }
      }
      if (ok) {
        // tail: wait until the MMA thread has released every stage, so that no arrive lands after exit
        for (int s = 0; s < NBS && ok; ++s, ++bit) {
          const uint32_t st = bit % NBS, ph = (bit / NBS) & 1u;
          if (b_armed[st] >= 0 && !mbar_wait(bar(BAR_B_EMPTY + st), ph ^ 1u, abort_flag, lim)) ok = false;
        }
      }
      if (!ok) {
        // copies in flight land on their full barriers: wait for the last phase armed on each
        for (int k = 0; k < KS; ++k)
          if (a_armed[k] >= 0) mbar_wait_cleanup(bar(BAR_A_FULL + k), (uint32_t)a_armed[k]);
        for (int s = 0; s < NBS; ++s)
          if (b_armed[s] >= 0) mbar_wait_cleanup(bar(BAR_B_FULL + s), (uint32_t)b_armed[s]);
      }
    }
    __syncwarp();
  } else if (warp == 1) {
    // ------------------------------ MMA issuer ------------------------------
    if (lane == 0) {
      bool ok = true, issued = false;
      uint32_t bit = 0, acc = 0, ta = 0;
      for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x, ++ta) {
        const bool more = tile + (int)gridDim.x < ntiles;
        for (int n = 0; n < NNCH && ok; ++n, ++acc) {
          const uint32_t buf = acc & 1u, aph = (acc >> 1) & 1u;
          if (!mbar_wait(bar(BAR_T_EMPTY + buf), aph ^ 1u, abort_flag, lim)) { ok = false; break; }
          asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
          const uint32_t d = tmem + buf * NCH;
          for (int ks = 0; ks < ksteps; ++ks, ++bit) {
            if (n == 0 && !mbar_wait(bar(BAR_A_FULL + ks), ta & 1u, abort_flag, lim)) { ok = false; break; }
            const uint32_t st = bit % NBS, ph = (bit / NBS) & 1u;
            if (!mbar_wait(bar(BAR_B_FULL + st), ph, abort_flag, lim)) { ok = false; break; }
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const uint32_t bh = sB + st * B_STAGE, bl = bh + B_PLANE;
            const uint32_t koff = (uint32_t)ks * 2u * (TM * 16);
            const uint64_t dAh = smem_desc(sAh + koff, TM * 16, 128), dAl = smem_desc(sAl + koff, TM * 16, 128);
            const uint64_t dBh = smem_desc(bh, NCH * 16, 128), dBl = smem_desc(bl, NCH * 16, 128);
            mma_tf32(d, dAh, dBh, ks > 0 ? 1u : 0u);
            mma_tf32(d, dAh, dBl, 1u);
            mma_tf32(d, dAl, dBh, 1u);
            issued = true;
            mma_commit(bar(BAR_B_EMPTY + st));
            // after the last slice's use of W chunk ks, release it for the CTA's next tile
            if (n == NNCH - 1 && more) mma_commit(bar(BAR_A_EMPTY + ks));
          }
          if (ok) mma_commit(bar(BAR_T_FULL + buf));
        }
      }
      if (!ok && issued) {
        // let the MMAs already issued finish before TMEM is released
        mma_commit(bar(BAR_SPARE));
        mbar_wait_cleanup(bar(BAR_SPARE), 0u);
      }
    }
    __syncwarp();
  } else {
    // ------------------------------ epilogue (warps 2..5) ------------------------------
    const int q = warp & 3;           // TMEM lane quarter this warp may access
    const int ew = warp - 2;          // staging buffers of this warp
    const uint32_t stg0 = sE + (uint32_t)ew * (uint32_t)EBUFS * E_BUF;
    bool ok = true;
    uint32_t acc = 0, piece = 0;
    for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
      const int row0 = tile * TM + 32 * q;
      for (int n = 0; n < NNCH; ++n, ++acc) {
        const uint32_t buf = acc & 1u, aph = (acc >> 1) & 1u;
        int good = 1;
        if (lane == 0) good = mbar_wait(bar(BAR_T_FULL + buf), aph, abort_flag, lim) ? 1 : 0;
        good = __shfl_sync(0xffffffffu, good, 0);
        if (!good) { ok = false; break; }
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        for (int p = 0; p < NCH / 32; ++p, ++piece) {
          uint32_t r[32];
          const uint32_t taddr = tmem + ((uint32_t)(32 * q) << 16) + buf * NCH + 32u * (uint32_t)p;
          asm volatile(
              "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
              "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
              : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
                "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
                "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
              : "r"(taddr)
              : "memory");
          asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
          const uint32_t stg = stg0 + (piece % (uint32_t)EBUFS) * E_BUF;
          // the store issued from this buffer EBUFS pieces ago must have finished reading it
          if (lane == 0) {
            if constexpr (EBUFS == 2) asm volatile("cp.async.bulk.wait_group.read 1;\n" ::: "memory");
            else asm volatile("cp.async.bulk.wait_group.read 0;\n" ::: "memory");
          }
          __syncwarp();
          // row = lane (128 bytes); 16-byte chunk c goes to chunk position c ^ (row & 7) (128B swizzle)
#pragma unroll
          for (int c = 0; c < 8; ++c) {
            const uint32_t a = stg + (uint32_t)lane * 128u + (uint32_t)((c ^ (lane & 7)) << 4);
            asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};\n" ::"r"(a), "r"(r[4 * c]), "r"(r[4 * c + 1]),
                         "r"(r[4 * c + 2]), "r"(r[4 * c + 3])
                         : "memory");
          }
          asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
          __syncwarp();
          if (lane == 0) {
            tma_store_2d(&mE, n * NCH + 32 * p, row0, stg);
            asm volatile("cp.async.bulk.commit_group;\n" ::: "memory");
          }
        }
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
        __syncwarp();
        if (lane == 0) mbar_arrive(bar(BAR_T_EMPTY + buf));
      }
    }
    if (lane == 0) asm volatile("cp.async.bulk.wait_group 0;\n" ::: "memory");
    __syncwarp();
  }

  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (threadIdx.x == 0 && *abort_flag) atomicExch(err, 1);
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;\n" ::"r"(tmem) : "memory");
  }
}

constexpr int GT = 256;   // gather threads per CTA
constexpr int GRUN = 32;  // consecutive rows a warp takes at a time (one row set-up per lane)

// Row-gather of one CSR row from its NX x NY x NZ boundary-cell block (NX, NY, NZ in {1, 2}).  Lane l < 27
// stands for local column node l of a cell: for each of the row's cells (fixed order cz, cy, cx) it loads
// E_c[l_i][l] -- a contiguous run of 27 values -- and adds it to the row's entry of that column in the
// warp's shared row.  All loads of the row are issued before the first add; the adds are ordered by cell,
// so every entry is summed in the same fixed order on every run.  The row is then written once,
// coalesced.
template <int NX, int NY, int NZ>
__device__ __forceinline__ void gather_cells(float* __restrict__ rb, const float* __restrict__ e0, int sy, int sz,
                                             int li0, int pos0, int cy, int cx, bool col, int lane) {
  constexpr int NC = NX * NY * NZ;
  float v[NC];
#pragma unroll
  for (int k = 0; k < NC; ++k) {
    const int kx = k % NX, ky = (k / NX) % NY, kz = k / (NX * NY);
    const int li = li0 - 2 * (kx + 3 * ky + 9 * kz);
    v[k] = col ? __ldg(e0 + kx * NE + ky * sy + kz * sz + li * 28) : 0.0f;
  }
#pragma unroll
  for (int k = 0; k < NC; ++k) {
    const int kx = k % NX, ky = (k / NX) % NY, kz = k / (NX * NY);
    if (col) rb[pos0 + 2 * ((kz * cy + ky) * cx + kx)] += v[k];
    __syncwarp();
  }
}

// One warp per CSR row, 32 consecutive rows at a time.  The row set-up (coordinates, row pointer, the
// row's cell block) is computed by lane k for row r0 + k, all 32 at once, and handed to the warp row by
// row with four shuffles: set-up that every lane used to repeat for every row was most of the kernel's
// instructions.  A Q2 row's column range along an axis starts at the lowest node of its first cell, so a
// lane's column position in the row depends only on the row's extents (cx, cy).
// 8 CTAs per SM (64 warps) by measurement: the kernel waits on memory latency, so occupancy pays more
// than the 32-register cap costs (40 bytes of spills): C3 Jacobian 0.918 (no floor, 48 registers) ->
// 0.877 (6 CTAs) -> 0.822 ms; two rows' loads in flight per warp at 62 registers was slower
__global__ void __launch_bounds__(GT, 8) k_q2_gather(Grid g, int64_t nrows, const float* __restrict__ E,
                                                  float* __restrict__ J, int ovw) {
  __shared__ float rows[GT / 32][128];
  const int lane = threadIdx.x & 31;
  float* rb = rows[threadIdx.x >> 5];
  const int64_t wid = ((int64_t)blockIdx.x * GT + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * GT) >> 5;
  const int ncx = g.nc[0], ncy = g.nc[1];
  const int sy = ncx * NE, sz = ncx * ncy * NE;  // cell strides (host checks they fit in 32 bits)
  const bool col = lane < 27;
  const int ljx = lane % 3, ljy = (lane / 3) % 3, ljz = lane / 9;
  for (int64_t r0 = wid * GRUN; r0 < nrows; r0 += nw * GRUN) {
    // ---- this lane's row r0 + lane: packed set-up
    // word: cx | cy << 3 | cz << 6 | cell pattern << 9 | fixed << 12 | (local row, or diagonal position) << 13
    uint32_t word = 0, cell = 0;
    int64_t rp = 0;
    if (r0 + lane < nrows) {
      int ix, iy, iz;
      mrgdev::decompose(g, r0 + lane, ix, iy, iz);
      const mrgdev::RowInfo R = mrgdev::row_info<2>(g, ix, iy, iz);
      rp = R.rp;
      word = (uint32_t)R.cx | ((uint32_t)R.cy << 3) | ((uint32_t)R.cz << 6);
      if (node_fixed(g, ix, iy, iz)) {
        word |= (1u << 12) | ((uint32_t)(mrgdev::diag_pos(R, ix, iy, iz) - R.rp) << 13);
      } else {
        int fx, fy, fz, nxc, nyc, nzc;
        axis_cells(ix, g.nn[0], 2, fx, nxc);
        axis_cells(iy, g.nn[1], 2, fy, nyc);
        axis_cells(iz, g.nn[2], 2, fz, nzc);
        const int li0 = (ix - 2 * fx) + 3 * (iy - 2 * fy) + 9 * (iz - 2 * fz);
        word |= ((uint32_t)((nxc - 1) | ((nyc - 1) << 1) | ((nzc - 1) << 2)) << 9) | ((uint32_t)li0 << 13);
        cell = (uint32_t)(fx + ncx * (fy + ncy * fz));
      }
    }
    const int nrun = (int)((nrows - r0 < GRUN) ? nrows - r0 : GRUN);
    for (int k = 0; k < nrun; ++k) {
      const uint32_t w = __shfl_sync(0xffffffffu, word, k);
      const uint32_t rlo = __shfl_sync(0xffffffffu, (uint32_t)rp, k);
      const uint32_t rhi = __shfl_sync(0xffffffffu, (uint32_t)((uint64_t)rp >> 32), k);
      const uint32_t c = __shfl_sync(0xffffffffu, cell, k);
      const int cx = (int)(w & 7u), cy = (int)((w >> 3) & 7u), cz = (int)((w >> 6) & 7u);
      const int len = cx * cy * cz;
      const int idx = (int)(w >> 13);
      float* row = J + (int64_t)(((uint64_t)rhi << 32) | rlo);
      if (w & (1u << 12)) {
        if (ovw) {
          for (int e = lane; e < len; e += 32) __stcs(row + e, e == idx ? 1.0f : 0.0f);
        } else if (lane == 0) {
          row[idx] = 1.0f;
        }
      } else {
        const int pos0 = (ljz * cy + ljy) * cx + ljx;
        const float* e0 = E + (int64_t)c * NE + lane;
        for (int e = lane; e < len; e += 32) rb[e] = 0.0f;
        __syncwarp();
        switch ((w >> 9) & 7u) {
          case 0: gather_cells<1, 1, 1>(rb, e0, sy, sz, idx, pos0, cy, cx, col, lane); break;
          case 1: gather_cells<2, 1, 1>(rb, e0, sy, sz, idx, pos0, cy, cx, col, lane); break;
          case 2: gather_cells<1, 2, 1>(rb, e0, sy, sz, idx, pos0, cy, cx, col, lane); break;
          case 3: gather_cells<2, 2, 1>(rb, e0, sy, sz, idx, pos0, cy, cx, col, lane); break;
          case 4: gather_cells<1, 1, 2>(rb, e0, sy, sz, idx, pos0, cy, cx, col, lane); break;
          case 5: gather_cells<2, 1, 2>(rb, e0, sy, sz, idx, pos0, cy, cx, col, lane); break;
          case 6: gather_cells<1, 2, 2>(rb, e0, sy, sz, idx, pos0, cy, cx, col, lane); break;
          default: gather_cells<2, 2, 2>(rb, e0, sy, sz, idx, pos0, cy, cx, col, lane); break;
        }
        for (int e = lane; e < len; e += 32) {
          if (ovw) __stcs(row + e, rb[e]); else row[e] += rb[e];
        }
        __syncwarp();
      }
    }
  }
}

// ---------------------------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------------------------
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
  });
  return fn;
}

int make_map(CUtensorMap* m, const void* gaddr, uint64_t inner, uint64_t outer, uint64_t row_bytes, uint32_t box_in,
             uint32_t box_out, CUtensorMapSwizzle sw) {
  PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn();
  if (!fn) return mrg_fail(MRG_ECUDA, "cuTensorMapEncodeTiled entry point not available");
  const cuuint64_t dims[2] = {inner, outer};
  const cuuint64_t strides[1] = {row_bytes};
  const cuuint32_t box[2] = {box_in, box_out};
  const cuuint32_t es[2] = {1, 1};
  CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void*>(gaddr), dims, strides, box, es,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, sw, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    char b[160];
    snprintf(b, sizeof b, "cuTensorMapEncodeTiled failed (%d) for a %llu x %llu map", (int)r,
             (unsigned long long)inner, (unsigned long long)outer);
    return mrg_fail(MRG_ECUDA, b);
  }
  return MRG_OK;
}

// TF32 with round-to-nearest (ties away from zero), host side: 10 explicit mantissa bits
float tf32_round_host(float x) {
  uint32_t u;
  memcpy(&u, &x, 4);
  if ((u & 0x7f800000u) != 0x7f800000u) u = (u + 0x1000u) & 0xffffe000u;
  float y;
  memcpy(&y, &u, 4);
  return y;
}

}  // namespace

struct Q2Tc {
  CUtensorMap mE;
  float* d_w = nullptr;   // W image: [tile][hi, lo][K chunk 28][cell 128][4]
  float* d_h = nullptr;   // H image: [slice 3][K step 14][hi, lo][K chunk 2][column 256][4]
  float* d_e = nullptr;   // [ntiles * 128][768] element matrices
  int ntiles = 0, ksteps = 0;
};

// Builds H^T (hi/lo) from the reference tables tab[(d*27 + q)*28 + j] (d = 0..2 gradients, 3 = values)
// and the axis scalings s[d] = 2 / h_d, allocates the coefficient and element buffers and encodes the
// tensor maps.  W is written by the residual pass into q2tc_w_planes().
int mrg_q2tc_create(mrg_problem* p, const double* tab, const double s[3], Q2Tc** out, cudaStream_t st) {
  Q2Tc* T = new Q2Tc();
  const bool thermal = p->kind == MRG_THERMAL;
  T->ntiles = (int)((p->ncell + TM - 1) / TM);
  T->ksteps = thermal ? 4 : KH / 8;
  std::vector<float> h((size_t)NNCH * KSTEPS_MAX * H_STAGE_FLOATS, 0.0f);
  // position of H^T[n][k] (plane 0 = hi, 1 = lo) in the stage image
  auto at = [&](int n, int k, int plane) {
    const int sl = n / NCH, col = n % NCH, ks = k / 8, c = (k % 8) / 4;
    return (size_t)(sl * KSTEPS_MAX + ks) * H_STAGE_FLOATS + (size_t)plane * (B_PLANE / 4) + (size_t)c * NCH * 4 +
           (size_t)col * 4 + (size_t)(k % 4);
  };
  auto G = [&](int d, int q, int j) { return tab[(d * 27 + q) * 28 + j]; };
  for (int l = 0; l < 27; ++l)
    for (int j = 0; j < 27; ++j) {
      const int n = 28 * l + j;
      for (int k = 0; k < KW; ++k) {
        double v;
        if (k < 27) {
          v = 0.0;
          for (int d = 0; d < 3; ++d) v += s[d] * s[d] * G(d, k, l) * G(d, k, j);
        } else {
          const int d = (k - 27) / 27, q = (k - 27) % 27;
          v = G(d, q, l) * G(3, q, j);
        }
        const float hi = tf32_round_host((float)v);
        h[at(n, k, 0)] = hi;
        h[at(n, k, 1)] = tf32_round_host((float)(v - (double)hi));
      }
    }
  auto fail = [&](int rc) {
    if (T->d_w) cudaFreeAsync(T->d_w, st);
    if (T->d_h) cudaFreeAsync(T->d_h, st);
    if (T->d_e) cudaFreeAsync(T->d_e, st);
    delete T;
    return rc;
  };
  const size_t wbytes = (size_t)T->ntiles * W_TILE_FLOATS * sizeof(float);
  cudaError_t e = cudaMallocAsync(&T->d_w, wbytes, st);
  // slots never written by the residual pass (K padding, the ew block of the thermal form, cells past
  // the end of the last tile) must read as zero
  if (e == cudaSuccess) e = cudaMemsetAsync(T->d_w, 0, wbytes, st);
  if (e == cudaSuccess) e = cudaMallocAsync(&T->d_h, h.size() * sizeof(float), st);
  if (e == cudaSuccess) e = cudaMallocAsync(&T->d_e, (size_t)T->ntiles * TM * NE * sizeof(float), st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(T->d_h, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return fail(mrg_cuda_check(e, "tensor-core Q2 buffers"));
  int rc = make_map(&T->mE, T->d_e, NE, (uint64_t)T->ntiles * TM, NE * 4, 32, 32, CU_TENSOR_MAP_SWIZZLE_128B);
  if (rc) return fail(rc);
  *out = T;
  return MRG_OK;
}

void mrg_q2tc_free(Q2Tc* T, cudaStream_t st) {
  if (!T) return;
  cudaFreeAsync(T->d_w, st);
  cudaFreeAsync(T->d_h, st);
  cudaFreeAsync(T->d_e, st);
  delete T;
}

float* mrg_q2tc_w_image(Q2Tc* T) { return T->d_w; }

// Element matrices (tensor cores) then the row gather into J (FP32 values of the canonical graph).
int mrg_q2tc_launch(const mrg_problem* p, Q2Tc* T, float* J, bool ovw, int* err, cudaStream_t s) {
  static std::once_flag once;
  static cudaError_t attr_err = cudaSuccess;
  std::call_once(once, [] {
    attr_err = cudaFuncSetAttribute(k_q2_elem_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
  });
  if (attr_err != cudaSuccess) return mrg_cuda_check(attr_err, "tensor-core element kernel smem attribute");
  int dev = 0, nsm = 0;
  MRG_CUDA(cudaGetDevice(&dev));
  MRG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const int grid = T->ntiles < nsm ? T->ntiles : nsm;
  k_q2_elem_tc<<<grid, THREADS, SMEM_BYTES, s>>>(T->d_w, T->d_h, T->mE, T->ntiles, T->ksteps, err, p->g.wait_ns,
                                                 p->g.withhold);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return mrg_cuda_check(e, "tensor-core element kernel launch");
  if ((int64_t)p->g.nc[0] * p->g.nc[1] * NE * 2 >= ((int64_t)1 << 31))
    return mrg_fail(MRG_ENOTSUP, "tensor-core Q2 path: an x-y cell plane is too large for 32-bit strides");
  const int64_t warps_needed = (p->ndof + GRUN - 1) / GRUN;
  int64_t blocks = (warps_needed * 32 + GT - 1) / GT;
  if (blocks > (int64_t)nsm * 16) blocks = (int64_t)nsm * 16;
  k_q2_gather<<<(unsigned)blocks, GT, 0, s>>>(p->g, p->ndof, T->d_e, J, ovw ? 1 : 0);
  e = cudaGetLastError();
  return e == cudaSuccess ? MRG_OK : mrg_cuda_check(e, "element gather launch");
}

int mrg_tc_smem_bytes() { return SMEM_BYTES; }
