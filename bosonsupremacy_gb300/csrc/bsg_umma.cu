// 3-way split TF32 GEMM on the 5th-generation tensor cores (tcgen05 / UMMA).
//
//   C[M, N] (fp32) = (A_hi + A_lo)[M, K] * (B_hi + B_lo)[N, K]^T
//                  ~ A_hi B_hi^T + A_hi B_lo^T + A_lo B_hi^T      (FP32 accumulation in TMEM)
//
// A and B are K-major fp32 arrays whose hi/lo parts are TF32-rounded, so the
// three products recover ~FP32 accuracy from TF32 tensor-core inputs.
// One CTA computes one 128 x 128 output tile:
//   warp 0 lane 0 : TMA producer (cp.async.bulk.tensor, 128B swizzle) into a
//                   3-stage ring of {A_hi, A_lo, B_hi, B_lo} 128 x 32 tiles
//   warp 1 lane 0 : MMA issuer, 3 x 4 tcgen05.mma (K = 8 each) per stage into a
//                   128 x 128 fp32 accumulator in TMEM, tcgen05.commit frees the stage
//   warps 0..3    : epilogue, tcgen05.ld 32 lanes x 32 columns per warp and step
// Every mbarrier wait is bounded; on a timeout the CTA records an error,
// frees its TMEM and returns.
#include <cuda.h>

#include <algorithm>
#include <cstring>

#include "bsg_internal.h"

namespace bsg {

constexpr int UM = 128, UN = 128, UK = 32;  // tile (UK fp32 = 128 bytes = one swizzle row)
constexpr int kStages = 3;
constexpr int kTileBytes = UM * UK * 4;      // 16 KB (A and B tiles are both 128 x 32)
constexpr int kStageBytes = 4 * kTileBytes;  // A_hi, A_lo, B_hi, B_lo
constexpr uint32_t kWaitLimit = 1u << 22;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// Bounded wait for the phase with the given parity; false on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  const uint32_t a = smem_u32(bar);
  for (uint32_t it = 0; it < kWaitLimit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
          smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(c0), "r"(c1)
      : "memory");
}

// Shared-memory matrix descriptor: K-major tile of 128-byte rows with the
// 128-byte swizzle (8-row atoms of 1024 bytes, SBO = 1024), version 1.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFFu) >> 4);  // start address
  d |= (uint64_t)(16u >> 4) << 16;           // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(1024u >> 4) << 32;         // stride byte offset
  d |= (uint64_t)1 << 46;                    // descriptor version
  d |= (uint64_t)2 << 61;                    // 128-byte swizzle
  return d;
}

// Instruction descriptor: kind::tf32, D = f32, A = B = tf32, both K-major, M = 128, N = 128.
__host__ __device__ constexpr uint32_t instr_desc_tf32() {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(UN >> 3) << 17) | ((uint32_t)(UM >> 4) << 24);
}

__device__ __forceinline__ void umma_tf32(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(
          tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

struct UmmaArgs {
  float* C;
  int M, N, K;
  int ldc;
  int* err;
  // grouped mode (non-null): row tile y covers A/C rows [x, y) and reads B
  // rows from z on (one B block per group, stacked in one tensor map)
  const int4* mtiles;
};

__global__ void __launch_bounds__(128, 1)
    umma_tf32x3_kernel(const __grid_constant__ CUtensorMap mA_hi, const __grid_constant__ CUtensorMap mA_lo,
                       const __grid_constant__ CUtensorMap mB_hi, const __grid_constant__ CUtensorMap mB_lo,
                       UmmaArgs g) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  // 1024-byte aligned stage buffers (the swizzle atom), barriers after them
  unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(base + kStages * kStageBytes);
  uint64_t* empty = full + kStages;
  uint64_t* accb = empty + kStages;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(accb + 1);
  int* fail = reinterpret_cast<int*>(tmem_slot + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int m0 = blockIdx.y * UM, m_end = g.M, b_row0 = 0;
  if (g.mtiles) {
    const int4 t = g.mtiles[blockIdx.y];
    m0 = t.x;
    m_end = t.y;
    b_row0 = t.z;
  }
  const int n0 = blockIdx.x * UN;
  const int nkb = (g.K + UK - 1) / UK;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(accb, 1);
    *fail = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(UN));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = *tmem_slot;

  if (warp == 0 && lane == 0) {
    // producer
    for (int kb = 0; kb < nkb; ++kb) {
      const int s = kb % kStages;
      if (kb >= kStages && !mbar_wait(&empty[s], ((kb / kStages) - 1) & 1)) {
        atomicExch(fail, 1);
        break;
      }
      if (*(volatile int*)fail) break;
      unsigned char* st = base + s * kStageBytes;
      mbar_expect_tx(&full[s], kStageBytes);
      const int k0 = kb * UK;
      tma_load_2d(st, &mA_hi, &full[s], k0, m0);
      tma_load_2d(st + kTileBytes, &mA_lo, &full[s], k0, m0);
      tma_load_2d(st + 2 * kTileBytes, &mB_hi, &full[s], k0, b_row0 + n0);
      tma_load_2d(st + 3 * kTileBytes, &mB_lo, &full[s], k0, b_row0 + n0);
    }
  } else if (warp == 1 && lane == 0) {
    // MMA issuer
    constexpr uint32_t idesc = instr_desc_tf32();
    bool ok = true;
    for (int kb = 0; kb < nkb && ok; ++kb) {
      const int s = kb % kStages;
      if (!mbar_wait(&full[s], (kb / kStages) & 1)) {
        atomicExch(fail, 1);
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint32_t sa = smem_u32(base + s * kStageBytes);
      for (int kk = 0; kk < UK / 8; ++kk) {
        const uint32_t off = kk * 32;  // 8 tf32 = 32 bytes along K inside the swizzled row
        const uint64_t ahi = smem_desc(sa + off), alo = smem_desc(sa + kTileBytes + off);
        const uint64_t bhi = smem_desc(sa + 2 * kTileBytes + off), blo = smem_desc(sa + 3 * kTileBytes + off);
        const uint32_t first = (kb == 0 && kk == 0) ? 0u : 1u;
        umma_tf32(tmem, ahi, bhi, idesc, first);
        umma_tf32(tmem, ahi, blo, idesc, 1u);
        umma_tf32(tmem, alo, bhi, idesc, 1u);
      }
      umma_commit(&empty[s]);
    }
    umma_commit(accb);
  }
  __syncwarp();
  // epilogue: all four warps
  const bool ready = mbar_wait(accb, 0);
  asm volatile("tcgen05.fence::after_thread_sync;");
  if (!ready) atomicExch(fail, 1);
  const int row = m0 + warp * 32 + lane;
  // tcgen05.ld is warp-collective: decide once per warp
  const bool ok = __all_sync(0xffffffffu, ready && !*(volatile int*)fail);
  if (ok) {
    for (int c = 0; c < UN; c += 32) {
      uint32_t r[32];
      const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
          "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
            "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
            "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (row < m_end) {
        float* out = g.C + (int64_t)row * g.ldc + n0 + c;
#pragma unroll
        for (int j = 0; j < 32; ++j)
          if (n0 + c + j < g.N) out[j] = __uint_as_float(r[j]);
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(UN));
  }
  if (threadIdx.x == 0 && *fail) atomicExch(g.err, 1);
}

// ---- persistent warp-specialised variant: 128 x 256 tiles ------------------
// One CTA per SM loops over output tiles.  Warp 0 lane 0 streams the four
// operand tiles of each 32-wide K block through a 2-stage ring (96 KB a
// stage); warp 1 lane 0 issues 3 x 4 tcgen05.mma (K = 8, N = 256) per stage
// into one of two TMEM accumulators (2 x 256 columns); warps 2-5 drain the
// other accumulator (tcgen05.ld, TMEM lane quarter = warp % 4) while the next
// tile accumulates.  Twice the N of the basic kernel halves the A traffic per
// flop; the double accumulator hides the epilogue.  Every wait is bounded.
constexpr int PN = 256;
constexpr int kPStages = 2;
constexpr int kPATile = UM * UK * 4;                    // 16 KB
constexpr int kPBTile = PN * UK * 4;                    // 32 KB
constexpr int kPStageBytes = 2 * kPATile + 2 * kPBTile;  // 96 KB

__host__ __device__ constexpr uint32_t instr_desc_tf32_n256() {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(PN >> 3) << 17) | ((uint32_t)(UM >> 4) << 24);
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__global__ void __launch_bounds__(192, 1)
    umma_tf32x3_persist_kernel(const __grid_constant__ CUtensorMap mA_hi, const __grid_constant__ CUtensorMap mA_lo,
                               const __grid_constant__ CUtensorMap mB_hi, const __grid_constant__ CUtensorMap mB_lo,
                               UmmaArgs g, int tiles_m, int tiles_n) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(base + kPStages * kPStageBytes);
  uint64_t* empty = full + kPStages;
  uint64_t* accf = empty + kPStages;  // [2] accumulator ready for the epilogue
  uint64_t* acce = accf + 2;          // [2] accumulator drained by the epilogue
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(acce + 2);
  int* fail = reinterpret_cast<int*>(tmem_slot + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nkb = (g.K + UK - 1) / UK;
  const int total = tiles_m * tiles_n;
  if (threadIdx.x == 0) {
    for (int s = 0; s < kPStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&accf[b], 1);
      mbar_init(&acce[b], 4);
    }
    *fail = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(2 * PN));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = *tmem_slot;
  auto tile_rows = [&](int tile, int& m0, int& m_end, int& b_row0, int& n0) {
    const int tm = tile / tiles_n, tn = tile % tiles_n;
    n0 = tn * PN;
    if (g.mtiles) {
      const int4 t = g.mtiles[tm];
      m0 = t.x;
      m_end = t.y;
      b_row0 = t.z;
    } else {
      m0 = tm * UM;
      m_end = g.M;
      b_row0 = 0;
    }
  };

  if (warp == 0 && lane == 0) {
    // producer
    uint32_t it = 0;
    for (int tile = blockIdx.x; tile < total && !*(volatile int*)fail; tile += gridDim.x) {
      int m0, m_end, b_row0, n0;
      tile_rows(tile, m0, m_end, b_row0, n0);
      for (int kb = 0; kb < nkb; ++kb, ++it) {
        const int s = it % kPStages;
        if (it >= kPStages && !mbar_wait(&empty[s], ((it / kPStages) - 1) & 1)) {
          atomicExch(fail, 1);
          break;
        }
        unsigned char* st = base + s * kPStageBytes;
        mbar_expect_tx(&full[s], kPStageBytes);
        const int k0 = kb * UK;
        tma_load_2d(st, &mA_hi, &full[s], k0, m0);
        tma_load_2d(st + kPATile, &mA_lo, &full[s], k0, m0);
        tma_load_2d(st + 2 * kPATile, &mB_hi, &full[s], k0, b_row0 + n0);
        tma_load_2d(st + 2 * kPATile + kPBTile, &mB_lo, &full[s], k0, b_row0 + n0);
      }
    }
  } else if (warp == 1 && lane == 0) {
    // MMA issuer
    constexpr uint32_t idesc = instr_desc_tf32_n256();
    uint32_t it = 0, t_local = 0;
    for (int tile = blockIdx.x; tile < total && !*(volatile int*)fail; tile += gridDim.x, ++t_local) {
      const uint32_t ab = t_local & 1;
      if (t_local >= 2 && !mbar_wait(&acce[ab], ((t_local / 2) - 1) & 1)) {
        atomicExch(fail, 1);
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint32_t dacc = tmem + ab * PN;
      bool ok = true;
      for (int kb = 0; kb < nkb; ++kb, ++it) {
        const int s = it % kPStages;
        if (!mbar_wait(&full[s], (it / kPStages) & 1)) {
          atomicExch(fail, 1);
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint32_t sa = smem_u32(base + s * kPStageBytes);
        for (int kk = 0; kk < UK / 8; ++kk) {
          const uint32_t off = kk * 32;
          const uint64_t ahi = smem_desc(sa + off), alo = smem_desc(sa + kPATile + off);
          const uint64_t bhi = smem_desc(sa + 2 * kPATile + off), blo = smem_desc(sa + 2 * kPATile + kPBTile + off);
          const uint32_t first = (kb == 0 && kk == 0) ? 0u : 1u;
          umma_tf32(dacc, ahi, bhi, idesc, first);
          umma_tf32(dacc, ahi, blo, idesc, 1u);
          umma_tf32(dacc, alo, bhi, idesc, 1u);
        }
        umma_commit(&empty[s]);
      }
      if (!ok) break;
      umma_commit(&accf[ab]);
    }
  } else if (warp >= 2) {
    // epilogue: TMEM lane quarter q = warp % 4 holds tile rows 32 q .. 32 q + 31
    const int q = warp & 3;
    uint32_t t_local = 0;
    for (int tile = blockIdx.x; tile < total; tile += gridDim.x, ++t_local) {
      const uint32_t ab = t_local & 1;
      const bool ready = mbar_wait(&accf[ab], (t_local / 2) & 1);
      asm volatile("tcgen05.fence::after_thread_sync;");
      if (!ready) atomicExch(fail, 1);
      if (!__all_sync(0xffffffffu, ready && !*(volatile int*)fail)) break;
      int m0, m_end, b_row0, n0;
      tile_rows(tile, m0, m_end, b_row0, n0);
      const int row = m0 + q * 32 + lane;
      for (int c = 0; c < PN; c += 32) {
        uint32_t r[32];
        const uint32_t taddr = tmem + ((uint32_t)(q * 32) << 16) + ab * PN + (uint32_t)c;
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
            "%14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
              "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
              "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
            : "r"(taddr));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        if (row < m_end) {
          float* out = g.C + (int64_t)row * g.ldc + n0 + c;
          if (n0 + c + 32 <= g.N && (reinterpret_cast<uintptr_t>(out) & 15) == 0) {
#pragma unroll
            for (int j = 0; j < 32; j += 4)
              *reinterpret_cast<float4*>(out + j) = make_float4(__uint_as_float(r[j]), __uint_as_float(r[j + 1]),
                                                                __uint_as_float(r[j + 2]), __uint_as_float(r[j + 3]));
          } else {
#pragma unroll
            for (int j = 0; j < 32; ++j)
              if (n0 + c + j < g.N) out[j] = __uint_as_float(r[j]);
          }
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;");
      __syncwarp();
      if (lane == 0) mbar_arrive(&acce[ab]);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * PN));
  }
  if (threadIdx.x == 0 && *fail) atomicExch(g.err, 1);
}

// Split x into TF32-rounded hi and the TF32-rounded remainder.
__global__ void split_tf32_kernel(const float* __restrict__ x, float* __restrict__ hi, float* __restrict__ lo,
                                  int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float v = x[i];
  uint32_t h;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(v));
  const float hf = __uint_as_float(h);
  uint32_t l;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(l) : "f"(v - hf));
  hi[i] = hf;
  lo[i] = __uint_as_float(l);
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static int get_encoder(EncodeTiledFn* fn) {
  static EncodeTiledFn cached = nullptr;
  if (!cached) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    BSG_CUDA(cudaGetDriverEntryPoint("cuTensorMapEncodeTiled", &p, cudaEnableDefault, &q));
    if (!p || q != cudaDriverEntryPointSuccess) {
      set_error("cuTensorMapEncodeTiled is not available from the driver");
      return BSG_ERR_CUDA;
    }
    cached = reinterpret_cast<EncodeTiledFn>(p);
  }
  *fn = cached;
  return BSG_OK;
}

// K-major [rows, K] fp32 tensor map with box_rows x 32 boxes and the 128-byte swizzle.
static int make_map(CUtensorMap* m, const float* ptr, int rows, int K, int box_rows = UM) {
  EncodeTiledFn enc;
  BSG_TRY(get_encoder(&enc));
  if ((reinterpret_cast<uintptr_t>(ptr) & 15) || (K % 4)) {
    set_error("tf32x3 GEMM: operands need 16-byte aligned rows (K %% 4 == 0)");
    return BSG_ERR_INVALID;
  }
  cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)K * 4};
  cuuint32_t box[2] = {UK, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(ptr), dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed (%d)", (int)r);
    return BSG_ERR_CUDA;
  }
  return BSG_OK;
}

int split_tf32(bsg_handle_t h, const float* x, float* hi, float* lo, int64_t n, cudaStream_t st) {
  if (n == 0) return BSG_OK;
  BSG_PROFILED(h, BSG_K_PREP, st, (double)n,
               (split_tf32_kernel<<<unsigned((n + 255) / 256), 256, 0, st>>>(x, hi, lo, n)));
  return BSG_OK;
}

int gemm_tf32x3(bsg_handle_t h, const float* Ahi, const float* Alo, const float* Bhi, const float* Blo, float* C,
                int M, int N, int K, int ldc, int* d_err, cudaStream_t st, bool profile, const int4* mtiles,
                int n_mtiles, int b_rows) {
  if (M == 0 || N == 0 || (mtiles && n_mtiles == 0)) return BSG_OK;
  CUtensorMap ma, mal, mb, mbl;
  const int b_total = mtiles ? b_rows : N;
  const bool persist = h->tune[BSG_TUNE_GEMM_KERNEL] == 1;
  BSG_TRY(make_map(&ma, Ahi, M, K));
  BSG_TRY(make_map(&mal, Alo, M, K));
  BSG_TRY(make_map(&mb, Bhi, b_total, K, persist ? PN : UM));
  BSG_TRY(make_map(&mbl, Blo, b_total, K, persist ? PN : UM));
  UmmaArgs g{C, M, N, K, ldc, d_err, mtiles};
  const int tiles_m = mtiles ? n_mtiles : (M + UM - 1) / UM;
  if (persist) {
    const size_t smem = (size_t)kPStages * kPStageBytes + 1024 + 256;
    static bool pattr = false;
    if (!pattr) {
      BSG_CUDA(cudaFuncSetAttribute(umma_tf32x3_persist_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)smem));
      pattr = true;
    }
    const int tiles_n = (N + PN - 1) / PN;
    const int total = tiles_m * tiles_n;
    const int grid = std::max(1, std::min(total, h->num_sms));
    if (profile) {
      BSG_PROFILED(h, BSG_K_CONTRACT, st, 2.0 * M * (double)N * K * 3.0,
                   (umma_tf32x3_persist_kernel<<<grid, 192, smem, st>>>(ma, mal, mb, mbl, g, tiles_m, tiles_n)));
    } else {
      umma_tf32x3_persist_kernel<<<grid, 192, smem, st>>>(ma, mal, mb, mbl, g, tiles_m, tiles_n);
      BSG_CUDA(cudaGetLastError());
    }
    return BSG_OK;
  }
  const size_t smem = (size_t)kStages * kStageBytes + 1024 + 256;
  static bool attr = false;
  if (!attr) {
    BSG_CUDA(cudaFuncSetAttribute(umma_tf32x3_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr = true;
  }
  dim3 grid((N + UN - 1) / UN, tiles_m);
  if (profile) {
    BSG_PROFILED(h, BSG_K_CONTRACT, st, 2.0 * M * (double)N * K * 3.0,
                 (umma_tf32x3_kernel<<<grid, 128, smem, st>>>(ma, mal, mb, mbl, g)));
  } else {
    umma_tf32x3_kernel<<<grid, 128, smem, st>>>(ma, mal, mb, mbl, g);
    BSG_CUDA(cudaGetLastError());
  }
  return BSG_OK;
}

}  // namespace bsg

using namespace bsg;

extern "C" int bsg_gemm_tf32x3(bsg_handle_t h, const float* A, const float* B, float* C, int M, int N, int K,
                               bsg_stream_t stream) {
  BSG_CHECK_ARG(h && A && B && C, "bsg_gemm_tf32x3: null pointer");
  BSG_CHECK_ARG(M >= 0 && N >= 0 && K > 0 && K % 4 == 0, "bsg_gemm_tf32x3: need K > 0, K %% 4 == 0");
  BSG_CUDA(cudaSetDevice(h->device));
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const size_t na = (size_t)M * K, nb = (size_t)N * K;
  auto al = [](size_t x) { return (x * 4 + 255) & ~size_t(255); };
  BSG_TRY(h->contract_ws.ensure(2 * al(na) + 2 * al(nb) + 256));
  char* b = reinterpret_cast<char*>(h->contract_ws.ptr);
  float* Ahi = reinterpret_cast<float*>(b);
  float* Alo = reinterpret_cast<float*>(b + al(na));
  float* Bhi = reinterpret_cast<float*>(b + 2 * al(na));
  float* Blo = reinterpret_cast<float*>(b + 2 * al(na) + al(nb));
  int* d_err = reinterpret_cast<int*>(b + 2 * al(na) + 2 * al(nb));
  BSG_CUDA(cudaMemsetAsync(d_err, 0, 4, st));
  BSG_TRY(split_tf32(h, A, Ahi, Alo, (int64_t)na, st));
  BSG_TRY(split_tf32(h, B, Bhi, Blo, (int64_t)nb, st));
  BSG_TRY(gemm_tf32x3(h, Ahi, Alo, Bhi, Blo, C, M, N, K, N, d_err, st, true));
  int err = 0;
  BSG_CUDA(cudaMemcpyAsync(&err, d_err, 4, cudaMemcpyDeviceToHost, st));
  BSG_CUDA(cudaStreamSynchronize(st));
  if (err) {
    set_error("bsg_gemm_tf32x3: a pipeline wait timed out");
    return BSG_ERR_CUDA;
  }
  return BSG_OK;
}
