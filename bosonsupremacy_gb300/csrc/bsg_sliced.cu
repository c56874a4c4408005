// Sliced GEMM on the 5th-generation tensor cores: FP64 results from BF16
// products with exact FP32 accumulation.
//
//   C[r, c] (fp64) = sum_k A[r, k] B[c, k]          A, B given in FP64
//
// Every row of A (and of B) is scaled by a power of two 2^e_row that bounds
// its largest entry and cut into S fixed-point slices of b bits:
//   A[r, k] = 2^(e_r - b) * sum_s v_s(r, k),   v_s = m_s 2^(-b s),  m_s integer,
// |m_0| <= 2^b, |m_s| <= 2^(b-1) (round to nearest at each step), so every
// slice value is exact in BF16.  The product of slice s of A and slice t of B
// is an integer times 2^(-b (s + t)); the L + 1 pairs of level L = s + t sum
// over k to at most K 2^(2b) max(1, 1 + (L - 1) / 4) in units of 2^(-b L), and with
// b chosen so that 3 K 2^(2b) < 2^23 that stays an integer below 2^23 for
// every L <= 9, so FP32 accumulation in TMEM adds a level without any
// rounding.  The CTA keeps eight accumulators per output tile: levels 0 .. 6
// (exact) and levels 7 .. S-1 together (at most 2^(-7b) of the result, so
// their FP32 rounding stays far below 2^-42 of it).  Pairs with s + t >= S
// are dropped: the result carries about b S bits of each operand row's
// scale.  The epilogue adds the accumulators in FP64 and applies
// 2^(e_r + e_c - 2b).  (Levels 3 and up shared one FP32 accumulator in a
// first version: its truncating accumulation, repeated over every pair and K
// step, cost up to 2^-30 of the row scale at K = 4096.)
//
// Kernel: persistent and warp-specialised like the 3xTF32 GEMM, 128 x 64
// output tiles.  Warp 0 lane 0 streams, for every (s, t) pair of the tile
// and every 64-wide K block, the 128 x 64 BF16 tile of A slice s and the
// 64 x 64 tile of B slice t (TMA, 128-byte swizzle) through a 6-stage ring;
// warp 1 lane 0 issues 4 tcgen05.mma (kind::f16, K = 16) per stage into the
// pair's level accumulator; warps 2-5 drain the tile's eight accumulators
// (8 x 64 = 512 TMEM columns, one set: the next tile's MMAs wait for the
// drain).  Every mbarrier wait is bounded; on a timeout the CTA records an
// error, frees its TMEM and returns.
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>

#include "bsg_internal.h"

namespace bsg {
namespace sliced {

constexpr int TM = 128, TN = 64, TK = 64;        // TK bf16 = 128 bytes = one swizzle row
constexpr int kStages = 9;                        // 216 KB of ring slots
constexpr int kATile = TM * TK * 2;               // 16 KB
constexpr int kBTile = TN * TK * 2;               // 8 KB
constexpr int kStageBytes = kATile + kBTile;      // 24 KB
constexpr int kAcc = 8;                           // levels 0 .. 6, 7+
constexpr int kTmemCols = kAcc * TN;              // 512
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
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
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
// K-major tile of 128-byte rows, 128-byte swizzle (8-row atoms of 1024 bytes).
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFFu) >> 4);
  d |= (uint64_t)(16u >> 4) << 16;
  d |= (uint64_t)(1024u >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}
// kind::f16 with BF16 A and B (format 1), FP32 D, both K-major, M = 128, N = 64.
__host__ __device__ constexpr uint32_t instr_desc_bf16() {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(TN >> 3) << 17) | ((uint32_t)(TM >> 4) << 24);
}
__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
          tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc));
}
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}
// 32 TMEM lanes x 16 consecutive columns (one FP32 value per lane and column).
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}

// I 2^x as an FP64 value, rounded to nearest even, assembled from integer
// operations (the FP64 pipe runs at ~1/64 of the FP32 one on this GPU); the
// rare result outside the normal range goes through ldexp.
__device__ __forceinline__ double scaled_int_to_double(long long I, int x) {
  if (I == 0) return 0.0;
  const unsigned long long sign = I < 0 ? (1ull << 63) : 0ull;
  unsigned long long a = I < 0 ? (unsigned long long)(-I) : (unsigned long long)I;
  const int n = __clzll((long long)a);
  a <<= n;                                   // leading one at bit 63
  unsigned long long m = a >> 11;            // 53 bits
  const unsigned long long rem = a & 0x7ffull;
  if (rem > 0x400ull || (rem == 0x400ull && (m & 1ull))) ++m;
  int E = 63 - n + x;                        // value = 1.m 2^E
  if (m >> 53) {                             // the rounding carried into bit 53
    m >>= 1;
    ++E;
  }
  if (E < -1022 || E > 1023) return ldexp(__ll2double_rn(I), x);
  return __longlong_as_double((long long)(sign | ((unsigned long long)(E + 1023) << 52) | (m & ((1ull << 52) - 1))));
}

// (s, t) of pair p in level order: level L holds pairs (0, L), (1, L-1), ..., (L, 0).
__device__ __forceinline__ void pair_of(int p, int& s, int& t, int& L) {
  L = 0;
  while ((L + 1) * (L + 2) / 2 <= p) ++L;
  s = p - L * (L + 1) / 2;
  t = L - s;
}

struct Args {
  double* C;           // [rows, ldc] fp64
  int ldc;
  int M, N, K;         // rows of C (non-grouped), columns, inner length
  int S, b;            // slices per row, bits per slice
  int a_rows, b_rows;  // rows of one A slice / one B slice in the stacked operands
  const int* ea;       // [a_rows] row exponents of A
  const int* eb;       // [b_rows] row exponents of B
  const int4* mtiles;  // grouped: row tile {first row, end row, B row offset, 0}
  int* err;
};

__global__ void __launch_bounds__(192, 1)
    sliced_gemm_kernel(const __grid_constant__ CUtensorMap mA, const __grid_constant__ CUtensorMap mB, Args g,
                       int tiles_m, int tiles_n) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(base + kStages * kStageBytes);
  uint64_t* empty = full + kStages;
  uint64_t* accf = empty + kStages;  // a tile's accumulators complete
  uint64_t* acce = accf + 1;         // drained by the epilogue
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(acce + 1);
  int* fail = reinterpret_cast<int*>(tmem_slot + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nkb = (g.K + TK - 1) / TK;
  const int npairs = g.S * (g.S + 1) / 2;
  const int total = tiles_m * tiles_n;
  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(accf, 1);
    mbar_init(acce, 4);
    *fail = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = *tmem_slot;
  auto tile_rows = [&](int tile, int& m0, int& m_end, int& b_row0, int& n0) {
    const int tm = tile / tiles_n, tn = tile % tiles_n;
    n0 = tn * TN;
    if (g.mtiles) {
      const int4 t = g.mtiles[tm];
      m0 = t.x;
      m_end = t.y;
      b_row0 = t.z;
    } else {
      m0 = tm * TM;
      m_end = g.M;
      b_row0 = 0;
    }
  };

  // Slice-resident order (S <= kStages slots): a slot holds slice s of both
  // operands for one K block, (A_s, B_s); all pairs of that K block are
  // issued from the S resident slots, so each slice tile is loaded once per K
  // block instead of once per pair (about a quarter of the L2 traffic per
  // MMA).  Slot s is freed after slice max(s, S-1-s), its last use; fill f
  // reuses the slot of fill f - kStages, freed no later than fill f - 1 since
  // kStages >= S.  Otherwise (S > kStages) pairs stream one (A_s, B_t) K
  // block per slot.
  const bool resident = g.S <= kStages;
  if (warp == 0 && lane == 0 && resident) {
    uint32_t it = 0;
    bool ok = true;
    for (int tile = blockIdx.x; tile < total && ok && !*(volatile int*)fail; tile += gridDim.x) {
      int m0, m_end, b_row0, n0;
      tile_rows(tile, m0, m_end, b_row0, n0);
      for (int kb = 0; kb < nkb && ok; ++kb)
        for (int sl = 0; sl < g.S; ++sl, ++it) {
          const int st = it % kStages;
          if (it >= kStages && !mbar_wait(&empty[st], ((it / kStages) - 1) & 1)) {
            atomicExch(fail, 1);
            ok = false;
            break;
          }
          unsigned char* sp = base + st * kStageBytes;
          mbar_expect_tx(&full[st], kStageBytes);
          tma_load_2d(sp, &mA, &full[st], kb * TK, sl * g.a_rows + m0);
          tma_load_2d(sp + kATile, &mB, &full[st], kb * TK, sl * g.b_rows + b_row0 + n0);
        }
    }
  } else if (warp == 1 && lane == 0 && resident) {
    constexpr uint32_t idesc = instr_desc_bf16();
    uint32_t it = 0, t_local = 0;
    bool ok = true;
    for (int tile = blockIdx.x; tile < total && ok && !*(volatile int*)fail; tile += gridDim.x, ++t_local) {
      if (t_local >= 1 && !mbar_wait(acce, (t_local - 1) & 1)) {
        atomicExch(fail, 1);
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;");
      uint32_t written = 0;  // accumulators already started in this tile
      for (int kb = 0; kb < nkb && ok; ++kb, it += g.S) {
        for (int sl = 0; sl < g.S; ++sl) {
          const uint32_t f = it + sl;
          if (!mbar_wait(&full[f % kStages], (f / kStages) & 1)) {
            atomicExch(fail, 1);
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;");
          // pairs whose later slice is sl: (sl, t) and (t, sl), t <= sl, sl + t <= S - 1
          for (int t = 0; t <= sl && sl + t <= g.S - 1; ++t)
            for (int sw = 0; sw < (t == sl ? 1 : 2); ++sw) {
              const int pa = sw ? t : sl, pb = sw ? sl : t;
              const int L = pa + pb, a = L < kAcc - 1 ? L : kAcc - 1;
              const uint32_t dacc = tmem + a * TN;
              const uint32_t sa = smem_u32(base + ((it + pa) % kStages) * kStageBytes);
              const uint32_t sb = smem_u32(base + ((it + pb) % kStages) * kStageBytes + kATile);
#pragma unroll
              for (int kk = 0; kk < TK / 16; ++kk) {
                const uint32_t acc_flag = (written >> a) & 1u;
                umma_bf16(dacc, smem_desc(sa + kk * 32), smem_desc(sb + kk * 32), idesc, acc_flag);
                written |= 1u << a;
              }
            }
          // free the slots whose last pair was just issued
          if (sl >= g.S - 1 - sl) umma_commit(&empty[(it + sl) % kStages]);
          if (g.S - 1 - sl < sl) umma_commit(&empty[(it + (g.S - 1 - sl)) % kStages]);
        }
      }
      if (!ok) break;
      umma_commit(accf);
    }
  } else if (warp == 0 && lane == 0) {
    // producer
    uint32_t it = 0;
    bool ok = true;
    for (int tile = blockIdx.x; tile < total && ok && !*(volatile int*)fail; tile += gridDim.x) {
      int m0, m_end, b_row0, n0;
      tile_rows(tile, m0, m_end, b_row0, n0);
      for (int p = 0; p < npairs && ok; ++p) {
        int s, t, L;
        pair_of(p, s, t, L);
        for (int kb = 0; kb < nkb; ++kb, ++it) {
          const int st = it % kStages;
          if (it >= kStages && !mbar_wait(&empty[st], ((it / kStages) - 1) & 1)) {
            atomicExch(fail, 1);
            ok = false;
            break;
          }
          unsigned char* sp = base + st * kStageBytes;
          mbar_expect_tx(&full[st], kStageBytes);
          tma_load_2d(sp, &mA, &full[st], kb * TK, s * g.a_rows + m0);
          tma_load_2d(sp + kATile, &mB, &full[st], kb * TK, t * g.b_rows + b_row0 + n0);
        }
      }
    }
  } else if (warp == 1 && lane == 0) {
    // MMA issuer
    constexpr uint32_t idesc = instr_desc_bf16();
    uint32_t it = 0, t_local = 0;
    bool ok = true;
    for (int tile = blockIdx.x; tile < total && ok && !*(volatile int*)fail; tile += gridDim.x, ++t_local) {
      if (t_local >= 1 && !mbar_wait(acce, (t_local - 1) & 1)) {
        atomicExch(fail, 1);
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;");
      for (int p = 0; p < npairs && ok; ++p) {
        int s, t, L;
        pair_of(p, s, t, L);
        const int a = L < kAcc - 1 ? L : kAcc - 1;
        const uint32_t dacc = tmem + a * TN;
        const bool first_pair = s == 0 && L <= kAcc - 1;  // (0, L) opens accumulator a
        for (int kb = 0; kb < nkb; ++kb, ++it) {
          const int st = it % kStages;
          if (!mbar_wait(&full[st], (it / kStages) & 1)) {
            atomicExch(fail, 1);
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;");
          const uint32_t sa = smem_u32(base + st * kStageBytes);
#pragma unroll
          for (int kk = 0; kk < TK / 16; ++kk) {
            const uint32_t off = kk * 32;  // 16 bf16 = 32 bytes along K inside the swizzled row
            const uint32_t acc_flag = (first_pair && kb == 0 && kk == 0) ? 0u : 1u;
            umma_bf16(dacc, smem_desc(sa + off), smem_desc(sa + kATile + off), idesc, acc_flag);
          }
          umma_commit(&empty[st]);
        }
      }
      if (!ok) break;
      umma_commit(accf);
    }
  } else if (warp >= 2) {
    // epilogue: TMEM lane quarter q = warp % 4 holds tile rows 32 q .. 32 q + 31
    const int q = warp & 3;
    // accumulators written per tile: levels 0 .. min(S, 8) - 1 (the others hold stale TMEM)
    const int n_acc = g.S < kAcc ? g.S : kAcc;
    uint32_t t_local = 0;
    for (int tile = blockIdx.x; tile < total; tile += gridDim.x, ++t_local) {
      const bool ready = mbar_wait(accf, t_local & 1);
      asm volatile("tcgen05.fence::after_thread_sync;");
      if (!ready) atomicExch(fail, 1);
      if (!__all_sync(0xffffffffu, ready && !*(volatile int*)fail)) break;
      int m0, m_end, b_row0, n0;
      tile_rows(tile, m0, m_end, b_row0, n0);
      const int row = m0 + q * 32 + lane;
      const bool live = row < m_end;
      const int er = live ? g.ea[row] : 0;
      // The levels are summed exactly as an int64 in units of 2^-G (G = b x the
      // last exact level): level a < 7 holds an integer times 2^(-b a), so
      // acc_a 2^(b a) converts to an int64 exactly; the combined levels 7+ are
      // rounded to the unit (below 2^-50 of the level-0 scale).  The int64
      // becomes the FP64 output by integer operations (scaled_int_to_double).
      const int G = g.b * (g.S - 1 < kAcc - 2 ? g.S - 1 : kAcc - 2);
      for (int c = 0; c < TN; c += 16) {
        long long v[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) v[j] = 0;
        const uint32_t lane_base = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)c;
        for (int a = 0; a < n_acc; ++a) {
          uint32_t r[16];
          tmem_ld16(lane_base + a * TN, r);
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
          const bool exact = a < kAcc - 1;
          const int up = exact ? g.b * a : G;                      // to an integer
          const float pw = __int_as_float((127 + up) << 23);      // 2^up (up <= 126)
          const int sh = exact ? G - g.b * a : 0;                  // to units of 2^-G
#pragma unroll
          for (int j = 0; j < 16; ++j) v[j] += __float2ll_rn(__uint_as_float(r[j]) * pw) << sh;
        }
        if (live) {
          double* out = g.C + (int64_t)row * g.ldc + n0 + c;
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const int col = n0 + c + j;
            if (col < g.N) out[j] = scaled_int_to_double(v[j], er + g.eb[b_row0 + col] - 2 * g.b - G);
          }
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;");
      __syncwarp();
      if (lane == 0) mbar_arrive(acce);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
  }
  if (threadIdx.x == 0 && *fail) atomicExch(g.err, 1);
}

// Row exponent of a row whose largest magnitude has the IEEE bits `mx`:
// the e with max |x| < 2^e (frexp's exponent), 0 for an all-zero row.
__device__ __forceinline__ int row_exponent(unsigned long long mx) {
  const int ex = int((mx >> 52) & 0x7ff);
  return mx == 0 ? 0 : (ex == 0 ? -1022 : ex - 1022);
}

// The S balanced b-bit digits of x 2^-e (|x| < 2^e) by integer arithmetic:
// x 2^-e = X 2^-62 with X an int64 (the 53-bit significand shifted into
// place; bits below 2^-62 of the row scale dropped), then digit s is X
// rounded to a multiple of 2^(62 - b (s + 1)), taken off X.  Slice s holds
// m_s 2^(-b s) (exact in BF16: |m_0| <= 2^b, |m_s| <= 2^(b-1) for s > 0).
__device__ __forceinline__ void slice_value(double x, int e, int b, int S, __nv_bfloat16* out, int64_t stride) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
  const int ex = int((bits >> 52) & 0x7ff);
  long long X = 0;
  if (ex != 0) {  // zero and subnormals (below 2^-1022) contribute nothing
    const unsigned long long mant = (bits & ((1ull << 52) - 1)) | (1ull << 52);
    const int sh = ex - 1075 + 62 - e;  // <= 9 since |x| < 2^e
    const unsigned long long m = sh >= 0 ? (mant << sh) : (sh > -64 ? (mant >> -sh) : 0ull);
    X = (bits >> 63) ? -(long long)m : (long long)m;
  }
  for (int s = 0; s < S; ++s) {
    const int shift = 62 - b * (s + 1);
    const long long m = (X + (1ll << (shift - 1))) >> shift;  // nearest multiple of 2^shift (ties up)
    X -= m << shift;
    // m_s 2^(-b s): the power of two built from its exponent bits (b s <= 126)
    out[(int64_t)s * stride] = __float2bfloat16_rn(__int2float_rn((int)m) * __int_as_float((127 - b * s) << 23));
  }
}

// One warp per row: the row's power-of-two scale (from the IEEE bits of its
// largest magnitude, an integer max) and its S slices.  x(q) is produced by
// `src`; slices land at out[s * slice_stride + row * K + q].
template <class Src>
__device__ __forceinline__ void slice_row(const Src& src, int row, int K, int S, int b, __nv_bfloat16* out,
                                          int64_t slice_stride, int* e_out) {
  const int lane = threadIdx.x & 31;
  unsigned long long mx = 0;
  for (int q = lane; q < K; q += 32) {
    const unsigned long long a = (unsigned long long)__double_as_longlong(src(q)) & 0x7fffffffffffffffull;
    mx = a > mx ? a : mx;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long v = __shfl_xor_sync(0xffffffffu, mx, o);
    mx = v > mx ? v : mx;
  }
  const int e = row_exponent(mx);
  if (lane == 0) e_out[row] = e;
  __nv_bfloat16* o = out + (int64_t)row * K;
  for (int q = lane; q < K; q += 32) slice_value(src(q), e, b, S, o + q, slice_stride);
}

// A rows of a contraction level: x(r, q) = E[parent[r]][q / 2].{re, im} * lam[q / 2].
__global__ void slice_env_kernel(const double2* __restrict__ E, const int32_t* __restrict__ pidx,
                                 const double* __restrict__ lam, int rows, int chi, int S, int b,
                                 __nv_bfloat16* __restrict__ A, int a_rows, int* __restrict__ ea) {
  const int row = int(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  if (row >= rows) return;  // warp-uniform
  const double* e = reinterpret_cast<const double*>(E + (int64_t)pidx[row] * chi);
  auto src = [&](int q) { return e[q] * lam[q >> 1]; };
  slice_row(src, row, 2 * chi, S, b, A, (int64_t)a_rows * 2 * chi, ea);
}

// T[n][c][k] = Gamma[k, c, n] (left) or Gamma[c, k, n] (right): 16 x 16 (c, k)
// tiles of all d photon numbers through shared memory, so both the reads
// (d-element runs of Gamma) and the writes (k-contiguous rows of T) coalesce.
constexpr int kTT = 16;
__global__ void transpose_gamma_kernel(const double2* __restrict__ G, int chi, int d, int left,
                                       double2* __restrict__ T) {
  extern __shared__ double2 tile[];  // [kTT][kTT][d]: (a, b, n) with a the slower Gamma index
  const int c0 = blockIdx.y * kTT, k0 = blockIdx.x * kTT;
  // Gamma index of tile entry (a, b): left a = k, b = c; right a = c, b = k
  const int a0 = left ? k0 : c0, b0 = left ? c0 : k0;
  const int per = kTT * d;  // contiguous elements of one a-row of the tile
  for (int t = threadIdx.x; t < kTT * per; t += blockDim.x) {
    const int a = t / per, r = t % per;
    const int ga = a0 + a, gb = b0 + r / d;
    if (ga < chi && gb < chi) tile[t] = G[((int64_t)ga * chi + gb) * d + (r % d)];
  }
  __syncthreads();
  for (int t = threadIdx.x; t < d * kTT * kTT; t += blockDim.x) {
    const int n = t / (kTT * kTT), cc = (t / kTT) % kTT, kk = t % kTT;
    const int c = c0 + cc, k = k0 + kk;
    if (c >= chi || k >= chi) continue;
    const int a = left ? kk : cc, bb = left ? cc : kk;
    T[((int64_t)n * chi + c) * chi + k] = tile[(a * kTT + bb) * d + n];
  }
}

// B rows of photon number n: Bt[n 2chi + 2c + eo][2k + ei] = {{Re, Im}, {-Im, Re}}[ei][eo] of
// T[n][c][k] (the transposed Gamma block).
__global__ void slice_gamma_kernel(const double2* __restrict__ T, int chi, int d, int S, int b,
                                   __nv_bfloat16* __restrict__ B, int b_rows, int* __restrict__ eb) {
  const int row = int(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int K2 = 2 * chi;
  if (row >= d * K2) return;  // warp-uniform
  const int n = row / K2, rc = row % K2, c = rc >> 1, eo = rc & 1;
  const double2* t = T + ((int64_t)n * chi + c) * chi;
  auto src = [&](int q) {
    const double2 v = t[q >> 1];
    const int ei = q & 1;
    return ei == 0 ? (eo == 0 ? v.x : v.y) : (eo == 0 ? -v.y : v.x);
  };
  slice_row(src, row, K2, S, b, B, (int64_t)b_rows * K2, eb);
}

// Slices of an FP64 row-major [rows, K] matrix (the C entry point).
__global__ void slice_dense_kernel(const double* __restrict__ X, int rows, int K, int S, int b,
                                   __nv_bfloat16* __restrict__ out, int* __restrict__ e) {
  const int row = int(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  if (row >= rows) return;  // warp-uniform
  const double* x = X + (int64_t)row * K;
  auto src = [&](int q) { return x[q]; };
  slice_row(src, row, K, S, b, out, (int64_t)rows * K, e);
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static int make_map_bf16(CUtensorMap* m, const __nv_bfloat16* ptr, int64_t rows, int K, int box_rows) {
  static EncodeTiledFn enc = nullptr;
  if (!enc) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    BSG_CUDA(cudaGetDriverEntryPoint("cuTensorMapEncodeTiled", &p, cudaEnableDefault, &q));
    if (!p || q != cudaDriverEntryPointSuccess) {
      set_error("cuTensorMapEncodeTiled is not available from the driver");
      return BSG_ERR_CUDA;
    }
    enc = reinterpret_cast<EncodeTiledFn>(p);
  }
  if ((reinterpret_cast<uintptr_t>(ptr) & 15) || (K % 8)) {
    set_error("sliced GEMM: operands need 16-byte aligned rows (K %% 8 == 0)");
    return BSG_ERR_INVALID;
  }
  cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)K * 2};
  cuuint32_t box[2] = {TK, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<__nv_bfloat16*>(ptr), dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed (%d)", (int)r);
    return BSG_ERR_CUDA;
  }
  return BSG_OK;
}

}  // namespace sliced

void sliced_params(int K, int* S, int* b) {
  // exact level sums: 3 K 2^(2b) < 2^23; about 42 bits per operand row
  int lk = 0;
  while ((1 << lk) < K) ++lk;
  const int bb = std::max(3, std::min(7, (21 - lk) / 2));
  *b = bb;
  *S = (42 + bb - 1) / bb;
}

size_t sliced_operand_bytes(int64_t rows, int K, int S) { return (size_t)S * rows * K * 2; }

int sliced_slice_env(const double2* E, const int32_t* pidx, const double* lam, int rows, int chi, int S, int b,
                     void* A, int* ea, cudaStream_t st) {
  if (rows == 0) return BSG_OK;
  sliced::slice_env_kernel<<<unsigned(((int64_t)rows * 32 + 255) / 256), 256, 0, st>>>(
      E, pidx, lam, rows, chi, S, b, reinterpret_cast<__nv_bfloat16*>(A), rows, ea);
  BSG_CUDA(cudaGetLastError());
  return BSG_OK;
}

size_t sliced_gamma_scratch_bytes(int chi, int d) { return (size_t)d * chi * chi * 16; }

int sliced_slice_gamma(const double2* G, int chi, int d, bool left, int S, int b, void* B, int* eb, void* scratch,
                       cudaStream_t st) {
  const int rows = d * 2 * chi;
  double2* T = reinterpret_cast<double2*>(scratch);
  const unsigned nt = unsigned((chi + sliced::kTT - 1) / sliced::kTT);
  const size_t smem = (size_t)sliced::kTT * sliced::kTT * d * sizeof(double2);
  if (smem > 48 * 1024)
    BSG_CUDA(cudaFuncSetAttribute(sliced::transpose_gamma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem));
  sliced::transpose_gamma_kernel<<<dim3(nt, nt), 256, smem, st>>>(G, chi, d, left ? 1 : 0, T);
  sliced::slice_gamma_kernel<<<unsigned(((int64_t)rows * 32 + 255) / 256), 256, 0, st>>>(
      T, chi, d, S, b, reinterpret_cast<__nv_bfloat16*>(B), rows, eb);
  BSG_CUDA(cudaGetLastError());
  return BSG_OK;
}

int sliced_gemm(bsg_handle_t h, const void* A, int a_rows, const int* ea, const void* B, int b_rows, const int* eb,
                double* C, int M, int N, int K, int ldc, int S, int b, int* d_err, cudaStream_t st, bool profile,
                const int4* mtiles, int n_mtiles) {
  using namespace sliced;
  if (M == 0 || N == 0 || (mtiles && n_mtiles == 0)) return BSG_OK;
  if (S < 1 || S > 12) {
    set_error("sliced GEMM: S=%d slices outside [1, 12]", S);
    return BSG_ERR_INVALID;
  }
  CUtensorMap ma, mb;
  BSG_TRY(make_map_bf16(&ma, reinterpret_cast<const __nv_bfloat16*>(A), (int64_t)S * a_rows, K, TM));
  BSG_TRY(make_map_bf16(&mb, reinterpret_cast<const __nv_bfloat16*>(B), (int64_t)S * b_rows, K, TN));
  Args g{C, ldc, M, N, K, S, b, a_rows, b_rows, ea, eb, mtiles, d_err};
  const int tiles_m = mtiles ? n_mtiles : (M + TM - 1) / TM;
  const int tiles_n = (N + TN - 1) / TN;
  const int total = tiles_m * tiles_n;
  const int grid = std::max(1, std::min(total, h->num_sms));
  const size_t smem = (size_t)kStages * kStageBytes + 1024 + 256;
  static bool attr = false;
  if (!attr) {
    BSG_CUDA(cudaFuncSetAttribute(sliced_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr = true;
  }
  const double pairs = S * (S + 1) / 2.0;
  if (profile) {
    BSG_PROFILED(h, BSG_K_CONTRACT, st, 2.0 * M * (double)N * K * pairs,
                 (sliced_gemm_kernel<<<grid, 192, smem, st>>>(ma, mb, g, tiles_m, tiles_n)));
  } else {
    sliced_gemm_kernel<<<grid, 192, smem, st>>>(ma, mb, g, tiles_m, tiles_n);
    BSG_CUDA(cudaGetLastError());
  }
  return BSG_OK;
}

}  // namespace bsg

using namespace bsg;

extern "C" int bsg_gemm_sliced(bsg_handle_t h, const double* A, const double* B, double* C, int M, int N, int K,
                               bsg_stream_t stream) {
  BSG_CHECK_ARG(h && A && B && C, "bsg_gemm_sliced: null pointer");
  BSG_CHECK_ARG(M >= 0 && N >= 0 && K > 0 && K % 8 == 0 && K <= (1 << 15),
                "bsg_gemm_sliced: need 0 < K <= 32768, K %% 8 == 0 (K=%d)", K);
  BSG_CUDA(cudaSetDevice(h->device));
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  int S = 0, b = 0;
  sliced_params(K, &S, &b);
  auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
  const size_t na = al(sliced_operand_bytes(M, K, S)), nb = al(sliced_operand_bytes(N, K, S));
  const size_t ne = al((size_t)(M + N) * 4);
  BSG_TRY(h->contract_ws.ensure(na + nb + ne + 256));
  char* w = reinterpret_cast<char*>(h->contract_ws.ptr);
  int* ea = reinterpret_cast<int*>(w + na + nb);
  int* eb = ea + M;
  int* d_err = reinterpret_cast<int*>(w + na + nb + ne);
  BSG_CUDA(cudaMemsetAsync(d_err, 0, 4, st));
  if (M) {
    sliced::slice_dense_kernel<<<unsigned(((int64_t)M * 32 + 255) / 256), 256, 0, st>>>(
        A, M, K, S, b, reinterpret_cast<__nv_bfloat16*>(w), ea);
  }
  if (N) {
    sliced::slice_dense_kernel<<<unsigned(((int64_t)N * 32 + 255) / 256), 256, 0, st>>>(
        B, N, K, S, b, reinterpret_cast<__nv_bfloat16*>(w + na), eb);
  }
  BSG_CUDA(cudaGetLastError());
  BSG_TRY(sliced_gemm(h, w, M, ea, w + na, N, eb, C, M, N, K, N, S, b, d_err, st, true, nullptr, 0));
  int err = 0;
  BSG_CUDA(cudaMemcpyAsync(&err, d_err, 4, cudaMemcpyDeviceToHost, st));
  BSG_CUDA(cudaStreamSynchronize(st));
  if (err) {
    set_error("bsg_gemm_sliced: a pipeline wait timed out");
    return BSG_ERR_CUDA;
  }
  return BSG_OK;
}
