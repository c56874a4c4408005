// Transfer contraction of the MPS for a batch of photon patterns.
//
// amp(n) = Gamma_0[0, :, n_0] Lambda_0 Gamma_1[:, :, n_1] Lambda_1 ... Gamma_{M-1}[:, 0, n_{M-1}]
// -- the transfer step of sampling_cpu.py:75-80 with the photon numbers fixed
// instead of drawn.  Patterns share prefixes and suffixes, so the batch is
// contracted meet-in-the-middle: left environments L(prefix) for every
// distinct prefix up to the middle site m, right environments R(suffix) for
// every distinct suffix from m+1, and amp = sum_a L[a] Lambda_m[a] R[a].
// Each level is a set of GEMMs, one per photon number n of the new site:
//   left : L_i[rows(n)] = (L_{i-1}[parents] * Lambda_{i-1}) @ Gamma_i[:, :, n]
//   right: R_i[rows(n)] = (R_{i+1}[parents] * Lambda_i)     @ Gamma_i[:, :, n]^T
// Rows of a level are keyed n-major on the GPU (photon number, then parent
// row), so every GEMM writes a contiguous block; the host reads the level's
// row counts to size the launches.  The GEMM gathers its A rows by parent
// index and applies Lambda on the fly.
#include <algorithm>
#include <cstring>
#include <type_traits>
#include <vector>

#include "bsg_cgemm.cuh"
#include "bsg_internal.h"

namespace bsg {

// Level 0 of a side: E[r, a] = Gamma[base + a*stride + n_r*1] (row 0 of site 0 or column 0 of site M-1).
template <class R>
__global__ void env_init_kernel(const typename Cx<R>::T* __restrict__ G, int64_t stride, const int32_t* __restrict__ nvals,
                                int rows, int chi, typename Cx<R>::T* __restrict__ E) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)rows * chi) return;
  const int r = int(t / chi), a = int(t % chi);
  E[t] = G[(int64_t)a * stride + nvals[r]];
}

// amp[p] = sum_a L[li[p], a] * lam[a] * R[ri[p], a], one warp per pattern.
template <class R>
__global__ void final_dot_kernel(const typename Cx<R>::T* __restrict__ L, const int32_t* __restrict__ li,
                                 const typename Cx<R>::T* __restrict__ Rt, const int32_t* __restrict__ ri,
                                 const double* __restrict__ lam, int chi, int64_t P, double2* __restrict__ amp) {
  const int64_t p = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  double sr = 0.0, si = 0.0;
  if constexpr (std::is_same<R, float>::value) {
    // FP32 environments: each lane's few products accumulate in FP32 FMAs
    // (their TF32x3 rounding dominates), the 32 lane sums in FP64; the
    // bond weights are converted once per block
    extern __shared__ float lam_f[];
    for (int a = threadIdx.x; a < chi; a += blockDim.x) lam_f[a] = lam ? float(lam[a]) : 1.f;
    __syncthreads();
    if (p >= P) return;  // after the block barrier
    const float2* l = reinterpret_cast<const float2*>(L) + (int64_t)li[p] * chi;
    const float2* r = reinterpret_cast<const float2*>(Rt) + (int64_t)ri[p] * chi;
    float fr = 0.f, fi = 0.f;
    for (int a = lane; a < chi; a += 32) {
      const float2 lv = l[a], rv = r[a];
      const float w = lam_f[a];
      const float lx = lv.x * w, ly = lv.y * w;
      fr = fmaf(lx, rv.x, fmaf(-ly, rv.y, fr));
      fi = fmaf(lx, rv.y, fmaf(ly, rv.x, fi));
    }
    sr = fr;
    si = fi;
  } else {
    if (p >= P) return;
    const typename Cx<R>::T* l = L + (int64_t)li[p] * chi;
    const typename Cx<R>::T* r = Rt + (int64_t)ri[p] * chi;
    for (int a = lane; a < chi; a += 32) {
      const double w = lam ? lam[a] : 1.0;
      const double lx = double(l[a].x) * w, ly = double(l[a].y) * w;
      sr += lx * double(r[a].x) - ly * double(r[a].y);
      si += lx * double(r[a].y) + ly * double(r[a].x);
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    sr += __shfl_xor_sync(0xffffffffu, sr, o);
    si += __shfl_xor_sync(0xffffffffu, si, o);
  }
  if (lane == 0) amp[p] = make_double2(sr, si);
}

// ---- split path: the complex GEMM as one real GEMM on interleaved (re, im) ----
// C_int[r, 2c+eo] = sum_{k, ei} A_int[r, 2k+ei] B_int[2k+ei, 2c+eo] with
// B_int[2k+ei, 2c+eo] = {{Re B, Im B}, {-Im B, Re B}}[ei][eo]; the tensor-core
// GEMM wants B K-major, i.e. Bt[2c+eo][2k+ei].  Both operands are split into
// TF32 hi + lo.  left: B(k, c) = Gamma[k, c, n]; right: B(k, c) = Gamma[c, k, n].
__device__ __forceinline__ void tf32_split(float v, float& hi, float& lo) {
  uint32_t h, l;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(v));
  hi = __uint_as_float(h);
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(l) : "f"(v - hi));
  lo = __uint_as_float(l);
}

// B block of photon number n = blockIdx.y at rows n * 2 chi of Bhi / Blo.
__global__ void build_bt_kernel(const float2* __restrict__ G, int chi, int d, int left, float* __restrict__ Bhi,
                                float* __restrict__ Blo) {
  const int64_t K2 = 2 * (int64_t)chi;
  const int n = blockIdx.y;
  Bhi += (size_t)n * K2 * K2;
  Blo += (size_t)n * K2 * K2;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= K2 * K2) return;
  const int row = int(t / K2), col = int(t % K2);
  const int c = row >> 1, eo = row & 1, k = col >> 1, ei = col & 1;
  const float2 v = left ? G[((int64_t)k * chi + c) * d + n] : G[((int64_t)c * chi + k) * d + n];
  const float x = ei == 0 ? (eo == 0 ? v.x : v.y) : (eo == 0 ? -v.y : v.x);
  float hi, lo;
  tf32_split(x, hi, lo);
  Bhi[t] = hi;
  Blo[t] = lo;
}

__global__ void build_a_kernel(const float2* __restrict__ E, const int32_t* __restrict__ pidx,
                               const double* __restrict__ lam, int rows, int chi, float* __restrict__ Ahi,
                               float* __restrict__ Alo) {
  const int64_t K2 = 2 * (int64_t)chi;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)rows * K2) return;
  const int r = int(t / K2), q = int(t % K2), k = q >> 1;
  const float2 v = E[(int64_t)pidx[r] * chi + k];
  const float x = float(double((q & 1) ? v.y : v.x) * lam[k]);
  float hi, lo;
  tf32_split(x, hi, lo);
  Ahi[t] = hi;
  Alo[t] = lo;
}

// ---- planning on the device: distinct prefixes per level, grouped by n -----
// Level l of a side keys every pattern by (n, parent row) with n its photon
// number at the level's site; the distinct keys, in n-major order, are the
// level's rows, so rows of one n are contiguous (one GEMM per n).  Per level:
// mark the keys (each pattern first taking its row of the previous level),
// scan them into row ids (writing each row's parent and n and the level's
// group bounds); the patterns take their rows of the last level at the end.
constexpr int kMaxLevels = 1024;

struct PlanArgs {
  const int32_t* pat;  // [M, P]: photon number of pattern p at site s is pat[s * P + p]
  int64_t P;
  int M, d;
  int32_t* cur;        // [P] row at the previous level (0 before level 0)
  int32_t* keys;       // [P]
  int32_t* flags;      // [d * P] zero on entry, left zero
  int32_t* idx;        // [d * P] row of each key
  int32_t* meta;       // [levels, d + 2]: rows, group[0..d]
  int* err;
};

// Patterns [P, M] -> [M, P] (32 x 32 tiles through shared memory), so the
// per-level kernels read one site's photon numbers contiguously.
__global__ void transpose_patterns_kernel(const int32_t* __restrict__ pat, int64_t P, int M, int32_t* __restrict__ patT) {
  __shared__ int32_t tile[32][33];
  const int64_t p0 = (int64_t)blockIdx.x * 32;
  const int s0 = blockIdx.y * 32;
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int64_t p = p0 + r;
    const int s = s0 + threadIdx.x;
    if (p < P && s < M) tile[r][threadIdx.x] = pat[p * M + s];
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int s = s0 + r;
    const int64_t p = p0 + threadIdx.x;
    if (p < P && s < M) patT[(int64_t)s * P + p] = tile[threadIdx.x][r];
  }
}

// Level `level` keys every pattern; for level > 0 the pattern first takes
// its row of level - 1 (the scan of that level is done).
__global__ void plan_mark_kernel(PlanArgs a, int site, int level) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= a.P) return;
  int prev = 1, row = 0;
  if (level > 0) {
    prev = a.meta[(level - 1) * (a.d + 2)];
    row = a.idx[a.keys[p]];
    a.cur[p] = row;
  }
  int n = a.pat[(int64_t)site * a.P + p];
  if (n < 0 || n >= a.d) {
    atomicExch(a.err, 1);
    n = 0;
  }
  const int key = n * prev + row;
  a.keys[p] = key;
  a.flags[key] = 1;
}

// One CTA: exclusive scan of flags[0, d * prev) into idx, rows' parent / n,
// the level's row count and group bounds; clears the flags it read.
__global__ void __launch_bounds__(1024) plan_scan_kernel(PlanArgs a, int level, int32_t* parent, int32_t* nval) {
  __shared__ int32_t warp_sums[32];
  __shared__ int32_t carry;
  const int d = a.d;
  const int prev = level == 0 ? 1 : a.meta[(level - 1) * (d + 2)];
  const int64_t size = (int64_t)d * prev;
  int32_t* meta = a.meta + level * (d + 2);
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  if (tid == 0) carry = 0;
  __syncthreads();
  for (int64_t base = 0; base < size; base += 1024) {
    const int64_t q = base + tid;
    const int f = q < size ? a.flags[q] : 0;
    int x = f;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[w] = x;
    __syncthreads();
    if (w == 0) {
      int v = warp_sums[lane];
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += y;
      }
      warp_sums[lane] = v;
    }
    __syncthreads();
    const int c0 = carry;
    const int excl = c0 + (w ? warp_sums[w - 1] : 0) + x - f;
    if (q < size) {
      a.idx[q] = excl;
      a.flags[q] = 0;
      if (q % prev == 0) meta[1 + q / prev] = excl;  // first row of photon number q / prev
      if (f) {
        parent[excl] = int32_t(q % prev);
        nval[excl] = int32_t(q / prev);
      }
    }
    __syncthreads();
    if (tid == 1023) carry = excl + f;
    __syncthreads();
  }
  if (tid == 0) {
    meta[0] = carry;
    meta[1 + d] = carry;
  }
}

// Multi-CTA form of plan_scan_kernel for large levels, in three launches over
// 1024-key tiles (the grid covers d * P keys, the bound of d * prev; tiles past
// the level's keys do nothing): per-tile flag counts, one CTA turning the
// counts into tile offsets (and the level's row count), then each tile's
// exclusive scan plus its offset.
__device__ __forceinline__ int block_incl_scan_1024(int x, int32_t* warp_sums) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[w] = x;
  __syncthreads();
  if (w == 0) {
    int v = warp_sums[lane];
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= o) v += y;
    }
    warp_sums[lane] = v;
  }
  __syncthreads();
  const int r = x + (w ? warp_sums[w - 1] : 0);
  __syncthreads();  // warp_sums may be reused
  return r;
}

__global__ void __launch_bounds__(1024) plan_count_kernel(PlanArgs a, int level, int32_t* tile_sum) {
  __shared__ int32_t warp_sums[32];
  const int prev = level == 0 ? 1 : a.meta[(level - 1) * (a.d + 2)];
  const int64_t size = (int64_t)a.d * prev;
  const int64_t q = (int64_t)blockIdx.x * 1024 + threadIdx.x;
  if ((int64_t)blockIdx.x * 1024 >= size) {  // block-uniform
    if (threadIdx.x == 0) tile_sum[blockIdx.x] = 0;
    return;
  }
  const int incl = block_incl_scan_1024(q < size ? a.flags[q] : 0, warp_sums);
  if (threadIdx.x == 1023) tile_sum[blockIdx.x] = incl;
}

__global__ void __launch_bounds__(1024) plan_offsets_kernel(PlanArgs a, int level, int32_t* tile_sum, int n_tiles) {
  __shared__ int32_t warp_sums[32];
  __shared__ int32_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < n_tiles; base += 1024) {
    const int t = base + threadIdx.x;
    const int v = t < n_tiles ? tile_sum[t] : 0;
    const int incl = block_incl_scan_1024(v, warp_sums);
    const int c0 = carry;
    if (t < n_tiles) tile_sum[t] = c0 + incl - v;  // exclusive offset of tile t
    __syncthreads();
    if (threadIdx.x == 1023) carry = c0 + incl;
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    int32_t* meta = a.meta + level * (a.d + 2);
    meta[0] = carry;
    meta[1 + a.d] = carry;
  }
}

__global__ void __launch_bounds__(1024) plan_place_kernel(PlanArgs a, int level, const int32_t* tile_off,
                                                          int32_t* parent, int32_t* nval) {
  __shared__ int32_t warp_sums[32];
  const int prev = level == 0 ? 1 : a.meta[(level - 1) * (a.d + 2)];
  const int64_t size = (int64_t)a.d * prev;
  if ((int64_t)blockIdx.x * 1024 >= size) return;  // block-uniform
  int32_t* meta = a.meta + level * (a.d + 2);
  const int64_t q = (int64_t)blockIdx.x * 1024 + threadIdx.x;
  const int f = q < size ? a.flags[q] : 0;
  const int excl = tile_off[blockIdx.x] + block_incl_scan_1024(f, warp_sums) - f;
  if (q < size) {
    a.idx[q] = excl;
    a.flags[q] = 0;
    if (q % prev == 0) meta[1 + q / prev] = excl;  // first row of photon number q / prev
    if (f) {
      parent[excl] = int32_t(q % prev);
      nval[excl] = int32_t(q / prev);
    }
  }
}

__global__ void plan_assign_kernel(PlanArgs a) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= a.P) return;
  a.cur[p] = a.idx[a.keys[p]];
}

struct SidePlan {
  std::vector<int> sites;                 // site of each level (left: 0..m, right: M-1..m+1)
  std::vector<int32_t> meta;              // host copy: per level rows, group[0..d]
  int32_t* parent = nullptr;              // device: level l rows at parent + l * P
  int32_t* nval = nullptr;
  int32_t* final_row = nullptr;           // device: [P] row at the last level
  int64_t P = 0;
  int d = 0;
  int rows(int l) const { return meta[(size_t)l * (d + 2)]; }
  int group(int l, int n) const { return meta[(size_t)l * (d + 2) + 1 + n]; }
};

static int plan_side_device(bsg_handle_t h, const int32_t* pat, int64_t P, int M, int d, const std::vector<int>& sites,
                            SidePlan& sp, int32_t* work, int* err, cudaStream_t st) {
  const int nl = int(sites.size());
  sp.sites = sites;
  sp.P = P;
  sp.d = d;
  // work: cur, keys [P] | flags, idx [d P] | meta [nl (d + 2)] | parent, nval [nl P] | tile sums
  PlanArgs a{};
  a.pat = pat;
  a.P = P;
  a.M = M;
  a.d = d;
  a.cur = work;
  a.keys = a.cur + P;
  a.flags = a.keys + P;
  a.idx = a.flags + (size_t)d * P;
  a.meta = a.idx + (size_t)d * P;
  a.err = err;
  sp.parent = a.meta + (size_t)nl * (d + 2);
  sp.nval = sp.parent + (size_t)nl * P;
  int32_t* tile_sum = sp.nval + (size_t)nl * P;  // [ceil(d P / 1024)]
  sp.final_row = a.cur;
  BSG_CUDA(cudaMemsetAsync(a.flags, 0, (size_t)d * P * 4, st));
  const unsigned blocks = unsigned((P + 255) / 256);
  // level l has at most d * min(P, d^l) keys: small levels use the one-CTA
  // scan, large ones the three-launch multi-CTA scan over d * P keys
  const int n_tiles = int(((int64_t)d * P + 1023) / 1024);
  int64_t bound = 1;  // d^l, capped
  for (int l = 0; l < nl; ++l) {
    bound = std::min<int64_t>(bound * d, (int64_t)d * P);
    int32_t* par = sp.parent + (size_t)l * P;
    int32_t* nv = sp.nval + (size_t)l * P;
    BSG_PROFILED(h, BSG_K_PREP, st, (double)P, (plan_mark_kernel<<<blocks, 256, 0, st>>>(a, sites[l], l)));
    if (bound <= 8192 || n_tiles <= 8) {
      BSG_PROFILED(h, BSG_K_PREP, st, (double)P, (plan_scan_kernel<<<1, 1024, 0, st>>>(a, l, par, nv)));
    } else {
      BSG_PROFILED(h, BSG_K_PREP, st, (double)P, (plan_count_kernel<<<n_tiles, 1024, 0, st>>>(a, l, tile_sum)));
      BSG_PROFILED(h, BSG_K_PREP, st, (double)P,
                   (plan_offsets_kernel<<<1, 1024, 0, st>>>(a, l, tile_sum, n_tiles)));
      BSG_PROFILED(h, BSG_K_PREP, st, (double)P,
                   (plan_place_kernel<<<n_tiles, 1024, 0, st>>>(a, l, tile_sum, par, nv)));
    }
  }
  // rows of the last level
  BSG_PROFILED(h, BSG_K_PREP, st, (double)P, (plan_assign_kernel<<<blocks, 256, 0, st>>>(a)));
  sp.meta.resize((size_t)nl * (d + 2));
  BSG_CUDA(cudaMemcpyAsync(sp.meta.data(), a.meta, sp.meta.size() * 4, cudaMemcpyDeviceToHost, st));
  return BSG_OK;
}

static size_t plan_side_words(int64_t P, int d, int levels) {
  return (size_t)2 * P + (size_t)2 * d * P + (size_t)levels * (d + 2) + (size_t)2 * levels * P +
         (size_t)((int64_t)d * P + 1023) / 1024;
}

template <class R>
static int run_contraction(bsg_handle_t h, const void* const* Gd, const double* lam, int M, int chi, int d,
                           const SidePlan& left, const SidePlan& right, int64_t P, double* amp, bool umma,
                           bool sliced, char* ws, cudaStream_t st) {
  using T = typename Cx<R>::T;
  // device memory: two env buffers per side (ping-pong)
  int64_t max_rows = 1;
  for (int l = 0; l < (int)left.sites.size(); ++l) max_rows = std::max<int64_t>(max_rows, left.rows(l));
  for (int l = 0; l < (int)right.sites.size(); ++l) max_rows = std::max<int64_t>(max_rows, right.rows(l));
  auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
  const size_t env_bytes = al((size_t)max_rows * chi * sizeof(T));
  const size_t a_bytes = umma ? al((size_t)max_rows * 2 * chi * 4) : 0;
  const size_t b_bytes = umma ? al((size_t)d * 4 * chi * chi * 4) : 0;
  // sliced: S BF16 slices of the level's A rows and of all d B blocks, row exponents
  int S = 0, bits = 0;
  if (sliced) sliced_params(2 * chi, &S, &bits);
  const size_t sa_bytes = sliced ? al(sliced_operand_bytes(max_rows, 2 * chi, S)) : 0;
  const size_t sb_bytes = sliced ? al(sliced_operand_bytes((int64_t)d * 2 * chi, 2 * chi, S)) : 0;
  const size_t se_bytes = sliced ? al((size_t)(max_rows + (int64_t)d * 2 * chi) * 4) : 0;
  const size_t st_bytes = sliced ? al(sliced_gamma_scratch_bytes(chi, d)) : 0;
  const size_t need = 4 * env_bytes + 2 * a_bytes + 2 * b_bytes + sa_bytes + sb_bytes + se_bytes + st_bytes + 256;
  BSG_TRY(h->contract_ws.ensure(need));
  char* base = reinterpret_cast<char*>(h->contract_ws.ptr);
  char* sp_base = base + 4 * env_bytes;
  float* Ahi = reinterpret_cast<float*>(sp_base);
  float* Alo = reinterpret_cast<float*>(sp_base + a_bytes);
  float* Bhi = reinterpret_cast<float*>(sp_base + 2 * a_bytes);
  float* Blo = reinterpret_cast<float*>(sp_base + 2 * a_bytes + b_bytes);
  char* sl_base = sp_base + 2 * a_bytes + 2 * b_bytes;
  void* Asl = sl_base;
  void* Bsl = sl_base + sa_bytes;
  int* ea = reinterpret_cast<int*>(sl_base + sa_bytes + sb_bytes);
  int* eb = ea + max_rows;
  void* Tsl = sl_base + sa_bytes + sb_bytes + se_bytes;  // transposed Gamma block of the level's site
  int* d_err = reinterpret_cast<int*>(sl_base + sa_bytes + sb_bytes + se_bytes + st_bytes);
  if (umma || sliced) BSG_CUDA(cudaMemsetAsync(d_err, 0, 4, st));
  T* E[4] = {reinterpret_cast<T*>(base), reinterpret_cast<T*>(base + env_bytes),
             reinterpret_cast<T*>(base + 2 * env_bytes), reinterpret_cast<T*>(base + 3 * env_bytes)};
  (void)ws;
  // tensor-core path: one grouped GEMM per level; its row tiles {first row,
  // end row of the photon-number group, B block row, 0}, all levels at once
  const int K2 = 2 * chi;
  std::vector<int4> tiles;
  std::vector<int> tile_off[2];
  if (umma || sliced) {
    const SidePlan* sps[2] = {&left, &right};
    for (int sd = 0; sd < 2; ++sd) {
      tile_off[sd].assign(sps[sd]->sites.size() + 1, 0);
      for (size_t l = 1; l < sps[sd]->sites.size(); ++l) {
        tile_off[sd][l] = int(tiles.size());
        for (int n = 0; n < d; ++n) {
          const int r0 = sps[sd]->group(int(l), n), r1 = sps[sd]->group(int(l), n + 1);
          for (int t0 = r0; t0 < r1; t0 += 128) tiles.push_back(make_int4(t0, r1, n * K2, 0));
        }
      }
      tile_off[sd][sps[sd]->sites.size()] = int(tiles.size());
    }
  }
  int4* d_tiles = nullptr;
  if ((umma || sliced) && !tiles.empty()) {
    BSG_TRY(h->plan.ensure(tiles.size() * sizeof(int4)));
    BSG_TRY(h->host_stage2.ensure(tiles.size() * sizeof(int4)));
    std::memcpy(h->host_stage2.ptr, tiles.data(), tiles.size() * sizeof(int4));
    d_tiles = reinterpret_cast<int4*>(h->plan.ptr);
    BSG_CUDA(cudaMemcpyAsync(d_tiles, h->host_stage2.ptr, tiles.size() * sizeof(int4), cudaMemcpyHostToDevice, st));
  }

  double flops = 0.0;
  auto side = [&](const SidePlan& sp, T* e0, T* e1, bool is_left) -> T* {
    T* prev = e0;
    T* curb = e1;
    // level 0: row 0 of Gamma_0 (left) or column 0 of Gamma_{M-1} (right)
    {
      const int s = sp.sites[0];
      const T* G = reinterpret_cast<const T*>(Gd[s]);
      const int64_t rows = sp.rows(0);
      // left: Gamma_0[0, a, n] at a*d + n ; right: Gamma_{M-1}[a, 0, n] at a*chi*d + n
      const int64_t stride = is_left ? d : (int64_t)chi * d;
      const int64_t tot = rows * chi;
      env_init_kernel<R><<<unsigned((tot + 255) / 256), 256, 0, st>>>(G, stride, sp.nval, (int)rows, chi, prev);
    }
    for (size_t l = 1; l < sp.sites.size(); ++l) {
      const int s = sp.sites[l];
      const T* G = reinterpret_cast<const T*>(Gd[s]);
      const int32_t* parent = sp.parent + l * sp.P;
      // left uses Lambda_{s-1}, right uses Lambda_s
      const double* lm = lam + (size_t)(is_left ? s - 1 : s) * chi;
      if constexpr (std::is_same<R, double>::value) {
        if (sliced) {
          // all photon numbers of the level in one grouped sliced GEMM
          const int rows = sp.rows(int(l));
          const int sd = is_left ? 0 : 1;
          const int t0 = tile_off[sd][l], nt = tile_off[sd][l + 1] - t0;
          if (sliced_slice_gamma(reinterpret_cast<const double2*>(G), chi, d, is_left, S, bits, Bsl, eb, Tsl, st) !=
                  BSG_OK ||
              sliced_slice_env(reinterpret_cast<const double2*>(prev), parent, lm, rows, chi, S, bits, Asl, ea, st) !=
                  BSG_OK ||
              sliced_gemm(h, Asl, rows, ea, Bsl, d * K2, eb, reinterpret_cast<double*>(curb), rows, K2, K2, K2, S,
                          bits, d_err, st, false, d_tiles + t0, nt) != BSG_OK)
            return nullptr;
          flops += 8.0 * rows * (double)chi * chi;
          std::swap(prev, curb);
          continue;
        }
      }
      if constexpr (std::is_same<R, float>::value) {
        if (umma) {
          // all photon numbers of the level in one grouped GEMM
          const int rows = sp.rows(int(l));
          const int sd = is_left ? 0 : 1;
          const int t0 = tile_off[sd][l], nt = tile_off[sd][l + 1] - t0;
          build_bt_kernel<<<dim3(unsigned(((int64_t)K2 * K2 + 255) / 256), d), 256, 0, st>>>(
              reinterpret_cast<const float2*>(G), chi, d, is_left ? 1 : 0, Bhi, Blo);
          build_a_kernel<<<unsigned(((int64_t)rows * K2 + 255) / 256), 256, 0, st>>>(
              reinterpret_cast<const float2*>(prev), parent, lm, rows, chi, Ahi, Alo);
          if (gemm_tf32x3(h, Ahi, Alo, Bhi, Blo, reinterpret_cast<float*>(curb), rows, K2, K2, K2, d_err, st, false,
                          d_tiles + t0, nt, d * K2) != BSG_OK)
            return nullptr;
          flops += 8.0 * rows * (double)chi * chi;
          std::swap(prev, curb);
          continue;
        }
      }
      for (int n = 0; n < d; ++n) {
        const int r0 = sp.group(int(l), n), r1 = sp.group(int(l), n + 1);
        if (r1 <= r0) continue;
        GemmArgs<R> g{};
        g.A = prev;
        g.pidx = parent + r0;
        g.lam = lm;
        g.B = G + n;
        g.sk = is_left ? (int64_t)chi * d : d;
        g.sc = is_left ? d : (int64_t)chi * d;
        g.C = curb + (int64_t)r0 * chi;
        g.rows = r1 - r0;
        g.K = chi;
        g.N = chi;
        dim3 grid((chi + TN - 1) / TN, (g.rows + TM - 1) / TM);
        cgemm_kernel<R><<<grid, 256, 0, st>>>(g);
        flops += 8.0 * g.rows * (double)chi * chi;
      }
      std::swap(prev, curb);
    }
    return prev;
  };
  cudaEvent_t ev = nullptr;
  if (h->prof.on) BSG_TRY(h->prof.begin(BSG_K_CONTRACT, st, &ev));
  T* Lend = side(left, E[0], E[1], true);
  if (!Lend) return BSG_ERR_CUDA;
  T* Rend = side(right, E[2], E[3], false);
  if (!Rend) return BSG_ERR_CUDA;
  const int mid = left.sites.back();
  final_dot_kernel<R><<<unsigned((P * 32 + 255) / 256), 256, std::is_same<R, float>::value ? chi * sizeof(float) : 0,
                        st>>>(
      Lend, left.final_row, Rend, right.final_row, lam + (size_t)mid * chi, chi, P, reinterpret_cast<double2*>(amp));
  BSG_CUDA(cudaGetLastError());
  if (h->prof.on) BSG_TRY(h->prof.end(BSG_K_CONTRACT, st, ev, flops + 8.0 * P * chi));
  int err = 0;
  if (umma || sliced) BSG_CUDA(cudaMemcpyAsync(&err, d_err, 4, cudaMemcpyDeviceToHost, st));
  BSG_CUDA(cudaStreamSynchronize(st));
  if (err) {
    set_error("bsg_pattern_amplitudes: a tensor-core pipeline wait timed out");
    return BSG_ERR_CUDA;
  }
  return BSG_OK;
}

}  // namespace bsg

using namespace bsg;

extern "C" int bsg_pattern_amplitudes(bsg_handle_t h, const void* const* Gammas, const double* Lambdas, int M, int chi,
                                      int d, const int32_t* patterns, int64_t P, int precision, double* amp,
                                      bsg_stream_t stream) {
  BSG_CHECK_ARG(h, "bsg_pattern_amplitudes: null handle");
  BSG_CHECK_ARG(Gammas && Lambdas && amp && (patterns || P == 0), "bsg_pattern_amplitudes: null pointer");
  BSG_CHECK_ARG(M >= 2 && chi >= 1 && d >= 1 && P >= 0, "bsg_pattern_amplitudes: bad sizes M=%d chi=%d d=%d", M, chi,
                d);
  BSG_CHECK_ARG(precision == BSG_PREC_FP64 || precision == BSG_PREC_SPLIT || precision == BSG_PREC_FP32 ||
                    precision == BSG_PREC_SLICED,
                "bsg_pattern_amplitudes: bad precision %d", precision);
  BSG_CHECK_ARG(precision != BSG_PREC_SLICED || chi % 4 == 0,
                "bsg_pattern_amplitudes: the sliced tensor-core path needs chi %% 4 == 0 (chi=%d)", chi);
  for (int i = 0; i < M; ++i) BSG_CHECK_ARG(Gammas[i], "bsg_pattern_amplitudes: Gamma %d is NULL", i);
  BSG_CUDA(cudaSetDevice(h->device));
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  if (P == 0) return BSG_OK;
  const int m = (M - 1) / 2;  // left levels 0..m, right levels M-1..m+1
  std::vector<int> ls, rs;
  for (int i = 0; i <= m; ++i) ls.push_back(i);
  for (int i = M - 1; i > m; --i) rs.push_back(i);
  BSG_CHECK_ARG(int(ls.size()) <= kMaxLevels && int(rs.size()) <= kMaxLevels, "bsg_pattern_amplitudes: M too large");
  BSG_CHECK_ARG((int64_t)d * P < INT32_MAX, "bsg_pattern_amplitudes: d * P = %lld too large", (long long)d * P);
  // planning workspace (both sides) + an error word
  const size_t wl = plan_side_words(P, d, int(ls.size())), wr = plan_side_words(P, d, int(rs.size()));
  BSG_TRY(h->sample_ws.ensure((wl + wr) * 4 + 256 + (size_t)M * P * 4));
  int32_t* work = reinterpret_cast<int32_t*>(h->sample_ws.ptr);
  int* perr = reinterpret_cast<int*>(work + wl + wr);
  int32_t* patT = work + wl + wr + 64;  // [M, P]
  BSG_CUDA(cudaMemsetAsync(perr, 0, 4, st));
  BSG_PROFILED(h, BSG_K_PREP, st, (double)P * M,
               (transpose_patterns_kernel<<<dim3(unsigned((P + 31) / 32), unsigned((M + 31) / 32)), dim3(32, 8), 0,
                                            st>>>(patterns, P, M, patT)));
  SidePlan left, right;
  BSG_TRY(plan_side_device(h, patT, P, M, d, ls, left, work, perr, st));
  BSG_TRY(plan_side_device(h, patT, P, M, d, rs, right, work + wl, perr, st));
  int herr = 0;
  BSG_CUDA(cudaMemcpyAsync(&herr, perr, 4, cudaMemcpyDeviceToHost, st));
  BSG_CUDA(cudaStreamSynchronize(st));  // level sizes for the GEMM launches
  if (herr) {
    set_error("bsg_pattern_amplitudes: a photon number is outside [0, d=%d)", d);
    return BSG_ERR_INVALID;
  }
  if (precision == BSG_PREC_FP64 || precision == BSG_PREC_SLICED)
    return run_contraction<double>(h, Gammas, Lambdas, M, chi, d, left, right, P, amp, false,
                                   precision == BSG_PREC_SLICED, nullptr, st);
  if (precision == BSG_PREC_SPLIT && chi % 2 != 0) {
    set_error("bsg_pattern_amplitudes: the tensor-core path needs an even chi");
    return BSG_ERR_INVALID;
  }
  return run_contraction<float>(h, Gammas, Lambdas, M, chi, d, left, right, P, amp, precision == BSG_PREC_SPLIT,
                                false, nullptr, st);
}

extern "C" int bsg_contract_patterns(bsg_handle_t h, const void* const* Gammas, const double* Lambdas, int M, int chi,
                                     int d, const int32_t* patterns, int64_t P, int precision, double* amp,
                                     bsg_stream_t stream) {
  return bsg_pattern_amplitudes(h, Gammas, Lambdas, M, chi, d, patterns, P, precision, amp, stream);
}
