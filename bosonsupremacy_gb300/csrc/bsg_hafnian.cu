// Batched repetition-aware hafnians and the fused per-site Gamma build.
//
// Every work item is one hafnian of Sigma restricted to a target index list
// with repeats.  Items are bucketed by the multiplicity partition of their
// target; a warp takes 32 items of one bucket and runs that bucket's
// partition program (bsg_programs.cpp) in lock-step, one item per lane, with
// the per-lane A (class pair) table and F (DP state) table in a per-warp
// scratch slice laid out [entry][lane] so every access is one coalesced line.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <type_traits>
#include <vector>

#include "bsg_arith.cuh"
#include "bsg_internal.h"

namespace bsg {

constexpr int kMaxInv = 64;
__constant__ double c_inv_d[kMaxInv];
__constant__ float2 c_inv_f[kMaxInv];
__constant__ double c_sqrt_fact[kMaxInv];  // sqrt(n!)
__constant__ double c_fact[kMaxInv];       // n! (as double)

static int ensure_tables() {
  static bool done = false;  // per process; constant memory is per device module
  static int dev_done = -1;
  int dev = 0;
  BSG_CUDA(cudaGetDevice(&dev));
  if (done && dev_done == dev) return BSG_OK;
  double inv_d[kMaxInv], sf[kMaxInv], f[kMaxInv];
  float2 inv_f[kMaxInv];
  for (int r = 0; r < kMaxInv; ++r) {
    inv_d[r] = r ? 1.0 / r : 0.0;
    float hi = float(inv_d[r]);
    inv_f[r] = make_float2(hi, float(inv_d[r] - double(hi)));
    f[r] = std::tgamma(double(r) + 1.0);
    sf[r] = std::sqrt(f[r]);
  }
  BSG_CUDA(cudaMemcpyToSymbol(c_inv_d, inv_d, sizeof(inv_d)));
  BSG_CUDA(cudaMemcpyToSymbol(c_inv_f, inv_f, sizeof(inv_f)));
  BSG_CUDA(cudaMemcpyToSymbol(c_sqrt_fact, sf, sizeof(sf)));
  BSG_CUDA(cudaMemcpyToSymbol(c_fact, f, sizeof(f)));
  done = true;
  dev_done = dev;
  return BSG_OK;
}

// ---------------------------------------------------------------------------
// Label rows: sparse (Sigma index, multiplicity) lists sorted by multiplicity,
// partition key, row sum and sqrt(prod num!) -- one thread per row.
// ---------------------------------------------------------------------------
struct RowTable {
  int32_t* entries;  // [rows, kMaxNnz] packed (sigma_idx << 8) | mult
  int32_t* nnz;      // [rows]
  int32_t* sum;      // [rows]
  uint64_t* key;     // [rows]
  double* rowfact;   // [rows] sqrt(prod num!)
};
constexpr int kMaxNnz = BSG_MAX_LABEL_NNZ;

__global__ void label_rows_kernel(const int8_t* __restrict__ num, int rows, int m, int sigma_offset, RowTable t,
                                  int* __restrict__ err) {
  int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows) return;
  int ent[kMaxNnz];
  int cnt = 0, sum = 0;
  uint64_t key = 0;
  double rf = 1.0;
  const int8_t* row = num + (size_t)r * m;
  for (int q = 0; q < m; ++q) {
    int v = row[q];
    if (v == 0) continue;
    if (v < 0 || v > kKeyMaxMult || cnt >= kMaxNnz) {
      atomicExch(err, 1);
      continue;
    }
    // insertion by multiplicity (stable on mode index)
    int e = ((sigma_offset + q) << 8) | v;
    int p = cnt++;
    while (p > 0 && (ent[p - 1] & 0xff) > v) {
      ent[p] = ent[p - 1];
      --p;
    }
    ent[p] = e;
    sum += v;
    key += uint64_t(1) << (kKeyBits * (v - 1));
    rf *= c_sqrt_fact[v];
  }
  for (int i = 0; i < cnt; ++i) t.entries[(size_t)r * kMaxNnz + i] = ent[i];
  t.nnz[r] = cnt;
  t.sum[r] = sum;
  t.key[r] = key;
  t.rowfact[r] = rf;
}

// ---------------------------------------------------------------------------
// Site classification: scatter every even-order (a, b, j) item into the
// bucket of its partition program.  Rows are visited in key-sorted order so
// that a warp usually shares one bucket (one aggregated atomic).
// ---------------------------------------------------------------------------
struct SitePlanDev {
  const int32_t* perm_l;  // sorted position -> left row
  const int32_t* grp_l;   // sorted position -> left key group
  const int32_t* perm_r;
  const int32_t* grp_r;
  const int32_t* bucket_of;  // [d][ngl][ngr] -> bucket or -1 (odd order)
  const int32_t* bucket_off;  // [nb] first slot
  int32_t* cursor;            // [nb]
  int32_t* items;             // slots
  int ngl, ngr, kl, kr, d;
};

__global__ void site_scatter_kernel(SitePlanDev p) {
  const int64_t total = (int64_t)p.d * p.kr * p.kl;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int lane = threadIdx.x & 31;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < total; base += stride) {
    int64_t i = base + threadIdx.x;
    int bucket = -1;
    int32_t item = 0;
    if (i < total) {
      int bs = int(i % p.kl);
      int64_t rest = i / p.kl;
      int as = int(rest % p.kr);
      int j = int(rest / p.kr);
      bucket = p.bucket_of[((size_t)j * p.ngl + p.grp_l[bs]) * p.ngr + p.grp_r[as]];
      item = (p.perm_r[as] << 20) | (p.perm_l[bs] << 8) | j;
    }
    unsigned active = __ballot_sync(0xffffffffu, bucket >= 0);
    if (bucket >= 0) {
      unsigned peers = __match_any_sync(active, bucket);
      int leader = __ffs(peers) - 1;
      int rank = __popc(peers & ((1u << lane) - 1));
      int slot0 = 0;
      if (lane == leader) slot0 = atomicAdd(&p.cursor[bucket], __popc(peers));
      slot0 = __shfl_sync(peers, slot0, leader);
      p.items[p.bucket_off[bucket] + slot0 + rank] = item;
    }
  }
}

// ---------------------------------------------------------------------------
// The DP kernel
// ---------------------------------------------------------------------------
struct ProgDev {
  const int32_t* k;
  const int32_t* nstates;
  const int32_t* state_off;
  const int32_t* st_trans_off;
  const int32_t* st_trans_cnt;
  const int32_t* st_ra;
  const uint32_t* trans;
};

enum { MODE_SITE = 0, MODE_TARGETS = 1, MODE_MATRICES = 2 };

struct DPArgs {
  ProgDev prog;
  const int32_t* items;
  const int32_t* chunk_prog;
  int64_t n_chunks;
  unsigned long long* counter;
  void* scratch;
  int pairs_max, states_max;
  const void* sigma;  // policy-typed
  int n_len;
  // site mode
  const int32_t* l_ent;
  const int32_t* l_nnz;
  const double* l_rowfact;
  const double* lambda;
  const int32_t* r_ent;
  const int32_t* r_nnz;
  const double* r_rowfact;
  const double* Z;
  int d, chi, out_c128;
  void* gamma;
  // target / matrices mode
  const int32_t* targets;
  int n;
  const double* den;
  double2* out;
};

template <int MODE>
__device__ __forceinline__ int build_classes(const DPArgs& a, int32_t item, int* cls, double& fac, int& j_out,
                                             int& ra_out, int& rb_out, int64_t& sig_base) {
  sig_base = 0;
  if (MODE == MODE_SITE) {
    int alpha = (item >> 20) & 0xfff, beta = (item >> 8) & 0xfff, j = item & 0xff;
    j_out = j;
    ra_out = alpha;
    rb_out = beta;
    const int32_t* le = a.l_ent + (size_t)beta * kMaxNnz;
    const int32_t* re = a.r_ent + (size_t)alpha * kMaxNnz;
    int nl = a.l_nnz[beta], nr = a.r_nnz[alpha];
    int il = 0, ir = 0, k = 0;
    bool jpend = j > 0;
    // three-way merge by multiplicity (j class first on ties)
    while (jpend || il < nl || ir < nr) {
      int ml = il < nl ? (le[il] & 0xff) : 1 << 20;
      int mr = ir < nr ? (re[ir] & 0xff) : 1 << 20;
      if (jpend && j <= ml && j <= mr) {
        cls[k++] = 0;
        jpend = false;
      } else if (ml <= mr) {
        cls[k++] = le[il++] >> 8;
      } else {
        cls[k++] = re[ir++] >> 8;
      }
    }
    fac = 1.0;
    return k;
  } else {
    // MODE_TARGETS: row of a [B, n] index array; MODE_MATRICES: 0..n-1
    const int n = a.n;
    int t[BSG_MAX_ORDER];
    if (MODE == MODE_TARGETS) {
      const int32_t* row = a.targets + (int64_t)item * n;
      for (int i = 0; i < n; ++i) {
        int v = row[i];
        int p = i;
        while (p > 0 && t[p - 1] > v) {
          t[p] = t[p - 1];
          --p;
        }
        t[p] = v;
      }
    } else {
      for (int i = 0; i < n; ++i) t[i] = i;
      sig_base = (int64_t)item * n * n;
    }
    // run-length classes, then order by multiplicity (stable)
    int ci[BSG_MAX_CLASSES], cm[BSG_MAX_CLASSES];
    int k = 0;
    fac = 1.0;
    for (int i = 0; i < n;) {
      int v = t[i], c = 0;
      while (i < n && t[i] == v) {
        ++i;
        ++c;
      }
      if (k < BSG_MAX_CLASSES) {
        int p = k++;
        while (p > 0 && cm[p - 1] > c) {
          ci[p] = ci[p - 1];
          cm[p] = cm[p - 1];
          --p;
        }
        ci[p] = v;
        cm[p] = c;
      }
      fac *= c_fact[c];
    }
    for (int c = 0; c < k; ++c) cls[c] = ci[c];
    return k;
  }
}

template <class P, int MODE>
__global__ void __launch_bounds__(256) dp_kernel(DPArgs a) {
  using C = typename P::C;
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const size_t slice = (size_t)(a.pairs_max + a.states_max) * 32;
  C* Ab = reinterpret_cast<C*>(a.scratch) + (size_t)warp * slice;
  C* Fb = Ab + (size_t)a.pairs_max * 32;
  const C* sig = reinterpret_cast<const C*>(a.sigma);
  while (true) {
    unsigned long long c = 0;
    if (lane == 0) c = atomicAdd(a.counter, 1ull);
    c = __shfl_sync(0xffffffffu, c, 0);
    if ((int64_t)c >= a.n_chunks) break;
    const int prog = a.chunk_prog[c];
    const int32_t item = a.items[c * 32 + lane];
    const bool live = item >= 0;
    const int kp = a.prog.k[prog];
    const int ns = a.prog.nstates[prog];
    const int so = a.prog.state_off[prog];

    int cls[BSG_MAX_CLASSES];
    double fac = 1.0;
    int j = 0, ia = 0, ib = 0;
    int64_t sb = 0;
    int k = kp;
    if (live) {
      k = build_classes<MODE>(a, item, cls, fac, j, ia, ib, sb);
    } else {
      for (int q = 0; q < kp; ++q) cls[q] = 0;
    }
    // gather the class-pair table (diagonal included)
    for (int bq = 0; bq < kp; ++bq) {
      const int64_t rowb = sb + (int64_t)cls[bq] * a.n_len;
      for (int aq = 0; aq <= bq; ++aq) {
        Ab[(size_t)pair_index(aq, bq) * 32 + lane] = sig[rowb + cls[aq]];
      }
    }
    (void)k;
    // run the program
    Fb[lane] = P::one();
    for (int s = 1; s < ns; ++s) {
      const int off = __ldg(a.prog.st_trans_off + so + s);
      const int cnt = __ldg(a.prog.st_trans_cnt + so + s);
      const int ra = __ldg(a.prog.st_ra + so + s);
      typename P::Acc acc = P::zero();
      for (int t = 0; t < cnt; ++t) {
        const uint32_t w = __ldg(a.prog.trans + off + t);
        const C av = Ab[(size_t)(w & 0xfffu) * 32 + lane];
        const C fv = Fb[(size_t)(w >> 12) * 32 + lane];
        P::mac(acc, av, fv);
      }
      Fb[(size_t)s * 32 + lane] = P::finish(acc, ra, c_inv_d, c_inv_f);
    }
    if (!live) continue;
    double2 v = P::to_c128(Fb[(size_t)(ns - 1) * 32 + lane]);
    if (MODE == MODE_SITE) {
      double scale = c_sqrt_fact[j] * a.l_rowfact[ib] * a.r_rowfact[ia] / a.Z[0];
      if (a.lambda) scale /= a.lambda[ib];
      const size_t o = ((size_t)ia * a.chi + ib) * a.d + j;
      if (a.out_c128) {
        reinterpret_cast<double2*>(a.gamma)[o] = make_double2(v.x * scale, v.y * scale);
      } else {
        reinterpret_cast<float2*>(a.gamma)[o] = make_float2(float(v.x * scale), float(v.y * scale));
      }
    } else {
      double s = fac;
      if (a.den) s /= a.den[item];
      a.out[item] = make_double2(v.x * s, v.y * s);
    }
  }
}

// Target-row partition keys (odd order -> ~0).
__global__ void target_keys_kernel(const int32_t* __restrict__ targets, int n, int64_t B, int n_len,
                                   uint64_t* __restrict__ keys, int* __restrict__ err) {
  int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  if (n & 1) {
    keys[b] = ~0ull;
    return;
  }
  int t[BSG_MAX_ORDER];
  const int32_t* row = targets + b * n;
  for (int i = 0; i < n; ++i) {
    int v = row[i];
    if (v < 0 || v >= n_len) {
      atomicExch(err, 1);
      v = 0;
    }
    int p = i;
    while (p > 0 && t[p - 1] > v) {
      t[p] = t[p - 1];
      --p;
    }
    t[p] = v;
  }
  uint64_t key = 0;
  int k = 0;
  for (int i = 0; i < n;) {
    int v = t[i], c = 0;
    while (i < n && t[i] == v) {
      ++i;
      ++c;
    }
    if (c > kKeyMaxMult) atomicExch(err, 2);
    key += uint64_t(1) << (kKeyBits * ((c > kKeyMaxMult ? kKeyMaxMult : c) - 1));
    ++k;
  }
  if (k > BSG_MAX_CLASSES) atomicExch(err, 3);
  keys[b] = key;
}

template <class C>
__global__ void convert_kernel(const double2* __restrict__ src, C* __restrict__ dst, int64_t n) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if constexpr (std::is_same<C, double2>::value) {
    dst[i] = src[i];
  } else if constexpr (std::is_same<C, float2>::value) {
    dst[i] = PrecF32::from_c128(src[i]);
  } else {
    dst[i] = PrecSplit::from_c128(src[i]);
  }
}

static size_t prec_bytes(int precision) {
  return precision == BSG_PREC_FP64 ? sizeof(double2) : precision == BSG_PREC_SPLIT ? sizeof(float4) : sizeof(float2);
}

// Converts Sigma (c128) into the precision's storage type inside `buf`.
static int convert_sigma(bsg_handle_t h, const double* src, int64_t n, int precision, bsg::DevBuf& buf,
                         const void** out, cudaStream_t st) {
  if (precision == BSG_PREC_FP64 || n == 0) {
    *out = src;
    return BSG_OK;
  }
  BSG_TRY(buf.ensure((size_t)n * prec_bytes(precision)));
  int threads = 256;
  int64_t blocks = (n + threads - 1) / threads;
  if (precision == BSG_PREC_SPLIT)
    convert_kernel<float4><<<(unsigned)blocks, threads, 0, st>>>(reinterpret_cast<const double2*>(src),
                                                                 reinterpret_cast<float4*>(buf.ptr), n);
  else
    convert_kernel<float2><<<(unsigned)blocks, threads, 0, st>>>(reinterpret_cast<const double2*>(src),
                                                                 reinterpret_cast<float2*>(buf.ptr), n);
  BSG_CUDA(cudaGetLastError());
  *out = buf.ptr;
  return BSG_OK;
}

// Host-side bucket layout shared by both planners.
struct Buckets {
  std::vector<int32_t> progs;    // bucket -> program
  std::vector<int64_t> counts;   // bucket -> items
  std::vector<int32_t> offsets;  // bucket -> first slot (multiple of 32)
  std::vector<int32_t> chunk_prog;
  int64_t slots = 0;
  int pairs_max = 1, states_max = 1;
};

static int layout_buckets(const bsg::ProgramSet& ps, Buckets& bk) {
  // order buckets by per-item cost, expensive first, so the work queue
  // starts the long programs early
  const int nb = int(bk.progs.size());
  std::vector<int> order(nb);
  std::iota(order.begin(), order.end(), 0);
  auto cost = [&](int b) {
    int p = bk.progs[b];
    int s0 = ps.state_off[p], ns = ps.nstates[p];
    int64_t tr = ps.st_trans_off[s0 + ns - 1] + ps.st_trans_cnt[s0 + ns - 1] - ps.st_trans_off[s0];
    return tr + ns;
  };
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return cost(x) > cost(y); });
  std::vector<int32_t> progs(nb);
  std::vector<int64_t> counts(nb);
  for (int i = 0; i < nb; ++i) {
    progs[i] = bk.progs[order[i]];
    counts[i] = bk.counts[order[i]];
  }
  bk.progs.swap(progs);
  bk.counts.swap(counts);
  bk.offsets.assign(nb, 0);
  bk.chunk_prog.clear();
  int64_t off = 0;
  for (int b = 0; b < nb; ++b) {
    bk.offsets[b] = int32_t(off);
    int64_t ch = (bk.counts[b] + 31) / 32;
    for (int64_t c = 0; c < ch; ++c) bk.chunk_prog.push_back(bk.progs[b]);
    off += ch * 32;
    int p = bk.progs[b];
    int kk = ps.k[p];
    bk.pairs_max = std::max(bk.pairs_max, kk * (kk + 1) / 2);
    bk.states_max = std::max(bk.states_max, ps.nstates[p]);
  }
  if (off > INT32_MAX) {
    set_error("too many work items in one launch (%lld)", (long long)off);
    return BSG_ERR_LIMIT;
  }
  bk.slots = off;
  return BSG_OK;
}

template <class P, int MODE>
static int launch_dp_t(bsg_handle_t h, DPArgs a, const Buckets& bk, cudaStream_t st) {
  using C = typename P::C;
  const size_t per_warp = (size_t)(bk.pairs_max + bk.states_max) * 32 * sizeof(C);
  const int threads = 256;
  int blocks_per_sm = 4;
  int64_t warps = (int64_t)h->num_sms * blocks_per_sm * (threads / 32);
  const size_t budget = size_t(2) << 30;  // at most 2 GiB of per-warp tables
  while (warps > (threads / 32) * (int64_t)h->num_sms && (size_t)warps * per_warp > budget) warps /= 2;
  int64_t need_chunks = std::max<int64_t>(bk.chunk_prog.size(), 1);
  int64_t w_use = std::min<int64_t>(warps, need_chunks);
  int blocks = int((w_use + (threads / 32) - 1) / (threads / 32));
  if (blocks < 1) blocks = 1;
  BSG_TRY(h->warp_scratch.ensure((size_t)blocks * (threads / 32) * per_warp));
  a.scratch = h->warp_scratch.ptr;
  a.pairs_max = bk.pairs_max;
  a.states_max = bk.states_max;
  dp_kernel<P, MODE><<<blocks, threads, 0, st>>>(a);
  BSG_CUDA(cudaGetLastError());
  return BSG_OK;
}

template <int MODE>
static int launch_dp(bsg_handle_t h, int precision, DPArgs a, const Buckets& bk, cudaStream_t st) {
  if (precision == BSG_PREC_FP64) return launch_dp_t<PrecF64, MODE>(h, a, bk, st);
  if (precision == BSG_PREC_SPLIT) return launch_dp_t<PrecSplit, MODE>(h, a, bk, st);
  return launch_dp_t<PrecF32, MODE>(h, a, bk, st);
}

static ProgDev prog_dev(const bsg::ProgramSet& ps) {
  return ProgDev{ps.d_k, ps.d_nstates, ps.d_state_off, ps.d_st_trans_off, ps.d_st_trans_cnt, ps.d_st_ra, ps.d_trans};
}

// Places item ids into bucket slots on the host (target / matrix modes).
static int plan_items_host(bsg_handle_t h, const std::vector<uint64_t>& keys, Buckets& bk,
                           std::vector<int32_t>& items) {
  auto& ps = h->programs;
  std::unordered_map<int32_t, int> bucket_of_prog;
  std::vector<int32_t> item_bucket(keys.size(), -1);
  for (size_t i = 0; i < keys.size(); ++i) {
    if (keys[i] == ~0ull) continue;
    int32_t prog;
    BSG_TRY(program_for_key(ps, keys[i], &prog));
    auto it = bucket_of_prog.find(prog);
    int b;
    if (it == bucket_of_prog.end()) {
      b = int(bk.progs.size());
      bucket_of_prog.emplace(prog, b);
      bk.progs.push_back(prog);
      bk.counts.push_back(0);
    } else {
      b = it->second;
    }
    bk.counts[b]++;
    item_bucket[i] = b;
  }
  // layout reorders buckets; remember the mapping by program
  std::vector<int32_t> progs_before = bk.progs;
  BSG_TRY(layout_buckets(ps, bk));
  std::unordered_map<int32_t, int> newb;
  for (size_t b = 0; b < bk.progs.size(); ++b) newb[bk.progs[b]] = int(b);
  items.assign(bk.slots, -1);
  std::vector<int64_t> cur(bk.progs.size(), 0);
  for (size_t i = 0; i < keys.size(); ++i) {
    if (item_bucket[i] < 0) continue;
    int b = newb[progs_before[item_bucket[i]]];
    items[bk.offsets[b] + cur[b]++] = int32_t(i);
  }
  return BSG_OK;
}

static int run_target_dp(bsg_handle_t h, int mode, const void* sig, int n_len, const int32_t* targets, int n,
                         int64_t B, const double* den, int precision, double* out, const std::vector<uint64_t>& keys,
                         cudaStream_t st) {
  Buckets bk;
  std::vector<int32_t> items;
  BSG_TRY(plan_items_host(h, keys, bk, items));
  BSG_TRY(programs_upload(h->programs, st));
  BSG_CUDA(cudaMemsetAsync(out, 0, (size_t)B * sizeof(double2), st));
  if (bk.slots == 0) return BSG_OK;
  const size_t chunks = bk.chunk_prog.size();
  BSG_TRY(h->items.ensure((size_t)bk.slots * 4 + chunks * 4 + 64));
  int32_t* d_items = reinterpret_cast<int32_t*>(h->items.ptr);
  int32_t* d_chunk = d_items + bk.slots;
  BSG_CUDA(cudaMemcpyAsync(d_items, items.data(), (size_t)bk.slots * 4, cudaMemcpyHostToDevice, st));
  BSG_CUDA(cudaMemcpyAsync(d_chunk, bk.chunk_prog.data(), chunks * 4, cudaMemcpyHostToDevice, st));
  BSG_TRY(h->misc.ensure(64));
  auto* counter = reinterpret_cast<unsigned long long*>(h->misc.ptr);
  BSG_CUDA(cudaMemsetAsync(counter, 0, 8, st));
  DPArgs a{};
  a.prog = prog_dev(h->programs);
  a.items = d_items;
  a.chunk_prog = d_chunk;
  a.n_chunks = (int64_t)chunks;
  a.counter = counter;
  a.sigma = sig;
  a.n_len = n_len;
  a.targets = targets;
  a.n = n;
  a.den = den;
  a.out = reinterpret_cast<double2*>(out);
  if (mode == MODE_TARGETS) BSG_TRY(launch_dp<MODE_TARGETS>(h, precision, a, bk, st));
  else BSG_TRY(launch_dp<MODE_MATRICES>(h, precision, a, bk, st));
  BSG_CUDA(cudaStreamSynchronize(st));  // host vectors above go out of scope
  return BSG_OK;
}

}  // namespace bsg

using namespace bsg;

extern "C" int bsg_hafnian_batched(bsg_handle_t h, const double* Sigma, int n_len, const int32_t* targets, int n,
                                   int64_t B, const double* denominator, int precision, double* out,
                                   bsg_stream_t stream) {
  BSG_CHECK_ARG(h, "bsg_hafnian_batched: null handle");
  BSG_CHECK_ARG(Sigma && out && (targets || n == 0 || B == 0), "bsg_hafnian_batched: null pointer");
  BSG_CHECK_ARG(n_len > 0 && n >= 0 && B >= 0, "bsg_hafnian_batched: bad sizes n_len=%d n=%d B=%lld", n_len, n,
                (long long)B);
  BSG_CHECK_ARG(n <= BSG_MAX_ORDER, "bsg_hafnian_batched: n=%d exceeds BSG_MAX_ORDER", n);
  BSG_CHECK_ARG(precision >= 0 && precision <= 2, "bsg_hafnian_batched: bad precision %d", precision);
  BSG_CUDA(cudaSetDevice(h->device));
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  BSG_TRY(ensure_tables());
  if (B == 0) return BSG_OK;
  BSG_TRY(h->keys.ensure((size_t)B * 8 + 64));
  uint64_t* d_keys = reinterpret_cast<uint64_t*>(h->keys.ptr);
  int* d_err = reinterpret_cast<int*>(d_keys + B);
  BSG_CUDA(cudaMemsetAsync(d_err, 0, 4, st));
  if (n == 0) {
    BSG_CUDA(cudaMemsetAsync(d_keys, 0, (size_t)B * 8, st));
  } else {
    target_keys_kernel<<<unsigned((B + 127) / 128), 128, 0, st>>>(targets, n, B, n_len, d_keys, d_err);
    BSG_CUDA(cudaGetLastError());
  }
  std::vector<uint64_t> keys(B);
  int err = 0;
  BSG_CUDA(cudaMemcpyAsync(keys.data(), d_keys, (size_t)B * 8, cudaMemcpyDeviceToHost, st));
  BSG_CUDA(cudaMemcpyAsync(&err, d_err, 4, cudaMemcpyDeviceToHost, st));
  BSG_CUDA(cudaStreamSynchronize(st));
  BSG_CHECK_ARG(err != 1, "bsg_hafnian_batched: target index outside [0, n_len)");
  if (err == 2) {
    set_error("bsg_hafnian_batched: an index repeats more than %d times", kKeyMaxMult);
    return BSG_ERR_LIMIT;
  }
  if (err == 3) {
    set_error("bsg_hafnian_batched: more than %d distinct indices in one target", BSG_MAX_CLASSES);
    return BSG_ERR_LIMIT;
  }
  const void* sig = nullptr;
  BSG_TRY(convert_sigma(h, Sigma, (int64_t)n_len * n_len, precision, h->sigma_ws, &sig, st));
  return run_target_dp(h, MODE_TARGETS, sig, n_len, targets, n, B, denominator, precision, out, keys, st);
}

extern "C" int bsg_hafnian_matrices(bsg_handle_t h, const double* A, int n, int64_t B, int precision, double* out,
                                    bsg_stream_t stream) {
  BSG_CHECK_ARG(h, "bsg_hafnian_matrices: null handle");
  BSG_CHECK_ARG(out && (A || n == 0 || B == 0), "bsg_hafnian_matrices: null pointer");
  BSG_CHECK_ARG(n >= 0 && B >= 0, "bsg_hafnian_matrices: bad sizes");
  BSG_CHECK_ARG(precision >= 0 && precision <= 2, "bsg_hafnian_matrices: bad precision %d", precision);
  if (n > BSG_MAX_CLASSES) {
    set_error("bsg_hafnian_matrices: n=%d exceeds BSG_MAX_CLASSES=%d distinct rows", n, BSG_MAX_CLASSES);
    return BSG_ERR_LIMIT;
  }
  BSG_CUDA(cudaSetDevice(h->device));
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  BSG_TRY(ensure_tables());
  if (B == 0) return BSG_OK;
  uint64_t key = (n & 1) ? ~0ull : (n == 0 ? 0ull : uint64_t(n));  // n classes of multiplicity 1
  std::vector<uint64_t> keys(B, key);
  const void* sig = nullptr;
  BSG_TRY(convert_sigma(h, A, (int64_t)B * n * n, precision, h->sigma_ws, &sig, st));
  return run_target_dp(h, MODE_MATRICES, sig, n, nullptr, n, B, nullptr, precision, out, keys, st);
}

extern "C" int bsg_build_site(bsg_handle_t h, int kind, const double* Sigma, int M_r, const int8_t* num_l, int k_l,
                              int m_l, const double* lambda_l, const int8_t* num_r, int k_r, int m_r, const double* Z,
                              int d, int chi, int precision, int out_dtype, void* Gamma, bsg_stream_t stream) {
  BSG_CHECK_ARG(h, "bsg_build_site: null handle");
  BSG_CHECK_ARG(kind >= BSG_SITE_FIRST && kind <= BSG_SITE_LAST, "bsg_build_site: bad kind %d", kind);
  BSG_CHECK_ARG(Sigma && Z && Gamma, "bsg_build_site: null pointer");
  BSG_CHECK_ARG(M_r >= 1 && d >= 1 && chi >= 1, "bsg_build_site: bad sizes M_r=%d d=%d chi=%d", M_r, d, chi);
  BSG_CHECK_ARG(chi <= 2048, "bsg_build_site: chi=%d exceeds 2048", chi);
  BSG_CHECK_ARG(d <= kKeyMaxMult + 1, "bsg_build_site: d=%d exceeds %d", d, kKeyMaxMult + 1);
  BSG_CHECK_ARG(precision >= 0 && precision <= 2, "bsg_build_site: bad precision %d", precision);
  BSG_CHECK_ARG(out_dtype == BSG_OUT_C64 || out_dtype == BSG_OUT_C128, "bsg_build_site: bad out_dtype");
  if (kind != BSG_SITE_LAST) {
    BSG_CHECK_ARG(num_l || k_l == 0 || m_l == 0, "bsg_build_site: num_l is NULL");
    BSG_CHECK_ARG(k_l >= 0 && k_l <= chi, "bsg_build_site: k_l=%d outside [0, chi]", k_l);
    BSG_CHECK_ARG(m_l == M_r - 1, "bsg_build_site: m_l=%d must equal M_r-1=%d", m_l, M_r - 1);
    BSG_CHECK_ARG(lambda_l || k_l == 0, "bsg_build_site: lambda_l is NULL");
  }
  if (kind != BSG_SITE_FIRST) {
    BSG_CHECK_ARG(num_r || k_r == 0, "bsg_build_site: num_r is NULL");
    BSG_CHECK_ARG(k_r >= 0 && k_r <= chi, "bsg_build_site: k_r=%d outside [0, chi]", k_r);
    BSG_CHECK_ARG(m_r == M_r, "bsg_build_site: m_r=%d must equal M_r=%d", m_r, M_r);
  }
  BSG_CUDA(cudaSetDevice(h->device));
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  BSG_TRY(ensure_tables());
  const size_t esz = out_dtype == BSG_OUT_C128 ? 16 : 8;
  BSG_CUDA(cudaMemsetAsync(Gamma, 0, (size_t)chi * chi * d * esz, st));

  // effective label tables: FIRST has one empty right row, LAST one empty left row
  const int KL = kind == BSG_SITE_LAST ? 1 : k_l;
  const int KR = kind == BSG_SITE_FIRST ? 1 : k_r;
  const int ML = kind == BSG_SITE_LAST ? 0 : m_l;
  const int MR = kind == BSG_SITE_FIRST ? 0 : m_r;
  if (KL == 0 || KR == 0) return BSG_OK;

  // row tables in the keys buffer
  auto align = [](size_t x) { return (x + 255) & ~size_t(255); };
  size_t off = 0;
  auto carve = [&](size_t bytes) {
    size_t o = off;
    off = align(off + bytes);
    return o;
  };
  const size_t o_lent = carve((size_t)KL * kMaxNnz * 4), o_lnnz = carve(KL * 4), o_lsum = carve(KL * 4),
               o_lkey = carve(KL * 8), o_lrf = carve(KL * 8);
  const size_t o_rent = carve((size_t)KR * kMaxNnz * 4), o_rnnz = carve(KR * 4), o_rsum = carve(KR * 4),
               o_rkey = carve(KR * 8), o_rrf = carve(KR * 8);
  const size_t o_err = carve(16), o_zero = carve(16);
  BSG_TRY(h->keys.ensure(off));
  char* kb = reinterpret_cast<char*>(h->keys.ptr);
  RowTable lt{reinterpret_cast<int32_t*>(kb + o_lent), reinterpret_cast<int32_t*>(kb + o_lnnz),
              reinterpret_cast<int32_t*>(kb + o_lsum), reinterpret_cast<uint64_t*>(kb + o_lkey),
              reinterpret_cast<double*>(kb + o_lrf)};
  RowTable rt{reinterpret_cast<int32_t*>(kb + o_rent), reinterpret_cast<int32_t*>(kb + o_rnnz),
              reinterpret_cast<int32_t*>(kb + o_rsum), reinterpret_cast<uint64_t*>(kb + o_rkey),
              reinterpret_cast<double*>(kb + o_rrf)};
  int* d_err = reinterpret_cast<int*>(kb + o_err);
  int8_t* d_zero = reinterpret_cast<int8_t*>(kb + o_zero);
  BSG_CUDA(cudaMemsetAsync(kb + o_err, 0, 32, st));
  label_rows_kernel<<<(KL + 127) / 128, 128, 0, st>>>(ML ? num_l : d_zero, KL, ML, 1, lt, d_err);
  label_rows_kernel<<<(KR + 127) / 128, 128, 0, st>>>(MR ? num_r : d_zero, KR, MR, M_r, rt, d_err);
  BSG_CUDA(cudaGetLastError());

  // read keys and sums back to plan
  BSG_TRY(h->host_stage.ensure((size_t)(KL + KR) * 12 + 16));
  uint64_t* hk = reinterpret_cast<uint64_t*>(h->host_stage.ptr);
  int32_t* hs = reinterpret_cast<int32_t*>(hk + KL + KR);
  int* herr = hs + KL + KR;
  BSG_CUDA(cudaMemcpyAsync(hk, lt.key, KL * 8, cudaMemcpyDeviceToHost, st));
  BSG_CUDA(cudaMemcpyAsync(hk + KL, rt.key, KR * 8, cudaMemcpyDeviceToHost, st));
  BSG_CUDA(cudaMemcpyAsync(hs, lt.sum, KL * 4, cudaMemcpyDeviceToHost, st));
  BSG_CUDA(cudaMemcpyAsync(hs + KL, rt.sum, KR * 4, cudaMemcpyDeviceToHost, st));
  BSG_CUDA(cudaMemcpyAsync(herr, d_err, 4, cudaMemcpyDeviceToHost, st));
  BSG_CUDA(cudaStreamSynchronize(st));
  if (*herr) {
    set_error("bsg_build_site: a label entry is negative, above %d, or a row has more than %d non-zeros",
              kKeyMaxMult, kMaxNnz);
    return BSG_ERR_LIMIT;
  }

  // group rows by key
  auto group = [](const uint64_t* key, int rows, std::vector<int32_t>& perm, std::vector<int32_t>& grp,
                  std::vector<uint64_t>& gkey, std::vector<int64_t>& gcnt) {
    perm.resize(rows);
    std::iota(perm.begin(), perm.end(), 0);
    std::stable_sort(perm.begin(), perm.end(), [&](int x, int y) { return key[x] < key[y]; });
    grp.resize(rows);
    for (int i = 0; i < rows; ++i) {
      if (i == 0 || key[perm[i]] != key[perm[i - 1]]) {
        gkey.push_back(key[perm[i]]);
        gcnt.push_back(0);
      }
      grp[i] = int32_t(gkey.size() - 1);
      gcnt.back()++;
    }
  };
  std::vector<int32_t> perm_l, grp_l, perm_r, grp_r;
  std::vector<uint64_t> gk_l, gk_r;
  std::vector<int64_t> gc_l, gc_r;
  group(hk, KL, perm_l, grp_l, gk_l, gc_l);
  group(hk + KL, KR, perm_r, grp_r, gk_r, gc_r);
  const int ngl = int(gk_l.size()), ngr = int(gk_r.size());
  std::vector<int> gsum_l(ngl), gsum_r(ngr);
  for (int g = 0; g < ngl; ++g) gsum_l[g] = key_order(gk_l[g]);
  for (int g = 0; g < ngr; ++g) gsum_r[g] = key_order(gk_r[g]);

  Buckets bk;
  std::unordered_map<int32_t, int> bucket_of_prog;
  std::vector<int32_t> bucket_of((size_t)d * ngl * ngr, -1);
  auto& ps = h->programs;
  for (int j = 0; j < d; ++j) {
    const uint64_t kj = key_add_class(0, j);
    for (int gl = 0; gl < ngl; ++gl) {
      for (int gr = 0; gr < ngr; ++gr) {
        int n = j + gsum_l[gl] + gsum_r[gr];
        if (n & 1) continue;
        if (n > BSG_MAX_ORDER) {
          set_error("bsg_build_site: hafnian order %d exceeds BSG_MAX_ORDER", n);
          return BSG_ERR_LIMIT;
        }
        int32_t prog;
        BSG_TRY(program_for_key(ps, kj + gk_l[gl] + gk_r[gr], &prog));
        auto it = bucket_of_prog.find(prog);
        int b;
        if (it == bucket_of_prog.end()) {
          b = int(bk.progs.size());
          bucket_of_prog.emplace(prog, b);
          bk.progs.push_back(prog);
          bk.counts.push_back(0);
        } else {
          b = it->second;
        }
        bk.counts[b] += gc_l[gl] * gc_r[gr];
        bucket_of[((size_t)j * ngl + gl) * ngr + gr] = b;
      }
    }
  }
  std::vector<int32_t> progs_before = bk.progs;
  BSG_TRY(layout_buckets(ps, bk));
  {
    std::unordered_map<int32_t, int> newb;
    for (size_t b = 0; b < bk.progs.size(); ++b) newb[bk.progs[b]] = int(b);
    for (auto& b : bucket_of)
      if (b >= 0) b = newb[progs_before[b]];
  }
  BSG_TRY(programs_upload(ps, st));
  const int nb = int(bk.progs.size());
  const size_t chunks = bk.chunk_prog.size();

  // upload the plan
  size_t poff = 0;
  auto pcarve = [&](size_t bytes) {
    size_t o = poff;
    poff = align(poff + bytes);
    return o;
  };
  const size_t p_perm_l = pcarve(KL * 4), p_grp_l = pcarve(KL * 4), p_perm_r = pcarve(KR * 4),
               p_grp_r = pcarve(KR * 4), p_bof = pcarve(bucket_of.size() * 4), p_boff = pcarve(nb * 4 + 4),
               p_cur = pcarve(nb * 4 + 4), p_chunk = pcarve(chunks * 4 + 4), p_ctr = pcarve(8);
  const size_t plan_bytes = poff;
  BSG_TRY(h->plan.ensure(plan_bytes));
  BSG_TRY(h->host_stage2.ensure(plan_bytes));
  char* hp = reinterpret_cast<char*>(h->host_stage2.ptr);
  std::memcpy(hp + p_perm_l, perm_l.data(), KL * 4);
  std::memcpy(hp + p_grp_l, grp_l.data(), KL * 4);
  std::memcpy(hp + p_perm_r, perm_r.data(), KR * 4);
  std::memcpy(hp + p_grp_r, grp_r.data(), KR * 4);
  std::memcpy(hp + p_bof, bucket_of.data(), bucket_of.size() * 4);
  std::memcpy(hp + p_boff, bk.offsets.data(), nb * 4);
  std::memset(hp + p_cur, 0, nb * 4 + 4);
  if (chunks) std::memcpy(hp + p_chunk, bk.chunk_prog.data(), chunks * 4);
  std::memset(hp + p_ctr, 0, 8);
  char* dp = reinterpret_cast<char*>(h->plan.ptr);
  BSG_CUDA(cudaMemcpyAsync(dp, hp, plan_bytes, cudaMemcpyHostToDevice, st));
  if (bk.slots == 0) return BSG_OK;
  BSG_TRY(h->items.ensure((size_t)bk.slots * 4));
  int32_t* d_items = reinterpret_cast<int32_t*>(h->items.ptr);
  BSG_CUDA(cudaMemsetAsync(d_items, 0xff, (size_t)bk.slots * 4, st));

  SitePlanDev sp{reinterpret_cast<int32_t*>(dp + p_perm_l), reinterpret_cast<int32_t*>(dp + p_grp_l),
                 reinterpret_cast<int32_t*>(dp + p_perm_r), reinterpret_cast<int32_t*>(dp + p_grp_r),
                 reinterpret_cast<int32_t*>(dp + p_bof),    reinterpret_cast<int32_t*>(dp + p_boff),
                 reinterpret_cast<int32_t*>(dp + p_cur),    d_items,
                 ngl, ngr, KL, KR, d};
  int64_t total = (int64_t)d * KL * KR;
  int sblocks = int(std::min<int64_t>((total + 255) / 256, (int64_t)h->num_sms * 8));
  site_scatter_kernel<<<std::max(sblocks, 1), 256, 0, st>>>(sp);
  BSG_CUDA(cudaGetLastError());

  const void* sig = nullptr;
  BSG_TRY(convert_sigma(h, Sigma, (int64_t)(2 * M_r) * (2 * M_r), precision, h->sigma_ws, &sig, st));
  DPArgs a{};
  a.prog = prog_dev(ps);
  a.items = d_items;
  a.chunk_prog = reinterpret_cast<int32_t*>(dp + p_chunk);
  a.n_chunks = (int64_t)chunks;
  a.counter = reinterpret_cast<unsigned long long*>(dp + p_ctr);
  a.sigma = sig;
  a.n_len = 2 * M_r;
  a.l_ent = lt.entries;
  a.l_nnz = lt.nnz;
  a.l_rowfact = lt.rowfact;
  a.lambda = kind == BSG_SITE_LAST ? nullptr : lambda_l;
  a.r_ent = rt.entries;
  a.r_nnz = rt.nnz;
  a.r_rowfact = rt.rowfact;
  a.Z = Z;
  a.d = d;
  a.chi = chi;
  a.out_c128 = out_dtype == BSG_OUT_C128;
  a.gamma = Gamma;
  return launch_dp<MODE_SITE>(h, precision, a, bk, st);
}
