// Batched repetition-aware hafnians, the fused per-site Gamma build and the
// whole-MPS build.
//
// Every work item is one hafnian of Sigma restricted to a target index list
// with repeats.  Items are bucketed by the multiplicity partition of their
// target; a warp takes 32 items of one bucket and runs that bucket's
// partition program (bsg_programs.cpp) in lock-step, one item per lane.  The
// class-pair values are read from the site's Sigma at each transition; the
// DP states (F) live in a per-warp ring slice laid out [entry][lane] so every
// access is one coalesced line.  The buckets of a set of sites share
// yielding launches with an atomic work counter; each 32-slot chunk finds its
// bucket (site and program) in a per-bucket prefix sum.
#include <algorithm>
#include <chrono>
#include <atomic>
#include <cmath>
#include <condition_variable>
#include <mutex>
#include <thread>
#include <unordered_set>
#include <cstring>
#include <functional>
#include <numeric>
#include <type_traits>
#include <vector>

#include <unistd.h>

#include "bsg_arith.cuh"
#include "bsg_internal.h"

namespace bsg {

constexpr int kMaxInv = 64;
__constant__ double c_inv_d[kMaxInv];
__constant__ float2 c_inv_f[kMaxInv];
__constant__ double c_sqrt_fact[kMaxInv];  // sqrt(n!)
__constant__ double c_fact[kMaxInv];       // n! (as double)
__constant__ float2 c_sqrt_fact2[kMaxInv]; // sqrt(n!) as an FP32 pair

static int ensure_tables() {
  static int dev_done = -1;
  int dev = 0;
  BSG_CUDA(cudaGetDevice(&dev));
  if (dev_done == dev) return BSG_OK;
  double inv_d[kMaxInv], sf[kMaxInv], f[kMaxInv];
  float2 inv_f[kMaxInv], sf2[kMaxInv];
  for (int r = 0; r < kMaxInv; ++r) {
    inv_d[r] = r ? 1.0 / r : 0.0;
    float hi = float(inv_d[r]);
    inv_f[r] = make_float2(hi, float(inv_d[r] - double(hi)));
    f[r] = std::tgamma(double(r) + 1.0);
    sf[r] = std::sqrt(f[r]);
    const float h2 = float(sf[r]);
    sf2[r] = make_float2(h2, float(sf[r] - double(h2)));
  }
  BSG_CUDA(cudaMemcpyToSymbol(c_sqrt_fact2, sf2, sizeof(sf2)));
  BSG_CUDA(cudaMemcpyToSymbol(c_inv_d, inv_d, sizeof(inv_d)));
  BSG_CUDA(cudaMemcpyToSymbol(c_inv_f, inv_f, sizeof(inv_f)));
  BSG_CUDA(cudaMemcpyToSymbol(c_sqrt_fact, sf, sizeof(sf)));
  BSG_CUDA(cudaMemcpyToSymbol(c_fact, f, sizeof(f)));
  dev_done = dev;
  return BSG_OK;
}

// ---------------------------------------------------------------------------
// Label rows: sparse (mode, multiplicity) lists sorted by multiplicity,
// partition key, row sum and sqrt(prod num!) -- one thread per row.  Rows of
// several cuts are handled in one launch (blockIdx.y = cut).
// ---------------------------------------------------------------------------
constexpr int kMaxNnz = BSG_MAX_LABEL_NNZ;

struct RowTable {  // arrays indexed [cut * rows_cap + row]
  int32_t* entries;  // [.., kMaxNnz] packed (mode << 8) | mult
  int32_t* nnz;
  int32_t* sum;
  uint64_t* key;
  double* rowfact;   // sqrt(prod num!)
  float2* rowfact2;  // the same as an unevaluated FP32 pair (hi, lo)
};

// One label row: its sorted (mode, multiplicity) entries, count, sum, key
// and sqrt(prod num!) into entry o of the table.
__device__ __forceinline__ void label_row(const int8_t* __restrict__ row, int m, const RowTable& t, size_t o,
                                          int* __restrict__ err) {
  int ent[kMaxNnz];
  int cnt = 0, sum = 0;
  uint64_t key = 0;
  double rf = 1.0;
  for (int q = 0; q < m; ++q) {
    int v = row[q];
    if (v == 0) continue;
    if (v < 0 || v > kKeyMaxMult || cnt >= kMaxNnz) {
      atomicExch(err, 1);
      continue;
    }
    int e = (q << 8) | v;
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
  for (int i = 0; i < cnt; ++i) t.entries[o * kMaxNnz + i] = ent[i];
  t.nnz[o] = cnt;
  t.sum[o] = sum;
  t.key[o] = key;
  t.rowfact[o] = rf;
  const float hi = float(rf);
  t.rowfact2[o] = make_float2(hi, float(rf - double(hi)));
}

__global__ void label_rows_kernel(const int8_t* __restrict__ num, int64_t cut_stride, int ld,
                                  const int32_t* __restrict__ rows, int m_base, int m_step, int rows_cap, RowTable t,
                                  int* __restrict__ err) {
  const int cut = blockIdx.y;
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows[cut]) return;
  label_row(num + cut * cut_stride + (int64_t)r * ld, m_base - m_step * cut, t, (size_t)cut * rows_cap + r, err);
}

// The per-cut row work of many instances in one launch: Lambda = sqrt(res)
// where res > tol (else 0) with the count of such rows, the label row tables
// and a copy of the kept-row count next to the keys, so that the host reads
// every instance's keys and counts with one copy.  blockIdx.y = (job, cut)
// through `map`, 128 rows per block along x.
struct CutRowsJob {
  const int8_t* num;    // [cuts, chi, ld] from the job's first cut
  const int32_t* kept;  // [cuts]
  const double* res;    // [cuts, chi]
  double* lambda;       // [cuts, chi]
  RowTable t;           // row tables from the first cut (rows_cap = chi)
  int32_t* above;       // [cuts] rows with res > tol (cleared before)
  int32_t* cnt;         // [cuts] copy of kept
  int* err;
  double tol;
  int chi, ld, m0;      // rows per cut, label row stride, modes right of the first cut
};

__global__ void cut_rows_batch_kernel(const CutRowsJob* __restrict__ jobs, const int2* __restrict__ map) {
  const int2 jc = map[blockIdx.y];
  const CutRowsJob& jb = jobs[jc.x];
  const int c = jc.y, chi = jb.chi;
  if ((int)(blockIdx.x * blockDim.x) >= chi) return;  // block-uniform
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  bool keep = false;
  if (r < chi) {
    const double v = jb.res[(size_t)c * chi + r];
    keep = v > jb.tol;
    jb.lambda[(size_t)c * chi + r] = keep ? sqrt(v) : 0.0;
  }
  const unsigned bal = __ballot_sync(0xffffffffu, keep);
  if ((threadIdx.x & 31) == 0 && bal) atomicAdd(jb.above + c, __popc(bal));
  const int rows = min(jb.kept[c], chi);  // a caller's kept count never indexes past the row tables
  if (blockIdx.x == 0 && threadIdx.x == 0) jb.cnt[c] = rows;
  if (r < rows)
    label_row(jb.num + ((size_t)c * chi + r) * jb.ld, jb.m0 - c, jb.t, (size_t)c * chi + r, jb.err);
}

// Left-row scale of a site: sqrt(prod num!) / (Z * Lambda) in FP64 and as an
// FP32 pair, so the DP epilogue needs no FP64 division (blockIdx.y = site).
struct LeftScaleJob {
  const double* rowfact;
  const double* lambda;  // null -> 1
  const double* Z;
  int rows;
  double* out_d;
  float2* out_f;
};

__global__ void left_scale_kernel(const LeftScaleJob* __restrict__ jobs) {
  const LeftScaleJob jb = jobs[blockIdx.y];
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= jb.rows) return;
  double v = jb.rowfact[r] / jb.Z[0];
  if (jb.lambda) v /= jb.lambda[r];
  jb.out_d[r] = v;
  const float hi = float(v);
  jb.out_f[r] = make_float2(hi, float(v - double(hi)));
}

// Lambda = sqrt(res) where res > err_tol (else 0) and the count of such rows.
__global__ void lambda_kernel(const double* __restrict__ res, int chi, double err_tol, double* __restrict__ lambda,
                              int32_t* __restrict__ rows_above) {
  const int c = blockIdx.x;
  int cnt = 0;
  for (int r = threadIdx.x; r < chi; r += blockDim.x) {
    double v = res[(size_t)c * chi + r];
    bool keep = v > err_tol;
    lambda[(size_t)c * chi + r] = keep ? sqrt(v) : 0.0;
    cnt += keep;
  }
  for (int o = 16; o > 0; o >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, o);
  __shared__ int s[32];
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = cnt;
  __syncthreads();
  if (threadIdx.x == 0) {
    int tot = 0;
    for (int w = 0; w < (int)(blockDim.x + 31) / 32; ++w) tot += s[w];
    rows_above[c] = tot;
  }
}

// ---------------------------------------------------------------------------
// Site classification: scatter every even-order (a, b, j) item into the
// bucket of its partition program.  Rows are visited in key-sorted order, so
// the items of one (j, left key group, right key group) combination are the
// |gl| x |gr| row pairs of two contiguous ranges: the host gives each
// combination its offset inside its bucket and an item's slot follows from
// the ranks of its rows inside their groups (no atomics; consecutive left
// rows land in consecutive slots).
// ---------------------------------------------------------------------------
struct SitePlanDev {
  const int32_t* perm_l;     // sorted position -> left row
  const int32_t* grp_l;      // sorted position -> left key group
  const int32_t* perm_r;
  const int32_t* grp_r;
  const int32_t* bucket_of;  // [ngl][ngr] -> global bucket or -1 (no even order)
  const int32_t* combo_off;  // [ngl][ngr] -> first slot of the combination inside its bucket
  const int8_t* combo_j;     // [ngl][ngr] -> the site multiplicity jmax its items carry
  const int32_t* gstart_l;   // [ngl] sorted position of the group's first row
  const int32_t* gcnt_l;     // [ngl] rows of the group
  const int32_t* gstart_r;   // [ngr]
  const int32_t* bucket_off; // [nb] first slot
  int32_t* items;            // slots
  int ngl, ngr, kl, kr, d;
};

// One launch per set of sites (blockIdx.y = site).  A thread takes one (right
// row, left row) pair in key-sorted order and writes its item: one multi-root
// program per pair evaluates every Gamma entry j of the pair's parity.
__global__ void site_scatter_kernel(const SitePlanDev* __restrict__ plans) {
  const SitePlanDev p = plans[blockIdx.y];
  const int64_t total = (int64_t)p.kr * p.kl;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += stride) {
    const int bs = int(i % p.kl), as = int(i / p.kl);
    const int gl = p.grp_l[bs], gr = p.grp_r[as];
    const int32_t within = (as - p.gstart_r[gr]) * p.gcnt_l[gl] + (bs - p.gstart_l[gl]);
    const int32_t ab = (p.perm_r[as] << 20) | (p.perm_l[bs] << 8);
    const size_t o = (size_t)gl * p.ngr + gr;
    const int bucket = p.bucket_of[o];
    if (bucket >= 0) p.items[p.bucket_off[bucket] + p.combo_off[o] + within] = ab | int(p.combo_j[o]);
  }
}

// The padding slots of each bucket (from its last item to its chunk end,
// fewer than 32) hold -1, which the DP reads as "no item"; a warp per bucket.
__global__ void pad_items_kernel(const int32_t* __restrict__ bucket_end, const int32_t* __restrict__ bucket_chunk,
                                 int nb, int32_t* __restrict__ items) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int b = int(t >> 5);
  if (b >= nb) return;
  const int64_t slot = (int64_t)bucket_end[b] + (t & 31);
  if (slot < (int64_t)bucket_chunk[b + 1] * 32) items[slot] = -1;
}

// The bucket of each chunk (the last b with bucket_chunk[b] <= c), so that a
// DP warp finds its chunk's bucket with one load.
__global__ void chunk_bucket_kernel(const int32_t* __restrict__ bucket_chunk, int nb, int64_t n_chunks,
                                    int32_t* __restrict__ out) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n_chunks) return;
  int lo = 0, hi = nb - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if ((int64_t)bucket_chunk[mid] <= c) lo = mid;
    else hi = mid - 1;
  }
  out[c] = lo;
}

// ---------------------------------------------------------------------------
// The DP kernel
// ---------------------------------------------------------------------------
struct ProgDev {
  const int32_t* k;
  const int32_t* nstates;
  const int32_t* state_off;
  const uint32_t* trans;
  const uint4* st_pack;  // {first transition, count | r_a << 16, F slot, class a} per state
};

enum { MODE_SITE = 0, MODE_TARGETS = 1, MODE_MATRICES = 2 };

struct SiteDesc {
  const void* sigma;    // policy-typed [2Mr, 2Mr]
  const double2* sigma64;  // the same Sigma in FP64 (the FP64 helper launch)
  int n_len, Mr;
  const int32_t* l_ent;  // left rows (cut `site`): entries/nnz/rowfact
  const int32_t* l_nnz;
  const double* l_rowfact;
  const double* lambda;  // null -> 1
  const int32_t* r_ent;  // right rows (cut `site-1`)
  const int32_t* r_nnz;
  const double* r_rowfact;
  const float2* r_rowfact2;
  const double* l_scale;   // rowfact / (Z Lambda) per left row
  const float2* l_scale2;  // the same as an FP32 pair
  const double* Z;
  void* gamma;
  int chi, d, out_c128;
};

struct DPArgs {
  ProgDev prog;
  const int32_t* items;
  // chunks (32 item slots) of bucket b are [bucket_chunk[b], bucket_chunk[b+1])
  const int32_t* bucket_chunk;  // [nb + 1]
  const int32_t* chunk_bucket;  // [chunks] the bucket of each chunk, or null (binary search in bucket_chunk)
  const int32_t* bucket_prog;   // [nb]
  const int32_t* bucket_site;   // [nb] (site mode)
  int nb;
  int64_t chunk_base;  // first chunk of this launch
  int64_t n_chunks;    // chunks of this launch
  unsigned long long* counter;
  void* scratch;
  int states_max;  // F ring entries of a warp's slice
  // yielding launches (quantum > 0): a warp leaves after `quantum` program
  // transitions, its block after all its warps; blocks take a per-warp table
  // slot from `slot_flags` [n_slots] and give it back before exiting.
  int64_t quantum;
  int* slot_flags;
  int n_slots;
  // site mode
  const SiteDesc* sites;
  // target / matrices mode
  const void* sigma;  // policy-typed
  int n_len;
  const int32_t* targets;
  int n;
  const double* den;
  double2* out;
};

template <int MODE>
__device__ __forceinline__ int build_classes(const DPArgs& a, const SiteDesc* sd, int32_t item, int* cls,
                                             double& fac, int64_t& sig_base) {
  sig_base = 0;
  fac = 1.0;
  if (MODE == MODE_SITE) {
    const int alpha = (item >> 20) & 0xfff, beta = (item >> 8) & 0xfff;
    const int32_t* le = sd->l_ent + (size_t)beta * kMaxNnz;
    const int32_t* re = sd->r_ent + (size_t)alpha * kMaxNnz;
    const int nl = sd->l_nnz[beta], nr = sd->r_nnz[alpha];
    const int roff = sd->Mr;
    int il = 0, ir = 0, k = 0;
    // left and right label classes merged by multiplicity (left first on
    // ties), then the site class, which the site programs keep last
    while (il < nl || ir < nr) {
      const int ml = il < nl ? (le[il] & 0xff) : 1 << 20;
      const int mr = ir < nr ? (re[ir] & 0xff) : 1 << 20;
      if (ml <= mr) cls[k++] = 1 + (le[il++] >> 8);
      else cls[k++] = roff + (re[ir++] >> 8);
    }
    cls[k++] = 0;
    return k;
  } else {
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
    int ci[BSG_MAX_CLASSES], cm[BSG_MAX_CLASSES];
    int k = 0;
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

// Table slot of a yielding DP block: a free flag of `flags`, probed from the
// block's SM onwards.  At most n resident blocks of one launch exist at a time
// (n = resident blocks per SM x SMs), so a free flag exists; the probe is
// bounded all the same and returns -1 when it gives up.
__device__ int acquire_dp_slot(int* flags, int n) {
  unsigned smid, nsmid;
  asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
  asm volatile("mov.u32 %0, %%nsmid;" : "=r"(nsmid));
  const unsigned per_sm = max(1u, (unsigned)n / max(1u, nsmid));
  int i = int((smid * per_sm) % (unsigned)n);
  for (int probe = 0; probe < 16 * n; ++probe) {
    if (*reinterpret_cast<volatile int*>(flags + i) == 0 && atomicCAS(flags + i, 0, 1) == 0) return i;
    if (++i == n) i = 0;
  }
  return -1;
}

// DP block size; the launch bound keeps 40 warps resident per SM (128- and
// 64-thread blocks measured slower)
constexpr int kDPThreads = 256;
constexpr int kDPWarps = kDPThreads / 32;

template <class P, int MODE>
__global__ void __launch_bounds__(kDPThreads, 1280 / kDPThreads) dp_kernel(DPArgs a) {
  using C = typename P::C;
  using CA = typename P::CA;
  using CF = typename P::CF;
  const int lane = threadIdx.x & 31;
  __shared__ int s_slot;
  int bslot = blockIdx.x;
  if (a.quantum > 0) {
    if (threadIdx.x == 0) s_slot = acquire_dp_slot(a.slot_flags, a.n_slots);
    __syncthreads();
    bslot = s_slot;
    if (bslot < 0) return;  // no slot: this block takes no work (a later launch drains the queue)
  }
  const int warp = bslot * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const size_t slice = (size_t)a.states_max * 32 * sizeof(CF);
  CF* Fb = reinterpret_cast<CF*>(reinterpret_cast<char*>(a.scratch) + (size_t)warp * slice);
  int64_t done = 0;  // program transitions this warp has run
  while (true) {
    if (a.quantum > 0 && done >= a.quantum) break;
    unsigned long long c = 0;
    if (lane == 0) c = atomicAdd(a.counter, 1ull);
    c = __shfl_sync(0xffffffffu, c, 0);
    if ((int64_t)c >= a.n_chunks) break;
    c += (unsigned long long)a.chunk_base;
    // bucket of chunk c: the last b with bucket_chunk[b] <= c (one load from
    // the per-chunk table where the plan has one, else a binary search)
    int lo = 0;
    if (a.chunk_bucket) {
      lo = __ldg(a.chunk_bucket + c);
    } else {
      int hi = a.nb - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if ((unsigned long long)a.bucket_chunk[mid] <= c) lo = mid;
        else hi = mid - 1;
      }
    }
    const int prog = a.bucket_prog[lo];
    const SiteDesc* sd = MODE == MODE_SITE ? a.sites + a.bucket_site[lo] : nullptr;
    const int32_t item = a.items[c * 32 + lane];
    const bool live = item >= 0;
    const int kp = a.prog.k[prog];
    const int ns = a.prog.nstates[prog];
    const int so = a.prog.state_off[prog];
    const C* sig = reinterpret_cast<const C*>(
        MODE == MODE_SITE ? (std::is_same<P, PrecF64>::value ? (const void*)sd->sigma64 : sd->sigma) : a.sigma);
    const int n_len = MODE == MODE_SITE ? sd->n_len : a.n_len;

    int cls[BSG_MAX_CLASSES];
    double fac = 1.0;
    int64_t sb = 0;
    if (live) {
      build_classes<MODE>(a, sd, item, cls, fac, sb);
    } else {
      for (int q = 0; q < kp; ++q) cls[q] = 0;
    }
    // class-pair values are read straight from Sigma at each transition
    // (Sigma is shared by every item of the site and stays in L1 / L2; a
    // per-item copy would double the warp's table footprint).  Sigma is
    // symmetric: in site mode each pair is read with the larger key as the
    // row, key = Sigma index - 1 as an unsigned word (the site mode, index 0,
    // ranks last).  The site mode and the right label's modes are usually
    // shared by the warp's lanes (one right row, consecutive left rows of one
    // key group), so the lanes read along one row of Sigma instead of down a
    // column.
    const int kb = MODE == MODE_SITE ? 1 : 0;
    for (int q = 0; q < kp; ++q) cls[q] -= kb;
    const C* sigp = sig + sb + (int64_t)kb * (n_len + 1);
    // transition word: (source F slot << 9) | (b << 2); every transition of a
    // state pairs its b with the state's first class a
    constexpr unsigned kFShift = sizeof(CF) == 16 ? 0u : sizeof(CF) == 8 ? 1u : 0u;
    static_assert(sizeof(CF) == 16 || sizeof(CF) == 8, "F entries of 8 or 16 bytes");
    const char* cls_b = reinterpret_cast<const char*>(cls);
    const char* Fl = reinterpret_cast<const char*>(Fb + lane);
    auto F_at = [&](uint32_t w) -> CF { return *reinterpret_cast<const CF*>(Fl + ((w & ~511u) >> kFShift)); };
    // site mode: Gamma entry (alpha, beta, j) of a root state (site multiplicity j)
    auto emit_site = [&](int j, const CF& v) {
      const int alpha = (item >> 20) & 0xfff, beta = (item >> 8) & 0xfff;
      const size_t o = ((size_t)alpha * sd->chi + beta) * sd->d + j;
      if constexpr (std::is_same<P, PrecSplit>::value) {
        if (!sd->out_c128) {
          // epilogue on the FP32 pipe: (hi + lo) * sqrt(j!) * l_scale * r_rowfact as FP32 pairs
          const float4 q = v;  // (re_h, im_h, re_l, im_l)
          const float2 js = c_sqrt_fact2[j], ls = sd->l_scale2[beta], rs = sd->r_rowfact2[alpha];
          float sh, sl, th, tl, re_h, re_l, im_h, im_l;
          PrecSplit::mul(js.x, js.y, ls.x, ls.y, sh, sl);
          PrecSplit::mul(sh, sl, rs.x, rs.y, th, tl);
          PrecSplit::mul(q.x, q.z, th, tl, re_h, re_l);
          PrecSplit::mul(q.y, q.w, th, tl, im_h, im_l);
          __stcs(reinterpret_cast<float2*>(sd->gamma) + o, make_float2(re_h + re_l, im_h + im_l));
          return;
        }
      }
      const double2 w = P::to_c128(v);
      const double scale = c_sqrt_fact[j] * sd->l_scale[beta] * sd->r_rowfact[alpha];
      if (sd->out_c128) {
        __stcs(reinterpret_cast<double2*>(sd->gamma) + o, make_double2(w.x * scale, w.y * scale));
      } else {
        __stcs(reinterpret_cast<float2*>(sd->gamma) + o, make_float2(float(w.x * scale), float(w.y * scale)));
      }
    };
    // run the program (the final coefficient stays in a register)
    Fb[lane] = P::one();
    CF fin = P::one();
    if (MODE == MODE_SITE) {
      // the empty state is a root only for j = 0 with empty labels
      const uint32_t tag0 = __ldg(&a.prog.st_pack[so].y) >> 16;
      if (tag0 && live) emit_site(int(tag0) - 1, fin);
    }
    for (int s = 1; s < ns; ++s) {
      const uint4 pk = __ldg(a.prog.st_pack + so + s);
      const int off = int(pk.x), cnt = int(pk.y & 0xffu), ra = int((pk.y >> 8) & 0xffu);
      const uint32_t ya = uint32_t(cls[pk.w]);
      done += cnt;
      auto A_at = [&](uint32_t w) -> CA {
        const uint32_t x = uint32_t(*reinterpret_cast<const int*>(cls_b + (w & 0x7cu)));
        if (MODE == MODE_SITE) return sigp[int(max(x, ya) * uint32_t(n_len) + min(x, ya))];
        return sigp[int(x * uint32_t(n_len) + ya)];
      };
      typename P::Acc acc = P::zero();
      // two transitions per step: both pairs of table loads are in flight
      // before the first multiply-add (states average ~2.4 transitions); the
      // first product starts the sum (mac_init) instead of adding to zero
      int t = 0;
      if (cnt >= 2) {
        const uint32_t w0 = __ldg(a.prog.trans + off);
        const uint32_t w1 = __ldg(a.prog.trans + off + 1);
        const CA av0 = A_at(w0);
        const CF fv0 = F_at(w0);
        const CA av1 = A_at(w1);
        const CF fv1 = F_at(w1);
        P::mac_init(acc, av0, fv0);
        P::mac(acc, av1, fv1);
        t = 2;
      } else if (cnt == 1) {
        const uint32_t w = __ldg(a.prog.trans + off);
        P::mac_init(acc, A_at(w), F_at(w));
        t = 1;
      }
      for (; t + 1 < cnt; t += 2) {
        const uint32_t w0 = __ldg(a.prog.trans + off + t);
        const uint32_t w1 = __ldg(a.prog.trans + off + t + 1);
        const CA av0 = A_at(w0);
        const CF fv0 = F_at(w0);
        const CA av1 = A_at(w1);
        const CF fv1 = F_at(w1);
        P::mac(acc, av0, fv0);
        P::mac(acc, av1, fv1);
      }
      if (t < cnt) {
        const uint32_t w = __ldg(a.prog.trans + off + t);
        const CA av = A_at(w);
        const CF fv = F_at(w);
        P::mac(acc, av, fv);
      }
      fin = P::finish(acc, ra, c_inv_d, c_inv_f);
      Fb[(size_t)pk.z * 32 + lane] = fin;
      if (MODE == MODE_SITE && (pk.y >> 16) && live) emit_site(int(pk.y >> 16) - 1, fin);
    }
    if (!live) continue;
    if (MODE != MODE_SITE) {
      const double2 v = P::to_c128(fin);
      double s = fac;
      if (a.den) s /= a.den[item];
      a.out[item] = make_double2(v.x * s, v.y * s);
    }
  }
  if (a.quantum > 0) {
    __syncthreads();  // every warp of the block is done with the slot's tables
    if (threadIdx.x == 0) {
      __threadfence();
      atomicExch(a.slot_flags + bslot, 0);
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
  return precision == BSG_PREC_FP64 ? sizeof(double2) : precision == BSG_PREC_SPLIT ? sizeof(PrecSplit::C) : sizeof(float2);
}

// Converts n c128 values at src into the precision's storage type at dst.
static int convert_into(bsg_handle_t h, const double* src, int64_t n, int precision, void* dst, cudaStream_t st) {
  if (n == 0) return BSG_OK;
  const int threads = 256;
  const int64_t blocks = (n + threads - 1) / threads;
  if (precision == BSG_PREC_FP64) {
    BSG_CUDA(cudaMemcpyAsync(dst, src, (size_t)n * 16, cudaMemcpyDeviceToDevice, st));
  } else if (precision == BSG_PREC_SPLIT) {
    BSG_PROFILED(h, BSG_K_PREP, st, (double)n,
                 (convert_kernel<PrecSplit::C><<<(unsigned)blocks, threads, 0, st>>>(
                     reinterpret_cast<const double2*>(src), reinterpret_cast<PrecSplit::C*>(dst), n)));
  } else {
    BSG_PROFILED(h, BSG_K_PREP, st, (double)n,
                 (convert_kernel<float2><<<(unsigned)blocks, threads, 0, st>>>(
                     reinterpret_cast<const double2*>(src), reinterpret_cast<float2*>(dst), n)));
  }
  return BSG_OK;
}

// Many conversions in one launch: job y converts jobs[y].n values (blocks
// along x cover the largest job).
struct ConvJob {
  const double2* src;
  void* dst;
  int64_t n;
};

template <class C>
__global__ void convert_jobs_kernel(const ConvJob* __restrict__ jobs) {
  const ConvJob jb = jobs[blockIdx.y];
  C* dst = reinterpret_cast<C*>(jb.dst);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < jb.n; i += (int64_t)gridDim.x * blockDim.x) {
    if constexpr (std::is_same<C, float2>::value) {
      dst[i] = PrecF32::from_c128(jb.src[i]);
    } else {
      dst[i] = PrecSplit::from_c128(jb.src[i]);
    }
  }
}

// jobs_host: pinned; jobs_dev: device room for n_jobs ConvJobs.  FP64 needs no conversion.
static int convert_many(bsg_handle_t h, const ConvJob* jobs_host, int n_jobs, void* jobs_dev, int precision,
                        cudaStream_t st) {
  if (n_jobs == 0 || precision == BSG_PREC_FP64) return BSG_OK;
  int64_t nmax = 0;
  double work = 0.0;
  for (int i = 0; i < n_jobs; ++i) {
    nmax = std::max(nmax, jobs_host[i].n);
    work += (double)jobs_host[i].n;
  }
  BSG_CUDA(cudaMemcpyAsync(jobs_dev, jobs_host, sizeof(ConvJob) * n_jobs, cudaMemcpyHostToDevice, st));
  const unsigned bx = unsigned(std::min<int64_t>((nmax + 255) / 256, 64));
  const ConvJob* jd = reinterpret_cast<const ConvJob*>(jobs_dev);
  if (precision == BSG_PREC_SPLIT) {
    BSG_PROFILED(h, BSG_K_PREP, st, work, (convert_jobs_kernel<PrecSplit::C><<<dim3(bx, n_jobs), 256, 0, st>>>(jd)));
  } else {
    BSG_PROFILED(h, BSG_K_PREP, st, work, (convert_jobs_kernel<float2><<<dim3(bx, n_jobs), 256, 0, st>>>(jd)));
  }
  return BSG_OK;
}

// The small device-to-host transfers of the whole-MPS build (cut status,
// label keys, row counts, flags) written by a kernel into the pinned staging
// buffer through its device mapping.  Copy-engine copies would queue behind
// the Gamma downloads of the host-output build: a group's label keys (which
// its host planning waits for) arrived ~10 ms late there.
constexpr int kHostCopyJobs = 6;
struct HostCopyJobs {
  uint32_t* dst[kHostCopyJobs];  // device addresses of pinned host words
  const uint32_t* src[kHostCopyJobs];
  int64_t words[kHostCopyJobs];
  int n;
};
__global__ void host_copy_kernel(const __grid_constant__ HostCopyJobs j) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int q = 0; q < j.n; ++q)
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < j.words[q]; i += stride)
      j.dst[q][i] = j.src[q][i];
  __threadfence_system();
}

// Span y of the list is set to its byte value: the 16-byte-aligned body by
// vector stores (blocks along x stride over it), the unaligned head and tail
// bytes by the first threads.
__global__ void fill_spans_kernel(const FillSpan* __restrict__ spans) {
  const FillSpan f = spans[blockIdx.y];
  if (f.bytes <= 0) return;
  unsigned char* p = reinterpret_cast<unsigned char*>(f.p);
  const int64_t mis = (16 - (int64_t)(reinterpret_cast<uintptr_t>(p) & 15)) & 15;
  const int64_t head = mis < f.bytes ? mis : f.bytes;
  const int64_t body = (f.bytes - head) / 16, tail0 = head + body * 16;
  const unsigned char b = (unsigned char)f.value;
  const unsigned w = 0x01010101u * b;
  const uint4 v = make_uint4(w, w, w, w);
  uint4* q = reinterpret_cast<uint4*>(p + head);
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = t; i < body; i += stride) q[i] = v;
  if (t < head) p[t] = b;
  if (t < f.bytes - tail0) p[tail0 + t] = b;
}

int fill_spans_dev(bsg_handle_t h, const FillSpan* dev_spans, int n, int64_t max_bytes, cudaStream_t st) {
  if (n == 0 || max_bytes <= 0) return BSG_OK;
  // about 8 vector stores per thread on the largest span, at most 64 blocks a span
  const unsigned bx = unsigned(std::max<int64_t>(1, std::min<int64_t>((max_bytes / 16 + 2047) / 2048, 64)));
  BSG_PROFILED(h, BSG_K_PREP, st, (double)n, (fill_spans_kernel<<<dim3(bx, n), 256, 0, st>>>(dev_spans)));
  return BSG_OK;
}

int fill_spans(bsg_handle_t h, const FillSpan* spans, int n, void* dev, void* stage, cudaStream_t st) {
  if (n == 0) return BSG_OK;
  int64_t mx = 0;
  for (int i = 0; i < n; ++i) mx = std::max(mx, spans[i].bytes);
  std::memcpy(stage, spans, sizeof(FillSpan) * n);
  BSG_CUDA(cudaMemcpyAsync(dev, stage, sizeof(FillSpan) * n, cudaMemcpyHostToDevice, st));
  return fill_spans_dev(h, reinterpret_cast<const FillSpan*>(dev), n, mx, st);
}

static int convert_sigma(bsg_handle_t h, const double* src, int64_t n, int precision, bsg::DevBuf& buf,
                         const void** out, cudaStream_t st) {
  if (precision == BSG_PREC_FP64 || n == 0) {
    *out = src;
    return BSG_OK;
  }
  BSG_TRY(buf.ensure((size_t)n * prec_bytes(precision)));
  BSG_TRY(convert_into(h, src, n, precision, buf.ptr, st));
  *out = buf.ptr;
  return BSG_OK;
}

// ---------------------------------------------------------------------------
// Host-side planning
// ---------------------------------------------------------------------------
struct Buckets {
  std::vector<int32_t> progs;    // bucket -> program
  std::vector<int32_t> sites;    // bucket -> site (0 in target/matrix modes)
  std::vector<int64_t> counts;   // bucket -> items
  std::vector<int32_t> offsets;  // bucket -> first slot (multiple of 32)
  std::vector<int32_t> chunk_start;  // bucket -> first chunk (nb + 1 entries)
  int64_t slots = 0;
  int states_max = 1;
  double work = 0.0;             // complex multiply-adds of all items
};

static int64_t prog_trans(const bsg::ProgramSet& ps, int p) {
  int s0 = ps.state_off[p], ns = ps.nstates[p];
  return (int64_t)ps.st_trans_off[s0 + ns - 1] + ps.st_trans_cnt[s0 + ns - 1] - ps.st_trans_off[s0];
}

// Orders buckets large-table programs first, then small-table programs
// (small_program), each group by per-item cost, expensive first so the work
// queue starts the long programs early; assigns padded slot ranges;
// `remap[old] = new`.
// Programs with at most `small_entries` table entries (class pairs + DP
// states) per item run in their own DP launch with small per-warp slices.
static bool small_program(const bsg::ProgramSet& ps, int p, int small_entries) {
  return ps.k[p] * (ps.k[p] + 1) / 2 + ps.fslots[p] <= small_entries;
}

static int layout_buckets(const bsg::ProgramSet& ps, int small_entries, Buckets& bk, std::vector<int32_t>& remap) {
  const int nb = int(bk.progs.size());
  std::vector<int> order(nb);
  std::iota(order.begin(), order.end(), 0);
  // stable order by descending cost, as a counting sort over the few
  // distinct costs (a cost depends only on the bucket's program)
  std::vector<int64_t> cost(nb);
  std::vector<int64_t> pcost(ps.k.size(), INT64_MIN);
  for (int b = 0; b < nb; ++b) {
    const int p = bk.progs[b];
    if (pcost[p] == INT64_MIN) {
      const bool small = small_program(ps, p, small_entries);
      pcost[p] = small ? -(int64_t(1) << 40) - prog_trans(ps, p) : prog_trans(ps, p);
    }
    cost[b] = pcost[p];
  }
  {
    std::vector<int64_t> uniq;
    for (size_t p = 0; p < pcost.size(); ++p)
      if (pcost[p] != INT64_MIN) uniq.push_back(pcost[p]);
    std::sort(uniq.begin(), uniq.end(), std::greater<int64_t>());
    uniq.erase(std::unique(uniq.begin(), uniq.end()), uniq.end());
    std::vector<int32_t> prank(pcost.size(), 0);
    for (size_t p = 0; p < pcost.size(); ++p)
      if (pcost[p] != INT64_MIN)
        prank[p] = int32_t(std::lower_bound(uniq.begin(), uniq.end(), pcost[p], std::greater<int64_t>()) - uniq.begin());
    std::vector<int> start(uniq.size() + 1, 0);
    for (int b = 0; b < nb; ++b) start[prank[bk.progs[b]] + 1]++;
    for (size_t r = 0; r < uniq.size(); ++r) start[r + 1] += start[r];
    for (int b = 0; b < nb; ++b) order[start[prank[bk.progs[b]]]++] = b;
  }
  Buckets out;
  remap.assign(nb, -1);
  out.progs.resize(nb);
  out.sites.resize(nb);
  out.counts.resize(nb);
  for (int i = 0; i < nb; ++i) {
    out.progs[i] = bk.progs[order[i]];
    out.sites[i] = bk.sites[order[i]];
    out.counts[i] = bk.counts[order[i]];
    remap[order[i]] = i;
  }
  out.offsets.assign(nb, 0);
  out.chunk_start.assign(nb + 1, 0);
  int64_t off = 0;
  for (int b = 0; b < nb; ++b) {
    out.offsets[b] = int32_t(off);
    out.chunk_start[b] = int32_t(off / 32);
    const int64_t ch = (out.counts[b] + 31) / 32;
    off += ch * 32;
    const int p = out.progs[b];
    out.states_max = std::max(out.states_max, ps.fslots[p]);
    out.work += (double)out.counts[b] * (double)prog_trans(ps, p);
    if (off > INT32_MAX) {
      set_error("too many work items in one launch (%lld)", (long long)off);
      return BSG_ERR_LIMIT;
    }
  }
  out.slots = off;
  out.chunk_start[nb] = int32_t(off / 32);
  bk = std::move(out);
  return BSG_OK;
}

// Per-site plan on the host: rows grouped by partition key, and the bucket
// of every (j, left group, right group) combination.
struct SitePlanHost {
  int KL = 0, KR = 0, ngl = 0, ngr = 0, d = 0;
  std::vector<int32_t> perm_l, grp_l, perm_r, grp_r, bucket_of, combo_off, gstart_l, gcnt_l, gstart_r;
  std::vector<int8_t> combo_j;
};

static void group_rows(const uint64_t* key, int rows, std::vector<int32_t>& perm, std::vector<int32_t>& grp,
                       std::vector<uint64_t>& gkey, std::vector<int64_t>& gcnt) {
  perm.resize(rows);
  std::iota(perm.begin(), perm.end(), 0);
  std::stable_sort(perm.begin(), perm.end(), [&](int x, int y) { return key[x] < key[y]; });
  grp.resize(rows);
  gkey.clear();
  gcnt.clear();
  for (int i = 0; i < rows; ++i) {
    if (i == 0 || key[perm[i]] != key[perm[i - 1]]) {
      gkey.push_back(key[perm[i]]);
      gcnt.push_back(0);
    }
    grp[i] = int32_t(gkey.size() - 1);
    gcnt.back()++;
  }
}

static ProgDev prog_dev(const bsg::ProgramSet& ps) {
  return ProgDev{ps.d_k, ps.d_nstates, ps.d_state_off, ps.d_trans, ps.d_st_pack};
}

// Launch shape for chunks [c0, c1) whose programs need at most smax F entries
// table entries per warp.
struct DPLaunch {
  int64_t c0 = 0, c1 = 0;
  int smax = 1;
  double work = 0.0;
  double wtrans = 0.0;  // program transitions of all chunks (one warp runs a chunk's program once)
  int blocks = 0;
  size_t per_warp = 0;
  int64_t quantum = 0;  // > 0: yielding launch with `slots` table slots
  int slots = 0;
};

// Yielding launch (quantum > 0) when the tables of every resident block fit
// the scratch budget: a warp leaves once it has run `quantum` transitions, so
// the SMs turn over to higher-priority streams within about one quantum.
// The grid covers the work either way: warps x quantum >= all transitions, or
// at least one warp per chunk (a warp takes one chunk before it may leave).
// Otherwise a persistent launch: every warp drains the queue.
template <class P>
static void dp_shape(bsg_handle_t h, int blocks_per_sm, int occupancy, DPLaunch& L) {
  const int threads = kDPThreads;
  L.per_warp = (size_t)L.smax * 32 * sizeof(typename P::CF);
  const size_t budget = (size_t)h->tune[BSG_TUNE_DP_SCRATCH_MIB] << 20;  // per-warp tables of one launch
  const int64_t q = (int64_t)h->tune[BSG_TUNE_DP_QUANTUM] * 256;
  const int64_t slots = (int64_t)h->num_sms * occupancy;
  if (q > 0 && occupancy > 0 && (size_t)slots * (threads / 32) * L.per_warp <= budget) {
    const int64_t by_work = slots + (int64_t)std::ceil(L.wtrans / double(q * (threads / 32)));
    const int64_t by_chunks = std::max<int64_t>(1, (L.c1 - L.c0 + (threads / 32) - 1) / (threads / 32));
    L.quantum = q;
    L.slots = int(slots);
    L.blocks = int(std::min<int64_t>(std::min(by_work, by_chunks), int64_t(1) << 30));
    return;
  }
  L.quantum = 0;
  L.slots = 0;
  int64_t warps = (int64_t)h->num_sms * blocks_per_sm * (threads / 32);
  while (warps > (threads / 32) * (int64_t)h->num_sms && (size_t)warps * L.per_warp > budget) warps /= 2;
  const int64_t w_use = std::min<int64_t>(warps, std::max<int64_t>(L.c1 - L.c0, 1));
  L.blocks = std::max<int>(1, int((w_use + (threads / 32) - 1) / (threads / 32)));
}

// Chunks come large-table programs first (layout_buckets).  Those run in one
// launch whose per-warp slices fit its largest program; small programs
// (small_program) run in a second launch with small slices, so their warps'
// tables stay in L1/L2.  Both launches share the scratch (same stream) and
// use separate work counters (a.counter[0..1]).
template <class P, int MODE>
static int launch_dp_t(bsg_handle_t h, DPArgs a, const Buckets& bk, bsg::DevBuf& scratch, cudaStream_t st) {
  const auto& ps = h->programs;
  const int nb = int(bk.progs.size());
  const int64_t nch = nb ? bk.chunk_start[nb] : 0;
  const int small_entries = h->tune[BSG_TUNE_DP_SMALL_ENTRIES];
  auto small = [&](int p) { return small_program(ps, p, small_entries); };
  DPLaunch Ls, Lb;
  int first_small = nb;  // buckets are large-table programs first (layout_buckets)
  while (first_small > 0 && small(bk.progs[first_small - 1])) --first_small;
  Lb.c1 = first_small < nb ? bk.chunk_start[first_small] : nch;
  Ls.c0 = Lb.c1;
  Ls.c1 = nch;
  // slice sizes from the buckets each launch actually runs
  for (int b = 0; b < nb; ++b) {
    const int p = bk.progs[b];
    DPLaunch& L = b < first_small ? Lb : Ls;
    L.smax = std::max(L.smax, ps.fslots[p]);
    L.work += (double)bk.counts[b] * (double)prog_trans(ps, p);
    L.wtrans += (double)(bk.chunk_start[b + 1] - bk.chunk_start[b]) * (double)prog_trans(ps, p);
    if (h->prof.on) {
      const double ch = double(bk.chunk_start[b + 1] - bk.chunk_start[b]);
      const int s0 = ps.state_off[p], ns = ps.nstates[p];
      for (double v : {b < first_small ? 0.0 : 1.0, ch, double(ps.k[p]), double(ps.fslots[p]), double(ns),
                       double(prog_trans(ps, p))})
        h->prof.dp_rows.push_back(v);
      auto& hist = h->prof.dp_state_hist;
      if (hist.size() < 65) hist.resize(65, 0.0);
      for (int q = 1; q < ns; ++q) hist[std::min(ps.st_trans_cnt[s0 + q], 64)] += ch;
    }
  }
  // FP64 helper (split precision, site mode): dp_kernel<PrecF64> on the
  // handle's second stream draws chunks from the same counters, so the FP64
  // pipe takes a share of the items while the FP32 pipe runs the split DP.
  const int helper_bps = h->tune[BSG_TUNE_DP_FP64_BLOCKS];
  const bool helper = MODE == MODE_SITE && std::is_same<P, PrecSplit>::value && helper_bps > 0;
  static_assert(sizeof(typename PrecF64::CF) == sizeof(typename P::CF) || !std::is_same<P, PrecSplit>::value, "");
  BSG_CUDA(cudaFuncSetAttribute(dp_kernel<P, MODE>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                h->tune[BSG_TUNE_DP_L1_CARVEOUT]));
  int occ = 0;
  if (!helper) BSG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, dp_kernel<P, MODE>, kDPThreads, 0));
  dp_shape<P>(h, h->tune[BSG_TUNE_DP_SMALL_BLOCKS], occ, Ls);
  dp_shape<P>(h, h->tune[BSG_TUNE_DP_BLOCKS_PER_SM], occ, Lb);
  const bool run_b = Lb.c1 > Lb.c0, run_s = Ls.c1 > Ls.c0 || !run_b;
  auto tables = [](const DPLaunch& L) { return (size_t)(L.quantum > 0 ? L.slots : L.blocks) * kDPWarps * L.per_warp; };
  size_t need = 0;
  if (run_s) need = std::max(need, tables(Ls));
  if (run_b) need = std::max(need, tables(Lb));
  // slot flags of the yielding launches (all free again when a launch ends)
  const size_t flags_off = (need + 255) & ~size_t(255);
  const int n_flags = std::max(run_s ? Ls.slots : 0, run_b ? Lb.slots : 0);
  if (n_flags > 0) need = flags_off + (size_t)n_flags * 4;
  DPLaunch Hs = Ls, Hb = Lb;  // helper shapes (same slices, fewer blocks)
  size_t helper_off = 0;
  if (helper) {
    Hs.blocks = std::min(Hs.blocks, h->num_sms * helper_bps);
    Hb.blocks = std::min(Hb.blocks, h->num_sms * helper_bps);
    helper_off = (need + 255) & ~size_t(255);
    size_t hneed = 0;
    if (run_s) hneed = std::max(hneed, (size_t)Hs.blocks * kDPWarps * Hs.per_warp);
    if (run_b) hneed = std::max(hneed, (size_t)Hb.blocks * kDPWarps * Hb.per_warp);
    need = helper_off + hneed;
  }
  BSG_TRY(scratch.ensure(need));
  int* flags = n_flags > 0 ? reinterpret_cast<int*>(reinterpret_cast<char*>(scratch.ptr) + flags_off) : nullptr;
  if (flags) BSG_CUDA(cudaMemsetAsync(flags, 0, (size_t)n_flags * 4, st));
  a.scratch = scratch.ptr;
  unsigned long long* ctr = a.counter;
  const DPLaunch* Ls_or_b[2] = {run_b ? &Lb : nullptr, run_s ? &Ls : nullptr};
  const DPLaunch* H_or_b[2] = {run_b ? &Hb : nullptr, run_s ? &Hs : nullptr};
  cudaStream_t aux = nullptr;
  cudaEvent_t ev_dp = nullptr;
  if (helper) {
    BSG_TRY(h->ensure_aux());
    aux = h->aux_stream;
    BSG_CUDA(cudaEventRecord(h->aux_fork, st));
    BSG_CUDA(cudaStreamWaitEvent(aux, h->aux_fork, 0));
    if (h->prof.on) BSG_TRY(h->prof.begin(BSG_K_DP, st, &ev_dp));
  }
  for (int i = 0; i < 2; ++i) {
    const DPLaunch* L = Ls_or_b[i];
    if (!L) continue;
    a.states_max = L->smax;
    a.chunk_base = L->c0;
    a.n_chunks = L->c1 - L->c0;
    a.counter = ctr + i;
    a.scratch = scratch.ptr;
    a.quantum = L->quantum;
    a.slot_flags = flags;
    a.n_slots = L->slots;
    if (helper) {
      dp_kernel<P, MODE><<<L->blocks, kDPThreads, 0, st>>>(a);
      BSG_CUDA(cudaGetLastError());
      DPArgs ha = a;
      ha.scratch = reinterpret_cast<char*>(scratch.ptr) + helper_off;
      dp_kernel<PrecF64, MODE><<<H_or_b[i]->blocks, kDPThreads, 0, aux>>>(ha);
      BSG_CUDA(cudaGetLastError());
    } else {
      BSG_PROFILED(h, BSG_K_DP, st, L->work, (dp_kernel<P, MODE><<<L->blocks, kDPThreads, 0, st>>>(a)));
      if (L->quantum > 0) {
        // drain: a persistent launch over the table slots finishes any chunk
        // left behind by a block that found no slot (normally none: it exits at once)
        DPArgs da = a;
        da.quantum = 0;
        dp_kernel<P, MODE><<<std::min(L->slots, h->num_sms), kDPThreads, 0, st>>>(da);
        BSG_CUDA(cudaGetLastError());
      }
    }
  }
  if (helper) {
    BSG_CUDA(cudaEventRecord(h->aux_join, aux));
    BSG_CUDA(cudaStreamWaitEvent(st, h->aux_join, 0));
    if (h->prof.on) BSG_TRY(h->prof.end(BSG_K_DP, st, ev_dp, Ls.work + Lb.work));
  }
  return BSG_OK;
}

template <int MODE>
static int launch_dp(bsg_handle_t h, int precision, DPArgs a, const Buckets& bk, bsg::DevBuf& scratch,
                     cudaStream_t st) {
  if (precision == BSG_PREC_FP64) return launch_dp_t<PrecF64, MODE>(h, a, bk, scratch, st);
  if (precision == BSG_PREC_SPLIT) return launch_dp_t<PrecSplit, MODE>(h, a, bk, scratch, st);
  return launch_dp_t<PrecF32, MODE>(h, a, bk, scratch, st);
}

// ---- target / matrix modes ------------------------------------------------
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
      bk.sites.push_back(0);
      bk.counts.push_back(0);
    } else {
      b = it->second;
    }
    bk.counts[b]++;
    item_bucket[i] = b;
  }
  std::vector<int32_t> remap;
  BSG_TRY(layout_buckets(ps, h->tune[BSG_TUNE_DP_SMALL_ENTRIES], bk, remap));
  items.assign(bk.slots, -1);
  std::vector<int64_t> cur(bk.progs.size(), 0);
  for (size_t i = 0; i < keys.size(); ++i) {
    if (item_bucket[i] < 0) continue;
    const int b = remap[item_bucket[i]];
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
  const int nb = int(bk.progs.size());
  BSG_TRY(h->items.ensure((size_t)bk.slots * 4 + (size_t)(2 * nb + 1) * 4 + 64));
  int32_t* d_items = reinterpret_cast<int32_t*>(h->items.ptr);
  int32_t* d_bchunk = d_items + bk.slots;
  int32_t* d_bprog = d_bchunk + nb + 1;
  BSG_CUDA(cudaMemcpyAsync(d_items, items.data(), (size_t)bk.slots * 4, cudaMemcpyHostToDevice, st));
  BSG_CUDA(cudaMemcpyAsync(d_bchunk, bk.chunk_start.data(), (size_t)(nb + 1) * 4, cudaMemcpyHostToDevice, st));
  BSG_CUDA(cudaMemcpyAsync(d_bprog, bk.progs.data(), (size_t)nb * 4, cudaMemcpyHostToDevice, st));
  BSG_TRY(h->misc.ensure(64));
  auto* counter = reinterpret_cast<unsigned long long*>(h->misc.ptr);
  BSG_CUDA(cudaMemsetAsync(counter, 0, 16, st));
  DPArgs a{};
  a.prog = prog_dev(h->programs);
  a.items = d_items;
  a.bucket_chunk = d_bchunk;
  a.bucket_prog = d_bprog;
  a.bucket_site = nullptr;
  a.nb = nb;
  a.counter = counter;
  a.sigma = sig;
  a.n_len = n_len;
  a.targets = targets;
  a.n = n;
  a.den = den;
  a.out = reinterpret_cast<double2*>(out);
  if (mode == MODE_TARGETS) BSG_TRY(launch_dp<MODE_TARGETS>(h, precision, a, bk, h->warp_scratch, st));
  else BSG_TRY(launch_dp<MODE_MATRICES>(h, precision, a, bk, h->warp_scratch, st));
  BSG_CUDA(cudaStreamSynchronize(st));  // the host vectors above go out of scope
  return BSG_OK;
}

// ---- parallel host planning ----------------------------------------------------
// Phase A (parallel): group each site's rows by key and list its (j, gl, gr)
// combinations with their partition keys.  Phase B (serial): generate the
// programs of keys not seen before.  Phase C (parallel): map combinations to
// per-site buckets.  Phase D (serial): concatenate the buckets of all sites.
// Worker threads kept for the life of the process (planning runs several
// parallel phases per call; starting threads each time cost more than the
// phases on small builds).  One parallel_for at a time uses the pool; a call
// that finds it busy (another handle planning on another thread) runs inline.
class PlanPool {
 public:
  explicit PlanPool(int workers) : owner(getpid()) {
    for (int t = 0; t < workers; ++t) th_.emplace_back([this] { work(); });
  }
  const pid_t owner;  // a forked child inherits this object but not its threads
  ~PlanPool() {
    {
      std::lock_guard<std::mutex> g(m_);
      stop_ = true;
    }
    cv_.notify_all();
    for (auto& x : th_) x.join();
  }
  std::mutex run_mutex;
  // Runs f(0..n-1) on the workers and the calling thread; returns when every
  // index is done.  It waits only for the workers that took the job: one that
  // wakes late (descheduled on a busy host) finds the job withdrawn and skips it.
  void run(int n, const std::function<void(int)>& f) {
    {
      std::lock_guard<std::mutex> g(m_);
      job_ = &f;
      n_ = n;
      next_.store(0);
      ++gen_;
    }
    cv_.notify_all();
    for (int i = next_++; i < n; i = next_++) f(i);
    std::unique_lock<std::mutex> g(m_);
    job_ = nullptr;  // no worker takes it from now on
    done_cv_.wait(g, [this] { return active_ == 0; });
  }

 private:
  void work() {
    uint64_t seen = 0;
    while (true) {
      const std::function<void(int)>* job;
      int n;
      {
        std::unique_lock<std::mutex> g(m_);
        cv_.wait(g, [&] { return stop_ || gen_ != seen; });
        if (stop_) return;
        seen = gen_;
        job = job_;
        n = n_;
        if (!job) continue;  // already finished by the others
        ++active_;
      }
      for (int i = next_++; i < n; i = next_++) (*job)(i);
      std::lock_guard<std::mutex> g(m_);
      if (--active_ == 0) done_cv_.notify_one();
    }
  }
  std::vector<std::thread> th_;
  std::mutex m_;
  std::condition_variable cv_, done_cv_;
  const std::function<void(int)>* job_ = nullptr;
  int n_ = 0, active_ = 0;
  uint64_t gen_ = 0;
  bool stop_ = false;
  std::atomic<int> next_{0};
};

template <class F>
static void parallel_for(int n, F&& f) {
  static const int hw = int(std::max(1u, std::thread::hardware_concurrency()));
  if (hw <= 1 || n < 4) {
    for (int i = 0; i < n; ++i) f(i);
    return;
  }
  static PlanPool pool(std::min(hw, 32) - 1);
  std::unique_lock<std::mutex> busy(pool.run_mutex, std::defer_lock);
  if (pool.owner != getpid() || !busy.try_lock()) {
    for (int i = 0; i < n; ++i) f(i);
    return;
  }
  const std::function<void(int)> fn = [&f](int i) { f(i); };
  pool.run(n, fn);
}

struct SiteCombos {
  std::vector<uint64_t> gk_l, gk_r;
  std::vector<int64_t> gc_l, gc_r;
  std::vector<uint64_t> keys;   // per (j, gl, gr): full key, or ~0 for odd order
  std::vector<int32_t> prog;    // its program, -1 until generated
  std::vector<uint64_t> missing;  // keys without a program yet
  int err = 0;
};

using plan_clk = std::chrono::steady_clock;
static double plan_ms_since(plan_clk::time_point& t) {
  const auto now = plan_clk::now();
  const double ms = std::chrono::duration<double, std::milli>(now - t).count();
  t = now;
  return ms;
}

// ph: when non-null, host ms of phases A-D are added to ph[0..3]
static int plan_sites_parallel(bsg::ProgramSet& ps, const uint64_t* const* kl, const int* KL,
                               const uint64_t* const* kr, const int* KR, int ns, const int* dv,
                               std::vector<SitePlanHost>& plans, Buckets& bk, double* ph = nullptr) {
  auto t_ph = plan_clk::now();
  plans.assign(ns, SitePlanHost());
  std::vector<SiteCombos> cb(ns);
  parallel_for(ns, [&](int s) {
    SitePlanHost& sp = plans[s];
    SiteCombos& c = cb[s];
    const int d = dv[s];
    sp.KL = KL[s];
    sp.KR = KR[s];
    sp.d = d;
    group_rows(kl[s], KL[s], sp.perm_l, sp.grp_l, c.gk_l, c.gc_l);
    group_rows(kr[s], KR[s], sp.perm_r, sp.grp_r, c.gk_r, c.gc_r);
    sp.ngl = int(c.gk_l.size());
    sp.ngr = int(c.gk_r.size());
    c.keys.assign((size_t)sp.ngl * sp.ngr, ~0ull);
    c.prog.assign(c.keys.size(), -1);
    // One site program per (left group, right group): its roots are the
    // even orders j + n_l + n_r over j = jmax, jmax - 2, ... >= 0 (jmax the
    // largest j < d of that parity), and its items carry j = jmax.  The
    // program index is only read here (phase B adds to it afterwards).
    for (int gl = 0; gl < sp.ngl; ++gl) {
      const int nl = key_order(c.gk_l[gl]);
      for (int gr = 0; gr < sp.ngr; ++gr) {
        const int nlr = nl + key_order(c.gk_r[gr]);
        const int jmax = (d - 1) - (((d - 1) + nlr) & 1);
        if (jmax < 0) continue;  // d = 1 and an odd order: no even hafnian
        if (jmax + nlr > BSG_MAX_ORDER) {
          c.err = 1;
          continue;
        }
        const size_t o = (size_t)gl * sp.ngr + gr;
        const uint64_t k = key_site_roots(c.gk_l[gl] + c.gk_r[gr], jmax);
        c.keys[o] = k;
        auto it = ps.index.find(k);
        if (it != ps.index.end()) c.prog[o] = it->second;
        else c.missing.push_back(k);
      }
    }
  });
  for (int s = 0; s < ns; ++s)
    if (cb[s].err) {
      set_error("site %d: hafnian order exceeds BSG_MAX_ORDER", s);
      return BSG_ERR_LIMIT;
    }
  if (ph) ph[0] += plan_ms_since(t_ph);
  // phase B: new programs (only the keys phase A did not find), built in
  // parallel and appended in site / key order
  {
    std::vector<uint64_t> uniq;
    std::unordered_set<uint64_t> seen_k;
    for (int s = 0; s < ns; ++s)
      for (uint64_t k : cb[s].missing)
        if (!ps.index.count(k) && seen_k.insert(k).second) uniq.push_back(k);
    std::vector<ProgramBuild> built(uniq.size());
    parallel_for(int(uniq.size()), [&](int i) { build_program(uniq[i], built[i]); });
    for (size_t i = 0; i < uniq.size(); ++i) {
      if (built[i].err != BSG_OK) {
        set_error("%s", built[i].msg.c_str());
        return built[i].err;
      }
      append_program(ps, uniq[i], built[i]);
    }
  }
  if (ph) ph[1] += plan_ms_since(t_ph);
  // phase C: per-site buckets (read-only program index)
  std::vector<std::vector<int32_t>> lprog(ns);
  std::vector<std::vector<int64_t>> lcount(ns);
  parallel_for(ns, [&](int s) {
    SitePlanHost& sp = plans[s];
    const SiteCombos& c = cb[s];
    std::unordered_map<int32_t, int32_t> local;
    sp.bucket_of.assign(c.keys.size(), -1);
    sp.combo_off.assign(c.keys.size(), 0);
    sp.combo_j.assign(c.keys.size(), 0);
    sp.gstart_l.assign(sp.ngl, 0);
    sp.gcnt_l.assign(sp.ngl, 0);
    sp.gstart_r.assign(sp.ngr, 0);
    for (int g = 0, at = 0; g < sp.ngl; at += int(c.gc_l[g]), ++g) {
      sp.gstart_l[g] = at;
      sp.gcnt_l[g] = int32_t(c.gc_l[g]);
    }
    for (int g = 0, at = 0; g < sp.ngr; at += int(c.gc_r[g]), ++g) sp.gstart_r[g] = at;
    for (int gl = 0; gl < sp.ngl; ++gl)
      for (int gr = 0; gr < sp.ngr; ++gr) {
        const size_t o = (size_t)gl * sp.ngr + gr;
        const uint64_t k = c.keys[o];
        if (k == ~0ull) continue;
        sp.combo_j[o] = int8_t(int(k >> kKeyRootShift) - 1);
        const int32_t prog = c.prog[o] >= 0 ? c.prog[o] : ps.index.find(k)->second;
        auto it = local.find(prog);
        int32_t b;
        if (it == local.end()) {
          b = int32_t(lprog[s].size());
          local.emplace(prog, b);
          lprog[s].push_back(prog);
          lcount[s].push_back(0);
        } else {
          b = it->second;
        }
        sp.combo_off[o] = int32_t(lcount[s][b]);
        lcount[s][b] += c.gc_l[gl] * c.gc_r[gr];
        sp.bucket_of[o] = b;
      }
  });
  if (ph) ph[2] += plan_ms_since(t_ph);
  // phase D: global bucket list
  std::vector<int32_t> base(ns, 0);
  for (int s = 0; s < ns; ++s) {
    base[s] = int32_t(bk.progs.size());
    for (size_t b = 0; b < lprog[s].size(); ++b) {
      bk.progs.push_back(lprog[s][b]);
      bk.sites.push_back(s);
      bk.counts.push_back(lcount[s][b]);
    }
  }
  parallel_for(ns, [&](int s) {
    for (auto& b : plans[s].bucket_of)
      if (b >= 0) b += base[s];
  });
  if (ph) ph[3] += plan_ms_since(t_ph);
  return BSG_OK;
}

// ---- site mode: shared by bsg_build_site (one site) and bsg_build_mps --------
struct SiteInput {
  int kind;
  int Mr;
  const void* sigma;  // policy-typed
  const double2* sigma64;  // FP64 copy
  const double* Z;
  const double* lambda;   // left rows (null for LAST)
  // (left scales are computed by run_sites)
  const uint64_t* hkey_l; // host copies of the row keys
  const uint64_t* hkey_r;
  int KL, KR;
  RowTable lt;            // device row tables (already offset to this cut)
  RowTable rt;
  void* gamma;
  int d = 0, chi = 0;     // this site's cutoff and bond dimension (0: the call's)
};

// Plans, uploads and launches the scatter + DP for a set of sites.
static int run_sites(bsg_handle_t h, const std::vector<SiteInput>& in, int d, int chi, int precision, int out_dtype,
                     bsg_handle_s::SiteSlot& slot, cudaStream_t st) {
  auto& ps = h->programs;
  const int ns = int(in.size());
  double* ph = h->prof.on ? h->prof.plan_ms : nullptr;
  const auto t_all = plan_clk::now();
  Buckets bk;
  std::vector<SitePlanHost> plans;
  {
    std::vector<const uint64_t*> kl(ns), kr(ns);
    std::vector<int> KL(ns), KR(ns), dv(ns);
    for (int s = 0; s < ns; ++s) {
      kl[s] = in[s].hkey_l;
      kr[s] = in[s].hkey_r;
      KL[s] = in[s].KL;
      KR[s] = in[s].KR;
      dv[s] = in[s].d ? in[s].d : d;
    }
    BSG_TRY(plan_sites_parallel(ps, kl.data(), KL.data(), kr.data(), KR.data(), ns, dv.data(), plans, bk, ph));
  }
  auto t_ph = plan_clk::now();
  std::vector<int32_t> remap;
  BSG_TRY(layout_buckets(ps, h->tune[BSG_TUNE_DP_SMALL_ENTRIES], bk, remap));
  parallel_for(ns, [&](int s) {
    for (auto& b : plans[s].bucket_of)
      if (b >= 0) b = remap[b];
  });
  if (ph) ph[4] += plan_ms_since(t_ph);
  BSG_TRY(programs_upload(ps, st));
  if (ph) ph[5] += plan_ms_since(t_ph);
  const int nb = int(bk.progs.size());

  // one plan buffer: site descs, per-site tables, bucket offsets/chunks/programs/sites, counters
  auto align = [](size_t x) { return (x + 255) & ~size_t(255); };
  size_t off = 0;
  auto carve = [&](size_t bytes) {
    size_t o = off;
    off = align(off + bytes);
    return o;
  };
  const size_t o_desc = carve(sizeof(SiteDesc) * ns);
  const size_t o_lsj = carve(sizeof(LeftScaleJob) * ns);
  const size_t o_fs = carve(sizeof(FillSpan) * ns);  // Gamma clears
  std::vector<size_t> o_pl(ns), o_gl(ns), o_pr(ns), o_gr(ns), o_bo(ns), o_co(ns), o_cj(ns), o_gsl(ns), o_gcl(ns),
      o_gsr(ns), o_lsd(ns), o_lsf(ns);
  int max_kl = 1;
  for (int s = 0; s < ns; ++s) {
    o_lsd[s] = carve((size_t)in[s].KL * 8);
    o_lsf[s] = carve((size_t)in[s].KL * 8);
    max_kl = std::max(max_kl, in[s].KL);
    o_pl[s] = carve(plans[s].perm_l.size() * 4);
    o_gl[s] = carve(plans[s].grp_l.size() * 4);
    o_pr[s] = carve(plans[s].perm_r.size() * 4);
    o_gr[s] = carve(plans[s].grp_r.size() * 4);
    o_bo[s] = carve(plans[s].bucket_of.size() * 4);
    o_co[s] = carve(plans[s].combo_off.size() * 4);
    o_cj[s] = carve(plans[s].combo_j.size());
    o_gsl[s] = carve(plans[s].gstart_l.size() * 4);
    o_gcl[s] = carve(plans[s].gcnt_l.size() * 4);
    o_gsr[s] = carve(plans[s].gstart_r.size() * 4);
  }
  const size_t o_boff = carve((size_t)nb * 4 + 4), o_bend = carve((size_t)nb * 4 + 4);
  const size_t o_bch = carve((size_t)nb * 4 + 4), o_bpr = carve((size_t)nb * 4 + 4),
               o_bsi = carve((size_t)nb * 4 + 4), o_ctr = carve(16), o_sp = carve(sizeof(SitePlanDev) * ns);
  const int64_t n_chunks = nb ? bk.chunk_start[nb] : 0;
  const size_t o_cbk = carve((size_t)n_chunks * 4 + 4);
  const size_t plan_bytes = off;
  BSG_TRY(slot.plan.ensure(plan_bytes));
  BSG_TRY(slot.stage.ensure(plan_bytes));
  char* hp = reinterpret_cast<char*>(slot.stage.ptr);
  char* dp = reinterpret_cast<char*>(slot.plan.ptr);
  SiteDesc* hd = reinterpret_cast<SiteDesc*>(hp + o_desc);
  LeftScaleJob* hl = reinterpret_cast<LeftScaleJob*>(hp + o_lsj);
  FillSpan* hfs = reinterpret_cast<FillSpan*>(hp + o_fs);
  const int out_c128 = out_dtype == BSG_OUT_C128;
  const size_t esz = out_c128 ? 16 : 8;
  int64_t gamma_max = 0;
  for (int s = 0; s < ns; ++s) {
    const size_t cs = in[s].chi ? in[s].chi : chi, ds = in[s].d ? in[s].d : d;
    hfs[s] = FillSpan{in[s].gamma, (int64_t)(cs * cs * ds * esz), 0};
    gamma_max = std::max(gamma_max, hfs[s].bytes);
  }
  // per-site descriptors and plan tables into the staging buffer (disjoint
  // regions, filled by the planning threads)
  parallel_for(ns, [&](int s) {
    const SiteInput& si = in[s];
    LeftScaleJob lj{};
    lj.rowfact = si.lt.rowfact;
    lj.lambda = si.kind == BSG_SITE_LAST ? nullptr : si.lambda;
    lj.Z = si.Z;
    lj.rows = si.KL;
    lj.out_d = reinterpret_cast<double*>(dp + o_lsd[s]);
    lj.out_f = reinterpret_cast<float2*>(dp + o_lsf[s]);
    hl[s] = lj;
    SiteDesc sd{};
    sd.sigma = si.sigma;
    sd.sigma64 = si.sigma64;
    sd.Mr = si.Mr;
    sd.n_len = 2 * si.Mr;
    sd.l_ent = si.lt.entries;
    sd.l_nnz = si.lt.nnz;
    sd.l_rowfact = si.lt.rowfact;
    sd.lambda = si.kind == BSG_SITE_LAST ? nullptr : si.lambda;
    sd.r_ent = si.rt.entries;
    sd.r_nnz = si.rt.nnz;
    sd.r_rowfact = si.rt.rowfact;
    sd.r_rowfact2 = si.rt.rowfact2;
    sd.l_scale = lj.out_d;
    sd.l_scale2 = lj.out_f;
    sd.Z = si.Z;
    sd.gamma = si.gamma;
    sd.chi = si.chi ? si.chi : chi;
    sd.d = si.d ? si.d : d;
    sd.out_c128 = out_c128;
    hd[s] = sd;
    std::memcpy(hp + o_pl[s], plans[s].perm_l.data(), plans[s].perm_l.size() * 4);
    std::memcpy(hp + o_gl[s], plans[s].grp_l.data(), plans[s].grp_l.size() * 4);
    std::memcpy(hp + o_pr[s], plans[s].perm_r.data(), plans[s].perm_r.size() * 4);
    std::memcpy(hp + o_gr[s], plans[s].grp_r.data(), plans[s].grp_r.size() * 4);
    std::memcpy(hp + o_bo[s], plans[s].bucket_of.data(), plans[s].bucket_of.size() * 4);
    std::memcpy(hp + o_co[s], plans[s].combo_off.data(), plans[s].combo_off.size() * 4);
    std::memcpy(hp + o_cj[s], plans[s].combo_j.data(), plans[s].combo_j.size());
    std::memcpy(hp + o_gsl[s], plans[s].gstart_l.data(), plans[s].gstart_l.size() * 4);
    std::memcpy(hp + o_gcl[s], plans[s].gcnt_l.data(), plans[s].gcnt_l.size() * 4);
    std::memcpy(hp + o_gsr[s], plans[s].gstart_r.data(), plans[s].gstart_r.size() * 4);
  });
  std::memcpy(hp + o_boff, bk.offsets.data(), (size_t)nb * 4);
  {
    int32_t* hend = reinterpret_cast<int32_t*>(hp + o_bend);
    for (int b = 0; b < nb; ++b) hend[b] = bk.offsets[b] + int32_t(bk.counts[b]);
  }
  if (nb) {
    std::memcpy(hp + o_bch, bk.chunk_start.data(), (size_t)(nb + 1) * 4);
    std::memcpy(hp + o_bpr, bk.progs.data(), (size_t)nb * 4);
    std::memcpy(hp + o_bsi, bk.sites.data(), (size_t)nb * 4);
  }
  std::memset(hp + o_ctr, 0, 16);
  BSG_TRY(slot.items.ensure(std::max<size_t>((size_t)bk.slots * 4, 4)));
  int32_t* d_items = reinterpret_cast<int32_t*>(slot.items.ptr);
  SitePlanDev* hsp = reinterpret_cast<SitePlanDev*>(hp + o_sp);
  int64_t max_pairs = 1;
  for (int s = 0; s < ns; ++s) {
    const SitePlanHost& p = plans[s];
    auto dptr = [&](size_t o) { return reinterpret_cast<int32_t*>(dp + o); };
    hsp[s] = SitePlanDev{dptr(o_pl[s]),  dptr(o_gl[s]),  dptr(o_pr[s]), dptr(o_gr[s]), dptr(o_bo[s]),
                         dptr(o_co[s]),  reinterpret_cast<const int8_t*>(dp + o_cj[s]),
                         dptr(o_gsl[s]), dptr(o_gcl[s]), dptr(o_gsr[s]), dptr(o_boff),
                         d_items,        p.ngl,          p.ngr,          p.KL,           p.KR,
                         p.d};
    max_pairs = std::max<int64_t>(max_pairs, (int64_t)p.KL * p.KR);
  }
  if (ph) ph[6] += plan_ms_since(t_ph);
  BSG_CUDA(cudaMemcpyAsync(dp, hp, plan_bytes, cudaMemcpyHostToDevice, st));
  BSG_PROFILED(h, BSG_K_PREP, st, (double)ns * max_kl,
               (left_scale_kernel<<<dim3((max_kl + 127) / 128, ns), 128, 0, st>>>(
                   reinterpret_cast<const LeftScaleJob*>(dp + o_lsj))));
  BSG_TRY(fill_spans_dev(h, reinterpret_cast<const FillSpan*>(dp + o_fs), ns, gamma_max, st));
  if (bk.slots == 0) return BSG_OK;
  BSG_PROFILED(h, BSG_K_PREP, st, (double)nb * 32,
               (pad_items_kernel<<<unsigned(((int64_t)nb * 32 + 255) / 256), 256, 0, st>>>(
                   reinterpret_cast<const int32_t*>(dp + o_bend), reinterpret_cast<const int32_t*>(dp + o_bch), nb,
                   d_items)));
  {
    // all sites in one launch: blocks per site so the launch covers ~8 blocks per SM
    const int64_t per_site = std::max<int64_t>(1, ((int64_t)h->num_sms * 8 + ns - 1) / ns);
    const int bx = int(std::max<int64_t>(1, std::min<int64_t>((max_pairs + 255) / 256, per_site)));
    double pairs = 0.0;
    for (int s = 0; s < ns; ++s) pairs += (double)plans[s].KL * plans[s].KR;
    BSG_PROFILED(h, BSG_K_PREP, st, pairs,
                 (site_scatter_kernel<<<dim3(bx, ns), 256, 0, st>>>(reinterpret_cast<const SitePlanDev*>(dp + o_sp))));
  }
  int32_t* d_cbk = reinterpret_cast<int32_t*>(dp + o_cbk);
  if (n_chunks > 0)
    BSG_PROFILED(h, BSG_K_PREP, st, (double)n_chunks,
                 (chunk_bucket_kernel<<<unsigned((n_chunks + 255) / 256), 256, 0, st>>>(
                     reinterpret_cast<const int32_t*>(dp + o_bch), nb, n_chunks, d_cbk)));
  DPArgs a{};
  a.prog = prog_dev(ps);
  a.items = d_items;
  a.bucket_chunk = reinterpret_cast<int32_t*>(dp + o_bch);
  a.chunk_bucket = d_cbk;
  a.bucket_prog = reinterpret_cast<int32_t*>(dp + o_bpr);
  a.bucket_site = reinterpret_cast<int32_t*>(dp + o_bsi);
  a.nb = nb;
  a.counter = reinterpret_cast<unsigned long long*>(dp + o_ctr);
  a.sites = reinterpret_cast<SiteDesc*>(dp + o_desc);
  const int rc = launch_dp<MODE_SITE>(h, precision, a, bk, slot.scratch, st);
  if (ph) {
    ph[5] += plan_ms_since(t_ph);
    ph[7] += std::chrono::duration<double, std::milli>(plan_clk::now() - t_all).count();
  }
  return rc;
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
    BSG_PROFILED(h, BSG_K_PREP, st, (double)B,
                 (target_keys_kernel<<<unsigned((B + 127) / 128), 128, 0, st>>>(targets, n, B, n_len, d_keys, d_err)));
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
  const uint64_t key = (n & 1) ? ~0ull : (n == 0 ? 0ull : uint64_t(n));  // n classes of multiplicity 1
  std::vector<uint64_t> keys(B, key);
  const void* sig = nullptr;
  BSG_TRY(convert_sigma(h, A, (int64_t)B * n * n, precision, h->sigma_ws, &sig, st));
  return run_target_dp(h, MODE_MATRICES, sig, n, nullptr, n, B, nullptr, precision, out, keys, st);
}

// Row tables of one label matrix [rows, m] into `buf` (carved) -- helper for bsg_build_site.
static int one_row_table(bsg_handle_t h, const int8_t* num, int rows, int m, char* base, size_t& off,
                         RowTable& t, int* d_rows, int* d_err, cudaStream_t st) {
  auto align = [](size_t x) { return (x + 255) & ~size_t(255); };
  auto carve = [&](size_t bytes) {
    size_t o = off;
    off = align(off + bytes);
    return base + o;
  };
  t.entries = reinterpret_cast<int32_t*>(carve((size_t)rows * kMaxNnz * 4));
  t.nnz = reinterpret_cast<int32_t*>(carve((size_t)rows * 4));
  t.sum = reinterpret_cast<int32_t*>(carve((size_t)rows * 4));
  t.key = reinterpret_cast<uint64_t*>(carve((size_t)rows * 8));
  t.rowfact = reinterpret_cast<double*>(carve((size_t)rows * 8));
  t.rowfact2 = reinterpret_cast<float2*>(carve((size_t)rows * 8));
  if (!base) return BSG_OK;  // sizing pass
  BSG_CUDA(cudaMemcpyAsync(d_rows, &rows, 4, cudaMemcpyHostToDevice, st));
  dim3 grid((rows + 127) / 128, 1);
  BSG_PROFILED(h, BSG_K_PREP, st, (double)rows,
               (label_rows_kernel<<<grid, 128, 0, st>>>(num, 0, m, d_rows, m, 0, rows, t, d_err)));
  return BSG_OK;
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
  const int KL = kind == BSG_SITE_LAST ? 1 : k_l;
  const int KR = kind == BSG_SITE_FIRST ? 1 : k_r;
  const int ML = kind == BSG_SITE_LAST ? 0 : m_l;
  const int MR = kind == BSG_SITE_FIRST ? 0 : m_r;
  if (KL == 0 || KR == 0) {
    const size_t esz = out_dtype == BSG_OUT_C128 ? 16 : 8;
    BSG_CUDA(cudaMemsetAsync(Gamma, 0, (size_t)chi * chi * d * esz, st));
    return BSG_OK;
  }
  // workspace: row tables, counters, converted Sigma
  const int64_t nsig = (int64_t)(2 * M_r) * (2 * M_r);
  size_t off = 0;
  RowTable lt{}, rt{};
  BSG_TRY(one_row_table(h, nullptr, KL, ML, nullptr, off, lt, nullptr, nullptr, st));
  BSG_TRY(one_row_table(h, nullptr, KR, MR, nullptr, off, rt, nullptr, nullptr, st));
  const size_t o_misc = off;
  off += 256 + 256;
  const size_t o_sig = off;
  off += (size_t)nsig * prec_bytes(precision) + 256;
  BSG_TRY(h->keys.ensure(off));
  char* kb = reinterpret_cast<char*>(h->keys.ptr);
  int* d_rows = reinterpret_cast<int*>(kb + o_misc);
  int* d_err = d_rows + 4;
  int8_t* d_zero = reinterpret_cast<int8_t*>(kb + o_misc + 256);
  BSG_CUDA(cudaMemsetAsync(kb + o_misc, 0, 512, st));
  off = 0;
  BSG_TRY(one_row_table(h, ML ? num_l : d_zero, KL, ML, kb, off, lt, d_rows, d_err, st));
  BSG_TRY(one_row_table(h, MR ? num_r : d_zero, KR, MR, kb, off, rt, d_rows + 1, d_err, st));
  // read keys back to plan
  BSG_TRY(h->host_stage.ensure((size_t)(KL + KR) * 8 + 16));
  uint64_t* hk = reinterpret_cast<uint64_t*>(h->host_stage.ptr);
  int* herr = reinterpret_cast<int*>(hk + KL + KR);
  BSG_CUDA(cudaMemcpyAsync(hk, lt.key, KL * 8, cudaMemcpyDeviceToHost, st));
  BSG_CUDA(cudaMemcpyAsync(hk + KL, rt.key, KR * 8, cudaMemcpyDeviceToHost, st));
  BSG_CUDA(cudaMemcpyAsync(herr, d_err, 4, cudaMemcpyDeviceToHost, st));
  BSG_CUDA(cudaStreamSynchronize(st));
  if (*herr) {
    set_error("bsg_build_site: a label entry is negative, above %d, or a row has more than %d non-zeros",
              kKeyMaxMult, kMaxNnz);
    return BSG_ERR_LIMIT;
  }
  void* sigc = kb + o_sig;
  BSG_TRY(convert_into(h, Sigma, nsig, precision, sigc, st));
  std::vector<SiteInput> in(1);
  in[0].kind = kind;
  in[0].Mr = M_r;
  in[0].sigma = sigc;
  in[0].sigma64 = reinterpret_cast<const double2*>(Sigma);
  in[0].Z = Z;
  in[0].lambda = lambda_l;
  in[0].hkey_l = hk;
  in[0].hkey_r = hk + KL;
  in[0].KL = KL;
  in[0].KR = KR;
  in[0].lt = lt;
  in[0].rt = rt;
  in[0].gamma = Gamma;
  return run_sites(h, in, d, chi, precision, out_dtype, h->slot[0], st);
}

// The whole-MPS build; with gammas_pinned / lambdas_pinned non-null, each
// build group's Gammas are copied to the host as soon as that group's DP is
// done (two copy streams), overlapping the copies with the other groups.
static int build_mps_impl(bsg_handle_t h, const double* sq_cov, int M, int d, int chi, double cut_tol,
                          double site_tol, int precision, int out_dtype, void* const* gammas_host,
                          double* Lambdas, double* res, int8_t* num, double* S, int32_t* kept,
                          void* const* gammas_pinned, double* lambdas_pinned, bsg_stream_t stream) {
  BSG_CHECK_ARG(h, "bsg_build_mps: null handle");
  BSG_CHECK_ARG(sq_cov && gammas_host && Lambdas && res && num && S && kept, "bsg_build_mps: null pointer");
  BSG_CHECK_ARG(M >= 2, "bsg_build_mps: need M >= 2 modes (M=%d)", M);
  BSG_CHECK_ARG(chi >= d && chi <= 2048, "bsg_build_mps: need d <= chi <= 2048");
  BSG_CHECK_ARG(d >= 1 && d <= kKeyMaxMult + 1, "bsg_build_mps: d=%d outside [1, %d]", d, kKeyMaxMult + 1);
  BSG_CHECK_ARG(precision >= 0 && precision <= 2, "bsg_build_mps: bad precision %d", precision);
  BSG_CHECK_ARG(out_dtype == BSG_OUT_C64 || out_dtype == BSG_OUT_C128, "bsg_build_mps: bad out_dtype");
  for (int i = 0; i < M; ++i) BSG_CHECK_ARG(gammas_host[i], "bsg_build_mps: Gamma pointer %d is NULL", i);
  BSG_CUDA(cudaSetDevice(h->device));
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  BSG_TRY(ensure_tables());
  const int nc = M - 1;
  using clk = std::chrono::steady_clock;
  auto ms_since = [](clk::time_point t) { return std::chrono::duration<double, std::milli>(clk::now() - t).count(); };
  // Three groups of cuts and sites, each on its own high-priority stream:
  //   right  cuts [T2, nc)   sites [T2 + 1, M)   (cheap cuts, small Sigma)
  //   left   cuts [0, T1)    sites [0, T1)       (cheap cuts, large-M_r Sigma)
  //   middle cuts [T1, T2)   sites [T1, T2 + 1)  (slow cuts; its sites also read cuts T1 - 1, T2)
  // Site i reads cuts i - 1 and i, so each group's Sigma, planning and DP can
  // start as soon as its own cuts are done: the edge groups' DP (most of the
  // hafnian work sits at both ends of the chain) runs on the SMs the slow
  // middle cuts leave idle.  Every group's DP runs on a low-priority stream
  // in yielding launches (dp_shape): DP blocks leave their SM after a bounded
  // amount of work, so the Williamson, thermal and Sigma kernels of the groups
  // still in flight take SMs within about one quantum instead of waiting for
  // a whole DP launch.  No kernel waits on another; streams are ordered by
  // events only.
  // The group boundaries T1 (left | middle) and T2 (middle | right) come
  // from the tuned shares below; host outputs take a smaller left group (it
  // finishes last, and what it leaves to download after the build is the
  // tail of the end-to-end time).
  int T1 = 0, T2 = nc;
  if (nc >= 6) {
    // built-in shares (measured at M=144): right 33 % / left 33 %, for the
    // device-resident build (82.2 -> 80.0 ms against 25 / 33) and when Gamma
    // goes to the host (e2e 78.2 -> 76.9 ms against right 40 % / left 30 %,
    // which led while the left group's factorisation ended ~10 ms later)
    const int lp = h->tune[BSG_TUNE_LEFT_PCT] ? h->tune[BSG_TUNE_LEFT_PCT] : 33;
    const int rp = h->tune[BSG_TUNE_RIGHT_PCT] ? h->tune[BSG_TUNE_RIGHT_PCT] : 33;
    T1 = std::max(1, nc * lp / 100);
    T2 = nc - std::max(1, nc * rp / 100);
    if (T2 <= T1) T2 = T1 + 1;  // shares above 100 %: a middle group of one cut
  }
  struct Group {
    int c0, c1, s0, s1;
    cudaStream_t stream, dp_stream;
    int slot;
  };
  // order of host planning: right, left, middle (the order their keys arrive)
  std::vector<Group> groups;
  if (T1 > 0) {
    BSG_TRY(h->ensure_aux());
    // DP streams by priority: dp_lo[0] > dp_lo[2] > dp_lo[1]; the order of the
    // groups (right, left, middle) over them is a tuning knob
    cudaStream_t hi = h->dp_lo[0], mid = h->dp_lo[2], lo = h->dp_lo[1];
    cudaStream_t ds[4][3] = {{hi, lo, mid}, {mid, hi, lo}, {lo, hi, mid}, {lo, mid, hi}};
    const int order = h->tune[BSG_TUNE_DP_ORDER];
    groups.push_back(Group{T2, nc, T2 + 1, M, h->grp[0], ds[order][0], 2});
    groups.push_back(Group{0, T1, 0, T1, h->grp[1], ds[order][1], 1});
    groups.push_back(Group{T1, T2, T1, T2 + 1, h->grp[2], ds[order][2], 0});
  } else {
    groups.push_back(Group{0, nc, 0, M, st, st, 0});
  }

  // 1. cut workspace and output clearing
  CutArgs cuts;
  BSG_TRY(cut_prepare(h, sq_cov, M, 1, nc, d, chi, cut_tol, res, num, S, kept, &cuts, st));
  const int ldS = 2 * (M - 1);

  // 2. workspace
  auto align = [](size_t x) { return (x + 255) & ~size_t(255); };
  size_t off = 0;
  auto carve = [&](size_t bytes) {
    size_t o = off;
    off = align(off + bytes);
    return o;
  };
  const size_t rows_cap = (size_t)chi;
  const size_t o_ent = carve((size_t)nc * rows_cap * kMaxNnz * 4), o_nnz = carve((size_t)nc * rows_cap * 4),
               o_sum = carve((size_t)nc * rows_cap * 4), o_key = carve((size_t)nc * rows_cap * 8),
               o_rf = carve((size_t)nc * rows_cap * 8), o_rf2 = carve((size_t)nc * rows_cap * 8);
  const size_t o_empty = carve(kMaxNnz * 4 + 64);  // one empty row (entries, nnz, rowfact, rowfact2)
  const size_t o_above = carve((size_t)nc * 4), o_err = carve(16 * 3), o_Z = carve((size_t)M * 8),
               o_status = carve((size_t)M * 4), o_jobs = carve(sizeof(SigmaJob) * M);
  std::vector<size_t> o_sig(M), o_sigc(M), o_sws(M);
  for (int i = 0; i < M; ++i) {
    const int Mr = i == 0 ? M : M - i;
    o_sig[i] = carve((size_t)(2 * Mr) * (2 * Mr) * 16);
    o_sigc[i] = precision == BSG_PREC_FP64 ? o_sig[i] : carve((size_t)(2 * Mr) * (2 * Mr) * prec_bytes(precision));
    o_sws[i] = carve(sigma_ws_bytes(Mr));
  }
  BSG_TRY(h->mps_ws.ensure(off));
  char* wb = reinterpret_cast<char*>(h->mps_ws.ptr);
  RowTable tab{reinterpret_cast<int32_t*>(wb + o_ent), reinterpret_cast<int32_t*>(wb + o_nnz),
               reinterpret_cast<int32_t*>(wb + o_sum), reinterpret_cast<uint64_t*>(wb + o_key),
               reinterpret_cast<double*>(wb + o_rf), reinterpret_cast<float2*>(wb + o_rf2)};
  RowTable empty{reinterpret_cast<int32_t*>(wb + o_empty), reinterpret_cast<int32_t*>(wb + o_empty + kMaxNnz * 4),
                 nullptr, nullptr, reinterpret_cast<double*>(wb + o_empty + kMaxNnz * 4 + 8),
                 reinterpret_cast<float2*>(wb + o_empty + kMaxNnz * 4 + 16)};
  int32_t* d_above = reinterpret_cast<int32_t*>(wb + o_above);
  int* d_err = reinterpret_cast<int*>(wb + o_err);  // one flag per group (16 bytes apart)
  double* d_Z = reinterpret_cast<double*>(wb + o_Z);
  int* d_status = reinterpret_cast<int*>(wb + o_status);
  // pinned staging: Sigma jobs, cut status, keys, counts, label flags
  BSG_TRY(h->host_stage.ensure(sizeof(SigmaJob) * M + (size_t)nc * 8 + (size_t)nc * (chi * 8 + 8) + 64));
  char* hs = reinterpret_cast<char*>(h->host_stage.ptr);
  int* hcut = reinterpret_cast<int*>(hs + sizeof(SigmaJob) * M);
  uint64_t* hkeys = reinterpret_cast<uint64_t*>(hcut + 2 * (size_t)nc);
  int32_t* hcnt = reinterpret_cast<int32_t*>(hkeys + (size_t)nc * chi);
  int32_t* habove = hcnt + nc;
  int* herr = habove + nc;  // one flag per group
  // the staging buffer's device address (pinned memory is mapped under
  // unified addressing; the small transfers below are kernel stores to it)
  char* hs_dev = nullptr;
  BSG_CUDA(cudaHostGetDevicePointer(reinterpret_cast<void**>(&hs_dev), hs, 0));
  auto to_dev = [&](const void* hp) { return reinterpret_cast<uint32_t*>(hs_dev + (reinterpret_cast<const char*>(hp) - hs)); };
  {
    // empty row: nnz 0, rowfact 1 (and as the FP32 pair (1, 0))
    std::vector<char> e(kMaxNnz * 4 + 64, 0);
    const double one = 1.0;
    const float2 one2 = make_float2(1.f, 0.f);
    std::memcpy(e.data() + kMaxNnz * 4 + 8, &one, 8);
    std::memcpy(e.data() + kMaxNnz * 4 + 16, &one2, 8);
    BSG_CUDA(cudaMemcpyAsync(wb + o_empty, e.data(), e.size(), cudaMemcpyHostToDevice, st));
  }
  BSG_CUDA(cudaMemsetAsync(d_err, 0, 16 * 3, st));
  BSG_CUDA(cudaMemsetAsync(d_status, 0, (size_t)M * 4, st));
  // Sigma jobs of every site
  SigmaJob* jobs = reinterpret_cast<SigmaJob*>(hs);
  for (int i = 0; i < M; ++i) {
    SigmaJob jb{};
    const size_t cut_l = (size_t)i, cut_r = (size_t)(i - 1);
    jb.Mr = i == 0 ? M : M - i;
    if (i == 0) {
      jb.S_l = S;  // cut 0, leading 2(M-1) block
      jb.ld_l = ldS;
      jb.S_r = sq_cov;
      jb.ld_r = 2 * M;
      jb.m_l = M - 1;
      jb.first = 1;
    } else {
      jb.m_l = i == M - 1 ? 0 : M - 1 - i;
      jb.S_l = jb.m_l ? S + cut_l * ldS * ldS : nullptr;
      jb.ld_l = ldS;
      jb.S_r = S + cut_r * ldS * ldS;
      jb.ld_r = ldS;
      jb.first = 0;
    }
    jb.Sigma = reinterpret_cast<double2*>(wb + o_sig[i]);
    jb.Z = d_Z + i;
    jb.ws = reinterpret_cast<double*>(wb + o_sws[i]);
    jb.status = d_status + i;
    jobs[i] = jb;
  }
  auto cut_table = [&](int c) {
    RowTable t = tab;
    const size_t o = (size_t)c * rows_cap;
    t.entries += o * kMaxNnz;
    t.nnz += o;
    t.sum += o;
    t.key += o;
    t.rowfact += o;
    t.rowfact2 += o;
    return t;
  };

  // 3. per group: Williamson, thermal, Lambda + label tables, keys to the
  // host (one event per group), then its Sigma; the middle group's labels and
  // Sigma also read the edge groups' boundary cuts
  const int ng = int(groups.size());
  // events: h->ev[g] = group g's Sigma done (its DP stream waits), h->ev[3] = the left group's
  // Williamson done (BSG_TUNE_DP_HOLD), h->ev[4..9] = final joins, h->ev[15] = the batched
  // build's keys on the host,
  // h->ev[10..12] = Gammas final (pinned copies), h->ev[13..14] = copy-stream joins,
  // h->ev[16 + 3 g + q] (q < 3) = site part q of group g final (host outputs)
  cudaEvent_t ev_keys[3] = {}, ev_done[3] = {};
  // profiling timeline: per group Williamson done, keys on host, Sigma done, DP done
  cudaEvent_t tl0 = nullptr, tl[3][4] = {};
  if (h->prof.on) {
    BSG_CUDA(cudaEventCreate(&tl0));
    BSG_CUDA(cudaEventRecord(tl0, st));
    for (auto& row : tl)
      for (auto& e : row) BSG_CUDA(cudaEventCreate(&e));
  }
  if (ng > 1) {
    BSG_CUDA(cudaEventRecord(h->aux_fork, st));
    for (int g = 0; g < ng; ++g) BSG_CUDA(cudaStreamWaitEvent(groups[g].stream, h->aux_fork, 0));
    for (int g = 0; g < ng; ++g) ev_done[g] = h->ev[g];
  }
  for (int g = 0; g < ng; ++g) {
    const Group& G = groups[g];
    cudaStream_t s2 = G.stream;
    const int nc_g = G.c1 - G.c0;
    BSG_TRY(cut_launch_williamson(h, cuts, G.c0, G.c1, s2));
    if (tl0) BSG_CUDA(cudaEventRecord(tl[g][0], s2));
    if (ng == 3 && g == 1 && h->tune[BSG_TUNE_DP_HOLD]) BSG_CUDA(cudaEventRecord(h->ev[3], s2));
    BSG_TRY(cut_launch_thermal(h, cuts, G.c0, G.c1, s2));
    HostCopyJobs hj{};
    auto add_copy = [&](void* hdst, const void* dsrc, int64_t bytes) {
      hj.dst[hj.n] = to_dev(hdst);
      hj.src[hj.n] = reinterpret_cast<const uint32_t*>(dsrc);
      hj.words[hj.n] = bytes / 4;
      ++hj.n;
    };
    // cut status and Jacobi sweeps (as cut_queue_status)
    add_copy(hcut + G.c0, cuts.status + G.c0, (int64_t)nc_g * 4);
    add_copy(hcut + cuts.n_cuts + G.c0, cuts.sweeps + G.c0, (int64_t)nc_g * 4);
    if (nc_g > 0) {
      BSG_PROFILED(h, BSG_K_PREP, s2, (double)nc_g * chi,
                   (lambda_kernel<<<nc_g, 256, 0, s2>>>(res + (size_t)G.c0 * chi, chi, site_tol,
                                                         Lambdas + (size_t)G.c0 * chi, d_above + G.c0)));
      BSG_PROFILED(h, BSG_K_PREP, s2, (double)nc_g * chi,
                   (label_rows_kernel<<<dim3((chi + 127) / 128, nc_g), 128, 0, s2>>>(
                       num + (size_t)G.c0 * chi * (M - 1), (int64_t)chi * (M - 1), M - 1, kept + G.c0,
                       M - 1 - G.c0, 1, chi, cut_table(G.c0), d_err + 4 * g)));
      add_copy(hkeys + (size_t)G.c0 * chi, tab.key + (size_t)G.c0 * chi, (int64_t)nc_g * chi * 8);
      add_copy(hcnt + G.c0, kept + G.c0, (int64_t)nc_g * 4);
      add_copy(habove + G.c0, d_above + G.c0, (int64_t)nc_g * 4);
    }
    add_copy(herr + g, d_err + 4 * g, 4);
    host_copy_kernel<<<8, 256, 0, s2>>>(hj);
    BSG_CUDA(cudaGetLastError());
    BSG_CUDA(cudaEventCreateWithFlags(&ev_keys[g], cudaEventDisableTiming));
    BSG_CUDA(cudaEventRecord(ev_keys[g], s2));
    if (tl0) BSG_CUDA(cudaEventRecord(tl[g][1], s2));
    if (g == ng - 1 && ng > 1) {
      // the middle sites read the boundary cuts T1 - 1 (left) and T2 (right):
      // their S (Sigma), Lambda and label tables (DP)
      for (int e = 0; e < ng - 1; ++e) BSG_CUDA(cudaStreamWaitEvent(s2, ev_keys[e], 0));
    }
    BSG_TRY(launch_sigma_jobs(h, jobs + G.s0, G.s1 - G.s0, wb + o_jobs + sizeof(SigmaJob) * G.s0, s2,
                              precision == BSG_PREC_SPLIT));
    for (int i = G.s0; i < G.s1; ++i) {
      const int Mr = i == 0 ? M : M - i;
      if (o_sigc[i] != o_sig[i])
        BSG_TRY(convert_into(h, reinterpret_cast<double*>(wb + o_sig[i]), (int64_t)(2 * Mr) * (2 * Mr), precision,
                             wb + o_sigc[i], s2));
    }
    if (tl0) BSG_CUDA(cudaEventRecord(tl[g][2], s2));
  }

  // 4. per group, as its keys arrive: plan its sites and launch their DP
  static const uint64_t zero_key = 0;
  int rc = BSG_OK;
  for (int g = 0; g < ng && rc == BSG_OK; ++g) {
    const Group& G = groups[g];
    {
      auto t_wait = clk::now();
      const cudaError_t e = cudaEventSynchronize(ev_keys[g]);
      if (e != cudaSuccess) {
        set_error("bsg_build_mps: %s", cudaGetErrorString(e));
        rc = BSG_ERR_CUDA;
        break;
      }
      h->prof.add_host(BSG_K_HOST_WAIT, ms_since(t_wait), 0.0);
    }
    // every cut this group's sites read has been checked once its keys are here
    rc = cut_check_status(h, cuts, G.c0, G.c1, hcut);
    if (rc != BSG_OK) break;
    if (herr[g]) {
      set_error("bsg_build_mps: a label row has a multiplicity above %d or more than %d non-zeros", kKeyMaxMult,
                kMaxNnz);
      rc = BSG_ERR_LIMIT;
      break;
    }
    auto t_plan = clk::now();
    std::vector<SiteInput> in(G.s1 - G.s0);
    for (int i = G.s0; i < G.s1 && rc == BSG_OK; ++i) {
      SiteInput& si = in[i - G.s0];
      si.kind = i == 0 ? BSG_SITE_FIRST : i == M - 1 ? BSG_SITE_LAST : BSG_SITE_MIDDLE;
      si.Mr = i == 0 ? M : M - i;
      si.sigma = wb + o_sigc[i];
      si.sigma64 = reinterpret_cast<const double2*>(wb + o_sig[i]);
      si.Z = d_Z + i;
      si.gamma = gammas_host[i];
      if (si.kind != BSG_SITE_LAST) {
        si.lt = cut_table(i);
        si.KL = habove[i];
        si.hkey_l = hkeys + (size_t)i * chi;
        si.lambda = Lambdas + (size_t)i * chi;
      } else {
        si.lt = empty;
        si.KL = 1;
        si.hkey_l = &zero_key;
        si.lambda = nullptr;
      }
      if (si.kind != BSG_SITE_FIRST) {
        si.rt = cut_table(i - 1);
        si.KR = hcnt[i - 1];
        si.hkey_r = hkeys + (size_t)(i - 1) * chi;
      } else {
        si.rt = empty;
        si.KR = 1;
        si.hkey_r = &zero_key;
      }
      if (si.KL == 0 || si.KR == 0) {
        set_error("bsg_build_mps: site %d has an empty bond (no Schmidt weight above the tolerance)", i);
        rc = BSG_ERR_INVALID;
      }
    }
    if (rc != BSG_OK) break;
    if (G.dp_stream != G.stream && rc == BSG_OK) {
      // the group's DP waits for its Sigma (and labels) on the group stream
      cudaError_t e = cudaEventRecord(ev_done[g], G.stream);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(G.dp_stream, ev_done[g], 0);
      // the right group's DP held until the left group's Williamson is done
      if (e == cudaSuccess && ng == 3 && g == 0 && h->tune[BSG_TUNE_DP_HOLD])
        e = cudaStreamWaitEvent(G.dp_stream, h->ev[3], 0);
      if (e != cudaSuccess) {
        set_error("bsg_build_mps: %s", cudaGetErrorString(e));
        rc = BSG_ERR_CUDA;
      }
    }
    // Host outputs: every group's DP runs in four site parts (34 / 34 / 22 /
    // 10 % of its sites, each part with its own plan / item / scratch slot)
    // and each part's Gammas download while the next part computes.  The
    // device-to-host link moves ~190 GB/s, so the 50 ms of downloads of the
    // largest workload must start early to stay off the end of the build; the
    // small last parts keep what is left after the build short.  The
    // device-resident build runs one launch set per group.
    const size_t gb = (size_t)chi * chi * d * (out_dtype == BSG_OUT_C128 ? 16 : 8);
    int copied = G.s0;  // sites of this group whose download is queued
    if (!in.empty() && rc == BSG_OK) {
      const int n_in = int(in.size());
      const bool split_parts = gammas_pinned && ng > 1 && n_in >= 4;
      const int parts = split_parts ? 4 : 1;
      const double cut_at[5] = {0.0, 0.34, 0.68, 0.90, 1.0};
      for (int q = 0; q < parts && rc == BSG_OK; ++q) {
        if (parts == 1) {
          rc = run_sites(h, in, d, chi, precision, out_dtype, h->slot[G.slot], G.dp_stream);
          break;
        }
        const int i0 = q == 0 ? 0 : std::max(q, int(cut_at[q] * n_in + 0.5));
        const int i1 = q + 1 == parts ? n_in : std::max(q + 1, int(cut_at[q + 1] * n_in + 0.5));
        if (i0 >= i1) continue;
        const std::vector<SiteInput> sub(in.begin() + i0, in.begin() + i1);
        rc = run_sites(h, sub, d, chi, precision, out_dtype, h->slot[q == 0 ? G.slot : 2 + 3 * g + q], G.dp_stream);
        if (rc == BSG_OK && q + 1 < parts) {
          cudaStream_t cp = h->copy[g & 1];
          cudaError_t e = cudaEventRecord(h->ev[16 + 3 * g + q], G.dp_stream);
          if (e == cudaSuccess) e = cudaStreamWaitEvent(cp, h->ev[16 + 3 * g + q], 0);
          for (int i = G.s0 + i0; i < G.s0 + i1 && e == cudaSuccess; ++i)
            e = cudaMemcpyAsync(gammas_pinned[i], gammas_host[i], gb, cudaMemcpyDeviceToHost, cp);
          if (e != cudaSuccess) {
            set_error("bsg_build_mps: %s", cudaGetErrorString(e));
            rc = BSG_ERR_CUDA;
          }
          copied = G.s0 + i1;
        }
      }
    }
    if (tl0 && rc == BSG_OK) cudaEventRecord(tl[g][3], G.dp_stream);
    h->prof.add_host(BSG_K_HOST_PLAN, ms_since(t_plan), 0.0);
    if (gammas_pinned && rc == BSG_OK) {
      // the rest of this group's Gammas are final once its DP stream gets here
      cudaStream_t cp = h->copy[g & 1];
      cudaError_t e = cudaEventRecord(h->ev[10 + g], G.dp_stream);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(cp, h->ev[10 + g], 0);
      for (int i = copied; i < G.s1 && e == cudaSuccess; ++i)
        e = cudaMemcpyAsync(gammas_pinned[i], gammas_host[i], gb, cudaMemcpyDeviceToHost, cp);
      if (e != cudaSuccess) {
        set_error("bsg_build_mps: %s", cudaGetErrorString(e));
        rc = BSG_ERR_CUDA;
      }
    }
  }
  // join every stream of every group into st before returning (also on
  // errors: the side streams must be idle before the workspaces are reused)
  if (ng > 1) {
    int e = 4;
    for (int g = 0; g < ng; ++g) {
      cudaEventRecord(h->ev[e], groups[g].stream);
      cudaStreamWaitEvent(st, h->ev[e], 0);
      ++e;
      if (groups[g].dp_stream != groups[g].stream) {
        cudaEventRecord(h->ev[e], groups[g].dp_stream);
        cudaStreamWaitEvent(st, h->ev[e], 0);
        ++e;
      }
    }
  }
  if (gammas_pinned && h->copy[0]) {
    for (int q = 0; q < 2; ++q) {
      cudaEventRecord(h->ev[13 + q], h->copy[q]);
      cudaStreamWaitEvent(st, h->ev[13 + q], 0);
    }
  }
  for (int g = 0; g < ng; ++g)
    if (ev_keys[g]) cudaEventDestroy(ev_keys[g]);
  if (rc != BSG_OK) {
    cudaStreamSynchronize(st);
    return rc;
  }
  if (gammas_pinned && ng == 1) {  // single group: copy after the build
    const size_t gb = (size_t)chi * chi * d * (out_dtype == BSG_OUT_C128 ? 16 : 8);
    for (int i = 0; i < M; ++i)
      BSG_CUDA(cudaMemcpyAsync(gammas_pinned[i], gammas_host[i], gb, cudaMemcpyDeviceToHost, st));
  }
  if (lambdas_pinned)
    BSG_CUDA(cudaMemcpyAsync(lambdas_pinned, Lambdas, (size_t)nc * chi * 8, cudaMemcpyDeviceToHost, st));
  // Sigma status (singular A) -- read after the DP so the check costs no extra wait
  std::vector<int> sst(M);
  BSG_CUDA(cudaMemcpyAsync(sst.data(), d_status, (size_t)M * 4, cudaMemcpyDeviceToHost, st));
  auto t_fin = clk::now();
  BSG_CUDA(cudaStreamSynchronize(st));
  h->prof.add_host(BSG_K_HOST_WAIT, ms_since(t_fin), 0.0);
  BSG_TRY(cut_read_phases(h, cuts, st));
  if (tl0) {
    h->prof.timeline.assign(12, -1.0);
    for (int g = 0; g < ng; ++g)
      for (int k = 0; k < 4; ++k) {
        float ms = -1.f;
        if (cudaEventElapsedTime(&ms, tl0, tl[g][k]) == cudaSuccess) h->prof.timeline[(size_t)g * 4 + k] = ms;
      }
    cudaEventDestroy(tl0);
    for (auto& row : tl)
      for (auto& e : row) cudaEventDestroy(e);
  }
  for (int i = 0; i < M; ++i)
    if (sst[i]) {
      set_error("bsg_build_mps: site %d: the Gaussian unitary's A block is singular", i);
      return BSG_ERR_NO_CONVERGE;
    }
  return BSG_OK;
}

// The whole MPS of n independent instances (each its own M, d, chi) with one
// launch per phase for all of them: the Williamson and top-chi kernels over
// every cut of every instance (cut_launch_batch), the Sigma phases over every
// site of every instance (launch_sigma_jobs), one host wait, then one item
// scatter and one set of DP launches over the items of every site of every
// instance (run_sites with per-site d and chi).  Per-instance outputs as in
// bsg_build_mps; gammas holds the instances' site pointers back to back.
// With cuts_given the cut data (res, num, S, kept) are inputs -- the kron
// step's files -- and only sites [lo[i], hi[i]) of instance i are built
// (their Lambda rows and label tables from the cuts they read).
static int build_mps_batch_impl(bsg_handle_t h, int n, const double* const* sq, const int* Ms, const int* ds,
                                const int* chis, double cut_tol, double site_tol, int precision, int out_dtype,
                                void* const* gammas, double* const* Lambdas, double* const* res,
                                int8_t* const* num, double* const* S, int32_t* const* kept, cudaStream_t st,
                                bool cuts_given = false, const int* lo = nullptr, const int* hi = nullptr) {
  using clk = std::chrono::steady_clock;
  auto ms_since = [](clk::time_point t0) {
    return std::chrono::duration<double, std::milli>(clk::now() - t0).count();
  };
  BSG_CHECK_ARG(n >= 1, "bsg_build_mps_batch: need at least one instance");
  BSG_CHECK_ARG(sq && Ms && ds && chis && gammas && Lambdas && res && num && S && kept,
                "bsg_build_mps_batch: null pointer");
  BSG_CHECK_ARG(precision >= 0 && precision <= 2, "bsg_build_mps_batch: bad precision %d", precision);
  BSG_CHECK_ARG(out_dtype == BSG_OUT_C64 || out_dtype == BSG_OUT_C128, "bsg_build_mps_batch: bad out_dtype");
  std::vector<int> site0(n + 1, 0), slo(n), shi(n), clo(n), chi_(n), cut0(n + 1, 0);
  std::vector<int64_t> key0(n + 1, 0);
  int chi_max = 0;
  for (int i = 0; i < n; ++i) {
    const int M = Ms[i], d = ds[i], chi = chis[i];
    BSG_CHECK_ARG(sq[i] && Lambdas[i] && res[i] && num[i] && S[i] && kept[i],
                  "bsg_build_mps_batch: instance %d: null pointer", i);
    BSG_CHECK_ARG(M >= 2, "bsg_build_mps_batch: instance %d: need M >= 2 modes (M=%d)", i, M);
    BSG_CHECK_ARG(chi >= d && chi <= 2048, "bsg_build_mps_batch: instance %d: need d <= chi <= 2048", i);
    BSG_CHECK_ARG(d >= 1 && d <= kKeyMaxMult + 1, "bsg_build_mps_batch: instance %d: d=%d outside [1, %d]", i, d,
                  kKeyMaxMult + 1);
    slo[i] = lo ? lo[i] : 0;
    shi[i] = hi ? hi[i] : M;
    BSG_CHECK_ARG(0 <= slo[i] && slo[i] < shi[i] && shi[i] <= M, "bsg_build_mps_batch: instance %d: sites [%d, %d) "
                  "outside [0, %d)", i, slo[i], shi[i], M);
    // cuts the sites read: [lo - 1, hi) within [0, M - 1)
    clo[i] = std::max(0, slo[i] - 1);
    chi_[i] = std::min(shi[i], M - 1);
    site0[i + 1] = site0[i] + (shi[i] - slo[i]);
    cut0[i + 1] = cut0[i] + (M - 1);
    key0[i + 1] = key0[i] + (int64_t)(M - 1) * chi;
    chi_max = std::max(chi_max, chi);
  }
  const int ns = site0[n], total_cuts = cut0[n];
  for (int s = 0; s < ns; ++s) BSG_CHECK_ARG(gammas[s], "bsg_build_mps_batch: Gamma pointer %d is NULL", s);
  BSG_CUDA(cudaSetDevice(h->device));
  BSG_TRY(ensure_tables());
  auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
  size_t off = 0;
  auto carve = [&](size_t bytes) {
    size_t o = off;
    off = al(off + bytes);
    return o;
  };
  struct Inst {
    size_t o_cut, o_ent, o_nnz, o_sum, o_rf, o_rf2, o_Z;
  };
  std::vector<Inst> I(n);
  std::vector<size_t> o_sig(ns), o_sigc(ns), o_sws(ns);
  size_t hoff = 0;
  auto hcarve = [&](size_t bytes) {
    size_t o = hoff;
    hoff = (hoff + bytes + 63) & ~size_t(63);
    return o;
  };
  for (int i = 0; i < n; ++i) {
    const int M = Ms[i], chi = chis[i], nc = M - 1;
    Inst& t = I[i];
    t.o_cut = cuts_given ? carve(0) : carve(cut_ws_bytes(M, 1, nc, chi));
    t.o_ent = carve((size_t)nc * chi * kMaxNnz * 4);
    t.o_nnz = carve((size_t)nc * chi * 4);
    t.o_sum = carve((size_t)nc * chi * 4);
    t.o_rf = carve((size_t)nc * chi * 8);
    t.o_rf2 = carve((size_t)nc * chi * 8);
    t.o_Z = carve((size_t)M * 8);
    for (int j = slo[i]; j < shi[i]; ++j) {
      const int s = site0[i] + j - slo[i], Mr = j == 0 ? M : M - j;
      o_sig[s] = carve((size_t)(2 * Mr) * (2 * Mr) * 16);
      o_sigc[s] = precision == BSG_PREC_FP64 ? o_sig[s] : carve((size_t)(2 * Mr) * (2 * Mr) * prec_bytes(precision));
      o_sws[s] = carve(sigma_ws_bytes(Mr));
    }
  }
  // Host-bound region, one device->host copy for all instances:
  // [label error per instance | Sigma status per site | rows above tol per cut]  cleared to 0,
  // [Williamson status per cut, then its sweeps, per instance]                   cleared to -1,
  // [kept-row count per cut | row keys per (cut, row)].
  const size_t hb_err = 0, hb_sst = hb_err + 4 * (size_t)n, hb_above = hb_sst + 4 * (size_t)ns;
  const size_t hb_cst = hb_above + 4 * (size_t)total_cuts, hb_cnt = hb_cst + 8 * (size_t)total_cuts;
  const size_t hb_keys = (hb_cnt + 4 * (size_t)total_cuts + 7) & ~size_t(7);
  const size_t hb_bytes = hb_keys + 8 * (size_t)key0[n];
  const size_t o_hb = carve(hb_bytes), h_hb = hcarve(hb_bytes);
  const size_t o_empty = carve(kMaxNnz * 4 + 64), h_empty = hcarve(kMaxNnz * 4 + 64);
  const size_t cargs_bytes = al(sizeof(CutArgs) * n) + al(sizeof(int2) * total_cuts);
  const size_t o_cargs = carve(cargs_bytes), h_cargs = hcarve(cargs_bytes);
  const int max_spans = 6 * n + 2;
  const size_t o_fill = carve(sizeof(FillSpan) * max_spans), h_fill = hcarve(sizeof(FillSpan) * max_spans);
  const size_t rows_bytes = al(sizeof(CutRowsJob) * n) + sizeof(int2) * (size_t)total_cuts;
  const size_t o_rows = carve(rows_bytes), h_rows = hcarve(rows_bytes);
  const size_t o_jobs = carve(sizeof(SigmaJob) * ns), h_jobs = hcarve(sizeof(SigmaJob) * ns);
  const size_t o_conv = carve(sizeof(ConvJob) * ns), h_conv = hcarve(sizeof(ConvJob) * ns);
  BSG_TRY(h->mps_ws.ensure(off));
  BSG_TRY(h->host_stage.ensure(hoff));
  char* wb = reinterpret_cast<char*>(h->mps_ws.ptr);
  char* hs = reinterpret_cast<char*>(h->host_stage.ptr);
  char* hb = wb + o_hb;   // device
  char* hbh = hs + h_hb;  // its host copy
  auto table = [&](int i, int c) {
    const Inst& t = I[i];
    const size_t o = (size_t)c * chis[i];
    return RowTable{reinterpret_cast<int32_t*>(wb + t.o_ent) + o * kMaxNnz, reinterpret_cast<int32_t*>(wb + t.o_nnz) + o,
                    reinterpret_cast<int32_t*>(wb + t.o_sum) + o,
                    reinterpret_cast<uint64_t*>(hb + hb_keys) + key0[i] + o,
                    reinterpret_cast<double*>(wb + t.o_rf) + o, reinterpret_cast<float2*>(wb + t.o_rf2) + o};
  };
  RowTable empty{reinterpret_cast<int32_t*>(wb + o_empty), reinterpret_cast<int32_t*>(wb + o_empty + kMaxNnz * 4),
                 nullptr, nullptr, reinterpret_cast<double*>(wb + o_empty + kMaxNnz * 4 + 8),
                 reinterpret_cast<float2*>(wb + o_empty + kMaxNnz * 4 + 16)};
  {
    // empty row: nnz 0, rowfact 1 (and as the FP32 pair (1, 0))
    char* e = hs + h_empty;
    std::memset(e, 0, kMaxNnz * 4 + 64);
    const double one = 1.0;
    const float2 one2 = make_float2(1.f, 0.f);
    std::memcpy(e + kMaxNnz * 4 + 8, &one, 8);
    std::memcpy(e + kMaxNnz * 4 + 16, &one2, 8);
    BSG_CUDA(cudaMemcpyAsync(wb + o_empty, e, kMaxNnz * 4 + 64, cudaMemcpyHostToDevice, st));
  }
  // 1. every instance's output and status clears in one launch, then every
  //    cut of every instance: Williamson and top-chi, one launch each
  std::vector<CutArgs> cargs(n);
  std::vector<FillSpan> spans;
  spans.reserve(max_spans);
  spans.push_back(FillSpan{hb, (int64_t)hb_cst, 0});
  spans.push_back(FillSpan{hb + hb_cst, (int64_t)(8 * (size_t)total_cuts), 0xff});
  if (!cuts_given)
    for (int i = 0; i < n; ++i) {
      const int M = Ms[i], nc = M - 1;
      BSG_TRY(cut_prepare_at(h, wb + I[i].o_cut, sq[i], M, 1, nc, ds[i], chis[i], cut_tol, res[i], num[i], S[i],
                             kept[i], &cargs[i], st, &spans));
      // the cut status lands in the host-bound region
      cargs[i].status = reinterpret_cast<int*>(hb + hb_cst) + 2 * (size_t)cut0[i];
      cargs[i].sweeps = cargs[i].status + nc;
    }
  BSG_TRY(fill_spans(h, spans.data(), int(spans.size()), wb + o_fill, hs + h_fill, st));
  if (!cuts_given) BSG_TRY(cut_launch_batch(h, cargs.data(), n, wb + o_cargs, hs + h_cargs, st));
  // 2. Lambda, label rows and keys of the cuts the sites read, one launch,
  //    then the host-bound region in one copy
  {
    CutRowsJob* rj = reinterpret_cast<CutRowsJob*>(hs + h_rows);
    int2* rmap = reinterpret_cast<int2*>(hs + h_rows + al(sizeof(CutRowsJob) * n));
    int n_rows = 0;
    double work = 0.0;
    for (int i = 0; i < n; ++i) {
      const int M = Ms[i], chi = chis[i], c0 = clo[i], nci = chi_[i] - clo[i];
      CutRowsJob jb{};
      jb.num = num[i] + (size_t)c0 * chi * (M - 1);
      jb.kept = kept[i] + c0;
      jb.res = res[i] + (size_t)c0 * chi;
      jb.lambda = Lambdas[i] + (size_t)c0 * chi;
      jb.t = table(i, c0);
      jb.above = reinterpret_cast<int32_t*>(hb + hb_above) + cut0[i] + c0;
      jb.cnt = reinterpret_cast<int32_t*>(hb + hb_cnt) + cut0[i] + c0;
      jb.err = reinterpret_cast<int*>(hb + hb_err) + i;
      jb.tol = site_tol;
      jb.chi = chi;
      jb.ld = M - 1;
      jb.m0 = M - 1 - c0;
      rj[i] = jb;
      for (int c = 0; c < nci; ++c) rmap[n_rows++] = make_int2(i, c);
      work += (double)nci * chi;
    }
    if (n_rows > 0) {
      BSG_CUDA(cudaMemcpyAsync(wb + o_rows, hs + h_rows, al(sizeof(CutRowsJob) * n) + sizeof(int2) * n_rows,
                               cudaMemcpyHostToDevice, st));
      BSG_PROFILED(h, BSG_K_PREP, st, work,
                   (cut_rows_batch_kernel<<<dim3((chi_max + 127) / 128, n_rows), 128, 0, st>>>(
                       reinterpret_cast<const CutRowsJob*>(wb + o_rows),
                       reinterpret_cast<const int2*>(wb + o_rows + al(sizeof(CutRowsJob) * n)))));
    }
    BSG_CUDA(cudaMemcpyAsync(hbh, hb, hb_bytes, cudaMemcpyDeviceToHost, st));
  }
  // the host plans as soon as the keys are here, while the GPU builds Sigma
  BSG_TRY(h->ensure_aux());
  BSG_CUDA(cudaEventRecord(h->ev[15], st));
  // 3. Sigma of every site of every instance in one set of launches
  SigmaJob* jobs = reinterpret_cast<SigmaJob*>(hs + h_jobs);
  for (int i = 0; i < n; ++i) {
    const int M = Ms[i], ldS = 2 * (M - 1);
    for (int j = slo[i]; j < shi[i]; ++j) {
      const int s = site0[i] + j - slo[i];
      SigmaJob jb{};
      jb.Mr = j == 0 ? M : M - j;
      if (j == 0) {
        jb.S_l = S[i];
        jb.ld_l = ldS;
        jb.S_r = sq[i];
        jb.ld_r = 2 * M;
        jb.m_l = M - 1;
        jb.first = 1;
      } else {
        jb.m_l = j == M - 1 ? 0 : M - 1 - j;
        jb.S_l = jb.m_l ? S[i] + (size_t)j * ldS * ldS : nullptr;
        jb.ld_l = ldS;
        jb.S_r = S[i] + (size_t)(j - 1) * ldS * ldS;
        jb.ld_r = ldS;
        jb.first = 0;
      }
      jb.Sigma = reinterpret_cast<double2*>(wb + o_sig[s]);
      jb.Z = reinterpret_cast<double*>(wb + I[i].o_Z) + j;
      jb.ws = reinterpret_cast<double*>(wb + o_sws[s]);
      jb.status = reinterpret_cast<int*>(hb + hb_sst) + s;
      jobs[s] = jb;
    }
  }
  BSG_TRY(launch_sigma_jobs(h, jobs, ns, wb + o_jobs, st, precision == BSG_PREC_SPLIT));
  // every site's Sigma into the DP's storage type, one launch
  ConvJob* conv = reinterpret_cast<ConvJob*>(hs + h_conv);
  int n_conv = 0;
  for (int i = 0; i < n; ++i)
    for (int j = slo[i]; j < shi[i]; ++j) {
      const int s = site0[i] + j - slo[i], Mr = j == 0 ? Ms[i] : Ms[i] - j;
      if (o_sigc[s] != o_sig[s])
        conv[n_conv++] = ConvJob{reinterpret_cast<const double2*>(wb + o_sig[s]), wb + o_sigc[s],
                                 (int64_t)(2 * Mr) * (2 * Mr)};
    }
  BSG_TRY(convert_many(h, conv, n_conv, wb + o_conv, precision, st));
  // 4. one host wait: every instance's cut status, row counts and keys (the
  // Sigma launches keep running; the DP launches queue behind them on st)
  {
    auto t_wait = clk::now();
    BSG_CUDA(cudaEventSynchronize(h->ev[15]));
    h->prof.add_host(BSG_K_HOST_WAIT, ms_since(t_wait), 0.0);
  }
  auto t_plan = clk::now();
  static const uint64_t zero_key = 0;
  std::vector<SiteInput> in(ns);
  for (int i = 0; i < n; ++i) {
    const int M = Ms[i], chi = chis[i], nc = M - 1;
    if (!cuts_given)
      BSG_TRY(cut_check_status(h, cargs[i], 0, nc, reinterpret_cast<const int*>(hbh + hb_cst) + 2 * (size_t)cut0[i]));
    if (reinterpret_cast<const int*>(hbh + hb_err)[i]) {
      set_error("bsg_build_mps_batch: instance %d: a label row has a multiplicity above %d or more than %d non-zeros",
                i, kKeyMaxMult, kMaxNnz);
      return BSG_ERR_LIMIT;
    }
    const uint64_t* hkeys = reinterpret_cast<const uint64_t*>(hbh + hb_keys) + key0[i];
    const int32_t* hcnt = reinterpret_cast<const int32_t*>(hbh + hb_cnt) + cut0[i];
    const int32_t* habove = reinterpret_cast<const int32_t*>(hbh + hb_above) + cut0[i];
    for (int j = slo[i]; j < shi[i]; ++j) {
      const int s = site0[i] + j - slo[i];
      SiteInput& si = in[s];
      si.kind = j == 0 ? BSG_SITE_FIRST : j == M - 1 ? BSG_SITE_LAST : BSG_SITE_MIDDLE;
      si.Mr = j == 0 ? M : M - j;
      si.sigma = wb + o_sigc[s];
      si.sigma64 = reinterpret_cast<const double2*>(wb + o_sig[s]);
      si.Z = reinterpret_cast<const double*>(wb + I[i].o_Z) + j;
      si.gamma = gammas[s];
      si.d = ds[i];
      si.chi = chi;
      if (si.kind != BSG_SITE_LAST) {
        si.lt = table(i, j);
        si.KL = habove[j];
        si.hkey_l = hkeys + (size_t)j * chi;
        si.lambda = Lambdas[i] + (size_t)j * chi;
      } else {
        si.lt = empty;
        si.KL = 1;
        si.hkey_l = &zero_key;
        si.lambda = nullptr;
      }
      if (si.kind != BSG_SITE_FIRST) {
        si.rt = table(i, j - 1);
        si.KR = hcnt[j - 1];
        si.hkey_r = hkeys + (size_t)(j - 1) * chi;
      } else {
        si.rt = empty;
        si.KR = 1;
        si.hkey_r = &zero_key;
      }
      if (si.KL == 0 || si.KR == 0) {
        set_error("bsg_build_mps_batch: instance %d site %d has an empty bond", i, j);
        return BSG_ERR_INVALID;
      }
    }
  }
  // 5. the items of every site of every instance: one scatter, one DP launch set
  BSG_TRY(run_sites(h, in, ds[0], chis[0], precision, out_dtype, h->slot[0], st));
  h->prof.add_host(BSG_K_HOST_PLAN, ms_since(t_plan), 0.0);
  // Sigma status (singular A), read after the DP
  const int32_t* sst = reinterpret_cast<const int32_t*>(hbh + hb_sst);
  BSG_CUDA(cudaMemcpyAsync(hbh + hb_sst, hb + hb_sst, 4 * (size_t)ns, cudaMemcpyDeviceToHost, st));
  {
    auto t_fin = clk::now();
    BSG_CUDA(cudaStreamSynchronize(st));
    h->prof.add_host(BSG_K_HOST_WAIT, ms_since(t_fin), 0.0);
  }
  for (int i = 0; i < n; ++i)
    for (int j = slo[i]; j < shi[i]; ++j)
      if (sst[site0[i] + j - slo[i]]) {
        set_error("bsg_build_mps_batch: instance %d site %d: the Gaussian unitary's A block is singular", i, j);
        return BSG_ERR_NO_CONVERGE;
      }
  return BSG_OK;
}

extern "C" int bsg_build_mps(bsg_handle_t h, const double* sq_cov, int M, int d, int chi, double cut_tol,
                             double site_tol, int precision, int out_dtype, void* const* gammas_host,
                             double* Lambdas, double* res, int8_t* num, double* S, int32_t* kept,
                             bsg_stream_t stream) {
  return build_mps_impl(h, sq_cov, M, d, chi, cut_tol, site_tol, precision, out_dtype, gammas_host, Lambdas, res,
                        num, S, kept, nullptr, nullptr, stream);
}

extern "C" int bsg_build_mps_batch(bsg_handle_t h, int n, const double* const* sq_covs, const int* M, const int* d,
                                   const int* chi, double cut_tol, double site_tol, int precision, int out_dtype,
                                   void* const* gammas, double* const* Lambdas, double* const* res,
                                   int8_t* const* num, double* const* S, int32_t* const* kept, bsg_stream_t stream) {
  BSG_CHECK_ARG(h, "bsg_build_mps_batch: null handle");
  return build_mps_batch_impl(h, n, sq_covs, M, d, chi, cut_tol, site_tol, precision, out_dtype, gammas, Lambdas,
                              res, num, S, kept, reinterpret_cast<cudaStream_t>(stream));
}

extern "C" int bsg_build_sites(bsg_handle_t h, const double* sq_cov, int M, int d, int chi, double site_tol,
                               int precision, int out_dtype, int s0, int s1, const double* res, const int8_t* num,
                               const double* S, const int32_t* kept, void* const* gammas, double* Lambdas,
                               bsg_stream_t stream) {
  BSG_CHECK_ARG(h, "bsg_build_sites: null handle");
  const double* sq[1] = {sq_cov};
  double* lam[1] = {Lambdas};
  double* rs[1] = {const_cast<double*>(res)};
  int8_t* nm[1] = {const_cast<int8_t*>(num)};
  double* Ss[1] = {const_cast<double*>(S)};
  int32_t* kp[1] = {const_cast<int32_t*>(kept)};
  return build_mps_batch_impl(h, 1, sq, &M, &d, &chi, 0.0, site_tol, precision, out_dtype, gammas, lam, rs, nm, Ss,
                              kp, reinterpret_cast<cudaStream_t>(stream), true, &s0, &s1);
}

extern "C" int bsg_build_mps_to_host(bsg_handle_t h, const double* sq_cov, int M, int d, int chi, double cut_tol,
                                     double site_tol, int precision, int out_dtype, void* const* gammas_dev,
                                     void* const* gammas_pinned, double* Lambdas, double* lambdas_pinned,
                                     double* res, int8_t* num, double* S, int32_t* kept, bsg_stream_t stream) {
  BSG_CHECK_ARG(gammas_pinned && lambdas_pinned, "bsg_build_mps_to_host: null host pointer");
  for (int i = 0; i < M; ++i) BSG_CHECK_ARG(gammas_pinned[i], "bsg_build_mps_to_host: host Gamma %d is NULL", i);
  return build_mps_impl(h, sq_cov, M, d, chi, cut_tol, site_tol, precision, out_dtype, gammas_dev, Lambdas, res,
                        num, S, kept, gammas_pinned, lambdas_pinned, stream);
}
