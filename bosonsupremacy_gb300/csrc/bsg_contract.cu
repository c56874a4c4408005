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
// Rows of a level are grouped by n on the host so every GEMM writes a
// contiguous block.  The GEMM gathers its A rows by parent index and applies
// Lambda on the fly.
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
  if (p >= P) return;
  const typename Cx<R>::T* l = L + (int64_t)li[p] * chi;
  const typename Cx<R>::T* r = Rt + (int64_t)ri[p] * chi;
  double sr = 0.0, si = 0.0;
  for (int a = lane; a < chi; a += 32) {
    const double w = lam ? lam[a] : 1.0;
    const double lx = double(l[a].x) * w, ly = double(l[a].y) * w;
    sr += lx * double(r[a].x) - ly * double(r[a].y);
    si += lx * double(r[a].y) + ly * double(r[a].x);
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

__global__ void build_bt_kernel(const float2* __restrict__ G, int n, int chi, int d, int left, float* __restrict__ Bhi,
                                float* __restrict__ Blo) {
  const int64_t K2 = 2 * (int64_t)chi;
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

// ---- host planning: distinct prefixes per level grouped by photon number ----
struct SidePlan {
  std::vector<int> sites;                     // site of each level (left: 0..m, right: M-1..m+1)
  std::vector<std::vector<int32_t>> parent;   // per level: parent row (level-1) of each row
  std::vector<std::vector<int32_t>> nval;     // per level: photon number of each row
  std::vector<std::vector<int32_t>> group;    // per level: first row of each photon number (d+1 entries)
  std::vector<int32_t> final_row;             // per pattern: row at the last level
};

static void plan_side(const int32_t* pat, int64_t P, int M, int d, const std::vector<int>& sites, SidePlan& sp) {
  sp.sites = sites;
  const int nl = int(sites.size());
  sp.parent.assign(nl, {});
  sp.nval.assign(nl, {});
  sp.group.assign(nl, {});
  std::vector<int32_t> cur(P, 0), nxt(P);
  int64_t prev_rows = 1;
  for (int l = 0; l < nl; ++l) {
    const int s = sites[l];
    // key = parent * d + n -> first-appearance id, then regroup by n
    std::vector<int32_t> id((size_t)prev_rows * d, -1);
    std::vector<int32_t> par, nv;
    for (int64_t p = 0; p < P; ++p) {
      const int n = pat[p * M + s];
      const int64_t key = (int64_t)cur[p] * d + n;
      if (id[key] < 0) {
        id[key] = int32_t(par.size());
        par.push_back(cur[p]);
        nv.push_back(n);
      }
      nxt[p] = id[key];
    }
    const int rows = int(par.size());
    std::vector<int32_t> start(d + 1, 0);
    for (int r = 0; r < rows; ++r) start[nv[r] + 1]++;
    for (int n = 0; n < d; ++n) start[n + 1] += start[n];
    std::vector<int32_t> pos(start.begin(), start.end() - 1), remap(rows);
    for (int r = 0; r < rows; ++r) remap[r] = pos[nv[r]]++;
    std::vector<int32_t> par2(rows), nv2(rows);
    for (int r = 0; r < rows; ++r) {
      par2[remap[r]] = par[r];
      nv2[remap[r]] = nv[r];
    }
    for (int64_t p = 0; p < P; ++p) cur[p] = remap[nxt[p]];
    sp.parent[l].swap(par2);
    sp.nval[l].swap(nv2);
    sp.group[l].swap(start);
    prev_rows = rows;
  }
  sp.final_row = cur;
}

template <class R>
static int run_contraction(bsg_handle_t h, const void* const* Gd, const double* lam, int M, int chi, int d,
                           const SidePlan& left, const SidePlan& right, int64_t P, double* amp, bool umma,
                           cudaStream_t st) {
  using T = typename Cx<R>::T;
  // device memory: two env buffers per side (ping-pong) + index arrays
  auto rows_of = [](const SidePlan& s, int l) { return (int64_t)s.parent[l].size(); };
  int64_t max_rows = 1;
  for (int l = 0; l < (int)left.sites.size(); ++l) max_rows = std::max(max_rows, rows_of(left, l));
  for (int l = 0; l < (int)right.sites.size(); ++l) max_rows = std::max(max_rows, rows_of(right, l));
  int64_t idx_total = 2 * P;
  for (auto* sp : {&left, &right})
    for (size_t l = 0; l < sp->sites.size(); ++l) idx_total += 2 * (int64_t)sp->parent[l].size();
  auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
  const size_t env_bytes = al((size_t)max_rows * chi * sizeof(T));
  const size_t a_bytes = umma ? al((size_t)max_rows * 2 * chi * 4) : 0;
  const size_t b_bytes = umma ? al((size_t)4 * chi * chi * 4) : 0;
  const size_t need = 4 * env_bytes + al((size_t)idx_total * 4) + 2 * a_bytes + 2 * b_bytes + 256;
  BSG_TRY(h->contract_ws.ensure(need));
  char* base = reinterpret_cast<char*>(h->contract_ws.ptr);
  char* sp_base = base + 4 * env_bytes + al((size_t)idx_total * 4);
  float* Ahi = reinterpret_cast<float*>(sp_base);
  float* Alo = reinterpret_cast<float*>(sp_base + a_bytes);
  float* Bhi = reinterpret_cast<float*>(sp_base + 2 * a_bytes);
  float* Blo = reinterpret_cast<float*>(sp_base + 2 * a_bytes + b_bytes);
  int* d_err = reinterpret_cast<int*>(sp_base + 2 * a_bytes + 2 * b_bytes);
  if (umma) BSG_CUDA(cudaMemsetAsync(d_err, 0, 4, st));
  T* E[4] = {reinterpret_cast<T*>(base), reinterpret_cast<T*>(base + env_bytes),
             reinterpret_cast<T*>(base + 2 * env_bytes), reinterpret_cast<T*>(base + 3 * env_bytes)};
  int32_t* idx = reinterpret_cast<int32_t*>(base + 4 * env_bytes);
  // stage all index arrays in pinned memory, one copy
  BSG_TRY(h->host_stage2.ensure((size_t)idx_total * 4 + 64));
  int32_t* hidx = reinterpret_cast<int32_t*>(h->host_stage2.ptr);
  int64_t off = 0;
  struct LevelIdx {
    int64_t parent_off, nval_off;
  };
  std::vector<LevelIdx> li_l(left.sites.size()), li_r(right.sites.size());
  auto put = [&](const SidePlan& sp, std::vector<LevelIdx>& li) {
    for (size_t l = 0; l < sp.sites.size(); ++l) {
      li[l].parent_off = off;
      std::memcpy(hidx + off, sp.parent[l].data(), sp.parent[l].size() * 4);
      off += (int64_t)sp.parent[l].size();
      li[l].nval_off = off;
      std::memcpy(hidx + off, sp.nval[l].data(), sp.nval[l].size() * 4);
      off += (int64_t)sp.nval[l].size();
    }
  };
  put(left, li_l);
  put(right, li_r);
  const int64_t fin_l = off;
  std::memcpy(hidx + off, left.final_row.data(), (size_t)P * 4);
  off += P;
  const int64_t fin_r = off;
  std::memcpy(hidx + off, right.final_row.data(), (size_t)P * 4);
  off += P;
  BSG_CUDA(cudaMemcpyAsync(idx, hidx, (size_t)off * 4, cudaMemcpyHostToDevice, st));

  double flops = 0.0;
  auto side = [&](const SidePlan& sp, const std::vector<LevelIdx>& li, T* e0, T* e1, bool is_left) -> T* {
    T* prev = e0;
    T* curb = e1;
    // level 0: row 0 of Gamma_0 (left) or column 0 of Gamma_{M-1} (right)
    {
      const int s = sp.sites[0];
      const T* G = reinterpret_cast<const T*>(Gd[s]);
      const int64_t rows = (int64_t)sp.parent[0].size();
      // left: Gamma_0[0, a, n] at a*d + n ; right: Gamma_{M-1}[a, 0, n] at a*chi*d + n
      const int64_t stride = is_left ? d : (int64_t)chi * d;
      const int64_t tot = rows * chi;
      env_init_kernel<R><<<unsigned((tot + 255) / 256), 256, 0, st>>>(G, stride, idx + li[0].nval_off, (int)rows, chi,
                                                                         prev);
    }
    for (size_t l = 1; l < sp.sites.size(); ++l) {
      const int s = sp.sites[l];
      const T* G = reinterpret_cast<const T*>(Gd[s]);
      // left uses Lambda_{s-1}, right uses Lambda_s
      const double* lm = lam + (size_t)(is_left ? s - 1 : s) * chi;
      for (int n = 0; n < d; ++n) {
        const int r0 = sp.group[l][n], r1 = sp.group[l][n + 1];
        if (r1 <= r0) continue;
        if constexpr (std::is_same<R, float>::value) {
          if (umma) {
            const int64_t K2 = 2 * (int64_t)chi, rows = r1 - r0;
            build_bt_kernel<<<unsigned((K2 * K2 + 255) / 256), 256, 0, st>>>(
                reinterpret_cast<const float2*>(G), n, chi, d, is_left ? 1 : 0, Bhi, Blo);
            build_a_kernel<<<unsigned((rows * K2 + 255) / 256), 256, 0, st>>>(
                reinterpret_cast<const float2*>(prev), idx + li[l].parent_off + r0, lm, (int)rows, chi, Ahi, Alo);
            if (gemm_tf32x3(h, Ahi, Alo, Bhi, Blo, reinterpret_cast<float*>(curb + (int64_t)r0 * chi), (int)rows,
                            (int)K2, (int)K2, (int)K2, d_err, st, false) != BSG_OK)
              return nullptr;
            flops += 8.0 * rows * (double)chi * chi;
            continue;
          }
        }
        GemmArgs<R> g{};
        g.A = prev;
        g.pidx = idx + li[l].parent_off + r0;
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
  T* Lend = side(left, li_l, E[0], E[1], true);
  if (!Lend) return BSG_ERR_CUDA;
  T* Rend = side(right, li_r, E[2], E[3], false);
  if (!Rend) return BSG_ERR_CUDA;
  const int mid = left.sites.back();
  final_dot_kernel<R><<<unsigned((P * 32 + 255) / 256), 256, 0, st>>>(
      Lend, idx + fin_l, Rend, idx + fin_r, lam + (size_t)mid * chi, chi, P, reinterpret_cast<double2*>(amp));
  BSG_CUDA(cudaGetLastError());
  if (h->prof.on) BSG_TRY(h->prof.end(BSG_K_CONTRACT, st, ev, flops + 8.0 * P * chi));
  int err = 0;
  if (umma) BSG_CUDA(cudaMemcpyAsync(&err, d_err, 4, cudaMemcpyDeviceToHost, st));
  BSG_CUDA(cudaStreamSynchronize(st));  // the pinned index staging is reused by the next call
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
  BSG_CHECK_ARG(precision == BSG_PREC_FP64 || precision == BSG_PREC_SPLIT || precision == BSG_PREC_FP32,
                "bsg_pattern_amplitudes: bad precision %d", precision);
  for (int i = 0; i < M; ++i) BSG_CHECK_ARG(Gammas[i], "bsg_pattern_amplitudes: Gamma %d is NULL", i);
  BSG_CUDA(cudaSetDevice(h->device));
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  if (P == 0) return BSG_OK;
  std::vector<int32_t> pat((size_t)P * M);
  BSG_CUDA(cudaMemcpyAsync(pat.data(), patterns, pat.size() * 4, cudaMemcpyDeviceToHost, st));
  BSG_CUDA(cudaStreamSynchronize(st));
  for (size_t i = 0; i < pat.size(); ++i)
    if (pat[i] < 0 || pat[i] >= d) {
      set_error("bsg_pattern_amplitudes: photon number %d outside [0, d=%d)", pat[i], d);
      return BSG_ERR_INVALID;
    }
  const int m = (M - 1) / 2;  // left levels 0..m, right levels M-1..m+1
  std::vector<int> ls, rs;
  for (int i = 0; i <= m; ++i) ls.push_back(i);
  for (int i = M - 1; i > m; --i) rs.push_back(i);
  SidePlan left, right;
  plan_side(pat.data(), P, M, d, ls, left);
  plan_side(pat.data(), P, M, d, rs, right);
  if (precision == BSG_PREC_FP64)
    return run_contraction<double>(h, Gammas, Lambdas, M, chi, d, left, right, P, amp, false, st);
  if (precision == BSG_PREC_SPLIT && chi % 2 != 0) {
    set_error("bsg_pattern_amplitudes: the tensor-core path needs an even chi");
    return BSG_ERR_INVALID;
  }
  return run_contraction<float>(h, Gammas, Lambdas, M, chi, d, left, right, P, amp, precision == BSG_PREC_SPLIT, st);
}
