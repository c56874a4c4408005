// Photon-number sampling of the MPS (sampling_cpu.py:30-117, the GPU twin
// distributed_sampling.py:62-155) and the batched displacement operators it
// uses (sampling_cpu.py:133-148).
//
// Per batch of n samples:
//   alpha[b, m] = (mu_x + i mu_p)[b, m] / 2,  mu = sqrtW @ normals      (hbar = 2)
//   site 0 : t[b] = (sum_a Gamma_0[a, :, :]) D(alpha[b, 0])^T            [chi, dd]
//   site i : t[b] = ((pre[b] * Lambda_{i-1}) @ Gamma_i.reshape(chi, chi*d)).reshape(chi, d) D(alpha[b, i])^T
//   p[b, k] = sum_m |t[b, m, k]|^2 Lambda_i[m]^2   (last site: |t[b, 0, k]|^2)
//   k_b     = #{k : u[b, i] > cumsum(p[b] / sum p[b])[k]}                 (inverse CDF)
//   pre[b]  = t[b, :, k_b]
// The chain GEMM runs on the tensor cores (3xTF32, tcgen05) or as a SIMT
// FP64 / FP32 GEMM; one warp per sample fuses the displacement, the
// probabilities, the draw and the collapse.  D(alpha) is never stored: it
// is rebuilt per (sample, site) from a fixed eigen-decomposition of the
// truncated generator (below), which is exact for the truncated expm the
// reference computes with scipy.
//
// Displacement: in the dd-dimensional truncation, alpha a^dag - alpha^* a =
// r U P (-i X) P^-1 U^-1 with alpha = r e^{i theta}, U = diag(e^{i k theta}),
// P = diag(i^k) and X = a + a^dag (real symmetric tridiagonal).  With
// X = V diag(x) V^T:
//   D_kj = e^{i (k - j)(theta + pi/2)} sum_m V_km V_jm e^{-i r x_m}.
#include <cmath>
#include <cstring>
#include <type_traits>
#include <vector>

#include "bsg_cgemm.cuh"
#include "bsg_internal.h"

namespace bsg {

constexpr int kMaxDD = BSG_MAX_DD;
constexpr int kSampleWarps = 4;  // warps (samples) per 128-thread block

// Eigen-decomposition of X = a + a^dag in dd dimensions by cyclic Jacobi
// rotations (host, FP64).  V is row-major [dd][dd] with eigenvectors in columns.
static void position_eigs(int dd, std::vector<double>& V, std::vector<double>& x) {
  std::vector<double> A((size_t)dd * dd, 0.0);
  for (int k = 0; k + 1 < dd; ++k) A[(size_t)k * dd + k + 1] = A[(size_t)(k + 1) * dd + k] = std::sqrt(double(k + 1));
  V.assign((size_t)dd * dd, 0.0);
  for (int k = 0; k < dd; ++k) V[(size_t)k * dd + k] = 1.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0;
    for (int p = 0; p < dd; ++p)
      for (int q = p + 1; q < dd; ++q) off += A[(size_t)p * dd + q] * A[(size_t)p * dd + q];
    if (off < 1e-300) break;
    for (int p = 0; p < dd; ++p)
      for (int q = p + 1; q < dd; ++q) {
        const double apq = A[(size_t)p * dd + q];
        if (std::fabs(apq) < 1e-300) continue;
        const double app = A[(size_t)p * dd + p], aqq = A[(size_t)q * dd + q];
        const double tau = (aqq - app) / (2.0 * apq);
        const double t = (tau >= 0 ? 1.0 : -1.0) / (std::fabs(tau) + std::sqrt(1.0 + tau * tau));
        const double c = 1.0 / std::sqrt(1.0 + t * t), s = t * c;
        for (int k = 0; k < dd; ++k) {  // A <- A J (columns p, q)
          const double akp = A[(size_t)k * dd + p], akq = A[(size_t)k * dd + q];
          A[(size_t)k * dd + p] = c * akp - s * akq;
          A[(size_t)k * dd + q] = s * akp + c * akq;
        }
        for (int k = 0; k < dd; ++k) {  // A <- J^T A (rows p, q)
          const double apk = A[(size_t)p * dd + k], aqk = A[(size_t)q * dd + k];
          A[(size_t)p * dd + k] = c * apk - s * aqk;
          A[(size_t)q * dd + k] = s * apk + c * aqk;
        }
        for (int k = 0; k < dd; ++k) {  // V <- V J
          const double vkp = V[(size_t)k * dd + p], vkq = V[(size_t)k * dd + q];
          V[(size_t)k * dd + p] = c * vkp - s * vkq;
          V[(size_t)k * dd + q] = s * vkp + c * vkq;
        }
      }
  }
  x.resize(dd);
  for (int k = 0; k < dd; ++k) x[k] = A[(size_t)k * dd + k];
}

// Device tables for one dd: x[dd] and W[k][j][m] = V_km V_jm (k, j, m < dd),
// in FP64 and (after them) as FP32 copies for the FP32-precision paths.
static int displacement_tables(bsg_handle_t h, int dd, const double** x_dev, const double** W_dev,
                               const float** xf_dev, const float** Wf_dev, cudaStream_t st) {
  static_assert(sizeof(double) == 8, "");
  const size_t nx = (size_t)dd, nw = (size_t)dd * dd * dd;
  if (h->disp_dd != dd) {
    std::vector<double> V, x;
    position_eigs(dd, V, x);
    std::vector<double> host(nx + nw);
    std::memcpy(host.data(), x.data(), nx * 8);
    for (int k = 0; k < dd; ++k)
      for (int j = 0; j < dd; ++j)
        for (int m = 0; m < dd; ++m)
          host[nx + ((size_t)k * dd + j) * dd + m] = V[(size_t)k * dd + m] * V[(size_t)j * dd + m];
    std::vector<float> hostf(host.size());
    for (size_t i = 0; i < host.size(); ++i) hostf[i] = float(host[i]);
    BSG_TRY(h->disp_tab.ensure(host.size() * 12));
    BSG_CUDA(cudaMemcpyAsync(h->disp_tab.ptr, host.data(), host.size() * 8, cudaMemcpyHostToDevice, st));
    BSG_CUDA(cudaMemcpyAsync(reinterpret_cast<char*>(h->disp_tab.ptr) + host.size() * 8, hostf.data(),
                             hostf.size() * 4, cudaMemcpyHostToDevice, st));
    BSG_CUDA(cudaStreamSynchronize(st));
    h->disp_dd = dd;
  }
  *x_dev = reinterpret_cast<const double*>(h->disp_tab.ptr);
  *W_dev = *x_dev + nx;
  *xf_dev = reinterpret_cast<const float*>(*x_dev + nx + nw);
  *Wf_dev = *xf_dev + nx;
  return BSG_OK;
}

// e^{-i r x_m} (lanes m < dd) and e^{i p phi} (p = lane - 15) into per-warp
// shared arrays, then D[k][j] for k < dd, j < jmax.
__device__ __forceinline__ void sincos_r(double a, double* s, double* c) { sincos(a, s, c); }
__device__ __forceinline__ void sincos_r(float a, float* s, float* c) { sincosf(a, s, c); }
__device__ __forceinline__ double atan2_r(double y, double x) { return atan2(y, x); }
__device__ __forceinline__ float atan2_r(float y, float x) { return atan2f(y, x); }

// D(alpha) in precision R (the FP32 paths build it with FP32 math and tables).
template <class R>
__device__ void build_displacement(double2 al, int dd, int jmax, const R* __restrict__ x, const R* __restrict__ W,
                                   typename Cx<R>::T* ex, typename Cx<R>::T* ph, typename Cx<R>::T* D, int lane) {
  using T = typename Cx<R>::T;
  const R ax = R(al.x), ay = R(al.y);
  const R r = sqrt(ax * ax + ay * ay);
  const R phi = atan2_r(ay, ax) + R(1.5707963267948966);
  if (lane < dd) {
    R s, c;
    sincos_r(-r * x[lane], &s, &c);
    T v;
    v.x = c;
    v.y = s;
    ex[lane] = v;
  }
  if (lane < 31) {
    R s, c;
    sincos_r(R(lane - 15) * phi, &s, &c);
    T v;
    v.x = c;
    v.y = s;
    ph[lane] = v;
  }
  __syncwarp();
  for (int e = lane; e < dd * jmax; e += 32) {
    const int k = e / jmax, j = e % jmax;
    const R* w = W + ((size_t)k * dd + j) * dd;
    R sr = R(0), si = R(0);
    for (int m = 0; m < dd; ++m) {
      const R wm = w[m];
      sr += wm * ex[m].x;
      si += wm * ex[m].y;
    }
    const T p = ph[k - j + 15];
    T v;
    v.x = p.x * sr - p.y * si;
    v.y = p.x * si + p.y * sr;
    D[k * kMaxDD + j] = v;
  }
  __syncwarp();
}

__global__ void displacements_kernel(const double2* __restrict__ alpha, int64_t count, int dd,
                                     const double* __restrict__ x, const double* __restrict__ W,
                                     double2* __restrict__ out) {
  __shared__ double2 ex[kSampleWarps][kMaxDD], ph[kSampleWarps][32], D[kSampleWarps][kMaxDD * kMaxDD];
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t item = (int64_t)blockIdx.x * kSampleWarps + wib;
  if (item >= count) return;  // warp-uniform
  build_displacement<double>(alpha[item], dd, dd, x, W, ex[wib], ph[wib], D[wib], lane);
  for (int e = lane; e < dd * dd; e += 32) out[item * dd * dd + e] = D[wib][(e / dd) * kMaxDD + e % dd];
}

// alpha[b, m] = (sqrtW[m, :] . z[:, b] + i sqrtW[M + m, :] . z[:, b]) / 2
__global__ void alpha_kernel(const double* __restrict__ sqrtW, const double* __restrict__ z, int M, int64_t n,
                             int64_t b0, int64_t nb, double2* __restrict__ alpha) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nb * M) return;
  const int64_t b = t % nb;
  const int m = int(t / nb);
  const double* wx = sqrtW + (size_t)m * 2 * M;
  const double* wp = sqrtW + (size_t)(M + m) * 2 * M;
  double sx = 0.0, sp = 0.0;
  for (int q = 0; q < 2 * M; ++q) {
    const double zq = z[(size_t)q * n + b0 + b];
    sx = fma(wx[q], zq, sx);
    sp = fma(wp[q], zq, sp);
  }
  alpha[b * M + m] = make_double2(0.5 * sx, 0.5 * sp);
}

// T0[m, j] = sum_a Gamma_0[a, m, j]
template <class R>
__global__ void site0_kernel(const typename Cx<R>::T* __restrict__ G, int chi, int d,
                             typename Cx<R>::T* __restrict__ T0) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= chi * d) return;
  double sr = 0.0, si = 0.0;
  for (int a = 0; a < chi; ++a) {
    const typename Cx<R>::T v = G[(size_t)a * chi * d + t];
    sr += double(v.x);
    si += double(v.y);
  }
  T0[t].x = R(sr);
  T0[t].y = R(si);
}

// Bt[2(c d + j) + eo][2k + ei] (TF32 hi / lo) of Gamma_i[k, c, j]: the
// interleaved real form of the complex GEMM, K-major for the tensor cores.
__global__ void sample_bt_kernel(const float2* __restrict__ G, int chi, int d, float* __restrict__ Bhi,
                                 float* __restrict__ Blo) {
  const int64_t K2 = 2 * (int64_t)chi, N2 = 2 * (int64_t)chi * d;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= K2 * N2) return;
  const int64_t row = t / K2;
  const int col = int(t % K2);
  const int64_t cj = row >> 1;
  const int eo = int(row & 1), k = col >> 1, ei = col & 1;
  const float2 v = G[(int64_t)k * chi * d + cj];
  const float x = ei == 0 ? (eo == 0 ? v.x : v.y) : (eo == 0 ? -v.y : v.x);
  uint32_t hb, lb;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(hb) : "f"(x));
  const float hi = __uint_as_float(hb);
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(lb) : "f"(x - hi));
  Bhi[t] = hi;
  Blo[t] = __uint_as_float(lb);
}

template <class R>
struct SampleArgs {
  const typename Cx<R>::T* T;  // [nb, chi, d] (site > 0) or [chi, d] (site 0)
  int64_t t_stride;            // complex elements between samples (0 at site 0)
  const double2* alpha;        // [nb, M]
  const R* x;                  // [dd]
  const R* W;                  // [dd, dd, dd]
  const double* lam;           // Lambda_site [chi]; null at the last site
  const double* u;             // thresholds of this site for the chunk [nb]
  int64_t nb;
  int M, site, chi, d, dd;
  int64_t* samples;            // [nb, M] (chunk base)
  typename Cx<R>::T* pre;      // SIMT: next A [nb, chi] = pre * Lambda_site
  float* a_hi;                 // split: next A, interleaved real [nb, 2 chi], TF32 hi
  float* a_lo;                 //        and lo
};

// DDM: compile-time bound of dd (4, 8, 12 or 16) for the per-lane arrays and
// the unrolled dd x d products (a bound of 16 for dd = 8 ran 4x the
// instructions under predication)
template <class R, bool SPLIT, int DDM>
__global__ void __launch_bounds__(32 * kSampleWarps) sample_kernel(SampleArgs<R> a) {
  using T = typename Cx<R>::T;
  __shared__ T ex[kSampleWarps][kMaxDD], ph[kSampleWarps][32], D[kSampleWarps][kMaxDD * kMaxDD];
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t b = (int64_t)blockIdx.x * kSampleWarps + wib;
  if (b >= a.nb) return;  // warp-uniform
  const int d = a.d, dd = a.dd, chi = a.chi;
  const int jmax = d < dd ? d : dd;  // columns of t beyond d are zero
  build_displacement<R>(a.alpha[b * a.M + a.site], dd, jmax, a.x, a.W, ex[wib], ph[wib], D[wib], lane);
  const T* tb = a.T + b * a.t_stride;
  const T* Dw = D[wib];
  const bool last = a.lam == nullptr;
  R p[DDM];
#pragma unroll
  for (int k = 0; k < DDM; ++k) p[k] = R(0);
  for (int m = lane; m < (last ? 1 : chi); m += 32) {
    T t[DDM];
#pragma unroll
    for (int j = 0; j < DDM; ++j) {
      if (j < jmax) {
        t[j] = tb[(size_t)m * d + j];
      } else {
        t[j].x = R(0);
        t[j].y = R(0);
      }
    }
    const R w = last ? R(1) : R(a.lam[m]) * R(a.lam[m]);
#pragma unroll
    for (int k = 0; k < DDM; ++k) {
      if (k < dd) {
        R zr = R(0), zi = R(0);
#pragma unroll
        for (int j = 0; j < DDM; ++j) {
          if (j < jmax) {
            const T dk = Dw[k * kMaxDD + j];
            zr += dk.x * t[j].x - dk.y * t[j].y;
            zi += dk.x * t[j].y + dk.y * t[j].x;
          }
        }
        p[k] += w * (zr * zr + zi * zi);
      }
    }
  }
#pragma unroll
  for (int k = 0; k < DDM; ++k)
    for (int o = 16; o > 0; o >>= 1) p[k] += __shfl_xor_sync(0xffffffffu, p[k], o);
  // inverse CDF, as the reference: normalise, cumulative sum, count thresholds above
  R tot = R(0);
#pragma unroll
  for (int k = 0; k < DDM; ++k)
    if (k < dd) tot += p[k];
  const R u = R(a.u[b]);
  R cum = R(0);
  int cnt = 0;
#pragma unroll
  for (int k = 0; k < DDM; ++k) {
    if (k < dd) {
      cum += p[k] / tot;
      cnt += u > cum ? 1 : 0;
    }
  }
  if (lane == 0) a.samples[b * a.M + a.site] = cnt;
  if (last) return;
  // collapse: pre[m] = t[m, cnt] (zero when cnt == dd, as the reference's
  // one-hot selection leaves it), times Lambda_site[m] for the next GEMM
  for (int m = lane; m < chi; m += 32) {
    R zr = R(0), zi = R(0);
    if (cnt < dd) {
      for (int j = 0; j < jmax; ++j) {
        const T tj = tb[(size_t)m * d + j];
        const T dk = Dw[cnt * kMaxDD + j];
        zr += dk.x * tj.x - dk.y * tj.y;
        zi += dk.x * tj.y + dk.y * tj.x;
      }
    }
    const R l = R(a.lam[m]);
    zr *= l;
    zi *= l;
    if constexpr (SPLIT) {
      uint32_t hb;
      asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(hb) : "f"(float(zr)));
      const float hr = __uint_as_float(hb);
      asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(hb) : "f"(float(zi)));
      const float hi_ = __uint_as_float(hb);
      uint32_t lr, li;
      asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(lr) : "f"(float(zr) - hr));
      asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(li) : "f"(float(zi) - hi_));
      const size_t o = (size_t)b * 2 * chi + 2 * m;
      *reinterpret_cast<float2*>(a.a_hi + o) = make_float2(hr, hi_);
      *reinterpret_cast<float2*>(a.a_lo + o) = make_float2(__uint_as_float(lr), __uint_as_float(li));
    } else {
      T v;
      v.x = zr;
      v.y = zi;
      a.pre[(size_t)b * chi + m] = v;
    }
  }
}

template <class R, bool SPLIT>
static int run_sampler(bsg_handle_t h, const void* const* Gd, const double* lam, int M, int chi, int d, int dd,
                       const double* sqrtW, const double* normals, const double* uniforms, int64_t n,
                       int64_t* samples, cudaStream_t st) {
  using T = typename Cx<R>::T;
  const double* xd;
  const double* Wd;
  const float* xf;
  const float* Wf;
  BSG_TRY(displacement_tables(h, dd, &xd, &Wd, &xf, &Wf, st));
  auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
  // per-sample bytes: T, next A, alpha
  const size_t per = (size_t)chi * d * sizeof(T) + (SPLIT ? (size_t)chi * 16 : (size_t)chi * sizeof(T)) + (size_t)M * 16;
  const size_t budget = size_t(16) << 30;
  int64_t chunk = std::max<int64_t>(1, std::min<int64_t>(n, (int64_t)(budget / per)));
  if (SPLIT) chunk = std::min<int64_t>(chunk, (int64_t)1 << 30);
  const size_t o_T = 0, o_A = al((size_t)chunk * chi * d * sizeof(T));
  const size_t a_bytes = SPLIT ? al((size_t)chunk * 2 * chi * 4) : al((size_t)chunk * chi * sizeof(T));
  const size_t o_Alo = o_A + a_bytes, o_al = o_Alo + (SPLIT ? a_bytes : 0);
  const size_t o_B = o_al + al((size_t)chunk * M * 16);
  const size_t b_bytes = SPLIT ? al((size_t)4 * chi * chi * d * 4) : 0;
  const size_t o_T0 = o_B + 2 * b_bytes, o_err = o_T0 + al((size_t)chi * d * sizeof(T));
  BSG_TRY(h->sample_ws.ensure(o_err + 256));
  char* base = reinterpret_cast<char*>(h->sample_ws.ptr);
  T* Tb = reinterpret_cast<T*>(base + o_T);
  T* pre = reinterpret_cast<T*>(base + o_A);
  float* a_hi = reinterpret_cast<float*>(base + o_A);
  float* a_lo = reinterpret_cast<float*>(base + o_Alo);
  double2* alpha = reinterpret_cast<double2*>(base + o_al);
  float* Bhi = reinterpret_cast<float*>(base + o_B);
  float* Blo = reinterpret_cast<float*>(base + o_B + b_bytes);
  T* T0 = reinterpret_cast<T*>(base + o_T0);
  int* d_err = reinterpret_cast<int*>(base + o_err);
  BSG_CUDA(cudaMemsetAsync(d_err, 0, 4, st));
  BSG_PROFILED(h, BSG_K_SAMPLE, st, (double)chi * d,
               (site0_kernel<R><<<(chi * d + 255) / 256, 256, 0, st>>>(reinterpret_cast<const T*>(Gd[0]), chi, d,
                                                                        T0)));
  for (int64_t b0 = 0; b0 < n; b0 += chunk) {
    const int64_t nb = std::min<int64_t>(chunk, n - b0);
    BSG_PROFILED(h, BSG_K_SAMPLE, st, (double)nb * M * 4 * M,
                 (alpha_kernel<<<unsigned((nb * M + 255) / 256), 256, 0, st>>>(sqrtW, normals, M, n, b0, nb,
                                                                                alpha)));
    const unsigned sblocks = unsigned((nb + kSampleWarps - 1) / kSampleWarps);
    for (int i = 0; i < M; ++i) {
      SampleArgs<R> sa{};
      if (i == 0) {
        sa.T = T0;
        sa.t_stride = 0;
      } else {
        // T = A @ Gamma_i.reshape(chi, chi d)
        if constexpr (SPLIT) {
          const int64_t K2 = 2 * (int64_t)chi, N2 = 2 * (int64_t)chi * d;
          BSG_PROFILED(h, BSG_K_SAMPLE, st, (double)K2 * N2,
                       (sample_bt_kernel<<<unsigned((K2 * N2 + 255) / 256), 256, 0, st>>>(
                           reinterpret_cast<const float2*>(Gd[i]), chi, d, Bhi, Blo)));
          cudaEvent_t ev = nullptr;
          if (h->prof.on) BSG_TRY(h->prof.begin(BSG_K_CONTRACT, st, &ev));
          BSG_TRY(gemm_tf32x3(h, a_hi, a_lo, Bhi, Blo, reinterpret_cast<float*>(Tb), (int)nb, (int)N2, (int)K2,
                              (int)N2, d_err, st, false));
          if (h->prof.on) BSG_TRY(h->prof.end(BSG_K_CONTRACT, st, ev, 8.0 * nb * (double)chi * chi * d));
        } else {
          GemmArgs<R> g{};
          g.A = pre;
          g.pidx = nullptr;
          g.lam = nullptr;
          g.B = reinterpret_cast<const T*>(Gd[i]);
          g.sk = (int64_t)chi * d;
          g.sc = 1;
          g.C = Tb;
          g.rows = (int)nb;
          g.K = chi;
          g.N = chi * d;
          dim3 grid((g.N + TN - 1) / TN, (g.rows + TM - 1) / TM);
          BSG_PROFILED(h, BSG_K_CONTRACT, st, 8.0 * nb * (double)chi * chi * d,
                       (cgemm_kernel<R><<<grid, 256, 0, st>>>(g)));
        }
        sa.T = Tb;
        sa.t_stride = (int64_t)chi * d;
      }
      sa.alpha = alpha;
      if constexpr (std::is_same<R, double>::value) {
        sa.x = xd;
        sa.W = Wd;
      } else {
        sa.x = xf;
        sa.W = Wf;
      }
      sa.lam = i < M - 1 ? lam + (size_t)i * chi : nullptr;
      sa.u = uniforms + (size_t)i * n + b0;
      sa.nb = nb;
      sa.M = M;
      sa.site = i;
      sa.chi = chi;
      sa.d = d;
      sa.dd = dd;
      sa.samples = samples + b0 * M;
      sa.pre = pre;
      sa.a_hi = a_hi;
      sa.a_lo = a_lo;
      if (dd <= 4)
        BSG_PROFILED(h, BSG_K_SAMPLE, st, (double)nb * chi * dd * d,
                     (sample_kernel<R, SPLIT, 4><<<sblocks, 32 * kSampleWarps, 0, st>>>(sa)));
      else if (dd <= 8)
        BSG_PROFILED(h, BSG_K_SAMPLE, st, (double)nb * chi * dd * d,
                     (sample_kernel<R, SPLIT, 8><<<sblocks, 32 * kSampleWarps, 0, st>>>(sa)));
      else if (dd <= 12)
        BSG_PROFILED(h, BSG_K_SAMPLE, st, (double)nb * chi * dd * d,
                     (sample_kernel<R, SPLIT, 12><<<sblocks, 32 * kSampleWarps, 0, st>>>(sa)));
      else
        BSG_PROFILED(h, BSG_K_SAMPLE, st, (double)nb * chi * dd * d,
                     (sample_kernel<R, SPLIT, kMaxDD><<<sblocks, 32 * kSampleWarps, 0, st>>>(sa)));
    }
  }
  int err = 0;
  BSG_CUDA(cudaMemcpyAsync(&err, d_err, 4, cudaMemcpyDeviceToHost, st));
  BSG_CUDA(cudaStreamSynchronize(st));
  if (err) {
    set_error("bsg_sample: a tensor-core pipeline wait timed out");
    return BSG_ERR_CUDA;
  }
  return BSG_OK;
}

}  // namespace bsg

using namespace bsg;

extern "C" int bsg_displacements(bsg_handle_t h, const double* alpha, int64_t count, int dd, double* D,
                                 bsg_stream_t stream) {
  BSG_CHECK_ARG(h, "bsg_displacements: null handle");
  BSG_CHECK_ARG((alpha && D) || count == 0, "bsg_displacements: null pointer");
  BSG_CHECK_ARG(count >= 0 && dd >= 1 && dd <= kMaxDD, "bsg_displacements: need 1 <= dd <= %d (dd=%d)", kMaxDD, dd);
  BSG_CUDA(cudaSetDevice(h->device));
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  if (count == 0) return BSG_OK;
  const double* xd;
  const double* Wd;
  const float* xf;
  const float* Wf;
  BSG_TRY(displacement_tables(h, dd, &xd, &Wd, &xf, &Wf, st));
  BSG_PROFILED(h, BSG_K_SAMPLE, st, (double)count * dd * dd * dd,
               (displacements_kernel<<<unsigned((count + kSampleWarps - 1) / kSampleWarps), 32 * kSampleWarps, 0,
                                       st>>>(reinterpret_cast<const double2*>(alpha), count, dd, xd, Wd,
                                             reinterpret_cast<double2*>(D))));
  return BSG_OK;
}

extern "C" int bsg_sample(bsg_handle_t h, const void* const* Gammas, const double* Lambdas, int M, int chi, int d,
                          int dd, const double* sqrtW, const double* normals, const double* uniforms, int64_t n,
                          int precision, int64_t* samples, bsg_stream_t stream) {
  BSG_CHECK_ARG(h, "bsg_sample: null handle");
  BSG_CHECK_ARG(Gammas && Lambdas && sqrtW && normals && uniforms && samples, "bsg_sample: null pointer");
  BSG_CHECK_ARG(M >= 2 && chi >= 1 && d >= 1 && n >= 0, "bsg_sample: bad sizes M=%d chi=%d d=%d", M, chi, d);
  BSG_CHECK_ARG(dd >= d && dd <= kMaxDD, "bsg_sample: need d <= dd <= %d (d=%d, dd=%d)", kMaxDD, d, dd);
  BSG_CHECK_ARG(precision == BSG_PREC_FP64 || precision == BSG_PREC_SPLIT || precision == BSG_PREC_FP32,
                "bsg_sample: bad precision %d", precision);
  BSG_CHECK_ARG((int64_t)chi * d <= INT32_MAX / 2, "bsg_sample: chi * d too large");
  for (int i = 0; i < M; ++i) BSG_CHECK_ARG(Gammas[i], "bsg_sample: Gamma %d is NULL", i);
  BSG_CUDA(cudaSetDevice(h->device));
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  if (n == 0) return BSG_OK;
  if (precision == BSG_PREC_FP64)
    return run_sampler<double, false>(h, Gammas, Lambdas, M, chi, d, dd, sqrtW, normals, uniforms, n, samples, st);
  if (precision == BSG_PREC_FP32)
    return run_sampler<float, false>(h, Gammas, Lambdas, M, chi, d, dd, sqrtW, normals, uniforms, n, samples, st);
  BSG_CHECK_ARG(chi % 2 == 0 && chi >= 16, "bsg_sample: the tensor-core path needs an even chi >= 16 (chi=%d)", chi);
  return run_sampler<float, true>(h, Gammas, Lambdas, M, chi, d, dd, sqrtW, normals, uniforms, n, samples, st);
}
