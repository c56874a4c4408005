// Sigma (Fock-amplitude generating matrix) of a site's Gaussian unitary, FP64.
//
// The reference builds Sigma from a Bloch-Messiah decomposition (polar SVD,
// SVD of the squeezing block, a matrix square root; MPS_cpu.py:189-229,
// 305-312, 357-372).  The same matrix follows from the complex form of the
// symplectic S = (1 (+) S_l)^{-1} S_r directly:
//   A = (Sxx + Spp + i(Spx - Sxp))/2,  B = (Sxx - Spp + i(Spx + Sxp))/2,
//   X = conj(A)^{-1},  Sigma = [[B X, X^T], [X, -X conj(B)]],  Z = sqrt|det A|.
// Site 0 uses the pure covariance V' = L sq_cov L^T instead of a Williamson
// decomposition of the full state: with N, Mc the A/B-formulas applied to V',
// Sigma11 = Mc conj(N + I)^{-1} and Z = (det((N + I)/2))^{1/4}.
// (1 (+) S_l)^{-1} uses the symplectic inverse [[e^T, -b^T], [-c^T, a^T]] of
// S_l = [[a, b], [c, e]].
// One CTA per job; every job is independent, so many sites run in one launch.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <type_traits>

#include "bsg_df.cuh"
#include "bsg_internal.h"

namespace bsg {

// Row r of L = (1 (+) S_l)^{-1} applied to column c of matrix In (In[k][c] = in[k*ld + c],
// or in[c*ld + k] when trans).
__device__ __forceinline__ double apply_L(const SigmaJob& jb, int r, int c, const double* in, int ld, bool trans) {
  const int Mr = jb.Mr, ml = jb.m_l;
  auto at = [&](int k) { return trans ? in[(size_t)c * ld + k] : in[(size_t)k * ld + c]; };
  const bool inner_r = (r != 0 && r != Mr);
  if (!inner_r || ml == 0) return at(r);
  // inner index of r in S_l coordinates
  const int rl = r < Mr ? r - 1 : ml + (r - Mr - 1);
  const int n2 = jb.ld_l;
  const double* S = jb.S_l;
  double acc = 0.0;
  // Linv[rl][kl]: rl<ml: [e^T | -b^T] row rl -> e[k][rl] (k<ml), -b[k][rl] (k<ml)
  //               rl>=ml: [-c^T | a^T] row rl-ml -> -c[k][rl-ml], a[k][rl-ml]
  if (rl < ml) {
    for (int k = 0; k < ml; ++k) {
      double e_ = S[(size_t)(ml + k) * n2 + (ml + rl)];  // e[k][rl]
      double b_ = S[(size_t)k * n2 + (ml + rl)];         // b[k][rl]
      acc = fma(e_, at(1 + k), acc);
      acc = fma(-b_, at(Mr + 1 + k), acc);
    }
  } else {
    const int q = rl - ml;
    for (int k = 0; k < ml; ++k) {
      double c_ = S[(size_t)(ml + k) * n2 + q];  // c[k][q]
      double a_ = S[(size_t)k * n2 + q];         // a[k][q]
      acc = fma(-c_, at(1 + k), acc);
      acc = fma(a_, at(Mr + 1 + k), acc);
    }
  }
  return acc;
}

// One CTA per call: the whole Sigma construction of one site (the
// descriptor travels as a kernel parameter, so no host-to-device copy).
// In-place Gauss-Jordan with partial pivoting on G = [A' | I] (Mr x 2Mr
// complex, leading dimension n2, global memory): the right half becomes
// A'^-1 and sh.logdet log|det A'| (*status = 1 on a zero pivot).  A step
// updates only the columns that can be non-zero in its pivot row -- the
// columns of A' not yet eliminated and the columns of the inverse already
// reached by earlier pivots (the original indices of the rows pivoted so
// far) -- so a step costs Mr x Mr updates, not Mr x 2Mr; the pivot row and
// the multipliers sit in shared memory and a warp updates one row.  Column
// col is not written back (it is never read again).
constexpr int kGJMaxModes = 1024;
struct GJShared {
  double2 f[kGJMaxModes];  // multipliers G[r][col] of this step
  double2 v[kGJMaxModes];  // the scaled pivot row on the active columns
  int cols[kGJMaxModes];   // the active columns
  int orig[kGJMaxModes];   // original row of each row position (row swaps)
  double val[32];
  int idx[32];
  double logdet;
  float4 inv4;  // 1 / pivot, double-float (gj_inverse_df)
  int piv;
};

__device__ void gj_inverse(double2* G, int Mr, int n2, int* status, GJShared& sh) {
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
  for (int r = tid; r < Mr; r += nt) sh.orig[r] = r;
  if (tid == 0) sh.logdet = 0.0;
  __syncthreads();
  for (int col = 0; col < Mr; ++col) {
    double best = -1.0;
    int bi = col;
    for (int r = col + tid; r < Mr; r += nt) {
      const double2 v = G[(size_t)r * n2 + col];
      const double m = v.x * v.x + v.y * v.y;
      if (m > best) {
        best = m;
        bi = r;
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const double ob = __shfl_down_sync(0xffffffffu, best, o);
      const int oi = __shfl_down_sync(0xffffffffu, bi, o);
      if (ob > best || (ob == best && oi < bi)) {
        best = ob;
        bi = oi;
      }
    }
    if (lane == 0) {
      sh.val[warp] = best;
      sh.idx[warp] = bi;
    }
    __syncthreads();
    if (tid == 0) {
      double b = sh.val[0];
      int i0 = sh.idx[0];
      for (int w = 1; w < nw; ++w)
        if (sh.val[w] > b || (sh.val[w] == b && sh.idx[w] < i0)) {
          b = sh.val[w];
          i0 = sh.idx[w];
        }
      sh.piv = i0;
      if (!(b > 0.0)) *status = 1;
      sh.logdet += 0.5 * log(b > 0.0 ? b : 1e-300);
      if (i0 != col) {
        const int t = sh.orig[i0];
        sh.orig[i0] = sh.orig[col];
        sh.orig[col] = t;
      }
    }
    __syncthreads();
    const int p = sh.piv;
    if (p != col) {
      for (int c = tid; c < n2; c += nt) {
        const double2 t = G[(size_t)p * n2 + c];
        G[(size_t)p * n2 + c] = G[(size_t)col * n2 + c];
        G[(size_t)col * n2 + c] = t;
      }
    }
    // active columns: A' columns col+1..Mr-1, then the inverse's columns Mr + orig[0..col]
    const int nleft = Mr - col - 1;
    for (int q = tid; q < Mr; q += nt) sh.cols[q] = q < nleft ? col + 1 + q : Mr + sh.orig[q - nleft];
    __syncthreads();
    const double2 pv = G[(size_t)col * n2 + col];
    const double den = pv.x * pv.x + pv.y * pv.y;
    const double2 inv = den > 0.0 ? make_double2(pv.x / den, -pv.y / den) : make_double2(0.0, 0.0);
    for (int q = tid; q < Mr; q += nt) {
      double2* cp = G + (size_t)col * n2 + sh.cols[q];
      const double2 v = *cp;
      const double2 w = make_double2(v.x * inv.x - v.y * inv.y, v.x * inv.y + v.y * inv.x);
      *cp = w;
      sh.v[q] = w;
    }
    for (int r = tid; r < Mr; r += nt) sh.f[r] = r == col ? make_double2(0.0, 0.0) : G[(size_t)r * n2 + col];
    __syncthreads();
    for (int r = warp; r < Mr; r += nw) {
      const double2 f = sh.f[r];
      if (f.x == 0.0 && f.y == 0.0) continue;
      double2* row = G + (size_t)r * n2;
      for (int q = lane; q < Mr; q += 32) {
        const double2 v = sh.v[q];
        double2* gp = row + sh.cols[q];
        double2 g = *gp;
        g.x -= f.x * v.x - f.y * v.y;
        g.y -= f.x * v.y + f.y * v.x;
        *gp = g;
      }
    }
    __syncthreads();
  }
}

__global__ void __launch_bounds__(1024) sigma_kernel(const SigmaJob jb) {
  const int Mr = jb.Mr, n2 = 2 * Mr;
  const int tid = threadIdx.x, nt = blockDim.x;
  double* P = jb.ws;                                     // [n2, n2]
  double* T = P + (size_t)n2 * n2;                       // [n2, n2]
  double2* G = reinterpret_cast<double2*>(T + (size_t)n2 * n2);  // [Mr, 2Mr]  (conj A' | I)
  double2* Bm = G + (size_t)Mr * n2;                     // [Mr, Mr]
  __shared__ GJShared sh;

  // P = L S_r (general) or L sq L^T (first)
  for (int i = tid; i < n2 * n2; i += nt) {
    int r = i / n2, c = i % n2;
    T[i] = apply_L(jb, r, c, jb.S_r, jb.ld_r, false);
  }
  __syncthreads();
  if (jb.first) {
    for (int i = tid; i < n2 * n2; i += nt) {
      int r = i / n2, c = i % n2;
      P[i] = apply_L(jb, r, c, T, n2, true);  // L (L sq)^T = L sq L^T
    }
  } else {
    for (int i = tid; i < n2 * n2; i += nt) P[i] = T[i];
  }
  __syncthreads();
  // A' and B parts; G = [conj(A') | I]
  for (int i = tid; i < Mr * Mr; i += nt) {
    int r = i / Mr, c = i % Mr;
    double xx = P[(size_t)r * n2 + c], xp = P[(size_t)r * n2 + Mr + c];
    double px = P[(size_t)(Mr + r) * n2 + c], pp = P[(size_t)(Mr + r) * n2 + Mr + c];
    double ar = 0.5 * (xx + pp), ai = 0.5 * (px - xp);
    if (jb.first && r == c) ar += 1.0;
    G[(size_t)r * n2 + c] = make_double2(ar, -ai);
    G[(size_t)r * n2 + Mr + c] = make_double2(r == c ? 1.0 : 0.0, 0.0);
    Bm[i] = make_double2(0.5 * (xx - pp), 0.5 * (px + xp));
  }
  __syncthreads();
  gj_inverse(G, Mr, n2, jb.status, sh);
  // X = right half of G
  auto X = [&](int r, int c) { return G[(size_t)r * n2 + Mr + c]; };
  for (int i = tid; i < Mr * Mr; i += nt) {
    int r = i / Mr, c = i % Mr;
    double2 s11 = make_double2(0.0, 0.0);
    for (int k = 0; k < Mr; ++k) {
      double2 b = Bm[(size_t)r * Mr + k], x = X(k, c);
      s11.x += b.x * x.x - b.y * x.y;
      s11.y += b.x * x.y + b.y * x.x;
    }
    jb.Sigma[(size_t)r * n2 + c] = s11;
    if (jb.first) {
      jb.Sigma[(size_t)r * n2 + Mr + c] = make_double2(0.0, 0.0);
      jb.Sigma[(size_t)(Mr + r) * n2 + c] = make_double2(0.0, 0.0);
      jb.Sigma[(size_t)(Mr + r) * n2 + Mr + c] = make_double2(0.0, 0.0);
    } else {
      jb.Sigma[(size_t)r * n2 + Mr + c] = X(c, r);       // X^T
      jb.Sigma[(size_t)(Mr + r) * n2 + c] = X(r, c);     // X
      double2 s22 = make_double2(0.0, 0.0);
      for (int k = 0; k < Mr; ++k) {
        double2 x = X(r, k), b = Bm[(size_t)k * Mr + c];  // X conj(B)
        s22.x += x.x * b.x + x.y * b.y;
        s22.y += -x.x * b.y + x.y * b.x;
      }
      jb.Sigma[(size_t)(Mr + r) * n2 + Mr + c] = make_double2(-s22.x, -s22.y);
    }
  }
  if (tid == 0) {
    double ld = sh.logdet;  // log|det A'|
    *jb.Z = jb.first ? exp(0.25 * (ld - Mr * log(2.0))) : exp(0.5 * ld);
  }
}

size_t sigma_ws_bytes(int Mr) { return (size_t)112 * Mr * Mr + 256; }

// ---- the same construction in three phases over many CTAs ------------------
// The one-CTA-per-site kernel above does ~24 M_r^3 FP64 FMAs on one SM; the
// products (P = L S_r, or L sq L^T at site 0, then B X and -X conj(B)) are
// tiled over many CTAs here, and only the Gauss-Jordan inversion stays one
// CTA per site.  Same arithmetic per element up to summation order.
// Workspace per job (doubles): P [n2 n2] | T [n2 n2] = L explicitly |
// G [M_r, 2 M_r] complex (site 0: L sq first) | Bm [M_r M_r] complex.

// T = L = 1 (+) S_l^{-1} (symplectic inverse [[e^T, -b^T], [-c^T, a^T]]) on
// the site-first ordering, identity on the site's own x and p rows.
__global__ void sigma_linv_kernel(const SigmaJob* __restrict__ jobs) {
  const SigmaJob jb = jobs[blockIdx.y];
  const int Mr = jb.Mr, n2 = 2 * Mr, ml = jb.m_l;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)n2 * n2) return;
  const int r = int(t / n2), c = int(t % n2);
  double* T = jb.ws + (size_t)n2 * n2;
  const bool inner_r = r != 0 && r != Mr, inner_c = c != 0 && c != Mr;
  double v;
  if (!inner_r || ml == 0) {
    v = r == c ? 1.0 : 0.0;
  } else if (!inner_c) {
    v = 0.0;
  } else {
    const int rl = r < Mr ? r - 1 : ml + (r - Mr - 1);
    const int kl = c < Mr ? c - 1 : ml + (c - Mr - 1);
    const int ld = jb.ld_l;
    const double* S = jb.S_l;
    if (rl < ml) v = kl < ml ? S[(size_t)(ml + kl) * ld + (ml + rl)] : -S[(size_t)(kl - ml) * ld + (ml + rl)];
    else v = kl < ml ? -S[(size_t)(ml + kl) * ld + (rl - ml)] : S[(size_t)(kl - ml) * ld + (rl - ml)];
  }
  T[t] = v;
}

// Double-float complex entries of the Gauss-Jordan matrix: (re s, re t,
// im s, im t), value s + t per part; s + t is renormalised to hi + lo on
// every store (Knuth's two-sum).
__device__ __forceinline__ float4 df_cnorm(float4 v) {
  const float2 r = df_norm(v.x, v.y), i = df_norm(v.z, v.w);
  return make_float4(r.x, r.y, i.x, i.y);
}
__device__ __forceinline__ double2 df_cval(float4 v) {
  return make_double2(double(v.x) + double(v.y), double(v.z) + double(v.w));
}
__device__ __forceinline__ float4 df_csplit(double2 v) {
  const float2 r = df_split(v.x), i = df_split(v.y);
  return make_float4(r.x, r.y, i.x, i.y);
}

// gj_inverse with G in double-float (float4 entries, same layout and size as
// double2): the pivot search, the row scaling and the rank-1 updates run on
// the FP32 pipe (four exact products per complex multiply-add); the pivot's
// reciprocal and log|pivot| in FP64.  Entries carry ~2^-48 relative error
// per operation (A' is well conditioned: its singular values are the
// cosh r_k of the site unitary's squeezing), which is what the
// split-precision DP reads of Sigma (FP32 pairs).
__device__ void gj_inverse_df(float4* G, int Mr, int n2, int* status, GJShared& sh) {
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
  float4* f4 = reinterpret_cast<float4*>(sh.f);
  float4* v4 = reinterpret_cast<float4*>(sh.v);
  for (int r = tid; r < Mr; r += nt) sh.orig[r] = r;
  if (tid == 0) sh.logdet = 0.0;
  __syncthreads();
  for (int col = 0; col < Mr; ++col) {
    float best = -1.f;
    int bi = col;
    for (int r = col + tid; r < Mr; r += nt) {
      const float4 v = G[(size_t)r * n2 + col];  // stored normalised: hi parts carry the magnitude
      const float m = v.x * v.x + v.z * v.z;
      if (m > best) {
        best = m;
        bi = r;
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const float ob = __shfl_down_sync(0xffffffffu, best, o);
      const int oi = __shfl_down_sync(0xffffffffu, bi, o);
      if (ob > best || (ob == best && oi < bi)) {
        best = ob;
        bi = oi;
      }
    }
    if (lane == 0) {
      sh.val[warp] = best;
      sh.idx[warp] = bi;
    }
    __syncthreads();
    if (tid == 0) {
      double b = sh.val[0];
      int i0 = sh.idx[0];
      for (int w = 1; w < nw; ++w)
        if (sh.val[w] > b || (sh.val[w] == b && sh.idx[w] < i0)) {
          b = sh.val[w];
          i0 = sh.idx[w];
        }
      sh.piv = i0;
      const double2 pv = df_cval(G[(size_t)i0 * n2 + col]);
      const double m = pv.x * pv.x + pv.y * pv.y;
      if (!(m > 0.0)) *status = 1;
      sh.logdet += 0.5 * log(m > 0.0 ? m : 1e-300);
      const double2 inv = m > 0.0 ? make_double2(pv.x / m, -pv.y / m) : make_double2(0.0, 0.0);
      sh.inv4 = df_csplit(inv);  // 1 / pivot
      if (i0 != col) {
        const int t = sh.orig[i0];
        sh.orig[i0] = sh.orig[col];
        sh.orig[col] = t;
      }
    }
    __syncthreads();
    const int p = sh.piv;
    if (p != col) {
      for (int c = tid; c < n2; c += nt) {
        const float4 t = G[(size_t)p * n2 + c];
        G[(size_t)p * n2 + c] = G[(size_t)col * n2 + c];
        G[(size_t)col * n2 + c] = t;
      }
    }
    const int nleft = Mr - col - 1;
    for (int q = tid; q < Mr; q += nt) sh.cols[q] = q < nleft ? col + 1 + q : Mr + sh.orig[q - nleft];
    __syncthreads();
    const float4 iv = sh.inv4;
    const float2 ir = make_float2(iv.x, iv.y), ii = make_float2(iv.z, iv.w);
    for (int q = tid; q < Mr; q += nt) {
      float4* cp = G + (size_t)col * n2 + sh.cols[q];
      const float4 v = *cp;
      const float2 vr = make_float2(v.x, v.y), vi = make_float2(v.z, v.w);
      float sr = 0.f, tr = 0.f, si = 0.f, ti = 0.f;
      df_mac(sr, tr, vr, ir);
      df_mac(sr, tr, make_float2(-vi.x, -vi.y), ii);
      df_mac(si, ti, vr, ii);
      df_mac(si, ti, vi, ir);
      const float4 w = df_cnorm(make_float4(sr, tr, si, ti));
      *cp = w;
      v4[q] = w;
    }
    for (int r = tid; r < Mr; r += nt) f4[r] = r == col ? make_float4(0.f, 0.f, 0.f, 0.f) : G[(size_t)r * n2 + col];
    __syncthreads();
    for (int r = warp; r < Mr; r += nw) {
      const float4 f = f4[r];
      if (f.x == 0.f && f.z == 0.f) continue;
      const float2 nfr = make_float2(-f.x, -f.y), fi = make_float2(f.z, f.w), nfi = make_float2(-f.z, -f.w);
      float4* row = G + (size_t)r * n2;
      for (int q = lane; q < Mr; q += 32) {
        const float4 v = v4[q];
        const float2 vr = make_float2(v.x, v.y), vi = make_float2(v.z, v.w);
        float4* gp = row + sh.cols[q];
        float4 g = *gp;
        // g -= f v: re -= fr vr - fi vi, im -= fr vi + fi vr
        df_mac(g.x, g.y, nfr, vr);
        df_mac(g.x, g.y, fi, vi);
        df_mac(g.z, g.w, nfr, vi);
        df_mac(g.z, g.w, nfi, vr);
        *gp = df_cnorm(g);
      }
    }
    __syncthreads();
  }
}

// MODE 0: C = L B0 with B0 = S_r (C -> P) or, at site 0, B0 = sq (C -> G region);
// MODE 1 (site 0 only): P = L C0^T with C0 = L sq.  64 x 64 tiles, 256 threads.
// DF: the products in double-float on the FP32 pipe (operands split once per
// tile load; the split-precision build, whose DP reads Sigma as FP32 pairs),
// else FP64.
template <int MODE, bool DF>
__global__ void __launch_bounds__(256) sigma_gemm_kernel(const SigmaJob* __restrict__ jobs) {
  const SigmaJob jb = jobs[blockIdx.y];
  if (MODE == 1 && !jb.first) return;
  const int n2 = 2 * jb.Mr, tn = (n2 + 63) / 64;
  if ((int)blockIdx.x >= tn * tn) return;
  const int i0 = (blockIdx.x / tn) * 64, j0 = (blockIdx.x % tn) * 64;
  const double* L = jb.ws + (size_t)n2 * n2;
  double* Gr = jb.ws + 2 * (size_t)n2 * n2;
  const double* B;
  int64_t bs0, bs1;  // B(k, j) = B[k * bs0 + j * bs1]
  double* C;
  if (MODE == 0) {
    B = jb.S_r;
    bs0 = jb.ld_r;
    bs1 = 1;
    C = jb.first ? Gr : jb.ws;
  } else {
    B = Gr;
    bs0 = 1;
    bs1 = n2;
    C = jb.ws;
  }
  using E = typename std::conditional<DF, float2, double>::type;
  __shared__ E As[16][65], Bs[16][65];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  double acc[4][4] = {};
  float s[4][4] = {}, t[4][4] = {};
  for (int k0 = 0; k0 < n2; k0 += 16) {
    for (int e = threadIdx.x; e < 64 * 16; e += 256) {
      const int ii = e / 16, kk = e % 16, i = i0 + ii, k = k0 + kk;
      const double av = (i < n2 && k < n2) ? L[(size_t)i * n2 + k] : 0.0;
      const int kb = e / 64, jj = e % 64, j = j0 + jj, k2 = k0 + kb;
      const double bv = (k2 < n2 && j < n2) ? B[(int64_t)k2 * bs0 + (int64_t)j * bs1] : 0.0;
      if constexpr (DF) {
        As[kk][ii] = df_split(av);
        Bs[kb][jj] = df_split(bv);
      } else {
        As[kk][ii] = av;
        Bs[kb][jj] = bv;
      }
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 16; ++kk) {
      E av[4], bv[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        av[q] = As[kk][ty * 4 + q];
        bv[q] = Bs[kk][tx * 4 + q];
      }
#pragma unroll
      for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int w = 0; w < 4; ++w) {
          if constexpr (DF) df_mac(s[q][w], t[q][w], av[q], bv[w]);
          else acc[q][w] = fma(av[q], bv[w], acc[q][w]);
        }
    }
    __syncthreads();
  }
#pragma unroll
  for (int q = 0; q < 4; ++q)
#pragma unroll
    for (int w = 0; w < 4; ++w) {
      const int i = i0 + ty * 4 + q, j = j0 + tx * 4 + w;
      if (i < n2 && j < n2) C[(size_t)i * n2 + j] = DF ? double(s[q][w]) + double(t[q][w]) : acc[q][w];
    }
}

// One CTA per job: A', B from P, Gauss-Jordan for X = conj(A')^{-1}, Z, and
// the X / X^T blocks of Sigma (zeros at site 0).  DF: the Gauss-Jordan in
// double-float (gj_inverse_df); its inverse half is turned back into FP64
// in place for the products that follow.
template <bool DF>
__global__ void __launch_bounds__(1024) sigma_gj_kernel(const SigmaJob* __restrict__ jobs) {
  const SigmaJob jb = jobs[blockIdx.x];
  const int Mr = jb.Mr, n2 = 2 * Mr;
  const int tid = threadIdx.x, nt = blockDim.x;
  double* P = jb.ws;
  double2* G = reinterpret_cast<double2*>(jb.ws + 2 * (size_t)n2 * n2);
  float4* G4 = reinterpret_cast<float4*>(G);
  double2* Bm = G + (size_t)Mr * n2;
  __shared__ GJShared sh;
  for (int i = tid; i < Mr * Mr; i += nt) {
    int r = i / Mr, c = i % Mr;
    double xx = P[(size_t)r * n2 + c], xp = P[(size_t)r * n2 + Mr + c];
    double px = P[(size_t)(Mr + r) * n2 + c], pp = P[(size_t)(Mr + r) * n2 + Mr + c];
    double ar = 0.5 * (xx + pp), ai = 0.5 * (px - xp);
    if (jb.first && r == c) ar += 1.0;
    const double2 a = make_double2(ar, -ai), e = make_double2(r == c ? 1.0 : 0.0, 0.0);
    if (DF) {
      G4[(size_t)r * n2 + c] = df_csplit(a);
      G4[(size_t)r * n2 + Mr + c] = df_csplit(e);
    } else {
      G[(size_t)r * n2 + c] = a;
      G[(size_t)r * n2 + Mr + c] = e;
    }
    Bm[i] = make_double2(0.5 * (xx - pp), 0.5 * (px + xp));
  }
  __syncthreads();
  if (DF) {
    gj_inverse_df(G4, Mr, n2, jb.status, sh);
    for (int i = tid; i < Mr * Mr; i += nt) {
      const size_t o = (size_t)(i / Mr) * n2 + Mr + i % Mr;
      const float4 v = G4[o];
      G[o] = df_cval(v);  // same 16 bytes, read before written by this thread
    }
    __syncthreads();
  } else {
    gj_inverse(G, Mr, n2, jb.status, sh);
  }
  for (int i = tid; i < Mr * Mr; i += nt) {
    const int r = i / Mr, c = i % Mr;
    if (jb.first) {
      jb.Sigma[(size_t)r * n2 + Mr + c] = make_double2(0.0, 0.0);
      jb.Sigma[(size_t)(Mr + r) * n2 + c] = make_double2(0.0, 0.0);
      jb.Sigma[(size_t)(Mr + r) * n2 + Mr + c] = make_double2(0.0, 0.0);
    } else {
      jb.Sigma[(size_t)r * n2 + Mr + c] = G[(size_t)c * n2 + Mr + r];  // X^T
      jb.Sigma[(size_t)(Mr + r) * n2 + c] = G[(size_t)r * n2 + Mr + c];  // X
    }
  }
  if (tid == 0) {
    double ld = sh.logdet;  // log|det A'|
    *jb.Z = jb.first ? exp(0.25 * (ld - Mr * log(2.0))) : exp(0.5 * ld);
  }
}

// Sigma11 = B X (every site) and Sigma22 = -X conj(B) (blockIdx.z = 1, not at
// site 0): complex products, 32 x 32 tiles, 256 threads with 2 x 2 outputs;
// DF as in sigma_gemm_kernel (each complex operand split into four floats).
template <bool DF>
__global__ void __launch_bounds__(256) sigma_cgemm_kernel(const SigmaJob* __restrict__ jobs) {
  const SigmaJob jb = jobs[blockIdx.y];
  const int z = blockIdx.z;
  if (z == 1 && jb.first) return;
  const int Mr = jb.Mr, n2 = 2 * Mr, tn = (Mr + 31) / 32;
  if ((int)blockIdx.x >= tn * tn) return;
  const int i0 = (blockIdx.x / tn) * 32, j0 = (blockIdx.x % tn) * 32;
  const double2* G = reinterpret_cast<const double2*>(jb.ws + 2 * (size_t)n2 * n2);
  const double2* Bm = G + (size_t)Mr * n2;
  auto Aop = [&](int i, int k) { return z == 0 ? Bm[(size_t)i * Mr + k] : G[(size_t)i * n2 + Mr + k]; };
  auto Bop = [&](int k, int j) {
    if (z == 0) return G[(size_t)k * n2 + Mr + j];
    const double2 b = Bm[(size_t)k * Mr + j];
    return make_double2(b.x, -b.y);
  };
  using E = typename std::conditional<DF, float4, double2>::type;  // DF: (re hi, re lo, im hi, im lo)
  auto put = [](double2 v) -> E {
    if constexpr (DF) {
      const float2 r = df_split(v.x), i = df_split(v.y);
      return make_float4(r.x, r.y, i.x, i.y);
    } else {
      return v;
    }
  };
  __shared__ E As[16][33], Bs[16][33];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  double2 acc[2][2] = {};
  float sr[2][2] = {}, tr[2][2] = {}, si[2][2] = {}, ti[2][2] = {};
  for (int k0 = 0; k0 < Mr; k0 += 16) {
    for (int e = threadIdx.x; e < 32 * 16; e += 256) {
      const int ii = e / 16, kk = e % 16, i = i0 + ii, k = k0 + kk;
      As[kk][ii] = put((i < Mr && k < Mr) ? Aop(i, k) : make_double2(0.0, 0.0));
      const int kb = e / 32, jj = e % 32, j = j0 + jj, k2 = k0 + kb;
      Bs[kb][jj] = put((k2 < Mr && j < Mr) ? Bop(k2, j) : make_double2(0.0, 0.0));
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 16; ++kk) {
#pragma unroll
      for (int q = 0; q < 2; ++q)
#pragma unroll
        for (int w = 0; w < 2; ++w) {
          const E av = As[kk][ty * 2 + q], bv = Bs[kk][tx * 2 + w];
          if constexpr (DF) {
            const float2 ar = make_float2(av.x, av.y), ai = make_float2(av.z, av.w);
            const float2 br = make_float2(bv.x, bv.y), bi = make_float2(bv.z, bv.w);
            df_mac(sr[q][w], tr[q][w], ar, br);
            df_mac(sr[q][w], tr[q][w], make_float2(-ai.x, -ai.y), bi);
            df_mac(si[q][w], ti[q][w], ar, bi);
            df_mac(si[q][w], ti[q][w], ai, br);
          } else {
            acc[q][w].x = fma(av.x, bv.x, fma(-av.y, bv.y, acc[q][w].x));
            acc[q][w].y = fma(av.x, bv.y, fma(av.y, bv.x, acc[q][w].y));
          }
        }
    }
    __syncthreads();
  }
  const double sg = z == 0 ? 1.0 : -1.0;
#pragma unroll
  for (int q = 0; q < 2; ++q)
#pragma unroll
    for (int w = 0; w < 2; ++w) {
      const int i = i0 + ty * 2 + q, j = j0 + tx * 2 + w;
      if (DF) acc[q][w] = make_double2(double(sr[q][w]) + double(tr[q][w]), double(si[q][w]) + double(ti[q][w]));
      if (i < Mr && j < Mr)
        jb.Sigma[(size_t)(z == 0 ? i : Mr + i) * n2 + (z == 0 ? j : Mr + j)] =
            make_double2(sg * acc[q][w].x, sg * acc[q][w].y);
    }
}

int launch_sigma_jobs(bsg_handle_t h, const SigmaJob* jobs_host, int n_jobs, void* jobs_dev, cudaStream_t st,
                      bool df_products) {
  if (n_jobs <= 0) return BSG_OK;
  BSG_CUDA(cudaMemcpyAsync(jobs_dev, jobs_host, sizeof(SigmaJob) * n_jobs, cudaMemcpyHostToDevice, st));
  double work = 0.0;
  int max_mr = 1, first_mr = 0;
  for (int i = 0; i < n_jobs; ++i) {
    const int Mr = jobs_host[i].Mr;
    work += (jobs_host[i].first ? 28.0 : 24.0) * Mr * Mr * (double)Mr;
    max_mr = std::max(max_mr, Mr);
    if (jobs_host[i].first) first_mr = std::max(first_mr, Mr);
  }
  const SigmaJob* jd = reinterpret_cast<const SigmaJob*>(jobs_dev);
  const int64_t n2 = 2 * (int64_t)max_mr, tn = (n2 + 63) / 64, tc = (max_mr + 31) / 32;
  cudaEvent_t ev = nullptr;
  if (h->prof.on) BSG_TRY(h->prof.begin(BSG_K_SIGMA, st, &ev));
  sigma_linv_kernel<<<dim3(unsigned((n2 * n2 + 255) / 256), n_jobs), 256, 0, st>>>(jd);
  const dim3 g0(unsigned(tn * tn), n_jobs), gc(unsigned(tc * tc), n_jobs, 2);
  if (df_products) sigma_gemm_kernel<0, true><<<g0, 256, 0, st>>>(jd);
  else sigma_gemm_kernel<0, false><<<g0, 256, 0, st>>>(jd);
  if (first_mr) {
    const int64_t t1 = (2 * (int64_t)first_mr + 63) / 64;
    const dim3 g1(unsigned(t1 * t1), n_jobs);
    if (df_products) sigma_gemm_kernel<1, true><<<g1, 256, 0, st>>>(jd);
    else sigma_gemm_kernel<1, false><<<g1, 256, 0, st>>>(jd);
  }
  if (df_products) sigma_gj_kernel<true><<<n_jobs, h->tune[BSG_TUNE_FACTOR_THREADS], 0, st>>>(jd);
  else sigma_gj_kernel<false><<<n_jobs, h->tune[BSG_TUNE_FACTOR_THREADS], 0, st>>>(jd);
  if (df_products) sigma_cgemm_kernel<true><<<gc, 256, 0, st>>>(jd);
  else sigma_cgemm_kernel<false><<<gc, 256, 0, st>>>(jd);
  BSG_CUDA(cudaGetLastError());
  if (h->prof.on) BSG_TRY(h->prof.end(BSG_K_SIGMA, st, ev, work));
  return BSG_OK;
}

static int single_job(bsg_handle_t h, SigmaJob jb, cudaStream_t st) {
  const size_t ws = sigma_ws_bytes(jb.Mr);
  BSG_TRY(h->sigma_ws.ensure(ws + sizeof(SigmaJob) + 512));
  char* base = reinterpret_cast<char*>(h->sigma_ws.ptr);
  jb.ws = reinterpret_cast<double*>(base);
  jb.status = reinterpret_cast<int*>(base + ws);
  BSG_CUDA(cudaMemsetAsync(jb.status, 0, 4, st));
  void* jd = base + ws + 256;
  BSG_TRY(h->host_stage.ensure(sizeof(SigmaJob)));
  // the job struct goes through pinned staging; sync before reuse is done by
  // the staging owner (the next planning call synchronises the stream)
  BSG_CUDA(cudaStreamSynchronize(st));
  std::memcpy(h->host_stage.ptr, &jb, sizeof(SigmaJob));
  return launch_sigma_jobs(h, reinterpret_cast<SigmaJob*>(h->host_stage.ptr), 1, jd, st, false);
}

}  // namespace bsg

using namespace bsg;

extern "C" int bsg_site_sigma(bsg_handle_t h, const double* S_l, int m_l, const double* S_r, int M_r, double* Sigma,
                              double* Z, bsg_stream_t stream) {
  BSG_CHECK_ARG(h, "bsg_site_sigma: null handle");
  BSG_CHECK_ARG(S_r && Sigma && Z, "bsg_site_sigma: null pointer");
  BSG_CHECK_ARG(M_r >= 1 && M_r <= 1024, "bsg_site_sigma: M_r=%d outside [1, 1024]", M_r);
  BSG_CHECK_ARG(m_l == 0 || m_l == M_r - 1, "bsg_site_sigma: m_l=%d must be 0 or M_r-1=%d", m_l, M_r - 1);
  BSG_CHECK_ARG(m_l == 0 || S_l, "bsg_site_sigma: S_l is NULL");
  BSG_CUDA(cudaSetDevice(h->device));
  SigmaJob jb{};
  jb.S_l = m_l ? S_l : nullptr;
  jb.S_r = S_r;
  jb.ld_l = 2 * m_l;
  jb.ld_r = 2 * M_r;
  jb.m_l = m_l;
  jb.Mr = M_r;
  jb.first = 0;
  jb.Sigma = reinterpret_cast<double2*>(Sigma);
  jb.Z = Z;
  return single_job(h, jb, reinterpret_cast<cudaStream_t>(stream));
}

extern "C" int bsg_first_sigma(bsg_handle_t h, const double* S_0, int M, const double* sq_cov, double* Sigma,
                               double* Z, bsg_stream_t stream) {
  BSG_CHECK_ARG(h, "bsg_first_sigma: null handle");
  BSG_CHECK_ARG(sq_cov && Sigma && Z && (S_0 || M == 1), "bsg_first_sigma: null pointer");
  BSG_CHECK_ARG(M >= 1 && M <= 1024, "bsg_first_sigma: M=%d outside [1, 1024]", M);
  BSG_CUDA(cudaSetDevice(h->device));
  SigmaJob jb{};
  jb.S_l = M > 1 ? S_0 : nullptr;
  jb.S_r = sq_cov;
  jb.ld_l = 2 * (M - 1);
  jb.ld_r = 2 * M;
  jb.m_l = M - 1;
  jb.Mr = M;
  jb.first = 1;
  jb.Sigma = reinterpret_cast<double2*>(Sigma);
  jb.Z = Z;
  return single_job(h, jb, reinterpret_cast<cudaStream_t>(stream));
}

// ---------------------------------------------------------------------------
// Allocation-free variant of bsg_site_sigma.
//
// Some callers cannot call cudaMalloc: code that runs while another allocator
// has reserved the device's memory for itself (a caching allocator or a
// serving runtime that owns all of HBM), latency-critical loops that must not
// pay the implicit device synchronisation of cudaMalloc/cudaFree, and plug-in
// hosts that forbid raw device allocation.  bsg_site_sigma_noalloc serves
// them: its scratch (a status word and the Gauss-Jordan workspace) is the
// file-scope device array below, sized for M_r <= 160 modes; the job
// descriptor is a kernel parameter.  Every GPU that loads this library holds
// the array until the process exits.  The array's device address is looked
// up once per device and kept, so the entry point does not survive a
// cudaDeviceReset of that device (the array may move).
// ---------------------------------------------------------------------------
namespace bsg {
constexpr int kNoAllocMaxModes = 160;
constexpr size_t kNoAllocStatusOff = 0;
constexpr size_t kNoAllocWsOff = 256;
constexpr size_t kNoAllocBytes = kNoAllocWsOff + 112ull * kNoAllocMaxModes * kNoAllocMaxModes + 256;  // ~2.75 MiB
constexpr int kNoAllocMaxDevices = 64;
static __device__ __align__(256) unsigned char g_noalloc_sigma_scratch[kNoAllocBytes];
static std::mutex g_noalloc_mu;
static char* g_noalloc_ptr[kNoAllocMaxDevices] = {};
}  // namespace bsg

extern "C" int bsg_site_sigma_noalloc(const double* S_l, int m_l, const double* S_r, int M_r, double* Sigma,
                                      double* Z, bsg_stream_t stream) {
  BSG_CHECK_ARG(S_r && Sigma && Z, "bsg_site_sigma_noalloc: null pointer");
  if (M_r < 1 || M_r > kNoAllocMaxModes) {
    set_error("bsg_site_sigma_noalloc: M_r=%d outside [1, %d], the modes its fixed scratch holds; use bsg_site_sigma",
              M_r, kNoAllocMaxModes);
    return BSG_ERR_LIMIT;
  }
  BSG_CHECK_ARG(m_l == 0 || m_l == M_r - 1, "bsg_site_sigma_noalloc: m_l=%d must be 0 or M_r-1=%d", m_l, M_r - 1);
  BSG_CHECK_ARG(m_l == 0 || S_l, "bsg_site_sigma_noalloc: S_l is NULL");
  int dev = 0;
  BSG_CUDA(cudaGetDevice(&dev));
  BSG_CHECK_ARG(dev >= 0 && dev < kNoAllocMaxDevices, "bsg_site_sigma_noalloc: device %d out of range", dev);
  char* base = nullptr;
  {
    // one-time set-up per device, with that device current: the device
    // address of the scratch array (its host-side name is only a stand-in)
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
      void* p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_sigma_scratch);
      if (e != cudaSuccess || !p) {
        set_error("bsg_site_sigma_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
        return BSG_ERR_CUDA;
      }
      g_noalloc_ptr[dev] = static_cast<char*>(p);
    }
    base = g_noalloc_ptr[dev];
  }
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  SigmaJob jb{};
  jb.S_l = m_l ? S_l : nullptr;
  jb.S_r = S_r;
  jb.ld_l = 2 * m_l;
  jb.ld_r = 2 * M_r;
  jb.m_l = m_l;
  jb.Mr = M_r;
  jb.first = 0;
  jb.Sigma = reinterpret_cast<double2*>(Sigma);
  jb.Z = Z;
  jb.ws = reinterpret_cast<double*>(base + kNoAllocWsOff);
  jb.status = reinterpret_cast<int*>(base + kNoAllocStatusOff);
  // the status word must start at zero; the workspace is fully overwritten
  BSG_CUDA(cudaMemsetAsync(base + kNoAllocStatusOff, 0, 4, st));
  sigma_kernel<<<1, 1024, 0, st>>>(jb);
  BSG_CUDA(cudaGetLastError());
  return BSG_OK;
}
