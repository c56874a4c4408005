// Per-cut Schmidt spectra: Williamson decomposition of the right block of each
// cut and the top-chi product-thermal weights with their Fock labels.
//
// Reference: williamson + get_cumsum_kron (kron_cpu.py:46-127; the CuPy twin
// distributed_kron.py:105-137).  One CTA per cut; a call launches its cuts
// in one range, the whole-MPS build in two ranges on two streams.
//
// Williamson (FP64):  V = L L^T (Cholesky);  G = L^{-1} Omega L^{-T} is
// antisymmetric with eigenvalues +-i/nu;  H = G^T G has eigenvalues 1/nu^2
// (each twice).  Cyclic Jacobi (round-robin parallel order, one 2x2 block per
// thread) diagonalises H; eigenvectors x are paired with y = G x/|G x| by
// Gram-Schmidt so that y^T G x = 1/nu.  Then S = L [y_i | x_i] nu_i^{-1/2}
// satisfies V = S diag(nu, nu) S^T and S Omega S^T = Omega -- a Williamson
// symplectic like the reference's (it differs from scipy's Schur-based one by
// a symplectic-orthogonal gauge per mode, which no physical output sees).
// Modes are ordered by nu descending.
//
// Truncation: the reference keeps the 1e5 largest products per step and the
// chi largest at the end.  Every factor is <= 1, so a product outside the top
// chi at some step has >= chi products above it whose best extensions
// dominate all of its extensions: keeping the top chi per step gives the same
// final set (up to exact ties).  Candidates res[i] * t[n] form a matrix sorted
// along both axes; each candidate's rank is found with d binary searches, so
// the top chi come out already sorted (ties broken by the flattened index
// i*d + n, the outer-product order of the reference).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "bsg_df.cuh"
#include "bsg_internal.h"

namespace bsg {

constexpr int kMaxCutModes = 256;  // modes in one cut's right block


__device__ double block_max(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < (int)(blockDim.x + 31) / 32; ++i) s = fmax(s, red[i]);
    red[32] = s;
  }
  __syncthreads();
  return red[32];
}

__device__ double block_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0) {
    for (int i = 0; i < (int)(blockDim.x + 31) / 32; ++i) s += red[i];
    red[32] = s;
  }
  __syncthreads();
  return red[32];
}

// Cyclic Jacobi on the symmetric m x m matrix Hm (shared or global memory;
// row stride ld, odd in shared memory so that the scattered rows of a
// rotation round fall in different banks), rows of QT accumulating the eigenvectors (QT <- J^T QT).  Round-robin
// order: n/2 disjoint rotations per step, each updating whole 2x2 blocks of
// J1^T B J2 (and the transposed block), so a step needs two barriers.  The
// rotation angles and the convergence sums run in T (FP32 for the FP32
// sweeps); warps take rows of the pair triangle and of QT, lanes their
// columns, so no thread divides an index.  Returns the number of sweeps, or
// -1 if max_sweeps did not converge.
template <class T>
__device__ __noinline__ int block_jacobi(T* Hm, int m, int ld, T* QT, int max_sweeps, double tol, double* red, T* cs, T* sn,
                                         int* pos) {
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
  const int P = m / 2;
  for (int sweep = 0; sweep < max_sweeps; ++sweep) {
    T off = T(0), dia = T(0);
    for (int i = warp; i < m; i += nw)
      for (int j = lane; j < m; j += 32) {
        const T h = Hm[(size_t)i * ld + j];
        if (i < j) off += h * h;
        else if (i == j) dia += h * h;
      }
    const double offs = block_sum(double(off), red);
    const double dias = block_sum(double(dia), red);
    if (offs <= tol * dias) return sweep;
    for (int step = 0; step < m - 1; ++step) {
      // round-robin pairing of this step: slot i holds index pos(i)
      auto pos_at = [&](int i) {  // (i - 1 + step) mod (m - 1), both terms below m - 1
        if (i == 0) return 0;
        const int v = i - 1 + step;
        return (v >= m - 1 ? v - (m - 1) : v) + 1;
      };
      for (int q0 = tid; q0 < P; q0 += nt) {
        int p = pos_at(q0), q = pos_at(m - 1 - q0);
        if (p > q) {
          const int x = p;
          p = q;
          q = x;
        }
        const T hpq = Hm[(size_t)p * ld + q];
        const T skip = sizeof(T) == 8 ? T(1e-17) : T(1e-8);
        T c_ = T(1), s_ = T(0);
        const T hpp = Hm[(size_t)p * ld + p], hqq = Hm[(size_t)q * ld + q];
        if (fabs(hpq) > T(1e-30) && fabs(hpq) > skip * sqrt(fabs(hpp * hqq))) {
          const T th = (hqq - hpp) / (T(2) * hpq);
          const T tt = (th >= T(0) ? T(1) : T(-1)) / (fabs(th) + sqrt(th * th + T(1)));
          c_ = T(1) / sqrt(tt * tt + T(1));
          s_ = tt * c_;
        }
        cs[q0] = c_;
        sn[q0] = s_;
        pos[q0] = p;
        pos[P + q0] = q;
      }
      __syncthreads();
      // 2 x 2 blocks (m1 <= m2) of the two-sided update, upper triangle of
      // pairs.  A pair whose rotation was skipped (c = 1, s = 0) leaves its
      // rows and columns unchanged (exactly), so a block of two such pairs is
      // not touched: once only the clustered pairs still rotate, a round
      // costs their rows and columns only.  The diagonal block of every pair
      // is written (a skipped pair's negligible h_pq becomes 0).
      for (int m2 = warp; m2 < P; m2 += nw) {
        const int p2 = pos[m2], q2 = pos[P + m2];
        const T c2 = cs[m2], s2 = sn[m2];
        for (int m1 = lane; m1 <= m2; m1 += 32) {
          const T c1 = cs[m1], s1 = sn[m1];
          if (s1 == T(0) && s2 == T(0) && m1 != m2) continue;
          const int p1 = pos[m1], q1 = pos[P + m1];
          const T b00 = Hm[(size_t)p1 * ld + p2], b01 = Hm[(size_t)p1 * ld + q2];
          const T b10 = Hm[(size_t)q1 * ld + p2], b11 = Hm[(size_t)q1 * ld + q2];
          const T r00 = c1 * b00 - s1 * b10, r01 = c1 * b01 - s1 * b11;
          const T r10 = s1 * b00 + c1 * b10, r11 = s1 * b01 + c1 * b11;
          const T o00 = c2 * r00 - s2 * r01;
          T o01 = s2 * r00 + c2 * r01;
          T o10 = c2 * r10 - s2 * r11;
          const T o11 = s2 * r10 + c2 * r11;
          if (m1 == m2) {
            o01 = T(0);
            o10 = T(0);
          }
          Hm[(size_t)p1 * ld + p2] = o00;
          Hm[(size_t)p1 * ld + q2] = o01;
          Hm[(size_t)q1 * ld + p2] = o10;
          Hm[(size_t)q1 * ld + q2] = o11;
          if (m1 != m2) {
            Hm[(size_t)p2 * ld + p1] = o00;
            Hm[(size_t)q2 * ld + p1] = o01;
            Hm[(size_t)p2 * ld + q1] = o10;
            Hm[(size_t)q2 * ld + q1] = o11;
          }
        }
      }
      for (int q0 = warp; q0 < P; q0 += nw) {
        const T c_ = cs[q0], s_ = sn[q0];
        if (s_ == T(0)) continue;  // the identity
        const int p = pos[q0], q = pos[P + q0];
        T* rp = QT + (size_t)p * m;
        T* rq = QT + (size_t)q * m;
        for (int j = lane; j < m; j += 32) {
          const T hp = rp[j], hq = rq[j];
          rp[j] = c_ * hp - s_ * hq;
          rq[j] = s_ * hp + c_ * hq;
        }
      }
      __syncthreads();
    }
  }
  return -1;
}

// ---- double-float products for the eigenvector refinement ------------------
// GB300's FP64 pipe runs ~1/73 of the FP32 rate, so the refinement's m x m
// products run as double-float arithmetic on the FP32 pipe: each FP64
// operand is split into an FP32 pair (hi + lo), each product term is formed
// with an exact FP32 product error (fma) plus the cross terms, and the sum
// is kept as an FP32 sum s with its exact rounding errors collected in t
// (Dekker / Knuth two-sum).  A term carries ~2^-48 relative error, a sum of
// m terms ~2^-48 sqrt(m) of sum |a b| -- ~1e-14 of the norm here, far below
// what the refinement needs to stop (corrections <= 1e-8, clustered
// numerators <= 1e-12 of the norm).
constexpr int kDfTile = 32;
constexpr int kDfLd = kDfTile + 2;  // float2 row stride of the tiles (16-byte aligned rows)
constexpr size_t kDfSmemBytes = 2 * kDfTile * kDfLd * sizeof(float2);

// C[i][j] = add[i][j] + sign * sum_q A(i, q) B(q, j) (+ diag where i == j),
// all m x m row-major, A(i, q) = ta ? A[q][i] : A[i][q], B(q, j) = tb ? B[j][q]
// : B[q][j].  sym: the result is symmetric -- only tiles on or above the
// diagonal are computed and mirrored.  b_upper: B(q, j) = 0 for q > j (B is
// the transpose of a lower-triangular factor), so the K loop of a column
// tile stops after its diagonal tile.  C must not alias A, B or add unless
// add == C (each entry of C is read before it is written, by the same
// thread).  tiles: kDfSmemBytes of shared memory.  Block-wide (barriers).
// NT threads (256, 512 or 1024): 32 x 32 output tiles, each thread a 2 x 2
// block of one of NT / 256 K groups (so every shared-memory load feeds two
// products and four accumulations run side by side); the groups' partial
// sums are added in a tree through shared memory at the end of a tile.
template <int NT>
__device__ __noinline__ void df_gemm_t(const double* A, bool ta, const double* B, bool tb, const double* add,
                                       double sign, double diag, double* C, int m, bool sym, float2* tiles,
                                       bool b_upper) {
  constexpr int G = NT / 256, KG = kDfTile / G, PER = kDfTile * kDfTile / NT;
  float2 (*As)[kDfLd] = reinterpret_cast<float2 (*)[kDfLd]>(tiles);  // [k][row]
  float2 (*Bs)[kDfLd] = reinterpret_cast<float2 (*)[kDfLd]>(tiles + kDfTile * kDfLd);  // [k][col]
  const int tid = threadIdx.x, g = tid >> 8, l = tid & 255, tx = l & 15, ty = l >> 4;
  const int nb = (m + kDfTile - 1) / kDfTile;
  // element e of a chunk: (row or column r, k c), consecutive threads along
  // the operand's contiguous index
  auto a_at = [&](int ti, int q0, int e, int& r, int& c) {
    if (ta) {
      r = e % kDfTile;
      c = e / kDfTile;
    } else {
      r = e / kDfTile;
      c = e % kDfTile;
    }
    const int ai = ti * kDfTile + r, aq = q0 + c;
    if (ai >= m || aq >= m) return 0.0;
    return ta ? A[(size_t)aq * m + ai] : A[(size_t)ai * m + aq];
  };
  auto b_at = [&](int tj, int q0, int e, int& r, int& c) {
    if (tb) {
      c = e % kDfTile;
      r = e / kDfTile;
    } else {
      c = e / kDfTile;
      r = e % kDfTile;
    }
    const int bq = q0 + c, bj = tj * kDfTile + r;
    if (bq >= m || bj >= m) return 0.0;
    return tb ? B[(size_t)bj * m + bq] : B[(size_t)bq * m + bj];
  };
  for (int ti = 0; ti < nb; ++ti)
    for (int tj = sym ? ti : 0; tj < nb; ++tj) {
      float s[4] = {0.f, 0.f, 0.f, 0.f}, t[4] = {0.f, 0.f, 0.f, 0.f};
      const int qend = b_upper ? min(m, (tj + 1) * kDfTile) : m;
      // the K chunk q0 is in registers while chunk q0 - 32 is multiplied
      double pa[PER], pb[PER];
      int r, c;
#pragma unroll
      for (int o = 0; o < PER; ++o) {
        pa[o] = a_at(ti, 0, tid + o * NT, r, c);
        pb[o] = b_at(tj, 0, tid + o * NT, r, c);
      }
      for (int q0 = 0; q0 < qend; q0 += kDfTile) {
#pragma unroll
        for (int o = 0; o < PER; ++o) {
          const int e = tid + o * NT;
          if (ta) {
            r = e % kDfTile;
            c = e / kDfTile;
          } else {
            r = e / kDfTile;
            c = e % kDfTile;
          }
          As[c][r] = df_split(pa[o]);
          if (tb) {
            c = e % kDfTile;
            r = e / kDfTile;
          } else {
            c = e / kDfTile;
            r = e % kDfTile;
          }
          Bs[c][r] = df_split(pb[o]);
        }
        __syncthreads();
        if (q0 + kDfTile < qend) {
#pragma unroll
          for (int o = 0; o < PER; ++o) {
            pa[o] = a_at(ti, q0 + kDfTile, tid + o * NT, r, c);
            pb[o] = b_at(tj, q0 + kDfTile, tid + o * NT, r, c);
          }
        }
#pragma unroll
        for (int kk = g * KG; kk < (g + 1) * KG; ++kk) {
          const float4 a = *reinterpret_cast<const float4*>(&As[kk][2 * ty]);
          const float4 b = *reinterpret_cast<const float4*>(&Bs[kk][2 * tx]);
          const float2 a0 = make_float2(a.x, a.y), a1 = make_float2(a.z, a.w);
          const float2 b0 = make_float2(b.x, b.y), b1 = make_float2(b.z, b.w);
          df_mac(s[0], t[0], a0, b0);
          df_mac(s[1], t[1], a0, b1);
          df_mac(s[2], t[2], a1, b0);
          df_mac(s[3], t[3], a1, b1);
        }
        __syncthreads();
      }
      // K groups: tree sum through shared memory (the tiles are free now)
      float2* red = tiles;
#pragma unroll
      for (int step = G / 2; step >= 1; step /= 2) {
        if (g >= step && g < 2 * step)
#pragma unroll
          for (int u = 0; u < 4; ++u) red[((g - step) * 256 + l) * 4 + u] = df_norm(s[u], t[u]);
        __syncthreads();
        if (g < step)
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const float2 v = red[(g * 256 + l) * 4 + u];
            const float w = s[u] + v.x;
            const float bb = w - s[u];
            t[u] += v.y + ((s[u] - (w - bb)) + (v.x - bb));
            s[u] = w;
          }
        __syncthreads();
      }
      if (g == 0)
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int i = ti * kDfTile + 2 * ty + (u >> 1), j = tj * kDfTile + 2 * tx + (u & 1);
          if (i >= m || j >= m) continue;
          double v = sign * (double(s[u]) + double(t[u]));
          if (add) v += add[(size_t)i * m + j];
          if (i == j) v += diag;
          C[(size_t)i * m + j] = v;
          // off-diagonal tiles are mirrored; a diagonal tile computes both halves itself
          if (sym && tj != ti) C[(size_t)j * m + i] = v;
        }
    }
  __syncthreads();
}

// The same tiling in FP64 (2 x 2 blocks per thread, NT / 256 K groups; the
// tiles hold doubles): for the few products whose results must keep FP64
// accuracy.
template <int NT>
__device__ __noinline__ void f64_gemm_t(const double* A, bool ta, const double* B, bool tb, const double* add,
                                        double sign, double diag, double* C, int m, bool sym, float2* tiles) {
  constexpr int G = NT / 256, KG = kDfTile / G, PER = kDfTile * kDfTile / NT;
  double (*As)[kDfLd] = reinterpret_cast<double (*)[kDfLd]>(tiles);
  double (*Bs)[kDfLd] = reinterpret_cast<double (*)[kDfLd]>(tiles + kDfTile * kDfLd);
  double* red = reinterpret_cast<double*>(tiles);
  const int tid = threadIdx.x, g = tid >> 8, l = tid & 255, tx = l & 15, ty = l >> 4;
  const int nb = (m + kDfTile - 1) / kDfTile;
  for (int ti = 0; ti < nb; ++ti)
    for (int tj = sym ? ti : 0; tj < nb; ++tj) {
      double sd[4] = {0.0, 0.0, 0.0, 0.0};
      for (int q0 = 0; q0 < m; q0 += kDfTile) {
#pragma unroll
        for (int o = 0; o < PER; ++o) {
          const int e = tid + o * NT;
          int r, c;
          if (ta) {
            r = e % kDfTile;
            c = e / kDfTile;
          } else {
            r = e / kDfTile;
            c = e % kDfTile;
          }
          const int ai = ti * kDfTile + r, aq = q0 + c;
          As[c][r] = (ai < m && aq < m) ? (ta ? A[(size_t)aq * m + ai] : A[(size_t)ai * m + aq]) : 0.0;
          if (tb) {
            c = e % kDfTile;
            r = e / kDfTile;
          } else {
            c = e / kDfTile;
            r = e % kDfTile;
          }
          const int bq = q0 + c, bj = tj * kDfTile + r;
          Bs[c][r] = (bq < m && bj < m) ? (tb ? B[(size_t)bj * m + bq] : B[(size_t)bq * m + bj]) : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int kk = g * KG; kk < (g + 1) * KG; ++kk) {
          const double a0 = As[kk][2 * ty], a1 = As[kk][2 * ty + 1], b0 = Bs[kk][2 * tx], b1 = Bs[kk][2 * tx + 1];
          sd[0] = fma(a0, b0, sd[0]);
          sd[1] = fma(a0, b1, sd[1]);
          sd[2] = fma(a1, b0, sd[2]);
          sd[3] = fma(a1, b1, sd[3]);
        }
        __syncthreads();
      }
      for (int gg = 1; gg < G; ++gg) {  // K groups added in group order
        if (g == gg)
#pragma unroll
          for (int u = 0; u < 4; ++u) red[l * 4 + u] = sd[u];
        __syncthreads();
        if (g == 0)
#pragma unroll
          for (int u = 0; u < 4; ++u) sd[u] += red[l * 4 + u];
        __syncthreads();
      }
      if (g == 0)
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int i = ti * kDfTile + 2 * ty + (u >> 1), j = tj * kDfTile + 2 * tx + (u & 1);
          if (i >= m || j >= m) continue;
          double v = sign * sd[u];
          if (add) v += add[(size_t)i * m + j];
          if (i == j) v += diag;
          C[(size_t)i * m + j] = v;
          if (sym && tj != ti) C[(size_t)j * m + i] = v;
        }
    }
  __syncthreads();
}

// The same block-wide product in FP64 (tiles: kDfSmemBytes, holding doubles).
__device__ void f64_gemm(const double* A, bool ta, const double* B, bool tb, const double* add, double sign,
                         double diag, double* C, int m, bool sym, float2* tiles) {
  if (blockDim.x >= 1024) f64_gemm_t<1024>(A, ta, B, tb, add, sign, diag, C, m, sym, tiles);
  else if (blockDim.x >= 512) f64_gemm_t<512>(A, ta, B, tb, add, sign, diag, C, m, sym, tiles);
  else f64_gemm_t<256>(A, ta, B, tb, add, sign, diag, C, m, sym, tiles);
}

__device__ void df_gemm(const double* A, bool ta, const double* B, bool tb, const double* add, double sign,
                        double diag, double* C, int m, bool sym, float2* tiles, bool b_upper = false) {
  if (blockDim.x >= 1024) df_gemm_t<1024>(A, ta, B, tb, add, sign, diag, C, m, sym, tiles, b_upper);
  else if (blockDim.x >= 512) df_gemm_t<512>(A, ta, B, tb, add, sign, diag, C, m, sym, tiles, b_upper);
  else df_gemm_t<256>(A, ta, B, tb, add, sign, diag, C, m, sym, tiles, b_upper);
}

// Mixed-precision symmetric eigen-decomposition of the m x m matrix Hm with
// eigenvector rows in QT: FP32 Jacobi sweeps on a rounded copy (the FP32
// pipe is ~64x the FP64 one on GB300) until the off-diagonal is ~1e-5 of the
// diagonal, then iterative refinement by matrix products only -- double-float
// products on the FP32 pipe (df_gemm), FP64 everywhere else (Ogita &
// Aishima, "Iterative refinement for symmetric eigenvalue decomposition",
// Japan J. Indust. Appl. Math. 35 (2018)).  With X the eigenvector columns
// (X = QT^T):
//   R = I - X^T X,  S = X^T Hm X,  lambda_i = s_ii / (1 - r_ii),
//   E_ij = (s_ij + lambda_j r_ij) / (lambda_j - lambda_i)  if |lambda_i - lambda_j| > delta,
//          r_ij / 2                                        otherwise (clusters, incl. i = j),
//   X <- X + X E,   delta = 2 (||S - diag(lambda)||_F + ||Hm||_F ||R||_F).
// Each step squares the error; clustered eigenvalues (every eigenvalue of
// G^T G is double) converge as an orthonormal basis of their subspace, which
// the pairing step resolves.  On return the diagonal of Hm holds the
// eigenvalues (the rest of Hm is overwritten).  s1, s2, s3: m*m doubles of
// scratch each.  Returns the FP32 sweeps used, or -1 if they did not reach
// the start tolerance of the refinement.
__device__ __noinline__ int mixed_jacobi(double* Hm, int m, double* QT, double* s1, double* s2, double* s3, double* s4,
                            double* red, double* cs, double* sn, int* pos, float* jsm, bool q_smem, float2* dft,
                            unsigned long long* sweep_log) {
  const int tid = threadIdx.x, nt = blockDim.x;
  const size_t mm = (size_t)m * m;
  // the FP32 copies: in shared memory when the launch reserved room for them
  // (the rotation rounds touch scattered rows and columns), else in s1
  // (the scattered 2 x 2 blocks of a rotation round are the shared-memory
  // win; the eigenvector rows are updated row-wise, coalesced, so for large
  // m only the matrix stays in shared memory)
  float* H32 = jsm ? jsm : reinterpret_cast<float*>(s1);
  const int ld = jsm ? m + 1 : m;  // s1 holds 2 m^2 floats
  float* Q32 = jsm ? (q_smem ? H32 + (size_t)m * ld : reinterpret_cast<float*>(s1)) : H32 + mm;
  const int lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
  for (int i = warp; i < m; i += nw)
    for (int j = lane; j < m; j += 32) {
      H32[(size_t)i * ld + j] = float(Hm[(size_t)i * m + j]);
      Q32[(size_t)i * m + j] = i == j ? 1.f : 0.f;
    }
  __syncthreads();
  unsigned long long t32 = 0;
  if (sweep_log && tid == 0) asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t32));
  const int sw32 =
      block_jacobi<float>(H32, m, ld, Q32, 24, 1e-10, red, reinterpret_cast<float*>(cs), reinterpret_cast<float*>(sn), pos);
  if (sweep_log && tid == 0) {
    unsigned long long t1;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t1));
    sweep_log[2] = t1 - t32;
  }
  for (size_t t = tid; t < mm; t += nt) {
    const double q = double(Q32[t]);
    QT[t] = q;
    s4[t] = q;  // kept for an FP64 restart
  }
  __syncthreads();
  double* lam = reinterpret_cast<double*>(cs);  // m doubles (cs and sn are adjacent: 2 kMaxCutModes)
  double anorm = 0.0;
  for (size_t t = tid; t < mm; t += nt) anorm += Hm[t] * Hm[t];
  anorm = sqrt(block_sum(anorm, red));
  // Ogita-Aishima steps until a step's largest off-diagonal correction is
  // at most 1e-8: each step squares the eigenvector error of every eigenvalue
  // gap above its cluster threshold, so after such a step the error is at
  // rounding level.  The FP32 start mixes nearly degenerate eigenvalues
  // (relative gaps ~1e-6, near-vacuum modes of middle cuts) by a few percent,
  // which three fixed steps left at ~1e-6.
  constexpr int kRefineMax = 8;
  int refined = 0;
  bool converged = false, settled = false;
  // pairs closer than tau_gap stay clustered (the FP32 start cannot separate
  // them, and a Newton step on an O(1) mixing diverges); unresolved clusters
  // are diagonalised at the end in FP64 on their own small blocks
  const double tau_gap = 1e-6 * anorm;
  double delta_last = 0.0;
  // profiling: time in the refinement's products and in the whole refinement
  unsigned long long t_ref0 = 0, t_gemm = 0, t_g0 = 0;
  auto stamp = [&]() {
    unsigned long long t = 0;
    if (sweep_log && tid == 0) asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
  };
  t_ref0 = stamp();
  for (int it = 0; it < kRefineMax; ++it) {
    // s2 = T = Hm QT^T, s1 = R = I - QT QT^T, s3 = S = QT T = QT Hm QT^T
    // (double-float products on the FP32 pipe; R and S symmetric)
    t_g0 = stamp();
    df_gemm(Hm, false, QT, true, nullptr, 1.0, 0.0, s2, m, false, dft);
    df_gemm(QT, false, QT, true, nullptr, -1.0, 1.0, s1, m, true, dft);
    df_gemm(QT, false, s2, false, nullptr, 1.0, 0.0, s3, m, true, dft);
    t_gemm += stamp() - t_g0;
    for (int i = tid; i < m; i += nt) lam[i] = s3[(size_t)i * m + i] / (1.0 - s1[(size_t)i * m + i]);
    __syncthreads();
    double so = 0.0, rr = 0.0;
    for (int i = warp; i < m; i += nw)
      for (int j = lane; j < m; j += 32) {
        const size_t t = (size_t)i * m + j;
        const double d = s3[t] - (i == j ? lam[i] : 0.0);
        so += d * d;
        rr += s1[t] * s1[t];
      }
    so = block_sum(so, red);
    rr = block_sum(rr, red);
    const double delta = 2.0 * (sqrt(so) + anorm * sqrt(rr));
    delta_last = delta;
    // s1 <- E (in place: E_ij reads s1_ij and s3_ij only).  cnum: the largest
    // numerator s_ij + lambda_j r_ij of a clustered pair -- rounding level for
    // an exactly degenerate pair, about gap x mixing for distinct eigenvalues
    // the clustering leaves unresolved
    double emax = 0.0, cnum = 0.0;
    for (int i = warp; i < m; i += nw)
      for (int j = lane; j < m; j += 32) {
        const size_t t = (size_t)i * m + j;
        const double r = s1[t], gap = lam[j] - lam[i];
        const bool sep = i != j && fabs(gap) > fmax(delta, tau_gap);
        const double e = sep ? (s3[t] + lam[j] * r) / gap : 0.5 * r;
        s1[t] = e;
        if (i != j) emax = fmax(emax, fabs(e));
        if (i != j && !sep) cnum = fmax(cnum, fabs(s3[t] + lam[j] * r));
      }
    emax = block_max(emax, red);
    cnum = block_max(cnum, red);
    // s2 = QT + E^T QT, then QT = s2
    t_g0 = stamp();
    df_gemm(s1, true, QT, false, QT, 1.0, 0.0, s2, m, false, dft);
    t_gemm += stamp() - t_g0;
    for (size_t t = tid; t < mm; t += nt) QT[t] = s2[t];
    __syncthreads();
    refined = it + 1;
    if (emax <= 1e-8) {  // the remaining error is ~emax^2
      settled = true;
      converged = cnum <= 1e-12 * anorm;
      break;
    }
  }
  if (settled && !converged && m <= kMaxCutModes) {  // (lam fills cs; sn is free for the small Jacobi)
    // Clusters (eigenvalues chained by gaps <= max(delta, tau_gap), in sorted
    // order) whose vectors are an orthonormal basis of their eigenspace but
    // still mixed.  S = QT Hm QT^T once (FP64, tiled);
    // for each cluster its p x p block (shared memory, odd stride, when it
    // fits in the FP32 Jacobi area: free now) by cyclic FP64 Jacobi, the
    // rotations gathered into a block-diagonal R (identity outside the
    // clusters) and QT <- R QT in one product.  The rotation scratch of the
    // small Jacobi is sn / pos + 256, so lam (cs) and the sorted order (pos)
    // survive.
    __shared__ int s_g0, s_g1;
    int* ord = pos;
    for (int i = tid; i < m; i += nt) {
      const double li = lam[i];
      int r = 0;
      for (int j = 0; j < m; ++j) r += (lam[j] < li) || (lam[j] == li && j < i);
      ord[r] = i;
    }
    if (tid == 0) s_g1 = 0;
    // S in FP64: the eigenvalues of a cluster of K near 1 carry a small nbar
    // in 1 - mu, which double-float products would blur
    f64_gemm(Hm, false, QT, true, nullptr, 1.0, 0.0, s2, m, false, dft);  // T = Hm QT^T
    f64_gemm(QT, false, s2, false, nullptr, 1.0, 0.0, s3, m, true, dft);  // S = QT T
    for (int i = warp; i < m; i += nw)
      for (int j = lane; j < m; j += 32) s2[(size_t)i * m + j] = i == j ? 1.0 : 0.0;  // R
    __syncthreads();
    const double chain = fmax(delta_last, tau_gap);
    const size_t jsm_bytes = jsm ? (size_t)m * (m + 1) * sizeof(float) : 0;  // the FP32 matrix area
    double* sblk = reinterpret_cast<double*>(jsm);
    double* rblk = s1;
    bool ok = true;
    while (true) {
      __syncthreads();  // every thread has read the previous cluster's bounds
      if (tid == 0) {
        int g0 = s_g1, g1 = g0 + 1;
        while (g1 < m && lam[ord[g1]] - lam[ord[g1 - 1]] <= chain) ++g1;
        s_g0 = g0;
        s_g1 = g1;
      }
      __syncthreads();
      const int g0 = s_g0, g1 = s_g1, p = g1 - g0;
      if (g0 >= m) break;
      if (p < 2) continue;
      const bool in_smem = (size_t)p * (p + 1) * sizeof(double) <= jsm_bytes;
      const int ldb = in_smem ? p + 1 : p;
      double* sb = in_smem ? sblk : s1 + (size_t)p * p;  // s1 holds 2 p^2 when p^2 <= m^2 / 2
      if (!in_smem && 2 * (size_t)p * p > (size_t)m * m) {  // no room: leave it to the restart
        ok = false;
        break;
      }
      for (int a = warp; a < p; a += nw)
        for (int b2 = lane; b2 < p; b2 += 32) {
          sb[(size_t)a * ldb + b2] = s3[(size_t)ord[g0 + a] * m + ord[g0 + b2]];
          rblk[(size_t)a * p + b2] = a == b2 ? 1.0 : 0.0;
        }
      __syncthreads();
      if (block_jacobi<double>(sb, p, ldb, rblk, 60, 1e-30, red, sn, sn + kMaxCutModes / 2, pos + 256) < 0) ok = false;
      for (int a = warp; a < p; a += nw) {
        for (int b2 = lane; b2 < p; b2 += 32) s2[(size_t)ord[g0 + a] * m + ord[g0 + b2]] = rblk[(size_t)a * p + b2];
        if (lane == 0) lam[ord[g0 + a]] = sb[(size_t)a * ldb + a];
      }
    }
    __syncthreads();
    if (ok) {
      df_gemm(s2, false, QT, false, nullptr, 1.0, 0.0, s3, m, false, dft);  // R QT
      for (size_t t = tid; t < mm; t += nt) QT[t] = s3[t];
      __syncthreads();
    }
    converged = ok;
  }
  if (sweep_log && tid == 0) {
    sweep_log[3] = t_gemm;
    sweep_log[4] = stamp() - t_ref0;
  }
  if (!converged) {
    // Eigenvalues closer than the FP32 start can separate (gaps ~1e-7 of the
    // norm: near-vacuum modes of cuts far from where the interferometer
    // couples, e.g. the banded M=216 workload's cuts 12 and up) come out of
    // the FP32 sweeps mixed by O(1): either the steps stop converging once
    // delta drops below their gap, or the mixed pair keeps delta above its
    // gap and stays a cluster (cnum above rounding).  Such a cut restarts
    // with FP64 Jacobi sweeps, which resolve any gap above the FP64 rounding
    // of Hm (still the input matrix), from the FP32 sweeps' eigenvector rows
    // X (s4) rather than the identity: X is made orthonormal to rounding by
    // two Newton-Schulz steps X <- (3 I - X X^T) X / 2 (its rows are
    // orthonormal to FP32 rounding, so each step squares ~1e-7), and the
    // sweeps run on X Hm X^T, whose off-diagonal is at FP32 rounding outside
    // the mixed clusters: ~4 sweeps instead of ~16 from the identity.  The
    // rotations act on X's rows, so QT ends as the eigenvector rows of Hm.
    // (The refined vectors are no start: a refinement that stopped
    // converging has left them far from orthonormal.)
    // (the steps in double-float: orthonormal to ~1e-14, far below the
    // pairing's tolerances; X Hm X^T below stays FP64 for the small nbar)
    for (int it = 0; it < 2; ++it) {
      df_gemm(s4, false, s4, true, nullptr, -0.5, 1.5, s1, m, true, dft);  // (3 I - X X^T) / 2
      df_gemm(s1, false, s4, false, nullptr, 1.0, 0.0, s2, m, false, dft);
      for (size_t t = tid; t < mm; t += nt) s4[t] = s2[t];
      __syncthreads();
    }
    f64_gemm(Hm, false, s4, true, nullptr, 1.0, 0.0, s2, m, false, dft);  // Hm X^T
    f64_gemm(s4, false, s2, false, nullptr, 1.0, 0.0, s3, m, true, dft);  // X Hm X^T
    for (size_t t = tid; t < mm; t += nt) {
      Hm[t] = s3[t];
      QT[t] = s4[t];
    }
    __syncthreads();
    const int sw64 = block_jacobi<double>(Hm, m, m, QT, 60, 1e-30, red, cs, sn, pos);
    if (sweep_log && tid == 0) {
      sweep_log[0] = (unsigned long long)(sw32 < 0 ? 99 : sw32);
      sweep_log[1] = 100 + (unsigned long long)(sw64 < 0 ? 99 : sw64);  // 100 + FP64 sweeps: the restart
    }
    __syncthreads();
    return sw64 < 0 ? -1 : (sw32 < 0 ? 0 : sw32);
  }
  for (int i = tid; i < m; i += nt) Hm[(size_t)i * m + i] = lam[i];
  if (sweep_log && tid == 0) {
    sweep_log[0] = (unsigned long long)(sw32 < 0 ? 99 : sw32);
    sweep_log[1] = (unsigned long long)refined;
  }
  __syncthreads();
  return sw32 < 0 ? -1 : sw32;
}

// In-place right-looking Cholesky of the m x m SPD matrix X (lower triangle,
// upper zeroed).  dinv, col: m doubles of shared memory each; dinv receives
// 1 / L_jj, col holds the scaled column of the current step, which the
// trailing update reads (warps take its rows, lanes their columns).
// Returns false if a pivot is not positive.
__device__ __noinline__ bool block_cholesky(double* X, int m, int* s_flag, double* dinv, double* col) {
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
  if (tid == 0) *s_flag = 0;
  __syncthreads();
  for (int j = 0; j < m; ++j) {
    if (tid == 0) {
      const double djj = X[(size_t)j * m + j];
      if (!(djj > 0.0)) *s_flag = 1;
      const double d = djj > 0.0 ? sqrt(djj) : 1.0;
      X[(size_t)j * m + j] = d;
      dinv[j] = 1.0 / d;
    }
    __syncthreads();
    if (*s_flag) return false;
    const double inv = dinv[j];
    for (int i = j + 1 + tid; i < m; i += nt) {
      const double v = X[(size_t)i * m + j] * inv;
      X[(size_t)i * m + j] = v;
      col[i] = v;
    }
    __syncthreads();
    for (int i = j + 1 + warp; i < m; i += nw) {
      const double xij = col[i];
      double* row = X + (size_t)i * m;
      for (int l = j + 1 + lane; l <= i; l += 32) row[l] -= xij * col[l];
    }
    __syncthreads();
  }
  for (int i = warp; i < m; i += nw)
    for (int l = i + 1 + lane; l < m; l += 32) X[(size_t)i * m + l] = 0.0;
  __syncthreads();
  return true;
}

// Phase timestamps of the Williamson kernel (profiling only): the global
// nanosecond timer at each phase boundary, taken as the latest of the warps'
// readings (lane 0 of each warp reads the timer and takes the maximum in
// shared memory before a barrier).  One thread's reading after a barrier
// does not mark the barrier: the compiler may schedule the timer read
// before it, so a thread that finished its share of a phase early would
// stamp the phase's end while other warps are still in it.  Called by every
// thread of the CTA (block-uniform; it holds a barrier when profiling).
__device__ __forceinline__ void phase_stamp(const CutArgs& a, int c, int i) {
  if (!a.phase_t) return;
  __shared__ unsigned long long s_pt[kCutTimedPhases];
  if (i == 0) {
    if (threadIdx.x < kCutTimedPhases) s_pt[threadIdx.x] = 0;
    __syncthreads();
  }
  if ((threadIdx.x & 31) == 0) {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    atomicMax(&s_pt[i], t);
  }
  __syncthreads();
  if (threadIdx.x == 0) a.phase_t[(size_t)c * kCutPhases + i] = s_pt[i];
}

// The Williamson decomposition of cut c of `a` by the whole CTA.
__device__ __forceinline__ void williamson_cut(const CutArgs& a, const int c) {
  const int L = a.L0 + c, M = a.M;
  const int k = M - L, n = 2 * k, nA = 2 * L;
  const int tid = threadIdx.x, nt = blockDim.x;
  const size_t nn = (size_t)n * n;
  double* A = a.ws + (size_t)c * a.ws_stride;  // V -> L (lower)
  double* W = A + nn;    // L^{-1}, later eigenvector rows
  double* Gm = W + nn;   // G = L^{-1} Omega L^{-T}
  double* H = Gm + nn;   // H (full path) / F and its reflectors (low-rank path) / accepted vectors
  double* X1 = H + nn;   // low-rank path: V_A -> L_A, then K = I - R R^T
  double* X2 = X1 + nn;  // low-rank path: L_A^{-1} C, then eigenvector rows of K
  // (X2 + nn, X2 + 2 nn: two more n^2 blocks of eigen-solver scratch; X2 + 3 nn:
  // the FP32 sweeps' eigenvectors, the start of an FP64 restart)
  double* MU = a.mu + (size_t)c * (2 * a.kmax);
  extern __shared__ double sm[];
  double* red = sm;                   // 33
  double* cs = red + 40;              // n/2
  double* sn = cs + kMaxCutModes;     // n/2
  int* pos = reinterpret_cast<int*>(sn + kMaxCutModes);  // n
  int* order = pos + 2 * kMaxCutModes;                   // n
  double* dots = reinterpret_cast<double*>(order + 2 * kMaxCutModes);  // n (also Householder taus)
  double* vec = dots + 2 * kMaxCutModes;                               // n
  double* vec2 = vec + 2 * kMaxCutModes;                               // n
  // double-float product tiles, then the FP32 Jacobi matrix (m (m + 1) floats)
  // and, with jac_q_smem, its eigenvector rows (m^2 floats)
  // when the launch reserved them
  float2* dft = reinterpret_cast<float2*>(vec2 + 2 * kMaxCutModes);
  float* jsm = a.jac_smem_m > 0 ? reinterpret_cast<float*>(reinterpret_cast<char*>(dft) + kDfSmemBytes) : nullptr;
  __shared__ int s_flag;
  __shared__ double s_scalar;
  __shared__ int s_pick[4], s_nb;  // blocked vacuum pairing: the block's candidates
  __shared__ float s_pickv[4];

  auto gidx = [&](int i) { return i < k ? L + i : M + L + (i - k); };
  phase_stamp(a, c, 0);
  // 1. V and the symmetry check of the reference (norm(V - V^T) < 1e-11)
  double asym = 0.0;
  const int lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
  for (int r = warp; r < n; r += nw)
    for (int q = lane; q < n; q += 32) {
      const double v = a.sq_cov[(size_t)gidx(r) * (2 * M) + gidx(q)];
      const double vt = a.sq_cov[(size_t)gidx(q) * (2 * M) + gidx(r)];
      A[(size_t)r * n + q] = v;
      asym += (v - vt) * (v - vt);
    }
  asym = block_sum(asym, red);
  if (asym >= 1e-22) {
    if (tid == 0) a.status[c] = 1;
    return;
  }
  phase_stamp(a, c, 1);
  // 2. Cholesky V = L L^T
  if (!block_cholesky(A, n, &s_flag, vec, vec2)) {
    if (tid == 0) a.status[c] = 2;
    return;
  }
  phase_stamp(a, c, 2);
  // 3. W = L^{-1}: forward substitution on all columns, row by row (1 / L_rr
  // in vec from the Cholesky; warps take rows, lanes columns)
  for (int i = warp; i < n; i += nw)
    for (int q = lane; q < n; q += 32) W[(size_t)i * n + q] = i == q ? 1.0 : 0.0;
  __syncthreads();
  for (int r = 0; r < n; ++r) {
    const double inv = vec[r];
    for (int q = tid; q <= r; q += nt) W[(size_t)r * n + q] *= inv;
    __syncthreads();
    const double* wr = W + (size_t)r * n;
    for (int i = r + 1 + warp; i < n; i += nw) {
      const double lir = A[(size_t)i * n + r];
      double* wi = W + (size_t)i * n;
      for (int q = lane; q <= r; q += 32) wi[q] -= lir * wr[q];
    }
    __syncthreads();
  }
  phase_stamp(a, c, 3);
  // 4. G = W Omega W^T (formed in the full path only; the low-rank path
  // applies it as two triangular products with W = L^{-1})
  int sweeps = 0;
  const bool g_dense = nA >= n;
  double* EV = g_dense ? W : X1;  // eigenvector rows of H
  if (g_dense) {
    // G[i][j] = sum_{r<k} W[i][r] W[j][r+k] - W[i][r+k] W[j][r] = sum_q W[i][q] Wp[j][q]
    // with Wp[j][q] = (Omega W^T)[q][j] = q < k ? W[j][q+k] : -W[j][q-k] (in X1),
    // a double-float product
    for (int i = warp; i < n; i += nw)
      for (int q = lane; q < n; q += 32)
        X1[(size_t)i * n + q] = q < k ? W[(size_t)i * n + q + k] : -W[(size_t)i * n + q - k];
    __syncthreads();
    df_gemm(W, false, X1, true, nullptr, 1.0, 0.0, Gm, n, false, dft);
    phase_stamp(a, c, 4);
    // 5a. full path: H = G^T G (double-float, symmetric), Jacobi with
    // eigenvector rows in W
    df_gemm(Gm, true, Gm, false, nullptr, 1.0, 0.0, H, n, true, dft);
    phase_stamp(a, c, 5);
    sweeps = mixed_jacobi(H, n, W, X1, X2, X2 + nn, X2 + 3 * nn, red, cs, sn, pos, jsm, a.jac_q_smem != 0, dft,
                          a.phase_t ? a.phase_t + (size_t)c * kCutPhases + 11 : nullptr);
    phase_stamp(a, c, 6);
    for (int i = tid; i < n; i += nt) MU[i] = H[(size_t)i * n + i];
  } else {
    phase_stamp(a, c, 4);
    // 5b. low-rank path (L < k): for a pure global state H = I - F F^T with
    // F = L^{-1} C^T L_A^{-T} (C the left-right block of sq_cov, V_A = L_A L_A^T),
    // so the non-trivial spectrum lives in range(F): QR of F, Jacobi on the
    // nA x nA matrix I - R R^T, and the complement of range(F) is the nu = 1 space.
    auto gA = [&](int i) { return i < L ? i : M + (i - L); };
    for (int r = warp; r < nA; r += nw) {
      for (int q = lane; q < nA; q += 32) X1[(size_t)r * nA + q] = a.sq_cov[(size_t)gA(r) * (2 * M) + gA(q)];
      for (int q = lane; q < n; q += 32) X2[(size_t)r * n + q] = a.sq_cov[(size_t)gA(r) * (2 * M) + gidx(q)];  // C [nA, n]
    }
    __syncthreads();
    if (!block_cholesky(X1, nA, &s_flag, vec, vec2)) {
      if (tid == 0) a.status[c] = 2;
      return;
    }
    // X2 <- L_A^{-1} C (forward substitution over rows; 1 / L_A,rr in vec)
    for (int r = 0; r < nA; ++r) {
      const double inv = vec[r];
      for (int q = tid; q < n; q += nt) X2[(size_t)r * n + q] *= inv;
      __syncthreads();
      const double* xr = X2 + (size_t)r * n;
      for (int i = r + 1 + warp; i < nA; i += nw) {
        const double l = X1[(size_t)i * nA + r];
        double* xi = X2 + (size_t)i * n;
        for (int q = lane; q < n; q += 32) xi[q] -= l * xr[q];
      }
      __syncthreads();
    }
    // F = W (L_A^{-1} C)^T [n, nA], stored transposed: row j of FT (in H,
    // row stride n) is column j of F, so the Householder QR and the
    // back-transformation below read and update contiguous rows.
    // FT[j][i] = sum_{r <= i} X2[j][r] W[i][r], with W read through its
    // transpose (in Gm, free in this path) for the i-consecutive lanes.
    double* WT = Gm;
    for (int r = warp; r < n; r += nw)
      for (int i = lane; i < n; i += 32) WT[(size_t)r * n + i] = W[(size_t)i * n + r];
    __syncthreads();
    double* FT = H;
    for (int j = warp; j < nA; j += nw) {
      const double* xj = X2 + (size_t)j * n;
      for (int i = lane; i < n; i += 32) {
        double s = 0.0;
#pragma unroll 8
        for (int r = 0; r <= i; ++r) s += WT[(size_t)r * n + i] * xj[r];
        FT[(size_t)j * n + i] = s;
      }
    }
    __syncthreads();
    // Householder QR of F (columns = rows of FT); taus in dots[], the current
    // reflector v (v_j = 1) staged in vec
    // (the reflector of a column by warp 0 alone: two block barriers per
    // column instead of five)
    for (int j = 0; j < nA; ++j) {
      double* fj = FT + (size_t)j * n;
      if (warp == 0) {
        double s2 = 0.0;
        for (int i = j + 1 + lane; i < n; i += 32) s2 += fj[i] * fj[i];
        for (int o = 16; o > 0; o >>= 1) s2 += __shfl_xor_sync(0xffffffffu, s2, o);
        const double x0 = fj[j];
        double beta = x0, tau = 0.0, scale = 0.0;
        if (s2 > 0.0) {
          beta = -copysign(sqrt(x0 * x0 + s2), x0);
          tau = (beta - x0) / beta;
          scale = 1.0 / (x0 - beta);
        }
        for (int i = j + 1 + lane; i < n; i += 32) {
          const double v = fj[i] * scale;
          fj[i] = v;
          vec[i] = v;
        }
        __syncwarp();
        if (lane == 0) {
          fj[j] = beta;
          dots[j] = tau;
          vec[j] = 1.0;
        }
      }
      __syncthreads();
      const double tau = dots[j];
      // apply to the trailing columns: one warp per column (row of FT)
      for (int col = j + 1 + warp; col < nA; col += nw) {
        double* fc = FT + (size_t)col * n;
        double d = 0.0;
        for (int i = j + lane; i < n; i += 32) d += vec[i] * fc[i];
        for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
        d *= tau;
        for (int i = j + lane; i < n; i += 32) fc[i] -= d * vec[i];
      }
      __syncthreads();
    }
    // K = I - R R^T into X1 (R[i][q] = FT[q][i], q >= i), eigenvector rows of
    // K (identity) into X2
    for (int i = warp; i < nA; i += nw)
      for (int j = lane; j < nA; j += 32) {
        double s = 0.0;
#pragma unroll 8
        for (int q = (i > j ? i : j); q < nA; ++q) s += FT[(size_t)q * n + i] * FT[(size_t)q * n + j];
        X1[(size_t)i * nA + j] = (i == j ? 1.0 : 0.0) - s;
      }
    __syncthreads();
    // Gm is free in this path (G is applied through W = L^{-1}, which the pairing still needs)
    phase_stamp(a, c, 5);
    sweeps = mixed_jacobi(X1, nA, X2, Gm, X2 + nn, X2 + 2 * nn, X2 + 3 * nn, red, cs, sn, pos, jsm, a.jac_q_smem != 0, dft,
                          a.phase_t ? a.phase_t + (size_t)c * kCutPhases + 11 : nullptr);
    phase_stamp(a, c, 6);
    for (int i = tid; i < n; i += nt) MU[i] = i < nA ? X1[(size_t)i * nA + i] : 1.0;
    __syncthreads();
    // eigenvector rows of H in the full space: u_i = Q z_i, z_i = [K eigvec; 0] or e_i
    // (into X1, so that W = L^{-1} survives for applying G)
    // (reflector j is row j of FT from column j + 1 on, with v_j = 1)
    for (int i = warp; i < n; i += nw) {
      double* z = EV + (size_t)i * n;
      for (int t = lane; t < n; t += 32) z[t] = i < nA ? (t < nA ? X2[(size_t)i * nA + t] : 0.0) : (t == i ? 1.0 : 0.0);
      __syncwarp();
      for (int j = nA - 1; j >= 0; --j) {
        const double* vj = FT + (size_t)j * n;
        double d = 0.0;
        for (int t = j + lane; t < n; t += 32) d += (t == j ? 1.0 : vj[t]) * z[t];
        for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
        d *= dots[j];
        for (int t = j + lane; t < n; t += 32) z[t] -= d * (t == j ? 1.0 : vj[t]);
        __syncwarp();
      }
    }
  }
  __syncthreads();
  if (tid == 0) a.sweeps[c] = sweeps < 0 ? a.max_sweeps : sweeps;
  if (sweeps < 0) {
    if (tid == 0) a.status[c] = 3;
    return;
  }
  phase_stamp(a, c, 7);
  // 7. order by mu ascending (nu descending), ties by index
  for (int i = tid; i < n; i += nt) {
    const double mi = MU[i];
    int r = 0;
    for (int j = 0; j < n; ++j) {
      const double mj = MU[j];
      r += (mj < mi) || (mj == mi && j < i);
    }
    order[r] = i;
  }
  __syncthreads();
  phase_stamp(a, c, 8);
  // 8. pair eigenvectors x with y = G x / |G x|.  Candidates are grouped in
  // even-sized clusters of (nearly) equal mu; inside a cluster the next x is
  // the candidate with the largest residual after projecting out the pairs
  // already taken (pivoted Gram-Schmidt), so a degenerate eigenspace of any
  // dimension (e.g. the nu = 1 vacuum modes) is always completed.  The
  // candidates' squared residuals are tracked in FP32 by subtraction (pivot
  // choice only); the chosen FP64 eigenvector (not its FP32 copy) is cleaned
  // by one projection against the accepted vectors of the cluster and of the
  // clusters whose mu is within 1e-4 of it.  The
  // products (projections, G x, norms) run in double-float on the FP32 pipe:
  // the accepted vectors are kept as FP32 pairs and the operator of G x (G,
  // or W = L^{-1} in the low-rank path) is split once; S below reads the
  // vectors back in FP64.
  // 1/nu of each pair is |G x| (x a unit eigenvector: |G x|^2 = mu).
  float2* Xacc2 = reinterpret_cast<float2*>(H);        // accepted vectors as rows
  float* c32 = reinterpret_cast<float*>(X2 + nn);       // FP32 candidates of the cluster
  float* r32 = reinterpret_cast<float*>(X2 + 2 * nn);   // their squared residuals
  float* xy32 = r32 + n;                                 // FP32 copies of x and y
  float2* tv = reinterpret_cast<float2*>(X2);           // 2n: W^T x and Omega W^T x
  float2* dots2 = reinterpret_cast<float2*>(dots);      // projection coefficients (negated)
  // The triangular W^T x and the projection update are sums per output of up
  // to n terms: with one thread per output only n of the CTA's threads would
  // work, so each sum is split into `segs` ranges whose partial sums (part,
  // segs x n pairs after tv in X2) are added in range order.
  const int segs = n >= 6 ? max(1, min(4, nt / n)) : 1;
  float2* part = tv + 2 * (size_t)n;
  // item u of the segmented sums is (column u % n, range u / n): with segs > 1
  // there are n * segs <= nt items, so u = tid, mapped once; with segs = 1 it
  // is (u, 0) (no integer division in the pair loop)
  const int my_j = tid % n, my_g = tid / n;
  // profiling: time in six parts of the pairing (cluster setup, pivots and
  // candidate loads, projections, G products, in-block Gram-Schmidt or
  // normalisation, residual tracking), accumulated by thread 0
  unsigned long long* pst = a.phase_t ? a.phase_t + (size_t)c * kCutPhases + 16 : nullptr;
  auto pstamp = [&]() {
    unsigned long long t = 0;
    if (pst && tid == 0) asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
  };
  auto pacc = [&](int part, unsigned long long t0) {
    if (pst && tid == 0) pst[part] += pstamp() - t0;
  };
  if (pst && tid == 0)
    for (int i = 0; i < 6; ++i) pst[i] = 0;
  unsigned long long tp = 0;
  // the operator of G x, split once: G in place (full path) or W into Gm
  // (free in the low-rank path)
  float2* Gop = reinterpret_cast<float2*>(Gm);
  {
    const double* src = g_dense ? Gm : W;
    for (size_t t = tid; t < nn; t += nt) Gop[t] = df_split(src[t]);  // in place: one element per thread
  }
  for (int i = tid; i < n; i += nt) vec2[i] = MU[order[i]];
  __syncthreads();
  int* used = reinterpret_cast<int*>(vec);  // n flags (vec reused as int storage)
  for (int i = tid; i < n; i += nt) used[i] = 0;
  __syncthreads();
  // out[r - r0] = sign * (row r of M) . x over columns [0, min(n, r + 1) if
  // tri else n) for rows r in [r0, r1): each warp takes four rows at a time
  // (four independent sums per lane), lanes the columns
  auto rows_dot = [&](const float2* Mr, int r0, int r1, const float2* x, float2* out, bool tri, float sign) {
    for (int rb = r0 + 4 * warp; rb < r1; rb += 4 * nw) {
      float s[4] = {0.f, 0.f, 0.f, 0.f}, t[4] = {0.f, 0.f, 0.f, 0.f};
      const int jend = tri ? min(n, rb + 4) : n;
      for (int j = lane; j < jend; j += 32) {
        const float2 xj = x[j];
#pragma unroll
        for (int u = 0; u < 4; ++u)
          if (rb + u < r1 && (!tri || j <= rb + u)) df_mac(s[u], t[u], Mr[(size_t)(rb + u) * n + j], xj);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        df_warp_sum(s[u], t[u]);
        if (lane == 0 && rb + u < r1) out[rb + u - r0] = df_norm(sign * s[u], sign * t[u]);
      }
    }
  };
  // y = G x with G = W Omega W^T
  auto apply_G = [&](const float2* x, float2* y) {
    if (g_dense) {
      rows_dot(Gop, 0, n, x, y, false, 1.f);
    } else {
      for (int u = tid; u < n * segs; u += nt) {  // t = W^T x (W lower triangular)
        const int j = segs == 1 ? u : my_j, g = segs == 1 ? 0 : my_g;
        const int len = (n - j + segs - 1) / segs, i0 = j + g * len, i1 = min(n, i0 + len);
        float s = 0.f, t = 0.f;
#pragma unroll 8
        for (int i = i0; i < i1; ++i) df_mac(s, t, Gop[(size_t)i * n + j], x[i]);
        if (segs == 1) tv[j] = df_norm(s, t);
        else part[(size_t)g * n + j] = df_norm(s, t);
      }
      __syncthreads();
      if (segs > 1) {
        for (int j = tid; j < n; j += nt) {
          float2 s = part[j];
          for (int g = 1; g < segs; ++g) s = df_add(s, part[(size_t)g * n + j]);
          tv[j] = s;
        }
        __syncthreads();
      }
      for (int j = tid; j < n; j += nt) {  // Omega t
        const float2 v = j < k ? tv[j + k] : tv[j - k];
        tv[n + j] = j < k ? v : make_float2(-v.x, -v.y);
      }
      __syncthreads();
      rows_dot(Gop, 0, n, tv + n, y, true, 1.f);  // y = W (Omega t)
    }
    __syncthreads();
  };
  // v -= sum over accepted rows [a0, a1) of (row . v) row, one pass
  auto project_out = [&](float2* v, int a0, int a1) {
    rows_dot(Xacc2, a0, a1, v, dots2, false, -1.f);  // negated coefficients
    __syncthreads();
    if (segs == 1) {
      for (int i = tid; i < n; i += nt) {
        float s = v[i].x, t = v[i].y;
#pragma unroll 8
        for (int av = a0; av < a1; ++av) df_mac(s, t, dots2[av - a0], Xacc2[(size_t)av * n + i]);
        v[i] = df_norm(s, t);
      }
    } else {
      const int len = (a1 - a0 + segs - 1) / segs;
      for (int u = tid; u < n * segs; u += nt) {
        const int i = segs == 1 ? u : my_j, g = segs == 1 ? 0 : my_g;
        const int b0 = a0 + g * len, b1 = min(a1, b0 + len);
        float s = 0.f, t = 0.f;
#pragma unroll 8
        for (int av = b0; av < b1; ++av) df_mac(s, t, dots2[av - a0], Xacc2[(size_t)av * n + i]);
        part[(size_t)g * n + i] = df_norm(s, t);
      }
      __syncthreads();
      for (int i = tid; i < n; i += nt) {
        float2 s = v[i];
        for (int g = 0; g < segs; ++g) s = df_add(s, part[(size_t)g * n + i]);
        v[i] = s;
      }
    }
    __syncthreads();
  };
  // |v|^2 over the block into *q (warp sums in double-float, the 32 warp
  // totals in FP64 by thread 0) and 1/|v| split, for every thread: thread 0
  // alone takes the FP64 square root and reciprocal (the FP64 pipe is narrow)
  auto norm_inv = [&](const float2* v, double* q) {
    float s = 0.f, t = 0.f;
    for (int i = tid; i < n; i += nt) df_mac(s, t, v[i], v[i]);
    df_warp_sum(s, t);
    if (lane == 0) red[warp] = double(s) + double(t);
    __syncthreads();
    if (tid == 0) {
      double tot = 0.0;
      for (int w = 0; w < nw; ++w) tot += red[w];
      red[32] = tot;
      red[33] = tot > 0.0 ? 1.0 / sqrt(tot) : 0.0;
    }
    __syncthreads();
    *q = red[32];
    return df_split(red[33]);
  };
  int acc = 0;
  int cb = 0;
  while (cb < n) {
    int ce = cb + 2;
    while (ce < n && !(vec2[ce] - vec2[ce - 1] > 1e-9 * fmax(fabs(vec2[ce]), 1e-300))) ce += 2;
    if (ce > n) ce = n;
    const int acc0 = acc, C = ce - cb;
    // accepted rows of earlier clusters whose mu lies within 1e-4 of this
    // cluster's: the eigen-solver leaves eigenvectors of such close
    // eigenvalues mixed by (its residual) / gap, ~1e-7 at gaps just above the
    // clustering threshold, so the new x are projected against them too
    // (accepted row r belongs to the cluster of sorted candidate r)
    int an = acc0;
    while (an > 0 && vec2[cb] - vec2[an - 1] <= 1e-4 * fabs(vec2[cb])) --an;
    tp = pstamp();
    // FP32 copies of the cluster's candidates and their squared norms
    for (int r = warp; r < C; r += nw) {
      const double* ev = EV + (size_t)order[cb + r] * n;
      for (int i = lane; i < n; i += 32) c32[(size_t)r * n + i] = df_split(ev[i]).x;  // no FP64 conversion
    }
    __syncthreads();
    for (int r = tid >> 5; r < C; r += nt >> 5) {
      float s = 0.f;
      for (int i = tid & 31; i < n; i += 32) s = fmaf(c32[(size_t)r * n + i], c32[(size_t)r * n + i], s);
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if ((tid & 31) == 0) r32[r] = s;
    }
    __syncthreads();
    // The exact nu = 1 block of the low-rank path (every mu exactly 1: the
    // complement of range(F)) is paired four candidates at a time: G maps it
    // onto itself with G^2 = -I, so after G is applied to the block's four
    // projected candidates at once, the in-block Gram-Schmidt needs no further
    // G products (G y_p = -x_p).  Per pair this reads W, the accepted
    // vectors and the FP32 candidates a quarter as often and takes ~6 block
    // barriers instead of ~16.
    bool vac = !g_dense && n >= 64 && C >= 8;
    for (int r = 0; r < C && vac; ++r) vac = vec2[cb + r] == 1.0;
    pacc(0, tp);
    if (vac) {
      float2* dotsb = tv + 6 * (size_t)n;   // [accepted row][4] negated projections
      float2* tvb = dotsb + 4 * (size_t)n;  // [q][2n]: W^T x_q and Omega W^T x_q
      float2* partb = tvb + 8 * (size_t)n;  // [range][q][n] partial sums
      float2* bred = dots2;                 // [warp][8] partial dots, then [8] totals at 256
      while (acc - acc0 < C) {
        tp = pstamp();
        // 1. up to four unused candidates with the largest residuals (the
        // first must exist; the others must keep a residual above 0.05)
        if (tid < 32) {
          const int want = min(4, (C - (acc - acc0)) / 2);
          int taken = 0;
          for (int q = 0; q < want; ++q) {
            float bv = -1.f;
            int best = -1;
            for (int r = lane; r < C; r += 32)
              if (!used[cb + r] && r32[r] > bv) {
                bv = r32[r];
                best = r;
              }
            for (int o = 16; o > 0; o >>= 1) {
              const float ov = __shfl_xor_sync(0xffffffffu, bv, o);
              const int ob = __shfl_xor_sync(0xffffffffu, best, o);
              if (ov > bv || (ov == bv && ob >= 0 && (best < 0 || ob < best))) {
                bv = ov;
                best = ob;
              }
            }
            if (best < 0 || !(bv > (q == 0 ? 1e-6f : 0.05f))) break;
            if (lane == 0) {
              used[cb + best] = 1;
              s_pick[q] = best;
              s_pickv[q] = bv;
            }
            __syncwarp();
            ++taken;
          }
          if (lane == 0) s_nb = taken;
        }
        __syncthreads();
        const int nb = s_nb;
        if (nb == 0) {
          if (tid == 0) a.status[c] = 4;
          return;
        }
        // 2. the candidates (FP64 eigenvectors, split) into the x rows acc + 2q
        for (int q = 0; q < nb; ++q) {
          float2* xq = Xacc2 + (size_t)(acc + 2 * q) * n;
          const double* ev = EV + (size_t)order[cb + s_pick[q]] * n;
          for (int i = tid; i < n; i += nt) xq[i] = df_split(ev[i]);
        }
        __syncthreads();
        pacc(1, tp);
        tp = pstamp();
        // the block's x rows; q >= nb repeats the last one (results dropped), so
        // the loops below carry no per-iteration guard and unroll, keeping
        // several loads per warp in flight (these loops are L2-latency bound)
        const float2* xr0 = Xacc2 + (size_t)acc * n;
        const float2* xr1 = Xacc2 + (size_t)(acc + 2 * min(1, nb - 1)) * n;
        const float2* xr2 = Xacc2 + (size_t)(acc + 2 * min(2, nb - 1)) * n;
        const float2* xr3 = Xacc2 + (size_t)(acc + 2 * min(3, nb - 1)) * n;
        // 3. project the block against the accepted vectors of the cluster
        // and of the clusters within 1e-4 below it (rows an .. acc0)
        if (acc > an) {
          for (int av = an + warp; av < acc; av += nw) {
            float ss[4] = {0.f, 0.f, 0.f, 0.f}, tt[4] = {0.f, 0.f, 0.f, 0.f};
            const float2* ra = Xacc2 + (size_t)av * n;
#pragma unroll 3
            for (int i = lane; i < n; i += 32) {
              const float2 r = ra[i];
              df_mac(ss[0], tt[0], r, xr0[i]);
              df_mac(ss[1], tt[1], r, xr1[i]);
              df_mac(ss[2], tt[2], r, xr2[i]);
              df_mac(ss[3], tt[3], r, xr3[i]);
            }
#pragma unroll
            for (int q = 0; q < 4; ++q) {
              if (q >= nb) break;
              df_warp_sum(ss[q], tt[q]);
              if (lane == 0) dotsb[(size_t)(av - an) * 4 + q] = df_norm(-ss[q], -tt[q]);
            }
          }
          __syncthreads();
          const int len = (acc - an + segs - 1) / segs;
          for (int u = tid; u < n * segs; u += nt) {
            const int i = segs == 1 ? u : my_j, g = segs == 1 ? 0 : my_g;
            const int b0 = an + g * len, b1 = min(acc, b0 + len);
            float ss[4] = {0.f, 0.f, 0.f, 0.f}, tt[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 8
            for (int av = b0; av < b1; ++av) {
              const float2 r = Xacc2[(size_t)av * n + i];
              const float4 d01 = *reinterpret_cast<const float4*>(dotsb + (size_t)(av - an) * 4);
              const float4 d23 = *reinterpret_cast<const float4*>(dotsb + (size_t)(av - an) * 4 + 2);
              df_mac(ss[0], tt[0], make_float2(d01.x, d01.y), r);
              df_mac(ss[1], tt[1], make_float2(d01.z, d01.w), r);
              df_mac(ss[2], tt[2], make_float2(d23.x, d23.y), r);
              df_mac(ss[3], tt[3], make_float2(d23.z, d23.w), r);
            }
#pragma unroll
            for (int q = 0; q < 4; ++q)
              if (q < nb) partb[((size_t)g * 4 + q) * n + i] = df_norm(ss[q], tt[q]);
          }
          __syncthreads();
          for (int q = 0; q < nb; ++q) {
            float2* xq = Xacc2 + (size_t)(acc + 2 * q) * n;
            for (int i = tid; i < n; i += nt) {
              float2 v = xq[i];
              for (int g = 0; g < segs; ++g) v = df_add(v, partb[((size_t)g * 4 + q) * n + i]);
              xq[i] = v;
            }
          }
          __syncthreads();
        }
        pacc(2, tp);
        tp = pstamp();
        // 4. z_q = G x_q = W (Omega (W^T x_q)), one pass over W per product
        for (int u = tid; u < n * segs; u += nt) {
          const int j = segs == 1 ? u : my_j, g = segs == 1 ? 0 : my_g;
          const int len = (n - j + segs - 1) / segs, i0 = j + g * len, i1 = min(n, i0 + len);
          float ss[4] = {0.f, 0.f, 0.f, 0.f}, tt[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 8
          for (int i = i0; i < i1; ++i) {
            const float2 w = Gop[(size_t)i * n + j];
            df_mac(ss[0], tt[0], w, xr0[i]);
            df_mac(ss[1], tt[1], w, xr1[i]);
            df_mac(ss[2], tt[2], w, xr2[i]);
            df_mac(ss[3], tt[3], w, xr3[i]);
          }
#pragma unroll
          for (int q = 0; q < 4; ++q)
            if (q < nb) partb[((size_t)g * 4 + q) * n + j] = df_norm(ss[q], tt[q]);
        }
        __syncthreads();
        for (int q = 0; q < nb; ++q)
          for (int j = tid; j < n; j += nt) {
            float2 v = partb[(size_t)q * n + j];
            for (int g = 1; g < segs; ++g) v = df_add(v, partb[((size_t)g * 4 + q) * n + j]);
            tvb[(size_t)q * 2 * n + j] = v;
          }
        __syncthreads();
        for (int q = 0; q < nb; ++q)
          for (int j = tid; j < n; j += nt) {  // Omega t
            const float2 v = j < k ? tvb[(size_t)q * 2 * n + j + k] : tvb[(size_t)q * 2 * n + j - k];
            tvb[(size_t)q * 2 * n + n + j] = j < k ? v : make_float2(-v.x, -v.y);
          }
        __syncthreads();
        const float2* ot0 = tvb + n;
        const float2* ot1 = tvb + (size_t)min(1, nb - 1) * 2 * n + n;
        const float2* ot2 = tvb + (size_t)min(2, nb - 1) * 2 * n + n;
        const float2* ot3 = tvb + (size_t)min(3, nb - 1) * 2 * n + n;
        for (int i = warp; i < n; i += nw) {
          float ss[4] = {0.f, 0.f, 0.f, 0.f}, tt[4] = {0.f, 0.f, 0.f, 0.f};
          const float2* wi = Gop + (size_t)i * n;
#pragma unroll 3
          for (int j = lane; j <= i; j += 32) {
            const float2 w = wi[j];
            df_mac(ss[0], tt[0], w, ot0[j]);
            df_mac(ss[1], tt[1], w, ot1[j]);
            df_mac(ss[2], tt[2], w, ot2[j]);
            df_mac(ss[3], tt[3], w, ot3[j]);
          }
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            if (q >= nb) break;
            df_warp_sum(ss[q], tt[q]);
            if (lane == 0) Xacc2[(size_t)(acc + 2 * q + 1) * n + i] = df_norm(ss[q], tt[q]);
          }
        }
        __syncthreads();
        pacc(3, tp);
        tp = pstamp();
        // 5. in-block Gram-Schmidt: x_q against the pairs accepted before it
        // (dots and |x_q|^2 in one reduction; |x_q - proj|^2 = |x_q|^2 -
        // sum of the squared coefficients), z_q with the same coefficients
        // through G x_p = y_p, G y_p = -x_p, both scaled by 1 / |x_q - proj|
        // (|G x| = |x| on this block); a candidate left with less than a
        // quarter of its residual goes back to the pool
        int nacc = 0;
        for (int q = 0; q < nb; ++q) {
          const float2* xq = Xacc2 + (size_t)(acc + 2 * q) * n;
          const float2* zq = xq + n;
          const int nd = 2 * nacc + 1;  // dots x_p . x_q, y_p . x_q (p < nacc), then |x_q|^2
          float ss[7], tt[7];
#pragma unroll
          for (int e = 0; e < 7; ++e) ss[e] = tt[e] = 0.f;
          for (int i = tid; i < n; i += nt) {
            const float2 v = xq[i];
#pragma unroll
            for (int e = 0; e < 6; ++e)
              if (e < nd - 1) df_mac(ss[e], tt[e], Xacc2[(size_t)(acc + e) * n + i], v);
            df_mac(ss[6], tt[6], v, v);
          }
#pragma unroll
          for (int e = 0; e < 7; ++e) {
            if (e < nd - 1 || e == 6) {
              df_warp_sum(ss[e], tt[e]);
              if (lane == 0) bred[warp * 8 + e] = df_norm(ss[e], tt[e]);
            }
          }
          __syncthreads();
          if (tid < 7 && (tid < nd - 1 || tid == 6)) {
            float2 v = bred[tid];
            for (int w = 1; w < nw; ++w) v = df_add(v, bred[w * 8 + tid]);
            bred[256 + tid] = v;
          }
          __syncthreads();
          double rem = df_val(bred[256 + 6]);
          for (int e = 0; e < nd - 1; ++e) {
            const double cc = df_val(bred[256 + e]);
            rem -= cc * cc;
          }
          if (nacc > 0 && !(rem > 0.25 * double(s_pickv[q]))) {  // block-uniform: back to the pool
            if (tid == 0) used[cb + s_pick[q]] = 0;
            __syncthreads();
            continue;
          }
          if (!(rem > 0.0)) {  // the block's first candidate has no residual left
            if (tid == 0) a.status[c] = 4;
            return;
          }
          if (tid == 0) red[34] = 1.0 / sqrt(rem);
          __syncthreads();
          const float2 inv = df_split(red[34]);
          float2 cf[6];
#pragma unroll
          for (int e = 0; e < 6; ++e) cf[e] = e < nd - 1 ? bred[256 + e] : make_float2(0.f, 0.f);
          float2* xo = Xacc2 + (size_t)(acc + 2 * nacc) * n;  // compacted slot (nacc <= q)
          float2* yo = xo + n;
          for (int i = tid; i < n; i += nt) {
            float sx = xq[i].x, tx = xq[i].y, sz = zq[i].x, tz = zq[i].y;
#pragma unroll
            for (int p = 0; p < 3; ++p) {
              if (p >= nacc) break;
              const float2 xp = Xacc2[(size_t)(acc + 2 * p) * n + i], yp = Xacc2[(size_t)(acc + 2 * p + 1) * n + i];
              const float2 c1 = make_float2(-cf[2 * p].x, -cf[2 * p].y), c2 = make_float2(-cf[2 * p + 1].x, -cf[2 * p + 1].y);
              // x -= c1 x_p + c2 y_p;  z -= c1 y_p - c2 x_p
              df_mac(sx, tx, c1, xp);
              df_mac(sx, tx, c2, yp);
              df_mac(sz, tz, c1, yp);
              df_mac(sz, tz, cf[2 * p + 1], xp);
            }
            const float2 xn = df_mul(df_norm(sx, tx), inv), zn = df_mul(df_norm(sz, tz), inv);
            xo[i] = xn;  // xo is row x_q itself or an earlier, unread (rejected) slot
            yo[i] = zn;
          }
          __syncthreads();
          if (tid == 0) MU[(acc + 2 * nacc) / 2] = sqrt(vec2[cb + s_pick[q]]);
          ++nacc;
        }
        pacc(4, tp);
        tp = pstamp();
        // 6. FP32 residual tracking for the accepted pairs of this block
        for (int e = 0; e < 2 * nacc; ++e) {
          const float2* v = Xacc2 + (size_t)(acc + e) * n;
          for (int i = tid; i < n; i += nt) xy32[(size_t)e * n + i] = v[i].x;
        }
        __syncthreads();
        for (int r = warp; r < C; r += nw) {
          if (used[cb + r]) continue;
          const float* w = c32 + (size_t)r * n;
          float sd[8];
#pragma unroll
          for (int e = 0; e < 8; ++e) sd[e] = 0.f;
          for (int i = lane; i < n; i += 32) {
            const float wi = w[i];
#pragma unroll
            for (int e = 0; e < 8; ++e)
              if (e < 2 * nacc) sd[e] = fmaf(xy32[(size_t)e * n + i], wi, sd[e]);
          }
          float sub = 0.f;
#pragma unroll
          for (int e = 0; e < 8; ++e) {
            if (e >= 2 * nacc) break;
            float v = sd[e];
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            sub += v * v;
          }
          if (lane == 0) r32[r] -= sub;
        }
        __syncthreads();
        pacc(5, tp);
        acc += 2 * nacc;
      }
      cb = ce;
      continue;
    }
    for (int pi = 0; pi < C / 2; ++pi) {
      if (tid < 32) {  // pivot: the unused candidate with the largest residual
        float bv = -1.f;
        int best = -1;
        for (int r = tid; r < C; r += 32)
          if (!used[cb + r] && r32[r] > bv) {
            bv = r32[r];
            best = r;
          }
        for (int o = 16; o > 0; o >>= 1) {
          const float ov = __shfl_xor_sync(0xffffffffu, bv, o);
          const int ob = __shfl_xor_sync(0xffffffffu, best, o);
          if (ov > bv || (ov == bv && ob >= 0 && (best < 0 || ob < best))) {
            bv = ov;
            best = ob;
          }
        }
        if (tid == 0) {
          s_flag = best;
          s_scalar = bv;
          if (best >= 0) used[cb + best] = 1;
        }
      }
      __syncthreads();
      const int best = s_flag;
      if (best < 0 || !(s_scalar > 1e-6)) {
        if (tid == 0) a.status[c] = 4;
        return;
      }
      float2* x = Xacc2 + (size_t)acc * n;
      float2* y = Xacc2 + (size_t)(acc + 1) * n;
      // x: the FP64 eigenvector itself (an FP32-rounded copy would leave the
      // eigenspace by ~1e-7), one projection pass (its residual is the
      // largest of the cluster, so one pass keeps orthogonality at rounding)
      for (int i = tid; i < n; i += nt) x[i] = df_split(EV[(size_t)order[cb + best] * n + i]);
      __syncthreads();
      project_out(x, an, acc);
      double nx;
      const float2 ix = norm_inv(x, &nx);
      for (int i = tid; i < n; i += nt) x[i] = df_mul(x[i], ix);
      __syncthreads();
      // y = G x / |G x| needs no projection: G maps the span of the accepted
      // pairs into itself (G x_j = |G x_j| y_j, G y_j = -|G x_j| x_j for
      // eigenvectors x_j of G^T G), so x orthogonal to that span makes G x
      // orthogonal to it up to rounding (checked to 1e-10 on every kind of
      // cut by the symplectic tests)
      apply_G(x, y);
      double gx;  // |G x|^2 = 1/nu^2
      const float2 iy = norm_inv(y, &gx);
      for (int i = tid; i < n; i += nt) {
        const float2 yi = df_mul(y[i], iy);
        y[i] = yi;
        xy32[i] = x[i].x;
        xy32[n + i] = yi.x;
      }
      // 1/nu of pair acc/2 (MU no longer needed by candidates): |G x| in the
      // full path; in the low-rank path the eigenvalue of K = I - R R^T
      // itself, whose 1 - mu = sigma^2 carries the small nbar of weakly
      // coupled modes to ~1e-16 absolute, where |G x| (through L^-1 twice)
      // loses cond(V) of it
      if (tid == 0) MU[acc / 2] = g_dense ? sqrt(gx) : sqrt(vec2[cb + best]);
      __syncthreads();
      // FP32 tracking: the candidates stay as they are (orthonormal); a
      // candidate's squared residual against the accepted orthonormal pairs
      // is |u|^2 - sum (a . u)^2, so each step subtracts (x . u)^2 + (y . u)^2
      // (two candidates per warp step: four independent sums per lane)
      for (int rb = 2 * warp; rb < C; rb += 2 * nw) {
        const bool u0 = !used[cb + rb], u1 = rb + 1 < C && !used[cb + rb + 1];
        if (!u0 && !u1) continue;
        const float* w0 = c32 + (size_t)rb * n;
        const float* w1 = w0 + n;
        float sx0 = 0.f, sy0 = 0.f, sx1 = 0.f, sy1 = 0.f;
        for (int i = lane; i < n; i += 32) {
          const float xi = xy32[i], yi = xy32[n + i];
          const float a0 = w0[i], a1 = u1 ? w1[i] : 0.f;
          sx0 = fmaf(xi, a0, sx0);
          sy0 = fmaf(yi, a0, sy0);
          sx1 = fmaf(xi, a1, sx1);
          sy1 = fmaf(yi, a1, sy1);
        }
        for (int o = 16; o > 0; o >>= 1) {
          sx0 += __shfl_xor_sync(0xffffffffu, sx0, o);
          sy0 += __shfl_xor_sync(0xffffffffu, sy0, o);
          sx1 += __shfl_xor_sync(0xffffffffu, sx1, o);
          sy1 += __shfl_xor_sync(0xffffffffu, sy1, o);
        }
        if (lane == 0) {
          if (u0) r32[rb] -= sx0 * sx0 + sy0 * sy0;
          if (u1) r32[rb + 1] -= sx1 * sx1 + sy1 * sy1;
        }
      }
      __syncthreads();
      acc += 2;
    }
    cb = ce;
  }
  if (acc != n) {
    if (tid == 0) a.status[c] = 4;
    return;
  }
  // the accepted vectors back to FP64 for S (in place: one element per thread)
  double* Xacc = H;
  for (size_t t = tid; t < nn; t += nt) Xacc[t] = df_val(Xacc2[t]);
  __syncthreads();
  phase_stamp(a, c, 9);
  // 9. S = L [y | x] nu^{-1/2}, nbar = max(0, (nu - 1)/2).  The products
  // R = Xacc L^T (row 2p of R is L x_p, row 2p + 1 is L y_p) run as one
  // double-float product on the FP32 pipe (the accepted vectors are
  // double-float values already; L is split), skipping the zero upper
  // triangle of L: k n^2 FP64 multiply-adds were ~5 ms of one CTA at n = 286.
  double* R = Gm;  // free after the pairing
  double* scl = vec;  // nu^{-1/2} per pair
  for (int pi = tid; pi < k; pi += nt) {
    const double s = MU[pi];  // 1/nu
    const double nb = (1.0 / s - 1.0) / 2.0;
    scl[pi] = sqrt(s);
    a.nbar[(size_t)c * a.kmax + pi] = nb > 0.0 ? nb : 0.0;
  }
  df_gemm(Xacc, false, A, true, nullptr, 1.0, 0.0, R, n, false, dft, true);
  {
    double* Sc = a.S + (size_t)c * a.ldS * a.ldS;
    for (int i = warp; i < n; i += nw)
      for (int col = lane; col < n; col += 32) {
        const int pi = col < k ? col : col - k;
        const int src = col < k ? 2 * pi + 1 : 2 * pi;
        Sc[(size_t)i * a.ldS + col] = R[(size_t)src * n + i] * scl[pi];
      }
  }
  __syncthreads();
  phase_stamp(a, c, 10);
  if (tid == 0) a.status[c] = 0;
}

// ---------------------------------------------------------------------------
// Top-chi product-thermal weights (one CTA per cut).
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long dbits(double x) { return (unsigned long long)__double_as_longlong(x); }

// The top-chi weights of cut c of `a` by the whole CTA.
__device__ __forceinline__ void thermal_cut(const CutArgs& a, const int c) {
  if (a.status[c] != 0) return;
  const int L = a.L0 + c, k = a.M - L, d = a.d, chi = a.chi;
  const int tid = threadIdx.x, nt = blockDim.x;
  extern __shared__ unsigned long long smu[];
  unsigned long long* prod = smu;                     // [d][chi] bit patterns
  double* cur = reinterpret_cast<double*>(prod + (size_t)d * chi);  // [chi]
  double* nxt = cur + chi;                             // [chi]
  double* t = nxt + chi;                               // [d]
  __shared__ int s_K, s_valid;
  uint32_t* rec = a.rec + (size_t)c * a.kmax * chi;
  const double* nb = a.nbar + (size_t)c * a.kmax;
  // step 0: the first mode, unfiltered (kron_cpu.py:106)
  for (int n = tid; n < d; n += nt) {
    double x = nb[0];
    cur[n] = 1.0 / (x + 1.0) * pow(x / (x + 1.0), (double)n);
    rec[n] = (uint32_t)n;
  }
  if (tid == 0) s_K = d;
  __syncthreads();
  for (int s = 1; s < k; ++s) {
    const int K = s_K;
    for (int n = tid; n < d; n += nt) {
      double x = nb[s];
      t[n] = 1.0 / (x + 1.0) * pow(x / (x + 1.0), (double)n);
    }
    __syncthreads();
    // item u = n * K + i (consecutive threads on consecutive candidates of one
    // column); (n, i) advance by (dn, di) per stride, so only the first item
    // of a thread and the stride take an integer division
    const int dn = nt / K, di = nt - dn * K, n0 = tid / K, i0 = tid - n0 * K;
    for (int u = tid, n = n0, i = i0; u < d * K; u += nt) {
      prod[(size_t)n * chi + i] = dbits(cur[i] * t[n]);
      n += dn;
      i += di;
      if (i >= K) {
        i -= K;
        ++n;
      }
    }
    if (tid == 0) s_valid = 0;
    __syncthreads();
    // number of valid (> err_tol) candidates
    const unsigned long long tol = dbits(a.err_tol);
    for (int n = tid; n < d; n += nt) {
      const unsigned long long* col = prod + (size_t)n * chi;
      int lo = 0, hi = K;  // first index with prod <= tol
      while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (col[mid] > tol) lo = mid + 1;
        else hi = mid;
      }
      atomicAdd(&s_valid, lo);
    }
    __syncthreads();
    const int Kn = min(chi, s_valid);
    uint32_t* rs = rec + (size_t)s * chi;
    for (int u = tid, n = n0, i = i0; u < d * K; u += nt, n += dn, i += di) {
      if (i >= K) {
        i -= K;
        ++n;
      }
      // the (i + 1)(n + 1) - 1 candidates (i' <= i, n' <= n) are >= v and come
      // first on ties (flattened order), so rank >= (i + 1)(n + 1) - 1
      if ((i + 1) * (n + 1) > Kn) continue;
      const unsigned long long v = prod[(size_t)n * chi + i];
      if (v <= tol) continue;
      int rank = 0;
      for (int n2 = 0; n2 < d && rank < Kn; ++n2) {
        const unsigned long long* col = prod + (size_t)n2 * chi;
        int lo = 0, hi = K;  // count of > v
        while (lo < hi) {
          int mid = (lo + hi) >> 1;
          if (col[mid] > v) lo = mid + 1;
          else hi = mid;
        }
        int gt = lo;
        hi = K;  // count of >= v
        while (lo < hi) {
          int mid = (lo + hi) >> 1;
          if (col[mid] >= v) lo = mid + 1;
          else hi = mid;
        }
        int ge = lo;
        int lim = i + (n2 < n ? 1 : 0);
        int ties = min(ge, lim) - gt;
        rank += gt + (ties > 0 ? ties : 0);
      }
      if (rank < Kn) {
        nxt[rank] = __longlong_as_double((long long)v);
        rs[rank] = ((uint32_t)i << 8) | (uint32_t)n;
      }
    }
    __syncthreads();
    for (int i = tid; i < Kn; i += nt) cur[i] = nxt[i];
    if (tid == 0) s_K = Kn;
    __syncthreads();
  }
  const int K = s_K;
  const int Kout = min(chi, K);
  // single-mode cuts keep the thermal row as is (already descending)
  for (int r = tid; r < Kout; r += nt) {
    a.res[(size_t)c * chi + r] = cur[r];
    int p = r;
    int8_t* row = a.num + ((size_t)c * chi + r) * (a.M - 1);
    for (int s = k - 1; s >= 1; --s) {
      uint32_t w = rec[(size_t)s * chi + p];
      row[s] = (int8_t)(w & 0xff);
      p = (int)(w >> 8);
    }
    row[0] = (int8_t)(rec[p] & 0xff);
  }
  if (tid == 0) a.kept[c] = Kout;
}

// One CTA per cut: cuts c0 + blockIdx.x of one call.
__global__ void __launch_bounds__(1024) williamson_kernel(const __grid_constant__ CutArgs a) {
  williamson_cut(a, a.c0 + blockIdx.x);
}
__global__ void __launch_bounds__(1024) thermal_kernel(const __grid_constant__ CutArgs a) {
  thermal_cut(a, a.c0 + blockIdx.x);
}
// Batched over independent instances: block b handles cut map[b].y of instance map[b].x.
__global__ void __launch_bounds__(1024) williamson_batch_kernel(const CutArgs* __restrict__ args,
                                                                const int2* __restrict__ map) {
  const int2 m = map[blockIdx.x];
  williamson_cut(args[m.x], m.y);
}
__global__ void __launch_bounds__(1024) thermal_batch_kernel(const CutArgs* __restrict__ args,
                                                             const int2* __restrict__ map) {
  const int2 m = map[blockIdx.x];
  thermal_cut(args[m.x], m.y);
}

}  // namespace bsg

using namespace bsg;

namespace bsg {

static size_t al256(size_t x) { return (x + 255) & ~size_t(255); }

// n^2 blocks of FP64 workspace per cut: V / L, L^-1, G, H, X1, X2 and three
// eigen-solver scratch blocks after X2
constexpr size_t kCutWsBlocks = 9;

// Bytes of cut workspace for n_cuts cuts of an M-mode state (cut_prepare_at).
size_t cut_ws_bytes(int M, int L0, int n_cuts, int chi) {
  const int kmax = M - L0, nmax = 2 * kmax;
  return al256((size_t)kCutWsBlocks * nmax * nmax * 8 * n_cuts) + al256((size_t)n_cuts * kmax * 8) +
         al256((size_t)n_cuts * kmax * chi * 4) + al256((size_t)n_cuts * 8) + al256((size_t)n_cuts * 2 * kmax * 8) +
         al256((size_t)n_cuts * kCutPhases * 8);
}

int cut_prepare(bsg_handle_t h, const double* sq_cov, int M, int L0, int n_cuts, int d, int chi, double err_tol,
                double* res, int8_t* num, double* S, int32_t* kept, CutArgs* out, cudaStream_t st) {
  BSG_CHECK_ARG(M >= 2 && L0 >= 1 && n_cuts >= 1 && L0 + n_cuts <= M, "bsg_cut_spectra: cuts [%d, %d) outside [1, M=%d)",
                L0, L0 + n_cuts, M);
  BSG_TRY(h->cut_ws.ensure(cut_ws_bytes(M, L0, n_cuts, chi)));
  return cut_prepare_at(h, reinterpret_cast<char*>(h->cut_ws.ptr), sq_cov, M, L0, n_cuts, d, chi, err_tol, res, num,
                        S, kept, out, st);
}

// Workspace (at `base`, cut_ws_bytes of it), output clearing and the launch
// arguments of a cut-spectra call.
int cut_prepare_at(bsg_handle_t h, char* base, const double* sq_cov, int M, int L0, int n_cuts, int d, int chi,
                   double err_tol, double* res, int8_t* num, double* S, int32_t* kept, CutArgs* out, cudaStream_t st,
                   std::vector<FillSpan>* defer) {
  BSG_CHECK_ARG(M >= 2 && L0 >= 1 && n_cuts >= 1 && L0 + n_cuts <= M, "bsg_cut_spectra: cuts [%d, %d) outside [1, M=%d)",
                L0, L0 + n_cuts, M);
  BSG_CHECK_ARG(M - L0 <= kMaxCutModes, "bsg_cut_spectra: %d modes in a cut exceeds %d", M - L0, kMaxCutModes);
  BSG_CHECK_ARG(d >= 1 && d <= 64 && chi >= d && chi <= 4096, "bsg_cut_spectra: need 1 <= d <= chi <= 4096, d <= 64");
  const size_t tsm = (size_t)d * chi * 8 + 2 * (size_t)chi * 8 + 64 * 8;
  if (tsm > 227 * 1024) {
    set_error("bsg_cut_spectra: d*chi=%d needs %zu bytes of shared memory", d * chi, tsm);
    return BSG_ERR_LIMIT;
  }
  const int kmax = M - L0, nmax = 2 * kmax;
  CutArgs a{};
  a.sq_cov = sq_cov;
  a.M = M;
  a.L0 = L0;
  a.n_cuts = n_cuts;
  a.d = d;
  a.chi = chi;
  a.err_tol = err_tol;
  a.ws_stride = (size_t)kCutWsBlocks * nmax * nmax;
  a.S = S;
  a.ldS = 2 * (M - 1);
  a.kmax = kmax;
  a.res = res;
  a.num = num;
  a.kept = kept;
  a.max_sweeps = 40;
  const size_t ws_bytes = a.ws_stride * 8 * n_cuts;
  const size_t nbar_bytes = (size_t)n_cuts * kmax * 8;
  const size_t mu_bytes = (size_t)n_cuts * 2 * kmax * 8;
  const size_t rec_bytes = (size_t)n_cuts * kmax * chi * 4;
  const size_t st_bytes = (size_t)n_cuts * 8;
  const size_t ph_bytes = (size_t)n_cuts * kCutPhases * 8;
  auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
  a.ws = reinterpret_cast<double*>(base);
  a.nbar = reinterpret_cast<double*>(base + al(ws_bytes));
  a.rec = reinterpret_cast<uint32_t*>(base + al(ws_bytes) + al(nbar_bytes));
  a.status = reinterpret_cast<int*>(base + al(ws_bytes) + al(nbar_bytes) + al(rec_bytes));
  a.sweeps = a.status + n_cuts;
  a.mu = reinterpret_cast<double*>(base + al(ws_bytes) + al(nbar_bytes) + al(rec_bytes) + al(st_bytes));
  a.phase_t = nullptr;
  if (h->prof.on)
    a.phase_t = reinterpret_cast<unsigned long long*>(base + al(ws_bytes) + al(nbar_bytes) + al(rec_bytes) +
                                                      al(st_bytes) + al(mu_bytes));
  // status -1: "did not finish" until the Williamson kernel writes it
  const FillSpan clears[6] = {{a.phase_t, a.phase_t ? (int64_t)ph_bytes : 0, 0},
                              {a.status, (int64_t)st_bytes, 0xff},
                              {res, (int64_t)n_cuts * chi * 8, 0},
                              {num, (int64_t)n_cuts * chi * (M - 1), 0},
                              {S, (int64_t)n_cuts * a.ldS * a.ldS * 8, 0},
                              {kept, (int64_t)n_cuts * 4, 0}};
  for (const FillSpan& f : clears) {
    if (f.bytes == 0) continue;
    if (defer) defer->push_back(f);
    else BSG_CUDA(cudaMemsetAsync(f.p, f.value, (size_t)f.bytes, st));
  }
  *out = a;
  return BSG_OK;
}

// Williamson decomposition of cuts [c0, c1) (relative to L0), one CTA each.
int cut_launch_williamson(bsg_handle_t h, const CutArgs& args, int c0, int c1, cudaStream_t st) {
  if (c1 <= c0) return BSG_OK;
  CutArgs a = args;
  a.c0 = c0;
  size_t wsm = (40 + 2 * kMaxCutModes) * 8 + 4 * kMaxCutModes * 4 + 6 * kMaxCutModes * 8 + kDfSmemBytes;
  // eigen-problem size of cut c: 2 min(L, k) (full path m = 2k, low-rank path m = 2L)
  int m_max = 0;
  for (int c = c0; c < c1; ++c) {
    const int L = a.L0 + c, k = a.M - L;
    m_max = std::max(m_max, 2 * std::min(L, k));
  }
  int smem_optin = 0;
  BSG_CUDA(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->device));
  const size_t jac = (size_t)m_max * (2 * m_max + 1) * sizeof(float), jac_h = (size_t)m_max * (m_max + 1) * sizeof(float);
  a.jac_smem_m = 0;
  a.jac_q_smem = 0;
  if (wsm + jac <= (size_t)smem_optin) {
    a.jac_smem_m = m_max;
    a.jac_q_smem = 1;
    wsm += jac;
  } else if (wsm + jac_h <= (size_t)smem_optin) {
    a.jac_smem_m = m_max;
    wsm += jac_h;
  }
  // two CTAs of half the threads per SM when two fit in its shared memory
  // (small eigen-problems): the factorisation steps are latency-bound, so
  // each SM serves two cuts for little more than one cut's time
  int threads = h->tune[BSG_TUNE_FACTOR_THREADS];
  if (h->tune[BSG_TUNE_FACTOR_DUAL] && threads >= 512) {
    int smem_sm = 0, reserved = 0;
    BSG_CUDA(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, h->device));
    BSG_CUDA(cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, h->device));
    if (2 * (wsm + (size_t)reserved + 64) <= (size_t)smem_sm) threads /= 2;
  }
  BSG_CUDA(cudaFuncSetAttribute(williamson_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)wsm));
  BSG_PROFILED(h, BSG_K_WILLIAMSON, st, 0.0, (williamson_kernel<<<c1 - c0, threads, wsm, st>>>(a)));
  return BSG_OK;
}

// Dynamic shared memory of a Williamson launch whose largest eigen-problem
// is m_max (the FP32 Jacobi matrices in shared memory when they fit).
static int williamson_smem(bsg_handle_t h, int m_max, size_t* wsm, int* jac_m, int* jac_q) {
  *wsm = (40 + 2 * kMaxCutModes) * 8 + 4 * kMaxCutModes * 4 + 6 * kMaxCutModes * 8 + kDfSmemBytes;
  int smem_optin = 0;
  BSG_CUDA(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->device));
  const size_t jac = (size_t)m_max * (2 * m_max + 1) * sizeof(float), jac_h = (size_t)m_max * (m_max + 1) * sizeof(float);
  *jac_m = 0;
  *jac_q = 0;
  if (*wsm + jac <= (size_t)smem_optin) {
    *jac_m = m_max;
    *jac_q = 1;
    *wsm += jac;
  } else if (*wsm + jac_h <= (size_t)smem_optin) {
    *jac_m = m_max;
    *wsm += jac_h;
  }
  return BSG_OK;
}

// Williamson, then top-chi selection, of every cut of n independent
// instances (their CutArgs, from cut_prepare_at), one launch each: block b
// takes one (instance, cut).  dev: device room for n CutArgs and the block
// map (batch_dev_bytes); stage: pinned host room of the same size.
size_t cut_batch_bytes(const CutArgs* args, int n) {
  size_t cuts = 0;
  for (int i = 0; i < n; ++i) cuts += (size_t)args[i].n_cuts;
  return al256(sizeof(CutArgs) * n) + al256(sizeof(int2) * cuts);
}

int cut_launch_batch(bsg_handle_t h, CutArgs* args, int n, void* dev, void* stage, cudaStream_t st) {
  int m_max = 0, total = 0, thermal_smem_max = 0;
  double ranked = 0.0;
  for (int i = 0; i < n; ++i) {
    CutArgs& a = args[i];
    a.c0 = 0;
    for (int c = 0; c < a.n_cuts; ++c) {
      const int L = a.L0 + c, k = a.M - L;
      m_max = std::max(m_max, 2 * std::min(L, k));
      ranked += (double)(a.M - a.L0 - c) * a.chi * a.d;
    }
    total += a.n_cuts;
    thermal_smem_max = std::max(thermal_smem_max, a.d * a.chi * 8 + 2 * a.chi * 8 + 64 * 8);
  }
  if (total == 0) return BSG_OK;
  size_t wsm = 0;
  int jac_m = 0, jac_q = 0;
  BSG_TRY(williamson_smem(h, m_max, &wsm, &jac_m, &jac_q));
  for (int i = 0; i < n; ++i) {
    args[i].jac_smem_m = jac_m;
    args[i].jac_q_smem = jac_q;
  }
  char* hs = reinterpret_cast<char*>(stage);
  std::memcpy(hs, args, sizeof(CutArgs) * n);
  int2* map = reinterpret_cast<int2*>(hs + al256(sizeof(CutArgs) * n));
  int b = 0;
  for (int i = 0; i < n; ++i)
    for (int c = 0; c < args[i].n_cuts; ++c) map[b++] = make_int2(i, c);
  BSG_CUDA(cudaMemcpyAsync(dev, stage, al256(sizeof(CutArgs) * n) + sizeof(int2) * total, cudaMemcpyHostToDevice, st));
  const CutArgs* dargs = reinterpret_cast<const CutArgs*>(dev);
  const int2* dmap = reinterpret_cast<const int2*>(reinterpret_cast<char*>(dev) + al256(sizeof(CutArgs) * n));
  BSG_CUDA(cudaFuncSetAttribute(williamson_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)wsm));
  BSG_PROFILED(h, BSG_K_WILLIAMSON, st, 0.0,
               (williamson_batch_kernel<<<total, h->tune[BSG_TUNE_FACTOR_THREADS], wsm, st>>>(dargs, dmap)));
  BSG_CUDA(cudaFuncSetAttribute(thermal_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, thermal_smem_max));
  BSG_PROFILED(h, BSG_K_THERMAL, st, ranked, (thermal_batch_kernel<<<total, 1024, thermal_smem_max, st>>>(dargs, dmap)));
  return BSG_OK;
}

// Top-chi selection of cuts [c0, c1) (after their Williamson launches).
int cut_launch_thermal(bsg_handle_t h, const CutArgs& args, int c0, int c1, cudaStream_t st) {
  if (c1 <= c0) return BSG_OK;
  CutArgs a = args;
  a.c0 = c0;
  const size_t tsm = (size_t)a.d * a.chi * 8 + 2 * (size_t)a.chi * 8 + 64 * 8;
  BSG_CUDA(cudaFuncSetAttribute(thermal_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tsm));
  double ranked = 0.0;
  for (int c = c0; c < c1; ++c) ranked += (double)(a.M - a.L0 - c) * a.chi * a.d;
  BSG_PROFILED(h, BSG_K_THERMAL, st, ranked, (thermal_kernel<<<c1 - c0, 1024, tsm, st>>>(a)));
  return BSG_OK;
}

// Copies the phase timestamps of the last profiled launch into the profiler
// (synchronises `st`; profiling only).
int cut_read_phases(bsg_handle_t h, const CutArgs& a, cudaStream_t st) {
  if (!a.phase_t) return BSG_OK;
  std::vector<unsigned long long> t((size_t)a.n_cuts * kCutPhases);
  BSG_CUDA(cudaMemcpyAsync(t.data(), a.phase_t, t.size() * 8, cudaMemcpyDeviceToHost, st));
  BSG_CUDA(cudaStreamSynchronize(st));
  h->prof.cut_phases.assign(t.size(), 0.0);
  for (int c = 0; c < a.n_cuts; ++c) {
    // a phase the cut skipped (the other path's stamp) is charged to the next one
    unsigned long long prev = t[(size_t)c * kCutPhases];
    for (int i = 1; i < kCutTimedPhases; ++i) {
      const unsigned long long v = t[(size_t)c * kCutPhases + i];
      if (v == 0 || prev == 0) continue;
      h->prof.cut_phases[(size_t)c * kCutPhases + i] = double(v - prev) * 1e-6;
      prev = v;
    }
    for (int i = kCutTimedPhases; i < kCutPhases; ++i)
      h->prof.cut_phases[(size_t)c * kCutPhases + i] = double(t[(size_t)c * kCutPhases + i]);
    for (int i = kCutTimedPhases + 2; i < kCutPhases; ++i) h->prof.cut_phases[(size_t)c * kCutPhases + i] *= 1e-6;  // ns -> ms
  }
  return BSG_OK;
}

int cut_queue_status(const CutArgs& a, int c0, int c1, int* hst, cudaStream_t st) {
  if (c1 <= c0) return BSG_OK;
  BSG_CUDA(cudaMemcpyAsync(hst + c0, a.status + c0, (size_t)(c1 - c0) * 4, cudaMemcpyDeviceToHost, st));
  BSG_CUDA(cudaMemcpyAsync(hst + a.n_cuts + c0, a.sweeps + c0, (size_t)(c1 - c0) * 4, cudaMemcpyDeviceToHost, st));
  return BSG_OK;
}

// Decodes the status of cuts [c0, c1) and adds their Williamson FMA count
// to the profiler.
int cut_check_status(bsg_handle_t h, const CutArgs& a, int c0, int c1, const int* status) {
  const int M = a.M, L0 = a.L0;
  // FP64 FMAs of the Williamson step: Cholesky n^3/3, L^-1 n^3/6, G n^3,
  // pairing ~n^3 (G x per pair, projections), S n^3/2; full path: H n^3 and
  // 12 n^3 for three refinement steps of the eigen-decomposition (its Jacobi
  // sweeps run in FP32); low-rank path (m = 2L < n): Cholesky m^3/3,
  // L_A^-1 C m^2 n/2, F n^2 m/2, QR 2 n m^2, K m^3/2, 12 m^3 refinement, Q z 2 n^2 m
  double fmas = 0.0;
  for (int c = c0; c < c1; ++c) {
    const double n = 2.0 * (M - L0 - c), m = 2.0 * (L0 + c);
    fmas += n * n * n * (1.0 / 3 + 1.0 / 6 + 1.0 + 1.0 + 0.5);
    if (m >= n) fmas += n * n * n * (1.0 + 12.0);
    else fmas += m * m * m / 3 + m * m * n / 2 + n * n * m / 2 + 2 * n * m * m + m * m * m / 2 + 12 * m * m * m + 2 * n * n * m;
  }
  h->prof.add_work(BSG_K_WILLIAMSON, fmas);
  for (int c = c0; c < c1; ++c) {
    if (status[c] == 1) {
      set_error("cut %d: the input matrix is not symmetric", L0 + c);
      return BSG_ERR_NOT_PD;
    }
    if (status[c] == 2) {
      set_error("cut %d: input matrix is not positive definite", L0 + c);
      return BSG_ERR_NOT_PD;
    }
    if (status[c] == 3) {
      set_error("cut %d: Jacobi eigen-solver did not converge", L0 + c);
      return BSG_ERR_NO_CONVERGE;
    }
    if (status[c] == 4) {
      set_error("cut %d: symplectic eigenvector pairing failed", L0 + c);
      return BSG_ERR_NO_CONVERGE;
    }
    if (status[c] != 0) {
      set_error("cut %d: Williamson kernel did not finish (status %d)", L0 + c, status[c]);
      return BSG_ERR_CUDA;
    }
  }
  return BSG_OK;
}

}  // namespace bsg

extern "C" int bsg_cut_spectra(bsg_handle_t h, const double* sq_cov, int M, int L0, int n_cuts, int d, int chi,
                               double err_tol, double* res, int8_t* num, double* S, int32_t* kept,
                               bsg_stream_t stream) {
  BSG_CHECK_ARG(h, "bsg_cut_spectra: null handle");
  BSG_CHECK_ARG(sq_cov && res && num && S && kept, "bsg_cut_spectra: null pointer");
  BSG_CUDA(cudaSetDevice(h->device));
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  CutArgs a;
  BSG_TRY(cut_prepare(h, sq_cov, M, L0, n_cuts, d, chi, err_tol, res, num, S, kept, &a, st));
  BSG_TRY(cut_launch_williamson(h, a, 0, n_cuts, st));
  BSG_TRY(cut_launch_thermal(h, a, 0, n_cuts, st));
  std::vector<int> status(2 * n_cuts);
  BSG_TRY(cut_queue_status(a, 0, n_cuts, status.data(), st));
  BSG_CUDA(cudaStreamSynchronize(st));
  BSG_TRY(cut_read_phases(h, a, st));
  return cut_check_status(h, a, 0, n_cuts, status.data());
}

extern "C" int bsg_cut_spectrum(bsg_handle_t h, const double* sq_cov, int M, int L, int d, int chi, double err_tol,
                                int64_t max_dim, double* res, int8_t* num, double* S, int32_t* kept,
                                bsg_stream_t stream) {
  BSG_CHECK_ARG(max_dim >= chi,
                "bsg_cut_spectrum: max_dim=%lld is below chi=%d (the per-step top-chi selection reproduces the "
                "reference's candidate cap only when max_dim >= chi)",
                (long long)max_dim, chi);
  return bsg_cut_spectra(h, sq_cov, M, L, 1, d, chi, err_tol, res, num, S, kept, stream);
}
