// Covariance decomposition on the GPU: the pure quantum part of a Gaussian
// covariance (get_decomposition.py:16-29).
//
//   minimise tr X  subject to  S1 = [[X, Omega], [-Omega, X]] >= 0,  S2 = cov - X >= 0
//
// (Omega = kron([[0, 1], [-1, 0]], I_M), xxpp order, n = 2M).  The reference
// hands this SDP to cvxpy/CVXOPT (get_decomposition.py:27).  Here it is
// solved by an infeasible-start primal-dual interior-point method with the
// HKM search direction and Mehrotra's predictor-corrector, every step on the
// device in FP64:
//
// * the Newton system reduces to the HKM Schur complement on the n(n+1)/2
//   free entries of X (svec basis): M_ab = tr(A1(E_a) S1^-1 A1(E_b) Z1) +
//   tr(E_a S2^-1 E_b Z2), assembled entry by entry (schur_kernel) and
//   factored by a blocked right-looking Cholesky (64 x 64 tiles: one CTA
//   factors the diagonal tile, one CTA per tile row solves the panel, the
//   trailing update is a lower-triangle tiled FP64 GEMM);
// * S1^-1 and S2^-1 come from the same Cholesky, a column-parallel inverse of
//   the factor and one GEMM;
// * step lengths: the largest step keeping S + a dS positive definite,
//   bracketed by batched Cholesky tests (one CTA per candidate step, 32
//   candidates on a geometric grid, then two rounds of 16 inside the bracket).
//
// Everything is bounded: the loop stops after max_iter iterations, every
// kernel runs a fixed trip count, and no kernel waits on another.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "bsg_internal.h"

namespace bsg {
namespace {

constexpr int kT = 64;  // Cholesky / GEMM tile

// ---------------------------------------------------------------------------
// C = alpha op(A) op(B) + beta C (row-major FP64).  64 x 64 output tile per
// CTA, 256 threads with 4 x 4 outputs each (rows ty + 16 p, columns tx + 16 q),
// K in chunks of 16 through shared memory.  tri: C is square and only its
// lower-triangle tiles are computed (blockIdx.x enumerates them row by row).
// ---------------------------------------------------------------------------
struct GemmArgs {
  const double* A;
  const double* B;
  double* C;
  int M, N, K, lda, ldb, ldc;
  int ta, tb, tri;
  double alpha, beta;
};

__global__ void __launch_bounds__(256) gemm_f64_kernel(GemmArgs g) {
  int ti, tj;
  if (g.tri) {
    const int b = blockIdx.x;
    int r = int((sqrt(8.0 * b + 1.0) - 1.0) * 0.5);
    while ((r + 1) * (r + 2) / 2 <= b) ++r;
    while (r > 0 && r * (r + 1) / 2 > b) --r;
    ti = r;
    tj = b - r * (r + 1) / 2;
  } else {
    ti = blockIdx.y;
    tj = blockIdx.x;
  }
  const int r0 = ti * kT, c0 = tj * kT;
  __shared__ double As[16][kT + 1];
  __shared__ double Bs[16][kT + 1];
  const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;
  double acc[4][4];
#pragma unroll
  for (int p = 0; p < 4; ++p)
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[p][q] = 0.0;
  for (int k0 = 0; k0 < g.K; k0 += 16) {
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int e = tid + 256 * u;
      int r, k;
      if (g.ta) { r = e & 63; k = e >> 6; } else { k = e & 15; r = e >> 4; }
      const int gr = r0 + r, gk = k0 + k;
      double v = 0.0;
      if (gr < g.M && gk < g.K) v = g.ta ? g.A[(size_t)gk * g.lda + gr] : g.A[(size_t)gr * g.lda + gk];
      As[k][r] = v;
      int c;
      if (g.tb) { k = e & 15; c = e >> 4; } else { c = e & 63; k = e >> 6; }
      const int gc = c0 + c, gk2 = k0 + k;
      double w = 0.0;
      if (gc < g.N && gk2 < g.K) w = g.tb ? g.B[(size_t)gc * g.ldb + gk2] : g.B[(size_t)gk2 * g.ldb + gc];
      Bs[k][c] = w;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 16; ++kk) {
      double a[4], b[4];
#pragma unroll
      for (int p = 0; p < 4; ++p) a[p] = As[kk][ty + 16 * p];
#pragma unroll
      for (int q = 0; q < 4; ++q) b[q] = Bs[kk][tx + 16 * q];
#pragma unroll
      for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[p][q] = fma(a[p], b[q], acc[p][q]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int p = 0; p < 4; ++p) {
    const int gr = r0 + ty + 16 * p;
    if (gr >= g.M) continue;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int gc = c0 + tx + 16 * q;
      if (gc >= g.N) continue;
      double* cp = g.C + (size_t)gr * g.ldc + gc;
      *cp = g.beta == 0.0 ? g.alpha * acc[p][q] : fma(g.alpha, acc[p][q], g.beta * *cp);
    }
  }
}

int gemm(const double* A, int lda, int ta, const double* B, int ldb, int tb, double* C, int ldc, int M, int N, int K,
         double alpha, double beta, cudaStream_t st, bool tri = false) {
  if (M <= 0 || N <= 0) return BSG_OK;
  GemmArgs g{A, B, C, M, N, K, lda, ldb, ldc, ta, tb, tri ? 1 : 0, alpha, beta};
  const int tm = (M + kT - 1) / kT, tn = (N + kT - 1) / kT;
  if (tri) {
    gemm_f64_kernel<<<unsigned((int64_t)tm * (tm + 1) / 2), 256, 0, st>>>(g);
  } else {
    gemm_f64_kernel<<<dim3(tn, tm), 256, 0, st>>>(g);
  }
  BSG_CUDA(cudaGetLastError());
  return BSG_OK;
}

// ---------------------------------------------------------------------------
// Blocked Cholesky (lower, in place, row-major) with a device failure flag:
// *info = (global column + 1) of the first non-positive pivot, else 0.
// ---------------------------------------------------------------------------
__global__ void potrf_tile_kernel(double* A, int lda, int n, int k0, int* info) {
  __shared__ double s[kT][kT + 1];
  __shared__ int bad;
  if (*reinterpret_cast<volatile int*>(info)) return;
  const int tb = min(kT, n - k0);
  for (int e = threadIdx.x; e < tb * tb; e += blockDim.x) {
    const int r = e / tb, c = e % tb;
    s[r][c] = c <= r ? A[(size_t)(k0 + r) * lda + k0 + c] : 0.0;
  }
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  for (int j = 0; j < tb; ++j) {
    if (threadIdx.x == 0) {
      const double d = s[j][j];
      if (!(d > 0.0)) bad = 1;
      else s[j][j] = sqrt(d);
    }
    __syncthreads();
    if (bad) {
      if (threadIdx.x == 0) atomicCAS(info, 0, k0 + j + 1);
      return;
    }
    const double djj = s[j][j];
    for (int i = j + 1 + threadIdx.x; i < tb; i += blockDim.x) s[i][j] /= djj;
    __syncthreads();
    const int w = tb - j - 1;
    for (int e = threadIdx.x; e < w * w; e += blockDim.x) {
      const int i = j + 1 + e / w, c = j + 1 + e % w;
      if (c <= i) s[i][c] -= s[i][j] * s[c][j];
    }
    __syncthreads();
  }
  for (int e = threadIdx.x; e < tb * tb; e += blockDim.x) {
    const int r = e / tb, c = e % tb;
    if (c <= r) A[(size_t)(k0 + r) * lda + k0 + c] = s[r][c];
  }
}

// Rows below the diagonal tile k0: A_ik <- A_ik L_kk^-T (one CTA per 64-row block).
// Dynamic shared memory: the diagonal tile and the 64-row block, kTrsmSmem bytes.
constexpr int kTrsmSmem = 2 * kT * (kT + 1) * (int)sizeof(double);

__global__ void trsm_panel_kernel(double* A, int lda, int n, int k0, const int* info) {
  extern __shared__ double trsm_sm[];
  double (*L)[kT + 1] = reinterpret_cast<double (*)[kT + 1]>(trsm_sm);
  double (*X)[kT + 1] = reinterpret_cast<double (*)[kT + 1]>(trsm_sm + kT * (kT + 1));
  if (*reinterpret_cast<const volatile int*>(info)) return;
  const int tb = min(kT, n - k0);
  const int row0 = k0 + tb + blockIdx.x * kT;
  const int rb = min(kT, n - row0);
  if (rb <= 0) return;
  for (int e = threadIdx.x; e < tb * tb; e += blockDim.x) {
    const int r = e / tb, c = e % tb;
    L[r][c] = c <= r ? A[(size_t)(k0 + r) * lda + k0 + c] : 0.0;
  }
  for (int e = threadIdx.x; e < rb * tb; e += blockDim.x) {
    const int r = e / tb, c = e % tb;
    X[r][c] = A[(size_t)(row0 + r) * lda + k0 + c];
  }
  __syncthreads();
  if (threadIdx.x < rb) {
    const int r = threadIdx.x;
    for (int c = 0; c < tb; ++c) {
      double v = X[r][c];
      for (int p = 0; p < c; ++p) v -= X[r][p] * L[c][p];
      X[r][c] = v / L[c][c];
    }
  }
  __syncthreads();
  for (int e = threadIdx.x; e < rb * tb; e += blockDim.x) {
    const int r = e / tb, c = e % tb;
    A[(size_t)(row0 + r) * lda + k0 + c] = X[r][c];
  }
}

int potrf(double* A, int n, int lda, int* info_dev, cudaStream_t st) {
  BSG_CUDA(cudaFuncSetAttribute(trsm_panel_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kTrsmSmem));
  BSG_CUDA(cudaMemsetAsync(info_dev, 0, sizeof(int), st));
  for (int k0 = 0; k0 < n; k0 += kT) {
    const int tb = std::min(kT, n - k0);
    potrf_tile_kernel<<<1, 256, 0, st>>>(A, lda, n, k0, info_dev);
    BSG_CUDA(cudaGetLastError());
    const int rest = n - k0 - tb;
    if (rest <= 0) continue;
    trsm_panel_kernel<<<(rest + kT - 1) / kT, 128, kTrsmSmem, st>>>(A, lda, n, k0, info_dev);
    BSG_CUDA(cudaGetLastError());
    double* P = A + (size_t)(k0 + tb) * lda + k0;
    BSG_TRY(gemm(P, lda, 0, P, lda, 1, A + (size_t)(k0 + tb) * lda + k0 + tb, lda, rest, rest, tb, -1.0, 1.0, st,
                 true));
  }
  return BSG_OK;
}

// ---------------------------------------------------------------------------
// Blocked triangular solves of one vector with the factor above: forward
// L y = b, then backward L^T x = y (in place).
// ---------------------------------------------------------------------------
__global__ void trsv_tile_kernel(const double* L, int ld, int n, int k0, double* b, int trans) {
  __shared__ double s[kT][kT + 1];
  __shared__ double x[kT];
  const int tb = min(kT, n - k0);
  for (int e = threadIdx.x; e < tb * tb; e += blockDim.x) {
    const int r = e / tb, c = e % tb;
    s[r][c] = c <= r ? L[(size_t)(k0 + r) * ld + k0 + c] : 0.0;
  }
  if (threadIdx.x < tb) x[threadIdx.x] = b[k0 + threadIdx.x];
  __syncthreads();
  const int t = threadIdx.x;
  if (!trans) {
    for (int c = 0; c < tb; ++c) {
      if (t == 0) x[c] /= s[c][c];
      __syncthreads();
      if (t > c && t < tb) x[t] -= s[t][c] * x[c];
      __syncthreads();
    }
  } else {
    for (int c = tb - 1; c >= 0; --c) {
      if (t == 0) x[c] /= s[c][c];
      __syncthreads();
      if (t < c) x[t] -= s[c][t] * x[c];
      __syncthreads();
    }
  }
  if (t < tb) b[k0 + t] = x[t];
}

// !trans: b[i] -= sum_c L[i][k0 + c] b[k0 + c] for i >= k0 + tb (a warp per row);
// trans:  b[j] -= sum_c L[k0 + c][j] b[k0 + c] for j < k0 (a thread per column).
__global__ void gemv_panel_kernel(const double* L, int ld, int n, int k0, double* b, int trans) {
  const int tb = min(kT, n - k0);
  if (!trans) {
    const int lane = threadIdx.x & 31;
    const int i = k0 + tb + blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (i >= n) return;
    double v = 0.0;
    for (int c = lane; c < tb; c += 32) v += L[(size_t)i * ld + k0 + c] * b[k0 + c];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) b[i] -= v;
  } else {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= k0) return;
    double v = 0.0;
    for (int c = 0; c < tb; ++c) v += L[(size_t)(k0 + c) * ld + j] * b[k0 + c];
    b[j] -= v;
  }
}

int potrs(const double* L, int n, int ld, double* b, cudaStream_t st) {
  for (int k0 = 0; k0 < n; k0 += kT) {
    trsv_tile_kernel<<<1, kT, 0, st>>>(L, ld, n, k0, b, 0);
    BSG_CUDA(cudaGetLastError());
    const int rest = n - std::min(n, k0 + kT);
    if (rest > 0) {
      gemv_panel_kernel<<<(rest + 7) / 8, 256, 0, st>>>(L, ld, n, k0, b, 0);
      BSG_CUDA(cudaGetLastError());
    }
  }
  const int last = ((n - 1) / kT) * kT;
  for (int k0 = last; k0 >= 0; k0 -= kT) {
    trsv_tile_kernel<<<1, kT, 0, st>>>(L, ld, n, k0, b, 1);
    BSG_CUDA(cudaGetLastError());
    if (k0 > 0) {
      gemv_panel_kernel<<<(k0 + 255) / 256, 256, 0, st>>>(L, ld, n, k0, b, 1);
      BSG_CUDA(cudaGetLastError());
    }
  }
  return BSG_OK;
}

// W = L^-1 for a lower-triangular L (a thread per column; column j is zero
// above row j).
__global__ void trinv_lower_kernel(const double* L, int ld, int n, double* W, int ldw) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  for (int i = 0; i < j; ++i) W[(size_t)i * ldw + j] = 0.0;
  for (int i = j; i < n; ++i) {
    double v = i == j ? 1.0 : 0.0;
    for (int k = j; k < i; ++k) v -= L[(size_t)i * ld + k] * W[(size_t)k * ldw + j];
    W[(size_t)i * ldw + j] = v / L[(size_t)i * ld + i];
  }
}

// ---------------------------------------------------------------------------
// Element-wise helpers (square matrices, row-major)
// ---------------------------------------------------------------------------
// out = a x + b y (+ c I when c != 0)
__global__ void axpby_kernel(int64_t len, int nd, double a, const double* x, double b, const double* y, double c,
                             double* out) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= len) return;
  double v = a != 0.0 ? a * x[e] : 0.0;  // a zero coefficient never reads its operand
  if (y && b != 0.0) v += b * y[e];
  if (c != 0.0 && nd > 0 && e / nd == e % nd) v += c;
  out[e] = v;
}

// A <- (A + A^T) / 2
__global__ void sym_kernel(double* A, int n) {
  const int i = blockIdx.y * 16 + threadIdx.y, j = blockIdx.x * 16 + threadIdx.x;
  if (i >= n || j >= n || j <= i) return;
  const double v = 0.5 * (A[(size_t)i * n + j] + A[(size_t)j * n + i]);
  A[(size_t)i * n + j] = v;
  A[(size_t)j * n + i] = v;
}

// out (n x n) = s * (U11 + U22) of a 2n x 2n matrix (the adjoint of A1)
__global__ void a1_adj_kernel(const double* U, int n, double s, double* out, int accumulate) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (int64_t)n * n) return;
  const int i = int(e / n), j = int(e % n);
  const double v = s * (U[(size_t)i * 2 * n + j] + U[(size_t)(n + i) * 2 * n + n + j]);
  out[e] = accumulate ? out[e] + v : v;
}

// out (2n x 2n) = a [[X, 0], [0, X]] + b R (+ C1 scaled by c, C1 = [[0, Om], [-Om, 0]],
// Om = [[0, I], [-I, 0]] (M = n / 2))
__global__ void a1_kernel(const double* X, int n, double a, const double* R, double b, double c, double* out) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int n2 = 2 * n;
  if (e >= (int64_t)n2 * n2) return;
  const int i = int(e / n2), j = int(e % n2);
  double v = 0.0;
  if (a != 0.0 && (i < n) == (j < n)) v = a * X[(size_t)(i % n) * n + (j % n)];
  if (R && b != 0.0) v += b * R[e];
  if (c != 0.0 && (i < n) != (j < n)) {
    // C1[i][j] = Om[i][j - n] (upper right) or -Om[i - n][j] (lower left)
    const int r = i < n ? i : i - n, q = i < n ? j - n : j;
    const int M = n / 2;
    double om = 0.0;
    if (r < M && q == r + M) om = 1.0;
    if (r >= M && q == r - M) om = -1.0;
    v += (i < n ? c : -c) * om;
  }
  out[e] = v;
}

// Dot products <a_k, b_k> in two deterministic stages (block partials, then one sum per job).
struct DotJob {
  const double* a;
  const double* b;
  int64_t len;
};
constexpr int kDotBlocks = 64;

__global__ void dot_partial_kernel(const DotJob* jobs, double* partial) {
  const DotJob jb = jobs[blockIdx.y];
  double v = 0.0;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < jb.len; e += (int64_t)gridDim.x * blockDim.x)
    v += jb.a[e] * jb.b[e];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  __shared__ double s[32];
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += s[w];
    partial[blockIdx.y * kDotBlocks + blockIdx.x] = t;
  }
}

__global__ void dot_final_kernel(const double* partial, int n_jobs, double* out) {
  const int j = threadIdx.x;
  if (j >= n_jobs) return;
  double t = 0.0;
  for (int b = 0; b < kDotBlocks; ++b) t += partial[j * kDotBlocks + b];
  out[j] = t;
}

// svec / smat over the upper-triangle index list (i <= j), basis
// E_a = alpha_a (e_i e_j^T + e_j e_i^T), alpha = 1/sqrt(2) off the diagonal, 1/2 on it.
__global__ void svec_kernel(const double* A, int n, const int2* ij, int m, double* v) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= m) return;
  const int2 p = ij[a];
  v[a] = p.x == p.y ? A[(size_t)p.x * n + p.x] : 1.4142135623730951 * A[(size_t)p.x * n + p.y];
}

__global__ void smat_kernel(const double* v, int n, const int2* ij, int m, double* A) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= m) return;
  const int2 p = ij[a];
  if (p.x == p.y) {
    A[(size_t)p.x * n + p.x] = v[a];
  } else {
    const double w = 0.7071067811865476 * v[a];
    A[(size_t)p.x * n + p.y] = w;
    A[(size_t)p.y * n + p.x] = w;
  }
}

// HKM Schur complement, lower triangle: M_ab = alpha_a alpha_b sum over the
// pairs (P, Z) = (P1 block (p, q), Z1 block (q, p)), p, q in {0, 1}, and
// (P2, Z2) of  P_jk Z_li + P_jl Z_ki + P_ik Z_lj + P_il Z_kj  (a = (i, j), b = (k, l)).
__global__ void schur_kernel(const double* P1, const double* Z1, const double* P2, const double* Z2, int n,
                             const int2* ij, int m, double* Msc) {
  const int a = blockIdx.y * 16 + threadIdx.y, b = blockIdx.x * 16 + threadIdx.x;
  if (blockIdx.x > blockIdx.y || a >= m || b > a) return;
  const int2 pa = ij[a], pb = ij[b];
  const int i = pa.x, j = pa.y, k = pb.x, l = pb.y;
  const int N1 = 2 * n;
  double v = 0.0;
#pragma unroll
  for (int p = 0; p < 2; ++p)
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const double* P = P1 + (size_t)p * n * N1 + q * n;  // block (p, q), leading dim N1
      const double* Z = Z1 + (size_t)q * n * N1 + p * n;  // block (q, p)
      v += P[(size_t)j * N1 + k] * Z[(size_t)l * N1 + i] + P[(size_t)j * N1 + l] * Z[(size_t)k * N1 + i] +
           P[(size_t)i * N1 + k] * Z[(size_t)l * N1 + j] + P[(size_t)i * N1 + l] * Z[(size_t)k * N1 + j];
    }
  v += P2[(size_t)j * n + k] * Z2[(size_t)l * n + i] + P2[(size_t)j * n + l] * Z2[(size_t)k * n + i] +
       P2[(size_t)i * n + k] * Z2[(size_t)l * n + j] + P2[(size_t)i * n + l] * Z2[(size_t)k * n + j];
  const double sa = i == j ? 0.5 : 0.7071067811865476, sb = k == l ? 0.5 : 0.7071067811865476;
  Msc[(size_t)a * m + b] = v * sa * sb;
}

// Positive-definiteness tests of S + alpha dS: CTA (c, job) copies the lower
// triangle into its workspace and runs a right-looking Cholesky there;
// ok[job * n_alpha + c] = 1 if every pivot was positive.
struct PdJob {
  const double* S;
  const double* dS;
  int n;
};

__global__ void __launch_bounds__(512) pd_test_kernel(const PdJob* jobs, const double* alphas, int n_alpha,
                                                      double* ws, size_t ws_stride, int* ok) {
  extern __shared__ double colj[];
  const PdJob jb = jobs[blockIdx.y];
  const int idx = blockIdx.y * n_alpha + blockIdx.x;
  const double al = alphas[idx];
  const int N = jb.n;
  double* T = ws + (size_t)idx * ws_stride;
  for (int64_t e = threadIdx.x; e < (int64_t)N * N; e += blockDim.x) {
    const int r = int(e / N), c = int(e % N);
    if (c <= r) T[e] = jb.S[e] + al * jb.dS[e];
  }
  __shared__ int bad;
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int j = 0; j < N; ++j) {
    if (threadIdx.x == 0) {
      const double d = T[(size_t)j * N + j];
      if (!(d > 0.0)) bad = 1;
      else T[(size_t)j * N + j] = sqrt(d);
    }
    __syncthreads();
    if (bad) break;
    const double djj = T[(size_t)j * N + j];
    for (int i = j + 1 + threadIdx.x; i < N; i += blockDim.x) {
      const double x = T[(size_t)i * N + j] / djj;
      T[(size_t)i * N + j] = x;
      colj[i] = x;
    }
    __syncthreads();
    for (int i = j + 1 + warp; i < N; i += nw) {
      const double lij = colj[i];
      for (int c = j + 1 + lane; c <= i; c += 32) T[(size_t)i * N + c] -= lij * colj[c];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) ok[idx] = bad ? 0 : 1;
}

}  // namespace

// ---------------------------------------------------------------------------
// The interior-point driver
// ---------------------------------------------------------------------------
struct DecompWs {
  int n, N1, m;
  double *V, *X, *S1, *S2, *Z1, *Z2, *Rp1, *Rp2, *Rd, *P1, *P2, *L1, *L2, *W, *T1, *T2, *G1, *G2, *dX, *dS1, *dS2,
      *dZ1, *dZ2, *aS1, *aS2, *aZ1, *aZ2, *base, *vec, *Msc, *pd_ws, *alphas, *partial, *dots;
  int2* ij;
  int *info, *ok;
  DotJob* djobs;
  PdJob* pjobs;
};

static constexpr int kPdAlphas = 32;

static unsigned blocks_for(int64_t len, int t = 256) { return unsigned((len + t - 1) / t); }

// Dots of up to 16 pairs: out[k] = <a_k, b_k>, returned on the host.
static int dots(DecompWs& w, const std::vector<DotJob>& jobs, double* host_out, double* stage, cudaStream_t st) {
  const int nj = int(jobs.size());
  std::memcpy(stage, jobs.data(), sizeof(DotJob) * nj);
  BSG_CUDA(cudaMemcpyAsync(w.djobs, stage, sizeof(DotJob) * nj, cudaMemcpyHostToDevice, st));
  dot_partial_kernel<<<dim3(kDotBlocks, nj), 256, 0, st>>>(w.djobs, w.partial);
  BSG_CUDA(cudaGetLastError());
  dot_final_kernel<<<1, 32, 0, st>>>(w.partial, nj, w.dots);
  BSG_CUDA(cudaGetLastError());
  BSG_CUDA(cudaMemcpyAsync(host_out, w.dots, sizeof(double) * nj, cudaMemcpyDeviceToHost, st));
  BSG_CUDA(cudaStreamSynchronize(st));
  return BSG_OK;
}

static int symmetrize(double* A, int n, cudaStream_t st) {
  const unsigned b = unsigned((n + 15) / 16);
  sym_kernel<<<dim3(b, b), dim3(16, 16), 0, st>>>(A, n);
  BSG_CUDA(cudaGetLastError());
  return BSG_OK;
}

// P = S^-1 by Cholesky (L), the inverse factor (W) and W^T W.
static int spd_inverse(const double* S, int n, double* L, double* W, double* P, int* info_dev, int* info_host,
                       cudaStream_t st) {
  BSG_CUDA(cudaMemcpyAsync(L, S, sizeof(double) * n * n, cudaMemcpyDeviceToDevice, st));
  BSG_TRY(potrf(L, n, n, info_dev, st));
  BSG_CUDA(cudaMemcpyAsync(info_host, info_dev, sizeof(int), cudaMemcpyDeviceToHost, st));
  BSG_CUDA(cudaStreamSynchronize(st));
  if (*info_host) {
    set_error("bsg_cov_decomposition: an iterate lost positive definiteness (pivot %d)", *info_host);
    return BSG_ERR_NO_CONVERGE;
  }
  trinv_lower_kernel<<<blocks_for(n, 64), 64, 0, st>>>(L, n, n, W, n);
  BSG_CUDA(cudaGetLastError());
  BSG_TRY(gemm(W, n, 1, W, n, 0, P, n, n, n, n, 1.0, 0.0, st));
  return symmetrize(P, n, st);
}

// out = sym(A B C) with n x n factors (T: scratch)
static int triple(const double* A, const double* B, const double* C, int n, double* T, double* out, cudaStream_t st) {
  BSG_TRY(gemm(A, n, 0, B, n, 0, T, n, n, n, n, 1.0, 0.0, st));
  BSG_TRY(gemm(T, n, 0, C, n, 0, out, n, n, n, n, 1.0, 0.0, st));
  return symmetrize(out, n, st);
}

// Largest step a (up to a_max) keeping every S_k + a dS_k positive
// definite: 32 candidates a_max 2^(-c/2), then two rounds of 16 inside the
// bracket; returns the largest candidate that passed (0 if none).
static int max_step(DecompWs& w, const PdJob* jobs, int nj, double a_max, double* host_alpha, int* host_ok,
                    double* stage, double* out, cudaStream_t st) {
  std::memcpy(stage, jobs, sizeof(PdJob) * nj);
  BSG_CUDA(cudaMemcpyAsync(w.pjobs, stage, sizeof(PdJob) * nj, cudaMemcpyHostToDevice, st));
  int nmax = 0;
  for (int k = 0; k < nj; ++k) nmax = std::max(nmax, jobs[k].n);
  const size_t smem = sizeof(double) * nmax;
  double lo = 0.0, hi = a_max;
  for (int round = 0; round < 3; ++round) {
    const int na = round == 0 ? kPdAlphas : 16;
    for (int k = 0; k < nj; ++k)
      for (int c = 0; c < na; ++c) {
        double a;
        if (round == 0) a = a_max * std::pow(2.0, -0.5 * c);
        else a = lo + (hi - lo) * (c + 1) / (na + 1);
        host_alpha[k * na + c] = a;
      }
    BSG_CUDA(cudaMemcpyAsync(w.alphas, host_alpha, sizeof(double) * nj * na, cudaMemcpyHostToDevice, st));
    pd_test_kernel<<<dim3(na, nj), 512, smem, st>>>(w.pjobs, w.alphas, na, w.pd_ws, (size_t)nmax * nmax, w.ok);
    BSG_CUDA(cudaGetLastError());
    BSG_CUDA(cudaMemcpyAsync(host_ok, w.ok, sizeof(int) * nj * na, cudaMemcpyDeviceToHost, st));
    BSG_CUDA(cudaStreamSynchronize(st));
    // a candidate passes when it passes for every job (each set {a : S + a dS > 0} is an interval from 0)
    double best = -1.0, fail = hi;
    for (int c = 0; c < na; ++c) {
      const double a = host_alpha[c];
      bool all = true;
      for (int k = 0; k < nj; ++k) all = all && host_ok[k * na + c];
      if (all) best = std::max(best, a);
      else fail = std::min(fail, a);
    }
    if (round == 0) {
      if (best == a_max) {
        *out = a_max;
        return BSG_OK;
      }
      if (best < 0) {
        *out = 0.0;
        return BSG_OK;
      }
      lo = best;
      hi = std::min(a_max, best * std::sqrt(2.0));
    } else {
      if (best > lo) lo = best;
      hi = std::min(hi, fail);
    }
  }
  *out = lo;
  return BSG_OK;
}

static int decompose(bsg_handle_t h, const double* cov, int M, double* out, double tol, int max_iter, double* info,
                     cudaStream_t st) {
  const int n = 2 * M, N1 = 2 * n;
  const int64_t m = (int64_t)n * (n + 1) / 2;
  BSG_CHECK_ARG(M >= 1 && m <= 200000, "bsg_cov_decomposition: M=%d outside [1, 315]", M);
  // workspace
  DecompWs w{};
  w.n = n;
  w.N1 = N1;
  w.m = int(m);
  const size_t nn = (size_t)n * n, NN = (size_t)N1 * N1;
  auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
  size_t off = 0;
  std::vector<std::pair<double**, size_t>> dbl = {
      {&w.V, nn},   {&w.X, nn},   {&w.S1, NN},  {&w.S2, nn},  {&w.Z1, NN},  {&w.Z2, nn},   {&w.Rp1, NN},
      {&w.Rp2, nn}, {&w.Rd, nn},  {&w.P1, NN},  {&w.P2, nn},  {&w.L1, NN},  {&w.L2, nn},   {&w.W, NN},
      {&w.T1, NN},  {&w.T2, NN},  {&w.G1, NN},  {&w.G2, nn},  {&w.dX, nn},  {&w.dS1, NN},  {&w.dS2, nn},
      {&w.dZ1, NN}, {&w.dZ2, nn}, {&w.aS1, NN}, {&w.aS2, nn}, {&w.aZ1, NN}, {&w.aZ2, nn},  {&w.base, nn},
      {&w.vec, (size_t)m},        {&w.alphas, 2 * kPdAlphas},   {&w.partial, 16 * kDotBlocks}, {&w.dots, 16},
      {&w.pd_ws, (size_t)2 * kPdAlphas * NN}, {&w.Msc, (size_t)m * m}};
  std::vector<size_t> offs;
  for (auto& d : dbl) {
    offs.push_back(off);
    off = al(off + d.second * sizeof(double));
  }
  const size_t o_ij = off;
  off = al(off + sizeof(int2) * m);
  const size_t o_info = off;
  off = al(off + 16);
  const size_t o_ok = off;
  off = al(off + sizeof(int) * 2 * kPdAlphas);
  const size_t o_dj = off;
  off = al(off + sizeof(DotJob) * 16);
  const size_t o_pj = off;
  off = al(off + sizeof(PdJob) * 4);
  {
    size_t free_b = 0, total_b = 0;
    BSG_CUDA(cudaMemGetInfo(&free_b, &total_b));
    if (off > h->decomp_ws.bytes && off - h->decomp_ws.bytes > free_b) {
      set_error("bsg_cov_decomposition: M=%d needs %.1f GB of device memory", M, off / 1e9);
      return BSG_ERR_LIMIT;
    }
  }
  BSG_TRY(h->decomp_ws.ensure(off));
  char* base = reinterpret_cast<char*>(h->decomp_ws.ptr);
  for (size_t k = 0; k < dbl.size(); ++k) *dbl[k].first = reinterpret_cast<double*>(base + offs[k]);
  w.ij = reinterpret_cast<int2*>(base + o_ij);
  w.info = reinterpret_cast<int*>(base + o_info);
  w.ok = reinterpret_cast<int*>(base + o_ok);
  w.djobs = reinterpret_cast<DotJob*>(base + o_dj);
  w.pjobs = reinterpret_cast<PdJob*>(base + o_pj);
  // pinned host room: index list, scalars, step candidates, job lists
  const size_t h_ij = 0, h_sc = al(sizeof(int2) * m), h_alpha = h_sc + 256, h_ok = h_alpha + al(sizeof(double) * 64),
               h_stage = h_ok + al(sizeof(int) * 64), h_bytes = h_stage + 1024;
  BSG_TRY(h->decomp_host.ensure(h_bytes));
  char* hb = reinterpret_cast<char*>(h->decomp_host.ptr);
  int2* hij = reinterpret_cast<int2*>(hb + h_ij);
  double* sc = reinterpret_cast<double*>(hb + h_sc);
  int* hinfo = reinterpret_cast<int*>(hb + h_sc + 240);
  double* halpha = reinterpret_cast<double*>(hb + h_alpha);
  int* hok = reinterpret_cast<int*>(hb + h_ok);
  double* stage = reinterpret_cast<double*>(hb + h_stage);
  {
    int64_t a = 0;
    for (int i = 0; i < n; ++i)
      for (int j = i; j < n; ++j) hij[a++] = make_int2(i, j);
    BSG_CUDA(cudaMemcpyAsync(w.ij, hij, sizeof(int2) * m, cudaMemcpyHostToDevice, st));
  }
  const unsigned bn = blocks_for(nn), bN = blocks_for(NN), bm = blocks_for(m);
  // V = sym(cov); X = 0; S = Z = xi I
  BSG_CUDA(cudaMemcpyAsync(w.V, cov, sizeof(double) * nn, cudaMemcpyDeviceToDevice, st));
  BSG_TRY(symmetrize(w.V, n, st));
  {
    std::vector<DotJob> j1 = {{w.V, w.V, (int64_t)nn}};
    BSG_TRY(dots(w, j1, sc, stage, st));
  }
  const double normV = std::sqrt(sc[0]);
  double vmax = 0.0;
  {
    // max |V| bounded by the Frobenius norm; the start only needs a scale
    vmax = normV;
  }
  const double xi = std::max({10.0, std::sqrt((double)n), vmax});
  BSG_CUDA(cudaMemsetAsync(w.X, 0, sizeof(double) * nn, st));
  axpby_kernel<<<bN, 256, 0, st>>>((int64_t)NN, N1, 0.0, w.Rp1, 0.0, nullptr, xi, w.S1);
  axpby_kernel<<<bn, 256, 0, st>>>((int64_t)nn, n, 0.0, w.Rp2, 0.0, nullptr, xi, w.S2);
  axpby_kernel<<<bN, 256, 0, st>>>((int64_t)NN, N1, 0.0, w.Rp1, 0.0, nullptr, xi, w.Z1);
  axpby_kernel<<<bn, 256, 0, st>>>((int64_t)nn, n, 0.0, w.Rp2, 0.0, nullptr, xi, w.Z2);
  BSG_CUDA(cudaGetLastError());
  const double nu = 3.0 * n, tau = 0.98;
  int it = 0, rc = BSG_ERR_NO_CONVERGE;
  double pobj = 0, dobj = 0, rel_gap = 0, pres = 0, dres = 0;
  for (it = 1; it <= max_iter; ++it) {
    // residuals: Rp1 = S1 - A1(X) - C1, Rp2 = S2 - V + X, Rd = A1*(Z1) - Z2 - I
    a1_kernel<<<bN, 256, 0, st>>>(w.X, n, -1.0, w.S1, 1.0, -1.0, w.Rp1);
    axpby_kernel<<<bn, 256, 0, st>>>((int64_t)nn, n, 1.0, w.S2, -1.0, w.V, 0.0, w.Rp2);
    axpby_kernel<<<bn, 256, 0, st>>>((int64_t)nn, n, 1.0, w.Rp2, 1.0, w.X, 0.0, w.Rp2);
    a1_adj_kernel<<<bn, 256, 0, st>>>(w.Z1, n, 1.0, w.Rd, 0);
    axpby_kernel<<<bn, 256, 0, st>>>((int64_t)nn, n, 1.0, w.Rd, -1.0, w.Z2, -1.0, w.Rd);
    BSG_CUDA(cudaGetLastError());
    // <Z1, C1> = sum over the off-diagonal blocks: a1_kernel(0, R=0, c=1) gives C1 in T1
    a1_kernel<<<bN, 256, 0, st>>>(w.X, n, 0.0, nullptr, 0.0, 1.0, w.T1);
    BSG_CUDA(cudaGetLastError());
    // trace X = <X, I>: I in T2 (n x n)
    axpby_kernel<<<bn, 256, 0, st>>>((int64_t)nn, n, 0.0, w.X, 0.0, nullptr, 1.0, w.T2);
    std::vector<DotJob> dj = {{w.X, w.T2, (int64_t)nn},    {w.Z1, w.T1, (int64_t)NN},   {w.Z2, w.V, (int64_t)nn},
                              {w.S1, w.Z1, (int64_t)NN},   {w.S2, w.Z2, (int64_t)nn},   {w.Rp1, w.Rp1, (int64_t)NN},
                              {w.Rp2, w.Rp2, (int64_t)nn}, {w.Rd, w.Rd, (int64_t)nn}};
    BSG_TRY(dots(w, dj, sc, stage, st));
    pobj = sc[0];
    dobj = -sc[1] - sc[2];
    const double gap = sc[3] + sc[4];
    const double mu = gap / nu;
    rel_gap = gap / (1.0 + std::fabs(pobj) + std::fabs(dobj));
    pres = std::max(std::sqrt(sc[5]), std::sqrt(sc[6])) / (1.0 + normV);
    dres = std::sqrt(sc[7]) / (1.0 + std::sqrt((double)n));
    if (rel_gap < tol && pres < tol && dres < tol) {
      rc = BSG_OK;
      break;
    }
    if (it == max_iter) break;
    // P = S^-1
    BSG_TRY(spd_inverse(w.S1, N1, w.L1, w.W, w.P1, w.info, hinfo, st));
    BSG_TRY(spd_inverse(w.S2, n, w.L2, w.W, w.P2, w.info, hinfo, st));
    // Schur complement and its factor (a tiny diagonal shift if rounding breaks definiteness)
    {
      const unsigned bt = unsigned((m + 15) / 16);
      schur_kernel<<<dim3(bt, bt), dim3(16, 16), 0, st>>>(w.P1, w.Z1, w.P2, w.Z2, n, w.ij, int(m), w.Msc);
      BSG_CUDA(cudaGetLastError());
      BSG_TRY(potrf(w.Msc, int(m), int(m), w.info, st));
      BSG_CUDA(cudaMemcpyAsync(hinfo, w.info, sizeof(int), cudaMemcpyDeviceToHost, st));
      BSG_CUDA(cudaStreamSynchronize(st));
      if (*hinfo) {
        set_error("bsg_cov_decomposition: the Schur complement lost definiteness at iteration %d (pivot %d)", it,
                  *hinfo);
        rc = BSG_ERR_NO_CONVERGE;
        break;
      }
    }
    // base = Rd + A1*(sym(P1 Rp1 Z1)) - sym(P2 Rp2 Z2)
    BSG_TRY(triple(w.P1, w.Rp1, w.Z1, N1, w.T1, w.T2, st));
    a1_adj_kernel<<<bn, 256, 0, st>>>(w.T2, n, 1.0, w.base, 0);
    BSG_CUDA(cudaGetLastError());
    BSG_TRY(triple(w.P2, w.Rp2, w.Z2, n, w.T1, w.dX, st));
    axpby_kernel<<<bn, 256, 0, st>>>((int64_t)nn, n, 1.0, w.base, -1.0, w.dX, 0.0, w.base);
    axpby_kernel<<<bn, 256, 0, st>>>((int64_t)nn, n, 1.0, w.base, 1.0, w.Rd, 0.0, w.base);
    BSG_CUDA(cudaGetLastError());
    // one Newton direction for targets G1, G2
    auto direction = [&]() -> int {
      // rhs = base + A1*(G1) - G2 (into dX), solved in the svec basis
      a1_adj_kernel<<<bn, 256, 0, st>>>(w.G1, n, 1.0, w.dX, 0);
      axpby_kernel<<<bn, 256, 0, st>>>((int64_t)nn, n, 1.0, w.dX, -1.0, w.G2, 0.0, w.dX);
      axpby_kernel<<<bn, 256, 0, st>>>((int64_t)nn, n, 1.0, w.dX, 1.0, w.base, 0.0, w.dX);
      svec_kernel<<<bm, 256, 0, st>>>(w.dX, n, w.ij, int(m), w.vec);
      BSG_CUDA(cudaGetLastError());
      BSG_TRY(potrs(w.Msc, int(m), int(m), w.vec, st));
      smat_kernel<<<bm, 256, 0, st>>>(w.vec, n, w.ij, int(m), w.dX);
      // dS1 = A1(dX) - Rp1, dS2 = -dX - Rp2
      a1_kernel<<<bN, 256, 0, st>>>(w.dX, n, 1.0, w.Rp1, -1.0, 0.0, w.dS1);
      axpby_kernel<<<bn, 256, 0, st>>>((int64_t)nn, n, -1.0, w.dX, -1.0, w.Rp2, 0.0, w.dS2);
      BSG_CUDA(cudaGetLastError());
      // dZ = G - sym(P dS Z)
      BSG_TRY(triple(w.P1, w.dS1, w.Z1, N1, w.T1, w.T2, st));
      axpby_kernel<<<bN, 256, 0, st>>>((int64_t)NN, N1, 1.0, w.G1, -1.0, w.T2, 0.0, w.dZ1);
      BSG_TRY(triple(w.P2, w.dS2, w.Z2, n, w.T1, w.T2, st));
      axpby_kernel<<<bn, 256, 0, st>>>((int64_t)nn, n, 1.0, w.G2, -1.0, w.T2, 0.0, w.dZ2);
      BSG_CUDA(cudaGetLastError());
      return BSG_OK;
    };
    // predictor: G = -Z
    axpby_kernel<<<bN, 256, 0, st>>>((int64_t)NN, N1, -1.0, w.Z1, 0.0, nullptr, 0.0, w.G1);
    axpby_kernel<<<bn, 256, 0, st>>>((int64_t)nn, n, -1.0, w.Z2, 0.0, nullptr, 0.0, w.G2);
    BSG_TRY(direction());
    double ap = 0, ad = 0;
    {
      const PdJob pj[2] = {{w.S1, w.dS1, N1}, {w.S2, w.dS2, n}};
      BSG_TRY(max_step(w, pj, 2, 1.0, halpha, hok, stage, &ap, st));
      const PdJob dj2[2] = {{w.Z1, w.dZ1, N1}, {w.Z2, w.dZ2, n}};
      BSG_TRY(max_step(w, dj2, 2, 1.0, halpha, hok, stage, &ad, st));
    }
    std::vector<DotJob> aj = {{w.S1, w.dZ1, (int64_t)NN},  {w.dS1, w.Z1, (int64_t)NN}, {w.dS1, w.dZ1, (int64_t)NN},
                              {w.S2, w.dZ2, (int64_t)nn},  {w.dS2, w.Z2, (int64_t)nn}, {w.dS2, w.dZ2, (int64_t)nn}};
    BSG_TRY(dots(w, aj, sc + 8, stage, st));
    const double mu_aff = (gap + ad * (sc[8] + sc[11]) + ap * (sc[9] + sc[12]) + ap * ad * (sc[10] + sc[13])) / nu;
    // Mehrotra's centring, kept >= 0.1: near the central path X converges
    // linearly in the gap (pure Mehrotra steps leave it ~sqrt(gap) away)
    const double sigma = std::max(0.1, std::min(1.0, std::pow(std::max(mu_aff, 0.0) / mu, 3.0)));
    // keep the affine step for the second-order term
    BSG_CUDA(cudaMemcpyAsync(w.aS1, w.dS1, sizeof(double) * NN, cudaMemcpyDeviceToDevice, st));
    BSG_CUDA(cudaMemcpyAsync(w.aZ1, w.dZ1, sizeof(double) * NN, cudaMemcpyDeviceToDevice, st));
    BSG_CUDA(cudaMemcpyAsync(w.aS2, w.dS2, sizeof(double) * nn, cudaMemcpyDeviceToDevice, st));
    BSG_CUDA(cudaMemcpyAsync(w.aZ2, w.dZ2, sizeof(double) * nn, cudaMemcpyDeviceToDevice, st));
    // corrector: G = sigma mu P - Z - sym(P dS_aff dZ_aff)
    BSG_TRY(triple(w.P1, w.aS1, w.aZ1, N1, w.T1, w.T2, st));
    axpby_kernel<<<bN, 256, 0, st>>>((int64_t)NN, N1, sigma * mu, w.P1, -1.0, w.Z1, 0.0, w.G1);
    axpby_kernel<<<bN, 256, 0, st>>>((int64_t)NN, N1, 1.0, w.G1, -1.0, w.T2, 0.0, w.G1);
    BSG_TRY(triple(w.P2, w.aS2, w.aZ2, n, w.T1, w.T2, st));
    axpby_kernel<<<bn, 256, 0, st>>>((int64_t)nn, n, sigma * mu, w.P2, -1.0, w.Z2, 0.0, w.G2);
    axpby_kernel<<<bn, 256, 0, st>>>((int64_t)nn, n, 1.0, w.G2, -1.0, w.T2, 0.0, w.G2);
    BSG_CUDA(cudaGetLastError());
    BSG_TRY(direction());
    {
      const PdJob pj[2] = {{w.S1, w.dS1, N1}, {w.S2, w.dS2, n}};
      double b = 0;
      BSG_TRY(max_step(w, pj, 2, 1.0 / tau, halpha, hok, stage, &b, st));
      ap = std::min(1.0, tau * b);
      const PdJob dj2[2] = {{w.Z1, w.dZ1, N1}, {w.Z2, w.dZ2, n}};
      BSG_TRY(max_step(w, dj2, 2, 1.0 / tau, halpha, hok, stage, &b, st));
      ad = std::min(1.0, tau * b);
    }
    if (ap <= 0.0 && ad <= 0.0) {
      set_error("bsg_cov_decomposition: no step keeps the iterates inside the cone (iteration %d)", it);
      break;
    }
    axpby_kernel<<<bn, 256, 0, st>>>((int64_t)nn, n, 1.0, w.X, ap, w.dX, 0.0, w.X);
    axpby_kernel<<<bN, 256, 0, st>>>((int64_t)NN, N1, 1.0, w.S1, ap, w.dS1, 0.0, w.S1);
    axpby_kernel<<<bn, 256, 0, st>>>((int64_t)nn, n, 1.0, w.S2, ap, w.dS2, 0.0, w.S2);
    axpby_kernel<<<bN, 256, 0, st>>>((int64_t)NN, N1, 1.0, w.Z1, ad, w.dZ1, 0.0, w.Z1);
    axpby_kernel<<<bn, 256, 0, st>>>((int64_t)nn, n, 1.0, w.Z2, ad, w.dZ2, 0.0, w.Z2);
    BSG_CUDA(cudaGetLastError());
    BSG_TRY(symmetrize(w.X, n, st));
    BSG_TRY(symmetrize(w.S1, N1, st));
    BSG_TRY(symmetrize(w.S2, n, st));
    BSG_TRY(symmetrize(w.Z1, N1, st));
    BSG_TRY(symmetrize(w.Z2, n, st));
  }
  BSG_TRY(symmetrize(w.X, n, st));
  BSG_CUDA(cudaMemcpyAsync(out, w.X, sizeof(double) * nn, cudaMemcpyDeviceToDevice, st));
  BSG_CUDA(cudaStreamSynchronize(st));
  if (info) {
    info[0] = std::min(it, max_iter);
    info[1] = rel_gap;
    info[2] = pres;
    info[3] = dres;
    info[4] = pobj;
    info[5] = dobj;
  }
  if (rc == BSG_ERR_NO_CONVERGE && it > max_iter - 1)
    set_error("bsg_cov_decomposition: no convergence to %.1e in %d iterations (gap %.2e)", tol, max_iter, rel_gap);
  return rc;
}

}  // namespace bsg

using namespace bsg;

extern "C" int bsg_cov_decomposition(bsg_handle_t h, const double* cov, int M, double* sq_cov, double tol,
                                     int max_iter, double* info, bsg_stream_t stream) {
  BSG_CHECK_ARG(h && cov && sq_cov, "bsg_cov_decomposition: null pointer");
  BSG_CHECK_ARG(tol > 0.0 && max_iter >= 1 && max_iter <= 1000, "bsg_cov_decomposition: need tol > 0, 1 <= max_iter "
                "<= 1000");
  BSG_CUDA(cudaSetDevice(h->device));
  return decompose(h, cov, M, sq_cov, tol, max_iter, info, reinterpret_cast<cudaStream_t>(stream));
}

extern "C" int bsg_potrf_f64(bsg_handle_t h, double* A, int n, int* info, bsg_stream_t stream) {
  BSG_CHECK_ARG(h && A && info, "bsg_potrf_f64: null pointer");
  BSG_CHECK_ARG(n >= 1, "bsg_potrf_f64: n=%d", n);
  BSG_CUDA(cudaSetDevice(h->device));
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  BSG_TRY(h->decomp_ws.ensure(256));
  int* dinfo = reinterpret_cast<int*>(h->decomp_ws.ptr);
  BSG_TRY(potrf(A, n, n, dinfo, st));
  BSG_CUDA(cudaMemcpyAsync(info, dinfo, sizeof(int), cudaMemcpyDeviceToHost, st));
  BSG_CUDA(cudaStreamSynchronize(st));
  return BSG_OK;
}
