// SIMT complex GEMM shared by the bond contraction and the sampler.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace bsg {

template <class R>
struct Cx;
template <>
struct Cx<float> {
  using T = float2;
};
template <>
struct Cx<double> {
  using T = double2;
};

// C[r, c] = sum_k (A[pidx[r], k] * lam[k]) * B(k, c) with B(k, c) = Bp[k*sk + c*sc]
// (complex; R = float: FP32 products and sums; R = double: FP64).
template <class R>
struct GemmArgs {
  const typename Cx<R>::T* A;  // [.., K] environment rows of the previous level
  const int32_t* pidx;         // [rows] parent row of each output row (null: row r)
  const double* lam;           // [K] or null
  const typename Cx<R>::T* B;  // Gamma slice base (already offset by n)
  int64_t sk, sc;
  typename Cx<R>::T* C;        // [rows, N]
  int rows, K, N;
};

constexpr int TM = 64, TN = 64, TK = 16;

template <class R>
__global__ void __launch_bounds__(256) cgemm_kernel(GemmArgs<R> g) {
  using T = typename Cx<R>::T;
  __shared__ T As[TK][TM + 1];
  __shared__ T Bs[TK][TN + 1];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;  // 16 x 16 threads, 4 x 4 outputs each
  const int r0 = blockIdx.y * TM, c0 = blockIdx.x * TN;
  R accr[4][4], acci[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) accr[i][j] = acci[i][j] = R(0);
  for (int k0 = 0; k0 < g.K; k0 += TK) {
    for (int t = threadIdx.x; t < TM * TK; t += 256) {
      const int rr = t / TK, kk = t % TK;
      const int r = r0 + rr, k = k0 + kk;
      T v;
      v.x = R(0);
      v.y = R(0);
      if (r < g.rows && k < g.K) {
        v = g.A[(int64_t)(g.pidx ? g.pidx[r] : r) * g.K + k];
        if (g.lam) {
          const R l = R(g.lam[k]);
          v.x *= l;
          v.y *= l;
        }
      }
      As[kk][rr] = v;
    }
    for (int t = threadIdx.x; t < TN * TK; t += 256) {
      const int kk = t / TN, cc = t % TN;
      const int k = k0 + kk, c = c0 + cc;
      T v;
      v.x = R(0);
      v.y = R(0);
      if (k < g.K && c < g.N) v = g.B[k * g.sk + c * g.sc];
      Bs[kk][cc] = v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < TK; ++kk) {
      T a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          accr[i][j] = fma(a[i].x, b[j].x, fma(-a[i].y, b[j].y, accr[i][j]));
          acci[i][j] = fma(a[i].x, b[j].y, fma(a[i].y, b[j].x, acci[i][j]));
        }
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int r = r0 + ty * 4 + i;
    if (r >= g.rows) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int c = c0 + tx * 4 + j;
      if (c < g.N) {
        T v;
        v.x = accr[i][j];
        v.y = acci[i][j];
        g.C[(int64_t)r * g.N + c] = v;
      }
    }
  }
}

}  // namespace bsg
