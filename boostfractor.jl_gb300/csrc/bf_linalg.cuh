// Dense complex linear algebra kernels of the transformer: tiled GEMM,
// batched Gauss-Jordan inversion, the per-frequency transfer-matrix chain and
// the FP64 boundary solve.  Templated on the complex type (float2 / double2).
#pragma once

#include "bf_common.cuh"

namespace bf {

// C[R][Ncol] = A[R][K] * B[K][Ncol] (row-major, complex), one 64x64 tile of C
// per CTA of 256 threads, each thread a 4x4 block; K staged in chunks of 16.
template <typename C>
__global__ void __launch_bounds__(256) k_cgemm(const C* __restrict__ A, const C* __restrict__ B,
                                               C* __restrict__ Cout, int R, int K, int Ncol) {
  constexpr int TM = 64, TN = 64, TK = 16;
  __shared__ C As[TK][TM + 1];
  __shared__ C Bs[TK][TN];
  const int tid = threadIdx.x;
  const int tr = tid / 16, tc = tid % 16;   // 16 x 16 threads, 4 x 4 outputs each
  const int r0 = blockIdx.y * TM, c0 = blockIdx.x * TN;
  C acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = mk(decltype(C().x)(0), decltype(C().x)(0));
  for (int k0 = 0; k0 < K; k0 += TK) {
    // A tile: 64 rows x 16 k
    for (int e = tid; e < TM * TK; e += 256) {
      const int rr = e / TK, kk = e % TK;
      const int gr = r0 + rr, gk = k0 + kk;
      As[kk][rr] = (gr < R && gk < K) ? A[(size_t)gr * K + gk] : mk(decltype(C().x)(0), decltype(C().x)(0));
    }
    for (int e = tid; e < TK * TN; e += 256) {
      const int kk = e / TN, cc = e % TN;
      const int gk = k0 + kk, gc = c0 + cc;
      Bs[kk][cc] = (gk < K && gc < Ncol) ? B[(size_t)gk * Ncol + gc] : mk(decltype(C().x)(0), decltype(C().x)(0));
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < TK; ++kk) {
      C a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][tr * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tc + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          acc[i][j].x += a[i].x * b[j].x - a[i].y * b[j].y;
          acc[i][j].y += a[i].x * b[j].y + a[i].y * b[j].x;
        }
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int gr = r0 + tr * 4 + i, gc = c0 + tc + 16 * j;
      if (gr < R && gc < Ncol) Cout[(size_t)gr * Ncol + gc] = acc[i][j];
    }
}

// ---- double-float (FP32 hi/lo pair) complex GEMM -----------------------------
// A complex number is a float4 (re_hi, re_lo, im_hi, im_lo) with re = re_hi +
// re_lo exactly representable to ~48 bits.  Products use the FMA-exact error
// of hi*hi plus the cross terms; sums use TwoSum, so a long, cancelling
// contraction keeps ~1e-14 relative accuracy on the FP32 pipes.
__device__ __forceinline__ float4 df_split(double2 v) {
  const float rh = (float)v.x, ih = (float)v.y;
  return make_float4(rh, (float)(v.x - (double)rh), ih, (float)(v.y - (double)ih));
}
__device__ __forceinline__ double2 df_join(float4 v) {
  return make_double2((double)v.x + (double)v.y, (double)v.z + (double)v.w);
}
// (sh, sl) += (xh + xl) * (yh + yl)
__device__ __forceinline__ void df_mac(float& sh, float& sl, float xh, float xl, float yh, float yl) {
  const float p = xh * yh;
  float e = fmaf(xh, yh, -p);
  e = fmaf(xh, yl, e);
  e = fmaf(xl, yh, e);
  const float t = sh + p;
  const float z = t - sh;
  const float err = (sh - (t - z)) + (p - z);
  sl += err + e;
  sh = t;
}

// C[R][Ncol] (complex128) = A[R][K] * B[K][Ncol], A and B double-float complex.
__global__ void __launch_bounds__(256) k_cgemm_df(const float4* __restrict__ A, const float4* __restrict__ B,
                                                  double2* __restrict__ Cout, int R, int K, int Ncol) {
  constexpr int TM = 64, TN = 64, TK = 8;
  __shared__ float4 As[TK][TM + 1];
  __shared__ float4 Bs[TK][TN];
  const int tid = threadIdx.x;
  const int tr = tid / 16, tc = tid % 16;
  const int r0 = blockIdx.y * TM, c0 = blockIdx.x * TN;
  // accumulators: real and imaginary parts as (hi, lo)
  float rh[4][4], rl[4][4], ih[4][4], il[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) rh[i][j] = rl[i][j] = ih[i][j] = il[i][j] = 0.0f;
  const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int k0 = 0; k0 < K; k0 += TK) {
    for (int e = tid; e < TM * TK; e += 256) {
      const int rr = e / TK, kk = e % TK;
      const int gr = r0 + rr, gk = k0 + kk;
      As[kk][rr] = (gr < R && gk < K) ? A[(size_t)gr * K + gk] : z4;
    }
    for (int e = tid; e < TK * TN; e += 256) {
      const int kk = e / TN, cc = e % TN;
      const int gk = k0 + kk, gc = c0 + cc;
      Bs[kk][cc] = (gk < K && gc < Ncol) ? B[(size_t)gk * Ncol + gc] : z4;
    }
    __syncthreads();
#pragma unroll 2
    for (int kk = 0; kk < TK; ++kk) {
      float4 a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][tr * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tc + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          // re += ar br - ai bi ; im += ar bi + ai br
          df_mac(rh[i][j], rl[i][j], a[i].x, a[i].y, b[j].x, b[j].y);
          df_mac(rh[i][j], rl[i][j], -a[i].z, -a[i].w, b[j].z, b[j].w);
          df_mac(ih[i][j], il[i][j], a[i].x, a[i].y, b[j].z, b[j].w);
          df_mac(ih[i][j], il[i][j], a[i].z, a[i].w, b[j].x, b[j].y);
        }
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int gr = r0 + tr * 4 + i, gc = c0 + tc + 16 * j;
      if (gr < R && gc < Ncol)
        Cout[(size_t)gr * Ncol + gc] =
            make_double2((double)rh[i][j] + (double)rl[i][j], (double)ih[i][j] + (double)il[i][j]);
    }
}

template <typename C>
__device__ __forceinline__ double cabs2(C v) {
  return (double)v.x * (double)v.x + (double)v.y * (double)v.y;
}

// Complex reciprocal computed in FP64.
template <typename C>
__device__ __forceinline__ C crecip(C v) {
  const double a = v.x, b = v.y;
  const double d = a * a + b * b;
  return mk((decltype(C().x))(a / d), (decltype(C().x))(-b / d));
}

// In-place Gauss-Jordan inversion with partial pivoting of the n x n matrix
// at M (row-major, leading dimension n) using the augmented buffer W
// (n x 2n, shared memory).  One CTA.  Returns nothing; singular pivots give
// inf/NaN like LAPACK's inv would report an error (the host checks).
template <typename C>
__device__ void cta_invert(C* M, C* W, int n, int* piv_s, double* red_v, int* red_i) {
  const int tid = threadIdx.x, nt = blockDim.x;
  const int w2 = 2 * n;
  for (int e = tid; e < n * w2; e += nt) {
    const int r = e / w2, c = e % w2;
    W[e] = c < n ? M[r * n + c] : mk((decltype(C().x))(c - n == r ? 1 : 0), (decltype(C().x))0);
  }
  __syncthreads();
  for (int c = 0; c < n; ++c) {
    // pivot: row p >= c with the largest |W[p][c]|
    double best = -1.0;
    int bi = c;
    for (int r = c + tid; r < n; r += nt) {
      const double v = cabs2(W[r * w2 + c]);
      if (v > best) { best = v; bi = r; }
    }
    red_v[tid] = best;
    red_i[tid] = bi;
    __syncthreads();
    for (int s = nt / 2; s > 0; s >>= 1) {
      if (tid < s) {
        if (red_v[tid + s] > red_v[tid] || (red_v[tid + s] == red_v[tid] && red_i[tid + s] < red_i[tid])) {
          red_v[tid] = red_v[tid + s];
          red_i[tid] = red_i[tid + s];
        }
      }
      __syncthreads();
    }
    const int p = red_i[0];
    if (p != c)
      for (int k = tid; k < w2; k += nt) {
        C t = W[c * w2 + k];
        W[c * w2 + k] = W[p * w2 + k];
        W[p * w2 + k] = t;
      }
    __syncthreads();
    const C inv = crecip(W[c * w2 + c]);
    __syncthreads();
    for (int k = tid; k < w2; k += nt) W[c * w2 + k] = cmul(W[c * w2 + k], inv);
    __syncthreads();
    // eliminate column c from every other row
    for (int e = tid; e < n * w2; e += nt) {
      const int r = e / w2, k = e % w2;
      if (r == c || k == c) continue;
      const C f = W[r * w2 + c];
      W[e] = csub(W[e], cmul(f, W[c * w2 + k]));
    }
    __syncthreads();
    for (int r = tid; r < n; r += nt)
      if (r != c) W[r * w2 + c] = mk((decltype(C().x))0, (decltype(C().x))0);
    __syncthreads();
  }
  for (int e = tid; e < n * n; e += nt) M[e] = W[(e / n) * w2 + n + (e % n)];
  __syncthreads();
  (void)piv_s;
}

}  // namespace bf
