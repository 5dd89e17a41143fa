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

// ---- complex64 operands, chunked double-float accumulation -------------------
// C[R][Ncol] (complex128) = A[R][K] * B[K][Ncol], A and B complex64.  Each
// thread sums TK = 16 consecutive products of an output in FP32 (error
// ~16 u of that chunk's terms) and folds the chunk into a (hi, lo) FP32 pair
// with TwoSum, so the rounding of a long contraction does not grow with K:
// the result carries the complex64 rounding of the operands (random, ~6e-8 of
// each term) and no accumulation drift.  64x64 tile per CTA of 256 threads, a
// 4x4 block per thread; the next K tile is prefetched into registers while
// the current one is multiplied.
__device__ __forceinline__ void two_sum_acc(float& hi, float& lo, float x) {
  const float t = hi + x;
  const float z = t - hi;
  lo += (hi - (t - z)) + (x - z);
  hi = t;
}

// blockIdx.z selects the K slice [z kchunk, (z+1) kchunk) and the output
// plane Cout + z R Ncol (split-K for grids that would not fill the SMs).
__global__ void __launch_bounds__(256, 1) k_cgemm_c64(const float2* __restrict__ A, const float2* __restrict__ B,
                                                       double2* __restrict__ Cout, int R, int K, int Ncol,
                                                       int kchunk) {
  constexpr int TM = 64, TN = 64, TK = 16;
  __shared__ float2 As[TK][TM + 1];
  __shared__ float2 Bs[TK][TN];
  const int tid = threadIdx.x;
  const int tr = tid / 16, tc = tid % 16;
  const int r0 = blockIdx.y * TM, c0 = blockIdx.x * TN;
  const int kbeg = blockIdx.z * kchunk, kend = min(K, kbeg + kchunk);
  Cout += (size_t)blockIdx.z * R * Ncol;
  float hr[4][4], lr[4][4], hi[4][4], li[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) hr[i][j] = lr[i][j] = hi[i][j] = li[i][j] = 0.0f;
  // each thread stages 4 A and 4 B elements per tile
  float2 pa[4], pb[4];
  auto fetch = [&](int k0) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int e = tid + 256 * q;
      const int rr = e / TK, kk = e % TK;
      const int gr = r0 + rr, gk = k0 + kk;
      pa[q] = (gr < R && gk < kend) ? A[(size_t)gr * K + gk] : make_float2(0.f, 0.f);
      const int kb = e / TN, cc = e % TN;
      const int gkb = k0 + kb, gc = c0 + cc;
      pb[q] = (gkb < kend && gc < Ncol) ? B[(size_t)gkb * Ncol + gc] : make_float2(0.f, 0.f);
    }
  };
  fetch(kbeg);
  for (int k0 = kbeg; k0 < kend; k0 += TK) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int e = tid + 256 * q;
      As[e % TK][e / TK] = pa[q];
      Bs[e / TN][e % TN] = pb[q];
    }
    __syncthreads();
    if (k0 + TK < kend) fetch(k0 + TK);
    float ar[4][4], ai[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) ar[i][j] = ai[i][j] = 0.0f;
#pragma unroll
    for (int kk = 0; kk < TK; ++kk) {
      float2 a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][tr * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tc + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          ar[i][j] = fmaf(a[i].x, b[j].x, ar[i][j]);
          ar[i][j] = fmaf(-a[i].y, b[j].y, ar[i][j]);
          ai[i][j] = fmaf(a[i].x, b[j].y, ai[i][j]);
          ai[i][j] = fmaf(a[i].y, b[j].x, ai[i][j]);
        }
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        two_sum_acc(hr[i][j], lr[i][j], ar[i][j]);
        two_sum_acc(hi[i][j], li[i][j], ai[i][j]);
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
            make_double2((double)hr[i][j] + (double)lr[i][j], (double)hi[i][j] + (double)li[i][j]);
    }
}

// Real-by-complex GEMM Cout[r][c] = sum_k A[r][k] B[k][c]: A real (FP32),
// B complex64, one FP32 product per term and accumulator, summed like
// k_cgemm_c64 (FP32 over a 16-term K tile, TwoSum-folded into double-float).
// A CTA computes a 128 x 32 tile; each of its 16 * 128 / RPT threads owns RPT rows
// and 2 columns.  RPT = 8 (256 threads, 203 registers, 8 warps per SM) is the
// one launched: RPT = 4 (512 threads, 119 registers, 16 warps per SM) gave
// the same transformer throughput on GB300 (4593 vs 4624 freq-points/s).
// blockIdx.z selects the K slice [z kchunk, (z+1) kchunk) and the output plane
// Cout + z R Ncol.
template <int RPT>
__global__ void __launch_bounds__(16 * 128 / RPT, 1) k_rcgemm_c64(const float* __restrict__ A,
                                                                  const float2* __restrict__ B,
                                                                  double2* __restrict__ Cout, int R, int K,
                                                                  int Ncol, int kchunk) {
  constexpr int TM = 128, TN = 32, TK = 16, NT = 16 * TM / RPT;
  constexpr int QA = TM * TK / NT, QB = TK * TN / NT;   // staged elements per thread
  __shared__ __align__(16) float As[TK][TM + 4];
  __shared__ __align__(16) float2 Bs[TK][TN];
  const int tid = threadIdx.x;
  const int tr = tid / 16, tc = tid % 16;
  const int r0 = blockIdx.y * TM, c0 = blockIdx.x * TN;
  const int kbeg = blockIdx.z * kchunk, kend = min(K, kbeg + kchunk);
  Cout += (size_t)blockIdx.z * R * Ncol;
  float hr[RPT][2], lr[RPT][2], hi[RPT][2], li[RPT][2], ar[RPT][2], ai[RPT][2];
#pragma unroll
  for (int i = 0; i < RPT; ++i)
#pragma unroll
    for (int j = 0; j < 2; ++j) hr[i][j] = lr[i][j] = hi[i][j] = li[i][j] = ar[i][j] = ai[i][j] = 0.0f;
  float pa[QA];
  float2 pb[QB];
  auto fetch = [&](int k0) {
#pragma unroll
    for (int q = 0; q < QA; ++q) {
      const int e = tid + NT * q;
      const int gr = r0 + e / TK, gk = k0 + e % TK;
      pa[q] = (gr < R && gk < kend) ? A[(size_t)gr * K + gk] : 0.0f;
    }
#pragma unroll
    for (int q = 0; q < QB; ++q) {
      const int e = tid + NT * q;
      const int gk = k0 + e / TN, gc = c0 + e % TN;
      pb[q] = (gk < kend && gc < Ncol) ? B[(size_t)gk * Ncol + gc] : make_float2(0.f, 0.f);
    }
  };
  fetch(kbeg);
  for (int k0 = kbeg; k0 < kend; k0 += TK) {
#pragma unroll
    for (int q = 0; q < QA; ++q) {
      const int e = tid + NT * q;
      As[e % TK][e / TK] = pa[q];
    }
#pragma unroll
    for (int q = 0; q < QB; ++q) {
      const int e = tid + NT * q;
      Bs[e / TN][e % TN] = pb[q];
    }
    __syncthreads();
    if (k0 + TK < kend) fetch(k0 + TK);
#pragma unroll
    for (int kk = 0; kk < TK; ++kk) {
      float a[RPT];
#pragma unroll
      for (int v = 0; v < RPT / 4; ++v) {
        const float4 a4 = *reinterpret_cast<const float4*>(&As[kk][tr * RPT + 4 * v]);
        a[4 * v] = a4.x;
        a[4 * v + 1] = a4.y;
        a[4 * v + 2] = a4.z;
        a[4 * v + 3] = a4.w;
      }
      const float2 b[2] = {Bs[kk][tc], Bs[kk][tc + 16]};
#pragma unroll
      for (int i = 0; i < RPT; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) {
          ar[i][j] = fmaf(a[i], b[j].x, ar[i][j]);
          ai[i][j] = fmaf(a[i], b[j].y, ai[i][j]);
        }
    }
#pragma unroll
    for (int i = 0; i < RPT; ++i)
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        two_sum_acc(hr[i][j], lr[i][j], ar[i][j]);
        two_sum_acc(hi[i][j], li[i][j], ai[i][j]);
        ar[i][j] = ai[i][j] = 0.0f;
      }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < RPT; ++i)
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const int gr = r0 + tr * RPT + i, gc = c0 + tc + 16 * j;
      if (gr < R && gc < Ncol)
        Cout[(size_t)gr * Ncol + gc] =
            make_double2((double)hr[i][j] + (double)lr[i][j], (double)hi[i][j] + (double)li[i][j]);
    }
}

// out[i] = sum over the split-K planes of part[z][i], in plane order
__global__ void k_sum_planes(double2* __restrict__ out, const double2* __restrict__ part, size_t n, int planes) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    double2 acc = part[i];
    for (int z = 1; z < planes; ++z) {
      const double2 v = part[(size_t)z * n + i];
      acc.x += v.x;
      acc.y += v.y;
    }
    out[i] = acc;
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
// (n x 2n, shared memory).  One CTA of up to 1024 threads; red_v / red_i hold
// at least 160 doubles / 80 ints of shared scratch.  The pivot (largest
// |W[p][c]|^2, lowest row on ties) is a warp-shuffle argmax, then one over
// the warps; its reciprocal is computed once and broadcast.  Magnitudes and
// the reciprocal use the matrix's own precision: a warp-wide FP64 instruction
// costs the same with one lane active, at 1/64 of the FP32 rate.  An exactly
// zero pivot (LAPACK getrf's info > 0, where Julia's inv raises
// SingularException) records `tag` in *sing (atomicMin); the inverse is then
// inf/NaN.
template <typename C>
__device__ void cta_invert(C* M, C* W, int n, int* sing, int tag, double* red_v, int* red_i) {
  using R = decltype(C().x);
  constexpr unsigned FULL = 0xffffffffu;
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nwarp = (nt + 31) >> 5;
  const int w2 = 2 * n;
  C* inv_s = reinterpret_cast<C*>(red_v + 64);   // the broadcast reciprocal
  for (int e = tid; e < n * w2; e += nt) {
    const int r = e / w2, c = e % w2;
    W[e] = c < n ? M[r * n + c] : mk((R)(c - n == r ? 1 : 0), (R)0);
  }
  __syncthreads();
  for (int c = 0; c < n; ++c) {
    // pivot: row p >= c with the largest |W[p][c]|
    R best = (R)-1;
    int bi = n;
    for (int r = c + tid; r < n; r += nt) {
      const C w = W[r * w2 + c];
      const R v = w.x * w.x + w.y * w.y;
      if (v > best) { best = v; bi = r; }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const R vo = __shfl_xor_sync(FULL, best, o);
      const int io = __shfl_xor_sync(FULL, bi, o);
      if (vo > best || (vo == best && io < bi)) { best = vo; bi = io; }
    }
    if (lane == 0) {
      red_v[warp] = (double)best;
      red_i[warp] = bi;
    }
    __syncthreads();
    if (warp == 0) {
      double v = lane < nwarp ? red_v[lane] : -1.0;
      int i = lane < nwarp ? red_i[lane] : n;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const double vo = __shfl_xor_sync(FULL, v, o);
        const int io = __shfl_xor_sync(FULL, i, o);
        if (vo > v || (vo == v && io < i)) { v = vo; i = io; }
      }
      if (lane == 0) red_i[64] = i < n ? i : c;
    }
    __syncthreads();
    const int p = red_i[64];
    if (p != c)
      for (int k = tid; k < w2; k += nt) {
        C t = W[c * w2 + k];
        W[c * w2 + k] = W[p * w2 + k];
        W[p * w2 + k] = t;
      }
    __syncthreads();
    if (tid == 0) {
      const C w = W[c * w2 + c];
      if (w.x == (R)0 && w.y == (R)0) atomicMin(sing, tag);
      const R d = w.x * w.x + w.y * w.y;
      *inv_s = mk(w.x / d, -w.y / d);
    }
    __syncthreads();
    const C inv = *inv_s;
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
      if (r != c) W[r * w2 + c] = mk((R)0, (R)0);
    __syncthreads();
  }
  for (int e = tid; e < n * n; e += nt) M[e] = W[(e / n) * w2 + n + (e % n)];
  __syncthreads();
}

}  // namespace bf
