// Register-resident FFT building blocks for the fused propagation kernels.
//
// A line of N = C*G*G points (N a power of two) is transformed by a "team" of
// G threads holding RR = C*G points each:
//   pass 1  every thread does an RR-point DFT over the points x[g + G*r]
//           (r = 0..RR-1) in registers and multiplies by W_N^(g*s);
//   exchange through a swizzled shared-memory tile (one write + one read);
//   pass 2  every thread does C G-point DFTs in registers.
// Afterwards thread g holds X[(g*C + j) + RR*q] in v[j*G + q].  The inverse is
// the exact adjoint (same exchange, conjugate roots) and returns the points to
// the x[g + G*r] layout, unnormalised (a factor N).
// With C = 2 the exchange can also run in two halves through a scratch tile of
// half the size (HALF): the same data movement, two more warp syncs.
#pragma once

#include "bf_common.cuh"

namespace bf {

// Unit roots W_1024^k = exp(-2 pi i k / 1024), filled from the host in FP64.
// Register FFTs index them with compile-time offsets, so they compile into
// constant-bank operands.  Defined here: this header belongs to exactly one
// translation unit (bf_device.cu).
__constant__ double2 c_root1024_d[1024];
__constant__ float2 c_root1024_f[1024];

template <typename C> __device__ __forceinline__ C root1024(int k);
template <> __device__ __forceinline__ float2 root1024<float2>(int k) { return c_root1024_f[k]; }
template <> __device__ __forceinline__ double2 root1024<double2>(int k) { return c_root1024_d[k]; }

// Butterfly adds.  For complex64 both halves go through one packed FP32x2
// instruction (add/sub.rn.f32x2, Blackwell): an FFT is mostly complex adds, so
// this halves its add instructions.  Each lane rounds exactly like a scalar add.
template <typename C> __device__ __forceinline__ C vadd(C a, C b) { return cadd(a, b); }
template <typename C> __device__ __forceinline__ C vsub(C a, C b) { return csub(a, b); }
template <> __device__ __forceinline__ float2 vadd<float2>(float2 a, float2 b) {
  float2 d;
  asm("{\n\t.reg .b64 pa, pb, pd;\n\tmov.b64 pa, {%2, %3};\n\tmov.b64 pb, {%4, %5};\n\t"
      "add.rn.f32x2 pd, pa, pb;\n\tmov.b64 {%0, %1}, pd;\n\t}"
      : "=f"(d.x), "=f"(d.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return d;
}
template <> __device__ __forceinline__ float2 vsub<float2>(float2 a, float2 b) {
  float2 d;
  asm("{\n\t.reg .b64 pa, pb, pd;\n\tmov.b64 pa, {%2, %3};\n\tmov.b64 pb, {%4, %5};\n\t"
      "sub.rn.f32x2 pd, pa, pb;\n\tmov.b64 {%0, %1}, pd;\n\t}"
      : "=f"(d.x), "=f"(d.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return d;
}

// v[i] *= W_M^k (forward) or conj(W_M^k) (inverse), k compile-time after unrolling.
template <int M, bool INV, typename C>
__device__ __forceinline__ C twiddle_mul(C a, int k) {
  if (k == 0) return a;
  if (4 * k == M) return cmul_mi<INV>(a);
  C w = root1024<C>(k * (1024 / M));
  return INV ? cmulc(a, w) : cmul(a, w);
}

template <int M>
__host__ __device__ constexpr int bitrev(int i) {
  int r = 0;
  for (int b = 1; b < M; b <<= 1) {
    r = (r << 1) | (i & 1);
    i >>= 1;
  }
  return r;
}

// In-register M-point DFT of v[OFF .. OFF+M-1] (radix-2 decimation in
// frequency followed by a static bit-reversal permutation).
template <int M, bool INV, int OFF, int LEN, typename C>
__device__ __forceinline__ void reg_dft(C (&v)[LEN]) {
  if constexpr (M == 1) {
    return;
  } else {
#pragma unroll
    for (int len = M; len >= 2; len >>= 1) {
      const int half = len >> 1;
#pragma unroll
      for (int i = 0; i < M; i += len) {
#pragma unroll
        for (int j = 0; j < half; ++j) {
          C a = v[OFF + i + j];
          C b = v[OFF + i + j + half];
          v[OFF + i + j] = vadd(a, b);
          v[OFF + i + j + half] = twiddle_mul<M, INV>(vsub(a, b), j * (M / len));
        }
      }
    }
#pragma unroll
    for (int i = 0; i < M; ++i) {
      const int r = bitrev<M>(i);
      if (r > i) {
        C t = v[OFF + i];
        v[OFF + i] = v[OFF + r];
        v[OFF + r] = t;
      }
    }
  }
}

// Zero pattern (bit p = point p is exactly zero) at the input of the stage of
// length len of an M-point DIF DFT whose inputs NZ .. M-1 are zero: a
// butterfly output is zero only if both of its inputs were.
template <int M, int NZ>
__host__ __device__ constexpr unsigned long long dif_zero_mask(int len) {
  unsigned long long z = 0;
  for (int p = NZ; p < M; ++p) z |= 1ull << p;
  for (int l = M; l > len; l >>= 1) {
    const int half = l >> 1;
    unsigned long long n = 0;
    for (int p = 0; p < M; ++p)
      if (((z >> p) & 1ull) && ((z >> (p ^ half)) & 1ull)) n |= 1ull << p;
    z = n;
  }
  return z;
}

// One DIF stage (length LEN) of reg_dft_nz, then the next.
template <int M, bool INV, int NZ, int LEN, int VLEN, typename C>
__device__ __forceinline__ void dif_stage_nz(C (&v)[VLEN]) {
  constexpr unsigned long long zm = dif_zero_mask<M, NZ>(LEN);
  constexpr int half = LEN / 2;
#pragma unroll
  for (int i = 0; i < M; i += LEN) {
#pragma unroll
    for (int j = 0; j < half; ++j) {
      const int pa = i + j, pb = pa + half;
      const bool za = (zm >> pa) & 1ull, zb = (zm >> pb) & 1ull;
      const int k = j * (M / LEN);
      if (za && zb) continue;
      const C a = v[pa], b = v[pb];
      if (zb) {
        v[pb] = twiddle_mul<M, INV>(a, k);
      } else if (za) {
        v[pa] = b;
        v[pb] = twiddle_mul<M, INV>(csub(czero_of(b), b), k);
      } else {
        v[pa] = vadd(a, b);
        v[pb] = twiddle_mul<M, INV>(vsub(a, b), k);
      }
    }
  }
  if constexpr (LEN > 2) dif_stage_nz<M, INV, NZ, LEN / 2>(v);
}

// reg_dft<M, INV, 0> of v[0 .. M-1] whose inputs v[NZ ..] are zero: butterflies
// with a zero input reduce to a copy and a twiddle, those with two zero inputs
// vanish.  The results are those of the dense DFT (adding an exact zero
// changes nothing but the sign of a zero).
template <int M, bool INV, int NZ, int LEN, typename C>
__device__ __forceinline__ void reg_dft_nz(C (&v)[LEN]) {
  if constexpr (NZ >= M || M < 2) {
    reg_dft<M, INV, 0>(v);
  } else {
    dif_stage_nz<M, INV, NZ, M>(v);
#pragma unroll
    for (int i = 0; i < M; ++i) {
      const int r = bitrev<M>(i);
      if (r > i) {
        C t = v[i];
        v[i] = v[r];
        v[r] = t;
      }
    }
  }
}

template <int N> struct TeamShape;
template <> struct TeamShape<8>   { static constexpr int G = 2,  RR = 4;  };
template <> struct TeamShape<16>  { static constexpr int G = 4,  RR = 4;  };
template <> struct TeamShape<32>  { static constexpr int G = 4,  RR = 8;  };
template <> struct TeamShape<64>  { static constexpr int G = 8,  RR = 8;  };
template <> struct TeamShape<128> { static constexpr int G = 8,  RR = 16; };
template <> struct TeamShape<256> { static constexpr int G = 16, RR = 16; };
template <> struct TeamShape<512> { static constexpr int G = 16, RR = 32; };

template <int N>
struct Team {
  static constexpr int G = TeamShape<N>::G;
  static constexpr int RR = TeamShape<N>::RR;
  static constexpr int C = RR / G;
  static_assert(C * G * G == N, "team shape");
  // scratch tile of one team, in complex elements; the pad staggers the tiles
  // of teams sharing a half-warp across shared-memory banks
  static constexpr int SCR = RR * G + (G < 16 ? G : 0);
  // the half-size tile of the two-half exchange: G rows of G points; the pad
  // puts the two teams of a half-warp on opposite halves of the banks
  static constexpr int SCRH = (RR / 2) * G + (G < 16 ? G : 0);
  template <bool HALF> __host__ __device__ static constexpr int scratch() { return HALF ? SCRH : SCR; }

  __device__ static __forceinline__ int swz(int s, int g) { return s * G + (g ^ (s / C)); }

  // forward: v[r] = x[g + G r]  ->  v[j*G + q] = X[(g*C + j) + RR*q];
  // NZ < RR: the caller guarantees v[NZ ..] == 0 (pruned first pass);
  // tw: the thread's RR inter-pass twiddles (registers or shared memory)
  template <int NZ = RR, bool HALF = false, typename Cx>
  __device__ static __forceinline__ void forward(Cx (&v)[RR], const Cx* tw, Cx* scr, int g) {
    reg_dft_nz<RR, false, NZ>(v);
#pragma unroll
    for (int s = 1; s < RR; ++s) v[s] = cmul(v[s], tw[s]);
    if constexpr (HALF) {
      static_assert(C == 2, "two-half exchange");
      // half j moves the points s = C t + j: row t, column g ^ t of the tile
      Cx w[RR];
#pragma unroll
      for (int j = 0; j < C; ++j) {
#pragma unroll
        for (int t = 0; t < G; ++t) scr[t * G + (g ^ t)] = v[C * t + j];
        __syncwarp();
#pragma unroll
        for (int gp = 0; gp < G; ++gp) w[j * G + gp] = scr[g * G + (gp ^ g)];
        __syncwarp();
      }
#pragma unroll
      for (int s = 0; s < RR; ++s) v[s] = w[s];
    } else {
#pragma unroll
      for (int s = 0; s < RR; ++s) scr[swz(s, g)] = v[s];
      __syncwarp();
#pragma unroll
      for (int j = 0; j < C; ++j)
#pragma unroll
        for (int gp = 0; gp < G; ++gp) v[j * G + gp] = scr[swz(g * C + j, gp)];
      __syncwarp();
    }
#pragma unroll
    for (int j = 0; j < C; ++j) reg_dft_sub<false>(v, j);
  }

  // inverse (adjoint of forward, unnormalised): v[j*G + q] = X[(g*C + j) + RR*q] -> v[r] = N x[g + G r]
  template <bool HALF = false, typename Cx>
  __device__ static __forceinline__ void inverse(Cx (&v)[RR], const Cx* tw, Cx* scr, int g) {
#pragma unroll
    for (int j = 0; j < C; ++j) reg_dft_sub<true>(v, j);
    if constexpr (HALF) {
      static_assert(C == 2, "two-half exchange");
      Cx w[RR];
#pragma unroll
      for (int j = 0; j < C; ++j) {
#pragma unroll
        for (int gp = 0; gp < G; ++gp) scr[g * G + (gp ^ g)] = v[j * G + gp];
        __syncwarp();
#pragma unroll
        for (int t = 0; t < G; ++t) w[C * t + j] = scr[t * G + (g ^ t)];
        __syncwarp();
      }
#pragma unroll
      for (int s = 0; s < RR; ++s) v[s] = w[s];
    } else {
#pragma unroll
      for (int j = 0; j < C; ++j)
#pragma unroll
        for (int gp = 0; gp < G; ++gp) scr[swz(g * C + j, gp)] = v[j * G + gp];
      __syncwarp();
#pragma unroll
      for (int s = 0; s < RR; ++s) v[s] = scr[swz(s, g)];
      __syncwarp();
    }
#pragma unroll
    for (int s = 1; s < RR; ++s) v[s] = cmulc(v[s], tw[s]);
    reg_dft<RR, true, 0>(v);
  }

 private:
  template <bool INV, typename Cx>
  __device__ static __forceinline__ void reg_dft_sub(Cx (&v)[RR], int j) {
    // j is a compile-time constant after unrolling of the caller's loop
    static_assert(C == 1 || C == 2, "team shape");
    if constexpr (C == 1) {
      reg_dft<G, INV, 0>(v);
    } else {
      if (j == 0) reg_dft<G, INV, 0>(v);
      else reg_dft<G, INV, G>(v);
    }
  }
};

// Per-thread inter-pass twiddles W_N^(g*s), s = 0..RR-1 (g*s < N always).
template <int N, typename Cx>
__device__ __forceinline__ void team_twiddles(Cx (&tw)[Team<N>::RR], int g) {
  static_assert(N <= 1024, "root table");
#pragma unroll
  for (int s = 0; s < Team<N>::RR; ++s) tw[s] = root1024<Cx>(g * s * (1024 / N));
}

}  // namespace bf
