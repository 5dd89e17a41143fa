// Transformer (mode matching) on the GPU: mode basis, propagation matrices,
// transfer-matrix chain and the final boundary solve
// (src/boost_fractor_transformer.jl:23-359).
//
// Propagation matrices P[m][m'] = <Psi_m | prop(Psi_m')> (:174-227) by region class:
//  * air regions without tilt or surface map ("k-space class"): by Parseval,
//    sum_x conj(Psi_m) IFFT(D FFT(mask Psi_m')) = (1/N^2) sum_k conj(U_m(k)) D(k) Phi_m'(k)
//    with U = FFT(Psi), Phi = FFT(mask Psi) frequency independent.  D depends on
//    k only through kx^2 + ky^2, so the sum folds over the mirror images of k:
//    P = W[nm^2 x K] * D[K x (freqs * regions)], one GEMM for the whole batch;
//  * disk regions ("pixel class"): P = diag(exp(-i kz_m dz)) sum_x conj(Psi_m) Psi_m'
//    TS(x) with TS the tilt/surface phase: P = V[nm^2 x Kd] * E[Kd x (freqs*regions)];
//    air regions with the 1D propagator use the same GEMM with TS = exp(-i k0 dz);
//  * air regions with a tilt or surface map, or the momentum-space propagator
//    ("field class"): every mode is propagated on the full grid and overlapped.
// The chain T <- T G_s blockdiag(P_s, P_s^-1) needs only its bottom block row;
// the final solve boost = -T22 \ axion_beam runs in FP64.
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <complex>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "../../include/boostfractor_gb300.h"
#include "bf_common.cuh"
#include "bf_device.cuh"
#include "bf_host.h"
#include "bf_linalg.cuh"

namespace bfmodes {
double besselj_zero(int nu, int m);
void seed_modes(int M, int L, const std::vector<double>& X, const std::vector<double>& Y, double diskR,
                std::vector<std::complex<double>>& out, std::vector<std::complex<double>>& kt);
}  // namespace bfmodes

using bf::RegionGeo;

struct bf_modes {
  int M = 0, L = 0, nm = 0, nx = 0, ny = 0;
  std::vector<double> X, Y;
  std::vector<cd> pat;   // [nm][ny][nx]
  std::vector<cd> kt;    // [nm]
  double2* d_pat = nullptr;
  unsigned long long id = 0;
  // the transformer's default emission, axion_induced_modes(coords, modes;
  // diskR) (transformer.jl:285), for the last diskR asked for; it depends on
  // the modes and diskR only, so solves do not recompute it
  std::mutex emit_mu;
  double emit_diskR = -1.0;
  std::vector<cd> emit;
  std::atomic<int> server_uses{0};   // serving-engine requests queued or running on it
};

void bf_modes_server_use(bf_modes* m, int delta) {
  if (m) m->server_uses += delta;
}

// engine-wide helpers from bf_api.cu
int bf_fail(bf_handle* h, int code, const std::string& msg);
int bf_general_prop(bf_handle* h, const bf_stack* s, int kind, bool fp64, void* buf, void* tmp, int nb,
                    const double* d_freqs, int region);

#define TCK(call)                                                                            \
  do {                                                                                       \
    cudaError_t e_ = (call);                                                                 \
    if (e_ != cudaSuccess)                                                                   \
      return bf_fail(h, BF_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_) + " (" + \
                  std::string(__FILE__).substr(std::string(__FILE__).find_last_of('/') + 1) + ":" +  \
                  std::to_string(__LINE__) + ")");    \
  } while (0)
#define TCKS(call)              \
  do {                          \
    int s_ = (call);            \
    if (s_ != BF_OK) return s_; \
  } while (0)

namespace {

constexpr double kC = 299792458.0;

__device__ __forceinline__ double2 dsqrt_c(double x, double y) {
  if (x == 0.0 && y == 0.0) return make_double2(0.0, y);
  // a zero imaginary part (real permittivities): with hypot(x, 0) = |x| the
  // general formula below reduces to these values in exact arithmetic; they
  // skip hypot and the division (FP64 runs at 1/64 of the FP32 rate)
  if (y == 0.0) return x > 0.0 ? make_double2(sqrt(x), y) : make_double2(0.0, copysign(sqrt(-x), y));
  double t = sqrt((fabs(x) + hypot(x, y)) * 0.5);
  if (x >= 0.0) return make_double2(t, y / (2.0 * t));
  return make_double2(fabs(y) / (2.0 * t), copysign(t, y));
}
__device__ __forceinline__ double2 dexp_c(double re, double im) {
  double s, c;
  sincos(im, &s, &c);
  if (re == 0.0) return make_double2(c, s);   // exp(0) = 1 exactly (propagating bins)
  const double m = exp(re);
  return make_double2(m * c, m * s);
}
// k0 = 2 pi / lambda sqrt(eps); a zero imaginary part keeps its sign
__device__ __forceinline__ double2 k0_c(double lambda, double er, double ei) {
  double2 s = dsqrt_c(er, ei);
  const double c = 2.0 * M_PI / lambda;
  return make_double2(c * s.x, c * s.y);
}

template <typename C> __device__ __forceinline__ C dto(double2 v);
template <> __device__ __forceinline__ float2 dto<float2>(double2 v) { return make_float2((float)v.x, (float)v.y); }
template <> __device__ __forceinline__ double2 dto<double2>(double2 v) { return v; }

// exp(re + i im) stored as C.  double2: FP64 throughout.  float2: the
// argument (FP64) is reduced to [-pi, pi] in FP64, then sincos/exp run in FP32;
// the result carries the complex64 rounding of the stored operand (~1e-7) and
// no loss from large phase arguments, at the FP32 rate instead of the FP64 one.
template <typename C> __device__ __forceinline__ C cexp_as(double re, double im);
template <> __device__ __forceinline__ double2 cexp_as<double2>(double re, double im) { return dexp_c(re, im); }
template <> __device__ __forceinline__ float2 cexp_as<float2>(double re, double im) {
  const double r = im - 6.283185307179586 * rint(im * 0.15915494309189535);
  float sn, cs;
  sincosf((float)r, &sn, &cs);
  const float m = expf((float)re);
  return make_float2(m * cs, m * sn);
}

struct RegionT {      // per-region data of a transformer solve
  double dz, er, ei, tx, ty;
  int klass;          // 0 k-space, 1 pixel (disk), 2 pixel (air, 1D propagator), 3 field
  int col;            // column block of the region in its class GEMM
};

// ---- setup kernels --------------------------------------------------------
// W[mm'][o] = scale * sum_{k in orbit o} conj(U_m(k)) Phi_m'(k)
template <typename C>
__global__ void k_build_w(C* W, const double2* U, const double2* Phi, const int* members, int K, int msz,
                          int nm, int npix, double scale) {
  const int o = blockIdx.x * blockDim.x + threadIdx.x;
  const int mm = blockIdx.y;
  if (o >= K) return;
  const int m = mm / nm, mp = mm % nm;
  double2 acc = make_double2(0.0, 0.0);
  for (int q = 0; q < msz; ++q) {
    const int k = members[(size_t)o * msz + q];
    if (k < 0) break;
    const double2 u = U[(size_t)m * npix + k], p = Phi[(size_t)mp * npix + k];
    acc.x += u.x * p.x + u.y * p.y;
    acc.y += u.x * p.y - u.y * p.x;
  }
  W[(size_t)mm * K + o] = dto<C>(make_double2(acc.x * scale, acc.y * scale));
}

// V[mm'][s] = conj(Psi_m(x_s)) Psi_m'(x_s) over the support pixels
template <typename C>
__global__ void k_build_v(C* V, const double2* pat, const int* supp, int Kd, int nm, int npix) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  const int mm = blockIdx.y;
  if (s >= Kd) return;
  const int m = mm / nm, mp = mm % nm;
  const int x = supp[s];
  const double2 a = pat[(size_t)m * npix + x], b = pat[(size_t)mp * npix + x];
  V[(size_t)mm * Kd + s] = dto<C>(make_double2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x));
}

// Upper triangle of W as real rows (valid when W is Hermitian in the mode
// pair: Phi = U, every mode zero outside the mask): pair t = (m, m') gives
// Wr[2t][o] = Re W[mm'][o], Wr[2t+1][o] = Im W[mm'][o], summed like k_build_w.
__global__ void k_build_wr(float* Wr, const double2* U, const double2* Phi, const int* members, const int2* tri,
                           int K, int msz, int npix, double scale) {
  const int o = blockIdx.x * blockDim.x + threadIdx.x;
  const int t = blockIdx.y;
  if (o >= K) return;
  const int2 mp = tri[t];
  double2 acc = make_double2(0.0, 0.0);
  for (int q = 0; q < msz; ++q) {
    const int k = members[(size_t)o * msz + q];
    if (k < 0) break;
    const double2 u = U[(size_t)mp.x * npix + k], p = Phi[(size_t)mp.y * npix + k];
    acc.x += u.x * p.x + u.y * p.y;
    acc.y += u.x * p.y - u.y * p.x;
  }
  Wr[(size_t)(2 * t) * K + o] = (float)(acc.x * scale);
  Wr[(size_t)(2 * t + 1) * K + o] = (float)(acc.y * scale);
}

// Upper triangle of V as real rows: pair t = (m, m') with m <= m' gives
// Vr[2t][s] = Re V[mm'][s] and Vr[2t+1][s] = Im V[mm'][s].  V is Hermitian in
// the mode pair (V[m'm] = conj V[mm']), so these rows determine all of it.
__global__ void k_build_vr(float* Vr, const double2* pat, const int* supp, const int2* tri, int Kd, int npix) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  const int t = blockIdx.y;
  if (s >= Kd) return;
  const int2 mp = tri[t];
  const int x = supp[s];
  const double2 a = pat[(size_t)mp.x * npix + x], b = pat[(size_t)mp.y * npix + x];
  Vr[(size_t)(2 * t) * Kd + s] = (float)(a.x * b.x + a.y * b.y);
  Vr[(size_t)(2 * t + 1) * Kd + s] = (float)(a.x * b.y - a.y * b.x);
}

// kz[e][f][o] = sqrt(k0^2 - kx^2 - ky^2) at the orbit representative o, for the
// distinct permittivities e of the k-space regions (FP64, once per solve)
__global__ void k_build_kz(double2* KZ, const int2* rep, int K, const double* freqs, int nf, const double2* eps,
                           const double* kX, const double* kY) {
  const int o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= K) return;
  const int e = blockIdx.z;
  const int2 sr = rep[o];
  const double kx = kX[sr.x], ky = kY[sr.y];
  for (int f = blockIdx.y; f < nf; f += gridDim.y) {
    const double2 k0 = k0_c(kC / freqs[f], eps[e].x, eps[e].y);
    const double2 k0sq = make_double2(k0.x * k0.x - k0.y * k0.y, k0.x * k0.y + k0.y * k0.x);
    const double re = (k0sq.x - kx * kx) - ky * ky;
    KZ[((size_t)e * nf + f) * K + o] = dsqrt_c(re, k0sq.y);
  }
}

// TF32 hi/lo pair of x: hi = tf32(x), lo = tf32(x - hi) (round to nearest)
__device__ __forceinline__ void tf32_split(float x, float& hi, float& lo) {
  uint32_t h, l;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(x));
  hi = __uint_as_float(h);
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(l) : "f"(x - hi));
  lo = __uint_as_float(l);
}
__device__ __forceinline__ void tf32_split_d(double x, float& hi, float& lo) {
  uint32_t h, l;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"((float)x));
  hi = __uint_as_float(h);
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(l) : "f"((float)(x - (double)hi)));
  lo = __uint_as_float(l);
}

// ---- operands of the tensor-core class GEMMs (BF_PREC_MIXED / BF_PREC_TF32) ----
// Both classes are Hermitian in the mode pair, so the tensor cores see the
// real-row form of the mixed path: A = the real rows of the upper triangle
// (Re and Im of W[mm'] or V[mm'] for m <= m', rows 2t and 2t + 1, padded with
// zero rows to a multiple of 128) and B^T = the complex operand column c as
// two real rows 2c (Re) and 2c + 1 (Im), all K-major TF32 hi/lo pairs with K
// padded to a multiple of 32.  The GEMM runs on B - c(column) instead of B,
// where the constant c is the operand's value at the centre of its domain
// (k-space: exp(-i k0 dz), the transverse-momentum-zero phasor; pixels: 1,
// an untilted flat disk); P adds c times the FP64 row sums of A back.  The
// summed terms are then ~|B - c| instead of ~1, which scales down every
// rounding error of the products and of the sums.

// exp(re + i im) - 1 as complex64, accurate relative to its own (often small)
// magnitude: the phase is reduced to [-pi, pi] in FP64, then
// cos t - 1 = -2 sin^2(t/2) and expm1 avoid the cancellation of exp - 1.
__device__ __forceinline__ float2 cexpm1_f(double re, double im) {
  const double r = im - 6.283185307179586 * rint(im * 0.15915494309189535);
  const float t = (float)r;
  const float h = sinf(0.5f * t), sn = sinf(t);
  const float cm1 = -2.0f * h * h;
  const float em = expm1f((float)re);
  return make_float2(fmaf(em, 1.0f + cm1, cm1), (em + 1.0f) * sn);
}

__device__ __forceinline__ void put_tf32(float* hi, float* lo, size_t i, float v) {
  float h, l;
  tf32_split(v, h, l);
  hi[i] = h;
  lo[i] = l;
}
__device__ __forceinline__ void put_tf32_d(float* hi, float* lo, size_t i, double v) {
  float h, l;
  tf32_split_d(v, h, l);
  hi[i] = h;
  lo[i] = l;
}

// A of the k-space class: the real rows of k_build_wr as TF32 pairs [Mp][Kp]
// (zero for o >= K; rows >= 2T are zeroed beforehand), and the same rows in
// FP64 (Ad [2T][K]) for the row sums.
__global__ void k_build_wr_tc(float* Ah, float* Al, double* Ad, const double2* U, const double2* Phi,
                              const int* members, const int2* tri, int K, int Kp, int msz, int npix, double scale) {
  const int o = blockIdx.x * blockDim.x + threadIdx.x;
  const int t = blockIdx.y;
  if (o >= Kp) return;
  double re = 0.0, im = 0.0;
  if (o < K) {
    const int2 mp = tri[t];
    double2 acc = make_double2(0.0, 0.0);
    for (int q = 0; q < msz; ++q) {
      const int k = members[(size_t)o * msz + q];
      if (k < 0) break;
      const double2 u = U[(size_t)mp.x * npix + k], p = Phi[(size_t)mp.y * npix + k];
      acc.x += u.x * p.x + u.y * p.y;
      acc.y += u.x * p.y - u.y * p.x;
    }
    re = acc.x * scale;
    im = acc.y * scale;
    Ad[(size_t)(2 * t) * K + o] = re;
    Ad[(size_t)(2 * t + 1) * K + o] = im;
  }
  put_tf32_d(Ah, Al, (size_t)(2 * t) * Kp + o, re);
  put_tf32_d(Ah, Al, (size_t)(2 * t + 1) * Kp + o, im);
}

// A of the pixel class: the real rows of k_build_vr as TF32 pairs [Mp][Kdp]
// and in FP64 (Ad [2T][Kd]).
__global__ void k_build_vr_tc(float* Ah, float* Al, double* Ad, const double2* pat, const int* supp,
                              const int2* tri, int Kd, int Kdp, int npix) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  const int t = blockIdx.y;
  if (s >= Kdp) return;
  double re = 0.0, im = 0.0;
  if (s < Kd) {
    const int2 mp = tri[t];
    const int x = supp[s];
    const double2 a = pat[(size_t)mp.x * npix + x], b = pat[(size_t)mp.y * npix + x];
    re = a.x * b.x + a.y * b.y;
    im = a.x * b.y - a.y * b.x;
    Ad[(size_t)(2 * t) * Kd + s] = re;
    Ad[(size_t)(2 * t + 1) * Kd + s] = im;
  }
  put_tf32_d(Ah, Al, (size_t)(2 * t) * Kdp + s, re);
  put_tf32_d(Ah, Al, (size_t)(2 * t + 1) * Kdp + s, im);
}

// g[r] = sum_k Ad[r][k] in FP64, one CTA of 256 threads per row (fixed order)
__global__ void k_rowsum(double* g, const double* Ad, int K) {
  __shared__ double red[256];
  const int r = blockIdx.x;
  double acc = 0.0;
  for (int k = threadIdx.x; k < K; k += blockDim.x) acc += Ad[(size_t)r * K + k];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) g[r] = red[0];
}

// Per column c = (r nf + f) npar + p of the k-space class (r: the request of
// a group solve, whose regions are regs[r nd ..]), for the tensor-core
// operand builder: c0 = exp(-i kz0 dz) with kz0 = sqrt(k0^2) (the phasor's
// transverse-momentum-zero wavenumber) in FP64 (C0, also added back by the
// scatter), and complex64 copies of c0, kz0, k0^2 and dz (col).
struct ColTC {
  float2 c0, kz0, k0sq;
  float dz;
  int ef;   // row of the column's (permittivity, frequency) in DKZ
};
__global__ void k_build_c0(double2* C0, ColTC* col, const double* freqs, int nf, int ncol, int nd,
                           const double2* eps, const RegionT* regs, const int* par_regions, const int* par_eps,
                           int npar) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncol) return;
  const int F = c / npar, p = c % npar, f = F % nf, r = F / nf;
  const double2 e = eps[par_eps[p]];
  const double2 k0 = k0_c(kC / freqs[f], e.x, e.y);
  const double2 k0sq = make_double2(k0.x * k0.x - k0.y * k0.y, k0.x * k0.y + k0.y * k0.x);
  const double2 kz0 = dsqrt_c(k0sq.x, k0sq.y);
  const double dz = regs[(size_t)r * nd + par_regions[p]].dz;
  const double2 c0 = dexp_c(kz0.y * dz, -kz0.x * dz);
  C0[c] = c0;
  ColTC q;
  q.c0 = make_float2((float)c0.x, (float)c0.y);
  q.kz0 = make_float2((float)kz0.x, (float)kz0.y);
  q.k0sq = make_float2((float)k0sq.x, (float)k0sq.y);
  q.dz = (float)dz;
  q.ef = par_eps[p] * nf + f;
  col[c] = q;
}

// Principal complex square root in FP32 with the conventions of dsqrt_c (a
// zero imaginary part keeps its sign, so real permittivities held as
// re - 0.0im give decaying evanescent roots).
__device__ __forceinline__ float2 fsqrt_c(float x, float y) {
  if (x == 0.f && y == 0.f) return make_float2(0.f, y);
  if (y == 0.f) return x > 0.f ? make_float2(sqrtf(x), y) : make_float2(0.f, copysignf(sqrtf(-x), y));
  const float t = sqrtf((fabsf(x) + hypotf(x, y)) * 0.5f);
  if (x >= 0.f) return make_float2(t, y / (2.f * t));
  return make_float2(fabsf(y) / (2.f * t), copysignf(t, y));
}

// exp(re + i im) - 1 for a modest phase |im| (a few radians), all in FP32:
// with s, c = sin, cos(im/2): cos im - 1 = -2 s^2 and sin im = 2 s c, and
// expm1, keep it accurate relative to its own magnitude (one sincosf; no
// expm1 for a lossless phase, re = 0).
__device__ __forceinline__ float2 cexpm1_ff(float re, float im) {
  float h, ch;
  sincosf(0.5f * im, &h, &ch);
  const float cm1 = -2.0f * h * h, sn = 2.0f * h * ch;
  const float em = re == 0.0f ? 0.0f : expm1f(re);
  return make_float2(fmaf(em, 1.0f + cm1, cm1), (em + 1.0f) * sn);
}

// DKZ[e][f][o] = kz - kz0 = -kt^2 / (kz + kz0) in FP32 for the distinct
// permittivities e of the k-space regions, once per (frequency, orbit): it has
// no cancellation, so FP32 carries it to ~1e-7 of its own size.  KT2[o] =
// kx^2 + ky^2 at the orbit representative.
__global__ void k_build_dkz(float2* DKZ, const float* KT2, int K, const double* freqs, int nf, const double2* eps) {
  const int o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= K) return;
  const int e = blockIdx.z;
  const float kt2 = KT2[o];
  for (int f = blockIdx.y; f < nf; f += gridDim.y) {
    const double2 k0 = k0_c(kC / freqs[f], eps[e].x, eps[e].y);
    const double2 k0sq = make_double2(k0.x * k0.x - k0.y * k0.y, k0.x * k0.y + k0.y * k0.x);
    const double2 kz0d = dsqrt_c(k0sq.x, k0sq.y);
    const float2 kz0 = make_float2((float)kz0d.x, (float)kz0d.y);
    const float2 kz = fsqrt_c((float)k0sq.x - kt2, (float)k0sq.y);
    const float2 den = make_float2(kz.x + kz0.x, kz.y + kz0.y);
    const float dn = den.x * den.x + den.y * den.y;
    DKZ[((size_t)e * nf + f) * K + o] = make_float2(-kt2 * den.x / dn, kt2 * den.y / dn);   // -kt2 / den
  }
}

// B^T of the k-space class: rows 2c, 2c + 1 = Re, Im of D[o][c] - c0[c] =
// c0 (exp(-i (kz - kz0) dz) - 1) as TF32 pairs [2 ncol][Kp], zero for o >= K;
// kz - kz0 from DKZ, the phase (kz - kz0) dz is a few radians at most.
__global__ void k_build_d_tc(float* Bh, float* Bl, const float2* DKZ, const ColTC* col, int K, int Kp, int ncol) {
  const int o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= Kp) return;
  for (int c = blockIdx.y; c < ncol; c += gridDim.y) {
    float2 v = make_float2(0.f, 0.f);
    if (o < K) {
      const ColTC q = col[c];
      const float2 dkz = DKZ[(size_t)q.ef * K + o];
      const float2 m1 = cexpm1_ff(dkz.y * q.dz, -dkz.x * q.dz);
      v = make_float2(q.c0.x * m1.x - q.c0.y * m1.y, q.c0.x * m1.y + q.c0.y * m1.x);
    }
    put_tf32(Bh, Bl, (size_t)(2 * c) * Kp + o, v.x);
    put_tf32(Bh, Bl, (size_t)(2 * c + 1) * Kp + o, v.y);
  }
}

// B^T of the pixel class: rows 2c, 2c + 1 = Re, Im of E[s][c] - 1 (the
// tilt/surface phase of k_build_e less its untilted, flat value) as TF32
// pairs [2 ncol][Kdp], zero for s >= Kd
__global__ void k_build_e_tc(float* Bh, float* Bl, const int* supp, int Kd, int Kdp, int nf, const RegionT* regs,
                             const int* pix_regions, int npx, const double2* K0, const double* X, const double* Y,
                             int nx, const double2* surf, int npix) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= Kdp) return;
  const int ncol = nf * npx;
  for (int c = blockIdx.y; c < ncol; c += gridDim.y) {
    float2 v = make_float2(0.f, 0.f);
    if (s < Kd) {
      const int reg = pix_regions[c % npx];
      const RegionT g = regs[reg];
      const double2 k0 = K0[c];
      if (g.klass == 2) {
        v = cexpm1_f(k0.y * g.dz, -k0.x * g.dz);   // propagator1D: exp(-i k0 dz), a large phase
      } else {
        // tilt and surface phases are small (k0 t ~ 0.1 rad): FP32 carries
        // them to ~1e-8 rad
        const int x = supp[s] % nx, y = supp[s] / nx;
        const float2 kf = make_float2((float)k0.x, (float)k0.y);
        const float t = fmaf((float)g.tx, (float)X[x], (float)g.ty * (float)Y[y]);
        float re = kf.y * t, im = -kf.x * t;
        if (surf) {
          const double2 sd = surf[(size_t)reg * npix + supp[s]];
          const float2 sv = make_float2((float)sd.x, (float)sd.y);
          re += kf.x * sv.y + kf.y * sv.x;
          im -= kf.x * sv.x - kf.y * sv.y;
        }
        v = cexpm1_ff(re, im);
      }
    }
    put_tf32(Bh, Bl, (size_t)(2 * c) * Kdp + s, v.x);
    put_tf32(Bh, Bl, (size_t)(2 * c + 1) * Kdp + s, v.y);
  }
}

// P from the tensor-core GEMM's output out[z][n][m] (FP32, n = 2c + {Re, Im}
// of column c, m = real row) with the subtracted constant added back:
// H[r][c] = sum_z out[z][2c..2c+1][r] + cc[c] g[r] (cc = null: 1), then
// P[m][m'] = X + iY and P[m'][m] = X - iY with X = H[2t], Y = H[2t+1], as
// k_scatter_herm; disk regions get diag(DG) from the left.
// One thread per (column c, pair t), t fastest: the reads of out are float2
// runs along m, the writes stay inside one column's matrix.  nrep > 1 (the
// pixel class of a group solve, the same for every request): the matrices of
// column (f, q) are written for frequencies f, f + nf, ...
template <typename PT>
__global__ void k_scatter_herm_tc(PT* P, const float* out, int Mp, int splits, const double2* cc, const double* g,
                                  int nf, int ncols, const RegionT* regs, const int* cls_regions, int nd, int nm,
                                  const double2* DG, const int2* tri, int T, int nrep) {
  const int ncol = nf * ncols;
  const size_t plane = (size_t)2 * ncol * Mp;
  const size_t total = (size_t)ncol * T;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const int c = (int)(i / T), t = (int)(i % T);
    const int2 mp = tri[t];
    const double g0 = g[2 * t], g1 = g[2 * t + 1];
    const int f = c / ncols, q = c % ncols;
    const int j = cls_regions[q];
    double xr = 0.0, xi = 0.0, yr = 0.0, yi = 0.0;
    for (int z = 0; z < splits; ++z) {
      const float2 re = *reinterpret_cast<const float2*>(out + z * plane + (size_t)(2 * c) * Mp + 2 * t);
      const float2 im = *reinterpret_cast<const float2*>(out + z * plane + (size_t)(2 * c + 1) * Mp + 2 * t);
      xr += (double)re.x;
      yr += (double)re.y;
      xi += (double)im.x;
      yi += (double)im.y;
    }
    const double2 k = cc ? cc[c] : make_double2(1.0, 0.0);
    xr += k.x * g0;
    xi += k.y * g0;
    yr += k.x * g1;
    yi += k.y * g1;
    double2 p1 = make_double2(xr - yi, xi + yr);
    double2 p2 = make_double2(xr + yi, xi - yr);
    if (DG && regs[j].klass == 1) {
      p1 = bf::cmul(DG[(size_t)c * nm + mp.x], p1);
      p2 = bf::cmul(DG[(size_t)c * nm + mp.y], p2);
    }
    for (int r = 0; r < nrep; ++r) {
      PT* Pj = P + ((size_t)(r * nf + f) * nd + j) * nm * nm;
      Pj[(size_t)mp.x * nm + mp.y] = dto<PT>(p1);
      if (mp.x != mp.y) Pj[(size_t)mp.y * nm + mp.x] = dto<PT>(p2);
    }
  }
}

// D[o][(r nf + f) npar + p] = exp(-i kz dz_p) (the k-space class GEMM
// operand); r is the request of a group solve, whose regions are regs[r nd ..].
template <typename C>
__global__ void k_build_d(C* D, const double2* KZ, int K, int nf, int ncol, int nd, const RegionT* regs,
                          const int* par_regions, const int* par_eps, int npar) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;   // (r nf + f) npar + p
  if (c >= ncol) return;
  const int F = c / npar, p = c % npar, f = F % nf, r = F / nf;
  const double dz = regs[(size_t)r * nd + par_regions[p]].dz;
  const double2* kzp = KZ + ((size_t)par_eps[p] * nf + f) * K;
  for (int o = blockIdx.y; o < K; o += gridDim.y) {
    const double2 kz = kzp[o];
    D[(size_t)o * ncol + c] = cexp_as<C>(kz.y * dz, -kz.x * dz);
  }
}

// k0[f][q] of the pixel-class regions (FP64)
__global__ void k_build_k0(double2* K0, const double* freqs, int nf, const RegionT* regs, const int* pix_regions,
                           int npx) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nf * npx) return;
  const RegionT g = regs[pix_regions[c % npx]];
  K0[c] = k0_c(kC / freqs[c / npx], g.er, g.ei);
}

// E[s][f*npx + q]: tilt/surface phase of pixel class regions at support pixel s
template <typename C>
__global__ void k_build_e(C* E, const int* supp, int Kd, int nf, const RegionT* regs, const int* pix_regions,
                          int npx, const double2* K0, const double* X, const double* Y, int nx,
                          const double2* surf, int npix) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  const int ncol = nf * npx;
  if (c >= ncol) return;
  const int q = c % npx;
  const int reg = pix_regions[q];
  const RegionT g = regs[reg];
  const double2 k0 = K0[c];
  for (int s = blockIdx.y; s < Kd; s += gridDim.y) {
    const int x = supp[s] % nx, y = supp[s] / nx;
    if constexpr (std::is_same<C, float2>::value) {
      double re, im;
      if (g.klass == 2) {
        re = k0.y * g.dz;   // propagator1D: exp(-i k0 dz)
        im = -k0.x * g.dz;
      } else {
        const double t = g.tx * X[x] + g.ty * Y[y];
        re = k0.y * t;
        im = -k0.x * t;
        if (surf) {
          const double2 sv = surf[(size_t)reg * npix + supp[s]];
          re += k0.x * sv.y + k0.y * sv.x;
          im -= k0.x * sv.x - k0.y * sv.y;
        }
      }
      E[(size_t)s * ncol + c] = cexp_as<C>(re, im);
    } else {
      double2 v;
      if (g.klass == 2) {
        v = dexp_c(k0.y * g.dz, -k0.x * g.dz);
      } else {
        const double2 a = dexp_c(k0.y * g.tx * X[x], -k0.x * g.tx * X[x]);
        const double2 b = dexp_c(k0.y * g.ty * Y[y], -k0.x * g.ty * Y[y]);
        v = bf::cmul(a, b);
        if (surf) {
          const double2 sv = surf[(size_t)reg * npix + supp[s]];
          const double re = k0.x * sv.x - k0.y * sv.y, im = k0.x * sv.y + k0.y * sv.x;
          v = bf::cmul(v, dexp_c(im, -re));
        }
      }
      E[(size_t)s * ncol + c] = v;
    }
  }
}

// diag[f][q][m] = exp(-i kz_m dz) with kz_m = sqrt(k0^2 - kT_m^2): the
// propagation of a pixel-class disk region in the mode basis (FP64)
__global__ void k_build_diag(double2* DG, const double2* K0, int nf, int npx, const RegionT* regs,
                             const int* pix_regions, const double2* kt, int nm) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= (size_t)nf * npx * nm) return;
  const int m = (int)(i % nm);
  const int c = (int)(i / nm);   // f * npx + q
  const RegionT g = regs[pix_regions[c % npx]];
  const double2 k0 = K0[c];
  const double2 k0sq = make_double2(k0.x * k0.x - k0.y * k0.y, k0.x * k0.y + k0.y * k0.x);
  const double2 t = kt[m];
  const double2 ktsq = make_double2(t.x * t.x - t.y * t.y, t.x * t.y + t.y * t.x);
  const double2 kz = dsqrt_c(k0sq.x - ktsq.x, k0sq.y - ktsq.y);
  DG[i] = dexp_c(kz.y * g.dz, -kz.x * g.dz);
}

// P[f][j][m][m'] from a class GEMM output G[mm'][f*ncols + col]; pixel-class
// disk regions get the propagation diag(exp(-i kz_m dz)) from the left.
template <typename PT>
__global__ void k_scatter_p(PT* P, const double2* Gm, int nf, int ncols, const RegionT* regs,
                            const int* cls_regions, int nd, int nm, const double2* DG, int nrep) {
  using C = double2;
  const int mm = blockIdx.x * blockDim.x + threadIdx.x;
  if (mm >= nm * nm) return;
  for (int c = blockIdx.y; c < nf * ncols; c += gridDim.y) {
    const int f = c / ncols, q = c % ncols;
    const int j = cls_regions[q];
    const RegionT g = regs[j];
    C v = Gm[(size_t)mm * (nf * ncols) + c];
    if (DG && g.klass == 1) v = bf::cmul(DG[(size_t)c * nm + mm / nm], v);
    for (int r = 0; r < nrep; ++r) P[(((size_t)(r * nf + f) * nd + j) * nm) * nm + mm] = dto<PT>(v);
  }
}

// P[f][j] of the pixel class from the real-row GEMM output H[2T][f*ncols + col]
// (rows of k_build_vr): with X = H[2t] and Y = H[2t+1],
// P[m][m'] = X + iY and P[m'][m] = X - iY; disk regions get diag(DG) from the left.
template <typename PT>
__global__ void k_scatter_herm(PT* P, const double2* H, int nf, int ncols, const RegionT* regs,
                               const int* cls_regions, int nd, int nm, const double2* DG, const int2* tri, int T,
                               int nrep) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  const int2 mp = tri[t];
  const size_t N = (size_t)nf * ncols;
  for (int c = blockIdx.y; c < nf * ncols; c += gridDim.y) {
    const int f = c / ncols, q = c % ncols;
    const int j = cls_regions[q];
    const double2 X = H[(size_t)(2 * t) * N + c], Y = H[(size_t)(2 * t + 1) * N + c];
    double2 p1 = make_double2(X.x - Y.y, X.y + Y.x);
    double2 p2 = make_double2(X.x + Y.y, X.y - Y.x);
    if (DG && regs[j].klass == 1) {
      p1 = bf::cmul(DG[(size_t)c * nm + mp.x], p1);
      p2 = bf::cmul(DG[(size_t)c * nm + mp.y], p2);
    }
    for (int r = 0; r < nrep; ++r) {
      PT* Pj = P + ((size_t)(r * nf + f) * nd + j) * nm * nm;
      Pj[(size_t)mp.x * nm + mp.y] = dto<PT>(p1);
      if (mp.x != mp.y) Pj[(size_t)mp.y * nm + mp.x] = dto<PT>(p2);
    }
  }
}

// field class: P[m][m'] = sum_x conj(Psi_m(x)) Q[m'][x]
template <typename PT, typename C>
__global__ void k_overlap(PT* P, const double2* pat, const C* Q, int nm, int npix) {
  const int mm = blockIdx.x;
  const int m = mm / nm, mp = mm % nm;
  __shared__ double2 red[256];
  double2 acc = make_double2(0.0, 0.0);
  for (int x = threadIdx.x; x < npix; x += blockDim.x) {
    const double2 a = pat[(size_t)m * npix + x];
    const double2 b = bf::to_d(Q[(size_t)mp * npix + x]);
    acc.x += a.x * b.x + a.y * b.y;
    acc.y += a.x * b.y - a.y * b.x;
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      red[threadIdx.x].x += red[threadIdx.x + s].x;
      red[threadIdx.x].y += red[threadIdx.x + s].y;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) P[mm] = dto<PT>(red[0]);
}

template <typename C>
__global__ void k_copy_modes(C* out, const double2* pat, int nm, int npix, int reps) {
  const size_t total = (size_t)reps * nm * npix;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x)
    out[i] = dto<C>(pat[i % ((size_t)nm * npix)]);
}

// ---- batched inversion, one warp per matrix (nm <= NM <= 32) -------------------
// Gauss-Jordan with partial pivoting: lane r keeps row r of [A | I] in
// registers (the column loop is unrolled, so every index is static); the
// pivot is a warp argmax (largest |a|^2, lowest row on ties), row swaps and
// the pivot-row broadcast are shuffles.  Rows nm..NM-1 are identity padding.
// The pivot magnitudes and the pivot reciprocal are computed in the matrix's
// own precision: FP32 for complex64 (a warp-wide FP64 instruction costs the
// same with one lane active, at 1/64 of the FP32 rate), FP64 for complex128.
// jl (nullable): invert only the regions jl[0 .. njl) of frequencies f0, f0 + 1, ...
// A warp holds 32 / NM matrices, one per segment of NM lanes (shuffles of
// width NM), so an 8 x 8 inverse does not leave 24 of 32 lanes idle.
template <typename C, int NM>
__global__ void __launch_bounds__(256) k_invert_warp(const C* P, C* Pinv, int nd, int j0, int nm, int nmat,
                                                     int* sing, int f0 = 0, const int* jl = nullptr, int njl = 0) {
  using R = decltype(C().x);
  constexpr unsigned FULL = 0xffffffffu;
  constexpr int SEG = 32 / NM;
  const int lane = threadIdx.x & 31, sl = lane % NM;
  const int first = (blockIdx.x * 8 + (threadIdx.x >> 5)) * SEG;
  if (first >= nmat) return;   // the whole warp leaves together
  const int idx = first + lane / NM;
  const bool valid = idx < nmat;
  const int nj = jl ? njl : nd - j0;
  const int q = valid ? idx : first;
  const int f = f0 + q / nj, j = jl ? jl[q % nj] : j0 + q % nj;
  const size_t off = (((size_t)f * nd + j) * nm) * nm;
  C a[NM], b[NM];
#pragma unroll
  for (int c = 0; c < NM; ++c) {
    if (sl < nm && c < nm) a[c] = P[off + (size_t)sl * nm + c];
    else a[c] = bf::mk(R(sl == c ? 1 : 0), R(0));
    b[c] = bf::mk(R(sl == c ? 1 : 0), R(0));
  }
#pragma unroll
  for (int c = 0; c < NM; ++c) {
    R v = sl >= c ? a[c].x * a[c].x + a[c].y * a[c].y : R(-1);
    int p = sl;
#pragma unroll
    for (int o = NM / 2; o > 0; o >>= 1) {
      const R vo = __shfl_xor_sync(FULL, v, o, NM);
      const int po = __shfl_xor_sync(FULL, p, o, NM);
      if (vo > v || (vo == v && po < p)) {
        v = vo;
        p = po;
      }
    }
    const int src = sl == c ? p : (sl == p ? c : sl);
#pragma unroll
    for (int k = 0; k < NM; ++k) {
      a[k].x = __shfl_sync(FULL, a[k].x, src, NM);
      a[k].y = __shfl_sync(FULL, a[k].y, src, NM);
      b[k].x = __shfl_sync(FULL, b[k].x, src, NM);
      b[k].y = __shfl_sync(FULL, b[k].y, src, NM);
    }
    if (sl == c) {
      if (valid && a[c].x == R(0) && a[c].y == R(0)) atomicMin(sing, f);   // exactly singular (LAPACK info > 0)
      const R d = a[c].x * a[c].x + a[c].y * a[c].y;
      const C inv = bf::mk(a[c].x / d, -a[c].y / d);
#pragma unroll
      for (int k = 0; k < NM; ++k) {
        a[k] = bf::cmul(a[k], inv);
        b[k] = bf::cmul(b[k], inv);
      }
    }
    const C fct = a[c];
#pragma unroll
    for (int k = 0; k < NM; ++k) {
      C pa, pb;
      pa.x = __shfl_sync(FULL, a[k].x, c, NM);
      pa.y = __shfl_sync(FULL, a[k].y, c, NM);
      pb.x = __shfl_sync(FULL, b[k].x, c, NM);
      pb.y = __shfl_sync(FULL, b[k].y, c, NM);
      if (sl != c) {
        a[k] = bf::csub(a[k], bf::cmul(fct, pa));
        b[k] = bf::csub(b[k], bf::cmul(fct, pb));
      }
    }
  }
  if (valid && sl < nm)
#pragma unroll
    for (int c = 0; c < NM; ++c)
      if (c < nm) Pinv[off + (size_t)sl * nm + c] = b[c];
}

// ---- batched inversion: Pinv[f][j] = inv(P[f][j]), j in [j0, nd) -----------
template <typename C>
__global__ void __launch_bounds__(256) k_invert(const C* P, C* Pinv, int nd, int j0, int nm, int* sing, int f0 = 0,
                                                const int* jl = nullptr) {
  extern __shared__ __align__(16) unsigned char sm[];
  C* W = reinterpret_cast<C*>(sm);
  double* red_v = reinterpret_cast<double*>(W + 2 * nm * nm);
  int* red_i = reinterpret_cast<int*>(red_v + 256);
  const int f = f0 + blockIdx.y, j = jl ? jl[blockIdx.x] : j0 + blockIdx.x;
  const size_t off = (((size_t)f * nd + j) * nm) * nm;
  C* M = Pinv + off;
  for (int e = threadIdx.x; e < nm * nm; e += blockDim.x) M[e] = P[off + e];
  __syncthreads();
  bf::cta_invert(M, W, nm, sing, f, red_v, red_i);
}

// ---- batched inversion of complex64 matrices, 16 < nm <= NB, in registers ----
// Gauss-Jordan by Jordan exchanges with implicit partial pivoting.  The matrix,
// padded to NB x NB with the identity, lives in registers, 4 x 4 entries per
// thread.  Step c takes the unused row p with the largest |A[p][c]|^2 (lowest
// row on ties), d = 1/A[p][c] and R[k] = -A[p][k] d, then
//   A[r][k] += A[r][c] R[k] (r != p, k != c),   A[r][c] = A[r][c] d (r != p),
//   A[p][k] = R[k] (k != c),                    A[p][c] = d.
// After nm steps row p_c expresses x_c in the y_{p_k}: inv[c][p_k] = A[p_c][k].
// Shared memory carries only the pivot column (double-buffered by step parity)
// and the scaled pivot row, so each step is 16 complex FMAs per thread against
// 8 shared loads.  An exactly zero pivot (the remaining column is zero, the
// case where LAPACK's getrf reports info > 0 and Julia's inv raises
// SingularException) records the frequency in *sing (atomicMin); the inverse
// is then inf/NaN.
__device__ __forceinline__ float2 pick4(const float2 (&v)[4], int s) {
  float2 r = v[0];
  if (s == 1) r = v[1];
  if (s == 2) r = v[2];
  if (s == 3) r = v[3];
  return r;
}

template <int NB>
__global__ void __launch_bounds__((NB / 4) * (NB / 4)) k_invert_reg(const float2* P, float2* Pinv, int nd, int j0,
                                                                  int nm, int* sing, int f0 = 0,
                                                                  const int* jl = nullptr) {
  constexpr int NBB = NB / 4, NT = NBB * NBB, RPL = NB / 32;
  constexpr unsigned FULL = 0xffffffffu;
  __shared__ float2 colv[2][NB], rowv[NB];
  __shared__ int piv[NB], cof[NB];
  __shared__ float2 dsh;
  __shared__ int psh;
  __shared__ float2 outs[NB * NB];
  const int tid = threadIdx.x, br = tid / NBB, bc = tid % NBB, lane = tid & 31;
  const int f = f0 + blockIdx.y, j = jl ? jl[blockIdx.x] : j0 + blockIdx.x;
  const size_t off = (((size_t)f * nd + j) * nm) * nm;
  float2 A[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int r = br * 4 + i, k = bc * 4 + q;
      A[i][q] = (r < nm && k < nm) ? P[off + (size_t)r * nm + k] : make_float2(r == k ? 1.f : 0.f, 0.f);
    }
  bool used[RPL];
#pragma unroll
  for (int q = 0; q < RPL; ++q) used[q] = false;
  for (int c = 0; c < nm; ++c) {
    const int cb = c >> 2, cs = c & 3;
    float2* cv = colv[c & 1];
    if (bc == cb)
#pragma unroll
      for (int i = 0; i < 4; ++i) cv[br * 4 + i] = pick4(A[i], cs);
    __syncthreads();
    if (tid < 32) {
      float best = -1.f;
      int bi = NB;
#pragma unroll
      for (int q = 0; q < RPL; ++q) {
        const int r = lane + 32 * q;
        if (r < nm && !used[q]) {
          const float2 a = cv[r];
          float v = a.x * a.x + a.y * a.y;
          if (v != v) v = INFINITY;   // NaN orders as largest: the argmax stays a total order
          if (v > best) { best = v; bi = r; }
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const float vo = __shfl_xor_sync(FULL, best, o);
        const int io = __shfl_xor_sync(FULL, bi, o);
        if (vo > best || (vo == best && io < bi)) { best = vo; bi = io; }
      }
      bi = min(bi, nm - 1);   // an unused row < nm always exists; keeps cv[] in bounds
#pragma unroll
      for (int q = 0; q < RPL; ++q)
        if (lane + 32 * q == bi) used[q] = true;
      if (lane == 0) {
        const float2 a = cv[bi];
        if (a.x == 0.f && a.y == 0.f) atomicMin(sing, f);   // exactly singular (LAPACK info > 0)
        const float s2 = a.x * a.x + a.y * a.y;
        dsh = make_float2(a.x / s2, -a.y / s2);
        psh = bi;
        piv[c] = bi;
        cof[bi] = c;
        cv[bi] = make_float2(0.f, 0.f);
      }
    }
    __syncthreads();
    const int p = psh;
    const float2 d = dsh;
    if (br == (p >> 2))
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        float2 a = A[0][q];
        if ((p & 3) == 1) a = A[1][q];
        if ((p & 3) == 2) a = A[2][q];
        if ((p & 3) == 3) a = A[3][q];
        const int k = bc * 4 + q;
        rowv[k] = k == c ? make_float2(0.f, 0.f)
                         : make_float2(-(a.x * d.x - a.y * d.y), -(a.x * d.y + a.y * d.x));
      }
    __syncthreads();
    float2 F[4], R[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) F[i] = cv[br * 4 + i];
#pragma unroll
    for (int q = 0; q < 4; ++q) R[q] = rowv[bc * 4 + q];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        A[i][q].x = fmaf(F[i].x, R[q].x, fmaf(-F[i].y, R[q].y, A[i][q].x));
        A[i][q].y = fmaf(F[i].x, R[q].y, fmaf(F[i].y, R[q].x, A[i][q].y));
      }
    // column c: A[r][c] d (r != p) and d; row p: R (k != c)
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int r = br * 4 + i;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int k = bc * 4 + q;
        if (k == c) {
          A[i][q] = r == p ? d : make_float2(F[i].x * d.x - F[i].y * d.y, F[i].x * d.y + F[i].y * d.x);
        } else if (r == p) {
          A[i][q] = R[q];
        }
      }
    }
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int r = br * 4 + i, k = bc * 4 + q;
      if (r < nm && k < nm) outs[cof[r] * nm + piv[k]] = A[i][q];
    }
  __syncthreads();
  for (int e = tid; e < nm * nm; e += NT) Pinv[off + e] = outs[e];
}

// Group solves: the inverses of regions jl[0 .. njl) of request 0 (frequencies
// [0, nf)) copied to requests 1 .. nreq-1, whose matrices there are the same.
template <typename C>
__global__ void k_copy_inverses(C* Pinv, int nd, int nm, int nf, int nreq, const int* jl, int njl) {
  const size_t n2 = (size_t)nm * nm;
  const size_t per = (size_t)nf * njl * n2;   // entries of request 0 to copy
  const size_t total = per * (nreq - 1);
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const size_t r = 1 + i / per, q = i % per;
    const size_t e = q % n2, fj = q / n2;
    const int f = (int)(fj / njl), j = jl[fj % njl];
    Pinv[(((r * nf + f) * nd) + j) * n2 + e] = Pinv[(((size_t)f * nd) + j) * n2 + e];
  }
}

// ---- the chain: one CTA per frequency ---------------------------------------
struct ChainRegion {
  double2 a, b, inv2n;   // G = (1/(2 n_r)) [[a I, b I], [b I, a I]]
  double2 S;             // axion S factor of the step
};

template <typename C>
__global__ void __launch_bounds__(256) k_chain(const C* P, const C* Pinv, const ChainRegion* cr, int nd,
                                               int nm, const double2* emit, C* T21g, C* T22g,
                                               double2* axg) {
  extern __shared__ __align__(16) unsigned char sm[];
  C* U = reinterpret_cast<C*>(sm);
  C* V = U + nm * nm;
  double2* ax = reinterpret_cast<double2*>(V + nm * nm);
  double2* em = ax + nm;
  const int f = blockIdx.x, tid = threadIdx.x, nt = blockDim.x;
  C* T21 = T21g + (size_t)f * nm * nm;
  C* T22 = T22g + (size_t)f * nm * nm;
  for (int e = tid; e < nm * nm; e += nt) {
    T21[e] = dto<C>(make_double2(0.0, 0.0));
    T22[e] = dto<C>(make_double2((e / nm) == (e % nm) ? 1.0 : 0.0, 0.0));
  }
  for (int m = tid; m < nm; m += nt) {
    ax[m] = make_double2(0.0, 0.0);
    em[m] = emit[m];
  }
  __syncthreads();
  for (int j = 1; j < nd; ++j) {
    const ChainRegion g = cr[j];
    // axion_beam += S (T21 + T22) emit   (uses T of the previous step)
    for (int m = tid; m < nm; m += nt) {
      double2 acc = make_double2(0.0, 0.0);
      for (int k = 0; k < nm; ++k) {
        const double2 t = bf::to_d(bf::cadd(T21[m * nm + k], T22[m * nm + k]));
        acc = bf::cadd(acc, bf::cmul(t, em[k]));
      }
      ax[m] = bf::cadd(ax[m], bf::cmul(g.S, acc));
    }
    // U = a T21 + b T22, V = b T21 + a T22
    const C a = dto<C>(g.a), b = dto<C>(g.b), s = dto<C>(g.inv2n);
    for (int e = tid; e < nm * nm; e += nt) {
      const C t1 = T21[e], t2 = T22[e];
      U[e] = bf::cadd(bf::cmul(a, t1), bf::cmul(b, t2));
      V[e] = bf::cadd(bf::cmul(b, t1), bf::cmul(a, t2));
    }
    __syncthreads();
    const C* Pj = P + (((size_t)f * nd + j) * nm) * nm;
    const C* Qj = Pinv + (((size_t)f * nd + j) * nm) * nm;
    // T21 = s U P, T22 = s V Pinv
    for (int e = tid; e < nm * nm; e += nt) {
      const int r = e / nm, c = e % nm;
      C acc1 = dto<C>(make_double2(0.0, 0.0)), acc2 = acc1;
      for (int k = 0; k < nm; ++k) {
        const C u = U[r * nm + k], v = V[r * nm + k];
        const C p = Pj[k * nm + c], q = Qj[k * nm + c];
        acc1.x += u.x * p.x - u.y * p.y;
        acc1.y += u.x * p.y + u.y * p.x;
        acc2.x += v.x * q.x - v.y * q.y;
        acc2.y += v.x * q.y + v.y * q.x;
      }
      T21[e] = bf::cmul(s, acc1);
      T22[e] = bf::cmul(s, acc2);
    }
    __syncthreads();
  }
  for (int m = tid; m < nm; m += nt) axg[(size_t)f * nm + m] = ax[m];
}

// ---- the chain in double-float (mixed path) -----------------------------------
// T21 and T22 accumulate 2(nd-1) matrix products; near a resonance the final
// solve amplifies their relative error by cond(T22) ~ 1e3-1e4, so complex64
// storage of T (rounding ~6e-8 per step) misses the 1e-4 bar on beta^2 while
// complex64 P and inverse(P) do not.  Here T is a (hi, lo) FP32 pair per
// component (~48 bits): products of its hi part with the complex64 P are made
// exact with FMA error terms and summed with TwoSum, its lo part is summed in
// FP32, and the scalar steps use double-float arithmetic -- all on the FP32
// pipes.  One CTA of 1024 threads per frequency; U, V, P_j and inverse(P_j)
// in shared memory.
struct DFc { float rh, rl, ih, il; };   // complex double-float

__device__ __forceinline__ void df_two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float z = s - a;
  e = (a - (s - z)) + (b - z);
}
__device__ __forceinline__ void df_fast_two_sum(float& hi, float& lo) {
  const float s = hi + lo;
  lo = lo - (s - hi);
  hi = s;
}
// (sh, sl) += a * b, the product exact
__device__ __forceinline__ void df_acc_prod(float& sh, float& sl, float a, float b) {
  const float p = a * b;
  const float e = fmaf(a, b, -p);
  float s, t;
  df_two_sum(sh, p, s, t);
  sh = s;
  sl += t + e;
}
__device__ __forceinline__ DFc dfc_from(double2 v) {
  DFc r;
  r.rh = (float)v.x;
  r.rl = (float)(v.x - (double)r.rh);
  r.ih = (float)v.y;
  r.il = (float)(v.y - (double)r.ih);
  return r;
}
__device__ __forceinline__ double2 dfc_to_d(DFc v) {
  return make_double2((double)v.rh + (double)v.rl, (double)v.ih + (double)v.il);
}
// x * y in double-float (x, y double-float; error ~1e-14 relative)
__device__ __forceinline__ DFc dfc_mul(DFc x, DFc y) {
  DFc r;
  float sh = 0.f, sl = 0.f;
  df_acc_prod(sh, sl, x.rh, y.rh);
  df_acc_prod(sh, sl, -x.ih, y.ih);
  sl += x.rh * y.rl + x.rl * y.rh - x.ih * y.il - x.il * y.ih;
  df_fast_two_sum(sh, sl);
  r.rh = sh;
  r.rl = sl;
  sh = 0.f;
  sl = 0.f;
  df_acc_prod(sh, sl, x.rh, y.ih);
  df_acc_prod(sh, sl, x.ih, y.rh);
  sl += x.rh * y.il + x.rl * y.ih + x.ih * y.rl + x.il * y.rh;
  df_fast_two_sum(sh, sl);
  r.ih = sh;
  r.il = sl;
  return r;
}
__device__ __forceinline__ DFc dfc_add(DFc x, DFc y) {
  DFc r;
  float e;
  df_two_sum(x.rh, y.rh, r.rh, e);
  r.rl = e + x.rl + y.rl;
  df_fast_two_sum(r.rh, r.rl);
  df_two_sum(x.ih, y.ih, r.ih, e);
  r.il = e + x.il + y.il;
  df_fast_two_sum(r.ih, r.il);
  return r;
}

__global__ void __launch_bounds__(1024) k_chain_df(const float2* P, const float2* Pinv, const ChainRegion* cr,
                                                  int nd, int nm, const double2* emit, DFc* T21g, DFc* T22g,
                                                  double2* axg, double2* T21out, double2* T22out, int par_axion,
                                                  DFc* Wg) {
  extern __shared__ __align__(16) unsigned char sm[];
  const int n2 = nm * nm;
  DFc* U = reinterpret_cast<DFc*>(sm);
  DFc* V = U + n2;
  float2* Ps = reinterpret_cast<float2*>(V + n2);
  float2* Qs = Ps + n2;
  double2* ax = reinterpret_cast<double2*>(Qs + n2);
  DFc* em = reinterpret_cast<DFc*>(ax + nm);
  const int f = blockIdx.x, tid = threadIdx.x, nt = blockDim.x;
  // T lives in shared memory when the launch gave room for it (T21g null):
  // the axion sum reads a row of T per step, one dependent load per entry
  DFc* T21 = T21g ? T21g + (size_t)f * n2 : em + nm;
  DFc* T22 = T21g ? T22g + (size_t)f * n2 : em + nm + n2;
  // par_axion (T in shared memory and room for one more matrix), or Wg (T in
  // global memory, a global scratch of one matrix per frequency): the axion
  // terms of all (m, k) are formed in parallel into Wt, then each row is
  // summed in k order as the serial form does (same values, shorter chain)
  DFc* Wt = par_axion ? em + nm + 2 * n2 : (Wg ? Wg + (size_t)f * n2 : nullptr);
  const DFc zero = {0.f, 0.f, 0.f, 0.f}, one = {1.f, 0.f, 0.f, 0.f};
  for (int e = tid; e < n2; e += nt) {
    T21[e] = zero;
    T22[e] = (e / nm) == (e % nm) ? one : zero;
  }
  for (int m = tid; m < nm; m += nt) {
    ax[m] = make_double2(0.0, 0.0);
    em[m] = dfc_from(emit[m]);
  }
  // one matrix entry per thread (small mode counts): the next region's P and
  // inverse(P) are loaded into registers one region ahead, so their latency
  // hides behind this region's products
  const bool ahead = n2 <= nt;
  float2 pn = make_float2(0.f, 0.f), qn = pn;
  if (ahead && tid < n2 && nd > 1) {
    pn = P[(((size_t)f * nd + 1) * nm) * nm + tid];
    qn = Pinv[(((size_t)f * nd + 1) * nm) * nm + tid];
  }
  __syncthreads();
  for (int j = 1; j < nd; ++j) {
    const ChainRegion g = cr[j];
    // axion_beam += S (T21 + T22) emit   (T of the previous step)
    if (Wt) {
      for (int e = tid; e < n2; e += nt) Wt[e] = dfc_mul(dfc_add(T21[e], T22[e]), em[e % nm]);
    } else {
      for (int m = tid; m < nm; m += nt) {
        DFc acc = zero;
        for (int k = 0; k < nm; ++k) acc = dfc_add(acc, dfc_mul(dfc_add(T21[m * nm + k], T22[m * nm + k]), em[k]));
        const double2 v = dfc_to_d(acc);
        ax[m] = bf::cadd(ax[m], bf::cmul(g.S, v));
      }
    }
    // U = a T21 + b T22, V = b T21 + a T22; stage P_j and inverse(P_j)
    const DFc a = dfc_from(g.a), b = dfc_from(g.b), sc = dfc_from(g.inv2n);
    for (int e = tid; e < n2; e += nt) {
      const DFc t1 = T21[e], t2 = T22[e];
      U[e] = dfc_add(dfc_mul(a, t1), dfc_mul(b, t2));
      V[e] = dfc_add(dfc_mul(b, t1), dfc_mul(a, t2));
    }
    if (ahead) {
      if (tid < n2) {
        Ps[tid] = pn;
        Qs[tid] = qn;
        if (j + 1 < nd) {
          pn = P[(((size_t)f * nd + j + 1) * nm) * nm + tid];
          qn = Pinv[(((size_t)f * nd + j + 1) * nm) * nm + tid];
        }
      }
    } else {
      const float2* Pj = P + (((size_t)f * nd + j) * nm) * nm;
      const float2* Qj = Pinv + (((size_t)f * nd + j) * nm) * nm;
      for (int e = tid; e < n2; e += nt) {
        Ps[e] = Pj[e];
        Qs[e] = Qj[e];
      }
    }
    __syncthreads();
    if (Wt)   // reads only Wt: runs alongside the product below, which rewrites T
      for (int m = tid; m < nm; m += nt) {
        DFc acc = zero;
#pragma unroll 8
        for (int k = 0; k < nm; ++k) acc = dfc_add(acc, Wt[m * nm + k]);
        const double2 v = dfc_to_d(acc);
        ax[m] = bf::cadd(ax[m], bf::cmul(g.S, v));
      }
    // T21 = s U P, T22 = s V inverse(P)
    for (int e = tid; e < n2; e += nt) {
      const int r = e / nm, c = e % nm;
      float r1h = 0.f, r1l = 0.f, i1h = 0.f, i1l = 0.f, r2h = 0.f, r2l = 0.f, i2h = 0.f, i2l = 0.f;
      for (int k = 0; k < nm; ++k) {
        const DFc u = U[r * nm + k], v = V[r * nm + k];
        const float2 p = Ps[k * nm + c], q = Qs[k * nm + c];
        df_acc_prod(r1h, r1l, u.rh, p.x);
        df_acc_prod(r1h, r1l, -u.ih, p.y);
        df_acc_prod(i1h, i1l, u.rh, p.y);
        df_acc_prod(i1h, i1l, u.ih, p.x);
        r1l = fmaf(u.rl, p.x, fmaf(-u.il, p.y, r1l));
        i1l = fmaf(u.rl, p.y, fmaf(u.il, p.x, i1l));
        df_acc_prod(r2h, r2l, v.rh, q.x);
        df_acc_prod(r2h, r2l, -v.ih, q.y);
        df_acc_prod(i2h, i2l, v.rh, q.y);
        df_acc_prod(i2h, i2l, v.ih, q.x);
        r2l = fmaf(v.rl, q.x, fmaf(-v.il, q.y, r2l));
        i2l = fmaf(v.rl, q.y, fmaf(v.il, q.x, i2l));
      }
      df_fast_two_sum(r1h, r1l);
      df_fast_two_sum(i1h, i1l);
      df_fast_two_sum(r2h, r2l);
      df_fast_two_sum(i2h, i2l);
      const DFc acc1 = {r1h, r1l, i1h, i1l}, acc2 = {r2h, r2l, i2h, i2l};
      T21[e] = dfc_mul(sc, acc1);
      T22[e] = dfc_mul(sc, acc2);
    }
    __syncthreads();
  }
  for (int m = tid; m < nm; m += nt) axg[(size_t)f * nm + m] = ax[m];
  for (int e = tid; e < n2; e += nt) {
    T21out[(size_t)f * n2 + e] = dfc_to_d(T21[e]);
    T22out[(size_t)f * n2 + e] = dfc_to_d(T22[e]);
  }
}

// ---- transformer_trace_back: per-region amplitudes, one CTA per frequency ----
// sol <- G_j blockdiag(P_j, inverse(P_j)) sol (+ S_j [emit; emit]), j = nd-1 .. 1,
// starting from vcat(input, reflected) in the last region; every region's
// vector is stored into its (2, nm) slice of the column-major (nd, 2, nm)
// output in column-major order, as the reference's slice assignment does
// (src/boost_fractor_transformer.jl:401, :419).  Vectors in FP64.
template <typename PT>
__global__ void __launch_bounds__(256) k_trace_back(const PT* P, const PT* Pinv, const ChainRegion* cr, int nd,
                                                    int nm, const double2* refl, const double2* inp,
                                                    int beam_stride, const double2* emit, int with_axion,
                                                    double2* out) {
  extern __shared__ __align__(16) unsigned char sm[];
  double2* Rv = reinterpret_cast<double2*>(sm);
  double2* Lv = Rv + nm;
  double2* R2 = Lv + nm;
  double2* L2 = R2 + nm;
  const int f = blockIdx.x, tid = threadIdx.x, nt = blockDim.x;
  double2* o = out + (size_t)f * nd * 2 * nm;
  for (int m = tid; m < nm; m += nt) {
    Rv[m] = inp[(size_t)f * beam_stride + m];
    Lv[m] = refl[(size_t)f * beam_stride + m];
  }
  __syncthreads();
  auto put = [&](int region) {
    for (int k = tid; k < 2 * nm; k += nt)
      o[region + (size_t)nd * ((k % 2) + 2 * (k / 2))] = k < nm ? Rv[k] : Lv[k - nm];
  };
  put(nd - 1);
  for (int st = 1; st < nd; ++st) {
    const int j = nd - st;
    const ChainRegion g = cr[j];
    const PT* Pj = P + (((size_t)f * nd + j) * nm) * nm;
    const PT* Qj = Pinv + (((size_t)f * nd + j) * nm) * nm;
    for (int r = tid; r < nm; r += nt) {
      double2 pr = make_double2(0.0, 0.0), ql = pr;
      for (int k = 0; k < nm; ++k) {
        pr = bf::cadd(pr, bf::cmul(bf::to_d(Pj[r * nm + k]), Rv[k]));
        ql = bf::cadd(ql, bf::cmul(bf::to_d(Qj[r * nm + k]), Lv[k]));
      }
      double2 nr = bf::cmul(g.inv2n, bf::cadd(bf::cmul(g.a, pr), bf::cmul(g.b, ql)));
      double2 nl = bf::cmul(g.inv2n, bf::cadd(bf::cmul(g.b, pr), bf::cmul(g.a, ql)));
      if (with_axion) {
        const double2 se = bf::cmul(g.S, emit[r]);
        nr = bf::cadd(nr, se);
        nl = bf::cadd(nl, se);
      }
      R2[r] = nr;
      L2[r] = nl;
    }
    __syncthreads();
    for (int m = tid; m < nm; m += nt) {
      Rv[m] = R2[m];
      Lv[m] = L2[m];
    }
    __syncthreads();
    put(j - 1);
  }
}

// ---- FP64 boundary solve: boost = -T22 \ ax, refl = -T22 \ (T21 reflect) ----
// An exactly zero pivot (Julia's `\` raises SingularException there,
// transformer.jl:346,356) records the frequency in *sing (atomicMin).
template <typename C>
__global__ void __launch_bounds__(256) k_final_solve(const C* T21g, const C* T22g, const double2* axg,
                                                     const double2* reflect, int nm, double2* boost,
                                                     double2* refl, double* beta2, int* sing) {
  extern __shared__ __align__(16) unsigned char sm[];
  const int f = blockIdx.x, tid = threadIdx.x, nt = blockDim.x;
  const int w = nm + 2;
  double2* A = reinterpret_cast<double2*>(sm);   // [nm][nm + 2]
  double* red_v = reinterpret_cast<double*>(A + nm * w);
  int* red_i = reinterpret_cast<int*>(red_v + 256);
  const C* T21 = T21g + (size_t)f * nm * nm;
  const C* T22 = T22g + (size_t)f * nm * nm;
  for (int e = tid; e < nm * nm; e += nt) A[(e / nm) * w + (e % nm)] = bf::to_d(T22[e]);
  for (int m = tid; m < nm; m += nt) {
    A[m * w + nm] = axg[(size_t)f * nm + m];
    double2 acc = make_double2(0.0, 0.0);
    if (reflect)
      for (int k = 0; k < nm; ++k) acc = bf::cadd(acc, bf::cmul(bf::to_d(T21[m * nm + k]), reflect[k]));
    A[m * w + nm + 1] = acc;
  }
  __syncthreads();
  // Gaussian elimination with partial pivoting (LAPACK getrf/getrs order)
  const int lane = tid & 31, wid = tid >> 5, nwarp = nt >> 5;
  for (int c = 0; c < nm; ++c) {
    // pivot: the largest |A[r][c]|^2 below the diagonal, the lowest row on
    // ties (a warp's candidates by shuffles, then the warps' in warp 0)
    double best = -1.0;
    int bi = c;
    for (int r = c + tid; r < nm; r += nt) {
      const double v = A[r * w + c].x * A[r * w + c].x + A[r * w + c].y * A[r * w + c].y;
      if (v > best) { best = v; bi = r; }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const double ov = __shfl_xor_sync(0xffffffffu, best, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
    }
    if (lane == 0) {
      red_v[wid] = best;
      red_i[wid] = bi;
    }
    __syncthreads();
    if (wid == 0) {
      best = lane < nwarp ? red_v[lane] : -1.0;
      bi = lane < nwarp ? red_i[lane] : nm;
      for (int o = 16; o > 0; o >>= 1) {
        const double ov = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
      }
      if (lane == 0) red_i[nwarp] = bi;
    }
    __syncthreads();
    const int p = red_i[nwarp];
    if (p != c)
      for (int k = tid; k < w; k += nt) {
        double2 t = A[c * w + k];
        A[c * w + k] = A[p * w + k];
        A[p * w + k] = t;
      }
    __syncthreads();
    const double2 piv = A[c * w + c];
    if (tid == 0 && piv.x == 0.0 && piv.y == 0.0) atomicMin(sing, f);   // T22 exactly singular
    // the multipliers l / piv, once per row (two FP64 divisions each), into
    // column c, which is cleared below
    const double d = piv.x * piv.x + piv.y * piv.y;
    for (int r = c + 1 + tid; r < nm; r += nt) {
      const double2 l = A[r * w + c];
      A[r * w + c] = make_double2((l.x * piv.x + l.y * piv.y) / d, (l.y * piv.x - l.x * piv.y) / d);
    }
    __syncthreads();
    for (int e = tid; e < (nm - c - 1) * (w - c - 1); e += nt) {
      const int r = c + 1 + e / (w - c - 1), k = c + 1 + e % (w - c - 1);
      A[r * w + k] = bf::csub(A[r * w + k], bf::cmul(A[r * w + c], A[c * w + k]));
    }
    __syncthreads();
    for (int r = c + 1 + tid; r < nm; r += nt) A[r * w + c] = make_double2(0.0, 0.0);
    __syncthreads();
  }
  // back substitution for both right-hand sides (serial per column, small)
  if (tid < 2) {
    const int col = nm + tid;
    for (int r = nm - 1; r >= 0; --r) {
      double2 acc = A[r * w + col];
      for (int k = r + 1; k < nm; ++k) acc = bf::csub(acc, bf::cmul(A[r * w + k], A[k * w + col]));
      const double2 piv = A[r * w + r];
      const double d = piv.x * piv.x + piv.y * piv.y;
      A[r * w + col] = make_double2((acc.x * piv.x + acc.y * piv.y) / d, (acc.y * piv.x - acc.x * piv.y) / d);
    }
  }
  __syncthreads();
  for (int m = tid; m < nm; m += nt) {
    const double2 x = A[m * w + nm];
    boost[(size_t)f * nm + m] = make_double2(-x.x, -x.y);
    if (refl) {
      const double2 y = A[m * w + nm + 1];
      refl[(size_t)f * nm + m] = make_double2(-y.x, -y.y);
    }
  }
  if (tid == 0 && beta2) {
    double s = 0.0;
    for (int m = 0; m < nm; ++m) {
      const double2 x = A[m * w + nm];
      s += x.x * x.x + x.y * x.y;
    }
    beta2[f] = s;
  }
}

// The boundary solve of k_final_solve for nm <= NM (8 or 16), one segment of
// NM lanes per frequency (32 / NM frequencies per warp): lane r holds row r of
// [T22 | axion_beam | T21 reflect] in registers, the pivot search is a shuffle
// argmax (largest |a|^2, lowest row on ties), the pivot row is broadcast by
// shuffles.  Every entry goes through the operations of k_final_solve in the
// same order (LU with partial pivoting, then back substitution); only the
// CTA-wide reductions and barriers are gone.
template <int NM>
__global__ void __launch_bounds__(256) k_final_solve_warp(const double2* T21g, const double2* T22g,
                                                          const double2* axg, const double2* reflect, int nm,
                                                          double2* boost, double2* refl, double* beta2, int* sing,
                                                          int nf) {
  constexpr unsigned FULL = 0xffffffffu;
  constexpr int W = NM + 2, SEG = 32 / NM;
  const int lane = threadIdx.x & 31, sl = lane % NM;
  const int first = (blockIdx.x * 8 + (threadIdx.x >> 5)) * SEG;
  if (first >= nf) return;   // the whole warp leaves together
  const int fi = first + lane / NM;
  const bool valid = fi < nf;
  const int f = valid ? fi : first;
  const double2* T21 = T21g + (size_t)f * nm * nm;
  const double2* T22 = T22g + (size_t)f * nm * nm;
  const bool row = sl < nm;
  double2 a[W];
#pragma unroll
  for (int k = 0; k < W; ++k) a[k] = make_double2(0.0, 0.0);
  if (row) {
#pragma unroll
    for (int k = 0; k < NM; ++k)
      if (k < nm) a[k] = T22[sl * nm + k];
    a[NM] = axg[(size_t)f * nm + sl];
    double2 acc = make_double2(0.0, 0.0);
    if (reflect)
      for (int k = 0; k < nm; ++k) acc = bf::cadd(acc, bf::cmul(T21[sl * nm + k], reflect[k]));
    a[NM + 1] = acc;
  }
  auto bcast = [&](double2 v, int src) {
    return make_double2(__shfl_sync(FULL, v.x, src, NM), __shfl_sync(FULL, v.y, src, NM));
  };
#pragma unroll
  for (int c = 0; c < NM; ++c) {
    if (c >= nm) break;
    double v = (row && sl >= c) ? a[c].x * a[c].x + a[c].y * a[c].y : -1.0;
    int p = (row && sl >= c) ? sl : NM;
#pragma unroll
    for (int o = NM / 2; o > 0; o >>= 1) {
      const double vo = __shfl_xor_sync(FULL, v, o, NM);
      const int po = __shfl_xor_sync(FULL, p, o, NM);
      if (vo > v || (vo == v && po < p)) { v = vo; p = po; }
    }
    if (p >= nm) p = c;
    // swap rows c and p
    const int src = sl == c ? p : (sl == p ? c : sl);
#pragma unroll
    for (int k = 0; k < W; ++k) a[k] = bcast(a[k], src);
    const double2 piv = bcast(a[c], c);
    if (valid && sl == 0 && piv.x == 0.0 && piv.y == 0.0) atomicMin(sing, f);   // T22 exactly singular
    const double d = piv.x * piv.x + piv.y * piv.y;
    const double2 l = a[c];
    const double2 fac = make_double2((l.x * piv.x + l.y * piv.y) / d, (l.y * piv.x - l.x * piv.y) / d);
#pragma unroll
    for (int k = 0; k < W; ++k) {
      if (k <= c || (k >= nm && k < NM)) continue;
      const double2 pk = bcast(a[k], c);
      if (row && sl > c) a[k] = bf::csub(a[k], bf::cmul(fac, pk));
    }
    if (row && sl > c) a[c] = make_double2(0.0, 0.0);
  }
  // back substitution for both right-hand sides, rows nm-1 .. 0
  double2 x0[NM], x1[NM];
#pragma unroll
  for (int r = NM - 1; r >= 0; --r) {
    if (r >= nm) {
      x0[r] = x1[r] = make_double2(0.0, 0.0);
      continue;
    }
    double2 acc0 = a[NM], acc1 = a[NM + 1];
#pragma unroll
    for (int k = r + 1; k < NM; ++k) {
      if (k >= nm) break;
      acc0 = bf::csub(acc0, bf::cmul(a[k], x0[k]));
      acc1 = bf::csub(acc1, bf::cmul(a[k], x1[k]));
    }
    const double2 pv = a[r];
    const double dd = pv.x * pv.x + pv.y * pv.y;
    const double2 s0 = make_double2((acc0.x * pv.x + acc0.y * pv.y) / dd, (acc0.y * pv.x - acc0.x * pv.y) / dd);
    const double2 s1 = make_double2((acc1.x * pv.x + acc1.y * pv.y) / dd, (acc1.y * pv.x - acc1.x * pv.y) / dd);
    x0[r] = bcast(s0, r);
    x1[r] = bcast(s1, r);
  }
  if (valid && row) {
#pragma unroll
    for (int m = 0; m < NM; ++m)
      if (m == sl) {
        boost[(size_t)f * nm + m] = make_double2(-x0[m].x, -x0[m].y);
        if (refl) refl[(size_t)f * nm + m] = make_double2(-x1[m].x, -x1[m].y);
      }
  }
  if (valid && sl == 0 && beta2) {
    double s = 0.0;
#pragma unroll
    for (int m = 0; m < NM; ++m)
      if (m < nm) s += x0[m].x * x0[m].x + x0[m].y * x0[m].y;
    beta2[f] = s;
  }
}

// axion_induced_modes / field2modes: c_m = sum conj(Psi_m) B_hat
__global__ void k_project(double2* out, const double2* pat, const double2* Bn, int nm, int npix) {
  const int m = blockIdx.x;
  __shared__ double2 red[256];
  double2 acc = make_double2(0.0, 0.0);
  for (int x = threadIdx.x; x < npix; x += blockDim.x) {
    const double2 a = pat[(size_t)m * npix + x], b = Bn[x];
    acc.x += a.x * b.x + a.y * b.y;
    acc.y += a.x * b.y - a.y * b.x;
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      red[threadIdx.x].x += red[threadIdx.x + s].x;
      red[threadIdx.x].y += red[threadIdx.x + s].y;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) out[m] = red[0];
}

}  // namespace

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
namespace {

static std::atomic<unsigned long long> g_modes_id{0};

const cd* as_cdp(const double* p) { return reinterpret_cast<const cd*>(p); }

int modes_upload(bf_handle* h, bf_modes* m) {
  TCKS(bf_dalloc(h, (void**)&m->d_pat, sizeof(cd) * m->pat.size()));
  TCK(cudaMemcpyAsync(m->d_pat, m->pat.data(), sizeof(cd) * m->pat.size(), cudaMemcpyHostToDevice, h->stream()));
  TCK(cudaStreamSynchronize(h->stream()));
  return BF_OK;
}

unsigned blocks_for(size_t n) { return (unsigned)std::max<size_t>(1, (n + 255) / 256); }

}  // namespace

// Transformer setup cached per (stack, modes, precision): W, V and the orbit
// and support tables.
struct TfCache {
  unsigned long long modes_id = 0, geo_version = ~0ull;
  int mode = -1;   // operands built for: 0 FP64, 1 complex64 (SIMT GEMM), 2 TF32 pairs (tensor cores)
  int K = 0, msz = 0, Kd = 0, nm = 0;
  DBuf W, V, rep, supp, U, Phi, members;
  // complex64 path: upper triangle of V as real rows (k_build_vr), pair table;
  // W the same way (Wr, k_build_wr) when every mode vanishes outside the mask
  DBuf Vr, Wr, tri;
  int T = 0;
  bool herm_w = false;
  // tensor-core path: the real rows of both classes as TF32 hi/lo pairs [Mp][Kp],
  // [Mp][Kdp] (rows padded to a multiple of 128, K to a multiple of 32) and
  // their FP64 row sums (gW, gV)
  DBuf Wh, Wl, Vh, Vl, gW, gV;
  DBuf KT2;   // kx^2 + ky^2 at each orbit representative (FP32)
  int Kp = 0, Kdp = 0, Mp = 0;
  std::vector<int2> rep_h;
};

static void tf_cache_delete(void* p) { delete static_cast<TfCache*>(p); }
static size_t tf_cache_bytes(const void* p) {
  const TfCache* c = static_cast<const TfCache*>(p);
  size_t b = 0;
  for (const DBuf* d : {&c->W, &c->V, &c->Vr, &c->Wr, &c->tri, &c->rep, &c->supp, &c->U, &c->Phi, &c->members,
                        &c->Wh, &c->Wl, &c->Vh, &c->Vl, &c->gW, &c->gV, &c->KT2})
    b += d->p ? d->n : 0;
  return b;
}

static int tf_setup(bf_handle* h, bf_stack* s, bf_modes* md, int mode, TfCache** out) {
  const bool fp64 = mode == 0;
  if (!s->tf_cache) {
    s->tf_cache = new TfCache();
    s->tf_cache_delete = tf_cache_delete;
    s->tf_cache_bytes = tf_cache_bytes;
  }
  TfCache& c = *static_cast<TfCache*>(s->tf_cache);
  *out = &c;
  // W and V depend on the modes, the grid and the disk mask only, none of
  // which a stack changes after creation (bf_stack_set_distance moves the
  // disks), so gap updates of an optimiser reuse them.
  if (c.modes_id == md->id && c.mode == mode) return BF_OK;
  for (DBuf* d : {&c.W, &c.V, &c.Vr, &c.Wr, &c.tri, &c.Wh, &c.Wl, &c.Vh, &c.Vl, &c.gW, &c.gV, &c.KT2}) d->release();
  cudaStream_t st = h->stream();
  const int nx = s->nx, ny = s->ny, nm = md->nm;
  const size_t npix = (size_t)nx * ny;
  const size_t csz = fp64 ? 16 : 8;   // double2 or float2 operands
  c.nm = nm;
  // orbits of the phasor symmetry in shifted (kX, kY) index space
  auto antisym = [](const std::vector<double>& k) {
    const size_t n = k.size();
    double mx = 0;
    for (double v : k) mx = std::max(mx, fabs(v));
    for (size_t i = 0; i < n; ++i)
      if (fabs(k[i] + k[n - 1 - i]) > 1e-12 * std::max(1.0, mx)) return false;
    return true;
  };
  const bool fx = antisym(s->kX), fy = antisym(s->kY);
  bool swp = nx == ny;
  if (swp)
    for (int i = 0; i < nx; ++i)
      if (fabs(s->kX[i] - s->kY[i]) > 1e-12 * std::max(1.0, fabs(s->kX[i]))) { swp = false; break; }
  std::map<std::pair<int, int>, int> orbit_of;
  std::vector<std::vector<int>> mem;
  c.rep_h.clear();
  for (int ky = 0; ky < ny; ++ky)
    for (int kx = 0; kx < nx; ++kx) {
      const int sx = (kx + nx / 2) % nx, sy = (ky + ny / 2) % ny;   // fftshift position
      int a = fx ? std::min(sx, nx - 1 - sx) : sx;
      int b = fy ? std::min(sy, ny - 1 - sy) : sy;
      if (swp && b < a) std::swap(a, b);
      auto key = std::make_pair(a, b);
      auto it = orbit_of.find(key);
      int o;
      if (it == orbit_of.end()) {
        o = (int)mem.size();
        orbit_of[key] = o;
        mem.emplace_back();
        c.rep_h.push_back(make_int2(sx, sy));
      } else {
        o = it->second;
      }
      mem[o].push_back(ky * nx + kx);
    }
  c.K = (int)mem.size();
  c.msz = 1;
  for (auto& v : mem) c.msz = std::max<int>(c.msz, (int)v.size());
  std::vector<int> members((size_t)c.K * c.msz, -1);
  for (int o = 0; o < c.K; ++o)
    for (size_t q = 0; q < mem[o].size(); ++q) members[(size_t)o * c.msz + q] = mem[o][q];
  TCKS(c.members.alloc(h, sizeof(int) * members.size()));
  TCK(cudaMemcpyAsync(c.members.p, members.data(), sizeof(int) * members.size(), cudaMemcpyHostToDevice, st));
  TCKS(c.rep.alloc(h, sizeof(int2) * c.K));
  TCK(cudaMemcpyAsync(c.rep.p, c.rep_h.data(), sizeof(int2) * c.K, cudaMemcpyHostToDevice, st));
  // U = FFT(Psi), Phi = FFT(mask Psi), FP64
  TCKS(c.U.alloc(h, sizeof(double2) * nm * npix));
  TCKS(c.Phi.alloc(h, sizeof(double2) * nm * npix));
  TCK(cudaMemcpyAsync(c.U.p, md->d_pat, sizeof(double2) * nm * npix, cudaMemcpyDeviceToDevice, st));
  TCK(cudaMemcpyAsync(c.Phi.p, md->d_pat, sizeof(double2) * nm * npix, cudaMemcpyDeviceToDevice, st));
  int e = bf::launch_mul_mask(true, c.Phi.p, nm, nx, ny, s->d_mask_full, st);
  if (!e) e = bf::launch_line_dft(true, c.U.p, nm, nx, ny, 0, 0, st);
  if (!e) e = bf::launch_line_dft(true, c.U.p, nm, nx, ny, 1, 0, st);
  if (!e) e = bf::launch_line_dft(true, c.Phi.p, nm, nx, ny, 0, 0, st);
  if (!e) e = bf::launch_line_dft(true, c.Phi.p, nm, nx, ny, 1, 0, st);
  if (e) return bf_fail(h, BF_ERR_CUDA, "mode FFTs failed");
  c.Kp = (c.K + 31) / 32 * 32;
  if (!fp64) {
    // Phi = FFT(mask Psi) equals U = FFT(Psi) bit for bit when no mode has a
    // non-zero pixel outside the (0/1) mask; W is then Hermitian in the mode
    // pair, W[m'm] = conj W[mm'], and its upper triangle determines it.
    c.herm_w = true;
    for (int m = 0; m < nm && c.herm_w; ++m)
      for (size_t x = 0; x < npix; ++x)
        if (!s->mask_full[x] && md->pat[(size_t)m * npix + x] != cd(0.0, 0.0)) {
          c.herm_w = false;
          break;
        }
    std::vector<int2> tri;
    for (int m = 0; m < nm; ++m)
      for (int mp = m; mp < nm; ++mp) tri.push_back(make_int2(m, mp));
    c.T = (int)tri.size();
    c.Mp = (2 * c.T + 127) / 128 * 128;
    TCKS(c.tri.alloc(h, sizeof(int2) * tri.size()));
    TCK(cudaMemcpyAsync(c.tri.p, tri.data(), sizeof(int2) * tri.size(), cudaMemcpyHostToDevice, st));
  }
  DBuf Ad;   // FP64 real rows of the tensor-core path, for the row sums
  {
    dim3 grid(blocks_for(c.K), nm * nm);
    const double scale = 1.0 / ((double)nx * (double)ny);
    bf::note_launch();
    if (fp64) {
      TCKS(c.W.alloc(h, csz * (size_t)nm * nm * c.K));
      k_build_w<double2><<<grid, 256, 0, st>>>(c.W.as<double2>(), c.U.as<double2>(), c.Phi.as<double2>(),
                                               c.members.as<int>(), c.K, c.msz, nm, (int)npix, scale);
    } else if (mode == 2 && c.herm_w) {
      const size_t n = (size_t)c.Mp * c.Kp;
      TCKS(c.Wh.alloc(h, sizeof(float) * n));
      TCKS(c.Wl.alloc(h, sizeof(float) * n));
      TCK(cudaMemsetAsync(c.Wh.p, 0, sizeof(float) * n, st));
      TCK(cudaMemsetAsync(c.Wl.p, 0, sizeof(float) * n, st));
      TCKS(Ad.alloc(h, sizeof(double) * 2 * (size_t)c.T * c.K));
      k_build_wr_tc<<<dim3(blocks_for(c.Kp), c.T), 256, 0, st>>>(
          c.Wh.as<float>(), c.Wl.as<float>(), Ad.as<double>(), c.U.as<double2>(), c.Phi.as<double2>(),
          c.members.as<int>(), c.tri.as<int2>(), c.K, c.Kp, c.msz, (int)npix, scale);
      TCK(cudaGetLastError());
      TCKS(c.gW.alloc(h, sizeof(double) * c.Mp));
      TCK(cudaMemsetAsync(c.gW.p, 0, sizeof(double) * c.Mp, st));
      bf::note_launch();
      k_rowsum<<<2 * c.T, 256, 0, st>>>(c.gW.as<double>(), Ad.as<double>(), c.K);
      std::vector<float> kt2(c.K);
      for (int o = 0; o < c.K; ++o) {
        const double kx = s->kX[c.rep_h[o].x], ky = s->kY[c.rep_h[o].y];
        kt2[o] = (float)(kx * kx + ky * ky);
      }
      TCKS(c.KT2.alloc(h, sizeof(float) * c.K));
      TCK(cudaMemcpyAsync(c.KT2.p, kt2.data(), sizeof(float) * c.K, cudaMemcpyHostToDevice, st));
      TCK(cudaStreamSynchronize(st));   // kt2 is a local host array
    } else if (c.herm_w) {
      TCKS(c.Wr.alloc(h, sizeof(float) * 2 * (size_t)c.T * c.K));
      k_build_wr<<<dim3(blocks_for(c.K), c.T), 256, 0, st>>>(c.Wr.as<float>(), c.U.as<double2>(),
                                                              c.Phi.as<double2>(), c.members.as<int>(),
                                                              c.tri.as<int2>(), c.K, c.msz, (int)npix, scale);
    } else {
      // modes reaching beyond the mask (W not Hermitian): complex64 W for the
      // SIMT GEMM (also on the tensor-core path)
      TCKS(c.W.alloc(h, csz * (size_t)nm * nm * c.K));
      k_build_w<float2><<<grid, 256, 0, st>>>(c.W.as<float2>(), c.U.as<double2>(), c.Phi.as<double2>(),
                                              c.members.as<int>(), c.K, c.msz, nm, (int)npix, scale);
    }
    TCK(cudaGetLastError());
  }
  // support pixels (any mode non-zero) and V
  std::vector<int> supp;
  for (size_t x = 0; x < npix; ++x) {
    bool nz = false;
    for (int m = 0; m < nm && !nz; ++m) nz = md->pat[(size_t)m * npix + x] != cd(0.0, 0.0);
    if (nz) supp.push_back((int)x);
  }
  if (supp.empty()) supp.push_back(0);
  c.Kd = (int)supp.size();
  TCKS(c.supp.alloc(h, sizeof(int) * supp.size()));
  TCK(cudaMemcpyAsync(c.supp.p, supp.data(), sizeof(int) * supp.size(), cudaMemcpyHostToDevice, st));
  c.Kdp = (c.Kd + 31) / 32 * 32;
  {
    dim3 grid(blocks_for(c.Kd), nm * nm);
    bf::note_launch();
    if (fp64) {
      TCKS(c.V.alloc(h, csz * (size_t)nm * nm * c.Kd));
      k_build_v<double2><<<grid, 256, 0, st>>>(c.V.as<double2>(), md->d_pat, c.supp.as<int>(), c.Kd, nm,
                                               (int)npix);
    } else if (mode == 1) {
      TCKS(c.Vr.alloc(h, sizeof(float) * 2 * (size_t)c.T * c.Kd));
      k_build_vr<<<dim3(blocks_for(c.Kd), c.T), 256, 0, st>>>(c.Vr.as<float>(), md->d_pat, c.supp.as<int>(),
                                                               c.tri.as<int2>(), c.Kd, (int)npix);
    } else {
      const size_t n = (size_t)c.Mp * c.Kdp;
      TCKS(c.Vh.alloc(h, sizeof(float) * n));
      TCKS(c.Vl.alloc(h, sizeof(float) * n));
      TCK(cudaMemsetAsync(c.Vh.p, 0, sizeof(float) * n, st));
      TCK(cudaMemsetAsync(c.Vl.p, 0, sizeof(float) * n, st));
      DBuf Vd;
      TCKS(Vd.alloc(h, sizeof(double) * 2 * (size_t)c.T * c.Kd));
      k_build_vr_tc<<<dim3(blocks_for(c.Kdp), c.T), 256, 0, st>>>(c.Vh.as<float>(), c.Vl.as<float>(), Vd.as<double>(),
                                                                  md->d_pat, c.supp.as<int>(), c.tri.as<int2>(),
                                                                  c.Kd, c.Kdp, (int)npix);
      TCK(cudaGetLastError());
      TCKS(c.gV.alloc(h, sizeof(double) * c.Mp));
      TCK(cudaMemsetAsync(c.gV.p, 0, sizeof(double) * c.Mp, st));
      bf::note_launch();
      k_rowsum<<<2 * c.T, 256, 0, st>>>(c.gV.as<double>(), Vd.as<double>(), c.Kd);
    }
    TCK(cudaGetLastError());
  }
  TCK(cudaStreamSynchronize(st));
  c.U.release();
  c.Phi.release();
  c.modes_id = md->id;
  c.geo_version = s->geo_version;
  c.mode = mode;
  return BF_OK;
}

static thread_local double g_tf_gemm_flops = 0.0;   // executed real flops of the class GEMMs of this thread's last solve
// CUDA events around each class-GEMM kernel of this thread's solve (profiling only)
static thread_local std::vector<std::pair<cudaEvent_t, cudaEvent_t>> g_gemm_ev;
static void gemm_ev_begin(bf_handle* h) {
  if (!h->profiling) return;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  cudaEventRecord(a, h->stream());
  g_gemm_ev.emplace_back(a, b);
}
static void gemm_ev_end(bf_handle* h) {
  if (!h->profiling || g_gemm_ev.empty()) return;
  cudaEventRecord(g_gemm_ev.back().second, h->stream());
}
// Sum of the recorded GEMM kernel times (after the stream has synchronised).
static double gemm_ev_collect() {
  double ms = 0.0;
  for (auto& e : g_gemm_ev) {
    float t = 0.f;
    if (cudaEventElapsedTime(&t, e.first, e.second) == cudaSuccess) ms += t;
    cudaEventDestroy(e.first);
    cudaEventDestroy(e.second);
  }
  g_gemm_ev.clear();
  cudaGetLastError();
  return ms;
}

static void tf_mark(bf_handle* h, int i) {
  if (!h->profiling) return;
  if (!h->ev[i]) cudaEventCreate(&h->ev[i]);
  cudaEventRecord(h->ev[i], h->stream());
}

// Class GEMM G = A * B with FP64 output: FP64 operands (FP64 path), or
// complex64 operands with chunked double-float accumulation (mixed path).
template <typename S>
static int launch_gemm(bf_handle* h, const S* A, const S* B, double2* Cm, int R, int K, int N) {
  g_tf_gemm_flops += 8.0 * (double)R * (double)K * (double)N;
  dim3 grid((N + 63) / 64, (R + 63) / 64);
  bf::note_launch();
  gemm_ev_begin(h);
  if constexpr (std::is_same<S, double2>::value) {
    bf::k_cgemm<double2><<<grid, 256, 0, h->stream()>>>(A, B, Cm, R, K, N);
  } else {
    // split K when the output tiles alone would leave SMs idle (few modes)
    const long tiles = (long)grid.x * grid.y;
    int splits = 1;
    while (splits < 16 && tiles * splits < 2 * 152 && K / (splits * 2) >= 256) splits *= 2;
    if (splits == 1) {
      bf::k_cgemm_c64<<<grid, 256, 0, h->stream()>>>(A, B, Cm, R, K, N, K);
    } else {
      const int kchunk = ((K + splits - 1) / splits + 15) / 16 * 16;
      DBuf part;
      TCKS(part.alloc(h, sizeof(double2) * (size_t)splits * R * N));
      grid.z = splits;
      bf::k_cgemm_c64<<<grid, 256, 0, h->stream()>>>(A, B, part.as<double2>(), R, K, N, kchunk);
      TCK(cudaGetLastError());
      const size_t n = (size_t)R * N;
      bf::note_launch();
      bf::k_sum_planes<<<blocks_for(n), 256, 0, h->stream()>>>(Cm, part.as<double2>(), n, splits);
    }
  }
  gemm_ev_end(h);
  TCK(cudaGetLastError());
  return BF_OK;
}

// Real-row class GEMM H = A * B (A real FP32 [R][K], B complex64 [K][N],
// H complex128 [R][N]) with the split-K rule of launch_gemm.
static int launch_rgemm(bf_handle* h, const float* A, const float2* B, double2* Hm, int R, int K, int N) {
  g_tf_gemm_flops += 4.0 * (double)R * (double)K * (double)N;
  dim3 grid((N + 31) / 32, (R + 127) / 128);
  const long tiles = (long)grid.x * grid.y;
  int splits = 1;
  while (splits < 16 && tiles * splits < 2 * 152 && K / (splits * 2) >= 256) splits *= 2;
  bf::note_launch();
  gemm_ev_begin(h);
  if (splits == 1) {
    bf::k_rcgemm_c64<8><<<grid, 256, 0, h->stream()>>>(A, B, Hm, R, K, N, K);
  } else {
    const int kchunk = ((K + splits - 1) / splits + 15) / 16 * 16;
    DBuf part;
    TCKS(part.alloc(h, sizeof(double2) * (size_t)splits * R * N));
    grid.z = splits;
    bf::k_rcgemm_c64<8><<<grid, 256, 0, h->stream()>>>(A, B, part.as<double2>(), R, K, N, kchunk);
    TCK(cudaGetLastError());
    const size_t n = (size_t)R * N;
    bf::note_launch();
    bf::k_sum_planes<<<blocks_for(n), 256, 0, h->stream()>>>(Hm, part.as<double2>(), n, splits);
  }
  gemm_ev_end(h);
  TCK(cudaGetLastError());
  return BF_OK;
}

// Class GEMM of the TF32 path on the tensor cores: out[splits][2 ncol][Mp]
// (FP32) = A [Mp][Kp] times the 2 ncol real rows of B^T [2 ncol][Kp] (TF32
// hi/lo pairs), K cut into slices only when the output tiles alone would
// leave SMs idle; k_scatter_herm_tc sums the slices in FP64.
// The K slicing of the tensor-core GEMM, per (device, M, N rounded up to a
// power of two, K): the heuristic's count, or, with the autotuner on, the
// fastest of 1, 2, 4, 8 slices timed once on the first call's operands (the
// output of the trials is scratch; every count gives the same sums up to FP32
// rounding of the slices).  Products whose output tiles already fill the GPU
// keep one slice untimed, so that group solves of varying size (a new N each)
// trigger no trials while serving.
static std::mutex g_split_mu;
static std::map<std::array<long long, 4>, int> g_split_tuned;

static int tc_pick_splits(bf_handle* h, const float* Ah, const float* Al, int Mp, int Kp, const float* Bh,
                          const float* Bl, int nrows_b, int* d_err, int* splits) {
  cudaStream_t st = h->stream();
  *splits = bf::tc_gemm_splits(Mp, nrows_b, Kp);
  if (!bf_autotune_enabled() || bf::tc_gemm_fills_gpu(Mp, nrows_b)) return BF_OK;
  long long nb = 1;
  while (nb < nrows_b) nb <<= 1;
  const std::array<long long, 4> key = {h->device, Mp, nb, Kp};
  {
    std::lock_guard<std::mutex> lock(g_split_mu);
    auto it = g_split_tuned.find(key);
    if (it != g_split_tuned.end()) {
      *splits = it->second;
      return BF_OK;
    }
  }
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  TCK(cudaStreamIsCapturing(st, &cap));
  if (cap != cudaStreamCaptureStatusNone) return BF_OK;
  const int ktiles = Kp / 32;
  std::vector<int> cand;
  for (int sp : {1, 2, 4, 8})
    if (sp == 1 || ktiles / sp >= 8) cand.push_back(sp);
  int best = *splits;
  std::string what;
  if (cand.size() > 1) {
    DBuf tmp;
    TCKS(tmp.alloc(h, sizeof(float) * (size_t)cand.back() * nrows_b * Mp));
    cudaEvent_t e0, e1;
    TCK(cudaEventCreate(&e0));
    TCK(cudaEventCreate(&e1));
    float tbest = 1e30f;
    for (int sp : cand) {
      float tv = 1e30f;
      for (int rep = 0; rep < 3; ++rep) {   // the first run warms up
        cudaEventRecord(e0, st);
        const int e = bf::tc_gemm_tf32x3(Ah, Al, Bh, Bl, Mp, nrows_b, Kp, sp, tmp.as<float>(), d_err, st, h->sm_cap);
        cudaEventRecord(e1, st);
        if (e || cudaEventSynchronize(e1) != cudaSuccess) {
          tv = 1e30f;
          break;
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0) tv = std::min(tv, ms);
      }
      what += " " + std::to_string(sp) + ":" + std::to_string(tv);
      if (tv < tbest) {
        tbest = tv;
        best = sp;
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaGetLastError();
  }
  {
    std::lock_guard<std::mutex> lock(g_split_mu);
    g_split_tuned[key] = best;
  }
  bf_tune_log("tc_gemm M=" + std::to_string(Mp) + " N=" + std::to_string(nrows_b) + " K=" + std::to_string(Kp) +
              " -> " + std::to_string(best) + " K slices (ms per launch by slices:" + what + ")");
  *splits = best;
  return BF_OK;
}

static int tc_class_gemm(bf_handle* h, const float* Ah, const float* Al, int Mp, int Kp, const float* Bh,
                         const float* Bl, int nrows_b, DBuf& out, int* splits, int* d_err) {
  cudaStream_t st = h->stream();
  g_tf_gemm_flops += 3.0 * 2.0 * (double)Mp * (double)Kp * (double)nrows_b;   // executed TF32 MMA work
  TCKS(tc_pick_splits(h, Ah, Al, Mp, Kp, Bh, Bl, nrows_b, d_err, splits));
  TCKS(out.alloc(h, sizeof(float) * (size_t)*splits * nrows_b * Mp));
  gemm_ev_begin(h);
  const int e = bf::tc_gemm_tf32x3(Ah, Al, Bh, Bl, Mp, nrows_b, Kp, *splits, out.as<float>(), d_err, st, h->sm_cap);
  gemm_ev_end(h);
  if (e) return bf_fail(h, BF_ERR_CUDA, std::string("tensor-core GEMM: ") + cudaGetErrorString((cudaError_t)e));
  return BF_OK;
}

// Propagation matrices of regions [j0, nd) for all frequencies into
// P[f][j][m][m'] stored as S, which is also the operand storage of the class
// GEMMs: double2 (FP64 path) or float2 (mixed path).  A group solve (nreq > 1)
// passes the regions of nreq requests (regs[r nd + j]) that differ only in the
// distances of their k-space (air) regions: P then holds nreq nf frequencies
// (request r at r nf + f), the k-space class runs nreq nf npar columns, and the
// pixel class (disks, identical across the group) runs once and is written
// for every request.
template <typename S>
static int tf_propagation_matrices(bf_handle* h, bf_stack* s, bf_modes* md, TfCache& c,
                                   const std::vector<RegionT>& regs, int j0, int nf,
                                   const std::vector<double>& freqs, int prop_kind, DBuf& P, int mode,
                                   int nreq = 1) {
  using C = double2;
  cudaStream_t st = h->stream();
  const int nd = s->nd, nm = md->nm, nx = s->nx, ny = s->ny;
  const size_t npix = (size_t)nx * ny;
  std::vector<int> kreg, preg, freg;
  for (int j = j0; j < nd; ++j) {
    if (regs[j].klass == 0) kreg.push_back(j);
    else if (regs[j].klass == 3) freg.push_back(j);
    else preg.push_back(j);
  }
  int* tc_err = reinterpret_cast<int*>(h->d_scalar + 2);   // set by the tensor-core GEMM on a wait timeout
  if (mode == 2) TCK(cudaMemsetAsync(tc_err, 0, sizeof(int), st));
  if (nreq > 1 && !freg.empty()) return bf_fail(h, BF_ERR_UNSUPPORTED, "group solve with tilted air regions");
  TCKS(P.ensure(h, sizeof(S) * (size_t)nreq * nf * nd * nm * nm));
  DBuf d_regs, d_freq, d_kt, d_list;
  TCKS(d_regs.alloc(h, sizeof(RegionT) * regs.size()));
  TCK(cudaMemcpyAsync(d_regs.p, regs.data(), sizeof(RegionT) * regs.size(), cudaMemcpyHostToDevice, st));
  TCKS(d_freq.alloc(h, sizeof(double) * nf));
  TCK(cudaMemcpyAsync(d_freq.p, freqs.data(), sizeof(double) * nf, cudaMemcpyHostToDevice, st));
  TCKS(d_kt.alloc(h, sizeof(cd) * nm));
  TCK(cudaMemcpyAsync(d_kt.p, md->kt.data(), sizeof(cd) * nm, cudaMemcpyHostToDevice, st));
  const RegionT* dr = d_regs.as<RegionT>();
  // k-space class: one GEMM W * D
  if (!kreg.empty()) {
    const int npar = (int)kreg.size();
    DBuf lst, D, G;
    TCKS(lst.alloc(h, sizeof(int) * npar));
    TCK(cudaMemcpyAsync(lst.p, kreg.data(), sizeof(int) * npar, cudaMemcpyHostToDevice, st));
    const int ncol = nreq * nf * npar;
    // distinct permittivities of the k-space regions (normally one: air)
    std::vector<double2> eps_list;
    std::vector<int> par_eps(npar);
    for (int p = 0; p < npar; ++p) {
      const RegionT& g = regs[kreg[p]];
      int e = 0;
      while (e < (int)eps_list.size() && !(eps_list[e].x == g.er && eps_list[e].y == g.ei)) ++e;
      if (e == (int)eps_list.size()) eps_list.push_back(make_double2(g.er, g.ei));
      par_eps[p] = e;
    }
    const int neps = (int)eps_list.size();
    DBuf d_eps, d_peps, KZ;
    TCKS(d_eps.alloc(h, sizeof(double2) * neps));
    TCK(cudaMemcpyAsync(d_eps.p, eps_list.data(), sizeof(double2) * neps, cudaMemcpyHostToDevice, st));
    TCKS(d_peps.alloc(h, sizeof(int) * npar));
    TCK(cudaMemcpyAsync(d_peps.p, par_eps.data(), sizeof(int) * npar, cudaMemcpyHostToDevice, st));
    const bool herm = mode == 1 && c.herm_w;   // real rows of W's upper triangle
    const bool tc = mode == 2 && c.herm_w;     // the same rows on the tensor cores
    if (!tc) {
      TCKS(G.alloc(h, sizeof(C) * (size_t)(herm ? 2 * c.T : nm * nm) * ncol));
      TCKS(KZ.alloc(h, sizeof(double2) * (size_t)neps * c.K * nf));
      bf::note_launch();
      k_build_kz<<<dim3(blocks_for(c.K), std::min(nf, 65535), neps), 256, 0, st>>>(
          KZ.as<double2>(), c.rep.as<int2>(), c.K, d_freq.as<double>(), nf, d_eps.as<double2>(), s->dkX, s->dkY);
      TCK(cudaGetLastError());
    }
    if (!tc) {
      TCKS(D.alloc(h, sizeof(S) * (size_t)c.K * ncol));
      bf::note_launch();
      k_build_d<S><<<dim3(blocks_for(ncol), std::min(c.K, 65535)), 256, 0, st>>>(
          D.as<S>(), KZ.as<double2>(), c.K, nf, ncol, nd, dr, lst.as<int>(), d_peps.as<int>(), npar);
      TCK(cudaGetLastError());
      if (herm) {
        if constexpr (std::is_same<S, float2>::value)
          TCKS(launch_rgemm(h, c.Wr.as<float>(), D.as<float2>(), G.as<C>(), 2 * c.T, c.K, ncol));
      } else {
        TCKS(launch_gemm<S>(h, c.W.as<S>(), D.as<S>(), G.as<C>(), nm * nm, c.K, ncol));
      }
    } else {
      DBuf C0, col, Bh, Bl, out;
      TCKS(C0.alloc(h, sizeof(double2) * ncol));
      TCKS(col.alloc(h, sizeof(ColTC) * ncol));
      bf::note_launch();
      k_build_c0<<<blocks_for(ncol), 256, 0, st>>>(C0.as<double2>(), col.as<ColTC>(), d_freq.as<double>(), nf,
                                                   ncol, nd, d_eps.as<double2>(), dr, lst.as<int>(),
                                                   d_peps.as<int>(), npar);
      TCK(cudaGetLastError());
      DBuf DKZ;
      TCKS(DKZ.alloc(h, sizeof(float2) * (size_t)neps * nf * c.K));
      bf::note_launch();
      k_build_dkz<<<dim3(blocks_for(c.K), std::min(nf, 65535), neps), 256, 0, st>>>(
          DKZ.as<float2>(), c.KT2.as<float>(), c.K, d_freq.as<double>(), nf, d_eps.as<double2>());
      TCK(cudaGetLastError());
      const size_t nb = (size_t)2 * ncol * c.Kp;
      TCKS(Bh.alloc(h, sizeof(float) * nb));
      TCKS(Bl.alloc(h, sizeof(float) * nb));
      bf::note_launch();
      k_build_d_tc<<<dim3(blocks_for(c.Kp), std::min(ncol, 65535)), 256, 0, st>>>(
          Bh.as<float>(), Bl.as<float>(), DKZ.as<float2>(), col.as<ColTC>(), c.K, c.Kp, ncol);
      TCK(cudaGetLastError());
      int splits = 1;
      TCKS(tc_class_gemm(h, c.Wh.as<float>(), c.Wl.as<float>(), c.Mp, c.Kp, Bh.as<float>(), Bl.as<float>(),
                         2 * ncol, out, &splits, tc_err));
      bf::note_launch();
      const unsigned gs = (unsigned)std::min<size_t>(blocks_for((size_t)ncol * c.T), 1u << 20);
      k_scatter_herm_tc<S><<<gs, 256, 0, st>>>(P.as<S>(), out.as<float>(), c.Mp, splits, C0.as<double2>(),
                                               c.gW.as<double>(), nreq * nf, npar, dr, lst.as<int>(), nd, nm,
                                               nullptr, c.tri.as<int2>(), c.T, 1);
      TCK(cudaGetLastError());
    }
    if (!tc) {
      bf::note_launch();
      if (herm) {
        dim3 gs(blocks_for(c.T), std::min(ncol, 65535));
        k_scatter_herm<S><<<gs, 256, 0, st>>>(P.as<S>(), G.as<C>(), nreq * nf, npar, dr, lst.as<int>(), nd, nm,
                                              nullptr, c.tri.as<int2>(), c.T, 1);
      } else {
        dim3 gs(blocks_for((size_t)nm * nm), std::min(ncol, 65535));
        k_scatter_p<S><<<gs, 256, 0, st>>>(P.as<S>(), G.as<C>(), nreq * nf, npar, dr, lst.as<int>(), nd, nm, nullptr,
                                           1);
      }
      TCK(cudaGetLastError());
    }
  }
  // pixel class: one GEMM V * E
  if (!preg.empty()) {
    const int npx = (int)preg.size();
    DBuf lst, E, G;
    TCKS(lst.alloc(h, sizeof(int) * npx));
    TCK(cudaMemcpyAsync(lst.p, preg.data(), sizeof(int) * npx, cudaMemcpyHostToDevice, st));
    const int ncol = nf * npx;
    const int grows = mode == 1 ? 2 * c.T : nm * nm;   // mode 1: real rows of the upper triangle
    if (mode != 2) TCKS(G.alloc(h, sizeof(C) * (size_t)grows * ncol));
    DBuf K0, DG;
    TCKS(K0.alloc(h, sizeof(double2) * (size_t)ncol));
    TCKS(DG.alloc(h, sizeof(double2) * (size_t)ncol * nm));
    bf::note_launch();
    k_build_k0<<<blocks_for(ncol), 256, 0, st>>>(K0.as<double2>(), d_freq.as<double>(), nf, dr, lst.as<int>(), npx);
    TCK(cudaGetLastError());
    bf::note_launch();
    k_build_diag<<<blocks_for((size_t)ncol * nm), 256, 0, st>>>(DG.as<double2>(), K0.as<double2>(), nf, npx, dr,
                                                               lst.as<int>(), d_kt.as<double2>(), nm);
    TCK(cudaGetLastError());
    if (mode != 2) {
      TCKS(E.alloc(h, sizeof(S) * (size_t)c.Kd * ncol));
      bf::note_launch();
      k_build_e<S><<<dim3(blocks_for(ncol), std::min(c.Kd, 65535)), 256, 0, st>>>(
          E.as<S>(), c.supp.as<int>(), c.Kd, nf, dr, lst.as<int>(), npx, K0.as<double2>(), s->dX, s->dY, nx,
          s->d_surf, (int)npix);
      TCK(cudaGetLastError());
      if constexpr (std::is_same<S, float2>::value)
        TCKS(launch_rgemm(h, c.Vr.as<float>(), E.as<float2>(), G.as<C>(), 2 * c.T, c.Kd, ncol));
      else
        TCKS(launch_gemm<S>(h, c.V.as<S>(), E.as<S>(), G.as<C>(), nm * nm, c.Kd, ncol));
    } else {
      DBuf Bh, Bl, out;
      const size_t nb = (size_t)2 * ncol * c.Kdp;
      TCKS(Bh.alloc(h, sizeof(float) * nb));
      TCKS(Bl.alloc(h, sizeof(float) * nb));
      bf::note_launch();
      k_build_e_tc<<<dim3(blocks_for(c.Kdp), std::min(ncol, 65535)), 256, 0, st>>>(
          Bh.as<float>(), Bl.as<float>(), c.supp.as<int>(), c.Kd, c.Kdp, nf, dr, lst.as<int>(), npx,
          K0.as<double2>(), s->dX, s->dY, nx, s->d_surf, (int)npix);
      TCK(cudaGetLastError());
      int splits = 1;
      TCKS(tc_class_gemm(h, c.Vh.as<float>(), c.Vl.as<float>(), c.Mp, c.Kdp, Bh.as<float>(), Bl.as<float>(),
                         2 * ncol, out, &splits, tc_err));
      bf::note_launch();
      const unsigned gs = (unsigned)std::min<size_t>(blocks_for((size_t)ncol * c.T), 1u << 20);
      k_scatter_herm_tc<S><<<gs, 256, 0, st>>>(P.as<S>(), out.as<float>(), c.Mp, splits, nullptr, c.gV.as<double>(),
                                               nf, npx, dr, lst.as<int>(), nd, nm, DG.as<double2>(),
                                               c.tri.as<int2>(), c.T, nreq);
      TCK(cudaGetLastError());
    }
    if (mode != 2) {
      bf::note_launch();
      if (mode == 1) {
        dim3 gs(blocks_for(c.T), std::min(ncol, 65535));
        k_scatter_herm<S><<<gs, 256, 0, st>>>(P.as<S>(), G.as<C>(), nf, npx, dr, lst.as<int>(), nd, nm,
                                              DG.as<double2>(), c.tri.as<int2>(), c.T, nreq);
      } else {
        dim3 gs(blocks_for((size_t)nm * nm), std::min(ncol, 65535));
        k_scatter_p<S><<<gs, 256, 0, st>>>(P.as<S>(), G.as<C>(), nf, npx, dr, lst.as<int>(), nd, nm,
                                           DG.as<double2>(), nreq);
      }
      TCK(cudaGetLastError());
    }
  }
  // field class: propagate every mode (FP64), then overlap
  if (!freg.empty()) {
    DBuf Q, tmp, fr;
    TCKS(Q.alloc(h, sizeof(C) * (size_t)nm * npix));
    TCKS(tmp.alloc(h, sizeof(C) * (size_t)nm * npix));
    TCKS(fr.alloc(h, sizeof(double) * nm));
    const int kind = prop_kind == BF_PROP_NOTILTS ? BF_PROP_NOTILTS : prop_kind;
    for (int f = 0; f < nf; ++f) {
      std::vector<double> fv(nm, freqs[f]);
      TCK(cudaMemcpyAsync(fr.p, fv.data(), sizeof(double) * nm, cudaMemcpyHostToDevice, st));
      for (int j : freg) {
        bf::note_launch();
        k_copy_modes<C><<<blocks_for((size_t)nm * npix), 256, 0, st>>>(Q.as<C>(), md->d_pat, nm, (int)npix, 1);
        TCK(cudaGetLastError());
        TCKS(bf_general_prop(h, s, kind, true, Q.p, tmp.p, nm, fr.as<double>(), j));
        bf::note_launch();
        k_overlap<S, C><<<nm * nm, 256, 0, st>>>(P.as<S>() + (((size_t)f * nd + j) * nm) * nm, md->d_pat, Q.as<C>(), nm,
                                              (int)npix);
        TCK(cudaGetLastError());
      }
    }
  }
  return BF_OK;
}

static int classify(bf_handle* h, const bf_stack* s, int prop_kind, const std::vector<cd>& eps,
                    std::vector<RegionT>& regs) {
  const int nd = s->nd;
  regs.resize(nd);
  for (int j = 0; j < nd; ++j) {
    RegionT& r = regs[j];
    r.dz = s->distance[j];
    r.er = eps[j].real();
    r.ei = eps[j].imag();
    r.tx = s->tilt_x[j];
    r.ty = s->tilt_y[j];
    const bool air = eps[j].real() == 1.0;   // is_air = real(eps) == 1 (transformer.jl:174)
    const bool flat = (r.tx == 0.0 && r.ty == 0.0 && !(s->d_surf && s->surf_nonzero[j])) || prop_kind == BF_PROP_NOTILTS;
    if (!air) r.klass = 1;
    else if (prop_kind == BF_PROP_1D) r.klass = 2;
    else if ((prop_kind == BF_PROP_3D || prop_kind == BF_PROP_NOTILTS) && flat) r.klass = 0;
    else r.klass = 3;
    r.col = 0;
  }
  (void)h;
  return BF_OK;
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" int bf_modes_create(bf_handle* h, int nx, int ny, const double* X, const double* Y, int three_dim,
                               int M, int L, double diskR, const double* pattern_input, const double* kT,
                               bf_modes** out) {
  if (!h || !out) return BF_ERR_INVALID;
  *out = nullptr;
  if (nx < 1 || ny < 1 || !X || !Y) return bf_fail(h, BF_ERR_INVALID, "empty grid");
  std::unique_ptr<bf_modes> m(new bf_modes());
  m->nx = nx; m->ny = ny;
  m->X.assign(X, X + nx);
  m->Y.assign(Y, Y + ny);
  const size_t npix = (size_t)nx * ny;
  if (!three_dim) {
    // SeedModes(ThreeDim=false): one mode of ones, kt = 0 (transformer.jl:58-63)
    m->M = 1; m->L = 0; m->nm = 1;
    m->pat.assign(npix, cd(1.0, 0.0));
    m->kt.assign(1, cd(0.0, 0.0));
  } else {
    if (M < 1 || L < 0) return bf_fail(h, BF_ERR_INVALID, "Mmax >= 1 and Lmax >= 0 required");
    m->M = M; m->L = L; m->nm = M * (2 * L + 1);
    if (pattern_input) {
      // pattern_input (M, 2L+1, nx, ny, 1) column-major, kT (M, 2L+1)
      if (!kT) return bf_fail(h, BF_ERR_INVALID, "you have to define kTs as well when putting in an input pattern");
      const int nl = 2 * L + 1;
      m->pat.assign((size_t)m->nm * npix, cd(0, 0));
      m->kt.assign(m->nm, cd(0, 0));
      const cd* pi = as_cdp(pattern_input);
      const cd* kt = as_cdp(kT);
      for (int mm = 0; mm < M; ++mm)
        for (int l = 0; l < nl; ++l) {
          const int k = mm * nl + l;
          m->kt[k] = kt[mm + (size_t)M * l];
          for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x)
              m->pat[(size_t)k * npix + (size_t)y * nx + x] =
                  pi[mm + (size_t)M * (l + (size_t)nl * (x + (size_t)nx * y))];
        }
    } else {
      std::vector<double> Xv(X, X + nx), Yv(Y, Y + ny);
      bfmodes::seed_modes(M, L, Xv, Yv, diskR, m->pat, m->kt);
    }
  }
  if (m->nm > 64) return bf_fail(h, BF_ERR_UNSUPPORTED, "at most 64 modes are supported");
  TCK(cudaSetDevice(h->device));
  TCKS(modes_upload(h, m.get()));
  m->id = ++g_modes_id;
  *out = m.release();
  return BF_OK;
}

extern "C" int bf_modes_destroy(bf_handle* h, bf_modes* m) {
  if (!h || !m) return BF_ERR_INVALID;
  if (m->server_uses.load() > 0)
    return bf_fail(h, BF_ERR_INVALID, "mode basis is in use by a serving engine: destroy the server first");
  cudaStreamSynchronize(h->stream());
  bf_dfree(h, m->d_pat);
  delete m;
  return BF_OK;
}

extern "C" int bf_modes_get(bf_handle* h, const bf_modes* m, int* nm_out, double* patterns, double* kt) {
  if (!h || !m) return BF_ERR_INVALID;
  if (nm_out) *nm_out = m->nm;
  const size_t npix = (size_t)m->nx * m->ny;
  const int nl = 2 * m->L + 1;
  if (patterns) {
    // (M, 2L+1, nx, ny, 1) column-major
    cd* o = reinterpret_cast<cd*>(patterns);
    for (int mm = 0; mm < m->M; ++mm)
      for (int l = 0; l < nl; ++l)
        for (int y = 0; y < m->ny; ++y)
          for (int x = 0; x < m->nx; ++x)
            o[mm + (size_t)m->M * (l + (size_t)nl * (x + (size_t)m->nx * y))] =
                m->pat[(size_t)(mm * nl + l) * npix + (size_t)y * m->nx + x];
  }
  if (kt) {
    cd* o = reinterpret_cast<cd*>(kt);
    for (int mm = 0; mm < m->M; ++mm)
      for (int l = 0; l < nl; ++l) o[mm + (size_t)m->M * l] = m->kt[mm * nl + l];
  }
  return BF_OK;
}

extern "C" int bf_axion_induced_modes(bf_handle* h, const bf_modes* m, const double* B, double velocity_x,
                                      double diskR, double f, double* out) {
  if (!h || !m || !out) return BF_ERR_INVALID;
  const double* X = m->X.data();
  const double* Y = m->Y.data();
  TCK(cudaSetDevice(h->device));
  const int nx = m->nx, ny = m->ny;
  const size_t npix = (size_t)nx * ny;
  std::vector<cd> b(npix, cd(1.0, 0.0));
  if (B) b.assign(as_cdp(B), as_cdp(B) + npix);
  if (velocity_x != 0.0) {
    const double ma = 2.0 * M_PI / (kC / f);
    for (int y = 0; y < ny; ++y)
      for (int x = 0; x < nx; ++x) {
        const double a = -ma * (-velocity_x) * X[x];
        b[(size_t)y * nx + x] *= cd(std::cos(a), std::sin(a));
      }
  }
  double n2 = 0.0;
  for (int y = 0; y < ny; ++y)
    for (int x = 0; x < nx; ++x) {
      const double xx = X[x] * X[x];
      const double yy = Y[y] * Y[y];
      if (!(std::sqrt(xx + yy) <= diskR)) b[(size_t)y * nx + x] = 0.0;
      n2 += std::norm(b[(size_t)y * nx + x]);
    }
  const double nn = std::sqrt(n2);
  for (auto& v : b) v /= nn;
  DBuf db, dout;
  TCKS(db.alloc(h, sizeof(cd) * npix));
  TCK(cudaMemcpyAsync(db.p, b.data(), sizeof(cd) * npix, cudaMemcpyHostToDevice, h->stream()));
  TCKS(dout.alloc(h, sizeof(cd) * m->nm));
  bf::note_launch();
  k_project<<<m->nm, 256, 0, h->stream()>>>(dout.as<double2>(), m->d_pat, db.as<double2>(), m->nm, (int)npix);
  TCK(cudaGetLastError());
  TCK(cudaMemcpyAsync(out, dout.p, sizeof(cd) * m->nm, cudaMemcpyDeviceToHost, h->stream()));
  TCK(cudaStreamSynchronize(h->stream()));
  return BF_OK;
}

extern "C" int bf_modes2field(bf_handle* h, const bf_modes* m, const double* coeffs, double* field) {
  if (!h || !m || !coeffs || !field) return BF_ERR_INVALID;
  const size_t npix = (size_t)m->nx * m->ny;
  std::vector<cd> acc(npix, cd(0, 0));
  const cd* c = as_cdp(coeffs);
  for (int k = 0; k < m->nm; ++k)
    for (size_t i = 0; i < npix; ++i) acc[i] += c[k] * m->pat[(size_t)k * npix + i];
  std::copy(acc.begin(), acc.end(), reinterpret_cast<cd*>(field));
  return BF_OK;
}

// One transformer solve (or, with only_matrices, the propagation matrices).
// fp64 selects FP64 class-GEMM operands; otherwise double-float operands on
// the FP32 pipes.  Propagation matrices, inverses, chain and solve are FP64.
// After a solve with the tensor-core GEMMs has synchronised: their error flag.
static int tc_status(bf_handle* h) {
  int e = 0;
  TCK(cudaMemcpyAsync(&e, reinterpret_cast<int*>(h->d_scalar + 2), sizeof(int), cudaMemcpyDeviceToHost,
                      h->stream()));
  TCK(cudaStreamSynchronize(h->stream()));
  if (e) return bf_fail(h, BF_ERR_TIMEOUT, "tensor-core GEMM: a bounded wait expired (stage " + std::to_string(e) + ")");
  return BF_OK;
}

// Antenna coupling fused after the boundary solve: out[f] = |sum_m
// conj(boost[f][m]) antenna[m]|^2, the coupled power of the optimiser cost
// (examples/transformer_optim_utilities.jl:137).
__global__ void k_coupled(double* out, const double2* boost, const double2* ant, int nm, int nf) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  double re = 0.0, im = 0.0;
  for (int m = 0; m < nm; ++m) {
    const double2 b = boost[(size_t)f * nm + m], a = ant[m];
    re += b.x * a.x + b.y * a.y;
    im += b.x * a.y - b.y * a.x;
  }
  out[f] = re * re + im * im;
}

struct CoupleArgs {
  const double* antenna;   // nm complex (the antenna's mode coefficients)
  double* out;             // nf coupled powers
};

// Inputs and output of transformer_trace_back (a solve that stops after the
// inverses and walks the regions instead of running the chain).
struct TraceArgs {
  const double* refl;   // reflected beam, nm complex (per frequency when per_freq)
  const double* inp;    // input beam, nm complex (per frequency when per_freq)
  int per_freq;
  int axion;
  double* out;          // nf x (nd, 2, nm) complex, column-major per frequency
};

// Dynamic shared-memory limit set on the solve kernels: the per-block maximum,
// the same for every launch, so that concurrent launches of one kernel with
// different sizes (serving workers) cannot lower it under one another.
constexpr int kMaxDynSmem = 227 * 1024;

// BF_ERR_SINGULAR when a solve met an exactly zero pivot, as Julia's inv
// (transformer.jl:247) and `\` (:346,356) raise SingularException; the
// outputs were still written (inf/NaN where the pivot was zero).
static int singular_status(bf_handle* h, const int* sing, int nf, const double* freqs) {
  char msg[192];
  if (sing[0] >= 0 && sing[0] < nf) {
    std::snprintf(msg, sizeof msg,
                  "SingularException: a propagation matrix is exactly singular (first at frequency index %d, %.9g Hz)",
                  sing[0], freqs[sing[0]]);
    return bf_fail(h, BF_ERR_SINGULAR, msg);
  }
  if (sing[1] >= 0 && sing[1] < nf) {
    std::snprintf(msg, sizeof msg,
                  "SingularException: the boundary system T22 is exactly singular (first at frequency index %d, %.9g Hz)",
                  sing[1], freqs[sing[1]]);
    return bf_fail(h, BF_ERR_SINGULAR, msg);
  }
  return BF_OK;
}

// PT: storage of the propagation matrices, their inverses and the chain:
// double2 (FP64 path) or float2 (mixed path); the boundary solve is FP64.
// group_regs (a group solve of nreq requests, see bf_transformer_group): the
// regions of every request, regs[r nd + j]; the results then cover nreq nf
// frequencies, request r at r nf + f.
template <typename PT>
static int tf_run_t(bf_handle* h, bf_stack* s, bf_modes* md, int nf, const double* freqs, int prop_kind,
                    const double* emit, const double* reflect, const double* pm, int pm_per_freq,
                    double* out_boost, double* out_refl, double* out_beta2, int mirror_1e30, int only_matrices,
                    double* out_pm, int mode, const TraceArgs* tb = nullptr, const CoupleArgs* cp = nullptr,
                    const PT* P_dev = nullptr, const std::vector<RegionT>* group_regs = nullptr, int nreq = 1) {
  constexpr bool fp64 = std::is_same<PT, double2>::value;
  cudaStream_t st = h->stream();
  const int nd = s->nd, nm = md->nm;
  std::vector<cd> eps(s->eps);
  if (mirror_1e30)
    for (auto& e : eps)
      if (std::isnan(e.real()) || std::isnan(e.imag())) e = cd(1e30, 0.0);   // transformer.jl:289
  std::vector<RegionT> regs;
  if (group_regs) regs = *group_regs;
  else classify(h, s, prop_kind, eps, regs);
  std::vector<double> fv(freqs, freqs + nf);
  DBuf P, Pinv;
  g_tf_gemm_flops = 0.0;
  gemm_ev_collect();
  tf_mark(h, 0);
  const unsigned long long l0 = bf::launch_count();
  if (pm) {
    // injected propagation matrices: [nf or 1][nd][nm][nm], each a Julia (nm, nm) column-major matrix
    std::vector<double2> hp((size_t)nf * nd * nm * nm);
    const cd* src = as_cdp(pm);
    for (int f = 0; f < nf; ++f)
      for (int j = 0; j < nd; ++j) {
        const cd* mj = src + ((size_t)(pm_per_freq ? f : 0) * nd + j) * nm * nm;
        for (int r = 0; r < nm; ++r)
          for (int cidx = 0; cidx < nm; ++cidx) {
            const cd v = mj[r + (size_t)nm * cidx];
            hp[(((size_t)f * nd + j) * nm + r) * nm + cidx] = make_double2(v.real(), v.imag());
          }
      }
    if (fp64) {
      TCKS(P.alloc(h, sizeof(double2) * hp.size()));
      TCK(cudaMemcpyAsync(P.p, hp.data(), sizeof(double2) * hp.size(), cudaMemcpyHostToDevice, st));
    } else {
      DBuf P64;
      TCKS(P64.alloc(h, sizeof(double2) * hp.size()));
      TCK(cudaMemcpyAsync(P64.p, hp.data(), sizeof(double2) * hp.size(), cudaMemcpyHostToDevice, st));
      TCKS(P.alloc(h, sizeof(PT) * hp.size()));
      if (bf::launch_convert(P64.p, true, P.p, false, hp.size(), st)) return bf_fail(h, BF_ERR_CUDA, "convert");
    }
  } else if (!P_dev) {
    TfCache* c = nullptr;
    TCKS(tf_setup(h, s, md, mode, &c));
    const int j0 = only_matrices ? 0 : 1;
    TCKS(tf_propagation_matrices<PT>(h, s, md, *c, regs, j0, nf, fv, prop_kind, P, mode, nreq));
  }
  // a group solve continues over all requests' frequencies (request r at r nf + f)
  std::vector<double> f_all;
  if (nreq > 1) {
    f_all.reserve((size_t)nreq * nf);
    for (int r = 0; r < nreq; ++r) f_all.insert(f_all.end(), freqs, freqs + nf);
    nf *= nreq;
    freqs = f_all.data();
  }
  if (only_matrices) {
    // out_pm: [nf][nd] Julia (nm, nm) column-major matrices
    std::vector<double2> hp((size_t)nf * nd * nm * nm);
    DBuf P64;
    const void* src = P.p;
    if (!fp64) {
      TCKS(P64.alloc(h, sizeof(double2) * hp.size()));
      if (bf::launch_convert(P.p, false, P64.p, true, hp.size(), st)) return bf_fail(h, BF_ERR_CUDA, "convert");
      src = P64.p;
    }
    TCK(cudaMemcpyAsync(hp.data(), src, sizeof(double2) * hp.size(), cudaMemcpyDeviceToHost, st));
    TCK(cudaStreamSynchronize(st));
    if (mode == 2) TCKS(tc_status(h));
    cd* o = reinterpret_cast<cd*>(out_pm);
    for (int f = 0; f < nf; ++f)
      for (int j = 0; j < nd; ++j)
        for (int r = 0; r < nm; ++r)
          for (int cidx = 0; cidx < nm; ++cidx) {
            const double2 v = hp[(((size_t)f * nd + j) * nm + r) * nm + cidx];
            o[((size_t)f * nd + j) * nm * nm + r + (size_t)nm * cidx] = cd(v.x, v.y);
          }
    return BF_OK;
  }
  tf_mark(h, 1);
  // P and its inverses in PT (complex64 on the mixed path: their rounding
  // moves beta^2 by ~1e-6); the chain's T in FP64 or double-float, and the
  // boundary solve, near resonance, in FP64.
  using D2 = PT;
  const D2* Pd = P_dev ? P_dev : P.as<D2>();
  TCKS(Pinv.alloc(h, sizeof(D2) * (size_t)nf * nd * nm * nm));
  // d_sing[0]: lowest frequency index with an exactly singular propagation
  // matrix, d_sing[1]: with an exactly singular T22 (0x7f7f7f7f = none); read
  // back with the solve's outputs
  int* d_sing = reinterpret_cast<int*>(h->d_scalar + 3);
  TCK(cudaMemsetAsync(d_sing, 0x7f, 2 * sizeof(int), st));
  int h_sing[2] = {0x7f7f7f7f, 0x7f7f7f7f};
  // inverses of regions [1, nd) for frequencies [f0, f0 + nfi), or of the
  // regions jl[0 .. njl) only
  auto invert = [&](int f0, int nfi, const int* jl, int njl) -> int {
    const int nj = jl ? njl : nd - 1;
    if (nfi <= 0 || nj <= 0) return BF_OK;
    if (nm <= 16) {
      const int nmat = nj * nfi;
      bf::note_launch();
      if (nm <= 8)
        k_invert_warp<D2, 8><<<(nmat + 31) / 32, 256, 0, st>>>(Pd, Pinv.as<D2>(), nd, 1, nm, nmat, d_sing, f0, jl,
                                                             njl);
      else
        k_invert_warp<D2, 16><<<(nmat + 15) / 16, 256, 0, st>>>(Pd, Pinv.as<D2>(), nd, 1, nm, nmat, d_sing, f0, jl,
                                                              njl);
    } else if (std::is_same<D2, float2>::value && nm <= 64) {
      dim3 grid(nj, nfi);
      bf::note_launch();
      if constexpr (std::is_same<D2, float2>::value) {
        if (nm <= 32) k_invert_reg<32><<<grid, 64, 0, st>>>(Pd, Pinv.as<D2>(), nd, 1, nm, d_sing, f0, jl);
        else k_invert_reg<64><<<grid, 256, 0, st>>>(Pd, Pinv.as<D2>(), nd, 1, nm, d_sing, f0, jl);
      }
    } else {
      const size_t smem = sizeof(D2) * 2 * nm * nm + 256 * (sizeof(double) + sizeof(int));
      TCK(cudaFuncSetAttribute(k_invert<D2>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxDynSmem));
      dim3 grid(nj, nfi);
      bf::note_launch();
      k_invert<D2><<<grid, 256, smem, st>>>(Pd, Pinv.as<D2>(), nd, 1, nm, d_sing, f0, jl);
    }
    TCK(cudaGetLastError());
    return BF_OK;
  };
  if (nreq > 1) {
    // a group: request 0 inverts every region; the others only their own
    // (k-space) air regions and take the disk regions' inverses from request 0
    const int nf0 = nf / nreq;
    std::vector<int> own, shared;
    for (int j = 1; j < nd; ++j) (regs[j].klass == 0 ? own : shared).push_back(j);
    DBuf d_own, d_shared;
    TCKS(invert(0, nf0, nullptr, 0));
    if (!own.empty()) {
      TCKS(d_own.alloc(h, sizeof(int) * own.size()));
      TCK(cudaMemcpyAsync(d_own.p, own.data(), sizeof(int) * own.size(), cudaMemcpyHostToDevice, st));
      TCKS(invert(nf0, nf - nf0, d_own.as<int>(), (int)own.size()));
    }
    if (!shared.empty()) {
      TCKS(d_shared.alloc(h, sizeof(int) * shared.size()));
      TCK(cudaMemcpyAsync(d_shared.p, shared.data(), sizeof(int) * shared.size(), cudaMemcpyHostToDevice, st));
      const size_t total = (size_t)nf0 * shared.size() * nm * nm * (nreq - 1);
      bf::note_launch();
      k_copy_inverses<D2><<<(unsigned)std::min<size_t>(blocks_for(total), 1u << 20), 256, 0, st>>>(
          Pinv.as<D2>(), nd, nm, nf0, nreq, d_shared.as<int>(), (int)shared.size());
      TCK(cudaGetLastError());
    }
  } else {
    TCKS(invert(0, nf, nullptr, 0));
  }
  // chain coefficients: step j uses n_left = sqrt(eps[j]), n_right = sqrt(eps[j-1])
  std::vector<ChainRegion> cr(nd);
  for (int j = 1; j < nd; ++j) {
    const cd nl = std::sqrt(eps[j]), nr = std::sqrt(eps[j - 1]);
    cr[j].a = make_double2((nr + nl).real(), (nr + nl).imag());
    cr[j].b = make_double2((nr - nl).real(), (nr - nl).imag());
    const cd inv = 1.0 / (2.0 * nr);
    cr[j].inv2n = make_double2(inv.real(), inv.imag());
    // axion_S_factor(n1 = sqrt(eps[j-1]), n0 = sqrt(eps[j])) = (1/n1^2 - 1/n0^2)/2
    const cd S = (1.0 / (nr * nr) - 1.0 / (nl * nl)) / 2.0;
    cr[j].S = make_double2(S.real(), S.imag());
  }
  std::vector<cd> em(nm);
  if (emit) {
    em.assign(as_cdp(emit), as_cdp(emit) + nm);
  } else {
    // default emit = axion_induced_modes(coords, modes; B=nothing, diskR) (transformer.jl:285),
    // computed once per (modes, diskR)
    std::lock_guard<std::mutex> lock(md->emit_mu);
    if (md->emit_diskR != s->diskR || (int)md->emit.size() != nm) {
      std::vector<cd> e(nm);
      TCKS(bf_axion_induced_modes(h, md, nullptr, 0.0, s->diskR, 10e9, reinterpret_cast<double*>(e.data())));
      md->emit = e;
      md->emit_diskR = s->diskR;
    }
    em = md->emit;
  }
  DBuf d_cr, d_em, T21, T22, ax, d_refl, boost, refl, b2;
  TCKS(d_cr.alloc(h, sizeof(ChainRegion) * nd));
  TCK(cudaMemcpyAsync(d_cr.p, cr.data(), sizeof(ChainRegion) * nd, cudaMemcpyHostToDevice, st));
  TCKS(d_em.alloc(h, sizeof(cd) * nm));
  TCK(cudaMemcpyAsync(d_em.p, em.data(), sizeof(cd) * nm, cudaMemcpyHostToDevice, st));
  if (tb) {
    const size_t nb = (size_t)(tb->per_freq ? nf : 1) * nm;
    DBuf d_in, d_rf, d_out;
    TCKS(d_in.alloc(h, sizeof(cd) * nb));
    TCK(cudaMemcpyAsync(d_in.p, tb->inp, sizeof(cd) * nb, cudaMemcpyHostToDevice, st));
    TCKS(d_rf.alloc(h, sizeof(cd) * nb));
    TCK(cudaMemcpyAsync(d_rf.p, tb->refl, sizeof(cd) * nb, cudaMemcpyHostToDevice, st));
    const size_t nout = (size_t)nf * nd * 2 * nm;
    TCKS(d_out.alloc(h, sizeof(cd) * nout));
    bf::note_launch();
    k_trace_back<D2><<<nf, 256, sizeof(double2) * 4 * nm, st>>>(
        Pd, Pinv.as<D2>(), d_cr.as<ChainRegion>(), nd, nm, d_rf.as<double2>(), d_in.as<double2>(),
        tb->per_freq ? nm : 0, d_em.as<double2>(), tb->axion, d_out.as<double2>());
    TCK(cudaGetLastError());
    TCK(cudaMemcpyAsync(tb->out, d_out.p, sizeof(cd) * nout, cudaMemcpyDeviceToHost, st));
    TCK(cudaMemcpyAsync(h_sing, d_sing, sizeof(h_sing), cudaMemcpyDeviceToHost, st));
    TCK(cudaStreamSynchronize(st));
    if (mode == 2 && !pm && !P_dev) TCKS(tc_status(h));
    return singular_status(h, h_sing, nf, freqs);
  }
  // T21 / T22 for the boundary solve, FP64
  TCKS(T21.alloc(h, sizeof(double2) * (size_t)nf * nm * nm));
  TCKS(T22.alloc(h, sizeof(double2) * (size_t)nf * nm * nm));
  TCKS(ax.alloc(h, sizeof(double2) * (size_t)nf * nm));
  if constexpr (fp64) {
    const size_t smem = sizeof(D2) * 2 * nm * nm + sizeof(double2) * 2 * nm;
    TCK(cudaFuncSetAttribute(k_chain<D2>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxDynSmem));
    bf::note_launch();
    k_chain<D2><<<nf, 256, smem, st>>>(Pd, Pinv.as<D2>(), d_cr.as<ChainRegion>(), nd, nm, d_em.as<double2>(),
                                       T21.as<D2>(), T22.as<D2>(), ax.as<double2>());
    TCK(cudaGetLastError());
  } else {
    DBuf T21df, T22df, Wdf;
    size_t smem = (sizeof(DFc) * 2 + sizeof(float2) * 2) * nm * nm + (sizeof(double2) + sizeof(DFc)) * nm;
    const bool t_in_smem = smem + sizeof(DFc) * 2 * nm * nm <= 160 * 1024;
    const bool par_axion = t_in_smem && smem + sizeof(DFc) * 3 * nm * nm <= 160 * 1024;
    if (t_in_smem) {
      smem += sizeof(DFc) * (par_axion ? 3 : 2) * nm * nm;
    } else {
      TCKS(T21df.alloc(h, sizeof(DFc) * (size_t)nf * nm * nm));
      TCKS(T22df.alloc(h, sizeof(DFc) * (size_t)nf * nm * nm));
      // the axion terms go to global scratch, so that their row sums (in k
      // order) are a short chain beside the products instead of a long one
      // before them
      TCKS(Wdf.alloc(h, sizeof(DFc) * (size_t)nf * nm * nm));
    }
    TCK(cudaFuncSetAttribute(k_chain_df, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxDynSmem));
    bf::note_launch();
    // one thread per matrix entry up to 1024 (at 64 modes one CTA per frequency
    // owns the SM's shared memory, and 32 warps hide the serial TwoSum chains;
    // at few modes small CTAs, many per SM, keep every warp busy)
    const int nthr = std::min(1024, std::max(32, (nm * nm + 31) / 32 * 32));
    k_chain_df<<<nf, nthr, smem, st>>>(Pd, Pinv.as<D2>(), d_cr.as<ChainRegion>(), nd, nm, d_em.as<double2>(),
                                      t_in_smem ? nullptr : T21df.as<DFc>(), t_in_smem ? nullptr : T22df.as<DFc>(),
                                      ax.as<double2>(), T21.as<double2>(),
                                      T22.as<double2>(), par_axion ? 1 : 0, t_in_smem ? nullptr : Wdf.as<DFc>());
    TCK(cudaGetLastError());
  }
  if (reflect) {
    TCKS(d_refl.alloc(h, sizeof(cd) * nm));
    TCK(cudaMemcpyAsync(d_refl.p, reflect, sizeof(cd) * nm, cudaMemcpyHostToDevice, st));
  }
  TCKS(boost.alloc(h, sizeof(cd) * (size_t)nf * nm));
  if (reflect) TCKS(refl.alloc(h, sizeof(cd) * (size_t)nf * nm));
  TCKS(b2.alloc(h, sizeof(double) * nf));
  if (nm <= 16) {
    bf::note_launch();
    if (nm <= 8)
      k_final_solve_warp<8><<<(nf + 31) / 32, 256, 0, st>>>(T21.as<double2>(), T22.as<double2>(), ax.as<double2>(),
                                                          reflect ? d_refl.as<double2>() : nullptr, nm,
                                                          boost.as<double2>(), reflect ? refl.as<double2>() : nullptr,
                                                          b2.as<double>(), d_sing + 1, nf);
    else
      k_final_solve_warp<16><<<(nf + 15) / 16, 256, 0, st>>>(T21.as<double2>(), T22.as<double2>(), ax.as<double2>(),
                                                           reflect ? d_refl.as<double2>() : nullptr, nm,
                                                           boost.as<double2>(), reflect ? refl.as<double2>() : nullptr,
                                                           b2.as<double>(), d_sing + 1, nf);
    TCK(cudaGetLastError());
  } else {
    const size_t smem = sizeof(double2) * nm * (nm + 2) + 256 * (sizeof(double) + sizeof(int));
    TCK(cudaFuncSetAttribute(k_final_solve<double2>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxDynSmem));
    bf::note_launch();
    k_final_solve<double2><<<nf, 256, smem, st>>>(T21.as<double2>(), T22.as<double2>(), ax.as<double2>(),
                                             reflect ? d_refl.as<double2>() : nullptr, nm, boost.as<double2>(),
                                             reflect ? refl.as<double2>() : nullptr, b2.as<double>(), d_sing + 1);
    TCK(cudaGetLastError());
  }
  DBuf d_ant, d_cpl;
  if (cp) {
    TCKS(d_ant.alloc(h, sizeof(cd) * nm));
    TCK(cudaMemcpyAsync(d_ant.p, cp->antenna, sizeof(cd) * nm, cudaMemcpyHostToDevice, st));
    TCKS(d_cpl.alloc(h, sizeof(double) * nf));
    bf::note_launch();
    k_coupled<<<blocks_for(nf), 256, 0, st>>>(d_cpl.as<double>(), boost.as<double2>(), d_ant.as<double2>(), nm, nf);
    TCK(cudaGetLastError());
  }
  tf_mark(h, 2);
  if (h->profiling) {
    TCK(cudaEventSynchronize(h->ev[2]));
    float t01 = 0, t12 = 0, t02 = 0;
    cudaEventElapsedTime(&t01, h->ev[0], h->ev[1]);
    cudaEventElapsedTime(&t12, h->ev[1], h->ev[2]);
    cudaEventElapsedTime(&t02, h->ev[0], h->ev[2]);
    h->prof[0] = t02;      // whole solve
    h->prof[1] = t01;      // propagation matrices (class GEMMs)
    h->prof[2] = t12;      // inverses, chain, boundary solve
    h->prof[4] = (double)g_gemm_ev.size();   // class-GEMM kernel launches
    h->prof[3] = gemm_ev_collect();          // device ms of the class-GEMM kernels alone
    h->prof[5] = (double)(bf::launch_count() - l0);
    h->prof[6] = g_tf_gemm_flops;
    h->prof[7] = nf;
    h->prof_valid = 1;
  }
  if (out_boost) TCK(cudaMemcpyAsync(out_boost, boost.p, sizeof(cd) * nf * nm, cudaMemcpyDeviceToHost, st));
  if (out_refl && reflect) TCK(cudaMemcpyAsync(out_refl, refl.p, sizeof(cd) * nf * nm, cudaMemcpyDeviceToHost, st));
  if (out_beta2) TCK(cudaMemcpyAsync(out_beta2, b2.p, sizeof(double) * nf, cudaMemcpyDeviceToHost, st));
  if (cp) TCK(cudaMemcpyAsync(cp->out, d_cpl.p, sizeof(double) * nf, cudaMemcpyDeviceToHost, st));
  TCK(cudaMemcpyAsync(h_sing, d_sing, sizeof(h_sing), cudaMemcpyDeviceToHost, st));
  TCK(cudaStreamSynchronize(st));
  if (mode == 2 && !pm && !P_dev) TCKS(tc_status(h));
  return singular_status(h, h_sing, nf, freqs);
}

// precision: BF_PREC_FP64 (mode 0), BF_PREC_MIXED or BF_PREC_TF32 (mode 2: the
// tensor-core overlap GEMMs), BF_PREC_MIXED_SIMT (mode 1: the SIMT GEMMs)
static int tf_run(bf_handle* h, bf_stack* s, bf_modes* md, int nf, const double* freqs, int prop_kind,
                  int precision, const double* emit, const double* reflect, const double* pm, int pm_per_freq,
                  double* out_boost, double* out_refl, double* out_beta2, int mirror_1e30, int only_matrices,
                  double* out_pm, const TraceArgs* tb = nullptr, const CoupleArgs* cp = nullptr) {
  if (precision == BF_PREC_FP64)
    return tf_run_t<double2>(h, s, md, nf, freqs, prop_kind, emit, reflect, pm, pm_per_freq, out_boost, out_refl,
                             out_beta2, mirror_1e30, only_matrices, out_pm, 0, tb, cp);
  return tf_run_t<float2>(h, s, md, nf, freqs, prop_kind, emit, reflect, pm, pm_per_freq, out_boost, out_refl,
                          out_beta2, mirror_1e30, only_matrices, out_pm, precision == BF_PREC_MIXED_SIMT ? 1 : 2, tb,
                          cp);
}

static int tf_check(bf_handle* h, bf_stack* s, bf_modes* md, int nf, const double* freqs, int prop_kind,
                    int precision) {
  if (!h) return BF_ERR_INVALID;
  if (!s || !md) return bf_fail(h, BF_ERR_INVALID, "null stack or modes");
  if (md->nx != s->nx || md->ny != s->ny) return bf_fail(h, BF_ERR_INVALID, "modes and stack grids differ");
  if (nf < 1 || !freqs) return bf_fail(h, BF_ERR_INVALID, "need at least one frequency");
  for (int i = 0; i < nf; ++i)
    if (!(freqs[i] > 0) || !std::isfinite(freqs[i])) return bf_fail(h, BF_ERR_INVALID, "bad frequency");
  if (prop_kind < 0 || prop_kind > 3) return bf_fail(h, BF_ERR_INVALID, "unknown propagator kind");
  if (precision != BF_PREC_FP64 && precision != BF_PREC_MIXED && precision != BF_PREC_TF32 &&
      precision != BF_PREC_MIXED_SIMT)
    return bf_fail(h, BF_ERR_INVALID, "unknown precision");
  if ((precision == BF_PREC_MIXED || precision == BF_PREC_TF32) && !bf::tc_gemm_available())
    return bf_fail(h, BF_ERR_UNSUPPORTED, "tensor-core GEMMs: the tensor-map encoder of the driver is unavailable");
  return BF_OK;
}

extern "C" int bf_transformer(bf_handle* h, bf_stack* s, bf_modes* md, int nf, const double* freqs, int prop_kind,
                              int precision, const double* emit, const double* reflect,
                              const double* propagation_matrices, int pm_per_freq, double* out_boost,
                              double* out_refl, double* out_beta2) {
  TCKS(tf_check(h, s, md, nf, freqs, prop_kind, precision));
  TCK(cudaSetDevice(h->device));
  return tf_run(h, s, md, nf, freqs, prop_kind, precision, emit, reflect, propagation_matrices,
                pm_per_freq, out_boost, out_refl, out_beta2, 1, 0, nullptr);
}

// ---- batched 1D model: one thread per (spacing configuration, frequency) ------
// transformer(bdry, coords, SeedModes(coords; ThreeDim=false); prop=propagator1D)
// with every matrix a scalar: P_j = exp(-i k0_j dz_j), T21' = s_j P_j (a_j T21 +
// b_j T22), T22' = s_j / P_j (b_j T21 + a_j T22), axion_beam += S_j (T21 + T22)
// emit, boost = -axion_beam / T22 (src/boost_fractor_transformer.jl:285-359).
// GB300's FP64 rate is 1/64 of FP32, so the per-region work is kept small:
// the boundary factors carry 1/(2 n_j) and the emission carries S_j (folded on
// the host); the phase k0 dz = pi (2 f / c) n dz goes through sincospi, whose
// argument reduction is exact and cheap; a lossless region (real eps, held as
// re - 0.0im, so Im n = -0.0 and exp(Im k0 dz) = 1 exactly) needs no exp, and
// its 1/P is conj(P).
struct Region1D {
  double2 a, b;   // (n_{j-1} + n_j) / (2 n_{j-1}),  (n_{j-1} - n_j) / (2 n_{j-1})
  double2 Se;     // S_j * emit
  double2 n;      // sqrt(eps_j) of the propagated region
};

__global__ void k_tf1d(const double* dist, int nd, const Region1D* rg, const double* freqs, int nf, int nconf,
                       double2* boost, double* beta2) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= (long)nconf * nf) return;
  const int c = (int)(i / nf), f = (int)(i % nf);
  const double* dz = dist + (size_t)c * nd;
  const double x2 = 2.0 * freqs[f] / kC;   // 2 / lambda: k0 = pi x2 n
  double2 t21 = make_double2(0.0, 0.0), t22 = make_double2(1.0, 0.0), ax = make_double2(0.0, 0.0);
  for (int j = 1; j < nd; ++j) {
    const Region1D g = rg[j];
    ax = bf::cadd(ax, bf::cmul(g.Se, bf::cadd(t21, t22)));
    double sn, cs;
    sincospi(x2 * g.n.x * dz[j], &sn, &cs);
    double2 P = make_double2(cs, -sn), Pi = make_double2(cs, sn);
    if (g.n.y != 0.0) {   // uniform across the warp: every thread is at region j
      const double m = exp(M_PI * x2 * g.n.y * dz[j]), mi = 1.0 / m;
      P = make_double2(m * cs, -m * sn);
      Pi = make_double2(mi * cs, mi * sn);
    }
    const double2 u = bf::cadd(bf::cmul(g.a, t21), bf::cmul(g.b, t22));
    const double2 v = bf::cadd(bf::cmul(g.b, t21), bf::cmul(g.a, t22));
    t21 = bf::cmul(u, P);
    t22 = bf::cmul(v, Pi);
  }
  const double d = t22.x * t22.x + t22.y * t22.y;
  const double2 q = make_double2(-(ax.x * t22.x + ax.y * t22.y) / d, -(ax.y * t22.x - ax.x * t22.y) / d);
  if (boost) boost[i] = q;
  beta2[i] = q.x * q.x + q.y * q.y;
}

// Cross-request batch: the transformer for nreq stacks that differ only in
// the distances of their k-space (untilted, flat air) regions, e.g. the stacks
// of several disk-position optimisers at one step.  One solve: the air-region
// overlaps of all requests form one GEMM, the disk regions' matrices are
// computed once, and the inverses, chains and boundary solves run over all
// nreq nf (request, frequency) pairs.  Outputs request-major: beta2[r nf + f],
// boost[(r nf + f) nm + m].
extern "C" int bf_transformer_group(bf_handle* h, int nreq, bf_stack* const* stacks, bf_modes* md, int nf,
                                    const double* freqs, int prop_kind, int precision, double* out_boost,
                                    double* out_beta2) {
  if (!h) return BF_ERR_INVALID;
  if (nreq < 1 || !stacks || !stacks[0]) return bf_fail(h, BF_ERR_INVALID, "empty group");
  TCKS(tf_check(h, stacks[0], md, nf, freqs, prop_kind, precision));
  const bf_stack* s0 = stacks[0];
  const int nd = s0->nd;
  auto same_eps = [](cd a, cd b) {
    return (a == b) || (std::isnan(a.real()) && std::isnan(b.real()) && a.imag() == b.imag());
  };
  std::vector<RegionT> all, r0;
  all.reserve((size_t)nreq * nd);
  for (int r = 0; r < nreq; ++r) {
    bf_stack* sr = stacks[r];
    if (!sr) return bf_fail(h, BF_ERR_INVALID, "null stack in group");
    bool ok = sr->nd == nd && sr->nx == s0->nx && sr->ny == s0->ny && sr->X == s0->X && sr->Y == s0->Y &&
              sr->diskR == s0->diskR && sr->tilt_x == s0->tilt_x && sr->tilt_y == s0->tilt_y &&
              (sr == s0 || (sr->surf.empty() && s0->surf.empty()));
    for (int j = 0; ok && j < nd; ++j) ok = same_eps(sr->eps[j], s0->eps[j]);
    if (!ok)
      return bf_fail(h, BF_ERR_INVALID,
                     "group: stacks must share grid, disk radius, permittivities and tilts, without surface maps");
    std::vector<cd> eps(sr->eps);
    for (auto& e : eps)
      if (std::isnan(e.real()) || std::isnan(e.imag())) e = cd(1e30, 0.0);   // transformer.jl:289
    std::vector<RegionT> rg;
    classify(h, sr, prop_kind, eps, rg);
    if (r == 0) r0 = rg;
    for (int j = 0; j < nd; ++j) {
      if (rg[j].klass != r0[j].klass)
        return bf_fail(h, BF_ERR_INVALID, "group: the stacks' regions fall in different overlap classes");
      if (j > 0 && rg[j].klass != 0 && rg[j].dz != r0[j].dz)
        return bf_fail(h, BF_ERR_INVALID, "group: only the distances of untilted air regions may differ");
    }
    all.insert(all.end(), rg.begin(), rg.end());
  }
  TCK(cudaSetDevice(h->device));
  bf_stack* s = stacks[0];
  if (precision == BF_PREC_FP64)
    return tf_run_t<double2>(h, s, md, nf, freqs, prop_kind, nullptr, nullptr, nullptr, 0, out_boost, nullptr,
                             out_beta2, 1, 0, nullptr, 0, nullptr, nullptr, nullptr, &all, nreq);
  return tf_run_t<float2>(h, s, md, nf, freqs, prop_kind, nullptr, nullptr, nullptr, 0, out_boost, nullptr,
                          out_beta2, 1, 0, nullptr, precision == BF_PREC_MIXED_SIMT ? 1 : 2, nullptr, nullptr,
                          nullptr, &all, nreq);
}

extern "C" int bf_transformer_1d_batch(bf_handle* h, int nconf, int nd, const double* distances, const double* eps,
                                       int nf, const double* freqs, const double* emit, double* out_boost,
                                       double* out_beta2) {
  if (!h) return BF_ERR_INVALID;
  if (nconf < 1 || nd < 3 || nf < 1 || !distances || !eps || !freqs || !out_beta2)
    return bf_fail(h, BF_ERR_INVALID, "transformer_1d_batch: empty or null input");
  for (size_t i = 0; i < (size_t)nconf * nd; ++i)
    if (!std::isfinite(distances[i])) return bf_fail(h, BF_ERR_INVALID, "non-finite distance");
  for (int i = 0; i < nf; ++i)
    if (!(freqs[i] > 0.0) || !std::isfinite(freqs[i]))
      return bf_fail(h, BF_ERR_INVALID, "frequencies must be finite and positive");
  TCK(cudaSetDevice(h->device));
  cudaStream_t st = h->stream();
  // permittivities as the stacks hold them (real eps as re - 0.0im), NaN mirror -> 1e30
  std::vector<cd> e(nd);
  for (int j = 0; j < nd; ++j) {
    cd v = as_cdp(eps)[j];
    if (std::isnan(v.real()) || std::isnan(v.imag())) v = cd(1e30, 0.0);
    e[j] = bfhost::eps_cast(v);
  }
  std::vector<Region1D> rg(nd);
  for (int j = 1; j < nd; ++j) {
    const cd nl = std::sqrt(e[j]), nr = std::sqrt(e[j - 1]);
    const cd inv = 1.0 / (2.0 * nr);
    const cd a = (nr + nl) * inv, b = (nr - nl) * inv;
    rg[j].a = make_double2(a.real(), a.imag());
    rg[j].b = make_double2(b.real(), b.imag());
    const cd S = (1.0 / (nr * nr) - 1.0 / (nl * nl)) / 2.0;
    const cd Se = S * (emit ? cd(emit[0], emit[1]) : cd(1.0, 0.0));
    rg[j].Se = make_double2(Se.real(), Se.imag());
    rg[j].n = make_double2(nl.real(), nl.imag());
  }
  const size_t npts = (size_t)nconf * nf;
  DBuf d_dist, d_rg, d_f, d_b, d_b2;
  TCKS(d_dist.alloc(h, sizeof(double) * (size_t)nconf * nd));
  TCK(cudaMemcpyAsync(d_dist.p, distances, sizeof(double) * (size_t)nconf * nd, cudaMemcpyHostToDevice, st));
  TCKS(d_rg.alloc(h, sizeof(Region1D) * nd));
  TCK(cudaMemcpyAsync(d_rg.p, rg.data(), sizeof(Region1D) * nd, cudaMemcpyHostToDevice, st));
  TCKS(d_f.alloc(h, sizeof(double) * nf));
  TCK(cudaMemcpyAsync(d_f.p, freqs, sizeof(double) * nf, cudaMemcpyHostToDevice, st));
  if (out_boost) TCKS(d_b.alloc(h, sizeof(double2) * npts));
  TCKS(d_b2.alloc(h, sizeof(double) * npts));
  bf::note_launch();
  tf_mark(h, 0);
  k_tf1d<<<(unsigned)((npts + 255) / 256), 256, 0, st>>>(d_dist.as<double>(), nd, d_rg.as<Region1D>(),
                                                          d_f.as<double>(), nf, nconf,
                                                          out_boost ? d_b.as<double2>() : nullptr, d_b2.as<double>());
  TCK(cudaGetLastError());
  tf_mark(h, 1);
  if (h->profiling) {
    TCK(cudaEventSynchronize(h->ev[1]));
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, h->ev[0], h->ev[1]);
    for (double& v : h->prof) v = 0.0;
    h->prof[0] = ms;   // the k_tf1d launch (inputs resident)
    h->prof[1] = ms;
    h->prof[5] = 1;
    h->prof[7] = nf;
    h->prof_valid = 1;
  }
  if (out_boost) TCK(cudaMemcpyAsync(out_boost, d_b.p, sizeof(double2) * npts, cudaMemcpyDeviceToHost, st));
  TCK(cudaMemcpyAsync(out_beta2, d_b2.p, sizeof(double) * npts, cudaMemcpyDeviceToHost, st));
  TCK(cudaStreamSynchronize(st));
  return BF_OK;
}

extern "C" int bf_transformer_coupled(bf_handle* h, bf_stack* s, bf_modes* md, int nf, const double* freqs,
                                      int prop_kind, int precision, const double* emit, const double* antenna,
                                      const double* propagation_matrices, int pm_per_freq, double* out_coupled,
                                      double* out_beta2) {
  TCKS(tf_check(h, s, md, nf, freqs, prop_kind, precision));
  if (!antenna || !out_coupled) return bf_fail(h, BF_ERR_INVALID, "null antenna or output");
  TCK(cudaSetDevice(h->device));
  CoupleArgs cp{antenna, out_coupled};
  return tf_run(h, s, md, nf, freqs, prop_kind, precision, emit, nullptr, propagation_matrices, pm_per_freq,
                nullptr, nullptr, out_beta2, 1, 0, nullptr, nullptr, &cp);
}

extern "C" int bf_transformer_trace_back(bf_handle* h, bf_stack* s, bf_modes* md, int nf, const double* freqs,
                                         int prop_kind, int precision, const double* reflected_beam,
                                         const double* input_beam, int beams_per_freq, int includes_axion,
                                         const double* emit, const double* propagation_matrices, int pm_per_freq,
                                         double* out) {
  TCKS(tf_check(h, s, md, nf, freqs, prop_kind, precision));
  if (!reflected_beam || !input_beam || !out) return bf_fail(h, BF_ERR_INVALID, "null beam or output");
  TCK(cudaSetDevice(h->device));
  TraceArgs tb{reflected_beam, input_beam, beams_per_freq ? 1 : 0, includes_axion ? 1 : 0, out};
  // the reference's trace-back does not replace a NaN mirror permittivity (no mutation here either)
  return tf_run(h, s, md, nf, freqs, prop_kind, precision, emit, nullptr, propagation_matrices,
                pm_per_freq, nullptr, nullptr, nullptr, 0, 0, nullptr, &tb);
}

extern "C" int bf_calc_propagation_matrices(bf_handle* h, bf_stack* s, bf_modes* md, int nf, const double* freqs,
                                            int prop_kind, int precision, double* out) {
  TCKS(tf_check(h, s, md, nf, freqs, prop_kind, precision));
  if (!out) return bf_fail(h, BF_ERR_INVALID, "null output");
  TCK(cudaSetDevice(h->device));
  return tf_run(h, s, md, nf, freqs, prop_kind, precision, nullptr, nullptr, nullptr, 0, nullptr,
                nullptr, nullptr, 0, 1, out);
}

// ---------------------------------------------------------------------------
// Propagation-matrix grid over gap spacings, with interpolation
// (examples/transformer_optim_utilities.jl:11-91: calc_propagation_matrices_grid,
// construct_prop_matrix_interpolation, interpolate_prop_matrix).
// ---------------------------------------------------------------------------
// Gaps are the regions 1, 3, ..., nd-1 (the reference's ind_gap = 2:2:n_region,
// the last region included); the others (mirror, disks) are computed once per
// frequency.  At grid point k every gap's distance is d0 + s0 + k ds.
struct bf_pgrid {
  bf_stack* s = nullptr;
  bf_modes* md = nullptr;
  int nf = 0, nd = 0, nm = 0, nsp = 0, ngap = 0;
  double s0 = 0.0, ds = 0.0;
  std::vector<double> freqs;
  std::vector<int> gap_of;   // region -> gap slot, or -1
  DBuf gap_d, solid, coef;   // gap_of on the device; solids [nf][nd][nm^2]; [ngap][nf][nsp + 2][nm^2]
  DBuf thomas;               // 1/(4 - c'_{k-1}) and c'_k of the spline system, 2 (nsp + 2) doubles
  int precision = BF_PREC_FP64;
  std::vector<cd> emit;      // the default emission (axion-induced modes), computed once
};

namespace {

// grid value of gap g at spacing k: coef[g][f][k + 1][e] = P_k[f][j][e]; solids at k = 0
template <typename PT>
__global__ void k_pgrid_gather(double2* coef, double2* solid, const PT* P, const int* gap_of, int nf, int nd, int nm2,
                               int nsp, int k) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= (size_t)nf * nd * nm2) return;
  const int e = (int)(i % nm2);
  const int j = (int)((i / nm2) % nd);
  const int f = (int)(i / ((size_t)nm2 * nd));
  const double2 v = bf::to_d(P[i]);
  const int g = gap_of[j];
  if (g >= 0)
    coef[(((size_t)g * nf + f) * (nsp + 2) + k + 1) * nm2 + e] = v;
  else if (k == 0)
    solid[i] = v;
}

// Cubic B-spline prefilter along the spacing axis, in place, with the
// boundary conditions of Interpolations.jl's Cubic(Natural(OnCell())): the
// spline interpolates y_1..y_n at the knots 1..n, (c_{k-1} + 4 c_k + c_{k+1})
// / 6 = y_k, and its second derivative vanishes at the cell edges 1/2 and
// n + 1/2, half a step outside the end knots.  With the end segments'
// polynomials extended there, S''(1/2) = 0 reads 3 c_0 - 7 c_1 + 5 c_2 - c_3
// = 0; eliminating c_0 and c_3 with the first two knot rows leaves
//   3 c_1 - c_2 = 3 y_1 - y_2,   c_{k-1} + 4 c_k + c_{k+1} = 6 y_k (k = 2..n-1),
//   -c_{n-1} + 3 c_n = 3 y_n - y_{n-1}
// (tridiagonal, diagonally dominant), then c_0 = 6 y_1 - 4 c_1 - c_2 and
// c_{n+1} = 6 y_n - 4 c_n - c_{n-1}.  Data y_k sit at coef[k]; the host
// supplies the Thomas factors 1/m_k and c'_k of this constant matrix.
__global__ void k_pgrid_prefilter(double2* coef, const double* thomas, int nseq_outer, int nm2, int nsp) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= (size_t)nseq_outer * nm2) return;
  const int e = (int)(i % nm2);
  double2* c = coef + (i / nm2) * (size_t)(nsp + 2) * nm2 + e;
  const int n = nsp;
  auto at = [&](int k) -> double2& { return c[(size_t)k * nm2]; };
  const double* inv_m = thomas;          // 1 / m_k, k = 1..n
  const double* cpr = thomas + (n + 2);  // c'_k, k = 1..n-1
  const double2 y1 = at(1), y2 = at(2), yn = at(n), yn1 = at(n - 1);
  // forward sweep: d'_k = (r_k - a_k d'_{k-1}) / m_k; sub-diagonal a_k = 1 inside, -1 in row n
  double2 prev = make_double2(0.0, 0.0);
  for (int k = 1; k <= n; ++k) {
    double2 r;
    double a;
    if (k == 1) {
      r = make_double2(3.0 * y1.x - y2.x, 3.0 * y1.y - y2.y);
      a = 0.0;
    } else if (k == n) {
      r = make_double2(3.0 * yn.x - yn1.x, 3.0 * yn.y - yn1.y);
      a = -1.0;
    } else {
      r = make_double2(6.0 * at(k).x, 6.0 * at(k).y);
      a = 1.0;
    }
    const double2 d = make_double2((r.x - a * prev.x) * inv_m[k], (r.y - a * prev.y) * inv_m[k]);
    at(k) = d;
    prev = d;
  }
  for (int k = n - 1; k >= 1; --k) {
    const double2 nx = at(k + 1);
    at(k) = make_double2(at(k).x - cpr[k] * nx.x, at(k).y - cpr[k] * nx.y);
  }
  at(0) = make_double2(6.0 * y1.x - 4.0 * at(1).x - at(2).x, 6.0 * y1.y - 4.0 * at(1).y - at(2).y);
  at(n + 1) = make_double2(6.0 * yn.x - 4.0 * at(n).x - at(n - 1).x, 6.0 * yn.y - 4.0 * at(n).y - at(n - 1).y);
}

// P[f][j][e] at the gap positions x[j] (data coordinates 1/2..n+1/2): uniform
// cubic B-spline weights on c_{i-1..i+2}, i = floor(x) clamped to 1..n-1, so
// the end segments' polynomials cover the half cells beyond the end knots
__global__ void k_pgrid_eval(double2* P, const double2* solid, const double2* coef, const int* gap_of,
                             const double* xpos, int nf, int nd, int nm2, int nsp) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= (size_t)nf * nd * nm2) return;
  const int e = (int)(i % nm2);
  const int j = (int)((i / nm2) % nd);
  const int f = (int)(i / ((size_t)nm2 * nd));
  const int g = gap_of[j];
  if (g < 0) {
    P[i] = solid[i];
    return;
  }
  const double x = xpos[j];
  int k = (int)floor(x);
  if (k >= nsp) k = nsp - 1;
  if (k < 1) k = 1;
  const double t = x - k, t2 = t * t, t3 = t2 * t;
  const double w0 = (1.0 - t) * (1.0 - t) * (1.0 - t) / 6.0;
  const double w1 = (3.0 * t3 - 6.0 * t2 + 4.0) / 6.0;
  const double w2 = (-3.0 * t3 + 3.0 * t2 + 3.0 * t + 1.0) / 6.0;
  const double w3 = t3 / 6.0;
  const double2* c = coef + ((size_t)g * nf + f) * (size_t)(nsp + 2) * nm2 + e;
  const double2 a = c[(size_t)(k - 1) * nm2], b = c[(size_t)k * nm2], d = c[(size_t)(k + 1) * nm2],
                q = c[(size_t)(k + 2) * nm2];
  P[i] = make_double2(w0 * a.x + w1 * b.x + w2 * d.x + w3 * q.x, w0 * a.y + w1 * b.y + w2 * d.y + w3 * q.y);
}

template <typename PT>
int pgrid_fill(bf_handle* h, bf_pgrid* G, int prop_kind, int mode) {
  bf_stack* s = G->s;
  cudaStream_t st = h->stream();
  const int nm2 = G->nm * G->nm;
  TfCache* c = nullptr;
  TCKS(tf_setup(h, s, G->md, mode, &c));
  std::vector<double> d0 = s->distance;
  DBuf P;
  int rc = BF_OK;
  for (int k = 0; k < G->nsp && rc == BF_OK; ++k) {
    for (int j = 0; j < G->nd; ++j)
      if (G->gap_of[j] >= 0) s->distance[j] = d0[j] + G->s0 + k * G->ds;
    std::vector<RegionT> regs;
    classify(h, s, prop_kind, s->eps, regs);
    rc = tf_propagation_matrices<PT>(h, s, G->md, *c, regs, 0, G->nf, G->freqs, prop_kind, P, mode);
    if (rc != BF_OK) break;
    bf::note_launch();
    k_pgrid_gather<PT><<<blocks_for((size_t)G->nf * G->nd * nm2), 256, 0, st>>>(
        G->coef.as<double2>(), G->solid.as<double2>(), P.as<PT>(), G->gap_d.as<int>(), G->nf, G->nd, nm2, G->nsp,
        k);
    if (cudaGetLastError() != cudaSuccess) rc = bf_fail(h, BF_ERR_CUDA, "pgrid gather");
  }
  s->distance = d0;   // the stack keeps its own distances
  if (rc != BF_OK) return rc;
  TCK(cudaStreamSynchronize(st));
  return BF_OK;
}

}  // namespace

extern "C" int bf_pgrid_create(bf_handle* h, bf_stack* s, bf_modes* md, int nf, const double* freqs, int nsp,
                               double spacing_first, double spacing_step, int prop_kind, int precision,
                               bf_pgrid** out) {
  if (!out) return BF_ERR_INVALID;
  *out = nullptr;
  TCKS(tf_check(h, s, md, nf, freqs, prop_kind, precision));
  if (precision == BF_PREC_TF32 || precision == BF_PREC_MIXED_SIMT)
    return bf_fail(h, BF_ERR_INVALID, "pgrid: BF_PREC_FP64 or BF_PREC_MIXED");
  if (nsp < 2 || nsp > BF_PGRID_MAX_SPACINGS || !(spacing_step > 0.0) || !std::isfinite(spacing_first))
    return bf_fail(h, BF_ERR_INVALID, "pgrid: 2..64 spacings with a positive step");
  TCK(cudaSetDevice(h->device));
  std::unique_ptr<bf_pgrid> G(new bf_pgrid());
  G->s = s;
  G->md = md;
  G->nf = nf;
  G->nd = s->nd;
  G->nm = md->nm;
  G->nsp = nsp;
  G->s0 = spacing_first;
  G->ds = spacing_step;
  G->freqs.assign(freqs, freqs + nf);
  G->gap_of.assign(s->nd, -1);
  for (int j = 1; j < s->nd; j += 2) G->gap_of[j] = G->ngap++;
  const size_t nm2 = (size_t)G->nm * G->nm;
  cudaStream_t st = h->stream();
  TCKS(G->gap_d.alloc(h, sizeof(int) * s->nd));
  TCK(cudaMemcpyAsync(G->gap_d.p, G->gap_of.data(), sizeof(int) * s->nd, cudaMemcpyHostToDevice, st));
  TCKS(G->solid.alloc(h, sizeof(double2) * nf * s->nd * nm2));
  TCKS(G->coef.alloc(h, sizeof(double2) * (size_t)G->ngap * nf * (nsp + 2) * nm2));
  // Thomas factors of the prefilter matrix (k_pgrid_prefilter): rows
  // (3, -1), (1, 4, 1) ..., (-1, 3); m_k = b_k - a_k c'_{k-1}, c'_k = u_k / m_k
  std::vector<double> th(2 * (nsp + 2), 0.0);
  double cp = 0.0;
  for (int k = 1; k <= nsp; ++k) {
    const double a = (k == 1) ? 0.0 : (k == nsp ? -1.0 : 1.0);
    const double b = (k == 1 || k == nsp) ? 3.0 : 4.0;
    const double u = (k == 1) ? -1.0 : (k == nsp ? 0.0 : 1.0);
    const double m = b - a * cp;
    th[k] = 1.0 / m;
    cp = u / m;
    th[(nsp + 2) + k] = cp;
  }
  TCKS(G->thomas.alloc(h, sizeof(double) * th.size()));
  TCK(cudaMemcpyAsync(G->thomas.p, th.data(), sizeof(double) * th.size(), cudaMemcpyHostToDevice, st));
  G->precision = precision;
  if (precision == BF_PREC_FP64) TCKS(pgrid_fill<double2>(h, G.get(), prop_kind, 0));
  else TCKS(pgrid_fill<float2>(h, G.get(), prop_kind, 1));
  G->emit.resize(G->nm);
  TCKS(bf_axion_induced_modes(h, md, nullptr, 0.0, s->diskR, 10e9, reinterpret_cast<double*>(G->emit.data())));
  const size_t nseq = (size_t)G->ngap * nf;
  bf::note_launch();
  k_pgrid_prefilter<<<blocks_for(nseq * nm2), 256, 0, st>>>(G->coef.as<double2>(), G->thomas.as<double>(), (int)nseq,
                                                           (int)nm2, nsp);
  TCK(cudaGetLastError());
  TCK(cudaStreamSynchronize(st));
  *out = G.release();
  return BF_OK;
}

void bf_pgrid_shape(const bf_pgrid* g, int* nf, int* nd, int* nm, bf_stack** stack) {
  *nf = g->nf;
  *nd = g->nd;
  *nm = g->nm;
  *stack = g->s;
}

extern "C" int bf_pgrid_destroy(bf_handle* h, bf_pgrid* g) {
  if (!h || !g) return BF_ERR_INVALID;
  cudaStreamSynchronize(h->stream());
  delete g;
  return BF_OK;
}

// Interpolated matrices into a device buffer [nf][nd][nm][nm] (row-major).
static int pgrid_eval(bf_handle* h, bf_pgrid* G, const double* dist_shift, DBuf& P) {
  std::vector<double> x(G->nd, 0.0);
  // the domain of an OnCell interpolation: half a step beyond the first and last spacing
  const double lo = G->s0 - 0.5 * G->ds, hi = G->s0 + (G->nsp - 0.5) * G->ds;
  for (int j = 0; j < G->nd; ++j) {
    if (G->gap_of[j] < 0) continue;
    // the last region keeps shift 0, as interpolate_prop_matrix does (utilities :84)
    const double sh = (j == G->nd - 1) ? 0.0 : dist_shift[(j - 1) / 2];
    if (!std::isfinite(sh) || sh < lo - 1e-12 * G->ds || sh > hi + 1e-12 * G->ds)
      return bf_fail(h, BF_ERR_INVALID, "pgrid: a shift lies outside the spacing grid [" + std::to_string(lo) +
                                            ", " + std::to_string(hi) + "]");
    x[j] = std::min(std::max(1.0 + (sh - G->s0) / G->ds, 0.5), G->nsp + 0.5);
  }
  cudaStream_t st = h->stream();
  const size_t nm2 = (size_t)G->nm * G->nm, n = (size_t)G->nf * G->nd * nm2;
  DBuf dx;
  TCKS(dx.alloc(h, sizeof(double) * G->nd));
  TCK(cudaMemcpyAsync(dx.p, x.data(), sizeof(double) * G->nd, cudaMemcpyHostToDevice, st));
  TCKS(P.ensure(h, sizeof(double2) * n));
  bf::note_launch();
  k_pgrid_eval<<<blocks_for(n), 256, 0, st>>>(P.as<double2>(), G->solid.as<double2>(), G->coef.as<double2>(),
                                             G->gap_d.as<int>(), dx.as<double>(), G->nf, G->nd, (int)nm2, G->nsp);
  TCK(cudaGetLastError());
  TCK(cudaStreamSynchronize(st));   // x (host) and dx may go once the kernel has read them
  return BF_OK;
}

extern "C" int bf_pgrid_matrices(bf_handle* h, bf_pgrid* G, const double* dist_shift, double* out) {
  if (!h || !G || !dist_shift || !out) return BF_ERR_INVALID;
  TCK(cudaSetDevice(h->device));
  DBuf P;
  TCKS(pgrid_eval(h, G, dist_shift, P));
  const size_t nm = G->nm, n = (size_t)G->nf * G->nd * nm * nm;
  std::vector<double2> hp(n);
  TCK(cudaMemcpy(hp.data(), P.p, sizeof(double2) * n, cudaMemcpyDeviceToHost));
  cd* o = reinterpret_cast<cd*>(out);
  for (size_t fj = 0; fj < (size_t)G->nf * G->nd; ++fj)
    for (size_t r = 0; r < nm; ++r)
      for (size_t q = 0; q < nm; ++q) {
        const double2 v = hp[(fj * nm + r) * nm + q];
        o[fj * nm * nm + r + nm * q] = cd(v.x, v.y);
      }
  return BF_OK;
}

static int pgrid_solve(bf_handle* h, bf_pgrid* G, const double* dist_shift, const double* emit, double* out_boost,
                       double* out_beta2, const CoupleArgs* cp) {
  DBuf P;
  TCKS(pgrid_eval(h, G, dist_shift, P));
  const double* em = emit ? emit : reinterpret_cast<const double*>(G->emit.data());
  if (G->precision == BF_PREC_FP64)
    return tf_run_t<double2>(h, G->s, G->md, G->nf, G->freqs.data(), BF_PROP_3D, em, nullptr, nullptr, 0,
                             out_boost, nullptr, out_beta2, 1, 0, nullptr, 0, nullptr, cp, P.as<double2>());
  // mixed grid: complex64 matrices, double-float chain, FP64 boundary solve
  const size_t n = (size_t)G->nf * G->nd * G->nm * G->nm;
  DBuf P32;
  TCKS(P32.alloc(h, sizeof(float2) * n));
  if (bf::launch_convert(P.p, true, P32.p, false, n, h->stream())) return bf_fail(h, BF_ERR_CUDA, "convert");
  return tf_run_t<float2>(h, G->s, G->md, G->nf, G->freqs.data(), BF_PROP_3D, em, nullptr, nullptr, 0, out_boost,
                          nullptr, out_beta2, 1, 0, nullptr, 1, nullptr, cp, P32.as<float2>());
}

extern "C" int bf_pgrid_transformer(bf_handle* h, bf_pgrid* G, const double* dist_shift, const double* emit,
                                    double* out_boost, double* out_beta2) {
  if (!h || !G || !dist_shift || (!out_boost && !out_beta2)) return BF_ERR_INVALID;
  TCK(cudaSetDevice(h->device));
  return pgrid_solve(h, G, dist_shift, emit, out_boost, out_beta2, nullptr);
}

// soft_box_penalty (utilities :150-160): 1 - (excess / depth)^6, the excess of
// the largest of the shifts and their sum over the upper soft bound (or of the
// lower soft bound over the smallest), depth 5 % of the box
static double soft_box_penalty(const double* shift, int n, double lo, double hi) {
  const double depth = (hi - lo) * 0.05, l = lo + depth, u = hi - depth;
  double mx = -INFINITY, mn = INFINITY, sum = 0.0;
  for (int k = 0; k < n; ++k) {
    mx = std::max(mx, shift[k]);
    mn = std::min(mn, shift[k]);
    sum += shift[k];
  }
  mx = std::max(mx, sum);
  mn = std::min(mn, sum);
  const double excess = std::max(std::max(mx - u, -(mn - l)), 0.0);
  return 1.0 - std::pow(excess / depth, 6);
}

// p_norm (utilities :211-215): max(X) (mean((X / max X)^p))^(1/p)
static double p_norm(const double* x, int n, double p) {
  double mag = -INFINITY;
  for (int k = 0; k < n; ++k) mag = std::max(mag, x[k]);
  double acc = 0.0;
  for (int k = 0; k < n; ++k) acc += std::pow(x[k] / mag, p);
  return mag * std::pow(acc / n, 1.0 / p);
}

extern "C" int bf_pgrid_cost(bf_handle* h, bf_pgrid* G, const double* dist_shift, const double* m_reflect, double p,
                             double* out_cost, double* out_coupled) {
  if (!h || !G || !dist_shift || !m_reflect || !out_cost) return BF_ERR_INVALID;
  if (!std::isfinite(p) || p == 0.0) return bf_fail(h, BF_ERR_INVALID, "pgrid cost: p must be finite and non-zero");
  TCK(cudaSetDevice(h->device));
  const int ndisk = G->ngap - 1;
  const double lo = G->s0 - 0.5 * G->ds, hi = G->s0 + (G->nsp - 0.5) * G->ds;
  // hard penalty outside the interpolation bounds (utilities :131-135)
  for (int k = 0; k < ndisk; ++k)
    if (!(lo < dist_shift[k] && dist_shift[k] < hi)) {
      *out_cost = 1000.0;
      return BF_OK;
    }
  const double penalty = soft_box_penalty(dist_shift, ndisk, lo, hi);
  std::vector<double> cpl(G->nf);
  CoupleArgs cp{m_reflect, cpl.data()};
  TCKS(pgrid_solve(h, G, dist_shift, nullptr, nullptr, nullptr, &cp));
  if (out_coupled) std::memcpy(out_coupled, cpl.data(), sizeof(double) * G->nf);
  *out_cost = -p_norm(cpl.data(), G->nf, p) * penalty;
  return BF_OK;
}
