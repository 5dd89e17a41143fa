// Device kernels of the GB300 boost-factor library.
//
// * k_fused_stage   -- the hot path: one launch runs one bounce stage of the
//   recursive Fourier propagation for every frequency of a batch.  Each CTA
//   propagates one or two region fields through the angular-spectrum
//   propagator (src/boost_fractor.jl:137-179) and applies the boundary's
//   reflection/transmission (src/boost_fractor_recurprop.jl:90-120, 310-345)
//   in its epilogue.  Fields are stored only on the pruned box of pixels the
//   disk mask can reach; the 2D FFT is separable, so the forward row pass,
//   the fused column pass (FFT, phasor, inverse FFT) and the inverse row pass
//   each touch only the lines that can be non-zero or are needed.
// * phasor / tilt table kernels -- FP64 phase arguments, stored in the field
//   precision.
// * general full-grid path -- any grid size (also odd sizes like 101), used
//   for the per-op propagator, the exit fields and the exact (unpruned) mode.
// * 1D-propagator solvers -- every pixel is independent.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>

#include <algorithm>
#include <vector>

#include "bf_common.cuh"
#include "bf_device.cuh"
#include "bf_fft.cuh"

namespace bf {

// Kernel launches made by the calling host thread (one handle's call runs on
// one thread, so per-call differences are exact even with several handles
// working concurrently).
static thread_local unsigned long long g_launches = 0;
unsigned long long launch_count() { return g_launches; }
void note_launch() { ++g_launches; }
void note_launches(unsigned long long n) { g_launches += n; }
void unnote_launches(unsigned long long n) { g_launches -= n; }
#define COUNT_LAUNCH() (++g_launches)

// Round an FP64 complex value to complex64 so that the modulus error is as
// small as possible: of the float pairs within one ulp of (re, im) take the one
// whose squared modulus is closest to the FP64 one.  Plain rounding leaves a
// random modulus error of ~6e-8 per value, and a phasor or twiddle that is
// applied to the same k-bin on every bounce turns that into a systematic gain
// or loss that compounds over hundreds of bounces.
__host__ __device__ inline float2 round_c64_host_device(double re, double im) {
  const float fr = (float)re, fi = (float)im;
  const double m2 = re * re + im * im;
  float best_r = fr, best_i = fi;
  double best = 1e300;
  for (int a = -1; a <= 1; ++a)
    for (int b = -1; b <= 1; ++b) {
      float cr = a == 0 ? fr : nextafterf(fr, a > 0 ? INFINITY : -INFINITY);
      float ci = b == 0 ? fi : nextafterf(fi, b > 0 ? INFINITY : -INFINITY);
      double d = fabs((double)cr * cr + (double)ci * ci - m2);
      // prefer the plain rounding on ties (keeps exact values exact)
      if (d < best || (d == best && a == 0 && b == 0)) {
        best = d;
        best_r = cr;
        best_i = ci;
      }
    }
  return make_float2(best_r, best_i);
}

void init_constant_roots() {
  static double2 hd[1024];
  static float2 hf[1024];
  for (int k = 0; k < 1024; ++k) {
    // exp(-2 pi i k / 1024); cos/sin evaluated on the first octant and mapped
    // by symmetry so that the table is exactly symmetric
    int q = k / 256, r = k % 256;
    double c, s;
    int rr = r <= 128 ? r : 256 - r;
    double a = M_PI * rr / 512.0;
    double cr = cos(a), sr = sin(a);
    if (r > 128) { double t = cr; cr = sr; sr = t; }
    // float copy of the first-octant pair, rounded for the smallest modulus error,
    // then mapped by the same exact symmetry as the FP64 pair
    const float2 o = round_c64_host_device(cr, sr);
    float cf, sf;
    // angle theta = 2 pi k / 1024 = q*pi/2 + 2 pi r/1024; (cos, sin) of theta
    switch (q) {
      case 0: c = cr; s = sr; cf = o.x; sf = o.y; break;
      case 1: c = -sr; s = cr; cf = -o.y; sf = o.x; break;
      case 2: c = -cr; s = -sr; cf = -o.x; sf = -o.y; break;
      default: c = sr; s = -cr; cf = o.y; sf = -o.x; break;
    }
    hd[k] = make_double2(c, -s);
    hf[k] = make_float2(cf, -sf);
  }
  cudaMemcpyToSymbol(c_root1024_d, hd, sizeof(hd));
  cudaMemcpyToSymbol(c_root1024_f, hf, sizeof(hf));
}

// ---------------------------------------------------------------------------
// small FP64 complex helpers (phase arguments are always FP64)
// ---------------------------------------------------------------------------
__device__ __forceinline__ double2 dcsqrt(double x, double y) {
  // principal square root honouring the sign of a zero imaginary part, so that
  // sqrt(a - 0.0im) = 0 - sqrt(|a|)im for a < 0 (evanescent bins decay)
  if (x == 0.0 && y == 0.0) return make_double2(0.0, y);
  // a zero imaginary part (real permittivities): with hypot(x, 0) = |x| the
  // general formula below reduces to these values in exact arithmetic; they
  // skip hypot and the division (FP64 runs at 1/64 of the FP32 rate)
  if (y == 0.0) return x > 0.0 ? make_double2(sqrt(x), y) : make_double2(0.0, copysign(sqrt(-x), y));
  double t = sqrt((fabs(x) + hypot(x, y)) * 0.5);
  if (x >= 0.0) return make_double2(t, y / (2.0 * t));
  return make_double2(fabs(y) / (2.0 * t), copysign(t, y));
}
__device__ __forceinline__ double2 dcexp(double re, double im) {
  double s, c;
  sincos(im, &s, &c);
  if (re == 0.0) return make_double2(c, s);   // exp(0) = 1 exactly (propagating bins)
  double m = exp(re);
  return make_double2(m * c, m * s);
}
// k0 = 2 pi / lambda * sqrt(eps), eps real -> re - 0.0im (src/boost_fractor.jl:140,:161)
__device__ __forceinline__ double2 k0_of(double lambda, double eps_re, double eps_im) {
  if (eps_im == 0.0) eps_im = -0.0;
  double2 s = dcsqrt(eps_re, eps_im);
  double c = 2.0 * M_PI / lambda;
  return make_double2(c * s.x, c * s.y);
}
// exp(-1im * sqrt(k0^2 - kx^2 - ky^2) * dz)
__device__ __forceinline__ double2 phasor_value(double2 k0, double kx, double ky, double dz) {
  double2 k0sq = make_double2(k0.x * k0.x - k0.y * k0.y, k0.x * k0.y + k0.y * k0.x);
  double re = (k0sq.x - kx * kx) - ky * ky;
  double2 kz = dcsqrt(re, k0sq.y);
  // -1im * kz * dz = (kz.y * dz, -kz.x * dz)
  return dcexp(kz.y * dz, -kz.x * dz);
}
// exp(-1im * k0 * t) for complex k0 and real t
__device__ __forceinline__ double2 phase_k0(double2 k0, double t) {
  return dcexp(k0.y * t, -k0.x * t);
}
// exp(-1im * k0 * s) for complex k0 and complex s
__device__ __forceinline__ double2 phase_k0c(double2 k0, double2 s) {
  double re = k0.x * s.x - k0.y * s.y, im = k0.x * s.y + k0.y * s.x;
  return dcexp(im, -re);
}

template <typename C> __device__ __forceinline__ C from_d(double2 v);
template <> __device__ __forceinline__ float2 from_d<float2>(double2 v) {
  return make_float2((float)v.x, (float)v.y);
}
template <> __device__ __forceinline__ double2 from_d<double2>(double2 v) { return v; }
// phase factors: modulus-aware rounding to complex64
template <typename C> __device__ __forceinline__ C from_d_phase(double2 v);
template <> __device__ __forceinline__ float2 from_d_phase<float2>(double2 v) {
  return round_c64_host_device(v.x, v.y);
}
template <> __device__ __forceinline__ double2 from_d_phase<double2>(double2 v) { return v; }
template <typename C> __device__ __forceinline__ C czero() { return from_d<C>(make_double2(0.0, 0.0)); }

#define SPEED_OF_LIGHT 299792458.0

// ---------------------------------------------------------------------------
// Fused box stage kernel
// ---------------------------------------------------------------------------
constexpr int kFusedThreads = 256;
constexpr int kSmemHeader = 128;

template <int N> __host__ __device__ constexpr int fused_pitch() { return N + 2; }

// Kernel-shape options of the fused stage (a bit mask): the inter-pass
// twiddles from a shared table instead of registers; team exchanges in two
// halves through half-size scratch; each column task's folded phasor row
// copied into the team's shared buffer (cp.async) while the team runs the
// forward transform, instead of loaded from L2 after it.  None changes the
// arithmetic.
constexpr int kModeTwShared = 1, kModeHalf = 2, kModeStage = 4;

// Complex elements of one team's shared region: its exchange scratch, then
// (kModeStage) the N/2-entry phasor row buffer.
template <int N, int MODE> __host__ __device__ constexpr int team_region() {
  return Team<N>::template scratch<(MODE & kModeHalf) != 0>() + ((MODE & kModeStage) ? N / 2 : 0);
}

__device__ __forceinline__ void cp_async16(void* dst_smem, const void* src_global) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((unsigned)__cvta_generic_to_shared(dst_smem)),
               "l"(src_global)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

template <typename C, int N>
struct FusedCtx {
  using T = Team<N>;
  static constexpr int G = T::G, RR = T::RR, CC = T::C;
  static constexpr int P = fused_pitch<N>();
};

// Phase 1 of one propagation: forward FFT along x of every box row.  Fields
// are stored pre-masked, so only register slots r < ceil(nbx/G) can hold box
// pixels.  A slot feeding an exit adds its (masked) input to the FP64 exit
// accumulator on the way.
template <typename C, int N, int NZ, int NT, bool HALF = false>
__device__ __forceinline__ void fused_phase1(const FusedArgs<C>& a, int f, int slot, int exitk, C* M,
                                             C* scr, const C* tw, int team, int g) {
  using X = FusedCtx<C, N>;
  constexpr int G = X::G, RR = X::RR, CC = X::CC, P = X::P;
  constexpr int NTEAM = NT;
  const int nbx = a.nbx, nby = a.nby;
  const C* src = a.state + ((size_t)f * a.nslots + slot) * (size_t)(nby * nbx);
  double2* acc = exitk >= 0 ? a.exitacc + ((size_t)exitk * a.nfreq + f) * (size_t)(nby * nbx) : nullptr;
  const int rv = (nbx + G - 1) / G;
  for (int base = 0; base < nby; base += NTEAM) {
    const int y = base + team;
    const bool act = y < nby;
    if (!__any_sync(0xffffffffu, act)) continue;   // the whole warp is idle
    const C* row = src + y * nbx;
    double2* arow = acc ? acc + y * nbx : nullptr;
    C v[RR];
#pragma unroll
    for (int r = 0; r < RR; ++r) {
      v[r] = czero<C>();
      if (r < NZ && r < rv) {
        const int x = g + G * r;
        if (act && x < nbx) {
          const C val = row[x];
          v[r] = val;
          if (arow) {
            double2 o = arow[x];
            double2 d = to_d(val);
            arow[x] = make_double2(o.x + d.x, o.y + d.y);
          }
        }
      }
    }
    X::T::template forward<NZ, HALF>(v, tw, scr, g);
    if (act) {
#pragma unroll
      for (int j = 0; j < CC; ++j)
#pragma unroll
        for (int q = 0; q < G; ++q) M[y * P + g * CC + j + RR * q] = v[j * G + q];
    }
  }
  __syncthreads();
}

// Phase 2: per column kx, forward FFT along y, phasor, inverse FFT along y,
// in place in M (only the nby box rows are read and written).  STAGE: the
// column's folded phasor row is copied into the team's buffer behind its
// scratch (cp.async, issued before the forward transform) and read from there.
template <typename C, int N, int NZ, int NT, bool HALF = false, bool STAGE = false>
__device__ __forceinline__ void fused_phase2(const FusedArgs<C>& a, const C* Q, C* M, C* scr,
                                             const C* tw, int team, int g) {
  using X = FusedCtx<C, N>;
  constexpr int G = X::G, RR = X::RR, CC = X::CC, P = X::P;
  constexpr int NTEAM = NT;
  const int nby = a.nby;
  const int QW = a.fold ? N / 2 : N;
  const int rv = (nby + G - 1) / G;
  C* qb = STAGE ? scr + X::T::template scratch<HALF>() : nullptr;
  for (int base = 0; base < N; base += NTEAM) {
    const int kx = base + team;
    const bool act = kx < N;
    if (!__any_sync(0xffffffffu, act)) continue;
    if constexpr (STAGE) {
      if (act && a.fold) {
        constexpr int E = 16 / sizeof(C);   // elements per 16-byte chunk
        const C* row = Q + (size_t)(kx < N / 2 ? kx : N - 1 - kx) * QW;
        for (int c = g; c < (N / 2) / E; c += G) cp_async16(qb + c * E, row + c * E);
      }
      cp_async_commit();
    }
    C v[RR];
#pragma unroll
    for (int r = 0; r < RR; ++r) {
      v[r] = czero<C>();
      if (r < NZ && r < rv) {
        const int y = g + G * r;
        if (act && y < nby) v[r] = M[y * P + kx];
      }
    }
    X::T::template forward<NZ, HALF>(v, tw, scr, g);
    if constexpr (STAGE) {
      cp_async_wait_all();
      __syncwarp();
    }
    if (act) {
      if (a.fold) {
        // bins k and N-1-k share a phasor; ky = g*CC + j + RR*q < N/2 exactly when q < G/2
        const C* Qrow = STAGE ? qb : Q + (size_t)(kx < N / 2 ? kx : N - 1 - kx) * QW;
#pragma unroll
        for (int j = 0; j < CC; ++j)
#pragma unroll
          for (int q = 0; q < G; ++q) {
            const int ky = g * CC + j + RR * q;
            v[j * G + q] = cmul(v[j * G + q], Qrow[q < G / 2 ? ky : N - 1 - ky]);
          }
      } else {
        const C* Qrow = Q + (size_t)kx * QW;
#pragma unroll
        for (int j = 0; j < CC; ++j)
#pragma unroll
          for (int q = 0; q < G; ++q) v[j * G + q] = cmul(v[j * G + q], Qrow[g * CC + j + RR * q]);
      }
    }
    // (the inverse's exchange syncs the warp: every lane has read the buffer
    // before the next task's copies overwrite it)
    X::T::template inverse<HALF>(v, tw, scr, g);
    if (act) {
#pragma unroll
      for (int r = 0; r < RR; ++r) {
        if (r < NZ && r < rv) {
          const int y = g + G * r;
          if (y < nby) M[y * P + kx] = v[r];
        }
      }
    }
  }
  __syncthreads();
}

// Phase 3: inverse FFT along x of every box row, tilt/surface map, then the
// epilogue: store the propagated field into obuf (first of two propagations)
// or apply the boundary mix and write the new (masked) fields.
template <typename C, int N, bool MIX, int NZ, int NT, bool HALF = false>
__device__ __forceinline__ void fused_phase3(const FusedArgs<C>& a, const StepDesc& sd, int f, int region,
                                             bool prop_is_b, C* M, C* scr, C* obuf,
                                             const C* tw, int team, int g) {
  using X = FusedCtx<C, N>;
  constexpr int G = X::G, RR = X::RR, CC = X::CC, P = X::P;
  constexpr int NTEAM = NT;
  const int nbx = a.nbx, nby = a.nby;
  const size_t plane = (size_t)nby * nbx;
  const int ti = a.tilt_idx[region];
  const C* tmap = ti >= 0 ? a.tilt + ((size_t)f * a.ntilt + ti) * plane : nullptr;
  C* stA = sd.sa >= 0 ? a.state + ((size_t)f * a.nslots + sd.sa) * plane : nullptr;
  C* stB = sd.sb >= 0 ? a.state + ((size_t)f * a.nslots + sd.sb) * plane : nullptr;
  const C* add = (MIX && sd.addA >= 0) ? a.addbuf + (size_t)sd.addA * plane : nullptr;
  const int rv = (nbx + G - 1) / G;
  C cAA, cAB, cBA, cBB;
  if (MIX) {
    const double2* cf = a.coefs + 4 * sd.coef;
    cAA = from_d<C>(cf[0]); cAB = from_d<C>(cf[1]); cBA = from_d<C>(cf[2]); cBB = from_d<C>(cf[3]);
  }
  for (int base = 0; base < nby; base += NTEAM) {
    const int y = base + team;
    const bool act = y < nby;
    if (!__any_sync(0xffffffffu, act)) continue;
    C v[RR];
#pragma unroll
    for (int j = 0; j < CC; ++j)
#pragma unroll
      for (int q = 0; q < G; ++q) v[j * G + q] = act ? M[y * P + g * CC + j + RR * q] : czero<C>();
    X::T::template inverse<HALF>(v, tw, scr, g);
    if (!act) continue;
#pragma unroll
    for (int r = 0; r < RR; ++r) {
      if (r >= NZ || r >= rv) continue;
      const int x = g + G * r;
      if (x >= nbx) continue;
      const int i = y * nbx + x;
      C p = v[r];
      if (tmap) p = cmul(p, tmap[i]);
      if (!MIX) {
        obuf[i] = p;
      } else {
        // new fields are stored masked (their next propagation masks them anyway)
        const bool in = a.mask[i] != 0;
        C tA, tB;
        if (prop_is_b) {
          tB = p;
          if (sd.ra >= 0) tA = obuf[i];
          else tA = stA ? stA[i] : czero<C>();
        } else {
          tA = p;
          tB = stB ? stB[i] : czero<C>();
        }
        if (stA) {
          C o = cadd(cmul(cAA, tA), cmul(cAB, tB));
          if (add) o = cadd(o, add[i]);
          stA[i] = in ? o : czero<C>();
        }
        if (stB) stB[i] = in ? cadd(cmul(cBA, tA), cmul(cBB, tB)) : czero<C>();
      }
    }
  }
}

// ---- joint step: both slots processed together ------------------------------
// The rows of A and of B form one task list (2 nby rows), and so do their
// columns (2 N), so the teams stay busy where a single field's nby rows leave
// most of them idle in the last round; the propagated fields stay in the row
// tiles MA, MB and the boundary mix runs as one pass over the box.  A team
// takes the tasks t0 + team, t0 + team + ts, ... (the fused kernel: t0 = 0,
// ts = its teams; the split-phase kernels spread the tasks over CTAs); the
// tasks of a slot that is not propagated (pa / pb false) are skipped.

// Phase 1, joint: forward FFT along x of the box rows of A (tasks < nby) and B.
template <typename C, int N, int NZ, int NT, bool SPLIT, bool HALF = false>
__device__ __forceinline__ void joint_phase1(const FusedArgs<C>& a, const StepDesc& sd, int f, C* MA, C* MB,
                                             C* scr, const C* tw, int team, int g, int t0, int ts,
                                             bool pa, bool pb) {
  using X = FusedCtx<C, N>;
  constexpr int G = X::G, RR = X::RR, CC = X::CC, P = X::P;
  const int nbx = a.nbx, nby = a.nby, ntask = 2 * nby;
  const int rv = (nbx + G - 1) / G;
  // the fused kernel's joint steps: all tasks of the CTA, both slots propagated
  const int T0 = SPLIT ? t0 : 0, TS = SPLIT ? ts : NT;
  for (int base = T0; base < ntask; base += TS) {
    const int t = base + team;
    const bool act = t < ntask && (!SPLIT || (t >= nby ? pb : pa));
    if (!__any_sync(0xffffffffu, act)) continue;
    const bool isb = act && t >= nby;
    const int y = act ? (isb ? t - nby : t) : 0;
    const int slot = isb ? sd.sb : sd.sa, exitk = isb ? sd.exitB : sd.exitA;
    const C* row = a.state + (((size_t)f * a.nslots + slot) * nby + y) * (size_t)nbx;
    double2* arow = exitk >= 0 ? a.exitacc + (((size_t)exitk * a.nfreq + f) * nby + y) * (size_t)nbx : nullptr;
    C v[RR];
#pragma unroll
    for (int r = 0; r < RR; ++r) {
      v[r] = czero<C>();
      if (r < NZ && r < rv) {
        const int x = g + G * r;
        if (act && x < nbx) {
          const C val = row[x];
          v[r] = val;
          if (arow) {
            double2 o = arow[x];
            double2 d = to_d(val);
            arow[x] = make_double2(o.x + d.x, o.y + d.y);
          }
        }
      }
    }
    X::T::template forward<NZ, HALF>(v, tw, scr, g);
    if (act) {
      C* M = isb ? MB : MA;
#pragma unroll
      for (int j = 0; j < CC; ++j)
#pragma unroll
        for (int q = 0; q < G; ++q) M[y * P + g * CC + j + RR * q] = v[j * G + q];
    }
  }
  __syncthreads();
}

// Ask L2 for the phasor row of column task t (rows of 128-byte lines, one per
// thread g of the team), so that it is there when the team reaches that task.
// QA / QB are null for a slot that is not propagated.
template <typename C, int N, bool MAYBE_NULL>
__device__ __forceinline__ void prefetch_qrow(const FusedArgs<C>& a, const C* QA, const C* QB, int t, int g) {
  if (t >= 2 * N) return;
  const int QW = a.fold ? N / 2 : N;
  const int kx = t < N ? t : t - N;
  const C* Q = t < N ? QA : QB;
  if (MAYBE_NULL && !Q) return;
  const C* row = Q + (size_t)(a.fold ? (kx < N / 2 ? kx : N - 1 - kx) : kx) * QW;
  const int lines = (int)((sizeof(C) * QW + 127) / 128);
  if (g < lines) asm volatile("prefetch.global.L2 [%0];" ::"l"(reinterpret_cast<const char*>(row) + 128 * g));
}

// Phase 2, joint: columns of A (tasks < N) and of B, each with its region's phasor.
// STAGE as fused_phase2 (the fused kernel only).
template <typename C, int N, int NZ, int NT, bool SPLIT, bool HALF = false, bool STAGE = false>
__device__ __forceinline__ void joint_phase2(const FusedArgs<C>& a, const C* QA, const C* QB, C* MA, C* MB, C* scr,
                                             const C* tw, int team, int g, int t0, int ts) {
  using X = FusedCtx<C, N>;
  constexpr int G = X::G, RR = X::RR, CC = X::CC, P = X::P;
  static_assert(!(SPLIT && STAGE), "staged phasor rows: fused kernel only");
  const int nby = a.nby;
  const int QW = a.fold ? N / 2 : N;
  const int rv = (nby + G - 1) / G;
  const int T0 = SPLIT ? t0 : 0, TS = SPLIT ? ts : NT;
  C* qb = STAGE ? scr + X::T::template scratch<HALF>() : nullptr;
  for (int base = T0; base < 2 * N; base += TS) {
    const int t = base + team;
    const bool act = t < 2 * N && (!SPLIT || (t >= N ? QB : QA) != nullptr);
    if (!__any_sync(0xffffffffu, act)) continue;
    const bool isb = act && t >= N;
    const int kx = act ? (isb ? t - N : t) : 0;
    C* M = isb ? MB : MA;
    const C* Q = isb ? QB : QA;
    if constexpr (STAGE) {
      if (act && a.fold) {
        constexpr int E = 16 / sizeof(C);   // elements per 16-byte chunk
        const C* row = Q + (size_t)(kx < N / 2 ? kx : N - 1 - kx) * QW;
        for (int c = g; c < (N / 2) / E; c += G) cp_async16(qb + c * E, row + c * E);
      }
      cp_async_commit();
      if (!a.fold) prefetch_qrow<C, N, SPLIT>(a, QA, QB, t + TS, g);
    } else {
      prefetch_qrow<C, N, SPLIT>(a, QA, QB, t + TS, g);
    }
    C v[RR];
#pragma unroll
    for (int r = 0; r < RR; ++r) {
      v[r] = czero<C>();
      if (r < NZ && r < rv) {
        const int y = g + G * r;
        if (act && y < nby) v[r] = M[y * P + kx];
      }
    }
    X::T::template forward<NZ, HALF>(v, tw, scr, g);
    if constexpr (STAGE) {
      cp_async_wait_all();
      __syncwarp();
    }
    if (act) {
      if (a.fold) {
        const C* Qrow = STAGE ? qb : Q + (size_t)(kx < N / 2 ? kx : N - 1 - kx) * QW;
#pragma unroll
        for (int j = 0; j < CC; ++j)
#pragma unroll
          for (int q = 0; q < G; ++q) {
            const int ky = g * CC + j + RR * q;
            v[j * G + q] = cmul(v[j * G + q], Qrow[q < G / 2 ? ky : N - 1 - ky]);
          }
      } else {
        const C* Qrow = Q + (size_t)kx * QW;
#pragma unroll
        for (int j = 0; j < CC; ++j)
#pragma unroll
          for (int q = 0; q < G; ++q) v[j * G + q] = cmul(v[j * G + q], Qrow[g * CC + j + RR * q]);
      }
    }
    // (the inverse's exchange syncs the warp before the buffer is refilled)
    X::T::template inverse<HALF>(v, tw, scr, g);
    if (act) {
#pragma unroll
      for (int r = 0; r < RR; ++r) {
        if (r < NZ && r < rv) {
          const int y = g + G * r;
          if (y < nby) M[y * P + kx] = v[r];
        }
      }
    }
  }
  __syncthreads();
}

// Phase 3, joint: inverse FFT along x of the box rows of A and B, times the
// region's tilt/surface map, written back in place into the row's first nbx
// entries (the team's exchange has already consumed the row).
template <typename C, int N, int NZ, int NT, bool SPLIT, bool HALF = false>
__device__ __forceinline__ void joint_phase3(const FusedArgs<C>& a, const StepDesc& sd, int f, C* MA, C* MB,
                                             C* scr, const C* tw, int team, int g, int t0, int ts,
                                             bool pa, bool pb) {
  using X = FusedCtx<C, N>;
  constexpr int G = X::G, RR = X::RR, CC = X::CC, P = X::P;
  const int nbx = a.nbx, nby = a.nby, ntask = 2 * nby;
  const size_t plane = (size_t)nby * nbx;
  const int tiA = (!SPLIT || pa) ? a.tilt_idx[sd.ra] : -1, tiB = (!SPLIT || pb) ? a.tilt_idx[sd.rb] : -1;
  const C* tA = tiA >= 0 ? a.tilt + ((size_t)f * a.ntilt + tiA) * plane : nullptr;
  const C* tB = tiB >= 0 ? a.tilt + ((size_t)f * a.ntilt + tiB) * plane : nullptr;
  const int rv = (nbx + G - 1) / G;
  const int T0 = SPLIT ? t0 : 0, TS = SPLIT ? ts : NT;
  for (int base = T0; base < ntask; base += TS) {
    const int t = base + team;
    const bool act = t < ntask && (!SPLIT || (t >= nby ? pb : pa));
    if (!__any_sync(0xffffffffu, act)) continue;
    const bool isb = act && t >= nby;
    const int y = act ? (isb ? t - nby : t) : 0;
    C* M = isb ? MB : MA;
    const C* tmap = isb ? tB : tA;
    C v[RR];
#pragma unroll
    for (int j = 0; j < CC; ++j)
#pragma unroll
      for (int q = 0; q < G; ++q) v[j * G + q] = act ? M[y * P + g * CC + j + RR * q] : czero<C>();
    X::T::template inverse<HALF>(v, tw, scr, g);
    if (!act) continue;
#pragma unroll
    for (int r = 0; r < RR; ++r) {
      if (r >= NZ || r >= rv) continue;
      const int x = g + G * r;
      if (x >= nbx) continue;
      C p = v[r];
      if (tmap) p = cmul(p, tmap[y * nbx + x]);
      M[y * P + x] = p;
    }
  }
  __syncthreads();
}

// Boundary mix of a step over the box: A' = cAA A~ + cAB B~ (+ add),
// B' = cBA A~ + cBB B~, stored masked; X~ is the propagated field (row tile)
// of a propagated slot, else the slot's stored field.  Pixels i0, i0 + is, ...
template <typename C, int N>
__device__ __forceinline__ void joint_mix(const FusedArgs<C>& a, const StepDesc& sd, int f, const C* MA,
                                          const C* MB, bool pa, bool pb, int i0, int is) {
  constexpr int P = FusedCtx<C, N>::P;
  const int nbx = a.nbx, nby = a.nby;
  const size_t plane = (size_t)nby * nbx;
  C* stA = sd.sa >= 0 ? a.state + ((size_t)f * a.nslots + sd.sa) * plane : nullptr;
  C* stB = sd.sb >= 0 ? a.state + ((size_t)f * a.nslots + sd.sb) * plane : nullptr;
  const C* add = sd.addA >= 0 ? a.addbuf + (size_t)sd.addA * plane : nullptr;
  const double2* cf = a.coefs + 4 * sd.coef;
  const C cAA = from_d<C>(cf[0]), cAB = from_d<C>(cf[1]), cBA = from_d<C>(cf[2]), cBB = from_d<C>(cf[3]);
  for (int i = i0; i < (int)plane; i += is) {
    const int y = i / nbx, x = i - y * nbx;
    const C A = pa ? MA[y * P + x] : (stA ? stA[i] : czero<C>());
    const C B = pb ? MB[y * P + x] : (stB ? stB[i] : czero<C>());
    const bool in = a.mask[i] != 0;
    if (stA) {
      C o = cadd(cmul(cAA, A), cmul(cAB, B));
      if (add) o = cadd(o, add[i]);
      stA[i] = in ? o : czero<C>();
    }
    if (stB) stB[i] = in ? cadd(cmul(cBA, A), cmul(cBB, B)) : czero<C>();
  }
}

// One bounce stage: grid = (steps of the stage, frequencies).  JOINT: steps
// with both slots propagated take the joint path (twice the row tile in
// shared memory).  NZ: box lines occupy at most NZ of a thread's RR register
// slots (x = g + G r < nbx, y = g + G r < nby only for r < NZ), so the first
// forward pass is pruned and the inverse stores only NZ slots.  MINB: CTAs
// per SM the registers are sized for.  MODE: kModeTwShared | kModeHalf |
// kModeStage (fewer registers or less shared memory per warp, so more warps
// per SM, and phasor rows staged ahead); the arithmetic, and so every result,
// is the same.
template <typename R, int N, bool JOINT, int NZ, int THREADS, int MINB, int MODE>
__global__ void __launch_bounds__(THREADS, MINB) k_fused_stage(FusedArgs<cplx_t<R>> a) {
  using C = cplx_t<R>;
  using X = FusedCtx<C, N>;
  constexpr int G = X::G, RR = X::RR, P = X::P;
  constexpr int NTEAM = THREADS / G;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int nby = a.nby;
  C* M = reinterpret_cast<C*>(smem_raw + kSmemHeader);
  C* scr_all = M + (JOINT ? 2 : 1) * nby * P;
  const int tid = threadIdx.x, team = tid / G, g = tid % G;
  constexpr bool HALF = (MODE & kModeHalf) != 0, STAGE = (MODE & kModeStage) != 0;
  C* scr = scr_all + team * team_region<N, MODE>();
  const StepDesc sd = a.steps[blockIdx.x];
  const int f = blockIdx.y;
  C twr[RR];
  const C* tw = twr;
  if constexpr ((MODE & kModeTwShared) != 0) {
    // tw[g][s] = W_N^(g s) behind the teams' regions, rows RR + 1 apart so
    // that the G threads of a team reading their s-th twiddle hit distinct banks
    C* tws = scr_all + NTEAM * team_region<N, MODE>();
    for (int i = tid; i < G * RR; i += THREADS)
      tws[(i / RR) * (RR + 1) + i % RR] = root1024<C>((i / RR) * (i % RR) * (1024 / N));
    __syncthreads();
    tw = tws + g * (RR + 1);
  } else {
    team_twiddles<N>(twr, g);
  }
  const int QW = a.fold ? N / 2 : N;
  auto qptr = [&](int region) -> const C* {
    return a.phasor + ((size_t)f * a.ntab + region) * (size_t)(QW * QW);
  };
  const bool pa = sd.ra >= 0, pb = sd.rb >= 0;
  if (JOINT && pa && pb) {
    C* MB = M + nby * P;
    prefetch_qrow<C, N, false>(a, qptr(sd.ra), qptr(sd.rb), team, g);
    joint_phase1<C, N, NZ, NTEAM, false, HALF>(a, sd, f, M, MB, scr, tw, team, g, 0, NTEAM, true, true);
    joint_phase2<C, N, NZ, NTEAM, false, HALF, STAGE>(a, qptr(sd.ra), qptr(sd.rb), M, MB, scr, tw, team, g, 0,
                                                      NTEAM);
    joint_phase3<C, N, NZ, NTEAM, false, HALF>(a, sd, f, M, MB, scr, tw, team, g, 0, NTEAM, true, true);
    joint_mix<C, N>(a, sd, f, M, MB, true, true, threadIdx.x, blockDim.x);
  } else if (pa && pb) {
    // A~ is parked in the A slot itself until the boundary mix
    C* obuf = a.state + ((size_t)f * a.nslots + sd.sa) * (size_t)(nby * a.nbx);
    fused_phase1<C, N, NZ, NTEAM, HALF>(a, f, sd.sa, sd.exitA, M, scr, tw, team, g);
    fused_phase2<C, N, NZ, NTEAM, HALF, STAGE>(a, qptr(sd.ra), M, scr, tw, team, g);
    fused_phase3<C, N, false, NZ, NTEAM, HALF>(a, sd, f, sd.ra, false, M, scr, obuf, tw, team, g);
    // no barrier: B's forward row pass writes row y of M through the same
    // team (y mod NTEAM) and the same per-thread elements that A's inverse row
    // pass just read from it, and A~ goes to global memory, read back in B's
    // mix by the same thread; program order already orders every access
    fused_phase1<C, N, NZ, NTEAM, HALF>(a, f, sd.sb, sd.exitB, M, scr, tw, team, g);
    fused_phase2<C, N, NZ, NTEAM, HALF, STAGE>(a, qptr(sd.rb), M, scr, tw, team, g);
    fused_phase3<C, N, true, NZ, NTEAM, HALF>(a, sd, f, sd.rb, true, M, scr, obuf, tw, team, g);
  } else if (pa) {
    fused_phase1<C, N, NZ, NTEAM, HALF>(a, f, sd.sa, sd.exitA, M, scr, tw, team, g);
    fused_phase2<C, N, NZ, NTEAM, HALF, STAGE>(a, qptr(sd.ra), M, scr, tw, team, g);
    fused_phase3<C, N, true, NZ, NTEAM, HALF>(a, sd, f, sd.ra, false, M, scr, nullptr, tw, team, g);
  } else if (pb) {
    fused_phase1<C, N, NZ, NTEAM, HALF>(a, f, sd.sb, sd.exitB, M, scr, tw, team, g);
    fused_phase2<C, N, NZ, NTEAM, HALF, STAGE>(a, qptr(sd.rb), M, scr, tw, team, g);
    fused_phase3<C, N, true, NZ, NTEAM, HALF>(a, sd, f, sd.rb, true, M, scr, nullptr, tw, team, g);
  }
}

// ---- split-phase stage: for stages with fewer steps x frequencies than SMs --
// The four phases of a step (forward rows, columns, inverse rows, boundary
// mix) run as four launches whose tasks are spread over blockIdx.z, so a
// stage with a handful of steps (one frequency, a short stack) still spreads
// its FFT work over many SMs.  The row tiles of step s, frequency f live in
// global memory at a.mg + (s nfreq + f) 2 nby P (A, then B) and stay in L2.
constexpr int kSplitThreads = 64;

template <typename R, int N, int NZ>
__global__ void __launch_bounds__(kSplitThreads) k_split_phase(FusedArgs<cplx_t<R>> a, int phase) {
  using C = cplx_t<R>;
  using X = FusedCtx<C, N>;
  constexpr int G = X::G, RR = X::RR, P = X::P;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int tid = threadIdx.x, team = tid / G, g = tid % G, nteam = blockDim.x / G;
  // programmatic dependent launch: let the next phase launch now, and wait for
  // the previous phase (its writes visible) before reading anything it wrote
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  C tw[RR];
  team_twiddles<N>(tw, g);
  asm volatile("griddepcontrol.wait;" ::: "memory");
  const StepDesc sd = a.steps[blockIdx.x];
  const int f = blockIdx.y;
  C* MA = a.mg + ((size_t)blockIdx.x * a.nfreq + f) * 2 * (size_t)a.nby * P;
  C* MB = MA + (size_t)a.nby * P;
  const bool pa = sd.ra >= 0, pb = sd.rb >= 0;
  if (phase == 3) {
    joint_mix<C, N>(a, sd, f, MA, MB, pa, pb, blockIdx.z * blockDim.x + tid, gridDim.z * blockDim.x);
    return;
  }
  C* scr = reinterpret_cast<C*>(smem_raw) + team * X::T::SCR;
  const int t0 = blockIdx.z * nteam, ts = gridDim.z * nteam;
  if (phase == 0) {
    joint_phase1<C, N, NZ, kSplitThreads / G, true>(a, sd, f, MA, MB, scr, tw, team, g, t0, ts, pa, pb);
  } else if (phase == 1) {
    const int QW = a.fold ? N / 2 : N;
    const C* QA = pa ? a.phasor + ((size_t)f * a.ntab + sd.ra) * (size_t)(QW * QW) : nullptr;
    const C* QB = pb ? a.phasor + ((size_t)f * a.ntab + sd.rb) * (size_t)(QW * QW) : nullptr;
    joint_phase2<C, N, NZ, kSplitThreads / G, true>(a, QA, QB, MA, MB, scr, tw, team, g, t0, ts);
  } else {
    joint_phase3<C, N, NZ, kSplitThreads / G, true>(a, sd, f, MA, MB, scr, tw, team, g, t0, ts, pa, pb);
  }
}

static int sm_count() {
  static int n = 0;
  if (!n) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n < 1) n = 1;
  }
  return n;
}

template <typename R, int N, int NZ>
static int launch_split(const FusedArgs<cplx_t<R>>& a, int nsteps, cudaStream_t st) {
  using T = Team<N>;
  const int nteam = kSplitThreads / T::G;
  const size_t smem = sizeof(cplx_t<R>) * nteam * T::SCR;
  const int zr = (2 * a.nby + nteam - 1) / nteam, zc = (2 * N + nteam - 1) / nteam;
  const int zm = (a.nbx * a.nby + kSplitThreads - 1) / kSplitThreads;
  const int z[4] = {zr, zc, zr, zm};
  // each phase may launch while the previous one drains (programmatic
  // dependent launch); the kernel waits for it before touching its data
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  for (int ph = 0; ph < 4; ++ph) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(nsteps, a.nfreq, z[ph]);
    cfg.blockDim = dim3(kSplitThreads);
    cfg.dynamicSmemBytes = ph == 3 ? 0 : smem;
    cfg.stream = st;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    COUNT_LAUNCH();
    const cudaError_t e = cudaLaunchKernelEx(&cfg, k_split_phase<R, N, NZ>, a, ph);
    if (e != cudaSuccess) return (int)e;
  }
  return 0;
}

// Bytes of the split-phase row tiles for a stage of `nsteps` steps.
size_t split_tile_bytes(int N, int nby, int nfreq, int nsteps, bool fp64) {
  return (size_t)nsteps * nfreq * 2 * nby * (N + 2) * (fp64 ? 16 : 8);
}

// Whether a stage of `nsteps` steps x `nfreq` frequencies takes the split path.
bool split_stage(int nsteps, int nfreq) { return (long long)nsteps * nfreq < sm_count(); }

template <int N, int MODE = 0>
static size_t fused_smem_for(int nby, size_t csz, int tiles = 1, int threads = kFusedThreads) {
  const size_t nteam = threads / Team<N>::G;
  const size_t twt = (MODE & kModeTwShared) ? (size_t)Team<N>::G * (Team<N>::RR + 1) : 0;   // twiddle table
  return kSmemHeader + csz * ((size_t)tiles * nby * fused_pitch<N>() + nteam * team_region<N, MODE>() + twt);
}

static size_t smem_for(int N, int nby, size_t csz) {
  switch (N) {
    case 8: return fused_smem_for<8>(nby, csz);
    case 16: return fused_smem_for<16>(nby, csz);
    case 32: return fused_smem_for<32>(nby, csz);
    case 64: return fused_smem_for<64>(nby, csz);
    case 128: return fused_smem_for<128>(nby, csz);
    case 256: return fused_smem_for<256>(nby, csz);
    default: return (size_t)-1;
  }
}

static const size_t kMaxSmem = 227 * 1024;

size_t fused_smem_bytes(int N, int nbx, int nby, bool fp64) {
  (void)nbx;
  return smem_for(N, nby, fp64 ? 16 : 8);
}

bool fused_split_only(int N, int nbx, int nby, bool fp64) {
  return N >= 64 && fused_smem_bytes(N, nbx, nby, fp64) > kMaxSmem;
}

bool fused_supported(int N, int nbx, int nby, bool fp64) {
  if (N < 8 || N > 256 || (N & (N - 1))) return false;
  if (nbx < 1 || nby < 1 || nbx > N || nby > N) return false;
  // row tiles too large for shared memory (complex128 at 256^2): every stage
  // takes the split-phase path, whose tiles live in global memory
  return fused_smem_bytes(N, nbx, nby, fp64) <= kMaxSmem || fused_split_only(N, nbx, nby, fp64);
}

// Shared memory of one SM (bytes) and what the driver reserves per CTA.
static const size_t kSmemPerSM = 228 * 1024, kSmemReservedPerCta = 1024;

// The dynamic shared-memory limit of a kernel is raised to the per-block
// maximum, the same value for every launch: launches of one kernel with
// different sizes from several host threads (the serving engine's workers)
// must not lower it under one another.
template <typename R, int N, bool JOINT, int NZ, int THREADS = kFusedThreads,
          int MINB = (sizeof(R) == 4 && N <= 128) ? 2 : 1, int MODE = 0>
static int launch_fused_v(const FusedArgs<cplx_t<R>>& a, dim3 grid, size_t smem, cudaStream_t st) {
  cudaError_t e = cudaFuncSetAttribute(k_fused_stage<R, N, JOINT, NZ, THREADS, MINB, MODE>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxSmem);
  if (e != cudaSuccess) return (int)e;
  k_fused_stage<R, N, JOINT, NZ, THREADS, MINB, MODE><<<grid, THREADS, smem, st>>>(a);
  return (int)cudaGetLastError();
}

// Register slots a box line may occupy in the pruned variants (complex64 for
// N >= 64, complex128 for N = 64, 128): 5 of 16 (3 of 8) covers boxes up to
// 5/16 of the grid, the disk of radius 0.15 m in the reference's 1 m window.
template <int N> constexpr int pruned_slots() { return (5 * Team<N>::RR + 15) / 16; }

// Shape of one fused-stage launch: shared memory of the single and doubled
// (joint) row tiles and whether the rule takes the joint path.
struct FusedShape {
  size_t smem, smem_j, smem512, smem_jl, smem_sl, smem_js, smem_ss, smem_s5;
  bool joint_rule, joint_fits, wide_fits;
  // complex64, N = 128: joint steps with 320 threads at 2 CTAs per SM and
  // shared twiddles (lean), separate slots at 3 CTAs per SM and shared
  // twiddles (lean), joint steps with staged phasor rows, separate slots at 3
  // CTAs per SM with shared twiddles and staged phasor rows, separate slots
  // with 20 teams (160 threads: 38 box rows in two rounds) at 3 CTAs per SM
  // with staged phasor rows
  bool joint_lean_fits, sep_lean_fits, joint_staged_fits, sep_staged_fits, sep5_staged_fits;
};
constexpr int kLeanJointThreads = 320, kSep5Threads = 160;
constexpr int kModeLean = kModeTwShared | kModeHalf;
constexpr int kModeHalfStaged = kModeHalf | kModeStage;
constexpr int kModeLeanStaged = kModeTwShared | kModeHalf | kModeStage;
template <int N>
static FusedShape fused_shape(int nby, size_t csz) {
  FusedShape f;
  f.smem = fused_smem_for<N>(nby, csz, 1);
  f.smem_j = fused_smem_for<N>(nby, csz, 2);
  f.smem512 = fused_smem_for<N>(nby, csz, 1, 512);
  // the joint path when the doubled row tile keeps as many CTAs per SM
  const int ctas = (csz == 8 && N <= 128) ? 2 : 1;
  f.joint_fits = f.smem_j <= kMaxSmem;
  f.joint_rule = f.joint_fits && (size_t)ctas * (f.smem_j + kSmemReservedPerCta) <= kSmemPerSM &&
                 (size_t)ctas * (f.smem + kSmemReservedPerCta) <= kSmemPerSM;
  f.wide_fits = csz == 8 && N == 256 && f.smem512 <= kMaxSmem;
  f.smem_jl = fused_smem_for<N, kModeLean>(nby, csz, 2, kLeanJointThreads);
  f.smem_sl = fused_smem_for<N, kModeLean>(nby, csz, 1, kFusedThreads);
  f.smem_js = fused_smem_for<N, kModeHalfStaged>(nby, csz, 2, kFusedThreads);
  f.smem_ss = fused_smem_for<N, kModeLeanStaged>(nby, csz, 1, kFusedThreads);
  f.smem_s5 = fused_smem_for<N, kModeHalfStaged>(nby, csz, 1, kSep5Threads);
  const bool c128 = csz == 8 && N == 128;
  f.joint_lean_fits = c128 && 2 * (f.smem_jl + kSmemReservedPerCta) <= kSmemPerSM;
  f.sep_lean_fits = c128 && 3 * (f.smem_sl + kSmemReservedPerCta) <= kSmemPerSM;
  f.joint_staged_fits = c128 && 2 * (f.smem_js + kSmemReservedPerCta) <= kSmemPerSM;
  f.sep_staged_fits = c128 && 3 * (f.smem_ss + kSmemReservedPerCta) <= kSmemPerSM;
  f.sep5_staged_fits = c128 && 3 * (f.smem_s5 + kSmemReservedPerCta) <= kSmemPerSM;
  return f;
}

template <int N>
static std::vector<int> fused_variants_t(int nbx, int nby, bool fp64) {
  const FusedShape f = fused_shape<N>(nby, fp64 ? 16 : 8);
  // the lean variants exist for boxes within the pruned register slots only
  const bool pruned = (std::max(nbx, nby) + Team<N>::G - 1) / Team<N>::G <= pruned_slots<N>();
  std::vector<int> v = {kFusedRule};
  if (f.smem > kMaxSmem) return v;
  v.push_back(kFusedSeparate);
  if (f.joint_fits) v.push_back(kFusedJoint);
  if (f.wide_fits) v.push_back(kFusedWide);
  if (f.joint_lean_fits && pruned) v.push_back(kFusedJointLean);
  if (f.sep_lean_fits && pruned) v.push_back(kFusedSeparateLean);
  if (f.joint_staged_fits && pruned) v.push_back(kFusedJointStaged);
  if (f.sep_staged_fits && pruned) v.push_back(kFusedSeparateStaged);
  if (f.sep5_staged_fits && pruned) v.push_back(kFusedSeparate160Staged);
  return v;
}

std::vector<int> fused_variants(int N, int nbx, int nby, bool fp64) {
  switch (N) {
    case 8: return fused_variants_t<8>(nbx, nby, fp64);
    case 16: return fused_variants_t<16>(nbx, nby, fp64);
    case 32: return fused_variants_t<32>(nbx, nby, fp64);
    case 64: return fused_variants_t<64>(nbx, nby, fp64);
    case 128: return fused_variants_t<128>(nbx, nby, fp64);
    case 256: return fused_variants_t<256>(nbx, nby, fp64);
    default: return {kFusedRule};
  }
}

template <typename R, int N>
static int launch_fused_t(const FusedArgs<cplx_t<R>>& a, int nsteps, cudaStream_t st) {
  const size_t csz = sizeof(cplx_t<R>);
  const FusedShape sh = fused_shape<N>(a.nby, csz);
  const size_t smem = sh.smem, smem_j = sh.smem_j;
  const bool split_only = smem > kMaxSmem;   // every stage in global-memory row tiles
  if (split_only && !(a.mg && N >= 64)) return (int)cudaErrorInvalidValue;
  constexpr int G = Team<N>::G, RR = Team<N>::RR;
  const int rv = (std::max(a.nbx, a.nby) + G - 1) / G;
  if (a.mg && N >= 64 && (split_only || split_stage(nsteps, a.nfreq))) {
    if constexpr ((sizeof(R) == 4 && N >= 64) || (sizeof(R) == 8 && (N == 64 || N == 128)))
      if (rv <= pruned_slots<N>()) return launch_split<R, N, pruned_slots<N>()>(a, nsteps, st);
    return launch_split<R, N, RR>(a, nsteps, st);
  }
  // the variant: the rule's choice, or one picked by the autotuner (an
  // invalid choice falls back to the rule)
  bool joint = sh.joint_rule, wide = sh.wide_fits && !sh.joint_rule;
  if (a.variant == kFusedSeparate) {
    joint = false;
    wide = false;
  } else if (a.variant == kFusedJoint && sh.joint_fits) {
    joint = true;
    wide = false;
  } else if (a.variant == kFusedWide && sh.wide_fits) {
    joint = false;
    wide = true;
  }
  dim3 grid(nsteps, a.nfreq);
  COUNT_LAUNCH();
  if constexpr (sizeof(R) == 4 && N == 128) {
    if (rv <= pruned_slots<N>()) {
      constexpr int NZ = pruned_slots<N>();
      if (a.variant == kFusedJointLean && sh.joint_lean_fits)
        return launch_fused_v<R, N, true, NZ, kLeanJointThreads, 2, kModeLean>(a, grid, sh.smem_jl, st);
      if (a.variant == kFusedSeparateLean && sh.sep_lean_fits)
        return launch_fused_v<R, N, false, NZ, kFusedThreads, 3, kModeLean>(a, grid, sh.smem_sl, st);
      if (a.variant == kFusedJointStaged && sh.joint_staged_fits)
        return launch_fused_v<R, N, true, NZ, kFusedThreads, 2, kModeHalfStaged>(a, grid, sh.smem_js, st);
      if (a.variant == kFusedSeparateStaged && sh.sep_staged_fits)
        return launch_fused_v<R, N, false, NZ, kFusedThreads, 3, kModeLeanStaged>(a, grid, sh.smem_ss, st);
      if (a.variant == kFusedSeparate160Staged && sh.sep5_staged_fits)
        return launch_fused_v<R, N, false, NZ, kSep5Threads, 3, kModeHalfStaged>(a, grid, sh.smem_s5, st);
    }
  }
  if constexpr (sizeof(R) == 4 && N == 256) {
    // one CTA per SM (the 256-point row tile): 512 threads (32 teams, at most
    // 128 registers each) when the team scratch still fits beside the tile
    if (wide)
      return rv <= pruned_slots<N>() ? launch_fused_v<R, N, false, pruned_slots<N>(), 512>(a, grid, sh.smem512, st)
                                     : launch_fused_v<R, N, false, Team<N>::RR, 512>(a, grid, sh.smem512, st);
  }
  if constexpr ((sizeof(R) == 4 && N >= 64) || (sizeof(R) == 8 && (N == 64 || N == 128))) {
    if (rv <= pruned_slots<N>())
      return joint ? launch_fused_v<R, N, true, pruned_slots<N>()>(a, grid, smem_j, st)
                   : launch_fused_v<R, N, false, pruned_slots<N>()>(a, grid, smem, st);
  }
  return joint ? launch_fused_v<R, N, true, RR>(a, grid, smem_j, st) : launch_fused_v<R, N, false, RR>(a, grid, smem, st);
}

template <typename R>
static int launch_fused_dispatch(int N, const FusedArgs<cplx_t<R>>& a, int nsteps, cudaStream_t st) {
  if (nsteps <= 0 || a.nfreq <= 0) return 0;
  switch (N) {
    case 8: return launch_fused_t<R, 8>(a, nsteps, st);
    case 16: return launch_fused_t<R, 16>(a, nsteps, st);
    case 32: return launch_fused_t<R, 32>(a, nsteps, st);
    case 64: return launch_fused_t<R, 64>(a, nsteps, st);
    case 128: return launch_fused_t<R, 128>(a, nsteps, st);
    case 256: return launch_fused_t<R, 256>(a, nsteps, st);
    default: return (int)cudaErrorInvalidValue;
  }
}

int launch_fused_stage_f(int N, const FusedArgs<float2>& a, int nsteps, cudaStream_t st) {
  return launch_fused_dispatch<float>(N, a, nsteps, st);
}
int launch_fused_stage_d(int N, const FusedArgs<double2>& a, int nsteps, cudaStream_t st) {
  return launch_fused_dispatch<double>(N, a, nsteps, st);
}

// ---------------------------------------------------------------------------
// Phasor and tilt tables
// ---------------------------------------------------------------------------
template <typename C>
__global__ void k_phasor_table(C* out, int nfreq, const double* freqs, int ntab, const int* regions,
                               const RegionGeo* geo, int N, const double* kX, const double* kY,
                               int fold) {
  const int W = fold ? N / 2 : N;
  const int per = W * W;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  const int t = blockIdx.y, f = blockIdx.z;
  if (idx >= per) return;
  const int kxb = idx / W, kyb = idx % W;
  const int sx = (kxb + N / 2) % N, sy = (kyb + N / 2) % N;
  const RegionGeo gg = geo[regions[t]];
  const double lambda = SPEED_OF_LIGHT / freqs[f];
  const double2 k0 = k0_of(lambda, gg.eps_re, gg.eps_im);
  double2 v = phasor_value(k0, kX[sx], kY[sy], gg.dz);
  const double sc = 1.0 / ((double)N * (double)N);   // a power of two: exact
  out[((size_t)f * ntab + t) * per + idx] = from_d_phase<C>(make_double2(v.x * sc, v.y * sc));
}

int launch_phasor_table(bool fp64, void* out, int nfreq, const double* d_freqs, int ntab,
                        const int* d_regions, const RegionGeo* d_geo, int N, const double* d_kX,
                        const double* d_kY, int fold, cudaStream_t st) {
  if (ntab <= 0 || nfreq <= 0) return 0;
  const int W = fold ? N / 2 : N;
  dim3 grid((W * W + 255) / 256, ntab, nfreq);
  if (fp64) { COUNT_LAUNCH(); k_phasor_table<double2><<<grid, 256, 0, st>>>((double2*)out, nfreq, d_freqs, ntab, d_regions, d_geo, N, d_kX, d_kY, fold); }
  else { COUNT_LAUNCH(); k_phasor_table<float2><<<grid, 256, 0, st>>>((float2*)out, nfreq, d_freqs, ntab, d_regions, d_geo, N, d_kX, d_kY, fold); }
  return (int)cudaGetLastError();
}

template <typename C>
__global__ void k_tilt_table(C* out, int nfreq, const double* freqs, int nmaps, const int* regions,
                             const RegionGeo* geo, int nbx, int nby, int bx0, int by0, int nx, int ny,
                             const double* X, const double* Y, const double2* surf) {
  const int per = nbx * nby;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  const int m = blockIdx.y, f = blockIdx.z;
  if (idx >= per) return;
  const int iy = idx / nbx, ix = idx % nbx;
  const int x = bx0 + ix, y = by0 + iy;
  const int reg = regions[m];
  const RegionGeo gg = geo[reg];
  const double lambda = SPEED_OF_LIGHT / freqs[f];
  const double2 k0 = k0_of(lambda, gg.eps_re, gg.eps_im);
  double2 v = cmul(phase_k0(k0, gg.tilt_x * X[x]), phase_k0(k0, gg.tilt_y * Y[y]));
  if (surf) v = cmul(v, phase_k0c(k0, surf[((size_t)reg * ny + y) * nx + x]));
  out[((size_t)f * nmaps + m) * per + idx] = from_d_phase<C>(v);
}

int launch_tilt_table(bool fp64, void* out, int nfreq, const double* d_freqs, int nmaps,
                      const int* d_regions, const RegionGeo* d_geo, int nbx, int nby, int bx0,
                      int by0, int nx, int ny, const double* d_X, const double* d_Y,
                      const double2* d_surf, cudaStream_t st) {
  if (nmaps <= 0 || nfreq <= 0) return 0;
  dim3 grid((nbx * nby + 255) / 256, nmaps, nfreq);
  if (fp64) { COUNT_LAUNCH(); k_tilt_table<double2><<<grid, 256, 0, st>>>((double2*)out, nfreq, d_freqs, nmaps, d_regions, d_geo, nbx, nby, bx0, by0, nx, ny, d_X, d_Y, d_surf); }
  else { COUNT_LAUNCH(); k_tilt_table<float2><<<grid, 256, 0, st>>>((float2*)out, nfreq, d_freqs, nmaps, d_regions, d_geo, nbx, nby, bx0, by0, nx, ny, d_X, d_Y, d_surf); }
  return (int)cudaGetLastError();
}

// ---------------------------------------------------------------------------
// General full-grid path
// ---------------------------------------------------------------------------
// One block transforms one line of length n held in shared memory: radix-2
// Stockham for powers of two, direct O(n^2) evaluation otherwise.  Roots are
// evaluated in FP64 (sincospi) for either field precision.
template <typename C>
__global__ void k_line_dft(C* data, int nx, int ny, int axis, int inverse) {
  extern __shared__ __align__(16) unsigned char sm[];
  const int n = axis == 0 ? nx : ny;
  C* buf0 = reinterpret_cast<C*>(sm);
  C* buf1 = buf0 + n;
  C* tw = buf1 + n;   // tw[m] = exp(-+2 pi i m / n)
  const int line = blockIdx.x, b = blockIdx.y;
  const size_t base = (size_t)b * nx * ny;
  const size_t stride = axis == 0 ? 1 : nx;
  const size_t off = axis == 0 ? (size_t)line * nx : (size_t)line;
  const double sgn = inverse ? 2.0 : -2.0;
  // power-of-two lengths up to 1024 take the unit roots from the constant
  // table (FP64, exactly symmetric) instead of one FP64 sincospi per entry
  const bool table = (n & (n - 1)) == 0 && n <= 1024;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    buf0[i] = data[base + off + i * stride];
    if (table) {
      const double2 r = c_root1024_d[i * (1024 / n)];   // exp(-2 pi i k / n)
      tw[i] = from_d<C>(make_double2(r.x, inverse ? -r.y : r.y));
    } else {
      double s, c;
      sincospi(sgn * (double)i / (double)n, &s, &c);
      tw[i] = from_d<C>(make_double2(c, s));
    }
  }
  __syncthreads();
  if ((n & (n - 1)) == 0) {
    // Stockham autosort, radix 2
    C* src = buf0;
    C* dst = buf1;
    for (int l = 1; l < n; l <<= 1) {   // l = size of the sub-transforms being combined
      const int tstep = n / (2 * l);
      for (int i = threadIdx.x; i < n / 2; i += blockDim.x) {
        const int j = i % l;            // position within sub-transform
        const int k = i / l;            // sub-transform index
        const C w = tw[j * tstep];
        C u = src[k * l + j];
        C v = cmul(src[k * l + j + n / 2], w);
        dst[2 * k * l + j] = cadd(u, v);
        dst[2 * k * l + j + l] = csub(u, v);
      }
      __syncthreads();
      C* t = src; src = dst; dst = t;
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) data[base + off + i * stride] = src[i];
  } else {
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
      double2 acc = make_double2(0.0, 0.0);
      int m = 0;
      for (int j = 0; j < n; ++j) {
        const double2 w = to_d(tw[m]);
        const double2 x = to_d(buf0[j]);
        acc.x += x.x * w.x - x.y * w.y;
        acc.y += x.x * w.y + x.y * w.x;
        m += k;
        if (m >= n) m -= n;
      }
      buf1[k] = from_d<C>(acc);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) data[base + off + i * stride] = buf1[i];
  }
}

int launch_line_dft(bool fp64, void* data, int nb, int nx, int ny, int axis, int inverse,
                    cudaStream_t st) {
  const int n = axis == 0 ? nx : ny;
  const int nlines = axis == 0 ? ny : nx;
  if (n <= 1) return 0;
  const size_t smem = (fp64 ? 16 : 8) * (size_t)(3 * n);
  if (smem > kMaxSmem) return (int)cudaErrorInvalidValue;
  dim3 grid(nlines, nb);
  int thr = n >= 256 ? 256 : ((n + 31) / 32) * 32;
  if (fp64) {
    if (smem > 48 * 1024) cudaFuncSetAttribute(k_line_dft<double2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxSmem);
      COUNT_LAUNCH();
      k_line_dft<double2><<<grid, thr, smem, st>>>((double2*)data, nx, ny, axis, inverse);
  } else {
    if (smem > 48 * 1024) cudaFuncSetAttribute(k_line_dft<float2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxSmem);
      COUNT_LAUNCH();
      k_line_dft<float2><<<grid, thr, smem, st>>>((float2*)data, nx, ny, axis, inverse);
  }
  return (int)cudaGetLastError();
}

template <typename C>
__global__ void k_mul_mask(C* data, size_t total, int npix, const unsigned char* mask) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x)
    if (!mask[i % npix]) data[i] = czero<C>();
}

static dim3 grid1d(size_t n) {
  size_t b = (n + 255) / 256;
  if (b > 65535 * 16) b = 65535 * 16;
  if (b < 1) b = 1;
  return dim3((unsigned)b);
}

int launch_mul_mask(bool fp64, void* data, int nb, int nx, int ny, const unsigned char* d_mask,
                    cudaStream_t st) {
  size_t total = (size_t)nb * nx * ny;
  if (fp64) { COUNT_LAUNCH(); k_mul_mask<double2><<<grid1d(total), 256, 0, st>>>((double2*)data, total, nx * ny, d_mask); }
  else { COUNT_LAUNCH(); k_mul_mask<float2><<<grid1d(total), 256, 0, st>>>((float2*)data, total, nx * ny, d_mask); }
  return (int)cudaGetLastError();
}

__device__ __forceinline__ double lambda_of(const double* freqs, const double* lambdas, int b) {
  return lambdas ? lambdas[b] : SPEED_OF_LIGHT / freqs[b];
}

template <typename C>
__global__ void k_mul_phasor_full(C* data, int nb, int nx, int ny, const double* freqs,
                                  const double* lambdas, RegionGeo g, const double* kX,
                                  const double* kY, int shifted, double scale) {
  const size_t total = (size_t)nb * nx * ny;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const int x = (int)(i % nx);
    const int y = (int)((i / nx) % ny);
    const int b = (int)(i / ((size_t)nx * ny));
    const int sx = shifted ? x : (x + nx / 2) % nx;
    const int sy = shifted ? y : (y + ny / 2) % ny;
    const double2 k0 = k0_of(lambda_of(freqs, lambdas, b), g.eps_re, g.eps_im);
    double2 p = phasor_value(k0, kX[sx], kY[sy], g.dz);
    p.x *= scale; p.y *= scale;
    double2 d = to_d(data[i]);
    data[i] = from_d<C>(cmul(d, p));
  }
}

int launch_mul_phasor_full(bool fp64, void* data, int nb, int nx, int ny, const double* d_freqs,
                           const double* d_lambda, RegionGeo g, const double* d_kX,
                           const double* d_kY, int shifted_layout, double scale, cudaStream_t st) {
  size_t total = (size_t)nb * nx * ny;
  if (fp64) { COUNT_LAUNCH(); k_mul_phasor_full<double2><<<grid1d(total), 256, 0, st>>>((double2*)data, nb, nx, ny, d_freqs, d_lambda, g, d_kX, d_kY, shifted_layout, scale); }
  else { COUNT_LAUNCH(); k_mul_phasor_full<float2><<<grid1d(total), 256, 0, st>>>((float2*)data, nb, nx, ny, d_freqs, d_lambda, g, d_kX, d_kY, shifted_layout, scale); }
  return (int)cudaGetLastError();
}

template <typename C>
__global__ void k_mul_tilt_full(C* data, int nb, int nx, int ny, const double* freqs,
                                const double* lambdas, RegionGeo g, const double* X, const double* Y,
                                const double2* surf, int only_if_nonzero) {
  const size_t total = (size_t)nb * nx * ny;
  const bool do_tilt = !only_if_nonzero || g.tilt_x != 0.0 || g.tilt_y != 0.0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const int x = (int)(i % nx);
    const int y = (int)((i / nx) % ny);
    const int b = (int)(i / ((size_t)nx * ny));
    const double2 k0 = k0_of(lambda_of(freqs, lambdas, b), g.eps_re, g.eps_im);
    double2 d = to_d(data[i]);
    if (do_tilt) d = cmul(d, cmul(phase_k0(k0, g.tilt_x * X[x]), phase_k0(k0, g.tilt_y * Y[y])));
    if (surf) d = cmul(d, phase_k0c(k0, surf[(size_t)y * nx + x]));
    data[i] = from_d<C>(d);
  }
}

int launch_mul_tilt_full(bool fp64, void* data, int nb, int nx, int ny, const double* d_freqs,
                         const double* d_lambda, RegionGeo g, const double* d_X, const double* d_Y,
                         const double2* d_surf, int only_if_nonzero, cudaStream_t st) {
  size_t total = (size_t)nb * nx * ny;
  if (fp64) { COUNT_LAUNCH(); k_mul_tilt_full<double2><<<grid1d(total), 256, 0, st>>>((double2*)data, nb, nx, ny, d_freqs, d_lambda, g, d_X, d_Y, d_surf, only_if_nonzero); }
  else { COUNT_LAUNCH(); k_mul_tilt_full<float2><<<grid1d(total), 256, 0, st>>>((float2*)data, nb, nx, ny, d_freqs, d_lambda, g, d_X, d_Y, d_surf, only_if_nonzero); }
  return (int)cudaGetLastError();
}

template <typename C>
__global__ void k_mul_phase1d(C* data, int nb, int npix, const double* freqs, const double* lambdas,
                              RegionGeo g) {
  const size_t total = (size_t)nb * npix;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const int b = (int)(i / npix);
    const double2 k0 = k0_of(lambda_of(freqs, lambdas, b), g.eps_re, g.eps_im);
    data[i] = from_d<C>(cmul(to_d(data[i]), phase_k0(k0, g.dz)));
  }
}

int launch_mul_scalar_phase_1d(bool fp64, void* data, int nb, int nx, int ny, const double* d_freqs,
                               const double* d_lambda, RegionGeo g, cudaStream_t st) {
  size_t total = (size_t)nb * nx * ny;
  if (fp64) { COUNT_LAUNCH(); k_mul_phase1d<double2><<<grid1d(total), 256, 0, st>>>((double2*)data, nb, nx * ny, d_freqs, d_lambda, g); }
  else { COUNT_LAUNCH(); k_mul_phase1d<float2><<<grid1d(total), 256, 0, st>>>((float2*)data, nb, nx * ny, d_freqs, d_lambda, g); }
  return (int)cudaGetLastError();
}

template <typename C>
__global__ void k_roll(const C* in, C* out, int nb, int nx, int ny, int sx, int sy) {
  const size_t total = (size_t)nb * nx * ny;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const int x = (int)(i % nx);
    const int y = (int)((i / nx) % ny);
    const size_t b = i / ((size_t)nx * ny);
    const int xs = ((x - sx) % nx + nx) % nx;
    const int ys = ((y - sy) % ny + ny) % ny;
    out[i] = in[(b * ny + ys) * nx + xs];
  }
}

int launch_roll(bool fp64, const void* in, void* out, int nb, int nx, int ny, int sx, int sy,
                cudaStream_t st) {
  size_t total = (size_t)nb * nx * ny;
  if (fp64) { COUNT_LAUNCH(); k_roll<double2><<<grid1d(total), 256, 0, st>>>((const double2*)in, (double2*)out, nb, nx, ny, sx, sy); }
  else { COUNT_LAUNCH(); k_roll<float2><<<grid1d(total), 256, 0, st>>>((const float2*)in, (float2*)out, nb, nx, ny, sx, sy); }
  return (int)cudaGetLastError();
}

template <typename CI, typename CO>
__global__ void k_convert(const CI* in, CO* out, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    out[i] = from_d<CO>(to_d(in[i]));
}

int launch_convert(const void* in, bool in_fp64, void* out, bool out_fp64, size_t n, cudaStream_t st) {
  if (in_fp64 && out_fp64) { COUNT_LAUNCH(); k_convert<double2, double2><<<grid1d(n), 256, 0, st>>>((const double2*)in, (double2*)out, n); }
  else if (in_fp64) { COUNT_LAUNCH(); k_convert<double2, float2><<<grid1d(n), 256, 0, st>>>((const double2*)in, (float2*)out, n); }
  else if (out_fp64) { COUNT_LAUNCH(); k_convert<float2, double2><<<grid1d(n), 256, 0, st>>>((const float2*)in, (double2*)out, n); }
  else { COUNT_LAUNCH(); k_convert<float2, float2><<<grid1d(n), 256, 0, st>>>((const float2*)in, (float2*)out, n); }
  return (int)cudaGetLastError();
}

// ---------------------------------------------------------------------------
// exits, broadcast, reductions
// ---------------------------------------------------------------------------
__global__ void k_exit_combine(double2* out, const double2* full, const double2* direct, double2 coef,
                               int nfreq, int npix) {
  const size_t total = (size_t)nfreq * npix;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    double2 v = cmul(coef, full[i]);
    if (direct) {
      double2 d = direct[i % npix];
      v = make_double2(v.x + d.x, v.y + d.y);
    }
    out[i] = v;
  }
}

int launch_exit_combine(double2* out, const double2* full, const double2* direct, double2 coef,
                        int nfreq, int npix, cudaStream_t st) {
  size_t total = (size_t)nfreq * npix;
  COUNT_LAUNCH();
  k_exit_combine<<<grid1d(total), 256, 0, st>>>(out, full, direct, coef, nfreq, npix);
  return (int)cudaGetLastError();
}

__global__ void k_embed_box(double2* full, const double2* box, int nfreq, int nx, int ny, int nbx,
                            int nby, int bx0, int by0) {
  const size_t total = (size_t)nfreq * nx * ny;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const int x = (int)(i % nx);
    const int y = (int)((i / nx) % ny);
    const size_t f = i / ((size_t)nx * ny);
    const int ix = x - bx0, iy = y - by0;
    double2 v = make_double2(0.0, 0.0);
    if (ix >= 0 && ix < nbx && iy >= 0 && iy < nby) v = box[(f * nby + iy) * nbx + ix];
    full[i] = v;
  }
}

int launch_embed_box(double2* full, const double2* box, int nfreq, int nx, int ny, int nbx, int nby,
                     int bx0, int by0, cudaStream_t st) {
  size_t total = (size_t)nfreq * nx * ny;
  COUNT_LAUNCH();
  k_embed_box<<<grid1d(total), 256, 0, st>>>(full, box, nfreq, nx, ny, nbx, nby, bx0, by0);
  return (int)cudaGetLastError();
}

template <typename C>
__global__ void k_broadcast(C* state, const double2* init, int nfreq, size_t per) {
  const size_t total = (size_t)nfreq * per;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x)
    state[i] = from_d<C>(init[i % per]);
}

int launch_broadcast_state(bool fp64, void* state, const double2* init, int nfreq, size_t per,
                           cudaStream_t st) {
  size_t total = (size_t)nfreq * per;
  if (fp64) { COUNT_LAUNCH(); k_broadcast<double2><<<grid1d(total), 256, 0, st>>>((double2*)state, init, nfreq, per); }
  else { COUNT_LAUNCH(); k_broadcast<float2><<<grid1d(total), 256, 0, st>>>((float2*)state, init, nfreq, per); }
  return (int)cudaGetLastError();
}

__global__ void k_beta2(double* beta2, const double2* E, int npix, double scale) {
  __shared__ double red[256];
  const int f = blockIdx.x;
  double s = 0.0;
  for (int i = threadIdx.x; i < npix; i += blockDim.x) {
    double2 v = E[(size_t)f * npix + i];
    s += v.x * v.x + v.y * v.y;
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) beta2[f] = red[0] * scale;
}

int launch_beta2(double* beta2, const double2* E, int nfreq, int npix, double scale, cudaStream_t st) {
  if (nfreq <= 0) return 0;
  COUNT_LAUNCH();
  k_beta2<<<nfreq, 256, 0, st>>>(beta2, E, npix, scale);
  return (int)cudaGetLastError();
}

template <typename C>
__global__ void k_maxabs(unsigned long long* out, const C* data, size_t n) {
  __shared__ double red[256];
  double m = 0.0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    double2 v = to_d(data[i]);
    m = fmax(m, hypot(v.x, v.y));
  }
  red[threadIdx.x] = m;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + w]);
    __syncthreads();
  }
  // non-negative doubles order like their bit patterns
  if (threadIdx.x == 0) atomicMax(out, (unsigned long long)__double_as_longlong(red[0]));
}

int launch_maxabs(double* d_out, const void* data, bool fp64, size_t n, cudaStream_t st) {
  cudaMemsetAsync(d_out, 0, sizeof(double), st);
  unsigned blocks = (unsigned)((n + 255) / 256);
  if (blocks > 1024) blocks = 1024;
  if (blocks < 1) blocks = 1;
  if (fp64) { COUNT_LAUNCH(); k_maxabs<double2><<<blocks, 256, 0, st>>>((unsigned long long*)d_out, (const double2*)data, n); }
  else { COUNT_LAUNCH(); k_maxabs<float2><<<blocks, 256, 0, st>>>((unsigned long long*)d_out, (const float2*)data, n); }
  return (int)cudaGetLastError();
}

// ---------------------------------------------------------------------------
// 1D propagator solvers: the field at every pixel bounces independently
// (prop = propagator1D multiplies by exp(-i k0 dz) and applies no mask).
// FP64 for both precisions.
// ---------------------------------------------------------------------------
__global__ void k_rfp1d(Rfp1dArgs a) {
  const size_t total = (size_t)a.nfreq * a.npix;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
    const int f = (int)(t / a.npix);
    const int p = (int)(t % a.npix);
    const int nd = a.nd;
    const double2* ph = a.phase + (size_t)f * nd;
    double2* S = (double2*)a.state;
    if (a.kind == 0) {
      // cheerleader (src/boost_fractor_recurprop.jl:226-363); exits in out[f][0]=right, [1]=left
      auto s_at = [&](int j) -> double2& { return S[((size_t)f * nd + j) * a.npix + p]; };
      double2* outR = a.out + ((size_t)f * 2 + 0) * a.npix + p;
      double2* outL = a.out + ((size_t)f * 2 + 1) * a.npix + p;
      auto em = [&](int j, int d) { return a.emit[((size_t)j * 2 + d) * a.npix + p]; };
      auto cf = [&](int i, int k) { return a.coef[4 * i + k]; };  // r_r, t_l, r_l, t_r
      if (a.do_init) {
        for (int j = 0; j < nd; ++j) s_at(j) = em(j, 0);
        for (int i = 1; i <= nd - 2; ++i) {
          s_at(i) = cmul(s_at(i), ph[i]);
          s_at(i + 1) = cadd(s_at(i + 1), cmul(cf(i, 3), s_at(i)));
          s_at(i) = cmul(s_at(i), cf(i, 0));
        }
        for (int j = 0; j <= nd - 2; ++j) s_at(j) = cadd(s_at(j), em(j, 1));
        s_at(nd - 2) = cadd(s_at(nd - 2), cmul(cf(nd - 2, 1), em(nd - 1, 1)));
        s_at(nd - 1) = cadd(s_at(nd - 1), cmul(cf(nd - 2, 2), em(nd - 1, 1)));
        *outR = s_at(nd - 1);
        *outL = s_at(0);
        // the exit regions live in out[] from here on
        s_at(nd - 1) = make_double2(0.0, 0.0);
        s_at(0) = make_double2(0.0, 0.0);
      }
      double2 eR = *outR, eL = *outL;
      for (int n = a.n_begin; n < a.n_end; ++n) {
        double2 f1 = cmul(s_at(1), ph[1]);
        eL = cadd(eL, cmul(cf(0, 1), f1));
        s_at(1) = cmul(f1, cf(0, 2));
        for (int i = 1; i <= nd - 3; ++i) {
          double2 fi = cmul(s_at(i), ph[i]);
          double2 fn = cmul(s_at(i + 1), ph[i + 1]);
          s_at(i + 1) = cadd(cmul(cf(i, 2), fn), cmul(cf(i, 3), fi));
          s_at(i) = cadd(cmul(cf(i, 0), fi), cmul(cf(i, 1), fn));
        }
        const int i = nd - 2;
        double2 fi = cmul(s_at(i), ph[i]);
        eR = cadd(eR, cmul(cf(i, 3), fi));
        s_at(i) = cmul(fi, cf(i, 0));
      }
      *outR = eR;
      *outL = eL;
    } else {
      // dancer (src/boost_fractor_recurprop.jl:25-146): nd trimmed regions,
      // boundaries 0..nd with r[nd] = 0 appended; coef[i].x = r[i]
      auto s_at = [&](int j, int d) -> double2& { return S[(((size_t)f * nd + j) * 2 + d) * a.npix + p]; };
      for (int n = a.n_begin; n < a.n_end; ++n) {
        const int rm = (n + a.rm_phase) & 1, lm = rm ^ 1;
        for (int i = 0; i <= nd; ++i) {
          if (i > 0) s_at(i - 1, rm) = cmul(s_at(i - 1, rm), ph[i - 1]);
          if (i < nd) s_at(i, lm) = cmul(s_at(i, lm), ph[i]);
          const double2 r = a.coef[4 * i];
          const double2 one_p = make_double2(1.0 + r.x, r.y), one_m = make_double2(1.0 - r.x, -r.y);
          const double2 mr = make_double2(-r.x, -r.y);
          if (i == 0) {
            s_at(0, lm) = cmul(s_at(0, lm), mr);
          } else if (i == nd) {
            double2 e = cmul(one_p, s_at(nd - 1, rm));
            double2* o = a.out + ((size_t)f * a.nout + (a.per_iter_out ? n : 0)) * a.npix + p;
            if (a.per_iter_out) *o = e;
            else *o = cadd(*o, e);
            s_at(nd - 1, rm) = cmul(s_at(nd - 1, rm), r);
          } else {
            double2 c = s_at(i - 1, rm);
            s_at(i - 1, rm) = cadd(cmul(r, c), cmul(one_m, s_at(i, lm)));
            s_at(i, lm) = cadd(cmul(mr, s_at(i, lm)), cmul(one_p, c));
          }
        }
      }
    }
  }
}

int launch_rfp1d(bool fp64, const Rfp1dArgs& a, cudaStream_t st) {
  (void)fp64;
  size_t total = (size_t)a.nfreq * a.npix;
  unsigned blocks = (unsigned)((total + 127) / 128);
  if (blocks < 1) blocks = 1;
  COUNT_LAUNCH();
  k_rfp1d<<<blocks, 128, 0, st>>>(a);
  return (int)cudaGetLastError();
}

}  // namespace bf
