// Device-side data structures and launcher declarations shared by the host
// engine (bf_api.cu) and the kernels (bf_device.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

namespace bf {

// One step of a bounce stage: two field slots A (left) and B (right) that meet
// at one boundary.  Each slot is optionally propagated through its region,
// then the boundary mixes them:
//   A' = cAA*A~ + cAB*B~ (+ add),   B' = cBA*A~ + cBB*B~
// where X~ is the propagated field (or the raw field if the slot is not
// propagated).  A slot that feeds an exit region also adds its masked,
// pre-propagation input to an FP64 exit accumulator; the exit field is the
// full-grid propagation of that sum (the propagator is linear).
struct StepDesc {
  int sa, sb;        // state slot of A / B, -1 = none
  int ra, rb;        // region of the propagator acting on A / B, -1 = not propagated
  int coef;          // index of the 4 mixing coefficients
  int exitA, exitB;  // exit accumulator index fed by A / B, -1 = none
  int addA;          // additive box term for A' (index), -1 = none
};

// Arguments of one launch of the fused box kernel (a whole stage, all
// frequencies of the batch).
template <typename C>
struct FusedArgs {
  int nfreq;          // frequencies in the batch (grid.y)
  int nbx, nby;       // pruned box (pixels that the disk mask can reach)
  int nslots;         // state slots per frequency
  int ntab;           // regions per frequency in the phasor table
  int fold;           // phasor table stores one quadrant (N/2 x N/2)
  C* state;           // [f][slot][nby][nbx]
  const C* phasor;    // [f][region][N/2][N/2] (fold) or [f][region][N][N], 1/N^2 included
  const C* tilt;      // [f][tilt_idx][nby][nbx]
  const int* tilt_idx;            // [region] -> tilt map index, -1 = identity
  int ntilt;                      // tilt maps per frequency
  const unsigned char* mask;      // [nby][nbx]
  const double2* coefs;           // [coef][4]
  double2* exitacc;               // [exit][f][nby][nbx]
  const C* addbuf;                // [add][nby][nbx] (frequency independent)
  const StepDesc* steps;          // this stage
  int* err;                       // set to 1 if a bounded wait gave up
  C* mg;                          // row tiles of the split-phase path [step][f][2][nby][N+2], or null
  int variant;                    // host side: fused-kernel variant (FusedVariant), 0 = by rule
};

// Variants of the fused stage kernel for stages that do not take the
// split-phase path.  All run the same per-pixel arithmetic in the same order,
// so they give the same results bit for bit; only their speed differs.
enum FusedVariant {
  kFusedRule = 0,       // joint steps when the doubled row tile keeps the CTAs per SM; 512 threads at N = 256 c64
  kFusedSeparate = 1,   // slots propagated one after the other, 256 threads
  kFusedJoint = 2,      // joint steps (both slots' row tiles in shared memory), 256 threads
  kFusedWide = 3,       // slots one after the other, 512 threads (complex64, N = 256)
  kFusedJointLean = 4,  // joint steps, 320 threads, 2 CTAs per SM, shared twiddles (complex64, N = 128)
  kFusedSeparateLean = 5,  // slots one after the other, 256 threads, 3 CTAs per SM, shared twiddles (c64, N = 128)
  kFusedJointStaged = 6,   // joint steps, 256 threads, phasor rows staged by cp.async (complex64, N = 128)
  kFusedSeparateStaged = 7,  // as kFusedSeparateLean, phasor rows staged by cp.async (complex64, N = 128)
  kFusedSeparate160Staged = 8,  // slots one after the other, 160 threads, 3 CTAs per SM, staged rows (c64, N = 128)
};
// The variants valid for a stage of this shape (kFusedRule first).
std::vector<int> fused_variants(int N, int nbx, int nby, bool fp64);

// Launch the fused stage kernel (templated on the grid size N and the field
// precision).  Returns a cudaError_t.
int launch_fused_stage_f(int N, const FusedArgs<float2>& a, int nsteps, cudaStream_t st);
int launch_fused_stage_d(int N, const FusedArgs<double2>& a, int nsteps, cudaStream_t st);
size_t fused_smem_bytes(int N, int nbx, int nby, bool fp64);
// True when the fused kernel's row tiles do not fit in shared memory, so that
// every stage runs the split-phase kernels (tiles in global memory).
bool fused_split_only(int N, int nbx, int nby, bool fp64);
bool fused_supported(int N, int nbx, int nby, bool fp64);
// Split-phase path (stages with fewer steps x frequencies than SMs): the row
// tiles it needs for a stage of nsteps steps, and whether a stage takes it.
size_t split_tile_bytes(int N, int nby, int nfreq, int nsteps, bool fp64);
bool split_stage(int nsteps, int nfreq);

// ---- split-TF32 tensor-core GEMM (bf_tcgemm.cu) --------------------------
// out[z][n][m] (FP32) = sum over the z-th of `splits` K slices of
// (Ahi Bhi + Ahi Blo + Alo Bhi)[m][n]; A [M][Kp], B [N][Kp] row-major FP32
// holding TF32-rounded hi/lo parts, M a multiple of 128, Kp of 32, bases
// 16-byte aligned.  The tensor-memory accumulator is drained into FP32
// registers every 32 K-elements.  *d_err becomes non-zero if a bounded wait in
// the kernel expired.  max_ctas > 0 caps the persistent grid (SMs left to
// other streams); 0 = one CTA per SM.
int tc_gemm_tf32x3(const float* Ahi, const float* Alo, const float* Bhi, const float* Blo, int M, int N, int Kp,
                   int splits, float* out, int* d_err, cudaStream_t st, int max_ctas = 0);
// True when the output tiles of an M x N product alone give every SM about
// four tiles (K slicing then only adds output traffic).
bool tc_gemm_fills_gpu(int M, int N);
// K slices for an M x N x Kp product: enough work units to keep every SM busy.
int tc_gemm_splits(int M, int N, int Kp);
bool tc_gemm_available();

// ---- phasor / tilt tables (FP64 phase arguments) -----------------------
struct RegionGeo {
  double dz;
  double eps_re, eps_im;
  double tilt_x, tilt_y;
};
// phasor[f][t][..] for table regions t (region ids in regions[t]); 1/(N*N) folded in.
int launch_phasor_table(bool fp64, void* out, int nfreq, const double* d_freqs, int ntab,
                        const int* d_regions, const RegionGeo* d_geo, int N, const double* d_kX,
                        const double* d_kY, int fold, cudaStream_t st);
// tilt[f][m][nby][nbx] = exp(-i k0 (tx x + ty y)) * exp(-i k0 surf) for map m of region regions[m]
int launch_tilt_table(bool fp64, void* out, int nfreq, const double* d_freqs, int nmaps,
                      const int* d_regions, const RegionGeo* d_geo, int nbx, int nby, int bx0,
                      int by0, int nx, int ny, const double* d_X, const double* d_Y,
                      const double2* d_surf /* [region][ny][nx] or null */, cudaStream_t st);

// ---- general full-grid path (any nx, ny) --------------------------------
// data [nb][ny][nx] complex, x fastest.
int launch_line_dft(bool fp64, void* data, int nb, int nx, int ny, int axis, int inverse,
                    cudaStream_t st);
int launch_mul_mask(bool fp64, void* data, int nb, int nx, int ny, const unsigned char* d_mask,
                    cudaStream_t st);
// phasor multiply in FFT bin order (fftshift folded): k0 per batch entry from freqs[b] and eps
int launch_mul_phasor_full(bool fp64, void* data, int nb, int nx, int ny, const double* d_freqs,
                           const double* d_lambda, RegionGeo g, const double* d_kX,
                           const double* d_kY, int shifted_layout, double scale, cudaStream_t st);
int launch_mul_tilt_full(bool fp64, void* data, int nb, int nx, int ny, const double* d_freqs,
                         const double* d_lambda, RegionGeo g, const double* d_X, const double* d_Y,
                         const double2* d_surf /* [ny][nx] or null */, int tilt_only_if_nonzero,
                         cudaStream_t st);
int launch_mul_scalar_phase_1d(bool fp64, void* data, int nb, int nx, int ny,
                               const double* d_freqs, const double* d_lambda, RegionGeo g,
                               cudaStream_t st);
int launch_roll(bool fp64, const void* in, void* out, int nb, int nx, int ny, int sx, int sy,
                cudaStream_t st);
int launch_convert(const void* in, bool in_fp64, void* out, bool out_fp64, size_t n,
                   cudaStream_t st);

// ---- box <-> full grid and exit fields ----------------------------------
// out[f][ny][nx] (complex128) = direct[ny][nx] + coef * full[f][ny][nx]
int launch_exit_combine(double2* out, const double2* full, const double2* direct,
                        double2 coef, int nfreq, int npix, cudaStream_t st);
// embed box acc [f][nby][nbx] (FP64) into full grid [f][ny][nx] (FP64)
int launch_embed_box(double2* full, const double2* box, int nfreq, int nx, int ny, int nbx,
                     int nby, int bx0, int by0, cudaStream_t st);
// state[f][slot][..] = init[slot][..] converted, for all f
int launch_broadcast_state(bool fp64, void* state, const double2* init, int nfreq,
                           size_t per_freq, cudaStream_t st);
// beta2[f] = scale * sum |E[f]|^2 (FP64 field)
int launch_beta2(double* beta2, const double2* E, int nfreq, int npix, double scale,
                 cudaStream_t st);
// maxabs over n complex values of either precision, result into *d_out (double)
int launch_maxabs(double* d_out, const void* data, bool fp64, size_t n, cudaStream_t st);

// ---- 1D propagator solvers (every pixel independent) --------------------
struct Rfp1dArgs {
  int kind;          // 0 = cheerleader, 1 = dancer
  int nfreq, npix, nd;
  int n_begin, n_end;  // bounce iterations [n_begin, n_end)
  int do_init;         // run the initial push-forward (cheerleader) before n_begin
  const double2* phase;  // [f][region] exp(-i k0 dz) (FP64)
  const double2* coef;   // [boundary][4]: cheerleader (r_r, t_l, r_l, t_r); dancer (r, ., ., .)
  void* state;           // cheerleader [f][nd][pix]; dancer [f][nd][2][pix]
  const double2* emit;   // [nd][2][pix] emission (FP64)
  double2* out;          // cheerleader: [f][2][pix] (right, left) accumulated exits
                         // dancer: [f][nslots_out][pix]
  int per_iter_out;      // dancer immediatesum = false
  int nout;              // dancer output slots per frequency (nmax+1 or 1)
  int rm_phase;          // dancer: physical index of the right-moving direction at n_begin
};
int launch_rfp1d(bool fp64, const Rfp1dArgs& a, cudaStream_t st);

void init_constant_roots();  // host: fill the unit-root tables (once per device)

// Kernel launches issued by this library since load (for launch accounting).
unsigned long long launch_count();
void note_launch();   // count a launch made outside bf_device.cu
void note_launches(unsigned long long n);   // kernels run by a replayed graph
void unnote_launches(unsigned long long n); // launches recorded into a graph that never ran

}  // namespace bf
