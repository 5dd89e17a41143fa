/*
 * boostfractor_gb300.h -- C ABI of the GB300-native boost-factor solvers.
 *
 * Drop-in boundary for the hot path of BoostFractor.jl: the coordinate
 * system, the boundary setup, the angular-spectrum propagators, the
 * recursive-Fourier-propagation solvers (dancer / cheerleader) and the
 * transfer-matrix mode matching (transformer).  Julia reaches it with
 * `ccall`; Python tests and benches with ctypes.
 *
 * Conventions
 *   - Every entry point returns an int status (BF_OK = 0); the message of the
 *     last failure is available from bf_last_error(handle).  Nothing throws
 *     across the ABI.
 *   - Arrays are the reference's Julia arrays passed as raw pointers:
 *     column-major, ComplexF64 interleaved (re, im) doubles.  A field E is
 *     (nx, ny) with x fastest; relative_surfaces is (nd, nx, ny) with the
 *     region index fastest; emit is (nd, 2, nx, ny).
 *   - Caller-owned host buffers are read or written only during the call.
 *     Device objects (stacks, mode bases) are owned by the handle.
 *   - A handle is not thread-safe: use one handle per host thread.  It owns
 *     one CUDA stream and its device allocations.
 */
#ifndef BOOSTFRACTOR_GB300_H
#define BOOSTFRACTOR_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define BF_OK              0
#define BF_ERR_INVALID     1  /* bad argument: shape mismatch, NaN geometry, null pointer
                                 (reference: DimensionMismatch, src/boost_fractor.jl:105;
                                 error(), src/boost_fractor_transformer.jl:101) */
#define BF_ERR_NOMEM       2  /* device allocation above the handle's HBM budget, or cudaMalloc failed */
#define BF_ERR_CUDA        3  /* a CUDA runtime call failed */
#define BF_ERR_TIMEOUT     4  /* a bounded wait expired */
#define BF_ERR_UNSUPPORTED 5  /* valid request outside what this build implements */
#define BF_ERR_SINGULAR    6  /* an exactly singular propagation matrix or boundary system T22
                                 (an exactly zero pivot); the outputs are still written, with
                                 inf/NaN where the pivot was zero (reference: SingularException
                                 from inv and \, src/boost_fractor_transformer.jl:247,346,356) */

/* ---- propagator plug-ins: the reference's `prop=` keyword ---------------- */
#define BF_PROP_3D       0  /* propagator              src/boost_fractor.jl:137-149 */
#define BF_PROP_NOTILTS  1  /* propagatorNoTilts       src/boost_fractor.jl:157-179 */
#define BF_PROP_MOMENTUM 2  /* propagatorMomentumSpace src/boost_fractor.jl:187-210 */
#define BF_PROP_1D       3  /* propagator1D            src/boost_fractor.jl:218-227 */

/* ---- arithmetic of a solve ---------------------------------------------- */
#define BF_PREC_FP64  0  /* complex128 fields, FP64 transforms (the plain FP64 path) */
#define BF_PREC_MIXED 1  /* complex64 fields and transforms; FP64 phase argument kz*dz,
                            FP64 exit (bounce-sum) accumulation, FP64 final solve.  In
                            the transformer: complex64 propagation matrices and inverses,
                            a double-float chain, and the Hermitian overlap GEMMs on the
                            tensor cores (split TF32, accumulator drained every 32 K) */
#define BF_PREC_TF32  2  /* transformer only: the same as BF_PREC_MIXED (the name of
                            its tensor-core overlap GEMMs) */
#define BF_PREC_MIXED_SIMT 3  /* transformer only, for comparison: BF_PREC_MIXED with the
                            overlap GEMMs on the FP32 SIMT pipes (double-float sums) */

/* ---- flags -------------------------------------------------------------- */
#define BF_OUT_DEVICE 1  /* output pointers are device pointers (results stay in HBM) */
#define BF_IN_DEVICE  2  /* field inputs are device pointers (e.g. BF_OUT_DEVICE results) */

typedef struct bf_handle bf_handle;
typedef struct bf_stack bf_stack;
typedef struct bf_modes bf_modes;

/* Library version (major*10000 + minor*100 + patch). */
int bf_version(void);

/* Create a handle on CUDA device `device`.  `hbm_budget_bytes` caps the
 * device memory the handle may hold (0 = no cap).  One stream per handle. */
int bf_create(int device, unsigned long long hbm_budget_bytes, bf_handle** out);
int bf_destroy(bf_handle* h);
/* Message of the last failed call on this handle ("" if none). */
const char* bf_last_error(const bf_handle* h);
/* Bytes of device memory the handle currently holds. */
unsigned long long bf_device_bytes(const bf_handle* h);

/* Run the handle's work on a caller's CUDA stream (a cudaStream_t passed as
 * void*); NULL returns to the handle's own stream.  No reference counterpart:
 * it lets a caller order the solves with its own device work. */
int bf_set_stream(bf_handle* h, void* cuda_stream);

/* Profiling of the pruned bounce solver.  When enabled, each solve records
 * CUDA events on the handle's stream; bf_last_profile fills out[8] with
 *   [0] device ms of the whole solve, [1] device ms of the bounce stages,
 *   [2] device ms of table setup, [3] device ms of the exit fields and beta^2,
 *   [4] bounce-stage kernel launches, [5] kernel launches of the solve,
 *   [6] propagations run in the bounce stages, [7] frequencies.
 * bf_transformer_1d_batch records [0] = [1] = device ms of its kernel, [5] = 1,
 * [7] = frequencies.  The transformer records [0] whole solve, [1] propagation
 * matrices, [2] inverses, chain and boundary solve, [3] the class-GEMM kernels
 * alone, [4] class-GEMM launches, [5] launches, [6] the class GEMMs' executed
 * real flops (three MMAs per product on the tensor cores), [7] frequencies.
 * Returns BF_ERR_INVALID when the last solve did not record a profile.
 * No reference counterpart (the reference only times with @time). */
int bf_set_profiling(bf_handle* h, int enable);
int bf_last_profile(const bf_handle* h, double* out);

/* ---- host-side geometry helpers (no GPU work) ---------------------------- */
/* get_kspace_coords: dk = 2pi/(2 max X), values -(n-1)/2*dk ... (n-1)/2*dk.
 * Replaces src/boost_fractor.jl:42-47 (used by SeedCoordinateSystem :30-34). */
int bf_get_kspace_coords(int n, const double* real_coords, double* kspace_out);
/* Fresnel reflectivities of SeedSetupBoundaries: r[0] = 1 (mirror),
 * r[i-1] = (sqrt(eps[i-1]) - sqrt(eps[i]))/(sqrt(eps[i-1]) + sqrt(eps[i])), i >= 2
 * (0-based), real eps taken as re - 0.0im.  eps: nd complex, r_out: nd-1 complex.
 * Replaces src/boost_fractor.jl:98-103. */
int bf_fresnel_reflectivities(int nd, const double* eps, double* r_out);

/* gauss_profile(coords; z, omega0, f): the normalised 2D Gaussian beam at
 * distance z from its waist, out (nx, ny) complex.  FP64 on the host.
 * Replaces src/beam_gaussian.jl:24-37. */
int bf_gauss_profile(int nx, int ny, const double* X, const double* Y, double z, double omega0, double f,
                     double* out);

/* ---- antenna coupling ----------------------------------------------------- */
/* unnormalized_match(Eout, Eantenna; dx, dy) for nb fields at once:
 * out[b] = dx dy sum_p E[b][p] conj(Eantenna[p]), E nb x npix complex (device
 * memory with BF_IN_DEVICE), Eantenna npix complex, out nb complex (host).
 * Replaces src/beam_coupling.jl:13-15. */
int bf_unnormalized_match(bf_handle* h, int nb, int npix, const double* E, const double* Eantenna, double dx,
                          double dy, int flags, double* out);

/* ---- per-op propagator: the `prop=` drop-in ------------------------------ */
/* E (nx, ny) complex, propagated in place by distance dz through a medium of
 * permittivity eps, like prop(E0, dz, diskR, eps, tilt_x, tilt_y, surface,
 * lambda, coords).  `surface` is (nx, ny) complex or NULL (= zeros).
 * prop_kind: BF_PROP_*; precision: BF_PREC_*.
 * Replaces src/boost_fractor.jl:137-227. */
int bf_propagate(bf_handle* h, int prop_kind, int precision,
                 double* E, int nx, int ny,
                 const double* X, const double* Y, const double* kX, const double* kY,
                 double dz, double diskR, double eps_re, double eps_im,
                 double tilt_x, double tilt_y, const double* surface, double lambda);

/* ---- propagation without allocation -------------------------------------- */
/* No counterpart in the reference.  The operation of bf_propagate at FP64 on a
 * field E_dev ((nx, ny) complex128, column-major) that already lives in device
 * memory, propagated in place on the handle's stream; the call does not wait
 * for the result.  Every piece of workspace is one static device array per
 * device, so the call makes no cudaMalloc / cudaFree and no other allocation:
 * for callers with a pre-sized device pool, or that must not stall the device
 * with cudaFree's implicit synchronisation.
 *   - nx, ny <= BF_NOALLOC_MAX_N; larger grids return BF_ERR_INVALID.
 *   - The first call on a device does the set-up (cudaGetSymbolAddress of the
 *     scratch with that device current) and caches the address.
 *   - One scratch per device for the whole process: overlapping calls (other
 *     streams, other threads) race on it; serialise them.
 * X, Y, kX, kY, surface are host arrays as in bf_propagate, copied on the
 * handle's stream: pageable ones are staged before the call returns, pinned
 * ones must stay valid and unchanged until the stream has run the call. */
#define BF_NOALLOC_MAX_N 256
int bf_propagate_noalloc(bf_handle* h, int prop_kind, double* E_dev, int nx, int ny,
                         const double* X, const double* Y, const double* kX, const double* kY,
                         double dz, double diskR, double eps_re, double eps_im,
                         double tilt_x, double tilt_y, const double* surface, double lambda);

/* ---- resident disk stacks ------------------------------------------------ */
/* Upload a SetupBoundaries (src/boost_fractor.jl:63-71) and a CoordinateSystem
 * (:21-28) once; the stack stays in HBM until bf_stack_destroy.
 *   nd regions; distance[nd]; r[nd-1] complex; eps[nd] complex (NaN allowed
 *   for the mirror region 0); tilt_x[nd], tilt_y[nd]; surfaces (nd, nx, ny)
 *   complex or NULL (= zeros); X[nx], Y[ny], kX[nx], kY[ny]; diskR. */
int bf_stack_create(bf_handle* h, int nd, const double* distance, const double* r,
                    const double* eps, const double* tilt_x, const double* tilt_y,
                    const double* surfaces, int nx, int ny, const double* X,
                    const double* Y, const double* kX, const double* kY, double diskR,
                    bf_stack** out);
int bf_stack_destroy(bf_handle* h, bf_stack* s);
/* Replace the region distances of a resident stack (optimiser step). */
int bf_stack_set_distance(bf_handle* h, bf_stack* s, const double* distance);
/* No counterpart in the reference.  The bounce-stage launches of a fused
 * solve are captured as a CUDA graph the second time the same launch sequence
 * comes (same plan, frequency batch, precision, workspace and handle) and
 * replayed by later solves, including after bf_stack_set_distance.  replays:
 * solves served by the graph so far; launches: kernels in the graph (0 when
 * none is held).  A stream that the caller is capturing gets plain launches. */
int bf_stack_graph_stats(bf_stack* s, unsigned long long* replays, unsigned long long* launches);

/* ---- recursive Fourier propagation -------------------------------------- */
/* cheerleader for nf frequencies of one resident stack, batched in one solve.
 * emit (nd, 2, nx, ny) complex or NULL (= dance_intro default), reflect
 * (nx, ny) complex or NULL.  Outputs per frequency f: out_right[f] (nx, ny)
 * complex, out_left[f] (if returnboth; else may be NULL), out_beta2[f] =
 * beta2_scale * sum |out_right[f]|^2 (may be NULL; the reference's boost
 * factor uses beta2_scale = dx*dy/(pi diskR^2), test/runtests.jl:74).
 * nmax+1 bounce iterations run while the field maximum stays >= amin.
 * flags: BF_OUT_DEVICE.
 * Replaces src/boost_fractor_recurprop.jl:226-363 (and dance_intro :153-201). */
int bf_stack_cheerleader(bf_handle* h, bf_stack* s, int nf, const double* freqs,
                         double amin, int nmax, int prop_kind, int precision,
                         const double* emit, const double* reflect, int returnboth,
                         double beta2_scale, int flags,
                         double* out_right, double* out_left, double* out_beta2);

/* dancer (legacy two-field bounce loop).  Output out[f] is (nx, ny) complex when
 * returnsum, else (nx, ny, nmax+1) complex per frequency.
 * Replaces src/boost_fractor_recurprop.jl:25-146. */
int bf_stack_dancer(bf_handle* h, bf_stack* s, int nf, const double* freqs,
                    double amin, int nmax, int prop_kind, int precision,
                    const double* emit, const double* reflect, int returnsum,
                    int immediatesum, double beta2_scale, int flags,
                    double* out, double* out_beta2);

/* One-shot forms with host buffers: create a stack, solve, destroy.  Same
 * arguments as bf_stack_create followed by the solver's. */
int bf_cheerleader(bf_handle* h, int nd, const double* distance, const double* r,
                   const double* eps, const double* tilt_x, const double* tilt_y,
                   const double* surfaces, int nx, int ny, const double* X,
                   const double* Y, const double* kX, const double* kY, double diskR,
                   int nf, const double* freqs, double amin, int nmax, int prop_kind,
                   int precision, const double* emit, const double* reflect,
                   int returnboth, double beta2_scale,
                   double* out_right, double* out_left, double* out_beta2);
int bf_dancer(bf_handle* h, int nd, const double* distance, const double* r,
              const double* eps, const double* tilt_x, const double* tilt_y,
              const double* surfaces, int nx, int ny, const double* X,
              const double* Y, const double* kX, const double* kY, double diskR,
              int nf, const double* freqs, double amin, int nmax, int prop_kind,
              int precision, const double* emit, const double* reflect,
              int returnsum, int immediatesum, double beta2_scale,
              double* out, double* out_beta2);

/* ---- transformer: mode basis -------------------------------------------- */
/* SeedModes(coords; ThreeDim, Mmax=M, Lmax=L, diskR, pattern_input, kT_arr):
 * three_dim = 0 gives one mode of ones (the 1D model); otherwise Bessel disk
 * modes J_l(j_{|l|,m} r/R) exp(-i l phi), zero outside r > diskR, unit
 * normalised, in the reference's flat order (m-1)(2L+1)+l+L, or the caller's
 * pattern_input (M, 2L+1, nx, ny, 1) complex with kT (M, 2L+1) complex.
 * At most 64 modes.  Replaces src/boost_fractor_transformer.jl:46-107. */
int bf_modes_create(bf_handle* h, int nx, int ny, const double* X, const double* Y, int three_dim,
                    int M, int L, double diskR, const double* pattern_input, const double* kT,
                    bf_modes** out);
int bf_modes_destroy(bf_handle* h, bf_modes* m);
/* Copy the mode patterns (M, 2L+1, nx, ny, 1) and mode_kt (M, 2L+1) out
 * (either pointer may be NULL); *nm receives M(2L+1). */
int bf_modes_get(bf_handle* h, const bf_modes* m, int* nm, double* patterns, double* kt);
/* Mode coefficients of the masked (r <= diskR), unit-normalised field B
 * ((nx, ny) complex, NULL = uniform), with the axion velocity phase when
 * velocity_x != 0; out: nm complex.  Replaces axion_induced_modes and
 * field2modes (src/boost_fractor_transformer.jl:115-156). */
int bf_axion_induced_modes(bf_handle* h, const bf_modes* m, const double* B, double velocity_x,
                           double diskR, double f, double* out);
/* Field (nx, ny) complex of nm mode coefficients.  Replaces modes2field (:161-167). */
int bf_modes2field(bf_handle* h, const bf_modes* m, const double* coeffs, double* field);

/* ---- transformer: propagation matrices and the transfer-matrix solve ----- */
/* Propagation (mode-mixing) matrices of every region for nf frequencies;
 * out: nf x nd Julia (nm, nm) complex column-major matrices.  The stack's
 * permittivities are used as given (a NaN mirror gives NaN, as in the
 * reference).  Replaces calc_propagation_matrices / propagation_matrix
 * (src/boost_fractor_transformer.jl:174-227, 274-280). */
int bf_calc_propagation_matrices(bf_handle* h, bf_stack* s, bf_modes* m, int nf, const double* freqs,
                                 int prop_kind, int precision, double* out);
/* transformer for nf frequencies of one resident stack (mirror eps NaN taken
 * as 1e30).  emit / reflect: nm complex or NULL (emit NULL = the default
 * axion-induced modes of the stack's diskR); propagation_matrices: NULL, or
 * (pm_per_freq ? nf : 1) x nd Julia (nm, nm) matrices to use instead of
 * computing them.  Outputs: out_boost[f] (nm complex), out_refl[f] (nm complex,
 * when reflect is given), out_beta2[f] = sum |boost|^2.
 * Replaces src/boost_fractor_transformer.jl:238-359. */
int bf_transformer(bf_handle* h, bf_stack* s, bf_modes* m, int nf, const double* freqs,
                   int prop_kind, int precision, const double* emit, const double* reflect,
                   const double* propagation_matrices, int pm_per_freq, double* out_boost,
                   double* out_refl, double* out_beta2);
/* bf_transformer (default emission) for nreq stacks at once that differ only in
 * the distances of their untilted air regions -- e.g. the stacks of several
 * disk-position optimisers at one step of each, the callers of
 * examples/transformer_optim_utilities.jl:99-144.  The stacks must share grid,
 * disk radius, permittivities, tilts and disk thicknesses and carry no surface
 * maps (else BF_ERR_INVALID).  One solve: the air-region overlaps of every
 * request form one GEMM, the disk regions' matrices are computed once, the
 * chains and boundary solves run over all (request, frequency) pairs.
 * Outputs request-major: out_beta2[r nf + f], out_boost[(r nf + f) nm + m]
 * (complex, NULL allowed).  Each request's result equals its own bf_transformer
 * within rounding.  No reference counterpart (the reference solves one stack
 * per call). */
int bf_transformer_group(bf_handle* h, int nreq, bf_stack* const* stacks, bf_modes* m, int nf,
                         const double* freqs, int prop_kind, int precision, double* out_boost,
                         double* out_beta2);

/* The transformer with the antenna coupling fused after the boundary solve:
 * out_coupled[f] = |sum_m conj(boost_m) antenna_m|^2, antenna = the antenna's
 * mode coefficients (field2modes of e.g. gauss_profile), nm complex; the
 * coupled power of the reference's optimiser cost
 * (examples/transformer_optim_utilities.jl:137).  Other arguments as in
 * bf_transformer (mirror eps NaN taken as 1e30); out_beta2 may be NULL. */
int bf_transformer_coupled(bf_handle* h, bf_stack* s, bf_modes* m, int nf, const double* freqs, int prop_kind,
                           int precision, const double* emit, const double* antenna,
                           const double* propagation_matrices, int pm_per_freq, double* out_coupled,
                           double* out_beta2);

/* Batched 1D model: transformer(bdry, coords, SeedModes(coords; ThreeDim=false);
 * prop=propagator1D) (src/boost_fractor_transformer.jl:285-359, the 1D model of
 * src/Analytical1D.py) for nconf spacing configurations x nf frequencies in one
 * launch, FP64.  distances: nconf x nd (configuration-major, each the nd region
 * distances of one booster); eps: nd complex shared by all (NaN mirror taken
 * as 1e30); emit: 1 complex or NULL (= 1, the axion-induced 1D mode).
 * out_boost (nconf x nf complex, or NULL) and out_beta2 (nconf x nf) = |boost|^2. */
int bf_transformer_1d_batch(bf_handle* h, int nconf, int nd, const double* distances, const double* eps, int nf,
                            const double* freqs, const double* emit, double* out_boost, double* out_beta2);

/* transformer_trace_back for nf frequencies: starting from vcat(input_beam,
 * reflected_beam) in the last region, apply G_s blockdiag(P_s, inv(P_s))
 * (+ axion_S_factor [emit; emit] when includes_axion) region by region.
 * reflected_beam, input_beam: nm complex each (nf x nm when beams_per_freq);
 * emit: nm complex or NULL (= the modes of a uniform field in the disk);
 * propagation_matrices as in bf_transformer.  out: per frequency the
 * reference's (nd, 2, nm) complex array, column-major, each region's
 * 2nm-vector stored in that slice's column-major order as the reference's
 * slice assignment does.  The stack's permittivities are used as they are
 * (a NaN mirror gives NaN, as in the reference).
 * Replaces src/boost_fractor_transformer.jl:372-421. */
int bf_transformer_trace_back(bf_handle* h, bf_stack* s, bf_modes* m, int nf, const double* freqs,
                              int prop_kind, int precision, const double* reflected_beam,
                              const double* input_beam, int beams_per_freq, int includes_axion,
                              const double* emit, const double* propagation_matrices, int pm_per_freq,
                              double* out);

/* ---- propagation-matrix grid for optimisers -------------------------------- */
/* calc_propagation_matrices_grid + construct_prop_matrix_interpolation +
 * interpolate_prop_matrix of examples/transformer_optim_utilities.jl:11-91,
 * resident on the device.  The gaps are the regions 1, 3, ..., nd-1 (the
 * reference's ind_gap = 2:2:n_region); at grid point k every gap's distance is
 * the stack's distance + spacing_first + k spacing_step, k < nsp; the other
 * regions are computed once.  The grid is interpolated along the spacing with
 * the cubic B-spline of Interpolations.jl's BSpline(Cubic(Natural(OnCell())))
 * (utilities :64): exact at the grid spacings, second derivative zero at the
 * cell edges half a step beyond the first and last spacing, and defined up to
 * those edges.  The stack and the modes must outlive the grid. */
typedef struct bf_pgrid bf_pgrid;
#define BF_PGRID_MAX_SPACINGS 64
int bf_pgrid_create(bf_handle* h, bf_stack* s, bf_modes* m, int nf, const double* freqs, int nsp,
                    double spacing_first, double spacing_step, int prop_kind, int precision, bf_pgrid** out);
int bf_pgrid_destroy(bf_handle* h, bf_pgrid* g);
/* Interpolated matrices at dist_shift (one shift per disk: gap region 2d+1
 * takes dist_shift[d]; the last region takes 0, as interpolate_prop_matrix
 * does).  out as bf_calc_propagation_matrices: nf x nd Julia (nm, nm) matrices.
 * A shift outside [spacing_first - step/2, last spacing + step/2] (the bounds
 * of the reference's interpolation object) gives BF_ERR_INVALID. */
int bf_pgrid_matrices(bf_handle* h, bf_pgrid* g, const double* dist_shift, double* out);
/* The transformer on the interpolated matrices, without leaving the device:
 * calc_boostfactor_modes (utilities :98-110).  out_boost nf x nm complex and/or
 * out_beta2 nf; emit nm complex or NULL (the axion-induced modes). */
int bf_pgrid_transformer(bf_handle* h, bf_pgrid* g, const double* dist_shift, const double* emit,
                         double* out_boost, double* out_beta2);
/* calc_boostfactor_cost (utilities :130-144, with soft_box_penalty :150-160 and
 * p_norm :211-215): the coupled power cpld[f] = |sum_m conj(boost[f][m])
 * m_reflect[m]|^2 (fused after the boundary solve) and *out_cost =
 * -p_norm(cpld, p) * penalty; 1000.0 without a solve when a shift is not
 * strictly inside the interpolation bounds.  m_reflect nm complex; the
 * reference uses p = -20; out_coupled nf or NULL (not written on the hard
 * penalty). */
int bf_pgrid_cost(bf_handle* h, bf_pgrid* g, const double* dist_shift, const double* m_reflect, double p,
                  double* out_cost, double* out_coupled);

/* ---- serving: a request loop over resident stacks ------------------------ */
/* No counterpart in the reference, whose callers (the optimiser utilities,
 * examples/transformer_optim_utilities.jl:11-144, and @distributed frequency
 * sweeps) call transformer / cheerleader once per candidate geometry.  A server
 * owns n_workers handles (one stream each).  Requests name a resident stack
 * (and mode basis); requests that arrive while others run are admitted as
 * workers and HBM budget free up, and run concurrently on the workers' streams.
 *   - Admission: a request's device footprint (workspace + per-solve buffers,
 *     an upper bound unless footprint_bytes is given) plus the bytes resident
 *     in served stacks plus the running requests' footprints must fit
 *     hbm_budget_bytes (0 = the device's free memory at creation).  Idle
 *     stacks' workspaces are released, least recently used first, to make
 *     room.  A request that cannot fit even alone fails at bf_submit with
 *     BF_ERR_NOMEM.
 *   - Order: requests on one stack run one at a time in submission order;
 *     queued requests on a stack that have the same solver settings and no
 *     geometry change are solved together as one frequency batch.
 *   - Each request reports its own beta^2 (and boost), identical to a solve of
 *     the same stack alone.
 * The stacks and mode bases must outlive the server (bf_server_destroy
 * releases the workspaces it grew on them). */
typedef struct bf_server bf_server;

#define BF_SOLVER_CHEERLEADER 0
#define BF_SOLVER_DANCER      1
#define BF_SOLVER_TRANSFORMER 2
#define BF_SOLVER_PGRID       3  /* bf_pgrid_transformer at the per-disk shifts in `distance`
                                    (the grid's frequencies; `freqs` must match them) */

#define BF_PENDING (-1)          /* request status: queued or running */
#define BF_SERVER_DRYRUN 1       /* schedule without device work: a request
                                    "runs" for nmax microseconds and occupies
                                    footprint_bytes; for testing the scheduler
                                    on machines without a GPU */
#define BF_SERVER_RESERVE_HBM 2  /* map the admission budget (at most the
                                    free memory less 2 GB) into the device's
                                    memory pool at creation, so that no solve
                                    has to grow the pool while others run */

typedef struct bf_request {
  int solver;                  /* BF_SOLVER_* */
  bf_stack* stack;             /* resident stack (bf_stack_create) */
  bf_modes* modes;             /* transformer: resident mode basis; else NULL */
  int nf;                      /* frequency count */
  const double* freqs;         /* nf frequencies [Hz], copied by bf_submit */
  const double* distance;      /* NULL, or nd new region distances set on the stack
                                  before the solve (an optimiser step), copied */
  int nmax;                    /* RFP: nmax + 1 bounce iterations */
  int prop_kind;               /* BF_PROP_* */
  int precision;               /* BF_PREC_* */
  double beta2_scale;          /* RFP: as in bf_stack_cheerleader; 0 = dx dy / (pi diskR^2) */
  double* out_beta2;           /* host, nf doubles, written before completion is reported */
  double* out_boost;           /* transformer: host nf x nm complex, or NULL */
  unsigned long long footprint_bytes;  /* 0 = the server's estimate */
  bf_pgrid* pgrid;             /* BF_SOLVER_PGRID: the grid (its stack is `stack`); else NULL */
  int lane;                    /* 0 = normal, 1 = latency lane (bf_server_set_latency_lane) */
} bf_request;

int bf_server_create(int device, unsigned long long hbm_budget_bytes, int n_workers, int flags,
                     bf_server** out);
/* Cancels queued requests (status BF_ERR_INVALID), waits for running ones,
 * releases the workspaces grown on served stacks and the workers. */
int bf_server_destroy(bf_server* s);
/* No counterpart in the reference.  Requests with lane = 1 run only on the
 * last n_lane workers (at least one worker stays normal), on streams of the
 * device's highest priority, and the other requests only on the normal
 * workers: short interactive requests (an optimiser's steps) are not queued
 * behind long ones and their kernels are scheduled ahead of the others'.
 * The normal workers' persistent tensor-core GEMM leaves the lane's share of
 * the SMs (n_lane / n_workers) free, and normal requests are admitted within
 * 7/8 of the HBM budget (the last eighth is the lane's).  Call once, before
 * the first bf_submit. */
int bf_server_set_latency_lane(bf_server* s, int n_lane);
int bf_submit(bf_server* s, const bf_request* req, unsigned long long* id);
/* Non-blocking: *status = BF_PENDING, or the request's final status (BF_OK or
 * an error code).  Reporting a final status releases the id.  times (NULL or
 * 3 doubles): submit, start and completion time in seconds since the server's
 * creation. */
int bf_poll(bf_server* s, unsigned long long id, int* status, double* times);
/* Blocks up to timeout_ms (< 0: no limit); BF_ERR_TIMEOUT if the request is
 * still pending then (the id stays valid). */
int bf_wait(bf_server* s, unsigned long long id, int timeout_ms, int* status, double* times);
/* out[10] for requests of one solver (BF_SOLVER_*) or all (-1): completed,
 * failed, frequency points, latency p50 / p99 / mean / max [ms], seconds from
 * the first submission to the last completion, requests solved as part of
 * another's batch, stack workspaces released for admission. */
int bf_server_stats(bf_server* s, int solver, double* out);
/* Starts a new statistics window (e.g. after warm-up requests): the counters
 * and latencies of bf_server_stats restart from zero; requests queued or
 * running are counted when they complete. */
int bf_server_reset_stats(bf_server* s);
const char* bf_server_last_error(const bf_server* s);

/* ---- autotuner --------------------------------------------------------------- */
/* No counterpart in the reference.  The first solve of each shape times the
 * fused stage kernel's variants (joint or separate slot propagation, 160,
 * 256, 320 or 512 threads, twiddles in registers or shared memory, 2 or 3 CTAs per SM,
 * phasor rows read from L2 or staged in shared memory;
 * all give the same results bit for bit) on scratch copies of its largest
 * stage, and the tensor-core GEMM's K slicing (1, 2, 4 or 8 slices, for GEMMs
 * whose output tiles do not already fill the GPU), and keeps the fastest per
 * device and shape for the rest of the process.
 * bf_autotune(0) switches this off (rule-based choices), bf_autotune(1) on
 * (the default); returns the previous setting.  bf_autotune_report copies the
 * decisions taken so far, one line each, into out (cap bytes, NUL-terminated)
 * and returns the full length. */
int bf_autotune(int enable);
int bf_autotune_report(char* out, int cap);

/* ---- test hooks ------------------------------------------------------------ */
/* No counterpart in the reference.  Force one fused stage kernel variant
 * (0 = the rule, 1 = separate, 2 = joint, 3 = 512 threads, 4 = joint with
 * 320 threads and shared twiddles, 5 = separate at 3 CTAs per SM with shared
 * twiddles, 6 = joint with phasor rows staged in shared memory, 7 = 5 with
 * staged phasor rows, 8 = separate with 160 threads at 3 CTAs per SM and
 * staged phasor rows; a variant that does not apply to a stage's shape runs
 * the rule;
 * -1 = back to the autotuner) for every later solve of this process, to check
 * that they agree; returns the previous setting. */
int bf_test_force_fused_variant(int variant);
/* No counterpart in the reference.  While `on` is non-zero, the tensor-core
 * overlap GEMM (BF_PREC_TF32) issues no operand copies, so its MMA warp's
 * bounded wait runs out after ~2 s and the solve returns BF_ERR_TIMEOUT with
 * the CUDA context intact: the test of the kernel's bounded waits. */
int bf_test_tc_withhold_loads(int on);

#ifdef __cplusplus
}
#endif
#endif /* BOOSTFRACTOR_GB300_H */
