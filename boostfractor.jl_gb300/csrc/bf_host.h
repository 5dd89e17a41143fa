// Host-side objects of the library: the handle (stream, allocations, error
// state) and resident disk stacks.  Geometry is evaluated in FP64 on the host
// exactly as the reference does (masks with strict/non-strict comparisons,
// Fresnel coefficients, dance_intro amplitudes); this file is compiled with
// -ffp-contract=off so the results match on x86-64 and aarch64.
#pragma once

#include <atomic>
#include <complex>
#include <mutex>
#include <cstdint>
#include <string>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "bf_device.cuh"

using cd = std::complex<double>;

struct bf_handle {
  int device = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t user_stream = nullptr;  // set by bf_set_stream; work goes there when non-null
  int sm_cap = 0;   // > 0: persistent kernels launch at most this many CTAs (SMs left to other streams)
  unsigned long long budget = 0;       // 0 = unlimited
  unsigned long long used = 0;
  std::unordered_map<void*, size_t> allocs;
  std::string err;
  double* d_scalar = nullptr;          // 8-byte reduction target
  // profiling of the last solve (bf_set_profiling / bf_last_profile)
  int profiling = 0;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  double prof[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  int prof_valid = 0;
  unsigned long long prof_launch0 = 0;
  cudaStream_t stream() const { return user_stream ? user_stream : own_stream; }
  // allocs/used may be changed by another thread that trims a stack whose
  // workspace this handle allocated (the serving engine's eviction)
  std::mutex alloc_mu;
};

int bf_dalloc(bf_handle* h, void** p, size_t bytes);
void bf_dfree(bf_handle* h, void* p);

// Device buffer owned by a handle; grows on demand and is reused across calls.
struct DBuf {
  bf_handle* h = nullptr;
  void* p = nullptr;
  size_t n = 0;
  DBuf() = default;
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  DBuf(DBuf&& o) noexcept : h(o.h), p(o.p), n(o.n) { o.p = nullptr; o.h = nullptr; o.n = 0; }
  DBuf& operator=(DBuf&& o) noexcept {
    if (this != &o) { release(); h = o.h; p = o.p; n = o.n; o.p = nullptr; o.h = nullptr; o.n = 0; }
    return *this;
  }
  ~DBuf() { release(); }
  int alloc(bf_handle* hh, size_t bytes) {
    release();
    h = hh;
    n = bytes;
    return bf_dalloc(h, &p, bytes);
  }
  // keep the allocation if it is large enough
  int ensure(bf_handle* hh, size_t bytes) {
    if (p && h == hh && n >= bytes) return 0;
    return alloc(hh, bytes);
  }
  void release() {
    if (h && p) bf_dfree(h, p);
    p = nullptr;
    n = 0;
  }
  template <typename T> T* as() const { return reinterpret_cast<T*>(p); }
};

// The bounce-stage launches of one solve, captured as a CUDA graph when the
// same launch sequence (plan, frequency batch, precision, buffers, handle)
// comes a second time, and replayed from then on with one graph launch.
struct StageGraph {
  cudaGraphExec_t exec = nullptr;
  int device = 0;
  std::string key;      // launch sequence that exec replays
  std::string pending;  // sequence run once uncaptured
  unsigned long long launches = 0;
  unsigned long long replays = 0;
  StageGraph() = default;
  StageGraph(const StageGraph&) = delete;
  StageGraph& operator=(const StageGraph&) = delete;
  void reset() {
    if (exec) {
      int prev = 0;
      cudaGetDevice(&prev);
      cudaSetDevice(device);
      cudaGraphExecDestroy(exec);
      cudaSetDevice(prev);
    }
    exec = nullptr;
    key.clear();
  }
  ~StageGraph() { reset(); }
};

// Per-stack device workspace reused across solves (no allocation on the
// steady-state path) and the cached bounce plan.
struct Workspace {
  DBuf freq, reg, phasor, tidx, tregs, tilt, init, state, add, coef, exitacc, steps, tmp, beta, mg;
  DBuf exit_full[2], direct[2];
  std::string plan_key;  // solver/nmax/emission of the cached plan
  std::vector<size_t> stage_off, stage_len;
  int nslots = 0, ntab = 0, ntilt = 0, nexit = 0, nadd = 0;
  std::vector<int> exit_region;
  std::vector<std::complex<double>> exit_coef;
  std::vector<int> has_direct;
  int tables_nf = -1;          // frequency batch the tables were built for
  std::vector<double> tables_freqs;
  int tables_fp64 = -1;
  unsigned long long tables_version = ~0ull;
  long long props_per_freq = 0;  // propagations in the fused stages, per frequency
  StageGraph graph;              // declared last: destroyed before the buffers it reads
};

struct bf_stack {
  int nd = 0, nx = 0, ny = 0;
  std::vector<double> distance, tilt_x, tilt_y;
  std::vector<cd> r, eps;          // r[nd-1], eps[nd]
  std::vector<cd> surf;            // [region][ny][nx] (empty = all zero)
  std::vector<uint8_t> surf_nonzero;  // [region]
  std::vector<double> X, Y, kX, kY;
  double diskR = 0.0;
  // strict propagator mask abs(x^2+y^2) < diskR^2 (src/boost_fractor.jl:159)
  std::vector<uint8_t> mask_full;  // [ny][nx]
  int bx0 = 0, by0 = 0, nbx = 0, nby = 0;
  std::vector<uint8_t> mask_box;   // [nby][nbx]
  bool kx_sym = false;             // kX, kY antisymmetric -> folded phasor tables
  // device copies
  double *dX = nullptr, *dY = nullptr, *dkX = nullptr, *dkY = nullptr;
  uint8_t *d_mask_full = nullptr, *d_mask_box = nullptr;
  double2* d_surf = nullptr;       // [region][ny][nx] or null
  bf::RegionGeo* d_geo = nullptr;  // [region]
  Workspace* ws = nullptr;
  unsigned long long geo_version = 0;  // bumps when the geometry changes
  // requests of a serving engine queued or running on the stack (a copy of
  // the stack starts with none)
  struct UseCount {
    std::atomic<int> n{0};
    UseCount() = default;
    UseCount(const UseCount&) {}
    UseCount& operator=(const UseCount&) { return *this; }
  } server_uses;
  void* tf_cache = nullptr;            // transformer setup (mode FFT overlaps) of this stack
  void (*tf_cache_delete)(void*) = nullptr;
  size_t (*tf_cache_bytes)(const void*) = nullptr;
};

// Device bytes held by a stack: geometry, bounce-loop workspace and the
// transformer's cached overlaps.
size_t bf_stack_device_bytes(const bf_stack* s);
// Release a stack's workspace and transformer cache (the geometry stays); the
// next solve rebuilds them.  The stack must be idle.
void bf_stack_trim(bf_stack* s);
int bf_pool_reserve(bf_handle* h, size_t bytes);
// Upper bound of the device bytes one solve adds to a stack (workspace,
// per-call buffers, outputs): solver 0 cheerleader, 1 dancer, 2 transformer
// with nm modes.
// Frequencies, regions, modes and stack of a propagation-matrix grid.
void bf_pgrid_shape(const bf_pgrid* g, int* nf, int* nd, int* nm, bf_stack** stack);
// Serving-engine requests queued or running on a mode basis (delta +1 / -1);
// bf_modes_destroy refuses while any are.
void bf_modes_server_use(bf_modes* m, int delta);
// Autotuner switch (bf_autotune) and its log of decisions (bf_autotune_report).
bool bf_autotune_enabled();
void bf_tune_log(const std::string& line);
size_t bf_solve_bytes_estimate(const bf_stack* s, int solver, int nf, int nm, int prop_kind, int precision);

namespace bfhost {

// Host geometry (FP64, reference semantics).
std::vector<uint8_t> strict_mask(const std::vector<double>& X, const std::vector<double>& Y, double R);
// dance_intro (src/boost_fractor_recurprop.jl:153-201) for regions eps[0..n-1]
// with mirror flag r0 == 1; out[n][2][ny][nx]
void dance_intro(const std::vector<cd>& eps, cd r0, const std::vector<double>& X,
                 const std::vector<double>& Y, double diskR, std::vector<cd>& out);
cd eps_cast(cd e);  // real eps -> re - 0.0im

}  // namespace bfhost
