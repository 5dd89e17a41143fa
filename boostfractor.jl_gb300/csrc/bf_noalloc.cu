// bf_propagate_noalloc: the per-op propagator on a field that already lives
// in device memory, with every piece of workspace in one static device array.
//
// Why a caller cannot allocate.  The library's other entry points take their
// workspace from cudaMalloc through the handle (DBuf / bf_dalloc) and free it
// with cudaFree.  Some callers cannot accept either call on their path:
//   * an optimiser or control loop that re-propagates a field thousands of
//     times per second with its own, pre-sized device pool: cudaFree waits for
//     the whole device to go idle, which stalls every other stream of the
//     process, and cudaMalloc can fail with out-of-memory in the middle of a
//     run once a neighbour (a co-resident solve, another framework's caching
//     allocator) holds the rest of HBM;
//   * code that runs while another library owns the allocator policy of the
//     process (a Julia CuArray pool, a PyTorch caching allocator) and must not
//     create allocations behind its back.
// For those callers this entry point allocates nothing on the device and
// nothing on the host on its success path; a failure only records its message
// in the handle's error string.
//
// Limits and rules:
//   * nx, ny <= BF_NOALLOC_MAX_N (256): the scratch below is sized for a
//     256 x 256 grid (about 2.1 MiB of static device memory per device).
//     Larger grids are rejected with BF_ERR_INVALID.
//   * The first call on a device performs the set-up: with that device
//     current it resolves the scratch's device address with
//     cudaGetSymbolAddress (which also loads this module's device globals if
//     the runtime deferred that) and caches it for the device.
//   * The host arrays X, Y, kX, kY (and the surface map of the 3D kind) are
//     copied into the scratch with cudaMemcpyAsync on the handle's stream.
//     From pageable memory the runtime stages them before the call returns;
//     from pinned memory the copy is asynchronous, so pinned arrays must stay
//     valid and unchanged until the stream has reached this call's work.
//   * There is ONE scratch per device, shared by every handle and thread of the
//     process.  Calls that overlap in time on the same device (different
//     streams, different host threads) race on it and give wrong results;
//     serialise them, e.g. by issuing them all on one stream.
//   * What must start at zero: nothing.  Every scratch byte a call reads is
//     written earlier in the same call (coordinates, frequency, mask, surface
//     map, the momentum-space roll buffer), so no clearing is needed between
//     calls; the surface map is read only by the 3D kind, and only when the
//     caller passes a non-zero one.
#include <math.h>

#include <cmath>
#include <complex>
#include <mutex>

#include "../../include/boostfractor_gb300.h"
#include "bf_common.cuh"
#include "bf_device.cuh"
#include "bf_host.h"

int bf_fail(bf_handle* h, int code, const std::string& msg);

namespace {

constexpr int kMaxN = BF_NOALLOC_MAX_N;
constexpr size_t kMaxPix = (size_t)kMaxN * kMaxN;
constexpr size_t kAlign = 256;
constexpr size_t round_up(size_t v) { return (v + kAlign - 1) / kAlign * kAlign; }
// byte offsets inside the scratch
constexpr size_t kOffX = 0;
constexpr size_t kOffY = kOffX + round_up(sizeof(double) * kMaxN);
constexpr size_t kOffKX = kOffY + round_up(sizeof(double) * kMaxN);
constexpr size_t kOffKY = kOffKX + round_up(sizeof(double) * kMaxN);
constexpr size_t kOffFreq = kOffKY + round_up(sizeof(double) * kMaxN);
constexpr size_t kOffSurf = kOffFreq + round_up(sizeof(double));
constexpr size_t kOffTmp = kOffSurf + round_up(sizeof(double2) * kMaxPix);
constexpr size_t kOffMask = kOffTmp + round_up(sizeof(double2) * kMaxPix);
constexpr size_t kScratchBytes = kOffMask + round_up(kMaxPix);

constexpr int kMaxDevices = 64;

}  // namespace

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// Disk mask with the host's exact FP64 operations: |x^2 + y^2| < R^2, each
// product and the sum rounded separately (no contraction), as the propagator's
// mask of src/boost_fractor.jl:150-151.
__global__ void k_noalloc_mask(unsigned char* mask, const double* X, const double* Y, int nx, int ny,
                               double R2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nx * ny) return;
  const int x = i % nx, y = i / nx;
  const double s = __dadd_rn(__dmul_rn(X[x], X[x]), __dmul_rn(Y[y], Y[y]));
  mask[i] = fabs(s) < R2 ? 1 : 0;
}

// The frequency into the scratch, passed by value (no host buffer to keep alive).
__global__ void k_noalloc_set_freq(double* dst, double freq) { *dst = freq; }

// Device address of the scratch for `device`, resolved once per device.
static int scratch_of(bf_handle* h, int device, unsigned char** out) {
  static std::mutex mu;
  static unsigned char* ptr[kMaxDevices] = {};
  if (device < 0 || device >= kMaxDevices)
    return bf_fail(h, BF_ERR_UNSUPPORTED, "bf_propagate_noalloc: device ordinal beyond 63");
  std::lock_guard<std::mutex> lock(mu);
  if (!ptr[device]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return bf_fail(h, BF_ERR_CUDA,
                     std::string("bf_propagate_noalloc: cudaGetSymbolAddress failed: ") + cudaGetErrorString(e));
    ptr[device] = static_cast<unsigned char*>(p);
  }
  *out = ptr[device];
  return BF_OK;
}

#define NK(call)                                                                                   \
  do {                                                                                             \
    const int e_ = (int)(call);                                                                    \
    if (e_ != 0)                                                                                   \
      return bf_fail(h, BF_ERR_CUDA,                                                               \
                     std::string("bf_propagate_noalloc: " #call ": ") + cudaGetErrorString((cudaError_t)e_)); \
  } while (0)

extern "C" int bf_propagate_noalloc(bf_handle* h, int prop_kind, double* E_dev, int nx, int ny,
                                    const double* X, const double* Y, const double* kX, const double* kY,
                                    double dz, double diskR, double eps_re, double eps_im, double tilt_x,
                                    double tilt_y, const double* surface, double lambda) {
  if (!h) return BF_ERR_INVALID;
  if (!E_dev || !X || !Y || !kX || !kY || nx < 1 || ny < 1)
    return bf_fail(h, BF_ERR_INVALID, "bf_propagate_noalloc: null pointer or empty grid");
  if (nx > kMaxN || ny > kMaxN)
    return bf_fail(h, BF_ERR_INVALID,
                   "bf_propagate_noalloc: grid " + std::to_string(nx) + " x " + std::to_string(ny) +
                       " exceeds the static scratch limit of " + std::to_string(kMaxN) + " x " +
                       std::to_string(kMaxN) + "; use bf_propagate");
  if (prop_kind < BF_PROP_3D || prop_kind > BF_PROP_1D)
    return bf_fail(h, BF_ERR_INVALID, "bf_propagate_noalloc: unknown propagator kind");
  if (!(lambda > 0.0) || !std::isfinite(dz))
    return bf_fail(h, BF_ERR_INVALID, "bf_propagate_noalloc: bad lambda or dz");
  NK(cudaSetDevice(h->device));
  cudaPointerAttributes pa;
  NK(cudaPointerGetAttributes(&pa, E_dev));
  if (pa.type != cudaMemoryTypeDevice && pa.type != cudaMemoryTypeManaged)
    return bf_fail(h, BF_ERR_INVALID, "bf_propagate_noalloc: E_dev is not device memory");
  if (pa.type == cudaMemoryTypeDevice && pa.device != h->device)
    return bf_fail(h, BF_ERR_INVALID, "bf_propagate_noalloc: E_dev lives on another device than the handle's");
  unsigned char* sc = nullptr;
  const int rs = scratch_of(h, h->device, &sc);
  if (rs != BF_OK) return rs;

  cudaStream_t st = h->stream();
  const size_t npix = (size_t)nx * ny;
  double* dX = reinterpret_cast<double*>(sc + kOffX);
  double* dY = reinterpret_cast<double*>(sc + kOffY);
  double* dkX = reinterpret_cast<double*>(sc + kOffKX);
  double* dkY = reinterpret_cast<double*>(sc + kOffKY);
  double* dfreq = reinterpret_cast<double*>(sc + kOffFreq);
  double2* dsurf = reinterpret_cast<double2*>(sc + kOffSurf);
  double2* dtmp = reinterpret_cast<double2*>(sc + kOffTmp);
  unsigned char* dmask = sc + kOffMask;

  // Pageable sources are staged by the runtime before cudaMemcpyAsync returns;
  // pinned ones are read when the stream gets there (see the rules above).
  const double freq = 299792458.0 / lambda;
  NK(cudaMemcpyAsync(dX, X, sizeof(double) * nx, cudaMemcpyHostToDevice, st));
  NK(cudaMemcpyAsync(dY, Y, sizeof(double) * ny, cudaMemcpyHostToDevice, st));
  NK(cudaMemcpyAsync(dkX, kX, sizeof(double) * nx, cudaMemcpyHostToDevice, st));
  NK(cudaMemcpyAsync(dkY, kY, sizeof(double) * ny, cudaMemcpyHostToDevice, st));
  bf::note_launch();
  k_noalloc_set_freq<<<1, 1, 0, st>>>(dfreq, freq);
  NK(cudaGetLastError());
  // only the 3D propagator applies a surface map
  bool surf_nonzero = false;
  if (surface && prop_kind == BF_PROP_3D)
    for (size_t i = 0; i < 2 * npix && !surf_nonzero; ++i) surf_nonzero = surface[i] != 0.0;
  if (surf_nonzero) NK(cudaMemcpyAsync(dsurf, surface, sizeof(double2) * npix, cudaMemcpyHostToDevice, st));
  if (prop_kind != BF_PROP_1D) {
    const int nb = (int)((npix + 255) / 256);
    bf::note_launch();
    k_noalloc_mask<<<nb, 256, 0, st>>>(dmask, dX, dY, nx, ny, diskR * diskR);
    NK(cudaGetLastError());
  }

  // The operation sequence of bf_propagate at FP64, on the caller's buffer.
  const cd eps = bfhost::eps_cast(cd(eps_re, eps_im));
  bf::RegionGeo g;
  g.dz = dz;
  g.eps_re = eps.real();
  g.eps_im = eps.imag();
  g.tilt_x = tilt_x;
  g.tilt_y = tilt_y;
  const double scale = 1.0 / ((double)nx * (double)ny);
  void* buf = E_dev;
  void* tmp = dtmp;
  const double2* surf = surf_nonzero ? dsurf : nullptr;
  switch (prop_kind) {
    case BF_PROP_3D:
    case BF_PROP_NOTILTS:
      NK(bf::launch_mul_mask(true, buf, 1, nx, ny, dmask, st));
      NK(bf::launch_line_dft(true, buf, 1, nx, ny, 0, 0, st));
      NK(bf::launch_line_dft(true, buf, 1, nx, ny, 1, 0, st));
      NK(bf::launch_mul_phasor_full(true, buf, 1, nx, ny, dfreq, nullptr, g, dkX, dkY, 0, scale, st));
      NK(bf::launch_line_dft(true, buf, 1, nx, ny, 1, 1, st));
      NK(bf::launch_line_dft(true, buf, 1, nx, ny, 0, 1, st));
      if (prop_kind == BF_PROP_3D)
        NK(bf::launch_mul_tilt_full(true, buf, 1, nx, ny, dfreq, nullptr, g, dX, dY, surf, 0, st));
      break;
    case BF_PROP_MOMENTUM:
      NK(bf::launch_mul_phasor_full(true, buf, 1, nx, ny, dfreq, nullptr, g, dkX, dkY, 1, scale, st));
      NK(bf::launch_roll(true, buf, tmp, 1, nx, ny, -(nx / 2), -(ny / 2), st));
      NK(bf::launch_line_dft(true, tmp, 1, nx, ny, 0, 1, st));
      NK(bf::launch_line_dft(true, tmp, 1, nx, ny, 1, 1, st));
      NK(bf::launch_mul_mask(true, tmp, 1, nx, ny, dmask, st));
      NK(bf::launch_mul_tilt_full(true, tmp, 1, nx, ny, dfreq, nullptr, g, dX, dY, nullptr, 1, st));
      NK(bf::launch_line_dft(true, tmp, 1, nx, ny, 0, 0, st));
      NK(bf::launch_line_dft(true, tmp, 1, nx, ny, 1, 0, st));
      NK(bf::launch_roll(true, tmp, buf, 1, nx, ny, nx / 2, ny / 2, st));
      break;
    case BF_PROP_1D:
      NK(bf::launch_mul_scalar_phase_1d(true, buf, 1, nx, ny, dfreq, nullptr, g, st));
      break;
  }
  return BF_OK;
}
