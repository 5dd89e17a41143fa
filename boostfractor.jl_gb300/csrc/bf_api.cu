// C ABI and host engine of the GB300 boost-factor library.
//
// The engine turns a reference solver call into device work:
//   * geometry (masks, Fresnel coefficients, dance_intro emission) in FP64 on
//     the host, once per resident stack;
//   * phasor tables exp(-i kz dz) and tilt/surface maps with FP64 phase
//     arguments on the device, once per (stack, frequency batch);
//   * the bounce loop as a sequence of stages of the fused box kernel.  The
//     cheerleader's step (n, i) needs step (n, i-1) and step (n-1, i+1), so all
//     steps with equal 2n+i run in one launch (a wavefront over iterations and
//     regions); the dancer's boundaries are independent within an iteration;
//   * the exit fields as one FP64 full-grid propagation of the accumulated
//     exit input per frequency.
// An exact full-grid mode (every propagation on the whole grid, exits summed
// per bounce) covers what the pruned mode cannot: amin != 0, per-bounce dancer
// output, grid sizes that are not powers of two or do not fit shared memory.
#include <math.h>
#include <string.h>

#include <cmath>
#include <functional>
#include <algorithm>
#include <cstring>
#include <atomic>
#include <map>
#include <array>
#include <cstdio>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "../../include/boostfractor_gb300.h"
#include "bf_common.cuh"
#include "bf_device.cuh"
#include "bf_host.h"

using bf::RegionGeo;
using bf::StepDesc;

// ---------------------------------------------------------------------------
// error plumbing and device memory
// ---------------------------------------------------------------------------
static int fail(bf_handle* h, int code, const std::string& msg) {
  if (h) h->err = msg;
  return code;
}
int bf_fail(bf_handle* h, int code, const std::string& msg) { return fail(h, code, msg); }

#define CK(call)                                                                         \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess)                                                               \
      return fail(h, BF_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_) + " (" + \
                  std::string(__FILE__).substr(std::string(__FILE__).find_last_of('/') + 1) + ":" +  \
                  std::to_string(__LINE__) + ")");   \
  } while (0)
#define CKL(call)                                                                        \
  do {                                                                                   \
    int e_ = (call);                                                                     \
    if (e_ != 0)                                                                         \
      return fail(h, BF_ERR_CUDA,                                                        \
                  std::string(#call) + ": " + cudaGetErrorString((cudaError_t)e_));      \
  } while (0)
#define CKS(call)               \
  do {                          \
    int s_ = (call);            \
    if (s_ != BF_OK) return s_; \
  } while (0)

// Device memory comes from one stream-ordered pool per device (allocations
// and frees are ordered on the handle's stream).  Unlike cudaMalloc/cudaFree,
// neither waits for the rest of the device, so handles working on different
// streams (the serving engine's workers) do not serialise each other.  Freed
// blocks stay in the pool for the next request; bf_destroy trims the pool.
// An allocation reuses a block freed on another stream only once that free
// has completed: the pool may not make one worker's stream wait for the work
// another worker has in flight (it grows instead).
static cudaMemPool_t device_pool(int device) {
  static std::mutex mu;
  static cudaMemPool_t pools[64] = {};
  if (device < 0 || device >= 64) return nullptr;
  std::lock_guard<std::mutex> lock(mu);
  if (!pools[device]) {
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    cudaMemPool_t p = nullptr;
    if (cudaMemPoolCreate(&p, &props) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    unsigned long long keep = ~0ull;
    cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep);
    int no = 0;
    cudaMemPoolSetAttribute(p, cudaMemPoolReuseAllowInternalDependencies, &no);
    pools[device] = p;
  }
  return pools[device];
}

int bf_dalloc(bf_handle* h, void** p, size_t bytes) {
  *p = nullptr;
  if (bytes == 0) bytes = 16;
  std::lock_guard<std::mutex> lock(h->alloc_mu);
  if (h->budget && h->used + bytes > h->budget)
    return fail(h, BF_ERR_NOMEM, "device allocation of " + std::to_string(bytes) +
                                     " bytes exceeds the handle's HBM budget");
  cudaMemPool_t pool = device_pool(h->device);
  cudaError_t e = pool ? cudaMallocFromPoolAsync(p, bytes, pool, h->stream()) : cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
    return fail(h, BF_ERR_NOMEM, std::string("device allocation: ") + cudaGetErrorString(e));
  }
  h->allocs[*p] = bytes;
  h->used += bytes;
  return BF_OK;
}

// Grow the device pool to hold `bytes`: allocated and freed at once on h's
// stream (the pool keeps freed memory), so that later allocations are served
// from memory already mapped.
int bf_pool_reserve(bf_handle* h, size_t bytes) {
  cudaMemPool_t pool = device_pool(h->device);
  if (!pool || !bytes) return BF_OK;
  void* p = nullptr;
  if (cudaMallocFromPoolAsync(&p, bytes, pool, h->stream()) != cudaSuccess) {
    cudaGetLastError();
    return fail(h, BF_ERR_NOMEM, "reserving " + std::to_string(bytes) + " bytes in the device pool");
  }
  CK(cudaFreeAsync(p, h->stream()));
  CK(cudaStreamSynchronize(h->stream()));
  return BF_OK;
}

void bf_dfree(bf_handle* h, void* p) {
  if (!p) return;
  std::lock_guard<std::mutex> lock(h->alloc_mu);
  auto it = h->allocs.find(p);
  if (it != h->allocs.end()) {
    h->used -= it->second;
    h->allocs.erase(it);
  }
  if (device_pool(h->device)) cudaFreeAsync(p, h->stream());
  else cudaFree(p);
}

static int upload(bf_handle* h, DBuf& b, const void* src, size_t bytes) {
  CKS(b.alloc(h, bytes));
  if (src && bytes) CK(cudaMemcpyAsync(b.p, src, bytes, cudaMemcpyHostToDevice, h->stream()));
  return BF_OK;
}

// ---------------------------------------------------------------------------
// host geometry
// ---------------------------------------------------------------------------
namespace bfhost {

cd eps_cast(cd e) {
  if (e.imag() == 0.0) return cd(e.real(), -0.0);
  return e;
}

std::vector<uint8_t> strict_mask(const std::vector<double>& X, const std::vector<double>& Y, double R) {
  const size_t nx = X.size(), ny = Y.size();
  std::vector<uint8_t> m(nx * ny);
  const double R2 = R * R;
  for (size_t y = 0; y < ny; ++y)
    for (size_t x = 0; x < nx; ++x) {
      double xx = X[x] * X[x];
      double yy = Y[y] * Y[y];
      double s = xx + yy;
      m[y * nx + x] = fabs(s) < R2 ? 1 : 0;
    }
  return m;
}

void dance_intro(const std::vector<cd>& eps, cd r0, const std::vector<double>& X,
                 const std::vector<double>& Y, double diskR, std::vector<cd>& out) {
  const size_t n = eps.size(), nx = X.size(), ny = Y.size(), npix = nx * ny;
  out.assign(n * 2 * npix, cd(0.0, 0.0));
  std::vector<double> bf(npix);
  const double R2 = diskR * diskR;
  for (size_t y = 0; y < ny; ++y)
    for (size_t x = 0; x < nx; ++x) {
      double xx = X[x] * X[x];
      double yy = Y[y] * Y[y];
      bf[y * nx + x] = (xx + yy) > R2 ? 0.0 : 1.0;   // recurprop.jl:160
    }
  for (size_t k = 0; k < n; ++k) {
    cd ax_r(0.0, 0.0);
    if (k == 0) {
      ax_r = (r0 == cd(1.0, 0.0)) ? cd(-1.0, 0.0) : cd(0.0, 0.0);
    } else {
      cd ei = eps[k - 1], em = eps[k];
      cd den = ei * std::sqrt(em) + em * std::sqrt(ei);
      ax_r = std::sqrt(em) * (1.0 - ei / em) / den;
    }
    cd ei = eps[k];
    cd em = (k == n - 1) ? cd(1.0, 0.0) : eps[k + 1];
    cd den = ei * std::sqrt(em) + em * std::sqrt(ei);
    cd ax_l = std::sqrt(ei) * (1.0 - em / ei) / den;
    for (size_t i = 0; i < npix; ++i) {
      out[(k * 2 + 0) * npix + i] = ax_r * bf[i];
      out[(k * 2 + 1) * npix + i] = ax_l * bf[i];
    }
  }
}

}  // namespace bfhost

static const cd* as_cd(const double* p) { return reinterpret_cast<const cd*>(p); }

static bool all_finite(const double* p, size_t n) {
  for (size_t i = 0; i < n; ++i)
    if (!std::isfinite(p[i])) return false;
  return true;
}

// ---------------------------------------------------------------------------
// handle
// ---------------------------------------------------------------------------
extern "C" int bf_version(void) { return 100; }

extern "C" int bf_create(int device, unsigned long long hbm_budget_bytes, bf_handle** out) {
  if (!out) return BF_ERR_INVALID;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) {
    cudaGetLastError();
    return BF_ERR_CUDA;
  }
  if (device < 0 || device >= ndev) return BF_ERR_INVALID;
  if (cudaSetDevice(device) != cudaSuccess) return BF_ERR_CUDA;
  bf_handle* h = new (std::nothrow) bf_handle();
  if (!h) return BF_ERR_NOMEM;
  h->device = device;
  h->budget = hbm_budget_bytes;
  if (cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete h;
    return BF_ERR_CUDA;
  }
  {
    // the constant root tables are per device; write them once, even when
    // several threads create handles at the same time
    static std::mutex mu;
    static bool roots_ready[64] = {false};
    std::lock_guard<std::mutex> lock(mu);
    if (device < 64 && !roots_ready[device]) {
      bf::init_constant_roots();
      roots_ready[device] = true;
    }
  }
  if (bf_dalloc(h, (void**)&h->d_scalar, 64) != BF_OK) {
    cudaStreamDestroy(h->own_stream);
    delete h;
    return BF_ERR_NOMEM;
  }
  *out = h;
  return BF_OK;
}

extern "C" int bf_destroy(bf_handle* h) {
  if (!h) return BF_ERR_INVALID;
  cudaSetDevice(h->device);
  cudaStreamSynchronize(h->stream());
  cudaMemPool_t pool = device_pool(h->device);
  for (auto& kv : h->allocs) {
    if (pool) cudaFreeAsync(kv.first, h->stream());
    else cudaFree(kv.first);
  }
  h->allocs.clear();
  cudaStreamSynchronize(h->stream());
  if (pool) cudaMemPoolTrimTo(pool, 0);
  for (auto& e : h->ev)
    if (e) cudaEventDestroy(e);
  cudaStreamDestroy(h->own_stream);
  delete h;
  return BF_OK;
}

extern "C" const char* bf_last_error(const bf_handle* h) { return h ? h->err.c_str() : ""; }

extern "C" unsigned long long bf_device_bytes(const bf_handle* h) { return h ? h->used : 0; }

// ---------------------------------------------------------------------------
// host-side helpers of SeedCoordinateSystem / SeedSetupBoundaries
// ---------------------------------------------------------------------------
extern "C" int bf_get_kspace_coords(int n, const double* real_coords, double* out) {
  if (n <= 0 || !real_coords || !out) return BF_ERR_INVALID;
  double mx = real_coords[0];
  for (int i = 1; i < n; ++i) mx = std::max(mx, real_coords[i]);
  const double mink = 2.0 * M_PI / (mx * 2.0);
  const double maxk = mink * (double)(n - 1) / 2.0;
  // -maxk + i*mink evaluated with one rounding (two-product / two-sum)
  for (int i = 0; i < n; ++i) {
    double p = (double)i * mink;
    double pe = fma((double)i, mink, -p);
    double s = -maxk + p;
    double bb = s + maxk;
    double se = (-maxk - (s - bb)) + (p - bb);
    out[i] = s + (se + pe);
  }
  return BF_OK;
}

// gauss_profile (src/beam_gaussian.jl:24-37), FP64 in the reference's order:
// r = sqrt(x^2 + y^2); amplitude omega0/omega(z) exp(-r^2/omega(z)^2);
// phase exp(-i (k z + k r^2 / (2 R(z)) - Psi(z))).
extern "C" int bf_gauss_profile(int nx, int ny, const double* X, const double* Y, double z, double omega0,
                                double f, double* out) {
  if (nx < 1 || ny < 1 || !X || !Y || !out || !(omega0 > 0.0) || !(f > 0.0)) return BF_ERR_INVALID;
  const double lambda = 299792458.0 / f;
  const double k = 2.0 * M_PI / lambda;
  const double zR = M_PI * omega0 * omega0 / lambda;
  const double omega = omega0 * std::sqrt(1.0 + (z / zR) * (z / zR));
  const double Rz = z * (1.0 + (zR / z) * (zR / z));
  const double psi = std::atan(z / zR);
  cd* o = reinterpret_cast<cd*>(out);
  for (int y = 0; y < ny; ++y)
    for (int x = 0; x < nx; ++x) {
      const double r = std::sqrt(X[x] * X[x] + Y[y] * Y[y]);
      const double r2 = r * r;
      const double amp = omega0 / omega * std::exp(-r2 / (omega * omega));
      const double ph = (k * z + k * r2 / (2.0 * Rz)) - psi;
      o[(size_t)y * nx + x] = amp * std::exp(cd(0.0, -ph));
    }
  return BF_OK;
}

extern "C" int bf_fresnel_reflectivities(int nd, const double* eps, double* r_out) {
  if (nd < 2 || !eps || !r_out) return BF_ERR_INVALID;
  cd* r = reinterpret_cast<cd*>(r_out);
  r[0] = cd(1.0, 0.0);
  for (int i = 2; i < nd; ++i) {
    cd a = std::sqrt(bfhost::eps_cast(as_cd(eps)[i - 1]));
    cd b = std::sqrt(bfhost::eps_cast(as_cd(eps)[i]));
    r[i - 1] = (a - b) / (a + b);
  }
  return BF_OK;
}

// ---------------------------------------------------------------------------
// stacks
// ---------------------------------------------------------------------------
static void geo_of(const bf_stack* s, std::vector<RegionGeo>& g) {
  g.resize(s->nd);
  for (int j = 0; j < s->nd; ++j) {
    cd e = s->eps[j];
    g[j].dz = s->distance[j];
    g[j].eps_re = e.real();
    g[j].eps_im = e.imag();
    g[j].tilt_x = s->tilt_x[j];
    g[j].tilt_y = s->tilt_y[j];
  }
}

static void stack_free(bf_handle* h, bf_stack* s) {
  delete s->ws;
  s->ws = nullptr;
  if (s->tf_cache && s->tf_cache_delete) s->tf_cache_delete(s->tf_cache);
  s->tf_cache = nullptr;
  bf_dfree(h, s->dX); bf_dfree(h, s->dY); bf_dfree(h, s->dkX); bf_dfree(h, s->dkY);
  bf_dfree(h, s->d_mask_full); bf_dfree(h, s->d_mask_box); bf_dfree(h, s->d_surf); bf_dfree(h, s->d_geo);
  s->dX = s->dY = s->dkX = s->dkY = nullptr;
  s->d_mask_full = s->d_mask_box = nullptr;
  s->d_surf = nullptr;
  s->d_geo = nullptr;
}

// The copy is stream-ordered after the stack's earlier work on h's stream; a
// copy from pageable memory is staged before cudaMemcpyAsync returns, so the
// local vector may go away without waiting for the stream.
static int stack_upload_geo(bf_handle* h, bf_stack* s) {
  std::vector<RegionGeo> g;
  geo_of(s, g);
  CK(cudaMemcpyAsync(s->d_geo, g.data(), sizeof(RegionGeo) * g.size(), cudaMemcpyHostToDevice, h->stream()));
  return BF_OK;
}

template <typename T>
static int dupload(bf_handle* h, T** dst, const T* src, size_t n) {
  CKS(bf_dalloc(h, (void**)dst, sizeof(T) * n));
  CK(cudaMemcpyAsync(*dst, src, sizeof(T) * n, cudaMemcpyHostToDevice, h->stream()));
  return BF_OK;
}

extern "C" int bf_stack_create(bf_handle* h, int nd, const double* distance, const double* r,
                               const double* eps, const double* tilt_x, const double* tilt_y,
                               const double* surfaces, int nx, int ny, const double* X,
                               const double* Y, const double* kX, const double* kY, double diskR,
                               bf_stack** out) {
  if (!h || !out) return BF_ERR_INVALID;
  *out = nullptr;
  if (nd < 3) return fail(h, BF_ERR_INVALID, "need at least 3 regions (mirror, gap, exit)");
  if (nx < 1 || ny < 1) return fail(h, BF_ERR_INVALID, "empty grid");
  if (!distance || !r || !eps || !tilt_x || !tilt_y || !X || !Y || !kX || !kY)
    return fail(h, BF_ERR_INVALID, "null geometry pointer");
  if (!all_finite(distance, nd) || !all_finite(tilt_x, nd) || !all_finite(tilt_y, nd) ||
      !all_finite(r, 2 * (size_t)(nd - 1)) || !all_finite(X, nx) || !all_finite(Y, ny) ||
      !all_finite(kX, nx) || !all_finite(kY, ny) || !std::isfinite(diskR))
    return fail(h, BF_ERR_INVALID, "non-finite geometry (distance, r, tilt, grid or diskR)");
  for (int j = 1; j < nd; ++j)
    if (!std::isfinite(eps[2 * j]) || !std::isfinite(eps[2 * j + 1]))
      return fail(h, BF_ERR_INVALID, "non-finite permittivity outside the mirror region");
  CK(cudaSetDevice(h->device));
  std::unique_ptr<bf_stack> s(new bf_stack());
  s->nd = nd; s->nx = nx; s->ny = ny; s->diskR = diskR;
  s->distance.assign(distance, distance + nd);
  s->tilt_x.assign(tilt_x, tilt_x + nd);
  s->tilt_y.assign(tilt_y, tilt_y + nd);
  s->r.assign(as_cd(r), as_cd(r) + nd - 1);
  s->eps.resize(nd);
  for (int j = 0; j < nd; ++j) s->eps[j] = bfhost::eps_cast(as_cd(eps)[j]);
  s->X.assign(X, X + nx); s->Y.assign(Y, Y + ny);
  s->kX.assign(kX, kX + nx); s->kY.assign(kY, kY + ny);
  const size_t npix = (size_t)nx * ny;
  s->surf_nonzero.assign(nd, 0);
  if (surfaces) {
    // Julia (nd, nx, ny) column-major -> [region][y][x]
    s->surf.resize((size_t)nd * npix);
    const cd* sc = as_cd(surfaces);
    for (int y = 0; y < ny; ++y)
      for (int x = 0; x < nx; ++x)
        for (int j = 0; j < nd; ++j) {
          cd v = sc[(size_t)j + (size_t)nd * ((size_t)x + (size_t)nx * y)];
          if (!std::isfinite(v.real()) || !std::isfinite(v.imag()))
            return fail(h, BF_ERR_INVALID, "non-finite surface map");
          s->surf[((size_t)j * ny + y) * nx + x] = v;
          if (v != cd(0.0, 0.0)) s->surf_nonzero[j] = 1;
        }
    bool any = false;
    for (int j = 0; j < nd; ++j) any = any || s->surf_nonzero[j];
    if (!any) s->surf.clear();
  }
  // masks and the pruned box
  s->mask_full = bfhost::strict_mask(s->X, s->Y, diskR);
  int x0 = nx, x1 = -1, y0 = ny, y1 = -1;
  for (int y = 0; y < ny; ++y)
    for (int x = 0; x < nx; ++x)
      if (s->mask_full[(size_t)y * nx + x]) {
        x0 = std::min(x0, x); x1 = std::max(x1, x);
        y0 = std::min(y0, y); y1 = std::max(y1, y);
      }
  if (x1 < 0) { x0 = 0; x1 = 0; y0 = 0; y1 = 0; }
  s->bx0 = x0; s->by0 = y0; s->nbx = x1 - x0 + 1; s->nby = y1 - y0 + 1;
  s->mask_box.resize((size_t)s->nbx * s->nby);
  for (int y = 0; y < s->nby; ++y)
    for (int x = 0; x < s->nbx; ++x)
      s->mask_box[(size_t)y * s->nbx + x] = s->mask_full[(size_t)(y + y0) * nx + (x + x0)];
  // phasor symmetry k(N-1-s) = -k(s) (folded quadrant tables)
  auto antisym = [](const std::vector<double>& k) {
    const size_t n = k.size();
    for (size_t i = 0; i < n; ++i) {
      double a = k[i], b = k[n - 1 - i];
      if (fabs(a + b) > 1e-12 * std::max(1.0, fabs(a))) return false;
    }
    return true;
  };
  s->kx_sym = antisym(s->kX) && antisym(s->kY);
  // device copies
  CKS(dupload(h, &s->dX, s->X.data(), nx));
  CKS(dupload(h, &s->dY, s->Y.data(), ny));
  CKS(dupload(h, &s->dkX, s->kX.data(), nx));
  CKS(dupload(h, &s->dkY, s->kY.data(), ny));
  CKS(dupload(h, &s->d_mask_full, s->mask_full.data(), npix));
  CKS(dupload(h, &s->d_mask_box, s->mask_box.data(), s->mask_box.size()));
  if (!s->surf.empty())
    CKS(dupload(h, &s->d_surf, reinterpret_cast<const double2*>(s->surf.data()), s->surf.size()));
  CKS(bf_dalloc(h, (void**)&s->d_geo, sizeof(RegionGeo) * nd));
  CKS(stack_upload_geo(h, s.get()));
  *out = s.release();
  return BF_OK;
}

extern "C" int bf_stack_destroy(bf_handle* h, bf_stack* s) {
  if (!h || !s) return BF_ERR_INVALID;
  // a serving engine's worker may be solving on it (its stream, not h's):
  // freeing the stack's memory now would pull it from under those kernels
  if (s->server_uses.n.load() > 0)
    return fail(h, BF_ERR_INVALID, "stack is in use by a serving engine: destroy the server first");
  cudaStreamSynchronize(h->stream());
  stack_free(h, s);
  delete s;
  return BF_OK;
}

static size_t dbuf_bytes(const DBuf& b) { return b.p ? b.n : 0; }

size_t bf_stack_device_bytes(const bf_stack* s) {
  if (!s) return 0;
  const size_t npix = (size_t)s->nx * s->ny;
  size_t b = sizeof(double) * 2 * ((size_t)s->nx + s->ny) + npix + (size_t)s->nbx * s->nby +
             sizeof(RegionGeo) * s->nd;
  if (s->d_surf) b += sizeof(double2) * s->nd * npix;
  if (const Workspace* w = s->ws) {
    for (const DBuf* d : {&w->freq, &w->reg, &w->phasor, &w->tidx, &w->tregs, &w->tilt, &w->init, &w->state,
                          &w->add, &w->coef, &w->exitacc, &w->steps, &w->tmp, &w->beta, &w->mg, &w->exit_full[0],
                          &w->exit_full[1], &w->direct[0], &w->direct[1]})
      b += dbuf_bytes(*d);
  }
  if (s->tf_cache && s->tf_cache_bytes) b += s->tf_cache_bytes(s->tf_cache);
  return b;
}

void bf_stack_trim(bf_stack* s) {
  if (!s) return;
  delete s->ws;
  s->ws = nullptr;
  if (s->tf_cache && s->tf_cache_delete) s->tf_cache_delete(s->tf_cache);
  s->tf_cache = nullptr;
}

size_t bf_solve_bytes_estimate(const bf_stack* s, int solver, int nf, int nm, int prop_kind, int precision) {
  const size_t npix = (size_t)s->nx * s->ny, plane = (size_t)s->nbx * s->nby;
  const size_t nd = (size_t)s->nd, F = (size_t)std::max(nf, 1);
  const size_t csz = precision == BF_PREC_FP64 ? 16 : 8;
  if (solver == 2) {
    // resident overlaps (orbit-folded k-space W over K orbits, pixel V over
    // the ~Kd support pixels, as real rows of the upper triangle and TF32
    // pairs, or complex128 on the FP64 path); per solve: P, inverses and the
    // chain per (frequency, region), and per column the class GEMM operands
    // (16 B per orbit or support pixel) and outputs
    const size_t m2 = (size_t)nm * nm, rows = ((m2 + nm + 127) / 128) * 128;
    const size_t K = s->kx_sym ? ((size_t)s->nx / 2 + 1) * ((size_t)s->ny / 2 + 1) : npix;
    size_t inmask = 0;
    for (uint8_t v : s->mask_full) inmask += v;
    const size_t Kd = std::min(npix, 2 * inmask + 64);   // modes cut near the disk radius
    size_t nair = 0;
    for (size_t j = 1; j < nd; ++j) nair += s->eps[j].real() == 1.0;
    const size_t ndisk = nd - 1 - nair;
    const size_t cache = s->tf_cache ? 0 : (16 * rows + 8 * rows) * (K + Kd) + 32 * (size_t)nm * npix;
    return cache + F * nd * (16 * 4 * m2 + 64) + F * (nair * (16 * K + 32 * rows) + ndisk * (16 * Kd + 32 * rows)) +
           16 * npix * nm * 2;
  }
  if (prop_kind == BF_PROP_1D) return F * (16 * 4 * nd * npix + 64);
  const size_t slots = 2 * nd + 2;
  // split-phase row tiles: at most (SMs = 160 here, an upper bound) step x
  // frequency pairs of two nby x (N + 2) tiles, or every step's when no stage
  // fits the fused kernel's shared memory
  const bool split_only = bf::fused_split_only(s->nx, s->nbx, s->nby, precision == BF_PREC_FP64);
  const size_t split = (split_only ? nd * F : 160) * 2 * (size_t)s->nby * (s->nx + 2) * csz;
  const size_t fused = F * (csz * (slots * plane + nd * npix + nd * plane) + 16 * (2 * plane + 3 * npix)) + split;
  const size_t full = F * (csz * (slots + 1) * npix + 16 * 3 * npix);
  return std::max(fused, full) + F * 64;
}

extern "C" int bf_stack_graph_stats(bf_stack* s, unsigned long long* replays, unsigned long long* launches) {
  if (!s || !replays || !launches) return BF_ERR_INVALID;
  *replays = s->ws ? s->ws->graph.replays : 0;
  *launches = s->ws && s->ws->graph.exec ? s->ws->graph.launches : 0;
  return BF_OK;
}

extern "C" int bf_stack_set_distance(bf_handle* h, bf_stack* s, const double* distance) {
  if (!h || !s || !distance) return BF_ERR_INVALID;
  if (!all_finite(distance, s->nd)) return fail(h, BF_ERR_INVALID, "non-finite distance");
  s->distance.assign(distance, distance + s->nd);
  s->geo_version++;
  return stack_upload_geo(h, s);
}

// ---------------------------------------------------------------------------
// general full-grid propagation of a batch [nb][ny][nx] through one region
// ---------------------------------------------------------------------------
static int general_prop(bf_handle* h, const bf_stack* s, int kind, bool fp64, void* buf, void* tmp,
                        int nb, const double* d_freqs, int region) {
  const int nx = s->nx, ny = s->ny;
  RegionGeo g;
  g.dz = s->distance[region];
  g.eps_re = s->eps[region].real();
  g.eps_im = s->eps[region].imag();
  g.tilt_x = s->tilt_x[region];
  g.tilt_y = s->tilt_y[region];
  const double2* surf = s->d_surf && s->surf_nonzero[region] ? s->d_surf + (size_t)region * nx * ny : nullptr;
  const double scale = 1.0 / ((double)nx * (double)ny);
  cudaStream_t st = h->stream();
  switch (kind) {
    case BF_PROP_3D:
    case BF_PROP_NOTILTS:
      CKL(bf::launch_mul_mask(fp64, buf, nb, nx, ny, s->d_mask_full, st));
      CKL(bf::launch_line_dft(fp64, buf, nb, nx, ny, 0, 0, st));
      CKL(bf::launch_line_dft(fp64, buf, nb, nx, ny, 1, 0, st));
      CKL(bf::launch_mul_phasor_full(fp64, buf, nb, nx, ny, d_freqs, nullptr, g, s->dkX, s->dkY, 0, scale, st));
      CKL(bf::launch_line_dft(fp64, buf, nb, nx, ny, 1, 1, st));
      CKL(bf::launch_line_dft(fp64, buf, nb, nx, ny, 0, 1, st));
      if (kind == BF_PROP_3D)
        CKL(bf::launch_mul_tilt_full(fp64, buf, nb, nx, ny, d_freqs, nullptr, g, s->dX, s->dY, surf, 0, st));
      return BF_OK;
    case BF_PROP_MOMENTUM:
      CKL(bf::launch_mul_phasor_full(fp64, buf, nb, nx, ny, d_freqs, nullptr, g, s->dkX, s->dkY, 1, scale, st));
      CKL(bf::launch_roll(fp64, buf, tmp, nb, nx, ny, -(nx / 2), -(ny / 2), st));
      CKL(bf::launch_line_dft(fp64, tmp, nb, nx, ny, 0, 1, st));
      CKL(bf::launch_line_dft(fp64, tmp, nb, nx, ny, 1, 1, st));
      CKL(bf::launch_mul_mask(fp64, tmp, nb, nx, ny, s->d_mask_full, st));
      CKL(bf::launch_mul_tilt_full(fp64, tmp, nb, nx, ny, d_freqs, nullptr, g, s->dX, s->dY, nullptr, 1, st));
      CKL(bf::launch_line_dft(fp64, tmp, nb, nx, ny, 0, 0, st));
      CKL(bf::launch_line_dft(fp64, tmp, nb, nx, ny, 1, 0, st));
      CKL(bf::launch_roll(fp64, tmp, buf, nb, nx, ny, nx / 2, ny / 2, st));
      return BF_OK;
    case BF_PROP_1D:
      CKL(bf::launch_mul_scalar_phase_1d(fp64, buf, nb, nx, ny, d_freqs, nullptr, g, st));
      return BF_OK;
    default:
      return fail(h, BF_ERR_INVALID, "unknown propagator kind");
  }
}

int bf_general_prop(bf_handle* h, const bf_stack* s, int kind, bool fp64, void* buf, void* tmp, int nb,
                    const double* d_freqs, int region) {
  return general_prop(h, s, kind, fp64, buf, tmp, nb, d_freqs, region);
}

// ---------------------------------------------------------------------------
// per-op propagator
// ---------------------------------------------------------------------------
extern "C" int bf_propagate(bf_handle* h, int prop_kind, int precision, double* E, int nx, int ny,
                            const double* X, const double* Y, const double* kX, const double* kY,
                            double dz, double diskR, double eps_re, double eps_im, double tilt_x,
                            double tilt_y, const double* surface, double lambda) {
  if (!h) return BF_ERR_INVALID;
  if (!E || !X || !Y || !kX || !kY || nx < 1 || ny < 1)
    return fail(h, BF_ERR_INVALID, "null pointer or empty grid");
  if (precision != BF_PREC_FP64 && precision != BF_PREC_MIXED)
    return fail(h, BF_ERR_INVALID, "unknown precision");
  if (!(lambda > 0.0) || !std::isfinite(dz)) return fail(h, BF_ERR_INVALID, "bad lambda or dz");
  CK(cudaSetDevice(h->device));
  // a one-region stack carrying this call's geometry
  bf_stack s;
  s.nd = 1; s.nx = nx; s.ny = ny; s.diskR = diskR;
  s.distance = {dz}; s.tilt_x = {tilt_x}; s.tilt_y = {tilt_y};
  s.eps = {bfhost::eps_cast(cd(eps_re, eps_im))};
  s.X.assign(X, X + nx); s.Y.assign(Y, Y + ny); s.kX.assign(kX, kX + nx); s.kY.assign(kY, kY + ny);
  const size_t npix = (size_t)nx * ny;
  s.surf_nonzero = {0};
  if (surface) {
    s.surf.assign(as_cd(surface), as_cd(surface) + npix);
    for (auto& v : s.surf) if (v != cd(0.0, 0.0)) s.surf_nonzero[0] = 1;
  }
  s.mask_full = bfhost::strict_mask(s.X, s.Y, diskR);
  DBuf bX, bY, bkX, bkY, bm, bsurf, bfreq, bE, bT, bE64;
  CKS(upload(h, bX, X, sizeof(double) * nx)); s.dX = bX.as<double>();
  CKS(upload(h, bY, Y, sizeof(double) * ny)); s.dY = bY.as<double>();
  CKS(upload(h, bkX, kX, sizeof(double) * nx)); s.dkX = bkX.as<double>();
  CKS(upload(h, bkY, kY, sizeof(double) * ny)); s.dkY = bkY.as<double>();
  CKS(upload(h, bm, s.mask_full.data(), npix)); s.d_mask_full = bm.as<uint8_t>();
  if (s.surf_nonzero[0]) {
    CKS(upload(h, bsurf, s.surf.data(), sizeof(cd) * npix));
    s.d_surf = bsurf.as<double2>();
  }
  const double f = 299792458.0 / lambda;
  CKS(upload(h, bfreq, &f, sizeof(double)));
  const bool fp64 = precision == BF_PREC_FP64;
  const size_t csz = fp64 ? 16 : 8;
  CKS(upload(h, bE64, E, 16 * npix));
  CKS(bE.alloc(h, csz * npix));
  CKS(bT.alloc(h, csz * npix));
  CKL(bf::launch_convert(bE64.p, true, bE.p, fp64, npix, h->stream()));
  CKS(general_prop(h, &s, prop_kind, fp64, bE.p, bT.p, 1, bfreq.as<double>(), 0));
  CKL(bf::launch_convert(bE.p, fp64, bE64.p, true, npix, h->stream()));
  CK(cudaMemcpyAsync(E, bE64.p, 16 * npix, cudaMemcpyDeviceToHost, h->stream()));
  CK(cudaStreamSynchronize(h->stream()));
  s.dX = s.dY = s.dkX = s.dkY = nullptr; s.d_mask_full = nullptr; s.d_surf = nullptr;
  return BF_OK;
}

// ---------------------------------------------------------------------------
// unnormalized_match (src/beam_coupling.jl:13-15), batched over fields
// ---------------------------------------------------------------------------
// out[b] = dx dy sum_p E[b][p] conj(A[p]); one CTA per field, FP64, fixed
// reduction order (a per-thread stride sum, then a tree).
__global__ void k_match(double2* out, const double2* E, const double2* A, size_t npix, double dxdy) {
  __shared__ double2 red[256];
  const double2* e = E + (size_t)blockIdx.x * npix;
  double2 acc = make_double2(0.0, 0.0);
  for (size_t p = threadIdx.x; p < npix; p += blockDim.x) {
    const double2 u = e[p], v = A[p];
    acc.x += u.x * v.x + u.y * v.y;
    acc.y += u.y * v.x - u.x * v.y;
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
  if (threadIdx.x == 0) out[blockIdx.x] = make_double2(red[0].x * dxdy, red[0].y * dxdy);
}

extern "C" int bf_unnormalized_match(bf_handle* h, int nb, int npix, const double* E, const double* Eantenna,
                                     double dx, double dy, int flags, double* out) {
  if (!h) return BF_ERR_INVALID;
  if (nb < 1 || npix < 1 || !E || !Eantenna || !out) return fail(h, BF_ERR_INVALID, "empty or null match input");
  CK(cudaSetDevice(h->device));
  cudaStream_t st = h->stream();
  DBuf dE, dA, dO;
  const double2* pe = reinterpret_cast<const double2*>(E);
  if (!(flags & BF_IN_DEVICE)) {
    CKS(upload(h, dE, E, sizeof(double2) * (size_t)nb * npix));
    pe = dE.as<double2>();
  }
  CKS(upload(h, dA, Eantenna, sizeof(double2) * (size_t)npix));
  CKS(dO.alloc(h, sizeof(double2) * nb));
  bf::note_launch();
  k_match<<<nb, 256, 0, st>>>(dO.as<double2>(), pe, dA.as<double2>(), (size_t)npix, dx * dy);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(out, dO.p, sizeof(double2) * nb, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return BF_OK;
}

// ---------------------------------------------------------------------------
// bounce-loop plans
// ---------------------------------------------------------------------------
struct Coef4 { cd aa, ab, ba, bb; };

struct Plan {
  // slots and stages of the pruned mode
  int nslots = 0;
  std::vector<int> tab_region;             // table index -> region id
  std::vector<std::vector<StepDesc>> stages;
  std::vector<Coef4> coefs;
  std::vector<std::vector<cd>> adds;       // box-sized additive terms (frequency independent)
  std::vector<std::vector<cd>> init;       // per slot, box-sized initial field
  int nexit = 0;
  std::vector<int> exit_region;            // region whose propagator makes exit k
  std::vector<cd> exit_coef;               // coefficient of exit k
  std::vector<std::vector<cd>> exit_direct;// full-grid direct term of exit k (may be empty)
};

static int coef_index(Plan& p, Coef4 c) {
  p.coefs.push_back(c);
  return (int)p.coefs.size() - 1;
}

// Box part of a full-grid field, pre-masked with the strict propagator mask:
// the pruned solver stores fields masked (their next use is a propagation,
// which masks them, src/boost_fractor.jl:159).
static std::vector<cd> box_of(const bf_stack* s, const cd* full) {
  std::vector<cd> b((size_t)s->nbx * s->nby);
  for (int y = 0; y < s->nby; ++y)
    for (int x = 0; x < s->nbx; ++x) {
      const size_t i = (size_t)y * s->nbx + x;
      b[i] = s->mask_box[i] ? full[(size_t)(y + s->by0) * s->nx + (x + s->bx0)] : cd(0.0, 0.0);
    }
  return b;
}

// emit in the solver's region layout [nreg][2][ny][nx] (full grid, FP64)
static void julia_emit_to_planes(const double* emit, int nreg, int nx, int ny, std::vector<cd>& out) {
  const size_t npix = (size_t)nx * ny;
  out.assign((size_t)nreg * 2 * npix, cd(0, 0));
  const cd* e = as_cd(emit);
  for (int y = 0; y < ny; ++y)
    for (int x = 0; x < nx; ++x)
      for (int d = 0; d < 2; ++d)
        for (int j = 0; j < nreg; ++j)
          out[((size_t)j * 2 + d) * npix + (size_t)y * nx + x] =
              e[(size_t)j + (size_t)nreg * ((size_t)d + 2 * ((size_t)x + (size_t)nx * y))];
}

static void julia_field_to_plane(const double* f, int nx, int ny, std::vector<cd>& out) {
  out.assign(as_cd(f), as_cd(f) + (size_t)nx * ny);  // (nx, ny) column-major == [y][x]
}

// Cheerleader emission (src/boost_fractor_recurprop.jl:260-273): [nd][2][npix]
static void cheer_emission(const bf_stack* s, const double* emit, const double* reflect,
                           std::vector<cd>& em) {
  const int nd = s->nd, nx = s->nx, ny = s->ny;
  const size_t npix = (size_t)nx * ny;
  if (reflect) {
    em.assign((size_t)nd * 2 * npix, cd(0, 0));
    std::vector<cd> rf;
    julia_field_to_plane(reflect, nx, ny, rf);
    std::copy(rf.begin(), rf.end(), em.begin() + ((size_t)(nd - 1) * 2 + 1) * npix);
  } else if (emit) {
    julia_emit_to_planes(emit, nd, nx, ny, em);
  } else {
    em.assign((size_t)nd * 2 * npix, cd(0, 0));
    std::vector<cd> eps(s->eps.begin() + 1, s->eps.end()), di;
    bfhost::dance_intro(eps, s->r[0], s->X, s->Y, s->diskR, di);
    std::copy(di.begin(), di.end(), em.begin() + 2 * npix);
  }
}

// Dancer initial fields (src/boost_fractor_recurprop.jl:53-63): trimmed regions [nd-1][2][npix]
static void dancer_emission(const bf_stack* s, const double* emit, const double* reflect,
                            std::vector<cd>& em) {
  const int R = s->nd - 1, nx = s->nx, ny = s->ny;
  const size_t npix = (size_t)nx * ny;
  if (reflect) {
    em.assign((size_t)R * 2 * npix, cd(0, 0));
    std::vector<cd> rf;
    julia_field_to_plane(reflect, nx, ny, rf);
    std::copy(rf.begin(), rf.end(), em.begin() + ((size_t)(R - 1) * 2 + 1) * npix);
  } else if (emit) {
    julia_emit_to_planes(emit, R, nx, ny, em);
  } else {
    std::vector<cd> eps(s->eps.begin() + 1, s->eps.end());
    bfhost::dance_intro(eps, s->r[0], s->X, s->Y, s->diskR, em);
  }
}

// boundary coefficients of the cheerleader (src/boost_fractor_recurprop.jl:241-244)
struct RT { cd r_r, t_l, r_l, t_r; };
static RT rt_of(cd r) { return RT{r, 1.0 - r, -r, 1.0 + r}; }

// Pruned cheerleader plan.  Slot j-1 holds region j (1 <= j <= nd-2); exit 0 =
// right (region nd-1), exit 1 = left (region 0).
static void plan_cheerleader(const bf_stack* s, int nmax, const std::vector<cd>& em, Plan& p) {
  const int nd = s->nd;
  const size_t npix = (size_t)s->nx * s->ny;
  auto E = [&](int j, int d) { return em.data() + ((size_t)j * 2 + d) * npix; };
  p.nslots = nd - 2;
  p.tab_region.clear();
  for (int j = 1; j <= nd - 2; ++j) p.tab_region.push_back(j);  // table index t = j-1
  p.init.resize(p.nslots);
  for (int j = 1; j <= nd - 2; ++j) p.init[j - 1] = box_of(s, E(j, 0));
  std::vector<RT> rt(nd - 1);
  for (int i = 0; i < nd - 1; ++i) rt[i] = rt_of(s->r[i]);
  // exits
  p.nexit = 2;
  p.exit_region = {nd - 2, 1};
  p.exit_coef = {rt[nd - 2].t_r, rt[0].t_l};
  p.exit_direct.resize(2);
  p.exit_direct[0].resize(npix);
  p.exit_direct[1].resize(npix);
  for (size_t i = 0; i < npix; ++i) {
    p.exit_direct[0][i] = E(nd - 1, 0)[i] + rt[nd - 2].r_l * E(nd - 1, 1)[i];
    p.exit_direct[1][i] = E(0, 0)[i] + E(0, 1)[i];
  }
  // additive left-moving emission folded into the push-forward (:290-300)
  p.adds.clear();
  std::vector<int> add_of(nd, -1);
  for (int j = 1; j <= nd - 2; ++j) {
    std::vector<cd> full(npix);
    for (size_t i = 0; i < npix; ++i) {
      cd v = E(j, 1)[i];
      if (j == nd - 2) v += rt[nd - 2].t_l * E(nd - 1, 1)[i];
      full[i] = v;
    }
    p.adds.push_back(box_of(s, full.data()));
    add_of[j] = (int)p.adds.size() - 1;
  }
  p.stages.clear();
  // push-forward (:281-287), sequential over i
  for (int i = 1; i <= nd - 2; ++i) {
    StepDesc d;
    d.sa = i - 1; d.ra = i - 1;
    d.exitA = -1; d.exitB = -1; d.addA = add_of[i];
    d.rb = -1;
    if (i + 1 <= nd - 2) {
      d.sb = i;
      d.coef = coef_index(p, Coef4{rt[i].r_r, 0.0, rt[i].t_r, 1.0});
    } else {
      d.sb = -1;
      d.exitA = 0;
      d.coef = coef_index(p, Coef4{rt[i].r_r, 0.0, 0.0, 0.0});
    }
    p.stages.push_back({d});
  }
  // main loop (:306-355) as wavefront stages tau = 2n + i
  const int c_first = coef_index(p, Coef4{0.0, 0.0, 0.0, rt[0].r_l});
  const int c_last = coef_index(p, Coef4{rt[nd - 2].r_r, 0.0, 0.0, 0.0});
  std::vector<int> c_mid(nd, -1);
  for (int i = 1; i <= nd - 3; ++i)
    c_mid[i] = coef_index(p, Coef4{rt[i].r_r, rt[i].t_l, rt[i].t_r, rt[i].r_l});
  const int imax = nd - 2;
  for (int tau = 0; tau <= 2 * nmax + imax; ++tau) {
    std::vector<StepDesc> st;
    for (int i = tau % 2; i <= imax; i += 2) {
      const int n = (tau - i) / 2;
      if (n < 0 || n > nmax) continue;
      StepDesc d;
      d.exitA = d.exitB = -1; d.addA = -1;
      if (i == 0) {
        d.sa = -1; d.ra = -1;
        d.sb = 0; d.rb = 0; d.exitB = 1; d.coef = c_first;
        if (imax == 0) { /* unreachable: nd >= 3 */ }
      } else if (i == imax) {
        d.sa = i - 1; d.ra = i - 1; d.exitA = 0;
        d.sb = -1; d.rb = -1; d.coef = c_last;
      } else {
        d.sa = i - 1; d.ra = i - 1;
        d.sb = i; d.rb = i; d.coef = c_mid[i];
      }
      st.push_back(d);
    }
    if (!st.empty()) p.stages.push_back(st);
  }
}

// Pruned dancer plan.  Trimmed region jt (= region jt+1) has slots 2jt+d; the
// physical index of the right-moving direction is n % 2.  One exit (right).
static void plan_dancer(const bf_stack* s, int nmax, const std::vector<cd>& em, Plan& p) {
  const int R = s->nd - 1;
  const size_t npix = (size_t)s->nx * s->ny;
  std::vector<cd> rt(R + 1);
  for (int i = 0; i < R; ++i) rt[i] = s->r[i];
  rt[R] = 0.0;
  p.nslots = 2 * R;
  p.tab_region.clear();
  for (int jt = 0; jt < R; ++jt) p.tab_region.push_back(jt + 1);
  p.init.resize(p.nslots);
  for (int jt = 0; jt < R; ++jt)
    for (int d = 0; d < 2; ++d) p.init[2 * jt + d] = box_of(s, em.data() + ((size_t)jt * 2 + d) * npix);
  p.nexit = 1;
  p.exit_region = {R};
  p.exit_coef = {1.0 + rt[R]};
  p.exit_direct.assign(1, std::vector<cd>());
  p.adds.clear();
  p.stages.clear();
  const int c0 = coef_index(p, Coef4{0.0, 0.0, 0.0, -rt[0]});
  const int cR = coef_index(p, Coef4{rt[R], 0.0, 0.0, 0.0});
  std::vector<int> cm(R + 1, -1);
  for (int i = 1; i < R; ++i) cm[i] = coef_index(p, Coef4{rt[i], 1.0 - rt[i], 1.0 + rt[i], -rt[i]});
  for (int n = 0; n <= nmax; ++n) {
    const int rm = n & 1, lm = rm ^ 1;
    std::vector<StepDesc> st;
    for (int i = 0; i <= R; ++i) {
      StepDesc d;
      d.exitA = d.exitB = -1; d.addA = -1;
      if (i == 0) {
        d.sa = -1; d.ra = -1; d.sb = 2 * 0 + lm; d.rb = 0; d.coef = c0;
      } else if (i == R) {
        d.sa = 2 * (R - 1) + rm; d.ra = R - 1; d.exitA = 0; d.sb = -1; d.rb = -1; d.coef = cR;
      } else {
        d.sa = 2 * (i - 1) + rm; d.ra = i - 1;
        d.sb = 2 * i + lm; d.rb = i;
        d.coef = cm[i];
      }
      st.push_back(d);
    }
    p.stages.push_back(st);
  }
}

// ---------------------------------------------------------------------------
// pruned (fused) solve
// ---------------------------------------------------------------------------
static int upload_cd_as(bf_handle* h, DBuf& b, const std::vector<cd>& v) {
  return upload(h, b, v.data(), sizeof(cd) * v.size());
}

static void prof_mark(bf_handle* h, int i) {
  if (!h->profiling) return;
  if (!h->ev[i]) cudaEventCreate(&h->ev[i]);
  cudaEventRecord(h->ev[i], h->stream());
}

// Solve with the fused box kernel.  The plan (stage descriptors, mixing
// coefficients, initial and additive boxes) is cached per stack under
// `key`; the phasor/tilt tables are cached per frequency batch; no device
// memory is allocated once the workspace has grown to the request's size.
// ---------------------------------------------------------------------------
// Autotuner.  The fused stage kernel has variants that give the same results
// bit for bit (FusedVariant: joint or separate slot propagation, 160 to 512
// threads, 2 or 3 CTAs per SM, twiddles in registers or shared memory,
// phasor rows from L2 or staged); which is fastest depends on the grid, the
// box, the precision and the frequency batch.  The first solve of a shape
// (the frequency count rounded up to a power of two) times every valid
// variant on its largest fused stage, three launches each on scratch copies
// of the state and the exit accumulators, and keeps the fastest for that
// shape on that device.  Solves on a stream being captured, and any solve
// while tuning is switched off (bf_autotune(0)), use the rule's choice.
// ---------------------------------------------------------------------------
namespace {
std::mutex g_tune_mu;
std::map<std::array<long long, 6>, int> g_fused_tuned;   // (device, N, nbx, nby, fp64, nf bucket) -> variant
std::vector<std::string> g_tune_log;
std::atomic<int> g_autotune{1};
std::atomic<int> g_force_variant{-1};
}  // namespace

bool bf_autotune_enabled() { return g_autotune.load() != 0; }

void bf_tune_log(const std::string& line) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  if (g_tune_log.size() < 4096) g_tune_log.push_back(line);
}

extern "C" int bf_autotune(int enable) { return g_autotune.exchange(enable ? 1 : 0); }

extern "C" int bf_autotune_report(char* out, int cap) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  std::string all;
  for (const auto& l : g_tune_log) all += l + "\n";
  if (out && cap > 0) {
    const size_t n = std::min(all.size(), (size_t)cap - 1);
    std::memcpy(out, all.data(), n);
    out[n] = 0;
  }
  return (int)all.size();
}

extern "C" int bf_test_force_fused_variant(int v) { return g_force_variant.exchange(v); }

template <typename C>
static int fused_autotune(bf_handle* h, const Workspace& w, const bf::FusedArgs<C>& a, int N, bool fp64,
                          cudaStream_t st, int* out) {
  *out = bf::kFusedRule;
  if (g_force_variant.load() >= 0) {
    *out = g_force_variant.load();
    return BF_OK;
  }
  if (!g_autotune.load()) return BF_OK;
  // frequency counts share a decision within a power of two (a batch of
  // requests of varying size, 64 .. 1024 frequencies, tunes a few times)
  long long nfb = 1;
  while (nfb < a.nfreq) nfb <<= 1;
  const std::array<long long, 6> key = {h->device, N, a.nbx, a.nby, (long long)fp64, nfb};
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    auto it = g_fused_tuned.find(key);
    if (it != g_fused_tuned.end()) {
      *out = it->second;
      return BF_OK;
    }
  }
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  CK(cudaStreamIsCapturing(st, &cap));
  if (cap != cudaStreamCaptureStatusNone) return BF_OK;
  std::vector<int> cand = bf::fused_variants(N, a.nbx, a.nby, fp64);
  cand.erase(cand.begin());   // the rule's choice is one of the explicit variants
  size_t kbest = (size_t)-1, lbest = 0;
  for (size_t k = 0; k < w.stage_len.size(); ++k)
    if ((N < 64 || !bf::split_stage((int)w.stage_len[k], a.nfreq)) && w.stage_len[k] > lbest) {
      lbest = w.stage_len[k];
      kbest = k;
    }
  int best = bf::kFusedRule;
  std::string what;
  if (cand.size() > 1 && kbest != (size_t)-1) {
    const size_t plane = (size_t)a.nbx * a.nby;
    DBuf st2, ex2;
    CKS(st2.alloc(h, sizeof(C) * (size_t)a.nfreq * a.nslots * plane));
    CKS(ex2.alloc(h, sizeof(double2) * (size_t)std::max(w.nexit, 1) * a.nfreq * plane));
    CK(cudaMemcpyAsync(st2.p, a.state, sizeof(C) * (size_t)a.nfreq * a.nslots * plane, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemsetAsync(ex2.p, 0, sizeof(double2) * (size_t)std::max(w.nexit, 1) * a.nfreq * plane, st));
    bf::FusedArgs<C> t = a;
    t.state = st2.as<C>();
    t.exitacc = ex2.as<double2>();
    t.steps = w.steps.as<StepDesc>() + w.stage_off[kbest];
    t.mg = nullptr;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    float tbest = 1e30f;
    std::vector<std::pair<int, float>> times;
    for (int v : cand) {
      t.variant = v;
      float tv = 1e30f;
      for (int rep = 0; rep < 4; ++rep) {   // the first launch warms up, the best of three counts
        cudaEventRecord(e0, st);
        const int e = fp64 ? bf::launch_fused_stage_d(N, *reinterpret_cast<bf::FusedArgs<double2>*>(&t), (int)lbest, st)
                           : bf::launch_fused_stage_f(N, *reinterpret_cast<bf::FusedArgs<float2>*>(&t), (int)lbest, st);
        cudaEventRecord(e1, st);
        if (e || cudaEventSynchronize(e1) != cudaSuccess) {
          tv = 1e30f;
          break;
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0) tv = std::min(tv, ms);
      }
      what += " v" + std::to_string(v) + "=" + (tv < 1e29f ? std::to_string(tv) : std::string("fail"));
      times.emplace_back(v, tv);
      if (tv < tbest) {
        tbest = tv;
        best = v;
      }
    }
    // within 1 % of the fastest at the timed (largest) stage, the variant
    // that was fastest over whole solves wins: the largest stage does not
    // show everything (at 20 disks, 128^2, complex64 the separate slots at 3
    // CTAs per SM with staged phasor rows are 2 % faster per solve than the
    // joint 320-thread variant although their largest stages time the same)
    for (int pref : {bf::kFusedSeparateStaged, bf::kFusedJointLean, bf::kFusedJointStaged}) {
      bool done = false;
      for (const auto& vt : times)
        if (vt.first == pref && vt.second <= 1.01f * tbest) {
          best = pref;
          done = true;
        }
      if (done) break;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaGetLastError();
  }
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_fused_tuned[key] = best;
  }
  bf_tune_log("fused N=" + std::to_string(N) + " box=" + std::to_string(a.nbx) + "x" + std::to_string(a.nby) +
              (fp64 ? " c128" : " c64") + " nf=" + std::to_string(a.nfreq) + " -> variant " + std::to_string(best) +
              " (ms per launch of " + std::to_string(lbest) + " steps:" + what + ")");
  *out = best;
  return BF_OK;
}

template <typename C>
static int run_fused(bf_handle* h, bf_stack* s, const std::string& key,
                     const std::function<void(Plan&)>& make_plan, bool fp64, int nf,
                     const double* freqs, std::vector<const double2*>& exits_out) {
  cudaStream_t st = h->stream();
  if (!s->ws) s->ws = new Workspace();
  Workspace& w = *s->ws;
  const int N = s->nx;
  const size_t plane = (size_t)s->nbx * s->nby;
  const size_t npix = (size_t)s->nx * s->ny;
  const size_t csz = sizeof(C);
  const int fold = s->kx_sym ? 1 : 0;
  const int QW = fold ? N / 2 : N;
  const std::string full_key = key + "|v" + std::to_string(s->geo_version) + (fp64 ? "|d" : "|f");
  prof_mark(h, 0);
  const unsigned long long l0 = bf::launch_count();
  // ---- plan (host) and its device copies, cached
  const bool new_plan = key.empty() || w.plan_key != full_key;
  if (new_plan) {
    Plan p;
    make_plan(p);
    w.plan_key.clear();
    w.nslots = p.nslots;
    w.ntab = (int)p.tab_region.size();
    w.nexit = p.nexit;
    w.exit_region = p.exit_region;
    w.exit_coef = p.exit_coef;
    CKS(upload(h, w.reg, p.tab_region.data(), sizeof(int) * w.ntab));
    std::vector<int> tidx(w.ntab, -1), tregs;
    for (int t = 0; t < w.ntab; ++t) {
      const int reg = p.tab_region[t];
      if (s->tilt_x[reg] != 0.0 || s->tilt_y[reg] != 0.0 || (s->d_surf && s->surf_nonzero[reg])) {
        tidx[t] = (int)tregs.size();
        tregs.push_back(reg);
      }
    }
    w.ntilt = (int)tregs.size();
    CKS(upload(h, w.tidx, tidx.data(), sizeof(int) * w.ntab));
    if (w.ntilt) CKS(upload(h, w.tregs, tregs.data(), sizeof(int) * w.ntilt));
    std::vector<cd> init((size_t)p.nslots * plane);
    for (int k = 0; k < p.nslots; ++k) std::copy(p.init[k].begin(), p.init[k].end(), init.begin() + k * plane);
    CKS(upload_cd_as(h, w.init, init));
    w.nadd = (int)p.adds.size();
    if (w.nadd) {
      std::vector<cd> adds(p.adds.size() * plane);
      for (size_t k = 0; k < p.adds.size(); ++k) std::copy(p.adds[k].begin(), p.adds[k].end(), adds.begin() + k * plane);
      DBuf b_add64;
      CKS(upload_cd_as(h, b_add64, adds));
      CKS(w.add.alloc(h, csz * adds.size()));
      CKL(bf::launch_convert(b_add64.p, true, w.add.p, fp64, adds.size(), st));
      CK(cudaStreamSynchronize(st));
    }
    std::vector<double2> coefs(4 * p.coefs.size());
    for (size_t k = 0; k < p.coefs.size(); ++k) {
      const Coef4& c = p.coefs[k];
      coefs[4 * k + 0] = make_double2(c.aa.real(), c.aa.imag());
      coefs[4 * k + 1] = make_double2(c.ab.real(), c.ab.imag());
      coefs[4 * k + 2] = make_double2(c.ba.real(), c.ba.imag());
      coefs[4 * k + 3] = make_double2(c.bb.real(), c.bb.imag());
    }
    CKS(upload(h, w.coef, coefs.data(), sizeof(double2) * coefs.size()));
    std::vector<StepDesc> all;
    w.stage_off.clear();
    w.stage_len.clear();
    for (auto& sv : p.stages) {
      w.stage_off.push_back(all.size());
      w.stage_len.push_back(sv.size());
      all.insert(all.end(), sv.begin(), sv.end());
    }
    CKS(upload(h, w.steps, all.data(), sizeof(StepDesc) * all.size()));
    w.has_direct.assign(p.nexit, 0);
    for (int k = 0; k < p.nexit; ++k)
      if (!p.exit_direct[k].empty()) {
        CKS(upload_cd_as(h, w.direct[k], p.exit_direct[k]));
        w.has_direct[k] = 1;
      }
    w.props_per_freq = 0;
    for (auto& d : all) w.props_per_freq += (d.ra >= 0) + (d.rb >= 0);
    CK(cudaStreamSynchronize(st));
    w.plan_key = key.empty() ? std::string() : full_key;
    w.tables_nf = -1;  // tilt-map assignment may have changed
  }
  // ---- tables, cached per frequency batch
  const bool new_tables = new_plan || w.tables_nf != nf || w.tables_fp64 != (int)fp64 ||
                          w.tables_version != s->geo_version ||
                          !std::equal(freqs, freqs + nf, w.tables_freqs.begin(), w.tables_freqs.end());
  if (new_tables) {
    CKS(w.freq.ensure(h, sizeof(double) * nf));
    CK(cudaMemcpyAsync(w.freq.p, freqs, sizeof(double) * nf, cudaMemcpyHostToDevice, st));
    CKS(w.phasor.ensure(h, csz * (size_t)nf * w.ntab * QW * QW));
    CKL(bf::launch_phasor_table(fp64, w.phasor.p, nf, w.freq.as<double>(), w.ntab, w.reg.as<int>(), s->d_geo, N,
                                s->dkX, s->dkY, fold, st));
    if (w.ntilt) {
      CKS(w.tilt.ensure(h, csz * (size_t)nf * w.ntilt * plane));
      CKL(bf::launch_tilt_table(fp64, w.tilt.p, nf, w.freq.as<double>(), w.ntilt, w.tregs.as<int>(), s->d_geo,
                                s->nbx, s->nby, s->bx0, s->by0, s->nx, s->ny, s->dX, s->dY, s->d_surf, st));
    }
    w.tables_nf = nf;
    w.tables_fp64 = fp64;
    w.tables_version = s->geo_version;
    w.tables_freqs.assign(freqs, freqs + nf);
  }
  // ---- state
  CKS(w.state.ensure(h, csz * (size_t)nf * w.nslots * plane));
  CKL(bf::launch_broadcast_state(fp64, w.state.p, w.init.as<double2>(), nf, (size_t)w.nslots * plane, st));
  CKS(w.exitacc.ensure(h, sizeof(double2) * (size_t)w.nexit * nf * plane));
  CK(cudaMemsetAsync(w.exitacc.p, 0, sizeof(double2) * (size_t)w.nexit * nf * plane, st));
  bf::FusedArgs<C> a;
  a.nfreq = nf; a.nbx = s->nbx; a.nby = s->nby; a.nslots = w.nslots; a.ntab = w.ntab; a.fold = fold;
  a.state = w.state.as<C>();
  a.phasor = w.phasor.as<C>();
  a.tilt = w.ntilt ? w.tilt.as<C>() : nullptr;
  a.tilt_idx = w.tidx.as<int>();
  a.ntilt = w.ntilt;
  a.mask = s->d_mask_box;
  a.coefs = w.coef.as<double2>();
  a.exitacc = w.exitacc.as<double2>();
  a.addbuf = w.nadd ? w.add.as<C>() : nullptr;
  a.err = reinterpret_cast<int*>(h->d_scalar + 1);
  CK(cudaMemsetAsync(a.err, 0, sizeof(int), st));
  // row tiles for the stages that take the split-phase path (fewer steps x
  // frequencies than SMs: short stacks, few frequencies, the wavefront's ends)
  {
    size_t split_len = 0;
    const bool split_only = bf::fused_split_only(N, s->nbx, s->nby, fp64);
    for (size_t len : w.stage_len)
      if (split_only || bf::split_stage((int)len, nf)) split_len = std::max(split_len, len);
    a.mg = nullptr;
    if (split_len && N >= 64) {
      CKS(w.mg.ensure(h, bf::split_tile_bytes(N, s->nby, nf, (int)split_len, fp64)));
      a.mg = w.mg.as<C>();
    }
  }
  a.variant = bf::kFusedRule;
  {
    int v = bf::kFusedRule;
    CKS(fused_autotune<C>(h, w, a, N, fp64, st, &v));
    a.variant = v;
  }
  prof_mark(h, 1);
  const unsigned long long l1 = bf::launch_count();
  auto run_stages = [&]() -> int {
    for (size_t k = 0; k < w.stage_off.size(); ++k) {
      a.steps = w.steps.as<StepDesc>() + w.stage_off[k];
      int e;
      if (fp64) e = bf::launch_fused_stage_d(N, *reinterpret_cast<bf::FusedArgs<double2>*>(&a), (int)w.stage_len[k], st);
      else e = bf::launch_fused_stage_f(N, *reinterpret_cast<bf::FusedArgs<float2>*>(&a), (int)w.stage_len[k], st);
      if (e) return fail(h, BF_ERR_CUDA, std::string("fused stage: ") + cudaGetErrorString((cudaError_t)e));
    }
    return BF_OK;
  };
  // The stage launches depend only on the request kind, the batch, the
  // precision, the workspace buffers, the handle and the stage sizes (not on
  // the distances, which reach the kernels through the tables): the second
  // solve with the same ones is captured into a CUDA graph and later solves,
  // optimiser steps included, replay it.
  std::string gkey = key + (fp64 ? "|d" : "|f");
  {
    const void* ptrs[] = {a.state, a.phasor, a.tilt, a.tilt_idx, a.mask, a.coefs, a.exitacc, a.addbuf,
                          a.err, w.steps.p, a.mg};
    const long long ints[] = {nf, a.nbx, a.nby, a.nslots, a.ntab, a.fold, a.ntilt, N, (long long)fp64,
                              (long long)w.stage_off.size(), h->device, a.variant};
    gkey.append(reinterpret_cast<const char*>(ptrs), sizeof(ptrs));
    gkey.append(reinterpret_cast<const char*>(ints), sizeof(ints));
    gkey.append(reinterpret_cast<const char*>(w.stage_off.data()), sizeof(size_t) * w.stage_off.size());
    gkey.append(reinterpret_cast<const char*>(w.stage_len.data()), sizeof(size_t) * w.stage_len.size());
  }
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  CK(cudaStreamIsCapturing(st, &cap));
  if (key.empty() || cap != cudaStreamCaptureStatusNone) {
    // no cached plan, or the caller is capturing this stream: plain launches
    CKS(run_stages());
  } else if (w.graph.exec && w.graph.key == gkey) {
    CK(cudaGraphLaunch(w.graph.exec, st));
    bf::note_launches(w.graph.launches);
    ++w.graph.replays;
  } else if (w.graph.pending == gkey) {
    w.graph.reset();
    w.graph.pending.clear();
    const unsigned long long c0 = bf::launch_count();
    int rc = BF_ERR_CUDA;
    cudaGraph_t g = nullptr;
    cudaError_t ce = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
    if (ce == cudaSuccess) {
      rc = run_stages();   // recorded, not run
      ce = cudaStreamEndCapture(st, &g);
    }
    cudaGraphExec_t ex = nullptr;
    const bool ok = rc == BF_OK && ce == cudaSuccess && g && cudaGraphInstantiate(&ex, g, 0) == cudaSuccess;
    if (g) cudaGraphDestroy(g);
    if (ok) {
      w.graph.exec = ex;
      w.graph.key = gkey;
      w.graph.device = h->device;
      w.graph.launches = bf::launch_count() - c0;
      CK(cudaGraphLaunch(ex, st));
    } else {
      // capture unavailable here: clear its error and launch directly
      cudaGetLastError();
      h->err.clear();
      bf::unnote_launches(bf::launch_count() - c0);   // recorded, never run
      CKS(run_stages());
    }
  } else {
    CKS(run_stages());
    w.graph.pending = gkey;
  }
  const unsigned long long l2 = bf::launch_count();
  prof_mark(h, 2);
  // ---- exits: one FP64 full-grid propagation of the accumulated input per frequency
  CKS(w.tmp.ensure(h, sizeof(double2) * nf * npix));
  exits_out.assign(w.nexit, nullptr);
  for (int k = 0; k < w.nexit; ++k) {
    CKS(w.exit_full[k].ensure(h, sizeof(double2) * nf * npix));
    CKL(bf::launch_embed_box(w.exit_full[k].as<double2>(), w.exitacc.as<double2>() + (size_t)k * nf * plane, nf,
                             s->nx, s->ny, s->nbx, s->nby, s->bx0, s->by0, st));
    CKS(general_prop(h, s, BF_PROP_3D, true, w.exit_full[k].p, w.tmp.p, nf, w.freq.as<double>(), w.exit_region[k]));
    cd c = w.exit_coef[k];
    CKL(bf::launch_exit_combine(w.exit_full[k].as<double2>(), w.exit_full[k].as<double2>(),
                                w.has_direct[k] ? w.direct[k].as<double2>() : nullptr,
                                make_double2(c.real(), c.imag()), nf, (int)npix, st));
    exits_out[k] = w.exit_full[k].as<double2>();
  }
  h->prof[4] = (double)(l2 - l1);
  h->prof[6] = (double)w.props_per_freq * nf;
  h->prof[7] = (double)nf;
  h->prof_launch0 = l0;
  return BF_OK;
}

// ---------------------------------------------------------------------------
// exact full-grid solve (reference dataflow, any grid, amin != 0)
// ---------------------------------------------------------------------------
namespace {
struct MixFullArgs {
  void* A; void* B;            // slot buffers [f][npix] (field precision)
  const double2* add;          // [npix] or null
  double2 caa, cab, cba, cbb;
  double2* exitA; double2 ceA; // exit accumulation of the propagated A (FP64), or null
  double2* exitB; double2 ceB;
  size_t exit_fstride;         // elements between frequencies in the exit buffers
  int exit_store;              // store instead of accumulate (per-bounce output)
  int nf, npix;
};
}

template <typename C>
__global__ void k_mix_full(MixFullArgs m) {
  const size_t total = (size_t)m.nf * m.npix;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const int f = (int)(i / m.npix), p = (int)(i % m.npix);
    double2 a = m.A ? bf::to_d(reinterpret_cast<C*>(m.A)[i]) : make_double2(0, 0);
    double2 b = m.B ? bf::to_d(reinterpret_cast<C*>(m.B)[i]) : make_double2(0, 0);
    if (m.exitA) {
      double2* e = m.exitA + (size_t)f * m.exit_fstride + p;
      double2 v = bf::cmul(m.ceA, a);
      *e = m.exit_store ? v : make_double2(e->x + v.x, e->y + v.y);
    }
    if (m.exitB) {
      double2* e = m.exitB + (size_t)f * m.exit_fstride + p;
      double2 v = bf::cmul(m.ceB, b);
      *e = m.exit_store ? v : make_double2(e->x + v.x, e->y + v.y);
    }
    if (m.A) {
      double2 o = bf::cadd(bf::cmul(m.caa, a), bf::cmul(m.cab, b));
      if (m.add) o = bf::cadd(o, m.add[p]);
      reinterpret_cast<C*>(m.A)[i] = bf::mk((decltype(C().x))o.x, (decltype(C().x))o.y);
    }
    if (m.B) {
      double2 o = bf::cadd(bf::cmul(m.cba, a), bf::cmul(m.cbb, b));
      reinterpret_cast<C*>(m.B)[i] = bf::mk((decltype(C().x))o.x, (decltype(C().x))o.y);
    }
  }
}

static double2 d2(cd c) { return make_double2(c.real(), c.imag()); }

// Exact full-grid bounce loop.  kind 0 = cheerleader, 1 = dancer.  Slots live
// as [slot][f][npix]; exits (FP64) as [exit][f][nout][npix].
static int run_full(bf_handle* h, const bf_stack* s, int solver, int prop_kind, bool fp64, int nf,
                    const double* d_freqs, double amin, int nmax, const std::vector<cd>& em,
                    int per_iter_out, std::vector<DBuf>& exits, int* n_done) {
  cudaStream_t st = h->stream();
  const size_t npix = (size_t)s->nx * s->ny;
  const size_t csz = fp64 ? 16 : 8;
  const int nd = s->nd;
  const int nslots = solver == 0 ? nd : 2 * (nd - 1);
  DBuf b_slots, b_tmp, b_em;
  CKS(b_slots.alloc(h, csz * (size_t)nslots * nf * npix));
  CKS(b_tmp.alloc(h, csz * (size_t)nf * npix));
  auto slot = [&](int k) -> void* { return (char*)b_slots.p + csz * (size_t)k * nf * npix; };
  // initial fields
  for (int k = 0; k < nslots; ++k) {
    const cd* src = nullptr;
    if (solver == 0) src = em.data() + ((size_t)k * 2 + 0) * npix;        // right-moving emission
    else src = em.data() + (size_t)k * npix;                               // [jt][d] == slot 2jt+d
    DBuf b;
    CKS(upload(h, b, src, sizeof(cd) * npix));
    CKL(bf::launch_broadcast_state(fp64, slot(k), b.as<double2>(), nf, npix, st));
    CK(cudaStreamSynchronize(st));
  }
  if (solver == 0) {
    // the exit regions are tracked in the FP64 exit buffers below
    CK(cudaMemsetAsync(slot(0), 0, csz * (size_t)nf * npix, st));
    CK(cudaMemsetAsync(slot(nd - 1), 0, csz * (size_t)nf * npix, st));
  }
  const int nout = per_iter_out ? nmax + 1 : 1;
  auto prop = [&](int k, int region) { return general_prop(h, s, prop_kind, fp64, slot(k), b_tmp.p, nf, d_freqs, region); };
  auto mix = [&](MixFullArgs m) -> int {
    m.nf = nf; m.npix = (int)npix;
    size_t total = (size_t)nf * npix;
    unsigned blocks = (unsigned)std::min<size_t>((total + 255) / 256, 65535 * 8);
    bf::note_launch();
    if (fp64) k_mix_full<double2><<<blocks, 256, 0, st>>>(m);
    else k_mix_full<float2><<<blocks, 256, 0, st>>>(m);
    CK(cudaGetLastError());
    return BF_OK;
  };
  auto maxabs_all = [&](double* out) -> int {
    CKL(bf::launch_maxabs(h->d_scalar, b_slots.p, fp64, (size_t)nslots * nf * npix, st));
    CK(cudaMemcpyAsync(out, h->d_scalar, sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return BF_OK;
  };
  *n_done = 0;
  if (solver == 0) {
    // cheerleader: slots are regions 0..nd-1 (exits 0 and nd-1 kept in the field
    // precision like the reference; results are also accumulated in FP64 exits)
    std::vector<RT> rt(nd - 1);
    for (int i = 0; i < nd - 1; ++i) rt[i] = rt_of(s->r[i]);
    exits.resize(2);
    for (int k = 0; k < 2; ++k) CKS(exits[k].alloc(h, sizeof(double2) * nf * npix));
    // exit buffers start from the initial emission of the exit regions
    {
      std::vector<cd> e0(npix), e1(npix);
      for (size_t i = 0; i < npix; ++i) {
        e0[i] = em[((size_t)(nd - 1) * 2 + 0) * npix + i];
        e1[i] = em[((size_t)0 * 2 + 0) * npix + i];
      }
      DBuf b0, b1;
      CKS(upload_cd_as(h, b0, e0));
      CKS(upload_cd_as(h, b1, e1));
      CKL(bf::launch_broadcast_state(true, exits[0].p, b0.as<double2>(), nf, npix, st));
      CKL(bf::launch_broadcast_state(true, exits[1].p, b1.as<double2>(), nf, npix, st));
      CK(cudaStreamSynchronize(st));
    }
    // push-forward (:281-287)
    for (int i = 1; i <= nd - 2; ++i) {
      CKS(prop(i, i));
      MixFullArgs m{};
      m.A = slot(i);
      m.caa = d2(rt[i].r_r);
      if (i + 1 <= nd - 2) {
        m.B = slot(i + 1); m.cba = d2(rt[i].t_r); m.cbb = d2(cd(1.0, 0.0));
      } else {
        m.exitA = exits[0].as<double2>(); m.ceA = d2(rt[i].t_r); m.exit_fstride = npix;
      }
      CKS(mix(m));
    }
    // left-moving emission (:290-300)
    for (int j = 0; j <= nd - 2; ++j) {
      std::vector<cd> a(npix);
      for (size_t i = 0; i < npix; ++i) {
        a[i] = em[((size_t)j * 2 + 1) * npix + i];
        if (j == nd - 2) a[i] += rt[nd - 2].t_l * em[((size_t)(nd - 1) * 2 + 1) * npix + i];
      }
      DBuf b;
      CKS(upload_cd_as(h, b, a));
      if (j == 0) {
        // add to the FP64 left exit: exit += 1 * a
        CKL(bf::launch_exit_combine(exits[1].as<double2>(), exits[1].as<double2>(), b.as<double2>(),
                                    make_double2(1.0, 0.0), nf, (int)npix, st));
      } else {
        MixFullArgs m{};
        m.A = slot(j); m.caa = d2(cd(1.0, 0.0)); m.add = b.as<double2>();
        CKS(mix(m));
      }
      CK(cudaStreamSynchronize(st));
    }
    {
      std::vector<cd> a(npix);
      for (size_t i = 0; i < npix; ++i) a[i] = rt[nd - 2].r_l * em[((size_t)(nd - 1) * 2 + 1) * npix + i];
      DBuf b;
      CKS(upload_cd_as(h, b, a));
      CKL(bf::launch_exit_combine(exits[0].as<double2>(), exits[0].as<double2>(), b.as<double2>(),
                                  make_double2(1.0, 0.0), nf, (int)npix, st));
      CK(cudaStreamSynchronize(st));
    }
    double a = 1.0;
    int n = 0;
    while (n <= nmax && a >= amin) {
      {  // i = 0
        CKS(prop(1, 1));
        MixFullArgs m{};
        m.B = slot(1); m.cbb = d2(rt[0].r_l);
        m.exitB = exits[1].as<double2>(); m.ceB = d2(rt[0].t_l); m.exit_fstride = npix;
        CKS(mix(m));
      }
      for (int i = 1; i <= nd - 3; ++i) {
        CKS(prop(i, i));
        CKS(prop(i + 1, i + 1));
        MixFullArgs m{};
        m.A = slot(i); m.B = slot(i + 1);
        m.caa = d2(rt[i].r_r); m.cab = d2(rt[i].t_l); m.cba = d2(rt[i].t_r); m.cbb = d2(rt[i].r_l);
        CKS(mix(m));
      }
      {
        const int i = nd - 2;
        CKS(prop(i, i));
        MixFullArgs m{};
        m.A = slot(i); m.caa = d2(rt[i].r_r);
        m.exitA = exits[0].as<double2>(); m.ceA = d2(rt[i].t_r); m.exit_fstride = npix;
        CKS(mix(m));
      }
      if (amin != 0.0) {
        // fields include the exit regions (recurprop.jl:350-352)
        double m1 = 0, m2 = 0, m3 = 0;
        CKS(maxabs_all(&m1));
        CKL(bf::launch_maxabs(h->d_scalar, exits[0].p, true, (size_t)nf * npix, st));
        CK(cudaMemcpyAsync(&m2, h->d_scalar, sizeof(double), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        CKL(bf::launch_maxabs(h->d_scalar, exits[1].p, true, (size_t)nf * npix, st));
        CK(cudaMemcpyAsync(&m3, h->d_scalar, sizeof(double), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        a = std::max(m1, std::max(m2, m3));
      }
      ++n;
    }
    *n_done = n;
  } else {
    // dancer: trimmed region jt = region jt+1, slot 2jt+d
    const int R = nd - 1;
    std::vector<cd> rtd(R + 1);
    for (int i = 0; i < R; ++i) rtd[i] = s->r[i];
    rtd[R] = 0.0;
    exits.resize(1);
    CKS(exits[0].alloc(h, sizeof(double2) * (size_t)nf * nout * npix));
    CK(cudaMemsetAsync(exits[0].p, 0, exits[0].n, st));
    double a = 1.0;
    int n = 0;
    while (n <= nmax && a >= amin) {
      const int rm = n & 1, lm = rm ^ 1;
      for (int i = 0; i <= R; ++i) {
        if (i > 0) CKS(prop(2 * (i - 1) + rm, i));
        if (i < R) CKS(prop(2 * i + lm, i + 1));
        const cd r = rtd[i];
        MixFullArgs m{};
        if (i == 0) {
          m.B = slot(2 * 0 + lm); m.cbb = d2(-r);
        } else if (i == R) {
          m.A = slot(2 * (R - 1) + rm); m.caa = d2(r);
          m.exitA = exits[0].as<double2>() + (per_iter_out ? (size_t)n * npix : 0);
          m.ceA = d2(1.0 + r);
          m.exit_fstride = (size_t)nout * npix;
          m.exit_store = per_iter_out;
        } else {
          m.A = slot(2 * (i - 1) + rm); m.B = slot(2 * i + lm);
          m.caa = d2(r); m.cab = d2(1.0 - r); m.cba = d2(1.0 + r); m.cbb = d2(-r);
        }
        CKS(mix(m));
      }
      if (amin != 0.0) CKS(maxabs_all(&a));
      ++n;
    }
    *n_done = n;
  }
  CK(cudaStreamSynchronize(st));
  return BF_OK;
}

// ---------------------------------------------------------------------------
// 1D propagator solve (every pixel independent)
// ---------------------------------------------------------------------------
static int run_1d(bf_handle* h, const bf_stack* s, int solver, int nf, const std::vector<double>& freqs,
                  double amin, int nmax, const std::vector<cd>& em, int per_iter_out,
                  std::vector<DBuf>& exits) {
  cudaStream_t st = h->stream();
  const size_t npix = (size_t)s->nx * s->ny;
  const int nd = s->nd;
  const int nreg = solver == 0 ? nd : nd - 1;
  // phase exp(-i k0 dz) per (f, region) in FP64 on the host (propagator1D, :218-227)
  std::vector<cd> ph((size_t)nf * nreg);
  for (int f = 0; f < nf; ++f) {
    const double lambda = 299792458.0 / freqs[f];
    for (int j = 0; j < nreg; ++j) {
      const int reg = solver == 0 ? j : j + 1;
      const cd se = std::sqrt(s->eps[reg]);
      const double c = 2.0 * M_PI / lambda;
      const cd k0(c * se.real(), c * se.imag());
      cd arg = cd(k0.imag() * s->distance[reg], -k0.real() * s->distance[reg]);
      ph[(size_t)f * nreg + j] = std::exp(arg);
    }
  }
  std::vector<cd> coef;
  if (solver == 0) {
    coef.resize(4 * (nd - 1));
    for (int i = 0; i < nd - 1; ++i) {
      RT t = rt_of(s->r[i]);
      coef[4 * i + 0] = t.r_r; coef[4 * i + 1] = t.t_l; coef[4 * i + 2] = t.r_l; coef[4 * i + 3] = t.t_r;
    }
  } else {
    coef.assign(4 * (nd), cd(0, 0));
    for (int i = 0; i < nd - 1; ++i) coef[4 * i] = s->r[i];
    coef[4 * (nd - 1)] = 0.0;
  }
  const int nout = per_iter_out ? nmax + 1 : 1;
  DBuf b_ph, b_coef, b_state, b_em;
  CKS(upload_cd_as(h, b_ph, ph));
  CKS(upload_cd_as(h, b_coef, coef));
  CKS(upload_cd_as(h, b_em, em));
  exits.resize(1);
  bf::Rfp1dArgs a{};
  a.kind = solver; a.nfreq = nf; a.npix = (int)npix; a.nd = nreg;
  a.phase = b_ph.as<double2>(); a.coef = b_coef.as<double2>(); a.emit = b_em.as<double2>();
  a.per_iter_out = per_iter_out;
  a.nout = nout;
  a.rm_phase = 0;
  if (solver == 0) {
    CKS(b_state.alloc(h, sizeof(double2) * (size_t)nf * nd * npix));
    CKS(exits[0].alloc(h, sizeof(double2) * (size_t)nf * 2 * npix));
  } else {
    CKS(b_state.alloc(h, sizeof(double2) * (size_t)nf * nreg * 2 * npix));
    // initial fields
    std::vector<cd> init((size_t)nf * nreg * 2 * npix);
    for (int f = 0; f < nf; ++f) std::copy(em.begin(), em.end(), init.begin() + (size_t)f * nreg * 2 * npix);
    CK(cudaMemcpyAsync(b_state.p, init.data(), sizeof(cd) * init.size(), cudaMemcpyHostToDevice, st));
    CK(cudaStreamSynchronize(st));
    CKS(exits[0].alloc(h, sizeof(double2) * (size_t)nf * nout * npix));
    CK(cudaMemsetAsync(exits[0].p, 0, exits[0].n, st));
  }
  a.state = b_state.p;
  a.out = exits[0].as<double2>();
  // output slots per frequency for the dancer (nmax+1 or 1)
  a.n_end = 0;
  if (amin == 0.0) {
    a.do_init = solver == 0;
    a.n_begin = 0; a.n_end = nmax + 1;
    CKL(bf::launch_rfp1d(false, a, st));
  } else {
    double amax = 1.0;
    int n = 0;
    a.do_init = solver == 0;
    a.n_begin = 0; a.n_end = 0;
    CKL(bf::launch_rfp1d(false, a, st));
    a.do_init = 0;
    while (n <= nmax && amax >= amin) {
      a.n_begin = n; a.n_end = n + 1;
      CKL(bf::launch_rfp1d(false, a, st));
      double m1 = 0, m2 = 0;
      CKL(bf::launch_maxabs(h->d_scalar, b_state.p, true, b_state.n / 16, st));
      CK(cudaMemcpyAsync(&m1, h->d_scalar, sizeof(double), cudaMemcpyDeviceToHost, st));
      CK(cudaStreamSynchronize(st));
      if (solver == 0) {
        CKL(bf::launch_maxabs(h->d_scalar, exits[0].p, true, exits[0].n / 16, st));
        CK(cudaMemcpyAsync(&m2, h->d_scalar, sizeof(double), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
      }
      amax = std::max(m1, m2);
      ++n;
    }
  }
  CK(cudaStreamSynchronize(st));
  return BF_OK;
}

// ---------------------------------------------------------------------------
// solver entry points
// ---------------------------------------------------------------------------
static int check_solver_args(bf_handle* h, bf_stack* s, int nf, const double* freqs, int nmax,
                             int prop_kind, int precision, double amin) {
  if (!h) return BF_ERR_INVALID;
  if (!s) return fail(h, BF_ERR_INVALID, "null stack");
  if (nf < 1 || !freqs) return fail(h, BF_ERR_INVALID, "need at least one frequency");
  if (nmax < 0) return fail(h, BF_ERR_INVALID, "nmax < 0");
  if (!all_finite(freqs, nf)) return fail(h, BF_ERR_INVALID, "non-finite frequency");
  for (int i = 0; i < nf; ++i)
    if (!(freqs[i] > 0)) return fail(h, BF_ERR_INVALID, "frequency must be positive");
  if (prop_kind < 0 || prop_kind > 3) return fail(h, BF_ERR_INVALID, "unknown propagator kind");
  if (precision == BF_PREC_TF32 || precision == BF_PREC_MIXED_SIMT)
    return fail(h, BF_ERR_INVALID, "BF_PREC_TF32 / BF_PREC_MIXED_SIMT apply to the transformer only");
  if (precision != BF_PREC_FP64 && precision != BF_PREC_MIXED) return fail(h, BF_ERR_INVALID, "unknown precision");
  if (!std::isfinite(amin)) return fail(h, BF_ERR_INVALID, "non-finite amin");
  return BF_OK;
}

// copy an FP64 [nf][npix] result to the caller (host or device)
static int deliver(bf_handle* h, double* dst, const void* src, size_t bytes, int flags) {
  if (!dst) return BF_OK;
  CK(cudaMemcpyAsync(dst, src, bytes, (flags & BF_OUT_DEVICE) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, h->stream()));
  return BF_OK;
}

static int finish_beta2(bf_handle* h, const DBuf& field, int nf, size_t npix, double scale,
                        double* out_beta2, int flags) {
  if (!out_beta2) return BF_OK;
  DBuf b;
  CKS(b.alloc(h, sizeof(double) * nf));
  CKL(bf::launch_beta2(b.as<double>(), field.as<double2>(), nf, (int)npix, scale, h->stream()));
  CKS(deliver(h, out_beta2, b.p, sizeof(double) * nf, flags));
  CK(cudaStreamSynchronize(h->stream()));
  return BF_OK;
}

// a bounded device-side wait that gave up leaves 1 in the handle's error word
static int check_device_error(bf_handle* h) {
  int err = 0;
  CK(cudaMemcpyAsync(&err, h->d_scalar + 1, sizeof(int), cudaMemcpyDeviceToHost, h->stream()));
  CK(cudaStreamSynchronize(h->stream()));
  if (err) return fail(h, BF_ERR_TIMEOUT, "a bounded wait for a shared-memory copy expired in the bounce kernel");
  return BF_OK;
}

static int finish_beta2_ptr(bf_handle* h, bf_stack* s, const double2* field, int nf, size_t npix,
                            double scale, double* out_beta2, int flags) {
  if (!out_beta2) return BF_OK;
  Workspace* w = s->ws;
  DBuf local;
  DBuf* b = w ? &w->beta : &local;
  CKS(b->ensure(h, sizeof(double) * nf));
  CKL(bf::launch_beta2(b->as<double>(), field, nf, (int)npix, scale, h->stream()));
  return deliver(h, out_beta2, b->p, sizeof(double) * nf, flags);
}

// close the profile of a solve: total device time, stage time, launches
static int finish_profile(bf_handle* h) {
  if (!h->profiling) return BF_OK;
  prof_mark(h, 3);
  CK(cudaEventSynchronize(h->ev[3]));
  float t03 = 0, t12 = 0, t01 = 0, t23 = 0;
  cudaEventElapsedTime(&t03, h->ev[0], h->ev[3]);
  cudaEventElapsedTime(&t12, h->ev[1], h->ev[2]);
  cudaEventElapsedTime(&t01, h->ev[0], h->ev[1]);
  cudaEventElapsedTime(&t23, h->ev[2], h->ev[3]);
  h->prof[0] = t03;
  h->prof[1] = t12;
  h->prof[2] = t01;
  h->prof[3] = t23;
  h->prof[5] = (double)(bf::launch_count() - h->prof_launch0);
  h->prof_valid = 1;
  return BF_OK;
}

extern "C" int bf_set_stream(bf_handle* h, void* stream) {
  if (!h) return BF_ERR_INVALID;
  h->user_stream = reinterpret_cast<cudaStream_t>(stream);
  return BF_OK;
}

extern "C" int bf_set_profiling(bf_handle* h, int enable) {
  if (!h) return BF_ERR_INVALID;
  h->profiling = enable ? 1 : 0;
  h->prof_valid = 0;
  return BF_OK;
}

extern "C" int bf_last_profile(const bf_handle* h, double* out) {
  if (!h || !out) return BF_ERR_INVALID;
  if (!h->prof_valid) return BF_ERR_INVALID;
  for (int i = 0; i < 8; ++i) out[i] = h->prof[i];
  return BF_OK;
}

extern "C" int bf_stack_cheerleader(bf_handle* h, bf_stack* s, int nf, const double* freqs,
                                    double amin, int nmax, int prop_kind, int precision,
                                    const double* emit, const double* reflect, int returnboth,
                                    double beta2_scale, int flags, double* out_right,
                                    double* out_left, double* out_beta2) {
  CKS(check_solver_args(h, s, nf, freqs, nmax, prop_kind, precision, amin));
  CK(cudaSetDevice(h->device));
  cudaStream_t st = h->stream();
  const size_t npix = (size_t)s->nx * s->ny;
  const bool fp64 = precision == BF_PREC_FP64;
  std::vector<double> hfreq(freqs, freqs + nf);
  std::vector<cd> em;
  std::vector<DBuf> exits;
  const double2* right = nullptr;
  const double2* left = nullptr;
  DBuf right_c, left_c;
  if (prop_kind == BF_PROP_1D) {
    cheer_emission(s, emit, reflect, em);
    CKS(run_1d(h, s, 0, nf, hfreq, amin, nmax, em, 0, exits));
    // exits[0] = [f][2][npix] -> split
    CKS(right_c.alloc(h, sizeof(double2) * nf * npix));
    CKS(left_c.alloc(h, sizeof(double2) * nf * npix));
    for (int f = 0; f < nf; ++f) {
      CK(cudaMemcpyAsync(right_c.as<double2>() + (size_t)f * npix, exits[0].as<double2>() + ((size_t)f * 2 + 0) * npix,
                         sizeof(double2) * npix, cudaMemcpyDeviceToDevice, st));
      CK(cudaMemcpyAsync(left_c.as<double2>() + (size_t)f * npix, exits[0].as<double2>() + ((size_t)f * 2 + 1) * npix,
                         sizeof(double2) * npix, cudaMemcpyDeviceToDevice, st));
    }
    right = right_c.as<double2>();
    left = left_c.as<double2>();
    CKS(deliver(h, out_right, right, sizeof(double2) * nf * npix, flags));
    if (returnboth) CKS(deliver(h, out_left, left, sizeof(double2) * nf * npix, flags));
    CKS(finish_beta2(h, right_c, nf, npix, beta2_scale, out_beta2, flags));
    CK(cudaStreamSynchronize(st));
    return BF_OK;
  }
  const bool fusable = (prop_kind == BF_PROP_3D || prop_kind == BF_PROP_NOTILTS) && amin == 0.0 &&
                       s->nx == s->ny && bf::fused_supported(s->nx, s->nbx, s->nby, fp64);
  if (fusable) {
    // NOTILTS: the tilt maps are identity, as if tilts and surfaces were zero
    bf_stack* sp = s;
    bf_stack tmp_stack;
    if (prop_kind == BF_PROP_NOTILTS) {
      tmp_stack = *s;
      std::fill(tmp_stack.tilt_x.begin(), tmp_stack.tilt_x.end(), 0.0);
      std::fill(tmp_stack.tilt_y.begin(), tmp_stack.tilt_y.end(), 0.0);
      tmp_stack.d_surf = nullptr;
      tmp_stack.ws = nullptr;
      tmp_stack.tf_cache = nullptr;
      sp = &tmp_stack;
    }
    const std::string key = (emit || reflect) ? std::string() : "cheer|" + std::to_string(nmax);
    auto mk = [&](Plan& p) {
      cheer_emission(sp, emit, reflect, em);
      plan_cheerleader(sp, nmax, em, p);
    };
    std::vector<const double2*> ex;
    int rc = fp64 ? run_fused<double2>(h, sp, key, mk, true, nf, freqs, ex)
                  : run_fused<float2>(h, sp, key, mk, false, nf, freqs, ex);
    if (rc == BF_OK) {
      rc = deliver(h, out_right, ex[0], sizeof(double2) * nf * npix, flags);
      if (rc == BF_OK && returnboth) rc = deliver(h, out_left, ex[1], sizeof(double2) * nf * npix, flags);
      if (rc == BF_OK) rc = finish_beta2_ptr(h, sp, ex[0], nf, npix, beta2_scale, out_beta2, flags);
    }
    if (rc == BF_OK) rc = finish_profile(h);
    if (rc == BF_OK) rc = check_device_error(h);
    if (sp != s) { delete tmp_stack.ws; tmp_stack.ws = nullptr; }
    if (rc != BF_OK) return rc;
  } else {
    int n_done = 0;
    cheer_emission(s, emit, reflect, em);
    DBuf b_freq;
    CKS(upload(h, b_freq, freqs, sizeof(double) * nf));
    CKS(run_full(h, s, 0, prop_kind, fp64, nf, b_freq.as<double>(), amin, nmax, em, 0, exits, &n_done));
    CKS(deliver(h, out_right, exits[0].p, sizeof(double2) * nf * npix, flags));
    if (returnboth) CKS(deliver(h, out_left, exits[1].p, sizeof(double2) * nf * npix, flags));
    CKS(finish_beta2(h, exits[0], nf, npix, beta2_scale, out_beta2, flags));
  }
  CK(cudaStreamSynchronize(st));
  return BF_OK;
}

extern "C" int bf_stack_dancer(bf_handle* h, bf_stack* s, int nf, const double* freqs, double amin,
                               int nmax, int prop_kind, int precision, const double* emit,
                               const double* reflect, int returnsum, int immediatesum,
                               double beta2_scale, int flags, double* out, double* out_beta2) {
  CKS(check_solver_args(h, s, nf, freqs, nmax, prop_kind, precision, amin));
  CK(cudaSetDevice(h->device));
  cudaStream_t st = h->stream();
  const size_t npix = (size_t)s->nx * s->ny;
  const bool fp64 = precision == BF_PREC_FP64;
  std::vector<double> hfreq(freqs, freqs + nf);
  std::vector<cd> em;
  const int per_iter = immediatesum ? 0 : 1;
  std::vector<DBuf> exits;
  int n_done = nmax + 1;
  if (prop_kind == BF_PROP_1D) {
    dancer_emission(s, emit, reflect, em);
    CKS(run_1d(h, s, 1, nf, hfreq, amin, nmax, em, per_iter, exits));
  } else {
    const bool fusable = (prop_kind == BF_PROP_3D || prop_kind == BF_PROP_NOTILTS) && amin == 0.0 &&
                         !per_iter && s->nx == s->ny &&
                         bf::fused_supported(s->nx, s->nbx, s->nby, fp64);
    if (fusable) {
      bf_stack* sp = s;
      bf_stack tmp_stack;
      if (prop_kind == BF_PROP_NOTILTS) {
        tmp_stack = *s;
        std::fill(tmp_stack.tilt_x.begin(), tmp_stack.tilt_x.end(), 0.0);
        std::fill(tmp_stack.tilt_y.begin(), tmp_stack.tilt_y.end(), 0.0);
        tmp_stack.d_surf = nullptr;
        tmp_stack.ws = nullptr;
        tmp_stack.tf_cache = nullptr;
      tmp_stack.tf_cache = nullptr;
        sp = &tmp_stack;
      }
      const std::string key = (emit || reflect) ? std::string() : "dancer|" + std::to_string(nmax);
      auto mk = [&](Plan& p) {
        dancer_emission(sp, emit, reflect, em);
        plan_dancer(sp, nmax, em, p);
      };
      std::vector<const double2*> ex;
      int rc = fp64 ? run_fused<double2>(h, sp, key, mk, true, nf, freqs, ex)
                    : run_fused<float2>(h, sp, key, mk, false, nf, freqs, ex);
      if (rc == BF_OK) {
        rc = deliver(h, out, ex[0], sizeof(double2) * nf * npix, flags);
        if (rc == BF_OK) rc = finish_beta2_ptr(h, sp, ex[0], nf, npix, beta2_scale, out_beta2, flags);
        if (rc == BF_OK) rc = finish_profile(h);
        if (rc == BF_OK) rc = check_device_error(h);
      }
      if (sp != s) { delete tmp_stack.ws; tmp_stack.ws = nullptr; }
      if (rc != BF_OK) return rc;
      CK(cudaStreamSynchronize(st));
      return BF_OK;
    } else {
      dancer_emission(s, emit, reflect, em);
      DBuf b_freq;
      CKS(upload(h, b_freq, freqs, sizeof(double) * nf));
      CKS(run_full(h, s, 1, prop_kind, fp64, nf, b_freq.as<double>(), amin, nmax, em, per_iter, exits, &n_done));
    }
  }
  const int nout = per_iter ? nmax + 1 : 1;
  if (per_iter && returnsum) {
    // sum(reverse(Eout, dims=3), dims=3): sum the per-bounce slots from the last
    std::vector<cd> all((size_t)nf * nout * npix), sum((size_t)nf * npix, cd(0, 0));
    CK(cudaMemcpyAsync(all.data(), exits[0].p, sizeof(cd) * all.size(), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    for (int f = 0; f < nf; ++f)
      for (int k = nout - 1; k >= 0; --k)
        for (size_t i = 0; i < npix; ++i) sum[(size_t)f * npix + i] += all[((size_t)f * nout + k) * npix + i];
    DBuf b;
    CKS(upload_cd_as(h, b, sum));
    CKS(deliver(h, out, b.p, sizeof(cd) * sum.size(), flags));
    CKS(finish_beta2(h, b, nf, npix, beta2_scale, out_beta2, flags));
  } else if (per_iter) {
    CKS(deliver(h, out, exits[0].p, sizeof(double2) * nf * nout * npix, flags));
    if (out_beta2) {
      // beta^2 of the summed field
      std::vector<cd> all((size_t)nf * nout * npix);
      CK(cudaMemcpyAsync(all.data(), exits[0].p, sizeof(cd) * all.size(), cudaMemcpyDeviceToHost, st));
      CK(cudaStreamSynchronize(st));
      std::vector<cd> sum((size_t)nf * npix, cd(0, 0));
      for (int f = 0; f < nf; ++f)
        for (int k = nout - 1; k >= 0; --k)
          for (size_t i = 0; i < npix; ++i) sum[(size_t)f * npix + i] += all[((size_t)f * nout + k) * npix + i];
      DBuf b;
      CKS(upload_cd_as(h, b, sum));
      CKS(finish_beta2(h, b, nf, npix, beta2_scale, out_beta2, flags));
    }
  } else {
    CKS(deliver(h, out, exits[0].p, sizeof(double2) * nf * npix, flags));
    CKS(finish_beta2(h, exits[0], nf, npix, beta2_scale, out_beta2, flags));
  }
  (void)n_done;
  CK(cudaStreamSynchronize(st));
  return BF_OK;
}

extern "C" int bf_cheerleader(bf_handle* h, int nd, const double* distance, const double* r,
                              const double* eps, const double* tilt_x, const double* tilt_y,
                              const double* surfaces, int nx, int ny, const double* X,
                              const double* Y, const double* kX, const double* kY, double diskR,
                              int nf, const double* freqs, double amin, int nmax, int prop_kind,
                              int precision, const double* emit, const double* reflect,
                              int returnboth, double beta2_scale, double* out_right,
                              double* out_left, double* out_beta2) {
  bf_stack* s = nullptr;
  int rc = bf_stack_create(h, nd, distance, r, eps, tilt_x, tilt_y, surfaces, nx, ny, X, Y, kX, kY, diskR, &s);
  if (rc != BF_OK) return rc;
  rc = bf_stack_cheerleader(h, s, nf, freqs, amin, nmax, prop_kind, precision, emit, reflect,
                            returnboth, beta2_scale, 0, out_right, out_left, out_beta2);
  bf_stack_destroy(h, s);
  return rc;
}

extern "C" int bf_dancer(bf_handle* h, int nd, const double* distance, const double* r,
                         const double* eps, const double* tilt_x, const double* tilt_y,
                         const double* surfaces, int nx, int ny, const double* X, const double* Y,
                         const double* kX, const double* kY, double diskR, int nf,
                         const double* freqs, double amin, int nmax, int prop_kind, int precision,
                         const double* emit, const double* reflect, int returnsum, int immediatesum,
                         double beta2_scale, double* out, double* out_beta2) {
  bf_stack* s = nullptr;
  int rc = bf_stack_create(h, nd, distance, r, eps, tilt_x, tilt_y, surfaces, nx, ny, X, Y, kX, kY, diskR, &s);
  if (rc != BF_OK) return rc;
  rc = bf_stack_dancer(h, s, nf, freqs, amin, nmax, prop_kind, precision, emit, reflect, returnsum,
                       immediatesum, beta2_scale, 0, out, out_beta2);
  bf_stack_destroy(h, s);
  return rc;
}
