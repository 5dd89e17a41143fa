// Split-TF32 GEMM on the 5th-generation tensor cores (tcgen05, sm_103a).
//
//   out[z][n][m] = sum_{k in slice z} (Ahi Bhi + Ahi Blo + Alo Bhi)[m][k][n]
//
// A is [M][Kp] and B is [N][Kp] (both K-major, FP32 containers holding values
// already rounded to TF32: hi = tf32(x), lo = tf32(x - hi)), M a multiple of
// 128 and Kp of 32.  The three products recover ~22 bits of each operand.
//
// Accuracy.  The tensor cores' FP32 accumulation truncates: about half an
// FP32 ulp of the running sum is lost per accumulating MMA, so a sum held in
// tensor memory for thousands of terms drifts (a depth of 2048 lost 2.4e-5
// relative on an all-positive sum).  Here the accumulator is restarted every
// K block of 32 (12 MMAs) and each block's sum is drained into FP32 registers
// of the epilogue warps, which add it with round-to-nearest.  The truncation
// then acts on 32-term partial sums only, and the running sum is an ordinary
// rounded FP32 sum.  Tensor memory holds two accumulators of 128 columns, so
// the MMAs of block g+1 run while block g is drained.
//
// One persistent CTA per SM walks the work units (128 x 128 output tile x K
// slice; M tiles fastest, so the CTAs in flight share B tiles in L2) with 6
// warps:
//   warp 0     one thread issues the TMA loads (128B-swizzled tiles of A_hi,
//              A_lo, B_hi, B_lo, 32 K-elements each) into a 3-stage ring;
//   warp 1     allocates 256 TMEM columns; one thread issues the MMAs
//              (kind::tf32, M = 128, N = 128, K = 8; 3 per K step, 12 per
//              block), committing each stage back to the producer and each
//              block's accumulator to the epilogue;
//   warps 2-5  drain the accumulator (tcgen05.ld 32x32b, each warp its 32
//              TMEM lanes = output rows) into 128 FP32 registers per thread,
//              release it, and store the finished tile column by column
//              (32 consecutive m per store: coalesced).
// Every mbarrier wait is bounded: after ~2 s of clock the waiting role records
// an error in *err and raises a CTA-wide abort flag, so the other roles stop
// at their next wait; the CTA still waits (bounded) for its copies and MMAs in
// flight and frees its tensor memory.
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <atomic>
#include <mutex>

#include "bf_device.cuh"

namespace bf {

namespace {

constexpr int kTM = 128, kTN = 128, kTK = 32, kStages = 3;
constexpr int kTileBytes = kTM * kTK * 4;              // 16 KB: one operand tile (also B, kTN = kTM)
constexpr int kStageBytes = 4 * kTileBytes;            // A_hi, A_lo, B_hi, B_lo
constexpr int kThreads = 192;
constexpr int kEpiWarps = 4;
constexpr uint32_t kTmemCols = 2 * kTN;                // two accumulators
constexpr long long kWaitCycles = 4000000000LL;        // ~2 s at 2 GHz

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
// Bounded wait for the phase with the given parity.  Gives up (false) when the
// CTA's abort flag is up, or after kWaitCycles, then records `code` in *err and
// raises the flag.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int* abort_flag, int* err,
                                          int code) {
  const long long t0 = clock64();
  for (;;) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok) return true;
    if (*abort_flag) return false;
    if (clock64() - t0 > kWaitCycles) {
      atomicExch(err, code);
      *abort_flag = 1;
      return false;
    }
  }
}
// The same wait without the abort flag (final drains of copies and MMAs in flight).
__device__ __forceinline__ bool mbar_wait_final(uint32_t bar, uint32_t parity, int* err, int code) {
  const long long t0 = clock64();
  for (;;) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok) return true;
    if (clock64() - t0 > kWaitCycles) {
      atomicExch(err, code);
      return false;
    }
  }
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
      : "memory");
}

// Shared-memory matrix descriptor: K-major operand, 128-byte swizzle, 8-row
// groups 1024 B apart (SBO), start address in 16-byte units.
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
  d |= (uint64_t)1 << 16;              // leading-dimension offset (unused with a 128B K extent)
  d |= (uint64_t)(1024 >> 4) << 32;    // stride-dimension offset
  d |= (uint64_t)1 << 46;              // descriptor version
  d |= (uint64_t)2 << 61;              // 128-byte swizzle
  return d;
}

// Instruction descriptor, kind::tf32: FP32 accumulator, TF32 A and B, both
// K-major, N = 128, M = 128.
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(kTN >> 3) << 17) |
                            ((uint32_t)(kTM >> 4) << 24);

__device__ __forceinline__ void umma_tf32(uint32_t tmem, uint64_t a, uint64_t b, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
      "l"(a), "l"(b), "r"(kIdesc), "r"(accumulate));
}
__device__ __forceinline__ void umma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// Work unit u -> (m tile, n tile, slice) and its K-tile range.
struct Unit {
  int m0, n0, z, kb, nkt;
};
__device__ __forceinline__ Unit unit_of(int u, int mt, int nt, int ktiles, int per) {
  Unit w;
  const int r = u % (mt * nt);
  w.z = u / (mt * nt);
  w.m0 = (r % mt) * kTM;
  w.n0 = (r / mt) * kTN;
  w.kb = w.z * per;
  w.nkt = max(0, min(ktiles, w.kb + per) - w.kb);
  return w;
}

__global__ void __launch_bounds__(kThreads, 1)
    k_tc_gemm_tf32x3(const __grid_constant__ CUtensorMap mAhi, const __grid_constant__ CUtensorMap mAlo,
                     const __grid_constant__ CUtensorMap mBhi, const __grid_constant__ CUtensorMap mBlo,
                     float* __restrict__ out, int M, int N, int ktiles, int per, int mt, int nt, int units,
                     int withhold, int* err) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  // 1024-byte alignment of the tile ring (128B swizzle atoms)
  unsigned char* smem = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + kStages * kStageBytes);
  // bars: full[kStages], empty[kStages], accF[2], accE[2], done
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * kStages + 5);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
  const uint32_t full0 = smem_u32(bars), empty0 = smem_u32(bars + kStages);
  const uint32_t accF0 = smem_u32(bars + 2 * kStages), accE0 = smem_u32(bars + 2 * kStages + 2);
  const uint32_t done = smem_u32(bars + 2 * kStages + 4);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(full0 + 8 * s, 1);
      mbar_init(empty0 + 8 * s, 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(accF0 + 8 * b, 1);
      mbar_init(accE0 + 8 * b, kEpiWarps);
    }
    mbar_init(done, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      // producer: TMA loads into the stage ring (none when a test withholds
      // them, so that the MMA warp's bounded wait runs out)
      uint32_t g = 0;
      bool ok = !withhold;
      for (int u = blockIdx.x; u < units && ok; u += gridDim.x) {
        const Unit w = unit_of(u, mt, nt, ktiles, per);
        for (int kt = 0; kt < w.nkt; ++kt, ++g) {
          const int s = (int)(g % kStages);
          if (g >= (uint32_t)kStages && !mbar_wait(empty0 + 8 * s, ((g / kStages) + 1) & 1, abort_flag, err, 1)) {
            ok = false;
            break;
          }
          const uint32_t st = smem_u32(smem + s * kStageBytes);
          const uint32_t fb = full0 + 8 * s;
          mbar_expect_tx(fb, kStageBytes);
          const int k = (w.kb + kt) * kTK;
          tma_load_2d(st, &mAhi, k, w.m0, fb);
          tma_load_2d(st + kTileBytes, &mAlo, k, w.m0, fb);
          tma_load_2d(st + 2 * kTileBytes, &mBhi, k, w.n0, fb);
          tma_load_2d(st + 3 * kTileBytes, &mBlo, k, w.n0, fb);
        }
      }
      // the copies of the last stages must have landed before the CTA exits
      const uint32_t first = g > (uint32_t)kStages ? g - kStages : 0;
      for (uint32_t q = first; q < g; ++q)
        if (!mbar_wait_final(full0 + 8 * (q % kStages), (q / kStages) & 1, err, 4)) break;
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // MMA issuer
      uint32_t g = 0;
      bool ok = true;
      for (int u = blockIdx.x; u < units && ok; u += gridDim.x) {
        const Unit w = unit_of(u, mt, nt, ktiles, per);
        for (int kt = 0; kt < w.nkt; ++kt, ++g) {
          const int s = (int)(g % kStages);
          const uint32_t b = g & 1;
          // the epilogue has drained this accumulator (block g - 2)
          if (g >= 2 && !mbar_wait(accE0 + 8 * b, ((g >> 1) + 1) & 1, abort_flag, err, 5)) {
            ok = false;
            break;
          }
          if (!mbar_wait(full0 + 8 * s, (g / kStages) & 1, abort_flag, err, 2)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t st = smem_u32(smem + s * kStageBytes);
          const uint64_t ahi = umma_desc(st), alo = umma_desc(st + kTileBytes);
          const uint64_t bhi = umma_desc(st + 2 * kTileBytes), blo = umma_desc(st + 3 * kTileBytes);
          const uint32_t acc = tmem + b * kTN;
#pragma unroll
          for (int kk = 0; kk < kTK / 8; ++kk) {
            const uint64_t adv = (uint64_t)(kk * 32 >> 4);   // 8 TF32 = 32 bytes along K
            umma_tf32(acc, ahi + adv, bhi + adv, kk > 0 ? 1u : 0u);
            umma_tf32(acc, ahi + adv, blo + adv, 1u);
            umma_tf32(acc, alo + adv, bhi + adv, 1u);
          }
          umma_commit(empty0 + 8 * s);
          umma_commit(accF0 + 8 * b);
        }
      }
      // no MMA may be in flight when the tensor memory is freed
      umma_commit(done);
      mbar_wait_final(done, 0, err, 6);
    }
  } else {
    // epilogue: drain every block's accumulator into registers; store each tile
    const int q = warp & 3;   // this warp's TMEM lane quarter
    const uint32_t lane_base = tmem + ((uint32_t)(q * 32) << 16);
    uint32_t g = 0;
    bool ok = true;
    for (int u = blockIdx.x; u < units && ok; u += gridDim.x) {
      const Unit w = unit_of(u, mt, nt, ktiles, per);
      float acc[kTN];
#pragma unroll
      for (int j = 0; j < kTN; ++j) acc[j] = 0.0f;
      for (int kt = 0; kt < w.nkt; ++kt, ++g) {
        const uint32_t b = g & 1;
        // every lane polls; the warp goes on only if all of them saw the phase
        // (the tcgen05.ld below is warp-collective)
        if (!__all_sync(0xffffffffu, mbar_wait(accF0 + 8 * b, (g >> 1) & 1, abort_flag, err, 3))) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
        for (int c0 = 0; c0 < kTN; c0 += 32) {
          uint32_t v[32];
          const uint32_t taddr = lane_base + b * kTN + (uint32_t)c0;
          asm volatile(
              "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
              "%14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
              : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]),
                "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]),
                "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
              : "r"(taddr));
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
          for (int j = 0; j < 32; ++j) acc[c0 + j] = __fadd_rn(acc[c0 + j], __uint_as_float(v[j]));
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncwarp();
        if (lane == 0) mbar_arrive(accE0 + 8 * b);
      }
      if (!ok) break;
      const int row = w.m0 + q * 32 + lane;
      float* dst = out + (size_t)w.z * N * M + row;
#pragma unroll
      for (int j = 0; j < kTN; ++j)
        if (w.n0 + j < N) dst[(size_t)(w.n0 + j) * M] = acc[j];
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
  }
}

using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                 const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encoder() {
  static std::once_flag once;
  static EncodeTiled fn = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiled>(p);
    else
      cudaGetLastError();
  });
  return fn;
}

// 2D map of a row-major [rows][kp] FP32 array, boxes of 32 x 128, 128B swizzle;
// rows past the end read as zeros.
bool make_map(CUtensorMap* m, const float* base, int rows, int kp) {
  EncodeTiled enc = encoder();
  if (!enc) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)kp, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)kp * sizeof(float)};
  const cuuint32_t box[2] = {(cuuint32_t)kTK, (cuuint32_t)kTM};
  const cuuint32_t estr[2] = {1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(base), dims, strides, box, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

int sm_count() {
  static std::once_flag once;
  static int n = 0;
  std::call_once(once, [] {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) !=
                                                   cudaSuccess)
      n = 0;
    cudaGetLastError();
  });
  return n > 0 ? n : 148;
}

std::atomic<int> g_withhold{0};

}  // namespace

size_t tc_gemm_smem_bytes() { return (size_t)kStages * kStageBytes + 1024 + 256; }

bool tc_gemm_available() { return encoder() != nullptr; }

bool tc_gemm_fills_gpu(int M, int N) {
  return (long)(M / kTM) * ((N + kTN - 1) / kTN) >= 4L * sm_count();
}

int tc_gemm_splits(int M, int N, int Kp) {
  const long tiles = (long)(M / kTM) * ((N + kTN - 1) / kTN);
  const int ktiles = Kp / kTK;
  const long want = 4L * sm_count();   // about four units per SM keeps the last wave short
  int splits = 1;
  while (tiles * splits < want && ktiles / (2 * splits) >= 8) splits *= 2;
  return splits;
}

int tc_gemm_tf32x3(const float* Ahi, const float* Alo, const float* Bhi, const float* Blo, int M, int N, int Kp,
                   int splits, float* out, int* d_err, cudaStream_t st, int max_ctas) {
  if (Kp % kTK || M % kTM || M < kTM || N < 1 || splits < 1) return (int)cudaErrorInvalidValue;
  // TMA: 16-byte aligned bases (pool allocations) and row strides
  for (const float* p : {Ahi, Alo, Bhi, Blo})
    if (reinterpret_cast<uintptr_t>(p) & 15) return (int)cudaErrorInvalidValue;
  CUtensorMap mAhi, mAlo, mBhi, mBlo;
  if (!make_map(&mAhi, Ahi, M, Kp) || !make_map(&mAlo, Alo, M, Kp) || !make_map(&mBhi, Bhi, N, Kp) ||
      !make_map(&mBlo, Blo, N, Kp))
    return (int)cudaErrorInvalidValue;
  const int ktiles = Kp / kTK;
  const int per = (ktiles + splits - 1) / splits;
  const int mt = M / kTM, nt = (N + kTN - 1) / kTN;
  const long units_l = (long)mt * nt * splits;
  if (units_l > 0x7fffffffL) return (int)cudaErrorInvalidValue;
  const int units = (int)units_l;
  const size_t smem = tc_gemm_smem_bytes();
  cudaError_t e = cudaFuncSetAttribute(k_tc_gemm_tf32x3, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return (int)e;
  // persistent CTAs: one per SM, or fewer when the caller leaves SMs to
  // other streams (a serving engine's latency lane)
  const int grid = std::min(units, max_ctas > 0 ? std::min(max_ctas, sm_count()) : sm_count());
  note_launch();
  k_tc_gemm_tf32x3<<<grid, kThreads, smem, st>>>(mAhi, mAlo, mBhi, mBlo, out, M, N, ktiles, per, mt, nt, units,
                                                 g_withhold.load() ? 1 : 0, d_err);
  return (int)cudaGetLastError();
}

}  // namespace bf

// Test hook: while `on` is non-zero, the tensor-core GEMM's producer issues no
// copies, so its MMA warp's bounded wait runs out (~2 s) and the solve returns
// BF_ERR_TIMEOUT with the context intact.  Nothing waits forever and no memory
// is touched that a normal launch would not touch.
extern "C" int bf_test_tc_withhold_loads(int on) {
  bf::g_withhold.store(on ? 1 : 0);
  return 0;
}
