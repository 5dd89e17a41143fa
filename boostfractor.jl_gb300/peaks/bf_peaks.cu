// Arithmetic-throughput probes of one GPU (FP32 FFMA, packed FP32x2 FFMA,
// FP64 DFMA), the denominators of the SIMT rooflines that the benchmark
// reports.  Not part of the solver library: bench.py loads this separately.
//
// Every thread runs 8 independent multiply-add chains for `iters` rounds, so
// the pipes, not the dependency latency, bound the rate; the chains' final
// values are summed and stored so that nothing is optimised away.
#include <cuda_runtime.h>

namespace {

constexpr int kChains = 8;

__global__ void k_ffma(float* out, int iters, float b, float c) {
  float a[kChains];
#pragma unroll
  for (int k = 0; k < kChains; ++k) a[k] = threadIdx.x * 1e-3f + k;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < kChains; ++k) a[k] = fmaf(a[k], b, c);
  }
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < kChains; ++k) s += a[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__device__ __forceinline__ void fma_x2(float& x, float& y, float b, float c) {
  asm("{\n\t.reg .b64 pa, pb, pc;\n\tmov.b64 pa, {%0, %1};\n\tmov.b64 pb, {%2, %2};\n\tmov.b64 pc, {%3, %3};\n\t"
      "fma.rn.f32x2 pa, pa, pb, pc;\n\tmov.b64 {%0, %1}, pa;\n\t}"
      : "+f"(x), "+f"(y)
      : "f"(b), "f"(c));
}

__global__ void k_ffma2(float* out, int iters, float b, float c) {
  float a[2 * kChains];
#pragma unroll
  for (int k = 0; k < 2 * kChains; ++k) a[k] = threadIdx.x * 1e-3f + k;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < kChains; ++k) fma_x2(a[2 * k], a[2 * k + 1], b, c);
  }
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < 2 * kChains; ++k) s += a[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void k_dfma(double* out, int iters, double b, double c) {
  double a[kChains];
#pragma unroll
  for (int k = 0; k < kChains; ++k) a[k] = threadIdx.x * 1e-3 + k;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < kChains; ++k) a[k] = fma(a[k], b, c);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < kChains; ++k) s += a[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

// kind 0: FP32 FFMA, 1: packed FP32x2 FFMA, 2: FP64 DFMA.  Runs `reps` launches
// of blocks_per_sm x SMs CTAs of 256 threads and returns the FLOP/s of the
// fastest (2 flops per multiply-add lane) in *out_tflops.  0 = OK.
extern "C" int bf_peak_probe(int kind, int iters, int reps, int blocks_per_sm, double* out_tflops) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 1;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 1;
  const int threads = 256, blocks = sms * blocks_per_sm;
  void* buf = nullptr;
  if (cudaMalloc(&buf, sizeof(double) * blocks * threads) != cudaSuccess) return 1;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  double best = 0.0;
  for (int r = 0; r < reps + 1; ++r) {   // the first launch warms up
    cudaEventRecord(e0);
    if (kind == 0) k_ffma<<<blocks, threads>>>((float*)buf, iters, 0.999999f, 1e-6f);
    else if (kind == 1) k_ffma2<<<blocks, threads>>>((float*)buf, iters, 0.999999f, 1e-6f);
    else k_dfma<<<blocks, threads>>>((double*)buf, iters, 0.999999999, 1e-9);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    const double lanes = (kind == 1 ? 2.0 : 1.0) * kChains;
    const double flops = 2.0 * lanes * iters * (double)blocks * threads;
    if (r > 0 && ms > 0.f) best = flops / (ms * 1e-3) / 1e12 > best ? flops / (ms * 1e-3) / 1e12 : best;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  const cudaError_t err = cudaGetLastError();
  cudaFree(buf);
  *out_tflops = best;
  return err == cudaSuccess ? 0 : 1;
}
