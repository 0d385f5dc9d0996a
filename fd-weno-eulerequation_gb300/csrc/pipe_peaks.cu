// Measures the arithmetic-pipe peaks that bound the stage kernels: FP64 FMA,
// FP32 FMA, FP64 division and FP64 square root throughput on the current
// GPU.  Prints one JSON object.  Used for the compute rooflines of the FP64
// (parity) and FP32 stage kernels.
//
//   _build/pipe_peaks [device]
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>

namespace {

constexpr int kChains = 8;
constexpr int kIters = 4096;

template <typename T>
__global__ void k_fma(T *out, T a, T b) {
  T x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) x[c] = T(threadIdx.x + c) * T(1e-3);
  for (int i = 0; i < kIters; ++i) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = fma(x[c], a, b);
  }
  T s = 0;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += x[c];
  if (s == T(-1.2345)) out[threadIdx.x] = s;  // never true; keeps the chains live
}

__global__ void k_ddiv(double *out, double b) {
  double x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) x[c] = 1.0 + (threadIdx.x + c) * 1e-3;
  for (int i = 0; i < kIters / 8; ++i) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = b / x[c];
  }
  double s = 0;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += x[c];
  if (s == -1.2345) out[threadIdx.x] = s;
}

__global__ void k_dsqrt(double *out) {
  double x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) x[c] = 2.0 + (threadIdx.x + c) * 1e-3;
  for (int i = 0; i < kIters / 8; ++i) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = sqrt(x[c]) + 1.0;
  }
  double s = 0;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += x[c];
  if (s == -1.2345) out[threadIdx.x] = s;
}

template <typename F>
float time_ms(F launch) {
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  launch();  // warm-up
  cudaEventRecord(e0);
  for (int r = 0; r < 3; ++r) launch();
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return ms / 3;
}

}  // namespace

int main(int argc, char **argv) {
  const int dev = argc > 1 ? std::atoi(argv[1]) : 0;
  if (cudaSetDevice(dev) != cudaSuccess) return 1;
  cudaDeviceProp p;
  cudaGetDeviceProperties(&p, dev);
  const int blocks = p.multiProcessorCount * 8, threads = 256;
  double *out = nullptr;
  cudaMalloc(&out, threads * sizeof(double));
  const double thr = double(blocks) * threads * kChains;
  const float ms64 = time_ms([&] { k_fma<double><<<blocks, threads>>>(out, 0.999999, 1e-7); });
  const float ms32 = time_ms([&] { k_fma<float><<<blocks, threads>>>((float *)out, 0.999999f, 1e-7f); });
  const float msdiv = time_ms([&] { k_ddiv<<<blocks, threads>>>(out, 1.000001); });
  const float mssq = time_ms([&] { k_dsqrt<<<blocks, threads>>>(out); });
  const cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    std::fprintf(stderr, "pipe_peaks: %s\n", cudaGetErrorString(e));
    return 1;
  }
  int clk_khz = 0;
  cudaDeviceGetAttribute(&clk_khz, cudaDevAttrClockRate, dev);
  std::printf(
      "{\"device\": \"%s\", \"sms\": %d, \"fp64_fma_tflops\": %.4f, \"fp32_fma_tflops\": %.3f, "
      "\"fp64_div_per_s\": %.4e, \"fp64_sqrt_per_s\": %.4e, \"clock_khz_attr\": %d}\n",
      p.name, p.multiProcessorCount, 2.0 * thr * kIters / (ms64 * 1e-3) / 1e12,
      2.0 * thr * kIters / (ms32 * 1e-3) / 1e12, thr * (kIters / 8) / (msdiv * 1e-3),
      thr * (kIters / 8) / (mssq * 1e-3), clk_khz);
  cudaFree(out);
  return 0;
}
