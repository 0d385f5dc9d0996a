// Measures the arithmetic-pipe peaks that bound the stage kernels: FP64 FMA,
// FP32 FMA, FP64 division and FP64 square root throughput on the current
// GPU; and with --link, the host-link rates that bound the end-to-end path
// (the state crossing each way): copy-engine transfers of a 4096^2 state
// (537 MB) between pinned host memory and the device in each direction and
// both at once, and the same transfers made by the SMs through mapped pinned
// memory.  Prints one JSON object.  Used for the compute rooflines of the
// FP64 (parity) and FP32 stage kernels and the bound of the e2e figure.
//
//   _build/pipe_peaks [device] [--link]
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

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

// SM-driven copy of n16 16-byte units (every index < n16 in both buffers).
__global__ void k_copy16(const double2 *__restrict__ src, double2 *__restrict__ dst, long long n16) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n16; i += stride) dst[i] = src[i];
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

// Host-link rates in GB/s; false on any CUDA error.
bool link_rates(int sms, double out[5]) {
  const size_t bytes = size_t(4) * 4096 * 4096 * sizeof(double);
  double *h_src = nullptr, *h_dst = nullptr, *d_a = nullptr, *d_b = nullptr;
  bool ok = cudaHostAlloc(&h_src, bytes, cudaHostAllocMapped) == cudaSuccess &&
            cudaHostAlloc(&h_dst, bytes, cudaHostAllocMapped) == cudaSuccess &&
            cudaMalloc(&d_a, bytes) == cudaSuccess && cudaMalloc(&d_b, bytes) == cudaSuccess;
  double *m_src = nullptr, *m_dst = nullptr;
  cudaStream_t s2 = nullptr;
  if (ok) ok = cudaHostGetDevicePointer((void **)&m_src, h_src, 0) == cudaSuccess &&
               cudaHostGetDevicePointer((void **)&m_dst, h_dst, 0) == cudaSuccess &&
               cudaStreamCreateWithFlags(&s2, cudaStreamNonBlocking) == cudaSuccess;
  if (ok) {
    for (size_t k = 0; k < bytes / sizeof(double); k += 512) h_src[k] = double(k);
    const double gb = double(bytes) / 1e9;
    const long long n16 = (long long)(bytes / 16);
    out[0] = gb / (1e-3 * time_ms([&] { cudaMemcpyAsync(d_a, h_src, bytes, cudaMemcpyHostToDevice, 0); }));
    out[1] = gb / (1e-3 * time_ms([&] { cudaMemcpyAsync(h_dst, d_b, bytes, cudaMemcpyDeviceToHost, 0); }));
    out[2] = 2.0 * gb / (1e-3 * time_ms([&] {
      cudaEvent_t done;
      cudaEventCreateWithFlags(&done, cudaEventDisableTiming);
      cudaMemcpyAsync(d_a, h_src, bytes, cudaMemcpyHostToDevice, 0);
      cudaMemcpyAsync(h_dst, d_b, bytes, cudaMemcpyDeviceToHost, s2);
      cudaEventRecord(done, s2);
      cudaStreamWaitEvent(0, done, 0);
      cudaEventDestroy(done);
    }));
    out[3] = gb / (1e-3 * time_ms([&] { k_copy16<<<sms * 8, 256>>>((const double2 *)m_src, (double2 *)d_a, n16); }));
    out[4] = gb / (1e-3 * time_ms([&] { k_copy16<<<sms * 8, 256>>>((const double2 *)d_a, (double2 *)m_dst, n16); }));
    ok = cudaDeviceSynchronize() == cudaSuccess;
  }
  if (s2) cudaStreamDestroy(s2);
  cudaFree(d_a);
  cudaFree(d_b);
  cudaFreeHost(h_src);
  cudaFreeHost(h_dst);
  return ok;
}

}  // namespace

int main(int argc, char **argv) {
  int dev = 0;
  bool link = false;
  for (int k = 1; k < argc; ++k) {
    if (std::strcmp(argv[k], "--link") == 0) link = true;
    else dev = std::atoi(argv[k]);
  }
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
      "\"fp64_div_per_s\": %.4e, \"fp64_sqrt_per_s\": %.4e, \"clock_khz_attr\": %d",
      p.name, p.multiProcessorCount, 2.0 * thr * kIters / (ms64 * 1e-3) / 1e12,
      2.0 * thr * kIters / (ms32 * 1e-3) / 1e12, thr * (kIters / 8) / (msdiv * 1e-3),
      thr * (kIters / 8) / (mssq * 1e-3), clk_khz);
  cudaFree(out);
  if (link) {
    double r[5];
    if (!link_rates(p.multiProcessorCount, r)) {
      std::fprintf(stderr, "pipe_peaks: host-link measurement failed: %s\n", cudaGetErrorString(cudaGetLastError()));
      return 1;
    }
    std::printf(", \"link_gbs\": {\"h2d_copy_engine\": %.1f, \"d2h_copy_engine\": %.1f, "
                "\"both_directions_copy_engines\": %.1f, \"h2d_sm_mapped\": %.1f, \"d2h_sm_mapped\": %.1f, "
                "\"bytes\": %zu}",
                r[0], r[1], r[2], r[3], r[4], size_t(4) * 4096 * 4096 * sizeof(double));
  }
  std::printf("}\n");
  return 0;
}
