// Issue-rate probe of the pipes the pair kernel uses, on the GPU it runs on:
// FP32 FMA (the pair kernel's roofline denominator), FP64 FMA (the FP64
// form's), FP32 <-> FP64 conversions (the integrator's), and the shared-memory
// atomics of the force sums (int32, fp32, fp64).  Each kernel runs a fixed,
// bounded number of independent operations per thread; every shared-memory
// index is masked into its array.  Prints one JSON object.
//
//   nvcc -O3 -gencode arch=compute_103a,code=sm_103a pipe_rates.cu -o pipe_rates
#include <cuda_runtime.h>

#include <cstdio>

#define CK(x)                                                                 \
  do {                                                                        \
    cudaError_t e_ = (x);                                                     \
    if (e_ != cudaSuccess) {                                                  \
      std::fprintf(stderr, "CUDA error %s at line %d\n", cudaGetErrorString(e_), __LINE__); \
      return 1;                                                               \
    }                                                                         \
  } while (0)

// 8 independent FMA chains per thread, 8 unrolled steps per iteration.
__global__ void k_ffma(float* out, int iters) {
  float a[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = threadIdx.x * 1e-3f + k;
  for (int i = 0; i < iters; ++i)
#pragma unroll
    for (int u = 0; u < 8; ++u)
#pragma unroll
      for (int k = 0; k < 8; ++k) a[k] = fmaf(a[k], 0.999f, 1e-4f);
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += a[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void k_dfma(double* out, int iters) {
  double a[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) a[k] = threadIdx.x * 1e-3 + k;
  for (int i = 0; i < iters; ++i)
#pragma unroll
    for (int u = 0; u < 8; ++u)
#pragma unroll
      for (int k = 0; k < 4; ++k) a[k] = fma(a[k], 0.999, 1e-4);
  out[blockIdx.x * blockDim.x + threadIdx.x] = a[0] + a[1] + a[2] + a[3];
}

// FP64 -> FP32 and FP32 -> FP64 conversions: 4 independent chains per thread;
// each step feeds the converted bits back through integer adds so that no
// conversion can be folded away.
__global__ void k_d2f(float* out, int iters) {
  long long b[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) b[k] = __double_as_longlong(1.0 + 1e-3 * (threadIdx.x + k));
  for (int i = 0; i < iters; ++i)
#pragma unroll
    for (int u = 0; u < 8; ++u)
#pragma unroll
      for (int k = 0; k < 4; ++k) b[k] += __float_as_int((float)__longlong_as_double(b[k])) & 0xff;
  out[blockIdx.x * blockDim.x + threadIdx.x] = (float)((b[0] ^ b[1] ^ b[2] ^ b[3]) & 0xffff);
}

__global__ void k_f2d(float* out, int iters) {
  int b[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) b[k] = __float_as_int(1.f + 1e-3f * (threadIdx.x + k));
  for (int i = 0; i < iters; ++i)
#pragma unroll
    for (int u = 0; u < 8; ++u)
#pragma unroll
      for (int k = 0; k < 4; ++k) b[k] += __double2loint((double)__int_as_float(b[k])) & 0xff;
  out[blockIdx.x * blockDim.x + threadIdx.x] = (float)((b[0] ^ b[1] ^ b[2] ^ b[3]) & 0xffff);
}

// Shared-memory atomic adds, 8 per iteration per thread, lanes on distinct
// addresses (the force sums' common case).
template <typename T>
__global__ void k_satom(float* out, int iters) {
  __shared__ T s[2048];
  for (int i = threadIdx.x; i < 2048; i += blockDim.x) s[i] = T(0);
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const T v = T(1 + lane);
  for (int i = 0; i < iters; ++i)
#pragma unroll
    for (int u = 0; u < 8; ++u) atomicAdd(&s[(w * 64 + lane + u * 37 + i * 5) & 2047], v);
  __syncthreads();
  out[blockIdx.x * blockDim.x + threadIdx.x] = (float)s[threadIdx.x & 2047];
}

int main() {
  cudaDeviceProp pr;
  CK(cudaGetDeviceProperties(&pr, 0));
  int clk_khz = 0;
  CK(cudaDeviceGetAttribute(&clk_khz, cudaDevAttrClockRate, 0));
  const int sms = pr.multiProcessorCount, threads = 256, blocks = sms * 8, n = threads * blocks;
  float* of = nullptr;
  double* od = nullptr;
  CK(cudaMalloc(&of, n * sizeof(float)));
  CK(cudaMalloc(&od, n * sizeof(double)));
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  // Best of 5 timed launches after one warm-up launch.
  auto time_ms = [&](auto launch) -> double {
    launch();
    cudaDeviceSynchronize();
    float best = 1e30f;
    for (int r = 0; r < 5; ++r) {
      cudaEventRecord(e0);
      launch();
      cudaEventRecord(e1);
      cudaEventSynchronize(e1);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (ms < best) best = ms;
    }
    return best;
  };
  const int it = 2000;
  const double t_ffma = time_ms([&] { k_ffma<<<blocks, threads>>>(of, it); });
  const double t_dfma = time_ms([&] { k_dfma<<<blocks, threads>>>(od, it / 16); });
  const double t_d2f = time_ms([&] { k_d2f<<<blocks, threads>>>(of, it / 16); });
  const double t_f2d = time_ms([&] { k_f2d<<<blocks, threads>>>(of, it / 16); });
  const double t_ai = time_ms([&] { k_satom<int><<<blocks, threads>>>(of, it / 8); });
  const double t_af = time_ms([&] { k_satom<float><<<blocks, threads>>>(of, it / 8); });
  const double t_ad = time_ms([&] { k_satom<double><<<blocks, threads>>>(of, it / 64); });
  CK(cudaGetLastError());
  CK(cudaDeviceSynchronize());
  const double hz = clk_khz * 1e3;
  auto per_clk = [&](double ops, double ms) { return ops / (ms * 1e-3) / sms / hz; };
  const double ffma_ops = (double)n * it * 64, dfma_ops = (double)n * (it / 16) * 32;
  std::printf(
      "{\"device\": \"%s\", \"sms\": %d, \"clock_mhz\": %.0f, "
      "\"ffma_per_clk_sm\": %.2f, \"fp32_tflops\": %.2f, "
      "\"dfma_per_clk_sm\": %.3f, \"fp64_tflops\": %.3f, "
      "\"cvt_f64_to_f32_per_clk_sm\": %.3f, \"cvt_f32_to_f64_per_clk_sm\": %.3f, "
      "\"smem_atomic_add_per_clk_sm\": {\"i32\": %.2f, \"f32\": %.2f, \"f64\": %.3f}}\n",
      pr.name, sms, hz * 1e-6, per_clk(ffma_ops, t_ffma), 2.0 * ffma_ops / (t_ffma * 1e-3) * 1e-12,
      per_clk(dfma_ops, t_dfma), 2.0 * dfma_ops / (t_dfma * 1e-3) * 1e-12,
      per_clk((double)n * (it / 16) * 32, t_d2f), per_clk((double)n * (it / 16) * 32, t_f2d),
      per_clk((double)n * (it / 8) * 8, t_ai), per_clk((double)n * (it / 8) * 8, t_af),
      per_clk((double)n * (it / 64) * 8, t_ad));
  cudaFree(of);
  cudaFree(od);
  return 0;
}
