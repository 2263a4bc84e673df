// Throughput of the special-function unit (MUFU) on this GPU, the unit that bounds the surrogate rollout: every
// hidden activation is one tanh.approx, and tanh.approx.f16x2 issues as two MUFU operations.
//
//   sfu_throughput
//
// Every SM runs eight CTAs of 256 threads; each thread chains eight independent tanh.approx.f32 streams through
// 4096 rounds (32 768 MUFU operations per thread, enough independent work to keep the unit busy), timed with CUDA
// events after a warm-up launch.  Prints the MUFU operations per second and per SM clock (at the SM clock it reads
// back), and exits non-zero on a CUDA error.
#include <cstdio>
#include <cuda_runtime.h>

constexpr int kRounds = 4096, kStreams = 8, kThreads = 256, kCtasPerSm = 8;

__global__ void __launch_bounds__(kThreads) sfu_kernel(float* out)
{
  float v[kStreams];
#pragma unroll
  for (int s = 0; s < kStreams; ++s) v[s] = 0.001f * (float)(threadIdx.x + s);
  for (int r = 0; r < kRounds; ++r)
#pragma unroll
    for (int s = 0; s < kStreams; ++s) asm volatile("tanh.approx.f32 %0, %0;" : "+f"(v[s]));
  float acc = 0.0f;
#pragma unroll
  for (int s = 0; s < kStreams; ++s) acc += v[s];
  out[blockIdx.x * blockDim.x + threadIdx.x] = acc;
}

int main()
{
  int dev = 0, sms = 0, clock_khz = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&clock_khz, cudaDevAttrClockRate, dev);
  const int blocks = sms * kCtasPerSm;
  float* out = nullptr;
  if (cudaMalloc(&out, sizeof(float) * (size_t)blocks * kThreads) != cudaSuccess) return 1;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  sfu_kernel<<<blocks, kThreads>>>(out);  // warm-up
  cudaEventRecord(e0);
  sfu_kernel<<<blocks, kThreads>>>(out);
  cudaEventRecord(e1);
  cudaError_t err = cudaEventSynchronize(e1);
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, e0, e1);
  if (err == cudaSuccess) err = cudaGetLastError();
  const double ops = (double)blocks * kThreads * kRounds * kStreams;
  const double per_s = ops / (ms * 1e-3);
  printf("{\"sms\": %d, \"ms\": %.4f, \"mufu_ops_per_s\": %.4e, \"mufu_ops_per_sm_clock\": %.2f, \"clock_mhz\": %.0f, "
         "\"status\": \"%s\"}\n",
         sms, ms, per_s, per_s / sms / (clock_khz * 1e3), clock_khz / 1e3, cudaGetErrorString(err));
  cudaFree(out);
  return err == cudaSuccess ? 0 : 1;
}
