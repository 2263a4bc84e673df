// mg_mlp.cuh — the 9 -> 64 -> 64 -> 5 surrogate MLP evaluated on the tensor cores for a tile of 128 samples.
//
// One CTA of 128 threads owns 128 samples (thread i = sample i = GEMM row i = TMEM lane i).  Per evaluation each
// layer is one BF16 GEMM with FP32 accumulation in TMEM: [128 x 16] x [16 x 64] (inputs padded from 9 to 16),
// [128 x 64] x [64 x 64], [128 x 64] x [64 x 16] (outputs padded from 5 to 16).  Thread 0 issues the tcgen05.mma
// instructions and commits them to an mbarrier; every thread reads its accumulator row back with tcgen05.ld, adds
// the bias, applies tanh and writes the BF16 activation row that feeds the next layer.  Weights stay resident in
// shared memory for the CTA's lifetime.
#pragma once

#include <cuda_bf16.h>

#include "mg_kernels.cuh"
#include "mg_tcgen05.cuh"

namespace mg
{
constexpr int kMlpIn = 9, kMlpHid = 64, kMlpOut = 5;
constexpr int kMlpW1 = 0, kMlpB1 = kMlpW1 + kMlpHid * kMlpIn, kMlpW2 = kMlpB1 + kMlpHid,
              kMlpB2 = kMlpW2 + kMlpHid * kMlpHid, kMlpW3 = kMlpB2 + kMlpHid, kMlpB3 = kMlpW3 + kMlpOut * kMlpHid,
              kMlpInMean = kMlpB3 + kMlpOut, kMlpInStd = kMlpInMean + kMlpIn, kMlpOutMean = kMlpInStd + kMlpIn,
              kMlpOutStd = kMlpOutMean + kMlpOut, kMlpNumParams = kMlpOutStd + kMlpOut;
static_assert(kMlpNumParams == MPPI_MLP_PARAMS, "MLP parameter layout");

// Shared-memory map of one MLP tile (bytes from a 1024-byte aligned base).
struct MlpSmem
{
  static constexpr int W1 = 0;          // 64 x 16 bf16
  static constexpr int W2 = 2048;       // 64 x 64 bf16
  static constexpr int W3 = 10240;      // 16 x 64 bf16
  static constexpr int A1 = 12288;      // 128 x 16 bf16
  static constexpr int A2 = 16384;      // 128 x 64 bf16 (hidden 1, then hidden 2)
  static constexpr int BIAS = 32768;    // fp32 b1[64] b2[64] b3[16]
  static constexpr int NORM = 33792;    // fp32 in_mean[9] in_std[9] out_mean[5] out_std[5] (+ pad)
  static constexpr int TOTAL = 34048;
  static constexpr uint32_t TMEM_COLS = 256;  // D1 at 0, D2 at 64, D3 at 128
};

// Byte offset of element (row, k) in the K-major core-matrix layout of a tile whose K extent is KD.
__device__ __forceinline__ int core_off(int row, int k, int KD)
{
  return ((row >> 3) * (KD >> 3) + (k >> 3)) * 128 + (row & 7) * 16 + (k & 7) * 2;
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b)
{
  const __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<const uint32_t*>(&v);
}

// Load the FP32 parameter vector (FNNHelper row-major layout) into BF16 operand tiles and FP32 biases.
__device__ __forceinline__ void mlp_load_weights(unsigned char* sm, const float* params)
{
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int e = tid; e < 64 * 16; e += nt)
  {
    const int n = e >> 4, k = e & 15;
    const float v = k < kMlpIn ? params[kMlpW1 + n * kMlpIn + k] : 0.0f;
    *reinterpret_cast<__nv_bfloat16*>(sm + MlpSmem::W1 + core_off(n, k, 16)) = __float2bfloat16_rn(v);
  }
  for (int e = tid; e < 64 * 64; e += nt)
  {
    const int n = e >> 6, k = e & 63;
    *reinterpret_cast<__nv_bfloat16*>(sm + MlpSmem::W2 + core_off(n, k, 64)) =
        __float2bfloat16_rn(params[kMlpW2 + n * kMlpHid + k]);
  }
  for (int e = tid; e < 16 * 64; e += nt)
  {
    const int n = e >> 6, k = e & 63;
    const float v = n < kMlpOut ? params[kMlpW3 + n * kMlpHid + k] : 0.0f;
    *reinterpret_cast<__nv_bfloat16*>(sm + MlpSmem::W3 + core_off(n, k, 64)) = __float2bfloat16_rn(v);
  }
  float* bias = reinterpret_cast<float*>(sm + MlpSmem::BIAS);
  for (int e = tid; e < 144; e += nt)
    bias[e] = e < 64 ? params[kMlpB1 + e] : e < 128 ? params[kMlpB2 + e - 64] : (e - 128 < kMlpOut ? params[kMlpB3 + e - 128] : 0.0f);
  float* nrm = reinterpret_cast<float*>(sm + MlpSmem::NORM);
  for (int e = tid; e < 28; e += nt) nrm[e] = params[kMlpInMean + e];
}

// One forward pass of the tile.  Thread i provides its normalised input row xin[9] and receives yout[5]
// (normalised outputs).  Returns false if a bounded wait gave up (the caller stops and frees TMEM).
__device__ __forceinline__ bool mlp_tile_forward(unsigned char* sm, uint32_t taddr, uint64_t* mbar, uint32_t& phase,
                                                 const float* xin, float* yout)
{
  const int m = threadIdx.x, warp = m >> 5;
  const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
  const uint32_t sbase = smem_u32(sm);
  const float* bias = reinterpret_cast<const float*>(sm + MlpSmem::BIAS);
  constexpr uint32_t kId64 = umma_idesc_bf16_f32(128, 64);
  constexpr uint32_t kId16 = umma_idesc_bf16_f32(128, 16);

  // ---- layer 1
  {
    uint4 c0, c1;
    c0.x = pack_bf16(xin[0], xin[1]);
    c0.y = pack_bf16(xin[2], xin[3]);
    c0.z = pack_bf16(xin[4], xin[5]);
    c0.w = pack_bf16(xin[6], xin[7]);
    c1.x = pack_bf16(xin[8], 0.0f);
    c1.y = c1.z = c1.w = 0u;
    *reinterpret_cast<uint4*>(sm + MlpSmem::A1 + core_off(m, 0, 16)) = c0;
    *reinterpret_cast<uint4*>(sm + MlpSmem::A1 + core_off(m, 8, 16)) = c1;
  }
  fence_proxy_async_smem();
  tc_fence_before_sync();
  __syncthreads();
  if (m == 0)
  {
    tc_fence_after_sync();
    umma_bf16(taddr + 0, umma_smem_desc(sbase + MlpSmem::A1, 128, 256), umma_smem_desc(sbase + MlpSmem::W1, 128, 256),
              kId64, 0u);
    umma_commit(mbar);
  }
  if (__syncthreads_or(!mbar_wait_bounded(mbar, phase, kMaxBarrierSpins) ? 1 : 0)) return false;  // CTA-uniform
  phase ^= 1u;
  tc_fence_after_sync();
#pragma unroll
  for (int q = 0; q < 4; ++q)
  {
    float v[16];
    tmem_ld16(taddr + lane_base + 16 * q, v);
    tmem_ld_wait();
#pragma unroll
    for (int h = 0; h < 2; ++h)
    {
      uint4 c;
      const float* b = bias + 16 * q + 8 * h;
      const float* x = v + 8 * h;
      c.x = pack_bf16(tanh_fast(x[0] + b[0]), tanh_fast(x[1] + b[1]));
      c.y = pack_bf16(tanh_fast(x[2] + b[2]), tanh_fast(x[3] + b[3]));
      c.z = pack_bf16(tanh_fast(x[4] + b[4]), tanh_fast(x[5] + b[5]));
      c.w = pack_bf16(tanh_fast(x[6] + b[6]), tanh_fast(x[7] + b[7]));
      *reinterpret_cast<uint4*>(sm + MlpSmem::A2 + core_off(m, 16 * q + 8 * h, 64)) = c;
    }
  }
  // ---- layer 2
  fence_proxy_async_smem();
  tc_fence_before_sync();
  __syncthreads();
  if (m == 0)
  {
    tc_fence_after_sync();
#pragma unroll
    for (int k = 0; k < 4; ++k)
      umma_bf16(taddr + 64, umma_smem_desc(sbase + MlpSmem::A2 + 256 * k, 128, 1024),
                umma_smem_desc(sbase + MlpSmem::W2 + 256 * k, 128, 1024), kId64, k > 0 ? 1u : 0u);
    umma_commit(mbar);
  }
  if (__syncthreads_or(!mbar_wait_bounded(mbar, phase, kMaxBarrierSpins) ? 1 : 0)) return false;  // CTA-uniform
  phase ^= 1u;
  tc_fence_after_sync();
#pragma unroll
  for (int q = 0; q < 4; ++q)
  {
    float v[16];
    tmem_ld16(taddr + lane_base + 64 + 16 * q, v);
    tmem_ld_wait();
#pragma unroll
    for (int h = 0; h < 2; ++h)
    {
      uint4 c;
      const float* b = bias + 64 + 16 * q + 8 * h;
      const float* x = v + 8 * h;
      c.x = pack_bf16(tanh_fast(x[0] + b[0]), tanh_fast(x[1] + b[1]));
      c.y = pack_bf16(tanh_fast(x[2] + b[2]), tanh_fast(x[3] + b[3]));
      c.z = pack_bf16(tanh_fast(x[4] + b[4]), tanh_fast(x[5] + b[5]));
      c.w = pack_bf16(tanh_fast(x[6] + b[6]), tanh_fast(x[7] + b[7]));
      *reinterpret_cast<uint4*>(sm + MlpSmem::A2 + core_off(m, 16 * q + 8 * h, 64)) = c;
    }
  }
  // ---- layer 3 (linear)
  fence_proxy_async_smem();
  tc_fence_before_sync();
  __syncthreads();
  if (m == 0)
  {
    tc_fence_after_sync();
#pragma unroll
    for (int k = 0; k < 4; ++k)
      umma_bf16(taddr + 128, umma_smem_desc(sbase + MlpSmem::A2 + 256 * k, 128, 1024),
                umma_smem_desc(sbase + MlpSmem::W3 + 256 * k, 128, 1024), kId16, k > 0 ? 1u : 0u);
    umma_commit(mbar);
  }
  if (__syncthreads_or(!mbar_wait_bounded(mbar, phase, kMaxBarrierSpins) ? 1 : 0)) return false;  // CTA-uniform
  phase ^= 1u;
  tc_fence_after_sync();
  {
    float v[16];
    tmem_ld16(taddr + lane_base + 128, v);
    tmem_ld_wait();
#pragma unroll
    for (int j = 0; j < kMlpOut; ++j) yout[j] = v[j] + bias[128 + j];
  }
  tc_fence_before_sync();
  return true;
}

// Rollout of the MLP bicycle model over every instance (defined in mg_mlp.cu).
mppi_status launch_mlp_rollout(const RolloutArgs<BicycleSlipMLPModel>& a, const float* mlp_d, int num_sms,
                               cudaStream_t s);

// Host twin of the surrogate dynamics in FP32 (exact tanh), used for the nominal state trajectory of a controller
// (Controller::computeOutputTrajectoryHelper, controller.cuh:664-684).
inline void mlp_host_dynamics(const float* P, const float* x, const float* u, float* xd)
{
  float sy, cy;
  sincos_f(x[2], &sy, &cy);
  xd[0] = x[3] * cy - x[4] * sy;
  xd[1] = x[3] * sy + x[4] * cy;
  float in[kMlpIn], h1[kMlpHid], h2[kMlpHid];
  for (int i = 0; i < 7; ++i) in[i] = (x[i] - P[kMlpInMean + i]) / P[kMlpInStd + i];
  for (int i = 0; i < 2; ++i) in[7 + i] = (u[i] - P[kMlpInMean + 7 + i]) / P[kMlpInStd + 7 + i];
  for (int j = 0; j < kMlpHid; ++j)
  {
    float z = P[kMlpB1 + j];
    for (int i = 0; i < kMlpIn; ++i) z = fmaf(P[kMlpW1 + j * kMlpIn + i], in[i], z);
    h1[j] = tanhf(z);
  }
  for (int j = 0; j < kMlpHid; ++j)
  {
    float z = P[kMlpB2 + j];
    for (int i = 0; i < kMlpHid; ++i) z = fmaf(P[kMlpW2 + j * kMlpHid + i], h1[i], z);
    h2[j] = tanhf(z);
  }
  for (int j = 0; j < kMlpOut; ++j)
  {
    float z = P[kMlpB3 + j];
    for (int i = 0; i < kMlpHid; ++i) z = fmaf(P[kMlpW3 + j * kMlpHid + i], h2[i], z);
    xd[2 + j] = z * P[kMlpOutStd + j] + P[kMlpOutMean + j];
  }
}

}  // namespace mg
