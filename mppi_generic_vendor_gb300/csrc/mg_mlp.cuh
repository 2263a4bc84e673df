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
// Device copy: the parameter vector followed by one scale per layer.  BF16 weights carry scale 1; FP8 weights hold
// E4M3 values q with W = q * scale, the scale applied to the FP32 accumulator in the epilogue.
constexpr int kMlpScale = kMlpNumParams, kMlpDevParams = kMlpScale + 3;

// Tiles of 128 samples per CTA of the surrogate rollout; its work items hold kMlpSamplesPerCta samples of one
// instance.  One tile per CTA measured fastest: two tiles per CTA halve the MMA round trips per tile but double the
// epilogue work between barriers and cut the resident CTAs per SM from 7 to 4, which cost more than they saved.
constexpr int kMlpTiles = 1;
constexpr int kMlpSamplesPerCta = 128 * kMlpTiles;

// Shared-memory map of an MLP CTA that evaluates NT tiles of 128 rows (bytes from a 1024-byte aligned base).  Each
// tile owns one 128 x 64 BF16 activation buffer: the 128 x 16 input rows of layer 1 sit in its first 4 KB (dead once
// the layer-1 MMA has completed), then hidden 1, then hidden 2 overwrite it, each after the MMA that read the previous
// contents has completed.
struct MlpSmem
{
  static constexpr int W1 = 0;          // 64 x 16 bf16
  static constexpr int W2 = 2048;       // 64 x 64 bf16
  static constexpr int W3 = 10240;      // 16 x 64 bf16
  static constexpr int BIAS = 12288;    // fp32 b1[64] b2[64] b3[16]
  static constexpr int NORM = 13312;    // fp32 in_mean[9] in_std[9] out_mean[5] out_std[5] layer_scale[3] pad
                                        //      1/in_std[9] (from float 32)
  static constexpr int ACT = 14336;     // NT x (128 x 64 bf16)
  static constexpr int ACT_BYTES = 16384;
  __host__ __device__ static constexpr int total(int nt) { return ACT + nt * ACT_BYTES; }
  // One 64-column accumulator per tile serves all three layers: each layer's result is read back into shared memory
  // before the next layer's MMA is issued.
  static constexpr uint32_t TILE_COLS = 64;
  __host__ __device__ static constexpr uint32_t tmem_cols(int nt) { return nt == 1 ? 64u : nt == 2 ? 128u : 256u; }
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

// Load the device parameter vector (FNNHelper row-major layout + layer scales) into BF16 operand tiles and FP32
// biases.  E4M3 values are exact in BF16, so FP8 weights reach the tensor cores unrounded.
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
  for (int e = tid; e < 31; e += nt) nrm[e] = params[kMlpInMean + e];  // normalisation + layer scales
  for (int e = tid; e < kMlpIn; e += nt) nrm[32 + e] = 1.0f / params[kMlpInStd + e];  // input scale reciprocals
}

// One forward pass of NT tiles.  Thread i provides the normalised input rows xin[n][9] of rows i of tiles n and
// receives yout[n][5] (normalised outputs).  Per layer every tile's MMAs are issued by thread 0 and committed to one
// mbarrier, so the CTA pays one round trip per layer for all of its tiles.  A bounded wait that gives up sets *fail
// (shared); every thread reads the flag after the next CTA barrier, so the pass returns false on all threads together
// (the caller stops and frees TMEM).  A failure in the last layer surfaces at the caller's next barrier.
template <int NT>
__device__ __forceinline__ bool mlp_tile_forward(unsigned char* sm, uint32_t taddr, uint64_t* mbar, uint32_t& phase,
                                                 volatile int* fail, const float (*xin)[kMlpIn],
                                                 float (*yout)[kMlpOut])
{
  const int m = threadIdx.x, warp = m >> 5;
  const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
  const uint32_t sbase = smem_u32(sm);
  const float* bias = reinterpret_cast<const float*>(sm + MlpSmem::BIAS);
  const float* lscale = reinterpret_cast<const float*>(sm + MlpSmem::NORM) + 28;
  const float s1 = lscale[0], s2 = lscale[1], s3 = lscale[2];
  constexpr uint32_t kId64 = umma_idesc_bf16_f32(128, 64);
  constexpr uint32_t kId16 = umma_idesc_bf16_f32(128, 16);

  // ---- layer 1: inputs padded from 9 to 16 columns
#pragma unroll
  for (int n = 0; n < NT; ++n)
  {
    const float* x = xin[n];
    uint4 c0, c1;
    c0.x = pack_bf16(x[0], x[1]);
    c0.y = pack_bf16(x[2], x[3]);
    c0.z = pack_bf16(x[4], x[5]);
    c0.w = pack_bf16(x[6], x[7]);
    c1.x = pack_bf16(x[8], 0.0f);
    c1.y = c1.z = c1.w = 0u;
    unsigned char* a1 = sm + MlpSmem::ACT + n * MlpSmem::ACT_BYTES;
    *reinterpret_cast<uint4*>(a1 + core_off(m, 0, 16)) = c0;
    *reinterpret_cast<uint4*>(a1 + core_off(m, 8, 16)) = c1;
  }
  fence_proxy_async_smem();
  tc_fence_before_sync();
  __syncthreads();
  if (*fail) return false;  // CTA-uniform: read after the barrier
  if (m == 0)
  {
    tc_fence_after_sync();
#pragma unroll
    for (int n = 0; n < NT; ++n)
      umma_bf16(taddr + n * MlpSmem::TILE_COLS,
                umma_smem_desc(sbase + MlpSmem::ACT + n * MlpSmem::ACT_BYTES, 128, 256),
                umma_smem_desc(sbase + MlpSmem::W1, 128, 256), kId64, 0u);
    umma_commit(mbar);
  }
  // one warp sleeps on the MMA's mbarrier, the others at the CTA barrier: waiting costs no issue slots
  if (warp == 0 && !mbar_wait_sleep_bounded(mbar, phase, kMaxSleepWaits)) *fail = 1;
  __syncthreads();
  phase ^= 1u;
  tc_fence_after_sync();

  // ---- hidden layers 1 and 2: bias + tanh epilogue into the tile's activation buffer, then the next GEMM
#pragma unroll
  for (int layer = 0; layer < 2; ++layer)
  {
    const float sc = layer == 0 ? s1 : s2;
#pragma unroll
    for (int n = 0; n < NT; ++n)
    {
      unsigned char* act = sm + MlpSmem::ACT + n * MlpSmem::ACT_BYTES;
#pragma unroll
      for (int q = 0; q < 4; ++q)
      {
        float v[16];
        tmem_ld16(taddr + n * MlpSmem::TILE_COLS + lane_base + 16 * q, v);
        tmem_ld_wait();
#pragma unroll
        for (int h = 0; h < 2; ++h)
        {
          uint4 c;
          // the biases as two 16-byte shared-memory reads (the same address across the warp: a broadcast)
          const float4 b0 = *reinterpret_cast<const float4*>(bias + 64 * layer + 16 * q + 8 * h);
          const float4 b1 = *reinterpret_cast<const float4*>(bias + 64 * layer + 16 * q + 8 * h + 4);
          const float* x = v + 8 * h;
          c.x = pack_bf16(tanh_fast(fmaf(x[0], sc, b0.x)), tanh_fast(fmaf(x[1], sc, b0.y)));
          c.y = pack_bf16(tanh_fast(fmaf(x[2], sc, b0.z)), tanh_fast(fmaf(x[3], sc, b0.w)));
          c.z = pack_bf16(tanh_fast(fmaf(x[4], sc, b1.x)), tanh_fast(fmaf(x[5], sc, b1.y)));
          c.w = pack_bf16(tanh_fast(fmaf(x[6], sc, b1.z)), tanh_fast(fmaf(x[7], sc, b1.w)));
          *reinterpret_cast<uint4*>(act + core_off(m, 16 * q + 8 * h, 64)) = c;
        }
      }
    }
    fence_proxy_async_smem();
    tc_fence_before_sync();
    __syncthreads();
    if (*fail) return false;  // CTA-uniform: read after the barrier
    if (m == 0)
    {
      tc_fence_after_sync();
      const uint32_t wb = sbase + (layer == 0 ? MlpSmem::W2 : MlpSmem::W3);
      const uint32_t id = layer == 0 ? kId64 : kId16;
#pragma unroll
      for (int n = 0; n < NT; ++n)
#pragma unroll
        for (int k = 0; k < 4; ++k)
          umma_bf16(taddr + n * MlpSmem::TILE_COLS,
                    umma_smem_desc(sbase + MlpSmem::ACT + n * MlpSmem::ACT_BYTES + 256 * k, 128, 1024),
                    umma_smem_desc(wb + 256 * k, 128, 1024), id, k > 0 ? 1u : 0u);
      umma_commit(mbar);
    }
    if (warp == 0 && !mbar_wait_sleep_bounded(mbar, phase, kMaxSleepWaits)) *fail = 1;
    __syncthreads();
    phase ^= 1u;
    tc_fence_after_sync();
  }

  // ---- linear output layer
#pragma unroll
  for (int n = 0; n < NT; ++n)
  {
    float v[16];
    tmem_ld16(taddr + n * MlpSmem::TILE_COLS + lane_base, v);
    tmem_ld_wait();
#pragma unroll
    for (int j = 0; j < kMlpOut; ++j) yout[n][j] = fmaf(v[j], s3, bias[128 + j]);
  }
  tc_fence_before_sync();
  return true;
}

// Rollout of the MLP bicycle model over every instance (defined in mg_mlp.cu).
// precision 0 / 1: tensor cores with BF16 / FP8 weights; 2: plain FP32 on the CUDA cores.  fused (may be null):
// generate the Gaussian control samples inside the rollout (every instance has T*C % 4 == 0).
mppi_status launch_mlp_rollout(const RolloutArgs<BicycleSlipMLPModel>& a, const float* mlp_d, int precision,
                               const FusedNoise* fused, int num_sms, cudaStream_t s);

// Analytic judge of the surrogate rollout.  Per instance the M lowest surrogate costs (M = ceil(fraction * K), the
// samples that carry the weight) are re-rolled with the analytic BicycleSlipModel in FP32.  Their costs become
// analytic - mean(analytic - surrogate), which ranks them by the exact model while keeping one cost scale with the
// samples that were not re-rolled (a per-instance shift leaves the MPPI weights unchanged), and the baseline is
// recomputed over the corrected costs.
struct JudgeArgs
{
  RolloutArgs<BicycleSlipMLPModel> r;  // instances, parameters, samples, costs and baseline of the rollout
  int num_instances;
  const int* sel_off;           // I + 1 entries: instance i owns judged slots sel_off[i] .. sel_off[i+1]-1
  const int* sel_inst;          // per judged slot: its instance
  int* sel;                     // per judged slot: sample index within the instance (ascending)
  float* judged_cost;           // per judged slot: analytic cost
  unsigned int* unjudged_min;   // per instance: ordered-int min over the samples that were not re-rolled
  float* stats;                 // per instance: mean(analytic - surrogate), mean |analytic - surrogate| / |analytic|
  int total;                    // judged slots over all instances
};
mppi_status launch_judge(const JudgeArgs& a, cudaStream_t s);

// Device parameter vector (kMlpDevParams floats) for precision 0 (BF16 weights, scales 1), 1 (FP8 E4M3 weights
// with one scale per layer, scale = max |W| / 448) or 2 (FP32, unchanged), and the FP32 parameters those weights
// represent (q * scale), used by the host twin.
void mlp_prepare(const float* params, int precision, float* dev_out, float* effective_out);
// Round to the nearest E4M3 value (ties to even, saturating at +-448).
float e4m3_round(float x);

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
