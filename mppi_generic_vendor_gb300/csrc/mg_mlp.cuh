// mg_mlp.cuh — the 9 -> 64 -> 64 -> 5 surrogate MLP evaluated on the tensor cores for a tile of 128 samples.
//
// One CTA of 128 threads owns 128 samples (thread i = sample i = GEMM row i = TMEM lane i).  Per evaluation each
// layer is one kind::f16 GEMM with FP32 accumulation in TMEM: [128 x 16] x [16 x 64] (inputs padded from 9 to 16),
// [128 x 64] x [64 x 64], [128 x 64] x [64 x 16] (outputs padded from 5 to 16).  Thread 0 issues the tcgen05.mma
// instructions and commits them to an mbarrier; every thread reads its accumulator row back with tcgen05.ld, applies
// tanh and writes the 16-bit activation row that feeds the next layer.  Weights stay resident in shared memory for
// the CTA's lifetime.
//
// Operand formats.  BF16 weights: BF16 operands, FP32 epilogue (tanh.approx.f32, then rounding to BF16).  FP8 weights
// (E4M3 values q with a power-of-two scale per layer): the weights q * scale are exact in FP16, so the operands are
// FP16 and the epilogue runs on packed pairs (conversion to FP16x2, tanh.approx.f16x2).  In both forms the layer
// scale is folded into the weight tile and the first layer's bias into the GEMM itself (two input columns hold 1.0,
// the matching weight columns the bias split into a high and a low 16-bit part), so the first epilogue is tanh alone.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>

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
// epilogue work between barriers and halve the resident CTAs per SM, which cost more than they saved.
constexpr int kMlpTiles = 1;
constexpr int kMlpSamplesPerCta = 128 * kMlpTiles;

// Shared-memory map of an MLP CTA that evaluates NT tiles of 128 rows (bytes from a 128-byte aligned base).  Each
// tile owns one 128 x 64 16-bit activation buffer: the 128 x 16 input rows of layer 1 sit in its first 4 KB (dead once
// the layer-1 MMA has completed), then hidden 1, then hidden 2 overwrite it, each after the MMA that read the previous
// contents has completed.  The output layer's B operand is 16 rows (N = 16, the smallest N of an M = 128 MMA) of which
// 5 are weights: only rows 0-7 are stored, rows 8-15 read the 1 KB that follows (biases and activations; finite or
// not, they only reach accumulator columns 8-15, which nothing reads).  With the normalisation constants passed as
// kernel parameters the FP16-operand CTA holds 27.3 KB, so eight fit an SM's 228 KB.
struct MlpSmem
{
  static constexpr int W1 = 0;          // 64 x 16 (9 weights, 2 bias parts, 5 zero columns)
  static constexpr int W2 = 2048;       // 64 x 64
  static constexpr int W3 = 10240;      // rows 0-7 of 16 x 64
  static constexpr int BIAS = 11264;    // fp16 b2[64], fp32 b3[16]
  static constexpr int BIAS_B3 = BIAS + 128;
  static constexpr int ACT = 11520;     // NT x (128 x 64)
  static constexpr int ACT_BYTES = 16384;
  // fp32 b2[64] after the activation buffers, BF16-operand form only
  __host__ __device__ static constexpr int bias_f32(int nt) { return ACT + nt * ACT_BYTES; }
  __host__ __device__ static constexpr int total(int nt, bool half) { return bias_f32(nt) + (half ? 0 : 256); }
  // One 64-column accumulator per tile serves all three layers: each layer's result is read back into shared memory
  // before the next layer's MMA is issued.
  static constexpr uint32_t TILE_COLS = 64;
  __host__ __device__ static constexpr uint32_t tmem_cols(int nt) { return nt == 1 ? 64u : nt == 2 ? 128u : 256u; }
};
static_assert(MlpSmem::W3 + 2048 <= MlpSmem::total(1, true), "the output weights' unused rows stay inside the CTA");

// Normalisation of the network's inputs and outputs, passed by value (kernel parameter space: read as constant-bank
// operands, no shared memory): physical input x enters as (x - in_mean) * in_scale, in_scale = 1 / in_std; output y
// leaves as y * out_std + out_mean.
struct MlpNorm
{
  float in_mean[kMlpIn], in_scale[kMlpIn], out_mean[kMlpOut], out_std[kMlpOut];
};
inline MlpNorm mlp_norm(const float* params)
{
  MlpNorm n;
  for (int i = 0; i < kMlpIn; ++i)
  {
    n.in_mean[i] = params[kMlpInMean + i];
    n.in_scale[i] = 1.0f / params[kMlpInStd + i];
  }
  for (int j = 0; j < kMlpOut; ++j)
  {
    n.out_mean[j] = params[kMlpOutMean + j];
    n.out_std[j] = params[kMlpOutStd + j];
  }
  return n;
}

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
__device__ __forceinline__ uint32_t pack_f16(float a, float b)
{
  const __half2 v = __floats2half2_rn(a, b);
  return *reinterpret_cast<const uint32_t*>(&v);
}
template <bool kHalf>
__device__ __forceinline__ uint32_t pack16(float a, float b)
{
  return kHalf ? pack_f16(a, b) : pack_bf16(a, b);
}
template <bool kHalf>
__device__ __forceinline__ void store16(unsigned char* p, float v)
{
  if constexpr (kHalf)
    *reinterpret_cast<__half*>(p) = __float2half_rn(v);
  else
    *reinterpret_cast<__nv_bfloat16*>(p) = __float2bfloat16_rn(v);
}
template <bool kHalf>
__device__ __forceinline__ float round16(float v)
{
  if constexpr (kHalf)
    return __half2float(__float2half_rn(v));
  else
    return __bfloat162float(__float2bfloat16_rn(v));
}

// Load the device parameter vector (FNNHelper row-major layout + layer scales) into 16-bit operand tiles (BF16, or
// FP16 when kHalf) and the remaining biases.  Each weight tile holds q * scale of its layer: exact for E4M3 values
// with a power-of-two scale in FP16 (and for BF16 weights, whose scale is 1).  Columns 9 and 10 of the first tile hold
// the first bias as a high and a low 16-bit part, multiplied by the input rows' constant 1.0 columns.
template <bool kHalf>
__device__ __forceinline__ void mlp_load_weights(unsigned char* sm, const float* params)
{
  const int tid = threadIdx.x, nt = blockDim.x;
  const float s1 = params[kMlpScale], s2 = params[kMlpScale + 1], s3 = params[kMlpScale + 2];
  for (int e = tid; e < 64 * 16; e += nt)
  {
    const int n = e >> 4, k = e & 15;
    const float b = params[kMlpB1 + n];
    const float v = k < kMlpIn        ? params[kMlpW1 + n * kMlpIn + k] * s1
                    : k == kMlpIn     ? b
                    : k == kMlpIn + 1 ? b - round16<kHalf>(b)
                                      : 0.0f;
    store16<kHalf>(sm + MlpSmem::W1 + core_off(n, k, 16), v);
  }
  for (int e = tid; e < 64 * 64; e += nt)
  {
    const int n = e >> 6, k = e & 63;
    store16<kHalf>(sm + MlpSmem::W2 + core_off(n, k, 64), params[kMlpW2 + n * kMlpHid + k] * s2);
  }
  for (int e = tid; e < 8 * 64; e += nt)
  {
    const int n = e >> 6, k = e & 63;
    const float v = n < kMlpOut ? params[kMlpW3 + n * kMlpHid + k] * s3 : 0.0f;
    store16<kHalf>(sm + MlpSmem::W3 + core_off(n, k, 64), v);
  }
  __half* b2_h = reinterpret_cast<__half*>(sm + MlpSmem::BIAS);
  float* b3 = reinterpret_cast<float*>(sm + MlpSmem::BIAS_B3);
  float* b2 = reinterpret_cast<float*>(sm + MlpSmem::bias_f32(kMlpTiles));
  for (int e = tid; e < kMlpHid; e += nt)
  {
    if constexpr (kHalf)
      b2_h[e] = __float2half_rn(params[kMlpB2 + e]);
    else
      b2[e] = params[kMlpB2 + e];
  }
  for (int e = tid; e < 16; e += nt) b3[e] = e < kMlpOut ? params[kMlpB3 + e] : 0.0f;
}

// One forward pass of NT tiles.  Thread i provides the normalised input rows xin[n][9] of rows i of tiles n and
// receives yout[n][5] (normalised outputs).  Per layer every tile's MMAs are issued by thread 0 and committed to one
// mbarrier, so the CTA pays one round trip per layer for all of its tiles.  A bounded wait that gives up sets *fail
// (shared); every thread reads the flag after the next CTA barrier, so the pass returns false on all threads together
// (the caller stops and frees TMEM).  A failure in the last layer surfaces at the caller's next barrier.
template <int NT, bool kHalf>
__device__ __forceinline__ bool mlp_tile_forward(unsigned char* sm, uint32_t taddr, uint64_t* mbar, uint32_t& phase,
                                                 volatile int* fail, const float (*xin)[kMlpIn],
                                                 float (*yout)[kMlpOut])
{
  const int m = threadIdx.x, warp = m >> 5;
  const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
  const uint32_t sbase = smem_u32(sm);
  const float* b2 = reinterpret_cast<const float*>(sm + MlpSmem::bias_f32(NT));
  const float* b3 = reinterpret_cast<const float*>(sm + MlpSmem::BIAS_B3);
  constexpr uint32_t kOutCol = 32;  // output-layer accumulator columns (after the packed hidden-2 columns)
  constexpr uint32_t kId64 = kHalf ? umma_idesc_f16_f32(128, 64) : umma_idesc_bf16_f32(128, 64);
  constexpr uint32_t kId16 = kHalf ? umma_idesc_f16_f32(128, 16) : umma_idesc_bf16_f32(128, 16);

  // ---- layer 1: inputs padded from 9 to 16 columns; columns 9 and 10 are 1.0 and pick up the first bias
#pragma unroll
  for (int n = 0; n < NT; ++n)
  {
    const float* x = xin[n];
    uint4 c0, c1;
    c0.x = pack16<kHalf>(x[0], x[1]);
    c0.y = pack16<kHalf>(x[2], x[3]);
    c0.z = pack16<kHalf>(x[4], x[5]);
    c0.w = pack16<kHalf>(x[6], x[7]);
    c1.x = pack16<kHalf>(x[8], 1.0f);
    c1.y = pack16<kHalf>(1.0f, 0.0f);
    c1.z = c1.w = 0u;
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
      umma_f16(taddr + n * MlpSmem::TILE_COLS,
                umma_smem_desc(sbase + MlpSmem::ACT + n * MlpSmem::ACT_BYTES, 128, 256),
                umma_smem_desc(sbase + MlpSmem::W1, 128, 256), kId64, 0u);
    umma_commit(mbar);
  }
  // every warp sleeps on the MMA's mbarrier (waiting costs no issue slots) and then reads its own TMEM lanes, so no
  // CTA barrier follows the wait
  if (!mbar_wait_sleep_bounded(mbar, phase, kMaxSleepWaits)) *fail = 1;
  phase ^= 1u;
  tc_fence_after_sync();

  // ---- hidden layers 1 and 2: tanh epilogue (plus the second bias), then the next GEMM.  Hidden 1 goes to the
  // tile's shared-memory activation buffer (the A operand of layer 2); hidden 2 goes back into TMEM columns 0-31 of
  // the tile's accumulator, packed two per column (each chunk overwrites columns already read), and is the A operand
  // of the output layer, whose result lands in columns 32-47: no shared-memory traffic for the output layer.
#pragma unroll
  for (int layer = 0; layer < 2; ++layer)
  {
#pragma unroll
    for (int n = 0; n < NT; ++n)
    {
      unsigned char* act = sm + MlpSmem::ACT + n * MlpSmem::ACT_BYTES;
#pragma unroll
      for (int q = 0; q < 4; ++q)
      {
        float v[16];
        uint32_t hp[8];  // layer 2: this chunk's eight packed activation columns
        tmem_ld16(taddr + n * MlpSmem::TILE_COLS + lane_base + 16 * q, v);
        tmem_ld_wait();
#pragma unroll
        for (int h = 0; h < 2; ++h)
        {
          uint4 c;
          const float* x = v + 8 * h;
          if constexpr (kHalf)
          {
            uint32_t z[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) z[j] = pack_f16(x[2 * j], x[2 * j + 1]);
            if (layer == 1)
            {
              // eight FP16 biases as one 16-byte shared-memory read (the same address across the warp: a broadcast)
              const uint4 b = *reinterpret_cast<const uint4*>(sm + MlpSmem::BIAS + 2 * (16 * q + 8 * h));
              const uint32_t bw[4] = { b.x, b.y, b.z, b.w };
#pragma unroll
              for (int j = 0; j < 4; ++j)
              {
                const __half2 t = __hadd2(*reinterpret_cast<const __half2*>(&z[j]),
                                          *reinterpret_cast<const __half2*>(&bw[j]));
                z[j] = *reinterpret_cast<const uint32_t*>(&t);
              }
            }
            c.x = tanh_f16x2(z[0]);
            c.y = tanh_f16x2(z[1]);
            c.z = tanh_f16x2(z[2]);
            c.w = tanh_f16x2(z[3]);
          }
          else if (layer == 0)
          {
            c.x = pack_bf16(tanh_fast(x[0]), tanh_fast(x[1]));
            c.y = pack_bf16(tanh_fast(x[2]), tanh_fast(x[3]));
            c.z = pack_bf16(tanh_fast(x[4]), tanh_fast(x[5]));
            c.w = pack_bf16(tanh_fast(x[6]), tanh_fast(x[7]));
          }
          else
          {
            // the biases as two 16-byte shared-memory reads (the same address across the warp: a broadcast)
            const float4 b0 = *reinterpret_cast<const float4*>(b2 + 16 * q + 8 * h);
            const float4 b1 = *reinterpret_cast<const float4*>(b2 + 16 * q + 8 * h + 4);
            c.x = pack_bf16(tanh_fast(x[0] + b0.x), tanh_fast(x[1] + b0.y));
            c.y = pack_bf16(tanh_fast(x[2] + b0.z), tanh_fast(x[3] + b0.w));
            c.z = pack_bf16(tanh_fast(x[4] + b1.x), tanh_fast(x[5] + b1.y));
            c.w = pack_bf16(tanh_fast(x[6] + b1.z), tanh_fast(x[7] + b1.w));
          }
          if (layer == 0)
            *reinterpret_cast<uint4*>(act + core_off(m, 16 * q + 8 * h, 64)) = c;
          else
          {
            hp[4 * h] = c.x;
            hp[4 * h + 1] = c.y;
            hp[4 * h + 2] = c.z;
            hp[4 * h + 3] = c.w;
          }
        }
        if (layer == 1) tmem_st8(taddr + n * MlpSmem::TILE_COLS + lane_base + 8 * q, hp);
      }
    }
    if (layer == 0)
      fence_proxy_async_smem();
    else
      tmem_st_wait();
    tc_fence_before_sync();
    __syncthreads();
    if (*fail) return false;  // CTA-uniform: read after the barrier
    if (m == 0)
    {
      tc_fence_after_sync();
#pragma unroll
      for (int n = 0; n < NT; ++n)
#pragma unroll
        for (int k = 0; k < 4; ++k)
        {
          if (layer == 0)
            umma_f16(taddr + n * MlpSmem::TILE_COLS,
                     umma_smem_desc(sbase + MlpSmem::ACT + n * MlpSmem::ACT_BYTES + 256 * k, 128, 1024),
                     umma_smem_desc(sbase + MlpSmem::W2 + 256 * k, 128, 1024), kId64, k > 0 ? 1u : 0u);
          else
            umma_f16_ts(taddr + n * MlpSmem::TILE_COLS + kOutCol, taddr + n * MlpSmem::TILE_COLS + 8 * k,
                        umma_smem_desc(sbase + MlpSmem::W3 + 256 * k, 128, 1024), kId16, k > 0 ? 1u : 0u);
        }
      umma_commit(mbar);
    }
    if (!mbar_wait_sleep_bounded(mbar, phase, kMaxSleepWaits)) *fail = 1;
    phase ^= 1u;
    tc_fence_after_sync();
  }

  // ---- linear output layer
#pragma unroll
  for (int n = 0; n < NT; ++n)
  {
    float v[16];
    tmem_ld16(taddr + n * MlpSmem::TILE_COLS + lane_base + kOutCol, v);
    tmem_ld_wait();
#pragma unroll
    for (int j = 0; j < kMlpOut; ++j) yout[n][j] = v[j] + b3[j];
  }
  tc_fence_before_sync();
  return true;
}

// Rollout of the MLP bicycle model over every instance (defined in mg_mlp.cu).
// precision 0 / 1: tensor cores with BF16 / FP8 weights; 2: plain FP32 on the CUDA cores.  fused (may be null):
// generate the Gaussian control samples inside the rollout (every instance has T*C % 4 == 0).
mppi_status launch_mlp_rollout(const RolloutArgs<BicycleSlipMLPModel>& a, const float* mlp_d, const MlpNorm& norm,
                               int precision, const FusedNoise* fused, int num_sms, cudaStream_t s);

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
// with one power-of-two scale per layer, the smallest with max |W| / scale <= 448) or 2 (FP32, unchanged), and the
// FP32 parameters those weights represent (q * scale), used by the host twin.
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
