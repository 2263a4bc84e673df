// mg_kernels.cuh — the MPPI iteration as three batched kernels: sample, rollout, weights+update.
//
// All kernels take a table of instances (independent controllers with their own K, T, parameters and nominal
// control) and a work list, so one launch serves any number of uneven instances.  Data layout in HBM:
//   samples   float[sum_i pad4(K_i*T_i*C)]   instance i at u_off, element ((k*T_i + t)*C + c)   ([D=1][K][T][C] of
//             the reference, sampling_distribution.cu:108-116)
//   costs     float[sum_i K_i]               instance i at k_off
//   weights   float[sum_i K_i]
//   mean      float[sum_i T_i*C]             instance i at t_off (the nominal control / importance sampler)
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "mg_math.cuh"
#include "mg_models.cuh"
#include "mg_ptx.cuh"

namespace mg
{
constexpr int kMaxC = MPPI_MAX_CONTROL_DIM;
constexpr int kMaxS = MPPI_MAX_STATE_DIM;

struct InstDesc
{
  int K, T;
  int k_off;         // into costs / weights
  int t_off;         // into mean (floats)
  long long u_off;   // into samples (floats, multiple of 4)
  long long spec_off;  // into the colored-noise spectrum (floats)
  int x_off;         // into x0 (floats)
  int num_chunks;    // weight/update chunks of this instance
  // the noise this instance draws: its own Philox stream and injected noise, or those of instance noise_inst (a
  // Tube-MPPI handle's second distribution with use_same_noise_for_all_distributions)
  int noise_inst;
  long long noise_off;       // injected Gaussian noise (floats, samples layout)
  long long noise_spec_off;  // injected colored-noise spectrum (floats)
};

// Uniform (per handle) sampling + constraint parameters.
struct SampleShared
{
  float std_dev[kMaxC];
  float inv_var[kMaxC];  // 1 / std_dev^2 (the surrogate rollout's likelihood term multiplies by it)
  float control_cost_coeff[kMaxC];
  float lower[kMaxC], upper[kMaxC], deadband[kMaxC], zero[kMaxC];
  float pure_pct;
  // The constraint pass after smoothing: 0 = Dynamics::enforceConstraints on every control (VanillaMPPIController);
  // 1 = ColoredMPPIController's pass, a plain clamp of control 1 to its range and nothing else
  // (colored_mppi_controller.cu:224-229).
  int final_clamp;
};

// Ordered-integer encoding of a float so unsigned atomicMin orders like the float (NaN counts as +inf).
__device__ __forceinline__ unsigned int float_to_ordered(float f)
{
  if (f != f) f = __int_as_float(0x7f800000);
  const unsigned int b = __float_as_uint(f);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__host__ __device__ __forceinline__ float ordered_to_float(unsigned int o)
{
  const unsigned int b = (o & 0x80000000u) ? (o & 0x7fffffffu) : ~o;
#if defined(__CUDA_ARCH__)
  return __uint_as_float(b);
#else
  float f;
  memcpy(&f, &b, 4);
  return f;
#endif
}
constexpr unsigned int kOrderedPosInf = 0xff800000u;

// ============================================================================================== 1. Gaussian sampler
// setGaussianControls (gaussian.cu:17-277) fused with the noise generation it consumes (curandGenerateNormal,
// gaussian.cu:375-395) and with Dynamics::enforceConstraints (dynamics.cu:107-126).  Each thread writes whole float4
// quads; the Philox block index of a quad is its quad index inside the instance, the Philox stream is the instance,
// and the Philox counter is the handle's iteration counter (read from device memory, so a captured graph advances
// it without host involvement).
struct SampleArgs
{
  const InstDesc* inst;
  const int2* work;  // (instance, first quad)
  int num_work;
  int quads_per_item;
  float* samples;
  const float* mean;
  const float* injected;  // standard-normal noise in samples layout, or nullptr for Philox
  const unsigned int* noise_counter;
  uint32_t seed_lo, seed_hi;
  int stride;
  float decay_pow;
  SampleShared sh;
};

template <int C>
__global__ void __launch_bounds__(256) gaussian_sample_kernel(const __grid_constant__ SampleArgs a)
{
  for (int item = blockIdx.x; item < a.num_work; item += gridDim.x)
  {
    const int2 w = a.work[item];
    const InstDesc d = a.inst[w.x];
    const long long n = (long long)d.K * d.T * C;
    const long long nq = (n + 3) / 4;
    const int TC = d.T * C;
    const float pure_threshold = (1.0f - a.sh.pure_pct) * (float)d.K;
    const uint32_t counter = a.noise_counter ? *a.noise_counter : 0u;
    const long long q_end = min((long long)w.y + a.quads_per_item, nq);
    for (long long q = (long long)w.y + threadIdx.x; q < q_end; q += blockDim.x)
    {
      float4 z;
      if (a.injected)
      {
        const float* src = a.injected + d.noise_off + 4 * q;
        if (4 * q + 3 < n)
        {
          z = *reinterpret_cast<const float4*>(src);
        }
        else
        {  // tail quad: never read past the caller's buffer
          z.x = src[0];
          z.y = (4 * q + 1 < n) ? src[1] : 0.0f;
          z.z = (4 * q + 2 < n) ? src[2] : 0.0f;
          z.w = 0.0f;
        }
      }
      else
      {
        z = philox_normal4((uint64_t)q, (uint32_t)d.noise_inst, counter, a.seed_lo, a.seed_hi);
      }
      float zz[4] = { z.x, z.y, z.z, z.w };
      float out[4];
#pragma unroll
      for (int j = 0; j < 4; ++j)
      {
        const long long e = 4 * q + j;
        const int k = (int)(e / TC);
        const int rem = (int)(e - (long long)k * TC);
        const int t = rem / C;
        const int c = rem - t * C;
        const float m = (e < n) ? a.mean[d.t_off + rem] : 0.0f;
        const float sd = a.decay_pow * a.sh.std_dev[c];
        float u;
        if (k == 0 || t < a.stride)
          u = m;
        else if ((float)k >= pure_threshold)
          u = sd * zz[j];
        else
          u = fmaf(sd, zz[j], m);
        out[j] = enforce_constraint(u, a.sh.lower[c], a.sh.upper[c], a.sh.deadband[c], a.sh.zero[c]);
      }
      float* dst = a.samples + d.u_off + 4 * q;
      if (4 * q + 3 < n)
      {
        *reinterpret_cast<float4*>(dst) = make_float4(out[0], out[1], out[2], out[3]);
      }
      else
      {
        for (int j = 0; j < 4; ++j)
          if (4 * q + j < n) dst[j] = out[j];
      }
    }
  }
}

// ============================================================================================== 2. rollout
// rolloutKernel (mppi_common.cu:35-153) restructured for the GB300: one thread per sample with its state in
// registers; the CTA stages a time chunk of its samples' controls in shared memory with coalesced 16-byte loads
// (rows padded by 4 floats so the per-thread 16-byte reads are bank-conflict free); running cost accumulates in FP32
// in reference order; cost = running / T + terminal / T (computeAndSaveCost, mppi_common.cu:879-889).  The CTA also
// folds its samples into the instance's minimum cost with one atomicMin, which the weight kernel consumes as the
// baseline.  The kernel is persistent: CTAs pull (instance, first sample) tiles from a work list ordered by
// decreasing cost through an atomic counter; the last CTA to finish resets the counters for the next launch.
// Weighted reduction done at the end of each rollout tile (the update kernel then only combines tiles): with the
// tile's own minimum cost b_l as baseline, w = expf(-(c - b_l) / lambda) (the arithmetic of the weight transform),
// the tile's partial sums S_l[t][c] = sum_k w_k u_k[t][c] (FP32, samples in index order) and sum w, sum w^2 (FP64).
// tile_finalize_kernel rescales each tile by exp(-(b_l - b) / lambda) with the instance's minimum b, which is the
// same weighted mean up to rounding, without reading the control samples from HBM a second time.
struct TileReduce
{
  float* partials;          // per work tile: T*C floats at poff[tile]; null: weights_update_kernel reduces instead
  const long long* poff;
  double* sums;             // per work tile: sum w, sum w^2 (tile baseline)
  unsigned int* tmin;       // per work tile: ordered-int minimum cost
  float lambda_inv;
  int u_stride;             // > 0: the fused rollout stages its tile's controls in dynamic shared memory,
                            // element-major with this row stride (an odd number >= samples per CTA)
};

// Combines the rollout tiles' partial reductions (TileReduce) into each instance's new mean, one CTA per instance:
// tile l is rescaled by r_l = exp(-(b_l - b) / lambda) (difference in FP64), b the instance's minimum cost;
// eta = sum_l r_l sum_w_l (FP64), mean[j] = sum_l r_l S_l[j] / eta (FP32, four interleaved partial sums over the
// tiles).  Then the same bookkeeping as weights_update_kernel's last block.  Dynamic shared memory: one float per
// tile of the largest instance.
struct FinalizeArgs
{
  const InstDesc* inst;
  int num_instances;
  const int* inst_tile0;  // per instance: its first tile (an instance's tiles are consecutive)
  int tile_samples;
  TileReduce tr;
  unsigned int* baseline_bits;
  unsigned int* inst_done;
  unsigned int* noise_counter;
  float* mean_out;
  float* baseline_norm;
  double* stats;
  int C;
  // Rollout-tail form (the fused rollout combines each instance in the CTA that finishes its last tile):
  unsigned int* inst_tiles_done;  // per instance: finished tiles of this launch (reset by the finalizing CTA)
  float* first_out;               // finish != 0: also smooth and clamp the new mean (finish_instance)
  int finish;
  // finish != 0 and host_mean != nullptr: the instance's results also go straight to these pinned host arrays
  // (device-accessible under unified addressing), so no device-to-host copy has to follow the solve
  float* host_mean;
  float* host_first;
  float* host_bn;
  double* host_stats;
  // with host_mean: the CTA that completes the launch copies the bounded-wait status word (status) here as well
  unsigned int* host_status;
  const unsigned int* status;
};

template <class Model>
struct RolloutArgs
{
  const InstDesc* inst;
  const int2* tiles;  // (instance, first sample)
  int num_tiles;
  const typename Model::DynParams* dyn;
  const typename Model::CostParams* cost;
  ModelAux aux;
  const float* x0;
  const float* samples;
  const float* mean;
  float* costs;
  unsigned int* baseline_bits;  // per instance, ordered-int min
  unsigned int* tile_counter;   // [0] = next tile, [1] = finished CTAs
  unsigned int* status;         // set non-zero if a bounded wait gave up
  float dt, lambda, alpha;
  int use_likelihood;
  int max_t;  // longest horizon of the handle
  SampleShared sh;
  TileReduce tr;
  int tail;          // the fused rollout finalizes each instance after its last tile (fin below)
  FinalizeArgs fin;
  uint32_t max_polls;  // rollout mode 4: polls of a noise warp's progress word before a rollout warp gives up
  int withhold_progress;  // diagnostics: mode 4's noise warps stage their quads without publishing progress
};

// The tile epilogue (all threads of the CTA; the tile's costs are in a.costs and its minimum in tile_min).  s_w holds
// one float per sample of the tile, s_red 64 doubles.
template <int C, class Args>
__device__ __forceinline__ void tile_reduce(const Args& a, const InstDesc& d, int tile, int first, int rows,
                                            unsigned int tile_min, float* s_w, double* s_red,
                                            const float* s_u = nullptr)
{
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5;
  const double bl = (double)ordered_to_float(tile_min);
  const double linv = (double)a.tr.lambda_inv;
  double sw = 0.0, sw2 = 0.0;
  for (int k = tid; k < rows; k += nt)
  {
    const float c = __ldcg(a.costs + d.k_off + first + k);
    const float w = expf((float)(-((double)c - bl) * linv));
    s_w[k] = w;
    sw += (double)w;
    sw2 += (double)w * (double)w;
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1)
  {
    sw += __shfl_xor_sync(0xffffffffu, sw, off);
    sw2 += __shfl_xor_sync(0xffffffffu, sw2, off);
  }
  if (lane == 0)
  {
    s_red[warp] = sw;
    s_red[32 + warp] = sw2;
  }
  __syncthreads();
  const int TC = d.T * C;
  const float* u = a.samples + d.u_off + (long long)first * TC;  // written earlier in this launch or by the sampler
  float* out = a.tr.partials + a.tr.poff[tile];
  for (int j = tid; j < TC; j += nt)
  {
    float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f, a3 = 0.0f;
    int k = 0;
    if (s_u)
    {
      // the tile's controls staged in shared memory by the rollout (same values, same order of operations)
      const float* r = s_u + (size_t)j * a.tr.u_stride;
      for (; k + 4 <= rows; k += 4)
      {
        a0 = fmaf(s_w[k], r[k], a0);
        a1 = fmaf(s_w[k + 1], r[k + 1], a1);
        a2 = fmaf(s_w[k + 2], r[k + 2], a2);
        a3 = fmaf(s_w[k + 3], r[k + 3], a3);
      }
      for (; k < rows; ++k) a0 = fmaf(s_w[k], r[k], a0);
    }
    else
    {
      for (; k + 4 <= rows; k += 4)
      {
        const float v0 = __ldcg(u + (long long)k * TC + j), v1 = __ldcg(u + (long long)(k + 1) * TC + j);
        const float v2 = __ldcg(u + (long long)(k + 2) * TC + j), v3 = __ldcg(u + (long long)(k + 3) * TC + j);
        a0 = fmaf(s_w[k], v0, a0);
        a1 = fmaf(s_w[k + 1], v1, a1);
        a2 = fmaf(s_w[k + 2], v2, a2);
        a3 = fmaf(s_w[k + 3], v3, a3);
      }
      for (; k < rows; ++k) a0 = fmaf(s_w[k], __ldcg(u + (long long)k * TC + j), a0);
    }
    out[j] = (a0 + a1) + (a2 + a3);
  }
  if (tid == 0)
  {
    double t0 = 0.0, t1 = 0.0;
    for (int wi = 0; wi < (nt + 31) / 32; ++wi)
    {
      t0 += s_red[wi];
      t1 += s_red[32 + wi];
    }
    a.tr.sums[2 * tile] = t0;
    a.tr.sums[2 * tile + 1] = t1;
    a.tr.tmin[tile] = tile_min;
  }
  __syncthreads();
}

// Instance i's combine, by all threads of the calling CTA (any block size up to 1024).  s_r: one float per tile of
// the instance; s_red: 64 doubles; s_eta: one float.  Leaves the instance's baseline reset for the next launch.
__device__ __forceinline__ void finalize_instance(const FinalizeArgs& a, int i, float* s_r, double* s_red,
                                                  float* s_eta)
{
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const InstDesc d = a.inst[i];
  const int nt = (d.K + a.tile_samples - 1) / a.tile_samples;
  const int t0 = a.inst_tile0[i];
  const float b = ordered_to_float(a.baseline_bits[i]);
  const double bd = (double)b;
  const double linv = (double)a.tr.lambda_inv;
  // The tiles' rescale factors: the baseline difference in FP64, the exponential in FP32 like the weights
  // themselves; the normaliser (and the sum of squared weights) accumulate in FP64.  FP64 is slow on this part, so
  // only the warps that hold tiles run it, and one thread combines the warps.
  double eta = 0.0, w2 = 0.0;
  for (int l = tid; l < nt; l += blockDim.x)
  {
    const float r = expf((float)(-((double)ordered_to_float(a.tr.tmin[t0 + l]) - bd) * linv));
    s_r[l] = r;
    const double rd = (double)r;
    eta += rd * __ldcg(a.tr.sums + 2 * (t0 + l));
    w2 += rd * rd * __ldcg(a.tr.sums + 2 * (t0 + l) + 1);
  }
  const int busy_warps = min((nt + 31) / 32, (int)(blockDim.x >> 5));  // at most 32
  if (warp < busy_warps)
  {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1)
    {
      eta += __shfl_xor_sync(0xffffffffu, eta, off);
      w2 += __shfl_xor_sync(0xffffffffu, w2, off);
    }
    if (lane == 0)
    {
      s_red[warp] = eta;
      s_red[32 + warp] = w2;
    }
  }
  __syncthreads();
  if (tid == 0)
  {
    eta = 0.0;
    w2 = 0.0;
    for (int wi = 0; wi < busy_warps; ++wi)
    {
      eta += s_red[wi];
      w2 += s_red[32 + wi];
    }
    *s_eta = (float)eta;
  }
  __syncthreads();
  // mean[j] = sum_l r_l S_l[j] / eta in FP32 (the weighted control average itself is FP32, as in the reference)
  const float eta_f = *s_eta;
  const int TC = d.T * a.C;
  const float* p0 = a.tr.partials + a.tr.poff[t0];
  for (int j = tid; j < TC; j += blockDim.x)
  {
    float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f, a3 = 0.0f;
    int l = 0;
    for (; l + 4 <= nt; l += 4)
    {
      a0 = fmaf(s_r[l], __ldcg(p0 + (long long)l * TC + j), a0);
      a1 = fmaf(s_r[l + 1], __ldcg(p0 + (long long)(l + 1) * TC + j), a1);
      a2 = fmaf(s_r[l + 2], __ldcg(p0 + (long long)(l + 2) * TC + j), a2);
      a3 = fmaf(s_r[l + 3], __ldcg(p0 + (long long)(l + 3) * TC + j), a3);
    }
    for (; l < nt; ++l) a0 = fmaf(s_r[l], __ldcg(p0 + (long long)l * TC + j), a0);
    a.mean_out[d.t_off + j] = ((a0 + a1) + (a2 + a3)) / eta_f;
  }
  if (tid == 0)
  {
    a.baseline_norm[2 * i] = b;
    a.baseline_norm[2 * i + 1] = (float)eta;
    a.stats[3 * i] = eta;
    a.stats[3 * i + 1] = w2;
    a.stats[3 * i + 2] = bd;
    a.baseline_bits[i] = kOrderedPosInf;
  }
}

// Controller::smoothControlTrajectoryHelper (controller.cuh:573-607) and the final constraint pass, on the device,
// by all threads of the CTA that has combined instance i: the new mean is smoothed in place with the 5-tap
// Savitzky-Golay filter [-3, 12, 17, 12, -3] / 35 (edges replicated, the first control kept; each tap product rounded
// to FP32 and added in tap order), then clamped, and the unclamped first control is recorded (the slide history).
// buf holds (T + 4) * C floats.
template <int C>
__device__ __forceinline__ void finish_instance(const InstDesc& d, int i, float* mean, float* first_out,
                                                const SampleShared& sh, float* buf)
{
  const int tid = threadIdx.x;
  const int T = d.T;
  float* u = mean + d.t_off;
  for (int e = tid; e < (T + 4) * C; e += blockDim.x)
  {
    const int tt = e / C, c = e - tt * C;
    const int src = min(max(tt - 2, 0), T - 1);
    buf[e] = u[src * C + c];
  }
  __syncthreads();
  const float coef[5] = { -3.0f / 35.0f, 12.0f / 35.0f, 17.0f / 35.0f, 12.0f / 35.0f, -3.0f / 35.0f };
  for (int e = tid; e < T * C; e += blockDim.x)
  {
    const int t = e / C, c = e - t * C;
    float v;
    if (t == 0)
    {
      v = buf[2 * C + c];
      first_out[i * C + c] = v;
    }
    else
    {
      float acc = 0.0f;
#pragma unroll
      for (int j = 0; j < 5; ++j) acc += coef[j] * buf[(t + j) * C + c];
      v = acc;
    }
    if (sh.final_clamp == 1)
      u[e] = c == 1 ? fminf(fmaxf(v, sh.lower[1]), sh.upper[1]) : v;
    else
      u[e] = enforce_constraint(v, sh.lower[c], sh.upper[c], sh.deadband[c], sh.zero[c]);
  }
}

// The end of a solve for instance i, by all threads of the CTA that has just written the instance's new mean: the
// smoothing and final clamp (finish_instance) and, with host pointers, the results copied straight to the pinned
// host block (device-accessible under unified addressing), so no device-to-host copy has to follow the solve.
template <int C>
__device__ __forceinline__ void finish_and_publish(const InstDesc& d, int i, float* mean, float* first_out,
                                                   const float* bn, const double* stats, const SampleShared& sh,
                                                   float* buf, float* host_mean, float* host_first, float* host_bn,
                                                   double* host_stats)
{
  const int tid = threadIdx.x;
  __syncthreads();  // the new mean is written
  finish_instance<C>(d, i, mean, first_out, sh, buf);
  if (host_mean)
  {
    __syncthreads();  // the smoothed mean and the first controls are written
    for (int e = tid; e < d.T * C; e += blockDim.x) host_mean[d.t_off + e] = mean[d.t_off + e];
    if (tid < C) host_first[i * C + tid] = first_out[i * C + tid];
    if (tid == 0)
    {
      host_bn[2 * i] = bn[2 * i];
      host_bn[2 * i + 1] = bn[2 * i + 1];
      for (int j = 0; j < 3; ++j) host_stats[3 * i + j] = stats[3 * i + j];
    }
  }
  __syncthreads();
}

// The running cost of step t (state cost on the stepped output y, control cost, likelihood-ratio term), in the
// reference's arithmetic (mppi_common.cu:105-144).  kLik: the likelihood-ratio term is on (control_cost_coeff != 0);
// a template flag, so a step has no branch.
template <class Model, bool kLik, class Args, class Ar = ExactArith>
__device__ __forceinline__ float step_cost(const Args& a, const InstDesc& d, const typename Model::CostParams& cp,
                                           int k, const float* u, int t, const float* y, Ar&& ar = Ar{})
{
  constexpr int C = Model::CONTROL_DIM;
  float c = Model::computeStateCost(cp, a.aux, y, t, ar) + Model::computeControlCost(cp, u, t);
  if constexpr (kLik)
  {
    // GaussianDistributionImpl::computeLikelihoodRatioCost (gaussian.cu:490-574)
    const bool zero_mean = (float)k >= (1.0f - a.sh.pure_pct) * (float)d.K;
    float lc = 0.0f;
    // coeff_i m_i (m_i - 2 u_i) / sd_i^2 added in control order; two controls per paired instruction (2 u formed as
    // u + u, exact like 2.0f * u)
#pragma unroll
    for (int i = 0; i + 1 < C; i += 2)
    {
      const float* mr = a.mean + d.t_off + t * C + i;
      const f32x2 m = zero_mean ? f32x2{ 0.0f, 0.0f } : f32x2{ mr[0], mr[1] };
      const f32x2 sd = { a.sh.std_dev[i], a.sh.std_dev[i + 1] };
      const f32x2 num = mul2(mul2({ a.sh.control_cost_coeff[i], a.sh.control_cost_coeff[i + 1] }, m),
                             sub2(m, add2({ u[i], u[i + 1] }, { u[i], u[i + 1] })));
      const f32x2 q = ar.div2(num, mul2(sd, sd));
      lc += q.x;
      lc += q.y;
    }
    if constexpr (C % 2 == 1)
    {
      const float m = zero_mean ? 0.0f : a.mean[d.t_off + t * C + C - 1];
      const float sd = a.sh.std_dev[C - 1];
      lc += ar.div(a.sh.control_cost_coeff[C - 1] * m * (m - 2.0f * u[C - 1]), sd * sd);
    }
    c += 0.5f * a.lambda * (1.0f - a.alpha) * lc;
  }
  return c;
}

// A step's running cost is evaluated one step late, after the next step's dynamics: both depend only on the same
// state, so the scheduler overlaps the cost's loads (costmap texels) and arithmetic with the dynamics chain.  The
// costs still enter the running sum in step order.  `t < 0`: nothing pending.
template <class Model>
struct PendingCost
{
  float y[Model::STATE_DIM];
  float u[Model::CONTROL_DIM];
  int t;
  __device__ __forceinline__ void reset(const float* x0)
  {
#pragma unroll
    for (int i = 0; i < Model::STATE_DIM; ++i) y[i] = x0[i];
#pragma unroll
    for (int i = 0; i < Model::CONTROL_DIM; ++i) u[i] = 0.0f;
    t = -1;
  }
};

// One step t of sample k under control u: Euler step, then the running cost of the previous step.
template <class Model, bool kLik, class Args, class Ar>
__device__ __forceinline__ void rollout_step(const Args& a, const InstDesc& d,
                                             const typename Model::DynParams& dp,
                                             const typename Model::CostParams& cp, int k, const float* u, int t,
                                             float* x, float& running, PendingCost<Model>& pc, Ar& ar)
{
  constexpr int S = Model::STATE_DIM;
  constexpr int C = Model::CONTROL_DIM;
  float xn[S];
  euler_step<Model>(dp, x, u, xn, a.dt, ar);
  const float c = step_cost<Model, kLik>(a, d, cp, k, pc.u, pc.t < 0 ? 0 : pc.t, pc.y, ar);
  running += pc.t >= 0 ? c : 0.0f;  // adding +0 leaves the (non-negative zero) initial sum unchanged
#pragma unroll
  for (int i = 0; i < S; ++i) pc.y[i] = x[i] = xn[i];
#pragma unroll
  for (int i = 0; i < C; ++i) pc.u[i] = u[i];
  pc.t = t;
}

// Adds the last pending step cost.
template <class Model, bool kLik, class Args>
__device__ __forceinline__ void rollout_flush(const Args& a, const InstDesc& d, const typename Model::CostParams& cp,
                                              int k, float& running, PendingCost<Model>& pc)
{
  if (pc.t >= 0) running += step_cost<Model, kLik>(a, d, cp, k, pc.u, pc.t, pc.y);
  pc.t = -1;
}

// Runs `steps(ar)`, a few rollout steps written against an arithmetic policy, with FastArith; if any of their
// divisions or angle wraps left the range where FastArith equals the IEEE result, restores the rollout state and runs
// the same steps again with ExactArith, so the outcome is bit-identical to ExactArith either way.  `steps` changes
// nothing but the state passed here, apart from stores that the replay repeats at the same addresses.  A run of four
// steps gives the scheduler one branch-free basic block to interleave the dynamics chain with the pending costs.
template <class Model, class Steps>
__device__ __forceinline__ void speculate_steps(float* x, float& running, PendingCost<Model>& pc, const Steps& steps)
{
  constexpr int S = Model::STATE_DIM;
  float xs[S];
#pragma unroll
  for (int i = 0; i < S; ++i) xs[i] = x[i];
  const float rs = running;
  const PendingCost<Model> ps = pc;
  FastArith fa;
  steps(fa);
  if (__builtin_expect(!fa.ok, 0))  // rare: keep the replay out of the hot path
  {
#pragma unroll
    for (int i = 0; i < S; ++i) x[i] = xs[i];
    running = rs;
    pc = ps;
    ExactArith ea;
    steps(ea);
  }
}

// The same for steps that change only the state x (dynamics without costs).
template <int S, class Steps>
__device__ __forceinline__ void speculate_dynamics(float* x, const Steps& steps)
{
  float xs[S];
#pragma unroll
  for (int i = 0; i < S; ++i) xs[i] = x[i];
  FastArith fa;
  steps(fa);
  if (__builtin_expect(!fa.ok, 0))  // rare: keep the replay out of the hot path
  {
#pragma unroll
    for (int i = 0; i < S; ++i) x[i] = xs[i];
    ExactArith ea;
    steps(ea);
  }
}

// The same for a pure function of the arguments (a step cost).
template <class F>
__device__ __forceinline__ float speculate_value(const F& f)
{
  FastArith fa;
  const float v = f(fa);
  if (__builtin_expect(fa.ok, 1)) return v;
  ExactArith ea;
  return f(ea);
}

// Control quads (float4 of the sample row) per speculated run: four steps.  Shorter runs pay the state save and the
// branch more often; much longer unrolled runs measured slower (instruction-cache pressure of the unrolled replay).
template <int C>
constexpr int kSpecQuads = C < 4 ? C : 1;

// Steps t0 .. t0+nt-1 of sample k from its staged control row.
template <class Model, bool kLik>
__device__ __forceinline__ void rollout_chunk(const RolloutArgs<Model>& a, const InstDesc& d,
                                              const typename Model::DynParams& dp,
                                              const typename Model::CostParams& cp, int k, const float* urow, int t0,
                                              int nt, float* x, float& running, PendingCost<Model>& pc)
{
  constexpr int C = Model::CONTROL_DIM;
  int tt = 0;
  if constexpr (4 % C == 0)
  {
    // 16-byte shared-memory reads; Q quads = four steps per speculated run
    constexpr int Q = kSpecQuads<C>;
    constexpr int NST = 4 * Q / C;
    for (; tt + NST <= nt; tt += NST)
    {
      float uu[4 * Q];
#pragma unroll
      for (int p = 0; p < Q; ++p)
      {
        const float4 v = *reinterpret_cast<const float4*>(urow + tt * C + 4 * p);
        uu[4 * p] = v.x;
        uu[4 * p + 1] = v.y;
        uu[4 * p + 2] = v.z;
        uu[4 * p + 3] = v.w;
      }
      speculate_steps<Model>(x, running, pc, [&](auto& ar) {
#pragma unroll
        for (int g = 0; g < NST; ++g)
          rollout_step<Model, kLik>(a, d, dp, cp, k, uu + g * C, t0 + tt + g, x, running, pc, ar);
      });
    }
  }
  for (; tt < nt; ++tt)
  {
    float u[C];
#pragma unroll
    for (int c = 0; c < C; ++c) u[c] = urow[tt * C + c];
    speculate_steps<Model>(x, running, pc, [&](auto& ar) {
      rollout_step<Model, kLik>(a, d, dp, cp, k, u, t0 + tt, x, running, pc, ar);
    });
  }
}

template <class Model, int NS, int TCH>
__global__ void __launch_bounds__(NS) rollout_kernel(const __grid_constant__ RolloutArgs<Model> a)
{
  constexpr int S = Model::STATE_DIM;
  constexpr int C = Model::CONTROL_DIM;
  constexpr int ROW = TCH * C + 4;  // floats per staged sample row
  static_assert((TCH * C) % 4 == 0, "time chunk must hold whole float4s");
  __shared__ __align__(16) float stage[NS * ROW];
  __shared__ int s_tile;
  __shared__ unsigned int s_min;
  __shared__ float s_tw[NS];  // tile_reduce: the tile's weights
  __shared__ double s_tred[64];

  const int tid = threadIdx.x;
  for (;;)
  {
    if (tid == 0)
    {
      s_tile = (int)atomicAdd(&a.tile_counter[0], 1u);
      s_min = kOrderedPosInf;
    }
    __syncthreads();
    const int tile = s_tile;
    if (tile >= a.num_tiles) break;
    const int2 w = a.tiles[tile];
    const InstDesc d = a.inst[w.x];
    const int k = w.y + tid;
    const bool active = k < d.K;
    const int rows = min(NS, d.K - w.y);
    const typename Model::DynParams dp = a.dyn[w.x];
    const typename Model::CostParams cp = a.cost[w.x];  // by value: loop-invariant for the whole tile

    float x[S];
#pragma unroll
    for (int i = 0; i < S; ++i) x[i] = a.x0[d.x_off + i];
    float running = 0.0f;
    PendingCost<Model> pc;
    pc.reset(x);
    const bool aligned = ((d.T * C) & 3) == 0;
    const float* base = a.samples + d.u_off + (long long)w.y * d.T * C;

    for (int t0 = 0; t0 < d.T; t0 += TCH)
    {
      const int nt = min(TCH, d.T - t0);
      // ---- stage controls [rows][t0, t0+nt) into shared memory
      if (aligned && (nt * C) % 4 == 0)
      {
        const int q_per_row = nt * C / 4;
        const int total_q = rows * q_per_row;
        for (int i = tid; i < total_q; i += NS)
        {
          const int r = i / q_per_row;
          const int qq = i - r * q_per_row;
          const float4 v = __ldg(reinterpret_cast<const float4*>(base + (long long)r * d.T * C + t0 * C) + qq);
          *reinterpret_cast<float4*>(&stage[r * ROW + 4 * qq]) = v;
        }
      }
      else
      {
        const int per_row = nt * C;
        const int total = rows * per_row;
        for (int i = tid; i < total; i += NS)
        {
          const int r = i / per_row;
          const int j = i - r * per_row;
          stage[r * ROW + j] = __ldg(base + (long long)r * d.T * C + t0 * C + j);
        }
      }
      __syncthreads();
      if (active)
      {
        if (a.use_likelihood)
          rollout_chunk<Model, true>(a, d, dp, cp, k, &stage[tid * ROW], t0, nt, x, running, pc);
        else
          rollout_chunk<Model, false>(a, d, dp, cp, k, &stage[tid * ROW], t0, nt, x, running, pc);
      }
      __syncthreads();
    }
    unsigned int o = kOrderedPosInf;
    if (active)
    {
      if (a.use_likelihood)
        rollout_flush<Model, true>(a, d, cp, k, running, pc);
      else
        rollout_flush<Model, false>(a, d, cp, k, running, pc);
      const float tf = (float)d.T;
      const float cost = running / tf + Model::terminalCost(cp, a.aux, x) / tf;
      a.costs[d.k_off + k] = cost;
      o = float_to_ordered(cost);
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) o = min(o, __shfl_xor_sync(0xffffffffu, o, off));
    if ((tid & 31) == 0) atomicMin(&s_min, o);
    __syncthreads();
    if (tid == 0) atomicMin(&a.baseline_bits[w.x], s_min);
    if (a.tr.partials) tile_reduce<C>(a, d, tile, w.y, rows, s_min, s_tw, s_tred);
  }
  // last CTA out resets the work counters for the next launch
  if (tid == 0)
  {
    __threadfence();
    const unsigned int done = atomicAdd(&a.tile_counter[1], 1u);
    if (done == gridDim.x - 1)
    {
      a.tile_counter[0] = 0u;
      a.tile_counter[1] = 0u;
      __threadfence();
    }
  }
}

// Gaussian sampling fused into the rollout (every instance has T*C % 4 == 0 and C divides 4).  Thread k draws the
// Philox quads of its own sample row (the same quad index, stream and counter as gaussian_sample_kernel, so the
// samples are bit-identical to the two-kernel path), applies setGaussianControls and the constraints, stores each
// quad once with a 16-byte store (the update kernel reads them) and integrates the 4/C steps it holds.  Nothing is
// read back from HBM; the next quad's Philox rounds are independent of the dynamics chain, so they fill its latency.
struct FusedNoise
{
  float* samples;         // written: the constrained control samples
  const float* injected;  // standard-normal noise in samples layout, or nullptr for Philox
  const unsigned int* noise_counter;
  uint32_t seed_lo, seed_hi;
  int stride;
  float decay_pow;
};

// setGaussianControls + constraints for the quad of elements rem0 .. rem0+3 of sample k's row (rem = t*C + c), as
// gaussian_sample_kernel computes them.
template <int C>
__device__ __forceinline__ float4 gaussian_quad(const SampleShared& sh, float4 mq, float decay_pow, int stride, int k,
                                                float pure_threshold, int rem0, float4 z)
{
  const float zz[4] = { z.x, z.y, z.z, z.w };
  const float mm[4] = { mq.x, mq.y, mq.z, mq.w };
  float out[4];
#pragma unroll
  for (int j = 0; j < 4; ++j)
  {
    const int rem = rem0 + j;
    const int t = rem / C, c = rem - t * C;
    const float m = mm[j];
    const float sd = decay_pow * sh.std_dev[c];
    float u;
    if (k == 0 || t < stride)
      u = m;
    else if ((float)k >= pure_threshold)
      u = sd * zz[j];
    else
      u = fmaf(sd, zz[j], m);
    out[j] = enforce_constraint(u, sh.lower[c], sh.upper[c], sh.deadband[c], sh.zero[c]);
  }
  return make_float4(out[0], out[1], out[2], out[3]);
}

// The same with the quad's nominal controls read from the instance's mean row (rem0 a multiple of 4, the row
// 16-byte aligned).
template <int C>
__device__ __forceinline__ float4 gaussian_quad(const SampleShared& sh, const float* mean_inst, float decay_pow,
                                                int stride, int k, float pure_threshold, int rem0, float4 z)
{
  return gaussian_quad<C>(sh, __ldg(reinterpret_cast<const float4*>(mean_inst + rem0)), decay_pow, stride, k,
                          pure_threshold, rem0, z);
}

// The four normals of Philox quad q of the instance's noise stream (or the injected ones).
__device__ __forceinline__ float4 fused_noise(const FusedNoise& f, const InstDesc& d, uint32_t counter, long long q)
{
  return f.injected ? *reinterpret_cast<const float4*>(f.injected + d.noise_off + 4 * q)
                    : philox_normal4((uint64_t)q, (uint32_t)d.noise_inst, counter, f.seed_lo, f.seed_hi);
}

// Re-roll of chosen samples for visualisation (VanillaMPPIController::calculateSampledStateTrajectories ->
// visualizeKernel, mppi_common.cu:371-533): one thread per chosen sample of one instance runs the sample's stored,
// constrained controls through the dynamics again and records the stepped state and the running cost of every step,
// in the rollout's arithmetic, so the sample's cost is (the step costs summed in step order) / T + terminal / T.
template <class Model>
__global__ void __launch_bounds__(128) sampled_trajectories_kernel(const __grid_constant__ RolloutArgs<Model> a,
                                                                   int inst, const int* idx, int n, float* states,
                                                                   float* step_costs, float* terminal)
{
  constexpr int S = Model::STATE_DIM;
  constexpr int C = Model::CONTROL_DIM;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const InstDesc d = a.inst[inst];
  const int k = idx[j];
  const typename Model::DynParams dp = a.dyn[inst];
  const typename Model::CostParams cp = a.cost[inst];
  float x[S];
#pragma unroll
  for (int i = 0; i < S; ++i) x[i] = a.x0[d.x_off + i];
  const float* us = a.samples + d.u_off + (long long)k * d.T * C;
  float* ys = states + (long long)j * d.T * S;
  for (int t = 0; t < d.T; ++t)
  {
    float u[C], xn[S];
#pragma unroll
    for (int c = 0; c < C; ++c) u[c] = us[t * C + c];
    euler_step<Model>(dp, x, u, xn, a.dt);
#pragma unroll
    for (int i = 0; i < S; ++i) ys[(long long)t * S + i] = x[i] = xn[i];
    step_costs[(long long)j * d.T + t] =
        a.use_likelihood ? step_cost<Model, true>(a, d, cp, k, u, t, x) : step_cost<Model, false>(a, d, cp, k, u, t, x);
  }
  terminal[j] = Model::terminalCost(cp, a.aux, x);
}

// Polls of a noise warp's progress word before a rollout warp gives up (each poll is one shared-memory read).
constexpr uint32_t kMaxProgressPolls = 1u << 22;
// Quads a noise warp publishes at a time.
constexpr int kNoiseChunkQuads = 4;

// The fused rollout.  kNoiseWarps: the CTA holds 2 * NS threads; threads NS .. 2NS-1 draw the tile's Gaussian
// control quads into the shared-memory stage (and the samples buffer) ahead of the rollout, publishing their progress
// per warp, while threads 0 .. NS-1 run only the dynamics and the costs, reading their controls from the stage.  The
// arithmetic of every sample is the same as with one thread per sample; the noise generation just leaves the
// rollout's dependent chain for other schedulers, which pays when the grid has fewer warps than the GPU has
// schedulers (small K).  Needs the stage (a.tr.u_stride > 0).
template <class Model, int NS, bool kNoiseWarps = false>
__global__ void __launch_bounds__(kNoiseWarps ? 2 * NS : NS)
    rollout_fused_kernel(const __grid_constant__ RolloutArgs<Model> a, const __grid_constant__ FusedNoise f)
{
  constexpr int S = Model::STATE_DIM;
  constexpr int C = Model::CONTROL_DIM;
  static_assert(4 % C == 0, "a quad must hold whole steps");
  static_assert((NS & (NS - 1)) == 0 && NS >= 32, "tile sizes are powers of two of at least a warp");
  constexpr int G = 4 / C;
  __shared__ int s_tile;
  __shared__ unsigned int s_min;
  __shared__ float s_tw[NS];  // tile_reduce: the tile's weights
  __shared__ double s_tred[64];
  // a.tr.u_stride > 0: the tile's controls, element-major; after the tile reduction the finalizing CTA reuses it
  extern __shared__ float s_u[];
  __shared__ int s_last;
  __shared__ float s_eta;
  __shared__ int s_prog[kNoiseWarps ? NS / 32 : 1];  // quads staged so far, per noise warp
  const int tid = threadIdx.x;
  const bool noise_warp = kNoiseWarps && tid >= NS;
  const int slot = tid & (NS - 1);  // the sample slot of this thread within the tile
  const uint32_t counter = f.noise_counter ? *f.noise_counter : 0u;
  for (;;)
  {
    if (tid == 0)
    {
      s_tile = (int)atomicAdd(&a.tile_counter[0], 1u);
      s_min = kOrderedPosInf;
    }
    if (kNoiseWarps && tid < NS / 32) s_prog[tid] = 0;
    __syncthreads();
    const int tile = s_tile;
    if (tile >= a.num_tiles) break;
    const int2 w = a.tiles[tile];
    const InstDesc d = a.inst[w.x];
    const int k = w.y + slot;
    const bool active = k < d.K;
    const typename Model::DynParams dp = a.dyn[w.x];
    const typename Model::CostParams cp = a.cost[w.x];
    float x[S];
#pragma unroll
    for (int i = 0; i < S; ++i) x[i] = a.x0[d.x_off + i];
    float running = 0.0f;
    PendingCost<Model> pc;
    pc.reset(x);
    if (noise_warp)
    {
      // draw the tile's quads in order into the stage and the samples buffer; publish after each chunk (the whole
      // warp takes part, active or not, so the progress word always advances)
      const int nq = d.T * C / 4;
      const long long q0 = (long long)k * nq;
      const float pure_threshold = (1.0f - a.sh.pure_pct) * (float)d.K;
      float* dst = f.samples + d.u_off + 4 * q0;
      const float4* mrow = reinterpret_cast<const float4*>(a.mean + d.t_off);
      const int us = a.tr.u_stride;
      volatile int* prog = s_prog + ((tid - NS) >> 5);
      for (int c0 = 0; c0 < nq; c0 += kNoiseChunkQuads)
      {
        const int c1 = min(c0 + kNoiseChunkQuads, nq);
        if (active)
          for (int qi = c0; qi < c1; ++qi)
          {
            const float4 o = gaussian_quad<C>(a.sh, __ldg(mrow + qi), f.decay_pow, f.stride, k, pure_threshold,
                                              4 * qi, fused_noise(f, d, counter, q0 + qi));
            *reinterpret_cast<float4*>(dst + 4 * qi) = o;
            float* col = s_u + (size_t)(4 * qi) * us + slot;
            col[0] = o.x;
            col[us] = o.y;
            col[2 * us] = o.z;
            col[3 * us] = o.w;
          }
        __syncwarp();
        if ((tid & 31) == 0 && !a.withhold_progress)
        {
          __threadfence_block();
          *prog = c1;
        }
      }
    }
    else if (kNoiseWarps && active)
    {
      // the rollout warps: controls from the stage once the paired noise warp has published them
      const int nq = d.T * C / 4;
      const int us = a.tr.u_stride;
      volatile int* prog = s_prog + (tid >> 5);
      bool waited_out = false;
      auto run = [&](auto lik) {
        auto quads = [&](int qi, auto q_const) {
          constexpr int Q = decltype(q_const)::value;
          if (*prog < qi + Q)
          {
            uint32_t i = 0;
            while (*prog < qi + Q && ++i < a.max_polls)
            {
            }
            waited_out |= i >= a.max_polls;
          }
          __threadfence_block();
          float out[4 * Q];
#pragma unroll
          for (int e = 0; e < 4 * Q; ++e) out[e] = s_u[(size_t)(4 * qi + e) * us + slot];
          speculate_steps<Model>(x, running, pc, [&](auto& ar) {
#pragma unroll
            for (int g = 0; g < G * Q; ++g)
              rollout_step<Model, decltype(lik)::value>(a, d, dp, cp, k, out + g * C, qi * G + g, x, running, pc, ar);
          });
        };
        int qi = 0;
        for (; qi + kSpecQuads<C> <= nq; qi += kSpecQuads<C>) quads(qi, std::integral_constant<int, kSpecQuads<C>>{});
        for (; qi < nq; ++qi) quads(qi, std::integral_constant<int, 1>{});
      };
      if (a.use_likelihood)
        run(std::true_type{});
      else
        run(std::false_type{});
      if (waited_out) atomicOr(a.status, 1u);
    }
    else if (active)
    {
      const int nq = d.T * C / 4;
      const long long q0 = (long long)k * nq;
      const float pure_threshold = (1.0f - a.sh.pure_pct) * (float)d.K;
      float* dst = f.samples + d.u_off + 4 * q0;
      const float4* mrow = reinterpret_cast<const float4*>(a.mean + d.t_off);
      const int us = a.tr.partials ? a.tr.u_stride : 0;
      auto run = [&](auto lik) {
        float4 zn = fused_noise(f, d, counter, q0);
        float4 mn = __ldg(mrow);
        // Q quads (Q * G steps) per speculated run
        auto quads = [&](int qi, auto q_const) {
          constexpr int Q = decltype(q_const)::value;
          float out[4 * Q];
#pragma unroll
          for (int p = 0; p < Q; ++p)
          {
            const float4 z = zn, m = mn;
            // the next quad's normals and nominal controls (the last quad reloads its own: no branch in the loop)
            const int qn = min(qi + p + 1, nq - 1);
            zn = fused_noise(f, d, counter, q0 + qn);
            mn = __ldg(mrow + qn);
            const float4 o = gaussian_quad<C>(a.sh, m, f.decay_pow, f.stride, k, pure_threshold, 4 * (qi + p), z);
            *reinterpret_cast<float4*>(dst + 4 * (qi + p)) = o;
            if (us)
            {
              float* col = s_u + (size_t)(4 * (qi + p)) * us + tid;
              col[0] = o.x;
              col[us] = o.y;
              col[2 * us] = o.z;
              col[3 * us] = o.w;
            }
            out[4 * p] = o.x;
            out[4 * p + 1] = o.y;
            out[4 * p + 2] = o.z;
            out[4 * p + 3] = o.w;
          }
          speculate_steps<Model>(x, running, pc, [&](auto& ar) {
#pragma unroll
            for (int g = 0; g < G * Q; ++g)
              rollout_step<Model, decltype(lik)::value>(a, d, dp, cp, k, out + g * C, qi * G + g, x, running, pc, ar);
          });
        };
        int qi = 0;
        for (; qi + kSpecQuads<C> <= nq; qi += kSpecQuads<C>) quads(qi, std::integral_constant<int, kSpecQuads<C>>{});
        for (; qi < nq; ++qi) quads(qi, std::integral_constant<int, 1>{});
      };
      if (a.use_likelihood)
        run(std::true_type{});
      else
        run(std::false_type{});
    }
    unsigned int o = kOrderedPosInf;
    if (active && !noise_warp)
    {
      if (a.use_likelihood)
        rollout_flush<Model, true>(a, d, cp, k, running, pc);
      else
        rollout_flush<Model, false>(a, d, cp, k, running, pc);
      const float tf = (float)d.T;
      const float cost = running / tf + Model::terminalCost(cp, a.aux, x) / tf;
      a.costs[d.k_off + k] = cost;
      o = float_to_ordered(cost);
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) o = min(o, __shfl_xor_sync(0xffffffffu, o, off));
    if ((tid & 31) == 0) atomicMin(&s_min, o);
    __syncthreads();
    if (tid == 0) atomicMin(&a.baseline_bits[w.x], s_min);
    if (a.tr.partials)
      tile_reduce<C>(a, d, tile, w.y, min(NS, d.K - w.y), s_min, s_tw, s_tred, a.tr.u_stride ? s_u : nullptr);
    if (a.tail)
    {
      // the CTA that finishes an instance's last tile combines the instance (threadfence reduction)
      __threadfence();  // this thread's partial sums before the tile counts as done
      __syncthreads();
      if (tid == 0)
        s_last = atomicAdd(&a.fin.inst_tiles_done[w.x], 1u) == (unsigned int)((d.K + NS - 1) / NS - 1);
      __syncthreads();
      if (s_last)
      {
        __threadfence();
        finalize_instance(a.fin, w.x, s_u, s_tred, &s_eta);
        if (tid == 0) a.fin.inst_tiles_done[w.x] = 0u;
        if (a.fin.finish)
          finish_and_publish<C>(d, w.x, a.fin.mean_out, a.fin.first_out, a.fin.baseline_norm, a.fin.stats, a.sh, s_u,
                                a.fin.host_mean, a.fin.host_first, a.fin.host_bn, a.fin.host_stats);
        __syncthreads();
      }
    }
  }
  if (tid == 0)
  {
    __threadfence();
    const unsigned int done = atomicAdd(&a.tile_counter[1], 1u);
    if (done == gridDim.x - 1)
    {
      a.tile_counter[0] = 0u;
      a.tile_counter[1] = 0u;
      // every CTA has read this launch's noise counter: advance it for the next launch
      if (a.tail && a.fin.noise_counter) *a.fin.noise_counter += 1u;
      // every CTA's give-up flag is set by now (each sets it before its own arrival above)
      if (a.tail && a.fin.host_status) *a.fin.host_status = *reinterpret_cast<volatile unsigned int*>(a.status);
      __threadfence();
    }
  }
}

// Cooperative rollout for problems too small to fill the GPU with one thread per sample (rollout mode 2): four
// lanes per sample.  All four integrate the dynamics chain (the same values, one issue per step), while the work
// off the chain is dealt out: lane j draws and rewrites Philox quad 4i + j of its row (one quad per four), keeps the
// states its quad's steps produce, and after each group of four quads evaluates the running costs of those steps;
// the costs are then gathered by shuffles and added in step order.  Samples and costs are bit-identical to
// rollout_fused_kernel's.
template <class Model, int NS>
__global__ void __launch_bounds__(4 * NS) rollout_coop_kernel(const __grid_constant__ RolloutArgs<Model> a,
                                                              const __grid_constant__ FusedNoise f)
{
  constexpr int S = Model::STATE_DIM;
  constexpr int C = Model::CONTROL_DIM;
  static_assert(4 % C == 0, "a quad must hold whole steps");
  constexpr int G = 4 / C;  // steps per quad
  constexpr int L = 4;      // lanes per sample
  __shared__ int s_tile;
  __shared__ unsigned int s_min;
  __shared__ float s_tw[NS];  // tile_reduce: the tile's weights
  __shared__ double s_tred[64];
  const int tid = threadIdx.x, j = tid & (L - 1);
  const uint32_t counter = f.noise_counter ? *f.noise_counter : 0u;
  for (;;)
  {
    if (tid == 0)
    {
      s_tile = (int)atomicAdd(&a.tile_counter[0], 1u);
      s_min = kOrderedPosInf;
    }
    __syncthreads();
    const int tile = s_tile;
    if (tile >= a.num_tiles) break;
    const int2 w = a.tiles[tile];
    const InstDesc d = a.inst[w.x];
    const int k = w.y + tid / L;
    const bool active = k < d.K;
    const typename Model::DynParams dp = a.dyn[w.x];
    const typename Model::CostParams cp = a.cost[w.x];
    float x[S];
#pragma unroll
    for (int i = 0; i < S; ++i) x[i] = a.x0[d.x_off + i];
    float running = 0.0f;
    const int nq = d.T * C / 4;  // quads per row (uniform over the CTA: one instance per tile)
    const long long q0 = (long long)(active ? k : w.y) * nq;
    const float pure_threshold = (1.0f - a.sh.pure_pct) * (float)d.K;
    float* dst = f.samples + d.u_off + 4 * q0;
    auto group = [&](auto lik) {
      for (int gi = 0; gi * L < nq; ++gi)
      {
        const int q = gi * L + j;  // this lane's quad
        float4 o = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (q < nq && active)
        {
          o = gaussian_quad<C>(a.sh, a.mean + d.t_off, f.decay_pow, f.stride, k, pure_threshold, 4 * q,
                               fused_noise(f, d, counter, q0 + q));
          *reinterpret_cast<float4*>(dst + 4 * q) = o;
        }
        const int nquads = min(L, nq - gi * L);
        float my_y[G][S];
        // quads jj .. jj+Q-1 of the group (Q * G steps) as one speculated run
        auto quads = [&](int jj, auto q_const) {
          constexpr int Q = decltype(q_const)::value;
          float v[4 * Q];
#pragma unroll
          for (int p = 0; p < Q; ++p)
          {
            v[4 * p] = __shfl_sync(0xffffffffu, o.x, jj + p, L);
            v[4 * p + 1] = __shfl_sync(0xffffffffu, o.y, jj + p, L);
            v[4 * p + 2] = __shfl_sync(0xffffffffu, o.z, jj + p, L);
            v[4 * p + 3] = __shfl_sync(0xffffffffu, o.w, jj + p, L);
          }
          speculate_dynamics<S>(x, [&](auto& ar) {
#pragma unroll
            for (int g = 0; g < G * Q; ++g)
            {
              float xn[S];
              euler_step<Model>(dp, x, v + g * C, xn, a.dt, ar);
#pragma unroll
              for (int i = 0; i < S; ++i)
              {
                if (jj + g / G == j) my_y[g % G][i] = xn[i];
                x[i] = xn[i];
              }
            }
          });
        };
        constexpr int QS = kSpecQuads<C>;
#pragma unroll
        for (int jj = 0; jj < L; jj += QS)
        {
          if (jj >= nquads) break;  // uniform over the CTA
          if (jj + QS <= nquads)
            quads(jj, std::integral_constant<int, QS>{});
          else
            quads(jj, std::integral_constant<int, 1>{});
        }
        // the running costs of this lane's steps, then all of the group's in step order
        float c[G];
        const float ov[4] = { o.x, o.y, o.z, o.w };
#pragma unroll
        for (int g = 0; g < G; ++g) c[g] = 0.0f;
        if (q < nq)  // a lane past the row's last quad has no steps (and must not read the mean past T)
        {
#pragma unroll
          for (int g = 0; g < G; ++g)
            c[g] = speculate_value([&](auto& ar) {
              return step_cost<Model, decltype(lik)::value>(a, d, cp, k, ov + g * C, q * G + g, my_y[g], ar);
            });
        }
#pragma unroll
        for (int jj = 0; jj < L; ++jj)
        {
          if (jj >= nquads) break;
#pragma unroll
          for (int g = 0; g < G; ++g) running += __shfl_sync(0xffffffffu, c[g], jj, L);
        }
      }
    };
    if (a.use_likelihood)
      group(std::true_type{});
    else
      group(std::false_type{});
    unsigned int o = kOrderedPosInf;
    if (active)
    {
      const float tf = (float)d.T;
      const float cost = running / tf + Model::terminalCost(cp, a.aux, x) / tf;
      if (j == 0) a.costs[d.k_off + k] = cost;
      o = float_to_ordered(cost);
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) o = min(o, __shfl_xor_sync(0xffffffffu, o, off));
    if ((tid & 31) == 0) atomicMin(&s_min, o);
    __syncthreads();
    if (tid == 0) atomicMin(&a.baseline_bits[w.x], s_min);
    if (a.tr.partials) tile_reduce<C>(a, d, tile, w.y, min(NS, d.K - w.y), s_min, s_tw, s_tred);
  }
  if (tid == 0)
  {
    __threadfence();
    const unsigned int done = atomicAdd(&a.tile_counter[1], 1u);
    if (done == gridDim.x - 1)
    {
      a.tile_counter[0] = 0u;
      a.tile_counter[1] = 0u;
      __threadfence();
    }
  }
}

// Split rollout for problems too small to fill the GPU with one thread per sample (the reference also keeps a split
// dynamics / cost rollout, rolloutDynamicsKernel + rolloutCostKernel, mppi_common.cu:155-369, and picks the faster by
// timing).  Kernel 1 runs only the dynamics chain (with the Gaussian sampling fused in) and stores every stepped state
// in states[instance][k][t][S] (instance offset u_off / C * S, exact because every row holds whole quads).  Kernel 2
// evaluates the running costs of all (k, t) in parallel, one warp per sample, and one lane adds them in step order,
// so the per-sample costs are bit-identical to the fused kernels'.
template <class Model, int NS>
__global__ void __launch_bounds__(NS) rollout_dyn_kernel(const __grid_constant__ RolloutArgs<Model> a,
                                                         const __grid_constant__ FusedNoise f, float* states)
{
  constexpr int S = Model::STATE_DIM;
  constexpr int C = Model::CONTROL_DIM;
  static_assert(4 % C == 0, "a quad must hold whole steps");
  constexpr int G = 4 / C;
  __shared__ int s_tile;
  const int tid = threadIdx.x;
  const uint32_t counter = f.noise_counter ? *f.noise_counter : 0u;
  for (;;)
  {
    if (tid == 0) s_tile = (int)atomicAdd(&a.tile_counter[0], 1u);
    __syncthreads();
    const int tile = s_tile;
    __syncthreads();
    if (tile >= a.num_tiles) break;
    const int2 w = a.tiles[tile];
    const InstDesc d = a.inst[w.x];
    const int k = w.y + tid;
    if (k < d.K)
    {
      const typename Model::DynParams dp = a.dyn[w.x];
      float x[S];
#pragma unroll
      for (int i = 0; i < S; ++i) x[i] = a.x0[d.x_off + i];
      const int nq = d.T * C / 4;
      const long long q0 = (long long)k * nq;
      const float pure_threshold = (1.0f - a.sh.pure_pct) * (float)d.K;
      float* dst = f.samples + d.u_off + 4 * q0;
      float* ys = states + d.u_off / C * S + (long long)k * d.T * S;
      float4 zn = fused_noise(f, d, counter, q0);
      auto quads = [&](int qi, auto q_const) {
        constexpr int Q = decltype(q_const)::value;
        float out[4 * Q];
#pragma unroll
        for (int p = 0; p < Q; ++p)
        {
          const float4 z = zn;
          zn = fused_noise(f, d, counter, q0 + min(qi + p + 1, nq - 1));
          const float4 o =
              gaussian_quad<C>(a.sh, a.mean + d.t_off, f.decay_pow, f.stride, k, pure_threshold, 4 * (qi + p), z);
          *reinterpret_cast<float4*>(dst + 4 * (qi + p)) = o;
          out[4 * p] = o.x;
          out[4 * p + 1] = o.y;
          out[4 * p + 2] = o.z;
          out[4 * p + 3] = o.w;
        }
        speculate_dynamics<S>(x, [&](auto& ar) {
#pragma unroll
          for (int g = 0; g < G * Q; ++g)
          {
            float xn[S];
            euler_step<Model>(dp, x, out + g * C, xn, a.dt, ar);
            float* yt = ys + (long long)(qi * G + g) * S;
#pragma unroll
            for (int i = 0; i < S; ++i) yt[i] = x[i] = xn[i];
          }
        });
      };
      int qi = 0;
      for (; qi + kSpecQuads<C> <= nq; qi += kSpecQuads<C>) quads(qi, std::integral_constant<int, kSpecQuads<C>>{});
      for (; qi < nq; ++qi) quads(qi, std::integral_constant<int, 1>{});
    }
  }
  if (tid == 0)
  {
    __threadfence();
    const unsigned int done = atomicAdd(&a.tile_counter[1], 1u);
    if (done == gridDim.x - 1)
    {
      a.tile_counter[0] = 0u;
      a.tile_counter[1] = 0u;
      __threadfence();
    }
  }
}

template <class Model, int NS, int WARPS>
__global__ void __launch_bounds__(WARPS * 32) rollout_cost_kernel(const __grid_constant__ RolloutArgs<Model> a,
                                                                  const float* states)
{
  constexpr int S = Model::STATE_DIM;
  constexpr int C = Model::CONTROL_DIM;
  extern __shared__ float s_cost[];  // [WARPS][T_max]
  __shared__ int s_tile;
  __shared__ unsigned int s_min;
  __shared__ float s_tw[NS];  // tile_reduce: the tile's weights
  __shared__ double s_tred[64];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (;;)
  {
    if (tid == 0)
    {
      s_tile = (int)atomicAdd(&a.tile_counter[0], 1u);
      s_min = kOrderedPosInf;
    }
    __syncthreads();
    const int tile = s_tile;
    if (tile >= a.num_tiles) break;
    const int2 w = a.tiles[tile];
    const InstDesc d = a.inst[w.x];
    const typename Model::CostParams cp = a.cost[w.x];
    float* my = s_cost + warp * a.max_t;
    unsigned int o = kOrderedPosInf;
    const int rows = min(NS, d.K - w.y);
    for (int r = warp; r < rows; r += WARPS)
    {
      const int k = w.y + r;
      const float* ys = states + d.u_off / C * S + (long long)k * d.T * S;
      const float* us = a.samples + d.u_off + (long long)k * d.T * C;
      for (int t = lane; t < d.T; t += 32)
      {
        float y[S], u[C];
#pragma unroll
        for (int i = 0; i < S; ++i) y[i] = ys[(long long)t * S + i];
#pragma unroll
        for (int i = 0; i < C; ++i) u[i] = us[t * C + i];
        my[t] = a.use_likelihood ? speculate_value([&](auto& ar) { return step_cost<Model, true>(a, d, cp, k, u, t, y, ar); })
                                 : speculate_value([&](auto& ar) { return step_cost<Model, false>(a, d, cp, k, u, t, y, ar); });
      }
      __syncwarp();
      if (lane == 0)
      {
        float running = 0.0f;
        for (int t = 0; t < d.T; ++t) running += my[t];
        float yT[S];
#pragma unroll
        for (int i = 0; i < S; ++i) yT[i] = ys[(long long)(d.T - 1) * S + i];
        const float tf = (float)d.T;
        const float cost = running / tf + Model::terminalCost(cp, a.aux, yT) / tf;
        a.costs[d.k_off + k] = cost;
        o = min(o, float_to_ordered(cost));
      }
      __syncwarp();
    }
    if (lane == 0) atomicMin(&s_min, o);
    __syncthreads();
    if (tid == 0) atomicMin(&a.baseline_bits[w.x], s_min);
    if (a.tr.partials) tile_reduce<C>(a, d, tile, w.y, rows, s_min, s_tw, s_tred);
  }
  if (tid == 0)
  {
    __threadfence();
    const unsigned int done = atomicAdd(&a.tile_counter[1], 1u);
    if (done == gridDim.x - 1)
    {
      a.tile_counter[0] = 0u;
      a.tile_counter[1] = 0u;
      __threadfence();
    }
  }
}

// Rollout with the controls staged by the bulk-copy engine.  Each thread owns one row of a double-buffered stage and
// copies its own sample's next time chunk with one cp.async.bulk while it integrates the current one; completion is
// tracked by one mbarrier per warp and buffer (32 arrivals, expect-tx bytes).  No shared data crosses threads inside
// the time loop, so warps run decoupled.  Every wait is bounded: a wait that gives up sets *status and the CTA stops.
// Requires T*C % 4 == 0 for every instance (16-byte aligned rows and chunks).
constexpr uint32_t kMaxBarrierSpins = 1u << 22;
constexpr uint32_t kMaxSleepWaits = 1u << 20;  // tries of up to ~1 us each: about a second before giving up

template <int NS, int C>
struct BulkRolloutShape
{
  static constexpr int TCH = (2 * NS * (32 * C + 4) * 4 <= 48 * 1024) ? 32 : (2 * NS * (16 * C + 4) * 4 <= 48 * 1024) ? 16 : 8;
  static constexpr int ROW = TCH * C + 4;
  static constexpr size_t SMEM = 2 * (size_t)NS * ROW * sizeof(float);
};

template <class Model, int NS, int TCH>
__global__ void __launch_bounds__(NS) rollout_kernel_bulk(const __grid_constant__ RolloutArgs<Model> a)
{
  constexpr int S = Model::STATE_DIM;
  constexpr int C = Model::CONTROL_DIM;
  constexpr int ROW = TCH * C + 4;
  constexpr int WARPS = NS / 32;
  static_assert((TCH * C) % 4 == 0 && NS % 32 == 0, "chunk rows must be whole 16-byte units");
  extern __shared__ __align__(16) float stage[];  // [2][NS][ROW]
  __shared__ __align__(8) uint64_t mbar[2][WARPS];
  __shared__ int s_tile;
  __shared__ unsigned int s_min;
  __shared__ float s_tw[NS];  // tile_reduce: the tile's weights
  __shared__ double s_tred[64];
  __shared__ int s_fail;  // CTA-uniform stop flag (read only after a barrier)

  const int tid = threadIdx.x, warp = tid >> 5;
  if (tid < 2 * WARPS) mbar_init(&mbar[tid / WARPS][tid % WARPS], 32);
  if (tid == 0) s_fail = 0;
  fence_mbarrier_init();
  __syncthreads();
  uint32_t parity = 0u;  // bit b = phase parity of buffer b
  int uses = 0;  // buffer of chunk j of the current tile is (uses + j) & 1
  bool failed = false;

  for (;;)
  {
    if (tid == 0)
    {
      s_tile = (int)atomicAdd(&a.tile_counter[0], 1u);
      s_min = kOrderedPosInf;
    }
    __syncthreads();
    const int tile = s_tile;
    if (tile >= a.num_tiles || s_fail) break;
    const int2 w = a.tiles[tile];
    const InstDesc d = a.inst[w.x];
    const int k = w.y + tid;
    const bool active = k < d.K;
    const typename Model::DynParams dp = a.dyn[w.x];
    const typename Model::CostParams cp = a.cost[w.x];  // by value: loop-invariant for the whole tile
    const float* my_row = a.samples + d.u_off + (long long)k * d.T * C;
    float* const my_stage0 = stage + tid * ROW;  // buffer b row: my_stage0 + b * NS * ROW

    float x[S];
#pragma unroll
    for (int i = 0; i < S; ++i) x[i] = a.x0[d.x_off + i];
    float running = 0.0f;
    PendingCost<Model> pc;
    pc.reset(x);
    const int nchunks = (d.T + TCH - 1) / TCH;
    auto issue = [&](int j) {
      const int b = (uses + j) & 1;
      const int t0 = j * TCH;
      const uint32_t bytes = (uint32_t)(min(TCH, d.T - t0) * C * 4);
      if (active)
      {
        fence_proxy_async_smem();  // this thread's earlier reads of its row precede the async overwrite
        mbar_arrive_expect_tx(&mbar[b][warp], bytes);
        bulk_copy_g2s(my_stage0 + b * NS * ROW, my_row + t0 * C, bytes, &mbar[b][warp]);
      }
      else
      {
        mbar_arrive(&mbar[b][warp]);
      }
    };
    issue(0);
    for (int j = 0; j < nchunks; ++j)
    {
      const int b = (uses + j) & 1;
      if (j + 1 < nchunks) issue(j + 1);
      if (!mbar_wait_bounded(&mbar[b][warp], (parity >> b) & 1u, kMaxBarrierSpins))
      {
        failed = true;
        s_fail = 1;
        atomicOr(a.status, 1u);
        // give the copy in flight one more bounded chance to land before the CTA leaves
        mbar_wait_bounded(&mbar[b][warp], (parity >> b) & 1u, kMaxBarrierSpins);
        if (j + 1 < nchunks) mbar_wait_bounded(&mbar[b ^ 1][warp], (parity >> (b ^ 1)) & 1u, kMaxBarrierSpins);
        break;
      }
      parity ^= (1u << b);
      const int t0 = j * TCH;
      if (active)
      {
        if (a.use_likelihood)
          rollout_chunk<Model, true>(a, d, dp, cp, k, my_stage0 + b * NS * ROW, t0, min(TCH, d.T - t0), x, running,
                                     pc);
        else
          rollout_chunk<Model, false>(a, d, dp, cp, k, my_stage0 + b * NS * ROW, t0, min(TCH, d.T - t0), x,
                                      running, pc);
      }
    }
    uses += nchunks;
    unsigned int o = kOrderedPosInf;
    if (active && !failed)
    {
      if (a.use_likelihood)
        rollout_flush<Model, true>(a, d, cp, k, running, pc);
      else
        rollout_flush<Model, false>(a, d, cp, k, running, pc);
      const float tf = (float)d.T;
      const float cost = running / tf + Model::terminalCost(cp, a.aux, x) / tf;
      a.costs[d.k_off + k] = cost;
      o = float_to_ordered(cost);
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) o = min(o, __shfl_xor_sync(0xffffffffu, o, off));
    if ((tid & 31) == 0) atomicMin(&s_min, o);
    __syncthreads();
    if (tid == 0) atomicMin(&a.baseline_bits[w.x], s_min);
    if (a.tr.partials) tile_reduce<C>(a, d, tile, w.y, min(NS, d.K - w.y), s_min, s_tw, s_tred);
  }
  if (tid == 0)
  {
    __threadfence();
    const unsigned int done = atomicAdd(&a.tile_counter[1], 1u);
    if (done == gridDim.x - 1)
    {
      a.tile_counter[0] = 0u;
      a.tile_counter[1] = 0u;
      __threadfence();
    }
  }
}

// ============================================================================================== 3. weights + update
// fullGPUcomputeWeights (mppi_common.cu:1067-1089) and weightedReductionKernelDeviceNorm (mppi_common.cu:746-773) in
// one multi-CTA kernel.  Each CTA owns a chunk of one instance's samples: it computes w_k = exp(-(c_k - b)/lambda)
// with the baseline subtraction in FP64, accumulates the chunk's sum of weights (FP64) and the chunk's weighted
// control sums sum_k w_k u_k[t][c] (FP32, one column per thread, coalesced rows), and writes them as partials.  The
// last CTA of an instance (arrival counter; no waiting) adds the partials in chunk order — a fixed order, so the
// result is deterministic — divides by the normaliser and writes the new nominal control, baseline and normaliser,
// then resets the instance's counters.  The last instance to finish advances the noise counter.
struct WeightsArgs
{
  const InstDesc* inst;
  const int4* chunks;  // (instance, k_begin, k_end, chunk index within instance)
  const long long* part_off;  // per chunk: offset of its partial row in `partials` (floats)
  const int* inst_chunk0;     // per instance: global index of its first chunk
  int num_chunks;
  int num_instances;
  const float* costs;
  float* weights;
  const float* samples;
  float* partials;
  double* part_w;   // per chunk: sum w, sum w^2
  unsigned int* baseline_bits;
  unsigned int* arrive;  // per instance
  unsigned int* inst_done;  // [0]
  unsigned int* noise_counter;
  float* mean_out;
  float* baseline_norm;  // per instance (baseline, normaliser)
  double* stats;         // per instance: normaliser, sum w^2, baseline
  float lambda_inv;
  int weights_given;        // 1: read w from `weights` instead of computing it from `costs`
  const float* given_norm;  // non-null: divide by given_norm[0] (a device float) instead of the summed weights
  // 0: the exponential transform; 1: TsallisTransform (mppi_common.cu:1004-1021) with tsallis_gamma / tsallis_r
  int transform;
  float tsallis_gamma, tsallis_r;
  // finish != 0 (the last iteration of a solve): the instance's last CTA also smooths and clamps the new mean
  // (finish_and_publish; dynamic shared memory of (T_max + 4) * C floats) and, with host_mean, publishes the results
  // to the pinned host block; the last instance's CTA then copies the status word to host_status
  int finish;
  float* first_out;
  SampleShared sh;
  float* host_mean;
  float* host_first;
  float* host_bn;
  double* host_stats;
  unsigned int* host_status;
  const unsigned int* status;
};

// TsallisTransform (mppi_common.cu:1004-1021), the ColoredMPPI controller's weight: with d = c - baseline,
// w = exp(log(1 - d / gamma) / (r - 1)) for d < gamma, else 0.  1 - d / gamma is formed in double from the float
// quotient and narrowed to float for the logarithm, as the reference's expression evaluates.
__device__ __forceinline__ float tsallis_weight(float c, float baseline, float gamma, float r)
{
  const float dif = c - baseline;
  return dif < gamma ? expf(logf((float)(1.0 - (double)(dif / gamma))) / (r - 1.0f)) : 0.0f;
}

template <int C>
__global__ void __launch_bounds__(256) weights_update_kernel(const __grid_constant__ WeightsArgs a)
{
  constexpr int MAXK = 256;  // samples per chunk held in shared memory
  __shared__ float s_w[MAXK];
  __shared__ double s_red[2][8];
  __shared__ unsigned int s_last;

  const int tid = threadIdx.x;
  const int4 ch = a.chunks[blockIdx.x];
  const InstDesc d = a.inst[ch.x];
  const int kb = ch.y, ke = ch.z, nk = ke - kb;
  const float b = ordered_to_float(a.baseline_bits[ch.x]);
  const double bd = (double)b;
  const double linv = (double)a.lambda_inv;

  // weights of this chunk
  double sw = 0.0, sw2 = 0.0;
  for (int i = tid; i < nk; i += blockDim.x)
  {
    float wk;
    if (a.weights_given)
    {
      wk = a.weights[d.k_off + kb + i];
    }
    else
    {
      const float c = a.costs[d.k_off + kb + i];
      if (a.transform == 1)
      {
        wk = tsallis_weight(c, b, a.tsallis_gamma, a.tsallis_r);
      }
      else
      {
        const double diff = (double)c - bd;
        wk = expf((float)(-diff * linv));
      }
      a.weights[d.k_off + kb + i] = wk;
    }
    s_w[i] = wk;
    sw += (double)wk;
    sw2 += (double)wk * (double)wk;
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1)
  {
    sw += __shfl_xor_sync(0xffffffffu, sw, off);
    sw2 += __shfl_xor_sync(0xffffffffu, sw2, off);
  }
  if ((tid & 31) == 0)
  {
    s_red[0][tid >> 5] = sw;
    s_red[1][tid >> 5] = sw2;
  }
  __syncthreads();

  // weighted control sums: thread j owns columns j, j + blockDim, ...
  const int TC = a.samples ? d.T * C : 0;
  const float* ubase = a.samples + d.u_off + (long long)kb * TC;
  float* prow = a.partials + a.part_off[blockIdx.x];
  const bool vec4 = TC > 0 && (TC & 3) == 0 && TC / 4 <= (int)blockDim.x &&
                    ((reinterpret_cast<uintptr_t>(ubase) | reinterpret_cast<uintptr_t>(prow)) & 15) == 0;
  if (vec4)
  {
    // 16-byte loads, up to eight samples in flight per thread: G groups of Q = TC / 4 threads, thread (g, j) sums float4
    // column j over samples g, g + G, ... in four interleaved accumulators, then the groups are combined in group
    // order (a fixed order, so the result does not depend on scheduling)
    __shared__ float4 s_part4[256];
    const int Q = TC >> 2;
    const int G = blockDim.x / Q;
    const int g = tid / Q, j = tid - g * Q;
    const float4* ub = reinterpret_cast<const float4*>(ubase);
    auto fma4 = [](float w, const float4& v, float4& acc) {
      acc.x = fmaf(w, v.x, acc.x);
      acc.y = fmaf(w, v.y, acc.y);
      acc.z = fmaf(w, v.z, acc.z);
      acc.w = fmaf(w, v.w, acc.w);
    };
    if (g < G)
    {
      float4 a0 = make_float4(0.f, 0.f, 0.f, 0.f), a1 = a0, a2 = a0, a3 = a0;
      int i = g;
      // eight 16-byte loads in flight per thread, then four per thread, then one
      for (; i + 7 * G < nk; i += 8 * G)
      {
        float4 v[8];
#pragma unroll
        for (int m = 0; m < 8; ++m) v[m] = __ldg(ub + (long long)(i + m * G) * Q + j);
        fma4(s_w[i], v[0], a0);
        fma4(s_w[i + G], v[1], a1);
        fma4(s_w[i + 2 * G], v[2], a2);
        fma4(s_w[i + 3 * G], v[3], a3);
        fma4(s_w[i + 4 * G], v[4], a0);
        fma4(s_w[i + 5 * G], v[5], a1);
        fma4(s_w[i + 6 * G], v[6], a2);
        fma4(s_w[i + 7 * G], v[7], a3);
      }
      for (; i + 3 * G < nk; i += 4 * G)
      {
        const float4 v0 = __ldg(ub + (long long)i * Q + j);
        const float4 v1 = __ldg(ub + (long long)(i + G) * Q + j);
        const float4 v2 = __ldg(ub + (long long)(i + 2 * G) * Q + j);
        const float4 v3 = __ldg(ub + (long long)(i + 3 * G) * Q + j);
        fma4(s_w[i], v0, a0);
        fma4(s_w[i + G], v1, a1);
        fma4(s_w[i + 2 * G], v2, a2);
        fma4(s_w[i + 3 * G], v3, a3);
      }
      for (; i < nk; i += G) fma4(s_w[i], __ldg(ub + (long long)i * Q + j), a0);
      s_part4[tid] = make_float4((a0.x + a1.x) + (a2.x + a3.x), (a0.y + a1.y) + (a2.y + a3.y),
                                 (a0.z + a1.z) + (a2.z + a3.z), (a0.w + a1.w) + (a2.w + a3.w));
    }
    __syncthreads();
    if (tid < Q)
    {
      float4 s = s_part4[tid];
      for (int gg = 1; gg < G; ++gg)
      {
        const float4 v = s_part4[gg * Q + tid];
        s = make_float4(s.x + v.x, s.y + v.y, s.z + v.z, s.w + v.w);
      }
      reinterpret_cast<float4*>(prow)[tid] = s;
    }
  }
  else if (TC > 0 && TC <= (int)blockDim.x)
  {
    // G groups of TC threads; group g sums samples g, g + G, ... of the chunk for column j, then the groups are
    // combined in group order (a fixed order, so the result does not depend on scheduling)
    __shared__ float s_part[256];
    const int G = blockDim.x / TC;
    const int g = tid / TC, j = tid - g * TC;
    float acc = 0.0f;
    if (g < G)
    {
      float acc0 = 0.0f, acc1 = 0.0f;
      int i = g;
      for (; i + G < nk; i += 2 * G)
      {
        acc0 = fmaf(s_w[i], __ldg(ubase + (long long)i * TC + j), acc0);
        acc1 = fmaf(s_w[i + G], __ldg(ubase + (long long)(i + G) * TC + j), acc1);
      }
      if (i < nk) acc0 = fmaf(s_w[i], __ldg(ubase + (long long)i * TC + j), acc0);
      acc = acc0 + acc1;
      s_part[tid] = acc;
    }
    __syncthreads();
    if (tid < TC)
    {
      float s = s_part[tid];
      for (int gg = 1; gg < G; ++gg) s += s_part[gg * TC + tid];
      prow[tid] = s;
    }
  }
  else
  {
    for (int j = tid; j < TC; j += blockDim.x)
    {
      float acc0 = 0.0f, acc1 = 0.0f, acc2 = 0.0f, acc3 = 0.0f;
      int i = 0;
      for (; i + 4 <= nk; i += 4)
      {
        acc0 = fmaf(s_w[i], __ldg(ubase + (long long)i * TC + j), acc0);
        acc1 = fmaf(s_w[i + 1], __ldg(ubase + (long long)(i + 1) * TC + j), acc1);
        acc2 = fmaf(s_w[i + 2], __ldg(ubase + (long long)(i + 2) * TC + j), acc2);
        acc3 = fmaf(s_w[i + 3], __ldg(ubase + (long long)(i + 3) * TC + j), acc3);
      }
      for (; i < nk; ++i) acc0 = fmaf(s_w[i], __ldg(ubase + (long long)i * TC + j), acc0);
      prow[j] = (acc0 + acc1) + (acc2 + acc3);
    }
  }
  if (tid == 0)
  {
    double t0 = 0.0, t1 = 0.0;
    for (int wi = 0; wi < (int)(blockDim.x >> 5); ++wi)
    {
      t0 += s_red[0][wi];
      t1 += s_red[1][wi];
    }
    a.part_w[2 * blockIdx.x] = t0;
    a.part_w[2 * blockIdx.x + 1] = t1;
  }

  // arrival: the last chunk of the instance finalises
  __threadfence();
  __syncthreads();
  if (tid == 0)
  {
    const unsigned int prev = atomicAdd(&a.arrive[ch.x], 1u);
    s_last = (prev == (unsigned int)(d.num_chunks - 1)) ? 1u : 0u;
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();

  // The instance's chunks are consecutive: partial rows TC floats apart from the first chunk's, and the (sum w,
  // sum w^2) pairs adjacent.  Loads are issued eight chunks ahead of the (in-order) additions.
  const int c0 = a.inst_chunk0[ch.x];
  const double* pw = a.part_w + 2 * c0;
  double eta = 0.0, w2 = 0.0;
#pragma unroll 8
  for (int c = 0; c < d.num_chunks; ++c)
  {
    eta += __ldcg(pw + 2 * c);
    w2 += __ldcg(pw + 2 * c + 1);
  }
  const double div = a.given_norm ? (double)a.given_norm[0] : eta;
  const float* p0 = a.partials + a.part_off[c0];
  for (int j = tid; j < TC; j += blockDim.x)
  {
    double s = 0.0;
#pragma unroll 8
    for (int c = 0; c < d.num_chunks; ++c) s += (double)__ldcg(p0 + (long long)c * TC + j);
    a.mean_out[d.t_off + j] = (float)(s / div);
  }
  if (tid == 0)
  {
    a.baseline_norm[2 * ch.x] = b;
    a.baseline_norm[2 * ch.x + 1] = (float)eta;
    a.stats[3 * ch.x] = eta;
    a.stats[3 * ch.x + 1] = w2;
    a.stats[3 * ch.x + 2] = bd;
    a.arrive[ch.x] = 0u;
    a.baseline_bits[ch.x] = kOrderedPosInf;
  }
  if (a.finish)
  {
    extern __shared__ float s_fin[];  // (T_max + 4) * C floats, launched only with finish
    finish_and_publish<C>(d, ch.x, a.mean_out, a.first_out, a.baseline_norm, a.stats, a.sh, s_fin, a.host_mean,
                          a.host_first, a.host_bn, a.host_stats);
  }
  if (tid == 0)
  {
    __threadfence();
    const unsigned int fin = atomicAdd(a.inst_done, 1u);
    if (fin == (unsigned int)(a.num_instances - 1))
    {
      // every earlier kernel of the solve has set its give-up flag by now
      if (a.host_status) *a.host_status = *reinterpret_cast<const volatile unsigned int*>(a.status);
      *a.inst_done = 0u;
      if (a.noise_counter) *a.noise_counter += 1u;
      __threadfence();
    }
  }
}

// With a.finish (the last iteration of a solve) the CTA also smooths and clamps the instance's new mean and, with
// host pointers, publishes the results to the pinned host block; the last CTA then copies the status word.  Dynamic
// shared memory: max(tiles of the largest instance, (T_max + 4) * C) floats, the tile factors and then the smoothing
// buffer.
template <int C>
__global__ void __launch_bounds__(256) tile_finalize_kernel(const __grid_constant__ FinalizeArgs a,
                                                            const __grid_constant__ SampleShared sh)
{
  extern __shared__ float s_r[];  // per tile of the instance: exp(-(b_l - b) / lambda); then the smoothing buffer
  __shared__ double s_red[64];
  __shared__ float s_eta;
  finalize_instance(a, blockIdx.x, s_r, s_red, &s_eta);
  if (a.finish)
    finish_and_publish<C>(a.inst[blockIdx.x], blockIdx.x, a.mean_out, a.first_out, a.baseline_norm, a.stats, sh, s_r,
                          a.host_mean, a.host_first, a.host_bn, a.host_stats);
  if (threadIdx.x == 0)
  {
    __threadfence();
    const unsigned int fin = atomicAdd(a.inst_done, 1u);
    if (fin == (unsigned int)(a.num_instances - 1))
    {
      *a.inst_done = 0u;
      if (a.noise_counter) *a.noise_counter += 1u;
      // every earlier kernel of the solve has set its give-up flag by now
      if (a.host_status) *a.host_status = *reinterpret_cast<const volatile unsigned int*>(a.status);
      __threadfence();
    }
  }
}

// Weights w = expf(-(c - b) / lambda) of every sample from its cost and its instance's baseline (baseline_norm), as
// weights_update_kernel computes them; used to serve mppi_get_sample_weights when the tiles did the reduction.
static __global__ void weights_from_costs_kernel(const InstDesc* inst, const float* costs, const float* baseline_norm,
                                                 float lambda_inv, float* weights)
{
  const int i = blockIdx.y;
  const InstDesc d = inst[i];
  const double bd = (double)baseline_norm[2 * i];
  const double linv = (double)lambda_inv;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < d.K; k += gridDim.x * blockDim.x)
    weights[d.k_off + k] = expf((float)(-((double)costs[d.k_off + k] - bd) * linv));
}

// Per-system minimum of costs into ordered-int slots (the baseline pass of fullGPUcomputeWeights,
// computeBaselineCost, mppi_common.cu:938-992), for the kernel-level weight-transform entry point.
static __global__ void min_cost_kernel(const float* costs, int num_rollouts, int num_systems, unsigned int* out_bits)
{
  const int sys = blockIdx.y;
  if (sys >= num_systems) return;
  unsigned int o = kOrderedPosInf;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < num_rollouts; k += gridDim.x * blockDim.x)
    o = min(o, float_to_ordered(costs[(size_t)sys * num_rollouts + k]));
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) o = min(o, __shfl_xor_sync(0xffffffffu, o, off));
  if ((threadIdx.x & 31) == 0) atomicMin(&out_bits[sys], o);
}

static __global__ void fill_u32_kernel(unsigned int* p, unsigned int v, int n)
{
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = v;
}

static __global__ void bump_counter_kernel(unsigned int* p) { *p += 1u; }

// ============================================================================================== test entry kernels
static __global__ void philox_normal_kernel(float* out, size_t n, uint32_t k0, uint32_t k1, uint64_t offset)
{
  const size_t nq = (n + 3) / 4;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < nq; q += (size_t)gridDim.x * blockDim.x)
  {
    const uint64_t blk = offset + q;
    const u32x4 r = philox4x32_10(u32x4{ (uint32_t)blk, (uint32_t)(blk >> 32), 0u, 0u }, k0, k1);
    float z[4];
    box_muller(r.x, r.y, &z[0], &z[1]);
    box_muller(r.z, r.w, &z[2], &z[3]);
    for (int j = 0; j < 4; ++j)
      if (4 * q + j < n) out[4 * q + j] = z[j];
  }
}

static __global__ void philox_raw_kernel(uint32_t* out, size_t nblocks, u32x4 ctr, uint32_t k0, uint32_t k1)
{
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < nblocks; i += (size_t)gridDim.x * blockDim.x)
  {
    u32x4 c = ctr;
    c.x += (uint32_t)i;
    const u32x4 r = philox4x32_10(c, k0, k1);
    out[4 * i] = r.x;
    out[4 * i + 1] = r.y;
    out[4 * i + 2] = r.z;
    out[4 * i + 3] = r.w;
  }
}

static __global__ void sincos_kernel(const float* x, float* s, float* c, size_t n)
{
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    sincos_f(x[i], &s[i], &c[i]);
}

}  // namespace mg
