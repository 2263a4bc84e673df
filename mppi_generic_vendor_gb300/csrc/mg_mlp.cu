// mg_mlp.cu — tensor-core evaluation of the surrogate MLP: a standalone forward entry point and the rollout kernel of
// the MLP bicycle model (the per-timestep inference over all samples is one tcgen05 GEMM chain per 128-sample tile,
// BF16 operands for BF16 weights and FP16 operands for FP8 weights, FP32 accumulation in TMEM; see mg_mlp.cuh).  The
// rollout's work items hold kMlpTiles tiles of one instance.
#include <algorithm>
#include <cmath>
#include <vector>

#include "mg_common.cuh"
#include "mg_mlp.cuh"

namespace mg
{
namespace
{
// A CTA of NT tiles holds MlpSmem::total(NT, half) bytes of shared memory and MlpSmem::tmem_cols(NT) TMEM columns:
// 27.3 KB (FP16 operands) or 27.5 KB (BF16) and 64 columns for one tile, so at most eight CTAs per SM by TMEM (512
// columns) and by shared memory; the columns of co-resident CTAs therefore fit the SM's 512, and an allocation never
// waits for another CTA.  The operand tiles are K-major without swizzling, which needs 16-byte alignment only (the
// dynamic block is 128-byte aligned).
constexpr size_t mlp_smem(bool half) { return MlpSmem::total(kMlpTiles, half); }

template <bool kHalf>
__global__ void __launch_bounds__(128) mlp_forward_kernel(const float* params, const __grid_constant__ MlpNorm nm,
                                                          const float* X, float* Y, int B, unsigned int* status)
{
  extern __shared__ __align__(128) unsigned char sm[];
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t s_tmem;
  __shared__ int s_fail;
  const int tid = threadIdx.x, warp = tid >> 5;
  if (warp == 0)
  {
    tmem_alloc(&s_tmem, MlpSmem::tmem_cols(1));
    tmem_relinquish();
  }
  if (tid == 0)
  {
    s_fail = 0;
    mbar_init(&mbar, 1);
    fence_mbarrier_init();
  }
  mlp_load_weights<kHalf>(sm, params);
  tc_fence_before_sync();
  __syncthreads();
  tc_fence_after_sync();
  const uint32_t taddr = s_tmem;
  uint32_t phase = 0;
  for (int tile = blockIdx.x; tile * 128 < B; tile += gridDim.x)
  {
    const int row = tile * 128 + tid;
    float x[1][kMlpIn], y[1][kMlpOut];
#pragma unroll
    for (int i = 0; i < kMlpIn; ++i)
      x[0][i] = row < B ? (X[(size_t)row * kMlpIn + i] - nm.in_mean[i]) * nm.in_scale[i] : 0.0f;
    if (!mlp_tile_forward<1, kHalf>(sm, taddr, &mbar, phase, &s_fail, x, y)) break;
    if (row < B)
#pragma unroll
      for (int j = 0; j < kMlpOut; ++j) Y[(size_t)row * kMlpOut + j] = y[0][j] * nm.out_std[j] + nm.out_mean[j];
  }
  tc_fence_before_sync();
  __syncthreads();
  if (tid == 0 && s_fail) atomicOr(status, 1u);
  if (warp == 0) tmem_dealloc(taddr, MlpSmem::tmem_cols(1));
}

// Plain FP32 surrogate evaluation on the CUDA cores, one thread per sample, as FNNHelper::forward evaluates it
// (fnn_helper.cu:418-495): weights in shared memory (read as broadcasts), activations in registers.  Products and
// sums are separate FP32 operations in FNNHelper's order, so the result differs from an FP32 host evaluation only by
// the last-place rounding of tanhf.
__device__ __forceinline__ void mlp_thread_forward(const float* P, const float* xin, float* y)
{
  float h1[kMlpHid];
#pragma unroll
  for (int j = 0; j < kMlpHid; ++j)
  {
    float z = P[kMlpB1 + j];
#pragma unroll
    for (int i = 0; i < kMlpIn; ++i) z = z + P[kMlpW1 + j * kMlpIn + i] * xin[i];
    h1[j] = tanhf(z);
  }
  // hidden unit j of layer 2 is folded into the outputs as soon as it is known: each output still sums its 64
  // terms in index order, starting from its bias
#pragma unroll
  for (int o = 0; o < kMlpOut; ++o) y[o] = P[kMlpB3 + o];
#pragma unroll 2
  for (int j = 0; j < kMlpHid; ++j)
  {
    float z = P[kMlpB2 + j];
    const float4* w = reinterpret_cast<const float4*>(P + kMlpW2 + j * kMlpHid);
#pragma unroll
    for (int i = 0; i < kMlpHid / 4; ++i)
    {
      const float4 v = w[i];
      z = z + v.x * h1[4 * i];
      z = z + v.y * h1[4 * i + 1];
      z = z + v.z * h1[4 * i + 2];
      z = z + v.w * h1[4 * i + 3];
    }
    const float h2 = tanhf(z);
#pragma unroll
    for (int o = 0; o < kMlpOut; ++o) y[o] = y[o] + P[kMlpW3 + o * kMlpHid + j] * h2;
  }
}

// costmap_gather_cell for the surrogate rollout: the cell index by round-to-nearest of p - 1/2 through the 1.5 * 2^23
// magic-number addition (FMA and integer pipes) instead of floorf and a float-to-int conversion, which run on the
// special-function unit that bounds the kernel.  Where p is an integer the index may be one below floor(p) with the
// fraction 1 instead of 0: the same bilinear value.
__device__ __forceinline__ Texels costmap_gather_cell_rn(const CostmapView& m, float px, float py)
{
  px = fminf(fmaxf(px, 0.0f), (float)(m.width - 1));
  py = fminf(fmaxf(py, 0.0f), (float)(m.height - 1));
  const float magic = 12582912.0f;  // 1.5 * 2^23: the sum's last mantissa bit has weight 1
  const f32x2 r = add2(sub2({ px, py }, { 0.5f, 0.5f }), { magic, magic });
  int x0 = (int)(__float_as_uint(r.x) - __float_as_uint(magic));
  int y0 = (int)(__float_as_uint(r.y) - __float_as_uint(magic));
  x0 = min(max(x0, 0), m.width - 2);
  y0 = min(max(y0, 0), m.height - 2);
  Texels t;
  t.fx = px - (float)x0;
  t.fy = py - (float)y0;
  const float* row0 = m.data + (size_t)y0 * m.width;
  const float* row1 = row0 + m.width;
  t.q00 = __ldg(row0 + x0);
  t.q01 = __ldg(row0 + x0 + 1);
  t.q10 = __ldg(row1 + x0);
  t.q11 = __ldg(row1 + x0 + 1);
  return t;
}

// Surrogate rollout: BicycleSlipModel with the (yaw, vx, vy, yaw_rate, steer) derivatives from the MLP and the
// x / y rows analytic (NeuralNetModel::computeKinematics, ar_nn_model.cu:119-124).  Persistent CTAs of 128 threads
// walk work items of 128 * kMlpTiles samples of one instance; thread i owns row i of every tile (samples
// first + i + 128 n).  The Euler step, the costmap cost and the likelihood term follow rolloutKernel
// (mppi_common.cu:105-152) exactly as the analytic rollout does.  kTensor: the network runs on the tensor cores
// (mlp_tile_forward, one MMA round trip per layer for all tiles of the CTA; kHalf: FP16 operands for FP8 weights,
// else BF16); otherwise in plain FP32 on the CUDA cores (mlp_thread_forward).
template <bool kTensor, bool kFused, bool kHalf>
__global__ void __launch_bounds__(kMlpSamplesPerCta) rollout_mlp_kernel(
    const __grid_constant__ RolloutArgs<BicycleSlipMLPModel> a, const float* mlp, const __grid_constant__ MlpNorm nm,
    const __grid_constant__ FusedNoise f)
{
  using Model = BicycleSlipMLPModel;
  // tensor cores: 128 threads, each owning row i of kMlpTiles tiles; CUDA cores: one thread per sample
  constexpr int S = Model::STATE_DIM, C = Model::CONTROL_DIM, NT = kTensor ? kMlpTiles : 1;
  static_assert(C == 2, "a fused noise quad holds two steps");
  const uint32_t counter = (kFused && f.noise_counter) ? *f.noise_counter : 0u;
  extern __shared__ __align__(128) unsigned char sm[];
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t s_tmem;
  __shared__ int s_tile;
  __shared__ unsigned int s_min;
  __shared__ int s_fail;
  const int tid = threadIdx.x, warp = tid >> 5;
  float* pf = reinterpret_cast<float*>(sm);  // FP32 path: the device parameter vector
  if constexpr (kTensor)
  {
    if (warp == 0)
    {
      tmem_alloc(&s_tmem, MlpSmem::tmem_cols(NT));
      tmem_relinquish();
    }
    if (tid == 0)
    {
      s_fail = 0;
      mbar_init(&mbar, 1);
      fence_mbarrier_init();
    }
    mlp_load_weights<kHalf>(sm, mlp);
    tc_fence_before_sync();
    __syncthreads();
    tc_fence_after_sync();
  }
  else
  {
    for (int e = tid; e < kMlpDevParams; e += blockDim.x) pf[e] = mlp[e];
    __syncthreads();
  }
  const uint32_t taddr = kTensor ? s_tmem : 0u;
  uint32_t phase = 0;
  const float* nrm = pf + kMlpInMean;  // CUDA cores: the normalisation in the shared parameter copy
  bool ok = true;
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
    int k[NT];
    bool active[NT];
    const float* urow[NT];
    float x[NT][S], running[NT];
    float2 u_next[NT];
    float4 uq[NT];  // kFused: the quad (steps t, t+1) generated for each row
    const float pure_threshold = (1.0f - a.sh.pure_pct) * (float)d.K;
    const long long nq_row = d.T * C / 4;
#pragma unroll
    for (int n = 0; n < NT; ++n)
    {
      k[n] = w.y + tid + 128 * n;  // NT == 1 on the CUDA cores, where tid spans the whole work item
      active[n] = k[n] < d.K;
      urow[n] = a.samples + d.u_off + (long long)(active[n] ? k[n] : w.y) * d.T * C;
#pragma unroll
      for (int i = 0; i < S; ++i) x[n][i] = a.x0[d.x_off + i];
      running[n] = 0.0f;
      uq[n] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      u_next[n] = (!kFused && active[n]) ? __ldg(reinterpret_cast<const float2*>(urow[n])) : make_float2(0.0f, 0.0f);
    }
    // Step t's running cost is added at step t + 1: its costmap texels are gathered before step t + 1's network
    // pass, which hides their latency, and blended after it.  The sum keeps step order.
    // The tensor-core forms are held to tolerances, so there the step's divisions by constants (the costmap's cell
    // size, the control variances) become products with host-computed reciprocals (kernel parameters): the
    // special-function unit that bounds this kernel then does no per-step division work.
    auto gather = [&](float px, float py) {
      if constexpr (kTensor)
      {
        const float ir = a.aux.map.inv_resolution;
        const f32x2 c = sub2(mul2(sub2({ px, py }, { a.aux.map.origin_x, a.aux.map.origin_y }), { ir, ir }),
                             { 0.5f, 0.5f });
        return costmap_gather_cell_rn(a.aux.map, c.x, c.y);
      }
      else
      {
        FastArith fa;
        Texels t = costmap_gather(a.aux.map, px, py, fa);
        if (__builtin_expect(!fa.ok, 0)) t = costmap_gather(a.aux.map, px, py);
        return t;
      }
    };
    auto step_cost_tx = [&](int n, const Texels& tx, const float* yv, const float* uv, int tt) {
      float c = Model::stateCostFromTexels(cp, tx, yv) + Model::computeControlCost(cp, uv, tt);
      if (a.use_likelihood)
      {
        // the two controls' terms as pairs; the divisions branch-free (the IEEE quotient, re-done exactly when an
        // operand leaves the range where the fast form is exact)
        const bool zero_mean = (float)k[n] >= (1.0f - a.sh.pure_pct) * (float)d.K;
        const float* mr = a.mean + d.t_off + tt * C;
        const f32x2 m = zero_mean ? f32x2{ 0.0f, 0.0f } : f32x2{ mr[0], mr[1] };
        const f32x2 sd = { a.sh.std_dev[0], a.sh.std_dev[1] };
        const f32x2 num = mul2(mul2({ a.sh.control_cost_coeff[0], a.sh.control_cost_coeff[1] }, m),
                               sub2(m, add2({ uv[0], uv[1] }, { uv[0], uv[1] })));
        f32x2 q;
        if constexpr (kTensor)
        {
          q = mul2(num, { a.sh.inv_var[0], a.sh.inv_var[1] });  // the surrogate forms: products with reciprocals
        }
        else
        {
          FastArith fa;
          q = fa.div2(num, mul2(sd, sd));
          if (__builtin_expect(!fa.ok, 0)) q = ExactArith{}.div2(num, mul2(sd, sd));
        }
        float lc = 0.0f;
        lc += q.x;
        lc += q.y;
        c += 0.5f * a.lambda * (1.0f - a.alpha) * lc;
      }
      return c;
    };
    float up[NT][2];
#pragma unroll
    for (int n = 0; n < NT; ++n) up[n][0] = up[n][1] = 0.0f;
    for (int t = 0; t < d.T && ok; ++t)
    {
      float u[NT][2], xin[NT][kMlpIn], y[NT][kMlpOut];
      Texels tx[NT];
#pragma unroll
      for (int n = 0; n < NT; ++n)
      {
        tx[n] = gather(x[n][0], x[n][1]);  // the state step t - 1 produced
        if constexpr (kFused)
        {
          // Gaussian sampling fused in, quad by quad, exactly as gaussian_sample_kernel would have written it
          if ((t & 1) == 0 && active[n])
          {
            const long long q = (long long)k[n] * nq_row + (t >> 1);
            uq[n] = gaussian_quad<C>(a.sh, a.mean + d.t_off, f.decay_pow, f.stride, k[n], pure_threshold, t * C,
                                     fused_noise(f, d, counter, q));
            *reinterpret_cast<float4*>(f.samples + d.u_off + 4 * q) = uq[n];
          }
          u[n][0] = (t & 1) ? uq[n].z : uq[n].x;
          u[n][1] = (t & 1) ? uq[n].w : uq[n].y;
        }
        else
        {
          u[n][0] = u_next[n].x;
          u[n][1] = u_next[n].y;
          if (active[n] && t + 1 < d.T) u_next[n] = __ldg(reinterpret_cast<const float2*>(urow[n] + (t + 1) * C));
        }
        if constexpr (kTensor)
        {
          // the inputs are rounded to 16 bits next, so a multiply by the reciprocal stands in for the division; the
          // nine inputs (state, then controls) in pairs
          const float raw[kMlpIn] = { x[n][0], x[n][1], x[n][2], x[n][3], x[n][4], x[n][5], x[n][6], u[n][0], u[n][1] };
#pragma unroll
          for (int i = 0; i + 1 < kMlpIn; i += 2)
          {
            const f32x2 v = mul2(sub2({ raw[i], raw[i + 1] }, { nm.in_mean[i], nm.in_mean[i + 1] }),
                                 { nm.in_scale[i], nm.in_scale[i + 1] });
            xin[n][i] = v.x;
            xin[n][i + 1] = v.y;
          }
          xin[n][8] = (raw[8] - nm.in_mean[8]) * nm.in_scale[8];
        }
        else
        {
#pragma unroll
          for (int i = 0; i < S; ++i) xin[n][i] = (x[n][i] - nrm[i]) / nrm[9 + i];
          xin[n][7] = (u[n][0] - nrm[7]) / nrm[16];
          xin[n][8] = (u[n][1] - nrm[8]) / nrm[17];
        }
      }
      if constexpr (kTensor)
      {
        ok = mlp_tile_forward<NT, kHalf>(sm, taddr, &mbar, phase, &s_fail, xin, y);
        if (!ok) break;
      }
      else
      {
        mlp_thread_forward(pf, xin[0], y[0]);
      }
#pragma unroll
      for (int n = 0; n < NT; ++n)
      {
        if (t > 0 && active[n]) running[n] += step_cost_tx(n, tx[n], x[n], up[n], t - 1);
        up[n][0] = u[n][0];
        up[n][1] = u[n][1];
        float xd[S];
        float sy, cy;
        if constexpr (kTensor)
          __sincosf(x[n][2], &sy, &cy);  // the surrogate's kinematics: the hardware sine and cosine suffice
        else
          sincos_f(x[n][2], &sy, &cy);
        // x' = vx cos - vy sin, y' = vx sin + vy cos: the products in pairs, the sums scalar (as the analytic model)
        const f32x2 kv = mul2({ x[n][3], x[n][3] }, { cy, sy }), kw = mul2({ x[n][4], x[n][4] }, { sy, cy });
        xd[0] = kv.x - kw.x;
        xd[1] = kv.y + kw.y;
        if constexpr (kTensor)
        {
          // denormalised outputs y * out_std + out_mean, paired fused multiply-adds
#pragma unroll
          for (int j = 0; j + 1 < kMlpOut; j += 2)
          {
            const f32x2 o = fma2({ y[n][j], y[n][j + 1] }, { nm.out_std[j], nm.out_std[j + 1] },
                                 { nm.out_mean[j], nm.out_mean[j + 1] });
            xd[2 + j] = o.x;
            xd[3 + j] = o.y;
          }
          xd[2 + kMlpOut - 1] = fmaf(y[n][kMlpOut - 1], nm.out_std[kMlpOut - 1], nm.out_mean[kMlpOut - 1]);
        }
        else
        {
#pragma unroll
          for (int j = 0; j < kMlpOut; ++j) xd[2 + j] = y[n][j] * nrm[23 + j] + nrm[18 + j];
        }
        // Euler step, two states per paired FMA
#pragma unroll
        for (int i = 0; i + 1 < S; i += 2)
        {
          const f32x2 xn = fma2({ xd[i], xd[i + 1] }, { a.dt, a.dt }, { x[n][i], x[n][i + 1] });
          x[n][i] = xn.x;
          x[n][i + 1] = xn.y;
        }
        x[n][S - 1] = fmaf(xd[S - 1], a.dt, x[n][S - 1]);
      }
    }
    if (ok)
#pragma unroll
      for (int n = 0; n < NT; ++n)
        if (active[n] && d.T > 0)
          running[n] += step_cost_tx(n, gather(x[n][0], x[n][1]), x[n], up[n], d.T - 1);
    if (!ok)
    {
      if (tid == 0) atomicOr(a.status, 1u);
      break;
    }
    unsigned int o = kOrderedPosInf;
#pragma unroll
    for (int n = 0; n < NT; ++n)
      if (active[n])
      {
        const float tf = (float)d.T;
        const float cost = running[n] / tf + Model::terminalCost(cp, a.aux, x[n]) / tf;
        a.costs[d.k_off + k[n]] = cost;
        o = min(o, float_to_ordered(cost));
      }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) o = min(o, __shfl_xor_sync(0xffffffffu, o, off));
    if ((tid & 31) == 0) atomicMin(&s_min, o);
    __syncthreads();
    if (tid == 0) atomicMin(&a.baseline_bits[w.x], s_min);
    if (kTensor && *reinterpret_cast<volatile int*>(&s_fail))  // CTA-uniform: set before the barrier above
    {
      if (tid == 0) atomicOr(a.status, 1u);
      break;
    }
  }
  if constexpr (kTensor)
  {
    tc_fence_before_sync();
    __syncthreads();
    if (warp == 0) tmem_dealloc(taddr, MlpSmem::tmem_cols(NT));
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

// Exclusive prefix counts of two flags over the CTA in thread order (ballot + popc per warp, one warp scans the
// warp totals), packed as (count of f0) | (count of f1) << 16; *total receives the CTA's packed counts.  s_warp
// holds 64 words; counts stay below 2^16 for blockDim.x <= 1024.  Every thread of the CTA must call it (three CTA
// barriers).
__device__ __forceinline__ unsigned int block_excl_count2(bool f0, bool f1, unsigned int* s_warp,
                                                          unsigned int* total)
{
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const unsigned int b0 = __ballot_sync(0xffffffffu, f0), b1 = __ballot_sync(0xffffffffu, f1);
  const unsigned int below = (1u << lane) - 1u;
  const unsigned int in_warp = (unsigned int)__popc(b0 & below) | ((unsigned int)__popc(b1 & below) << 16);
  if (lane == 0) s_warp[warp] = (unsigned int)__popc(b0) | ((unsigned int)__popc(b1) << 16);
  __syncthreads();
  if (warp == 0)
  {
    unsigned int v = lane < nw ? s_warp[lane] : 0u;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1)
    {
      const unsigned int n = __shfl_up_sync(0xffffffffu, v, off);
      if (lane >= off) v += n;
    }
    s_warp[32 + lane] = v;  // inclusive
  }
  __syncthreads();
  const unsigned int before = warp ? s_warp[32 + warp - 1] : 0u;
  *total = s_warp[32 + nw - 1];
  __syncthreads();
  return before + in_warp;
}

__device__ __forceinline__ unsigned int block_min_u32(unsigned int v, unsigned int* s_min)
{
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, off));
  if ((threadIdx.x & 31) == 0) s_min[threadIdx.x >> 5] = v;
  __syncthreads();
  unsigned int m = kOrderedPosInf;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m = min(m, s_min[w]);
  return m;
}

// One CTA per instance: radix selection (4 passes of 8 bits over the ordered-int costs) of the M-th smallest key,
// then an index-ordered compaction of the keys below it plus the first ties, so the judged set and its order are
// deterministic.  Also records the minimum over the samples that are not judged.  The first 16 keys of each thread
// (K <= 16384 at 1024 threads) stay in registers across the passes; keys beyond are read again per pass.
__global__ void __launch_bounds__(1024) judge_select_kernel(const __grid_constant__ JudgeArgs a)
{
  constexpr int KR = 16;
  __shared__ unsigned int hist[256];
  __shared__ unsigned int s_warp[64];
  __shared__ unsigned int s_min[32];
  __shared__ unsigned int s_bin, s_need;
  const int i = blockIdx.x, tid = threadIdx.x, nt = blockDim.x, lane = tid & 31;
  const int base = a.sel_off[i], M = a.sel_off[i + 1] - base;
  const InstDesc d = a.r.inst[i];
  const int K = d.K;
  const float* c = a.r.costs + d.k_off;
  if (M <= 0)
  {
    if (tid == 0) a.unjudged_min[i] = a.r.baseline_bits[i];
    return;
  }
  unsigned int kc[KR];
#pragma unroll
  for (int r = 0; r < KR; ++r)
  {
    const int k = tid + r * nt;
    kc[r] = k < K ? float_to_ordered(c[k]) : 0u;
  }
  const int cached = KR * nt;

  unsigned int prefix = 0u, mask = 0u, need = (unsigned int)M;
  for (int shift = 24; shift >= 0; shift -= 8)
  {
    for (int b = tid; b < 256; b += nt) hist[b] = 0u;
    __syncthreads();
    // the costs share their leading bits, so most lanes of a warp hit the same bin: one atomic per distinct bin
    // and warp (__match_any_sync) instead of one per lane
    auto count = [&](unsigned int key, bool valid) {
      const unsigned int bin = (valid && (key & mask) == prefix) ? ((key >> shift) & 255u) : 256u;
      const unsigned int same = __match_any_sync(0xffffffffu, bin);
      if (bin < 256u && lane == __ffs(same) - 1) atomicAdd(&hist[bin], __popc(same));
    };
#pragma unroll
    for (int r = 0; r < KR; ++r)
    {
      if (r * nt >= K) break;  // CTA-uniform
      count(kc[r], tid + r * nt < K);
    }
    for (int k0 = cached; k0 < K; k0 += nt)
    {
      const int k = k0 + tid;
      count(k < K ? float_to_ordered(c[k]) : 0u, k < K);
    }
    __syncthreads();
    // the first bin b whose inclusive count reaches `need` (255 if none does): lane L of warp 0 holds bins
    // 8L .. 8L+7, an inclusive scan over the lanes finds the lane, and that lane walks its eight bins
    if (tid < 32)
    {
      unsigned int h[8], own = 0u;
#pragma unroll
      for (int j = 0; j < 8; ++j)
      {
        h[j] = hist[8 * lane + j];
        own += h[j];
      }
      unsigned int incl = own;
#pragma unroll
      for (int off = 1; off < 32; off <<= 1)
      {
        const unsigned int n = __shfl_up_sync(0xffffffffu, incl, off);
        if (lane >= off) incl += n;
      }
      const unsigned int reach = __ballot_sync(0xffffffffu, incl >= need);
      const int L = reach ? __ffs(reach) - 1 : 31;
      if (lane == L)
      {
        unsigned int cum = incl - own;
        int b = 7;
#pragma unroll
        for (int j = 0; j < 7; ++j)
        {
          if (b == 7 && cum + h[j] >= need) b = j;
          if (b == 7) cum += h[j];
        }
        s_bin = 8u * (unsigned int)L + (unsigned int)b;
        s_need = need - cum;
      }
    }
    __syncthreads();
    prefix |= s_bin << shift;
    mask |= 255u << shift;
    need = s_need;
    __syncthreads();
  }
  // compaction: sample k is judged when key < thr, or key == thr among the first need_eq ties; its slot is the
  // number of judged samples before it in index order: (keys below thr before it) + min(ties before it, need_eq)
  const unsigned int thr = prefix, need_eq = need;
  unsigned int n_lt = 0u, n_eq = 0u, my_min = kOrderedPosInf;
  auto place = [&](unsigned int key, bool valid, int k) {
    const bool lt = valid && key < thr, eq = valid && key == thr;
    unsigned int tot;
    const unsigned int ex = block_excl_count2(lt, eq, s_warp, &tot);
    const unsigned int r_eq = n_eq + (ex >> 16);
    const bool sel = lt || (eq && r_eq < need_eq);
    const unsigned int pos = n_lt + (ex & 0xffffu) + min(r_eq, need_eq);
    if (sel && pos < (unsigned int)M) a.sel[base + pos] = k;
    if (valid && !sel) my_min = min(my_min, key);
    n_lt += tot & 0xffffu;
    n_eq += tot >> 16;
  };
#pragma unroll
  for (int r = 0; r < KR; ++r)
  {
    if (r * nt >= K) break;  // CTA-uniform
    place(kc[r], tid + r * nt < K, tid + r * nt);
  }
  for (int k0 = cached; k0 < K; k0 += nt)
  {
    const int k = k0 + tid;
    place(k < K ? float_to_ordered(c[k]) : 0u, k < K, k);
  }
  const unsigned int m = block_min_u32(my_min, s_min);
  if (tid == 0) a.unjudged_min[i] = m;
}

// One thread per judged sample: the analytic FP32 rollout of that sample, step for step as the analytic rollout
// kernel (Euler step, running cost on the stepped state, likelihood-ratio term, terminal cost).
__global__ void __launch_bounds__(128) judge_rollout_kernel(const __grid_constant__ JudgeArgs a)
{
  using Model = BicycleSlipModel;
  constexpr int S = Model::STATE_DIM, C = Model::CONTROL_DIM;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= a.total) return;
  const int i = a.sel_inst[j], k = a.sel[j];
  const InstDesc d = a.r.inst[i];
  const typename Model::DynParams& dp = a.r.dyn[i];
  const typename Model::CostParams& cp = a.r.cost[i];
  const float* urow = a.r.samples + d.u_off + (long long)k * d.T * C;
  float x[S];
#pragma unroll
  for (int s = 0; s < S; ++s) x[s] = a.r.x0[d.x_off + s];
  float running = 0.0f;
  PendingCost<Model> pc;
  pc.reset(x);
  // the same step as the analytic rollout kernels; the controls of the next eight steps are loaded while the current
  // eight run, so the chain of dependent steps does not wait on memory.  Rows start on 8-byte boundaries (T * C is
  // even); where T * C % 4 == 0 they also start on 16-byte ones and the eight steps are four 16-byte loads.
  const bool quads = ((d.T * C) & 3) == 0;
  const float4* uq = reinterpret_cast<const float4*>(urow);
  const float2* up = reinterpret_cast<const float2*>(urow);
  auto load8 = [&](int t0, float2 (&dst)[8]) {
    if (quads)
    {
#pragma unroll
      for (int j = 0; j < 4; ++j)
      {
        const float4 q = t0 + 2 * j < d.T ? __ldg(uq + t0 / 2 + j) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        dst[2 * j] = make_float2(q.x, q.y);
        dst[2 * j + 1] = make_float2(q.z, q.w);
      }
    }
    else
    {
#pragma unroll
      for (int j = 0; j < 8; ++j) dst[j] = t0 + j < d.T ? __ldg(up + t0 + j) : make_float2(0.0f, 0.0f);
    }
  };
  auto run = [&](auto lik) {
    float2 cur[8], nxt[8];
    load8(0, cur);
    for (int t0 = 0; t0 < d.T; t0 += 8)
    {
      if (t0 + 8 < d.T) load8(t0 + 8, nxt);
#pragma unroll
      for (int s = 0; s < 8; ++s)
      {
        const int t = t0 + s;
        if (t < d.T)
        {
          const float u[2] = { cur[s].x, cur[s].y };
          speculate_steps<Model>(x, running, pc, [&](auto& ar) {
            rollout_step<Model, decltype(lik)::value>(a.r, d, dp, cp, k, u, t, x, running, pc, ar);
          });
        }
      }
#pragma unroll
      for (int j = 0; j < 8; ++j) cur[j] = nxt[j];
    }
    rollout_flush<Model, decltype(lik)::value>(a.r, d, cp, k, running, pc);
  };
  if (a.r.use_likelihood)
    run(std::true_type{});
  else
    run(std::false_type{});
  const float tf = (float)d.T;
  a.judged_cost[j] = running / tf + Model::terminalCost(cp, a.r.aux, x) / tf;
}

// One CTA per instance: mean judge correction (fixed-order FP64 reduction), corrected costs written back, baseline
// recomputed over judged and unjudged samples.
__global__ void __launch_bounds__(256) judge_finalize_kernel(const __grid_constant__ JudgeArgs a)
{
  __shared__ double s_red[2][8];
  __shared__ unsigned int s_min[8];
  const int i = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int base = a.sel_off[i], M = a.sel_off[i + 1] - base;
  if (M <= 0) return;
  float* c = a.r.costs + a.r.inst[i].k_off;
  double sd = 0.0, sr = 0.0;
  for (int j = tid; j < M; j += blockDim.x)
  {
    const double nw = a.judged_cost[base + j], old = c[a.sel[base + j]];
    sd += nw - old;
    sr += fabs(nw - old) / fmax(fabs(nw), 1e-30);
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1)
  {
    sd += __shfl_xor_sync(0xffffffffu, sd, off);
    sr += __shfl_xor_sync(0xffffffffu, sr, off);
  }
  if (lane == 0)
  {
    s_red[0][warp] = sd;
    s_red[1][warp] = sr;
  }
  __syncthreads();
  double tsd = 0.0, tsr = 0.0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w)
  {
    tsd += s_red[0][w];
    tsr += s_red[1][w];
  }
  const double shift = tsd / M;
  unsigned int mn = kOrderedPosInf;
  for (int j = tid; j < M; j += blockDim.x)
  {
    const float v = (float)((double)a.judged_cost[base + j] - shift);
    c[a.sel[base + j]] = v;
    mn = min(mn, float_to_ordered(v));
  }
  const unsigned int m = block_min_u32(mn, s_min);
  if (tid == 0)
  {
    a.r.baseline_bits[i] = min(m, a.unjudged_min[i]);
    a.stats[2 * i] = (float)shift;
    a.stats[2 * i + 1] = (float)(tsr / M);
  }
}
}  // namespace

mppi_status launch_mlp_rollout(const RolloutArgs<BicycleSlipMLPModel>& a, const float* mlp_d, const MlpNorm& norm,
                               int precision, const FusedNoise* fused, int num_sms, cudaStream_t s)
{
  const bool tensor = precision != 2;
  auto kern = precision == 0 ? (fused ? rollout_mlp_kernel<true, true, false> : rollout_mlp_kernel<true, false, false>)
              : precision == 1 ? (fused ? rollout_mlp_kernel<true, true, true> : rollout_mlp_kernel<true, false, true>)
                               : (fused ? rollout_mlp_kernel<false, true, false> : rollout_mlp_kernel<false, false, false>);
  FusedNoise f{};
  if (fused) f = *fused;
  const size_t smem = tensor ? mlp_smem(precision == 1) : sizeof(float) * kMlpDevParams;
  MG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 1;
  MG_CUDA(resident_ctas_per_sm(kern, tensor ? 128 : kMlpSamplesPerCta, smem, &per_sm));
  per_sm = std::max(1, tensor ? std::min(per_sm, (int)(512 / MlpSmem::tmem_cols(kMlpTiles))) : per_sm);
  const int grid = std::max(1, std::min(a.num_tiles, per_sm * num_sms));
  kern<<<grid, tensor ? 128 : kMlpSamplesPerCta, smem, s>>>(a, mlp_d, norm, f);
  MG_CUDA(cudaGetLastError());
  return MPPI_OK;
}


mppi_status launch_judge(const JudgeArgs& a, cudaStream_t s)
{
  if (a.total <= 0) return MPPI_OK;
  judge_select_kernel<<<a.num_instances, 1024, 0, s>>>(a);
  MG_CUDA(cudaGetLastError());
  judge_rollout_kernel<<<(a.total + 127) / 128, 128, 0, s>>>(a);
  MG_CUDA(cudaGetLastError());
  judge_finalize_kernel<<<a.num_instances, 256, 0, s>>>(a);
  MG_CUDA(cudaGetLastError());
  return MPPI_OK;
}

float e4m3_round(float x)
{
  const float a = std::fabs(x);
  if (a == 0.0f) return x;
  if (a >= 448.0f) return std::copysign(448.0f, x);
  int e = 0;
  std::frexp(a, &e);               // a in [2^(e-1), 2^e)
  const int E = std::max(e - 1, -6);  // below 2^-6 the spacing stays that of the subnormals, 2^-9
  const float quantum = std::ldexp(1.0f, E - 3);
  const float q = std::min(std::nearbyint(a / quantum) * quantum, 448.0f);
  return std::copysign(q, x);
}

void mlp_prepare(const float* params, int precision, float* dev_out, float* effective_out)
{
  std::copy(params, params + kMlpNumParams, dev_out);
  std::copy(params, params + kMlpNumParams, effective_out);
  const int w_off[3] = { kMlpW1, kMlpW2, kMlpW3 };
  const int w_len[3] = { kMlpHid * kMlpIn, kMlpHid * kMlpHid, kMlpOut * kMlpHid };
  for (int l = 0; l < 3; ++l)
  {
    float scale = 1.0f;
    if (precision == 1)
    {
      // the smallest power of two that brings max |W| to at most 448 (the largest E4M3 value): q * scale is then
      // exact in FP32 and, for the weights of a trained layer, in FP16
      float amax = 0.0f;
      for (int e = 0; e < w_len[l]; ++e) amax = std::max(amax, std::fabs(params[w_off[l] + e]));
      if (amax > 0.0f)
      {
        int ex = 0;
        const float fr = std::frexp(amax / 448.0f, &ex);  // amax / 448 = fr * 2^ex, fr in [0.5, 1)
        scale = std::ldexp(1.0f, fr == 0.5f ? ex - 1 : ex);
      }
      for (int e = 0; e < w_len[l]; ++e)
      {
        const float q = e4m3_round(params[w_off[l] + e] / scale);
        dev_out[w_off[l] + e] = q;
        effective_out[w_off[l] + e] = q * scale;
      }
    }
    dev_out[kMlpScale + l] = scale;
  }
}
}  // namespace mg

using namespace mg;

extern "C" {

mppi_status mppi_mlp_quantize(const float* params, int precision, float* out, float* layer_scales)
{
  clear_error();
  MG_CHECK(params && out, "pointers must not be NULL");
  MG_CHECK(precision >= 0 && precision <= 2, "precision must be 0 (bf16), 1 (fp8 e4m3) or 2 (fp32)");
  for (int i = 0; i < MPPI_MLP_PARAMS; ++i) MG_CHECK(std::isfinite(params[i]), "parameter %d is not finite", i);
  std::vector<float> dev(kMlpDevParams), eff(kMlpNumParams);
  mlp_prepare(params, precision, dev.data(), eff.data());
  std::copy(dev.begin(), dev.begin() + kMlpNumParams, out);
  if (layer_scales) std::copy(dev.begin() + kMlpScale, dev.end(), layer_scales);
  return MPPI_OK;
}

mppi_status mppi_kernel_mlp_forward(const float* params, int precision, const float* X_d, float* Y_d, int batch,
                                    void* stream)
{
  clear_error();
  MG_CHECK(params && X_d && Y_d, "pointers must not be NULL");
  MG_CHECK(batch >= 1, "batch must be >= 1");
  MG_CHECK(precision == 0 || precision == 1, "the tensor-core forward takes precision 0 (bf16) or 1 (fp8 e4m3)");
  for (int i = 0; i < MPPI_MLP_PARAMS; ++i) MG_CHECK(std::isfinite(params[i]), "parameter %d is not finite", i);
  for (int i = 0; i < kMlpIn; ++i) MG_CHECK(params[kMlpInStd + i] > 0.0f, "input scale %d must be positive", i);
  std::vector<float> dev(kMlpDevParams), eff(kMlpNumParams);
  mlp_prepare(params, precision, dev.data(), eff.data());
  cudaStream_t s = (cudaStream_t)stream;
  void* buf = nullptr;
  const size_t bytes = sizeof(float) * kMlpDevParams + 256;
  cudaError_t e = cudaMallocAsync(&buf, bytes, s);
  if (e != cudaSuccess)
  {
    set_error("cudaMallocAsync failed: %s", cudaGetErrorString(e));
    return MPPI_ENOMEM;
  }
  float* p_d = (float*)buf;
  unsigned int* status = (unsigned int*)((char*)buf + sizeof(float) * kMlpDevParams + 128);
  mppi_status st = MPPI_OK;
  do
  {
    if ((e = cudaMemcpyAsync(p_d, dev.data(), sizeof(float) * kMlpDevParams, cudaMemcpyHostToDevice, s)) !=
        cudaSuccess)
      break;
    if ((e = cudaMemsetAsync(status, 0, sizeof(unsigned int), s)) != cudaSuccess) break;
    auto kern = precision == 1 ? mlp_forward_kernel<true> : mlp_forward_kernel<false>;
    const size_t smem = MlpSmem::total(1, precision == 1);
    if ((e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) != cudaSuccess)
      break;
    const int tiles = (batch + 127) / 128;
    kern<<<std::min(tiles, 8192), 128, smem, s>>>(p_d, mlp_norm(params), X_d, Y_d, batch, status);
    if ((e = cudaGetLastError()) != cudaSuccess) break;
    unsigned int h = 0;
    if ((e = cudaMemcpyAsync(&h, status, sizeof(h), cudaMemcpyDeviceToHost, s)) != cudaSuccess) break;
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) break;
    if (h)
    {
      set_error("a bounded wait for the tensor cores gave up");
      st = MPPI_ETIMEOUT;
    }
  } while (0);
  cudaFreeAsync(buf, s);
  if (e != cudaSuccess)
  {
    set_error("CUDA failure in mppi_kernel_mlp_forward: %s", cudaGetErrorString(e));
    return MPPI_ECUDA;
  }
  return st;
}

}  // extern "C"
