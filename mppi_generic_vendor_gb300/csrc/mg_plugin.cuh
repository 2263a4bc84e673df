// mg_plugin.cuh — the engine's model concept over a caller's Dynamics / Cost plugin pair (mppi_gb_plugin.cuh), and
// the two kernels that run plugin models: the rollout and the sampled-trajectory read-out.
//
// A plugin model runs rollout mode 0 as: the Gaussian (or colored) sampler kernel writes the constrained samples (or,
// for a plugin with its own enforceConstraints, the unconstrained ones, constrained step by step in the rollout),
// rollout_plugin_kernel integrates them (one thread per sample, controls staged per time chunk in shared memory with
// 16-byte loads, as rollout_kernel does) calling the plugin's step and computeRunningCost in the order of
// rolloutKernel (mppi_common.cu:105-152), folds the tile's weighted partial sums (tile_reduce), and
// tile_finalize_kernel combines the tiles of each instance.
#pragma once

#include <type_traits>

#include "mg_kernels.cuh"

namespace mg
{
// Whether a plugin's dynamics class defines its own enforceConstraints(state, control).
template <class T, class = void>
struct DefinesEnforceConstraints : std::false_type
{
};
template <class T>
struct DefinesEnforceConstraints<T, std::void_t<decltype(&T::enforceConstraints)>> : std::true_type
{
};

// Whether a plugin's dynamics class defines host Jacobians, bool computeGrad(const float* x, const float* u, float* A,
// float* B) (Dynamics::computeGrad, dynamics.cuh:236-242; used by the DDP feedback controller, which otherwise takes
// forward differences).
template <class T, class = void>
struct DefinesComputeGrad : std::false_type
{
};
template <class T>
struct DefinesComputeGrad<T, std::void_t<decltype(&T::computeGrad)>> : std::true_type
{
};

// The engine's Model concept for a plugin pair: the plugin structs are the parameter blocks (one per instance),
// copied to the device by value.  kOwnConstraints: the dynamics class defines enforceConstraints, which then
// replaces the engine's deadband + clamp: the samples are written unconstrained and each rollout step passes its
// control through the plugin's method with the current state and writes the result back (rolloutKernel,
// mppi_common.cu:114-123).
template <class D, class Cst>
struct PluginModel
{
  static constexpr int STATE_DIM = D::STATE_DIM, CONTROL_DIM = D::CONTROL_DIM, OUTPUT_DIM = D::OUTPUT_DIM;
  static constexpr int kModelId = MPPI_MODEL_PLUGIN;
  static constexpr bool kNeedsCostmap = false;
  static constexpr bool kMlp = false;
  static constexpr bool kPlugin = true;
  static constexpr bool kOwnConstraints = DefinesEnforceConstraints<D>::value;
  using DynParams = D;
  using CostParams = Cst;
};

// GaussianDistributionImpl::computeLikelihoodRatioCost (gaussian.cu:490-574) for control u of sample k at step t.
template <int C, class Args>
__device__ __forceinline__ float likelihood_ratio_cost(const Args& a, const InstDesc& d, int k, const float* u, int t)
{
  const bool zero_mean = (float)k >= (1.0f - a.sh.pure_pct) * (float)d.K;
  float lc = 0.0f;
#pragma unroll
  for (int i = 0; i < C; ++i)
  {
    const float m = zero_mean ? 0.0f : a.mean[d.t_off + t * C + i];
    const float sd = a.sh.std_dev[i];
    lc += a.sh.control_cost_coeff[i] * m * (m - 2.0f * u[i]) / (sd * sd);
  }
  return 0.5f * a.lambda * (1.0f - a.alpha) * lc;
}

// rolloutKernel (mppi_common.cu:35-153) over a plugin pair.  Persistent CTAs pull (instance, first sample) tiles;
// thread k integrates sample k: step (derivative, update, output), then the running cost on the output with the
// sample's crash flag, plus the likelihood-ratio term; cost = running / T + terminal(y_T) / T.
template <class Model, int NS, int TCH>
__global__ void __launch_bounds__(NS) rollout_plugin_kernel(const __grid_constant__ RolloutArgs<Model> a)
{
  constexpr int S = Model::STATE_DIM, C = Model::CONTROL_DIM, O = Model::OUTPUT_DIM;
  constexpr int ROW = TCH * C + 4;  // floats per staged sample row (padded so 16-byte reads avoid bank conflicts)
  static_assert((TCH * C) % 4 == 0, "time chunk must hold whole float4s");
  __shared__ __align__(16) float stage[NS * ROW];
  __shared__ int s_tile;
  __shared__ unsigned int s_min;
  __shared__ float s_tw[NS];
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
    const typename Model::DynParams dyn = a.dyn[w.x];
    const typename Model::CostParams cost = a.cost[w.x];
    float x[S], xn[S], xd[S], y[O];
#pragma unroll
    for (int i = 0; i < S; ++i) x[i] = a.x0[d.x_off + i];
#pragma unroll
    for (int i = 0; i < O; ++i) y[i] = 0.0f;
    dyn.stateToOutput(x, y);
    int crash = 0;
    float running = 0.0f;
    const bool aligned = ((d.T * C) & 3) == 0;
    const float* base = a.samples + d.u_off + (long long)w.y * d.T * C;
    for (int t0 = 0; t0 < d.T; t0 += TCH)
    {
      const int nt = min(TCH, d.T - t0);
      if (aligned && (nt * C) % 4 == 0)
      {
        const int q_per_row = nt * C / 4;
        for (int i = tid; i < rows * q_per_row; i += NS)
        {
          const int r = i / q_per_row, qq = i - r * q_per_row;
          *reinterpret_cast<float4*>(&stage[r * ROW + 4 * qq]) =
              __ldg(reinterpret_cast<const float4*>(base + (long long)r * d.T * C + t0 * C) + qq);
        }
      }
      else
      {
        const int per_row = nt * C;
        for (int i = tid; i < rows * per_row; i += NS)
        {
          const int r = i / per_row, j = i - r * per_row;
          stage[r * ROW + j] = __ldg(base + (long long)r * d.T * C + t0 * C + j);
        }
      }
      __syncthreads();
      if (active)
        for (int tt = 0; tt < nt; ++tt)
        {
          const int t = t0 + tt;
          float u[C];
#pragma unroll
          for (int c = 0; c < C; ++c) u[c] = stage[tid * ROW + tt * C + c];
          if constexpr (Model::kOwnConstraints)
          {
            // the plugin's constraint with the state, written back as the sample (the samples buffer is the
            // engine's own; the tile's weighted sums read it after the CTA barrier that follows)
            dyn.enforceConstraints(x, u);
            float* wb = const_cast<float*>(a.samples) + d.u_off + ((long long)k * d.T + t) * C;
#pragma unroll
            for (int c = 0; c < C; ++c) wb[c] = u[c];
          }
          dyn.step(x, xn, xd, u, y, t, a.dt);
          float c = cost.computeRunningCost(y, u, t, &crash);
          if (a.use_likelihood) c += likelihood_ratio_cost<C>(a, d, k, u, t);
          running += c;
#pragma unroll
          for (int i = 0; i < S; ++i) x[i] = xn[i];
        }
      __syncthreads();
    }
    unsigned int o = kOrderedPosInf;
    if (active)
    {
      const float tf = (float)d.T;
      const float c = running / tf + cost.terminalCost(y) / tf;
      a.costs[d.k_off + k] = c;
      o = float_to_ordered(c);
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) o = min(o, __shfl_xor_sync(0xffffffffu, o, off));
    if ((tid & 31) == 0) atomicMin(&s_min, o);
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

// visualizeKernel (mppi_common.cu:371-533) over a plugin pair: one thread per chosen sample re-runs its stored
// controls and records the output after each step, each step's running cost and the crash flag after each step.
template <class Model>
__global__ void __launch_bounds__(128) sampled_trajectories_plugin_kernel(const __grid_constant__ RolloutArgs<Model> a,
                                                                          int inst, const int* idx, int n,
                                                                          float* outputs, float* step_costs,
                                                                          float* terminal, int* crash_out)
{
  constexpr int S = Model::STATE_DIM, C = Model::CONTROL_DIM, O = Model::OUTPUT_DIM;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const InstDesc d = a.inst[inst];
  const int k = idx[j];
  const typename Model::DynParams dyn = a.dyn[inst];
  const typename Model::CostParams cost = a.cost[inst];
  float x[S], xn[S], xd[S], y[O];
#pragma unroll
  for (int i = 0; i < S; ++i) x[i] = a.x0[d.x_off + i];
#pragma unroll
  for (int i = 0; i < O; ++i) y[i] = 0.0f;
  dyn.stateToOutput(x, y);
  int crash = 0;
  const float* us = a.samples + d.u_off + (long long)k * d.T * C;
  for (int t = 0; t < d.T; ++t)
  {
    float u[C];
#pragma unroll
    for (int c = 0; c < C; ++c) u[c] = us[t * C + c];
    if constexpr (Model::kOwnConstraints) dyn.enforceConstraints(x, u);  // as visualizeKernel (mppi_common.cu:453)
    dyn.step(x, xn, xd, u, y, t, a.dt);
    float c = cost.computeRunningCost(y, u, t, &crash);
    if (a.use_likelihood) c += likelihood_ratio_cost<C>(a, d, k, u, t);
#pragma unroll
    for (int i = 0; i < O; ++i) outputs[((long long)j * d.T + t) * O + i] = y[i];
    step_costs[(long long)j * d.T + t] = c;
    if (crash_out) crash_out[(long long)j * d.T + t] = crash;
#pragma unroll
    for (int i = 0; i < S; ++i) x[i] = xn[i];
  }
  terminal[j] = cost.terminalCost(y);
}

}  // namespace mg
