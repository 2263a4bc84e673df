// mg_rmppi.cuh — the two kernels of the robust controller (R-MPPI):
//  * rmppi_rollout_kernel: rolloutRMPPIKernel (rmppi_kernels.cu:666-861).  The reference runs the nominal and the real
//    system of a sample as two threads (threadIdx.z) sharing the nominal state through shared memory; here they are
//    two neighbouring lanes of a warp, so the real system's feedback K_t (x_real - x_nominal) reads the nominal state
//    of the same step by a register shuffle.  Both controls pass through the constraints (deadband, clamp) every step and are written back
//    as the samples the update averages.  Costs (running cost on the stepped state, likelihood-ratio term, terminal
//    cost, all divided by T): the real system pays running + likelihood; the nominal one
//        0.5 J_nom + 0.5 max(min(J_real_fb, threshold), J_nom) + likelihood_nom,
//    with J_real_fb the real system's running cost plus the feedback cost (computeFeedbackCost, gaussian.cu:577-630).
//    The reference's device feedback (DeviceDDPImpl::k, ddp.cu:11-44) overwrites instead of accumulating for an even
//    control dimension; the kernel applies the whole product K_t e, as the reference's host DDPFeedback::k_ does.
//  * rmppi_eval_kernel: initEvalKernel (rmppi_kernels.cu:231-357): num_candidates x samples_per_candidate rollouts,
//    candidate c from its state with the samples of the nominal distribution read at t + stride_c (held at T-1).
// Both run the built-in models and a caller's plugin pair (its own step, computeRunningCost with the sample's crash
// flag, and its own enforceConstraints when it defines one).  One thread per sample, no shared memory and no waits.
// The evaluation's time loop issues each step's sample load kPrefetch steps ahead into a register ring (the loop runs
// in unrolled groups of kPrefetch steps so every ring slot is a fixed register).
#pragma once

#include "mg_kernels.cuh"
#include "mg_plugin.cuh"

namespace mg
{

// One increment of a device counter (the Philox noise counter after the candidate evaluation's sampling).
static __global__ void bump_u32_kernel(unsigned int* p) { *p += 1u; }

constexpr int kPrefetch = 4;  // steps between a load and its use

template <class Model>
struct RmppiArgs
{
  const InstDesc* inst;  // [0] nominal distribution, [1] real distribution
  float* samples;        // unconstrained samples in, the constrained controls (real: with feedback) out
  const float* mean;     // both distributions' means (the importance sampler)
  const float* x0;       // [nominal state | real state]
  const float* gains;    // per step a CONTROL_DIM x STATE_DIM gain, column-major
  float* costs;
  unsigned int* baseline_bits;  // per distribution: ordered-int minimum of its costs
  const typename Model::DynParams* dyn;
  const typename Model::CostParams* cost;
  ModelAux aux;
  SampleShared sh;  // the control constraints, standard deviations, cost coefficients and pure-noise share
  float lambda, alpha, dt, value_threshold;
  int use_likelihood;
};

// The control constraint of a step: a plugin's own enforceConstraints with the state, else the deadband and the clamp
// of the handle's ranges (Dynamics::enforceConstraints, dynamics.cu:107-126).
template <class Model, class Args>
__device__ __forceinline__ void rmppi_constrain(const Args& a, const typename Model::DynParams& dp, float* x, float* u)
{
  if constexpr (Model::kOwnConstraints)
  {
    dp.enforceConstraints(x, u);
  }
  else
  {
#pragma unroll
    for (int c = 0; c < Model::CONTROL_DIM; ++c)
      u[c] = enforce_constraint(u[c], a.sh.lower[c], a.sh.upper[c], a.sh.deadband[c], a.sh.zero[c]);
  }
}

// One step x -> xn under u and its running cost on the output y (Dynamics::step, Cost::computeRunningCost with the
// crash flag, cost.cu:39-53): a plugin's own step, or the explicit Euler step of a built-in model (y = xn).
template <class Model, class Args>
__device__ __forceinline__ float rmppi_step(const Args& a, const typename Model::DynParams& dp,
                                            const typename Model::CostParams& cp, const float* x, const float* u,
                                            float* xn, float* y, int t, int* crash)
{
  if constexpr (Model::kPlugin)
  {
    float xd[Model::STATE_DIM];
    dp.step(x, xn, xd, u, y, t, a.dt);
    return cp.computeRunningCost(y, u, t, crash);
  }
  else
  {
    euler_step<Model>(dp, x, u, xn, a.dt);
#pragma unroll
    for (int s = 0; s < Model::STATE_DIM; ++s) y[s] = xn[s];
    return Model::computeStateCost(cp, a.aux, xn, t) + Model::computeControlCost(cp, u, t);
  }
}

template <class Model, class Args>
__device__ __forceinline__ float rmppi_terminal(const Args& a, const typename Model::CostParams& cp, const float* y)
{
  if constexpr (Model::kPlugin)
    return cp.terminalCost(y);
  else
    return Model::terminalCost(cp, a.aux, y);
}

// GaussianDistributionImpl::computeFeedbackCost (gaussian.cu:577-630): 0.5 lambda (1 - alpha) sum_i coeff_i fb_i^2 /
// sd_i^2, the terms added in control order.
template <int C, class Args>
__device__ __forceinline__ float feedback_cost(const Args& a, const float* fb)
{
  float c = 0.0f;
#pragma unroll
  for (int i = 0; i < C; ++i) c += a.sh.control_cost_coeff[i] * (fb[i] * fb[i]) / (a.sh.std_dev[i] * a.sh.std_dev[i]);
  return 0.5f * a.lambda * (1.0f - a.alpha) * c;
}

// Lane 2i of a warp runs sample k's nominal system and lane 2i + 1 its real system (the reference's threadIdx.z = 0
// and 1): each lane carries one dependent chain of steps, and the real lane reads the nominal state of the same step
// from its partner by a shuffle.  Pairs past K run sample K - 1 without writing anything, so that every lane of a
// warp reaches each shuffle.
template <class Model>
__global__ void __launch_bounds__(128) rmppi_rollout_kernel(const __grid_constant__ RmppiArgs<Model> a)
{
  constexpr int S = Model::STATE_DIM, C = Model::CONTROL_DIM, O = Model::OUTPUT_DIM;
  constexpr unsigned kFull = 0xffffffffu;
  const InstDesc dn = a.inst[0], dr = a.inst[1];
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  const bool real = (threadIdx.x & 1) != 0;
  const bool active = (g >> 1) < dn.K;
  const int k = active ? (g >> 1) : dn.K - 1;
  const int nominal_lane = (threadIdx.x & 31) & ~1;
  const int T = dn.T;
  // the parameter blocks by value: the sample write-backs below cannot alias them
  const typename Model::DynParams dp = a.dyn[0];
  const typename Model::CostParams cp = a.cost[0];
  const InstDesc d = real ? dr : dn;
  float x[S], y[O];
  int crash = 0;  // crash_status of this lane's system (mppi_common.cu:85-86)
#pragma unroll
  for (int s = 0; s < S; ++s) x[s] = a.x0[(real ? S : 0) + s];
  float* row = a.samples + d.u_off + (long long)k * T * C;
  // nominal lane: running cost and likelihood apart; real lane: running + likelihood, and running + feedback cost
  float run = 0.0f, lik = 0.0f, extra = 0.0f;
  for (int t = 0; t < T; ++t)
  {
    float u[C], fb[C], x2[S], xnom[S], K[C * S];
    // this step's loads first (both lanes load the gain, the same for every lane, so that the load is issued before
    // the shuffles rather than behind the branch)
#pragma unroll
    for (int c = 0; c < C; ++c) u[c] = row[t * C + c];
#pragma unroll
    for (int i = 0; i < C * S; ++i) K[i] = a.gains[(size_t)t * C * S + i];
#pragma unroll
    for (int s = 0; s < S; ++s) xnom[s] = __shfl_sync(kFull, x[s], nominal_lane);
    if (real)
    {
      // the real system adds the feedback K_t (x_real - x_nominal) of this step
#pragma unroll
      for (int r = 0; r < C; ++r)
      {
        float acc = 0.0f;
#pragma unroll
        for (int c = 0; c < S; ++c) acc += K[r + c * C] * (x[c] - xnom[c]);
        fb[r] = acc;
      }
#pragma unroll
      for (int c = 0; c < C; ++c) u[c] = u[c] + fb[c];
    }
    rmppi_constrain<Model>(a, dp, x, u);
    if (active)
#pragma unroll
      for (int c = 0; c < C; ++c) row[t * C + c] = u[c];
    const float cs = rmppi_step<Model>(a, dp, cp, x, u, x2, y, t, &crash);
    if (real)
    {
      if (a.use_likelihood)
        run += cs + likelihood_ratio_cost<C>(a, d, k, u, t);
      else
        run += cs;
      extra += cs + feedback_cost<C>(a, fb);
    }
    else
    {
      run += cs;
      if (a.use_likelihood) lik += likelihood_ratio_cost<C>(a, d, k, u, t);
    }
#pragma unroll
    for (int s = 0; s < S; ++s) x[s] = x2[s];
  }
  const float term = rmppi_terminal<Model>(a, cp, y);
  run += term;
  if (real) extra += term;
  const float Tf = (float)T;
  run /= Tf;
  lik /= Tf;
  extra /= Tf;
  const float extra_r = __shfl_sync(kFull, extra, nominal_lane + 1);
  if (!active) return;
  if (real)
  {
    a.costs[dr.k_off + k] = run;
    atomicMin(&a.baseline_bits[1], float_to_ordered(run));
  }
  else
  {
    // 0.5 J_nom + 0.5 max(min(J_real_fb, threshold), J_nom), formed in double as the reference's double literals
    // make it
    float cost_n = (float)(0.5 * (double)run + 0.5 * (double)fmaxf(fminf(extra_r, a.value_threshold), run));
    cost_n += lik;
    a.costs[dn.k_off + k] = cost_n;
    atomicMin(&a.baseline_bits[0], float_to_ordered(cost_n));
  }
}

template <class Model>
struct RmppiEvalArgs
{
  InstDesc d;              // the nominal distribution: its samples, mean and K
  const float* samples;
  const float* mean;
  const float* cand_states;  // [num_cand][STATE_DIM]
  const int* cand_strides;   // [num_cand]
  int num_cand, per_cand;
  float* costs;              // [num_cand * per_cand]
  const typename Model::DynParams* dyn;
  const typename Model::CostParams* cost;
  ModelAux aux;
  SampleShared sh;
  float lambda, alpha, dt;
  int use_likelihood;
};

template <class Model>
__global__ void __launch_bounds__(64) rmppi_eval_kernel(const __grid_constant__ RmppiEvalArgs<Model> a)
{
  constexpr int S = Model::STATE_DIM, C = Model::CONTROL_DIM, O = Model::OUTPUT_DIM;
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= a.num_cand * a.per_cand) return;
  const int cand = g / a.per_cand, j = g - cand * a.per_cand;
  const int T = a.d.T, stride = a.cand_strides[cand];
  const typename Model::DynParams dp = a.dyn[0];
  const typename Model::CostParams cp = a.cost[0];
  const float* row = a.samples + a.d.u_off + (long long)j * T * C;
  float x[S], y[O];
#pragma unroll
  for (int s = 0; s < S; ++s) x[s] = a.cand_states[cand * S + s];
  float running = 0.0f;
  int crash = 0;
  // ring of the next kPrefetch steps' samples (step t reads the sample at min(t + stride, T - 1))
  float ring[kPrefetch][C];
#pragma unroll
  for (int j = 0; j < kPrefetch; ++j)
  {
    const int tc = min(j + stride, T - 1);
#pragma unroll
    for (int c = 0; c < C; ++c) ring[j][c] = row[tc * C + c];
  }
  for (int t0 = 0; t0 < T; t0 += kPrefetch)
#pragma unroll
  for (int j = 0; j < kPrefetch; ++j)
  {
    const int t = t0 + j;
    if (t >= T) break;
    float u[C], xn[S];
#pragma unroll
    for (int c = 0; c < C; ++c) u[c] = ring[j][c];
    {
      const int tn = min(t + kPrefetch + stride, T - 1);
#pragma unroll
      for (int c = 0; c < C; ++c) ring[j][c] = row[tn * C + c];
    }
    rmppi_constrain<Model>(a, dp, x, u);
    float c = rmppi_step<Model>(a, dp, cp, x, u, xn, y, t, &crash);
    // the likelihood term of sample g (its index among the evaluation rollouts) against the mean at step t
    if (a.use_likelihood) c += likelihood_ratio_cost<C>(a, a.d, g, u, t);
    running += c;
#pragma unroll
    for (int s = 0; s < S; ++s) x[s] = xn[s];
  }
  const float Tf = (float)T;
  a.costs[g] = running / Tf + rmppi_terminal<Model>(a, cp, y) / Tf;
}

}  // namespace mg
