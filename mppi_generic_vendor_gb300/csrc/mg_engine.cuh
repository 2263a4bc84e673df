// mg_engine.cuh — host side of the engine: the Controller / VanillaMPPIController re-designed for one GB300.
//
// Engine<Model> holds num_instances independent MPPI problems of one plugin pair.  One computeControl enqueues, for
// every optimisation iteration, three kernels that each cover all instances (sample, rollout, weights+update); the
// whole sequence, including the H2D copy of the initial states and nominal controls and the D2H copy of the results,
// is recorded once as a CUDA graph per optimisation stride and replayed.  The host then applies the reference's
// post-processing per instance: Savitzky-Golay smoothing, nominal state rollout and control clamp
// (VanillaMPPIController::computeControl, mppi_controller.cu:152-237).
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "mg_common.cuh"
#include "mg_colored.cuh"
#include "mg_kernels.cuh"
#include "mg_mlp.cuh"
#include "mg_plugin.cuh"
#include "mg_ddp.h"
#include "mg_rmppi.cuh"

namespace mg
{
struct CreateArgs
{
  int model;
  int num_instances;
  const int* K;
  const int* T;
  mppi_controller_params cp;
  mppi_sampling_params sp;
  mppi_control_constraints cc;
  const void* dyn;
  size_t dyn_bytes;
  const void* cost;
  size_t cost_bytes;
  const float* init_control;
  cudaStream_t stream;
};

class EngineBase
{
public:
  virtual ~EngineBase() {}
  virtual int model() const = 0;
  virtual int state_dim() const = 0;
  virtual int control_dim() const = 0;
  virtual int num_instances() const = 0;
  virtual void dims(int i, int* K, int* T) const = 0;
  virtual mppi_status compute_control(const float* x0, int stride) = 0;
  virtual mppi_status get_control_seq(float* out) = 0;
  virtual mppi_status set_control_seq(const float* in) = 0;
  virtual mppi_status slide_control_sequence(int steps) = 0;
  virtual mppi_status get_state_seq(float* out) = 0;
  virtual mppi_status get_baseline_normalizer(float* out, double* norm64) = 0;
  virtual mppi_status get_sample_costs(float* out) = 0;
  virtual mppi_status get_sample_weights(float* out) = 0;
  virtual mppi_status get_control_samples(float* out) = 0;
  virtual mppi_status get_sampled_trajectories(int i, const int* idx, int n, float* states, float* step_costs,
                                               float* terminal, int* crash) = 0;
  virtual int output_dim() const = 0;
  virtual mppi_status get_free_energy(int i, float* out6) = 0;
  virtual mppi_status set_dynamics_params(const void* p, size_t bytes) = 0;
  virtual mppi_status set_cost_params(const void* p, size_t bytes) = 0;
  virtual mppi_status set_sampling_params(const mppi_sampling_params* sp) = 0;
  virtual mppi_status set_controller_params(const mppi_controller_params* cp) = 0;
  virtual mppi_status set_costmap(const float* map, int w, int h, float res, float ox, float oy) = 0;
  virtual mppi_status inject_noise(const float* noise, size_t count) = 0;
  virtual mppi_status generate_samples(int stride, int iter) = 0;
  virtual mppi_status set_graph_mode(int enable) = 0;
  virtual mppi_status get_launch_config(int* ns, int* tch, int* kc) const = 0;
  // Rollout mode: 0 = one fused kernel, 1 = split dynamics / cost kernels, 2 = cooperative, 3 = sampler kernel then
  // the staged rollout, 4 = fused with noise warps; rollout_modes() is the bitmask available.
  virtual mppi_status set_rollout_mode(int mode) = 0;
  virtual int rollout_mode() const = 0;
  virtual int rollout_modes() const = 0;
  virtual mppi_status set_launch_config(int ns, int tch, int kc) = 0;
  virtual mppi_status autotune(const char* cache_path) = 0;
  virtual int kernels_per_compute() const = 0;
  virtual cudaStream_t stream() const = 0;
  virtual mppi_status enqueue_device_solves(int stride, int count) = 0;
  virtual mppi_status time_kernels(int stride, int reps, float* ms3) = 0;
  virtual mppi_status set_mlp(const float* params, size_t n, int precision) = 0;
  virtual mppi_status set_judge(float fraction) = 0;
  virtual mppi_status get_judge_stats(float* out) = 0;
  virtual mppi_status use_analytic(int enable) = 0;
  virtual mppi_status nominal_state_used(int* used) = 0;
  virtual mppi_status set_wait_diagnostics(uint32_t max_polls, int withhold_progress) = 0;
  // ancillary feedback controller (DDPFeedback, feedback_controllers/DDP/ddp.cu)
  virtual mppi_status set_feedback_params(const float* Q, const float* Qf, const float* R, int iterations) = 0;
  virtual mppi_status enable_feedback(int enable) = 0;
  virtual int feedback_enabled() const = 0;
  virtual mppi_status compute_feedback(const float* x0) = 0;
  virtual mppi_status get_feedback_gains(float* out) const = 0;
  virtual mppi_status feedback_control(const float* x, const float* goal, int t, float* u) const = 0;
  virtual mppi_status feedback_propagated_state_seq(float* out) = 0;
  // the robust controller's importance sampler (RobustMPPIController::updateImportanceSamplingControl)
  virtual mppi_status rmppi_update_importance_sampler(const float* x, int stride) = 0;
  virtual mppi_status rmppi_get_candidates(int* best, int* nominal_stride, float* states, int* strides, float* fe,
                                           float* eval_costs) const = 0;
};

// Factories, one per model translation unit.
mppi_status create_cartpole_engine(const CreateArgs& a, EngineBase** out);
mppi_status create_double_integrator_engine(const CreateArgs& a, EngineBase** out);
mppi_status create_bicycle_costmap_engine(const CreateArgs& a, EngineBase** out);
mppi_status create_bicycle_slip_engine(const CreateArgs& a, EngineBase** out);
mppi_status create_bicycle_slip_mlp_engine(const CreateArgs& a, EngineBase** out);

// Kernel-level rollout entry points, one per model translation unit.
mppi_status standalone_rollout_cartpole(const void* dyn, const void* cost, const mppi_sampling_params* sp,
                                        const float* x0_d, const float* controls_d, const float* mean_d,
                                        float* costs_d, int K, int T, float dt, float lambda, float alpha,
                                        cudaStream_t s);
mppi_status standalone_rollout_double_integrator(const void* dyn, const void* cost, const mppi_sampling_params* sp,
                                                 const float* x0_d, const float* controls_d, const float* mean_d,
                                                 float* costs_d, int K, int T, float dt, float lambda, float alpha,
                                                 cudaStream_t s);

// Rollout CTA sizes the engine instantiates; the time chunk follows from the 48 KB static shared-memory budget.
template <int NS, int C>
struct RolloutShape
{
  static constexpr int TCH = (NS * (32 * C + 4) * 4 <= 48 * 1024) ? 32 : 16;
};

inline SampleShared make_sample_shared(const mppi_sampling_params& sp, const mppi_control_constraints& cc,
                                       int final_clamp = 0)
{
  SampleShared sh{};
  sh.final_clamp = final_clamp;
  for (int i = 0; i < kMaxC; ++i)
  {
    sh.std_dev[i] = sp.std_dev[i];
    sh.inv_var[i] = 1.0f / (sp.std_dev[i] * sp.std_dev[i]);
    sh.control_cost_coeff[i] = sp.control_cost_coeff[i];
    sh.lower[i] = cc.lower[i];
    sh.upper[i] = cc.upper[i];
    sh.deadband[i] = cc.deadband[i];
    sh.zero[i] = cc.zero_control[i];
  }
  sh.pure_pct = sp.pure_noise_trajectories_percentage;
  return sh;
}

template <class Model>
class Engine : public EngineBase
{
public:
  static constexpr int S = Model::STATE_DIM;
  static constexpr int C = Model::CONTROL_DIM;
  using DynParams = typename Model::DynParams;
  using CostParams = typename Model::CostParams;

  ~Engine() override
  {
    if (stream_) cudaStreamSynchronize(stream_);
    invalidate_graphs();
    if (own_stream_ && stream_) cudaStreamDestroy(stream_);
  }

  static mppi_status create(const CreateArgs& a, EngineBase** out)
  {
    MG_CHECK(a.num_instances >= 1, "num_instances must be >= 1 (got %d)", a.num_instances);
    MG_CHECK(a.K && a.T, "num_rollouts and num_timesteps arrays are required");
    MG_CHECK(a.dyn_bytes == sizeof(DynParams), "dynamics parameter block is %zu bytes, model expects %zu",
             a.dyn_bytes, sizeof(DynParams));
    MG_CHECK(a.cost_bytes == sizeof(CostParams), "cost parameter block is %zu bytes, model expects %zu",
             a.cost_bytes, sizeof(CostParams));
    MG_CHECK(a.dyn && a.cost, "parameter blocks must not be NULL");
    std::unique_ptr<Engine> e(new Engine());
    MG_TRY(e->init(a));
    *out = e.release();
    return MPPI_OK;
  }

  int model() const override { return Model::kModelId; }
  int state_dim() const override { return S; }
  int output_dim() const override { return Model::OUTPUT_DIM; }
  int control_dim() const override { return C; }
  int num_instances() const override { return I_; }
  void dims(int i, int* K, int* T) const override
  {
    if (K) *K = K_[i];
    if (T) *T = T_[i];
  }
  cudaStream_t stream() const override { return stream_; }
  int kernels_per_compute() const override
  {
    int sampler = 1;
    if (sp_.kind == MPPI_SAMPLER_COLORED_NOISE)
    {
      sampler = 0;
      for (int k = 0; k < 5; ++k) sampler += class_begin_[k + 1] > class_begin_[k] ? 1 : 0;
    }
    const int judge = (Model::kMlp && !use_analytic_ && judge_total_ > 0) ? 3 : 0;
    const int iters = tube() ? 1 : cp_.num_iters;  // Tube-MPPI runs its iterations one graph launch at a time
    if (tail_finalize()) return iters;  // one fused rollout per iteration, nothing else
    if (fused()) sampler = 0;
    if (fused() && split_) sampler = 1;  // the cost kernel
    return (sampler + 2 + judge) * iters;  // the last combine smooths and constrains
  }

  // ------------------------------------------------------------------------------------------------ computeControl
  mppi_status compute_control(const float* x0, int stride) override
  {
    MG_CHECK(x0 != nullptr, "x0 must not be NULL");
    MG_CHECK(stride >= 0, "optimization_stride must be >= 0");
    if (tube()) return compute_control_tube(x0, stride);
    if (rmppi()) return compute_control_rmppi(x0, stride);
    MG_CHECK(!Model::kNeedsCostmap || aux_.map.data != nullptr, "this model needs a costmap (mppi_set_costmap)");
    MG_CHECK(!Model::kMlp || use_analytic_ || !mlp_host_.empty(), "this model needs surrogate weights (mppi_set_mlp)");
    for (int i = 0; i < I_ * S; ++i)
      if (!std::isfinite(x0[i]))
      {
        set_error("initial state has a non-finite entry at index %d", i);
        return MPPI_ENAN;
      }
    for (int i = 0; i < I_; ++i) prev_baseline_[i] = baseline_norm_[2 * i];
    if (cp_.controller == MPPI_CONTROLLER_COLORED && cp_.leash_active)
    {
      // ColoredMPPIController::computeControl (colored_mppi_controller.cu:150-153): the state the solve starts from
      // is held within state_leash_dist of the nominal state at step leash_jump_ of the previous solve
      // (Dynamics::enforceLeash, dynamics.cuh:445-463)
      if (traj_dirty_) compute_state_seq();
      leashed_x0_.assign(x0, x0 + (size_t)I_ * S);
      size_t so = 0;
      for (int i = 0; i < I_; ++i)
      {
        const int j = std::min(std::max(leash_jump_, 0), T_[i] - 1);
        const float* nominal = state_seq_.data() + so + (size_t)j * S;
        float* xo = leashed_x0_.data() + (size_t)i * S;
        for (int s = 0; s < S; ++s)
        {
          const float xt = x0[(size_t)i * S + s], xn = nominal[s], leash = cp_.state_leash_dist[s];
          const float diff = fabsf(xn - xt);
          xo[s] = leash < diff ? xt + fminf(fmaxf(xn - xt, -leash), leash) : xn;
        }
        so += (size_t)T_[i] * S;
      }
      x0 = leashed_x0_.data();
    }
    memcpy(x0_h_.p, x0, sizeof(float) * I_ * S);
    memcpy(mean_h_.p, control_.data(), sizeof(float) * control_.size());
    if (graph_mode_)
    {
      cudaGraphExec_t exec = nullptr;
      MG_TRY(get_graph(stride, &exec));
      MG_CUDA(cudaGraphLaunch(exec, stream_));
    }
    else
    {
      MG_TRY(enqueue_solve(stride));
    }
    MG_CUDA(cudaStreamSynchronize(stream_));
    return finish_solve(x0);
  }

  mppi_status get_control_seq(float* out) override
  {
    MG_CHECK(out, "out must not be NULL");
    memcpy(out, control_.data(), sizeof(float) * control_.size());
    return MPPI_OK;
  }
  mppi_status set_control_seq(const float* in) override
  {
    MG_CHECK(in, "in must not be NULL");
    memcpy(control_.data(), in, sizeof(float) * control_.size());
    return MPPI_OK;
  }
  // Controller::slideControlSequence -> saveControlHistoryHelper + slideControlSequenceHelper (controller.cuh:370-376,
  // 609-636).  The history only feeds smoothing variants the reference no longer uses, but it is kept for parity.
  mppi_status slide_control_sequence(int steps) override
  {
    MG_CHECK(steps >= 0, "steps must be >= 0");
    leash_jump_ = steps;  // ColoredMPPIController::slideControlSequence (colored_mppi_controller.cu:260-268)
    if (tube())
    {
      // TubeMPPIController::slideControlSequence (tube_mppi_controller.cu:313-324): the nominal state advances one
      // step along the nominal sequence (Dynamics::step, no constraint), then both sequences slide
      if (nominal_init_) advance_nominal_state();
    }
    // RobustMPPIController::slideControlSequence does nothing (robust_mppi_controller.cuh:186-190): the nominal
    // sequence slides inside the importance-sampler update (mppi_rmppi_update_importance_sampler)
    if (rmppi()) return MPPI_OK;
    for (int i = 0; i < I_; ++i) slide_one(i, steps);
    return MPPI_OK;
  }
  // Controller::saveControlHistoryHelper + slideControlSequenceHelper (controller.cuh:609-636) for instance i
  void slide_one(int i, int steps)
  {
    {
      float* u = control_.data() + t_off_[i];
      const int T = T_[i];
      float* hist = history_.data() + (size_t)i * 2 * C;
      if (steps == 1)
      {
        for (int c = 0; c < C; ++c)
        {
          hist[c] = hist[C + c];
          hist[C + c] = last_pre_smooth_[(size_t)i * C + c];
        }
      }
      else if (steps >= 2)
      {
        for (int c = 0; c < C; ++c)
        {
          hist[c] = u[(size_t)std::min(steps - 2, T - 1) * C + c];
          hist[C + c] = u[(size_t)std::min(steps - 1, T - 1) * C + c];
        }
      }
      for (int t = 0; t < T; ++t)
      {
        const int ind = std::min(t + steps, T - 1);
        for (int c = 0; c < C; ++c)
        {
          float v = u[(size_t)ind * C + c];
          if (t + steps > T - 1)
            v = (v - cc_.zero_control[c]) * cp_.slide_control_scale[c] + cc_.zero_control[c];
          u[(size_t)t * C + c] = v;
        }
      }
    }
  }
  mppi_status get_state_seq(float* out) override
  {
    MG_CHECK(out, "out must not be NULL");
    if (traj_dirty_) compute_state_seq();
    memcpy(out, state_seq_.data(), sizeof(float) * state_seq_.size());
    return MPPI_OK;
  }

  // computeOutputTrajectoryHelper (controller.cuh:664-684): x0, then T-1 steps under the constrained nominal controls
  // of the last solve, with the model's host twin (the surrogate in FP32 for the MLP model).
  void compute_state_seq()
  {
    float* xs = state_seq_.data();
    for (int i = 0; i < I_; ++i)
    {
      const int T = T_[i];
      const float* u = traj_u_.data() + t_off_[i];
      float x[S], xn[S];
      for (int s = 0; s < S; ++s) x[s] = xs[s] = traj_x0_[(size_t)i * S + s];
      for (int t = 0; t < T - 1; ++t)
      {
        const float* uc = u + (size_t)t * C;
        if constexpr (Model::kPlugin)
        {
          // the plugin's own step (Dynamics::step, dynamics.cu:142-152) on its host twin; a plugin with its own
          // enforceConstraints sees the smoothed control with the state first (controller.cuh:676-680)
          float xd[S], y[Model::OUTPUT_DIM], ucon[C];
          for (int c = 0; c < C; ++c) ucon[c] = uc[c];
          if constexpr (Model::kOwnConstraints) dyn_[i].enforceConstraints(x, ucon);
          dyn_[i].step(x, xn, xd, ucon, y, t, cp_.dt);
        }
        else if (Model::kMlp && !use_analytic_)
        {
          float xd[S];
          mlp_host_dynamics(mlp_host_.data(), x, uc, xd);
          for (int s = 0; s < S; ++s) xn[s] = fmaf(xd[s], cp_.dt, x[s]);
        }
        else if (cp_.controller == MPPI_CONTROLLER_COLORED)
        {
          // ColoredMPPI clamps only control 1 after smoothing; computeOutputTrajectoryHelper still passes every
          // control through enforceConstraints (controller.cuh:676-680).  (With a deadband and a smoothed control 1
          // outside its range the reference would constrain the unclamped value; the clamp comes first here.)
          float ucon[C];
          for (int c = 0; c < C; ++c)
            ucon[c] = enforce_constraint(uc[c], cc_.lower[c], cc_.upper[c], cc_.deadband[c], cc_.zero_control[c]);
          euler_step<Model>(dyn_[i], x, ucon, xn, cp_.dt);
        }
        else
        {
          euler_step<Model>(dyn_[i], x, uc, xn, cp_.dt);
        }
        for (int s = 0; s < S; ++s) x[s] = xs[(size_t)(t + 1) * S + s] = xn[s];
      }
      xs += (size_t)T * S;
    }
    traj_dirty_ = false;
  }
  mppi_status get_baseline_normalizer(float* out, double* norm64) override
  {
    if (out) memcpy(out, baseline_norm_.data(), sizeof(float) * 2 * I_);
    if (norm64)
      for (int i = 0; i < I_; ++i) norm64[i] = stats_[3 * i];
    return MPPI_OK;
  }
  mppi_status get_sample_costs(float* out) override { return copy_per_sample(costs_d_.p, out); }
  mppi_status get_sample_weights(float* out) override
  {
    if (weights_stale_)
    {
      // the tiles reduced without materialising the weights: derive them from the costs and the baselines
      weights_from_costs_kernel<<<dim3(std::max(1, std::min(64, (max_k_ + 255) / 256)), I_), 256, 0, stream_>>>(
          inst_d_.p, costs_d_.p, bn_d_.p, 1.0f / cp_.lambda, weights_d_.p);
      MG_CUDA(cudaGetLastError());
      weights_stale_ = false;
    }
    return copy_per_sample(weights_d_.p, out);
  }
  mppi_status get_control_samples(float* out) override
  {
    MG_CHECK(out, "out must not be NULL");
    MG_CUDA(cudaStreamSynchronize(stream_));
    size_t o = 0;
    for (int i = 0; i < I_; ++i)
    {
      const size_t n = (size_t)K_[i] * T_[i] * C;
      MG_CUDA(cudaMemcpy(out + o, samples_d_.p + u_off_[i], n * sizeof(float), cudaMemcpyDeviceToHost));
      o += n;
    }
    return MPPI_OK;
  }
  // VanillaMPPIController::calculateSampledStateTrajectories (visualizeKernel, mppi_common.cu:371-533): samples idx
  // of instance i of the last solve, re-rolled on the GPU.  The likelihood-ratio term uses the nominal sequence the
  // solve started from (the samples' own nominal when num_iters is 1).
  mppi_status get_sampled_trajectories(int i, const int* idx, int n, float* states, float* step_costs,
                                       float* terminal, int* crash) override
  {
    MG_CHECK(i >= 0 && i < I_, "instance %d out of range", i);
    MG_CHECK(n >= 0, "n must be >= 0");
    if (n == 0) return MPPI_OK;
    MG_CHECK(idx && states && step_costs && terminal, "pointers must not be NULL");
    for (int j = 0; j < n; ++j)
      MG_CHECK(idx[j] >= 0 && idx[j] < K_[i], "sample index %d (entry %d) is out of range", idx[j], j);
    if constexpr (Model::kMlp)
    {
      set_error("sampled trajectories are re-rolled with an analytic model; the surrogate model has none here");
      return MPPI_EUNSUPPORTED;
    }
    else
    {
      const int T = T_[i];
      constexpr int SO = Model::kPlugin ? Model::OUTPUT_DIM : S;  // plugins report outputs, the others states
      DevBuf<int> idx_d, crash_d;
      DevBuf<float> st_d, c_d, term_d, mean0_d;
      MG_TRY(idx_d.alloc(n));
      MG_TRY(crash_d.alloc((size_t)n * T));
      MG_TRY(st_d.alloc((size_t)n * T * SO));
      MG_TRY(c_d.alloc((size_t)n * T));
      MG_TRY(term_d.alloc(n));
      MG_TRY(mean0_d.alloc(control_.size()));
      MG_CUDA(cudaStreamSynchronize(stream_));
      MG_CUDA(cudaMemcpy(idx_d.p, idx, sizeof(int) * n, cudaMemcpyHostToDevice));
      MG_CUDA(cudaMemcpy(mean0_d.p, mean_h_.p, sizeof(float) * control_.size(), cudaMemcpyHostToDevice));
      RolloutArgs<Model> a = base_rollout_args();
      a.mean = mean0_d.p;
      if constexpr (Model::kPlugin)
      {
        sampled_trajectories_plugin_kernel<Model><<<(n + 127) / 128, 128, 0, stream_>>>(
            a, i, idx_d.p, n, st_d.p, c_d.p, term_d.p, crash_d.p);
      }
      else
      {
        // the built-in costs never set a crash flag
        MG_CUDA(cudaMemsetAsync(crash_d.p, 0, sizeof(int) * (size_t)n * T, stream_));
        sampled_trajectories_kernel<Model><<<(n + 127) / 128, 128, 0, stream_>>>(a, i, idx_d.p, n, st_d.p, c_d.p,
                                                                                   term_d.p);
      }
      MG_CUDA(cudaGetLastError());
      MG_CUDA(cudaStreamSynchronize(stream_));
      MG_CUDA(cudaMemcpy(states, st_d.p, sizeof(float) * n * T * SO, cudaMemcpyDeviceToHost));
      if (crash) MG_CUDA(cudaMemcpy(crash, crash_d.p, sizeof(int) * n * T, cudaMemcpyDeviceToHost));
      MG_CUDA(cudaMemcpy(step_costs, c_d.p, sizeof(float) * n * T, cudaMemcpyDeviceToHost));
      MG_CUDA(cudaMemcpy(terminal, term_d.p, sizeof(float) * n, cudaMemcpyDeviceToHost));
      return MPPI_OK;
    }
  }
  // computeFreeEnergy (mppi_common.cu:1101-1117) from the device sums of w and w^2.
  mppi_status get_free_energy(int i, float* out6) override
  {
    MG_CHECK(i >= 0 && i < I_, "instance %d out of range", i);
    MG_CHECK(out6, "out must not be NULL");
    const float lambda = cp_.lambda;
    const int K = K_[i];
    const float norm = (float)(stats_[3 * i] / K);
    const float var = (float)stats_[3 * i + 1];
    const float baseline = baseline_norm_[2 * i];
    const float fe = -lambda * logf(norm) + baseline;
    const float fe_var = lambda * (var / K - norm * norm);
    const float weird = fe_var / (norm * sqrtf(1.0f * K));
    out6[0] = fe;
    out6[1] = fe_var;
    out6[2] = lambda * (weird + 0.5f * weird * weird);
    out6[3] = baseline_norm_[2 * i + 1] / (float)K;
    out6[4] = baseline - prev_baseline_[i];
    out6[5] = prev_baseline_[i];
    return MPPI_OK;
  }

  // One parameter block for every instance, or one block per instance (bytes = I * block).
  template <class P>
  mppi_status replace_params(std::vector<P>& host, P* dev, const void* p, size_t bytes, const char* what)
  {
    MG_CHECK(p && (bytes == sizeof(P) || bytes == sizeof(P) * I_),
             "%s parameters must be one %zu-byte block (all instances) or %d of them (one per instance)", what,
             sizeof(P), I_);
    if (bytes == sizeof(P))
      for (int i = 0; i < I_; ++i) memcpy(&host[i], p, sizeof(P));
    else
      memcpy(host.data(), p, sizeof(P) * I_);
    MG_CUDA(cudaMemcpyAsync(dev, host.data(), sizeof(P) * I_, cudaMemcpyHostToDevice, stream_));
    MG_CUDA(cudaStreamSynchronize(stream_));
    return MPPI_OK;
  }
  mppi_status set_dynamics_params(const void* p, size_t bytes) override
  {
    return replace_params(dyn_, dyn_d_.p, p, bytes, "dynamics");
  }
  mppi_status set_cost_params(const void* p, size_t bytes) override
  {
    return replace_params(cost_, cost_d_.p, p, bytes, "cost");
  }
  mppi_status set_sampling_params(const mppi_sampling_params* sp) override
  {
    MG_CHECK(sp, "sampling params must not be NULL");
    MG_TRY(check_sampling(*sp));
    const bool kind_changed = sp->kind != sp_.kind;
    if (kind_changed) injected_d_.reset();
    sp_ = *sp;
    if (kind_changed) MG_TRY(build_work_lists());  // the rollout kernel (fused or not) and its grid follow the kind
    MG_TRY(refresh_noise_sources());
    MG_TRY(build_colored_tables());
    invalidate_graphs();
    return MPPI_OK;
  }
  mppi_status set_controller_params(const mppi_controller_params* cp) override
  {
    MG_CHECK(cp, "controller params must not be NULL");
    MG_TRY(check_controller(*cp));
    const bool tile_reduce_before = tile_reduce_active();
    const bool was_rmppi = rmppi();
    cp_ = *cp;
    if (rmppi() && !was_rmppi)
    {
      // RobustMPPIController's constructor turns its feedback on (robust_mppi_controller.cu:37-43)
      fb_enabled_ = true;
      std::fill(fb_gains_.begin(), fb_gains_.end(), 0.0f);
    }
    if (tile_reduce_active() != tile_reduce_before)
    {
      // the weight path changed: mode 4 needs the tile reduction, and the rollout's shared memory follows it
      if (rollout_mode_ == 4 && !noise_warps_available()) rollout_mode_ = 0;
      MG_TRY(build_work_lists());
    }
    MG_TRY(refresh_noise_sources());
    invalidate_graphs();
    return MPPI_OK;
  }
  mppi_status check_controller(const mppi_controller_params& cp) const
  {
    MG_CHECK(cp.num_iters >= 1, "num_iters must be >= 1");
    MG_CHECK(cp.lambda > 0.0f && std::isfinite(cp.lambda), "lambda must be positive");
    MG_CHECK(std::isfinite(cp.dt), "dt must be finite");
    MG_CHECK(cp.controller == MPPI_CONTROLLER_VANILLA || cp.controller == MPPI_CONTROLLER_COLORED ||
                 cp.controller == MPPI_CONTROLLER_TUBE || cp.controller == MPPI_CONTROLLER_RMPPI,
             "controller must be MPPI_CONTROLLER_VANILLA (0), MPPI_CONTROLLER_COLORED (1), MPPI_CONTROLLER_TUBE (2) "
             "or MPPI_CONTROLLER_RMPPI (3)");
    MG_CHECK(std::isfinite(cp.nominal_threshold), "nominal_threshold must be finite");
    if (cp.controller == MPPI_CONTROLLER_TUBE && !K_.empty())
      MG_CHECK(I_ == 2 && K_[0] == K_[1] && T_[0] == T_[1],
               "a Tube-MPPI handle holds two instances of equal num_rollouts and num_timesteps (actual, nominal)");
    if (cp.controller == MPPI_CONTROLLER_RMPPI)
    {
      MG_CHECK(!Model::kMlp, "R-MPPI runs analytic models (the built-in ones and plugins)");
      MG_CHECK(std::isfinite(cp.value_function_threshold), "value_function_threshold must be finite");
      // RobustMPPIController::updateNumCandidates (robust_mppi_controller.cu:424-457)
      MG_CHECK(cp.num_candidate_nominal_states >= 3 && cp.num_candidate_nominal_states % 2 == 1,
               "num_candidate_nominal_states must be odd and >= 3 (got %d)", cp.num_candidate_nominal_states);
      MG_CHECK(cp.num_eval_samples_per_candidate >= 1, "num_eval_samples_per_candidate must be >= 1");
      if (!K_.empty())
      {
        MG_CHECK(I_ == 2 && K_[0] == K_[1] && T_[0] == T_[1] && T_[0] >= 2,
                 "an R-MPPI handle holds two instances of equal num_rollouts and num_timesteps >= 2 (nominal, real)");
        MG_CHECK((long long)cp.num_candidate_nominal_states * cp.num_eval_samples_per_candidate <= K_[0],
                 "num_candidate_nominal_states x num_eval_samples_per_candidate must not exceed num_rollouts");
        MG_CHECK(sp_.kind == MPPI_SAMPLER_GAUSSIAN, "R-MPPI samples Gaussian noise");
      }
    }
    MG_CHECK(std::isfinite(cp.tsallis_gamma) && std::isfinite(cp.tsallis_r), "tsallis_gamma and tsallis_r must be "
             "finite");
    MG_CHECK(cp.controller != MPPI_CONTROLLER_COLORED || cp.tsallis_gamma == 0.0f || cp.tsallis_r != 1.0f,
             "tsallis_r = 1 makes the Tsallis exponent 1 / (r - 1) infinite");
    for (int i = 0; i < S; ++i)
      MG_CHECK(std::isfinite(cp.state_leash_dist[i]) && cp.state_leash_dist[i] >= 0.0f,
               "state_leash_dist[%d] must be finite and >= 0", i);
    return MPPI_OK;
  }
  mppi_status set_costmap(const float* map, int w, int h, float res, float ox, float oy) override
  {
    MG_CHECK(map && w >= 2 && h >= 2 && res > 0.0f, "costmap needs data, width/height >= 2 and resolution > 0");
    MG_TRY(costmap_d_.alloc((size_t)w * h));
    MG_CUDA(cudaMemcpy(costmap_d_.p, map, sizeof(float) * w * h, cudaMemcpyHostToDevice));
    aux_.map = CostmapView{ costmap_d_.p, w, h, 1.0f / res, res, ox, oy };
    invalidate_graphs();
    return MPPI_OK;
  }

  mppi_status inject_noise(const float* noise, size_t count) override
  {
    if (!noise)
    {
      injected_d_.reset();
      invalidate_graphs();
      return MPPI_OK;
    }
    const bool colored = sp_.kind == MPPI_SAMPLER_COLORED_NOISE;
    size_t need = 0;
    for (int i = 0; i < I_; ++i)
      need += colored ? (size_t)K_[i] * C * (T_[i] + 1) * 2 : (size_t)K_[i] * T_[i] * C;
    MG_CHECK(count == need, "injected noise has %zu floats, expected %zu", count, need);
    for (size_t j = 0; j < count; ++j)
      if (!std::isfinite(noise[j]))
      {
        set_error("injected noise has a non-finite entry at index %zu", j);
        return MPPI_ENAN;
      }
    if (colored)
    {
      // spectrum layout [K][C][F][2] per instance, instances concatenated (spec_off)
      MG_TRY(injected_d_.alloc(count));
      MG_CUDA(cudaMemcpy(injected_d_.p, noise, count * sizeof(float), cudaMemcpyHostToDevice));
    }
    else
    {
      MG_TRY(injected_d_.alloc(samples_d_.n));
      size_t o = 0;
      for (int i = 0; i < I_; ++i)
      {
        const size_t n = (size_t)K_[i] * T_[i] * C;
        MG_CUDA(cudaMemcpy(injected_d_.p + u_off_[i], noise + o, n * sizeof(float), cudaMemcpyHostToDevice));
        o += n;
      }
    }
    invalidate_graphs();
    return MPPI_OK;
  }

  mppi_status generate_samples(int stride, int iter) override
  {
    MG_CHECK(stride >= 0 && iter >= 0, "stride and iteration must be >= 0");
    memcpy(mean_h_.p, control_.data(), sizeof(float) * control_.size());
    MG_CUDA(cudaMemcpyAsync(mean_d_.p, mean_h_.p, sizeof(float) * control_.size(), cudaMemcpyHostToDevice, stream_));
    MG_TRY(launch_sampler(stride, iter));
    bump_counter_kernel<<<1, 1, 0, stream_>>>(counters_d_.p + 3);
    MG_CUDA(cudaGetLastError());
    MG_CUDA(cudaStreamSynchronize(stream_));
    return MPPI_OK;
  }

  mppi_status set_graph_mode(int enable) override
  {
    graph_mode_ = enable != 0;
    return MPPI_OK;
  }
  // The split rollout needs the fused Gaussian sampler (whole quads per row), an analytic model, and room for the
  // stepped states of every sample (at most 256 MB).
  bool split_available() const
  {
    if (!fusable() || (Model::kMlp && !use_analytic_)) return false;
    return (double)total_u_ / C * S * sizeof(float) <= 256.0 * 1024 * 1024;
  }
  // The cooperative rollout (four lanes per sample) needs the fused Gaussian sampler and an analytic model.
  bool coop_available() const { return fusable() && !(Model::kMlp && !use_analytic_); }
  // Mode 3 runs the Gaussian sampler as its own kernel and the rollout on the written samples (for the surrogate:
  // the tensor-core rollout reading its controls from memory instead of drawing them).
  bool unfused_available() const { return fusable(); }
  // Mode 4 is the fused rollout with noise warps; it reads its controls from the shared-memory stage, so the longest
  // horizon must fit the stage of the smallest tile (tile sizes whose stage does not fit run mode 0's kernel).
  bool noise_warps_available() const
  {
    return fusable() && tile_reduce_active() && fused_stage_bytes_max<32>() != 0;
  }
  int rollout_modes() const override
  {
    return 1 | (split_available() ? 2 : 0) | (coop_available() ? 4 : 0) | (unfused_available() ? 8 : 0) |
           (noise_warps_available() ? 16 : 0);
  }
  int rollout_mode() const override { return rollout_mode_; }
  mppi_status set_rollout_mode(int mode) override
  {
    MG_CHECK(mode >= 0 && mode <= 4, "rollout mode must be 0 (fused), 1 (split dynamics / cost), 2 (cooperative), "
             "3 (sampler kernel, then the staged rollout) or 4 (fused with noise warps)");
    MG_CHECK(mode != 1 || split_available(),
             "the split rollout needs Gaussian sampling, T*C %% 4 == 0, an analytic model and <= 256 MB of states");
    MG_CHECK(mode != 2 || coop_available(), "the cooperative rollout needs Gaussian sampling, T*C %% 4 == 0 and an "
             "analytic model");
    MG_CHECK(mode != 3 || unfused_available(), "rollout mode 3 needs Gaussian sampling and T*C %% 4 == 0");
    MG_CHECK(mode != 4 || noise_warps_available(), "rollout mode 4 needs Gaussian sampling, T*C %% 4 == 0, an analytic "
             "model and a horizon whose controls fit the shared-memory stage");
    if (mode == 1 && !states_d_.p) MG_TRY(states_d_.alloc((size_t)total_u_ / C * S));
    rollout_mode_ = mode;
    split_ = mode == 1;
    MG_TRY(build_work_lists());  // the rollout grid follows the kernel's occupancy
    invalidate_graphs();
    return MPPI_OK;
  }
  mppi_status get_launch_config(int* ns, int* tch, int* kc) const override
  {
    if (ns) *ns = ns_;
    if (tch) *tch = tch_for(ns_);
    if (kc) *kc = kc_;
    return MPPI_OK;
  }
  mppi_status set_launch_config(int ns, int tch, int kc) override
  {
    MG_CHECK(ns == 32 || ns == 64 || ns == 128 || ns == 256, "rollout samples per CTA must be 32, 64, 128 or 256");
    if (Model::kMlp) ns = kMlpSamplesPerCta;  // the surrogate rollout's work items are fixed
    MG_CHECK(kc >= 32 && kc <= 256 && (kc % 32) == 0, "reduction samples per CTA must be a multiple of 32 in [32, 256]");
    (void)tch;
    ns_ = ns;
    kc_ = kc;
    MG_TRY(build_work_lists());
    invalidate_graphs();
    return MPPI_OK;
  }
  mppi_status autotune(const char* cache_path) override;

  // Surrogate weights for the MLP model (ignored by analytic models): host FP32 copy for the nominal trajectory,
  // device FP32 copy the rollout kernel converts to BF16 tensor-core operands.
  mppi_status set_mlp(const float* params, size_t n, int precision) override
  {
    if constexpr (!Model::kMlp)
    {
      set_error("this handle's model has no learned surrogate");
      return MPPI_EUNSUPPORTED;
    }
    else
      return set_mlp_impl(params, n, precision);
  }
  mppi_status set_mlp_impl(const float* params, size_t n, int precision)
  {
    MG_CHECK(params && n == (size_t)MPPI_MLP_PARAMS, "the MLP parameter vector holds %d floats", MPPI_MLP_PARAMS);
    MG_CHECK(precision >= 0 && precision <= 2, "MLP precision must be 0 (bf16), 1 (fp8 e4m3) or 2 (fp32)");
    for (size_t i = 0; i < n; ++i) MG_CHECK(std::isfinite(params[i]), "MLP parameter %zu is not finite", i);
    for (int i = 0; i < kMlpIn; ++i) MG_CHECK(params[kMlpInStd + i] > 0.0f, "MLP input scale %d must be positive", i);
    std::vector<float> dev(kMlpDevParams);
    mlp_host_.resize(kMlpNumParams);
    mlp_prepare(params, precision, dev.data(), mlp_host_.data());
    mlp_precision_ = precision;
    MG_TRY(mlp_d_.alloc(kMlpDevParams));
    MG_CUDA(cudaMemcpy(mlp_d_.p, dev.data(), sizeof(float) * kMlpDevParams, cudaMemcpyHostToDevice));
    invalidate_graphs();
    return MPPI_OK;
  }

  mppi_status set_judge(float fraction) override
  {
    if constexpr (!Model::kMlp)
    {
      set_error("the analytic judge applies to the surrogate model only");
      return MPPI_EINVAL;
    }
    else
    {
      MG_CHECK(std::isfinite(fraction) && fraction >= 0.0f && fraction <= 1.0f, "judge fraction must be in [0, 1]");
      judge_frac_ = fraction;
      MG_TRY(build_judge_lists());
      invalidate_graphs();
      return MPPI_OK;
    }
  }

  mppi_status get_judge_stats(float* out) override
  {
    MG_CHECK(out, "out must not be NULL");
    if (Model::kMlp && judge_total_ > 0 && !use_analytic_)
    {
      MG_CUDA(cudaStreamSynchronize(stream_));
      MG_CUDA(cudaMemcpy(out, judge_stats_d_.p, sizeof(float) * 2 * I_, cudaMemcpyDeviceToHost));
      return MPPI_OK;
    }
    std::fill(out, out + 2 * I_, 0.0f);
    return MPPI_OK;
  }

  mppi_status use_analytic(int enable) override
  {
    if constexpr (!Model::kMlp)
    {
      set_error("only the surrogate model has an analytic fallback");
      return MPPI_EINVAL;
    }
    else
    {
      use_analytic_ = enable != 0;
      MG_TRY(build_work_lists());  // the rollout kernel, and so its grid, changes
      invalidate_graphs();
      return MPPI_OK;
    }
  }

  // Diagnostics: the bound of rollout mode 4's progress-word poll (0 restores the default) and whether its noise
  // warps withhold their progress (so the rollout warps' bounded wait runs out).
  mppi_status set_wait_diagnostics(uint32_t max_polls, int withhold_progress) override
  {
    max_polls_ = max_polls ? max_polls : kMaxProgressPolls;
    withhold_progress_ = withhold_progress != 0;
    invalidate_graphs();
    return MPPI_OK;
  }

  // ------------------------------------------------------------------------------------------ DDP feedback
  // The instance whose nominal trajectory the feedback tracks: Tube-MPPI's nominal system (its getControlSeq and
  // getTargetStateSeq, tube_mppi_controller.cuh:61-72), R-MPPI's nominal system (instance 0), else the handle's single
  // controller.
  int fb_instance() const { return tube() ? 1 : 0; }
  size_t state_off(int i) const
  {
    size_t off = 0;
    for (int j = 0; j < i; ++j) off += (size_t)T_[j] * S;
    return off;
  }

  // xdot of instance i's model on the host, the function the solver linearises (ModelWrapperDDP::f,
  // ddp_model_wrapper.h:66-79: the derivative the model's step computes)
  void host_xdot(int i, const float* x, const float* u, float* xd) const
  {
    if constexpr (Model::kPlugin)
    {
      float xn[S], y[Model::OUTPUT_DIM];
      dyn_[i].step(x, xn, xd, u, y, 0, cp_.dt);
    }
    else if constexpr (Model::kMlp)
    {
      if (!use_analytic_)
        mlp_host_dynamics(mlp_host_.data(), x, u, xd);
      else
        Model::computeDynamics(dyn_[i], x, u, xd);
    }
    else
    {
      Model::computeDynamics(dyn_[i], x, u, xd);
    }
  }

  // d xdot / dx and d xdot / du (row-major, zeroed by the caller): the model's analytic computeGrad where it has one,
  // else forward differences (ModelWrapperDDP::df, ddp_model_wrapper.h:81-94)
  void host_jacobian(int i, const float* x, const float* u, double* A, double* B) const
  {
    if constexpr (Model::kPlugin)
    {
      if constexpr (DefinesComputeGrad<typename Model::DynParams>::value)
      {
        float Af[S * S] = {}, Bf[S * C] = {};
        if (dyn_[i].computeGrad(x, u, Af, Bf))
        {
          for (int e = 0; e < S * S; ++e) A[e] = Af[e];
          for (int e = 0; e < S * C; ++e) B[e] = Bf[e];
          return;
        }
      }
    }
    else if constexpr (HasAnalyticGrad<Model>::value)
    {
      if (!(Model::kMlp && !use_analytic_) && Model::computeGrad(dyn_[i], x, u, A, B)) return;
    }
    numeric_jacobian<S, C>([&](const float* xx, const float* uu, float* xd) { host_xdot(i, xx, uu, xd); }, x, u, A,
                           B);
  }

  mppi_status feedback_shape_ok() const
  {
    MG_CHECK(I_ == 1 || tube() || rmppi(),
             "the feedback controller serves a single controller (or Tube-MPPI's / R-MPPI's nominal system)");
    return MPPI_OK;
  }

  // FeedbackController::setParams with DDPParams (ddp.cu:81-87): NULL keeps a matrix
  mppi_status set_feedback_params(const float* Q, const float* Qf, const float* R, int iterations) override
  {
    MG_CHECK(iterations >= 1, "num_iterations must be >= 1 (got %d)", iterations);
    auto load = [](std::vector<double>& dst, const float* src, int n) {
      if (!src) return true;
      for (int e = 0; e < n; ++e)
        if (!std::isfinite(src[e])) return false;
      for (int e = 0; e < n; ++e) dst[e] = src[e];
      return true;
    };
    std::vector<double> q = fb_w_.Q, qf = fb_w_.Qf, r = fb_w_.R;
    MG_CHECK(load(q, Q, S * S) && load(qf, Qf, S * S) && load(r, R, C * C), "feedback weights must be finite");
    fb_w_.Q.swap(q);
    fb_w_.Qf.swap(qf);
    fb_w_.R.swap(r);
    fb_w_.iterations = iterations;
    return MPPI_OK;
  }

  // Controller::initFeedback (controller.cuh:265-269: on, gains reset to zero by initTrackingController) and
  // disableFeedbackController (:730-733)
  mppi_status enable_feedback(int enable) override
  {
    MG_TRY(feedback_shape_ok());
    fb_enabled_ = enable != 0;
    if (fb_enabled_) std::fill(fb_gains_.begin(), fb_gains_.end(), 0.0f);
    return MPPI_OK;
  }
  int feedback_enabled() const override { return fb_enabled_ ? 1 : 0; }

  // Controller::computeFeedback(state) (controller.cuh:551-565): DDP from x0 around getTargetStateSeq() and
  // getControlSeq(); nothing while feedback is off
  mppi_status compute_feedback(const float* x0) override
  {
    MG_CHECK(x0, "state must not be NULL");
    MG_TRY(feedback_shape_ok());
    // RobustMPPIController::computeFeedback does nothing (robust_mppi_controller.cuh:192-196): its gains come with the
    // importance-sampler update
    if (rmppi()) return MPPI_OK;
    return run_feedback(x0);
  }
  mppi_status run_feedback(const float* x0)
  {
    if (!fb_enabled_) return MPPI_OK;
    const int i = fb_instance();
    MG_CHECK(T_[i] >= 2, "the feedback controller needs at least two time steps");
    if (traj_dirty_) compute_state_seq();
    auto f = [&](const float* x, const float* u, float* xd) { host_xdot(i, x, u, xd); };
    auto df = [&](const float* x, const float* u, double* A, double* B) { host_jacobian(i, x, u, A, B); };
    const bool ok = ddp_tracking_gains<S, C>(f, df, x0, state_seq_.data() + state_off(i), control_.data() + t_off_[i],
                                             T_[i], cp_.dt, fb_w_, cc_.lower, cc_.upper, fb_gains_.data());
    MG_CHECK(ok, "DDP feedback: a control Hessian is not positive definite (check R)");
    return MPPI_OK;
  }

  mppi_status get_feedback_gains(float* out) const override
  {
    MG_CHECK(out, "out must not be NULL");
    memcpy(out, fb_gains_.data(), sizeof(float) * fb_gains_.size());
    return MPPI_OK;
  }

  // Controller::getFeedbackControl (controller.cuh:567-571): K_t (x - goal)
  mppi_status feedback_control(const float* x, const float* goal, int t, float* u) const override
  {
    MG_CHECK(x && goal && u, "state, goal_state and out must not be NULL");
    const int T = T_[fb_instance()];
    MG_CHECK(t >= 0 && t < T, "t must be in [0, %d) (got %d)", T, t);
    ddp_feedback_control<S, C>(fb_gains_.data(), t, x, goal, u);
    return MPPI_OK;
  }

  // Controller::computeFeedbackPropagatedStateSeq (controller.cuh:495-517): from the state the last solve started
  // at, each step's control is the nominal control plus the feedback against that step's target state, stepped by
  // the model without constraints; with feedback off the previous result stays
  mppi_status feedback_propagated_state_seq(float* out) override
  {
    MG_TRY(feedback_shape_ok());
    if (fb_enabled_)
    {
      if (traj_dirty_) compute_state_seq();
      const int i = fb_instance(), T = T_[i];
      const float* xt = state_seq_.data() + state_off(i);
      const float* un = control_.data() + t_off_[i];
      float x[S], xn[S], u[C], ufb[C];
      for (int s = 0; s < S; ++s) x[s] = fb_prop_[s] = state_seq_[s];  // actual state sequence, column 0
      for (int t = 0; t < T - 1; ++t)
      {
        ddp_feedback_control<S, C>(fb_gains_.data(), t, x, xt + (size_t)t * S, ufb);
        for (int c = 0; c < C; ++c) u[c] = un[(size_t)t * C + c] + ufb[c];
        model_step(i, x, u, xn, t);
        for (int s = 0; s < S; ++s) x[s] = fb_prop_[(size_t)(t + 1) * S + s] = xn[s];
      }
    }
    if (out) memcpy(out, fb_prop_.data(), sizeof(float) * fb_prop_.size());
    return MPPI_OK;
  }

  // ------------------------------------------------------------------------------------------------ R-MPPI
  bool rmppi() const { return cp_.controller == MPPI_CONTROLLER_RMPPI; }

  // RobustMPPIController::computeLineSearchWeights (robust_mppi_controller.cu:480-498): column i of the 3 x N weights
  // (row-major here) mixes the nominal trajectory's first state, its second state and the real state
  void line_search_weights(std::vector<float>& w) const
  {
    const int N = cp_.num_candidate_nominal_states, h = N / 2;
    w.assign((size_t)3 * N, 0.0f);
    for (int i = 0; i < h + 1; ++i)
    {
      w[i] = 1 - i / float(h);
      w[N + i] = i / float(h);
      w[2 * N + i] = 0.0f;
    }
    for (int i = 1; i < h + 1; ++i)
    {
      w[h + i] = 0.0f;
      w[N + h + i] = 1 - i / float(h);
      w[2 * N + h + i] = i / float(h);
    }
  }

  mppi_status launch_rmppi_rollout()
  {
    MG_CHECK(fb_gains_d_.p != nullptr, "the R-MPPI rollout needs a solve first (mppi_compute_control uploads its gains)");
    RmppiArgs<Model> a{};
    a.inst = inst_d_.p;
    a.samples = samples_d_.p;
    a.mean = mean_d_.p;
    a.x0 = x0_d_.p;
    a.gains = fb_gains_d_.p;
    a.costs = costs_d_.p;
    a.baseline_bits = baseline_bits_d_.p;
    a.dyn = dyn_d_.p;
    a.cost = cost_d_.p;
    a.aux = aux_;
    a.sh = make_sample_shared(sp_, cc_);  // the real constraints (the samples came unconstrained)
    a.lambda = cp_.lambda;
    a.alpha = cp_.alpha;
    a.dt = cp_.dt;
    a.value_threshold = cp_.value_function_threshold;
    a.use_likelihood = 0;
    for (int c = 0; c < C; ++c)
      if (sp_.control_cost_coeff[c] != 0.0f) a.use_likelihood = 1;
    // two lanes per sample (nominal, real)
    rmppi_rollout_kernel<Model><<<(2 * K_[0] + 127) / 128, 128, 0, stream_>>>(a);
    MG_CUDA(cudaGetLastError());
    return MPPI_OK;
  }

  // RobustMPPIController::computeControl (robust_mppi_controller.cu:635-744): per iteration one graph launch of the
  // device work of both distributions (samples around the nominal sequence, the coupled rollout, weights and update);
  // the iteration's nominal sequence is the next iteration's importance sampler.  Both sequences are smoothed at the
  // end and the nominal state trajectory is recomputed.  x is the real system's state.
  mppi_status compute_control_rmppi(const float* x, int stride)
  {
    if constexpr (Model::kMlp)
    {
      set_error("R-MPPI runs analytic models (the built-in ones and plugins)");
      return MPPI_EUNSUPPORTED;
    }
    for (int i = 0; i < S; ++i)
      if (!std::isfinite(x[i]))
      {
        set_error("initial state has a non-finite entry at index %d", i);
        return MPPI_ENAN;
      }
    MG_CHECK(!Model::kNeedsCostmap || aux_.map.data != nullptr, "this model needs a costmap (mppi_set_costmap)");
    if (!nominal_init_) nominal_x0_.assign(S, 0.0f);  // nominal_state_ before the first importance-sampler update
    if (!fb_gains_d_.p) MG_TRY(fb_gains_d_.alloc(fb_gains_.size()));
    MG_CUDA(cudaMemcpyAsync(fb_gains_d_.p, fb_gains_.data(), sizeof(float) * fb_gains_.size(), cudaMemcpyHostToDevice,
                            stream_));
    for (int i = 0; i < I_; ++i) prev_baseline_[i] = baseline_norm_[2 * i];
    const size_t tc = (size_t)T_[0] * C;
    for (int it = 0; it < cp_.num_iters; ++it)
    {
      memcpy(x0_h_.p, nominal_x0_.data(), sizeof(float) * S);
      memcpy(x0_h_.p + S, x, sizeof(float) * S);
      memcpy(mean_h_.p + t_off_[0], control_.data() + t_off_[0], sizeof(float) * tc);
      memcpy(mean_h_.p + t_off_[1], control_.data() + t_off_[0], sizeof(float) * tc);
      host_iter_ = it;
      const mppi_status st = launch_host_iteration(stride);
      host_iter_ = 0;
      MG_TRY(st);
      MG_CUDA(cudaStreamSynchronize(stream_));
      memcpy(control_.data(), out_mean_h_.p, sizeof(float) * control_.size());
      memcpy(baseline_norm_.data(), out_bn_h_.p, sizeof(float) * 2 * I_);
      memcpy(stats_.data(), out_stats_h_.p, sizeof(double) * 3 * I_);
    }
    smooth_host(control_.data() + t_off_[0], T_[0]);
    smooth_host(control_.data() + t_off_[1], T_[1]);
    state_trajectory(0, nominal_x0_.data(), control_.data() + t_off_[0], state_seq_.data());
    state_trajectory(1, x, control_.data() + t_off_[1], state_seq_.data() + (size_t)T_[0] * S);
    traj_dirty_ = false;
    for (int i = 0; i < I_; ++i)
      if (!std::isfinite(baseline_norm_[2 * i]) || !(stats_[3 * i] > 0.0))
      {
        set_error("a sampled cost or the normaliser is not finite (NaN state or noise?)");
        return MPPI_ENAN;
      }
    return MPPI_OK;
  }

  // RobustMPPIController::updateImportanceSamplingControl (robust_mppi_controller.cu:548-627)
  mppi_status rmppi_update_importance_sampler(const float* x, int stride) override
  {
    MG_CHECK(rmppi(), "mppi_rmppi_update_importance_sampler needs an R-MPPI handle");
    MG_CHECK(x, "state must not be NULL");
    MG_CHECK(stride >= 0, "optimization_stride must be >= 0");
    for (int i = 0; i < S; ++i)
      if (!std::isfinite(x[i]))
      {
        set_error("state has a non-finite entry at index %d", i);
        return MPPI_ENAN;
      }
    if constexpr (Model::kMlp)
    {
      set_error("R-MPPI runs analytic models (the built-in ones and plugins)");
      return MPPI_EUNSUPPORTED;
    }
    else
    {
      MG_CHECK(!Model::kNeedsCostmap || aux_.map.data != nullptr, "this model needs a costmap (mppi_set_costmap)");
      const int N = cp_.num_candidate_nominal_states, J = cp_.num_eval_samples_per_candidate;
      if (!nominal_init_)
      {
        // computeNominalStateAndStride (:571-578): the first state is the nominal state
        nominal_x0_.assign(x, x + S);
        nominal_init_ = true;
        rm_nominal_stride_ = 0;
      }
      else
      {
        // candidates on the lines nominal x_0 -> nominal x_1 -> real state (getInitNominalStateCandidates, :351-363)
        // with their strides round((0, stride, stride) . w_i) (computeImportanceSamplerStride, :500-511)
        const float* p0 = state_seq_.data();
        const float* p1 = p0 + S;
        std::vector<float> w;
        line_search_weights(w);
        rm_cand_.assign((size_t)N * S, 0.0f);
        rm_strides_.assign(N, 0);
        const float sf = (float)stride;
        for (int i = 0; i < N; ++i)
        {
          for (int s = 0; s < S; ++s) rm_cand_[(size_t)i * S + s] = (p0[s] * w[i] + p1[s] * w[N + i]) + x[s] * w[2 * N + i];
          rm_strides_[i] = (int)std::round((0.0f * w[i] + sf * w[N + i]) + sf * w[2 * N + i]);
        }
        // the nominal distribution's samples around the nominal sequence (copyNominalControlToDevice,
        // generateSamples), then initEvalKernel
        const size_t tc = (size_t)T_[0] * C;
        memcpy(mean_h_.p + t_off_[0], control_.data() + t_off_[0], sizeof(float) * tc);
        memcpy(mean_h_.p + t_off_[1], control_.data() + t_off_[0], sizeof(float) * tc);
        MG_CUDA(cudaMemcpyAsync(mean_d_.p, mean_h_.p, sizeof(float) * control_.size(), cudaMemcpyHostToDevice, stream_));
        if (rm_cand_d_.n < (size_t)N * S) MG_TRY(rm_cand_d_.alloc((size_t)N * S));
        if (rm_strides_d_.n < (size_t)N) MG_TRY(rm_strides_d_.alloc(N));
        if (rm_eval_d_.n < (size_t)N * J) MG_TRY(rm_eval_d_.alloc((size_t)N * J));
        MG_CUDA(cudaMemcpyAsync(rm_cand_d_.p, rm_cand_.data(), sizeof(float) * N * S, cudaMemcpyHostToDevice, stream_));
        MG_CUDA(cudaMemcpyAsync(rm_strides_d_.p, rm_strides_.data(), sizeof(int) * N, cudaMemcpyHostToDevice, stream_));
        MG_TRY(launch_sampler(stride, 0));
        RmppiEvalArgs<Model> e{};
        e.d = inst_h_[0];
        e.samples = samples_d_.p;
        e.mean = mean_d_.p;
        e.cand_states = rm_cand_d_.p;
        e.cand_strides = rm_strides_d_.p;
        e.num_cand = N;
        e.per_cand = J;
        e.costs = rm_eval_d_.p;
        e.dyn = dyn_d_.p;
        e.cost = cost_d_.p;
        e.aux = aux_;
        e.sh = make_sample_shared(sp_, cc_);
        e.lambda = cp_.lambda;
        e.alpha = cp_.alpha;
        e.dt = cp_.dt;
        e.use_likelihood = 0;
        for (int c = 0; c < C; ++c)
          if (sp_.control_cost_coeff[c] != 0.0f) e.use_likelihood = 1;
        rmppi_eval_kernel<Model><<<(N * J + 63) / 64, 64, 0, stream_>>>(e);
        MG_CUDA(cudaGetLastError());
        bump_u32_kernel<<<1, 1, 0, stream_>>>(counters_d_.p + 3);  // the solve draws fresh noise
        MG_CUDA(cudaGetLastError());
        rm_eval_.assign((size_t)N * J, 0.0f);
        MG_CUDA(cudaMemcpyAsync(rm_eval_.data(), rm_eval_d_.p, sizeof(float) * N * J, cudaMemcpyDeviceToHost, stream_));
        MG_CUDA(cudaStreamSynchronize(stream_));
        // computeBestIndex (:527-546): the free energy of each candidate's samples against the smallest evaluated
        // cost; the last candidate below the threshold wins (the previous choice stays when none is)
        float baseline = rm_eval_[0];
        for (int g = 1; g < N * J; ++g)
          if (rm_eval_[g] < baseline) baseline = rm_eval_[g];
        rm_fe_.assign(N, 0.0f);
        for (int i = 0; i < N; ++i)
        {
          float fe = 0.0f;
          for (int j = 0; j < J; ++j)
            fe += expf((float)(-1.0 / (double)cp_.lambda * (double)(rm_eval_[(size_t)i * J + j] - baseline)));
          fe = (float)((double)fe / (1.0 * J));
          fe = -cp_.lambda * logf(fe) + baseline;
          rm_fe_[i] = fe;
          if (fe < cp_.value_function_threshold) rm_best_ = i;
        }
        nominal_used_ = rm_best_;
        rm_nominal_stride_ = rm_strides_[rm_best_];
        nominal_x0_.assign(rm_cand_.begin() + (size_t)rm_best_ * S, rm_cand_.begin() + (size_t)(rm_best_ + 1) * S);
      }
      // the nominal sequence slides by the nominal stride; its state trajectory follows; the feedback gains are
      // computed from the real state around it (computeNominalFeedbackGains, :629-633)
      slide_one(0, rm_nominal_stride_);
      state_trajectory(0, nominal_x0_.data(), control_.data() + t_off_[0], state_seq_.data());
      traj_dirty_ = false;
      MG_TRY(run_feedback(x));
      return MPPI_OK;
    }
  }

  mppi_status rmppi_get_candidates(int* best, int* nominal_stride, float* states, int* strides, float* fe,
                                   float* eval_costs) const override
  {
    MG_CHECK(rmppi(), "mppi_rmppi_get_candidates needs an R-MPPI handle");
    if (best) *best = rm_best_;
    if (nominal_stride) *nominal_stride = rm_nominal_stride_;
    const int N = cp_.num_candidate_nominal_states, J = cp_.num_eval_samples_per_candidate;
    auto copy = [](const auto& v, auto* dst, size_t n) {
      for (size_t e = 0; e < n; ++e) dst[e] = e < v.size() ? v[e] : 0;
    };
    if (states) copy(rm_cand_, states, (size_t)N * S);
    if (strides) copy(rm_strides_, strides, (size_t)N);
    if (fe) copy(rm_fe_, fe, (size_t)N);
    if (eval_costs) copy(rm_eval_, eval_costs, (size_t)N * J);
    return MPPI_OK;
  }

  // ------------------------------------------------------------------------------------------------ Tube-MPPI
  bool tube() const { return cp_.controller == MPPI_CONTROLLER_TUBE; }

  mppi_status nominal_state_used(int* used) override
  {
    MG_CHECK(tube() || rmppi(), "only a Tube-MPPI or R-MPPI handle keeps a nominal system");
    *used = nominal_used_;
    return MPPI_OK;
  }

  // One state step of instance i's model from x with control u (Dynamics::step; no constraint applied).
  void model_step(int i, const float* x, const float* u, float* xn, int t) const
  {
    if constexpr (Model::kPlugin)
    {
      float xd[S], y[Model::OUTPUT_DIM];
      dyn_[i].step(x, xn, xd, u, y, t, cp_.dt);
    }
    else if constexpr (Model::kMlp)
    {
      if (!use_analytic_)
      {
        float xd[S];
        mlp_host_dynamics(mlp_host_.data(), x, u, xd);
        for (int s = 0; s < S; ++s) xn[s] = fmaf(xd[s], cp_.dt, x[s]);
        return;
      }
      euler_step<Model>(dyn_[i], x, u, xn, cp_.dt);
    }
    else
    {
      euler_step<Model>(dyn_[i], x, u, xn, cp_.dt);
    }
  }

  // Controller::computeStateTrajectoryHelper (controller.cuh:645-662): x0, then T-1 steps, each control passed
  // through enforceConstraints first.
  void state_trajectory(int i, const float* x0, const float* u, float* out) const
  {
    const int T = T_[i];
    float x[S], xn[S], uc[C];
    for (int s = 0; s < S; ++s) x[s] = out[s] = x0[s];
    for (int t = 0; t < T - 1; ++t)
    {
      if constexpr (Model::kOwnConstraints)
      {
        for (int c = 0; c < C; ++c) uc[c] = u[(size_t)t * C + c];
        dyn_[i].enforceConstraints(x, uc);
      }
      else
      {
        for (int c = 0; c < C; ++c)
          uc[c] = enforce_constraint(u[(size_t)t * C + c], cc_.lower[c], cc_.upper[c], cc_.deadband[c],
                                     cc_.zero_control[c]);
      }
      model_step(i, x, uc, xn, t);
      for (int s = 0; s < S; ++s) x[s] = out[(size_t)(t + 1) * S + s] = xn[s];
    }
  }

  // TubeMPPIController::computeStateTrajectory (tube_mppi_controller.cu:334-341): the nominal system from the nominal
  // state along the nominal sequence, the actual system from the given state along the actual sequence.
  void tube_state_trajectories(const float* x_actual)
  {
    state_trajectory(0, x_actual, control_.data() + t_off_[0], state_seq_.data());
    state_trajectory(1, nominal_x0_.data(), control_.data() + t_off_[1], state_seq_.data() + (size_t)T_[0] * S);
    traj_dirty_ = false;
  }

  // TubeMPPIController::updateNominalState (tube_mppi_controller.cu:343-349)
  void advance_nominal_state()
  {
    float xn[S];
    model_step(1, nominal_x0_.data(), control_.data() + t_off_[1], xn, 0);
    for (int s = 0; s < S; ++s) nominal_x0_[s] = xn[s];
  }

  // Controller::smoothControlTrajectoryHelper (controller.cuh:573-607) on the host, in the order of the device
  // smoothing (finish_instance): each tap product rounded to FP32 and added in tap order, u[0] kept.
  // A plugin with its own enforceConstraints: the final pass after smoothing on the host, the plugin's method with a
  // zero state on every control (mppi_controller.cu:222-226), or ColoredMPPIController's clamp of control 1 alone
  // (colored_mppi_controller.cu:224-229).  The smoothed sequence came back unconstrained (sample_shared).
  void final_constraints_host()
  {
    for (int i = 0; i < I_; ++i)
      for (int t = 0; t < T_[i]; ++t)
      {
        float* u = control_.data() + t_off_[i] + (size_t)t * C;
        if (cp_.controller == MPPI_CONTROLLER_COLORED)
        {
          if (C > 1) u[1] = fminf(fmaxf(u[1], cc_.lower[1]), cc_.upper[1]);
        }
        else if constexpr (Model::kOwnConstraints)
        {
          float zero[S] = {};
          dyn_[i].enforceConstraints(zero, u);
        }
      }
  }

  void smooth_host(float* u, int T) const
  {
    const float coef[5] = { -3.0f / 35.0f, 12.0f / 35.0f, 17.0f / 35.0f, 12.0f / 35.0f, -3.0f / 35.0f };
    std::vector<float> buf((size_t)(T + 4) * C);
    for (int e = 0; e < (T + 4) * C; ++e)
    {
      const int tt = e / C, c = e - tt * C;
      buf[e] = u[(size_t)std::min(std::max(tt - 2, 0), T - 1) * C + c];
    }
    for (int t = 1; t < T; ++t)
      for (int c = 0; c < C; ++c)
      {
        float acc = 0.0f;
        for (int j = 0; j < 5; ++j) acc += coef[j] * buf[(size_t)(t + j) * C + c];
        u[(size_t)t * C + c] = acc;
      }
  }

  // One iteration of a host-iterated solve (iteration host_iter_): its graph, or plain stream launches.
  mppi_status launch_host_iteration(int stride)
  {
    if (graph_mode_)
    {
      cudaGraphExec_t exec = nullptr;
      MG_TRY(get_graph(stride, &exec));
      MG_CUDA(cudaGraphLaunch(exec, stream_));
      return MPPI_OK;
    }
    return enqueue_solve(stride);
  }

  // TubeMPPIController::computeControl (tube_mppi_controller.cu:158-296): per iteration one graph launch of the
  // device work of both systems (sample, rollout, weights, update, no smoothing), then the nominal-state decision on
  // the host; the nominal sequence is smoothed once at the end.
  mppi_status compute_control_tube(const float* x, int stride)
  {
    for (int i = 0; i < S; ++i)
      if (!std::isfinite(x[i]))
      {
        set_error("initial state has a non-finite entry at index %d", i);
        return MPPI_ENAN;
      }
    if (!nominal_init_)
    {
      nominal_x0_.assign(x, x + S);
      nominal_init_ = true;
    }
    for (int i = 0; i < I_; ++i) prev_baseline_[i] = baseline_norm_[2 * i];
    for (int it = 0; it < cp_.num_iters; ++it)
    {
      memcpy(x0_h_.p, x, sizeof(float) * S);
      memcpy(x0_h_.p + S, nominal_x0_.data(), sizeof(float) * S);
      memcpy(mean_h_.p, control_.data(), sizeof(float) * control_.size());
      host_iter_ = it;
      const mppi_status st = launch_host_iteration(stride);
      host_iter_ = 0;
      MG_TRY(st);
      MG_CUDA(cudaStreamSynchronize(stream_));
      if (status_h_.p[0] != 0u)
      {
        status_h_.p[0] = 0u;
        MG_CUDA(cudaMemsetAsync(status_d_, 0, sizeof(unsigned int), stream_));
        MG_CUDA(cudaStreamSynchronize(stream_));
        set_error("a bounded wait for staged control data gave up inside the rollout kernel");
        return MPPI_ETIMEOUT;
      }
      memcpy(control_.data(), out_mean_h_.p, sizeof(float) * control_.size());
      memcpy(baseline_norm_.data(), out_bn_h_.p, sizeof(float) * 2 * I_);
      memcpy(stats_.data(), out_stats_h_.p, sizeof(double) * 3 * I_);
      tube_state_trajectories(x);
      if (baseline_norm_[0] < baseline_norm_[2] + cp_.nominal_threshold)
      {
        // the disturbance that separated the systems improved the cost: the nominal system restarts from the actual
        nominal_used_ = 0;
        const size_t ts = (size_t)T_[0] * S, tc = (size_t)T_[0] * C;
        std::copy(state_seq_.begin(), state_seq_.begin() + ts, state_seq_.begin() + ts);
        nominal_x0_.assign(x, x + S);
        std::copy(control_.begin() + t_off_[0], control_.begin() + t_off_[0] + tc, control_.begin() + t_off_[1]);
      }
      else
      {
        nominal_used_ = 1;
      }
    }
    smooth_host(control_.data() + t_off_[1], T_[1]);
    tube_state_trajectories(x);
    for (int i = 0; i < I_; ++i)
      if (!std::isfinite(baseline_norm_[2 * i]) || !(stats_[3 * i] > 0.0))
      {
        set_error("a sampled cost or the normaliser is not finite (NaN state or noise?)");
        return MPPI_ENAN;
      }
    return MPPI_OK;
  }

  mppi_status enqueue_device_solves(int stride, int count) override
  {
    MG_CHECK(stride >= 0 && count >= 0, "stride and count must be >= 0");
    MG_CHECK(!Model::kNeedsCostmap || aux_.map.data != nullptr, "this model needs a costmap (mppi_set_costmap)");
    MG_CHECK(!Model::kMlp || use_analytic_ || !mlp_host_.empty(), "this model needs surrogate weights (mppi_set_mlp)");
    auto it = device_graphs_.find(stride);
    cudaGraphExec_t exec = nullptr;
    if (it == device_graphs_.end())
    {
      cudaGraph_t g = nullptr;
      MG_CUDA(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
      mppi_status st = enqueue_kernels(stride);
      cudaError_t ce = cudaStreamEndCapture(stream_, &g);
      if (st != MPPI_OK)
      {
        if (g) cudaGraphDestroy(g);
        (void)cudaGetLastError();  // the invalidated capture's error stays with this call
        return st;
      }
      MG_CUDA(ce);
      ce = cudaGraphInstantiate(&exec, g, 0);
      cudaGraphDestroy(g);
      MG_CUDA(ce);
      device_graphs_[stride] = exec;
    }
    else
    {
      exec = it->second;
    }
    for (int i = 0; i < count; ++i) MG_CUDA(cudaGraphLaunch(exec, stream_));
    return MPPI_OK;
  }

  mppi_status time_kernels(int stride, int reps, float* ms3) override
  {
    MG_CHECK(ms3 && reps >= 1, "need an output array and reps >= 1");
    MG_CHECK(!Model::kNeedsCostmap || aux_.map.data != nullptr, "this model needs a costmap (mppi_set_costmap)");
    MG_CHECK(!Model::kMlp || use_analytic_ || !mlp_host_.empty(), "this model needs surrogate weights (mppi_set_mlp)");
    cudaEvent_t ev[4];
    for (auto& e : ev) MG_CUDA(cudaEventCreate(&e));
    float tot[3] = { 0, 0, 0 };
    for (int r = 0; r < reps + 1; ++r)
    {
      MG_CUDA(cudaEventRecord(ev[0], stream_));
      if (!fused()) MG_TRY(launch_sampler(stride, 0));
      MG_CUDA(cudaEventRecord(ev[1], stream_));
      MG_TRY(launch_rollout(stride, 0));
      MG_CUDA(cudaEventRecord(ev[2], stream_));
      MG_TRY(launch_weights(0));
      MG_CUDA(cudaEventRecord(ev[3], stream_));
      MG_CUDA(cudaEventSynchronize(ev[3]));
      if (r == 0) continue;  // warm-up
      for (int k = 0; k < 3; ++k)
      {
        float ms = 0.0f;
        MG_CUDA(cudaEventElapsedTime(&ms, ev[k], ev[k + 1]));
        tot[k] += ms;
      }
    }
    for (auto& e : ev) cudaEventDestroy(e);
    for (int k = 0; k < 3; ++k) ms3[k] = tot[k] / reps;
    return MPPI_OK;
  }

private:
  Engine() = default;

  static int tch_for(int ns)
  {
    switch (ns)
    {
      case 32: return RolloutShape<32, C>::TCH;
      case 64: return RolloutShape<64, C>::TCH;
      case 128: return RolloutShape<128, C>::TCH;
      default: return RolloutShape<256, C>::TCH;
    }
  }

  mppi_status check_sampling(const mppi_sampling_params& sp)
  {
    MG_CHECK(sp.kind == MPPI_SAMPLER_GAUSSIAN || sp.kind == MPPI_SAMPLER_COLORED_NOISE, "unknown sampler kind %d",
             sp.kind);
    for (int c = 0; c < C; ++c)
      MG_CHECK(std::isfinite(sp.std_dev[c]) && sp.std_dev[c] >= 0.0f, "std_dev[%d] must be finite and >= 0", c);
    MG_CHECK(sp.pure_noise_trajectories_percentage >= 0.0f && sp.pure_noise_trajectories_percentage <= 1.0f,
             "pure_noise_trajectories_percentage must be in [0, 1]");
    if (sp.kind == MPPI_SAMPLER_COLORED_NOISE)
    {
      for (int c = 0; c < C; ++c) MG_CHECK(std::isfinite(sp.exponents[c]), "exponents[%d] must be finite", c);
      MG_CHECK(std::isfinite(sp.offset_decay_rate) && std::isfinite(sp.fmin), "offset_decay_rate and fmin must be finite");
      for (int T : T_)
        MG_CHECK(T <= kColoredMaxT, "the colored-noise sampler supports num_timesteps <= %d (got %d)", kColoredMaxT, T);
    }
    return MPPI_OK;
  }

  mppi_status init(const CreateArgs& a)
  {
    I_ = a.num_instances;
    MG_TRY(check_controller(a.cp));
    cp_ = a.cp;
    cc_ = a.cc;
    K_.assign(a.K, a.K + I_);
    T_.assign(a.T, a.T + I_);
    MG_TRY(check_controller(cp_));  // the Tube-MPPI shape rule needs K and T
    MG_TRY(check_sampling(a.sp));
    sp_ = a.sp;
    long long total_u = 0;
    int total_k = 0, total_t = 0;
    for (int i = 0; i < I_; ++i)
    {
      MG_CHECK(K_[i] >= 1, "num_rollouts[%d] must be >= 1 (got %d)", i, K_[i]);
      MG_CHECK(T_[i] >= 1, "num_timesteps[%d] must be >= 1 (got %d)", i, T_[i]);
      MG_CHECK((long long)K_[i] * T_[i] * C < (1LL << 31), "instance %d is too large", i);
      k_off_.push_back(total_k);
      t_off_.push_back(total_t);
      u_off_.push_back(total_u);
      total_k += K_[i];
      total_t += T_[i] * C;
      total_u += ((long long)K_[i] * T_[i] * C + 3) / 4 * 4;
    }
    total_k_ = total_k;
    use_bulk_ = true;
    for (int i = 0; i < I_; ++i)
      if (((long long)T_[i] * C) % 4 != 0) use_bulk_ = false;
    dyn_.assign((const DynParams*)a.dyn, (const DynParams*)a.dyn + I_);
    cost_.assign((const CostParams*)a.cost, (const CostParams*)a.cost + I_);
    control_.assign((size_t)total_t, 0.0f);
    if (a.init_control) memcpy(control_.data(), a.init_control, sizeof(float) * total_t);
    size_t total_s = 0;
    for (int i = 0; i < I_; ++i) total_s += (size_t)T_[i] * S;
    state_seq_.assign(total_s, 0.0f);
    history_.assign((size_t)I_ * 2 * C, 0.0f);
    last_pre_smooth_.assign((size_t)I_ * C, 0.0f);
    baseline_norm_.assign((size_t)2 * I_, 0.0f);
    stats_.assign((size_t)3 * I_, 0.0);
    prev_baseline_.assign(I_, 0.0f);
    memset(&aux_, 0, sizeof(aux_));
    fb_w_.Q.assign((size_t)S * S, 0.0);
    fb_w_.Qf.assign((size_t)S * S, 0.0);
    fb_w_.R.assign((size_t)C * C, 0.0);
    for (int e = 0; e < S; ++e) fb_w_.Q[(size_t)e * S + e] = fb_w_.Qf[(size_t)e * S + e] = 1.0;
    for (int e = 0; e < C; ++e) fb_w_.R[(size_t)e * C + e] = 1.0;
    fb_gains_.assign((size_t)T_[fb_instance()] * C * S, 0.0f);
    fb_prop_.assign((size_t)T_[fb_instance()] * S, 0.0f);

    if (a.stream)
    {
      stream_ = a.stream;
    }
    else
    {
      MG_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
      own_stream_ = true;
    }
    int dev = 0;
    MG_CUDA(cudaGetDevice(&dev));
    MG_CUDA(cudaDeviceGetAttribute(&num_sms_, cudaDevAttrMultiProcessorCount, dev));

    MG_TRY(samples_d_.alloc((size_t)total_u));
    total_u_ = total_u;
    MG_CUDA(cudaMemset(samples_d_.p, 0, sizeof(float) * samples_d_.n));
    MG_TRY(costs_d_.alloc(total_k));
    MG_TRY(weights_d_.alloc(total_k));
    MG_CUDA(cudaMemset(costs_d_.p, 0, sizeof(float) * total_k));
    MG_CUDA(cudaMemset(weights_d_.p, 0, sizeof(float) * total_k));
    // Per-solve I/O in one block so a solve needs one host-to-device and one device-to-host copy:
    //   [x0 | mean] is copied in, [mean | first | baseline,normaliser | status | stats] is copied out.
    {
      auto up16 = [](size_t b) { return (b + 15) / 16 * 16; };
      // the mean row starts on a 16-byte boundary: the fused samplers read it as float4 (odd S leaves a gap)
      const size_t o_x0 = 0, o_mean = up16(o_x0 + sizeof(float) * I_ * S);
      const size_t o_first = o_mean + sizeof(float) * total_t;
      const size_t o_bn = o_first + sizeof(float) * I_ * C;
      const size_t o_status = o_bn + sizeof(float) * 2 * I_;
      const size_t o_stats = up16(o_status + sizeof(unsigned int));
      const size_t o_end = o_stats + sizeof(double) * 3 * I_;
      io_in_bytes_ = o_mean + sizeof(float) * total_t;
      io_out_off_ = o_mean;
      io_out_bytes_ = o_end - o_mean;
      MG_TRY(io_d_.alloc(o_end));
      MG_CUDA(cudaMemset(io_d_.p, 0, o_end));
      MG_TRY(io_in_h_.alloc(io_in_bytes_));
      MG_TRY(io_out_h_.alloc(io_out_bytes_));
      memset(io_in_h_.p, 0, io_in_bytes_);
      unsigned char* d = io_d_.p;
      x0_d_.view(reinterpret_cast<float*>(d + o_x0), (size_t)I_ * S);
      mean_d_.view(reinterpret_cast<float*>(d + o_mean), total_t);
      MG_CHECK((reinterpret_cast<uintptr_t>(mean_d_.p) & 15) == 0, "internal: the mean row must be 16-byte aligned");
      first_d_.view(reinterpret_cast<float*>(d + o_first), (size_t)I_ * C);
      bn_d_.view(reinterpret_cast<float*>(d + o_bn), (size_t)2 * I_);
      status_d_ = reinterpret_cast<unsigned int*>(d + o_status);
      stats_d_.view(reinterpret_cast<double*>(d + o_stats), (size_t)3 * I_);
      x0_h_.view(reinterpret_cast<float*>(io_in_h_.p + o_x0), (size_t)I_ * S);
      mean_h_.view(reinterpret_cast<float*>(io_in_h_.p + o_mean), total_t);
      unsigned char* h = io_out_h_.p - o_mean;  // same offsets as the device block
      out_mean_h_.view(reinterpret_cast<float*>(h + o_mean), total_t);
      first_h_.view(reinterpret_cast<float*>(h + o_first), (size_t)I_ * C);
      out_bn_h_.view(reinterpret_cast<float*>(h + o_bn), (size_t)2 * I_);
      status_h_.view(reinterpret_cast<unsigned int*>(h + o_status), 1);
      out_stats_h_.view(reinterpret_cast<double*>(h + o_stats), (size_t)3 * I_);
    }
    MG_TRY(dyn_d_.alloc(I_));
    MG_TRY(cost_d_.alloc(I_));
    MG_CUDA(cudaMemcpy(dyn_d_.p, dyn_.data(), sizeof(DynParams) * I_, cudaMemcpyHostToDevice));
    MG_CUDA(cudaMemcpy(cost_d_.p, cost_.data(), sizeof(CostParams) * I_, cudaMemcpyHostToDevice));
    MG_TRY(baseline_bits_d_.alloc(I_));
    MG_TRY(arrive_d_.alloc(I_));
    MG_TRY(counters_d_.alloc(8));
    MG_CUDA(cudaMemset(arrive_d_.p, 0, sizeof(unsigned int) * I_));
    MG_CUDA(cudaMemset(counters_d_.p, 0, sizeof(unsigned int) * 8));
    fill_u32_kernel<<<1, 256, 0, stream_>>>(baseline_bits_d_.p, kOrderedPosInf, I_);
    MG_CUDA(cudaGetLastError());
    max_t_ = *std::max_element(T_.begin(), T_.end());  // sizes per-launch shared buffers (split cost kernel)
    if (Model::kMlp) ns_ = kMlpSamplesPerCta;
    if constexpr ((4 % C) == 0 && !Model::kPlugin)
    {
      MG_TRY(allow_fused_stage<32>());
      MG_TRY(allow_fused_stage<64>());
      MG_TRY(allow_fused_stage<128>());
      MG_TRY(allow_fused_stage<256>());
    }
    MG_TRY(build_work_lists());
    MG_TRY(build_colored_tables());
    MG_TRY(build_judge_lists());
    MG_CUDA(cudaStreamSynchronize(stream_));
    return MPPI_OK;
  }

  // Per-T tables for the colored-noise sampler (mg_colored.cu).  Twiddles are computed in double and rounded to float:
  //   T = 32, 64, 128 (four lanes per row): none here, the kernel's twiddles are the constant table c_w256;
  //   T = 256 (one warp per row, R = 8): packing twiddles e^{2 pi i k / 2T} (k < T), then the register-stage
  //     twiddles [log2 R][R][32] and the lane-stage twiddles [5][32] of the decimation-in-frequency inverse FFT;
  //   other T: the full table e^{2 pi i j / 2T}, j < 2T, for the direct transform.
  // Frequency scales and sigma are computed in float in the order of the reference's host code
  // (colored_noise.cu:294-333); decay^t with powf as rearrangeNoise does (colored_noise.cu:44).
  mppi_status build_colored_tables()
  {
    if (sp_.kind != MPPI_SAMPLER_COLORED_NOISE) return MPPI_OK;
    MG_TRY(colored_init_constants());
    std::vector<float> tab;
    std::map<int, std::pair<int, int4>> by_t;
    std::vector<int> tab_off(I_);
    std::vector<int4> parts(I_);
    auto align4 = [&]() {
      while (tab.size() % 4) tab.push_back(0.0f);
    };
    auto push_tw = [&](double num, double den) {
      tab.push_back((float)std::cos(2.0 * M_PI * num / den));
      tab.push_back((float)std::sin(2.0 * M_PI * num / den));
    };
    for (int i = 0; i < I_; ++i)
    {
      const int T = T_[i];
      auto it = by_t.find(T);
      if (it == by_t.end())
      {
        const int N = 2 * T, F = T + 1;
        const int base = (int)tab.size();
        const bool quad = (T == 32 || T == 64 || T == 128);
        int lane_off = 0;
        if (T == 256)
        {
          const int R = T / 32;
          for (int k = 0; k < T; ++k) push_tw(k, N);
          int s = 0;
          for (int hr = R / 2; hr >= 1; hr >>= 1, ++s)
            for (int r = 0; r < R; ++r)
              for (int lane = 0; lane < 32; ++lane)
                push_tw((r & hr) == 0 ? lane + 32 * (r % (2 * hr)) : 0, 64.0 * hr);
          lane_off = (int)tab.size() - base;
          for (int st = 0; st < 5; ++st)
          {
            const int half = 16 >> st;
            for (int lane = 0; lane < 32; ++lane)
              push_tw((lane & half) ? (lane % (2 * half)) - half : 0, 2.0 * half);
          }
        }
        else if (!quad)
        {
          for (int j = 0; j < N; ++j) push_tw(j, N);
        }
        align4();
        // fftfreq (colored_noise.cuh:24-34) and the cutoff / scale loop (colored_noise.cu:294-317)
        std::vector<float> freq(F), scale((size_t)F * C, 0.0f);
        for (int j = 0; j < F; ++j) freq[j] = j / (1.0f * N);
        const float cutoff = fmaxf(sp_.fmin, 1.0f / N);
        int smaller = 0;
        for (int f = 0; f < F; ++f)
        {
          if (freq[f] < cutoff)
            smaller++;
          else if (smaller < F)
            for (int j = 0; j < smaller; ++j)
            {
              freq[j] = freq[smaller];
              for (int c = 0; c < C; ++c) scale[(size_t)j * C + c] = powf(freq[smaller], -sp_.exponents[c] / 2.0f);
            }
          for (int c = 0; c < C; ++c) scale[(size_t)f * C + c] = powf(freq[f], -sp_.exponents[c] / 2.0f);
        }
        int4 p;
        p.x = (int)tab.size() - base;
        tab.insert(tab.end(), scale.begin(), scale.end());
        align4();
        p.y = (int)tab.size() - base;
        for (int c = 0; c < C; ++c)  // sigma (colored_noise.cu:320-328)
        {
          float s = 0.0f;
          for (int j = 1; j < F - 1; ++j) s += scale[(size_t)j * C + c] * scale[(size_t)j * C + c];
          const float last = scale[(size_t)(F - 1) * C + c] * ((1.0f + (N % 2)) / 2.0f);
          s += last * last;
          tab.push_back(2.0f * sqrtf(s) / N);
        }
        align4();
        p.z = (int)tab.size() - base;
        for (int t = 0; t < T; ++t)
          tab.push_back(sp_.offset_decay_rate == 0.0f ? 0.0f : powf(sp_.offset_decay_rate, (float)t));
        align4();
        p.w = lane_off;
        it = by_t.emplace(T, std::make_pair(base, p)).first;
      }
      tab_off[i] = it->second.first;
      parts[i] = it->second.second;
    }
    MG_TRY(ctab_d_.alloc(tab.size()));
    MG_TRY(ctab_off_d_.alloc(I_));
    MG_TRY(ctab_parts_d_.alloc(I_));
    MG_CUDA(cudaMemcpy(ctab_d_.p, tab.data(), sizeof(float) * tab.size(), cudaMemcpyHostToDevice));
    MG_CUDA(cudaMemcpy(ctab_off_d_.p, tab_off.data(), sizeof(int) * I_, cudaMemcpyHostToDevice));
    MG_CUDA(cudaMemcpy(ctab_parts_d_.p, parts.data(), sizeof(int4) * I_, cudaMemcpyHostToDevice));
    return MPPI_OK;
  }

  // Work lists: rollout tiles ordered by decreasing horizon (the cost of a tile is proportional to T), sampler items,
  // and weight/update chunks with the offsets of their partial rows.
  // Which noise each instance draws (InstDesc::noise_*): its own, except that the second distribution of a Tube-MPPI
  // or R-MPPI handle draws the first one's when use_same_noise_for_all_distributions is set (generateSamples copies
  // one draw to every distribution, gaussian.cu:378-390).
  void set_noise_sources(std::vector<InstDesc>& inst) const
  {
    const bool shared = (tube() || rmppi()) && sp_.use_same_noise_for_all_distributions != 0;
    for (int i = 0; i < I_; ++i)
    {
      const int src = shared ? 0 : i;
      inst[i].noise_inst = src;
      inst[i].noise_off = inst[src].u_off;
      inst[i].noise_spec_off = inst[src].spec_off;
    }
  }
  // after a change of the controller kind or of the sampling parameters
  mppi_status refresh_noise_sources()
  {
    if (inst_h_.empty()) return MPPI_OK;
    set_noise_sources(inst_h_);
    MG_CUDA(cudaStreamSynchronize(stream_));
    MG_CUDA(cudaMemcpy(inst_d_.p, inst_h_.data(), sizeof(InstDesc) * I_, cudaMemcpyHostToDevice));
    return MPPI_OK;
  }

  mppi_status build_work_lists()
  {
    std::vector<InstDesc> inst(I_);
    std::vector<int2> tiles, swork, cwork, cwork_cls[5];
    std::vector<int4> chunks;
    std::vector<long long> part_off;
    std::vector<int> chunk0(I_);
    long long poff = 0, spec = 0;
    for (int i = 0; i < I_; ++i)
    {
      InstDesc& d = inst[i];
      d.K = K_[i];
      d.T = T_[i];
      d.k_off = k_off_[i];
      d.t_off = t_off_[i];
      d.u_off = u_off_[i];
      d.spec_off = spec;
      spec += (long long)K_[i] * C * (T_[i] + 1) * 2;
      d.x_off = i * S;
      const int cls = colored_class(T_[i]);
      for (int k0 = 0; k0 < K_[i]; k0 += colored_class_spb<C>(cls)) cwork_cls[cls].push_back(make_int2(i, k0));
      d.num_chunks = (K_[i] + kc_ - 1) / kc_;
      chunk0[i] = (int)chunks.size();
      for (int c = 0; c < d.num_chunks; ++c)
      {
        chunks.push_back(make_int4(i, c * kc_, std::min(K_[i], (c + 1) * kc_), c));
        part_off.push_back(poff);
        poff += (long long)T_[i] * C;
      }
      const long long nq = ((long long)K_[i] * T_[i] * C + 3) / 4;
      for (long long q = 0; q < nq; q += kSampleQuadsPerItem) swork.push_back(make_int2(i, (int)q));
    }
    std::vector<int> order(I_);
    for (int i = 0; i < I_; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return T_[x] > T_[y]; });
    std::vector<int> inst_tile0(I_, 0);
    std::vector<long long> tile_poff;
    long long tpoff = 0;
    max_tiles_per_inst_ = 1;
    max_k_ = 1;
    for (int i : order)
    {
      inst_tile0[i] = (int)tiles.size();
      max_tiles_per_inst_ = std::max(max_tiles_per_inst_, (K_[i] + ns_ - 1) / ns_);
      max_k_ = std::max(max_k_, K_[i]);
      for (int k0 = 0; k0 < K_[i]; k0 += ns_)
      {
        tiles.push_back(make_int2(i, k0));
        tile_poff.push_back(tpoff);  // an instance's tile rows are consecutive, T*C floats apart
        tpoff += (long long)T_[i] * C;
      }
    }
    num_tiles_ = (int)tiles.size();
    MG_CHECK(sizeof(double) * (size_t)max_tiles_per_inst_ <= 200 * 1024,
             "too many rollout tiles in one instance (%d); raise the samples per CTA", max_tiles_per_inst_);
    MG_TRY(tile_part_d_.alloc((size_t)std::max<long long>(tpoff, 1)));
    MG_TRY(tile_poff_d_.alloc(tile_poff.size()));
    MG_TRY(tile_sums_d_.alloc(2 * tile_poff.size()));
    MG_TRY(tile_min_d_.alloc(tile_poff.size()));
    MG_TRY(inst_tile0_d_.alloc(I_));
    MG_TRY(inst_tiles_done_d_.alloc(I_));
    MG_CUDA(cudaMemset(inst_tiles_done_d_.p, 0, sizeof(unsigned int) * I_));
    MG_CUDA(cudaMemcpy(tile_poff_d_.p, tile_poff.data(), sizeof(long long) * tile_poff.size(), cudaMemcpyHostToDevice));
    MG_CUDA(cudaMemcpy(inst_tile0_d_.p, inst_tile0.data(), sizeof(int) * I_, cudaMemcpyHostToDevice));
    num_chunks_ = (int)chunks.size();
    num_swork_ = (int)swork.size();
    class_begin_[0] = 0;
    for (int k = 0; k < 5; ++k)
    {
      cwork.insert(cwork.end(), cwork_cls[k].begin(), cwork_cls[k].end());
      class_begin_[k + 1] = (int)cwork.size();
    }
    num_cwork_ = (int)cwork.size();
    MG_TRY(inst_d_.alloc(I_));
    MG_TRY(tiles_d_.alloc(tiles.size()));
    MG_TRY(swork_d_.alloc(swork.size()));
    MG_TRY(cwork_d_.alloc(cwork.size()));
    MG_CUDA(cudaMemcpy(cwork_d_.p, cwork.data(), sizeof(int2) * cwork.size(), cudaMemcpyHostToDevice));
    MG_TRY(chunks_d_.alloc(chunks.size()));
    MG_TRY(part_off_d_.alloc(part_off.size()));
    MG_TRY(chunk0_d_.alloc(I_));
    MG_TRY(partials_d_.alloc((size_t)std::max<long long>(poff, 1)));
    MG_TRY(part_w_d_.alloc(2 * chunks.size()));
    set_noise_sources(inst);
    inst_h_ = inst;
    MG_CUDA(cudaMemcpy(inst_d_.p, inst.data(), sizeof(InstDesc) * I_, cudaMemcpyHostToDevice));
    MG_CUDA(cudaMemcpy(tiles_d_.p, tiles.data(), sizeof(int2) * tiles.size(), cudaMemcpyHostToDevice));
    MG_CUDA(cudaMemcpy(swork_d_.p, swork.data(), sizeof(int2) * swork.size(), cudaMemcpyHostToDevice));
    MG_CUDA(cudaMemcpy(chunks_d_.p, chunks.data(), sizeof(int4) * chunks.size(), cudaMemcpyHostToDevice));
    MG_CUDA(cudaMemcpy(part_off_d_.p, part_off.data(), sizeof(long long) * part_off.size(), cudaMemcpyHostToDevice));
    MG_CUDA(cudaMemcpy(chunk0_d_.p, chunk0.data(), sizeof(int) * I_, cudaMemcpyHostToDevice));
    // persistent rollout grid: every SM filled to its occupancy limit, never more CTAs than tiles
    int per_sm = 1;
    MG_TRY(rollout_occupancy(&per_sm));
    rollout_grid_ = std::max(1, std::min(num_tiles_, per_sm * num_sms_));
    return MPPI_OK;
  }

  // Dynamic shared memory of the fused rollout: the tile's controls, staged for the tile reduction (0: the reduction
  // reads them back from L2 instead, for horizons too long to stage).
  template <int NS>
  size_t fused_stage_bytes_max() const
  {
    const size_t b = sizeof(float) * (size_t)max_t_ * C * (NS + 1);
    return b <= 200 * 1024 ? b : 0;
  }
  template <int NS>
  size_t fused_stage_bytes() const
  {
    return tile_reduce_active() ? fused_stage_bytes_max<NS>() : 0;
  }
  // The fused rollout's dynamic shared memory: the staged controls, reused by the CTA that finalizes an instance
  // for the per-tile rescale factors and for the smoothing buffer.
  template <int NS>
  size_t fused_dyn_bytes(bool stage) const
  {
    const int max_k = *std::max_element(K_.begin(), K_.end());
    const size_t tiles = sizeof(float) * (size_t)((max_k + NS - 1) / NS);
    const size_t smooth = sizeof(float) * (size_t)(max_t_ + 4) * C;
    return std::max(stage ? fused_stage_bytes_max<NS>() : (size_t)0, std::max(tiles, smooth));
  }
  // Opts the fused rollout into its shared-memory size once, at creation (never during graph capture).
  template <int NS>
  mppi_status allow_fused_stage()
  {
    MG_CUDA(raise_smem_cap(rollout_fused_kernel<Model, NS>, fused_dyn_bytes<NS>(true)));
    MG_CUDA(raise_smem_cap(rollout_fused_kernel<Model, NS, true>, fused_dyn_bytes<NS>(true)));
    return MPPI_OK;
  }

  // The fused rollout (mode 0) with tile reduction also combines each instance and, in the last iteration, smooths
  // it: no finalize or smoothing kernel follows it.
  bool tail_finalize() const
  {
    return tile_reduce_active() && fused() && !split_ && (rollout_mode_ == 0 || rollout_mode_ == 4);
  }
  // Mode 4 at this tile size: the stage holds the longest horizon.
  template <int NS>
  bool noise_warps_now() const
  {
    return rollout_mode_ == 4 && fused_stage_bytes<NS>() != 0;
  }

  FinalizeArgs finalize_args() const
  {
    FinalizeArgs f{};
    f.inst = inst_d_.p;
    f.num_instances = I_;
    f.inst_tile0 = inst_tile0_d_.p;
    f.tile_samples = ns_;
    f.tr.partials = tile_part_d_.p;
    f.tr.poff = tile_poff_d_.p;
    f.tr.sums = tile_sums_d_.p;
    f.tr.tmin = tile_min_d_.p;
    f.tr.lambda_inv = 1.0f / cp_.lambda;
    f.baseline_bits = baseline_bits_d_.p;
    f.inst_done = counters_d_.p + 2;
    f.noise_counter = counters_d_.p + 3;
    f.mean_out = mean_d_.p;
    f.baseline_norm = bn_d_.p;
    f.stats = stats_d_.p;
    f.C = C;
    f.inst_tiles_done = inst_tiles_done_d_.p;
    f.first_out = first_d_.p;
    f.finish = 0;
    f.host_mean = f.host_first = f.host_bn = nullptr;
    f.host_stats = nullptr;
    f.host_status = nullptr;
    f.status = status_d_;
    return f;
  }

  template <int NS>
  void launch_fused(RolloutArgs<Model> a, const FusedNoise& f, int iter)
  {
    const size_t stage = fused_stage_bytes<NS>();
    a.tr.u_stride = stage ? NS + 1 : 0;
    if (tail_finalize())
    {
      a.tail = 1;
      a.fin = finalize_args();
      a.fin.finish = !tube() && iter == cp_.num_iters - 1;
      if (a.fin.finish && direct_out_)
      {
        a.fin.host_mean = out_mean_h_.p;
        a.fin.host_first = first_h_.p;
        a.fin.host_bn = out_bn_h_.p;
        a.fin.host_stats = out_stats_h_.p;
        a.fin.host_status = status_h_.p;
      }
    }
    if (noise_warps_now<NS>())
      rollout_fused_kernel<Model, NS, true><<<rollout_grid_, 2 * NS, fused_dyn_bytes<NS>(true), stream_>>>(a, f);
    else
      rollout_fused_kernel<Model, NS><<<rollout_grid_, NS, fused_dyn_bytes<NS>(stage != 0), stream_>>>(a, f);
  }

  template <int NS>
  mppi_status occupancy_ns(int* per_sm)
  {
    if constexpr (Model::kPlugin)
    {
      MG_CUDA(resident_ctas_per_sm(rollout_plugin_kernel<Model, NS, RolloutShape<NS, C>::TCH>, NS, 0, per_sm));
      if (*per_sm < 1) *per_sm = 1;
      return MPPI_OK;
    }
    else
    {
      return occupancy_builtin<NS>(per_sm);
    }
  }
  template <int NS>
  mppi_status occupancy_builtin(int* per_sm)
  {
    if constexpr ((4 % C) == 0)
      if (fused())
      {
        if (split_)
          MG_CUDA(resident_ctas_per_sm(rollout_dyn_kernel<Model, NS>, NS, 0, per_sm));
        else if (rollout_mode_ == 2)
          MG_CUDA(resident_ctas_per_sm(rollout_coop_kernel<Model, NS>, 4 * NS, 0, per_sm));
        else if (noise_warps_now<NS>())
          MG_CUDA(resident_ctas_per_sm(rollout_fused_kernel<Model, NS, true>, 2 * NS, fused_dyn_bytes<NS>(true),
                                       per_sm));
        else
          MG_CUDA(resident_ctas_per_sm(rollout_fused_kernel<Model, NS>, NS,
                                       fused_dyn_bytes<NS>(fused_stage_bytes<NS>() != 0), per_sm));
        return MPPI_OK;
      }
    if (use_bulk_)
    {
      using B = BulkRolloutShape<NS, C>;
      MG_CUDA(resident_ctas_per_sm(rollout_kernel_bulk<Model, NS, B::TCH>, NS, B::SMEM, per_sm));
    }
    else
    {
      constexpr int TCH = RolloutShape<NS, C>::TCH;
      MG_CUDA(resident_ctas_per_sm(rollout_kernel<Model, NS, TCH>, NS, 0, per_sm));
    }
    if (*per_sm < 1) *per_sm = 1;
    return MPPI_OK;
  }
  mppi_status rollout_occupancy(int* per_sm)
  {
    switch (ns_)
    {
      case 32: return occupancy_ns<32>(per_sm);
      case 64: return occupancy_ns<64>(per_sm);
      case 128: return occupancy_ns<128>(per_sm);
      default: return occupancy_ns<256>(per_sm);
    }
  }

  mppi_status launch_sampler(int stride, int iter)
  {
    SampleArgs a;
    a.inst = inst_d_.p;
    a.work = swork_d_.p;
    a.num_work = num_swork_;
    a.quads_per_item = kSampleQuadsPerItem;
    a.samples = samples_d_.p;
    a.mean = mean_d_.p;
    a.injected = injected_d_.p;
    a.noise_counter = counters_d_.p + 3;
    a.seed_lo = (uint32_t)cp_.seed;
    a.seed_hi = (uint32_t)(cp_.seed >> 32);
    a.stride = stride;
    a.decay_pow = powf(sp_.std_dev_decay, (float)iter);
    a.sh = sample_shared();
    if (sp_.kind == MPPI_SAMPLER_COLORED_NOISE) return launch_colored(a);
    const int grid = std::min(num_swork_, 8 * num_sms_);
    gaussian_sample_kernel<C><<<grid, 256, 0, stream_>>>(a);
    MG_CUDA(cudaGetLastError());
    return MPPI_OK;
  }

  mppi_status launch_colored(const SampleArgs& s)
  {
    for (int T : T_)
      MG_CHECK(s.stride < 2 * T, "optimization_stride (%d) must be below 2 * num_timesteps for colored noise",
               s.stride);
    ColoredArgs a;
    a.inst = inst_d_.p;
    a.work = cwork_d_.p;
    a.num_work = num_cwork_;
    a.tables = ctab_d_.p;
    a.tab_off = ctab_off_d_.p;
    a.tab_parts = ctab_parts_d_.p;
    a.samples = samples_d_.p;
    a.mean = mean_d_.p;
    a.injected_spec = injected_d_.p;
    a.noise_counter = s.noise_counter;
    a.seed_lo = s.seed_lo;
    a.seed_hi = s.seed_hi;
    a.stride = s.stride;
    a.decay_pow = s.decay_pow;
    a.sh = s.sh;
    return launch_colored_sampler<C>(a, class_begin_, max_t_, num_sms_, stream_);
  }

  template <int NS>
  void launch_rollout_ns(const RolloutArgs<Model>& a)
  {
    if (use_bulk_)
    {
      using B = BulkRolloutShape<NS, C>;
      rollout_kernel_bulk<Model, NS, B::TCH><<<rollout_grid_, NS, B::SMEM, stream_>>>(a);
    }
    else
    {
      constexpr int TCH = RolloutShape<NS, C>::TCH;
      rollout_kernel<Model, NS, TCH><<<rollout_grid_, NS, 0, stream_>>>(a);
    }
  }
  // Gaussian noise is generated inside the rollout (rollout_fused_kernel) when every row holds whole quads of steps;
  // the standalone sampler then runs only for mppi_generate_samples.
  // Gaussian sampling can run inside the rollout kernels (every row holds whole control quads) ...
  bool fusable() const { return !Model::kPlugin && sp_.kind == MPPI_SAMPLER_GAUSSIAN && (4 % C) == 0 && use_bulk_; }
  // ... and does, unless rollout mode 3 asks for the separate sampler kernel.
  bool fused() const { return fusable() && rollout_mode_ != 3 && !rmppi(); }

  FusedNoise fused_noise_args(int stride, int iter) const
  {
    FusedNoise f;
    f.samples = samples_d_.p;
    f.injected = injected_d_.p;
    f.noise_counter = counters_d_.p + 3;
    f.seed_lo = (uint32_t)cp_.seed;
    f.seed_hi = (uint32_t)(cp_.seed >> 32);
    f.stride = stride;
    f.decay_pow = powf(sp_.std_dev_decay, (float)iter);
    return f;
  }

  template <int NS>
  mppi_status launch_cost_kernel(const RolloutArgs<Model>& a)
  {
    constexpr int WARPS = 4;
    auto kern = rollout_cost_kernel<Model, NS, WARPS>;
    // one row of max_t_ step costs per warp; every instance's T is at most max_t_ (set at create)
    MG_CHECK(max_t_ >= *std::max_element(T_.begin(), T_.end()), "internal: horizon bound not set");
    const size_t smem = sizeof(float) * WARPS * (size_t)max_t_;
    MG_CUDA(raise_smem_cap(kern, smem));
    int per_sm = 1;
    MG_CUDA(resident_ctas_per_sm(kern, WARPS * 32, smem, &per_sm));
    const int grid = std::max(1, std::min(num_tiles_, per_sm * num_sms_));
    kern<<<grid, WARPS * 32, smem, stream_>>>(a, states_d_.p);
    MG_CUDA(cudaGetLastError());
    return MPPI_OK;
  }

  // The rollout arguments every rollout kernel shares.
  RolloutArgs<Model> base_rollout_args() const
  {
    RolloutArgs<Model> a{};
    a.inst = inst_d_.p;
    a.tiles = tiles_d_.p;
    a.num_tiles = num_tiles_;
    a.dyn = dyn_d_.p;
    a.cost = cost_d_.p;
    a.aux = aux_;
    a.x0 = x0_d_.p;
    a.samples = samples_d_.p;
    a.mean = mean_d_.p;
    a.costs = costs_d_.p;
    a.baseline_bits = baseline_bits_d_.p;
    a.tile_counter = counters_d_.p;
    a.status = status_d_;
    a.dt = cp_.dt;
    a.lambda = cp_.lambda;
    a.alpha = cp_.alpha;
    a.use_likelihood = 0;
    for (int c = 0; c < C; ++c)
      if (sp_.control_cost_coeff[c] != 0.0f) a.use_likelihood = 1;
    a.max_t = max_t_;
    a.sh = sample_shared();
    a.max_polls = max_polls_;
    a.withhold_progress = withhold_progress_ ? 1 : 0;
    return a;
  }

  mppi_status launch_rollout(int stride, int iter)
  {
    if constexpr (!Model::kMlp)
      if (rmppi()) return launch_rmppi_rollout();
    if constexpr (Model::kPlugin)
    {
      RolloutArgs<Model> a = base_rollout_args();
      a.tr.partials = tile_part_d_.p;
      a.tr.poff = tile_poff_d_.p;
      a.tr.sums = tile_sums_d_.p;
      a.tr.tmin = tile_min_d_.p;
      a.tr.lambda_inv = 1.0f / cp_.lambda;
      if (!tile_reduce_active()) a.tr.partials = nullptr;
      switch (ns_)
      {
        case 32: launch_plugin_ns<32>(a); break;
        case 64: launch_plugin_ns<64>(a); break;
        case 128: launch_plugin_ns<128>(a); break;
        default: launch_plugin_ns<256>(a); break;
      }
      MG_CUDA(cudaGetLastError());
      return MPPI_OK;
    }
    else
    {
      return launch_rollout_builtin(stride, iter);
    }
  }
  template <int NS>
  void launch_plugin_ns(const RolloutArgs<Model>& a)
  {
    rollout_plugin_kernel<Model, NS, RolloutShape<NS, C>::TCH><<<rollout_grid_, NS, 0, stream_>>>(a);
  }
  mppi_status launch_rollout_builtin(int stride, int iter)
  {
    RolloutArgs<Model> a = base_rollout_args();
    if (tile_reduce_active())
    {
      a.tr.partials = tile_part_d_.p;
      a.tr.poff = tile_poff_d_.p;
      a.tr.sums = tile_sums_d_.p;
      a.tr.tmin = tile_min_d_.p;
      a.tr.lambda_inv = 1.0f / cp_.lambda;
    }
    if constexpr (Model::kMlp)
      if (!use_analytic_)
      {
        const FusedNoise fn = fused_noise_args(stride, iter);
        MG_TRY(launch_mlp_rollout(a, mlp_d_.p, mlp_norm(mlp_host_.data()), mlp_precision_, fused() ? &fn : nullptr,
                                  num_sms_, stream_));
        if (judge_total_ == 0) return MPPI_OK;
        JudgeArgs j;
        j.r = a;
        j.num_instances = I_;
        j.sel_off = judge_off_d_.p;
        j.sel_inst = judge_inst_d_.p;
        j.sel = judge_sel_d_.p;
        j.judged_cost = judge_cost_d_.p;
        j.unjudged_min = judge_min_d_.p;
        j.stats = judge_stats_d_.p;
        j.total = judge_total_;
        return launch_judge(j, stream_);
      }
    if constexpr ((4 % C) == 0)
      if (fused() && split_)
      {
        const FusedNoise f = fused_noise_args(stride, iter);
        switch (ns_)
        {
          case 32: rollout_dyn_kernel<Model, 32><<<rollout_grid_, 32, 0, stream_>>>(a, f, states_d_.p); break;
          case 64: rollout_dyn_kernel<Model, 64><<<rollout_grid_, 64, 0, stream_>>>(a, f, states_d_.p); break;
          case 128: rollout_dyn_kernel<Model, 128><<<rollout_grid_, 128, 0, stream_>>>(a, f, states_d_.p); break;
          default: rollout_dyn_kernel<Model, 256><<<rollout_grid_, 256, 0, stream_>>>(a, f, states_d_.p); break;
        }
        MG_CUDA(cudaGetLastError());
        switch (ns_)
        {
          case 32: MG_TRY(launch_cost_kernel<32>(a)); break;
          case 64: MG_TRY(launch_cost_kernel<64>(a)); break;
          case 128: MG_TRY(launch_cost_kernel<128>(a)); break;
          default: MG_TRY(launch_cost_kernel<256>(a)); break;
        }
        return MPPI_OK;
      }
    if constexpr ((4 % C) == 0)
      if (fused() && rollout_mode_ == 2)
      {
        const FusedNoise f = fused_noise_args(stride, iter);
        switch (ns_)
        {
          case 32: rollout_coop_kernel<Model, 32><<<rollout_grid_, 128, 0, stream_>>>(a, f); break;
          case 64: rollout_coop_kernel<Model, 64><<<rollout_grid_, 256, 0, stream_>>>(a, f); break;
          case 128: rollout_coop_kernel<Model, 128><<<rollout_grid_, 512, 0, stream_>>>(a, f); break;
          default: rollout_coop_kernel<Model, 256><<<rollout_grid_, 1024, 0, stream_>>>(a, f); break;
        }
        MG_CUDA(cudaGetLastError());
        return MPPI_OK;
      }
    if constexpr ((4 % C) == 0)
      if (fused())
      {
        const FusedNoise f = fused_noise_args(stride, iter);
        switch (ns_)
        {
          case 32: launch_fused<32>(a, f, iter); break;
          case 64: launch_fused<64>(a, f, iter); break;
          case 128: launch_fused<128>(a, f, iter); break;
          default: launch_fused<256>(a, f, iter); break;
        }
        MG_CUDA(cudaGetLastError());
        return MPPI_OK;
      }
    switch (ns_)
    {
      case 32: launch_rollout_ns<32>(a); break;
      case 64: launch_rollout_ns<64>(a); break;
      case 128: launch_rollout_ns<128>(a); break;
      default: launch_rollout_ns<256>(a); break;
    }
    MG_CUDA(cudaGetLastError());
    return MPPI_OK;
  }

  // The rollout tiles reduce the samples themselves (TileReduce) unless the surrogate rollout is in use (its judge
  // rewrites costs after the rollout) or the weights are Tsallis weights (not a product of a per-tile factor and a
  // tile-local weight, so they need the instance's baseline first); then weights_update_kernel reads the samples
  // again.
  bool tile_reduce_active() const { return !(Model::kMlp && !use_analytic_) && !tsallis() && !rmppi(); }
  // ColoredMPPIController::computeControl's weight choice (colored_mppi_controller.cu:197-207): Tsallis weights when
  // gamma and r are both non-zero, else the exponential transform.
  bool tsallis() const
  {
    return cp_.controller == MPPI_CONTROLLER_COLORED && cp_.tsallis_gamma != 0.0f && cp_.tsallis_r != 0.0f;
  }
  SampleShared sample_shared() const
  {
    SampleShared sh = make_sample_shared(sp_, cc_, cp_.controller == MPPI_CONTROLLER_COLORED ? 1 : 0);
    if (Model::kOwnConstraints || rmppi())
    {
      // the plugin's enforceConstraints replaces the deadband + clamp, and R-MPPI constrains each step's control
      // (with the feedback added) inside its rollout: samples and the smoothed mean leave the GPU unconstrained (an
      // infinite range with no deadband leaves every value as it is)
      for (int c = 0; c < kMaxC; ++c)
      {
        sh.lower[c] = -INFINITY;
        sh.upper[c] = INFINITY;
        sh.deadband[c] = 0.0f;
      }
    }
    return sh;
  }

  // Iteration `iter` of a solve: the combine of the instances (tile partial sums or the weights pass); the last
  // iteration's combine also smooths and clamps the new means and, in a solve whose results go straight to the host
  // block (direct_out_), publishes them there.
  mppi_status launch_weights(int iter)
  {
    if (tail_finalize())  // the fused rollout combined the instances itself
    {
      weights_stale_ = true;
      return MPPI_OK;
    }
    const bool finish = !tube() && !rmppi() && iter == cp_.num_iters - 1;
    const size_t fin_floats = finish ? (size_t)(max_t_ + 4) * C : 0;
    if (tile_reduce_active())
    {
      FinalizeArgs f = finalize_args();
      f.finish = finish ? 1 : 0;
      if (finish && direct_out_)
      {
        f.host_mean = out_mean_h_.p;
        f.host_first = first_h_.p;
        f.host_bn = out_bn_h_.p;
        f.host_stats = out_stats_h_.p;
        f.host_status = status_h_.p;
      }
      const size_t smem = sizeof(float) * std::max((size_t)max_tiles_per_inst_, fin_floats);
      MG_CUDA(raise_smem_cap(tile_finalize_kernel<C>, smem));
      tile_finalize_kernel<C><<<I_, 256, smem, stream_>>>(f, sample_shared());
      MG_CUDA(cudaGetLastError());
      weights_stale_ = true;
      return MPPI_OK;
    }
    weights_stale_ = false;
    WeightsArgs a{};
    a.inst = inst_d_.p;
    a.chunks = chunks_d_.p;
    a.part_off = part_off_d_.p;
    a.inst_chunk0 = chunk0_d_.p;
    a.num_chunks = num_chunks_;
    a.num_instances = I_;
    a.costs = costs_d_.p;
    a.weights = weights_d_.p;
    a.samples = samples_d_.p;
    a.partials = partials_d_.p;
    a.part_w = part_w_d_.p;
    a.baseline_bits = baseline_bits_d_.p;
    a.arrive = arrive_d_.p;
    a.inst_done = counters_d_.p + 2;
    a.noise_counter = counters_d_.p + 3;
    a.mean_out = mean_d_.p;
    a.baseline_norm = bn_d_.p;
    a.stats = stats_d_.p;
    a.lambda_inv = 1.0f / cp_.lambda;
    a.weights_given = 0;
    a.given_norm = nullptr;
    a.transform = tsallis() ? 1 : 0;
    a.tsallis_gamma = cp_.tsallis_gamma;
    a.tsallis_r = cp_.tsallis_r;
    a.finish = finish ? 1 : 0;
    a.first_out = first_d_.p;
    a.sh = sample_shared();
    a.status = status_d_;
    if (finish && direct_out_)
    {
      a.host_mean = out_mean_h_.p;
      a.host_first = first_h_.p;
      a.host_bn = out_bn_h_.p;
      a.host_stats = out_stats_h_.p;
      a.host_status = status_h_.p;
    }
    const size_t smem = sizeof(float) * fin_floats;
    MG_CUDA(raise_smem_cap(weights_update_kernel<C>, smem));
    weights_update_kernel<C><<<num_chunks_, 256, smem, stream_>>>(a);
    MG_CUDA(cudaGetLastError());
    return MPPI_OK;
  }

  // num_iters x (sample, rollout, weights+update), in stream order.
  mppi_status enqueue_kernels(int stride)
  {
    // the smoothing + constraints of the new nominal sequences (the host post-processing of computeControl) run in
    // the last iteration's combine: the fused rollout's finalizing CTAs, tile_finalize_kernel or the weights pass;
    // Tube-MPPI smooths its nominal sequence on the host
    // Tube-MPPI and R-MPPI iterate on the host, one launch per iteration: host_iter_ is that iteration's index (the
    // sampler's std_dev_decay power)
    const bool host_loop = tube() || rmppi();
    for (int it = 0; it < (host_loop ? 1 : cp_.num_iters); ++it)
    {
      const int iter = host_loop ? host_iter_ : it;
      if (!fused()) MG_TRY(launch_sampler(stride, iter));
      MG_TRY(launch_rollout(stride, iter));
      MG_TRY(launch_weights(iter));
    }
    return MPPI_OK;
  }

  // The device work of one computeControl, in stream order.
  mppi_status enqueue_solve(int stride)
  {
    const size_t tc = control_.size();
    (void)tc;
    MG_CUDA(cudaMemcpyAsync(io_d_.p, io_in_h_.p, io_in_bytes_, cudaMemcpyHostToDevice, stream_));
    // the CTAs that finish the solve write the results to the pinned host block themselves
    direct_out_ = !tube() && !rmppi();
    const mppi_status st = enqueue_kernels(stride);
    const bool direct = direct_out_;
    direct_out_ = false;
    MG_TRY(st);
    if (!direct)
      MG_CUDA(cudaMemcpyAsync(io_out_h_.p, io_d_.p + io_out_off_, io_out_bytes_, cudaMemcpyDeviceToHost, stream_));
    return MPPI_OK;
  }

  mppi_status get_graph(int stride, cudaGraphExec_t* exec)
  {
    // a host-iterated solve (Tube-MPPI, R-MPPI) with a decaying sampling deviation captures one graph per iteration
    const int key = ((tube() || rmppi()) && sp_.std_dev_decay != 1.0f) ? stride + (host_iter_ << 20) : stride;
    auto it = graphs_.find(key);
    if (it != graphs_.end())
    {
      *exec = it->second;
      return MPPI_OK;
    }
    cudaGraph_t g = nullptr;
    MG_CUDA(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
    mppi_status st = enqueue_solve(stride);
    cudaError_t ce = cudaStreamEndCapture(stream_, &g);
    if (st != MPPI_OK)
    {
      if (g) cudaGraphDestroy(g);
      (void)cudaGetLastError();  // the invalidated capture's error stays with this call
      return st;
    }
    if (ce != cudaSuccess)
    {
      set_error("cudaStreamEndCapture failed: %s", cudaGetErrorString(ce));
      return MPPI_ECUDA;
    }
    cudaGraphExec_t e = nullptr;
    ce = cudaGraphInstantiate(&e, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess)
    {
      set_error("cudaGraphInstantiate failed: %s", cudaGetErrorString(ce));
      return MPPI_ECUDA;
    }
    graphs_[key] = e;
    *exec = e;
    return MPPI_OK;
  }

  void invalidate_graphs()
  {
    for (auto& kv : graphs_) cudaGraphExecDestroy(kv.second);
    graphs_.clear();
    for (auto& kv : device_graphs_) cudaGraphExecDestroy(kv.second);
    device_graphs_.clear();
  }

  // Host post-processing of computeControl (mppi_controller.cu:208-227).
  mppi_status finish_solve(const float* x0)
  {
    if (status_h_.p[0] != 0u)
    {
      status_h_.p[0] = 0u;
      MG_CUDA(cudaMemsetAsync(status_d_, 0, sizeof(unsigned int), stream_));
      MG_CUDA(cudaStreamSynchronize(stream_));
      set_error("a bounded wait for staged control data gave up inside the rollout kernel");
      return MPPI_ETIMEOUT;
    }
    memcpy(control_.data(), out_mean_h_.p, sizeof(float) * control_.size());
    memcpy(baseline_norm_.data(), out_bn_h_.p, sizeof(float) * 2 * I_);
    memcpy(stats_.data(), out_stats_h_.p, sizeof(double) * 3 * I_);
    // control_ arrives smoothed and constrained (finish_instance in the last combine); first_h_ holds the unclamped
    // first controls
    memcpy(last_pre_smooth_.data(), first_h_.p, sizeof(float) * I_ * C);
    bool bad = false;
    for (int i = 0; i < I_; ++i)
      if (!std::isfinite(baseline_norm_[2 * i]) || !(stats_[3 * i] > 0.0)) bad = true;
    // the nominal state trajectory is rolled out when it is first read (get_state_seq), from these snapshots
    traj_u_ = control_;
    traj_x0_.assign(x0, x0 + (size_t)I_ * S);
    traj_dirty_ = true;
    if constexpr (Model::kOwnConstraints) final_constraints_host();
    if (bad)
    {
      set_error("a sampled cost or the normaliser is not finite (NaN state or noise?)");
      return MPPI_ENAN;
    }
    return MPPI_OK;
  }

  mppi_status copy_per_sample(const float* src_d, float* out)
  {
    MG_CHECK(out, "out must not be NULL");
    MG_CUDA(cudaStreamSynchronize(stream_));
    MG_CUDA(cudaMemcpy(out, src_d, sizeof(float) * total_k_, cudaMemcpyDeviceToHost));
    return MPPI_OK;
  }

  static constexpr int kSampleQuadsPerItem = 2048;

  int I_ = 0;
  std::vector<int> K_, T_, k_off_, t_off_;
  std::vector<long long> u_off_;
  int total_k_ = 0;
  mppi_controller_params cp_{};
  mppi_sampling_params sp_{};
  mppi_control_constraints cc_{};
  std::vector<DynParams> dyn_;
  std::vector<CostParams> cost_;
  ModelAux aux_{};
  std::vector<float> control_, state_seq_, history_, last_pre_smooth_, baseline_norm_, prev_baseline_;
  std::vector<float> traj_u_, traj_x0_;  // constrained nominal controls and x0 of the last solve
  std::vector<float> leashed_x0_;        // ColoredMPPI with the leash on: the initial states the solve starts from
  int leash_jump_ = 1;                   // steps of the last slide (ColoredMPPIController::leash_jump_)
  std::vector<float> nominal_x0_;        // Tube-MPPI: the nominal system's state
  bool nominal_init_ = false;            // Tube-MPPI: nominal_x0_ set (nominalStateInit_)
  int nominal_used_ = 0;                 // Tube-MPPI: the last iteration kept the nominal system
  uint32_t max_polls_ = kMaxProgressPolls;  // rollout mode 4's bounded poll (mppi_set_wait_diagnostics)
  bool withhold_progress_ = false;          // mode 4's noise warps publish no progress (mppi_set_wait_diagnostics)
  bool traj_dirty_ = false;
  int host_iter_ = 0;  // the iteration of a host-iterated solve (Tube-MPPI, R-MPPI) being enqueued
  std::vector<double> stats_;
  bool fb_enabled_ = false;                // Controller::enable_feedback_
  DdpWeights fb_w_;                        // DDPParams: identities and one iteration until set
  std::vector<float> fb_gains_, fb_prop_;  // gains of the feedback instance; feedback-propagated states
  DevBuf<float> fb_gains_d_;               // the gains for R-MPPI's rollout
  // R-MPPI's importance sampler: the last candidate evaluation and the chosen candidate
  std::vector<float> rm_cand_, rm_fe_, rm_eval_;
  std::vector<int> rm_strides_;
  DevBuf<float> rm_cand_d_, rm_eval_d_;
  DevBuf<int> rm_strides_d_;
  int rm_best_ = 0, rm_nominal_stride_ = 0;

  cudaStream_t stream_ = nullptr;
  bool own_stream_ = false;
  int num_sms_ = 1;
  bool graph_mode_ = true;
  std::map<int, cudaGraphExec_t> graphs_, device_graphs_;

  int ns_ = 128;  // rollout samples per CTA
  int kc_ = 128;  // weight/update samples per CTA
  int num_tiles_ = 0, num_chunks_ = 0, num_swork_ = 0, rollout_grid_ = 1;

  DevBuf<float> samples_d_, costs_d_, weights_d_, mean_d_, x0_d_, partials_d_, bn_d_, injected_d_, costmap_d_;
  DevBuf<double> part_w_d_, stats_d_;
  DevBuf<DynParams> dyn_d_;
  DevBuf<CostParams> cost_d_;
  DevBuf<unsigned int> baseline_bits_d_, arrive_d_, counters_d_;
  DevBuf<InstDesc> inst_d_;
  std::vector<InstDesc> inst_h_;  // host copy of inst_d_
  DevBuf<int2> tiles_d_, swork_d_, cwork_d_;
  DevBuf<float> ctab_d_;
  DevBuf<int> ctab_off_d_;
  DevBuf<int4> ctab_parts_d_;
  int num_cwork_ = 0, max_t_ = 1;
  int class_begin_[6] = { 0, 0, 0, 0, 0, 0 };
  DevBuf<int4> chunks_d_;
  DevBuf<long long> part_off_d_;
  DevBuf<int> chunk0_d_;
  PinnedBuf<float> x0_h_, mean_h_, out_mean_h_, out_bn_h_;
  PinnedBuf<double> out_stats_h_;
  PinnedBuf<unsigned int> status_h_;
  DevBuf<float> first_d_;    // per instance: unclamped first control of the last solve (slide history)
  PinnedBuf<float> first_h_;
  // one block per direction for the per-solve copies; x0_d_, mean_d_, first_d_, bn_d_, stats_d_ and the host
  // staging buffers are views into them
  DevBuf<unsigned char> io_d_;
  PinnedBuf<unsigned char> io_in_h_, io_out_h_;
  size_t io_in_bytes_ = 0, io_out_off_ = 0, io_out_bytes_ = 0;
  unsigned int* status_d_ = nullptr;  // set non-zero by a kernel whose bounded wait gave up
  std::vector<float> mlp_host_;  // surrogate parameters as the tensor cores see them (MLP models only)
  DevBuf<float> mlp_d_;
  long long total_u_ = 0;      // control-sample floats over all instances
  bool split_ = false;         // split dynamics / cost rollout (rollout mode 1)
  int rollout_mode_ = 0;       // 0 fused, 1 split, 2 cooperative, 3 sampler kernel + staged, 4 fused + noise warps
  bool direct_out_ = false;    // enqueue_solve: the finishing rollout CTA writes the results to the host block
  // tile reduction (TileReduce): per tile partial rows, (sum w, sum w^2), minimum; first tile of each instance
  DevBuf<float> tile_part_d_;
  DevBuf<long long> tile_poff_d_;
  DevBuf<double> tile_sums_d_;
  DevBuf<unsigned int> tile_min_d_;
  DevBuf<int> inst_tile0_d_;
  DevBuf<unsigned int> inst_tiles_done_d_;
  int max_tiles_per_inst_ = 1, max_k_ = 1;
  bool weights_stale_ = false;  // weights_d_ not yet derived from the last costs
  DevBuf<float> states_d_;     // split rollout: stepped states [instance][k][t][S]
  int mlp_precision_ = 0;      // 0 bf16 / 1 fp8 tensor cores, 2 fp32 CUDA cores
  bool use_analytic_ = false;  // MLP models: roll out the analytic model instead
  float judge_frac_ = 0.01f;   // MLP models: fraction of samples re-rolled by the analytic judge
  int judge_total_ = 0;
  DevBuf<int> judge_off_d_, judge_inst_d_, judge_sel_d_;
  DevBuf<float> judge_cost_d_, judge_stats_d_;
  DevBuf<unsigned int> judge_min_d_;

  // Judged slots per instance: ceil(judge_frac_ * K_i), capped at K_i.
  mppi_status build_judge_lists()
  {
    judge_total_ = 0;
    if (!Model::kMlp || judge_frac_ <= 0.0f) return MPPI_OK;
    std::vector<int> off(I_ + 1, 0), inst;
    for (int i = 0; i < I_; ++i)
    {
      const int m = std::min(K_[i], (int)std::ceil((double)judge_frac_ * K_[i]));
      off[i + 1] = off[i] + m;
      inst.insert(inst.end(), m, i);
    }
    judge_total_ = off[I_];
    MG_TRY(judge_off_d_.alloc(I_ + 1));
    MG_TRY(judge_inst_d_.alloc(std::max(1, judge_total_)));
    MG_TRY(judge_sel_d_.alloc(std::max(1, judge_total_)));
    MG_TRY(judge_cost_d_.alloc(std::max(1, judge_total_)));
    MG_TRY(judge_stats_d_.alloc(2 * I_));
    MG_TRY(judge_min_d_.alloc(I_));
    MG_CUDA(cudaMemcpy(judge_off_d_.p, off.data(), sizeof(int) * (I_ + 1), cudaMemcpyHostToDevice));
    if (judge_total_)
      MG_CUDA(cudaMemcpy(judge_inst_d_.p, inst.data(), sizeof(int) * judge_total_, cudaMemcpyHostToDevice));
    MG_CUDA(cudaMemset(judge_stats_d_.p, 0, sizeof(float) * 2 * I_));
    return MPPI_OK;
  }
  bool use_bulk_ = false;  // every instance has T*C % 4 == 0: stage controls with the bulk-copy engine
};

// Autotuner: times one full solve (non-graph) per candidate launch shape with CUDA events and keeps the fastest.
// Candidates: rollout samples per CTA {32, 64, 128, 256} x update samples per CTA {64, 128, 256}.  The cache is a
// small JSON object {"<key>": [ns, kc], ...} keyed by the model id and the instance shapes.
mppi_status autotune_impl(EngineBase* e, const char* cache_path, const std::string& key,
                          mppi_status (*time_one)(EngineBase*, float*));

template <class Model>
mppi_status Engine<Model>::autotune(const char* cache_path)
{
  std::string key = "m" + std::to_string(Model::kModelId) + "_i" + std::to_string(I_);
  unsigned long long h = 1469598103934665603ULL;
  for (int i = 0; i < I_; ++i)
  {
    h = (h ^ (unsigned long long)K_[i]) * 1099511628211ULL;
    h = (h ^ (unsigned long long)T_[i]) * 1099511628211ULL;
  }
  key += "_" + std::to_string(h);
  auto time_one = [](EngineBase* base, float* ms) -> mppi_status {
    Engine* self = static_cast<Engine*>(base);
    std::vector<float> x0((size_t)self->I_ * S, 0.0f);
    memcpy(self->x0_h_.p, x0.data(), sizeof(float) * x0.size());
    memcpy(self->mean_h_.p, self->control_.data(), sizeof(float) * self->control_.size());
    cudaEvent_t e0, e1;
    MG_CUDA(cudaEventCreate(&e0));
    MG_CUDA(cudaEventCreate(&e1));
    MG_TRY(self->enqueue_solve(1));  // warm-up
    MG_CUDA(cudaEventRecord(e0, self->stream_));
    for (int r = 0; r < 3; ++r) MG_TRY(self->enqueue_solve(1));
    MG_CUDA(cudaEventRecord(e1, self->stream_));
    MG_CUDA(cudaEventSynchronize(e1));
    MG_CUDA(cudaEventElapsedTime(ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return MPPI_OK;
  };
  return autotune_impl(this, cache_path, key, time_one);
}

// Kernel-level rollout of one instance (launchRolloutKernel, mppi_common.cu:1335-1361): temporary descriptors and
// counters are allocated on the stream and freed after the launch.
template <class Model>
mppi_status standalone_rollout(const void* dyn, const void* cost, const mppi_sampling_params* sp, const float* x0_d,
                               const float* controls_d, const float* mean_d, float* costs_d, int K, int T, float dt,
                               float lambda, float alpha, cudaStream_t s)
{
  constexpr int C = Model::CONTROL_DIM;
  constexpr int NS = 128;
  constexpr int TCH = RolloutShape<NS, C>::TCH;
  MG_CHECK(K >= 1 && T >= 1, "K and T must be >= 1");
  MG_CHECK(((uintptr_t)controls_d & 15) == 0, "controls must be 16-byte aligned");
  InstDesc d{};
  d.K = K;
  d.T = T;
  d.num_chunks = 1;
  std::vector<int2> tiles;
  for (int k0 = 0; k0 < K; k0 += NS) tiles.push_back(make_int2(0, k0));
  DevBuf<InstDesc> inst_d;
  DevBuf<int2> tiles_d;
  DevBuf<typename Model::DynParams> dyn_d;
  DevBuf<typename Model::CostParams> cost_d;
  DevBuf<unsigned int> cnt_d;
  MG_TRY(inst_d.alloc(1));
  MG_TRY(tiles_d.alloc(tiles.size()));
  MG_TRY(dyn_d.alloc(1));
  MG_TRY(cost_d.alloc(1));
  MG_TRY(cnt_d.alloc(4));
  MG_CUDA(cudaMemcpyAsync(inst_d.p, &d, sizeof(d), cudaMemcpyHostToDevice, s));
  MG_CUDA(cudaMemcpyAsync(tiles_d.p, tiles.data(), sizeof(int2) * tiles.size(), cudaMemcpyHostToDevice, s));
  MG_CUDA(cudaMemcpyAsync(dyn_d.p, dyn, sizeof(typename Model::DynParams), cudaMemcpyHostToDevice, s));
  MG_CUDA(cudaMemcpyAsync(cost_d.p, cost, sizeof(typename Model::CostParams), cudaMemcpyHostToDevice, s));
  MG_CUDA(cudaMemsetAsync(cnt_d.p, 0, sizeof(unsigned int) * 4, s));
  fill_u32_kernel<<<1, 32, 0, s>>>(cnt_d.p + 2, kOrderedPosInf, 1);
  RolloutArgs<Model> a{};
  a.inst = inst_d.p;
  a.tiles = tiles_d.p;
  a.num_tiles = (int)tiles.size();
  a.dyn = dyn_d.p;
  a.cost = cost_d.p;
  memset(&a.aux, 0, sizeof(a.aux));
  a.x0 = x0_d;
  a.samples = controls_d;
  a.mean = mean_d;
  a.costs = costs_d;
  a.baseline_bits = cnt_d.p + 2;
  a.tile_counter = cnt_d.p;
  a.status = cnt_d.p + 3;
  a.dt = dt;
  a.lambda = lambda;
  a.alpha = alpha;
  a.use_likelihood = 0;
  for (int c = 0; c < C; ++c)
    if (sp->control_cost_coeff[c] != 0.0f) a.use_likelihood = 1;
  mppi_control_constraints cc;
  mppi_default_constraints(&cc);
  a.sh = make_sample_shared(*sp, cc);
  rollout_kernel<Model, NS, TCH><<<(int)tiles.size(), NS, 0, s>>>(a);
  MG_CUDA(cudaGetLastError());
  MG_CUDA(cudaStreamSynchronize(s));
  return MPPI_OK;
}

}  // namespace mg
