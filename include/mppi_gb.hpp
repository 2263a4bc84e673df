/*
 * mppi_gb.hpp — C++ host mirror of MPPI-Generic's plugin / controller surface over the C ABI (mppi_gb.h).
 *
 * Header only, C++17, no CUDA or Eigen types: plugin objects carry the engine's POD parameter blocks, and
 * VanillaMPPIController keeps the reference's template signature and method names
 * (include/mppi/controllers/MPPI/mppi_controller.cuh:14-78, include/mppi/controllers/controller.cuh:70-1058), so a
 * reference-side caller changes its includes and types, not its control loop.  Control trajectories are
 * std::array<float, C * MAX_TIMESTEPS> in the memory order of the reference's column-major Eigen control_trajectory
 * (C x MAX_T): element (c, t) at t * C + c.  Errors surface as mppi_gb::Error exceptions in the caller's code; the C
 * ABI underneath never throws.
 */
#ifndef MPPI_GB_HPP
#define MPPI_GB_HPP

#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "mppi_gb.h"

namespace mppi_gb
{
class Error : public std::runtime_error
{
public:
  Error(mppi_status s, const std::string& what) : std::runtime_error(what), status(s) {}
  mppi_status status;
};

inline void check(mppi_status s, const char* call)
{
  if (s != MPPI_OK) throw Error(s, std::string(call) + ": " + mppi_last_error_string());
}

// ---- Dynamics plugins (Dynamics<CLASS_T, PARAMS_T>, dynamics.cuh:68-72) ------------------------------------------

// Shared part: the control ranges, deadband and zero control of Dynamics::enforceConstraints (dynamics.cu:107-126).
template <int S, int C, int MODEL>
struct DynamicsBase
{
  static constexpr int STATE_DIM = S, CONTROL_DIM = C, OUTPUT_DIM = S;
  static constexpr int MODEL_ID = MODEL;
  mppi_control_constraints constraints;
  DynamicsBase() { mppi_default_constraints(&constraints); }
  // Dynamics::setControlRanges (dynamics.cuh:145): (lower, upper) per control, as the reference's float2 x / y.
  void setControlRanges(const std::array<std::pair<float, float>, C>& ranges)
  {
    for (int i = 0; i < C; ++i)
    {
      constraints.lower[i] = ranges[i].first;
      constraints.upper[i] = ranges[i].second;
    }
  }
  void setControlDeadbands(const std::array<float, C>& deadband)
  {
    for (int i = 0; i < C; ++i) constraints.deadband[i] = deadband[i];
  }
};

// CartpoleDynamics (cartpole_dynamics.cuh): cart mass, pole mass, pole length; g = 9.81.
struct CartpoleDynamics : DynamicsBase<4, 1, MPPI_MODEL_CARTPOLE>
{
  using DYN_PARAMS_T = mppi_cartpole_params;
  DYN_PARAMS_T params;
  explicit CartpoleDynamics(float cart_mass = 1.0f, float pole_mass = 1.0f, float pole_length = 1.0f)
      : params{ cart_mass, pole_mass, pole_length, 9.81f }
  {
  }
  DYN_PARAMS_T getParams() const { return params; }
  void setParams(const DYN_PARAMS_T& p) { params = p; }
};

// DoubleIntegratorDynamics (di_dynamics.cu:46-53): no parameters.
struct DoubleIntegratorDynamics : DynamicsBase<4, 2, MPPI_MODEL_DOUBLE_INTEGRATOR>
{
  using DYN_PARAMS_T = mppi_double_integrator_params;
  DYN_PARAMS_T params{ 0.0f };
  DYN_PARAMS_T getParams() const { return params; }
  void setParams(const DYN_PARAMS_T& p) { params = p; }
};

// Kinematic bicycle (x, y, yaw, v) with control (accel, steer); the engine's plugin (no reference model).
struct BicycleDynamics : DynamicsBase<4, 2, MPPI_MODEL_BICYCLE_COSTMAP>
{
  using DYN_PARAMS_T = mppi_bicycle_params;
  DYN_PARAMS_T params;
  explicit BicycleDynamics(float wheelbase = 2.5f) : params{ wheelbase }
  {
    setControlRanges({ std::pair<float, float>{ -3.0f, 3.0f }, { -1.0f, 1.0f } });
  }
};

// 7-state dynamic bicycle with linear tyres; the engine's plugin (no reference model).
struct BicycleSlipDynamics : DynamicsBase<7, 2, MPPI_MODEL_BICYCLE_SLIP>
{
  using DYN_PARAMS_T = mppi_bicycle_slip_params;
  BicycleSlipDynamics() { setControlRanges({ std::pair<float, float>{ -1.0f, 1.0f }, { -1.0f, 1.0f } }); }
  // mass, yaw inertia, lf, lr, cornering stiffness, max drive force, drag, max steer, steer time constant, min vx
  DYN_PARAMS_T params{ 1500.0f, 2500.0f, 1.2f, 1.3f, 8.0e4f, 4000.0f, 50.0f, 0.5f, 0.1f, 1.0f };
};

// The same vehicle with its derivatives from the learned 9 -> 64 -> 64 -> 5 surrogate (NeuralNetModel,
// ar_nn_model.cu:127-156, evaluated on the tensor cores).  precision: 0 BF16, 1 FP8 E4M3 + per-layer scale, 2 FP32.
struct BicycleSlipMLPDynamics : DynamicsBase<7, 2, MPPI_MODEL_BICYCLE_SLIP_MLP>
{
  using DYN_PARAMS_T = mppi_bicycle_slip_params;
  // mass, yaw inertia, lf, lr, cornering stiffness, max drive force, drag, max steer, steer time constant, min vx
  DYN_PARAMS_T params{ 1500.0f, 2500.0f, 1.2f, 1.3f, 8.0e4f, 4000.0f, 50.0f, 0.5f, 0.1f, 1.0f };
  std::vector<float> network;  // MPPI_MLP_PARAMS floats (FNNHelper layout + scaling)
  int precision = 0;
  float judge_fraction = 0.01f;
  BicycleSlipMLPDynamics() { setControlRanges({ std::pair<float, float>{ -1.0f, 1.0f }, { -1.0f, 1.0f } }); }
  BicycleSlipMLPDynamics(std::vector<float> weights, int precision_ = 0) : BicycleSlipMLPDynamics()
  {
    network = std::move(weights);
    precision = precision_;
  }
};

// ---- Cost plugins (Cost<CLASS_T, PARAMS_T, DYN_PARAMS_T>, cost.cuh:34-35) ----------------------------------------

struct CartpoleSwingupCost
{
  using COST_PARAMS_T = mppi_cartpole_cost_params;
  COST_PARAMS_T params;
  explicit CartpoleSwingupCost(float x_coeff = 10.0f, float x_dot_coeff = 1.0f, float cos_coeff = 100.0f,
                               float theta_dot_coeff = 1.0f, float terminal_coeff = 0.0f)
      : params{ x_coeff, x_dot_coeff, cos_coeff, theta_dot_coeff, terminal_coeff }
  {
  }
  COST_PARAMS_T getParams() const { return params; }
  void setParams(const COST_PARAMS_T& p) { params = p; }
};

struct DoubleIntegratorObstacleCost
{
  using COST_PARAMS_T = mppi_di_obstacle_cost_params;
  COST_PARAMS_T params{};
  DoubleIntegratorObstacleCost()
  {
    for (int i = 0; i < 4; ++i) params.coeff[i] = i < 2 ? 1.0f : 0.1f;
    params.obstacle_cost = 1000.0f;
  }
  void addObstacle(float x, float y, float radius)
  {
    if (params.num_obstacles >= MPPI_MAX_OBSTACLES) throw Error(MPPI_EINVAL, "too many obstacles");
    params.obstacle_x[params.num_obstacles] = x;
    params.obstacle_y[params.num_obstacles] = y;
    params.obstacle_radius[params.num_obstacles] = radius;
    ++params.num_obstacles;
  }
};

// Costmap cost shared by the bicycle models; the map is row-major float[height][width].
struct CostmapCost
{
  using COST_PARAMS_T = mppi_costmap_cost_params;
  COST_PARAMS_T params{ 1.0f, 8.0f, 1.0f, 0.0f, 0.0f };
  std::vector<float> map;
  int width = 0, height = 0;
  float resolution = 0.1f, origin_x = 0.0f, origin_y = 0.0f;
};

// ---- Sampling distributions (GaussianDistribution / ColoredNoiseDistribution) ------------------------------------

struct GaussianDistribution
{
  mppi_sampling_params params;
  GaussianDistribution()
  {
    mppi_default_sampling_params(&params);
    params.kind = MPPI_SAMPLER_GAUSSIAN;
  }
  template <std::size_t C>
  explicit GaussianDistribution(const std::array<float, C>& std_dev) : GaussianDistribution()
  {
    for (std::size_t i = 0; i < C; ++i) params.std_dev[i] = std_dev[i];
  }
};

struct ColoredNoiseDistribution
{
  mppi_sampling_params params;
  ColoredNoiseDistribution()
  {
    mppi_default_sampling_params(&params);
    params.kind = MPPI_SAMPLER_COLORED_NOISE;
  }
  template <std::size_t C>
  ColoredNoiseDistribution(const std::array<float, C>& std_dev, const std::array<float, C>& exponents)
      : ColoredNoiseDistribution()
  {
    for (std::size_t i = 0; i < C; ++i)
    {
      params.std_dev[i] = std_dev[i];
      params.exponents[i] = exponents[i];
    }
  }
};

// ---- the ancillary feedback controller: DDPFeedback<DYN_T, NUM_TIMESTEPS> (feedback_controllers/DDP/ddp.cuh:104-160)

template <int N>
std::array<float, N * N> identity_matrix()
{
  std::array<float, N * N> m{};
  for (int i = 0; i < N; ++i) m[(size_t)i * N + i] = 1.0f;
  return m;
}

// DDPParams (ddp.cuh:16-25): tracking weights Q, Q_f (STATE_DIM x STATE_DIM) and R (CONTROL_DIM x CONTROL_DIM),
// column-major like the reference's Eigen matrices, identities by default, and the number of DDP iterations.
template <class DYN_T>
struct DDPParams
{
  static constexpr int S = DYN_T::STATE_DIM, C = DYN_T::CONTROL_DIM;
  std::array<float, S * S> Q = identity_matrix<S>();
  std::array<float, S * S> Q_f = identity_matrix<S>();
  std::array<float, C * C> R = identity_matrix<C>();
  int num_iterations = 1;
};

// DDPFeedbackState (ddp.cuh:28-37): per step a CONTROL_DIM x STATE_DIM gain, column-major.
template <class DYN_T, int N_TIMESTEPS>
struct DDPFeedbackState
{
  static constexpr int FEEDBACK_SIZE = DYN_T::CONTROL_DIM * DYN_T::STATE_DIM * N_TIMESTEPS;
  static constexpr int NUM_TIMESTEPS = N_TIMESTEPS;
  std::array<float, FEEDBACK_SIZE> fb_gain_traj_{};
  bool operator==(const DDPFeedbackState& other) const { return fb_gain_traj_ == other.fb_gain_traj_; }
};

// The object a controller is built with.  It holds the DDPParams; the controller's handle runs the solver
// (mppi_compute_feedback) on the host after a solve, and setParams reaches every controller built with it, as the
// reference's controller shares the feedback object.
template <class DYN_T, int NUM_TIMESTEPS>
class DDPFeedback
{
public:
  using TEMPLATED_PARAMS = DDPParams<DYN_T>;
  using TEMPLATED_FEEDBACK_STATE = DDPFeedbackState<DYN_T, NUM_TIMESTEPS>;
  DDPFeedback(DYN_T* model, float dt, int num_timesteps = NUM_TIMESTEPS)
      : model_(model), dt_(dt), num_timesteps_(num_timesteps)
  {
  }
  TEMPLATED_PARAMS getParams() const { return params_; }
  void setParams(const TEMPLATED_PARAMS& params)
  {
    params_ = params;
    for (mppi_handle* h : handles_) push(h);
  }
  float getDt() const { return dt_; }
  int getNumTimesteps() const { return num_timesteps_; }

  // used by the controllers built with this object
  void attach(mppi_handle* h)
  {
    handles_.push_back(h);
    push(h);
  }
  void detach(mppi_handle* h) { handles_.erase(std::remove(handles_.begin(), handles_.end(), h), handles_.end()); }

private:
  void push(mppi_handle* h) const
  {
    check(mppi_set_feedback_params(h, params_.Q.data(), params_.Q_f.data(), params_.R.data(), params_.num_iterations),
          "mppi_set_feedback_params");
  }
  DYN_T* model_;
  float dt_;
  int num_timesteps_;
  TEMPLATED_PARAMS params_{};
  std::vector<mppi_handle*> handles_;
};

// No feedback object: the slot of the reference's constructor left empty; turning feedback on then tracks with
// identity weights.
struct NoFeedback
{
};

// ---- VanillaMPPIController<DYN_T, COST_T, FB_T, MAX_TIMESTEPS, NUM_ROLLOUTS, SAMPLING_T> ---------------------------

// Free-energy statistics of the last computeControl (MPPIFreeEnergyStatistics::real_sys, controller.cuh:22-38).
struct FreeEnergyStatistics
{
  float freeEnergyMean, freeEnergyVariance, freeEnergyModifiedVariance, normalizerPercent, increase,
      previousBaseline;
};

template <class DYN_T, class COST_T, class FB_T, int MAX_TIMESTEPS, int NUM_ROLLOUTS,
          class SAMPLING_T = GaussianDistribution>
class VanillaMPPIController
{
public:
  static constexpr int S = DYN_T::STATE_DIM, C = DYN_T::CONTROL_DIM;
  // the template arguments, as the reference's Controller exposes them (controller.cuh:76-95)
  using TEMPLATED_DYNAMICS = DYN_T;
  using TEMPLATED_COSTS = COST_T;
  using TEMPLATED_SAMPLING = SAMPLING_T;
  using TEMPLATED_PARAMS = mppi_controller_params;
  using state_array = std::array<float, S>;
  using control_array = std::array<float, C>;
  using control_trajectory = std::array<float, C * MAX_TIMESTEPS>;  // (c, t) at t * C + c
  using state_trajectory = std::array<float, S * MAX_TIMESTEPS>;
  using sampled_cost_traj = std::vector<float>;

  // mppi_controller.cu:16-29 (Controller::Controller, controller.cuh:111-153); stream is a cudaStream_t or null.
  using TEMPLATED_FEEDBACK_STATE = DDPFeedbackState<DYN_T, MAX_TIMESTEPS>;
  using TEMPLATED_FEEDBACK_PARAMS = DDPParams<DYN_T>;

  VanillaMPPIController(DYN_T* model, COST_T* cost, FB_T* fb_controller, SAMPLING_T* sampler, float dt,
                        int max_iter, float lambda, float alpha, int num_timesteps = MAX_TIMESTEPS,
                        const control_trajectory& init_control_traj = control_trajectory{}, void* stream = nullptr,
                        uint64_t seed = 0)
      : VanillaMPPIController(1, model, cost, fb_controller, sampler,
                              make_params(dt, max_iter, lambda, alpha, num_timesteps, seed), init_control_traj, stream)
  {
  }

protected:
  static mppi_controller_params make_params(float dt, int max_iter, float lambda, float alpha, int num_timesteps,
                                            uint64_t seed, int controller = MPPI_CONTROLLER_VANILLA)
  {
    mppi_controller_params p;
    mppi_default_controller_params(&p);
    p.dt = dt;
    p.num_iters = max_iter;
    p.lambda = lambda;
    p.alpha = alpha;
    p.num_timesteps = num_timesteps;
    p.seed = seed;
    p.controller = controller;
    return p;
  }
  // A handle of `distributions` instances of NUM_ROLLOUTS x num_timesteps (two for Tube-MPPI and R-MPPI, the
  // reference's sampling distributions), every instance starting from init_control_traj.
  VanillaMPPIController(int distributions, DYN_T* model, COST_T* cost, FB_T* fb_controller, SAMPLING_T* sampler,
                        const mppi_controller_params& params, const control_trajectory& init_control_traj,
                        void* stream)
      : T_(params.num_timesteps), D_(distributions), constraints_(model->constraints), params_(params)
  {
    if (T_ < 1 || T_ > MAX_TIMESTEPS) throw Error(MPPI_EINVAL, "num_timesteps out of range");
    std::vector<int> K(D_, NUM_ROLLOUTS), T(D_, T_);
    std::vector<float> init((size_t)D_ * T_ * C);
    for (int d = 0; d < D_; ++d) std::copy(init_control_traj.begin(), init_control_traj.begin() + T_ * C,
                                           init.begin() + (size_t)d * T_ * C);
    std::vector<typename DYN_T::DYN_PARAMS_T> dyn(D_, model->params);
    std::vector<typename COST_T::COST_PARAMS_T> cst(D_, cost->params);
    check(mppi_create(DYN_T::MODEL_ID, D_, K.data(), T.data(), &params_, &sampler->params, &model->constraints,
                      dyn.data(), sizeof(model->params), cst.data(), sizeof(cost->params), init.data(), stream, &h_),
          "mppi_create");
    try
    {
      configure(*model, *cost);
      // the feedback object's parameters go to the handle; feedback stays off until initFeedback()
      if constexpr (!std::is_same<FB_T, NoFeedback>::value)
      {
        if (fb_controller)
        {
          fb_controller->attach(h_);
          fb_ = fb_controller;
        }
      }
      else
      {
        (void)fb_controller;
      }
    }
    catch (...)
    {
      mppi_destroy(h_);
      throw;
    }
  }

public:
  ~VanillaMPPIController()
  {
    if constexpr (!std::is_same<FB_T, NoFeedback>::value)
      if (fb_) fb_->detach(h_);
    if (h_) mppi_destroy(h_);
  }
  VanillaMPPIController(const VanillaMPPIController&) = delete;
  VanillaMPPIController& operator=(const VanillaMPPIController&) = delete;

  // VanillaMPPIController::computeControl (mppi_controller.cu:152-237).
  void computeControl(const state_array& state, int optimization_stride = 1)
  {
    check(mppi_compute_control(h_, state.data(), optimization_stride), "mppi_compute_control");
  }
  // Controller::getControlSeq (controller.cuh:425-428): the first num_timesteps columns are the solution.
  control_trajectory getControlSeq() const { return control_of(seq_instance_); }
  // Controller::setParams with init_control_traj_ (controller.cuh:857-876); every distribution gets the sequence.
  void setControlSeq(const control_trajectory& u)
  {
    std::vector<float> all((size_t)D_ * T_ * C);
    for (int d = 0; d < D_; ++d) std::copy(u.begin(), u.begin() + T_ * C, all.begin() + (size_t)d * T_ * C);
    check(mppi_set_control_seq(h_, all.data()), "mppi_set_control_seq");
  }
  // Controller::updateImportanceSamplingControl (controller.cuh:322-329): nothing here; the robust controller's
  // replaces it.  BasePlant calls it before every slide (base_plant.hpp:536-540).
  void updateImportanceSamplingControl(const state_array&, int) {}
  // Controller::slideControlSequence (controller.cuh:370-376).
  void slideControlSequence(int steps)
  {
    check(mppi_slide_control_sequence(h_, steps), "mppi_slide_control_sequence");
  }
  // Controller::getTargetStateSeq (controller.cuh:433).
  state_trajectory getTargetStateSeq() const { return state_of(target_instance_); }
  // Controller::getBaselineCost / getNormalizerCost (controller.cuh:526-533) of distribution ind.
  float getBaselineCost(int ind = 0) const { return baseline_normalizer(2 * ind); }
  float getNormalizerCost(int ind = 0) const { return baseline_normalizer(2 * ind + 1); }
  // Controller::getSampledCostSeq (controller.cuh:449-452): the weights the transform leaves in the cost array (of the
  // distribution the controller reports: the real system's for R-MPPI, the actual one's for Tube-MPPI).
  sampled_cost_traj getSampledCostSeq() const
  {
    sampled_cost_traj all((size_t)D_ * NUM_ROLLOUTS);
    check(mppi_get_sample_weights(h_, all.data()), "mppi_get_sample_weights");
    return sampled_cost_traj(all.begin() + (size_t)cost_instance_ * NUM_ROLLOUTS,
                             all.begin() + (size_t)(cost_instance_ + 1) * NUM_ROLLOUTS);
  }
  // Per-sample trajectory costs before the weight transform (same distribution).
  sampled_cost_traj getSampleCosts() const
  {
    sampled_cost_traj all((size_t)D_ * NUM_ROLLOUTS);
    check(mppi_get_sample_costs(h_, all.data()), "mppi_get_sample_costs");
    return sampled_cost_traj(all.begin() + (size_t)cost_instance_ * NUM_ROLLOUTS,
                             all.begin() + (size_t)(cost_instance_ + 1) * NUM_ROLLOUTS);
  }
  // Controller::setParams / getParams (controller.cuh:842-876) for lambda, alpha, dt, iterations and slide scale.
  void setParams(const mppi_controller_params& p)
  {
    check(mppi_set_controller_params(h_, &p), "mppi_set_controller_params");
    params_ = p;
  }
  mppi_controller_params getParams() const { return params_; }
  // Controller::setSamplingParams (controller.cuh:852).
  void setSamplingParams(const SAMPLING_T& sampler)
  {
    check(mppi_set_sampling_params(h_, &sampler.params), "mppi_set_sampling_params");
  }
  // Dynamics / Cost setParams after a change on the plugin objects.
  void updateModel(const DYN_T& model)
  {
    check(mppi_set_dynamics_params(h_, &model.params, sizeof(model.params)), "mppi_set_dynamics_params");
  }
  void updateCost(const COST_T& cost)
  {
    check(mppi_set_cost_params(h_, &cost.params, sizeof(cost.params)), "mppi_set_cost_params");
  }
  // Dynamics::setParams / Cost::setParams from a parameter block (what BasePlant::updateParameters hands over).
  void setDynamicsParams(const typename DYN_T::DYN_PARAMS_T& p)
  {
    check(mppi_set_dynamics_params(h_, &p, sizeof(p)), "mppi_set_dynamics_params");
  }
  void setCostParams(const typename COST_T::COST_PARAMS_T& p)
  {
    check(mppi_set_cost_params(h_, &p, sizeof(p)), "mppi_set_cost_params");
  }
  int getNumTimesteps() const { return T_; }
  float getDt() const { return params_.dt; }
  // Controller::getFreeEnergyStatistics (controller.cuh:540-543).
  FreeEnergyStatistics getFreeEnergyStatistics() const
  {
    float v[6];
    check(mppi_get_free_energy(h_, 0, v), "mppi_get_free_energy");
    return FreeEnergyStatistics{ v[0], v[1], v[2], v[3], v[4], v[5] };
  }
  mppi_handle* handle() const { return h_; }

  // Sampled trajectories for visualisation (Controller::setTopNSampledControlTrajectoriesHelper, controller.cuh:762;
  // calculateSampledStateTrajectories, mppi_controller.cu:280-284; getSampledOutputTrajectories /
  // getSampledCostTrajectories / getTopTransformedCosts, controller.cuh:281-314).  The top-N samples by weight of
  // the last computeControl are re-rolled on the GPU; extra sample indices (a random share, as
  // copySampledControlFromDevice draws them) can be passed in front of them.
  void setTopNSampledControlTrajectories(int n) { top_n_ = n; }
  void calculateSampledStateTrajectories(const std::vector<int>& extra_samples = {})
  {
    std::vector<int> idx(extra_samples);
    sampled_cost_traj w;
    if (top_n_ > 0)
    {
      w = getSampledCostSeq();
      std::vector<int> top(top_n_);
      check(mppi_select_top_samples(w.data(), NUM_ROLLOUTS, top_n_, top.data()), "mppi_select_top_samples");
      idx.insert(idx.end(), top.begin(), top.end());
    }
    const int n = (int)idx.size();
    sampled_states_.assign((size_t)n * T_ * S, 0.0f);
    sampled_costs_.assign((size_t)n * T_, 0.0f);
    sampled_terminal_.assign((size_t)n, 0.0f);
    if (n > 0)
      check(mppi_get_sampled_trajectories(h_, 0, idx.data(), n, sampled_states_.data(), sampled_costs_.data(),
                                          sampled_terminal_.data(), nullptr),
            "mppi_get_sampled_trajectories");
    top_costs_.clear();
    const float norm = top_n_ > 0 ? getNormalizerCost() : 1.0f;
    for (int j = n - top_n_; j < n && top_n_ > 0; ++j) top_costs_.push_back(w[idx[j]] / norm);
    sampled_idx_ = idx;
  }
  // Per re-rolled sample: states [t][s] (the outputs equal the states for these models) and step costs [t].
  std::vector<std::vector<float>> getSampledOutputTrajectories() const
  {
    std::vector<std::vector<float>> out;
    for (size_t j = 0; j < sampled_idx_.size(); ++j)
      out.emplace_back(sampled_states_.begin() + j * T_ * S, sampled_states_.begin() + (j + 1) * T_ * S);
    return out;
  }
  std::vector<std::vector<float>> getSampledCostTrajectories() const
  {
    std::vector<std::vector<float>> out;
    for (size_t j = 0; j < sampled_idx_.size(); ++j)
      out.emplace_back(sampled_costs_.begin() + j * T_, sampled_costs_.begin() + (j + 1) * T_);
    return out;
  }
  std::vector<float> getTopTransformedCosts() const { return top_costs_; }

  // ---- the feedback controller (Controller, controller.cuh:265-269, 347-414, 495-571, 730-743)
  // The enabled flag is kept here as well, so that getCurrentControl (called by a plant's state-estimator thread
  // while another thread optimises) does not enter the handle.
  void initFeedback()
  {
    check(mppi_enable_feedback(h_, 1), "mppi_enable_feedback");
    fb_enabled_ = true;
  }
  void disableFeedbackController()
  {
    check(mppi_enable_feedback(h_, 0), "mppi_enable_feedback");
    fb_enabled_ = false;
  }
  bool getFeedbackEnabled() const { return fb_enabled_.load(); }
  void setFeedbackParams(const TEMPLATED_FEEDBACK_PARAMS& p)
  {
    check(mppi_set_feedback_params(h_, p.Q.data(), p.Q_f.data(), p.R.data(), p.num_iterations),
          "mppi_set_feedback_params");
  }
  // Controller::computeFeedback(state): DDP from `state` around the nominal trajectory of the last solve.
  void computeFeedback(const state_array& state)
  {
    check(mppi_compute_feedback(h_, state.data()), "mppi_compute_feedback");
  }
  TEMPLATED_FEEDBACK_STATE getFeedbackState() const
  {
    TEMPLATED_FEEDBACK_STATE fb{};
    check(mppi_get_feedback_gains(h_, fb.fb_gain_traj_.data()), "mppi_get_feedback_gains");
    return fb;
  }
  // Controller::getFeedbackControl: K_t (state - goal_state).
  control_array getFeedbackControl(const state_array& state, const state_array& goal_state, int t) const
  {
    control_array u{};
    check(mppi_get_feedback_control(h_, state.data(), goal_state.data(), t, u.data()), "mppi_get_feedback_control");
    return u;
  }
  void computeFeedbackPropagatedStateSeq()
  {
    check(mppi_get_feedback_propagated_state_seq(h_, fb_prop_.data()), "mppi_get_feedback_propagated_state_seq");
  }
  state_trajectory getFeedbackPropagatedStateSeq() const { return fb_prop_; }
  // Controller::interpolateControls / interpolateState (controller.cuh:383-403): linear between the bracketing
  // steps (both indices held inside the horizon, where the reference reads column lower + 1 unchecked).
  control_array interpolateControls(double rel_time, const control_trajectory& c_traj) const
  {
    int lo, hi;
    const double a = bracket(rel_time, &lo, &hi);
    control_array u{};
    for (int c = 0; c < C; ++c)
      u[c] = (float)((1.0 - a) * c_traj[(size_t)lo * C + c] + a * c_traj[(size_t)hi * C + c]);
    return u;
  }
  state_array interpolateState(const state_trajectory& s_traj, double rel_time) const
  {
    int lo, hi;
    const double a = bracket(rel_time, &lo, &hi);
    state_array x{};
    for (int s = 0; s < S; ++s)
      x[s] = (float)((1.0 - a) * s_traj[(size_t)lo * S + s] + a * s_traj[(size_t)hi * S + s]);
    return x;
  }
  // FeedbackController::interpolateFeedback_ (feedback.cuh:216-228): the gains of the bracketing steps blended.
  control_array interpolateFeedback(const state_array& state, const state_array& target_nominal_state,
                                    double rel_time, const TEMPLATED_FEEDBACK_STATE& fb_state) const
  {
    int lo, hi;
    const double a = bracket(rel_time, &lo, &hi);
    control_array u{};
    for (int r = 0; r < C; ++r)
    {
      float k_lo = 0.0f, k_hi = 0.0f;
      for (int c = 0; c < S; ++c)
      {
        const float e = state[c] - target_nominal_state[c];
        k_lo += fb_state.fb_gain_traj_[(size_t)lo * C * S + r + (size_t)c * C] * e;
        k_hi += fb_state.fb_gain_traj_[(size_t)hi * C * S + r + (size_t)c * C] * e;
      }
      u[r] = (float)((1.0 - a) * k_lo + a * k_hi);
    }
    return u;
  }
  // Controller::getCurrentControl (controller.cuh:347-362): nominal control at rel_time plus, with feedback on,
  // the interpolated feedback, then the constraints with a zero state (deadband, then clamp; dynamics.cu:107-126).
  control_array getCurrentControl(const state_array& state, double rel_time, const state_array& target_nominal_state,
                                  const control_trajectory& c_traj, const TEMPLATED_FEEDBACK_STATE& fb_state) const
  {
    control_array u = interpolateControls(rel_time, c_traj);
    if (getFeedbackEnabled())
    {
      const control_array fb = interpolateFeedback(state, target_nominal_state, rel_time, fb_state);
      for (int c = 0; c < C; ++c) u[c] += fb[c];
    }
    for (int c = 0; c < C; ++c)
    {
      const float db = constraints_.deadband[c];
      if (std::fabs(u[c]) < db)
        u[c] = constraints_.zero_control[c];
      else
        u[c] += db * -(float)((u[c] > 0.0f) - (u[c] < 0.0f));
      u[c] = std::fmin(std::fmax(constraints_.lower[c], u[c]), constraints_.upper[c]);
    }
    return u;
  }

protected:
  control_trajectory control_of(int d) const
  {
    std::vector<float> all((size_t)D_ * T_ * C);
    check(mppi_get_control_seq(h_, all.data()), "mppi_get_control_seq");
    control_trajectory out{};
    std::copy(all.begin() + (size_t)d * T_ * C, all.begin() + (size_t)(d + 1) * T_ * C, out.begin());
    return out;
  }
  state_trajectory state_of(int d) const
  {
    std::vector<float> all((size_t)D_ * T_ * S);
    check(mppi_get_state_seq(h_, all.data()), "mppi_get_state_seq");
    state_trajectory out{};
    std::copy(all.begin() + (size_t)d * T_ * S, all.begin() + (size_t)(d + 1) * T_ * S, out.begin());
    return out;
  }
  double bracket(double rel_time, int* lo, int* hi) const
  {
    const double dt = params_.dt;
    const int lower = (int)(rel_time / dt);
    *lo = std::min(std::max(lower, 0), T_ - 1);
    *hi = std::min(std::max(lower + 1, 0), T_ - 1);
    return (rel_time - lower * dt) / dt;
  }

  float baseline_normalizer(int which) const
  {
    std::vector<float> bn((size_t)2 * D_);
    check(mppi_get_baseline_normalizer(h_, bn.data(), nullptr), "mppi_get_baseline_normalizer");
    return bn.at(which);
  }
  template <class D, class Co>
  void configure(const D& model, const Co& cost)
  {
    if constexpr (std::is_same<Co, CostmapCost>::value)
      if (!cost.map.empty())
        check(mppi_set_costmap(h_, cost.map.data(), cost.width, cost.height, cost.resolution, cost.origin_x,
                               cost.origin_y),
              "mppi_set_costmap");
    if constexpr (std::is_same<D, BicycleSlipMLPDynamics>::value)
    {
      if (!model.network.empty())
        check(mppi_set_mlp(h_, model.network.data(), model.network.size(), model.precision), "mppi_set_mlp");
      check(mppi_set_judge(h_, model.judge_fraction), "mppi_set_judge");
    }
  }

  mppi_handle* h_ = nullptr;
  int T_ = MAX_TIMESTEPS;
  int D_ = 1;               // sampling distributions (instances) of the handle
  int seq_instance_ = 0;    // the distribution getControlSeq returns
  int target_instance_ = 0; // the distribution getTargetStateSeq returns
  int cost_instance_ = 0;   // the distribution getSampledCostSeq returns
  mppi_control_constraints constraints_{};
  FB_T* fb_ = nullptr;
  std::atomic<bool> fb_enabled_{ false };
  state_trajectory fb_prop_{};
  mppi_controller_params params_{};
  int top_n_ = 0;
  std::vector<int> sampled_idx_;
  std::vector<float> sampled_states_, sampled_costs_, sampled_terminal_, top_costs_;
};

// ---- ColoredMPPIController (controllers/ColoredMPPI/colored_mppi_controller.cuh:40-196) ----------------------------
// The MPPI iteration with Tsallis weights once gamma and r are both non-zero, an optional state leash and, after
// smoothing, a clamp of control 1 only.
template <class DYN_T, class COST_T, class FB_T, int MAX_TIMESTEPS, int NUM_ROLLOUTS,
          class SAMPLING_T = ColoredNoiseDistribution>
class ColoredMPPIController : public VanillaMPPIController<DYN_T, COST_T, FB_T, MAX_TIMESTEPS, NUM_ROLLOUTS, SAMPLING_T>
{
  using Base = VanillaMPPIController<DYN_T, COST_T, FB_T, MAX_TIMESTEPS, NUM_ROLLOUTS, SAMPLING_T>;

public:
  using typename Base::control_trajectory;
  ColoredMPPIController(DYN_T* model, COST_T* cost, FB_T* fb_controller, SAMPLING_T* sampler, float dt, int max_iter,
                        float lambda, float alpha, int num_timesteps = MAX_TIMESTEPS,
                        const control_trajectory& init_control_traj = control_trajectory{}, void* stream = nullptr,
                        uint64_t seed = 0)
      : Base(1, model, cost, fb_controller, sampler,
             Base::make_params(dt, max_iter, lambda, alpha, num_timesteps, seed, MPPI_CONTROLLER_COLORED),
             init_control_traj, stream)
  {
  }
  void setGamma(float gamma) { update([&](mppi_controller_params& p) { p.tsallis_gamma = gamma; }); }
  float getGamma() const { return this->params_.tsallis_gamma; }
  void setRExp(float r) { update([&](mppi_controller_params& p) { p.tsallis_r = r; }); }
  float getRExp() const { return this->params_.tsallis_r; }
  void setLeashActive(bool active) { update([&](mppi_controller_params& p) { p.leash_active = active ? 1 : 0; }); }
  bool getLeashActive() const { return this->params_.leash_active != 0; }
  void setStateLeashLength(float length, int index)
  {
    update([&](mppi_controller_params& p) { p.state_leash_dist[index] = length; });
  }
  float getStateLeashLength(int index) const { return this->params_.state_leash_dist[index]; }

private:
  template <class F>
  void update(F&& f)
  {
    mppi_controller_params p = this->params_;
    f(p);
    this->setParams(p);
  }
};

// ---- TubeMPPIController (controllers/Tube-MPPI/tube_mppi_controller.cuh:29-141) ------------------------------------
// Two distributions, the actual system (0) and the nominal system (1); getControlSeq / getTargetStateSeq are the
// nominal system's; the feedback controller is on from construction and tracks the nominal system.
template <class DYN_T, class COST_T, class FB_T, int MAX_TIMESTEPS, int NUM_ROLLOUTS,
          class SAMPLING_T = GaussianDistribution>
class TubeMPPIController : public VanillaMPPIController<DYN_T, COST_T, FB_T, MAX_TIMESTEPS, NUM_ROLLOUTS, SAMPLING_T>
{
  using Base = VanillaMPPIController<DYN_T, COST_T, FB_T, MAX_TIMESTEPS, NUM_ROLLOUTS, SAMPLING_T>;

public:
  using typename Base::control_trajectory;
  using typename Base::state_trajectory;
  TubeMPPIController(DYN_T* model, COST_T* cost, FB_T* fb_controller, SAMPLING_T* sampler, float dt, int max_iter,
                     float lambda, float alpha, int num_timesteps = MAX_TIMESTEPS,
                     const control_trajectory& init_control_traj = control_trajectory{}, void* stream = nullptr,
                     uint64_t seed = 0, float nominal_threshold = 20.0f)
      : Base(2, model, cost, fb_controller, sampler, tube_params(dt, max_iter, lambda, alpha, num_timesteps, seed,
                                                                 nominal_threshold),
             init_control_traj, stream)
  {
    this->seq_instance_ = 1;
    this->target_instance_ = 1;
    this->initFeedback();
  }
  control_trajectory getActualControlSeq() const { return this->control_of(0); }
  state_trajectory getActualStateSeq() const { return this->state_of(0); }
  float getNominalThreshold() const { return this->params_.nominal_threshold; }
  void setNominalThreshold(float threshold)
  {
    mppi_controller_params p = this->params_;
    p.nominal_threshold = threshold;
    this->setParams(p);
  }
  // FreeEnergyStatistics::nominal_state_used of the last computeControl
  int getNominalStateUsed() const
  {
    int used = 0;
    check(mppi_get_nominal_state_used(this->h_, &used), "mppi_get_nominal_state_used");
    return used;
  }

private:
  static mppi_controller_params tube_params(float dt, int max_iter, float lambda, float alpha, int T, uint64_t seed,
                                            float threshold)
  {
    mppi_controller_params p = Base::make_params(dt, max_iter, lambda, alpha, T, seed, MPPI_CONTROLLER_TUBE);
    p.nominal_threshold = threshold;
    return p;
  }
};

// ---- RobustMPPIController (controllers/R-MPPI/robust_mppi_controller.cuh:59-322) -----------------------------------
// Two distributions in the reference's order, nominal (0) and real (1); updateImportanceSamplingControl before each
// computeControl; getControlSeq is the real system's sequence, getTargetStateSeq the nominal trajectory;
// slideControlSequence and computeFeedback do nothing, as in the reference.
template <class DYN_T, class COST_T, class FB_T, int MAX_TIMESTEPS, int NUM_ROLLOUTS,
          class SAMPLING_T = GaussianDistribution>
class RobustMPPIController : public VanillaMPPIController<DYN_T, COST_T, FB_T, MAX_TIMESTEPS, NUM_ROLLOUTS, SAMPLING_T>
{
  using Base = VanillaMPPIController<DYN_T, COST_T, FB_T, MAX_TIMESTEPS, NUM_ROLLOUTS, SAMPLING_T>;

public:
  using typename Base::control_trajectory;
  using typename Base::state_array;
  RobustMPPIController(DYN_T* model, COST_T* cost, FB_T* fb_controller, SAMPLING_T* sampler, float dt, int max_iter,
                       float lambda, float alpha, float value_function_threshold, int num_timesteps = MAX_TIMESTEPS,
                       const control_trajectory& init_control_traj = control_trajectory{},
                       int num_candidate_nominal_states = 9, int optimization_stride = 1, void* stream = nullptr,
                       uint64_t seed = 0, int num_eval_samples_per_candidate = 64)
      : Base(2, model, cost, fb_controller, sampler,
             rmppi_params(dt, max_iter, lambda, alpha, num_timesteps, seed, value_function_threshold,
                          num_candidate_nominal_states, num_eval_samples_per_candidate),
             init_control_traj, stream),
        optimization_stride_(optimization_stride)
  {
    this->seq_instance_ = 1;
    this->target_instance_ = 0;
    this->cost_instance_ = 1;
    this->initFeedback();
  }
  // RobustMPPIController::updateImportanceSamplingControl (robust_mppi_controller.cu:548-569)
  void updateImportanceSamplingControl(const state_array& state, int stride)
  {
    check(mppi_rmppi_update_importance_sampler(this->h_, state.data(), stride), "mppi_rmppi_update_importance_sampler");
  }
  state_array getNominalState() const
  {
    const auto s = this->state_of(0);
    state_array x{};
    std::copy(s.begin(), s.begin() + Base::S, x.begin());
    return x;
  }
  int getBestIndex() const
  {
    int best = 0;
    check(mppi_rmppi_get_candidates(this->h_, &best, nullptr, nullptr, nullptr, nullptr, nullptr),
          "mppi_rmppi_get_candidates");
    return best;
  }
  std::vector<float> getCandidateFreeEnergy() const
  {
    std::vector<float> fe(this->params_.num_candidate_nominal_states);
    check(mppi_rmppi_get_candidates(this->h_, nullptr, nullptr, nullptr, nullptr, fe.data(), nullptr),
          "mppi_rmppi_get_candidates");
    return fe;
  }
  float getValueFunctionThreshold() const { return this->params_.value_function_threshold; }
  int getNumCandidates() const { return this->params_.num_candidate_nominal_states; }
  int getOptimizationStride() const { return optimization_stride_; }

private:
  static mppi_controller_params rmppi_params(float dt, int max_iter, float lambda, float alpha, int T, uint64_t seed,
                                             float threshold, int candidates, int eval_samples)
  {
    mppi_controller_params p = Base::make_params(dt, max_iter, lambda, alpha, T, seed, MPPI_CONTROLLER_RMPPI);
    p.value_function_threshold = threshold;
    p.num_candidate_nominal_states = candidates;
    p.num_eval_samples_per_candidate = eval_samples;
    return p;
  }
  int optimization_stride_;
};

}  // namespace mppi_gb

#endif  // MPPI_GB_HPP
