/*
 * mppi_gb_plant.hpp — BasePlant<CONTROLLER_T>, the receding-horizon driver of MPPI-Generic
 * (include/mppi/core/base_plant.hpp:24-620), for controllers of the C++ mirror (mppi_gb.hpp).
 *
 * A plant owns a controller and runs it against a robot.  The state estimator calls updateState(state, time), which
 * publishes (pubControl) the control for that time from the latest solution; runControlLoop re-optimises at hz from
 * the newest state, sliding the nominal sequence by the robot time that passed (at least the target stride).
 * Parameter blocks may be handed in from any thread (set*Params) and are applied between optimisations
 * (updateParameters).  A subclass provides the robot side: pubControl, pubNominalState, pubFreeEnergyStatistics,
 * checkStatus, getCurrentTime and getPoseTime, as in the reference.
 *
 * With the controller's feedback on, every solve is followed by the DDP feedback computation (computeFeedback from
 * the state optimised from) and the published control is the controller's getCurrentControl: the nominal control
 * at the requested time plus the interpolated feedback against the interpolated nominal state, constrained.
 *
 * Differences from the reference: no buffered-dynamics hook, and the wait for a new state is bounded (max_wait_s),
 * after which the iteration returns false instead of spinning forever.
 */
#ifndef MPPI_GB_PLANT_HPP
#define MPPI_GB_PLANT_HPP

#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <cmath>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <thread>

#include "mppi_gb.hpp"

namespace mppi_gb
{
template <class CONTROLLER_T>
class BasePlant
{
public:
  static constexpr int S = CONTROLLER_T::S, C = CONTROLLER_T::C;
  using s_array = typename CONTROLLER_T::state_array;
  using c_array = typename CONTROLLER_T::control_array;
  using s_traj = typename CONTROLLER_T::state_trajectory;
  using c_traj = typename CONTROLLER_T::control_trajectory;
  using DYN_PARAMS_T = typename CONTROLLER_T::TEMPLATED_DYNAMICS::DYN_PARAMS_T;
  using COST_PARAMS_T = typename CONTROLLER_T::TEMPLATED_COSTS::COST_PARAMS_T;
  using CONTROLLER_PARAMS_T = typename CONTROLLER_T::TEMPLATED_PARAMS;
  using SAMPLER_T = typename CONTROLLER_T::TEMPLATED_SAMPLING;
  using FB_STATE_T = typename CONTROLLER_T::TEMPLATED_FEEDBACK_STATE;

  std::shared_ptr<CONTROLLER_T> controller_;

  // BasePlant(controller, hz, optimization_stride) (base_plant.hpp:131-145)
  BasePlant(std::shared_ptr<CONTROLLER_T> controller, int hz, int optimization_stride)
      : controller_(std::move(controller)), hz_(hz), optimization_stride_(optimization_stride)
  {
    state_.fill(0.0f);
    state_traj_.fill(0.0f);
    control_traj_.fill(0.0f);
  }
  virtual ~BasePlant() = default;

  // ---- the robot side (pure virtual in the reference, base_plant.hpp:147-169)
  virtual void pubControl(const c_array& u) = 0;
  virtual void pubNominalState(const s_array& s) = 0;
  virtual void pubFreeEnergyStatistics(const FreeEnergyStatistics& fe_stats) = 0;
  virtual int checkStatus() = 0;
  virtual double getCurrentTime() = 0;
  virtual double getPoseTime() = 0;

  // ---- state and timing
  virtual double getStateTime() { return state_time_.load(); }
  virtual s_array getState()
  {
    std::lock_guard<std::mutex> lck(access_guard_);
    return state_;
  }
  s_traj getStateTraj()
  {
    std::lock_guard<std::mutex> lck(access_guard_);
    return state_traj_;
  }
  c_traj getControlTraj()
  {
    std::lock_guard<std::mutex> lck(access_guard_);
    return control_traj_;
  }
  void setDebugMode(bool mode) { debug_mode_ = mode; }
  void resetStateTime() { last_used_state_update_time_ = -1.0; }
  FB_STATE_T getFeedbackState()
  {
    std::lock_guard<std::mutex> lck(access_guard_);
    return feedback_state_;
  }
  double getAvgFeedbackTime() const { return avg_feedback_time_ms_; }
  double getAvgOptimizationTime() const { return avg_optimize_time_ms_; }
  double getAvgLoopTime() const { return avg_loop_time_ms_; }
  int getTargetOptimizationStride() const { return optimization_stride_; }
  int getLastOptimizationStride() const { return last_optimization_stride_; }
  void setTargetOptimizationStride(int new_val) { optimization_stride_ = new_val; }
  int getHz() const { return hz_; }
  void setHz(int hz) { hz_ = hz; }
  int getNumIterations() const { return num_iter_; }

  // BasePlant::setSolution (base_plant.hpp:274-287)
  virtual void setSolution(const s_traj& state_seq, const c_traj& control_seq, const FB_STATE_T& fb_state,
                           double timestamp)
  {
    std::lock_guard<std::mutex> guard(access_guard_);
    last_used_state_update_time_ = timestamp;
    state_traj_ = state_seq;
    control_traj_ = control_seq;
    feedback_state_ = fb_state;
    ++num_iter_;
  }

  // BasePlant::updateState (base_plant.hpp:289-321): store the estimate and, once a solution exists and `time` lies
  // inside its horizon after the state it was computed from, publish the control for `time`.
  virtual void updateState(const s_array& state, double time)
  {
    c_array u{};
    s_array nominal{};
    bool publish = false;
    {
      std::lock_guard<std::mutex> guard(access_guard_);
      state_ = state;
      state_time_ = time;
      has_received_state_ = true;
      if (num_iter_ == 0) return;
      const double t0 = last_used_state_update_time_;
      const double dt = controller_->getDt();
      const double since = time - t0;
      if (since > 0.0 && time >= t0 && time < t0 + dt * controller_->getNumTimesteps())
      {
        nominal = controller_->interpolateState(state_traj_, since);
        u = controller_->getCurrentControl(state, since, nominal, control_traj_, feedback_state_);
        publish = true;
      }
    }
    if (publish)
    {
      pubControl(u);
      if (debug_mode_) pubNominalState(nominal);
    }
  }

  // ---- parameters from any thread (base_plant.hpp:361-410), applied by updateParameters
  virtual void setDynamicsParams(const DYN_PARAMS_T& params)
  {
    std::lock_guard<std::mutex> guard(params_guard_);
    dynamics_params_ = params;
    has_new_dynamics_params_ = true;
  }
  virtual void setCostParams(const COST_PARAMS_T& params)
  {
    std::lock_guard<std::mutex> guard(params_guard_);
    cost_params_ = params;
    has_new_cost_params_ = true;
  }
  virtual void setControllerParams(const CONTROLLER_PARAMS_T& params)
  {
    std::lock_guard<std::mutex> guard(params_guard_);
    controller_params_ = params;
    has_new_controller_params_ = true;
  }
  virtual void setSamplerParams(const SAMPLER_T& sampler)
  {
    std::lock_guard<std::mutex> guard(params_guard_);
    sampler_ = sampler;
    has_new_sampler_params_ = true;
  }
  bool hasNewDynamicsParams() const { return has_new_dynamics_params_; }
  bool hasNewCostParams() const { return has_new_cost_params_; }
  bool hasNewControllerParams() const { return has_new_controller_params_; }
  bool hasNewSamplerParams() const { return has_new_sampler_params_; }

  // BasePlant::updateParameters (base_plant.hpp:412-451)
  virtual bool updateParameters()
  {
    std::lock_guard<std::mutex> guard(params_guard_);
    bool changed = false;
    if (has_new_cost_params_.exchange(false))
    {
      controller_->setCostParams(cost_params_);
      changed = true;
    }
    if (has_new_dynamics_params_.exchange(false))
    {
      controller_->setDynamicsParams(dynamics_params_);
      changed = true;
    }
    if (has_new_controller_params_.exchange(false))
    {
      controller_->setParams(controller_params_);
      changed = true;
    }
    if (has_new_sampler_params_.exchange(false))
    {
      controller_->setSamplingParams(sampler_);
      changed = true;
    }
    return changed;
  }

  // BasePlant::runControlIteration (base_plant.hpp:466-595): wait (bounded) for a state newer than the last one
  // optimised from, apply pending parameters, slide the nominal sequence by the robot time that passed (at least
  // the target stride, rounded as std::round) and optimise.  Returns false when nothing was optimised.
  bool runControlIteration(std::atomic<bool>* is_alive, double max_wait_s = 1.0)
  {
    using clock = std::chrono::steady_clock;
    const auto loop_start = clock::now();
    if (!is_alive->load()) return false;
    const auto wait_start = clock::now();
    while (is_alive->load())
    {
      const bool first = num_iter_ == 0 && has_received_state_;
      if (first || (has_received_state_ && getStateTime() != last_used_state_update_time_)) break;
      if (std::chrono::duration<double>(clock::now() - wait_start).count() >= max_wait_s) return false;
      std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
    if (!is_alive->load()) return false;
    updateParameters();
    s_array state;
    double state_time;
    {
      std::lock_guard<std::mutex> guard(access_guard_);
      state = state_;
      state_time = state_time_;
    }
    for (float v : state)
      if (!std::isfinite(v)) return false;
    status_ = checkStatus();
    if (num_iter_ == 0)
    {
      last_optimization_stride_ = 0;
    }
    else
    {
      const double dt = state_time - last_used_state_update_time_;
      last_optimization_stride_ = std::max((int)std::round(dt / controller_->getDt()), optimization_stride_);
    }
    if (last_optimization_stride_ > 0 && last_optimization_stride_ < controller_->getNumTimesteps())
    {
      // the robust controller's importance sampler first (a no-op for the others), then the slide
      controller_->updateImportanceSamplingControl(state, last_optimization_stride_);
      controller_->slideControlSequence(last_optimization_stride_);
    }
    const auto opt_start = clock::now();
    controller_->computeControl(state, last_optimization_stride_);
    const FreeEnergyStatistics fe = controller_->getFreeEnergyStatistics();
    const c_traj u = controller_->getControlSeq();
    for (int i = 0; i < C * controller_->getNumTimesteps(); ++i)
      if (!std::isfinite(u[i])) throw std::runtime_error("control trajectory inside the plant has a NaN");
    const s_traj s = controller_->getTargetStateSeq();
    for (int i = 0; i < S * controller_->getNumTimesteps(); ++i)
      if (!std::isfinite(s[i])) throw std::runtime_error("state trajectory inside the plant has a NaN");
    optimization_duration_ = std::chrono::duration<double, std::milli>(clock::now() - opt_start).count();
    const auto fb_start = clock::now();
    FB_STATE_T fb_state{};
    if (controller_->getFeedbackEnabled())
    {
      controller_->computeFeedback(state);
      fb_state = controller_->getFeedbackState();
    }
    feedback_duration_ = std::chrono::duration<double, std::milli>(clock::now() - fb_start).count();
    setSolution(s, u, fb_state, state_time);
    pubFreeEnergyStatistics(fe);
    controller_->computeFeedbackPropagatedStateSeq();
    const double n = num_iter_;
    avg_optimize_time_ms_ += (optimization_duration_ - avg_optimize_time_ms_) / n;
    avg_feedback_time_ms_ += (feedback_duration_ - avg_feedback_time_ms_) / n;
    optimize_loop_duration_ = std::chrono::duration<double, std::milli>(clock::now() - loop_start).count();
    avg_loop_time_ms_ += (optimize_loop_duration_ - avg_loop_time_ms_) / n;
    return true;
  }

  // BasePlant::runControlLoop (base_plant.hpp:597-620): optimise until is_alive is cleared, then wait until the
  // robot time has moved on by stride / hz (applying parameters meanwhile).
  void runControlLoop(std::atomic<bool>* is_alive)
  {
    while (is_alive->load())
    {
      runControlIteration(is_alive);
      const double wait_until = last_used_state_update_time_ + (1.0 / hz_) * optimization_stride_;
      const auto sleep_start = std::chrono::steady_clock::now();
      while (is_alive->load() && wait_until > getStateTime())
      {
        updateParameters();
        std::this_thread::sleep_for(std::chrono::microseconds(50));
      }
      sleep_duration_ =
          std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - sleep_start).count();
      if (num_iter_ > 0) avg_sleep_time_ms_ += (sleep_duration_ - avg_sleep_time_ms_) / num_iter_;
    }
  }

protected:
  std::mutex access_guard_, params_guard_;
  int hz_ = 10;
  int optimization_stride_ = 1;
  int last_optimization_stride_ = 0;
  bool debug_mode_ = false;
  s_array state_{};
  s_traj state_traj_{};
  c_traj control_traj_{};
  FB_STATE_T feedback_state_{};
  std::atomic<double> state_time_{ 0.0 };
  std::atomic<double> last_used_state_update_time_{ 0.0 };
  std::atomic<bool> has_received_state_{ false };
  std::atomic<bool> has_new_dynamics_params_{ false }, has_new_cost_params_{ false },
      has_new_controller_params_{ false }, has_new_sampler_params_{ false };
  DYN_PARAMS_T dynamics_params_{};
  COST_PARAMS_T cost_params_{};
  CONTROLLER_PARAMS_T controller_params_{};
  SAMPLER_T sampler_{};
  std::atomic<int> num_iter_{ 0 };
  int status_ = 1;
  double optimization_duration_ = 0.0, optimize_loop_duration_ = 0.0, sleep_duration_ = 0.0, feedback_duration_ = 0.0;
  double avg_optimize_time_ms_ = 0.0, avg_loop_time_ms_ = 0.0, avg_sleep_time_ms_ = 0.0, avg_feedback_time_ms_ = 0.0;
};
}  // namespace mppi_gb

#endif  // MPPI_GB_PLANT_HPP
