/*
 * mppi_gb_plugin.cuh — bring your own Dynamics and Cost plugins to the GB300 MPPI engine.
 *
 * MPPI-Generic's plugin surface is CRTP: a dynamics class derives from Dynamics<CLASS_T, PARAMS_T> and defines
 * device computeDynamics (include/mppi/dynamics/dynamics.cuh:369), optionally computeKinematics, computeStateDeriv,
 * step, updateState and stateToOutput (:377-402); a cost derives from Cost<CLASS_T, PARAMS_T, DYN_PARAMS_T> and
 * defines device computeStateCost(y, t, theta_c, crash) and terminalCost(y, theta_c), optionally computeControlCost
 * and computeRunningCost(y, u, t, theta_c, crash) (include/mppi/cost_functions/cost.cuh:146-222).  The controller
 * then instantiates its kernels over those classes.
 *
 * Here the same: derive a plain struct from mppi_gb::Dynamics<YourDyn, S, C[, O]> and another from
 * mppi_gb::Cost<YourCost, O, C>, give them the same method names, and put MPPI_GB_PLUGIN(name, YourDyn, YourCost)
 * in one .cu file.  Compiling that file (nvcc -gencode arch=compute_103a,code=sm_103a --fmad=false -shared -Xcompiler
 * -fPIC, -I<this directory>, linked against libmppi_gb.so) instantiates the engine over the two classes and exports
 * three C functions:
 *
 *   mppi_status name_create(int num_instances, const int* num_rollouts, const int* num_timesteps,
 *                           const mppi_controller_params*, const mppi_sampling_params*,
 *                           const mppi_control_constraints*, const void* dyn_params, size_t dyn_bytes,
 *                           const void* cost_params, size_t cost_bytes, const float* init_control, void* stream,
 *                           mppi_handle** out);      (mppi_create's arguments without the model id)
 *   mppi_status name_model_dims(int* state_dim, int* control_dim, int* output_dim);
 *   mppi_status name_param_sizes(size_t* dyn_bytes, size_t* cost_bytes);
 *
 * The handle is an ordinary mppi_handle: every mppi_* entry point of mppi_gb.h applies to it.  dyn_params and
 * cost_params are arrays of the plugin structs themselves (one per instance, or one for all), copied to the GPU by
 * value as the reference copies its plugin objects (Managed::GPUSetup, include/mppi/utils/managed.cuh:120-131), so
 * the structs must be trivially copyable and hold their parameters as members.
 *
 * Differences from the reference's surface, all from running one sample per GPU thread:
 *  - no theta_s / theta_c shared-memory scratch arguments (a sample's state lives in registers);
 *  - methods are const and __host__ __device__ (the host twin computes the nominal state trajectory);
 *  - enforceConstraints: by default the engine's, the reference's default (deadband, then clamp to the control ranges
 *    of the handle's mppi_control_constraints), applied when the samples are written.  A dynamics class that defines
 *        void enforceConstraints(float* state, float* control) const
 *    replaces it, with the reference's placement: the samples are written unconstrained, each rollout step passes
 *    its control through the method with the current state and writes the result back as the sample
 *    (rolloutKernel, mppi_common.cu:114-123), the sampled-trajectory re-roll does the same (:453), the nominal state
 *    trajectory applies it with the state to the smoothed sequence (controller.cuh:676-680), and the final pass after
 *    smoothing applies it with a zero state to every control (mppi_controller.cu:222-226);
 *  - crash is one int per sample, zero at the start of every rollout, passed to each running cost call, and reported
 *    per step by mppi_get_sampled_trajectories (the reference's crash_status_d, mppi_common.cu:371-376);
 *  - computeGrad (Dynamics::computeGrad, dynamics.cuh:236-242) is optional and host-only: a dynamics class that
 *    defines
 *        bool computeGrad(const float* state, const float* control, float* A, float* B) const
 *    with A = d xdot / d state (row-major STATE_DIM x STATE_DIM) and B = d xdot / d control (row-major STATE_DIM x
 *    CONTROL_DIM), both zero on entry, gives the DDP feedback controller (mppi_compute_feedback) its Jacobians;
 *    without it, or when it returns false, the controller takes forward differences of the step's derivative, as
 *    the reference's ModelWrapperDDP does (ddp_model_wrapper.h:81-94).
 * The plugin rollout is a sampler kernel followed by one rollout kernel (one thread per sample, the tile's controls
 * staged in shared memory, the tile's weighted partial sums at the end), then the per-instance combine.
 */
#ifndef MPPI_GB_PLUGIN_CUH
#define MPPI_GB_PLUGIN_CUH

#include <type_traits>

#include "mppi_gb.h"

#define MPPI_GB_HD __host__ __device__ __forceinline__

namespace mppi_gb
{
/* Dynamics<CLASS_T, S, C, O> (Dynamics<CLASS_T, PARAMS_T>, dynamics.cuh:68-77).  CLASS_T defines
 *   computeDynamics(const float* state, const float* control, float* state_der) const
 * and may redefine any of the methods below (a member of the same name in CLASS_T hides the default). */
template <class CLASS_T, int S, int C, int O = S>
struct Dynamics
{
  static constexpr int STATE_DIM = S, CONTROL_DIM = C, OUTPUT_DIM = O;

  /* kinematic part of the derivative (dynamics.cuh:377), nothing by default */
  MPPI_GB_HD void computeKinematics(const float* state, float* state_der) const {}

  /* computeKinematics, then computeDynamics (dynamics.cu:93-105) */
  MPPI_GB_HD void computeStateDeriv(const float* state, const float* control, float* state_der) const
  {
    self().computeKinematics(state, state_der);
    self().computeDynamics(state, control, state_der);
  }

  /* next = state + state_der * dt, one fused multiply-add per element (dynamics.cu:128-140) */
  MPPI_GB_HD void updateState(const float* state, float* next_state, const float* state_der, float dt) const
  {
#pragma unroll
    for (int i = 0; i < S; ++i) next_state[i] = fmaf(state_der[i], dt, state[i]);
  }

  /* output = the first O states (dynamics.cu:154-165) */
  MPPI_GB_HD void stateToOutput(const float* state, float* output) const
  {
#pragma unroll
    for (int i = 0; i < O && i < S; ++i) output[i] = state[i];
  }

  /* one step: derivative, update, output (dynamics.cu:142-152) */
  MPPI_GB_HD void step(const float* state, float* next_state, float* state_der, const float* control, float* output,
                       int t, float dt) const
  {
    self().computeStateDeriv(state, control, state_der);
    self().updateState(state, next_state, state_der, dt);
    self().stateToOutput(next_state, output);
  }

private:
  MPPI_GB_HD const CLASS_T& self() const { return static_cast<const CLASS_T&>(*this); }
};

/* Cost<CLASS_T, O, C> (Cost<CLASS_T, PARAMS_T, DYN_PARAMS_T>, cost.cuh:34-35).  CLASS_T defines
 *   float computeStateCost(const float* output, int t, int* crash) const
 *   float terminalCost(const float* output) const
 * and may redefine computeControlCost and computeRunningCost. */
template <class CLASS_T, int O, int C>
struct Cost
{
  static constexpr int OUTPUT_DIM = O, CONTROL_DIM = C;

  /* cost.cuh:205-210: zero by default */
  MPPI_GB_HD float computeControlCost(const float* control, int t, int* crash) const { return 0.0f; }

  /* state cost + control cost (cost.cuh:212-222) */
  MPPI_GB_HD float computeRunningCost(const float* output, const float* control, int t, int* crash) const
  {
    return self().computeStateCost(output, t, crash) + self().computeControlCost(control, t, crash);
  }

private:
  MPPI_GB_HD const CLASS_T& self() const { return static_cast<const CLASS_T&>(*this); }
};
}  // namespace mppi_gb

#include "../mppi_generic_vendor_gb300/csrc/mg_plugin_create.cuh"

/* Instantiates the engine over (DYN_T, COST_T) and exports NAME_create, NAME_model_dims and NAME_param_sizes. */
#define MPPI_GB_PLUGIN(NAME, DYN_T, COST_T)                                                                          \
  extern "C" mppi_status NAME##_create(int num_instances, const int* num_rollouts, const int* num_timesteps,         \
                                       const mppi_controller_params* params, const mppi_sampling_params* sampling,   \
                                       const mppi_control_constraints* constraints, const void* dyn_params,          \
                                       size_t dyn_bytes, const void* cost_params, size_t cost_bytes,                \
                                       const float* init_control, void* stream, mppi_handle** out)                   \
  {                                                                                                                  \
    return ::mg::plugin_create<DYN_T, COST_T>(num_instances, num_rollouts, num_timesteps, params, sampling,         \
                                              constraints, dyn_params, dyn_bytes, cost_params, cost_bytes,         \
                                              init_control, stream, out);                                          \
  }                                                                                                                  \
  extern "C" mppi_status NAME##_model_dims(int* state_dim, int* control_dim, int* output_dim)                        \
  {                                                                                                                  \
    if (state_dim) *state_dim = DYN_T::STATE_DIM;                                                                    \
    if (control_dim) *control_dim = DYN_T::CONTROL_DIM;                                                              \
    if (output_dim) *output_dim = DYN_T::OUTPUT_DIM;                                                                 \
    return MPPI_OK;                                                                                                  \
  }                                                                                                                  \
  extern "C" mppi_status NAME##_param_sizes(size_t* dyn_bytes, size_t* cost_bytes)                                   \
  {                                                                                                                  \
    if (dyn_bytes) *dyn_bytes = sizeof(DYN_T);                                                                       \
    if (cost_bytes) *cost_bytes = sizeof(COST_T);                                                                    \
    return MPPI_OK;                                                                                                  \
  }

#endif /* MPPI_GB_PLUGIN_CUH */
