/*
 * mppi_gb.h — C ABI of the GB300-native MPPI engine (libmppi_gb.so).
 *
 * The engine stands in for MPPI-Generic's plain MPPI path: a VanillaMPPIController built from a Dynamics plugin,
 * a Cost plugin and a Gaussian or colored-noise SamplingDistribution.  Every entry point below names the reference
 * interface it replaces (paths relative to the MPPI-Generic source tree).
 *
 * Conventions
 *  - Every function returns an mppi_status; none calls exit() or throws across the ABI (the reference exits the
 *    process from HANDLE_ERROR, include/mppi/utils/gpu_err_chk.cuh:32-40).  mppi_last_error_string() explains the
 *    most recent failure on the calling thread.
 *  - Plain pointers and sizes only.  "host" pointers are ordinary CPU memory; "device" pointers are CUDA global
 *    memory on the current device.  Streams are passed as void* (a cudaStream_t).
 *  - Control sequences are float[T][C] (time-major, control innermost), which is the memory order of the reference's
 *    column-major Eigen control_trajectory (C x MAX_T).  Control samples are float[K][T][C] per instance, the
 *    reference's control_samples_d_ layout (sampling_distribution.cu:108-116).
 *  - A handle owns all of its device memory and is not thread-safe: use one handle per thread.
 *  - A handle holds num_instances independent controllers (each with its own K, T, plugin parameters, nominal
 *    control and state).  num_instances == 1 is the reference's single VanillaMPPIController.  Arrays that take
 *    "all instances" are the concatenation over instances in index order.
 */
#ifndef MPPI_GB_H
#define MPPI_GB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MPPI_GB_ABI_VERSION 3
#define MPPI_MAX_STATE_DIM 8
#define MPPI_MAX_CONTROL_DIM 4
#define MPPI_MAX_OBSTACLES 8

typedef enum mppi_status
{
  MPPI_OK = 0,
  MPPI_EINVAL = 1,      /* bad argument, size or parameter (reference: precondition exit(), mppi_common.cu:1302-1313) */
  MPPI_ECUDA = 2,       /* a CUDA runtime call failed (reference: HANDLE_ERROR exit) */
  MPPI_ENAN = 3,        /* non-finite input state, noise or baseline cost */
  MPPI_ETIMEOUT = 4,    /* a bounded device-side wait gave up */
  MPPI_ENOMEM = 5,      /* device or host allocation failed */
  MPPI_EUNSUPPORTED = 6 /* model / sampler combination not built */
} mppi_status;

/* Concrete plugin pairs (Dynamics + Cost) compiled into the library. */
typedef enum mppi_model
{
  MPPI_MODEL_CARTPOLE = 1,            /* CartpoleDynamics (cartpole_dynamics.cu:87-105) + swing-up cost */
  MPPI_MODEL_DOUBLE_INTEGRATOR = 2,   /* DoubleIntegratorDynamics (di_dynamics.cu:46-53) + goal/obstacle cost */
  MPPI_MODEL_BICYCLE_COSTMAP = 3,     /* kinematic bicycle + bilinear costmap + speed cost (no reference model) */
  MPPI_MODEL_BICYCLE_SLIP = 4,        /* 7-state dynamic bicycle with linear tyres (no reference model) */
  MPPI_MODEL_BICYCLE_SLIP_MLP = 5,    /* same cost, dynamics from the learned MLP surrogate */
  MPPI_MODEL_PLUGIN = 100             /* a caller's Dynamics / Cost plugin pair, instantiated by MPPI_GB_PLUGIN
                                         (mppi_gb_plugin.cuh); created by the plugin library's NAME_create */
} mppi_model;

typedef enum mppi_sampler_kind
{
  MPPI_SAMPLER_GAUSSIAN = 0,      /* GaussianDistributionImpl (gaussian.cuh:98) */
  MPPI_SAMPLER_COLORED_NOISE = 1  /* ColoredNoiseDistributionImpl (colored_noise.cuh:79) */
} mppi_sampler_kind;

/* Controller kinds: which controller's computeControl the handle runs. */
typedef enum mppi_controller_kind
{
  MPPI_CONTROLLER_VANILLA = 0, /* VanillaMPPIController (mppi_controller.cu:152-237) */
  MPPI_CONTROLLER_COLORED = 1, /* ColoredMPPIController (colored_mppi_controller.cu:145-249): Tsallis weights when
                                  tsallis_gamma != 0 and tsallis_r != 0, state leash, final clamp of control 1 only */
  MPPI_CONTROLLER_TUBE = 2,    /* TubeMPPIController (tube_mppi_controller.cu:158-296): the handle holds exactly two
                                  instances of equal K and T, the reference's two sampling distributions
                                  [D = 2][K][T][C]: instance 0 is the actual system, rolled out from the state
                                  given to mppi_compute_control (STATE_DIM floats), instance 1 the nominal system,
                                  rolled out from the handle's nominal state (the first state given, then advanced
                                  one step along the nominal sequence by every slide).  After each iteration the
                                  nominal pair takes over the actual pair's state and control sequences when the
                                  actual baseline is below the nominal baseline + nominal_threshold.  Only the
                                  nominal sequence is smoothed; neither is clamped.  The ancillary feedback
                                  controller (mppi_compute_feedback) tracks the nominal system. */
  MPPI_CONTROLLER_RMPPI = 3    /* RobustMPPIController (robust_mppi_controller.cu:635-744): two instances of equal K
                                  and T, the reference's distributions [D = 2][K][T][C] in its order: instance 0 the
                                  nominal system, rolled out from the nominal state, instance 1 the real system,
                                  rolled out from the state given to mppi_compute_control (STATE_DIM floats) with
                                  the DDP feedback K_t (x_real - x_nominal) added to its controls.  Both sample
                                  around the nominal sequence (the importance sampler); the nominal costs blend in
                                  the real system's (rolloutRMPPIKernel, rmppi_kernels.cu:666-861).  Call
                                  mppi_rmppi_update_importance_sampler before each mppi_compute_control.  Analytic
                                  models (built-in and plugin pairs) with Gaussian sampling. */
} mppi_controller_kind;

/* ControllerParams (include/mppi/controllers/controller.cuh:46-68) and the fields ColoredMPPIParams adds
 * (colored_mppi_controller.cuh:17-22).  Block dimensions are chosen by the engine. */
typedef struct mppi_controller_params
{
  float dt;
  float lambda;
  float alpha;
  int num_timesteps; /* T; per-instance values for batches are passed separately */
  int num_iters;     /* optimisation iterations per computeControl */
  uint64_t seed;     /* Philox key */
  float slide_control_scale[MPPI_MAX_CONTROL_DIM];
  int controller;    /* mppi_controller_kind (default MPPI_CONTROLLER_VANILLA) */
  float tsallis_r;   /* ColoredMPPIParams::r (default 2.0) */
  float tsallis_gamma; /* ColoredMPPIParams::gamma (default 0 = exponential weights) */
  int leash_active;  /* ColoredMPPIController::leash_active_ (default 0); the leash holds x0 near the nominal state
                        at the step the last slideControlSequence moved by (leash_jump_, 1 before any slide) */
  float state_leash_dist[MPPI_MAX_STATE_DIM]; /* ColoredMPPIParams::state_leash_dist_ (default 0) */
  float nominal_threshold; /* TubeMPPIParams::nominal_threshold_ (tube_mppi_controller.cuh:20, default 20) */
  float value_function_threshold;    /* RobustMPPIParams::value_function_threshold_ (robust_mppi_controller.cuh:17,
                                        default 1000) */
  int num_candidate_nominal_states;  /* RobustMPPIParams::num_candidate_nominal_states_ (default 9; odd, >= 3) */
  int num_eval_samples_per_candidate; /* samples per candidate of the initial-state evaluation (the eval kernel's
                                         block width in the reference; default 64); candidates x samples <= K */
} mppi_controller_params;

/* GaussianParamsImpl (gaussian.cuh:21-61) and ColoredNoiseParamsImpl (colored_noise.cuh:44-73). */
typedef struct mppi_sampling_params
{
  int kind; /* mppi_sampler_kind */
  float std_dev[MPPI_MAX_CONTROL_DIM];
  float control_cost_coeff[MPPI_MAX_CONTROL_DIM];
  float pure_noise_trajectories_percentage; /* default 0.01 */
  float std_dev_decay;                      /* default 1.0 */
  float exponents[MPPI_MAX_CONTROL_DIM];    /* colored noise: PSD ~ 1/f^exponent */
  float offset_decay_rate;                  /* colored noise, default 0.97 */
  float fmin;                               /* colored noise low-frequency cutoff, default 0 */
  int use_same_noise_for_all_distributions; /* SamplingParams (sampling_distribution.cuh:20), default 1: the two
                                               distributions of a Tube-MPPI or R-MPPI handle draw the same standard
                                               normals
                                               (gaussian.cu:378-390), each around its own mean; independent
                                               controllers of a batched handle always draw their own */
} mppi_sampling_params;

/* Dynamics::control_rngs_, control_deadband_, zero_control_ (dynamics.cuh:508; dynamics.cu:107-126). */
typedef struct mppi_control_constraints
{
  float lower[MPPI_MAX_CONTROL_DIM];
  float upper[MPPI_MAX_CONTROL_DIM];
  float deadband[MPPI_MAX_CONTROL_DIM];
  float zero_control[MPPI_MAX_CONTROL_DIM];
} mppi_control_constraints;

/* ---- plugin parameter blocks ------------------------------------------------------------------------------------ */

/* CartpoleDynamicsParams (cartpole_dynamics.cuh); gravity is the reference's gravity_ = 9.81 constant. */
typedef struct mppi_cartpole_params
{
  float cart_mass;
  float pole_mass;
  float pole_length;
  float gravity;
} mppi_cartpole_params;

/* Swing-up cost: x_coeff*x^2 + x_dot_coeff*xdot^2 + cos_coeff*(1+cos theta)^2 + theta_dot_coeff*thetadot^2,
 * terminal cost = terminal_coeff * (same expression).  Same API as CartpoleQuadraticCost
 * (cartpole_quadratic_cost.cu:20-43). */
typedef struct mppi_cartpole_cost_params
{
  float x_coeff;
  float x_dot_coeff;
  float cos_coeff;
  float theta_dot_coeff;
  float terminal_coeff;
} mppi_cartpole_cost_params;

/* DoubleIntegratorDynamics has no parameters on the MPPI path (di_dynamics.cu:46-53). */
typedef struct mppi_double_integrator_params
{
  float reserved;
} mppi_double_integrator_params;

/* Quadratic-to-goal cost (QuadraticCostImpl, quadratic_cost.cu:35-48) plus obstacle_cost when the position lies
 * strictly inside any circle (composed like DoubleIntegratorCircleCost, double_integrator_circle_cost.cu:8-32). */
typedef struct mppi_di_obstacle_cost_params
{
  float goal[4];
  float coeff[4];
  float terminal_coeff;
  int num_obstacles;
  float obstacle_x[MPPI_MAX_OBSTACLES];
  float obstacle_y[MPPI_MAX_OBSTACLES];
  float obstacle_radius[MPPI_MAX_OBSTACLES];
  float obstacle_cost;
} mppi_di_obstacle_cost_params;

/* Kinematic bicycle: state (x, y, yaw, v), control (accel, steer).  Closest reference: DubinsDynamics
 * (dubins.cu:60-65). */
typedef struct mppi_bicycle_params
{
  float wheelbase;
} mppi_bicycle_params;

/* Costmap cost: map_coeff * bilinear(map, x, y) + speed_coeff * (v - speed_target)^2.  The map itself is uploaded with
 * mppi_set_costmap().  Replaces the TwoDTextureHelper query (two_d_texture_helper.cu:66-72, CPU twin :151). */
typedef struct mppi_costmap_cost_params
{
  float map_coeff;
  float speed_target;
  float speed_coeff;
  float steer_coeff;
  float terminal_coeff;
} mppi_costmap_cost_params;

/* Dynamic bicycle with linear tyres: state (x, y, yaw, vx, vy, yaw_rate, steer), control (throttle, steer_cmd). */
typedef struct mppi_bicycle_slip_params
{
  float mass;
  float yaw_inertia;
  float lf;
  float lr;
  float cornering_stiffness;
  float max_drive_force;
  float drag;
  float max_steer;
  float steer_time_constant;
  float min_vx;
} mppi_bicycle_slip_params;

/* ---- controller handle (Controller / VanillaMPPIController, controller.cuh:70-1058, mppi_controller.cuh:14-78) --- */

typedef struct mppi_handle mppi_handle;

/* Version and build information. */
int mppi_abi_version(void);
/* Dims of a model: writes STATE_DIM, CONTROL_DIM, OUTPUT_DIM (Dynamics::STATE_DIM etc., dynamics.cuh:75-77). */
mppi_status mppi_model_dims(int model, int* state_dim, int* control_dim, int* output_dim);
/* Size in bytes of the dynamics / cost parameter blocks a model expects. */
mppi_status mppi_model_param_sizes(int model, size_t* dyn_bytes, size_t* cost_bytes);
/* Reference defaults: ControllerParams, GaussianParamsImpl/ColoredNoiseParamsImpl, and unbounded constraints. */
void mppi_default_controller_params(mppi_controller_params* p);
void mppi_default_sampling_params(mppi_sampling_params* p);
void mppi_default_constraints(mppi_control_constraints* c);

/* Message describing the last failure on this thread ("" if none). */
const char* mppi_last_error_string(void);

/*
 * Create a controller holding num_instances independent MPPI problems.
 * Replaces the VanillaMPPIController constructor (mppi_controller.cu:16-29 -> Controller::Controller,
 * controller.cuh:111-153).  num_rollouts[i] / num_timesteps[i] give K_i and T_i; dyn_params and cost_params point to
 * num_instances consecutive parameter blocks of dyn_bytes / cost_bytes each (sizes from mppi_model_param_sizes).
 * init_control (may be NULL = zeros) holds the concatenated initial control sequences.  stream may be NULL, in which
 * case the handle creates its own non-blocking stream.
 */
mppi_status mppi_create(int model, int num_instances, const int* num_rollouts, const int* num_timesteps,
                        const mppi_controller_params* params, const mppi_sampling_params* sampling,
                        const mppi_control_constraints* constraints, const void* dyn_params, size_t dyn_bytes,
                        const void* cost_params, size_t cost_bytes, const float* init_control, void* stream,
                        mppi_handle** out);
/* Frees every device and host resource (Controller::~Controller -> freeCudaMem, controller.cuh:196-218). */
mppi_status mppi_destroy(mppi_handle* h);

/* Number of instances, and K / T of instance i. */
mppi_status mppi_get_instance_dims(const mppi_handle* h, int instance, int* num_rollouts, int* num_timesteps);
/* The handle's model id (MPPI_MODEL_PLUGIN for plugin handles), STATE_DIM, CONTROL_DIM and OUTPUT_DIM (any may be
 * NULL).  Dynamics::STATE_DIM / CONTROL_DIM / OUTPUT_DIM (dynamics.cuh:75-77) of the handle's plugin. */
mppi_status mppi_get_model_dims(const mppi_handle* h, int* model, int* state_dim, int* control_dim, int* output_dim);
/* Wrap an engine that a plugin library built (MPPI_GB_PLUGIN's NAME_create calls this) in a handle of this library.
 * abi_version must equal MPPI_GB_ABI_VERSION; on success the handle owns the engine (mppi_destroy frees it).  No
 * counterpart in the reference, whose plugin templates are instantiated inside the caller's own program. */
mppi_status mppi_handle_adopt(void* engine, int abi_version, mppi_handle** out);

/*
 * One MPC solve for every instance: num_iters x (sample -> rollout -> weights -> update), then the host-side
 * Savitzky-Golay smoothing, nominal state rollout and control clamp.  x0 is host float[num_instances][STATE_DIM].
 * Replaces VanillaMPPIController::computeControl(state, optimization_stride) (mppi_controller.cu:152-237).
 */
mppi_status mppi_compute_control(mppi_handle* h, const float* x0, int optimization_stride);

/* Nominal control sequences, host float[sum_i T_i * C].  Controller::getControlSeq (controller.cuh:425-428). */
mppi_status mppi_get_control_seq(mppi_handle* h, float* out);
/* Overwrite the nominal control sequences (ControllerParams::init_control_traj_ / setParams, controller.cuh:857-876). */
mppi_status mppi_set_control_seq(mppi_handle* h, const float* in);
/* Shift every instance's sequence by steps (Controller::slideControlSequence, controller.cuh:370-376, 609-636). */
mppi_status mppi_slide_control_sequence(mppi_handle* h, int steps);
/* Nominal state trajectories, host float[sum_i T_i * STATE_DIM] (Controller::getTargetStateSeq, controller.cuh:433). */
mppi_status mppi_get_state_seq(mppi_handle* h, float* out);
/* Baseline (min cost) and normaliser (sum of exp weights) of the last iteration, host float[2 * num_instances]
 * as (baseline, normaliser) pairs (Controller::getBaselineCost / getNormalizerCost, controller.cuh:526-533).
 * The normaliser is accumulated in double on the device; normalizer_fp64 (may be NULL) receives it unrounded. */
mppi_status mppi_get_baseline_normalizer(mppi_handle* h, float* out, double* normalizer_fp64);
/* Per-sample trajectory costs before the weight transform, host float[sum_i K_i]. */
mppi_status mppi_get_sample_costs(mppi_handle* h, float* out);
/* Per-sample unnormalised weights exp(-(c - baseline)/lambda), host float[sum_i K_i].  This is what the reference's
 * Controller::getSampledCostSeq returns after an iteration (controller.cuh:449-452; the array is transformed in
 * place by fullGPUcomputeWeights, mppi_common.cu:1067-1089). */
mppi_status mppi_get_sample_weights(mppi_handle* h, float* out);
/* Control samples of the last iteration after the constraints were applied, host float[sum_i K_i*T_i*C].
 * SamplingDistribution::getControlSample (sampling_distribution.cuh:234-236). */
mppi_status mppi_get_control_samples(mppi_handle* h, float* out);
/* Sampled-trajectory read-out for visualisation (VanillaMPPIController::calculateSampledStateTrajectories ->
 * visualizeKernel, mppi_common.cu:371-533; getSampledOutputTrajectories / getSampledCostTrajectories,
 * controller.cuh:281-289): samples idx[0..n-1] of `instance` from the last mppi_compute_control are re-rolled on the
 * GPU from their stored, constrained controls.  states[n][T][S] holds the state after each step, step_costs[n][T] the
 * running cost of each step and terminal[n] the terminal cost; the sample's cost is (the step costs summed in step
 * order) / T + terminal / T, bit for bit.  The likelihood-ratio term uses the nominal sequence the solve started
 * from.  crash_status (may be NULL) receives int[n][T], the sample's crash flag after each step's running cost
 * (crash_status_d of visualizeKernel, mppi_common.cu:371-376; always 0 for the built-in costs).  For a plugin handle
 * states holds the outputs (stateToOutput) after each step, [n][T][OUTPUT_DIM].  Analytic models and plugins only
 * (MPPI_EUNSUPPORTED for the surrogate). */
mppi_status mppi_get_sampled_trajectories(mppi_handle* h, int instance, const int* idx, int n, float* states,
                                          float* step_costs, float* terminal, int* crash_status);
/* Controller::copyTopControlFromDevice's selection (controller.cu:126-181), on the host: the n highest of
 * weights[0..num_samples-1] (the transformed costs, mppi_get_sample_weights), by the reference's replacement scan,
 * in the order of its list slots.  No handle or GPU involved. */
mppi_status mppi_select_top_samples(const float* weights, int num_samples, int n, int* indices);
/* RobustMPPIController::updateImportanceSamplingControl (robust_mppi_controller.cu:548-569), before each
 * mppi_compute_control of an R-MPPI handle: the first call takes `state` (the real system's) as the nominal state;
 * later calls place num_candidate_nominal_states candidates on the lines from the nominal trajectory's first state
 * to its second and on to `state` (getInitNominalStateCandidates / computeLineSearchWeights, :351-363, 480-511),
 * roll out num_eval_samples_per_candidate samples from each (initEvalKernel, rmppi_kernels.cu:231-357), and take the
 * last candidate whose free energy is below value_function_threshold (computeBestIndex, :527-546) as the nominal
 * state, with its stride; then the nominal sequence slides by that stride, its state trajectory is recomputed and the
 * DDP feedback gains are computed from `state` (computeNominalFeedbackGains). */
mppi_status mppi_rmppi_update_importance_sampler(mppi_handle* h, const float* state, int optimization_stride);
/* The last candidate evaluation of an R-MPPI handle: best_index and nominal_stride (either may be NULL), and when not
 * NULL candidate_states[num_candidates][STATE_DIM], candidate_strides[num_candidates], candidate_free_energy
 * [num_candidates] and eval_costs[num_candidates * num_eval_samples_per_candidate]. */
mppi_status mppi_rmppi_get_candidates(mppi_handle* h, int* best_index, int* nominal_stride, float* candidate_states,
                                      int* candidate_strides, float* candidate_free_energy, float* eval_costs);

/* Tube-MPPI handles: 1 if the last iteration kept the nominal system (its baseline was not beaten by the actual
 * system's, FreeEnergyStatistics::nominal_state_used), else 0. */
mppi_status mppi_get_nominal_state_used(mppi_handle* h, int* used);

/* ---- ancillary feedback controller: DDP around the nominal trajectory (DDPFeedback,
 *      feedback_controllers/DDP/ddp.cu:48-120; the solver ddp/ddp.h:40-195 with the tracking costs of
 *      ddp/ddp_tracking_costs.h), computed on the host after a solve.  It serves a handle with one instance, or a
 *      Tube-MPPI handle, where it tracks the nominal system (getControlSeq / getTargetStateSeq of
 *      tube_mppi_controller.cuh:61-72). ------------------------------------------------------------------------ */

/* DDPParams (feedback_controllers/DDP/ddp.cuh:16-25): tracking weights Q and Q_f (STATE_DIM x STATE_DIM) and R
 * (CONTROL_DIM x CONTROL_DIM), column-major; NULL keeps the current matrix (identity at creation); num_iterations
 * >= 1 (1 at creation). */
mppi_status mppi_set_feedback_params(mppi_handle* h, const float* Q, const float* Q_f, const float* R,
                                     int num_iterations);
/* 1: Controller::initFeedback (controller.cuh:265-269), feedback on with the gains reset to zero; 0:
 * disableFeedbackController (controller.cuh:730-733). */
mppi_status mppi_enable_feedback(mppi_handle* h, int enable);
/* Controller::getFeedbackEnabled (controller.cuh:740-743). */
mppi_status mppi_get_feedback_enabled(const mppi_handle* h, int* enabled);
/* Controller::computeFeedback(state) (controller.cuh:551-565): DDP from `state` (host float[STATE_DIM]) around the
 * nominal state trajectory and the control sequence of the last solve, for the gains of every step; nothing while
 * feedback is off.  MPPI_EINVAL when a control Hessian of the backward pass is not positive definite, where the
 * reference's solver exits the process (ddp.h:130-139). */
mppi_status mppi_compute_feedback(mppi_handle* h, const float* state);
/* The gains (DDPFeedbackState::fb_gain_traj_, ddp.cuh:28-37): host float[T][CONTROL_DIM * STATE_DIM], step t's
 * CONTROL_DIM x STATE_DIM matrix column-major (element (r, c) at t * C * S + r + c * C); the last step's is zero. */
mppi_status mppi_get_feedback_gains(const mppi_handle* h, float* out);
/* Controller::getFeedbackControl (controller.cuh:567-571) = DDPFeedback::k_ (ddp.cuh:139-146): out[CONTROL_DIM] =
 * K_t (state - goal_state), 0 <= t < T. */
mppi_status mppi_get_feedback_control(const mppi_handle* h, const float* state, const float* goal_state, int t,
                                      float* out);
/* Controller::computeFeedbackPropagatedStateSeq + getFeedbackPropagatedStateSeq (controller.cuh:495-524): host
 * float[T][STATE_DIM], from the state the last solve started at, each step under the nominal control plus the
 * feedback against that step's target state, stepped by the model without constraints.  Recomputed while feedback
 * is on; with feedback off the previous result (zeros at first) is returned. */
mppi_status mppi_get_feedback_propagated_state_seq(mppi_handle* h, float* out);
/* The same solver without a handle or a GPU, over a built-in analytic model's host dynamics (MPPI_MODEL_CARTPOLE,
 * DOUBLE_INTEGRATOR, BICYCLE_COSTMAP with analytic Jacobians; BICYCLE_SLIP with forward differences): gains_out
 * receives float[T][CONTROL_DIM * STATE_DIM] for the nominal trajectory target_states[T][STATE_DIM] /
 * nominal_controls[T][CONTROL_DIM] from x0, control range control_min / control_max, weights as above (NULL =
 * identity). */
mppi_status mppi_ddp_feedback_gains(int model, const void* dyn_params, size_t dyn_bytes, int num_timesteps, float dt,
                                    const float* x0, const float* target_states, const float* nominal_controls,
                                    const float* Q, const float* Q_f, const float* R, int num_iterations,
                                    const float* control_min, const float* control_max, float* gains_out);
/* Free-energy statistics of instance i (MPPIFreeEnergyStatistics, controller.cuh:22-38; computeFreeEnergy,
 * mppi_common.cu:1101-1117): out[0..5] = mean, variance, modified variance, normaliser percent, increase,
 * previous baseline. */
mppi_status mppi_get_free_energy(mppi_handle* h, int instance, float* out6);

/* Replace the model parameters (Dynamics::setParams / Cost::setParams): one block of the model's parameter struct
 * for every instance (bytes = sizeof the struct), or one block per instance (bytes = instances * sizeof). */
mppi_status mppi_set_dynamics_params(mppi_handle* h, const void* dyn_params, size_t dyn_bytes);
mppi_status mppi_set_cost_params(mppi_handle* h, const void* cost_params, size_t cost_bytes);
/* Replace the sampling parameters (Controller::setSamplingParams, controller.cuh:852). */
mppi_status mppi_set_sampling_params(mppi_handle* h, const mppi_sampling_params* sampling);
/* Set lambda / alpha / num_iters / dt / slide scale (Controller::setParams, controller.cuh:857-876). */
mppi_status mppi_set_controller_params(mppi_handle* h, const mppi_controller_params* params);

/* Costmap for MPPI_MODEL_BICYCLE_COSTMAP / BICYCLE_SLIP*: row-major float[height][width], cell (0,0) centred at
 * (origin_x + resolution/2, origin_y + resolution/2).  All instances share one map. */
mppi_status mppi_set_costmap(mppi_handle* h, const float* map, int width, int height, float resolution,
                             float origin_x, float origin_y);

/* Surrogate weights for MPPI_MODEL_BICYCLE_SLIP_MLP: 9->64->64->5 tanh MLP, fp32 row-major W1[64][9], b1[64],
 * W2[64][64], b2[64], W3[5][64], b3[5] (FNNHelper layout, fnn_helper.cu:353-382), plus input / output scaling.
 * precision 0 = bf16 weights on the tensor cores (BF16 operands), 1 = fp8 e4m3 weights with one power-of-two scale
 * per layer on the tensor cores (FP16 operands, in which q * scale is exact), both with FP32 accumulation; 2 = plain
 * FP32 on the CUDA cores (one thread per sample, as FNNHelper evaluates it). */
mppi_status mppi_set_mlp(mppi_handle* h, const float* params, size_t num_params, int precision);

/* Analytic judge of the surrogate rollout (MPPI_MODEL_BICYCLE_SLIP_MLP only): after the surrogate rollout the
 * ceil(fraction * K_i) lowest-cost samples of every instance are re-rolled with the analytic dynamic bicycle in FP32;
 * their costs become analytic - mean(analytic - surrogate) and the baseline is recomputed.  fraction 0 disables it;
 * the default is 0.01.  No counterpart in the reference, whose NeuralNetModel rollouts are not checked. */
mppi_status mppi_set_judge(mppi_handle* h, float fraction);
/* Per instance after the last computeControl: out[2*i] = mean(analytic - surrogate) cost over the judged samples,
 * out[2*i+1] = mean |analytic - surrogate| / |analytic|.  Zeros when the judge is off. */
mppi_status mppi_get_judge_stats(mppi_handle* h, float* out);
/* Fallback: roll out the analytic model instead of the surrogate (1) or the surrogate again (0). */
mppi_status mppi_use_analytic_dynamics(mppi_handle* h, int enable);

/*
 * Parity hook: use the given standard-normal noise for every subsequent iteration instead of Philox noise.
 * Gaussian: host float[sum_i K_i*T_i*C], the epsilon that curandGenerateNormal writes before setGaussianControls
 * (gaussian.cu:375-431).  Colored noise: host float[sum_i K_i*C*(T_i+1)*2], the complex spectrum before
 * configureFrequencyNoise (colored_noise.cu:343).  noise == NULL clears the injection.  On a Tube-MPPI or R-MPPI
 * handle with use_same_noise_for_all_distributions both distributions read instance 0's part (the second part is
 * ignored), as the reference's generateSamples copies one draw to every distribution (gaussian.cu:378-390).
 */
mppi_status mppi_inject_noise(mppi_handle* h, const float* noise, size_t count);

/* Run only the sampler of iteration iteration_num (SamplingDistribution::generateSamples, gaussian.cu:375-431 /
 * colored_noise.cu:285-392); the result is readable with mppi_get_control_samples. */
mppi_status mppi_generate_samples(mppi_handle* h, int optimization_stride, int iteration_num);

/* 1 = record each computeControl as a CUDA graph and replay it (default), 0 = plain stream launches. */
mppi_status mppi_set_graph_mode(mppi_handle* h, int enable);
/* Choose launch shapes by timing candidates on the device; cache_path (may be NULL) is a JSON file that stores and
 * restores the choice per (model, instance shape) key. */
mppi_status mppi_autotune(mppi_handle* h, const char* cache_path);
/* Rollout mode: 0 = one fused kernel per iteration (sampling, dynamics and costs, one thread per sample), 1 = split
 * dynamics / cost kernels (the dynamics chain alone, then all (k, t) costs in parallel, as the reference's
 * rolloutDynamicsKernel + rolloutCostKernel, mppi_common.cu:155-369), 2 = cooperative (four lanes per sample share
 * the sampling and cost work off the dynamics chain), 3 = the Gaussian sampler as its own kernel, then the rollout
 * on the staged samples (the reference's order: generateSamples, then the rollout kernel), 4 = the fused kernel with
 * noise warps (a second set of warps per CTA draws the tile's samples into shared memory ahead of the rollout warps,
 * which run only the dynamics and costs).  Modes 1, 2 and 4 are for problems too small to fill the GPU with one
 * thread per sample; all give bit-identical samples and costs.
 * available (may be NULL) receives the bitmask of modes this handle supports (bit m = mode m); modes 1 to 4 need
 * Gaussian sampling, T * C % 4 == 0 and an analytic model, mode 1 also at most 256 MB of stepped states, mode 4 a
 * horizon whose controls fit the shared-memory stage (T * C * 33 floats <= 200 KB).
 * mppi_autotune times every available mode. */
mppi_status mppi_set_rollout_mode(mppi_handle* h, int mode);
mppi_status mppi_get_rollout_mode(const mppi_handle* h, int* mode, int* available);
/* The launch shape in use: samples per rollout CTA, time chunk, samples per reduction CTA. */
mppi_status mppi_get_launch_config(const mppi_handle* h, int* rollout_samples_per_cta, int* rollout_time_chunk,
                                   int* reduction_samples_per_cta);
mppi_status mppi_set_launch_config(mppi_handle* h, int rollout_samples_per_cta, int rollout_time_chunk,
                                   int reduction_samples_per_cta);
/* Diagnostics (no counterpart in the reference) of rollout mode 4's one bounded wait: a rollout warp polls its noise
 * warp's progress word in shared memory at most max_polls times per quad of controls (0 restores the default, 2^22),
 * then gives up; the solve returns MPPI_ETIMEOUT and the handle stays usable.  withhold_progress != 0 makes the noise
 * warps stage their quads without publishing progress, so a test can make the wait run out on purpose (the kernel
 * still ends: every wait is bounded). */
mppi_status mppi_set_wait_diagnostics(mppi_handle* h, uint32_t max_polls, int withhold_progress);
/* Number of kernels one computeControl launches (for launch accounting). */
mppi_status mppi_kernels_per_compute(const mppi_handle* h, int* count);
/* Enqueue `count` device-resident solves (num_iters x sample/rollout/update each, as one replayed CUDA graph) on the
 * handle's stream without copying anything to or from the host and without synchronising: the initial states and
 * nominal controls already on the device are reused and the nominal controls keep evolving on the device.  This is
 * the steady-state GPU path of computeControl without its host round trip. */
mppi_status mppi_enqueue_solve(mppi_handle* h, int optimization_stride, int count);
/* Wait for the handle's stream. */
mppi_status mppi_synchronize(mppi_handle* h);
/* Average device time in ms of one launch of each kernel (ms_out[0] sampler, [1] rollout, [2] weights+update),
 * measured with CUDA events on the handle's stream over `reps` iterations. */
mppi_status mppi_time_kernels(mppi_handle* h, int optimization_stride, int reps, float* ms_out3);
/* The stream the handle enqueues on (a cudaStream_t). */
void* mppi_get_stream(const mppi_handle* h);

/* ---- learned dynamics surrogate (no reference counterpart; the reference only runs pre-trained networks,
 *      FNNHelper / NeuralNetModel, fnn_helper.cu:418-495, ar_nn_model.cu:127-156) ---------------------------------- */

/* 9 -> 64 -> 64 -> 5 tanh MLP: inputs (x, y, yaw, vx, vy, yaw_rate, steer, throttle, steer_cmd) normalised as
 * (v - in_mean) / in_std; outputs d/dt (yaw, vx, vy, yaw_rate, steer) as out * out_std + out_mean.  A parameter
 * vector is W1[64][9], b1[64], W2[64][64], b2[64], W3[5][64], b3[5], in_mean[9], in_std[9], out_mean[5],
 * out_std[5] (MPPI_MLP_PARAMS floats). */
#define MPPI_MLP_WEIGHTS 5125
#define MPPI_MLP_PARAMS 5153

typedef struct mppi_surrogate_config
{
  int num_transitions;               /* training set size (default 1 << 20) */
  float state_lower[7];              /* box the training states are drawn from, uniformly */
  float state_upper[7];
  uint64_t seed;
} mppi_surrogate_config;

typedef struct mppi_surrogate mppi_surrogate;

void mppi_default_surrogate_config(mppi_surrogate_config* cfg);
mppi_status mppi_surrogate_create(const mppi_bicycle_slip_params* dyn, const mppi_surrogate_config* cfg, void* stream,
                                  mppi_surrogate** out);
mppi_status mppi_surrogate_destroy(mppi_surrogate* s);
/* Draw the training transitions on the GPU from the analytic model and fix the input / output normalisation. */
mppi_status mppi_surrogate_generate(mppi_surrogate* s);
/* `steps` Adam steps on random mini-batches of `batch` transitions, learning rate decaying geometrically from lr to
 * lr_final; loss_out (may be NULL) receives the mini-batch loss of every step. */
mppi_status mppi_surrogate_train(mppi_surrogate* s, int steps, int batch, float lr, float lr_final, float* loss_out);
/* Weight format the training passes use (quantisation-aware training): 2 = FP32 (default), 0 = weights rounded to
 * BF16, 1 = E4M3 with the per-layer power-of-two scale of mppi_mlp_quantize.  Forward and backward run through the
 * rounded weights; Adam updates the FP32 master weights with that gradient (straight-through estimator). */
mppi_status mppi_surrogate_set_weight_format(mppi_surrogate* s, int precision);
/* Loss and parameter gradient on a given normalised batch (host X[B][9], Y[B][5]) with the training kernels (in the
 * weight format set above). */
mppi_status mppi_surrogate_gradient(mppi_surrogate* s, const float* X, const float* Y, int batch, float* grad_out,
                                    float* loss_out);
/* Root-mean-square error per output, in physical units, on n fresh transitions of the analytic model. */
mppi_status mppi_surrogate_validate(mppi_surrogate* s, int n, float* rmse5);
mppi_status mppi_surrogate_get_params(mppi_surrogate* s, float* out);
mppi_status mppi_surrogate_set_params(mppi_surrogate* s, const float* in);

/* Surrogate forward pass on the tensor cores (16-bit operands, FP32 accumulation) for `batch` rows of physical inputs
 * X_d[batch][9], writing physical outputs Y_d[batch][5] (device pointers); params is the host parameter vector and
 * precision selects BF16 (0) or FP8 E4M3 weights with one power-of-two scale per layer (1, FP16 operands).  The evaluation FNNHelper::forward
 * performs per sample (fnn_helper.cu:418-495), as one GEMM chain per 128 rows. */
mppi_status mppi_kernel_mlp_forward(const float* params, int precision, const float* X_d, float* Y_d, int batch,
                                    void* stream);
/* The weights the tensor cores see for a precision: out[MPPI_MLP_PARAMS] is params with every weight replaced by its
 * quantised value q (BF16 rounding happens on the device; FP8: the E4M3 value of W / scale), layer_scales[3] (may be
 * NULL) the per-layer scales (1 for BF16; for FP8 the smallest power of two with max |W| / scale <= 448).  W is
 * represented as q * scale. */
mppi_status mppi_mlp_quantize(const float* params, int precision, float* out, float* layer_scales);

/* ---- kernel-level entry points (mppi::kernels launchers, include/mppi/core/mppi_common.cuh:206-258) ----------- */

/* baseline = min, w = exp(-(c - baseline) * lambda_inv) in place, normaliser = sum w; out2[2*s] = baseline,
 * out2[2*s+1] = normaliser for each of num_systems arrays of num_rollouts costs (device pointers).
 * Replaces launchWeightTransformKernel (mppi_common.cu:1483-1506).  Scratch is allocated per call. */
mppi_status mppi_kernel_weight_transform(float* costs_d, float* out2_d, float lambda_inv, int num_rollouts,
                                         int num_systems, void* stream);
/* new_u[t][c] = sum_k (w_k / normaliser) u_k[t][c], normaliser read from baseline_norm_d[2*index+1] (device).
 * Replaces launchWeightedReductionKernel, device-normaliser variant (mppi_common.cu:1438-1454).  Scratch is
 * allocated per call. */
mppi_status mppi_kernel_weighted_reduction(const float* weights_d, const float* controls_d, float* new_u_d,
                                           const float* baseline_norm_d, int index, int num_timesteps,
                                           int num_rollouts, int control_dim, void* stream);
/* Same result as mppi_kernel_weighted_reduction for callers that may not allocate memory (a control loop with a
 * frozen memory map, a process whose GPU memory belongs to another allocator, a build that forbids allocation after
 * start-up).  No counterpart in the reference.  The scratch is one 4 MiB array inside the library's device image,
 * kept by every GPU that loads the library until exit; every call outside stream capture looks up its address on
 * the current device (cudaGetSymbolAddress) and a call under capture reuses the last address found there, so make
 * the first call on a device before any stream capture.  Limits: num_rollouts <= 65536 and
 * num_timesteps * control_dim <= 1024, else MPPI_EINVAL.  Calls share the array: calls that overlap on the GPU race
 * and must be serialised by the caller. */
mppi_status mppi_kernel_weighted_reduction_noalloc(const float* weights_d, const float* controls_d, float* new_u_d,
                                                   const float* baseline_norm_d, int index, int num_timesteps,
                                                   int num_rollouts, int control_dim, void* stream);
/* Rollout of K samples from x0 with the given (already constrained) controls, writing per-sample costs (device).
 * Replaces launchRolloutKernel (mppi_common.cu:1335-1361).  mean_d (float[T*C]) feeds the likelihood-ratio term. */
mppi_status mppi_kernel_rollout(int model, const void* dyn_params, size_t dyn_bytes, const void* cost_params,
                                size_t cost_bytes, const mppi_sampling_params* sampling, const float* x0_d,
                                const float* controls_d, const float* mean_d, float* costs_d, int num_rollouts,
                                int num_timesteps, float dt, float lambda, float alpha, void* stream);
/* In-place rewrite of standard-normal noise into control samples with constraints applied (setGaussianControls,
 * gaussian.cu:17-277, followed by Dynamics::enforceConstraints, dynamics.cu:107-126). */
mppi_status mppi_kernel_gaussian_controls(float* samples_d, const float* mean_d, const float* std_dev_h,
                                          const mppi_control_constraints* constraints, int num_rollouts,
                                          int num_timesteps, int control_dim, int optimization_stride,
                                          float std_dev_decay_pow, float pure_noise_percentage, void* stream);
/* Philox4x32-10 standard normals (Box-Muller) for n floats at counter offset, device output. */
mppi_status mppi_kernel_philox_normal(float* out_d, size_t n, uint64_t seed, uint64_t offset, void* stream);
/* Raw Philox4x32-10 blocks: out[4*i..4*i+3] = philox(ctr = {ctr0 + i, ctr1, ctr2, ctr3}, key), device output. */
mppi_status mppi_kernel_philox_raw(uint32_t* out_d, size_t nblocks, const uint32_t ctr[4], const uint32_t key[2],
                                   void* stream);
/* The engine's single-precision sine/cosine evaluated on n inputs (device), for bit-level parity checks. */
mppi_status mppi_kernel_sincos(const float* x_d, float* sin_d, float* cos_d, size_t n, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* MPPI_GB_H */
