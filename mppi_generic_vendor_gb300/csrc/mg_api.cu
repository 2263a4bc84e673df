// mg_api.cu — extern "C" entry points of libmppi_gb.so (declared in include/mppi_gb.h).
#include <cfloat>
#include <chrono>
#include <cstdarg>
#include <cstdio>
#include <fstream>
#include <sstream>

#include "mg_engine.cuh"

struct mppi_handle
{
  mg::EngineBase* engine;
};

namespace mg
{
static thread_local std::string g_last_error;

void set_error(const char* fmt, ...)
{
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
}

void clear_error() { g_last_error.clear(); }

// Minimal reader/writer for the autotune cache: a flat JSON object of "key": [ns, kc, rollout_mode] entries.
static bool cache_lookup(const char* path, const std::string& key, int* ns, int* kc, int* mode)
{
  if (!path) return false;
  std::ifstream f(path);
  if (!f) return false;
  std::stringstream ss;
  ss << f.rdbuf();
  const std::string s = ss.str();
  const std::string pat = "\"" + key + "\"";
  size_t p = s.find(pat);
  if (p == std::string::npos) return false;
  p = s.find('[', p);
  if (p == std::string::npos) return false;
  *mode = 0;
  return sscanf(s.c_str() + p, "[%d, %d, %d]", ns, kc, mode) >= 2 || sscanf(s.c_str() + p, "[%d,%d,%d]", ns, kc, mode) >= 2;
}

static void cache_store(const char* path, const std::string& key, int ns, int kc, int mode)
{
  if (!path) return;
  std::string body;
  {
    std::ifstream f(path);
    if (f)
    {
      std::stringstream ss;
      ss << f.rdbuf();
      body = ss.str();
    }
  }
  // keep the other entries: strip braces and re-emit
  std::string inner;
  size_t b = body.find('{'), e = body.rfind('}');
  if (b != std::string::npos && e != std::string::npos && e > b) inner = body.substr(b + 1, e - b - 1);
  // drop an old entry for this key
  const std::string pat = "\"" + key + "\"";
  size_t p = inner.find(pat);
  if (p != std::string::npos)
  {
    size_t q = inner.find(']', p);
    size_t end = (q == std::string::npos) ? inner.size() : q + 1;
    if (end < inner.size() && inner[end] == ',') end++;
    inner.erase(p, end - p);
  }
  while (!inner.empty() && (inner.back() == ',' || inner.back() == ' ' || inner.back() == '\n')) inner.pop_back();
  while (!inner.empty() && (inner.front() == ',' || inner.front() == ' ' || inner.front() == '\n')) inner.erase(0, 1);
  std::ofstream f(path);
  f << "{";
  if (!inner.empty()) f << inner << ", ";
  f << pat << ": [" << ns << ", " << kc << ", " << mode << "]}\n";
}

mppi_status autotune_impl(EngineBase* e, const char* cache_path, const std::string& key,
                          mppi_status (*time_one)(EngineBase*, float*))
{
  int ns = 0, kc = 0, mode = 0;
  if (cache_lookup(cache_path, key, &ns, &kc, &mode))
  {
    MG_TRY(e->set_launch_config(ns, 0, kc));
    return e->set_rollout_mode((e->rollout_modes() >> mode) & 1 ? mode : 0);
  }
  const int ns_c[4] = { 32, 64, 128, 256 };
  const int kc_c[3] = { 64, 128, 256 };
  float best = FLT_MAX;
  int best_ns = 128, best_kc = 128, best_mode = 0;
  for (int m = 0; m < 5; ++m)
  {
    if (!((e->rollout_modes() >> m) & 1)) continue;
    MG_TRY(e->set_rollout_mode(m));
    for (int a : ns_c)
      for (int b : kc_c)
      {
        MG_TRY(e->set_launch_config(a, 0, b));
        float ms = 0.0f;
        MG_TRY(time_one(e, &ms));
        if (ms < best)
        {
          best = ms;
          best_ns = a;
          best_kc = b;
          best_mode = m;
        }
      }
  }
  MG_TRY(e->set_rollout_mode(best_mode));
  MG_TRY(e->set_launch_config(best_ns, 0, best_kc));
  cache_store(cache_path, key, best_ns, best_kc, best_mode);
  return MPPI_OK;
}

static mppi_status model_dims(int model, int* s, int* c, int* o, size_t* db, size_t* cb)
{
  int S = 0, C = 0;
  size_t d = 0, q = 0;
  switch (model)
  {
    case MPPI_MODEL_CARTPOLE:
      S = CartpoleModel::STATE_DIM;
      C = CartpoleModel::CONTROL_DIM;
      d = sizeof(CartpoleModel::DynParams);
      q = sizeof(CartpoleModel::CostParams);
      break;
    case MPPI_MODEL_DOUBLE_INTEGRATOR:
      S = DoubleIntegratorModel::STATE_DIM;
      C = DoubleIntegratorModel::CONTROL_DIM;
      d = sizeof(DoubleIntegratorModel::DynParams);
      q = sizeof(DoubleIntegratorModel::CostParams);
      break;
    case MPPI_MODEL_BICYCLE_COSTMAP:
      S = BicycleCostmapModel::STATE_DIM;
      C = BicycleCostmapModel::CONTROL_DIM;
      d = sizeof(BicycleCostmapModel::DynParams);
      q = sizeof(BicycleCostmapModel::CostParams);
      break;
    case MPPI_MODEL_BICYCLE_SLIP:
    case MPPI_MODEL_BICYCLE_SLIP_MLP:
      S = BicycleSlipModel::STATE_DIM;
      C = BicycleSlipModel::CONTROL_DIM;
      d = sizeof(BicycleSlipModel::DynParams);
      q = sizeof(BicycleSlipModel::CostParams);
      break;
    default: set_error("unknown model id %d", model); return MPPI_EINVAL;
  }
  if (s) *s = S;
  if (c) *c = C;
  if (o) *o = S;
  if (db) *db = d;
  if (cb) *cb = q;
  return MPPI_OK;
}

// Scratch for the kernel-level update entry points, allocated on the stream and released after use.
struct StreamScratch
{
  void* p = nullptr;
  cudaStream_t s;
  explicit StreamScratch(cudaStream_t st) : s(st) {}
  ~StreamScratch()
  {
    if (p) cudaFreeAsync(p, s);
  }
  mppi_status alloc(size_t bytes)
  {
    cudaError_t e = cudaMallocAsync(&p, bytes, s);
    if (e != cudaSuccess)
    {
      p = nullptr;
      set_error("cudaMallocAsync(%zu) failed: %s", bytes, cudaGetErrorString(e));
      return MPPI_ENOMEM;
    }
    return MPPI_OK;
  }
};

}  // namespace mg

using namespace mg;

#define HANDLE_OK(h)                                                                                                  \
  do                                                                                                                  \
  {                                                                                                                   \
    if (!(h) || !(h)->engine)                                                                                         \
    {                                                                                                                 \
      set_error("invalid handle");                                                                                    \
      return MPPI_EINVAL;                                                                                             \
    }                                                                                                                 \
  } while (0)

extern "C" {

int mppi_abi_version(void) { return MPPI_GB_ABI_VERSION; }

const char* mppi_last_error_string(void) { return g_last_error.c_str(); }

mppi_status mppi_model_dims(int model, int* state_dim, int* control_dim, int* output_dim)
{
  return model_dims(model, state_dim, control_dim, output_dim, nullptr, nullptr);
}

mppi_status mppi_model_param_sizes(int model, size_t* dyn_bytes, size_t* cost_bytes)
{
  return model_dims(model, nullptr, nullptr, nullptr, dyn_bytes, cost_bytes);
}

void mppi_default_controller_params(mppi_controller_params* p)
{
  if (!p) return;
  memset(p, 0, sizeof(*p));
  p->dt = 0.02f;
  p->lambda = 1.0f;
  p->alpha = 0.0f;
  p->num_timesteps = 100;
  p->num_iters = 1;
  p->seed = 0;
  p->controller = MPPI_CONTROLLER_VANILLA;
  p->tsallis_r = 2.0f;  // ColoredMPPIParams defaults (colored_mppi_controller.cuh:17-22)
  p->tsallis_gamma = 0.0f;
  p->leash_active = 0;
  p->nominal_threshold = 20.0f;  // TubeMPPIParams (tube_mppi_controller.cuh:20)
  p->value_function_threshold = 1000.0f;  // RobustMPPIParams (robust_mppi_controller.cuh:15-22)
  p->num_candidate_nominal_states = 9;
  p->num_eval_samples_per_candidate = 64;
}

void mppi_default_sampling_params(mppi_sampling_params* p)
{
  if (!p) return;
  memset(p, 0, sizeof(*p));
  p->kind = MPPI_SAMPLER_GAUSSIAN;
  for (int i = 0; i < MPPI_MAX_CONTROL_DIM; ++i) p->std_dev[i] = 1.0f;
  p->pure_noise_trajectories_percentage = 0.01f;
  p->std_dev_decay = 1.0f;
  p->offset_decay_rate = 0.97f;
  p->fmin = 0.0f;
  p->use_same_noise_for_all_distributions = 1;
}

void mppi_default_constraints(mppi_control_constraints* c)
{
  if (!c) return;
  for (int i = 0; i < MPPI_MAX_CONTROL_DIM; ++i)
  {
    c->lower[i] = -FLT_MAX;
    c->upper[i] = FLT_MAX;
    c->deadband[i] = 0.0f;
    c->zero_control[i] = 0.0f;
  }
}

mppi_status mppi_create(int model, int num_instances, const int* num_rollouts, const int* num_timesteps,
                        const mppi_controller_params* params, const mppi_sampling_params* sampling,
                        const mppi_control_constraints* constraints, const void* dyn_params, size_t dyn_bytes,
                        const void* cost_params, size_t cost_bytes, const float* init_control, void* stream,
                        mppi_handle** out)
{
  clear_error();
  MG_CHECK(out, "out must not be NULL");
  *out = nullptr;
  MG_CHECK(params && sampling, "controller and sampling parameters are required");
  CreateArgs a;
  a.model = model;
  a.num_instances = num_instances;
  a.K = num_rollouts;
  a.T = num_timesteps;
  a.cp = *params;
  a.sp = *sampling;
  if (constraints)
    a.cc = *constraints;
  else
    mppi_default_constraints(&a.cc);
  a.dyn = dyn_params;
  a.dyn_bytes = dyn_bytes;
  a.cost = cost_params;
  a.cost_bytes = cost_bytes;
  a.init_control = init_control;
  a.stream = (cudaStream_t)stream;
  EngineBase* e = nullptr;
  mppi_status st;
  switch (model)
  {
    case MPPI_MODEL_CARTPOLE: st = create_cartpole_engine(a, &e); break;
    case MPPI_MODEL_DOUBLE_INTEGRATOR: st = create_double_integrator_engine(a, &e); break;
    case MPPI_MODEL_BICYCLE_COSTMAP: st = create_bicycle_costmap_engine(a, &e); break;
    case MPPI_MODEL_BICYCLE_SLIP: st = create_bicycle_slip_engine(a, &e); break;
    case MPPI_MODEL_BICYCLE_SLIP_MLP: st = create_bicycle_slip_mlp_engine(a, &e); break;
    default: set_error("unknown model id %d", model); return MPPI_EINVAL;
  }
  if (st != MPPI_OK) return st;
  mppi_handle* h = new mppi_handle;
  h->engine = e;
  *out = h;
  return MPPI_OK;
}

mppi_status mppi_handle_adopt(void* engine, int abi_version, mppi_handle** out)
{
  clear_error();
  MG_CHECK(out, "out must not be NULL");
  *out = nullptr;
  MG_CHECK(engine, "engine must not be NULL");
  MG_CHECK(abi_version == MPPI_GB_ABI_VERSION,
           "the plugin was built against ABI version %d of mppi_gb.h; this library is version %d: rebuild the plugin",
           abi_version, MPPI_GB_ABI_VERSION);
  mppi_handle* h = new mppi_handle;
  h->engine = static_cast<EngineBase*>(engine);
  *out = h;
  return MPPI_OK;
}

mppi_status mppi_get_model_dims(const mppi_handle* h, int* model, int* state_dim, int* control_dim, int* output_dim)
{
  HANDLE_OK(h);
  if (model) *model = h->engine->model();
  if (state_dim) *state_dim = h->engine->state_dim();
  if (control_dim) *control_dim = h->engine->control_dim();
  if (output_dim) *output_dim = h->engine->output_dim();
  return MPPI_OK;
}

mppi_status mppi_set_wait_diagnostics(mppi_handle* h, uint32_t max_polls, int withhold_progress)
{
  HANDLE_OK(h);
  return h->engine->set_wait_diagnostics(max_polls, withhold_progress);
}

mppi_status mppi_get_nominal_state_used(mppi_handle* h, int* used)
{
  HANDLE_OK(h);
  MG_CHECK(used, "used must not be NULL");
  return h->engine->nominal_state_used(used);
}

mppi_status mppi_rmppi_update_importance_sampler(mppi_handle* h, const float* state, int optimization_stride)
{
  HANDLE_OK(h);
  return h->engine->rmppi_update_importance_sampler(state, optimization_stride);
}
mppi_status mppi_rmppi_get_candidates(mppi_handle* h, int* best_index, int* nominal_stride, float* candidate_states,
                                      int* candidate_strides, float* candidate_free_energy, float* eval_costs)
{
  HANDLE_OK(h);
  return h->engine->rmppi_get_candidates(best_index, nominal_stride, candidate_states, candidate_strides,
                                         candidate_free_energy, eval_costs);
}

mppi_status mppi_set_feedback_params(mppi_handle* h, const float* Q, const float* Q_f, const float* R,
                                     int num_iterations)
{
  HANDLE_OK(h);
  return h->engine->set_feedback_params(Q, Q_f, R, num_iterations);
}
mppi_status mppi_enable_feedback(mppi_handle* h, int enable)
{
  HANDLE_OK(h);
  return h->engine->enable_feedback(enable);
}
mppi_status mppi_get_feedback_enabled(const mppi_handle* h, int* enabled)
{
  HANDLE_OK(h);
  MG_CHECK(enabled, "enabled must not be NULL");
  *enabled = h->engine->feedback_enabled();
  return MPPI_OK;
}
mppi_status mppi_compute_feedback(mppi_handle* h, const float* state)
{
  HANDLE_OK(h);
  return h->engine->compute_feedback(state);
}
mppi_status mppi_get_feedback_gains(const mppi_handle* h, float* out)
{
  HANDLE_OK(h);
  return h->engine->get_feedback_gains(out);
}
mppi_status mppi_get_feedback_control(const mppi_handle* h, const float* state, const float* goal_state, int t,
                                      float* out)
{
  HANDLE_OK(h);
  return h->engine->feedback_control(state, goal_state, t, out);
}
mppi_status mppi_get_feedback_propagated_state_seq(mppi_handle* h, float* out)
{
  HANDLE_OK(h);
  MG_CHECK(out, "out must not be NULL");
  return h->engine->feedback_propagated_state_seq(out);
}

mppi_status mppi_ddp_feedback_gains(int model, const void* dyn_params, size_t dyn_bytes, int num_timesteps, float dt,
                                    const float* x0, const float* target_states, const float* nominal_controls,
                                    const float* Q, const float* Q_f, const float* R, int num_iterations,
                                    const float* control_min, const float* control_max, float* gains_out)
{
  MG_CHECK(dyn_params && x0 && target_states && nominal_controls && control_min && control_max && gains_out,
           "pointer arguments other than the weights must not be NULL");
  MG_CHECK(num_timesteps >= 2, "num_timesteps must be >= 2 (got %d)", num_timesteps);
  MG_CHECK(num_iterations >= 1, "num_iterations must be >= 1 (got %d)", num_iterations);
  MG_CHECK(std::isfinite(dt) && dt > 0.0f, "dt must be positive");
  auto run = [&](auto model_tag) -> mppi_status {
    using Model = decltype(model_tag);
    constexpr int S = Model::STATE_DIM, C = Model::CONTROL_DIM;
    using P = typename Model::DynParams;
    MG_CHECK(dyn_bytes == sizeof(P), "dyn_bytes must be %zu for this model (got %zu)", sizeof(P), dyn_bytes);
    P p;
    memcpy(&p, dyn_params, sizeof(P));
    DdpWeights w;
    w.Q.assign((size_t)S * S, 0.0);
    w.Qf.assign((size_t)S * S, 0.0);
    w.R.assign((size_t)C * C, 0.0);
    for (int e = 0; e < S; ++e) w.Q[(size_t)e * S + e] = w.Qf[(size_t)e * S + e] = 1.0;
    for (int e = 0; e < C; ++e) w.R[(size_t)e * C + e] = 1.0;
    if (Q)
      for (int e = 0; e < S * S; ++e) w.Q[e] = Q[e];
    if (Q_f)
      for (int e = 0; e < S * S; ++e) w.Qf[e] = Q_f[e];
    if (R)
      for (int e = 0; e < C * C; ++e) w.R[e] = R[e];
    w.iterations = num_iterations;
    auto f = [&](const float* x, const float* u, float* xd) { Model::computeDynamics(p, x, u, xd); };
    auto df = [&](const float* x, const float* u, double* A, double* B) {
      if constexpr (HasAnalyticGrad<Model>::value)
      {
        if (Model::computeGrad(p, x, u, A, B)) return;
      }
      numeric_jacobian<S, C>(f, x, u, A, B);
    };
    const bool ok = ddp_tracking_gains<S, C>(f, df, x0, target_states, nominal_controls, num_timesteps, dt, w,
                                             control_min, control_max, gains_out);
    MG_CHECK(ok, "DDP feedback: a control Hessian is not positive definite (check R)");
    return MPPI_OK;
  };
  switch (model)
  {
    case MPPI_MODEL_CARTPOLE: return run(CartpoleModel{});
    case MPPI_MODEL_DOUBLE_INTEGRATOR: return run(DoubleIntegratorModel{});
    case MPPI_MODEL_BICYCLE_COSTMAP: return run(BicycleCostmapModel{});
    case MPPI_MODEL_BICYCLE_SLIP: return run(BicycleSlipModel{});
    default: set_error("mppi_ddp_feedback_gains: model %d has no host dynamics here", model); return MPPI_EUNSUPPORTED;
  }
}

mppi_status mppi_destroy(mppi_handle* h)
{
  if (!h) return MPPI_OK;
  delete h->engine;
  delete h;
  return MPPI_OK;
}

mppi_status mppi_get_instance_dims(const mppi_handle* h, int instance, int* num_rollouts, int* num_timesteps)
{
  HANDLE_OK(h);
  MG_CHECK(instance >= 0 && instance < h->engine->num_instances(), "instance %d out of range", instance);
  h->engine->dims(instance, num_rollouts, num_timesteps);
  return MPPI_OK;
}

mppi_status mppi_compute_control(mppi_handle* h, const float* x0, int optimization_stride)
{
  HANDLE_OK(h);
  return h->engine->compute_control(x0, optimization_stride);
}

mppi_status mppi_get_control_seq(mppi_handle* h, float* out)
{
  HANDLE_OK(h);
  return h->engine->get_control_seq(out);
}
mppi_status mppi_set_control_seq(mppi_handle* h, const float* in)
{
  HANDLE_OK(h);
  return h->engine->set_control_seq(in);
}
mppi_status mppi_slide_control_sequence(mppi_handle* h, int steps)
{
  HANDLE_OK(h);
  return h->engine->slide_control_sequence(steps);
}
mppi_status mppi_get_state_seq(mppi_handle* h, float* out)
{
  HANDLE_OK(h);
  return h->engine->get_state_seq(out);
}
mppi_status mppi_get_baseline_normalizer(mppi_handle* h, float* out, double* normalizer_fp64)
{
  HANDLE_OK(h);
  return h->engine->get_baseline_normalizer(out, normalizer_fp64);
}
mppi_status mppi_get_sample_costs(mppi_handle* h, float* out)
{
  HANDLE_OK(h);
  return h->engine->get_sample_costs(out);
}
mppi_status mppi_get_sample_weights(mppi_handle* h, float* out)
{
  HANDLE_OK(h);
  return h->engine->get_sample_weights(out);
}
mppi_status mppi_get_control_samples(mppi_handle* h, float* out)
{
  HANDLE_OK(h);
  return h->engine->get_control_samples(out);
}
mppi_status mppi_get_sampled_trajectories(mppi_handle* h, int instance, const int* idx, int n, float* states,
                                          float* step_costs, float* terminal, int* crash_status)
{
  HANDLE_OK(h);
  return h->engine->get_sampled_trajectories(instance, idx, n, states, step_costs, terminal, crash_status);
}
mppi_status mppi_select_top_samples(const float* weights, int num_samples, int n, int* indices)
{
  clear_error();
  MG_CHECK(weights && indices, "pointers must not be NULL");
  MG_CHECK(num_samples >= 1 && n >= 1 && n <= num_samples, "need 1 <= n <= num_samples");
  // Controller::copyTopControlFromDevice (controller.cu:126-181): start from the first n samples, then every later
  // weight strictly above the current minimum of the list replaces that minimum (first minimum in list order)
  for (int s = 0; s < n; ++s) indices[s] = s;
  int mi = 0;
  float mv = weights[indices[0]];
  auto find_min = [&]() {
    mi = 0;
    mv = weights[indices[0]];
    for (int s = 1; s < n; ++s)
      if (weights[indices[s]] < mv)
      {
        mv = weights[indices[s]];
        mi = s;
      }
  };
  find_min();
  for (int k = n; k < num_samples; ++k)
    if (weights[k] > mv)
    {
      indices[mi] = k;
      find_min();
    }
  return MPPI_OK;
}
mppi_status mppi_get_free_energy(mppi_handle* h, int instance, float* out6)
{
  HANDLE_OK(h);
  return h->engine->get_free_energy(instance, out6);
}
mppi_status mppi_set_dynamics_params(mppi_handle* h, const void* dyn_params, size_t dyn_bytes)
{
  HANDLE_OK(h);
  return h->engine->set_dynamics_params(dyn_params, dyn_bytes);
}
mppi_status mppi_set_cost_params(mppi_handle* h, const void* cost_params, size_t cost_bytes)
{
  HANDLE_OK(h);
  return h->engine->set_cost_params(cost_params, cost_bytes);
}
mppi_status mppi_set_sampling_params(mppi_handle* h, const mppi_sampling_params* sampling)
{
  HANDLE_OK(h);
  return h->engine->set_sampling_params(sampling);
}
mppi_status mppi_set_controller_params(mppi_handle* h, const mppi_controller_params* params)
{
  HANDLE_OK(h);
  return h->engine->set_controller_params(params);
}
mppi_status mppi_set_costmap(mppi_handle* h, const float* map, int width, int height, float resolution,
                             float origin_x, float origin_y)
{
  HANDLE_OK(h);
  return h->engine->set_costmap(map, width, height, resolution, origin_x, origin_y);
}
mppi_status mppi_set_mlp(mppi_handle* h, const float* params, size_t num_params, int precision)
{
  HANDLE_OK(h);
  return h->engine->set_mlp(params, num_params, precision);
}
mppi_status mppi_set_judge(mppi_handle* h, float fraction)
{
  HANDLE_OK(h);
  return h->engine->set_judge(fraction);
}
mppi_status mppi_get_judge_stats(mppi_handle* h, float* out)
{
  HANDLE_OK(h);
  return h->engine->get_judge_stats(out);
}
mppi_status mppi_use_analytic_dynamics(mppi_handle* h, int enable)
{
  HANDLE_OK(h);
  return h->engine->use_analytic(enable);
}
mppi_status mppi_inject_noise(mppi_handle* h, const float* noise, size_t count)
{
  HANDLE_OK(h);
  return h->engine->inject_noise(noise, count);
}
mppi_status mppi_generate_samples(mppi_handle* h, int optimization_stride, int iteration_num)
{
  HANDLE_OK(h);
  return h->engine->generate_samples(optimization_stride, iteration_num);
}
mppi_status mppi_set_graph_mode(mppi_handle* h, int enable)
{
  HANDLE_OK(h);
  return h->engine->set_graph_mode(enable);
}
mppi_status mppi_autotune(mppi_handle* h, const char* cache_path)
{
  HANDLE_OK(h);
  return h->engine->autotune(cache_path);
}
mppi_status mppi_set_rollout_mode(mppi_handle* h, int mode)
{
  HANDLE_OK(h);
  return h->engine->set_rollout_mode(mode);
}
mppi_status mppi_get_rollout_mode(const mppi_handle* h, int* mode, int* available)
{
  HANDLE_OK(h);
  if (mode) *mode = h->engine->rollout_mode();
  if (available) *available = h->engine->rollout_modes();
  return MPPI_OK;
}
mppi_status mppi_get_launch_config(const mppi_handle* h, int* rollout_samples_per_cta, int* rollout_time_chunk,
                                   int* reduction_samples_per_cta)
{
  HANDLE_OK(h);
  return h->engine->get_launch_config(rollout_samples_per_cta, rollout_time_chunk, reduction_samples_per_cta);
}
mppi_status mppi_set_launch_config(mppi_handle* h, int rollout_samples_per_cta, int rollout_time_chunk,
                                   int reduction_samples_per_cta)
{
  HANDLE_OK(h);
  return h->engine->set_launch_config(rollout_samples_per_cta, rollout_time_chunk, reduction_samples_per_cta);
}
mppi_status mppi_kernels_per_compute(const mppi_handle* h, int* count)
{
  HANDLE_OK(h);
  MG_CHECK(count, "count must not be NULL");
  *count = h->engine->kernels_per_compute();
  return MPPI_OK;
}
mppi_status mppi_enqueue_solve(mppi_handle* h, int optimization_stride, int count)
{
  HANDLE_OK(h);
  return h->engine->enqueue_device_solves(optimization_stride, count);
}
mppi_status mppi_synchronize(mppi_handle* h)
{
  HANDLE_OK(h);
  MG_CUDA(cudaStreamSynchronize(h->engine->stream()));
  return MPPI_OK;
}
mppi_status mppi_time_kernels(mppi_handle* h, int optimization_stride, int reps, float* ms_out3)
{
  HANDLE_OK(h);
  return h->engine->time_kernels(optimization_stride, reps, ms_out3);
}
void* mppi_get_stream(const mppi_handle* h)
{
  if (!h || !h->engine) return nullptr;
  return (void*)h->engine->stream();
}

// ---------------------------------------------------------------------------------------------- kernel-level entries

mppi_status mppi_kernel_weight_transform(float* costs_d, float* out2_d, float lambda_inv, int num_rollouts,
                                         int num_systems, void* stream)
{
  clear_error();
  MG_CHECK(costs_d && out2_d, "device pointers must not be NULL");
  MG_CHECK(num_rollouts >= 1 && num_systems >= 1, "num_rollouts and num_systems must be >= 1");
  cudaStream_t s = (cudaStream_t)stream;
  const int kc = 256;
  std::vector<InstDesc> inst(num_systems);
  std::vector<int4> chunks;
  std::vector<long long> part_off;
  std::vector<int> chunk0(num_systems);
  for (int i = 0; i < num_systems; ++i)
  {
    InstDesc& d = inst[i];
    memset(&d, 0, sizeof(d));
    d.K = num_rollouts;
    d.T = 1;
    d.k_off = i * num_rollouts;
    d.num_chunks = (num_rollouts + kc - 1) / kc;
    chunk0[i] = (int)chunks.size();
    for (int c = 0; c < d.num_chunks; ++c)
    {
      chunks.push_back(make_int4(i, c * kc, std::min(num_rollouts, (c + 1) * kc), c));
      part_off.push_back(0);
    }
  }
  const size_t nch = chunks.size();
  // one scratch block: descriptors, chunk table, offsets, chunk0, part_w, stats, counters
  size_t off = 0;
  auto take = [&](size_t bytes) {
    size_t o = off;
    off += (bytes + 255) / 256 * 256;
    return o;
  };
  const size_t o_inst = take(sizeof(InstDesc) * num_systems), o_chunks = take(sizeof(int4) * nch),
               o_poff = take(sizeof(long long) * nch), o_c0 = take(sizeof(int) * num_systems),
               o_pw = take(sizeof(double) * 2 * nch), o_stats = take(sizeof(double) * 3 * num_systems),
               o_bits = take(sizeof(unsigned int) * num_systems), o_arr = take(sizeof(unsigned int) * num_systems),
               o_cnt = take(sizeof(unsigned int) * 4), o_part = take(sizeof(float) * 4);
  StreamScratch scr(s);
  MG_TRY(scr.alloc(off));
  char* base = (char*)scr.p;
  MG_CUDA(cudaMemcpyAsync(base + o_inst, inst.data(), sizeof(InstDesc) * num_systems, cudaMemcpyHostToDevice, s));
  MG_CUDA(cudaMemcpyAsync(base + o_chunks, chunks.data(), sizeof(int4) * nch, cudaMemcpyHostToDevice, s));
  MG_CUDA(cudaMemcpyAsync(base + o_poff, part_off.data(), sizeof(long long) * nch, cudaMemcpyHostToDevice, s));
  MG_CUDA(cudaMemcpyAsync(base + o_c0, chunk0.data(), sizeof(int) * num_systems, cudaMemcpyHostToDevice, s));
  MG_CUDA(cudaMemsetAsync(base + o_arr, 0, sizeof(unsigned int) * num_systems, s));
  MG_CUDA(cudaMemsetAsync(base + o_cnt, 0, sizeof(unsigned int) * 4, s));
  unsigned int* bits = (unsigned int*)(base + o_bits);
  fill_u32_kernel<<<1, 256, 0, s>>>(bits, kOrderedPosInf, num_systems);
  dim3 mg_grid((num_rollouts + 255) / 256, num_systems);
  if (mg_grid.x > 64) mg_grid.x = 64;
  min_cost_kernel<<<mg_grid, 256, 0, s>>>(costs_d, num_rollouts, num_systems, bits);
  WeightsArgs a{};
  a.inst = (const InstDesc*)(base + o_inst);
  a.chunks = (const int4*)(base + o_chunks);
  a.part_off = (const long long*)(base + o_poff);
  a.inst_chunk0 = (const int*)(base + o_c0);
  a.num_chunks = (int)nch;
  a.num_instances = num_systems;
  a.costs = costs_d;
  a.weights = costs_d;  // in place, as fullGPUcomputeWeights transforms the cost array
  a.samples = nullptr;
  a.partials = (float*)(base + o_part);
  a.part_w = (double*)(base + o_pw);
  a.baseline_bits = bits;
  a.arrive = (unsigned int*)(base + o_arr);
  a.inst_done = (unsigned int*)(base + o_cnt);
  a.noise_counter = nullptr;
  a.mean_out = nullptr;
  a.baseline_norm = out2_d;
  a.stats = (double*)(base + o_stats);
  a.lambda_inv = lambda_inv;
  a.weights_given = 0;
  a.given_norm = nullptr;
  weights_update_kernel<1><<<(int)nch, 256, 0, s>>>(a);
  MG_CUDA(cudaGetLastError());
  return MPPI_OK;
}

mppi_status mppi_kernel_weighted_reduction(const float* weights_d, const float* controls_d, float* new_u_d,
                                           const float* baseline_norm_d, int index, int num_timesteps,
                                           int num_rollouts, int control_dim, void* stream)
{
  clear_error();
  MG_CHECK(weights_d && controls_d && new_u_d && baseline_norm_d, "device pointers must not be NULL");
  MG_CHECK(num_rollouts >= 1 && num_timesteps >= 1, "num_rollouts and num_timesteps must be >= 1");
  MG_CHECK(control_dim >= 1 && control_dim <= MPPI_MAX_CONTROL_DIM, "control_dim must be in [1, %d]",
           MPPI_MAX_CONTROL_DIM);
  MG_CHECK(index >= 0, "index must be >= 0");
  cudaStream_t s = (cudaStream_t)stream;
  const int kc = 128;
  const int nch = (num_rollouts + kc - 1) / kc;
  const int TC = num_timesteps * control_dim;
  InstDesc d;
  memset(&d, 0, sizeof(d));
  d.K = num_rollouts;
  d.T = num_timesteps;
  d.num_chunks = nch;
  std::vector<int4> chunks;
  std::vector<long long> part_off;
  for (int c = 0; c < nch; ++c)
  {
    chunks.push_back(make_int4(0, c * kc, std::min(num_rollouts, (c + 1) * kc), c));
    part_off.push_back((long long)c * TC);
  }
  const int chunk0 = 0;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    size_t o = off;
    off += (bytes + 255) / 256 * 256;
    return o;
  };
  const size_t o_inst = take(sizeof(InstDesc)), o_chunks = take(sizeof(int4) * nch),
               o_poff = take(sizeof(long long) * nch), o_c0 = take(sizeof(int)), o_pw = take(sizeof(double) * 2 * nch),
               o_stats = take(sizeof(double) * 3), o_cnt = take(sizeof(unsigned int) * 4),
               o_bn = take(sizeof(float) * 2), o_part = take(sizeof(float) * (size_t)nch * TC);
  StreamScratch scr(s);
  MG_TRY(scr.alloc(off));
  char* base = (char*)scr.p;
  MG_CUDA(cudaMemcpyAsync(base + o_inst, &d, sizeof(d), cudaMemcpyHostToDevice, s));
  MG_CUDA(cudaMemcpyAsync(base + o_chunks, chunks.data(), sizeof(int4) * nch, cudaMemcpyHostToDevice, s));
  MG_CUDA(cudaMemcpyAsync(base + o_poff, part_off.data(), sizeof(long long) * nch, cudaMemcpyHostToDevice, s));
  MG_CUDA(cudaMemcpyAsync(base + o_c0, &chunk0, sizeof(int), cudaMemcpyHostToDevice, s));
  MG_CUDA(cudaMemsetAsync(base + o_cnt, 0, sizeof(unsigned int) * 4, s));
  WeightsArgs a{};
  a.inst = (const InstDesc*)(base + o_inst);
  a.chunks = (const int4*)(base + o_chunks);
  a.part_off = (const long long*)(base + o_poff);
  a.inst_chunk0 = (const int*)(base + o_c0);
  a.num_chunks = nch;
  a.num_instances = 1;
  a.costs = nullptr;
  a.weights = const_cast<float*>(weights_d);
  a.samples = controls_d;
  a.partials = (float*)(base + o_part);
  a.part_w = (double*)(base + o_pw);
  a.baseline_bits = (unsigned int*)(base + o_cnt + 3 * sizeof(unsigned int));
  a.arrive = (unsigned int*)(base + o_cnt);
  a.inst_done = (unsigned int*)(base + o_cnt + sizeof(unsigned int));
  a.noise_counter = nullptr;
  a.mean_out = new_u_d;
  a.baseline_norm = (float*)(base + o_bn);
  a.stats = (double*)(base + o_stats);
  a.lambda_inv = 1.0f;
  a.weights_given = 1;
  a.given_norm = baseline_norm_d + 2 * (size_t)index + 1;
  switch (control_dim)
  {
    case 1: weights_update_kernel<1><<<nch, 256, 0, s>>>(a); break;
    case 2: weights_update_kernel<2><<<nch, 256, 0, s>>>(a); break;
    case 3: weights_update_kernel<3><<<nch, 256, 0, s>>>(a); break;
    default: weights_update_kernel<4><<<nch, 256, 0, s>>>(a); break;
  }
  MG_CUDA(cudaGetLastError());
  return MPPI_OK;
}

mppi_status mppi_kernel_rollout(int model, const void* dyn_params, size_t dyn_bytes, const void* cost_params,
                                size_t cost_bytes, const mppi_sampling_params* sampling, const float* x0_d,
                                const float* controls_d, const float* mean_d, float* costs_d, int num_rollouts,
                                int num_timesteps, float dt, float lambda, float alpha, void* stream)
{
  clear_error();
  size_t db = 0, cb = 0;
  MG_TRY(model_dims(model, nullptr, nullptr, nullptr, &db, &cb));
  MG_CHECK(dyn_params && cost_params && sampling, "parameter pointers must not be NULL");
  MG_CHECK(dyn_bytes == db && cost_bytes == cb, "parameter block sizes do not match the model");
  MG_CHECK(x0_d && controls_d && costs_d, "device pointers must not be NULL");
  cudaStream_t s = (cudaStream_t)stream;
  switch (model)
  {
    case MPPI_MODEL_CARTPOLE:
      return standalone_rollout_cartpole(dyn_params, cost_params, sampling, x0_d, controls_d, mean_d, costs_d,
                                         num_rollouts, num_timesteps, dt, lambda, alpha, s);
    case MPPI_MODEL_DOUBLE_INTEGRATOR:
      return standalone_rollout_double_integrator(dyn_params, cost_params, sampling, x0_d, controls_d, mean_d,
                                                  costs_d, num_rollouts, num_timesteps, dt, lambda, alpha, s);
    default: set_error("kernel-level rollout is built for the cartpole and double-integrator models"); return MPPI_EUNSUPPORTED;
  }
}

mppi_status mppi_kernel_gaussian_controls(float* samples_d, const float* mean_d, const float* std_dev_h,
                                          const mppi_control_constraints* constraints, int num_rollouts,
                                          int num_timesteps, int control_dim, int optimization_stride,
                                          float std_dev_decay_pow, float pure_noise_percentage, void* stream)
{
  clear_error();
  MG_CHECK(samples_d && mean_d && std_dev_h, "pointers must not be NULL");
  MG_CHECK(((uintptr_t)samples_d & 15) == 0, "samples must be 16-byte aligned");
  MG_CHECK(num_rollouts >= 1 && num_timesteps >= 1, "num_rollouts and num_timesteps must be >= 1");
  MG_CHECK(control_dim >= 1 && control_dim <= 2, "control_dim must be 1 or 2");
  cudaStream_t s = (cudaStream_t)stream;
  InstDesc d;
  memset(&d, 0, sizeof(d));
  d.K = num_rollouts;
  d.T = num_timesteps;
  const long long nq = ((long long)num_rollouts * num_timesteps * control_dim + 3) / 4;
  const int qpi = 2048;
  std::vector<int2> work;
  for (long long q = 0; q < nq; q += qpi) work.push_back(make_int2(0, (int)q));
  size_t off = 0;
  auto take = [&](size_t bytes) {
    size_t o = off;
    off += (bytes + 255) / 256 * 256;
    return o;
  };
  const size_t o_inst = take(sizeof(InstDesc)), o_work = take(sizeof(int2) * work.size());
  StreamScratch scr(s);
  MG_TRY(scr.alloc(off));
  char* base = (char*)scr.p;
  MG_CUDA(cudaMemcpyAsync(base + o_inst, &d, sizeof(d), cudaMemcpyHostToDevice, s));
  MG_CUDA(cudaMemcpyAsync(base + o_work, work.data(), sizeof(int2) * work.size(), cudaMemcpyHostToDevice, s));
  mppi_sampling_params sp;
  mppi_default_sampling_params(&sp);
  for (int c = 0; c < control_dim; ++c) sp.std_dev[c] = std_dev_h[c];
  sp.pure_noise_trajectories_percentage = pure_noise_percentage;
  mppi_control_constraints cc;
  if (constraints)
    cc = *constraints;
  else
    mppi_default_constraints(&cc);
  SampleArgs a;
  a.inst = (const InstDesc*)(base + o_inst);
  a.work = (const int2*)(base + o_work);
  a.num_work = (int)work.size();
  a.quads_per_item = qpi;
  a.samples = samples_d;
  a.mean = mean_d;
  a.injected = samples_d;  // in place: each thread reads and writes the same quad
  a.noise_counter = nullptr;
  a.seed_lo = a.seed_hi = 0;
  a.stride = optimization_stride;
  a.decay_pow = std_dev_decay_pow;
  a.sh = make_sample_shared(sp, cc);
  const int grid = std::min((int)work.size(), 1024);
  if (control_dim == 1)
    gaussian_sample_kernel<1><<<grid, 256, 0, s>>>(a);
  else
    gaussian_sample_kernel<2><<<grid, 256, 0, s>>>(a);
  MG_CUDA(cudaGetLastError());
  return MPPI_OK;
}

mppi_status mppi_kernel_philox_normal(float* out_d, size_t n, uint64_t seed, uint64_t offset, void* stream)
{
  clear_error();
  MG_CHECK(out_d, "out must not be NULL");
  if (n == 0) return MPPI_OK;
  const size_t nq = (n + 3) / 4;
  const int grid = (int)std::min<size_t>((nq + 255) / 256, 4096);
  philox_normal_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(out_d, n, (uint32_t)seed, (uint32_t)(seed >> 32),
                                                                offset);
  MG_CUDA(cudaGetLastError());
  return MPPI_OK;
}

mppi_status mppi_kernel_philox_raw(uint32_t* out_d, size_t nblocks, const uint32_t ctr[4], const uint32_t key[2],
                                   void* stream)
{
  clear_error();
  MG_CHECK(out_d && ctr && key, "pointers must not be NULL");
  if (nblocks == 0) return MPPI_OK;
  const int grid = (int)std::min<size_t>((nblocks + 255) / 256, 4096);
  philox_raw_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(out_d, nblocks, u32x4{ ctr[0], ctr[1], ctr[2], ctr[3] },
                                                             key[0], key[1]);
  MG_CUDA(cudaGetLastError());
  return MPPI_OK;
}

mppi_status mppi_kernel_sincos(const float* x_d, float* sin_d, float* cos_d, size_t n, void* stream)
{
  clear_error();
  MG_CHECK(x_d && sin_d && cos_d, "device pointers must not be NULL");
  if (n == 0) return MPPI_OK;
  const int grid = (int)std::min<size_t>((n + 255) / 256, 4096);
  sincos_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(x_d, sin_d, cos_d, n);
  MG_CUDA(cudaGetLastError());
  return MPPI_OK;
}

}  // extern "C"
