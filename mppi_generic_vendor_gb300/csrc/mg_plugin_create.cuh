// mg_plugin_create.cuh — instantiation of the engine over a caller's plugin pair (included by
// include/mppi_gb_plugin.cuh, expanded by MPPI_GB_PLUGIN in the caller's own translation unit).
//
// The caller's library instantiates Engine<PluginModel<D, Cst>> (every kernel it launches is compiled into that
// library) and hands the engine to libmppi_gb.so with mppi_handle_adopt, so the handle is served by the same C entry
// points as the built-in models.  This stands in for the reference's template instantiation of its controller over
// the caller's plugin classes (Controller<DYN_T, COST_T, ...>, controller.cuh:70-72).
#pragma once

#include <type_traits>

#include "mg_engine.cuh"

namespace mg
{
template <class D, class Cst>
mppi_status plugin_create(int num_instances, const int* num_rollouts, const int* num_timesteps,
                          const mppi_controller_params* params, const mppi_sampling_params* sampling,
                          const mppi_control_constraints* constraints, const void* dyn_params, size_t dyn_bytes,
                          const void* cost_params, size_t cost_bytes, const float* init_control, void* stream,
                          mppi_handle** out)
{
  static_assert(std::is_trivially_copyable<D>::value && std::is_trivially_copyable<Cst>::value,
                "plugin structs are copied to the GPU by value: they must be trivially copyable");
  static_assert(D::STATE_DIM >= 1 && D::STATE_DIM <= MPPI_MAX_STATE_DIM, "STATE_DIM must be in [1, 8]");
  static_assert(D::CONTROL_DIM >= 1 && D::CONTROL_DIM <= MPPI_MAX_CONTROL_DIM, "CONTROL_DIM must be in [1, 4]");
  static_assert(Cst::OUTPUT_DIM == D::OUTPUT_DIM && Cst::CONTROL_DIM == D::CONTROL_DIM,
                "the cost's OUTPUT_DIM / CONTROL_DIM must match the dynamics'");
  clear_error();
  MG_CHECK(out, "out must not be NULL");
  *out = nullptr;
  MG_CHECK(params && sampling, "controller and sampling parameters are required");
  CreateArgs a;
  a.model = MPPI_MODEL_PLUGIN;
  a.num_instances = num_instances;
  a.K = num_rollouts;
  a.T = num_timesteps;
  a.cp = *params;
  a.sp = *sampling;
  if (constraints)
    a.cc = *constraints;
  else
    mppi_default_constraints(&a.cc);
  // one plugin struct for every instance, or one per instance
  std::vector<unsigned char> dyn_all, cost_all;
  MG_CHECK(dyn_params && cost_params, "parameter blocks must not be NULL");
  MG_CHECK(num_instances >= 1, "num_instances must be >= 1 (got %d)", num_instances);
  auto expand = [&](const void* p, size_t bytes, size_t one, std::vector<unsigned char>& v, const char* what) {
    if (bytes == one * (size_t)num_instances) return (const void*)p;
    if (bytes != one) return (const void*)nullptr;
    v.resize(one * num_instances);
    for (int i = 0; i < num_instances; ++i) memcpy(v.data() + one * i, p, one);
    (void)what;
    return (const void*)v.data();
  };
  a.dyn = expand(dyn_params, dyn_bytes, sizeof(D), dyn_all, "dynamics");
  a.cost = expand(cost_params, cost_bytes, sizeof(Cst), cost_all, "cost");
  MG_CHECK(a.dyn, "dynamics parameters are %zu bytes; the plugin expects %zu (all instances) or %zu (one each)",
           dyn_bytes, sizeof(D), sizeof(D) * num_instances);
  MG_CHECK(a.cost, "cost parameters are %zu bytes; the plugin expects %zu (all instances) or %zu (one each)",
           cost_bytes, sizeof(Cst), sizeof(Cst) * num_instances);
  a.dyn_bytes = sizeof(D);
  a.cost_bytes = sizeof(Cst);
  a.init_control = init_control;
  a.stream = (cudaStream_t)stream;
  EngineBase* e = nullptr;
  using PluginEngine = Engine<PluginModel<D, Cst>>;
  MG_TRY(PluginEngine::create(a, &e));
  const mppi_status st = mppi_handle_adopt(e, MPPI_GB_ABI_VERSION, out);
  if (st != MPPI_OK) delete e;
  return st;
}
}  // namespace mg
