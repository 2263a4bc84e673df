// Double-integrator instantiation of the engine (DoubleIntegratorDynamics + goal/obstacle cost).
#include "mg_engine.cuh"

namespace mg
{
mppi_status create_double_integrator_engine(const CreateArgs& a, EngineBase** out)
{
  return Engine<DoubleIntegratorModel>::create(a, out);
}

mppi_status standalone_rollout_double_integrator(const void* dyn, const void* cost, const mppi_sampling_params* sp,
                                                 const float* x0_d, const float* controls_d, const float* mean_d,
                                                 float* costs_d, int K, int T, float dt, float lambda, float alpha,
                                                 cudaStream_t s)
{
  return standalone_rollout<DoubleIntegratorModel>(dyn, cost, sp, x0_d, controls_d, mean_d, costs_d, K, T, dt, lambda,
                                                   alpha, s);
}
}  // namespace mg
