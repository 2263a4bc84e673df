// Cartpole instantiation of the engine (CartpoleDynamics + swing-up cost).
#include "mg_engine.cuh"

namespace mg
{
mppi_status create_cartpole_engine(const CreateArgs& a, EngineBase** out)
{
  return Engine<CartpoleModel>::create(a, out);
}

mppi_status standalone_rollout_cartpole(const void* dyn, const void* cost, const mppi_sampling_params* sp,
                                        const float* x0_d, const float* controls_d, const float* mean_d,
                                        float* costs_d, int K, int T, float dt, float lambda, float alpha,
                                        cudaStream_t s)
{
  return standalone_rollout<CartpoleModel>(dyn, cost, sp, x0_d, controls_d, mean_d, costs_d, K, T, dt, lambda, alpha,
                                           s);
}
}  // namespace mg
