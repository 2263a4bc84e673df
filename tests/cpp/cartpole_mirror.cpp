// The C++ host mirror (include/mppi_gb.hpp): the receding-horizon cart-pole loop of MPPI-Generic's
// examples/cartpole_example.cu:62-85 written with the reference's class and method names (VanillaMPPIController
// <DYN_T, COST_T, FB_T, MAX_TIMESTEPS, NUM_ROLLOUTS, SAMPLING_T>, computeControl, getControlSeq,
// slideControlSequence, getBaselineCost), plus a kinematic-bicycle controller on a costmap to exercise the
// plugin-specific set-up.  Exits 0 when the pole has been held up for more than 100 of 500 steps and the bicycle
// controller produced finite controls.
#include <cmath>
#include <cstdio>
#include <vector>

#include "mppi_gb.hpp"

using namespace mppi_gb;

int main()
{
  constexpr int T = 100, K = 2048;
  CartpoleDynamics dyn(1.0f, 1.0f, 1.0f);
  dyn.setControlRanges({ std::pair<float, float>{ -5.0f, 5.0f } });
  CartpoleSwingupCost cost(10.0f, 1.0f, 100.0f, 1.0f, 0.0f);
  GaussianDistribution sampler(std::array<float, 1>{ 1.0f });
  NoFeedback fb;
  VanillaMPPIController<CartpoleDynamics, CartpoleSwingupCost, NoFeedback, T, K> controller(
      &dyn, &cost, &fb, &sampler, 0.02f, 1, 1.0f, 0.0f, T, {}, nullptr, 42);
  std::array<double, 4> x = { 0.0, 0.0, 0.0, 0.0 };
  int upright = 0;
  for (int step = 0; step < 500; ++step)
  {
    controller.computeControl({ (float)x[0], (float)x[1], (float)x[2], (float)x[3] }, 1);
    const auto u = controller.getControlSeq();
    const double f = u[0], s = std::sin(x[2]), c = std::cos(x[2]);
    const double xdd = (f + s * (x[3] * x[3] + 9.81 * c)) / (1.0 + s * s);
    const double tdd = (-f * c - x[3] * x[3] * c * s - 2.0 * 9.81 * s) / (1.0 + s * s);
    x[0] += 0.02 * x[1];
    x[1] += 0.02 * xdd;
    x[2] += 0.02 * x[3];
    x[3] += 0.02 * tdd;
    controller.slideControlSequence(1);
    if (1.0 + std::cos(x[2]) < 0.05) ++upright;
  }
  std::printf("cart-pole: upright for %d of 500 steps, last baseline %.4f, normaliser %.4f\n", upright,
              controller.getBaselineCost(), controller.getNormalizerCost());
  // visualisation read-out: the five highest-weight samples of the last solve, re-rolled on the GPU
  controller.setTopNSampledControlTrajectories(5);
  controller.calculateSampledStateTrajectories({ 0, 1 });
  const auto vis = controller.getSampledOutputTrajectories();
  const auto top = controller.getTopTransformedCosts();
  bool vis_ok = vis.size() == 7 && top.size() == 5 && vis[0].size() == (size_t)4 * T;
  for (float v : top) vis_ok = vis_ok && v > 0.0f && v <= 1.0f;
  std::printf("sampled trajectories: %zu, top weights ok %d\n", vis.size(), (int)vis_ok);

  BicycleDynamics bike(2.5f);
  CostmapCost map_cost;
  map_cost.width = map_cost.height = 64;
  map_cost.map.assign(64 * 64, 0.0f);
  for (int r = 0; r < 64; ++r)
    for (int q = 0; q < 64; ++q) map_cost.map[r * 64 + q] = 0.01f * (float)((r - 32) * (r - 32) + (q - 32) * (q - 32));
  GaussianDistribution bike_sampler(std::array<float, 2>{ 1.0f, 0.3f });
  VanillaMPPIController<BicycleDynamics, CostmapCost, NoFeedback, 50, 1024> bike_controller(
      &bike, &map_cost, &fb, &bike_sampler, 0.02f, 2, 2.0f, 0.0f);
  bike_controller.computeControl({ 3.0f, 3.0f, 0.3f, 4.0f });
  const auto ub = bike_controller.getControlSeq();
  bool finite = true;
  for (int i = 0; i < 2 * 50; ++i) finite = finite && std::isfinite(ub[i]);
  bool threw = false;
  try
  {
    bike_controller.slideControlSequence(-1);
  }
  catch (const Error& e)
  {
    threw = e.status == MPPI_EINVAL;
  }
  std::printf("bicycle: finite controls %d, bad argument reported %d\n", (int)finite, (int)threw);
  return upright > 100 && finite && threw && vis_ok ? 0 : 1;
}
