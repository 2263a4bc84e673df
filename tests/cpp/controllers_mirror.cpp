// The C++ mirror's ColoredMPPIController, TubeMPPIController and RobustMPPIController (include/mppi_gb.hpp) on the
// GPU: each drives a simulated double integrator from (-1, -1) to the goal (1, 1) in a receding-horizon loop
// (Tube-MPPI and R-MPPI apply the nominal control plus the DDP feedback against the nominal state, as the reference's
// getCurrentControl does; R-MPPI updates its importance sampler before every solve).  Each must bring the robot from
// 2.83 to within 0.5 of the goal at a speed below 1.5 (the cost penalises speed lightly, so the robot still swings
// about the goal after 4 s); the robust controller's getNominalState must start its target trajectory, and its
// candidate free energies must be finite.
// Exits 0 on success.
#include <cmath>
#include <cstdio>

#include "mppi_gb.hpp"

using Dyn = mppi_gb::DoubleIntegratorDynamics;
using Cost = mppi_gb::DoubleIntegratorObstacleCost;
using FB = mppi_gb::DDPFeedback<Dyn, 50>;
constexpr int T = 50, K = 1024;
constexpr float DT = 0.02f;

static void robot_step(std::array<float, 4>& x, float u0, float u1)
{
  x[0] += DT * x[2];
  x[1] += DT * x[3];
  x[2] += DT * u0;
  x[3] += DT * u1;
}

static bool at_goal(const std::array<float, 4>& x, const char* name)
{
  const float d = std::hypot(x[0] - 1.0f, x[1] - 1.0f), v = std::hypot(x[2], x[3]);
  std::printf("%s: distance to goal %.3f, speed %.3f\n", name, d, v);
  return d < 0.5f && v < 1.5f;
}

int main()
{
  int failures = 0;
  Dyn dyn;
  dyn.setControlRanges({ std::pair<float, float>{ -2.0f, 2.0f }, { -2.0f, 2.0f } });
  Cost cost;
  cost.params.goal[0] = cost.params.goal[1] = 1.0f;
  cost.params.terminal_coeff = 5.0f;
  // ---- ColoredMPPI (exponential weights with the default gamma = 0, then Tsallis weights)
  {
    mppi_gb::ColoredNoiseDistribution sampler(std::array<float, 2>{ 1.0f, 1.0f }, std::array<float, 2>{ 1.0f, 1.0f });
    mppi_gb::ColoredMPPIController<Dyn, Cost, mppi_gb::NoFeedback, T, K> ctrl(&dyn, &cost, nullptr, &sampler, DT, 1,
                                                                              1.0f, 0.0f);
    ctrl.setGamma(1.0f);
    ctrl.setRExp(2.0f);
    std::array<float, 4> x{ -1.0f, -1.0f, 0.0f, 0.0f };
    for (int it = 0; it < 200; ++it)
    {
      ctrl.computeControl(x, 1);
      const auto u = ctrl.getControlSeq();
      robot_step(x, u[0], u[1]);
      ctrl.slideControlSequence(1);
    }
    if (!at_goal(x, "colored") || ctrl.getGamma() != 1.0f) ++failures;
  }
  // ---- Tube-MPPI with feedback
  {
    mppi_gb::GaussianDistribution sampler(std::array<float, 2>{ 1.0f, 1.0f });
    FB fb(&dyn, DT);
    mppi_gb::TubeMPPIController<Dyn, Cost, FB, T, K> ctrl(&dyn, &cost, &fb, &sampler, DT, 1, 1.0f, 0.0f);
    std::array<float, 4> x{ -1.0f, -1.0f, 0.0f, 0.0f };
    for (int it = 0; it < 200; ++it)
    {
      ctrl.computeControl(x, 1);
      ctrl.computeFeedback(x);
      const auto u = ctrl.getControlSeq();
      const auto nominal = ctrl.getTargetStateSeq();
      const std::array<float, 4> xn{ nominal[0], nominal[1], nominal[2], nominal[3] };
      const auto ufb = ctrl.getFeedbackControl(x, xn, 0);
      robot_step(x, u[0] + ufb[0], u[1] + ufb[1]);
      ctrl.slideControlSequence(1);
    }
    const auto nominal_u = ctrl.getControlSeq();
    const auto actual_u = ctrl.getActualControlSeq();
    (void)actual_u;
    if (!at_goal(x, "tube") || !ctrl.getFeedbackEnabled() || !std::isfinite(nominal_u[0])) ++failures;
  }
  // ---- R-MPPI
  {
    mppi_gb::GaussianDistribution sampler(std::array<float, 2>{ 1.0f, 1.0f });
    FB fb(&dyn, DT);
    mppi_gb::RobustMPPIController<Dyn, Cost, FB, T, K> ctrl(&dyn, &cost, &fb, &sampler, DT, 1, 1.0f, 0.0f, 1000.0f, T,
                                                            mppi_gb::RobustMPPIController<Dyn, Cost, FB, T, K>::
                                                                control_trajectory{},
                                                            5, 1, nullptr, 0, 32);
    std::array<float, 4> x{ -1.0f, -1.0f, 0.0f, 0.0f };
    int bad = 0;
    for (int it = 0; it < 200; ++it)
    {
      ctrl.updateImportanceSamplingControl(x, 1);
      ctrl.computeControl(x, 1);
      const auto u = ctrl.getControlSeq();
      const auto target = ctrl.getTargetStateSeq();
      const auto xn = ctrl.getNominalState();
      for (int s = 0; s < 4; ++s) bad += xn[s] != target[s];
      const auto ufb = ctrl.getFeedbackControl(x, xn, 0);
      robot_step(x, u[0] + ufb[0], u[1] + ufb[1]);
      for (float f : ctrl.getCandidateFreeEnergy()) bad += !std::isfinite(f);
    }
    std::printf("robust: best candidate %d of %d\n", ctrl.getBestIndex(), ctrl.getNumCandidates());
    if (!at_goal(x, "robust") || bad) ++failures;
  }
  return failures == 0 ? 0 : 1;
}
