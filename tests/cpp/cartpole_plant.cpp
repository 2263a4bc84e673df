// The C++ BasePlant (include/mppi_gb_plant.hpp) driving the real GPU controller of the C++ mirror: a simulated
// cart-pole robot whose state estimator reports every 5 ms of robot time (updateState, which publishes the control
// interpolated at that time) while the plant re-optimises every 20 ms of robot time from the newest state.
//  1. single-threaded: the robot and runControlIteration alternate; the pole must be swung up and held
//     (1 + cos theta < 0.05) for more than 100 of the 500 control periods, every iteration must slide by the
//     target stride, and a parameter block handed over between iterations must reach the controller;
//  2. threaded: runControlLoop on its own thread against the robot on the main thread, stopped through is_alive;
//  3. with the DDP feedback controller on: every solve is followed by computeFeedback, the plant keeps the gains of
//     the last solve and publishes getCurrentControl (nominal control plus feedback, constrained): the gains must be
//     finite and not all zero, the published controls inside the control range, the feedback-propagated states
//     finite and starting at the state optimised from.
// Exits 0 on success.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <memory>
#include <thread>

#include "mppi_gb_plant.hpp"

using Controller = mppi_gb::VanillaMPPIController<mppi_gb::CartpoleDynamics, mppi_gb::CartpoleSwingupCost,
                                                  mppi_gb::NoFeedback, 100, 2048>;
using Feedback = mppi_gb::DDPFeedback<mppi_gb::CartpoleDynamics, 100>;
using FBController = mppi_gb::VanillaMPPIController<mppi_gb::CartpoleDynamics, mppi_gb::CartpoleSwingupCost, Feedback,
                                                    100, 2048>;

template <class CTRL>
class CartpolePlantT : public mppi_gb::BasePlant<CTRL>
{
public:
  using Base = mppi_gb::BasePlant<CTRL>;
  using Base::Base;
  std::atomic<float> u{ 0.0f }, max_abs_u{ 0.0f };
  std::atomic<int> published{ 0 }, stats{ 0 };
  double now = 0.0;
  void pubControl(const typename Base::c_array& v) override
  {
    u = v[0];
    max_abs_u = std::max(max_abs_u.load(), std::fabs(v[0]));
    ++published;
  }
  void pubNominalState(const typename Base::s_array&) override {}
  void pubFreeEnergyStatistics(const mppi_gb::FreeEnergyStatistics& fe) override
  {
    if (std::isfinite(fe.freeEnergyMean)) ++stats;
  }
  int checkStatus() override { return 0; }
  double getCurrentTime() override { return now; }
  double getPoseTime() override { return now; }
};
using CartpolePlant = CartpolePlantT<Controller>;

// explicit Euler of the cart-pole ODE (cartpole_dynamics.cu:48-67) over h seconds
static void robot_step(double* x, double f, double h)
{
  const double s = std::sin(x[2]), c = std::cos(x[2]), mc = 1.0, mp = 1.0, l = 1.0, g = 9.81;
  const double xdd = (f + mp * s * (l * x[3] * x[3] + g * c)) / (mc + mp * s * s);
  const double tdd = (-f * c - mp * l * x[3] * x[3] * c * s - (mc + mp) * g * s) / (l * (mc + mp * s * s));
  x[0] += h * x[1];
  x[1] += h * xdd;
  x[2] += h * x[3];
  x[3] += h * tdd;
}

static Controller::state_array as_state(const double* x)
{
  return Controller::state_array{ (float)x[0], (float)x[1], (float)x[2], (float)x[3] };
}

static std::shared_ptr<Controller> make_controller()
{
  mppi_gb::CartpoleDynamics dyn(1.0f, 1.0f, 1.0f);
  dyn.setControlRanges({ std::pair<float, float>{ -5.0f, 5.0f } });
  mppi_gb::CartpoleSwingupCost cost(10.0f, 1.0f, 100.0f, 1.0f, 0.0f);
  mppi_gb::GaussianDistribution sampler(std::array<float, 1>{ 1.0f });
  return std::make_shared<Controller>(&dyn, &cost, nullptr, &sampler, 0.02f, 1, 1.0f, 0.0f, 100,
                                      Controller::control_trajectory{}, nullptr, 42);
}

int main()
{
  int failures = 0;
  // ---- 1. single-threaded, deterministic robot time
  {
    CartpolePlant plant(make_controller(), 50, 1);
    std::atomic<bool> alive{ true };
    double x[4] = { 0.0, 0.0, 0.0, 0.0 };
    plant.updateState(as_state(x), 0.0);
    int upright = 0, bad_stride = 0;
    for (int k = 0; k < 500; ++k)
    {
      if (!plant.runControlIteration(&alive)) ++failures;
      if (k > 0 && plant.getLastOptimizationStride() != 1) ++bad_stride;
      if (k == 250)
      {
        // a new cost block from "another thread": cart position no longer penalised
        mppi_gb::CartpoleSwingupCost c2(0.0f, 1.0f, 100.0f, 1.0f, 0.0f);
        plant.setCostParams(c2.params);
      }
      for (int sub = 0; sub < 4; ++sub)
      {
        robot_step(x, plant.u.load(), 0.005);
        plant.now += 0.005;
        plant.updateState(as_state(x), plant.now);
      }
      if (1.0 + std::cos(x[2]) < 0.05) ++upright;
    }
    std::printf("single-threaded: %d iterations, %d published controls, upright for %d of 500 periods, theta=%.3f\n",
                plant.getNumIterations(), plant.published.load(), upright, x[2]);
    if (plant.getNumIterations() != 500 || upright <= 100 || bad_stride || plant.hasNewCostParams() ||
        plant.stats.load() != 500 || plant.published.load() < 1500)
    {
      std::printf("FAILED: bad_stride=%d new_cost_pending=%d stats=%d\n", bad_stride, (int)plant.hasNewCostParams(),
                  plant.stats.load());
      ++failures;
    }
  }
  // ---- 2. runControlLoop on its own thread
  {
    CartpolePlant plant(make_controller(), 50, 1);
    std::atomic<bool> alive{ true };
    double x[4] = { 0.0, 0.0, 0.0, 0.0 };
    plant.updateState(as_state(x), 0.0);
    std::thread loop([&] { plant.runControlLoop(&alive); });
    for (int k = 0; k < 2000 && plant.getNumIterations() < 40; ++k)
    {
      robot_step(x, plant.u.load(), 0.005);
      plant.now += 0.005;
      plant.updateState(as_state(x), plant.now);
      std::this_thread::sleep_for(std::chrono::milliseconds(1));
    }
    alive = false;
    loop.join();
    std::printf("threaded: %d iterations, average optimisation %.3f ms\n", plant.getNumIterations(),
                plant.getAvgOptimizationTime());
    if (plant.getNumIterations() < 40) ++failures;
  }
  // ---- 3. the DDP feedback controller on
  {
    mppi_gb::CartpoleDynamics dyn(1.0f, 1.0f, 1.0f);
    dyn.setControlRanges({ std::pair<float, float>{ -5.0f, 5.0f } });
    mppi_gb::CartpoleSwingupCost cost(10.0f, 1.0f, 100.0f, 1.0f, 0.0f);
    mppi_gb::GaussianDistribution sampler(std::array<float, 1>{ 1.0f });
    Feedback fb(&dyn, 0.02f);
    auto ctrl = std::make_shared<FBController>(&dyn, &cost, &fb, &sampler, 0.02f, 1, 1.0f, 0.0f, 100,
                                               FBController::control_trajectory{}, nullptr, 7);
    auto params = fb.getParams();
    params.Q = { 10.0f, 0, 0, 0, 0, 1.0f, 0, 0, 0, 0, 50.0f, 0, 0, 0, 0, 1.0f };
    params.R = { 0.1f };
    fb.setParams(params);  // reaches the controller built with fb
    ctrl->initFeedback();
    CartpolePlantT<FBController> plant(ctrl, 50, 1);
    std::atomic<bool> alive{ true };
    double x[4] = { 0.0, 0.0, 0.0, 0.0 };
    plant.updateState(as_state(x), 0.0);
    for (int k = 0; k < 200; ++k)
    {
      if (!plant.runControlIteration(&alive)) ++failures;
      for (int sub = 0; sub < 4; ++sub)
      {
        robot_step(x, plant.u.load(), 0.005);
        plant.now += 0.005;
        plant.updateState(as_state(x), plant.now);
      }
    }
    const auto gains = plant.getFeedbackState();
    int nonzero = 0, nonfinite = 0;
    for (float g : gains.fb_gain_traj_)
    {
      nonzero += g != 0.0f;
      nonfinite += !std::isfinite(g);
    }
    const auto prop = ctrl->getFeedbackPropagatedStateSeq();
    const auto target = ctrl->getTargetStateSeq();
    int prop_bad = 0;
    for (int i = 0; i < 4 * 100; ++i) prop_bad += !std::isfinite(prop[i]);
    for (int i = 0; i < 4; ++i) prop_bad += prop[i] != target[i];
    std::printf("feedback: %d iterations, %d non-zero gains, max |u| published %.3f, average feedback %.3f ms, "
                "theta=%.3f\n",
                plant.getNumIterations(), nonzero, plant.max_abs_u.load(), plant.getAvgFeedbackTime(), x[2]);
    if (plant.getNumIterations() != 200 || nonzero == 0 || nonfinite || prop_bad || plant.max_abs_u.load() > 5.0f ||
        !(plant.getAvgFeedbackTime() > 0.0) || !ctrl->getFeedbackEnabled())
    {
      std::printf("FAILED: nonfinite=%d prop_bad=%d\n", nonfinite, prop_bad);
      ++failures;
    }
  }
  return failures == 0 ? 0 : 1;
}
