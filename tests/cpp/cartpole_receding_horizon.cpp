// A reference-side C++ caller of the C ABI: the receding-horizon cart-pole loop of MPPI-Generic's
// examples/cartpole_example.cu:62-85 (computeControl, apply the first control, step the plant, slide the sequence),
// written against include/mppi_gb.h only.  The swing-up cost 100 (1 + cos theta)^2 puts the pole up at theta = pi;
// the program exits 0 when the pole has been held up (1 + cos theta < 0.05) for more than 100 of 500 steps.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "mppi_gb.h"

static void check(mppi_status s, const char* what)
{
  if (s != MPPI_OK)
  {
    std::fprintf(stderr, "%s failed: %s\n", what, mppi_last_error_string());
    std::exit(2);
  }
}

int main()
{
  const int K = 2048, T = 100;
  mppi_controller_params p;
  mppi_default_controller_params(&p);
  p.dt = 0.02f;
  p.lambda = 1.0f;
  p.num_timesteps = T;
  p.num_iters = 1;
  p.seed = 42;
  mppi_sampling_params sp;
  mppi_default_sampling_params(&sp);
  sp.std_dev[0] = 1.0f;
  mppi_control_constraints cc;
  mppi_default_constraints(&cc);
  cc.lower[0] = -5.0f;
  cc.upper[0] = 5.0f;
  const mppi_cartpole_params dyn = { 1.0f, 1.0f, 1.0f, 9.81f };
  const mppi_cartpole_cost_params cost = { 10.0f, 1.0f, 100.0f, 1.0f, 0.0f };
  mppi_handle* h = nullptr;
  check(mppi_create(MPPI_MODEL_CARTPOLE, 1, &K, &T, &p, &sp, &cc, &dyn, sizeof dyn, &cost, sizeof cost, nullptr,
                    nullptr, &h),
        "mppi_create");
  // plant: explicit Euler of the cart-pole ODE (cartpole_dynamics.cu:48-67), starting at rest, pole down
  double x[4] = { 0.0, 0.0, 0.0, 0.0 };
  std::vector<float> u(T);
  int upright = 0;
  for (int step = 0; step < 500; ++step)
  {
    const float xf[4] = { (float)x[0], (float)x[1], (float)x[2], (float)x[3] };
    check(mppi_compute_control(h, xf, 1), "mppi_compute_control");
    check(mppi_get_control_seq(h, u.data()), "mppi_get_control_seq");
    const double f = u[0], s = std::sin(x[2]), c = std::cos(x[2]);
    const double mc = 1.0, mp = 1.0, l = 1.0, g = 9.81;
    const double xdd = (f + mp * s * (l * x[3] * x[3] + g * c)) / (mc + mp * s * s);
    const double tdd = (-f * c - mp * l * x[3] * x[3] * c * s - (mc + mp) * g * s) / (l * (mc + mp * s * s));
    x[0] += 0.02 * x[1];
    x[1] += 0.02 * xdd;
    x[2] += 0.02 * x[3];
    x[3] += 0.02 * tdd;
    check(mppi_slide_control_sequence(h, 1), "mppi_slide_control_sequence");
    if (1.0 + std::cos(x[2]) < 0.05) ++upright;
  }
  check(mppi_destroy(h), "mppi_destroy");
  std::printf("final state x=%.3f xdot=%.3f theta=%.3f thetadot=%.3f; upright for %d of 500 steps\n", x[0], x[1],
              x[2], x[3], upright);
  return upright > 100 ? 0 : 1;
}
