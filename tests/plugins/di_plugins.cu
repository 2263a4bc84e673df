// Three Dynamics / Cost plugin pairs written against include/mppi_gb_plugin.cuh, outside the engine's sources, the
// way a user of the library would write them: the double integrator (DoubleIntegratorDynamics, di_dynamics.cu:46-53)
// with an optional linear damping, once with the default Euler step and its analytic Jacobians (computeGrad, for the
// DDP feedback controller), once with its own step override (semi-implicit: velocity first, then position with the
// new velocity; no computeGrad, so the feedback controller differentiates numerically) and once with its own
// enforceConstraints; and
// QuadraticCostImpl's state cost (quadratic_cost.cu:35-48) with a crash wall that uses the crash argument of
// computeRunningCost: once x > wall_x the sample's crash flag stays set and every later step pays crash_cost.
#include "mppi_gb_plugin.cuh"

struct DIPlugin : mppi_gb::Dynamics<DIPlugin, 4, 2>
{
  float damping;
  MPPI_GB_HD void computeDynamics(const float* x, const float* u, float* xd) const
  {
    xd[0] = x[2];
    xd[1] = x[3];
    xd[2] = u[0] - damping * x[2];
    xd[3] = u[1] - damping * x[3];
  }
  // host Jacobians for the DDP feedback controller (Dynamics::computeGrad, dynamics.cuh:236-242)
  bool computeGrad(const float*, const float*, float* A, float* B) const
  {
    A[0 * 4 + 2] = 1.0f;
    A[1 * 4 + 3] = 1.0f;
    A[2 * 4 + 2] = -damping;
    A[3 * 4 + 3] = -damping;
    B[2 * 2 + 0] = 1.0f;
    B[3 * 2 + 1] = 1.0f;
    return true;
  }
};

struct DISymplecticPlugin : mppi_gb::Dynamics<DISymplecticPlugin, 4, 2>
{
  float damping;
  MPPI_GB_HD void computeDynamics(const float* x, const float* u, float* xd) const
  {
    xd[0] = x[2];
    xd[1] = x[3];
    xd[2] = u[0] - damping * x[2];
    xd[3] = u[1] - damping * x[3];
  }
  MPPI_GB_HD void step(const float* x, float* xn, float* xd, const float* u, float* y, int t, float dt) const
  {
    computeStateDeriv(x, u, xd);
    xn[2] = fmaf(xd[2], dt, x[2]);
    xn[3] = fmaf(xd[3], dt, x[3]);
    xn[0] = fmaf(xn[2], dt, x[0]);
    xn[1] = fmaf(xn[3], dt, x[1]);
    stateToOutput(xn, y);
  }
};

// Its own enforceConstraints (Dynamics::enforceConstraints, dynamics.cu:107-126, overridden): an acceleration limit
// that shrinks with speed, |u_i| <= max(0.5, a_max - speed_gain * |v_i|), in place of the handle's control ranges.
struct DIConstrainedPlugin : mppi_gb::Dynamics<DIConstrainedPlugin, 4, 2>
{
  float damping;
  float a_max;
  float speed_gain;
  MPPI_GB_HD void computeDynamics(const float* x, const float* u, float* xd) const
  {
    xd[0] = x[2];
    xd[1] = x[3];
    xd[2] = u[0] - damping * x[2];
    xd[3] = u[1] - damping * x[3];
  }
  MPPI_GB_HD void enforceConstraints(float* x, float* u) const
  {
#pragma unroll
    for (int i = 0; i < 2; ++i)
    {
      const float amax = fmaxf(0.5f, a_max - speed_gain * fabsf(x[2 + i]));
      u[i] = fminf(fmaxf(u[i], -amax), amax);
    }
  }
};

struct QuadraticWallCost : mppi_gb::Cost<QuadraticWallCost, 4, 2>
{
  float s_goal[4];
  float s_coeffs[4];
  float wall_x;
  float crash_cost;
  float terminal_coeff;
  MPPI_GB_HD float quad(const float* y) const
  {
    float cost = 0.0f;
#pragma unroll
    for (int i = 0; i < 4; ++i)
    {
      const float e = y[i] - s_goal[i];
      cost += e * e * s_coeffs[i];
    }
    return cost;
  }
  MPPI_GB_HD float computeStateCost(const float* y, int t, int* crash) const
  {
    float cost = quad(y);
    if (y[0] > wall_x) *crash = 1;
    if (*crash) cost += crash_cost;
    return cost;
  }
  MPPI_GB_HD float terminalCost(const float* y) const { return quad(y) * terminal_coeff; }
};

MPPI_GB_PLUGIN(di_quadratic, DIPlugin, QuadraticWallCost)
MPPI_GB_PLUGIN(di_symplectic_quadratic, DISymplecticPlugin, QuadraticWallCost)
MPPI_GB_PLUGIN(di_constrained_quadratic, DIConstrainedPlugin, QuadraticWallCost)
