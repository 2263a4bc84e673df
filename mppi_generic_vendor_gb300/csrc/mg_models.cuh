// mg_models.cuh — Dynamics + Cost plugins compiled into the engine.
//
// Each model type mirrors the reference's plugin contract: compile-time STATE_DIM / CONTROL_DIM / OUTPUT_DIM
// (dynamics.cuh:75-77), computeDynamics(x, u, xdot) (dynamics.cuh:369), Euler step (dynamics.cu:128-152),
// computeStateCost(y, t) + computeControlCost(u, t) (cost.cuh:146, 205) and terminalCost(y) (cost.cuh:161).  The
// functions are __host__ __device__ so the host side reuses them for the nominal state trajectory
// (Controller::computeOutputTrajectoryHelper, controller.cuh:664-684), as the reference's plugins carry host twins.
//
// Control constraints are the generic per-control clamp + deadband of Dynamics::enforceConstraints and depend only on
// the control, so the engine applies them once when the samples are written (the reference applies them inside the
// rollout and writes the constrained control back, mppi_common.cu:117-124; both leave the same values in the sample
// buffer and feed the same controls to the dynamics).
#pragma once

#include "../../include/mppi_gb.h"
#include "mg_math.cuh"

namespace mg
{
// Read-only view of a row-major costmap; cell (0, 0) is centred at origin + resolution / 2.
struct CostmapView
{
  const float* data;
  int width, height;
  float inv_resolution;  // 1 / resolution: the surrogate rollout's lookup multiplies by it; the exact one divides
  float resolution, origin_x, origin_y;
};

// Bilinear lookup with clamp-to-edge addressing, in the order of the reference's CPU texture twin
// (TwoDTextureHelper::queryTextureCPU, two_d_texture_helper.cu:151-235).  The reference's GPU path uses the texture
// unit (tex2D, two_d_texture_helper.cu:66-72), whose interpolation weights are 9-bit fixed point; the engine
// interpolates in FP32 on both sides.
struct Texels
{
  float q00, q01, q10, q11, fx, fy;
};

// The texels and fractions around cell coordinates (px, py) (clamped to the map).
MG_HD Texels costmap_gather_cell(const CostmapView& m, float px, float py)
{
  px = fminf(fmaxf(px, 0.0f), (float)(m.width - 1));
  py = fminf(fmaxf(py, 0.0f), (float)(m.height - 1));
  int x0 = (int)floorf(px);
  int y0 = (int)floorf(py);
  x0 = x0 < m.width - 2 ? x0 : m.width - 2;
  y0 = y0 < m.height - 2 ? y0 : m.height - 2;
  Texels t;
  const f32x2 fr = sub2({ px, py }, { (float)x0, (float)y0 });
  t.fx = fr.x;
  t.fy = fr.y;
  const float* row0 = m.data + (size_t)y0 * m.width;
  const float* row1 = row0 + m.width;
#if defined(__CUDA_ARCH__)
  t.q00 = __ldg(row0 + x0);
  t.q01 = __ldg(row0 + x0 + 1);
  t.q10 = __ldg(row1 + x0);
  t.q11 = __ldg(row1 + x0 + 1);
#else
  t.q00 = row0[x0];
  t.q01 = row0[x0 + 1];
  t.q10 = row1[x0];
  t.q11 = row1[x0 + 1];
#endif
  return t;
}

// The four texels and the interpolation fractions of point (x, y); split from the blend so a rollout can issue the
// loads well before it needs the value.
template <class Ar = ExactArith>
MG_HD Texels costmap_gather(const CostmapView& m, float x, float y, Ar&& ar = Ar{})
{
  // (x, y) as a pair: offsets, the divisions by the cell size and the half-cell shift
  const f32x2 pp = sub2(ar.div2(sub2({ x, y }, { m.origin_x, m.origin_y }), { m.resolution, m.resolution }),
                        { 0.5f, 0.5f });
  return costmap_gather_cell(m, pp.x, pp.y);
}

// top = q00 (1 - fx) + q01 fx and bot = q10 (1 - fx) + q11 fx, then top (1 - fy) + bot fy: the products in pairs, every
// sum scalar (a paired add of paired products is fused into a paired FMA by the code generator, which would change
// the rounding)
MG_HD float costmap_blend(const Texels& t)
{
  const float gx = 1.0f - t.fx;
  const f32x2 p = mul2({ t.q00, t.q10 }, { gx, gx });
  const f32x2 r = mul2({ t.q01, t.q11 }, { t.fx, t.fx });
  const f32x2 w = mul2({ p.x + r.x, p.y + r.y }, { 1.0f - t.fy, t.fy });
  return w.x + w.y;
}

template <class Ar = ExactArith>
MG_HD float costmap_bilinear(const CostmapView& m, float x, float y, Ar&& ar = Ar{})
{
  return costmap_blend(costmap_gather(m, x, y, ar));
}

// Shared (per-launch) data that some costs need besides their parameter block.
struct ModelAux
{
  CostmapView map;
};

// --------------------------------------------------------------------------------------------------------- cartpole
// CartpoleDynamics (cartpole_dynamics.cu:87-105) with the swing-up running cost
// x_coeff*x^2 + x_dot_coeff*xdot^2 + cos_coeff*(1 + cos theta)^2 + theta_dot_coeff*thetadot^2.
struct CartpoleModel
{
  static constexpr int STATE_DIM = 4, CONTROL_DIM = 1, OUTPUT_DIM = 4;
  static constexpr int kModelId = MPPI_MODEL_CARTPOLE;
  static constexpr bool kNeedsCostmap = false;
  static constexpr bool kMlp = false;
  static constexpr bool kPlugin = false;
  static constexpr bool kOwnConstraints = false;  // the engine's deadband + clamp, applied when sampling
  static constexpr int kFlopsPerStep = 60;  // counted from the source below (sin/cos polynomial included)
  using DynParams = mppi_cartpole_params;
  using CostParams = mppi_cartpole_cost_params;

  template <class Ar = ExactArith>
  static MG_HD void computeDynamics(const DynParams& p, const float* x, const float* u, float* xd, Ar&& ar = Ar{})
  {
    const float th = ar.wrap(x[2]);
    float s, c;
    sincos_f(th, &s, &c);
    const float td = x[3], f = u[0];
    const float mc = p.cart_mass, mp = p.pole_mass, lp = p.pole_length, g = p.gravity;
    const float den = mc + mp * (s * s);
    // the two accelerations' divisions as one pair
    const float num1 = f + mp * s * (lp * (td * td) + g * c);
    const float num3 = -f * c - mp * lp * (td * td) * c * s - (mc + mp) * g * s;
    const f32x2 acc = ar.div2({ num1, num3 }, { den, lp * den });
    xd[0] = x[1];
    xd[1] = acc.x;
    xd[2] = td;
    xd[3] = acc.y;
  }
  // Host Jacobians of xdot (CartpoleDynamics::computeGrad, cartpole_dynamics.cu:10-45): A = d xdot / dx (row-major
  // 4 x 4), B = d xdot / du (4 x 1), differentiated from the two accelerations above in double.
  static bool computeGrad(const DynParams& p, const float* x, const float* u, double* A, double* B)
  {
    const double th = x[2], td = x[3], f = u[0];
    const double mc = p.cart_mass, mp = p.pole_mass, lp = p.pole_length, g = p.gravity;
    const double s = std::sin(th), c = std::cos(th);
    const double den = mc + mp * s * s, dden = 2.0 * mp * s * c;  // d den / d theta
    const double n1 = f + mp * s * (lp * td * td + g * c);
    const double n3 = -f * c - mp * lp * td * td * c * s - (mc + mp) * g * s;
    const double dn1 = mp * c * (lp * td * td + g * c) - mp * g * s * s;
    const double dn3 = f * s - mp * lp * td * td * (c * c - s * s) - (mc + mp) * g * c;
    A[0 * 4 + 1] = 1.0;
    A[1 * 4 + 2] = dn1 / den - n1 * dden / (den * den);
    A[1 * 4 + 3] = 2.0 * mp * lp * td * s / den;
    A[2 * 4 + 3] = 1.0;
    A[3 * 4 + 2] = dn3 / (lp * den) - n3 * dden / (lp * den * den);
    A[3 * 4 + 3] = -2.0 * mp * td * c * s / den;
    B[1] = 1.0 / den;
    B[3] = -c / (lp * den);
    return true;
  }
  template <class Ar = ExactArith>
  static MG_HD float computeStateCost(const CostParams& q, const ModelAux&, const float* y, int, Ar&& ar = Ar{})
  {
    const float th = ar.wrap(y[2]);
    float s, c;
    sincos_f(th, &s, &c);
    const float a = 1.0f + c;
    // x_coeff x^2 + x_dot_coeff xdot^2 + cos_coeff (1 + cos)^2 + theta_dot_coeff thetadot^2, added left to right; the
    // squares and coefficient products in pairs
    const f32x2 s01 = { y[0], y[1] }, s23 = { a, y[3] };
    const f32x2 t01 = mul2({ q.x_coeff, q.x_dot_coeff }, mul2(s01, s01));
    const f32x2 t23 = mul2({ q.cos_coeff, q.theta_dot_coeff }, mul2(s23, s23));
    return t01.x + t01.y + t23.x + t23.y;
  }
  static MG_HD float computeControlCost(const CostParams&, const float*, int) { return 0.0f; }
  template <class Ar = ExactArith>
  static MG_HD float terminalCost(const CostParams& q, const ModelAux& aux, const float* y, Ar&& ar = Ar{})
  {
    return computeStateCost(q, aux, y, 0, ar) * q.terminal_coeff;
  }
};

// -------------------------------------------------------------------------------------------- double integrator
// DoubleIntegratorDynamics (di_dynamics.cu:46-53); cost = QuadraticCostImpl-style weighted squared error to the goal
// (quadratic_cost.cu:35-48) + obstacle_cost if strictly inside any circle (composed like
// DoubleIntegratorCircleCost, double_integrator_circle_cost.cu:8-32).
struct DoubleIntegratorModel
{
  static constexpr int STATE_DIM = 4, CONTROL_DIM = 2, OUTPUT_DIM = 4;
  static constexpr int kModelId = MPPI_MODEL_DOUBLE_INTEGRATOR;
  static constexpr bool kNeedsCostmap = false;
  static constexpr bool kMlp = false;
  static constexpr bool kPlugin = false;
  static constexpr bool kOwnConstraints = false;  // the engine's deadband + clamp, applied when sampling
  static constexpr int kFlopsPerStep = 8 + 11 + 8 * 6;
  using DynParams = mppi_double_integrator_params;
  using CostParams = mppi_di_obstacle_cost_params;

  template <class Ar = ExactArith>
  static MG_HD void computeDynamics(const DynParams&, const float* x, const float* u, float* xd, Ar&& = Ar{})
  {
    xd[0] = x[2];
    xd[1] = x[3];
    xd[2] = u[0];
    xd[3] = u[1];
  }
  // Host Jacobians (DoubleIntegratorDynamics::computeGrad, di_dynamics.cu:24-34): A = d xdot / dx (row-major 4 x 4),
  // B = d xdot / du (4 x 2).
  static bool computeGrad(const DynParams&, const float*, const float*, double* A, double* B)
  {
    A[0 * 4 + 2] = 1.0;
    A[1 * 4 + 3] = 1.0;
    B[2 * 2 + 0] = 1.0;
    B[3 * 2 + 1] = 1.0;
    return true;
  }
  // coeff_0 d_0^2 + coeff_1 d_1^2 + coeff_2 d_2^2 + coeff_3 d_3^2 added left to right, d = y - goal; the
  // subtractions and products in (position, velocity) pairs
  static MG_HD float quad(const CostParams& q, const float* y)
  {
    const f32x2 d01 = sub2({ y[0], y[1] }, { q.goal[0], q.goal[1] });
    const f32x2 d23 = sub2({ y[2], y[3] }, { q.goal[2], q.goal[3] });
    const f32x2 t01 = mul2({ q.coeff[0], q.coeff[1] }, mul2(d01, d01));
    const f32x2 t23 = mul2({ q.coeff[2], q.coeff[3] }, mul2(d23, d23));
    return t01.x + t01.y + t23.x + t23.y;
  }
  template <class Ar = ExactArith>
  static MG_HD float computeStateCost(const CostParams& q, const ModelAux&, const float* y, int, Ar&& = Ar{})
  {
    float cost = quad(q, y);
    bool inside = false;
    // fixed trip count with a guard, so the obstacle table can live in registers for a whole rollout; the offsets
    // and squares of (x, y) as pairs, their sum ox^2 + oy^2 scalar
#pragma unroll
    for (int j = 0; j < MPPI_MAX_OBSTACLES; ++j)
    {
      const f32x2 o = sub2({ y[0], y[1] }, { q.obstacle_x[j], q.obstacle_y[j] });
      const f32x2 o2 = mul2(o, o);
      const float r = q.obstacle_radius[j];
      inside = inside || (j < q.num_obstacles && o2.x + o2.y < r * r);
    }
    if (inside) cost = cost + q.obstacle_cost;
    return cost;
  }
  static MG_HD float computeControlCost(const CostParams&, const float*, int) { return 0.0f; }
  template <class Ar = ExactArith>
  static MG_HD float terminalCost(const CostParams& q, const ModelAux&, const float* y, Ar&& = Ar{})
  {
    return quad(q, y) * q.terminal_coeff;
  }
};

// --------------------------------------------------------------------------------------------- kinematic bicycle
// State (x, y, yaw, v), control (accel, steer).  xdot = v cos yaw, ydot = v sin yaw, yawdot = v tan(steer) / L,
// vdot = accel (closest reference model: DubinsDynamics, dubins.cu:60-65).  Cost: costmap + speed tracking + steer
// effort.
struct BicycleCostmapModel
{
  static constexpr int STATE_DIM = 4, CONTROL_DIM = 2, OUTPUT_DIM = 4;
  static constexpr int kModelId = MPPI_MODEL_BICYCLE_COSTMAP;
  static constexpr bool kNeedsCostmap = true;
  static constexpr bool kMlp = false;
  static constexpr bool kPlugin = false;
  static constexpr bool kOwnConstraints = false;  // the engine's deadband + clamp, applied when sampling
  static constexpr int kFlopsPerStep = 2 * 22 + 12 + 25;
  using DynParams = mppi_bicycle_params;
  using CostParams = mppi_costmap_cost_params;

  template <class Ar = ExactArith>
  static MG_HD void computeDynamics(const DynParams& p, const float* x, const float* u, float* xd, Ar&& ar = Ar{})
  {
    float sy, cy, sd, cd;
    sincos_f(x[2], &sy, &cy);
    sincos_f(u[1], &sd, &cd);
    const f32x2 vxy = mul2({ x[3], x[3] }, { cy, sy });
    xd[0] = vxy.x;
    xd[1] = vxy.y;
    xd[2] = ar.div(x[3] * ar.div(sd, cd), p.wheelbase);
    xd[3] = u[0];
  }
  // Host Jacobians of the kinematic bicycle in double: A = d xdot / dx (row-major 4 x 4), B = d xdot / du (4 x 2).
  static bool computeGrad(const DynParams& p, const float* x, const float* u, double* A, double* B)
  {
    const double yaw = x[2], v = x[3], steer = u[1], L = p.wheelbase;
    const double sy = std::sin(yaw), cy = std::cos(yaw), cd = std::cos(steer);
    A[0 * 4 + 2] = -v * sy;
    A[0 * 4 + 3] = cy;
    A[1 * 4 + 2] = v * cy;
    A[1 * 4 + 3] = sy;
    A[2 * 4 + 3] = std::tan(steer) / L;
    B[2 * 2 + 1] = v / (L * cd * cd);
    B[3 * 2 + 0] = 1.0;
    return true;
  }
  template <class Ar = ExactArith>
  static MG_HD float speedMapCost(const CostParams& q, const ModelAux& aux, const float* y, Ar&& ar = Ar{})
  {
    const float dv = y[3] - q.speed_target;
    return q.map_coeff * costmap_bilinear(aux.map, y[0], y[1], ar) + q.speed_coeff * (dv * dv);
  }
  template <class Ar = ExactArith>
  static MG_HD float computeStateCost(const CostParams& q, const ModelAux& aux, const float* y, int, Ar&& ar = Ar{})
  {
    return speedMapCost(q, aux, y, ar);
  }
  static MG_HD float computeControlCost(const CostParams& q, const float* u, int) { return q.steer_coeff * (u[1] * u[1]); }
  template <class Ar = ExactArith>
  static MG_HD float terminalCost(const CostParams& q, const ModelAux& aux, const float* y, Ar&& ar = Ar{})
  {
    return speedMapCost(q, aux, y, ar) * q.terminal_coeff;
  }
};

// ------------------------------------------------------------------------------------------ dynamic bicycle (slip)
// State (x, y, yaw, vx, vy, yaw_rate, steer), control (throttle, steer_cmd); linear tyres with one cornering stiffness,
// first-order steering actuator.  Kinematic rows follow NeuralNetModel::computeKinematics (ar_nn_model.cu:119-124).
struct BicycleSlipModel
{
  static constexpr int STATE_DIM = 7, CONTROL_DIM = 2, OUTPUT_DIM = 7;
  static constexpr int kModelId = MPPI_MODEL_BICYCLE_SLIP;
  static constexpr bool kNeedsCostmap = true;
  static constexpr bool kMlp = false;
  static constexpr bool kPlugin = false;
  static constexpr bool kOwnConstraints = false;  // the engine's deadband + clamp, applied when sampling
  static constexpr int kFlopsPerStep = 3 * 22 + 45 + 25;
  using DynParams = mppi_bicycle_slip_params;
  using CostParams = mppi_costmap_cost_params;

  static MG_HD void computeKinematics(const float* x, float* xd)
  {
    float sy, cy;
    sincos_f(x[2], &sy, &cy);
    xd[0] = x[3] * cy - x[4] * sy;
    xd[1] = x[3] * sy + x[4] * cy;
    xd[2] = x[5];
  }
  template <class Ar = ExactArith>
  static MG_HD void computeDynamics(const DynParams& p, const float* x, const float* u, float* xd, Ar&& ar = Ar{})
  {
    float sy, cy;
    sincos_f(x[2], &sy, &cy);
    const float vx = x[3], vy = x[4], r = x[5], d = x[6];
    const float vxs = fmaxf(vx, p.min_vx);
    // scalar on purpose: paired forms of this model's arithmetic raise the fused rollout's register count by a third
    // (fewer resident CTAs), which costs more than the saved instructions
    const float alpha_f = d - ar.div(vy + p.lf * r, vxs);
    const float alpha_r = ar.div(-(vy - p.lr * r), vxs);
    const float fyf = p.cornering_stiffness * alpha_f;
    const float fyr = p.cornering_stiffness * alpha_r;
    float sd, cd;
    sincos_f(d, &sd, &cd);
    const float fx = p.max_drive_force * u[0] - p.drag * vx;
    xd[0] = vx * cy - vy * sy;
    xd[1] = vx * sy + vy * cy;
    xd[2] = r;
    xd[3] = ar.div(fx - fyf * sd, p.mass) + vy * r;
    xd[4] = ar.div(fyr + fyf * cd, p.mass) - vx * r;
    xd[5] = ar.div(p.lf * fyf * cd - p.lr * fyr, p.yaw_inertia);
    xd[6] = ar.div(u[1] * p.max_steer - d, p.steer_time_constant);
  }
  template <class Ar = ExactArith>
  static MG_HD float speedMapCost(const CostParams& q, const ModelAux& aux, const float* y, Ar&& ar = Ar{})
  {
    return stateCostFromTexels(q, costmap_gather(aux.map, y[0], y[1], ar), y);
  }
  // The state cost from texels gathered earlier (costmap_gather at y[0], y[1]): the same arithmetic as speedMapCost.
  static MG_HD float stateCostFromTexels(const CostParams& q, const Texels& tx, const float* y)
  {
    const float dv = y[3] - q.speed_target;
    return q.map_coeff * costmap_blend(tx) + q.speed_coeff * (dv * dv);
  }
  template <class Ar = ExactArith>
  static MG_HD float computeStateCost(const CostParams& q, const ModelAux& aux, const float* y, int, Ar&& ar = Ar{})
  {
    return speedMapCost(q, aux, y, ar);
  }
  static MG_HD float computeControlCost(const CostParams& q, const float* u, int) { return q.steer_coeff * (u[1] * u[1]); }
  template <class Ar = ExactArith>
  static MG_HD float terminalCost(const CostParams& q, const ModelAux& aux, const float* y, Ar&& ar = Ar{})
  {
    return speedMapCost(q, aux, y, ar) * q.terminal_coeff;
  }
};

// Learned-surrogate variant of the dynamic bicycle: same state, controls, parameters and cost; the (yaw, vx, vy,
// yaw_rate, steer) derivatives come from the MLP (evaluated on the tensor cores by the engine's MLP rollout kernel).
struct BicycleSlipMLPModel : BicycleSlipModel
{
  static constexpr int kModelId = MPPI_MODEL_BICYCLE_SLIP_MLP;
  static constexpr bool kMlp = true;
};

// Euler step shared by every model (Dynamics::step -> updateState, dynamics.cu:128-152): x' = x + xdot * dt as one
// fused multiply-add (the form the reference's device code compiles to).
template <class Model, class Ar = ExactArith>
MG_HD void euler_step(const typename Model::DynParams& p, const float* x, const float* u, float* x_next, float dt,
                      Ar&& ar = Ar{})
{
  float xd[Model::STATE_DIM];
  Model::computeDynamics(p, x, u, xd, ar);
  // two states per paired FMA
#pragma unroll
  for (int i = 0; i + 1 < Model::STATE_DIM; i += 2)
  {
    const f32x2 n = fma2({ xd[i], xd[i + 1] }, { dt, dt }, { x[i], x[i + 1] });
    x_next[i] = n.x;
    x_next[i + 1] = n.y;
  }
  if constexpr (Model::STATE_DIM % 2 == 1)
    x_next[Model::STATE_DIM - 1] = fmaf(xd[Model::STATE_DIM - 1], dt, x[Model::STATE_DIM - 1]);
}

}  // namespace mg
