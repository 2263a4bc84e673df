// mppi_oracle.cpp — CPU oracle for the GB300 MPPI engine.
//
// TEST INFRASTRUCTURE ONLY.  This file restates MPPI-Generic's plain MPPI path on the CPU so that tests, the smoke
// check and the CPU baseline of the benchmark can check the CUDA engine against it.  Nothing in the engine links,
// imports or calls this code.
//
// Every function cites the reference source it follows (paths relative to the MPPI-Generic tree).  Floating-point
// arithmetic follows the reference's expression order; the build uses -ffp-contract=off and writes fused
// multiply-adds explicitly where the reference's device code contracts them (Euler update, mean + sigma*eps), so the
// float instantiation is bit-identical to the engine's rollout whenever both sides see the same inputs.  The double
// instantiation (libm trig, FP64 throughout) is the accuracy judge ("FP64 host rollout").
//
// Parity pins: the known answers of the reference's own tests (smoothing 61/35 and slide, controller_generic_tests.cu
// :214-282; cartpole equilibrium, cartpole_dynamics_tests.cu:24-45; min / normaliser, normexp_kernel_tests.cu:45-256;
// weighted reduction, weightedreduction_kernel_tests.cu:276-389), the Philox4x32-10 known-answer vectors of its
// published definition, and the reference's NumPy colored-noise script (scripts/colored_noise.py) run with injected
// normals.  The reference library itself cannot be compiled here (Eigen, cnpy, gtest are absent).

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <type_traits>
#include <vector>

#include "../include/mppi_gb.h"

namespace orc
{
// ------------------------------------------------------------------------------------------------ own trigonometry
// Cody–Waite reduction by pi/2 with a three-part constant, then Taylor polynomials of sin and cos on [-pi/4, pi/4]
// (coefficients are +-1/n! rounded to float).  The engine evaluates the same published method with the same
// operations; the reference's device code uses the __sinf/__cosf intrinsics (cartpole_dynamics.cu:90-91).
static const float kTwoOverPi = 0x1.45f306p-1f;
static const float kPio2A = 0x1.921fb6p+0f;
static const float kPio2B = -0x1.777a5cp-25f;
static const float kPio2C = -0x1.ee59dap-50f;

static inline void sincos_f(float x, float* s_out, float* c_out)
{
  const float q = rintf(x * kTwoOverPi);
  float r = fmaf(-q, kPio2A, x);
  r = fmaf(-q, kPio2B, r);
  r = fmaf(-q, kPio2C, r);
  const float r2 = r * r;
  float ps = fmaf(0x1.71de3ap-19f, r2, -0x1.a01a02p-13f);
  ps = fmaf(ps, r2, 0x1.111112p-7f);
  ps = fmaf(ps, r2, -0x1.555556p-3f);
  const float sr = fmaf(ps, r2 * r, r);
  float pc = fmaf(-0x1.27e4fcp-22f, r2, 0x1.a01a02p-16f);
  pc = fmaf(pc, r2, -0x1.6c16c2p-10f);
  pc = fmaf(pc, r2, 0x1.555556p-5f);
  pc = fmaf(pc, r2, -0.5f);
  const float cr = fmaf(pc, r2, 1.0f);
  const int n = ((int)q) & 3;
  float s, c;
  switch (n)
  {
    case 0: s = sr; c = cr; break;
    case 1: s = cr; c = -sr; break;
    case 2: s = -sr; c = -cr; break;
    default: s = -cr; c = sr; break;
  }
  *s_out = s;
  *c_out = c;
}

// Trigonometry of the float instantiation: 0 = the engine's sincos_f above (the default; bit-identical to the
// engine), 1 = libm sinf / cosf, the functions the reference's host twins call (CartpoleDynamics::computeDynamics,
// cartpole_dynamics.cu:48-53), to measure what the choice of sine / cosine moves.
static std::atomic<int> g_trig_mode{ 0 };

template <class R>
struct M;
template <>
struct M<float>
{
  static inline void sincos(float x, float* s, float* c)
  {
    if (g_trig_mode.load(std::memory_order_relaxed) == 1)
    {
      *s = sinf(x);
      *c = cosf(x);
      return;
    }
    sincos_f(x, s, c);
  }
  static inline float fma(float a, float b, float c) { return fmaf(a, b, c); }
  static inline float sqrt(float a) { return sqrtf(a); }
  static inline float fabs(float a) { return fabsf(a); }
  static inline float fmin(float a, float b) { return fminf(a, b); }
  static inline float fmax(float a, float b) { return fmaxf(a, b); }
  static inline float floor(float a) { return floorf(a); }
  // angle_utils::normalizeAngle(float) (include/mppi/utils/angle_utils.cuh:23-29)
  static inline float normalize_angle(float a)
  {
    const float r = fmodf(a + (float)M_PI, (float)(2.0 * M_PI));
    if (r <= 0.0f) return r + (float)M_PI;
    return r - (float)M_PI;
  }
};
template <>
struct M<double>
{
  static inline void sincos(double x, double* s, double* c) { *s = std::sin(x); *c = std::cos(x); }
  static inline double fma(double a, double b, double c) { return std::fma(a, b, c); }
  static inline double sqrt(double a) { return std::sqrt(a); }
  static inline double fabs(double a) { return std::fabs(a); }
  static inline double fmin(double a, double b) { return std::fmin(a, b); }
  static inline double fmax(double a, double b) { return std::fmax(a, b); }
  static inline double floor(double a) { return std::floor(a); }
  // angle_utils::normalizeAngle(double) (angle_utils.cuh:16-21)
  static inline double normalize_angle(double a)
  {
    const double r = std::fmod(a + M_PI, 2.0 * M_PI);
    if (r <= 0.0) return r + M_PI;
    return r - M_PI;
  }
};

// ------------------------------------------------------------------------------------------------ Philox4x32-10
// Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3" (SC 2011): ten rounds of
// (hi,lo) = mulhilo(M, c) with the Weyl key schedule.
static inline void philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4])
{
  uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
  uint32_t k0 = key_in[0], k1 = key_in[1];
  for (int r = 0; r < 10; ++r)
  {
    if (r > 0)
    {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    const uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    const uint32_t n0 = hi1 ^ c1 ^ k0;
    const uint32_t n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
  }
  out[0] = c0;
  out[1] = c1;
  out[2] = c2;
  out[3] = c3;
}

// ------------------------------------------------------------------------------------------------ plugins
// Each model: STATE_DIM S, CONTROL_DIM C, dynamics derivative, running (state + control) cost and terminal cost with
// the reference's Dynamics / Cost method meanings (dynamics.cuh:369-407, cost.cuh:146-222).
struct CostmapView
{
  const float* data = nullptr;
  int width = 0, height = 0;
  float resolution = 1.0f, origin_x = 0.0f, origin_y = 0.0f;
};

// Bilinear lookup, clamp-to-edge, cell-centred samples: the CPU twin of the reference's texture query
// (TwoDTextureHelper::queryTextureCPU, two_d_texture_helper.cu:151-235) in map coordinates.
template <class R>
static inline R costmap_bilinear(const CostmapView& m, R x, R y)
{
  R px = (x - (R)m.origin_x) / (R)m.resolution - (R)0.5;
  R py = (y - (R)m.origin_y) / (R)m.resolution - (R)0.5;
  px = M<R>::fmin(M<R>::fmax(px, (R)0), (R)(m.width - 1));
  py = M<R>::fmin(M<R>::fmax(py, (R)0), (R)(m.height - 1));
  int x0 = std::min((int)M<R>::floor(px), m.width - 2);
  int y0 = std::min((int)M<R>::floor(py), m.height - 2);
  const R fx = px - (R)x0;
  const R fy = py - (R)y0;
  const float* row0 = m.data + (size_t)y0 * m.width;
  const float* row1 = row0 + m.width;
  const R top = (R)row0[x0] * ((R)1 - fx) + (R)row0[x0 + 1] * fx;
  const R bot = (R)row1[x0] * ((R)1 - fx) + (R)row1[x0 + 1] * fx;
  return top * ((R)1 - fy) + bot * fy;
}

template <class R>
static inline bool libm_float()
{
  return std::is_same<R, float>::value && g_trig_mode.load(std::memory_order_relaxed) == 1;
}

template <class R>
struct Cartpole
{
  static const int S = 4, C = 1;
  const mppi_cartpole_params& p;
  const mppi_cartpole_cost_params& q;
  // CartpoleDynamics::computeDynamics, device version (cartpole_dynamics.cu:87-105); with libm trigonometry the host
  // twin (cartpole_dynamics.cu:48-67), which takes sinf / cosf of the unwrapped angle
  void deriv(const R* x, const R* u, R* xd) const
  {
    const R th = libm_float<R>() ? x[2] : M<R>::normalize_angle(x[2]);
    R s, c;
    M<R>::sincos(th, &s, &c);
    const R td = x[3], f = u[0];
    const R mc = p.cart_mass, mp = p.pole_mass, lp = p.pole_length, g = p.gravity;
    xd[0] = x[1];
    xd[1] = (f + mp * s * (lp * (td * td) + g * c)) / (mc + mp * (s * s));
    xd[2] = td;
    xd[3] = (-f * c - mp * lp * (td * td) * c * s - (mc + mp) * g * s) / (lp * (mc + mp * (s * s)));
  }
  R state_cost(const R* y, int) const
  {
    const R th = M<R>::normalize_angle(y[2]);
    R s, c;
    M<R>::sincos(th, &s, &c);
    const R a = (R)1 + c;
    return (R)q.x_coeff * (y[0] * y[0]) + (R)q.x_dot_coeff * (y[1] * y[1]) + (R)q.cos_coeff * (a * a) +
           (R)q.theta_dot_coeff * (y[3] * y[3]);
  }
  R control_cost(const R*, int) const { return (R)0; }
  R terminal_cost(const R* y) const { return state_cost(y, 0) * (R)q.terminal_coeff; }
};

template <class R>
struct DoubleIntegrator
{
  static const int S = 4, C = 2;
  const mppi_di_obstacle_cost_params& q;
  // DoubleIntegratorDynamics::computeDynamics (di_dynamics.cu:46-53)
  void deriv(const R* x, const R* u, R* xd) const
  {
    xd[0] = x[2];
    xd[1] = x[3];
    xd[2] = u[0];
    xd[3] = u[1];
  }
  // QuadraticCostImpl (quadratic_cost.cu:35-48) + obstacle indicator (double_integrator_circle_cost.cu:8-32)
  R quad(const R* y) const
  {
    const R d0 = y[0] - (R)q.goal[0], d1 = y[1] - (R)q.goal[1], d2 = y[2] - (R)q.goal[2], d3 = y[3] - (R)q.goal[3];
    return (R)q.coeff[0] * (d0 * d0) + (R)q.coeff[1] * (d1 * d1) + (R)q.coeff[2] * (d2 * d2) +
           (R)q.coeff[3] * (d3 * d3);
  }
  R state_cost(const R* y, int) const
  {
    R cost = quad(y);
    bool inside = false;
    for (int j = 0; j < q.num_obstacles; ++j)
    {
      const R ox = y[0] - (R)q.obstacle_x[j];
      const R oy = y[1] - (R)q.obstacle_y[j];
      const R r = (R)q.obstacle_radius[j];
      inside = inside || (ox * ox + oy * oy < r * r);
    }
    if (inside) cost = cost + (R)q.obstacle_cost;
    return cost;
  }
  R control_cost(const R*, int) const { return (R)0; }
  R terminal_cost(const R* y) const { return quad(y) * (R)q.terminal_coeff; }
};

template <class R>
struct BicycleCostmap
{
  static const int S = 4, C = 2;
  const mppi_bicycle_params& p;
  const mppi_costmap_cost_params& q;
  const CostmapView& map;
  // kinematic bicycle: xdot = v cos(yaw), ydot = v sin(yaw), yawdot = v tan(steer) / L, vdot = accel
  // (closest reference model: DubinsDynamics::computeDynamics, dubins.cu:60-65)
  void deriv(const R* x, const R* u, R* xd) const
  {
    R sy, cy, sd, cd;
    M<R>::sincos(x[2], &sy, &cy);
    M<R>::sincos(u[1], &sd, &cd);
    xd[0] = x[3] * cy;
    xd[1] = x[3] * sy;
    xd[2] = x[3] * (sd / cd) / (R)p.wheelbase;
    xd[3] = u[0];
  }
  R speed(const R* y) const
  {
    const R dv = y[3] - (R)q.speed_target;
    return (R)q.map_coeff * costmap_bilinear<R>(map, y[0], y[1]) + (R)q.speed_coeff * (dv * dv);
  }
  R state_cost(const R* y, int) const { return speed(y); }
  R control_cost(const R* u, int) const { return (R)q.steer_coeff * (u[1] * u[1]); }
  R terminal_cost(const R* y) const { return speed(y) * (R)q.terminal_coeff; }
};

template <class R>
struct BicycleSlip
{
  static const int S = 7, C = 2;
  const mppi_bicycle_slip_params& p;
  const mppi_costmap_cost_params& q;
  const CostmapView& map;
  // 7-state dynamic bicycle with linear tyres; state (x, y, yaw, vx, vy, r, steer), control (throttle, steer_cmd).
  // Kinematic rows follow NeuralNetModel::computeKinematics (ar_nn_model.cu:119-124); the tyre rows are the analytic
  // model the surrogate is trained on.
  void deriv(const R* x, const R* u, R* xd) const
  {
    R sy, cy;
    M<R>::sincos(x[2], &sy, &cy);
    const R vx = x[3], vy = x[4], r = x[5], d = x[6];
    const R vxs = M<R>::fmax(vx, (R)p.min_vx);
    const R af = d - (vy + (R)p.lf * r) / vxs;
    const R ar = -(vy - (R)p.lr * r) / vxs;
    const R fyf = (R)p.cornering_stiffness * af;
    const R fyr = (R)p.cornering_stiffness * ar;
    R sd, cd;
    M<R>::sincos(d, &sd, &cd);
    const R fx = (R)p.max_drive_force * u[0] - (R)p.drag * vx;
    xd[0] = vx * cy - vy * sy;
    xd[1] = vx * sy + vy * cy;
    xd[2] = r;
    xd[3] = (fx - fyf * sd) / (R)p.mass + vy * r;
    xd[4] = (fyr + fyf * cd) / (R)p.mass - vx * r;
    xd[5] = ((R)p.lf * fyf * cd - (R)p.lr * fyr) / (R)p.yaw_inertia;
    xd[6] = (u[1] * (R)p.max_steer - d) / (R)p.steer_time_constant;
  }
  R speed(const R* y) const
  {
    const R dv = y[3] - (R)q.speed_target;
    return (R)q.map_coeff * costmap_bilinear<R>(map, y[0], y[1]) + (R)q.speed_coeff * (dv * dv);
  }
  R state_cost(const R* y, int) const { return speed(y); }
  R control_cost(const R* u, int) const { return (R)q.steer_coeff * (u[1] * u[1]); }
  R terminal_cost(const R* y) const { return speed(y) * (R)q.terminal_coeff; }
};

// ------------------------------------------------------------------------------------------------ sampler
// setGaussianControls (include/mppi/sampling_distributions/gaussian/gaussian.cu:17-277), scalar path: sample 0 and
// t < stride take the mean; samples at or beyond (1 - p) * K are zero-mean; the rest mean + decay*sigma*eps.  The
// reference's device code contracts mean + sigma*eps into one fused multiply-add.
static void gaussian_rewrite(const float* eps, const float* mean, const float* std_dev, int K, int T, int C,
                             int stride, float std_dev_decay_pow, float pure_pct, float* out)
{
  for (int k = 0; k < K; ++k)
    for (int t = 0; t < T; ++t)
      for (int c = 0; c < C; ++c)
      {
        const size_t i = ((size_t)k * T + t) * C + c;
        const float sd = std_dev_decay_pow * std_dev[c];
        float u;
        if (k == 0 || t < stride)
          u = mean[t * C + c];
        else if ((float)k >= (1.0f - pure_pct) * (float)K)
          u = sd * eps[i];
        else
          u = fmaf(sd, eps[i], mean[t * C + c]);
        out[i] = u;
      }
}

// Dynamics::enforceConstraints (dynamics.cu:107-126; host twin dynamics.cuh:247-261)
static inline float enforce_constraint(float u, const mppi_control_constraints& cc, int i)
{
  if (fabsf(u) < cc.deadband[i])
    u = cc.zero_control[i];
  else
    u += cc.deadband[i] * -(u >= 0 ? 1.0f : -1.0f);
  return fminf(fmaxf(cc.lower[i], u), cc.upper[i]);
}

// GaussianDistributionImpl::computeLikelihoodRatioCost (gaussian.cu:490-574)
template <class R>
static inline R likelihood_cost(const R* u, const float* mean_t, const mppi_sampling_params& sp, int C, int k, int K,
                                R lambda, R alpha)
{
  R cost = 0;
  const bool zero_mean = (float)k >= (1.0f - sp.pure_noise_trajectories_percentage) * (float)K;
  for (int i = 0; i < C; ++i)
  {
    const R m = zero_mean ? (R)0 : (R)mean_t[i];
    const R sd = (R)sp.std_dev[i];
    cost += (R)sp.control_cost_coeff[i] * m * (m - (R)2 * u[i]) / (sd * sd);
  }
  return (R)0.5 * lambda * ((R)1 - alpha) * cost;
}

// Models that carry a crash flag through the rollout (the plugin-test pair) step themselves and take the flag in
// their running cost.
template <class M_, class = void>
struct HasCrash : std::false_type
{
};
template <class M_>
struct HasCrash<M_, std::void_t<decltype(M_::kCrash)>> : std::true_type
{
};

// ------------------------------------------------------------------------------------------------ rollout
// Per-sample rollout in the order of rolloutKernel (mppi_common.cu:105-152) and its host twin launchCPURolloutKernel
// (tests/include/kernel_tests/core/rollout_kernel_test.cu:504-541): read u, enforce constraints, write u back, Euler
// step (dynamics.cu:128-152), running cost on the stepped output, terminal cost, divide by T.
template <class R, class Model>
static void rollout_range(const Model& m, const float* x0, float* controls, bool write_back, const float* mean,
                          const mppi_sampling_params& sp, const mppi_control_constraints& cc, float lambda,
                          float alpha, int K, int T, float dt, int k_begin, int k_end, double* costs_out,
                          R* traj_out /* optional [k][T][S] */)
{
  const int S = Model::S, C = Model::C;
  const bool use_likelihood = std::any_of(sp.control_cost_coeff, sp.control_cost_coeff + C,
                                          [](float v) { return v != 0.0f; });
  for (int k = k_begin; k < k_end; ++k)
  {
    R x[MPPI_MAX_STATE_DIM], xn[MPPI_MAX_STATE_DIM], xd[MPPI_MAX_STATE_DIM], u[MPPI_MAX_CONTROL_DIM];
    for (int i = 0; i < S; ++i) x[i] = (R)x0[i];
    R running = 0;
    int crash = 0;  // crash_status (mppi_common.cu:85-86): zero at the start of every rollout
    for (int t = 0; t < T; ++t)
    {
      float* uk = controls + ((size_t)k * T + t) * C;
      bool own = false;
      if constexpr (HasCrash<Model>::value) own = m.lim != nullptr;
      if (own)
      {
        // a plugin's own enforceConstraints, with the state (rolloutKernel, mppi_common.cu:114-123)
        if constexpr (HasCrash<Model>::value)
        {
          for (int i = 0; i < C; ++i) u[i] = (R)uk[i];
          m.constrain(x, u);
          if (write_back)
            for (int i = 0; i < C; ++i) uk[i] = (float)u[i];
        }
      }
      else
      {
        for (int i = 0; i < C; ++i)
        {
          const float uc = enforce_constraint(uk[i], cc, i);
          if (write_back) uk[i] = uc;
          u[i] = (R)uc;
        }
      }
      R step_cost;
      if constexpr (HasCrash<Model>::value)
      {
        // plugin pair: its own step, and computeRunningCost with the sample's crash flag
        m.step(x, u, xn, (R)dt);
        step_cost = m.running_cost(xn, u, t, &crash);
      }
      else
      {
        m.deriv(x, u, xd);
        for (int i = 0; i < S; ++i) xn[i] = M<R>::fma(xd[i], (R)dt, x[i]);
        step_cost = m.state_cost(xn, t) + m.control_cost(u, t);
      }
      if (use_likelihood) step_cost += likelihood_cost<R>(u, mean + (size_t)t * C, sp, C, k, K, (R)lambda, (R)alpha);
      running += step_cost;
      if (traj_out)
        for (int i = 0; i < S; ++i) traj_out[((size_t)k * T + t) * S + i] = xn[i];
      for (int i = 0; i < S; ++i) x[i] = xn[i];
    }
    // computeAndSaveCost (mppi_common.cu:879-889): running / T + terminal / T
    costs_out[k] = (double)(running / (R)T + m.terminal_cost(x) / (R)T);
  }
}

// 9 -> 64 -> 64 -> 5 tanh MLP with a linear output layer (FNNHelper::forward, fnn_helper.cu:353-382; the last layer
// applies no non-linearity, :368-379).  Parameters are one flat vector: W1[64][9], b1[64], W2[64][64], b2[64],
// W3[5][64], b3[5] (row-major, output index first, as FNNHelper's theta_ layout).
constexpr int kIn = 9, kHid = 64, kOut = 5;
constexpr int kW1 = 0, kB1 = kW1 + kHid * kIn, kW2 = kB1 + kHid, kB2 = kW2 + kHid * kHid, kW3 = kB2 + kHid,
              kB3 = kW3 + kOut * kHid, kNumParams = kB3 + kOut;

template <class R>
static void mlp_forward(const R* p, const R* x, R* h1, R* h2, R* y)
{
  for (int j = 0; j < kHid; ++j)
  {
    R z = p[kB1 + j];
    for (int i = 0; i < kIn; ++i) z += p[kW1 + j * kIn + i] * x[i];
    h1[j] = std::tanh(z);
  }
  for (int j = 0; j < kHid; ++j)
  {
    R z = p[kB2 + j];
    for (int i = 0; i < kHid; ++i) z += p[kW2 + j * kHid + i] * h1[i];
    h2[j] = std::tanh(z);
  }
  for (int j = 0; j < kOut; ++j)
  {
    R z = p[kB3 + j];
    for (int i = 0; i < kHid; ++i) z += p[kW3 + j * kHid + i] * h2[i];
    y[j] = z;
  }
}

// Surrogate parameters of the MLP bicycle model (set with orc_set_mlp): the network above followed by the input and
// output normalisation (in_mean[9], in_std[9], out_mean[5], out_std[5]), 5153 floats, kept in both precisions.
constexpr int kInMean = kNumParams, kInStd = kInMean + kIn, kOutMean = kInStd + kIn, kOutStd = kOutMean + kOut,
              kSurrogateParams = kOutStd + kOut;
static std::vector<double> g_mlp_d;
static std::vector<float> g_mlp_f;
template <class R> static const R* mlp_params();
template <> const double* mlp_params<double>() { return g_mlp_d.data(); }
template <> const float* mlp_params<float>() { return g_mlp_f.data(); }

template <class R>
struct BicycleSlipMLP : BicycleSlip<R>
{
  // Kinematic rows as NeuralNetModel::computeKinematics (ar_nn_model.cu:119-124); the other five derivatives come
  // from the network on the normalised (state, control) row (NeuralNetModel::computeDynamics, ar_nn_model.cu:127-156)
  // evaluated in precision R with exact tanh.
  void deriv(const R* x, const R* u, R* xd) const
  {
    const R* P = mlp_params<R>();
    R sy, cy;
    M<R>::sincos(x[2], &sy, &cy);
    xd[0] = x[3] * cy - x[4] * sy;
    xd[1] = x[3] * sy + x[4] * cy;
    R in[kIn], h1[kHid], h2[kHid], y[kOut];
    for (int i = 0; i < 7; ++i) in[i] = (x[i] - P[kInMean + i]) / P[kInStd + i];
    for (int i = 0; i < 2; ++i) in[7 + i] = (u[i] - P[kInMean + 7 + i]) / P[kInStd + 7 + i];
    mlp_forward<R>(P, in, h1, h2, y);
    for (int j = 0; j < kOut; ++j) xd[2 + j] = y[j] * P[kOutStd + j] + P[kOutMean + j];
  }
};

// The plugin pair of the engine's plugin tests (tests/plugins/di_plugins.cu), restated: DoubleIntegratorDynamics
// (di_dynamics.cu:46-53) with an optional linear damping, stepped by the default Euler update or (symplectic) by the
// plugin's own step override (velocity first, then position with the new velocity); QuadraticCostImpl's device
// state cost (quadratic_cost.cu:35-48, the square written as a product) with a crash wall: once x > wall_x the
// sample's crash flag stays set and every later step pays crash_cost (the crash argument of computeRunningCost,
// cost.cuh:221-222).
struct mppi_test_di_plugin
{
  float damping;
};
// The third test pair's dynamics: the same double integrator with its own enforceConstraints, an acceleration limit
// that shrinks with speed, |u_i| <= max(0.5, a_max - speed_gain * |v_i|).
struct mppi_test_di_constrained_plugin
{
  float damping;
  float a_max;
  float speed_gain;
};
struct mppi_test_quad_wall_cost
{
  float s_goal[4];
  float s_coeffs[4];
  float wall_x;
  float crash_cost;
  float terminal_coeff;
};
constexpr int kTestPluginEuler = 101, kTestPluginSymplectic = 102, kTestPluginConstrained = 103;

template <class R>
struct TestDIPlugin
{
  static const int S = 4, C = 2;
  static constexpr bool kCrash = true;
  const mppi_test_di_plugin& p;
  const mppi_test_quad_wall_cost& q;
  bool symplectic;
  const mppi_test_di_constrained_plugin* lim;  // non-null: the plugin's own enforceConstraints
  // the plugin's enforceConstraints(state, control), in the arithmetic of its device code
  void constrain(const R* x, R* u) const
  {
    for (int i = 0; i < 2; ++i)
    {
      const R amax = std::fmax((R)0.5, (R)lim->a_max - (R)lim->speed_gain * std::fabs(x[2 + i]));
      u[i] = std::fmin(std::fmax(u[i], -amax), amax);
    }
  }
  void deriv(const R* x, const R* u, R* xd) const
  {
    xd[0] = x[2];
    xd[1] = x[3];
    xd[2] = u[0] - (R)p.damping * x[2];
    xd[3] = u[1] - (R)p.damping * x[3];
  }
  void step(const R* x, const R* u, R* xn, R dt) const
  {
    R xd[4];
    deriv(x, u, xd);
    if (symplectic)
    {
      xn[2] = M<R>::fma(xd[2], dt, x[2]);
      xn[3] = M<R>::fma(xd[3], dt, x[3]);
      xn[0] = M<R>::fma(xn[2], dt, x[0]);
      xn[1] = M<R>::fma(xn[3], dt, x[1]);
    }
    else
    {
      for (int i = 0; i < 4; ++i) xn[i] = M<R>::fma(xd[i], dt, x[i]);
    }
  }
  R quad(const R* y) const
  {
    R cost = 0;
    for (int i = 0; i < 4; ++i)
    {
      const R e = y[i] - (R)q.s_goal[i];
      cost += e * e * (R)q.s_coeffs[i];
    }
    return cost;
  }
  R running_cost(const R* y, const R*, int, int* crash) const
  {
    R cost = quad(y);
    if (y[0] > (R)q.wall_x) *crash = 1;
    if (*crash) cost += (R)q.crash_cost;
    return cost;
  }
  R state_cost(const R* y, int) const { return quad(y); }
  R control_cost(const R*, int) const { return (R)0; }
  R terminal_cost(const R* y) const { return quad(y) * (R)q.terminal_coeff; }
};

struct ModelBlob
{
  int model;
  const void* dyn;
  const void* cost;
  CostmapView map;
};

template <class R, class F>
static void with_model(const ModelBlob& b, F&& f)
{
  switch (b.model)
  {
    case MPPI_MODEL_CARTPOLE:
    {
      Cartpole<R> m{ *(const mppi_cartpole_params*)b.dyn, *(const mppi_cartpole_cost_params*)b.cost };
      f(m);
      break;
    }
    case MPPI_MODEL_DOUBLE_INTEGRATOR:
    {
      DoubleIntegrator<R> m{ *(const mppi_di_obstacle_cost_params*)b.cost };
      f(m);
      break;
    }
    case MPPI_MODEL_BICYCLE_COSTMAP:
    {
      BicycleCostmap<R> m{ *(const mppi_bicycle_params*)b.dyn, *(const mppi_costmap_cost_params*)b.cost, b.map };
      f(m);
      break;
    }
    case MPPI_MODEL_BICYCLE_SLIP:
    {
      BicycleSlip<R> m{ *(const mppi_bicycle_slip_params*)b.dyn, *(const mppi_costmap_cost_params*)b.cost, b.map };
      f(m);
      break;
    }
    case MPPI_MODEL_BICYCLE_SLIP_MLP:
    {
      BicycleSlipMLP<R> m{ { *(const mppi_bicycle_slip_params*)b.dyn, *(const mppi_costmap_cost_params*)b.cost,
                             b.map } };
      f(m);
      break;
    }
    case kTestPluginEuler:
    case kTestPluginSymplectic:
    case kTestPluginConstrained:
    {
      TestDIPlugin<R> m{ *(const mppi_test_di_plugin*)b.dyn, *(const mppi_test_quad_wall_cost*)b.cost,
                         b.model == kTestPluginSymplectic,
                         b.model == kTestPluginConstrained ? (const mppi_test_di_constrained_plugin*)b.dyn : nullptr };
      f(m);
      break;
    }
    default: break;
  }
}

static int model_state_dim(int model)
{
  switch (model)
  {
    case MPPI_MODEL_CARTPOLE: return 4;
    case MPPI_MODEL_DOUBLE_INTEGRATOR: return 4;
    case MPPI_MODEL_BICYCLE_COSTMAP: return 4;
    case MPPI_MODEL_BICYCLE_SLIP: return 7;
    case MPPI_MODEL_BICYCLE_SLIP_MLP: return g_mlp_d.empty() ? 0 : 7;
    case kTestPluginEuler: return 4;
    case kTestPluginSymplectic: return 4;
    case kTestPluginConstrained: return 4;
    default: return 0;
  }
}
static int model_control_dim(int model)
{
  switch (model)
  {
    case MPPI_MODEL_CARTPOLE: return 1;
    case MPPI_MODEL_DOUBLE_INTEGRATOR: return 2;
    case MPPI_MODEL_BICYCLE_COSTMAP: return 2;
    case MPPI_MODEL_BICYCLE_SLIP: return 2;
    case MPPI_MODEL_BICYCLE_SLIP_MLP: return 2;
    case kTestPluginEuler: return 2;
    case kTestPluginSymplectic: return 2;
    case kTestPluginConstrained: return 2;
    default: return 0;
  }
}

template <class R>
static void rollout_parallel(const ModelBlob& b, const float* x0, float* controls, bool write_back, const float* mean,
                             const mppi_sampling_params& sp, const mppi_control_constraints& cc, float lambda,
                             float alpha, int K, int T, float dt, double* costs, int threads, R* traj)
{
  if (threads < 1) threads = 1;
  threads = std::min(threads, K);
  std::vector<std::thread> pool;
  const int per = (K + threads - 1) / threads;
  for (int w = 0; w < threads; ++w)
  {
    const int kb = w * per, ke = std::min(K, kb + per);
    if (kb >= ke) break;
    pool.emplace_back([&, kb, ke]() {
      with_model<R>(b, [&](auto& m) {
        rollout_range<R>(m, x0, controls, write_back, mean, sp, cc, lambda, alpha, K, T, dt, kb, ke, costs, traj);
      });
    });
  }
  for (auto& th : pool) th.join();
}

// ------------------------------------------------------------------------------------------------ weights
// fullGPUcomputeWeights semantics (mppi_common.cu:938-1089): baseline = min cost, w = expf(-lambda_inv*(c - b)),
// normaliser = sum of w; the host normaliser sums in double (computeNormalizer, mppi_common.cu:1091-1099).
static void weights(const float* costs, int K, float lambda_inv, float* w, float* baseline, double* normalizer)
{
  float b = costs[0];
  for (int k = 1; k < K; ++k)
    if (costs[k] < b) b = costs[k];  // computeBestIndex (mppi_common.cu:918-936)
  double sum = 0.0;
  for (int k = 0; k < K; ++k)
  {
    const float d = costs[k] - b;
    w[k] = expf(-lambda_inv * d);
    sum += w[k];
  }
  *baseline = b;
  *normalizer = sum;
}

// TsallisTransform (mppi_common.cu:1004-1021), ColoredMPPI's alternative to the exponential: with d = c - baseline,
// w = exp(log(1 - d / gamma) / (r - 1)) for d < gamma, else 0.  The reference forms 1 - d / gamma with a double 1.0
// (the float quotient promoted), so the log's argument is that double narrowed back to float; kept here.
static void tsallis(const float* costs, int K, float gamma, float r, float baseline, float* w)
{
  for (int k = 0; k < K; ++k)
  {
    const float d = costs[k] - baseline;
    w[k] = d < gamma ? expf(logf((float)(1.0 - (double)(d / gamma))) / (r - 1.0f)) : 0.0f;
  }
}

// strideControlWeightReduction + rolloutWeightReductionAndSaveControl (mppi_common.cu:1151-1196):
// u_new[t][c] = sum_k (w_k / eta) * u_k[t][c].  Accumulated in double here (exact-ish reference value).
static void weighted_mean(const float* w, float normalizer, const float* controls, int K, int T, int C, double* out,
                          double* abs_out)
{
  const size_t TC = (size_t)T * C;
  std::fill(out, out + TC, 0.0);
  if (abs_out) std::fill(abs_out, abs_out + TC, 0.0);
  for (int k = 0; k < K; ++k)
  {
    const float wk = w[k] / normalizer;
    const float* uk = controls + (size_t)k * TC;
    for (size_t j = 0; j < TC; ++j)
    {
      out[j] += (double)wk * (double)uk[j];
      if (abs_out) abs_out[j] += std::fabs((double)wk * (double)uk[j]);
    }
  }
}

// Controller::smoothControlTrajectoryHelper (controller.cuh:573-607): 5-tap Savitzky-Golay [-3,12,17,12,-3]/35,
// left edge replicates u[0], right edge replicates u[T-1], u[0] kept.
static void smooth(float* u, int T, int C)
{
  const float coef[5] = { -3.0f / 35.0f, 12.0f / 35.0f, 17.0f / 35.0f, 12.0f / 35.0f, -3.0f / 35.0f };
  std::vector<float> buf((size_t)(T + 4) * C);
  for (int c = 0; c < C; ++c)
  {
    buf[0 * C + c] = u[c];
    buf[1 * C + c] = u[c];
    for (int t = 0; t < T; ++t) buf[(size_t)(t + 2) * C + c] = u[(size_t)t * C + c];
    buf[(size_t)(T + 2) * C + c] = u[(size_t)(T - 1) * C + c];
    buf[(size_t)(T + 3) * C + c] = u[(size_t)(T - 1) * C + c];
  }
  for (int t = 1; t < T; ++t)
    for (int c = 0; c < C; ++c)
    {
      float acc = 0.0f;
      for (int j = 0; j < 5; ++j) acc += coef[j] * buf[(size_t)(t + j) * C + c];
      u[(size_t)t * C + c] = acc;
    }
}

// Controller::slideControlSequenceHelper (controller.cuh:609-621)
static void slide(float* u, int T, int C, int steps, const float* scale, const float* zero)
{
  for (int i = 0; i < T; ++i)
  {
    const int ind = std::min(i + steps, T - 1);
    for (int c = 0; c < C; ++c)
    {
      float v = u[(size_t)ind * C + c];
      if (i + steps > T - 1) v = (v - zero[c]) * scale[c] + zero[c];
      u[(size_t)i * C + c] = v;
    }
  }
}

// ------------------------------------------------------------------------------------------------ colored noise
// ColoredNoiseDistributionImpl::generateSamples (colored_noise.cu:285-392) with fftfreq (colored_noise.cuh:24-34):
// per-frequency scale s_f = f^(-beta/2) with frequencies below the cutoff raised to it, sigma from the scales,
// configureFrequencyNoise (:12-37), an unnormalised inverse real FFT of length 2T (evaluated here as a direct DFT
// in double), and rearrangeNoise (:39-56).
static void colored_scales(int T, int C, const float* exponents, float fmin, std::vector<float>& scale /*[F][C]*/,
                           std::vector<float>& sigma /*[C]*/)
{
  const int N = 2 * T;
  const int F = N / 2 + 1;
  std::vector<float> freq(F);
  for (int i = 0; i < F; ++i) freq[i] = i / (1.0f * N);
  const float cutoff = fmaxf(fmin, 1.0f / N);
  scale.assign((size_t)F * C, 0.0f);
  int smaller = 0;
  for (int i = 0; i < F; ++i)
  {
    if (freq[i] < cutoff)
      smaller++;
    else if (smaller < F)
      for (int j = 0; j < smaller; ++j)
      {
        freq[j] = freq[smaller];
        for (int k = 0; k < C; ++k) scale[(size_t)j * C + k] = powf(freq[smaller], -exponents[k] / 2.0f);
      }
    for (int k = 0; k < C; ++k) scale[(size_t)i * C + k] = powf(freq[i], -exponents[k] / 2.0f);
  }
  sigma.assign(C, 0.0f);
  for (int k = 0; k < C; ++k)
  {
    float s = 0.0f;
    for (int j = 1; j < F - 1; ++j) s += scale[(size_t)j * C + k] * scale[(size_t)j * C + k];
    const float last = scale[(size_t)(F - 1) * C + k] * ((1.0f + (N % 2)) / 2.0f);
    s += last * last;
    sigma[k] = 2.0f * sqrtf(s) / N;
  }
}

static void colored_noise(const float* spectrum /*[K][C][F][2]*/, int K, int T, int C, const float* exponents,
                          float fmin, float decay, int offset_t, float* eps_out /*[K][T][C]*/, int threads)
{
  const int N = 2 * T, F = T + 1;
  std::vector<float> scale, sigma;
  colored_scales(T, C, exponents, fmin, scale, sigma);
  std::vector<double> cosb((size_t)N), sinb((size_t)N);
  for (int i = 0; i < N; ++i)
  {
    cosb[i] = std::cos(2.0 * M_PI * i / N);
    sinb[i] = std::sin(2.0 * M_PI * i / N);
  }
  auto work = [&](int kb, int ke) {
    std::vector<double> x((size_t)T + 1);
    std::vector<int> needed;
    for (int k = kb; k < ke; ++k)
      for (int c = 0; c < C; ++c)
      {
        const float* z = spectrum + ((size_t)k * C + c) * F * 2;
        auto eval = [&](int n) {
          double acc = (double)(z[0] * scale[c]);
          for (int f = 1; f < F; ++f)
          {
            const double re = (double)(z[2 * f] * scale[(size_t)f * C + c]);
            double im = (double)(z[2 * f + 1] * scale[(size_t)f * C + c]);
            if (f == F - 1 && (F % 2 == 1)) im = 0.0;
            const int idx = (int)(((long long)f * n) % N);
            if (2 * f == N)
              acc += re * cosb[idx];
            else
              acc += 2.0 * (re * cosb[idx] - im * sinb[idx]);
          }
          return acc;
        };
        const double xo = eval(offset_t);
        for (int t = 0; t < T; ++t)
        {
          const double xt = eval(t);
          const double d = decay == 0.0f ? 0.0 : (double)powf(decay, (float)t);
          eps_out[((size_t)k * T + t) * C + c] = (float)((xt - xo * d) / ((double)sigma[c] * N));
        }
      }
  };
  if (threads < 1) threads = 1;
  threads = std::min(threads, K);
  std::vector<std::thread> pool;
  const int per = (K + threads - 1) / threads;
  for (int w = 0; w < threads; ++w)
  {
    const int kb = w * per, ke = std::min(K, kb + per);
    if (kb < ke) pool.emplace_back(work, kb, ke);
  }
  for (auto& th : pool) th.join();
}

// ------------------------------------------------------------------------------------------------ MLP surrogate
// Mean squared error over B samples and 5 outputs and its gradient by hand back-propagation (FP64).
static double mlp_loss_grad(const double* p, const float* X, const float* Y, int B, double* g)
{
  std::fill(g, g + kNumParams, 0.0);
  double loss = 0.0;
  const double scale = 2.0 / ((double)B * kOut);
  for (int b = 0; b < B; ++b)
  {
    double x[kIn], h1[kHid], h2[kHid], y[kOut], dy[kOut], dh2[kHid], dh1[kHid];
    for (int i = 0; i < kIn; ++i) x[i] = X[(size_t)b * kIn + i];
    mlp_forward<double>(p, x, h1, h2, y);
    for (int j = 0; j < kOut; ++j)
    {
      const double e = y[j] - (double)Y[(size_t)b * kOut + j];
      loss += e * e;
      dy[j] = scale * e;
      g[kB3 + j] += dy[j];
      for (int i = 0; i < kHid; ++i) g[kW3 + j * kHid + i] += dy[j] * h2[i];
    }
    for (int i = 0; i < kHid; ++i)
    {
      double s = 0.0;
      for (int j = 0; j < kOut; ++j) s += dy[j] * p[kW3 + j * kHid + i];
      dh2[i] = s * (1.0 - h2[i] * h2[i]);
    }
    for (int j = 0; j < kHid; ++j)
    {
      g[kB2 + j] += dh2[j];
      for (int i = 0; i < kHid; ++i) g[kW2 + j * kHid + i] += dh2[j] * h1[i];
    }
    for (int i = 0; i < kHid; ++i)
    {
      double s = 0.0;
      for (int j = 0; j < kHid; ++j) s += dh2[j] * p[kW2 + j * kHid + i];
      dh1[i] = s * (1.0 - h1[i] * h1[i]);
    }
    for (int j = 0; j < kHid; ++j)
    {
      g[kB1 + j] += dh1[j];
      for (int i = 0; i < kIn; ++i) g[kW1 + j * kIn + i] += dh1[j] * x[i];
    }
  }
  return loss / ((double)B * kOut);
}

}  // namespace orc

// ================================================================================================= C interface
extern "C" {

int orc_mlp_num_params(void) { return orc::kNumParams; }

// Surrogate parameters (network + normalisation, 5153 floats) used by the MLP bicycle model.
void orc_set_mlp(const float* params)
{
  orc::g_mlp_f.assign(params, params + orc::kSurrogateParams);
  orc::g_mlp_d.assign(params, params + orc::kSurrogateParams);
}

// Forward pass of B samples (X float[B][9], Y float[B][5]) in FP64 with FP32 parameters.
void orc_mlp_forward(const float* params, const float* X, int B, double* Y)
{
  std::vector<double> p(params, params + orc::kNumParams);
  for (int b = 0; b < B; ++b)
  {
    double x[orc::kIn], h1[orc::kHid], h2[orc::kHid];
    for (int i = 0; i < orc::kIn; ++i) x[i] = X[(size_t)b * orc::kIn + i];
    orc::mlp_forward<double>(p.data(), x, h1, h2, Y + (size_t)b * orc::kOut);
  }
}

// MSE loss and its parameter gradient (hand back-propagation, FP64).
double orc_mlp_loss_grad(const double* params, const float* X, const float* Y, int B, double* grad)
{
  return orc::mlp_loss_grad(params, X, Y, B, grad);
}

void orc_set_trig_mode(int mode) { orc::g_trig_mode.store(mode == 1 ? 1 : 0); }
int orc_get_trig_mode(void) { return orc::g_trig_mode.load(); }

void orc_sincosf(const float* x, float* s, float* c, size_t n)
{
  for (size_t i = 0; i < n; ++i) orc::sincos_f(x[i], &s[i], &c[i]);
}

float orc_normalize_angle(float a) { return orc::M<float>::normalize_angle(a); }

void orc_philox4x32_10(const uint32_t* ctr, const uint32_t* key, uint32_t* out) { orc::philox4x32_10(ctr, key, out); }

void orc_gaussian_rewrite(const float* eps, const float* mean, const float* std_dev, int K, int T, int C, int stride,
                          float std_dev_decay_pow, float pure_pct, float* out)
{
  orc::gaussian_rewrite(eps, mean, std_dev, K, T, C, stride, std_dev_decay_pow, pure_pct, out);
}

void orc_enforce_constraints(float* u, size_t n_rows, int C, const mppi_control_constraints* cc)
{
  for (size_t r = 0; r < n_rows; ++r)
    for (int i = 0; i < C; ++i) u[r * C + i] = orc::enforce_constraint(u[r * C + i], *cc, i);
}

// Single-step dynamics derivative of a model (float or double), for plugin-level tests.
int orc_dynamics_deriv(int model, const void* dyn, const void* cost, const double* x, const double* u, double* xd,
                       int fp64)
{
  orc::ModelBlob b{ model, dyn, cost, {} };
  const int S = orc::model_state_dim(model), C = orc::model_control_dim(model);
  if (!S) return 1;
  if (fp64)
  {
    orc::with_model<double>(b, [&](auto& m) { m.deriv(x, u, xd); });
  }
  else
  {
    float xf[MPPI_MAX_STATE_DIM] = {}, uf[MPPI_MAX_CONTROL_DIM] = {}, xdf[MPPI_MAX_STATE_DIM] = {};
    for (int i = 0; i < S; ++i) xf[i] = (float)x[i];
    for (int i = 0; i < C; ++i) uf[i] = (float)u[i];
    orc::with_model<float>(b, [&](auto& m) { m.deriv(xf, uf, xdf); });
    for (int i = 0; i < S; ++i) xd[i] = xdf[i];
  }
  return 0;
}

// Rollout of K samples; controls are constrained and written back (float[K][T][C], in/out).  costs_out is
// double[K] (the float instantiation's values are exactly representable).  traj_out (may be NULL) receives
// double[K][T][S] stepped states.
int orc_rollout(int model, const void* dyn, const void* cost, const float* map, int map_w, int map_h, float map_res,
                float map_ox, float map_oy, const float* x0, float* controls, const float* mean,
                const mppi_sampling_params* sp, const mppi_control_constraints* cc, float lambda, float alpha, int K,
                int T, float dt, double* costs_out, double* traj_out, int threads, int fp64)
{
  orc::ModelBlob b{ model, dyn, cost, { map, map_w, map_h, map_res, map_ox, map_oy } };
  if (!orc::model_state_dim(model)) return 1;
  if (fp64)
  {
    orc::rollout_parallel<double>(b, x0, controls, true, mean, *sp, *cc, lambda, alpha, K, T, dt, costs_out, threads,
                                  traj_out);
  }
  else
  {
    std::vector<float> traj;
    const int S = orc::model_state_dim(model);
    if (traj_out) traj.resize((size_t)K * T * S);
    orc::rollout_parallel<float>(b, x0, controls, true, mean, *sp, *cc, lambda, alpha, K, T, dt, costs_out, threads,
                                 traj_out ? traj.data() : nullptr);
    if (traj_out)
      for (size_t i = 0; i < traj.size(); ++i) traj_out[i] = traj[i];
  }
  return 0;
}

void orc_weights(const float* costs, int K, float lambda_inv, float* w, float* baseline, double* normalizer)
{
  orc::weights(costs, K, lambda_inv, w, baseline, normalizer);
}

void orc_tsallis(const float* costs, int K, float gamma, float r, float baseline, float* w)
{
  orc::tsallis(costs, K, gamma, r, baseline, w);
}

void orc_weighted_mean(const float* w, float normalizer, const float* controls, int K, int T, int C, double* out,
                       double* abs_out)
{
  orc::weighted_mean(w, normalizer, controls, K, T, C, out, abs_out);
}

void orc_smooth(float* u, int T, int C) { orc::smooth(u, T, C); }

void orc_slide(float* u, int T, int C, int steps, const float* scale, const float* zero)
{
  orc::slide(u, T, C, steps, scale, zero);
}

void orc_colored_scales(int T, int C, const float* exponents, float fmin, float* scale_out /*[F][C]*/,
                        float* sigma_out /*[C]*/)
{
  std::vector<float> s, sg;
  orc::colored_scales(T, C, exponents, fmin, s, sg);
  std::copy(s.begin(), s.end(), scale_out);
  std::copy(sg.begin(), sg.end(), sigma_out);
}

void orc_colored_noise(const float* spectrum, int K, int T, int C, const float* exponents, float fmin, float decay,
                       int offset_t, float* eps_out, int threads)
{
  orc::colored_noise(spectrum, K, T, C, exponents, fmin, decay, offset_t, eps_out, threads);
}

// One VanillaMPPIController::computeControl (include/mppi/controllers/MPPI/mppi_controller.cu:152-237) for a single
// instance with given per-iteration standard-normal noise (eps: num_iters x [K][T][C], already colored if the
// sampler is colored) — the "injected identical noise buffer" of the parity definition.  control (float[T][C]) is the
// nominal sequence in/out; the function also returns the last iteration's costs, weights, samples, baseline and
// normaliser, and the nominal state trajectory (float[T][S], computeOutputTrajectoryHelper, controller.cuh:664-684).
int orc_compute_control(int model, const void* dyn, const void* cost, const float* map, int map_w, int map_h,
                        float map_res, float map_ox, float map_oy, const mppi_controller_params* cp,
                        const mppi_sampling_params* sp, const mppi_control_constraints* cc, int K, int T,
                        const float* x0, const float* eps, int eps_per_iter_stride_zero, int stride, float* control,
                        float* costs_out, float* weights_out, float* samples_out, float* baseline_out,
                        double* normalizer_out, float* state_seq_out, int threads)
{
  orc::ModelBlob b{ model, dyn, cost, { map, map_w, map_h, map_res, map_ox, map_oy } };
  const int S = orc::model_state_dim(model), C = orc::model_control_dim(model);
  if (!S) return 1;
  const size_t n = (size_t)K * T * C;
  std::vector<float> samples(n), w(K), costs_f(K);
  std::vector<double> costs(K), mean_d((size_t)T * C);
  float baseline = 0.0f;
  double normalizer = 0.0;
  // ColoredMPPIController (colored_mppi_controller.cu:145-249): Tsallis weights when gamma and r are non-zero, and a
  // final clamp of control 1 alone
  const bool colored = cp->controller == MPPI_CONTROLLER_COLORED;
  const bool tsallis = colored && cp->tsallis_gamma != 0.0f && cp->tsallis_r != 0.0f;
  for (int it = 0; it < cp->num_iters; ++it)
  {
    const float* e = eps + (eps_per_iter_stride_zero ? 0 : (size_t)it * n);
    orc::gaussian_rewrite(e, control, sp->std_dev, K, T, C, stride, powf(sp->std_dev_decay, (float)it),
                          sp->pure_noise_trajectories_percentage, samples.data());
    orc::rollout_parallel<float>(b, x0, samples.data(), true, control, *sp, *cc, cp->lambda, cp->alpha, K, T,
                                 cp->dt, costs.data(), threads, nullptr);
    for (int k = 0; k < K; ++k) costs_f[k] = (float)costs[k];
    orc::weights(costs_f.data(), K, 1.0f / cp->lambda, w.data(), &baseline, &normalizer);
    if (tsallis)
    {
      orc::tsallis(costs_f.data(), K, cp->tsallis_gamma, cp->tsallis_r, baseline, w.data());
      normalizer = 0.0;
      for (int k = 0; k < K; ++k) normalizer += w[k];  // computeNormalizer (mppi_common.cu:1091-1099)
    }
    orc::weighted_mean(w.data(), (float)normalizer, samples.data(), K, T, C, mean_d.data(), nullptr);
    for (size_t j = 0; j < (size_t)T * C; ++j) control[j] = (float)mean_d[j];
  }
  orc::smooth(control, T, C);
  // computeOutputTrajectoryHelper: x0, then T-1 constrained Euler steps of the nominal sequence
  if (state_seq_out)
  {
    float x[MPPI_MAX_STATE_DIM], xd[MPPI_MAX_STATE_DIM], u[MPPI_MAX_CONTROL_DIM];
    for (int i = 0; i < S; ++i) x[i] = state_seq_out[i] = x0[i];
    orc::with_model<float>(b, [&](auto& m) {
      for (int t = 0; t < T - 1; ++t)
      {
        // the constraint inside computeOutputTrajectoryHelper (controller.cuh:676-680)
        for (int i = 0; i < C; ++i) u[i] = orc::enforce_constraint(control[(size_t)t * C + i], *cc, i);
        float xn[MPPI_MAX_STATE_DIM];
        if constexpr (orc::HasCrash<std::decay_t<decltype(m)>>::value)
        {
          if (m.lim)
          {
            for (int i = 0; i < C; ++i) u[i] = control[(size_t)t * C + i];
            m.constrain(x, u);
          }
          m.step(x, u, xn, cp->dt);
        }
        else
        {
          m.deriv(x, u, xd);
          for (int i = 0; i < S; ++i) xn[i] = fmaf(xd[i], cp->dt, x[i]);
        }
        for (int i = 0; i < S; ++i) x[i] = state_seq_out[(size_t)(t + 1) * S + i] = xn[i];
      }
    });
  }
  bool own = false;
  orc::with_model<float>(b, [&](auto& m) {
    if constexpr (orc::HasCrash<std::decay_t<decltype(m)>>::value) own = m.lim != nullptr;
  });
  if (own && !colored)
  {
    // the final pass with a plugin's own enforceConstraints: a zero state (mppi_controller.cu:222-226)
    orc::with_model<float>(b, [&](auto& m) {
      if constexpr (orc::HasCrash<std::decay_t<decltype(m)>>::value)
      {
        const float zero[MPPI_MAX_STATE_DIM] = {};
        for (int t = 0; t < T; ++t) m.constrain(zero, control + (size_t)t * C);
      }
    });
  }
  else
  {
    for (int t = 0; t < T; ++t)
      for (int i = 0; i < C; ++i)
      {
        float& v = control[(size_t)t * C + i];
        if (!colored)
          v = orc::enforce_constraint(v, *cc, i);
        else if (i == 1)
          v = fminf(fmaxf(v, cc->lower[1]), cc->upper[1]);  // colored_mppi_controller.cu:224-229
      }
  }
  if (costs_out) std::copy(costs_f.begin(), costs_f.end(), costs_out);
  if (weights_out) std::copy(w.begin(), w.end(), weights_out);
  if (samples_out) std::copy(samples.begin(), samples.end(), samples_out);
  if (baseline_out) *baseline_out = baseline;
  if (normalizer_out) *normalizer_out = normalizer;
  return 0;
}

// TubeMPPIController::computeControl (include/mppi/controllers/Tube-MPPI/tube_mppi_controller.cu:158-296) for one
// controller: distribution 0 (actual system, from x_actual, around control[0]) and distribution 1 (nominal system,
// from nominal_x0, around control[1]) each sample K controls from their own eps block ([2][K][T][C], the same every
// iteration), roll out, weight and update; after each iteration the nominal pair takes the actual pair's state and
// control sequences when baseline_actual < baseline_nominal + nominal_threshold.  Then the nominal sequence is
// smoothed and both state trajectories are recomputed (computeStateTrajectoryHelper, controller.cuh:645-662).
int orc_tube_compute_control(int model, const void* dyn, const void* cost, const float* map, int map_w, int map_h,
                             float map_res, float map_ox, float map_oy, const mppi_controller_params* cp,
                             const mppi_sampling_params* sp, const mppi_control_constraints* cc, int K, int T,
                             const float* x_actual, float* nominal_x0, const float* eps, int stride, float* control,
                             float* costs_out, float* weights_out, float* samples_out, float* baselines_out,
                             double* normalizers_out, int* nominal_used_out, float* state_seq_out, int threads)
{
  orc::ModelBlob b{ model, dyn, cost, { map, map_w, map_h, map_res, map_ox, map_oy } };
  const int S = orc::model_state_dim(model), C = orc::model_control_dim(model);
  if (!S) return 1;
  const size_t n = (size_t)K * T * C, tc = (size_t)T * C;
  std::vector<float> samples(2 * n), w(2 * K), costs_f(2 * K);
  std::vector<double> costs(K), mean_d(tc);
  float baseline[2] = { 0.0f, 0.0f };
  double normalizer[2] = { 0.0, 0.0 };
  int nominal_used = 0;
  auto state_traj = [&](const float* x0, const float* u, float* out) {
    float x[MPPI_MAX_STATE_DIM], xn[MPPI_MAX_STATE_DIM], xd[MPPI_MAX_STATE_DIM], uc[MPPI_MAX_CONTROL_DIM];
    for (int i = 0; i < S; ++i) x[i] = out[i] = x0[i];
    orc::with_model<float>(b, [&](auto& m) {
      for (int t = 0; t < T - 1; ++t)
      {
        for (int i = 0; i < C; ++i) uc[i] = orc::enforce_constraint(u[(size_t)t * C + i], *cc, i);
        if constexpr (orc::HasCrash<std::decay_t<decltype(m)>>::value)
        {
          if (m.lim)
          {
            for (int i = 0; i < C; ++i) uc[i] = u[(size_t)t * C + i];
            m.constrain(x, uc);
          }
          m.step(x, uc, xn, cp->dt);
        }
        else
        {
          m.deriv(x, uc, xd);
          for (int i = 0; i < S; ++i) xn[i] = fmaf(xd[i], cp->dt, x[i]);
        }
        for (int i = 0; i < S; ++i) x[i] = out[(size_t)(t + 1) * S + i] = xn[i];
      }
    });
  };
  for (int it = 0; it < cp->num_iters; ++it)
  {
    for (int d = 0; d < 2; ++d)
    {
      float* sd = samples.data() + d * n;
      float* ctl = control + d * tc;
      orc::gaussian_rewrite(eps + d * n, ctl, sp->std_dev, K, T, C, stride, powf(sp->std_dev_decay, (float)it),
                            sp->pure_noise_trajectories_percentage, sd);
      orc::rollout_parallel<float>(b, d == 0 ? x_actual : nominal_x0, sd, true, ctl, *sp, *cc, cp->lambda,
                                   cp->alpha, K, T, cp->dt, costs.data(), threads, nullptr);
      for (int k = 0; k < K; ++k) costs_f[d * K + k] = (float)costs[k];
      orc::weights(costs_f.data() + d * K, K, 1.0f / cp->lambda, w.data() + d * K, &baseline[d], &normalizer[d]);
      orc::weighted_mean(w.data() + d * K, (float)normalizer[d], sd, K, T, C, mean_d.data(), nullptr);
      for (size_t j = 0; j < tc; ++j) ctl[j] = (float)mean_d[j];
    }
    state_traj(x_actual, control, state_seq_out);
    state_traj(nominal_x0, control + tc, state_seq_out + (size_t)T * S);
    if (baseline[0] < baseline[1] + cp->nominal_threshold)
    {
      nominal_used = 0;
      std::copy(state_seq_out, state_seq_out + (size_t)T * S, state_seq_out + (size_t)T * S);
      std::copy(x_actual, x_actual + S, nominal_x0);
      std::copy(control, control + tc, control + tc);
    }
    else
    {
      nominal_used = 1;
    }
  }
  orc::smooth(control + tc, T, C);
  state_traj(x_actual, control, state_seq_out);
  state_traj(nominal_x0, control + tc, state_seq_out + (size_t)T * S);
  if (costs_out) std::copy(costs_f.begin(), costs_f.end(), costs_out);
  if (weights_out) std::copy(w.begin(), w.end(), weights_out);
  if (samples_out) std::copy(samples.begin(), samples.end(), samples_out);
  for (int d = 0; d < 2; ++d)
  {
    if (baselines_out) baselines_out[d] = baseline[d];
    if (normalizers_out) normalizers_out[d] = normalizer[d];
  }
  if (nominal_used_out) *nominal_used_out = nominal_used;
  return 0;
}

// One nominal-state update of TubeMPPIController::slideControlSequence (updateNominalState,
// tube_mppi_controller.cu:343-349): x <- step(x, u), no constraint.
}  // extern "C"

// ---- R-MPPI (the robust controller's two rollouts), for the built-in models in float ------------------------------

namespace orc
{
// One step's control constraint for the robust controller's rollouts: the plugin-test pair's own enforceConstraints
// with the state when it has one, else the deadband and clamp (Dynamics::enforceConstraints, dynamics.cu:107-126).
template <class Model>
static void rm_constrain(const Model& m, const float* x, float* u, const mppi_control_constraints& cc)
{
  if constexpr (HasCrash<Model>::value)
    if (m.lim)
    {
      m.constrain(x, u);
      return;
    }
  for (int c = 0; c < Model::C; ++c) u[c] = enforce_constraint(u[c], cc, c);
}

// One step x -> xn and its running cost on the stepped state: the plugin-test pair's own step and computeRunningCost
// with the system's crash flag, else the Euler step and state + control cost.
template <class Model>
static float rm_step(const Model& m, const float* x, const float* u, float* xn, int t, float dt, int* crash)
{
  if constexpr (HasCrash<Model>::value)
  {
    m.step(x, u, xn, dt);
    return m.running_cost(xn, u, t, crash);
  }
  else
  {
    float xd[MPPI_MAX_STATE_DIM];
    m.deriv(x, u, xd);
    for (int s = 0; s < Model::S; ++s) xn[s] = fmaf(xd[s], dt, x[s]);
    return m.state_cost(xn, t) + m.control_cost(u, t);
  }
}

// rolloutRMPPIKernel (rmppi_kernels.cu:666-861) for samples [kb, ke): per step the nominal system's sample,
// constrained and written back; the real system's sample plus the feedback K_t (x_real - x_nominal) (the whole
// product, as DDPFeedback::k_ forms it, ddp.cuh:139-146), constrained and written back; Euler steps; running costs
// on the stepped states (each system with its own crash flag for the plugin-test pair).  The real system pays running + likelihood; the nominal one 0.5 J_nom + 0.5 max(min(J_fb,
// threshold), J_nom) + likelihood_nom, J_fb the real running cost plus the feedback cost (computeFeedbackCost,
// gaussian.cu:577-630); all divided by T, terminal costs added before.
template <class Model>
static void rmppi_rollout_range(const Model& m, const float* x0n, const float* x0r, float* un_all, float* ur_all,
                                const float* mean_n, const float* mean_r, const float* gains,
                                const mppi_sampling_params& sp, const mppi_control_constraints& cc, float lambda,
                                float alpha, float thr, int K, int T, float dt, int kb, int ke, float* cost_n_out,
                                float* cost_r_out)
{
  const int S = Model::S, C = Model::C;
  const bool use_likelihood = std::any_of(sp.control_cost_coeff, sp.control_cost_coeff + C,
                                          [](float v) { return v != 0.0f; });
  for (int k = kb; k < ke; ++k)
  {
    float xn[MPPI_MAX_STATE_DIM], xr[MPPI_MAX_STATE_DIM];
    for (int s = 0; s < S; ++s)
    {
      xn[s] = x0n[s];
      xr[s] = x0r[s];
    }
    float run_n = 0.0f, lik_n = 0.0f, run_r = 0.0f, extra_r = 0.0f;
    int crash_n = 0, crash_r = 0;
    for (int t = 0; t < T; ++t)
    {
      float* un = un_all + ((size_t)k * T + t) * C;
      float* ur = ur_all + ((size_t)k * T + t) * C;
      float u_n[MPPI_MAX_CONTROL_DIM], u_r[MPPI_MAX_CONTROL_DIM], fb[MPPI_MAX_CONTROL_DIM];
      float xn2[MPPI_MAX_STATE_DIM], xr2[MPPI_MAX_STATE_DIM];
      for (int c = 0; c < C; ++c) u_n[c] = un[c];
      rm_constrain(m, xn, u_n, cc);
      for (int c = 0; c < C; ++c) un[c] = u_n[c];
      for (int r = 0; r < C; ++r)
      {
        float acc = 0.0f;
        for (int c = 0; c < S; ++c) acc += gains[(size_t)t * C * S + r + (size_t)c * C] * (xr[c] - xn[c]);
        fb[r] = acc;
      }
      for (int c = 0; c < C; ++c) u_r[c] = ur[c] + fb[c];
      rm_constrain(m, xr, u_r, cc);
      for (int c = 0; c < C; ++c) ur[c] = u_r[c];
      const float cn = rm_step(m, xn, u_n, xn2, t, dt, &crash_n);
      const float cr = rm_step(m, xr, u_r, xr2, t, dt, &crash_r);
      run_n += cn;
      if (use_likelihood)
      {
        lik_n += likelihood_cost<float>(u_n, mean_n + (size_t)t * C, sp, C, k, K, lambda, alpha);
        run_r += cr + likelihood_cost<float>(u_r, mean_r + (size_t)t * C, sp, C, k, K, lambda, alpha);
      }
      else
      {
        run_r += cr;
      }
      float fc = 0.0f;
      for (int i = 0; i < C; ++i)
        fc += sp.control_cost_coeff[i] * (fb[i] * fb[i]) / (sp.std_dev[i] * sp.std_dev[i]);
      extra_r += cr + 0.5f * lambda * (1.0f - alpha) * fc;
      for (int s = 0; s < S; ++s)
      {
        xn[s] = xn2[s];
        xr[s] = xr2[s];
      }
    }
    run_n += m.terminal_cost(xn);
    const float tr = m.terminal_cost(xr);
    run_r += tr;
    extra_r += tr;
    const float Tf = (float)T;
    run_n /= Tf;
    lik_n /= Tf;
    run_r /= Tf;
    extra_r /= Tf;
    float cn = (float)(0.5 * (double)run_n + 0.5 * (double)fmaxf(fminf(extra_r, thr), run_n));
    cn += lik_n;
    cost_n_out[k] = cn;
    cost_r_out[k] = run_r;
  }
}

// initEvalKernel (rmppi_kernels.cu:231-357): rollout g = candidate * per_cand + j from the candidate's state with
// sample j of the nominal distribution read at min(t + stride, T - 1), constrained, not written back; running cost
// plus the likelihood term of sample index g against the mean at t; cost = running / T + terminal / T.
template <class Model>
static void rmppi_eval_range(const Model& m, const float* cand, const int* strides, int per_cand,
                             const float* samples, const float* mean, const mppi_sampling_params& sp,
                             const mppi_control_constraints& cc, float lambda, float alpha, int K, int T, float dt,
                             int gb, int ge, float* out)
{
  const int S = Model::S, C = Model::C;
  const bool use_likelihood = std::any_of(sp.control_cost_coeff, sp.control_cost_coeff + C,
                                          [](float v) { return v != 0.0f; });
  for (int g = gb; g < ge; ++g)
  {
    const int ci = g / per_cand, j = g - ci * per_cand, stride = strides[ci];
    float x[MPPI_MAX_STATE_DIM], xn[MPPI_MAX_STATE_DIM], u[MPPI_MAX_CONTROL_DIM];
    for (int s = 0; s < S; ++s) x[s] = cand[(size_t)ci * S + s];
    float running = 0.0f;
    int crash = 0;
    for (int t = 0; t < T; ++t)
    {
      const int tc = std::min(t + stride, T - 1);
      for (int c = 0; c < C; ++c) u[c] = samples[((size_t)j * T + tc) * C + c];
      rm_constrain(m, x, u, cc);
      float c = rm_step(m, x, u, xn, t, dt, &crash);
      if (use_likelihood) c += likelihood_cost<float>(u, mean + (size_t)t * C, sp, C, g, K, lambda, alpha);
      running += c;
      for (int s = 0; s < S; ++s) x[s] = xn[s];
    }
    out[g] = running / (float)T + m.terminal_cost(x) / (float)T;
  }
}

static bool rmppi_model(int model)
{
  return (model >= MPPI_MODEL_CARTPOLE && model <= MPPI_MODEL_BICYCLE_SLIP) ||
         (model >= kTestPluginEuler && model <= kTestPluginConstrained);
}
}  // namespace orc

extern "C" {

int orc_rmppi_rollout(int model, const void* dyn, const void* cost, const float* map, int map_w, int map_h,
                      float map_res, float map_ox, float map_oy, const float* x0_nom, const float* x0_real,
                      float* samples_nom, float* samples_real, const float* mean_nom, const float* mean_real,
                      const float* gains, const mppi_sampling_params* sp, const mppi_control_constraints* cc,
                      float lambda, float alpha, float threshold, int K, int T, float dt, float* costs_nom,
                      float* costs_real, int threads)
{
  if (!orc::rmppi_model(model)) return 1;
  orc::ModelBlob b{ model, dyn, cost, { map, map_w, map_h, map_res, map_ox, map_oy } };
  threads = std::max(1, std::min(threads, K));
  std::vector<std::thread> pool;
  const int per = (K + threads - 1) / threads;
  for (int w = 0; w < threads; ++w)
  {
    const int kb = w * per, ke = std::min(K, kb + per);
    if (kb >= ke) break;
    pool.emplace_back([&, kb, ke]() {
      orc::with_model<float>(b, [&](auto& m) {
        orc::rmppi_rollout_range(m, x0_nom, x0_real, samples_nom, samples_real, mean_nom, mean_real, gains, *sp, *cc,
                                 lambda, alpha, threshold, K, T, dt, kb, ke, costs_nom, costs_real);
      });
    });
  }
  for (auto& th : pool) th.join();
  return 0;
}

int orc_rmppi_eval(int model, const void* dyn, const void* cost, const float* map, int map_w, int map_h,
                   float map_res, float map_ox, float map_oy, const float* cand_states, const int* cand_strides,
                   int num_cand, int per_cand, const float* samples, const float* mean,
                   const mppi_sampling_params* sp, const mppi_control_constraints* cc, float lambda, float alpha,
                   int K, int T, float dt, float* costs_out)
{
  if (!orc::rmppi_model(model)) return 1;
  orc::ModelBlob b{ model, dyn, cost, { map, map_w, map_h, map_res, map_ox, map_oy } };
  orc::with_model<float>(b, [&](auto& m) {
    orc::rmppi_eval_range(m, cand_states, cand_strides, per_cand, samples, mean, *sp, *cc, lambda, alpha, K, T, dt, 0,
                          num_cand * per_cand, costs_out);
  });
  return 0;
}

int orc_step_state(int model, const void* dyn, const void* cost, const float* u, float dt, float* x)
{
  orc::ModelBlob b{ model, dyn, cost, { nullptr, 0, 0, 1.0f, 0.0f, 0.0f } };
  const int S = orc::model_state_dim(model);
  if (!S) return 1;
  float xn[MPPI_MAX_STATE_DIM], xd[MPPI_MAX_STATE_DIM];
  orc::with_model<float>(b, [&](auto& m) {
    if constexpr (orc::HasCrash<std::decay_t<decltype(m)>>::value)
    {
      m.step(x, u, xn, dt);
    }
    else
    {
      m.deriv(x, u, xd);
      for (int i = 0; i < S; ++i) xn[i] = fmaf(xd[i], dt, x[i]);
    }
  });
  for (int i = 0; i < S; ++i) x[i] = xn[i];
  return 0;
}

}  // extern "C"
