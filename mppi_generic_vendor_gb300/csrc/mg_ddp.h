// mg_ddp.h — the ancillary feedback controller of the reference (DDPFeedback, feedback_controllers/DDP/ddp.cu:48-120):
// differential dynamic programming around a nominal trajectory with a quadratic tracking cost, run on the host after a
// solve; its time-varying gains K_t give the feedback control K_t (x - x_target_t) that Tube-MPPI and the plant add to
// the nominal control.
//
// The solver restates DDP::run (ddp/ddp.h:40-195) for TrackingCostDDP / TrackingTerminalCost (ddp/ddp_tracking_costs.h):
//   * forward rollout of the nominal controls from x0 with explicit Euler, x_{i+1} = x_i + f(x_i, u_i) dt, where
//     controls 0 .. H-3 are clamped to the control range first (the last one is not, as in the reference loop);
//   * per iteration: Jacobians Phi_k = I + A_k dt, B_k dt; running cost (x - x*)' Q (x - x*) + (u - u*)' R (u - u*)
//     with gradient (Q (x - x*), R (u - u*)) and Hessian diag(Q, R) (the reference's gradient omits the factor 2 of
//     its cost; kept); terminal cost on Q_f around the last target state;
//   * backward pass for k = H-2 .. 0:
//       qx = l_x dt + Phi' Vx,  qu = l_u dt + B' Vx,  qux = B' Vxx Phi,  qxx = Q dt + Phi' Vxx Phi,
//       quu = R dt + B' Vxx B,  K_k = -quu^-1 qux,  k_k = -quu^-1 qu,
//       Vxx = sym(qxx + qux' K_k),  Vx = qx + qux' k_k;
//   * forward pass with a halving line search on the feedforward step, accepted at once in the first iteration.
// Gains K_{H-1} stay zero.  Linear algebra in double on the host; the dynamics are the model's FP32 host twin.
// The gain of step t is stored as the reference stores an Eigen C x S matrix: element (r, c) at t * C * S + r + c * C.
#pragma once

#include <cmath>
#include <cstring>
#include <type_traits>
#include <utility>
#include <vector>

namespace mg
{

// Whether a built-in model has host Jacobians, static bool computeGrad(const DynParams&, const float* x,
// const float* u, double* A, double* B) (the reference's HasAnalyticGrad test, ddp/ddp_model_wrapper.h:7-16).
template <class M, class = void>
struct HasAnalyticGrad : std::false_type
{
};
template <class M>
struct HasAnalyticGrad<M, std::void_t<decltype(M::computeGrad(std::declval<const typename M::DynParams&>(),
                                                               std::declval<const float*>(),
                                                               std::declval<const float*>(), std::declval<double*>(),
                                                               std::declval<double*>()))>> : std::true_type
{
};

// Tracking-cost weights and iteration count (DDPParams, feedback_controllers/DDP/ddp.cuh:16-25): Q and Qf are
// S x S, R is C x C, all column-major like the reference's Eigen matrices; the defaults are identities and one
// iteration.
struct DdpWeights
{
  std::vector<double> Q, Qf, R;
  int iterations = 1;
};

// Forward-difference Jacobian of xdot = f(x, u) in FP32, as Eigen's NumericalDiff (Forward, epsfcn 0) evaluates it
// for models without an analytic computeGrad (ddp/ddp_dynamics.h:96-101): step h_j = sqrt(FLT_EPSILON) |v_j|, or
// sqrt(FLT_EPSILON) where v_j = 0; column j = (f(v + h_j e_j) - f(v)) / h_j.  A is S x S, B is S x C, row-major.
template <int S, int C, class F>
void numeric_jacobian(const F& f, const float* x, const float* u, double* A, double* B)
{
  const float eps = std::sqrt(1.1920929e-7f);
  float v[S + C], f0[S], f1[S];
  for (int s = 0; s < S; ++s) v[s] = x[s];
  for (int c = 0; c < C; ++c) v[S + c] = u[c];
  f(v, v + S, f0);
  for (int j = 0; j < S + C; ++j)
  {
    float h = eps * std::fabs(v[j]);
    if (h == 0.0f) h = eps;
    const float keep = v[j];
    v[j] = keep + h;
    f(v, v + S, f1);
    v[j] = keep;
    for (int s = 0; s < S; ++s)
    {
      const double d = (double)((f1[s] - f0[s]) / h);
      if (j < S)
        A[s * S + j] = d;
      else
        B[s * C + (j - S)] = d;
    }
  }
}

// DDP::run for the tracking cost.  f(x, u, xdot) evaluates the dynamics; df(x, u, A, B) writes the continuous-time
// Jacobians (row-major S x S and S x C).  x_target [H][S] and u_nom [H][C] are the nominal trajectory (the target
// states and the controls the solver starts from, as Controller::computeFeedback passes them, controller.cuh:562-565);
// u_min / u_max the control range.  gains receives H * C * S floats.  Returns false (and leaves gains untouched) if
// a quu block is not positive definite, where the reference's LDLT check exits the process (ddp.h:130-139).
template <int S, int C, class F, class DF>
bool ddp_tracking_gains(const F& f, const DF& df, const float* x0, const float* x_target, const float* u_nom, int H,
                        float dt, const DdpWeights& w, const float* u_min, const float* u_max, float* gains)
{
  if (H < 2) return false;
  const double Dt = (double)dt;
  std::vector<float> x((size_t)H * S), u((size_t)H * C);
  std::memcpy(u.data(), u_nom, sizeof(float) * (size_t)H * C);
  for (int s = 0; s < S; ++s) x[s] = x0[s];
  auto clamp_u = [&](float* uk) {
    for (int c = 0; c < C; ++c) uk[c] = std::fmax(std::fmin(uk[c], u_max[c]), u_min[c]);
  };
  auto euler = [&](const float* xk, const float* uk, float* xn) {
    float xd[S];
    f(xk, uk, xd);
    for (int s = 0; s < S; ++s) xn[s] = xk[s] + xd[s] * dt;
  };
  for (int i = 1; i < H; ++i)
  {
    if (i < H - 1) clamp_u(&u[(size_t)(i - 1) * C]);
    euler(&x[(size_t)(i - 1) * S], &u[(size_t)(i - 1) * C], &x[(size_t)i * S]);
  }
  auto Q = [&](int r, int c) { return w.Q[(size_t)r + (size_t)c * S]; };
  auto Qf = [&](int r, int c) { return w.Qf[(size_t)r + (size_t)c * S]; };
  auto R = [&](int r, int c) { return w.R[(size_t)r + (size_t)c * C]; };
  // running cost of (x, u) at step k (TrackingCostDDP::c)
  auto run_cost = [&](const float* xk, const float* uk, int k) {
    double cs = 0.0, cu = 0.0;
    for (int r = 0; r < S; ++r)
      for (int c = 0; c < S; ++c)
        cs += ((double)xk[r] - x_target[(size_t)k * S + r]) * Q(r, c) * ((double)xk[c] - x_target[(size_t)k * S + c]);
    for (int r = 0; r < C; ++r)
      for (int c = 0; c < C; ++c)
        cu += ((double)uk[r] - u_nom[(size_t)k * C + r]) * R(r, c) * ((double)uk[c] - u_nom[(size_t)k * C + c]);
    return cs + cu;
  };
  const float* xf = x_target + (size_t)(H - 1) * S;

  std::vector<double> Phi((size_t)H * S * S), Bm((size_t)H * S * C);  // discrete Jacobians, row-major
  std::vector<double> Kg((size_t)H * C * S, 0.0), kff((size_t)H * C, 0.0);  // K_k row-major C x S, k_k
  std::vector<double> prev_cost;
  for (int it = 0; it < w.iterations; ++it)
  {
    for (int k = 0; k < H; ++k)
    {
      double* A = &Phi[(size_t)k * S * S];
      double* B = &Bm[(size_t)k * S * C];
      std::fill(A, A + S * S, 0.0);
      std::fill(B, B + S * C, 0.0);
      df(&x[(size_t)k * S], &u[(size_t)k * C], A, B);
      for (int e = 0; e < S * S; ++e) A[e] *= Dt;
      for (int e = 0; e < S * C; ++e) B[e] *= Dt;
      for (int s = 0; s < S; ++s) A[s * S + s] += 1.0;
    }
    // boundary: Vxx = sym(Qf), Vx = Qf (x_{H-1} - xf), V = terminal cost
    double Vxx[S * S], Vx[S];
    double V_term = 0.0;
    for (int r = 0; r < S; ++r)
      for (int c = 0; c < S; ++c) Vxx[r * S + c] = 0.5 * (Qf(r, c) + Qf(c, r));
    for (int r = 0; r < S; ++r)
    {
      double acc = 0.0;
      for (int c = 0; c < S; ++c) acc += Qf(r, c) * ((double)x[(size_t)(H - 1) * S + c] - xf[c]);
      Vx[r] = acc;
    }
    for (int r = 0; r < S; ++r) V_term += ((double)x[(size_t)(H - 1) * S + r] - xf[r]) * Vx[r];
    for (int k = H - 2; k >= 0; --k)
    {
      const double* P = &Phi[(size_t)k * S * S];
      const double* B = &Bm[(size_t)k * S * C];
      double lx[S], lu[C];
      for (int r = 0; r < S; ++r)
      {
        double acc = 0.0;
        for (int c = 0; c < S; ++c) acc += Q(r, c) * ((double)x[(size_t)k * S + c] - x_target[(size_t)k * S + c]);
        lx[r] = acc;
      }
      for (int r = 0; r < C; ++r)
      {
        double acc = 0.0;
        for (int c = 0; c < C; ++c) acc += R(r, c) * ((double)u[(size_t)k * C + c] - u_nom[(size_t)k * C + c]);
        lu[r] = acc;
      }
      double VP[S * S], VB[S * C];  // Vxx Phi, Vxx B
      for (int r = 0; r < S; ++r)
      {
        for (int c = 0; c < S; ++c)
        {
          double acc = 0.0;
          for (int m = 0; m < S; ++m) acc += Vxx[r * S + m] * P[m * S + c];
          VP[r * S + c] = acc;
        }
        for (int c = 0; c < C; ++c)
        {
          double acc = 0.0;
          for (int m = 0; m < S; ++m) acc += Vxx[r * S + m] * B[m * C + c];
          VB[r * C + c] = acc;
        }
      }
      double qx[S], qu[C], qux[C * S], qxx[S * S], quu[C * C];
      for (int r = 0; r < S; ++r)
      {
        double acc = lx[r] * Dt;
        for (int m = 0; m < S; ++m) acc += P[m * S + r] * Vx[m];
        qx[r] = acc;
        for (int c = 0; c < S; ++c)
        {
          double a2 = Q(r, c) * Dt;
          for (int m = 0; m < S; ++m) a2 += P[m * S + r] * VP[m * S + c];
          qxx[r * S + c] = a2;
        }
      }
      for (int r = 0; r < C; ++r)
      {
        double acc = lu[r] * Dt;
        for (int m = 0; m < S; ++m) acc += B[m * C + r] * Vx[m];
        qu[r] = acc;
        for (int c = 0; c < S; ++c)
        {
          double a2 = 0.0;
          for (int m = 0; m < S; ++m) a2 += B[m * C + r] * VP[m * S + c];
          qux[r * S + c] = a2;
        }
        for (int c = 0; c < C; ++c)
        {
          double a2 = R(r, c) * Dt;
          for (int m = 0; m < S; ++m) a2 += B[m * C + r] * VB[m * C + c];
          quu[r * C + c] = a2;
        }
      }
      // quu = L D L' from its lower triangle, as Eigen's LDLT reads it (no pivoting: quu is symmetric positive
      // definite for a positive definite R), then K = -quu^-1 qux and k = -quu^-1 qu column by column
      double Lf[C * C] = {}, D[C];
      for (int j = 0; j < C; ++j)
      {
        double d = quu[j * C + j];
        for (int m = 0; m < j; ++m) d -= Lf[j * C + m] * Lf[j * C + m] * D[m];
        if (!(d > 0.0) || !std::isfinite(d)) return false;
        D[j] = d;
        Lf[j * C + j] = 1.0;
        for (int i = j + 1; i < C; ++i)
        {
          double v = quu[i * C + j];
          for (int m = 0; m < j; ++m) v -= Lf[i * C + m] * Lf[j * C + m] * D[m];
          Lf[i * C + j] = v / d;
        }
      }
      auto solve = [&](const double* rhs, double* out) {  // out = -quu^-1 rhs
        double y[C];
        for (int i = 0; i < C; ++i)
        {
          double v = -rhs[i];
          for (int m = 0; m < i; ++m) v -= Lf[i * C + m] * y[m];
          y[i] = v;
        }
        for (int i = 0; i < C; ++i) y[i] /= D[i];
        for (int i = C - 1; i >= 0; --i)
        {
          double v = y[i];
          for (int m = i + 1; m < C; ++m) v -= Lf[m * C + i] * out[m];
          out[i] = v;
        }
      };
      double* Kk = &Kg[(size_t)k * C * S];
      for (int c = 0; c < S; ++c)
      {
        double col[C], sol[C];
        for (int r = 0; r < C; ++r) col[r] = qux[r * S + c];
        solve(col, sol);
        for (int r = 0; r < C; ++r) Kk[r * S + c] = sol[r];
      }
      solve(qu, &kff[(size_t)k * C]);
      // value function back one step
      double nVxx[S * S], nVx[S];
      for (int r = 0; r < S; ++r)
      {
        for (int c = 0; c < S; ++c)
        {
          double acc = qxx[r * S + c];
          for (int m = 0; m < C; ++m) acc += qux[m * S + r] * Kk[m * S + c];
          nVxx[r * S + c] = acc;
        }
        double acc = qx[r];
        for (int m = 0; m < C; ++m) acc += qux[m * S + r] * kff[(size_t)k * C + m];
        nVx[r] = acc;
      }
      for (int r = 0; r < S; ++r)
        for (int c = 0; c < S; ++c) Vxx[r * S + c] = 0.5 * (nVxx[r * S + c] + nVxx[c * S + r]);
      std::memcpy(Vx, nVx, sizeof(Vx));
    }
    // forward pass with line search (the result of the last iteration's pass becomes the nominal trajectory)
    double alpha = 1.0;
    std::vector<float> xn((size_t)H * S), un((size_t)H * C);
    std::vector<double> cost(H);
    for (;;)
    {
      std::fill(un.begin(), un.end(), 0.0f);
      for (int s = 0; s < S; ++s) xn[s] = x[s];
      double total = 0.0;
      for (int k = 0; k < H - 1; ++k)
      {
        float* uk = &un[(size_t)k * C];
        const double* Kk = &Kg[(size_t)k * C * S];
        for (int r = 0; r < C; ++r)
        {
          double v = (double)u[(size_t)k * C + r] + alpha * kff[(size_t)k * C + r];
          for (int c = 0; c < S; ++c) v += Kk[r * S + c] * ((double)xn[(size_t)k * S + c] - x[(size_t)k * S + c]);
          uk[r] = (float)v;
        }
        clamp_u(uk);
        euler(&xn[(size_t)k * S], uk, &xn[(size_t)(k + 1) * S]);
        cost[k] = run_cost(&xn[(size_t)k * S], uk, k) * Dt;
        total += cost[k];
      }
      cost[H - 1] = V_term;
      total += V_term;
      double prev_total = 0.0;
      for (double c : prev_cost) prev_total += c;
      if (it == 0 || alpha < 1e-4 || total <= prev_total)
      {
        x.swap(xn);
        u.swap(un);
        prev_cost = cost;
        break;
      }
      alpha *= 0.5;
    }
  }
  // the gains in the reference's storage: per step an Eigen C x S matrix, column-major
  for (int k = 0; k < H; ++k)
    for (int r = 0; r < C; ++r)
      for (int c = 0; c < S; ++c) gains[(size_t)k * C * S + r + (size_t)c * C] = (float)Kg[(size_t)k * C * S + r * S + c];
  return true;
}

// The feedback control K_t (x - x_goal) (DDPFeedback::k_, feedback_controllers/DDP/ddp.cuh:139-146).
template <int S, int C>
void ddp_feedback_control(const float* gains, int t, const float* x, const float* x_goal, float* u)
{
  const float* K = gains + (size_t)t * C * S;
  for (int r = 0; r < C; ++r)
  {
    float acc = 0.0f;
    for (int c = 0; c < S; ++c) acc += K[r + c * C] * (x[c] - x_goal[c]);
    u[r] = acc;
  }
}

}  // namespace mg
