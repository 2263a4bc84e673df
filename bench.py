"""Benchmark of the GB300 MPPI engine: MPPI iterations/s and sample-steps/s on one GPU.

A step is one MPPI iteration (sample -> rollout -> weights -> update) over every instance of the workload.
* value — sample-steps/s of device-resident solves (inputs already in HBM; mppi_enqueue_solve), timed with CUDA events
  on the engine's stream; max over ranks; whole-job aggregate.
* e2e   — the same metric through the public computeControl call with host buffers: the H2D copy of the initial
  states and nominal controls, the device work, the D2H copy of the result and the host post-processing are inside
  the timed region every step.
* roofline — the dominant kernel's algorithmic bytes per launch / its CUDA-event duration, against the measured HBM
  copy bandwidth.
* cpu_baseline — the CPU oracle (a restatement of the reference's host rollout + weight + update path) on a bounded
  sample of the same workload, all host threads.

``--workload cartpole_rmppi`` times the robust controller (R-MPPI), a host-iterated controller: every iteration runs
the importance-sampler update (candidate evaluation kernel, free energies and the DDP gains on the host) and the solve
through the public calls, so its line reports the end-to-end rate as `value` too, with the solve's kernel times
beside it.  ``--workload cartpole_tube`` does the same for Tube-MPPI (solve, feedback gains, one-step slide).

Multi-GPU: the path does not shard across GPUs; ``--gpus N`` under torchrun runs N independent replicas (weak scaling).
``--impl reference`` times the reference's CPU path (the oracle port) and prints its own line.
"""
from __future__ import annotations

import argparse
import json
import os
import shutil
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

METRIC = "MPPI sample-steps/s (iters/s x sum_i K_i*T_i) on 1 GB300"
UNIT = "sample-steps/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default: enough for about 1.2 s of device time, at least 20)")
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="batched_slip_mlp", choices=["batched_di", "cartpole", "bicycle",
                                                                 "batched_di_gaussian", "slip_mlp",
                                                                 "batched_slip_mlp", "cartpole_rmppi",
                                                                 "cartpole_tube"])
    ap.add_argument("--precision", default=None, choices=["bf16", "fp8", "fp32"],
                    help="surrogate workloads: weight precision (default bf16 for slip_mlp, fp8 for batched_slip_mlp)")
    ap.add_argument("--instances", type=int, default=256, help="batched workloads: number of instances")
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="CPU baseline sample budget")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def measured_peaks(kind="hbm"):
    """(peak, provenance): HBM copy GB/s, or burst bf16 TFLOP/s for a tensor-core kernel."""
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return (float(d["hbm_gbs"]) if kind == "hbm" else float(d["bf16_tflops"])), "measured"
    return (6800.0 if kind == "hbm" else 1900.0), "fallback"


# FLOPs of one surrogate evaluation (9 -> 64 -> 64 -> 5; multiply-adds counted as 2), per sample-step
MLP_FLOPS = 2 * (9 * 64 + 64 * 64 + 64 * 5)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.t = None

    def start(self):
        if shutil.which("nvidia-smi") is None:
            return
        self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                      "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE,
                                     stderr=subprocess.DEVNULL, text=True)
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.t:
            self.t.join(timeout=2)
        sm, mx, reasons = [], None, set()
        names = ["active", "hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names[1:], parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def build_workload(name, seed, stream, instances=256, precision=None, params=None, describe_only=False):
    """The named workload; describe_only: its shapes and description without creating a controller (no GPU work)."""
    from mppi_generic_vendor_gb300 import workloads as W

    kw = dict(seed=seed, stream=stream, describe_only=describe_only)
    if name == "slip_mlp":
        return W.slip_mlp(precision=precision or "bf16", params=params, **kw)
    if name == "batched_slip_mlp":
        return W.batched_slip_mlp(num_instances=instances if instances != 256 else 128, precision=precision or "fp8",
                                  params=params, **kw)
    if name == "batched_di":
        return W.batched_di(num_instances=instances, colored=True, **kw)
    if name == "batched_di_gaussian":
        return W.batched_di(num_instances=instances, colored=False, **kw)
    if name == "cartpole":
        return W.cartpole(**kw)
    if name == "cartpole_rmppi":
        return W.cartpole_rmppi(**kw)
    if name == "cartpole_tube":
        return W.cartpole_tube(**kw)
    return W.bicycle(**kw)


def config_of(wl, ws):
    """The `config` object of a bench line for workload wl at ws GPUs (shared by the GPU and the reference arm)."""
    return {"workload": wl.name, **wl.description, "num_iters": wl.num_iters,
            "sample_steps_per_iter": wl.sample_steps_per_iter,
            "l2": ("inputs larger than L2 (samples buffer %.0f MB)" % (wl.control_floats * 4 / 1e6))
            if wl.control_floats * 4 > 129e6 else
            "working set %.1f MB fits in L2; device-resident value is L2-warm" % (wl.control_floats * 4 / 1e6),
            "parallelism": "replicas" if ws > 1 else "single GPU"}


def algorithmic_bytes(wl, colored: bool):
    """Minimum HBM bytes per launch of each kernel (control samples are 4 B each, costs / weights 4 B per sample)."""
    n = wl.control_floats
    k = int(wl.K.sum())
    spec = int(np.sum(wl.K.astype(np.int64) * (wl.T + 1))) * wl.control_dim * 2 if colored else 0
    sampler = 4 * n  # write the constrained samples (Philox noise is generated in registers)
    rollout = 4 * n + 4 * k  # read the samples, write the costs
    update = 4 * n + 8 * k  # read the samples and costs, write the weights
    del spec
    return {"sampler": sampler, "rollout": rollout, "update": update}


_SURROGATE = {}
ROLLOUT_MODE_NAMES = ["fused", "split", "cooperative", "sampled", "fused_noise_warps"]


def surrogate_params(weight_format="fp32"):
    """Surrogate weights for the surrogate workloads, trained once per process on the GPU by the engine's own kernels,
    with quantisation-aware fine-tuning for a BF16 / FP8 deployment (the CPU baseline of the reference arm, which has
    no GPU, falls back to a fixed seeded initialisation)."""
    key = "p" if weight_format == "fp32" else "p_" + weight_format
    if key not in _SURROGATE and "p" in _SURROGATE and _SURROGATE.get("cpu_only"):
        return _SURROGATE["p"]
    if key not in _SURROGATE:
        try:
            if _SURROGATE.get("cpu_only"):
                raise RuntimeError("no GPU on this arm")
            from mppi_generic_vendor_gb300 import workloads as W

            _SURROGATE[key] = W.train_surrogate(weight_format=weight_format)
        except Exception:
            rng = np.random.default_rng(7)
            p = np.zeros(5153, np.float32)
            p[:576] = rng.normal(0, 1 / 3, 576)
            p[640:4736] = rng.normal(0, 1 / 8, 4096)
            p[4800:5120] = rng.normal(0, 1 / 8, 320)
            p[5134:5143] = [15.0, 15.0, 1.8, 4.0, 1.2, 0.9, 0.3, 0.6, 0.6]
            p[5125:5134] = [25.6, 25.6, 0.0, 8.0, 0.0, 0.0, 0.0, 0.0, 0.0]
            p[5148:5153] = 1.0
            _SURROGATE[key] = p
    return _SURROGATE[key]


def surrogate_extras(args, wl, stream):
    """Surrogate workloads: the plain GPU form (the same instances, analytic model in FP32, one controller per
    instance solved one after another) timed on the same GPU; the cost error of each instance's nominal control
    sequence under the surrogate against the FP64 analytic rollout; and the final trajectory cost: MPPI on the
    surrogate (judge on) against MPPI on the analytic model, both from zero control sequences for the same number of
    iterations, each final sequence costed by the FP64 analytic rollout."""
    import oracle
    from mppi_generic_vendor_gb300 import (BatchedMPPIController, BicycleSlipDynamics, GaussianDistribution,
                                           VanillaMPPIController)
    from mppi_generic_vendor_gb300 import _abi as A
    from mppi_generic_vendor_gb300 import workloads as W

    ctrl = wl.controller
    n = ctrl.num_instances
    x0 = wl.x0.reshape(n, 7)
    cmap = W.gaussian_bump_costmap(0)
    # plain GPU form
    plain = [VanillaMPPIController(BicycleSlipDynamics(), W._slip_cost(cmap), None,
                                   GaussianDistribution(std_dev=(0.5, 0.5)), 0.02, 1, 2.0, 0.0, int(wl.T[i]),
                                   int(wl.K[i]), seed=i, stream=stream) for i in range(n)]
    for c, x in zip(plain, x0):
        c.computeControl(x, 1)
    reps = max(2, min(5, args.steps))
    t0 = time.perf_counter()
    for _ in range(reps):
        for c, x in zip(plain, x0):
            c.computeControl(x, 1)
    plain_s = (time.perf_counter() - t0) / reps
    for c in plain:
        c.close()
    # final-cost error: sample 0 of an iteration is the nominal sequence (noise-free); judge off for this read-out
    ctrl.setJudge(0.0)
    ctrl.computeControl(wl.x0, 1)
    costs = ctrl.sample_costs()
    samples = ctrl.control_samples()
    ctrl.setJudge(0.01)
    errs = []
    u_off = 0
    sp = GaussianDistribution(std_dev=(0.5, 0.5)).to_c()
    for i in range(n):
        K, T = int(wl.K[i]), int(wl.T[i])
        u0 = samples[u_off:u_off + T * 2].reshape(T, 2)
        u_off += K * T * 2
        if i >= 16:
            continue
        c64, _, _ = oracle.rollout(A.MODEL_BICYCLE_SLIP, BicycleSlipDynamics().getParams(), ctrl._cost_arr[i],
                                   x0[i], u0, u0, sp, ctrl.constraints_, 2.0, 0.0, 1, T, 0.02,
                                   costmap=(cmap, 0.1, (0.0, 0.0)), fp64=True, state_dim=7)
        k0 = int(np.sum(wl.K[:i]))
        errs.append(abs(float(costs[k0]) - float(c64[0])) / abs(float(c64[0])))
    # final trajectory cost after `iters` MPPI iterations from zero sequences, surrogate (batched) vs analytic
    iters, nchk = 10, min(n, 16)
    ctrl.setControlSeqs([np.zeros((2, int(t)), np.float32) for t in wl.T])
    for _ in range(iters):
        ctrl.computeControl(wl.x0, 1)
    u_sur = ctrl.getControlSeqs()

    def cost64(i, u):
        ut = np.ascontiguousarray(np.asarray(u, np.float32).T)
        c64, _, _ = oracle.rollout(A.MODEL_BICYCLE_SLIP, BicycleSlipDynamics().getParams(), ctrl._cost_arr[i], x0[i],
                                   ut, ut, sp, ctrl.constraints_, 2.0, 0.0, 1, int(wl.T[i]), 0.02,
                                   costmap=(cmap, 0.1, (0.0, 0.0)), fp64=True, state_dim=7)
        return float(c64[0])

    rel = []
    for i in range(nchk):
        c = VanillaMPPIController(BicycleSlipDynamics(), W._slip_cost(cmap), None,
                                  GaussianDistribution(std_dev=(0.5, 0.5)), 0.02, 1, 2.0, 0.0, int(wl.T[i]),
                                  int(wl.K[i]), seed=i, stream=stream)
        for _ in range(iters):
            c.computeControl(x0[i], 1)
        u_ana = c.getControlSeq()
        c.close()
        rel.append(cost64(i, u_sur[i]) / cost64(i, u_ana) - 1.0)
    rel = np.array(rel)
    # batched analytic: the same instances in one handle with the analytic model in FP32 (no surrogate), timed like
    # `value` (device-resident solves, CUDA events on the handle's stream)
    import torch

    ana = BatchedMPPIController(BicycleSlipDynamics(), W._slip_cost(cmap), GaussianDistribution(std_dev=(0.5, 0.5)),
                                wl.K, wl.T, dt=0.02, max_iter=1, lambda_=2.0, seed=0, stream=stream)
    ana.computeControl(wl.x0, 1)
    ana.autotune(ROOT / "mppi_generic_vendor_gb300" / "_build" / "autotune_cache.json")
    ana.computeControl(wl.x0, 1)
    ana.enqueueSolve(1, 3)
    ana.synchronize()
    n_ana = max(20, min(400, args.steps))
    s = torch.cuda.ExternalStream(stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    ana.enqueueSolve(1, n_ana)
    e1.record(s)
    e1.synchronize()
    ana_s = e0.elapsed_time(e1) / 1e3 / n_ana
    ana.close()
    return {"plain_gpu": {"form": "analytic model, FP32, one controller per instance, solved in turn "
                                  "(computeControl with host buffers)",
                          "iters_per_s": 1.0 / plain_s,
                          "sample_steps_per_s": wl.sample_steps_per_iter / plain_s},
            "batched_analytic_gpu": {"form": "analytic model, FP32, all instances in one handle, device-resident "
                                             "solves (as value)",
                                     "iters_per_s": 1.0 / ana_s, "ms_per_iter": 1e3 * ana_s,
                                     "sample_steps_per_s": wl.sample_steps_per_iter / ana_s},
            "surrogate_cost_error": {"vs": "FP64 analytic rollout of each instance's nominal control sequence",
                                     "instances": len(errs), "median": float(np.median(errs)),
                                     "max": float(np.max(errs))},
            "final_trajectory_cost": {"vs": "MPPI on the analytic model, same instances, %d iterations from zero "
                                            "sequences; both final sequences costed by the FP64 analytic rollout"
                                            % iters,
                                      "instances": int(nchk), "median_rel": float(np.median(rel)),
                                      "max_rel": float(rel.max()),
                                      "within_1pct": int(np.sum(rel <= 0.01))}}


# ------------------------------------------------------------------------------------------------ CPU baseline
def cpu_baseline(name, seed, budget_s):
    """Time the CPU oracle (host rollout + weights + update, all threads) on a bounded sample of the workload."""
    import oracle
    from mppi_generic_vendor_gb300 import _abi as A
    from mppi_generic_vendor_gb300 import workloads as W

    threads = oracle.threads_default()
    rng = np.random.default_rng(seed)
    done_steps, elapsed, iters, inst_done = 0, 0.0, 0, 0
    if name in ("batched_di", "batched_di_gaussian"):
        colored = name == "batched_di"
        Ks, Ts, costs, x0 = W.batched_di_params(seed)
        cp = A.default_controller_params(native=False)
        cp.dt, cp.lambda_, cp.num_iters = 0.02, 1.0, 1
        sp = A.default_sampling_params(native=False)
        sp.std_dev[0] = sp.std_dev[1] = 0.5
        cc = A.default_constraints(native=False)
        for i in range(2):
            cc.lower[i], cc.upper[i] = -1.0, 1.0
        dyn = A.DoubleIntegratorParams(0.0)
        i = 0
        while elapsed < budget_s and i < len(Ks):
            K, T = int(Ks[i]), int(Ts[i])
            # the noise is prepared outside the timed region (the CPU path consumes the GPU's noise buffer)
            if colored:
                spec = rng.standard_normal(K * 2 * (T + 1) * 2).astype(np.float32)
                eps = oracle.colored_noise(spec, K, T, 2, [1.0, 1.0], decay=0.97, offset_t=1, threads=threads)
            else:
                eps = rng.standard_normal(K * T * 2).astype(np.float32)
            t0 = time.perf_counter()
            oracle.compute_control(A.MODEL_DOUBLE_INTEGRATOR, dyn, costs[i].getParams(), cp, sp, cc, K, T, 2, 4,
                                   x0[4 * i:4 * i + 4], eps, np.zeros((T, 2), np.float32), threads=threads)
            elapsed += time.perf_counter() - t0
            done_steps += K * T
            i += 1
        inst_done = i
        sample = f"{inst_done} of 256 instances (sum K*T = {done_steps}), one iteration each"
    elif name == "cartpole_rmppi":
        # one R-MPPI iteration on the host: the candidate evaluation (9 x 64 rollouts), the coupled rollout of both
        # systems (2 x 2048), weights and the weighted mean of both distributions, and the DDP gains of the
        # importance-sampler update.  The gains come from the engine's host DDP solver (mppi_ddp_feedback_gains),
        # the same host code the GPU arm runs between its launches.
        import ctypes as C

        K, T, N, J = 2048, 100, 9, 64
        dyn, cost = A.CartpoleParams(1, 1, 1, 9.81), A.CartpoleCostParams(10, 1, 100, 1, 0)
        sp = A.default_sampling_params(native=False)
        sp.std_dev[0] = 1.0
        cc = A.default_constraints(native=False)
        cc.lower[0], cc.upper[0] = -5.0, 5.0
        x0 = np.array([0.0, 0.0, 1.0, 0.0], np.float32)
        u = np.zeros((T, 1), np.float32)
        xt = np.repeat(x0[None], T, axis=0)
        cand = np.repeat(x0[None], N, axis=0)
        strides = np.zeros(N, np.int32)
        gains = np.zeros(T * 4, np.float32)
        eye4, eye1 = np.eye(4, dtype=np.float32), np.eye(1, dtype=np.float32)
        fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
        lo, hi = np.array([-5.0], np.float32), np.array([5.0], np.float32)
        while elapsed < budget_s and iters < 200:
            eps = rng.standard_normal(K * T).astype(np.float32)
            raw = (eps * np.float32(1.0) + np.tile(u.reshape(-1), K)).astype(np.float32)
            t0 = time.perf_counter()
            oracle.rmppi_eval(A.MODEL_CARTPOLE, dyn, cost, cand, strides, J, raw, u, sp, cc, 1.0, 0.0, K, T, 0.02)
            A.lib().mppi_ddp_feedback_gains(A.MODEL_CARTPOLE, C.cast(C.pointer(dyn), C.c_void_p), C.sizeof(dyn), T,
                                            0.02, fp(x0), fp(xt), fp(u), fp(eye4), fp(eye4), fp(eye1), 1, fp(lo),
                                            fp(hi), fp(gains))
            cn, cr, un, ur = oracle.rmppi_rollout(A.MODEL_CARTPOLE, dyn, cost, x0, x0, raw, raw, u, u,
                                                  np.tile(gains.reshape(T, 4), 1), sp, cc, 1.0, 0.0, 1000.0, K, T,
                                                  0.02, threads=threads)
            for c, smp in ((cn, un), (cr, ur)):
                w, _, n = oracle.weights(c, lambda_inv=np.float32(1.0))
                mean, _ = oracle.weighted_mean(w, np.float32(n), smp, K, T, 1)
            elapsed += time.perf_counter() - t0
            u = mean.astype(np.float32).reshape(T, 1)
            done_steps += 2 * K * T + N * J * T
            iters += 1
        sample = f"{iters} R-MPPI iterations of K=2048 x 2, T=100, 9 x 64 evaluation rollouts"
    elif name == "cartpole_tube":
        # one Tube-MPPI iteration on the host: the oracle's iteration over both distributions (rollouts, weights,
        # updates, the nominal-state decision, smoothing, state trajectories) and the feedback gains around the
        # nominal trajectory by the engine's host DDP solver, the same host code the GPU arm runs after its solve
        import ctypes as C

        K, T = 2048, 100
        dyn, cost = A.CartpoleParams(1, 1, 1, 9.81), A.CartpoleCostParams(10, 1, 100, 1, 0)
        cp = A.default_controller_params(native=False)
        cp.dt, cp.lambda_, cp.num_iters = 0.02, 1.0, 1
        cp.controller, cp.nominal_threshold = A.CONTROLLER_TUBE, 20.0
        sp = A.default_sampling_params(native=False)
        sp.std_dev[0] = 1.0
        cc = A.default_constraints(native=False)
        cc.lower[0], cc.upper[0] = -5.0, 5.0
        x0 = np.array([0.0, 0.0, 1.0, 0.0], np.float32)
        xn = x0.copy()
        ctl = np.zeros((2, T, 1), np.float32)
        gains = np.zeros(T * 4, np.float32)
        eye4, eye1 = np.eye(4, dtype=np.float32), np.eye(1, dtype=np.float32)
        fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
        lo, hi = np.array([-5.0], np.float32), np.array([5.0], np.float32)
        while elapsed < budget_s and iters < 200:
            e = rng.standard_normal(K * T).astype(np.float32)
            eps = np.concatenate([e, e])
            t0 = time.perf_counter()
            r = oracle.tube_compute_control(A.MODEL_CARTPOLE, dyn, cost, cp, sp, cc, K, T, 1, 4, x0, xn, eps, ctl,
                                            threads=threads)
            xt = np.ascontiguousarray(r["state_seq"][1])
            un = np.ascontiguousarray(r["control"][1])
            A.lib().mppi_ddp_feedback_gains(A.MODEL_CARTPOLE, C.cast(C.pointer(dyn), C.c_void_p), C.sizeof(dyn), T,
                                            0.02, fp(x0), fp(xt), fp(un), fp(eye4), fp(eye4), fp(eye1), 1, fp(lo),
                                            fp(hi), fp(gains))
            elapsed += time.perf_counter() - t0
            ctl = r["control"]
            done_steps += 2 * K * T
            iters += 1
        sample = f"{iters} Tube-MPPI iterations of K=2048 x 2, T=100 (sequences not slid)"
    elif name in ("slip_mlp", "batched_slip_mlp"):
        # the surrogate model in FP32 on the host (the oracle's restatement of the GPU rollout), same shapes
        params = surrogate_params()
        oracle.set_mlp(params)
        if name == "slip_mlp":
            shapes = [(16384, 100)]
        else:
            r = np.random.default_rng(seed + 5)
            shapes = list(zip(r.integers(2048, 16385, size=128).tolist(), r.choice([50, 100, 200], size=128).tolist()))
        cmap = (W.gaussian_bump_costmap(seed), 0.1, (0.0, 0.0))
        cp = A.default_controller_params(native=False)
        cp.dt, cp.lambda_, cp.num_iters = 0.02, 2.0, 1
        sp = A.default_sampling_params(native=False)
        sp.std_dev[0] = sp.std_dev[1] = 0.5
        cc = A.default_constraints(native=False)
        for i in range(2):
            cc.lower[i], cc.upper[i] = -1.0, 1.0
        dyn = A.BicycleSlipParams(1500.0, 2500.0, 1.2, 1.3, 8e4, 4000.0, 50.0, 0.5, 0.1, 1.0)
        cost = A.CostmapCostParams(1.0, 8.0, 1.0, 0.5, 2.0)
        x0 = np.array([25.0, 25.0, 0.3, 6.0, 0.0, 0.0, 0.0], np.float32)
        i = 0
        while elapsed < budget_s and iters < 200:
            K, T = shapes[i % len(shapes)]
            eps = rng.standard_normal(K * T * 2).astype(np.float32)
            t0 = time.perf_counter()
            oracle.compute_control(A.MODEL_BICYCLE_SLIP_MLP, dyn, cost, cp, sp, cc, K, T, 2, 7, x0, eps,
                                   np.zeros((T, 2), np.float32), costmap=cmap, threads=threads)
            elapsed += time.perf_counter() - t0
            done_steps += K * T
            iters += 1
            i += 1
        sample = f"{iters} MPPI iterations of the FP32 surrogate model ({'K=16384, T=100' if name == 'slip_mlp' else 'the first instances of the 128'})"
    else:
        wl_k, wl_t = (2048, 100) if name == "cartpole" else (16384, 100)
        if name == "cartpole":
            model, S, Cd = A.MODEL_CARTPOLE, 4, 1
            dyn, cost = A.CartpoleParams(1, 1, 1, 9.81), A.CartpoleCostParams(10, 1, 100, 1, 0)
            cmap = None
            lam, std = 1.0, (1.0,)
            lo, hi = [(-5.0, 5.0)], None
            x0 = np.array([0.0, 0.0, 1.0, 0.0], np.float32)
        else:
            model, S, Cd = A.MODEL_BICYCLE_COSTMAP, 4, 2
            dyn, cost = A.BicycleParams(2.5), A.CostmapCostParams(1.0, 8.0, 1.0, 0.0, 0.0)
            cmap = (W.gaussian_bump_costmap(seed), 0.1, (0.0, 0.0))
            lam, std = 2.0, (1.0, 0.3)
            lo = [(-3.0, 3.0), (-1.0, 1.0)]
            x0 = np.array([25.0, 25.0, 0.3, 4.0], np.float32)
        cp = A.default_controller_params(native=False)
        cp.dt, cp.lambda_, cp.num_iters = 0.02, lam, 1
        sp = A.default_sampling_params(native=False)
        for i, s in enumerate(std):
            sp.std_dev[i] = s
        cc = A.default_constraints(native=False)
        for i, (a, b) in enumerate(lo):
            cc.lower[i], cc.upper[i] = a, b
        u = np.zeros((wl_t, Cd), np.float32)
        while elapsed < budget_s and iters < 200:
            eps = rng.standard_normal(wl_k * wl_t * Cd).astype(np.float32)
            t0 = time.perf_counter()
            r = oracle.compute_control(model, dyn, cost, cp, sp, cc, wl_k, wl_t, Cd, S, x0, eps, u, costmap=cmap,
                                       threads=threads)
            elapsed += time.perf_counter() - t0
            u = r["control"]
            done_steps += wl_k * wl_t
            iters += 1
        sample = f"{iters} MPPI iterations of K={wl_k}, T={wl_t}"
    return {"value": done_steps / elapsed, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample,
            "seconds": round(elapsed, 3)}


# ------------------------------------------------------------------------------------------------ replicas
def max_over_ranks(value: float, dist=None) -> float:
    """The maximum of a per-rank number over all ranks (identity without a process group)."""
    if dist is None or not dist.is_initialized():
        return float(value)
    import torch

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: float, seconds_max: float, world_size: int) -> float:
    """Aggregate throughput of independent replicas: every rank processed `units_per_rank`, the job took the
    slowest rank's time."""
    return world_size * units_per_rank / seconds_max


# ------------------------------------------------------------------------------------------------ GPU arm
def run_gpu(args, ws, rank, local):
    import torch

    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from mppi_generic_vendor_gb300 import build as B

    B.build()
    stream = torch.cuda.Stream()
    surrogate = args.workload in ("slip_mlp", "batched_slip_mlp")
    wprec = args.precision or ("fp8" if args.workload == "batched_slip_mlp" else "bf16")
    wl = build_workload(args.workload, seed=0, stream=stream.cuda_stream, instances=args.instances,
                        precision=args.precision, params=surrogate_params(wprec) if surrogate else None)
    ctrl = wl.controller
    colored = args.workload == "batched_di"
    x0 = wl.x0
    # launch shapes chosen by the engine's autotuner (timed once, cached by model and instance shapes)
    ctrl.computeControl(x0, 1)
    ctrl.autotune(ROOT / "mppi_generic_vendor_gb300" / "_build" / "autotune_cache.json")
    # ---------------- device-resident throughput
    ctrl.computeControl(x0, 1)  # uploads x0 and the nominal controls, builds the graphs
    ctrl.enqueueSolve(1, max(args.warmup, 3))
    ctrl.synchronize()
    if args.steps is None:
        # enough steps for about 1.2 s of device time (the clock sampler sees several readings under load)
        p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        p0.record(stream)
        ctrl.enqueueSolve(1, 3)
        p1.record(stream)
        p1.synchronize()
        args.steps = int(min(5000, max(20, np.ceil(1200.0 / (p0.elapsed_time(p1) / 3)))))
        args.steps = int(max_over_ranks(args.steps, dist))  # every rank times the same number of steps
    clocks = ClockSampler(local)
    clocks.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    # the profiler range (a no-op without a profiler) marks the timed steps for a launch list under
    # `ncu --profile-from-start off`
    torch.cuda.profiler.start()
    with torch.cuda.stream(stream):
        e0.record(stream)
        ctrl.enqueueSolve(1, args.steps)
        e1.record(stream)
    torch.cuda.synchronize()
    torch.cuda.profiler.stop()
    ms = e0.elapsed_time(e1)
    clk = clocks.stop()
    ms = max_over_ranks(ms, dist)
    steps_per_iter = wl.sample_steps_per_iter
    iters = args.steps * wl.num_iters
    value = whole_job_rate(steps_per_iter * iters, ms / 1e3, ws)
    iters_per_s = iters / (ms / 1e3)
    kernels = ctrl.kernelsPerCompute()
    # ---------------- per-kernel timing and roofline
    kms = [float(v) for v in ctrl.timeKernels(1, reps=max(3, min(10, args.steps)))]
    names = ["sampler", "rollout", "update"]
    abytes = algorithmic_bytes(wl, colored)
    dom = int(np.argmax(kms))
    peak, peak_kind = measured_peaks()
    achieved = abytes[names[dom]] / (kms[dom] * 1e-3) / 1e9
    if surrogate:
        # the surrogate rollout is a chain of tensor-core GEMMs: FLOPs against the bf16 peak
        dom = 1
        peak, peak_kind = measured_peaks("tensor")
        achieved = MLP_FLOPS * steps_per_iter / (kms[1] * 1e-3) / 1e12
    sfu = None
    sfile = ROOT / "profiles" / "sfu.json"
    if surrogate and sfile.exists():
        try:
            sj = json.loads(sfile.read_text())
            ent = sj.get(wl.name)
            if ent:
                # the unit that binds the surrogate rollout: every hidden activation is one MUFU tanh
                ach = float(ent["mufu_ops_per_sample_step"]) * steps_per_iter / (kms[1] * 1e-3)
                peak_sfu = float(sj["peak_mufu_ops_per_s"])
                sfu = {"unit": "MUFU ops/s", "achieved": ach, "peak": peak_sfu, "frac": ach / peak_sfu,
                       "ops_per_sample_step": float(ent["mufu_ops_per_sample_step"]),
                       "peak_kind": "measured (tests/cuda/sfu_throughput.cu)",
                       "time": "rollout incl. judge kernels"}
        except Exception:
            sfu = None
    traffic = None
    tfile = ROOT / "profiles" / "dram_traffic.json"
    if tfile.exists():
        try:
            tj = json.loads(tfile.read_text())
            ent = tj.get(wl.name, {}).get(names[dom])
            if ent:
                traffic = float(ent["bytes_per_unit"]) * (wl.control_floats if ent["unit"] == "control_float"
                                                          else steps_per_iter)
        except Exception:
            traffic = None
    # ---------------- end to end through computeControl with host buffers
    for _ in range(max(args.warmup, 3)):
        ctrl.computeControlFlat(x0, 1)
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ctrl.computeControlFlat(x0, 1)
        u = ctrl.control_flat()
    e2e_s = max_over_ranks(time.perf_counter() - t0, dist)
    e2e = whole_job_rate(steps_per_iter * iters, e2e_s, ws)
    n_inst = wl.controller.num_instances
    h2d = 4 * (n_inst * wl.state_dim + int(np.sum(wl.T)) * wl.control_dim)
    d2h = 4 * int(np.sum(wl.T)) * wl.control_dim + 8 * n_inst + 24 * n_inst + u.nbytes
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded; shapes of the benchmark configuration)",
        "config": config_of(wl, ws),
        "iters_per_s": iters_per_s,
        "launch_config": {**dict(zip(["rollout_samples_per_cta", "rollout_time_chunk", "reduction_samples_per_cta"],
                                     ctrl.launchConfig())),
                          "rollout_mode": ROLLOUT_MODE_NAMES[ctrl.rolloutMode()[0]]},
        "kernel_ms": {n: float(v) for n, v in zip(names, kms)},
        "roofline": ({"bound": "hbm", "kernel": names[dom], "achieved": achieved, "peak": peak, "unit": "GB/s",
                      "frac": achieved / peak, "peak_kind": peak_kind, "traffic": traffic,
                      "algorithmic_bytes": abytes[names[dom]]} if not surrogate else
                     {"bound": "tensor", "kernel": "rollout (surrogate + judge)", "achieved": achieved, "peak": peak,
                      "unit": "TFLOP/s", "frac": achieved / peak, "peak_kind": peak_kind, "traffic": traffic,
                      "algorithmic_flops": MLP_FLOPS * steps_per_iter, "binding_unit_sfu": sfu}),
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "iters_per_s": ws * iters / e2e_s},
        "gpu_launches": kernels * args.steps,
    }
    if clk:
        line["clocks"] = clk
    if surrogate:
        line["dtype"] = {"bf16": "bf16 weights, f32 accumulate/state", "fp8": "fp8-e4m3 weights, f32 accumulate/state",
                         "fp32": "f32"}[wl.description["precision"]]
        line.update(surrogate_extras(args, wl, stream.cuda_stream))
        # the metric's comparison: surrogate + batched against the plain GPU form (and against batching the
        # analytic model, which needs no surrogate)
        line["speedup"] = {
            "vs_plain_gpu": iters_per_s / line["plain_gpu"]["iters_per_s"],
            "vs_plain_gpu_e2e": line["e2e"]["iters_per_s"] / line["plain_gpu"]["iters_per_s"],
            "vs_batched_analytic_gpu": iters_per_s / line["batched_analytic_gpu"]["iters_per_s"]}
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args.workload, 0, args.cpu_seconds)
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctrl.close()
    if dist:
        dist.destroy_process_group()


def run_host_iterated(args, ws, rank, local):
    """A host-iterated controller's iteration through its public calls with host buffers, timed end to end: R-MPPI
    (updateImportanceSamplingControl + computeControl) or Tube-MPPI (computeControl + computeFeedback + a one-step
    slide); the solve's kernels (sampler, rollout, weights + update) timed with CUDA events on its stream."""
    import torch

    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from mppi_generic_vendor_gb300 import build as B

    B.build()
    stream = torch.cuda.Stream()
    wl = build_workload(args.workload, seed=0, stream=stream.cuda_stream)
    ctrl, x0 = wl.controller, wl.x0
    tube = args.workload == "cartpole_tube"

    def iteration():
        if tube:
            # TubeMPPIController in a receding-horizon loop: solve, feedback gains, slide by one step
            ctrl.computeControl(x0, 1)
            ctrl.computeFeedback(x0)
            u = ctrl.getControlSeq()
            ctrl.slideControlSequence(1)
            return u
        ctrl.updateImportanceSamplingControl(x0, 1)
        ctrl.computeControl(x0, 1)
        return ctrl.getControlSeq()

    for _ in range(max(args.warmup, 3)):
        iteration()
    if args.steps is None:
        t0 = time.perf_counter()
        for _ in range(3):
            iteration()
        args.steps = int(min(5000, max(20, np.ceil(1.2 / ((time.perf_counter() - t0) / 3)))))
        args.steps = int(max_over_ranks(args.steps, dist))
    clocks = ClockSampler(local)
    clocks.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        u = iteration()
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - t0, dist)
    clk = clocks.stop()
    steps_per_iter = wl.sample_steps_per_iter
    e2e = whole_job_rate(steps_per_iter * args.steps, e2e_s, ws)
    kms = [float(v) for v in ctrl.timeKernels(1, reps=10)]
    K, T = int(wl.K[0]), int(wl.T[0])
    S, Cd = wl.state_dim, wl.control_dim
    if tube:
        # the rollout of both distributions reads their samples and writes 2 K costs
        abytes = 2 * (4 * K * T * Cd) + 8 * K
        kname = "rollout of both distributions (one T-step chain per sample)"
        h2d = 4 * (2 * S + 2 * T * Cd)
        d2h = 4 * 2 * T * Cd + u.nbytes
    else:
        # the coupled rollout reads and writes both distributions' samples, writes 2 K costs and reads the gains
        abytes = 2 * (8 * K * T * Cd) + 8 * K + 4 * T * Cd * S
        kname = "rmppi_rollout_kernel (two lanes per sample, latency-bound chain)"
        h2d = 4 * (2 * S + 2 * T * Cd + T * Cd * S) + 4 * S
        d2h = 4 * 2 * T * Cd + 4 * 9 * 64 + u.nbytes
    peak, peak_kind = measured_peaks()
    achieved = abytes / (kms[1] * 1e-3) / 1e9
    line = {
        "metric": METRIC, "value": e2e, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * e2e_s / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded; shapes of the benchmark configuration)",
        "config": config_of(wl, ws), "host_iterated": True,
        "iters_per_s": args.steps / e2e_s,
        "kernel_ms": {"sampler": kms[0], "rollout": kms[1], "update": kms[2]},
        "roofline": {"bound": "hbm", "kernel": kname,
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": peak_kind, "traffic": None, "algorithmic_bytes": abytes},
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "iters_per_s": ws * args.steps / e2e_s},
        # the solve's kernels, plus for R-MPPI the update's sampler, candidate evaluation and counter bump
        "gpu_launches": (ctrl.kernelsPerCompute() + (0 if tube else 3)) * args.steps,
    }
    if clk:
        line["clocks"] = clk
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args.workload, 0, args.cpu_seconds)
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctrl.close()
    if dist:
        dist.destroy_process_group()


def run_reference(args, ws, rank):
    if rank != 0:
        return
    _SURROGATE["cpu_only"] = True
    if args.steps is None:
        args.steps = 10
    per_step = max(1.0, args.cpu_seconds / max(1, args.steps + args.warmup))
    for _ in range(args.warmup):
        cpu_baseline(args.workload, 0, per_step)
    vals = []
    t0 = time.perf_counter()
    last = None
    for _ in range(args.steps):
        last = cpu_baseline(args.workload, 0, per_step)
        vals.append(last["value"])
    total = time.perf_counter() - t0
    v = float(np.mean(vals))
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded; shapes of the benchmark configuration)",
            "config": config_of(build_workload(args.workload, 0, 0, instances=args.instances, precision=args.precision,
                                               describe_only=True), ws), "impl": "reference",
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": last["cores"], "kind": "port",
                             "sample": last["sample"]},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    ws, rank, local = dist_env()
    if args.impl == "reference":
        run_reference(args, ws, rank)
        return
    if args.workload in ("cartpole_rmppi", "cartpole_tube"):
        run_host_iterated(args, ws, rank, local)
        return
    run_gpu(args, ws, rank, local)


if __name__ == "__main__":
    main()
