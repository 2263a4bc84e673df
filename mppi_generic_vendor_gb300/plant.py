"""Receding-horizon driver with the reference's BasePlant interface (include/mppi/core/base_plant.hpp:24-620).

A plant owns a controller and runs it against a robot: a state estimator calls ``updateState(state, time)``, which
publishes the control for that time from the latest solution; ``runControlLoop`` re-optimises at ``hz`` from the
newest state, sliding the nominal sequence by the robot time that passed.  Subclasses provide the robot side
(``pubControl``, ``pubNominalState``, ``pubFreeEnergyStatistics``, ``checkStatus``, ``getCurrentTime``,
``getPoseTime``), as in the reference.  Parameter updates arrive from any thread and are applied between
optimisations.  With the controller's feedback on, each solve is followed by the DDP feedback computation, and the
published control is the controller's getCurrentControl: the nominal control at the requested time plus the
feedback against the interpolated nominal state, constrained.

The controller is any object with the ``VanillaMPPIController`` methods used here (``computeControl``,
``getControlSeq``, ``getTargetStateSeq``, ``slideControlSequence``, ``getFreeEnergyStatistics``, ``getDt``,
``getNumTimesteps`` and, for parameter updates, ``updateDynamicsParams``, ``updateCostParams``, ``setParams``,
``setSamplingParams``).  A controller without ``getCurrentControl`` (and the feedback methods) has the nominal
sequence interpolated at the requested time published.
"""
from __future__ import annotations

import math
import threading
import time

import numpy as np


class BasePlant:
    def __init__(self, controller, hz: int = 10, optimization_stride: int = 1):
        self.controller_ = controller
        self.hz_ = int(hz)
        self.optimization_stride_ = int(optimization_stride)
        self.last_optimization_stride_ = 0
        self.debug_mode_ = False
        self._guard = threading.Lock()
        self._param_guard = threading.Lock()
        self._pending = {}  # kind -> parameters waiting for updateParameters
        self.state_ = None
        self.state_time_ = 0.0
        self.has_received_state_ = False
        self.last_used_state_update_time_ = 0.0
        self.state_traj_ = None
        self.control_traj_ = None
        self.feedback_state_ = None
        self.feedback_duration_ = 0.0
        self.avg_feedback_time_ms_ = 0.0
        self.num_iter_ = 0
        self.status_ = 0
        self.optimization_duration_ = 0.0
        self.optimize_loop_duration_ = 0.0
        self.sleep_duration_ = 0.0
        self.avg_optimize_time_ms_ = 0.0
        self.avg_loop_time_ms_ = 0.0
        self.avg_sleep_time_ms_ = 0.0

    # ---- robot side (BasePlant's pure virtual functions)
    def pubControl(self, u):
        raise NotImplementedError

    def pubNominalState(self, s):
        raise NotImplementedError

    def pubFreeEnergyStatistics(self, stats):
        raise NotImplementedError

    def checkStatus(self) -> int:
        raise NotImplementedError

    def getCurrentTime(self) -> float:
        raise NotImplementedError

    def getPoseTime(self) -> float:
        raise NotImplementedError

    # ---- state and timing
    def getStateTime(self) -> float:
        return self.state_time_

    def getState(self):
        with self._guard:
            return None if self.state_ is None else self.state_.copy()

    def setDebugMode(self, mode: bool):
        self.debug_mode_ = bool(mode)

    def getHz(self) -> int:
        return self.hz_

    def setHz(self, hz: int):
        self.hz_ = int(hz)

    def getTargetOptimizationStride(self) -> int:
        return self.optimization_stride_

    def setTargetOptimizationStride(self, stride: int):
        self.optimization_stride_ = int(stride)

    def getLastOptimizationStride(self) -> int:
        return self.last_optimization_stride_

    def getAvgOptimizationTime(self) -> float:
        return self.avg_optimize_time_ms_

    def getAvgLoopTime(self) -> float:
        return self.avg_loop_time_ms_

    def _interpolate(self, traj, steps: float):
        """Column of a (dim, T) trajectory at fractional step `steps` (linear between steps, held at the ends)."""
        T = traj.shape[1]
        i = min(max(int(math.floor(steps)), 0), T - 1)
        j = min(i + 1, T - 1)
        a = min(max(steps - i, 0.0), 1.0)
        return (1.0 - a) * traj[:, i] + a * traj[:, j]

    def updateState(self, state, t: float):
        """BasePlant::updateState (base_plant.hpp:289-321): store the estimate and, once a solution exists and `t`
        lies inside its horizon after the state it was computed from, publish the control for `t`."""
        with self._guard:
            self.state_ = np.asarray(state, dtype=np.float32).copy()
            self.state_time_ = float(t)
            self.has_received_state_ = True
            if self.num_iter_ == 0:
                return
            t0 = self.last_used_state_update_time_
            u_traj, s_traj, fb_state = self.control_traj_, self.state_traj_, self.feedback_state_
            x = self.state_
        c = self.controller_
        dt = c.getDt()
        since = t - t0
        if since > 0 and t0 <= t < t0 + dt * c.getNumTimesteps():
            if hasattr(c, "getCurrentControl"):
                target = c.interpolateState(s_traj, since)
                self.pubControl(c.getCurrentControl(x, since, target, u_traj, fb_state))
                if self.debug_mode_:
                    self.pubNominalState(target)
            else:
                self.pubControl(self._interpolate(u_traj, since / dt))
                if self.debug_mode_:
                    self.pubNominalState(self._interpolate(s_traj, since / dt))

    # ---- parameter updates from any thread (set*Params, then applied by updateParameters)
    def setDynamicsParams(self, params):
        with self._param_guard:
            self._pending["dynamics"] = params

    def setCostParams(self, params):
        with self._param_guard:
            self._pending["cost"] = params

    def setControllerParams(self, params):
        with self._param_guard:
            self._pending["controller"] = params

    def setSamplerParams(self, sampler):
        with self._param_guard:
            self._pending["sampler"] = sampler

    def hasNewDynamicsParams(self) -> bool:
        return "dynamics" in self._pending

    def hasNewCostParams(self) -> bool:
        return "cost" in self._pending

    def hasNewControllerParams(self) -> bool:
        return "controller" in self._pending

    def hasNewSamplerParams(self) -> bool:
        return "sampler" in self._pending

    def updateParameters(self) -> bool:
        """BasePlant::updateParameters (base_plant.hpp:412-451): hand pending parameters to the controller."""
        with self._param_guard:
            pending, self._pending = self._pending, {}
        c = self.controller_
        if "cost" in pending:
            c.updateCostParams(pending["cost"])
        if "dynamics" in pending:
            c.updateDynamicsParams(pending["dynamics"])
        if "controller" in pending:
            c.setParams(pending["controller"])
        if "sampler" in pending:
            c.setSamplingParams(pending["sampler"])
        return bool(pending)

    # ---- optimisation
    def setSolution(self, state_seq, control_seq, timestamp: float, feedback_state=None):
        with self._guard:
            self.last_used_state_update_time_ = float(timestamp)
            self.state_traj_ = state_seq
            self.control_traj_ = control_seq
            self.feedback_state_ = feedback_state
            self.num_iter_ += 1

    def getFeedbackState(self):
        return self.feedback_state_

    def getAvgFeedbackTime(self) -> float:
        return self.avg_feedback_time_ms_

    def runControlIteration(self, is_alive: threading.Event, poll_s: float = 5e-5, max_wait_s: float = 1.0) -> bool:
        """BasePlant::runControlIteration (base_plant.hpp:466-595): wait (bounded) for a state newer than the last
        one optimised from, apply pending parameters, slide the nominal sequence by the robot time that passed (at
        least the target stride) and optimise.  Returns False when nothing was optimised."""
        loop_start = time.perf_counter()
        if not is_alive.is_set():
            return False
        waited = 0.0
        while is_alive.is_set():
            first = self.num_iter_ == 0 and self.has_received_state_
            if first or (self.has_received_state_ and self.getStateTime() != self.last_used_state_update_time_):
                break
            if waited >= max_wait_s:
                return False
            time.sleep(poll_s)
            waited += poll_s
        if not is_alive.is_set():
            return False
        self.updateParameters()
        with self._guard:
            state = self.state_.copy()
            state_time = self.state_time_
        if not np.all(np.isfinite(state)):
            return False
        self.status_ = self.checkStatus()
        c = self.controller_
        if self.num_iter_ == 0:
            self.last_optimization_stride_ = 0
        else:
            robot_dt = state_time - self.last_used_state_update_time_
            steps = robot_dt / c.getDt()  # rounded half away from zero, as std::round
            self.last_optimization_stride_ = max(int(math.copysign(math.floor(abs(steps) + 0.5), steps)),
                                                 self.optimization_stride_)
        if 0 < self.last_optimization_stride_ < c.getNumTimesteps():
            # the robust controller's importance sampler first (a no-op for the others), then the slide
            if getattr(c, "updateImportanceSamplingControl", None) is not None:
                c.updateImportanceSamplingControl(state, self.last_optimization_stride_)
            c.slideControlSequence(self.last_optimization_stride_)
        opt_start = time.perf_counter()
        c.computeControl(state, self.last_optimization_stride_)
        stats = c.getFreeEnergyStatistics()
        u = np.asarray(c.getControlSeq())
        if not np.all(np.isfinite(u)):
            raise RuntimeError("control trajectory inside the plant has a NaN")
        s = np.asarray(c.getTargetStateSeq())
        if not np.all(np.isfinite(s)):
            raise RuntimeError("state trajectory inside the plant has a NaN")
        self.optimization_duration_ = (time.perf_counter() - opt_start) * 1e3
        fb_start = time.perf_counter()
        fb_state = None
        if getattr(c, "getFeedbackEnabled", None) is not None and c.getFeedbackEnabled():
            c.computeFeedback(state)
            fb_state = c.getFeedbackState()
        self.feedback_duration_ = (time.perf_counter() - fb_start) * 1e3
        self.setSolution(s, u, state_time, fb_state)
        self.pubFreeEnergyStatistics(stats)
        if getattr(c, "computeFeedbackPropagatedStateSeq", None) is not None:
            c.computeFeedbackPropagatedStateSeq()
        n = self.num_iter_
        self.avg_optimize_time_ms_ += (self.optimization_duration_ - self.avg_optimize_time_ms_) / n
        self.avg_feedback_time_ms_ += (self.feedback_duration_ - self.avg_feedback_time_ms_) / n
        self.optimize_loop_duration_ = (time.perf_counter() - loop_start) * 1e3
        self.avg_loop_time_ms_ += (self.optimize_loop_duration_ - self.avg_loop_time_ms_) / n
        return True

    def runControlLoop(self, is_alive: threading.Event):
        """BasePlant::runControlLoop (base_plant.hpp:597-620): optimise at hz until is_alive is cleared, sleeping
        the rest of each period."""
        period = 1.0 / max(self.hz_, 1)
        while is_alive.is_set():
            start = time.perf_counter()
            ran = self.runControlIteration(is_alive)
            rest = period - (time.perf_counter() - start)
            self.sleep_duration_ = max(rest, 0.0) * 1e3
            if ran and self.num_iter_:
                self.avg_sleep_time_ms_ += (self.sleep_duration_ - self.avg_sleep_time_ms_) / self.num_iter_
            if rest > 0:
                time.sleep(rest)

    def start(self) -> threading.Event:
        """Run runControlLoop on a thread; clear the returned event to stop it (join with stop())."""
        alive = threading.Event()
        alive.set()
        self._thread = threading.Thread(target=self.runControlLoop, args=(alive,), daemon=True)
        self._thread.start()
        self._alive = alive
        return alive

    def stop(self):
        if getattr(self, "_alive", None) is not None:
            self._alive.clear()
            self._thread.join()
            self._alive = None
