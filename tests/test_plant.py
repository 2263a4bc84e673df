"""BasePlant (base_plant.hpp:24-620) host logic on the CPU with a stand-in controller: state / control timing,
optimisation stride from robot time, sliding, parameter hand-over between threads, NaN guards, the paced loop."""
import threading
import time

import numpy as np
import pytest

from mppi_generic_vendor_gb300.plant import BasePlant


class FakeController:
    """Records the calls the plant makes; its control sequence is u[0, t] = t + solves (a ramp shifted per solve)."""

    def __init__(self, T=50, dt=0.02):
        self.T, self.dt, self.calls, self.solves = T, dt, [], 0
        self.nan = False

    def getDt(self):
        return self.dt

    def getNumTimesteps(self):
        return self.T

    def computeControl(self, state, stride):
        self.calls.append(("compute", np.array(state), stride))
        self.solves += 1

    def slideControlSequence(self, steps):
        self.calls.append(("slide", steps))

    def getControlSeq(self):
        u = np.arange(self.T, dtype=np.float32)[None, :] + self.solves
        return u * np.nan if self.nan else u

    def getTargetStateSeq(self):
        return np.zeros((4, self.T), np.float32)

    def getFreeEnergyStatistics(self):
        return {"freeEnergyMean": 1.0}

    def updateCostParams(self, p):
        self.calls.append(("cost", p))

    def updateDynamicsParams(self, p):
        self.calls.append(("dyn", p))

    def setParams(self, p):
        self.calls.append(("params", p))

    def setSamplingParams(self, p):
        self.calls.append(("sampler", p))


class RecordingPlant(BasePlant):
    def __init__(self, controller, **kw):
        super().__init__(controller, **kw)
        self.published, self.nominal, self.stats = [], [], []

    def pubControl(self, u):
        self.published.append(np.array(u))

    def pubNominalState(self, s):
        self.nominal.append(np.array(s))

    def pubFreeEnergyStatistics(self, stats):
        self.stats.append(stats)

    def checkStatus(self):
        return 0

    def getCurrentTime(self):
        return time.perf_counter()

    def getPoseTime(self):
        return self.getStateTime()


def alive():
    e = threading.Event()
    e.set()
    return e


def test_first_solve_then_control_interpolated_in_time():
    c = FakeController()
    plant = RecordingPlant(c)
    plant.updateState(np.zeros(4), 0.0)
    assert plant.published == []  # no solution yet
    assert plant.runControlIteration(alive())
    assert c.calls[0][0] == "compute" and c.calls[0][2] == 0  # first solve: stride 0, no slide
    plant.updateState(np.ones(4), 0.05)  # 2.5 steps after the solved state
    assert len(plant.published) == 1
    assert np.allclose(plant.published[0], [2.5 + 1.0])  # ramp of solve 1 at step 2.5
    plant.updateState(np.ones(4), 0.05 + 50 * 0.02)  # beyond the horizon: nothing published
    assert len(plant.published) == 1


@pytest.mark.parametrize("robot_dt,target,expect", [(0.05, 1, 3), (0.03, 1, 2), (0.01, 1, 1), (0.02, 4, 4),
                                                    (0.07, 1, 4)])
def test_optimization_stride_follows_robot_time(robot_dt, target, expect):
    """stride = max(round(robot time since the last solve / dt), target stride), rounding halves away from zero as
    std::round does; the nominal sequence slides by it before the solve."""
    c = FakeController()
    plant = RecordingPlant(c, optimization_stride=target)
    plant.updateState(np.zeros(4), 1.0)
    plant.runControlIteration(alive())
    plant.updateState(np.zeros(4), 1.0 + robot_dt)
    assert plant.runControlIteration(alive())
    assert plant.getLastOptimizationStride() == expect
    assert ("slide", expect) in c.calls
    assert c.calls[-1][0] == "compute" and c.calls[-1][2] == expect


def test_waits_for_a_new_state_and_gives_up_bounded():
    c = FakeController()
    plant = RecordingPlant(c)
    plant.updateState(np.zeros(4), 0.0)
    assert plant.runControlIteration(alive())
    t0 = time.perf_counter()
    assert not plant.runControlIteration(alive(), max_wait_s=0.05)  # same state time: nothing to optimise
    assert time.perf_counter() - t0 < 2.0
    assert sum(1 for k in c.calls if k[0] == "compute") == 1
    stopped = threading.Event()
    assert not plant.runControlIteration(stopped)


def test_parameters_hand_over_between_threads():
    c = FakeController()
    plant = RecordingPlant(c)
    t = threading.Thread(target=lambda: (plant.setCostParams("cost-1"), plant.setDynamicsParams("dyn-1"),
                                         plant.setSamplerParams("sampler-1"), plant.setControllerParams("ctl-1")))
    t.start()
    t.join()
    assert plant.hasNewCostParams() and plant.hasNewDynamicsParams()
    plant.updateState(np.zeros(4), 0.0)
    plant.runControlIteration(alive())
    kinds = [k[0] for k in c.calls]
    assert kinds.index("cost") < kinds.index("compute") and kinds.index("dyn") < kinds.index("compute")
    assert "sampler" in kinds and "params" in kinds
    assert not plant.hasNewCostParams() and not plant.updateParameters()


def test_nan_guards():
    c = FakeController()
    plant = RecordingPlant(c)
    plant.updateState(np.array([0.0, np.nan, 0.0, 0.0]), 0.0)
    assert not plant.runControlIteration(alive())  # a NaN state is not optimised from
    assert c.calls == []
    plant.updateState(np.zeros(4), 0.1)
    c.nan = True
    with pytest.raises(RuntimeError):
        plant.runControlIteration(alive())


def test_paced_control_loop_runs_and_stops():
    c = FakeController()
    plant = RecordingPlant(c, hz=200)
    plant.updateState(np.zeros(4), 0.0)
    plant.start()
    t = 0.0
    for _ in range(20):
        t += 0.02
        plant.updateState(np.zeros(4), t)
        time.sleep(0.005)
    plant.stop()
    n = plant.num_iter_
    assert n >= 3 and len(plant.stats) == n
    assert plant.getAvgLoopTime() >= plant.getAvgOptimizationTime() >= 0.0
    time.sleep(0.05)
    assert plant.num_iter_ == n  # stopped
