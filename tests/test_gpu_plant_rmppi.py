"""The Python BasePlant (mppi_generic_vendor_gb300/plant.py) driving the GPU's RobustMPPIController with the DDP
feedback (base_plant.hpp:466-595 with RobustMPPIController): a simulated double integrator reports its state every
5 ms of robot time, the plant re-optimises every 20 ms.  Each iteration runs the importance-sampler update before
the (no-op) slide, the solve, and the feedback state of the solve; the published control is getCurrentControl (the
real system's control plus the interpolated feedback against the nominal state, constrained).  In 4 s of robot time
the robot must close most of its distance to the goal (2.83 to under 1.0), the controls stay inside their range and
the plant must hold non-zero gains."""
import numpy as np
import pytest

from mppi_generic_vendor_gb300 import (DDPFeedback, DDPParams, DoubleIntegratorDynamics, DoubleIntegratorObstacleCost,
                                       GaussianDistribution, RobustMPPIController)
from mppi_generic_vendor_gb300.plant import BasePlant

pytestmark = pytest.mark.gpu


class DIPlant(BasePlant):
    def __init__(self, controller):
        super().__init__(controller, hz=50, optimization_stride=1)
        self.now = 0.0
        self.u = np.zeros(2, np.float32)
        self.published = []

    def pubControl(self, u):
        self.u = np.asarray(u, np.float32)
        self.published.append(self.u.copy())

    def pubNominalState(self, s):
        pass

    def pubFreeEnergyStatistics(self, stats):
        pass

    def checkStatus(self):
        return 0

    def getCurrentTime(self):
        return self.now

    def getPoseTime(self):
        return self.now


def test_python_plant_drives_robust_mppi():
    import threading

    dt = 0.02
    dyn = DoubleIntegratorDynamics()
    dyn.setControlRanges([(-2.0, 2.0), (-2.0, 2.0)])
    cost = DoubleIntegratorObstacleCost(goal=(1.0, 1.0, 0.0, 0.0), coeff=(1.0, 1.0, 0.5, 0.5), terminal_coeff=5.0)
    fb = DDPFeedback(dyn, dt)
    fb.setParams(DDPParams(np.diag([4.0, 4.0, 1.0, 1.0]), None, np.diag([0.5, 0.5]), 1))
    ctrl = RobustMPPIController(dyn, cost, fb, GaussianDistribution(std_dev=(1.0, 1.0)), dt, 1, 1.0, 0.0, 1000.0, 50,
                                1024, num_candidate_nominal_states=5, num_eval_samples_per_candidate=32)
    plant = DIPlant(ctrl)
    alive = threading.Event()
    alive.set()
    x = np.array([-1.0, -1.0, 0.0, 0.0], np.float64)
    plant.updateState(x.astype(np.float32), 0.0)
    h = 0.005
    for _ in range(200):
        assert plant.runControlIteration(alive)
        for _ in range(4):
            u = plant.u.astype(np.float64)
            x = x + h * np.array([x[2], x[3], u[0], u[1]])
            plant.now += h
            plant.updateState(x.astype(np.float32), plant.now)
    d = float(np.hypot(x[0] - 1.0, x[1] - 1.0))
    assert d < 1.0, d
    pub = np.array(plant.published)
    assert len(pub) >= 600 and np.all(np.abs(pub) <= 2.0 + 1e-6)
    fs = plant.getFeedbackState()
    assert fs is not None and np.any(fs.fb_gain_traj_ != 0)
    assert plant.getAvgFeedbackTime() >= 0.0
    assert 0 <= ctrl.getBestIndex() < 5
    # the nominal state the plant's importance-sampler updates chose starts the target trajectory
    assert np.array_equal(ctrl.getNominalState(), ctrl.getTargetStateSeq()[:, 0])
    ctrl.close()
