"""TubeMPPIController on the GPU against the oracle's restatement (tube_mppi_controller.cu:158-349): the two
sampling distributions [D = 2][K][T][C] (actual and nominal system) given the same injected noise, the nominal-state
decision, the smoothing of the nominal sequence only, both state trajectories, and the nominal state's advance by
a slide."""
import numpy as np
import pytest

import _parity
import oracle
from mppi_generic_vendor_gb300 import DoubleIntegratorDynamics, DoubleIntegratorObstacleCost, GaussianDistribution
from mppi_generic_vendor_gb300 import TubeMPPIController

pytestmark = pytest.mark.gpu


def _tube(K, T, threshold, same_noise=True):
    dyn = DoubleIntegratorDynamics()
    dyn.setControlRanges([(-2.0, 2.0), (-2.0, 2.0)])
    cost = DoubleIntegratorObstacleCost(goal=(1.5, -0.5, 0.0, 0.0), coeff=(1.0, 1.0, 0.1, 0.1), terminal_coeff=5.0,
                                        obstacles=[(0.7, 0.0, 0.3)], obstacle_cost=100.0)
    sampler = GaussianDistribution(std_dev=(0.6, 0.6), use_same_noise_for_all_distributions=same_noise)
    return TubeMPPIController(dyn, cost, None, sampler, 0.02, 1, 1.0, 0.0, T, K, nominal_threshold=threshold)


def _draw(rng, K, T, same_noise):
    """Injected noise for both distributions: with use_same_noise_for_all_distributions the second reads the first's
    (generateSamples copies one draw, gaussian.cu:378-390), so the oracle gets the first half twice."""
    if same_noise:
        e = rng.standard_normal(K * T * 2).astype(np.float32)
        return np.concatenate([e, e])
    return rng.standard_normal(2 * K * T * 2).astype(np.float32)


def _check(ctrl, ref, K, T):
    costs = ctrl.sample_costs().reshape(2, K)
    assert np.array_equal(costs.view(np.uint32), ref["costs"].view(np.uint32))
    bn, _ = ctrl.baseline_normalizer()
    assert bn[0, 0] == ref["baselines"][0] and bn[1, 0] == ref["baselines"][1]
    assert ctrl.nominalStateUsed() == ref["nominal_used"]
    d = [dict(control=ref["control"][i], weights=ref["weights"][i], normalizer=ref["normalizers"][i],
              samples=ref["samples"][i]) for i in range(2)]
    # the actual sequence is the (unsmoothed) update of distribution 0; the nominal one the smoothed update of
    # distribution 1, or of distribution 0 when the nominal system took over the actual one
    _parity.check_control(ctrl.getActualControlSeq().T, d[0], K, T, 2, smoothed=False)
    src = d[1] if ref["nominal_used"] else d[0]
    _parity.check_control(ctrl.getNominalControlSeq().T, dict(src, control=ref["control"][1]), K, T, 2)
    states = ctrl.getTargetStateSeqs()
    # the state trajectories follow from the sequences (host steps on both sides); compared where the sequences are
    # bit-identical, and otherwise within the sequences' tolerance carried through T steps
    for i in range(2):
        assert np.allclose(states[i].T, ref["state_seq"][i], rtol=1e-4, atol=1e-5), i


@pytest.mark.parametrize("threshold", [20.0, -1e9])
@pytest.mark.parametrize("same_noise", [True, False])
def test_tube_solve_slide_solve_matches_oracle(threshold, same_noise):
    K, T = 2048, 48
    rng = np.random.default_rng(11 if threshold > 0 else 12)
    ctrl = _tube(K, T, threshold, same_noise)
    init = rng.uniform(-0.5, 0.5, (T, 2)).astype(np.float32)
    ctrl.setControlSeq(init.T)
    x = np.array([0.0, 0.0, 0.3, -0.2], np.float32)
    eps = _draw(rng, K, T, same_noise)
    injected = eps.copy()
    if same_noise:  # the engine reads only the first half, so the second may hold anything
        injected[K * T * 2:] = rng.standard_normal(K * T * 2).astype(np.float32)
    ctrl.injectNoise(injected)
    ctrl.computeControl(x, 1)
    ref = oracle.tube_compute_control(ctrl.model_id, ctrl._dyn_arr[0], ctrl._cost_arr[0], ctrl.getParams(),
                                      ctrl.sampler_.to_c(), ctrl.constraints_, K, T, 2, 4, x, x, eps,
                                      np.stack([init, init]))
    _check(ctrl, ref, K, T)
    # slide: the nominal state advances one step along the nominal sequence, both sequences slide; then a disturbed
    # actual state and fresh noise
    u_nom, u_act = ctrl.getNominalControlSeq().T.copy(), ctrl.getActualControlSeq().T.copy()
    nominal_x0 = oracle.step_state(ctrl.model_id, ctrl._dyn_arr[0], ctrl._cost_arr[0], ref["nominal_x0"], u_nom[0],
                                   0.02)
    ctrl.slideControlSequence(1)
    zero = np.zeros(2, np.float32)
    seqs = np.stack([oracle.slide(u_act, 1, [0.0, 0.0], zero), oracle.slide(u_nom, 1, [0.0, 0.0], zero)])
    assert np.array_equal(ctrl.getActualControlSeq().T, seqs[0])
    assert np.array_equal(ctrl.getNominalControlSeq().T, seqs[1])
    # the reference's getControlSeq / getTargetStateSeq of a Tube-MPPI controller are the nominal system's
    assert np.array_equal(ctrl.getControlSeq(), ctrl.getNominalControlSeq())
    x2 = np.array([0.05, -0.03, 0.25, -0.1], np.float32)
    eps2 = _draw(rng, K, T, same_noise)
    ctrl.injectNoise(eps2)
    ctrl.computeControl(x2, 1)
    ref2 = oracle.tube_compute_control(ctrl.model_id, ctrl._dyn_arr[0], ctrl._cost_arr[0], ctrl.getParams(),
                                       ctrl.sampler_.to_c(), ctrl.constraints_, K, T, 2, 4, x2, nominal_x0, eps2,
                                       seqs)
    _check(ctrl, ref2, K, T)
    assert np.array_equal(ctrl.getNominalStateSeq()[:, 0], ref2["nominal_x0"])
    assert ref2["nominal_used"] == (0 if threshold > 0 else 1)
    ctrl.close()


def test_tube_iterations_apply_the_std_dev_decay():
    """Two iterations with std_dev_decay = 0.8: the second iteration's samples are drawn with 0.8 sigma
    (generateSamples(stride, opt_iter), tube_mppi_controller.cu:188-196) although the solve iterates on the host.  The
    second iteration starts from the first one's means, which the engine sums in FP32 and the oracle in FP64, so the
    costs agree to 1e-4 here rather than bit for bit (without the decay they would differ by percents)."""
    K, T = 2048, 48
    dyn = DoubleIntegratorDynamics()
    dyn.setControlRanges([(-2.0, 2.0), (-2.0, 2.0)])
    cost = DoubleIntegratorObstacleCost(goal=(1.5, -0.5, 0.0, 0.0), coeff=(1.0, 1.0, 0.1, 0.1), terminal_coeff=5.0,
                                        obstacles=[(0.7, 0.0, 0.3)], obstacle_cost=100.0)
    sampler = GaussianDistribution(std_dev=(0.6, 0.6), std_dev_decay=0.8)
    ctrl = TubeMPPIController(dyn, cost, None, sampler, 0.02, 2, 1.0, 0.0, T, K, nominal_threshold=-1e9)
    rng = np.random.default_rng(21)
    init = rng.uniform(-0.5, 0.5, (T, 2)).astype(np.float32)
    ctrl.setControlSeq(init.T)
    x = np.array([0.0, 0.0, 0.3, -0.2], np.float32)
    eps = _draw(rng, K, T, True)
    ctrl.injectNoise(eps)
    ctrl.computeControl(x, 1)
    ref = oracle.tube_compute_control(ctrl.model_id, ctrl._dyn_arr[0], ctrl._cost_arr[0], ctrl.getParams(),
                                      ctrl.sampler_.to_c(), ctrl.constraints_, K, T, 2, 4, x, x, eps,
                                      np.stack([init, init]))
    costs = ctrl.sample_costs().reshape(2, K)
    rel = np.abs(costs - ref["costs"]) / np.abs(ref["costs"])
    assert rel.max() < 1e-4, rel.max()
    ctrl.close()


@pytest.mark.parametrize("same_noise", [True, False])
def test_tube_distributions_share_philox_noise(same_noise):
    """With both distributions around the same mean, use_same_noise_for_all_distributions gives bit-identical
    samples for the two (one Philox draw); without it they are independent."""
    K, T = 1024, 32
    ctrl = _tube(K, T, 20.0, same_noise)
    init = np.random.default_rng(3).uniform(-0.5, 0.5, (T, 2)).astype(np.float32)
    ctrl.setControlSeq(init.T)
    ctrl.generateSamples(1, 0)
    s = ctrl.control_samples().reshape(2, K, T, 2)
    assert np.array_equal(s[0], s[1]) == same_noise
    ctrl.close()


def test_tube_requires_two_equal_instances():
    from mppi_generic_vendor_gb300 import BatchedMPPIController, MPPIError

    dyn = DoubleIntegratorDynamics()
    ctrl = BatchedMPPIController(dyn, DoubleIntegratorObstacleCost(), GaussianDistribution(std_dev=(0.5, 0.5)),
                                 [256, 512], [16, 16])
    cp = ctrl.getParams()
    cp.controller = 2
    with pytest.raises(MPPIError):
        ctrl.setParams(cp)
    ctrl.close()
