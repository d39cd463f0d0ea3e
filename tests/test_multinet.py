"""The multi-network Method-of-Moments estimator (mom_estimate_multinet).

The reference's acceptance test (tests/testthat/test-multinet.R) fits a
2-network model (density and recip per network) on the panels of
fixtures/multinet/multinet.json.gz and requires every estimate within
1.0 * SE + 0.2 of the frozen fit. The same test runs here over the CPU oracle
(CPU) and over the GPU engine (`-m gpu`); the targets must equal the fixture's
exactly. The fixture stays with the reference; on the GPU the fit over the GPU
engine is compared with the fit over the CPU oracle on a synthetic panel of
the same shape.
"""
import gzip
import json
import os

import numpy as np
import pytest

from cusna_gb300 import effects as E
from cusna_gb300 import multinet as MN
from cusna_gb300 import workloads as WL
from tests.conftest import FIXTURES


class OracleMultiEngine:
    """The estimator's engine interface over the CPU oracle."""

    def __init__(self, port):
        self.port = port

    def simulate_multi(self, m):
        return self.port.simulate_multi(m)

    def network_stats_batch(self, A, n, k, *desc):
        return np.stack([self.port.network_stats(a, n, k, *desc) for a in A])

    def cross_stats(self, A, wp, t, parm):
        return self.port.cross_stats(A, wp, t, parm)


def load_fixture():
    path = os.path.join(FIXTURES, "multinet", "multinet.json.gz")
    if not os.path.exists(path):
        pytest.skip("reference fixtures not present")
    g = json.load(gzip.open(path))
    S = g["settings"]
    ctl = dict(firstg=S["firstg"], nsub=int(S["nsub"]), n2=tuple(int(x) for x in S["n2"]),
               batch2=int(S["batch2"]), n1=int(S["n1"]), n3=int(S["n3"]), nD=int(S["nD"]),
               diagonalize=S["diagonalize"], seed=int(S["seed"]))
    nets = [[np.array(w, dtype=float) for w in g["netA_waves"]],
            [np.array(w, dtype=float) for w in g["netB_waves"]]]
    return g, ctl, nets


def effects_by_net():
    return [[E.cusna_effect("density"), E.cusna_effect("recip")],
            [E.cusna_effect("density"), E.cusna_effect("recip")]]


def check_fit(fit, g):
    assert fit.param_names == g["param_names"]
    th, se = np.asarray(g["theta"]), np.asarray(g["se"])
    assert len(fit.theta) == 6
    for i in range(6):
        assert abs(fit.theta[i] - th[i]) < 1.0 * se[i] + 0.2, (i, fit.theta, th, se)


def test_multinet_targets_match_fixture(port):
    g, ctl, nets = load_fixture()
    mn = MN.saom_multinet_data(nets)
    specs = [E.build_specs(effs) for effs in effects_by_net()]
    est = MN.multi_mom_estimator(mn.internal, specs, ctl, OracleMultiEngine(port))
    np.testing.assert_array_equal(est.targets, g["targets"])
    assert est.param_names == g["param_names"]


def test_multinet_estimate_within_se_of_reference_cpu(port):
    g, ctl, nets = load_fixture()
    fit = MN.mom_estimate_multinet(MN.saom_multinet_data(nets), effects_by_net(), control=ctl,
                                   engine=OracleMultiEngine(port))
    check_fit(fit, g)


def test_multinet_cross_effect_targets(port):
    """A cross effect's target is its statistic on the observed end wave
    against the source network's period-start predictor."""
    g, ctl, nets = load_fixture()
    mn = MN.saom_multinet_data(nets)
    effs = [[E.cusna_effect("density"), E.cusna_effect("crprod", net_ref=2)],
            [E.cusna_effect("density"), E.cusna_effect("to", net_ref=1)]]
    specs = [E.build_specs(x) for x in effs]
    est = MN.multi_mom_estimator(mn.internal, specs, ctl, OracleMultiEngine(port))
    A1, B0 = nets[0][1] != 0, nets[1][0] != 0
    B1, A0 = nets[1][1] != 0, nets[0][0] != 0
    assert est.targets[est.eff_pos[1]] == float((A1 & B0).sum())
    assert est.targets[est.eff_pos[3]] == float(sum(int((A0[i] & B1[:, j]).sum())
                                                    for i in range(50) for j in range(50) if B1[i, j]))
    assert est.param_names[2] == "net0 crprod<-net1"


def test_multinet_input_errors():
    with pytest.raises(ValueError):
        MN.saom_multinet_data([[np.zeros((3, 3)), np.zeros((3, 3))]])
    with pytest.raises(ValueError):
        MN.saom_multinet_data([[np.zeros((3, 3)), np.zeros((3, 3))],
                               [np.zeros((3, 3)), np.zeros((3, 3)), np.zeros((3, 3))]])
    with pytest.raises(ValueError):
        MN.saom_multinet_data([[np.zeros((3, 3)), np.zeros((3, 3))],
                               [np.zeros((4, 4)), np.zeros((4, 4))]])
    mn = MN.saom_multinet_data([[np.zeros((3, 3)), np.zeros((3, 3))]] * 2)
    with pytest.raises(ValueError):
        MN.mom_estimate_multinet(mn, [[E.cusna_effect("density")]])


@pytest.mark.gpu
def test_multinet_gpu_fit_matches_cpu_fit(gpu_lib, port):
    """On a synthetic 2-network panel (the reference test's panel shape), the fit
    over the GPU engine and the fit over the CPU oracle draw the same seeds and
    simulate identical trajectories; they agree to a small fraction of an SE."""
    from cusna_gb300 import sim
    waves = WL.multinet_panel(sim.simulate_multi)
    ref_waves = WL.multinet_panel(port.simulate_multi)
    for a, b in zip(waves, ref_waves):
        for x, y in zip(a, b):
            np.testing.assert_array_equal(x, y)
    data = MN.saom_multinet_data(waves)
    ctl = dict(firstg=0.4, nsub=2, n2=(8, 10), batch2=64, n1=100, n3=300, nD=100,
               diagonalize=0.2, seed=5)
    fg = MN.mom_estimate_multinet(data, effects_by_net(), control=ctl)
    fc = MN.mom_estimate_multinet(data, effects_by_net(), control=ctl,
                                  engine=OracleMultiEngine(port))
    np.testing.assert_array_equal(fg.targets, fc.targets)
    assert np.max(np.abs(fg.theta - fc.theta) / fc.se) < 0.1, (fg.theta, fc.theta, fc.se)
