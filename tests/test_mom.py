"""The Method-of-Moments estimator (restatement of R/mom.R) over the CPU oracle
against the reference's fixture estimate.json.gz (estimates within SE + 0.1,
the bar of tests/testthat/test-estimate.R:24-28; targets equal), and over the
GPU simulator against the same estimator over the CPU oracle."""
import gzip
import json
import os

import numpy as np
import pytest

from cusna_gb300 import data as D
from cusna_gb300 import effects as E
from cusna_gb300 import mom
from cusna_gb300 import workloads as WL

ES = E.make_effect_spec


def _fixture_configs(fixtures_dir):
    g = json.load(gzip.open(os.path.join(fixtures_dir, "estimate", "estimate.json.gz")))
    S = g["settings"]
    ctl = dict(firstg=S["firstg"], nsub=S["nsub"], n2=tuple(S["n2"]), batch2=S["batch2"],
               n1=S["n1"], n3=S["n3"], nD=S["nD"], diagonalize=S["diagonalize"],
               seed=S["seed"], maxdegree=0)
    waves = [np.array(w, dtype=float) for w in g["inputs"]["s50_waves"]]
    alc = np.array(g["inputs"]["alcohol"], dtype=float)
    base = [ES(x) for x in ("density", "recip", "transTrip")]
    cfgs = {
        "baseline": (D.build_saom_data(waves), base, None, False),
        "baseline_cond": (D.build_saom_data(waves), base, None, True),
        "covariate": (D.build_saom_data(waves), base + [ES("egoX", alc[:, 0]), ES("altX", alc[:, 0]),
                                                        ES("simX", alc[:, 0])], None, False),
        "coevol": (D.build_saom_data(waves, behavior=alc),
                   base + [ES("egoX", dyn=True), ES("altX", dyn=True), ES("simX", dyn=True)],
                   [E.make_beh_effect_spec(x) for x in ("linear", "quad", "avSim")], False),
    }
    return g, ctl, cfgs


@pytest.mark.parametrize("name", ["baseline", "baseline_cond", "covariate", "coevol"])
def test_mom_over_oracle_matches_reference_estimates(port, fixtures_dir, name):
    g, ctl, cfgs = _fixture_configs(fixtures_dir)
    d, effs, bef, cond = cfgs[name]
    est = mom.mom_estimator(d, effs, bef, None, cond, ctl, engine=port)
    gold = g["configs"][name]
    np.testing.assert_allclose(est.targets, gold["targets"], rtol=1e-7)  # test-targets.R tolerance
    assert est.param_names == gold["param_names"]
    fit = mom.mom_run(est, engine=port, backend="cpu")
    th_ref, se_ref = np.array(gold["theta"]), np.array(gold["se"])
    assert (np.abs(fit.theta - th_ref) < se_ref + 0.1).all(), (fit.theta, th_ref)


def test_mom_building_blocks():
    """Guarded step, diagonalised inverse and pseudo-inverse (R/mom.R:14-20, 184-197)."""
    Dm = np.array([[2.0, 0.5], [0.3, 1.0]])
    inv = mom.mom_dinv(Dm, 0.2)
    mix = 0.8 * Dm + 0.2 * np.diag(np.diag(Dm))
    np.testing.assert_allclose(inv @ mix, np.eye(2), atol=1e-12)
    sing = np.array([[1.0, 1.0], [1.0, 1.0]])
    np.testing.assert_allclose(mom.safe_solve(sing), np.linalg.pinv(sing), atol=1e-12)

    class Est:
        conditional, coevol, P = False, False, 2
    step = mom.guard_step(Est, np.array([5.0, 4.0, -2.0]), np.array([4.9, 0.5, 3.0]))
    np.testing.assert_allclose(step, [2.5, 0.5, 1.0])


SCHEDULE = dict(firstg=0.4, nsub=2, n2=(15, 20), batch2=128, n1=300, nD=300, n3=800,
                diagonalize=0.2, seed=7, maxdegree=0)


@pytest.mark.gpu
def test_gpu_mom_agrees_with_oracle_mom(gpu_lib, port):
    """Conditional MoM on the synthetic n=50 panel: the GPU fit and the fit over
    the CPU oracle agree within their standard errors."""
    waves = WL.c1_panel(mom.GpuEngine())
    np.testing.assert_array_equal(waves[1], WL.c1_panel(port)[1])   # same trajectory
    d = D.build_saom_data(waves)
    effs = [ES(x) for x in ("density", "recip", "transTrip")]
    fits = {}
    for label, eng in (("gpu", mom.GpuEngine()), ("cpu", port)):
        est = mom.mom_estimator(d, effs, None, None, True, SCHEDULE, engine=eng)
        fits[label] = mom.mom_run(est, engine=eng, backend=label)
    g, c = fits["gpu"], fits["cpu"]
    np.testing.assert_array_equal(g.targets, c.targets)
    assert (np.abs(g.theta - c.theta) < np.maximum(g.se, c.se)).all(), (g.theta, c.theta)


@pytest.mark.gpu
def test_gpu_mom_through_replayed_plans(gpu_lib):
    """The estimator over PlanEngine (each round a CUDA-graph replay of a plan
    prepared once) reaches the estimates of the estimator over one-shot batch
    calls within their standard errors; on 24 uneven groups too."""
    waves = WL.c1_panel(mom.GpuEngine())
    d = D.build_saom_data(waves)
    effs = [ES(x) for x in ("density", "recip", "transTrip")]
    fits = {}
    for label, eng in (("batch", mom.GpuEngine()), ("plan", mom.PlanEngine())):
        est = mom.mom_estimator(d, effs, None, None, True, SCHEDULE, engine=eng)
        fits[label] = mom.mom_run(est, engine=eng)
    a, b = fits["batch"], fits["plan"]
    assert (np.abs(a.theta - b.theta) < np.maximum(a.se, b.se)).all(), (a.theta, b.theta)
    groups = WL.c3_groups(mom.GpuEngine(), n_groups=24, seed=5)
    datas = [D.build_saom_data(w) for w, _ in groups]
    geffs = [WL.c3_effects(c) for _, c in groups]
    ctl = dict(SCHEDULE, batch2=1)
    eng = mom.PlanEngine()
    est = mom.mom_estimator_groups(datas, geffs, ctl, engine=eng)
    fit = mom.mom_run(est, engine=eng)
    assert (np.abs(fit.theta - WL.C3_THETA) < 6 * fit.se + 0.05).all(), (fit.theta, fit.se)
    eng.close()


def test_joint_estimator_over_groups_sums_periods(port):
    """Groups as extra periods (R/mom.R:143-182): targets are the sum of the
    groups' targets, every (group, period) is one unit with its own target
    distance, and a simulation round covers all units."""
    groups = WL.c3_groups(port, n_groups=3, seed=11)
    datas = [D.build_saom_data(w) for w, _ in groups]
    effs = [WL.c3_effects(c) for _, c in groups]
    ctl = dict(mom.DEFAULT_CONTROL)
    est = mom.mom_estimator_groups(datas, effs, ctl, engine=port)
    singles = [mom.mom_estimator(d, e, None, None, True, ctl, engine=port) for d, e in zip(datas, effs)]
    assert est.P == 6 and est.p == 4 and est.conditional
    np.testing.assert_allclose(est.targets, np.sum([s.targets for s in singles], axis=0))
    np.testing.assert_array_equal(est.dists, np.concatenate([s.dists for s in singles]))
    rng = np.random.Generator(np.random.PCG64(2))
    s = mom.mom_simulate(est, WL.C3_THETA, 3, rng, port)
    assert s.stats.shape == (3, 4) and len(s.pieces) == 6
    # conditional: every unit stopped at its own observed distance
    assert (s.ntim > 0).all()
