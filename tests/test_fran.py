"""The FRAN backend (cusna_fran, R/fran.R:26-80): one chain per call in the
simstats0c layout, over the CPU oracle (CPU) and over the GPU plan engine
(`-m gpu`)."""
import numpy as np
import pytest

from cusna_gb300 import fran as FR
from cusna_gb300 import mom
from cusna_gb300 import workloads as WL
from cusna_gb300.glue import marshal_period

EFFECTS = ["density", "recip", "transTrip"]


def panel(engine, n=40, seed=3):
    """Three waves: Bernoulli(0.06), then two periods simulated at rate 5."""
    from cusna_gb300 import effects as E
    specs = [E.make_effect_spec(nm) for nm in EFFECTS]
    waves = [WL.bernoulli_net(n, 0.06, seed=seed).astype(np.int64)]
    for s in (41, 42):
        m = marshal_period(WL.period_inputs(waves[-1], specs), 1, s, 5.0,
                           np.array([-2.2, 1.8, 0.3]), want_ends=True)
        waves.append(engine.simulate_batch([m])[0]["a_ends"][0].astype(np.int64))
    return waves


def test_fran_layout_and_checks(port):
    waves = panel(port)
    f = FR.cusna_fran(waves, EFFECTS, conditional=False, seed=5, engine=port)
    est = f.estimator
    assert est.p == 2 + 3
    out = f({"theta": [5.0, 5.0, -2.2, 1.8, 0.3]})
    assert out["fra"].shape == (2, 5) and out["sc"].shape == (2, 5)
    assert out["ntim0"].shape == (2,) and out["OK"] and out["feasible"]
    # per-period rows: the rate statistic of period q sits in column q only
    assert out["fra"][0, 1] == 0 and out["fra"][1, 0] == 0
    assert f.counter == 1
    with pytest.raises(ValueError, match="parameters"):
        f({"theta": [1.0, 2.0]})
    with pytest.raises(ValueError, match="conditional"):
        f({"theta": [5.0, 5.0, -2.2, 1.8, 0.3], "cconditional": True})


def test_fran_is_reproducible_and_matches_the_estimator(port):
    waves = panel(port)
    th = np.array([-2.2, 1.8, 0.3])
    a = FR.cusna_fran(waves, EFFECTS, conditional=True, seed=9, engine=port)
    b = FR.cusna_fran(waves, EFFECTS, conditional=True, seed=9, engine=port)
    for _ in range(3):
        x, y = a({"theta": th}), b({"theta": th})
        np.testing.assert_array_equal(x["fra"], y["fra"])
        np.testing.assert_array_equal(x["sc"], y["sc"])
    # one call is one chain of mom_simulate with the same generator state
    c = FR.cusna_fran(waves, EFFECTS, conditional=True, seed=4, engine=port)
    rng = np.random.Generator(np.random.PCG64(4))
    s = mom.mom_simulate(c.estimator, th, 1, rng, port)
    out = c({"theta": th})
    np.testing.assert_array_equal(out["fra"], np.stack([sp[0] for sp, _ in s.pieces]))


@pytest.mark.gpu
def test_gpu_fran_plan_engine(gpu_lib):
    eng = mom.GpuEngine()
    waves = panel(eng)
    th = np.array([5.0, 5.0, -2.2, 1.8, 0.3])
    a = FR.cusna_fran(waves, EFFECTS, conditional=False, seed=2)
    b = FR.cusna_fran(waves, EFFECTS, conditional=False, seed=2)
    calls = 300
    fa = []
    for _ in range(calls):
        x, y = a({"theta": th}), b({"theta": th})
        np.testing.assert_array_equal(x["fra"], y["fra"])
        fa.append(x["fra"].sum(axis=0))
    fa = np.array(fa)
    # the single-chain statistics average to the many-chain mean
    s = mom.mom_simulate(a.estimator, th, 4000, np.random.default_rng(1), eng)
    mean, sd = s.stats.mean(axis=0), s.stats.std(axis=0)
    z = (fa.mean(axis=0) - mean) / (sd / np.sqrt(calls) + 1e-12)
    assert np.all(np.abs(z) < 5.0), z
    a.engine.close()
    b.engine.close()
