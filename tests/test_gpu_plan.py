"""Replayable plans (cusna_saom_plan_*): problems of uneven size prepared once
and re-simulated in one persistent launch, optionally replayed from a CUDA
graph. Every launch must equal the one-shot batch call on the same problems
with Philox key seed + epoch and the parameters in force, bit for bit."""
import numpy as np
import pytest

from cusna_gb300 import sim as G
from cusna_gb300 import workloads as WL
from cusna_gb300.glue import marshal_period

pytestmark = pytest.mark.gpu


def _problems(kind, sizes, M, seed0=5, theta_scale=1.0, seed_shift=0):
    out = []
    for i, n in enumerate(sizes):
        c = WL.parity_case(kind, seed=i, n=n, M=M)
        th = np.asarray(c["theta"], dtype=np.float64) * theta_scale
        out.append(marshal_period(c["inp"], M, seed0 + 100 * i + seed_shift, c["lam"], th,
                                  lamb=c.get("lamb", 0.0), thetab=c.get("thetab")))
    return out


def _same(a: dict, b: dict, tag):
    assert set(a) == set(b), tag
    for k in a:
        np.testing.assert_array_equal(a[k], b[k], err_msg=f"{tag}:{k}")


@pytest.mark.parametrize("kind", ["covariate", "conditional", "structural", "coevol"])
def test_plan_launches_equal_batch_calls(kind):
    sizes = [97, 20, 45, 64, 33]              # uneven; ordered longest-first inside
    ms = _problems(kind, sizes, M=5)
    plan = G.SimPlan(ms, use_graph=True)
    # launch 0: the problems' own seeds
    plan.launch()
    got = plan.outputs()
    ref = G.simulate_batch(_problems(kind, sizes, M=5))
    for q in range(len(sizes)):
        _same(got[q], ref[q], f"{kind} launch0 q{q}")
    # launch 1 with new theta: seed + 1, tables rebuilt on the device
    th_new = []
    for i, n in enumerate(sizes):
        c = WL.parity_case(kind, seed=i, n=n, M=5)
        th_new.append(np.asarray(c["theta"], dtype=np.float64) * 0.8)
    plan.set_params(theta=np.array([np.asarray(t, np.float32) for t in th_new]))
    plan.launch()
    got = plan.outputs()
    ref = G.simulate_batch(_problems(kind, sizes, M=5, theta_scale=0.8, seed_shift=1))
    for q in range(len(sizes)):
        _same(got[q], ref[q], f"{kind} launch1 q{q}")
    plan.close()


def test_plan_graph_replay_equals_direct_launches():
    sizes = [80, 40, 60]
    a = G.SimPlan(_problems("covariate", sizes, M=4), use_graph=True)
    b = G.SimPlan(_problems("covariate", sizes, M=4), use_graph=False)
    for epoch in range(3):
        a.launch()
        b.launch()
        for q, (x, y) in enumerate(zip(a.outputs(), b.outputs())):
            _same(x, y, f"epoch {epoch} q{q}")
    # resetting the epoch replays the first launch
    a.set_epoch(0)
    a.launch()
    ref = G.simulate_batch(_problems("covariate", sizes, M=4))
    for q in range(len(sizes)):
        _same(a.outputs()[q], ref[q], f"reset q{q}")
    a.close()
    b.close()


def test_plan_with_a_parameter_row_per_chain():
    sizes = [50, 30]
    M = 6
    rng = np.random.Generator(np.random.PCG64(3))
    ms, ref_ms = [], []
    for i, n in enumerate(sizes):
        c = WL.parity_case("covariate", seed=i, n=n, M=M)
        k = c["inp"].k
        th = np.asarray(c["theta"], dtype=np.float64)[None, :] + 0.2 * rng.standard_normal((M, k))
        lam = c["lam"] * (1 + 0.1 * rng.random(M))
        ms.append(marshal_period(c["inp"], M, 7 + i, lam, th))
        ref_ms.append(marshal_period(c["inp"], M, 7 + i, lam, th))
    plan = G.SimPlan(ms, per_chain=True, use_graph=True)
    plan.launch()
    ref = G.simulate_batch(ref_ms)
    for q in range(len(sizes)):
        _same(plan.outputs()[q], ref[q], f"per-chain q{q}")
    plan.close()


def test_plan_rejects_mixed_outputs():
    a = WL.parity_case("covariate", seed=0, n=30, M=2)
    b = WL.parity_case("covariate", seed=1, n=30, M=2)
    ms = [marshal_period(a["inp"], 2, 1, a["lam"], a["theta"]),
          marshal_period(b["inp"], 2, 1, b["lam"], b["theta"], want_ends=True)]
    with pytest.raises(ValueError):
        G.SimPlan(ms)
