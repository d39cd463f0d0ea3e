"""Surrogate-assisted Method of Moments.

CPU: the host logic over the CPU oracle engine -- the per-period decomposition
of the estimator, start-wave features, training designs, the trust region of
the surrogate's Robbins-Monro, the response-surface Jacobian, and the judge
with plain-simulation takeover (a surrogate that is wrong on purpose).
GPU: on the n=300 panel, the surrogate-assisted fit reaches the plain GPU
fit's estimates (within 0.1 SE, all |t-conv| < 0.1) with fewer simulations and
in less wall time; and the same fit with the network's term off (the response
surface alone) shows what the trained network adds."""
import numpy as np
import pytest

from cusna_gb300 import data as D
from cusna_gb300 import effects as E
from cusna_gb300 import mom
from cusna_gb300 import surrogate as S
from cusna_gb300 import workloads as WL

ES = E.make_effect_spec


@pytest.fixture(scope="module")
def c1_est(port):
    waves = WL.c1_panel(port)
    d = D.build_saom_data(waves)
    effs = [ES(x) for x in ("density", "recip", "transTrip")]
    ctl = dict(mom.DEFAULT_CONTROL)
    return mom.mom_estimator(d, effs, None, None, False, ctl, engine=port)


def test_period_blocks_follow_the_parameter_layouts(c1_est):
    est = c1_est
    b = S.period_blocks(est)
    assert [list(x) for x in b] == [[0, 2, 3, 4], [1, 2, 3, 4]]     # rate q + shared effects
    est_c = mom.Estimator(**{**est.__dict__, "conditional": True, "p": est.k})
    assert [list(x) for x in S.period_blocks(est_c)] == [[0, 1, 2], [0, 1, 2]]
    est_b = mom.Estimator(**{**est.__dict__, "coevol": True, "kb": 2, "p": 2 * est.P + est.k + 2})
    assert [list(x) for x in S.period_blocks(est_b)] == [[0, 2, 4, 5, 6, 7, 8], [1, 3, 4, 5, 6, 7, 8]]


def test_period_features_are_start_wave_statistics(c1_est, port):
    est = c1_est
    f = S.period_features(est, port, 12)
    assert f.shape == (2, 12)
    for q in range(2):
        x = np.asarray(est.per[q]["inp"].x0)
        assert f[q, 0] == x.sum()                       # density statistic = tie count
        assert f[q, 3] == pytest.approx(x.sum() / est.n)
        assert f[q, 4] == est.dists[q] and f[q, 5] == est.n
        assert np.all(f[q, 6:] == 0)                   # zero padding
    assert S.period_features(est, port, 2).shape == (2, 2)


def test_designs_match_their_spread_and_keep_rates_positive(c1_est):
    est = c1_est
    rng = np.random.Generator(np.random.PCG64(3))
    centre = np.array([0.2, 5.0, -2.0, 1.5, 0.3])
    th = S.draw_thetas(est, centre, 40000, rng, "iso", 0.5)
    assert (th[:, :2] > 0).all()
    np.testing.assert_allclose(th[:, 2:].mean(axis=0), centre[2:], atol=0.01)
    np.testing.assert_allclose(th[:, 2:].std(axis=0), 0.5, rtol=0.02)
    L = np.linalg.cholesky(np.array([[1.0, 0.3, 0, 0, 0], [0.3, 2.0, 0, 0, 0], [0, 0, 0.5, 0.1, 0],
                                     [0, 0, 0.1, 0.2, 0], [0, 0, 0, 0, 0.05]]))
    th = S.draw_thetas(est, np.array([9.0, 9.0, -2.0, 1.5, 0.3]), 40000, rng, "se", 2.0, L)
    np.testing.assert_allclose(np.cov(th, rowvar=False), 4.0 * L @ L.T, atol=0.15)
    lo, hi = S.design_box(th)
    assert ((th >= lo).mean(axis=0) > 0.99).all() and ((th <= hi).mean(axis=0) > 0.99).all()


class _Linear:
    """A surrogate that is exactly E[s](theta) = targets + D0 (theta - root)."""

    def __init__(self, est, root, D0):
        self.est, self.root, self.D0 = est, root, D0

    def mean(self, theta):
        return self.est.targets + self.D0 @ (theta - self.root)

    def mean_and_jacobian(self, theta):
        return self.mean(theta), self.D0


def test_rm_on_surrogate_finds_the_root_inside_its_trust_region(c1_est):
    est = c1_est
    rng = np.random.Generator(np.random.PCG64(5))
    root = np.array([6.0, 6.2, -2.4, 2.0, 0.4])
    D0 = np.diag([300.0, 280.0, 500.0, 200.0, 900.0]) + rng.normal(0, 10, (5, 5))
    sur = _Linear(est, root, D0)
    box = (root - 1.0, root + 1.0)
    th = S._rm_on_surrogate(est, sur, root + np.array([0.5, -0.5, 0.3, -0.3, 0.2]), est.control, box)
    np.testing.assert_allclose(th, root, atol=1e-3)    # averaged iterates of a noise-free RM
    # a root outside the trust region: the iterates stop at its boundary
    box = (root - 1.0, root.copy())
    box[1][2] = root[2] - 0.25
    th = S._rm_on_surrogate(est, sur, root - 0.5, est.control, box)
    assert th[2] == pytest.approx(root[2] - 0.25) and (th <= box[1] + 1e-12).all()


def test_response_surface_jacobian_matches_finite_differences():
    m = S.MlpSurrogate.__new__(S.MlpSurrogate)       # host-side parts only, no GPU
    m.n_in, m.n_out, m.n_group, m.degree = 16, 3, 8, 2
    rng = np.random.Generator(np.random.PCG64(0))
    xs = rng.standard_normal((4, 16))
    m.groups = np.unique(xs[:, 8:], axis=0)
    m.C = rng.standard_normal((m._basis(xs).shape[1], 3))
    m.Cg = [m.C + 0.1 * i for i in range(len(m.groups))]
    assert m._basis(xs).shape == (4, 8 + 36 + 1)
    J = m._shortcut_jac(xs, xs, 8)
    h = 1e-6
    for k in range(8):
        e = np.zeros(16)
        e[k] = h
        fd = (m._shortcut(xs + e, xs) - m._shortcut(xs - e, xs)) / (2 * h)
        np.testing.assert_allclose(J[:, :, k], fd, atol=1e-6)


def test_judge_rejects_a_wrong_surrogate_and_plain_simulation_takes_over(c1_est, port):
    """The surrogate claims the targets are met at a theta whose density is off
    by 0.3; phase 3 measures its error, plain simulation takes over with
    Newton steps, and the fit ends with every |t-conv| below the bound."""
    est = c1_est
    rng = np.random.Generator(np.random.PCG64(9))
    theta0 = np.array([6.0, 6.0, *WL.C1_THETA])
    theta0[2] += 0.3

    class Liar:
        def mean(self, theta):
            return est.targets.copy()
    th, p3, judge, takeovers = S.judge_and_take_over(est, Liar(), theta0, port, rng, 2000,
                                                     bound=0.1, max_takeovers=4)
    assert not judge[0]["passed"] and judge[0]["error"].max() > 0.1
    assert takeovers >= 1 and judge[-1]["passed"]
    assert np.abs(p3[4]).max() < 0.1
    assert abs(th[2] - theta0[2]) > 0.1                 # the takeover moved density


# ---- GPU ---------------------------------------------------------------------
@pytest.fixture(scope="module")
def c5_gpu():
    """The n=300 panel's estimator on the GPU plan engine, warmed up (the
    period kernel specialised to this model, the network's kernels and
    training graphs, the plain fit's plans and graphs), and its plain fit
    from the data-generating theta."""
    eng = mom.PlanEngine(use_graph=True)
    waves, cov = WL.c5_panel(mom.GpuEngine())
    est = mom.mom_estimator(D.build_saom_data(waves), WL.c5_effects(cov), None, None, False,
                            dict(mom.DEFAULT_CONTROL), engine=eng)
    centre = WL.c5_theta_true()
    from cusna_gb300 import sim
    for _ in range(3):
        mom.mom_simulate(est, centre, 64, np.random.default_rng(0), mom.GpuEngine())
    sim.specialise_wait(900.0)
    r = np.random.default_rng(0)
    S.MlpSurrogate(S.N_IN, est.k + 1, S.HIDDEN).fit(r.standard_normal((2048, S.N_IN)),
                                                      r.standard_normal((2048, est.k + 1)),
                                                      epochs=2, n_group=S.N_IN - est.k - 1)
    mom.mom_run(est, theta0=centre, engine=eng)
    plain = mom.mom_run(est, theta0=centre, engine=eng)
    yield est, eng, centre, plain
    eng.close()


@pytest.mark.gpu
def test_gpu_surrogate_fit_matches_plain_fit_with_fewer_simulations(c5_gpu):
    est, eng, centre, plain = c5_gpu
    sf = S.mom_run_surrogate(est, centre, S.SurrogateControl(), eng)
    fs = sf.fit
    assert sf.fallback is None
    assert np.abs(fs.tconv).max() < 0.1 and np.abs(plain.tconv).max() < 0.1
    assert (np.abs(fs.theta - plain.theta) < 0.1 * plain.se).all(), \
        np.abs(fs.theta - plain.theta) / plain.se
    plain_sims = plain.n_sims * est.P
    assert sf.n_period_sims < 0.7 * plain_sims
    assert fs.wall_time < plain.wall_time, (fs.wall_time, plain.wall_time)
    # the surrogate alone (before any takeover) was judged: its error is recorded
    assert np.isfinite(sf.judge[0]["error"]).all()


@pytest.mark.gpu
def test_gpu_what_the_network_adds_over_the_response_surface(c5_gpu):
    """The same fit with the network's term off (the response surface alone)
    against the fit with it. On the first stage's held-out training pairs the
    network removes most of the surface's residual error; the first stage's
    surrogate estimate then lies far closer to the plain fit's, the plain
    pilots accept it, and the fit finishes on the surrogate. The surface alone
    leads the pilots astray, plain simulation takes over, and the fit needs
    more simulations and more time."""
    est, eng, centre, plain = c5_gpu
    on = S.mom_run_surrogate(est, centre, S.SurrogateControl(), eng)
    off = S.mom_run_surrogate(est, centre, S.SurrogateControl(network=False), eng)
    st_on, st_off = on.stages[0], off.stages[0]
    assert np.all(st_off["gate"] == 0) and np.any(st_on["gate"] > 0)
    assert np.mean(st_on["val_net"]) < 0.5 * np.mean(st_on["val_surface"]), \
        (st_on["val_net"], st_on["val_surface"])
    dist_on = np.max(np.abs(st_on["theta"] - plain.theta) / plain.se)
    dist_off = np.max(np.abs(st_off["theta"] - plain.theta) / plain.se)
    assert dist_on < dist_off, (dist_on, dist_off)
    assert on.fallback is None and off.fallback is not None
    assert off.n_period_sims > on.n_period_sims
    assert off.fit.wall_time > on.fit.wall_time
