"""Method-of-Moments Robbins-Monro estimator of a SAOM (RSiena-style).

A Python restatement of the reference's R estimator R/mom.R:1-269 (cran/cusna
0.1.1): the estimator context (.mom_estimator), per-period simulation
(.run_period_sim / .mom_simulate), the score-function derivative, the
diagonalised inverse, the guarded step and the three phases (.mom_run). All
periods of one simulation round run in one launch of the GPU simulator
(cusna_saom_simulate_batch); the behaviour statistics run on the GPU too.

The simulation engine is pluggable: `GpuEngine` (the product) or any object
with the same three methods (`simulate_batch`, `network_stats`,
`behavior_stats`), which is how the tests run the identical estimator over the
CPU oracle.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np

from . import data as D
from . import effects as E
from . import targets as TG
from .glue import PeriodInputs, marshal_period

DEFAULT_CONTROL = dict(firstg=0.4, nsub=4, n2=(40, 40, 60, 80), batch2=256, n1=1000, n3=4000,
                       nD=1000, diagonalize=0.2, seed=1234, maxdegree=0)   # R/mom.R:26-28


class GpuEngine:
    """The GB300 simulator behind the estimator."""

    def simulate_batch(self, ms):
        from . import sim
        return sim.simulate_batch(ms)

    def network_stats(self, *args):
        from . import sim
        return sim.network_stats(*args)

    def behavior_stats(self, *args):
        from . import sim
        return sim.behavior_stats(*args)


class PlanEngine(GpuEngine):
    """GpuEngine whose simulation rounds run as replayable plans
    (cusna_gb300.sim.SimPlan), one per chain count M: every (period or group)
    problem is marshalled and moved to the device once; a round writes the new
    parameters into the plan's device buffers and replays its CUDA graph, and
    only the moment outputs come back. Round r of a plan simulates with Philox
    keys seed + r, seeds drawn once per plan from the estimator's stream."""

    OUTPUTS = ("stats", "scores", "ntim", "dist_stat", "bdist", "bscores", "z_end")

    def __init__(self, use_graph: bool = True):
        self.use_graph = use_graph
        self._plans = {}

    def simulate_round(self, est, theta, M: int, rng, scores: bool = True) -> list:
        """scores=False: a plan whose results leave the scores out, so the
        simulator forms no score sums (the Robbins-Monro steps of phase 2 read
        only the statistics)."""
        from . import sim
        lam, th, lamb, thb, _ = split_theta(est, theta)
        key = (id(est), int(M), bool(scores))
        plan = self._plans.get(key)
        if plan is None:
            ms = [marshal_period(d["inp"], M, int(rng.integers(1, np.iinfo(np.int32).max)), lam[q], th,
                                 lamb=lamb[q], thetab=thb if est.kb else None)
                  for q, d in enumerate(est.per)]
            if not scores:
                for m in ms:
                    m.drop_outputs(("scores", "bscores"))
            plan = sim.SimPlan(ms, use_graph=self.use_graph)
            self._plans[key] = plan
        else:
            rows = dict(theta=np.asarray(th, dtype=np.float32)[None, :],
                        lam=np.asarray(lam, dtype=np.float32)[:, None])
            if est.kb:
                rows.update(lamb=np.asarray(lamb, dtype=np.float32)[:, None],
                            thetab=np.asarray(thb, dtype=np.float32)[None, :])
            plan.set_params(**rows)
        plan.launch()
        return plan.outputs([o for o in self.OUTPUTS if o in plan.outs])

    def close(self):
        for p in self._plans.values():
            p.close()
        self._plans.clear()


def pinv(m, tol=np.sqrt(np.finfo(float).eps)):
    """Moore-Penrose pseudo-inverse by SVD (R/mom.R:15-19)."""
    u, s, vt = np.linalg.svd(m)
    keep = s > max(tol * s[0], 0)
    return (vt[keep].T / s[keep]) @ u[:, keep].T


def safe_solve(m):
    try:
        return np.linalg.solve(m, np.eye(m.shape[0]))
    except np.linalg.LinAlgError:
        return pinv(m)


@dataclass
class Estimator:
    """Estimator context (R/mom.R:24-83)."""
    data: D.SaomData
    effects: list
    beh_effects: list | None
    conditional: bool
    control: dict
    n: int
    P: int
    k: int
    kb: int
    p: int
    symflag: int
    targets: np.ndarray
    param_names: list
    rate_consts: np.ndarray
    dists: np.ndarray
    bty: np.ndarray
    per: list                       # per period: dict with PeriodInputs and extras
    coevol: bool = False
    mom_targets: object = None


def mom_estimator(data: D.SaomData, effects, beh_effects=None, rate_effects=None,
                  conditional=False, control=None, engine=None) -> Estimator:
    ctl = dict(DEFAULT_CONTROL)
    ctl.update(control or {})
    engine = engine or GpuEngine()
    n, P, k = data.n, data.n_periods, len(effects)
    coevol = bool(beh_effects)
    kb = len(beh_effects) if coevol else 0
    if rate_effects:
        raise ValueError("rate effects are not yet supported in the estimator.")  # R/mom.R:33
    beh = data.beh
    symflag = 1 if data.symmetric else 0
    mt = TG.mom_targets(data, effects, engine.network_stats, beh_effects, rate_effects,
                        conditional, beh_stats=engine.behavior_stats)
    p = 2 * P + k + kb if coevol else (k if conditional else P + k)
    eff_names = [e.name for e in effects]
    if coevol:
        names = ([f"rate net (p{q})" for q in range(1, P + 1)] +
                 [f"rate beh (p{q})" for q in range(1, P + 1)] + eff_names +
                 ["beh " + e.name for e in beh_effects])
    elif conditional:
        names = list(eff_names)
    else:
        names = [f"rate (period {q})" for q in range(1, P + 1)] + eff_names
    rate_consts = (np.array([float(D.rate_const(data, q)) for q in range(1, P + 1)])
                   if data.has_composition else np.zeros(P))
    dists = np.array([float(D.observed_distance(data, q)) for q in range(1, P + 1)])
    bty = np.array([e.type_id for e in beh_effects], dtype=np.int32) if coevol else np.zeros(0, np.int32)
    wtab = E.effect_wtabs(effects, n)
    int_idx = E.interaction_comp_idx(effects) if any(E.is_interaction(e) for e in effects) else None
    per = []
    for q in range(1, P + 1):
        z_start = D.beh_values_less_missing_starts(beh, q) if coevol else None
        pe = E.prepare_effects_v2(effects, n, q, beh if coevol else None, z_start)
        inp = PeriodInputs(x0=data.imputed[q - 1], type_ids=pe.type_ids, vmat=pe.vmat, wtab=wtab,
                           vb=pe.v_dyn, p1=pe.p1, p2=pe.p2, vmiss=pe.vmiss,
                           etypes=np.zeros(k, np.int32), dyn_flags=pe.dyn_flags,
                           dyc_idx=pe.dyc_idx, int_idx=int_idx, maxdegree=int(ctl["maxdegree"]),
                           conditional=1 if conditional else 0,
                           target_dist=int(dists[q - 1]) if conditional else 0, symflag=symflag)
        extra = {}
        if coevol:
            inp.bty = bty
            inp.z0 = beh.imputed[:, q - 1].astype(np.int32)
            inp.bkdist = D.beh_kmask_dist(beh, q).astype(np.int32)
            inp.zmin, inp.zmax = beh.zmin, beh.zmax
            inp.zbar, inp.brange, inp.bsimmean = beh.overall_mean, beh.range, beh.sim_mean
            extra["xnet"] = D.network_less_missing_start(data, q)
        per.append(dict(inp=inp, **extra))
    return Estimator(data, effects, beh_effects, conditional, ctl, n, P, k, kb, p, symflag,
                     mt.target_vector, names, rate_consts, dists, bty, per, coevol, mt)


def mom_estimator_groups(datas, effects_list, control=None, engine=None) -> Estimator:
    """Joint conditional Method of Moments over independent groups that share
    the model's parameters. The reference has no multi-group estimator; groups
    are treated exactly as extra periods of one estimator (R/mom.R:143-182 sum
    statistics and derivatives over periods): the targets are summed over every
    group's periods, each (group, period) is one simulated unit with its own
    conditional target distance, and one round simulates all units."""
    ests = [mom_estimator(d, effs, None, None, True, control, engine)
            for d, effs in zip(datas, effects_list)]
    e0 = ests[0]
    for e in ests[1:]:
        if e.k != e0.k or e.param_names != e0.param_names:
            raise ValueError("every group needs the same effects")
    per = [u for e in ests for u in e.per]
    P = len(per)
    return Estimator(e0.data, e0.effects, None, True, e0.control, max(e.n for e in ests), P,
                     e0.k, 0, e0.p, e0.symflag, np.sum([e.targets for e in ests], axis=0),
                     list(e0.param_names), np.zeros(P),
                     np.concatenate([e.dists for e in ests]), e0.bty, per, False, None)


def split_theta(est: Estimator, theta):
    """(lam per period, theta_eval, lamb per period, theta_beh, offset), R/mom.R:131-138."""
    P, k, p = est.P, est.k, est.p
    theta = np.asarray(theta, dtype=np.float64)
    if est.coevol:
        return theta[:P], theta[2 * P:2 * P + k], theta[P:2 * P], theta[2 * P + k:p], 2 * P
    if est.conditional:
        return np.ones(P), theta, np.zeros(P), np.zeros(0), 0
    return theta[:P], theta[P:p], np.zeros(P), np.zeros(0), P


@dataclass
class SimRound:
    stats: np.ndarray               # (M, p) summed over periods
    pieces: list                    # per period (sp, scp)
    ntim: np.ndarray                # (M, P)
    nets: list | None = None
    z_ends: list | None = None


def mom_simulate(est: Estimator, theta, M: int, rng, engine, keep_nets=False,
                 theta_rows=None, scores=True) -> SimRound:
    """All periods of one round in one batch launch (R/mom.R:129-170).
    theta_rows: optional (M, p) per-chain parameters (the simulator honours
    per-chain theta; used to generate surrogate training data). scores=False:
    only the statistics are wanted (a plan engine then has the simulator skip
    the score sums, and the pieces' score columns are zero)."""
    P, p, k, kb = est.P, est.p, est.k, est.kb
    lam, th, lamb, thb, off = split_theta(est, theta)
    if theta_rows is None and not keep_nets and hasattr(engine, "simulate_round"):
        outs = (engine.simulate_round(est, theta, M, rng) if scores
                else engine.simulate_round(est, theta, M, rng, scores=False))
    else:
        ms = []
        for q in range(P):
            seed = int(rng.integers(1, np.iinfo(np.int32).max))
            d = est.per[q]
            if theta_rows is not None:
                tr = np.asarray(theta_rows, dtype=np.float64).reshape(M, p)
                lam_arg = np.ones(M) if est.conditional else tr[:, q]
                th_arg = tr[:, off:off + k]
                lamb_arg = tr[:, P + q] if est.coevol else 0.0
                thb_arg = tr[:, off + k:p] if kb else None
            else:
                lam_arg, th_arg, lamb_arg, thb_arg = lam[q], th, lamb[q], (thb if kb else None)
            m = marshal_period(d["inp"], M, seed, lam_arg, th_arg, lamb=lamb_arg,
                               thetab=thb_arg, want_ends=keep_nets)
            if not scores:
                m.drop_outputs(("scores", "bscores"))
            ms.append(m)
        outs = engine.simulate_batch(ms)
    stats_acc = np.zeros((M, p))
    pieces, nets, z_ends = [], ([] if keep_nets else None), ([] if keep_nets and est.coevol else None)
    ntim = np.zeros((M, P))
    for q, r in enumerate(outs):
        sp = np.zeros((M, p))
        scp = np.zeros((M, p))
        scores = (r["scores"].astype(np.float64) if "scores" in r
                  else np.zeros((M, k + 1)))
        bscores = r["bscores"] if "bscores" in r else np.zeros((M, kb + 1))
        if not est.conditional:
            sp[:, q] = r["dist_stat"] + est.rate_consts[q]
            scp[:, q] = scores[:, 0]
        if est.coevol:
            d = est.per[q]
            bstats = engine.behavior_stats(r["z_end"], est.bty, d["xnet"], d["inp"].bkdist,
                                           est.data.beh.overall_mean, est.data.beh.range,
                                           est.data.beh.sim_mean)
            sp[:, P + q] = r["bdist"]
            scp[:, P + q] = bscores[:, 0]
            sp[:, off + k:p] = bstats
            scp[:, off + k:p] = bscores[:, 1:kb + 1]
            if keep_nets:
                z_ends.append(r["z_end"])
        sp[:, off:off + k] = r["stats"]
        scp[:, off:off + k] = scores[:, 1:k + 1]
        ntim[:, q] = r["ntim"]
        stats_acc += sp
        pieces.append((sp, scp))
        if keep_nets:
            nets.append(r["a_ends"])
    return SimRound(stats_acc, pieces, ntim, nets, z_ends)


def mom_derivative(pieces) -> np.ndarray:
    """Score-function derivative summed per period (R/mom.R:173-182)."""
    p = pieces[0][0].shape[1]
    M = pieces[0][0].shape[0]
    Dm = np.zeros((p, p))
    for sp, scp in pieces:
        s_c = sp - sp.mean(axis=0)
        sc_c = scp - scp.mean(axis=0)
        Dm += s_c.T @ sc_c / M
    return Dm


def mom_dinv(Dm, diagonalize):
    mix = (1 - diagonalize) * Dm + diagonalize * np.diag(np.diag(Dm))
    return safe_solve(mix)


def guard_step(est: Estimator, theta, step):
    """Step cap and rate floor (R/mom.R:189-197)."""
    cap = np.maximum(1.0, 0.5 * np.abs(theta))
    step = np.minimum(np.maximum(step, -cap), cap)
    n_rates = 0 if est.conditional else (2 * est.P if est.coevol else est.P)
    for m in range(n_rates):
        if theta[m] - step[m] < 0.1 * theta[m]:
            step[m] = 0.5 * theta[m]
    return step


def default_theta0(est: Estimator):
    """R/mom.R:199-211."""
    ev0 = np.array([-1.0 if e.name == "density" else 0.0 for e in est.effects])
    if est.conditional:
        return ev0
    rate_t = est.targets[:est.P]
    lam0 = 1.5 * rate_t / est.n + 1.0
    if est.coevol:
        bd = est.targets[est.P:2 * est.P]
        return np.concatenate([lam0, 1.5 * bd / est.n + 1.0, ev0, np.zeros(est.kb)])
    return np.concatenate([lam0, ev0])


@dataclass
class MomFit:
    theta: np.ndarray
    se: np.ndarray
    tconv: np.ndarray
    tconv_max: float
    param_names: list
    targets: np.ndarray
    sim_means: np.ndarray
    D: np.ndarray
    msf: np.ndarray
    conditional: bool
    rate_est: np.ndarray | None
    rate_sd: np.ndarray | None
    n_sims: int
    wall_time: float
    backend: str
    sims: list | None = None
    sims_behavior: list | None = None
    phase_times: dict = field(default_factory=dict)


def phase3(est, theta, engine, rng, n3, return_nets=False):
    """Phase 3 (R/mom.R:250-258): D, msf, convergence t-ratios and SEs."""
    s = mom_simulate(est, theta, n3, rng, engine, keep_nets=return_nets)
    Dm = mom_derivative(s.pieces)
    dinv = safe_solve(Dm)
    msf = np.cov(s.stats, rowvar=False)
    msf = np.atleast_2d(msf)
    dev = s.stats.mean(axis=0) - est.targets
    with np.errstate(divide="ignore", invalid="ignore"):
        tconv = dev / np.sqrt(np.diag(msf))
    tconv_max = float(np.sqrt(dev @ safe_solve(msf) @ dev))
    cov = dinv @ msf @ dinv.T
    se = np.sqrt(np.abs(np.diag(cov)))
    return s, Dm, msf, dev, tconv, tconv_max, se


def mom_run(est: Estimator, theta0=None, engine=None, verbose=False, return_nets=False,
            backend="gpu") -> MomFit:
    """The Robbins-Monro loop (R/mom.R:215-269)."""
    engine = engine or GpuEngine()
    ctl = est.control
    t0 = time.perf_counter()
    n2 = list(ctl["n2"])
    n_sims = ctl["n1"] + ctl["n3"] + sum(ctl["nD"] + n2[s] * ctl["batch2"] for s in range(ctl["nsub"]))
    rng = np.random.Generator(np.random.PCG64(int(ctl["seed"])))
    theta = np.asarray(theta0 if theta0 is not None else default_theta0(est), dtype=np.float64)
    times = {}
    # phase 1
    ta = time.perf_counter()
    s = mom_simulate(est, theta, ctl["n1"], rng, engine)
    dinv = mom_dinv(mom_derivative(s.pieces), ctl["diagonalize"])
    dev = s.stats.mean(axis=0) - est.targets
    theta = theta - guard_step(est, theta, 0.5 * ctl["firstg"] * (dinv @ dev))
    times["phase1"] = time.perf_counter() - ta
    if verbose:
        print("[phase 1] theta =", np.round(theta, 3))
    # phase 2
    ta = time.perf_counter()
    for sub in range(ctl["nsub"]):
        gain = ctl["firstg"] * (0.5 ** sub)
        s = mom_simulate(est, theta, ctl["nD"], rng, engine)
        dinv = mom_dinv(mom_derivative(s.pieces), ctl["diagonalize"])
        thav = np.zeros(est.p)
        for _ in range(int(n2[sub])):
            s = mom_simulate(est, theta, ctl["batch2"], rng, engine, scores=False)
            dev = s.stats.mean(axis=0) - est.targets
            theta = theta - guard_step(est, theta, gain * (dinv @ dev))
            thav += theta
        theta = thav / n2[sub]
        if verbose:
            print(f"[phase 2.{sub + 1}] gain={gain:.3f} theta = {np.round(theta, 3)}")
    times["phase2"] = time.perf_counter() - ta
    # phase 3
    ta = time.perf_counter()
    s, Dm, msf, dev, tconv, tconv_max, se = phase3(est, theta, engine, rng, ctl["n3"], return_nets)
    times["phase3"] = time.perf_counter() - ta
    rate_est = s.ntim.mean(axis=0) if est.conditional else None
    rate_sd = s.ntim.std(axis=0, ddof=1) if est.conditional else None
    return MomFit(theta, se, tconv, tconv_max, est.param_names, est.targets,
                  s.stats.mean(axis=0), Dm, msf, est.conditional, rate_est, rate_sd,
                  int(n_sims), time.perf_counter() - t0, backend, s.nets, s.z_ends, times)


def native_problems(est: Estimator):
    """The periods as the C estimator takes them: one marshalled problem per
    period (host arrays; M, seed, theta and lam are placeholders the estimator
    overwrites)."""
    if est.kb or est.coevol or any(d["inp"].nrate for d in est.per):
        raise ValueError("cusna_mom_estimate fits network effects only (no behaviour or rate effects)")
    return [marshal_period(d["inp"], 1, 1, 1.0, np.zeros(est.k)) for d in est.per]


def mom_run_native(est: Estimator, theta0=None, use_graph: bool = True) -> MomFit:
    """The Robbins-Monro fit through the library's C entry point
    cusna_mom_estimate (the same phases as mom_run, run in C++ over replayable
    plans, with no Python between rounds). Network-effect models only."""
    import ctypes as C
    from . import abi
    lib = abi.load_library()
    ms = native_problems(est)
    probs = (abi.SaomProblem * est.P)(*[m.problem for m in ms])
    ctl = est.control
    n2 = np.ascontiguousarray(ctl["n2"], dtype=np.int32)
    rc = np.ascontiguousarray(est.rate_consts, dtype=np.float64)
    tg = np.ascontiguousarray(est.targets, dtype=np.float64)
    o = abi.MomOptions(struct_version=abi.ABI_VERSION, conditional=int(est.conditional),
                       firstg=float(ctl["firstg"]), nsub=int(ctl["nsub"]), n2=n2.ctypes.data,
                       batch2=int(ctl["batch2"]), n1=int(ctl["n1"]), nD=int(ctl["nD"]),
                       n3=int(ctl["n3"]), diagonalize=float(ctl["diagonalize"]) or -1.0,
                       seed=int(ctl["seed"]) or 1234, rate_consts=rc.ctypes.data,
                       use_graph=1 if use_graph else -1)
    p, P = est.p, est.P
    out = {x: np.zeros(p) for x in ("theta", "se", "tconv", "sim_means")}
    out["D"], out["msf"] = np.zeros((p, p)), np.zeros((p, p))
    out["rate_est"], out["rate_sd"] = np.zeros(P), np.zeros(P)
    if theta0 is not None:
        out["theta"][:] = theta0
    r = abi.MomResult(struct_version=abi.ABI_VERSION, use_start=int(theta0 is not None),
                      **{x: a.ctypes.data for x, a in out.items()})
    st = lib.cusna_mom_estimate(probs, P, tg.ctypes.data, p, C.byref(o), C.byref(r))
    if st != 0:
        raise RuntimeError(f"cusna_mom_estimate failed ({st}): {lib.cusna_last_error().decode()}")
    times = dict(zip(("phase1", "phase2", "phase3"), r.phase_seconds))
    return MomFit(out["theta"], out["se"], out["tconv"], float(r.tconv_max), est.param_names,
                  est.targets, out["sim_means"], out["D"], out["msf"], est.conditional,
                  out["rate_est"] if est.conditional else None,
                  out["rate_sd"] if est.conditional else None, int(r.n_sims),
                  float(r.wall_seconds), "gpu-native", phase_times=times)


def mom_control(firstg=0.4, nsub=4, n2=(40, 40, 60, 80), batch2=256, n1=1000, n3=4000,
                nD=1000, diagonalize=0.2, seed=1234) -> dict:
    """Control settings (R/estimate.R:21-28)."""
    return dict(firstg=firstg, nsub=int(nsub), n2=tuple(float(x) for x in n2),
                batch2=int(batch2), n1=int(n1), n3=int(n3), nD=int(nD),
                diagonalize=diagonalize, seed=int(seed))


def mom_estimate(data: D.CusnaData, effects, beh_effects=None, rate_effects=None,
                 conditional=False, maxdegree=0, control=None, verbose=False,
                 return_nets=False, engine=None) -> MomFit:
    """Method-of-Moments estimation of a SAOM (R/estimate.R:66-98)."""
    if not isinstance(data, D.CusnaData):
        raise ValueError("`data` must be created with saom_data().")
    if not effects:
        raise ValueError("`effects` must be a non-empty list of cusna_effect objects.")
    specs = E.build_specs(effects)
    bspecs = [E.make_beh_effect_spec(e.name) for e in beh_effects] if beh_effects else None
    rspecs = [E.make_rate_effect_spec(e["name"], e.get("cov")) for e in rate_effects] if rate_effects else None
    ctl = dict(control or mom_control())
    ctl["maxdegree"] = int(maxdegree)
    ctl["n2"] = tuple(int(x) for x in ctl["n2"])
    est = mom_estimator(data.internal, specs, bspecs, rspecs, conditional, ctl, engine)
    return mom_run(est, engine=engine, verbose=verbose, return_nets=return_nets)


def saom_simulate(data: D.CusnaData, effects, theta, nsim=100, beh_effects=None,
                  conditional=False, maxdegree=0, seed=None, return_nets=True, engine=None):
    """Forward simulation at fixed theta (R/simulate.R:24-59)."""
    specs = E.build_specs(effects)
    bspecs = [E.make_beh_effect_spec(e.name) for e in beh_effects] if beh_effects else None
    est = mom_estimator(data.internal, specs, bspecs, None, conditional,
                        dict(maxdegree=int(maxdegree)), engine)
    theta = np.asarray(theta, dtype=np.float64)
    if theta.shape != (est.p,) or np.isnan(theta).any():
        raise ValueError(f"`theta` must have {est.p} values ({', '.join(est.param_names)}), "
                         "the layout of coef() for this model.")
    rng = np.random.Generator(np.random.PCG64(0 if seed is None else int(seed)))
    s = mom_simulate(est, theta, int(nsim), rng, engine or GpuEngine(), keep_nets=return_nets)
    return dict(stats=s.stats, targets=est.targets, theta=theta,
                durations=s.ntim if est.conditional else None, nets=s.nets,
                behavior=s.z_ends, nsim=int(nsim), n_periods=est.P,
                conditional=est.conditional, param_names=est.param_names)
