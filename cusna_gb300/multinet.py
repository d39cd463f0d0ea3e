"""Multi-network co-evolution: data container and the Method-of-Moments
estimator over the multi-network simulator.

A Python restatement of the reference's R/multinet.R (saom_multinet_data,
mom_estimate_multinet) and R/mom.R:281-479 (.batch_net_stats,
.multi_mom_estimator, .multi_default_theta0, .multi_guard_step,
.multi_mom_simulate, .multi_mom_run). Estimation is unconditional: per network
one basic rate per period, then that network's effects. Each simulation round
runs all chains of a period in one cusna_saom_simulate_multi call; the
statistics of the end networks (evaluation and cross-network) are computed on
the GPU too (cusna_network_stats_gpu, cusna_cross_stats).

The engine is pluggable as in cusna_gb300.mom: `MultiGpuEngine` (the product)
or any object with `simulate_multi(m)`, `network_stats_batch(A, ...)` and
`cross_stats(A, wp, t, parm)`; the tests pass the CPU oracle the same way.
"""
from __future__ import annotations

import time
from dataclasses import dataclass

import numpy as np

from . import data as D
from . import effects as E
from .glue import MultiInputs, marshal_multi
from .mom import DEFAULT_CONTROL, MomFit, mom_derivative, mom_dinv, safe_solve


class MultiGpuEngine:
    """The GB300 multi-network simulator and statistics."""

    def simulate_multi(self, m) -> dict:
        from . import sim
        return sim.simulate_multi(m)

    def network_stats_batch(self, A, n, k, *desc) -> np.ndarray:
        from . import sim
        return np.atleast_2d(sim.network_stats(A, n, k, *desc))

    def cross_stats(self, A, wp, t, parm) -> np.ndarray:
        from . import sim
        return sim.cross_stats(A, wp, t, parm)


@dataclass
class MultiNetData:
    """One SaomData per network over one actor set (R/multinet.R:10-23)."""
    nets: list
    D: int
    n: int
    n_periods: int


@dataclass
class CusnaMultinetData:
    """User-facing container (saom_multinet_data, R/multinet.R:37-56)."""
    internal: MultiNetData
    n_networks: int
    n_waves: int
    n_periods: int


def saom_multinet_data(waves_list, composition=None, cc_option=1) -> CusnaMultinetData:
    """Several dependent networks over one actor set (R/multinet.R:37-56)."""
    if not isinstance(waves_list, (list, tuple)) or len(waves_list) < 2:
        raise ValueError("`waves_list` must be a list of >= 2 networks, each a list of wave "
                         "matrices.")
    n_waves = len(waves_list[0])
    for net in waves_list:
        if not isinstance(net, (list, tuple)) or len(net) < 2:
            raise ValueError("each network must be a list of >= 2 wave matrices.")
        if len(net) != n_waves:
            raise ValueError("all networks must have the same number of waves.")
    nets = [D.build_saom_data([np.asarray(w) for w in net], composition=composition,
                              cc_option=cc_option) for net in waves_list]
    n0, p0 = nets[0].n, nets[0].n_periods
    for d, nd in enumerate(nets):
        if nd.n != n0:
            raise ValueError(f"network {d + 1}: actor set size differs")
        if nd.n_periods != p0:
            raise ValueError(f"network {d + 1}: wave count differs")
    internal = MultiNetData(nets, len(nets), n0, p0)
    return CusnaMultinetData(internal, len(waves_list), n_waves, n_waves - 1)


def batch_net_stats(engine, a_masked, effects, net: D.SaomData, cross_pred, p: int,
                    symflag: int) -> np.ndarray:
    """(M, k) statistics of masked end networks a_masked (M, n, n) for one
    network's effects: evaluation effects by the network statistics, cross
    effects against the source network's period-start predictor
    (R/mom.R:281-307)."""
    a_masked = np.asarray(a_masked)
    M, n = a_masked.shape[0], a_masked.shape[1]
    k = len(effects)
    tids = np.array([int(e.type_id) for e in effects])
    is_cross = np.isin(tids, E.CROSS_IDS)
    out = np.zeros((M, k))
    nc = np.flatnonzero(~is_cross)
    if nc.size:
        sub = [effects[q] for q in nc]
        pe = E.prepare_effects_v2(sub, n, p, None, None)
        wtab = E.effect_wtabs(sub, n)
        a_start = net.imputed[p - 1]
        od0 = a_start.sum(axis=1).astype(np.int32)
        id0 = a_start.sum(axis=0).astype(np.int32)
        out[:, nc] = engine.network_stats_batch(a_masked, n, len(sub), pe.type_ids, pe.p1, pe.p2,
                                                pe.vmat, pe.vmiss, pe.dyn_flags, pe.v_dyn, od0,
                                                id0, wtab, symflag)
    for q in np.flatnonzero(is_cross):
        e = effects[q]
        wp = cross_pred[int(e.net_ref)]
        out[:, q] = engine.cross_stats(a_masked, wp, int(e.type_id), float(e.parm or 0.0))
    return out


@dataclass
class MultiEstimator:
    """Estimator context (R/mom.R:309-363)."""
    mn: MultiNetData
    D: int
    P: int
    n: int
    k: int
    p: int
    effects: list
    specs_by_net: list
    netof: np.ndarray
    rate_pos: np.ndarray        # (D, P)
    eff_pos: np.ndarray         # (k,)
    symf: np.ndarray
    targets: np.ndarray
    rate_targets: np.ndarray    # (D, P)
    rate_consts: np.ndarray     # (D, P)
    cross_pred: list            # per period: per network the start predictor
    param_names: list
    control: dict


def multi_mom_estimator(mn: MultiNetData, specs_by_net, control=None,
                        engine=None) -> MultiEstimator:
    ctl = dict(DEFAULT_CONTROL)
    ctl.update(control or {})
    engine = engine or MultiGpuEngine()
    Dn, P, n, nets = mn.D, mn.n_periods, mn.n, mn.nets
    effects = [e for effs in specs_by_net for e in effs]
    netof = np.array([d for d in range(Dn) for _ in specs_by_net[d]], dtype=np.int32)
    k = len(effects)
    rate_pos = np.zeros((Dn, P), dtype=np.int64)
    eff_pos = np.zeros(k, dtype=np.int64)
    names, pos, eidx = [], 0, 0
    for d in range(Dn):
        for m in range(P):
            rate_pos[d, m] = pos
            pos += 1
            names.append(f"rate net{d} (p{m + 1})")
        for e in specs_by_net[d]:
            eff_pos[eidx] = pos
            eidx += 1
            pos += 1
            nr = "" if e.net_ref is None else f"<-net{e.net_ref}"
            names.append(f"net{d} {e.name}{nr}")
    p = pos
    symf = np.array([1 if nd.symmetric else 0 for nd in nets], dtype=np.int32)
    rate_targets = np.array([[float(D.rate_target(nd, m)) for m in range(1, P + 1)] for nd in nets])
    rate_consts = np.array([[float(D.rate_const(nd, m)) for m in range(1, P + 1)] for nd in nets])
    cross_pred = [[D.network_less_missing_start(nd, m) for nd in nets] for m in range(1, P + 1)]
    targets = np.zeros(p)
    for d in range(Dn):
        for m in range(P):
            targets[rate_pos[d, m]] = rate_targets[d, m]
    eidx = 0
    for d in range(Dn):
        eff_d = specs_by_net[d]
        if eff_d:
            for m in range(1, P + 1):
                tg = batch_net_stats(engine, D.target_network(nets[d], m)[None], eff_d, nets[d],
                                     cross_pred[m - 1], m, int(symf[d]))
                for q in range(len(eff_d)):
                    targets[eff_pos[eidx + q]] += tg[0, q]
        eidx += len(eff_d)
    return MultiEstimator(mn, Dn, P, n, k, p, effects, list(specs_by_net), netof, rate_pos,
                          eff_pos, symf, targets, rate_targets, rate_consts, cross_pred, names, ctl)


def multi_default_theta0(est: MultiEstimator) -> np.ndarray:
    """R/mom.R:365-374."""
    th = np.zeros(est.p)
    for d in range(est.D):
        for m in range(est.P):
            th[est.rate_pos[d, m]] = 1.5 * est.rate_targets[d, m] / est.n + 1.0
    for q, e in enumerate(est.effects):
        if e.name == "density":
            th[est.eff_pos[q]] = -1.0
    return th


def multi_guard_step(est: MultiEstimator, theta, step) -> np.ndarray:
    """Step cap and rate floor (R/mom.R:376-384)."""
    cap = np.maximum(1.0, 0.5 * np.abs(theta))
    step = np.minimum(np.maximum(step, -cap), cap)
    for d in range(est.D):
        for m in range(est.P):
            q = est.rate_pos[d, m]
            if theta[q] - step[q] < 0.1 * theta[q]:
                step[q] = 0.5 * theta[q]
    return step


@dataclass
class MultiRound:
    stats: np.ndarray     # (M, p) summed over periods
    pieces: list          # per period (sp, scp)
    ntim: np.ndarray      # (M, P)


def multi_mom_simulate(est: MultiEstimator, theta, M: int, rng, engine) -> MultiRound:
    """One round: every period's M chains in one multi-network call, then the
    rate statistics (distance over kdist), masked end networks and their
    statistics (R/mom.R:386-439)."""
    Dn, P, k, p, n, nets = est.D, est.P, est.k, est.p, est.n, est.mn.nets
    theta = np.asarray(theta, dtype=np.float64)
    th_flat = theta[est.eff_pos]
    wtab = E.effect_wtabs(est.effects, n)
    etypes = E.effect_etypes(est.effects)
    netref = E.effect_netrefs(est.effects)
    stats_acc = np.zeros((M, p))
    pieces = []
    ntim = np.zeros((M, P))
    for m in range(1, P + 1):
        lam_d = np.array([theta[est.rate_pos[d, m - 1]] for d in range(Dn)])
        seed = int(rng.integers(1, np.iinfo(np.int32).max))
        pe_m = E.prepare_effects_v2(est.effects, n, m, None, None)
        inp = MultiInputs(x0s=[nd.imputed[m - 1] for nd in nets], type_ids=pe_m.type_ids,
                          netof=est.netof, netref=netref, etypes=etypes, wtab=wtab,
                          p1=pe_m.p1, p2=pe_m.p2, vmat=pe_m.vmat,
                          perm=[D.permitted(nd, m) for nd in nets], symf=est.symf)
        r = engine.simulate_multi(marshal_multi(inp, M, seed, lam_d, th_flat))
        rscores = np.asarray(r["rscores"], dtype=np.float64).reshape(M, Dn)
        scores = np.asarray(r["scores"], dtype=np.float64).reshape(M, k)
        a_ends = np.asarray(r["a_ends"]).reshape(M, Dn, n, n)
        sp = np.zeros((M, p))
        scp = np.zeros((M, p))
        eidx = 0
        for d in range(Dn):
            nd = nets[d]
            x0d = nd.imputed[m - 1] != 0
            kdist = D.kmask_dist(nd, m)
            keep, force = D.stat_keep_force(nd, m)
            ad = a_ends[:, d] != 0
            dist_stat = ((ad != x0d[None]) & kdist[None]).sum(axis=(1, 2))
            a_masked = ((ad & keep[None]) | force[None]).astype(np.uint8)
            q = est.rate_pos[d, m - 1]
            sp[:, q] = dist_stat + est.rate_consts[d, m - 1]
            scp[:, q] = rscores[:, d]
            eff_d = est.specs_by_net[d]
            if eff_d:
                sd = batch_net_stats(engine, a_masked, eff_d, nd, est.cross_pred[m - 1], m,
                                     int(est.symf[d]))
                for qq in range(len(eff_d)):
                    sp[:, est.eff_pos[eidx + qq]] = sd[:, qq]
                    scp[:, est.eff_pos[eidx + qq]] = scores[:, eidx + qq]
            eidx += len(eff_d)
        ntim[:, m - 1] = r["ntim"]
        stats_acc += sp
        pieces.append((sp, scp))
    return MultiRound(stats_acc, pieces, ntim)


def multi_mom_run(est: MultiEstimator, theta0=None, engine=None, verbose=False,
                  backend="gpu") -> MomFit:
    """The unconditional Robbins-Monro loop (R/mom.R:441-479)."""
    engine = engine or MultiGpuEngine()
    ctl = est.control
    t0 = time.perf_counter()
    n2 = list(ctl["n2"])
    n_sims = ctl["n1"] + ctl["n3"] + sum(ctl["nD"] + n2[s] * ctl["batch2"]
                                         for s in range(ctl["nsub"]))
    rng = np.random.Generator(np.random.PCG64(int(ctl["seed"])))
    theta = np.asarray(theta0 if theta0 is not None else multi_default_theta0(est),
                       dtype=np.float64)
    times = {}
    ta = time.perf_counter()
    s = multi_mom_simulate(est, theta, ctl["n1"], rng, engine)
    dinv = mom_dinv(mom_derivative(s.pieces), ctl["diagonalize"])
    dev = s.stats.mean(axis=0) - est.targets
    theta = theta - multi_guard_step(est, theta, 0.5 * ctl["firstg"] * (dinv @ dev))
    times["phase1"] = time.perf_counter() - ta
    if verbose:
        print("[phase 1] theta =", np.round(theta, 3))
    ta = time.perf_counter()
    for sub in range(ctl["nsub"]):
        gain = ctl["firstg"] * (0.5 ** sub)
        s = multi_mom_simulate(est, theta, ctl["nD"], rng, engine)
        dinv = mom_dinv(mom_derivative(s.pieces), ctl["diagonalize"])
        thav = np.zeros(est.p)
        for _ in range(int(n2[sub])):
            s = multi_mom_simulate(est, theta, ctl["batch2"], rng, engine)
            dev = s.stats.mean(axis=0) - est.targets
            theta = theta - multi_guard_step(est, theta, gain * (dinv @ dev))
            thav += theta
        theta = thav / n2[sub]
        if verbose:
            print(f"[phase 2.{sub + 1}] theta = {np.round(theta, 3)}")
    times["phase2"] = time.perf_counter() - ta
    ta = time.perf_counter()
    s = multi_mom_simulate(est, theta, ctl["n3"], rng, engine)
    Dm = mom_derivative(s.pieces)
    dinv = safe_solve(Dm)
    msf = np.atleast_2d(np.cov(s.stats, rowvar=False))
    dev = s.stats.mean(axis=0) - est.targets
    with np.errstate(divide="ignore", invalid="ignore"):
        tconv = dev / np.sqrt(np.diag(msf))
    tconv_max = float(np.sqrt(dev @ safe_solve(msf) @ dev))
    se = np.sqrt(np.abs(np.diag(dinv @ msf @ dinv.T)))
    times["phase3"] = time.perf_counter() - ta
    return MomFit(theta, se, tconv, tconv_max, est.param_names, est.targets,
                  s.stats.mean(axis=0), Dm, msf, False, None, None, int(n_sims),
                  time.perf_counter() - t0, backend, None, None, times)


def mom_estimate_multinet(data: CusnaMultinetData, effects_by_net, control=None,
                          verbose=False, engine=None) -> MomFit:
    """Method-of-Moments estimation of a multi-network co-evolution model
    (R/multinet.R:69-98). effects_by_net: one list of cusna_effect objects per
    network; cross-network effects carry net_ref = the 1-based source network."""
    if not isinstance(data, CusnaMultinetData):
        raise ValueError("`data` must be created with saom_multinet_data().")
    if not isinstance(effects_by_net, (list, tuple)) or len(effects_by_net) != data.n_networks:
        raise ValueError("`effects_by_net` must be a list with one effects list per network "
                         f"({data.n_networks}).")
    specs_by_net = []
    for effs in effects_by_net:
        if not isinstance(effs, (list, tuple)):
            raise ValueError("each element of `effects_by_net` must be a list of effects.")
        specs_by_net.append(E.build_specs(effs))
    ctl = dict(control or {})
    if "n2" in ctl:
        ctl["n2"] = tuple(int(x) for x in ctl["n2"])
    est = multi_mom_estimator(data.internal, specs_by_net, ctl, engine)
    return multi_mom_run(est, engine=engine, verbose=verbose)
