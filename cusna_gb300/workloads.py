"""Seeded synthetic workloads of the period simulator.

The reference's benchmark panel data are not used. Seeded synthetic panels
with the published shapes, sizes and densities stand in for them:

  c2_period()   n=200, 4096 chains, 8 evaluation effects, unconditional
  c4_period()   n=1000, 1024 chains, network-behaviour co-evolution
  c1_panel()    n=50, 3 waves (waves 2-3 simulated from a seed)
  parity_case() small problems covering every effect type and struct option

All networks have a zero diagonal; covariates are rounded to float32 and
centred in float64 as R/effects.R:139-147 centres them.
"""
from __future__ import annotations

import numpy as np

from . import data as D
from . import effects as E
from .glue import PeriodInputs


def bernoulli_net(n: int, p: float, seed: int) -> np.ndarray:
    rng = np.random.Generator(np.random.PCG64(seed))
    a = (rng.random((n, n)) < p).astype(np.uint8)
    np.fill_diagonal(a, 0)
    return a


def normal_cov(n: int, seed: int) -> np.ndarray:
    rng = np.random.Generator(np.random.PCG64(seed))
    return rng.standard_normal(n).astype(np.float32).astype(np.float64)


def period_inputs(x0, effects, p: int = 1, beh=None, z_start=None, beh_effects=None,
                  conditional=0, target_dist=0, symflag=0) -> PeriodInputs:
    """Descriptors of one period from effect specs (R/mom.R:62-76 conventions)."""
    n = np.asarray(x0).shape[0]
    pe = E.prepare_effects_v2(effects, n, p, beh, z_start)
    inp = PeriodInputs(x0=np.asarray(x0), type_ids=pe.type_ids, vmat=pe.vmat,
                       wtab=E.effect_wtabs(effects, n), vb=pe.v_dyn, p1=pe.p1, p2=pe.p2,
                       vmiss=pe.vmiss, dyn_flags=pe.dyn_flags, dyc_idx=pe.dyc_idx,
                       int_idx=E.interaction_comp_idx(effects) if any(E.is_interaction(e) for e in effects) else None,
                       etypes=E.effect_etypes(effects),
                       conditional=conditional, target_dist=target_dist, symflag=symflag)
    if beh_effects:
        inp.bty = np.array([e.type_id for e in beh_effects], dtype=np.int32)
        inp.z0 = np.asarray(z_start if z_start is not None else beh.imputed[:, p - 1]).astype(np.int32)
        inp.bkdist = D.beh_kmask_dist(beh, p).astype(np.int32)
        inp.zmin, inp.zmax = beh.zmin, beh.zmax
        inp.zbar, inp.brange, inp.bsimmean = beh.overall_mean, beh.range, beh.sim_mean
    return inp


# ---- C2: batched plain period simulation ------------------------------------
C2_THETA = np.array([-2.8, 1.8, 0.3, -0.1, 0.05, 0.2, 0.1, 0.8])
C2_EFFECTS = ["density", "recip", "transTrip", "cycle3", "inPop", "egoX", "altX", "simX"]


def c2_period(n: int = 200, M: int = 4096):
    """(PeriodInputs, M, seed, lam, theta) for the n=200 covariate workload."""
    x0 = bernoulli_net(n, 0.03, seed=2)
    cov = normal_cov(n, seed=3)
    effs = [E.make_effect_spec(nm) for nm in C2_EFFECTS[:5]]
    effs += [E.make_effect_spec(nm, cov) for nm in C2_EFFECTS[5:]]
    return period_inputs(x0, effs), M, 42, 8.0, C2_THETA.copy()


# ---- C4: network-behaviour co-evolution ------------------------------------
C4_THETA = np.array([-3.0, 2.0, 0.3, 0.1, 0.1, 0.5])
C4_THETAB = np.array([0.2, -0.1, 0.5])


def c4_period(n: int = 1000, M: int = 1024):
    """(PeriodInputs, M, seed, lam, theta, lamb, thetab) for n=1000 co-evolution.
    Behaviour starts uniform on 1..5; its summaries (mean, range, similarity
    mean) are those of the start wave."""
    x0 = bernoulli_net(n, 0.008, seed=5)
    rng = np.random.Generator(np.random.PCG64(6))
    z = rng.integers(1, 6, size=n).astype(np.float64)
    beh = D.build_behavior_data(np.stack([z, z], axis=1), n, 2)
    effs = [E.make_effect_spec(nm) for nm in ("density", "recip", "transTrip")]
    effs += [E.make_effect_spec(nm, dyn=True) for nm in ("egoX", "altX", "simX")]
    bef = [E.make_beh_effect_spec(nm) for nm in ("linear", "quad", "avAlt")]
    inp = period_inputs(x0, effs, 1, beh, D.beh_values_less_missing_starts(beh, 1), bef)
    inp.z0 = beh.imputed[:, 0].astype(np.int32)
    return inp, M, 77, 4.0, C4_THETA.copy(), 2.0, C4_THETAB.copy()


# ---- parity cases -----------------------------------------------------------

def _rng(seed):
    return np.random.Generator(np.random.PCG64(seed))


ALL_NET_TYPES = list(range(0, 32))  # 0..31; 32 = interaction built separately


def parity_case(kind: str, seed: int = 0, n: int = 40, M: int = 6):
    """Small problems for exact GPU-vs-CPU comparisons. Returns a dict with the
    PeriodInputs and the run arguments (M, seed, lam, theta, lamb, thetab)."""
    r = _rng(1000 + seed)
    x0 = bernoulli_net(n, 0.08, seed=seed + 17)
    cov = np.round(r.standard_normal(n), 3)
    bcov = (r.random(n) < 0.5).astype(np.float64)
    out = dict(M=M, seed=int(r.integers(1, 2**62)), lam=float(r.uniform(3, 8)), lamb=0.0,
               thetab=None)
    if kind == "baseline":
        effs = [E.make_effect_spec(x) for x in ("density", "recip", "transTrip")]
        theta = np.array([-2.0, 0.8, 0.15])
        inp = period_inputs(x0, effs)
    elif kind == "covariate":
        effs = [E.make_effect_spec(x) for x in ("density", "recip", "transTrip", "cycle3", "inPop")]
        effs += [E.make_effect_spec(x, cov) for x in ("egoX", "altX", "simX")]
        effs += [E.make_effect_spec("sameX", bcov)]
        theta = np.array([-2.2, 1.2, 0.2, -0.1, 0.05, 0.2, 0.1, 0.7, 0.3])
        inp = period_inputs(x0, effs)
    elif kind == "structural":
        names = ["density", "recip", "transTrip", "cycle3", "inPop", "transTies", "transRecTrip",
                 "inPopSqrt", "outPop", "outPopSqrt", "inAct", "inActSqrt", "outAct",
                 "outActSqrt", "outTrunc", "reciAct", "transTriads"]
        effs = [E.make_effect_spec(x) for x in names]
        theta = np.concatenate([[-1.5, 0.8, 0.1], r.uniform(-0.08, 0.08, len(names) - 3)])
        inp = period_inputs(x0, effs)
    elif kind == "gw":
        names = ["density", "recip", "gwesp", "gwespFB", "gwespBF", "gwespBB", "gwdspFF",
                 "gwdspFB"]
        effs = [E.make_effect_spec(x) for x in names]
        theta = np.array([-1.8, 0.7, 0.3, 0.2, -0.1, 0.1, -0.05, -0.05])
        inp = period_inputs(x0, effs)
    elif kind == "covariate_all":
        effs = [E.make_effect_spec("density")]
        for x in ("egoX", "altX", "simX", "sameX", "higher", "egoXaltX", "egoPlusAltX"):
            effs.append(E.make_effect_spec(x, cov if x != "sameX" else bcov))
        effs.append(E.make_effect_spec("altRThresholdX", cov, parm=0))
        theta = np.concatenate([[-2.0], r.uniform(-0.3, 0.3, len(effs) - 1)])
        inp = period_inputs(x0, effs)
    elif kind == "interaction":
        effs = [E.make_effect_spec(x) for x in ("density", "recip", "transTrip")]
        effs += [E.make_effect_spec("egoX", cov)]
        effs += [E.make_interaction_spec([1, 3]), E.make_interaction_spec([0, 2, 3])]
        theta = np.array([-2.0, 1.0, 0.2, 0.1, 0.3, -0.05])
        inp = period_inputs(x0, effs)
    elif kind == "typed":
        effs = [E.make_effect_spec("density"), E.make_effect_spec("recip"),
                E.make_effect_spec("egoPlusAltX", cov, etype="creation"),
                E.make_effect_spec("egoPlusAltX", cov, etype="endow")]
        theta = np.array([-2.0, 1.0, 0.2, -0.3])
        inp = period_inputs(x0, effs)
    elif kind == "coevol":
        z = r.integers(1, 6, size=(n, 2)).astype(np.float64)
        beh = D.build_behavior_data(z, n, 2)
        effs = [E.make_effect_spec(x) for x in ("density", "recip", "transTrip")]
        effs += [E.make_effect_spec(x, dyn=True) for x in ("egoX", "altX", "simX")]
        bef = [E.make_beh_effect_spec(x) for x in ("linear", "quad", "avAlt", "avSim", "totSim")]
        inp = period_inputs(x0, effs, 1, beh, D.beh_values_less_missing_starts(beh, 1), bef)
        theta = np.array([-2.0, 0.8, 0.2, 0.1, -0.1, 0.5])
        out.update(lamb=2.5, thetab=np.array([0.2, -0.1, 0.4, 0.3, -0.2]))
    elif kind == "conditional":
        effs = [E.make_effect_spec(x) for x in ("density", "recip", "transTrip")]
        theta = np.array([-2.0, 0.9, 0.2])
        inp = period_inputs(x0, effs, conditional=1, target_dist=int(0.6 * n))
        out["lam"] = 1.0
    elif kind == "masks":
        effs = [E.make_effect_spec(x) for x in ("density", "recip", "transTrip", "outTrunc")]
        effs[3].parm = 3.0
        theta = np.array([-1.8, 0.9, 0.2, 0.1])
        inp = period_inputs(x0, effs)
        off = ~np.eye(n, dtype=bool)
        inp.kdist = (r.random((n, n)) < 0.9) & off
        inp.perm = (r.random((n, n)) < 0.85) & off
        inp.keep = (r.random((n, n)) < 0.9) & off
        inp.force = (r.random((n, n)) < 0.02) & off
        inp.maxdegree = 6
        inp.sim_start = x0 & (r.random((n, n)) < 0.9)
        inp.od0 = x0.sum(axis=1)
        inp.id0 = x0.sum(axis=0)
    elif kind == "composition":
        effs = [E.make_effect_spec(x) for x in ("density", "recip", "transTrip")]
        theta = np.array([-2.0, 0.8, 0.2])
        inp = period_inputs(x0, effs)
        inactive = r.random(n) < 0.15
        act = np.concatenate([np.nonzero(~inactive)[0], np.nonzero(inactive)[0]])
        inp.act, inp.nact, inp.inactive = act.astype(np.int32), int((~inactive).sum()), inactive
    elif kind == "symmetric":
        a = np.triu(x0, 1)
        x0s = (a | a.T).astype(np.uint8)
        effs = [E.make_effect_spec(x) for x in ("density", "transTriads", "gwesp")]
        theta = np.array([-1.5, 0.2, 0.3])
        inp = period_inputs(x0s, effs, symflag=1)
    elif kind == "rates":
        effs = [E.make_effect_spec(x) for x in ("density", "recip", "transTrip")]
        theta = np.array([-2.0, 0.8, 0.2])
        inp = period_inputs(x0, effs)
        inp.rkind = np.array([0, 1, 2], dtype=np.int32)
        inp.ralpha = np.array([0.3, 0.05, -0.04], dtype=np.float32)
        inp.ru = np.stack([cov, np.zeros(n), np.zeros(n)]).astype(np.float32)
    else:
        raise ValueError(kind)
    out["inp"] = inp
    out["theta"] = theta
    return out


PARITY_KINDS = ["baseline", "covariate", "structural", "gw", "covariate_all", "interaction",
                "typed", "coevol", "conditional", "masks", "composition", "symmetric", "rates"]


# ---- C1: synthetic 3-wave panel, waves 2-3 simulated ------------------------
C1_THETA = np.array([-2.5, 2.0, 0.4])


def simulate_next_wave(engine, x, effects_names, lam, theta, seed):
    """One unconditional period from network x with the given effects; the end
    network of chain 0 is the next wave."""
    from .glue import marshal_period
    effs = [E.make_effect_spec(nm) for nm in effects_names]
    inp = period_inputs(x, effs)
    m = marshal_period(inp, 1, seed, lam, theta, want_ends=True)
    return engine.simulate_batch([m])[0]["a_ends"][0].astype(np.int64)


def c1_panel(engine, n: int = 50):
    """Wave 1 Bernoulli(0.05) (seed 1); waves 2 and 3 simulated with rate 6,
    density -2.5, recip 2.0, transTrip 0.4 (Philox seeds 11 and 12)."""
    names = ("density", "recip", "transTrip")
    w1 = bernoulli_net(n, 0.05, seed=1).astype(np.int64)
    w2 = simulate_next_wave(engine, w1, names, 6.0, C1_THETA, 11)
    w3 = simulate_next_wave(engine, w2, names, 6.0, C1_THETA, 12)
    return [w1, w2, w3]


# ---- C5: surrogate-assisted MoM panel ---------------------------------------
C5_LAMBDA = 7.0
C5_THETA = np.array([-2.6, 2.0, 0.35, -0.15, 0.04, 0.1, 0.9])
C5_EFFECTS = ["density", "recip", "transTrip", "cycle3", "inPop", "altX", "simX"]


def c5_effects(cov):
    """The seven evaluation effects of the n=300 surrogate panel."""
    return [E.make_effect_spec(nm, cov if nm.endswith("X") else None) for nm in C5_EFFECTS]


def c5_panel(engine, n: int = 300):
    """Wave 1 Bernoulli(0.03) (seed 7), covariate N(0,1) (seed 8); waves 2 and 3
    simulated with rate 7 and C5_THETA (Philox seeds 21 and 22). Returns
    (waves, covariate)."""
    from .glue import marshal_period
    cov = normal_cov(n, seed=8)
    effs = c5_effects(cov)
    waves = [bernoulli_net(n, 0.03, seed=7).astype(np.int64)]
    for seed in (21, 22):
        m = marshal_period(period_inputs(waves[-1], effs), 1, seed, C5_LAMBDA, C5_THETA,
                           want_ends=True)
        waves.append(engine.simulate_batch([m])[0]["a_ends"][0].astype(np.int64))
    return waves, cov


def c5_theta_true() -> np.ndarray:
    """The data-generating parameter vector in the unconditional estimator's
    layout (rate per period, then the evaluation effects)."""
    return np.concatenate([[C5_LAMBDA, C5_LAMBDA], C5_THETA])


# ---- C3: uneven multi-group panel --------------------------------------------
C3_THETA = np.array([-2.5, 2.0, 0.4, 0.5])
C3_EFFECTS = ["density", "recip", "transTrip", "sameX"]


def c3_effects(cov):
    """density, recip, transTrip and sameX of the group's binary covariate."""
    return [E.make_effect_spec(nm, cov if nm == "sameX" else None) for nm in C3_EFFECTS]


def c3_groups(engine, n_groups: int = 512, seed: int = 4, lam: float = 6.0):
    """Groups of n ~ Uniform{20..400} actors with wave-1 density ~ Uniform[0.02,
    0.10] and a binary covariate ~ Bernoulli(0.5) (numpy PCG64 streams from
    `seed`); waves 2 and 3 simulated for all groups in one batched call per wave
    with rate `lam` and C3_THETA (Philox seeds 31 + group, 41 + group).
    Returns a list of (waves, covariate) per group."""
    from .glue import marshal_period
    r = np.random.Generator(np.random.PCG64(seed))
    ns = r.integers(20, 401, size=n_groups)
    dens = r.uniform(0.02, 0.10, size=n_groups)
    covs = [(r.random(int(n)) < 0.5).astype(np.float64) for n in ns]
    waves = [[bernoulli_net(int(n), float(p), seed=seed * 100003 + g).astype(np.int64)]
             for g, (n, p) in enumerate(zip(ns, dens))]
    for w, base in ((1, 31), (2, 41)):
        ms = [marshal_period(period_inputs(waves[g][-1], c3_effects(covs[g])), 1, base + g, lam,
                             C3_THETA, want_ends=True) for g in range(n_groups)]
        outs = engine.simulate_batch(ms)
        for g in range(n_groups):
            waves[g].append(outs[g]["a_ends"][0].astype(np.int64))
    return [(waves[g], covs[g]) for g in range(n_groups)]


# ---- multi-network parity cases ------------------------------------------------
MULTI_KINDS = ["cross", "typed_cov", "symmetric", "dyadic", "empty_net"]


def multi_case(kind: str, seed: int = 0, n: int = 40, M: int = 4, D: int = 2):
    """Small multi-network periods for exact GPU-vs-CPU comparisons: D start
    networks on n actors, per-network effects with cross-network effects of
    every type (33..37) reading the other networks. "dyadic" adds a dyadic
    covariate effect (type 22) and reciAct (19, which the multi-network engine
    evaluates with a reciprocated degree of 0); "empty_net" leaves the last
    network without effects (its ministeps choose uniformly). Returns
    (MultiInputs, seed, lam (D,), theta (k,))."""
    from .glue import MultiInputs
    r = _rng(2000 + seed)
    x0s = [bernoulli_net(n, 0.06 + 0.02 * d, seed=seed * 31 + d) for d in range(D)]
    cov = np.round(r.standard_normal(n), 3)
    effs, netof, th, dyadic = [], [], [], []
    for d in range(D):
        src = (d + 1) % D
        if kind == "empty_net" and d == D - 1:
            continue
        if kind == "cross":
            spec = [("density", None, None, -2.0), ("recip", None, None, 0.9),
                    ("transTrip", None, None, 0.15), ("crprod", None, src, 0.6),
                    ("crprodRecip", None, src, 0.3), ("crprodMutual", None, src, -0.2),
                    ("from", None, src, 0.1), ("to", None, src, 0.05)]
        elif kind == "typed_cov":
            spec = [("density", None, None, -2.1), ("recip", None, None, 1.0),
                    ("inPop", None, None, 0.05), ("altX", cov, None, 0.2),
                    ("simX", cov, None, 0.5), ("egoPlusAltX", cov, None, 0.3),
                    ("crprod", None, src, 0.7)]
        elif kind == "symmetric":
            spec = [("density", None, None, -1.6), ("transTriads", None, None, 0.2),
                    ("crprod", None, src, 0.5)]
        elif kind == "dyadic":
            spec = [("density", None, None, -2.0), ("recip", None, None, 0.8),
                    ("X", None, None, 0.9), ("reciAct", None, None, 0.1),
                    ("to", None, src, 0.2)]
        elif kind == "empty_net":
            spec = [("density", None, None, -1.9), ("recip", None, None, 0.7),
                    ("crprod", None, D - 1, 0.8), ("from", None, D - 1, 0.1)]
        else:
            raise ValueError(kind)
        for name, cv, ref, t in spec:
            # the dyadic covariate effect reads the multi problem's dyc; its
            # descriptor row is a density row with the type id set afterwards
            dyadic.append(name == "X")
            e = E.make_effect_spec("density" if name == "X" else name, cv, net_ref=ref)
            if name == "egoPlusAltX":
                e = E.make_effect_spec(name, cv, etype="creation" if d == 0 else "endow")
            effs.append(e)
            netof.append(d)
            th.append(t)
    pe = E.prepare_effects_v2(effs, n, 1, None, None)
    symf = np.ones(D, np.int32) if kind == "symmetric" else np.zeros(D, np.int32)
    if kind == "symmetric":
        x0s = [((np.triu(x, 1) | np.triu(x, 1).T) != 0).astype(np.uint8) for x in x0s]
    p1 = np.asarray(pe.p1, dtype=np.float64).copy()
    for q, e in enumerate(effs):
        if e.name == "from":
            p1[q] = 2.0 if seed % 2 else 1.0   # square-root variant on odd seeds
    tids = np.asarray(pe.type_ids, np.int32).copy()
    dyc_idx = -np.ones(len(effs), np.int32)
    dyc = None
    if any(dyadic):
        tids[np.asarray(dyadic)] = E.EFF_X
        dyc_idx[np.asarray(dyadic)] = 0
        dyc = np.round(r.standard_normal((n, n)), 3)
        np.fill_diagonal(dyc, 0.0)
    inp = MultiInputs(x0s=x0s, type_ids=tids,
                      netof=np.asarray(netof, np.int32), netref=E.effect_netrefs(effs),
                      etypes=E.effect_etypes(effs), wtab=E.effect_wtabs(effs, n), p1=p1,
                      p2=np.asarray(pe.p2), vmat=np.asarray(pe.vmat), symf=symf, dyc=dyc,
                      dyc_idx=dyc_idx)
    lam = np.array([3.0 + 1.5 * d + r.uniform(0, 1) for d in range(D)])
    return inp, int(r.integers(1, 2 ** 62)), lam, np.array(th)


# ---- multi-network panels ------------------------------------------------------
# Two co-evolving networks on 50 actors with density and recip each, the shape
# of the reference's multi-network estimation test; parameters near its fit.
MN_LAMBDA = np.array([5.3, 7.5])
MN_THETA = np.array([-2.15, 2.3, -2.4, 2.9])   # net0 density, recip, net1 density, recip


def multinet_panel(simulate_multi, n: int = 50, seed: int = 12):
    """Wave 1 of each network Bernoulli(0.045) (seeds 12, 13); wave 2 of both
    simulated jointly at MN_LAMBDA, MN_THETA (Philox seed 31) through
    simulate_multi (a marshalled multi-network period -> outputs). Returns the
    waves of each network."""
    from .glue import MultiInputs, marshal_multi
    x0s = [bernoulli_net(n, 0.045, seed=seed + d) for d in range(2)]
    specs = [E.make_effect_spec(nm) for nm in ("density", "recip")] * 2
    pe = E.prepare_effects_v2(specs, n, 1, None, None)
    inp = MultiInputs(x0s=x0s, type_ids=np.asarray(pe.type_ids, np.int32),
                      netof=np.array([0, 0, 1, 1], np.int32), netref=E.effect_netrefs(specs),
                      etypes=E.effect_etypes(specs), wtab=E.effect_wtabs(specs, n), p1=pe.p1,
                      p2=pe.p2, vmat=pe.vmat, symf=np.zeros(2, np.int32))
    out = simulate_multi(marshal_multi(inp, 1, 31, MN_LAMBDA, MN_THETA))
    ends = np.asarray(out["a_ends"]).reshape(2, n, n)
    return [[x0s[d].astype(np.int64), ends[d].astype(np.int64)] for d in range(2)]
