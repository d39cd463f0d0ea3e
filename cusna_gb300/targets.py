"""Moment targets of a SAOM fit: the observed-wave statistics Robbins-Monro
matches.

A Python restatement of the reference's R target assembly R/targets.R (cran/cusna
0.1.1). The statistic of one network and the behaviour statistics are delegated
to the functions passed in (`net_stats`, `beh_stats`). The product passes its
GPU implementations (cusna_network_stats_gpu / cusna_behavior_stats_gpu); the
tests also pass the CPU oracle, against the reference fixture
tests/testthat/fixtures/targets/targets.json.gz.

net_stats(a, n, k, type_ids, p1, p2, vmat, vmiss, dyn_flags, vb, od0, id0, wtab,
          symflag) -> (k,) float64
beh_stats(z_batch (M,n), bty, xnet, bkdist, zbar, brange, bsimmean) -> (M, kb)
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import data as D
from .effects import effect_wtabs, prepare_effects_v2, rate_cov_values


def eval_targets(data: D.SaomData, effects, net_stats, symflag=None) -> np.ndarray:
    """Per-period evaluation targets (P x k), R/targets.R:19-40."""
    n, P, k = data.n, data.n_periods, len(effects)
    beh = data.beh
    if symflag is None:
        symflag = 1 if data.symmetric else 0
    wtab = effect_wtabs(effects, n)
    out = np.zeros((P, k))
    for p in range(1, P + 1):
        z_start = D.beh_values_less_missing_starts(beh, p) if beh is not None else None
        pe = prepare_effects_v2(effects, n, p, beh, z_start)
        a_start = data.imputed[p - 1]
        a_tgt = D.target_network(data, p)
        od0 = a_start.sum(axis=1).astype(np.int32)
        id0 = a_start.sum(axis=0).astype(np.int32)
        out[p - 1, :] = net_stats(a_tgt, n, k, pe.type_ids, pe.p1, pe.p2, pe.vmat, pe.vmiss,
                                  pe.dyn_flags, pe.v_dyn, od0, id0, wtab, symflag)
    return out


def beh_targets(data: D.SaomData, beh_effects, beh_stats) -> np.ndarray:
    """Per-period behaviour targets (P x kb), R/targets.R:43-59."""
    beh = data.beh
    if beh is None:
        raise ValueError("behavior targets need co-evolving behavior data.")
    P, kb = data.n_periods, len(beh_effects)
    bty = np.array([e.type_id for e in beh_effects], dtype=np.int32)
    out = np.zeros((P, kb))
    for p in range(1, P + 1):
        z_end = beh.imputed[:, p]
        xnet = D.network_less_missing_start(data, p)
        bkdist = D.beh_kmask_dist(beh, p).astype(np.int32)
        out[p - 1, :] = np.asarray(beh_stats(z_end[None, :], bty, xnet, bkdist,
                                             beh.overall_mean, beh.range, beh.sim_mean)).ravel()
    return out


def basic_rate_targets(data: D.SaomData) -> np.ndarray:
    """R/targets.R:66-70 (composition gate)."""
    fn = D.rate_target if data.has_composition else D.observed_distance
    return np.array([float(fn(data, p)) for p in range(1, data.n_periods + 1)])


def rate_effect_targets(data: D.SaomData, rate_effects) -> np.ndarray:
    """R/targets.R:75-91."""
    P, nr = data.n_periods, len(rate_effects)
    out = np.zeros((P, nr))
    for p in range(1, P + 1):
        rows = D.rate_target_rows(data, p)
        for r, e in enumerate(rate_effects):
            kind = e["kind"]
            if kind == 0:
                w = rate_cov_values(e, p)
            elif kind == 1:
                w = D.network_less_missing(data, p).sum(axis=1)
            else:
                w = D.network_less_missing(data, p).sum(axis=0)
            out[p - 1, r] = float(np.sum(np.asarray(w, dtype=np.float64) * rows))
    return out


def beh_rate_targets(data: D.SaomData) -> np.ndarray:
    """R/targets.R:129-133."""
    return np.array([float(D.beh_observed_distance(data.beh, p))
                     for p in range(1, data.n_periods + 1)])


@dataclass
class MomTargets:
    eval: np.ndarray
    beh: np.ndarray | None
    basic_rate: np.ndarray
    rate_eff: np.ndarray | None
    beh_rate: np.ndarray | None
    target_vector: np.ndarray
    layout: list


def mom_targets(data: D.SaomData, effects, net_stats, beh_effects=None, rate_effects=None,
                conditional=True, beh_stats=None) -> MomTargets:
    """Targets and the theta-ordered target vector (R/targets.R:99-126).
    Layouts: unconditional [rate x P, rate-eff x nr, eval x k]; conditional
    [rate-eff x nr, eval x k]; coevolution [net rate x P, beh rate x P,
    eval x k, beh x kb]."""
    eval_t = eval_targets(data, effects, net_stats)
    basic = basic_rate_targets(data)
    rate_eff = rate_effect_targets(data, rate_effects) if rate_effects else None
    beh_t = beh_targets(data, beh_effects, beh_stats) if beh_effects else None
    bh_rate = beh_rate_targets(data) if beh_t is not None else None
    eval_vec = eval_t.sum(axis=0)
    parts, layout = [], []
    if beh_t is not None:
        parts += [basic, bh_rate, eval_vec, beh_t.sum(axis=0)]
        layout = ["net_rate", "beh_rate", "eval", "beh"]
    else:
        if not conditional:
            parts.append(basic); layout.append("rate")
        if rate_eff is not None:
            parts.append(rate_eff.sum(axis=0)); layout.append("rate_eff")
        parts.append(eval_vec); layout.append("eval")
    return MomTargets(eval_t, beh_t, basic, rate_eff, bh_rate,
                      np.concatenate([np.ravel(x) for x in parts]), layout)
