"""SAOM panel data conventions: wave parsing, imputation, composition change,
behaviour summaries and the per-period masks the simulator and the moment
targets read.

A Python restatement of the reference's R data engine R/data.R (cran/cusna
0.1.1), which has no compiled counterpart. Periods are 1-based (p in 1..P,
spanning waves p and p+1) as in the reference. Every function cites the lines
it follows. The reference's data fixtures (tests/testthat/fixtures/data/*.json.gz)
pin these functions bit for bit.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

NA_CODE, STRUCT_ZERO, STRUCT_ONE = 9, 10, 11          # R/data.R:20-22


def _round_half_even(x):
    return np.round(np.asarray(x, dtype=np.float64))


def parse_wave(w) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """One raw wave -> (vals 0/1 int, miss bool, struct bool). R/data.R:27-55."""
    w = np.asarray(w)
    if w.ndim != 2 or w.shape[0] != w.shape[1]:
        raise ValueError("each wave must be a square matrix.")
    n = w.shape[0]
    if np.issubdtype(w.dtype, np.floating) and np.isnan(w).any():
        miss = np.isnan(w)
        wi = np.where(miss, 0.0, w)
        wi = np.trunc(wi).astype(np.int64)
    else:
        wi = _round_half_even(w).astype(np.int64)
        miss = wi == NA_CODE
    struct = (wi == STRUCT_ZERO) | (wi == STRUCT_ONE)
    vals = wi.copy()
    vals[wi == STRUCT_ZERO] = 0
    vals[wi == STRUCT_ONE] = 1
    vals[miss] = 0
    chk = vals[~miss & ~struct]
    if not np.isin(chk, (0, 1)).all():
        raise ValueError("tie values must be 0/1/9(NA)/10/11 or NaN")
    idx = np.arange(n)
    vals[idx, idx] = 0
    miss = miss.copy(); struct = struct.copy()
    miss[idx, idx] = False
    struct[idx, idx] = False
    return vals.astype(np.int64), miss, struct


@dataclass
class BehaviorData:
    """Dependent behaviour variable, R/data.R:213-259."""
    n: int
    n_waves: int
    values: np.ndarray           # n x nw float (NaN missing)
    miss: np.ndarray             # n x nw bool
    imputed: np.ndarray          # n x nw int
    overall_mean: float
    zmin: int
    zmax: int
    range: float
    sim_mean: float


def build_behavior_data(values, n: int, nw: int) -> BehaviorData:
    """R/data.R:213-259 (overallMean, range, simMean, imputation)."""
    v = np.array(values, dtype=np.float64).reshape(n, nw)
    miss = np.isnan(v)
    obs = v[~miss]
    wave_means = np.array([v[~miss[:, m], m].mean() for m in range(nw)])
    overall_mean = float(np.mean(wave_means))
    zmin, zmax = int(obs.min()), int(obs.max())
    rng = float(zmax - zmin)
    tot, cnt = 0.0, 0
    if nw >= 2:
        for m in range(nw - 1):
            x = v[~np.isnan(v[:, m]), m]
            if len(x) > 1:
                d = 1.0 - np.abs(x[:, None] - x[None, :]) / rng
                tot += float(d.sum()) - len(x)
                cnt += len(x) * (len(x) - 1)
    sim_mean = tot / cnt if cnt > 0 else 0.0
    imp = v.copy()
    allna = miss.all(axis=1)
    if allna.any():
        vals, counts = np.unique(obs, return_counts=True)
        imp[allna, :] = vals[np.argmax(counts)]
    first = imp[:, 0].copy()
    for m in range(1, nw):
        first = np.where(np.isnan(first), imp[:, m], first)
    imp[:, 0] = first
    for m in range(1, nw):
        imp[:, m] = np.where(np.isnan(imp[:, m]), imp[:, m - 1], imp[:, m])
    if np.isnan(imp).any():
        raise ValueError("behavior imputation failed.")
    imputed = _round_half_even(imp).astype(np.int64)
    return BehaviorData(n, nw, v, miss, imputed, overall_mean, zmin, zmax, rng, sim_mean)


@dataclass
class SaomData:
    """Internal SAOM data object, R/data.R:96-117."""
    n: int
    n_waves: int
    vals: list
    miss: list
    struct: list
    imputed: list
    rawvals: list
    symmetric: bool
    has_composition: bool = False
    comp_active: np.ndarray | None = None
    comp_intervals: list | None = None
    cc_option: int = 1
    beh: BehaviorData | None = None

    @property
    def n_periods(self) -> int:
        return self.n_waves - 1


def build_saom_data(waves, behavior=None, composition=None, cc_option=1) -> SaomData:
    """Parse, impute, test symmetry, apply composition and behaviour.
    R/data.R:60-118."""
    if not isinstance(waves, (list, tuple)) or len(waves) < 2:
        raise ValueError("`waves` must be a list of at least two adjacency matrices.")
    parsed = [parse_wave(w) for w in waves]
    n = parsed[0][0].shape[0]
    nw = len(parsed)
    for p in parsed:
        if p[0].shape[0] != n:
            raise ValueError("all waves must have the same node set.")
    vals = [p[0] for p in parsed]
    miss = [p[1] for p in parsed]
    struct = [p[2] for p in parsed]
    imputed = [vals[0].copy()]
    for m in range(1, nw):                                   # R/data.R:80-87
        w = vals[m].copy()
        mm = miss[m]
        w[mm] = imputed[m - 1][mm]
        imputed.append(w)
    symmetric = all(                                         # R/data.R:90-94
        np.array_equal(vals[m], vals[m].T) and np.array_equal(miss[m], miss[m].T)
        and np.array_equal(struct[m], struct[m].T) for m in range(nw))
    obj = SaomData(n=n, n_waves=nw, vals=vals, miss=[m.copy() for m in miss],
                   struct=struct, imputed=imputed, rawvals=[v.copy() for v in vals],
                   symmetric=bool(symmetric), cc_option=int(cc_option))
    if composition is not None:
        obj = apply_composition(obj, composition, cc_option)
    if behavior is not None:
        if composition is not None:
            raise ValueError("composition change with a dependent behavior is not supported.")
        obj.beh = build_behavior_data(behavior, n, nw)
    return obj


def apply_composition(obj: SaomData, composition, cc_option) -> SaomData:
    """RSiena composition-change data treatment, R/data.R:123-210."""
    n, nw = obj.n, obj.n_waves
    cc = int(cc_option)
    if cc not in (1, 2, 3):
        raise ValueError("ccOption must be 1, 2 or 3.")
    if len(composition) != n:
        raise ValueError("composition needs one interval list per actor.")
    intervals = []
    active_start = np.zeros((n, nw), dtype=bool)
    for j in range(n):
        flat = np.array(composition[j], dtype=np.float64).ravel()
        if len(flat) < 2 or len(flat) % 2 != 0:
            raise ValueError(f"actor {j + 1}: interval list must have an even length.")
        if not np.all(flat == np.round(flat)):
            raise ValueError(f"actor {j + 1}: only integer event times are supported.")
        pairs = []
        for q in range(len(flat) // 2):
            s, e = int(flat[2 * q]), int(flat[2 * q + 1])
            if not (1 <= s <= e <= nw):
                raise ValueError(f"actor {j + 1}: interval ({s},{e}) outside 1..{nw}")
            pairs.append((s, e))
            active_start[j, s - 1:e] = True
        intervals.append(pairs)
    action = np.zeros((n, nw), dtype=np.int64)
    for j in range(n):
        for m in range(nw):
            if active_start[j, m]:
                continue
            prec = active_start[j, :m].any() if m > 0 else False
            succ = active_start[j, m + 1:].any() if m < nw - 1 else False
            action[j, m] = 1 if not prec else (2 if not succ else 3)
    for m in range(nw):
        for code in (1, 3, 2):
            for j in np.nonzero(action[:, m] == code)[0]:
                row_na = obj.miss[m][j, :].copy()
                zero_branch = ((code == 1 and cc in (1, 2)) or (code == 3 and cc in (1, 2))
                               or (code == 2 and cc == 1))
                if zero_branch:
                    obj.miss[m][j, row_na] = False
                    obj.miss[m][row_na, j] = False
                    obj.rawvals[m][j, row_na] = 0
                    obj.rawvals[m][row_na, j] = 0
                    if code == 1 or m == 0:
                        obj.imputed[m][j, row_na] = 0
                        obj.imputed[m][row_na, j] = 0
                    else:
                        obj.imputed[m][j, row_na] = obj.imputed[m - 1][j, row_na]
                        obj.imputed[m][row_na, j] = obj.imputed[m - 1][row_na, j]
                else:
                    obj.miss[m][j, :] = True
                    obj.miss[m][:, j] = True
                    obj.miss[m][j, j] = False
    P = nw - 1
    obj.has_composition = True
    obj.comp_intervals = intervals
    obj.comp_active = active_start[:, :P].T.copy()           # P x n
    return obj


# ---------------------------------------------------------------- period masks
# R/data.R:264-362. p is 1-based; index python lists with p-1 / p.

def _offdiag_false(m):
    m = m.copy()
    np.fill_diagonal(m, False)
    return m


def kmask_dist(obj: SaomData, p: int) -> np.ndarray:
    k = ~(obj.miss[p - 1] | obj.miss[p] | obj.struct[p - 1] | obj.struct[p])
    return _offdiag_false(k)


def observed_distance(obj: SaomData, p: int) -> int:
    excl = obj.miss[p - 1] | obj.miss[p] | obj.struct[p - 1] | obj.struct[p]
    diff = (obj.rawvals[p - 1] != obj.rawvals[p]) & ~excl
    return int(_offdiag_false(diff).sum())


def _rate_diff(obj, p):
    a = (obj.imputed[p - 1] != 0) & ~obj.miss[p - 1]
    b = (obj.imputed[p] != 0) & ~obj.miss[p - 1] & ~obj.miss[p]
    diff = (a ^ b) & ~obj.struct[p - 1] & ~obj.struct[p]
    return _offdiag_false(diff)


def _rate_const_mask(obj, p):
    cc = ((obj.imputed[p - 1] != 0) & ~obj.miss[p - 1] & obj.miss[p]
          & ~obj.struct[p - 1] & ~obj.struct[p])
    return _offdiag_false(cc)


def rate_target(obj, p):
    return int(_rate_diff(obj, p).sum())


def rate_const(obj, p):
    return int(_rate_const_mask(obj, p).sum())


def rate_target_rows(obj, p):
    return _rate_diff(obj, p).sum(axis=1).astype(np.int64)


def rate_const_rows(obj, p):
    return _rate_const_mask(obj, p).sum(axis=1).astype(np.int64)


def network_less_missing(obj, p):
    return ((obj.imputed[p - 1] != 0) & ~obj.miss[p - 1]).astype(np.int64)


def network_less_missing_start(obj, p):
    return ((obj.imputed[p - 1] != 0) & ~obj.miss[p - 1] & ~obj.miss[p]).astype(np.int64)


def stat_keep_force(obj, p):
    """(keep, force): statistic network = (A & keep) | force. R/data.R:319-331."""
    keep = ~(obj.miss[p - 1] | obj.miss[p])
    force = np.zeros((obj.n, obj.n), dtype=bool)
    s1 = obj.struct[p]
    keep = keep & ~s1
    force[s1] = obj.imputed[p][s1] != 0
    s0 = obj.struct[p - 1]
    keep = keep & ~s0
    force[s0] = obj.imputed[p - 1][s0] != 0
    return _offdiag_false(keep), _offdiag_false(force)


def stat_keep_force_struct(obj, p):
    """Structural replacements only, R/data.R:335-347."""
    keep = np.ones((obj.n, obj.n), dtype=bool)
    force = np.zeros((obj.n, obj.n), dtype=bool)
    s1 = obj.struct[p]
    keep = keep & ~s1
    force[s1] = obj.imputed[p][s1] != 0
    s0 = obj.struct[p - 1]
    keep = keep & ~s0
    force[s0] = obj.imputed[p - 1][s0] != 0
    return _offdiag_false(keep), _offdiag_false(force)


def stat_network(obj, a, p):
    keep, force = stat_keep_force(obj, p)
    return (((np.asarray(a) != 0) & keep) | force).astype(np.int64)


def target_network(obj, p):
    return stat_network(obj, obj.imputed[p], p)


def permitted(obj, p):
    return _offdiag_false(~obj.struct[p - 1])


# ------------------------------------------------------- behaviour period masks
# R/data.R:366-383

def beh_kmask_dist(beh: BehaviorData, p: int) -> np.ndarray:
    return ~(beh.miss[:, p - 1] | beh.miss[:, p])


def beh_observed_distance(beh: BehaviorData, p: int) -> int:
    d = np.abs(beh.imputed[:, p] - beh.imputed[:, p - 1])
    return int(d[beh_kmask_dist(beh, p)].sum())


def beh_values_less_missing_starts(beh: BehaviorData, p: int) -> np.ndarray:
    return np.where(beh.miss[:, p - 1], 0.0, beh.imputed[:, p - 1].astype(np.float64))


def beh_stat_values(beh: BehaviorData, z_end, p: int) -> np.ndarray:
    u = np.asarray(z_end, dtype=np.float64) - beh.overall_mean
    u[~beh_kmask_dist(beh, p)] = 0.0
    return u


@dataclass
class CusnaData:
    """User-facing SAOM data container (saom_data(), R/data.R:405-423)."""
    internal: SaomData
    n: int
    n_waves: int
    n_periods: int
    has_behavior: bool
    has_composition: bool


def saom_data(waves, behavior=None, composition=None, cc_option=1) -> CusnaData:
    """Longitudinal SAOM data (R/data.R:405-423)."""
    if not isinstance(waves, (list, tuple)) or len(waves) < 2:
        raise ValueError("`waves` must be a list of at least two adjacency matrices.")
    mats = [np.asarray(w) for w in waves]
    for m in mats:
        if m.ndim != 2 or m.shape[0] != m.shape[1]:
            raise ValueError("each wave must be a square matrix.")
    n = mats[0].shape[0]
    if not all(m.shape[0] == n for m in mats):
        raise ValueError("all waves must share the same actor set (same dimension).")
    internal = build_saom_data(mats, behavior=behavior, composition=composition,
                               cc_option=cc_option)
    return CusnaData(internal, n, len(mats), len(mats) - 1, behavior is not None,
                     composition is not None)
