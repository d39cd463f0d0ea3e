"""Effect registry and float64 effect descriptors.

A Python restatement of the reference's R effect layer R/effects.R (cran/cusna
0.1.1): the name -> type-id table, default parameters, gwesp weights and
prepare_effects_v2, which builds the descriptor arrays the C ABI consumes. The
reference fixture tests/testthat/fixtures/effects/effects.json.gz pins it.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

# numeric effect ids shared with the simulator (R/effects.R:14-23)
EFF = dict(
    density=0, recip=1, transTrip=2, cycle3=3, inPop=4, transTies=5, transRecTrip=6,
    inPopSqrt=7, outPop=8, outPopSqrt=9, egoX=10, altX=11, simX=12, sameX=13,
    inAct=14, inActSqrt=15, outAct=16, outActSqrt=17, outTrunc=18, reciAct=19,
    higher=20, egoXaltX=21, X=22, transTriads=23, gwesp=24, egoPlusAltX=25,
    gwespFB=26, gwespBF=27, gwespBB=28, gwdspFF=29, gwdspFB=30, altRThresholdX=31,
    interaction=32, crprod=33, crprodRecip=34, crprodMutual=35, **{"from": 36}, to=37)

STRUCTURAL = dict(density=0, recip=1, transTrip=2, cycle3=3, inPop=4, transTies=5,
                  transRecTrip=6, inPopSqrt=7, outPop=8, outPopSqrt=9, inAct=14,
                  inActSqrt=15, outAct=16, outActSqrt=17, outTrunc=18, reciAct=19,
                  transTriads=23, gwesp=24, gwespFF=24, gwespFB=26, gwespBF=27,
                  gwespBB=28, gwdspFF=29, gwdspFB=30)                  # R/effects.R:25-30
COVARIATE = dict(egoX=10, altX=11, simX=12, sameX=13, higher=20, egoXaltX=21,
                 egoPlusAltX=25, altRThresholdX=31)                    # :31-32
CROSSNET = dict(crprod=33, crprodRecip=34, crprodMutual=35, to=37, **{"from": 36})
DYADIC = dict(X=22)
GW_FAMILY = (24, 26, 27, 28, 29, 30)
CROSS_IDS = (33, 34, 35, 36, 37)
RATE_KINDS = dict(RateX=0, outRate=1, inRate=2)
BEH_NAMES = dict(linear=0, quad=1, avAlt=2, avSim=3, totSim=4)
ETYPES = dict(eval=0, creation=1, endow=2)
EFF_SIMX, EFF_X, EFF_ALTRTHRX, EFF_EGOPLUSALTX, EFF_INTERACTION = 12, 22, 31, 25, 32
DEG_P1 = (18, 8, 9, 14, 15)
DEFAULT_PARM = dict(outTrunc=1.0, outPop=1.0, inAct=1.0, outPopSqrt=0.0, inActSqrt=0.0,
                    gwesp=69.0, gwespFF=69.0, gwespFB=69.0, gwespBF=69.0, gwespBB=69.0,
                    gwdspFF=69.0, gwdspFB=69.0, altRThresholdX=0.0)   # :45-48
INT_COERCE = ("gwesp", "gwespFF", "gwespFB", "gwespBF", "gwespBB", "gwdspFF",
              "gwdspFB", "altRThresholdX")


def gwesp_weights(parm, n: int) -> np.ndarray:
    """RSiena GwespFunction cumulative weights w[s] = e^a (1 - (1 - e^-a)^s),
    w[0] = 0 (R/effects.R:53-63). Sequential float64 loop as in the reference."""
    alpha = 0.01 * float(parm)
    w = np.zeros(n + 1)
    factor = 1.0 - math.exp(-alpha)
    pw = 1.0
    ea = math.exp(alpha)
    for s in range(1, n + 1):
        pw = pw * factor
        w[s] = ea * (1.0 - pw)
    return w


@dataclass
class EffectSpec:
    name: str
    type_id: int
    cov: object = None
    parm: float = 1.0
    dyn: bool = False
    etype: str = "eval"
    net_ref: int | None = None
    needs_cov: bool = False
    comps: tuple = ()


def make_effect_spec(name, cov=None, parm=None, dyn=False, etype="eval",
                     net_ref=None) -> EffectSpec:
    """R/effects.R:66-111."""
    if etype not in ETYPES:
        raise ValueError(f"unknown effect type {etype}")
    spec = EffectSpec(name=name, type_id=-1, cov=cov, parm=parm, dyn=bool(dyn),
                      etype=etype, net_ref=net_ref)
    if name in CROSSNET:
        if net_ref is None:
            raise ValueError(f"{name} requires net_ref (the other dependent network index)")
        spec.type_id = CROSSNET[name]
        spec.needs_cov = False
        if spec.parm is None:
            spec.parm = DEFAULT_PARM.get(name, 1.0)
        return spec
    if name in STRUCTURAL:
        spec.type_id = STRUCTURAL[name]
        spec.needs_cov = False
    elif name in COVARIATE:
        spec.type_id = COVARIATE[name]
        spec.needs_cov = not spec.dyn
        if spec.cov is None and spec.needs_cov:
            raise ValueError(f"{name} requires a covariate")
    elif name in DYADIC:
        spec.type_id = DYADIC[name]
        spec.needs_cov = True
        w = None if spec.cov is None else np.asarray(spec.cov)
        if w is None or w.ndim not in (2, 3) or w.shape[0] != w.shape[1]:
            raise ValueError(f"{name} requires an (n,n) or (n,n,periods) dyadic covariate")
    else:
        raise ValueError(f"unknown effect {name}")
    if spec.parm is None:
        spec.parm = DEFAULT_PARM.get(name, 1.0)
    if name in INT_COERCE:
        spec.parm = float(math.trunc(spec.parm))
    return spec


def make_beh_effect_spec(name) -> EffectSpec:
    if name not in BEH_NAMES:
        raise ValueError(f"unknown behavior effect {name}")
    return EffectSpec(name=name, type_id=BEH_NAMES[name])


def make_rate_effect_spec(name, cov=None) -> dict:
    if name not in RATE_KINDS:
        raise ValueError(f"unknown rate effect {name}")
    kind = RATE_KINDS[name]
    if kind == 0 and cov is None:
        raise ValueError("RateX requires a covariate")
    return dict(name=name, cov=cov, kind=kind)


def make_interaction_spec(comps) -> EffectSpec:
    """comps are 0-based positions (R/effects.R:129-134)."""
    c0 = tuple(int(c) for c in comps)
    if len(c0) not in (2, 3):
        raise ValueError("interaction needs 2 or 3 components")
    return EffectSpec(name="unspInt", type_id=EFF_INTERACTION, comps=c0, parm=1.0)


def is_interaction(e) -> bool:
    return e.type_id == EFF_INTERACTION


def _cov_array(v):
    return np.array(v, dtype=np.float64)


def effect_cov_values(spec: EffectSpec, p: int = 1) -> np.ndarray:
    """Centred covariate of period p (grand mean over all columns), :139-147."""
    v = _cov_array(spec.cov)
    gmean = np.nanmean(v)
    if v.ndim <= 1:
        return v.ravel() - gmean
    col = min(p, v.shape[1])
    return v[:, col - 1] - gmean


def effect_sim_params(spec: EffectSpec) -> tuple[float, float]:
    """(1/range, simMean) pooled over covariate columns, :150-166."""
    v = _cov_array(spec.cov)
    rng = np.nanmax(v) - np.nanmin(v)
    cols = v.reshape(-1, 1) if v.ndim <= 1 else v
    tot, cnt = 0.0, 0
    for m in range(cols.shape[1]):
        x = cols[~np.isnan(cols[:, m]), m]
        if len(x) > 1:
            d = 1.0 - np.abs(x[:, None] - x[None, :]) / rng
            tot += float(d.sum()) - len(x)
            cnt += len(x) * (len(x) - 1)
    with np.errstate(divide="ignore"):   # R: 1/0 = Inf
        inv = np.float64(1.0) / np.float64(rng)
    return float(inv), (tot / cnt if cnt > 0 else 0.0)


def rate_cov_values(spec: dict, p: int = 1) -> np.ndarray:
    v = _cov_array(spec["cov"])
    gmean = np.nanmean(v)
    vm = v.ravel() - gmean if v.ndim <= 1 else v[:, min(p, v.shape[1]) - 1] - gmean
    return np.where(np.isnan(vm), 0.0, vm)


@dataclass
class Descriptors:
    type_ids: np.ndarray
    p1: np.ndarray
    p2: np.ndarray
    vmat: np.ndarray
    dyn_flags: np.ndarray
    v_dyn: np.ndarray
    dymats: list
    dyc_idx: np.ndarray
    vmiss: np.ndarray


def prepare_effects_v2(effects, n: int, p: int = 1, beh=None, z_start=None) -> Descriptors:
    """float64 descriptor bundle for period p (R/effects.R:176-238)."""
    k = len(effects)
    type_ids = np.array([int(e.type_id) for e in effects], dtype=np.int32)
    p1 = np.zeros(k); p2 = np.zeros(k)
    vmat = np.zeros((k, n)); vmiss = np.zeros((k, n), dtype=np.int32)
    dyn_flags = np.array([1 if e.dyn else 0 for e in effects], dtype=np.int32)
    dymats = []
    dyc_idx = np.full(k, -1, dtype=np.int32)
    off = ~np.eye(n, dtype=bool)
    for idx, e in enumerate(effects):
        t = int(e.type_id)
        if t == EFF_SIMX:
            if e.dyn:
                if beh is not None:
                    with np.errstate(divide="ignore"):   # R: 1/0 = Inf
                        p1[idx] = np.float64(1.0) / np.float64(beh.range)
                    p2[idx] = beh.sim_mean
            else:
                p1[idx], p2[idx] = effect_sim_params(e)
        elif t in DEG_P1:
            p1[idx] = float(e.parm)
        elif t == EFF_ALTRTHRX:
            p1[idx] = float(math.trunc(e.parm))
        elif t in CROSS_IDS:
            p1[idx] = float(e.parm)
        if t == EFF_X:
            w = np.array(e.cov, dtype=np.float64)
            if w.ndim == 3:
                flat = w.reshape(n * n, w.shape[2], order="F")
                gmean = np.nanmean(flat[off.ravel(order="F"), :])
                wm = w[:, :, min(p, w.shape[2]) - 1] - gmean
            else:
                wm = w - np.mean(w[off])
            wm = wm.copy()
            np.fill_diagonal(wm, 0.0)
            dymats.append(wm)
            dyc_idx[idx] = len(dymats) - 1
        elif e.needs_cov and not e.dyn:
            vv = effect_cov_values(e, p)
            if len(vv) != n:
                raise ValueError(f"{e.name}: covariate length != n")
            miss = np.isnan(vv)
            vmiss[idx, :] = miss.astype(np.int32)
            vmat[idx, :] = np.where(miss, 0.0, vv)
        elif e.dyn and beh is not None:
            vmiss[idx, :] = beh.miss[:, min(p, beh.miss.shape[1]) - 1].astype(np.int32)
    if (dyn_flags == 1).any() and beh is not None and z_start is not None:
        v_dyn = np.asarray(z_start, dtype=np.float64) - beh.overall_mean
    else:
        v_dyn = np.zeros(n)
    return Descriptors(type_ids, p1, p2, vmat, dyn_flags, v_dyn, dymats, dyc_idx, vmiss)


def interaction_comp_idx(effects) -> np.ndarray:
    """(k,3) 0-based component indices, -1 padded (R/effects.R:241-262)."""
    k = len(effects)
    out = np.full((k, 3), -1, dtype=np.int32)
    for ei, e in enumerate(effects):
        if not is_interaction(e):
            continue
        for slot, ci in enumerate(e.comps):
            if not (0 <= ci < ei):
                raise ValueError(f"interaction component {ci} must precede position {ei}")
            comp = effects[ci]
            if is_interaction(comp):
                raise ValueError("nested interactions not supported")
            if comp.etype != "eval":
                raise ValueError("interaction components must be eval effects")
            out[ei, slot] = ci
    return out


def effect_etypes(effects) -> np.ndarray:
    """R/effects.R:265-274."""
    out = []
    for e in effects:
        et = ETYPES[e.etype or "eval"]
        if et != 0 and e.type_id != EFF_EGOPLUSALTX:
            raise ValueError("creation/endowment types are supported for egoPlusAltX only")
        out.append(et)
    return np.array(out, dtype=np.int32)


def effect_netrefs(effects) -> np.ndarray:
    return np.array([-1 if e.net_ref is None else int(e.net_ref) for e in effects],
                    dtype=np.int32)


def effect_wtabs(effects, n: int) -> np.ndarray:
    """(k, n+1) gwesp/gwdsp weight tables (R/effects.R:285-294)."""
    tabs = np.zeros((len(effects), n + 1))
    for i, e in enumerate(effects):
        if int(e.type_id) in GW_FAMILY:
            tabs[i, :] = gwesp_weights(e.parm, n)
    return tabs


def typed_pair_matrix(spec: EffectSpec, n: int, p: int = 1) -> np.ndarray:
    """(n,n) f_ij for a typed egoPlusAltX effect (R/effects.R:297-312)."""
    if int(spec.type_id) != EFF_EGOPLUSALTX:
        raise ValueError("typed_pair_matrix supports egoPlusAltX only")
    v = effect_cov_values(spec, p)
    cov = _cov_array(spec.cov)
    miss = np.isnan(cov.ravel()) if cov.ndim <= 1 else np.isnan(cov[:, min(p, cov.shape[1]) - 1])
    vv = np.where(miss, 0.0, v)
    ok2 = ~(miss[:, None] | miss[None, :])
    f = (vv[:, None] + vv[None, :]) * ok2
    np.fill_diagonal(f, 0.0)
    return f


# ---- public model-specification constructors (R/effects.R:333-411) ----------

@dataclass
class CusnaEffect:
    name: str
    covariate: object = None
    parameter: float | None = None
    dyn: bool = False
    type: str = "eval"
    net_ref: int | None = None


def cusna_effect(name, covariate=None, parameter=None, dyn=False, type="eval",
                 net_ref=None) -> CusnaEffect:
    if type not in ("eval", "creation", "endow"):
        raise ValueError("type must be eval, creation or endow")
    if not isinstance(name, str):
        raise ValueError("`name` must be a single effect name (a string).")
    return CusnaEffect(name, covariate, parameter, bool(dyn), type, net_ref)


@dataclass
class CusnaBehEffect:
    name: str


def cusna_beh_effect(name) -> CusnaBehEffect:
    if not isinstance(name, str):
        raise ValueError("`name` must be a single behavior-effect name (a string).")
    return CusnaBehEffect(name)


@dataclass
class CusnaInteraction:
    components: tuple


def cusna_interaction(components) -> CusnaInteraction:
    comps = tuple(int(c) for c in components)
    if len(comps) < 2 or len(comps) > 3 or any(c < 1 for c in comps):
        raise ValueError("`components` must be 2 or 3 positive positions in the effects list.")
    return CusnaInteraction(comps)


def build_specs(effects) -> list:
    """Model specs -> internal specs; 1-based positions become 0-based
    (R/estimate.R:32-45)."""
    out = []
    for e in effects:
        if isinstance(e, CusnaInteraction):
            out.append(make_interaction_spec([c - 1 for c in e.components]))
        elif isinstance(e, CusnaEffect):
            out.append(make_effect_spec(e.name, cov=e.covariate, parm=e.parameter, dyn=e.dyn,
                                        etype=e.type,
                                        net_ref=None if e.net_ref is None else int(e.net_ref) - 1))
        else:
            raise ValueError("`effects` must contain cusna_effect / cusna_interaction objects.")
    return out
