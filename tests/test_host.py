"""Host-side conventions against the reference's fixtures: data masks
(fixtures/data/*.json.gz, bit-exact), effect descriptors (effects.json.gz,
1e-9) and moment targets (targets.json.gz, 1e-7), the tolerances of
tests/testthat/test-data.R, test-effects.R and test-targets.R."""
import gzip
import json
import os

import numpy as np
import pytest

from cusna_gb300 import data as D
from cusna_gb300 import effects as E
from cusna_gb300 import targets as T

DATA_SETS = ["s50", "s50_beh", "s50miss", "s50str", "knecht", "cow", "synth"]


def _arr(x, dtype=np.float64):
    return np.array([[np.nan if v is None else v for v in row] for row in x], dtype=dtype) \
        if isinstance(x[0], list) else np.array([np.nan if v is None else v for v in x], dtype=dtype)


def load(fixtures_dir, *parts):
    return json.load(gzip.open(os.path.join(fixtures_dir, *parts)))


@pytest.mark.parametrize("name", DATA_SETS)
def test_data_conventions_match_fixture(fixtures_dir, name):
    g = load(fixtures_dir, "data", f"{name}.json.gz")
    waves = [np.array(w, dtype=np.float64) for w in g["waves_input"]]
    beh = None if g["behavior_input"] is None else _arr(g["behavior_input"])
    d = D.build_saom_data(waves, behavior=beh, composition=g["composition_input"],
                          cc_option=g["meta"]["cc_option"])
    assert d.symmetric == g["meta"]["symmetric"]
    assert d.has_composition == g["meta"]["has_composition"]
    for m in range(d.n_waves):
        np.testing.assert_array_equal(d.imputed[m], np.array(g["imputed"][m]))
        np.testing.assert_array_equal(d.miss[m], np.array(g["miss"][m]) != 0)
        np.testing.assert_array_equal(d.struct[m], np.array(g["struct"][m]) != 0)
        np.testing.assert_array_equal(d.rawvals[m], np.array(g["rawvals"][m]))
    if g["comp_active"] is not None:
        np.testing.assert_array_equal(d.comp_active, np.array(g["comp_active"]) != 0)
    for p, per in enumerate(g["periods"], start=1):
        np.testing.assert_array_equal(D.kmask_dist(d, p), np.array(per["kmask_dist"]) != 0)
        assert D.observed_distance(d, p) == per["observed_distance"]
        assert D.rate_target(d, p) == per["rate_target"]
        assert D.rate_const(d, p) == per["rate_const"]
        np.testing.assert_array_equal(D.rate_target_rows(d, p), per["rate_target_rows"])
        np.testing.assert_array_equal(D.rate_const_rows(d, p), per["rate_const_rows"])
        np.testing.assert_array_equal(D.network_less_missing(d, p), per["network_less_missing"])
        np.testing.assert_array_equal(D.network_less_missing_start(d, p),
                                      per["network_less_missing_start"])
        keep, force = D.stat_keep_force(d, p)
        np.testing.assert_array_equal(keep, np.array(per["keep"]) != 0)
        np.testing.assert_array_equal(force, np.array(per["force"]) != 0)
        keepS, forceS = D.stat_keep_force_struct(d, p)
        np.testing.assert_array_equal(keepS, np.array(per["keepS"]) != 0)
        np.testing.assert_array_equal(forceS, np.array(per["forceS"]) != 0)
        np.testing.assert_array_equal(D.target_network(d, p), per["target_network"])
        np.testing.assert_array_equal(D.permitted(d, p), np.array(per["permitted"]) != 0)
    if g["behavior"] is not None:
        b, gb = d.beh, g["behavior"]
        assert b.zmin == gb["zmin"] and b.zmax == gb["zmax"] and b.range == gb["range"]
        np.testing.assert_allclose(b.overall_mean, gb["overall_mean"], rtol=1e-14)
        np.testing.assert_allclose(b.sim_mean, gb["sim_mean"], rtol=1e-12)
        np.testing.assert_array_equal(b.imputed, np.array(gb["imputed"]))
        np.testing.assert_array_equal(b.miss, np.array(gb["miss"]) != 0)
        for p, per in enumerate(gb["periods"], start=1):
            np.testing.assert_array_equal(D.beh_kmask_dist(b, p), np.array(per["kmask_dist"]) != 0)
            assert D.beh_observed_distance(b, p) == per["observed_distance"]
            np.testing.assert_allclose(D.beh_values_less_missing_starts(b, p),
                                       per["values_less_missing_starts"], rtol=1e-15)
            np.testing.assert_allclose(D.beh_stat_values(b, b.imputed[:, p], p),
                                       per["stat_values_target"], rtol=1e-12, atol=1e-15)


def test_effect_descriptors_match_fixture(fixtures_dir):
    g = load(fixtures_dir, "effects", "effects.json.gz")
    n = g["n"]
    inp = g["inputs"]
    v_change = _arr(inp["v_change"])
    covs = dict(v_const=_arr(inp["v_const"]), v_change=v_change, v_miss=_arr(inp["v_miss"]),
                dyad_const=_arr(inp["dyad_const"]),
                dyad_change=np.stack([np.array(m) for m in g["dyad_change"]], axis=2))
    beh = D.build_behavior_data(v_change, n, 3)

    def build(r):
        if r.get("interaction"):
            return E.make_interaction_spec(r["comps"])
        return E.make_effect_spec(r["name"], cov=covs.get(r.get("cov")), parm=r.get("parm"),
                                  dyn=bool(r.get("dyn")), etype=r.get("etype") or "eval",
                                  net_ref=r.get("net_ref"))

    for cfg in g["configs"]:
        effs = [build(r) for r in cfg["recipe"]]
        p = cfg["period"] + 1
        use_beh = bool(cfg.get("use_beh"))
        z_start = D.beh_values_less_missing_starts(beh, p) if use_beh else None
        pe = E.prepare_effects_v2(effs, n, p, beh if use_beh else None, z_start)
        name = cfg["name"]
        np.testing.assert_array_equal(pe.type_ids, cfg["type_ids"], name)
        np.testing.assert_allclose(pe.p1, cfg["p1"], rtol=1e-9, atol=1e-12, err_msg=name)
        np.testing.assert_allclose(pe.p2, cfg["p2"], rtol=1e-9, atol=1e-12, err_msg=name)
        np.testing.assert_allclose(pe.vmat, _arr(cfg["vmat"]), rtol=1e-9, atol=1e-12, err_msg=name)
        np.testing.assert_array_equal(pe.dyn_flags, cfg["dyn_flags"], name)
        np.testing.assert_allclose(pe.v_dyn, cfg["v_dyn"], rtol=1e-9, atol=1e-12, err_msg=name)
        np.testing.assert_array_equal(pe.dyc_idx, cfg["dyc_idx"], name)
        np.testing.assert_array_equal(pe.vmiss.ravel(), cfg["vmiss"], name)
        if cfg.get("dymats"):
            for j, dm in enumerate(cfg["dymats"]):
                np.testing.assert_allclose(pe.dymats[j], _arr(dm), rtol=1e-9, atol=1e-12)
        np.testing.assert_allclose(E.effect_wtabs(effs, n), _arr(cfg["wtab"]), rtol=1e-9,
                                   atol=1e-12, err_msg=name)
        np.testing.assert_array_equal(E.interaction_comp_idx(effs), np.array(cfg["int_idx"]), name)
        np.testing.assert_array_equal(E.effect_etypes(effs), cfg["etypes"], name)
        np.testing.assert_array_equal(E.effect_netrefs(effs), cfg["netrefs"], name)
        if cfg.get("typed_F"):
            for j, e in enumerate(effs):
                np.testing.assert_allclose(E.typed_pair_matrix(e, n, p), _arr(cfg["typed_F"][j]),
                                           rtol=1e-9, atol=1e-12)
    for parm, w in g["gwesp_weights"].items():
        np.testing.assert_allclose(E.gwesp_weights(float(parm), n), w, rtol=1e-12)


def test_moment_targets_match_fixture(fixtures_dir, port):
    g = load(fixtures_dir, "targets", "targets.json.gz")
    covs = dict(alc_const=_arr(g["inputs"]["alc_const"]), alc_change=_arr(g["inputs"]["alc_change"]))
    for cfg in g["configs"]:
        waves = [np.array(w, dtype=np.float64) for w in cfg["waves_input"]]
        beh = None if cfg["behavior_input"] is None else _arr(cfg["behavior_input"])
        d = D.build_saom_data(waves, behavior=beh, composition=cfg["composition_input"])
        effs = [E.make_effect_spec(r["name"], cov=covs.get(r.get("cov")), parm=r.get("parm"),
                                   dyn=bool(r.get("dyn")), etype=r.get("etype") or "eval",
                                   net_ref=r.get("net_ref")) for r in cfg["effects"]]
        bef = [E.make_beh_effect_spec(x) for x in cfg["beh_effects"]] if cfg["beh_effects"] else None
        ref = [E.make_rate_effect_spec(r["name"], covs.get(r.get("cov")))
               for r in cfg["rate_effects"]] if cfg["rate_effects"] else None
        mt = T.mom_targets(d, effs, port.network_stats, bef, ref, cfg["conditional"],
                           beh_stats=port.behavior_stats)
        o = cfg["out"]
        tol = dict(rtol=1e-7, atol=1e-7, err_msg=cfg["name"])
        np.testing.assert_allclose(mt.eval, _arr(o["eval_targets"]), **tol)
        np.testing.assert_allclose(mt.basic_rate, o["rate_targets"], **tol)
        if o.get("beh_targets") is not None:
            np.testing.assert_allclose(mt.beh, _arr(o["beh_targets"]), **tol)
            np.testing.assert_allclose(mt.beh_rate, o["bdists"], **tol)
        if o.get("rate_eff_targets") is not None:
            np.testing.assert_allclose(mt.rate_eff.sum(axis=0), o["rate_eff_targets"], **tol)
        np.testing.assert_allclose(mt.target_vector, o["target_vector"], **tol)
