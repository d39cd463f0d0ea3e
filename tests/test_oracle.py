"""Pins the CPU oracle: against the reference's golden vectors (sim.json.gz),
against the reference engine compiled from its own sources, against the
committed golden vectors, and against the published Philox4x32-10 answers."""
import gzip
import json
import os

import numpy as np
import pytest

from cusna_gb300 import data as D
from cusna_gb300 import effects as E
from cusna_gb300 import workloads as WL
from cusna_gb300.glue import PeriodInputs, marshal_period
from tests.conftest import GOLDEN
from tests.golden.make_golden import SEEDS, case_digest, run_case

# Random123 known-answer vectors for philox4x32 with 10 rounds
PHILOX_KAT = [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]


def test_philox_known_answers(port):
    for ctr, key, want in PHILOX_KAT:
        assert tuple(int(x) for x in port.philox(ctr, key)) == want


def _sim_fixture_inputs(g, cfg, d, effects, beh_effects=None):
    """Marshal one sim.json.gz configuration as tests/testthat/test-sim.R:20-36 does."""
    n, M, p = d.n, cfg["M"], cfg["m"] + 1
    beh = d.beh
    z_start = D.beh_values_less_missing_starts(beh, p) if beh is not None else None
    pe = E.prepare_effects_v2(effects, n, p, beh, z_start)
    inp = PeriodInputs(x0=d.imputed[p - 1], type_ids=pe.type_ids, vmat=pe.vmat,
                       wtab=E.effect_wtabs(effects, n), vb=pe.v_dyn, p1=pe.p1, p2=pe.p2,
                       vmiss=pe.vmiss, dyn_flags=pe.dyn_flags, dyc_idx=pe.dyc_idx,
                       symflag=1 if d.symmetric else 0)
    if beh_effects:
        inp.bty = np.array([e.type_id for e in beh_effects])
        inp.z0 = beh.imputed[:, p - 1]
        inp.bkdist = D.beh_kmask_dist(beh, p).astype(np.int32)
        inp.zmin, inp.zmax = beh.zmin, beh.zmax
        inp.zbar, inp.brange, inp.bsimmean = beh.overall_mean, beh.range, beh.sim_mean
    return marshal_period(inp, M, cfg["seed"], cfg["lam"], np.array(cfg["theta"]),
                          lamb=cfg.get("lamb", 0.0), thetab=np.array(cfg.get("thetab", [])))


def sim_fixture_cases(fixtures_dir):
    g = json.load(gzip.open(os.path.join(fixtures_dir, "sim", "sim.json.gz")))
    waves = [np.array(w, dtype=np.float64) for w in g["inputs"]["s50_waves"]]
    alc = np.array(g["inputs"]["alcohol"], dtype=np.float64)
    S = E.make_effect_spec
    base = [S(x) for x in ("density", "recip", "transTrip")]
    d = D.build_saom_data(waves)
    d_beh = D.build_saom_data(waves, behavior=alc)
    cov = base + [S("egoX", alc[:, 0]), S("altX", alc[:, 0]), S("simX", alc[:, 0])]
    dyn = base + [S("egoX", dyn=True), S("altX", dyn=True), S("simX", dyn=True)]
    bef = [E.make_beh_effect_spec(x) for x in ("linear", "quad", "avSim")]
    return [
        ("baseline", g["baseline"], lambda: _sim_fixture_inputs(g, g["baseline"], d, base)),
        ("covariate", g["covariate"], lambda: _sim_fixture_inputs(g, g["covariate"], d, cov)),
        ("coevol", g["coevol"], lambda: _sim_fixture_inputs(g, g["coevol"], d_beh, dyn, bef)),
    ]


def check_sim_fixture(out, gold):
    """tests/testthat/test-sim.R:43-72: integers identical, stats 1e-9, scores 2e-4.
    The oracle meets a stricter bar: every output equal."""
    for key in ("dist", "dist_stat", "steps", "bdist", "z_end"):
        if key in gold and key in out:
            np.testing.assert_array_equal(out[key], np.array(gold[key]))
    np.testing.assert_array_equal(out["stats"], np.array(gold["stats"]))
    np.testing.assert_array_equal(out["scores"], np.array(gold["scores"], dtype=np.float32))
    np.testing.assert_array_equal(out["ntim"], np.array(gold["ntim"]))
    if "bscores" in gold:
        np.testing.assert_array_equal(out["bscores"], np.array(gold["bscores"], dtype=np.float32))


@pytest.mark.parametrize("which", [0, 1, 2])
def test_oracle_reproduces_reference_golden_sim(port, fixtures_dir, which):
    name, gold, make = sim_fixture_cases(fixtures_dir)[which]
    check_sim_fixture(port.simulate(make()), gold)


@pytest.mark.parametrize("kind", WL.PARITY_KINDS)
@pytest.mark.parametrize("seed", SEEDS)
def test_oracle_matches_committed_golden(port, kind, seed):
    c = WL.parity_case(kind, seed=seed)
    gold = np.load(os.path.join(GOLDEN, f"parity_{kind}_{seed}.npz"))
    assert str(gold["digest"]) == case_digest(c), "golden inputs drifted: regenerate"
    out = run_case(port, c)
    for key in out:
        np.testing.assert_array_equal(out[key], gold[key], err_msg=key)


@pytest.mark.parametrize("kind", WL.PARITY_KINDS)
def test_oracle_matches_reference_engine_live(port, ref_engine, kind):
    c = WL.parity_case(kind, seed=7, n=45, M=4)
    a, b = run_case(port, c), run_case(ref_engine, c)
    for key in a:
        np.testing.assert_array_equal(a[key], b[key], err_msg=key)


def test_oracle_network_and_behavior_stats_match_reference(port, ref_engine):
    r = np.random.Generator(np.random.PCG64(3))
    n = 37
    for kind in ("structural", "gw", "covariate_all", "covariate"):
        c = WL.parity_case(kind, seed=3, n=n)
        inp = c["inp"]
        a = (r.random((n, n)) < 0.15).astype(np.uint8)
        np.fill_diagonal(a, 0)
        args = (a, n, inp.k, inp.type_ids, inp.p1, inp.p2, inp.vmat, inp.vmiss, inp.dyn_flags,
                inp.vb, a.sum(1), a.sum(0), inp.wtab, 0)
        np.testing.assert_array_equal(port.network_stats(*args), ref_engine.network_stats(*args))
    z = r.integers(1, 6, size=(5, n))
    xnet = (r.random((n, n)) < 0.1).astype(np.uint8)
    bk = (r.random(n) < 0.9).astype(np.int32)
    for bty in ([0, 1, 2, 3, 4],):
        np.testing.assert_array_equal(port.behavior_stats(z, bty, xnet, bk, 3.1, 4.0, 0.6),
                                      ref_engine.behavior_stats(z, bty, xnet, bk, 3.1, 4.0, 0.6))


def test_oracle_hand_computed_stats(port):
    """tests/testthat/test-stats.R:19-49 known answers."""
    a = np.zeros((3, 3), dtype=np.uint8)
    a[0, 1] = a[1, 0] = a[1, 2] = 1
    out = port.network_stats(a, 3, 3, [0, 1, 2], np.zeros(3), np.zeros(3), np.zeros((3, 3)),
                             np.zeros((3, 3)), np.zeros(3), np.zeros(3), a.sum(1), a.sum(0),
                             np.zeros((3, 4)), 0)
    np.testing.assert_array_equal(out, [3.0, 2.0, 0.0])
    z = np.array([[1, 2, 3, 2]])
    xnet = np.zeros((4, 4), dtype=np.uint8)
    xnet[0, 1:] = 1
    out = port.behavior_stats(z, [0, 1], xnet, np.ones(4), 2.0, 2.0, 0.0)
    u = np.array([1, 2, 3, 2]) - 2.0
    np.testing.assert_array_equal(out[0], [u.sum(), (u ** 2).sum()])


def test_conditional_run_stops_at_target(port):
    """tests/testthat/test-nets.R:42: a conditional run ends exactly at the
    observed distance, and end networks keep a zero diagonal."""
    c = WL.parity_case("conditional", seed=2)
    out = run_case(port, c)
    assert (out["dist"] == c["inp"].target_dist).all()
    assert (out["dist_stat"] == c["inp"].target_dist).all()
    for a in out["a_ends"]:
        assert not np.diag(a).any()
