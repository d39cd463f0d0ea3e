"""The multi-network simulator (cusna_saom_simulate_multi) and the
cross-network statistics (cusna_cross_stats).

CPU: the oracle's multi-network chain and cross statistics against the
reference engine's committed outputs (tests/golden/multi_*.npz,
cross_stats.npz) and against the reference engine live; hand-computed cross
statistics; argument errors of the GPU library that are reported before any
device work.

GPU (`-m gpu`): the library against the same golden vectors and against the
oracle on wider cases (3 and 4 networks, word-edge n, networks too large for
shared memory). Bar, as for the single-network simulator: trajectories, steps,
rate scores and end networks identical; ntim within 1e-13 relative; float32
scores within one float32 ulp.
"""
import ctypes as C
import os

import numpy as np
import pytest

from cusna_gb300 import abi
from cusna_gb300 import workloads as WL
from cusna_gb300.glue import marshal_multi
from tests.conftest import GOLDEN
from tests.test_gpu_parity import assert_within_one_ulp
from tests.golden.make_golden import (CROSS_TYPES, MULTI_M, SEEDS, cross_case, multi_digest,
                                      run_multi)

EXACT = ("steps", "rscores", "a_ends")


def assert_multi_parity(got: dict, ref: dict, tag=""):
    assert set(ref) <= set(got), (tag, set(ref) - set(got))
    for key, b in ref.items():
        a = got[key]
        msg = f"{tag}:{key}"
        if key in EXACT:
            np.testing.assert_array_equal(a, b, err_msg=msg)
        elif key == "ntim":
            np.testing.assert_allclose(a, b, rtol=1e-13, atol=0, err_msg=msg)
        else:  # float32 scores
            assert_within_one_ulp(a, b, msg)


def golden(kind, seed):
    case = WL.multi_case(kind, seed=seed, M=MULTI_M)
    g = np.load(os.path.join(GOLDEN, f"multi_{kind}_{seed}.npz"))
    assert str(g["digest"]) == multi_digest(case), "golden inputs drifted: regenerate"
    return case, {k: g[k] for k in g.files if k != "digest"}


# ---- oracle (CPU) -------------------------------------------------------------

@pytest.mark.parametrize("kind", WL.MULTI_KINDS)
@pytest.mark.parametrize("seed", SEEDS)
def test_oracle_multi_matches_committed_golden(port, kind, seed):
    case, ref = golden(kind, seed)
    out = run_multi(port, case)
    for key in ref:
        np.testing.assert_array_equal(out[key], ref[key], err_msg=key)


@pytest.mark.parametrize("kind", WL.MULTI_KINDS)
@pytest.mark.parametrize("D", [2, 3])
def test_oracle_multi_matches_reference_engine_live(port, ref_engine, kind, D):
    case = WL.multi_case(kind, seed=5 + D, n=37, M=MULTI_M, D=D)
    a, b = run_multi(port, case), run_multi(ref_engine, case)
    for key in a:
        np.testing.assert_array_equal(a[key], b[key], err_msg=key)


def test_oracle_cross_stats_match_committed_golden(port):
    g = np.load(os.path.join(GOLDEN, "cross_stats.npz"))
    for seed in SEEDS:
        a, w = cross_case(seed)
        for t, parm in CROSS_TYPES:
            np.testing.assert_array_equal(port.cross_stats(a, w, t, parm),
                                          g[f"s{seed}_t{t}_p{int(parm)}"], err_msg=f"{seed}/{t}")


def hand_cross(a, w, t, parm):
    """The cross statistics written out from their definitions."""
    n = a.shape[0]
    tot = 0.0
    for i in range(n):
        for j in range(n):
            if not a[i, j]:
                continue
            if t == 33:
                tot += w[i, j]
            elif t == 34:
                tot += w[j, i]
            elif t == 35:
                tot += w[i, j] * w[j, i]
            elif t == 36:
                s = int(np.sum(w[i] & w[j]))
                tot += np.sqrt(s) if parm >= 2 else s
            else:
                tot += int(np.sum(w[i] & a[:, j]))
    return tot


def test_oracle_cross_stats_hand_computed(port):
    a, w = cross_case(9, n=11, M=2)
    for t, parm in CROSS_TYPES:
        got = port.cross_stats(a, w, t, parm)
        want = [hand_cross(x, w, t, parm) for x in a]
        np.testing.assert_allclose(got, want, rtol=1e-14, err_msg=str(t))


def test_multi_status_codes_before_device_work(built_lib):
    lib = built_lib
    assert lib.cusna_saom_simulate_multi(None, None) == abi.ERR_NULL_ARG
    inp, seed, lam, th = WL.multi_case("cross", seed=0)
    m = marshal_multi(inp, 3, seed, lam, th)
    P, R = C.byref(m.problem), C.byref(m.result)
    for field, bad in (("D", 1), ("D", 5), ("n", 0), ("W", 7), ("k", 0), ("k", 25), ("M", 0)):
        old = getattr(m.problem, field)
        setattr(m.problem, field, bad)
        assert lib.cusna_saom_simulate_multi(P, R) == abi.ERR_SHAPE, (field, bad)
        setattr(m.problem, field, old)
    for name, bad_val, want in (("netof", 2, abi.ERR_SHAPE), ("netref", 7, abi.ERR_SHAPE),
                                ("dyc_idx", 1, abi.ERR_SHAPE), ("dyc_idx", 0, abi.ERR_NULL_ARG)):
        arr = np.array(m.keep[name])
        e = 3   # a cross effect of network 0
        arr[e] = bad_val
        m.keep[name + "_bad"] = arr
        setattr(m.problem, name, arr.ctypes.data)
        assert lib.cusna_saom_simulate_multi(P, R) == want, name
        setattr(m.problem, name, m.keep[name].ctypes.data)
    old = m.problem.netof
    m.problem.netof = None
    assert lib.cusna_saom_simulate_multi(P, R) == abi.ERR_NULL_ARG
    m.problem.netof = old
    a, w = cross_case(0, n=8, M=1)
    out = np.zeros(1)
    assert lib.cusna_cross_stats(None, w.ctypes.data, 8, 1, 33, 0.0, out.ctypes.data) == abi.ERR_NULL_ARG
    assert lib.cusna_cross_stats(a.ctypes.data, w.ctypes.data, 8, 1, 32, 0.0,
                                 out.ctypes.data) == abi.ERR_UNSUPPORTED
    if lib.cusna_has_cuda() == 0:
        assert lib.cusna_saom_simulate_multi(P, R) == abi.ERR_NO_CUDA


# ---- GPU --------------------------------------------------------------------------

class GpuMulti:
    def simulate_multi(self, m):
        from cusna_gb300 import sim
        return sim.simulate_multi(m)


@pytest.mark.gpu
@pytest.mark.parametrize("kind", WL.MULTI_KINDS)
@pytest.mark.parametrize("seed", SEEDS)
def test_gpu_multi_matches_reference_golden(gpu_lib, kind, seed):
    case, ref = golden(kind, seed)
    assert_multi_parity(run_multi(GpuMulti(), case), ref, f"{kind}/{seed}")


@pytest.mark.gpu
@pytest.mark.parametrize("D", [2, 3, 4])
@pytest.mark.parametrize("n", [5, 31, 32, 33, 65])
def test_gpu_multi_matches_oracle(gpu_lib, port, D, n):
    # "cross" has 8 effects per network: 4 networks would exceed CUSNA_MAXEFF
    kinds = ("cross", "dyadic", "symmetric") if D <= 3 else ("dyadic", "symmetric", "empty_net")
    for kind in kinds:
        case = WL.multi_case(kind, seed=10 * D + n, n=n, M=MULTI_M, D=D)
        assert_multi_parity(run_multi(GpuMulti(), case), run_multi(port, case),
                            f"{kind}/D={D}/n={n}")


@pytest.mark.gpu
def test_gpu_multi_networks_in_global_scratch(gpu_lib, port):
    """Three networks of 800 actors do not fit one team's shared memory: rows and
    columns live in global scratch, with the same results."""
    case = WL.multi_case("cross", seed=3, n=800, M=2, D=3)
    from cusna_gb300.glue import marshal_multi as mm
    inp, seed, lam, th = case
    lam = np.asarray(lam) * 0.25     # a short period keeps the oracle quick
    a = GpuMulti().simulate_multi(mm(inp, 2, seed, lam, th))
    b = port.simulate_multi(mm(inp, 2, seed, lam, th))
    assert_multi_parity(a, b, "n=800/D=3")


@pytest.mark.gpu
def test_gpu_cross_stats(gpu_lib, port):
    from cusna_gb300 import sim
    g = np.load(os.path.join(GOLDEN, "cross_stats.npz"))
    for seed in SEEDS:
        a, w = cross_case(seed)
        for t, parm in CROSS_TYPES:
            got = sim.cross_stats(a, w, t, parm)
            want = g[f"s{seed}_t{t}_p{int(parm)}"]
            if t == 36 and parm >= 2:   # a sum of square roots, added in another order
                np.testing.assert_allclose(got, want, rtol=1e-13)
            else:
                np.testing.assert_array_equal(got, want)
    a, w = cross_case(4, n=97, M=5)
    for t, parm in CROSS_TYPES:
        np.testing.assert_allclose(sim.cross_stats(a, w, t, parm), port.cross_stats(a, w, t, parm),
                                   rtol=1e-13, err_msg=str(t))
