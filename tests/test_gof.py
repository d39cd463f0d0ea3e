"""Statistics of end-network batches: the sienaGOF auxiliary distributions
(cusna_gof_distribution) and the typed creation / endowment statistic
(cusna_typed_stats).

CPU: the oracle against the reference's committed outputs
(tests/golden/gof_typed.npz) and the reference engine live; hand-computed
distributions; argument errors of the GPU library before any device work.
GPU (`-m gpu`): the library against the same golden vectors and the oracle;
at sizes the oracle's O(n^3) geodesic loop cannot reach, against breadth-first
distances from scipy. Bar: the distributions (integer counts) identical; the
typed statistic (a float64 sum added in another order) within 1e-12 of the
sum of |F| over the pairs.
"""
import ctypes as C
import os

import numpy as np
import pytest

from cusna_gb300 import abi
from tests.conftest import GOLDEN
from tests.golden.make_golden import GOF_LEVELS, GOF_SIZES, gof_case

MASKS = ("keep", "force", "keepS", "forceS", "miss_m", "miss_m1")


def gold():
    return np.load(os.path.join(GOLDEN, "gof_typed.npz"))


def check_typed(got, want, F):
    tol = 1e-12 * max(1.0, float(np.abs(F).sum()))
    np.testing.assert_allclose(got, want, rtol=0, atol=tol)


# ---- oracle (CPU) -------------------------------------------------------------

def test_oracle_gof_and_typed_match_committed_golden(port):
    g = gold()
    for seed, n in enumerate(GOF_SIZES):
        a, x0, F, masks = gof_case(seed, n)
        for kind, lv in GOF_LEVELS.items():
            np.testing.assert_array_equal(port.gof_distribution(a, kind, lv), g[f"n{n}_gof{kind}"])
        for et in (1, 2):
            np.testing.assert_array_equal(port.typed_stats(a, et, F, x0, **masks),
                                          g[f"n{n}_typed{et}"])
            np.testing.assert_array_equal(port.typed_stats(a, et, F, x0), g[f"n{n}_typed{et}_nomask"])


@pytest.mark.parametrize("n", [3, 17, 40])
def test_oracle_gof_and_typed_match_reference_live(port, ref_engine, n):
    a, x0, F, masks = gof_case(50 + n, n, M=4, p=0.12)
    for kind, lv in ((0, [0, 1, 3, 7]), (1, [2, 5]), (2, [0, 1, 2, 5, 50]), (2, [3])):
        np.testing.assert_array_equal(port.gof_distribution(a, kind, lv),
                                      ref_engine.gof_distribution(a, kind, lv))
    for et in (1, 2):
        np.testing.assert_array_equal(port.typed_stats(a, et, F, x0, **masks),
                                      ref_engine.typed_stats(a, et, F, x0, **masks))


def test_oracle_gof_hand_computed(port):
    """A directed path 0 -> 1 -> 2 -> 3 and an isolated actor 4."""
    a = np.zeros((5, 5), np.uint8)
    a[0, 1] = a[1, 2] = a[2, 3] = 1
    # in-degrees 0,1,1,1,0; out-degrees 1,1,1,0,0
    np.testing.assert_array_equal(port.gof_distribution(a, 0, [0, 1]), [[2, 5]])
    np.testing.assert_array_equal(port.gof_distribution(a, 1, [0, 1]), [[2, 5]])
    # pairs within 1: 3; within 2: 5; within 3: 6; unreachable 20 - 6
    np.testing.assert_array_equal(port.gof_distribution(a, 2, [1, 2, 3]), [[3, 5, 6, 14]])
    F = np.arange(25, dtype=float).reshape(5, 5)
    x0 = np.zeros((5, 5), np.uint8)
    x0[0, 1] = x0[4, 0] = 1
    # created: (1,2), (2,3); lost: (4,0), reported negated
    np.testing.assert_array_equal(port.typed_stats(a, 1, F, x0), [F[1, 2] + F[2, 3]])
    np.testing.assert_array_equal(port.typed_stats(a, 2, F, x0), [-F[4, 0]])


def test_gof_status_codes_before_device_work(built_lib):
    lib = built_lib
    a = np.zeros((1, 4, 4), np.uint8)
    lv = np.array([1, 2], np.int32)
    out = np.zeros(8)
    assert lib.cusna_gof_distribution(None, 4, 1, 0, lv.ctypes.data, 2, out.ctypes.data) == abi.ERR_NULL_ARG
    assert lib.cusna_gof_distribution(a.ctypes.data, 4, 1, 0, lv.ctypes.data, 0, out.ctypes.data) == abi.ERR_NULL_ARG
    assert lib.cusna_gof_distribution(a.ctypes.data, 4, 1, 3, lv.ctypes.data, 2, out.ctypes.data) == abi.ERR_UNSUPPORTED
    neg = np.array([-1, 2], np.int32)
    assert lib.cusna_gof_distribution(a.ctypes.data, 4, 1, 2, neg.ctypes.data, 2, out.ctypes.data) == abi.ERR_SHAPE
    F = np.zeros((4, 4))
    assert lib.cusna_typed_stats(a.ctypes.data, 4, 1, 1, None, a.ctypes.data, None, None, None,
                                 None, None, None, out.ctypes.data) == abi.ERR_NULL_ARG
    assert lib.cusna_typed_stats(a.ctypes.data, 0, 1, 1, F.ctypes.data, a.ctypes.data, None, None,
                                 None, None, None, None, out.ctypes.data) == abi.ERR_NULL_ARG


# ---- GPU --------------------------------------------------------------------------

@pytest.mark.gpu
def test_gpu_gof_and_typed_match_reference_golden(gpu_lib):
    from cusna_gb300 import sim
    g = gold()
    for seed, n in enumerate(GOF_SIZES):
        a, x0, F, masks = gof_case(seed, n)
        for kind, lv in GOF_LEVELS.items():
            np.testing.assert_array_equal(sim.gof_distribution(a, kind, lv), g[f"n{n}_gof{kind}"],
                                          err_msg=f"n={n} kind={kind}")
        for et in (1, 2):
            check_typed(sim.typed_stats(a, et, F, x0, **masks), g[f"n{n}_typed{et}"], F)
            check_typed(sim.typed_stats(a, et, F, x0), g[f"n{n}_typed{et}_nomask"], F)


@pytest.mark.gpu
@pytest.mark.parametrize("n", [32, 64, 97, 130])
def test_gpu_gof_and_typed_match_oracle(gpu_lib, port, n):
    from cusna_gb300 import sim
    a, x0, F, masks = gof_case(70 + n, n, M=5, p=0.04)
    for kind, lv in ((0, list(range(0, 12))), (1, [0, 2, 4, 200]), (2, [0, 1, 2, 3, 4, 6, 9, 1000])):
        np.testing.assert_array_equal(sim.gof_distribution(a, kind, lv),
                                      port.gof_distribution(a, kind, lv), err_msg=f"kind={kind}")
    for et in (1, 2):
        check_typed(sim.typed_stats(a, et, F, x0, **masks), port.typed_stats(a, et, F, x0, **masks), F)


def bfs_within(a, levels):
    """Ordered pairs within each geodesic level and the unreachable pairs, from
    scipy's unweighted shortest paths."""
    from scipy.sparse import csr_matrix
    from scipy.sparse.csgraph import shortest_path
    n = a.shape[0]
    A = a.copy()
    np.fill_diagonal(A, 0)
    d = shortest_path(csr_matrix(A), unweighted=True, directed=True)
    off = ~np.eye(n, dtype=bool)
    row = [int(((d <= k) & off).sum()) if k > 0 else 0 for k in levels]
    row.append(int(n * (n - 1) - ((d <= max(levels)) & off).sum()) if max(levels) > 0
               else n * (n - 1))
    return row


@pytest.mark.gpu
@pytest.mark.parametrize("n,p", [(600, 0.004), (1500, 0.0015)])
def test_gpu_geodesic_large_networks(gpu_lib, n, p):
    """n=600: the rows fit the CTA's shared memory; n=1500: they are read from
    global memory."""
    pytest.importorskip("scipy")
    from cusna_gb300 import sim
    r = np.random.default_rng(n)
    a = (r.random((3, n, n)) < p).astype(np.uint8)
    lv = [1, 2, 3, 5, 8, 13, 40, 5000]
    got = sim.gof_distribution(a, 2, lv)
    for c in range(3):
        np.testing.assert_array_equal(got[c], bfs_within(a[c], lv), err_msg=f"chain {c}")
    deg = sim.gof_distribution(a, 0, [0, 1, 2, 3, 10])
    ind = a.sum(axis=1)
    np.testing.assert_array_equal(deg, [[(ind[c] <= k).sum() for k in [0, 1, 2, 3, 10]]
                                        for c in range(3)])
