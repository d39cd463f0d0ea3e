"""GPU parity: libcusna_gb300 through its C ABI against the reference engine's
committed outputs and the CPU oracle on the same seeded inputs.

Bar (the reference's own test-sim.R bar is integers identical, stats 1e-9,
scores 2e-4; this one is stricter):
  * trajectories and every integer output identical: dist, dist_stat, steps,
    bdist, z_end, actor_dist, the dense end networks;
  * stats within 1e-12 relative (identical bits except where CUDA's pow/sqrt
    differ from the C library's by an ulp);
  * ntim within 1e-13 relative (CUDA's log may differ from glibc's by an ulp);
  * float32 scores within one float32 ulp: each ministep's score sums are
    double-float (48-bit significands) or float64 on the GPU and float64 on
    the CPU, added in another order, so the float64 scores differ by far less
    than a float32 ulp and their float32 roundings by at most one ulp.
"""
import ctypes as C
import os

import numpy as np
import pytest

from cusna_gb300 import sim as G
from cusna_gb300 import workloads as WL
from cusna_gb300.abi import ERR_NULL_ARG, ERR_SHAPE, CudaError
from cusna_gb300.glue import marshal_period
from tests.conftest import GOLDEN
from tests.golden.make_golden import SEEDS, case_digest, run_case

pytestmark = pytest.mark.gpu

EXACT = ("dist", "dist_stat", "steps", "bdist", "z_end", "actor_dist", "a_ends")


def assert_parity(gpu: dict, ref: dict, tag=""):
    assert set(ref) <= set(gpu), (tag, set(ref) - set(gpu))
    for key, b in ref.items():
        a = gpu[key]
        msg = f"{tag}:{key}"
        if key in EXACT:
            np.testing.assert_array_equal(a, b, err_msg=msg)
        elif key == "ntim":
            np.testing.assert_allclose(a, b, rtol=1e-13, atol=0, err_msg=msg)
        elif key == "stats":
            np.testing.assert_allclose(a, b, rtol=1e-12, atol=1e-12, err_msg=msg)
        else:  # float32 scores
            assert_within_one_ulp(a, b, msg)


def assert_within_one_ulp(a, b, msg=""):
    """float32 arrays equal to within one ulp of the larger magnitude (NaN
    where the other is NaN)."""
    a = np.asarray(a, dtype=np.float32)
    b = np.asarray(b, dtype=np.float32)
    assert a.shape == b.shape, msg
    nan = np.isnan(a) | np.isnan(b)
    np.testing.assert_array_equal(np.isnan(a), np.isnan(b), err_msg=msg + " (NaN)")
    ulp = np.spacing(np.maximum(np.abs(a), np.abs(b)))
    diff = np.abs(a.astype(np.float64) - b.astype(np.float64))
    bad = ~nan & (diff > ulp)
    if bad.any():
        idx = np.argwhere(bad)[0]
        raise AssertionError(f"{msg}: {int(bad.sum())} values more than one float32 ulp apart, "
                             f"first at {tuple(idx)}: {a[tuple(idx)]!r} vs {b[tuple(idx)]!r}")


class GpuEngine:
    """Adapter so tests can call run_case() on the GPU like on the oracle."""

    def __init__(self, **opts):
        self.opts = opts

    def simulate(self, m):
        if self.opts:
            return G.simulate_ex(m, G.options(**self.opts))
        return G.simulate(m)


@pytest.mark.parametrize("kind", WL.PARITY_KINDS)
@pytest.mark.parametrize("seed", SEEDS)
def test_gpu_matches_reference_golden(gpu_lib, kind, seed):
    c = WL.parity_case(kind, seed=seed)
    gold = np.load(os.path.join(GOLDEN, f"parity_{kind}_{seed}.npz"))
    assert str(gold["digest"]) == case_digest(c)
    out = run_case(GpuEngine(), c)
    assert_parity(out, {k: gold[k] for k in gold.files if k != "digest"}, f"{kind}/{seed}")


@pytest.mark.parametrize("n", [1, 2, 5, 31, 32, 33, 63, 64, 65, 97])
def test_gpu_matches_oracle_at_word_edges(gpu_lib, port, n):
    kinds = ("covariate", "structural", "coevol") if n >= 5 else ("baseline", "structural")
    for kind in kinds:
        c = WL.parity_case(kind, seed=n, n=n, M=5)
        assert_parity(run_case(GpuEngine(), c), run_case(port, c), f"{kind}/n={n}")


@pytest.mark.parametrize("G_", [1, 2, 4, 8])
def test_gpu_launch_shape_does_not_change_results(gpu_lib, port, G_):
    """Every output, the float32 scores included, is bit-identical for every
    team size and chains-per-CTA (the autotuner may pick any of them)."""
    for kind in ("covariate", "gw", "coevol", "rates", "masks"):
        c = WL.parity_case(kind, seed=11, n=70, M=6)
        ref = run_case(GpuEngine(warps_per_chain=1, chains_per_cta=1), c)
        assert_parity(ref, run_case(port, c), f"{kind}/oracle")
        for tpc in (1, 2, 4):
            if 32 * G_ * tpc > 512:
                continue
            got = run_case(GpuEngine(warps_per_chain=G_, chains_per_cta=tpc), c)
            for key in ref:
                np.testing.assert_array_equal(got[key], ref[key], err_msg=f"{kind}/G={G_}x{tpc}:{key}")


def test_gpu_n200_covariate_workload_vs_oracle(gpu_lib, port):
    inp, M, seed, lam, theta = WL.c2_period(M=24)
    m1 = marshal_period(inp, M, seed, lam, theta, want_ends=True)
    m2 = marshal_period(inp, M, seed, lam, theta, want_ends=True)
    assert_parity(G.simulate(m1), port.simulate(m2), "c2")


def test_gpu_n1000_coevolution_vs_oracle(gpu_lib, port):
    inp, M, seed, lam, theta, lamb, thetab = WL.c4_period(M=2)
    args = dict(lamb=lamb, thetab=thetab)
    out = G.simulate(marshal_period(inp, M, seed, lam, theta, **args))
    ref = port.simulate(marshal_period(inp, M, seed, lam, theta, **args))
    assert_parity(out, ref, "c4")


def test_gpu_chain_offset_splits_chains(gpu_lib):
    c = WL.parity_case("coevol", seed=5, M=8)
    whole = run_case(GpuEngine(), c)
    c4 = dict(c, M=4)
    first = run_case(GpuEngine(chain_offset=0), c4)
    second = run_case(GpuEngine(chain_offset=4), c4)
    for key in whole:
        np.testing.assert_array_equal(np.concatenate([first[key], second[key]]), whole[key], key)


def test_gpu_batch_equals_separate_calls(gpu_lib):
    cases = [WL.parity_case(k, seed=3, n=n, M=m)
             for k, n, m in (("baseline", 30, 5), ("coevol", 77, 3), ("gw", 50, 4), ("masks", 41, 6))]
    ms = [marshal_period(c["inp"], c["M"], c["seed"], c["lam"], c["theta"], lamb=c["lamb"],
                         thetab=c["thetab"], want_ends=True) for c in cases]
    batch = G.simulate_batch(ms)
    for c, b in zip(cases, batch):
        single = run_case(GpuEngine(), c)
        for key in single:
            np.testing.assert_array_equal(b[key], single[key], key)


def test_gpu_device_pointer_mode(gpu_lib):
    torch = pytest.importorskip("torch")
    c = WL.parity_case("covariate", seed=9, M=7)
    host = run_case(GpuEngine(), c)
    m = marshal_period(c["inp"], c["M"], c["seed"], c["lam"], c["theta"], want_ends=True)
    dev = {}
    for name, arr in m.keep.items():
        t = torch.from_numpy(np.ascontiguousarray(arr).view(np.uint8).reshape(-1)).cuda()
        dev[name] = t
        field = name[4:] if name.startswith("out_") else name
        target = m.result if name.startswith("out_") else m.problem
        setattr(target, field, t.data_ptr())
    G.simulate_ex(m, G.options(device_ptrs=True))
    torch.cuda.synchronize()
    for name, arr in m.keep.items():
        if name.startswith("out_"):
            got = dev[name].cpu().numpy().view(arr.dtype).reshape(arr.shape)
            np.testing.assert_array_equal(got, host[name[4:]], name)


def test_gpu_network_and_behavior_stats(gpu_lib, port):
    r = np.random.Generator(np.random.PCG64(4))
    n = 45
    for kind in ("structural", "gw", "covariate_all", "covariate", "coevol"):
        c = WL.parity_case(kind, seed=4, n=n)
        inp = c["inp"]
        A = (r.random((6, n, n)) < 0.12).astype(np.uint8)
        for a in A:
            np.fill_diagonal(a, 0)
        out = G.network_stats(A, n, inp.k, inp.type_ids, inp.p1, inp.p2, inp.vmat, inp.vmiss,
                              inp.dyn_flags, inp.vb, A[0].sum(1), A[0].sum(0), inp.wtab, 0)
        for m_ in range(len(A)):
            ref = port.network_stats(A[m_], n, inp.k, inp.type_ids, inp.p1, inp.p2, inp.vmat,
                                     inp.vmiss, inp.dyn_flags, inp.vb, A[0].sum(1), A[0].sum(0),
                                     inp.wtab, 0)
            np.testing.assert_allclose(out[m_], ref, rtol=1e-12, atol=1e-12)
    z = r.integers(1, 6, size=(9, n))
    xnet = (r.random((n, n)) < 0.1).astype(np.uint8)
    bk = (r.random(n) < 0.9).astype(np.int32)
    bty = [0, 1, 2, 3, 4]
    np.testing.assert_allclose(G.behavior_stats(z, bty, xnet, bk, 3.1, 4.0, 0.6),
                               port.behavior_stats(z, bty, xnet, bk, 3.1, 4.0, 0.6),
                               rtol=1e-13, atol=1e-13)


def test_gpu_error_statuses(gpu_lib):
    lib = gpu_lib
    assert lib.cusna_saom_simulate_period(None, None) == ERR_NULL_ARG
    c = WL.parity_case("baseline", seed=1)
    m = marshal_period(c["inp"], c["M"], c["seed"], c["lam"], c["theta"])
    m.problem.struct_version = 2
    assert lib.cusna_saom_simulate_period(C.byref(m.problem), C.byref(m.result)) == ERR_SHAPE
    m.problem.struct_version = 1
    m.problem.W = m.problem.W + 1
    assert lib.cusna_saom_simulate_period(C.byref(m.problem), C.byref(m.result)) == ERR_SHAPE
    assert b"bad shape" in lib.cusna_last_error()
    m.problem.W = m.problem.W - 1
    m.problem.k = 25
    assert lib.cusna_saom_simulate_period(C.byref(m.problem), C.byref(m.result)) == ERR_SHAPE
    m.problem.k = c["inp"].k
    m.problem.theta = None
    assert lib.cusna_saom_simulate_period(C.byref(m.problem), C.byref(m.result)) == ERR_NULL_ARG
    with pytest.raises(CudaError):
        G.simulate(m)


def test_gpu_large_n_rows_in_global_scratch(gpu_lib, port):
    """n = 1500 (out-rows and in-rows 282 KB each, beyond shared memory): the
    chain state moves to global scratch and the trajectory is unchanged."""
    c = WL.parity_case("conditional", seed=3, n=1500, M=2)
    c["inp"].target_dist = 400
    assert_parity(run_case(GpuEngine(), c), run_case(port, c), "n1500")


def test_gpu_predictors_beyond_float32_range_choose_as_the_reference(gpu_lib, port):
    """A parameter near the float32 maximum makes float32 predictors infinite
    or NaN: those keys certify nothing, the exact float64 keys decide, the
    score sums of those ministeps run in float64, and the trajectories and
    scores still equal the CPU engine's."""
    c = WL.parity_case("structural", seed=8, n=40, M=4)
    th = np.asarray(c["theta"], dtype=np.float64).copy()
    th[1] = 3.0e38
    c = dict(c, theta=th)
    for spec in (-1, 1):
        got = run_case(GpuEngine(specialise=spec), c)
        ref = run_case(port, c)
        for key in ("steps", "dist", "dist_stat", "a_ends"):
            if key in ref:
                np.testing.assert_array_equal(got[key], ref[key], err_msg=f"{spec}:{key}")
        np.testing.assert_allclose(got["ntim"], ref["ntim"], rtol=1e-13, atol=0)
        assert_within_one_ulp(got["scores"], ref["scores"], f"{spec}:scores")
