"""Validation mode: a per-ministep trace checked step by step against the
reference chooser, and caller-supplied random words in place of Philox.

The reference chooser is src/libcusna_saom_cpu.cpp:166-287 (the draws at :167,
the Gumbel argmax with ties to the lowest alter at :235-269, the distance
update at :277-282). The oracle restates it and writes the same trace
(oracle_simulate_period_validate), so a divergence shows the first ministep
where the GPU and the reference differ, instead of only a different end state.

CPU tests pin the oracle's validation mode itself: its outputs equal the plain
call's; its trace replays to the returned end network and distance; words
equal to the Philox outputs reproduce the Philox run. GPU tests compare the
GPU's traces with the oracle's, record for record, on every parity kind, at
the word edges of the bit rows, on the n=200 covariate workload, across launch
shapes, with the float64 score sums, and on supplied words that force near
ties and exact ties of the Gumbel keys.
"""
import numpy as np
import pytest

from cusna_gb300 import sim as G
from cusna_gb300 import workloads as WL
from cusna_gb300.glue import marshal_period
from tests.test_gpu_parity import assert_parity

TRACE_CAP = 4096


def _marshal(c):
    return marshal_period(c["inp"], c["M"], c["seed"], c["lam"], c["theta"], lamb=c["lamb"],
                          thetab=c["thetab"], want_ends=True)


def _philox_words(port, c, steps):
    """The Philox outputs the engine draws in ministeps 0..steps-1 of each
    chain, laid out as the validation mode's supplied words."""
    n, M, seed = c["inp"].x0.shape[0], c["M"], c["seed"]
    key = [seed & 0xFFFFFFFF, seed >> 32]
    us = np.zeros((M, steps, 4 + n), dtype=np.uint32)
    for ch in range(M):
        for s in range(steps):
            us[ch, s, :4] = port.philox([s, ch, 0, 0], key)
            for j in range(n):
                us[ch, s, 4 + j] = port.philox([s, ch, 1, j], key)[0]
    return us


def _check_trace(tr, out, c):
    """Records 0..steps-1 are the chain's ministeps in order, the rest -1; the
    network steps' distance changes add up to dist; toggling the recorded
    choices on the simulation's start network gives the end network."""
    inp = c["inp"]
    n = inp.x0.shape[0]
    start = inp.sim_start if getattr(inp, "sim_start", None) is not None else inp.x0
    for ch in range(c["M"]):
        st = int(out["steps"][ch])
        assert st <= TRACE_CAP
        rec = tr[ch, :st]
        np.testing.assert_array_equal(rec[:, 0], np.arange(st))
        assert (tr[ch, st:] == -1).all()
        net = rec[rec[:, 2] >= 0]
        assert int(net[:, 3].sum()) == int(out["dist"][ch])
        if inp.symflag or getattr(inp, "inactive", None) is not None:
            continue
        a = np.asarray(start, dtype=np.uint8).copy()
        for _, i, j, _ in net:
            if j != i:
                a[i, j] ^= 1
        np.testing.assert_array_equal(a, out["a_ends"][ch].reshape(n, n))


# ---- the oracle's validation mode (CPU) -------------------------------------

@pytest.mark.parametrize("kind", WL.PARITY_KINDS)
def test_oracle_trace_is_consistent_with_its_outputs(port, kind):
    c = WL.parity_case(kind, seed=0)
    plain = port.simulate(_marshal(c))
    out, tr = port.simulate_validate(_marshal(c), TRACE_CAP)
    for key in plain:
        np.testing.assert_array_equal(out[key], plain[key], err_msg=key)
    _check_trace(tr, out, c)


@pytest.mark.parametrize("kind", ["covariate", "coevol", "rates"])
def test_oracle_supplied_philox_words_reproduce_the_philox_run(port, kind):
    c = WL.parity_case(kind, seed=1, n=24, M=3)
    plain, tr0 = port.simulate_validate(_marshal(c), TRACE_CAP)
    us = _philox_words(port, c, 40)
    out, tr = port.simulate_validate(_marshal(c), TRACE_CAP, ustream=us)
    for key in plain:
        np.testing.assert_array_equal(out[key], plain[key], err_msg=key)
    np.testing.assert_array_equal(tr, tr0)


def test_oracle_supplied_words_drive_the_chooser(port):
    """Different words give a different trajectory; the chooser takes the
    alter the words make best."""
    c = WL.parity_case("baseline", seed=2, n=30, M=2)
    us, expect = _near_tie_words(c)
    out, tr = port.simulate_validate(_marshal(c), TRACE_CAP, ustream=us)
    for ch in range(c["M"]):
        assert tr[ch, 0, 1] == expect[ch][0] and tr[ch, 0, 2] == expect[ch][1]


def _near_tie_words(c):
    """Supplied words for ministep 0 of each chain (then Philox): a focal actor
    i and two alters j1 < j2 with identical change statistics (so identical
    predictors) whose Gumbel keys are a near tie (words w and w + 1 with
    u = 0.99: keys f + 4.6, 2.3e-8 apart, far inside the float32 keys' error
    bound of ~6e-6, so only the exact float64 keys can decide; the larger word
    wins) on even chains, and an exact tie (equal words: the lower alter wins,
    as the reference's strict > keeps it) on odd chains. Every other alter,
    and the "no change" option, get word 0 (key f - 3.13); the predictors of
    this model span less than the 7.7 between the two. Returns the words and,
    per chain, the expected (focal actor, choice)."""
    inp = c["inp"]
    a = np.asarray(inp.x0, dtype=np.int64)
    n = a.shape[0]
    M = c["M"]
    us = np.zeros((M, 1, 4 + n), dtype=np.uint32)
    expect = []
    rng = np.random.Generator(np.random.PCG64(5))
    for ch in range(M):
        for _ in range(1000):
            i = int(rng.integers(n))
            # baseline statistics of toggling i -> j: a_ij, a_ji and the two-path count
            tp = a[i] @ a.T + a[i] @ a  # |out_i & out_j| + |out_i & in_j| over j
            groups = {}
            for j in range(n):
                if j != i:
                    groups.setdefault((a[i, j], a[j, i], tp[j]), []).append(j)
            pairs = [g for g in groups.values() if len(g) >= 2]
            if pairs:
                j1, j2 = pairs[int(rng.integers(len(pairs)))][:2]
                break
        us[ch, 0, 0] = 1 << 31                       # waiting time
        us[ch, 0, 1] = 0                             # network ministep
        us[ch, 0, 2] = int((i + 0.5) / n * 2**32)    # focal actor i
        w = int(0.99 * 2**32)
        us[ch, 0, 4 + j1] = w
        us[ch, 0, 4 + j2] = w + (1 if ch % 2 == 0 else 0)
        expect.append((i, j2 if ch % 2 == 0 else j1))
    return us, expect


# ---- the GPU against the oracle ---------------------------------------------

def _gpu_vs_oracle(port, c, tag, **kw):
    us = kw.pop("ustream", None)
    got, tr = G.simulate_validate(_marshal(c), TRACE_CAP, ustream=us, **kw)
    ref, rtr = port.simulate_validate(_marshal(c), TRACE_CAP, ustream=us)
    first = np.argwhere((tr != rtr).any(axis=2))
    assert first.size == 0, f"{tag}: traces differ first at (chain, ministep) {first[0]}: " \
                            f"gpu {tr[tuple(first[0])]} oracle {rtr[tuple(first[0])]}"
    assert_parity(got, ref, tag)
    return got, tr


@pytest.mark.gpu
@pytest.mark.parametrize("kind", WL.PARITY_KINDS)
def test_gpu_trace_equals_oracle_trace(gpu_lib, port, kind):
    c = WL.parity_case(kind, seed=0)
    out, tr = _gpu_vs_oracle(port, c, kind)
    _check_trace(tr, out, c)


@pytest.mark.gpu
@pytest.mark.parametrize("n", [31, 32, 33, 63, 64, 65])
def test_gpu_trace_at_word_edges(gpu_lib, port, n):
    for kind in ("covariate", "structural", "coevol"):
        _gpu_vs_oracle(port, WL.parity_case(kind, seed=n, n=n, M=4), f"{kind}/n={n}")


@pytest.mark.gpu
def test_gpu_trace_on_the_n200_covariate_workload(gpu_lib, port):
    inp, M, seed, lam, theta = WL.c2_period(M=8)
    c = dict(inp=inp, M=M, seed=seed, lam=lam, theta=theta, lamb=0.0, thetab=None)
    out, _ = _gpu_vs_oracle(port, c, "c2")
    assert int(out["steps"].max()) <= TRACE_CAP


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(1, 1), (2, 2), (4, 1), (8, 1)])
def test_gpu_trace_does_not_depend_on_the_launch_shape(gpu_lib, port, shape):
    for kind in ("covariate", "gw", "coevol", "rates"):
        c = WL.parity_case(kind, seed=7, n=70, M=4)
        _gpu_vs_oracle(port, c, f"{kind}/{shape}", warps_per_chain=shape[0],
                       chains_per_cta=shape[1])


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["covariate", "coevol", "interaction", "gw", "rates"])
def test_gpu_float64_score_sums_match_the_double_float_ones(gpu_lib, port, kind):
    """lse64 forms every ministep's score sums in float64 (the reference's
    arithmetic per alter); the default double-float sums give the same
    trajectory and scores within one float32 ulp of them."""
    c = WL.parity_case(kind, seed=3, n=50, M=5)
    a, ta = _gpu_vs_oracle(port, c, f"{kind}/lse64", lse64=True)
    b, tb = _gpu_vs_oracle(port, c, f"{kind}/double-float")
    np.testing.assert_array_equal(ta, tb)


@pytest.mark.gpu
def test_gpu_supplied_philox_words_reproduce_the_philox_run(gpu_lib, port):
    c = WL.parity_case("coevol", seed=1, n=24, M=3)
    plain, tr0 = G.simulate_validate(_marshal(c), TRACE_CAP)
    out, tr = G.simulate_validate(_marshal(c), TRACE_CAP, ustream=_philox_words(port, c, 40))
    for key in plain:
        np.testing.assert_array_equal(out[key], plain[key], err_msg=key)
    np.testing.assert_array_equal(tr, tr0)
    ref = G.simulate(_marshal(c))
    for key in ref:
        np.testing.assert_array_equal(plain[key], ref[key], err_msg=key)


@pytest.mark.gpu
def test_gpu_near_ties_of_the_gumbel_keys(gpu_lib, port):
    """Supplied words make the first ministep of each chain a near tie (keys
    7e-10 apart) or an exact tie between two alters with equal predictors: the
    float32 keys cannot certify either, so the exact float64 keys decide, and
    the choice equals the reference chooser's (the larger word; the lower
    alter on an exact tie)."""
    c = WL.parity_case("baseline", seed=2, n=40, M=8)
    us, expect = _near_tie_words(c)
    _, tr = _gpu_vs_oracle(port, c, "near-tie", ustream=us)
    for ch in range(c["M"]):
        assert (tr[ch, 0, 1], tr[ch, 0, 2]) == expect[ch], ch
