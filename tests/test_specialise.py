"""The period kernel specialised to an effect plan (compiled at run time with
NVRTC; csrc/saom_jit.cu).

CPU: the generated source of every parity case's effect plan compiles (no
device needed), and a compiled plan is written to the on-disk cache and read
back by a fresh process. GPU (`-m gpu`): every output of the specialised kernel is
bit-identical to the library kernel's on every parity case and at the word
edges, and a replayable plan switches to the specialised kernel once it is
compiled without changing any output.
"""
import concurrent.futures as cf

import numpy as np
import pytest

from cusna_gb300 import workloads as WL
from cusna_gb300.glue import marshal_period
from tests.golden.make_golden import run_case


def marshal(c, **kw):
    return marshal_period(c["inp"], c["M"], c["seed"], c["lam"], c["theta"], lamb=c["lamb"],
                          thetab=c["thetab"], **kw)


def test_specialised_source_compiles_for_every_parity_case(built_lib, monkeypatch):
    from cusna_gb300 import sim
    monkeypatch.setenv("CUSNA_JIT_CACHE", "0")     # compile, whatever a cache holds
    cases = [WL.parity_case(kind, seed=0) for kind in WL.PARITY_KINDS]
    ms = [marshal(c) for c in cases]
    # NVRTC releases the interpreter while it compiles: one thread per case
    with cf.ThreadPoolExecutor(max_workers=8) as ex:
        secs = list(ex.map(sim.specialise_check, ms))
    assert all(s > 0 for s in secs)


_CHILD = """
import sys, json
sys.path.insert(0, {root!r})
from cusna_gb300 import sim, workloads as WL
from cusna_gb300.glue import marshal_period
c = WL.parity_case("covariate", seed=0)
m = marshal_period(c["inp"], c["M"], c["seed"], c["lam"], c["theta"])
print(json.dumps(sim.specialise_check(m)))
"""


def test_compiled_plans_are_cached_on_disk_for_the_next_process(built_lib, tmp_path):
    """The first process compiles the plan (seconds) and writes it under
    CUSNA_JIT_CACHE_DIR; a second, fresh process finds it and loads it in
    milliseconds; CUSNA_JIT_CACHE=0 compiles again."""
    import json
    import os
    import subprocess
    import sys
    from tests.conftest import ROOT
    env = dict(os.environ, CUSNA_JIT_CACHE_DIR=str(tmp_path))
    env.pop("CUSNA_JIT_CACHE", None)

    def run(e):
        r = subprocess.run([sys.executable, "-c", _CHILD.format(root=ROOT)], env=e,
                           capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stderr[-2000:]
        return json.loads(r.stdout.strip().splitlines()[-1])
    first = run(env)
    files = list(tmp_path.glob("jit_*.bin"))
    assert len(files) == 1 and files[0].stat().st_size > 10000
    second = run(env)
    assert first > 1.0 and second < 0.5 * first and second < 1.0, (first, second)
    assert run(dict(env, CUSNA_JIT_CACHE="0")) > 1.0


class Engine:
    def __init__(self, specialise):
        self.specialise = specialise

    def simulate(self, m):
        from cusna_gb300 import sim
        o = sim.options(specialise=self.specialise)
        out = sim.simulate_ex(m, o)
        assert o.specialised == (1 if self.specialise > 0 else 0)
        return out


def assert_identical(a, b, tag):
    assert set(a) == set(b)
    for key in a:
        np.testing.assert_array_equal(a[key], b[key], err_msg=f"{tag}:{key}")


@pytest.mark.gpu
@pytest.mark.parametrize("kind", WL.PARITY_KINDS)
def test_gpu_specialised_kernel_is_bit_identical(gpu_lib, kind):
    c = WL.parity_case(kind, seed=3)
    assert_identical(run_case(Engine(1), c), run_case(Engine(-1), c), kind)


@pytest.mark.gpu
@pytest.mark.parametrize("n", [5, 33, 64, 200])
def test_gpu_specialised_kernel_at_word_edges(gpu_lib, n):
    for kind in ("covariate", "structural", "interaction"):
        c = WL.parity_case(kind, seed=n, n=n, M=6)
        assert_identical(run_case(Engine(1), c), run_case(Engine(-1), c), f"{kind}/n={n}")


@pytest.mark.gpu
def test_gpu_plan_switches_to_the_specialised_kernel(gpu_lib):
    """A plan compiles its effect plan in the background after a few launches;
    once the specialised kernel is loaded, launches still equal the one-shot
    calls with the same seeds and epochs."""
    from cusna_gb300 import sim
    c = WL.parity_case("covariate_all", seed=11, n=70, M=16)
    ms = [marshal(c)]
    plan = sim.SimPlan(ms, use_graph=True)
    try:
        outs = []
        for epoch in range(8):
            plan.set_epoch(epoch)
            plan.launch()
            outs.append(plan.outputs()[0])
            if epoch == 3:
                sim.specialise_wait(600.0)
        for epoch in (0, 5, 7):
            m = marshal_period(c["inp"], c["M"], c["seed"] + epoch, c["lam"], c["theta"],
                               lamb=c["lamb"], thetab=c["thetab"])
            ref = sim.simulate_ex(m, sim.options(specialise=-1))
            for key, v in outs[epoch].items():
                np.testing.assert_array_equal(v, ref[key], err_msg=f"epoch {epoch}: {key}")
    finally:
        plan.close()


def test_specialised_multi_network_source_compiles(built_lib):
    from cusna_gb300 import sim
    from cusna_gb300.glue import marshal_multi
    ms = []
    for kind in WL.MULTI_KINDS:
        inp, seed, lam, th = WL.multi_case(kind, seed=1)
        ms.append(marshal_multi(inp, 2, seed, lam, th))
    with cf.ThreadPoolExecutor(max_workers=8) as ex:
        secs = list(ex.map(sim.specialise_check_multi, ms))
    assert all(s > 0 for s in secs)


@pytest.mark.gpu
@pytest.mark.parametrize("kind,D,n", [("cross", 2, 40), ("dyadic", 3, 33), ("symmetric", 4, 65),
                                      ("empty_net", 3, 50)])
def test_gpu_specialised_multi_network_kernel_is_bit_identical(gpu_lib, kind, D, n):
    """With specialisation off the library kernel runs; with compile-on-first-use
    the specialised kernel runs; the outputs are the same bit for bit."""
    from cusna_gb300 import sim
    from cusna_gb300.glue import marshal_multi
    inp, seed, lam, th = WL.multi_case(kind, seed=n, n=n, M=6, D=D)
    try:
        sim.specialise_mode(0)
        lib_out = sim.simulate_multi(marshal_multi(inp, 6, seed, lam, th))
        sim.specialise_mode(2)
        spec_out = sim.simulate_multi(marshal_multi(inp, 6, seed, lam, th))
    finally:
        sim.specialise_mode(-1)
    assert_identical(lib_out, spec_out, f"{kind}/D={D}/n={n}")
