"""cusna_saom_simulate_period_static, the entry point for callers that cannot
allocate device memory: a host whose device memory is all handed out by its
own allocator (an R session that reserved the GPU for another framework, an
embedding application with a fixed memory budget), or a latency-bound loop
that must not enter the allocator. It must give the same results as
cusna_saom_simulate_period on the same problem, call after call, although all
its scratch is one fixed device array that every call reuses. The file name
makes pytest run it after every other test."""
import ctypes as C

import numpy as np
import pytest

from cusna_gb300 import workloads as WL
from cusna_gb300.abi import ERR_UNSUPPORTED, OK
from cusna_gb300.glue import marshal_period
from tests.golden.make_golden import run_case
from tests.test_gpu_parity import GpuEngine, assert_parity

pytestmark = pytest.mark.gpu


def _to_device(m, torch):
    """Copy every array of a marshalled period to the GPU and point the
    structs at the copies (the caller's allocations, made by the test)."""
    dev = {}
    for name, arr in m.keep.items():
        t = torch.from_numpy(np.ascontiguousarray(arr).view(np.uint8).reshape(-1).copy()).cuda()
        dev[name] = t
        field = name[4:] if name.startswith("out_") else name
        target = m.result if name.startswith("out_") else m.problem
        setattr(target, field, t.data_ptr())
    return dev


def _outputs(m, dev):
    return {name[4:]: dev[name].cpu().numpy().view(arr.dtype).reshape(arr.shape)
            for name, arr in m.keep.items() if name.startswith("out_")}


@pytest.mark.parametrize("kind,n,M", [("covariate", 60, 7), ("coevol", 45, 5),
                                      ("structural", 70, 4), ("gw", 50, 6), ("masks", 41, 5),
                                      ("baseline", 33, 3), ("covariate_all", 40, 4),
                                      ("interaction", 40, 4), ("typed", 40, 4),
                                      ("conditional", 40, 4), ("composition", 40, 4),
                                      ("symmetric", 40, 4), ("rates", 40, 4)])
def test_static_entry_point_matches_allocating_one(gpu_lib, kind, n, M):
    torch = pytest.importorskip("torch")
    c = WL.parity_case(kind, seed=21, n=n, M=M)
    ref = run_case(GpuEngine(), c)
    m = marshal_period(c["inp"], c["M"], c["seed"], c["lam"], c["theta"], lamb=c["lamb"],
                       thetab=c["thetab"], want_ends=True)
    dev = _to_device(m, torch)
    for call in range(2):       # two calls in a row share the static scratch
        for name in dev:
            if name.startswith("out_"):
                dev[name].zero_()
        st = gpu_lib.cusna_saom_simulate_period_static(C.byref(m.problem), C.byref(m.result), None)
        assert st == OK, gpu_lib.cusna_last_error()
        torch.cuda.synchronize()
        assert_parity(_outputs(m, dev), ref, f"{kind}/call{call}")


def test_static_entry_point_refuses_oversized_problems(gpu_lib):
    """The n=1000, 1024-chain co-evolution workload keeps each running chain's
    in-rows in scratch (about 128 KB per resident chain, some 19 MB in all),
    more than the 16 MiB array: the call must refuse it, name the size, and
    leave the allocating entry points able to run it."""
    torch = pytest.importorskip("torch")
    inp, M, seed, lam, theta, lamb, thetab = WL.c4_period(M=1024)
    m = marshal_period(inp, M, seed, lam, theta, lamb=lamb, thetab=thetab)
    _to_device(m, torch)
    st = gpu_lib.cusna_saom_simulate_period_static(C.byref(m.problem), C.byref(m.result), None)
    assert st == ERR_UNSUPPORTED
    assert b"scratch" in gpu_lib.cusna_last_error()
