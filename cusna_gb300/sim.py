"""Python front end of the GB300 period simulator (libcusna_gb300.so).

`simulate(m)` runs one marshalled period (cusna_gb300.glue.Marshalled) through
`cusna_saom_simulate_period`, the reference-facing C-ABI entry point.
`simulate_ex` / `simulate_batch` reach the extension entry points
(device-resident buffers, chain offsets, one launch for many problems).
There is no CPU path: every call goes to the CUDA library, which raises
`CudaError` when it reports a failure.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .abi import (ABI_VERSION, GpuOptions, SaomProblem, SaomResult, check, load_library)
from .glue import Marshalled, result_dict


def options(device_ptrs=False, chain_offset=0, warps_per_chain=0, chains_per_cta=0,
            stream=None) -> GpuOptions:
    o = GpuOptions()
    C.memset(C.addressof(o), 0, C.sizeof(o))
    o.struct_version = ABI_VERSION
    o.device_ptrs = int(bool(device_ptrs))
    o.chain_offset = int(chain_offset)
    o.warps_per_chain = int(warps_per_chain)
    o.chains_per_cta = int(chains_per_cta)
    o.stream = stream
    return o


def simulate(m: Marshalled) -> dict:
    lib = load_library()
    st = lib.cusna_saom_simulate_period(C.byref(m.problem), C.byref(m.result))
    check(st, "cusna_saom_simulate_period", lib)
    return result_dict(m)


def simulate_ex(m: Marshalled, opts: GpuOptions) -> dict:
    lib = load_library()
    st = lib.cusna_saom_simulate_period_ex(C.byref(m.problem), C.byref(m.result), C.byref(opts))
    check(st, "cusna_saom_simulate_period_ex", lib)
    return result_dict(m)


def simulate_batch(ms: list[Marshalled], opts: GpuOptions | None = None) -> list[dict]:
    lib = load_library()
    probs = (SaomProblem * len(ms))(*[m.problem for m in ms])
    ress = (SaomResult * len(ms))(*[m.result for m in ms])
    st = lib.cusna_saom_simulate_batch(probs, ress, len(ms), C.byref(opts) if opts else None)
    check(st, "cusna_saom_simulate_batch", lib)
    return [result_dict(m) for m in ms]


def network_stats(a, n, k, type_ids, p1, p2, vmat, vmiss, dyn_flags, vb, od0, id0, wtab,
                  symflag) -> np.ndarray:
    """Statistics of one or more networks on the GPU (a: (n,n) or (M,n,n))."""
    lib = load_library()
    A = np.ascontiguousarray(np.asarray(a) != 0, dtype=np.uint8)
    single = A.ndim == 2
    if single:
        A = A[None]
    M = A.shape[0]

    def c(x, dt):
        return None if x is None else np.ascontiguousarray(np.asarray(x, dtype=dt))
    arrs = [c(type_ids, np.int32), c(p1, np.float64), c(p2, np.float64), c(vmat, np.float64),
            None if vmiss is None else c(np.asarray(vmiss) != 0, np.uint8), c(dyn_flags, np.int32),
            c(vb, np.float64), c(od0, np.int32), c(id0, np.int32), c(wtab, np.float64)]
    P = [None if x is None else x.ctypes.data for x in arrs]
    out = np.zeros((M, k))
    st = lib.cusna_network_stats_gpu(A.ctypes.data, n, M, k, *P, int(symflag), out.ctypes.data)
    check(st, "cusna_network_stats_gpu", lib)
    return out[0] if single else out


def behavior_stats(z_batch, bty, xnet, bkdist, zbar, brange, bsimmean) -> np.ndarray:
    lib = load_library()
    z = np.ascontiguousarray(np.atleast_2d(np.asarray(z_batch, dtype=np.int32)))
    M, n = z.shape
    b = np.ascontiguousarray(np.asarray(bty, dtype=np.int32))
    x = np.ascontiguousarray(np.asarray(xnet) != 0, dtype=np.uint8)
    bk = None if bkdist is None else np.ascontiguousarray(np.asarray(bkdist, dtype=np.int32))
    out = np.zeros((M, len(b)))
    st = lib.cusna_behavior_stats_gpu(z.ctypes.data, n, M, len(b), b.ctypes.data, x.ctypes.data,
                                      None if bk is None else bk.ctypes.data, float(zbar),
                                      float(brange), float(bsimmean), out.ctypes.data)
    check(st, "cusna_behavior_stats_gpu", lib)
    return out
