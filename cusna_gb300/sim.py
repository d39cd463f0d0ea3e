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

from .abi import (ABI_VERSION, GpuOptions, SaomProblem, SaomResult, ValidationOptions, check,
                  load_library)
from .glue import Marshalled, result_dict


def options(device_ptrs=False, chain_offset=0, warps_per_chain=0, chains_per_cta=0,
            stream=None, specialise=0) -> GpuOptions:
    """specialise: 0 as CUSNA_JIT says, -1 never run the specialised kernel, 1
    compile it now (cusna_gpu_options.specialise)."""
    o = GpuOptions()
    C.memset(C.addressof(o), 0, C.sizeof(o))
    o.struct_version = ABI_VERSION
    o.device_ptrs = int(bool(device_ptrs))
    o.chain_offset = int(chain_offset)
    o.warps_per_chain = int(warps_per_chain)
    o.chains_per_cta = int(chains_per_cta)
    o.stream = stream
    o.specialise = int(specialise)
    return o


def specialise_check(m: Marshalled) -> float:
    """Compile the period kernel specialised to m's effect plan (NVRTC, no
    device needed); returns the compile time in seconds, raises on failure."""
    lib = load_library()
    buf = C.create_string_buffer(1 << 16)
    sec = C.c_double(0.0)
    st = lib.cusna_saom_specialise_check(C.byref(m.problem), buf, len(buf), C.byref(sec))
    if st != 0:
        raise RuntimeError(f"specialised kernel: status {st}: {buf.value.decode()[:2000]}")
    return sec.value


def specialise_check_multi(m) -> float:
    """specialise_check for a marshalled multi-network period (marshal_multi)."""
    lib = load_library()
    buf = C.create_string_buffer(1 << 16)
    sec = C.c_double(0.0)
    st = lib.cusna_saom_specialise_check_multi(C.byref(m.problem), buf, len(buf), C.byref(sec))
    if st != 0:
        raise RuntimeError(f"specialised multi-network kernel: status {st}: "
                           f"{buf.value.decode()[:2000]}")
    return sec.value


def specialise_mode(mode: int) -> None:
    """Override CUSNA_JIT for the process: 0 never, 1 background after a few
    uses, 2 on first use, -1 back to the environment's setting."""
    lib = load_library()
    check(lib.cusna_saom_specialise_mode(int(mode)), "cusna_saom_specialise_mode", lib)


def specialise_wait(seconds: float = 120.0) -> int:
    """Wait for background compilations of specialised kernels; returns how
    many have completed."""
    lib = load_library()
    n = C.c_int32(0)
    lib.cusna_saom_specialise_wait(float(seconds), C.byref(n))
    return int(n.value)


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


def simulate_validate(m: Marshalled, trace_cap: int = 0, ustream=None, lse64: bool = False,
                      warps_per_chain: int = 0, chains_per_cta: int = 0):
    """Validation mode (cusna_saom_simulate_period_validate): the outputs and
    the per-ministep trace, an int32 array M x trace_cap x 4 of (step, focal
    actor, choice, distance change), -1 past a chain's last ministep; the
    choice is the chosen alter, or -(d + 2) for a behaviour step d. ustream
    (M x steps x (4 + n) uint32) replaces the Philox outputs of each chain's
    first `steps` ministeps; lse64 forms the score sums in float64 at every
    ministep."""
    lib = load_library()
    M = int(m.problem.M)
    tr = np.full((M, max(int(trace_cap), 0), 4), -1, dtype=np.int32)
    us = None if ustream is None else np.ascontiguousarray(ustream, dtype=np.uint32)
    o = ValidationOptions()
    C.memset(C.addressof(o), 0, C.sizeof(o))
    o.struct_version = ABI_VERSION
    o.trace_cap = int(trace_cap)
    o.trace = tr.ctypes.data if trace_cap else None
    o.ustream_steps = 0 if us is None else int(us.shape[1])
    o.ustream = None if us is None else us.ctypes.data
    o.lse64 = int(bool(lse64))
    o.warps_per_chain = int(warps_per_chain)
    o.chains_per_cta = int(chains_per_cta)
    st = lib.cusna_saom_simulate_period_validate(C.byref(m.problem), C.byref(m.result), C.byref(o))
    check(st, "cusna_saom_simulate_period_validate", lib)
    return result_dict(m), tr


def simulate_batch(ms: list[Marshalled], opts: GpuOptions | None = None) -> list[dict]:
    lib = load_library()
    probs = (SaomProblem * len(ms))(*[m.problem for m in ms])
    ress = (SaomResult * len(ms))(*[m.result for m in ms])
    st = lib.cusna_saom_simulate_batch(probs, ress, len(ms), C.byref(opts) if opts else None)
    check(st, "cusna_saom_simulate_batch", lib)
    return [result_dict(m) for m in ms]


PARAM_FIELDS = ("theta", "lam", "lamb", "thetab")


class SimPlan:
    """Replayable simulation of many marshalled problems (cusna_saom_plan_*).

    Every input moves to device memory once. The parameters (theta, lam, lamb,
    thetab) live in contiguous device buffers holding one row per problem
    (shared by its M chains; `per_chain=True` keeps a row per chain), which
    `set_params` rewrites between launches. Outputs go to contiguous device
    buffers, one per output name, which `outputs` copies back in one transfer
    each. `launch` re-simulates every problem in one persistent kernel, the
    first time with Philox key = the problem's seed and then seed + 1, seed +
    2, ... (the epoch advances on the device); with `use_graph` the launch is
    replayed from a CUDA graph. Device buffers are torch tensors (allocation
    only); the simulation is the library's."""

    def __init__(self, ms: list[Marshalled], per_chain: bool = False, use_graph: bool = True):
        import torch
        self.torch = torch
        self.lib = load_library()
        self.dev = torch.device("cuda", torch.cuda.current_device())
        self.use_graph = bool(use_graph)
        self.count = len(ms)
        self.M = [int(m.problem.M) for m in ms]
        probs = (SaomProblem * self.count)()
        ress = (SaomResult * self.count)()
        self._keep = []
        self.params, self.outs = {}, {}
        for q, m in enumerate(ms):
            probs[q] = SaomProblem.from_buffer_copy(m.problem)
            ress[q] = SaomResult.from_buffer_copy(m.result)
        keys = {k for k in ms[0].keep if k.startswith("out_") or k in PARAM_FIELDS}
        for q, m in enumerate(ms):
            if {k for k in m.keep if k.startswith("out_") or k in PARAM_FIELDS} != keys:
                raise ValueError("a plan's problems must carry the same parameters and outputs")
            # every host pointer of the struct copy is replaced by a device one
            for name, a in m.keep.items():
                if not (name.startswith("out_") or name in PARAM_FIELDS):
                    setattr(probs[q], name, self._upload(a).data_ptr())
        # parameter buffers: rows of each problem back to back
        for name in PARAM_FIELDS:
            if name not in ms[0].keep:
                continue
            rows = []
            for m in ms:
                a = np.asarray(m.keep[name], dtype=np.float32).reshape(int(m.problem.M), -1)
                rows.append(a if per_chain else a[:1])
            width = rows[0].shape[1]
            host = np.concatenate(rows, axis=0)
            t = self._upload(host)
            off = np.cumsum([0] + [r.shape[0] for r in rows])
            for q in range(self.count):
                setattr(probs[q], name, t.data_ptr() + 4 * width * int(off[q]))
            self.params[name] = (t, width, off)
        for name in [k for k in ms[0].keep if k.startswith("out_")]:
            arrs = [np.asarray(m.keep[name]) for m in ms]
            sizes = [a.size for a in arrs]
            off = np.cumsum([0] + sizes)
            t = torch.empty(int(off[-1]) * arrs[0].itemsize, dtype=torch.uint8, device=self.dev)
            self._keep.append(t)
            for q in range(self.count):
                setattr(ress[q], name[4:], t.data_ptr() + arrs[0].itemsize * int(off[q]))
            self.outs[name[4:]] = (t, arrs[0].dtype, [a.shape for a in arrs], off)
        self._probs, self._ress = probs, ress
        plan = C.c_void_p()
        check(self.lib.cusna_saom_plan_create(probs, ress, self.count, 0 if per_chain else 1,
                                              C.byref(plan)), "cusna_saom_plan_create", self.lib)
        self.plan = plan

    def _upload(self, a):
        a = np.ascontiguousarray(a)
        t = self.torch.from_numpy(a.view(np.uint8).reshape(-1).copy()).to(self.dev)
        self._keep.append(t)
        return t

    def _stream(self):
        return self.torch.cuda.current_stream(self.dev).cuda_stream

    def set_params(self, **rows):
        """Write parameters for the next launch: name=(count, width) rows, or
        one row broadcast to every problem (rows of a per-chain plan:
        (sum of M, width))."""
        for name, val in rows.items():
            t, width, off = self.params[name]
            n_rows = int(off[-1])
            a = np.asarray(val, dtype=np.float32).reshape(-1, width)
            if a.shape[0] == 1 and n_rows > 1:
                a = np.repeat(a, n_rows, axis=0)
            if a.shape[0] != n_rows:
                raise ValueError(f"{name}: {a.shape[0]} rows for {n_rows}")
            t.copy_(self.torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).reshape(-1)))

    def set_epoch(self, epoch: int):
        check(self.lib.cusna_saom_plan_set_epoch(self.plan, int(epoch)),
              "cusna_saom_plan_set_epoch", self.lib)

    def launch(self):
        check(self.lib.cusna_saom_plan_launch(self.plan, self._stream(), 1 if self.use_graph else 0),
              "cusna_saom_plan_launch", self.lib)

    def shape(self):
        g, t, c = C.c_int32(), C.c_int32(), C.c_int32()
        self.lib.cusna_saom_plan_shape(self.plan, C.byref(g), C.byref(t), C.byref(c))
        return g.value, t.value, c.value

    def outputs(self, names=None) -> list[dict]:
        """Per problem, the named outputs of the last launch (host arrays)."""
        names = names or list(self.outs)
        res = [dict() for _ in range(self.count)]
        for name in names:
            t, dt, shapes, off = self.outs[name]
            host = t.cpu().numpy().view(dt)
            for q in range(self.count):
                res[q][name] = host[int(off[q]):int(off[q + 1])].reshape(shapes[q])
        return res

    def close(self):
        if getattr(self, "plan", None) is not None and self.plan.value:
            self.lib.cusna_saom_plan_destroy(self.plan)
            self.plan = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


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


def simulate_multi(m) -> dict:
    """One marshalled multi-network period (cusna_gb300.glue.marshal_multi)
    through cusna_saom_simulate_multi."""
    lib = load_library()
    st = lib.cusna_saom_simulate_multi(C.byref(m.problem), C.byref(m.result))
    check(st, "cusna_saom_simulate_multi", lib)
    return result_dict(m)


def cross_stats(a_batch, wp, t, parm=0.0) -> np.ndarray:
    """Cross-network statistic of type t (33..37) of own networks a_batch
    ((n,n) or (M,n,n)) against the source predictor wp, on the GPU."""
    lib = load_library()
    a = np.ascontiguousarray(np.asarray(a_batch) != 0, dtype=np.uint8)
    if a.ndim == 2:
        a = a[None]
    M, n = a.shape[0], a.shape[1]
    w = np.ascontiguousarray(np.asarray(wp) != 0, dtype=np.uint8)
    out = np.zeros(M)
    st = lib.cusna_cross_stats(a.ctypes.data, w.ctypes.data, n, M, int(t), float(parm),
                               out.ctypes.data)
    check(st, "cusna_cross_stats", lib)
    return out


def _u8(x):
    return None if x is None else np.ascontiguousarray(np.asarray(x) != 0, dtype=np.uint8)


def typed_stats(a_batch, etype, F, x0, keep=None, force=None, keepS=None, forceS=None,
                miss_m=None, miss_m1=None) -> np.ndarray:
    """Creation (etype 1) or endowment (2, negated) statistic of one typed
    effect over end networks a_batch ((n,n) or (M,n,n)), on the GPU."""
    lib = load_library()
    a = _u8(a_batch)
    if a.ndim == 2:
        a = a[None]
    M, n = a.shape[0], a.shape[1]
    Fm = np.ascontiguousarray(np.asarray(F, dtype=np.float64))
    arrs = [_u8(x0), _u8(keep), _u8(force), _u8(keepS), _u8(forceS), _u8(miss_m), _u8(miss_m1)]
    P = [None if x is None else x.ctypes.data for x in arrs]
    out = np.zeros(M)
    st = lib.cusna_typed_stats(a.ctypes.data, n, M, int(etype), Fm.ctypes.data, *P,
                               out.ctypes.data)
    check(st, "cusna_typed_stats", lib)
    return out


def gof_distribution(a_batch, kind, levls) -> np.ndarray:
    """sienaGOF auxiliary distribution of end networks a_batch ((n,n) or
    (M,n,n)) on the GPU: kind 0 in-degree / 1 out-degree cumulative counts per
    level, (M, len(levls)); kind 2 ordered pairs within each geodesic level and
    the unreachable pairs, (M, len(levls) + 1)."""
    lib = load_library()
    a = _u8(a_batch)
    if a.ndim == 2:
        a = a[None]
    M, n = a.shape[0], a.shape[1]
    lv = np.ascontiguousarray(np.asarray(levls, dtype=np.int32))
    cols = len(lv) + 1 if kind == 2 else len(lv)
    out = np.zeros((M, cols))
    st = lib.cusna_gof_distribution(a.ctypes.data, n, M, int(kind), lv.ctypes.data, len(lv),
                                    out.ctypes.data)
    check(st, "cusna_gof_distribution", lib)
    return out


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
