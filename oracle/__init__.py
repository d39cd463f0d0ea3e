"""CPU ORACLE for the SAOM period simulator -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this
package; the product (cusna_gb300) never does. Two CPU engines sit behind the
same interface:

  * Oracle("port") -- oracle/cusna_oracle.c, a C restatement of the reference
    engine (src/libcusna_saom_cpu.cpp), built by `make -C oracle`;
  * Oracle("reference") -- the reference engine itself compiled from its own
    sources into oracle/_ref/ (`make -C oracle ref`). It only exists where the
    reference sources are present.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "libcusna_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libcusna_ref.so")
# the reference package checked out beside this repository, unless
# CUSNA_REFERENCE_DIR names another place; absent on machines without it
REF_SRC = os.environ.get("CUSNA_REFERENCE_DIR",
                         os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference"))


def build(ref: bool = True) -> None:
    """Compile the oracle (and the reference engine when its sources exist)."""
    subprocess.check_call(["make", "-s", "-C", HERE])
    if ref and os.path.exists(os.path.join(REF_SRC, "src", "libcusna_saom_cpu.cpp")):
        subprocess.check_call(["make", "-s", "-C", HERE, "ref", f"REF={REF_SRC}"])


def reference_available() -> bool:
    return os.path.exists(REF_SO)


class Oracle:
    """ctypes front end to one CPU engine ("port" or "reference")."""

    def __init__(self, kind: str = "port"):
        from cusna_gb300.abi import SaomProblem, SaomResult
        self.kind = kind
        path = PORT_SO if kind == "port" else REF_SO
        if not os.path.exists(path):
            if kind == "port":
                build(ref=False)
            else:
                raise FileNotFoundError(path)
        self.lib = C.CDLL(path)
        pre = "oracle_" if kind == "port" else "cusna_"
        sim = "oracle_simulate_period" if kind == "port" else "cusna_saom_simulate_period_cpu"
        self._sim = getattr(self.lib, sim)
        self._sim.argtypes = [C.POINTER(SaomProblem), C.POINTER(SaomResult)]
        self._sim.restype = C.c_int32
        vp, i32 = C.c_void_p, C.c_int32
        self._ns = getattr(self.lib, pre + "network_stats")
        self._ns.argtypes = [vp, i32, i32, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, i32, vp]
        self._ns.restype = i32
        self._bs = getattr(self.lib, pre + "behavior_stats")
        self._bs.argtypes = [vp, i32, i32, i32, vp, vp, vp, C.c_double, C.c_double,
                             C.c_double, vp]
        self._bs.restype = i32
        from cusna_gb300.abi import MultiProblem, MultiResult
        self._multi = getattr(self.lib, "oracle_simulate_multi" if kind == "port"
                              else "cusna_saom_simulate_multi_cpu")
        self._multi.argtypes = [C.POINTER(MultiProblem), C.POINTER(MultiResult)]
        self._multi.restype = i32
        self._cross = getattr(self.lib, "oracle_cross_stats" if kind == "port" else "cusna_cross_stats")
        self._cross.argtypes = [vp, vp, i32, i32, i32, C.c_double, vp]
        self._cross.restype = i32
        self._typed = getattr(self.lib, "oracle_typed_stats" if kind == "port" else "cusna_typed_stats")
        self._typed.argtypes = [vp, i32, i32, i32, vp, vp, vp, vp, vp, vp, vp, vp, vp]
        self._typed.restype = i32
        self._gof = getattr(self.lib, "oracle_gof_distribution" if kind == "port"
                            else "cusna_gof_distribution")
        self._gof.argtypes = [vp, i32, i32, i32, vp, i32, vp]
        self._gof.restype = i32
        if kind == "port":
            self._val = self.lib.oracle_simulate_period_validate
            self._val.argtypes = [C.POINTER(SaomProblem), C.POINTER(SaomResult), vp, i32, vp, i32]
            self._val.restype = i32
            self._ph = self.lib.oracle_philox4x32
            self._ph.argtypes = [vp, vp, vp]
            self._ph.restype = i32
            self.lib.oracle_max_threads.restype = i32

    def max_threads(self) -> int:
        if self.kind == "port":
            return int(self.lib.oracle_max_threads())
        return os.cpu_count() or 1

    def simulate(self, m, threads: int = 0) -> dict:
        """Run a marshalled period (cusna_gb300.glue.Marshalled); returns the
        output arrays by name."""
        from cusna_gb300.glue import result_dict
        m.problem.threads = int(threads)
        st = self._sim(C.byref(m.problem), C.byref(m.result))
        if st != 0:
            raise RuntimeError(f"{self.kind} simulate_period status {st}")
        return result_dict(m)

    def simulate_validate(self, m, trace_cap: int = 0, ustream=None, threads: int = 0):
        """Validation mode of the port (no counterpart in the reference): the
        outputs and the per-ministep trace (M x trace_cap x 4 int32: step,
        actor, choice, distance change; -1 past a chain's end), optionally
        with supplied words (M x steps x (4 + n) uint32) in place of Philox."""
        from cusna_gb300.glue import result_dict
        M = int(m.problem.M)
        tr = np.full((M, max(int(trace_cap), 0), 4), -1, dtype=np.int32)
        us = None if ustream is None else np.ascontiguousarray(ustream, dtype=np.uint32)
        steps = 0 if us is None else int(us.shape[1])
        m.problem.threads = int(threads)
        st = self._val(C.byref(m.problem), C.byref(m.result), tr.ctypes.data if trace_cap else None,
                       int(trace_cap), None if us is None else us.ctypes.data, steps)
        if st != 0:
            raise RuntimeError(f"{self.kind} simulate_period_validate status {st}")
        return result_dict(m), tr

    def simulate_multi(self, m) -> dict:
        """A marshalled multi-network period (cusna_gb300.glue.marshal_multi)."""
        from cusna_gb300.glue import result_dict
        st = self._multi(C.byref(m.problem), C.byref(m.result))
        if st != 0:
            raise RuntimeError(f"{self.kind} simulate_multi status {st}")
        return result_dict(m)

    def cross_stats(self, a_batch, wp, t, parm=0.0) -> np.ndarray:
        a = np.ascontiguousarray(np.asarray(a_batch) != 0, dtype=np.uint8)
        if a.ndim == 2:
            a = a[None]
        M, n = a.shape[0], a.shape[1]
        w = np.ascontiguousarray(np.asarray(wp) != 0, dtype=np.uint8)
        out = np.zeros(M)
        st = self._cross(a.ctypes.data, w.ctypes.data, n, M, int(t), float(parm), out.ctypes.data)
        if st != 0:
            raise RuntimeError(f"{self.kind} cross_stats status {st}")
        return out

    def typed_stats(self, a_batch, etype, F, x0, keep=None, force=None, keepS=None,
                    forceS=None, miss_m=None, miss_m1=None) -> np.ndarray:
        def u8(x):
            return None if x is None else np.ascontiguousarray(np.asarray(x) != 0, dtype=np.uint8)
        a = u8(a_batch)
        if a.ndim == 2:
            a = a[None]
        M, n = a.shape[0], a.shape[1]
        Fm = np.ascontiguousarray(np.asarray(F, dtype=np.float64))
        arrs = [u8(x0), u8(keep), u8(force), u8(keepS), u8(forceS), u8(miss_m), u8(miss_m1)]
        P = [None if x is None else x.ctypes.data for x in arrs]
        out = np.zeros(M)
        st = self._typed(a.ctypes.data, n, M, int(etype), Fm.ctypes.data, *P, out.ctypes.data)
        if st != 0:
            raise RuntimeError(f"{self.kind} typed_stats status {st}")
        return out

    def gof_distribution(self, a_batch, kind, levls) -> np.ndarray:
        a = np.ascontiguousarray(np.asarray(a_batch) != 0, dtype=np.uint8)
        if a.ndim == 2:
            a = a[None]
        M, n = a.shape[0], a.shape[1]
        lv = np.ascontiguousarray(np.asarray(levls, dtype=np.int32))
        out = np.zeros((M, len(lv) + 1 if kind == 2 else len(lv)))
        st = self._gof(a.ctypes.data, n, M, int(kind), lv.ctypes.data, len(lv), out.ctypes.data)
        if st != 0:
            raise RuntimeError(f"{self.kind} gof_distribution status {st}")
        return out

    def simulate_batch(self, ms, threads: int = 0) -> list:
        """The engine interface of cusna_gb300.mom: one call per period."""
        return [self.simulate(m, threads=threads) for m in ms]

    def network_stats(self, a, n, k, type_ids, p1, p2, vmat, vmiss, dyn_flags, vb, od0, id0,
                      wtab, symflag) -> np.ndarray:
        def c(x, dt):
            return None if x is None else np.ascontiguousarray(np.asarray(x, dtype=dt))
        arrs = [c(np.asarray(a) != 0, np.uint8), c(type_ids, np.int32), c(p1, np.float64),
                c(p2, np.float64), c(vmat, np.float64),
                None if vmiss is None else c(np.asarray(vmiss) != 0, np.uint8),
                c(dyn_flags, np.int32), c(vb, np.float64), c(od0, np.int32), c(id0, np.int32),
                c(wtab, np.float64)]
        out = np.zeros(k)
        P = [None if x is None else x.ctypes.data for x in arrs]
        st = self._ns(P[0], n, k, P[1], P[2], P[3], P[4], P[5], P[6], P[7], P[8], P[9], P[10],
                      int(symflag), out.ctypes.data)
        if st != 0:
            raise RuntimeError(f"network_stats status {st}")
        return out

    def behavior_stats(self, z_batch, bty, xnet, bkdist, zbar, brange, bsimmean) -> np.ndarray:
        z = np.ascontiguousarray(np.atleast_2d(np.asarray(z_batch, dtype=np.int32)))
        M, n = z.shape
        b = np.ascontiguousarray(np.asarray(bty, dtype=np.int32))
        x = np.ascontiguousarray(np.asarray(xnet) != 0, dtype=np.uint8)
        bk = None if bkdist is None else np.ascontiguousarray(np.asarray(bkdist, dtype=np.int32))
        out = np.zeros((M, len(b)))
        st = self._bs(z.ctypes.data, n, M, len(b), b.ctypes.data, x.ctypes.data,
                      None if bk is None else bk.ctypes.data, float(zbar), float(brange),
                      float(bsimmean), out.ctypes.data)
        if st != 0:
            raise RuntimeError(f"behavior_stats status {st}")
        return out

    def philox(self, counter, key) -> np.ndarray:
        ctr = np.ascontiguousarray(np.asarray(counter, dtype=np.uint32))
        ky = np.ascontiguousarray(np.asarray(key, dtype=np.uint32))
        out = np.zeros(4, dtype=np.uint32)
        self._ph(ctr.ctypes.data, ky.ctypes.data, out.ctypes.data)
        return out
