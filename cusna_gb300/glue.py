"""Marshalling of one SAOM period into the C ABI structs, as the reference's
cpp11 glue does (src/cusna_saom_glue.cpp:57-189, `cusna_simulate_period_cpu_`).

`marshal_period()` builds a `cusna_saom_problem` / `cusna_saom_result` pair
from numpy arrays and keeps the arrays alive in the returned `Marshalled`.
These are the glue's conventions: dense start network -> packed out/in rows;
lam and theta broadcast over the M chains as float32; only the *64 descriptors
set; nact = n; brange = 1 without behaviour. The same structs feed the GPU entry
point and, in the tests, the CPU oracle.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from .abi import ABI_VERSION, SaomProblem, SaomResult, pack_rows, ptr


@dataclass
class PeriodInputs:
    """Chain-invariant inputs of one period (the glue's argument list)."""
    x0: np.ndarray                       # dense n*n start network
    type_ids: np.ndarray                 # (k,)
    vmat: np.ndarray | None = None       # (k,n) float64
    wtab: np.ndarray | None = None       # (k,n+1) float64
    vb: np.ndarray | None = None         # (n,) float64 centred start behaviour
    p1: np.ndarray | None = None
    p2: np.ndarray | None = None
    vmiss: np.ndarray | None = None      # (k,n)
    etypes: np.ndarray | None = None
    dyn_flags: np.ndarray | None = None
    dyc_idx: np.ndarray | None = None
    int_idx: np.ndarray | None = None    # (k,3) interaction components, -1 padded
    maxdegree: int = 0
    conditional: int = 0
    target_dist: int = 0
    symflag: int = 0
    # behaviour (kb > 0)
    bty: np.ndarray | None = None
    z0: np.ndarray | None = None
    bkdist: np.ndarray | None = None
    zmin: int = 0
    zmax: int = 0
    zbar: float = 0.0
    brange: float = 0.0
    bsimmean: float = 0.0
    # struct options the glue leaves at their defaults
    sim_start: np.ndarray | None = None  # dense simulation start network
    kdist: np.ndarray | None = None      # dense masks
    perm: np.ndarray | None = None
    keep: np.ndarray | None = None
    force: np.ndarray | None = None
    od0: np.ndarray | None = None
    id0: np.ndarray | None = None
    act: np.ndarray | None = None        # active actor ids first
    nact: int | None = None
    inactive: np.ndarray | None = None   # bool (n,) -> inactw + has_comp
    rkind: np.ndarray | None = None
    ralpha: np.ndarray | None = None
    ru: np.ndarray | None = None         # (nrate, n)

    @property
    def n(self) -> int:
        return int(np.asarray(self.x0).shape[0])

    @property
    def k(self) -> int:
        return int(len(self.type_ids))

    @property
    def kb(self) -> int:
        return 0 if self.bty is None else int(len(self.bty))

    @property
    def nrate(self) -> int:
        return 0 if self.rkind is None else int(len(self.rkind))


@dataclass
class Marshalled:
    problem: SaomProblem
    result: SaomResult
    keep: dict = field(default_factory=dict)     # numpy arrays the structs point at

    def out(self, name):
        return self.keep.get("out_" + name)

    def drop_outputs(self, names):
        """Stop requesting the named outputs (their result pointers become NULL)."""
        for name in names:
            if self.keep.pop("out_" + name, None) is not None:
                setattr(self.result, name, None)


def _c(a, dt):
    return np.ascontiguousarray(np.asarray(a, dtype=dt))


def marshal_period(inp: PeriodInputs, M: int, seed: int, lam, theta, lamb=0.0, thetab=None,
                   want_ends: bool = False, outputs=("stats", "scores", "ntim", "dist",
                                                     "dist_stat", "steps")) -> Marshalled:
    """Build the problem/result structs for M chains of one period.

    lam / lamb: scalar (broadcast, as the glue does) or length-M vector.
    theta: (k,) broadcast, or (M,k) per chain. thetab likewise (kb,) or (M,kb).
    """
    n, k, kb, nr = inp.n, inp.k, inp.kb, inp.nrate
    W = (n + 31) // 32
    keep = {}

    def hold(name, arr):
        keep[name] = arr
        return ptr(arr)

    p = SaomProblem()
    C.memset(C.addressof(p), 0, C.sizeof(p))
    p.struct_version = ABI_VERSION
    p.n, p.W, p.k, p.M, p.threads = n, W, k, int(M), 0
    x0 = np.asarray(inp.x0) != 0
    out_rows, in_rows = pack_rows(x0)
    p.x0_out = hold("x0_out", out_rows)
    p.x0_in = hold("x0_in", in_rows)
    if inp.sim_start is not None:
        so, si = pack_rows(np.asarray(inp.sim_start) != 0)
        p.sim_out = hold("sim_out", so)
        p.sim_in = hold("sim_in", si)
    lamv = np.broadcast_to(np.asarray(lam, dtype=np.float64), (M,)).astype(np.float32)
    p.lam = hold("lam", _c(lamv, np.float32))
    th = np.asarray(theta, dtype=np.float64)
    thv = np.broadcast_to(th, (M, k)) if th.ndim == 1 else th.reshape(M, k)
    p.theta = hold("theta", _c(thv.astype(np.float32), np.float32))
    p.type_ids = hold("type_ids", _c(inp.type_ids, np.int32))
    p.etypes = hold("etypes", _c(inp.etypes if inp.etypes is not None else np.zeros(k), np.int32))
    p.dyn_flags = hold("dyn_flags", _c(inp.dyn_flags if inp.dyn_flags is not None else np.zeros(k), np.int32))
    p.dyc_idx = hold("dyc_idx", _c(inp.dyc_idx if inp.dyc_idx is not None else -np.ones(k), np.int32))
    if inp.int_idx is not None:
        ii = _c(inp.int_idx, np.int32).reshape(k, 3)
        p.int0 = hold("int0", _c(ii[:, 0], np.int32))
        p.int1 = hold("int1", _c(ii[:, 1], np.int32))
        p.int2 = hold("int2", _c(ii[:, 2], np.int32))
    vm = np.zeros((k, n)) if inp.vmat is None else inp.vmat
    p.vmiss = hold("vmiss", _c((np.zeros((k, n)) if inp.vmiss is None else inp.vmiss) != 0, np.uint8))
    p.vmat64 = hold("vmat64", _c(vm, np.float64))
    p.wtab64 = hold("wtab64", _c(np.zeros((k, n + 1)) if inp.wtab is None else inp.wtab, np.float64))
    p.vb64 = hold("vb64", _c(np.zeros(n) if inp.vb is None else inp.vb, np.float64))
    p.p1_64 = hold("p1_64", _c(np.zeros(k) if inp.p1 is None else inp.p1, np.float64))
    p.p2_64 = hold("p2_64", _c(np.zeros(k) if inp.p2 is None else inp.p2, np.float64))
    p.maxdegree = int(inp.maxdegree)
    p.conditional = int(inp.conditional)
    p.target_dist = int(inp.target_dist)
    p.symflag = int(inp.symflag)
    p.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
    p.nact = n
    p.brange = 1.0
    for name, m in (("kdist", inp.kdist), ("perm", inp.perm), ("keep_out", inp.keep),
                    ("force_out", inp.force)):
        if m is not None:
            setattr(p, name, hold(name, pack_rows(np.asarray(m) != 0)[0]))
    if inp.od0 is not None:
        p.od0 = hold("od0", _c(inp.od0, np.int32))
    if inp.id0 is not None:
        p.id0 = hold("id0", _c(inp.id0, np.int32))
    if inp.act is not None:
        p.act = hold("act", _c(inp.act, np.int32))
        p.nact = int(inp.nact if inp.nact is not None else len(inp.act))
    if inp.inactive is not None:
        bits = np.zeros(W * 32, dtype=np.uint8)
        bits[:n] = np.asarray(inp.inactive) != 0
        p.inactw = hold("inactw", np.packbits(bits, bitorder="little").view(np.uint32).copy())
        p.has_comp = 1
    if kb > 0:
        p.kb = kb
        lbv = np.broadcast_to(np.asarray(lamb, dtype=np.float64), (M,)).astype(np.float32)
        p.lamb = hold("lamb", _c(lbv, np.float32))
        tb = np.asarray(thetab, dtype=np.float64)
        tbv = np.broadcast_to(tb, (M, kb)) if tb.ndim == 1 else tb.reshape(M, kb)
        p.thetab = hold("thetab", _c(tbv.astype(np.float32), np.float32))
        p.bty = hold("bty", _c(inp.bty, np.int32))
        p.z0 = hold("z0", _c(inp.z0, np.int32))
        p.bkdist = hold("bkdist", _c(inp.bkdist if inp.bkdist is not None else np.ones(n), np.int32))
        p.zmin, p.zmax = int(inp.zmin), int(inp.zmax)
        p.zbar = float(np.float32(inp.zbar))
        p.brange = float(np.float32(inp.brange))
        p.bsimmean = float(np.float32(inp.bsimmean))
    if nr > 0:
        p.nrate = nr
        p.rkind = hold("rkind", _c(inp.rkind, np.int32))
        p.ralpha = hold("ralpha", _c(inp.ralpha, np.float32))
        p.ru = hold("ru", _c(inp.ru if inp.ru is not None else np.zeros((nr, n)), np.float32))

    r = SaomResult()
    C.memset(C.addressof(r), 0, C.sizeof(r))
    r.struct_version = ABI_VERSION
    shapes = dict(stats=((M, k), np.float64), ntim=((M,), np.float64),
                  scores=((M, k + 1), np.float32), dist=((M,), np.int32),
                  dist_stat=((M,), np.int32), steps=((M,), np.int32))
    if kb > 0:
        shapes.update(bdist=((M,), np.int32), bscores=((M, kb + 1), np.float32),
                      z_end=((M, n), np.int32))
    if nr > 0:
        shapes.update(rscores=((M, nr), np.float32), actor_dist=((M, n), np.int32))
    wanted = set(outputs)
    if kb > 0:
        wanted |= {"bdist", "bscores", "z_end"}
    if nr > 0:
        wanted |= {"rscores", "actor_dist"}
    for name, (shape, dt) in shapes.items():
        if name in wanted:
            arr = np.zeros(shape, dtype=dt)
            setattr(r, name, hold("out_" + name, arr))
    if want_ends:
        ae = np.zeros((M, n, n), dtype=np.uint8)
        r.want_end_nets = 1
        r.a_ends = hold("out_a_ends", ae)
    return Marshalled(p, r, keep)


def result_dict(m: Marshalled) -> dict:
    return {k[4:]: v for k, v in m.keep.items() if k.startswith("out_")}


@dataclass
class MultiInputs:
    """One multi-network period (the arguments of the reference glue's
    cusna_simulate_multi_cpu_, src/cusna_saom_glue.cpp:230-290): D start
    networks on n shared actors and the effects of all networks."""
    x0s: list                     # D dense n*n start networks
    type_ids: np.ndarray          # k
    netof: np.ndarray             # k, 0..D-1
    netref: np.ndarray            # k, source network of cross effects (else -1)
    etypes: np.ndarray            # k
    wtab: np.ndarray              # k*(n+1)
    p1: np.ndarray                # k
    p2: np.ndarray                # k
    vmat: np.ndarray              # k*n
    perm: list | None = None      # D dense n*n permitted dyads (None: all i != j)
    symf: np.ndarray | None = None  # D
    dyc: np.ndarray | None = None   # n*n dyadic covariate (read by type 22)
    dyc_idx: np.ndarray | None = None  # k: 0 reads dyc, -1 none (None: all -1)

    @property
    def n(self):
        return int(np.asarray(self.x0s[0]).shape[0])

    @property
    def D(self):
        return len(self.x0s)

    @property
    def k(self):
        return len(self.type_ids)


def marshal_multi(inp: MultiInputs, M: int, seed: int, lam, theta,
                  want_ends: bool = True) -> Marshalled:
    """cusna_saom_multi_problem/result for M chains, marshalled as the glue does
    (float32 descriptors and parameters, every actor active).
    lam: (D,) broadcast or (M, D); theta: (k,) broadcast or (M, k)."""
    from .abi import MultiProblem, MultiResult
    n, D, k = inp.n, inp.D, inp.k
    W = (n + 31) // 32
    keep = {}

    def hold(name, arr):
        keep[name] = arr
        return ptr(arr)

    p = MultiProblem()
    C.memset(C.addressof(p), 0, C.sizeof(p))
    p.struct_version = ABI_VERSION
    p.n, p.W, p.k, p.M, p.D, p.threads = n, W, k, int(M), D, 0
    outs, ins, perms = [], [], []
    for d in range(D):
        o, i_ = pack_rows(np.asarray(inp.x0s[d]) != 0)
        outs.append(o)
        ins.append(i_)
        pm = (np.asarray(inp.perm[d]) != 0) if inp.perm is not None else ~np.eye(n, dtype=bool)
        perms.append(pack_rows(pm)[0])
    p.x0_out = hold("x0_out", np.concatenate(outs))
    p.x0_in = hold("x0_in", np.concatenate(ins))
    p.perm = hold("perm", np.concatenate(perms))
    lv = np.asarray(lam, dtype=np.float64)
    lv = np.broadcast_to(lv, (M, D)) if lv.ndim == 1 else lv.reshape(M, D)
    p.lam = hold("lam", _c(lv.astype(np.float32), np.float32))
    th = np.asarray(theta, dtype=np.float64)
    th = np.broadcast_to(th, (M, k)) if th.ndim == 1 else th.reshape(M, k)
    p.theta = hold("theta", _c(th.astype(np.float32), np.float32))
    p.type_ids = hold("type_ids", _c(inp.type_ids, np.int32))
    p.etypes = hold("etypes", _c(inp.etypes, np.int32))
    p.netof = hold("netof", _c(inp.netof, np.int32))
    p.netref = hold("netref", _c(inp.netref, np.int32))
    p.wtab = hold("wtab", _c(inp.wtab, np.float32))
    p.p1 = hold("p1", _c(inp.p1, np.float32))
    p.p2 = hold("p2", _c(inp.p2, np.float32))
    p.vmat = hold("vmat", _c(inp.vmat, np.float32))
    p.dyc_idx = hold("dyc_idx", _c(inp.dyc_idx if inp.dyc_idx is not None
                                   else -np.ones(k), np.int32))
    if inp.dyc is not None:
        p.dyc = hold("dyc", _c(inp.dyc, np.float32))
    p.symf = hold("symf", _c(inp.symf if inp.symf is not None else np.zeros(D), np.int32))
    p.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
    p.act = hold("act", np.arange(n, dtype=np.int32))
    p.nact = n
    r = MultiResult()
    C.memset(C.addressof(r), 0, C.sizeof(r))
    r.struct_version = ABI_VERSION
    r.rscores = hold("out_rscores", np.zeros((M, D), np.float32))
    r.scores = hold("out_scores", np.zeros((M, k), np.float32))
    r.ntim = hold("out_ntim", np.zeros(M, np.float64))
    r.steps = hold("out_steps", np.zeros(M, np.int32))
    if want_ends:
        r.a_ends = hold("out_a_ends", np.zeros((M, D, n, n), np.uint8))
    return Marshalled(p, r, keep)
