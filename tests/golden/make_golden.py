"""Generate the golden vectors in tests/golden/ from the REFERENCE CPU engine.

    make -C oracle ref && python tests/golden/make_golden.py

The reference engine is cran/cusna's src/libcusna_saom_cpu.cpp compiled from
its own sources into oracle/_ref/libcusna_ref.so (oracle/Makefile). Inputs are
the seeded parity cases of cusna_gb300.workloads.parity_case, regenerated
identically by the tests; each file stores a digest of its inputs so a change
to the generator is detected instead of silently compared.

Output: tests/golden/parity_<kind>_<seed>.npz with every output array of the
reference call (stats, scores, ntim, dist, dist_stat, steps, behaviour and
rate outputs, a_ends); tests/golden/multi_<kind>_<seed>.npz, the same for the
multi-network simulator (cusna_saom_simulate_multi_cpu) on the seeded cases of
cusna_gb300.workloads.multi_case; tests/golden/cross_stats.npz, the reference's
cusna_cross_stats on seeded networks; tests/golden/gof_typed.npz, its
cusna_gof_distribution and cusna_typed_stats on seeded networks.
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from cusna_gb300 import workloads as WL  # noqa: E402
from cusna_gb300.glue import marshal_period  # noqa: E402

SEEDS = (0, 1)


def case_digest(c) -> str:
    """Digest of a parity case's inputs (arrays and scalars)."""
    h = hashlib.sha256()
    inp = c["inp"]
    for name in sorted(vars(inp)):
        v = getattr(inp, name)
        h.update(name.encode())
        if v is None:
            h.update(b"none")
        else:
            h.update(np.ascontiguousarray(np.asarray(v, dtype=np.float64)).tobytes())
    for key in ("M", "seed", "lam", "lamb"):
        h.update(repr(c[key]).encode())
    for key in ("theta", "thetab"):
        h.update(b"none" if c[key] is None else np.asarray(c[key], dtype=np.float64).tobytes())
    return h.hexdigest()


def run_case(engine, c) -> dict:
    m = marshal_period(c["inp"], c["M"], c["seed"], c["lam"], c["theta"], lamb=c["lamb"],
                       thetab=c["thetab"], want_ends=True)
    return engine.simulate(m)


def multi_digest(case) -> str:
    """Digest of a multi-network case's inputs (MultiInputs, seed, lam, theta)."""
    inp, seed, lam, theta = case
    h = hashlib.sha256()
    for name in sorted(vars(inp)):
        v = getattr(inp, name)
        h.update(name.encode())
        if v is None:
            h.update(b"none")
        else:
            h.update(np.ascontiguousarray(np.asarray(v, dtype=np.float64)).tobytes())
    h.update(repr(seed).encode())
    for v in (lam, theta):
        h.update(np.asarray(v, dtype=np.float64).tobytes())
    return h.hexdigest()


MULTI_M = 4


def run_multi(engine, case) -> dict:
    """One multi-network period on an engine with simulate_multi (the oracle's
    two CPU engines or the GPU adapter of the tests)."""
    from cusna_gb300.glue import marshal_multi
    inp, seed, lam, theta = case
    return engine.simulate_multi(marshal_multi(inp, MULTI_M, seed, lam, theta))


def cross_case(seed: int, n: int = 37, M: int = 3):
    """Own networks (M, n, n) and a source predictor (n, n) for the cross
    statistics."""
    r = np.random.Generator(np.random.PCG64(500 + seed))
    a = (r.random((M, n, n)) < 0.12).astype(np.uint8)
    w = (r.random((n, n)) < 0.15).astype(np.uint8)
    for x in list(a) + [w]:
        np.fill_diagonal(x, 0)
    return a, w


CROSS_TYPES = ((33, 0.0), (34, 0.0), (35, 0.0), (36, 1.0), (36, 2.0), (37, 0.0))


def gof_case(seed: int, n: int, M: int = 3, p: float = 0.08):
    """End networks (M, n, n) with a few self-ties, the start network x0, a
    per-pair effect matrix F with a zero diagonal and six masks, for the typed
    statistics and the GoF distributions."""
    r = np.random.Generator(np.random.PCG64(900 + seed))
    a = (r.random((M, n, n)) < p).astype(np.uint8)
    for x in a:
        x[np.arange(n), np.arange(n)] = r.random(n) < 0.05
    x0 = (r.random((n, n)) < p).astype(np.uint8)
    np.fill_diagonal(x0, 0)
    F = np.round(r.standard_normal((n, n)), 4)
    np.fill_diagonal(F, 0.0)
    masks = {nm: (r.random((n, n)) < q).astype(np.uint8)
             for nm, q in (("keep", 0.9), ("force", 0.05), ("keepS", 0.95), ("forceS", 0.03),
                           ("miss_m", 0.05), ("miss_m1", 0.05))}
    return a, x0, F, masks


GOF_SIZES = (1, 2, 31, 33, 65)
GOF_LEVELS = {0: [0, 1, 2, 3, 5, 8], 1: [0, 1, 2, 4, 6], 2: [1, 2, 3, 4, 6, 100]}


def main() -> None:
    from oracle import Oracle, reference_available
    if not reference_available():
        raise SystemExit("oracle/_ref/libcusna_ref.so missing: run `make -C oracle ref`")
    ref = Oracle("reference")
    for kind in WL.PARITY_KINDS:
        for seed in SEEDS:
            c = WL.parity_case(kind, seed=seed)
            out = run_case(ref, c)
            path = os.path.join(HERE, f"parity_{kind}_{seed}.npz")
            np.savez_compressed(path, digest=np.array(case_digest(c)), **out)
            print(path, os.path.getsize(path))
    for kind in WL.MULTI_KINDS:
        for seed in SEEDS:
            case = WL.multi_case(kind, seed=seed, M=MULTI_M)
            out = run_multi(ref, case)
            path = os.path.join(HERE, f"multi_{kind}_{seed}.npz")
            np.savez_compressed(path, digest=np.array(multi_digest(case)), **out)
            print(path, os.path.getsize(path))
    cross = {}
    for seed in SEEDS:
        a, w = cross_case(seed)
        for t, parm in CROSS_TYPES:
            cross[f"s{seed}_t{t}_p{int(parm)}"] = ref.cross_stats(a, w, t, parm)
    path = os.path.join(HERE, "cross_stats.npz")
    np.savez_compressed(path, **cross)
    print(path, os.path.getsize(path))
    gof = {}
    for seed, n in enumerate(GOF_SIZES):
        a, x0, F, masks = gof_case(seed, n)
        for kind, lv in GOF_LEVELS.items():
            gof[f"n{n}_gof{kind}"] = ref.gof_distribution(a, kind, lv)
        for et in (1, 2):
            gof[f"n{n}_typed{et}"] = ref.typed_stats(a, et, F, x0, **masks)
            gof[f"n{n}_typed{et}_nomask"] = ref.typed_stats(a, et, F, x0)
    path = os.path.join(HERE, "gof_typed.npz")
    np.savez_compressed(path, **gof)
    print(path, os.path.getsize(path))


if __name__ == "__main__":
    main()
