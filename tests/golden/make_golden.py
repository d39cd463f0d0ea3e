"""Generate the golden vectors in tests/golden/ from the REFERENCE CPU engine.

    make -C oracle ref && python tests/golden/make_golden.py

The reference engine is cran/cusna's src/libcusna_saom_cpu.cpp compiled from
its own sources into oracle/_ref/libcusna_ref.so (oracle/Makefile). Inputs are
the seeded parity cases of cusna_gb300.workloads.parity_case, regenerated
identically by the tests; each file stores a digest of its inputs so a change
to the generator is detected instead of silently compared.

Output: tests/golden/parity_<kind>_<seed>.npz with every output array of the
reference call (stats, scores, ntim, dist, dist_stat, steps, behaviour and
rate outputs, a_ends).
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


if __name__ == "__main__":
    main()
