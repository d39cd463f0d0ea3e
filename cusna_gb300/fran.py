"""A FRAN backend: one chain per call for an external Robbins-Monro driver.

A Python restatement of the reference's `cusna_fran()` (R/fran.R:26-80), the
closure RSiena's `siena07()` calls once per Robbins-Monro iteration: it builds
the estimator context once, and each call simulates ONE chain of every period
at the caller's theta and returns the per-period statistics (`fra`), scores
(`sc`) and elapsed times (`ntim0`) in the simstats0c layout (periods x
parameters).

One chain per call is latency-bound on a GPU. The backend therefore runs the
periods as a replayable plan replayed from a CUDA graph (`mom.PlanEngine`):
the problems stay on the device, a call writes theta into the plan's
parameter rows, replays the graph and copies back the moment outputs. Period
seeds are drawn once from the closure's generator; call r uses Philox keys
seed + r, so a run is reproducible for a given `seed`.
"""
from __future__ import annotations

import numpy as np

from . import data as D
from . import effects as E
from . import mom

COVARIATE_EFFECTS = ("egoX", "altX", "simX", "sameX", "higher", "egoXaltX", "egoPlusAltX",
                     "altRThresholdX")   # R/fran.R:29-30


def cusna_fran(waves, effect_names, covariate=None, conditional=True, seed=0, engine=None):
    """The FRAN closure (R/fran.R:26-80). effect_names are in the order of the
    caller's theta after the basic rates; covariate is shared by the covariate
    effects. Returns fran(z) -> dict(fra, sc, ntim0, OK, feasible) with z a
    mapping holding "theta" (and optionally "cconditional"); fran.counter
    counts the calls."""
    data = D.saom_data(waves)
    effects = [E.cusna_effect(nm, covariate=covariate if nm in COVARIATE_EFFECTS else None)
               for nm in effect_names]
    conditional = bool(conditional)
    engine = engine or mom.PlanEngine(use_graph=True)
    est = mom.mom_estimator(data.internal, E.build_specs(effects), None, None, conditional,
                            dict(mom.DEFAULT_CONTROL), engine=engine)
    rng = np.random.Generator(np.random.PCG64(int(seed)))

    def fran(z, x=None):
        theta = np.asarray(z["theta"], dtype=np.float64).ravel()
        cc = z.get("cconditional") if hasattr(z, "get") else None
        if cc is not None and bool(cc) != conditional:
            raise ValueError(f"cusna_fran(conditional = {conditional}) does not match the "
                             f"algorithm (cond = {bool(cc)}).")
        if theta.shape[0] != est.p:
            raise ValueError(f"siena07() passed {theta.shape[0]} parameters, but the cusna model "
                             f"has {est.p} ({', '.join(est.param_names)}); check `effect_names` "
                             "against the RSiena effects object.")
        fran.counter += 1
        s = mom.mom_simulate(est, theta, 1, rng, engine)
        fra = np.stack([sp[0] for sp, _ in s.pieces])
        sc = np.stack([scp[0] for _, scp in s.pieces])
        return {"fra": fra, "sc": sc, "ntim0": s.ntim[0].copy(), "OK": True, "feasible": True}

    fran.counter = 0
    fran.estimator = est
    fran.engine = engine
    return fran
