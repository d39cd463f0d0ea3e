"""The Method-of-Moments fit through the C ABI (cusna_mom_estimate,
csrc/mom_estimator.cu), driven by a C program as the reference's R glue would
drive it: the program fills one cusna_saom_problem per period of the n=50,
3-wave panel (every array a C literal, floating point as exact hex), the
targets and the options, calls cusna_mom_estimate and prints the estimate.
There is no Python in its process.

CPU: the program links; without a device the call returns CUSNA_ERR_NO_CUDA;
argument errors (NULL, p that does not fit the model, a behaviour period) are
reported before any device work, and the Python wrapper refuses models the
entry point does not fit.
GPU (`-m gpu`): the C program's conditional fit (the reference's defaults,
n3 = 1000, from its default start) reaches the Python estimator's fit of the
same model over the same plans within half a standard error with every
|t-conv| below 0.1; the unconditional fit does the same; and the wrapper's
fit agrees with the C program's.
"""
import os
import subprocess

import numpy as np
import pytest

from cusna_gb300 import abi
from cusna_gb300 import data as D
from cusna_gb300 import effects as E
from cusna_gb300 import mom
from cusna_gb300 import workloads as WL
from tests.conftest import ROOT
from tests.test_c_caller import CTYPE, c_literal, c_scalar, find_array


def c1_estimator(engine, conditional, n3=1000):
    waves = WL.c1_panel(engine)
    effs = [E.make_effect_spec(x) for x in ("density", "recip", "transTrip")]
    ctl = dict(mom.DEFAULT_CONTROL)
    ctl["n3"] = n3
    return mom.mom_estimator(D.build_saom_data(waves), effs, None, None, conditional, ctl,
                             engine=engine)


def c_fit_program(est, p_arg=None, null_periods=False) -> str:
    """Source of a C program that fits est through cusna_mom_estimate."""
    ms = mom.native_problems(est)
    P, p = est.P, est.p
    decls, body = [], []
    for q, m in enumerate(ms):
        for name, ctype in abi.SaomProblem._fields_:
            v = getattr(m.problem, name)
            if ctype is abi.C.c_void_p:
                if not v:
                    continue
                _, a = find_array(m.keep, v)
                vals = ", ".join(c_literal(x, a.dtype) for x in a.reshape(-1)) or "0"
                decls.append(f"static {CTYPE[a.dtype]} p{q}_{name}[{max(a.size, 1)}] = {{{vals}}};")
                body.append(f"  per[{q}].{name} = (void *)p{q}_{name};")
            else:
                body.append(f"  per[{q}].{name} = {c_scalar(v, ctype)};")
    f64 = np.dtype(np.float64)
    decls.append("static double targets[%d] = {%s};"
                 % (p, ", ".join(c_literal(x, f64) for x in est.targets)))
    decls.append("static double rate_consts[%d] = {%s};"
                 % (P, ", ".join(c_literal(x, f64) for x in est.rate_consts)))
    ctl = est.control
    prints = []
    for name, size in (("theta", p), ("se", p), ("tconv", p), ("rate_est", P)):
        prints.append(f'  printf("out {name}"); for (int j = 0; j < {size}; ++j) '
                      f'printf(" %a", {name}[j]); printf("\\n");')
    return "\n".join([
        "#include <stdint.h>", "#include <stdio.h>", "#include <string.h>",
        '#include "libcusna.h"', *decls,
        "int main(void) {",
        f"  cusna_saom_problem per[{P}];",
        "  memset(per, 0, sizeof per);",
        *body,
        "  cusna_mom_options o;",
        "  memset(&o, 0, sizeof o);",
        "  o.struct_version = CUSNA_ABI_VERSION;",
        f"  o.conditional = {int(est.conditional)};",
        f"  o.n3 = {int(ctl['n3'])};",
        f"  o.seed = {int(ctl['seed'])}ULL;",
        "  o.rate_consts = rate_consts;",
        f"  double theta[{p}], se[{p}], tconv[{p}], rate_est[{P}];",
        "  cusna_mom_result r;",
        "  memset(&r, 0, sizeof r);",
        "  r.struct_version = CUSNA_ABI_VERSION;",
        "  r.theta = theta; r.se = se; r.tconv = tconv; r.rate_est = rate_est;",
        '  printf("null %d\\n", (int)cusna_mom_estimate(NULL, 0, NULL, 0, &o, &r));',
        f"  const int st = (int)cusna_mom_estimate({'NULL' if null_periods else 'per'}, {P}, "
        f"targets, {p if p_arg is None else p_arg}, &o, &r);",
        '  printf("status %d\\n", st);',
        '  if (st != 0) { printf("error %s\\n", cusna_last_error()); return 0; }',
        *prints,
        '  printf("tconv_max %a\\n", r.tconv_max);',
        '  printf("n_sims %lld\\n", (long long)r.n_sims);',
        '  printf("wall %a\\n", r.wall_seconds);',
        "  return 0;", "}", ""])


def run_program(src_text, tmp_path, name="fit") -> dict:
    src = tmp_path / f"{name}.c"
    exe = tmp_path / name
    src.write_text(src_text)
    libdir = os.path.dirname(abi.LIB_PATH)
    subprocess.check_call(["gcc", "-std=c11", "-O1", "-I" + os.path.join(ROOT, "include"),
                           str(src), "-L" + libdir, "-lcusna_gb300", "-Wl,-rpath," + libdir,
                           "-lm", "-o", str(exe)])
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=900, check=True).stdout
    res = {}
    for line in out.splitlines():
        head, _, rest = line.partition(" ")
        if head == "out":
            key, _, vals = rest.partition(" ")
            res[key] = np.array([float.fromhex(v) for v in vals.split()])
        elif head == "error":
            res["error"] = rest
        else:
            res[head] = rest.split()
    return res


def test_c_program_links_and_reports_argument_errors(built_lib, port, tmp_path):
    est = c1_estimator(port, conditional=True)
    res = run_program(c_fit_program(est), tmp_path)
    assert res["null"] == [str(abi.ERR_NULL_ARG)]
    if res.get("status") == [str(abi.ERR_NO_CUDA)]:
        assert "no CUDA device" in res["error"]
    else:
        assert res["status"] == ["0"]
    # p must be the model's parameter count (k conditional, P + k otherwise)
    res = run_program(c_fit_program(est, p_arg=est.p + 1), tmp_path, "bad_p")
    assert res["status"] == [str(abi.ERR_SHAPE)] and "parameters" in res["error"]
    res = run_program(c_fit_program(est, null_periods=True), tmp_path, "null_periods")
    assert res["status"] == [str(abi.ERR_NULL_ARG)]


def test_wrapper_refuses_models_with_behaviour(c1_est_port_uncond):
    est = c1_est_port_uncond
    beh = mom.Estimator(**{**est.__dict__, "coevol": True, "kb": 1})
    with pytest.raises(ValueError, match="network effects only"):
        mom.native_problems(beh)


@pytest.fixture(scope="module")
def c1_est_port_uncond(port):
    return c1_estimator(port, conditional=False)


def test_behaviour_period_is_unsupported_before_device_work(built_lib, c1_est_port_uncond):
    """A period with behaviour effects: CUSNA_ERR_UNSUPPORTED whether or not a
    device is present (arguments are checked first)."""
    import ctypes as C
    est = c1_est_port_uncond
    ms = mom.native_problems(est)
    probs = (abi.SaomProblem * est.P)(*[m.problem for m in ms])
    probs[1].kb = 1
    lib = abi.load_library()
    tg = np.ascontiguousarray(est.targets)
    th = np.zeros(est.p)
    o = abi.MomOptions(struct_version=abi.ABI_VERSION)
    r = abi.MomResult(struct_version=abi.ABI_VERSION, theta=th.ctypes.data)
    st = lib.cusna_mom_estimate(probs, est.P, tg.ctypes.data, est.p, C.byref(o), C.byref(r))
    assert st == abi.ERR_UNSUPPORTED and b"period 1" in lib.cusna_last_error()
    o.struct_version = 7
    st = lib.cusna_mom_estimate(probs, est.P, tg.ctypes.data, est.p, C.byref(o), C.byref(r))
    assert st == abi.ERR_SHAPE


# ---- GPU ---------------------------------------------------------------------
def python_fit(est):
    eng = mom.PlanEngine(use_graph=True)
    try:
        return mom.mom_run(est, engine=eng)
    finally:
        eng.close()


@pytest.mark.gpu
@pytest.mark.parametrize("conditional", [True, False])
def test_gpu_c_program_fit_matches_the_python_estimator(gpu_lib, tmp_path, conditional):
    est = c1_estimator(mom.GpuEngine(), conditional=conditional)
    res = run_program(c_fit_program(est), tmp_path)
    assert res["status"] == ["0"], res.get("error")
    fit = python_fit(est)
    assert np.all(np.isfinite(res["theta"])) and np.all(res["se"] > 0)
    assert np.abs(res["tconv"]).max() < 0.1, res["tconv"]
    assert np.abs(fit.tconv).max() < 0.1, fit.tconv
    diff = np.abs(res["theta"] - fit.theta) / fit.se
    assert diff.max() < 0.5, (res["theta"], fit.theta, fit.se)
    np.testing.assert_allclose(res["se"], fit.se, rtol=0.25)
    ctl = est.control
    n_sims = ctl["n1"] + ctl["n3"] + sum(ctl["nD"] + n * ctl["batch2"] for n in ctl["n2"])
    assert res["n_sims"] == [str(int(n_sims))]
    if conditional:
        np.testing.assert_allclose(res["rate_est"], fit.rate_est, rtol=0.1)


@pytest.mark.gpu
def test_gpu_native_wrapper_fit_matches_the_c_program(gpu_lib, tmp_path):
    """mom_run_native (ctypes over the same entry point, same seed) gives the
    C program's estimate bit for bit: the fit is a function of its inputs."""
    est = c1_estimator(mom.GpuEngine(), conditional=True)
    res = run_program(c_fit_program(est), tmp_path)
    fit = mom.mom_run_native(est)
    np.testing.assert_array_equal(fit.theta, res["theta"])
    np.testing.assert_array_equal(fit.se, res["se"])
    assert fit.wall_time > 0 and set(fit.phase_times) == {"phase1", "phase2", "phase3"}
