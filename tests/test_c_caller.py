"""A C caller of the boundary, as the reference's cpp11 glue is one
(src/cusna_saom_glue.cpp:57-189): a C program compiled against
include/libcusna.h and linked with -lcusna_gb300, with no Python in the
process, fills cusna_saom_problem / cusna_saom_result from arrays, calls
cusna_saom_simulate_period and prints every output exactly (hex floats).

The program is generated from a marshalled problem: every input array becomes
a C array literal (floating point as exact hex literals) and every scalar an
assignment, so the C call sees the bytes the ctypes call sees.

CPU: the program links, the utilities answer as documented, and the simulator
returns the status a host without a device gets. GPU (`-m gpu`): its outputs
equal the ctypes call's bit for bit and the CPU oracle's to the parity bar.
"""
import ctypes as C
import math
import os
import subprocess

import numpy as np
import pytest

from cusna_gb300 import abi
from cusna_gb300 import workloads as WL
from cusna_gb300.glue import marshal_period
from tests.conftest import ROOT

CTYPE = {np.dtype(np.int8): "int8_t", np.dtype(np.uint8): "uint8_t",
         np.dtype(np.int16): "int16_t", np.dtype(np.uint16): "uint16_t",
         np.dtype(np.int32): "int32_t", np.dtype(np.uint32): "uint32_t",
         np.dtype(np.int64): "int64_t", np.dtype(np.uint64): "uint64_t",
         np.dtype(np.float32): "float", np.dtype(np.float64): "double"}


def c_literal(v, dt: np.dtype) -> str:
    if dt.kind == "f":
        x = float(v)
        if math.isnan(x):
            return "NAN"
        if math.isinf(x):
            return "INFINITY" if x > 0 else "-INFINITY"
        return x.hex() + ("f" if dt == np.float32 else "")
    x = int(v)
    if dt.kind == "u":
        return f"{x}ULL" if dt.itemsize == 8 else f"{x}U"
    if x == -(2 ** (8 * dt.itemsize - 1)):
        return f"({x + 1}LL-1)"
    return f"{x}LL" if dt.itemsize == 8 else str(x)


def c_scalar(v, ctype) -> str:
    if ctype in (C.c_float, C.c_double):
        return c_literal(v, np.dtype(np.float32 if ctype is C.c_float else np.float64))
    if ctype is C.c_uint64:
        return f"{int(v)}ULL"
    return str(int(v))


def find_array(keep: dict, addr: int):
    for name, a in keep.items():
        if isinstance(a, np.ndarray) and a.ctypes.data == addr:
            return name, np.ascontiguousarray(a)
    raise KeyError(f"no kept array at {addr:#x}")


def c_program(m) -> str:
    """Source of a C program that makes m's call through the C ABI."""
    decls, body, prints = [], [], []
    for name, ctype in abi.SaomProblem._fields_:
        v = getattr(m.problem, name)
        if ctype is abi.C.c_void_p:
            if not v:
                continue
            _, a = find_array(m.keep, v)
            vals = ", ".join(c_literal(x, a.dtype) for x in a.reshape(-1)) or "0"
            decls.append(f"static {CTYPE[a.dtype]} in_{name}[{max(a.size, 1)}] = {{{vals}}};")
            body.append(f"  p.{name} = (void *)in_{name};")
        else:
            body.append(f"  p.{name} = {c_scalar(v, ctype)};")
    outs = []
    for name, ctype in abi.SaomResult._fields_:
        v = getattr(m.result, name)
        if ctype is abi.C.c_void_p:
            if not v:
                continue
            _, a = find_array(m.keep, v)
            decls.append(f"static {CTYPE[a.dtype]} out_{name}[{max(a.size, 1)}];")
            body.append(f"  r.{name} = (void *)out_{name};")
            outs.append((name, a))
        else:
            body.append(f"  r.{name} = {c_scalar(v, ctype)};")
    for name, a in outs:
        fmt, cast = ("%a", "(double)") if a.dtype.kind == "f" else ("%lld", "(long long)")
        prints.append(f'  printf("out {name}"); for (size_t q = 0; q < {a.size}; ++q) '
                      f'printf(" {fmt}", {cast}out_{name}[q]); printf("\\n");')
    return "\n".join([
        "#include <math.h>", "#include <stdint.h>", "#include <stdio.h>", "#include <string.h>",
        '#include "libcusna.h"', *decls,
        "int main(void) {",
        '  printf("abi %d\\n", (int)cusna_abi_version());',
        '  printf("has_cuda %d\\n", (int)cusna_has_cuda());',
        "  uint32_t ctr[4] = {0x243F6A88u, 0x85A308D3u, 0x13198A2Eu, 0x03707344u};",
        "  uint32_t key[2] = {0xA4093822u, 0x299F31D0u}, ph[4];",
        "  const int ps = (int)cusna_philox4x32(ctr, key, ph);",
        '  printf("philox %d %08x %08x %08x %08x\\n", ps, ph[0], ph[1], ph[2], ph[3]);',
        '  printf("null %d\\n", (int)cusna_saom_simulate_period(NULL, NULL));',
        "  cusna_saom_problem p; cusna_saom_result r;",
        "  memset(&p, 0, sizeof p); memset(&r, 0, sizeof r);",
        *body,
        "  const int st = (int)cusna_saom_simulate_period(&p, &r);",
        '  printf("status %d\\n", st);',
        '  if (st != 0) { printf("error %s\\n", cusna_last_error()); return 0; }',
        *prints,
        "  return 0;", "}", ""])


def run_c_caller(m, tmp_path) -> dict:
    src = tmp_path / "caller.c"
    exe = tmp_path / "caller"
    src.write_text(c_program(m))
    libdir = os.path.dirname(abi.LIB_PATH)
    subprocess.check_call(["gcc", "-std=c11", "-O1", "-I" + os.path.join(ROOT, "include"),
                           str(src), "-L" + libdir, "-lcusna_gb300", "-Wl,-rpath," + libdir,
                           "-lm", "-o", str(exe)])
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300, check=True).stdout
    res = {"outputs": {}}
    for line in out.splitlines():
        head, _, rest = line.partition(" ")
        if head == "out":
            name, _, vals = rest.partition(" ")
            res["outputs"][name] = vals.split()
        elif head == "error":
            res["error"] = rest
        else:
            res[head] = rest.split()
    return res


def small_problem():
    c = WL.parity_case("covariate", seed=4, n=37, M=3)
    return marshal_period(c["inp"], c["M"], c["seed"], c["lam"], c["theta"], lamb=c["lamb"],
                          thetab=c["thetab"])


def test_c_caller_links_and_calls_the_library(built_lib, tmp_path):
    res = run_c_caller(small_problem(), tmp_path)
    assert res["abi"] == ["1"]
    assert res["philox"] == ["0", "d16cfe09", "94fdcceb", "5001e420", "24126ea1"]
    assert res["null"] == [str(abi.ERR_NULL_ARG)]
    if res["has_cuda"] == ["0"]:
        assert res["status"] == [str(abi.ERR_NO_CUDA)]
        assert "no CUDA device" in res["error"]
    else:
        assert res["status"] == ["0"]


@pytest.mark.gpu
def test_gpu_c_caller_matches_ctypes_and_oracle(gpu_lib, port, tmp_path):
    from cusna_gb300 import sim
    from tests.test_gpu_parity import assert_parity
    m = small_problem()
    res = run_c_caller(m, tmp_path)
    assert res["status"] == ["0"], res.get("error")
    via_ctypes = sim.simulate(small_problem())
    got = {}
    for name, vals in res["outputs"].items():
        ref = via_ctypes[name]
        if ref.dtype.kind == "f":
            a = np.array([float.fromhex(v) for v in vals], dtype=ref.dtype)
        else:
            a = np.array([int(v) for v in vals], dtype=ref.dtype)
        got[name] = a.reshape(ref.shape)
        np.testing.assert_array_equal(got[name], ref, err_msg=name)   # bit for bit
    assert_parity(got, port.simulate(small_problem()), "c caller")
