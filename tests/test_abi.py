"""The C ABI boundary: struct layouts (ctypes mirror vs include/libcusna.h vs
the reference header src/libcusna.h), the exported symbol set, and the
status codes returned before any device work (NULL, shape, version)."""
import ctypes as C
import os
import subprocess
import tempfile

import numpy as np
import pytest

from cusna_gb300 import abi
from cusna_gb300 import workloads as WL
from cusna_gb300.glue import marshal_period
from tests.conftest import REFERENCE, ROOT

STRUCTS = [("cusna_saom_problem", abi.SaomProblem), ("cusna_saom_result", abi.SaomResult),
           ("cusna_saom_multi_problem", abi.MultiProblem),
           ("cusna_saom_multi_result", abi.MultiResult)]


def c_offsets(include_dir: str) -> dict:
    """sizeof/offsetof of every ABI struct as a C compiler lays them out."""
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "libcusna.h"', "int main(void){"]
    for cname, cls in STRUCTS:
        lines.append(f'printf("{cname}.size %zu\\n", sizeof({cname}));')
        for f, _ in cls._fields_:
            lines.append(f'printf("{cname}.{f} %zu\\n", offsetof({cname}, {f}));')
    lines.append("return 0;}")
    with tempfile.TemporaryDirectory() as td:
        src = os.path.join(td, "off.c")
        exe = os.path.join(td, "off")
        open(src, "w").write("\n".join(lines))
        subprocess.check_call(["gcc", "-I" + include_dir, src, "-o", exe])
        out = subprocess.check_output([exe], text=True)
    return {k: int(v) for k, v in (ln.split() for ln in out.strip().splitlines())}


def ctypes_offsets() -> dict:
    d = {}
    for cname, cls in STRUCTS:
        d[cname + ".size"] = C.sizeof(cls)
        for f, _ in cls._fields_:
            d[f"{cname}.{f}"] = getattr(cls, f).offset
    return d


def test_ctypes_mirror_matches_header():
    assert c_offsets(os.path.join(ROOT, "include")) == ctypes_offsets()


def test_header_layout_matches_reference_header():
    ref_inc = os.path.join(REFERENCE, "src")
    if not os.path.exists(os.path.join(ref_inc, "libcusna.h")):
        pytest.skip("reference header not present")
    assert c_offsets(ref_inc) == c_offsets(os.path.join(ROOT, "include"))


def test_library_exports_every_declared_symbol(built_lib):
    import re
    header = open(os.path.join(ROOT, "include", "libcusna.h")).read()
    code = re.sub(r"/\*.*?\*/", "", header, flags=re.S)
    declared = set(re.findall(r"CUSNA_API[^;(]*?\b(cusna_\w+)\s*\(", code))
    assert declared == set(abi.EXPORTED_SYMBOLS)
    for name in abi.EXPORTED_SYMBOLS:
        assert hasattr(built_lib, name), name
    assert built_lib.cusna_abi_version() == 1
    assert b"sm_103a" in built_lib.cusna_version_string()


def test_philox_and_pack_bits_utilities(built_lib):
    ctr = (C.c_uint32 * 4)(0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344)
    key = (C.c_uint32 * 2)(0xA4093822, 0x299F31D0)
    out = (C.c_uint32 * 4)()
    assert built_lib.cusna_philox4x32(ctr, key, out) == abi.OK
    assert tuple(out) == (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)
    r = np.random.Generator(np.random.PCG64(0))
    for n in (1, 31, 32, 33, 70):
        a = (r.random((n, n)) < 0.3).astype(np.uint8)
        W = (n + 31) // 32
        o = np.zeros(n * W, np.uint32)
        i = np.zeros(n * W, np.uint32)
        w = C.c_int32()
        assert built_lib.cusna_pack_bits(a.ctypes.data, n, o.ctypes.data, i.ctypes.data,
                                         C.byref(w)) == abi.OK
        ro, ri = abi.pack_rows(a)
        assert w.value == W
        np.testing.assert_array_equal(o.reshape(n, W), ro)
        np.testing.assert_array_equal(i.reshape(n, W), ri)
        np.testing.assert_array_equal(abi.unpack_rows(ro, n), a)
    assert built_lib.cusna_pack_bits(None, 3, None, None, None) == abi.ERR_NULL_ARG


def test_status_codes_before_device_work(built_lib):
    lib = built_lib
    assert lib.cusna_saom_simulate_period(None, None) == abi.ERR_NULL_ARG
    c = WL.parity_case("baseline", seed=1)
    m = marshal_period(c["inp"], c["M"], c["seed"], c["lam"], c["theta"])
    P, R = C.byref(m.problem), C.byref(m.result)
    m.problem.struct_version = 7
    assert lib.cusna_saom_simulate_period(P, R) == abi.ERR_SHAPE
    m.problem.struct_version = 1
    for field, bad in (("n", 0), ("n", 8193), ("W", 9), ("k", 0), ("M", 0), ("k", 25)):
        old = getattr(m.problem, field)
        setattr(m.problem, field, bad)
        assert lib.cusna_saom_simulate_period(P, R) == abi.ERR_SHAPE, (field, bad)
        setattr(m.problem, field, old)
    old = m.problem.type_ids
    m.problem.type_ids = None
    assert lib.cusna_saom_simulate_period(P, R) == abi.ERR_NULL_ARG
    m.problem.type_ids = old
    if lib.cusna_has_cuda() == 0:
        assert lib.cusna_saom_simulate_period(P, R) == abi.ERR_NO_CUDA
        assert b"no CUDA device" in lib.cusna_last_error()


def test_interaction_components_are_validated(built_lib):
    c = WL.parity_case("interaction", seed=0)
    m = marshal_period(c["inp"], c["M"], c["seed"], c["lam"], c["theta"])
    bad = np.array(m.keep["int1"])
    bad[4] = 5   # component not earlier than the interaction itself
    m.keep["int1_bad"] = bad
    m.problem.int1 = bad.ctypes.data
    assert built_lib.cusna_saom_simulate_period(C.byref(m.problem), C.byref(m.result)) == abi.ERR_SHAPE


def test_product_has_no_cpu_fallback():
    """The package never imports the oracle, and the library refuses to load
    from a missing path instead of falling back to anything."""
    pkg = os.path.join(ROOT, "cusna_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith(".py"):
                src = open(os.path.join(dirpath, f)).read()
                assert "import oracle" not in src and "from oracle" not in src, f
    with pytest.raises(RuntimeError):
        abi.load_library("/nonexistent/libcusna_gb300.so")
