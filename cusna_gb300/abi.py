"""ctypes mirror of the libcusna C ABI (include/libcusna.h).

The struct layouts follow the reference header src/libcusna.h:90-208 field for
field; `tests/test_abi.py` checks every offset against a C compiler. This module
also loads the GB300 library (libcusna_gb300.so). There is no CPU fallback: if
the library is missing, `load_library()` raises.
"""
from __future__ import annotations

import atexit
import ctypes as C
import os

import numpy as np

ABI_VERSION = 1
MAXEFF, MAXBEFF, MAXRATE, MAXNET, MAX_N = 24, 6, 4, 4, 8192

STATUS = {0: "CUSNA_OK", 1: "CUSNA_ERR_NULL_ARG", 2: "CUSNA_ERR_SHAPE",
          3: "CUSNA_ERR_NO_CUDA", 4: "CUSNA_ERR_CUDA", 5: "CUSNA_ERR_UNSUPPORTED",
          6: "CUSNA_ERR_INTERNAL"}
OK, ERR_NULL_ARG, ERR_SHAPE, ERR_NO_CUDA, ERR_CUDA, ERR_UNSUPPORTED, ERR_INTERNAL = range(7)

_p = C.c_void_p
_PROBLEM_FIELDS = [
    ("struct_version", C.c_int32),
    ("n", C.c_int32), ("W", C.c_int32), ("k", C.c_int32), ("M", C.c_int32),
    ("threads", C.c_int32),
    ("x0_out", _p), ("x0_in", _p), ("sim_out", _p), ("sim_in", _p),
    ("lam", _p), ("theta", _p),
    ("type_ids", _p), ("etypes", _p), ("wtab", _p), ("p1", _p), ("p2", _p),
    ("vmat", _p), ("vmiss", _p), ("dyc_idx", _p), ("dyc", _p),
    ("int0", _p), ("int1", _p), ("int2", _p), ("dyn_flags", _p),
    ("kdist", _p), ("keep_out", _p), ("keep_in", _p), ("force_out", _p),
    ("force_in", _p), ("perm", _p),
    ("od0", _p), ("id0", _p),
    ("maxdegree", C.c_int32), ("need_mask", C.c_int32), ("conditional", C.c_int32),
    ("target_dist", C.c_int32), ("symflag", C.c_int32),
    ("seed", C.c_uint64),
    ("has_comp", C.c_int32), ("nact", C.c_int32), ("act", _p), ("inactw", _p),
    ("kb", C.c_int32), ("lamb", _p), ("thetab", _p), ("bty", _p), ("z0", _p),
    ("vb", _p), ("bkdist", _p),
    ("zmin", C.c_int32), ("zmax", C.c_int32),
    ("zbar", C.c_float), ("brange", C.c_float), ("bsimmean", C.c_float),
    ("nrate", C.c_int32), ("rkind", _p), ("ralpha", _p), ("ru", _p),
    ("vmat64", _p), ("wtab64", _p), ("vb64", _p), ("p1_64", _p), ("p2_64", _p),
]


class SaomProblem(C.Structure):
    """cusna_saom_problem (src/libcusna.h:90-180)."""
    _fields_ = _PROBLEM_FIELDS


class SaomResult(C.Structure):
    """cusna_saom_result (src/libcusna.h:185-208)."""
    _fields_ = [
        ("struct_version", C.c_int32),
        ("stats", _p), ("ntim", _p), ("scores", _p),
        ("dist", _p), ("dist_stat", _p), ("steps", _p),
        ("bdist", _p), ("bscores", _p), ("z_end", _p),
        ("rscores", _p), ("actor_dist", _p),
        ("want_end_nets", C.c_int32), ("a_ends", _p),
    ]


class MultiProblem(C.Structure):
    """cusna_saom_multi_problem (src/libcusna.h:238-267)."""
    _fields_ = [
        ("struct_version", C.c_int32), ("n", C.c_int32), ("W", C.c_int32), ("k", C.c_int32),
        ("M", C.c_int32), ("D", C.c_int32), ("threads", C.c_int32),
        ("x0_out", _p), ("x0_in", _p), ("lam", _p), ("theta", _p),
        ("type_ids", _p), ("etypes", _p), ("netof", _p), ("netref", _p),
        ("wtab", _p), ("p1", _p), ("p2", _p), ("vmat", _p), ("dyc", _p), ("dyc_idx", _p),
        ("perm", _p), ("symf", _p), ("seed", C.c_uint64), ("act", _p), ("nact", C.c_int32),
    ]


class MultiResult(C.Structure):
    """cusna_saom_multi_result (src/libcusna.h:271-278)."""
    _fields_ = [
        ("struct_version", C.c_int32), ("rscores", _p), ("scores", _p), ("ntim", _p),
        ("steps", _p), ("a_ends", _p),
    ]


class GpuOptions(C.Structure):
    """cusna_gpu_options (extension, include/libcusna.h)."""
    _fields_ = [
        ("struct_version", C.c_int32), ("device_ptrs", C.c_int32),
        ("chain_offset", C.c_uint32), ("warps_per_chain", C.c_int32),
        ("chains_per_cta", C.c_int32), ("launches", C.c_int32),
        ("stream", _p), ("elapsed_ms", C.c_double), ("ministeps", C.c_int64),
        ("specialise", C.c_int32), ("specialised", C.c_int32),
    ]


class ValidationOptions(C.Structure):
    """cusna_validation_options (extension, include/libcusna.h)."""
    _fields_ = [
        ("struct_version", C.c_int32), ("trace_cap", C.c_int32), ("trace", _p),
        ("ustream_steps", C.c_int32), ("ustream", _p), ("lse64", C.c_int32),
        ("warps_per_chain", C.c_int32), ("chains_per_cta", C.c_int32),
    ]


class MomOptions(C.Structure):
    """cusna_mom_options (include/libcusna.h): 0 in a field means its default."""
    _fields_ = [
        ("struct_version", C.c_int32), ("conditional", C.c_int32), ("firstg", C.c_double),
        ("nsub", C.c_int32), ("n2", _p), ("batch2", C.c_int32), ("n1", C.c_int32),
        ("nD", C.c_int32), ("n3", C.c_int32), ("diagonalize", C.c_double), ("seed", C.c_uint64),
        ("rate_consts", _p), ("use_graph", C.c_int32), ("verbose", C.c_int32),
    ]


class MomResult(C.Structure):
    """cusna_mom_result (include/libcusna.h): caller-owned output arrays."""
    _fields_ = [
        ("struct_version", C.c_int32), ("use_start", C.c_int32), ("theta", _p), ("se", _p),
        ("tconv", _p), ("sim_means", _p), ("D", _p), ("msf", _p), ("rate_est", _p),
        ("rate_sd", _p), ("tconv_max", C.c_double),
        ("n_sims", C.c_int64), ("wall_seconds", C.c_double),
        ("phase_seconds", C.c_double * 3),
    ]


def _here() -> str:
    return os.path.dirname(os.path.abspath(__file__))


LIB_PATH = os.path.join(_here(), "_lib", "libcusna_gb300.so")

_lib = None


def load_library(path: str | None = None):
    """Load libcusna_gb300.so and declare its symbols. Raises if it is absent:
    the simulator has no CPU path."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(
            f"libcusna_gb300.so not found at {p}; build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'` (no CPU fallback)")
    lib = C.CDLL(p)
    i32, u32 = C.c_int32, C.c_uint32
    P = C.POINTER
    lib.cusna_saom_simulate_period.argtypes = [P(SaomProblem), P(SaomResult)]
    lib.cusna_saom_simulate_period.restype = i32
    lib.cusna_saom_simulate_period_ex.argtypes = [P(SaomProblem), P(SaomResult), P(GpuOptions)]
    lib.cusna_saom_simulate_period_ex.restype = i32
    lib.cusna_saom_simulate_batch.argtypes = [P(SaomProblem), P(SaomResult), i32, P(GpuOptions)]
    lib.cusna_saom_simulate_batch.restype = i32
    lib.cusna_pack_bits.argtypes = [_p, i32, _p, _p, P(i32)]
    lib.cusna_pack_bits.restype = i32
    lib.cusna_philox4x32.argtypes = [P(u32), P(u32), P(u32)]
    lib.cusna_philox4x32.restype = i32
    lib.cusna_abi_version.restype = i32
    lib.cusna_version_string.restype = C.c_char_p
    lib.cusna_has_cuda.restype = i32
    lib.cusna_last_error.restype = C.c_char_p
    lib.cusna_network_stats_gpu.argtypes = [_p, i32, i32, i32, _p, _p, _p, _p, _p, _p,
                                            _p, _p, _p, _p, i32, _p]
    lib.cusna_network_stats_gpu.restype = i32
    lib.cusna_behavior_stats_gpu.argtypes = [_p, i32, i32, i32, _p, _p, _p,
                                             C.c_double, C.c_double, C.c_double, _p]
    lib.cusna_behavior_stats_gpu.restype = i32
    lib.cusna_saom_simulate_period_validate.argtypes = [P(SaomProblem), P(SaomResult),
                                                        P(ValidationOptions)]
    lib.cusna_saom_simulate_period_validate.restype = i32
    lib.cusna_saom_simulate_period_static.argtypes = [P(SaomProblem), P(SaomResult), _p]
    lib.cusna_saom_simulate_period_static.restype = i32
    lib.cusna_saom_plan_create.argtypes = [P(SaomProblem), P(SaomResult), i32, i32, P(_p)]
    lib.cusna_saom_plan_create.restype = i32
    lib.cusna_saom_plan_launch.argtypes = [_p, _p, i32]
    lib.cusna_saom_plan_launch.restype = i32
    lib.cusna_saom_plan_set_epoch.argtypes = [_p, C.c_uint64]
    lib.cusna_saom_plan_set_epoch.restype = i32
    lib.cusna_saom_plan_shape.argtypes = [_p, P(i32), P(i32), P(i32)]
    lib.cusna_saom_plan_shape.restype = i32
    lib.cusna_saom_plan_destroy.argtypes = [_p]
    lib.cusna_saom_plan_destroy.restype = None
    lib.cusna_mom_estimate.argtypes = [P(SaomProblem), i32, _p, i32, P(MomOptions), P(MomResult)]
    lib.cusna_mom_estimate.restype = i32
    sz, f32 = C.c_size_t, C.c_float
    lib.cusna_mlp_param_count.argtypes = [i32, i32, i32]
    lib.cusna_mlp_param_count.restype = sz
    lib.cusna_mlp_workspace_bytes.argtypes = [i32, i32, i32, i32]
    lib.cusna_mlp_workspace_bytes.restype = sz
    lib.cusna_mlp_init.argtypes = [_p, i32, i32, i32, C.c_uint64, _p]
    lib.cusna_mlp_init.restype = i32
    lib.cusna_mlp_forward.argtypes = [_p, _p, i32, _p, _p, sz, i32, i32, i32, _p]
    lib.cusna_mlp_forward.restype = i32
    lib.cusna_mlp_grad.argtypes = [_p, _p, _p, _p, i32, _p, _p, _p, sz, i32, i32, i32, _p]
    lib.cusna_mlp_grad.restype = i32
    lib.cusna_mlp_train_step.argtypes = [_p, _p, _p, _p, _p, _p, _p, i32, i32, f32, f32, f32,
                                         f32, _p, _p, sz, i32, i32, i32, _p]
    lib.cusna_mlp_train_step.restype = i32
    lib.cusna_mlp_train_steps.argtypes = [_p, _p, _p, _p, _p, _p, _p, i32, i32, _p, _p, _p, sz,
                                          i32, i32, i32, i32, _p]
    lib.cusna_mlp_train_steps.restype = i32
    lib.cusna_mlp_jacobian.argtypes = [_p, _p, i32, i32, _p, _p, _p, sz, i32, i32, i32, _p]
    lib.cusna_mlp_jacobian.restype = i32
    lib.cusna_saom_simulate_multi.argtypes = [P(MultiProblem), P(MultiResult)]
    lib.cusna_saom_simulate_multi.restype = i32
    lib.cusna_cross_stats.argtypes = [_p, _p, i32, i32, i32, C.c_double, _p]
    lib.cusna_cross_stats.restype = i32
    lib.cusna_typed_stats.argtypes = [_p, i32, i32, i32, _p, _p, _p, _p, _p, _p, _p, _p, _p]
    lib.cusna_typed_stats.restype = i32
    lib.cusna_gof_distribution.argtypes = [_p, i32, i32, i32, _p, i32, _p]
    lib.cusna_gof_distribution.restype = i32
    lib.cusna_saom_specialise_check.argtypes = [P(SaomProblem), C.c_char_p, sz, P(C.c_double)]
    lib.cusna_saom_specialise_check.restype = i32
    lib.cusna_saom_specialise_wait.argtypes = [C.c_double, P(i32)]
    lib.cusna_saom_specialise_wait.restype = i32
    lib.cusna_saom_specialise_check_multi.argtypes = [P(MultiProblem), C.c_char_p, sz,
                                                      P(C.c_double)]
    lib.cusna_saom_specialise_check_multi.restype = i32
    lib.cusna_saom_specialise_mode.argtypes = [i32]
    lib.cusna_saom_specialise_mode.restype = i32
    if path is None:
        _lib = lib
        # a specialised period kernel may still be compiling in the library's
        # background thread: let it finish before the interpreter (and the
        # compiler library it uses) is torn down
        atexit.register(lambda: lib.cusna_saom_specialise_wait(600.0, None))
    return lib


# Symbols include/libcusna.h declares; tests check the library exports each one.
EXPORTED_SYMBOLS = [
    "cusna_saom_simulate_period", "cusna_pack_bits", "cusna_philox4x32",
    "cusna_abi_version", "cusna_version_string", "cusna_has_cuda", "cusna_last_error",
    "cusna_saom_simulate_period_ex", "cusna_saom_simulate_batch",
    "cusna_network_stats_gpu", "cusna_behavior_stats_gpu",
    "cusna_saom_simulate_period_static", "cusna_saom_simulate_period_validate",
    "cusna_saom_plan_create", "cusna_saom_plan_launch", "cusna_saom_plan_set_epoch",
    "cusna_saom_plan_shape", "cusna_saom_plan_destroy", "cusna_mom_estimate",
    "cusna_mlp_param_count", "cusna_mlp_workspace_bytes", "cusna_mlp_init", "cusna_mlp_forward",
    "cusna_mlp_grad", "cusna_mlp_train_step", "cusna_mlp_train_steps", "cusna_mlp_jacobian",
    "cusna_saom_simulate_multi", "cusna_cross_stats", "cusna_typed_stats",
    "cusna_gof_distribution", "cusna_saom_specialise_check", "cusna_saom_specialise_wait",
    "cusna_saom_specialise_check_multi", "cusna_saom_specialise_mode",
]

# cusna_adam_hyper: int32 step, float lr, beta1, beta2, eps, c1, c2
ADAM_HYPER = np.dtype([("step", "<i4"), ("lr", "<f4"), ("beta1", "<f4"), ("beta2", "<f4"),
                       ("eps", "<f4"), ("c1", "<f4"), ("c2", "<f4")])


def adam_hyper_bytes(step=0, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8) -> np.ndarray:
    """The bytes of a cusna_adam_hyper block (uint8 array) for a device copy."""
    h = np.zeros(1, dtype=ADAM_HYPER)
    h["step"], h["lr"], h["beta1"], h["beta2"], h["eps"] = step, lr, beta1, beta2, eps
    return h.view(np.uint8).copy()


def ptr(a) -> int | None:
    """Address of a numpy array (None for None)."""
    if a is None:
        return None
    return a.ctypes.data


class CudaError(RuntimeError):
    pass


def check(status: int, what: str, lib=None) -> None:
    if status != OK:
        detail = ""
        if lib is not None:
            try:
                detail = (lib.cusna_last_error() or b"").decode()
            except Exception:  # pragma: no cover - best effort
                detail = ""
        raise CudaError(f"{what} failed: {STATUS.get(status, status)}"
                        + (f" ({detail})" if detail else ""))


def pack_rows(dense: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """Dense n*n 0/1 matrix -> (out rows, in rows), n*W uint32 each, bit (j&31)
    of word (j>>5); the packing of src/cusna_saom_glue.cpp:22-32."""
    d = np.ascontiguousarray(dense != 0)
    n = d.shape[0]
    W = (n + 31) // 32

    def rows(m):
        padded = np.zeros((n, W * 32), dtype=np.uint8)
        padded[:, :n] = m
        by = np.packbits(padded, axis=1, bitorder="little")
        return np.ascontiguousarray(by).view(np.uint32).reshape(n, W).copy()

    return rows(d), rows(d.T)


def unpack_rows(rows: np.ndarray, n: int) -> np.ndarray:
    """Inverse of pack_rows for one set of rows -> dense uint8 n*n."""
    W = (n + 31) // 32
    by = np.ascontiguousarray(rows.reshape(n, W).astype(np.uint32)).view(np.uint8)
    bits = np.unpackbits(by, axis=1, bitorder="little")
    return bits[:, :n].astype(np.uint8)
