"""Build libcusna_gb300.so in-tree with nvcc for sm_103a.

    python -m cusna_gb300.build          # or __graft_entry__.build()

Each .cu file under csrc/ compiles in parallel into an object; one link step
makes cusna_gb300/_lib/libcusna_gb300.so. -fmad=false keeps every float64
multiply and add separately rounded, as the reference CPU engine's arithmetic is
(explicit fma() calls are still fused where the code asks for them).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libcusna_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-ffp-contract=off",
              "-Xcompiler", "-fvisibility=hidden", "-DLIBCUSNA_BUILD",
              "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found")
    return path


# device headers the run-time specialisation (csrc/saom_jit.cu) compiles with
# NVRTC; they are embedded into the library as strings
JIT_HEADERS = ["saom_common.cuh", "saom_kernel.cuh", "saom_stats.cuh", "saom_chain.cuh",
               "saom_period.cuh", "saom_multi_kernel.cuh"]


def write_jit_sources(build_dir: str) -> None:
    """Write build_dir/jit_sources.inc: the JIT headers as raw string literals
    (rewritten only when their text changes)."""
    delim = "cusnajit"
    parts = ["// generated by cusna_gb300/build.py from csrc/: do not edit\n"]
    for name in JIT_HEADERS:
        text = open(os.path.join(CSRC, name)).read()
        if ")" + delim + '"' in text:
            raise RuntimeError(f"{name} contains the raw-string delimiter")
        parts.append(f'static const char kJitSrc_{name.replace(".", "_")}[] = R"{delim}(' + text +
                     f')' + delim + '";\n')
    parts.append("static const int kJitHeaderCount = %d;\n" % len(JIT_HEADERS))
    parts.append("static const char *const kJitHeaderNames[] = {" +
                 ", ".join(f'"{n}"' for n in JIT_HEADERS) + "};\n")
    parts.append("static const char *const kJitHeaderSources[] = {" +
                 ", ".join(f'kJitSrc_{n.replace(".", "_")}' for n in JIT_HEADERS) + "};\n")
    text = "".join(parts)
    path = os.path.join(build_dir, "jit_sources.inc")
    if not os.path.exists(path) or open(path).read() != text:
        with open(path, "w") as f:
            f.write(text)


def sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, ptxas_info: bool = False, force: bool = False,
          out: str | None = None, extra_flags: list[str] | None = None) -> str:
    """Compile and link; `out`/`extra_flags` build a variant elsewhere (e.g. a
    different register budget) without touching the in-tree library."""
    lib_path = out or LIB
    build_dir = BUILD_DIR if out is None else os.path.join(os.path.dirname(out), "_build_" +
                                                           os.path.basename(out).replace(".so", ""))
    os.makedirs(os.path.dirname(lib_path), exist_ok=True)
    os.makedirs(build_dir, exist_ok=True)
    extra = list(extra_flags or []) + ["-I" + build_dir]
    write_jit_sources(build_dir)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(ROOT, "include", "libcusna.h"))
    srcs = sources()
    objs = []
    jobs = []
    for s in srcs:
        o = os.path.join(build_dir, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        if force or ptxas_info or _stale(o, [s] + headers):
            cmd = [nvcc()] + ARCH + NVCC_FLAGS + extra + ["-c", s, "-o", o]
            if ptxas_info:
                cmd += ["-Xptxas", "-v"]
            jobs.append(cmd)
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
            results = list(ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs))
        for cmd, r in zip(jobs, results):
            if verbose or ptxas_info or r.returncode != 0:
                sys.stderr.write(r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError("nvcc failed: " + " ".join(cmd))
    if force or jobs or _stale(lib_path, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", lib_path] + objs + ["-lcudart", "-ldl"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
    return lib_path


if __name__ == "__main__":
    print(build(verbose=True, ptxas_info="-v" in sys.argv, force="-f" in sys.argv))
