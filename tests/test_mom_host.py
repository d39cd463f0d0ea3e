"""The C++ host algebra of the C-ABI estimator (csrc/mom_host.h, used by
cusna_mom_estimate) against the Python estimator's (cusna_gb300.mom), on the CPU.

A small C++ program includes the header alone (it has no CUDA), reads matrices
and vectors from standard input and prints its results. The checks: inverses
of well-conditioned matrices, the pseudo-inverse of singular ones (R's
.safe_solve falls back to it, R/mom.R:15-22), the score-function derivative
summed over periods (:173-182), the diagonalised inverse (:184-187), and the
guarded step with its rate floor (:189-197).
"""
import os
import subprocess
from types import SimpleNamespace

import numpy as np
import pytest

from cusna_gb300 import mom
from tests.conftest import ROOT

DRIVER = r"""
#include <cstdio>
#include <string>
#include <vector>
#include "mom_host.h"
using namespace cusna;
static std::vector<double> rd(int n) {
  std::vector<double> v(n);
  for (int i = 0; i < n; ++i) if (std::scanf("%lf", &v[i]) != 1) v[i] = 0.0;
  return v;
}
static void pr(const std::vector<double> &v) {
  for (double x : v) std::printf("%.17g ", x);
  std::printf("\n");
}
int main() {
  char cmd[16];
  while (std::scanf("%15s", cmd) == 1) {
    std::string c(cmd);
    if (c == "solve" || c == "pinv") {
      int p; std::scanf("%d", &p);
      const Mat A = rd(p * p);
      pr(c == "solve" ? mom_safe_solve(A, p) : mom_pinv(A, p));
    } else if (c == "deriv") {
      int P, M, p; std::scanf("%d %d %d", &P, &M, &p);
      std::vector<std::vector<double>> sp(P), scp(P);
      for (int q = 0; q < P; ++q) { sp[q] = rd(M * p); scp[q] = rd(M * p); }
      pr(mom_derivative(sp, scp, M, p));
    } else if (c == "dinv") {
      int p; double w; std::scanf("%d %lf", &p, &w);
      pr(mom_dinv(rd(p * p), p, w));
    } else if (c == "guard") {
      int n, nr; std::scanf("%d %d", &n, &nr);
      const std::vector<double> th = rd(n), st = rd(n);
      pr(mom_guard_step(th, st, nr));
    }
  }
  return 0;
}
"""


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    d = tmp_path_factory.mktemp("mom_host")
    src, exe = d / "drv.cpp", d / "drv"
    src.write_text(DRIVER)
    subprocess.check_call(["g++", "-std=c++17", "-O1", "-I" + os.path.join(ROOT, "cusna_gb300", "csrc"),
                           str(src), "-o", str(exe)])

    def run(lines):
        out = subprocess.run([str(exe)], input="\n".join(lines) + "\n", capture_output=True,
                             text=True, check=True, timeout=60).stdout
        return [np.array([float(x) for x in ln.split()]) for ln in out.strip().splitlines()]
    return run


def fmt(a):
    return " ".join(repr(float(x)) for x in np.ravel(a))


def test_inverse_and_pseudo_inverse(driver):
    rng = np.random.Generator(np.random.PCG64(1))
    cases, lines = [], []
    for p in (1, 3, 5, 9):
        A = rng.standard_normal((p, p)) + p * np.eye(p)
        cases.append(("solve", A, np.linalg.inv(A)))
        lines.append(f"solve {p} {fmt(A)}")
    for p, rank in ((4, 2), (6, 5), (3, 1)):
        U = rng.standard_normal((p, rank))
        V = rng.standard_normal((rank, p))
        A = U @ V                                   # singular: solve() fails, pinv follows
        cases.append(("solve", A, mom.pinv(A)))
        lines.append(f"solve {p} {fmt(A)}")
        cases.append(("pinv", A, mom.pinv(A)))
        lines.append(f"pinv {p} {fmt(A)}")
    got = driver(lines)
    for (kind, A, ref), g in zip(cases, got):
        np.testing.assert_allclose(g.reshape(ref.shape), ref, rtol=1e-9, atol=1e-10 * np.abs(ref).max(),
                                   err_msg=f"{kind} p={A.shape[0]}")


def test_derivative_and_diagonalised_inverse(driver):
    rng = np.random.Generator(np.random.PCG64(2))
    lines, refs = [], []
    for P, M, p in ((1, 50, 3), (2, 200, 5), (4, 37, 8)):
        pieces = []
        for _ in range(P):
            sp = rng.standard_normal((M, p)) * 3 + 10
            sp[:, 0] = np.round(sp[:, 0])              # integer-valued statistics too
            scp = 0.5 * sp + rng.standard_normal((M, p))
            pieces.append((sp, scp))
        Dm = mom.mom_derivative(pieces)
        lines.append(f"deriv {P} {M} {p} " + " ".join(fmt(sp) + " " + fmt(scp) for sp, scp in pieces))
        refs.append(Dm)
        for w in (0.0, 0.2, 1.0):
            lines.append(f"dinv {p} {w!r} {fmt(Dm)}")
            refs.append(mom.mom_dinv(Dm, w))
    got = driver(lines)
    for ref, g in zip(refs, got):
        np.testing.assert_allclose(g.reshape(ref.shape), ref, rtol=1e-9, atol=1e-12 * np.abs(ref).max())


@pytest.mark.parametrize("conditional", [False, True])
def test_guarded_step(driver, conditional):
    rng = np.random.Generator(np.random.PCG64(3))
    P, k = 2, 4
    est = SimpleNamespace(P=P, conditional=conditional, coevol=False)
    n = k if conditional else P + k
    lines, refs = [], []
    for _ in range(40):
        theta = rng.standard_normal(n) * 3
        if not conditional:
            theta[:P] = np.abs(theta[:P]) + 0.5         # rates are positive
        step = rng.standard_normal(n) * rng.choice([0.1, 2.0, 20.0])
        lines.append(f"guard {n} {0 if conditional else P} {fmt(theta)} {fmt(step)}")
        refs.append(mom.guard_step(est, theta, step.copy()))
    got = driver(lines)
    for ref, g in zip(refs, got):
        np.testing.assert_array_equal(g, ref)
