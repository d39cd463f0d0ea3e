"""Error bounds the simulator's float32 alter pass relies on, checked on the
device against float64:
  * the float32 estimate of log(-log u) (loglog_est) is within 4e-6;
  * the float32 linear predictor sum_e fl32(theta_e * fl32(d_e)), added in
    effect order, is within (k + 8) 2^-24 sum_e |term_e| of the float64
    predictor sum_e theta_e d_e added in the same order (random and
    cancelling inputs, integer and real statistics, k = 1..24)."""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PROGRAM = r'''
#include <cstdio>
#include <cstdlib>
#include <cstdint>
#include "saom_common.cuh"
using namespace cusna;
__global__ void k_gumbel(const uint32_t *x, float *est, double *ref, int n) {
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    est[q] = loglog_est(x[q]);
    ref[q] = log(-log(unif01(x[q])));
  }
}
// one predictor per thread: k terms theta (float) times d (double), as the
// float64 path (change_stats<true>) and the float32 path (change_stats32) add them
__global__ void k_pred(const float *th, const double *d, const int *ks, int kmax, float *f32,
                       float *absf, double *f64, int n) {
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    float f = 0.f, a = 0.f;
    double g = 0.0;
    for (int e = 0; e < ks[q]; ++e) {
      const float t = th[(size_t)q * kmax + e];
      const double v = d[(size_t)q * kmax + e];
      const float term = __fmul_rn(t, (float)v);
      f = __fadd_rn(f, term);
      a = __fadd_rn(a, fabsf(term));
      g = __dadd_rn(g, __dmul_rn((double)t, v));
    }
    f32[q] = f; absf[q] = a; f64[q] = g;
  }
}
int main(int argc, char **argv) {
  const int n = atoi(argv[1]), kmax = 24;
  FILE *fi = fopen(argv[2], "rb");
  uint32_t *x = (uint32_t *)malloc((size_t)n * 4);
  float *th = (float *)malloc((size_t)n * kmax * 4);
  double *d = (double *)malloc((size_t)n * kmax * 8);
  int *ks = (int *)malloc((size_t)n * 4);
  if (fread(x, 4, n, fi) != (size_t)n || fread(th, 4, (size_t)n * kmax, fi) != (size_t)n * kmax ||
      fread(d, 8, (size_t)n * kmax, fi) != (size_t)n * kmax || fread(ks, 4, n, fi) != (size_t)n) return 2;
  fclose(fi);
  uint32_t *dx; float *ge, *dth, *df32, *dabs; double *gr, *dd, *df64; int *dks;
  cudaMalloc(&dx, (size_t)n * 4); cudaMalloc(&ge, (size_t)n * 4); cudaMalloc(&gr, (size_t)n * 8);
  cudaMalloc(&dth, (size_t)n * kmax * 4); cudaMalloc(&dd, (size_t)n * kmax * 8);
  cudaMalloc(&dks, (size_t)n * 4); cudaMalloc(&df32, (size_t)n * 4); cudaMalloc(&dabs, (size_t)n * 4);
  cudaMalloc(&df64, (size_t)n * 8);
  cudaMemcpy(dx, x, (size_t)n * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(dth, th, (size_t)n * kmax * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(dd, d, (size_t)n * kmax * 8, cudaMemcpyHostToDevice);
  cudaMemcpy(dks, ks, (size_t)n * 4, cudaMemcpyHostToDevice);
  k_gumbel<<<256, 256>>>(dx, ge, gr, n);
  k_pred<<<256, 256>>>(dth, dd, dks, kmax, df32, dabs, df64, n);
  if (cudaDeviceSynchronize() != cudaSuccess) return 3;
  float *g1 = (float *)malloc((size_t)n * 4), *f1 = (float *)malloc((size_t)n * 4), *a1 = (float *)malloc((size_t)n * 4);
  double *g2 = (double *)malloc((size_t)n * 8), *f2 = (double *)malloc((size_t)n * 8);
  cudaMemcpy(g1, ge, (size_t)n * 4, cudaMemcpyDeviceToHost);
  cudaMemcpy(g2, gr, (size_t)n * 8, cudaMemcpyDeviceToHost);
  cudaMemcpy(f1, df32, (size_t)n * 4, cudaMemcpyDeviceToHost);
  cudaMemcpy(a1, dabs, (size_t)n * 4, cudaMemcpyDeviceToHost);
  cudaMemcpy(f2, df64, (size_t)n * 8, cudaMemcpyDeviceToHost);
  FILE *o = fopen(argv[3], "wb");
  fwrite(g1, 4, n, o); fwrite(g2, 8, n, o); fwrite(f1, 4, n, o); fwrite(a1, 4, n, o); fwrite(f2, 8, n, o);
  fclose(o);
  return 0;
}
'''


def test_float32_pass_error_bounds(tmp_path):
    from cusna_gb300.build import ARCH, CSRC, nvcc
    src = tmp_path / "mathcheck.cu"
    exe = tmp_path / "mathcheck"
    src.write_text(PROGRAM)
    subprocess.check_call([nvcc()] + ARCH + ["-O3", "-fmad=false", "-std=c++17", "-I" + CSRC,
                                             str(src), "-o", str(exe)])
    r = np.random.Generator(np.random.PCG64(5))
    n, kmax = 1 << 18, 24
    x = r.integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32)
    x[:4] = [0, 0xFFFFFFFF, 0x7FFFFFFF, 0x80000000]
    th = (r.standard_normal((n, kmax)) * np.exp(r.uniform(-6, 1.5, (n, kmax)))).astype(np.float32)
    # integer counts (exact in float32), real covariate terms, and large degrees
    kind = r.integers(0, 3, (n, kmax))
    d = np.where(kind == 0, r.integers(-60, 61, (n, kmax)).astype(np.float64),
                 np.where(kind == 1, r.standard_normal((n, kmax)) * 3.0,
                          r.integers(-8000, 8001, (n, kmax)).astype(np.float64)))
    # cancelling predictors: the last term undoes the sum of the others
    canc = r.random(n) < 0.25
    part = (th[:, :-1].astype(np.float64) * d[:, :-1]).sum(axis=1)
    th[canc, -1] = 1.0
    d[canc, -1] = -part[canc] + r.standard_normal(int(canc.sum())) * 1e-3
    ks = r.integers(1, kmax + 1, n).astype(np.int32)
    ks[canc] = kmax
    inp = tmp_path / "in.bin"
    with open(inp, "wb") as f:
        f.write(x.tobytes())
        f.write(np.ascontiguousarray(th).tobytes())
        f.write(np.ascontiguousarray(d).tobytes())
        f.write(ks.tobytes())
    out = tmp_path / "out.bin"
    subprocess.check_call([str(exe), str(n), str(inp), str(out)])
    buf = open(out, "rb").read()
    o = 0
    est = np.frombuffer(buf[o:o + 4 * n], np.float32).astype(np.float64); o += 4 * n
    exact = np.frombuffer(buf[o:o + 8 * n], np.float64); o += 8 * n
    f32 = np.frombuffer(buf[o:o + 4 * n], np.float32).astype(np.float64); o += 4 * n
    absf = np.frombuffer(buf[o:o + 4 * n], np.float32).astype(np.float64); o += 4 * n
    f64 = np.frombuffer(buf[o:o + 8 * n], np.float64)
    assert np.abs(est - exact).max() < 4e-6
    bound = (ks + 8) * 2.0 ** -24 * absf
    assert (np.abs(f32 - f64) <= bound).all(), np.max(np.abs(f32 - f64) / np.maximum(bound, 1e-300))
