"""Accuracy of the simulator's device math against CUDA's own functions:
the table-driven exp of the log-sum-exp weights (within 2 ulp of CUDA's
exp over its whole input range) and the float32 Gumbel-key estimate (within
its stated 4e-6 bound of the float64 key)."""
import os
import subprocess

import numpy as np
import pytest

from tests.conftest import ROOT

pytestmark = pytest.mark.gpu

PROGRAM = r'''
#include <cstdio>
#include <cstdlib>
#include <cstdint>
#include "saom_common.cuh"
using namespace cusna;
__global__ void k_exp(const double *y, double *mine, double *ref, int n) {
  __shared__ double tab[64];
  for (int x = threadIdx.x; x < 64; x += blockDim.x) tab[x] = kExp2Frac64[x];
  __syncthreads();
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    mine[q] = exp_weight(y[q], tab);
    ref[q] = exp(y[q]);
  }
}
__global__ void k_gumbel(const uint32_t *x, float *est, double *ref, int n) {
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    est[q] = loglog_est(x[q]);
    ref[q] = log(-log(unif01(x[q])));
  }
}
int main(int argc, char **argv) {
  const int n = atoi(argv[1]);
  FILE *f = fopen(argv[2], "rb");
  double *y = (double *)malloc(n * 8);
  uint32_t *x = (uint32_t *)malloc(n * 4);
  if (fread(y, 8, n, f) != (size_t)n || fread(x, 4, n, f) != (size_t)n) return 2;
  fclose(f);
  double *dy, *dm, *dr, *gr; float *ge; uint32_t *dx;
  cudaMalloc(&dy, n * 8); cudaMalloc(&dm, n * 8); cudaMalloc(&dr, n * 8);
  cudaMalloc(&dx, n * 4); cudaMalloc(&ge, n * 4); cudaMalloc(&gr, n * 8);
  cudaMemcpy(dy, y, n * 8, cudaMemcpyHostToDevice);
  cudaMemcpy(dx, x, n * 4, cudaMemcpyHostToDevice);
  k_exp<<<256, 256>>>(dy, dm, dr, n);
  k_gumbel<<<256, 256>>>(dx, ge, gr, n);
  if (cudaDeviceSynchronize() != cudaSuccess) return 3;
  double *m = (double *)malloc(n * 8), *r = (double *)malloc(n * 8), *g2 = (double *)malloc(n * 8);
  float *g1 = (float *)malloc(n * 4);
  cudaMemcpy(m, dm, n * 8, cudaMemcpyDeviceToHost);
  cudaMemcpy(r, dr, n * 8, cudaMemcpyDeviceToHost);
  cudaMemcpy(g1, ge, n * 4, cudaMemcpyDeviceToHost);
  cudaMemcpy(g2, gr, n * 8, cudaMemcpyDeviceToHost);
  FILE *o = fopen(argv[3], "wb");
  fwrite(m, 8, n, o); fwrite(r, 8, n, o); fwrite(g1, 4, n, o); fwrite(g2, 8, n, o);
  fclose(o);
  return 0;
}
'''


def test_exp_weight_and_gumbel_estimate(tmp_path):
    from cusna_gb300.build import ARCH, CSRC, nvcc
    src = tmp_path / "mathcheck.cu"
    exe = tmp_path / "mathcheck"
    src.write_text(PROGRAM)
    subprocess.check_call([nvcc()] + ARCH + ["-O3", "-fmad=false", "-std=c++17", "-I" + CSRC,
                                             str(src), "-o", str(exe)])
    r = np.random.Generator(np.random.PCG64(5))
    n = 1 << 20
    y = np.concatenate([-r.exponential(3.0, n // 2), r.uniform(-700, 0, n // 4),
                        -r.uniform(0, 1e-3, n // 4)])
    y[:4] = [0.0, -0.0, -700.0, -1e-300]
    x = r.integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32)
    x[:4] = [0, 0xFFFFFFFF, 0x7FFFFFFF, 0x80000000]
    inp = tmp_path / "in.bin"
    with open(inp, "wb") as f:
        f.write(y.astype(np.float64).tobytes())
        f.write(x.tobytes())
    out = tmp_path / "out.bin"
    subprocess.check_call([str(exe), str(n), str(inp), str(out)])
    buf = open(out, "rb").read()
    mine = np.frombuffer(buf[:8 * n], np.float64)
    ref = np.frombuffer(buf[8 * n:16 * n], np.float64)
    est = np.frombuffer(buf[16 * n:20 * n], np.float32).astype(np.float64)
    exact = np.frombuffer(buf[20 * n:], np.float64)
    ulp = np.abs(mine - ref) / np.spacing(np.maximum(ref, np.finfo(np.float64).tiny))
    assert ulp.max() <= 2.0, ulp.max()
    assert np.abs(est - exact).max() < 4e-6
