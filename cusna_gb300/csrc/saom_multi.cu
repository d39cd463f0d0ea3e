// saom_multi.cu -- host launchers of the multi-network period kernel
// (saom_multi_kernel.cuh) and the cross-network statistics kernels.
#include "saom_multi_kernel.cuh"
#include "saom_launch.h"

namespace cusna {

int multi_blocks_per_sm(int threads, size_t dyn_smem) {
  int blocks = 0;
  auto kern = threads <= 256 ? multi_kernel<256> : multi_kernel<512>;
  if (raise_dyn_smem((const void *)kern, dyn_smem) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, kern, threads, dyn_smem) !=
      cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return blocks;
}

cudaError_t launch_multi(const LaunchShape &sh, const DevProblem *nets, const MultiDev &md, int M,
                         unsigned long long *counter, uint32_t *cols_scratch,
                         uint32_t *rows_scratch, size_t cols_words, cudaStream_t st) {
  const int threads = 32 * sh.G * sh.teams_per_cta;
  const size_t dyn = sh.lay.bytes * md.D * sh.teams_per_cta;
  auto kern = threads <= 256 ? multi_kernel<256> : multi_kernel<512>;
  cudaError_t e = raise_dyn_smem((const void *)kern, dyn);
  if (e != cudaSuccess) return e;
  kern<<<sh.ctas, threads, dyn, st>>>(nets, md, M, counter, sh.lay, sh.G, cols_scratch,
                                      rows_scratch, cols_words);
  return cudaGetLastError();
}

// ---- cross-network statistics (src/libcusna_saom_cpu.cpp:819-857) ----------
// Rows of dense uint8 matrices packed into W words each (word w of row r holds
// columns 32w .. 32w+31), one thread per word.
__global__ void pack_rows_kernel(const uint8_t *__restrict__ a, long long rows, int n, int W,
                                 uint32_t *__restrict__ out) {
  const long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= rows * W) return;
  const long long r = x / W;
  const int w = (int)(x % W);
  const uint8_t *src = a + r * n;
  uint32_t v = 0;
  for (int b = 0; b < 32; ++b) {
    const int col = 32 * w + b;
    if (col < n && src[col]) v |= 1u << b;
  }
  out[x] = v;
}

// One CTA per chain: the cross statistic of own network a (dense rows a, packed
// rows ar) against the source predictor wp (dense, packed rows wr).
//   33 sum a_ij wp_ij      34 sum a_ij wp_ji      35 sum a_ij wp_ij wp_ji
//   36 sum a_ij s_ij, s_ij = |wp row i & wp row j| (sqrt when parm >= 2)
//   37 sum a_ij (wp a)_ij = sum over wp_ih = 1 of |a row i & a row h|
// Integer sums are exact in any order; the square-root sum of 36 adds in a
// fixed order for a given launch.
__global__ void __launch_bounds__(256) cross_stats_kernel(const uint8_t *__restrict__ a,
                                                          const uint8_t *__restrict__ wp,
                                                          const uint32_t *__restrict__ ar,
                                                          const uint32_t *__restrict__ wr, int n,
                                                          int W, int t, double parm,
                                                          double *__restrict__ out) {
  __shared__ double part[8];
  const int c = blockIdx.x;
  const size_t nn = (size_t)n * n;
  const uint8_t *A = a + (size_t)c * nn;
  const uint32_t *AR = ar ? ar + (size_t)c * n * W : nullptr;
  double acc = 0.0;
  for (size_t q = threadIdx.x; q < nn; q += blockDim.x) {
    const int i = (int)(q / n), j = (int)(q % n);
    switch (t) {
      case 33: acc += (double)(A[q] & wp[q]); break;
      case 34: acc += (double)(A[q] & wp[(size_t)j * n + i]); break;
      case 35: acc += (double)(A[q] & wp[q] & wp[(size_t)j * n + i]); break;
      case 36:
        if (A[q]) {
          int s = 0;
          for (int w = 0; w < W; ++w) s += __popc(wr[(size_t)i * W + w] & wr[(size_t)j * W + w]);
          acc += parm >= 2.0 ? sqrt((double)s) : (double)s;
        }
        break;
      default:  // 37: q = (i, h) over the predictor
        if (wp[q]) {
          int s = 0;
          for (int w = 0; w < W; ++w) s += __popc(AR[(size_t)i * W + w] & AR[(size_t)j * W + w]);
          acc += (double)s;
        }
        break;
    }
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(kFull, acc, o);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int x = 0; x < (int)(blockDim.x >> 5); ++x) s += part[x];
    out[c] = s;
  }
}

cudaError_t launch_pack_rows(const uint8_t *a, long long rows, int n, int W, uint32_t *out,
                             cudaStream_t st) {
  const long long words = rows * W;
  pack_rows_kernel<<<(unsigned)((words + 255) / 256), 256, 0, st>>>(a, rows, n, W, out);
  return cudaGetLastError();
}

cudaError_t launch_cross_stats(const uint8_t *a, const uint8_t *wp, int n, int M, int t,
                               double parm, uint32_t *ar, uint32_t *wr, double *out,
                               cudaStream_t st) {
  const int W = (n + 31) / 32;
  if (t == 36) {
    const long long words = (long long)n * W;
    pack_rows_kernel<<<(unsigned)((words + 255) / 256), 256, 0, st>>>(wp, n, n, W, wr);
  }
  if (t == 37) {
    const long long words = (long long)M * n * W;
    pack_rows_kernel<<<(unsigned)((words + 255) / 256), 256, 0, st>>>(a, (long long)M * n, n, W, ar);
  }
  cross_stats_kernel<<<M, 256, 0, st>>>(a, wp, t == 37 ? ar : nullptr, t == 36 ? wr : nullptr, n,
                                        W, t, parm, out);
  return cudaGetLastError();
}

}  // namespace cusna
