// saom_gof.cu -- statistics of batches of end networks on the GPU: the typed
// (creation / endowment) statistic and the sienaGOF auxiliary distributions
// (src/libcusna_saom_cpu.cpp:691-765). One CTA per chain.
#include "saom_launch.h"

namespace cusna {

namespace {

// Sum over the CTA in a fixed order (warp shuffles, then the warps' partials
// in warp order), so a launch's result does not depend on scheduling.
__device__ double cta_sum(double v, double *part) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += part[w];
  __syncthreads();
  return s;
}

}  // namespace

// Creation (etype 1): sum of F over ties of (a & keep) | force absent from x0
// and not missing at the period start. Endowment (2): sum of F over ties of x0
// absent from (a & keepS) | forceS and not missing at the end, negated. A NULL
// mask reads as all-1 (keep, keepS) or all-0 (the others).
__global__ void __launch_bounds__(256) typed_stats_kernel(
    const uint8_t *__restrict__ a, int n, int etype, const double *__restrict__ F,
    const uint8_t *__restrict__ x0, const uint8_t *__restrict__ keep,
    const uint8_t *__restrict__ force, const uint8_t *__restrict__ keepS,
    const uint8_t *__restrict__ forceS, const uint8_t *__restrict__ miss_m,
    const uint8_t *__restrict__ miss_m1, double *__restrict__ out) {
  __shared__ double part[8];
  const size_t nn = (size_t)n * n;
  const uint8_t *A = a + (size_t)blockIdx.x * nn;
  double acc = 0.0;
  for (size_t q = threadIdx.x; q < nn; q += blockDim.x) {
    bool hit;
    if (etype == 1) {
      const int st = (A[q] & (keep ? keep[q] : 1)) | (force ? force[q] : 0);
      hit = st && !x0[q] && !(miss_m && miss_m[q]);
    } else {
      const int st = (A[q] & (keepS ? keepS[q] : 1)) | (forceS ? forceS[q] : 0);
      hit = x0[q] && !st && !(miss_m1 && miss_m1[q]);
    }
    if (hit) acc += F[q];
  }
  const double s = cta_sum(acc, part);
  if (threadIdx.x == 0) out[blockIdx.x] = etype == 1 ? s : -s;
}

// In-degree (kind 0) or out-degree (kind 1) distribution: per level the number
// of actors whose degree is at most the level. Degrees are counted with
// coalesced reads (a column per thread for in-degrees, a row per warp for
// out-degrees), histogrammed, and the histogram's prefix sums answer every
// level. hist holds n+1 counters per CTA in shared memory.
__global__ void __launch_bounds__(512) degree_dist_kernel(const uint8_t *__restrict__ a, int n,
                                                          int kind,
                                                          const int *__restrict__ levls,
                                                          int nlev, double *__restrict__ out) {
  extern __shared__ int hist[];
  const size_t nn = (size_t)n * n;
  const uint8_t *A = a + (size_t)blockIdx.x * nn;
  for (int v = threadIdx.x; v <= n; v += blockDim.x) hist[v] = 0;
  __syncthreads();
  if (kind == 0) {
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
      int d = 0;
      for (int i = 0; i < n; ++i) d += A[(size_t)i * n + j] != 0;
      atomicAdd(&hist[d], 1);
    }
  } else {
    const int lane = threadIdx.x & 31, warps = blockDim.x >> 5;
    for (int i = threadIdx.x >> 5; i < n; i += warps) {
      int d = 0;
      for (int j = lane; j < n; j += 32) d += A[(size_t)i * n + j] != 0;
      for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(kFull, d, o);
      if (lane == 0) atomicAdd(&hist[d], 1);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0)
    for (int v = 1; v <= n; ++v) hist[v] += hist[v - 1];   // actors with degree <= v
  __syncthreads();
  for (int L = threadIdx.x; L < nlev; L += blockDim.x) {
    const int lv = levls[L];
    out[(size_t)blockIdx.x * nlev + L] = lv < 0 ? 0.0 : (double)hist[lv < n ? lv : n];
  }
}

// Geodesic distribution: for every source s a breadth-first search over the
// chain's packed rows R (W words per row), one warp per source. reach holds the
// actors other than s within the current distance, front those first reached
// at it; a step ORs the rows of the front into a copy of reach (nxt). The
// number of actors first reached at distance k is added to added[k] of the
// chain (k = 1..K, K the largest level needed, at most n - 1, beyond which
// nothing changes); within-distance counts are its prefix sums. Per warp 3W
// words of shared scratch follow the optional copy of the rows.
__global__ void __launch_bounds__(512) geodesic_kernel(const uint32_t *__restrict__ rows_g,
                                                       int n, int W, int K, int rows_in_smem,
                                                       unsigned long long *__restrict__ added) {
  extern __shared__ __align__(16) uint32_t sm[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, warps = blockDim.x >> 5;
  const uint32_t *Rg = rows_g + (size_t)blockIdx.x * n * W;
  const size_t rows_words = rows_in_smem ? (size_t)n * W : 0;
  for (size_t x = threadIdx.x; x < rows_words; x += blockDim.x) sm[x] = Rg[x];
  __syncthreads();
  const uint32_t *R = rows_in_smem ? sm : Rg;
  uint32_t *reach = sm + rows_words + (size_t)warp * 3 * W;
  uint32_t *front = reach + W, *nxt = front + W;
  unsigned long long *acc = added + (size_t)blockIdx.x * (K + 1);
  for (int s = warp; s < n; s += warps) {
    const int sw = s >> 5;
    const uint32_t sbit = 1u << (s & 31);
    int cnt = 0;
    for (int x = lane; x < W; x += 32) {
      const uint32_t v = R[(size_t)s * W + x] & (x == sw ? ~sbit : ~0u);
      reach[x] = v;
      front[x] = v;
      cnt += __popc(v);
    }
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(kFull, cnt, o);
    if (lane == 0 && cnt) atomicAdd(&acc[1], (unsigned long long)cnt);
    __syncwarp();
    for (int k = 2; k <= K && cnt > 0; ++k) {
      for (int x = lane; x < W; x += 32) nxt[x] = reach[x];
      for (int wi = 0; wi < W; ++wi) {
        uint32_t fw = front[wi];
        while (fw) {
          const int m = 32 * wi + __ffs(fw) - 1;
          fw &= fw - 1;
          const uint32_t *Rm = R + (size_t)m * W;
          for (int x = lane; x < W; x += 32) nxt[x] |= Rm[x];
        }
      }
      __syncwarp();   // every lane has read the whole front
      int nw = 0;
      for (int x = lane; x < W; x += 32) {
        const uint32_t v = nxt[x] & (x == sw ? ~sbit : ~0u);
        const uint32_t f = v & ~reach[x];
        front[x] = f;
        reach[x] = v;
        nw += __popc(f);
      }
      for (int o = 16; o > 0; o >>= 1) nw += __shfl_xor_sync(kFull, nw, o);
      __syncwarp();
      if (nw == 0) break;
      if (lane == 0) atomicAdd(&acc[k], (unsigned long long)nw);
    }
  }
}

// Per chain (one thread each): the within-distance count of every level, the
// prefix sum of added[1..min(level, K)] (a level <= 0 has no pair), then the
// unreachable pairs n(n-1) minus those within distance K.
__global__ void geodesic_out_kernel(const unsigned long long *__restrict__ added, int M, int n,
                                    int K, const int *__restrict__ levls, int nlev,
                                    double *__restrict__ out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= M) return;
  const unsigned long long *acc = added + (size_t)c * (K + 1);
  double *o = out + (size_t)c * (nlev + 1);
  for (int L = 0; L < nlev; ++L) {
    const int top = levls[L] < K ? levls[L] : K;
    unsigned long long w = 0;
    for (int k = 1; k <= top; ++k) w += acc[k];
    o[L] = (double)w;
  }
  unsigned long long w = 0;
  for (int k = 1; k <= K; ++k) w += acc[k];
  o[nlev] = (double)((long long)n * (n - 1) - (long long)w);
}

cudaError_t launch_typed_stats(const uint8_t *a, int n, int M, int etype, const double *F,
                               const uint8_t *x0, const uint8_t *keep, const uint8_t *force,
                               const uint8_t *keepS, const uint8_t *forceS,
                               const uint8_t *miss_m, const uint8_t *miss_m1, double *out,
                               cudaStream_t st) {
  typed_stats_kernel<<<M, 256, 0, st>>>(a, n, etype, F, x0, keep, force, keepS, forceS, miss_m,
                                        miss_m1, out);
  return cudaGetLastError();
}

size_t gof_scratch_words(int n, int M, int kind, int K) {
  if (kind != 2 || K < 1) return 0;
  const size_t W = (size_t)(n + 31) / 32;
  return (size_t)M * n * W;
}

cudaError_t launch_gof(const uint8_t *a, int n, int M, int kind, const int *levls, int nlev,
                       int K, uint32_t *rows, unsigned long long *added, double *out,
                       int smem_optin, cudaStream_t st) {
  if (kind == 0 || kind == 1) {
    const size_t dyn = (size_t)(n + 1) * 4;
    cudaError_t e = raise_dyn_smem((const void *)degree_dist_kernel, dyn);
    if (e != cudaSuccess) return e;
    degree_dist_kernel<<<M, 512, dyn, st>>>(a, n, kind, levls, nlev, out);
    return cudaGetLastError();
  }
  const int W = (n + 31) / 32;
  if (K >= 1) {
    cudaError_t e = launch_pack_rows(a, (long long)M * n, n, W, rows, st);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(added, 0, (size_t)M * (K + 1) * sizeof(unsigned long long), st);
    if (e != cudaSuccess) return e;
    const int threads = 512;
    const size_t scratch = (size_t)(threads / 32) * 3 * W * 4;
    const size_t rows_bytes = (size_t)n * W * 4;
    const int in_smem = scratch + rows_bytes <= (size_t)smem_optin;
    const size_t dyn = scratch + (in_smem ? rows_bytes : 0);
    e = raise_dyn_smem((const void *)geodesic_kernel, dyn);
    if (e != cudaSuccess) return e;
    geodesic_kernel<<<M, threads, dyn, st>>>(rows, n, W, K, in_smem, added);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  geodesic_out_kernel<<<(M + 127) / 128, 128, 0, st>>>(added, M, n, K, levls, nlev, out);
  return cudaGetLastError();
}

}  // namespace cusna
