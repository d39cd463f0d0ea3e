// saom_sim.cu -- kernels of the GB300 SAOM period simulator: the persistent
// period kernel, the standalone statistic kernels and the input-preparation
// kernels. Host code (validation, memory, the C ABI) is in saom_api.cu.
#include "saom_period.cuh"
#include "saom_launch.h"

#include <map>
#include <mutex>
#include <utility>

namespace cusna {

// ---- standalone statistics (cusna_network_stats_gpu / behavior_stats_gpu) ----

// One warp per network: pack the dense network into word-major rows/cols in
// shared memory, then the same statistic code as the period kernel.
__global__ void netstats_kernel(const uint8_t *__restrict__ a_batch, int M, StatDesc D,
                                double *out, size_t slice_bytes) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int n = D.n, W = D.W;
  Team T;
  T.G = 1; T.L = 32; T.tl = threadIdx.x & 31; T.warp = 0; T.lane = T.tl; T.bar = 0;
  const int tw = threadIdx.x >> 5;
  unsigned char *base = smem + (size_t)tw * slice_bytes;
  uint32_t *R = (uint32_t *)base;
  uint32_t *Cc = R + (size_t)W * n;
  int *od = (int *)(Cc + (size_t)W * n);
  int *id = od + n;
  double *red = (double *)(((uintptr_t)(id + n) + 15) & ~(uintptr_t)15);
  for (int c = blockIdx.x * (blockDim.x >> 5) + tw; c < M; c += gridDim.x * (blockDim.x >> 5)) {
    const uint8_t *a = a_batch + (size_t)c * n * n;
    for (int x = T.tl; x < W * n; x += 32) {
      const int w = x / n, r = x % n;
      uint32_t ro = 0, co = 0;
      for (int b = 0; b < 32; ++b) {
        const int q = 32 * w + b;
        if (q < n) {
          ro |= (uint32_t)(a[(size_t)r * n + q] != 0) << b;
          co |= (uint32_t)(a[(size_t)q * n + r] != 0) << b;
        }
      }
      R[x] = ro;
      Cc[x] = co;
    }
    __syncwarp();
    for (int x = T.tl; x < n; x += 32) {
      int o = 0, i2 = 0;
      for (int w = 0; w < W; ++w) { o += __popc(R[w * n + x]); i2 += __popc(Cc[w * n + x]); }
      od[x] = o;
      id[x] = i2;
    }
    __syncwarp();
    network_stats_team(T, D, R, Cc, od, id, red, out + (size_t)c * D.k);
    __syncwarp();
  }
}

// Behaviour statistics (src/libcusna_saom_cpu.cpp:768-817): one warp per chain.
// Per-actor terms are formed in parallel; lane 0 adds them in actor order, and
// the avAlt/avSim inner sums run over alters in ascending order, as the
// reference adds them.
__global__ void behstats_kernel(const int *__restrict__ z_batch, int n, int M, int kb,
                                const int *__restrict__ bty, const uint8_t *__restrict__ xnet,
                                const int *__restrict__ bkdist, double zbar, double brange,
                                double bsimmean, double *out) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int lane = threadIdx.x & 31, tw = threadIdx.x >> 5;
  double *u = (double *)smem + (size_t)tw * 2 * n;
  double *term = u + n;
  for (int c = blockIdx.x * (blockDim.x >> 5) + tw; c < M; c += gridDim.x * (blockDim.x >> 5)) {
    const int *z = z_batch + (size_t)c * n;
    for (int i = lane; i < n; i += 32) {
      const bool ok = bkdist ? bkdist[i] != 0 : true;
      u[i] = ok ? __dsub_rn((double)z[i], zbar) : 0.0;
    }
    __syncwarp();
    for (int e = 0; e < kb; ++e) {
      const int t = bty[e];
      if (t == 2 || t == 3 || t == 4) {
        for (int i = lane; i < n; i += 32) {
          const uint8_t *xr = xnet + (size_t)i * n;
          const bool oki = bkdist ? bkdist[i] != 0 : true;
          double s = 0.0, od = 0.0, nb = 0.0;
          if (t == 2) {
            for (int j = 0; j < n; ++j) if (xr[j]) { od += 1.0; s = __dadd_rn(s, u[j]); }
            term[i] = od <= 0.0 ? 0.0 : __dmul_rn(u[i], __ddiv_rn(s, od));
            if (od <= 0.0) term[i] = -0.0;  // marker: skipped actor
          } else {
            for (int j = 0; j < n; ++j) {
              if (!xr[j]) continue;
              const bool okj = bkdist ? bkdist[j] != 0 : true;
              if (okj) {
                nb += 1.0;
                s = __dadd_rn(s, __dsub_rn(1.0, __ddiv_rn(fabs(__dsub_rn(u[i], u[j])), brange)));
              }
            }
            s = __dsub_rn(s, __dmul_rn(nb, bsimmean));
            if (t == 3) s = nb > 0.0 ? __ddiv_rn(s, nb) : 0.0;
            term[i] = oki ? s : -0.0;
          }
        }
      }
      __syncwarp();
      if (lane == 0) {
        double acc = 0.0;
        if (t == 0) for (int i = 0; i < n; ++i) acc = __dadd_rn(acc, u[i]);
        else if (t == 1) for (int i = 0; i < n; ++i) acc = __dadd_rn(acc, __dmul_rn(u[i], u[i]));
        else if (t >= 2 && t <= 4)
          for (int i = 0; i < n; ++i) {
            // skipped actors contribute nothing (the reference `continue`s);
            // adding -0.0 leaves every partial sum unchanged
            acc = __dadd_rn(acc, term[i]);
          }
        out[(size_t)c * kb + e] = acc;
      }
      __syncwarp();
    }
  }
}

// ---- input preparation ------------------------------------------------------

// Row-major n*W bit rows -> word-major W*n; optionally also the transposed
// matrix (in-rows) word-major. def_offdiag: when src is null, fill with the
// all-ones off-diagonal matrix (the reference's default masks).
__global__ void prep_bits_kernel(const uint32_t *src, int n, int W, uint32_t *dstT,
                                 uint32_t *dstcT, int def_mode) {
  const size_t total = (size_t)W * n;
  for (size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x; x < total;
       x += (size_t)gridDim.x * blockDim.x) {
    const int w = (int)(x / n), r = (int)(x % n);
    uint32_t v = 0, vc = 0;
    for (int b = 0; b < 32; ++b) {
      const int q = 32 * w + b;
      if (q >= n) break;
      int bit_rq, bit_qr;
      if (src) {
        bit_rq = (src[(size_t)r * W + w] >> b) & 1;                 // a[r][q]
        bit_qr = (src[(size_t)q * W + (r >> 5)] >> (r & 31)) & 1;  // a[q][r]
      } else {
        bit_rq = bit_qr = def_mode == 1 ? (q != r) : 0;
      }
      v |= (uint32_t)bit_rq << b;
      vc |= (uint32_t)bit_qr << b;
    }
    if (dstT) dstT[x] = v;
    if (dstcT) dstcT[x] = vc;
  }
}

// float64 descriptor with the reference's precedence: the *64 array if given,
// else the float array promoted, else zeros (src/libcusna_saom_cpu.cpp:337-350).
__global__ void prep_desc_kernel(const double *d64, const float *d32, size_t cnt, double *dst) {
  for (size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x; x < cnt;
       x += (size_t)gridDim.x * blockDim.x)
    dst[x] = d64 ? d64[x] : (d32 ? (double)d32[x] : 0.0);
}

__global__ void fill_int_kernel(int *dst, size_t cnt, int mode, int value) {
  for (size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x; x < cnt;
       x += (size_t)gridDim.x * blockDim.x)
    dst[x] = mode == 0 ? value : (int)x;  // mode 1: identity (act)
}

// ---- launch wrappers used by the host code ----------------------------------

// Kernels launched by this thread (reported through cusna_gpu_options).
thread_local long long g_launches = 0;
long long kernel_launches() { return g_launches; }
void note_launch() { ++g_launches; }
static cudaError_t counted(cudaError_t e) {
  if (e == cudaSuccess) ++g_launches;
  return e;
}

// A kernel's dynamic shared memory limit is one value per function and
// device, shared by every host thread. Setting it to each launch's own size
// would let one thread lower it between another thread's setting and launch,
// and fail that launch; so the limit only rises.
cudaError_t raise_dyn_smem(const void *func, size_t bytes) {
  static std::mutex mu;
  static std::map<std::pair<int, const void *>, size_t> limit;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lk(mu);
  size_t &cur = limit[{dev, func}];
  if (bytes <= cur) return cudaSuccess;
  e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess) cur = bytes;
  return e;
}

template <int MAXT, bool VALID>
static int blocks_per_sm_t(int threads, size_t dyn_smem) {
  if (raise_dyn_smem((const void *)period_kernel<MAXT, VALID>, dyn_smem) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  int b = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, period_kernel<MAXT, VALID>, threads,
                                                    dyn_smem) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return b;
}

// The validation build exists for CTAs of up to 256 threads only.
int period_blocks_per_sm(int threads, size_t dyn_smem, bool valid) {
  if (valid) return threads <= 256 ? blocks_per_sm_t<256, true>(threads, dyn_smem) : 0;
  return threads <= 256 ? blocks_per_sm_t<256, false>(threads, dyn_smem)
                        : blocks_per_sm_t<512, false>(threads, dyn_smem);
}

cudaError_t launch_period(const LaunchShape &sh, const DevProblem *probs, const long long *unit_start,
                          int nprob, long long total, unsigned long long *counter,
                          uint32_t *cols_scratch, uint32_t *rows_scratch, size_t cols_words,
                          cudaStream_t st, bool valid) {
  const int threads = 32 * sh.G * sh.teams_per_cta;
  const size_t dyn = sh.lay.bytes * sh.teams_per_cta;
  if (valid && threads > 256) return cudaErrorInvalidConfiguration;
  auto kern = valid ? period_kernel<256, true>
                    : (threads <= 256 ? period_kernel<256, false> : period_kernel<512, false>);
  cudaError_t e = raise_dyn_smem((const void *)kern, dyn);
  if (e != cudaSuccess) return e;
  kern<<<sh.ctas, threads, dyn, st>>>(probs, unit_start, nprob, total, counter, sh.lay, sh.G,
                                      cols_scratch, rows_scratch, cols_words);
  return counted(cudaGetLastError());
}

// ---- replayable plans --------------------------------------------------------
// Each launch of a plan simulates with Philox key = the problem's seed plus the
// plan's epoch (64-bit, so epoch 0 is the plain call), then advances the epoch.
__global__ void plan_epoch_kernel(DevProblem *probs, const unsigned long long *base_seed,
                                  int count, unsigned long long *epoch) {
  __shared__ unsigned long long e;
  if (threadIdx.x == 0) e = *epoch;
  __syncthreads();
  for (int q = threadIdx.x; q < count; q += blockDim.x) {
    const unsigned long long s = base_seed[q] + e;
    probs[q].k0 = (uint32_t)(s & 0xFFFFFFFFull);
    probs[q].k1 = (uint32_t)(s >> 32);
  }
  __syncthreads();
  if (threadIdx.x == 0) *epoch = e + 1;
}

// Rebuilds the theta-premultiplied term tables of a plan's problems from the
// current parameter row (one block per table): entry x of effect e's table is
// theta_e * x for a count table and theta_e * value_x for a lookup table,
// rounded as the host builds them.
__global__ void plan_retheta_kernel(const DevProblem *probs, const PlanTable *tabs) {
  const PlanTable T = tabs[blockIdx.x];
  const DevProblem &P = probs[T.q];
  const double th = (double)P.theta[T.e];
  double *tab = const_cast<double *>(P.tab);
  for (int x = threadIdx.x; x < T.size; x += blockDim.x) {
    const double v = T.kind == K_CNT ? (double)x : tab[T.offd + x];
    tab[T.offt + x] = __dmul_rn(th, v);
  }
}

cudaError_t launch_plan_prologue(DevProblem *probs, const unsigned long long *base_seed, int count,
                                 unsigned long long *epoch, const PlanTable *tabs, int n_tabs,
                                 cudaStream_t st) {
  plan_epoch_kernel<<<1, 256, 0, st>>>(probs, base_seed, count, epoch);
  cudaError_t e = counted(cudaGetLastError());
  if (e != cudaSuccess || n_tabs == 0) return e;
  plan_retheta_kernel<<<n_tabs, 128, 0, st>>>(probs, tabs);
  return counted(cudaGetLastError());
}

cudaError_t launch_netstats(const uint8_t *a, int M, const StatDesc &D, double *out, int sms,
                            cudaStream_t st) {
  const size_t slice = al16((size_t)2 * D.W * D.n * 4 + (size_t)2 * D.n * 4) + 32 * 8 + 64;
  int warps = (int)((200 * 1024) / slice);
  if (warps > 8) warps = 8;
  if (warps < 1) return cudaErrorInvalidValue;
  cudaError_t e = raise_dyn_smem((const void *)netstats_kernel, slice * warps);
  if (e != cudaSuccess) return e;
  int blocks = (M + warps - 1) / warps;
  if (blocks > 4 * sms) blocks = 4 * sms;
  netstats_kernel<<<blocks, 32 * warps, slice * warps, st>>>(a, M, D, out, slice);
  return counted(cudaGetLastError());
}

cudaError_t launch_behstats(const int *z, int n, int M, int kb, const int *bty, const uint8_t *xnet,
                            const int *bkdist, double zbar, double brange, double bsimmean,
                            double *out, int sms, cudaStream_t st) {
  const size_t per = (size_t)2 * n * 8;
  int warps = (int)((200 * 1024) / per);
  if (warps > 8) warps = 8;
  if (warps < 1) return cudaErrorInvalidValue;
  cudaError_t e = raise_dyn_smem((const void *)behstats_kernel, per * warps);
  if (e != cudaSuccess) return e;
  int blocks = (M + warps - 1) / warps;
  if (blocks > 4 * sms) blocks = 4 * sms;
  behstats_kernel<<<blocks, 32 * warps, per * warps, st>>>(z, n, M, kb, bty, xnet, bkdist, zbar,
                                                           brange, bsimmean, out);
  return counted(cudaGetLastError());
}

cudaError_t launch_prep_bits(const uint32_t *src, int n, int W, uint32_t *dstT, uint32_t *dstcT,
                             int def_mode, cudaStream_t st) {
  const size_t total = (size_t)W * n;
  int blocks = (int)((total + 255) / 256);
  if (blocks > 1024) blocks = 1024;
  if (blocks < 1) blocks = 1;
  prep_bits_kernel<<<blocks, 256, 0, st>>>(src, n, W, dstT, dstcT, def_mode);
  return counted(cudaGetLastError());
}

cudaError_t launch_prep_desc(const double *d64, const float *d32, size_t cnt, double *dst,
                             cudaStream_t st) {
  if (cnt == 0) return cudaSuccess;
  int blocks = (int)((cnt + 255) / 256);
  if (blocks > 1024) blocks = 1024;
  prep_desc_kernel<<<blocks, 256, 0, st>>>(d64, d32, cnt, dst);
  return counted(cudaGetLastError());
}

cudaError_t launch_fill_int(int *dst, size_t cnt, int mode, int value, cudaStream_t st) {
  if (cnt == 0) return cudaSuccess;
  int blocks = (int)((cnt + 255) / 256);
  if (blocks > 1024) blocks = 1024;
  fill_int_kernel<<<blocks, 256, 0, st>>>(dst, cnt, mode, value);
  return counted(cudaGetLastError());
}

}  // namespace cusna
