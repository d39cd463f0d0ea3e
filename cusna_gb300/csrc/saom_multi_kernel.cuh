// saom_multi_kernel.cuh -- the multi-network period kernel (cusna_saom_simulate_multi).
// Compiled into the library (saom_multi.cu) and, specialised to the networks'
// effect plans, at run time by NVRTC (saom_jit.cu).
//
// Restates the reference's multi-network chain (src/libcusna_saom_cpu.cpp:
// 463-552, simulate_one_multi) on the GB300 team design. D networks share the
// actors; a team keeps one shared-memory slice per network (bit rows and
// columns, degrees, the network's effect plan and parameters), laid out one
// after another, so a cross-network effect reads network w's rows at a fixed
// stride from network 0's. Each ministep draws the waiting time from the total
// rate, the network in proportion to its rate and the focal actor (32
// ministeps at a time, the reference's counters (msteps, chain, 0, 0)), then
// runs the single-network choice (net_choice) on the chosen network's slice.
#pragma once
#include "saom_chain.cuh"

namespace cusna {

__device__ __forceinline__ Slice multi_slice(unsigned char *base, const SliceLayout &lay, int d,
                                             uint32_t *cols_g, uint32_t *rows_g,
                                             size_t cols_words) {
  return carve(base + (size_t)d * lay.bytes, lay, cols_g ? cols_g + (size_t)d * cols_words : nullptr,
               rows_g ? rows_g + (size_t)d * cols_words : nullptr);
}

static __device__ void run_chain_multi(const Team &T, const DevProblem *nets, const MultiDev &md,
                                unsigned char *base, const SliceLayout &lay, uint32_t *cols_g,
                                uint32_t *rows_g, size_t cols_words, int c) {
  const int D = md.D, n = md.n, L = T.L;
  const uint32_t chain = (uint32_t)c;
  for (int d = 0; d < D; ++d)
    chain_init(T, nets[d], multi_slice(base, lay, d, cols_g, rows_g, cols_words), c);
  double lam_d[kMaxNet];
  double lam_tot = 0.0;
  for (int d = 0; d < D; ++d) {
    lam_d[d] = (double)md.lam[(size_t)c * D + d];
    lam_tot = __dadd_rn(lam_tot, lam_d[d]);
  }
  const double den = __dmul_rn((double)md.nact, lam_tot);
  long long ms = 0, msd[kMaxNet] = {};
  double t = 0.0;
  double dbuf[kMaxEff];
  const Slice S0 = multi_slice(base, lay, 0, cols_g, rows_g, cols_words);
  // network w's rows: rows0 + w*net_stride words (in shared memory the slices
  // follow one another; in global scratch each network has cols_words)
  const uint32_t *rows0 = S0.rowsT;
  const size_t net_stride = rows_g ? cols_words : lay.bytes / 4;
  for (;;) {
    const int slot = (int)(ms & 31);
    if (slot == 0) {
      if (T.warp == 0) {
        uint32_t rr[4];
        philox10((uint32_t)(ms + T.lane), chain, 0u, 0u, md.k0, md.k1, rr);
        S0.rtau[T.lane] = __ddiv_rn(-log(unif01(rr[0])), den);
        const double uv = __dmul_rn(unif01(rr[1]), lam_tot);
        int d = 0;
        double acc = lam_d[0];
        while (d < D - 1 && uv >= acc) {
          d += 1;
          acc = __dadd_rn(acc, lam_d[d]);
        }
        S0.rnet[T.lane] = d;
        long long idx = (long long)__dmul_rn(unif01(rr[2]), (double)md.nact);
        if (idx >= md.nact) idx = md.nact - 1;
        S0.rfocal[T.lane] = md.act[idx];
      }
      T.sync();
    }
    t = __dadd_rn(t, S0.rtau[slot]);
    if (t > 1.0) break;
    const int d = S0.rnet[slot], i = S0.rfocal[slot];
    const DevProblem &P = nets[d];
    const Slice S = multi_slice(base, lay, d, cols_g, rows_g, cols_words);
    const int jstar = net_choice<true>(T, P, S, i, ms, chain, dbuf, rows0, net_stride, d);
    const int aij_star = bit_of(S.rowsT, n, i, jstar);
    T.sync();
    if (T.tl < P.k) {
      const int e = T.tl;
      const double s0 = S.red[32 * T.G], se = S.red[32 * T.G + 1 + e];
      S.sc[e] = __dadd_rn(S.sc[e], __dsub_rn(S.dstar[e], __ddiv_rn(se, s0)));
    }
    ++ms;
    ++msd[d];
    if (jstar != i && T.tl == 0) {
      const int j = jstar, dl = 1 - 2 * aij_star;
      S.rowsT[(j >> 5) * n + i] ^= 1u << (j & 31);
      S.colsT[(i >> 5) * n + j] ^= 1u << (i & 31);
      S.indeg[j] += dl;
      S.outdeg[i] += dl;
      if (P.symflag) {
        S.rowsT[(i >> 5) * n + j] ^= 1u << (i & 31);
        S.colsT[(j >> 5) * n + i] ^= 1u << (j & 31);
        S.indeg[i] += dl;
        S.outdeg[j] += dl;
      }
    }
    T.sync();
    if (ms >= kMaxSteps) break;
  }
  // outputs (src/libcusna_saom_cpu.cpp:549-551, :594-600)
  if (T.tl == 0) {
    if (md.ntim) md.ntim[c] = t;
    if (md.steps) md.steps[c] = (int)ms;
    if (md.rscores)
      for (int d = 0; d < D; ++d)
        md.rscores[(size_t)c * D + d] =
            (float)__dsub_rn(__ddiv_rn((double)msd[d], lam_d[d]), (double)md.nact);
  }
  for (int d = 0; d < D; ++d) {
    const Slice S = multi_slice(base, lay, d, cols_g, rows_g, cols_words);
    if (md.scores)
      for (int q = T.tl; q < md.goff[d + 1] - md.goff[d]; q += L)
        md.scores[(size_t)c * md.k + md.gidx[md.goff[d] + q]] = (float)S.sc[q];
    if (md.a_ends) {
      uint8_t *out = md.a_ends + ((size_t)c * D + d) * n * n;
      for (size_t x = T.tl; x < (size_t)n * n; x += L) {
        const int r = (int)(x / n), col = (int)(x % n);
        out[x] = (uint8_t)bit_of(S.rowsT, n, r, col);
      }
    }
  }
  T.sync();
}

template <int MAXT>
__global__ void __launch_bounds__(MAXT, 1)
multi_kernel(const DevProblem *__restrict__ nets, MultiDev md, int M,
             unsigned long long *counter, SliceLayout lay, int G, uint32_t *cols_scratch,
             uint32_t *rows_scratch, size_t cols_words) {
  extern __shared__ __align__(16) unsigned char smem[];
  Team T;
  T.G = G;
  T.L = 32 * G;
  const int tw = threadIdx.x / T.L;
  T.tl = threadIdx.x % T.L;
  T.warp = T.tl >> 5;
  T.lane = T.tl & 31;
  T.bar = 1 + tw;
  const int teams_per_cta = blockDim.x / T.L;
  const size_t slot = (size_t)blockIdx.x * teams_per_cta + tw;
  unsigned char *base = smem + (size_t)tw * lay.bytes * md.D;
  uint32_t *cg = cols_scratch ? cols_scratch + slot * md.D * cols_words : nullptr;
  uint32_t *rg = rows_scratch ? rows_scratch + slot * md.D * cols_words : nullptr;
  const Slice S0 = multi_slice(base, lay, 0, cg, rg, cols_words);
  // each network's exponential table (ordered before use by chain_init's barriers)
  for (int d = 0; d < md.D; ++d)
    fill_exp_table(multi_slice(base, lay, d, cg, rg, cols_words).etab, T.tl, T.L);
  for (;;) {
    long long u = 0;
    if (T.tl == 0) u = (long long)atomicAdd(counter, 1ull);
    if (G == 1) {
      u = __shfl_sync(kFull, u, 0);
    } else {
      if (T.tl == 0) ((long long *)(S0.misc + 8))[0] = u;
      T.sync();
      u = ((long long *)(S0.misc + 8))[0];
      T.sync();
    }
    if (u >= M) break;
    run_chain_multi(T, nets, md, base, lay, cg, rg, cols_words, (int)u);
  }
}

}  // namespace cusna
