// saom_period.cuh -- the persistent period kernel and the end of a chain.
// Compiled into the library (saom_sim.cu) and, specialised to one effect plan,
// at run time by NVRTC (saom_jit.cu).
#pragma once
#include "saom_chain.cuh"

namespace cusna {

__device__ void chain_finish(const Team &T, const DevProblem &P, const Slice &S, int c,
                             long long dist, long long bdist, long long ms, long long msb,
                             double t, double rho, double lam, double lamb) {
  const int n = P.n, W = P.W, k = P.k;
  T.sync();
  // composition change: restore inactive actors' rows and columns to x0
  // (src/libcusna_saom_cpu.cpp:290-291)
  if (P.has_comp) {
    for (int i = 0; i < n; ++i) {
      if (!((P.inact[i >> 5] >> (i & 31)) & 1u)) continue;
      for (int w = T.tl; w < W; w += T.L) {
        S.rowsT[w * n + i] = P.x0T[w * n + i];
        S.colsT[w * n + i] = P.x0cT[w * n + i];
      }
      T.sync();
      const uint32_t bit = 1u << (i & 31);
      const int wi = i >> 5;
      for (int j = T.tl; j < n; j += T.L) {
        if (j == i) continue;
        S.rowsT[wi * n + j] = (S.rowsT[wi * n + j] & ~bit) | (P.x0T[wi * n + j] & bit);
        S.colsT[wi * n + j] = (S.colsT[wi * n + j] & ~bit) | (P.x0cT[wi * n + j] & bit);
      }
      T.sync();
    }
  }
  // dense end network (src/libcusna_saom_cpu.cpp:410-412), 4 bytes per store
  if (P.a_ends) {
    uint8_t *out = P.a_ends + (size_t)c * n * n;
    const size_t nn = (size_t)n * n;
    if ((nn & 3) == 0 && (((uintptr_t)out) & 3) == 0) {
      uint32_t *o4 = (uint32_t *)out;
      for (size_t q = T.tl; q < nn / 4; q += T.L) {
        uint32_t v = 0;
#pragma unroll
        for (int b = 0; b < 4; ++b) {
          const size_t x = 4 * q + b;
          const int i = (int)(x / n), j = (int)(x % n);
          v |= (uint32_t)bit_of(S.rowsT, n, i, j) << (8 * b);
        }
        o4[q] = v;
      }
    } else {
      for (size_t x = T.tl; x < nn; x += T.L) {
        const int i = (int)(x / n), j = (int)(x % n);
        out[x] = (uint8_t)bit_of(S.rowsT, n, i, j);
      }
    }
  }
  // distance over kdist (:293-296)
  long long ds = 0;
  for (int i = T.tl; i < n; i += T.L) {
    int cnt = 0;
    for (int w = 0; w < W; ++w)
      cnt += __popc((S.rowsT[w * n + i] ^ P.x0T[w * n + i]) & P.kdistT[w * n + i]);
    if (P.actor_dist) P.actor_dist[(size_t)c * n + i] = cnt;
    ds += cnt;
  }
  ds = team_sum_ll(T, ds, S.red);
  if (P.kb > 0 && P.z_end)
    for (int x = T.tl; x < n; x += T.L) P.z_end[(size_t)c * n + x] = S.z[x];
  // statistics of the masked end network (A & keep) | force (:413-421)
  if (P.stats) {
    T.sync();
    for (int x = T.tl; x < W * n; x += T.L) {
      S.rowsT[x] = (S.rowsT[x] & P.keepT[x]) | P.forceT[x];
      S.colsT[x] = (S.colsT[x] & P.keepcT[x]) | P.forcecT[x];
    }
    T.sync();
    for (int x = T.tl; x < n; x += T.L) {
      int od = 0, id = 0;
      for (int w = 0; w < W; ++w) {
        od += __popc(S.rowsT[w * n + x]);
        id += __popc(S.colsT[w * n + x]);
      }
      S.outdeg[x] = od;
      S.indeg[x] = id;
    }
    T.sync();
    StatDesc D;
    D.vmat = P.vmat; D.vb = P.vb; D.wtab = P.wtab; D.p1 = P.p1; D.p2 = P.p2;
    D.vmiss = P.vmiss; D.dyn = P.dyn; D.od0 = P.od0; D.id0 = P.id0; D.type_ids = P.type_ids;
    D.n = n; D.W = W; D.k = k; D.symflag = P.symflag;
    network_stats_team(T, D, S.rowsT, S.colsT, S.outdeg, S.indeg, S.red, P.stats + (size_t)c * k);
  }
  if (T.tl == 0) {
    if (P.dist) P.dist[c] = (int)dist;
    if (P.dist_stat) P.dist_stat[c] = (int)ds;
    if (P.steps) P.steps[c] = (int)ms;
    if (P.ntim) P.ntim[c] = t;
    if (P.scores) {
      const double moves = (double)(ms - msb);
      const double rate_score = P.nrate > 0 ? __dsub_rn(__ddiv_rn(moves, lam), rho)
                                            : __dsub_rn(__ddiv_rn(moves, lam), (double)P.nact);
      P.scores[(size_t)c * (k + 1)] = (float)rate_score;
      for (int e = 0; e < k; ++e) P.scores[(size_t)c * (k + 1) + 1 + e] = (float)S.sc[e];
    }
    if (P.kb > 0) {
      if (P.bdist) P.bdist[c] = (int)bdist;
      if (P.bscores) {
        P.bscores[(size_t)c * (P.kb + 1)] =
            (float)__dsub_rn(__ddiv_rn((double)msb, lamb), (double)P.nact);
        for (int e = 0; e < P.kb; ++e) P.bscores[(size_t)c * (P.kb + 1) + 1 + e] = (float)S.bsc[e];
      }
    }
    if (P.nrate > 0 && P.rscores)
      for (int q = 0; q < P.nrate; ++q) P.rscores[(size_t)c * P.nrate + q] = (float)S.rsc[q];
  }
  T.sync();
}

// Persistent period kernel: every team repeatedly takes the next chain of the
// launch's work list (all chains of all problems) until the list is empty.
// MAXT is the largest CTA the instantiation serves: 256 threads with a register
// budget for three CTAs per SM (teams of up to 8 warps), or 512 (16-warp teams).
#ifndef CUSNA_MINB_256
#define CUSNA_MINB_256 2  // resident 256-thread CTAs per SM the register budget allows
#endif
// VALID: the validation build (trace records and caller-supplied words).
template <int MAXT, bool VALID = false>
__global__ void __launch_bounds__(MAXT, MAXT == 512 ? 1 : CUSNA_MINB_256)
period_kernel(const DevProblem *__restrict__ probs, const long long *__restrict__ unit_start,
              int nprob, long long total, unsigned long long *counter, SliceLayout lay, int G,
              uint32_t *cols_scratch, uint32_t *rows_scratch, size_t cols_words) {
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
  Slice S = carve(smem + (size_t)tw * lay.bytes, lay,
                  cols_scratch ? cols_scratch + slot * cols_words : nullptr,
                  rows_scratch ? rows_scratch + slot * cols_words : nullptr);
  fill_exp_table(S.etab, T.tl, T.L);  // ordered before its first use by chain_init's barriers
  for (;;) {
    long long u = 0;
    if (T.tl == 0) u = (long long)atomicAdd(counter, 1ull);
    if (G == 1) {
      u = __shfl_sync(kFull, u, 0);
    } else {
      if (T.tl == 0) ((long long *)(S.misc + 8))[0] = u;
      T.sync();
      u = ((long long *)(S.misc + 8))[0];
      T.sync();
    }
    if (u >= total) break;
    int lo = 0, hi = nprob - 1;
    while (lo < hi) {  // last problem whose first unit is <= u
      const int mid = (lo + hi + 1) >> 1;
      if (unit_start[mid] <= u) lo = mid; else hi = mid - 1;
    }
    const DevProblem &P = probs[lo];
    run_chain<VALID>(T, P, S, (int)(u - unit_start[lo]));
  }
}

}  // namespace cusna
