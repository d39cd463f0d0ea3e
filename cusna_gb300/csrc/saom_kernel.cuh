// saom_kernel.cuh -- the GB300 period-simulator kernel.
//
// One team of G warps (G = 1, 2, 4, 8 or 16) runs one chain at a time. Teams
// take chains from a global work counter, so a launch holds one team per
// resident slot and runs until the queue is empty (a persistent kernel). Each
// team owns a slice of dynamic shared memory: the chain's out-rows and in-rows
// as word-major bitsets, degrees, behaviour values and per-alter scratch.
//
// A network ministep (src/libcusna_saom_cpu.cpp:229-287) is one pass over the
// alters j, which the team's lanes split in strides of 32*G: change statistics
// d_je from popcounts of the bitsets, the linear predictor f_j = sum_e theta_e
// d_je in float32 with a rigorous error bound, the float32 Gumbel key
// g_j = f_j - log(-log u_j) with its bound, and an online log-sum-exp of the
// score sums. The keys decide the chosen alter when the best key's lower bound
// beats every other key's upper bound; otherwise the exact float64 keys of the
// alters still in range decide, ties to the smaller j, as the reference
// chooses. u_j comes from the reference's Philox counters (msteps, chain, 1,
// j), so the chosen alter, and therefore the whole trajectory, equals the CPU
// engine's.
#pragma once
#include "saom_common.cuh"

namespace cusna {

// ---------------------------------------------------------------- team sync
struct Team {
  int G, L, tl, warp, lane, bar;
  __device__ __forceinline__ void sync() const {
    if (G == 1) __syncwarp();
    else asm volatile("bar.sync %0, %1;" ::"r"(bar), "r"(L) : "memory");
  }
};

// Per-team shared-memory slice. Sizes depend on the launch's largest problem.
struct Slice {
  uint32_t *rowsT;   // W*n
  uint32_t *colsT;   // W*n (shared or global scratch)
  short *indeg, *outdeg;  // n each (degrees < 2^15 as n <= 8192)
  int *z;
  float *gbuf;       // n   upper bounds of the float32 Gumbel keys
  float *blk;        // ceil(n/32)*2*(k+1)  per 32-alter block: the score sums as
                     //   double-float pairs (or k+1 doubles on the float64 path)
  uint32_t *okbits;  // W
  int *tp;           // n   (transTies / gwdsp)
  int *tq;           // n   (gwdspFB)
  uint32_t *tpeq;    // 2W  (transTies masks tp==0, tp==1)
  double *crate;     // n   (non-basic rates)
  double *red;       // 32*G + 32 reduction scratch
  double *th;        // k  parameters of the current chain
  float *th32;       // k  the same parameters (they are float32 inputs)
  double *sc;        // k  scores
  double *dstar;     // k  change statistics of the chosen alter
  double *thb, *bsc; // kb
  double *rsc;       // nrate
  double *p1, *p2;   // k
  int *tid, *ety, *dyn, *i0, *i1, *i2, *bty, *rkind;
  int *misc;         // 16 ints: team broadcast slots
  double *rtau;      // 32 constant-rate draws: time increments,
  int *rnet, *rfocal; //   network/behaviour flag, focal actor,
  uint32_t *rr3;     //   behaviour uniform
  int *ekind, *ecfn, *eoffd, *eofft;  // k  effect plan
  double *stepd, *stept;  // 4k  per-ministep K_STEP magnitudes and terms
  float *stepd32, *stept32;  // 4k  their float32 roundings
  float *stepdlo32, *steptlo32;  // 4k  and the remainders (double-float pairs)
  float2 *etab;      // 64   2^(j/64) as double-float pairs (the score exponential)
};

struct SliceLayout {
  size_t bytes;  // per team
  size_t o_rows, o_cols, o_indeg, o_outdeg, o_z, o_g, o_blk, o_ok, o_tp, o_tq, o_tpeq, o_crate, o_red, o_th, o_sc, o_dstar, o_thb, o_bsc, o_rsc, o_p1, o_p2, o_tid,
      o_ety, o_dyn, o_i0, o_i1, o_i2, o_bty, o_rkind, o_misc, o_rtau, o_rnet, o_rfocal, o_rr3, o_ekind, o_ecfn, o_eoffd, o_eofft,
      o_stepd, o_stept, o_th32, o_stepd32, o_stept32, o_stepdlo32, o_steptlo32, o_etab;
};

__host__ __device__ inline size_t al16(size_t x) { return (x + 15) & ~(size_t)15; }

// Layout of one team slice for maxima (n, k, ...) over the launch.
__host__ __device__ inline SliceLayout make_layout(int n, int W, int k, int kb, int nrate, int G,
                                                   bool rows_in_smem, bool cols_in_smem,
                                                   bool need_tp, bool need_gw, bool need_tq) {
  SliceLayout s{};
  size_t o = 0;
  auto put = [&](size_t &field, size_t bytes) { field = o; o = al16(o + bytes); };
  put(s.o_rows, rows_in_smem ? (size_t)W * n * 4 : 0);
  put(s.o_cols, cols_in_smem ? (size_t)W * n * 4 : 0);
  put(s.o_indeg, (size_t)n * 2);
  put(s.o_outdeg, (size_t)n * 2);
  put(s.o_z, (size_t)n * 4);
  put(s.o_g, (size_t)n * 4);
  put(s.o_blk, (size_t)((n + 31) / 32) * 2 * (k + 1) * 4);
  put(s.o_ok, (size_t)W * 4);
  put(s.o_tp, need_tp || need_gw ? (size_t)n * 4 : 0);
  put(s.o_tq, need_tq ? (size_t)n * 4 : 0);
  put(s.o_tpeq, need_tp ? (size_t)W * 8 : 0);
  put(s.o_crate, nrate > 0 ? (size_t)n * 8 : 0);
  put(s.o_red, (size_t)32 * G * 8 + 32 * 8);   // 32 slots per warp, then 32 team values
  put(s.o_th, (size_t)k * 8);
  put(s.o_sc, (size_t)k * 8);
  put(s.o_dstar, (size_t)k * 8);
  put(s.o_thb, (size_t)(kb + 1) * 8);
  put(s.o_bsc, (size_t)(kb + 1) * 8);
  put(s.o_rsc, (size_t)(nrate + 1) * 8);
  put(s.o_p1, (size_t)k * 8);
  put(s.o_p2, (size_t)k * 8);
  put(s.o_tid, (size_t)k * 4);
  put(s.o_ety, (size_t)k * 4);
  put(s.o_dyn, (size_t)k * 4);
  put(s.o_i0, (size_t)k * 4);
  put(s.o_i1, (size_t)k * 4);
  put(s.o_i2, (size_t)k * 4);
  put(s.o_bty, (size_t)(kb + 1) * 4);
  put(s.o_rkind, (size_t)(nrate + 1) * 4);
  put(s.o_misc, 16 * 4);
  put(s.o_rtau, 32 * 8);
  put(s.o_rnet, 32 * 4);
  put(s.o_rfocal, 32 * 4);
  put(s.o_rr3, 32 * 4);
  put(s.o_ekind, (size_t)k * 4);
  put(s.o_ecfn, (size_t)k * 4);
  put(s.o_eoffd, (size_t)k * 4);
  put(s.o_eofft, (size_t)k * 4);
  put(s.o_stepd, (size_t)k * 4 * 8);
  put(s.o_stept, (size_t)k * 4 * 8);
  put(s.o_th32, (size_t)k * 4);
  put(s.o_stepd32, (size_t)k * 4 * 4);
  put(s.o_stept32, (size_t)k * 4 * 4);
  put(s.o_stepdlo32, (size_t)k * 4 * 4);
  put(s.o_steptlo32, (size_t)k * 4 * 4);
  put(s.o_etab, (size_t)64 * 8);
  s.bytes = al16(o);
  return s;
}

__device__ __forceinline__ Slice carve(unsigned char *base, const SliceLayout &L,
                                       uint32_t *cols_global, uint32_t *rows_global) {
  Slice s;
  s.rowsT = rows_global ? rows_global : (uint32_t *)(base + L.o_rows);
  s.colsT = cols_global ? cols_global : (uint32_t *)(base + L.o_cols);
  s.indeg = (short *)(base + L.o_indeg);
  s.outdeg = (short *)(base + L.o_outdeg);
  s.z = (int *)(base + L.o_z);
  s.gbuf = (float *)(base + L.o_g);
  s.blk = (float *)(base + L.o_blk);
  s.okbits = (uint32_t *)(base + L.o_ok);
  s.tp = (int *)(base + L.o_tp);
  s.tq = (int *)(base + L.o_tq);
  s.tpeq = (uint32_t *)(base + L.o_tpeq);
  s.crate = (double *)(base + L.o_crate);
  s.red = (double *)(base + L.o_red);
  s.th = (double *)(base + L.o_th);
  s.sc = (double *)(base + L.o_sc);
  s.dstar = (double *)(base + L.o_dstar);
  s.thb = (double *)(base + L.o_thb);
  s.bsc = (double *)(base + L.o_bsc);
  s.rsc = (double *)(base + L.o_rsc);
  s.p1 = (double *)(base + L.o_p1);
  s.p2 = (double *)(base + L.o_p2);
  s.tid = (int *)(base + L.o_tid);
  s.ety = (int *)(base + L.o_ety);
  s.dyn = (int *)(base + L.o_dyn);
  s.i0 = (int *)(base + L.o_i0);
  s.i1 = (int *)(base + L.o_i1);
  s.i2 = (int *)(base + L.o_i2);
  s.bty = (int *)(base + L.o_bty);
  s.rkind = (int *)(base + L.o_rkind);
  s.misc = (int *)(base + L.o_misc);
  s.rtau = (double *)(base + L.o_rtau);
  s.rnet = (int *)(base + L.o_rnet);
  s.rfocal = (int *)(base + L.o_rfocal);
  s.rr3 = (uint32_t *)(base + L.o_rr3);
  s.ekind = (int *)(base + L.o_ekind);
  s.ecfn = (int *)(base + L.o_ecfn);
  s.eoffd = (int *)(base + L.o_eoffd);
  s.eofft = (int *)(base + L.o_eofft);
  s.stepd = (double *)(base + L.o_stepd);
  s.stept = (double *)(base + L.o_stept);
  s.th32 = (float *)(base + L.o_th32);
  s.stepd32 = (float *)(base + L.o_stepd32);
  s.stept32 = (float *)(base + L.o_stept32);
  s.stepdlo32 = (float *)(base + L.o_stepdlo32);
  s.steptlo32 = (float *)(base + L.o_steptlo32);
  s.etab = (float2 *)(base + L.o_etab);
  return s;
}

__device__ __forceinline__ int bit_of(const uint32_t *T, int n, int row, int col) {
  return (T[(col >> 5) * n + row] >> (col & 31)) & 1;
}

// ---------------------------------------------------------------- reductions
// Sum of V doubles over the 32 lanes of a warp by recursive halving: stage s
// exchanges half of the remaining values with the lane 16>>s away, so a lane
// does V-1 + (5 - log2 V) additions instead of 5V. Afterwards the lane holds the
// warp total of quantity q(lane) in v[0]; lanes with bit 0 clear report it.
__device__ __forceinline__ double radd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float radd(float a, float b) { return __fadd_rn(a, b); }

template <int V, class R>
__device__ __forceinline__ int warp_multi_sum(R (&v)[V], int lane) {
  int q = 0;
  int cnt = V;
#pragma unroll
  for (int s = 0; (1 << s) < V; ++s) {
    const int o = 16 >> s;
    const int half = V >> (s + 1);
    const bool up = (lane & o) != 0;
#pragma unroll
    for (int x = 0; x < half; ++x) {
      const R send = up ? v[x] : v[x + half];
      const R keep = up ? v[x + half] : v[x];
      const R got = __shfl_xor_sync(kFull, send, o);
      v[x] = radd(keep, got);
    }
    if (up) q += half;
    cnt = half;
  }
  (void)cnt;
  // remaining butterfly stages (lanes sharing a quantity)
#pragma unroll
  for (int s = 0; s < 5; ++s) {
    const int o = 16 >> s;
    if ((1 << s) >= V) v[0] = radd(v[0], __shfl_xor_sync(kFull, v[0], o));
  }
  return q;
}

// Recursive halving over V double-float pairs (h[q], l[q]), any V <= 32: at
// stage s (partner lane^(16>>s)) a lane holding c values keeps the lower
// m = ceil(c/2) (bit clear) or the upper c - m, shifted down (bit set; an odd
// c pads the upper half with a zero), and adds its partner's copies, so every
// stage takes ceil(c/2) additions and V values need about V + 3 in all.
// Afterwards the lane's h[0], l[0] is the warp total of quantity q (returned)
// when *real is set; each quantity has exactly one such lane. ff_add is
// symmetric in its operands (TwoSum's error term is exact).
template <int V>
__device__ __forceinline__ int warp_multi_sum_ff(float (&h)[V], float (&l)[V], int lane,
                                                 bool *real) {
  int q = 0, r = V;  // r: how many of the lane's values are real
  int c = V;
#pragma unroll
  for (int s = 0; s < 5; ++s) {
    const int o = 16 >> s;
    const int m = (c + 1) >> 1;
    const bool up = (lane & o) != 0;
#pragma unroll
    for (int x = 0; x < m; ++x) {
      const bool pair = m + x < c;
      const float vh = pair ? h[pair ? m + x : 0] : 0.f, vl = pair ? l[pair ? m + x : 0] : 0.f;
      const float sh = up ? h[x] : vh, sl = up ? l[x] : vl;
      float kh = up ? vh : h[x], kl = up ? vl : l[x];
      const float gh = __shfl_xor_sync(kFull, sh, o), gl = __shfl_xor_sync(kFull, sl, o);
      ff_add(kh, kl, gh, gl);
      h[x] = kh;
      l[x] = kl;
    }
    if (up) {
      q += m;
      r = r > m ? r - m : 0;
    } else {
      r = r < m ? r : m;
    }
    c = m;
  }
  *real = r > 0;
  return q;
}

// Sum of K double-float pairs (h[e], l[e]) in a fixed pairwise tree, two
// additions per packed instruction: h[x] += h[x + m] for the upper half at
// each level (an odd count leaves its middle element for the next level).
template <int K>
__device__ __forceinline__ float2 ff_tree_sum(float (&h)[K], float (&l)[K]) {
  int c = K;
#pragma unroll
  for (int s = 0; s < 5; ++s) {
    if (c > 1) {
      const int m = (c + 1) >> 1, na = c - m;
#pragma unroll
      for (int x = 0; x + 1 < na; x += 2) {
        float2 ah = make_float2(h[x], h[x + 1]), al = make_float2(l[x], l[x + 1]);
        ff_add2(ah, al, make_float2(h[x + m], h[x + 1 + m]), make_float2(l[x + m], l[x + 1 + m]));
        h[x] = ah.x;
        h[x + 1] = ah.y;
        l[x] = al.x;
        l[x + 1] = al.y;
      }
      if (na & 1) ff_add(h[na - 1], l[na - 1], h[na - 1 + m], l[na - 1 + m]);
      c = m;
    }
  }
  return make_float2(h[0], l[0]);
}

__device__ __forceinline__ long long warp_max_ll(long long x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    long long y = __shfl_xor_sync(kFull, x, o);
    x = y > x ? y : x;
  }
  return x;
}

__device__ __forceinline__ float warp_max_f(float x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x = fmaxf(x, __shfl_xor_sync(kFull, x, o));
  return x;
}

__device__ __forceinline__ long long warp_sum_ll(long long x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(kFull, x, o);
  return x;
}

// Team-wide helpers. `red` is the team's scratch (>= 32*G doubles).
__device__ __forceinline__ long long team_max_ll(const Team &T, long long x, double *red) {
  x = warp_max_ll(x);
  if (T.G == 1) return x;
  long long *r = (long long *)red;
  T.sync();
  if (T.lane == 0) r[T.warp] = x;
  T.sync();
  long long m = r[0];
  for (int w = 1; w < T.G; ++w) m = r[w] > m ? r[w] : m;
  return m;
}

__device__ __forceinline__ float team_max_f(const Team &T, float x, double *red) {
  x = warp_max_f(x);
  if (T.G == 1) return x;
  float *r = (float *)red;
  T.sync();
  if (T.lane == 0) r[T.warp] = x;
  T.sync();
  float m = r[0];
  for (int w = 1; w < T.G; ++w) m = fmaxf(m, r[w]);
  return m;
}

__device__ __forceinline__ long long team_sum_ll(const Team &T, long long x, double *red) {
  x = warp_sum_ll(x);
  if (T.G == 1) return x;
  long long *r = (long long *)red;
  T.sync();
  if (T.lane == 0) r[T.warp] = x;
  T.sync();
  long long m = 0;
  for (int w = 0; w < T.G; ++w) m += r[w];
  return m;
}

// Argmax of (key, -j) over the team: larger key wins, ties to the smaller j.
__device__ __forceinline__ int team_argmax(const Team &T, long long key, int j, double *red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    long long k2 = __shfl_xor_sync(kFull, key, o);
    int j2 = __shfl_xor_sync(kFull, j, o);
    if (k2 > key || (k2 == key && j2 < j)) { key = k2; j = j2; }
  }
  if (T.G == 1) return j;
  long long *rk = (long long *)red;
  int *rj = (int *)(red + T.G);
  T.sync();
  if (T.lane == 0) { rk[T.warp] = key; rj[T.warp] = j; }
  T.sync();
  long long bk = rk[0];
  int bj = rj[0];
  for (int w = 1; w < T.G; ++w)
    if (rk[w] > bk || (rk[w] == bk && rj[w] < bj)) { bk = rk[w]; bj = rj[w]; }
  return bj;
}

// ------------------------------------------------------- change statistics
// Per-ministep context shared by all alters (uniform over the team).
struct StepCtx {
  int i, od_i, id_i, rdeg_i;
  double zvi;
  // multi-network teams: network w's rows are rows0 + w*net_stride words
  const uint32_t *rows0;
  size_t net_stride;
};

// Popcount of (A_word(a) & B_word(b)) summed over the W words.
__device__ __forceinline__ int pc2(const uint32_t *A, int a, const uint32_t *B, int b, int n, int W) {
  int c = 0;
  for (int w = 0; w < W; ++w) c += __popc(A[w * n + a] & B[w * n + b]);
  return c;
}

// Exact (double)c for 0 <= c < 2^31 built on the integer pipes.
__device__ __forceinline__ double i2d(int c) {
  if (c == 0) return 0.0;
  const int e = 31 - __clz(c);
  const unsigned long long m = ((unsigned long long)(unsigned)c << (52 - e)) & 0xFFFFFFFFFFFFFull;
  return __longlong_as_double((long long)((((unsigned long long)(1023 + e)) << 52) | m));
}
// x * delta for delta = +-1 is exact, so it is a sign flip (sgn = 0 or 1<<63).
__device__ __forceinline__ double flip(double x, unsigned long long sgn) {
  return __longlong_as_double(__double_as_longlong(x) ^ (long long)sgn);
}

// Generic change statistic of one effect (src/libcusna_saom_cpu.cpp:49-101 and
// :246-251): the reference formula evaluated per alter. Used for the kinds no
// table covers (gwdsp, interactions, dyadic covariates of very large n).
static __device__ __noinline__ double gen_stat(const DevProblem &P, const Slice &S, const StepCtx &X,
                                        int e, int j, int aij, int aji, int ri_cj, int ri_rj,
                                        int rj_ci, int ci_cj, int ci_rj, const double *d) {
  const int n = P.n, W = P.W, i = X.i, t = S.tid[e];
  const unsigned long long sg = aij ? 0x8000000000000000ull : 0ull;
  const double dl = aij ? -1.0 : 1.0;
  if (t == 32) {
    const int c2 = S.i2[e];
    double v = c2 < 0 ? dl : 1.0;
    v = __dmul_rn(v, __dmul_rn(d[S.i0[e]], d[S.i1[e]]));
    if (c2 >= 0) v = __dmul_rn(v, d[c2]);
    return v;
  }
  double vi = 0.0, vj = 0.0;
  if ((t >= 10 && t <= 13) || t == 20 || t == 21 || t == 25 || t == 31) {
    const bool dy = S.dyn[e] != 0;
    vi = dy ? X.zvi : P.vmat[(size_t)e * n + i];
    vj = dy ? __dsub_rn((double)S.z[j], P.zbar) : P.vmat[(size_t)e * n + j];
  }
  switch (t) {
    case 7: return flip(sqrt(i2d(S.indeg[j] + 1 - aij)), sg);
    case 9: return flip(sqrt(i2d(S.outdeg[j])), sg);
    case 24: return flip(P.wtab[(size_t)e * (n + 1) + ri_cj], sg);
    case 26: return flip(P.wtab[(size_t)e * (n + 1) + ri_rj], sg);
    case 27: return flip(P.wtab[(size_t)e * (n + 1) + ci_cj], sg);
    case 28: return flip(P.wtab[(size_t)e * (n + 1) + ci_rj], sg);
    case 11: return flip(vj, sg);
    case 12: return flip(__dsub_rn(__dsub_rn(1.0, __dmul_rn(fabs(__dsub_rn(vi, vj)), S.p1[e])), S.p2[e]), sg);
    case 13: return flip(fabs(__dsub_rn(vi, vj)) < 1e-9 ? 1.0 : 0.0, sg);
    case 20:
      if (vi > __dadd_rn(vj, 1e-9)) return dl;
      if (fabs(__dsub_rn(vi, vj)) <= 1e-9) return flip(0.5, sg);
      return 0.0;
    case 21: return __dmul_rn(flip(vi, sg), vj);
    case 25: return flip(__dadd_rn(vi, vj), sg);
    case 31: return flip(vj >= __dsub_rn(S.p1[e], 1e-12) ? 1.0 : 0.0, sg);
    case 29: case 30: {
      // over h in out_j (29) or in_j (30), h != i, ascending h as the reference
      // adds: the gw weight difference at p_h = |out_i & in_h| (29) or
      // |out_i & out_h| (30), both precomputed for this ministep
      const double *wr = P.wtab + (size_t)e * (n + 1);
      const uint32_t *B = (t == 29) ? S.rowsT : S.colsT;
      const int *pc = (t == 29) ? S.tp : S.tq;
      double acc = 0.0;
      for (int w = 0; w < W; ++w) {
        uint32_t m = B[w * n + j];
        if ((i >> 5) == w) m &= ~(1u << (i & 31));
        while (m) {
          const int h = (w << 5) + __ffs(m) - 1;
          m &= m - 1;
          const int p = pc[h];
          acc = __dadd_rn(acc, aij ? __dsub_rn(wr[p], wr[p - 1]) : __dsub_rn(wr[p + 1], wr[p]));
        }
      }
      return flip(acc, sg);
    }
    default: return 0.0;
  }
}

// Per-ministep magnitudes of the K_STEP effects (types 10, 14-19): for each
// (a_ij, a_ji) the reference's d and theta * d, into stepd/stept[e*4 + q],
// q = 2*a_ij + a_ji. Lanes take (e, q) pairs.
__device__ __forceinline__ void step_values(const Team &T, const DevProblem &P, const Slice &S,
                                            const StepCtx &X) {
  for (int x = T.tl; x < 4 * P.k; x += T.L) {
    const int e = x >> 2, q = x & 3;
    if (S.ekind[e] != K_STEP) continue;
    const int aij = q >> 1, aji = q & 1;
    const unsigned long long sg = aij ? 0x8000000000000000ull : 0ull;
    const double dl = aij ? -1.0 : 1.0;
    double v;
    switch (S.tid[e]) {
      case 10: v = flip(S.dyn[e] ? X.zvi : P.vmat[(size_t)e * P.n + X.i], sg); break;
      case 14: v = flip(i2d(X.id_i), sg); break;
      case 15: v = flip(sqrt(i2d(X.id_i)), sg); break;
      case 16: v = flip(__dadd_rn(__dmul_rn(2.0, i2d(X.od_i)), dl), sg); break;
      case 17: {
        const double d0 = i2d(X.od_i), d1 = __dadd_rn(d0, dl);
        v = __dsub_rn(__dmul_rn(d1, sqrt(d1)), __dmul_rn(d0, sqrt(d0)));
        break;
      }
      case 18: {
        const double d0 = i2d(X.od_i);
        v = __dsub_rn(fmin(__dadd_rn(d0, dl), S.p1[e]), fmin(d0, S.p1[e]));
        break;
      }
      case 19:
        v = flip(__dadd_rn(i2d(X.rdeg_i), __dmul_rn((double)aji, __dadd_rn(i2d(X.od_i), dl))), sg);
        break;
      default: v = 0.0; break;
    }
    const double tv = __dmul_rn(S.th[e], v);
    const float v32 = (float)v, t32 = (float)tv;
    S.stepd[x] = v;
    S.stept[x] = tv;
    S.stepd32[x] = v32;
    S.stept32[x] = t32;
    S.stepdlo32[x] = (float)__dsub_rn(v, (double)v32);
    S.steptlo32[x] = (float)__dsub_rn(tv, (double)t32);
  }
}

// Change statistics of toggling i -> j for all k effects into d[0..k-1]
// (src/libcusna_saom_cpu.cpp:49-101 per effect type, :243-261 for the loop with
// interactions and creation/endowment zeroing), and with TERMS the linear
// predictor f = sum_e theta_e d_e in the reference's e-order. Popcounts of the
// word-major bitsets replace the reference's O(n) dense loops; they count the
// same sets:
//   |out_i & in_j| = #{h: a_ih a_hj}      |out_i & out_j| = #{h: a_ih a_jh}
//   |out_j & in_i| = #{h: a_jh a_hi}      |in_i & in_j|   = #{h: a_hi a_hj}
//   |in_i & out_j| = #{h: a_hi a_jh}
// Every d and every term equals the reference's float64 value: delta * x is a
// sign flip, table entries are the reference's expressions evaluated once, and
// f adds the terms in e-order (terms of zeroed effects are +-0 and change
// nothing, so they are skipped).
// Cross-network change statistic magnitude (before the sign of the toggle) of
// toggling i -> j in the own network for cross effect type t, reading network
// w's current rows (src/libcusna_saom_cpu.cpp:431-444): 33 a_w[i][j], 34
// a_w[j][i], 35 both, 36 |out_w(i) & out_w(j)|, 37 |out_w(i) & in_own(j)|.
__device__ __forceinline__ int cross_count(const Slice &S, const StepCtx &X, int n, int W, int t,
                                           int w, int i, int j) {
  const uint32_t *Rw = X.rows0 + (size_t)w * X.net_stride;
  switch (t) {
    case 33: return bit_of(Rw, n, i, j);
    case 34: return bit_of(Rw, n, j, i);
    case 35: return bit_of(Rw, n, i, j) & bit_of(Rw, n, j, i);
    case 36: {
      int c = 0;
      for (int x = 0; x < W; ++x) c += __popc(Rw[x * n + i] & Rw[x * n + j]);
      return c;
    }
    default: {  // 37
      int c = 0;
      for (int x = 0; x < W; ++x) c += __popc(Rw[x * n + i] & S.colsT[x * n + j]);
      return c;
    }
  }
}

// MULTI: the kernel serves multi-network problems (cross effects K_CROSS);
// the single-network kernel compiles without that branch.
template <bool TERMS, bool MULTI>
__device__ __forceinline__ double change_stats(const DevProblem &P, const Slice &S,
                                               const StepCtx &X, int j, int aij, int aji,
                                               double *d) {
  const int n = P.n, W = P.W, k = P.k, i = X.i;
  const unsigned long long sg = aij ? 0x8000000000000000ull : 0ull;
  const int fl = P.flags;
  int ri_cj = 0, ri_rj = 0, rj_ci = 0, ci_cj = 0, ci_rj = 0, ricirj = 0;
  if (fl & (F_PC_RI_CJ | F_PC_RI_RJ | F_PC_RJ_CI | F_PC_CI_CJ | F_PC_CI_RJ | F_PC_RICIRJ)) {
    const uint32_t *R = S.rowsT, *Cc = S.colsT;
    for (int w = 0; w < W; ++w) {
      const uint32_t ri = R[w * n + i], rj = R[w * n + j];
      const uint32_t ci = Cc[w * n + i], cj = Cc[w * n + j];
      if (fl & F_PC_RI_CJ) ri_cj += __popc(ri & cj);
      if (fl & F_PC_RI_RJ) ri_rj += __popc(ri & rj);
      if (fl & F_PC_RJ_CI) rj_ci += __popc(rj & ci);
      if (fl & F_PC_CI_CJ) ci_cj += __popc(ci & cj);
      if (fl & F_PC_CI_RJ) ci_rj += __popc(ci & rj);
      if (fl & F_PC_RICIRJ) ricirj += __popc(ri & ci & rj);
    }
  }
  const bool ttab = (fl & F_THETA_TAB) != 0;
  double f = 0.0;
#pragma unroll 1
  for (int e = 0; e < k; ++e) {
    const int kind = S.ekind[e], cfn = S.ecfn[e];
    double v, term = 0.0;
    bool has_term = TERMS;
    if (kind == K_CNT) {
      int c;
      switch (cfn) {
        case 0: c = 1; break;
        case 1: c = aji; break;
        case 2: c = ri_cj + ri_rj; break;
        case 3: c = rj_ci; break;
        case 4: c = S.indeg[j] + 1 - aij; break;
        case 5: {
          c = 0;
          const uint32_t *eq = S.tpeq + (aij ? W : 0);
          for (int w = 0; w < W; ++w)
            c += __popc(S.rowsT[w * n + i] & S.rowsT[w * n + j] & eq[w]);
          if (S.tp[j] > 0) ++c;
          break;
        }
        case 6: c = (aji ? ri_cj : 0) + ricirj; break;
        default: c = S.outdeg[j]; break;  // 7
      }
      v = flip(i2d(c), sg);
      if (TERMS) term = ttab ? flip(P.tab[S.eofft[e] + c], sg) : __dmul_rn(S.th[e], v);
    } else if (kind == K_LOOK) {
      int idx;
      switch (cfn) {
        case 4: idx = S.indeg[j] + 1 - aij; break;
        case 7: idx = S.outdeg[j]; break;
        case 8: idx = ri_cj; break;
        case 9: idx = ri_rj; break;
        case 10: idx = ci_cj; break;
        case 11: idx = ci_rj; break;
        case 12: idx = j; break;
        case 13: idx = S.z[j] - P.zlo; break;
        case 14: idx = i * n + j; break;
        default: idx = (S.z[i] - P.zlo) * P.zR + (S.z[j] - P.zlo); break;  // 15
      }
      v = flip(P.tab[S.eoffd[e] + idx], sg);
      if (TERMS) term = ttab ? flip(P.tab[S.eofft[e] + idx], sg) : __dmul_rn(S.th[e], v);
    } else if (kind == K_STEP) {
      const int q = 2 * aij + aji;
      v = S.stepd[4 * e + q];
      term = S.stept[4 * e + q];
    } else if (kind == K_ZERO) {
      v = 0.0;
      has_term = false;
    } else if (MULTI && kind == K_CROSS) {
      const int c = cross_count(S, X, n, W, cfn, S.eoffd[e], i, j);
      v = flip((cfn == 36 && S.p1[e] >= 2.0) ? sqrt(i2d(c)) : i2d(c), sg);
      if (TERMS) term = __dmul_rn(S.th[e], v);
    } else {
      v = gen_stat(P, S, X, e, j, aij, aji, ri_cj, ri_rj, rj_ci, ci_cj, ci_rj, d);
      if (TERMS) term = __dmul_rn(S.th[e], v);
    }
    if ((S.ety[e] == 1 && aij) || (S.ety[e] == 2 && !aij)) {
      v = 0.0;
      has_term = false;
    }
    d[e] = v;
    if (has_term) f = __dadd_rn(f, term);
  }
  return f;
}

// float32 image of change_stats<true> for the shortlist pass: d32[e] is the
// float32 rounding of the change statistic d_e (exact for the integer counts;
// an interaction is the float32 product of its components), and the return
// value is f32 = sum_e fl32(theta_e * d32[e]), added in the reference's e-order
// in float32; *absf = sum_e |fl32(theta_e * d32[e])|. With u = 2^-24 each term
// differs from theta_e d_e by at most 7u|term| (at most five roundings in an
// interaction product, one in the product with theta) and the k additions add
// at most (k-1)u absf, so |f32 - f| <= (k + 8) u absf for the float64 predictor
// f of change_stats<true> (itself within 2^-50 absf of the exact sum).
//
// The same pass carries the double-float images the score sums use:
// d32lo[e] with d32[e] + d32lo[e] = d_e to about 2^-48 (0 for the integer
// counts), and the predictor as a double-float pair *fx, within about
// 2^-47 absf of f: each term's remainder (an exact Dekker product for integer
// counts; theta times the table's float32 remainder for looked-up values)
// plus the exact TwoSum error of each float32 addition (fx->x = f32 here; the
// specialised build adds the term pairs in a packed tree instead).
template <bool MULTI>
__device__ __forceinline__ float change_stats32(const DevProblem &P, const Slice &S,
                                                const StepCtx &X, int j, int aij, int aji,
                                                float *d32, float *d32lo, float *absf,
                                                float2 *fx) {
  const int n = P.n, W = P.W, k = P.k, i = X.i;
  const int fl = P.flags;
  int ri_cj = 0, ri_rj = 0, rj_ci = 0, ci_cj = 0, ci_rj = 0, ricirj = 0;
  if (fl & (F_PC_RI_CJ | F_PC_RI_RJ | F_PC_RJ_CI | F_PC_CI_CJ | F_PC_CI_RJ | F_PC_RICIRJ)) {
    const uint32_t *R = S.rowsT, *Cc = S.colsT;
    for (int w = 0; w < W; ++w) {
      const uint32_t ri = R[w * n + i], rj = R[w * n + j];
      const uint32_t ci = Cc[w * n + i], cj = Cc[w * n + j];
      if (fl & F_PC_RI_CJ) ri_cj += __popc(ri & cj);
      if (fl & F_PC_RI_RJ) ri_rj += __popc(ri & rj);
      if (fl & F_PC_RJ_CI) rj_ci += __popc(rj & ci);
      if (fl & F_PC_CI_CJ) ci_cj += __popc(ci & cj);
      if (fl & F_PC_CI_RJ) ci_rj += __popc(ci & rj);
      if (fl & F_PC_RICIRJ) ricirj += __popc(ri & ci & rj);
    }
  }
  const uint32_t sg = aij ? 0x80000000u : 0u;
  float f = 0.f, a = 0.f, fo = 0.f;
#pragma unroll 1
  for (int e = 0; e < k; ++e) {
    const int kind = S.ekind[e], cfn = S.ecfn[e];
    const float th = S.th32[e];
    float v, vlo = 0.f, term = 0.f, tlo = 0.f;
    bool has_term = true;
    if (kind == K_CNT) {
      int c;
      switch (cfn) {
        case 0: c = 1; break;
        case 1: c = aji; break;
        case 2: c = ri_cj + ri_rj; break;
        case 3: c = rj_ci; break;
        case 4: c = S.indeg[j] + 1 - aij; break;
        case 5: {
          c = 0;
          const uint32_t *eq = S.tpeq + (aij ? W : 0);
          for (int w = 0; w < W; ++w)
            c += __popc(S.rowsT[w * n + i] & S.rowsT[w * n + j] & eq[w]);
          if (S.tp[j] > 0) ++c;
          break;
        }
        case 6: c = (aji ? ri_cj : 0) + ricirj; break;
        default: c = S.outdeg[j]; break;  // 7
      }
      v = __uint_as_float(__float_as_uint((float)c) ^ sg);
      term = __fmul_rn(th, v);
      tlo = fmaf(th, v, -term);
    } else if (kind == K_LOOK) {
      int idx;
      switch (cfn) {
        case 4: idx = S.indeg[j] + 1 - aij; break;
        case 7: idx = S.outdeg[j]; break;
        case 8: idx = ri_cj; break;
        case 9: idx = ri_rj; break;
        case 10: idx = ci_cj; break;
        case 11: idx = ci_rj; break;
        case 12: idx = j; break;
        case 13: idx = S.z[j] - P.zlo; break;
        case 14: idx = i * n + j; break;
        default: idx = (S.z[i] - P.zlo) * P.zR + (S.z[j] - P.zlo); break;  // 15
      }
      const float2 t2 = P.tab2[S.eoffd[e] + idx];
      v = __uint_as_float(__float_as_uint(t2.x) ^ sg);
      vlo = __uint_as_float(__float_as_uint(t2.y) ^ sg);
      term = __fmul_rn(th, v);
      tlo = fmaf(th, vlo, fmaf(th, v, -term));
    } else if (kind == K_STEP) {
      const int q = 2 * aij + aji;
      v = S.stepd32[4 * e + q];
      vlo = S.stepdlo32[4 * e + q];
      term = S.stept32[4 * e + q];
      tlo = S.steptlo32[4 * e + q];
    } else if (kind == K_ZERO) {
      v = 0.f;
      has_term = false;
    } else if (MULTI && kind == K_CROSS) {
      const int c = cross_count(S, X, n, W, cfn, S.eoffd[e], i, j);
      const bool rt = cfn == 36 && S.p1[e] >= 2.0;
      const float m = rt ? sqrtf((float)c) : (float)c;
      // sqrt(c) = m + (c - m^2) / (2m) to ~2^-48 (one Newton step; the residual is exact)
      const float mlo = (rt && c > 0) ? __fdiv_rn(fmaf(-m, m, (float)c), __fmul_rn(2.f, m)) : 0.f;
      v = __uint_as_float(__float_as_uint(m) ^ sg);
      vlo = __uint_as_float(__float_as_uint(mlo) ^ sg);
      term = __fmul_rn(th, v);
      tlo = fmaf(th, vlo, fmaf(th, v, -term));
    } else if (S.tid[e] == 32) {
      const int c0 = S.i0[e], c1 = S.i1[e], c2 = S.i2[e];
      v = __fmul_rn(d32[c0], d32[c1]);
      vlo = __fadd_rn(fmaf(d32[c0], d32[c1], -v),
                      fmaf(d32[c0], d32lo[c1], __fmul_rn(d32lo[c0], d32[c1])));
      if (c2 >= 0) {
        const float v2 = __fmul_rn(v, d32[c2]);
        vlo = __fadd_rn(fmaf(v, d32[c2], -v2), fmaf(v, d32lo[c2], __fmul_rn(vlo, d32[c2])));
        v = v2;
      } else if (aij) {
        v = -v;
        vlo = -vlo;
      }
      term = __fmul_rn(th, v);
      tlo = fmaf(th, vlo, fmaf(th, v, -term));
    } else {
      const double v64 = gen_stat(P, S, X, e, j, aij, aji, ri_cj, ri_rj, rj_ci, ci_cj, ci_rj, nullptr);
      v = (float)v64;
      vlo = (float)__dsub_rn(v64, (double)v);
      term = __fmul_rn(th, v);
      tlo = fmaf(th, vlo, fmaf(th, v, -term));
    }
    if ((S.ety[e] == 1 && aij) || (S.ety[e] == 2 && !aij)) {
      v = 0.f;
      vlo = 0.f;
      has_term = false;
    }
    d32[e] = v;
    d32lo[e] = vlo;
    if (has_term) {
      float err;
      two_sum(f, term, f, err);
      fo = __fadd_rn(fo, __fadd_rn(err, tlo));
      a = __fadd_rn(a, fabsf(term));
    }
  }
  *absf = a;
  *fx = make_float2(f, fo);
  return f;
}

// Behaviour change statistic, src/libcusna_saom_cpu.cpp:103-113.
__device__ __forceinline__ double beh_stat(int t, double dl, double zc, long long nb, double zs,
                                           long long nh, long long ne, long long nl, double br,
                                           double bs) {
  double tc;
  switch (t) {
    case 0: return dl;
    case 1: return __dmul_rn(__dadd_rn(__dmul_rn(2.0, zc), dl), dl);
    case 2: return nb > 0 ? __ddiv_rn(__dmul_rn(dl, zs), (double)nb) : 0.0;
    case 3:
      if (nb == 0) return 0.0;
      tc = dl > 0 ? (double)(nh - ne - nl) : (double)(nl - ne - nh);
      return __ddiv_rn(tc, __dmul_rn(br, (double)nb));
    case 4:
      if (nb == 0) return 0.0;
      tc = dl > 0 ? (double)(nh - ne - nl) : (double)(nl - ne - nh);
      return __dsub_rn(__ddiv_rn(tc, br), __dmul_rn((double)nb, bs));
  }
  return 0.0;
}

}  // namespace cusna
