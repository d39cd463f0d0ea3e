// saom_chain.cuh -- one chain of one period, run by a team of G warps.
// Restates src/libcusna_saom_cpu.cpp:142-303 (simulate_one) and :394-422 (the
// per-chain outputs) over word-major bitsets.
#pragma once
#include "saom_kernel.cuh"
#include "saom_stats.cuh"

namespace cusna {

// Load the chain's start state and parameters into the team slice.
__device__ __forceinline__ void chain_init(const Team &T, const DevProblem &P, const Slice &S,
                                           int c) {
  const int n = P.n, W = P.W, k = P.k, L = T.L;
  for (int x = T.tl; x < W * n; x += L) {
    S.rowsT[x] = P.simT[x];
    S.colsT[x] = P.simcT[x];
  }
  for (int e = T.tl; e < k; e += L) {
    S.th32[e] = P.theta[(size_t)c * P.prow * k + e];
    S.th[e] = (double)S.th32[e];
    S.sc[e] = 0.0;
    S.tid[e] = P.type_ids[e];
    S.ety[e] = P.etypes[e];
    S.dyn[e] = P.dyn[e];
    S.i0[e] = P.int0[e];
    S.i1[e] = P.int1[e];
    S.i2[e] = P.int2[e];
    S.p1[e] = P.p1[e];
    S.p2[e] = P.p2[e];
    S.ekind[e] = P.ekind[e];
    S.ecfn[e] = P.ecfn[e];
    S.eoffd[e] = P.eoffd[e];
    S.eofft[e] = P.eofft[e];
  }
  for (int e = T.tl; e < P.kb; e += L) {
    S.thb[e] = P.thetab ? (double)P.thetab[(size_t)c * P.prow * P.kb + e] : 0.0;
    S.bsc[e] = 0.0;
    S.bty[e] = P.bty[e];
  }
  for (int q = T.tl; q < P.nrate; q += L) {
    S.rsc[q] = 0.0;
    S.rkind[q] = P.rkind[q];
  }
  if (P.flags & F_HAS_Z)
    for (int x = T.tl; x < n; x += L) S.z[x] = P.z0[x];
  if (P.nrate > 0)
    for (int x = T.tl; x < n; x += L) S.crate[x] = 1.0;
  if (T.tl == 0) {
    S.misc[12] = -1;  // last ministep whose score sums need the float64 path
    S.misc[13] = c;   // the chain's index within its problem (validation words)
  }
  T.sync();
  for (int x = T.tl; x < n; x += L) {
    int od = 0, id = 0;
    for (int w = 0; w < W; ++w) {
      od += __popc(S.rowsT[w * n + x]);
      id += __popc(S.colsT[w * n + x]);
    }
    S.outdeg[x] = od;
    S.indeg[x] = id;
  }
  T.sync();
}

// Per-ministep helper arrays: transTies two-path counts and masks, gwdsp counts.
__device__ __forceinline__ void step_helpers(const Team &T, const DevProblem &P, const Slice &S,
                                             int i) {
  const int n = P.n, W = P.W;
  const bool tp = (P.flags & (F_NEED_TP | F_NEED_GW29)) != 0;
  const bool tq = (P.flags & F_NEED_GW30) != 0;
  if (!tp && !tq) return;
  for (int h = T.tl; h < n; h += T.L) {
    int a = 0, b = 0;
    for (int w = 0; w < W; ++w) {
      const uint32_t ri = S.rowsT[w * n + i];
      if (tp) a += __popc(ri & S.colsT[w * n + h]);
      if (tq) b += __popc(ri & S.rowsT[w * n + h]);
    }
    if (tp) S.tp[h] = a;
    if (tq) S.tq[h] = b;
  }
  T.sync();
  if (P.flags & F_NEED_TP) {
    // masks {h : tp_h == 0} and {h : tp_h == 1}, word-parallel via ballots
    for (int hb = 32 * T.warp; hb < W * 32; hb += T.L) {
      const int h = hb + T.lane;
      const int v = h < n ? S.tp[h] : -1;
      const uint32_t z0 = __ballot_sync(kFull, v == 0), z1 = __ballot_sync(kFull, v == 1);
      if (T.lane == 0) { S.tpeq[hb >> 5] = z0; S.tpeq[W + (hb >> 5)] = z1; }
    }
    T.sync();
  }
}

// The four Philox words of ministep ms, counter (ms, chain, 0, 0) as the
// reference draws them (src/libcusna_saom_cpu.cpp:167); in validation mode
// (VALID) the caller's words for that ministep while they last.
template <bool VALID>
__device__ __forceinline__ void step_words(const DevProblem &P, const Slice &S, long long ms,
                                           uint32_t chain, uint32_t out[4]) {
  if (VALID && P.ustream && ms < P.ustream_steps) {
    const uint32_t *u =
        P.ustream + ((size_t)S.misc[13] * P.ustream_steps + (size_t)ms) * (4 + (size_t)P.n);
    out[0] = u[0]; out[1] = u[1]; out[2] = u[2]; out[3] = u[3];
    return;
  }
  philox10((uint32_t)ms, chain, 0u, 0u, P.k0, P.k1, out);
}

// The Gumbel word of alter j in ministep ms: first output of counter
// (ms, chain, 1, j) (src/libcusna_saom_cpu.cpp:266), or the caller's word.
template <bool VALID>
__device__ __forceinline__ uint32_t alter_word(const DevProblem &P, const Slice &S, long long ms,
                                               uint32_t chain, int j) {
  if (VALID && P.ustream && ms < P.ustream_steps)
    return P.ustream[((size_t)S.misc[13] * P.ustream_steps + (size_t)ms) * (4 + (size_t)P.n) + 4 +
                     (size_t)j];
  uint32_t ph[4];
  philox10((uint32_t)ms, chain, 1u, (uint32_t)j, P.k0, P.k1, ph);
  return ph[0];
}

// Behaviour ministep (src/libcusna_saom_cpu.cpp:202-227), run by the team's
// lane 0 in the reference's order. Updates z, bsc, *bdist; returns the step
// d in {-1, 0, 1}.
static __device__ int beh_step(const DevProblem &P, const Slice &S, int i, uint32_t r3,
                         long long *bdist) {
  const int n = P.n, W = P.W, kb = P.kb;
  const int zi = S.z[i];
  const double zc = __dsub_rn((double)zi, P.zbar);
  long long nb = 0, nh = 0, ne = 0, nl = 0;
  double zs = 0.0;
  for (int w = 0; w < W; ++w) {
    uint32_t m = S.rowsT[w * n + i];
    while (m) {
      const int j = (w << 5) + __ffs(m) - 1;
      m &= m - 1;
      const int zj = S.z[j];
      ++nb;
      zs = __dadd_rn(zs, __dsub_rn((double)zj, P.zbar));
      if (zj > zi) ++nh; else if (zj == zi) ++ne; else ++nl;
    }
  }
  const bool up = zi < P.zmax, dn = zi > P.zmin;
  double cup[8], cdn[8];
  double fu = 0.0, fd = 0.0;
  for (int e = 0; e < kb; ++e) {
    cup[e] = beh_stat(S.bty[e], 1.0, zc, nb, zs, nh, ne, nl, P.brange, P.bsimmean);
    cdn[e] = beh_stat(S.bty[e], -1.0, zc, nb, zs, nh, ne, nl, P.brange, P.bsimmean);
    fu = __dadd_rn(fu, __dmul_rn(S.thb[e], cup[e]));
    fd = __dadd_rn(fd, __dmul_rn(S.thb[e], cdn[e]));
  }
  double mx = 0.0;
  if (up && fu > mx) mx = fu;
  if (dn && fd > mx) mx = fd;
  double pd = dn ? exp(__dsub_rn(fd, mx)) : 0.0;
  double p0 = exp(-mx);
  double pu = up ? exp(__dsub_rn(fu, mx)) : 0.0;
  const double ps = __dadd_rn(__dadd_rn(pd, p0), pu);
  pd = __ddiv_rn(pd, ps);
  p0 = __ddiv_rn(p0, ps);
  pu = __ddiv_rn(pu, ps);
  const double uc = unif01(r3);
  const int d = uc < pd ? -1 : (uc < __dadd_rn(pd, p0) ? 0 : 1);
  for (int e = 0; e < kb; ++e) {
    double s = d == 1 ? cup[e] : (d == -1 ? cdn[e] : 0.0);
    if (up) s = __dsub_rn(s, __dmul_rn(pu, cup[e]));
    if (dn) s = __dsub_rn(s, __dmul_rn(pd, cdn[e]));
    S.bsc[e] = __dadd_rn(S.bsc[e], s);
  }
  if (d != 0) {
    if (P.bkdist[i]) {
      const long long z0 = P.z0[i];
      long long a = (long long)(zi + d) - z0, b = (long long)zi - z0;
      *bdist += (a < 0 ? -a : a) - (b < 0 ? -b : b);
    }
    S.z[i] = zi + d;
  }
  return d;
}

// Non-basic rate draw (src/libcusna_saom_cpu.cpp:170-193). The actor rates are
// computed in parallel; lane 0 then forms S0, the rate-score sums and the focal
// actor in the reference's sequential order. Returns the focal actor, or -1
// when an unconditional period ends.
static __device__ int rate_draw(const Team &T, const DevProblem &P, const Slice &S, const uint32_t rr[4],
                         double lam, double &t, double &rho) {
  const int n = P.n, nr = P.nrate;
  for (int idx = T.tl; idx < P.nact; idx += T.L) {
    const int a2 = P.act[idx];
    double s = 0.0;
    for (int q = 0; q < nr; ++q) {
      const int rk = S.rkind[q];
      const double u = rk == 0 ? P.ru[(size_t)q * n + a2]
                               : (rk == 1 ? (double)S.outdeg[a2] : (double)S.indeg[a2]);
      s = __dadd_rn(s, __dmul_rn(P.ralpha[q], u));
    }
    if (s > 30.0) s = 30.0; else if (s < -30.0) s = -30.0;
    S.crate[a2] = exp(s);
  }
  T.sync();
  int focal = -1;
  if (T.tl == 0) {
    double S0 = 0.0, rs[4] = {0.0, 0.0, 0.0, 0.0};
    for (int idx = 0; idx < P.nact; ++idx) {
      const int a2 = P.act[idx];
      const double cc = S.crate[a2];
      S0 = __dadd_rn(S0, cc);
      for (int q = 0; q < nr; ++q) {
        const int rk = S.rkind[q];
        const double u = rk == 0 ? P.ru[(size_t)q * n + a2]
                                 : (rk == 1 ? (double)S.outdeg[a2] : (double)S.indeg[a2]);
        rs[q] = __dadd_rn(rs[q], __dmul_rn(cc, u));
      }
    }
    const double tau = __ddiv_rn(-log(unif01(rr[0])), __dmul_rn(lam, S0));
    double tau_eff = tau;
    if (!P.cond && __dadd_rn(t, tau) > 1.0) tau_eff = __dsub_rn(1.0, t);
    rho = __dadd_rn(rho, __dmul_rn(tau_eff, S0));
    for (int q = 0; q < nr; ++q)
      S.rsc[q] = __dsub_rn(S.rsc[q], __dmul_rn(__dmul_rn(tau_eff, lam), rs[q]));
    t = __dadd_rn(t, tau);
    if (!P.cond && t > 1.0) {
      focal = -1;
    } else {
      const double tgt = __dmul_rn(unif01(rr[2]), S0);
      double acc = 0.0;
      focal = P.act[P.nact - 1];
      for (int idx = 0; idx < P.nact; ++idx) {
        acc = __dadd_rn(acc, S.crate[P.act[idx]]);
        if (acc >= tgt) { focal = P.act[idx]; break; }
      }
    }
    S.misc[0] = focal;
    ((double *)(S.misc + 2))[0] = t;
    ((double *)(S.misc + 4))[0] = rho;
  }
  T.sync();
  focal = S.misc[0];
  t = ((double *)(S.misc + 2))[0];
  rho = ((double *)(S.misc + 4))[0];
  T.sync();
  return focal;
}

// Best float32 Gumbel key b1 at alter j1 with its error bound e1, and the
// largest upper bound (key + its error bound) of every other alter. The
// float32 keys certify the choice when b1 - e1 > ub2.
struct KeyTop {
  float b1, e1, ub2;
  int j1;
};
// alters reach a lane in ascending j: a key equal to the best is not better
// (its upper bound then reaches b1, which sends the choice to float64). A NaN
// key or bound (float32 overflow, or non-finite inputs) certifies nothing: it
// raises ub2 to infinity, so the exact float64 keys decide.
__device__ __forceinline__ void keytop_add(KeyTop &t, float g, float E, int j) {
  if (g > t.b1) {
    t.ub2 = fmaxf(t.ub2, __fadd_rn(t.b1, t.e1));
    t.b1 = g;
    t.e1 = E;
    t.j1 = j;
  } else {
    const float u = __fadd_rn(g, E);
    t.ub2 = (u != u) ? INFINITY : fmaxf(t.ub2, u);
  }
}
__device__ __forceinline__ void keytop_merge(KeyTop &a, const KeyTop &c) {
  if (c.b1 > a.b1 || (c.b1 == a.b1 && c.j1 < a.j1)) {
    a.ub2 = fmaxf(fmaxf(a.ub2, c.ub2), __fadd_rn(a.b1, a.e1));
    a.b1 = c.b1;
    a.e1 = c.e1;
    a.j1 = c.j1;
  } else {
    a.ub2 = fmaxf(fmaxf(a.ub2, c.ub2), __fadd_rn(c.b1, c.e1));
  }
}
__device__ __forceinline__ KeyTop team_keytop(const Team &T, KeyTop x, double *red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    KeyTop y;
    y.b1 = __shfl_xor_sync(kFull, x.b1, o);
    y.e1 = __shfl_xor_sync(kFull, x.e1, o);
    y.ub2 = __shfl_xor_sync(kFull, x.ub2, o);
    y.j1 = __shfl_xor_sync(kFull, x.j1, o);
    keytop_merge(x, y);
  }
  if (T.G == 1) return x;
  float *rb = (float *)red;          // 3 floats per warp
  int *rj = (int *)(rb + 3 * T.G);   // 1 int per warp
  T.sync();
  if (T.lane == 0) {
    rb[3 * T.warp] = x.b1;
    rb[3 * T.warp + 1] = x.e1;
    rb[3 * T.warp + 2] = x.ub2;
    rj[T.warp] = x.j1;
  }
  T.sync();
  KeyTop a{rb[0], rb[1], rb[2], rj[0]};
  for (int w = 1; w < T.G; ++w) keytop_merge(a, KeyTop{rb[3 * w], rb[3 * w + 1], rb[3 * w + 2], rj[w]});
  return a;
}

__device__ __forceinline__ bool is_nan64(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  return ((b >> 52) & 0x7FF) == 0x7FF && (b & 0xFFFFFFFFFFFFFull) != 0;
}

// The score sums are formed per alter group: the 32-alter blocks b (alter j
// in block j >> 5, on lane j & 31) fall into nsb groups, block b into group
// b mod nsb, with nsb fixed by n alone. A team of G warps takes groups g,
// g+G, ...; each group costs one warp reduction, so networks of up to 16
// blocks use at most four groups (up to four blocks each; teams of up to four
// warps share them), and larger ones a multiple of 4 with up to two blocks per
// group (shared evenly by teams of up to 16 warps). A lane adds its alters of a group in ascending
// block order into double-float accumulators, one warp reduction per group
// follows, and the group records are combined in group order: every sum's
// order depends on n and j only, never on the team size.
__host__ __device__ __forceinline__ int lse_groups(int nb) {
  // up to 16 blocks: about four blocks per group, at least two groups (so a
  // team of two warps shares the pass); beyond: about two blocks per group
  if (nb <= 16) return nb < 4 ? nb : 4;
  const int g = 4 * ((nb + 7) / 8);
  return g < nb ? g : nb;
}

// Adds one alter's score quantities to the lane's accumulators, held as
// packed pairs of quantities (quantities 2x and 2x+1 in H[x], L[x]):
// quantity 0 the weight w = exp(f_j) relative to the "no change" alter
// (whose predictor is 0), quantity 1+e the product w * d_e (not for the "no
// change" alter). Every product is a Dekker product of the weight's pair with
// d_e's pair, added with TwoSum, two quantities per instruction. LOMASK: bit
// e set when d_e may have a double-float remainder (integer counts have none).
// first (uniform over the warp): the accumulators are still zero, so the
// products are stored as they are (what TwoSum onto zero would give, bit for
// bit).
template <int V, unsigned LOMASK>
__device__ __forceinline__ void lse_accumulate(float2 (&H)[(V + 1) / 2], float2 (&L)[(V + 1) / 2],
                                               float wh, float wl, const float *d32,
                                               const float *d32lo, bool weighted, int k,
                                               bool first) {
  const float2 w2 = make_float2(wh, wh), wl2 = make_float2(wl, wl);
#pragma unroll
  for (int x = 0; x < (V + 1) / 2; ++x) {
    const int qa = 2 * x, qb = 2 * x + 1;
    // d of quantity q: 1 for the weight itself, d_{q-1} for a product, 0
    // beyond the model's effects or for the "no change" alter
    const bool ua = qa == 0 || (weighted && qa - 1 < k), ub = qb < V && weighted && qb - 1 < k;
    const float da = qa == 0 ? 1.f : (ua ? d32[qa - 1] : 0.f);
    const float db = ub ? d32[qb - 1] : 0.f;
    const float2 d2 = make_float2(da, db);
    const float2 p = __fmul2_rn(w2, d2);
    float2 pl = __ffma2_rn(wl2, d2, __ffma2_rn(w2, d2, make_float2(-p.x, -p.y)));
    const bool la = qa > 0 && ((LOMASK >> (qa - 1)) & 1u), lb = (LOMASK >> (qb - 1)) & 1u;
    if (la || lb) {
      const float2 dl2 =
          make_float2(la && ua ? d32lo[qa - 1] : 0.f, lb && ub ? d32lo[qb - 1] : 0.f);
      pl = __ffma2_rn(w2, dl2, pl);
    }
    if (first) {
      H[x] = p;
      L[x] = pl;
    } else {
      ff_add2(H[x], L[x], p, pl);
    }
  }
}

// The group sums of the warp's lanes reduced by the fixed recursive-halving
// warp reduction; the lane holding quantity q stores it as the pair
// rec[2q], rec[2q+1].
template <int V>
__device__ __forceinline__ void lse_store(float *rec, float (&h)[V], float (&l)[V], int k,
                                          int lane) {
  bool writer;
  const int q = warp_multi_sum_ff<V>(h, l, lane, &writer);
  if (writer && q <= k) {
    rec[2 * q] = h[0];
    rec[2 * q + 1] = l[0];
  }
}

// The group records combined by one warp of the team: lane q adds quantity
// q's records in group order (double-float). Quantity q lands in
// S.red[32G + q] as a double, past the warp slots the team reductions use.
__device__ __forceinline__ void combine_groups(const Team &T, const Slice &S, int nsb, int k) {
  const int q = T.lane;
  if (q > k) return;
  const float *rec = S.blk + 2 * q;
  const size_t stride = 2 * (size_t)(k + 1);
  float h = rec[0], l = rec[1];
  for (int g = 1; g < nsb; ++g) ff_add(h, l, rec[g * stride], rec[g * stride + 1]);
  S.red[32 * T.G + q] = __dadd_rn((double)h, (double)l);
}

// The float64 predictor f_j of alter j (and its change statistics in d): the
// reference's value bit for bit (effect order, separately rounded products
// and sums).
template <bool MULTI>
__device__ __forceinline__ double f64_of(const DevProblem &P, const Slice &S, const StepCtx &X,
                                         int j, double *d, int net) {
  const int n = P.n, i = X.i;
  const int aij = bit_of(S.rowsT, n, i, j), aji = bit_of(S.colsT, n, i, j);
  (void)net;
#if defined(CUSNA_JIT_SPEC)
  return jit_change_stats<true>(P, S, X, j, aij, aji, d);
#elif defined(CUSNA_JIT_MULTI)
  return jit_change_stats<true>(net, P, S, X, j, aij, aji, d);
#else
  return change_stats<true, MULTI>(P, S, X, j, aij, aji, d);
#endif
}

// The score sums in float64 as the reference forms them
// (src/libcusna_saom_cpu.cpp:271-274): lmax = the largest predictor of a
// permitted alter (at least the "no change" alter's 0), then sume = sum of
// exp(f_j - lmax) and wsum_e = sum of exp(f_j - lmax) d_je over permitted
// alters, every f_j and d_je the reference's float64 value. The sums run per
// 32-alter block (fixed warp reduction) and over blocks in order, so they do
// not depend on the team size; results land in S.red[32G + q]. Used when a
// predictor leaves the double-float exponential's range or is not finite,
// and at every ministep under F_LSE64. Called by the whole team.
template <bool MULTI, int VQ>
static __device__ __noinline__ void lse_float64(const Team &T, const DevProblem &P,
                                                const Slice &S, const StepCtx &X, double *d,
                                                int net) {
  constexpr int V = VQ <= 8 ? 8 : (VQ <= 16 ? 16 : 32);  // warp_multi_sum's power of two
  const int n = P.n, k = P.k, L = T.L, i = X.i;
  long long mk = dkey(0.0);
  for (int j = T.tl; j < n; j += L) {
    if (j == i || !((S.okbits[j >> 5] >> (j & 31)) & 1u)) continue;
    const double f = f64_of<MULTI>(P, S, X, j, d, net);
    if (!is_nan64(f)) {
      const long long kf = dkey(f);
      mk = kf > mk ? kf : mk;
    }
  }
  const double lmax = dunkey(team_max_ll(T, mk, S.red));
  double *rec64 = (double *)S.blk;
  for (int jb = 32 * T.warp; jb < n; jb += L) {
    const int j = jb + T.lane;
    double w = 0.0;
    bool weighted = false;
    if (j < n && ((S.okbits[j >> 5] >> (j & 31)) & 1u)) {
      if (j == i) {
        w = exp(-lmax);
      } else {
        w = exp(__dsub_rn(f64_of<MULTI>(P, S, X, j, d, net), lmax));
        weighted = true;
      }
    }
    double v[V];
    v[0] = w;
#pragma unroll
    for (int q = 1; q < V; ++q) v[q] = (weighted && q - 1 < k) ? __dmul_rn(w, d[q - 1]) : 0.0;
    const int q = warp_multi_sum<V>(v, T.lane);
    const bool writer = (V >= 32) || ((T.lane & ((32 / V) - 1)) == 0);
    if (writer && q <= k) rec64[(size_t)(jb >> 5) * (k + 1) + q] = v[0];
  }
  T.sync();
  if (T.warp == 0) {
    const int nb = (n + 31) >> 5;
    double v[V];
#pragma unroll
    for (int q = 0; q < V; ++q) v[q] = 0.0;
    for (int b = T.lane; b < nb; b += 32)
#pragma unroll
      for (int q = 0; q < V; ++q)
        if (q <= k) v[q] = __dadd_rn(v[q], rec64[(size_t)b * (k + 1) + q]);
    const int q = warp_multi_sum<V>(v, T.lane);
    const bool writer = (V >= 32) || ((T.lane & ((32 / V) - 1)) == 0);
    if (writer && q <= k) S.red[32 * T.G + q] = v[0];
  }
}

// Compile-time width of the score sums (the k + 1 quantities in a specialised
// build; the library build rounds k + 1 up to a power of two) and the mask of
// effects whose change statistic can have a double-float remainder (LOMASK).
#if defined(CUSNA_JIT_SPEC)
#define CUSNA_LSE_V (CUSNA_JIT_K + 1)
#define CUSNA_LSE_LOMASK CUSNA_JIT_LOMASK
#else
#define CUSNA_LSE_LOMASK 0xFFFFFFFFu
#endif

// Per-thread scratch of one alter's change statistics in the pass over the
// alters: the model's k in the specialised build, the capacity otherwise.
#if defined(CUSNA_JIT_K)
constexpr int kScratchK = CUSNA_JIT_K;
#else
constexpr int kScratchK = kMaxEff;
#endif

// The pass over the alters of one network ministep (see net_choice): per
// alter the change statistics, the float32 Gumbel key with its error bound
// (into *best and S.gbuf), the permitted-alter bits (S.okbits) and, when the
// double-float score sums are wanted (fast_sums), the alter's score
// quantities into its lane's group accumulators; each group's sums end in its
// record in S.blk. Returns true on lanes that saw a predictor outside the
// double-float exponential's range.
template <bool MULTI, bool VALID, int V>
__device__ __forceinline__ bool alter_pass(const Team &T, const DevProblem &P, const Slice &S,
                                           const StepCtx &X, long long ms, uint32_t chain,
                                           KeyTop &best, bool fast_sums, int net) {
  const int n = P.n, k = P.k, i = X.i;
  (void)net;
  const float ecoef = (float)(k + 10) * 5.9604644775390625e-8f;
  const int nb = (n + 31) >> 5, nsb = lse_groups(nb);
#ifdef CUSNA_JIT_K
  constexpr int KS = CUSNA_JIT_K;
#else
  const int KS = k;
#endif
  bool wide = false;
  // without score sums the blocks are simply dealt to the warps in turn
  const int ng = fast_sums ? nsb : nb;
  for (int g = T.warp; g < ng; g += T.G) {
    float2 AH[(V + 1) / 2], AL[(V + 1) / 2];
#pragma unroll
    for (int x = 0; x < (V + 1) / 2; ++x) {
      AH[x] = make_float2(0.f, 0.f);
      AL[x] = make_float2(0.f, 0.f);
    }
    for (int b = g; b < nb; b += ng) {
      const int j = (b << 5) + T.lane;
      // the alter's float32 change statistics and their double-float
      // remainders: in the specialised build every index is a constant, so
      // these stay in registers
      float d32[kScratchK], d32lo[kScratchK];
      bool ok = false, stay = false;
      float f = 0.f;
      float2 fx = make_float2(0.f, 0.f);
      if (j < n) {
        const int aij = bit_of(S.rowsT, n, i, j);
        float ub = -INFINITY;
        stay = j == i;
        ok = stay || (bit_of(P.permT, n, i, j) && !(P.maxdeg > 0 && aij == 0 && X.od_i >= P.maxdeg));
        if (ok) {
          float absf = 0.f;
#if defined(CUSNA_JIT_SPEC)
          // the effect plan compiled in (saom_jit.cu): the same float32 values
          if (!stay)
            f = jit_change_stats32(P, S, X, j, aij, bit_of(S.colsT, n, i, j), d32, d32lo, &absf,
                                   &fx);
#elif defined(CUSNA_JIT_MULTI)
          if (!stay)
            f = jit_change_stats32(net, P, S, X, j, aij, bit_of(S.colsT, n, i, j), d32, d32lo,
                                   &absf, &fx);
#else
          if (!stay)
            f = change_stats32<MULTI>(P, S, X, j, aij, bit_of(S.colsT, n, i, j), d32, d32lo,
                                      &absf, &fx);
#endif
          const float gk = __fsub_rn(f, loglog_est(alter_word<VALID>(P, S, ms, chain, j)));
          const float E = __fadd_rn(__fmul_rn(ecoef, absf), 6e-6f);
          ub = __fadd_rn(gk, E);
          keytop_add(best, gk, E, j);
        }
        S.gbuf[j] = ub;
      }
      const uint32_t okb = __ballot_sync(kFull, ok);
      if (T.lane == 0) S.okbits[b] = okb;
      // the group's first block initialises every lane's accumulators (a lane
      // without a permitted alter there stores zeros); later blocks add the
      // permitted alters
      const bool first = b == g;
      if (fast_sums && (ok || first)) {
        float wh = ok ? 1.f : 0.f, wl = 0.f;  // the "no change" alter: exp(0)
        if (ok && !stay) {
          if (fabsf(f) <= kFFExpMax) {
            exp_ff(fx.x, fx.y, S.etab, wh, wl);
          } else {  // also NaN
            wide = true;
            wh = 0.f;
          }
        }
        lse_accumulate<V, CUSNA_LSE_LOMASK>(AH, AL, wh, wl, d32, d32lo, ok && !stay, KS, first);
      }
    }
    if (fast_sums) {
      float ah[V], al[V];
#pragma unroll
      for (int q = 0; q < V; ++q) {
        ah[q] = (q & 1) ? AH[q >> 1].y : AH[q >> 1].x;
        al[q] = (q & 1) ? AL[q >> 1].y : AL[q >> 1].x;
      }
      lse_store<V>(S.blk + (size_t)g * 2 * (k + 1), ah, al, KS, T.lane);
    }
  }
  return wide;
}

// One network ministep of focal actor i on the network of slice S, up to the
// choice: change statistics, float32 keys and the double-float score sums, the
// certified or exact float64 choice, and the chosen alter's float64 change
// statistics in S.dstar. Returns j*. The score sums are left in S.red[32G + q]
// (float64) for the score update. d (float64) is per-thread scratch of k
// values.
// MULTI: the network is one of a multi-network problem's, whose network w has
// its rows at rows0 + w*net_stride words (cross effects read them).
// VALID: validation mode (caller-supplied words in place of Philox).
template <bool MULTI, bool VALID = false>
__device__ __forceinline__ int net_choice(const Team &T, const DevProblem &P, const Slice &S,
                                          int i, long long ms, uint32_t chain, double *d,
                                          const uint32_t *rows0 = nullptr,
                                          size_t net_stride = 0, int net = 0) {
  const int n = P.n, W = P.W, k = P.k, L = T.L;
  (void)net;
  step_helpers(T, P, S, i);
  StepCtx X;
  X.i = i;
  X.od_i = S.outdeg[i];
  X.id_i = S.indeg[i];
  X.rdeg_i = 0;
  if (P.flags & F_NEED_RDEG)
    for (int w = 0; w < W; ++w) X.rdeg_i += __popc(S.rowsT[w * n + i] & S.colsT[w * n + i]);
  X.zvi = (P.flags & F_HAS_Z) ? __dsub_rn((double)S.z[i], P.zbar) : 0.0;
  X.rows0 = rows0;
  X.net_stride = net_stride;
  if (P.flags & F_HAS_STEP) {
    step_values(T, P, S, X);
    T.sync();
  }

  // ---- one pass over the alters (alter_pass) -------------------------------
  // Lane by lane: integer change statistics, the
  // float32 predictor f32_j (change_stats32) and the float32 Gumbel key
  // g_j = f32_j - loglog_est(u_j) with u_j from the reference's counters
  // (msteps, chain, 1, j). The key is within
  //   E_j = (k + 10) 2^-24 absf_j + 6e-6
  // of the float64 key f_j - log(-log u_j): (k + 8) u absf_j for f32_j, 4e-6
  // for loglog_est and u (absf_j + 23) for the subtraction (|f32_j| <= absf_j,
  // |log(-log u)| < 23). gbuf[j] keeps the upper bound g_j + E_j.
  // The score sums are formed per group of alters (lse_groups; the grouping
  // and every order of addition depend on n and j only) in double-float
  // arithmetic: the predictor as a double-float pair (within ~2^-47 absf_j of
  // the reference's float64 f_j), its exponential relative to the "no change"
  // alter (exp_ff, relative error ~2e-14), and the weighted change
  // statistics; the groups are combined after the choice in group order
  // (combine_groups), so the scores do not depend on the launch shape. A
  // predictor outside [-60, 60] (or not finite) sends the ministep's sums to
  // the float64 path (lse_float64), as does F_LSE64. Without requested scores
  // (F_NO_SCORES) no sums are formed.
  KeyTop best{-INFINITY, 0.f, -INFINITY, 0x7FFFFFFF};
  const bool want_sums = (P.flags & F_NO_SCORES) == 0;
  const bool fast_sums = want_sums && (P.flags & F_LSE64) == 0;
#ifdef CUSNA_LSE_V
  const bool wide = alter_pass<MULTI, VALID, CUSNA_LSE_V>(T, P, S, X, ms, chain, best,
                                                          fast_sums, net);
#else
  bool wide;
  if (k + 1 <= 8)
    wide = alter_pass<MULTI, VALID, 8>(T, P, S, X, ms, chain, best, fast_sums, net);
  else if (k + 1 <= 16)
    wide = alter_pass<MULTI, VALID, 16>(T, P, S, X, ms, chain, best, fast_sums, net);
  else
    wide = alter_pass<MULTI, VALID, 32>(T, P, S, X, ms, chain, best, fast_sums, net);
#endif
  if (__any_sync(kFull, wide) && T.lane == 0) S.misc[12] = (int)ms;
  T.sync();
  const KeyTop top = team_keytop(T, best, S.red + 26 * T.G);

  // ---- the chosen alter ---------------------------------------------------
  // The float32 keys decide when the best key's lower bound exceeds every
  // other alter's upper bound. Otherwise every permitted alter whose upper
  // bound is not below that lower bound (a NaN on either side counts as
  // reaching it) gets its exact float64 key (the reference's
  // f_j - log(-log u_j)) and those decide, ties to the smaller j. The "no
  // change" alter always has a finite key, so a choice always exists.
  int jstar;
  const float lb = __fsub_rn(top.b1, top.e1);
  if (lb > top.ub2) {
    jstar = top.j1;
  } else {
    long long bk = dkey(-1e300);
    int bj = 0x7FFFFFFF;
    for (int j = T.tl; j < n; j += L) {
      const bool okj = (S.okbits[j >> 5] >> (j & 31)) & 1u;
      if (okj && !(S.gbuf[j] < lb)) {
        const double f = j != i ? f64_of<MULTI>(P, S, X, j, d, net) : 0.0;
        const double g = __dsub_rn(f, log(-log(unif01(alter_word<VALID>(P, S, ms, chain, j)))));
        if (is_nan64(g)) continue;
        const long long kg = dkey(g);
        if (kg > bk || (kg == bk && j < bj)) { bk = kg; bj = j; }
      }
    }
    jstar = team_argmax(T, bk, bj, S.red + 29 * T.G);
  }
  // never an index outside the network, whatever the inputs
  if ((unsigned)jstar >= (unsigned)n) jstar = i;

  // the score sums: normally the block records combined into quantity q (0:
  // sum of weights, 1+e: weighted sum of d_e), by a warp other than the
  // chosen alter's owner, which meanwhile forms the chosen alter's float64
  // statistics; on the float64 path, the whole team
  const bool sums64 = want_sums && (!fast_sums || S.misc[12] == (int)ms);
  if (sums64) {
#ifdef CUSNA_LSE_V
    lse_float64<MULTI, CUSNA_LSE_V>(T, P, S, X, d, net);
#else
    if (k + 1 <= 8) lse_float64<MULTI, 8>(T, P, S, X, d, net);
    else if (k + 1 <= 16) lse_float64<MULTI, 16>(T, P, S, X, d, net);
    else lse_float64<MULTI, 32>(T, P, S, X, d, net);
#endif
  } else if (fast_sums) {
    const int owner_warp = (jstar % L) >> 5;
    if (T.warp == (T.G > 1 ? (owner_warp + 1) % T.G : 0)) {
      const int nsb = lse_groups((n + 31) >> 5);
#ifdef CUSNA_JIT_K
      combine_groups(T, S, nsb, CUSNA_JIT_K);
#else
      combine_groups(T, S, nsb, k);
#endif
    }
  }

  // ---- the chosen alter's change statistics, in float64 as the reference
  // adds them (for the score update only)
  if (want_sums && T.tl == jstar % L) {
    if (jstar == i) {
      for (int e = 0; e < k; ++e) S.dstar[e] = 0.0;
    } else {
      const int aij = bit_of(S.rowsT, n, i, jstar);
      const int aji = bit_of(S.colsT, n, i, jstar);
#if defined(CUSNA_JIT_SPEC)
      jit_change_stats<false>(P, S, X, jstar, aij, aji, d);
#elif defined(CUSNA_JIT_MULTI)
      jit_change_stats<false>(net, P, S, X, jstar, aij, aji, d);
#else
      change_stats<false, MULTI>(P, S, X, jstar, aij, aji, d);
#endif
      for (int e = 0; e < k; ++e) S.dstar[e] = d[e];
    }
  }
  return jstar;
}

// Validation trace record of ministep ms (validation mode only): (step,
// focal actor, choice, change of the distance); the choice is the chosen alter
// of a network ministep, or -(d + 2) for a behaviour step d.
template <bool VALID>
__device__ __forceinline__ void trace_put(const DevProblem &P, int c, long long ms, int actor,
                                          int choice, long long delta) {
  if (!VALID || !P.trace || ms >= P.trace_cap) return;
  int *t = P.trace + ((size_t)c * P.trace_cap + (size_t)ms) * 4;
  t[0] = (int)ms;
  t[1] = actor;
  t[2] = choice;
  t[3] = (int)delta;
}

// One chain: the ministep loop and the chain's outputs.
template <bool VALID>
static __device__ void run_chain(const Team &T, const DevProblem &P, const Slice &S, int c) {
  const int n = P.n, k = P.k;
  const uint32_t chain = P.chain_offset + (uint32_t)c;
  chain_init(T, P, S, c);

  const double lam = (double)P.lam[c * P.prow];
  const double lamb = P.lamb ? (double)P.lamb[c * P.prow] : 0.0;
  // the reference's constant-rate expressions (src/libcusna_saom_cpu.cpp:195,197)
  const double den = __dmul_rn((double)P.nact, __dadd_rn(lam, lamb));
  const double pnet = __ddiv_rn(lam, __dadd_rn(lam, lamb));
  long long dist = 0, bdist = 0, ms = 0, msb = 0;
  double t = 0.0, rho = 0.0;
  double d[kMaxEff];

  for (;;) {
    int i;
    bool is_net;
    uint32_t r3;
    if (P.nrate > 0) {
      uint32_t rr[4];
      step_words<VALID>(P, S, ms, chain, rr);
      i = rate_draw(T, P, S, rr, lam, t, rho);
      if (i < 0) break;
      is_net = true;
      r3 = rr[3];
    } else {
      // constant rate (:195-199). The draws of 32 ministeps are formed at
      // once, one per lane of warp 0 (they depend only on the counters), and
      // the time is accumulated in order, so every value equals the reference's.
      const int slot = (int)(ms & 31);
      if (slot == 0) {
        if (T.warp == 0) {
          uint32_t rr[4];
          step_words<VALID>(P, S, ms + T.lane, chain, rr);
          S.rtau[T.lane] = __ddiv_rn(-log(unif01(rr[0])), den);
          S.rnet[T.lane] = (P.kb == 0 || unif01(rr[1]) < pnet) ? 1 : 0;
          long long idx = (long long)__dmul_rn(unif01(rr[2]), (double)P.nact);
          if (idx >= P.nact) idx = P.nact - 1;
          S.rfocal[T.lane] = P.act[idx];
          S.rr3[T.lane] = rr[3];
        }
        T.sync();
      }
      t = __dadd_rn(t, S.rtau[slot]);
      if (!P.cond && t > 1.0) break;
      is_net = S.rnet[slot] != 0;
      i = S.rfocal[slot];
      r3 = S.rr3[slot];
    }

    if (!is_net) {
      if (T.tl == 0) {
        const long long bd0 = bdist;
        const int dz = beh_step(P, S, i, r3, &bdist);
        trace_put<VALID>(P, c, ms, i, -(dz + 2), bdist - bd0);
      }
      T.sync();
      ++msb;
      ++ms;
      if (P.cond && dist >= P.target_dist) break;
      if (ms >= kMaxSteps) break;
      continue;
    }

    const int jstar = net_choice<false, VALID>(T, P, S, i, ms, chain, d);
    const int aij_star = bit_of(S.rowsT, n, i, jstar);
    T.sync();
    if (!(P.flags & F_NO_SCORES) && T.tl < k) {
      const int e = T.tl;
      const double s0 = S.red[32 * T.G], se = S.red[32 * T.G + 1 + e];
      S.sc[e] = __dadd_rn(S.sc[e], __dsub_rn(S.dstar[e], __ddiv_rn(se, s0)));
    }
    const long long dist0 = dist;
    ++ms;
    if (jstar != i) {
      const int j = jstar;
      const long long chg = P.symflag ? 2 : 1;
      if (bit_of(P.kdistT, n, i, j))
        dist += (aij_star == bit_of(P.x0T, n, i, j)) ? chg : -chg;
      if (T.tl == 0) {
        const int dl = 1 - 2 * aij_star;
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
    }
    if (T.tl == 0) trace_put<VALID>(P, c, ms - 1, i, jstar, dist - dist0);
    if (P.nrate > 0 && T.tl == 0) {
      for (int q = 0; q < P.nrate; ++q) {
        const int rk = S.rkind[q];
        const double u = rk == 0 ? P.ru[(size_t)q * n + i]
                                 : (rk == 1 ? (double)S.outdeg[i] : (double)S.indeg[i]);
        S.rsc[q] = __dadd_rn(S.rsc[q], u);
      }
    }
    T.sync();
    if (P.cond && dist >= P.target_dist) break;
    if (ms >= kMaxSteps) break;
  }

  chain_finish(T, P, S, c, dist, bdist, ms, msb, t, rho, lam, lamb);
}

}  // namespace cusna
