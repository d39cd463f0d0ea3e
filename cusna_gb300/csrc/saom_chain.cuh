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
    S.th[e] = (double)P.theta[(size_t)c * P.prow * k + e];
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
  for (int x = T.tl; x < 64; x += L) S.exptab[x] = kExp2Frac64[x];
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

// Behaviour ministep (src/libcusna_saom_cpu.cpp:202-227), run by the team's
// lane 0 in the reference's order. Returns nothing; updates z, bsc, *bdist.
__device__ void beh_step(const DevProblem &P, const Slice &S, int i, uint32_t r3,
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
}

// Non-basic rate draw (src/libcusna_saom_cpu.cpp:170-193). The actor rates are
// computed in parallel; lane 0 then forms S0, the rate-score sums and the focal
// actor in the reference's sequential order. Returns the focal actor, or -1
// when an unconditional period ends.
__device__ int rate_draw(const Team &T, const DevProblem &P, const Slice &S, const uint32_t rr[4],
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

// Top-2 of the float32 Gumbel estimates: best value b1 at alter j1 (ties to
// the smaller j) and the largest value b2 of every other alter.
struct Top2 {
  float b1, b2;
  int j1;
};
__device__ __forceinline__ void top2_merge(Top2 &a, const Top2 &c) {
  if (c.b1 > a.b1 || (c.b1 == a.b1 && c.j1 < a.j1)) {
    a.b2 = fmaxf(c.b2, a.b1);
    a.b1 = c.b1;
    a.j1 = c.j1;
  } else {
    a.b2 = fmaxf(a.b2, c.b1);
  }
}
__device__ __forceinline__ Top2 team_top2(const Team &T, Top2 x, double *red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    Top2 y;
    y.b1 = __shfl_xor_sync(kFull, x.b1, o);
    y.b2 = __shfl_xor_sync(kFull, x.b2, o);
    y.j1 = __shfl_xor_sync(kFull, x.j1, o);
    top2_merge(x, y);
  }
  if (T.G == 1) return x;
  float *rb = (float *)red;
  int *rj = (int *)(red + T.G);
  T.sync();
  if (T.lane == 0) { rb[2 * T.warp] = x.b1; rb[2 * T.warp + 1] = x.b2; rj[T.warp] = x.j1; }
  T.sync();
  Top2 a{rb[0], rb[1], rj[0]};
  for (int w = 1; w < T.G; ++w) top2_merge(a, Top2{rb[2 * w], rb[2 * w + 1], rj[w]});
  return a;
}

// float32 image of y (finite, <= 0) truncated toward zero: relative error
// below 2^-23, formed on the integer pipes. Values below -1e4 (never in the
// Gumbel shortlist, whose members have y >= -26.1) become -inf.
__device__ __forceinline__ float shortlist_f32(double y) {
  if (!(y > -1e4)) return -INFINITY;
  const unsigned long long b = (unsigned long long)__double_as_longlong(y);
  const int fe = (int)((b >> 52) & 0x7FF) - 1023 + 127;
  if (fe <= 0) return 0.0f;
  const unsigned m = (unsigned)((b >> 29) & 0x7FFFFFu);
  return __uint_as_float((unsigned)((b >> 63) << 31) | ((unsigned)fe << 23) | m);
}

__device__ __forceinline__ bool is_nan64(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  return ((b >> 52) & 0x7FF) == 0x7FF && (b & 0xFFFFFFFFFFFFFull) != 0;
}

// Team sums of sume and wsum[0..k-1]: warp recursive halving over V >= k+1
// values, then one slot per (quantity, warp) in red[q*G + warp].
template <int V>
__device__ __forceinline__ void lse_reduce(const Team &T, const Slice &S, double sume,
                                           const double *wsum, int k) {
  double v[V];
  v[0] = sume;
#pragma unroll
  for (int q = 1; q < V; ++q) v[q] = (q - 1 < k) ? wsum[q - 1] : 0.0;
  const int q = warp_multi_sum<V>(v, T.lane);
  const bool writer = (V >= 32) || ((T.lane & ((32 / V) - 1)) == 0);
  if (writer && q <= k) S.red[q * T.G + T.warp] = v[0];
}

// One chain: the ministep loop and the chain's outputs.
__device__ void run_chain(const Team &T, const DevProblem &P, const Slice &S, int c) {
  const int n = P.n, W = P.W, k = P.k, L = T.L;
  const uint32_t chain = P.chain_offset + (uint32_t)c;
  chain_init(T, P, S, c);

  const double lam = (double)P.lam[c * P.prow];
  const double lamb = P.lamb ? (double)P.lamb[c * P.prow] : 0.0;
  // the reference's constant-rate expressions (src/libcusna_saom_cpu.cpp:195,197)
  const double den = __dmul_rn((double)P.nact, __dadd_rn(lam, lamb));
  const double pnet = __ddiv_rn(lam, __dadd_rn(lam, lamb));
  long long dist = 0, bdist = 0, ms = 0, msb = 0;
  double t = 0.0, rho = 0.0;
  double d[24], wsum[24], dbest[24];

  for (;;) {
    int i;
    bool is_net;
    uint32_t r3;
    if (P.nrate > 0) {
      uint32_t rr[4];
      philox10((uint32_t)ms, chain, 0u, 0u, P.k0, P.k1, rr);
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
          philox10((uint32_t)(ms + T.lane), chain, 0u, 0u, P.k0, P.k1, rr);
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
      if (T.tl == 0) beh_step(P, S, i, r3, &bdist);
      T.sync();
      ++msb;
      ++ms;
      if (P.cond && dist >= P.target_dist) break;
      if (ms >= kMaxSteps) break;
      continue;
    }

    step_helpers(T, P, S, i);
    StepCtx X;
    X.i = i;
    X.od_i = S.outdeg[i];
    X.id_i = S.indeg[i];
    X.rdeg_i = 0;
    if (P.flags & F_NEED_RDEG)
      for (int w = 0; w < W; ++w) X.rdeg_i += __popc(S.rowsT[w * n + i] & S.colsT[w * n + i]);
    X.zvi = (P.flags & F_HAS_Z) ? __dsub_rn((double)S.z[i], P.zbar) : 0.0;
    if (P.flags & F_HAS_STEP) {
      step_values(T, P, S, X);
      T.sync();
    }

    // ---- pass 1: change statistics, f_j, lmax ------------------------------
    long long kmax = dkey(-1e30);
    for (int jb = 32 * T.warp; jb < n; jb += L) {
      const int j = jb + T.lane;
      bool ok = false;
      if (j < n) {
        const int aij = bit_of(S.rowsT, n, i, j);
        double f = 0.0;
        if (j == i) {
          ok = true;
        } else {
          ok = bit_of(P.permT, n, i, j) &&
               !(P.maxdeg > 0 && aij == 0 && X.od_i >= P.maxdeg);
          if (ok) {
            const int aji = bit_of(S.colsT, n, i, j);
            f = change_stats<true>(P, S, X, j, aij, aji, d);
          }
        }
        S.fbuf[j] = f;
        // a NaN predictor never raises the maximum (the reference compares
        // f > lmax) and is never chosen (its Gumbel key compares false)
        if (ok && !is_nan64(f)) {
          const long long kf = dkey(f);
          kmax = kf > kmax ? kf : kmax;
        }
      }
      const uint32_t okb = __ballot_sync(kFull, ok);
      if (T.lane == 0) S.okbits[jb >> 5] = okb;
    }
    const double lmax = dunkey(team_max_ll(T, kmax, S.red));
    T.sync();

    // ---- pass 2: log-sum-exp sums and float32 Gumbel estimates --------------
    // The estimate of g_j - lmax, shortlist_f32(f_j - lmax) - loglog_est(u_j),
    // is within 2^-23*26.1 + 2.2e-6 + 2^-24*23 < 7e-6 of the float64 value for
    // every alter that can be the argmax (those have f_j - lmax >= -26.1, as
    // their key is at least the key of the lmax alter, >= -3.2).
    double sume = 0.0;
    for (int e = 0; e < k; ++e) wsum[e] = 0.0;
    Top2 best{-INFINITY, -INFINITY, 0x7FFFFFFF};
    for (int j = T.tl; j < n; j += L) {
      if (!((S.okbits[j >> 5] >> (j & 31)) & 1u)) {
        S.gbuf[j] = -INFINITY;
        continue;
      }
      const double y = __dsub_rn(S.fbuf[j], lmax);
      const double wj = exp_weight(y, S.exptab);
      sume = __dadd_rn(sume, wj);
      if (j != i) {
        const int aij = bit_of(S.rowsT, n, i, j);
        const int aji = bit_of(S.colsT, n, i, j);
        change_stats<false>(P, S, X, j, aij, aji, d);
        for (int e = 0; e < k; ++e) wsum[e] = fma(wj, d[e], wsum[e]);
      }
      uint32_t ph[4];
      philox10((uint32_t)ms, chain, 1u, (uint32_t)j, P.k0, P.k1, ph);
      const float gt = shortlist_f32(y) - loglog_est(ph[0]);
      S.gbuf[j] = gt;
      if (gt > best.b1) {  // j ascending within a lane: ties keep the earlier j
        best.b2 = best.b1;
        best.b1 = gt;
        best.j1 = j;
        if (j != i)
          for (int e = 0; e < k; ++e) dbest[e] = d[e];
      } else {
        best.b2 = fmaxf(best.b2, gt);
      }
    }
    const int jsaved = best.j1;
    if (k + 1 <= 8) lse_reduce<8>(T, S, sume, wsum, k);
    else if (k + 1 <= 16) lse_reduce<16>(T, S, sume, wsum, k);
    else lse_reduce<32>(T, S, sume, wsum, k);
    const Top2 top = team_top2(T, best, S.red + 26 * T.G);

    // ---- the chosen alter ---------------------------------------------------
    // The float estimates decide unless the top two are within the window;
    // then the shortlist's exact float64 keys decide, ties to the smaller j.
    int jstar;
    if (top.b1 - top.b2 > kGumbelWindow) {
      jstar = top.j1;
    } else {
      long long bk = dkey(-1e300);
      int bj = 0x7FFFFFFF;
      const float thr = top.b1 - kGumbelWindow;
      for (int j = T.tl; j < n; j += L) {
        if (S.gbuf[j] >= thr) {
          uint32_t ph[4];
          philox10((uint32_t)ms, chain, 1u, (uint32_t)j, P.k0, P.k1, ph);
          const double g = __dsub_rn(S.fbuf[j], log(-log(unif01(ph[0]))));
          if (is_nan64(g)) continue;
          const long long kg = dkey(g);
          if (kg > bk || (kg == bk && j < bj)) { bk = kg; bj = j; }
        }
      }
      jstar = team_argmax(T, bk, bj, S.red + 29 * T.G);
    }

    // ---- score update (lane e updates effect e) and toggle ----------------
    if (T.tl == jstar % L) {
      if (jstar == i) {
        for (int e = 0; e < k; ++e) S.dstar[e] = 0.0;
      } else if (jsaved == jstar) {
        for (int e = 0; e < k; ++e) S.dstar[e] = dbest[e];
      } else {
        const int aij = bit_of(S.rowsT, n, i, jstar);
        const int aji = bit_of(S.colsT, n, i, jstar);
        change_stats<false>(P, S, X, jstar, aij, aji, d);
        for (int e = 0; e < k; ++e) S.dstar[e] = d[e];
      }
    }
    const int aij_star = bit_of(S.rowsT, n, i, jstar);
    T.sync();
    if (T.tl < k) {
      const int e = T.tl;
      double s0 = 0.0, se = 0.0;
      for (int w = 0; w < T.G; ++w) {
        s0 = __dadd_rn(s0, S.red[w]);
        se = __dadd_rn(se, S.red[(e + 1) * T.G + w]);
      }
      S.sc[e] = __dadd_rn(S.sc[e], __dsub_rn(S.dstar[e], __ddiv_rn(se, s0)));
    }
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
