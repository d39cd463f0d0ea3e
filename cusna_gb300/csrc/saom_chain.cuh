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
    S.th[e] = (double)P.theta[(size_t)c * k + e];
    S.sc[e] = 0.0;
    S.tid[e] = P.type_ids[e];
    S.ety[e] = P.etypes[e];
    S.dyn[e] = P.dyn[e];
    S.i0[e] = P.int0[e];
    S.i1[e] = P.int1[e];
    S.i2[e] = P.int2[e];
    S.p1[e] = P.p1[e];
    S.p2[e] = P.p2[e];
  }
  for (int e = T.tl; e < P.kb; e += L) {
    S.thb[e] = P.thetab ? (double)P.thetab[(size_t)c * P.kb + e] : 0.0;
    S.bsc[e] = 0.0;
    S.bty[e] = P.bty[e];
  }
  for (int q = T.tl; q < P.nrate; q += L) {
    S.rsc[q] = 0.0;
    S.rkind[q] = P.rkind[q];
  }
  if (P.kb > 0)
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

// One chain: the ministep loop and the chain's outputs.
__device__ void run_chain(const Team &T, const DevProblem &P, const Slice &S, int c) {
  const int n = P.n, W = P.W, k = P.k, L = T.L;
  const uint32_t chain = P.chain_offset + (uint32_t)c;
  chain_init(T, P, S, c);

  const double lam = (double)P.lam[c];
  const double lamb = P.lamb ? (double)P.lamb[c] : 0.0;
  long long dist = 0, bdist = 0, ms = 0, msb = 0;
  double t = 0.0, rho = 0.0;
  double d[24];
  double wsum[24];

  for (;;) {
    uint32_t rr[4];
    philox10((uint32_t)ms, chain, 0u, 0u, P.k0, P.k1, rr);
    int i;
    bool is_net;
    if (P.nrate > 0) {
      i = rate_draw(T, P, S, rr, lam, t, rho);
      if (i < 0) break;
      is_net = true;
    } else {
      // constant rate (src/libcusna_saom_cpu.cpp:195-199); every lane computes
      // the same scalars
      const double den = __dmul_rn((double)P.nact, __dadd_rn(lam, lamb));
      t = __dadd_rn(t, __ddiv_rn(-log(unif01(rr[0])), den));
      if (!P.cond && t > 1.0) break;
      is_net = P.kb == 0 || unif01(rr[1]) < __ddiv_rn(lam, __dadd_rn(lam, lamb));
      long long idx = (long long)__dmul_rn(unif01(rr[2]), (double)P.nact);
      if (idx >= P.nact) idx = P.nact - 1;
      i = P.act[idx];
    }

    if (!is_net) {
      if (T.tl == 0) beh_step(P, S, i, rr[3], &bdist);
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
    X.zvi = P.kb > 0 ? __dsub_rn((double)S.z[i], P.zbar) : 0.0;

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
            change_stats(P, S, X, j, aij, aji, d);
            for (int e = 0; e < k; ++e) f = __dadd_rn(f, __dmul_rn(S.th[e], d[e]));
          }
        }
        S.fbuf[j] = f;
        // a NaN predictor never raises the maximum (the reference compares
        // f > lmax) and is never chosen (its Gumbel key compares false)
        if (ok && !isnan(f)) {
          const long long kf = dkey(f);
          kmax = kf > kmax ? kf : kmax;
        }
      }
      const uint32_t okb = __ballot_sync(kFull, ok);
      if (T.lane == 0) S.okbits[jb >> 5] = okb;
    }
    const double lmax = dunkey(team_max_ll(T, kmax, S.red));
    T.sync();

    // ---- pass 2: log-sum-exp sums and the float32 Gumbel estimates ---------
    double sume = 0.0;
    for (int e = 0; e < k; ++e) wsum[e] = 0.0;
    float gbest = -INFINITY;
    for (int j = T.tl; j < n; j += L) {
      if (!((S.okbits[j >> 5] >> (j & 31)) & 1u)) {
        S.gbuf[j] = -INFINITY;
        continue;
      }
      const double y = __dsub_rn(S.fbuf[j], lmax);
      const double wj = exp(y);
      sume = __dadd_rn(sume, wj);
      if (j != i) {
        const int aij = bit_of(S.rowsT, n, i, j);
        const int aji = bit_of(S.colsT, n, i, j);
        change_stats(P, S, X, j, aij, aji, d);
        for (int e = 0; e < k; ++e) wsum[e] = fma(wj, d[e], wsum[e]);
      }
      uint32_t ph[4];
      philox10((uint32_t)ms, chain, 1u, (uint32_t)j, P.k0, P.k1, ph);
      const float gt = (float)y - loglog_est(ph[0]);
      S.gbuf[j] = gt;
      gbest = fmaxf(gbest, gt);
    }
    // team sums of sume and wsum[0..k-1] into red[q*G + warp]
    {
      double v[32];
#pragma unroll
      for (int q = 0; q < 32; ++q) v[q] = 0.0;
      v[0] = sume;
#pragma unroll
      for (int q = 1; q < 32; ++q)
        if (q - 1 < k) v[q] = wsum[q - 1];
      const int q = warp_multi_sum<32>(v, T.lane);
      const float gmax0 = team_max_f(T, gbest, S.red);
      T.sync();
      if (q <= k) S.red[q * T.G + T.warp] = v[0];
      if (T.tl == 0) ((float *)(S.misc + 6))[0] = gmax0;
      T.sync();
    }
    const float gmax = ((float *)(S.misc + 6))[0];

    // ---- pass 3: exact Gumbel keys of the shortlist ------------------------
    long long bk = dkey(-1e300);
    int bj = 0x7FFFFFFF;
    const float thr = gmax - kGumbelWindow;
    for (int j = T.tl; j < n; j += L) {
      if (S.gbuf[j] >= thr) {
        uint32_t ph[4];
        philox10((uint32_t)ms, chain, 1u, (uint32_t)j, P.k0, P.k1, ph);
        const double g = __dsub_rn(S.fbuf[j], log(-log(unif01(ph[0]))));
        const long long kg = dkey(g);
        if (kg > bk || (kg == bk && j < bj)) { bk = kg; bj = j; }
      }
    }
    const int jstar = team_argmax(T, bk, bj, S.red + 26 * T.G);

    // ---- score update and toggle (team lane 0) -----------------------------
    if (T.tl == 0) {
      double tot[25];
      for (int q = 0; q <= k; ++q) {
        double s = 0.0;
        for (int w = 0; w < T.G; ++w) s = __dadd_rn(s, S.red[q * T.G + w]);
        tot[q] = s;
      }
      if (jstar != i) {
        const int aij = bit_of(S.rowsT, n, i, jstar);
        const int aji = bit_of(S.colsT, n, i, jstar);
        change_stats(P, S, X, jstar, aij, aji, d);
      } else {
        for (int e = 0; e < k; ++e) d[e] = 0.0;
      }
      for (int e = 0; e < k; ++e)
        S.sc[e] = __dadd_rn(S.sc[e], __dsub_rn(d[e], __ddiv_rn(tot[e + 1], tot[0])));
    }
    ++ms;
    if (jstar != i) {
      const int j = jstar;
      const int aij = bit_of(S.rowsT, n, i, j);
      const long long chg = P.symflag ? 2 : 1;
      if (bit_of(P.kdistT, n, i, j))
        dist += (aij == bit_of(P.x0T, n, i, j)) ? chg : -chg;
      T.sync();  // every lane has read the pre-toggle state
      if (T.tl == 0) {
        const int dl = 1 - 2 * aij;
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
