// saom_stats.cuh -- evaluation statistics of a network held in a team slice,
// and the end-of-chain outputs.
//
// Restates src/libcusna_saom_cpu.cpp:608-689 (cusna_network_stats) on
// word-major bitsets. Integer-valued statistics (tie counts, two-path sums,
// squared degrees, 0/0.5/1 indicator sums) are exact in any order and are
// summed by all lanes. Every other statistic is a float64 sum whose rounding
// depends on the order, so the team's lane 0 adds its terms in the reference's
// order (actors ascending, or ties in row-major order), giving identical bits.
#pragma once
#include "saom_kernel.cuh"

namespace cusna {

// src/libcusna_saom_cpu.cpp:608-616
__device__ __forceinline__ double deg_term(int t, double pm, double cur, double start) {
  if (t == 8 || t == 9) {
    if (pm >= 1.0) return t == 9 ? sqrt(cur) : cur;
    return pm == 0.0 ? start : __dadd_rn(cur, start);
  }
  if (pm >= 1.0) return t == 15 ? sqrt(cur) : cur;
  const double s = pm == 0.0 ? start : __dadd_rn(cur, start);
  return t == 15 ? sqrt(s) : s;
}

struct StatDesc {
  const double *vmat, *vb, *wtab, *p1, *p2;
  const uint8_t *vmiss;
  const int *dyn, *od0, *id0, *type_ids;
  int n, W, k, symflag;
};

// Statistics of the network in (R, C) (word-major rows / in-rows) with degrees
// outdeg/indeg already filled. out[k] is written by team lane 0.
template <class DegT>
__device__ inline void network_stats_team(const Team &T, const StatDesc &D, const uint32_t *R,
                                          const uint32_t *Cc, const DegT *outdeg,
                                          const DegT *indeg, double *red, double *out) {
  const int n = D.n, W = D.W, k = D.k;
  for (int e = 0; e < k; ++e) {
    const int t = D.type_ids[e];
    const double pm = D.p1 ? D.p1[e] : 0.0, q2 = D.p2 ? D.p2[e] : 0.0;
    const bool dy = D.dyn && D.dyn[e];
    const double *wr = D.wtab ? D.wtab + (size_t)e * (n + 1) : nullptr;
    auto V = [&](int x) -> double {
      return dy ? (D.vb ? D.vb[x] : 0.0) : (D.vmat ? D.vmat[(size_t)e * n + x] : 0.0);
    };
    auto MISS = [&](int x) -> bool { return D.vmiss && D.vmiss[(size_t)e * n + x]; };
    double acc = 0.0;
    bool integer = true;
    long long part = 0;
    switch (t) {
      case 0: case 1: case 2: case 3: case 23: case 5: case 6: case 4: case 16: case 19:
      case 13: case 20: case 31:
        // integer-valued (20 counts halves): all lanes, one row i per lane
        for (int i = T.tl; i < n; i += T.L) {
          long long s = 0;
          if (t == 0) s = outdeg[i];
          else if (t == 4) s = (long long)indeg[i] * indeg[i];
          else if (t == 16) s = (long long)outdeg[i] * outdeg[i];
          else if (t == 1 || t == 19) {
            int rd = 0;
            for (int w = 0; w < W; ++w) rd += __popc(R[w * n + i] & Cc[w * n + i]);
            s = t == 1 ? rd : (long long)outdeg[i] * rd;
          } else {
            for (int w = 0; w < W; ++w) {
              uint32_t m = R[w * n + i];
              if (t == 6) m &= Cc[w * n + i];
              while (m) {
                const int j = (w << 5) + __ffs(m) - 1;
                m &= m - 1;
                if (t == 2 || t == 23 || t == 5 || t == 6) {
                  const int aa = pc2(R, i, Cc, j, n, W);  // (a@a)_ij
                  s += (t == 5) ? (aa > 0) : aa;
                } else if (t == 3) {
                  s += pc2(R, j, Cc, i, n, W);            // tie i->j adds (a@a)_ji
                } else if (t == 13) {
                  if (!MISS(i) && !MISS(j)) s += fabs(V(i) - V(j)) < 1e-9 ? 1 : 0;
                } else if (t == 20) {  // twice the term: 0, 1 or 2
                  if (MISS(i) || MISS(j)) s += 1;
                  else {
                    const double dd = V(i) - V(j);
                    s += 2 * (dd > 1e-9 ? 1 : 0) + (fabs(dd) <= 1e-9 ? 1 : 0);
                  }
                } else if (t == 31) {
                  if (!MISS(j) && V(j) >= pm - 1e-12) s += 1;
                }
              }
            }
          }
          part += s;
        }
        part = team_sum_ll(T, part, red);
        acc = (double)part;
        if (t == 0 && D.symflag) acc = acc * 0.5;
        if (t == 3) acc = acc / 3.0;
        if (t == 23) acc = acc / 6.0;
        if (t == 20) acc = acc * 0.5;
        break;
      default:
        integer = false;
        break;
    }
    if (!integer && T.tl == 0) {
      switch (t) {
        case 7: for (int j = 0; j < n; ++j) acc = __dadd_rn(acc, pow((double)indeg[j], 1.5)); break;
        case 8: case 9:
          for (int i = 0; i < n; ++i)
            acc = __dadd_rn(acc, __dmul_rn((double)indeg[i],
                                           deg_term(t, pm, (double)outdeg[i], D.od0 ? (double)D.od0[i] : 0.0)));
          break;
        case 14: case 15:
          for (int i = 0; i < n; ++i)
            acc = __dadd_rn(acc, __dmul_rn((double)outdeg[i],
                                           deg_term(t, pm, (double)indeg[i], D.id0 ? (double)D.id0[i] : 0.0)));
          break;
        case 17: for (int i = 0; i < n; ++i) acc = __dadd_rn(acc, pow((double)outdeg[i], 1.5)); break;
        case 18: for (int i = 0; i < n; ++i) acc = __dadd_rn(acc, fmin((double)outdeg[i], pm)); break;
        case 10: for (int i = 0; i < n; ++i) if (!MISS(i)) acc = __dadd_rn(acc, __dmul_rn((double)outdeg[i], V(i))); break;
        case 11: for (int i = 0; i < n; ++i) if (!MISS(i)) acc = __dadd_rn(acc, __dmul_rn((double)indeg[i], V(i))); break;
        case 12: case 21: case 25: case 24: case 26: case 27: case 28:
          for (int i = 0; i < n; ++i)
            for (int w = 0; w < W; ++w) {
              uint32_t m = R[w * n + i];
              while (m) {
                const int j = (w << 5) + __ffs(m) - 1;
                m &= m - 1;
                double term;
                if (t == 12 || t == 21 || t == 25) {
                  if (MISS(i) || MISS(j)) continue;
                  if (t == 12) term = __dsub_rn(__dsub_rn(1.0, __dmul_rn(fabs(__dsub_rn(V(i), V(j))), pm)), q2);
                  else if (t == 21) term = __dmul_rn(V(i), V(j));
                  else term = __dadd_rn(V(i), V(j));
                } else {
                  int cnt;
                  if (t == 24) cnt = pc2(R, i, Cc, j, n, W);        // (a@a)_ij
                  else if (t == 26) cnt = pc2(R, i, R, j, n, W);    // (a@a^T)_ij
                  else if (t == 27) cnt = pc2(Cc, i, Cc, j, n, W);  // (a^T@a)_ij
                  else cnt = pc2(Cc, i, R, j, n, W);                // (a^T@a^T)_ij
                  term = wr[cnt];
                }
                acc = __dadd_rn(acc, term);
              }
            }
          break;
        case 29: case 30:
          for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) {
              if (i == j) continue;
              const int cnt = (t == 29) ? pc2(R, i, Cc, j, n, W) : pc2(R, i, R, j, n, W);
              acc = __dadd_rn(acc, wr[cnt]);
            }
          break;
        default: acc = 0.0; break;  // 22 and 32: the reference reports 0
      }
    }
    if (T.tl == 0) out[e] = acc;
  }
}

// End of one chain (src/libcusna_saom_cpu.cpp:290-302 and :394-422).
__device__ void chain_finish(const Team &T, const DevProblem &P, const Slice &S, int c,
                             long long dist, long long bdist, long long ms, long long msb,
                             double t, double rho, double lam, double lamb);

}  // namespace cusna
