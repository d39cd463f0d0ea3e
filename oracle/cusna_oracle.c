/* ==========================================================================
 * cusna_oracle.c -- CPU ORACLE for the SAOM period simulator. TEST
 * INFRASTRUCTURE ONLY: tests, the smoke check and the CPU-baseline leg of the
 * benchmark use it as the checker. The product library (libcusna_gb300.so)
 * never links or calls it.
 *
 * A plain-C restatement of the reference CPU engine of cran/cusna 0.1.1:
 *   src/libcusna_saom_cpu.cpp:30-425  period simulator (Philox, change
 *                                     statistics, ministep loop, entry point)
 *   src/libcusna_saom_cpu.cpp:606-689 evaluation statistics of one network
 *   src/libcusna_saom_cpu.cpp:691-765 typed statistics, GoF distributions
 *   src/libcusna_saom_cpu.cpp:767-817 behaviour statistics
 *   src/libcusna_saom_cpu.cpp:427-604 multi-network simulator
 *   src/libcusna_saom_cpu.cpp:819-857 cross-network statistics
 * Each function names the lines it follows. The restatement keeps the
 * reference's dense n*n uint8 layout, loop orders and float64 operation order
 * (so it reproduces the reference bit for bit), and therefore also its
 * algorithmic cost: the timed CPU baseline runs the same O(n) loops per alter.
 *
 * Parity pins: the reference's golden vectors tests/testthat/fixtures/sim/
 * sim.json.gz (three configurations, integer outputs identical, float outputs
 * equal) and the reference engine itself, compiled from its own sources into
 * oracle/_ref/ by oracle/Makefile, on seeded synthetic inputs.
 *
 * Build with -ffp-contract=off: a fused multiply-add changes float64 results,
 * and gcc contracts by default on aarch64.
 * ========================================================================== */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "libcusna.h"

#ifdef _OPENMP
#include <omp.h>
#endif

#define ORACLE_MAX_STEPS 4000000L   /* src/libcusna_saom_cpu.cpp:115 */

/* ---- Philox4x32-10 and the uniform map (src/libcusna_saom_cpu.cpp:32-46) -- */
static void ph4(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                uint32_t k0, uint32_t k1, uint32_t out[4]) {
    for (int r = 0; r < 10; ++r) {
        uint64_t m0 = (uint64_t)0xD2511F53u * (uint64_t)c0;
        uint64_t m1 = (uint64_t)0xCD9E8D57u * (uint64_t)c2;
        uint32_t y0 = (uint32_t)(m1 >> 32) ^ c1 ^ k0;
        uint32_t y1 = (uint32_t)m1;
        uint32_t y2 = (uint32_t)(m0 >> 32) ^ c3 ^ k1;
        uint32_t y3 = (uint32_t)m0;
        c0 = y0; c1 = y1; c2 = y2; c3 = y3;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

static double unif(uint32_t x) { return ((double)x + 0.5) * (1.0 / 4294967296.0); }

/* ---- chain-invariant inputs (src/libcusna_saom_cpu.cpp:117-135) ---------- */
typedef struct {
    int n, k, kb, nrate;
    const uint8_t *x0, *xs, *kd, *pm;        /* dense n*n                   */
    double lam, lamb;
    const double *th, *thb;
    const int32_t *tid, *ety, *dyn, *dyi, *i0, *i1, *i2, *bty, *rk;
    const double *wt, *p1, *p2, *vm, *dym, *ra, *ru;
    const int32_t *z0, *bkd, *act;
    int zmin, zmax, nact, has_comp, sym, maxdeg, cond, target;
    double zbar, brange, bsim;
    const uint8_t *inact;
    uint32_t k0, k1;
    int need_tp, need_rdeg;
    /* validation mode (no counterpart in the reference): a per-ministep trace
     * and caller-supplied 32-bit words in place of the Philox outputs */
    int32_t *trace;          /* M*trace_cap records (step, actor, choice, delta) */
    int trace_cap;
    const uint32_t *us;      /* M*us_steps*(4+n) words, or NULL */
    int us_steps;
} octx;

/* The four words of ministep ms of chain c: Philox counter (ms, c, 0, 0)
 * (src/libcusna_saom_cpu.cpp:167), or the supplied words while they last. */
static void step_words(const octx *C, uint32_t chain, long ms, uint32_t rr[4]) {
    if (C->us && ms < C->us_steps) {
        const uint32_t *u = C->us + ((size_t)chain * C->us_steps + (size_t)ms) * (4 + (size_t)C->n);
        rr[0] = u[0]; rr[1] = u[1]; rr[2] = u[2]; rr[3] = u[3];
    } else {
        ph4((uint32_t)ms, chain, 0u, 0u, C->k0, C->k1, rr);
    }
}

/* The Gumbel word of alter j in ministep ms: Philox counter (ms, c, 1, j),
 * first output (src/libcusna_saom_cpu.cpp:266), or the supplied word. */
static uint32_t alter_word(const octx *C, uint32_t chain, long ms, int j) {
    uint32_t rr[4];
    if (C->us && ms < C->us_steps)
        return C->us[((size_t)chain * C->us_steps + (size_t)ms) * (4 + (size_t)C->n) + 4 + (size_t)j];
    ph4((uint32_t)ms, chain, 1u, (uint32_t)j, C->k0, C->k1, rr);
    return rr[0];
}

/* Record one ministep of chain `chain` in the validation trace. */
static void trace_put(const octx *C, uint32_t chain, long ms, int actor, int choice, long delta) {
    if (!C->trace || ms >= C->trace_cap) return;
    int32_t *t = C->trace + ((size_t)chain * C->trace_cap + (size_t)ms) * 4;
    t[0] = (int32_t)ms; t[1] = actor; t[2] = choice; t[3] = (int32_t)delta;
}

/* Change statistic of toggling i->j for one effect type, mutable state `a`
 * (dense), degrees, two-path counts tp (type 5). src/libcusna_saom_cpu.cpp:49-101. */
static double change_stat(int t, const uint8_t *a, int n, const long *ind,
                          const long *outd, long rdeg, const int *tp,
                          double vi, double vj, double dyw, double q1, double q2,
                          int i, int j, double dl, const double *w) {
    const uint8_t *ri = a + (size_t)i * n, *rj = a + (size_t)j * n;
    long c = 0;
    int h, m;
    switch (t) {
    case 0: return dl;
    case 1: return dl * (double)rj[i];
    case 2:
        for (h = 0; h < n; ++h)
            if (ri[h]) { c += a[(size_t)h * n + j] ? 1 : 0; c += rj[h] ? 1 : 0; }
        return dl * (double)c;
    case 3: case 23:
        for (h = 0; h < n; ++h) if (rj[h] && a[(size_t)h * n + i]) ++c;
        return dl * (double)c;
    case 4: return dl * (double)(ind[j] + (1 - ri[j]));
    case 5: {
        int want = ri[j] ? 1 : 0;
        for (h = 0; h < n; ++h) if (ri[h] && rj[h] && tp[h] == want) ++c;
        if (tp[j] > 0) ++c;
        return dl * (double)c;
    }
    case 6:
        if (rj[i]) for (h = 0; h < n; ++h) if (ri[h] && a[(size_t)h * n + j]) ++c;
        for (h = 0; h < n; ++h) if (ri[h] && a[(size_t)h * n + i] && rj[h]) ++c;
        return dl * (double)c;
    case 7: return dl * sqrt((double)(ind[j] + (1 - ri[j])));
    case 8: return dl * (double)outd[j];
    case 9: return dl * sqrt((double)outd[j]);
    case 10: return dl * vi;
    case 11: return dl * vj;
    case 12: return dl * (1.0 - fabs(vi - vj) * q1 - q2);
    case 13: return dl * (fabs(vi - vj) < 1e-9 ? 1.0 : 0.0);
    case 14: return dl * (double)ind[i];
    case 15: return dl * sqrt((double)ind[i]);
    case 16: return dl * (2.0 * (double)outd[i] + dl);
    case 17: { double d0 = (double)outd[i], d1 = d0 + dl; return d1 * sqrt(d1) - d0 * sqrt(d0); }
    case 18: { double d0 = (double)outd[i]; return fmin(d0 + dl, q1) - fmin(d0, q1); }
    case 19: return dl * ((double)rdeg + (double)rj[i] * ((double)outd[i] + dl));
    case 20:
        if (vi > vj + 1e-9) return dl;
        if (fabs(vi - vj) <= 1e-9) return dl * 0.5;
        return 0.0;
    case 21: return dl * vi * vj;
    case 22: return dl * dyw;
    case 24:
        for (h = 0; h < n; ++h) if (ri[h] && a[(size_t)h * n + j]) ++c;
        return dl * w[c];
    case 25: return dl * (vi + vj);
    case 26:
        for (h = 0; h < n; ++h) if (ri[h] && rj[h]) ++c;
        return dl * w[c];
    case 27:
        for (h = 0; h < n; ++h) if (a[(size_t)h * n + i] && a[(size_t)h * n + j]) ++c;
        return dl * w[c];
    case 28:
        for (h = 0; h < n; ++h) if (a[(size_t)h * n + i] && rj[h]) ++c;
        return dl * w[c];
    case 29: case 30: {
        int xij = ri[j];
        double acc = 0.0;
        for (h = 0; h < n; ++h) {
            int link = (t == 29) ? rj[h] : a[(size_t)h * n + j];
            if (!link || h == i) continue;
            int p = 0;
            for (m = 0; m < n; ++m) {
                int second = (t == 29) ? a[(size_t)m * n + h] : a[(size_t)h * n + m];
                if (ri[m] && second) ++p;
            }
            acc += xij ? (w[p] - w[p - 1]) : (w[p + 1] - w[p]);
        }
        return dl * acc;
    }
    case 31: return dl * (vj >= q1 - 1e-12 ? 1.0 : 0.0);
    default: return 0.0;
    }
}

/* Behaviour change statistic, src/libcusna_saom_cpu.cpp:103-113. */
static double beh_change(int t, double dl, double zc, long nb, double zs,
                         long nh, long ne, long nl, double br, double bs) {
    double tc;
    switch (t) {
    case 0: return dl;
    case 1: return (2.0 * zc + dl) * dl;
    case 2: return nb > 0 ? dl * zs / (double)nb : 0.0;
    case 3:
        if (nb == 0) return 0.0;
        tc = dl > 0 ? (double)(nh - ne - nl) : (double)(nl - ne - nh);
        return tc / (br * (double)nb);
    case 4:
        if (nb == 0) return 0.0;
        tc = dl > 0 ? (double)(nh - ne - nl) : (double)(nl - ne - nh);
        return tc / br - (double)nb * bs;
    default: return 0.0;
    }
}

typedef struct {
    long dist, dist_stat, steps;
    double t, rate_score, brate_score, bdist;
} ochain;

/* One chain's ministep loop, src/libcusna_saom_cpu.cpp:142-303. All buffers
 * are caller-provided scratch for this chain. */
static void run_chain(const octx *C, uint32_t chain, uint8_t *a, int32_t *z,
                      double *sc, double *bsc, double *rsc, long *adist,
                      long *ind, long *outd, double *fj, double *dsb, uint8_t *okb,
                      int *tp, double *crate, double *wsum, ochain *o) {
    const int n = C->n, k = C->k, kb = C->kb, nr = C->nrate;
    double cup[CUSNA_MAXBEFF], cdn[CUSNA_MAXBEFF], ub[CUSNA_MAXRATE], rs[CUSNA_MAXRATE];
    long dist = 0, bdist = 0, ms = 0, msb = 0;
    double t = 0.0, rho = 0.0;
    uint32_t rr[4];
    int i, j, e, q;

    for (i = 0; i < n; ++i) { ind[i] = 0; outd[i] = 0; }
    for (i = 0; i < n; ++i)
        for (j = 0; j < n; ++j) {
            uint8_t v = C->xs[(size_t)i * n + j];
            a[(size_t)i * n + j] = v;
            if (v) { ind[j]++; outd[i]++; }
        }
    for (i = 0; i < n; ++i) { z[i] = C->z0[i]; crate[i] = 1.0; }
    for (e = 0; e < k; ++e) sc[e] = 0.0;
    for (e = 0; e < kb; ++e) bsc[e] = 0.0;
    for (q = 0; q < nr; ++q) rsc[q] = 0.0;

    for (;;) {
        int is_net;
        step_words(C, chain, ms, rr);
        if (nr > 0) {                       /* :170-193 non-basic rate draw */
            double S0 = 0.0, tau, tau_eff, tgt, acc;
            int idx;
            for (q = 0; q < nr; ++q) rs[q] = 0.0;
            for (idx = 0; idx < C->nact; ++idx) {
                int a2 = C->act[idx];
                double s = 0.0, cc;
                for (q = 0; q < nr; ++q) {
                    double u = C->rk[q] == 0 ? C->ru[(size_t)q * n + a2]
                             : C->rk[q] == 1 ? (double)outd[a2] : (double)ind[a2];
                    ub[q] = u;
                    s += C->ra[q] * u;
                }
                if (s > 30.0) s = 30.0; else if (s < -30.0) s = -30.0;
                cc = exp(s);
                crate[a2] = cc;
                S0 += cc;
                for (q = 0; q < nr; ++q) rs[q] += cc * ub[q];
            }
            tau = -log(unif(rr[0])) / (C->lam * S0);
            tau_eff = tau;
            if (!C->cond && t + tau > 1.0) tau_eff = 1.0 - t;
            rho += tau_eff * S0;
            for (q = 0; q < nr; ++q) rsc[q] -= tau_eff * C->lam * rs[q];
            t += tau;
            if (!C->cond && t > 1.0) break;
            is_net = 1;
            tgt = unif(rr[2]) * S0;
            acc = 0.0;
            i = C->act[C->nact - 1];
            for (idx = 0; idx < C->nact; ++idx) {
                acc += crate[C->act[idx]];
                if (acc >= tgt) { i = C->act[idx]; break; }
            }
        } else {                            /* :195-199 constant rate */
            long idx;
            t += -log(unif(rr[0])) / ((double)C->nact * (C->lam + C->lamb));
            if (!C->cond && t > 1.0) break;
            is_net = kb == 0 || unif(rr[1]) < C->lam / (C->lam + C->lamb);
            idx = (long)(unif(rr[2]) * C->nact);
            if (idx >= C->nact) idx = C->nact - 1;
            i = C->act[idx];
        }

        if (!is_net) {                      /* :202-227 behaviour ministep */
            int zi = z[i], up, dn, d;
            double zc = (double)zi - C->zbar, zs = 0.0, fu = 0.0, fd = 0.0, mx;
            double pd, p0, pu, ps, uc;
            long nb = 0, nh = 0, ne = 0, nl = 0;
            for (j = 0; j < n; ++j)
                if (a[(size_t)i * n + j]) {
                    int zj = z[j];
                    nb++;
                    zs += (double)zj - C->zbar;
                    if (zj > zi) nh++; else if (zj == zi) ne++; else nl++;
                }
            up = zi < C->zmax;
            dn = zi > C->zmin;
            for (e = 0; e < kb; ++e) {
                cup[e] = beh_change(C->bty[e], 1.0, zc, nb, zs, nh, ne, nl, C->brange, C->bsim);
                cdn[e] = beh_change(C->bty[e], -1.0, zc, nb, zs, nh, ne, nl, C->brange, C->bsim);
                fu += C->thb[e] * cup[e];
                fd += C->thb[e] * cdn[e];
            }
            mx = 0.0;
            if (up && fu > mx) mx = fu;
            if (dn && fd > mx) mx = fd;
            pd = dn ? exp(fd - mx) : 0.0;
            p0 = exp(-mx);
            pu = up ? exp(fu - mx) : 0.0;
            ps = pd + p0 + pu;
            pd /= ps; p0 /= ps; pu /= ps;
            uc = unif(rr[3]);
            d = uc < pd ? -1 : (uc < pd + p0 ? 0 : 1);
            for (e = 0; e < kb; ++e) {
                double s = d == 1 ? cup[e] : (d == -1 ? cdn[e] : 0.0);
                if (up) s -= pu * cup[e];
                if (dn) s -= pd * cdn[e];
                bsc[e] += s;
            }
            {
                long bd0 = bdist;
                if (d != 0) {
                    if (C->bkd[i]) bdist += labs((long)(zi + d - C->z0[i])) - labs((long)zi - C->z0[i]);
                    z[i] = zi + d;
                }
                trace_put(C, chain, ms, i, -(d + 2), bdist - bd0);
            }
            msb++; ms++;
            if (C->cond && dist >= C->target) break;
            if (ms >= ORACLE_MAX_STEPS) break;
            continue;
        }

        /* :229-233 per-ministep helpers */
        if (C->need_tp) {
            int x, h;
            for (h = 0; h < n; ++h) tp[h] = 0;
            for (x = 0; x < n; ++x)
                if (a[(size_t)i * n + x])
                    for (h = 0; h < n; ++h) tp[h] += a[(size_t)x * n + h];
        }
        long rdeg = 0;
        if (C->need_rdeg) {
            int h;
            for (h = 0; h < n; ++h) if (a[(size_t)i * n + h] && a[(size_t)h * n + i]) rdeg++;
        }
        double zvi = (double)z[i] - C->zbar;

        /* :235-269 alters: change statistics, f, Gumbel-max choice */
        double gbest = -1e30, lmax = -1e30;
        int jstar = i;
        for (j = 0; j < n; ++j) {
            double f = 0.0;
            int ok = 1;
            double *dj = dsb + (size_t)j * k;
            if (j == i) {
                for (e = 0; e < k; ++e) dj[e] = 0.0;
            } else {
                uint8_t aij = a[(size_t)i * n + j];
                if (!C->pm[(size_t)i * n + j]) ok = 0;
                else if (C->maxdeg > 0 && aij == 0 && outd[i] >= C->maxdeg) ok = 0;
                if (ok) {
                    double dl = 1.0 - 2.0 * aij;
                    double zvj = (double)z[j] - C->zbar;
                    for (e = 0; e < k; ++e) {
                        double d;
                        if (C->tid[e] == 32) {      /* :246-251 interaction */
                            d = C->i2[e] < 0 ? dl : 1.0;
                            d *= dj[C->i0[e]] * dj[C->i1[e]];
                            if (C->i2[e] >= 0) d *= dj[C->i2[e]];
                            dj[e] = d;
                            f += C->th[e] * d;
                            continue;
                        }
                        {
                            double vi = C->dyn[e] ? zvi : C->vm[(size_t)e * n + i];
                            double vj = C->dyn[e] ? zvj : C->vm[(size_t)e * n + j];
                            double dyw = C->dyi[e] >= 0 ? C->dym[((size_t)C->dyi[e] * n + i) * n + j] : 0.0;
                            d = change_stat(C->tid[e], a, n, ind, outd, rdeg, tp, vi, vj, dyw,
                                            C->p1[e], C->p2[e], i, j, dl, C->wt + (size_t)e * (n + 1));
                        }
                        if ((C->ety[e] == 1 && aij == 1) || (C->ety[e] == 2 && aij == 0)) d = 0.0;
                        dj[e] = d;
                        f += C->th[e] * d;
                    }
                }
            }
            okb[j] = (uint8_t)ok;
            fj[j] = f;
            if (ok && f > lmax) lmax = f;
            if (ok) {
                double g = f - log(-log(unif(alter_word(C, chain, ms, j))));
                if (g > gbest || (g == gbest && j < jstar)) { gbest = g; jstar = j; }
            }
        }

        /* :271-274 log-sum-exp score */
        {
            double sume = 0.0;
            for (e = 0; e < k; ++e) wsum[e] = 0.0;
            for (j = 0; j < n; ++j)
                if (okb[j]) {
                    double w = exp(fj[j] - lmax);
                    sume += w;
                    for (e = 0; e < k; ++e) wsum[e] += w * dsb[(size_t)j * k + e];
                }
            for (e = 0; e < k; ++e) sc[e] += dsb[(size_t)jstar * k + e] - wsum[e] / sume;
        }
        long dist0 = dist;
        long ms0 = ms;
        ms++;

        /* :277-282 toggle */
        if (jstar != i) {
            int jj = jstar;
            long dlt = 1 - 2 * (long)a[(size_t)i * n + jj];
            long chg = C->sym ? 2 : 1;
            if (C->kd[(size_t)i * n + jj])
                dist += (a[(size_t)i * n + jj] == C->x0[(size_t)i * n + jj]) ? chg : -chg;
            ind[jj] += dlt; outd[i] += dlt;
            a[(size_t)i * n + jj] = (uint8_t)(1 - a[(size_t)i * n + jj]);
            if (C->sym) {
                ind[i] += dlt; outd[jj] += dlt;
                a[(size_t)jj * n + i] = (uint8_t)(1 - a[(size_t)jj * n + i]);
            }
        }
        trace_put(C, chain, ms0, i, jstar, dist - dist0);
        if (nr > 0)
            for (q = 0; q < nr; ++q)
                rsc[q] += C->rk[q] == 0 ? C->ru[(size_t)q * n + i]
                        : C->rk[q] == 1 ? (double)outd[i] : (double)ind[i];

        if (C->cond && dist >= C->target) break;
        if (ms >= ORACLE_MAX_STEPS) break;
    }

    /* :290-302 end of chain */
    if (C->has_comp)
        for (i = 0; i < n; ++i)
            if (C->inact[i])
                for (j = 0; j < n; ++j) {
                    a[(size_t)i * n + j] = C->x0[(size_t)i * n + j];
                    a[(size_t)j * n + i] = C->x0[(size_t)j * n + i];
                }
    {
        long ds = 0;
        for (i = 0; i < n; ++i) {
            long cnt = 0;
            for (j = 0; j < n; ++j)
                if (C->kd[(size_t)i * n + j] && a[(size_t)i * n + j] != C->x0[(size_t)i * n + j]) cnt++;
            adist[i] = cnt;
            ds += cnt;
        }
        o->dist_stat = ds;
    }
    o->dist = dist;
    o->steps = ms;
    o->t = t;
    o->rate_score = nr > 0 ? (double)(ms - msb) / C->lam - rho
                           : (double)(ms - msb) / C->lam - (double)C->nact;
    o->brate_score = kb > 0 ? (double)msb / C->lamb - (double)C->nact : 0.0;
    o->bdist = (double)bdist;
}

/* Unpack n*W bit rows to dense n*n, src/libcusna_saom_cpu.cpp:306-311. */
static void bits_to_dense(const uint32_t *rows, int n, int W, uint8_t *dense) {
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j)
            dense[(size_t)i * n + j] = (uint8_t)((rows[(size_t)i * W + (j >> 5)] >> (j & 31)) & 1u);
}

static void offdiag(uint8_t *m, int n, uint8_t on) {
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) m[(size_t)i * n + j] = (uint8_t)(i != j ? on : 0);
}

/* Evaluation statistics, src/libcusna_saom_cpu.cpp:608-689. */
static double degree_term(int t, double pm, double cur, double start) {
    double s;
    if (t == 8 || t == 9) {
        if (pm >= 1.0) return t == 9 ? sqrt(cur) : cur;
        return pm == 0.0 ? start : cur + start;
    }
    if (pm >= 1.0) return t == 15 ? sqrt(cur) : cur;
    s = pm == 0.0 ? start : cur + start;
    return t == 15 ? sqrt(s) : s;
}

static void two_path(const uint8_t *a, int n, int rowT, int colT, int *M) {
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            int s = 0;
            for (int h = 0; h < n; ++h) {
                int l = rowT ? a[(size_t)h * n + i] : a[(size_t)i * n + h];
                int r = colT ? a[(size_t)j * n + h] : a[(size_t)h * n + j];
                s += l & r;
            }
            M[(size_t)i * n + j] = s;
        }
}

cusna_status oracle_network_stats(const uint8_t *a, int32_t n, int32_t k,
                                  const int32_t *type_ids, const double *p1, const double *p2,
                                  const double *vmat, const uint8_t *vmiss, const int32_t *dyn_flags,
                                  const double *vb, const int32_t *od0, const int32_t *id0,
                                  const double *wtab, int32_t symflag, double *out) {
    if (!a || !type_ids || !out || n < 1 || n > CUSNA_MAX_N || k < 1) return CUSNA_ERR_NULL_ARG;
    size_t nn = (size_t)n * n;
    double *ind = (double *)calloc((size_t)n, sizeof(double));
    double *outd = (double *)calloc((size_t)n, sizeof(double));
    int *aa = NULL, *fb = NULL, *bf = NULL, *bb = NULL;
    int need_aa = 0, need_fb = 0, need_bf = 0, need_bb = 0;
    int i, j, e;
    for (i = 0; i < n; ++i)
        for (j = 0; j < n; ++j)
            if (a[(size_t)i * n + j]) { outd[i] += 1.0; ind[j] += 1.0; }
    for (e = 0; e < k; ++e) {
        int t = type_ids[e];
        if (t == 2 || t == 3 || t == 5 || t == 6 || t == 23 || t == 24 || t == 29) need_aa = 1;
        if (t == 26 || t == 30) need_fb = 1;
        if (t == 27) need_bf = 1;
        if (t == 28) need_bb = 1;
    }
    if (need_aa) { aa = (int *)malloc(nn * sizeof(int)); two_path(a, n, 0, 0, aa); }
    if (need_fb) { fb = (int *)malloc(nn * sizeof(int)); two_path(a, n, 0, 1, fb); }
    if (need_bf) { bf = (int *)malloc(nn * sizeof(int)); two_path(a, n, 1, 0, bf); }
    if (need_bb) { bb = (int *)malloc(nn * sizeof(int)); two_path(a, n, 1, 1, bb); }

    for (e = 0; e < k; ++e) {
        int t = type_ids[e];
        double acc = 0.0;
        const double *wr = wtab ? wtab + (size_t)e * (n + 1) : NULL;
        double pm = p1 ? p1[e] : 0.0, q2 = p2 ? p2[e] : 0.0;
        int dy = dyn_flags && dyn_flags[e];
#define V(ii) (dy ? (vb ? vb[ii] : 0.0) : (vmat ? vmat[(size_t)e * n + (ii)] : 0.0))
#define MISS(ii) (vmiss && vmiss[(size_t)e * n + (ii)])
        size_t q;
        switch (t) {
        case 0: for (i = 0; i < n; ++i) acc += outd[i]; if (symflag) acc *= 0.5; break;
        case 1: for (i = 0; i < n; ++i) for (j = 0; j < n; ++j) acc += (a[(size_t)i * n + j] && a[(size_t)j * n + i]); break;
        case 2: for (q = 0; q < nn; ++q) if (a[q]) acc += aa[q]; break;
        case 3: for (i = 0; i < n; ++i) for (j = 0; j < n; ++j) if (a[(size_t)j * n + i]) acc += aa[(size_t)i * n + j]; acc /= 3.0; break;
        case 23: for (q = 0; q < nn; ++q) if (a[q]) acc += aa[q]; acc /= 6.0; break;
        case 5: for (q = 0; q < nn; ++q) if (a[q] && aa[q] > 0) acc += 1.0; break;
        case 6: for (i = 0; i < n; ++i) for (j = 0; j < n; ++j) if (a[(size_t)i * n + j] && a[(size_t)j * n + i]) acc += aa[(size_t)i * n + j]; break;
        case 4: for (j = 0; j < n; ++j) acc += ind[j] * ind[j]; break;
        case 7: for (j = 0; j < n; ++j) acc += pow(ind[j], 1.5); break;
        case 8: case 9: for (i = 0; i < n; ++i) acc += ind[i] * degree_term(t, pm, outd[i], od0 ? od0[i] : 0.0); break;
        case 14: case 15: for (i = 0; i < n; ++i) acc += outd[i] * degree_term(t, pm, ind[i], id0 ? id0[i] : 0.0); break;
        case 16: for (i = 0; i < n; ++i) acc += outd[i] * outd[i]; break;
        case 17: for (i = 0; i < n; ++i) acc += pow(outd[i], 1.5); break;
        case 18: for (i = 0; i < n; ++i) acc += fmin(outd[i], pm); break;
        case 19:
            for (i = 0; i < n; ++i) {
                double rd = 0;
                for (j = 0; j < n; ++j) rd += (a[(size_t)i * n + j] && a[(size_t)j * n + i]);
                acc += outd[i] * rd;
            }
            break;
        case 10: for (i = 0; i < n; ++i) if (!MISS(i)) acc += outd[i] * V(i); break;
        case 11: for (i = 0; i < n; ++i) if (!MISS(i)) acc += ind[i] * V(i); break;
        case 12: for (i = 0; i < n; ++i) for (j = 0; j < n; ++j) if (a[(size_t)i * n + j] && !MISS(i) && !MISS(j)) acc += 1.0 - fabs(V(i) - V(j)) * pm - q2; break;
        case 13: for (i = 0; i < n; ++i) for (j = 0; j < n; ++j) if (a[(size_t)i * n + j] && !MISS(i) && !MISS(j)) acc += fabs(V(i) - V(j)) < 1e-9 ? 1.0 : 0.0; break;
        case 20:
            for (i = 0; i < n; ++i) for (j = 0; j < n; ++j) if (a[(size_t)i * n + j]) {
                double val;
                if (MISS(i) || MISS(j)) val = 0.5;
                else { double d = V(i) - V(j); val = (d > 1e-9 ? 1.0 : 0.0) + 0.5 * (fabs(d) <= 1e-9 ? 1.0 : 0.0); }
                acc += val;
            }
            break;
        case 21: for (i = 0; i < n; ++i) for (j = 0; j < n; ++j) if (a[(size_t)i * n + j] && !MISS(i) && !MISS(j)) acc += V(i) * V(j); break;
        case 25: for (i = 0; i < n; ++i) for (j = 0; j < n; ++j) if (a[(size_t)i * n + j] && !MISS(i) && !MISS(j)) acc += V(i) + V(j); break;
        case 31: for (i = 0; i < n; ++i) for (j = 0; j < n; ++j) if (a[(size_t)i * n + j] && !MISS(j) && V(j) >= pm - 1e-12) acc += 1.0; break;
        case 24: for (i = 0; i < n; ++i) for (j = 0; j < n; ++j) if (a[(size_t)i * n + j]) acc += wr[aa[(size_t)i * n + j]]; break;
        case 26: for (i = 0; i < n; ++i) for (j = 0; j < n; ++j) if (a[(size_t)i * n + j]) acc += wr[fb[(size_t)i * n + j]]; break;
        case 27: for (i = 0; i < n; ++i) for (j = 0; j < n; ++j) if (a[(size_t)i * n + j]) acc += wr[bf[(size_t)i * n + j]]; break;
        case 28: for (i = 0; i < n; ++i) for (j = 0; j < n; ++j) if (a[(size_t)i * n + j]) acc += wr[bb[(size_t)i * n + j]]; break;
        case 29: for (i = 0; i < n; ++i) for (j = 0; j < n; ++j) if (i != j) acc += wr[aa[(size_t)i * n + j]]; break;
        case 30: for (i = 0; i < n; ++i) for (j = 0; j < n; ++j) if (i != j) acc += wr[fb[(size_t)i * n + j]]; break;
        default: break;
        }
#undef V
#undef MISS
        out[e] = acc;
    }
    free(ind); free(outd); free(aa); free(fb); free(bf); free(bb);
    return CUSNA_OK;
}

/* Behaviour statistics, src/libcusna_saom_cpu.cpp:768-817. */
cusna_status oracle_behavior_stats(const int32_t *z_batch, int32_t n, int32_t M, int32_t kb,
                                   const int32_t *bty, const uint8_t *xnet, const int32_t *bkdist,
                                   double zbar, double brange, double bsimmean, double *out) {
    if (!z_batch || !bty || !xnet || !out || n < 1 || n > CUSNA_MAX_N || M < 1 || kb < 1)
        return CUSNA_ERR_NULL_ARG;
    double *ok = (double *)malloc((size_t)n * sizeof(double));
    double *od = (double *)malloc((size_t)n * sizeof(double));
    double *nb = (double *)malloc((size_t)n * sizeof(double));
    double *u = (double *)malloc((size_t)n * sizeof(double));
    int i, j, c, e;
    for (i = 0; i < n; ++i) ok[i] = bkdist ? (bkdist[i] ? 1.0 : 0.0) : 1.0;
    for (i = 0; i < n; ++i) {
        double o = 0.0, b = 0.0;
        for (j = 0; j < n; ++j) if (xnet[(size_t)i * n + j]) { o += 1.0; b += ok[j]; }
        od[i] = o; nb[i] = b;
    }
    for (c = 0; c < M; ++c) {
        const int32_t *z = z_batch + (size_t)c * n;
        for (i = 0; i < n; ++i) u[i] = ok[i] ? ((double)z[i] - zbar) : 0.0;
        for (e = 0; e < kb; ++e) {
            int t = bty[e];
            double acc = 0.0;
            if (t == 0) { for (i = 0; i < n; ++i) acc += u[i]; }
            else if (t == 1) { for (i = 0; i < n; ++i) acc += u[i] * u[i]; }
            else if (t == 2) {
                for (i = 0; i < n; ++i) {
                    double s = 0.0;
                    if (od[i] <= 0.0) continue;
                    for (j = 0; j < n; ++j) if (xnet[(size_t)i * n + j]) s += u[j];
                    acc += u[i] * (s / od[i]);
                }
            } else if (t == 3 || t == 4) {
                for (i = 0; i < n; ++i) {
                    double s = 0.0;
                    if (ok[i] == 0.0) continue;
                    for (j = 0; j < n; ++j)
                        if (xnet[(size_t)i * n + j] && ok[j] != 0.0) s += 1.0 - fabs(u[i] - u[j]) / brange;
                    s -= nb[i] * bsimmean;
                    if (t == 3) s = nb[i] > 0.0 ? s / nb[i] : 0.0;
                    acc += s;
                }
            }
            out[(size_t)c * kb + e] = acc;
        }
    }
    free(ok); free(od); free(nb); free(u);
    return CUSNA_OK;
}

/* Entry point, src/libcusna_saom_cpu.cpp:315-425. `threads` > 0 caps the
 * OpenMP team (the reference reads its thread count from the OpenMP runtime).
 * trace / us: the validation mode's trace and supplied words (NULL: none). */
static cusna_status simulate_period(const cusna_saom_problem *pb, cusna_saom_result *r,
                                    int32_t *trace, int32_t trace_cap, const uint32_t *us,
                                    int32_t us_steps) {
    if (!pb || !r) return CUSNA_ERR_NULL_ARG;
    if (pb->struct_version != CUSNA_ABI_VERSION) return CUSNA_ERR_SHAPE;
    const int n = pb->n, W = pb->W, k = pb->k, M = pb->M, kb = pb->kb, nr = pb->nrate;
    if (n < 1 || n > CUSNA_MAX_N || W != (n + 31) / 32 || k < 1 || M < 1) return CUSNA_ERR_SHAPE;
    const size_t nn = (size_t)n * n;
    int i, e, q;

    uint8_t *x0 = (uint8_t *)malloc(nn), *xs = (uint8_t *)malloc(nn);
    uint8_t *kd = (uint8_t *)malloc(nn), *pm = (uint8_t *)malloc(nn);
    uint8_t *keep = (uint8_t *)malloc(nn), *force = (uint8_t *)calloc(nn, 1);
    bits_to_dense(pb->x0_out, n, W, x0);
    bits_to_dense(pb->sim_out ? pb->sim_out : pb->x0_out, n, W, xs);
    if (pb->kdist) bits_to_dense(pb->kdist, n, W, kd); else offdiag(kd, n, 1);
    if (pb->perm) bits_to_dense(pb->perm, n, W, pm); else offdiag(pm, n, 1);
    if (pb->keep_out) bits_to_dense(pb->keep_out, n, W, keep); else offdiag(keep, n, 1);
    if (pb->force_out) bits_to_dense(pb->force_out, n, W, force);

    /* :334-361 parameters and float64 descriptors (theta row 0) */
    double *th = (double *)malloc((size_t)k * sizeof(double));
    double thb[CUSNA_MAXBEFF + 1];
    for (e = 0; e < k; ++e) th[e] = pb->theta[e];
    for (e = 0; e < kb && e < CUSNA_MAXBEFF; ++e) thb[e] = pb->thetab ? pb->thetab[e] : 0.0;
    double *wt = (double *)malloc((size_t)k * (n + 1) * sizeof(double));
    for (size_t x = 0; x < (size_t)k * (n + 1); ++x)
        wt[x] = pb->wtab64 ? pb->wtab64[x] : (pb->wtab ? pb->wtab[x] : 0.0);
    double *p1 = (double *)malloc((size_t)k * sizeof(double));
    double *p2 = (double *)malloc((size_t)k * sizeof(double));
    double *vm = (double *)malloc((size_t)k * n * sizeof(double));
    for (e = 0; e < k; ++e) {
        p1[e] = pb->p1_64 ? pb->p1_64[e] : (pb->p1 ? pb->p1[e] : 0.0);
        p2[e] = pb->p2_64 ? pb->p2_64[e] : (pb->p2 ? pb->p2[e] : 0.0);
    }
    for (size_t x = 0; x < (size_t)k * n; ++x)
        vm[x] = pb->vmat64 ? pb->vmat64[x] : (pb->vmat ? pb->vmat[x] : 0.0);
    double *vb = (double *)malloc((size_t)n * sizeof(double));
    for (i = 0; i < n; ++i) vb[i] = pb->vb64 ? pb->vb64[i] : (pb->vb ? pb->vb[i] : 0.0);
    double ra[CUSNA_MAXRATE] = {0};
    double *ru = (double *)calloc((size_t)(nr ? nr : 1) * n, sizeof(double));
    for (q = 0; q < nr && q < CUSNA_MAXRATE; ++q) ra[q] = pb->ralpha[q];
    for (size_t x = 0; nr && x < (size_t)nr * n; ++x) ru[x] = pb->ru[x];
    double *dym = (double *)calloc(nn, sizeof(double));   /* :354 zero dyadic covariate */
    int32_t *z0 = (int32_t *)calloc((size_t)n, sizeof(int32_t));
    int32_t *bkd = (int32_t *)malloc((size_t)n * sizeof(int32_t));
    int32_t *act = (int32_t *)malloc((size_t)n * sizeof(int32_t));
    uint8_t *inact = (uint8_t *)calloc((size_t)n, 1);
    for (i = 0; i < n && pb->z0; ++i) z0[i] = pb->z0[i];
    for (i = 0; i < n; ++i) bkd[i] = pb->bkdist ? pb->bkdist[i] : 1;
    for (i = 0; i < n; ++i) act[i] = pb->act ? pb->act[i] : i;
    if (pb->has_comp && pb->inactw)
        for (i = 0; i < n; ++i) inact[i] = (uint8_t)((pb->inactw[i >> 5] >> (i & 31)) & 1u);
    int need_tp = 0, need_rdeg = 0;
    for (e = 0; e < k; ++e) { if (pb->type_ids[e] == 5) need_tp = 1; if (pb->type_ids[e] == 19) need_rdeg = 1; }

    octx C;
    memset(&C, 0, sizeof(C));
    C.n = n; C.k = k; C.kb = kb; C.nrate = nr;
    C.x0 = x0; C.xs = xs; C.kd = kd; C.pm = pm;
    C.lam = pb->lam ? pb->lam[0] : 1.0;
    C.lamb = pb->lamb ? pb->lamb[0] : 0.0;
    C.th = th; C.thb = thb;
    C.tid = pb->type_ids; C.ety = pb->etypes; C.dyn = pb->dyn_flags; C.dyi = pb->dyc_idx;
    C.i0 = pb->int0; C.i1 = pb->int1; C.i2 = pb->int2; C.bty = pb->bty; C.rk = pb->rkind;
    C.wt = wt; C.p1 = p1; C.p2 = p2; C.vm = vm; C.dym = dym; C.ra = ra; C.ru = ru;
    C.z0 = z0; C.zmin = pb->zmin; C.zmax = pb->zmax;
    C.zbar = pb->zbar; C.brange = pb->brange; C.bsim = pb->bsimmean;
    C.bkd = bkd; C.act = act; C.nact = pb->act ? pb->nact : n; C.inact = inact;
    C.has_comp = pb->has_comp; C.sym = pb->symflag; C.maxdeg = pb->maxdegree;
    C.cond = pb->conditional; C.target = pb->target_dist;
    C.k0 = (uint32_t)(pb->seed & 0xFFFFFFFFu); C.k1 = (uint32_t)(pb->seed >> 32);
    C.need_tp = need_tp; C.need_rdeg = need_rdeg;
    C.trace = trace_cap > 0 ? trace : NULL; C.trace_cap = trace_cap;
    C.us = us_steps > 0 ? us : NULL; C.us_steps = us_steps;

    /* The reference dereferences etypes, dyn_flags and dyc_idx for every
     * effect; the glue always passes them. Default them here so the oracle
     * also accepts problems that leave them NULL. */
    int32_t *zeros = (int32_t *)calloc((size_t)k, sizeof(int32_t));
    int32_t *minus = (int32_t *)malloc((size_t)k * sizeof(int32_t));
    for (e = 0; e < k; ++e) minus[e] = -1;
    if (!C.ety) C.ety = zeros;
    if (!C.dyn) C.dyn = zeros;
    if (!C.dyi) C.dyi = minus;
    if (!C.i0) C.i0 = minus;
    if (!C.i1) C.i1 = minus;
    if (!C.i2) C.i2 = minus;

    int c;
#ifdef _OPENMP
    int nthr = pb->threads > 0 ? pb->threads : omp_get_max_threads();
    #pragma omp parallel for schedule(static) num_threads(nthr)
#endif
    for (c = 0; c < M; ++c) {
        uint8_t *a = (uint8_t *)malloc(nn);
        int32_t *z = (int32_t *)malloc((size_t)n * sizeof(int32_t));
        double *sc = (double *)malloc((size_t)k * sizeof(double));
        double bsc[CUSNA_MAXBEFF + 1], rsc[CUSNA_MAXRATE + 1];
        long *ad = (long *)malloc((size_t)n * sizeof(long));
        long *ind = (long *)malloc((size_t)n * sizeof(long));
        long *outd = (long *)malloc((size_t)n * sizeof(long));
        double *fj = (double *)malloc((size_t)n * sizeof(double));
        double *dsb = (double *)malloc((size_t)n * k * sizeof(double));
        uint8_t *okb = (uint8_t *)malloc((size_t)n);
        int *tp = (int *)calloc((size_t)n, sizeof(int));
        double *crate = (double *)malloc((size_t)n * sizeof(double));
        double *wsum = (double *)malloc((size_t)k * sizeof(double));
        ochain o;
        int x, y;
        run_chain(&C, (uint32_t)c, a, z, sc, bsc, rsc, ad, ind, outd, fj, dsb, okb, tp, crate, wsum, &o);
        if (r->dist) r->dist[c] = (int32_t)o.dist;
        if (r->dist_stat) r->dist_stat[c] = (int32_t)o.dist_stat;
        if (r->steps) r->steps[c] = (int32_t)o.steps;
        if (r->ntim) r->ntim[c] = o.t;
        if (r->scores) {
            r->scores[(size_t)c * (k + 1)] = (float)o.rate_score;
            for (x = 0; x < k; ++x) r->scores[(size_t)c * (k + 1) + 1 + x] = (float)sc[x];
        }
        if (kb > 0) {
            if (r->bdist) r->bdist[c] = (int32_t)(long)o.bdist;
            if (r->z_end) for (x = 0; x < n; ++x) r->z_end[(size_t)c * n + x] = z[x];
            if (r->bscores) {
                r->bscores[(size_t)c * (kb + 1)] = (float)o.brate_score;
                for (x = 0; x < kb; ++x) r->bscores[(size_t)c * (kb + 1) + 1 + x] = (float)bsc[x];
            }
        }
        if (nr > 0) {
            if (r->rscores) for (x = 0; x < nr; ++x) r->rscores[(size_t)c * nr + x] = (float)rsc[x];
            if (r->actor_dist) for (x = 0; x < n; ++x) r->actor_dist[(size_t)c * n + x] = (int32_t)ad[x];
        }
        if (r->want_end_nets && r->a_ends)
            memcpy(r->a_ends + (size_t)c * nn, a, nn);
        if (r->stats) {
            uint8_t *msk = (uint8_t *)malloc(nn);
            for (size_t w = 0; w < nn; ++w) msk[w] = (uint8_t)((a[w] & keep[w]) | force[w]);
            oracle_network_stats(msk, n, k, pb->type_ids, p1, p2, vm, pb->vmiss, pb->dyn_flags,
                                 vb, pb->od0, pb->id0, wt, pb->symflag, r->stats + (size_t)c * k);
            free(msk);
        }
        (void)y;
        free(a); free(z); free(sc); free(ad); free(ind); free(outd); free(fj); free(dsb);
        free(okb); free(tp); free(crate); free(wsum);
    }

    free(x0); free(xs); free(kd); free(pm); free(keep); free(force);
    free(th); free(wt); free(p1); free(p2); free(vm); free(vb); free(ru); free(dym);
    free(z0); free(bkd); free(act); free(inact); free(zeros); free(minus);
    return CUSNA_OK;
}

cusna_status oracle_simulate_period(const cusna_saom_problem *pb, cusna_saom_result *r) {
    return simulate_period(pb, r, NULL, 0, NULL, 0);
}

/* Validation mode (no counterpart in the reference): the same simulation,
 * writing for each ministep s < trace_cap of chain c the record
 * trace[(c*trace_cap + s)*4 ..] = (s, focal actor, choice, distance change),
 * where the choice is the chosen alter of a network ministep (the actor itself
 * for "no change") or -(d + 2) for a behaviour step d in {-1, 0, 1}, and the
 * change is that of the network distance (of the behaviour distance for a
 * behaviour ministep); and, for ministeps s < us_steps, reading the 4 + n
 * words us[((c*us_steps + s)*(4 + n) ..] in place of the Philox outputs: words
 * 0-3 replace counter (s, c, 0, 0), word 4 + j the first output of counter
 * (s, c, 1, j). Records of unused slots are left as they were. */
cusna_status oracle_simulate_period_validate(const cusna_saom_problem *pb, cusna_saom_result *r,
                                             int32_t *trace, int32_t trace_cap,
                                             const uint32_t *us, int32_t us_steps) {
    if (trace_cap < 0 || us_steps < 0 || (trace_cap > 0 && !trace) || (us_steps > 0 && !us))
        return CUSNA_ERR_NULL_ARG;
    return simulate_period(pb, r, trace, trace_cap, us, us_steps);
}

cusna_status oracle_philox4x32(const uint32_t counter[4], const uint32_t key[2], uint32_t out[4]) {
    if (!counter || !key || !out) return CUSNA_ERR_NULL_ARG;
    ph4(counter[0], counter[1], counter[2], counter[3], key[0], key[1], out);
    return CUSNA_OK;
}

/* Dense to out/in bit rows, as the glue packs them (src/cusna_saom_glue.cpp:22-32). */
cusna_status oracle_pack_bits(const uint8_t *dense, int32_t n, uint32_t *out_rows,
                              uint32_t *in_rows, int32_t *W_out) {
    if (!dense || !out_rows || !in_rows) return CUSNA_ERR_NULL_ARG;
    if (n < 1 || n > CUSNA_MAX_N) return CUSNA_ERR_SHAPE;
    int W = (n + 31) / 32;
    memset(out_rows, 0, (size_t)n * W * sizeof(uint32_t));
    memset(in_rows, 0, (size_t)n * W * sizeof(uint32_t));
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j)
            if (dense[(size_t)i * n + j]) {
                out_rows[(size_t)i * W + (j >> 5)] |= 1u << (j & 31);
                in_rows[(size_t)j * W + (i >> 5)] |= 1u << (i & 31);
            }
    if (W_out) *W_out = W;
    return CUSNA_OK;
}

int32_t oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ==== multi-network co-evolution: src/libcusna_saom_cpu.cpp:427-604 ======= */

/* Cross-network change statistic of toggling i->j in the own network, reading
 * the CURRENT dense state aw of the source network (ax: the own network, for
 * type 37). src/libcusna_saom_cpu.cpp:431-444. */
static double cross_change(int t, const uint8_t *aw, const uint8_t *ax, int n, int i, int j,
                           double dl, double parm) {
    switch (t) {
        case 33: return dl * (double)aw[(size_t)i * n + j];
        case 34: return dl * (double)aw[(size_t)j * n + i];
        case 35: return dl * (double)(aw[(size_t)i * n + j] & aw[(size_t)j * n + i]);
        case 36: {
            long c = 0;
            for (int h = 0; h < n; ++h)
                if (aw[(size_t)i * n + h] && aw[(size_t)j * n + h]) ++c;
            return dl * (parm >= 2.0 ? sqrt((double)c) : (double)c);
        }
        case 37: {
            long c = 0;
            for (int h = 0; h < n; ++h)
                if (aw[(size_t)i * n + h] && ax[(size_t)h * n + j]) ++c;
            return dl * (double)c;
        }
    }
    return 0.0;
}

typedef struct {
    int n, k, D, nact, need_tp;
    const uint8_t *a0, *perm;                 /* D*n*n                          */
    const double *lam, *th;                   /* M*D, M*k                       */
    const int32_t *tid, *netof, *netref, *ety, *dyi, *symf, *act;
    const double *wt, *p1, *p2, *vm, *dy;     /* dy: n*n or NULL                */
    uint32_t k0, k1;
} mctx;

/* One unconditional multi-network chain. src/libcusna_saom_cpu.cpp:463-552. */
static void run_chain_multi(const mctx *C, uint32_t chain, uint8_t *a, double *scores,
                            double *rscores, double *ntim, long *steps) {
    const int n = C->n, k = C->k, D = C->D;
    const double *lam_d = C->lam + (size_t)chain * D;
    const double *th = C->th + (size_t)chain * k;
    long *indeg = calloc((size_t)D * n, sizeof(long)), *outdeg = calloc((size_t)D * n, sizeof(long));
    long *msd = calloc((size_t)D, sizeof(long));
    double *df = malloc((size_t)n * sizeof(double)), *wsum = malloc((size_t)k * sizeof(double));
    double *dsb = calloc((size_t)n * k, sizeof(double));
    uint8_t *okb = malloc((size_t)n);
    int *tp = calloc((size_t)n, sizeof(int));
    for (int d = 0; d < D; ++d)
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) {
                uint8_t v = C->a0[((size_t)d * n + i) * n + j];
                a[((size_t)d * n + i) * n + j] = v;
                if (v) { indeg[(size_t)d * n + j]++; outdeg[(size_t)d * n + i]++; }
            }
    double lam_tot = 0.0;
    for (int d = 0; d < D; ++d) lam_tot += lam_d[d];
    for (int e = 0; e < k; ++e) scores[e] = 0.0;
    long ms = 0;
    double t = 0.0;
    uint32_t rr[4];
    for (;;) {
        ph4((uint32_t)ms, chain, 0u, 0u, C->k0, C->k1, rr);
        t += -log(unif(rr[0])) / ((double)C->nact * lam_tot);
        if (t > 1.0) break;
        double uv = unif(rr[1]) * lam_tot;
        int d = 0;
        double acc = lam_d[0];
        while (d < D - 1 && uv >= acc) { d += 1; acc += lam_d[d]; }
        long idx = (long)(unif(rr[2]) * C->nact);
        if (idx >= C->nact) idx = C->nact - 1;
        const int i = C->act[idx];
        uint8_t *ad = a + (size_t)d * n * n;
        const long *ind = indeg + (size_t)d * n, *outd = outdeg + (size_t)d * n;
        if (C->need_tp) {
            for (int h = 0; h < n; ++h) tp[h] = 0;
            for (int x = 0; x < n; ++x)
                if (ad[(size_t)i * n + x])
                    for (int h = 0; h < n; ++h) tp[h] += ad[(size_t)x * n + h];
        }
        double gbest = -1e30, lmax = -1e30;
        int jstar = i;
        for (int j = 0; j < n; ++j) {
            double f = 0.0;
            int ok = 1;
            if (j == i) {
                for (int e = 0; e < k; ++e) dsb[(size_t)j * k + e] = 0.0;
            } else if (!C->perm[((size_t)d * n + i) * n + j]) {
                ok = 0;
            } else {
                const double dl = 1.0 - 2.0 * ad[(size_t)i * n + j];
                for (int e = 0; e < k; ++e) {
                    if (C->netof[e] != d) { dsb[(size_t)j * k + e] = 0.0; continue; }
                    double dd;
                    if (C->tid[e] >= 33) {
                        dd = cross_change(C->tid[e], a + (size_t)C->netref[e] * n * n, ad, n, i, j,
                                          dl, C->p1[e]);
                    } else {
                        const double dyw = (C->dy && C->dyi[e] >= 0)
                                               ? C->dy[((size_t)C->dyi[e] * n + i) * n + j] : 0.0;
                        dd = change_stat(C->tid[e], ad, n, ind, outd, 0, tp,
                                         C->vm[(size_t)e * n + i], C->vm[(size_t)e * n + j], dyw,
                                         C->p1[e], C->p2[e], i, j, dl, C->wt + (size_t)e * (n + 1));
                    }
                    if ((C->ety[e] == 1 && ad[(size_t)i * n + j] == 1) ||
                        (C->ety[e] == 2 && ad[(size_t)i * n + j] == 0)) dd = 0.0;
                    dsb[(size_t)j * k + e] = dd;
                    f += th[e] * dd;
                }
            }
            okb[j] = (uint8_t)ok;
            df[j] = f;
            if (ok && f > lmax) lmax = f;
            ph4((uint32_t)ms, chain, 1u, (uint32_t)j, C->k0, C->k1, rr);
            if (ok) {
                const double g = f - log(-log(unif(rr[0])));
                if (g > gbest || (g == gbest && j < jstar)) { gbest = g; jstar = j; }
            }
        }
        double sume = 0.0;
        for (int e = 0; e < k; ++e) wsum[e] = 0.0;
        for (int j = 0; j < n; ++j)
            if (okb[j]) {
                const double w = exp(df[j] - lmax);
                sume += w;
                for (int e = 0; e < k; ++e) wsum[e] += w * dsb[(size_t)j * k + e];
            }
        for (int e = 0; e < k; ++e)
            if (C->netof[e] == d) scores[e] += dsb[(size_t)jstar * k + e] - wsum[e] / sume;
        ms++;
        msd[d]++;
        if (jstar != i) {
            const int j = jstar;
            const long dl = 1 - 2 * ad[(size_t)i * n + j];
            indeg[(size_t)d * n + j] += dl;
            outdeg[(size_t)d * n + i] += dl;
            ad[(size_t)i * n + j] = (uint8_t)(1 - ad[(size_t)i * n + j]);
            if (C->symf[d]) {
                indeg[(size_t)d * n + i] += dl;
                outdeg[(size_t)d * n + j] += dl;
                ad[(size_t)j * n + i] = (uint8_t)(1 - ad[(size_t)j * n + i]);
            }
        }
        if (ms >= ORACLE_MAX_STEPS) break;
    }
    for (int d = 0; d < D; ++d) rscores[d] = (double)msd[d] / lam_d[d] - (double)C->nact;
    *ntim = t;
    *steps = ms;
    free(indeg); free(outdeg); free(msd); free(df); free(wsum); free(dsb); free(okb); free(tp);
}

/* Entry point. src/libcusna_saom_cpu.cpp:555-604 (composition restore is off
 * there, as here). */
cusna_status oracle_simulate_multi(const cusna_saom_multi_problem *pb,
                                   cusna_saom_multi_result *r) {
    if (!pb || !r) return CUSNA_ERR_NULL_ARG;
    if (pb->struct_version != CUSNA_ABI_VERSION) return CUSNA_ERR_SHAPE;
    const int n = pb->n, W = pb->W, k = pb->k, M = pb->M, D = pb->D;
    if (n < 1 || n > CUSNA_MAX_N || W != (n + 31) / 32 || k < 1 || k > CUSNA_MAXEFF || M < 1 ||
        D < 2 || D > CUSNA_MAXNET)
        return CUSNA_ERR_SHAPE;
    const size_t nn = (size_t)n * n;
    uint8_t *a0 = malloc((size_t)D * nn), *perm = malloc((size_t)D * nn);
    for (int d = 0; d < D; ++d) {
        bits_to_dense(pb->x0_out + (size_t)d * n * W, n, W, a0 + (size_t)d * nn);
        if (pb->perm) bits_to_dense(pb->perm + (size_t)d * n * W, n, W, perm + (size_t)d * nn);
        else { memset(perm + (size_t)d * nn, 1, nn); offdiag(perm + (size_t)d * nn, n, 1); }
    }
    double *lam = malloc((size_t)M * D * sizeof(double)), *th = malloc((size_t)M * k * sizeof(double));
    double *wt = calloc((size_t)k * (n + 1), sizeof(double)), *p1 = calloc((size_t)k, sizeof(double));
    double *p2 = calloc((size_t)k, sizeof(double)), *vm = calloc((size_t)k * n, sizeof(double));
    for (size_t q = 0; q < (size_t)M * D; ++q) lam[q] = pb->lam[q];
    for (size_t q = 0; q < (size_t)M * k; ++q) th[q] = pb->theta[q];
    if (pb->wtab) for (size_t q = 0; q < (size_t)k * (n + 1); ++q) wt[q] = pb->wtab[q];
    for (int e = 0; e < k; ++e) { p1[e] = pb->p1 ? pb->p1[e] : 0.0; p2[e] = pb->p2 ? pb->p2[e] : 0.0; }
    if (pb->vmat) for (size_t q = 0; q < (size_t)k * n; ++q) vm[q] = pb->vmat[q];
    double *dy = NULL;
    if (pb->dyc) { dy = malloc(nn * sizeof(double)); for (size_t q = 0; q < nn; ++q) dy[q] = pb->dyc[q]; }
    int32_t *dyi = malloc((size_t)k * sizeof(int32_t)), *act = malloc((size_t)n * sizeof(int32_t));
    for (int e = 0; e < k; ++e) dyi[e] = pb->dyc_idx ? pb->dyc_idx[e] : -1;
    for (int i = 0; i < n; ++i) act[i] = pb->act ? pb->act[i] : i;
    mctx C;
    C.n = n; C.k = k; C.D = D; C.nact = pb->act ? pb->nact : n;
    C.need_tp = 0;
    for (int e = 0; e < k; ++e) if (pb->type_ids[e] == 5) C.need_tp = 1;
    C.a0 = a0; C.perm = perm; C.lam = lam; C.th = th;
    C.tid = pb->type_ids; C.netof = pb->netof; C.netref = pb->netref; C.ety = pb->etypes;
    C.dyi = dyi; C.symf = pb->symf; C.act = act;
    C.wt = wt; C.p1 = p1; C.p2 = p2; C.vm = vm; C.dy = dy;
    C.k0 = (uint32_t)(pb->seed & 0xFFFFFFFFu); C.k1 = (uint32_t)(pb->seed >> 32);
#pragma omp parallel for schedule(static)
    for (int c = 0; c < M; ++c) {
        uint8_t *a = malloc((size_t)D * nn);
        double *sc = malloc((size_t)k * sizeof(double)), *rs = malloc((size_t)D * sizeof(double));
        double nt;
        long st;
        run_chain_multi(&C, (uint32_t)c, a, sc, rs, &nt, &st);
        if (r->ntim) r->ntim[c] = nt;
        if (r->steps) r->steps[c] = (int32_t)st;
        if (r->rscores) for (int d = 0; d < D; ++d) r->rscores[(size_t)c * D + d] = (float)rs[d];
        if (r->scores) for (int e = 0; e < k; ++e) r->scores[(size_t)c * k + e] = (float)sc[e];
        if (r->a_ends) memcpy(r->a_ends + (size_t)c * D * nn, a, (size_t)D * nn);
        free(a); free(sc); free(rs);
    }
    free(a0); free(perm); free(lam); free(th); free(wt); free(p1); free(p2); free(vm); free(dy);
    free(dyi); free(act);
    return CUSNA_OK;
}

/* Cross-network statistic of M own networks against the source predictor.
 * src/libcusna_saom_cpu.cpp:819-857. */
cusna_status oracle_cross_stats(const uint8_t *a_batch, const uint8_t *wp, int32_t n, int32_t M,
                                int32_t t, double parm, double *out) {
    if (!a_batch || !wp || !out || n < 1 || n > CUSNA_MAX_N || M < 1) return CUSNA_ERR_NULL_ARG;
    const size_t nn = (size_t)n * n;
    double *star = NULL;
    if (t == 36) {
        star = malloc(nn * sizeof(double));
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) {
                long s = 0;
                for (int h = 0; h < n; ++h) s += wp[(size_t)i * n + h] & wp[(size_t)j * n + h];
                star[(size_t)i * n + j] = (parm >= 2.0) ? sqrt((double)s) : (double)s;
            }
    }
    for (int c = 0; c < M; ++c) {
        const uint8_t *a = a_batch + (size_t)c * nn;
        double acc = 0.0;
        switch (t) {
            case 33: for (size_t q = 0; q < nn; ++q) acc += (a[q] & wp[q]); break;
            case 34:
                for (int i = 0; i < n; ++i)
                    for (int j = 0; j < n; ++j) acc += (a[(size_t)i * n + j] & wp[(size_t)j * n + i]);
                break;
            case 35:
                for (int i = 0; i < n; ++i)
                    for (int j = 0; j < n; ++j)
                        acc += (a[(size_t)i * n + j] & wp[(size_t)i * n + j] & wp[(size_t)j * n + i]);
                break;
            case 36: for (size_t q = 0; q < nn; ++q) if (a[q]) acc += star[q]; break;
            case 37:
                for (int i = 0; i < n; ++i)
                    for (int j = 0; j < n; ++j) {
                        if (!a[(size_t)i * n + j]) continue;
                        long s = 0;
                        for (int h = 0; h < n; ++h) s += wp[(size_t)i * n + h] & a[(size_t)h * n + j];
                        acc += (double)s;
                    }
                break;
            default: free(star); return CUSNA_ERR_UNSUPPORTED;
        }
        out[c] = acc;
    }
    free(star);
    return CUSNA_OK;
}

/* Creation / endowment statistic of one typed effect over M end networks.
 * src/libcusna_saom_cpu.cpp:691-714: creation sums F over gained ties of the
 * statistic network ((a & keep) | force, not in x0, not missing at the start);
 * endowment sums F over lost ties of the structural-only statistic network
 * (in x0, not in (a & keepS) | forceS, not missing at the end) and is reported
 * negated. NULL masks: keep/keepS all 1, force/forceS and the missing masks
 * all 0. */
cusna_status oracle_typed_stats(const uint8_t *a_batch, int32_t n, int32_t M, int32_t etype,
                                const double *F, const uint8_t *x0, const uint8_t *keep,
                                const uint8_t *force, const uint8_t *keepS,
                                const uint8_t *forceS, const uint8_t *miss_m,
                                const uint8_t *miss_m1, double *out) {
    if (!a_batch || !F || !x0 || !out || n < 1 || M < 1) return CUSNA_ERR_NULL_ARG;
    const size_t nn = (size_t)n * n;
    for (int c = 0; c < M; ++c) {
        const uint8_t *a = a_batch + (size_t)c * nn;
        double s = 0.0;
        for (size_t q = 0; q < nn; ++q) {
            if (etype == 1) {
                const int st = (a[q] & (keep ? keep[q] : 1)) | (force ? force[q] : 0);
                if (st && !x0[q] && !(miss_m && miss_m[q])) s += F[q];
            } else {
                const int st = (a[q] & (keepS ? keepS[q] : 1)) | (forceS ? forceS[q] : 0);
                if (x0[q] && !st && !(miss_m1 && miss_m1[q])) s += F[q];
            }
        }
        out[c] = etype == 1 ? s : -s;
    }
    return CUSNA_OK;
}

/* sienaGOF auxiliary distributions. src/libcusna_saom_cpu.cpp:716-765.
 * kind 0 / 1: per level L the number of actors whose in- / out-degree is at
 * most levls[L]. kind 2: per level the number of ordered pairs i != j within
 * geodesic distance levls[L] (reachability grown one step at a time from the
 * network, the diagonal cleared after each step), then the unreachable pairs
 * n(n-1) - (pairs within the largest level). */
cusna_status oracle_gof_distribution(const uint8_t *a_batch, int32_t n, int32_t M, int32_t kind,
                                     const int32_t *levls, int32_t nlev, double *out) {
    if (!a_batch || !levls || !out || n < 1 || M < 1 || nlev < 1) return CUSNA_ERR_NULL_ARG;
    const size_t nn = (size_t)n * n;
    if (kind == 0 || kind == 1) {
        int *deg = malloc((size_t)n * sizeof(int));
        for (int c = 0; c < M; ++c) {
            const uint8_t *a = a_batch + (size_t)c * nn;
            memset(deg, 0, (size_t)n * sizeof(int));
            for (int i = 0; i < n; ++i)
                for (int j = 0; j < n; ++j)
                    if (a[(size_t)i * n + j]) deg[kind == 0 ? j : i]++;
            for (int L = 0; L < nlev; ++L) {
                long cnt = 0;
                for (int v = 0; v < n; ++v) cnt += deg[v] <= levls[L];
                out[(size_t)c * nlev + L] = (double)cnt;
            }
        }
        free(deg);
        return CUSNA_OK;
    }
    if (kind != 2) return CUSNA_ERR_UNSUPPORTED;
    int maxk = 0;
    for (int L = 0; L < nlev; ++L) if (levls[L] > maxk) maxk = levls[L];
    uint8_t *cur = malloc(nn), *nxt = malloc(nn);
    long *within = calloc((size_t)maxk + 1, sizeof(long));
    for (int c = 0; c < M; ++c) {
        const uint8_t *a = a_batch + (size_t)c * nn;
        for (size_t q = 0; q < nn; ++q) cur[q] = a[q] != 0;
        for (int k = 1; k <= maxk; ++k) {
            long cnt = 0;
            for (int i = 0; i < n; ++i)
                for (int j = 0; j < n; ++j) cnt += i != j && cur[(size_t)i * n + j];
            within[k] = cnt;
            if (k == maxk) break;
            for (int i = 0; i < n; ++i)
                for (int j = 0; j < n; ++j) {
                    uint8_t r = cur[(size_t)i * n + j];
                    for (int m = 0; !r && m < n; ++m) r = cur[(size_t)i * n + m] && a[(size_t)m * n + j];
                    nxt[(size_t)i * n + j] = r;
                }
            for (int i = 0; i < n; ++i) nxt[(size_t)i * n + i] = 0;
            uint8_t *t = cur; cur = nxt; nxt = t;
        }
        for (int L = 0; L < nlev; ++L) out[(size_t)c * (nlev + 1) + L] = (double)within[levls[L]];
        out[(size_t)c * (nlev + 1) + nlev] = (double)((long)n * (n - 1) - within[maxk]);
    }
    free(cur); free(nxt); free(within);
    return CUSNA_OK;
}
