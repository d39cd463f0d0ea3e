// mom_estimator.cu -- cusna_mom_estimate: the Robbins-Monro Method-of-Moments
// fit of R/mom.R:129-269 in C++ over replayable plans (host code only).
//
// The reference runs its estimator in R (.mom_run, R/mom.R:215-269) and calls
// the simulator once per period and round through the cpp11 glue. Here the
// whole fit sits behind the C ABI: the periods are prepared once per chain
// count as plans (cusna_saom_plan_*: bit rows, descriptors and effect plans in
// device memory the library allocates), a round writes the parameter rows,
// replays the plan's CUDA graph and reads back only the moment outputs, and
// the phase-2 rounds ask for the statistics alone, so the simulator forms no
// score sums there. The Robbins-Monro algebra is the reference's, step for
// step: the score-function derivative summed over periods (R/mom.R:173-182),
// the diagonalised inverse (:184-187), the guarded step (:189-197), the
// default start (:199-211), phases 1-3 (:224-268).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <memory>
#include <random>
#include <string>
#include <vector>

#include "libcusna.h"
#include "mom_host.h"
#include "saom_launch.h"

namespace cusna {
namespace {

void mom_err(const char *fmt, ...) __attribute__((format(printf, 1, 2)));
void mom_err(const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  set_last_error(buf);
}

#define MCU(call)                                                           \
  do {                                                                      \
    cudaError_t e_ = (call);                                                \
    if (e_ != cudaSuccess) {                                                \
      mom_err("%s failed: %s", #call, cudaGetErrorString(e_));             \
      return CUSNA_ERR_CUDA;                                                \
    }                                                                       \
  } while (0)

// ---- one chain count's plan: the periods on the device ------------------------
struct DevMem {
  std::vector<void *> blocks;
  ~DevMem() {
    for (void *b : blocks) cudaFree(b);
  }
  void *alloc(size_t bytes) {
    void *p = nullptr;
    if (cudaMalloc(&p, bytes ? bytes : 1) != cudaSuccess) return nullptr;
    blocks.push_back(p);
    return p;
  }
};

struct Plan {
  int M = 0;
  bool scores = true;
  cusna_saom_plan *plan = nullptr;
  DevMem mem;
  std::vector<cusna_saom_problem> probs;
  std::vector<cusna_saom_result> ress;
  float *theta_dev = nullptr, *lam_dev = nullptr;  // P rows of k, P values
  double *stats_dev = nullptr, *ntim_dev = nullptr;
  float *scores_dev = nullptr;
  int32_t *dstat_dev = nullptr;
  ~Plan() {
    if (plan) cusna_saom_plan_destroy(plan);
  }
};

struct Model {
  const cusna_saom_problem *periods;
  int P, k, p, n;
  bool cond;
  std::vector<double> rate_consts, targets;
};

// A device copy of one host array of cnt elements (null stays null).
template <class T>
cusna_status dev_copy(DevMem &mem, const T *src, size_t cnt, const T **dst, cudaStream_t st) {
  *dst = nullptr;
  if (!src) return CUSNA_OK;
  T *d = (T *)mem.alloc(cnt * sizeof(T));
  if (!d) { mom_err("cudaMalloc of %zu bytes failed", cnt * sizeof(T)); return CUSNA_ERR_CUDA; }
  MCU(cudaMemcpyAsync(d, src, cnt * sizeof(T), cudaMemcpyHostToDevice, st));
  *dst = d;
  return CUSNA_OK;
}

cusna_status make_plan(const Model &m, int M, bool scores, uint64_t *seed_state, cudaStream_t st,
                       std::unique_ptr<Plan> &out) {
  std::unique_ptr<Plan> pl(new Plan());
  pl->M = M;
  pl->scores = scores;
  const int P = m.P, k = m.k;
  pl->theta_dev = (float *)pl->mem.alloc((size_t)P * k * 4);
  pl->lam_dev = (float *)pl->mem.alloc((size_t)P * 4);
  pl->stats_dev = (double *)pl->mem.alloc((size_t)P * M * k * 8);
  pl->ntim_dev = (double *)pl->mem.alloc((size_t)P * M * 8);
  pl->dstat_dev = (int32_t *)pl->mem.alloc((size_t)P * M * 4);
  if (scores) pl->scores_dev = (float *)pl->mem.alloc((size_t)P * M * (k + 1) * 4);
  if (!pl->theta_dev || !pl->lam_dev || !pl->stats_dev || !pl->ntim_dev || !pl->dstat_dev ||
      (scores && !pl->scores_dev)) {
    mom_err("cudaMalloc of the plan's outputs failed");
    return CUSNA_ERR_CUDA;
  }
  MCU(cudaMemsetAsync(pl->theta_dev, 0, (size_t)P * k * 4, st));
  std::vector<float> ones(P, 1.0f);
  MCU(cudaMemcpyAsync(pl->lam_dev, ones.data(), (size_t)P * 4, cudaMemcpyHostToDevice, st));
  pl->probs.resize(P);
  pl->ress.resize(P);
  cusna_status s;
  for (int q = 0; q < P; ++q) {
    const cusna_saom_problem &h = m.periods[q];
    cusna_saom_problem d = h;
    const size_t n = (size_t)h.n, W = (size_t)h.W, kk = (size_t)h.k, nr = (size_t)h.nrate;
    d.M = M;
    d.threads = 0;
    // the Philox key of the period's stream (the plan adds its epoch per round)
    *seed_state = *seed_state * 6364136223846793005ull + 1442695040888963407ull;
    d.seed = *seed_state >> 1;
    d.theta = pl->theta_dev + (size_t)q * k;
    d.lam = pl->lam_dev + q;
    d.lamb = nullptr;
    d.thetab = nullptr;
    d.dyc = nullptr;
    d.keep_in = nullptr;
    d.force_in = nullptr;
    if ((s = dev_copy(pl->mem, h.x0_out, n * W, &d.x0_out, st)) ||
        (s = dev_copy(pl->mem, h.x0_in, n * W, &d.x0_in, st)) ||
        (s = dev_copy(pl->mem, h.sim_out, n * W, &d.sim_out, st)) ||
        (s = dev_copy(pl->mem, h.sim_in, n * W, &d.sim_in, st)) ||
        (s = dev_copy(pl->mem, h.type_ids, kk, &d.type_ids, st)) ||
        (s = dev_copy(pl->mem, h.etypes, kk, &d.etypes, st)) ||
        (s = dev_copy(pl->mem, h.wtab, kk * (n + 1), &d.wtab, st)) ||
        (s = dev_copy(pl->mem, h.p1, kk, &d.p1, st)) ||
        (s = dev_copy(pl->mem, h.p2, kk, &d.p2, st)) ||
        (s = dev_copy(pl->mem, h.vmat, kk * n, &d.vmat, st)) ||
        (s = dev_copy(pl->mem, h.vmiss, kk * n, &d.vmiss, st)) ||
        (s = dev_copy(pl->mem, h.dyc_idx, kk, &d.dyc_idx, st)) ||
        (s = dev_copy(pl->mem, h.int0, kk, &d.int0, st)) ||
        (s = dev_copy(pl->mem, h.int1, kk, &d.int1, st)) ||
        (s = dev_copy(pl->mem, h.int2, kk, &d.int2, st)) ||
        (s = dev_copy(pl->mem, h.dyn_flags, kk, &d.dyn_flags, st)) ||
        (s = dev_copy(pl->mem, h.kdist, n * W, &d.kdist, st)) ||
        (s = dev_copy(pl->mem, h.keep_out, n * W, &d.keep_out, st)) ||
        (s = dev_copy(pl->mem, h.force_out, n * W, &d.force_out, st)) ||
        (s = dev_copy(pl->mem, h.perm, n * W, &d.perm, st)) ||
        (s = dev_copy(pl->mem, h.od0, n, &d.od0, st)) ||
        (s = dev_copy(pl->mem, h.id0, n, &d.id0, st)) ||
        (s = dev_copy(pl->mem, h.act, n, &d.act, st)) ||
        (s = dev_copy(pl->mem, h.inactw, W, &d.inactw, st)) ||
        (s = dev_copy(pl->mem, h.bty, (size_t)h.kb, &d.bty, st)) ||
        (s = dev_copy(pl->mem, h.z0, n, &d.z0, st)) ||
        (s = dev_copy(pl->mem, h.vb, n, &d.vb, st)) ||
        (s = dev_copy(pl->mem, h.bkdist, n, &d.bkdist, st)) ||
        (s = dev_copy(pl->mem, h.rkind, nr, &d.rkind, st)) ||
        (s = dev_copy(pl->mem, h.ralpha, nr, &d.ralpha, st)) ||
        (s = dev_copy(pl->mem, h.ru, nr * n, &d.ru, st)) ||
        (s = dev_copy(pl->mem, h.vmat64, kk * n, &d.vmat64, st)) ||
        (s = dev_copy(pl->mem, h.wtab64, kk * (n + 1), &d.wtab64, st)) ||
        (s = dev_copy(pl->mem, h.vb64, n, &d.vb64, st)) ||
        (s = dev_copy(pl->mem, h.p1_64, kk, &d.p1_64, st)) ||
        (s = dev_copy(pl->mem, h.p2_64, kk, &d.p2_64, st)))
      return s;
    pl->probs[q] = d;
    cusna_saom_result r;
    std::memset(&r, 0, sizeof r);
    r.struct_version = CUSNA_ABI_VERSION;
    r.stats = pl->stats_dev + (size_t)q * M * k;
    r.ntim = pl->ntim_dev + (size_t)q * M;
    r.dist_stat = pl->dstat_dev + (size_t)q * M;
    r.scores = scores ? pl->scores_dev + (size_t)q * M * (k + 1) : nullptr;
    pl->ress[q] = r;
  }
  MCU(cudaStreamSynchronize(st));
  if ((s = cusna_saom_plan_create(pl->probs.data(), pl->ress.data(), P, 1, &pl->plan)) != CUSNA_OK)
    return s;
  out = std::move(pl);
  return CUSNA_OK;
}

// One round: the moment statistics (M x p, summed over periods) and, with
// scores, the per-period pieces (sp, scp) the derivative needs
// (R/mom.R:143-168; the rate statistic is the period's distance plus its
// constant, the rate score the first score column).
struct Round {
  int M;
  std::vector<double> stats;                 // M x p
  std::vector<std::vector<double>> sp, scp;  // per period, M x p
  std::vector<double> ntim;                  // M x P
};

cusna_status simulate_round(const Model &m, Plan &pl, const std::vector<double> &theta,
                            bool use_graph, cudaStream_t st, Round &R) {
  const int P = m.P, k = m.k, p = m.p, M = pl.M;
  const int off = m.cond ? 0 : P;
  std::vector<float> th((size_t)P * k), lam(P);
  for (int q = 0; q < P; ++q) {
    for (int e = 0; e < k; ++e) th[(size_t)q * k + e] = (float)theta[off + e];
    lam[q] = m.cond ? 1.0f : (float)theta[q];
  }
  MCU(cudaMemcpyAsync(pl.theta_dev, th.data(), th.size() * 4, cudaMemcpyHostToDevice, st));
  MCU(cudaMemcpyAsync(pl.lam_dev, lam.data(), lam.size() * 4, cudaMemcpyHostToDevice, st));
  cusna_status s = cusna_saom_plan_launch(pl.plan, (void *)st, use_graph ? 1 : 0);
  if (s != CUSNA_OK) return s;
  std::vector<double> stats((size_t)P * M * k), ntim((size_t)P * M);
  std::vector<int32_t> dstat((size_t)P * M);
  std::vector<float> sc(pl.scores ? (size_t)P * M * (k + 1) : 0);
  MCU(cudaMemcpyAsync(stats.data(), pl.stats_dev, stats.size() * 8, cudaMemcpyDeviceToHost, st));
  MCU(cudaMemcpyAsync(ntim.data(), pl.ntim_dev, ntim.size() * 8, cudaMemcpyDeviceToHost, st));
  MCU(cudaMemcpyAsync(dstat.data(), pl.dstat_dev, dstat.size() * 4, cudaMemcpyDeviceToHost, st));
  if (pl.scores)
    MCU(cudaMemcpyAsync(sc.data(), pl.scores_dev, sc.size() * 4, cudaMemcpyDeviceToHost, st));
  MCU(cudaStreamSynchronize(st));
  R.M = M;
  R.stats.assign((size_t)M * p, 0.0);
  R.ntim.assign((size_t)M * P, 0.0);
  R.sp.assign(pl.scores ? P : 0, std::vector<double>());
  R.scp.assign(pl.scores ? P : 0, std::vector<double>());
  for (int q = 0; q < P; ++q) {
    std::vector<double> sp((size_t)M * p, 0.0), scp;
    if (pl.scores) scp.assign((size_t)M * p, 0.0);
    for (int c = 0; c < M; ++c) {
      const size_t u = (size_t)q * M + c;
      double *row = sp.data() + (size_t)c * p;
      if (!m.cond) row[q] = (double)dstat[u] + m.rate_consts[q];
      for (int e = 0; e < k; ++e) row[off + e] = stats[u * k + e];
      if (pl.scores) {
        double *srow = scp.data() + (size_t)c * p;
        const float *s = sc.data() + u * (k + 1);
        if (!m.cond) srow[q] = (double)s[0];
        for (int e = 0; e < k; ++e) srow[off + e] = (double)s[1 + e];
      }
      R.ntim[(size_t)c * P + q] = ntim[u];
    }
    for (size_t x = 0; x < sp.size(); ++x) R.stats[x] += sp[x];
    if (pl.scores) {
      R.sp[q] = std::move(sp);
      R.scp[q] = std::move(scp);
    }
  }
  return CUSNA_OK;
}

Mat derivative(const Round &R, int p) { return mom_derivative(R.sp, R.scp, R.M, p); }

std::vector<double> guard_step(const Model &m, const std::vector<double> &theta,
                               std::vector<double> step) {
  return mom_guard_step(theta, std::move(step), m.cond ? 0 : m.P);
}

std::vector<double> deviation(const Round &R, const Model &m) {
  std::vector<double> d = mom_col_means(R.stats, R.M, m.p);
  for (int j = 0; j < m.p; ++j) d[j] -= m.targets[j];
  return d;
}

void print_theta(const char *tag, const std::vector<double> &theta) {
  std::fprintf(stderr, "%s theta =", tag);
  for (double x : theta) std::fprintf(stderr, " %.3f", x);
  std::fprintf(stderr, "\n");
}

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

}  // namespace
}  // namespace cusna

using namespace cusna;

extern "C" CUSNA_API cusna_status cusna_mom_estimate(const cusna_saom_problem *periods, int32_t P,
                                                     const double *targets, int32_t p,
                                                     const cusna_mom_options *opts,
                                                     cusna_mom_result *result) {
  set_last_error("");
  if (!periods || !targets || !opts || !result || !result->theta) {
    mom_err("periods, targets, options, result and result->theta are required");
    return CUSNA_ERR_NULL_ARG;
  }
  if (opts->struct_version != CUSNA_ABI_VERSION || result->struct_version != CUSNA_ABI_VERSION) {
    mom_err("options or result struct_version mismatch");
    return CUSNA_ERR_SHAPE;
  }
  if (P < 1) { mom_err("P = %d periods", P); return CUSNA_ERR_SHAPE; }
  const double t_start = now_s();
  Model m;
  m.periods = periods;
  m.P = P;
  m.k = periods[0].k;
  m.n = periods[0].n;
  m.cond = opts->conditional != 0;
  m.p = m.cond ? m.k : P + m.k;
  if (p != m.p) { mom_err("p = %d, the model has %d parameters", p, m.p); return CUSNA_ERR_SHAPE; }
  for (int q = 0; q < P; ++q) {
    const cusna_saom_problem &h = periods[q];
    if (h.struct_version != CUSNA_ABI_VERSION) { mom_err("period %d struct_version", q); return CUSNA_ERR_SHAPE; }
    if (h.k != m.k) { mom_err("period %d has k = %d, period 0 k = %d", q, h.k, m.k); return CUSNA_ERR_SHAPE; }
    if (h.kb != 0 || h.nrate != 0) {
      mom_err("period %d: behaviour and non-basic rate effects are not estimated by this entry point", q);
      return CUSNA_ERR_UNSUPPORTED;
    }
    if ((h.conditional != 0) != m.cond) {
      mom_err("period %d: conditional = %d but the options say %d", q, h.conditional, (int)m.cond);
      return CUSNA_ERR_SHAPE;
    }
  }
  m.targets.assign(targets, targets + p);
  m.rate_consts.assign(P, 0.0);
  if (opts->rate_consts) m.rate_consts.assign(opts->rate_consts, opts->rate_consts + P);
  // control, with mom_control()'s defaults (R/estimate.R:21-28)
  const double firstg = opts->firstg > 0 ? opts->firstg : 0.4;
  const int nsub = opts->nsub > 0 ? opts->nsub : 4;
  std::vector<int> n2(nsub);
  const int n2_def[4] = {40, 40, 60, 80};
  for (int s = 0; s < nsub; ++s) n2[s] = opts->n2 ? opts->n2[s] : n2_def[s < 4 ? s : 3];
  const int batch2 = opts->batch2 > 0 ? opts->batch2 : 256;
  const int n1 = opts->n1 > 0 ? opts->n1 : 1000;
  const int nD = opts->nD > 0 ? opts->nD : 1000;
  const int n3 = opts->n3 > 0 ? opts->n3 : 4000;
  const double diag_w = opts->diagonalize > 0 ? opts->diagonalize : opts->diagonalize < 0 ? 0.0 : 0.2;
  const bool use_graph = opts->use_graph >= 0;
  uint64_t seed_state = opts->seed ? opts->seed : 1234;
  for (int s = 0; s < nsub; ++s)
    if (n2[s] < 1) { mom_err("n2[%d] = %d", s, n2[s]); return CUSNA_ERR_SHAPE; }

  // start: the caller's, or the reference's default (R/mom.R:199-211)
  std::vector<double> theta(p);
  if (result->use_start) {
    theta.assign(result->theta, result->theta + p);
  } else {
    std::vector<int32_t> tid(m.k);
    std::memcpy(tid.data(), periods[0].type_ids, (size_t)m.k * 4);
    const int off = m.cond ? 0 : P;
    for (int q = 0; q < off; ++q) theta[q] = 1.5 * m.targets[q] / m.n + 1.0;
    for (int e = 0; e < m.k; ++e) theta[off + e] = tid[e] == 0 ? -1.0 : 0.0;
  }

  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    mom_err("no CUDA device");
    return CUSNA_ERR_NO_CUDA;
  }
  cudaStream_t st = nullptr;
  MCU(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  struct StreamGuard {
    cudaStream_t s;
    ~StreamGuard() { cudaStreamDestroy(s); }
  } guard{st};

  // one plan per (chain count, scores): phase 1, the subphase derivatives,
  // phase 3 with scores; the phase-2 iterations without
  std::vector<std::unique_ptr<Plan>> plans;
  auto plan_for = [&](int M, bool scores, Plan **out) -> cusna_status {
    for (auto &pl : plans)
      if (pl->M == M && pl->scores == scores) { *out = pl.get(); return CUSNA_OK; }
    std::unique_ptr<Plan> pl;
    cusna_status s = make_plan(m, M, scores, &seed_state, st, pl);
    if (s != CUSNA_OK) return s;
    if (opts->verbose) std::fprintf(stderr, "[plan] %d periods x %d chains%s\n", P, M, scores ? "" : ", no scores");
    plans.push_back(std::move(pl));
    *out = plans.back().get();
    return CUSNA_OK;
  };
  auto round = [&](int M, bool scores, Round &R) -> cusna_status {
    Plan *pl = nullptr;
    cusna_status s = plan_for(M, scores, &pl);
    if (s != CUSNA_OK) return s;
    return simulate_round(m, *pl, theta, use_graph, st, R);
  };

  cusna_status s;
  Round R;
  // phase 1 (R/mom.R:224-229)
  double t0 = now_s();
  std::unique_ptr<NvtxRange> range(new NvtxRange("mom phase 1"));
  if ((s = round(n1, true, R)) != CUSNA_OK) return s;
  {
    const Mat di = mom_dinv(derivative(R, p), p, diag_w);
    std::vector<double> step = mom_matvec(di, deviation(R, m), p);
    for (double &x : step) x *= 0.5 * firstg;
    step = guard_step(m, theta, step);
    for (int j = 0; j < p; ++j) theta[j] -= step[j];
  }
  result->phase_seconds[0] = now_s() - t0;
  if (opts->verbose) print_theta("[phase 1]", theta);
  // phase 2 (R/mom.R:233-248)
  t0 = now_s();
  range.reset();  // ranges nest: the old one ends before the next begins
  range.reset(new NvtxRange("mom phase 2"));
  for (int sub = 0; sub < nsub; ++sub) {
    const double gain = firstg * std::pow(0.5, sub);
    if ((s = round(nD, true, R)) != CUSNA_OK) return s;
    const Mat di = mom_dinv(derivative(R, p), p, diag_w);
    std::vector<double> thav(p, 0.0);
    for (int it = 0; it < n2[sub]; ++it) {
      if ((s = round(batch2, false, R)) != CUSNA_OK) return s;
      std::vector<double> step = mom_matvec(di, deviation(R, m), p);
      for (double &x : step) x *= gain;
      step = guard_step(m, theta, step);
      for (int j = 0; j < p; ++j) {
        theta[j] -= step[j];
        thav[j] += theta[j];
      }
    }
    for (int j = 0; j < p; ++j) theta[j] = thav[j] / n2[sub];
    if (opts->verbose) {
      char tag[64];
      std::snprintf(tag, sizeof tag, "[phase 2.%d] gain=%.3f", sub + 1, gain);
      print_theta(tag, theta);
    }
  }
  result->phase_seconds[1] = now_s() - t0;
  // phase 3 (R/mom.R:250-258)
  t0 = now_s();
  range.reset();
  range.reset(new NvtxRange("mom phase 3"));
  if ((s = round(n3, true, R)) != CUSNA_OK) return s;
  const Mat D = derivative(R, p);
  const Mat dinv = mom_safe_solve(D, p);
  const std::vector<double> mu = mom_col_means(R.stats, R.M, p);
  Mat msf((size_t)p * p, 0.0);
  for (int c = 0; c < R.M; ++c)
    for (int a = 0; a < p; ++a) {
      const double x = R.stats[(size_t)c * p + a] - mu[a];
      for (int b = 0; b < p; ++b) msf[(size_t)a * p + b] += x * (R.stats[(size_t)c * p + b] - mu[b]);
    }
  for (double &x : msf) x /= (R.M - 1);
  std::vector<double> dev(p);
  for (int j = 0; j < p; ++j) dev[j] = mu[j] - m.targets[j];
  const std::vector<double> md = mom_matvec(mom_safe_solve(msf, p), dev, p);
  double q2 = 0.0;
  for (int j = 0; j < p; ++j) q2 += dev[j] * md[j];
  // cov = dinv msf dinv^T
  Mat tmp((size_t)p * p, 0.0), cov((size_t)p * p, 0.0);
  for (int a = 0; a < p; ++a)
    for (int b = 0; b < p; ++b)
      for (int c = 0; c < p; ++c) tmp[(size_t)a * p + b] += dinv[(size_t)a * p + c] * msf[(size_t)c * p + b];
  for (int a = 0; a < p; ++a)
    for (int b = 0; b < p; ++b)
      for (int c = 0; c < p; ++c) cov[(size_t)a * p + b] += tmp[(size_t)a * p + c] * dinv[(size_t)b * p + c];
  result->phase_seconds[2] = now_s() - t0;
  range.reset();

  for (int j = 0; j < p; ++j) {
    result->theta[j] = theta[j];
    if (result->se) result->se[j] = std::sqrt(std::fabs(cov[(size_t)j * p + j]));
    if (result->tconv) result->tconv[j] = dev[j] / std::sqrt(msf[(size_t)j * p + j]);
    if (result->sim_means) result->sim_means[j] = mu[j];
  }
  // conditional fits estimate the rates from the simulated times (R/mom.R:260-266)
  for (int q = 0; q < P && m.cond; ++q) {
    double a = 0.0, b = 0.0;
    for (int c = 0; c < R.M; ++c) a += R.ntim[(size_t)c * P + q];
    a /= R.M;
    for (int c = 0; c < R.M; ++c) b += (R.ntim[(size_t)c * P + q] - a) * (R.ntim[(size_t)c * P + q] - a);
    if (result->rate_est) result->rate_est[q] = a;
    if (result->rate_sd) result->rate_sd[q] = std::sqrt(b / (R.M - 1));
  }
  if (result->D) std::memcpy(result->D, D.data(), D.size() * 8);
  if (result->msf) std::memcpy(result->msf, msf.data(), msf.size() * 8);
  result->tconv_max = std::sqrt(std::max(q2, 0.0));
  long long n_sims = (long long)n1 + n3;
  for (int sub = 0; sub < nsub; ++sub) n_sims += nD + (long long)n2[sub] * batch2;
  result->n_sims = n_sims;
  result->wall_seconds = now_s() - t_start;
  return CUSNA_OK;
}
