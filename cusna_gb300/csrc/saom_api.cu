// saom_api.cu -- host side of libcusna_gb300: argument validation with the
// reference's status codes, a per-thread device arena and stream, input
// preparation, the launch-shape autotuner, and the C ABI of include/libcusna.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "libcusna.h"
#include "saom_jit.h"
#include "saom_launch.h"
#include "saom_stats.cuh"

namespace cusna {
namespace {

thread_local std::string g_err;

void set_err(const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_err = buf;
}

#define CU(call)                                                                        \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess) {                                                            \
      set_err("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
      return CUSNA_ERR_CUDA;                                                            \
    }                                                                                   \
  } while (0)

// Per-thread device state: stream, growable device arena, device properties.
struct Ctx {
  int device = -1;
  int sms = 0;
  int smem_sm = 0, smem_optin = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  void *arena = nullptr;
  size_t cap = 0;
  ~Ctx() {
    // the CUDA runtime may already be torn down at thread exit; free best-effort
    if (arena) cudaFree(arena);
  }
};
thread_local Ctx g_ctx;

cusna_status ensure_ctx() {
  Ctx &c = g_ctx;
  if (c.device >= 0) return CUSNA_OK;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count < 1) {
    cudaGetLastError();
    set_err("no CUDA device");
    return CUSNA_ERR_NO_CUDA;
  }
  int dev = 0;
  CU(cudaGetDevice(&dev));
  CU(cudaDeviceGetAttribute(&c.sms, cudaDevAttrMultiProcessorCount, dev));
  CU(cudaDeviceGetAttribute(&c.smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
  CU(cudaDeviceGetAttribute(&c.smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  CU(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
  CU(cudaEventCreate(&c.ev0));
  CU(cudaEventCreate(&c.ev1));
  c.device = dev;
  return CUSNA_OK;
}

cusna_status ensure_arena(size_t bytes) {
  Ctx &c = g_ctx;
  if (bytes <= c.cap) return CUSNA_OK;
  if (c.arena) {
    CU(cudaStreamSynchronize(c.stream));
    CU(cudaFree(c.arena));
    c.arena = nullptr;
    c.cap = 0;
  }
  size_t want = std::max(bytes, (size_t)64 << 20);
  want = std::max(want, bytes + bytes / 4);
  CU(cudaMalloc(&c.arena, want));
  c.cap = want;
  return CUSNA_OK;
}

// Bump planner over the arena: first pass records sizes, then pointers.
struct Planner {
  size_t off = 0;
  size_t take(size_t bytes) {
    const size_t o = off;
    off = (off + bytes + 255) & ~(size_t)255;
    return o;
  }
};

template <class T>
T *at(size_t off) {
  return reinterpret_cast<T *>(static_cast<char *>(g_ctx.arena) + off);
}


// Per-problem host-side facts read during validation, and the effect plan.
struct Facts {
  std::vector<int> tid, i0, i1, i2, rk, ety;
  // effect plan of the specialised kernel (saom_jit.h): with the problem's
  // actor count compiled in (spec_w), and with it read at run time (spec)
  std::string spec, spec_w;
  JitPlan jplan;
  int flags = 0;
  std::vector<int> kind, cfn, offd, offt;  // effect plan, k each
  std::vector<int> tsize;                  // theta-table length per effect (0: none)
  // multi-network problems: one network's effects as a problem of their own
  bool multi = false;
  std::vector<int> cross_src;              // source network per effect (cross effects)
  std::vector<int> dci;                    // dyadic covariate index per effect (-1 none)
  std::vector<double> dyc;                 // the dyadic covariate, n*n (empty: none)
  std::vector<double> pool;                // its tables
  int zlo = 0, zR = 1;
};

template <class T>
cusna_status fetch_vec(const T *src, size_t cnt, bool dev, std::vector<T> &dst) {
  dst.clear();
  if (!src || cnt == 0) return CUSNA_OK;
  dst.resize(cnt);
  if (dev) CU(cudaMemcpy(dst.data(), src, cnt * sizeof(T), cudaMemcpyDeviceToHost));
  else std::memcpy(dst.data(), src, cnt * sizeof(T));
  return CUSNA_OK;
}

// float64 descriptor with the CPU engine's precedence (*64, else float, else 0)
cusna_status fetch_desc(const double *d64, const float *d32, size_t cnt, bool dev,
                        std::vector<double> &out) {
  out.assign(cnt, 0.0);
  cusna_status s;
  if (d64) return fetch_vec(d64, cnt, dev, out);
  if (d32) {
    std::vector<float> f;
    if ((s = fetch_vec(d32, cnt, dev, f)) != CUSNA_OK) return s;
    for (size_t q = 0; q < cnt; ++q) out[q] = (double)f[q];
  }
  return CUSNA_OK;
}

// Dyadic covariate magnitude of types 12, 20, 21, 25 for covariate values
// (vi, vj): the expressions of src/libcusna_saom_cpu.cpp:72,80-81,84 without the
// delta factor (this file is compiled without floating-point contraction).
double dyad_value(int t, double vi, double vj, double q1, double q2) {
  switch (t) {
    case 12: return 1.0 - std::fabs(vi - vj) * q1 - q2;
    case 20: return vi > vj + 1e-9 ? 1.0 : (std::fabs(vi - vj) <= 1e-9 ? 0.5 : 0.0);
    case 21: return vi * vj;
    default: return vi + vj;  // 25
  }
}

// The effect plan (see K_* in saom_common.cuh): per effect how the kernel
// forms d and theta*d, and the tables it reads. Term tables (theta * magnitude)
// are built when every chain has the same theta, the usual case; otherwise the
// kernel multiplies.
cusna_status build_plan(const cusna_saom_problem *p, bool dev, Facts &F, bool one_row) {
  const int n = p->n, k = p->k, M = one_row ? 1 : p->M;
  cusna_status s;
  std::vector<float> th;
  if ((s = fetch_vec(p->theta, (size_t)M * k, dev, th)) != CUSNA_OK) return s;
  bool uniform = true;
  for (int c = 1; c < M && uniform; ++c)
    if (std::memcmp(&th[(size_t)c * k], &th[0], k * sizeof(float)) != 0) uniform = false;
  std::vector<double> vm, wt, p1, p2;
  std::vector<int> dyn, z0;
  if ((s = fetch_desc(p->vmat64, p->vmat, (size_t)k * n, dev, vm)) != CUSNA_OK) return s;
  if ((s = fetch_desc(p->wtab64, p->wtab, (size_t)k * (n + 1), dev, wt)) != CUSNA_OK) return s;
  if ((s = fetch_desc(p->p1_64, p->p1, (size_t)k, dev, p1)) != CUSNA_OK) return s;
  if ((s = fetch_desc(p->p2_64, p->p2, (size_t)k, dev, p2)) != CUSNA_OK) return s;
  if ((s = fetch_vec(p->dyn_flags, (size_t)k, dev, dyn)) != CUSNA_OK) return s;
  if ((s = fetch_vec(p->z0, (size_t)n, dev, z0)) != CUSNA_OK) return s;
  if (dyn.empty()) dyn.assign(k, 0);
  if (z0.empty()) z0.assign(n, 0);
  bool has_dyn = false;
  for (int e = 0; e < k; ++e) has_dyn |= dyn[e] != 0;
  const bool has_z = p->kb > 0 || has_dyn;
  // reachable behaviour values: the start values and, with behaviour
  // dynamics, [zmin, zmax] (a ministep moves z by one within those bounds)
  long long lo = *std::min_element(z0.begin(), z0.end()), hi = *std::max_element(z0.begin(), z0.end());
  if (p->kb > 0) { lo = std::min<long long>(lo, p->zmin); hi = std::max<long long>(hi, p->zmax); }
  const long long zR = hi - lo + 1;
  const double zbar = (double)p->zbar;
  const bool zalt_ok = has_z && zR <= 65536;
  const bool zdyad_ok = has_z && zR <= 256;
  F.zlo = (int)lo;
  F.zR = (int)std::max<long long>(1, std::min<long long>(zR, 65536));
  F.kind.assign(k, K_GEN); F.cfn.assign(k, 0); F.offd.assign(k, 0); F.offt.assign(k, 0);
  F.tsize.assign(k, 0);
  F.pool.clear();
  auto add = [&](size_t cnt) { const size_t o = F.pool.size(); F.pool.resize(o + cnt, 0.0); return (int)o; };
  auto cnt_table = [&](int e, int cfn, size_t size) {
    F.kind[e] = K_CNT; F.cfn[e] = cfn;
    if (uniform) {
      F.offt[e] = add(size);
      F.tsize[e] = (int)size;
      for (size_t c = 0; c < size; ++c) F.pool[F.offt[e] + c] = (double)th[e] * (double)c;
    }
  };
  auto look_table = [&](int e, int cfn, size_t size, auto value) {
    F.kind[e] = K_LOOK; F.cfn[e] = cfn;
    F.offd[e] = add(size);
    for (size_t x = 0; x < size; ++x) F.pool[F.offd[e] + x] = value(x);
    if (uniform) {
      F.offt[e] = add(size);
      F.tsize[e] = (int)size;
      for (size_t x = 0; x < size; ++x) F.pool[F.offt[e] + x] = (double)th[e] * F.pool[F.offd[e] + x];
    }
  };
  const size_t N = (size_t)n;
  int fl = 0;
  for (int e = 0; e < k; ++e) {
    const int t = F.tid[e];
    const double *v = &vm[(size_t)e * n];
    switch (t) {
      case 0: cnt_table(e, 0, 2); break;
      case 1: cnt_table(e, 1, 2); break;
      case 2: cnt_table(e, 2, 2 * N + 1); break;
      case 3: case 23: cnt_table(e, 3, N + 1); break;
      case 4: cnt_table(e, 4, N + 2); break;
      case 5: cnt_table(e, 5, 2 * N + 2); break;
      case 6: cnt_table(e, 6, 2 * N + 1); break;
      case 8: cnt_table(e, 7, N + 1); break;
      case 7: look_table(e, 4, N + 2, [](size_t c) { return std::sqrt((double)c); }); break;
      case 9: look_table(e, 7, N + 1, [](size_t c) { return std::sqrt((double)c); }); break;
      case 10: case 14: case 15: case 16: case 17: case 18: case 19:
        F.kind[e] = K_STEP; fl |= F_HAS_STEP; break;
      case 11: case 31: {
        const double q1 = p1[e];
        auto f = [&](double x) { return t == 11 ? x : (x >= q1 - 1e-12 ? 1.0 : 0.0); };
        if (dyn[e]) {
          if (zalt_ok) look_table(e, 13, (size_t)zR, [&](size_t x) { return f((double)(lo + (long long)x) - zbar); });
        } else {
          look_table(e, 12, N, [&](size_t j) { return f(v[j]); });
        }
        break;
      }
      case 12: case 20: case 21: case 25: {
        const double q1 = p1[e], q2 = p2[e];
        if (dyn[e]) {
          if (zdyad_ok)
            look_table(e, 15, (size_t)(zR * zR), [&](size_t x) {
              const double vi = (double)(lo + (long long)(x / zR)) - zbar;
              const double vj = (double)(lo + (long long)(x % zR)) - zbar;
              return dyad_value(t, vi, vj, q1, q2);
            });
        } else if (n <= 1024) {
          look_table(e, 14, N * N, [&](size_t x) { return dyad_value(t, v[x / N], v[x % N], q1, q2); });
        }
        break;
      }
      case 22:
        // a dyadic covariate: the multi-network engine reads it
        // (src/libcusna_saom_cpu.cpp:509), the single-network one zero-fills
        if (F.multi && !F.dyc.empty() && F.dci[e] == 0)
          look_table(e, 14, N * N, [&](size_t x) { return F.dyc[x]; });
        else
          F.kind[e] = K_ZERO;
        break;
      case 33: case 34: case 35: case 36: case 37:
        // cross-network effects read another network of a multi-network
        // problem; a single-network problem has none, and the reference's
        // change statistic of these types there is 0
        if (F.multi) { F.kind[e] = K_CROSS; F.cfn[e] = t; F.offd[e] = F.cross_src[e]; }
        else F.kind[e] = K_ZERO;
        break;
      case 24: look_table(e, 8, N + 1, [&](size_t c) { return wt[(size_t)e * (n + 1) + c]; }); break;
      case 26: look_table(e, 9, N + 1, [&](size_t c) { return wt[(size_t)e * (n + 1) + c]; }); break;
      case 27: look_table(e, 10, N + 1, [&](size_t c) { return wt[(size_t)e * (n + 1) + c]; }); break;
      case 28: look_table(e, 11, N + 1, [&](size_t c) { return wt[(size_t)e * (n + 1) + c]; }); break;
      case 32:
        // interactions are formed from their components in the single-network
        // engine; the multi-network change statistic of the type is 0
        if (F.multi) F.kind[e] = K_ZERO;
        break;
      case 13: case 29: case 30: break;  // K_GEN
      default: F.kind[e] = K_ZERO; break;       // unknown ids: the reference's 0
    }
  }
  if (F.pool.empty()) F.pool.push_back(0.0);
  if (uniform) fl |= F_THETA_TAB;
  if (has_z) fl |= F_HAS_Z;
  F.flags |= fl;
  return CUSNA_OK;
}

// one_row: the parameter arrays hold one row shared by every chain (plans).
cusna_status validate(const cusna_saom_problem *p, const cusna_saom_result *r, bool dev,
                      Facts &F, bool one_row = false) {
  if (!p || !r) { set_err("problem or result is NULL"); return CUSNA_ERR_NULL_ARG; }
  if (p->struct_version != CUSNA_ABI_VERSION) {
    set_err("struct_version %d != %d", p->struct_version, CUSNA_ABI_VERSION);
    return CUSNA_ERR_SHAPE;
  }
  const int n = p->n, k = p->k;
  if (n < 1 || n > CUSNA_MAX_N || p->W != (n + 31) / 32 || k < 1 || p->M < 1) {
    set_err("bad shape n=%d W=%d k=%d M=%d", n, p->W, k, p->M);
    return CUSNA_ERR_SHAPE;
  }
  if (k > CUSNA_MAXEFF || p->kb < 0 || p->kb > CUSNA_MAXBEFF || p->nrate < 0 ||
      p->nrate > CUSNA_MAXRATE) {
    set_err("capacity exceeded k=%d kb=%d nrate=%d", k, p->kb, p->nrate);
    return CUSNA_ERR_SHAPE;
  }
  if (!p->x0_out || !p->theta || !p->lam || !p->type_ids) {
    set_err("x0_out, theta, lam and type_ids are required");
    return CUSNA_ERR_NULL_ARG;
  }
  if (p->kb > 0 && !p->bty) { set_err("bty is required when kb > 0"); return CUSNA_ERR_NULL_ARG; }
  if (p->nrate > 0 && (!p->rkind || !p->ralpha || !p->ru)) {
    set_err("rkind, ralpha and ru are required when nrate > 0");
    return CUSNA_ERR_NULL_ARG;
  }
  if (p->act && (p->nact < 1 || p->nact > n)) { set_err("nact %d out of range", p->nact); return CUSNA_ERR_SHAPE; }
  auto fetch = [&](const int32_t *src, int cnt, std::vector<int> &dst, int def) -> cusna_status {
    dst.assign(cnt, def);
    if (!src || cnt == 0) return CUSNA_OK;
    if (dev) CU(cudaMemcpy(dst.data(), src, cnt * sizeof(int), cudaMemcpyDeviceToHost));
    else std::memcpy(dst.data(), src, cnt * sizeof(int));
    return CUSNA_OK;
  };
  cusna_status s;
  if ((s = fetch(p->type_ids, k, F.tid, 0)) != CUSNA_OK) return s;
  if ((s = fetch(p->int0, k, F.i0, -1)) != CUSNA_OK) return s;
  if ((s = fetch(p->int1, k, F.i1, -1)) != CUSNA_OK) return s;
  if ((s = fetch(p->int2, k, F.i2, -1)) != CUSNA_OK) return s;
  if ((s = fetch(p->rkind, p->nrate, F.rk, 0)) != CUSNA_OK) return s;
  if ((s = fetch(p->etypes, k, F.ety, 0)) != CUSNA_OK) return s;
  if (p->act) {
    std::vector<int> act;
    if ((s = fetch(p->act, p->nact, act, 0)) != CUSNA_OK) return s;
    for (int v : act)
      if (v < 0 || v >= n) { set_err("act entry %d out of range", v); return CUSNA_ERR_SHAPE; }
  }
  int fl = 0;
  for (int e = 0; e < k; ++e) {
    const int t = F.tid[e];
    switch (t) {
      case 2: fl |= F_PC_RI_CJ | F_PC_RI_RJ; break;
      case 3: case 23: fl |= F_PC_RJ_CI; break;
      case 5: fl |= F_NEED_TP; break;
      case 6: fl |= F_PC_RI_CJ | F_PC_RICIRJ; break;
      case 19:
        // the multi-network engine passes a reciprocated degree of 0
        // (src/libcusna_saom_cpu.cpp:510)
        if (!F.multi) fl |= F_NEED_RDEG;
        break;
      case 24: fl |= F_PC_RI_CJ; break;
      case 26: fl |= F_PC_RI_RJ; break;
      case 27: fl |= F_PC_CI_CJ; break;
      case 28: fl |= F_PC_CI_RJ; break;
      case 29: fl |= F_NEED_GW29; break;
      case 30: fl |= F_NEED_GW30; break;
      case 32:
        if (F.multi) break;
        fl |= F_HAS_INTER;
        if (F.i0[e] < 0 || F.i0[e] >= e || F.i1[e] < 0 || F.i1[e] >= e || F.i2[e] >= e) {
          set_err("interaction %d: components must be earlier effects", e);
          return CUSNA_ERR_SHAPE;
        }
        break;
      default: break;
    }
  }
  F.flags = fl;
  if ((s = build_plan(p, dev, F, one_row)) != CUSNA_OK) return s;
  {
    JitPlan &J = F.jplan;
    J.pc_flags = F.flags & (F_PC_RI_CJ | F_PC_RI_RJ | F_PC_RJ_CI | F_PC_CI_CJ | F_PC_CI_RJ |
                            F_PC_RICIRJ);
    J.kind = F.kind; J.cfn = F.cfn; J.tid = F.tid; J.ety = F.ety;
    J.i0 = F.i0; J.i1 = F.i1; J.i2 = F.i2;
    if (!F.multi) {
      F.spec = jit_spec_source(J);
      J.n = p->n;
      F.spec_w = jit_spec_source(J);
      J.n = 0;
    }
  }
  // gwdsp change statistics index the weight table at p+1 with p <= n-2 on a
  // network without self-ties; a self-tie in the start network could push p to
  // n and read past the table, so such problems are rejected
  if (fl & (F_NEED_GW29 | F_NEED_GW30)) {
    const int W = p->W;
    std::vector<uint32_t> rows((size_t)n * W);
    for (const uint32_t *src : {p->x0_out, p->sim_out}) {
      if (!src) continue;
      if (dev) CU(cudaMemcpy(rows.data(), src, rows.size() * 4, cudaMemcpyDeviceToHost));
      else std::memcpy(rows.data(), src, rows.size() * 4);
      for (int i = 0; i < n; ++i)
        if ((rows[(size_t)i * W + (i >> 5)] >> (i & 31)) & 1u) {
          set_err("gwdsp effects need a start network without self-ties (actor %d)", i);
          return CUSNA_ERR_SHAPE;
        }
    }
  }
  return CUSNA_OK;
}

// Sizes of the arrays a problem points at (for host -> device copies).
struct RawSizes {
  size_t rows, theta, lam, lamb, thetab, k4, k8, kn8, kn4f, kn1, wt8, wt4, n4, n8, n4f, W4, ru8,
      ru4f, r4, rf;
};

// Device layout of one prepared problem.
struct ProbBufs {
  size_t x0T, x0cT, simT, simcT, kdistT, permT, keepT, forceT, keepcT, forcecT;
  size_t vmat, wtab, p1, p2, vb, ralpha, ru;
  size_t etypes, dyn, i0, i1, i2, act, z0, bkdist, inact, vmiss;
  size_t ekind, ecfn, eoffd, eofft, pool, pool2;
  // raw copies (host mode)
  size_t r_x0, r_sim, r_kd, r_pm, r_keep, r_force, r_theta, r_lam, r_lamb, r_thetab, r_tid,
      r_ety, r_dyn, r_i0, r_i1, r_i2, r_vmat64, r_vmat32, r_wtab64, r_wtab32, r_p164, r_p132,
      r_p264, r_p232, r_vb64, r_vb32, r_vmiss, r_od0, r_id0, r_act, r_inact, r_z0, r_bkd, r_bty,
      r_rk, r_ra, r_ru;
  // outputs (host mode)
  size_t o_stats, o_ntim, o_scores, o_dist, o_dstat, o_steps, o_bdist, o_bscores, o_zend,
      o_rscores, o_adist, o_aends;
};

const size_t NONE = ~(size_t)0;

struct Job {
  const cusna_saom_problem *p;
  cusna_saom_result *r;
  Facts F;
  ProbBufs B;
};

size_t maybe(Planner &pl, const void *ptr, size_t bytes) {
  return ptr ? pl.take(bytes) : NONE;
}

void plan_problem(Planner &pl, Job &J, bool dev) {
  const cusna_saom_problem *p = J.p;
  const cusna_saom_result *r = J.r;
  const size_t n = p->n, W = p->W, k = p->k, M = p->M, kb = p->kb, nr = p->nrate;
  const size_t bits = W * n * 4;
  ProbBufs &B = J.B;
  B.x0T = pl.take(bits); B.x0cT = pl.take(bits); B.simT = pl.take(bits); B.simcT = pl.take(bits);
  B.kdistT = pl.take(bits); B.permT = pl.take(bits); B.keepT = pl.take(bits);
  B.forceT = pl.take(bits); B.keepcT = pl.take(bits); B.forcecT = pl.take(bits);
  B.vmat = pl.take(k * n * 8); B.wtab = pl.take(k * (n + 1) * 8);
  B.p1 = pl.take(k * 8); B.p2 = pl.take(k * 8); B.vb = pl.take(n * 8);
  B.ralpha = pl.take((nr + 1) * 8); B.ru = pl.take((nr + 1) * n * 8);
  B.etypes = pl.take(k * 4); B.dyn = pl.take(k * 4); B.i0 = pl.take(k * 4);
  B.i1 = pl.take(k * 4); B.i2 = pl.take(k * 4); B.act = pl.take(n * 4);
  B.z0 = pl.take(n * 4); B.bkdist = pl.take(n * 4); B.inact = pl.take(W * 4);
  B.vmiss = NONE;
  B.ekind = pl.take(k * 4); B.ecfn = pl.take(k * 4); B.eoffd = pl.take(k * 4);
  B.eofft = pl.take(k * 4); B.pool = pl.take(J.F.pool.size() * 8);
  B.pool2 = pl.take(J.F.pool.size() * 8);
  if (!dev) {
    B.r_x0 = pl.take(n * W * 4);
    B.r_sim = maybe(pl, p->sim_out, n * W * 4);
    B.r_kd = maybe(pl, p->kdist, n * W * 4);
    B.r_pm = maybe(pl, p->perm, n * W * 4);
    B.r_keep = maybe(pl, p->keep_out, n * W * 4);
    B.r_force = maybe(pl, p->force_out, n * W * 4);
    B.r_theta = pl.take(M * k * 4);
    B.r_lam = pl.take(M * 4);
    B.r_lamb = maybe(pl, p->lamb, M * 4);
    B.r_thetab = maybe(pl, p->thetab, M * kb * 4);
    B.r_tid = pl.take(k * 4);
    B.r_ety = maybe(pl, p->etypes, k * 4);
    B.r_dyn = maybe(pl, p->dyn_flags, k * 4);
    B.r_i0 = maybe(pl, p->int0, k * 4);
    B.r_i1 = maybe(pl, p->int1, k * 4);
    B.r_i2 = maybe(pl, p->int2, k * 4);
    B.r_vmat64 = maybe(pl, p->vmat64, k * n * 8);
    B.r_vmat32 = p->vmat64 ? NONE : maybe(pl, p->vmat, k * n * 4);
    B.r_wtab64 = maybe(pl, p->wtab64, k * (n + 1) * 8);
    B.r_wtab32 = p->wtab64 ? NONE : maybe(pl, p->wtab, k * (n + 1) * 4);
    B.r_p164 = maybe(pl, p->p1_64, k * 8);
    B.r_p132 = p->p1_64 ? NONE : maybe(pl, p->p1, k * 4);
    B.r_p264 = maybe(pl, p->p2_64, k * 8);
    B.r_p232 = p->p2_64 ? NONE : maybe(pl, p->p2, k * 4);
    B.r_vb64 = maybe(pl, p->vb64, n * 8);
    B.r_vb32 = p->vb64 ? NONE : maybe(pl, p->vb, n * 4);
    B.r_vmiss = maybe(pl, p->vmiss, k * n);
    B.r_od0 = maybe(pl, p->od0, n * 4);
    B.r_id0 = maybe(pl, p->id0, n * 4);
    B.r_act = maybe(pl, p->act, n * 4);
    B.r_inact = (p->has_comp && p->inactw) ? pl.take(W * 4) : NONE;
    B.r_z0 = maybe(pl, p->z0, n * 4);
    B.r_bkd = maybe(pl, p->bkdist, n * 4);
    B.r_bty = kb ? pl.take(kb * 4) : NONE;
    B.r_rk = nr ? pl.take(nr * 4) : NONE;
    B.r_ra = nr ? pl.take(nr * 4) : NONE;
    B.r_ru = nr ? pl.take(nr * n * 4) : NONE;
    B.o_stats = maybe(pl, r->stats, M * k * 8);
    B.o_ntim = maybe(pl, r->ntim, M * 8);
    B.o_scores = maybe(pl, r->scores, M * (k + 1) * 4);
    B.o_dist = maybe(pl, r->dist, M * 4);
    B.o_dstat = maybe(pl, r->dist_stat, M * 4);
    B.o_steps = maybe(pl, r->steps, M * 4);
    B.o_bdist = kb ? maybe(pl, r->bdist, M * 4) : NONE;
    B.o_bscores = kb ? maybe(pl, r->bscores, M * (kb + 1) * 4) : NONE;
    B.o_zend = kb ? maybe(pl, r->z_end, M * n * 4) : NONE;
    B.o_rscores = nr ? maybe(pl, r->rscores, M * nr * 4) : NONE;
    B.o_adist = nr ? maybe(pl, r->actor_dist, M * n * 4) : NONE;
    B.o_aends = (r->want_end_nets && r->a_ends) ? pl.take(M * n * n) : NONE;
  }
}

// Host -> device copy of one raw array into its arena slot; returns its device
// pointer (or the caller's device pointer in device mode).
template <class T>
const T *stage(const T *src, size_t off, size_t bytes, bool dev, cudaStream_t st, cusna_status &s) {
  if (!src) return nullptr;
  if (dev) return src;
  if (off == NONE) return nullptr;
  cudaError_t e = cudaMemcpyAsync(at<char>(off), src, bytes, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) {
    set_err("H2D copy failed: %s", cudaGetErrorString(e));
    s = CUSNA_ERR_CUDA;
  }
  return at<T>(off);
}

cusna_status prepare(Job &J, bool dev, DevProblem &D, uint32_t chain_offset) {
  const cusna_saom_problem *p = J.p;
  cusna_saom_result *r = J.r;
  const ProbBufs &B = J.B;
  cudaStream_t st = g_ctx.stream;
  const int n = p->n, W = p->W, k = p->k, M = p->M, kb = p->kb, nr = p->nrate;
  cusna_status s = CUSNA_OK;
  const size_t bitsz = (size_t)n * W * 4;

  const uint32_t *x0 = stage(p->x0_out, B.r_x0, bitsz, dev, st, s);
  const uint32_t *sim = stage(p->sim_out, B.r_sim, bitsz, dev, st, s);
  const uint32_t *kd = stage(p->kdist, B.r_kd, bitsz, dev, st, s);
  const uint32_t *pm = stage(p->perm, B.r_pm, bitsz, dev, st, s);
  const uint32_t *kp = stage(p->keep_out, B.r_keep, bitsz, dev, st, s);
  const uint32_t *fo = stage(p->force_out, B.r_force, bitsz, dev, st, s);
  const float *theta = stage(p->theta, B.r_theta, (size_t)M * k * 4, dev, st, s);
  const float *lam = stage(p->lam, B.r_lam, (size_t)M * 4, dev, st, s);
  const float *lamb = stage(p->lamb, B.r_lamb, (size_t)M * 4, dev, st, s);
  const float *thetab = kb ? stage(p->thetab, B.r_thetab, (size_t)M * kb * 4, dev, st, s) : nullptr;
  const int *tid = stage(p->type_ids, B.r_tid, (size_t)k * 4, dev, st, s);
  const int *ety = stage(p->etypes, B.r_ety, (size_t)k * 4, dev, st, s);
  const int *dyn = stage(p->dyn_flags, B.r_dyn, (size_t)k * 4, dev, st, s);
  const int *ri0 = stage(p->int0, B.r_i0, (size_t)k * 4, dev, st, s);
  const int *ri1 = stage(p->int1, B.r_i1, (size_t)k * 4, dev, st, s);
  const int *ri2 = stage(p->int2, B.r_i2, (size_t)k * 4, dev, st, s);
  const double *vm64 = stage(p->vmat64, B.r_vmat64, (size_t)k * n * 8, dev, st, s);
  const float *vm32 = p->vmat64 ? nullptr : stage(p->vmat, B.r_vmat32, (size_t)k * n * 4, dev, st, s);
  const double *wt64 = stage(p->wtab64, B.r_wtab64, (size_t)k * (n + 1) * 8, dev, st, s);
  const float *wt32 = p->wtab64 ? nullptr : stage(p->wtab, B.r_wtab32, (size_t)k * (n + 1) * 4, dev, st, s);
  const double *p164 = stage(p->p1_64, B.r_p164, (size_t)k * 8, dev, st, s);
  const float *p132 = p->p1_64 ? nullptr : stage(p->p1, B.r_p132, (size_t)k * 4, dev, st, s);
  const double *p264 = stage(p->p2_64, B.r_p264, (size_t)k * 8, dev, st, s);
  const float *p232 = p->p2_64 ? nullptr : stage(p->p2, B.r_p232, (size_t)k * 4, dev, st, s);
  const double *vb64 = stage(p->vb64, B.r_vb64, (size_t)n * 8, dev, st, s);
  const float *vb32 = p->vb64 ? nullptr : stage(p->vb, B.r_vb32, (size_t)n * 4, dev, st, s);
  const uint8_t *vmiss = stage(p->vmiss, B.r_vmiss, (size_t)k * n, dev, st, s);
  const int *od0 = stage(p->od0, B.r_od0, (size_t)n * 4, dev, st, s);
  const int *id0 = stage(p->id0, B.r_id0, (size_t)n * 4, dev, st, s);
  const int *act = stage(p->act, B.r_act, (size_t)n * 4, dev, st, s);
  const uint32_t *inact = (p->has_comp && p->inactw) ? stage(p->inactw, B.r_inact, (size_t)W * 4, dev, st, s) : nullptr;
  const int *z0 = stage(p->z0, B.r_z0, (size_t)n * 4, dev, st, s);
  const int *bkd = stage(p->bkdist, B.r_bkd, (size_t)n * 4, dev, st, s);
  const int *bty = kb ? stage(p->bty, B.r_bty, (size_t)kb * 4, dev, st, s) : nullptr;
  const int *rk = nr ? stage(p->rkind, B.r_rk, (size_t)nr * 4, dev, st, s) : nullptr;
  const float *ra = nr ? stage(p->ralpha, B.r_ra, (size_t)nr * 4, dev, st, s) : nullptr;
  const float *ru = nr ? stage(p->ru, B.r_ru, (size_t)nr * n * 4, dev, st, s) : nullptr;
  if (s != CUSNA_OK) return s;

  // canonical word-major networks
  CU(launch_prep_bits(x0, n, W, at<uint32_t>(B.x0T), at<uint32_t>(B.x0cT), 0, st));
  CU(launch_prep_bits(sim ? sim : x0, n, W, at<uint32_t>(B.simT), at<uint32_t>(B.simcT), 0, st));
  CU(launch_prep_bits(kd, n, W, at<uint32_t>(B.kdistT), nullptr, 1, st));
  CU(launch_prep_bits(pm, n, W, at<uint32_t>(B.permT), nullptr, 1, st));
  CU(launch_prep_bits(kp, n, W, at<uint32_t>(B.keepT), at<uint32_t>(B.keepcT), 1, st));
  CU(launch_prep_bits(fo, n, W, at<uint32_t>(B.forceT), at<uint32_t>(B.forcecT), 2, st));
  // float64 descriptors
  CU(launch_prep_desc(vm64, vm32, (size_t)k * n, at<double>(B.vmat), st));
  CU(launch_prep_desc(wt64, wt32, (size_t)k * (n + 1), at<double>(B.wtab), st));
  CU(launch_prep_desc(p164, p132, (size_t)k, at<double>(B.p1), st));
  CU(launch_prep_desc(p264, p232, (size_t)k, at<double>(B.p2), st));
  CU(launch_prep_desc(vb64, vb32, (size_t)n, at<double>(B.vb), st));
  if (nr) {
    CU(launch_prep_desc(nullptr, ra, (size_t)nr, at<double>(B.ralpha), st));
    CU(launch_prep_desc(nullptr, ru, (size_t)nr * n, at<double>(B.ru), st));
  }
  // integer descriptors with the CPU engine's defaults
  auto icopy = [&](const int *src, size_t off, size_t cnt, int mode, int def) -> cusna_status {
    if (src) CU(cudaMemcpyAsync(at<int>(off), src, cnt * 4, cudaMemcpyDeviceToDevice, st));
    else CU(launch_fill_int(at<int>(off), cnt, mode, def, st));
    return CUSNA_OK;
  };
  if ((s = icopy(ety, B.etypes, k, 0, 0)) != CUSNA_OK) return s;
  if ((s = icopy(dyn, B.dyn, k, 0, 0)) != CUSNA_OK) return s;
  if ((s = icopy(ri0, B.i0, k, 0, -1)) != CUSNA_OK) return s;
  if ((s = icopy(ri1, B.i1, k, 0, -1)) != CUSNA_OK) return s;
  if ((s = icopy(ri2, B.i2, k, 0, -1)) != CUSNA_OK) return s;
  if ((s = icopy(z0, B.z0, n, 0, 0)) != CUSNA_OK) return s;
  if ((s = icopy(bkd, B.bkdist, n, 0, 1)) != CUSNA_OK) return s;
  if (act) {
    CU(cudaMemcpyAsync(at<int>(B.act), act, (size_t)p->nact * 4, cudaMemcpyDeviceToDevice, st));
  } else {
    CU(launch_fill_int(at<int>(B.act), n, 1, 0, st));
  }
  if (inact) CU(cudaMemcpyAsync(at<uint32_t>(B.inact), inact, (size_t)W * 4, cudaMemcpyDeviceToDevice, st));
  else CU(cudaMemsetAsync(at<uint32_t>(B.inact), 0, (size_t)W * 4, st));

  std::memset(&D, 0, sizeof D);
  D.n = n; D.W = W; D.k = k; D.kb = kb; D.nrate = nr; D.M = M;
  D.chain_offset = chain_offset;
  D.cond = p->conditional; D.target_dist = p->target_dist; D.symflag = p->symflag;
  D.maxdeg = p->maxdegree; D.has_comp = p->has_comp && p->inactw; D.nact = p->act ? p->nact : n;
  D.k0 = (uint32_t)(p->seed & 0xFFFFFFFFu);
  D.k1 = (uint32_t)(p->seed >> 32);
  D.flags = J.F.flags | ((r->want_end_nets && r->a_ends) ? F_WANT_ENDS : 0);
  D.zmin = p->zmin; D.zmax = p->zmax; D.zlo = J.F.zlo; D.zR = J.F.zR;
  D.zbar = (double)p->zbar; D.brange = (double)p->brange; D.bsimmean = (double)p->bsimmean;
  D.type_ids = tid; D.etypes = at<int>(B.etypes); D.dyn = at<int>(B.dyn);
  D.int0 = at<int>(B.i0); D.int1 = at<int>(B.i1); D.int2 = at<int>(B.i2);
  D.p1 = at<double>(B.p1); D.p2 = at<double>(B.p2); D.vmat = at<double>(B.vmat);
  D.wtab = at<double>(B.wtab); D.vmiss = vmiss; D.vb = at<double>(B.vb);
  D.od0 = od0; D.id0 = id0; D.bty = bty; D.rkind = rk;
  D.ralpha = at<double>(B.ralpha); D.ru = at<double>(B.ru);
  D.act = at<int>(B.act); D.inact = at<uint32_t>(B.inact);
  D.z0 = at<int>(B.z0); D.bkdist = at<int>(B.bkdist);
  D.x0T = at<uint32_t>(B.x0T); D.x0cT = at<uint32_t>(B.x0cT);
  D.simT = at<uint32_t>(B.simT); D.simcT = at<uint32_t>(B.simcT);
  D.kdistT = at<uint32_t>(B.kdistT); D.permT = at<uint32_t>(B.permT);
  D.keepT = at<uint32_t>(B.keepT); D.forceT = at<uint32_t>(B.forceT);
  D.keepcT = at<uint32_t>(B.keepcT); D.forcecT = at<uint32_t>(B.forcecT);
  D.lam = lam; D.theta = theta; D.lamb = lamb; D.thetab = thetab;
  D.prow = 1;
  CU(cudaMemcpyAsync(at<int>(B.ekind), J.F.kind.data(), (size_t)k * 4, cudaMemcpyHostToDevice, st));
  CU(cudaMemcpyAsync(at<int>(B.ecfn), J.F.cfn.data(), (size_t)k * 4, cudaMemcpyHostToDevice, st));
  CU(cudaMemcpyAsync(at<int>(B.eoffd), J.F.offd.data(), (size_t)k * 4, cudaMemcpyHostToDevice, st));
  CU(cudaMemcpyAsync(at<int>(B.eofft), J.F.offt.data(), (size_t)k * 4, cudaMemcpyHostToDevice, st));
  CU(cudaMemcpyAsync(at<double>(B.pool), J.F.pool.data(), J.F.pool.size() * 8, cudaMemcpyHostToDevice, st));
  {
    // lookup values as double-float pairs: the float32 rounding (the float32
    // pass) and the float32 rounding of the remainder (the score sums); a
    // pageable copy is staged before cudaMemcpyAsync returns, so the local
    // vector may go
    std::vector<float> p2(2 * J.F.pool.size());
    for (size_t x = 0; x < J.F.pool.size(); ++x) {
      p2[2 * x] = (float)J.F.pool[x];
      p2[2 * x + 1] = (float)(J.F.pool[x] - (double)p2[2 * x]);
    }
    CU(cudaMemcpyAsync(at<float>(B.pool2), p2.data(), p2.size() * 4, cudaMemcpyHostToDevice, st));
  }
  D.ekind = at<int>(B.ekind); D.ecfn = at<int>(B.ecfn); D.eoffd = at<int>(B.eoffd);
  D.eofft = at<int>(B.eofft); D.tab = at<double>(B.pool); D.tab2 = at<float2>(B.pool2);
  auto out = [&](void *user, size_t off) -> void * {
    if (!user) return nullptr;
    return dev ? user : (off == NONE ? nullptr : at<char>(off));
  };
  D.stats = (double *)out(r->stats, B.o_stats);
  D.ntim = (double *)out(r->ntim, B.o_ntim);
  D.scores = (float *)out(r->scores, B.o_scores);
  D.dist = (int *)out(r->dist, B.o_dist);
  D.dist_stat = (int *)out(r->dist_stat, B.o_dstat);
  D.steps = (int *)out(r->steps, B.o_steps);
  if (kb) {
    D.bdist = (int *)out(r->bdist, B.o_bdist);
    D.bscores = (float *)out(r->bscores, B.o_bscores);
    D.z_end = (int *)out(r->z_end, B.o_zend);
  }
  if (nr) {
    D.rscores = (float *)out(r->rscores, B.o_rscores);
    D.actor_dist = (int *)out(r->actor_dist, B.o_adist);
  }
  D.a_ends = (r->want_end_nets && r->a_ends) ? (uint8_t *)out(r->a_ends, B.o_aends) : nullptr;
  return CUSNA_OK;
}

cusna_status fetch_outputs(Job &J) {
  const cusna_saom_problem *p = J.p;
  cusna_saom_result *r = J.r;
  const ProbBufs &B = J.B;
  cudaStream_t st = g_ctx.stream;
  const size_t n = p->n, k = p->k, M = p->M, kb = p->kb, nr = p->nrate;
  auto get = [&](void *dst, size_t off, size_t bytes) -> cusna_status {
    if (!dst || off == NONE) return CUSNA_OK;
    CU(cudaMemcpyAsync(dst, at<char>(off), bytes, cudaMemcpyDeviceToHost, st));
    return CUSNA_OK;
  };
  cusna_status s;
  if ((s = get(r->stats, B.o_stats, M * k * 8)) != CUSNA_OK) return s;
  if ((s = get(r->ntim, B.o_ntim, M * 8)) != CUSNA_OK) return s;
  if ((s = get(r->scores, B.o_scores, M * (k + 1) * 4)) != CUSNA_OK) return s;
  if ((s = get(r->dist, B.o_dist, M * 4)) != CUSNA_OK) return s;
  if ((s = get(r->dist_stat, B.o_dstat, M * 4)) != CUSNA_OK) return s;
  if ((s = get(r->steps, B.o_steps, M * 4)) != CUSNA_OK) return s;
  if (kb) {
    if ((s = get(r->bdist, B.o_bdist, M * 4)) != CUSNA_OK) return s;
    if ((s = get(r->bscores, B.o_bscores, M * (kb + 1) * 4)) != CUSNA_OK) return s;
    if ((s = get(r->z_end, B.o_zend, M * n * 4)) != CUSNA_OK) return s;
  }
  if (nr) {
    if ((s = get(r->rscores, B.o_rscores, M * nr * 4)) != CUSNA_OK) return s;
    if ((s = get(r->actor_dist, B.o_adist, M * n * 4)) != CUSNA_OK) return s;
  }
  if (r->want_end_nets && r->a_ends)
    if ((s = get(r->a_ends, B.o_aends, M * n * n)) != CUSNA_OK) return s;
  return CUSNA_OK;
}

// ---- launch-shape autotuner ---------------------------------------------------
// The simulator is bound by the float64 pipe, whose instructions have long
// latencies, so the shape that wins keeps the most warps resident per SM while
// every resident team has a chain to run. For each team size G (warps per
// chain), chain state in shared memory or in-rows in global scratch, and teams
// per CTA, the CUDA occupancy calculator gives the resident CTAs per SM (shared
// memory, registers and warps all count). The score is the number of warps that
// will be busy: min(resident teams, chains) * G per SM, capped at 48; ties go to
// smaller teams (fewer barriers) and to in-rows in shared memory.
std::vector<LaunchShape> rank_shapes(int nmax, int Wmax, int kmax, int kbmax, int nrmax, bool tp,
                                     bool gw, bool tq, long long total_units, int force_G,
                                     int force_tpc, int nets = 1,
                                     const JitKernel *jk = nullptr, bool valid = false) {
  const Ctx &c = g_ctx;
  std::vector<std::pair<double, LaunchShape>> all;
  const int Gs[5] = {1, 2, 4, 8, 16};
  for (int gi = 0; gi < 5; ++gi) {
    const int G = Gs[gi];
    if (force_G && G != force_G) continue;
    // placements: everything in shared memory; the in-rows in global scratch
    // (L1-cached; a candidate even when shared memory suffices, as it frees
    // shared memory for more chains per SM); the out-rows too, only when
    // neither of the first two fits
    bool placed = false;
    for (int place = 0; place < 3; ++place) {
      if (place == 2 && placed) break;
      const bool rows_smem = place < 2, cols_smem = place == 0;
      LaunchShape sh{};
      sh.G = G;
      sh.cols_in_smem = cols_smem;
      sh.rows_in_smem = rows_smem;
      sh.lay = make_layout(nmax, Wmax, kmax, kbmax, nrmax, G, rows_smem, cols_smem, tp, gw, tq);
      if (sh.lay.bytes * nets > (size_t)c.smem_optin) continue;
      bool any = false;
      for (int tpc = 1; tpc <= 16; tpc *= 2) {
        if (force_tpc && tpc != force_tpc) continue;
        const int threads = 32 * G * tpc;
        if (threads > (valid ? 256 : 512) || (G > 1 && tpc > 15)) continue;
        const size_t dyn = sh.lay.bytes * nets * tpc;
        if (dyn > (size_t)c.smem_optin) continue;
        const int per_sm = jk ? jit_blocks_per_sm(*jk, threads, dyn)
                              : (nets > 1 ? multi_blocks_per_sm(threads, dyn)
                                          : period_blocks_per_sm(threads, dyn, valid));
        if (per_sm < 1) continue;
        const double teams_sm = (double)per_sm * tpc;
        const double chains_sm = (double)total_units / c.sms;
        const double busy_warps = std::min(teams_sm, std::max(chains_sm, 1.0)) * G;
        // ties: smaller teams (fewer barriers), state on chip, then larger CTAs
        const double score = std::min(busy_warps, 48.0) * 100.0 - G - (cols_smem ? 0.0 : 50.0) -
                             (rows_smem ? 0.0 : 50.0) + tpc * 0.01;
        LaunchShape x = sh;
        x.teams_per_cta = tpc;
        const long long want = (total_units + tpc - 1) / tpc;
        x.ctas = (int)std::max<long long>(1, std::min<long long>((long long)c.sms * per_sm, want));
        all.push_back({score, x});
        any = true;
      }
      placed |= any;
    }
  }
  std::stable_sort(all.begin(), all.end(),
                   [](const std::pair<double, LaunchShape> &a, const std::pair<double, LaunchShape> &b) {
                     return a.first > b.first;
                   });
  std::vector<LaunchShape> out;
  for (auto &x : all) out.push_back(x.second);
  return out;
}

// ---- empirical autotuner ---------------------------------------------------------
// The occupancy model ranks shapes, but the best team size depends on how the
// per-ministep team work (reductions, barriers) trades against the per-alter
// work, which it does not model. Results do not depend on the shape (every
// output is bit-identical for every shape), so the tuner explores on real
// calls: successive calls with the same signature each try one of the model's
// two best shapes of each team size (G = 1, 2, 4, 8, 16, in the model's
// order), timed with events, and later calls use the fastest.
// CUSNA_AUTOTUNE=0 keeps the model's choice.
struct TuneKey {
  int dev, nmax, Wmax, kmax, kbmax, nrmax, flags, pad;
  long long units;
};
struct TuneEntry {
  TuneKey key;
  std::vector<LaunchShape> cand;
  std::vector<float> ms;
  size_t next = 0;
  int best = -1;
};
std::mutex g_tune_mu;
std::vector<TuneEntry> g_tune;

bool tuning_enabled() {
  static const bool on = [] {
    const char *e = std::getenv("CUSNA_AUTOTUNE");
    return !(e && e[0] == '0');
  }();
  return on;
}

TuneKey tune_key(int nmax, int Wmax, int kmax, int kbmax, int nrmax, bool tp, bool gw, bool tq,
                 long long units, bool jit = false) {
  TuneKey k;
  std::memset(&k, 0, sizeof k);
  k.dev = g_ctx.device; k.nmax = nmax; k.Wmax = Wmax; k.kmax = kmax; k.kbmax = kbmax;
  k.nrmax = nrmax; k.flags = (tp ? 1 : 0) | (gw ? 2 : 0) | (tq ? 4 : 0) | (jit ? 8 : 0);
  k.units = units;
  return k;
}

// The specialised kernel of a launch: every problem must have the same effect
// plan. spec_mode: 0 as CUSNA_JIT says, -1 never, 1 compile now if needed.
// The specialisation a launch of these problems can use: with the actor count
// compiled in when every problem has the same, else with it read at run time;
// "" when the effect plans differ.
std::string launch_spec(const std::vector<Job> &jobs) {
  if (jobs.empty() || jobs[0].F.spec.empty()) return "";
  // CUSNA_JIT_FIXED_N=0: never compile the actor count in
  static const bool fixed_n = [] {
    const char *e = std::getenv("CUSNA_JIT_FIXED_N");
    return !(e && e[0] == '0');
  }();
  bool same_w = fixed_n, same = true;
  for (const Job &J : jobs) {
    same_w = same_w && J.F.spec_w == jobs[0].F.spec_w;
    same = same && J.F.spec == jobs[0].F.spec;
  }
  return same_w ? jobs[0].F.spec_w : (same ? jobs[0].F.spec : "");
}

bool jit_for(const std::vector<Job> &jobs, int spec_mode, JitKernel *jk) {
  if (spec_mode < 0) return false;
  const std::string spec = launch_spec(jobs);
  if (spec.empty()) return false;
  // spec_mode 1: compile and load now (tests, and callers that know the
  // effect plan will run long enough)
  return jit_get(spec, jk, spec_mode > 0);
}

// the model's two best shapes of each team size, in the model's order
// Two candidates per team size G, in the model's order: its best shape for
// that G and the best with the other placement of the in-rows (shared memory
// or global scratch), or without one its second best.
std::vector<LaunchShape> tuning_candidates(const std::vector<LaunchShape> &ranked) {
  std::vector<LaunchShape> c;
  for (size_t i = 0; i < ranked.size(); ++i) {
    const LaunchShape &first = ranked[i];
    bool seen = false;
    for (const LaunchShape &x : c) seen |= x.G == first.G;
    if (seen) continue;
    c.push_back(first);
    const LaunchShape *second = nullptr;
    for (size_t j = i + 1; j < ranked.size() && !second; ++j)
      if (ranked[j].G == first.G && ranked[j].cols_in_smem != first.cols_in_smem)
        second = &ranked[j];
    for (size_t j = i + 1; j < ranked.size() && !second; ++j)
      if (ranked[j].G == first.G) second = &ranked[j];
    if (second) c.push_back(*second);
  }
  return c;
}

TuneEntry &tune_entry(const TuneKey &key, const std::vector<LaunchShape> &cand) {
  for (auto &e : g_tune)
    if (std::memcmp(&e.key, &key, sizeof key) == 0) return e;
  TuneEntry e;
  e.key = key;
  e.cand = cand;
  e.ms.assign(cand.size(), INFINITY);
  if (!tuning_enabled() || cand.size() < 2) { e.next = cand.size(); e.best = 0; }
  g_tune.push_back(e);
  return g_tune.back();
}

// The shape for this call; *trial is the candidate being timed, or -1.
LaunchShape tuner_pick(const TuneKey &key, const std::vector<LaunchShape> &cand, int *trial) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  TuneEntry &e = tune_entry(key, cand);
  if (e.next < e.cand.size()) {
    *trial = (int)e.next++;
    return e.cand[*trial];
  }
  *trial = -1;
  return e.cand[e.best >= 0 ? e.best : 0];
}

void tuner_record(const TuneKey &key, int trial, float ms) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  for (auto &e : g_tune)
    if (std::memcmp(&e.key, &key, sizeof key) == 0) {
      if (trial >= 0 && (size_t)trial < e.ms.size()) e.ms[trial] = ms;
      int b = 0;
      for (size_t x = 1; x < e.ms.size(); ++x)
        if (e.ms[x] < e.ms[b]) b = (int)x;
      e.best = b;
      return;
    }
}

// Register limit check of a shape: the kernel is compiled for 512 threads with
// the full register file, so any CTA size up to 512 fits.
cusna_status run_jobs(std::vector<Job> &jobs, bool dev, cusna_gpu_options *opts,
                      const cusna_validation_options *vo = nullptr) {
  cusna_status s;
  if ((s = ensure_ctx()) != CUSNA_OK) return s;
  if (opts && opts->stream) {
    // run on the caller's stream: adopt it for this call
  }
  cudaStream_t st = (opts && opts->stream) ? (cudaStream_t)opts->stream : g_ctx.stream;
  cudaStream_t own = g_ctx.stream;
  g_ctx.stream = st;
  struct Restore { cudaStream_t &ref; cudaStream_t v; ~Restore() { ref = v; } } restore{g_ctx.stream, own};

  const uint32_t off0 = opts ? opts->chain_offset : 0;
  const long long launches0 = kernel_launches();
  int nmax = 0, Wmax = 0, kmax = 0, kbmax = 0, nrmax = 0;
  bool tp = false, gw = false, tq = false;
  long long total = 0;
  for (auto &J : jobs) {
    nmax = std::max(nmax, J.p->n); Wmax = std::max(Wmax, J.p->W); kmax = std::max(kmax, J.p->k);
    kbmax = std::max(kbmax, J.p->kb); nrmax = std::max(nrmax, J.p->nrate);
    tp |= (J.F.flags & F_NEED_TP) != 0;
    gw |= (J.F.flags & (F_NEED_GW29 | F_NEED_TP)) != 0;
    tq |= (J.F.flags & F_NEED_GW30) != 0;
    total += J.p->M;
  }
  const bool valid = vo != nullptr;
  const int fG = valid ? vo->warps_per_chain : (opts ? opts->warps_per_chain : 0);
  const int fT = valid ? vo->chains_per_cta : (opts ? opts->chains_per_cta : 0);
  JitKernel jk;
  // the validation build is the library kernel's
  const bool use_jit = !valid && jit_for(jobs, opts ? opts->specialise : 0, &jk);
  std::vector<LaunchShape> ranked =
      rank_shapes(nmax, Wmax, kmax, kbmax, nrmax, tp, gw, tq, total, fG, fT, 1,
                  use_jit ? &jk : nullptr, valid);
  if (ranked.empty()) {
    set_err("no launch shape fits n=%d in shared memory", nmax);
    return CUSNA_ERR_UNSUPPORTED;
  }
  // a forced shape is used as given; otherwise the autotuner picks (and may be
  // timing one of its candidates in this call)
  int trial = -1;
  const TuneKey tkey = tune_key(nmax, Wmax, kmax, kbmax, nrmax, tp, gw, tq, total, use_jit);
  const LaunchShape sh = (fG || fT || valid) ? ranked[0]
                                             : tuner_pick(tkey, tuning_candidates(ranked), &trial);
  Planner pl;
  for (auto &J : jobs) plan_problem(pl, J, dev);
  // validation: the trace records and the supplied words of the (one) problem
  const size_t trace_words = valid ? (size_t)jobs[0].p->M * vo->trace_cap * 4 : 0;
  const size_t us_words =
      valid ? (size_t)jobs[0].p->M * vo->ustream_steps * (4 + (size_t)jobs[0].p->n) : 0;
  const size_t o_trace = trace_words ? pl.take(trace_words * 4) : NONE;
  const size_t o_us = us_words ? pl.take(us_words * 4) : NONE;
  const size_t o_probs = pl.take(sizeof(DevProblem) * jobs.size());
  const size_t o_units = pl.take(sizeof(long long) * (jobs.size() + 1));
  const size_t o_counter = pl.take(sizeof(unsigned long long));
  const size_t teams = (size_t)sh.ctas * sh.teams_per_cta;
  const size_t cols_words = (size_t)Wmax * nmax;
  const size_t o_cols = sh.cols_in_smem ? NONE : pl.take(teams * cols_words * 4);
  const size_t o_rows = sh.rows_in_smem ? NONE : pl.take(teams * cols_words * 4);
  if ((s = ensure_arena(pl.off)) != CUSNA_OK) return s;

  std::vector<DevProblem> hp(jobs.size());
  std::vector<long long> units(jobs.size() + 1, 0);
  for (size_t q = 0; q < jobs.size(); ++q) {
    if ((s = prepare(jobs[q], dev, hp[q], off0)) != CUSNA_OK) return s;
    // no scores requested: the kernel forms no score sums
    if (!hp[q].scores) hp[q].flags |= F_NO_SCORES;
    units[q + 1] = units[q] + jobs[q].p->M;
  }
  if (valid) {
    DevProblem &D = hp[0];
    if (vo->lse64) D.flags |= F_LSE64;
    if (o_trace != NONE) {
      // records of ministeps a chain does not reach stay -1
      CU(cudaMemsetAsync(at<char>(o_trace), 0xFF, trace_words * 4, st));
      D.trace = at<int>(o_trace);
      D.trace_cap = vo->trace_cap;
    }
    if (o_us != NONE) {
      CU(cudaMemcpyAsync(at<char>(o_us), vo->ustream, us_words * 4, cudaMemcpyHostToDevice, st));
      D.ustream = at<uint32_t>(o_us);
      D.ustream_steps = vo->ustream_steps;
    }
  }
  CU(cudaMemcpyAsync(at<char>(o_probs), hp.data(), sizeof(DevProblem) * hp.size(),
                     cudaMemcpyHostToDevice, st));
  CU(cudaMemcpyAsync(at<char>(o_units), units.data(), sizeof(long long) * units.size(),
                     cudaMemcpyHostToDevice, st));
  CU(cudaMemsetAsync(at<char>(o_counter), 0, sizeof(unsigned long long), st));
  CU(cudaEventRecord(g_ctx.ev0, st));
  if (use_jit)
    CU(launch_period_jit(jk, sh, at<DevProblem>(o_probs), at<long long>(o_units), (int)jobs.size(),
                         total, at<unsigned long long>(o_counter),
                         o_cols == NONE ? nullptr : at<uint32_t>(o_cols),
                         o_rows == NONE ? nullptr : at<uint32_t>(o_rows), cols_words, st));
  else
    CU(launch_period(sh, at<DevProblem>(o_probs), at<long long>(o_units), (int)jobs.size(), total,
                     at<unsigned long long>(o_counter),
                     o_cols == NONE ? nullptr : at<uint32_t>(o_cols),
                     o_rows == NONE ? nullptr : at<uint32_t>(o_rows), cols_words, st, valid));
  CU(cudaEventRecord(g_ctx.ev1, st));
  if (!dev)
    for (auto &J : jobs)
      if ((s = fetch_outputs(J)) != CUSNA_OK) return s;
  if (o_trace != NONE)
    CU(cudaMemcpyAsync(vo->trace, at<char>(o_trace), trace_words * 4, cudaMemcpyDeviceToHost, st));
  CU(cudaStreamSynchronize(st));
  float ms = 0.f;
  CU(cudaEventElapsedTime(&ms, g_ctx.ev0, g_ctx.ev1));
  if (trial >= 0) tuner_record(tkey, trial, ms);
  if (opts) {
    opts->elapsed_ms = ms;
    opts->warps_per_chain = sh.G;
    opts->chains_per_cta = sh.teams_per_cta;
    opts->launches = (int32_t)(kernel_launches() - launches0);
    opts->specialised = use_jit ? 1 : 0;
  }
  return CUSNA_OK;
}

void order_longest_first(std::vector<Job> &jobs);

cusna_status simulate(const cusna_saom_problem *problems, cusna_saom_result *results, int count,
                      cusna_gpu_options *opts) {
  if (!problems || !results) { set_err("problem or result is NULL"); return CUSNA_ERR_NULL_ARG; }
  if (count < 1) { set_err("count %d < 1", count); return CUSNA_ERR_SHAPE; }
  if (opts && opts->struct_version != CUSNA_ABI_VERSION) {
    set_err("options struct_version %d", opts->struct_version);
    return CUSNA_ERR_SHAPE;
  }
  const bool dev = opts && opts->device_ptrs;
  cusna_status s;
  // host-mode arguments are checked before touching the device, so shape and
  // NULL errors are reported exactly as the CPU engine reports them
  if (dev && (s = ensure_ctx()) != CUSNA_OK) return s;
  std::vector<Job> jobs(count);
  for (int q = 0; q < count; ++q) {
    jobs[q].p = &problems[q];
    jobs[q].r = &results[q];
    if ((s = validate(&problems[q], &results[q], dev, jobs[q].F)) != CUSNA_OK) return s;
  }
  if ((s = ensure_ctx()) != CUSNA_OK) return s;
  order_longest_first(jobs);
  s = run_jobs(jobs, dev, opts);
  if (s == CUSNA_OK && opts) {
    long long tot = 0;
    // ministep totals are only known in host mode (steps copied back)
    for (auto &J : jobs)
      if (!dev && J.r->steps)
        for (int c = 0; c < J.p->M; ++c) tot += J.r->steps[c];
    opts->ministeps = tot;
  }
  return s;
}

// Relative cost of one chain of a problem, for ordering the persistent
// kernel's work longest first: ministeps grow with n and each ministep visits
// n alters with k effects.
double chain_cost(const cusna_saom_problem *p) {
  return (double)p->n * (double)p->n * (double)(p->k + 4);
}

void order_longest_first(std::vector<Job> &jobs) {
  std::stable_sort(jobs.begin(), jobs.end(),
                   [](const Job &a, const Job &b) { return chain_cost(a.p) > chain_cost(b.p); });
}

// ---- multi-network periods (src/libcusna_saom_cpu.cpp:427-604) ----------------
// Each network's effects become a single-network problem of their own (its
// start network, permitted dyads, effect plan and tables), checked and
// prepared by the single-network code; the multi kernel gives a team one
// slice per network and picks the network of each ministep.
struct MultiNet {
  cusna_saom_problem q;
  cusna_saom_result r;
  std::vector<int> eidx;  // the network's effects, in the caller's order
  std::vector<int> tid, ety;
  std::vector<float> th, lam, p1, p2, vm, wt;
};

// check_only: validate and compile the specialised kernel (no device), with
// the compiler log in *log and the compile time in *seconds.
cusna_status simulate_multi(const cusna_saom_multi_problem *pb, cusna_saom_multi_result *r,
                            bool check_only = false, std::string *log = nullptr,
                            double *seconds = nullptr) {
  if (!pb || !r) { set_err("problem or result is NULL"); return CUSNA_ERR_NULL_ARG; }
  if (pb->struct_version != CUSNA_ABI_VERSION || r->struct_version != CUSNA_ABI_VERSION) {
    set_err("struct_version %d/%d != %d", pb->struct_version, r->struct_version, CUSNA_ABI_VERSION);
    return CUSNA_ERR_SHAPE;
  }
  const int n = pb->n, W = pb->W, k = pb->k, M = pb->M, D = pb->D;
  if (n < 1 || n > CUSNA_MAX_N || W != (n + 31) / 32 || k < 1 || k > CUSNA_MAXEFF || M < 1 ||
      D < 2 || D > CUSNA_MAXNET) {
    set_err("bad shape n=%d W=%d k=%d M=%d D=%d", n, W, k, M, D);
    return CUSNA_ERR_SHAPE;
  }
  if (!pb->x0_out || !pb->lam || !pb->theta || !pb->type_ids || !pb->netof) {
    set_err("x0_out, lam, theta, type_ids and netof are required");
    return CUSNA_ERR_NULL_ARG;
  }
  if (pb->act) {
    if (pb->nact < 1 || pb->nact > n) { set_err("nact %d out of range", pb->nact); return CUSNA_ERR_SHAPE; }
    for (int x = 0; x < pb->nact; ++x)
      if (pb->act[x] < 0 || pb->act[x] >= n) { set_err("act entry %d out of range", pb->act[x]); return CUSNA_ERR_SHAPE; }
  }
  std::vector<MultiNet> nets(D);
  std::vector<int> gidx, goff(D + 1, 0);
  bool any_dyc = false;
  for (int e = 0; e < k; ++e) {
    const int d = pb->netof[e], t = pb->type_ids[e];
    if (d < 0 || d >= D) { set_err("netof[%d] = %d out of range", e, d); return CUSNA_ERR_SHAPE; }
    if (t >= 33 && t <= 37) {
      const int w = pb->netref ? pb->netref[e] : 0;
      if (w < 0 || w >= D) { set_err("netref[%d] = %d out of range", e, w); return CUSNA_ERR_SHAPE; }
    }
    const int dci = pb->dyc_idx ? pb->dyc_idx[e] : -1;
    // one dyadic covariate matrix: the reference indexes dyc[(idx*n + i)*n + j]
    // within an n*n copy
    if (dci < -1 || dci > 0) { set_err("dyc_idx[%d] = %d: one dyadic covariate", e, dci); return CUSNA_ERR_SHAPE; }
    if (dci == 0 && !pb->dyc) { set_err("dyc_idx[%d] = 0 without dyc", e); return CUSNA_ERR_NULL_ARG; }
    any_dyc |= dci == 0 && t == 22;
    nets[d].eidx.push_back(e);
  }
  std::vector<double> dyc;
  if (any_dyc) {
    dyc.resize((size_t)n * n);
    for (size_t x = 0; x < dyc.size(); ++x) dyc[x] = (double)pb->dyc[x];
  }
  std::vector<Job> jobs(D);
  int kmax = 0;
  bool tp = false, gw = false, tq = false;
  for (int d = 0; d < D; ++d) {
    MultiNet &N = nets[d];
    goff[d + 1] = goff[d] + (int)N.eidx.size();
    for (int e : N.eidx) gidx.push_back(e);
    // a network without effects chooses uniformly: one zero effect stands in
    const bool empty = N.eidx.empty();
    const int kd = empty ? 1 : (int)N.eidx.size();
    N.tid.assign(kd, 22); N.ety.assign(kd, 0);
    N.p1.assign(kd, 0.f); N.p2.assign(kd, 0.f);
    N.vm.assign((size_t)kd * n, 0.f); N.wt.assign((size_t)kd * (n + 1), 0.f);
    N.th.assign((size_t)M * kd, 0.f); N.lam.resize(M);
    Facts &F = jobs[d].F;
    F.multi = true;
    F.cross_src.assign(kd, 0);
    F.dci.assign(kd, -1);
    for (int q = 0; q < (int)N.eidx.size(); ++q) {
      const int e = N.eidx[q];
      N.tid[q] = pb->type_ids[e];
      N.ety[q] = pb->etypes ? pb->etypes[e] : 0;
      N.p1[q] = pb->p1 ? pb->p1[e] : 0.f;
      N.p2[q] = pb->p2 ? pb->p2[e] : 0.f;
      if (pb->vmat) std::memcpy(&N.vm[(size_t)q * n], pb->vmat + (size_t)e * n, (size_t)n * 4);
      if (pb->wtab)
        std::memcpy(&N.wt[(size_t)q * (n + 1)], pb->wtab + (size_t)e * (n + 1), (size_t)(n + 1) * 4);
      for (int c = 0; c < M; ++c) N.th[(size_t)c * kd + q] = pb->theta[(size_t)c * k + e];
      F.cross_src[q] = pb->netref ? pb->netref[e] : 0;
      F.dci[q] = pb->dyc_idx ? pb->dyc_idx[e] : -1;
    }
    for (int c = 0; c < M; ++c) N.lam[c] = pb->lam[(size_t)c * D + d];
    if (any_dyc) F.dyc = dyc;
    cusna_saom_problem &q = N.q;
    std::memset(&q, 0, sizeof q);
    q.struct_version = CUSNA_ABI_VERSION;
    q.n = n; q.W = W; q.k = kd; q.M = M;
    q.x0_out = pb->x0_out + (size_t)d * n * W;
    q.perm = pb->perm ? pb->perm + (size_t)d * n * W : nullptr;
    q.lam = N.lam.data(); q.theta = N.th.data();
    q.type_ids = N.tid.data(); q.etypes = N.ety.data();
    q.p1 = N.p1.data(); q.p2 = N.p2.data(); q.vmat = N.vm.data(); q.wtab = N.wt.data();
    q.symflag = pb->symf ? pb->symf[d] : 0;
    q.seed = pb->seed;
    q.act = pb->act; q.nact = pb->act ? pb->nact : n;
    std::memset(&N.r, 0, sizeof N.r);
    N.r.struct_version = CUSNA_ABI_VERSION;
    jobs[d].p = &N.q;
    jobs[d].r = &N.r;
    cusna_status s = validate(&N.q, &N.r, false, F);
    if (s != CUSNA_OK) return s;
    kmax = std::max(kmax, kd);
    tp |= (F.flags & F_NEED_TP) != 0;
    gw |= (F.flags & (F_NEED_GW29 | F_NEED_TP)) != 0;
    tq |= (F.flags & F_NEED_GW30) != 0;
  }
  // the multi-network kernel specialised to the networks' effect plans
  std::vector<JitPlan> jplans;
  for (int d = 0; d < D; ++d) {
    jplans.push_back(jobs[d].F.jplan);
    jplans.back().n = n;   // the networks share the actors
  }
  const std::string mspec = jit_multi_spec_source(jplans);
  if (check_only) {
    if (jit_compile_only(mspec, log, seconds) != 0) {
      set_err("specialised multi-network kernel did not compile");
      return CUSNA_ERR_UNSUPPORTED;
    }
    return CUSNA_OK;
  }
  cusna_status s;
  if ((s = ensure_ctx()) != CUSNA_OK) return s;
  cudaStream_t st = g_ctx.stream;
  JitKernel jk;
  const bool use_jit = jit_get(mspec, &jk);
  const std::vector<LaunchShape> ranked =
      rank_shapes(n, W, kmax, 0, 0, tp, gw, tq, M, 0, 0, D, use_jit ? &jk : nullptr);
  if (ranked.empty()) {
    set_err("no launch shape fits %d networks of n=%d", D, n);
    return CUSNA_ERR_UNSUPPORTED;
  }
  // the autotuner as for single networks, under a key of its own (the
  // network count in the flags)
  TuneKey tkey = tune_key(n, W, kmax, 0, 0, tp, gw, tq, M, use_jit);
  tkey.flags |= (D << 8) | (1 << 7);
  int trial = -1;
  const LaunchShape sh = tuner_pick(tkey, tuning_candidates(ranked), &trial);
  Planner pl;
  for (auto &J : jobs) plan_problem(pl, J, false);
  const size_t o_probs = pl.take(sizeof(DevProblem) * D);
  const size_t o_counter = pl.take(sizeof(unsigned long long));
  const size_t o_lam = pl.take((size_t)M * D * 4);
  const size_t o_gidx = pl.take((size_t)k * 4);
  const size_t o_rs = r->rscores ? pl.take((size_t)M * D * 4) : NONE;
  const size_t o_sc = r->scores ? pl.take((size_t)M * k * 4) : NONE;
  const size_t o_nt = r->ntim ? pl.take((size_t)M * 8) : NONE;
  const size_t o_st = r->steps ? pl.take((size_t)M * 4) : NONE;
  const size_t o_ae = r->a_ends ? pl.take((size_t)M * D * n * n) : NONE;
  const size_t teams = (size_t)sh.ctas * sh.teams_per_cta;
  const size_t cols_words = (size_t)W * n;
  const size_t o_cols = sh.cols_in_smem ? NONE : pl.take(teams * D * cols_words * 4);
  const size_t o_rows = sh.rows_in_smem ? NONE : pl.take(teams * D * cols_words * 4);
  if ((s = ensure_arena(pl.off)) != CUSNA_OK) return s;
  std::vector<DevProblem> hp(D);
  for (int d = 0; d < D; ++d)
    if ((s = prepare(jobs[d], false, hp[d], 0)) != CUSNA_OK) return s;
  MultiDev md{};
  md.D = D; md.n = n; md.W = W; md.k = k;
  md.nact = pb->act ? pb->nact : n;
  md.act = hp[0].act;
  md.lam = at<float>(o_lam);
  md.k0 = (uint32_t)(pb->seed & 0xFFFFFFFFu);
  md.k1 = (uint32_t)(pb->seed >> 32);
  for (int d = 0; d <= D; ++d) md.goff[d] = goff[d];
  md.gidx = at<int>(o_gidx);
  md.rscores = o_rs == NONE ? nullptr : at<float>(o_rs);
  md.scores = o_sc == NONE ? nullptr : at<float>(o_sc);
  md.ntim = o_nt == NONE ? nullptr : at<double>(o_nt);
  md.steps = o_st == NONE ? nullptr : at<int>(o_st);
  md.a_ends = o_ae == NONE ? nullptr : at<uint8_t>(o_ae);
  CU(cudaMemcpyAsync(at<char>(o_probs), hp.data(), sizeof(DevProblem) * D, cudaMemcpyHostToDevice, st));
  CU(cudaMemcpyAsync(at<char>(o_lam), pb->lam, (size_t)M * D * 4, cudaMemcpyHostToDevice, st));
  CU(cudaMemcpyAsync(at<char>(o_gidx), gidx.data(), (size_t)k * 4, cudaMemcpyHostToDevice, st));
  CU(cudaMemsetAsync(at<char>(o_counter), 0, sizeof(unsigned long long), st));
  CU(cudaEventRecord(g_ctx.ev0, st));
  if (use_jit)
    CU(launch_multi_jit(jk, sh, at<DevProblem>(o_probs), md, M, at<unsigned long long>(o_counter),
                        o_cols == NONE ? nullptr : at<uint32_t>(o_cols),
                        o_rows == NONE ? nullptr : at<uint32_t>(o_rows), cols_words, st));
  else
    CU(launch_multi(sh, at<DevProblem>(o_probs), md, M, at<unsigned long long>(o_counter),
                    o_cols == NONE ? nullptr : at<uint32_t>(o_cols),
                    o_rows == NONE ? nullptr : at<uint32_t>(o_rows), cols_words, st));
  CU(cudaEventRecord(g_ctx.ev1, st));
  auto get = [&](void *dst, size_t off, size_t bytes) -> cusna_status {
    if (!dst || off == NONE) return CUSNA_OK;
    CU(cudaMemcpyAsync(dst, at<char>(off), bytes, cudaMemcpyDeviceToHost, st));
    return CUSNA_OK;
  };
  if ((s = get(r->rscores, o_rs, (size_t)M * D * 4)) != CUSNA_OK) return s;
  if ((s = get(r->scores, o_sc, (size_t)M * k * 4)) != CUSNA_OK) return s;
  if ((s = get(r->ntim, o_nt, (size_t)M * 8)) != CUSNA_OK) return s;
  if ((s = get(r->steps, o_st, (size_t)M * 4)) != CUSNA_OK) return s;
  if ((s = get(r->a_ends, o_ae, (size_t)M * D * n * n)) != CUSNA_OK) return s;
  CU(cudaStreamSynchronize(st));
  if (trial >= 0) {
    float ms = 0.f;
    CU(cudaEventElapsedTime(&ms, g_ctx.ev0, g_ctx.ev1));
    tuner_record(tkey, trial, ms);
  }
  return CUSNA_OK;
}

}  // namespace

}  // namespace cusna

// ---- replayable plans ----------------------------------------------------------
// A plan holds everything a launch reads in device memory of its own, so a
// launch only enqueues kernels: no allocation, no host copy, no wait. Launches
// can therefore be captured into a CUDA graph and replayed.
struct cusna_saom_plan {
  int device = -1;
  void *mem = nullptr;
  cusna::LaunchShape sh{};
  cusna::DevProblem *probs = nullptr;
  long long *units = nullptr;
  unsigned long long *counter = nullptr, *epoch = nullptr, *seeds = nullptr;
  cusna::PlanTable *tabs = nullptr;
  int count = 0, n_tabs = 0;
  long long total = 0;
  uint32_t *cols = nullptr, *rows = nullptr;
  size_t cols_words = 0;
  cudaGraphExec_t graph = nullptr;
  // autotuning over the first launches (one timed trial per candidate shape)
  std::vector<cusna::LaunchShape> cand;
  std::vector<float> cand_ms;
  size_t trial = 0;
  bool pending = false;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // the specialised kernel of the plan's effect plan, once it is available
  std::string spec;
  bool jit = false;
  cusna::JitKernel jk;
};

namespace cusna {
namespace {

void plan_free(cusna_saom_plan *P) {
  if (!P) return;
  if (P->graph) cudaGraphExecDestroy(P->graph);
  if (P->ev0) cudaEventDestroy(P->ev0);
  if (P->ev1) cudaEventDestroy(P->ev1);
  if (P->mem) cudaFree(P->mem);
  delete P;
}

cusna_status plan_create(const cusna_saom_problem *problems, cusna_saom_result *results, int count,
                         int shared_params, cusna_saom_plan **out) {
  if (!problems || !results || !out) { set_err("problems, results and plan are required"); return CUSNA_ERR_NULL_ARG; }
  *out = nullptr;
  if (count < 1) { set_err("count %d < 1", count); return CUSNA_ERR_SHAPE; }
  if (shared_params != 0 && shared_params != 1) { set_err("shared_params must be 0 or 1"); return CUSNA_ERR_SHAPE; }
  cusna_status s;
  if ((s = ensure_ctx()) != CUSNA_OK) return s;
  const bool one = shared_params == 1;
  std::vector<Job> jobs(count);
  for (int q = 0; q < count; ++q) {
    jobs[q].p = &problems[q];
    jobs[q].r = &results[q];
    if ((s = validate(&problems[q], &results[q], true, jobs[q].F, one)) != CUSNA_OK) return s;
    // with a row per chain the kernel multiplies (rows may differ at a later launch)
    if (!one) jobs[q].F.flags &= ~F_THETA_TAB;
  }
  order_longest_first(jobs);
  int nmax = 0, Wmax = 0, kmax = 0, kbmax = 0, nrmax = 0;
  bool tp = false, gw = false, tq = false;
  long long total = 0;
  for (auto &J : jobs) {
    nmax = std::max(nmax, J.p->n); Wmax = std::max(Wmax, J.p->W); kmax = std::max(kmax, J.p->k);
    kbmax = std::max(kbmax, J.p->kb); nrmax = std::max(nrmax, J.p->nrate);
    tp |= (J.F.flags & F_NEED_TP) != 0;
    gw |= (J.F.flags & (F_NEED_GW29 | F_NEED_TP)) != 0;
    tq |= (J.F.flags & F_NEED_GW30) != 0;
    total += J.p->M;
  }
  const std::vector<LaunchShape> ranked =
      rank_shapes(nmax, Wmax, kmax, kbmax, nrmax, tp, gw, tq, total, 0, 0);
  if (ranked.empty()) { set_err("no launch shape fits n=%d", nmax); return CUSNA_ERR_UNSUPPORTED; }
  std::vector<LaunchShape> cand = tuning_candidates(ranked);
  {
    // a signature the tuner has settled needs no exploration
    const TuneKey key = tune_key(nmax, Wmax, kmax, kbmax, nrmax, tp, gw, tq, total);
    std::lock_guard<std::mutex> lk(g_tune_mu);
    for (auto &e : g_tune)
      if (std::memcmp(&e.key, &key, sizeof key) == 0 && e.next >= e.cand.size() && e.best >= 0)
        cand = {e.cand[e.best]};
  }
  if (!tuning_enabled()) cand.resize(1);
  const LaunchShape sh = cand[0];
  size_t teams = 0;
  bool cols_global = false, rows_global = false;
  for (const LaunchShape &x : cand) {
    teams = std::max(teams, (size_t)x.ctas * x.teams_per_cta);
    cols_global |= !x.cols_in_smem;
    rows_global |= !x.rows_in_smem;
  }
  std::vector<PlanTable> tabs;
  for (int q = 0; q < count; ++q) {
    const Facts &F = jobs[q].F;
    if (!(F.flags & F_THETA_TAB)) continue;
    for (int e = 0; e < jobs[q].p->k; ++e)
      if (F.tsize[e] > 0) tabs.push_back(PlanTable{q, e, F.kind[e], F.offt[e], F.offd[e], F.tsize[e]});
  }
  Planner pl;
  for (auto &J : jobs) plan_problem(pl, J, true);
  const size_t o_probs = pl.take(sizeof(DevProblem) * count);
  const size_t o_units = pl.take(sizeof(long long) * (count + 1));
  const size_t o_counter = pl.take(8), o_epoch = pl.take(8), o_seeds = pl.take(8 * (size_t)count);
  const size_t o_tabs = pl.take(sizeof(PlanTable) * std::max<size_t>(1, tabs.size()));
  const size_t cols_words = (size_t)Wmax * nmax;
  const size_t o_cols = cols_global ? pl.take(teams * cols_words * 4) : NONE;
  const size_t o_rows = rows_global ? pl.take(teams * cols_words * 4) : NONE;

  cusna_saom_plan *P = new cusna_saom_plan();
  P->cand = cand;
  P->cand_ms.assign(cand.size(), INFINITY);
  P->trial = cand.size() > 1 ? 0 : cand.size();
  if (cand.size() > 1 &&
      (cudaEventCreate(&P->ev0) != cudaSuccess || cudaEventCreate(&P->ev1) != cudaSuccess)) {
    cudaGetLastError();
    plan_free(P);
    set_err("plan: cudaEventCreate failed");
    return CUSNA_ERR_CUDA;
  }
  P->device = g_ctx.device;
  if (cudaMalloc(&P->mem, pl.off) != cudaSuccess) {
    cudaGetLastError();
    plan_free(P);
    set_err("plan: cudaMalloc of %zu bytes failed", pl.off);
    return CUSNA_ERR_CUDA;
  }
  // prepare() places each problem in the thread's arena: point the arena at the
  // plan's memory for the duration
  struct ArenaSwap {
    void *arena; size_t cap;
    ~ArenaSwap() { g_ctx.arena = arena; g_ctx.cap = cap; }
  } restore{g_ctx.arena, g_ctx.cap};
  g_ctx.arena = P->mem;
  g_ctx.cap = pl.off;
  std::vector<DevProblem> hp(count);
  std::vector<long long> units(count + 1, 0);
  std::vector<unsigned long long> seeds(count);
  for (int q = 0; q < count; ++q) {
    if ((s = prepare(jobs[q], true, hp[q], 0)) != CUSNA_OK) { plan_free(P); return s; }
    if (!hp[q].scores) hp[q].flags |= F_NO_SCORES;  // no score sums without scores
    hp[q].prow = one ? 0 : 1;
    units[q + 1] = units[q] + jobs[q].p->M;
    seeds[q] = (unsigned long long)jobs[q].p->seed;
  }
  cudaStream_t st = g_ctx.stream;
  auto up = [&](size_t off, const void *src, size_t bytes) {
    return cudaMemcpyAsync(at<char>(off), src, bytes, cudaMemcpyHostToDevice, st);
  };
  cudaError_t e = up(o_probs, hp.data(), sizeof(DevProblem) * count);
  if (e == cudaSuccess) e = up(o_units, units.data(), sizeof(long long) * units.size());
  if (e == cudaSuccess) e = up(o_seeds, seeds.data(), 8 * seeds.size());
  if (e == cudaSuccess && !tabs.empty()) e = up(o_tabs, tabs.data(), sizeof(PlanTable) * tabs.size());
  if (e == cudaSuccess) e = cudaMemsetAsync(at<char>(o_counter), 0, 8, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(at<char>(o_epoch), 0, 8, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    set_err("plan: staging failed: %s", cudaGetErrorString(e));
    plan_free(P);
    return CUSNA_ERR_CUDA;
  }
  P->sh = sh;
  P->probs = at<DevProblem>(o_probs);
  P->units = at<long long>(o_units);
  P->counter = at<unsigned long long>(o_counter);
  P->epoch = at<unsigned long long>(o_epoch);
  P->seeds = at<unsigned long long>(o_seeds);
  P->tabs = at<PlanTable>(o_tabs);
  P->count = count;
  P->n_tabs = (int)tabs.size();
  P->total = total;
  P->cols = o_cols == NONE ? nullptr : at<uint32_t>(o_cols);
  P->rows = o_rows == NONE ? nullptr : at<uint32_t>(o_rows);
  P->cols_words = cols_words;
  P->spec = launch_spec(jobs);
  *out = P;
  return CUSNA_OK;
}

// Kernel launches only (capture-safe): epoch and term tables, work counter,
// the persistent period kernel.
cusna_status plan_enqueue(cusna_saom_plan *P, const LaunchShape &sh, cudaStream_t st) {
  CU(launch_plan_prologue(P->probs, P->seeds, P->count, P->epoch, P->tabs, P->n_tabs, st));
  CU(cudaMemsetAsync(P->counter, 0, sizeof(unsigned long long), st));
  if (P->jit)
    CU(launch_period_jit(P->jk, sh, P->probs, P->units, P->count, P->total, P->counter,
                         sh.cols_in_smem ? nullptr : P->cols, sh.rows_in_smem ? nullptr : P->rows,
                         P->cols_words, st));
  else
    CU(launch_period(sh, P->probs, P->units, P->count, P->total, P->counter,
                     sh.cols_in_smem ? nullptr : P->cols, sh.rows_in_smem ? nullptr : P->rows,
                     P->cols_words, st));
  return CUSNA_OK;
}

cusna_status plan_launch(cusna_saom_plan *P, cudaStream_t st, bool graph) {
  if (!P) { set_err("plan is NULL"); return CUSNA_ERR_NULL_ARG; }
  int dev = -1;
  CU(cudaGetDevice(&dev));
  if (dev != P->device) { set_err("plan belongs to device %d, current is %d", P->device, dev); return CUSNA_ERR_UNSUPPORTED; }
  // autotuning: the first launches are timed trials of the candidate shapes
  // (never inside a stream capture); the fastest is kept, before any graph
  if (P->pending) {
    float ms = 0.f;
    CU(cudaEventSynchronize(P->ev1));
    CU(cudaEventElapsedTime(&ms, P->ev0, P->ev1));
    P->cand_ms[P->trial - 1] = ms;
    P->pending = false;
    size_t b = 0;
    for (size_t x = 1; x < P->cand_ms.size(); ++x)
      if (P->cand_ms[x] < P->cand_ms[b]) b = x;
    P->sh = P->cand[b];
  }
  cudaStreamCaptureStatus cap_status = cudaStreamCaptureStatusNone;
  CU(cudaStreamIsCapturing(st, &cap_status));
  if (!P->jit && !P->pending && !P->spec.empty() && cap_status == cudaStreamCaptureStatusNone &&
      jit_get(P->spec, &P->jk)) {
    // the specialised kernel is ready: time the candidate shapes again with it
    // and capture a new graph (same smem layout, so every candidate fits the
    // plan's scratch)
    P->jit = true;
    if (P->cand.size() > 1) {
      P->trial = 0;
      P->cand_ms.assign(P->cand.size(), INFINITY);
    }
    if (P->graph) {
      cudaGraphExecDestroy(P->graph);
      P->graph = nullptr;
    }
  }
  if (P->trial < P->cand.size() && cap_status == cudaStreamCaptureStatusNone) {
    const LaunchShape sh = P->cand[P->trial];
    CU(cudaEventRecord(P->ev0, st));
    const cusna_status s = plan_enqueue(P, sh, st);
    CU(cudaEventRecord(P->ev1, st));
    ++P->trial;
    P->pending = s == CUSNA_OK;
    return s;
  }
  if (!graph) return plan_enqueue(P, P->sh, st);
  if (!P->graph) {
    cudaStream_t cap = nullptr;
    CU(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeRelaxed);
    if (e != cudaSuccess) {
      cudaStreamDestroy(cap);
      set_err("plan: begin capture failed: %s", cudaGetErrorString(e));
      return CUSNA_ERR_CUDA;
    }
    cusna_status s = plan_enqueue(P, P->sh, cap);
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(cap, &g);   // ends the capture on every path
    cudaStreamDestroy(cap);
    if (s != CUSNA_OK || e != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      if (s == CUSNA_OK) set_err("plan: capture failed: %s", cudaGetErrorString(e));
      return s != CUSNA_OK ? s : CUSNA_ERR_CUDA;
    }
    e = cudaGraphInstantiate(&P->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      P->graph = nullptr;
      set_err("plan: graph instantiation failed: %s", cudaGetErrorString(e));
      return CUSNA_ERR_CUDA;
    }
  }
  CU(cudaGraphLaunch(P->graph, st));
  return CUSNA_OK;
}

}  // namespace

// Error text for cusna_last_error() from the other translation units.
void set_last_error(const char *msg) { g_err = msg; }

}  // namespace cusna

using namespace cusna;

extern "C" {

CUSNA_API cusna_status cusna_saom_simulate_period(const cusna_saom_problem *problem,
                                                  cusna_saom_result *result) {
  g_err.clear();
  if (!problem || !result) { set_err("problem or result is NULL"); return CUSNA_ERR_NULL_ARG; }
  NvtxRange r("cusna_saom_simulate_period");
  return simulate(problem, result, 1, nullptr);
}

CUSNA_API cusna_status cusna_saom_simulate_period_ex(const cusna_saom_problem *problem,
                                                     cusna_saom_result *result,
                                                     cusna_gpu_options *opts) {
  g_err.clear();
  if (!problem || !result) { set_err("problem or result is NULL"); return CUSNA_ERR_NULL_ARG; }
  NvtxRange r("cusna_saom_simulate_period_ex");
  return simulate(problem, result, 1, opts);
}

CUSNA_API cusna_status cusna_saom_simulate_period_validate(const cusna_saom_problem *problem,
                                                           cusna_saom_result *result,
                                                           const cusna_validation_options *vo) {
  using namespace cusna;
  g_err.clear();
  if (!problem || !result || !vo) { set_err("problem, result or options is NULL"); return CUSNA_ERR_NULL_ARG; }
  if (vo->struct_version != CUSNA_ABI_VERSION) {
    set_err("validation options struct_version %d", vo->struct_version);
    return CUSNA_ERR_SHAPE;
  }
  if (vo->trace_cap < 0 || vo->ustream_steps < 0 || (vo->trace_cap > 0 && !vo->trace) ||
      (vo->ustream_steps > 0 && !vo->ustream)) {
    set_err("trace or ustream is NULL (or a negative count)");
    return CUSNA_ERR_NULL_ARG;
  }
  if (vo->warps_per_chain < 0 || vo->warps_per_chain > 8 || vo->chains_per_cta < 0 ||
      32 * (vo->warps_per_chain ? vo->warps_per_chain : 1) *
              (vo->chains_per_cta ? vo->chains_per_cta : 1) > 256) {
    set_err("the validation build runs CTAs of at most 256 threads");
    return CUSNA_ERR_UNSUPPORTED;
  }
  Job J;
  J.p = problem;
  J.r = result;
  cusna_status s = validate(problem, result, false, J.F);
  if (s != CUSNA_OK) return s;
  if ((s = ensure_ctx()) != CUSNA_OK) return s;
  std::vector<Job> jobs(1, J);
  return run_jobs(jobs, false, nullptr, vo);
}

CUSNA_API cusna_status cusna_saom_simulate_batch(const cusna_saom_problem *problems,
                                                 cusna_saom_result *results, int32_t count,
                                                 cusna_gpu_options *opts) {
  g_err.clear();
  NvtxRange r("cusna_saom_simulate_batch");
  return simulate(problems, results, count, opts);
}

CUSNA_API cusna_status cusna_saom_specialise_check(const cusna_saom_problem *problem, char *log,
                                                   size_t log_len, double *seconds) {
  g_err.clear();
  if (!problem) { set_err("problem is NULL"); return CUSNA_ERR_NULL_ARG; }
  cusna_saom_result dummy;
  std::memset(&dummy, 0, sizeof dummy);
  dummy.struct_version = CUSNA_ABI_VERSION;
  Facts F;
  cusna_status s = validate(problem, &dummy, false, F);
  if (s != CUSNA_OK) return s;
  std::string text;
  double sec = 0.0;
  const int st = jit_compile_only(F.spec_w, &text, &sec);
  if (seconds) *seconds = sec;
  if (log && log_len) {
    const size_t m = std::min(log_len - 1, text.size());
    std::memcpy(log, text.data(), m);
    log[m] = 0;
  }
  if (st != 0) {
    set_err("specialised kernel did not compile: %.400s", text.c_str());
    return CUSNA_ERR_UNSUPPORTED;
  }
  return CUSNA_OK;
}

CUSNA_API cusna_status cusna_saom_specialise_check_multi(const cusna_saom_multi_problem *problem,
                                                         char *log, size_t log_len,
                                                         double *seconds) {
  g_err.clear();
  if (!problem) { set_err("problem is NULL"); return CUSNA_ERR_NULL_ARG; }
  cusna_saom_multi_result dummy;
  std::memset(&dummy, 0, sizeof dummy);
  dummy.struct_version = CUSNA_ABI_VERSION;
  std::string text;
  const cusna_status st = simulate_multi(problem, &dummy, true, &text, seconds);
  if (log && log_len) {
    const size_t m = std::min(log_len - 1, text.size());
    std::memcpy(log, text.data(), m);
    log[m] = 0;
  }
  return st;
}

CUSNA_API cusna_status cusna_saom_specialise_mode(int32_t mode) {
  if (mode < -1 || mode > 2) { set_err("specialise mode %d", mode); return CUSNA_ERR_SHAPE; }
  jit_set_mode(mode);
  return CUSNA_OK;
}

CUSNA_API cusna_status cusna_saom_specialise_wait(double seconds, int32_t *compiled) {
  const int c = jit_wait(seconds);
  if (compiled) *compiled = c;
  return CUSNA_OK;
}

CUSNA_API cusna_status cusna_saom_simulate_multi(const cusna_saom_multi_problem *problem,
                                                 cusna_saom_multi_result *result) {
  g_err.clear();
  NvtxRange r("cusna_saom_simulate_multi");
  return simulate_multi(problem, result);
}

CUSNA_API cusna_status cusna_saom_plan_create(const cusna_saom_problem *problems,
                                             cusna_saom_result *results, int32_t count,
                                             int32_t shared_params, cusna_saom_plan **plan) {
  g_err.clear();
  NvtxRange r("cusna_saom_plan_create");
  return plan_create(problems, results, count, shared_params, plan);
}

CUSNA_API cusna_status cusna_saom_plan_launch(cusna_saom_plan *plan, void *stream,
                                             int32_t use_graph) {
  g_err.clear();
  NvtxRange r("cusna_saom_plan_launch");
  return plan_launch(plan, (cudaStream_t)stream, use_graph != 0);
}

CUSNA_API cusna_status cusna_saom_plan_set_epoch(cusna_saom_plan *plan, uint64_t epoch) {
  g_err.clear();
  if (!plan) { set_err("plan is NULL"); return CUSNA_ERR_NULL_ARG; }
  CU(cudaMemcpy(plan->epoch, &epoch, sizeof(epoch), cudaMemcpyHostToDevice));
  return CUSNA_OK;
}

CUSNA_API cusna_status cusna_saom_plan_shape(const cusna_saom_plan *plan, int32_t *warps_per_chain,
                                            int32_t *chains_per_cta, int32_t *ctas) {
  if (!plan) return CUSNA_ERR_NULL_ARG;
  if (warps_per_chain) *warps_per_chain = plan->sh.G;
  if (chains_per_cta) *chains_per_cta = plan->sh.teams_per_cta;
  if (ctas) *ctas = plan->sh.ctas;
  return CUSNA_OK;
}

CUSNA_API void cusna_saom_plan_destroy(cusna_saom_plan *plan) {
  if (plan) cudaDeviceSynchronize();   // no launch of the plan may still be running
  plan_free(plan);
}

CUSNA_API cusna_status cusna_pack_bits(const uint8_t *dense, int32_t n, uint32_t *out_rows,
                                       uint32_t *in_rows, int32_t *W_out) {
  if (!dense || !out_rows || !in_rows) return CUSNA_ERR_NULL_ARG;
  if (n < 1 || n > CUSNA_MAX_N) return CUSNA_ERR_SHAPE;
  const int W = (n + 31) / 32;
  std::memset(out_rows, 0, (size_t)n * W * 4);
  std::memset(in_rows, 0, (size_t)n * W * 4);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j)
      if (dense[(size_t)i * n + j]) {
        out_rows[(size_t)i * W + (j >> 5)] |= 1u << (j & 31);
        in_rows[(size_t)j * W + (i >> 5)] |= 1u << (i & 31);
      }
  if (W_out) *W_out = W;
  return CUSNA_OK;
}

CUSNA_API cusna_status cusna_philox4x32(const uint32_t counter[4], const uint32_t key[2],
                                        uint32_t out[4]) {
  if (!counter || !key || !out) return CUSNA_ERR_NULL_ARG;
  philox10(counter[0], counter[1], counter[2], counter[3], key[0], key[1], out);
  return CUSNA_OK;
}

CUSNA_API int32_t cusna_abi_version(void) { return CUSNA_ABI_VERSION; }

CUSNA_API const char *cusna_version_string(void) {
  return "cusna-gb300 0.1 (sm_103a period simulator)";
}

CUSNA_API int32_t cusna_has_cuda(void) {
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return count > 0 ? 1 : 0;
}

CUSNA_API const char *cusna_last_error(void) { return g_err.c_str(); }

CUSNA_API cusna_status cusna_network_stats_gpu(
    const uint8_t *a_batch, int32_t n, int32_t M, int32_t k, const int32_t *type_ids,
    const double *p1, const double *p2, const double *vmat, const uint8_t *vmiss,
    const int32_t *dyn_flags, const double *vb, const int32_t *od0, const int32_t *id0,
    const double *wtab, int32_t symflag, double *out) {
  g_err.clear();
  if (!a_batch || !type_ids || !out) { set_err("a_batch, type_ids and out are required"); return CUSNA_ERR_NULL_ARG; }
  if (n < 1 || n > CUSNA_MAX_N || k < 1 || M < 1) { set_err("bad shape"); return CUSNA_ERR_SHAPE; }
  cusna_status s = ensure_ctx();
  if (s != CUSNA_OK) return s;
  cudaStream_t st = g_ctx.stream;
  const size_t nn = (size_t)n * n;
  Planner pl;
  const size_t oa = pl.take(nn * M), ot = pl.take(k * 4), o1 = pl.take(k * 8), o2 = pl.take(k * 8);
  const size_t ov = pl.take((size_t)k * n * 8), om = pl.take((size_t)k * n), od = pl.take(k * 4);
  const size_t ob = pl.take((size_t)n * 8), oo = pl.take((size_t)n * 4), oi = pl.take((size_t)n * 4);
  const size_t ow = pl.take((size_t)k * (n + 1) * 8), oout = pl.take((size_t)M * k * 8);
  if ((s = ensure_arena(pl.off)) != CUSNA_OK) return s;
  auto put = [&](size_t off, const void *src, size_t bytes) -> bool {
    if (!src) return false;
    return cudaMemcpyAsync(at<char>(off), src, bytes, cudaMemcpyHostToDevice, st) == cudaSuccess;
  };
  CU(cudaMemcpyAsync(at<char>(oa), a_batch, nn * M, cudaMemcpyHostToDevice, st));
  put(ot, type_ids, k * 4);
  StatDesc D{};
  D.type_ids = at<int>(ot);
  D.p1 = put(o1, p1, k * 8) ? at<double>(o1) : nullptr;
  D.p2 = put(o2, p2, k * 8) ? at<double>(o2) : nullptr;
  D.vmat = put(ov, vmat, (size_t)k * n * 8) ? at<double>(ov) : nullptr;
  D.vmiss = put(om, vmiss, (size_t)k * n) ? at<uint8_t>(om) : nullptr;
  D.dyn = put(od, dyn_flags, k * 4) ? at<int>(od) : nullptr;
  D.vb = put(ob, vb, (size_t)n * 8) ? at<double>(ob) : nullptr;
  D.od0 = put(oo, od0, (size_t)n * 4) ? at<int>(oo) : nullptr;
  D.id0 = put(oi, id0, (size_t)n * 4) ? at<int>(oi) : nullptr;
  D.wtab = put(ow, wtab, (size_t)k * (n + 1) * 8) ? at<double>(ow) : nullptr;
  D.n = n; D.W = (n + 31) / 32; D.k = k; D.symflag = symflag;
  CU(launch_netstats(at<uint8_t>(oa), M, D, at<double>(oout), g_ctx.sms, st));
  CU(cudaMemcpyAsync(out, at<char>(oout), (size_t)M * k * 8, cudaMemcpyDeviceToHost, st));
  CU(cudaStreamSynchronize(st));
  return CUSNA_OK;
}

CUSNA_API cusna_status cusna_cross_stats(const uint8_t *a_batch, const uint8_t *wp, int32_t n,
                                         int32_t M, int32_t t, double parm, double *out) {
  g_err.clear();
  // the reference reports every argument error as a NULL argument
  // (src/libcusna_saom_cpu.cpp:823-824) and an unknown type as unsupported
  if (!a_batch || !wp || !out || n < 1 || n > CUSNA_MAX_N || M < 1) {
    set_err("a_batch, wp and out are required; 1 <= n <= %d, M >= 1", CUSNA_MAX_N);
    return CUSNA_ERR_NULL_ARG;
  }
  if (t < 33 || t > 37) { set_err("cross effect type %d", t); return CUSNA_ERR_UNSUPPORTED; }
  cusna_status s = ensure_ctx();
  if (s != CUSNA_OK) return s;
  cudaStream_t st = g_ctx.stream;
  const size_t nn = (size_t)n * n, W = (size_t)(n + 31) / 32;
  Planner pl;
  const size_t oa = pl.take(nn * M), ow = pl.take(nn), oout = pl.take((size_t)M * 8);
  const size_t oar = t == 37 ? pl.take((size_t)M * n * W * 4) : NONE;
  const size_t owr = t == 36 ? pl.take((size_t)n * W * 4) : NONE;
  if ((s = ensure_arena(pl.off)) != CUSNA_OK) return s;
  CU(cudaMemcpyAsync(at<char>(oa), a_batch, nn * M, cudaMemcpyHostToDevice, st));
  CU(cudaMemcpyAsync(at<char>(ow), wp, nn, cudaMemcpyHostToDevice, st));
  CU(launch_cross_stats(at<uint8_t>(oa), at<uint8_t>(ow), n, M, t, parm,
                        oar == NONE ? nullptr : at<uint32_t>(oar),
                        owr == NONE ? nullptr : at<uint32_t>(owr), at<double>(oout), st));
  CU(cudaMemcpyAsync(out, at<char>(oout), (size_t)M * 8, cudaMemcpyDeviceToHost, st));
  CU(cudaStreamSynchronize(st));
  return CUSNA_OK;
}

CUSNA_API cusna_status cusna_typed_stats(const uint8_t *a_batch, int32_t n, int32_t M,
                                         int32_t etype, const double *F, const uint8_t *x0,
                                         const uint8_t *keep, const uint8_t *force,
                                         const uint8_t *keepS, const uint8_t *forceS,
                                         const uint8_t *miss_m, const uint8_t *miss_m1,
                                         double *out) {
  g_err.clear();
  // argument errors as the reference reports them (src/libcusna_saom_cpu.cpp:697)
  if (!a_batch || !F || !x0 || !out || n < 1 || M < 1) {
    set_err("a_batch, F, x0 and out are required; n >= 1, M >= 1");
    return CUSNA_ERR_NULL_ARG;
  }
  cusna_status s = ensure_ctx();
  if (s != CUSNA_OK) return s;
  cudaStream_t st = g_ctx.stream;
  const size_t nn = (size_t)n * n;
  Planner pl;
  const size_t oa = pl.take(nn * M), oF = pl.take(nn * 8), ox = pl.take(nn), oout = pl.take((size_t)M * 8);
  const uint8_t *masks[6] = {keep, force, keepS, forceS, miss_m, miss_m1};
  size_t om[6];
  for (int q = 0; q < 6; ++q) om[q] = masks[q] ? pl.take(nn) : NONE;
  if ((s = ensure_arena(pl.off)) != CUSNA_OK) return s;
  CU(cudaMemcpyAsync(at<char>(oa), a_batch, nn * M, cudaMemcpyHostToDevice, st));
  CU(cudaMemcpyAsync(at<char>(oF), F, nn * 8, cudaMemcpyHostToDevice, st));
  CU(cudaMemcpyAsync(at<char>(ox), x0, nn, cudaMemcpyHostToDevice, st));
  const uint8_t *dm[6];
  for (int q = 0; q < 6; ++q) {
    dm[q] = nullptr;
    if (om[q] == NONE) continue;
    CU(cudaMemcpyAsync(at<char>(om[q]), masks[q], nn, cudaMemcpyHostToDevice, st));
    dm[q] = at<uint8_t>(om[q]);
  }
  CU(launch_typed_stats(at<uint8_t>(oa), n, M, etype, at<double>(oF), at<uint8_t>(ox), dm[0],
                        dm[1], dm[2], dm[3], dm[4], dm[5], at<double>(oout), st));
  CU(cudaMemcpyAsync(out, at<char>(oout), (size_t)M * 8, cudaMemcpyDeviceToHost, st));
  CU(cudaStreamSynchronize(st));
  return CUSNA_OK;
}

CUSNA_API cusna_status cusna_gof_distribution(const uint8_t *a_batch, int32_t n, int32_t M,
                                              int32_t kind, const int32_t *levls, int32_t nlev,
                                              double *out) {
  g_err.clear();
  // argument errors as the reference reports them (src/libcusna_saom_cpu.cpp:719)
  if (!a_batch || !levls || !out || n < 1 || M < 1 || nlev < 1) {
    set_err("a_batch, levls and out are required; n >= 1, M >= 1, nlev >= 1");
    return CUSNA_ERR_NULL_ARG;
  }
  if (kind < 0 || kind > 2) { set_err("gof kind %d", kind); return CUSNA_ERR_UNSUPPORTED; }
  int maxlev = 0;
  for (int L = 0; L < nlev; ++L) {
    // a negative geodesic level indexes before the reference's count table
    if (kind == 2 && levls[L] < 0) { set_err("geodesic level %d < 0", levls[L]); return CUSNA_ERR_SHAPE; }
    maxlev = std::max(maxlev, (int)levls[L]);
  }
  // nothing changes beyond distance n - 1
  const int K = kind == 2 ? std::min(maxlev, n - 1) : 0;
  cusna_status s = ensure_ctx();
  if (s != CUSNA_OK) return s;
  cudaStream_t st = g_ctx.stream;
  const size_t nn = (size_t)n * n;
  const size_t cols = kind == 2 ? (size_t)nlev + 1 : (size_t)nlev;
  Planner pl;
  const size_t oa = pl.take(nn * M), ol = pl.take((size_t)nlev * 4), oout = pl.take((size_t)M * cols * 8);
  const size_t words = gof_scratch_words(n, M, kind, K);
  const size_t orow = words ? pl.take(words * 4) : NONE;
  const size_t oadd = kind == 2 ? pl.take((size_t)M * (K + 1) * 8) : NONE;
  if ((s = ensure_arena(pl.off)) != CUSNA_OK) return s;
  CU(cudaMemcpyAsync(at<char>(oa), a_batch, nn * M, cudaMemcpyHostToDevice, st));
  CU(cudaMemcpyAsync(at<char>(ol), levls, (size_t)nlev * 4, cudaMemcpyHostToDevice, st));
  CU(launch_gof(at<uint8_t>(oa), n, M, kind, at<int>(ol), nlev, K,
                orow == NONE ? nullptr : at<uint32_t>(orow),
                oadd == NONE ? nullptr : at<unsigned long long>(oadd), at<double>(oout),
                g_ctx.smem_optin, st));
  CU(cudaMemcpyAsync(out, at<char>(oout), (size_t)M * cols * 8, cudaMemcpyDeviceToHost, st));
  CU(cudaStreamSynchronize(st));
  return CUSNA_OK;
}

CUSNA_API cusna_status cusna_behavior_stats_gpu(const int32_t *z_batch, int32_t n, int32_t M,
                                                int32_t kb, const int32_t *bty,
                                                const uint8_t *xnet, const int32_t *bkdist,
                                                double zbar, double brange, double bsimmean,
                                                double *out) {
  g_err.clear();
  if (!z_batch || !bty || !xnet || !out) { set_err("z_batch, bty, xnet and out are required"); return CUSNA_ERR_NULL_ARG; }
  if (n < 1 || n > CUSNA_MAX_N || M < 1 || kb < 1) { set_err("bad shape"); return CUSNA_ERR_SHAPE; }
  cusna_status s = ensure_ctx();
  if (s != CUSNA_OK) return s;
  cudaStream_t st = g_ctx.stream;
  Planner pl;
  const size_t oz = pl.take((size_t)M * n * 4), ob = pl.take(kb * 4), ox = pl.take((size_t)n * n);
  const size_t ok = pl.take((size_t)n * 4), oo = pl.take((size_t)M * kb * 8);
  if ((s = ensure_arena(pl.off)) != CUSNA_OK) return s;
  CU(cudaMemcpyAsync(at<char>(oz), z_batch, (size_t)M * n * 4, cudaMemcpyHostToDevice, st));
  CU(cudaMemcpyAsync(at<char>(ob), bty, kb * 4, cudaMemcpyHostToDevice, st));
  CU(cudaMemcpyAsync(at<char>(ox), xnet, (size_t)n * n, cudaMemcpyHostToDevice, st));
  if (bkdist) CU(cudaMemcpyAsync(at<char>(ok), bkdist, (size_t)n * 4, cudaMemcpyHostToDevice, st));
  CU(launch_behstats(at<int>(oz), n, M, kb, at<int>(ob), at<uint8_t>(ox),
                     bkdist ? at<int>(ok) : nullptr, zbar, brange, bsimmean, at<double>(oo),
                     g_ctx.sms, st));
  CU(cudaMemcpyAsync(out, at<char>(oo), (size_t)M * kb * 8, cudaMemcpyDeviceToHost, st));
  CU(cudaStreamSynchronize(st));
  return CUSNA_OK;
}

}  // extern "C"
