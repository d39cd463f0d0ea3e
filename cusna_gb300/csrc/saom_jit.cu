// saom_jit.cu -- run-time specialisation of the period kernel to one effect
// plan: source generation, NVRTC compilation in a background thread, module
// loading and launch through driver entry points. See saom_jit.h.
#include <cuda.h>
#include <dlfcn.h>
#include <unistd.h>
#include <sys/stat.h>
#include <nvrtc.h>
#include <nvtx3/nvToolsExt.h>

#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <functional>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "saom_jit.h"
#include "jit_sources.inc"   // kJitHeaderNames / kJitHeaderSources (build.py)

namespace cusna {

// ---- generated source --------------------------------------------------------
// Each effect becomes the branch of change_stats32 / change_stats
// (saom_kernel.cuh) that its kind selects, with the kind, count function,
// type, creation/endowment type and interaction components as constants.
// Offsets, theta and every table stay run-time values, so one compiled plan
// serves every problem with that plan.
namespace {

struct Gen {
  std::string s;
  char buf[640];
  template <class... A>
  void put(const char *fmt, A... a) {
    std::snprintf(buf, sizeof buf, fmt, a...);
    s += buf;
  }
};

const int kPcAll = F_PC_RI_CJ | F_PC_RI_RJ | F_PC_RJ_CI | F_PC_CI_CJ | F_PC_CI_RJ | F_PC_RICIRJ;

void gen_pair_counts(Gen &g, int fl) {
  g.s += "  int ri_cj = 0, ri_rj = 0, rj_ci = 0, ci_cj = 0, ci_rj = 0, ricirj = 0;\n"
         "  (void)ri_cj; (void)ri_rj; (void)rj_ci; (void)ci_cj; (void)ci_rj; (void)ricirj;\n";
  if (!(fl & kPcAll)) return;
  g.s += "  for (int w = 0; w < W; ++w) {\n"
         "    const uint32_t ri = S.rowsT[w * n + i], rj = S.rowsT[w * n + j];\n"
         "    const uint32_t ci = S.colsT[w * n + i], cj = S.colsT[w * n + j];\n"
         "    (void)ri; (void)rj; (void)ci; (void)cj;\n";
  if (fl & F_PC_RI_CJ) g.s += "    ri_cj += __popc(ri & cj);\n";
  if (fl & F_PC_RI_RJ) g.s += "    ri_rj += __popc(ri & rj);\n";
  if (fl & F_PC_RJ_CI) g.s += "    rj_ci += __popc(rj & ci);\n";
  if (fl & F_PC_CI_CJ) g.s += "    ci_cj += __popc(ci & cj);\n";
  if (fl & F_PC_CI_RJ) g.s += "    ci_rj += __popc(ci & rj);\n";
  if (fl & F_PC_RICIRJ) g.s += "    ricirj += __popc(ri & ci & rj);\n";
  g.s += "  }\n";
}

// the integer magnitude c of a K_CNT effect, or the table index of a K_LOOK one
void gen_count(Gen &g, int cfn) {
  switch (cfn) {
    case 0: g.s += "    const int c = 1;\n"; break;
    case 1: g.s += "    const int c = aji;\n"; break;
    case 2: g.s += "    const int c = ri_cj + ri_rj;\n"; break;
    case 3: g.s += "    const int c = rj_ci;\n"; break;
    case 4: g.s += "    const int c = S.indeg[j] + 1 - aij;\n"; break;
    case 5:
      g.s += "    int c = 0;\n"
             "    const uint32_t *eq = S.tpeq + (aij ? W : 0);\n"
             "    for (int w = 0; w < W; ++w)\n"
             "      c += __popc(S.rowsT[w * n + i] & S.rowsT[w * n + j] & eq[w]);\n"
             "    if (S.tp[j] > 0) ++c;\n";
      break;
    case 6: g.s += "    const int c = (aji ? ri_cj : 0) + ricirj;\n"; break;
    default: g.s += "    const int c = S.outdeg[j];\n"; break;
  }
}
void gen_index(Gen &g, int cfn) {
  switch (cfn) {
    case 4: g.s += "    const int idx = S.indeg[j] + 1 - aij;\n"; break;
    case 7: g.s += "    const int idx = S.outdeg[j];\n"; break;
    case 8: g.s += "    const int idx = ri_cj;\n"; break;
    case 9: g.s += "    const int idx = ri_rj;\n"; break;
    case 10: g.s += "    const int idx = ci_cj;\n"; break;
    case 11: g.s += "    const int idx = ci_rj;\n"; break;
    case 12: g.s += "    const int idx = j;\n"; break;
    case 13: g.s += "    const int idx = S.z[j] - P.zlo;\n"; break;
    case 14: g.s += "    const int idx = i * n + j;\n"; break;
    default: g.s += "    const int idx = (S.z[i] - P.zlo) * P.zR + (S.z[j] - P.zlo);\n"; break;
  }
}

// the actor and word counts: constants when the plan fixes them
void gen_shape(Gen &g, const JitPlan &J) {
  if (J.n > 0) g.put("  constexpr int n = %d, W = %d;\n", J.n, (J.n + 31) / 32);
  else g.s += "  const int n = P.n, W = P.W;\n";
}

// jit_change_stats32<sfx> and jit_change_stats<sfx><TERMS> of one effect plan
void gen_functions(Gen &g, const JitPlan &J, const std::string &sfx, bool multi) {
  const int k = (int)J.kind.size();
  const int fl = J.pc_flags;
  const char *x = sfx.c_str();
  // float32 pass (change_stats32), with the double-float remainders of the
  // change statistics and of the predictor for the score sums
  g.put("__device__ __forceinline__ float jit_change_stats32%s(const DevProblem &P, const Slice &S,\n"
        "    const StepCtx &X, int j, int aij, int aji, float *d32, float *d32lo, float *absf,\n"
        "    float2 *fx) {\n", x);
  g.s += "  const int i = X.i;\n";
  gen_shape(g, J);
  g.s += "  (void)n; (void)W; (void)i; (void)aji; (void)d32lo;\n";
  gen_pair_counts(g, fl);
  g.put("  const uint32_t sg = aij ? 0x80000000u : 0u;\n"
        "  float f = 0.f, a = 0.f, tt[%d], tl[%d];\n", k, k);
  for (int e = 0; e < k; ++e) {
    const int kind = J.kind[e], cfn = J.cfn[e], t = J.tid[e];
    g.put("  {  // effect %d: type %d, kind %d, function %d\n", e, t, kind, cfn);
    g.put("    const float th = S.th32[%d];\n", e);
    g.s += "    float v, vlo = 0.f, term = 0.f, tlo = 0.f;\n    bool has_term = true;\n"
           "    (void)th; (void)vlo;\n";
    if (kind == K_CNT) {
      gen_count(g, cfn);
      g.s += "    v = __uint_as_float(__float_as_uint((float)c) ^ sg);\n"
             "    term = __fmul_rn(th, v);\n";
      // c in {0, 1} (density, reciprocity): theta * v is exact
      if (cfn != 0 && cfn != 1) g.s += "    tlo = fmaf(th, v, -term);\n";
    } else if (kind == K_LOOK) {
      gen_index(g, cfn);
      g.put("    const float2 t2 = P.tab2[S.eoffd[%d] + idx];\n"
            "    v = __uint_as_float(__float_as_uint(t2.x) ^ sg);\n"
            "    vlo = __uint_as_float(__float_as_uint(t2.y) ^ sg);\n"
            "    term = __fmul_rn(th, v);\n"
            "    tlo = fmaf(th, vlo, fmaf(th, v, -term));\n", e);
    } else if (kind == K_STEP) {
      g.put("    const int q = 2 * aij + aji;\n"
            "    v = S.stepd32[%d + q];\n    vlo = S.stepdlo32[%d + q];\n"
            "    term = S.stept32[%d + q];\n    tlo = S.steptlo32[%d + q];\n",
            4 * e, 4 * e, 4 * e, 4 * e);
    } else if (kind == K_ZERO) {
      g.s += "    v = 0.f;\n    has_term = false;\n";
    } else if (multi && kind == K_CROSS) {
      g.put("    const int c = cross_count(S, X, n, W, %d, S.eoffd[%d], i, j);\n"
            "    const bool rt = %d == 36 && S.p1[%d] >= 2.0;\n"
            "    const float m = rt ? sqrtf((float)c) : (float)c;\n"
            "    const float mlo = (rt && c > 0) ? __fdiv_rn(fmaf(-m, m, (float)c), __fmul_rn(2.f, m)) : 0.f;\n"
            "    v = __uint_as_float(__float_as_uint(m) ^ sg);\n"
            "    vlo = __uint_as_float(__float_as_uint(mlo) ^ sg);\n"
            "    term = __fmul_rn(th, v);\n"
            "    tlo = fmaf(th, vlo, fmaf(th, v, -term));\n", cfn, e, cfn, e);
    } else if (t == 32) {
      const int c0 = J.i0[e], c1 = J.i1[e], c2 = J.i2[e];
      g.put("    v = __fmul_rn(d32[%d], d32[%d]);\n"
            "    vlo = __fadd_rn(fmaf(d32[%d], d32[%d], -v),\n"
            "                    fmaf(d32[%d], d32lo[%d], __fmul_rn(d32lo[%d], d32[%d])));\n",
            c0, c1, c0, c1, c0, c1, c0, c1);
      if (c2 >= 0)
        g.put("    {\n      const float v2 = __fmul_rn(v, d32[%d]);\n"
              "      vlo = __fadd_rn(fmaf(v, d32[%d], -v2), fmaf(v, d32lo[%d], __fmul_rn(vlo, d32[%d])));\n"
              "      v = v2;\n    }\n", c2, c2, c2, c2);
      else g.s += "    if (aij) { v = -v; vlo = -vlo; }\n";
      g.s += "    term = __fmul_rn(th, v);\n"
             "    tlo = fmaf(th, vlo, fmaf(th, v, -term));\n";
    } else {
      g.put("    {\n      const double v64 = gen_stat(P, S, X, %d, j, aij, aji, ri_cj, ri_rj, rj_ci,\n"
            "                                  ci_cj, ci_rj, nullptr);\n"
            "      v = (float)v64;\n      vlo = (float)__dsub_rn(v64, (double)v);\n    }\n"
            "    term = __fmul_rn(th, v);\n"
            "    tlo = fmaf(th, vlo, fmaf(th, v, -term));\n", e);
    }
    if (J.ety[e] == 1) g.s += "    if (aij) { v = 0.f; vlo = 0.f; has_term = false; }\n";
    else if (J.ety[e] == 2) g.s += "    if (!aij) { v = 0.f; vlo = 0.f; has_term = false; }\n";
    g.put("    d32[%d] = v;\n    d32lo[%d] = vlo;\n", e, e);
    g.put("    tt[%d] = has_term ? term : 0.f;\n    tl[%d] = has_term ? tlo : 0.f;\n", e, e);
    g.s += "    if (has_term) {\n      f = __fadd_rn(f, term);\n"
           "      a = __fadd_rn(a, fabsf(term));\n    }\n  }\n";
  }
  // the predictor as a double-float pair: the terms' pairs added in a fixed
  // packed tree (f, the float32 sum in effect order, keys the choice)
  g.put("  *absf = a;\n  *fx = ff_tree_sum<%d>(tt, tl);\n  return f;\n}\n", k);
  // float64 evaluation (change_stats): the chosen alter and uncertified choices
  g.put("template <bool TERMS>\n"
        "__device__ __forceinline__ double jit_change_stats%s(const DevProblem &P, const Slice &S,\n"
        "    const StepCtx &X, int j, int aij, int aji, double *d) {\n", x);
  g.s += "  const int i = X.i;\n";
  gen_shape(g, J);
  g.s += "  (void)n; (void)W; (void)i; (void)aji;\n"
         "  const unsigned long long sg = aij ? 0x8000000000000000ull : 0ull;\n"
         "  const bool ttab = (P.flags & F_THETA_TAB) != 0;\n  (void)ttab;\n";
  gen_pair_counts(g, fl);
  g.s += "  double f = 0.0;\n";
  for (int e = 0; e < k; ++e) {
    const int kind = J.kind[e], cfn = J.cfn[e];
    g.put("  {  // effect %d\n", e);
    g.s += "    double v, term = 0.0;\n    bool has_term = TERMS;\n";
    if (kind == K_CNT) {
      gen_count(g, cfn);
      g.put("    v = flip(i2d(c), sg);\n"
            "    if (TERMS) term = ttab ? flip(P.tab[S.eofft[%d] + c], sg) : __dmul_rn(S.th[%d], v);\n",
            e, e);
    } else if (kind == K_LOOK) {
      gen_index(g, cfn);
      g.put("    v = flip(P.tab[S.eoffd[%d] + idx], sg);\n"
            "    if (TERMS) term = ttab ? flip(P.tab[S.eofft[%d] + idx], sg) : __dmul_rn(S.th[%d], v);\n",
            e, e, e);
    } else if (kind == K_STEP) {
      g.put("    const int q = 2 * aij + aji;\n"
            "    v = S.stepd[%d + q];\n    term = S.stept[%d + q];\n", 4 * e, 4 * e);
    } else if (kind == K_ZERO) {
      g.s += "    v = 0.0;\n    has_term = false;\n";
    } else if (multi && kind == K_CROSS) {
      g.put("    const int c = cross_count(S, X, n, W, %d, S.eoffd[%d], i, j);\n"
            "    v = flip((%d == 36 && S.p1[%d] >= 2.0) ? sqrt(i2d(c)) : i2d(c), sg);\n"
            "    if (TERMS) term = __dmul_rn(S.th[%d], v);\n", cfn, e, cfn, e, e);
    } else {
      g.put("    v = gen_stat(P, S, X, %d, j, aij, aji, ri_cj, ri_rj, rj_ci, ci_cj, ci_rj, d);\n"
            "    if (TERMS) term = __dmul_rn(S.th[%d], v);\n", e, e);
    }
    if (J.ety[e] == 1) g.s += "    if (aij) { v = 0.0; has_term = false; }\n";
    else if (J.ety[e] == 2) g.s += "    if (!aij) { v = 0.0; has_term = false; }\n";
    g.put("    d[%d] = v;\n", e);
    g.s += "    if (has_term) f = __dadd_rn(f, term);\n  }\n";
  }
  g.s += "  return f;\n}\n";
}

}  // namespace

// Effects whose change statistic can have a double-float remainder: every
// kind but the integer counts (and the zero dyadic covariate).
unsigned lo_mask(const JitPlan &J) {
  unsigned m = 0;
  for (size_t e = 0; e < J.kind.size(); ++e)
    if (J.kind[e] != K_CNT && J.kind[e] != K_ZERO) m |= 1u << e;
  return m;
}

std::string jit_spec_source(const JitPlan &J) {
  Gen g;
  g.put("#define CUSNA_JIT_SPEC 1\n#define CUSNA_JIT_K %d\n#define CUSNA_JIT_LOMASK 0x%xu\n"
        "namespace cusna {\n", (int)J.kind.size(), lo_mask(J));
  gen_functions(g, J, "", false);
  g.s += "}  // namespace cusna\n";
  return g.s;
}

std::string jit_multi_spec_source(const std::vector<JitPlan> &nets) {
  Gen g;
  g.s += std::string(kJitMultiTag) + "\n#define CUSNA_JIT_MULTI 1\nnamespace cusna {\n";
  const int D = (int)nets.size();
  for (int d = 0; d < D; ++d) gen_functions(g, nets[d], "_n" + std::to_string(d), true);
  // the chosen network's plan (warp-uniform per ministep)
  g.s += "__device__ __forceinline__ float jit_change_stats32(int net, const DevProblem &P,\n"
         "    const Slice &S, const StepCtx &X, int j, int aij, int aji, float *d32, float *d32lo,\n"
         "    float *absf, float2 *fx) {\n"
         "  switch (net) {\n";
  for (int d = 0; d < D; ++d)
    g.put("    case %d: return jit_change_stats32_n%d(P, S, X, j, aij, aji, d32, d32lo, absf, fx);\n",
          d, d);
  g.s += "    default: *absf = 0.f; *fx = make_float2(0.f, 0.f); return 0.f;\n  }\n}\n";
  g.s += "template <bool TERMS>\n"
         "__device__ __forceinline__ double jit_change_stats(int net, const DevProblem &P,\n"
         "    const Slice &S, const StepCtx &X, int j, int aij, int aji, double *d) {\n"
         "  switch (net) {\n";
  for (int d = 0; d < D; ++d)
    g.put("    case %d: return jit_change_stats_n%d<TERMS>(P, S, X, j, aij, aji, d);\n", d, d);
  g.s += "    default: return 0.0;\n  }\n}\n}  // namespace cusna\n";
  return g.s;
}

namespace {

// ---- NVRTC, loaded at run time (the library has no link-time dependency) -----
struct Nvrtc {
  bool ok = false;
  decltype(&nvrtcCreateProgram) create = nullptr;
  decltype(&nvrtcAddNameExpression) add_name = nullptr;
  decltype(&nvrtcCompileProgram) compile = nullptr;
  decltype(&nvrtcGetProgramLogSize) log_size = nullptr;
  decltype(&nvrtcGetProgramLog) get_log = nullptr;
  decltype(&nvrtcGetCUBINSize) cubin_size = nullptr;
  decltype(&nvrtcGetCUBIN) get_cubin = nullptr;
  decltype(&nvrtcGetLoweredName) lowered = nullptr;
  decltype(&nvrtcDestroyProgram) destroy = nullptr;
  decltype(&nvrtcVersion) version = nullptr;  // optional (the cache key)
};

Nvrtc load_nvrtc() {
  Nvrtc N;
  const char *names[] = {"libnvrtc.so.13", "libnvrtc.so", "/usr/local/cuda/lib64/libnvrtc.so.13",
                         "/usr/local/cuda/lib64/libnvrtc.so"};
  void *h = nullptr;
  for (const char *nm : names)
    if ((h = dlopen(nm, RTLD_NOW | RTLD_LOCAL))) break;
  if (!h) return N;
  bool ok = true;
  auto sym = [&](auto &fp, const char *name) {
    fp = reinterpret_cast<std::remove_reference_t<decltype(fp)>>(dlsym(h, name));
    ok = ok && fp != nullptr;
  };
  sym(N.create, "nvrtcCreateProgram");
  sym(N.add_name, "nvrtcAddNameExpression");
  sym(N.compile, "nvrtcCompileProgram");
  sym(N.log_size, "nvrtcGetProgramLogSize");
  sym(N.get_log, "nvrtcGetProgramLog");
  sym(N.cubin_size, "nvrtcGetCUBINSize");
  sym(N.get_cubin, "nvrtcGetCUBIN");
  sym(N.lowered, "nvrtcGetLoweredName");
  sym(N.destroy, "nvrtcDestroyProgram");
  N.version = reinterpret_cast<decltype(&nvrtcVersion)>(dlsym(h, "nvrtcVersion"));
  N.ok = ok;
  return N;
}

const Nvrtc &nvrtc() {
  static const Nvrtc N = load_nvrtc();
  return N;
}

// ---- driver entry points (module loading and launch) --------------------------
struct Driver {
  bool ok = false;
  decltype(&cuModuleLoadData) load = nullptr;
  decltype(&cuModuleUnload) unload = nullptr;
  decltype(&cuModuleGetFunction) get_function = nullptr;
  decltype(&cuFuncSetAttribute) set_attr = nullptr;
  decltype(&cuLaunchKernel) launch = nullptr;
  decltype(&cuOccupancyMaxActiveBlocksPerMultiprocessor) occupancy = nullptr;
};

Driver load_driver() {
  Driver D;
  bool ok = true;
  auto sym = [&](auto &fp, const char *name) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion(name, &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    fp = reinterpret_cast<std::remove_reference_t<decltype(fp)>>(p);
    ok = ok && p != nullptr;
  };
  sym(D.load, "cuModuleLoadData");
  sym(D.get_function, "cuModuleGetFunction");
  sym(D.set_attr, "cuFuncSetAttribute");
  sym(D.launch, "cuLaunchKernel");
  sym(D.occupancy, "cuOccupancyMaxActiveBlocksPerMultiprocessor");
  const bool required = ok;
  sym(D.unload, "cuModuleUnload");   // optional: only a failed load's clean-up
  ok = required;
  cudaGetLastError();
  D.ok = ok;
  return D;
}

const Driver &driver() {
  static const Driver D = load_driver();
  return D;
}

// ---- compilation -------------------------------------------------------------
const char *kPeriodNames[2] = {"cusna::period_kernel<256>", "cusna::period_kernel<512>"};
const char *kMultiNames[2] = {"cusna::multi_kernel<256>", "cusna::multi_kernel<512>"};

bool is_multi(const std::string &spec) {
  return spec.compare(0, std::strlen(kJitMultiTag), kJitMultiTag) == 0;
}

struct Compiled {
  int status = -1;             // 0 ok
  std::vector<char> cubin;
  std::string lowered[2];
  std::string log;
  double seconds = 0.0;
};

// ---- on-disk cache of compiled specialisations -------------------------------
// A compiled plan is written to CUSNA_JIT_CACHE_DIR (default
// $XDG_CACHE_HOME/cusna_gb300, else ~/.cache/cusna_gb300; CUSNA_JIT_CACHE=0
// turns the cache off) under a 128-bit hash of everything the compilation
// depends on: the generated source, the text of every device header it
// includes, the compiler options and the NVRTC version. A later process then
// loads the cubin instead of compiling (milliseconds instead of seconds), and
// a plan found in the cache is used from its first call. Files are written to
// a temporary name and renamed, so a reader never sees a partial file.
struct CacheKey {
  uint64_t a = 1469598103934665603ull, b = 1099511628211ull * 31;
  void add(const void *p, size_t n) {
    const unsigned char *c = (const unsigned char *)p;
    for (size_t i = 0; i < n; ++i) {
      a = (a ^ c[i]) * 1099511628211ull;                 // FNV-1a
      b = (b + c[i] + 1) * 0x9E3779B97F4A7C15ull ^ (b >> 29);
    }
  }
  void add(const std::string &s) { add(s.data(), s.size()); add("\0", 1); }
};

std::string cache_dir() {
  const char *off = std::getenv("CUSNA_JIT_CACHE");
  if (off && off[0] == '0') return "";
  if (const char *d = std::getenv("CUSNA_JIT_CACHE_DIR")) return d;
  if (const char *x = std::getenv("XDG_CACHE_HOME")) return std::string(x) + "/cusna_gb300";
  if (const char *h = std::getenv("HOME")) return std::string(h) + "/.cache/cusna_gb300";
  return "";
}

std::string compile_options_text() {
  std::string minb = "-DCUSNA_MINB_256=2";
  if (const char *m = std::getenv("CUSNA_JIT_MINB")) minb = std::string("-DCUSNA_MINB_256=") + m;
  return minb;
}

// the cache file of a generated source ("" when the cache is off)
std::string cache_path(const std::string &src) {
  const std::string dir = cache_dir();
  if (dir.empty()) return "";
  static const std::string headers = [] {
    std::string h;
    for (int q = 0; q < kJitHeaderCount; ++q) h += std::string(kJitHeaderNames[q]) + kJitHeaderSources[q];
    return h;
  }();
  CacheKey k;
  k.add(src);
  k.add(headers);
  k.add(compile_options_text());
  int major = 0, minor = 0;
  if (nvrtc().version) nvrtc().version(&major, &minor);
  k.add(&major, sizeof major);
  k.add(&minor, sizeof minor);
  char name[80];
  std::snprintf(name, sizeof name, "/jit_%016llx%016llx.bin", (unsigned long long)k.a,
                (unsigned long long)k.b);
  return dir + name;
}

bool cache_read(const std::string &path, Compiled &C) {
  if (path.empty()) return false;
  FILE *f = std::fopen(path.c_str(), "rb");
  if (!f) return false;
  char magic[8] = {};
  uint64_t len[3] = {};
  bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, "CUSNAJC1", 8) == 0 &&
            std::fread(len, sizeof len[0], 3, f) == 3 && len[0] < 4096 && len[1] < 4096 &&
            len[2] > 0 && len[2] < ((uint64_t)1 << 30);
  if (ok) {
    C.lowered[0].resize(len[0]);
    C.lowered[1].resize(len[1]);
    C.cubin.resize(len[2]);
    ok = std::fread(&C.lowered[0][0], 1, len[0], f) == len[0] &&
         std::fread(&C.lowered[1][0], 1, len[1], f) == len[1] &&
         std::fread(C.cubin.data(), 1, len[2], f) == len[2];
  }
  std::fclose(f);
  if (ok) C.status = 0;
  return ok;
}

void cache_write(const std::string &path, const Compiled &C) {
  if (path.empty() || C.status != 0) return;
  const std::string dir = path.substr(0, path.rfind('/'));
  // create the directory and its parent (~/.cache) when missing
  const std::string parent = dir.substr(0, dir.rfind('/'));
  if (!parent.empty()) mkdir(parent.c_str(), 0755);
  mkdir(dir.c_str(), 0755);
  const std::string tmp = path + ".tmp" + std::to_string((long long)getpid());
  FILE *f = std::fopen(tmp.c_str(), "wb");
  if (!f) return;
  const uint64_t len[3] = {C.lowered[0].size(), C.lowered[1].size(), C.cubin.size()};
  bool ok = std::fwrite("CUSNAJC1", 1, 8, f) == 8 && std::fwrite(len, sizeof len[0], 3, f) == 3 &&
            std::fwrite(C.lowered[0].data(), 1, len[0], f) == len[0] &&
            std::fwrite(C.lowered[1].data(), 1, len[1], f) == len[1] &&
            std::fwrite(C.cubin.data(), 1, len[2], f) == len[2];
  ok = (std::fclose(f) == 0) && ok;
  if (!ok || std::rename(tmp.c_str(), path.c_str()) != 0) std::remove(tmp.c_str());
}

std::string full_source(const std::string &spec) {
  return std::string("#include \"saom_kernel.cuh\"\n") + spec +
         (is_multi(spec) ? "#include \"saom_multi_kernel.cuh\"\n" : "#include \"saom_period.cuh\"\n");
}

// true when the plan's compiled kernel is in the on-disk cache
bool cached(const std::string &spec) {
  const std::string path = cache_path(full_source(spec));
  return !path.empty() && access(path.c_str(), R_OK) == 0;
}

Compiled compile_spec(const std::string &spec) {
  Compiled C;
  const bool multi = is_multi(spec);
  const char *const *kNames = multi ? kMultiNames : kPeriodNames;
  const std::string src = full_source(spec);
  const std::string cpath = cache_path(src);
  {
    const auto t0 = std::chrono::steady_clock::now();
    if (cache_read(cpath, C)) {
      C.log = "loaded from the on-disk cache " + cpath;
      C.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
      return C;
    }
    C = Compiled();
  }
  const Nvrtc &N = nvrtc();
  if (!N.ok) {
    C.log = "NVRTC is not available";
    return C;
  }
  // CUSNA_JIT_SOURCE_DIR: also write the generated translation unit there (a
  // file per plan, named by a hash of its text), so it can be read, or
  // compiled offline with nvcc against csrc/ for its register report
  if (const char *dir = std::getenv("CUSNA_JIT_SOURCE_DIR")) {
    char name[64];
    std::snprintf(name, sizeof name, "/cusna_jit_%016zx.cu", std::hash<std::string>{}(src));
    if (FILE *f = std::fopen((std::string(dir) + name).c_str(), "w")) {
      std::fwrite(src.data(), 1, src.size(), f);
      std::fclose(f);
    }
  }
  const auto t0 = std::chrono::steady_clock::now();
  nvtxRangePushA("specialise: NVRTC compile");
  struct PopRange {
    ~PopRange() { nvtxRangePop(); }
  } pop_range;
  nvrtcProgram prog = nullptr;
  if (N.create(&prog, src.c_str(), "cusna_period_jit.cu", kJitHeaderCount, kJitHeaderSources,
               kJitHeaderNames) != NVRTC_SUCCESS) {
    C.log = "nvrtcCreateProgram failed";
    return C;
  }
  for (int q = 0; q < 2; ++q) N.add_name(prog, kNames[q]);
  // CUSNA_JIT_MINB: resident 256-thread CTAs per SM the register budget of
  // the 256-thread instantiation allows (default 2: 128 registers). Measured
  // on the n=200, 4096-chain workload: with the double-float score sums 2
  // gives 90.3 ms against 92.9 for 3 (80 registers, which spill); the earlier
  // float32 sums ran best with 3.
  const std::string minb = compile_options_text();
  const char *opts[] = {"--gpu-architecture=sm_103a", "-std=c++17", "--fmad=false",
                        "-default-device", "-DLIBCUSNA_BUILD", minb.c_str()};
  const nvrtcResult r = N.compile(prog, (int)(sizeof opts / sizeof opts[0]), opts);
  size_t ls = 0;
  N.log_size(prog, &ls);
  if (ls > 1) {
    C.log.resize(ls);
    N.get_log(prog, &C.log[0]);
  }
  if (r == NVRTC_SUCCESS) {
    size_t cs = 0;
    N.cubin_size(prog, &cs);
    C.cubin.resize(cs);
    N.get_cubin(prog, C.cubin.data());
    bool names_ok = true;
    for (int q = 0; q < 2; ++q) {
      const char *lw = nullptr;
      if (N.lowered(prog, kNames[q], &lw) != NVRTC_SUCCESS || !lw) names_ok = false;
      else C.lowered[q] = lw;
    }
    C.status = names_ok && cs > 0 ? 0 : -1;
  }
  N.destroy(&prog);
  C.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  cache_write(cpath, C);
  return C;
}

// ---- registry and the background compiler ----------------------------------------
enum { S_IDLE = 0, S_QUEUED = 1, S_COMPILED = 2, S_LOADED = 3, S_FAILED = -1 };

struct Entry {
  int state = S_IDLE;
  int uses = 0;
  Compiled comp;
  CUmodule mod = nullptr;
  JitKernel k;
};

struct Registry {
  std::mutex mu;
  std::condition_variable cv;
  std::unordered_map<std::string, std::unique_ptr<Entry>> map;
  std::deque<std::pair<std::string, Entry *>> queue;
  bool busy = false;
  bool worker = false;
  bool stopping = false;
  int compiled = 0;
};

// never destroyed: the background compiler may still run at process exit
Registry &reg() {
  static Registry *R = new Registry();
  return *R;
}

void stop_worker_at_exit();

void worker_loop() {
  Registry &R = reg();
  bool first = true;
  for (;;) {
    std::pair<std::string, Entry *> job;
    {
      std::unique_lock<std::mutex> lk(R.mu);
      R.cv.wait(lk, [&] { return !R.queue.empty() || R.stopping; });
      if (R.stopping) return;
      job = R.queue.front();
      R.queue.pop_front();
      R.busy = true;
    }
    Compiled c = compile_spec(job.first);
    // what the compiler built lazily during its first full compilation is
    // destroyed at exit before the handlers registered earlier: register the
    // stop handler once more, after it
    if (first) std::atexit(stop_worker_at_exit);
    first = false;
    {
      std::lock_guard<std::mutex> lk(R.mu);
      job.second->comp = std::move(c);
      job.second->state = job.second->comp.status == 0 ? S_COMPILED : S_FAILED;
      if (job.second->state == S_COMPILED) ++R.compiled;
      R.busy = false;
    }
    R.cv.notify_all();
  }
}

// One tiny compilation with the plans' options in the calling thread, before
// the stop handler is first registered: the compiler library constructs its
// lazily built state here, so at exit (handlers and static destructors run in
// the reverse order of their registration) the handler's wait for a
// compilation in flight comes before that state is destroyed.
void warm_up_compiler() {
  const Nvrtc &N = nvrtc();
  if (!N.ok) return;
  nvrtcProgram prog = nullptr;
  const char *src = "extern \"C\" __global__ void cusna_warm_up(float *x) { x[threadIdx.x] += 1.0f; }\n";
  if (N.create(&prog, src, "cusna_warm_up.cu", 0, nullptr, nullptr) != NVRTC_SUCCESS) return;
  const std::string minb = compile_options_text();
  const char *opts[] = {"--gpu-architecture=sm_103a", "-std=c++17", "--fmad=false",
                        "-default-device", "-DLIBCUSNA_BUILD", minb.c_str()};
  N.compile(prog, (int)(sizeof opts / sizeof opts[0]), opts);
  N.destroy(&prog);
}

// At process exit: drop queued compilations and wait for the one in flight,
// so NVRTC is not inside a compilation while the process tears it down.
void stop_worker_at_exit() {
  Registry &R = reg();
  std::unique_lock<std::mutex> lk(R.mu);
  R.stopping = true;
  for (auto &job : R.queue) job.second->state = S_IDLE;
  R.queue.clear();
  R.cv.notify_all();
  R.cv.wait(lk, [&] { return !R.busy; });
}

int uses_before_compile() {
  const char *s = std::getenv("CUSNA_JIT_AFTER");
  const int v = s ? std::atoi(s) : 3;
  return v < 1 ? 1 : v;
}

// module load in the calling thread's context (the caller holds no capture)
bool load_entry(Entry &E) {
  const Driver &D = driver();
  if (!D.ok) return false;
  if (D.load(&E.mod, E.comp.cubin.data()) != CUDA_SUCCESS) return false;
  CUfunction f[2];
  for (int q = 0; q < 2; ++q)
    if (D.get_function(&f[q], E.mod, E.comp.lowered[q].c_str()) != CUDA_SUCCESS) {
      if (D.unload) D.unload(E.mod);
      E.mod = nullptr;
      return false;
    }
  E.k.f256 = (void *)f[0];
  E.k.f512 = (void *)f[1];
  return true;
}

}  // namespace

namespace {
std::atomic<int> g_mode_override{-1};   // -1: none
}

void jit_set_mode(int mode) { g_mode_override.store(mode); }

int jit_mode() {
  const int o = g_mode_override.load();
  if (o >= 0) return o;
  static const int mode = [] {
    const char *s = std::getenv("CUSNA_JIT");
    if (!s) return 1;
    if (!std::strcmp(s, "0") || !std::strcmp(s, "off")) return 0;
    if (!std::strcmp(s, "sync")) return 2;
    return 1;
  }();
  return mode;
}

bool jit_get(const std::string &spec, JitKernel *out, bool now) {
  const int mode = jit_mode();
  if (mode == 0) return false;
  now = now || mode == 2;
  Registry &R = reg();
  Entry *E = nullptr;
  bool compile_now = false;
  // a loaded module belongs to the device (context) it was loaded on, so the
  // registry holds one entry per device and plan; a second device compiles
  // its own copy (from the on-disk cache when that is on)
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    dev = 0;
  }
  const std::string key = std::to_string(dev) + '\n' + spec;
  {
    std::lock_guard<std::mutex> lk(R.mu);
    auto &slot = R.map[key];
    if (!slot) slot.reset(new Entry());
    E = slot.get();
    if (E->state == S_LOADED) {
      *out = E->k;
      return true;
    }
    if (E->state == S_FAILED) return false;
    ++E->uses;
    // a plan in the on-disk cache loads in milliseconds: take it now
    if (E->state == S_IDLE && !now && E->uses == 1 && cached(spec)) now = true;
    if (E->state == S_IDLE && (now || E->uses >= uses_before_compile())) {
      if (now) {
        E->state = S_QUEUED;
        compile_now = true;
      } else {
        E->state = S_QUEUED;
        R.queue.emplace_back(spec, E);
        if (!R.worker) {
          R.worker = true;
          // the compiler library is loaded and has compiled once first, so
          // this handler runs before its static destructors at exit
          warm_up_compiler();
          std::atexit(stop_worker_at_exit);
          std::thread(worker_loop).detach();
        }
        R.cv.notify_all();
      }
    }
  }
  if (compile_now) {
    Compiled c = compile_spec(spec);
    {
      std::lock_guard<std::mutex> lk(R.mu);
      E->comp = std::move(c);
      E->state = E->comp.status == 0 ? S_COMPILED : S_FAILED;
      if (E->state == S_COMPILED) ++R.compiled;
    }
    // other threads asking for the same plan now wait on its state
    R.cv.notify_all();
  }
  std::unique_lock<std::mutex> lk(R.mu);
  // asked for it now while the background compiler has it: wait for that
  if (now && E->state == S_QUEUED) R.cv.wait(lk, [&] { return E->state != S_QUEUED; });
  if (E->state == S_LOADED) {
    *out = E->k;
    return true;
  }
  if (E->state != S_COMPILED) return false;
  if (!load_entry(*E)) {
    E->state = S_FAILED;
    return false;
  }
  E->state = S_LOADED;
  *out = E->k;
  return true;
}

// The dynamic shared memory limit of a loaded function only rises, for the
// reason raise_dyn_smem gives (one value per function, shared by threads).
static bool raise_jit_dyn_smem(CUfunction f, size_t bytes) {
  static std::mutex mu;
  static std::unordered_map<CUfunction, size_t> limit;
  const Driver &D = driver();
  std::lock_guard<std::mutex> lk(mu);
  size_t &cur = limit[f];
  if (bytes <= cur) return true;
  if (D.set_attr(f, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, (int)bytes) != CUDA_SUCCESS)
    return false;
  cur = bytes;
  return true;
}

int jit_blocks_per_sm(const JitKernel &K, int threads, size_t dyn_smem) {
  const Driver &D = driver();
  CUfunction f = (CUfunction)(threads <= 256 ? K.f256 : K.f512);
  if (!D.ok || !f) return 0;
  if (!raise_jit_dyn_smem(f, dyn_smem)) return 0;
  int blocks = 0;
  if (D.occupancy(&blocks, f, threads, dyn_smem) != CUDA_SUCCESS) return 0;
  return blocks;
}

cudaError_t launch_period_jit(const JitKernel &K, const LaunchShape &sh, const DevProblem *probs,
                              const long long *unit_start, int nprob, long long total,
                              unsigned long long *counter, uint32_t *cols_scratch,
                              uint32_t *rows_scratch, size_t cols_words, cudaStream_t st) {
  const Driver &D = driver();
  const int threads = 32 * sh.G * sh.teams_per_cta;
  const size_t dyn = sh.lay.bytes * sh.teams_per_cta;
  CUfunction f = (CUfunction)(threads <= 256 ? K.f256 : K.f512);
  if (!D.ok || !f) return cudaErrorInvalidDeviceFunction;
  if (!raise_jit_dyn_smem(f, dyn)) return cudaErrorInvalidValue;
  SliceLayout lay = sh.lay;
  int G = sh.G;
  void *args[] = {&probs, &unit_start, &nprob, &total, &counter, &lay, &G, &cols_scratch,
                  &rows_scratch, &cols_words};
  const CUresult r = D.launch(f, (unsigned)sh.ctas, 1, 1, (unsigned)threads, 1, 1, (unsigned)dyn,
                              (CUstream)st, args, nullptr);
  if (r != CUDA_SUCCESS) return cudaErrorLaunchFailure;
  note_launch();
  return cudaSuccess;
}

cudaError_t launch_multi_jit(const JitKernel &K, const LaunchShape &sh, const DevProblem *nets,
                             const MultiDev &md, int M, unsigned long long *counter,
                             uint32_t *cols_scratch, uint32_t *rows_scratch, size_t cols_words,
                             cudaStream_t st) {
  const Driver &D = driver();
  const int threads = 32 * sh.G * sh.teams_per_cta;
  const size_t dyn = sh.lay.bytes * md.D * sh.teams_per_cta;
  CUfunction f = (CUfunction)(threads <= 256 ? K.f256 : K.f512);
  if (!D.ok || !f) return cudaErrorInvalidDeviceFunction;
  if (!raise_jit_dyn_smem(f, dyn)) return cudaErrorInvalidValue;
  MultiDev mdv = md;
  SliceLayout lay = sh.lay;
  int G = sh.G, Mv = M;
  void *args[] = {&nets, &mdv, &Mv, &counter, &lay, &G, &cols_scratch, &rows_scratch, &cols_words};
  const CUresult r = D.launch(f, (unsigned)sh.ctas, 1, 1, (unsigned)threads, 1, 1, (unsigned)dyn,
                              (CUstream)st, args, nullptr);
  if (r != CUDA_SUCCESS) return cudaErrorLaunchFailure;
  note_launch();
  return cudaSuccess;
}

int jit_compile_only(const std::string &spec, std::string *log, double *seconds) {
  Compiled c = compile_spec(spec);
  if (log) *log = c.log;
  if (seconds) *seconds = c.seconds;
  return c.status;
}

int jit_wait(double seconds) {
  Registry &R = reg();
  std::unique_lock<std::mutex> lk(R.mu);
  R.cv.wait_for(lk, std::chrono::duration<double>(seconds),
                [&] { return R.queue.empty() && !R.busy; });
  return R.compiled;
}

}  // namespace cusna
