// saom_static.cu -- cusna_saom_simulate_period_static: the period simulator for
// callers that cannot allocate device memory.
//
// Some callers cannot call cudaMalloc. Hosts whose device memory is
// handed out by another allocator may have none left for a second allocator:
// an R session that pre-reserves the GPU for a framework is one case, an
// embedding application with a fixed memory budget another. Latency-sensitive
// callers also want no allocator calls on their path. This entry point serves
// them. The caller passes device-resident inputs and outputs, as in the
// device-pointer mode of cusna_saom_simulate_period_ex. Every other buffer the
// kernels need lives in one file-scope __device__ array of
// kStaticScratchBytes: the prepared bit matrices and descriptors, the effect
// plan, the launch's work counter and, for large n, the in-rows. Every GPU that
// loads the library holds that array until the process exits.
//
// Calls share the array, and it keeps the last call's contents. Each call
// rewrites everything it reads and clears the work counter before the launch.
// Two calls whose GPU work overlaps (on two streams or from two host threads)
// overwrite each other's scratch and race. Callers must serialise them.
#include <cuda_runtime.h>

#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>

#include "libcusna.h"
#include "saom_launch.h"

namespace cusna {
namespace {

constexpr size_t kStaticScratchBytes = (size_t)16 << 20;  // 16 MiB per device
static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

constexpr int kMaxDevices = 64;
std::atomic<unsigned char *> g_scratch_addr[kMaxDevices];

// Device address of the scratch array on the current device. Host code may
// not use the array's name as a device address (it names a host-side stand-in),
// so the address is looked up once per device, with that device current.
cusna_status scratch_address(unsigned char **out) {
  int count = 0, dev = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count < 1) {
    cudaGetLastError();
    set_last_error("no CUDA device");
    return CUSNA_ERR_NO_CUDA;
  }
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    set_last_error("current device index unavailable or too large");
    return CUSNA_ERR_UNSUPPORTED;
  }
  unsigned char *p = g_scratch_addr[dev].load();
  if (!p) {
    const cudaError_t e = cudaGetSymbolAddress((void **)&p, g_static_scratch);
    if (e != cudaSuccess) {
      char buf[256];
      snprintf(buf, sizeof buf, "cudaGetSymbolAddress of the static scratch failed: %s",
               cudaGetErrorString(e));
      set_last_error(buf);
      return CUSNA_ERR_CUDA;
    }
    g_scratch_addr[dev].store(p);
  }
  *out = p;
  return CUSNA_OK;
}

// Any self-tie (a_ii) in word-major rows: flag[0] = 1.
__global__ void self_tie_kernel(const uint32_t *rowsT, int n, int *flag) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    if ((rowsT[(i >> 5) * n + i] >> (i & 31)) & 1u) flag[0] = 1;
}

struct Bump {
  size_t off = 0;
  size_t take(size_t bytes) {
    const size_t o = off;
    off = (off + bytes + 255) & ~(size_t)255;
    return o;
  }
};

// Queues a read of `cnt` ints of a device array into host storage (fixed-size,
// no heap) on the caller's stream, so it follows the caller's own writes of
// those inputs on that stream; the caller synchronises the stream before
// reading dst.
bool read_ints(const int32_t *src, int cnt, int *dst, int def, cudaStream_t s) {
  for (int q = 0; q < cnt; ++q) dst[q] = def;
  if (!src || cnt == 0) return true;
  return cudaMemcpyAsync(dst, src, (size_t)cnt * 4, cudaMemcpyDeviceToHost, s) == cudaSuccess;
}

thread_local int t_act[CUSNA_MAX_N];  // static storage for validating act

#define SCU(call)                                                                     \
  do {                                                                                \
    cudaError_t e_ = (call);                                                          \
    if (e_ != cudaSuccess) {                                                          \
      char b_[256];                                                                   \
      snprintf(b_, sizeof b_, "%s failed: %s", #call, cudaGetErrorString(e_));       \
      set_last_error(b_);                                                             \
      return CUSNA_ERR_CUDA;                                                          \
    }                                                                                 \
  } while (0)

}  // namespace
}  // namespace cusna

using namespace cusna;

extern "C" CUSNA_API cusna_status cusna_saom_simulate_period_static(
    const cusna_saom_problem *p, cusna_saom_result *r, void *stream) {
  set_last_error("");
  if (!p || !r) { set_last_error("problem or result is NULL"); return CUSNA_ERR_NULL_ARG; }
  if (p->struct_version != CUSNA_ABI_VERSION) {
    set_last_error("struct_version mismatch");
    return CUSNA_ERR_SHAPE;
  }
  const int n = p->n, W = p->W, k = p->k, M = p->M, kb = p->kb, nr = p->nrate;
  if (n < 1 || n > CUSNA_MAX_N || W != (n + 31) / 32 || k < 1 || M < 1 || k > CUSNA_MAXEFF ||
      kb < 0 || kb > CUSNA_MAXBEFF || nr < 0 || nr > CUSNA_MAXRATE) {
    set_last_error("bad shape (n, W, k, M, kb or nrate)");
    return CUSNA_ERR_SHAPE;
  }
  if (!p->x0_out || !p->theta || !p->lam || !p->type_ids || (kb > 0 && !p->bty) ||
      (nr > 0 && (!p->rkind || !p->ralpha || !p->ru))) {
    set_last_error("a required input pointer is NULL");
    return CUSNA_ERR_NULL_ARG;
  }
  if (p->act && (p->nact < 1 || p->nact > n)) { set_last_error("nact out of range"); return CUSNA_ERR_SHAPE; }
  unsigned char *base = nullptr;
  cusna_status st = scratch_address(&base);
  if (st != CUSNA_OK) return st;
  cudaStream_t s = (cudaStream_t)stream;

  // ---- small descriptors, read into fixed host storage --------------------
  int tid[CUSNA_MAXEFF], i0[CUSNA_MAXEFF], i1[CUSNA_MAXEFF], i2[CUSNA_MAXEFF], dyn[CUSNA_MAXEFF];
  if (!read_ints(p->type_ids, k, tid, 0, s) || !read_ints(p->int0, k, i0, -1, s) ||
      !read_ints(p->int1, k, i1, -1, s) || !read_ints(p->int2, k, i2, -1, s) ||
      !read_ints(p->dyn_flags, k, dyn, 0, s) ||
      (p->act && !read_ints(p->act, p->nact, t_act, 0, s)) ||
      cudaStreamSynchronize(s) != cudaSuccess) {
    cudaGetLastError();
    set_last_error("reading effect descriptors from the device failed");
    return CUSNA_ERR_CUDA;
  }
  if (p->act) {
    for (int q = 0; q < p->nact; ++q)
      if (t_act[q] < 0 || t_act[q] >= n) { set_last_error("act entry out of range"); return CUSNA_ERR_SHAPE; }
  }
  // effect plan without tables: counts (the kernel multiplies by theta),
  // per-ministep constants, and the generic per-alter path for the rest
  int kind[CUSNA_MAXEFF], cfn[CUSNA_MAXEFF];
  int fl = 0;
  bool has_dyn = false;
  for (int e = 0; e < k; ++e) {
    const int t = tid[e];
    kind[e] = K_GEN; cfn[e] = 0;
    has_dyn |= dyn[e] != 0;
    switch (t) {
      case 0: kind[e] = K_CNT; cfn[e] = 0; break;
      case 1: kind[e] = K_CNT; cfn[e] = 1; break;
      case 2: kind[e] = K_CNT; cfn[e] = 2; fl |= F_PC_RI_CJ | F_PC_RI_RJ; break;
      case 3: case 23: kind[e] = K_CNT; cfn[e] = 3; fl |= F_PC_RJ_CI; break;
      case 4: kind[e] = K_CNT; cfn[e] = 4; break;
      case 5: kind[e] = K_CNT; cfn[e] = 5; fl |= F_NEED_TP; break;
      case 6: kind[e] = K_CNT; cfn[e] = 6; fl |= F_PC_RI_CJ | F_PC_RICIRJ; break;
      case 8: kind[e] = K_CNT; cfn[e] = 7; break;
      case 10: case 14: case 15: case 16: case 17: case 18:
        kind[e] = K_STEP; fl |= F_HAS_STEP; break;
      case 19: kind[e] = K_STEP; fl |= F_HAS_STEP | F_NEED_RDEG; break;
      case 22: kind[e] = K_ZERO; break;
      case 24: fl |= F_PC_RI_CJ; break;
      case 26: fl |= F_PC_RI_RJ; break;
      case 27: fl |= F_PC_CI_CJ; break;
      case 28: fl |= F_PC_CI_RJ; break;
      case 29: fl |= F_NEED_GW29; break;
      case 30: fl |= F_NEED_GW30; break;
      case 32:
        fl |= F_HAS_INTER;
        if (i0[e] < 0 || i0[e] >= e || i1[e] < 0 || i1[e] >= e || i2[e] >= e) {
          set_last_error("interaction components must be earlier effects");
          return CUSNA_ERR_SHAPE;
        }
        break;
      case 7: case 9: case 11: case 12: case 13: case 20: case 21: case 25: case 31: break;
      default: kind[e] = K_ZERO; break;
    }
  }
  if (kb > 0 || has_dyn) fl |= F_HAS_Z;
  if (r->want_end_nets && r->a_ends) fl |= F_WANT_ENDS;
  if (!r->scores) fl |= F_NO_SCORES;  // no score sums without scores

  // ---- launch shape (as the autotuned entry points choose it) ------------
  int dev = 0, sms = 0, smem_optin = 0;
  SCU(cudaGetDevice(&dev));
  SCU(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  SCU(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  const bool need_tp = (fl & F_NEED_TP) != 0, need_gw = (fl & (F_NEED_GW29 | F_NEED_TP)) != 0;
  const bool need_tq = (fl & F_NEED_GW30) != 0;
  LaunchShape best{};
  double best_score = -1.0;
  for (int G = 1; G <= 16; G *= 2)
    for (int cs = 1; cs >= 0; --cs) {
      LaunchShape sh{};
      sh.G = G;
      sh.cols_in_smem = cs;
      sh.rows_in_smem = true;
      sh.lay = make_layout(n, W, k, kb, nr, G, true, cs, need_tp, need_gw, need_tq);
      if (sh.lay.bytes > (size_t)smem_optin) continue;
      for (int tpc = 1; tpc <= 16; tpc *= 2) {
        const int threads = 32 * G * tpc;
        if (threads > 512 || (G > 1 && tpc > 15) || sh.lay.bytes * tpc > (size_t)smem_optin) continue;
        const int per_sm = period_blocks_per_sm(threads, sh.lay.bytes * tpc);
        if (per_sm < 1) continue;
        const double teams_sm = (double)per_sm * tpc;
        const double busy = (teams_sm < (double)M / sms ? teams_sm : ((double)M / sms > 1 ? (double)M / sms : 1.0)) * G;
        const double score = (busy < 48 ? busy : 48) * 100.0 - G - (cs ? 0.0 : 50.0) - tpc * 0.01;
        if (score > best_score) {
          best_score = score;
          best = sh;
          best.teams_per_cta = tpc;
          const long long want = ((long long)M + tpc - 1) / tpc;
          const long long cap = (long long)sms * per_sm;
          best.ctas = (int)(want < cap ? want : cap);
        }
      }
    }
  if (best_score < 0) { set_last_error("no launch shape fits this n in shared memory"); return CUSNA_ERR_UNSUPPORTED; }

  // ---- scratch layout ----------------------------------------------------
  const size_t bits = (size_t)W * n * 4;
  Bump b;
  const size_t oX = b.take(bits), oXc = b.take(bits), oS = b.take(bits), oSc = b.take(bits),
               oK = b.take(bits), oP = b.take(bits), oKp = b.take(bits), oF = b.take(bits),
               oKc = b.take(bits), oFc = b.take(bits);
  const size_t oV = b.take((size_t)k * n * 8), oWt = b.take((size_t)k * (n + 1) * 8),
               o1 = b.take((size_t)k * 8), o2 = b.take((size_t)k * 8), oVb = b.take((size_t)n * 8),
               oRa = b.take((size_t)(nr + 1) * 8), oRu = b.take((size_t)(nr + 1) * n * 8);
  const size_t oEt = b.take((size_t)k * 4), oDy = b.take((size_t)k * 4), oI0 = b.take((size_t)k * 4),
               oI1 = b.take((size_t)k * 4), oI2 = b.take((size_t)k * 4), oAct = b.take((size_t)n * 4),
               oZ0 = b.take((size_t)n * 4), oBk = b.take((size_t)n * 4), oIn = b.take((size_t)W * 4);
  const size_t oKind = b.take((size_t)k * 4), oCfn = b.take((size_t)k * 4),
               oOffd = b.take((size_t)k * 4), oTab = b.take(8);
  const size_t oProb = b.take(sizeof(DevProblem)), oUnits = b.take(2 * sizeof(long long)),
               oCnt = b.take(sizeof(unsigned long long)), oFlag = b.take(sizeof(int));
  const size_t teams = (size_t)best.ctas * best.teams_per_cta;
  const size_t oCols = best.cols_in_smem ? 0 : b.take(teams * (size_t)W * n * 4);
  if (b.off > kStaticScratchBytes) {
    char buf[200];
    snprintf(buf, sizeof buf,
             "this problem needs %zu bytes of scratch; the no-allocation entry point holds %zu",
             b.off, kStaticScratchBytes);
    set_last_error(buf);
    return CUSNA_ERR_UNSUPPORTED;
  }
  auto U32 = [&](size_t o) { return (uint32_t *)(base + o); };
  auto I32 = [&](size_t o) { return (int *)(base + o); };
  auto F64 = [&](size_t o) { return (double *)(base + o); };

  // ---- prepared inputs ---------------------------------------------------
  SCU(launch_prep_bits(p->x0_out, n, W, U32(oX), U32(oXc), 0, s));
  SCU(launch_prep_bits(p->sim_out ? p->sim_out : p->x0_out, n, W, U32(oS), U32(oSc), 0, s));
  SCU(launch_prep_bits(p->kdist, n, W, U32(oK), nullptr, 1, s));
  SCU(launch_prep_bits(p->perm, n, W, U32(oP), nullptr, 1, s));
  SCU(launch_prep_bits(p->keep_out, n, W, U32(oKp), U32(oKc), 1, s));
  SCU(launch_prep_bits(p->force_out, n, W, U32(oF), U32(oFc), 2, s));
  if (fl & (F_NEED_GW29 | F_NEED_GW30)) {
    // gwdsp weight indices stay inside the table only without self-ties
    SCU(cudaMemsetAsync(base + oFlag, 0, sizeof(int), s));
    self_tie_kernel<<<(n + 255) / 256, 256, 0, s>>>(U32(oS), n, I32(oFlag));
    self_tie_kernel<<<(n + 255) / 256, 256, 0, s>>>(U32(oX), n, I32(oFlag));
    int flag = 0;
    SCU(cudaMemcpyAsync(&flag, base + oFlag, sizeof(int), cudaMemcpyDeviceToHost, s));
    SCU(cudaStreamSynchronize(s));
    if (flag) { set_last_error("gwdsp effects need a start network without self-ties"); return CUSNA_ERR_SHAPE; }
  }
  SCU(launch_prep_desc(p->vmat64, p->vmat64 ? nullptr : p->vmat, (size_t)k * n, F64(oV), s));
  SCU(launch_prep_desc(p->wtab64, p->wtab64 ? nullptr : p->wtab, (size_t)k * (n + 1), F64(oWt), s));
  SCU(launch_prep_desc(p->p1_64, p->p1_64 ? nullptr : p->p1, (size_t)k, F64(o1), s));
  SCU(launch_prep_desc(p->p2_64, p->p2_64 ? nullptr : p->p2, (size_t)k, F64(o2), s));
  SCU(launch_prep_desc(p->vb64, p->vb64 ? nullptr : p->vb, (size_t)n, F64(oVb), s));
  if (nr) {
    SCU(launch_prep_desc(nullptr, p->ralpha, (size_t)nr, F64(oRa), s));
    SCU(launch_prep_desc(nullptr, p->ru, (size_t)nr * n, F64(oRu), s));
  }
  auto icopy = [&](const int32_t *src, size_t o, size_t cnt, int def) -> cudaError_t {
    if (src) return cudaMemcpyAsync(I32(o), src, cnt * 4, cudaMemcpyDeviceToDevice, s);
    return launch_fill_int(I32(o), cnt, 0, def, s);
  };
  SCU(icopy(p->etypes, oEt, k, 0));
  SCU(icopy(p->dyn_flags, oDy, k, 0));
  SCU(icopy(p->int0, oI0, k, -1));
  SCU(icopy(p->int1, oI1, k, -1));
  SCU(icopy(p->int2, oI2, k, -1));
  SCU(icopy(p->z0, oZ0, n, 0));
  SCU(icopy(p->bkdist, oBk, n, 1));
  if (p->act) SCU(cudaMemcpyAsync(I32(oAct), p->act, (size_t)p->nact * 4, cudaMemcpyDeviceToDevice, s));
  else SCU(launch_fill_int(I32(oAct), n, 1, 0, s));
  if (p->has_comp && p->inactw)
    SCU(cudaMemcpyAsync(U32(oIn), p->inactw, (size_t)W * 4, cudaMemcpyDeviceToDevice, s));
  else
    SCU(cudaMemsetAsync(U32(oIn), 0, (size_t)W * 4, s));
  int zeros[CUSNA_MAXEFF] = {0};
  SCU(cudaMemcpyAsync(I32(oKind), kind, (size_t)k * 4, cudaMemcpyHostToDevice, s));
  SCU(cudaMemcpyAsync(I32(oCfn), cfn, (size_t)k * 4, cudaMemcpyHostToDevice, s));
  SCU(cudaMemcpyAsync(I32(oOffd), zeros, (size_t)k * 4, cudaMemcpyHostToDevice, s));
  SCU(cudaMemsetAsync(base + oTab, 0, 8, s));

  DevProblem D;
  std::memset(&D, 0, sizeof D);
  D.n = n; D.W = W; D.k = k; D.kb = kb; D.nrate = nr; D.M = M;
  D.chain_offset = 0;
  D.cond = p->conditional; D.target_dist = p->target_dist; D.symflag = p->symflag;
  D.maxdeg = p->maxdegree; D.has_comp = p->has_comp && p->inactw; D.nact = p->act ? p->nact : n;
  D.k0 = (uint32_t)(p->seed & 0xFFFFFFFFu);
  D.k1 = (uint32_t)(p->seed >> 32);
  D.flags = fl;
  D.zmin = p->zmin; D.zmax = p->zmax; D.zlo = 0; D.zR = 1;
  D.zbar = (double)p->zbar; D.brange = (double)p->brange; D.bsimmean = (double)p->bsimmean;
  D.type_ids = p->type_ids; D.etypes = I32(oEt); D.dyn = I32(oDy);
  D.int0 = I32(oI0); D.int1 = I32(oI1); D.int2 = I32(oI2);
  D.p1 = F64(o1); D.p2 = F64(o2); D.vmat = F64(oV); D.wtab = F64(oWt); D.vmiss = p->vmiss;
  D.vb = F64(oVb); D.od0 = p->od0; D.id0 = p->id0; D.bty = p->bty; D.rkind = p->rkind;
  D.ralpha = F64(oRa); D.ru = F64(oRu); D.act = I32(oAct); D.inact = U32(oIn);
  D.z0 = I32(oZ0); D.bkdist = I32(oBk);
  D.x0T = U32(oX); D.x0cT = U32(oXc); D.simT = U32(oS); D.simcT = U32(oSc);
  D.kdistT = U32(oK); D.permT = U32(oP); D.keepT = U32(oKp); D.forceT = U32(oF);
  D.keepcT = U32(oKc); D.forcecT = U32(oFc);
  D.lam = p->lam; D.theta = p->theta; D.lamb = p->lamb; D.thetab = kb ? p->thetab : nullptr;
  D.prow = 1;
  D.ekind = I32(oKind); D.ecfn = I32(oCfn); D.eoffd = I32(oOffd); D.eofft = I32(oOffd);
  D.tab = F64(oTab);
  D.tab2 = nullptr;  // no lookup tables in this plan
  D.stats = r->stats; D.ntim = r->ntim; D.scores = r->scores; D.dist = r->dist;
  D.dist_stat = r->dist_stat; D.steps = r->steps;
  if (kb) { D.bdist = r->bdist; D.bscores = r->bscores; D.z_end = r->z_end; }
  if (nr) { D.rscores = r->rscores; D.actor_dist = r->actor_dist; }
  D.a_ends = (r->want_end_nets && r->a_ends) ? r->a_ends : nullptr;
  const long long units[2] = {0, (long long)M};
  SCU(cudaMemcpyAsync(base + oProb, &D, sizeof D, cudaMemcpyHostToDevice, s));
  SCU(cudaMemcpyAsync(base + oUnits, units, sizeof units, cudaMemcpyHostToDevice, s));
  SCU(cudaMemsetAsync(base + oCnt, 0, sizeof(unsigned long long), s));  // work counter starts at 0
  SCU(launch_period(best, (const DevProblem *)(base + oProb), (const long long *)(base + oUnits), 1,
                    (long long)M, (unsigned long long *)(base + oCnt),
                    best.cols_in_smem ? nullptr : U32(oCols), nullptr, (size_t)W * n, s));
  SCU(cudaStreamSynchronize(s));
  return CUSNA_OK;
}
