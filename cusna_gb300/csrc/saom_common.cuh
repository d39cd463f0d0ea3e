// saom_common.cuh -- device-side problem descriptor and small helpers of the
// GB300 SAOM period simulator.
#pragma once
#ifdef __CUDACC_RTC__
// compiled at run time by NVRTC (saom_jit.cu): device code only, no host headers
typedef unsigned int uint32_t;
typedef int int32_t;
typedef unsigned long long uint64_t;
typedef long long int64_t;
typedef unsigned char uint8_t;
typedef unsigned short uint16_t;
typedef unsigned long long uintptr_t;
#define INFINITY __int_as_float(0x7f800000)
#else
#include <cstdint>
#include <cuda_runtime.h>
#endif

namespace cusna {

// Runaway-chain cap of the CPU engine (src/libcusna_saom_cpu.cpp:115).
constexpr long long kMaxSteps = 4000000;
constexpr int kMaxEff = 24;  // network effects per model (CUSNA_MAXEFF)
constexpr unsigned kFull = 0xFFFFFFFFu;

// Problem flags (DevProblem::flags).
enum : int {
  F_NEED_TP = 1 << 0,      // transTies: two-path counts tp[h] = |out_i & in_h|
  F_NEED_RDEG = 1 << 1,    // reciAct: reciprocated degree of i
  F_NEED_GW29 = 1 << 2,    // gwdspFF: per-h weight differences over tp
  F_NEED_GW30 = 1 << 3,    // gwdspFB: per-h weight differences over |out_i & out_h|
  F_WANT_ENDS = 1 << 4,    // dense end networks requested
  F_HAS_INTER = 1 << 5,    // interaction effects present
  F_PC_RI_CJ = 1 << 6,     // popcount needs of the change statistics
  F_PC_RI_RJ = 1 << 7,
  F_PC_RJ_CI = 1 << 8,
  F_PC_CI_CJ = 1 << 9,
  F_PC_CI_RJ = 1 << 10,
  F_PC_RICIRJ = 1 << 11,
  F_COLS_GLOBAL = 1 << 12, // the chain's in-rows live in global scratch
  F_THETA_TAB = 1 << 13,   // term tables hold theta_e * d for every chain
  F_HAS_STEP = 1 << 14,    // some effect is constant within a ministep
  F_HAS_Z = 1 << 15,       // behaviour values are read (behaviour or dynamic covariates)
};

// How the change statistic d_e of toggling i -> j is formed (DevProblem::ekind).
// Every kind yields d_e = delta * magnitude, the reference's value, and with
// F_THETA_TAB the term theta_e * d_e comes from a table of theta_e * magnitude
// (theta_e * (-m) = -(theta_e * m) exactly, so the table needs no sign).
enum : int {
  K_GEN = 0,   // computed in full per alter (gwdsp, interactions, large dyadic)
  K_CNT = 1,   // integer magnitude c (ecfn selects which count); term table T[c]
  K_LOOK = 2,  // magnitude D[idx], term T[idx]; idx from ecfn (sqrt, gw weight,
               // alter covariate, dyadic covariate tables)
  K_STEP = 3,  // magnitude depends only on (i, a_ij, a_ji): formed per ministep
  K_ZERO = 4,  // the dyadic covariate X, which the CPU engine zero-fills
  K_CROSS = 5, // multi-network cross effect (ecfn = type 33..37) reading network eoffd
};

// Multi-network problem: what the multi-network kernel needs beyond the
// per-network problems (one DevProblem per network, holding its effects).
constexpr int kMaxNet = 4;  // CUSNA_MAXNET
struct MultiDev {
  int D, n, W, nact, k;
  const int *act;                 // nact active actors first
  const float *lam;               // M*D rates
  uint32_t k0, k1;                // Philox key
  int goff[kMaxNet + 1];          // network d's effects: gidx[goff[d] .. goff[d+1])
  const int *gidx;                // their indices in the caller's effect order
  float *rscores, *scores;        // device outputs (any may be null)
  double *ntim;
  int *steps;
  uint8_t *a_ends;
};

// Canonical device form of one cusna_saom_problem. Every network is stored
// word-major: element (w, j) of an n-actor bit matrix is word w of actor j's
// row, at index w*n + j. Word w of row i, bit b, is the tie i -> 32*w + b.
struct DevProblem {
  int n, W, k, kb, nrate, M;
  uint32_t chain_offset;
  int cond, target_dist, symflag, maxdeg, has_comp, nact;
  uint32_t k0, k1;
  int flags;
  int zmin, zmax;
  int zlo, zR;  // range of reachable behaviour values (lookup tables)
  double zbar, brange, bsimmean;

  // effect descriptors
  const int *type_ids, *etypes, *dyn, *int0, *int1, *int2;  // k
  const double *p1, *p2;                                    // k
  const double *vmat;                                       // k*n
  const double *wtab;                                       // k*(n+1)
  const uint8_t *vmiss;                                     // k*n or null
  const double *vb;                                         // n (statistics)
  const int *od0, *id0;                                     // n or null
  const int *bty;                                           // kb
  const int *rkind;                                         // nrate
  const double *ralpha, *ru;                                // nrate, nrate*n
  const int *act;                                           // n
  const uint32_t *inact;                                    // W bits
  const int *z0, *bkdist;                                   // n

  // networks, word-major W*n
  const uint32_t *x0T, *x0cT, *simT, *simcT, *kdistT, *permT;
  const uint32_t *keepT, *forceT, *keepcT, *forcecT;       // statistic masks

  // per-chain parameters: chain c reads row c * prow (prow 1: one row per
  // chain, as the ABI lays them out; 0: one row shared by every chain)
  const float *lam, *theta, *lamb, *thetab;
  int prow;

  // effect plan (k each) and its table pool
  const int *ekind, *ecfn, *eoffd, *eofft;
  const double *tab;
  const float *tab32;  // float32 copy of tab's lookup values (the float32 pass)

  // outputs (chain-major), any may be null
  double *stats, *ntim;
  float *scores;
  int *dist, *dist_stat, *steps;
  int *bdist;
  float *bscores;
  int *z_end;
  float *rscores;
  int *actor_dist;
  uint8_t *a_ends;
};

// ---- Philox4x32-10 (the generator of src/libcusna_saom_cpu.cpp:32-45) ----
__host__ __device__ __forceinline__ void philox10(uint32_t c0, uint32_t c1, uint32_t c2,
                                                  uint32_t c3, uint32_t k0, uint32_t k1,
                                                  uint32_t out[4]) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
#ifdef __CUDA_ARCH__
    uint32_t hi0 = __umulhi(0xD2511F53u, c0), hi1 = __umulhi(0xCD9E8D57u, c2);
#else
    uint32_t hi0 = (uint32_t)(((uint64_t)0xD2511F53u * c0) >> 32);
    uint32_t hi1 = (uint32_t)(((uint64_t)0xCD9E8D57u * c2) >> 32);
#endif
    uint32_t lo0 = 0xD2511F53u * c0, lo1 = 0xCD9E8D57u * c2;
    uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

// u = (x + 0.5) 2^-32, computed exactly in float64.
__device__ __forceinline__ double unif01(uint32_t x) {
  return __dmul_rn(__dadd_rn((double)x, 0.5), 2.3283064365386962890625e-10);
}

// Monotone int64 key of a double: a < b  <=>  dkey(a) < dkey(b) (no NaNs).
// Lets max/argmax over doubles run on the integer pipes.
__device__ __forceinline__ long long dkey(double x) {
  long long b = __double_as_longlong(x);
  return b ^ ((b >> 63) & 0x7FFFFFFFFFFFFFFFLL);
}
__device__ __forceinline__ double dunkey(long long k) {
  long long b = k ^ ((k >> 63) & 0x7FFFFFFFFFFFFFFFLL);
  return __longlong_as_double(b);
}

// float32 estimate of log(-log(u)), u = (x + 0.5) 2^-32, used to shortlist the
// Gumbel-max candidates. Error bound (from the documented <= 1 ulp error of
// logf/log1pf and the 2^-24 rounding of the inputs):
//   L = -log(u) is estimated with relative error < 5e-7 (for u >= 1/2 through
//   log1p of v = 1 - u, which is formed exactly from ~x), and log(L) lies in
//   [-22.9, 3.2], so |estimate - log(-log u)| < 5e-7 + 23 * 1.2e-7 < 4e-6.
__device__ __forceinline__ float loglog_est(uint32_t x) {
  float L;
  if (x < 0x80000000u) {
    float uf = ((float)x + 0.5f) * 2.3283064365386962890625e-10f;
    L = -logf(uf);
  } else {
    float vf = ((float)(0xFFFFFFFFu - x) + 0.5f) * 2.3283064365386962890625e-10f;
    L = -log1pf(-vf);
  }
  return logf(L);
}


}  // namespace cusna
