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
  F_LSE64 = 1 << 16,       // score log-sum-exp in float64 at every ministep (validation)
  F_NO_SCORES = 1 << 17,   // no scores requested: the score sums are not formed
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
  // tab's lookup values as double-float pairs: .x the float32 rounding (the
  // float32 pass), .y the float32 rounding of the remainder (x + y is tab's
  // value to ~2^-48, for the score sums); one 8-byte load per lookup
  const float2 *tab2;

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

  // validation mode (period_kernel<MAXT, true> only): per-ministep trace
  // records (step, actor, choice, distance change), trace_cap per chain, and
  // caller-supplied words replacing the Philox outputs of the first
  // ustream_steps ministeps of each chain (4 + n words per ministep)
  int *trace;
  int trace_cap;
  const uint32_t *ustream;
  int ustream_steps;
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

// ---- double-float arithmetic ------------------------------------------------
// An unevaluated pair (h, l) of float32 values stands for h + l, with |l| at
// most about 2^-24 |h|: 48 significant bits on the float32 pipes, which on
// this GPU run 64 times as many operations per cycle as the float64 pipe.
// The error-free transformations are Knuth's TwoSum and Dekker's product
// through a fused multiply-add (T. J. Dekker, "A floating-point technique for
// extending the available precision", Numer. Math. 18, 1971). Every sum uses
// the _rn intrinsics, so no compiler contraction or reassociation can change
// the result.

// s + e = a + b exactly, s = fl(a + b).
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// (ah, al) += (bh, bl), keeping the pair unnormalised: the rounding error of
// the high sum joins the low parts, whose own rounding is ~2^-24 of them.
__device__ __forceinline__ void ff_add(float &ah, float &al, float bh, float bl) {
  float s, e;
  two_sum(ah, bh, s, e);
  ah = s;
  al = __fadd_rn(__fadd_rn(al, bl), e);
}

// The same on two independent pairs at once with the packed float32x2
// instructions of this architecture (__fadd2_rn, __ffma2_rn: each component
// rounded as __fadd_rn / __fmaf_rn), which issue one instruction for two
// operations. a - b is fma(b, -1, a), one rounding of the exact difference.
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {
  return __ffma2_rn(b, make_float2(-1.f, -1.f), a);
}
__device__ __forceinline__ void ff_add2(float2 &ah, float2 &al, float2 bh, float2 bl) {
  const float2 s = __fadd2_rn(ah, bh);
  const float2 bb = sub2(s, ah);
  const float2 e = __fadd2_rn(sub2(ah, sub2(s, bb)), sub2(bh, bb));
  ah = s;
  al = __fadd2_rn(__fadd2_rn(al, bl), e);
}

// Largest |x| the double-float exponential accepts; the score sums fall back
// to float64 when a predictor leaves this range (or is not finite).
constexpr float kFFExpMax = 60.f;

// ln(2)/64 split as C1 + C2 + C3: C1 has 11 significant bits, so N*C1 is exact
// for |N| < 2^13 (|x| <= 60 gives |N| <= 5540); C2 and C3 are the next two
// float32 roundings of the remainder (the split leaves 1.8e-22).
constexpr float kLn2o64C1 = 0x1.63p-7f;
constexpr float kLn2o64C2 = -0x1.bd0106p-19f;
constexpr float kLn2o64C3 = 0x1.cf79acp-46f;
constexpr float k64oLn2 = 0x1.715476p+6f;   // 64/ln(2), only to choose N

// The table 2^(j/64), j = 0..63, as double-float pairs (h, l): computed from
// the float64 exp2, whose error is far below the pair's 2^-48.
__device__ __forceinline__ void fill_exp_table(float2 *tab, int tl, int L) {
  for (int j = tl; j < 64; j += L) {
    const double v = exp2((double)j * 0.015625);
    const float h = (float)v;
    tab[j] = make_float2(h, (float)__dsub_rn(v, (double)h));
  }
}

// exp(xh + xl) as a double-float pair (wh, wl) for |xh| <= kFFExpMax, relative
// error below about 2e-14. Tang's table-driven method (P. T. P. Tang, "Table-
// driven implementation of the exponential function in IEEE floating-point
// arithmetic", ACM TOMS 15(2), 1989) in double-float arithmetic:
//   x = N ln2/64 + r, |r| <= ln2/128 (Cody-Waite reduction with the three-part
//   constant above, the first product exact, the second through Dekker's
//   product, so r is known to ~1e-18);
//   exp(r) - 1 = r + r^2/2 + r^3/6 + r^4/24 + r^5/120 (the omitted terms are
//   below 4e-17): the first two terms in double-float, the rest in float32
//   (their sum is below 2.7e-8, so its rounding is below 2e-15);
//   exp(x) = 2^(N>>6) * 2^((N&63)/64) * exp(r), the table entry multiplied in
//   double-float and the power of two applied exactly to both halves.
__device__ __forceinline__ void exp_ff(float xh, float xl, const float2 *tab, float &wh,
                                       float &wl) {
  const float Nf = rintf(__fmul_rn(xh, k64oLn2));
  const int N = (int)Nf;
  const float t1 = fmaf(-Nf, kLn2o64C1, xh);  // exact
  const float p = __fmul_rn(Nf, kLn2o64C2);
  const float pe = fmaf(Nf, kLn2o64C2, -p);  // p + pe = N C2 exactly
  float rh, e;
  two_sum(t1, -p, rh, e);
  const float rl = __fadd_rn(__fsub_rn(__fsub_rn(e, pe), __fmul_rn(Nf, kLn2o64C3)), xl);
  // r^2 = sqh + sql (dropping rl^2 < 1e-19)
  const float sqh = __fmul_rn(rh, rh);
  const float sql = fmaf(__fmul_rn(2.f, rh), rl, fmaf(rh, rh, -sqh));
  // r^3/6 + r^4/24 + r^5/120, plus the r^2 rl / 2 part of the cubic term
  const float q = fmaf(__fmul_rn(sqh, rh),
                       fmaf(rh, fmaf(rh, 8.3333333333e-3f, 4.1666666667e-2f), 1.6666666667e-1f),
                       __fmul_rn(__fmul_rn(0.5f, sqh), rl));
  float sh, e1;
  two_sum(rh, __fmul_rn(0.5f, sqh), sh, e1);
  const float sl = __fadd_rn(__fadd_rn(__fadd_rn(rl, __fmul_rn(0.5f, sql)), q), e1);
  // T (1 + sh + sl), T = 2^((N & 63)/64) in [1, 2) as (T.x, T.y)
  const float2 T = tab[N & 63];
  const float ph = __fmul_rn(T.x, sh);
  const float pl = fmaf(T.x, sh, -ph);
  const float h = __fadd_rn(T.x, ph);  // |T.x| >= 1 > |ph|: Fast2Sum
  float l = __fsub_rn(ph, __fsub_rn(h, T.x));
  l = __fadd_rn(l, __fadd_rn(pl, fmaf(T.x, sl, fmaf(T.y, sh, T.y))));
  // 2^(N >> 6), N >> 6 in [-87, 86]: a normal float32
  const float s = __int_as_float(((N >> 6) + 127) << 23);
  wh = __fmul_rn(h, s);
  wl = __fmul_rn(l, s);
}

}  // namespace cusna
