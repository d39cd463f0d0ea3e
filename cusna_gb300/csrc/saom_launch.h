// saom_launch.h -- launch wrappers shared by the kernels (saom_sim.cu) and the
// host code (saom_api.cu).
#pragma once
#include <nvtx3/nvToolsExt.h>
#include <cuda_runtime.h>
#include <cstdint>
#include "saom_common.cuh"
#include "saom_kernel.cuh"
#include "libcusna.h"

namespace cusna {

struct StatDesc;

// Launch shape of the period kernel, chosen by the autotuner (saom_api.cu).
struct LaunchShape {
  int G;              // warps per chain
  int teams_per_cta;  // chains per CTA
  int ctas;           // grid size (persistent: ctas * teams_per_cta resident teams)
  bool cols_in_smem;  // in-rows in shared memory (else global scratch)
  bool rows_in_smem;  // out-rows in shared memory (else global scratch)
  SliceLayout lay;
};

cudaError_t launch_period(const LaunchShape &sh, const DevProblem *probs, const long long *unit_start,
                          int nprob, long long total, unsigned long long *counter,
                          uint32_t *cols_scratch, uint32_t *rows_scratch, size_t cols_words,
                          cudaStream_t st, bool valid = false);
// valid: the validation build of the period kernel (trace, supplied words;
// CTAs of at most 256 threads)
int period_blocks_per_sm(int threads, size_t dyn_smem, bool valid = false);

static_assert(kMaxNet == CUSNA_MAXNET, "network capacity of the kernels and the ABI");
static_assert(kMaxEff == CUSNA_MAXEFF, "effect capacity of the kernels and the ABI");
int multi_blocks_per_sm(int threads, size_t dyn_smem);
cudaError_t launch_multi(const LaunchShape &sh, const DevProblem *nets, const MultiDev &md, int M,
                         unsigned long long *counter, uint32_t *cols_scratch,
                         uint32_t *rows_scratch, size_t cols_words, cudaStream_t st);
// Cross-network statistic of M dense own networks a against the dense source
// predictor wp; ar (M*n*W words, type 37) and wr (n*W words, type 36) are
// scratch for packed rows.
cudaError_t launch_cross_stats(const uint8_t *a, const uint8_t *wp, int n, int M, int t,
                               double parm, uint32_t *ar, uint32_t *wr, double *out,
                               cudaStream_t st);
// Rows of dense uint8 matrices (rows x n) packed into W words per row.
cudaError_t launch_pack_rows(const uint8_t *a, long long rows, int n, int W, uint32_t *out,
                             cudaStream_t st);
// Typed (creation / endowment) statistic of M dense end networks.
cudaError_t launch_typed_stats(const uint8_t *a, int n, int M, int etype, const double *F,
                               const uint8_t *x0, const uint8_t *keep, const uint8_t *force,
                               const uint8_t *keepS, const uint8_t *forceS,
                               const uint8_t *miss_m, const uint8_t *miss_m1, double *out,
                               cudaStream_t st);
// sienaGOF distributions of M dense end networks (kind 0 in-degree, 1
// out-degree, 2 geodesic with K = min(largest level, n - 1)); rows (M*n*W
// words) and added (M*(K+1)) are scratch of the geodesic kind.
size_t gof_scratch_words(int n, int M, int kind, int K);
cudaError_t launch_gof(const uint8_t *a, int n, int M, int kind, const int *levls, int nlev,
                       int K, uint32_t *rows, unsigned long long *added, double *out,
                       int smem_optin, cudaStream_t st);

// One theta-premultiplied term table of a plan's problem q, effect e (pool
// offsets of the table and, for lookup tables, of its values).
struct PlanTable {
  int q, e, kind, offt, offd, size;
};
// Before each launch of a plan: advance the epoch (Philox keys) and rebuild the
// term tables from the current parameters.
cudaError_t launch_plan_prologue(DevProblem *probs, const unsigned long long *base_seed, int count,
                                 unsigned long long *epoch, const PlanTable *tabs, int n_tabs,
                                 cudaStream_t st);
long long kernel_launches();  // kernels launched so far by the calling thread
void note_launch();           // counts a launch made outside the wrappers here
// Raises a kernel's dynamic shared memory limit on the current device to at
// least `bytes`; never lowers it (see saom_sim.cu).
cudaError_t raise_dyn_smem(const void *func, size_t bytes);
void set_last_error(const char *msg);  // text of cusna_last_error() for this thread

// A named range on the calling thread's timeline for profilers (NVTX, header
// only: without an attached tool each push and pop is a call that returns).
struct NvtxRange {
  explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange &) = delete;
  NvtxRange &operator=(const NvtxRange &) = delete;
};
cudaError_t launch_netstats(const uint8_t *a, int M, const StatDesc &D, double *out, int sms,
                            cudaStream_t st);
cudaError_t launch_behstats(const int *z, int n, int M, int kb, const int *bty, const uint8_t *xnet,
                            const int *bkdist, double zbar, double brange, double bsimmean,
                            double *out, int sms, cudaStream_t st);
cudaError_t launch_prep_bits(const uint32_t *src, int n, int W, uint32_t *dstT, uint32_t *dstcT,
                             int def_mode, cudaStream_t st);
cudaError_t launch_prep_desc(const double *d64, const float *d32, size_t cnt, double *dst,
                             cudaStream_t st);
cudaError_t launch_fill_int(int *dst, size_t cnt, int mode, int value, cudaStream_t st);

}  // namespace cusna
