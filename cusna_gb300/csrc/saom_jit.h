// saom_jit.h -- the period kernel specialised to one effect plan, compiled at
// run time with NVRTC (saom_jit.cu).
//
// The float32 pass over the alters evaluates every effect of the model for
// every alter. The library's kernel reads each effect's kind from shared memory
// and dispatches per alter; the specialised kernel has the effect plan written
// out as straight-line code (the same float32 operations in the same order, so
// every output is bit-identical to the library kernel's). A plan is compiled in
// a background thread once it has been used a few times (CUSNA_JIT_AFTER,
// default 3); until then, and whenever NVRTC is unavailable, the library kernel
// runs. CUSNA_JIT=0 disables the specialisation, CUSNA_JIT=sync compiles on
// first use.
#pragma once
#include <cuda_runtime.h>
#include <string>
#include <vector>
#include "saom_launch.h"

namespace cusna {

// The effect plan the specialised code is generated from.
struct JitPlan {
  int pc_flags = 0;  // F_PC_* popcount needs
  int n = 0;         // actors when every problem of the launch has the same
                     // number (compiled in with W: the popcount loops unroll
                     // and the strides are constants), else 0
  std::vector<int> kind, cfn, tid, ety, i0, i1, i2;
};

// Source text of the specialised effect evaluation (the key of the compiled
// kernel): of the period kernel for one plan, or of the multi-network kernel
// for the networks' plans (its text starts with kJitMultiTag).
std::string jit_spec_source(const JitPlan &J);
std::string jit_multi_spec_source(const std::vector<JitPlan> &nets);
constexpr const char *kJitMultiTag = "// cusna specialisation: multi-network kernel";

// 0: off, 1: background compilation after CUSNA_JIT_AFTER uses, 2: compile on
// first use.
int jit_mode();
// Overrides CUSNA_JIT for the process (mode as jit_mode; -1 restores it).
void jit_set_mode(int mode);

// Handles of a compiled and loaded specialisation (CUfunction of the 256- and
// 512-thread instantiations).
struct JitKernel {
  void *f256 = nullptr, *f512 = nullptr;
};

// Counts a use of spec and, once it is compiled, loads it in the calling
// thread's context. Returns true with *out filled when the specialised kernel
// can run. Must not be called while a stream is being captured.
// now: compile (or wait for the background compiler) before returning.
bool jit_get(const std::string &spec, JitKernel *out, bool now = false);
// Resident CTAs per SM of the specialised kernel (0 on failure).
int jit_blocks_per_sm(const JitKernel &K, int threads, size_t dyn_smem);
cudaError_t launch_period_jit(const JitKernel &K, const LaunchShape &sh, const DevProblem *probs,
                              const long long *unit_start, int nprob, long long total,
                              unsigned long long *counter, uint32_t *cols_scratch,
                              uint32_t *rows_scratch, size_t cols_words, cudaStream_t st);
cudaError_t launch_multi_jit(const JitKernel &K, const LaunchShape &sh, const DevProblem *nets,
                             const MultiDev &md, int M, unsigned long long *counter,
                             uint32_t *cols_scratch, uint32_t *rows_scratch, size_t cols_words,
                             cudaStream_t st);
// NVRTC compile of spec without loading it (no device needed): 0 on success,
// else the NVRTC log in *log.
int jit_compile_only(const std::string &spec, std::string *log, double *seconds);
// Waits up to `seconds` until no compilation is queued or running; returns the
// number of specialisations compiled so far.
int jit_wait(double seconds);

}  // namespace cusna
