/* ==========================================================================
 * libcusna.h -- C ABI of the GB300 (sm_103a) SAOM period simulator.
 *
 * This header is the drop-in boundary of cusna's period simulator. The first
 * part declares the same POD structs (field for field, byte-identical layout),
 * status codes, capacity limits and entry points as the reference header
 * src/libcusna.h of cran/cusna 0.1.1. A caller written against that header (the
 * cpp11 glue src/cusna_saom_glue.cpp:57-189) compiles and links against
 * libcusna_gb300.so unchanged. The second part (marked EXTENSION) adds new
 * entry points. They have no counterpart in the reference, so nothing existing
 * has to change for them.
 *
 * Conventions (src/libcusna.h:28-35):
 *   - extern "C", fixed-width integer types, caller-allocated buffers, and NULL
 *     skips an optional output;
 *   - every struct starts with struct_version == CUSNA_ABI_VERSION;
 *   - matrices are row-major. A "packed bit row" holds W = ceil(n/32) uint32
 *     words per actor. Bit (j & 31) of word (j >> 5) is the tie to actor j.
 *
 * Every entry point is synchronous: its outputs are final when it returns.
 * The library keeps no caller pointer after returning.
 * ========================================================================== */
#ifndef LIBCUSNA_H
#define LIBCUSNA_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#  ifdef LIBCUSNA_BUILD
#    define CUSNA_API __declspec(dllexport)
#  else
#    define CUSNA_API __declspec(dllimport)
#  endif
#else
#  define CUSNA_API __attribute__((visibility("default")))
#endif

/* Capacity limits (src/libcusna.h:61-65). */
#define CUSNA_MAXEFF  24  /* network effects per model            */
#define CUSNA_MAXBEFF 6   /* behaviour effects per model          */
#define CUSNA_MAXRATE 4   /* non-basic rate effects               */
#define CUSNA_MAXNET  4   /* co-evolving networks (multi-net ABI) */
#define CUSNA_MAX_N   8192

#define CUSNA_ABI_VERSION 1  /* src/libcusna.h:69 */

/* Status codes (src/libcusna.h:72-80). */
typedef enum cusna_status {
    CUSNA_OK              = 0,
    CUSNA_ERR_NULL_ARG    = 1,  /* a required pointer is NULL                  */
    CUSNA_ERR_SHAPE       = 2,  /* n/W/k/M out of range or inconsistent        */
    CUSNA_ERR_NO_CUDA     = 3,  /* no usable CUDA device                       */
    CUSNA_ERR_CUDA        = 4,  /* a CUDA call failed; see cusna_last_error()  */
    CUSNA_ERR_UNSUPPORTED = 5,  /* option this build does not implement        */
    CUSNA_ERR_INTERNAL    = 6   /* e.g. a chain hit the step cap               */
} cusna_status;

/* --------------------------------------------------------------------------
 * One SAOM period, M chains (src/libcusna.h:90-180). n actors, W words per
 * actor, k network effects, M chains.
 * -------------------------------------------------------------------------- */
typedef struct cusna_saom_problem {
    int32_t struct_version;   /* CUSNA_ABI_VERSION                            */

    int32_t n;                /* actors, 1..CUSNA_MAX_N                       */
    int32_t W;                /* (n + 31) / 32                                */
    int32_t k;                /* network effects, 1..CUSNA_MAXEFF             */
    int32_t M;                /* chains                                       */
    int32_t threads;          /* ignored here: launch shape is autotuned      */

    const uint32_t *x0_out;   /* n*W out-ties of the period's start network   */
    const uint32_t *x0_in;    /* n*W in-ties (transposed rows); not read      */
    const uint32_t *sim_out;  /* [opt] simulation start rows (else x0_out)    */
    const uint32_t *sim_in;   /* [opt] not read                               */

    const float *lam;         /* M basic rates (chain c reads lam[c])         */
    const float *theta;       /* M*k evaluation parameters (row c = chain c)  */

    const int32_t *type_ids;  /* k effect type ids 0..32                      */
    const int32_t *etypes;    /* [opt] k: 0 eval, 1 creation, 2 endowment     */
    const float   *wtab;      /* [opt] k*(n+1) gwesp/gwdsp weights            */
    const float   *p1;        /* [opt] k effect parameter 1                   */
    const float   *p2;        /* [opt] k effect parameter 2                   */
    const float   *vmat;      /* [opt] k*n covariate values                   */
    const uint8_t *vmiss;     /* [opt] k*n covariate-missing flags (stats)    */
    const int32_t *dyc_idx;   /* [opt] k dyadic covariate index or -1         */
    const float   *dyc;       /* [opt] not read (the CPU engine zero-fills)   */
    const int32_t *int0;      /* [opt] k interaction component 0 or -1        */
    const int32_t *int1;      /* [opt] k interaction component 1 or -1        */
    const int32_t *int2;      /* [opt] k interaction component 2 or -1        */
    const int32_t *dyn_flags; /* [opt] k: covariate is the behaviour (0/1)    */

    const uint32_t *kdist;    /* [opt] n*W dyads counted in the distance      */
    const uint32_t *keep_out; /* [opt] n*W statistic net = (A & keep) | force */
    const uint32_t *keep_in;  /* [opt] not read                               */
    const uint32_t *force_out;/* [opt] n*W                                    */
    const uint32_t *force_in; /* [opt] not read                               */
    const uint32_t *perm;     /* [opt] n*W toggleable dyads                   */

    const int32_t *od0;       /* [opt] n start out-degrees (degree stats)     */
    const int32_t *id0;       /* [opt] n start in-degrees                     */

    int32_t maxdegree;        /* > 0 forbids new ties at the bound            */
    int32_t need_mask;        /* not read                                     */
    int32_t conditional;      /* 1: stop at target_dist (internal rate)       */
    int32_t target_dist;      /* conditional stopping distance                */
    int32_t symflag;          /* symmetric network: paired toggles            */
    uint64_t seed;            /* Philox key: low word k0, high word k1        */

    int32_t has_comp;         /* restore inactive actors at the period end    */
    int32_t nact;             /* active actors (read when act != NULL)        */
    const int32_t  *act;      /* [opt] n: active actor ids first              */
    const uint32_t *inactw;   /* [opt] W: inactive-actor bitmask              */

    int32_t kb;               /* behaviour effects 0..CUSNA_MAXBEFF           */
    const float   *lamb;      /* [opt] M behaviour rates                      */
    const float   *thetab;    /* [opt] M*kb behaviour parameters              */
    const int32_t *bty;       /* [opt] kb behaviour type ids 0..4             */
    const int32_t *z0;        /* [opt] n start behaviour values               */
    const float   *vb;        /* [opt] n centred start behaviour              */
    const int32_t *bkdist;    /* [opt] n: actor counted in behaviour distance */
    int32_t zmin, zmax;
    float   zbar, brange, bsimmean;

    int32_t nrate;            /* non-basic rate effects 0..CUSNA_MAXRATE      */
    const int32_t *rkind;     /* [opt] nrate: 0 RateX, 1 outRate, 2 inRate    */
    const float   *ralpha;    /* [opt] nrate rate parameters                  */
    const float   *ru;        /* [opt] nrate*n RateX covariate values         */

    /* float64 descriptors. When non-NULL they take precedence over the float
     * fields above, as in the CPU engine (src/libcusna_saom_cpu.cpp:337-350).
     * The cpp11 glue sets only these (src/cusna_saom_glue.cpp:101-103). */
    const double *vmat64;     /* [opt] k*n                                    */
    const double *wtab64;     /* [opt] k*(n+1)                                */
    const double *vb64;       /* [opt] n                                      */
    const double *p1_64;      /* [opt] k                                      */
    const double *p2_64;      /* [opt] k                                      */
} cusna_saom_problem;

/* Outputs, caller-allocated; NULL skips one (src/libcusna.h:185-208). */
typedef struct cusna_saom_result {
    int32_t struct_version;

    double  *stats;      /* [M*k]      statistics of the masked end network   */
    double  *ntim;       /* [M]        simulated time                         */
    float   *scores;     /* [M*(k+1)]  column 0 rate score, then k effects    */
    int32_t *dist;       /* [M]        signed distance walked vs x0           */
    int32_t *dist_stat;  /* [M]        |x_end xor x0| over kdist              */
    int32_t *steps;      /* [M]        ministeps taken                        */

    int32_t *bdist;      /* [opt] [M]          (kb > 0)                       */
    float   *bscores;    /* [opt] [M*(kb+1)]   (kb > 0)                       */
    int32_t *z_end;      /* [opt] [M*n]        (kb > 0)                       */

    float   *rscores;    /* [opt] [M*nrate]    (nrate > 0)                    */
    int32_t *actor_dist; /* [opt] [M*n]        (nrate > 0)                    */

    int32_t  want_end_nets;
    uint8_t *a_ends;     /* [opt] [M*n*n] dense end networks, row-major       */
} cusna_saom_result;

/* Run M chains of one period on the GPU (src/libcusna.h:210-213; the
 * reference declares it but ships no definition). Chain c draws from Philox
 * counters (msteps, c, 0, 0) and (msteps, c, 1, j) under key `seed`, as
 * src/libcusna_saom_cpu.cpp:167,266 do, so trajectories equal the CPU
 * engine's for the same seed. Returns CUSNA_ERR_NO_CUDA without a device. */
CUSNA_API cusna_status cusna_saom_simulate_period(
    const cusna_saom_problem *problem, cusna_saom_result *result);

/* --------------------------------------------------------------------------
 * Utilities (src/libcusna.h:297-305, :527-530).
 * -------------------------------------------------------------------------- */

/* Pack a dense row-major uint8 n*n adjacency into out rows and in rows (n*W
 * words each, caller-allocated); *W_out = W (src/libcusna.h:299-301). */
CUSNA_API cusna_status cusna_pack_bits(
    const uint8_t *dense, int32_t n,
    uint32_t *out_rows, uint32_t *in_rows, int32_t *W_out);

/* One Philox4x32-10 block, the generator of the simulator (src/libcusna.h:
 * 304-305; the round function is src/libcusna_saom_cpu.cpp:32-45). */
CUSNA_API cusna_status cusna_philox4x32(
    const uint32_t counter[4], const uint32_t key[2], uint32_t out[4]);

CUSNA_API int32_t     cusna_abi_version(void);     /* CUSNA_ABI_VERSION      */
CUSNA_API const char *cusna_version_string(void);  /* build description      */
CUSNA_API int32_t     cusna_has_cuda(void);        /* 1 if a device is usable */
CUSNA_API const char *cusna_last_error(void);      /* per-thread error detail */

/* ==========================================================================
 * EXTENSION: GB300 entry points. None of these exists in the reference; the
 * reference-facing symbols above do not depend on them.
 * ========================================================================== */

/* Launch and memory options for the _ex entry points. Zero-initialise and set
 * struct_version; zero in every other field means "default". */
typedef struct cusna_gpu_options {
    int32_t  struct_version;   /* CUSNA_ABI_VERSION                           */
    int32_t  device_ptrs;      /* 1: every problem/result pointer except the
                                  struct itself is a device pointer            */
    uint32_t chain_offset;     /* global index of chain 0 (Philox counter word
                                  1), so M chains can be split across calls or
                                  GPUs with identical results                  */
    int32_t  warps_per_chain;  /* 0 = autotuned                               */
    int32_t  chains_per_cta;   /* 0 = autotuned                               */
    int32_t  launches;         /* out: kernels this call launched             */
    void    *stream;           /* cudaStream_t to run on (NULL = the library's
                                  own per-thread stream)                       */
    double   elapsed_ms;       /* out: device time of the simulation kernels  */
    int64_t  ministeps;        /* out: ministeps summed over all chains       */
    int32_t  specialise;       /* in: 0 as CUSNA_JIT says (compile the period
                                  kernel for the effect plan in the background
                                  after a few uses), -1 never, 1 compile now  */
    int32_t  specialised;      /* out: 1 if the specialised kernel ran        */
} cusna_gpu_options;

/* cusna_saom_simulate_period with options (device-resident buffers, chain
 * offset, stream) and device timing written back into *opts. */
CUSNA_API cusna_status cusna_saom_simulate_period_ex(
    const cusna_saom_problem *problem, cusna_saom_result *result,
    cusna_gpu_options *opts);

/* Run `count` independent problems (periods, groups, parameter points) in one
 * persistent launch. Problems may have different n, k, M and effects; chains of
 * all problems share one work queue. Each result is the same as a separate
 * cusna_saom_simulate_period call on that problem. */
CUSNA_API cusna_status cusna_saom_simulate_batch(
    const cusna_saom_problem *problems, cusna_saom_result *results,
    int32_t count, cusna_gpu_options *opts);

/* ---- validation mode (no counterpart in the reference) ----------------------
 * cusna_saom_simulate_period with a per-ministep trace, for checking a
 * trajectory step by step against the reference chooser
 * (src/libcusna_saom_cpu.cpp:166-287), and optionally with caller-supplied
 * random words in place of the Philox outputs. Every pointer is a host pointer.
 *
 * trace (trace_cap > 0): M*trace_cap records of 4 int32, chain-major; record s
 * of chain c is (s, focal actor, choice, distance change) for the chain's
 * ministep s < trace_cap. The choice of a network ministep is the chosen alter
 * (the actor itself for "no change"), of a behaviour ministep -(d + 2) for the
 * step d in {-1, 0, 1}; the change is that of the network distance (of the
 * behaviour distance for a behaviour ministep). Records past a chain's last
 * ministep are -1.
 *
 * ustream (ustream_steps > 0): M*ustream_steps*(4 + n) uint32 words,
 * chain-major; for ministep s < ustream_steps of chain c the 4 + n words at
 * ((c*ustream_steps + s)*(4 + n)) replace the Philox outputs: words 0-3 those
 * of counter (s, c, 0, 0) (waiting time, network/behaviour choice, focal
 * actor, behaviour step), word 4 + j the first output of counter (s, c, 1, j)
 * (alter j's Gumbel draw). Later ministeps draw from Philox as usual.
 *
 * lse64 = 1 forms the score sums in float64 at every ministep, as the
 * reference does (otherwise in double-float, with float64 only where a
 * predictor leaves [-60, 60]). warps_per_chain / chains_per_cta (0: chosen by
 * the library) force the launch shape; the validation build runs CTAs of at
 * most 256 threads. The call runs the library's own kernel, never a
 * specialised one, and no result depends on the launch shape. */
typedef struct cusna_validation_options {
    int32_t  struct_version;   /* CUSNA_ABI_VERSION                           */
    int32_t  trace_cap;        /* trace records per chain (0: no trace)        */
    int32_t *trace;            /* [opt] M*trace_cap*4 int32                   */
    int32_t  ustream_steps;    /* ministeps per chain with supplied words      */
    const uint32_t *ustream;   /* [opt] M*ustream_steps*(4+n) uint32           */
    int32_t  lse64;            /* 1: score sums in float64 at every ministep   */
    int32_t  warps_per_chain;  /* 0 = library's choice, else 1, 2, 4 or 8      */
    int32_t  chains_per_cta;   /* 0 = library's choice                         */
} cusna_validation_options;

CUSNA_API cusna_status cusna_saom_simulate_period_validate(
    const cusna_saom_problem *problem, cusna_saom_result *result,
    const cusna_validation_options *opts);

/* Evaluation statistics of M end networks on the GPU: the batched device
 * counterpart of the reference's host cusna_network_stats
 * (src/libcusna_saom_cpu.cpp:619-689). `a_batch` is M*n*n dense uint8 (the
 * statistic network per chain); the descriptors are those of
 * cusna_network_stats. Fills out[M*k]. */
CUSNA_API cusna_status cusna_network_stats_gpu(
    const uint8_t *a_batch, int32_t n, int32_t M, int32_t k,
    const int32_t *type_ids, const double *p1, const double *p2,
    const double *vmat, const uint8_t *vmiss, const int32_t *dyn_flags,
    const double *vb, const int32_t *od0, const int32_t *id0,
    const double *wtab, int32_t symflag, double *out);

/* Behaviour statistics of M end behaviour vectors on the GPU, the device
 * counterpart of cusna_behavior_stats (src/libcusna_saom_cpu.cpp:768-817).
 * Same arguments; fills out[M*kb]. */
CUSNA_API cusna_status cusna_behavior_stats_gpu(
    const int32_t *z_batch, int32_t n, int32_t M, int32_t kb,
    const int32_t *bty, const uint8_t *xnet, const int32_t *bkdist,
    double zbar, double brange, double bsimmean, double *out);

/* cusna_saom_simulate_period for callers that cannot allocate device memory.
 * No counterpart in the reference. Callers that cannot call cudaMalloc
 * include hosts whose device memory belongs to another allocator and
 * latency-bound loops that must not enter the allocator. The call allocates
 * nothing. It is not safe inside a stream capture: it waits for its own work
 * before returning and copies a few small host arrays. Every problem
 * and result pointer must be a device pointer (as with device_ptrs in
 * cusna_gpu_options), and the work runs on `stream` (a cudaStream_t; NULL for
 * the default stream); the few descriptor arrays the host reads are copied
 * on that stream, after the caller's own work there. The call returns once
 * the results are written.
 * Its scratch is one fixed 16 MiB array in device memory. Every GPU that loads
 * the library holds that array until the process exits. A problem that needs
 * more scratch is refused with CUSNA_ERR_UNSUPPORTED and the size in
 * cusna_last_error(); so is a problem whose chain out-rows do not fit one
 * CTA's shared memory (n beyond about 1,200-1,300 actors, depending on the
 * model). The first call on each device looks up the array's
 * device address (once). All calls share the array: calls whose GPU work
 * overlaps, from two streams
 * or two threads, race on it and must be serialised by the caller. */
CUSNA_API cusna_status cusna_saom_simulate_period_static(
    const cusna_saom_problem *problem, cusna_saom_result *result, void *stream);

/* ---- replayable plans (no counterpart in the reference) ---------------------
 * A plan prepares `count` problems once and then simulates all of them again at
 * every launch, in one persistent kernel, with the work ordered longest chain
 * first. It is built for loops that simulate the same problems many times with
 * new parameters: Robbins-Monro rounds over many periods or groups.
 *
 * cusna_saom_plan_create: every problem and result pointer is a DEVICE pointer
 * (as with device_ptrs in cusna_gpu_options) and must stay valid for the plan's
 * lifetime. The start networks and descriptors are copied into the plan;
 * type_ids, od0, id0, vmiss, bty and rkind are read in place. theta, lam, lamb
 * and thetab are read again at every launch, so the caller may rewrite them
 * between launches. With shared_params = 1 each of them holds ONE row used by
 * all M chains (theta k floats, lam 1 float, ...); with 0 they hold a row per
 * chain, as in cusna_saom_problem. Each launch overwrites the results.
 * Launch e (counting from 0, or from cusna_saom_plan_set_epoch) uses Philox key
 * seed + e for each problem, so launch 0 reproduces cusna_saom_simulate_batch.
 *
 * cusna_saom_plan_launch only enqueues kernels on `stream`: no allocation, no
 * host copy, no wait, so it may run inside a stream capture. With use_graph != 0
 * the launch is captured once into a CUDA graph (on a private stream; the first
 * such call must not itself be inside a capture) and replayed afterwards.
 * Launches of one plan must not overlap. */
typedef struct cusna_saom_plan cusna_saom_plan;
CUSNA_API cusna_status cusna_saom_plan_create(const cusna_saom_problem *problems,
                                             cusna_saom_result *results, int32_t count,
                                             int32_t shared_params, cusna_saom_plan **plan);
CUSNA_API cusna_status cusna_saom_plan_launch(cusna_saom_plan *plan, void *stream,
                                             int32_t use_graph);
CUSNA_API cusna_status cusna_saom_plan_set_epoch(cusna_saom_plan *plan, uint64_t epoch);
/* The launch shape the autotuner chose for the plan. */
CUSNA_API cusna_status cusna_saom_plan_shape(const cusna_saom_plan *plan,
                                            int32_t *warps_per_chain, int32_t *chains_per_cta,
                                            int32_t *ctas);
/* Waits for the device, then frees the plan and its device memory. */
CUSNA_API void cusna_saom_plan_destroy(cusna_saom_plan *plan);

/* ---- Method-of-Moments estimator (src/libcusna.h:532-542 reserves the opaque
 * cusna_mom_options / cusna_mom_result for it; this defines them) ------------
 * The Robbins-Monro MoM fit of R/mom.R:129-269 (phases 1-3: derivative,
 * diagonalised inverse, guarded steps, averaged phase-2 iterates, phase-3
 * standard errors and convergence t-ratios) in C++ over replayable plans:
 * every period (or group-period) of the model is prepared once on the device,
 * and each round only rewrites the parameters and replays the plan's CUDA
 * graph; the phase-2 rounds ask for the statistics alone (no score sums).
 *
 * periods[0..P): one cusna_saom_problem per period as the glue fills it for
 * the CPU engine (host pointers; x0/sim start networks, descriptors,
 * conditional and target_dist). Their M, seed, theta and lam are ignored (the
 * estimator sets them). Network effects only: kb and nrate must be 0.
 * targets[0..p): the observed moments in the estimator's layout
 * (R/targets.R:99-126): unconditional p = P + k, the P observed distances then
 * the k effect statistics summed over periods; conditional p = k.
 * result->theta[0..p): the start when use_start is set (else the reference's
 * default start, R/mom.R:199-211: rates 1.5 d/n + 1, density -1, others 0);
 * the estimate on return. The other output arrays may be NULL.
 * Every option left 0 takes the reference's default (mom_control(),
 * R/estimate.R:21-28), so a zeroed struct is the reference's control;
 * diagonalize < 0 asks for weight 0 (no diagonalisation). */
typedef struct cusna_mom_options {
    int32_t  struct_version;  /* CUSNA_ABI_VERSION                             */
    int32_t  conditional;     /* 1: conditional MoM (periods stop at target_dist) */
    double   firstg;          /* initial gain (0: 0.4)                          */
    int32_t  nsub;            /* phase-2 subphases (0: 4)                       */
    const int32_t *n2;        /* [nsub] iterations per subphase (NULL: 40, 40, 60, 80, then 80) */
    int32_t  batch2;          /* chains per phase-2 iteration (0: 256)          */
    int32_t  n1;              /* phase-1 chains (0: 1000)                       */
    int32_t  nD;              /* chains per subphase derivative (0: 1000)       */
    int32_t  n3;              /* phase-3 chains (0: 4000)                       */
    double   diagonalize;     /* weight of diag(D) in the inverse (0: 0.2; < 0: weight 0, the full D) */
    uint64_t seed;            /* seeds of the periods' Philox streams (0: 1234) */
    const double *rate_consts;/* [opt] P constants added to the distance statistics
                                 (composition changes, R/mom.R:160)           */
    int32_t  use_graph;       /* 1 (default, 0 = 1): replay rounds from CUDA graphs; -1 plain launches */
    int32_t  verbose;         /* 1: the estimate after each phase on stderr (R/mom.R:230, :245-246) */
} cusna_mom_options;

typedef struct cusna_mom_result {
    int32_t  struct_version;
    int32_t  use_start;       /* in: 1 = start from theta                       */
    double  *theta;           /* [p] in/out                                     */
    double  *se;              /* [opt] [p] standard errors                      */
    double  *tconv;           /* [opt] [p] convergence t-ratios                 */
    double  *sim_means;       /* [opt] [p] phase-3 simulated means              */
    double  *D;               /* [opt] [p*p] phase-3 score-function derivative  */
    double  *msf;             /* [opt] [p*p] phase-3 covariance of the statistics */
    double  *rate_est;        /* [opt] [P] conditional: mean simulated time per period */
    double  *rate_sd;         /* [opt] [P] conditional: its standard deviation  */
    double   tconv_max;       /* out: overall maximum convergence ratio         */
    int64_t  n_sims;          /* out: chains simulated per period               */
    double   wall_seconds;    /* out                                            */
    double   phase_seconds[3];/* out: phases 1, 2, 3                            */
} cusna_mom_result;

CUSNA_API cusna_status cusna_mom_estimate(const cusna_saom_problem *periods, int32_t P,
                                          const double *targets, int32_t p,
                                          const cusna_mom_options *opts,
                                          cusna_mom_result *result);

/* ---- multi-network co-evolution (src/libcusna.h:219-291) --------------------
 * D one-mode networks (2..CUSNA_MAXNET) on one actor set. Each ministep picks a
 * network with probability proportional to its rate, then one actor of it
 * toggles (or keeps) one tie. netof[e] is the network effect e belongs to;
 * cross-network effects (type ids 33 crprod, 34 crprodRecip, 35 crprodMutual,
 * 36 from, 37 to) read the current state of network netref[e]. The simulator
 * returns scores, rate scores, times, steps and the end networks; statistics
 * are computed from the end networks (cusna_network_stats_gpu,
 * cusna_cross_stats). Structs as the reference lays them out. As in the
 * reference engine, interactions (type 32) change nothing, reciAct (19) sees a
 * reciprocated degree of 0, and dyc is one n*n dyadic covariate (dyc_idx -1 or
 * 0, read by type 22). */
typedef struct cusna_saom_multi_problem {
    int32_t struct_version;   /* CUSNA_ABI_VERSION                              */
    int32_t n;                /* actors, shared by the D networks               */
    int32_t W;                /* (n + 31) / 32                                  */
    int32_t k;                /* network effects over all networks, <= MAXEFF   */
    int32_t M;                /* chains                                         */
    int32_t D;                /* networks, 2..CUSNA_MAXNET                      */
    int32_t threads;          /* unused by this build                           */

    const uint32_t *x0_out;   /* D*n*W packed out-ties of the start networks    */
    const uint32_t *x0_in;    /* D*n*W packed in-ties                           */
    const float   *lam;       /* M*D per-chain, per-network basic rates         */
    const float   *theta;     /* M*k per-chain parameters                       */

    const int32_t *type_ids;  /* k effect type ids                              */
    const int32_t *etypes;    /* k: 0 evaluation, 1 creation, 2 endowment       */
    const int32_t *netof;     /* k: network of each effect, 0..D-1              */
    const int32_t *netref;    /* k: source network of a cross effect, else 0    */
    const float   *wtab;      /* k*(n+1) weight tables                          */
    const float   *p1;        /* k                                              */
    const float   *p2;        /* k                                              */
    const float   *vmat;      /* k*n covariate values                           */
    const float   *dyc;       /* [opt] dyadic covariates                        */
    const int32_t *dyc_idx;   /* k: index into dyc, or -1                       */
    const uint32_t *perm;     /* [opt] D*n*W permitted dyads (NULL: all i != j) */
    const int32_t *symf;      /* D per-network symmetric flags                  */
    uint64_t seed;            /* Philox key                                     */
    const int32_t *act;       /* [opt] active actors first                      */
    int32_t nact;             /* active actor count                             */
} cusna_saom_multi_problem;

typedef struct cusna_saom_multi_result {
    int32_t struct_version;
    float   *rscores;         /* [opt] M*D per-network basic-rate scores        */
    float   *scores;          /* [opt] M*k effect scores                        */
    double  *ntim;            /* [opt] M elapsed simulated time                 */
    int32_t *steps;           /* [opt] M ministeps                              */
    uint8_t *a_ends;          /* [opt] M*D*n*n dense end networks (row-major)   */
} cusna_saom_multi_result;

/* M chains of one multi-network period on the GPU (replaces the declaration at
 * src/libcusna.h:280-285 and the CPU mirror cusna_saom_simulate_multi_cpu,
 * src/libcusna_saom_cpu.cpp:427-604). Trajectories equal the CPU mirror's. */
CUSNA_API cusna_status cusna_saom_simulate_multi(
    const cusna_saom_multi_problem *problem, cusna_saom_multi_result *result);

/* Cross-network statistic of M own end networks a_batch (M*n*n dense uint8)
 * against the source network's period-start predictor wp (n*n dense uint8)
 * for cross effect type t (33..37; parm: 36 takes square roots when >= 2),
 * into out[M] (src/libcusna.h:366-374; CPU src/libcusna_saom_cpu.cpp:819-857).
 * Computed on the GPU. */
CUSNA_API cusna_status cusna_cross_stats(
    const uint8_t *a_batch, const uint8_t *wp, int32_t n, int32_t M,
    int32_t t, double parm, double *out);

/* Creation / endowment statistic of one typed effect over M end networks
 * a_batch (M*n*n dense uint8), computed on the GPU (replaces
 * src/libcusna.h:319-331; CPU src/libcusna_saom_cpu.cpp:691-714). etype 1
 * (creation) sums F (n*n float64) over ties of (a & keep) | force absent from
 * the start network x0 and not missing at the period start (miss_m); any other
 * etype (endowment) sums F over ties of x0 absent from (a & keepS) | forceS and
 * not missing at the end (miss_m1), and reports the sum negated. Masks are
 * dense n*n uint8 and optional (NULL: keep/keepS all 1, the others all 0).
 * out[M]. The sum is added in another order than the CPU engine's: equal
 * within float64 rounding of the sum of |F|. */
CUSNA_API cusna_status cusna_typed_stats(
    const uint8_t *a_batch, int32_t n, int32_t M, int32_t etype,
    const double *F, const uint8_t *x0,
    const uint8_t *keep, const uint8_t *force,
    const uint8_t *keepS, const uint8_t *forceS,
    const uint8_t *miss_m, const uint8_t *miss_m1, double *out);

/* sienaGOF auxiliary distributions of M end networks a_batch (M*n*n dense
 * uint8), computed on the GPU (replaces src/libcusna.h:333-343; CPU
 * src/libcusna_saom_cpu.cpp:716-765). kind 0 / 1: per level the number of
 * actors with in- / out-degree at most levls[L], out is M*nlev. kind 2: per
 * level the ordered pairs i != j within geodesic distance levls[L], then the
 * unreachable pairs, out is M*(nlev+1); a negative geodesic level is
 * CUSNA_ERR_SHAPE. Counts equal the CPU engine's. */
CUSNA_API cusna_status cusna_gof_distribution(
    const uint8_t *a_batch, int32_t n, int32_t M, int32_t kind,
    const int32_t *levls, int32_t nlev, double *out);

/* ---- period kernel specialised to an effect plan (no counterpart) ----------
 * The library's period kernel evaluates the model's effects through a per-
 * effect dispatch. For a model used repeatedly, the library compiles (NVRTC,
 * in a background thread, after CUSNA_JIT_AFTER uses of the same effect plan,
 * default 3) a copy of the kernel with the effect plan written out, and runs it
 * once it is ready; every output is bit-identical to the library kernel's.
 * CUSNA_JIT=0 disables this, CUSNA_JIT=sync compiles on first use, and
 * cusna_gpu_options.specialise overrides it per call.
 * cusna_saom_specialise_check validates problem (host pointers) and compiles
 * its specialised kernel without loading it (no device needed): CUSNA_OK, or
 * CUSNA_ERR_UNSUPPORTED with the compiler log in log[0..log_len) and
 * cusna_last_error(); *seconds (may be NULL) receives the compile time.
 * cusna_saom_specialise_wait waits up to `seconds` for background compilations
 * and writes how many have completed to *compiled (may be NULL). */
CUSNA_API cusna_status cusna_saom_specialise_check(const cusna_saom_problem *problem, char *log,
                                                   size_t log_len, double *seconds);
CUSNA_API cusna_status cusna_saom_specialise_wait(double seconds, int32_t *compiled);
/* Overrides CUSNA_JIT for the process: 0 never specialise, 1 compile in the
 * background after a few uses, 2 compile on first use, -1 back to CUSNA_JIT. */
CUSNA_API cusna_status cusna_saom_specialise_mode(int32_t mode);
/* cusna_saom_specialise_check for the multi-network kernel (the networks'
 * effect plans of a multi-network problem). cusna_saom_simulate_multi runs the
 * specialised kernel once it is compiled, with bit-identical outputs. */
CUSNA_API cusna_status cusna_saom_specialise_check_multi(const cusna_saom_multi_problem *problem,
                                                         char *log, size_t log_len,
                                                         double *seconds);

/* ---- moment surrogate (no counterpart in the reference) --------------------
 * A multilayer perceptron n_in -> hidden -> hidden -> n_out with GELU
 * activations, used by the estimator to stand in for simulated moments in
 * Robbins-Monro phases 1-2. Products run on the tensor cores with bfloat16
 * operands and float32 accumulation; parameters, gradients and Adam moments are
 * float32 in one buffer of cusna_mlp_param_count() floats laid out
 * [W1 (hidden x n_in) | b1 | W2 (hidden x hidden) | b2 | W3 (n_out x hidden) | b3].
 * n_in and hidden are multiples of 16 (hidden <= 4096), 1 <= n_out <= 16.
 * Every pointer is a device pointer; work is a device workspace of at least
 * cusna_mlp_workspace_bytes(.., batch) bytes (work_bytes, checked); the work
 * runs asynchronously on `stream` (a cudaStream_t, NULL for the default). */
CUSNA_API size_t cusna_mlp_param_count(int32_t n_in, int32_t hidden, int32_t n_out);
CUSNA_API size_t cusna_mlp_workspace_bytes(int32_t n_in, int32_t hidden, int32_t n_out,
                                           int32_t batch);
/* He-normal hidden-layer weights from a Philox stream keyed by seed; the
 * output layer and the biases start at zero (the untrained network predicts
 * zero). */
CUSNA_API cusna_status cusna_mlp_init(float *params, int32_t n_in, int32_t hidden,
                                      int32_t n_out, uint64_t seed, void *stream);
/* y[batch x n_out] = network(x[batch x n_in]). */
CUSNA_API cusna_status cusna_mlp_forward(const float *params, const float *x, int32_t batch,
                                         float *y, void *work, size_t work_bytes, int32_t n_in,
                                         int32_t hidden, int32_t n_out, void *stream);
/* Mean squared error of the network on rows rows[0..batch) of x and t (rows
 * NULL: the first batch rows) and its gradient with respect to every parameter
 * into grad; *loss (device, may be NULL) receives the loss. batch is a multiple
 * of 16. */
CUSNA_API cusna_status cusna_mlp_grad(const float *params, const float *x, const float *t,
                                      const int32_t *rows, int32_t batch, float *grad,
                                      float *loss, void *work, size_t work_bytes, int32_t n_in,
                                      int32_t hidden, int32_t n_out, void *stream);
/* cusna_mlp_grad followed by one Adam step (step = 1, 2, ...; bias-corrected)
 * on params with moment buffers adam_m and adam_v. */
CUSNA_API cusna_status cusna_mlp_train_step(float *params, float *grad, float *adam_m,
                                            float *adam_v, const float *x, const float *t,
                                            const int32_t *rows, int32_t batch, int32_t step,
                                            float lr, float beta1, float beta2, float eps,
                                            float *loss, void *work, size_t work_bytes,
                                            int32_t n_in, int32_t hidden, int32_t n_out,
                                            void *stream);
/* Adam hyperparameters and step counter in device memory: each step adds one
 * to `step` and writes the bias corrections c1 = 1 - beta1^step and
 * c2 = 1 - beta2^step on the device, so the host may change lr between calls
 * by writing it, without changing any argument. */
typedef struct cusna_adam_hyper {
    int32_t step;
    float lr, beta1, beta2, eps;
    float c1, c2;
} cusna_adam_hyper;
/* n_steps Adam steps on consecutive minibatches: step s uses rows
 * rows[s*batch .. (s+1)*batch) of x and t (rows NULL: rows 0..batch each
 * step); losses[s] (device, may be NULL) receives step s's loss. With
 * use_graph != 0 the sequence is captured once into a CUDA graph per distinct
 * argument set (a few are cached, oldest evicted) and replayed on `stream`;
 * the contents of rows, x, t and *hyper may change between replays. Graph
 * capture uses a private stream: the first call with a new argument set must
 * not itself run inside a stream capture. */
CUSNA_API cusna_status cusna_mlp_train_steps(float *params, float *grad, float *adam_m,
                                             float *adam_v, const float *x, const float *t,
                                             const int32_t *rows, int32_t batch, int32_t n_steps,
                                             cusna_adam_hyper *hyper, float *losses, void *work,
                                             size_t work_bytes, int32_t n_in, int32_t hidden,
                                             int32_t n_out, int32_t use_graph, void *stream);
/* Outputs y[batch x n_out] and their Jacobian J[batch x n_out x n_wrt] with
 * respect to the first n_wrt inputs (forward-mode, float32). */
CUSNA_API cusna_status cusna_mlp_jacobian(const float *params, const float *x, int32_t batch,
                                          int32_t n_wrt, float *y, float *J, void *work,
                                          size_t work_bytes, int32_t n_in, int32_t hidden,
                                          int32_t n_out, void *stream);

#ifdef __cplusplus
}  /* extern "C" */
#endif

#endif  /* LIBCUSNA_H */
