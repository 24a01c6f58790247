/*
 * gelio.h -- C ABI of the GB300 (sm_103a) Geliosphere SDE engine.
 *
 * This is the drop-in boundary that replaces the reference's CUDAKernel
 * library and the log.dat -> spectrum evaluation for the four heliospheric
 * transport models.  Every entry point is plain C: no C++ types, no torch
 * types, caller-owned memory, an int32 status return, no exit() and no
 * exceptions across the boundary (the reference calls exit() from
 * gpuErrchk, CUDAKernel/include/CudaErrorCheck.cuh:25-41).
 *
 * Reference interfaces replaced (paths relative to the reference project):
 *   gelio_run / gelio_run_async
 *       AbstractGpuSimulation::prepareAndRunSimulation(ParamsCarrier*)
 *         CUDAKernel/include/AbstractGpuSimulation.hpp:23-32, implemented by
 *         OneDimensionFpGpuModel.cpp:7-40, OneDimensionBpGpuModel.cpp:7-43,
 *         SolarPropLikeGpuModel.cpp:7-44, GeliosphereGpuModel.cpp:7-44, which
 *         drive runOneDimensionFpSimulation (OneDimensionFpModel.cu:150-203),
 *         runOneDimensionBpSimulation (OneDimensionBpModel.cu:149-200),
 *         runSolarPropLikeSimulation (SolarPropLikeModel.cu:256-306) and
 *         runGeliosphereSimulation (GeliosphereModel.cu:399-449);
 *       fused with the evaluators TwoDimensionBpResults::runAlgorithm
 *         (Algorithm/src/TwoDimensionBpResults.cpp:13-133),
 *         OneDimensionBpResults::runAlgorithm (OneDimensionBpResults.cpp:13-112),
 *         OneDimensionFpResults::runAlgorithm (OneDimensionFpResults.cpp:13-113).
 *   gelio_evaluate
 *       the evaluators above when run on an existing log.dat
 *       (--evaluation mode, Input/src/ParseParams.cpp:71-74).
 *   gelio_replay
 *       no reference counterpart: per-trajectory exit states for checking
 *       the kernels against the FP64 oracle that replays the same Philox
 *       random stream.
 *   gelio_create / gelio_destroy
 *       the per-call cudaMalloc/cudaFree of *GpuModel::prepareAndRunSimulation
 *       (e.g. GeliosphereGpuModel.cpp:17-43) become a context that owns the
 *       device buffers across calls.
 *
 * Units follow the reference's __constant__ parameters
 * (CUDAKernel/src/CosmicConstants.cu:14-41): K0 in AU^2/s, V in AU/s,
 * dt in s, r in AU, angles in rad, kinetic energies in GeV.
 */
#ifndef GELIO_H
#define GELIO_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GELIO_ABI_VERSION 1

/* Status codes.  Values >= GELIO_WARN_FIRST are warnings: the outputs are
 * complete and valid, but something the caller asked for was bounded. */
enum {
    GELIO_OK = 0,
    GELIO_ERR_INVALID_ARGUMENT = 1,
    GELIO_ERR_NO_DEVICE = 2,
    GELIO_ERR_CUDA = 3,
    GELIO_ERR_OUT_OF_MEMORY = 4,
    GELIO_ERR_TIMEOUT = 5,        /* the device watchdog stopped the run */
    GELIO_ERR_UNSUPPORTED = 6,
    GELIO_ERR_NOT_TRAINED = 7,
    GELIO_WARN_FIRST = 100,
    GELIO_WARN_RECORDS_TRUNCATED = 100, /* exit records beyond record_capacity were binned but not stored */
    GELIO_WARN_STEP_CAP = 101           /* some trajectories hit max_steps_per_particle */
};

enum {
    GELIO_MODEL_1D_FP = 0,          /* 1D forward-in-time F-p   (OneDimensionFpModel.cu) */
    GELIO_MODEL_1D_BP = 1,          /* 1D backward-in-time B-p  (OneDimensionBpModel.cu) */
    GELIO_MODEL_2D_SOLARPROP = 2,   /* 2D SolarProp-like        (SolarPropLikeModel.cu)  */
    GELIO_MODEL_2D_GELIOSPHERE = 3  /* 2D Geliosphere           (GeliosphereModel.cu)    */
};

enum {
    /* CosmicUtils.cu:17-34 getTkinInjection(global index): 1e4 energies per
     * GeV, T = floor(s/1e4) + (s mod 1e4 + 1)/1e4, wrapping at
     * injection_max * 1e4.  Default of the 1D GPU models. */
    GELIO_INJ_REFERENCE_UNIFORM = 0,
    /* CosmicUtils.cu:36-40 getSolarPropInjection: T = 0.01 * 1.5^(s mod 30).
     * Default of the 2D GPU models (use_uniform_injection = 0). */
    GELIO_INJ_SOLARPROP_GRID = 1,
    /* inj_points energies log-spaced over [inj_min, inj_max]; particle s is
     * injected at point s mod inj_points (equal particles per point). */
    GELIO_INJ_LOG_GRID = 2,
    /* log-uniform over [inj_min, inj_max], drawn from the particle's Philox stream. */
    GELIO_INJ_LOG_UNIFORM = 3,
    /* CpuImplementations/include/Constants.hpp:234-239 getTkinInjection(id,
     * 1e-4, injection_max, 10000): the CPU models' linear grid. */
    GELIO_INJ_CPU_UNIFORM = 4
};

enum {
    GELIO_PREC_FP32 = 0,   /* FP32 steps with compensated state updates (default) */
    GELIO_PREC_FP64 = 1    /* FP64 steps (the 1D B-p FP64-step variant; any model) */
};

/* gelio_sim_params.flags */
#define GELIO_FLAG_SOLARPROP_THETA_DRIFT_POLARITY 0x1
    /* SolarProp-like: scale the theta drift by the simulation polarity, as the
     * CPU model does (SolarPropLikeCpuModel.cpp:202).  Unset = the reference
     * GPU kernel, whose theta drift uses a fixed polarity of +1
     * (SolarPropLikeModel.cu:213 with CosmicConstants.cu:37). */

/* One simulation: everything the reference copies into __constant__ memory
 * in setConstants / setSolarPropConstants / setGeliosphereModelConstants
 * (CUDAKernel/src/CosmicConstants.cu:43-111), resolved by the caller. */
typedef struct gelio_sim_params {
    int32_t model;              /* GELIO_MODEL_* */
    int32_t injection;          /* GELIO_INJ_* */
    int64_t n_particles;        /* test particles of this simulation (>= 0) */
    float K0;                   /* AU^2/s */
    float V;                    /* AU/s, solar-wind speed magnitude (> 0).  The 1D B-p
                                   model runs with -V as the reference does
                                   (CosmicConstants.cu:73-83). */
    float dt;                   /* s */
    float r_injection;          /* AU: backward models start here; F-p starts at 100.0001 AU */
    float theta_injection;      /* rad (2D models) */
    float tilt;                 /* rad, alphaM */
    float polarity;             /* +1 or -1 */
    float ratio;                /* K_perp / K_par (2D) */
    float delta0;               /* C_delta (Geliosphere) */
    float injection_max;        /* GeV, GELIO_INJ_REFERENCE_UNIFORM / CPU_UNIFORM maximum (reference 101) */
    float inj_min;              /* GeV, GELIO_INJ_LOG_GRID / LOG_UNIFORM range */
    float inj_max;
    int32_t inj_points;         /* GELIO_INJ_LOG_GRID points (1..GELIO_GRID_MAX) */
    int32_t flags;              /* GELIO_FLAG_* */
    uint64_t seed;              /* Philox key (low, high 32 bits); independent of batch position */
    float grid_min;             /* GeV, log-binned 1 AU spectrum ("grid" section) */
    float grid_max;
    int32_t grid_bins;          /* 0..GELIO_GRID_MAX; 0 = none */
    int32_t reserved;
} gelio_sim_params;

#define GELIO_GRID_MAX 320

/* Per-simulation output.  Every section is FP64: per-bin sum of weights,
 * sum of squared weights (for per-bin Monte Carlo variance) and count.
 * Sections of the other dimensionality are zero.
 *
 * 1D sections (OneDimensionBpResults.cpp:13-112 / OneDimensionFpResults.cpp:13-113):
 *   log_*  1D B-p: 80 log bins (NT=80, 0.01-200 GeV) at indices 1..79 exactly
 *          as spelog[] is filled; 1D F-p: the 24-bin layout at 0..23.
 *   e2_* / e3_* / e4_*  the 1e2, 1e3 and 4e2 linear binnings (spe1e2[], ...).
 * 2D sections (TwoDimensionBpResults.cpp:13-133), binned on the injection energy:
 *   sp_*   SolarProp +-1% windows around SPbins[1..29] with the Weber, Usoskin
 *          ("JGR") and Burger LIS weights (speSP, speJGR, speBurger, speN);
 *   uly_*  2 Ulysses bins (Burger weight), indices 1..2;
 *   ams_*  70 AMS bins (Burger weight), indices 1..70.
 * grid section (all models; no reference counterpart): grid_bins log bins over
 *   [grid_min, grid_max] of the 1 AU energy (backward models: injection
 *   energy; F-p: crossing energy), 3 weights per model:
 *   2D:   J_LIS(T_exit) * p_1AU^2 / p_exit^2 for Weber, Usoskin, Burger;
 *   1D B-p: the reference weight Yamada(p_exit) * p_1AU^2, Weber, Burger;
 *   1D F-p: the reference weight, 0, 0.
 */
typedef struct gelio_spectra {
    double log_w[300], log_w2[300], log_n[300];
    double e2_w[100], e2_w2[100], e2_n[100];
    double e3_w[1000], e3_w2[1000], e3_n[1000];
    double e4_w[400], e4_w2[400], e4_n[400];
    double sp_weber[31], sp_jgr[31], sp_burger[31], sp_n[31];
    double sp_weber2[31], sp_jgr2[31], sp_burger2[31];
    double uly_w[4], uly_w2[4], uly_n[4];
    double ams_w[72], ams_w2[72], ams_n[72];
    double grid_w[3][GELIO_GRID_MAX];
    double grid_w2[3][GELIO_GRID_MAX];
    double grid_n[GELIO_GRID_MAX];
    double n_particles;   /* particles simulated */
    double n_records;     /* records binned */
    double n_steps;       /* particle-steps */
    double n_lost;        /* ended without a record */
    double n_step_capped;
    double reserved[11];
} gelio_spectra;

/* One record of the reference's log.dat (written when the caller keeps log
 * files, remove_log_files_after_simulation = 0). */
typedef struct gelio_exit_record {
    int64_t particle;     /* index within its simulation */
    int32_t sim;          /* index into the gelio_sim_params array */
    float t_injection;    /* GeV at injection */
    float t_exit;         /* GeV at the record (B-p/2D: 100 AU exit; F-p: 1 AU crossing) */
    float r;              /* AU */
    float theta;          /* rad (2D) */
    float sumac;          /* F-p accumulated sum of 4V dt/(3r) (OneDimensionFpModel.cu:88) */
} gelio_exit_record;

typedef struct gelio_run_opts {
    int32_t precision;            /* GELIO_PREC_* */
    int32_t plain;                /* 0 = persistent work-queue kernel with warp refill
                                     (default); 1 = one thread per particle, one
                                     launch per simulation, no refill (the plain
                                     baseline kernel) */
    int32_t compact;              /* FP32 persistent kernel register budget: 0 = tuned
                                     default, 1 = <= 128 registers (2 CTAs of 256 per
                                     SM), 2 = <= 85 registers (3 CTAs of 256 per SM) */
    int32_t block_size;           /* 0 = tuned default */
    int32_t blocks_per_sm;        /* 0 = occupancy maximum */
    int32_t refill_interval;      /* steps between warp refills (multiple of 4); 0 = tuned */
    int32_t use_graph;            /* capture the launch sequence in a CUDA graph and replay it */
    int32_t reserved0;
    uint64_t max_steps_per_particle; /* 0 = 100,000,000 */
    double time_limit_s;          /* device watchdog; 0 = none */
    gelio_exit_record *records;   /* optional host buffer (log.dat records) */
    int64_t record_capacity;
} gelio_run_opts;

typedef struct gelio_run_stats {
    int64_t n_particles;
    int64_t n_records;
    int64_t n_steps;
    int64_t n_lost;
    int64_t n_step_capped;
    int64_t n_records_stored;
    int64_t n_records_dropped;
    double kernel_ms;       /* SDE kernel device time (CUDA events on the run's stream) */
    double total_ms;        /* whole call, host wall clock */
    int32_t block_size;
    int32_t blocks_per_sm;
    int32_t grid_size;
    int32_t refill_interval;
} gelio_run_stats;

/* Per-trajectory result of gelio_replay. */
typedef struct gelio_trajectory {
    int32_t status;       /* 0 = ended with a record, 1 = ended without one, 2 = step cap */
    uint32_t steps;       /* steps taken */
    int32_t n_records;    /* records written (F-p may cross 1 AU several times) */
    float t_injection;
    float t_final;        /* energy when the trajectory ended */
    float r_final;
    float theta_final;    /* 2D: theta; F-p: sumac */
    float t_record;       /* first record: energy, r, theta/sumac */
    float r_record;
    float aux_record;
} gelio_trajectory;

typedef struct gelio_ctx gelio_ctx;

const char *gelio_status_string(int32_t status);
int32_t gelio_abi_version(void);

/* Allocation hook.  No counterpart in the reference: its GpuModel classes
 * allocate with cudaMallocManaged / cudaMalloc / cudaMallocHost inside each
 * prepareAndRunSimulation (e.g. CUDAKernel/src/GeliosphereGpuModel.cpp:
 * 17-22), and a failed allocation ends the process through gpuErrchk
 * (CUDAKernel/include/CudaErrorCheck.cuh:31-41).  Here every device and
 * pinned-host allocation the engine makes (contexts, surrogates) first calls
 * hook(kind, bytes, user); a nonzero return refuses it, and the call that
 * needed the memory returns GELIO_ERR_OUT_OF_MEMORY, as on an exhausted
 * device: no memory is taken, and the context or surrogate stays usable (a
 * later call allocates again).  This lets a host application hold the
 * engine to a memory budget.  One hook per process; NULL removes it.  The
 * hook may run on any thread that calls the engine and must not call it. */
enum { GELIO_ALLOC_DEVICE = 0, GELIO_ALLOC_PINNED_HOST = 1 };
typedef int32_t (*gelio_alloc_hook)(int32_t kind, uint64_t bytes, void *user);
int32_t gelio_set_alloc_hook(gelio_alloc_hook hook, void *user);

/* Text of the last CUDA failure on the calling thread (empty if none):
 * the CUDA error name and message and where it was raised.  Diagnostics
 * only; the status codes are the contract. */
const char *gelio_last_error(void);

/* Create a context on CUDA device `device`.  Returns GELIO_ERR_NO_DEVICE when
 * no CUDA device is usable; there is no CPU fallback. */
int32_t gelio_create(gelio_ctx **out, int32_t device);
int32_t gelio_destroy(gelio_ctx *ctx);

/* Run n_sims simulations (any mix of models) in one persistent launch and
 * return their binned spectra.  sims, out (n_sims entries), stats and opts
 * are host memory; opts and stats may be NULL. */
int32_t gelio_run(gelio_ctx *ctx, const gelio_sim_params *sims, int32_t n_sims,
                  const gelio_run_opts *opts, gelio_spectra *out,
                  gelio_run_stats *stats);

/* Stream-ordered variant for callers whose inputs and outputs live in device
 * memory: d_sims and d_out are device pointers (n_sims entries), `stream` is a
 * cudaStream_t (NULL = the context's stream).  Nothing is synchronised and no
 * host copy is made; opts is host memory (records are not supported here). */
int32_t gelio_run_async(gelio_ctx *ctx, const gelio_sim_params *d_sims,
                        int32_t n_sims, const gelio_run_opts *opts,
                        gelio_spectra *d_out, void *stream);

/* Read the statistics of the last gelio_run_async on the context
 * (synchronises the context's work). */
int32_t gelio_last_stats(gelio_ctx *ctx, gelio_run_stats *stats);

/* Per-trajectory exit states of particles [first, first + count) of one
 * simulation, in the requested precision (host output, count entries).
 * max_steps > 0 stops every trajectory after that many steps (status 2), so
 * states can be compared at a fixed step; 0 = 100,000,000. */
int32_t gelio_replay(gelio_ctx *ctx, const gelio_sim_params *sim,
                     int64_t first, int64_t count, int32_t precision,
                     uint64_t max_steps, gelio_trajectory *out);

/* Bin existing log.dat rows on the device, as the evaluators do.  rows is
 * row-major [n_rows][n_cols] host doubles in the column order of the
 * reference log.dat of that model (2D: 6 columns, 1D B-p: 4, 1D F-p: 5). */
int32_t gelio_evaluate(gelio_ctx *ctx, int32_t model, const double *rows,
                       int64_t n_rows, int32_t n_cols, gelio_spectra *out);

/* Pick the block size and refill interval by timing short runs of a sample
 * batch (n simulations, typically the production batch with fewer particles
 * each) and store the choice in the context for the model of the first
 * non-empty simulation; the chosen options are written to *best (host).
 * The figure of merit is particle-steps per second of the SDE kernels. */
int32_t gelio_autotune(gelio_ctx *ctx, const gelio_sim_params *sims, int32_t n,
                       gelio_run_opts *best);

/* Run n_sims (<= GELIO_NOALLOC_MAX_SIMS) simulations without allocating any
 * memory.  No counterpart in the reference: it serves callers that cannot
 * call cudaMalloc -- code that runs where device allocation is not allowed
 * or not wanted, such as a host application with a fixed device-memory
 * budget or a plugin that must not own allocations.  The caller passes the
 * inputs and outputs in device memory (d_sims: n_sims gelio_sim_params;
 * d_out: n_sims gelio_spectra) and a stream (NULL = the legacy default
 * stream); no context is needed.  All scratch lives in one static device
 * array of GELIO_NOALLOC_SCRATCH_BYTES that every GPU loading the library
 * holds until the process exits.  The first call on a device sets that
 * device up (resolves the array's address, fills tables, queries
 * occupancy), so it should be made before any stream capture; a set-up that
 * fails is retried by the next call, and after a cudaDeviceReset the process
 * must be restarted before this entry point is called again.  Calls share
 * the array: calls that overlap on the GPU (other streams, other threads)
 * race and corrupt each other.  The call waits for its own work on `stream`
 * and returns its status.  Of the options, precision, refill_interval,
 * max_steps_per_particle and time_limit_s apply; exit records, the plain
 * kernel and any other launch shape (block_size, blocks_per_sm, compact,
 * use_graph non-zero) are GELIO_ERR_UNSUPPORTED; more than
 * GELIO_NOALLOC_MAX_SIMS simulations is GELIO_ERR_INVALID_ARGUMENT. */
#define GELIO_NOALLOC_MAX_SIMS 8
#define GELIO_NOALLOC_SCRATCH_BYTES 1049344
int32_t gelio_run_noalloc(const gelio_sim_params *d_sims, int32_t n_sims,
                          const gelio_run_opts *opts, gelio_spectra *d_out,
                          void *stream);

/* Measure this device's FP32 SIMT throughput (FMA chains; FLOP/s with an
 * FMA counted as 2) and special-function-unit throughput (ex2.approx chains,
 * operations/s), in TFLOP/s and Gop/s.  A measurement helper for rooflines;
 * no reference counterpart. */
int32_t gelio_measure_peaks(gelio_ctx *ctx, double *fp32_tflops, double *xu_gops);

/* ------------------------------------------------------------------------
 * Spectrum surrogate (no reference counterpart: a learned addition on top
 * of the reference's Monte Carlo method).
 *
 * An ensemble of MLPs 7 -> 256 -> 256 -> 256 -> 256 -> 1 (SiLU, BF16
 * weights and activations, FP32 accumulation) maps a 2D Geliosphere
 * simulation's (K0, V, tilt, polarity, r_injection, theta_injection) and a
 * 1 AU kinetic energy T to ln(J_mod(T) / J_LIS(T)).  It is trained on the
 * GPU, by this library's own forward and backward kernels (tcgen05 GEMMs),
 * on spectra this library's Monte Carlo produced, and falls back to the
 * Monte Carlo where the members disagree.
 * ------------------------------------------------------------------------ */
typedef struct gelio_surrogate gelio_surrogate;

#define GELIO_SURR_FEATURES 7
#define GELIO_SURR_PARAMS 199681   /* FP32 parameters of one member (flat layout below) */
/* Flat layout: W1 [256][7], b1 [256], W2 [256][256], b2, W3, b3, W4, b4,
 * w5 [256], b5 [1]; W_l[o][i] multiplies input i into output o. */

typedef struct gelio_surrogate_opts {
    int32_t members;        /* ensemble size (0: 5) */
    int32_t batch_rows;     /* training batch rows, a multiple of 256 (0: 16384) */
    int32_t lis;            /* LIS of the target ratio: 0 Weber, 1 Usoskin 2005, 2 Burger */
    int32_t min_count;      /* grid points with fewer exits are not trained on (0: 64) */
    float lr;               /* Adam learning rate, cosine-decayed ... (0: 2e-3) */
    float lr_final;         /* ... to this over the run (0: 2e-5) */
    float fallback_std;     /* ensemble std of ln ratio above which the MC runs (0: 0.03) */
    float t_min, t_max;     /* energy range [GeV] that std is tested over (0: 0.1, 10) */
    int32_t reserved0;
    uint64_t seed;          /* initial weights and shuffling */
    int32_t reserved[8];
} gelio_surrogate_opts;

int32_t gelio_surrogate_create(gelio_ctx *ctx, const gelio_surrogate_opts *opts, gelio_surrogate **out);
void gelio_surrogate_destroy(gelio_surrogate *s);

/* Normalised network input of one (simulation, energy [GeV]). */
int32_t gelio_surrogate_features(const gelio_sim_params *sim, double t_gev, float out[7]);

/* Training rows from Monte Carlo spectra: every 2D Geliosphere simulation
 * run with GELIO_INJ_LOG_GRID (grid_bins = 0) contributes, for each grid
 * point j with at least min_count exits, features(sim, T_j) and
 * ln((grid_w[lis][j] / grid_n[j]) / J_LIS(T_j)).  *n_rows: rows held. */
int32_t gelio_surrogate_add_spectra(gelio_surrogate *s, const gelio_sim_params *sims,
                                    const gelio_spectra *spectra, int32_t n, int64_t *n_rows);

/* Training rows given directly: normalised inputs x [n][7], targets t [n]. */
int32_t gelio_surrogate_add_rows(gelio_surrogate *s, const float *x, const float *t, int64_t n,
                                 int64_t *n_rows);

/* `epochs` passes of Adam over the held rows for every member (MSE on the
 * ln ratio); last_loss[members] receives each member's last-epoch loss. */
int32_t gelio_surrogate_train(gelio_surrogate *s, int32_t epochs, float *last_loss);

/* Ensemble mean and standard deviation of ln(J_mod / J_LIS) at each
 * GELIO_INJ_LOG_GRID point of each simulation; outputs hold the points of
 * sims[0], then sims[1], ... (sum of inj_points entries). */
int32_t gelio_surrogate_predict(gelio_surrogate *s, const gelio_sim_params *sims, int32_t n,
                                double *ln_ratio, double *ln_std);

/* predict, then run the Monte Carlo (gelio_run with mc_opts, the sims'
 * own particle counts) for every simulation whose largest std over
 * [t_min, t_max] exceeds fallback_std and return its ratio there
 * (ln_std = 0, used_mc[i] = 1). */
int32_t gelio_surrogate_spectra(gelio_surrogate *s, const gelio_sim_params *sims, int32_t n,
                                const gelio_run_opts *mc_opts, double *ln_ratio, double *ln_std,
                                int32_t *used_mc);

/* Device time of the last predict / forward call (from the upload of its
 * inputs to its last kernel) and the GEMM FLOP it performed (rows padded to
 * the batch, first-layer K padded to 64): the surrogate's tensor roofline. */
int32_t gelio_surrogate_last_inference(gelio_surrogate *s, double *device_ms, double *flop);

/* Member m's FP32 parameters (GELIO_SURR_PARAMS floats), for persistence
 * and checks; set_params also clears that member's Adam state. */
int32_t gelio_surrogate_get_params(gelio_surrogate *s, int32_t member, float *params);
int32_t gelio_surrogate_set_params(gelio_surrogate *s, int32_t member, const float *params);

/* One forward pass of member m on normalised inputs x [n][7] -> y [n]. */
int32_t gelio_surrogate_forward(gelio_surrogate *s, int32_t member, const float *x, int32_t n, float *y);

/* Mean squared error and its gradient (GELIO_SURR_PARAMS floats) for member
 * m on x [n][7] and targets t [n], n <= batch_rows; no update. */
int32_t gelio_surrogate_gradient(gelio_surrogate *s, int32_t member, const float *x, const float *t,
                                 int32_t n, float *loss, float *grad);

#ifdef __cplusplus
}
#endif

#endif /* GELIO_H */
