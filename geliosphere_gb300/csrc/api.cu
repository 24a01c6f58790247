// C ABI of the GB300 Geliosphere engine (declared in include/gelio.h).
//
// One context owns the device buffers, a stream, CUDA events and the tuned
// launch shapes.  A run is a fixed, graph-capturable sequence on the stream:
//   memset control + histogram slices
//   k_prepare   (validate, derive per-simulation data, group sims by model,
//                particle prefix sums)
//   k_persistent<model>  for each model present (one launch for a whole batch)
//   k_reduce    (Neumaier sum of the slices -> gelio_spectra per simulation)
// The reference allocates and frees every buffer inside each
// prepareAndRunSimulation call (e.g. GeliosphereGpuModel.cpp:17-43) and
// synchronises three times per 4,096-particle chunk.
#include <cuda_runtime.h>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "gelio.h"
#include "alloc.cuh"
#include "kernels.cuh"

namespace gelio {

// ---------------------------------------------------------------------------
// Allocation hook (gelio_set_alloc_hook): consulted before every device and
// pinned-host allocation of the engine.
// ---------------------------------------------------------------------------
static std::atomic<gelio_alloc_hook> g_alloc_hook{nullptr};
static std::atomic<void *> g_alloc_user{nullptr};

static bool alloc_refused(int32_t kind, size_t bytes) {
  const gelio_alloc_hook h = g_alloc_hook.load();
  return h != nullptr && h(kind, (uint64_t)bytes, g_alloc_user.load()) != 0;
}

cudaError_t dev_malloc_raw(void **p, size_t bytes) {
  if (alloc_refused(GELIO_ALLOC_DEVICE, bytes)) { *p = nullptr; return cudaErrorMemoryAllocation; }
  return cudaMalloc(p, bytes);
}

cudaError_t pinned_malloc_raw(void **p, size_t bytes) {
  if (alloc_refused(GELIO_ALLOC_PINNED_HOST, bytes)) { *p = nullptr; return cudaErrorMemoryAllocation; }
  return cudaMallocHost(p, bytes);
}

cudaError_t fp_launch(bool, int, unsigned, unsigned, size_t, cudaStream_t, const KArgs &);
cudaError_t bp_launch(bool, int, unsigned, unsigned, size_t, cudaStream_t, const KArgs &);
cudaError_t solarprop_launch(bool, int, unsigned, unsigned, size_t, cudaStream_t, const KArgs &);
cudaError_t geliosphere_launch(bool, int, unsigned, unsigned, size_t, cudaStream_t, const KArgs &);
const void *fp_kernel(bool, int);
const void *bp_kernel(bool, int);
const void *solarprop_kernel(bool, int);
const void *geliosphere_kernel(bool, int);
cudaError_t fp_tables(const BinTables &);
cudaError_t bp_tables(const BinTables &);
cudaError_t solarprop_tables(const BinTables &);
cudaError_t geliosphere_tables(const BinTables &);

static cudaError_t launch_model(int m, bool persistent, int prec, unsigned grid, unsigned block,
                                size_t smem, cudaStream_t st, const KArgs &a) {
  switch (m) {
    case kModelFp: return fp_launch(persistent, prec, grid, block, smem, st, a);
    case kModelBp: return bp_launch(persistent, prec, grid, block, smem, st, a);
    case kModelSolarProp: return solarprop_launch(persistent, prec, grid, block, smem, st, a);
    default: return geliosphere_launch(persistent, prec, grid, block, smem, st, a);
  }
}
static const void *model_kernel(int m, bool persistent, int prec) {
  switch (m) {
    case kModelFp: return fp_kernel(persistent, prec);
    case kModelBp: return bp_kernel(persistent, prec);
    case kModelSolarProp: return solarprop_kernel(persistent, prec);
    default: return geliosphere_kernel(persistent, prec);
  }
}

// ---------------------------------------------------------------------------
// Parameter validation (host and device).
// ---------------------------------------------------------------------------
__host__ __device__ inline bool finite_pos(float x) { return x > 0.0f && x < 3.0e38f; }

__host__ __device__ inline int validate_params(const gelio_sim_params &p) {
  if (p.model < 0 || p.model > 3) return GELIO_ERR_INVALID_ARGUMENT;
  if (p.injection < 0 || p.injection > 4) return GELIO_ERR_INVALID_ARGUMENT;
  if (p.n_particles < 0) return GELIO_ERR_INVALID_ARGUMENT;
  if (!finite_pos(p.K0) || !finite_pos(p.V) || !finite_pos(p.dt)) return GELIO_ERR_INVALID_ARGUMENT;
  if (p.model != GELIO_MODEL_1D_FP && !finite_pos(p.r_injection)) return GELIO_ERR_INVALID_ARGUMENT;
  if (p.model >= GELIO_MODEL_2D_SOLARPROP) {
    if (!(p.theta_injection > 0.0f && p.theta_injection < 3.1416f)) return GELIO_ERR_INVALID_ARGUMENT;
    if (!(p.polarity == 1.0f || p.polarity == -1.0f)) return GELIO_ERR_INVALID_ARGUMENT;
    if (!(p.ratio >= 0.0f && p.ratio <= 1.0f)) return GELIO_ERR_INVALID_ARGUMENT;
    if (!(p.tilt >= 0.0f && p.tilt < 1.6f)) return GELIO_ERR_INVALID_ARGUMENT;
    if (p.model == GELIO_MODEL_2D_GELIOSPHERE && !(p.delta0 >= 0.0f && p.delta0 < 1.0f))
      return GELIO_ERR_INVALID_ARGUMENT;
  }
  if (p.injection == GELIO_INJ_REFERENCE_UNIFORM || p.injection == GELIO_INJ_CPU_UNIFORM) {
    if (!(p.injection_max >= 0.001f && p.injection_max < 1.0e6f)) return GELIO_ERR_INVALID_ARGUMENT;
  }
  if (p.injection == GELIO_INJ_LOG_GRID || p.injection == GELIO_INJ_LOG_UNIFORM) {
    if (!finite_pos(p.inj_min) || !finite_pos(p.inj_max) || !(p.inj_min <= p.inj_max))
      return GELIO_ERR_INVALID_ARGUMENT;
    if (p.injection == GELIO_INJ_LOG_GRID && (p.inj_points < 1 || p.inj_points > GELIO_GRID_MAX))
      return GELIO_ERR_INVALID_ARGUMENT;
  }
  if (p.grid_bins < 0 || p.grid_bins > GELIO_GRID_MAX) return GELIO_ERR_INVALID_ARGUMENT;
  if (p.grid_bins > 0 && !(finite_pos(p.grid_min) && p.grid_min < p.grid_max && p.grid_max < 3.0e38f))
    return GELIO_ERR_INVALID_ARGUMENT;
  return GELIO_OK;
}

// ---------------------------------------------------------------------------
// Device kernels of the run sequence.
// ---------------------------------------------------------------------------
__global__ void k_prepare(const gelio_sim_params *__restrict__ p, int n, SimDev *sims,
                          float *tables, Groups g, Control *ctl) {
  if (threadIdx.x == 0) ctl->t_start = globaltimer_ns();
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const gelio_sim_params q = p[i];
    const int err = validate_params(q);
    if (err != GELIO_OK) {
      atomicCAS(&ctl->status, 0u, (unsigned)err);
      atomicExch(&ctl->bad_sim, i);
    }
    SimDev s;
    s.K0 = q.K0; s.V = q.V; s.dt = q.dt; s.r_inj = q.r_injection; s.theta_inj = q.theta_injection;
    s.tilt = q.tilt; s.polarity = q.polarity; s.ratio = q.ratio; s.delta0 = q.delta0;
    s.injection_max = q.injection_max; s.inj_min = q.inj_min; s.inj_max = q.inj_max;
    s.model = q.model; s.injection = q.injection; s.inj_points = q.inj_points; s.flags = q.flags;
    s.key0 = (uint32_t)q.seed;
    s.key1 = (uint32_t)(q.seed >> 32);
    s.n_particles = q.n_particles;
    s.grid_is_points = 0;
    s.grid_bins = 0;
    s.grid_min = q.grid_min; s.grid_max = q.grid_max;
    s.grid_log_lo = 0.0; s.grid_inv_dlog = 0.0;
    if (q.grid_bins == 0 && q.injection == GELIO_INJ_LOG_GRID && q.model != GELIO_MODEL_1D_FP) {
      s.grid_is_points = 1;
      s.grid_bins = q.inj_points;
    } else if (q.grid_bins > 0) {
      s.grid_bins = q.grid_bins;
      s.grid_log_lo = log((double)q.grid_min);
      s.grid_inv_dlog = (double)q.grid_bins / (log((double)q.grid_max) - log((double)q.grid_min));
    }
    if (err == GELIO_OK && q.injection == GELIO_INJ_LOG_GRID) {
      const double lmin = log((double)q.inj_min), lmax = log((double)q.inj_max);
      const int np = q.inj_points;
      for (int k = 0; k < np; ++k) {
        const double f = (np > 1) ? (double)k / (double)(np - 1) : 0.0;
        tables[(size_t)i * GELIO_GRID_MAX + k] = (float)exp(lmin + f * (lmax - lmin));
      }
    }
    sims[i] = s;
  }
  __syncthreads();
  if (threadIdx.x < 4) {
    const int m = threadIdx.x;
    int c = 0;
    unsigned long long acc = 0;
    int *idx = g.sim_idx + (size_t)m * n;
    unsigned long long *pre = g.prefix + (size_t)m * (n + 1);
    for (int i = 0; i < n; ++i) {
      if (p[i].model == m) {
        idx[c] = i;
        pre[c] = acc;
        acc += (unsigned long long)(p[i].n_particles > 0 ? p[i].n_particles : 0);
        ++c;
      }
    }
    pre[c] = acc;
    ctl->group_count[m] = (unsigned long long)c;
  }
}

// out[s][i] = Neumaier sum over slices of part[slice][s][i].
__global__ void k_reduce(const double *__restrict__ part, int n_slices, long long n_total,
                         double *__restrict__ out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_total) return;
  double s = 0.0, c = 0.0;
  for (int j = 0; j < n_slices; ++j) {
    const double x = part[(size_t)j * n_total + i];
    const double t = s + x;
    if (fabs(s) >= fabs(x)) c += (s - t) + x;
    else c += (x - t) + s;
    s = t;
  }
  out[i] = s + c;
}

// Evaluate log.dat rows (gelio_evaluate): one thread per row into slices.
__global__ void k_evaluate(const double *__restrict__ rows, long long n_rows, int n_cols,
                           int model, int n_slices, double *part) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_rows) return;
  const double *row = rows + (size_t)i * n_cols;
  double *slice = part + (size_t)(blockIdx.x % n_slices) * kSpecDoubles;
  Contribution C;
  const double one = 1.0;
  if (model >= kModelSolarProp) {
    eval_2d(round6(row[0]), round6(row[1]), c_tables, C);
    const double w[3] = {C.w[0], C.w[1], C.w[2]};
    if (C.b_sp) {
      atomicAdd(&slice[kOffSpWeber + C.b_sp], w[0]);
      atomicAdd(&slice[kOffSpJgr + C.b_sp], w[1]);
      atomicAdd(&slice[kOffSpBurger + C.b_sp], w[2]);
      atomicAdd(&slice[kOffSpWeber2 + C.b_sp], w[0] * w[0]);
      atomicAdd(&slice[kOffSpJgr2 + C.b_sp], w[1] * w[1]);
      atomicAdd(&slice[kOffSpBurger2 + C.b_sp], w[2] * w[2]);
      atomicAdd(&slice[kOffSpN + C.b_sp], one);
    }
    if (C.b_uly) {
      atomicAdd(&slice[kOffUlyW + C.b_uly], w[2]);
      atomicAdd(&slice[kOffUlyW2 + C.b_uly], w[2] * w[2]);
      atomicAdd(&slice[kOffUlyN + C.b_uly], one);
    }
    if (C.b_ams) {
      atomicAdd(&slice[kOffAmsW + C.b_ams], w[2]);
      atomicAdd(&slice[kOffAmsW2 + C.b_ams], w[2] * w[2]);
      atomicAdd(&slice[kOffAmsN + C.b_ams], one);
    }
  } else {
    if (model == kModelBp) {
      eval_bp(round6(row[1]), round6(row[0]), c_tables, C);
    } else {
      double T1;
      eval_fp(round6(row[0]), round6(row[1]), round6(row[2]), round6(row[4]), c_tables, C, T1);
    }
    const double w = C.w[0];
    if (C.b_log >= 0) {
      atomicAdd(&slice[kOffLogW + C.b_log], w);
      atomicAdd(&slice[kOffLogW2 + C.b_log], w * w);
      atomicAdd(&slice[kOffLogN + C.b_log], one);
    }
    if (C.b_e2) { atomicAdd(&slice[kOffE2W + C.b_e2 - 1], w); atomicAdd(&slice[kOffE2W2 + C.b_e2 - 1], w * w); atomicAdd(&slice[kOffE2N + C.b_e2 - 1], one); }
    if (C.b_e3) { atomicAdd(&slice[kOffE3W + C.b_e3 - 1], w); atomicAdd(&slice[kOffE3W2 + C.b_e3 - 1], w * w); atomicAdd(&slice[kOffE3N + C.b_e3 - 1], one); }
    if (C.b_e4) { atomicAdd(&slice[kOffE4W + C.b_e4 - 1], w); atomicAdd(&slice[kOffE4W2 + C.b_e4 - 1], w * w); atomicAdd(&slice[kOffE4N + C.b_e4 - 1], one); }
  }
  atomicAdd(&slice[kOffNRecords], one);
}

// Throughput probes for the roofline denominators.
__global__ void k_peak_fma(float *out, int iters) {
  float a0 = threadIdx.x * 1e-3f, a1 = a0 + 1.f, a2 = a0 + 2.f, a3 = a0 + 3.f;
  float a4 = a0 + 4.f, a5 = a0 + 5.f, a6 = a0 + 6.f, a7 = a0 + 7.f;
  const float b = 0.999999f, c = 1e-7f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      a0 = fmaf(a0, b, c); a1 = fmaf(a1, b, c); a2 = fmaf(a2, b, c); a3 = fmaf(a3, b, c);
      a4 = fmaf(a4, b, c); a5 = fmaf(a5, b, c); a6 = fmaf(a6, b, c); a7 = fmaf(a7, b, c);
    }
  }
  const float s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
  if (s == 123.456f) out[0] = s;
}

__global__ void k_peak_xu(float *out, int iters) {
  float a0 = threadIdx.x * 1e-6f, a1 = a0 + 0.1f, a2 = a0 + 0.2f, a3 = a0 + 0.3f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      asm volatile("ex2.approx.ftz.f32 %0, %0;" : "+f"(a0));
      asm volatile("ex2.approx.ftz.f32 %0, %0;" : "+f"(a1));
      asm volatile("ex2.approx.ftz.f32 %0, %0;" : "+f"(a2));
      asm volatile("ex2.approx.ftz.f32 %0, %0;" : "+f"(a3));
    }
  }
  const float s = a0 + a1 + a2 + a3;
  if (s == 123.456f) out[0] = s;
}

// Launch wrappers for the allocation-free entry point (noalloc.cu), which
// runs the same sequence on its own static scratch.
cudaError_t launch_prepare(const gelio_sim_params *p, int n, SimDev *sims, float *tables, Groups g,
                           Control *ctl, cudaStream_t st) {
  k_prepare<<<1, 256, 0, st>>>(p, n, sims, tables, g, ctl);
  return cudaGetLastError();
}
cudaError_t launch_reduce(const double *part, int n_slices, long long n_total, double *out,
                          cudaStream_t st) {
  k_reduce<<<(unsigned)((n_total + 255) / 256), 256, 0, st>>>(part, n_slices, n_total, out);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Host tables from the reference definitions.
// ---------------------------------------------------------------------------
void build_tables(BinTables &t) {
  static const double sp[32] = {0, 0.01, 0.015, 0.0225, 0.03375, 0.050625,
    0.0759375, 0.113906, 0.170859, 0.256289, 0.384434, 0.57665,
    0.864976, 1.29746, 1.9462, 2.91929, 4.37894, 6.56841, 9.85261,
    14.7789, 22.1684, 33.2526, 49.8789, 74.8183, 112.227, 168.341,
    252.512, 378.768, 568.151, 852.227, 1278.34, 0.0};
  static const double uly[4] = {0, 0.125, 0.250, 2.0};
  static const double ams[72] = {4.924000e-01, 6.207000e-01, 7.637000e-01, 9.252000e-01, 1.105000e+00,
    1.303000e+00, 1.523000e+00, 1.765000e+00, 2.034000e+00, 2.329000e+00, 2.652000e+00, 3.005000e+00,
    3.390000e+00, 3.810000e+00, 4.272000e+00, 4.774000e+00, 5.317000e+00, 5.906000e+00, 6.546000e+00,
    7.236000e+00, 7.981000e+00, 8.787000e+00, 9.653000e+00, 1.060000e+01, 1.160000e+01, 1.264000e+01,
    1.379000e+01, 1.504000e+01, 1.639000e+01, 1.784000e+01, 1.938000e+01, 2.103000e+01, 2.283000e+01,
    2.478000e+01, 2.683000e+01, 2.903000e+01, 3.138000e+01, 3.387000e+01, 3.657000e+01, 3.947000e+01,
    4.257000e+01, 4.587000e+01, 4.942000e+01, 5.322000e+01, 5.727000e+01, 6.162000e+01, 6.632000e+01,
    7.137000e+01, 7.677000e+01, 8.257000e+01, 8.882000e+01, 9.557000e+01, 1.031000e+02, 1.111000e+02,
    1.196000e+02, 1.291000e+02, 1.401000e+02, 1.526000e+02, 1.666000e+02, 1.826000e+02, 2.006000e+02,
    2.211000e+02, 2.451000e+02, 2.741000e+02, 3.096000e+02, 3.536000e+02, 4.091000e+02, 4.821000e+02,
    5.831000e+02, 7.316000e+02, 9.751000e+02, 1.464000e+03};
  memcpy(t.sp, sp, sizeof(t.sp));
  memcpy(t.uly, uly, sizeof(t.uly));
  memcpy(t.ams, ams, sizeof(t.ams));
  // OneDimensionBpResults.cpp:25-31 with NT = 80, Tmin = 0.01, Tmax = 200.
  const double dlT = log10(200.0 / 0.01) / 80;
  const double X = log10(200.0);
  for (int i = 0; i < 80; i++) t.bp_log[i] = exp((X - (i * dlT)) * log(10.0));
  t.bp_log[80] = 0.0;
  // OneDimensionFpResults.cpp:24-27.
  for (int i = 0; i < 25; i++) t.fp_log[i] = exp((((i + 1) / 5.0) - 3.0) * log(10));
  // getSolarPropInjection energies 0.01 * 1.5^k, rounded once to FP32.
  for (int k = 0; k < 30; ++k) t.sp30[k] = (float)(0.01 * pow(1.5, k));
}

}  // namespace gelio

using namespace gelio;

// ---------------------------------------------------------------------------
// Context.
// ---------------------------------------------------------------------------
struct Tuned {
  int block = 256, blocks_per_sm = 0, refill = 0, compact = 1;
};

struct gelio_ctx {
  int device = 0;
  int sm_count = 0;
  int max_smem_optin = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev_k0 = nullptr, ev_k1 = nullptr;
  std::mutex mu;
  // device buffers
  int cap_sims = 0;
  gelio_sim_params *d_params = nullptr;
  SimDev *d_sims = nullptr;
  float *d_tables = nullptr;
  int *d_gsim = nullptr;
  unsigned long long *d_gpre = nullptr;
  Control *d_ctl = nullptr;
  double *d_part = nullptr;
  size_t part_bytes = 0;
  double *d_out = nullptr;
  size_t out_bytes = 0;
  gelio_exit_record *d_rec = nullptr;
  size_t rec_cap = 0;
  gelio_trajectory *d_traj = nullptr;
  size_t traj_cap = 0;
  double *d_rows = nullptr;
  size_t rows_bytes = 0;
  // pinned staging
  gelio_sim_params *h_params = nullptr;
  int h_params_cap = 0;
  gelio_spectra *h_out = nullptr;      // pinned staging of graph-mode outputs
  int h_out_cap = 0;
  Control *h_ctl = nullptr;
  // graph cache
  cudaGraphExec_t graph = nullptr;
  unsigned long long graph_key[8] = {0};
  const void *graph_bufs[12] = {};     // buffer addresses the cached graph was captured with
  // tuning and last run
  Tuned tuned[4][2];
  int occ_cache[4][3][8][5] = {};   // [model][kernel variant][block/32 - 1][smem slots]
  gelio_run_stats last{};
  int last_n_slices = 1;
  bool last_timed = false;
};

// Text of the last CUDA failure seen by this thread (gelio_last_error).
static thread_local char g_last_error[256] = "";

void gelio::note_cuda_error(cudaError_t e, const char *file, int line) {
  snprintf(g_last_error, sizeof(g_last_error), "%s (%s) at %s:%d", cudaGetErrorName(e), cudaGetErrorString(e), file,
           line);
}

static int map_cuda_at(cudaError_t e, int line) {
  if (e != cudaSuccess) gelio::note_cuda_error(e, "api.cu", line);
  if (e == cudaSuccess) return GELIO_OK;
  if (e == cudaErrorMemoryAllocation) return GELIO_ERR_OUT_OF_MEMORY;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver || e == cudaErrorInvalidDevice)
    return GELIO_ERR_NO_DEVICE;
  return GELIO_ERR_CUDA;
}
#define map_cuda(e) map_cuda_at((e), __LINE__)

#define GELIO_TRY(expr)                        \
  do {                                         \
    cudaError_t e_ = (expr);                   \
    if (e_ != cudaSuccess) return map_cuda(e_); \
  } while (0)

// Grow a device buffer: the larger buffer is allocated before the old one is
// released, so a refused or failed allocation leaves the context with the
// buffers (and the cached graph) it had.
template <class T>
static cudaError_t grow(T *&ptr, size_t &cap_bytes, size_t need_bytes) {
  if (need_bytes <= cap_bytes && ptr != nullptr) return cudaSuccess;
  T *fresh = nullptr;
  cudaError_t e = dev_malloc(&fresh, need_bytes);
  if (e != cudaSuccess) return e;
  if (ptr) cudaFree(ptr);
  ptr = fresh;
  cap_bytes = need_bytes;
  return cudaSuccess;
}

// Pinned host staging, grown the same way.
template <class T>
static cudaError_t grow_pinned(T *&ptr, int &cap, int need) {
  if (need <= cap && ptr != nullptr) return cudaSuccess;
  T *fresh = nullptr;
  cudaError_t e = pinned_malloc(&fresh, sizeof(T) * (size_t)need);
  if (e != cudaSuccess) return e;
  if (ptr) cudaFreeHost(ptr);
  ptr = fresh;
  cap = need;
  return cudaSuccess;
}

static void release(gelio_ctx *c) {
  if (c->graph) cudaGraphExecDestroy(c->graph);
  cudaFree(c->d_params); cudaFree(c->d_sims); cudaFree(c->d_tables); cudaFree(c->d_gsim);
  cudaFree(c->d_gpre); cudaFree(c->d_ctl); cudaFree(c->d_part); cudaFree(c->d_out);
  cudaFree(c->d_rec); cudaFree(c->d_traj); cudaFree(c->d_rows);
  if (c->h_params) cudaFreeHost(c->h_params);
  if (c->h_out) cudaFreeHost(c->h_out);
  if (c->h_ctl) cudaFreeHost(c->h_ctl);
  if (c->ev_k0) cudaEventDestroy(c->ev_k0);
  if (c->ev_k1) cudaEventDestroy(c->ev_k1);
  if (c->stream) cudaStreamDestroy(c->stream);
}

// Per-simulation buffers for n simulations: all five new buffers are
// allocated before the old ones are released, so a refused or failed
// allocation leaves the context as it was.
static int ensure_sims(gelio_ctx *c, int n) {
  if (n <= c->cap_sims) return GELIO_OK;
  int cap = 16;
  while (cap < n) cap *= 2;
  gelio_sim_params *params = nullptr;
  SimDev *sims = nullptr;
  float *tables = nullptr;
  int *gsim = nullptr;
  unsigned long long *gpre = nullptr;
  cudaError_t e = dev_malloc(&params, sizeof(gelio_sim_params) * cap);
  if (e == cudaSuccess) e = dev_malloc(&sims, sizeof(SimDev) * cap);
  if (e == cudaSuccess) e = dev_malloc(&tables, sizeof(float) * GELIO_GRID_MAX * cap);
  if (e == cudaSuccess) e = dev_malloc(&gsim, sizeof(int) * 4 * cap);
  if (e == cudaSuccess) e = dev_malloc(&gpre, sizeof(unsigned long long) * 4 * (cap + 1));
  if (e != cudaSuccess) {
    cudaFree(params); cudaFree(sims); cudaFree(tables); cudaFree(gsim); cudaFree(gpre);
    return map_cuda(e);
  }
  cudaFree(c->d_params); cudaFree(c->d_sims); cudaFree(c->d_tables); cudaFree(c->d_gsim); cudaFree(c->d_gpre);
  c->d_params = params; c->d_sims = sims; c->d_tables = tables; c->d_gsim = gsim; c->d_gpre = gpre;
  c->cap_sims = cap;
  if (c->graph) { cudaGraphExecDestroy(c->graph); c->graph = nullptr; }
  return GELIO_OK;
}

static int choose_slices(int n_sims) {
  // keep the slice buffer near 64 MB at most
  const double per = (double)n_sims * kSpecDoubles * 8.0;
  int s = (int)(64.0e6 / per);
  if (s > 16) s = 16;
  if (s < 1) s = 1;
  return s;
}

static int default_refill(int model) { return (model == kModelFp) ? 4 : 16; }

struct LaunchShape {
  unsigned grid, block;
  size_t smem;
  int smem_slots;
  int refill;
  int blocks_per_sm;
};

// Kernel variant of a run: 1 = FP64, 2 = FP32 compact (<= 85 registers), 0 = FP32.
static int kernel_variant(const gelio_ctx *c, int model, const gelio_run_opts *o) {
  if (o && o->precision == GELIO_PREC_FP64) return 1;
  const int compact = (o && o->compact > 0) ? o->compact : c->tuned[model][0].compact;
  return compact == 2 ? 2 : 0;
}

static int shape_for(gelio_ctx *c, int model, int prec, int n_in_group_hint, const gelio_run_opts *o,
                     LaunchShape &s) {
  const Tuned &t = c->tuned[model][prec == 1 ? 1 : 0];
  s.block = (o && o->block_size > 0) ? (unsigned)o->block_size : (unsigned)t.block;
  if (s.block % 32 != 0 || s.block > 256 || s.block < 32) return GELIO_ERR_INVALID_ARGUMENT;
  s.refill = (o && o->refill_interval > 0) ? o->refill_interval : (t.refill > 0 ? t.refill : default_refill(model));
  if (s.refill % 4 != 0 || s.refill > 4096) return GELIO_ERR_INVALID_ARGUMENT;
  const int win_doubles = (model >= kModelSolarProp) ? (kWinHi - kWin2DLo) : (kWinHi - kWin1DLo);
  const size_t per_slot = (size_t)win_doubles * 8;
  const size_t qbytes = (size_t)(s.block / 32) * (kQueue * sizeof(QEnt) + sizeof(int));
  // occupancy per (model, precision, block, smem slots), cached: no CUDA
  // call that a stream capture would reject happens while enqueueing
  const int bi = (int)s.block / 32 - 1;
  const void *kfn = model_kernel(model, true, prec);
  auto occupancy = [&](int slots_, int &occ_) -> int {
    int &cached = c->occ_cache[model][prec][bi][slots_];
    if (cached == 0) {
      int occ = 0;
      GELIO_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kfn, (int)s.block,
                                                              (size_t)slots_ * per_slot + qbytes));
      cached = (occ < 1) ? -1 : occ;
    }
    occ_ = cached;
    return GELIO_OK;
  };
  // shared-memory histograms for up to 4 simulations (2D) / 1 simulation
  // (1D) of the launch, but never at the cost of resident warps: the slot
  // count keeps the occupancy that the registers allow
  int occ0 = 0;
  int rc0 = occupancy(0, occ0);
  if (rc0 != GELIO_OK) return rc0;
  if (occ0 < 1) return GELIO_ERR_UNSUPPORTED;
  const int max_slots = (model >= kModelSolarProp) ? 4 : 1;
  int slots = (n_in_group_hint >= 1 && n_in_group_hint <= max_slots) ? n_in_group_hint : 0;
  while (slots > 0) {
    if ((size_t)slots * per_slot + qbytes <= (size_t)c->max_smem_optin) {
      int occs = 0;
      rc0 = occupancy(slots, occs);
      if (rc0 != GELIO_OK) return rc0;
      if (occs >= occ0) break;
    }
    slots = (slots == n_in_group_hint) ? 0 : slots - 1;   // all of the group's sims or none
  }
  s.smem_slots = slots;
  s.smem = (size_t)slots * per_slot + qbytes;
  int occ = 0;
  rc0 = occupancy(slots, occ);
  if (rc0 != GELIO_OK) return rc0;
  if (occ < 1) return GELIO_ERR_UNSUPPORTED;
  int bps = (o && o->blocks_per_sm > 0) ? o->blocks_per_sm : (t.blocks_per_sm > 0 ? t.blocks_per_sm : occ);
  if (bps > occ) bps = occ;
  s.blocks_per_sm = bps;
  s.grid = (unsigned)(c->sm_count * bps);
  return GELIO_OK;
}

extern "C" {

const char *gelio_status_string(int32_t s) {
  switch (s) {
    case GELIO_OK: return "ok";
    case GELIO_ERR_INVALID_ARGUMENT: return "invalid argument";
    case GELIO_ERR_NO_DEVICE: return "no usable CUDA device";
    case GELIO_ERR_CUDA: return "CUDA error";
    case GELIO_ERR_OUT_OF_MEMORY: return "out of device memory";
    case GELIO_ERR_TIMEOUT: return "device watchdog time limit reached";
    case GELIO_ERR_UNSUPPORTED: return "unsupported configuration";
    case GELIO_ERR_NOT_TRAINED: return "surrogate not trained";
    case GELIO_WARN_RECORDS_TRUNCATED: return "exit records truncated to record_capacity";
    case GELIO_WARN_STEP_CAP: return "some trajectories reached max_steps_per_particle";
    default: return "unknown status";
  }
}

int32_t gelio_abi_version(void) { return GELIO_ABI_VERSION; }

const char *gelio_last_error(void) { return g_last_error; }

int32_t gelio_create(gelio_ctx **out, int32_t device) {
  if (out == nullptr) return GELIO_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) return GELIO_ERR_NO_DEVICE;
  if (device < 0 || device >= n) return GELIO_ERR_INVALID_ARGUMENT;
  gelio_ctx *c = new (std::nothrow) gelio_ctx();
  if (!c) return GELIO_ERR_OUT_OF_MEMORY;
  c->device = device;
  int rc = GELIO_OK;
  do {
    if ((e = cudaSetDevice(device)) != cudaSuccess) { rc = map_cuda(e); break; }
    cudaDeviceProp prop;
    if ((e = cudaGetDeviceProperties(&prop, device)) != cudaSuccess) { rc = map_cuda(e); break; }
    if (prop.major < 10) { rc = GELIO_ERR_UNSUPPORTED; break; }
    c->sm_count = prop.multiProcessorCount;
    c->max_smem_optin = (int)prop.sharedMemPerBlockOptin;
    if ((e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking)) != cudaSuccess) { rc = map_cuda(e); break; }
    if ((e = cudaEventCreate(&c->ev_k0)) != cudaSuccess) { rc = map_cuda(e); break; }
    if ((e = cudaEventCreate(&c->ev_k1)) != cudaSuccess) { rc = map_cuda(e); break; }
    if ((e = dev_malloc(&c->d_ctl, sizeof(Control))) != cudaSuccess) { rc = map_cuda(e); break; }
    if ((e = pinned_malloc(&c->h_ctl, sizeof(Control))) != cudaSuccess) { rc = map_cuda(e); break; }
    BinTables t;
    build_tables(t);
    if ((e = fp_tables(t)) != cudaSuccess || (e = bp_tables(t)) != cudaSuccess ||
        (e = solarprop_tables(t)) != cudaSuccess || (e = geliosphere_tables(t)) != cudaSuccess ||
        (e = set_tables_tu(t)) != cudaSuccess) { rc = map_cuda(e); break; }
    // dynamic shared memory of the persistent kernels: opt in once, up to the
    // largest histogram window (4 simulations of a 2D model)
    for (int m = 0; m < 4 && rc == GELIO_OK; ++m)
      for (int p = 0; p < 3 && rc == GELIO_OK; ++p) {
        const int win = (m >= kModelSolarProp) ? 4 * (kWinHi - kWin2DLo) : (kWinHi - kWin1DLo);
        const int need = win * 8 + 8 * (kQueue * (int)sizeof(QEnt) + (int)sizeof(int));
        const int bytes = need <= c->max_smem_optin ? need : c->max_smem_optin;
        e = cudaFuncSetAttribute(model_kernel(m, true, p), cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        if (e != cudaSuccess) rc = map_cuda(e);
      }
    if (rc != GELIO_OK) break;
    rc = ensure_sims(c, 16);
  } while (0);
  if (rc != GELIO_OK) {
    release(c);
    delete c;
    return rc;
  }
  *out = c;
  return GELIO_OK;
}

int32_t gelio_destroy(gelio_ctx *c) {
  if (!c) return GELIO_ERR_INVALID_ARGUMENT;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  release(c);
  delete c;
  return GELIO_OK;
}

}  // extern "C"

// Enqueue one run on `st`.  d_params already holds n sims.  model_mask /
// counts are known for host runs (mask 0 = unknown: launch all four models).
static int enqueue_run(gelio_ctx *c, int n, const gelio_run_opts *o, double *d_out, cudaStream_t st,
                       unsigned model_mask, const int *model_counts, gelio_exit_record *d_rec,
                       size_t rec_cap, bool timed) {
  const int prec = (o && o->precision == GELIO_PREC_FP64) ? 1 : 0;
  const int n_slices = choose_slices(n);
  (void)cudaGetLastError();   // launch checks below must see only this run's errors
  GELIO_TRY(grow(c->d_part, c->part_bytes, (size_t)n_slices * n * kSpecDoubles * 8));
  GELIO_TRY(cudaMemsetAsync(c->d_ctl, 0, sizeof(Control), st));
  GELIO_TRY(cudaMemsetAsync(c->d_part, 0, (size_t)n_slices * n * kSpecDoubles * 8, st));
  Groups g{c->d_gsim, c->d_gpre};
  k_prepare<<<1, 256, 0, st>>>(c->d_params, n, c->d_sims, c->d_tables, g, c->d_ctl);
  GELIO_TRY(cudaGetLastError());
  KArgs a{};
  a.sims = c->d_sims;
  a.inj_tables = c->d_tables;
  a.groups = g;
  a.n_sims = n;
  a.n_slices = n_slices;
  a.part = c->d_part;
  a.ctl = c->d_ctl;
  a.records = d_rec;
  a.record_capacity = rec_cap;
  unsigned long long ms = (o && o->max_steps_per_particle) ? o->max_steps_per_particle : 100000000ull;
  if (ms > 0xfffffff0ull) ms = 0xfffffff0ull;
  a.max_steps = ms;
  a.time_limit_ns = (o && o->time_limit_s > 0.0) ? (unsigned long long)(o->time_limit_s * 1e9) : 0ull;
  if (timed) GELIO_TRY(cudaEventRecord(c->ev_k0, st));
  LaunchShape first{};
  int variant = prec;
  bool have_first = false;
  for (int m = 0; m < 4; ++m) {
    if (model_mask && !(model_mask & (1u << m))) continue;
    const bool plain = o && o->plain;
    if (plain) {
      // one launch per simulation of this model, one thread per particle
      if (!model_counts) return GELIO_ERR_UNSUPPORTED;
      for (int s = 0; s < n; ++s) {
        if (c->h_params[s].model != m || c->h_params[s].n_particles <= 0) continue;
        const unsigned block = (o->block_size > 0) ? (unsigned)o->block_size : 256u;
        const unsigned long long cnt = (unsigned long long)c->h_params[s].n_particles;
        a.plain_sim = s;
        a.plain_first = 0;
        a.plain_count = cnt;
        a.replay = nullptr;
        const unsigned long long grid = (cnt + block - 1) / block;
        if (grid > 0x7fffffffull) return GELIO_ERR_INVALID_ARGUMENT;
        GELIO_TRY(launch_model(m, false, prec, (unsigned)grid, block, 0, st, a));
        if (!have_first) { first = LaunchShape{(unsigned)grid, block, 0, 0, 0, 0}; have_first = true; }
      }
      continue;
    }
    LaunchShape s;
    const int hint = model_counts ? model_counts[m] : n;
    variant = kernel_variant(c, m, o);
    int rc = shape_for(c, m, variant, hint, o, s);
    if (rc != GELIO_OK) return rc;
    a.smem_slots = s.smem_slots;
    a.refill = s.refill;
    GELIO_TRY(launch_model(m, true, variant, s.grid, s.block, s.smem, st, a));
    if (!have_first) { first = s; have_first = true; }
  }
  if (timed) GELIO_TRY(cudaEventRecord(c->ev_k1, st));
  const long long total = (long long)n * kSpecDoubles;
  k_reduce<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(c->d_part, n_slices, total, d_out);
  GELIO_TRY(cudaGetLastError());
  GELIO_TRY(cudaMemcpyAsync(c->h_ctl, c->d_ctl, sizeof(Control), cudaMemcpyDeviceToHost, st));
  c->last.block_size = (int)first.block;
  c->last.grid_size = (int)first.grid;
  c->last.blocks_per_sm = first.blocks_per_sm;
  c->last.refill_interval = first.refill;
  c->last_n_slices = n_slices;
  c->last_timed = timed;
  return GELIO_OK;
}

static int check_opts(const gelio_run_opts *o) {
  if (!o) return GELIO_OK;
  if (o->precision != GELIO_PREC_FP32 && o->precision != GELIO_PREC_FP64) return GELIO_ERR_INVALID_ARGUMENT;
  if (o->block_size < 0 || o->blocks_per_sm < 0 || o->refill_interval < 0) return GELIO_ERR_INVALID_ARGUMENT;
  if (o->time_limit_s < 0.0 || !(o->time_limit_s == o->time_limit_s)) return GELIO_ERR_INVALID_ARGUMENT;
  if (o->record_capacity < 0 || (o->record_capacity > 0 && o->records == nullptr)) return GELIO_ERR_INVALID_ARGUMENT;
  return GELIO_OK;
}

extern "C" {

int32_t gelio_run(gelio_ctx *c, const gelio_sim_params *sims, int32_t n, const gelio_run_opts *o,
                  gelio_spectra *out, gelio_run_stats *stats) {
  const auto t0 = std::chrono::steady_clock::now();
  if (!c || (n > 0 && (!sims || !out)) || n < 0 || n > kMaxSims) return GELIO_ERR_INVALID_ARGUMENT;
  int rc = check_opts(o);
  if (rc != GELIO_OK) return rc;
  for (int i = 0; i < n; ++i)
    if ((rc = validate_params(sims[i])) != GELIO_OK) return rc;
  std::lock_guard<std::mutex> lock(c->mu);
  GELIO_TRY(cudaSetDevice(c->device));
  if (stats) memset(stats, 0, sizeof(*stats));
  if (n == 0) return GELIO_OK;
  if ((rc = ensure_sims(c, n)) != GELIO_OK) return rc;
  if (n > c->h_params_cap) GELIO_TRY(grow_pinned(c->h_params, c->h_params_cap, c->cap_sims));
  memcpy(c->h_params, sims, sizeof(gelio_sim_params) * n);
  unsigned mask = 0;
  int counts[4] = {0, 0, 0, 0};
  for (int i = 0; i < n; ++i) { mask |= 1u << sims[i].model; counts[sims[i].model]++; }
  GELIO_TRY(grow(c->d_out, c->out_bytes, (size_t)n * sizeof(gelio_spectra)));
  size_t rec_cap = 0;
  if (o && o->record_capacity > 0) {
    rec_cap = (size_t)o->record_capacity;
    size_t bytes = c->rec_cap * sizeof(gelio_exit_record);
    GELIO_TRY(grow(c->d_rec, bytes, rec_cap * sizeof(gelio_exit_record)));
    c->rec_cap = rec_cap;
  }
  cudaStream_t st = c->stream;
  const bool graph = o && o->use_graph && !(o->plain);
  const unsigned long long key[8] = {(unsigned long long)n, mask,
    (unsigned long long)(o ? o->precision : 0) | ((unsigned long long)(o ? o->compact : 0) << 8),
    (unsigned long long)(o ? o->block_size : 0) << 32 | (unsigned)(o ? o->blocks_per_sm : 0),
    (unsigned long long)(o ? o->refill_interval : 0), (unsigned long long)rec_cap,
    (unsigned long long)(o ? o->max_steps_per_particle : 0),
    (unsigned long long)((o ? o->time_limit_s : 0.0) * 1e9)};
  if (graph && n > c->h_out_cap) GELIO_TRY(grow_pinned(c->h_out, c->h_out_cap, c->cap_sims));
  if (graph) {
    // graphs copy through pinned staging (pageable host memory cannot be a
    // memcpy node); the staging pointer is fixed, so the graph is reusable
    // buffers the run grows lazily are grown here: no allocation may happen
    // while the stream is being captured
    GELIO_TRY(grow(c->d_part, c->part_bytes, (size_t)choose_slices(n) * n * kSpecDoubles * 8));
    // a cached graph holds the addresses it was captured with: any buffer
    // regrown since (by a run of another size, or after a refused
    // allocation) makes it stale
    const void *bufs[12] = {c->d_params, c->d_sims, c->d_tables, c->d_gsim, c->d_gpre, c->d_ctl,
                            c->d_part, c->d_out, c->d_rec, c->h_params, c->h_out, c->h_ctl};
    const bool hit = c->graph && memcmp(key, c->graph_key, sizeof(key)) == 0 &&
                     memcmp(bufs, c->graph_bufs, sizeof(bufs)) == 0;
    if (!hit) {
      if (c->graph) { cudaGraphExecDestroy(c->graph); c->graph = nullptr; }
      cudaGraph_t gr;
      GELIO_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
      cudaError_t e = cudaMemcpyAsync(c->d_params, c->h_params, sizeof(gelio_sim_params) * n,
                                      cudaMemcpyHostToDevice, st);
      int erc = (e == cudaSuccess) ? enqueue_run(c, n, o, c->d_out, st, mask, counts, rec_cap ? c->d_rec : nullptr, rec_cap, true)
                                   : map_cuda(e);
      if (erc == GELIO_OK) {
        e = cudaMemcpyAsync(c->h_out, c->d_out, sizeof(gelio_spectra) * n, cudaMemcpyDeviceToHost, st);
        if (e != cudaSuccess) erc = map_cuda(e);
      }
      cudaError_t ee = cudaStreamEndCapture(st, &gr);
      if (erc != GELIO_OK) { if (ee == cudaSuccess) cudaGraphDestroy(gr); return erc; }
      GELIO_TRY(ee);
      e = cudaGraphInstantiate(&c->graph, gr, 0);
      cudaGraphDestroy(gr);
      GELIO_TRY(e);
      memcpy(c->graph_key, key, sizeof(key));
      memcpy(c->graph_bufs, bufs, sizeof(bufs));
    }
    GELIO_TRY(cudaGraphLaunch(c->graph, st));
  } else {
    GELIO_TRY(cudaMemcpyAsync(c->d_params, c->h_params, sizeof(gelio_sim_params) * n, cudaMemcpyHostToDevice, st));
    rc = enqueue_run(c, n, o, c->d_out, st, mask, counts, rec_cap ? c->d_rec : nullptr, rec_cap, true);
    if (rc != GELIO_OK) { cudaStreamSynchronize(st); return rc; }
    GELIO_TRY(cudaMemcpyAsync(out, c->d_out, sizeof(gelio_spectra) * n, cudaMemcpyDeviceToHost, st));
  }
  GELIO_TRY(cudaStreamSynchronize(st));
  if (graph) memcpy(out, c->h_out, sizeof(gelio_spectra) * n);
  const Control &h = *c->h_ctl;
  if (h.status != 0) return (int)h.status;
  int64_t stored = 0;
  if (rec_cap) {
    stored = (int64_t)((h.rec_count < rec_cap) ? h.rec_count : rec_cap);
    if (stored > 0)
      GELIO_TRY(cudaMemcpy(o->records, c->d_rec, sizeof(gelio_exit_record) * stored, cudaMemcpyDeviceToHost));
  }
  gelio_run_stats s{};
  for (int i = 0; i < n; ++i) {
    s.n_particles += (int64_t)out[i].n_particles;
    s.n_records += (int64_t)out[i].n_records;
    s.n_steps += (int64_t)out[i].n_steps;
    s.n_lost += (int64_t)out[i].n_lost;
    s.n_step_capped += (int64_t)out[i].n_step_capped;
  }
  s.n_records_stored = stored;
  s.n_records_dropped = (int64_t)h.rec_dropped;
  float kms = 0.f;
  if (cudaEventElapsedTime(&kms, c->ev_k0, c->ev_k1) != cudaSuccess) {
    kms = 0.f;                  // e.g. events replayed from a graph: no kernel time
    (void)cudaGetLastError();
  }
  s.kernel_ms = kms;
  s.total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  s.block_size = c->last.block_size;
  s.grid_size = c->last.grid_size;
  s.blocks_per_sm = c->last.blocks_per_sm;
  s.refill_interval = c->last.refill_interval;
  c->last = s;
  if (stats) *stats = s;
  if (s.n_records_dropped > 0) return GELIO_WARN_RECORDS_TRUNCATED;
  if (s.n_step_capped > 0) return GELIO_WARN_STEP_CAP;
  return GELIO_OK;
}

int32_t gelio_run_async(gelio_ctx *c, const gelio_sim_params *d_sims, int32_t n, const gelio_run_opts *o,
                        gelio_spectra *d_out, void *stream) {
  if (!c || n < 0 || n > kMaxSims || (n > 0 && (!d_sims || !d_out))) return GELIO_ERR_INVALID_ARGUMENT;
  int rc = check_opts(o);
  if (rc != GELIO_OK) return rc;
  if (o && (o->plain || o->record_capacity > 0)) return GELIO_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(c->mu);
  GELIO_TRY(cudaSetDevice(c->device));
  if (n == 0) return GELIO_OK;
  if ((rc = ensure_sims(c, n)) != GELIO_OK) return rc;
  cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
  GELIO_TRY(cudaMemcpyAsync(c->d_params, d_sims, sizeof(gelio_sim_params) * n, cudaMemcpyDeviceToDevice, st));
  rc = enqueue_run(c, n, o, (double *)d_out, st, 0u, nullptr, nullptr, 0, true);
  return rc;
}

int32_t gelio_last_stats(gelio_ctx *c, gelio_run_stats *stats) {
  if (!c || !stats) return GELIO_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(c->mu);
  GELIO_TRY(cudaSetDevice(c->device));
  GELIO_TRY(cudaDeviceSynchronize());
  *stats = c->last;
  if (c->last_timed) {
    float kms = 0.f;
    if (cudaEventElapsedTime(&kms, c->ev_k0, c->ev_k1) == cudaSuccess) stats->kernel_ms = kms;
    else (void)cudaGetLastError();
  }
  return (c->h_ctl->status != 0) ? (int)c->h_ctl->status : GELIO_OK;
}

int32_t gelio_replay(gelio_ctx *c, const gelio_sim_params *sim, int64_t first, int64_t count,
                     int32_t precision, uint64_t max_steps, gelio_trajectory *out) {
  if (!c || !sim || first < 0 || count < 0 || (count > 0 && !out)) return GELIO_ERR_INVALID_ARGUMENT;
  if (precision != GELIO_PREC_FP32 && precision != GELIO_PREC_FP64) return GELIO_ERR_INVALID_ARGUMENT;
  int rc = validate_params(*sim);
  if (rc != GELIO_OK) return rc;
  if (count == 0) return GELIO_OK;
  if (count > (int64_t)1 << 31) return GELIO_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(c->mu);
  GELIO_TRY(cudaSetDevice(c->device));
  (void)cudaGetLastError();
  if ((rc = ensure_sims(c, 1)) != GELIO_OK) return rc;
  size_t tb = c->traj_cap * sizeof(gelio_trajectory);
  GELIO_TRY(grow(c->d_traj, tb, (size_t)count * sizeof(gelio_trajectory)));
  c->traj_cap = tb / sizeof(gelio_trajectory);
  GELIO_TRY(grow(c->d_part, c->part_bytes, (size_t)kSpecDoubles * 8));
  cudaStream_t st = c->stream;
  GELIO_TRY(cudaMemcpyAsync(c->d_params, sim, sizeof(gelio_sim_params), cudaMemcpyHostToDevice, st));
  GELIO_TRY(cudaMemsetAsync(c->d_ctl, 0, sizeof(Control), st));
  GELIO_TRY(cudaMemsetAsync(c->d_part, 0, (size_t)kSpecDoubles * 8, st));
  Groups g{c->d_gsim, c->d_gpre};
  k_prepare<<<1, 256, 0, st>>>(c->d_params, 1, c->d_sims, c->d_tables, g, c->d_ctl);
  GELIO_TRY(cudaGetLastError());
  KArgs a{};
  a.sims = c->d_sims;
  a.inj_tables = c->d_tables;
  a.groups = g;
  a.n_sims = 1;
  a.n_slices = 1;
  a.part = c->d_part;
  a.ctl = c->d_ctl;
  a.max_steps = (max_steps > 0 && max_steps < 0xfffffff0ull) ? max_steps : 100000000ull;
  a.plain_sim = 0;
  a.plain_first = (unsigned long long)first;
  a.plain_count = (unsigned long long)count;
  a.replay = c->d_traj;
  const unsigned grid = (unsigned)((count + 127) / 128);
  GELIO_TRY(launch_model(sim->model, false, precision, grid, 128, 0, st, a));
  GELIO_TRY(cudaMemcpyAsync(out, c->d_traj, sizeof(gelio_trajectory) * count, cudaMemcpyDeviceToHost, st));
  GELIO_TRY(cudaMemcpyAsync(c->h_ctl, c->d_ctl, sizeof(Control), cudaMemcpyDeviceToHost, st));
  GELIO_TRY(cudaStreamSynchronize(st));
  return (c->h_ctl->status != 0) ? (int)c->h_ctl->status : GELIO_OK;
}

int32_t gelio_evaluate(gelio_ctx *c, int32_t model, const double *rows, int64_t n_rows, int32_t n_cols,
                       gelio_spectra *out) {
  if (!c || !out || n_rows < 0 || (n_rows > 0 && !rows) || model < 0 || model > 3) return GELIO_ERR_INVALID_ARGUMENT;
  const int need_cols = (model >= kModelSolarProp) ? 6 : (model == kModelBp ? 4 : 5);
  if (n_cols < need_cols) return GELIO_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(c->mu);
  GELIO_TRY(cudaSetDevice(c->device));
  memset(out, 0, sizeof(*out));
  if (n_rows == 0) return GELIO_OK;
  const int n_slices = 16;
  GELIO_TRY(grow(c->d_part, c->part_bytes, (size_t)n_slices * kSpecDoubles * 8));
  GELIO_TRY(grow(c->d_out, c->out_bytes, sizeof(gelio_spectra)));
  cudaStream_t st = c->stream;
  const size_t bytes = (size_t)n_rows * n_cols * sizeof(double);
  GELIO_TRY(grow(c->d_rows, c->rows_bytes, bytes));
  GELIO_TRY(cudaMemcpyAsync(c->d_rows, rows, bytes, cudaMemcpyHostToDevice, st));
  GELIO_TRY(cudaMemsetAsync(c->d_part, 0, (size_t)n_slices * kSpecDoubles * 8, st));
  const unsigned grid = (unsigned)((n_rows + 255) / 256);
  (void)cudaGetLastError();
  k_evaluate<<<grid, 256, 0, st>>>(c->d_rows, n_rows, n_cols, model, n_slices, c->d_part);
  GELIO_TRY(cudaGetLastError());
  k_reduce<<<(kSpecDoubles + 255) / 256, 256, 0, st>>>(c->d_part, n_slices, kSpecDoubles, c->d_out);
  GELIO_TRY(cudaGetLastError());
  GELIO_TRY(cudaMemcpyAsync(out, c->d_out, sizeof(gelio_spectra), cudaMemcpyDeviceToHost, st));
  GELIO_TRY(cudaStreamSynchronize(st));
  return GELIO_OK;
}

int32_t gelio_set_alloc_hook(gelio_alloc_hook hook, void *user) {
  g_alloc_user.store(user);
  g_alloc_hook.store(hook);
  return GELIO_OK;
}

int32_t gelio_measure_peaks(gelio_ctx *c, double *fp32_tflops, double *xu_gops) {
  if (!c || !fp32_tflops || !xu_gops) return GELIO_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(c->mu);
  GELIO_TRY(cudaSetDevice(c->device));
  float *d = nullptr;
  GELIO_TRY(dev_malloc(&d, sizeof(float)));
  const unsigned grid = (unsigned)c->sm_count * 8u, block = 256u;
  const int it_f = 2048, it_x = 512;
  float best_f = 1e30f, best_x = 1e30f;
  for (int rep = 0; rep < 4; ++rep) {
    float ms = 0.f;
    cudaEventRecord(c->ev_k0, c->stream);
    k_peak_fma<<<grid, block, 0, c->stream>>>(d, it_f);
    cudaEventRecord(c->ev_k1, c->stream);
    GELIO_TRY(cudaEventSynchronize(c->ev_k1));
    cudaEventElapsedTime(&ms, c->ev_k0, c->ev_k1);
    if (rep > 0 && ms < best_f) best_f = ms;
    cudaEventRecord(c->ev_k0, c->stream);
    k_peak_xu<<<grid, block, 0, c->stream>>>(d, it_x);
    cudaEventRecord(c->ev_k1, c->stream);
    GELIO_TRY(cudaEventSynchronize(c->ev_k1));
    cudaEventElapsedTime(&ms, c->ev_k0, c->ev_k1);
    if (rep > 0 && ms < best_x) best_x = ms;
  }
  cudaFree(d);
  GELIO_TRY(cudaGetLastError());
  const double threads = (double)grid * block;
  *fp32_tflops = threads * it_f * 16.0 * 8.0 * 2.0 / (best_f * 1e-3) / 1e12;
  *xu_gops = threads * it_x * 16.0 * 4.0 / (best_x * 1e-3) / 1e9;
  return GELIO_OK;
}

}  // extern "C"

// Device of a context, for the surrogate built on it.
int gelio_internal_device(const gelio_ctx *c) { return c ? c->device : 0; }

extern "C" {

int32_t gelio_autotune(gelio_ctx *c, const gelio_sim_params *sims, int32_t n, gelio_run_opts *best) {
  if (!c || !sims || n < 1 || n > kMaxSims) return GELIO_ERR_INVALID_ARGUMENT;
  int rc;
  int64_t total = 0;
  int model = -1;
  for (int i = 0; i < n; ++i) {
    if ((rc = validate_params(sims[i])) != GELIO_OK) return rc;
    total += sims[i].n_particles;
    if (model < 0 && sims[i].n_particles > 0) model = sims[i].model;
  }
  if (total <= 0) return GELIO_ERR_INVALID_ARGUMENT;
  static const int blocks[2] = {128, 256};
  static const int refills[4] = {8, 16, 32, 64};
  static const int compacts[2] = {1, 2};
  double best_rate = -1.0;
  gelio_run_opts bo{};
  std::vector<gelio_spectra> tmp(n);
  // one untimed run first (lazy allocations), then every shape once
  {
    gelio_run_opts o{};
    gelio_run_stats s{};
    rc = gelio_run(c, sims, n, &o, tmp.data(), &s);
    if (rc != GELIO_OK && rc < GELIO_WARN_FIRST) return rc;
  }
  for (int ci = 0; ci < 2; ++ci)
  for (int bi = 0; bi < 2; ++bi) {
    for (int ri = 0; ri < 4; ++ri) {
      gelio_run_opts o{};
      o.compact = compacts[ci];
      o.block_size = blocks[bi];
      o.refill_interval = refills[ri];
      gelio_run_stats s{};
      rc = gelio_run(c, sims, n, &o, tmp.data(), &s);
      if (rc != GELIO_OK && rc < GELIO_WARN_FIRST) return rc;
      const double rate = (s.kernel_ms > 0.0) ? (double)s.n_steps / s.kernel_ms : 0.0;
      if (rate > best_rate) {
        best_rate = rate;
        bo = o;
        bo.blocks_per_sm = s.blocks_per_sm;
      }
    }
  }
  std::lock_guard<std::mutex> lock(c->mu);
  if (model >= 0) {
    Tuned &t = c->tuned[model][0];
    t.block = bo.block_size;
    t.refill = bo.refill_interval;
    t.compact = bo.compact;
    t.blocks_per_sm = 0;
    // a cached graph was captured with the shapes chosen before
    if (c->graph) { cudaGraphExecDestroy(c->graph); c->graph = nullptr; }
  }
  if (best) *best = bo;
  return GELIO_OK;
}

}  // extern "C"
