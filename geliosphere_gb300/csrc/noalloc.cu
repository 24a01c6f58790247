// gelio_run_noalloc: the persistent SDE path for callers that cannot call
// cudaMalloc -- code running where device allocation is not allowed or not
// wanted (inside a host application with a fixed device-memory budget, a
// plugin that must not own allocations, a process whose allocator is locked
// by another runtime).  Every byte of scratch the kernels need (control
// block, per-simulation tables, model grouping, histogram slices) lives in
// one file-scope device array of fixed size; the caller passes the inputs
// and outputs, already in device memory.  No cudaMalloc, cudaFree or
// allocating library call is made.
#include <cuda_runtime.h>
#include <cstdint>
#include <cstring>
#include <mutex>

#include "gelio.h"
#include "kernels.cuh"

namespace gelio {

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
cudaError_t launch_prepare(const gelio_sim_params *, int, SimDev *, float *, Groups, Control *, cudaStream_t);
cudaError_t launch_reduce(const double *, int, long long, double *, cudaStream_t);
void build_tables(BinTables &t);

namespace {

constexpr int kMaxN = GELIO_NOALLOC_MAX_SIMS;
constexpr int kSlices = 2;

// Byte layout of the scratch array (each part 256-byte aligned).
constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }
constexpr size_t kOffCtl = 0;
constexpr size_t kOffSims = align256(kOffCtl + sizeof(Control));
constexpr size_t kOffTables = align256(kOffSims + sizeof(SimDev) * kMaxN);
constexpr size_t kOffGsim = align256(kOffTables + sizeof(float) * GELIO_GRID_MAX * kMaxN);
constexpr size_t kOffGpre = align256(kOffGsim + sizeof(int) * 4 * kMaxN);
constexpr size_t kOffPart = align256(kOffGpre + sizeof(unsigned long long) * 4 * (kMaxN + 1));
constexpr size_t kScratchBytes = align256(kOffPart + sizeof(double) * (size_t)kSlices * kMaxN * kSpecDoubles);
static_assert(kScratchBytes == GELIO_NOALLOC_SCRATCH_BYTES, "gelio.h states the scratch size");
static_assert((256 / 32) * (kQueue * sizeof(QEnt) + sizeof(int)) <= 48 * 1024, "queues fit the default shared memory");

}  // namespace

// The scratch.  Every GPU that loads the library holds it until the process
// exits; all calls on a device share it.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

namespace {

struct DeviceSetup {
  bool done = false;
  unsigned char *scratch = nullptr;   // device address of g_noalloc_scratch
  int sm_count = 0;
  int occ[3] = {0, 0, 0};             // CTAs of 256 per SM, per kernel variant, model-independent bound
};

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
DeviceSetup g_setup[kMaxDevices];

const void *persistent_kernel(int m, int variant) {
  switch (m) {
    case kModelFp: return fp_kernel(true, variant);
    case kModelBp: return bp_kernel(true, variant);
    case kModelSolarProp: return solarprop_kernel(true, variant);
    default: return geliosphere_kernel(true, variant);
  }
}

cudaError_t launch(int m, int variant, unsigned grid, unsigned block, size_t smem, cudaStream_t st,
                   const KArgs &a) {
  switch (m) {
    case kModelFp: return fp_launch(true, variant, grid, block, smem, st, a);
    case kModelBp: return bp_launch(true, variant, grid, block, smem, st, a);
    case kModelSolarProp: return solarprop_launch(true, variant, grid, block, smem, st, a);
    default: return geliosphere_launch(true, variant, grid, block, smem, st, a);
  }
}

constexpr unsigned kBlock = 256;
constexpr size_t kQueueBytes = (kBlock / 32) * (kQueue * sizeof(QEnt) + sizeof(int));

// Once per device, with that device current: resolve the scratch array's
// device address, fill the bin tables and record the occupancy.  Runs on the
// first call of gelio_run_noalloc on the device, so that first call should
// not be made while a stream is being captured.  The device counts as set up
// only once every step has succeeded: a failed set-up (e.g. a first call
// made during a capture, where the table copies are refused) is retried by
// the next call.  What it records outlives a cudaDeviceReset, which clears
// the tables: after a reset the process must be restarted before calling
// gelio_run_noalloc again.
int setup_device(int dev, DeviceSetup *&out) {
  std::lock_guard<std::mutex> lock(g_setup_mu);
  DeviceSetup &s = g_setup[dev];
  out = &s;
  if (s.done) return GELIO_OK;
  void *ptr = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
  if (e != cudaSuccess || ptr == nullptr) return GELIO_ERR_CUDA;
  BinTables t;
  build_tables(t);
  if (fp_tables(t) != cudaSuccess || bp_tables(t) != cudaSuccess || solarprop_tables(t) != cudaSuccess ||
      geliosphere_tables(t) != cudaSuccess)
    return GELIO_ERR_CUDA;
  int sm_count = 0;
  if (cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return GELIO_ERR_CUDA;
  int occ_v[2] = {0, 0};
  for (int v = 0; v < 2; ++v) {
    int lowest = 1 << 30;
    for (int m = 0; m < 4; ++m) {
      // kQueueBytes is below the 48 KB every kernel may use without opting
      // in, so no function attribute (shared with gelio_run) is changed
      const void *k = persistent_kernel(m, v);
      int occ = 0;
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, (int)kBlock, kQueueBytes) != cudaSuccess || occ < 1)
        return GELIO_ERR_UNSUPPORTED;
      if (occ < lowest) lowest = occ;
    }
    occ_v[v] = lowest;
  }
  s.scratch = static_cast<unsigned char *>(ptr);
  s.sm_count = sm_count;
  s.occ[0] = occ_v[0];
  s.occ[1] = occ_v[1];
  s.done = true;
  return GELIO_OK;
}

}  // namespace
}  // namespace gelio

using namespace gelio;

extern "C" int32_t gelio_run_noalloc(const gelio_sim_params *d_sims, int32_t n_sims,
                                     const gelio_run_opts *opts, gelio_spectra *d_out, void *stream) {
  if (n_sims < 0 || n_sims > kMaxN) return GELIO_ERR_INVALID_ARGUMENT;   // beyond the scratch
  if (n_sims > 0 && (d_sims == nullptr || d_out == nullptr)) return GELIO_ERR_INVALID_ARGUMENT;
  if (opts && (opts->plain || opts->record_capacity > 0 || opts->records != nullptr)) return GELIO_ERR_UNSUPPORTED;
  // the launch shape is fixed (blocks of 256, the occupancy bound per SM,
  // histograms in the scratch, no graph of its own): asking for another
  // one is refused rather than ignored
  if (opts && (opts->block_size != 0 || opts->blocks_per_sm != 0 || opts->compact != 0 || opts->use_graph != 0))
    return GELIO_ERR_UNSUPPORTED;
  if (opts && opts->precision != GELIO_PREC_FP32 && opts->precision != GELIO_PREC_FP64)
    return GELIO_ERR_INVALID_ARGUMENT;
  if (opts && (opts->refill_interval < 0 || opts->refill_interval % 4 != 0 || opts->refill_interval > 4096 ||
               !(opts->time_limit_s >= 0.0)))
    return GELIO_ERR_INVALID_ARGUMENT;
  if (n_sims == 0) return GELIO_OK;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return GELIO_ERR_NO_DEVICE;
  DeviceSetup *s = nullptr;
  int rc = setup_device(dev, s);
  if (rc != GELIO_OK) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  (void)cudaGetLastError();

  unsigned char *base = s->scratch;
  Control *ctl = reinterpret_cast<Control *>(base + kOffCtl);
  SimDev *sims = reinterpret_cast<SimDev *>(base + kOffSims);
  float *tables = reinterpret_cast<float *>(base + kOffTables);
  Groups g{reinterpret_cast<int *>(base + kOffGsim), reinterpret_cast<unsigned long long *>(base + kOffGpre)};
  double *part = reinterpret_cast<double *>(base + kOffPart);
  const size_t part_bytes = sizeof(double) * (size_t)kSlices * n_sims * kSpecDoubles;

  // the scratch keeps the previous call's contents: clear what accumulates
  if (cudaMemsetAsync(ctl, 0, sizeof(Control), st) != cudaSuccess) return GELIO_ERR_CUDA;
  if (cudaMemsetAsync(part, 0, part_bytes, st) != cudaSuccess) return GELIO_ERR_CUDA;
  if (launch_prepare(d_sims, n_sims, sims, tables, g, ctl, st) != cudaSuccess) return GELIO_ERR_CUDA;

  const int variant = (opts && opts->precision == GELIO_PREC_FP64) ? 1 : 0;
  KArgs a{};
  a.sims = sims;
  a.inj_tables = tables;
  a.groups = g;
  a.n_sims = n_sims;
  a.n_slices = kSlices;
  a.part = part;
  a.ctl = ctl;
  unsigned long long ms = (opts && opts->max_steps_per_particle) ? opts->max_steps_per_particle : 100000000ull;
  if (ms > 0xfffffff0ull) ms = 0xfffffff0ull;
  a.max_steps = ms;
  a.time_limit_ns = (opts && opts->time_limit_s > 0.0) ? (unsigned long long)(opts->time_limit_s * 1e9) : 0ull;
  a.smem_slots = 0;                        // histograms go to the scratch slices
  const unsigned grid = (unsigned)(s->sm_count * s->occ[variant]);
  for (int m = 0; m < 4; ++m) {
    a.refill = (opts && opts->refill_interval > 0) ? opts->refill_interval : (m == kModelFp ? 4 : 16);
    if (launch(m, variant, grid, kBlock, kQueueBytes, st, a) != cudaSuccess) return GELIO_ERR_CUDA;
  }
  if (launch_reduce(part, kSlices, (long long)n_sims * kSpecDoubles, reinterpret_cast<double *>(d_out), st) !=
      cudaSuccess)
    return GELIO_ERR_CUDA;
  unsigned status = 0;
  if (cudaMemcpyAsync(&status, &ctl->status, sizeof(status), cudaMemcpyDeviceToHost, st) != cudaSuccess)
    return GELIO_ERR_CUDA;
  if (cudaStreamSynchronize(st) != cudaSuccess) return GELIO_ERR_CUDA;
  return (int32_t)status;
}
