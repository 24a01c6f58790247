// Spectrum surrogate: an ensemble of small MLPs trained on the GPU, on
// spectra the Monte Carlo kernels produced, by the tcgen05 kernels of
// mlp_kernels.cuh.  The network maps a 2D Geliosphere simulation's
// (K0, V, tilt, polarity, r, theta) and a 1 AU kinetic energy T to
// ln(J_mod(T) / J_LIS(T)); the ensemble's spread decides when a query falls
// back to the Monte Carlo.  No reference counterpart (a learned addition on
// top of the reference's method).
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <random>
#include <vector>

#include "gelio.h"
#include "alloc.cuh"
#include "mlp_kernels.cuh"

int gelio_internal_device(const gelio_ctx *c);

namespace gelio {
namespace mlp {
namespace {

using bf16 = __nv_bfloat16;

// cuTensorMapEncodeTiled through the runtime's driver entry point (no
// libcuda link dependency).
using EncodeFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                              const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                              CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeFn encode_fn() {
  static EncodeFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeFn>(p);
  });
  return fn;
}

// BF16 matrix [outer][inner] (inner contiguous), tiles of {64, box_outer}
// with the 128-byte swizzle; out-of-range rows read as zero.
bool make_map(CUtensorMap *m, const void *ptr, uint64_t inner, uint64_t outer, uint32_t box_outer) {
  EncodeFn f = encode_fn();
  if (!f) return false;
  const cuuint64_t dims[2] = {inner, outer};
  const cuuint64_t strides[1] = {inner * 2};
  const cuuint32_t box[2] = {64, box_outer};
  const cuuint32_t estr[2] = {1, 1};
  return f(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(ptr), dims, strides, box, estr,
           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Local interstellar spectra of the evaluators (TwoDimensionBpResults.cpp:50-60),
// for the training targets.
double lis(int which, double T) {
  const double l = std::log(T);
  if (which == 0) {
    return 21.1 * std::exp(-2.8 * l) / (1.0 + 5.85 * std::exp(-1.22 * l) + 1.18 * std::exp(-2.54 * l));
  }
  if (which == 1) {
    const double tt = T + 0.938, t2 = tt + 0.938;
    const double beta = std::sqrt(T * t2) / tt;
    const double tem = std::exp(-3.93 * std::log((T + 0.67) / 1.67));
    return 2.7e3 * std::exp(1.12 * l) * tem / (beta * beta);
  }
  const double p = std::sqrt(T * T + 2.0 * T * 0.938);
  return 1.9e4 * std::exp(-2.78 * std::log(p)) / (1.0 + 0.4866 * std::exp(-2.51 * std::log(p)));
}

// LOG_GRID energies exactly as the kernels build them.
float grid_energy(const gelio_sim_params &s, int j) {
  const double lmin = std::log((double)s.inj_min), lmax = std::log((double)s.inj_max);
  const double f = (s.inj_points > 1) ? (double)j / (double)(s.inj_points - 1) : 0.0;
  return (float)std::exp(lmin + f * (lmax - lmin));
}

uint64_t splitmix(uint64_t &x) {
  uint64_t z = (x += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

struct Member {
  float *P = nullptr, *M1 = nullptr, *M2 = nullptr;
  bf16 *W1 = nullptr, *W[3] = {}, *WT[3] = {};
  CUtensorMap mW1, mW[3], mWT[3];
  int adam_t = 0;
  bool trained = false;
};

}  // namespace
}  // namespace mlp
}  // namespace gelio

using namespace gelio::mlp;

struct gelio_surrogate {
  gelio_ctx *ctx = nullptr;
  gelio_surrogate_opts o{};
  int device = 0, sm_count = 0, rows = 0;   // rows = batch rows
  int k_split = 256, splits = 0;
  cudaStream_t stream = nullptr;
  std::vector<Member> mem;
  // activations and gradients of one batch
  bf16 *X0 = nullptr, *X0T = nullptr, *Z[4] = {}, *X[3] = {}, *XT[4] = {}, *dH[4] = {}, *dHT[4] = {};
  float *yhat = nullptr, *y = nullptr, *dy = nullptr, *partial = nullptr, *grad = nullptr, *loss_part = nullptr;
  float *step_loss = nullptr;
  int step_loss_cap = 0;
  int *ident = nullptr;      // 0, 1, ..., rows - 1
  int *order = nullptr;      // this epoch's shuffled row order
  size_t order_cap = 0;
  unsigned *error = nullptr;
  CUtensorMap mX0, mX[3], mdH[4], mdHT[4], mX0T, mXT[3];
  // training rows (host) and their device copy
  std::vector<float> feats, targ;
  float *d_feats = nullptr, *d_targ = nullptr;
  size_t d_rows_cap = 0, d_rows_used = 0;
  float *d_query = nullptr, *d_yq = nullptr;   // inference inputs / outputs
  size_t query_cap = 0;
  // predict: simulations and their row offsets on the device, member outputs
  // [E][stride], ensemble mean / std [2][rows], pinned staging of both ends
  unsigned char *d_pup = nullptr;     // [n] gelio_sim_params, then [n + 1] row offsets
  size_t pup_cap = 0;
  float *d_py = nullptr;
  double *d_pstat = nullptr;
  size_t prows_cap = 0;
  unsigned char *h_pstage = nullptr;
  size_t pstage_cap = 0;
  // inference batches: larger than training batches, so every SM gets
  // several tiles per launch and the resident weights are loaded once per tile
  // group rather than once per tile
  int qrows = 0;
  bf16 *Q0 = nullptr, *Q[2] = {};
  float *qy = nullptr;
  int *qident = nullptr;
  CUtensorMap mQ0, mQ[2];
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;    // device time of the last inference
  double last_ms = 0.0, last_flop = 0.0;
  bool dirty = true;
  std::mutex mu;
};

namespace {

int cuda_status_at(cudaError_t e, int line) {
  if (e == cudaSuccess) return GELIO_OK;
  gelio::note_cuda_error(e, "mlp.cu", line);
  if (e == cudaErrorMemoryAllocation) return GELIO_ERR_OUT_OF_MEMORY;
  return GELIO_ERR_CUDA;
}
#define cuda_status(e) cuda_status_at((e), __LINE__)
#define SUR_TRY(x)                            \
  do {                                        \
    cudaError_t e_ = (x);                     \
    if (e_ != cudaSuccess) return cuda_status(e_); \
  } while (0)

template <int MODE>
int launch_gemm(gelio_surrogate *s, const CUtensorMap &A, const CUtensorMap &B, GemmArgs a) {
  a.error = s->error;
  a.timeout_ns = 2000000000ull;
  if (a.splits < 1) a.splits = 1;
  if (a.k_per_split <= 0) a.k_per_split = a.K;
  const int tiles = ((a.M + kTileM - 1) / kTileM) * a.splits;
  const int grid = std::max(1, std::min(tiles, s->sm_count));
  k_mlp_gemm<MODE><<<grid, kGemmThreads, kGemmSmem, s->stream>>>(A, B, a);
  return cuda_status(cudaGetLastError());
}

int set_smem_attrs() {
  static int rc = -1;
  static std::once_flag once;
  std::call_once(once, [] {
    cudaError_t e = cudaSuccess;
    auto set = [&](const void *f) {
      if (e == cudaSuccess)
        e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGemmSmem);
    };
    set((const void *)k_mlp_gemm<FWD>);
    set((const void *)k_mlp_gemm<FWD_LAST>);
    set((const void *)k_mlp_gemm<INFER>);
    set((const void *)k_mlp_gemm<INFER_LAST>);
    set((const void *)k_mlp_gemm<DX>);
    set((const void *)k_mlp_gemm<DW>);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute((const void *)k_mlp_infer_fused, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)kFusedSmem);
    rc = cuda_status(e);
  });
  return rc;
}

void free_all(gelio_surrogate *s) {
  auto f = [](void *p) { if (p) cudaFree(p); };
  for (auto &m : s->mem) {
    f(m.P); f(m.M1); f(m.M2); f(m.W1);
    for (int i = 0; i < 3; ++i) { f(m.W[i]); f(m.WT[i]); }
  }
  f(s->X0); f(s->X0T);
  for (int i = 0; i < 4; ++i) { f(s->Z[i]); f(s->XT[i]); f(s->dH[i]); f(s->dHT[i]); }
  for (int i = 0; i < 3; ++i) f(s->X[i]);
  f(s->yhat); f(s->y); f(s->dy); f(s->partial); f(s->grad); f(s->loss_part); f(s->step_loss);
  f(s->ident); f(s->order); f(s->error); f(s->d_feats); f(s->d_targ); f(s->d_query); f(s->d_yq);
  f(s->Q0); f(s->Q[0]); f(s->Q[1]); f(s->qy); f(s->qident);
  f(s->d_pup); f(s->d_py); f(s->d_pstat);
  if (s->h_pstage) cudaFreeHost(s->h_pstage);
  if (s->ev0) cudaEventDestroy(s->ev0);
  if (s->ev1) cudaEventDestroy(s->ev1);
  if (s->stream) cudaStreamDestroy(s->stream);
}

int pack(gelio_surrogate *s, Member &m) {
  const int n = kWidth * kWidth;
  k_pack<<<(n + 255) / 256, 256, 0, s->stream>>>(m.P, m.W1, m.W[0], m.W[1], m.W[2], m.WT[0], m.WT[1], m.WT[2]);
  return cuda_status(cudaGetLastError());
}

int check_error(gelio_surrogate *s) {
  unsigned e = 0;
  SUR_TRY(cudaMemcpyAsync(&e, s->error, sizeof(e), cudaMemcpyDeviceToHost, s->stream));
  SUR_TRY(cudaStreamSynchronize(s->stream));
  if (e) {
    cudaMemsetAsync(s->error, 0, sizeof(unsigned), s->stream);
    cudaStreamSynchronize(s->stream);
    return GELIO_ERR_TIMEOUT;
  }
  return GELIO_OK;
}

// Forward (training form) + backward of member m on the gathered batch;
// gradient into s->grad, squared-error sum into *loss_slot (device).
int forward_backward(gelio_surrogate *s, Member &m, int n_valid, float *loss_slot) {
  const int R = s->rows;
  int rc;
  GemmArgs a{};
  a.M = R; a.N = kWidth; a.ldt = R; a.splits = 1;
  // forward
  a.K = kInPad; a.bias = m.P + kOffB1; a.z_out = s->Z[0]; a.x_out = s->X[0]; a.xt_out = s->XT[0];
  if ((rc = launch_gemm<FWD>(s, s->mX0, m.mW1, a)) != GELIO_OK) return rc;
  a.K = kWidth; a.bias = m.P + kOffB2; a.z_out = s->Z[1]; a.x_out = s->X[1]; a.xt_out = s->XT[1];
  if ((rc = launch_gemm<FWD>(s, s->mX[0], m.mW[0], a)) != GELIO_OK) return rc;
  a.bias = m.P + kOffB3; a.z_out = s->Z[2]; a.x_out = s->X[2]; a.xt_out = s->XT[2];
  if ((rc = launch_gemm<FWD>(s, s->mX[1], m.mW[1], a)) != GELIO_OK) return rc;
  a.bias = m.P + kOffB4; a.z_out = s->Z[3]; a.x_out = nullptr; a.xt_out = s->XT[3];
  a.w5 = m.P + kOffW5; a.b5 = m.P + kOffB5; a.y_out = s->yhat;
  SUR_TRY(cudaMemsetAsync(s->yhat, 0, (size_t)R * 4, s->stream));
  if ((rc = launch_gemm<FWD_LAST>(s, s->mX[2], m.mW[2], a)) != GELIO_OK) return rc;
  // head
  const int hb = (R + kThreads - 1) / kThreads;
  k_head_backward<<<hb, kThreads, 0, s->stream>>>(s->yhat, s->y, n_valid, R, m.P + kOffW5, s->Z[3], s->dH[3],
                                                   s->dHT[3], s->dy, s->loss_part);
  k_sum_f32<<<1, 256, 0, s->stream>>>(s->loss_part, hb, loss_slot);
  k_rowsum_bf16<<<kWidth, 256, 0, s->stream>>>(s->XT[3], R, s->dy, s->grad + kOffW5);
  k_sum_f32<<<1, 256, 0, s->stream>>>(s->dy, R, s->grad + kOffB5);
  SUR_TRY(cudaGetLastError());
  // hidden layers, top down
  const int offW[4] = {kOffW1, kOffW2, kOffW3, kOffW4};
  const int offB[4] = {kOffB1, kOffB2, kOffB3, kOffB4};
  for (int l = 4; l >= 1; --l) {
    const int li = l - 1;
    GemmArgs d{};
    d.M = kWidth; d.K = R; d.k_per_split = s->k_split; d.splits = s->splits; d.partial = s->partial; d.ldt = R;
    d.N = (l == 1) ? kInPad : kWidth;
    const CUtensorMap &Bm = (l == 1) ? s->mX0T : s->mXT[l - 2];
    if ((rc = launch_gemm<DW>(s, s->mdHT[li], Bm, d)) != GELIO_OK) return rc;
    const int fan_in = (l == 1) ? kFeatures : kWidth;
    k_reduce_dw<<<(kWidth * fan_in + 255) / 256, 256, 0, s->stream>>>(s->partial, s->splits, d.N, fan_in,
                                                                      s->grad + offW[li]);
    k_rowsum_bf16<<<kWidth, 256, 0, s->stream>>>(s->dHT[li], R, nullptr, s->grad + offB[li]);
    SUR_TRY(cudaGetLastError());
    if (l >= 2) {
      GemmArgs x{};
      x.M = R; x.N = kWidth; x.K = kWidth; x.splits = 1; x.ldt = R;
      x.z_prev = s->Z[li - 1]; x.dh_out = s->dH[li - 1]; x.dht_out = s->dHT[li - 1];
      if ((rc = launch_gemm<DX>(s, s->mdH[li], m.mWT[li - 1], x)) != GELIO_OK) return rc;
    }
  }
  return GELIO_OK;
}


// Inference of member m on the first `M` rows of the inference batch
// (M a multiple of 128); outputs in s->qy.
int forward_infer_q(gelio_surrogate *s, Member &m, int M) {
  int rc;
  GemmArgs a{};
  a.M = M; a.N = kWidth; a.ldt = s->qrows; a.splits = 1;
  a.K = kInPad; a.bias = m.P + kOffB1; a.x_out = s->Q[0];
  if ((rc = launch_gemm<INFER>(s, s->mQ0, m.mW1, a)) != GELIO_OK) return rc;
  a.K = kWidth; a.bias = m.P + kOffB2; a.x_out = s->Q[1];
  if ((rc = launch_gemm<INFER>(s, s->mQ[0], m.mW[0], a)) != GELIO_OK) return rc;
  a.bias = m.P + kOffB3; a.x_out = s->Q[0];
  if ((rc = launch_gemm<INFER>(s, s->mQ[1], m.mW[1], a)) != GELIO_OK) return rc;
  a.bias = m.P + kOffB4; a.x_out = nullptr; a.w5 = m.P + kOffW5; a.b5 = m.P + kOffB5; a.y_out = s->qy;
  SUR_TRY(cudaMemsetAsync(s->qy, 0, (size_t)M * 4, s->stream));
  return launch_gemm<INFER_LAST>(s, s->mQ[0], m.mW[2], a);
}

// Upload x rows [n][7] to the training-row buffer tail used as scratch and
// gather them (identity order, padding to the batch).
int stage_rows(gelio_surrogate *s, float *d_x, float *d_t, int n) {
  k_gather<<<(s->rows + 127) / 128, 128, 0, s->stream>>>(d_x, d_t, s->ident, n, 0, s->rows, s->X0, s->X0T, s->y);
  return cuda_status(cudaGetLastError());
}

bool valid_member(gelio_surrogate *s, int m) { return s && m >= 0 && m < (int)s->mem.size(); }

// Inference of members [m0, m1) on n rows x [n][7]: one upload, one gather
// per batch of rows shared by the members, outputs y[(m - m0) * n + row].
int infer_rows(gelio_surrogate *s, int m0, int m1, const float *x, size_t n, float *y) {
  if (n == 0) return GELIO_OK;
  const size_t E = (size_t)(m1 - m0);
  if (n > s->query_cap) {
    if (s->d_query) cudaFree(s->d_query);
    if (s->d_yq) cudaFree(s->d_yq);
    s->d_query = s->d_yq = nullptr;
    s->query_cap = 0;
    SUR_TRY(gelio::dev_malloc(&s->d_query, n * kFeatures * 4));
    SUR_TRY(gelio::dev_malloc(&s->d_yq, n * 16 * 4));
    s->query_cap = n;
  }
  SUR_TRY(cudaMemcpyAsync(s->d_query, x, n * kFeatures * 4, cudaMemcpyHostToDevice, s->stream));
  SUR_TRY(cudaEventRecord(s->ev0, s->stream));
  size_t padded = 0;
  for (size_t off = 0; off < n; off += (size_t)s->qrows) {
    const int c = (int)std::min<size_t>((size_t)s->qrows, n - off);
    const int M = (c + kTileM - 1) / kTileM * kTileM;     // only the tiles this chunk needs
    padded += (size_t)M;
    k_gather<<<(M + 127) / 128, 128, 0, s->stream>>>(s->d_query + off * kFeatures, nullptr, s->qident, c, 0, M,
                                                     s->Q0, nullptr, nullptr);
    SUR_TRY(cudaGetLastError());
    for (size_t e = 0; e < E; ++e) {
      const int rc = forward_infer_q(s, s->mem[m0 + e], M);
      if (rc != GELIO_OK) return rc;
      SUR_TRY(cudaMemcpyAsync(s->d_yq + e * n + off, s->qy, (size_t)c * 4, cudaMemcpyDeviceToDevice, s->stream));
    }
  }
  SUR_TRY(cudaEventRecord(s->ev1, s->stream));
  SUR_TRY(cudaMemcpyAsync(y, s->d_yq, E * n * 4, cudaMemcpyDeviceToHost, s->stream));
  const int rc = check_error(s);
  float ms = 0.f;
  if (rc == GELIO_OK && cudaEventElapsedTime(&ms, s->ev0, s->ev1) == cudaSuccess) {
    s->last_ms = ms;
    // FLOP of the GEMMs over the rows actually multiplied (each inference
    // batch padded to a multiple of 128 rows; first layer K padded to 64)
    s->last_flop = 2.0 * (double)padded * (double)E *
                   ((double)kInPad * kWidth + 3.0 * kWidth * kWidth + (double)kWidth);
  }
  return rc;
}

void default_opts(gelio_surrogate_opts &o) {
  std::memset(&o, 0, sizeof(o));
  o.members = 5;
  o.batch_rows = 16384;
  o.lis = 1;
  o.min_count = 64;
  o.lr = 2e-3f;
  o.lr_final = 2e-5f;
  o.fallback_std = 0.03f;
  o.t_min = 0.1f;
  o.t_max = 10.0f;
  o.seed = 1;
}

}  // namespace

extern "C" {

int32_t gelio_surrogate_features(const gelio_sim_params *sim, double T, float *out) {
  if (!sim || !out || !(T > 0.0)) return GELIO_ERR_INVALID_ARGUMENT;
  const double k0_cm2 = (double)sim->K0 / 4.4683705e-27;
  const double v_kms = (double)sim->V / 6.68458712e-9;
  const double rad = 180.0 / 3.14159265358979323846;
  out[0] = (float)((std::log10(k0_cm2) - 22.5) * 2.0);
  out[1] = (float)((v_kms - 550.0) / 200.0);
  out[2] = (float)(((double)sim->tilt * rad - 40.0) / 35.0);
  out[3] = (float)sim->polarity;
  out[4] = (float)(((double)sim->r_injection - 40.5) / 39.5);
  out[5] = (float)(((double)sim->theta_injection * rad - 90.0) / 80.0);
  out[6] = (float)(std::log10(T) / 2.0);
  return GELIO_OK;
}

int32_t gelio_surrogate_create(gelio_ctx *ctx, const gelio_surrogate_opts *opts, gelio_surrogate **out) {
  if (!ctx || !out) return GELIO_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  gelio_surrogate_opts o;
  default_opts(o);
  if (opts) {
    o = *opts;
    gelio_surrogate_opts d;
    default_opts(d);
    if (o.members <= 0) o.members = d.members;
    if (o.batch_rows <= 0) o.batch_rows = d.batch_rows;
    if (o.min_count <= 0) o.min_count = d.min_count;
    if (!(o.lr > 0.f)) o.lr = d.lr;
    if (!(o.lr_final > 0.f)) o.lr_final = d.lr_final;
    if (!(o.fallback_std > 0.f)) o.fallback_std = d.fallback_std;
    if (!(o.t_min > 0.f)) o.t_min = d.t_min;
    if (!(o.t_max > o.t_min)) o.t_max = d.t_max;
  }
  if (o.members > 16 || o.batch_rows % 256 != 0 || o.batch_rows > (1 << 20) || o.lis < 0 || o.lis > 2)
    return GELIO_ERR_INVALID_ARGUMENT;
  auto *s = new gelio_surrogate();
  s->ctx = ctx;
  s->o = o;
  s->device = gelio_internal_device(ctx);
  s->rows = o.batch_rows;
  s->splits = s->rows / s->k_split;
  int rc = GELIO_OK;
  auto fail = [&](int r) { free_all(s); delete s; return r; };
  if (cudaSetDevice(s->device) != cudaSuccess) return fail(GELIO_ERR_NO_DEVICE);
  (void)cudaGetLastError();   // a launch check below must see only this call's errors
  if (!encode_fn()) return fail(GELIO_ERR_UNSUPPORTED);
  if ((rc = set_smem_attrs()) != GELIO_OK) return fail(rc);
  cudaDeviceGetAttribute(&s->sm_count, cudaDevAttrMultiProcessorCount, s->device);
  if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) return fail(GELIO_ERR_CUDA);
  if (cudaEventCreate(&s->ev0) != cudaSuccess || cudaEventCreate(&s->ev1) != cudaSuccess) return fail(GELIO_ERR_CUDA);
  const size_t R = (size_t)s->rows;
  auto alloc = [&](void **p, size_t bytes) {
    if (rc != GELIO_OK) return;
    cudaError_t e = gelio::dev_malloc(p, bytes);
    if (e == cudaSuccess) e = cudaMemset(*p, 0, bytes);
    rc = cuda_status(e);
  };
  alloc((void **)&s->X0, R * kInPad * 2);
  alloc((void **)&s->X0T, (size_t)kInPad * R * 2);
  for (int i = 0; i < 4; ++i) {
    alloc((void **)&s->Z[i], R * kWidth * 2);
    alloc((void **)&s->XT[i], R * kWidth * 2);
    alloc((void **)&s->dH[i], R * kWidth * 2);
    alloc((void **)&s->dHT[i], R * kWidth * 2);
  }
  for (int i = 0; i < 3; ++i) alloc((void **)&s->X[i], R * kWidth * 2);
  alloc((void **)&s->yhat, R * 4);
  alloc((void **)&s->y, R * 4);
  alloc((void **)&s->dy, R * 4);
  alloc((void **)&s->partial, (size_t)s->splits * kWidth * kWidth * 4);
  alloc((void **)&s->grad, (size_t)kParams * 4);
  alloc((void **)&s->loss_part, (R / kThreads + 1) * 4);
  alloc((void **)&s->ident, R * 4);
  s->qrows = std::max(s->rows, 65536);
  const size_t Rq = (size_t)s->qrows;
  alloc((void **)&s->Q0, Rq * kInPad * 2);
  alloc((void **)&s->Q[0], Rq * kWidth * 2);
  alloc((void **)&s->Q[1], Rq * kWidth * 2);
  alloc((void **)&s->qy, Rq * 4);
  alloc((void **)&s->qident, Rq * 4);
  alloc((void **)&s->error, 4);
  s->mem.resize(o.members);
  for (auto &m : s->mem) {
    alloc((void **)&m.P, (size_t)kParams * 4);
    alloc((void **)&m.M1, (size_t)kParams * 4);
    alloc((void **)&m.M2, (size_t)kParams * 4);
    alloc((void **)&m.W1, (size_t)kWidth * kInPad * 2);
    for (int i = 0; i < 3; ++i) {
      alloc((void **)&m.W[i], (size_t)kWidth * kWidth * 2);
      alloc((void **)&m.WT[i], (size_t)kWidth * kWidth * 2);
    }
  }
  if (rc != GELIO_OK) return fail(rc);
  bool ok = make_map(&s->mX0, s->X0, kInPad, R, kTileM) && make_map(&s->mX0T, s->X0T, R, kInPad, kInPad);
  for (int i = 0; i < 3; ++i) {
    ok = ok && make_map(&s->mX[i], s->X[i], kWidth, R, kTileM);
    ok = ok && make_map(&s->mXT[i], s->XT[i], R, kWidth, kWidth);
  }
  ok = ok && make_map(&s->mQ0, s->Q0, kInPad, Rq, kTileM) && make_map(&s->mQ[0], s->Q[0], kWidth, Rq, kTileM) &&
       make_map(&s->mQ[1], s->Q[1], kWidth, Rq, kTileM);
  for (int i = 0; i < 4; ++i) {
    ok = ok && make_map(&s->mdH[i], s->dH[i], kWidth, R, kTileM);
    ok = ok && make_map(&s->mdHT[i], s->dHT[i], R, kWidth, kTileM);
  }
  for (auto &m : s->mem) {
    ok = ok && make_map(&m.mW1, m.W1, kInPad, kWidth, kWidth);
    for (int i = 0; i < 3; ++i) {
      ok = ok && make_map(&m.mW[i], m.W[i], kWidth, kWidth, kWidth);
      ok = ok && make_map(&m.mWT[i], m.WT[i], kWidth, kWidth, kWidth);
    }
  }
  if (!ok) return fail(GELIO_ERR_CUDA);
  // initial weights: uniform(+-sqrt(3 / fan_in)), zero biases
  uint64_t st = o.seed * 0x2545F4914F6CDD1Dull + 12345;
  std::vector<float> p(kParams);
  for (size_t e = 0; e < s->mem.size(); ++e) {
    std::fill(p.begin(), p.end(), 0.0f);
    auto fill = [&](int off, int n, int fan_in) {
      const double a = std::sqrt(3.0 / fan_in);
      for (int i = 0; i < n; ++i) p[off + i] = (float)(a * (2.0 * ((splitmix(st) >> 11) * 0x1.0p-53) - 1.0));
    };
    fill(kOffW1, kWidth * kFeatures, kFeatures);
    fill(kOffW2, kWidth * kWidth, kWidth);
    fill(kOffW3, kWidth * kWidth, kWidth);
    fill(kOffW4, kWidth * kWidth, kWidth);
    fill(kOffW5, kWidth, kWidth);
    if (cudaMemcpy(s->mem[e].P, p.data(), (size_t)kParams * 4, cudaMemcpyHostToDevice) != cudaSuccess)
      return fail(GELIO_ERR_CUDA);
    if ((rc = pack(s, s->mem[e])) != GELIO_OK) return fail(rc);
  }
  {
    std::vector<int> id(R);
    for (size_t i = 0; i < R; ++i) id[i] = (int)i;
    if (cudaMemcpy(s->ident, id.data(), R * 4, cudaMemcpyHostToDevice) != cudaSuccess) return fail(GELIO_ERR_CUDA);
    std::vector<int> idq(Rq);
    for (size_t i = 0; i < Rq; ++i) idq[i] = (int)i;
    if (cudaMemcpy(s->qident, idq.data(), Rq * 4, cudaMemcpyHostToDevice) != cudaSuccess)
      return fail(GELIO_ERR_CUDA);
  }
  if (cudaStreamSynchronize(s->stream) != cudaSuccess) return fail(GELIO_ERR_CUDA);
  *out = s;
  return GELIO_OK;
}

void gelio_surrogate_destroy(gelio_surrogate *s) {
  if (!s) return;
  cudaSetDevice(s->device);
  if (s->stream) cudaStreamSynchronize(s->stream);
  free_all(s);
  delete s;
}

int32_t gelio_surrogate_add_spectra(gelio_surrogate *s, const gelio_sim_params *sims, const gelio_spectra *spectra,
                                    int32_t n, int64_t *n_rows) {
  if (!s || n < 0 || (n > 0 && (!sims || !spectra))) return GELIO_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(s->mu);
  for (int i = 0; i < n; ++i) {
    const gelio_sim_params &q = sims[i];
    if (q.model != GELIO_MODEL_2D_GELIOSPHERE || q.injection != GELIO_INJ_LOG_GRID || q.grid_bins != 0)
      return GELIO_ERR_INVALID_ARGUMENT;
  }
  for (int i = 0; i < n; ++i) {
    const gelio_sim_params &q = sims[i];
    for (int j = 0; j < q.inj_points; ++j) {
      const double cnt = spectra[i].grid_n[j];
      const double w = spectra[i].grid_w[s->o.lis][j];
      if (cnt < s->o.min_count || !(w > 0.0)) continue;
      const double T = grid_energy(q, j);
      float f[kFeatures];
      gelio_surrogate_features(&q, T, f);
      s->feats.insert(s->feats.end(), f, f + kFeatures);
      s->targ.push_back((float)std::log((w / cnt) / lis(s->o.lis, T)));
    }
  }
  s->dirty = true;
  if (n_rows) *n_rows = (int64_t)s->targ.size();
  return GELIO_OK;
}

int32_t gelio_surrogate_add_rows(gelio_surrogate *s, const float *x, const float *t, int64_t n, int64_t *n_rows) {
  if (!s || n < 0 || (n > 0 && (!x || !t))) return GELIO_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(s->mu);
  s->feats.insert(s->feats.end(), x, x + (size_t)n * kFeatures);
  s->targ.insert(s->targ.end(), t, t + (size_t)n);
  s->dirty = true;
  if (n_rows) *n_rows = (int64_t)s->targ.size();
  return GELIO_OK;
}

int32_t gelio_surrogate_train(gelio_surrogate *s, int32_t epochs, float *last_loss) {
  if (!s || epochs < 0) return GELIO_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(s->mu);
  const size_t nrow = s->targ.size();
  if (nrow == 0) return GELIO_ERR_NOT_TRAINED;
  SUR_TRY(cudaSetDevice(s->device));
  (void)cudaGetLastError();   // a launch check below must see only this call's errors
  if (s->dirty) {
    if (nrow > s->d_rows_cap) {
      if (s->d_feats) cudaFree(s->d_feats);
      if (s->d_targ) cudaFree(s->d_targ);
      s->d_feats = s->d_targ = nullptr;
      SUR_TRY(gelio::dev_malloc(&s->d_feats, nrow * kFeatures * 4));
      SUR_TRY(gelio::dev_malloc(&s->d_targ, nrow * 4));
      s->d_rows_cap = nrow;
    }
    SUR_TRY(cudaMemcpy(s->d_feats, s->feats.data(), nrow * kFeatures * 4, cudaMemcpyHostToDevice));
    SUR_TRY(cudaMemcpy(s->d_targ, s->targ.data(), nrow * 4, cudaMemcpyHostToDevice));
    s->d_rows_used = nrow;
    s->dirty = false;
  }
  const int R = s->rows;
  const int steps = (int)std::max<size_t>(1, nrow / (size_t)R);
  if (steps > s->step_loss_cap) {
    if (s->step_loss) cudaFree(s->step_loss);
    s->step_loss = nullptr;
    SUR_TRY(gelio::dev_malloc(&s->step_loss, sizeof(float) * steps));
    s->step_loss_cap = steps;
  }
  if (nrow > s->order_cap) {
    if (s->order) cudaFree(s->order);
    s->order = nullptr;
    SUR_TRY(gelio::dev_malloc(&s->order, nrow * sizeof(int)));
    s->order_cap = nrow;
  }
  const long long total = (long long)epochs * steps;
  std::vector<int> order(nrow);
  std::vector<float> sl(steps);
  for (size_t e = 0; e < s->mem.size(); ++e) {
    Member &m = s->mem[e];
    std::mt19937_64 rng(s->o.seed * 1000003ull + e);
    for (size_t i = 0; i < nrow; ++i) order[i] = (int)i;
    double loss = 0.0;
    for (int ep = 0; ep < epochs; ++ep) {
      std::shuffle(order.begin(), order.end(), rng);
      // the host order is reshuffled next epoch: the copy completes first
      SUR_TRY(cudaMemcpyAsync(s->order, order.data(), nrow * sizeof(int), cudaMemcpyHostToDevice, s->stream));
      SUR_TRY(cudaStreamSynchronize(s->stream));
      for (int st = 0; st < steps; ++st) {
        const long long off = (long long)st * R;
        const int nv = (int)std::min<long long>(R, (long long)nrow - off);
        k_gather<<<(R + 127) / 128, 128, 0, s->stream>>>(s->d_feats, s->d_targ, s->order, (long long)nrow, off, R,
                                                         s->X0, s->X0T, s->y);
        int rc = forward_backward(s, m, nv, s->step_loss + st);
        if (rc != GELIO_OK) return rc;
        const long long t = (long long)ep * steps + st;
        const double frac = total > 1 ? (double)t / (double)(total - 1) : 1.0;
        const float lr = (float)(s->o.lr_final + 0.5 * (s->o.lr - s->o.lr_final) * (1.0 + std::cos(M_PI * frac)));
        ++m.adam_t;
        const float c1 = 1.0f - std::pow(0.9f, (float)m.adam_t), c2 = 1.0f - std::pow(0.999f, (float)m.adam_t);
        k_adam<<<(kParams + 255) / 256, 256, 0, s->stream>>>(m.P, s->grad, m.M1, m.M2, kParams, lr, 0.9f, 0.999f,
                                                             1e-8f, c1, c2);
        if ((rc = pack(s, m)) != GELIO_OK) return rc;
      }
      if (ep == epochs - 1) {
        SUR_TRY(cudaMemcpyAsync(sl.data(), s->step_loss, sizeof(float) * steps, cudaMemcpyDeviceToHost, s->stream));
        SUR_TRY(cudaStreamSynchronize(s->stream));
        loss = 0.0;
        for (int st = 0; st < steps; ++st) loss += sl[st];
        loss /= (double)std::min<size_t>(nrow, (size_t)steps * R);
      }
    }
    int rc = check_error(s);
    if (rc != GELIO_OK) return rc;
    if (last_loss) last_loss[e] = (float)loss;
    m.trained = true;
  }
  return GELIO_OK;
}

// Every member on the first c rows of the inference batch (s->Q0, zero past
// c up to a whole tile) in one launch of the fused network kernel; member e's
// outputs go to y[e * stride + row].
int infer_fused(gelio_surrogate *s, int c, float *y, long long stride) {
  const int E = (int)s->mem.size();
  if (E > kFusedMaxMembers) return GELIO_ERR_UNSUPPORTED;
  FusedMaps maps;
  maps.q0 = s->mQ0;
  FusedArgs a{};
  for (int e = 0; e < E; ++e) {
    maps.w[e][0] = s->mem[e].mW1;
    for (int l = 0; l < 3; ++l) maps.w[e][l + 1] = s->mem[e].mW[l];
    a.P[e] = s->mem[e].P;
  }
  a.M = c;
  a.n_pairs = (c + 2 * kTileM - 1) / (2 * kTileM);
  a.E = E;
  a.stride = stride;
  a.y = y;
  a.error = s->error;
  a.timeout_ns = 2000000000ull;
  const int items = E * a.n_pairs;
  const int grid = std::max(1, std::min(items, s->sm_count));
  k_mlp_infer_fused<<<grid, kFusedThreads, kFusedSmem, s->stream>>>(maps, a);
  return cuda_status(cudaGetLastError());
}

// Ensemble inference of every LOG_GRID point of sims[0..n): the simulations
// and their row offsets go up (one copy from pinned staging), the features
// are built on the device per inference batch, every member's layers run on
// the batch, k_ensemble forms mean and std, and the two come back in one copy.
int infer_sims(gelio_surrogate *s, const gelio_sim_params *sims, int n, size_t rows, double *ln_ratio,
               double *ln_std) {
  const size_t E = s->mem.size();
  const size_t stride = (rows + kTileM - 1) / kTileM * kTileM;
  // device layout: [n] gelio_sim_params, [n + 1] row offsets (both uploaded
  // in one copy), then [n] QuerySim built on the device
  const size_t up = (size_t)n * sizeof(gelio_sim_params) + (size_t)(n + 1) * sizeof(long long);
  const size_t qoff = (up + 63) / 64 * 64;
  const size_t down = 2 * rows * sizeof(double);
  // the simulations and their row offsets travel in one copy, so they share
  // one allocation (n * 96 bytes keeps the offsets 8-byte aligned)
  const size_t dev_bytes = qoff + (size_t)n * sizeof(QuerySim);
  if (dev_bytes > s->pup_cap) {
    unsigned char *fresh = nullptr;
    SUR_TRY(gelio::dev_malloc(&fresh, dev_bytes));
    if (s->d_pup) cudaFree(s->d_pup);
    s->d_pup = fresh;
    s->pup_cap = dev_bytes;
  }
  const gelio_sim_params *d_psims = reinterpret_cast<const gelio_sim_params *>(s->d_pup);
  const long long *d_pfirst = reinterpret_cast<const long long *>(s->d_pup + (size_t)n * sizeof(gelio_sim_params));
  QuerySim *d_pq = reinterpret_cast<QuerySim *>(s->d_pup + qoff);
  if (stride > s->prows_cap) {
    if (s->d_py) cudaFree(s->d_py);
    if (s->d_pstat) cudaFree(s->d_pstat);
    s->d_py = nullptr;
    s->d_pstat = nullptr;
    s->prows_cap = 0;
    SUR_TRY(gelio::dev_malloc(&s->d_py, 16 * stride * sizeof(float)));
    SUR_TRY(gelio::dev_malloc(&s->d_pstat, 2 * stride * sizeof(double)));
    s->prows_cap = stride;
  }
  if (std::max(up, down) > s->pstage_cap) {
    if (s->h_pstage) cudaFreeHost(s->h_pstage);
    s->h_pstage = nullptr;
    s->pstage_cap = 0;
    SUR_TRY(gelio::pinned_malloc(&s->h_pstage, std::max(up, down)));
    s->pstage_cap = std::max(up, down);
  }
  std::memcpy(s->h_pstage, sims, (size_t)n * sizeof(gelio_sim_params));
  long long *first = reinterpret_cast<long long *>(s->h_pstage + (size_t)n * sizeof(gelio_sim_params));
  first[0] = 0;
  for (int i = 0; i < n; ++i) first[i + 1] = first[i] + sims[i].inj_points;
  SUR_TRY(cudaEventRecord(s->ev0, s->stream));
  SUR_TRY(cudaMemcpyAsync(s->d_pup, s->h_pstage, up, cudaMemcpyHostToDevice, s->stream));
  k_query_sims<<<(n + 127) / 128, 128, 0, s->stream>>>(d_psims, n, d_pq);
  SUR_TRY(cudaGetLastError());
  // the fused kernel adds the two column halves of each head output into y
  SUR_TRY(cudaMemsetAsync(s->d_py, 0, E * stride * sizeof(float), s->stream));
  size_t padded = 0;
  for (size_t off = 0; off < rows; off += (size_t)s->qrows) {
    const int c = (int)std::min<size_t>((size_t)s->qrows, rows - off);
    const int M = (c + kTileM - 1) / kTileM * kTileM;
    padded += (size_t)(c + 2 * kTileM - 1) / (2 * kTileM) * (2 * kTileM);   // rows the fused kernel multiplies
    k_query_features<<<(M + 127) / 128, 128, 0, s->stream>>>(d_pq, d_pfirst, n, (long long)off, c, M, s->Q0);
    SUR_TRY(cudaGetLastError());
    const int rc = infer_fused(s, c, s->d_py + off, (long long)stride);
    if (rc != GELIO_OK) return rc;
  }
  k_ensemble<<<(unsigned)((rows + 255) / 256), 256, 0, s->stream>>>(s->d_py, (int)E, (long long)rows,
                                                                    (long long)stride, s->d_pstat,
                                                                    s->d_pstat + rows);
  SUR_TRY(cudaGetLastError());
  SUR_TRY(cudaEventRecord(s->ev1, s->stream));
  SUR_TRY(cudaMemcpyAsync(s->h_pstage, s->d_pstat, down, cudaMemcpyDeviceToHost, s->stream));
  const int rc = check_error(s);
  if (rc != GELIO_OK) return rc;
  const double *st = reinterpret_cast<const double *>(s->h_pstage);
  std::memcpy(ln_ratio, st, rows * sizeof(double));
  if (ln_std) std::memcpy(ln_std, st + rows, rows * sizeof(double));
  float ms = 0.f;
  if (cudaEventElapsedTime(&ms, s->ev0, s->ev1) == cudaSuccess) {
    s->last_ms = ms;
    s->last_flop = 2.0 * (double)padded * (double)E *
                   ((double)kInPad * kWidth + 3.0 * kWidth * kWidth + (double)kWidth);
  }
  return GELIO_OK;
}

int32_t gelio_surrogate_forward(gelio_surrogate *s, int32_t member, const float *x, int32_t n, float *y) {
  if (!valid_member(s, member) || n < 0 || (n > 0 && (!x || !y))) return GELIO_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(s->mu);
  SUR_TRY(cudaSetDevice(s->device));
  (void)cudaGetLastError();   // a launch check below must see only this call's errors
  return infer_rows(s, member, member + 1, x, (size_t)n, y);
}

int32_t gelio_surrogate_gradient(gelio_surrogate *s, int32_t member, const float *x, const float *t, int32_t n,
                                 float *loss, float *grad) {
  if (!valid_member(s, member) || n <= 0 || !x || !t || !grad) return GELIO_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(s->mu);
  if (n > s->rows) return GELIO_ERR_INVALID_ARGUMENT;
  SUR_TRY(cudaSetDevice(s->device));
  (void)cudaGetLastError();   // a launch check below must see only this call's errors
  float *d_x = nullptr, *d_t = nullptr, *d_loss = nullptr;
  int rc = GELIO_OK;
  if (gelio::dev_malloc(&d_x, (size_t)n * kFeatures * 4) != cudaSuccess || gelio::dev_malloc(&d_t, (size_t)n * 4) != cudaSuccess ||
      gelio::dev_malloc(&d_loss, 4) != cudaSuccess)
    rc = GELIO_ERR_OUT_OF_MEMORY;
  if (rc == GELIO_OK && (cudaMemcpyAsync(d_x, x, (size_t)n * kFeatures * 4, cudaMemcpyHostToDevice, s->stream) !=
                             cudaSuccess ||
                         cudaMemcpyAsync(d_t, t, (size_t)n * 4, cudaMemcpyHostToDevice, s->stream) != cudaSuccess))
    rc = GELIO_ERR_CUDA;
  if (rc == GELIO_OK) rc = stage_rows(s, d_x, d_t, n);
  if (rc == GELIO_OK) rc = forward_backward(s, s->mem[member], n, d_loss);
  float l = 0.f;
  if (rc == GELIO_OK &&
      (cudaMemcpyAsync(grad, s->grad, (size_t)kParams * 4, cudaMemcpyDeviceToHost, s->stream) != cudaSuccess ||
       cudaMemcpyAsync(&l, d_loss, 4, cudaMemcpyDeviceToHost, s->stream) != cudaSuccess))
    rc = GELIO_ERR_CUDA;
  if (rc == GELIO_OK) rc = check_error(s);
  cudaStreamSynchronize(s->stream);
  if (loss) *loss = l / (float)n;
  cudaFree(d_x);
  cudaFree(d_t);
  cudaFree(d_loss);
  return rc;
}

int32_t gelio_surrogate_last_inference(gelio_surrogate *s, double *device_ms, double *flop) {
  if (!s) return GELIO_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(s->mu);
  if (device_ms) *device_ms = s->last_ms;
  if (flop) *flop = s->last_flop;
  return GELIO_OK;
}

int32_t gelio_surrogate_get_params(gelio_surrogate *s, int32_t member, float *params) {
  if (!valid_member(s, member) || !params) return GELIO_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(s->mu);
  SUR_TRY(cudaSetDevice(s->device));
  (void)cudaGetLastError();   // a launch check below must see only this call's errors
  SUR_TRY(cudaMemcpyAsync(params, s->mem[member].P, (size_t)kParams * 4, cudaMemcpyDeviceToHost, s->stream));
  SUR_TRY(cudaStreamSynchronize(s->stream));
  return GELIO_OK;
}

int32_t gelio_surrogate_set_params(gelio_surrogate *s, int32_t member, const float *params) {
  if (!valid_member(s, member) || !params) return GELIO_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(s->mu);
  SUR_TRY(cudaSetDevice(s->device));
  (void)cudaGetLastError();   // a launch check below must see only this call's errors
  Member &m = s->mem[member];
  SUR_TRY(cudaMemcpyAsync(m.P, params, (size_t)kParams * 4, cudaMemcpyHostToDevice, s->stream));
  SUR_TRY(cudaMemsetAsync(m.M1, 0, (size_t)kParams * 4, s->stream));
  SUR_TRY(cudaMemsetAsync(m.M2, 0, (size_t)kParams * 4, s->stream));
  m.adam_t = 0;
  int rc = pack(s, m);
  if (rc != GELIO_OK) return rc;
  SUR_TRY(cudaStreamSynchronize(s->stream));
  m.trained = true;
  return GELIO_OK;
}

int32_t gelio_surrogate_predict(gelio_surrogate *s, const gelio_sim_params *sims, int32_t n, double *ln_ratio,
                                double *ln_std) {
  if (!s || n < 0 || (n > 0 && (!sims || !ln_ratio))) return GELIO_ERR_INVALID_ARGUMENT;
  for (auto &m : s->mem)
    if (!m.trained) return GELIO_ERR_NOT_TRAINED;
  size_t rows = 0;
  for (int i = 0; i < n; ++i) {
    if (sims[i].injection != GELIO_INJ_LOG_GRID || sims[i].inj_points < 1 || sims[i].inj_points > GELIO_GRID_MAX ||
        !(sims[i].inj_min > 0.f) || !(sims[i].inj_max > 0.f))
      return GELIO_ERR_INVALID_ARGUMENT;
    rows += (size_t)sims[i].inj_points;
  }
  if (rows == 0) return GELIO_OK;
  std::lock_guard<std::mutex> lock(s->mu);
  SUR_TRY(cudaSetDevice(s->device));
  (void)cudaGetLastError();   // a launch check below must see only this call's errors
  return infer_sims(s, sims, n, rows, ln_ratio, ln_std);
}

int32_t gelio_surrogate_spectra(gelio_surrogate *s, const gelio_sim_params *sims, int32_t n,
                                const gelio_run_opts *mc_opts, double *ln_ratio, double *ln_std, int32_t *used_mc) {
  if (!s || n < 0 || (n > 0 && (!sims || !ln_ratio || !ln_std))) return GELIO_ERR_INVALID_ARGUMENT;
  int rc = gelio_surrogate_predict(s, sims, n, ln_ratio, ln_std);
  if (rc != GELIO_OK) return rc;
  std::vector<int> need;
  std::vector<size_t> first(n + 1, 0);
  for (int i = 0; i < n; ++i) first[i + 1] = first[i] + (size_t)sims[i].inj_points;
  for (int i = 0; i < n; ++i) {
    double worst = 0.0;
    for (int j = 0; j < sims[i].inj_points; ++j) {
      const double T = grid_energy(sims[i], j);
      if (T >= s->o.t_min && T <= s->o.t_max) worst = std::max(worst, ln_std[first[i] + j]);
    }
    const bool mc = worst > s->o.fallback_std;
    if (used_mc) used_mc[i] = mc ? 1 : 0;
    if (mc) need.push_back(i);
  }
  if (need.empty()) return GELIO_OK;
  std::vector<gelio_sim_params> sub;
  for (int i : need) sub.push_back(sims[i]);
  std::vector<gelio_spectra> out(sub.size());
  rc = gelio_run(s->ctx, sub.data(), (int32_t)sub.size(), mc_opts, out.data(), nullptr);
  if (rc != GELIO_OK && rc < GELIO_WARN_FIRST) return rc;
  for (size_t k = 0; k < need.size(); ++k) {
    const int i = need[k];
    for (int j = 0; j < sims[i].inj_points; ++j) {
      const double cnt = out[k].grid_n[j], w = out[k].grid_w[s->o.lis][j];
      const double T = grid_energy(sims[i], j);
      ln_ratio[first[i] + j] = (cnt > 0 && w > 0) ? std::log((w / cnt) / lis(s->o.lis, T)) : NAN;
      ln_std[first[i] + j] = 0.0;
    }
  }
  return GELIO_OK;
}

}  // extern "C"
