// Persistent and plain SDE kernels, templated on the model and precision.
//
// Persistent kernel (the default path): one CTA per SM slot, every lane owns
// one trajectory at a time.  Lanes whose particle has ended are refilled at
// warp level every `refill` steps: a ballot of idle lanes, one 64-bit
// atomicAdd per warp on the model's ticket counter, and each idle lane takes
// ticket base + rank.  Tickets run over all particles of all simulations of
// the model in the launch (a whole batch CSV in one launch); the ticket ->
// (simulation, particle) map is a binary search of the particle prefix sums.
// This replaces the reference's host loop of 4,096-particle chunks with three
// device synchronisations each (GeliosphereModel.cu:426-445), and its
// warp-wide wait for the slowest particle.
//
// Exits are evaluated in the kernel (evaluation.cuh) and accumulated, per
// warp, by key (simulation, injection energy): lanes with the same key are
// combined with __match_any_sync + shuffles and one lane adds the sums into a
// per-CTA shared-memory histogram (FP64 sum, sum of squares and count per
// bin).  At the end each CTA adds its histogram into one of S global slices;
// a reduce kernel sums the slices with Neumaier compensation.
#pragma once
#include <cstdint>
#include "gelio.h"
#include "philox.cuh"
#include "physics.cuh"
#include "evaluation.cuh"

namespace gelio {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kMaxSims = 65536;

// Launch-wide control block (device memory, zeroed per run).
struct Control {
  unsigned long long ticket[4];
  unsigned long long rec_count;
  unsigned long long rec_dropped;
  unsigned int status;
  unsigned int abort;
  int bad_sim;
  int pad;
  unsigned long long group_count[4];
  unsigned long long t_start;      // %globaltimer when the prepare kernel ran
};

// Simulation grouping by model, written by the prepare kernel.
struct Groups {
  int *sim_idx;                   // [4][n_sims]: simulation indices of model m
  unsigned long long *prefix;     // [4][n_sims + 1]: particle prefix sums
};

struct KArgs {
  const SimDev *sims;
  const float *inj_tables;        // [n_sims][GELIO_GRID_MAX] LOG_GRID energies
  Groups groups;
  int n_sims;
  int n_slices;
  double *part;                   // [n_slices][n_sims][kSpecDoubles]
  Control *ctl;
  gelio_exit_record *records;     // optional
  unsigned long long record_capacity;
  unsigned long long max_steps;
  unsigned long long time_limit_ns; // 0 = no watchdog
  int smem_slots;                 // >0: histograms of the group's first smem_slots sims in shared memory
  int refill;                     // steps between refills (multiple of 4)
  // plain / replay kernel
  int plain_sim;                  // simulation index of a plain launch
  unsigned long long plain_first, plain_count;
  gelio_trajectory *replay;       // optional per-particle output
};

// Bin tables; every translation unit holds its own copy (no relocatable
// device code), filled through set_tables_tu().
static __constant__ BinTables c_tables;
static inline cudaError_t set_tables_tu(const BinTables &t) {
  return cudaMemcpyToSymbol(c_tables, &t, sizeof(BinTables));
}

__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Window of gelio_spectra that a model touches in shared memory.
template <int MODEL> struct Window {
  static constexpr int lo = (MODEL >= kModelSolarProp) ? kWin2DLo : kWin1DLo;
  static constexpr int size = kWinHi - lo;
};

// Histogram sink of one CTA: shared memory for the first smem_slots group
// simulations, otherwise the CTA's global slice.
template <int MODEL> struct Sink {
  double *sh;          // shared window array, or nullptr
  int smem_slots;
  double *slice;       // this CTA's slice: [n_sims][kSpecDoubles]
  __device__ __forceinline__ void add(int slot, int sim, int off, double v) const {
    if (slot < smem_slots) atomicAdd(&sh[slot * Window<MODEL>::size + (off - Window<MODEL>::lo)], v);
    else atomicAdd(&slice[(size_t)sim * kSpecDoubles + off], v);
  }
};

// Injection energy of particle pid of simulation sd.
__device__ __forceinline__ float injection_energy(const SimDev &sd, const float *table,
                                                  unsigned long long pid) {
  switch (sd.injection) {
    case GELIO_INJ_REFERENCE_UNIFORM: return inj_reference_uniform(pid, sd.injection_max);
    case GELIO_INJ_SOLARPROP_GRID: return inj_solarprop(pid, c_tables.sp30);
    case GELIO_INJ_LOG_GRID: return table[pid % (unsigned long long)sd.inj_points];
    case GELIO_INJ_LOG_UNIFORM: {
      Philox4 c; c.x = 0u; c.y = kStreamInjection; c.z = (uint32_t)pid; c.w = (uint32_t)(pid >> 32);
      const Philox4 o = philox4x32_10(c, sd.key0, sd.key1);
      const double u = ((double)o.x + 0.5) * 2.3283064365386963e-10;
      const double lmin = log((double)sd.inj_min), lmax = log((double)sd.inj_max);
      return (float)exp(lmin + u * (lmax - lmin));
    }
    default: return inj_cpu_uniform(pid, sd.injection_max);
  }
}

template <int MODEL, class R>
__device__ __forceinline__ void init_lane(Lane<R> &L, Consts<R> &K, const SimDev &sd,
                                          const float *table, int sim, unsigned long long pid) {
  make_consts(sd, K);
  L.sim = sim;
  L.pid = pid;
  L.key0 = sd.key0;
  L.key1 = sd.key1;
  L.steps = 0;
  const float Tinj = injection_energy(sd, table, pid);
  L.Tinj = Tinj;
  L.T.set((R)Tinj);
  const R T0 = (R)kT0;
  L.thn = 0.0f;
  if constexpr (MODEL == kModelGeliosphere || MODEL == kModelSolarProp) {
    L.r.set((R)sd.r_inj);
    L.th.set((R)sd.theta_inj);
  } else if constexpr (MODEL == kModelBp) {
    L.r.set((R)sd.r_inj);
    L.P.set(Math<R>::sqrt((R)Tinj * ((R)Tinj + R(2) * T0)));
    L.Pt = L.P.v;
    L.q = Math<R>::rsqrt(L.Pt * L.Pt + T0 * T0);
  } else {
    L.r.set((R)100.0001f);
    L.P.set(Math<R>::sqrt((R)Tinj * ((R)Tinj + R(2) * T0)));
    L.Pt = L.P.v;
    L.q = Math<R>::rsqrt(L.Pt * L.Pt + T0 * T0);
    L.sumac.set(R(0));
  }
  if (sd.grid_is_points) L.gbin = (int)(pid % (unsigned long long)sd.inj_points);
  else L.gbin = grid_log_bin((double)Tinj, sd.grid_log_lo, sd.grid_inv_dlog, sd.grid_bins);
}

// Pending exit of a lane (2D / B-p models).
struct Pending {
  float Tinj, Texit, r, aux;
  int sim, slot, gbin;
  unsigned long long pid;
};

__device__ __forceinline__ void append_records(const KArgs &a, unsigned mask, const Pending &p, int model) {
  if (a.records == nullptr) return;
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(mask) - 1;
  unsigned long long base = 0;
  if (lane == leader) base = atomicAdd(&a.ctl->rec_count, (unsigned long long)__popc(mask));
  base = __shfl_sync(mask, base, leader);
  const unsigned long long idx = base + __popc(mask & lanemask_lt());
  if (idx < a.record_capacity) {
    gelio_exit_record rec;
    rec.particle = (int64_t)p.pid;
    rec.sim = p.sim;
    rec.t_injection = p.Tinj;
    rec.t_exit = p.Texit;
    rec.r = p.r;
    rec.theta = (model >= kModelSolarProp) ? p.aux : 0.0f;
    rec.sumac = (model == kModelFp) ? p.aux : 0.0f;
    a.records[idx] = rec;
  }
  if (lane == leader) {
    const unsigned long long n = (unsigned long long)__popc(mask);
    const unsigned long long room = (base < a.record_capacity) ? a.record_capacity - base : 0ull;
    if (n > room) atomicAdd(&a.ctl->rec_dropped, n - room);
  }
}

// Append one exit record (any lane, no warp synchronisation).
template <class R>
__device__ __forceinline__ void append_record_one(const KArgs &a, const Lane<R> &L, int model) {
  const unsigned long long idx = atomicAdd(&a.ctl->rec_count, 1ull);
  if (idx < a.record_capacity) {
    gelio_exit_record rec;
    rec.particle = (int64_t)L.pid;
    rec.sim = L.sim;
    rec.t_injection = L.Tinj;
    rec.t_exit = (float)L.T.v;
    rec.r = (float)L.r.v;
    rec.theta = (model >= kModelSolarProp) ? (float)theta_full(L) : 0.0f;
    rec.sumac = 0.0f;
    a.records[idx] = rec;
  } else {
    atomicAdd(&a.ctl->rec_dropped, 1ull);
  }
}

// Warp-aggregated flush of the pending exits of the lanes in `mask` (all of
// which execute this call).  Backward models only.
template <int MODEL>
__device__ __noinline__ void flush_pending(const Sink<MODEL> &sink, unsigned mask, const Pending &p) {
  constexpr int NV = 13;   // w[3], w2[3], gw[3], gw2[3], count
  const int lane = threadIdx.x & 31;
  Contribution C;
  const double Ti = round6((double)p.Tinj);
  const double Te = round6((double)p.Texit);
  if constexpr (MODEL >= kModelSolarProp) eval_2d(Ti, Te, c_tables, C);
  else eval_bp(Ti, Te, c_tables, C);
  double v[NV];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    v[j] = C.w[j];
    v[3 + j] = C.w[j] * C.w[j];
    v[6 + j] = C.gw[j];
    v[9 + j] = C.gw[j] * C.gw[j];
  }
  v[12] = 1.0;
  const unsigned long long key = ((unsigned long long)(unsigned)p.sim << 32) | __float_as_uint(p.Tinj);
  const unsigned peers = __match_any_sync(mask, key);
  const int leader = __ffs(peers) - 1;
  double acc[NV];
#pragma unroll
  for (int j = 0; j < NV; ++j) acc[j] = v[j];
  if (__popc(mask) > 1) {
    for (unsigned m = mask; m; m &= m - 1) {
      const int src = __ffs(m) - 1;
#pragma unroll
      for (int j = 0; j < NV; ++j) {
        const double x = __shfl_sync(mask, v[j], src);
        if (lane == leader && src != lane && ((peers >> src) & 1u)) acc[j] += x;
      }
    }
  }
  if (lane == leader) {
    const int s = p.sim, sl = p.slot;
    const double cnt = acc[12];
    if constexpr (MODEL >= kModelSolarProp) {
      if (C.b_sp) {
        sink.add(sl, s, kOffSpWeber + C.b_sp, acc[0]);
        sink.add(sl, s, kOffSpJgr + C.b_sp, acc[1]);
        sink.add(sl, s, kOffSpBurger + C.b_sp, acc[2]);
        sink.add(sl, s, kOffSpWeber2 + C.b_sp, acc[3]);
        sink.add(sl, s, kOffSpJgr2 + C.b_sp, acc[4]);
        sink.add(sl, s, kOffSpBurger2 + C.b_sp, acc[5]);
        sink.add(sl, s, kOffSpN + C.b_sp, cnt);
      }
      if (C.b_uly) {
        sink.add(sl, s, kOffUlyW + C.b_uly, acc[2]);
        sink.add(sl, s, kOffUlyW2 + C.b_uly, acc[5]);
        sink.add(sl, s, kOffUlyN + C.b_uly, cnt);
      }
      if (C.b_ams) {
        sink.add(sl, s, kOffAmsW + C.b_ams, acc[2]);
        sink.add(sl, s, kOffAmsW2 + C.b_ams, acc[5]);
        sink.add(sl, s, kOffAmsN + C.b_ams, cnt);
      }
    } else {
      if (C.b_log >= 0) {
        sink.add(sl, s, kOffLogW + C.b_log, acc[0]);
        sink.add(sl, s, kOffLogW2 + C.b_log, acc[3]);
        sink.add(sl, s, kOffLogN + C.b_log, cnt);
      }
      if (C.b_e2) {
        sink.add(sl, s, kOffE2W + C.b_e2 - 1, acc[0]);
        sink.add(sl, s, kOffE2W2 + C.b_e2 - 1, acc[3]);
        sink.add(sl, s, kOffE2N + C.b_e2 - 1, cnt);
      }
      if (C.b_e3) {
        sink.add(sl, s, kOffE3W + C.b_e3 - 1, acc[0]);
        sink.add(sl, s, kOffE3W2 + C.b_e3 - 1, acc[3]);
        sink.add(sl, s, kOffE3N + C.b_e3 - 1, cnt);
      }
      if (C.b_e4) {
        sink.add(sl, s, kOffE4W + C.b_e4 - 1, acc[0]);
        sink.add(sl, s, kOffE4W2 + C.b_e4 - 1, acc[3]);
        sink.add(sl, s, kOffE4N + C.b_e4 - 1, cnt);
      }
    }
    if (p.gbin >= 0) {
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        sink.add(sl, s, kOffGridW + j * GELIO_GRID_MAX + p.gbin, acc[6 + j]);
        sink.add(sl, s, kOffGridW2 + j * GELIO_GRID_MAX + p.gbin, acc[9 + j]);
      }
      sink.add(sl, s, kOffGridN + p.gbin, cnt);
    }
    sink.add(sl, s, kOffNRecords, cnt);
  }
}

// Per-warp queue of exits awaiting evaluation (shared memory).  Lanes push
// their exit and take a new particle at once; when 32 exits are queued the
// warp evaluates them with every lane busy, so the FP64 evaluation is paid
// once per 32 exits instead of once per window with a lane or two active.
struct QEnt {
  float Tinj, Texit;
  int sim;
  unsigned slot_gbin;        // group slot (low 16 bits), grid bin + 1 (high 16 bits)
};
constexpr int kQueue = 64;   // entries per warp (<= 31 left + 32 pushed)
// F-p: at most this many running trajectories in a warp whose tickets are
// exhausted switch to normals drawn by the whole warp (>= 4 groups ahead each)
constexpr int kCoopLanes = 8;
static_assert(32 * 4 * sizeof(double) <= kQueue * sizeof(QEnt), "cooperative normals fit a warp's queue area");

template <int MODEL>
__device__ __forceinline__ void flush_queue(const KArgs &a, const Sink<MODEL> &sink, const QEnt *q,
                                            int base, int count) {
  const int lane = threadIdx.x & 31;
  const unsigned mask = (count >= 32) ? kFull : ((1u << count) - 1u);
  if (lane < count) {
    const QEnt e = q[base + lane];
    Pending p;
    p.Tinj = e.Tinj;
    p.Texit = e.Texit;
    p.sim = e.sim;
    p.slot = (int)(e.slot_gbin & 0xffffu);
    p.gbin = (int)(e.slot_gbin >> 16) - 1;
    flush_pending<MODEL>(sink, mask, p);
  }
}

// Direct (non-aggregated) F-p record of one 1 AU crossing, passed by value:
// a reference to the lane, the simulation or the kernel arguments would put
// them in local memory for the whole step loop (the call is out of line),
// lengthening every step.
struct FpCrossing {
  float Tinj, Texit, rrec, sumac;
  int sim, slot, grid_bins;
  unsigned long long pid;
  double grid_log_lo, grid_inv_dlog;
};

template <class R>
__device__ __forceinline__ FpCrossing fp_crossing(const Lane<R> &L, const SimDev &sd, int slot) {
  FpCrossing x;
  x.Tinj = L.Tinj;
  x.Texit = (float)L.T.v;
  x.rrec = L.rrec;
  x.sumac = (float)L.sumac.v;
  x.sim = L.sim;
  x.slot = slot;
  x.grid_bins = sd.grid_bins;
  x.pid = L.pid;
  x.grid_log_lo = sd.grid_log_lo;
  x.grid_inv_dlog = sd.grid_inv_dlog;
  return x;
}

static __device__ __noinline__ void emit_fp(Control *ctl, gelio_exit_record *records,
                                     unsigned long long record_capacity, Sink<kModelFp> sink,
                                     FpCrossing x) {
  const double p100 = round6(p_si((double)x.Tinj));
  const double p1 = round6(p_si((double)x.Texit));
  const double rr = round6((double)x.rrec);
  const double sm = round6((double)x.sumac);
  Contribution C;
  double T1;
  eval_fp(p100, p1, rr, sm, c_tables, C, T1);
  const int s = x.sim, slot = x.slot;
  const double w = C.w[0], w2 = w * w;
  if (C.b_log >= 0) { sink.add(slot, s, kOffLogW + C.b_log, w); sink.add(slot, s, kOffLogW2 + C.b_log, w2); sink.add(slot, s, kOffLogN + C.b_log, 1.0); }
  if (C.b_e2) { sink.add(slot, s, kOffE2W + C.b_e2 - 1, w); sink.add(slot, s, kOffE2W2 + C.b_e2 - 1, w2); sink.add(slot, s, kOffE2N + C.b_e2 - 1, 1.0); }
  if (C.b_e3) { sink.add(slot, s, kOffE3W + C.b_e3 - 1, w); sink.add(slot, s, kOffE3W2 + C.b_e3 - 1, w2); sink.add(slot, s, kOffE3N + C.b_e3 - 1, 1.0); }
  if (C.b_e4) { sink.add(slot, s, kOffE4W + C.b_e4 - 1, w); sink.add(slot, s, kOffE4W2 + C.b_e4 - 1, w2); sink.add(slot, s, kOffE4N + C.b_e4 - 1, 1.0); }
  const int gb = grid_log_bin(T1, x.grid_log_lo, x.grid_inv_dlog, x.grid_bins);
  if (gb >= 0) {
    sink.add(slot, s, kOffGridW + gb, w);
    sink.add(slot, s, kOffGridW2 + gb, w2);
    sink.add(slot, s, kOffGridN + gb, 1.0);
  }
  sink.add(slot, s, kOffNRecords, 1.0);
  if (records != nullptr) {
    const unsigned long long idx = atomicAdd(&ctl->rec_count, 1ull);
    if (idx < record_capacity) {
      gelio_exit_record rec;
      rec.particle = (int64_t)x.pid;
      rec.sim = s;
      rec.t_injection = x.Tinj;
      rec.t_exit = x.Texit;
      rec.r = x.rrec;
      rec.theta = 0.0f;
      rec.sumac = x.sumac;
      records[idx] = rec;
    } else {
      atomicAdd(&ctl->rec_dropped, 1ull);
    }
  }
}

// Advance one lane by one step of MODEL; normals are drawn per step group.
// Returns the step result; `z` carries the per-call normals.
template <int MODEL, class R>
__device__ __forceinline__ int model_step(Lane<R> &L, const Consts<R> &K, const R *z, int j) {
  if constexpr (MODEL == kModelGeliosphere) return step_geliosphere(L, K, z[0], z[1], z[2]);
  else if constexpr (MODEL == kModelSolarProp) return step_solarprop(L, K, z[2 * j], z[2 * j + 1]);
  else if constexpr (MODEL == kModelBp) return step_bp(L, K, z[j]);
  else return step_fp(L, K, z[j]);
}

template <int MODEL> struct StepsPerCall {
  static constexpr int value = (MODEL == kModelGeliosphere) ? 1 : (MODEL == kModelSolarProp) ? 2 : 4;
};

// 2D Geliosphere draws three normals per step (the reference's other two
// multiply B13 = B23 = 0).  Each group of four steps takes its twelve normals
// from three Philox calls, counters 3 g, 3 g + 1, 3 g + 2 for group
// g = step / 4: step 4 g + p uses normals 3 p .. 3 p + 2 of the group, and
// the ones a call draws ahead are carried in the lane.  Particles start only
// at refill boundaries (multiples of four steps), so the lanes of a warp
// share the phase p and the fourth step's skipped draw is warp-uniform.
template <class R>
__device__ __forceinline__ void draw_geliosphere(Lane<R> &L, R *z) {
  const uint32_t p = L.steps & 3u;
  R a[4] = {R(0), R(0), R(0), R(0)};
  if (p != 3u) normals4<R>(L.key0, L.key1, 3u * (L.steps >> 2) + p, kStreamSde, L.pid, a);
  if (p == 0u) {
    z[0] = a[0]; z[1] = a[1]; z[2] = a[2]; L.zc0 = a[3];
  } else if (p == 1u) {
    z[0] = L.zc0; z[1] = a[0]; z[2] = a[1]; L.zc0 = a[2]; L.zc1 = a[3];
  } else if (p == 2u) {
    z[0] = L.zc0; z[1] = L.zc1; z[2] = a[0]; L.zc0 = a[1]; L.zc1 = a[2]; L.zc2 = a[3];
  } else {
    z[0] = L.zc0; z[1] = L.zc1; z[2] = L.zc2;
  }
}

template <int MODEL, class R>
__device__ __forceinline__ void draw(Lane<R> &L, R *z) {
  if constexpr (MODEL == kModelGeliosphere) {
    draw_geliosphere<R>(L, z);
  } else {
    constexpr int spc = StepsPerCall<MODEL>::value;
    normals4<R>(L.key0, L.key1, L.steps / spc, kStreamSde, L.pid, z);
  }
}

// The 1D models draw the normals of their next group of four steps while the
// current group integrates: the Philox rounds and Box-Muller do not depend
// on the trajectory, so they fill the latency of the step's dependent chain.
template <int MODEL> struct Prefetch {
  static constexpr bool value = (MODEL == kModelFp || MODEL == kModelBp);
};

template <int MODEL, class R>
__device__ __forceinline__ void draw_group(const Lane<R> &L, uint32_t group, R *z) {
  normals4<R>(L.key0, L.key1, group, kStreamSde, L.pid, z);
}

// Particle handed out by the u-th ticket of a simulation of n particles.
// On a grid injection (particle i takes grid point i mod P, the energies
// ascending with the point) the tickets walk the points in ascending order:
// the lowest energies, whose trajectories are the longest, start first and
// the run does not end waiting for a long trajectory that started late.
// Every particle is still handed out exactly once, and a trajectory depends
// only on its index, so the results do not change.
__device__ __forceinline__ unsigned long long ticket_particle(unsigned long long u, unsigned long long n,
                                                              unsigned long long P) {
  // (32-bit arithmetic; a simulation of 2^32 particles or more keeps index order)
  if (P <= 1 || n <= P || n > 0xffffffffull) return u;
  const uint32_t uu = (uint32_t)u, p = (uint32_t)P;
  const uint32_t qv = (uint32_t)n / p, rm = (uint32_t)n % p;   // points g < rm hold qv + 1 particles
  const uint32_t head = rm * (qv + 1u);
  uint32_t g, k;
  if (uu < head) {
    g = uu / (qv + 1u);
    k = uu - g * (qv + 1u);
  } else {
    const uint32_t v = uu - head;
    g = rm + v / qv;
    k = v - (g - rm) * qv;
  }
  return (unsigned long long)g + (unsigned long long)p * k;
}

__device__ __forceinline__ unsigned long long grid_points(const SimDev &sd) {
  if (sd.injection == GELIO_INJ_LOG_GRID) return (unsigned long long)sd.inj_points;
  if (sd.injection == GELIO_INJ_SOLARPROP_GRID) return 30ull;
  return 0ull;
}

__device__ __forceinline__ int find_group_index(const unsigned long long *prefix, int n,
                                                unsigned long long t, int hint) {
  if (hint >= 0 && hint < n && prefix[hint] <= t && t < prefix[hint + 1]) return hint;
  int lo = 0, hi = n - 1;          // largest g with prefix[g] <= t
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (prefix[mid] <= t) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// ---------------------------------------------------------------------------
// Persistent kernel.
// ---------------------------------------------------------------------------
// MINB: CTAs of 256 threads the register budget is sized for (2: <= 128
// registers; 3: <= 85 registers with some spilling); picked by the autotuner.
template <int MODEL, class R, int MINB>
__global__ void __launch_bounds__(256, MINB) k_persistent(const KArgs a) {
  extern __shared__ double sh_hist[];
  const int gn = (int)a.ctl->group_count[MODEL];
  if (gn == 0 || a.ctl->status != 0) return;
  const int *gsim = a.groups.sim_idx + (size_t)MODEL * a.n_sims;
  const unsigned long long *gpre = a.groups.prefix + (size_t)MODEL * (a.n_sims + 1);
  const unsigned long long total = gpre[gn];
  const int slots = (gn <= a.smem_slots) ? gn : 0;
  constexpr int W = Window<MODEL>::size;
  for (int i = threadIdx.x; i < slots * W; i += blockDim.x) sh_hist[i] = 0.0;
  // the exit queues and their lengths follow the histogram window (sized
  // for a.smem_slots)
  QEnt *qbase = reinterpret_cast<QEnt *>(sh_hist + (size_t)a.smem_slots * W);
  QEnt *q = qbase + (threadIdx.x >> 5) * kQueue;
  int *qlen = reinterpret_cast<int *>(qbase + (blockDim.x >> 5) * kQueue) + (threadIdx.x >> 5);
  if ((threadIdx.x & 31) == 0) *qlen = 0;
  __syncthreads();
  Sink<MODEL> sink;
  sink.sh = sh_hist;
  sink.smem_slots = slots;
  sink.slice = a.part + (size_t)(blockIdx.x % a.n_slices) * a.n_sims * kSpecDoubles;

  const int lane = threadIdx.x & 31;
  Lane<R> L;
  Consts<R> K;
  SimDev sd;
  bool active = false, drained = false;
  // 1D models, warp-uniform: every ticket is handed out, so no lane of this
  // warp will be refilled again and the window grows to cut the votes
  bool exhausted = false;
  int slot = 0, g = -1;
  unsigned window = 0;
  R zq[4] = {R(0), R(0), R(0), R(0)};     // 1D models: normals of the lane's next step group

  for (;;) {
    // 1) evaluate and bin queued exits, 32 at a time with every lane busy
    if constexpr (MODEL != kModelFp) {
      __syncwarp();
      const int qn = *(volatile int *)qlen;
      if (qn >= 32) {
        flush_queue<MODEL>(a, sink, q, qn - 32, 32);
        __syncwarp();
        if (lane == 0) *qlen = qn - 32;
        __syncwarp();
      }
    }
    // 2) refill idle lanes from the ticket counter
    unsigned ab = 0;
    if (a.time_limit_ns != 0ull && (window & 7u) == 0u) {
      if (lane == 0) {
        ab = *(volatile unsigned *)&a.ctl->abort;
        if (!ab && globaltimer_ns() - a.ctl->t_start > a.time_limit_ns) {
          atomicExch(&a.ctl->abort, 1u);
          atomicCAS(&a.ctl->status, 0u, (unsigned)GELIO_ERR_TIMEOUT);
          ab = 1;
        }
      }
      ab = __shfl_sync(kFull, ab, 0);
      if (ab) {
        if (active) { sink.add(slot, L.sim, kOffNSteps, (double)L.steps); }
        active = false;
        drained = true;
      }
    }
    ++window;
    const unsigned need = __ballot_sync(kFull, !active && !drained);
    if (need) {
      const int leader = __ffs(need) - 1;
      unsigned long long base = 0;
      if (lane == leader) base = atomicAdd(&a.ctl->ticket[MODEL], (unsigned long long)__popc(need));
      base = __shfl_sync(kFull, base, leader);
      if (Prefetch<MODEL>::value && base + (unsigned long long)__popc(need) >= total) exhausted = true;
      if (!active && !drained) {
        const unsigned long long t = base + __popc(need & lanemask_lt());
        if (t < total) {
          g = find_group_index(gpre, gn, t, g);
          const int sim = gsim[g];
          sd = a.sims[sim];
          slot = g;
          const unsigned long long pid = ticket_particle(t - gpre[g], gpre[g + 1] - gpre[g], grid_points(sd));
          init_lane<MODEL, R>(L, K, sd, a.inj_tables + (size_t)sim * GELIO_GRID_MAX, sim, pid);
          if constexpr (Prefetch<MODEL>::value) draw_group<MODEL, R>(L, 0u, zq);
          sink.add(slot, sim, kOffNParticles, 1.0);
          active = true;
        } else {
          drained = true;
        }
      }
    }
    if (!__any_sync(kFull, active)) {
      if constexpr (MODEL != kModelFp) {
        const int qn = *(volatile int *)qlen;
        if (qn > 0) flush_queue<MODEL>(a, sink, q, 0, qn);
      }
      break;
    }
    // 3) integrate `refill` steps (1D: at least 64 once the tickets are exhausted)
    constexpr int spc = StepsPerCall<MODEL>::value;
    const int win = (Prefetch<MODEL>::value && exhausted && a.refill < 64) ? 64 : a.refill;
    const uint32_t cap32 = (a.max_steps > 0xffffffffull) ? 0xffffffffu : (uint32_t)a.max_steps;
    // F-p runs end on the latency of their longest chain: one test per step
    // covers the rare events (a crossing record, a stop, the step cap), and a
    // stopped lane leaves its group of four steps at once
    auto fp_group = [&](const R *z) {
      if constexpr (MODEL == kModelFp) {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int res = step_fp(L, K, z[j]);
          ++L.steps;
          if (res != kContinue || L.steps >= cap32) {
            if (res == kRecordAndContinue || res == kRecordAndStop)
              emit_fp(a.ctl, a.records, a.record_capacity, sink, fp_crossing(L, sd, slot));
            if (res == kRecordAndStop || res == kStop) {
              active = false;
              sink.add(slot, L.sim, kOffNSteps, (double)L.steps);
            } else if (L.steps >= cap32) {
              active = false;
              sink.add(slot, L.sim, kOffNSteps, (double)L.steps);
              sink.add(slot, L.sim, kOffNCapped, 1.0);
            }
            if (!active) break;
          }
        }
      }
    };
    if constexpr (MODEL == kModelFp) {
      // The tail of an F-p run: this warp's tickets are exhausted and at most
      // kCoopLanes of its trajectories still run (often one chain of ~10^6
      // steps).  A trajectory's normals depend only on (key, particle, group
      // of four steps), so every lane of the warp draws one group for one of
      // the running trajectories -- 32 / n groups ahead for each of n -- into
      // the warp's exit-queue area (F-p queues no exits), and the running
      // lanes then integrate those groups without drawing: a lone chain pays
      // one warp-wide draw per 128 steps instead of one per 4 steps on its
      // own instruction stream.  The normals are those of the per-lane draws
      // (a lane at a window start is at a group boundary), so the results are
      // identical.
      const unsigned act = __ballot_sync(kFull, active);
      const int na = __popc(act);
      if (exhausted && na <= kCoopLanes) {
        R *coop = reinterpret_cast<R *>(q);            // [na][G][4] normals, <= 128 entries
        const int G = 32 / na;
        const int jt = lane % na, gi = lane / na;     // this lane draws group gi of the jt-th running lane
        unsigned m = act;
        for (int t = 0; t < jt; ++t) m &= m - 1u;
        const int src = __ffs(m) - 1;
        const uint32_t k0 = __shfl_sync(kFull, L.key0, src);
        const uint32_t k1 = __shfl_sync(kFull, L.key1, src);
        const uint32_t st = __shfl_sync(kFull, L.steps, src);
        const unsigned long long pid = __shfl_sync(kFull, L.pid, src);
        R zz[4];
        normals4<R>(k0, k1, st / 4u + (uint32_t)gi, kStreamSde, pid, zz);
        if (gi < G) {
#pragma unroll
          for (int j = 0; j < 4; ++j) coop[(jt * G + gi) * 4 + j] = zz[j];
        }
        __syncwarp();
        const int me = __popc(act & lanemask_lt());
        for (int g = 0; g < G; ++g) {
          if (active) {
            R z[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) z[j] = coop[(me * G + g) * 4 + j];
            fp_group(z);
          }
        }
        __syncwarp();                                  // the buffer is drawn again next window
        continue;
      }
    }
    for (int k = 0; k < win; k += spc) {
      if (active) {
        R z[4];
        if constexpr (Prefetch<MODEL>::value) {
#pragma unroll
          for (int j = 0; j < 4; ++j) z[j] = zq[j];
          draw_group<MODEL, R>(L, L.steps / spc + 1u, zq);
        } else {
          draw<MODEL, R>(L, z);
        }
        if constexpr (MODEL == kModelFp) {
          fp_group(z);
        } else {
#pragma unroll
          for (int j = 0; j < spc; ++j) {
            if (active) {
              const int res = model_step<MODEL, R>(L, K, z, j);
              ++L.steps;
              // one test per step covers the rare events: an exit, a stop,
              // the step cap (an exit on the capped step counts as an exit)
              if (res != kContinue || L.steps >= cap32) {
                active = false;
                sink.add(slot, L.sim, kOffNSteps, (double)L.steps);
                if (res == kRecordAndStop) {
                  // queue the exit (at most one per lane per window: <= 63 entries)
                  QEnt e;
                  e.Tinj = L.Tinj;
                  e.Texit = (float)L.T.v;
                  e.sim = L.sim;
                  e.slot_gbin = ((unsigned)(L.gbin + 1) << 16) | ((unsigned)slot & 0xffffu);
                  q[atomicAdd(qlen, 1)] = e;
                  if (a.records != nullptr) append_record_one(a, L, MODEL);
                } else if (res != kContinue) {
                  sink.add(slot, L.sim, kOffNLost, 1.0);
                } else {
                  sink.add(slot, L.sim, kOffNCapped, 1.0);
                }
              }
            }
          }
        }
      }
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < slots * W; i += blockDim.x) {
    const double v = sh_hist[i];
    if (v != 0.0) {
      const int sl = i / W;
      atomicAdd(&sink.slice[(size_t)gsim[sl] * kSpecDoubles + Window<MODEL>::lo + (i - sl * W)], v);
    }
  }
}

// ---------------------------------------------------------------------------
// Plain kernel: one thread per particle of one simulation, no refill (the
// baseline of one simulation per launch) and the per-trajectory replay.
// ---------------------------------------------------------------------------
template <int MODEL, class R>
__global__ void __launch_bounds__(256, (sizeof(R) == 4) ? 2 : 1) k_plain(const KArgs a) {
  if (a.ctl->status != 0) return;
  const unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = i < a.plain_count;
  const int sim = a.plain_sim;
  Sink<MODEL> sink;
  sink.sh = nullptr;
  sink.smem_slots = 0;
  sink.slice = a.part + (size_t)(blockIdx.x % a.n_slices) * a.n_sims * kSpecDoubles;
  const SimDev sd = a.sims[sim];
  Lane<R> L;
  Consts<R> K;
  bool active = false, pending = false;
  Pending pd;
  int status = 1, nrec = 0;
  float t_rec = 0.f, r_rec = 0.f, aux_rec = 0.f;
  if (valid) {
    init_lane<MODEL, R>(L, K, sd, a.inj_tables + (size_t)sim * GELIO_GRID_MAX, sim, a.plain_first + i);
    sink.add(1 << 30, sim, kOffNParticles, 1.0);
    active = true;
  }
  constexpr int spc = StepsPerCall<MODEL>::value;
  while (active) {
    R z[4];
    draw<MODEL, R>(L, z);
#pragma unroll
    for (int j = 0; j < spc; ++j) {
      if (active) {
        const int res = model_step<MODEL, R>(L, K, z, j);
        ++L.steps;
        if (res == kRecordAndContinue || res == kRecordAndStop) {
          if (nrec == 0) {
            t_rec = (float)L.T.v;
            r_rec = (MODEL == kModelFp) ? L.rrec : (float)L.r.v;
            aux_rec = (MODEL == kModelFp) ? (float)L.sumac.v : (float)theta_full(L);
          }
          ++nrec;
        }
        if constexpr (MODEL == kModelFp) {
          if (res == kRecordAndContinue || res == kRecordAndStop)
            emit_fp(a.ctl, a.records, a.record_capacity, sink, fp_crossing(L, sd, 1 << 30));
          if (res != kContinue && res != kRecordAndContinue) { active = false; status = (nrec > 0) ? 0 : 1; }
        } else if (res != kContinue) {
          active = false;
          if (res == kRecordAndStop) {
            pending = true;
            status = 0;
            pd.Tinj = L.Tinj; pd.Texit = (float)L.T.v; pd.r = (float)L.r.v; pd.aux = (float)theta_full(L);
            pd.sim = sim; pd.slot = 1 << 30; pd.gbin = L.gbin; pd.pid = L.pid;
          } else {
            status = 1;
            sink.add(1 << 30, sim, kOffNLost, 1.0);
          }
        }
        if (active && L.steps >= a.max_steps) {
          active = false;
          status = 2;
          sink.add(1 << 30, sim, kOffNCapped, 1.0);
        }
      }
    }
  }
  if (valid) sink.add(1 << 30, sim, kOffNSteps, (double)L.steps);
  if constexpr (MODEL != kModelFp) {
    const unsigned pm = __ballot_sync(kFull, pending);
    if (pending) {
      append_records(a, pm, pd, MODEL);
      flush_pending<MODEL>(sink, pm, pd);
    }
  }
  if (valid && a.replay != nullptr) {
    gelio_trajectory t;
    t.status = status;
    t.steps = L.steps;
    t.n_records = nrec;
    t.t_injection = L.Tinj;
    t.t_final = (float)L.T.v;
    t.r_final = (float)L.r.v;
    t.theta_final = (MODEL == kModelFp) ? (float)L.sumac.v : (float)theta_full(L);
    t.t_record = t_rec;
    t.r_record = r_rec;
    t.aux_record = aux_rec;
    a.replay[i] = t;
  }
}

// Host-side entry points of one model's translation unit.
// prec: 0 = FP32 (<= 128 registers), 1 = FP64, 2 = FP32 compact (<= 85 registers)
#define GELIO_DEFINE_MODEL_ENTRIES(NAME, MODEL)                                              \
  cudaError_t NAME##_launch(bool persistent, int prec, unsigned grid, unsigned block,        \
                            size_t smem, cudaStream_t st, const KArgs &a) {                  \
    if (persistent) {                                                                        \
      if (prec == 1) k_persistent<MODEL, double, 1><<<grid, block, smem, st>>>(a);           \
      else if (prec == 2) k_persistent<MODEL, float, 3><<<grid, block, smem, st>>>(a);       \
      else k_persistent<MODEL, float, 2><<<grid, block, smem, st>>>(a);                      \
    } else {                                                                                 \
      if (prec == 1) k_plain<MODEL, double><<<grid, block, 0, st>>>(a);                      \
      else k_plain<MODEL, float><<<grid, block, 0, st>>>(a);                                 \
    }                                                                                        \
    return cudaGetLastError();                                                               \
  }                                                                                          \
  const void *NAME##_kernel(bool persistent, int prec) {                                     \
    if (persistent) return prec == 1 ? (const void *)k_persistent<MODEL, double, 1>          \
                         : prec == 2 ? (const void *)k_persistent<MODEL, float, 3>           \
                                     : (const void *)k_persistent<MODEL, float, 2>;          \
    return prec == 1 ? (const void *)k_plain<MODEL, double> : (const void *)k_plain<MODEL, float>; \
  }                                                                                          \
  cudaError_t NAME##_tables(const BinTables &t) { return set_tables_tu(t); }

}  // namespace gelio
