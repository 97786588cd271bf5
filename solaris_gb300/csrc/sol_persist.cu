// Persistent RungeKuttaFehlberg78 driver for systems whose sinks see few
// sources (a handful of massive bodies and many light ones, e.g. a star, two
// giants and hundreds of test particles, with or without a gas nebula).
//
// Such a system is latency-bound: an evaluation is a few thousand pairs, so a
// kernel per stage spends its time launching.  Here one cooperative launch
// runs whole sequences of driver calls.  Every thread owns one body for the
// whole launch, so the stage sums, rm3, the force epilogue (Kepler term, gas
// drag, migration) and the final sum of its body only touch its own data;
// the only data that crosses threads is the source table of the massive
// bodies (positions, G m, position * rm3), written by their owners and read
// by every sink after one grid barrier per stage.  The error norm takes one
// more barrier, after which every CTA derives the same step-size decision
// from the same block maxima.  The arithmetic is that of the stage, force
// and control kernels of the graph path (and so of the reference,
// RungeKuttaFehlberg78.cpp:66-262, Acceleration.cpp:166-329): results are
// bit-identical to the host-driven loop.
//
// What bounds it on the GB300: an FP64 warp instruction costs about the same
// whatever the number of active lanes, and a stage is a dependent chain of
// ~175 FP64 instructions per body (IEEE sqrt and division of rm3 and of each
// pair, the stage sums), ~7-9 us whatever the bodies per CTA (measured from 1
// to 128).  The group driver (sol_group.cu) spreads that chain over lanes and
// SM sub-partitions and takes every system it can hold (about 3x faster);
// this one-thread-per-body form remains for systems with more light bodies
// than the group layout holds.
//
// Grid barriers spin on a generation counter with an iteration limit; a CTA
// that runs out raises SOL_DEV_TIMEOUT and an abort flag that makes every
// other CTA leave at its next barrier.
#include <atomic>
#include <mutex>
#include <cmath>
#include <cstring>

#include "sol_crmath.cuh"

namespace {

#define RET(x)                   \
  do {                           \
    int r_ = (x);                \
    if (r_ != SOL_OK) return r_; \
  } while (0)

constexpr int kMaxBlock = 128;
constexpr int kBodiesPerCta = 64;
constexpr int kMaxSources = 32;    // sources per sink handled by one thread
constexpr int kTabArrays = 7;      // x, y, z, G m, x rm3, y rm3, z rm3

// RKF78 stage sums in the reference's order (RungeKuttaFehlberg78.cpp:169-232)
__constant__ int p_rk_k[13];
__constant__ int p_rk_idx[13][9];
__constant__ double p_rk_a[13][9];

struct PersistArgs {
  ForceCtx fc;
  double* y0;           // resident state [6N]
  double* f[13];        // f0 = accel, f1..f12
  double* yscale;
  double* ynew;
  double* err;
  double* tab;          // source table, 2 buffers x kTabArrays x kMaxSources
  double* partial;      // block maxima of |error / yscale|
  unsigned* bar_count;  // grid barrier
  unsigned* bar_gen;
  int* abort_flag;
  sol_ctrl* ctrl;
  int n;
  int bpc;              // bodies per CTA (the first bpc threads of a CTA own one body each)
  int ns_max;           // sources of the sinks with the most (<= kMaxSources)
  int n_steps;
};

// Grid-wide barrier among the co-resident CTAs of a cooperative launch.
// Returns false when the wait ran out or another CTA gave up.
__device__ bool grid_barrier(const PersistArgs& P, int* s_abort) {
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned* gen = P.bar_gen;
    const unsigned g = *gen;
    __threadfence();
    if (atomicAdd(P.bar_count, 1u) == gridDim.x - 1) {
      *P.bar_count = 0;
      __threadfence();
      atomicAdd(P.bar_gen, 1u);
    } else {
      bool ok = false;
      for (uint32_t k = 0; k < SOL_SPIN_LIMIT; ++k) {
        if (*gen != g) {
          ok = true;
          break;
        }
        if (*(volatile int*)P.abort_flag) break;
        __nanosleep(32);
      }
      if (!ok) {
        if (!*(volatile int*)P.abort_flag) atomicOr(&P.ctrl->dev_status, SOL_DEV_TIMEOUT);
        atomicExch(P.abort_flag, 1);
      }
    }
    __threadfence();
    *s_abort = *(volatile int*)P.abort_flag;
  }
  __syncthreads();
  return *s_abort == 0;
}

// The owner of body i computes rm3_i for the state y and, for a source body,
// its entry of the source table (as k_prepass does).
__device__ __forceinline__ void own_prepass(const PersistArgs& P, int i, const double* y, double* tab, double& rm3) {
  rm3 = 0.0;
  if (i >= P.n) return;
  const double x = y[0], yy = y[1], z = y[2];
  if (i >= 1) {
    const double r2 = x * x + yy * yy + z * z;
    double r;
    sol_ref_rinv3(r2, r, rm3);
    P.fc.rm3[i] = rm3;
  }
  if (i < P.ns_max) {
    const double gm = i >= 1 ? SOL_GAUSS2 * P.fc.mass[i] : 0.0;
    tab[0 * kMaxSources + i] = x;
    tab[1 * kMaxSources + i] = yy;
    tab[2 * kMaxSources + i] = z;
    tab[3 * kMaxSources + i] = gm;
    tab[4 * kMaxSources + i] = x * rm3;
    tab[5 * kMaxSources + i] = yy * rm3;
    tab[6 * kMaxSources + i] = z * rm3;
  }
}

// GravityAC for sink i from the shared copy of the source table, then the gas
// terms: the operation order of k_gravity_ac<FP64>.
__device__ __forceinline__ void own_force(const PersistArgs& P, int i, const double* y, double rm3i, const double* st,
                                          double t, uint32_t flags, double* out) {
  const ForceCtx& fc = P.fc;
  if (i == 0) {
    for (int k = 0; k < 6; ++k) out[k] = 0.0;
    fc.nn_idx[0] = -1;
    fc.nn_dist[0] = 0.0;
    return;
  }
  const Classes& c = fc.cls;
  const int ns = (fc.type[i] <= SOL_PROTO_PLANET) ? c.nm + c.n_spl : c.nm;
  const double xi = y[0], yi = y[1], zi = y[2];
  double ax = 0.0, ay = 0.0, az = 0.0;
  long long rminb = __double_as_longlong(1.0e10);
  int nn = -1;
  for (int j = 1; j < ns; ++j) {
    if (j == i) continue;
    const double xij = st[0 * kMaxSources + j] - xi;
    const double yij = st[1 * kMaxSources + j] - yi;
    const double zij = st[2 * kMaxSources + j] - zi;
    const double rij2 = xij * xij + yij * yij + zij * zij;
    double rij, rijm3;
    sol_ref_rinv3(rij2, rij, rijm3);
    const long long rb = __double_as_longlong(rij);
    if (rb < rminb) {
      rminb = rb;
      nn = j;
    }
    const double gm = st[3 * kMaxSources + j];
    ax += gm * (xij * rijm3 - st[4 * kMaxSources + j]);
    ay += gm * (yij * rijm3 - st[5 * kMaxSources + j]);
    az += gm * (zij * rijm3 - st[6 * kMaxSources + j]);
  }
  const double mu = SOL_GAUSS2 * (fc.mass[0] + fc.mass[i]);
  double a[3];
  a[0] = -mu * rm3i * xi;  // Kepler term first (Acceleration.cpp:281-283)
  a[1] = -mu * rm3i * yi;
  a[2] = -mu * rm3i * zi;
  a[0] += ax;
  a[1] += ay;
  a[2] += az;
  fc.nn_idx[i] = nn;
  fc.nn_dist[i] = nn >= 0 ? __longlong_as_double(rminb) : 0.0;
  add_gas_terms(fc, i, y, t, flags, a);
  out[0] = y[3];
  out[1] = y[4];
  out[2] = y[5];
  out[3] = a[0];
  out[4] = a[1];
  out[5] = a[2];
}

struct Shared {
  double tab[kTabArrays * kMaxSources];
  double red[kMaxBlock];
  double t, h, h_next, h_did, error_max, eps;
  long long n_acc, n_rej;
  int status, accepted, abort;
};

// One evaluation: the owner's stage input ytmp and its prepass, the barrier,
// the copy of the source table into shared memory, the force.
__device__ bool evaluate(const PersistArgs& P, Shared& S, int i, const double* yin, int& buf, uint32_t flags,
                         double* fout) {
  double* tab = P.tab + (size_t)buf * kTabArrays * kMaxSources;
  double rm3 = 0.0;
  own_prepass(P, i, yin, tab, rm3);
  if (!grid_barrier(P, &S.abort)) return false;
  for (int k = threadIdx.x; k < kTabArrays * kMaxSources; k += blockDim.x) S.tab[k] = __ldcg(tab + k);
  __syncthreads();
  if (i < P.n) own_force(P, i, yin, rm3, S.tab, S.t, flags, fout);
  buf ^= 1;
  return true;
}

__global__ void __launch_bounds__(kMaxBlock) k_persist_rkf78(PersistArgs P) {
  __shared__ Shared S;
  const int i = threadIdx.x < P.bpc ? blockIdx.x * P.bpc + threadIdx.x : P.n;  // P.n: no body
  const bool live = i < P.n;
  double y0[6], yt[6], fo[6];
  if (live)
    for (int k = 0; k < 6; ++k) y0[k] = P.y0[6 * i + k];
  if (threadIdx.x == 0) {
    const sol_ctrl c = *P.ctrl;
    S.t = c.t;
    S.h = c.h;
    S.h_next = c.h_next;
    S.h_did = c.h_did;
    S.error_max = c.error_max;
    S.eps = c.eps;
    S.n_acc = c.n_accepted;
    S.n_rej = c.n_rejected;
    S.status = c.dev_status;
    S.abort = 0;
  }
  __syncthreads();
  int buf = 0;
  bool ok = true;
  for (int step = 0; step < P.n_steps && ok && S.status == 0; ++step) {
    if (threadIdx.x == 0) {  // Driver: bodyData->h = timeLine->hNext (:74-75)
      S.h = S.h_next;
      S.accepted = 0;
    }
    __syncthreads();
    // first evaluation with every term on (:77-82) and yscale (:87-89)
    ok = evaluate(P, S, i, y0, buf, SOL_EVAL_ALL, fo);
    if (!ok) break;
    double ys[6];
    if (live) {
      for (int k = 0; k < 6; ++k) {
        P.f[0][6 * i + k] = fo[k];
        ys[k] = fabs(y0[k]) + fabs(S.h * fo[k]) + 1.0e-30;
        P.yscale[6 * i + k] = ys[k];
      }
    }
    for (;;) {
      const double h = S.h;
      for (int r = 1; r <= 12 && ok; ++r) {
        if (live) {
          const int K = p_rk_k[r];
          for (int k = 0; k < 6; ++k) {
            const int e = 6 * i + k;
            double acc = p_rk_a[r][0] * P.f[p_rk_idx[r][0]][e];
            for (int q = 1; q < K; ++q) acc = acc + p_rk_a[r][q] * P.f[p_rk_idx[r][q]][e];
            yt[k] = y0[k] + h * acc;
          }
        }
        // migration only at the first evaluation of a driver call (:94-95)
        ok = evaluate(P, S, i, yt, buf, SOL_EVAL_GAS_DRAG, fo);
        if (ok && live)
          for (int k = 0; k < 6; ++k) P.f[r][6 * i + k] = fo[k];
      }
      if (!ok) break;
      // final sum, error estimate and the scaled norm (:236-242, :252-262)
      double m = 0.0;
      double yn[6];
      if (live) {
        const double D1_0 = 41.0 / 840.0, D1_5 = 34.0 / 105.0, D1_6 = 9.0 / 35.0, D1_8 = 9.0 / 280.0,
                     D1_10 = 41.0 / 840.0;
        for (int k = 0; k < 6; ++k) {
          const int e = 6 * i + k;
          const double f0 = P.f[0][e], f10 = P.f[10][e];
          yn[k] = y0[k] + h * (D1_0 * f0 + D1_5 * P.f[5][e] + D1_6 * (P.f[6][e] + P.f[7][e]) +
                               D1_8 * (P.f[8][e] + P.f[9][e]) + D1_10 * f10);
          const double ee = h * fabs(f0 + f10 - P.f[11][e] - P.f[12][e]) * 41.0 / 840.0;
          P.ynew[e] = yn[k];
          P.err[e] = ee;
          const double qq = fabs(ee / ys[k]);
          m = qq > m ? qq : m;  // a NaN entry never replaces the maximum
        }
      }
      S.red[threadIdx.x] = m;
      __syncthreads();
      for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w && S.red[threadIdx.x + w] > S.red[threadIdx.x]) S.red[threadIdx.x] = S.red[threadIdx.x + w];
        __syncthreads();
      }
      if (threadIdx.x == 0) P.partial[blockIdx.x] = S.red[0];
      ok = grid_barrier(P, &S.abort);
      if (!ok) break;
      if (threadIdx.x == 0) {  // every CTA takes the same decision (:98-133)
        double mx = 0.0;
        for (int b = 0; b < (int)gridDim.x; ++b) {
          const double o = __ldcg(P.partial + b);
          if (o > mx) mx = o;
        }
        const double em = mx / S.eps;
        S.error_max = em;
        if (em < 1.0) {
          S.h_did = h;
          S.t += S.h_did;
          S.h_next = em > 1.89e-4 ? (0.9 * h * sol_inv_root<5>(em)) : (5.0 * h);
          S.h = S.h_next;
          S.accepted = 1;
          S.n_acc++;
        } else {
          S.n_rej++;
          const double hTemp = 0.9 * h * sol_inv_root<4>(em);
          const double hn = fabs(hTemp) > fabs(0.1 * h) ? hTemp : 0.1 * h;
          S.h = hn;
          if (S.t + hn == S.t) S.status |= SOL_DEV_UNDERFLOW;
        }
      }
      __syncthreads();
      if (S.accepted) {
        if (live)
          for (int k = 0; k < 6; ++k) {
            y0[k] = yn[k];
            P.y0[6 * i + k] = yn[k];
          }
        break;
      }
      if (S.status) break;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    sol_ctrl* c = P.ctrl;
    c->t = S.t;
    c->h = S.h;
    c->h_next = S.h_next;
    c->h_did = S.h_did;
    c->error_max = S.error_max;
    c->accepted = S.accepted;
    c->n_accepted = S.n_acc;
    c->n_rejected = S.n_rej;
    atomicOr(&c->dev_status, S.status);
  }
}

int upload_persist_tableau() {
  // once per device; contexts of several host threads may arrive together
  static std::atomic<bool> done[64];
  static std::mutex upload_mutex;
  int dev = 0;
  SOL_CUDA(cudaGetDevice(&dev));
  if (dev >= 0 && dev < 64 && done[dev].load(std::memory_order_acquire)) return SOL_OK;
  std::lock_guard<std::mutex> upload_lock(upload_mutex);
  if (dev >= 0 && dev < 64 && done[dev].load(std::memory_order_relaxed)) return SOL_OK;
  int k[13] = {0};
  int idx[13][9] = {{0}};
  double a[13][9] = {{0}};
  const Rkf78Table& T = sol_rkf78_table();
  for (int r = 1; r <= 12; ++r) {
    k[r] = T.k[r];
    for (int q = 0; q < T.k[r]; ++q) {
      idx[r][q] = T.idx[r][q];
      a[r][q] = T.a[r][q];
    }
  }
  SOL_CUDA(cudaMemcpyToSymbol(p_rk_k, k, sizeof(k)));
  SOL_CUDA(cudaMemcpyToSymbol(p_rk_idx, idx, sizeof(idx)));
  SOL_CUDA(cudaMemcpyToSymbol(p_rk_a, a, sizeof(a)));
  if (dev >= 0 && dev < 64) done[dev].store(true, std::memory_order_release);
  return SOL_OK;
}

}  // namespace

// Whether the system runs its RKF78 driver calls on the persistent path.
int sol_persist_eligible(const sol_ctx* c) {
  if (c->barycentric || c->n > 65536) return 0;
  return c->cls.nm + c->cls.n_spl <= kMaxSources;
}

// n_steps RKF78 driver calls in one cooperative launch.  Returns SOL_ERR_STATE
// (nothing launched) when the grid cannot be co-resident.
int sol_persist_rkf78(sol_ctx* c, int n_steps) {
  if (!c->d_persist) {
    const size_t doubles = 2 * kTabArrays * kMaxSources + 4096 + 8;
    if (cudaMalloc((void**)&c->d_persist, sizeof(double) * doubles) != cudaSuccess) {
      sol_set_error("cudaMalloc of the persistent-driver scratch failed");
      return SOL_ERR_NOMEM;
    }
    SOL_CUDA(cudaMemset(c->d_persist, 0, sizeof(double) * doubles));
  }
  // 64 bodies per CTA: measured best for 256 bodies (1 star, 2 giants, 253
  // test particles: 153 us per attempt against 158 / 168 us at 128 / 32) and
  // for 8,193 bodies with gas drag (395 us against 418 / 418 us)
  const int bpc = kBodiesPerCta;
  const int block = bpc;
  const int grid = (c->n + bpc - 1) / bpc;
  if (grid > 4096) return SOL_ERR_STATE;
  int per_sm = 0, n_sm = 0;
  SOL_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_persist_rkf78, block, 0));
  SOL_CUDA(cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, c->device));
  if (grid > per_sm * n_sm) return SOL_ERR_STATE;
  RET(upload_persist_tableau());
  PersistArgs P;
  memset(&P, 0, sizeof(P));
  P.fc = c->fc;
  P.y0 = c->d_y0;
  P.f[0] = c->d_accel;
  for (int k = 1; k < 13; ++k) P.f[k] = c->d_fk[k];
  P.yscale = c->d_yscale;
  P.ynew = c->d_y;
  P.err = c->d_err;
  P.tab = c->d_persist;
  P.partial = c->d_persist + 2 * kTabArrays * kMaxSources;
  unsigned* words = reinterpret_cast<unsigned*>(c->d_persist + 2 * kTabArrays * kMaxSources + 4096);
  P.bar_count = words;
  P.bar_gen = words + 1;
  P.abort_flag = reinterpret_cast<int*>(words + 2);
  P.ctrl = c->d_ctrl;
  P.n = c->n;
  P.bpc = bpc;
  P.ns_max = c->cls.nm + c->cls.n_spl;
  P.n_steps = n_steps;
  // fresh barrier words for this launch
  SOL_CUDA(cudaMemsetAsync(words, 0, 4 * sizeof(unsigned), c->stream));
  void* args[] = {&P};
  SOL_CUDA(cudaLaunchCooperativeKernel((const void*)k_persist_rkf78, grid, block, args, 0, c->stream));
  SOL_LAUNCHED();
  return SOL_OK;
}
