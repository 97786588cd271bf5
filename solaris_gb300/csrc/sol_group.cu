// RungeKuttaFehlberg78 driver for systems whose sinks see few sources, with
// the work of every stage spread over the lanes and warps of a group of CTAs.
//
// What bounds such a system on the GB300 is the FP64 pipe's cost per warp
// instruction: one FP64 warp instruction occupies its SM sub-partition for
// ~64 cycles whether 1 or 32 lanes are active, and independent instructions
// of one warp do not overlap (measured).  A thread that owns a body and runs
// its whole stage (rm3, every pair, the sums, the next stage input) issues
// ~175 FP64 instructions in a row, ~11,000 cycles per stage whatever the
// number of bodies.  Here a stage is three short phases, each spread over the
// lanes (one lane per body, per pair, per (body, component), per element)
// and over the four sub-partitions of every SM:
//   1. rm3 of every sink, the pair terms d_ij / |d_ij|^3 and |d_ij| of every
//      (sink, source) pair, and the gas terms (drag, migration) of every sink,
//      side by side in different warps;
//   2. per (sink, component), the Kepler term and the sum over the sources
//      in the reference's order, plus the gas term;
//   3. per element, the next stage input (or the final sum, the error
//      estimate and its scaled norm).
// The sources (the first nm + n_spl bodies: star, planets, super-
// planetesimals) are integrated redundantly by every CTA: each CTA holds
// their whole stage history, so no data crosses CTAs during an attempt, and
// one group barrier per attempt carries the error norm.  Each CTA also owns
// a contiguous range of the other bodies.  The arithmetic, operation by
// operation, is that of the persistent and host-driven drivers (and so of the
// reference, RungeKuttaFehlberg78.cpp:66-262, Acceleration.cpp:166-329): the
// results are bit-identical.
//
// The group barrier spins on a generation counter with an iteration limit; a
// CTA that runs out raises SOL_DEV_TIMEOUT and an abort flag that makes every
// other CTA leave at its next barrier.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "sol_internal.cuh"

namespace {

#define RET(x)                   \
  do {                           \
    int r_ = (x);                \
    if (r_ != SOL_OK) return r_; \
  } while (0)

constexpr int kBlock = 128;       // one warp per SM sub-partition
constexpr int kMaxSources = 32;   // nm + n_spl
constexpr int kMaxLocal = 64;     // other bodies per CTA
constexpr int kMinLocal = 16;
constexpr int kSpreadSmem = 116 * 1024;  // > half of the 228 KB of an SM

__constant__ int g_rk_k[13];
__constant__ int g_rk_idx[13][9];
__constant__ double g_rk_a[13][9];

struct GroupArgs {
  ForceCtx fc;
  double* y0;           // resident state [6N]
  double* accel;        // f0 of the last driver call
  double* yscale;
  double* ynew;
  double* err;
  double* partial;      // CTA maxima of |error / yscale|
  unsigned* bar_count;  // group barrier
  unsigned* bar_gen;
  int* abort_flag;
  sol_ctrl* ctrl;
  int n;
  int ns;               // sources: nm + n_spl
  int local;            // other bodies per CTA
  int n_steps;
  // shared-memory layout (offsets in doubles)
  int o_f, o_y0, o_yt, o_ys, o_yn, o_rm3, o_pp, o_prb, o_xr, o_gm, o_gbuf, o_red, o_mu, o_int;
};

__device__ bool group_barrier(const GroupArgs& P, int* s_abort) {
  __syncthreads();
  if (gridDim.x > 1 && threadIdx.x == 0) {
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

struct Ctl {
  double t, h, h_next, h_did, error_max, eps;
  long long n_acc, n_rej;
  int status, accepted, abort, npair;
};

// Per-CTA view of the shared memory.  Sink slot s < ns is source (body) s,
// slot s >= ns is body l0 + s - ns.
struct View {
  double* f;    // [13][6 * nsink]
  double* y0;   // [6 * nsink]
  double* yt;   // stage input
  double* ys;   // yscale
  double* yn;   // final sum
  double* rm3;  // [nsink]
  double* pp;   // [3][nsink][ns]: d_ij * |d_ij|^-3 per component
  long long* prb;  // [nsink][ns]: bits of |d_ij|
  double* xr;   // [3][ns]: x_j rm3_j of the sources
  double* gm;   // [ns]: G m_j (0 for j = 0)
  double* gbuf; // [3 * nsink]: drag or migration buffer of each sink
  double* red;  // [kBlock]
  double* mu;   // [nsink]: G (m_0 + m_i)
  int* mig;     // [nsink]: migType of each sink
  int* body;    // [nsink]: body index of each slot
  int* nsrc;    // [nsink]: sources of the sink (nm + n_spl or nm)
  int* kind;    // [nsink]: gas buffer kind
  int* pair;    // [npair]: sink slot * 32 + source of every (sink, source) pair
  int nsink, npair;
};

// Which gas buffer a body uses (Acceleration::ComputeAstroCentric :176-243):
// 1 drag, 2 type-I migration, 3 type-II migration, 0 none.
__device__ __forceinline__ int gas_kind(const ForceCtx& fc, int i) {
  if (!fc.gas.present) return 0;
  const Classes& c = fc.cls;
  if (i >= c.nm && i < c.nm + c.n_spl + c.n_pl) return 1;
  if (fc.has_mig1 && i >= c.n_central + c.n_giant && i < c.nm) return 2;
  if (fc.has_mig2 && i >= c.n_central && i < c.n_central + c.n_giant) return 3;
  return 0;
}

__device__ __forceinline__ double* global_gas_buf(const ForceCtx& fc, int i, int kind) {
  const Classes& c = fc.cls;
  if (kind == 1) return fc.drag + 3 * (i - c.nm);
  if (kind == 2) return fc.mig1 + 3 * (i - (c.n_central + c.n_giant));
  return fc.mig2 + 3 * (i - c.n_central);
}

// The buffer part of add_gas_terms: drag evaluated at every evaluation with
// the drag flag, migration only with its flag and while migType allows it
// (a migration that reaches its stop sets migType to No).  Out of line: its
// thousands of instructions inlined into the stage loop evict the hot path
// from the instruction cache (measured: 3x slower stages without gas).
__device__ __noinline__ void gas_compute(const ForceCtx& fc, int i, int kind, const double* yi, double t,
                                            uint32_t flags, double* buf, int* mig) {
  const GasDev& g = fc.gas;
  const double m0 = fc.mass[0];
  double d[3];
  if (kind == 1) {
    if (!(flags & SOL_EVAL_GAS_DRAG)) return;
    sol_gas_drag(g, sol_reduction_factor(g, t), m0, yi, fc.radius[i], fc.density[i], fc.cd[i], fc.gamma_stokes[i],
                 fc.gamma_epstein[i], d);
  } else if (kind == 2) {
    if (!((flags & SOL_EVAL_TYPE_I) && *mig == SOL_MIGRATION_TYPE_I)) return;
    if (!sol_migration_type1(g, sol_reduction_factor(g, t), m0, fc.mass[i], fc.mig_stop_at[i], yi, d))
      *mig = SOL_MIGRATION_NO;
  } else {
    if (!((flags & SOL_EVAL_TYPE_II) && *mig == SOL_MIGRATION_TYPE_II)) return;
    if (!sol_migration_type2(g, sol_reduction_factor(g, t), m0, fc.mass[i], fc.mig_stop_at[i], yi, d))
      *mig = SOL_MIGRATION_NO;
  }
  buf[0] = d[0];
  buf[1] = d[1];
  buf[2] = d[2];
}

// One force evaluation of the CTA's sinks on the stage input V.yt (phases 1
// and 2); writes f[r] and, where this CTA owns the body, rm3, the nearest
// neighbour and the gas buffers in global memory.
__device__ __noinline__ void evaluate(const GroupArgs& P, const View& V, double t, uint32_t flags, int r) {
  const ForceCtx& fc = P.fc;
  const int ns = P.ns, nsink = V.nsink;
  const bool home = blockIdx.x == 0;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  // phase 1: the three kinds of work in separate virtual warps
  const int w_rm3 = (nsink + 31) >> 5;
  const int w_pair = (V.npair + 31) >> 5;
  const int w_gas = fc.gas.present ? (nsink + 31) >> 5 : 0;
  for (int vw = warp; vw < w_rm3 + w_pair + w_gas; vw += nwarps) {
    if (vw < w_rm3) {
      const int s = vw * 32 + lane;
      if (s < nsink) {
        const int i = V.body[s];
        const double* y = V.yt + 6 * s;
        double rm3 = 0.0;
        if (i >= 1) {  // Acceleration.cpp:259-261
          const double x = y[0], yy = y[1], z = y[2];
          const double r2 = x * x + yy * yy + z * z;
          const double rr = __dsqrt_rn(r2);
          rm3 = __ddiv_rn(1.0, r2 * rr);
          if (s >= ns || home) fc.rm3[i] = rm3;
        }
        V.rm3[s] = rm3;
        if (s < ns) {
          V.xr[0 * ns + s] = y[0] * rm3;
          V.xr[1 * ns + s] = y[1] * rm3;
          V.xr[2 * ns + s] = y[2] * rm3;
        }
      }
    } else if (vw < w_rm3 + w_pair) {
      const int p = (vw - w_rm3) * 32 + lane;
      if (p < V.npair) {
        const int s = V.pair[p] >> 5, j = V.pair[p] & 31;
        const double* yi = V.yt + 6 * s;
        const double* yj = V.yt + 6 * j;  // source j is slot j
        const double xij = yj[0] - yi[0];
        const double yij = yj[1] - yi[1];
        const double zij = yj[2] - yi[2];
        const double rij2 = xij * xij + yij * yij + zij * zij;
        const double rij = __dsqrt_rn(rij2);
        const double rijm3 = __ddiv_rn(1.0, rij2 * rij);
        V.prb[s * ns + j] = __double_as_longlong(rij);
        V.pp[(0 * nsink + s) * ns + j] = xij * rijm3;
        V.pp[(1 * nsink + s) * ns + j] = yij * rijm3;
        V.pp[(2 * nsink + s) * ns + j] = zij * rijm3;
      }
    } else {
      const int s = (vw - w_rm3 - w_pair) * 32 + lane;
      if (s < nsink && V.kind[s]) {
        const int i = V.body[s], kind = V.kind[s];
        gas_compute(fc, i, kind, V.yt + 6 * s, t, flags, V.gbuf + 3 * s, V.mig + s);
        if (s >= ns || home) {
          double* gb = global_gas_buf(fc, i, kind);
          gb[0] = V.gbuf[3 * s + 0];
          gb[1] = V.gbuf[3 * s + 1];
          gb[2] = V.gbuf[3 * s + 2];
          if (kind >= 2) fc.mig_type[i] = V.mig[s];
        }
      }
    }
  }
  __syncthreads();
  // phase 2: per (sink, component) the GravityAC sum, then the gas term
  double* fr = V.f + (size_t)r * 6 * nsink;
  for (int q = threadIdx.x; q < 3 * nsink; q += blockDim.x) {
    const int s = q / 3, k = q - 3 * s;
    const int i = V.body[s];
    const double* yi = V.yt + 6 * s;
    if (i == 0) {
      fr[6 * s + k] = 0.0;
      fr[6 * s + 3 + k] = 0.0;
      if (k == 0 && home) {
        fc.nn_idx[0] = -1;
        fc.nn_dist[0] = 0.0;
      }
      continue;
    }
    const int nsi = V.nsrc[s];
    const double* pp = V.pp + (size_t)(k * nsink + s) * ns;
    const double* xr = V.xr + k * ns;
    double acc = 0.0;
    for (int j = 1; j < nsi; ++j) {
      if (j == i) continue;
      acc += V.gm[j] * (pp[j] - xr[j]);
    }
    double a = -V.mu[s] * V.rm3[s] * yi[k];  // Kepler term first (Acceleration.cpp:281-283)
    a += acc;
    const int kind = V.kind[s];
    if (kind == 1 || (kind >= 2 && V.mig[s] != SOL_MIGRATION_NO)) a += V.gbuf[3 * s + k];
    fr[6 * s + k] = yi[3 + k];
    fr[6 * s + 3 + k] = a;
    if (k == 0 && (s >= ns || home)) {  // nearest neighbour: smallest |d_ij|, the first in j order
      long long rminb = __double_as_longlong(1.0e10);
      int nn = -1;
      const long long* prb = V.prb + s * ns;
      for (int j = 1; j < nsi; ++j) {
        if (j == i) continue;
        const long long rb = prb[j];
        if (rb < rminb) {
          rminb = rb;
          nn = j;
        }
      }
      fc.nn_idx[i] = nn;
      fc.nn_dist[i] = nn >= 0 ? __longlong_as_double(rminb) : 0.0;
    }
  }
  __syncthreads();
}

// phase 3: stage input r = y0 + h sum_q a[r][q] f[idx[r][q]] (the reference's term order)
__device__ __forceinline__ void stage_input(const View& V, int r, double h) {
  const int K = g_rk_k[r];
  const int ne = 6 * V.nsink;
  for (int e = threadIdx.x; e < ne; e += blockDim.x) {
    double acc = g_rk_a[r][0] * V.f[(size_t)g_rk_idx[r][0] * ne + e];
    for (int q = 1; q < K; ++q) acc = acc + g_rk_a[r][q] * V.f[(size_t)g_rk_idx[r][q] * ne + e];
    V.yt[e] = V.y0[e] + h * acc;
  }
  __syncthreads();
}

__global__ void __launch_bounds__(kBlock) k_group_rkf78(GroupArgs P) {
  extern __shared__ __align__(16) double smem[];
  __shared__ Ctl S;
  const ForceCtx& fc = P.fc;
  const int ns = P.ns;
  const int l0 = ns + blockIdx.x * P.local;
  const int l1 = min(l0 + P.local, P.n);
  View V;
  V.nsink = ns + max(l1 - l0, 0);
  V.f = smem + P.o_f;
  V.y0 = smem + P.o_y0;
  V.yt = smem + P.o_yt;
  V.ys = smem + P.o_ys;
  V.yn = smem + P.o_yn;
  V.rm3 = smem + P.o_rm3;
  V.pp = smem + P.o_pp;
  V.prb = reinterpret_cast<long long*>(smem + P.o_prb);
  V.xr = smem + P.o_xr;
  V.gm = smem + P.o_gm;
  V.gbuf = smem + P.o_gbuf;
  V.red = smem + P.o_red;
  V.mu = smem + P.o_mu;
  const int smax = ns + P.local;
  V.mig = reinterpret_cast<int*>(smem + P.o_int);
  V.body = V.mig + smax;
  V.nsrc = V.body + smax;
  V.kind = V.nsrc + smax;
  V.pair = V.kind + smax;
  const int nsink = V.nsink, ne = 6 * nsink;
  const bool home = blockIdx.x == 0;
  for (int s = threadIdx.x; s < nsink; s += blockDim.x) {
    const int i = s < ns ? s : l0 + s - ns;
    V.body[s] = i;
    V.mig[s] = fc.mig_type[i];
    const int kind = gas_kind(fc, i);
    V.kind[s] = kind;
    V.nsrc[s] = (fc.type[i] <= SOL_PROTO_PLANET) ? ns : fc.cls.nm;
    V.mu[s] = SOL_GAUSS2 * (fc.mass[0] + fc.mass[i]);
    for (int k = 0; k < 3; ++k) V.gbuf[3 * s + k] = kind ? global_gas_buf(fc, i, kind)[k] : 0.0;
    if (s < ns) V.gm[s] = s >= 1 ? SOL_GAUSS2 * fc.mass[s] : 0.0;
  }
  __syncthreads();
  if (threadIdx.x == 0) {  // the (sink, source) pairs of GravityAC: sinks i >= 1, sources 1 <= j < nsrc, j != i
    int np = 0;
    for (int s = 0; s < nsink; ++s) {
      const int i = V.body[s];
      if (i == 0) continue;
      for (int j = 1; j < V.nsrc[s]; ++j)
        if (j != i) V.pair[np++] = s * 32 + j;
    }
    V.npair = np;
    S.npair = np;
  }
  for (int e = threadIdx.x; e < ne; e += blockDim.x) {
    const int s = e / 6, k = e - 6 * s;
    const int i = s < ns ? s : l0 + s - ns;
    V.y0[e] = P.y0[6 * i + k];
  }
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
  V.npair = S.npair;
  bool ok = true;
  int parity = 0;  // partials are double-buffered: a slot is rewritten two barriers after it was read
  for (int step = 0; step < P.n_steps && ok && S.status == 0; ++step) {
    if (threadIdx.x == 0) {  // Driver: bodyData->h = timeLine->hNext (:74-75)
      S.h = S.h_next;
      S.accepted = 0;
    }
    __syncthreads();
    // first evaluation with every term on (:77-82) and yscale (:87-89)
    for (int e = threadIdx.x; e < ne; e += blockDim.x) V.yt[e] = V.y0[e];
    __syncthreads();
    evaluate(P, V, S.t, SOL_EVAL_ALL, 0);
    for (int e = threadIdx.x; e < ne; e += blockDim.x) {
      const double f0 = V.f[e];
      V.ys[e] = fabs(V.y0[e]) + fabs(S.h * f0) + 1.0e-30;
      const int s = e / 6;
      if (s >= ns || home) {
        const int i = V.body[s], k = e - 6 * s;
        P.accel[6 * i + k] = f0;
        P.yscale[6 * i + k] = V.ys[e];
      }
    }
    __syncthreads();
    for (;;) {
      const double h = S.h;
      for (int r = 1; r <= 12; ++r) {
        stage_input(V, r, h);
        // migration only at the first evaluation of a driver call (:94-95)
        evaluate(P, V, S.t, SOL_EVAL_GAS_DRAG, r);
      }
      // final sum, error estimate and the scaled norm (:236-242, :252-262)
      double m = 0.0;
      for (int e = threadIdx.x; e < ne; e += blockDim.x) {
        const double D1_0 = 41.0 / 840.0, D1_5 = 34.0 / 105.0, D1_6 = 9.0 / 35.0, D1_8 = 9.0 / 280.0,
                     D1_10 = 41.0 / 840.0;
        const double* F = V.f;
        const double f0 = F[e], f10 = F[(size_t)10 * ne + e];
        const double yn = V.y0[e] + h * (D1_0 * f0 + D1_5 * F[(size_t)5 * ne + e] +
                                         D1_6 * (F[(size_t)6 * ne + e] + F[(size_t)7 * ne + e]) +
                                         D1_8 * (F[(size_t)8 * ne + e] + F[(size_t)9 * ne + e]) + D1_10 * f10);
        const double ee = h * fabs(f0 + f10 - F[(size_t)11 * ne + e] - F[(size_t)12 * ne + e]) * 41.0 / 840.0;
        V.yn[e] = yn;
        const int s = e / 6;
        if (s >= ns || home) {
          const int i = V.body[s], k = e - 6 * s;
          P.ynew[6 * i + k] = yn;
          P.err[6 * i + k] = ee;
        }
        const double qq = fabs(ee / V.ys[e]);
        m = qq > m ? qq : m;  // a NaN entry never replaces the maximum
      }
      V.red[threadIdx.x] = m;
      __syncthreads();
      for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w && V.red[threadIdx.x + w] > V.red[threadIdx.x]) V.red[threadIdx.x] = V.red[threadIdx.x + w];
        __syncthreads();
      }
      double* partial = P.partial + (size_t)parity * gridDim.x;
      parity ^= 1;
      if (threadIdx.x == 0) partial[blockIdx.x] = V.red[0];
      ok = group_barrier(P, &S.abort);
      if (!ok) break;
      if (threadIdx.x == 0) {  // every CTA takes the same decision (:98-133)
        double mx = 0.0;
        for (int b = 0; b < (int)gridDim.x; ++b) {
          const double o = gridDim.x > 1 ? __ldcg(partial + b) : V.red[0];
          if (o > mx) mx = o;
        }
        const double em = mx / S.eps;
        S.error_max = em;
        if (em < 1.0) {
          S.h_did = h;
          S.t += S.h_did;
          S.h_next = em > 1.89e-4 ? (0.9 * h * pow(em, -0.2)) : (5.0 * h);
          S.h = S.h_next;
          S.accepted = 1;
          S.n_acc++;
        } else {
          S.n_rej++;
          const double hTemp = 0.9 * h * pow(em, -0.25);
          const double hn = fabs(hTemp) > fabs(0.1 * h) ? hTemp : 0.1 * h;
          S.h = hn;
          if (S.t + hn == S.t) S.status |= SOL_DEV_UNDERFLOW;
        }
      }
      __syncthreads();
      if (S.accepted) {
        for (int e = threadIdx.x; e < ne; e += blockDim.x) {
          V.y0[e] = V.yn[e];
          const int s = e / 6;
          if (s >= ns || home) P.y0[6 * V.body[s] + (e - 6 * s)] = V.yn[e];
        }
        __syncthreads();
        break;
      }
      if (S.status) break;
    }
  }
  if (home && threadIdx.x == 0) {
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

int upload_group_tableau() {
  static bool done[64] = {};
  int dev = 0;
  SOL_CUDA(cudaGetDevice(&dev));
  if (dev >= 0 && dev < 64 && done[dev]) return SOL_OK;
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
  SOL_CUDA(cudaMemcpyToSymbol(g_rk_k, k, sizeof(k)));
  SOL_CUDA(cudaMemcpyToSymbol(g_rk_idx, idx, sizeof(idx)));
  SOL_CUDA(cudaMemcpyToSymbol(g_rk_a, a, sizeof(a)));
  if (dev >= 0 && dev < 64) done[dev] = true;
  return SOL_OK;
}

// Shared-memory layout for nsink sinks of ns sources (offsets in doubles).
size_t layout(GroupArgs& P, int nsink, int ns) {
  size_t o = 0;
  auto take = [&](int& field, size_t doubles) {
    field = (int)o;
    o += (doubles + 1) & ~(size_t)1;  // 16-byte alignment
  };
  take(P.o_f, (size_t)13 * 6 * nsink);
  take(P.o_y0, (size_t)6 * nsink);
  take(P.o_yt, (size_t)6 * nsink);
  take(P.o_ys, (size_t)6 * nsink);
  take(P.o_yn, (size_t)6 * nsink);
  take(P.o_rm3, (size_t)nsink);
  take(P.o_pp, (size_t)3 * nsink * ns);
  take(P.o_prb, (size_t)nsink * ns);
  take(P.o_xr, (size_t)3 * ns);
  take(P.o_gm, (size_t)ns);
  take(P.o_gbuf, (size_t)3 * nsink);
  take(P.o_red, (size_t)kBlock);
  take(P.o_mu, (size_t)nsink);
  // ints: migType, body index, sources, gas kind (nsink each) and the pair list (nsink * ns)
  take(P.o_int, ((size_t)4 * nsink + (size_t)nsink * ns + 1) / 2);
  return o * sizeof(double);
}

}  // namespace

// Whether the system can run its RKF78 driver calls on the group path.
int sol_group_eligible(const sol_ctx* c) {
  if (c->barycentric) return 0;
  const int ns = c->cls.nm + c->cls.n_spl;
  return ns >= 1 && ns <= kMaxSources && c->n - ns <= 152 * 2 * kMaxLocal;
}

// n_steps RKF78 driver calls in one cooperative launch of the group kernel.
// Returns SOL_ERR_STATE (nothing launched) when the system does not fit.
int sol_group_rkf78(sol_ctx* c, int n_steps) {
  if (!sol_group_eligible(c)) return SOL_ERR_STATE;
  if (!c->d_persist) {
    const size_t doubles = 2 * 7 * 32 + 4096 + 8;
    if (cudaMalloc((void**)&c->d_persist, sizeof(double) * doubles) != cudaSuccess) {
      sol_set_error("cudaMalloc of the persistent-driver scratch failed");
      return SOL_ERR_NOMEM;
    }
    SOL_CUDA(cudaMemset(c->d_persist, 0, sizeof(double) * doubles));
  }
  int n_sm = 0;
  SOL_CUDA(cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, c->device));
  GroupArgs P;
  memset(&P, 0, sizeof(P));
  const int ns = c->cls.nm + c->cls.n_spl;
  // bodies per CTA: the smallest power of two from 16 whose grid is co-resident
  int local = 0, grid = 0;
  size_t smem = 0;
  for (int cand = kMinLocal; cand <= kMaxLocal; cand *= 2) {
    const int others = c->n - ns;
    const int g = others > 0 ? (others + cand - 1) / cand : 1;
    // at least half an SM's shared memory, so that the CTAs spread one per SM:
    // CTAs packed onto one SM would share its FP64 pipes
    const size_t sm = std::max(layout(P, ns + cand, ns), (size_t)kSpreadSmem);
    if (sm > 200 * 1024) break;
    SOL_CUDA(cudaFuncSetAttribute(k_group_rkf78, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    int per_sm = 0;
    SOL_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_group_rkf78, kBlock, sm));
    if (g <= per_sm * n_sm && g <= 2048) {
      local = cand;
      grid = g;
      smem = sm;
      break;
    }
  }
  if (!local) return SOL_ERR_STATE;
  layout(P, ns + local, ns);
  RET(upload_group_tableau());
  P.fc = c->fc;
  P.y0 = c->d_y0;
  P.accel = c->d_accel;
  P.yscale = c->d_yscale;
  P.ynew = c->d_y;
  P.err = c->d_err;
  P.partial = c->d_persist + 2 * 7 * 32;
  unsigned* words = reinterpret_cast<unsigned*>(c->d_persist + 2 * 7 * 32 + 4096);
  P.bar_count = words;
  P.bar_gen = words + 1;
  P.abort_flag = reinterpret_cast<int*>(words + 2);
  P.ctrl = c->d_ctrl;
  P.n = c->n;
  P.ns = ns;
  P.local = local;
  P.n_steps = n_steps;
  SOL_CUDA(cudaMemsetAsync(words, 0, 4 * sizeof(unsigned), c->stream));
  void* args[] = {&P};
  SOL_CUDA(cudaLaunchCooperativeKernel((const void*)k_group_rkf78, grid, kBlock, args, smem, c->stream));
  SOL_LAUNCHED();
  return SOL_OK;
}
