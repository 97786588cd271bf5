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
// other CTA leave at its next barrier.  (sol_set_wait_test lowers the limit
// and can keep one CTA from arriving, so that tests reach this path.)
#include <atomic>
#include <mutex>
#include <algorithm>
#include <cmath>
#include <cstring>

#include "sol_crmath.cuh"

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
// Phase-1 work per virtual warp in cycles (measured on the GB300, one warp:
// pow 5,800, exp 1,100, log10 2,200, sqrt 680, division 430, an FP64 add or
// multiply 64), for the greedy schedule of the virtual warps onto the warps.
constexpr int kCostRm3 = 2000, kCostPair = 2000, kCostMig = 30000;
constexpr int kCostRole0 = 6600, kCostRole1 = 8200, kCostRole2 = 6700, kCostRole3 = 9800;  // the drag's roles
constexpr int kMaxVw = 3 + 96 + 12 + 3;  // rm3 + pairs + drag roles + migration virtual warps of 96 sinks
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
  unsigned spin;        // spin limit of the group barrier
  int skip_cta;         // failure-path tests: this CTA never arrives (-1: none)
  sol_ctrl* ctrl;
  int n;
  int ns;               // sources: nm + n_spl
  int local;            // other bodies per CTA
  int n_steps;
  int rk4;              // RungeKutta4 driver calls instead of RungeKuttaFehlberg78
  int sim;              // the Simulator's step loop (sol_run_until)
  double e3, h3, cf;    // its event thresholds (0: off)
  sol_sim_line* line;
  int* reason;
  int* ev;              // per-CTA event flags, double-buffered
  double* yprev;        // the state at the start of a step that stops with an event (or null)
  // shared-memory layout (offsets in doubles)
  int o_f, o_y0, o_yt, o_ys, o_yn, o_rm3, o_pp, o_prb, o_xr, o_gm, o_gbuf, o_red, o_mu, o_dv, o_int;
};

__device__ bool group_barrier(const GroupArgs& P, int* s_abort) {
  __syncthreads();
  if (gridDim.x > 1 && threadIdx.x == 0) {
    volatile unsigned* gen = P.bar_gen;
    const unsigned g = *gen;
    __threadfence();
    if ((int)blockIdx.x != P.skip_cta && atomicAdd(P.bar_count, 1u) == gridDim.x - 1) {
      *P.bar_count = 0;
      __threadfence();
      atomicAdd(P.bar_gen, 1u);
    } else {
      bool ok = false;
      for (uint32_t k = 0; k < P.spin; ++k) {
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
  double fac[4];  // RungeKutta4: ReductionFactor at the stage times t + c h
  double t, h, h_next, h_did, error_max, eps;
  long long n_acc, n_rej;
  int status, accepted, abort, npair, ndrag, nmig;
  double m0pt, factor;
  int event, stop, reason, flush;
  sol_sim_line L;
  unsigned char sched_n[8];
  unsigned char sched[8 * kMaxVw];
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
  int* dlist;   // [ndrag]: slots of the planetesimals (drag)
  int* mlist;   // [nmig]: slots of the migrating bodies
  int nsink, npair, ndrag, nmig;
  double factor, m0pt;  // ReductionFactor at the step's time, m0^pt
  const unsigned char* sched;  // [2][4][kMaxVw]: virtual warps of each warp (0: with migration, 1: without)
  const unsigned char* sched_n;  // [2][4]
  int* event;                    // set when an event predicate holds on the attempt's last evaluation
  double* dv;                    // [6][nsink]: the drag's partial results of each planetesimal
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

// Migration of one massive body (the migration part of add_gas_terms): only
// with its flag and while migType allows it (a migration that reaches its
// stop sets migType to No).  Out of line, like the drag: thousands of
// instructions inlined into the stage loop evict the hot path from the
// instruction cache (measured: 3x slower stages).
__device__ __noinline__ void mig_compute(const ForceCtx& fc, int i, int kind, const double* yi, double factor,
                                         uint32_t flags, double* buf, int* mig) {
  const GasDev& g = fc.gas;
  const double m0 = fc.mass[0];
  double d[3];
  if (kind == 2) {
    if (!((flags & SOL_EVAL_TYPE_I) && *mig == SOL_MIGRATION_TYPE_I)) return;
    if (!sol_migration_type1(g, factor, m0, fc.mass[i], fc.mig_stop_at[i], yi, d)) *mig = SOL_MIGRATION_NO;
  } else {
    if (!((flags & SOL_EVAL_TYPE_II) && *mig == SOL_MIGRATION_TYPE_II)) return;
    if (!sol_migration_type2(g, factor, m0, fc.mass[i], fc.mig_stop_at[i], yi, d)) *mig = SOL_MIGRATION_NO;
  }
  buf[0] = d[0];
  buf[1] = d[1];
  buf[2] = d[2];
}

// The regime part of GasDragAC (Acceleration.cpp:364-401) from lambda(r),
// r, the density's two factors and the gas velocity.
__device__ __forceinline__ void drag_finish(const GasDev& g, double factor, double m0pt, const double* yi,
                                           double radius, double density, double cd, double gs, double ge,
                                           double lambda, double r, double ex, double rp, double vgx, double vgy,
                                           double out[3]) {
  const double ux = yi[3] - vgx, uy = yi[4] - vgy, uz = yi[5] - 0.0;
  const double rho = rp * ex;
  const double rhoGas = factor * rho;
  double C;
  if (radius <= 0.1 * lambda) {
    // MeanThermalSpeed_CMU(m0, r) -> Temperature_CMU(r, m0) (arguments swapped, :241)
    const double cT = g.sh_c * g.sh_c * r * g.mmw * g.ctp;
    const double vth = g.cvth * sqrt(cT * m0pt);
    C = ge * vth * rhoGas;
  } else if (radius >= 10.0 * lambda) {
    const double ul = sqrt(ux * ux + uy * uy + uz * uz);
    C = gs * ul * rhoGas;
  } else {
    const double l1 = 0.1 * lambda, l2 = 10.0 * lambda;
    const double gE = 1.0 / (density * l1);
    const double gS = 3.0 / 8.0 * cd / (density * l2);
    const double cT = g.sh_c * g.sh_c * r * g.mmw * g.ctp;
    const double vth = g.cvth * sqrt(cT * m0pt);
    const double ul = sqrt(ux * ux + uy * uy + uz * uz);
    const double K = gS * ul / (gE * vth);
    const double eta = l2 / l1;
    const double kappa = log10(K) / log10(eta);
    const double gamma = gE * vth * pow(l1, -kappa);
    C = gamma * pow(radius, kappa) * rhoGas;
  }
  out[0] = -C * ux;
  out[1] = -C * uy;
  out[2] = -C * uz;
}

// One of the four independent parts of GasDragAC (Acceleration.cpp:342-363,
// gas_velocity and gas_density_at of GasComponent.cpp:97-157) for the
// planetesimal of this lane, in the operations of sol_gas_drag:
//   role 0: r and the mean free path lambda(r);
//   role 1: the density's vertical exponential exp(-(z / h(rc))^2);
//   role 2: the density's power law (or the inner-edge form);
//   role 3: the gas velocity with its eta(rc) correction.
// A warp takes one role for 32 planetesimals, so its lanes share the
// exponent of their pow and run the same instructions; the four roles run in
// four warps at once and drag_finish combines them.
__device__ __noinline__ void drag_role(const GasDev& g, int role, double m0, const double* yi, double out[2]) {
  const double x = yi[0], y = yi[1], z = yi[2];
  if (role == 0) {
    const double r = sqrt(x * x + y * y + z * z);
    out[0] = sol_pl(g.mfp_c, g.mfp_i, r);
    out[1] = r;
  } else if (role == 1) {
    const double rc = sqrt(x * x + y * y);
    const double hh = sol_pl(g.sh_c, g.sh_i, rc);
    const double qq = z / hh;
    out[0] = exp(-(qq * qq));
  } else if (role == 2) {
    const double rc = sqrt(x * x + y * y);
    if (g.inner_edge < rc) {
      out[0] = sol_pl(g.rho_c, g.rho_i, rc);
    } else {
      const double r2c = rc * rc;
      out[0] = (g.rho_c * pow(g.inner_edge, g.rho_i - 4.0)) * (r2c * r2c);
    }
  } else {
    double vgx = 0.0, vgy = 0.0;
    const double mu = SOL_GAUSS2 * m0;
    const double rc = sqrt(x * x + y * y);
    const double vc = sqrt(mu / rc);
    if (x == 0.0 && y == 0.0) {
    } else if (y == 0.0) {
      vgy = x > 0.0 ? vc : -vc;
    } else if (x == 0.0) {
      vgx = y > 0.0 ? -vc : vc;
    } else if (x >= y) {
      const double p = y / x;
      vgy = x >= 0 ? vc / sqrt(1.0 + p * p) : -vc / sqrt(1.0 + p * p);
      vgx = -vgy * p;
    } else {
      const double p = x / y;
      vgx = y >= 0 ? -vc / sqrt(1.0 + p * p) : vc / sqrt(1.0 + p * p);
      vgy = -vgx * p;
    }
    const double v = sqrt(1.0 - 2.0 * sol_pl(g.eta_c, g.eta_i, rc));
    vgx *= v;
    vgy *= v;
    out[0] = vgx;
    out[1] = vgy;
  }
}

// One force evaluation of the CTA's sinks on the stage input V.yt (phases 1
// and 2); writes f[r] and, where this CTA owns the body, rm3, the nearest
// neighbour and the gas buffers in global memory.
__device__ __noinline__ void evaluate(const GroupArgs& P, const View& V, double t, uint32_t flags, int r) {
  const ForceCtx& fc = P.fc;
  const int ns = P.ns, nsink = V.nsink;
  const bool home = blockIdx.x == 0;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // phase 1: the three kinds of work in separate virtual warps
  const int w_rm3 = (nsink + 31) >> 5;
  const int w_pair = (V.npair + 31) >> 5;
  const int sidx = (flags & (SOL_EVAL_TYPE_I | SOL_EVAL_TYPE_II)) ? 0 : 1;
  const bool drag = V.ndrag > 0 && (flags & SOL_EVAL_GAS_DRAG);
  const int w_role = (V.ndrag + 31) >> 5;  // virtual warps per drag role
  const int w_drag = V.ndrag > 0 ? 4 * w_role : 0;
  const int nmine = warp < 4 ? V.sched_n[sidx * 4 + warp] : 0;
  for (int t = 0; t < nmine; ++t) {
    const int vw = V.sched[(sidx * 4 + warp) * kMaxVw + t];
    if (!drag && vw >= w_rm3 + w_pair && vw < w_rm3 + w_pair + w_drag) continue;
    if (vw < w_rm3) {
      const int s = vw * 32 + lane;
      if (s < nsink) {
        const int i = V.body[s];
        const double* y = V.yt + 6 * s;
        double rm3 = 0.0;
        if (i >= 1) {  // Acceleration.cpp:259-261
          const double x = y[0], yy = y[1], z = y[2];
          const double r2 = x * x + yy * yy + z * z;
          double rr;
          sol_ref_rinv3(r2, rr, rm3);
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
        double rij, rijm3;
        sol_ref_rinv3(rij2, rij, rijm3);
        V.prb[s * ns + j] = __double_as_longlong(rij);
        V.pp[(0 * nsink + s) * ns + j] = xij * rijm3;
        V.pp[(1 * nsink + s) * ns + j] = yij * rijm3;
        V.pp[(2 * nsink + s) * ns + j] = zij * rijm3;
      }
    } else if (vw < w_rm3 + w_pair + w_drag) {  // drag: one role for 32 planetesimals
      const int role = (vw - w_rm3 - w_pair) / w_role;
      const int d = ((vw - w_rm3 - w_pair) - role * w_role) * 32 + lane;
      if (d < V.ndrag) {
        const int sd = V.dlist[d];
        double o[2];
        drag_role(fc.gas, role, fc.mass[0], V.yt + 6 * sd, o);
        const int k0 = role == 0 ? 0 : role == 1 ? 2 : role == 2 ? 3 : 4;
        V.dv[k0 * nsink + d] = o[0];
        if (role == 0 || role == 3) V.dv[(k0 + 1) * nsink + d] = o[1];
      }
    } else {  // migration: a lane per massive body
      const int m = (vw - w_rm3 - w_pair - w_drag) * 32 + lane;
      if (m < V.nmig) {
        const int s = V.mlist[m], i = V.body[s], kind = V.kind[s];
        mig_compute(fc, i, kind, V.yt + 6 * s, V.factor, flags, V.gbuf + 3 * s, V.mig + s);
        if (s >= ns || home) {
          double* gb = global_gas_buf(fc, i, kind);
          gb[0] = V.gbuf[3 * s + 0];
          gb[1] = V.gbuf[3 * s + 1];
          gb[2] = V.gbuf[3 * s + 2];
          fc.mig_type[i] = V.mig[s];
        }
      }
    }
  }
  __syncthreads();
  if (drag) {  // phase 1b: the drag's regime part from the four roles, a lane per planetesimal
    for (int d = threadIdx.x; d < V.ndrag; d += blockDim.x) {
      const int sd = V.dlist[d], i = V.body[sd];
      double out[3];
      drag_finish(fc.gas, V.factor, V.m0pt, V.yt + 6 * sd, fc.radius[i], fc.density[i], fc.cd[i],
                  fc.gamma_stokes[i], fc.gamma_epstein[i], V.dv[0 * nsink + d], V.dv[1 * nsink + d],
                  V.dv[2 * nsink + d], V.dv[3 * nsink + d], V.dv[4 * nsink + d], V.dv[5 * nsink + d], out);
      for (int k = 0; k < 3; ++k) V.gbuf[3 * sd + k] = out[k];
      if (sd >= ns || home) {
        double* gb = global_gas_buf(fc, i, 1);
        for (int k = 0; k < 3; ++k) gb[k] = out[k];
      }
    }
    __syncthreads();
  }
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
      if (P.sim && r == (P.rk4 ? 3 : 12)) {  // CheckEvent's predicates on the step's last evaluation
        const double rm3 = V.rm3[s];
        const bool ev = (P.e3 > 0.0 && rm3 < P.e3) || (P.h3 > 0.0 && rm3 > P.h3) ||
                        (P.cf > 0.0 && nn >= 0 && P.cf * (fc.radius[i] + fc.radius[nn]) > __longlong_as_double(rminb));
        if (ev) atomicOr(V.event, 1);
      }
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

// Simulator::DecisionMaking up to where the host has work
// (Simulator.cpp:181-250), after an accepted step of S.h_did; thread 0.
__device__ __forceinline__ void sim_decision(Ctl& S, int any) {
  sol_sim_line& L = S.L;
  L.steps += 1;
  L.elapsed += S.h_did;
  L.last_save += S.h_did;
  S.flush = 0;
  if (any) {
    S.reason = SOL_STOP_EVENT;
    S.stop = 1;
  } else {
    const double clock = L.relative_end ? L.elapsed : S.t;
    if (fabs(clock) >= fabs(L.length)) {
      S.reason = SOL_STOP_LENGTH;
      S.stop = 1;
    } else {
      if (fabs(clock + S.h_next) > fabs(L.length)) S.h_next = L.length - clock;
      if (fabs(L.last_save) >= fabs(L.output)) {
        S.reason = SOL_STOP_OUTPUT;
        S.stop = 1;
      } else {
        if (fabs(L.last_save + S.h_next) > fabs(L.output)) S.h_next = L.output - L.last_save;
        S.flush = (L.steps % 100) == 0;  // Tools::CheckAgainstSmallestNumber every CheckForSM steps
      }
    }
  }
  S.h = S.h_next;
}

// An accepted step: y0 <- the new state (flushed below the smallest number
// when due), written where this CTA owns the body; the step-start state kept
// when the step stops with an event.
__device__ __forceinline__ void commit_step(const GroupArgs& P, const View& V, const Ctl& S, int ne, int ns,
                                            bool home) {
  const bool keep_start = P.sim && P.yprev && S.stop && S.reason == SOL_STOP_EVENT;
  for (int e = threadIdx.x; e < ne; e += blockDim.x) {
    double v = V.yn[e];
    const int s = e / 6;
    if (keep_start && (s >= ns || home)) P.yprev[6 * V.body[s] + (e - 6 * s)] = V.y0[e];
    if (S.flush && fabs(v) < 1.0e-50) v = 0.0;
    V.y0[e] = v;
    if (s >= ns || home) P.y0[6 * V.body[s] + (e - 6 * s)] = v;
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
  V.dlist = V.pair + smax * ns;
  V.mlist = V.dlist + smax;
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
  for (int e = threadIdx.x; e < ne; e += blockDim.x) {
    const int s = e / 6, k = e - 6 * s;
    const int i = s < ns ? s : l0 + s - ns;
    V.y0[e] = P.y0[6 * i + k];
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
    int nd = 0, nmg = 0;
    for (int q = 0; q < nsink; ++q) {
      if (V.kind[q] == 1) V.dlist[nd++] = q;
      else if (V.kind[q] >= 2) V.mlist[nmg++] = q;
    }
    S.ndrag = nd;
    S.nmig = nmg;
    S.m0pt = fc.gas.present ? pow(fc.mass[0], fc.gas.pt) : 0.0;
    // phase-1 schedules: the virtual warps (rm3, pairs, drag roles,
    // migration) onto the four warps, longest first onto the least loaded
    const int w_rm3 = (nsink + 31) >> 5, w_pair = (np + 31) >> 5;
    const int w_role = (nd + 31) >> 5, w_drag = nd > 0 ? 4 * w_role : 0;
    for (int sidx = 0; sidx < 2; ++sidx) {
      const int w_mig = (sidx == 0 && nmg > 0) ? (nmg + 31) >> 5 : 0;
      const int nvw = w_rm3 + w_pair + w_drag + w_mig;
      int load[4] = {0, 0, 0, 0}, cnt[4] = {0, 0, 0, 0};
      bool done[kMaxVw];
      for (int vw = 0; vw < nvw; ++vw) done[vw] = false;
      for (int it = 0; it < nvw; ++it) {
        int pick = -1, pc = -1;
        for (int vw = 0; vw < nvw; ++vw) {
          if (done[vw]) continue;
          int c2;
          if (vw < w_rm3) c2 = kCostRm3;
          else if (vw < w_rm3 + w_pair) c2 = kCostPair;
          else if (vw < w_rm3 + w_pair + w_drag) {
            const int role = (vw - w_rm3 - w_pair) / w_role;
            c2 = role == 0 ? kCostRole0 : role == 1 ? kCostRole1 : role == 2 ? kCostRole2 : kCostRole3;
          }
          else c2 = kCostMig;
          if (c2 > pc) {
            pc = c2;
            pick = vw;
          }
        }
        done[pick] = true;
        int wmin = 0;
        for (int w = 1; w < 4; ++w)
          if (load[w] < load[wmin]) wmin = w;
        load[wmin] += pc;
        S.sched[(sidx * 4 + wmin) * kMaxVw + cnt[wmin]++] = (unsigned char)pick;
      }
      for (int w = 0; w < 4; ++w) S.sched_n[sidx * 4 + w] = (unsigned char)cnt[w];
    }
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
    S.event = 0;
    S.stop = 0;
    S.reason = SOL_STOP_STEPS;
    S.flush = 0;
    if (P.sim) S.L = *P.line;
  }
  __syncthreads();
  V.npair = S.npair;
  V.ndrag = S.ndrag;
  V.nmig = S.nmig;
  V.m0pt = S.m0pt;
  V.sched = S.sched;
  V.sched_n = S.sched_n;
  V.event = &S.event;
  V.dv = smem + P.o_dv;
  bool ok = true;
  int parity = 0;  // partials are double-buffered: a slot is rewritten two barriers after it was read
  for (int step = 0; step < P.n_steps && ok && S.status == 0 && !S.stop; ++step) {
    if (threadIdx.x == 0) {  // Driver: bodyData->h = timeLine->hNext (:74-75)
      S.h = S.h_next;
      S.accepted = 0;
      // RKF78 evaluates every stage at the step's start time; RK4 at t + c h
      // (RungeKutta4.cpp:101-116)
      S.factor = fc.gas.present ? sol_reduction_factor(fc.gas, S.t) : 1.0;
      if (P.rk4) {
        const double cst[4] = {0.0, 1.0 / 2.0, 1.0 / 2.0, 1.0};
        for (int q = 0; q < 4; ++q) S.fac[q] = fc.gas.present ? sol_reduction_factor(fc.gas, S.t + cst[q] * S.h) : 1.0;
      }
    }
    __syncthreads();
    V.factor = S.factor;
    // first evaluation with every term on (:77-82) and yscale (:87-89)
    for (int e = threadIdx.x; e < ne; e += blockDim.x) V.yt[e] = V.y0[e];
    __syncthreads();
    evaluate(P, V, S.t, SOL_EVAL_ALL, 0);
    if (P.rk4) {  // RungeKutta4::Driver and Step (RungeKutta4.cpp:20-129)
      for (int e = threadIdx.x; e < ne; e += blockDim.x) {
        const int s = e / 6;
        if (s >= ns || home) P.accel[6 * V.body[s] + (e - 6 * s)] = V.f[e];
      }
      const double h = S.h;
      const double a[4] = {0.0, 1.0 / 2.0, 1.0 / 2.0, 1.0};  // a21, a32, a43
      for (int r = 1; r <= 3; ++r) {
        const double* fp = V.f + (size_t)(r - 1) * ne;
        for (int e = threadIdx.x; e < ne; e += blockDim.x) V.yt[e] = V.y0[e] + h * (a[r] * fp[e]);
        __syncthreads();
        V.factor = S.fac[r];
        evaluate(P, V, S.t, SOL_EVAL_GAS_DRAG, r);
      }
      const double b1 = 1.0 / 6.0, b2 = 1.0 / 3.0, b3 = 1.0 / 3.0, b4 = 1.0 / 6.0;
      for (int e = threadIdx.x; e < ne; e += blockDim.x) {
        const double* F = V.f;
        const double yn = V.y0[e] + h * (b1 * F[e] + b2 * F[(size_t)ne + e] + b3 * F[(size_t)2 * ne + e] +
                                         b4 * F[(size_t)3 * ne + e]);
        V.yn[e] = yn;
        const int s = e / 6;
        if (s >= ns || home) P.ynew[6 * V.body[s] + (e - 6 * s)] = yn;
      }
      int any_ev = 0;
      if (P.sim) {  // the event flags of every CTA
        int* evp = P.ev + (size_t)parity * gridDim.x;
        parity ^= 1;
        if (threadIdx.x == 0) evp[blockIdx.x] = S.event;
        ok = group_barrier(P, &S.abort);
        if (!ok) break;
        if (threadIdx.x < 32) {
          for (int b = threadIdx.x; b < (int)gridDim.x; b += 32) any_ev |= gridDim.x > 1 ? __ldcg(evp + b) : S.event;
          any_ev = (int)__reduce_or_sync(0xFFFFFFFFu, (unsigned)any_ev);
        }
      } else {
        __syncthreads();
      }
      if (threadIdx.x == 0) {
        S.h_did = h;
        S.t += S.h_did;
        S.h_next = h;  // RK4 keeps its step size (and a clamp of it)
        S.accepted = 1;
        S.n_acc++;
        if (P.sim) sim_decision(S, any_ev);
        S.event = 0;
      }
      __syncthreads();
      commit_step(P, V, S, ne, ns, home);
      continue;
    }
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
      int* evp = P.sim ? P.ev + (size_t)parity * gridDim.x : nullptr;
      parity ^= 1;
      if (threadIdx.x == 0) {
        partial[blockIdx.x] = V.red[0];
        if (P.sim) evp[blockIdx.x] = S.event;
      }
      ok = group_barrier(P, &S.abort);
      if (!ok) break;
      // warp 0 gathers every CTA's partial maximum and event flag at once
      double mx = 0.0;
      int any_ev = 0;
      if (threadIdx.x < 32) {
        for (int b = threadIdx.x; b < (int)gridDim.x; b += 32) {
          const double o = gridDim.x > 1 ? __ldcg(partial + b) : V.red[0];
          mx = o > mx ? o : mx;
          if (P.sim) any_ev |= gridDim.x > 1 ? __ldcg(evp + b) : S.event;
        }
        for (int w = 16; w > 0; w >>= 1) {
          const double o = __shfl_xor_sync(0xFFFFFFFFu, mx, w);
          mx = o > mx ? o : mx;
        }
        any_ev = (int)__reduce_or_sync(0xFFFFFFFFu, (unsigned)any_ev);
      }
      if (threadIdx.x == 0) {  // every CTA takes the same decision (:98-133)
        const double em = mx / S.eps;
        S.error_max = em;
        if (em < 1.0) {
          S.h_did = h;
          S.t += S.h_did;
          S.h_next = em > 1.89e-4 ? (0.9 * h * sol_inv_root<5>(em)) : (5.0 * h);
          S.h = S.h_next;
          S.accepted = 1;
          S.n_acc++;
          if (P.sim) sim_decision(S, any_ev);
        } else {
          S.n_rej++;
          const double hTemp = 0.9 * h * sol_inv_root<4>(em);
          const double hn = fabs(hTemp) > fabs(0.1 * h) ? hTemp : 0.1 * h;
          S.h = hn;
          if (S.t + hn == S.t) S.status |= SOL_DEV_UNDERFLOW;
        }
        S.event = 0;
      }
      __syncthreads();
      if (S.accepted) {
        commit_step(P, V, S, ne, ns, home);
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
    if (P.sim) {
      sol_sim_line L = S.L;
      L.time = S.t;
      L.h_next = S.h_next;
      L.h_did = S.h_did;
      *P.line = L;
      *P.reason = S.stop ? S.reason : SOL_STOP_STEPS;
    }
  }
}

int upload_group_tableau() {
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
  SOL_CUDA(cudaMemcpyToSymbol(g_rk_k, k, sizeof(k)));
  SOL_CUDA(cudaMemcpyToSymbol(g_rk_idx, idx, sizeof(idx)));
  SOL_CUDA(cudaMemcpyToSymbol(g_rk_a, a, sizeof(a)));
  if (dev >= 0 && dev < 64) done[dev].store(true, std::memory_order_release);
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
  take(P.o_dv, (size_t)6 * nsink);
  // ints: migType, body index, sources, gas kind (nsink each), the pair list (nsink * ns),
  // the drag and migration lists (nsink each)
  take(P.o_int, ((size_t)6 * nsink + (size_t)nsink * ns + 1) / 2);
  return o * sizeof(double);
}

}  // namespace

// Whether the system can run its RKF78 / RK4 driver calls on the group path.
int sol_group_eligible(const sol_ctx* c) {
  if (c->barycentric) return 0;
  const int ns = c->cls.nm + c->cls.n_spl;
  return ns >= 1 && ns <= kMaxSources && c->n - ns <= 152 * 2 * kMaxLocal;
}

// n_steps RKF78 (or, with rk4, RungeKutta4) driver calls in one cooperative
// launch of the group kernel.  Returns SOL_ERR_STATE (nothing launched) when
// the system does not fit.
int sol_group_rkf78(sol_ctx* c, int n_steps, const GroupSim* sim, int rk4) {
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
  P.spin = c->test_spin ? c->test_spin : SOL_SPIN_LIMIT;
  P.skip_cta = c->test_skip_cta;
  P.ctrl = c->d_ctrl;
  P.n = c->n;
  P.ns = ns;
  P.local = local;
  P.n_steps = n_steps;
  P.rk4 = rk4 ? 1 : 0;
  if (sim) {
    if (grid > kGroupMaxCtas) return SOL_ERR_STATE;
    P.sim = 1;
    P.e3 = sim->e3;
    P.h3 = sim->h3;
    P.cf = sim->cf;
    P.line = sim->line;
    P.reason = sim->reason;
    P.ev = sim->ev;
    P.yprev = sim->yprev;
  }
  SOL_CUDA(cudaMemsetAsync(words, 0, 4 * sizeof(unsigned), c->stream));
  void* args[] = {&P};
  SOL_CUDA(cudaLaunchCooperativeKernel((const void*)k_group_rkf78, grid, kBlock, args, smem, c->stream));
  SOL_LAUNCHED();
  return SOL_OK;
}
