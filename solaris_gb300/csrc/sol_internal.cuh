// Internal definitions shared by the translation units of libsolaris_gb300.
// The library is compiled with --fmad=false: plain arithmetic below rounds
// every operation like the reference's x86-64 build; fused multiply-adds are
// written out explicitly (__fma_rn) where they are intended.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/solaris_gb300.h"

#define SOL_GAUSS2 2.959122082855911025e-4  // Solaris/Constants.h:29
#define SOL_GAUSS 1.720209895e-2            // Solaris/Constants.h:28
#define SOL_PI 3.14159265358979323846
#define SOL_SQRT_TWO_PI 2.50662827463100024161

// ---- error reporting --------------------------------------------------------
void sol_set_error(const char* fmt, ...);
int sol_cuda_fail(cudaError_t e, const char* what, const char* file, int line);
#define SOL_CUDA(call)                                                        \
  do {                                                                        \
    cudaError_t e_ = (call);                                                  \
    if (e_ != cudaSuccess) return sol_cuda_fail(e_, #call, __FILE__, __LINE__); \
  } while (0)
#define SOL_LAUNCHED()                                                        \
  do {                                                                        \
    sol_count_launch();                                                       \
    cudaError_t e_ = cudaPeekAtLastError();                                   \
    if (e_ != cudaSuccess) return sol_cuda_fail(e_, "kernel launch", __FILE__, __LINE__); \
  } while (0)
void sol_count_launch();

// Spin limit of every bounded device wait (mbarrier phases).
#define SOL_SPIN_LIMIT (1u << 26)

// Device status word bits (sol_ctrl::dev_status).
#define SOL_DEV_TIMEOUT 1
#define SOL_DEV_UNDERFLOW 2
#define SOL_DEV_MAXITER 4

// ---- gas model on the device (GasComponent, Solaris/GasComponent.cpp) -------
struct GasDev {
  int present;
  int decrease_type;
  int quirks;
  int barycentric;
  double alpha, time_scale, t0, t1, inner_edge, mmw;
  double eta_c, eta_i, tau_c, tau_i, sh_c, sh_i, rho_c, rho_i, mfp_c, mfp_i;
  // function-local statics of GasComponent::MeanThermalSpeed_CMU /
  // Temperature_CMU (:223-241), computed once on the host.
  double cvth, ctp, pt;
  double abs_rho_index;  // |density.index| as the reference build evaluates it
};

// Layout of a system's bodies (NBodies, Solaris/NBodies.h:62-88).
struct Classes {
  int n;          // total
  int n_central;
  int n_giant;
  int n_rocky;
  int n_proto;
  int n_spl;      // super-planetesimals
  int n_pl;       // planetesimals
  int nm;         // NOfMassive = central + giant + rocky + proto
};

// Time of a force evaluation: t = *base + c * (*h) (device-driven), or t_host.
struct TimeSpec {
  const double* base;
  const double* h;
  double c;
  double t_host;
};

// Device control block of the integrator drivers.
struct sol_ctrl {
  double t;          // TimeLine::time
  double h;          // BodyData::h (trial step of the current attempt)
  double h_next;     // TimeLine::hNext
  double h_did;      // TimeLine::hDid
  double error_max;  // last GetErrorMax
  double eps;        // integrator epsilon
  int accepted;      // 1 once the current driver call has accepted a step
  int iter;          // Dormand-Prince iteration counter
  int dev_status;    // SOL_DEV_* bits
  int pad;
  long long n_accepted, n_rejected, n_evals;
  int steps_left;    // driver calls still to run in a device-side loop
  int keep_going;    // condition of the device-side step loop
};

// Force-evaluation arguments that do not change between calls.
struct ForceCtx {
  Classes cls;
  int npad;            // padded source count (multiple of the tile)
  int barycentric;
  int precision;
  GasDev gas;
  const int32_t* type;
  int32_t* mig_type;   // mutated by migration (Acceleration.cpp:439-443)
  const double* mig_stop_at;
  const double* mass;
  const double* radius;
  const double* density;
  const double* cd;
  const double* gamma_stokes;
  const double* gamma_epstein;
  double* rm3;         // Acceleration::rm3
  int32_t* nn_idx;     // BodyData::indexOfNN
  double* nn_dist;     // BodyData::distanceOfNN
  double* src;         // SoA source arrays: 8 x npad doubles
  double* drag;        // accelGasDrag [3 * (spl + pl)]
  double* mig1;        // accelMigrationTypeI [3 * (rocky + proto)]
  double* mig2;        // accelMigrationTypeII [3 * giant]
  double* ind_part;    // per-block partial sums of the indirect term
  double* ind_sum;     // [6]: indirect sums over [1, nm) and [1, nm + spl)
  int n_ind_blocks;
  int has_mig1, has_mig2;
  // sinks evaluated: [sink_lo, sink_hi); sink_hi == 0 means every body (a
  // rank of a sink-partitioned system evaluates its own block)
  int sink_lo, sink_hi;
};
__host__ __device__ __forceinline__ int sol_sink_hi(const ForceCtx& fc) { return fc.sink_hi ? fc.sink_hi : fc.cls.n; }

// A captured driver call (RKF78 or DP) with its device-side attempt loop.
struct DriverGraph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int precision = -1;
  int valid = 0;
  int k_pro = 0, k_body = 0, k_epi = 0;  // kernels per prologue / attempt / epilogue
};
void sol_graph_release(DriverGraph& G);
void sol_capture_begin();
void sol_capture_end();
long long sol_capture_count();

struct sol_adjoint_state;
void sol_adjoint_free(sol_adjoint_state* a);

struct sol_ctx {
  int device;
  cudaStream_t stream;
  sol_nbodies counts;
  Classes cls;
  int n, nv, npad;
  int barycentric;
  int precision;
  uint32_t eval_flags;
  int has_gas;
  sol_gas_component gas_host;
  double eps;
  ForceCtx fc;
  // device buffers
  int32_t *d_type, *d_mig_type;
  double *d_mig_stop_at, *d_mass, *d_radius, *d_density, *d_cd, *d_gs, *d_ge;
  double *d_rm3, *d_nn_dist, *d_src, *d_drag, *d_mig1, *d_mig2, *d_ind_part, *d_ind_sum;
  int32_t* d_nn_idx;
  double *d_y0, *d_y, *d_accel, *d_yscale, *d_err, *d_ytmp, *d_fk[13];
  double *d_io_in, *d_io_out;  // boundary staging for host-buffer calls
  double* d_partial;           // block partial maxima of the error norm
  double* d_part;              // per-chunk partial sums of the split pair kernels
  int n_partial;
  sol_ctrl* d_ctrl;
  sol_ctrl* h_ctrl;            // pinned mirror
  double* h_stage;             // pinned staging (max(6N, 3N) doubles)
  int state_valid;
  int last_eval_valid;
  int device_loop;         // RKF78 / DP attempts looped on the device (CUDA graph)
  DriverGraph graphs[2];   // [0] RKF78, [1] DP
  long long graph_steps;   // driver calls run as graphs since the last sol_driver
  int graph_used;
  sol_adjoint_state* adj;  // checkpoints and buffers of the discrete adjoint
  double* d_persist;       // source tables, block maxima and barrier words of the persistent driver
  void* d_sim;             // the step loop's line, stop reason and event flags (sol_run_until)
  double* d_ystart;        // the state at the start of the last step of sol_run_until (collision records)
  int32_t* h_id;           // BodyData::id on the host (output records carry ids)
  // failure-path test hooks (sol_set_wait_test): the group barrier's spin
  // limit (0: SOL_SPIN_LIMIT) and a CTA that skips its arrivals (-1: none)
  unsigned test_spin;
  int test_skip_cta;
};

// ---- launch helpers (defined in sol_force.cu / sol_integrate.cu) --------------
int sol_force_launch(sol_ctx* c, const double* d_y, double* d_dydt, TimeSpec ts, uint32_t flags);
int sol_force_launch_parts(sol_ctx* c, const double* d_y, double* d_dydt, TimeSpec ts, uint32_t flags, int parts);
int sol_integrator_run(sol_ctx* c, int integrator, int n_steps);
int sol_rkf78_single_attempt(sol_ctx* c, double t, double h, const double* d_y0, double* d_y, double* d_err,
                             double* error_max);
int sol_events_launch(sol_ctx* c, const double* d_y0, double ej, double hc, double cf, sol_event* d_out,
                      int capacity, int* d_count);
int sol_integrals_launch(sol_ctx* c, const double* d_y0, double* d_out16);
int sol_bench_stage_kernels(sol_ctx* c, int reps, double* ms_per_attempt);
// RKF78 stage sums in the reference's term order (RungeKuttaFehlberg78.cpp:169-232):
// stage r = y0 + h * sum_q a[r][q] f[idx[r][q]], q < k[r]
struct Rkf78Table {
  int k[13];
  int idx[13][9];
  double a[13][9];
};
const Rkf78Table& sol_rkf78_table();
int sol_persist_eligible(const sol_ctx* c);
int sol_persist_rkf78(sol_ctx* c, int n_steps);
int sol_group_eligible(const sol_ctx* c);
// The Simulator's step loop inside the group driver (sol_run_until): event
// thresholds (0: off), and device memory for the line, the stop reason and
// double-buffered per-CTA event flags.
struct GroupSim {
  double e3, h3, cf;
  sol_sim_line* line;
  int* reason;
  int* ev;        // [2 * kGroupMaxCtas]
  double* yprev;  // when not null: the state at the start of the step that stops with an event
};
constexpr int kGroupMaxCtas = 2048;
int sol_group_rkf78(sol_ctx* c, int n_steps, const GroupSim* sim = nullptr, int rk4 = 0);
int sol_fp64_peak_launch(int device, double* flops);
void sol_noalloc_wait_test(unsigned spin_limit, int withhold_tile);
int sol_fp64_rates_launch(int device, double rates[3], double* sm_mhz);
int sol_fp32_rates_launch(int device, double rates[2], double* sm_mhz);
int sol_check_pair_math_launch(int device, int mode, long long n, unsigned long long seed, long long* result);

// ---- PTX helpers: bulk copies (TMA engine) with mbarrier completion --------
__device__ __forceinline__ uint32_t sol_smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void sol_mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(sol_smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void sol_fence_barrier_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void sol_fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void sol_mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(sol_smem_u32(bar)), "r"(bytes)
               : "memory");
}
// 1-D bulk copy global -> shared; src, dst 16-byte aligned, bytes % 16 == 0.
__device__ __forceinline__ void sol_bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          sol_smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(sol_smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ uint32_t sol_mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(sol_smem_u32(bar)), "r"(parity)
      : "memory");
  return ok;
}
// Bounded wait: returns false (and the caller records SOL_DEV_TIMEOUT) when
// the phase did not complete within SOL_SPIN_LIMIT polls.
__device__ __forceinline__ bool sol_mbar_wait(uint64_t* bar, uint32_t parity) {
  for (uint32_t k = 0; k < SOL_SPIN_LIMIT; ++k)
    if (sol_mbar_try_wait(bar, parity)) return true;
  return false;
}
// The same with a caller-given limit (failure-path tests lower it); every
// poll suspends the thread for at most ~1 us (suspendTimeHint, ns), so the
// limit also bounds the wait's duration: 2^26 polls ~ 1 min at most, 4,096
// polls ~ 4 ms.
__device__ __forceinline__ uint32_t sol_mbar_try_wait_1us(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, 1000;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(sol_smem_u32(bar)), "r"(parity)
      : "memory");
  return ok;
}
__device__ __forceinline__ bool sol_mbar_wait_n(uint64_t* bar, uint32_t parity, uint32_t limit) {
  for (uint32_t k = 0; k < limit; ++k)
    if (sol_mbar_try_wait_1us(bar, parity)) return true;
  return false;
}

// ---- step-size control powers ------------------------------------------------
// pow(em, -e) for the RKF78 control's pow(errorMax, PGROW = -0.2) and
// pow(errorMax, PSHRNK = -0.25) (RungeKuttaFehlberg78.cpp:61-62, :113, :129),
// with e the double nearest 1/N, correctly rounded, as the reference's libm
// pow is but for ~8e-4 of its calls (measured for e = 0.2: it lands on the
// other neighbour of values within ~4e-4 ulp of a midpoint); a step's h
// differing in the last bit moves the next error estimate far more, through
// its cancellation.  The double 0.2
// exceeds 1/5 by 1/90071992547409920: em^-e = em^(-1/5) (1 - delta ln em),
// a shift of up to ~0.4 ulp that the final correction carries; ln em comes
// from FP32 (error ~1e-6), which leaves results within ~1e-7 ulp of a
// midpoint undecided (measured: 5e-8 of samples round the other way,
// a band 4,000 times narrower than libm's).  For N = 4 the result is
// correctly rounded but within ~2^-100 of a midpoint.  A library pow is a chain of ~5,800 cycles on the GPU, on
// the critical path of every attempt of the latency-bound drivers.  Here:
// an FP32 seed exp2(-log2(em)/N) (relative error < 2^-17 for |log2 em| <=
// 100), two Newton steps for em y^N = 1, y <- y + (y/N)(1 - em y^N)
// (2^-17 -> 2^-33 -> 2^-64 plus rounding), then the residual 1 - em y^N in
// double-double (TwoProduct by FMA; 1 - q is exact by Sterbenz) and one
// correction y + y t / N added with a single rounding.  Outside
// 2^-100 < em < 2^100 the library pow is taken.
template <int N>
__device__ __forceinline__ double sol_inv_root(double em) {
  const unsigned hi = (unsigned)__double2hiint(em);
  const int e = (int)(hi >> 20) - 1023;  // em > 0
  if (e <= -100 || e >= 100) return pow(em, -1.0 / N);
  const float ef = __uint_as_float(((unsigned)(e + 127) << 23) | ((hi & 0xFFFFFu) << 3));
  const float ys = exp2f(-__log2f(ef) * (1.0f / N));
  const unsigned yb = __float_as_uint(ys);
  double y = __hiloint2double((int)((((yb >> 23) - 127 + 1023) << 20) | ((yb & 0x7FFFFFu) >> 3)), (int)(yb << 29));
#pragma unroll
  for (int it = 0; it < 2; ++it) {
    const double y2 = y * y;
    const double yn = (N == 4) ? y2 * y2 : (y2 * y2) * y;
    const double t = __fma_rn(-em, yn, 1.0);
    y = __fma_rn(y * (1.0 / N), t, y);
  }
  // y^N as p + pe (double-double), then em y^N as q + qe
  const double p2 = y * y;
  const double e2 = __fma_rn(y, y, -p2);
  const double p4 = p2 * p2;
  const double e4 = __fma_rn(p2, p2, -p4) + 2.0 * p2 * e2;
  double p = p4, pe = e4;
  if (N == 5) {
    p = p4 * y;
    pe = __fma_rn(p4, y, -p) + e4 * y;
  }
  const double q = em * p;
  const double qe = __fma_rn(em, p, -q) + em * pe;
  const double t = (1.0 - q) - qe;
  // the exponent's own rounding: RN(1/N) - 1/N (0 for N = 4)
  constexpr double kDelta = (N == 5) ? 1.0 / 90071992547409920.0 : 0.0;
  const double corr = (N == 5) ? t * (1.0 / N) - kDelta * (double)__logf(ef) : t * (1.0 / N);
  return y + y * corr;
}

// pow(x, 1.0 / N) for N = 7 (DormandPrince's step control,
// DormandPrince.cpp:156) and N = 3 (the radius after a merge), correctly
// rounded: the library pow (within a few ulp) is stepped to the neighbour
// where x' - t^N changes sign between the midpoints around it,
// x' = x^(N e) = x (1 + N delta ln x), e the double nearest 1/N and
// delta = e - 1/N (-1/54043195528445952 for N = 3, -1/126100789566373888 for
// N = 7), everything in double-double.  One thread evaluates it per attempt
// or per merge: latency is no concern.
__device__ __forceinline__ int root_power_sign(double xh, double xl, double th, double tl, int n) {
  double ph = th, pl = tl;
  for (int k = 1; k < n; ++k) {
    const double h = ph * th;
    const double l = __fma_rn(ph, th, -h) + (ph * tl + pl * th);
    ph = h + l;
    pl = l - (ph - h);
  }
  const double d = (ph - xh) + (pl - xl);  // ph - xh is exact: t^N and x agree to a few ulp
  return (d > 0.0) - (d < 0.0);
}

template <int N>
__device__ __noinline__ double sol_pow_recip_cr(double x) {
  static_assert(N == 3 || N == 7, "exponent offsets are tabulated for 1/3 and 1/7");
  constexpr double kDelta = N == 3 ? -1.0 / 54043195528445952.0 : -1.0 / 126100789566373888.0;
  double y = pow(x, 1.0 / N);
  if (!(x > 0.0) || !(y > 0.0) || !(y < 1.0e300)) return y;
  const double xl = x * (N * kDelta) * log(x);
  for (int it = 0; it < 4; ++it) {
    const long long yb = __double_as_longlong(y);
    const double up = 0.5 * (__longlong_as_double(yb + 1) - y);
    const double dn = 0.5 * (y - __longlong_as_double(yb - 1));
    if (root_power_sign(x, xl, y, -dn, N) > 0)
      y = __longlong_as_double(yb - 1);  // the root lies below the lower midpoint
    else if (root_power_sign(x, xl, y, up, N) < 0)
      y = __longlong_as_double(yb + 1);
    else
      break;
  }
  return y;
}

// ---- gas-model device functions (restated from Solaris/GasComponent.cpp) ----
__device__ __forceinline__ double sol_pl(double c, double idx, double x) { return c * pow(x, idx); }

__device__ __forceinline__ double sol_reduction_factor(const GasDev& g, double t) {  // :36-61
  switch (g.decrease_type) {
    case SOL_GAS_CONSTANT: return 1.0;
    case SOL_GAS_LINEAR:
      if (t <= g.t0) return 1.0;
      if (t > g.t0 && t <= g.t1) return 1.0 - (t - g.t0) / (g.t1 - g.t0);
      return 0.0;
    case SOL_GAS_EXPONENTIAL: return exp(-t / g.time_scale);
    default: return 1.0;
  }
}

// Acceleration::GasDragAC body for one planetesimal (Acceleration.cpp:342-401)
__device__ __forceinline__ void sol_gas_drag(const GasDev& g, double factor, double m0, const double* yi,
                                             double radius, double density, double cd, double gs, double ge,
                                             double out[3]) {
  double x = yi[0], y = yi[1], z = yi[2];
  double r = sqrt(x * x + y * y + z * z);
  // gas_velocity -> circular_velocity (GasComponent.cpp:97-138)
  double vgx = 0.0, vgy = 0.0;
  {
    double mu = SOL_GAUSS2 * m0;
    double rc = sqrt(x * x + y * y);
    double vc = sqrt(mu / rc);
    if (x == 0.0 && y == 0.0) {
    } else if (y == 0.0) {
      vgy = x > 0.0 ? vc : -vc;
    } else if (x == 0.0) {
      vgx = y > 0.0 ? -vc : vc;
    } else if (x >= y) {
      double p = y / x;
      vgy = x >= 0 ? vc / sqrt(1.0 + p * p) : -vc / sqrt(1.0 + p * p);
      vgx = -vgy * p;
    } else {
      double p = x / y;
      vgx = y >= 0 ? -vc / sqrt(1.0 + p * p) : vc / sqrt(1.0 + p * p);
      vgy = -vgx * p;
    }
    double v = sqrt(1.0 - 2.0 * sol_pl(g.eta_c, g.eta_i, rc));
    vgx *= v;
    vgy *= v;
  }
  double ux = yi[3] - vgx, uy = yi[4] - vgy, uz = yi[5] - 0.0;
  // gas_density_at (GasComponent.cpp:141-157)
  double rho;
  {
    double rc = sqrt(x * x + y * y);
    double hh = sol_pl(g.sh_c, g.sh_i, rc);
    double q = z / hh;
    double arg = q * q;
    if (g.inner_edge < rc) {
      rho = sol_pl(g.rho_c, g.rho_i, rc) * exp(-arg);
    } else {
      double a = g.rho_c * pow(g.inner_edge, g.rho_i - 4.0);
      double r2c = rc * rc;
      rho = a * (r2c * r2c) * exp(-arg);
    }
  }
  double rhoGas = factor * rho;
  double lambda = sol_pl(g.mfp_c, g.mfp_i, r);
  double C;
  if (radius <= 0.1 * lambda) {
    // MeanThermalSpeed_CMU(m0, r) -> Temperature_CMU(r, m0) (arguments swapped, :241)
    double cT = g.sh_c * g.sh_c * r * g.mmw * g.ctp;
    double vth = g.cvth * sqrt(cT * pow(m0, g.pt));
    C = ge * vth * rhoGas;
  } else if (radius >= 10.0 * lambda) {
    double ul = sqrt(ux * ux + uy * uy + uz * uz);
    C = gs * ul * rhoGas;
  } else {
    double l1 = 0.1 * lambda, l2 = 10.0 * lambda;
    double gE = 1.0 / (density * l1);
    double gS = 3.0 / 8.0 * cd / (density * l2);
    double cT = g.sh_c * g.sh_c * r * g.mmw * g.ctp;
    double vth = g.cvth * sqrt(cT * pow(m0, g.pt));
    double ul = sqrt(ux * ux + uy * uy + uz * uz);
    double K = gS * ul / (gE * vth);
    double eta = l2 / l1;
    double kappa = log10(K) / log10(eta);
    double gamma = gE * vth * pow(l1, -kappa);
    C = gamma * pow(radius, kappa) * rhoGas;
  }
  out[0] = -C * ux;
  out[1] = -C * uy;
  out[2] = -C * uz;
}

// Ephemeris::CalculateOrbitalElement(mu, phase, &a, &e) (Ephemeris.cpp:10-41)
__device__ __forceinline__ void sol_orbital_a_e(double mu, const double* p, int quirks, double* a, double* e) {
  double v2 = p[3] * p[3] + p[4] * p[4] + p[5] * p[5];
  double rl = sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
  double h = v2 / 2.0 + (-mu / rl);
  *a = 0.0;
  *e = 0.0;
  if (h >= 0.0) return;  // the status is ignored by the callers (Acceleration.cpp:452)
  double cx = p[1] * p[5] - p[2] * p[4];
  double cy = p[2] * p[3] - p[0] * p[5];
  double cz = p[0] * p[4] - p[1] * p[3];
  double c2 = cx * cx + cy * cy + cz * cz;
  double e2 = 1.0 + 2.0 * c2 * h / (mu * mu);
  double ae2 = (quirks & SOL_QUIRK_INT_ABS) ? (double)abs((int)e2) : fabs(e2);
  if (ae2 < 1.0e-14) e2 = 0.0;
  *e = sqrt(e2);
  *a = -mu / (2.0 * h);
}

// Acceleration::TypeIMigrationTime (Acceleration.cpp:766-777)
__device__ __forceinline__ double sol_type1_migration_time(const GasDev& g, double C, double O, double ar, double er,
                                                           double h) {
  double Cm = 2.0 / (2.7 + 1.1 * g.abs_rho_index) / O;
  double er1 = er / (1.3 * h);
  double er2 = er / (1.1 * h);
  double frac = (1.0 + er1 * er1 * er1 * er1 * er1) / (1.0 - er2 * er2 * er2 * er2);
  return Cm * C * (ar * ar) * frac;
}

// Acceleration::TypeIEccentricityDampingTime (Acceleration.cpp:779-789)
__device__ __forceinline__ double sol_type1_ecc_damping_time(double C, double O, double ar, double er, double h) {
  double Ce = 0.1 / (0.78 * O);
  double q = er / h;
  double fr = 1.0 + 0.25 * (q * q * q);
  return Ce * C * (ar * ar * ar * ar) * fr;
}

// Acceleration::TauNu (Acceleration.cpp:831-849)
__device__ __forceinline__ double sol_tau_nu(const GasDev& g, double r, double O) {
  double h = sol_pl(g.sh_c, g.sh_i, r);
  if (g.tau_i == 2) {
    double q = r / h;
    return g.tau_c * (q * q) / (g.alpha * O);
  }
  return g.tau_c * pow(r / h, g.tau_i) / (g.alpha * O);
}

// MigrationTypeIAC body (Acceleration.cpp:435-481); returns false when the body
// stops migrating (r <= migStopAt), which the caller records.
__device__ __forceinline__ bool sol_migration_type1(const GasDev& g, double factor, double m0, double m,
                                                    double stop_at, const double* yi, double out[3]) {
  double r2 = yi[0] * yi[0] + yi[1] * yi[1] + yi[2] * yi[2];
  double r = sqrt(r2);
  if (r <= stop_at) {
    out[0] = out[1] = out[2] = 0.0;
    return false;
  }
  double a, e;
  sol_orbital_a_e(SOL_GAUSS2 * (m0 + m), yi, g.quirks, &a, &e);
  double O = SOL_GAUSS * sqrt((m0 + m) / (a * a * a));
  double md = sol_pl(g.rho_c, g.rho_i, r) * sol_pl(g.sh_c, g.sh_i, r) * SOL_SQRT_TWO_PI;
  double C = (m0 * m0) / (m * md * a * a);
  double h = sol_pl(g.sh_c, g.sh_i, r);
  double ar = h / r;
  double er = e * r;
  double tm = 0.0;
  if (e < 1.1 * h / r) {
    tm = sol_type1_migration_time(g, C, O, ar, er, h);
    tm = 1.0 / tm;
  }
  double te = sol_type1_ecc_damping_time(C, O, ar, er, h);
  double ti = te;
  double vr = yi[0] * yi[3] + yi[1] * yi[4] + yi[2] * yi[5];
  te = 2.0 * vr / (r2 * te);
  ti = 2.0 / ti;
  out[0] = -factor * (tm * yi[3] + te * yi[0]);
  out[1] = -factor * (tm * yi[4] + te * yi[1]);
  out[2] = -factor * (tm * yi[5] + te * yi[2] + ti * yi[5]);
  return true;
}

// MigrationTypeIIAC body (Acceleration.cpp:498-524; barycentric :727-760)
__device__ __forceinline__ bool sol_migration_type2(const GasDev& g, double factor, double m0, double m,
                                                    double stop_at, const double* yi, double out[3]) {
  double r2 = yi[0] * yi[0] + yi[1] * yi[1] + yi[2] * yi[2];
  double r = sqrt(r2);
  if (r <= stop_at) {
    out[0] = out[1] = out[2] = 0.0;
    return false;
  }
  double a, e;
  sol_orbital_a_e(SOL_GAUSS2 * (m0 + m), yi, g.quirks, &a, &e);
  double O = SOL_GAUSS * sqrt((m0 + m) / (a * a * a));
  double tau = sol_tau_nu(g, r, O);
  double c0 = (g.barycentric && (g.quirks & SOL_QUIRK_BC_TAU_NU)) ? tau : 1.0 / tau;
  double vr = yi[3] * yi[0] + yi[4] * yi[1] + yi[5] * yi[2];
  double c1 = vr / r2;
  out[0] = -factor * (c0 * (0.5 * yi[3] + 50 * (c1 * yi[0])));
  out[1] = -factor * (c0 * (0.5 * yi[4] + 50 * (c1 * yi[1])));
  out[2] = -factor * (c0 * (0.5 * yi[5] + 50 * (c1 * yi[2]) + yi[5]));
  return true;
}

// ---- epilogue: drag and migration of one sink (ComputeAstroCentric :176-243) --
__device__ __forceinline__ void add_gas_terms(const ForceCtx& fc, int i, const double* yi, double t,
                                              uint32_t flags, double a[3]) {
  const GasDev& g = fc.gas;
  if (!g.present) return;
  const Classes& c = fc.cls;
  const double m0 = fc.mass[0];
  const int lower_drag = c.nm, upper_drag = c.nm + c.n_spl + c.n_pl;
  if (i >= lower_drag && i < upper_drag) {
    double* buf = fc.drag + 3 * (i - lower_drag);
    if (flags & SOL_EVAL_GAS_DRAG) {
      double d[3];
      sol_gas_drag(g, sol_reduction_factor(g, t), m0, yi, fc.radius[i], fc.density[i], fc.cd[i],
                   fc.gamma_stokes[i], fc.gamma_epstein[i], d);
      buf[0] = d[0];
      buf[1] = d[1];
      buf[2] = d[2];
    }
    a[0] += buf[0];
    a[1] += buf[1];
    a[2] += buf[2];
    return;
  }
  const int lower1 = c.n_central + c.n_giant;
  if (fc.has_mig1 && i >= lower1 && i < c.nm) {
    double* buf = fc.mig1 + 3 * (i - lower1);
    if ((flags & SOL_EVAL_TYPE_I) && fc.mig_type[i] == SOL_MIGRATION_TYPE_I) {
      double d[3];
      if (!sol_migration_type1(g, sol_reduction_factor(g, t), m0, fc.mass[i], fc.mig_stop_at[i], yi, d))
        fc.mig_type[i] = SOL_MIGRATION_NO;
      buf[0] = d[0];
      buf[1] = d[1];
      buf[2] = d[2];
    }
    if (fc.mig_type[i] != SOL_MIGRATION_NO) {
      a[0] += buf[0];
      a[1] += buf[1];
      a[2] += buf[2];
    }
    return;
  }
  const int lower2 = c.n_central;
  if (fc.has_mig2 && i >= lower2 && i < c.n_central + c.n_giant) {
    double* buf = fc.mig2 + 3 * (i - lower2);
    if ((flags & SOL_EVAL_TYPE_II) && fc.mig_type[i] == SOL_MIGRATION_TYPE_II) {
      double d[3];
      if (!sol_migration_type2(g, sol_reduction_factor(g, t), m0, fc.mass[i], fc.mig_stop_at[i], yi, d))
        fc.mig_type[i] = SOL_MIGRATION_NO;
      buf[0] = d[0];
      buf[1] = d[1];
      buf[2] = d[2];
    }
    if (fc.mig_type[i] != SOL_MIGRATION_NO) {
      a[0] += buf[0];
      a[1] += buf[1];
      a[2] += buf[2];
    }
  }
}
