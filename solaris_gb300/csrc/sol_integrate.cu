// Integrator drivers on the device: RungeKuttaFehlberg78, RungeKutta4 and
// DormandPrince (Solaris/RungeKuttaFehlberg78.cpp, RungeKutta4.cpp,
// DormandPrince.cpp).
//
// Stage combinations, the final sums and the error estimates are streaming
// kernels over the 6N state (read k vectors, write one) in the reference's
// operation order, so that with the FP64 force they reproduce the reference
// bit for bit.  The error norm is reduced on the device and the step-size
// decision (accept / shrink / grow, underflow, retry limit) is taken by a
// one-thread control kernel that updates the device control block; the host
// only reads the control block to decide whether to launch another attempt.
#include <atomic>
#include <mutex>
#include <cmath>
#include <cstring>
#include <vector>

#include "sol_internal.cuh"

namespace {

constexpr int kBlock = 256;
constexpr int kMaxTerms = 9;

struct StageArgs {
  const double* f[kMaxTerms];
  double a[kMaxTerms];
};

inline int grid_for(int n) {
  int g = (n + kBlock - 1) / kBlock;
  return g < 1 ? 1 : (g > 152 * 16 ? 152 * 16 : g);
}

// yt = y0 + h * (a0 f0 + a1 f1 + ...), summed left to right
// (RungeKuttaFehlberg78.cpp:170-232, RungeKutta4.cpp:413-433).
template <int K>
__global__ void k_stage(int nv, const double* __restrict__ y0, double* __restrict__ out, StageArgs s,
                        const sol_ctrl* ctrl) {
  const double h = ctrl->h;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += gridDim.x * blockDim.x) {
    double acc = s.a[0] * s.f[0][i];
#pragma unroll
    for (int k = 1; k < K; ++k) acc = acc + s.a[k] * s.f[k][i];
    out[i] = y0[i] + h * acc;
  }
}

// yscale = |y0| + |h f0| + TINY (RungeKuttaFehlberg78.cpp:87-89)
__global__ void k_yscale(int nv, const double* __restrict__ y0, const double* __restrict__ f0,
                         double* __restrict__ ys, const sol_ctrl* ctrl) {
  const double h = ctrl->h;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += gridDim.x * blockDim.x)
    ys[i] = fabs(y0[i]) + fabs(h * f0[i]) + 1.0e-30;
}

struct Rkf78FinalArgs {
  const double* f[13];
};

// The 7th-order result, the error estimate and the block maxima of
// |error / yscale| (RungeKuttaFehlberg78.cpp:236-242, :252-262).
__global__ void k_rkf78_final(int nv, const double* __restrict__ y0, Rkf78FinalArgs fa, double* __restrict__ y,
                              double* __restrict__ err, const double* __restrict__ ys, double* __restrict__ partial,
                              const sol_ctrl* ctrl) {
  const double h = ctrl->h;
  const double D1_0 = 41.0 / 840.0, D1_5 = 34.0 / 105.0, D1_6 = 9.0 / 35.0, D1_8 = 9.0 / 280.0,
               D1_10 = 41.0 / 840.0;
  double m = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += gridDim.x * blockDim.x) {
    const double f0 = fa.f[0][i], f10 = fa.f[10][i];
    y[i] = y0[i] + h * (D1_0 * f0 + D1_5 * fa.f[5][i] + D1_6 * (fa.f[6][i] + fa.f[7][i]) +
                        D1_8 * (fa.f[8][i] + fa.f[9][i]) + D1_10 * f10);
    double e = h * fabs(f0 + f10 - fa.f[11][i] - fa.f[12][i]) * 41.0 / 840.0;
    err[i] = e;
    double q = fabs(e / ys[i]);
    m = q > m ? q : m;  // as GetErrorMax: a NaN entry never replaces the maximum
  }
  __shared__ double red[kBlock];
  red[threadIdx.x] = m;
  __syncthreads();
  for (int w = kBlock / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      double o = red[threadIdx.x + w];
      if (o > red[threadIdx.x]) red[threadIdx.x] = o;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

// The 7th-order result alone (RungeKuttaFehlberg78.cpp:236-238)
__global__ void k_rkf78_y(int nv, const double* __restrict__ y0, Rkf78FinalArgs fa, double* __restrict__ y,
                          const sol_ctrl* ctrl) {
  const double h = ctrl->h;
  const double D1_0 = 41.0 / 840.0, D1_5 = 34.0 / 105.0, D1_6 = 9.0 / 35.0, D1_8 = 9.0 / 280.0,
               D1_10 = 41.0 / 840.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += gridDim.x * blockDim.x)
    y[i] = y0[i] + h * (D1_0 * fa.f[0][i] + D1_5 * fa.f[5][i] + D1_6 * (fa.f[6][i] + fa.f[7][i]) +
                        D1_8 * (fa.f[8][i] + fa.f[9][i]) + D1_10 * fa.f[10][i]);
}

// max over block partials -> ctrl->error_max (divided by eps for RKF78)
__global__ void k_reduce_max(const double* __restrict__ partial, int np, sol_ctrl* ctrl, int divide_eps) {
  __shared__ double red[kBlock];
  double m = 0.0;
  for (int b = threadIdx.x; b < np; b += blockDim.x) {
    double o = partial[b];
    if (o > m) m = o;
  }
  red[threadIdx.x] = m;
  __syncthreads();
  for (int w = kBlock / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      double o = red[threadIdx.x + w];
      if (o > red[threadIdx.x]) red[threadIdx.x] = o;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) ctrl->error_max = divide_eps ? red[0] / ctrl->eps : red[0];
}

// Keep iterating the device-side attempt loop while no attempt has been
// accepted and no error has been raised.
__device__ __forceinline__ void set_loop_condition(const sol_ctrl* c, cudaGraphConditionalHandle h, int use) {
  if (use) cudaGraphSetConditional(h, (!c->accepted && c->dev_status == 0) ? 1u : 0u);
}

// Step-size control of RungeKuttaFehlberg78::Driver (:98-133).
__global__ void k_control_rkf78(sol_ctrl* c, cudaGraphConditionalHandle hcond, int use_cond) {
  const double em = c->error_max;
  const double h = c->h;
  if (em < 1.0) {
    c->h_did = h;
    c->t += c->h_did;
    c->h_next = em > 1.89e-4 ? (0.9 * h * sol_inv_root<5>(em)) : (5.0 * h);
    c->h = c->h_next;
    c->accepted = 1;
    c->n_accepted++;
  } else {
    c->n_rejected++;
    double hTemp = 0.9 * h * sol_inv_root<4>(em);
    double hn = fabs(hTemp) > fabs(0.1 * h) ? hTemp : 0.1 * h;
    c->h = hn;
    double tNew = c->t + hn;
    if (tNew == c->t) c->dev_status |= SOL_DEV_UNDERFLOW;
  }
  set_loop_condition(c, hcond, use_cond);
}

// RungeKutta4::Driver bookkeeping (RungeKutta4.cpp:355-365)
__global__ void k_control_rk4(sol_ctrl* c) {
  c->h_did = c->h;
  c->t += c->h_did;
  c->h_next = c->h;
  c->accepted = 1;
  c->n_accepted++;
}

// Begin a driver call: bodyData->h = timeLine->hNext (RungeKuttaFehlberg78.cpp:74-75).
// In a graph it also arms the attempt loop, which does not run once an
// earlier driver call has raised an error.
__global__ void k_begin_step(sol_ctrl* c, cudaGraphConditionalHandle hcond, int use_cond) {
  c->h = c->h_next;
  c->accepted = 0;
  c->iter = 0;
  set_loop_condition(c, hcond, use_cond);
}

// swap(y0, y) of an accepted driver call (RungeKuttaFehlberg78.cpp:132)
__global__ void k_accept_copy(int nv, double* __restrict__ y0, const double* __restrict__ y, const sol_ctrl* c) {
  if (!c->accepted) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += gridDim.x * blockDim.x) y0[i] = y[i];
}

// ---- Dormand-Prince RKN 7(6), DormandPrince::Step2 (:246-491) ---------------
struct DpStageArgs {
  const double* f[8];
  double a[8];
  double ck;  // c[k]
};

template <int K>
__global__ void k_dp_stage(int n, const double* __restrict__ y0, double* __restrict__ yt, DpStageArgs s,
                           const sol_ctrl* ctrl) {
  const double h = ctrl->h;
  const double h2 = h * h;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < 3 * n; q += gridDim.x * blockDim.x) {
    const int nn = 6 * (q / 3) + (q % 3);
    double var = s.a[0] * s.f[0][nn + 3];
#pragma unroll
    for (int l = 1; l < K; ++l) var = var + s.a[l] * s.f[l][nn + 3];
    yt[nn] = y0[nn] + s.ck * h * y0[nn + 3] + h2 * (var);
    yt[nn + 3] = y0[nn + 3] + h * (var);
  }
}

struct DpFinalArgs {
  const double* f[9];
  double b[9], bdh[9];
};

__global__ void k_dp_final(int n, const double* __restrict__ y0, DpFinalArgs s, double* __restrict__ y,
                           double* __restrict__ err, double* __restrict__ partial, const sol_ctrl* ctrl) {
  const double h = ctrl->h;
  const double h2 = h * h;
  double m = 0.0;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < 3 * n; q += gridDim.x * blockDim.x) {
    const int nn = 6 * (q / 3) + (q % 3);
    const double f0 = s.f[0][nn + 3], f4 = s.f[4][nn + 3], f5 = s.f[5][nn + 3], f6 = s.f[6][nn + 3],
                 f7 = s.f[7][nn + 3], f8 = s.f[8][nn + 3];
    y[nn] = y0[nn] + h * y0[nn + 3] +
            h2 * (s.b[0] * f0 + s.b[4] * f4 + s.b[5] * f5 + s.b[6] * f6 + s.b[7] * f7 + s.b[8] * f8);
    double e = h2 * fabs(f7 - f8) / 20.0;
    err[nn] = e;
    y[nn + 3] = y0[nn + 3] + h * (s.bdh[0] * f0 + s.bdh[4] * f4 + s.bdh[5] * f5 + s.bdh[6] * f6 + s.bdh[7] * f7);
    err[nn + 3] = 0.0;
    double q2 = fabs(e);
    m = q2 > m ? q2 : m;
  }
  __shared__ double red[kBlock];
  red[threadIdx.x] = m;
  __syncthreads();
  for (int w = kBlock / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      double o = red[threadIdx.x + w];
      if (o > red[threadIdx.x]) red[threadIdx.x] = o;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

// DormandPrince::Driver loop condition and step update (:145-164)
__global__ void k_control_dp(sol_ctrl* c, cudaGraphConditionalHandle hcond, int use_cond) {
  const double em = c->error_max;
  const double h = c->h;
  c->iter++;
  c->h_did = h;
  c->h_next = em < 1.0e-20 ? 2.0 * h : 0.9 * h * sol_pow_recip_cr<7>(c->eps / em);
  if (em > c->eps && c->iter <= 10) {
    c->n_rejected++;
    c->h = c->h_next;  // the next attempt uses timeLine->hNext
  } else if (c->iter > 10) {
    c->dev_status |= SOL_DEV_MAXITER;
  } else {
    c->t += c->h_did;
    c->accepted = 1;
    c->n_accepted++;
  }
  set_loop_condition(c, hcond, use_cond);
}

// RKF78 stage tableau (RungeKuttaFehlberg78.cpp:41-56): per stage, the k
// indices it reads and the coefficients, in the order of the reference sums.
struct Rkf78Stage {
  int k;
  int idx[kMaxTerms];
  double a[kMaxTerms];
};

const Rkf78Stage* rkf78_stages() {
  static Rkf78Stage st[13];
  // filled once; contexts of several host threads may arrive together
  static std::atomic<bool> init{false};
  static std::mutex init_mutex;
  std::unique_lock<std::mutex> init_lock(init_mutex, std::defer_lock);
  if (!init.load(std::memory_order_acquire) && (init_lock.lock(), !init.load(std::memory_order_relaxed))) {
    auto set = [](Rkf78Stage& s, std::initializer_list<int> idx, std::initializer_list<double> a) {
      s.k = (int)idx.size();
      int p = 0;
      for (int v : idx) s.idx[p++] = v;
      p = 0;
      for (double v : a) s.a[p++] = v;
    };
    set(st[1], {0}, {2.0 / 27.0});
    set(st[2], {0, 1}, {1.0 / 36.0, 1.0 / 12.0});
    set(st[3], {0, 2}, {1.0 / 24.0, 1.0 / 8.0});
    set(st[4], {0, 2, 3}, {5.0 / 12.0, -25.0 / 16.0, 25.0 / 16.0});
    set(st[5], {0, 3, 4}, {1.0 / 20.0, 1.0 / 4.0, 1.0 / 5.0});
    set(st[6], {0, 3, 4, 5}, {-25.0 / 108.0, 125.0 / 108.0, -65.0 / 27.0, 125.0 / 54.0});
    set(st[7], {0, 4, 5, 6}, {31.0 / 300.0, 61.0 / 225.0, -2.0 / 9.0, 13.0 / 900.0});
    set(st[8], {0, 3, 4, 5, 6, 7}, {2.0, -53.0 / 6.0, 704.0 / 45.0, -107.0 / 9.0, 67.0 / 90.0, 3.0});
    set(st[9], {0, 3, 4, 5, 6, 7, 8},
        {-91.0 / 108.0, 23.0 / 108.0, -976.0 / 135.0, 311.0 / 54.0, -19.0 / 60.0, 17.0 / 6.0, -1.0 / 12.0});
    set(st[10], {0, 3, 4, 5, 6, 7, 8, 9},
        {2383.0 / 4100.0, -341.0 / 164.0, 4496.0 / 1025.0, -301.0 / 82.0, 2133.0 / 4100.0, 45.0 / 82.0,
         45.0 / 164.0, 18.0 / 41.0});
    set(st[11], {0, 5, 6, 7, 8, 9}, {3.0 / 205.0, -6.0 / 41.0, -3.0 / 205.0, -3.0 / 41.0, 3.0 / 41.0, 6.0 / 41.0});
    set(st[12], {0, 3, 4, 5, 6, 7, 8, 9, 11},
        {-1777.0 / 4100.0, -341.0 / 164.0, 4496.0 / 1025.0, -289.0 / 82.0, 2193.0 / 4100.0, 51.0 / 82.0,
         33.0 / 164.0, 12.0 / 41.0, 1.0});
    init.store(true, std::memory_order_release);
  }
  return st;
}

int launch_stage(sol_ctx* c, int k, const StageArgs& s, const double* y0, double* out) {
  const int g = grid_for(c->nv);
  switch (k) {
    case 1: k_stage<1><<<g, kBlock, 0, c->stream>>>(c->nv, y0, out, s, c->d_ctrl); break;
    case 2: k_stage<2><<<g, kBlock, 0, c->stream>>>(c->nv, y0, out, s, c->d_ctrl); break;
    case 3: k_stage<3><<<g, kBlock, 0, c->stream>>>(c->nv, y0, out, s, c->d_ctrl); break;
    case 4: k_stage<4><<<g, kBlock, 0, c->stream>>>(c->nv, y0, out, s, c->d_ctrl); break;
    case 6: k_stage<6><<<g, kBlock, 0, c->stream>>>(c->nv, y0, out, s, c->d_ctrl); break;
    case 7: k_stage<7><<<g, kBlock, 0, c->stream>>>(c->nv, y0, out, s, c->d_ctrl); break;
    case 8: k_stage<8><<<g, kBlock, 0, c->stream>>>(c->nv, y0, out, s, c->d_ctrl); break;
    case 9: k_stage<9><<<g, kBlock, 0, c->stream>>>(c->nv, y0, out, s, c->d_ctrl); break;
    default: sol_set_error("stage with %d terms", k); return SOL_ERR_ARG;
  }
  SOL_LAUNCHED();
  return SOL_OK;
}

#define RET(x)              \
  do {                      \
    int r_ = (x);           \
    if (r_ != SOL_OK) return r_; \
  } while (0)

// Force at stage s of the current attempt: time = ctrl->t + c * ctrl->h.
inline TimeSpec stage_time(sol_ctx* c, double coef) {
  TimeSpec ts;
  ts.base = &c->d_ctrl->t;
  ts.h = &c->d_ctrl->h;
  ts.c = coef;
  ts.t_host = 0.0;
  return ts;
}

// One RKF78 attempt (RungeKuttaFehlberg78::Step, :147-250): 12 stages, the
// final sum, the error estimate and its norm.  The time of every stage is the
// step's start time (:168, :173-234).
// fl: the evaluate flags of the stage evaluations; the Driver leaves only the
// gas drag on (migration only at its first evaluation, :94-95).
int rkf78_attempt(sol_ctx* c, const double* y0, double* y, double* err, uint32_t fl = SOL_EVAL_GAS_DRAG) {
  const Rkf78Stage* st = rkf78_stages();
  double* fk[13];
  fk[0] = c->d_accel;
  for (int k = 1; k < 13; ++k) fk[k] = c->d_fk[k];
  for (int r = 1; r <= 12; ++r) {
    StageArgs s;
    memset(&s, 0, sizeof(s));
    for (int k = 0; k < st[r].k; ++k) {
      s.f[k] = fk[st[r].idx[k]];
      s.a[k] = st[r].a[k];
    }
    RET(launch_stage(c, st[r].k, s, y0, c->d_ytmp));
    RET(sol_force_launch(c, c->d_ytmp, fk[r], stage_time(c, 0.0), fl));
  }
  Rkf78FinalArgs fa;
  for (int k = 0; k < 13; ++k) fa.f[k] = fk[k];
  const int g = grid_for(c->nv);
  k_rkf78_final<<<g, kBlock, 0, c->stream>>>(c->nv, y0, fa, y, err, c->d_yscale, c->d_partial, c->d_ctrl);
  SOL_LAUNCHED();
  k_reduce_max<<<1, kBlock, 0, c->stream>>>(c->d_partial, g, c->d_ctrl, 1);
  SOL_LAUNCHED();
  return SOL_OK;
}

int read_ctrl(sol_ctx* c) {
  SOL_CUDA(cudaMemcpyAsync(c->h_ctrl, c->d_ctrl, sizeof(sol_ctrl), cudaMemcpyDeviceToHost, c->stream));
  SOL_CUDA(cudaStreamSynchronize(c->stream));
  return SOL_OK;
}

int ctrl_status(sol_ctx* c) {
  int ds = c->h_ctrl->dev_status;
  if (ds & SOL_DEV_TIMEOUT) {
    sol_set_error("a bounded device wait ran out");
    return SOL_ERR_TIMEOUT;
  }
  if (ds & SOL_DEV_UNDERFLOW) {
    sol_set_error("Stepsize-underflow occurred during Runge-Kutta-Fehlberg7(8) step!");
    return SOL_ERR_UNDERFLOW;
  }
  if (ds & SOL_DEV_MAXITER) {
    sol_set_error("An error occurred during Prince-Dormand driver: iteration number exceeded maxIter!");
    return SOL_ERR_MAXITER;
  }
  return SOL_OK;
}

int rkf78_driver_step(sol_ctx* c) {
  k_begin_step<<<1, 1, 0, c->stream>>>(c->d_ctrl, 0, 0);
  SOL_LAUNCHED();
  // Driver: all evaluate flags on for the first evaluation (:77-82)
  RET(sol_force_launch(c, c->d_y0, c->d_accel, stage_time(c, 0.0), SOL_EVAL_ALL));
  const int g = grid_for(c->nv);
  k_yscale<<<g, kBlock, 0, c->stream>>>(c->nv, c->d_y0, c->d_accel, c->d_yscale, c->d_ctrl);
  SOL_LAUNCHED();
  for (int attempt = 0;; ++attempt) {
    RET(rkf78_attempt(c, c->d_y0, c->d_y, c->d_err));
    k_control_rkf78<<<1, 1, 0, c->stream>>>(c->d_ctrl, 0, 0);
    SOL_LAUNCHED();
    RET(read_ctrl(c));
    RET(ctrl_status(c));
    if (c->h_ctrl->accepted) break;
  }
  SOL_CUDA(cudaMemcpyAsync(c->d_y0, c->d_y, sizeof(double) * c->nv, cudaMemcpyDeviceToDevice, c->stream));
  return SOL_OK;
}

// RungeKutta4::Step (RungeKutta4.cpp:58-129): three stages from f0 = d_accel
// and the final sum into y.
int rk4_attempt(sol_ctx* c, const double* y0, double* y, uint32_t fl = SOL_EVAL_GAS_DRAG) {
  const double a21 = 1.0 / 2.0, a32 = 1.0 / 2.0, a43 = 1.0;
  const double b1 = 1.0 / 6.0, b2 = 1.0 / 3.0, b3 = 1.0 / 3.0, b4 = 1.0 / 6.0;
  const double c2 = 1.0 / 2.0, c3 = 1.0 / 2.0, c4 = 1.0;
  StageArgs s;
  memset(&s, 0, sizeof(s));
  s.f[0] = c->d_accel;
  s.a[0] = a21;
  RET(launch_stage(c, 1, s, y0, c->d_ytmp));
  RET(sol_force_launch(c, c->d_ytmp, c->d_fk[1], stage_time(c, c2), fl));
  s.f[0] = c->d_fk[1];
  s.a[0] = a32;
  RET(launch_stage(c, 1, s, y0, c->d_ytmp));
  RET(sol_force_launch(c, c->d_ytmp, c->d_fk[2], stage_time(c, c3), fl));
  s.f[0] = c->d_fk[2];
  s.a[0] = a43;
  RET(launch_stage(c, 1, s, y0, c->d_ytmp));
  RET(sol_force_launch(c, c->d_ytmp, c->d_fk[3], stage_time(c, c4), fl));
  StageArgs fs;
  memset(&fs, 0, sizeof(fs));
  fs.f[0] = c->d_accel;
  fs.f[1] = c->d_fk[1];
  fs.f[2] = c->d_fk[2];
  fs.f[3] = c->d_fk[3];
  fs.a[0] = b1;
  fs.a[1] = b2;
  fs.a[2] = b3;
  fs.a[3] = b4;
  return launch_stage(c, 4, fs, y0, y);
}

int rk4_driver_step(sol_ctx* c) {
  // RungeKutta4::Driver (RungeKutta4.cpp:20-57)
  k_begin_step<<<1, 1, 0, c->stream>>>(c->d_ctrl, 0, 0);
  SOL_LAUNCHED();
  RET(sol_force_launch(c, c->d_y0, c->d_accel, stage_time(c, 0.0), SOL_EVAL_ALL));
  RET(rk4_attempt(c, c->d_y0, c->d_y));
  k_control_rk4<<<1, 1, 0, c->stream>>>(c->d_ctrl);
  SOL_LAUNCHED();
  SOL_CUDA(cudaMemcpyAsync(c->d_y0, c->d_y, sizeof(double) * c->nv, cudaMemcpyDeviceToDevice, c->stream));
  return SOL_OK;
}

struct DpTab {
  double b[9], bdh[9], c[9], a[9][8];
};

const DpTab& dp_tab() {
  // DormandPrince::DormandPrince (DormandPrince.cpp:37-124)
  static DpTab T;
  // filled once; contexts of several host threads may arrive together
  static std::atomic<bool> init{false};
  static std::mutex init_mutex;
  std::unique_lock<std::mutex> init_lock(init_mutex, std::defer_lock);
  if (!init.load(std::memory_order_acquire) && (init_lock.lock(), !init.load(std::memory_order_relaxed))) {
    memset(&T, 0, sizeof(T));
    double sQ = sqrt(21.0);
    T.b[0] = 1.0 / 20.0; T.b[4] = 8.0 / 45.0; T.b[5] = 7.0 * (7.0 + sQ) / 360.0;
    T.b[6] = 7.0 * (7.0 - sQ) / 360.0; T.b[7] = -1.0 / 20.0; T.b[8] = 1.0 / 20.0;
    T.bdh[0] = 1.0 / 20.0; T.bdh[4] = 16.0 / 45.0; T.bdh[5] = 49.0 / 180.0; T.bdh[6] = 49.0 / 180.0;
    T.bdh[7] = 1.0 / 20.0;
    T.c[1] = 1.0 / 10.0; T.c[2] = 1.0 / 5.0; T.c[3] = 3.0 / 8.0; T.c[4] = 1.0 / 2.0;
    T.c[5] = (7.0 - sQ) / 14.0; T.c[6] = (7.0 + sQ) / 14.0; T.c[7] = 1.0; T.c[8] = 1.0;
    T.a[1][0] = 1.0 / 200.0;
    T.a[2][0] = 1.0 / 150.0; T.a[2][1] = 1.0 / 75.0;
    T.a[3][0] = 171.0 / 8192.0; T.a[3][1] = 45.0 / 4096.0; T.a[3][2] = 315.0 / 8192.0;
    T.a[4][0] = 5.0 / 288.0; T.a[4][1] = 25.0 / 528.0; T.a[4][2] = 25.0 / 672.0; T.a[4][3] = 16.0 / 693.0;
    T.a[5][0] = (1003.0 - 205.0 * sQ) / 12348.0; T.a[5][1] = -25.0 * (751.0 - 173.0 * sQ) / 90552.0;
    T.a[5][2] = 25.0 * (624.0 - 137.0 * sQ) / 43218.0; T.a[5][3] = -128.0 * (361.0 - 79.0 * sQ) / 237699.0;
    T.a[5][4] = (3411.0 - 745.0 * sQ) / 24696.0;
    T.a[6][0] = (793.0 + 187.0 * sQ) / 12348.0; T.a[6][1] = -25.0 * (331.0 + 113.0 * sQ) / 90552.0;
    T.a[6][2] = 25.0 * (1044.0 + 247.0 * sQ) / 43218.0;
    T.a[6][3] = -128.0 * (14885.0 + 3779.0 * sQ) / 9745659.0;
    T.a[6][4] = (3327.0 + 797.0 * sQ) / 24696.0; T.a[6][5] = -(581.0 + 127.0 * sQ) / 1722.0;
    T.a[7][0] = -(157.0 - 3.0 * sQ) / 378.0; T.a[7][1] = 25.0 * (143.0 - 10.0 * sQ) / 2772.0;
    T.a[7][2] = -25.0 * (876.0 + 55.0 * sQ) / 3969.0; T.a[7][3] = 1280.0 * (913.0 + 18.0 * sQ) / 596673.0;
    T.a[7][4] = -(1353.0 + 26.0 * sQ) / 2268.0; T.a[7][5] = 7.0 * (1777.0 + 377.0 * sQ) / 4428.0;
    T.a[7][6] = 7.0 * (5.0 - sQ) / 36.0;
    T.a[8][0] = 1.0 / 20.0; T.a[8][4] = 8.0 / 45.0; T.a[8][5] = 7.0 * (7.0 + sQ) / 360.0;
    T.a[8][6] = 7.0 * (7.0 - sQ) / 360.0;
    init.store(true, std::memory_order_release);
  }
  return T;
}

int launch_dp_stage(sol_ctx* c, int k, const DpStageArgs& s) {
  const int g = grid_for(3 * c->n);
  switch (k) {
    case 1: k_dp_stage<1><<<g, kBlock, 0, c->stream>>>(c->n, c->d_y0, c->d_ytmp, s, c->d_ctrl); break;
    case 2: k_dp_stage<2><<<g, kBlock, 0, c->stream>>>(c->n, c->d_y0, c->d_ytmp, s, c->d_ctrl); break;
    case 3: k_dp_stage<3><<<g, kBlock, 0, c->stream>>>(c->n, c->d_y0, c->d_ytmp, s, c->d_ctrl); break;
    case 4: k_dp_stage<4><<<g, kBlock, 0, c->stream>>>(c->n, c->d_y0, c->d_ytmp, s, c->d_ctrl); break;
    case 5: k_dp_stage<5><<<g, kBlock, 0, c->stream>>>(c->n, c->d_y0, c->d_ytmp, s, c->d_ctrl); break;
    case 6: k_dp_stage<6><<<g, kBlock, 0, c->stream>>>(c->n, c->d_y0, c->d_ytmp, s, c->d_ctrl); break;
    case 7: k_dp_stage<7><<<g, kBlock, 0, c->stream>>>(c->n, c->d_y0, c->d_ytmp, s, c->d_ctrl); break;
    default: sol_set_error("dp stage %d", k); return SOL_ERR_ARG;
  }
  SOL_LAUNCHED();
  return SOL_OK;
}

// One DormandPrince::Step2 attempt: 8 stages, the final sums, the error and its norm.
int dp_attempt(sol_ctx* c, uint32_t fl = SOL_EVAL_GAS_DRAG) {
  const DpTab& T = dp_tab();
  double* f[9];
  f[0] = c->d_accel;
  for (int k = 1; k < 9; ++k) f[k] = c->d_fk[k];
  {
    for (int k = 1; k < 9; ++k) {
      DpStageArgs s;
      memset(&s, 0, sizeof(s));
      int nt = 0;
      if (k == 8) {
        const int idx[4] = {0, 4, 5, 6};
        for (int q = 0; q < 4; ++q) {
          s.f[q] = f[idx[q]];
          s.a[q] = T.a[8][idx[q]];
        }
        nt = 4;
      } else {
        for (int l = 0; l < k; ++l) {
          s.f[l] = f[l];
          s.a[l] = T.a[k][l];
        }
        nt = k;
      }
      s.ck = T.c[k];
      RET(launch_dp_stage(c, nt, s));
      RET(sol_force_launch(c, c->d_ytmp, f[k], stage_time(c, T.c[k]), fl));
    }
    DpFinalArgs fa;
    for (int k = 0; k < 9; ++k) {
      fa.f[k] = f[k];
      fa.b[k] = T.b[k];
      fa.bdh[k] = T.bdh[k];
    }
    const int g = grid_for(3 * c->n);
    k_dp_final<<<g, kBlock, 0, c->stream>>>(c->n, c->d_y0, fa, c->d_y, c->d_err, c->d_partial, c->d_ctrl);
    SOL_LAUNCHED();
    k_reduce_max<<<1, kBlock, 0, c->stream>>>(c->d_partial, g, c->d_ctrl, 0);
    SOL_LAUNCHED();
  }
  return SOL_OK;
}

int dp_driver_step(sol_ctx* c) {
  k_begin_step<<<1, 1, 0, c->stream>>>(c->d_ctrl, 0, 0);
  SOL_LAUNCHED();
  RET(sol_force_launch(c, c->d_y0, c->d_accel, stage_time(c, 0.0), SOL_EVAL_ALL));
  for (;;) {
    RET(dp_attempt(c));
    k_control_dp<<<1, 1, 0, c->stream>>>(c->d_ctrl, 0, 0);
    SOL_LAUNCHED();
    RET(read_ctrl(c));
    RET(ctrl_status(c));
    if (c->h_ctrl->accepted) break;
  }
  SOL_CUDA(cudaMemcpyAsync(c->d_y0, c->d_y, sizeof(double) * c->nv, cudaMemcpyDeviceToDevice, c->stream));
  return SOL_OK;
}

// ---- device-side driver loop: one CUDA graph per driver call ------------------
// prologue (begin, first evaluation, yscale) -> WHILE (attempt, control) ->
// accept copy.  The control kernel sets the WHILE condition, so rejected
// attempts are retried on the device with no host round trip; the host only
// launches the graph once per driver call and reads the control block at the
// end of the whole sequence.
struct CaptureGuard {  // kernels captured into a graph are counted when the graph runs
  CaptureGuard() { sol_capture_begin(); }
  ~CaptureGuard() { sol_capture_end(); }
};

int capture_deps(cudaStream_t st, std::vector<cudaGraphNode_t>& out) {
  cudaStreamCaptureStatus cs;
  const cudaGraphNode_t* deps = nullptr;
  size_t nd = 0;
  SOL_CUDA(cudaStreamGetCaptureInfo(st, &cs, nullptr, nullptr, &deps, nullptr, &nd));
  out.assign(deps, deps + nd);
  return SOL_OK;
}

int build_driver_graph(sol_ctx* c, int integrator, DriverGraph& G) {
  CaptureGuard guard;
  const cudaStreamCaptureMode mode = cudaStreamCaptureModeThreadLocal;
  cudaGraph_t graph = nullptr;
  SOL_CUDA(cudaGraphCreate(&graph, 0));
  int rc = SOL_OK;
  cudaGraphConditionalHandle hcond;
  std::vector<cudaGraphNode_t> deps;
  cudaGraph_t tmp = nullptr;
  long long k0 = sol_capture_count();
  auto fail = [&](int r) {
    cudaStreamCaptureStatus cs;
    if (cudaStreamIsCapturing(c->stream, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone) {
      cudaGraph_t junk = nullptr;
      cudaStreamEndCapture(c->stream, &junk);
    }
    cudaGetLastError();
    cudaGraphDestroy(graph);
    return r;
  };
  if (cudaGraphConditionalHandleCreate(&hcond, graph, 0, 0) != cudaSuccess) return fail(SOL_ERR_CUDA);
  // prologue
  if (cudaStreamBeginCaptureToGraph(c->stream, graph, nullptr, nullptr, 0, mode) != cudaSuccess) return fail(SOL_ERR_CUDA);
  k_begin_step<<<1, 1, 0, c->stream>>>(c->d_ctrl, hcond, 1);
  sol_count_launch();
  if ((rc = sol_force_launch(c, c->d_y0, c->d_accel, stage_time(c, 0.0), SOL_EVAL_ALL))) return fail(rc);
  if (integrator == SOL_RUNGE_KUTTA_FEHLBERG78) {
    k_yscale<<<grid_for(c->nv), kBlock, 0, c->stream>>>(c->nv, c->d_y0, c->d_accel, c->d_yscale, c->d_ctrl);
    sol_count_launch();
  }
  if ((rc = capture_deps(c->stream, deps))) return fail(rc);
  if (cudaStreamEndCapture(c->stream, &tmp) != cudaSuccess) return fail(SOL_ERR_CUDA);
  G.k_pro = (int)(sol_capture_count() - k0);
  // attempt loop
  cudaGraphNodeParams cp = {};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = hcond;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  cudaGraphNode_t cnode;
  if (cudaGraphAddNode(&cnode, graph, deps.data(), nullptr, deps.size(), &cp) != cudaSuccess) return fail(SOL_ERR_CUDA);
  cudaGraph_t body = cp.conditional.phGraph_out[0];
  k0 = sol_capture_count();
  if (cudaStreamBeginCaptureToGraph(c->stream, body, nullptr, nullptr, 0, mode) != cudaSuccess) return fail(SOL_ERR_CUDA);
  if (integrator == SOL_RUNGE_KUTTA_FEHLBERG78) {
    if ((rc = rkf78_attempt(c, c->d_y0, c->d_y, c->d_err))) return fail(rc);
    k_control_rkf78<<<1, 1, 0, c->stream>>>(c->d_ctrl, hcond, 1);
  } else {
    if ((rc = dp_attempt(c))) return fail(rc);
    k_control_dp<<<1, 1, 0, c->stream>>>(c->d_ctrl, hcond, 1);
  }
  sol_count_launch();
  if (cudaStreamEndCapture(c->stream, &tmp) != cudaSuccess) return fail(SOL_ERR_CUDA);
  G.k_body = (int)(sol_capture_count() - k0);
  // epilogue
  k0 = sol_capture_count();
  if (cudaStreamBeginCaptureToGraph(c->stream, graph, &cnode, nullptr, 1, mode) != cudaSuccess) return fail(SOL_ERR_CUDA);
  k_accept_copy<<<grid_for(c->nv), kBlock, 0, c->stream>>>(c->nv, c->d_y0, c->d_y, c->d_ctrl);
  sol_count_launch();
  if (cudaStreamEndCapture(c->stream, &tmp) != cudaSuccess) return fail(SOL_ERR_CUDA);
  G.k_epi = (int)(sol_capture_count() - k0);
  cudaGraphExec_t exec = nullptr;
  if (cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) return fail(SOL_ERR_CUDA);
  G.graph = graph;
  G.exec = exec;
  G.precision = c->precision;
  G.valid = 1;
  return SOL_OK;
}

}  // namespace

int sol_integrator_run(sol_ctx* c, int integrator, int n_steps) {
  // few-source systems: every driver call of the sequence in one cooperative
  // launch (falls through when the grid cannot be co-resident)
  if ((integrator == SOL_RUNGE_KUTTA_FEHLBERG78 || integrator == SOL_RUNGE_KUTTA4) && c->device_loop &&
      n_steps > 0 && sol_group_eligible(c)) {
    const int r = sol_group_rkf78(c, n_steps, nullptr, integrator == SOL_RUNGE_KUTTA4);
    if (r != SOL_ERR_STATE) return r;
  }
  if (integrator == SOL_RUNGE_KUTTA_FEHLBERG78 && c->device_loop && n_steps > 0) {
    if (sol_persist_eligible(c)) {
      const int r = sol_persist_rkf78(c, n_steps);
      if (r != SOL_ERR_STATE) return r;
    }
  }
  const int gi = integrator == SOL_RUNGE_KUTTA_FEHLBERG78 ? 0 : (integrator == SOL_DORMAND_PRINCE ? 1 : -1);
  if (gi >= 0 && c->device_loop && n_steps > 0) {
    DriverGraph& G = c->graphs[gi];
    if (G.valid && G.precision != c->precision) sol_graph_release(G);
    if (!G.valid && build_driver_graph(c, integrator, G) != SOL_OK) {
      c->device_loop = 0;  // graphs unavailable here: keep the host-driven loop
      cudaGetLastError();
    } else {
      for (int s = 0; s < n_steps; ++s) SOL_CUDA(cudaGraphLaunch(G.exec, c->stream));
      c->graph_steps += n_steps;
      c->graph_used = gi + 1;
      return SOL_OK;
    }
  }
  for (int s = 0; s < n_steps; ++s) {
    int r;
    if (integrator == SOL_RUNGE_KUTTA_FEHLBERG78) r = rkf78_driver_step(c);
    else if (integrator == SOL_RUNGE_KUTTA4) r = rk4_driver_step(c);
    else if (integrator == SOL_DORMAND_PRINCE) r = dp_driver_step(c);
    else {
      sol_set_error("unknown integrator %d", integrator);
      return SOL_ERR_ARG;
    }
    if (r != SOL_OK) return r;
  }
  return SOL_OK;
}

int sol_rkf78_single_attempt(sol_ctx* c, double t, double h, const double* d_y0, double* d_y, double* d_err,
                             double* error_max) {
  // ctrl t and h from the host, then the Driver's first evaluation, yscale and one attempt
  sol_ctrl hc;
  memset(&hc, 0, sizeof(hc));
  hc.t = t;
  hc.h = h;
  hc.h_next = h;
  hc.eps = c->eps;
  SOL_CUDA(cudaMemcpyAsync(c->d_ctrl, &hc, sizeof(hc), cudaMemcpyHostToDevice, c->stream));
  RET(sol_force_launch(c, d_y0, c->d_accel, stage_time(c, 0.0), SOL_EVAL_ALL));
  const int g = grid_for(c->nv);
  k_yscale<<<g, kBlock, 0, c->stream>>>(c->nv, d_y0, c->d_accel, c->d_yscale, c->d_ctrl);
  SOL_LAUNCHED();
  RET(rkf78_attempt(c, d_y0, d_y, d_err));
  RET(read_ctrl(c));
  RET(ctrl_status(c));
  *error_max = c->h_ctrl->error_max;
  return SOL_OK;
}

int sol_integrate_partials_needed(int nv) { return grid_for(nv); }

const Rkf78Table& sol_rkf78_table() {
  static Rkf78Table T;
  // filled once; contexts of several host threads may arrive together
  static std::atomic<bool> init{false};
  static std::mutex init_mutex;
  std::unique_lock<std::mutex> init_lock(init_mutex, std::defer_lock);
  if (!init.load(std::memory_order_acquire) && (init_lock.lock(), !init.load(std::memory_order_relaxed))) {
    memset(&T, 0, sizeof(T));
    const Rkf78Stage* st = rkf78_stages();
    for (int r = 1; r <= 12; ++r) {
      T.k[r] = st[r].k;
      for (int q = 0; q < st[r].k; ++q) {
        T.idx[r][q] = st[r].idx[q];
        T.a[r][q] = st[r].a[q];
      }
    }
    init.store(true, std::memory_order_release);
  }
  return T;
}

// The elementwise kernels of one RKF78 attempt alone -- 12 stage sums, the
// fused final sum / error estimate / scaled norm and the norm reduction --
// over the context's stage vectors, timed with CUDA events on the context's
// stream: their HBM bytes per attempt are 8 * 6N * 93 (79 passes of the
// stage sums, 9 of the final sum, 5 of the error norm).
int sol_bench_stage_kernels(sol_ctx* c, int reps, double* ms_per_attempt) {
  const Rkf78Stage* st = rkf78_stages();
  double* fk[13];
  fk[0] = c->d_accel;
  for (int k = 1; k < 13; ++k) fk[k] = c->d_fk[k];
  auto one = [&]() -> int {
    for (int r = 1; r <= 12; ++r) {
      StageArgs sa;
      memset(&sa, 0, sizeof(sa));
      for (int k = 0; k < st[r].k; ++k) {
        sa.f[k] = fk[st[r].idx[k]];
        sa.a[k] = st[r].a[k];
      }
      // each stage writes its own input vector, as the attempt's evaluations would read it
      RET(launch_stage(c, st[r].k, sa, c->d_y0, r < 12 ? c->d_fk[r + 1] : c->d_ytmp));
    }
    Rkf78FinalArgs fa;
    for (int k = 0; k < 13; ++k) fa.f[k] = fk[k];
    const int g = grid_for(c->nv);
    k_rkf78_final<<<g, kBlock, 0, c->stream>>>(c->nv, c->d_y0, fa, c->d_y, c->d_err, c->d_yscale, c->d_partial,
                                              c->d_ctrl);
    SOL_LAUNCHED();
    k_reduce_max<<<1, kBlock, 0, c->stream>>>(c->d_partial, g, c->d_ctrl, 1);
    SOL_LAUNCHED();
    return SOL_OK;
  };
  RET(one());  // warm-up
  cudaEvent_t e0, e1;
  SOL_CUDA(cudaEventCreate(&e0));
  SOL_CUDA(cudaEventCreate(&e1));
  SOL_CUDA(cudaEventRecord(e0, c->stream));
  int rc = SOL_OK;
  for (int r = 0; r < reps && rc == SOL_OK; ++r) rc = one();
  SOL_CUDA(cudaEventRecord(e1, c->stream));
  SOL_CUDA(cudaEventSynchronize(e1));
  float ms = 0.0f;
  SOL_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *ms_per_attempt = ms / reps;
  return rc;
}

// One attempt from the resident d_y0 with f0 = d_accel (and, for RKF78, the
// yscale in d_yscale; k_yscale fills it from f0 when compute_yscale is set):
// RungeKuttaFehlberg78::Step, RungeKutta4::Step or DormandPrince::Step2 with
// the given evaluate flags, into d_y and d_err; the error norm of RKF78 / DP
// lands in the control block.  t and h come from the host.
int sol_attempt_launch(sol_ctx* c, int integrator, double t, double h, uint32_t flags, int compute_yscale) {
  sol_ctrl hc;
  memset(&hc, 0, sizeof(hc));
  hc.t = t;
  hc.h = h;
  hc.h_next = h;
  hc.eps = c->eps;
  SOL_CUDA(cudaMemcpyAsync(c->d_ctrl, &hc, sizeof(hc), cudaMemcpyHostToDevice, c->stream));
  if (integrator == SOL_RUNGE_KUTTA_FEHLBERG78) {
    if (compute_yscale) {
      k_yscale<<<grid_for(c->nv), kBlock, 0, c->stream>>>(c->nv, c->d_y0, c->d_accel, c->d_yscale, c->d_ctrl);
      SOL_LAUNCHED();
    }
    RET(rkf78_attempt(c, c->d_y0, c->d_y, c->d_err, flags));
  } else if (integrator == SOL_RUNGE_KUTTA4) {
    RET(rk4_attempt(c, c->d_y0, c->d_y, flags));
  } else if (integrator == SOL_DORMAND_PRINCE) {
    RET(dp_attempt(c, flags));
  } else {
    sol_set_error("unknown integrator %d", integrator);
    return SOL_ERR_ARG;
  }
  RET(read_ctrl(c));
  return ctrl_status(c);
}

// One fixed-h RungeKuttaFehlberg78::Step without the error estimate: the first
// evaluation at y0, 12 stages and the 7th-order result into y.  Stage inputs go
// to stage_out[r] when given (r = 1..12), else to the context's scratch.  h is
// the control block's.
int sol_rkf78_stages(sol_ctx* c, const double* d_y0, double* d_y, double* const* stage_out) {
  const Rkf78Stage* st = rkf78_stages();
  double* fk[13];
  fk[0] = c->d_accel;
  for (int k = 1; k < 13; ++k) fk[k] = c->d_fk[k];
  RET(sol_force_launch(c, d_y0, fk[0], stage_time(c, 0.0), SOL_EVAL_ALL));
  for (int r = 1; r <= 12; ++r) {
    StageArgs sa;
    memset(&sa, 0, sizeof(sa));
    for (int k = 0; k < st[r].k; ++k) {
      sa.f[k] = fk[st[r].idx[k]];
      sa.a[k] = st[r].a[k];
    }
    if (r > 10) break;  // stages 11 and 12 enter only the error estimate
    double* out = (stage_out && stage_out[r]) ? stage_out[r] : c->d_ytmp;
    RET(launch_stage(c, st[r].k, sa, d_y0, out));
    RET(sol_force_launch(c, out, fk[r], stage_time(c, 0.0), SOL_EVAL_GAS_DRAG));
  }
  Rkf78FinalArgs fa;
  for (int k = 0; k < 13; ++k) fa.f[k] = fk[k];
  const int g = grid_for(c->nv);
  k_rkf78_y<<<g, kBlock, 0, c->stream>>>(c->nv, d_y0, fa, d_y, c->d_ctrl);
  SOL_LAUNCHED();
  return SOL_OK;
}

void sol_graph_release(DriverGraph& G) {
  if (G.exec) cudaGraphExecDestroy(G.exec);
  if (G.graph) cudaGraphDestroy(G.graph);
  G = DriverGraph{};
}
