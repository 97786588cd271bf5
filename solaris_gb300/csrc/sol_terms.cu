// Entry points behind the C++ class facade (Acceleration, RungeKuttaFehlberg78,
// RungeKutta4, DormandPrince with the reference's member functions): one term
// of Acceleration::Compute at a time, the scalar migration helpers, the
// integrators' GetErrorMax on caller arrays, single attempts from a caller's
// f0, and read-back of the vectors a Driver call leaves in BodyData and
// Acceleration.  Everything is evaluated on the device with the same device
// functions the fused force kernels use.
#include <cmath>
#include <cstring>

#include "sol_internal.cuh"

int sol_attempt_launch(sol_ctx* c, int integrator, double t, double h, uint32_t flags, int compute_yscale);

namespace {

constexpr int kBlock = 256;

// GasDragAC (Acceleration.cpp:331-422), MigrationTypeIAC (:424-485) and
// MigrationTypeIIAC (:487-528) over their body ranges, into rows i - lower of
// out.  Migration rows of bodies with another migType are left untouched, as
// the reference's `continue` leaves them.
__global__ void k_gas_term(ForceCtx fc, const double* __restrict__ y, double t, int term, int lower, int upper,
                           double* __restrict__ out) {
  const int i = lower + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= upper) return;
  const GasDev& g = fc.gas;
  double yi[6];
  for (int k = 0; k < 6; ++k) yi[k] = y[6 * i + k];
  const double factor = sol_reduction_factor(g, t);
  const double m0 = fc.mass[0];
  double d[3];
  if (term == SOL_TERM_GAS_DRAG) {
    sol_gas_drag(g, factor, m0, yi, fc.radius[i], fc.density[i], fc.cd[i], fc.gamma_stokes[i], fc.gamma_epstein[i],
                 d);
  } else if (term == SOL_TERM_TYPE_I) {
    if (fc.mig_type[i] != SOL_MIGRATION_TYPE_I) return;
    if (!sol_migration_type1(g, factor, m0, fc.mass[i], fc.mig_stop_at[i], yi, d)) fc.mig_type[i] = SOL_MIGRATION_NO;
  } else {
    if (fc.mig_type[i] != SOL_MIGRATION_TYPE_II) return;
    if (!sol_migration_type2(g, factor, m0, fc.mass[i], fc.mig_stop_at[i], yi, d)) fc.mig_type[i] = SOL_MIGRATION_NO;
  }
  double* o = out + 3 * (i - lower);
  o[0] = d[0];
  o[1] = d[1];
  o[2] = d[2];
}

__global__ void k_helper(GasDev g, int which, double a0, double a1, double a2, double a3, double a4, double* out) {
  if (which == SOL_HELPER_TYPE_I_MIGRATION_TIME)
    *out = sol_type1_migration_time(g, a0, a1, a2, a3, a4);
  else if (which == SOL_HELPER_TYPE_I_ECC_DAMPING_TIME)
    *out = sol_type1_ecc_damping_time(a0, a1, a2, a3, a4);
  else
    *out = sol_tau_nu(g, a0, a1);
}

// max_i |yerr_i / yscale_i| (or |yerr_i| without yscale).  The comparison
// `v > m` is the reference's: NaN entries never replace the running maximum.
__global__ void k_err_max_part(int n, const double* __restrict__ yerr, const double* __restrict__ yscale,
                               double* __restrict__ partial) {
  __shared__ double sm[kBlock];
  double m = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double v = yscale ? fabs(yerr[i] / yscale[i]) : fabs(yerr[i]);
    if (v > m) m = v;
  }
  sm[threadIdx.x] = m;
  __syncthreads();
  for (int s = kBlock / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s && sm[threadIdx.x + s] > sm[threadIdx.x]) sm[threadIdx.x] = sm[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = sm[0];
}

__global__ void k_err_max_final(const double* __restrict__ partial, int np, double* __restrict__ out) {
  __shared__ double sm[kBlock];
  double m = 0.0;
  for (int i = threadIdx.x; i < np; i += kBlock)
    if (partial[i] > m) m = partial[i];
  sm[threadIdx.x] = m;
  __syncthreads();
  for (int s = kBlock / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s && sm[threadIdx.x + s] > sm[threadIdx.x]) sm[threadIdx.x] = sm[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sm[0];
}

#define RET(x)                   \
  do {                           \
    int r_ = (x);                \
    if (r_ != SOL_OK) return r_; \
  } while (0)

int prologue(const sol_ctx* c) {
  if (!c) {
    sol_set_error("null context");
    return SOL_ERR_ARG;
  }
  SOL_CUDA(cudaSetDevice(c->device));
  return SOL_OK;
}

int finish(sol_ctx* c) {
  SOL_CUDA(cudaMemcpyAsync(c->h_ctrl, c->d_ctrl, sizeof(sol_ctrl), cudaMemcpyDeviceToHost, c->stream));
  SOL_CUDA(cudaStreamSynchronize(c->stream));
  if (c->h_ctrl->dev_status & SOL_DEV_TIMEOUT) {
    sol_set_error("a bounded device wait ran out in the force kernel");
    return SOL_ERR_TIMEOUT;
  }
  return SOL_OK;
}

}  // namespace

extern "C" {

int sol_accel_term(sol_ctx* c, int32_t term, double t, const double* y, double* out) {
  RET(prologue(c));
  if (!y || !out || term < SOL_TERM_GRAVITY || term > SOL_TERM_TYPE_II) {
    sol_set_error("sol_accel_term: bad arguments");
    return SOL_ERR_ARG;
  }
  if (term != SOL_TERM_GRAVITY && !c->has_gas) {
    sol_set_error("sol_accel_term: the context has no nebula");
    return SOL_ERR_STATE;
  }
  SOL_CUDA(cudaMemcpyAsync(c->d_io_in, y, sizeof(double) * c->nv, cudaMemcpyHostToDevice, c->stream));
  SOL_CUDA(cudaMemsetAsync(&c->d_ctrl->dev_status, 0, sizeof(int), c->stream));
  if (term == SOL_TERM_GRAVITY) {
    // GravityAC / GravityBC alone: the force kernels with the nebula switched
    // off for this launch (the kernels take the context by value)
    const ForceCtx saved = c->fc;
    c->fc.gas.present = 0;
    TimeSpec ts{nullptr, nullptr, 0.0, t};
    const int rc = sol_force_launch(c, c->d_io_in, c->d_io_out, ts, 0);
    c->fc = saved;
    RET(rc);
    SOL_CUDA(cudaMemcpyAsync(out, c->d_io_out, sizeof(double) * c->nv, cudaMemcpyDeviceToHost, c->stream));
    c->last_eval_valid = 1;
    return finish(c);
  }
  const Classes& cl = c->cls;
  int lower, upper;
  if (term == SOL_TERM_GAS_DRAG) {
    lower = cl.nm;
    upper = cl.nm + cl.n_spl + cl.n_pl;
  } else if (term == SOL_TERM_TYPE_I) {
    lower = cl.n_central + cl.n_giant;
    upper = cl.nm;
  } else {
    lower = cl.n_central;
    upper = cl.n_central + cl.n_giant;
  }
  const int rows = upper - lower;
  if (rows <= 0) return SOL_OK;
  SOL_CUDA(cudaMemcpyAsync(c->d_io_out, out, sizeof(double) * 3 * rows, cudaMemcpyHostToDevice, c->stream));
  k_gas_term<<<(rows + kBlock - 1) / kBlock, kBlock, 0, c->stream>>>(c->fc, c->d_io_in, t, term, lower, upper,
                                                                      c->d_io_out);
  SOL_LAUNCHED();
  SOL_CUDA(cudaMemcpyAsync(out, c->d_io_out, sizeof(double) * 3 * rows, cudaMemcpyDeviceToHost, c->stream));
  return finish(c);
}

int sol_migration_helper(sol_ctx* c, int32_t which, const double* args, double* out) {
  RET(prologue(c));
  if (!args || !out || which < SOL_HELPER_TYPE_I_MIGRATION_TIME || which > SOL_HELPER_TAU_NU) {
    sol_set_error("sol_migration_helper: bad arguments");
    return SOL_ERR_ARG;
  }
  if (which != SOL_HELPER_TYPE_I_ECC_DAMPING_TIME && !c->has_gas) {
    sol_set_error("sol_migration_helper: the context has no nebula");
    return SOL_ERR_STATE;
  }
  const int na = which == SOL_HELPER_TAU_NU ? 2 : 5;
  double a[5] = {0, 0, 0, 0, 0};
  for (int k = 0; k < na; ++k) a[k] = args[k];
  double* d_out = c->d_partial + c->n_partial;
  k_helper<<<1, 1, 0, c->stream>>>(c->fc.gas, which, a[0], a[1], a[2], a[3], a[4], d_out);
  SOL_LAUNCHED();
  SOL_CUDA(cudaMemcpyAsync(out, d_out, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  SOL_CUDA(cudaStreamSynchronize(c->stream));
  return SOL_OK;
}

int sol_error_max(sol_ctx* c, int32_t integrator, int32_t n, const double* yerr, const double* yscale,
                  double epsilon, double* out) {
  const bool rkf = integrator == SOL_RUNGE_KUTTA_FEHLBERG78;
  if (!yerr || !out || n < 0 || (c && n > c->nv) || (!rkf && integrator != SOL_DORMAND_PRINCE) ||
      (rkf && !yscale)) {
    sol_set_error("sol_error_max: bad arguments");
    return SOL_ERR_ARG;
  }
  double m = 0.0;
  if (n > 0) {
    // with a context its staging buffers and stream; without one (the
    // reference's GetErrorMax takes no Acceleration) temporary buffers on the
    // current device's default stream
    cudaStream_t st = c ? c->stream : 0;
    double *d_err, *d_scale, *d_part;
    int blocks = (n + kBlock - 1) / kBlock;
    if (c) {
      SOL_CUDA(cudaSetDevice(c->device));
      d_err = c->d_io_in;
      d_scale = c->d_io_out;
      d_part = c->d_partial;
      if (blocks > c->n_partial) blocks = c->n_partial;
    } else {
      if (blocks > 4096) blocks = 4096;
      void* p = nullptr;
      SOL_CUDA(cudaMalloc(&p, sizeof(double) * (2 * (size_t)n + blocks + 1)));
      d_err = (double*)p;
      d_scale = d_err + n;
      d_part = d_scale + n;
    }
    double* d_out = d_part + (c ? c->n_partial : blocks);
    int rc = SOL_OK;
    cudaError_t e = cudaMemcpyAsync(d_err, yerr, sizeof(double) * n, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && rkf) e = cudaMemcpyAsync(d_scale, yscale, sizeof(double) * n, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
      k_err_max_part<<<blocks, kBlock, 0, st>>>(n, d_err, rkf ? d_scale : nullptr, d_part);
      sol_count_launch();
      k_err_max_final<<<1, kBlock, 0, st>>>(d_part, blocks, d_out);
      sol_count_launch();
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&m, d_out, sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) rc = sol_cuda_fail(e, "sol_error_max", __FILE__, __LINE__);
    if (!c) cudaFree(d_err);
    if (rc != SOL_OK) return rc;
  }
  *out = rkf ? m / epsilon : m;
  return SOL_OK;
}

int sol_integrator_attempt(sol_ctx* c, int32_t integrator, double t, double h, const double* y0, const double* f0,
                           const double* yscale, double* y, double* error, double* error_max) {
  RET(prologue(c));
  if (!y0 || !f0 || !y) {
    sol_set_error("sol_integrator_attempt: y0, f0 and y are required");
    return SOL_ERR_ARG;
  }
  const size_t bytes = sizeof(double) * c->nv;
  SOL_CUDA(cudaMemcpyAsync(c->d_y0, y0, bytes, cudaMemcpyHostToDevice, c->stream));
  SOL_CUDA(cudaMemcpyAsync(c->d_accel, f0, bytes, cudaMemcpyHostToDevice, c->stream));
  const int rkf = integrator == SOL_RUNGE_KUTTA_FEHLBERG78;
  if (rkf && yscale) SOL_CUDA(cudaMemcpyAsync(c->d_yscale, yscale, bytes, cudaMemcpyHostToDevice, c->stream));
  c->state_valid = 1;
  RET(sol_attempt_launch(c, integrator, t, h, c->eval_flags, rkf && !yscale));
  SOL_CUDA(cudaMemcpyAsync(y, c->d_y, bytes, cudaMemcpyDeviceToHost, c->stream));
  if (error && integrator != SOL_RUNGE_KUTTA4)
    SOL_CUDA(cudaMemcpyAsync(error, c->d_err, bytes, cudaMemcpyDeviceToHost, c->stream));
  SOL_CUDA(cudaStreamSynchronize(c->stream));
  if (error_max) *error_max = integrator == SOL_RUNGE_KUTTA4 ? 0.0 : c->h_ctrl->error_max;
  c->last_eval_valid = 1;
  return SOL_OK;
}

int sol_get_driver_vectors(sol_ctx* c, double* accel, double* yscale, double* error) {
  RET(prologue(c));
  const size_t bytes = sizeof(double) * c->nv;
  if (accel) SOL_CUDA(cudaMemcpyAsync(accel, c->d_accel, bytes, cudaMemcpyDeviceToHost, c->stream));
  if (yscale) SOL_CUDA(cudaMemcpyAsync(yscale, c->d_yscale, bytes, cudaMemcpyDeviceToHost, c->stream));
  if (error) SOL_CUDA(cudaMemcpyAsync(error, c->d_err, bytes, cudaMemcpyDeviceToHost, c->stream));
  SOL_CUDA(cudaStreamSynchronize(c->stream));
  return SOL_OK;
}

int sol_get_side_buffers(sol_ctx* c, double* drag, double* mig1, double* mig2) {
  RET(prologue(c));
  const Classes& cl = c->cls;
  const size_t nd = 3 * (size_t)(cl.n_spl + cl.n_pl), n1 = 3 * (size_t)(cl.n_rocky + cl.n_proto),
               n2 = 3 * (size_t)cl.n_giant;
  if (drag && nd) SOL_CUDA(cudaMemcpyAsync(drag, c->d_drag, sizeof(double) * nd, cudaMemcpyDeviceToHost, c->stream));
  if (mig1 && n1) SOL_CUDA(cudaMemcpyAsync(mig1, c->d_mig1, sizeof(double) * n1, cudaMemcpyDeviceToHost, c->stream));
  if (mig2 && n2) SOL_CUDA(cudaMemcpyAsync(mig2, c->d_mig2, sizeof(double) * n2, cudaMemcpyDeviceToHost, c->stream));
  SOL_CUDA(cudaStreamSynchronize(c->stream));
  return SOL_OK;
}

}  // extern "C"
