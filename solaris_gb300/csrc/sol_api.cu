// C-ABI entry points of libsolaris_gb300 (include/solaris_gb300.h).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "sol_internal.cuh"

int sol_force_tile();
int sol_force_part_doubles(const sol_ctx* c);
int sol_force_uses_chunk_partials(const sol_ctx* c, int precision);
int sol_force_prepass_blocks(int npad);
int sol_force_src_doubles();
int sol_force_launch_sinks(sol_ctx* c, const double* d_y, double* d_dydt, TimeSpec ts, uint32_t flags, int lo, int hi);
int sol_integrate_partials_needed(int nv);
int sol_potential_launch(sol_ctx* c, const double* d_y0, double* d_part, int* nparts);

// ---- errors and counters -----------------------------------------------------
static thread_local char g_err[1024] = "";
static std::atomic<long long> g_launches{0};
static thread_local int g_capturing = 0;
static thread_local long long g_captured = 0;

void sol_set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

int sol_cuda_fail(cudaError_t e, const char* what, const char* file, int line) {
  sol_set_error("CUDA error %d (%s) in %s at %s:%d", (int)e, cudaGetErrorString(e), what, file, line);
  return SOL_ERR_CUDA;
}

// Kernels launched into a stream capture are counted per captured kernel and
// added to the launch count each time their graph runs.
void sol_count_launch() {
  if (g_capturing)
    ++g_captured;
  else
    g_launches.fetch_add(1, std::memory_order_relaxed);
}
void sol_capture_begin() {
  g_capturing = 1;
  g_captured = 0;
}
void sol_capture_end() { g_capturing = 0; }
long long sol_capture_count() { return g_captured; }

#define RET(x)                   \
  do {                           \
    int r_ = (x);                \
    if (r_ != SOL_OK) return r_; \
  } while (0)

// ---- reference constants (Solaris/Constants.h) --------------------------------
namespace {
const double kSolarToKilogram = 1.98911e30;
const double kAuToMeter = 1.495978707e11;
const double kDayToSecond = 86400.0;
const double kBoltzmanSI = 1.3806488e-23;
const double kProtonMassSI = 1.672621777e-27;
double kilogram_to_solar() { return 1.0 / kSolarToKilogram; }
double meter_to_au() { return 1.0 / kAuToMeter; }
double gram_per_cm3_to_solar_per_au3() {
  double l = 1.0e-2 * meter_to_au();
  return (1.0 / (1.0e3 * kSolarToKilogram)) / (l * l * l);
}
double proton_mass_cmu() { return kProtonMassSI * kilogram_to_solar(); }
double boltzman_cmu() {
  double m = meter_to_au(), s = 1.0 / kDayToSecond;
  return kBoltzmanSI * (kilogram_to_solar() * (m * m)) / (s * s);
}
double proton_mass_boltzman_cmu() { return 1.0 / (boltzman_cmu() / proton_mass_cmu()); }

GasDev make_gas_dev(const sol_gas_component* g, int barycentric) {
  GasDev d;
  memset(&d, 0, sizeof(d));
  if (!g) return d;
  d.present = 1;
  d.decrease_type = g->decrease_type;
  d.quirks = g->quirks;
  d.barycentric = barycentric;
  d.alpha = g->alpha;
  d.time_scale = g->time_scale;
  d.t0 = g->t0;
  d.t1 = g->t1;
  d.inner_edge = g->inner_edge;
  d.mmw = g->mean_molecular_weight;
  d.eta_c = g->eta.c;
  d.eta_i = g->eta.index;
  d.tau_c = g->tau.c;
  d.tau_i = g->tau.index;
  d.sh_c = g->scale_height.c;
  d.sh_i = g->scale_height.index;
  d.rho_c = g->density.c;
  d.rho_i = g->density.index;
  d.mfp_c = g->mean_free_path.c;
  d.mfp_i = g->mean_free_path.index;
  // GasComponent.cpp:223-241 (statics evaluated on first use)
  d.cvth = sqrt((8.0 * boltzman_cmu()) / (3.14159265358979323846 * g->mean_molecular_weight * proton_mass_cmu()));
  d.ctp = 2.959122082855911025e-4 * proton_mass_boltzman_cmu();
  d.pt = 2.0 * g->scale_height.index - 3.0;
  d.abs_rho_index = (g->quirks & SOL_QUIRK_INT_ABS) ? (double)std::abs((int)g->density.index) : fabs(g->density.index);
  return d;
}

template <class T>
int dev_alloc(T** p, size_t count) {
  *p = nullptr;
  if (count == 0) count = 1;
  cudaError_t e = cudaMalloc((void**)p, sizeof(T) * count);
  if (e != cudaSuccess) {
    sol_set_error("cudaMalloc of %zu bytes failed: %s", sizeof(T) * count, cudaGetErrorString(e));
    return SOL_ERR_NOMEM;
  }
  e = cudaMemset(*p, 0, sizeof(T) * count);
  if (e != cudaSuccess) return sol_cuda_fail(e, "cudaMemset", __FILE__, __LINE__);
  return SOL_OK;
}

template <class T>
int upload(T* d, const T* h, size_t count, T fill) {
  if (h) {
    SOL_CUDA(cudaMemcpy(d, h, sizeof(T) * count, cudaMemcpyHostToDevice));
  } else if (fill != T(0)) {
    std::vector<T> v(count, fill);
    SOL_CUDA(cudaMemcpy(d, v.data(), sizeof(T) * count, cudaMemcpyHostToDevice));
  }
  return SOL_OK;
}

void free_ctx(sol_ctx* c) {
  if (!c) return;
  void* ptrs[] = {c->d_type, c->d_mig_type, c->d_mig_stop_at, c->d_mass, c->d_radius, c->d_density, c->d_cd,
                  c->d_gs, c->d_ge, c->d_rm3, c->d_nn_dist, c->d_src, c->d_drag, c->d_mig1, c->d_mig2,
                  c->d_ind_part, c->d_ind_sum, c->d_nn_idx, c->d_y0, c->d_y, c->d_accel, c->d_yscale, c->d_err,
                  c->d_ytmp, c->d_io_in, c->d_io_out, c->d_partial, c->d_ctrl, c->d_part};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  for (int k = 0; k < 13; ++k)
    if (c->d_fk[k]) cudaFree(c->d_fk[k]);
  for (int k = 0; k < 2; ++k) sol_graph_release(c->graphs[k]);
  sol_adjoint_free(c->adj);
  if (c->d_persist) cudaFree(c->d_persist);
  if (c->d_sim) cudaFree(c->d_sim);
  if (c->d_ystart) cudaFree(c->d_ystart);
  free(c->h_id);
  if (c->h_ctrl) cudaFreeHost(c->h_ctrl);
  if (c->h_stage) cudaFreeHost(c->h_stage);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

int check_ctx(const sol_ctx* c) {
  if (!c) {
    sol_set_error("null context");
    return SOL_ERR_ARG;
  }
  return SOL_OK;
}

int set_device(const sol_ctx* c) {
  SOL_CUDA(cudaSetDevice(c->device));
  return SOL_OK;
}
}  // namespace

extern "C" {

const char* sol_last_error(void) { return g_err; }

int sol_version(void) { return 100; }

int sol_kernel_launch_count(int64_t* count) {
  if (!count) return SOL_ERR_ARG;
  *count = g_launches.load();
  return SOL_OK;
}

int sol_gas_component_init(sol_gas_component* g) {
  // GasComponent::GasComponent (Solaris/GasComponent.cpp:9-34)
  if (!g) {
    sol_set_error("null gas component");
    return SOL_ERR_ARG;
  }
  memset(g, 0, sizeof(*g));
  g->inner_edge = 10.0 * (1.0 / 215.094);
  g->alpha = 2.0e-3;
  g->mean_molecular_weight = 2.3;
  g->particle_diameter = 3.0e-10;
  g->time_scale = 0.0;
  g->t0 = 0.0;
  g->t1 = 0.0;
  g->decrease_type = SOL_GAS_CONSTANT;
  g->quirks = SOL_QUIRKS_REFERENCE;
  g->eta = sol_power_law{0.0019, 0.5};
  g->tau = sol_power_law{2.0 / 3.0, 2.0};
  g->scale_height = sol_power_law{0.02, 1.25};
  g->density = sol_power_law{1.4e-9 * gram_per_cm3_to_solar_per_au3(), -2.75};
  double d = g->particle_diameter * meter_to_au();
  double clambda =
      g->mean_molecular_weight * proton_mass_cmu() / (sqrt(2.0) * 3.14159265358979323846 * (d * d) * g->density.c);
  g->mean_free_path = sol_power_law{clambda, -g->density.index};
  return SOL_OK;
}

int sol_create(const sol_body_data* b, const sol_gas_component* gas, int32_t barycentric, int32_t device,
               sol_ctx** out) {
  if (!b || !out) {
    sol_set_error("null argument to sol_create");
    return SOL_ERR_ARG;
  }
  *out = nullptr;
  const sol_nbodies& k = b->n;
  const int counts[7] = {k.central_body, k.giant_planet, k.rocky_planet, k.proto_planet, k.super_planetesimal,
                         k.planetesimal, k.test_particle};
  long long n = 0;
  for (int q = 0; q < 7; ++q) {
    if (counts[q] < 0) {
      sol_set_error("negative body count");
      return SOL_ERR_ARG;
    }
    n += counts[q];
  }
  if (k.central_body != 1 || n < 1 || n > (1 << 26)) {
    sol_set_error("need exactly one central body and 1 <= N <= 2^26 bodies (got central=%d, N=%lld)",
                  k.central_body, n);
    return SOL_ERR_ARG;
  }
  if (!b->type || !b->mass) {
    sol_set_error("body type and mass arrays are required");
    return SOL_ERR_ARG;
  }
  // bodies must be sorted by BodyType (Simulator::Insert, Solaris/Simulator.cpp:467-483)
  int expect = 0;
  for (int q = 0; q < 7; ++q) {
    for (int r = 0; r < counts[q]; ++r, ++expect) {
      if (b->type[expect] != q + 1) {
        sol_set_error("body %d has type %d, expected %d: bodies must be sorted by type", expect, b->type[expect],
                      q + 1);
        return SOL_ERR_ARG;
      }
    }
  }
  if (gas && (gas->decrease_type < 0 || gas->decrease_type > 2)) {
    sol_set_error("unknown gas decrease type %d", gas->decrease_type);
    return SOL_ERR_ARG;
  }
  int ndev = 0;
  SOL_CUDA(cudaGetDeviceCount(&ndev));
  if (device < 0 || device >= ndev) {
    sol_set_error("device %d not available (%d devices)", device, ndev);
    return SOL_ERR_ARG;
  }
  SOL_CUDA(cudaSetDevice(device));

  sol_ctx* c = new sol_ctx;
  memset(c, 0, sizeof(*c));
  c->device = device;
  c->counts = k;
  c->n = (int)n;
  c->nv = 6 * c->n;
  const int tile = sol_force_tile();
  c->npad = ((c->n + tile - 1) / tile) * tile;
  c->barycentric = barycentric ? 1 : 0;
  c->precision = SOL_PRECISION_FP64;
  c->eval_flags = SOL_EVAL_ALL;
  c->eps = pow(10, -10.0);  // RungeKuttaFehlberg78.cpp:38-39
  c->device_loop = 1;
  c->test_skip_cta = -1;
  c->has_gas = gas != nullptr;
  if (gas) c->gas_host = *gas;
  Classes& cl = c->cls;
  cl.n = c->n;
  cl.n_central = k.central_body;
  cl.n_giant = k.giant_planet;
  cl.n_rocky = k.rocky_planet;
  cl.n_proto = k.proto_planet;
  cl.n_spl = k.super_planetesimal;
  cl.n_pl = k.planetesimal;
  cl.nm = k.central_body + k.giant_planet + k.rocky_planet + k.proto_planet;

  int rc = SOL_OK;
  auto fail = [&](int r) {
    free_ctx(c);
    return r;
  };
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    sol_set_error("cudaStreamCreate failed");
    return fail(SOL_ERR_CUDA);
  }
  const size_t N = c->n, NV = c->nv;
  c->h_id = (int32_t*)malloc(sizeof(int32_t) * N);
  if (!c->h_id) {
    sol_set_error("host allocation failed");
    return fail(SOL_ERR_NOMEM);
  }
  for (size_t i = 0; i < N; ++i) c->h_id[i] = b->id ? b->id[i] : (int32_t)i;
  if ((rc = dev_alloc(&c->d_type, N)) || (rc = dev_alloc(&c->d_mig_type, N)) ||
      (rc = dev_alloc(&c->d_mig_stop_at, N)) || (rc = dev_alloc(&c->d_mass, N)) ||
      (rc = dev_alloc(&c->d_radius, N)) || (rc = dev_alloc(&c->d_density, N)) || (rc = dev_alloc(&c->d_cd, N)) ||
      (rc = dev_alloc(&c->d_gs, N)) || (rc = dev_alloc(&c->d_ge, N)) || (rc = dev_alloc(&c->d_rm3, N)) ||
      (rc = dev_alloc(&c->d_nn_dist, N)) || (rc = dev_alloc(&c->d_nn_idx, N)) ||
      (rc = dev_alloc(&c->d_src, (size_t)sol_force_src_doubles() * c->npad)) ||
      (rc = dev_alloc(&c->d_drag, 3 * (size_t)(cl.n_spl + cl.n_pl))) ||
      (rc = dev_alloc(&c->d_mig1, 3 * (size_t)(cl.n_rocky + cl.n_proto))) ||
      (rc = dev_alloc(&c->d_mig2, 3 * (size_t)cl.n_giant)) ||
      (rc = dev_alloc(&c->d_ind_part, 6 * (size_t)sol_force_prepass_blocks(c->npad))) ||
      (rc = dev_alloc(&c->d_ind_sum, 8)) || (rc = dev_alloc(&c->d_y0, NV)) || (rc = dev_alloc(&c->d_y, NV)) ||
      (rc = dev_alloc(&c->d_accel, NV)) || (rc = dev_alloc(&c->d_yscale, NV)) || (rc = dev_alloc(&c->d_err, NV)) ||
      (rc = dev_alloc(&c->d_ytmp, NV)) || (rc = dev_alloc(&c->d_io_in, NV)) || (rc = dev_alloc(&c->d_io_out, NV)))
    return fail(rc);
  for (int q = 0; q < 13; ++q)
    if ((rc = dev_alloc(&c->d_fk[q], NV))) return fail(rc);
  c->n_partial = sol_integrate_partials_needed(NV);
  // d_part (chunk partials of the 2-D split kernel) is allocated when a split
  // precision is first selected for a system that uses that kernel
  if ((rc = dev_alloc(&c->d_partial, (size_t)c->n_partial + 16)) || (rc = dev_alloc(&c->d_ctrl, 1))) return fail(rc);
  if (cudaMallocHost((void**)&c->h_ctrl, sizeof(sol_ctrl)) != cudaSuccess ||
      cudaMallocHost((void**)&c->h_stage, sizeof(double) * NV) != cudaSuccess) {
    sol_set_error("cudaMallocHost failed");
    return fail(SOL_ERR_NOMEM);
  }
  if ((rc = upload(c->d_type, (const int32_t*)b->type, N, 0)) ||
      (rc = upload(c->d_mig_type, (const int32_t*)b->mig_type, N, 0)) ||
      (rc = upload(c->d_mig_stop_at, b->mig_stop_at, N, 0.0)) || (rc = upload(c->d_mass, b->mass, N, 0.0)) ||
      (rc = upload(c->d_radius, b->radius, N, 0.0)) || (rc = upload(c->d_density, b->density, N, 0.0)) ||
      (rc = upload(c->d_cd, b->cd, N, 0.0)) || (rc = upload(c->d_gs, b->gamma_stokes, N, 0.0)) ||
      (rc = upload(c->d_ge, b->gamma_epstein, N, 0.0)))
    return fail(rc);
  {
    std::vector<int32_t> nn(N, -1);
    if (cudaMemcpy(c->d_nn_idx, nn.data(), sizeof(int32_t) * N, cudaMemcpyHostToDevice) != cudaSuccess)
      return fail(SOL_ERR_CUDA);
  }
  sol_ctrl h0;
  memset(&h0, 0, sizeof(h0));
  h0.eps = c->eps;
  if (cudaMemcpy(c->d_ctrl, &h0, sizeof(h0), cudaMemcpyHostToDevice) != cudaSuccess) return fail(SOL_ERR_CUDA);

  ForceCtx& fc = c->fc;
  fc.cls = cl;
  fc.npad = c->npad;
  fc.barycentric = c->barycentric;
  fc.precision = c->precision;
  fc.gas = make_gas_dev(gas, c->barycentric);
  fc.type = c->d_type;
  fc.mig_type = c->d_mig_type;
  fc.mig_stop_at = c->d_mig_stop_at;
  fc.mass = c->d_mass;
  fc.radius = c->d_radius;
  fc.density = c->d_density;
  fc.cd = c->d_cd;
  fc.gamma_stokes = c->d_gs;
  fc.gamma_epstein = c->d_ge;
  fc.rm3 = c->d_rm3;
  fc.nn_idx = c->d_nn_idx;
  fc.nn_dist = c->d_nn_dist;
  fc.src = c->d_src;
  fc.drag = c->d_drag;
  fc.mig1 = c->d_mig1;
  fc.mig2 = c->d_mig2;
  fc.ind_part = c->d_ind_part;
  fc.ind_sum = c->d_ind_sum;
  fc.n_ind_blocks = sol_force_prepass_blocks(c->npad);
  // buffers exist only where the reference allocates them (Acceleration.cpp:200-204, :222-226)
  fc.has_mig1 = cl.n_proto > 0;
  fc.has_mig2 = cl.n_giant > 0;
  *out = c;
  return SOL_OK;
}

int sol_destroy(sol_ctx* c) {
  if (!c) return SOL_OK;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  free_ctx(c);
  return SOL_OK;
}

int sol_set_precision(sol_ctx* c, int32_t p) {
  RET(check_ctx(c));
  if (p != SOL_PRECISION_FP64 && p != SOL_PRECISION_SPLIT && p != SOL_PRECISION_SPLIT_FF) {
    sol_set_error("unknown precision %d", p);
    return SOL_ERR_ARG;
  }
  if (p != SOL_PRECISION_FP64 && c->barycentric) {
    // GravityBC_* (Acceleration.cpp:541-634) has only the reference form here
    sol_set_error("precision %d: barycentric contexts compute in FP64 only", p);
    return SOL_ERR_ARG;
  }
  if (p != SOL_PRECISION_FP64 && !c->barycentric && !c->d_part && sol_force_uses_chunk_partials(c, p)) {
    RET(set_device(c));
    RET(dev_alloc(&c->d_part, (size_t)sol_force_part_doubles(c)));
  }
  c->precision = p;
  c->fc.precision = p;
  return SOL_OK;
}

int sol_set_eval_flags(sol_ctx* c, uint32_t flags) {
  RET(check_ctx(c));
  c->eval_flags = flags & SOL_EVAL_ALL;
  return SOL_OK;
}

int sol_get_n_total(const sol_ctx* c, int32_t* n) {
  RET(check_ctx(c));
  if (!n) return SOL_ERR_ARG;
  *n = c->n;
  return SOL_OK;
}

int sol_accel_compute(sol_ctx* c, double t, const double* y, double* dydt, double* rm3, int32_t* nn_idx,
                      double* nn_dist) {
  RET(check_ctx(c));
  if (!y || !dydt) {
    sol_set_error("y and dydt are required");
    return SOL_ERR_ARG;
  }
  RET(set_device(c));
  SOL_CUDA(cudaMemcpyAsync(c->d_io_in, y, sizeof(double) * c->nv, cudaMemcpyHostToDevice, c->stream));
  TimeSpec ts{nullptr, nullptr, 0.0, t};
  SOL_CUDA(cudaMemsetAsync(&c->d_ctrl->dev_status, 0, sizeof(int), c->stream));
  RET(sol_force_launch(c, c->d_io_in, c->d_io_out, ts, c->eval_flags));
  SOL_CUDA(cudaMemcpyAsync(dydt, c->d_io_out, sizeof(double) * c->nv, cudaMemcpyDeviceToHost, c->stream));
  if (rm3) SOL_CUDA(cudaMemcpyAsync(rm3, c->d_rm3, sizeof(double) * c->n, cudaMemcpyDeviceToHost, c->stream));
  if (nn_idx)
    SOL_CUDA(cudaMemcpyAsync(nn_idx, c->d_nn_idx, sizeof(int32_t) * c->n, cudaMemcpyDeviceToHost, c->stream));
  if (nn_dist)
    SOL_CUDA(cudaMemcpyAsync(nn_dist, c->d_nn_dist, sizeof(double) * c->n, cudaMemcpyDeviceToHost, c->stream));
  SOL_CUDA(cudaMemcpyAsync(c->h_ctrl, c->d_ctrl, sizeof(sol_ctrl), cudaMemcpyDeviceToHost, c->stream));
  SOL_CUDA(cudaStreamSynchronize(c->stream));
  c->last_eval_valid = 1;
  if (c->h_ctrl->dev_status & SOL_DEV_TIMEOUT) {
    sol_set_error("a bounded device wait ran out in the force kernel");
    return SOL_ERR_TIMEOUT;
  }
  return SOL_OK;
}

int sol_get_mig_type(const sol_ctx* c, int32_t* mig_type) {
  RET(check_ctx(c));
  if (!mig_type) return SOL_ERR_ARG;
  RET(set_device(c));
  SOL_CUDA(cudaStreamSynchronize(c->stream));
  SOL_CUDA(cudaMemcpy(mig_type, c->d_mig_type, sizeof(int32_t) * c->n, cudaMemcpyDeviceToHost));
  return SOL_OK;
}

int sol_set_state(sol_ctx* c, const double* y0) {
  RET(check_ctx(c));
  if (!y0) return SOL_ERR_ARG;
  RET(set_device(c));
  SOL_CUDA(cudaMemcpyAsync(c->d_y0, y0, sizeof(double) * c->nv, cudaMemcpyHostToDevice, c->stream));
  SOL_CUDA(cudaStreamSynchronize(c->stream));
  c->state_valid = 1;
  return SOL_OK;
}

int sol_get_state(sol_ctx* c, double* y0) {
  RET(check_ctx(c));
  if (!y0) return SOL_ERR_ARG;
  RET(set_device(c));
  SOL_CUDA(cudaMemcpyAsync(y0, c->d_y0, sizeof(double) * c->nv, cudaMemcpyDeviceToHost, c->stream));
  SOL_CUDA(cudaStreamSynchronize(c->stream));
  return SOL_OK;
}

int sol_set_device_loop(sol_ctx* c, int32_t enable) {
  RET(check_ctx(c));
  c->device_loop = enable ? 1 : 0;
  return SOL_OK;
}

int sol_set_tolerance(sol_ctx* c, double eps) {
  RET(check_ctx(c));
  if (!(eps > 0)) {
    sol_set_error("tolerance must be positive");
    return SOL_ERR_ARG;
  }
  c->eps = eps;
  return SOL_OK;
}

int sol_driver(sol_ctx* c, int32_t integrator, sol_time_line* tl, int32_t n_steps, sol_step_stats* stats) {
  RET(check_ctx(c));
  if (!tl || n_steps < 0) {
    sol_set_error("bad driver arguments");
    return SOL_ERR_ARG;
  }
  if (!c->state_valid) {
    sol_set_error("no state: call sol_set_state first");
    return SOL_ERR_STATE;
  }
  RET(set_device(c));
  sol_ctrl h0;
  memset(&h0, 0, sizeof(h0));
  h0.t = tl->time;
  h0.h_next = tl->h_next;
  h0.h_did = tl->h_did;
  h0.h = tl->h_next;
  h0.eps = c->eps;
  SOL_CUDA(cudaMemcpyAsync(c->d_ctrl, &h0, sizeof(h0), cudaMemcpyHostToDevice, c->stream));
  c->graph_steps = 0;
  c->graph_used = 0;
  int rc = sol_integrator_run(c, integrator, n_steps);
  SOL_CUDA(cudaMemcpyAsync(c->h_ctrl, c->d_ctrl, sizeof(sol_ctrl), cudaMemcpyDeviceToHost, c->stream));
  SOL_CUDA(cudaStreamSynchronize(c->stream));
  const sol_ctrl& hc = *c->h_ctrl;
  if (c->graph_used) {
    const DriverGraph& G = c->graphs[c->graph_used - 1];
    const long long attempts = hc.n_accepted + hc.n_rejected;
    g_launches.fetch_add(c->graph_steps * (G.k_pro + G.k_epi) + attempts * G.k_body, std::memory_order_relaxed);
  }
  if (rc == SOL_OK) rc = [&]() {
    if (hc.dev_status & SOL_DEV_TIMEOUT) {
      sol_set_error("a bounded device wait ran out");
      return (int)SOL_ERR_TIMEOUT;
    }
    if (hc.dev_status & SOL_DEV_UNDERFLOW) {
      sol_set_error("Stepsize-underflow occurred during Runge-Kutta-Fehlberg7(8) step!");
      return (int)SOL_ERR_UNDERFLOW;
    }
    if (hc.dev_status & SOL_DEV_MAXITER) {
      sol_set_error("An error occurred during Prince-Dormand driver: iteration number exceeded maxIter!");
      return (int)SOL_ERR_MAXITER;
    }
    return (int)SOL_OK;
  }();
  tl->time = hc.t;
  tl->h_next = hc.h_next;
  tl->h_did = hc.h_did;
  if (stats) {
    stats->accepted += hc.n_accepted;
    stats->rejected += hc.n_rejected;
    const long long per = integrator == SOL_RUNGE_KUTTA_FEHLBERG78 ? 12 : integrator == SOL_DORMAND_PRINCE ? 8 : 3;
    stats->evaluations += hc.n_accepted * (per + 1) + hc.n_rejected * per;
  }
  c->last_eval_valid = 1;
  if (rc == SOL_OK && (hc.dev_status & SOL_DEV_TIMEOUT)) {
    sol_set_error("a bounded device wait ran out");
    return SOL_ERR_TIMEOUT;
  }
  return rc;
}

int sol_driver_host(sol_ctx* c, int32_t integrator, double* y0, sol_time_line* tl, int32_t n_steps,
                    sol_step_stats* stats) {
  RET(sol_set_state(c, y0));
  int rc = sol_driver(c, integrator, tl, n_steps, stats);
  int rc2 = sol_get_state(c, y0);
  return rc != SOL_OK ? rc : rc2;
}

int sol_rkf78_step(sol_ctx* c, double t, double h, const double* y0, double* y, double* error, double* error_max) {
  RET(check_ctx(c));
  if (!y0 || !y) return SOL_ERR_ARG;
  RET(set_device(c));
  SOL_CUDA(cudaMemcpyAsync(c->d_io_in, y0, sizeof(double) * c->nv, cudaMemcpyHostToDevice, c->stream));
  double em = 0.0;
  RET(sol_rkf78_single_attempt(c, t, h, c->d_io_in, c->d_io_out, c->d_err, &em));
  SOL_CUDA(cudaMemcpyAsync(y, c->d_io_out, sizeof(double) * c->nv, cudaMemcpyDeviceToHost, c->stream));
  if (error) SOL_CUDA(cudaMemcpyAsync(error, c->d_err, sizeof(double) * c->nv, cudaMemcpyDeviceToHost, c->stream));
  SOL_CUDA(cudaStreamSynchronize(c->stream));
  if (error_max) *error_max = em;
  c->last_eval_valid = 1;
  return SOL_OK;
}

int sol_get_last_eval(sol_ctx* c, double* rm3, int32_t* nn_idx, double* nn_dist) {
  RET(check_ctx(c));
  RET(set_device(c));
  SOL_CUDA(cudaStreamSynchronize(c->stream));
  if (rm3) SOL_CUDA(cudaMemcpy(rm3, c->d_rm3, sizeof(double) * c->n, cudaMemcpyDeviceToHost));
  if (nn_idx) SOL_CUDA(cudaMemcpy(nn_idx, c->d_nn_idx, sizeof(int32_t) * c->n, cudaMemcpyDeviceToHost));
  if (nn_dist) SOL_CUDA(cudaMemcpy(nn_dist, c->d_nn_dist, sizeof(double) * c->n, cudaMemcpyDeviceToHost));
  return SOL_OK;
}

namespace {

constexpr double kSmallestNumber = 1.0e-50;  // Solaris/Constants.h:17
constexpr long long kCheckForSm = 100;       // Solaris/Constants.h:16

__global__ void k_flush_smallest(int nv, double* __restrict__ y) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nv; e += gridDim.x * blockDim.x)
    if (fabs(y[e]) < kSmallestNumber) y[e] = 0.0;
}

int flush_launch(sol_ctx* c) {
  const int g = std::min((c->nv + 255) / 256, 1024);
  k_flush_smallest<<<g, 256, 0, c->stream>>>(c->nv, c->d_y0);
  SOL_LAUNCHED();
  return SOL_OK;
}

// Whether an event predicate of CheckEvent holds on the last evaluation.
int events_pending(sol_ctx* c, double ej, double hc, double cf, bool* pending) {
  *pending = false;
  if (!(ej > 0.0) && !(hc > 0.0) && !(cf > 0.0)) return SOL_OK;
  int* d_cnt = static_cast<int*>(c->d_sim);
  RET(sol_events_launch(c, c->d_y0, ej, hc, cf, nullptr, 0, d_cnt));
  int cnt = 0;
  SOL_CUDA(cudaMemcpyAsync(&cnt, d_cnt, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  SOL_CUDA(cudaStreamSynchronize(c->stream));
  *pending = cnt > 0;
  return SOL_OK;
}

// sol_sim_line + stop reason + event flags of the group driver
constexpr size_t kSimBytes = 256 + sizeof(int) * 2 * kGroupMaxCtas;

int ensure_sim(sol_ctx* c) {
  if (!c->d_sim) {
    if (cudaMalloc(&c->d_sim, kSimBytes) != cudaSuccess) {
      sol_set_error("cudaMalloc of the step-loop scratch failed");
      return SOL_ERR_NOMEM;
    }
    SOL_CUDA(cudaMemset(c->d_sim, 0, kSimBytes));
  }
  if (!c->d_ystart) {  // bodies are only ever removed: the first size holds
    if (cudaMalloc((void**)&c->d_ystart, sizeof(double) * (size_t)c->nv) != cudaSuccess) {
      sol_set_error("cudaMalloc of the step-start state failed");
      return SOL_ERR_NOMEM;
    }
  }
  return SOL_OK;
}

}  // namespace

int sol_get_step_start(sol_ctx* c, double* y) {
  RET(check_ctx(c));
  if (!y || !c->d_ystart) {
    sol_set_error("sol_get_step_start: no step loop with collisions has run");
    return SOL_ERR_STATE;
  }
  RET(set_device(c));
  SOL_CUDA(cudaMemcpyAsync(y, c->d_ystart, sizeof(double) * (size_t)c->nv, cudaMemcpyDeviceToHost, c->stream));
  SOL_CUDA(cudaStreamSynchronize(c->stream));
  return SOL_OK;
}

int sol_flush_smallest(sol_ctx* c) {
  RET(check_ctx(c));
  if (!c->state_valid) {
    sol_set_error("no state: call sol_set_state first");
    return SOL_ERR_STATE;
  }
  RET(set_device(c));
  RET(flush_launch(c));
  SOL_CUDA(cudaStreamSynchronize(c->stream));
  return SOL_OK;
}

int sol_run_until(sol_ctx* c, int32_t integrator, sol_sim_line* L, int32_t max_steps, double ejection,
                  double hit_centrum, double collision_factor, int32_t* reason, sol_step_stats* stats) {
  RET(check_ctx(c));
  if (!L || !reason || max_steps < 1) {
    sol_set_error("sol_run_until: bad arguments");
    return SOL_ERR_ARG;
  }
  if (!c->state_valid) {
    sol_set_error("no state: call sol_set_state first");
    return SOL_ERR_STATE;
  }
  RET(set_device(c));
  RET(ensure_sim(c));
  const double e3 = ejection > 0 ? 1.0 / (ejection * ejection * ejection) : 0.0;
  const double h3 = hit_centrum > 0 ? 1.0 / (hit_centrum * hit_centrum * hit_centrum) : 0.0;
  // the whole loop on the device: RKF78 and RK4 systems of few sources
  const bool rk4 = integrator == SOL_RUNGE_KUTTA4;
  if ((integrator == SOL_RUNGE_KUTTA_FEHLBERG78 || rk4) && c->device_loop && sol_group_eligible(c)) {
    char* base = static_cast<char*>(c->d_sim);
    GroupSim sim;
    sim.e3 = e3;
    sim.h3 = h3;
    sim.cf = collision_factor > 0 ? collision_factor : 0.0;
    sim.line = reinterpret_cast<sol_sim_line*>(base);
    sim.reason = reinterpret_cast<int*>(base + 128);
    sim.ev = reinterpret_cast<int*>(base + 256);
    sim.yprev = collision_factor > 0 ? c->d_ystart : nullptr;
    sol_ctrl h0;
    memset(&h0, 0, sizeof(h0));
    h0.t = L->time;
    h0.h_next = L->h_next;
    h0.h_did = L->h_did;
    h0.h = L->h_next;
    h0.eps = c->eps;
    const int stop_steps = SOL_STOP_STEPS;
    SOL_CUDA(cudaMemcpyAsync(c->d_ctrl, &h0, sizeof(h0), cudaMemcpyHostToDevice, c->stream));
    SOL_CUDA(cudaMemcpyAsync(sim.line, L, sizeof(*L), cudaMemcpyHostToDevice, c->stream));
    SOL_CUDA(cudaMemcpyAsync(sim.reason, &stop_steps, sizeof(int), cudaMemcpyHostToDevice, c->stream));
    const int r = sol_group_rkf78(c, max_steps, &sim, rk4);
    if (r != SOL_ERR_STATE) {
      if (r != SOL_OK) return r;
      SOL_CUDA(cudaMemcpyAsync(c->h_ctrl, c->d_ctrl, sizeof(sol_ctrl), cudaMemcpyDeviceToHost, c->stream));
      SOL_CUDA(cudaMemcpyAsync(L, sim.line, sizeof(*L), cudaMemcpyDeviceToHost, c->stream));
      SOL_CUDA(cudaMemcpyAsync(reason, sim.reason, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
      SOL_CUDA(cudaStreamSynchronize(c->stream));
      const sol_ctrl& hc = *c->h_ctrl;
      c->last_eval_valid = 1;
      if (stats) {
        stats->accepted += hc.n_accepted;
        stats->rejected += hc.n_rejected;
        stats->evaluations += rk4 ? hc.n_accepted * 4 : hc.n_accepted * 13 + hc.n_rejected * 12;
      }
      if (hc.dev_status & SOL_DEV_TIMEOUT) {
        sol_set_error("a bounded device wait ran out");
        return SOL_ERR_TIMEOUT;
      }
      if (hc.dev_status & SOL_DEV_UNDERFLOW) {
        sol_set_error("Stepsize-underflow occurred during Runge-Kutta-Fehlberg7(8) step!");
        return SOL_ERR_UNDERFLOW;
      }
      return SOL_OK;
    }
  }
  // any other integrator or path: the same loop on the host, one driver call per step
  for (int k = 0; k < max_steps; ++k) {
    if (collision_factor > 0)
      SOL_CUDA(cudaMemcpyAsync(c->d_ystart, c->d_y0, sizeof(double) * (size_t)c->nv, cudaMemcpyDeviceToDevice,
                               c->stream));
    sol_time_line tl = {L->time, L->h_next, L->h_did};
    RET(sol_driver(c, integrator, &tl, 1, stats));
    L->time = tl.time;
    L->h_next = tl.h_next;
    L->h_did = tl.h_did;
    L->steps += 1;
    L->elapsed += L->h_did;
    L->last_save += L->h_did;
    bool pending = false;
    RET(events_pending(c, ejection, hit_centrum, collision_factor, &pending));
    if (pending) {
      *reason = SOL_STOP_EVENT;
      return SOL_OK;
    }
    const double clock = L->relative_end ? L->elapsed : L->time;
    if (fabs(clock) >= fabs(L->length)) {
      *reason = SOL_STOP_LENGTH;
      return SOL_OK;
    }
    if (fabs(clock + L->h_next) > fabs(L->length)) L->h_next = L->length - clock;
    if (fabs(L->last_save) >= fabs(L->output)) {
      *reason = SOL_STOP_OUTPUT;
      return SOL_OK;
    }
    if (fabs(L->last_save + L->h_next) > fabs(L->output)) L->h_next = L->output - L->last_save;
    if (L->steps % kCheckForSm == 0) {
      RET(flush_launch(c));
    }
  }
  SOL_CUDA(cudaStreamSynchronize(c->stream));
  *reason = SOL_STOP_STEPS;
  return SOL_OK;
}

int sol_check_events(sol_ctx* c, double ejection, double hit_centrum, double collision_factor, sol_event* out,
                     int32_t capacity, int32_t* n_out) {
  RET(check_ctx(c));
  if (!n_out || capacity < 0 || (capacity > 0 && !out)) return SOL_ERR_ARG;
  RET(set_device(c));
  // predicates read the state the events are reported at (the accepted y0)
  sol_event* d_ev = nullptr;
  int* d_cnt = nullptr;
  const int cap = capacity > 0 ? capacity : 1;
  SOL_CUDA(cudaMallocAsync((void**)&d_ev, sizeof(sol_event) * cap, c->stream));
  SOL_CUDA(cudaMallocAsync((void**)&d_cnt, sizeof(int), c->stream));
  int rc = sol_events_launch(c, c->d_y0, ejection, hit_centrum, collision_factor, d_ev, capacity, d_cnt);
  int cnt = 0;
  std::vector<sol_event> tmp(cap);
  if (rc == SOL_OK) {
    SOL_CUDA(cudaMemcpyAsync(&cnt, d_cnt, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    SOL_CUDA(cudaMemcpyAsync(tmp.data(), d_ev, sizeof(sol_event) * cap, cudaMemcpyDeviceToHost, c->stream));
  }
  cudaFreeAsync(d_ev, c->stream);
  cudaFreeAsync(d_cnt, c->stream);
  SOL_CUDA(cudaStreamSynchronize(c->stream));
  if (rc != SOL_OK) return rc;
  const int m = std::min(cnt, capacity);
  // the order in which Simulator::CheckEvent visits bodies: ejection and
  // hit-centrum by body index, then collisions by body index
  std::sort(tmp.begin(), tmp.begin() + m, [](const sol_event& a, const sol_event& b) {
    int pa = a.kind == SOL_EVENT_COLLISION, pb = b.kind == SOL_EVENT_COLLISION;
    if (pa != pb) return pa < pb;
    int ia = pa ? a.idx1 : a.idx2, ib = pb ? b.idx1 : b.idx2;
    if (ia != ib) return ia < ib;
    return a.kind < b.kind;
  });
  for (int q = 0; q < m; ++q) out[q] = tmp[q];
  *n_out = cnt;
  return SOL_OK;
}

constexpr int kExactPotentialMax = 1024;

int sol_integrals(sol_ctx* c, const double* y0_or_null, double o[16]) {
  RET(check_ctx(c));
  if (!o) return SOL_ERR_ARG;
  RET(set_device(c));
  const int N = c->n;
  std::vector<double> y(c->nv), mass(N), pe(N);
  const double* d_y = c->d_y0;
  if (y0_or_null) {
    SOL_CUDA(cudaMemcpyAsync(c->d_io_in, y0_or_null, sizeof(double) * c->nv, cudaMemcpyHostToDevice, c->stream));
    d_y = c->d_io_in;
  }
  // Calculate::PotentialEnergy (Calculate.cpp:139-159) adds every ordered
  // pair into one running sum.  Up to kExactPotentialMax bodies (scenario
  // sizes, ~1 M pairs at most) that sum runs here in the reference's order,
  // bit for bit; above, the device sums each unordered pair once into
  // per-CTA partials (k_potential_pairs) and the host adds those in order.
  const bool exact_order = N <= kExactPotentialMax;
  int nparts = 0;
  if (!exact_order) {
    RET(sol_potential_launch(c, d_y, c->d_io_out, &nparts));
    SOL_CUDA(cudaMemcpyAsync(pe.data(), c->d_io_out, sizeof(double) * nparts, cudaMemcpyDeviceToHost, c->stream));
  }
  SOL_CUDA(cudaMemcpyAsync(y.data(), d_y, sizeof(double) * c->nv, cudaMemcpyDeviceToHost, c->stream));
  SOL_CUDA(cudaMemcpyAsync(mass.data(), c->d_mass, sizeof(double) * N, cudaMemcpyDeviceToHost, c->stream));
  SOL_CUDA(cudaStreamSynchronize(c->stream));
  // O(N) parts of Calculate::Integrals (Solaris/Calculate.cpp:43-172)
  const int nm = c->cls.nm;
  double M = 0.0;
  for (int i = 0; i < nm; i++) M += mass[i];
  o[0] = M;
  double bc[6] = {0, 0, 0, 0, 0, 0};
  for (int i = 0; i < N; i++)
    for (int j = 0; j < 6; j++) bc[j] += mass[i] * y[6 * i + j];
  for (int j = 0; j < 6; j++) o[1 + j] = bc[j] / M;
  o[7] = sqrt(o[1] * o[1] + o[2] * o[2] + o[3] * o[3]);
  o[8] = sqrt(o[4] * o[4] + o[5] * o[5] + o[6] * o[6]);
  double cx = 0, cy = 0, cz = 0;
  for (int i = 0; i < N; i++) {
    const double* p = &y[6 * i];
    double m = mass[i];
    cx += m * (p[1] * p[5] - p[2] * p[4]);
    cy += m * (p[2] * p[3] - p[0] * p[5]);
    cz += m * (p[0] * p[4] - p[1] * p[3]);
  }
  o[9] = cx;
  o[10] = cy;
  o[11] = cz;
  o[12] = sqrt(cx * cx + cy * cy + cz * cz);
  double ke = 0.0;
  for (int i = 0; i < N; i++) {
    const double* p = &y[6 * i];
    ke += 0.5 * mass[i] * (p[3] * p[3] + p[4] * p[4] + p[5] * p[5]);
  }
  o[13] = ke;
  double pes = 0.0;
  if (exact_order) {
    for (int i = 0; i < N; i++) {
      const double* pi = &y[6 * i];
      for (int j = 0; j < N; j++) {
        if (i == j) continue;
        const double* pj = &y[6 * j];
        const double dx = pj[0] - pi[0];
        const double dy = pj[1] - pi[1];
        const double dz = pj[2] - pi[2];
        const double rij = sqrt(dx * dx + dy * dy + dz * dz);
        pes += mass[i] * mass[j] / rij;
      }
    }
  } else {
    double unordered = 0.0;
    for (int b = 0; b < nparts; b++) unordered += pe[b];
    pes = 2.0 * unordered;
  }
  o[14] = pes * (0.5 * 2.959122082855911025e-4);
  o[15] = o[13] - o[14];
  return SOL_OK;
}

int sol_get_stream(sol_ctx* c, void** stream) {
  RET(check_ctx(c));
  if (!stream) return SOL_ERR_ARG;
  *stream = (void*)c->stream;
  return SOL_OK;
}

int sol_bench_stages(sol_ctx* c, int32_t reps, double* ms_per_attempt) {
  RET(check_ctx(c));
  if (!ms_per_attempt || reps < 1) return SOL_ERR_ARG;
  RET(set_device(c));
  return sol_bench_stage_kernels(c, reps, ms_per_attempt);
}

int sol_bench_force(sol_ctx* c, int32_t precision, int32_t reps, double* ms_per_launch) {
  RET(check_ctx(c));
  if (!ms_per_launch || reps < 1) return SOL_ERR_ARG;
  if (!c->state_valid) {
    sol_set_error("no state: call sol_set_state first");
    return SOL_ERR_STATE;
  }
  RET(set_device(c));
  const int saved = c->precision;
  RET(sol_set_precision(c, precision));
  TimeSpec ts{nullptr, nullptr, 0.0, 0.0};
  int rc = sol_force_launch_parts(c, c->d_y0, c->d_io_out, ts, SOL_EVAL_GAS_DRAG, 3);  // warm-up, sources
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (rc == SOL_OK && (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)) rc = SOL_ERR_CUDA;
  if (rc == SOL_OK && cudaEventRecord(e0, c->stream) != cudaSuccess) rc = SOL_ERR_CUDA;
  for (int r = 0; r < reps && rc == SOL_OK; ++r)
    rc = sol_force_launch_parts(c, c->d_y0, c->d_io_out, ts, SOL_EVAL_GAS_DRAG, 2);
  if (rc == SOL_OK && cudaEventRecord(e1, c->stream) != cudaSuccess) rc = SOL_ERR_CUDA;
  float ms = 0.0f;
  if (rc == SOL_OK && (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess))
    rc = SOL_ERR_CUDA;
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  c->precision = saved;
  c->fc.precision = saved;
  if (rc != SOL_OK) {
    if (rc == SOL_ERR_CUDA) sol_set_error("CUDA event timing failed");
    return rc;
  }
  *ms_per_launch = (double)ms / reps;
  return SOL_OK;
}

int sol_measure_fp64_peak(int32_t device, double* flops) {
  if (!flops) return SOL_ERR_ARG;
  return sol_fp64_peak_launch(device, flops);
}

int sol_accel_sinks_device(sol_ctx* c, double t, const double* d_y, int32_t sink_begin, int32_t sink_end,
                           double* d_dydt) {
  RET(check_ctx(c));
  if (!d_y || !d_dydt || sink_begin < 0 || sink_end < sink_begin || sink_end > c->n) {
    sol_set_error("sol_accel_sinks_device: bad arguments (sinks [%d, %d) of %d bodies)", sink_begin, sink_end, c->n);
    return SOL_ERR_ARG;
  }
  if (c->barycentric) {
    sol_set_error("sol_accel_sinks_device: heliocentric contexts only");
    return SOL_ERR_ARG;
  }
  RET(set_device(c));
  TimeSpec ts{nullptr, nullptr, 0.0, t};
  RET(sol_force_launch_sinks(c, d_y, d_dydt, ts, c->eval_flags, sink_begin, sink_end));
  c->last_eval_valid = 1;
  return SOL_OK;
}

int sol_set_wait_test(sol_ctx* c, uint32_t spin_limit, int32_t withhold) {
  if (withhold < -1) {
    sol_set_error("sol_set_wait_test: withhold must be -1 (none) or an index");
    return SOL_ERR_ARG;
  }
  if (!c) {
    sol_noalloc_wait_test(spin_limit, withhold);
    return SOL_OK;
  }
  c->test_spin = spin_limit;
  c->test_skip_cta = withhold;
  return SOL_OK;
}

int sol_measure_fp32_pipe(int32_t device, double rates[2], double* sm_mhz) {
  if (!rates) return SOL_ERR_ARG;
  return sol_fp32_rates_launch(device, rates, sm_mhz);
}

int sol_measure_fp64_pipe(int32_t device, double rates[3], double* sm_mhz) {
  if (!rates) return SOL_ERR_ARG;
  return sol_fp64_rates_launch(device, rates, sm_mhz);
}

int sol_check_pair_math(int32_t device, int32_t mode, int64_t n, uint64_t seed, int64_t result[3]) {
  if (!result || mode < 0 || mode > 9 || n < 0) return SOL_ERR_ARG;
  long long r[3];
  RET(sol_check_pair_math_launch(device, mode, (long long)n, (unsigned long long)seed, r));
  for (int k = 0; k < 3; ++k) result[k] = r[k];
  return SOL_OK;
}

}  // extern "C"
