// Batched ensembles: thousands of independent systems of uneven size, each
// integrated with its own adaptive RungeKuttaFehlberg78 step
// (Solaris/RungeKuttaFehlberg78.cpp:66-262) and GravityAC force
// (Solaris/Acceleration.cpp:248-329), in one persistent launch.
//
// Each CTA takes a system from an atomic work queue (systems sorted largest
// first) and runs n driver calls for it: first evaluation, yscale, attempts of
// 12 stage sums and 12 evaluations, the final sum, the error norm and the
// step control, all with block barriers only.  Stage vectors live in a
// per-CTA scratch slot in global memory (L2-resident while the CTA works on
// the system); the source table of an evaluation lives in shared memory.
// FP64 mode follows the reference's operation order exactly, so each system
// evolves as the single-system path (and the reference) would.
#include <atomic>
#include <mutex>
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "sol_internal.cuh"
#include "sol_crmath.cuh"

namespace {

struct EnsSys {
  int off;     // first body in the concatenated arrays
  int n;       // bodies
  int nm;      // NOfMassive
  int ns_max;  // sources of massive sinks: nm + super-planetesimals
};

struct EnsCtrl {
  double t, h, h_next, h_did, error_max;
  int status, accepted;
  long long n_acc, n_rej;
};

constexpr int kVecs = 17;  // f0..f12, yscale, ytmp, y, error
enum { V_YSCALE = 13, V_YTMP = 14, V_Y = 15, V_ERR = 16 };

// RKF78 tableau in the reference's summation order (RungeKuttaFehlberg78.cpp:41-56, :169-232)
__constant__ int c_rk_k[13];
__constant__ int c_rk_idx[13][9];
__constant__ double c_rk_a[13][9];

__device__ __forceinline__ double block_max(double v, double* red) {
  // NaN entries never replace the maximum, as GetErrorMax
  const int tid = threadIdx.x;
  red[tid] = v;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (tid < w) {
      double o = red[tid + w];
      if (o > red[tid]) red[tid] = o;
    }
    __syncthreads();
  }
  double r = red[0];
  __syncthreads();
  return r;
}

// GravityAC for one system by one CTA.  FP64: the reference's loops and
// operation order.  SPLIT_FF: float-float pairs with the indirect term summed
// once per evaluation.
template <int PREC>
__device__ void ens_force(const EnsSys& S, const double* __restrict__ m, const double* __restrict__ yin,
                          double* __restrict__ fout, double* __restrict__ rm3, double* __restrict__ tab, int ns_cap,
                          double* red) {
  const int tid = threadIdx.x, bd = blockDim.x;
  const int n = S.n;
  for (int i = tid; i < n; i += bd) {
    if (i >= 1) {
      const double x = yin[6 * i], y = yin[6 * i + 1], z = yin[6 * i + 2];
      const double r2 = x * x + y * y + z * z;
      double r, rm3i;
      sol_ref_rinv3(r2, r, rm3i);
      rm3[i] = rm3i;
    } else {
      rm3[0] = 0.0;
    }
  }
  __syncthreads();
  // source table: x, y, z, G m, x rm3, y rm3, z rm3 (FP64) / x, y, z, (G m hi, lo) (SPLIT_FF)
  double* tx = tab;
  double* ty = tab + ns_cap;
  double* tz = tab + 2 * ns_cap;
  double* tg = tab + 3 * ns_cap;
  double* tpx = tab + 4 * ns_cap;
  double* tpy = tab + 5 * ns_cap;
  double* tpz = tab + 6 * ns_cap;
  for (int j = tid; j < S.ns_max; j += bd) {
    const double x = yin[6 * j], y = yin[6 * j + 1], z = yin[6 * j + 2];
    const double gm = j >= 1 ? SOL_GAUSS2 * m[j] : 0.0;
    tx[j] = x;
    ty[j] = y;
    tz[j] = z;
    if constexpr (PREC == SOL_PRECISION_FP64) {
      tg[j] = gm;
      tpx[j] = x * rm3[j];
      tpy[j] = y * rm3[j];
      tpz[j] = z * rm3[j];
    } else {
      const float gh = __double2float_rn(gm);
      reinterpret_cast<float2*>(tg)[j] = make_float2(gh, __double2float_rn(gm - (double)gh));
      tpx[j] = gm * (x * rm3[j]);  // indirect contributions q_j
      tpy[j] = gm * (y * rm3[j]);
      tpz[j] = gm * (z * rm3[j]);
    }
  }
  __syncthreads();
  double ind_m[3] = {0, 0, 0}, ind_all[3] = {0, 0, 0};
  if constexpr (PREC != SOL_PRECISION_FP64) {
    // indirect-term totals over [1, nm) and [1, ns_max): one warp, fixed order
    if (tid < 32) {
      double a[6] = {0, 0, 0, 0, 0, 0};
      for (int j = 1 + tid; j < S.ns_max; j += 32) {
        const int o = j < S.nm ? 0 : 3;
        a[o] += tpx[j];
        a[o + 1] += tpy[j];
        a[o + 2] += tpz[j];
      }
#pragma unroll
      for (int k = 0; k < 6; ++k)
        for (int w = 16; w > 0; w >>= 1) a[k] += __shfl_down_sync(0xffffffffu, a[k], w);
      if (tid == 0)
        for (int k = 0; k < 6; ++k) red[k] = a[k];
    }
    __syncthreads();
    for (int k = 0; k < 3; ++k) {
      ind_m[k] = red[k];
      ind_all[k] = red[k] + red[3 + k];
    }
    __syncthreads();
  }
  for (int i = tid; i < n; i += bd) {
    double* out = fout + 6 * i;
    if (i == 0) {
      for (int k = 0; k < 6; ++k) out[k] = 0.0;
      continue;
    }
    const double xi = yin[6 * i], yi = yin[6 * i + 1], zi = yin[6 * i + 2];
    const int ns = i < S.nm ? S.ns_max : S.nm;
    const double mu = SOL_GAUSS2 * (m[0] + m[i]);
    double a0 = -mu * rm3[i] * xi, a1 = -mu * rm3[i] * yi, a2 = -mu * rm3[i] * zi;
    if constexpr (PREC == SOL_PRECISION_FP64) {
      double ax = 0.0, ay = 0.0, az = 0.0;
      // two sources per step (independent chains that interleave), added in
      // ascending order; an odd last source pairs with itself
      for (int j = 1; j < ns; j += 2) {
        const int jb[2] = {j, min(j + 1, ns - 1)};
        double xij[2], yij[2], zij[2], rij2[2];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          xij[u] = tx[jb[u]] - xi;
          yij[u] = ty[jb[u]] - yi;
          zij[u] = tz[jb[u]] - zi;
          const double q = xij[u] * xij[u] + yij[u] * yij[u] + zij[u] * zij[u];
          rij2[u] = jb[u] != i ? q : 1.0;
        }
        double rij[2], rijm3[2];
        sol_ref_rinv3_x2(rij2[0], rij2[1], rij[0], rijm3[0], rij[1], rijm3[1]);
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          double t0, t1, t2;
          const int q = jb[u];
          sol_ref_terms(tg[q], rijm3[u], xij[u], yij[u], zij[u], tpx[q], tpy[q], tpz[q], t0, t1, t2);
          if (q != i && (u == 0 || jb[1] != jb[0])) {
            ax += t0;
            ay += t1;
            az += t2;
          }
        }
      }
      a0 += ax;
      a1 += ay;
      a2 += az;
    } else {
      FFAcc A;
      for (int k = 0; k < 3; ++k) A.h[k] = A.l[k] = 0.0f;
      double fbx = 0.0, fby = 0.0, fbz = 0.0;
      float r2h, r2l;
      const float2* tg2 = reinterpret_cast<const float2*>(tg);
      for (int j = 1; j < ns; j++)
        ff_pair_accumulate(tx[j] - xi, ty[j] - yi, tz[j] - zi, tg2[j], A, fbx, fby, fbz, r2h, r2l);
      const double* ind = i < S.nm ? ind_all : ind_m;
      const double own0 = i < ns ? tpx[i] : 0.0, own1 = i < ns ? tpy[i] : 0.0, own2 = i < ns ? tpz[i] : 0.0;
      a0 += (((double)A.h[0] + (double)A.l[0]) + fbx) - (ind[0] - own0);
      a1 += (((double)A.h[1] + (double)A.l[1]) + fby) - (ind[1] - own1);
      a2 += (((double)A.h[2] + (double)A.l[2]) + fbz) - (ind[2] - own2);
    }
    out[0] = yin[6 * i + 3];
    out[1] = yin[6 * i + 4];
    out[2] = yin[6 * i + 5];
    out[3] = a0;
    out[4] = a1;
    out[5] = a2;
  }
  __syncthreads();
}

template <int PREC>
__global__ void k_ensemble_rkf78(const EnsSys* __restrict__ systems, const int* __restrict__ order,
                                 EnsCtrl* __restrict__ ctrl, double* __restrict__ y0_all,
                                 const double* __restrict__ mass_all, double* __restrict__ scratch,
                                 size_t slot_doubles, int max_nv, int ns_cap, int* queue, int n_sys, int n_steps,
                                 double eps) {
  extern __shared__ __align__(16) double tab[];  // source table, 7 x ns_cap doubles
  __shared__ double red[1024];
  __shared__ int s_sys;
  __shared__ EnsCtrl C;
  const int tid = threadIdx.x, bd = blockDim.x;
  double* slot = scratch + (size_t)blockIdx.x * slot_doubles;
  double* f[13];
  for (int k = 0; k < 13; ++k) f[k] = slot + (size_t)k * max_nv;
  double* yscale = slot + (size_t)V_YSCALE * max_nv;
  double* ytmp = slot + (size_t)V_YTMP * max_nv;
  double* ynew = slot + (size_t)V_Y * max_nv;
  double* err = slot + (size_t)V_ERR * max_nv;
  double* rm3 = slot + (size_t)kVecs * max_nv;
  for (;;) {
    if (tid == 0) s_sys = atomicAdd(queue, 1);
    __syncthreads();
    const int q = s_sys;
    if (q >= n_sys) return;
    const int si = order[q];
    const EnsSys S = systems[si];
    double* y0 = y0_all + 6 * (size_t)S.off;
    const double* m = mass_all + S.off;
    const int nv = 6 * S.n;
    if (tid == 0) C = ctrl[si];
    __syncthreads();
    for (int step = 0; step < n_steps; ++step) {
      if (C.status) break;
      __syncthreads();
      if (tid == 0) {  // Driver: bodyData->h = timeLine->hNext
        C.h = C.h_next;
        C.accepted = 0;
      }
      __syncthreads();
      ens_force<PREC>(S, m, y0, f[0], rm3, tab, ns_cap, red);
      {
        const double h = C.h;
        for (int e = tid; e < nv; e += bd) yscale[e] = fabs(y0[e]) + fabs(h * f[0][e]) + 1.0e-30;
      }
      __syncthreads();
      for (;;) {
        const double h = C.h;
        for (int r = 1; r <= 12; ++r) {
          const int K = c_rk_k[r];
          for (int e = tid; e < nv; e += bd) {
            double acc = c_rk_a[r][0] * slot[(size_t)c_rk_idx[r][0] * max_nv + e];
            for (int k = 1; k < K; ++k) acc = acc + c_rk_a[r][k] * slot[(size_t)c_rk_idx[r][k] * max_nv + e];
            ytmp[e] = y0[e] + h * acc;
          }
          __syncthreads();
          ens_force<PREC>(S, m, ytmp, f[r], rm3, tab, ns_cap, red);
        }
        double mx = 0.0;
        const double D1_0 = 41.0 / 840.0, D1_5 = 34.0 / 105.0, D1_6 = 9.0 / 35.0, D1_8 = 9.0 / 280.0,
                     D1_10 = 41.0 / 840.0;
        for (int e = tid; e < nv; e += bd) {
          const double f0 = f[0][e], f10 = f[10][e];
          ynew[e] = y0[e] + h * (D1_0 * f0 + D1_5 * f[5][e] + D1_6 * (f[6][e] + f[7][e]) +
                                 D1_8 * (f[8][e] + f[9][e]) + D1_10 * f10);
          const double ee = h * fabs(f0 + f10 - f[11][e] - f[12][e]) * 41.0 / 840.0;
          err[e] = ee;
          const double qq = fabs(ee / yscale[e]);
          mx = qq > mx ? qq : mx;
        }
        mx = block_max(mx, red);
        if (tid == 0) {  // step-size control (RungeKuttaFehlberg78.cpp:98-133)
          const double em = mx / eps;
          C.error_max = em;
          if (em < 1.0) {
            C.h_did = h;
            C.t += C.h_did;
            C.h_next = em > 1.89e-4 ? (0.9 * h * sol_inv_root<5>(em)) : (5.0 * h);
            C.h = C.h_next;
            C.accepted = 1;
            C.n_acc++;
          } else {
            C.n_rej++;
            double hTemp = 0.9 * h * sol_inv_root<4>(em);
            double hn = fabs(hTemp) > fabs(0.1 * h) ? hTemp : 0.1 * h;
            C.h = hn;
            if (C.t + hn == C.t) C.status = SOL_ERR_UNDERFLOW;
          }
        }
        __syncthreads();
        if (C.accepted || C.status) break;
      }
      if (C.accepted)
        for (int e = tid; e < nv; e += bd) y0[e] = ynew[e];
      __syncthreads();
    }
    if (tid == 0) ctrl[si] = C;
    __syncthreads();
  }
}

template <int PREC>
int launch_ensemble(int grid, int block, size_t smem, cudaStream_t st, const EnsSys* sys, const int* order,
                    EnsCtrl* ctrl, double* y0, const double* mass, double* scratch, size_t slot, int max_nv,
                    int ns_cap, int* queue, int n_sys, int n_steps, double eps) {
  if (smem > 48 * 1024)
    SOL_CUDA(cudaFuncSetAttribute(k_ensemble_rkf78<PREC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k_ensemble_rkf78<PREC><<<grid, block, smem, st>>>(sys, order, ctrl, y0, mass, scratch, slot, max_nv, ns_cap, queue,
                                                    n_sys, n_steps, eps);
  SOL_LAUNCHED();
  return SOL_OK;
}

int upload_tableau() {
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
  auto set = [&](int r, std::initializer_list<int> ix, std::initializer_list<double> co) {
    k[r] = (int)ix.size();
    int p = 0;
    for (int v : ix) idx[r][p++] = v;
    p = 0;
    for (double v : co) a[r][p++] = v;
  };
  set(1, {0}, {2.0 / 27.0});
  set(2, {0, 1}, {1.0 / 36.0, 1.0 / 12.0});
  set(3, {0, 2}, {1.0 / 24.0, 1.0 / 8.0});
  set(4, {0, 2, 3}, {5.0 / 12.0, -25.0 / 16.0, 25.0 / 16.0});
  set(5, {0, 3, 4}, {1.0 / 20.0, 1.0 / 4.0, 1.0 / 5.0});
  set(6, {0, 3, 4, 5}, {-25.0 / 108.0, 125.0 / 108.0, -65.0 / 27.0, 125.0 / 54.0});
  set(7, {0, 4, 5, 6}, {31.0 / 300.0, 61.0 / 225.0, -2.0 / 9.0, 13.0 / 900.0});
  set(8, {0, 3, 4, 5, 6, 7}, {2.0, -53.0 / 6.0, 704.0 / 45.0, -107.0 / 9.0, 67.0 / 90.0, 3.0});
  set(9, {0, 3, 4, 5, 6, 7, 8},
      {-91.0 / 108.0, 23.0 / 108.0, -976.0 / 135.0, 311.0 / 54.0, -19.0 / 60.0, 17.0 / 6.0, -1.0 / 12.0});
  set(10, {0, 3, 4, 5, 6, 7, 8, 9},
      {2383.0 / 4100.0, -341.0 / 164.0, 4496.0 / 1025.0, -301.0 / 82.0, 2133.0 / 4100.0, 45.0 / 82.0, 45.0 / 164.0,
       18.0 / 41.0});
  set(11, {0, 5, 6, 7, 8, 9}, {3.0 / 205.0, -6.0 / 41.0, -3.0 / 205.0, -3.0 / 41.0, 3.0 / 41.0, 6.0 / 41.0});
  set(12, {0, 3, 4, 5, 6, 7, 8, 9, 11},
      {-1777.0 / 4100.0, -341.0 / 164.0, 4496.0 / 1025.0, -289.0 / 82.0, 2193.0 / 4100.0, 51.0 / 82.0,
       33.0 / 164.0, 12.0 / 41.0, 1.0});
  SOL_CUDA(cudaMemcpyToSymbol(c_rk_k, k, sizeof(k)));
  SOL_CUDA(cudaMemcpyToSymbol(c_rk_idx, idx, sizeof(idx)));
  SOL_CUDA(cudaMemcpyToSymbol(c_rk_a, a, sizeof(a)));
  if (dev >= 0 && dev < 64) done[dev].store(true, std::memory_order_release);
  return SOL_OK;
}

}  // namespace

struct sol_ensemble {
  int device;
  cudaStream_t stream;
  int n_sys, total_bodies, max_n, max_nv, ns_cap;
  int precision;
  double eps;
  int block, ctas_per_sm, n_sm, grid;
  EnsSys* d_sys;
  int* d_order;
  EnsCtrl* d_ctrl;
  double *d_y0, *d_mass, *d_scratch;
  size_t slot_doubles;
  int* d_queue;
  std::vector<int> offsets;
  std::vector<EnsSys> sys_host;
};

#define RET(x)                   \
  do {                           \
    int r_ = (x);                \
    if (r_ != SOL_OK) return r_; \
  } while (0)

namespace {
int ens_alloc_scratch(sol_ensemble* e) {
  if (e->d_scratch) cudaFree(e->d_scratch);
  e->d_scratch = nullptr;
  e->grid = e->n_sm * e->ctas_per_sm;
  e->slot_doubles = (size_t)kVecs * e->max_nv + e->max_n + 32;
  cudaError_t r = cudaMalloc((void**)&e->d_scratch, sizeof(double) * e->slot_doubles * e->grid);
  if (r != cudaSuccess) {
    sol_set_error("ensemble scratch allocation failed: %s", cudaGetErrorString(r));
    return SOL_ERR_NOMEM;
  }
  return SOL_OK;
}

void ens_free(sol_ensemble* e) {
  if (!e) return;
  void* p[] = {e->d_sys, e->d_order, e->d_ctrl, e->d_y0, e->d_mass, e->d_scratch, e->d_queue};
  for (void* q : p)
    if (q) cudaFree(q);
  if (e->stream) cudaStreamDestroy(e->stream);
  delete e;
}

int ens_run(sol_ensemble* e, int n_steps) {
  SOL_CUDA(cudaMemsetAsync(e->d_queue, 0, sizeof(int), e->stream));
  const size_t smem = sizeof(double) * 7 * (size_t)e->ns_cap;
  if (e->precision == SOL_PRECISION_FP64)
    return launch_ensemble<SOL_PRECISION_FP64>(e->grid, e->block, smem, e->stream, e->d_sys, e->d_order, e->d_ctrl,
                                               e->d_y0, e->d_mass, e->d_scratch, e->slot_doubles, e->max_nv,
                                               e->ns_cap, e->d_queue, e->n_sys, n_steps, e->eps);
  return launch_ensemble<SOL_PRECISION_SPLIT_FF>(e->grid, e->block, smem, e->stream, e->d_sys, e->d_order,
                                                 e->d_ctrl, e->d_y0, e->d_mass, e->d_scratch, e->slot_doubles,
                                                 e->max_nv, e->ns_cap, e->d_queue, e->n_sys, n_steps, e->eps);
}
}  // namespace

extern "C" {

int sol_ensemble_create(const sol_body_data* systems, int32_t n_systems, int32_t device, sol_ensemble** out) {
  if (!systems || n_systems < 1 || !out) {
    sol_set_error("sol_ensemble_create: bad arguments");
    return SOL_ERR_ARG;
  }
  *out = nullptr;
  std::vector<EnsSys> sys(n_systems);
  int total = 0, max_n = 0, ns_cap = 1;
  for (int s = 0; s < n_systems; ++s) {
    const sol_nbodies& k = systems[s].n;
    const int c[7] = {k.central_body, k.giant_planet, k.rocky_planet, k.proto_planet, k.super_planetesimal,
                      k.planetesimal, k.test_particle};
    int n = 0;
    for (int q = 0; q < 7; ++q) {
      if (c[q] < 0) {
        sol_set_error("system %d: negative body count", s);
        return SOL_ERR_ARG;
      }
      n += c[q];
    }
    if (k.central_body != 1 || !systems[s].type || !systems[s].mass) {
      sol_set_error("system %d: need one central body, type and mass arrays", s);
      return SOL_ERR_ARG;
    }
    int expect = 0;
    for (int q = 0; q < 7; ++q)
      for (int r = 0; r < c[q]; ++r, ++expect)
        if (systems[s].type[expect] != q + 1) {
          sol_set_error("system %d: bodies must be sorted by type", s);
          return SOL_ERR_ARG;
        }
    sys[s].off = total;
    sys[s].n = n;
    sys[s].nm = k.central_body + k.giant_planet + k.rocky_planet + k.proto_planet;
    sys[s].ns_max = sys[s].nm + k.super_planetesimal;
    total += n;
    max_n = std::max(max_n, n);
    ns_cap = std::max(ns_cap, sys[s].ns_max);
  }
  if (ns_cap > 2048) {
    sol_set_error("ensemble systems may have at most 2048 attracting bodies (got %d)", ns_cap);
    return SOL_ERR_ARG;
  }
  int ndev = 0;
  SOL_CUDA(cudaGetDeviceCount(&ndev));
  if (device < 0 || device >= ndev) {
    sol_set_error("device %d not available", device);
    return SOL_ERR_ARG;
  }
  SOL_CUDA(cudaSetDevice(device));
  RET(upload_tableau());
  sol_ensemble* e = new sol_ensemble();
  e->device = device;
  e->n_sys = n_systems;
  e->total_bodies = total;
  e->max_n = max_n;
  e->max_nv = 6 * max_n;
  e->ns_cap = (ns_cap + 1) & ~1;  // even, so the float2 table stays aligned
  e->precision = SOL_PRECISION_FP64;
  e->eps = pow(10, -10.0);
  e->block = 128;
  e->ctas_per_sm = 4;
  SOL_CUDA(cudaDeviceGetAttribute(&e->n_sm, cudaDevAttrMultiProcessorCount, device));
  e->sys_host = sys;
  auto fail = [&](int r) {
    ens_free(e);
    return r;
  };
  if (cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking) != cudaSuccess) return fail(SOL_ERR_CUDA);
  // systems largest first, so the queue ends on small ones
  std::vector<int> order(n_systems);
  for (int s = 0; s < n_systems; ++s) order[s] = s;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return sys[a].n > sys[b].n; });
  std::vector<double> mass(total);
  for (int s = 0; s < n_systems; ++s) memcpy(&mass[sys[s].off], systems[s].mass, sizeof(double) * sys[s].n);
  std::vector<EnsCtrl> ctrl(n_systems);
  memset(ctrl.data(), 0, sizeof(EnsCtrl) * n_systems);
  if (cudaMalloc((void**)&e->d_sys, sizeof(EnsSys) * n_systems) != cudaSuccess ||
      cudaMalloc((void**)&e->d_order, sizeof(int) * n_systems) != cudaSuccess ||
      cudaMalloc((void**)&e->d_ctrl, sizeof(EnsCtrl) * n_systems) != cudaSuccess ||
      cudaMalloc((void**)&e->d_y0, sizeof(double) * 6 * (size_t)total) != cudaSuccess ||
      cudaMalloc((void**)&e->d_mass, sizeof(double) * total) != cudaSuccess ||
      cudaMalloc((void**)&e->d_queue, sizeof(int)) != cudaSuccess) {
    sol_set_error("ensemble allocation failed");
    return fail(SOL_ERR_NOMEM);
  }
  if (cudaMemcpy(e->d_sys, sys.data(), sizeof(EnsSys) * n_systems, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(e->d_order, order.data(), sizeof(int) * n_systems, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(e->d_ctrl, ctrl.data(), sizeof(EnsCtrl) * n_systems, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(e->d_mass, mass.data(), sizeof(double) * total, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemset(e->d_y0, 0, sizeof(double) * 6 * (size_t)total) != cudaSuccess)
    return fail(SOL_ERR_CUDA);
  int rc = ens_alloc_scratch(e);
  if (rc) return fail(rc);
  *out = e;
  return SOL_OK;
}

int sol_ensemble_destroy(sol_ensemble* e) {
  if (!e) return SOL_OK;
  cudaSetDevice(e->device);
  cudaStreamSynchronize(e->stream);
  ens_free(e);
  return SOL_OK;
}

int sol_ensemble_set_precision(sol_ensemble* e, int32_t precision) {
  if (!e || (precision != SOL_PRECISION_FP64 && precision != SOL_PRECISION_SPLIT_FF)) {
    sol_set_error("ensemble precision must be SOL_PRECISION_FP64 or SOL_PRECISION_SPLIT_FF");
    return SOL_ERR_ARG;
  }
  e->precision = precision;
  return SOL_OK;
}

int sol_ensemble_set_tolerance(sol_ensemble* e, double eps) {
  if (!e || !(eps > 0)) return SOL_ERR_ARG;
  e->eps = eps;
  return SOL_OK;
}

int sol_ensemble_set_state(sol_ensemble* e, const double* y0_all, const sol_time_line* tls) {
  if (!e || !y0_all || !tls) return SOL_ERR_ARG;
  SOL_CUDA(cudaSetDevice(e->device));
  SOL_CUDA(cudaMemcpyAsync(e->d_y0, y0_all, sizeof(double) * 6 * (size_t)e->total_bodies, cudaMemcpyHostToDevice,
                           e->stream));
  std::vector<EnsCtrl> ctrl(e->n_sys);
  memset(ctrl.data(), 0, sizeof(EnsCtrl) * e->n_sys);
  for (int s = 0; s < e->n_sys; ++s) {
    ctrl[s].t = tls[s].time;
    ctrl[s].h_next = tls[s].h_next;
    ctrl[s].h_did = tls[s].h_did;
    ctrl[s].h = tls[s].h_next;
  }
  SOL_CUDA(cudaMemcpyAsync(e->d_ctrl, ctrl.data(), sizeof(EnsCtrl) * e->n_sys, cudaMemcpyHostToDevice, e->stream));
  SOL_CUDA(cudaStreamSynchronize(e->stream));
  return SOL_OK;
}

int sol_ensemble_get_state(sol_ensemble* e, double* y0_all, sol_time_line* tls, int32_t* status) {
  if (!e) return SOL_ERR_ARG;
  SOL_CUDA(cudaSetDevice(e->device));
  if (y0_all)
    SOL_CUDA(cudaMemcpyAsync(y0_all, e->d_y0, sizeof(double) * 6 * (size_t)e->total_bodies, cudaMemcpyDeviceToHost,
                             e->stream));
  std::vector<EnsCtrl> ctrl(e->n_sys);
  SOL_CUDA(cudaMemcpyAsync(ctrl.data(), e->d_ctrl, sizeof(EnsCtrl) * e->n_sys, cudaMemcpyDeviceToHost, e->stream));
  SOL_CUDA(cudaStreamSynchronize(e->stream));
  for (int s = 0; s < e->n_sys; ++s) {
    if (tls) {
      tls[s].time = ctrl[s].t;
      tls[s].h_next = ctrl[s].h_next;
      tls[s].h_did = ctrl[s].h_did;
    }
    if (status) status[s] = ctrl[s].status;
  }
  return SOL_OK;
}

int sol_ensemble_advance(sol_ensemble* e, int32_t n_steps, sol_step_stats* stats) {
  if (!e || n_steps < 0) return SOL_ERR_ARG;
  SOL_CUDA(cudaSetDevice(e->device));
  std::vector<EnsCtrl> before;
  if (stats) {
    before.resize(e->n_sys);
    SOL_CUDA(cudaMemcpyAsync(before.data(), e->d_ctrl, sizeof(EnsCtrl) * e->n_sys, cudaMemcpyDeviceToHost,
                             e->stream));
  }
  RET(ens_run(e, n_steps));
  std::vector<EnsCtrl> after(e->n_sys);
  SOL_CUDA(cudaMemcpyAsync(after.data(), e->d_ctrl, sizeof(EnsCtrl) * e->n_sys, cudaMemcpyDeviceToHost, e->stream));
  SOL_CUDA(cudaStreamSynchronize(e->stream));
  int failed = 0;
  for (int s = 0; s < e->n_sys; ++s) {
    if (after[s].status) failed++;
    if (stats) {
      const long long acc = after[s].n_acc - before[s].n_acc, rej = after[s].n_rej - before[s].n_rej;
      stats->accepted += acc;
      stats->rejected += rej;
      stats->evaluations += acc * 13 + rej * 12;
    }
  }
  if (failed) {
    sol_set_error("%d systems stopped with a step-size underflow", failed);
    return SOL_ERR_UNDERFLOW;
  }
  return SOL_OK;
}

int sol_ensemble_configure(sol_ensemble* e, int32_t threads_per_system, int32_t systems_per_sm) {
  if (!e || threads_per_system < 32 || threads_per_system > 1024 || (threads_per_system & 31) ||
      systems_per_sm < 1 || systems_per_sm > 32) {
    sol_set_error("threads per system must be a multiple of 32 in [32, 1024], systems per SM in [1, 32]");
    return SOL_ERR_ARG;
  }
  SOL_CUDA(cudaSetDevice(e->device));
  e->block = threads_per_system;
  if (e->ctas_per_sm != systems_per_sm) {
    e->ctas_per_sm = systems_per_sm;
    RET(ens_alloc_scratch(e));
  }
  return SOL_OK;
}

int sol_ensemble_autotune(sol_ensemble* e, int32_t steps, int32_t* threads_out, int32_t* systems_per_sm_out,
                          double* best_ms_out) {
  // Times one advance of `steps` driver calls for each launch shape on a copy
  // of the current state, restores the state, and keeps the fastest shape.
  if (!e || steps < 1) return SOL_ERR_ARG;
  SOL_CUDA(cudaSetDevice(e->device));
  const size_t ny = 6 * (size_t)e->total_bodies;
  double* y_save = nullptr;
  EnsCtrl* c_save = nullptr;
  SOL_CUDA(cudaMalloc((void**)&y_save, sizeof(double) * ny));
  SOL_CUDA(cudaMalloc((void**)&c_save, sizeof(EnsCtrl) * e->n_sys));
  SOL_CUDA(cudaMemcpyAsync(y_save, e->d_y0, sizeof(double) * ny, cudaMemcpyDeviceToDevice, e->stream));
  SOL_CUDA(cudaMemcpyAsync(c_save, e->d_ctrl, sizeof(EnsCtrl) * e->n_sys, cudaMemcpyDeviceToDevice, e->stream));
  cudaEvent_t a, b;
  SOL_CUDA(cudaEventCreate(&a));
  SOL_CUDA(cudaEventCreate(&b));
  const int blocks[] = {64, 128, 256};
  const int per_sm[] = {2, 4, 8, 16};
  double best = 1e300;
  int bb = e->block, bs = e->ctas_per_sm;
  int rc = SOL_OK;
  for (int B : blocks) {
    for (int P : per_sm) {
      if ((rc = sol_ensemble_configure(e, B, P))) break;
      cudaMemcpyAsync(e->d_y0, y_save, sizeof(double) * ny, cudaMemcpyDeviceToDevice, e->stream);
      cudaMemcpyAsync(e->d_ctrl, c_save, sizeof(EnsCtrl) * e->n_sys, cudaMemcpyDeviceToDevice, e->stream);
      cudaEventRecord(a, e->stream);
      if ((rc = ens_run(e, steps))) break;
      cudaEventRecord(b, e->stream);
      if (cudaEventSynchronize(b) != cudaSuccess) {
        rc = SOL_ERR_CUDA;
        break;
      }
      float ms = 0;
      cudaEventElapsedTime(&ms, a, b);
      if (ms < best) {
        best = ms;
        bb = B;
        bs = P;
      }
    }
    if (rc) break;
  }
  cudaMemcpyAsync(e->d_y0, y_save, sizeof(double) * ny, cudaMemcpyDeviceToDevice, e->stream);
  cudaMemcpyAsync(e->d_ctrl, c_save, sizeof(EnsCtrl) * e->n_sys, cudaMemcpyDeviceToDevice, e->stream);
  cudaStreamSynchronize(e->stream);
  cudaFree(y_save);
  cudaFree(c_save);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (rc) return rc;
  RET(sol_ensemble_configure(e, bb, bs));
  if (threads_out) *threads_out = bb;
  if (systems_per_sm_out) *systems_per_sm_out = bs;
  if (best_ms_out) *best_ms_out = best;
  return SOL_OK;
}

}  // extern "C"
