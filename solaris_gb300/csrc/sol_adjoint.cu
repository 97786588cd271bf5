// Discrete adjoint of the fixed-step RungeKuttaFehlberg78 integration
// (RungeKuttaFehlberg78::Step at constant h, y_{n+1} = the 7th-order result,
// Solaris/RungeKuttaFehlberg78.cpp:147-250) with GravityAC forces
// (Solaris/Acceleration.cpp:248-329).
//
// Forward: n fixed steps on the device, the state stored every K steps.
// Backward, one segment of K steps at a time from the last: the segment is
// recomputed from its checkpoint with every stage state Y_k (k = 0..10) of
// every step kept; then, step by step from the last, the stage adjoints
//   w_k = h b_k lambda + h sum_{j>k} a_jk nu_j,   nu_k = J(Y_k)^T w_k
// and lambda_n = lambda_{n+1} + sum_k nu_k, with the mass gradient
// accumulated from the same w_k.  Stages 11 and 12 only enter the error
// estimate, so their adjoints are zero.  J^T w is a hand-written
// vector-Jacobian product of the pair force (one warp per body).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "sol_internal.cuh"

int sol_rkf78_stages(sol_ctx* c, const double* d_y0, double* d_y, double* const* stage_out);

namespace {

constexpr int kBlock = 256;
constexpr int kWarpsPerBlock = 8;
constexpr int kAdjStages = 11;  // stages 0..10 reach y_{n+1}

// RKF78 tableau (RungeKuttaFehlberg78.cpp:41-56): a[j][k] and the weights b
const double kA[13][13] = {
    {0},
    {2.0 / 27.0},
    {1.0 / 36.0, 1.0 / 12.0},
    {1.0 / 24.0, 0, 1.0 / 8.0},
    {5.0 / 12.0, 0, -25.0 / 16.0, 25.0 / 16.0},
    {1.0 / 20.0, 0, 0, 1.0 / 4.0, 1.0 / 5.0},
    {-25.0 / 108.0, 0, 0, 125.0 / 108.0, -65.0 / 27.0, 125.0 / 54.0},
    {31.0 / 300.0, 0, 0, 0, 61.0 / 225.0, -2.0 / 9.0, 13.0 / 900.0},
    {2.0, 0, 0, -53.0 / 6.0, 704.0 / 45.0, -107.0 / 9.0, 67.0 / 90.0, 3.0},
    {-91.0 / 108.0, 0, 0, 23.0 / 108.0, -976.0 / 135.0, 311.0 / 54.0, -19.0 / 60.0, 17.0 / 6.0, -1.0 / 12.0},
    {2383.0 / 4100.0, 0, 0, -341.0 / 164.0, 4496.0 / 1025.0, -301.0 / 82.0, 2133.0 / 4100.0, 45.0 / 82.0,
     45.0 / 164.0, 18.0 / 41.0},
    {3.0 / 205.0, 0, 0, 0, 0, -6.0 / 41.0, -3.0 / 205.0, -3.0 / 41.0, 3.0 / 41.0, 6.0 / 41.0, 0},
    {-1777.0 / 4100.0, 0, 0, -341.0 / 164.0, 4496.0 / 1025.0, -289.0 / 82.0, 2193.0 / 4100.0, 51.0 / 82.0,
     33.0 / 164.0, 12.0 / 41.0, 0, 1.0}};
const double kB[13] = {41.0 / 840.0, 0, 0, 0, 0, 34.0 / 105.0, 9.0 / 35.0, 9.0 / 35.0, 9.0 / 280.0, 9.0 / 280.0,
                       41.0 / 840.0, 0, 0};

struct Lin {
  const double* v[kAdjStages + 1];
  double c[kAdjStages + 1];
  int k;
};

// out = base + scale * sum_i c_i v_i (base may be null)
__global__ void k_lincomb(int nv, double* __restrict__ out, const double* __restrict__ base, double scale, Lin L) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nv; e += gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int i = 0; i < L.k; ++i) acc = __fma_rn(L.c[i], L.v[i][e], acc);
    out[e] = base ? __fma_rn(scale, acc, base[e]) : scale * acc;
  }
}

// Structure-of-arrays view of (state, cotangent) for the VJP: x, y, z, m, wx, wy, wz
__global__ void k_vjp_prepass(int n, const double* __restrict__ Y, const double* __restrict__ w,
                              const double* __restrict__ mass, double* __restrict__ soa) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  soa[0 * n + i] = Y[6 * i];
  soa[1 * n + i] = Y[6 * i + 1];
  soa[2 * n + i] = Y[6 * i + 2];
  soa[3 * n + i] = mass[i];
  soa[4 * n + i] = w[6 * i + 3];
  soa[5 * n + i] = w[6 * i + 4];
  soa[6 * n + i] = w[6 * i + 5];
}

__device__ __forceinline__ void tensor_apply(double dx, double dy, double dz, double rm3, double rm5, double vx,
                                             double vy, double vz, double& ox, double& oy, double& oz) {
  // T(d) v = v / r^3 - 3 d (d . v) / r^5
  const double dv = __fma_rn(dx, vx, __fma_rn(dy, vy, dz * vz));
  const double s = 3.0 * rm5 * dv;
  ox = __fma_rn(vx, rm3, -s * dx);
  oy = __fma_rn(vy, rm3, -s * dy);
  oz = __fma_rn(vz, rm3, -s * dz);
}

// nu = J(Y)^T w for the heliocentric gravity with Kepler and indirect terms.
// One warp per body k; lanes split the other bodies j and the warp sums in a
// fixed shuffle order.  Also dm[k] += w . d(dydt)/d m_k, and the per-body
// terms of d/d m_0 into m0_part[k].
__global__ void k_vjp(int n, int nm, int nspl, const double* __restrict__ soa, const double* __restrict__ w,
                      double* __restrict__ nu, double* __restrict__ dm, double* __restrict__ m0_part) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int k = warp;
  if (k >= n) return;
  const double* X = soa;
  const double* Yy = soa + n;
  const double* Z = soa + 2 * n;
  const double* M = soa + 3 * n;
  const double* WX = soa + 4 * n;
  const double* WY = soa + 5 * n;
  const double* WZ = soa + 6 * n;
  if (k == 0) {  // the central body's state is fixed: its dydt is 0 (Acceleration.cpp:266)
    if (lane < 6) nu[lane] = 0.0;
    if (lane == 0) m0_part[0] = 0.0;
    return;
  }
  const double xk = X[k], yk = Yy[k], zk = Z[k], mk = M[k];
  const double wkx = WX[k], wky = WY[k], wkz = WZ[k];
  const int ns_k = k < nm ? nm + nspl : nm;
  const bool k_is_source = k < nm + nspl;  // source of some sink
  const double G = SOL_GAUSS2;
  double gx = 0, gy = 0, gz = 0;     // J_r^T w from pair terms
  double Wx = 0, Wy = 0, Wz = 0;     // sum of w_v over the sinks that have k as a source
  double dmk = 0;                    // pair part of dL/dm_k
  for (int j = 1 + lane; j < n; j += 32) {
    if (j == k) continue;
    const int ns_j = j < nm ? nm + nspl : nm;
    const bool k_src_of_j = k < ns_j;
    const bool j_src_of_k = j < ns_k;
    if (!k_src_of_j && !j_src_of_k) continue;
    const double dx = X[j] - xk, dy = Yy[j] - yk, dz = Z[j] - zk;  // r_j - r_k
    const double r2 = __fma_rn(dx, dx, __fma_rn(dy, dy, dz * dz));
    const double rinv = rsqrt(r2);
    const double rm3 = rinv * rinv * rinv;
    const double rm5 = rm3 * rinv * rinv;
    const double wjx = WX[j], wjy = WY[j], wjz = WZ[j];
    // v = [k source of j] m_k w_j - [j source of k] m_j w_k
    double vx = 0, vy = 0, vz = 0;
    if (k_src_of_j) {
      vx = mk * wjx;
      vy = mk * wjy;
      vz = mk * wjz;
      Wx += wjx;
      Wy += wjy;
      Wz += wjz;
      // d a_j / d m_k = G (r_k - r_j) / |r_k - r_j|^3 (direct part)
      dmk -= rm3 * __fma_rn(dx, wjx, __fma_rn(dy, wjy, dz * wjz));
    }
    if (j_src_of_k) {
      const double mj = M[j];
      vx = __fma_rn(-mj, wkx, vx);
      vy = __fma_rn(-mj, wky, vy);
      vz = __fma_rn(-mj, wkz, vz);
    }
    double tx, ty, tz;
    tensor_apply(dx, dy, dz, rm3, rm5, vx, vy, vz, tx, ty, tz);
    gx += tx;
    gy += ty;
    gz += tz;
  }
  for (int o = 16; o > 0; o >>= 1) {
    gx += __shfl_down_sync(0xffffffffu, gx, o);
    gy += __shfl_down_sync(0xffffffffu, gy, o);
    gz += __shfl_down_sync(0xffffffffu, gz, o);
    Wx += __shfl_down_sync(0xffffffffu, Wx, o);
    Wy += __shfl_down_sync(0xffffffffu, Wy, o);
    Wz += __shfl_down_sync(0xffffffffu, Wz, o);
    dmk += __shfl_down_sync(0xffffffffu, dmk, o);
  }
  if (lane != 0) return;
  // Kepler term -G (m0 + m_k) r_k / |r_k|^3 and indirect term -G m_k r_k / |r_k|^3 (for the sinks of k)
  const double r2 = __fma_rn(xk, xk, __fma_rn(yk, yk, zk * zk));
  const double rinv = rsqrt(r2);
  const double rm3 = rinv * rinv * rinv;
  const double rm5 = rm3 * rinv * rinv;
  const double m0 = M[0];
  double kx, ky, kz;
  tensor_apply(xk, yk, zk, rm3, rm5, -(m0 + mk) * wkx - (k_is_source ? mk * Wx : 0.0),
               -(m0 + mk) * wky - (k_is_source ? mk * Wy : 0.0), -(m0 + mk) * wkz - (k_is_source ? mk * Wz : 0.0),
               kx, ky, kz);
  nu[6 * k + 0] = G * (gx + kx);
  nu[6 * k + 1] = G * (gy + ky);
  nu[6 * k + 2] = G * (gz + kz);
  nu[6 * k + 3] = w[6 * k + 0];  // d(position)/dt = velocity
  nu[6 * k + 4] = w[6 * k + 1];
  nu[6 * k + 5] = w[6 * k + 2];
  const double rk_w = __fma_rn(xk, wkx, __fma_rn(yk, wky, zk * wkz)) * rm3;  // w_k . r_k / |r_k|^3
  const double rk_W = k_is_source ? __fma_rn(xk, Wx, __fma_rn(yk, Wy, zk * Wz)) * rm3 : 0.0;
  dm[k] += G * (dmk - rk_w - rk_W);
  m0_part[k] = -G * rk_w;
}

// dm[0] += sum of the per-body parts, one block, fixed order
__global__ void k_sum_m0(int n, const double* __restrict__ part, double* __restrict__ dm) {
  __shared__ double red[kBlock];
  double a = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) a += part[i];
  red[threadIdx.x] = a;
  __syncthreads();
  for (int s = kBlock / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) dm[0] += red[0];
}

inline int grid_for(int n) {
  int g = (n + kBlock - 1) / kBlock;
  return g < 1 ? 1 : (g > 152 * 16 ? 152 * 16 : g);
}

#define RET(x)                   \
  do {                           \
    int r_ = (x);                \
    if (r_ != SOL_OK) return r_; \
  } while (0)

}  // namespace

// Adjoint state kept in the context between forward and backward.
struct sol_adjoint_state {
  int n_steps = 0, every = 0, n_cp = 0;
  double h = 0.0;
  double* d_cp = nullptr;     // checkpoints, (n_cp) x 6N
  double* d_stages = nullptr; // every x 11 x 6N stage states of one segment
  double* d_nu = nullptr;     // 11 x 6N stage adjoints
  double* d_lam = nullptr;    // 6N
  double* d_w = nullptr;      // 6N
  double* d_soa = nullptr;    // 7N
  double* d_dm = nullptr;     // N
  double* d_m0p = nullptr;    // N
  double* d_tmp = nullptr;    // 6N
};

void sol_adjoint_free(sol_adjoint_state* a) {
  if (!a) return;
  double* p[] = {a->d_cp, a->d_stages, a->d_nu, a->d_lam, a->d_w, a->d_soa, a->d_dm, a->d_m0p, a->d_tmp};
  for (double* q : p)
    if (q) cudaFree(q);
  delete a;
}

namespace {
int set_fixed_h(sol_ctx* c, double h) {
  sol_ctrl hc;
  memset(&hc, 0, sizeof(hc));
  hc.h = h;
  hc.h_next = h;
  hc.eps = c->eps;
  SOL_CUDA(cudaMemcpyAsync(c->d_ctrl, &hc, sizeof(hc), cudaMemcpyHostToDevice, c->stream));
  return SOL_OK;
}

int vjp(sol_ctx* c, sol_adjoint_state* a, const double* Y, const double* w, double* nu) {
  const int n = c->n;
  k_vjp_prepass<<<(n + kBlock - 1) / kBlock, kBlock, 0, c->stream>>>(n, Y, w, c->d_mass, a->d_soa);
  SOL_LAUNCHED();
  const int threads = kWarpsPerBlock * 32;
  k_vjp<<<(n + kWarpsPerBlock - 1) / kWarpsPerBlock, threads, 0, c->stream>>>(
      n, c->cls.nm, c->cls.n_spl, a->d_soa, w, nu, a->d_dm, a->d_m0p);
  SOL_LAUNCHED();
  k_sum_m0<<<1, kBlock, 0, c->stream>>>(n, a->d_m0p, a->d_dm);
  SOL_LAUNCHED();
  return SOL_OK;
}
}  // namespace

extern "C" int sol_adjoint_forward(sol_ctx* c, double h, int32_t n_steps, int32_t every, const double* y0,
                                   double* y_final) {
  if (!c || !y0 || n_steps < 1 || every < 1 || !(h != 0.0)) {
    sol_set_error("sol_adjoint_forward: bad arguments");
    return SOL_ERR_ARG;
  }
  if (c->barycentric || c->has_gas) {
    sol_set_error("the adjoint covers heliocentric gravity without a nebula");
    return SOL_ERR_ARG;
  }
  SOL_CUDA(cudaSetDevice(c->device));
  sol_adjoint_free(c->adj);
  c->adj = new sol_adjoint_state();
  sol_adjoint_state* a = c->adj;
  a->n_steps = n_steps;
  a->every = every;
  a->h = h;
  a->n_cp = (n_steps + every - 1) / every;
  const size_t nv = c->nv;
  auto alloc = [&](double** p, size_t cnt) -> int {
    if (cudaMalloc((void**)p, sizeof(double) * (cnt ? cnt : 1)) != cudaSuccess) {
      sol_set_error("adjoint allocation of %zu doubles failed", cnt);
      return SOL_ERR_NOMEM;
    }
    return SOL_OK;
  };
  RET(alloc(&a->d_cp, (size_t)a->n_cp * nv));
  SOL_CUDA(cudaMemcpyAsync(c->d_y0, y0, sizeof(double) * nv, cudaMemcpyHostToDevice, c->stream));
  RET(set_fixed_h(c, h));
  for (int s = 0; s < n_steps; ++s) {
    if (s % every == 0)
      SOL_CUDA(cudaMemcpyAsync(a->d_cp + (size_t)(s / every) * nv, c->d_y0, sizeof(double) * nv,
                               cudaMemcpyDeviceToDevice, c->stream));
    RET(sol_rkf78_stages(c, c->d_y0, c->d_y, nullptr));
    SOL_CUDA(cudaMemcpyAsync(c->d_y0, c->d_y, sizeof(double) * nv, cudaMemcpyDeviceToDevice, c->stream));
  }
  c->state_valid = 1;
  if (y_final) SOL_CUDA(cudaMemcpyAsync(y_final, c->d_y0, sizeof(double) * nv, cudaMemcpyDeviceToHost, c->stream));
  SOL_CUDA(cudaStreamSynchronize(c->stream));
  return SOL_OK;
}

extern "C" int sol_adjoint_backward(sol_ctx* c, const double* dl_dy_final, double* dl_dy0, double* dl_dmass) {
  if (!c || !dl_dy_final || !c->adj || !c->adj->d_cp) {
    sol_set_error("sol_adjoint_backward: run sol_adjoint_forward first");
    return SOL_ERR_STATE;
  }
  SOL_CUDA(cudaSetDevice(c->device));
  sol_adjoint_state* a = c->adj;
  const size_t nv = c->nv;
  const int n = c->n;
  auto alloc = [&](double** p, size_t cnt) -> int {
    if (*p) return SOL_OK;
    if (cudaMalloc((void**)p, sizeof(double) * (cnt ? cnt : 1)) != cudaSuccess) {
      sol_set_error("adjoint allocation of %zu doubles failed", cnt);
      return SOL_ERR_NOMEM;
    }
    return SOL_OK;
  };
  RET(alloc(&a->d_stages, (size_t)a->every * kAdjStages * nv));
  RET(alloc(&a->d_nu, (size_t)kAdjStages * nv));
  RET(alloc(&a->d_lam, nv));
  RET(alloc(&a->d_w, nv));
  RET(alloc(&a->d_soa, 7 * (size_t)n));
  RET(alloc(&a->d_dm, n));
  RET(alloc(&a->d_m0p, n));
  RET(alloc(&a->d_tmp, nv));
  SOL_CUDA(cudaMemcpyAsync(a->d_lam, dl_dy_final, sizeof(double) * nv, cudaMemcpyHostToDevice, c->stream));
  SOL_CUDA(cudaMemsetAsync(a->d_dm, 0, sizeof(double) * n, c->stream));
  RET(set_fixed_h(c, a->h));
  const double h = a->h;
  const int g = grid_for((int)nv);
  for (int seg = a->n_cp - 1; seg >= 0; --seg) {
    const int s0 = seg * a->every;
    const int s1 = std::min(a->n_steps, s0 + a->every);
    // recompute the segment, keeping the stage states Y_0..Y_10 of every step
    SOL_CUDA(cudaMemcpyAsync(a->d_tmp, a->d_cp + (size_t)seg * nv, sizeof(double) * nv, cudaMemcpyDeviceToDevice,
                             c->stream));
    for (int s = s0; s < s1; ++s) {
      double* base = a->d_stages + (size_t)(s - s0) * kAdjStages * nv;
      double* outs[13];
      for (int k = 0; k < 13; ++k) outs[k] = k < kAdjStages ? base + (size_t)k * nv : nullptr;
      SOL_CUDA(cudaMemcpyAsync(outs[0], a->d_tmp, sizeof(double) * nv, cudaMemcpyDeviceToDevice, c->stream));
      RET(sol_rkf78_stages(c, outs[0], a->d_tmp, outs));
    }
    // backward through the segment's steps
    for (int s = s1 - 1; s >= s0; --s) {
      const double* Ys = a->d_stages + (size_t)(s - s0) * kAdjStages * nv;
      for (int k = kAdjStages - 1; k >= 0; --k) {
        Lin L;
        memset(&L, 0, sizeof(L));
        L.v[L.k] = a->d_lam;
        L.c[L.k++] = kB[k];
        for (int j = k + 1; j < kAdjStages; ++j)
          if (kA[j][k] != 0.0) {
            L.v[L.k] = a->d_nu + (size_t)j * nv;
            L.c[L.k++] = kA[j][k];
          }
        k_lincomb<<<g, kBlock, 0, c->stream>>>((int)nv, a->d_w, nullptr, h, L);
        SOL_LAUNCHED();
        RET(vjp(c, a, Ys + (size_t)k * nv, a->d_w, a->d_nu + (size_t)k * nv));
      }
      Lin L;
      memset(&L, 0, sizeof(L));
      for (int k = 0; k < kAdjStages; ++k) {
        L.v[L.k] = a->d_nu + (size_t)k * nv;
        L.c[L.k++] = 1.0;
      }
      k_lincomb<<<g, kBlock, 0, c->stream>>>((int)nv, a->d_w, a->d_lam, 1.0, L);
      SOL_LAUNCHED();
      std::swap(a->d_w, a->d_lam);
    }
  }
  if (dl_dy0) SOL_CUDA(cudaMemcpyAsync(dl_dy0, a->d_lam, sizeof(double) * nv, cudaMemcpyDeviceToHost, c->stream));
  if (dl_dmass) SOL_CUDA(cudaMemcpyAsync(dl_dmass, a->d_dm, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
  SOL_CUDA(cudaStreamSynchronize(c->stream));
  return SOL_OK;
}

extern "C" int sol_set_masses(sol_ctx* c, const double* mass) {
  if (!c || !mass) return SOL_ERR_ARG;
  SOL_CUDA(cudaSetDevice(c->device));
  SOL_CUDA(cudaMemcpyAsync(c->d_mass, mass, sizeof(double) * c->n, cudaMemcpyHostToDevice, c->stream));
  SOL_CUDA(cudaStreamSynchronize(c->stream));
  // captured driver graphs read masses from device memory: nothing to rebuild
  return SOL_OK;
}
