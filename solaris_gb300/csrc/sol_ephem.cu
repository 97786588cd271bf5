// Initial conditions in bulk: Ephemeris::CalculatePhase and
// Ephemeris::KeplerEquationSolver (Solaris/Ephemeris.cpp:141-211) for many
// bodies at once, one thread per body -- the phase of every body of an
// ensemble from its orbital elements.
#include <cmath>
#include <vector>

#include "sol_internal.cuh"

namespace {

constexpr int kBlock = 256;

// KeplerEquationSolver (:187-211): starting value, then Newton steps until the
// change is at most eps (at most 25 steps).  With SOL_QUIRK_INT_ABS the change
// is measured as the reference build does it, through int abs(): the loop
// ends as soon as it is below 1.
__device__ int kepler(double e, double m, double eps, int quirks, double* E) {
  if (e == 0.0 || m == 0.0 || m == SOL_PI) {
    *E = m;
    return 0;
  }
  double EE = m + e * (sin(m)) / (1.0 - sin(m + e) + sin(m));
  double E1 = 0.0, err;
  int step = 0;
  do {
    E1 = EE - (EE - e * sin(EE) - m) / (1.0 - e * cos(EE));
    const double d = E1 - EE;
    err = (quirks & SOL_QUIRK_INT_ABS) ? (double)abs((int)d) : fabs(d);
    EE = E1;
    step++;
  } while (err > eps && step <= 25);
  *E = EE;
  return step > 25 ? 1 : 0;
}

// CalculatePhase (:141-176); elements = {a, e, i, argument of pericentre,
// longitude of node, mean anomaly}.
__global__ void k_phase(int n, const double* __restrict__ mu, const double* __restrict__ el, int quirks,
                        double* __restrict__ ph, int32_t* __restrict__ status) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= n) return;
  const double* q = el + 6 * b;
  double* out = ph + 6 * b;
  const double e = q[1];
  double E = 0.0;
  if (kepler(e, q[5], 1.0e-14, quirks, &E)) {
    status[b] = SOL_ERR_ORBIT;
    for (int k = 0; k < 6; ++k) out[k] = 0.0;
    return;
  }
  const double v = 2.0 * atan(sqrt((1.0 + e) / (1.0 - e)) * tan(E / 2.0));
  const double a = q[0];
  const double p = a * (1.0 - e * e);
  const double r = p / (1.0 + e * cos(v));
  const double kszi = r * cos(v);
  const double eta = r * sin(v);
  const double vKszi = -sqrt(mu[b] / p) * sin(v);
  const double vEta = sqrt(mu[b] / p) * (e + cos(v));
  const double cw = cos(q[3]), sw = sin(q[3]), cO = cos(q[4]), sO = sin(q[4]), ci = cos(q[2]), si = sin(q[2]);
  const double P[3] = {cw * cO - sw * sO * ci, cw * sO + sw * cO * ci, sw * si};
  const double Q[3] = {-sw * cO - cw * sO * ci, -sw * sO + cw * cO * ci, cw * si};
  for (int k = 0; k < 3; ++k) {
    out[k] = kszi * P[k] + eta * Q[k];
    out[3 + k] = vKszi * P[k] + vEta * Q[k];
  }
  status[b] = SOL_OK;
}

}  // namespace

extern "C" int sol_phases_from_elements(int32_t device, int32_t n, const double* mu, const double* elements,
                                        int32_t quirks, double* phases, int32_t* status) {
  if (n < 0 || (n > 0 && (!mu || !elements || !phases))) {
    sol_set_error("sol_phases_from_elements: bad arguments");
    return SOL_ERR_ARG;
  }
  if (n == 0) return SOL_OK;
  SOL_CUDA(cudaSetDevice(device));
  cudaStream_t st;
  SOL_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  double *d_mu = nullptr, *d_el = nullptr, *d_ph = nullptr;
  int32_t* d_st = nullptr;
  int rc = SOL_OK;
  std::vector<int32_t> h_st;
  auto step = [&](cudaError_t e, const char* what) {
    if (rc == SOL_OK && e != cudaSuccess) rc = sol_cuda_fail(e, what, __FILE__, __LINE__);
  };
  const size_t nb = (size_t)n;
  step(cudaMallocAsync((void**)&d_mu, sizeof(double) * nb, st), "cudaMallocAsync");
  step(cudaMallocAsync((void**)&d_el, sizeof(double) * 6 * nb, st), "cudaMallocAsync");
  step(cudaMallocAsync((void**)&d_ph, sizeof(double) * 6 * nb, st), "cudaMallocAsync");
  step(cudaMallocAsync((void**)&d_st, sizeof(int32_t) * nb, st), "cudaMallocAsync");
  if (rc == SOL_OK) {
    step(cudaMemcpyAsync(d_mu, mu, sizeof(double) * nb, cudaMemcpyHostToDevice, st), "copy mu");
    step(cudaMemcpyAsync(d_el, elements, sizeof(double) * 6 * nb, cudaMemcpyHostToDevice, st), "copy elements");
  }
  if (rc == SOL_OK) {
    k_phase<<<(n + kBlock - 1) / kBlock, kBlock, 0, st>>>(n, d_mu, d_el, quirks, d_ph, d_st);
    sol_count_launch();
    step(cudaGetLastError(), "k_phase");
  }
  h_st.resize(nb);
  if (rc == SOL_OK) {
    step(cudaMemcpyAsync(phases, d_ph, sizeof(double) * 6 * nb, cudaMemcpyDeviceToHost, st), "copy phases");
    step(cudaMemcpyAsync(h_st.data(), d_st, sizeof(int32_t) * nb, cudaMemcpyDeviceToHost, st), "copy status");
  }
  for (void* p : {(void*)d_mu, (void*)d_el, (void*)d_ph, (void*)d_st})
    if (p) cudaFreeAsync(p, st);
  step(cudaStreamSynchronize(st), "synchronize");
  cudaStreamDestroy(st);
  if (rc != SOL_OK) return rc;
  int bad = 0;
  for (size_t b = 0; b < nb; ++b) {
    if (status) status[b] = h_st[b];
    bad += h_st[b] != SOL_OK;
  }
  if (bad) {
    sol_set_error("Kepler's equation did not converge for %d bodies", bad);
    return SOL_ERR_ORBIT;
  }
  return SOL_OK;
}
