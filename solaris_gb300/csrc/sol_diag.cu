// Event predicates, integrals and the FP64 throughput microbenchmark.
#include "sol_internal.cuh"

namespace {

constexpr int kBlock = 256;

// Simulator::CheckEvent predicates (Solaris/Simulator.cpp:626-645, :690-729),
// evaluated on the outputs of the last force evaluation: rm3 for ejection and
// hit-centrum, the nearest-neighbour arrays for collisions.  Each hit is
// appended with an atomic counter; the host orders the list as the reference
// visits bodies.
__global__ void k_events(int n, const double* __restrict__ rm3, const int32_t* __restrict__ nn_idx,
                         const double* __restrict__ nn_dist, const double* __restrict__ radius,
                         const double* __restrict__ y0, double ejection, double hit_centrum, double factor,
                         sol_event* out, int capacity, int* count) {
  const double e3 = ejection > 0 ? 1.0 / (ejection * ejection * ejection) : 0.0;
  const double h3 = hit_centrum > 0 ? 1.0 / (hit_centrum * hit_centrum * hit_centrum) : 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    if (i >= 1) {
      const double* p = y0 + 6 * i;
      double r = sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
      if (ejection > 0 && rm3[i] < e3) {
        int k = atomicAdd(count, 1);
        if (k < capacity) out[k] = sol_event{SOL_EVENT_EJECTION, 0, i, 0, r};
      }
      if (hit_centrum > 0 && rm3[i] > h3) {
        int k = atomicAdd(count, 1);
        if (k < capacity) out[k] = sol_event{SOL_EVENT_HIT_CENTRUM, 0, i, 0, r};
      }
    }
    if (factor > 0) {
      int j = nn_idx[i];
      if (j >= 0 && factor * (radius[i] + radius[j]) > nn_dist[i]) {
        int k = atomicAdd(count, 1);
        if (k < capacity) out[k] = sol_event{SOL_EVENT_COLLISION, i, j, 0, nn_dist[i]};
      }
    }
  }
}

// Per-body potential-energy sums of Calculate::PotentialEnergy
// (Solaris/Calculate.cpp:139-159): pe[i] = sum_{j != i} m_i m_j / r_ij, sources
// staged through shared memory; the host finishes the O(N) parts.
__global__ void k_potential(int n, const double* __restrict__ y0, const double* __restrict__ mass,
                            double* __restrict__ pe) {
  __shared__ double sx[kBlock], sy[kBlock], sz[kBlock], sm[kBlock];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double xi = 0, yi = 0, zi = 0, mi = 0;
  if (i < n) {
    xi = y0[6 * i];
    yi = y0[6 * i + 1];
    zi = y0[6 * i + 2];
    mi = mass[i];
  }
  double acc = 0.0;
  for (int j0 = 0; j0 < n; j0 += kBlock) {
    int j = j0 + threadIdx.x;
    if (j < n) {
      sx[threadIdx.x] = y0[6 * j];
      sy[threadIdx.x] = y0[6 * j + 1];
      sz[threadIdx.x] = y0[6 * j + 2];
      sm[threadIdx.x] = mass[j];
    }
    __syncthreads();
    const int lim = min(kBlock, n - j0);
    if (i < n)
      for (int q = 0; q < lim; ++q) {
        if (j0 + q == i) continue;
        double dx = sx[q] - xi, dy = sy[q] - yi, dz = sz[q] - zi;
        double rij = __dsqrt_rn(dx * dx + dy * dy + dz * dz);
        acc += __ddiv_rn(mi * sm[q], rij);
      }
    __syncthreads();
  }
  if (i < n) pe[i] = acc;
}

// Dependent FMA chains: FP64 pipe throughput.
__global__ void k_dfma_peak(double seed, double b, double* out, int iters) {
  double v[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) v[c] = seed + threadIdx.x * 1e-9 + c * 1e-3;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int c = 0; c < 8; ++c) v[c] = __fma_rn(v[c], b, 1.0000001);
  }
  double s = 0;
#pragma unroll
  for (int c = 0; c < 8; ++c) s += v[c];
  if (s == -12345.0) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

int sol_events_launch(sol_ctx* c, const double* d_y0, double ej, double hc, double cf, sol_event* d_out,
                      int capacity, int* d_count) {
  SOL_CUDA(cudaMemsetAsync(d_count, 0, sizeof(int), c->stream));
  int g = (c->n + kBlock - 1) / kBlock;
  k_events<<<g, kBlock, 0, c->stream>>>(c->n, c->d_rm3, c->d_nn_idx, c->d_nn_dist, c->d_radius, d_y0, ej, hc, cf,
                                        d_out, capacity, d_count);
  SOL_LAUNCHED();
  return SOL_OK;
}

int sol_potential_launch(sol_ctx* c, const double* d_y0, double* d_pe) {
  int g = (c->n + kBlock - 1) / kBlock;
  k_potential<<<g, kBlock, 0, c->stream>>>(c->n, d_y0, c->d_mass, d_pe);
  SOL_LAUNCHED();
  return SOL_OK;
}

int sol_fp64_peak_launch(int device, double* flops) {
  SOL_CUDA(cudaSetDevice(device));
  int nsm = 0;
  SOL_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device));
  const int threads = 256, blocks = nsm * 8, iters = 4096;
  double* out = nullptr;
  SOL_CUDA(cudaMalloc(&out, sizeof(double) * threads * blocks));
  cudaEvent_t e0, e1;
  SOL_CUDA(cudaEventCreate(&e0));
  SOL_CUDA(cudaEventCreate(&e1));
  k_dfma_peak<<<blocks, threads>>>(1.0, 0.999999, out, 256);  // warm-up
  SOL_LAUNCHED();
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    SOL_CUDA(cudaEventRecord(e0));
    k_dfma_peak<<<blocks, threads>>>(1.0, 0.999999, out, iters);
    SOL_LAUNCHED();
    SOL_CUDA(cudaEventRecord(e1));
    SOL_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    SOL_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    if (ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  const double fmas = (double)threads * blocks * 8.0 * iters;
  *flops = 2.0 * fmas / (best * 1e-3);
  return SOL_OK;
}
