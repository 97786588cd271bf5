// Event predicates, integrals, the FP64 throughput microbenchmark and the
// self-check of the reference-form pair arithmetic.
#include "sol_crmath.cuh"

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

// Calculate::PotentialEnergy (Solaris/Calculate.cpp:139-159) above the
// exact-order size: the sum over unordered pairs of m_i m_j / r_ij, each
// pair evaluated once (the reference adds every ordered pair, i.e. each
// unordered pair twice, and halves the total).  CTA b takes the sink block
// I = b and the source blocks (I + d) mod nb for d = 0 .. nb/2, except that
// for an even nb the block at distance nb/2 goes to the lower half only:
// every unordered block pair once, every CTA about nb/2 blocks.  The block
// itself (d = 0) takes j > i.  1/r_ij is the FP32 rsqrt seed y corrected in
// FP64 by r^-1 = y (1 + e/2 + 3/8 e^2), e = 1 - r^2 y^2 (|e| < 2^-20, series
// truncation ~2^-65): y and y^2 exact from the seed's bits, 3/8 e^2 in FP32,
// so a pair costs 10 FP64 instructions (against ~23 with IEEE sqrt and
// division).  Coincident bodies (r_ij = 0) add m_j inf, scaled by m_i at the
// end: +inf, or NaN where either mass is 0, as the reference's
// m_i m_j / 0 gives.  Each thread sums its sink's terms per block with a
// compensated running sum, scales by m_i, and the CTA adds its threads' sums
// in thread order: part[b], deterministic.
constexpr int kPotBlock = 128;

__global__ void __launch_bounds__(kPotBlock) k_potential_pairs(int n, const double* __restrict__ y0,
                                                               const double* __restrict__ mass,
                                                               double* __restrict__ part) {
  __shared__ double sx[kPotBlock], sy[kPotBlock], sz[kPotBlock], sm[kPotBlock];
  __shared__ double red[kPotBlock];
  const int nb = (n + kPotBlock - 1) / kPotBlock;
  const int I = blockIdx.x;
  const int i = I * kPotBlock + threadIdx.x;
  double xi = 0, yi = 0, zi = 0, mi = 0;
  if (i < n) {
    xi = y0[6 * i];
    yi = y0[6 * i + 1];
    zi = y0[6 * i + 2];
    mi = mass[i];
  }
  const int dmax = (nb % 2 == 0 && I >= nb / 2) ? nb / 2 - 1 : nb / 2;
  double s = 0.0, c = 0.0;
  for (int d = 0; d <= dmax; ++d) {
    const int J = (I + d) % nb;
    const int j = J * kPotBlock + threadIdx.x;
    __syncthreads();
    if (j < n) {
      sx[threadIdx.x] = y0[6 * j];
      sy[threadIdx.x] = y0[6 * j + 1];
      sz[threadIdx.x] = y0[6 * j + 2];
      sm[threadIdx.x] = mass[j];
    }
    __syncthreads();
    const int lim = min(kPotBlock, n - J * kPotBlock);
    const int q0 = d == 0 ? threadIdx.x + 1 : 0;  // the block itself: j > i
    double acc = 0.0;
    if (i < n)
      for (int q = q0; q < lim; ++q) {
        const double dx = sx[q] - xi, dy = sy[q] - yi, dz = sz[q] - zi;
        const double r2 = __fma_rn(dx, dx, __fma_rn(dy, dy, dz * dz));
        const float yf = sol_rsqrt_seed(r2);
        const double e = __fma_rn(-r2, sol_seed_square(yf), 1.0);
        const double corr = __fma_rn(0.5, e, sol_one_plus_ce2(e, 0.375f));
        const double t = sm[q] * sol_seed_double(yf);
        acc = r2 > 0.0 ? __fma_rn(t, corr, acc) : acc + sm[q] * __longlong_as_double(0x7FF0000000000000LL);
      }
    // compensated running sum of the blocks (Knuth's TwoSum) while it is finite
    const double u = s + acc;
    if (isfinite(u)) {
      const double bp = u - s;
      c += (s - (u - bp)) + (acc - bp);
    }
    s = u;
  }
  red[threadIdx.x] = i < n ? mi * (s + c) : 0.0;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < kPotBlock; ++k) t += red[k];
    part[I] = t;
  }
}

// FP64 pipe throughput: kRateChains independent chains of one FP64
// instruction kind per thread (OP 0 DFMA, 1 DADD, 2 DMUL), a grid of exactly
// the CTAs the SMs hold at once.  Thread 0 of CTA 0 records the SM cycles
// (clock64) and the nanoseconds (%globaltimer) between its first and last
// chain step: their ratio is the SM clock the rate was measured at.  (The
// CTA's own duration is not the launch's: the warp schedulers favour the
// oldest warps, so the CTAs of an SM largely finish one after another.)
// Chains converge (v -> v b + c with b < 1, the sum and product kept near
// 1): no subnormal or special operand is ever formed.
constexpr int kRateChains = 16;
constexpr int kRateThreads = 256;

template <int OP>
__global__ void __launch_bounds__(kRateThreads) k_fp64_rate(double b, double c, double* out, long long* cycles,
                                                            int iters) {
  double v[kRateChains];
#pragma unroll
  for (int k = 0; k < kRateChains; ++k) v[k] = 1.0 + threadIdx.x * 1e-12 + k * 1e-6;
  const long long t0 = clock64();
  unsigned long long g0 = 0, g1 = 0;
  if (blockIdx.x == 0 && threadIdx.x == 0) asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(g0));
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int k = 0; k < kRateChains; ++k) {
      if constexpr (OP == 0) v[k] = __fma_rn(v[k], b, c);
      if constexpr (OP == 1) v[k] = __dadd_rn(v[k], (it & 1) ? c : -c);
      if constexpr (OP == 2) v[k] = __dmul_rn(v[k], (it & 1) ? b : 1.0 / b);
    }
  }
  const long long t1 = clock64();
  if (blockIdx.x == 0 && threadIdx.x == 0) asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(g1));
  double s = 0;
#pragma unroll
  for (int k = 0; k < kRateChains; ++k) s += v[k];
  if (s == -12345.0) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    cycles[0] = t1 - t0;
    cycles[1] = (long long)(g1 - g0);
  }
}

// FP32 pipe throughput: OP 0 scalar FFMA chains, OP 1 paired FFMA2 chains
// (two lanes per instruction), kRateChains per thread as above; the rate is
// counted in FP32 lane operations (an FFMA2 is two).
template <int OP>
__global__ void __launch_bounds__(kRateThreads) k_fp32_rate(float b, float c, float* out, long long* cycles,
                                                            int iters) {
  float2 v[kRateChains];
#pragma unroll
  for (int k = 0; k < kRateChains; ++k) v[k] = make_float2(1.0f + threadIdx.x * 1e-7f + k * 1e-4f, 1.0f - k * 1e-4f);
  const long long t0 = clock64();
  unsigned long long g0 = 0, g1 = 0;
  if (blockIdx.x == 0 && threadIdx.x == 0) asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(g0));
  const float2 b2 = make_float2(b, b), c2 = make_float2(c, c);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int k = 0; k < kRateChains; ++k) {
      if constexpr (OP == 0) v[k].x = __fmaf_rn(v[k].x, b, c);
      if constexpr (OP == 1) v[k] = __ffma2_rn(v[k], b2, c2);
    }
  }
  const long long t1 = clock64();
  if (blockIdx.x == 0 && threadIdx.x == 0) asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(g1));
  float s = 0;
#pragma unroll
  for (int k = 0; k < kRateChains; ++k) s += v[k].x + v[k].y;
  if (s == -12345.0f) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    cycles[0] = t1 - t0;
    cycles[1] = (long long)(g1 - g0);
  }
}

// Self-check of sol_ref_rinv3 (correctly rounded sqrt and 1 / (a sqrt a))
// and of its reciprocal step against IEEE sqrt and division, on seeded
// samples (splitmix64 of the sample index):
//   0: a log-uniform over [2^-200, 2^200];
//   1: a = (1 + i 2^-25 + (i^2 +- 1) 2^-52) 4^k, whose square root lies
//      i 2^-27 ulp from a midpoint (i < 11,000): both sides of the 2^-16 band;
//   2: a = squared distance of two positions uniform in a 100 AU box;
//   3: d = (1 - x 2^-53) 2^s (x odd < 2^21), whose reciprocal lies x^2 2^-54
//      ulp from a midpoint, from approximations up to 300 ulps off;
//   4: d log-uniform over [2^-200, 2^200], approximations up to 300 ulps off;
//   5: a = (1 + u, 2 +- u or 4 - u) 4^k, u log-uniform over [2^-60, 2^-10]:
//      square roots and reciprocals next to powers of two;
//   6: the integer-pipe multiply sol_exact_dmul against the FP64 instruction,
//      random signed operands with exponents over [2^-300, 2^300];
//   7: the same with significands whose product sits next to 2^104 or 2^106,
//      zeros and squares;
//   8, 9: the step-size powers pow(em, -0.2) and pow(em, -0.25)
//      (sol_inv_root; the exponent is the double -0.2, slightly beyond -1/5),
//      em log-uniform over [2^-13, 2^30]: y = em^-e is correctly rounded iff
//      em^(N e) t^N - 1 (N e = 1 + 5 delta for the double 0.2), evaluated in
//      double-double at the midpoints t = y -+ ulp/2, changes sign between
//      them.
__device__ __forceinline__ unsigned long long mix64(unsigned long long x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

__device__ __forceinline__ double unit_double(unsigned long long h) { return (double)(h >> 11) * 0x1.0p-53; }


// em' t^N - 1 for t = th + tl (double-double), em' = em + el, in
// double-double; its sign
__device__ __forceinline__ int root_residual_sign(double em, double el, double th, double tl, int N) {
  // p = t^N by repeated double-double multiplication
  double ph = th, pl = tl;
  for (int k = 1; k < N; ++k) {
    const double h = ph * th;
    const double l = __fma_rn(ph, th, -h) + (ph * tl + pl * th);
    ph = h + l;
    pl = l - (ph - h);
  }
  const double qh = em * ph;
  const double ql = __fma_rn(em, ph, -qh) + (em * pl + el * ph);
  const double d = (qh - 1.0) + ql;  // qh - 1 is exact (qh near 1)
  return (d > 0.0) - (d < 0.0);
}

__global__ void k_check_rinv3(int mode, long long n, unsigned long long seed, unsigned long long* counts,
                              long long* first) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x; s < n; s += stride) {
    const unsigned long long h1 = mix64(seed ^ mix64((unsigned long long)s));
    const unsigned long long h2 = mix64(h1);
    bool ok = true, bad = false;
    if (mode >= 8) {
      const long long E = 1023 - 13 + (long long)(h2 % 44);
      const double em = __longlong_as_double((E << 52) | (long long)(h1 & 0xFFFFFFFFFFFFFull));
      const int N = mode == 8 ? 5 : 4;
      const double y = N == 5 ? sol_inv_root<5>(em) : sol_inv_root<4>(em);
      const long long yb = __double_as_longlong(y);
      const double half = 0.5 * (__longlong_as_double(yb + 1) - y);   // half an ulp above y
      const double halfd = 0.5 * (y - __longlong_as_double(yb - 1));  // half an ulp below y
      // em^(N e) = em em^(N delta) = em (1 + N delta ln em)
      const double el = N == 5 ? em * (5.0 / 90071992547409920.0) * log(em) : 0.0;
      bad = !(root_residual_sign(em, el, y, -halfd, N) <= 0 && root_residual_sign(em, el, y, half, N) >= 0);
    } else if (mode >= 6) {
      unsigned long long ea = 1023 - 300 + (h1 >> 52) % 601, eb = 1023 - 300 + (h2 >> 52) % 601;
      unsigned long long ma = h1 & 0xFFFFFFFFFFFFFull, mb = h2 & 0xFFFFFFFFFFFFFull;
      if (mode == 7) {
        const unsigned w = (unsigned)((h1 >> 44) & 3);
        if (w == 0) {
          ma |= 0xFFFFFFF000000ull;
          mb |= 0xFFFFFFF000000ull;
        } else if (w == 1) {
          ma &= 0x0000000FFFFFFull;
          mb &= 0x00000000FFFFFull;
        } else if (w == 2) {
          mb = ma;
          eb = ea;
        } else if ((h2 >> 40) & 1) {
          ma = 0;
          ea = 0;
        } else {
          mb = 0;
          eb = 0;
        }
      }
      const double a = __longlong_as_double((long long)((ea << 52) | ma | ((h1 & 1ull) << 63)));
      const double b = __longlong_as_double((long long)((eb << 52) | mb | ((h2 & 1ull) << 63)));
      const double e = sol_exact_dmul(a, b, ok);
      bad = ok && (__double_as_longlong(e) != __double_as_longlong(__dmul_rn(a, b)));
    } else if (mode <= 2 || mode == 5) {
      double a;
      if (mode == 5) {
        const double u = unit_double(h1) * __longlong_as_double((long long)(1023 - 10 - (long long)(h2 % 51)) << 52);
        const int w = (int)((h2 >> 32) % 4);
        const double m = w == 0 ? 1.0 + u : w == 1 ? 2.0 + u : w == 2 ? 2.0 - u : 4.0 - u;
        const long long k = (long long)((h2 >> 40) % 201) - 100;
        a = m * __longlong_as_double((1023 + 2 * k) << 52);
      } else if (mode == 0) {
        const long long E = 1023 - 200 + (long long)(h2 % 401);
        a = __longlong_as_double((E << 52) | (long long)(h1 & 0xFFFFFFFFFFFFFull));
      } else if (mode == 1) {
        const long long i = 1 + (long long)(h1 % 11000);
        const long long t = i * i + (((h1 >> 40) & 1) ? 1 : -1);
        const long long k = (long long)(h2 % 201) - 100;
        a = __longlong_as_double(((1023 + 2 * k) << 52) | ((i << 27) + t));
      } else {
        const unsigned long long h3 = mix64(h2), h4 = mix64(h3), h5 = mix64(h4), h6 = mix64(h5);
        const double dx = 100.0 * unit_double(h1) - 100.0 * unit_double(h2);
        const double dy = 100.0 * unit_double(h3) - 100.0 * unit_double(h4);
        const double dz = 100.0 * unit_double(h5) - 100.0 * unit_double(h6);
        a = dx * dx + dy * dy + dz * dz;
      }
      double r, rm3;
      ok = sol_ref_rinv3_fast(a, r, rm3);
      if (ok) {
        const double rr = __dsqrt_rn(a);
        const double w = __ddiv_rn(1.0, a * rr);
        bad = (__double_as_longlong(r) != __double_as_longlong(rr)) ||
              (__double_as_longlong(rm3) != __double_as_longlong(w));
      }
    } else {
      double d;
      if (mode == 3) {
        const long long x = (long long)((h1 % (1ull << 21)) | 1ull);
        const long long sc = (long long)(h2 % 201) - 100;
        d = __longlong_as_double(((1022 + sc) << 52) | ((1LL << 52) - x));
      } else {
        const long long E = 1023 - 200 + (long long)(h2 % 401);
        d = __longlong_as_double((E << 52) | (long long)(h1 & 0xFFFFFFFFFFFFFull));
      }
      const double w = __ddiv_rn(1.0, d);
      const long long zb = __double_as_longlong(w) + ((long long)((h2 >> 20) % 601) - 300);
      const long long wb = solcr::rcp_from_approx(d, zb, ok);
      bad = ok && (wb != __double_as_longlong(w));
    }
    if (!ok) atomicAdd(&counts[1], 1ull);
    if (bad) {
      atomicAdd(&counts[0], 1ull);
      atomicMin(reinterpret_cast<unsigned long long*>(first), (unsigned long long)s);
    }
  }
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

int sol_potential_launch(sol_ctx* c, const double* d_y0, double* d_part, int* nparts) {
  const int g = (c->n + kPotBlock - 1) / kPotBlock;
  k_potential_pairs<<<g, kPotBlock, 0, c->stream>>>(c->n, d_y0, c->d_mass, d_part);
  *nparts = g;
  SOL_LAUNCHED();
  return SOL_OK;
}

namespace {
template <int OP>
int fp64_rate_one(int nsm, double* out, long long* d_cycles, double* rate, double* mhz) {
  int per_sm = 0;
  SOL_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fp64_rate<OP>, kRateThreads, 0));
  if (per_sm < 1) per_sm = 1;
  const int blocks = nsm * per_sm, iters = 8192;
  const double b = 1.0 - 1.0 / 1048576.0, c = 1.0 / 1048576.0;
  cudaEvent_t e0, e1;
  SOL_CUDA(cudaEventCreate(&e0));
  SOL_CUDA(cudaEventCreate(&e1));
  k_fp64_rate<OP><<<blocks, kRateThreads>>>(b, c, out, d_cycles, 1024);  // warm-up (clocks ramp)
  SOL_LAUNCHED();
  float best = 1e30f;
  long long best_cycles[2] = {0, 1};
  for (int rep = 0; rep < 5; ++rep) {
    SOL_CUDA(cudaEventRecord(e0));
    k_fp64_rate<OP><<<blocks, kRateThreads>>>(b, c, out, d_cycles, iters);
    SOL_LAUNCHED();
    SOL_CUDA(cudaEventRecord(e1));
    SOL_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    SOL_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    if (ms < best) {
      best = ms;
      SOL_CUDA(cudaMemcpy(best_cycles, d_cycles, 2 * sizeof(long long), cudaMemcpyDeviceToHost));
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *rate = (double)blocks * kRateThreads * kRateChains * iters / (best * 1e-3);
  *mhz = best_cycles[1] > 0 ? 1e3 * (double)best_cycles[0] / (double)best_cycles[1] : 0.0;
  return SOL_OK;
}
}  // namespace

int sol_fp64_rates_launch(int device, double rates[3], double* sm_mhz) {
  SOL_CUDA(cudaSetDevice(device));
  int nsm = 0, max_per_sm = 32;
  SOL_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device));
  double* out = nullptr;
  long long* cyc = nullptr;
  SOL_CUDA(cudaMalloc(&out, sizeof(double) * (size_t)nsm * max_per_sm * kRateThreads));
  SOL_CUDA(cudaMalloc(&cyc, 2 * sizeof(long long)));
  double mhz[3] = {0, 0, 0};
  int rc = fp64_rate_one<0>(nsm, out, cyc, &rates[0], &mhz[0]);
  if (rc == SOL_OK) rc = fp64_rate_one<1>(nsm, out, cyc, &rates[1], &mhz[1]);
  if (rc == SOL_OK) rc = fp64_rate_one<2>(nsm, out, cyc, &rates[2], &mhz[2]);
  cudaFree(out);
  cudaFree(cyc);
  if (rc == SOL_OK && sm_mhz) *sm_mhz = mhz[0];
  return rc;
}

namespace {
template <int OP>
int fp32_rate_one(int nsm, float* out, long long* d_cycles, double* rate, double* mhz) {
  int per_sm = 0;
  SOL_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fp32_rate<OP>, kRateThreads, 0));
  if (per_sm < 1) per_sm = 1;
  const int blocks = nsm * per_sm, iters = 65536;
  const float b = 1.0f - 1.0f / 4096.0f, c = 1.0f / 4096.0f;
  cudaEvent_t e0, e1;
  SOL_CUDA(cudaEventCreate(&e0));
  SOL_CUDA(cudaEventCreate(&e1));
  k_fp32_rate<OP><<<blocks, kRateThreads>>>(b, c, out, d_cycles, 4096);  // warm-up
  SOL_LAUNCHED();
  float best = 1e30f;
  long long best_cycles[2] = {0, 1};
  for (int rep = 0; rep < 5; ++rep) {
    SOL_CUDA(cudaEventRecord(e0));
    k_fp32_rate<OP><<<blocks, kRateThreads>>>(b, c, out, d_cycles, iters);
    SOL_LAUNCHED();
    SOL_CUDA(cudaEventRecord(e1));
    SOL_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    SOL_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    if (ms < best) {
      best = ms;
      SOL_CUDA(cudaMemcpy(best_cycles, d_cycles, 2 * sizeof(long long), cudaMemcpyDeviceToHost));
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  const double lanes = OP == 1 ? 2.0 : 1.0;
  *rate = lanes * (double)blocks * kRateThreads * kRateChains * iters / (best * 1e-3);
  *mhz = best_cycles[1] > 0 ? 1e3 * (double)best_cycles[0] / (double)best_cycles[1] : 0.0;
  return SOL_OK;
}
}  // namespace

int sol_fp32_rates_launch(int device, double rates[2], double* sm_mhz) {
  SOL_CUDA(cudaSetDevice(device));
  int nsm = 0;
  SOL_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device));
  float* out = nullptr;
  long long* cyc = nullptr;
  SOL_CUDA(cudaMalloc(&out, sizeof(float) * (size_t)nsm * 32 * kRateThreads));
  SOL_CUDA(cudaMalloc(&cyc, 2 * sizeof(long long)));
  double mhz[2] = {0, 0};
  int rc = fp32_rate_one<0>(nsm, out, cyc, &rates[0], &mhz[0]);
  if (rc == SOL_OK) rc = fp32_rate_one<1>(nsm, out, cyc, &rates[1], &mhz[1]);
  cudaFree(out);
  cudaFree(cyc);
  if (rc == SOL_OK && sm_mhz) *sm_mhz = mhz[1];
  return rc;
}

int sol_fp64_peak_launch(int device, double* flops) {
  double rates[3], mhz = 0;
  const int rc = sol_fp64_rates_launch(device, rates, &mhz);
  if (rc == SOL_OK) *flops = 2.0 * rates[0];
  return rc;
}

int sol_check_pair_math_launch(int device, int mode, long long n, unsigned long long seed, long long* result) {
  SOL_CUDA(cudaSetDevice(device));
  int nsm = 0;
  SOL_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device));
  unsigned long long* d = nullptr;
  SOL_CUDA(cudaMalloc(&d, 3 * sizeof(unsigned long long)));
  const unsigned long long init[3] = {0ull, 0ull, ~0ull};
  int rc = SOL_OK;
  if (cudaMemcpy(d, init, sizeof(init), cudaMemcpyHostToDevice) != cudaSuccess) rc = SOL_ERR_CUDA;
  if (rc == SOL_OK) {
    k_check_rinv3<<<nsm * 8, 256>>>(mode, n, seed, d, reinterpret_cast<long long*>(d + 2));
    SOL_LAUNCHED();
    unsigned long long h[3];
    if (cudaGetLastError() != cudaSuccess || cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = SOL_ERR_CUDA;
    else {
      result[0] = (long long)h[0];
      result[1] = (long long)h[1];
      result[2] = h[2] == ~0ull ? -1 : (long long)h[2];
    }
  }
  cudaFree(d);
  if (rc != SOL_OK) sol_set_error("pair arithmetic self-check: CUDA error");
  return rc;
}
