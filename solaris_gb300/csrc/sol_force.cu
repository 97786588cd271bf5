// Force evaluation: the GB300 replacement of Acceleration::Compute
// (Solaris/Acceleration.cpp:60-246) and its gravity, gas-drag and migration
// terms.
//
// One evaluation is three launches:
//   k_prepass     one thread per body: rm3[j] = 1/|r_j|^3 exactly as
//                 GravityAC computes it (:256-264), and the structure-of-arrays
//                 source table {x, y, z, G m, x rm3, y rm3, z rm3} that the pair
//                 kernel streams; per-block partial sums of the indirect term.
//   k_ind_reduce  one block: the indirect-term totals (SPLIT only).
//   k_gravity_*   one thread per sink body; source tiles of TJ bodies are
//                 staged in shared memory by bulk copies (cp.async.bulk, the
//                 TMA engine) completing on an mbarrier, double buffered.  The
//                 epilogue adds gas drag and type-I/II migration for the sink.
#include <cstdio>
#include <cstring>
#include <atomic>
#include <mutex>

#include "sol_internal.cuh"
#include "sol_crmath.cuh"
#include "sol_pair.cuh"

int sol_force_uses_chunk_partials(const sol_ctx* c, int precision);

namespace {

constexpr int kSinkBlock = 128;  // sinks per CTA
constexpr int kTile = 256;       // sources per shared-memory tile
constexpr int kPrepassBlock = 256;

enum SrcArray { SX = 0, SY, SZ, SGM, SPX, SPY, SPZ, SGF, SRC_ARRAYS = 8 };  // SGF: G m as (hi, lo) floats
// Float table of the SPLIT_FF 2-D kernel, after the SRC_ARRAYS doubles: each
// coordinate as its grid triple a + b + c (f2_grid_disp in sol_pair.cuh) and
// G m as (hi, lo), one float array each (two sources load as one float2).
enum FTab { FAX = 0, FBX, FCX, FAY, FBY, FCY, FAZ, FBZ, FCZ, FGH, FGL, FTAB_USED = 11, FTAB_ARRAYS = 12 };
constexpr int kSrcDoubles = SRC_ARRAYS + FTAB_ARRAYS / 2;  // doubles per padded body in the source table
// ind_sum slots: [0..5] the indirect sums, [6] the grid G1 of the float table,
// [7] (low word) the running maximum |coordinate| as FP32 bits (atomicMax)
constexpr int kIndGrid = 6, kIndMaxWord = 7;

constexpr int kChunkTiles = 16;             // sources per work unit of the 2-D pair kernel
constexpr int kChunk = kChunkTiles * kTile;  // 4,096
enum PartSlot { PAX = 0, PAY, PAZ, PR2, PIDX, PART_SLOTS = 5 };

__device__ __forceinline__ double eval_time(const TimeSpec& ts) {
  return ts.base ? (*ts.base + ts.c * (*ts.h)) : ts.t_host;
}

// ---- prepass ----------------------------------------------------------------
__device__ __forceinline__ float* ftab(const ForceCtx& fc) { return reinterpret_cast<float*>(fc.src + (size_t)SRC_ARRAYS * fc.npad); }

// prec: SOL_PRECISION_*.  The split forms also sum the indirect term; SPLIT_FF
// (2-D kernel, ff = 1) also takes the largest |coordinate| and writes G m as
// float (hi, lo) arrays of the float table.
__global__ void k_prepass(ForceCtx fc, const double* __restrict__ y, int split, int ff) {
  const int n = fc.cls.n;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  double q[6] = {0, 0, 0, 0, 0, 0};  // indirect contributions: massive range, super-planetesimal range
  unsigned mbits = 0;                 // |coordinate| maximum as FP32 bits, rounded up
  if (j < fc.npad) {
    double x = 0, yy = 0, z = 0, gm = 0, px = 0, py = 0, pz = 0;
    if (j < n) {
      x = y[6 * j + 0];
      yy = y[6 * j + 1];
      z = y[6 * j + 2];
      double rm3 = 0.0;
      if (j >= 1) {
        if (!fc.barycentric) {
          // Acceleration.cpp:259-261
          double r2 = x * x + yy * yy + z * z;
          double r;
          sol_ref_rinv3(r2, r, rm3);
          fc.rm3[j] = rm3;
        }
        gm = SOL_GAUSS2 * fc.mass[j];
      }
      px = x * rm3;
      py = yy * rm3;
      pz = z * rm3;
      if (fc.barycentric) gm = fc.mass[j];  // GravityBC uses m_j and scales by G at the end
      if (split && j >= 1) {
        int slot = (j < fc.cls.nm) ? 0 : ((j < fc.cls.nm + fc.cls.n_spl) ? 3 : -1);
        if (slot >= 0) {
          q[slot + 0] = gm * px;
          q[slot + 1] = gm * py;
          q[slot + 2] = gm * pz;
        }
      }
    }
    double* s = fc.src;
    const int np = fc.npad;
    s[SX * np + j] = x;
    s[SY * np + j] = yy;
    s[SZ * np + j] = z;
    s[SGM * np + j] = gm;
    s[SPX * np + j] = px;
    s[SPY * np + j] = py;
    s[SPZ * np + j] = pz;
    float gh = __double2float_rn(gm);
    float gl = __double2float_rn(gm - (double)gh);
    reinterpret_cast<float2*>(s + (size_t)SGF * np)[j] = make_float2(gh, gl);
    if (ff) {
      float* T = ftab(fc);
      T[(size_t)FGH * np + j] = gh;
      T[(size_t)FGL * np + j] = gl;
      const double m = fmax(fabs(x), fmax(fabs(yy), fabs(z)));
      mbits = __float_as_uint(__double2float_ru(m));
    }
  }
  if (ff) {
    const unsigned wmax = __reduce_max_sync(0xFFFFFFFFu, mbits);
    if ((threadIdx.x & 31) == 0 && wmax) atomicMax(reinterpret_cast<unsigned*>(fc.ind_sum + kIndMaxWord), wmax);
  }
  if (!split) return;
  // fixed-order block tree reduction of the indirect contributions
  __shared__ double red[6][kPrepassBlock];
  for (int k = 0; k < 6; ++k) red[k][threadIdx.x] = q[k];
  __syncthreads();
  for (int w = kPrepassBlock / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
      for (int k = 0; k < 6; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int k = 0; k < 6; ++k) fc.ind_part[6 * blockIdx.x + k] = red[k][0];
}

__global__ void k_ind_reduce(ForceCtx fc) {
  // one block of 256 threads: strided partial sums then a fixed tree.
  __shared__ double red[6][256];
  double a[6] = {0, 0, 0, 0, 0, 0};
  for (int b = threadIdx.x; b < fc.n_ind_blocks; b += blockDim.x)
    for (int k = 0; k < 6; ++k) a[k] += fc.ind_part[6 * b + k];
  for (int k = 0; k < 6; ++k) red[k][threadIdx.x] = a[k];
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w)
      for (int k = 0; k < 6; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    // [0..2]: sum over [1, nm); [3..5]: sum over [1, nm + n_spl)
    for (int k = 0; k < 3; ++k) {
      fc.ind_sum[k] = red[k][0];
      fc.ind_sum[3 + k] = red[k][0] + red[3 + k][0];
    }
    // the float table's grid: G1 = 2^(E - 23) with every |coordinate| < 2^E
    // (then read and cleared for the next evaluation's maximum)
    unsigned* word = reinterpret_cast<unsigned*>(fc.ind_sum + kIndMaxWord);
    const unsigned mb = *word;
    const int E = mb ? (int)((mb >> 23) & 0xFFu) - 127 + 1 : 0;
    fc.ind_sum[kIndGrid] = ldexp(1.0, max(E, -90) - 23);
    *word = 0u;
  }
}

// Grid triples of every coordinate (f2_grid_disp): a = G1 rint(x / G1),
// b = G2 rint((x - a) / G2), c = float(x - a - b); a and b are exact floats
// (at most 2^23 of their grid), x - a and x - a - b exact doubles.  Padding
// bodies get zeros.
__global__ void k_split_table(ForceCtx fc, const double* __restrict__ y) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= fc.npad) return;
  const double G1 = fc.ind_sum[kIndGrid];
  const double G2 = G1 * 0x1.0p-24;
  const double iG1 = 1.0 / G1, iG2 = 1.0 / G2;  // powers of two: exact
  float* T = ftab(fc);
  const int np = fc.npad;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const double x = j < fc.cls.n ? y[6 * j + k] : 0.0;
    const double a = rint(x * iG1) * G1;
    const double r = x - a;
    const double b = rint(r * iG2) * G2;
    T[(size_t)(FAX + 3 * k) * np + j] = (float)a;
    T[(size_t)(FBX + 3 * k) * np + j] = (float)b;
    T[(size_t)(FCX + 3 * k) * np + j] = __double2float_rn(r - b);
  }
}

// ---- tile pipeline -----------------------------------------------------------
template <int NARR>
struct TileSmem {
  double v[2][NARR][kTile];
  uint64_t bar[2];
};

template <int NARR>
__device__ __forceinline__ void issue_tile(TileSmem<NARR>& sm, const double* src, int npad, int tile, int stage) {
  sol_mbar_expect_tx(&sm.bar[stage], NARR * kTile * 8);
  for (int k = 0; k < NARR; ++k)
    sol_bulk_g2s(&sm.v[stage][k][0], src + (size_t)k * npad + (size_t)tile * kTile, kTile * 8, &sm.bar[stage]);
}

// Reference-form pair arithmetic (GravityAC, Acceleration.cpp:294-317): IEEE
// sqrt and division, no contraction, sources in ascending order.
__device__ __forceinline__ void pair_fp64(const TileSmem<7>& sm, int st, int jj, int j, int i, int ns, double xi,
                                          double yi, double zi, double& ax, double& ay, double& az, long long& rminb,
                                          int& nn) {
  if (j >= 1 && j < ns && j != i) {
    double xij = sm.v[st][SX][jj] - xi;
    double yij = sm.v[st][SY][jj] - yi;
    double zij = sm.v[st][SZ][jj] - zi;
    double rij2 = xij * xij + yij * yij + zij * zij;
    double rij, rijm3;
    sol_ref_rinv3(rij2, rij, rijm3);
    long long rb = __double_as_longlong(rij);
    if (rb < rminb) {
      rminb = rb;
      nn = j;
    }
    double gm = sm.v[st][SGM][jj];
    ax += gm * (xij * rijm3 - sm.v[st][SPX][jj]);
    ay += gm * (yij * rijm3 - sm.v[st][SPY][jj]);
    az += gm * (zij * rijm3 - sm.v[st][SPZ][jj]);
  }
}

// Split pair arithmetic: FP64 displacement and r^2; rsqrt seed in FP32 with
// the FP64 <-> FP32 conversions done by integer operations on the bit
// patterns (they stay off the FP64 pipe); one FP64 Newton correction of
// r^-3 carried to second order in the residual e = 1 - r^2 y0^2:
//   r^-3 = y0^3 (1 - e)^(-3/2) = y0^3 (1 + 3/2 e + 15/8 e^2 + O(e^3)),
// |e| < 2^-20, so the truncation is below 1e-18.  The seed's square and cube
// come from the integer pipe (sol_seed_square_cube), and so does t = 3/2 e +
// 15/8 e^2 (sol_split_t), leaving FP64 the residual e, G m y0^3 and
// G m y0^3 + (G m y0^3) t by one DFMA (split_gm_rinv3): with the
// displacement, r^2 and the three accumulations, 12 FP64 operations per pair,
// the floor of this recipe.
__device__ __forceinline__ double split_gm_rinv3(double r2, double gm) {
  // the seed of r2 == 0 (the sink itself) is finite
  double u, y3;
  sol_seed_square_cube(sol_rsqrt_seed(r2), u, y3);
  const double e = __fma_rn(-r2, u, 1.0);
  const double gy = gm * y3;
  return __fma_rn(gy, sol_split_t(e), gy);
}

__device__ __forceinline__ void pair_split(const TileSmem<4>& sm, int st, int jj, int j, int i, int ns, double xi,
                                           double yi, double zi, double& ax, double& ay, double& az,
                                           long long& r2minb, int& nn) {
  double dx = sm.v[st][SX][jj] - xi;
  double dy = sm.v[st][SY][jj] - yi;
  double dz = sm.v[st][SZ][jj] - zi;
  double r2 = __fma_rn(dx, dx, __fma_rn(dy, dy, dz * dz));
  double gm = (j < ns) ? sm.v[st][SGM][jj] : 0.0;  // gm of j == 0 and of padding is 0
  double s = split_gm_rinv3(r2, gm);
  ax = __fma_rn(s, dx, ax);
  ay = __fma_rn(s, dy, ay);
  az = __fma_rn(s, dz, az);
  long long rb = __double_as_longlong(r2);
  bool better = (rb < r2minb) & (j >= 1) & (j < ns) & (j != i);
  r2minb = better ? rb : r2minb;
  nn = better ? j : nn;
}

__device__ __forceinline__ void two_sum(double& s, double& c, double a) {
  double t = s + a;
  double bp = t - s;
  double err = (s - (t - bp)) + (a - bp);
  s = t;
  c += err;
}

// spin: the limit of every mbarrier wait; withhold >= 0: that tile is never
// copied, so its wait runs out (failure-path tests only; -1 in production).
template <int PREC>
__global__ void __launch_bounds__(kSinkBlock) k_gravity_ac(ForceCtx fc, const double* __restrict__ y,
                                                           double* __restrict__ dydt, TimeSpec ts, uint32_t flags,
                                                           int* dev_status, uint32_t spin, int withhold) {
  constexpr int NARR = (PREC == SOL_PRECISION_FP64) ? 7 : 4;
  __shared__ __align__(128) TileSmem<NARR> sm;
  const Classes& c = fc.cls;
  const int n = sol_sink_hi(fc);  // sinks [sink_lo, n)
  const int i = fc.sink_lo + blockIdx.x * kSinkBlock + threadIdx.x;
  const int i_first = fc.sink_lo + blockIdx.x * kSinkBlock;
  // NOfMassive of GravityAC (:285-289); types are sorted, so the first sink
  // of the CTA has the largest source range.
  const int ns_cta = (fc.type[min(i_first, n - 1)] <= SOL_PROTO_PLANET) ? c.nm + c.n_spl : c.nm;
  const int ns = (i < n && fc.type[i] <= SOL_PROTO_PLANET) ? c.nm + c.n_spl : c.nm;
  const int ntiles = (ns_cta + kTile - 1) / kTile;

  double xi = 0, yi = 0, zi = 0;
  if (i < n) {
    xi = y[6 * i + 0];
    yi = y[6 * i + 1];
    zi = y[6 * i + 2];
  }
  if (threadIdx.x == 0) {
    sol_mbar_init(&sm.bar[0], 1);
    sol_mbar_init(&sm.bar[1], 1);
    sol_fence_barrier_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (ntiles > 0 && withhold != 0) issue_tile<NARR>(sm, fc.src, fc.npad, 0, 0);
    if (ntiles > 1 && withhold != 1) issue_tile<NARR>(sm, fc.src, fc.npad, 1, 1);
  }

  double ax = 0.0, ay = 0.0, az = 0.0;  // FP64: running sums; SPLIT: tile partials
  double sx = 0.0, sy = 0.0, sz = 0.0, cx = 0.0, cy = 0.0, cz = 0.0;  // SPLIT compensated totals
  long long rminb = (PREC == SOL_PRECISION_FP64) ? __double_as_longlong(1.0e10) : __double_as_longlong(1.0e20);
  int nn = -1;
  int issued = ntiles < 2 ? ntiles : 2;
  int t = 0;
  bool timed_out = false;

  for (; t < ntiles; ++t) {
    const int st = t & 1;
    const uint32_t parity = (t >> 1) & 1;
    const bool ok = sol_mbar_wait_n(&sm.bar[st], parity, spin);
    const int j0 = t * kTile;
    const int jmax = min(kTile, ns_cta - j0);  // sources beyond the CTA's range are never read
    if (ok && i < n && i >= 1) {
      if constexpr (PREC == SOL_PRECISION_FP64) {
#pragma unroll 4
        for (int jj = 0; jj < jmax; ++jj)
          pair_fp64(*reinterpret_cast<TileSmem<7>*>(&sm), st, jj, j0 + jj, i, ns, xi, yi, zi, ax, ay, az, rminb,
                    nn);
      } else {
        double tx = 0.0, ty = 0.0, tz = 0.0;
#pragma unroll 4
        for (int jj = 0; jj < jmax; ++jj)
          pair_split(*reinterpret_cast<TileSmem<4>*>(&sm), st, jj, j0 + jj, i, ns, xi, yi, zi, tx, ty, tz, rminb,
                     nn);
        two_sum(sx, cx, tx);
        two_sum(sy, cy, ty);
        two_sum(sz, cz, tz);
      }
    }
    // every thread is done with stage st; a timeout anywhere stops the whole CTA
    if (__syncthreads_or(!ok)) {
      timed_out = true;
      break;
    }
    if (threadIdx.x == 0 && t + 2 < ntiles) {
      sol_fence_proxy_async();
      if (t + 2 != withhold) issue_tile<NARR>(sm, fc.src, fc.npad, t + 2, st);
    }
    if (t + 2 < ntiles) issued = t + 3;
  }
  if (timed_out) {
    if (threadIdx.x == 0) {
      atomicOr(dev_status, SOL_DEV_TIMEOUT);
      // drain the copies still in flight (bounded) before the CTA exits
      for (int u = t; u < issued; ++u) sol_mbar_wait_n(&sm.bar[u & 1], (u >> 1) & 1, spin);
    }
    __syncthreads();
    return;
  }
  if (i >= n) return;
  double* out = dydt + 6 * i;
  if (i == 0) {  // GravityAC :253-254, :266
    for (int k = 0; k < 6; ++k) out[k] = 0.0;
    fc.nn_idx[0] = -1;
    fc.nn_dist[0] = 0.0;
    return;
  }
  const double* yv = y + 6 * i;
  const double mu = SOL_GAUSS2 * (fc.mass[0] + fc.mass[i]);
  const double rm3i = fc.rm3[i];
  double a[3];
  a[0] = -mu * rm3i * xi;  // Kepler term first (:281-283)
  a[1] = -mu * rm3i * yi;
  a[2] = -mu * rm3i * zi;
  if constexpr (PREC == SOL_PRECISION_FP64) {
    a[0] += ax;
    a[1] += ay;
    a[2] += az;
    fc.nn_idx[i] = nn;
    fc.nn_dist[i] = nn >= 0 ? __longlong_as_double(rminb) : 0.0;
  } else {
    const double* S = fc.ind_sum + ((fc.type[i] <= SOL_PROTO_PLANET) ? 3 : 0);
    const bool src_i = i < ns;
    const double* s = fc.src;
    const int np = fc.npad;
    double own[3] = {0.0, 0.0, 0.0};
    if (src_i) {
      double gmi = s[SGM * np + i];
      own[0] = gmi * s[SPX * np + i];
      own[1] = gmi * s[SPY * np + i];
      own[2] = gmi * s[SPZ * np + i];
    }
    a[0] += (sx + cx) - (S[0] - own[0]);
    a[1] += (sy + cy) - (S[1] - own[1]);
    a[2] += (sz + cz) - (S[2] - own[2]);
    // the reference's rij for the chosen neighbour (Acceleration.cpp:301-305), bit for bit
    double rij = 0.0;
    if (nn >= 0) {
      const double xij = y[6 * nn + 0] - xi, yij = y[6 * nn + 1] - yi, zij = y[6 * nn + 2] - zi;
      rij = __dsqrt_rn(xij * xij + yij * yij + zij * zij);
      if (!(rij < 1.0e10)) nn = -1;
    }
    fc.nn_idx[i] = nn;
    fc.nn_dist[i] = nn >= 0 ? rij : 0.0;
  }
  add_gas_terms(fc, i, yv, eval_time(ts), flags, a);
  out[0] = yv[3];
  out[1] = yv[4];
  out[2] = yv[5];
  out[3] = a[0];
  out[4] = a[1];
  out[5] = a[2];
}

// ---- FP64 GravityAC for systems of up to a few ten thousand bodies ----------
// One thread per sink leaves most SMs idle when the sinks number a few
// thousand or fewer.  Here a CTA takes kFewSinks sinks: producer warps compute
// the pair terms of a tile of kFewTile sources for all of them in parallel
// (the reference's arithmetic, Acceleration.cpp:294-317) into a
// double-buffered shared tile, while warp 0 adds the previous tile's terms
// per sink and component in ascending source order.  The sums are the
// reference's sequential sums, so the result is bit-identical to it and to
// k_gravity_ac, with kFewSinks x kFewTile-way parallelism per CTA.  Measured
// on the GB300 it matches or beats k_gravity_ac from 1,033 to 65,536 bodies
// (9.0 / 13.7 G pairs/s at 1,033 / 32,768 all-massive bodies), so it serves
// every system whose sinks see at least one tile of sources.
constexpr int kFewSinks = 4;
constexpr int kFewProducers = 7;                      // warps 1..7
constexpr int kFewTile = kFewProducers * 32;          // 224 sources per round
constexpr int kFewTerms = kFewSinks * 3;              // (sink, component) lanes of warp 0

__global__ void __launch_bounds__(256) k_gravity_ac_few(ForceCtx fc, const double* __restrict__ y,
                                                        double* __restrict__ dydt, TimeSpec ts, uint32_t flags) {
  // the nearest-neighbour candidates reuse the term tiles once the last one
  // has been added
  static_assert(sizeof(long long) * kFewSinks * kFewTile + sizeof(int) * kFewSinks * kFewTile <=
                    sizeof(double) * 2 * kFewTile * kFewTerms,
                "candidate arrays must fit in the term tiles");
  __shared__ __align__(16) double terms[2][kFewTile][kFewTerms];
  long long(*nn_r)[kFewTile] = reinterpret_cast<long long(*)[kFewTile]>(&terms[0][0][0]);
  int(*nn_j)[kFewTile] = reinterpret_cast<int(*)[kFewTile]>(&terms[0][0][0] + kFewSinks * kFewTile);
  __shared__ double sink_pos[kFewSinks][3];
  __shared__ int sink_ns[kFewSinks];
  __shared__ double acc[kFewTerms];
  const Classes& c = fc.cls;
  const int n = sol_sink_hi(fc);  // sinks [sink_lo, n)
  const int i0 = fc.sink_lo + blockIdx.x * kFewSinks;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x < kFewSinks) {
    const int i = i0 + threadIdx.x;
    const bool live = i < n && i >= 1;
    sink_ns[threadIdx.x] = live ? ((fc.type[i] <= SOL_PROTO_PLANET) ? c.nm + c.n_spl : c.nm) : 0;
    for (int k = 0; k < 3; ++k) sink_pos[threadIdx.x][k] = i < n ? y[6 * i + k] : 0.0;
  }
  __syncthreads();
  int ns_cta = 0;
  for (int s = 0; s < kFewSinks; ++s) ns_cta = max(ns_cta, sink_ns[s]);
  const int rounds = (ns_cta + kFewTile - 1) / kFewTile;
  const double* src = fc.src;
  const int np = fc.npad;

  // producer state: the first minimum over this thread's columns, per sink
  long long rminb[kFewSinks];
  int nn[kFewSinks];
  for (int s = 0; s < kFewSinks; ++s) {
    rminb[s] = __double_as_longlong(1.0e10);
    nn[s] = -1;
  }
  // accumulator state (warp 0, lanes < kFewTerms): lane = component * kFewSinks + sink
  const int a_s = lane % kFewSinks;
  const int a_i = i0 + a_s;
  const int a_ns = (lane < kFewTerms) ? sink_ns[a_s] : 0;
  double a_sum = 0.0;

  // round r: producers fill buffer r & 1 with sources [r * kFewTile, ...);
  // warp 0 adds buffer (r - 1) & 1
  for (int r = 0; r <= rounds; ++r) {
    if (warp > 0 && r < rounds) {
      const int p = threadIdx.x - 32;
      const int j = r * kFewTile + p;
      if (j < ns_cta) {
        const double xj = src[SX * np + j], yj = src[SY * np + j], zj = src[SZ * np + j];
        const double gm = src[SGM * np + j], px = src[SPX * np + j], py = src[SPY * np + j],
                     pz = src[SPZ * np + j];
        double* out = &terms[r & 1][p][0];
        // two sinks per step, branch-free up to the stores (their chains interleave)
#pragma unroll
        for (int s = 0; s < kFewSinks; s += 2) {
          double xij[2], yij[2], zij[2], rij2[2];
          bool valid[2];
#pragma unroll
          for (int u = 0; u < 2; ++u) {
            valid[u] = j >= 1 && j < sink_ns[s + u] && j != i0 + s + u;
            xij[u] = xj - sink_pos[s + u][0];
            yij[u] = yj - sink_pos[s + u][1];
            zij[u] = zj - sink_pos[s + u][2];
            const double q = xij[u] * xij[u] + yij[u] * yij[u] + zij[u] * zij[u];
            rij2[u] = valid[u] ? q : 1.0;
          }
          double rij[2], rijm3[2];
          sol_ref_rinv3_x2(rij2[0], rij2[1], rij[0], rijm3[0], rij[1], rijm3[1]);
#pragma unroll
          for (int u = 0; u < 2; ++u) {
            double tx, ty, tz;
            sol_ref_terms(gm, rijm3[u], xij[u], yij[u], zij[u], px, py, pz, tx, ty, tz);
            if (valid[u]) {
              const long long rb = __double_as_longlong(rij[u]);
              if (rb < rminb[s + u]) {
                rminb[s + u] = rb;
                nn[s + u] = j;
              }
              out[0 * kFewSinks + s + u] = tx;
              out[1 * kFewSinks + s + u] = ty;
              out[2 * kFewSinks + s + u] = tz;
            }
          }
        }
      }
    } else if (warp == 0 && r > 0 && lane < kFewTerms) {
      const int rr = r - 1;
      const int j0 = rr * kFewTile;
      const int pmax = min(kFewTile, a_ns - j0);
      for (int p = 0; p < pmax; ++p) {
        const int j = j0 + p;
        if (j >= 1 && j != a_i) a_sum += terms[rr & 1][p][lane];
      }
    }
    __syncthreads();
  }
  // nearest neighbour: the smallest distance, ties to the lowest index -- the
  // reference's first strict minimum in ascending order
  if (warp > 0) {
    const int p = threadIdx.x - 32;
    for (int s = 0; s < kFewSinks; ++s) {
      nn_r[s][p] = rminb[s];
      nn_j[s][p] = nn[s];
    }
  }
  if (warp == 0 && lane < kFewTerms) acc[lane] = a_sum;
  __syncthreads();
  if (threadIdx.x >= kFewSinks) return;
  const int s = threadIdx.x;
  const int i = i0 + s;
  if (i >= n) return;
  double* out = dydt + 6 * i;
  if (i == 0) {  // GravityAC :253-254, :266
    for (int k = 0; k < 6; ++k) out[k] = 0.0;
    fc.nn_idx[0] = -1;
    fc.nn_dist[0] = 0.0;
    return;
  }
  long long best = __double_as_longlong(1.0e10);
  int bj = -1;
  const int pmax = min(kFewTile, ns_cta);  // producers beyond the source count hold no candidate
  for (int p = 0; p < pmax; ++p) {
    const long long rb = nn_r[s][p];
    const int jb = nn_j[s][p];
    if (jb >= 0 && (rb < best || (rb == best && jb < bj))) {
      best = rb;
      bj = jb;
    }
  }
  const double* yv = y + 6 * i;
  const double xi = sink_pos[s][0], yi = sink_pos[s][1], zi = sink_pos[s][2];
  const double mu = SOL_GAUSS2 * (fc.mass[0] + fc.mass[i]);
  const double rm3i = fc.rm3[i];
  double a[3];
  a[0] = -mu * rm3i * xi;  // Kepler term first (:281-283)
  a[1] = -mu * rm3i * yi;
  a[2] = -mu * rm3i * zi;
  a[0] += acc[0 * kFewSinks + s];
  a[1] += acc[1 * kFewSinks + s];
  a[2] += acc[2 * kFewSinks + s];
  fc.nn_idx[i] = bj;
  fc.nn_dist[i] = bj >= 0 ? __longlong_as_double(best) : 0.0;
  add_gas_terms(fc, i, yv, eval_time(ts), flags, a);
  out[0] = yv[3];
  out[1] = yv[4];
  out[2] = yv[5];
  out[3] = a[0];
  out[4] = a[1];
  out[5] = a[2];
}

// ---- FP64 GravityAC, 32 sinks per CTA ----------------------------------------
// The FP64 pipe spends 64 cycles on every warp instruction however many of
// its lanes are active, so the in-order sums of k_gravity_ac_few (12 of 32
// lanes) cost almost a third of its pair work.  Here a CTA takes up to 32
// sinks and alternates two phases per round of kWideTile sources:
//  A. every thread computes one source's terms against a quarter of the
//     sinks (the reference arithmetic, Acceleration.cpp:294-317) into a
//     shared row; the nearest-neighbour candidates of each sink are reduced
//     across the warp with three 32-bit minimum reductions (high word, low
//     word, index) and kept by one lane of the warp;
//  B. three full warps -- warp c for component c, lane s for sink s -- add the
//     round's terms in ascending source order.
// The sums are the reference's sequential sums (bit-identical to
// k_gravity_ac_few); a sum costs 3 FP64 warp instructions per round.  A CTA
// takes spc <= 32 sinks: the host picks spc so that the CTAs fill whole
// waves of three per SM (the per-round cost 14/32 spc + 3 FP64 warp
// instructions per source, times the waves, is smallest).  A 64-source tile
// (49.7 KB) and 85 registers give three CTAs, 24 warps, per SM: measured at
// 65,536 bodies 151 ms, against 157 ms with four CTAs per SM (64 registers,
// spilling) and 169 ms with a 128-source tile and two.
constexpr int kWideSinks = 32;
constexpr int kWideWarps = 8;
constexpr int kWideCtasPerSm = 3;                      // 24 warps per SM: six per sub-partition
constexpr int kWideTile = 64;                          // sources per round
constexpr int kWideGroups = kWideWarps * 32 / kWideTile;  // sink quarters: thread = (quarter, source)
constexpr int kWideRow = 3 * kWideSinks + 1;           // doubles per source row (odd: conflict-free columns)
constexpr size_t kWideSmem = sizeof(double) * kWideTile * kWideRow;  // 49,664 bytes
constexpr int kMaxDevices = 64;
// below this many sinks per CTA the 4-sink kernel's finer grid wins (measured)
constexpr int kWideMinSinks = 6;

// Phase A of k_gravity_ac_wide for sink s: the pair term into the shared
// row, the warp's nearest-neighbour candidate.
__device__ __forceinline__ void wide_sink(int s, int s0, int j, bool jin, int i0, int lane, double xj, double yj,
                                          double zj, double gm, double px, double py, double pz,
                                          const double (*sink_pos)[3], const int* sink_ns, double* row,
                                          unsigned long long& best, int& best_j) {
  const bool valid = jin && j >= 1 && j < sink_ns[s] && j != i0 + s;
  const double xij = xj - sink_pos[s][0];
  const double yij = yj - sink_pos[s][1];
  const double zij = zj - sink_pos[s][2];
  const double q = xij * xij + yij * yij + zij * zij;
  double rij, rijm3;
  sol_ref_rinv3(valid ? q : 1.0, rij, rijm3);
  double tx, ty, tz;
  sol_ref_terms(gm, rijm3, xij, yij, zij, px, py, pz, tx, ty, tz);
  if (valid) {
    row[0 * kWideSinks + s] = tx;
    row[1 * kWideSinks + s] = ty;
    row[2 * kWideSinks + s] = tz;
  }
  // the warp's smallest (rij, j): high word, then low word, then index
  const unsigned long long key = valid ? (unsigned long long)__double_as_longlong(rij) : ~0ull;
  const unsigned hi = (unsigned)(key >> 32);
  const unsigned mhi = __reduce_min_sync(0xFFFFFFFFu, hi);
  const unsigned lo = (hi == mhi) ? (unsigned)key : 0xFFFFFFFFu;
  const unsigned mlo = __reduce_min_sync(0xFFFFFFFFu, lo);
  const unsigned jj = (hi == mhi && (unsigned)key == mlo) ? (unsigned)j : 0xFFFFFFFFu;
  const unsigned mj = __reduce_min_sync(0xFFFFFFFFu, jj);
  const unsigned long long mkey = ((unsigned long long)mhi << 32) | mlo;
  if (lane == s - s0 && mkey < best) {  // later rounds hold larger indices: ties keep the earlier
    best = mkey;
    best_j = (int)mj;
  }
}

__global__ void __launch_bounds__(kWideWarps * 32, kWideCtasPerSm) k_gravity_ac_wide(ForceCtx fc, const double* __restrict__ y,
                                                                        double* __restrict__ dydt, TimeSpec ts,
                                                                        uint32_t flags, int spc) {
  extern __shared__ __align__(16) double wide_terms[];  // [kWideTile][kWideRow]
  __shared__ double sink_pos[kWideSinks][3];
  __shared__ int sink_ns[kWideSinks];
  __shared__ double acc[3][kWideSinks];
  __shared__ unsigned long long nn_key[kWideWarps][kWideSinks];
  __shared__ int nn_j[kWideWarps][kWideSinks];
  const Classes& c = fc.cls;
  const int n = sol_sink_hi(fc);  // sinks [sink_lo, n)
  const int i0 = fc.sink_lo + blockIdx.x * spc;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x < kWideSinks) {
    const int i = i0 + threadIdx.x;
    const bool live = i < n && i >= 1 && threadIdx.x < spc;
    sink_ns[threadIdx.x] = live ? ((fc.type[i] <= SOL_PROTO_PLANET) ? c.nm + c.n_spl : c.nm) : 0;
    for (int k = 0; k < 3; ++k) sink_pos[threadIdx.x][k] = i < n ? y[6 * i + k] : 0.0;
  }
  __syncthreads();
  int ns_cta = 0;
  for (int s = 0; s < kWideSinks; ++s) ns_cta = max(ns_cta, sink_ns[s]);
  const int rounds = (ns_cta + kWideTile - 1) / kWideTile;
  const double* src = fc.src;
  const int np = fc.npad;

  // lane s of every warp: the first minimum of sink g ceil(spc/4) + s
  // (g = warp / 2, its quarter of the sinks) over this warp's sources
  unsigned long long best = (unsigned long long)__double_as_longlong(1.0e10);
  int best_j = -1;
  // phase-B lanes: component warp, sink lane
  const int b_i = i0 + lane;
  const int b_ns = sink_ns[lane];
  double a_sum = 0.0;

  for (int r = 0; r < rounds; ++r) {
    // ---- phase A ----
    {
      const int p = threadIdx.x % kWideTile;
      const int quarter = (spc + kWideGroups - 1) / kWideGroups;
      const int s0 = (threadIdx.x / kWideTile) * quarter;
      const int s1 = min(s0 + quarter, spc);
      const int j = r * kWideTile + p;
      const bool jin = j < ns_cta;
      double xj = 0, yj = 0, zj = 0, gm = 0, px = 0, py = 0, pz = 0;
      if (jin) {
        xj = src[SX * np + j];
        yj = src[SY * np + j];
        zj = src[SZ * np + j];
        gm = src[SGM * np + j];
        px = src[SPX * np + j];
        py = src[SPY * np + j];
        pz = src[SPZ * np + j];
      }
      double* row = wide_terms + (size_t)p * kWideRow;
      for (int s = s0; s < s1; ++s)
        wide_sink(s, s0, j, jin, i0, lane, xj, yj, zj, gm, px, py, pz, sink_pos, sink_ns, row, best, best_j);
    }
    __syncthreads();
    // ---- phase B ----
    if (warp < 3) {
      const int j0 = r * kWideTile;
      const int pmax = min(kWideTile, b_ns - j0);
      const double* col = wide_terms + warp * kWideSinks + lane;
      for (int p = 0; p < pmax; ++p) {
        const int j = j0 + p;
        if (j >= 1 && j != b_i) a_sum += col[(size_t)p * kWideRow];
      }
    }
    __syncthreads();
  }
  nn_key[warp][lane] = best;
  nn_j[warp][lane] = best_j;
  if (warp < 3) acc[warp][lane] = a_sum;
  __syncthreads();
  if (threadIdx.x >= spc) return;
  const int s = threadIdx.x;
  const int i = i0 + s;
  if (i >= n) return;
  double* out = dydt + 6 * i;
  if (i == 0) {  // GravityAC :253-254, :266
    for (int k = 0; k < 6; ++k) out[k] = 0.0;
    fc.nn_idx[0] = -1;
    fc.nn_dist[0] = 0.0;
    return;
  }
  constexpr int kWarpsPerGroup = kWideTile / 32;
  const int quarter = (spc + kWideGroups - 1) / kWideGroups;
  const int w0 = (s / quarter) * kWarpsPerGroup;
  const int hl = s % quarter;
  unsigned long long bk = nn_key[w0][hl];
  int bj = nn_j[w0][hl];
  for (int w = w0 + 1; w < w0 + kWarpsPerGroup; ++w) {
    const unsigned long long k2 = nn_key[w][hl];
    const int j2 = nn_j[w][hl];
    if (j2 >= 0 && (bj < 0 || k2 < bk || (k2 == bk && j2 < bj))) {
      bk = k2;
      bj = j2;
    }
  }
  const double* yv = y + 6 * i;
  const double xi = sink_pos[s][0], yi = sink_pos[s][1], zi = sink_pos[s][2];
  const double mu = SOL_GAUSS2 * (fc.mass[0] + fc.mass[i]);
  const double rm3i = fc.rm3[i];
  double a[3];
  a[0] = -mu * rm3i * xi;  // Kepler term first (:281-283)
  a[1] = -mu * rm3i * yi;
  a[2] = -mu * rm3i * zi;
  a[0] += acc[0][s];
  a[1] += acc[1][s];
  a[2] += acc[2][s];
  fc.nn_idx[i] = bj;
  fc.nn_dist[i] = bj >= 0 ? __longlong_as_double((long long)bk) : 0.0;
  add_gas_terms(fc, i, yv, eval_time(ts), flags, a);
  out[0] = yv[3];
  out[1] = yv[4];
  out[2] = yv[5];
  out[3] = a[0];
  out[4] = a[1];
  out[5] = a[2];
}

// GravityBC_SelfInteracting / _NonSelfInteracting (Acceleration.cpp:541-634):
// massive sinks and non-massive sinks both sum over massive sources in
// descending order, scale by G at the end; no rm3.
__global__ void __launch_bounds__(kSinkBlock) k_gravity_bc(ForceCtx fc, const double* __restrict__ y,
                                                           double* __restrict__ dydt, TimeSpec ts,
                                                           uint32_t flags) {
  const int n = fc.cls.n;
  const int i = blockIdx.x * kSinkBlock + threadIdx.x;
  if (i >= n) return;
  const double* s = fc.src;
  const int np = fc.npad;
  const double* yv = y + 6 * i;
  double xi = yv[0], yi = yv[1], zi = yv[2];
  double a[3] = {0.0, 0.0, 0.0};
  long long rminb = __double_as_longlong(1.0e10);
  int nn = -1;
  for (int j = fc.cls.nm - 1; j >= 0; j--) {
    if (j == i) continue;
    double dx = s[SX * np + j] - xi;
    double dy = s[SY * np + j] - yi;
    double dz = s[SZ * np + j] - zi;
    double rij2 = dx * dx + dy * dy + dz * dz;
    double rij = __dsqrt_rn(rij2);
    long long rb = __double_as_longlong(rij);
    if (rb < rminb) {
      rminb = rb;
      nn = j;
    }
    double cc = __ddiv_rn(s[SGM * np + j] * 1.0, rij2 * rij);
    a[0] += cc * dx;
    a[1] += cc * dy;
    a[2] += cc * dz;
  }
  a[0] *= SOL_GAUSS2;
  a[1] *= SOL_GAUSS2;
  a[2] *= SOL_GAUSS2;
  fc.nn_idx[i] = nn;
  fc.nn_dist[i] = nn >= 0 ? __longlong_as_double(rminb) : 0.0;
  add_gas_terms(fc, i, yv, eval_time(ts), flags, a);
  double* out = dydt + 6 * i;
  out[0] = yv[3];
  out[1] = yv[4];
  out[2] = yv[5];
  out[3] = a[0];
  out[4] = a[1];
  out[5] = a[2];
}


// 2-D pair kernel of the SPLIT form: blockIdx.x = block of kSinkBlock sinks,
// blockIdx.y = chunk of `chunk` sources.  Each CTA writes, per sink, its
// partial acceleration sum and nearest-neighbour candidate for the chunk;
// k_combine adds the chunks in a fixed order.  Many small work units let the
// block scheduler balance the FP64 pipe load across SMs.  (SPLIT_FF has its
// own 2-D kernel, k_pairs_ff.)
template <int MODE>
__global__ void __launch_bounds__(kSinkBlock) k_pairs(ForceCtx fc, const double* __restrict__ y,
                                                      double* __restrict__ part, int* dev_status, int chunk) {
  static_assert(MODE == SOL_PRECISION_SPLIT, "k_pairs serves the SPLIT form");
  constexpr int NARR = 4;  // x, y, z and G m
  __shared__ __align__(128) TileSmem<NARR> sm;
  const Classes& c = fc.cls;
  const int n = sol_sink_hi(fc);  // sinks [sink_lo, n)
  const int np = fc.npad;
  const int i = fc.sink_lo + blockIdx.x * kSinkBlock + threadIdx.x;
  const int i_first = fc.sink_lo + blockIdx.x * kSinkBlock;
  const int ns_cta = (fc.type[min(i_first, n - 1)] <= SOL_PROTO_PLANET) ? c.nm + c.n_spl : c.nm;
  const int ns = (i < n && fc.type[i] <= SOL_PROTO_PLANET) ? c.nm + c.n_spl : c.nm;
  const int j_begin = blockIdx.y * chunk;
  const int j_end = min(j_begin + chunk, ns_cta);
  const int t_begin = j_begin / kTile;
  const int ntiles = j_end > j_begin ? (j_end - j_begin + kTile - 1) / kTile : 0;
  const int arr[NARR] = {SX, SY, SZ, SGM};

  double xi = 0, yi = 0, zi = 0;
  if (i < n) {
    xi = y[6 * i + 0];
    yi = y[6 * i + 1];
    zi = y[6 * i + 2];
  }
  if (threadIdx.x == 0) {
    sol_mbar_init(&sm.bar[0], 1);
    sol_mbar_init(&sm.bar[1], 1);
    sol_fence_barrier_init();
  }
  __syncthreads();
  auto issue = [&](int t, int stage) {
    sol_mbar_expect_tx(&sm.bar[stage], NARR * kTile * 8);
    for (int k = 0; k < NARR; ++k)
      sol_bulk_g2s(&sm.v[stage][k][0], fc.src + (size_t)arr[k] * np + (size_t)(t_begin + t) * kTile, kTile * 8,
                   &sm.bar[stage]);
  };
  if (threadIdx.x == 0) {
    if (ntiles > 0) issue(0, 0);
    if (ntiles > 1) issue(1, 1);
  }
  double ax = 0.0, ay = 0.0, az = 0.0;  // chunk sums of the per-tile partials
  double cx = 0.0, cy = 0.0, cz = 0.0;  // compensation terms
  long long r2minb = __double_as_longlong(1.0e20);
  int nn = -1;
  int issued = ntiles < 2 ? ntiles : 2;
  int t = 0;
  bool timed_out = false;
  for (; t < ntiles; ++t) {
    const int st = t & 1;
    const bool ok = sol_mbar_wait(&sm.bar[st], (t >> 1) & 1);
    const int j0 = (t_begin + t) * kTile;
    const int jmax = min(kTile, j_end - j0);  // sources beyond the chunk's range are never read
    if (ok && i < n && i >= 1) {
      double tx = 0.0, ty = 0.0, tz = 0.0;
#pragma unroll 4
      for (int jj = 0; jj < jmax; ++jj)
        pair_split(*reinterpret_cast<TileSmem<4>*>(&sm), st, jj, j0 + jj, i, ns, xi, yi, zi, tx, ty, tz, r2minb, nn);
      two_sum(ax, cx, tx);
      two_sum(ay, cy, ty);
      two_sum(az, cz, tz);
    }
    if (__syncthreads_or(!ok)) {
      timed_out = true;
      break;
    }
    if (threadIdx.x == 0 && t + 2 < ntiles) {
      sol_fence_proxy_async();
      issue(t + 2, st);
    }
    if (t + 2 < ntiles) issued = t + 3;
  }
  if (timed_out) {
    if (threadIdx.x == 0) {
      atomicOr(dev_status, SOL_DEV_TIMEOUT);
      for (int u = t; u < issued; ++u) sol_mbar_wait(&sm.bar[u & 1], (u >> 1) & 1);
    }
    __syncthreads();
    return;
  }
  if (i >= n) return;
  const size_t base = (size_t)blockIdx.y * PART_SLOTS * np + i;
  part[base + PAX * np] = ax + cx;
  part[base + PAY * np] = ay + cy;
  part[base + PAZ * np] = az + cz;
  part[base + PR2 * np] = nn >= 0 ? __longlong_as_double(r2minb) : 1.0e300;
  part[base + PIDX * np] = __longlong_as_double((long long)nn);
}

// ---- SPLIT_FF 2-D kernel: float-float pairs with no FP64 instruction -------
// Same grid as k_pairs (blockIdx.x: kSinkBlock sinks; blockIdx.y: a chunk of
// sources, 1 to kChunkTiles tiles as split_chunk chooses so that the grid
// fills the GPU) and the same partial outputs for k_combine.  The sources'
// grid triples and G m (hi, lo) arrive tile by tile in shared memory by bulk
// copies; each thread takes two sources per step in paired FP32
// instructions: the displacement from the grid triples (exact parts, no
// FP64), r^2, G m r^-3 and the accumulation in float-float (sol_pair.cuh).
// Pairs closer than the grid G1 (|d| < G1, where the triple displacement
// would lose relative accuracy) take FP64 arithmetic, as pairs below 1e-12 AU
// do in the other float-float kernels.  Tiles whose sources are all valid
// for every sink of the warp (no sink index, no central body, no source
// beyond a sink's source count or the chunk) run without per-pair tests.
constexpr int kFF = FTAB_USED;

struct FFTile {
  float v[2][kFF][kTile];
  uint64_t bar[2];
};

// One FP64 pair of the close-pair branch: G m r^-3 d into (fx, fy, fz);
// r^2 for the nearest-neighbour comparison as (hi, lo) floats.
__device__ __forceinline__ void ff_close_pair(const ForceCtx& fc, int j, double xi, double yi, double zi, float gh,
                                           float gl, double& fx, double& fy, double& fz, float& r2h, float& r2l) {
  const double* s = fc.src;
  const int np = fc.npad;
  const double dx = s[SX * np + j] - xi, dy = s[SY * np + j] - yi, dz = s[SZ * np + j] - zi;
  const double r2 = __fma_rn(dx, dx, __fma_rn(dy, dy, dz * dz));
  r2h = __double2float_rn(r2);
  r2l = __double2float_rn(r2 - (double)r2h);
  if (r2 > 0.0) {
    const double rinv = __drcp_rn(__dsqrt_rn(r2));
    const double sd = ((double)gh + (double)gl) * (rinv * rinv * rinv);
    fx = __fma_rn(sd, dx, fx);
    fy = __fma_rn(sd, dy, fy);
    fz = __fma_rn(sd, dz, fz);
  }
}

// Nearest-neighbour candidate: the smallest r^2 (hi, then lo), the first in
// ascending source order.
__device__ __forceinline__ void ff_nn(float r2h, float r2l, bool ok, int j, float& mh, float& ml, int& nn) {
  const bool better = ok & ((r2h < mh) | ((r2h == mh) & (r2l < ml)));
  mh = better ? r2h : mh;
  ml = better ? r2l : ml;
  nn = better ? j : nn;
}

// Two sources (j, j + 1) of the tile against the sink, their table rows in
// sv (one float2 per row).  MASKED: per-pair validity (source range, the
// sink itself, the chunk end) is tested.  The accumulators are renormalised
// when renorm is set: after the second pair of every group of four sources,
// as ff_four_sources does, so a sink gets the same bits whether its warp
// takes a tile on the masked path or the fast one.
template <bool MASKED>
__device__ __forceinline__ void ff_two_sources(const float2* sv, int j, int i, int ns, int jend, bool renorm,
                                               const float* ai, const float* bi, const float* ci, float thr,
                                               const ForceCtx& fc, double xi, double yi, double zi, float2* Ah,
                                               float2* Al, double& fx, double& fy, double& fz, float& mh, float& ml,
                                               int& nn) {
  float2 h[3], l[3];
#pragma unroll
  for (int k = 0; k < 3; ++k)
    f2_grid_disp(sv[FAX + 3 * k], sv[FBX + 3 * k], sv[FCX + 3 * k], ai[k], bi[k], ci[k], h[k], l[k]);
  float2 gh = sv[FGH];
  float2 gl = sv[FGL];
  float2 r2h, r2l;
  f2_ff_r2(h, l, r2h, r2l);
  bool ok0 = true, ok1 = true;
  if constexpr (MASKED) {
    ok0 = (j >= 1) & (j < ns) & (j != i) & (j < jend);
    ok1 = (j + 1 >= 1) & (j + 1 < ns) & (j + 1 != i) & (j + 1 < jend);
  }
  float2 qh = r2h, ql = r2l;
  if (!ok0 || r2h.x < thr) {
    if (ok0) ff_close_pair(fc, j, xi, yi, zi, gh.x, gl.x, fx, fy, fz, r2h.x, r2l.x);
    gh.x = gl.x = 0.0f;
    qh.x = 1.0f;
    ql.x = 0.0f;
  }
  if (!ok1 || r2h.y < thr) {
    if (ok1) ff_close_pair(fc, j + 1, xi, yi, zi, gh.y, gl.y, fx, fy, fz, r2h.y, r2l.y);
    gh.y = gl.y = 0.0f;
    qh.y = 1.0f;
    ql.y = 0.0f;
  }
  float2 sh, se;
  f2_ff_gm_rinv3(qh, ql, gh, gl, sh, se);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    f2_ff_accumulate_lazy(Ah[k], Al[k], sh, se, h[k], l[k]);
    if (renorm) f2_fast_two_sum(Ah[k], Al[k], Ah[k], Al[k]);
  }
  ff_nn(r2h.x, r2l.x, ok0, j, mh, ml, nn);
  ff_nn(r2h.y, r2l.y, ok1, j + 1, mh, ml, nn);
}


// Four sources (j .. j + 3) of a fast tile: the displacements and r^2 of both
// pairs of sources first, one test for a close pair among the four, then
// G m r^-3 and the accumulation of both in one basic block, the branch no
// longer splitting the step into short blocks the scheduler cannot
// interleave (16.10 -> 14.96 ms at 65,536 bodies); the accumulators are
// renormalised once per step instead of after each half (14.52 ms); the
// nearest-neighbour update runs only when the four sources' smallest r^2
// reaches the running minimum, which over a sink's sources happens about
// ln(N) times (13.92 ms).  The update itself is exact either way.
__device__ __forceinline__ void ff_close_lane(const ForceCtx& fc, int j, double xi, double yi, double zi, float& gh,
                                              float& gl, double& fx, double& fy, double& fz, float& r2h, float& r2l,
                                              float& qh, float& ql, float thr) {
  if (r2h < thr) {
    ff_close_pair(fc, j, xi, yi, zi, gh, gl, fx, fy, fz, r2h, r2l);
    gh = gl = 0.0f;
    qh = 1.0f;
    ql = 0.0f;
  }
}
__device__ __forceinline__ void ff_four_sources(const float2* va, const float2* vb, int j, const float* ai,
                                                const float* bi, const float* ci, float thr, const ForceCtx& fc,
                                                double xi, double yi, double zi, float2* Ah, float2* Al, double& fx,
                                                double& fy, double& fz, float& mh, float& ml, int& nn) {
  float2 ha[3], la[3], hb[3], lb[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    f2_grid_disp(va[FAX + 3 * k], va[FBX + 3 * k], va[FCX + 3 * k], ai[k], bi[k], ci[k], ha[k], la[k]);
    f2_grid_disp(vb[FAX + 3 * k], vb[FBX + 3 * k], vb[FCX + 3 * k], ai[k], bi[k], ci[k], hb[k], lb[k]);
  }
  float2 gha = va[FGH], gla = va[FGL], ghb = vb[FGH], glb = vb[FGL];
  float2 r2ha, r2la, r2hb, r2lb;
  f2_ff_r2(ha, la, r2ha, r2la);
  f2_ff_r2(hb, lb, r2hb, r2lb);
  float2 qha = r2ha, qla = r2la, qhb = r2hb, qlb = r2lb;
  const float m4 = fminf(fminf(r2ha.x, r2ha.y), fminf(r2hb.x, r2hb.y));
  if (m4 < thr) {
    ff_close_lane(fc, j, xi, yi, zi, gha.x, gla.x, fx, fy, fz, r2ha.x, r2la.x, qha.x, qla.x, thr);
    ff_close_lane(fc, j + 1, xi, yi, zi, gha.y, gla.y, fx, fy, fz, r2ha.y, r2la.y, qha.y, qla.y, thr);
    ff_close_lane(fc, j + 2, xi, yi, zi, ghb.x, glb.x, fx, fy, fz, r2hb.x, r2lb.x, qhb.x, qlb.x, thr);
    ff_close_lane(fc, j + 3, xi, yi, zi, ghb.y, glb.y, fx, fy, fz, r2hb.y, r2lb.y, qhb.y, qlb.y, thr);
  }
  float2 sha, sea, shb, seb;
  f2_ff_gm_rinv3(qha, qla, gha, gla, sha, sea);
  f2_ff_gm_rinv3(qhb, qlb, ghb, glb, shb, seb);
#pragma unroll
  for (int k = 0; k < 3; ++k) {  // both halves, one renormalisation
    f2_ff_accumulate_lazy(Ah[k], Al[k], sha, sea, ha[k], la[k]);
    f2_ff_accumulate_lazy(Ah[k], Al[k], shb, seb, hb[k], lb[k]);
    f2_fast_two_sum(Ah[k], Al[k], Ah[k], Al[k]);
  }
  // a new nearest neighbour is rare: only when the four sources' smallest
  // r^2 reaches the running minimum (or a close pair replaced an r^2)
  if (m4 <= mh || m4 < thr) {
    ff_nn(r2ha.x, r2la.x, true, j, mh, ml, nn);
    ff_nn(r2ha.y, r2la.y, true, j + 1, mh, ml, nn);
    ff_nn(r2hb.x, r2lb.x, true, j + 2, mh, ml, nn);
    ff_nn(r2hb.y, r2lb.y, true, j + 3, mh, ml, nn);
  }
}

// Three CTAs per SM (up to 170 registers): the four-source step keeps both
// halves' temporaries live at once.
__global__ void __launch_bounds__(kSinkBlock, 3) k_pairs_ff(ForceCtx fc, const double* __restrict__ y,
                                                         double* __restrict__ part, int* dev_status, int chunk) {
  __shared__ __align__(128) FFTile sm;
  const Classes& c = fc.cls;
  const int n = sol_sink_hi(fc);  // sinks [sink_lo, n)
  const int np = fc.npad;
  const int i = fc.sink_lo + blockIdx.x * kSinkBlock + threadIdx.x;
  const int i_first = fc.sink_lo + blockIdx.x * kSinkBlock;
  const int ns_cta = (fc.type[min(i_first, n - 1)] <= SOL_PROTO_PLANET) ? c.nm + c.n_spl : c.nm;
  const int ns = (i < n && fc.type[i] <= SOL_PROTO_PLANET) ? c.nm + c.n_spl : c.nm;
  const int j_begin = blockIdx.y * chunk;
  const int j_end = min(j_begin + chunk, ns_cta);
  const int t_begin = j_begin / kTile;
  const int ntiles = j_end > j_begin ? (j_end - j_begin + kTile - 1) / kTile : 0;
  const bool live = i < n && i >= 1;

  const float* T = ftab(fc);
  float ai[3], bi[3], ci[3];
  double xi = 0, yi = 0, zi = 0;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    ai[k] = i < n ? T[(size_t)(FAX + 3 * k) * np + i] : 0.0f;
    bi[k] = i < n ? T[(size_t)(FBX + 3 * k) * np + i] : 0.0f;
    ci[k] = i < n ? T[(size_t)(FCX + 3 * k) * np + i] : 0.0f;
  }
  if (i < n) {
    xi = y[6 * i + 0];
    yi = y[6 * i + 1];
    zi = y[6 * i + 2];
  }
  const double G1 = fc.ind_sum[kIndGrid];
  // |d| < max(G1, 2^-50): the FP64 branch (the floor keeps every r^2 the
  // float-float path sees a normal float)
  const float thr = fmaxf((float)(G1 * G1), 7.888609052210118e-31f);

  if (threadIdx.x == 0) {
    sol_mbar_init(&sm.bar[0], 1);
    sol_mbar_init(&sm.bar[1], 1);
    sol_fence_barrier_init();
  }
  __syncthreads();
  auto issue = [&](int t, int stage) {
    sol_mbar_expect_tx(&sm.bar[stage], kFF * kTile * 4);
    for (int k = 0; k < kFF; ++k)
      sol_bulk_g2s(&sm.v[stage][k][0], T + (size_t)k * np + (size_t)(t_begin + t) * kTile, kTile * 4,
                   &sm.bar[stage]);
  };
  if (threadIdx.x == 0) {
    if (ntiles > 0) issue(0, 0);
    if (ntiles > 1) issue(1, 1);
  }
  double ax = 0.0, ay = 0.0, az = 0.0, cx = 0.0, cy = 0.0, cz = 0.0;  // chunk sums, compensated
  double fx = 0.0, fy = 0.0, fz = 0.0;                                  // close pairs, FP64
  float mh = 3.0e38f, ml = 0.0f;
  int nn = -1;
  int issued = ntiles < 2 ? ntiles : 2;
  int t = 0;
  bool timed_out = false;
  for (; t < ntiles; ++t) {
    const int st = t & 1;
    const bool ok = sol_mbar_wait(&sm.bar[st], (t >> 1) & 1);
    const int j0 = (t_begin + t) * kTile;
    const int jend = min(j0 + kTile, j_end);
    // the warp's sinks all see every source of the tile, none of them is in it
    const bool clean = live && j0 >= 1 && jend == j0 + kTile && j0 + kTile <= ns && (i < j0 || i >= j0 + kTile);
    const bool fast = __all_sync(0xFFFFFFFFu, clean);
    if (ok && live) {
      float2 Ah[3], Al[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) Ah[k] = Al[k] = make_float2(0.0f, 0.0f);
      if (fast) {
        // four sources per step: one 16-byte shared load per table row
#pragma unroll 1
        for (int jj = 0; jj < kTile; jj += 4) {
          float2 va[kFF], vb[kFF];
#pragma unroll
          for (int k = 0; k < kFF; ++k) {
            const float4 q = *reinterpret_cast<const float4*>(&sm.v[st][k][jj]);
            va[k] = make_float2(q.x, q.y);
            vb[k] = make_float2(q.z, q.w);
          }
          ff_four_sources(va, vb, j0 + jj, ai, bi, ci, thr, fc, xi, yi, zi, Ah, Al, fx, fy, fz, mh, ml, nn);
        }
      } else {
        for (int jj = 0; jj < jend - j0; jj += 2) {
          float2 va[kFF];
#pragma unroll
          for (int k = 0; k < kFF; ++k) va[k] = *reinterpret_cast<const float2*>(&sm.v[st][k][jj]);
          ff_two_sources<true>(va, j0 + jj, i, ns, jend, (jj & 2) != 0, ai, bi, ci, thr, fc, xi, yi, zi, Ah, Al, fx,
                               fy, fz, mh, ml, nn);
        }
      }
      // the tile's float-float partials (even and odd sources) into the FP64 chunk sums
      two_sum(ax, cx, ((double)Ah[0].x + (double)Al[0].x) + ((double)Ah[0].y + (double)Al[0].y));
      two_sum(ay, cy, ((double)Ah[1].x + (double)Al[1].x) + ((double)Ah[1].y + (double)Al[1].y));
      two_sum(az, cz, ((double)Ah[2].x + (double)Al[2].x) + ((double)Ah[2].y + (double)Al[2].y));
    }
    if (__syncthreads_or(!ok)) {
      timed_out = true;
      break;
    }
    if (threadIdx.x == 0 && t + 2 < ntiles) {
      sol_fence_proxy_async();
      issue(t + 2, st);
    }
    if (t + 2 < ntiles) issued = t + 3;
  }
  if (timed_out) {
    if (threadIdx.x == 0) {
      atomicOr(dev_status, SOL_DEV_TIMEOUT);
      for (int u = t; u < issued; ++u) sol_mbar_wait(&sm.bar[u & 1], (u >> 1) & 1);
    }
    __syncthreads();
    return;
  }
  if (i >= n) return;
  const size_t base = (size_t)blockIdx.y * PART_SLOTS * np + i;
  part[base + PAX * np] = (ax + cx) + fx;
  part[base + PAY * np] = (ay + cy) + fy;
  part[base + PAZ * np] = (az + cz) + fz;
  part[base + PR2 * np] = nn >= 0 ? (double)mh + (double)ml : 1.0e300;
  part[base + PIDX * np] = __longlong_as_double((long long)nn);
}

// Per sink: the chunk partials in chunk order, the nearest neighbour (the
// smallest r^2, ties to the lower index as the reference's ascending scan),
// distanceOfNN recomputed in the reference's FP64 arithmetic for the chosen
// neighbour, the Kepler and indirect terms, and the gas terms.
__global__ void k_combine(ForceCtx fc, const double* __restrict__ y, double* __restrict__ dydt,
                          const double* __restrict__ part, int nchunk, TimeSpec ts, uint32_t flags) {
  const Classes& c = fc.cls;
  const int n = sol_sink_hi(fc);  // sinks [sink_lo, n)
  const int np = fc.npad;
  const int i = fc.sink_lo + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double* out = dydt + 6 * i;
  if (i == 0) {
    for (int k = 0; k < 6; ++k) out[k] = 0.0;
    fc.nn_idx[0] = -1;
    fc.nn_dist[0] = 0.0;
    return;
  }
  const double* yv = y + 6 * i;
  double sx = 0.0, sy = 0.0, sz = 0.0, ex = 0.0, ey = 0.0, ez = 0.0;
  double best = 1.0e300;
  int nn = -1;
  for (int ch = 0; ch < nchunk; ++ch) {
    const size_t base = (size_t)ch * PART_SLOTS * np + i;
    two_sum(sx, ex, part[base + PAX * np]);
    two_sum(sy, ey, part[base + PAY * np]);
    two_sum(sz, ez, part[base + PAZ * np]);
    const double r2 = part[base + PR2 * np];
    const int j = (int)__double_as_longlong(part[base + PIDX * np]);
    if (j >= 0 && r2 < best) {
      best = r2;
      nn = j;
    }
  }
  const int ns = (fc.type[i] <= SOL_PROTO_PLANET) ? c.nm + c.n_spl : c.nm;
  const double mu = SOL_GAUSS2 * (fc.mass[0] + fc.mass[i]);
  const double rm3i = fc.rm3[i];
  const double xi = yv[0], yi = yv[1], zi = yv[2];
  double a[3];
  a[0] = -mu * rm3i * xi;
  a[1] = -mu * rm3i * yi;
  a[2] = -mu * rm3i * zi;
  const double* S = fc.ind_sum + ((fc.type[i] <= SOL_PROTO_PLANET) ? 3 : 0);
  const double* s = fc.src;
  double own[3] = {0.0, 0.0, 0.0};
  if (i < ns) {
    const double gmi = s[SGM * np + i];
    own[0] = gmi * s[SPX * np + i];
    own[1] = gmi * s[SPY * np + i];
    own[2] = gmi * s[SPZ * np + i];
  }
  a[0] += (sx + ex) - (S[0] - own[0]);
  a[1] += (sy + ey) - (S[1] - own[1]);
  a[2] += (sz + ez) - (S[2] - own[2]);
  if (nn >= 0) {
    // the reference's rij for this j (Acceleration.cpp:301-305), bit for bit
    const double xij = y[6 * nn + 0] - xi, yij = y[6 * nn + 1] - yi, zij = y[6 * nn + 2] - zi;
    const double rij = __dsqrt_rn(xij * xij + yij * yij + zij * zij);
    if (rij < 1.0e10) {
      fc.nn_idx[i] = nn;
      fc.nn_dist[i] = rij;
    } else {
      fc.nn_idx[i] = -1;
      fc.nn_dist[i] = 0.0;
    }
  } else {
    fc.nn_idx[i] = -1;
    fc.nn_dist[i] = 0.0;
  }
  add_gas_terms(fc, i, yv, eval_time(ts), flags, a);
  out[0] = yv[3];
  out[1] = yv[4];
  out[2] = yv[5];
  out[3] = a[0];
  out[4] = a[1];
  out[5] = a[2];
}

// ---- split forms for systems of up to kFewSplitMax bodies --------------------
// The 2-D split kernel has ceil(N / 128) x ceil(N / 4096) work units, too few
// to fill the GPU below ~16,000 bodies.  Here one warp takes one sink and its
// lanes split the sources (lane l takes l, l + 32, ...): each lane
// accumulates its share in the split arithmetic (SPLIT: FP64 FMA; SPLIT_FF:
// float-float folded into compensated FP64 every kFoldRounds of its
// sources), then the warp adds the 32 partials in a fixed shuffle tree with
// compensation (deterministic) and lane 0 finishes as k_combine does.  Every
// FP64 instruction runs on full warps: on the GB300 the FP64 pipe is scarce
// and is charged per warp instruction.
constexpr int kFewSplitWarps = 8;
constexpr int kFewSplitMax = 16384;  // SPLIT: the warp-per-sink kernel up to here
constexpr int kFfMinBodies = 4096;   // SPLIT_FF: k_pairs_ff from here (below, the warp-per-sink kernel)
constexpr int kFoldRounds = 64;

__device__ __forceinline__ void warp_two_sum(double& s, double& c) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const double so = __shfl_down_sync(0xffffffffu, s, off);
    const double co = __shfl_down_sync(0xffffffffu, c, off);
    two_sum(s, c, so);
    c += co;
  }
}

template <int MODE>
__global__ void __launch_bounds__(kFewSplitWarps * 32) k_pairs_few(ForceCtx fc, const double* __restrict__ y,
                                                                   double* __restrict__ dydt, TimeSpec ts,
                                                                   uint32_t flags) {
  const Classes& c = fc.cls;
  const int n = sol_sink_hi(fc);  // sinks [sink_lo, n)
  const int np = fc.npad;
  const int lane = threadIdx.x & 31;
  const int i = fc.sink_lo + blockIdx.x * kFewSplitWarps + (threadIdx.x >> 5);
  if (i >= n) return;  // whole warps leave together
  const int ns = (i >= 1) ? ((fc.type[i] <= SOL_PROTO_PLANET) ? c.nm + c.n_spl : c.nm) : 0;
  const double xi = y[6 * i + 0], yi = y[6 * i + 1], zi = y[6 * i + 2];
  const double* sx = fc.src + (size_t)SX * np;
  const double* sy = fc.src + (size_t)SY * np;
  const double* sz = fc.src + (size_t)SZ * np;
  double ax = 0.0, ay = 0.0, az = 0.0, cx = 0.0, cy = 0.0, cz = 0.0;
  double r2best = 1.0e300;  // this lane's first minimum of r^2 (ascending j)
  int nn = -1;
  if constexpr (MODE == SOL_PRECISION_SPLIT) {
    const double* sg = fc.src + (size_t)SGM * np;
    long long r2b = __double_as_longlong(1.0e20);
#pragma unroll 4
    for (int j = lane; j < ns; j += 32) {
      const double dx = sx[j] - xi, dy = sy[j] - yi, dz = sz[j] - zi;
      const double r2 = __fma_rn(dx, dx, __fma_rn(dy, dy, dz * dz));
      const double gm = (j >= 1 && j != i) ? sg[j] : 0.0;  // the sink itself and the central body: 0
      const double sc = split_gm_rinv3(r2, gm);
      ax = __fma_rn(sc, dx, ax);
      ay = __fma_rn(sc, dy, ay);
      az = __fma_rn(sc, dz, az);
      const long long rb = __double_as_longlong(r2);
      const bool better = (rb < r2b) & (j >= 1) & (j != i);
      r2b = better ? rb : r2b;
      nn = better ? j : nn;
    }
    if (nn >= 0) r2best = __longlong_as_double(r2b);
  } else {
    const float2* sg = reinterpret_cast<const float2*>(fc.src + (size_t)SGF * np);
    FFAcc A;
#pragma unroll
    for (int k = 0; k < 3; ++k) A.h[k] = A.l[k] = 0.0f;
    double fx = 0.0, fy = 0.0, fz = 0.0;  // the FP64 branch of very close pairs
    float mh = 1.0e20f, ml = 0.0f;
    int round = 0;
#pragma unroll 2
    for (int j = lane; j < ns; j += 32) {
      const float2 g = (j >= 1) ? sg[j] : make_float2(0.0f, 0.0f);  // the sink itself contributes 0 * d = 0
      float r2h, r2l;
      ff_pair_accumulate(sx[j] - xi, sy[j] - yi, sz[j] - zi, g, A, fx, fy, fz, r2h, r2l);
      const bool better = ((r2h < mh) | ((r2h == mh) & (r2l < ml))) & (j >= 1) & (j != i);
      mh = better ? r2h : mh;
      ml = better ? r2l : ml;
      nn = better ? j : nn;
      if (++round == kFoldRounds) {
        round = 0;
        two_sum(ax, cx, (double)A.h[0] + (double)A.l[0]);
        two_sum(ay, cy, (double)A.h[1] + (double)A.l[1]);
        two_sum(az, cz, (double)A.h[2] + (double)A.l[2]);
#pragma unroll
        for (int k = 0; k < 3; ++k) A.h[k] = A.l[k] = 0.0f;
      }
    }
    // the float-float remainder and the FP64 close pairs
    two_sum(ax, cx, ((double)A.h[0] + (double)A.l[0]) + fx);
    two_sum(ay, cy, ((double)A.h[1] + (double)A.l[1]) + fy);
    two_sum(az, cz, ((double)A.h[2] + (double)A.l[2]) + fz);
    if (nn >= 0) r2best = (double)mh + (double)ml;
  }
  warp_two_sum(ax, cx);
  warp_two_sum(ay, cy);
  warp_two_sum(az, cz);
  // nearest neighbour: the smallest r^2, ties to the lower index
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const double ro = __shfl_down_sync(0xffffffffu, r2best, off);
    const int jo = __shfl_down_sync(0xffffffffu, nn, off);
    if (jo >= 0 && (nn < 0 || ro < r2best || (ro == r2best && jo < nn))) {
      r2best = ro;
      nn = jo;
    }
  }
  if (lane != 0) return;
  double* out = dydt + 6 * i;
  if (i == 0) {
    for (int k = 0; k < 6; ++k) out[k] = 0.0;
    fc.nn_idx[0] = -1;
    fc.nn_dist[0] = 0.0;
    return;
  }
  const double* yv = y + 6 * i;
  const double mu = SOL_GAUSS2 * (fc.mass[0] + fc.mass[i]);
  const double rm3i = fc.rm3[i];
  double a[3];
  a[0] = -mu * rm3i * xi;
  a[1] = -mu * rm3i * yi;
  a[2] = -mu * rm3i * zi;
  const double* S = fc.ind_sum + ((fc.type[i] <= SOL_PROTO_PLANET) ? 3 : 0);
  const double* src = fc.src;
  double own[3] = {0.0, 0.0, 0.0};
  if (i < ns) {
    const double gmi = src[SGM * np + i];
    own[0] = gmi * src[SPX * np + i];
    own[1] = gmi * src[SPY * np + i];
    own[2] = gmi * src[SPZ * np + i];
  }
  a[0] += (ax + cx) - (S[0] - own[0]);
  a[1] += (ay + cy) - (S[1] - own[1]);
  a[2] += (az + cz) - (S[2] - own[2]);
  double rij = 0.0;
  if (nn >= 0) {
    // the reference's rij for this j (Acceleration.cpp:301-305), bit for bit
    const double xij = y[6 * nn + 0] - xi, yij = y[6 * nn + 1] - yi, zij = y[6 * nn + 2] - zi;
    rij = __dsqrt_rn(xij * xij + yij * yij + zij * zij);
    if (!(rij < 1.0e10)) nn = -1;
  }
  fc.nn_idx[i] = nn;
  fc.nn_dist[i] = nn >= 0 ? rij : 0.0;
  add_gas_terms(fc, i, yv, eval_time(ts), flags, a);
  out[0] = yv[3];
  out[1] = yv[4];
  out[2] = yv[5];
  out[3] = a[0];
  out[4] = a[1];
  out[5] = a[2];
}

}  // namespace

// parts: 1 = prepass (and indirect totals), 2 = pair kernel, 3 = both.
// Sources per CTA of the 2-D split kernels: SPLIT takes kChunk; SPLIT_FF a
// chunk of 1..kChunkTiles tiles: among the grids that give every SM at least
// the CTAs k_pairs_ff holds at once, the one whose busiest SM has the least
// work (its CTAs times the tiles of a CTA plus half a tile of per-CTA work),
// ties to the larger chunk; the finest chunk when no grid is that large.
// Small systems fill the GPU, and sizes just past a whole number of CTAs
// per SM avoid a nearly empty last round.
static int split_chunk(const sol_ctx* c, int precision) {
  if (precision != SOL_PRECISION_SPLIT_FF) return kChunk;
  // per device, filled on first use; contexts of several host threads may
  // race to fill them with the same values, hence the atomics
  static std::atomic<int> sms[kMaxDevices], resident[kMaxDevices];
  const int dev = (c->device >= 0 && c->device < kMaxDevices) ? c->device : 0;
  if (sms[dev].load(std::memory_order_relaxed) == 0) {
    int nsm = 0, per_sm = 0;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->device) != cudaSuccess || nsm < 1) nsm = 152;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pairs_ff, kSinkBlock, 0) != cudaSuccess ||
        per_sm < 1)
      per_sm = 3;
    resident[dev].store(per_sm, std::memory_order_relaxed);
    sms[dev].store(nsm, std::memory_order_release);
  }
  const long nb = (c->n + kSinkBlock - 1) / kSinkBlock;
  const long nsm = sms[dev].load(std::memory_order_acquire);
  const long res = resident[dev].load(std::memory_order_relaxed);
  int best_ct = 1;
  double best = 1e300;
  for (int ct = kChunkTiles; ct >= 1; ct >>= 1) {
    const long ctas = nb * ((c->n + ct * kTile - 1) / (ct * kTile));
    if (ctas < res * nsm) continue;
    const double cost = (double)((ctas + nsm - 1) / nsm) * (ct + 0.5);
    if (cost < best) {
      best = cost;
      best_ct = ct;
    }
  }
  return best_ct * kTile;
}

// The sinks of fc's range [sink_lo, sol_sink_hi) (every body by default);
// the prepass always covers every body (the sources).
static int force_launch(sol_ctx* c, const ForceCtx& fc, const double* d_y, double* d_dydt, TimeSpec ts,
                        uint32_t flags, int parts) {
  const int nsink = sol_sink_hi(fc) - fc.sink_lo;
  const int split = (c->precision != SOL_PRECISION_FP64 && !c->barycentric) ? 1 : 0;
  // SPLIT_FF systems beyond the warp-per-sink kernel run k_pairs_ff on the float table
  const int ff2d = split && c->precision == SOL_PRECISION_SPLIT_FF && sol_force_uses_chunk_partials(c, c->precision);
  if (parts & 1) {
    const int nb_pre = (fc.npad + kPrepassBlock - 1) / kPrepassBlock;
    k_prepass<<<nb_pre, kPrepassBlock, 0, c->stream>>>(fc, d_y, split, ff2d);
    SOL_LAUNCHED();
    if (split && !c->barycentric) {
      k_ind_reduce<<<1, 256, 0, c->stream>>>(fc);
      SOL_LAUNCHED();
    }
    if (ff2d) {
      k_split_table<<<nb_pre, kPrepassBlock, 0, c->stream>>>(fc, d_y);
      SOL_LAUNCHED();
    }
  }
  if (!(parts & 2) || nsink <= 0) return SOL_OK;
  const int nb = (nsink + kSinkBlock - 1) / kSinkBlock;
  if (c->barycentric) {
    k_gravity_bc<<<nb, kSinkBlock, 0, c->stream>>>(fc, d_y, d_dydt, ts, flags);
    SOL_LAUNCHED();
    return SOL_OK;
  }
  // sinks with fewer sources than one producer tile (a few massive bodies and
  // many light ones) are cheaper with one thread per sink
  if (!split && c->cls.nm + c->cls.n_spl >= kFewTile) {
    // per device: the SM count, once the wide kernel's shared-memory size is
    // allowed (contexts of several host threads may race to set it: the same
    // values, hence an atomic published after the attribute call)
    static std::atomic<int> wide_sms[kMaxDevices];
    const int dev = (c->device >= 0 && c->device < kMaxDevices) ? c->device : 0;
    int wsm = wide_sms[dev].load(std::memory_order_acquire);
    if (wsm == 0) {
      int nsm = 0;
      SOL_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->device));
      SOL_CUDA(cudaFuncSetAttribute(k_gravity_ac_wide, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kWideSmem));
      wide_sms[dev].store(nsm, std::memory_order_release);
      wsm = nsm;
    }
    // sinks per CTA: the fewest whole waves of two CTAs per SM, then the
    // cheapest of that and the next two wave counts
    const int slots = kWideCtasPerSm * wsm;
    int spc = 0;
    {
      const int k0 = (nsink + slots * kWideSinks - 1) / (slots * kWideSinks);
      double best = 1e300;
      for (int k = k0; k < k0 + 3; ++k) {
        const int sp = (nsink + k * slots - 1) / (k * slots);
        const double cost = k * (0.4375 * sp + 3.0);
        if (cost < best) {
          best = cost;
          spc = sp;
        }
      }
    }
    if (spc >= kWideMinSinks) {
      k_gravity_ac_wide<<<(nsink + spc - 1) / spc, kWideWarps * 32, kWideSmem, c->stream>>>(fc, d_y, d_dydt, ts,
                                                                                            flags, spc);
    } else {
      k_gravity_ac_few<<<(nsink + kFewSinks - 1) / kFewSinks, 256, 0, c->stream>>>(fc, d_y, d_dydt, ts, flags);
    }
    SOL_LAUNCHED();
    return SOL_OK;
  }
  if (split && !sol_force_uses_chunk_partials(c, c->precision)) {
    const int grid = (nsink + kFewSplitWarps - 1) / kFewSplitWarps;
    if (c->precision == SOL_PRECISION_SPLIT_FF)
      k_pairs_few<SOL_PRECISION_SPLIT_FF><<<grid, kFewSplitWarps * 32, 0, c->stream>>>(fc, d_y, d_dydt, ts, flags);
    else
      k_pairs_few<SOL_PRECISION_SPLIT><<<grid, kFewSplitWarps * 32, 0, c->stream>>>(fc, d_y, d_dydt, ts, flags);
    SOL_LAUNCHED();
    return SOL_OK;
  }
  if (split) {
    if (!c->d_part) {
      sol_set_error("split precision selected without sol_set_precision");
      return SOL_ERR_STATE;
    }
    const int chunk = split_chunk(c, c->precision);
    const int nchunk = (c->n + chunk - 1) / chunk;
    dim3 grid(nb, nchunk);
    if (c->precision == SOL_PRECISION_SPLIT_FF)
      k_pairs_ff<<<grid, kSinkBlock, 0, c->stream>>>(fc, d_y, c->d_part, &c->d_ctrl->dev_status, chunk);
    else
      k_pairs<SOL_PRECISION_SPLIT><<<grid, kSinkBlock, 0, c->stream>>>(fc, d_y, c->d_part, &c->d_ctrl->dev_status,
                                                                      chunk);
    SOL_LAUNCHED();
    k_combine<<<(nsink + 255) / 256, 256, 0, c->stream>>>(fc, d_y, d_dydt, c->d_part, nchunk, ts, flags);
  } else {
    k_gravity_ac<SOL_PRECISION_FP64><<<nb, kSinkBlock, 0, c->stream>>>(fc, d_y, d_dydt, ts, flags,
                                                                       &c->d_ctrl->dev_status, SOL_SPIN_LIMIT, -1);
  }
  SOL_LAUNCHED();
  return SOL_OK;
}

int sol_force_launch_parts(sol_ctx* c, const double* d_y, double* d_dydt, TimeSpec ts, uint32_t flags, int parts) {
  return force_launch(c, c->fc, d_y, d_dydt, ts, flags, parts);
}

int sol_force_launch(sol_ctx* c, const double* d_y, double* d_dydt, TimeSpec ts, uint32_t flags) {
  return sol_force_launch_parts(c, d_y, d_dydt, ts, flags, 3);
}

// Sinks [lo, hi) only (heliocentric contexts): a rank's block of a
// sink-partitioned system.
int sol_force_launch_sinks(sol_ctx* c, const double* d_y, double* d_dydt, TimeSpec ts, uint32_t flags, int lo,
                           int hi) {
  ForceCtx fc = c->fc;
  fc.sink_lo = lo;
  fc.sink_hi = hi;
  return force_launch(c, fc, d_y, d_dydt, ts, flags, 3);
}

int sol_force_tile() { return kTile; }
int sol_force_src_doubles() { return kSrcDoubles; }
// chunk partials for either split form's 2-D kernel
int sol_force_part_doubles(const sol_ctx* c) {
  const int a = (c->n + kChunk - 1) / kChunk;
  const int ff = split_chunk(c, SOL_PRECISION_SPLIT_FF);
  const int b = (c->n + ff - 1) / ff;
  return (a > b ? a : b) * PART_SLOTS * c->npad;
}
// whether the split forms of this system run the 2-D kernel (and need its
// chunk partials); the same test as the dispatch in sol_force_launch_parts
int sol_force_uses_chunk_partials(const sol_ctx* c, int precision) {
  const int few_max = precision == SOL_PRECISION_SPLIT_FF ? kFfMinBodies - 1 : kFewSplitMax;
  return !(c->n <= few_max && c->cls.nm + c->cls.n_spl >= kTile);
}
int sol_force_prepass_blocks(int npad) { return (npad + kPrepassBlock - 1) / kPrepassBlock; }

// ---- caller-allocated variant ---------------------------------------------------
// sol_gravity_noalloc serves callers that must not allocate device memory
// themselves: code running under someone else's memory manager (a host
// framework that owns every device byte, a fixed-budget plugin) or in a
// real-time loop where an allocation would stall.  Its scratch -- the
// structure-of-arrays source table, the per-block indirect-term partials and
// a status word -- is this file-scope array, sized for at most
// kNoAllocMaxBodies bodies (about 1 MiB), present on every device that loads
// the library until the process exits.
namespace {
constexpr int kNoAllocMaxBodies = 16384;
constexpr int kNoAllocPrepassBlocks = kNoAllocMaxBodies / kPrepassBlock;
constexpr size_t kNoAllocSrc = (size_t)SRC_ARRAYS * kNoAllocMaxBodies;
constexpr size_t kNoAllocPart = 6 * (size_t)kNoAllocPrepassBlocks;
constexpr size_t kNoAllocDoubles = kNoAllocSrc + kNoAllocPart + 8 /* sums */ + 8 /* status */;
static_assert(kNoAllocMaxBodies % kTile == 0, "scratch must hold whole tiles");
}  // namespace

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocDoubles];

namespace {
std::mutex g_noalloc_mu;
double* g_noalloc_addr[64];  // device address of g_noalloc_scratch, per device ordinal
// failure-path test hook (sol_set_wait_test with no context): the mbarrier
// spin limit of the next calls (0: SOL_SPIN_LIMIT) and a tile never copied
std::atomic<unsigned> g_noalloc_spin{0};
std::atomic<int> g_noalloc_withhold{-1};

// Host code cannot use g_noalloc_scratch as a device address: resolve it once
// per device, with that device current.  The same first call loads every
// kernel instance this entry point launches (with CUDA's lazy module loading
// a kernel's first launch would otherwise load it then), so later calls --
// of either precision -- do no loading work.
int noalloc_scratch(double** out) {
  int dev = 0;
  SOL_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) {
    sol_set_error("device ordinal %d out of range", dev);
    return SOL_ERR_ARG;
  }
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return sol_cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)", __FILE__, __LINE__);
    cudaFuncAttributes fa;
    SOL_CUDA(cudaFuncGetAttributes(&fa, k_prepass));
    SOL_CUDA(cudaFuncGetAttributes(&fa, k_ind_reduce));
    SOL_CUDA(cudaFuncGetAttributes(&fa, k_gravity_ac<SOL_PRECISION_FP64>));
    SOL_CUDA(cudaFuncGetAttributes(&fa, k_gravity_ac<SOL_PRECISION_SPLIT>));
    g_noalloc_addr[dev] = (double*)p;
  }
  *out = g_noalloc_addr[dev];
  return SOL_OK;
}

int* noalloc_status_word(double* scratch) { return (int*)(scratch + kNoAllocSrc + kNoAllocPart + 8); }
}  // namespace

void sol_noalloc_wait_test(unsigned spin_limit, int withhold_tile) {
  g_noalloc_spin.store(spin_limit);
  g_noalloc_withhold.store(withhold_tile);
}

extern "C" int sol_gravity_noalloc_status(void* stream, int32_t* status) {
  double* scratch = nullptr;
  int rc = noalloc_scratch(&scratch);
  if (rc != SOL_OK) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  int word = 0;
  SOL_CUDA(cudaMemcpyAsync(&word, noalloc_status_word(scratch), sizeof(int), cudaMemcpyDeviceToHost, st));
  SOL_CUDA(cudaStreamSynchronize(st));
  if (status) *status = word;
  if (word & SOL_DEV_TIMEOUT) {
    sol_set_error("sol_gravity_noalloc: a bounded device wait ran out; the outputs of that call are incomplete");
    return SOL_ERR_TIMEOUT;
  }
  return SOL_OK;
}

extern "C" int sol_gravity_noalloc(const sol_nbodies* counts, const int32_t* d_type, const double* d_mass,
                                   const double* d_y, double* d_dydt, double* d_rm3, int32_t* d_nn_idx,
                                   double* d_nn_dist, int32_t precision, void* stream) {
  if (!counts || !d_type || !d_mass || !d_y || !d_dydt || !d_rm3 || !d_nn_idx || !d_nn_dist) {
    sol_set_error("sol_gravity_noalloc: null argument");
    return SOL_ERR_ARG;
  }
  const sol_nbodies& k = *counts;
  const int parts[7] = {k.central_body, k.giant_planet, k.rocky_planet, k.proto_planet, k.super_planetesimal,
                        k.planetesimal, k.test_particle};
  long long n = 0;
  for (int q = 0; q < 7; ++q) {
    if (parts[q] < 0) {
      sol_set_error("sol_gravity_noalloc: negative body count");
      return SOL_ERR_ARG;
    }
    n += parts[q];
  }
  if (k.central_body != 1) {
    sol_set_error("sol_gravity_noalloc: need exactly one central body");
    return SOL_ERR_ARG;
  }
  if (n > kNoAllocMaxBodies) {
    sol_set_error("sol_gravity_noalloc: %lld bodies exceed the fixed scratch capacity of %d bodies", n,
                  kNoAllocMaxBodies);
    return SOL_ERR_ARG;
  }
  if (precision != SOL_PRECISION_FP64 && precision != SOL_PRECISION_SPLIT) {
    sol_set_error("sol_gravity_noalloc: unknown precision %d", precision);
    return SOL_ERR_ARG;
  }
  double* scratch = nullptr;
  int rc = noalloc_scratch(&scratch);
  if (rc != SOL_OK) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  ForceCtx fc;
  memset(&fc, 0, sizeof(fc));
  fc.cls.n = (int)n;
  fc.cls.n_central = k.central_body;
  fc.cls.n_giant = k.giant_planet;
  fc.cls.n_rocky = k.rocky_planet;
  fc.cls.n_proto = k.proto_planet;
  fc.cls.n_spl = k.super_planetesimal;
  fc.cls.n_pl = k.planetesimal;
  fc.cls.nm = k.central_body + k.giant_planet + k.rocky_planet + k.proto_planet;
  fc.npad = (int)(((n + kTile - 1) / kTile) * kTile);
  fc.precision = precision;
  fc.type = d_type;
  fc.mass = d_mass;
  fc.rm3 = d_rm3;
  fc.nn_idx = d_nn_idx;
  fc.nn_dist = d_nn_dist;
  fc.src = scratch;  // SRC_ARRAYS x npad doubles at stride npad
  fc.ind_part = scratch + kNoAllocSrc;
  fc.ind_sum = scratch + kNoAllocSrc + kNoAllocPart;
  fc.n_ind_blocks = (fc.npad + kPrepassBlock - 1) / kPrepassBlock;
  int* status = noalloc_status_word(scratch);
  // The array keeps the previous call's contents: the source table and the
  // partials are rewritten in full below, the status word must start at zero.
  SOL_CUDA(cudaMemsetAsync(status, 0, sizeof(int), st));
  // rm3[0] (the central body) is never computed and reads as 0, as in the
  // reference, whose rm3 array starts zeroed (Acceleration.cpp:65-69).
  SOL_CUDA(cudaMemsetAsync(d_rm3, 0, sizeof(double), st));
  const int split = precision == SOL_PRECISION_SPLIT;
  k_prepass<<<fc.n_ind_blocks, kPrepassBlock, 0, st>>>(fc, d_y, split, 0);
  SOL_LAUNCHED();
  if (split) {
    k_ind_reduce<<<1, 256, 0, st>>>(fc);
    SOL_LAUNCHED();
  }
  TimeSpec ts{nullptr, nullptr, 0.0, 0.0};
  const int nb = (int)((n + kSinkBlock - 1) / kSinkBlock);
  const unsigned spin_hook = g_noalloc_spin.load();
  const unsigned spin = spin_hook ? spin_hook : SOL_SPIN_LIMIT;
  const int withhold = g_noalloc_withhold.load();
  if (split)
    k_gravity_ac<SOL_PRECISION_SPLIT><<<nb, kSinkBlock, 0, st>>>(fc, d_y, d_dydt, ts, 0u, status, spin, withhold);
  else
    k_gravity_ac<SOL_PRECISION_FP64><<<nb, kSinkBlock, 0, st>>>(fc, d_y, d_dydt, ts, 0u, status, spin, withhold);
  SOL_LAUNCHED();
  return SOL_OK;
}
