// Events applied on the device: Simulator::CheckEvent (Solaris/Simulator.cpp:
// 621-735) with RemoveBody (:737-771) and HandleCollision (:773-935).
//
// Order as in the reference: every ejection (rm3 below 1 / R_ej^3, logged and
// removed), then every hit-centrum body (rm3 above 1 / R_hc^3, merged into
// the central body and removed), then the nearest-neighbour collisions in
// body order (factor (R_i + R_j) above the nearest-neighbour distance: the
// lighter body merges into the heavier, ties to the lower index; momentum and
// mass add up, radius from the summed volume, density from mass over volume),
// each merger removed and its own nearest neighbour cleared.
//
// Steps without events cost one parallel predicate pass and a 4-byte read.
// With candidates, one warp walks the bodies in order 32 at a time,
// re-evaluating the predicates of the rest of each group after every merge
// (a merge changes a radius), then the bodies are compacted in parallel.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "sol_internal.cuh"

namespace {

constexpr int kBlock = 256;

struct EvArgs {
  int n;
  double time;
  double e3, h3, factor;  // 1 / R_ej^3, 1 / R_hc^3 (0: off), collision factor (<= 0: off)
  int32_t* id;
  int32_t* type;
  double* mass;
  double* radius;
  double* density;
  double* y0;
  const double* rm3;
  int32_t* nn_idx;
  const double* nn_dist;
  uint8_t* removed;
  sol_affair* log;
  int* n_log;
  int* n_candidates;
  int* removed_per_class;  // [8] by BodyType
};

__device__ __forceinline__ bool collides(const EvArgs& A, int i) {
  const int j = A.nn_idx[i];
  return j >= 0 && !A.removed[j] && A.factor * (A.radius[i] + A.radius[j]) > A.nn_dist[i];
}

// Is there anything to do?  Ejection / hit-centrum flags and collision
// candidates at the current radii.
__global__ void k_event_scan(EvArgs A) {
  int c = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < A.n; i += gridDim.x * blockDim.x) {
    if (i >= 1 && ((A.e3 > 0.0 && A.rm3[i] < A.e3) || (A.h3 > 0.0 && A.rm3[i] > A.h3))) ++c;
    if (A.factor > 0.0 && collides(A, i)) ++c;
  }
  if (c) atomicAdd(A.n_candidates, c);
}

__device__ void log_affair(const EvArgs& A, int type, int idx1, int idx2, int b1, int b2) {
  const int k = (*A.n_log)++;
  sol_affair& f = A.log[k];
  f.type = type;
  f.idx1 = idx1;
  f.idx2 = idx2;
  f.id1 = A.id[b1];
  f.id2 = A.id[b2];
  f.pad = 0;
  f.time = A.time;
  for (int q = 0; q < 6; ++q) {
    f.phase1[q] = A.y0[6 * b1 + q];
    f.phase2[q] = A.y0[6 * b2 + q];
  }
}

// Survivor and merger of HandleCollision (:773-782): the heavier survives,
// equal masses to the lower index.
__device__ __forceinline__ void survivor(const EvArgs& A, int a, int b, int& s, int& m) {
  if (A.mass[a] == A.mass[b]) {
    s = a < b ? a : b;
    m = a > b ? a : b;
  } else {
    s = A.mass[a] > A.mass[b] ? a : b;
    m = A.mass[a] < A.mass[b] ? a : b;
  }
}

// CalculatePhaseAfterCollision (:799-825) and
// CalculateCharacteristicsAfterCollision (:827-880) of merger m into s.
__device__ void merge(const EvArgs& A, int s, int m) {
  const double ms = A.mass[s];
  const double mm = A.type[m] == SOL_SUPER_PLANETESIMAL
                        ? A.density[m] * (4.0 / 3.0 * SOL_PI * (A.radius[m] * A.radius[m] * A.radius[m]))
                        : A.mass[m];
  const double M = ms + mm;
  if (A.type[s] != SOL_CENTRAL_BODY)
    for (int q = 0; q < 6; ++q) A.y0[6 * s + q] = 1.0 / M * (ms * A.y0[6 * s + q] + mm * A.y0[6 * m + q]);
  A.mass[s] = M;
  if (A.radius[s] != 0.0) {
    if (A.radius[m] == 0.0) {
      A.density[m] = A.density[s];
      A.radius[m] = sol_pow_recip_cr<3>(3.0 / (4.0 * SOL_PI) * A.mass[m] / A.density[m]);
    }
    const double rs = A.radius[s], rm = A.radius[m];
    const double vol = 4.0 / 3.0 * SOL_PI * (rs * rs * rs + rm * rm * rm);
    A.radius[s] = sol_pow_recip_cr<3>(3.0 / (4.0 * SOL_PI) * vol);
    A.density[s] = M / vol;
  }
}

__device__ void remove_body(const EvArgs& A, int i) {
  A.removed[i] = 1;
  const int t = A.type[i];
  if (t >= 0 && t < 8) A.removed_per_class[t]++;
}

// One warp, in order.  Ejections and hit-centrum bodies are found before any
// removal, so their log carries the original index; a collision's carries
// the positions among the bodies present at that moment.  Logged phases are
// those before a merge.
__device__ int position(const EvArgs& A, int b) {  // index among the bodies still present
  int p = 0;
  for (int q = 0; q < b; ++q) p += !A.removed[q];
  return p;
}

__global__ void k_event_apply(EvArgs A) {
  const int lane = threadIdx.x;
  if (lane == 0) *A.n_log = 0;
  __syncwarp();
  // ejections, then hit-centrum bodies (detected on the state before removals)
  for (int kind = 0; kind < 2; ++kind) {
    for (int base = 0; base < A.n; base += 32) {
      const int i = base + lane;
      bool hit = false;
      if (i < A.n && i >= 1 && !A.removed[i])
        hit = kind == 0 ? (A.e3 > 0.0 && A.rm3[i] < A.e3) : (A.h3 > 0.0 && A.rm3[i] > A.h3);
      const unsigned mask = __ballot_sync(0xffffffffu, hit);
      if (lane == 0) {
        for (int l = 0; l < 32; ++l) {
          if (!(mask & (1u << l))) continue;
          const int b = base + l;
          if (kind == 0) {
            log_affair(A, 0, 0, b, 0, b);  // Ejection
          } else {
            log_affair(A, 1, 0, b, 0, b);  // HitCentrum: into the central body
            int s, m;
            survivor(A, 0, b, s, m);
            if (A.type[m] != SOL_TEST_PARTICLE) merge(A, s, m);
          }
          remove_body(A, b);
        }
      }
      __syncwarp();
    }
  }
  if (!(A.factor > 0.0)) return;
  // collisions in body order; a merge changes radii, so the predicates of the
  // rest of a group are evaluated again after each one
  for (int base = 0; base < A.n; base += 32) {
    int start = 0;
    while (start < 32) {
      const int i = base + lane;
      const bool cand = lane >= start && i < A.n && !A.removed[i] && collides(A, i);
      const unsigned mask = __ballot_sync(0xffffffffu, cand);
      if (!mask) break;
      const int l = __ffs(mask) - 1;
      if (lane == 0) {
        const int b = base + l;
        const int j = A.nn_idx[b];
        int s, m;
        survivor(A, b, j, s, m);
        if (A.type[m] != SOL_TEST_PARTICLE) {
          log_affair(A, 3, position(A, s), position(A, m), s, m);  // Collision
          merge(A, s, m);
          remove_body(A, m);
          A.nn_idx[m] = -1;
        } else {
          A.nn_idx[b] = -1;  // a test particle does not merge (HandleCollision :784-785): handled once
        }
      }
      __syncwarp();
      start = l + 1;
    }
  }
}

// exclusive prefix count of the kept bodies: per-block counts, then one
// block scans them, then every body finds its new index
__global__ void k_keep_count(int n, const uint8_t* __restrict__ removed, int* __restrict__ block_count) {
  __shared__ int cnt;
  if (threadIdx.x == 0) cnt = 0;
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && !removed[i]) atomicAdd(&cnt, 1);
  __syncthreads();
  if (threadIdx.x == 0) block_count[blockIdx.x] = cnt;
}

__global__ void k_keep_scan(int nb, int* __restrict__ block_count) {
  if (threadIdx.x != 0) return;
  int acc = 0;
  for (int b = 0; b < nb; ++b) {
    const int c = block_count[b];
    block_count[b] = acc;
    acc += c;
  }
}

struct CompactArgs {
  int n;
  const uint8_t* removed;
  const int* block_offset;
  int* new_index;  // -1 for removed
};

__global__ void k_new_index(CompactArgs C) {
  __shared__ uint8_t keep[kBlock];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  keep[threadIdx.x] = (i < C.n && !C.removed[i]) ? 1 : 0;
  __syncthreads();
  if (i >= C.n) return;
  if (!keep[threadIdx.x]) {
    C.new_index[i] = -1;
    return;
  }
  int k = C.block_offset[blockIdx.x];
  for (int t = 0; t < (int)threadIdx.x; ++t) k += keep[t];
  C.new_index[i] = k;
}

template <class T>
__global__ void k_gather(int n, int width, const int* __restrict__ new_index, const T* __restrict__ in,
                         T* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int k = new_index[i];
  if (k < 0) return;
  for (int q = 0; q < width; ++q) out[(size_t)k * width + q] = in[(size_t)i * width + q];
}

// side buffers hold rows for a class range [lo, hi) of the bodies
__global__ void k_gather_rows(int lo_old, int hi_old, int lo_new, const int* __restrict__ new_index,
                              const double* __restrict__ in, double* __restrict__ out) {
  const int i = lo_old + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= hi_old) return;
  const int k = new_index[i];
  if (k < 0) return;
  for (int q = 0; q < 3; ++q) out[3 * (k - lo_new) + q] = in[3 * (i - lo_old) + q];
}

}  // namespace

int sol_force_part_doubles(const sol_ctx* c);
int sol_force_uses_chunk_partials(const sol_ctx* c, int precision);

extern "C" int sol_handle_events(sol_ctx* c, double time, double ejection, double hit_centrum,
                                 double collision_factor, sol_affair* log, int32_t capacity, int32_t* n_log) {
  if (!c || !n_log || capacity < 0 || (capacity > 0 && !log)) {
    sol_set_error("sol_handle_events: bad arguments");
    return SOL_ERR_ARG;
  }
  *n_log = 0;
  if (c->barycentric) {
    sol_set_error("events are defined for the heliocentric frame (rm3)");
    return SOL_ERR_ARG;
  }
  if (!c->last_eval_valid || !c->state_valid) {
    sol_set_error("no evaluation yet: run a driver call or a force evaluation first");
    return SOL_ERR_STATE;
  }
  SOL_CUDA(cudaSetDevice(c->device));
  const int n = c->n;
  // scratch: removed flags, log, counters, new indices, block offsets
  const int nb = (n + kBlock - 1) / kBlock;
  uint8_t* d_removed = nullptr;
  sol_affair* d_log = nullptr;
  int* d_words = nullptr;  // [0] n_log, [1] n_candidates, [2..9] removed per class, then new_index[n], offsets[nb]
  const size_t words = 10 + (size_t)n + (size_t)nb;
  int rc = SOL_OK;
  auto ck = [&](cudaError_t e, const char* what) {
    if (rc == SOL_OK && e != cudaSuccess) rc = sol_cuda_fail(e, what, __FILE__, __LINE__);
  };
  ck(cudaMallocAsync((void**)&d_removed, (size_t)n, c->stream), "cudaMallocAsync");
  ck(cudaMallocAsync((void**)&d_log, sizeof(sol_affair) * (size_t)n, c->stream), "cudaMallocAsync");
  ck(cudaMallocAsync((void**)&d_words, sizeof(int) * words, c->stream), "cudaMallocAsync");
  if (rc == SOL_OK) {
    ck(cudaMemsetAsync(d_removed, 0, (size_t)n, c->stream), "memset");
    ck(cudaMemsetAsync(d_words, 0, sizeof(int) * 10, c->stream), "memset");
  }
  EvArgs A;
  memset(&A, 0, sizeof(A));
  A.n = n;
  A.time = time;
  A.e3 = ejection > 0 ? 1.0 / (ejection * ejection * ejection) : 0.0;
  A.h3 = hit_centrum > 0 ? 1.0 / (hit_centrum * hit_centrum * hit_centrum) : 0.0;
  A.factor = collision_factor;
  A.type = const_cast<int32_t*>(c->d_type);
  A.mass = c->d_mass;
  A.radius = c->d_radius;
  A.density = c->d_density;
  A.y0 = c->d_y0;
  A.rm3 = c->d_rm3;
  A.nn_idx = c->d_nn_idx;
  A.nn_dist = c->d_nn_dist;
  A.removed = d_removed;
  A.log = d_log;
  A.n_log = d_words;
  A.n_candidates = d_words + 1;
  A.removed_per_class = d_words + 2;
  // device copy of the ids (the context keeps them on the host)
  int32_t* d_id = nullptr;
  ck(cudaMallocAsync((void**)&d_id, sizeof(int32_t) * (size_t)n, c->stream), "cudaMallocAsync");
  ck(cudaMemcpyAsync(d_id, c->h_id, sizeof(int32_t) * (size_t)n, cudaMemcpyHostToDevice, c->stream), "ids");
  A.id = d_id;
  int cand = 0;
  if (rc == SOL_OK) {
    k_event_scan<<<nb < 1024 ? nb : 1024, kBlock, 0, c->stream>>>(A);
    sol_count_launch();
    ck(cudaGetLastError(), "k_event_scan");
    ck(cudaMemcpyAsync(&cand, A.n_candidates, sizeof(int), cudaMemcpyDeviceToHost, c->stream), "count");
    ck(cudaStreamSynchronize(c->stream), "synchronize");
  }
  int nlog = 0;
  int per_class[8] = {0};
  if (rc == SOL_OK && cand > 0) {
    k_event_apply<<<1, 32, 0, c->stream>>>(A);
    sol_count_launch();
    ck(cudaGetLastError(), "k_event_apply");
    ck(cudaMemcpyAsync(&nlog, A.n_log, sizeof(int), cudaMemcpyDeviceToHost, c->stream), "log count");
    ck(cudaMemcpyAsync(per_class, A.removed_per_class, sizeof(per_class), cudaMemcpyDeviceToHost, c->stream),
       "removed count");
    ck(cudaStreamSynchronize(c->stream), "synchronize");
  }
  int n_removed = 0;
  for (int t = 0; t < 8; ++t) n_removed += per_class[t];
  if (rc == SOL_OK && nlog > 0 && capacity > 0)
    ck(cudaMemcpyAsync(log, d_log, sizeof(sol_affair) * (size_t)(nlog < capacity ? nlog : capacity),
                       cudaMemcpyDeviceToHost, c->stream),
       "log");
  if (rc == SOL_OK && n_removed > 0) {
    // compaction: new indices, then every per-body array through a scratch copy
    int* d_new = d_words + 10;
    int* d_off = d_new + n;
    k_keep_count<<<nb, kBlock, 0, c->stream>>>(n, d_removed, d_off);
    k_keep_scan<<<1, 32, 0, c->stream>>>(nb, d_off);
    CompactArgs C{n, d_removed, d_off, d_new};
    k_new_index<<<nb, kBlock, 0, c->stream>>>(C);
    for (int k = 0; k < 3; ++k) sol_count_launch();
    double* tmp = c->d_ytmp;  // 6N doubles of scratch
    auto gather_d = [&](double* arr, int width) {
      k_gather<double><<<nb, kBlock, 0, c->stream>>>(n, width, d_new, arr, tmp);
      sol_count_launch();
      ck(cudaMemcpyAsync(arr, tmp, sizeof(double) * (size_t)(n - n_removed) * width, cudaMemcpyDeviceToDevice,
                         c->stream),
         "compact");
    };
    auto gather_i = [&](int32_t* arr) {
      k_gather<int32_t><<<nb, kBlock, 0, c->stream>>>(n, 1, d_new, arr, reinterpret_cast<int32_t*>(tmp));
      sol_count_launch();
      ck(cudaMemcpyAsync(arr, tmp, sizeof(int32_t) * (size_t)(n - n_removed), cudaMemcpyDeviceToDevice, c->stream),
         "compact");
    };
    gather_d(c->d_y0, 6);
    for (double* a : {c->d_mig_stop_at, c->d_mass, c->d_radius, c->d_density, c->d_cd, c->d_gs, c->d_ge, c->d_rm3})
      gather_d(a, 1);
    gather_i(c->d_type);
    gather_i(c->d_mig_type);
    gather_i(d_id);
    // side buffers, by class range
    const Classes o = c->cls;
    sol_nbodies k = c->counts;
    k.central_body -= per_class[SOL_CENTRAL_BODY];
    k.giant_planet -= per_class[SOL_GIANT_PLANET];
    k.rocky_planet -= per_class[SOL_ROCKY_PLANET];
    k.proto_planet -= per_class[SOL_PROTO_PLANET];
    k.super_planetesimal -= per_class[SOL_SUPER_PLANETESIMAL];
    k.planetesimal -= per_class[SOL_PLANETESIMAL];
    k.test_particle -= per_class[SOL_TEST_PARTICLE];
    Classes nw = o;
    nw.n = n - n_removed;
    nw.n_central = k.central_body;
    nw.n_giant = k.giant_planet;
    nw.n_rocky = k.rocky_planet;
    nw.n_proto = k.proto_planet;
    nw.n_spl = k.super_planetesimal;
    nw.n_pl = k.planetesimal;
    nw.nm = k.central_body + k.giant_planet + k.rocky_planet + k.proto_planet;
    struct Range {
      double* buf;
      int lo_old, hi_old, lo_new, hi_new;
    } ranges[3] = {{c->d_drag, o.nm, o.nm + o.n_spl + o.n_pl, nw.nm, nw.nm + nw.n_spl + nw.n_pl},
                   {c->d_mig1, o.n_central + o.n_giant, o.nm, nw.n_central + nw.n_giant, nw.nm},
                   {c->d_mig2, o.n_central, o.n_central + o.n_giant, nw.n_central, nw.n_central + nw.n_giant}};
    for (const Range& r : ranges) {
      const int rows = r.hi_old - r.lo_old;
      if (rows <= 0 || !r.buf) continue;
      k_gather_rows<<<(rows + kBlock - 1) / kBlock, kBlock, 0, c->stream>>>(r.lo_old, r.hi_old, r.lo_new, d_new,
                                                                            r.buf, tmp);
      sol_count_launch();
      if (r.hi_new > r.lo_new)
        ck(cudaMemcpyAsync(r.buf, tmp, sizeof(double) * 3 * (size_t)(r.hi_new - r.lo_new),
                           cudaMemcpyDeviceToDevice, c->stream),
           "compact side buffer");
    }
    // nearest neighbours are those of the next evaluation
    ck(cudaMemsetAsync(c->d_nn_idx, 0xff, sizeof(int32_t) * (size_t)n, c->stream), "nn");
    ck(cudaMemsetAsync(c->d_nn_dist, 0, sizeof(double) * (size_t)n, c->stream), "nn");
    std::vector<int32_t> ids((size_t)(n - n_removed));
    ck(cudaMemcpyAsync(ids.data(), d_id, sizeof(int32_t) * ids.size(), cudaMemcpyDeviceToHost, c->stream), "ids");
    ck(cudaStreamSynchronize(c->stream), "synchronize");
    if (rc == SOL_OK) {
      memcpy(c->h_id, ids.data(), sizeof(int32_t) * ids.size());
      c->counts = k;
      c->cls = nw;
      c->fc.cls = nw;
      c->n = nw.n;
      c->nv = 6 * nw.n;
      c->fc.has_mig1 = nw.n_proto > 0 && c->fc.has_mig1;
      c->fc.has_mig2 = nw.n_giant > 0 && c->fc.has_mig2;
      for (int g = 0; g < 2; ++g) sol_graph_release(c->graphs[g]);  // captured with the old body count
      // a smaller system may move to the 2-D split kernel, which needs its partials
      if (c->precision != SOL_PRECISION_FP64 && !c->d_part && sol_force_uses_chunk_partials(c, c->precision)) {
        if (cudaMalloc((void**)&c->d_part, sizeof(double) * (size_t)sol_force_part_doubles(c)) != cudaSuccess) {
          sol_set_error("cudaMalloc of the split partials failed");
          rc = SOL_ERR_NOMEM;
        }
      }
      sol_adjoint_free(c->adj);
      c->adj = nullptr;
      c->last_eval_valid = 0;
    }
  }
  for (void* p : {(void*)d_removed, (void*)d_log, (void*)d_words, (void*)d_id})
    if (p) cudaFreeAsync(p, c->stream);
  ck(cudaStreamSynchronize(c->stream), "synchronize");
  *n_log = nlog;
  return rc;
}

// SaveTwoBodyAffair (Solaris/BinaryFileAdapter.cpp:244-261): int32 event id,
// int32 type (EventType: 0 ejection, 1 hit centrum, 3 collision), int32
// body ids, 6 + 6 doubles of phases, double time; appended to path.
extern "C" int sol_write_affairs(const char* path, const sol_affair* affairs, int32_t n, int32_t first_event_id) {
  if (!path || n < 0 || (n > 0 && !affairs)) {
    sol_set_error("sol_write_affairs: bad arguments");
    return SOL_ERR_ARG;
  }
  FILE* f = fopen(path, "ab");
  if (!f) {
    sol_set_error("cannot open %s for appending", path);
    return SOL_ERR_ARG;
  }
  bool ok = true;
  for (int k = 0; k < n && ok; ++k) {
    const sol_affair& a = affairs[k];
    const int32_t head[4] = {first_event_id + k, a.type, a.id1, a.id2};
    ok = fwrite(head, sizeof(head), 1, f) == 1 && fwrite(a.phase1, sizeof(double), 6, f) == 6 &&
         fwrite(a.phase2, sizeof(double), 6, f) == 6 && fwrite(&a.time, sizeof(double), 1, f) == 1;
  }
  if (fclose(f) != 0) ok = false;
  if (!ok) {
    sol_set_error("writing %s failed", path);
    return SOL_ERR_ARG;
  }
  return SOL_OK;
}

extern "C" int sol_get_bodies(sol_ctx* c, sol_nbodies* counts, int32_t* id, int32_t* type, double* mass,
                              double* radius, double* density) {
  if (!c) {
    sol_set_error("null context");
    return SOL_ERR_ARG;
  }
  SOL_CUDA(cudaSetDevice(c->device));
  const size_t n = (size_t)c->n;
  if (counts) *counts = c->counts;
  if (id) memcpy(id, c->h_id, sizeof(int32_t) * n);
  if (type) SOL_CUDA(cudaMemcpyAsync(type, c->d_type, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, c->stream));
  if (mass) SOL_CUDA(cudaMemcpyAsync(mass, c->d_mass, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
  if (radius) SOL_CUDA(cudaMemcpyAsync(radius, c->d_radius, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
  if (density)
    SOL_CUDA(cudaMemcpyAsync(density, c->d_density, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
  SOL_CUDA(cudaStreamSynchronize(c->stream));
  return SOL_OK;
}
