// Output of the integration in the files and record layouts of the
// reference's BinaryFileAdapter (Solaris/BinaryFileAdapter.cpp:107-219):
// phases (time, body count, then id and x y z vx vy vz per body; binary or
// text) and integrals (a length-prefixed header once, then element count,
// time and the 16 values of Calculate::Integrals per record).
//
// A phases snapshot costs the integration one device-to-device copy of the
// state on the context's stream; a copy stream brings the snapshot into
// pinned host memory and a writer thread appends the record, so the next
// driver calls run while the previous snapshot is written.
#include <cstdio>
#include <cstring>
#include <condition_variable>
#include <deque>
#include <iomanip>
#include <mutex>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "sol_internal.cuh"

namespace {

// The header the reference writes before the first integrals record
// (BinaryFileAdapter.cpp:182-188): part of the file format.
const char kIntegralsHeader[] =
    "time [day], mass [Solar], bary center position r: x [AU], y [AU], z [AU], bary center velocity v: x [AU/day], "
    "y [AU/day], z [AU/day], length of r [AU], length of v [AU/day], angular momentum vector c: x, y, z, length of c, "
    "kinetic energy, potential energy, total energy";

void put_bytes(std::string& s, const void* p, size_t n) { s.append(reinterpret_cast<const char*>(p), n); }

std::string phases_record(double time, int n, const double* y, const int32_t* id, bool text) {
  std::string out;
  if (!text) {  // BinaryFileAdapter::SavePhases / SavePhase, BINARY
    out.reserve(12 + (size_t)n * 52);
    put_bytes(out, &time, sizeof(time));
    put_bytes(out, &n, sizeof(n));
    for (int i = 0; i < n; ++i) {
      put_bytes(out, &id[i], sizeof(int32_t));
      put_bytes(out, &y[6 * i], 6 * sizeof(double));
    }
    return out;
  }
  std::ostringstream w;  // TEXT: the same stream manipulators
  w << std::setw(15) << std::setprecision(10) << time;
  w << std::setw(8) << n;
  for (int i = 0; i < n; ++i) {
    w << std::setw(8) << id[i];
    for (int k = 0; k < 6; ++k) w << std::setw(15) << std::setprecision(6) << y[6 * i + k];
  }
  w << std::endl;
  return w.str();
}

std::string integrals_record(double time, int n, const double* v, bool header) {
  std::string out;
  if (header) {
    const int len = (int)strlen(kIntegralsHeader);
    put_bytes(out, &len, sizeof(len));
    out.append(kIntegralsHeader, len);
  }
  const int n_element = n + 1;
  put_bytes(out, &n_element, sizeof(n_element));
  put_bytes(out, &time, sizeof(time));
  put_bytes(out, v, (size_t)n * sizeof(double));
  return out;
}

int copy_out(const std::string& s, char* buf, int64_t cap, int64_t* len) {
  if (len) *len = (int64_t)s.size();
  if (!buf) return SOL_OK;  // size query
  if (cap < (int64_t)s.size()) {
    sol_set_error("record needs %lld bytes, buffer has %lld", (long long)s.size(), (long long)cap);
    return SOL_ERR_ARG;
  }
  memcpy(buf, s.data(), s.size());
  return SOL_OK;
}

constexpr int kSlots = 3;

struct Job {
  int kind;  // 0 phases, 1 integrals
  int slot;
  double time;
  int n;
  std::vector<int32_t> id;
  double integrals[16];
};

}  // namespace

struct sol_output {
  sol_ctx* ctx;
  bool text;
  FILE* phases;
  FILE* integrals;
  bool integrals_header;
  cudaStream_t copy;
  double* d_snap[kSlots];
  double* h_snap[kSlots];
  cudaEvent_t ev_snap[kSlots], ev_host[kSlots];
  bool busy[kSlots];
  int next;
  std::mutex mu;
  std::condition_variable cv;
  std::deque<Job> jobs;
  bool stop;
  int status;
  std::string error;
  std::thread worker;
};

namespace {

void worker_loop(sol_output* o) {
  cudaSetDevice(o->ctx->device);
  for (;;) {
    Job job;
    {
      std::unique_lock<std::mutex> lk(o->mu);
      o->cv.wait(lk, [&] { return o->stop || !o->jobs.empty(); });
      if (o->jobs.empty()) return;
      job = std::move(o->jobs.front());
      o->jobs.pop_front();
    }
    std::string rec;
    FILE* f = nullptr;
    int st = SOL_OK;
    std::string msg;
    if (job.kind == 0) {
      const cudaError_t e = cudaEventSynchronize(o->ev_host[job.slot]);
      if (e != cudaSuccess) {
        st = SOL_ERR_CUDA;
        msg = std::string("snapshot copy failed: ") + cudaGetErrorString(e);
      } else {
        rec = phases_record(job.time, job.n, o->h_snap[job.slot], job.id.data(), o->text);
        f = o->phases;
      }
    } else {
      rec = integrals_record(job.time, 16, job.integrals, !o->integrals_header);
      o->integrals_header = true;
      f = o->integrals;
    }
    if (st == SOL_OK && f && (fwrite(rec.data(), 1, rec.size(), f) != rec.size() || fflush(f) != 0)) {
      st = SOL_ERR_ARG;
      msg = "writing an output record failed";
    }
    std::lock_guard<std::mutex> lk(o->mu);
    if (job.kind == 0) o->busy[job.slot] = false;
    if (st != SOL_OK && o->status == SOL_OK) {
      o->status = st;
      o->error = msg;
    }
    o->cv.notify_all();
  }
}

FILE* open_append(const char* path, bool* was_empty) {
  if (!path || !*path) return nullptr;
  FILE* f = fopen(path, "ab");
  if (f && was_empty) {
    fseek(f, 0, SEEK_END);
    *was_empty = ftell(f) == 0;
  }
  return f;
}

void destroy(sol_output* o) {
  if (!o) return;
  {
    std::lock_guard<std::mutex> lk(o->mu);
    o->stop = true;
  }
  o->cv.notify_all();
  if (o->worker.joinable()) o->worker.join();
  cudaSetDevice(o->ctx->device);
  for (int s = 0; s < kSlots; ++s) {
    if (o->d_snap[s]) cudaFree(o->d_snap[s]);
    if (o->h_snap[s]) cudaFreeHost(o->h_snap[s]);
    if (o->ev_snap[s]) cudaEventDestroy(o->ev_snap[s]);
    if (o->ev_host[s]) cudaEventDestroy(o->ev_host[s]);
  }
  if (o->copy) cudaStreamDestroy(o->copy);
  if (o->phases) fclose(o->phases);
  if (o->integrals) fclose(o->integrals);
  delete o;
}

}  // namespace

extern "C" {

int sol_format_phases_record(double time, int32_t n, const double* y, const int32_t* id, int32_t text, char* buf,
                             int64_t capacity, int64_t* length) {
  if (n < 0 || (n > 0 && (!y || !id))) {
    sol_set_error("sol_format_phases_record: bad arguments");
    return SOL_ERR_ARG;
  }
  return copy_out(phases_record(time, n, y, id, text != 0), buf, capacity, length);
}

int sol_format_integrals_record(double time, int32_t n, const double* integrals, int32_t header, char* buf,
                                int64_t capacity, int64_t* length) {
  if (n < 0 || (n > 0 && !integrals)) {
    sol_set_error("sol_format_integrals_record: bad arguments");
    return SOL_ERR_ARG;
  }
  return copy_out(integrals_record(time, n, integrals, header != 0), buf, capacity, length);
}

int sol_output_open(sol_ctx* c, const char* phases_path, const char* integrals_path, int32_t text, sol_output** out) {
  if (!c || !out) {
    sol_set_error("sol_output_open: bad arguments");
    return SOL_ERR_ARG;
  }
  *out = nullptr;
  SOL_CUDA(cudaSetDevice(c->device));
  sol_output* o = new sol_output();
  o->ctx = c;
  o->text = text != 0;
  o->status = SOL_OK;
  bool empty = true;
  o->phases = open_append(phases_path, nullptr);
  o->integrals = open_append(integrals_path, &empty);
  o->integrals_header = !empty;  // the header opens a new integrals file
  if ((phases_path && *phases_path && !o->phases) || (integrals_path && *integrals_path && !o->integrals)) {
    sol_set_error("cannot open an output file for appending");
    destroy(o);
    return SOL_ERR_ARG;
  }
  const size_t bytes = sizeof(double) * c->nv;
  bool ok = cudaStreamCreateWithFlags(&o->copy, cudaStreamNonBlocking) == cudaSuccess;
  for (int s = 0; s < kSlots && ok; ++s) {
    ok = cudaMalloc((void**)&o->d_snap[s], bytes) == cudaSuccess &&
         cudaMallocHost((void**)&o->h_snap[s], bytes) == cudaSuccess &&
         cudaEventCreateWithFlags(&o->ev_snap[s], cudaEventDisableTiming) == cudaSuccess &&
         cudaEventCreateWithFlags(&o->ev_host[s], cudaEventDisableTiming) == cudaSuccess;
  }
  if (!ok) {
    sol_set_error("output buffers could not be allocated");
    destroy(o);
    return SOL_ERR_NOMEM;
  }
  o->worker = std::thread(worker_loop, o);
  *out = o;
  return SOL_OK;
}

int sol_output_save_phases(sol_output* o, double time) {
  if (!o || !o->phases) {
    sol_set_error("sol_output_save_phases: no phases file");
    return SOL_ERR_ARG;
  }
  sol_ctx* c = o->ctx;
  if (!c->state_valid) {
    sol_set_error("no state: call sol_set_state first");
    return SOL_ERR_STATE;
  }
  SOL_CUDA(cudaSetDevice(c->device));
  int s;
  {
    std::unique_lock<std::mutex> lk(o->mu);
    o->cv.wait(lk, [&] { return !o->busy[o->next]; });
    if (o->status != SOL_OK) {
      sol_set_error("%s", o->error.c_str());
      return o->status;
    }
    s = o->next;
    o->busy[s] = true;
    o->next = (o->next + 1) % kSlots;
  }
  const size_t bytes = sizeof(double) * c->nv;
  // the state as the compute stream has it now; the copy to the host overlaps
  // with whatever the compute stream runs next
  cudaError_t e = cudaMemcpyAsync(o->d_snap[s], c->d_y0, bytes, cudaMemcpyDeviceToDevice, c->stream);
  if (e == cudaSuccess) e = cudaEventRecord(o->ev_snap[s], c->stream);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(o->copy, o->ev_snap[s], 0);
  if (e == cudaSuccess) e = cudaMemcpyAsync(o->h_snap[s], o->d_snap[s], bytes, cudaMemcpyDeviceToHost, o->copy);
  if (e == cudaSuccess) e = cudaEventRecord(o->ev_host[s], o->copy);
  if (e != cudaSuccess) {
    std::lock_guard<std::mutex> lk(o->mu);
    o->busy[s] = false;
    return sol_cuda_fail(e, "phases snapshot", __FILE__, __LINE__);
  }
  Job job;
  job.kind = 0;
  job.slot = s;
  job.time = time;
  job.n = c->n;
  job.id.assign(c->h_id, c->h_id + c->n);
  {
    std::lock_guard<std::mutex> lk(o->mu);
    o->jobs.push_back(std::move(job));
  }
  o->cv.notify_all();
  return SOL_OK;
}

int sol_output_save_integrals(sol_output* o, double time) {
  if (!o || !o->integrals) {
    sol_set_error("sol_output_save_integrals: no integrals file");
    return SOL_ERR_ARG;
  }
  Job job;
  job.kind = 1;
  job.slot = -1;
  job.time = time;
  job.n = 16;
  const int rc = sol_integrals(o->ctx, nullptr, job.integrals);
  if (rc != SOL_OK) return rc;
  {
    std::lock_guard<std::mutex> lk(o->mu);
    o->jobs.push_back(std::move(job));
  }
  o->cv.notify_all();
  return SOL_OK;
}

int sol_output_flush(sol_output* o) {
  if (!o) return SOL_ERR_ARG;
  std::unique_lock<std::mutex> lk(o->mu);
  o->cv.wait(lk, [&] {
    if (!o->jobs.empty()) return false;
    for (int s = 0; s < kSlots; ++s)
      if (o->busy[s]) return false;
    return true;
  });
  if (o->status != SOL_OK) sol_set_error("%s", o->error.c_str());
  return o->status;
}

int sol_output_close(sol_output* o) {
  if (!o) return SOL_OK;
  const int rc = sol_output_flush(o);
  destroy(o);
  return rc;
}

}  // extern "C"
