// Contexts behind the C++ class facade and the host read-back of the members
// the reference classes leave in host memory.
//
// An Acceleration owns up to two libsolaris_gb300 contexts (heliocentric and
// barycentric frame, the second only if a caller asks for it).  A context is
// built from a snapshot of the body set: counts, id, type, migType and the
// per-body parameters, plus the nebula's gas component.  Every call compares
// the caller's BodyData and Nebula with the snapshot and rebuilds the
// contexts when they differ, so the caller keeps the reference's freedom to
// remove, merge or edit bodies between calls (Simulator::RemoveBody and
// HandleCollision, Simulator.cpp:737-935).  migType changes made on the
// device (a migrating body reaching migStopAt) are copied into BodyData and
// the snapshot after every call.
//
// Environment: SOLARIS_GB300_PRECISION = fp64 (default) | split | split_ff
// selects the pair arithmetic; SOLARIS_GB300_DEVICE the CUDA device.
#include "facade_state.h"

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <mutex>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

#include "Acceleration.h"
#include "BodyData.h"
#include "Error.h"
#include "GasComponent.h"
#include "Nebula.h"
#include "TimeLine.h"

namespace solgb_facade {
namespace {

constexpr int kInts = 3;  // id, type, migType
constexpr int kDbls = 7;  // migStopAt, mass, radius, density, cD, gammaStokes, gammaEpstein

struct Snapshot {
  int counts[7] = {0, 0, 0, 0, 0, 0, 0};
  int total = -1;
  std::vector<int32_t> ints;
  std::vector<double> dbls;
  bool has_gas = false;
  sol_gas_component gas;
  int precision = 0;
};

struct Entry {
  bool barycentric = false;
  sol_ctx* ctx[2] = {nullptr, nullptr};
  Snapshot snap;
};

std::mutex g_mu;
std::unordered_map<const Acceleration*, Entry*> g_table;

int env_precision() {
  const char* p = std::getenv("SOLARIS_GB300_PRECISION");
  if (!p) return SOL_PRECISION_FP64;
  const std::string s(p);
  if (s == "split") return SOL_PRECISION_SPLIT;
  if (s == "split_ff") return SOL_PRECISION_SPLIT_FF;
  return SOL_PRECISION_FP64;
}

int env_device() {
  const char* p = std::getenv("SOLARIS_GB300_DEVICE");
  return p ? std::atoi(p) : 0;
}

// A failure found by the facade itself (not by a library call) is reported
// with its own message instead of the library's last one.
thread_local std::string g_msg;

void set_error(const std::string& msg) { g_msg = msg; }

void counts_of(BodyData* bd, int c[7]) {
  const NBodies& n = bd->nBodies;
  c[0] = n.centralBody;
  c[1] = n.giantPlanet;
  c[2] = n.rockyPlanet;
  c[3] = n.protoPlanet;
  c[4] = n.superPlanetsimal;
  c[5] = n.planetsimal;
  c[6] = n.testParticle;
}

const int* int_array(BodyData* bd, int k) {
  return k == 0 ? bd->id : k == 1 ? bd->type : bd->migType;
}

const double* dbl_array(BodyData* bd, int k) {
  switch (k) {
    case 0: return bd->migStopAt;
    case 1: return bd->mass;
    case 2: return bd->radius;
    case 3: return bd->density;
    case 4: return bd->cD;
    case 5: return bd->gammaStokes;
    default: return bd->gammaEpstein;
  }
}

void gas_of(Nebula* neb, sol_gas_component* g) {
  sol_gas_component_init(g);  // quirk bits of the reference build
  GasComponent& gc = neb->gasComponent;
  g->alpha = gc.alpha;
  g->decrease_type = (int32_t)gc.type;
  g->time_scale = gc.timeScale;
  g->t0 = gc.t0;
  g->t1 = gc.t1;
  g->inner_edge = gc.innerEdge;
  g->mean_molecular_weight = gc.meanMolecularWeight;
  g->particle_diameter = gc.particleDiameter;
  g->eta = sol_power_law{gc.eta.c, gc.eta.index};
  g->tau = sol_power_law{gc.tau.c, gc.tau.index};
  g->scale_height = sol_power_law{gc.scaleHeight.c, gc.scaleHeight.index};
  g->density = sol_power_law{gc.density.c, gc.density.index};
  g->mean_free_path = sol_power_law{gc.meanFreePath.c, gc.meanFreePath.index};
}

// Does the snapshot still describe the caller's body set and nebula?
bool unchanged(const Snapshot& s, BodyData* bd, const sol_gas_component& gas, bool has_gas, int precision) {
  int c[7];
  counts_of(bd, c);
  if (s.total != bd->nBodies.total || std::memcmp(c, s.counts, sizeof(c)) != 0) return false;
  if (s.has_gas != has_gas || s.precision != precision) return false;
  if (has_gas && std::memcmp(&s.gas, &gas, sizeof(gas)) != 0) return false;
  const size_t n = (size_t)s.total;
  for (int k = 0; k < kInts; ++k) {
    const int* a = int_array(bd, k);
    if (a && std::memcmp(a, s.ints.data() + k * n, n * sizeof(int32_t)) != 0) return false;
  }
  for (int k = 0; k < kDbls; ++k) {
    const double* a = dbl_array(bd, k);
    if (a && std::memcmp(a, s.dbls.data() + k * n, n * sizeof(double)) != 0) return false;
  }
  return true;
}

void take_snapshot(Snapshot& s, BodyData* bd, const sol_gas_component& gas, bool has_gas, int precision) {
  counts_of(bd, s.counts);
  s.total = bd->nBodies.total;
  const size_t n = (size_t)s.total;
  s.ints.assign(kInts * n, 0);
  s.dbls.assign(kDbls * n, 0.0);
  for (int k = 0; k < kInts; ++k)
    if (const int* a = int_array(bd, k)) std::memcpy(s.ints.data() + k * n, a, n * sizeof(int32_t));
  for (int k = 0; k < kDbls; ++k)
    if (const double* a = dbl_array(bd, k)) std::memcpy(s.dbls.data() + k * n, a, n * sizeof(double));
  s.has_gas = has_gas;
  s.gas = gas;
  s.precision = precision;
}

void drop_contexts(Entry* e) {
  for (int f = 0; f < 2; ++f) {
    if (e->ctx[f]) sol_destroy(e->ctx[f]);
    e->ctx[f] = nullptr;
  }
}

Entry* entry_of(const Acceleration* acc) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_table.find(acc);
  return it == g_table.end() ? nullptr : it->second;
}

// The context of acc's current body set in the given frame (nullptr with
// Error::_errMsg set on failure).
sol_ctx* context(Acceleration* acc, bool bary) {
  Entry* e = entry_of(acc);
  if (!e) {
    set_error("Acceleration object not registered with the GB300 facade");
    return nullptr;
  }
  BodyData* bd = acc->bodyData;
  if (!bd || bd->nBodies.total <= 0) {
    set_error("Acceleration has no bodies");
    return nullptr;
  }
  int c[7];
  counts_of(bd, c);
  int sum = 0;
  for (int k = 0; k < 7; ++k) sum += c[k];
  if (sum != bd->nBodies.total) {
    set_error("NBodies::total differs from the sum of the class counts");
    return nullptr;
  }
  sol_gas_component gas;
  std::memset(&gas, 0, sizeof(gas));
  const bool has_gas = acc->nebula != nullptr;
  if (has_gas) gas_of(acc->nebula, &gas);
  const int precision = env_precision();
  if (!unchanged(e->snap, bd, gas, has_gas, precision)) {
    drop_contexts(e);
    take_snapshot(e->snap, bd, gas, has_gas, precision);
  }
  const int f = bary ? 1 : 0;
  if (!e->ctx[f]) {
    const Snapshot& s = e->snap;
    const size_t n = (size_t)s.total;
    sol_body_data sd;
    sd.n = sol_nbodies{s.counts[0], s.counts[1], s.counts[2], s.counts[3], s.counts[4], s.counts[5], s.counts[6]};
    sd.id = s.ints.data();
    sd.type = s.ints.data() + n;
    sd.mig_type = s.ints.data() + 2 * n;
    sd.mig_stop_at = s.dbls.data();
    sd.mass = s.dbls.data() + n;
    sd.radius = s.dbls.data() + 2 * n;
    sd.density = s.dbls.data() + 3 * n;
    sd.cd = s.dbls.data() + 4 * n;
    sd.gamma_stokes = s.dbls.data() + 5 * n;
    sd.gamma_epstein = s.dbls.data() + 6 * n;
    sol_ctx* ctx = nullptr;
    if (sol_create(&sd, has_gas ? &s.gas : nullptr, bary ? 1 : 0, env_device(), &ctx) != SOL_OK) return nullptr;
    // barycentric contexts have the FP64 form only
    if (sol_set_precision(ctx, bary ? SOL_PRECISION_FP64 : precision) != SOL_OK) {
      sol_destroy(ctx);
      return nullptr;
    }
    e->ctx[f] = ctx;
  }
  return e->ctx[f];
}

uint32_t flags_of(const Acceleration* acc) {
  return (acc->evaluateGasDrag ? SOL_EVAL_GAS_DRAG : 0u) | (acc->evaluateTypeIMigration ? SOL_EVAL_TYPE_I : 0u) |
         (acc->evaluateTypeIIMigration ? SOL_EVAL_TYPE_II : 0u);
}

// The reference allocates these lazily on first use (Acceleration.cpp:65-69,
// :180-184, :200-204, :222-226).  accelMigrationTypeI covers rocky and proto
// planets, the range the reference indexes it with.
void ensure_host_buffers(Acceleration* acc) {
  BodyData* bd = acc->bodyData;
  NBodies& nb = bd->nBodies;
  if (!acc->rm3) acc->rm3 = new double[nb.total]();
  if (!acc->nebula) return;
  if (!acc->accelGasDrag && nb.NOfPlAndSpl() > 0) acc->accelGasDrag = new double[3 * nb.NOfPlAndSpl()]();
  if (!acc->accelMigrationTypeI && nb.protoPlanet > 0)
    acc->accelMigrationTypeI = new double[3 * (nb.rockyPlanet + nb.protoPlanet)]();
  if (!acc->accelMigrationTypeII && nb.giantPlanet > 0) acc->accelMigrationTypeII = new double[3 * nb.giantPlanet]();
}

// migType as the device left it, into BodyData and the snapshot; a change
// makes the other frame's context stale.
int read_mig_type(Acceleration* acc, sol_ctx* c, bool bary) {
  BodyData* bd = acc->bodyData;
  Entry* e = entry_of(acc);
  const int n = bd->nBodies.total;
  std::vector<int32_t> m((size_t)n);
  if (sol_get_mig_type(c, m.data()) != SOL_OK) return 1;
  int32_t* snap = e->snap.ints.data() + 2 * (size_t)n;
  if (std::memcmp(m.data(), snap, sizeof(int32_t) * n) != 0) {
    std::memcpy(snap, m.data(), sizeof(int32_t) * n);
    if (bd->migType) std::memcpy(bd->migType, m.data(), sizeof(int32_t) * n);
    const int other = bary ? 0 : 1;
    if (e->ctx[other]) {
      sol_destroy(e->ctx[other]);
      e->ctx[other] = nullptr;
    }
  }
  return 0;
}

// Everything an evaluation leaves on the host in the reference: rm3
// (heliocentric only), the nearest-neighbour arrays, migType and the side
// buffers.
int read_back(Acceleration* acc, sol_ctx* c, bool bary) {
  ensure_host_buffers(acc);
  BodyData* bd = acc->bodyData;
  if (sol_get_last_eval(c, bary ? nullptr : acc->rm3, bd->indexOfNN, bd->distanceOfNN) != SOL_OK) return 1;
  if (read_mig_type(acc, c, bary)) return 1;
  if (acc->nebula &&
      sol_get_side_buffers(c, acc->accelGasDrag, acc->accelMigrationTypeI, acc->accelMigrationTypeII) != SOL_OK)
    return 1;
  return 0;
}

}  // namespace

int fail(const char* file, const char* function, long line) {
  if (!g_msg.empty()) {
    Error::_errMsg = g_msg;
    g_msg.clear();
  } else {
    const char* m = sol_last_error();
    if (m && *m) Error::_errMsg = m;
  }
  Error::PushLocation(file, function, line);
  return 1;
}

void attach(const Acceleration* acc, bool barycentric) {
  std::lock_guard<std::mutex> lk(g_mu);
  Entry*& e = g_table[acc];
  if (!e) e = new Entry();
  e->barycentric = barycentric;
}

void detach(const Acceleration* acc) {
  Entry* e = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_table.find(acc);
    if (it == g_table.end()) return;
    e = it->second;
    g_table.erase(it);
  }
  drop_contexts(e);
  delete e;
}

bool barycentric_of(const Acceleration* acc) {
  Entry* e = entry_of(acc);
  return e && e->barycentric;
}

int compute(Acceleration* acc, bool bary, double t, const double* y, double* dydt) {
  sol_ctx* c = context(acc, bary);
  if (!c) return 1;
  if (sol_set_eval_flags(c, flags_of(acc)) != SOL_OK) return 1;
  if (sol_accel_compute(c, t, y, dydt, nullptr, nullptr, nullptr) != SOL_OK) return 1;
  return read_back(acc, c, bary);
}

int term(Acceleration* acc, bool bary, int which, double t, const double* y, double* out, int row_begin,
         int row_end) {
  sol_ctx* c = context(acc, bary);
  if (!c) return 1;
  BodyData* bd = acc->bodyData;
  const int n = bd->nBodies.total;
  if (which != SOL_TERM_GRAVITY || row_begin < 0) {
    if (sol_accel_term(c, which, t, y, out) != SOL_OK) return 1;
    return read_back(acc, c, bary);
  }
  // a block of body rows of the gravity term
  std::vector<double> full(6 * (size_t)n), rm3((size_t)n), nd((size_t)n);
  std::vector<int32_t> nn((size_t)n);
  if (sol_accel_term(c, which, t, y, full.data()) != SOL_OK) return 1;
  if (sol_get_last_eval(c, rm3.data(), nn.data(), nd.data()) != SOL_OK) return 1;
  for (int i = row_begin; i < row_end && i < n; ++i) {
    for (int k = 0; k < 6; ++k) out[6 * i + k] = full[6 * (size_t)i + k];
    if (bd->indexOfNN) bd->indexOfNN[i] = nn[i];
    if (bd->distanceOfNN) bd->distanceOfNN[i] = nd[i];
  }
  return 0;
}

double helper(Acceleration* acc, bool bary, int which, const double* args) {
  double out = std::numeric_limits<double>::quiet_NaN();
  sol_ctx* c = context(acc, bary);
  if (!c || sol_migration_helper(c, which, args, &out) != SOL_OK) {
    fail(__FILE__, __func__, __LINE__);
    return std::numeric_limits<double>::quiet_NaN();
  }
  return out;
}

int driver(int integrator, double epsilon, BodyData* bd, Acceleration* acc, TimeLine* tl) {
  const bool bary = barycentric_of(acc);
  sol_ctx* c = context(acc, bary);
  if (!c) return 1;
  if (sol_set_tolerance(c, epsilon) != SOL_OK) return 1;
  bd->time = tl->time;
  if (integrator != SOL_DORMAND_PRINCE) bd->h = tl->hNext;
  // the Driver's first evaluation has every term on; afterwards only the drag
  acc->evaluateGasDrag = true;
  acc->evaluateTypeIMigration = true;
  acc->evaluateTypeIIMigration = true;
  const size_t nv = (size_t)bd->nBodies.NOfVar();
  std::memcpy(bd->y, bd->y0, nv * sizeof(double));  // y receives the new state, y0 keeps the old
  sol_time_line t{tl->time, tl->hNext, tl->hDid};
  const int rc = sol_driver_host(c, integrator, bd->y, &t, 1, nullptr);
  acc->evaluateTypeIMigration = false;
  acc->evaluateTypeIIMigration = false;
  if (rc != SOL_OK) return 1;
  if (sol_get_driver_vectors(c, bd->accel, integrator == SOL_RUNGE_KUTTA_FEHLBERG78 ? bd->yscale : nullptr,
                             integrator != SOL_RUNGE_KUTTA4 ? bd->error : nullptr) != SOL_OK)
    return 1;
  if (read_back(acc, c, bary)) return 1;
  tl->time = t.time;
  tl->hNext = t.h_next;
  tl->hDid = t.h_did;
  bd->time = tl->time;
  bd->h = integrator == SOL_DORMAND_PRINCE ? t.h_did : t.h_next;
  std::swap(bd->y0, bd->y);
  return 0;
}

int attempt(int integrator, double epsilon, BodyData* bd, Acceleration* acc) {
  const bool bary = barycentric_of(acc);
  sol_ctx* c = context(acc, bary);
  if (!c) return 1;
  if (sol_set_tolerance(c, epsilon) != SOL_OK || sol_set_eval_flags(c, flags_of(acc)) != SOL_OK) return 1;
  double em = 0.0;
  if (sol_integrator_attempt(c, integrator, bd->time, bd->h, bd->y0, bd->accel, nullptr, bd->y,
                             integrator != SOL_RUNGE_KUTTA4 ? bd->error : nullptr, &em) != SOL_OK)
    return 1;
  return read_back(acc, c, bary);
}

double error_max(int integrator, int n, const double* yerr, const double* yscale, double epsilon) {
  double out = std::numeric_limits<double>::quiet_NaN();
  if (sol_error_max(nullptr, integrator, n, yerr, yscale, epsilon, &out) != SOL_OK) fail(__FILE__, __func__, __LINE__);
  return out;
}

}  // namespace solgb_facade
