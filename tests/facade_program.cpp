// Drives the C++ class facade the way the reference's Simulator drives its
// classes (BodyData + Nebula + Acceleration + an integrator + TimeLine) and
// dumps everything the calls leave behind, for tests/test_gpu_facade.py.
//
//   facade_program <input.bin> <output.bin>
//
// Input (little-endian): int32 counts[7], integrator, n_steps, has_gas,
// remove_body (index to remove after the first n_steps, -1 = none), n_steps2;
// sol_gas_component (raw); double t0, h0; per body int32 id, type, migType;
// double migStopAt, mass, radius, density, cD, gammaStokes, gammaEpstein;
// double y0[6N].
// Output: records (int32 name length, name, int32 kind 0 = f64 / 1 = i32,
// int64 count, data).
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "Acceleration.h"
#include "BodyData.h"
#include "DormandPrince.h"
#include "Error.h"
#include "Nebula.h"
#include "RungeKutta4.h"
#include "RungeKuttaFehlberg78.h"
#include "TimeLine.h"
#include "solaris_gb300.h"

namespace {

FILE* g_out = nullptr;

void put(const std::string& name, const double* p, int64_t n) {
  int32_t len = (int32_t)name.size(), kind = 0;
  std::fwrite(&len, 4, 1, g_out);
  std::fwrite(name.data(), 1, len, g_out);
  std::fwrite(&kind, 4, 1, g_out);
  std::fwrite(&n, 8, 1, g_out);
  std::fwrite(p, 8, (size_t)n, g_out);
}

void put(const std::string& name, const int* p, int64_t n) {
  int32_t len = (int32_t)name.size(), kind = 1;
  std::fwrite(&len, 4, 1, g_out);
  std::fwrite(name.data(), 1, len, g_out);
  std::fwrite(&kind, 4, 1, g_out);
  std::fwrite(&n, 8, 1, g_out);
  std::fwrite(p, 4, (size_t)n, g_out);
}

void put_status(const std::string& name, int rc) {
  put(name, &rc, 1);
  if (rc != 0) {
    const std::vector<double> msg(Error::_errMsg.begin(), Error::_errMsg.end());
    put(name + "_msg", msg.data(), (int64_t)msg.size());
  }
}

template <class T>
bool get(FILE* f, T* p, size_t n) {
  return std::fread(p, sizeof(T), n, f) == n;
}

void fill_counts(NBodies& nb, const int32_t c[7]) {
  nb.centralBody = c[0];
  nb.giantPlanet = c[1];
  nb.rockyPlanet = c[2];
  nb.protoPlanet = c[3];
  nb.superPlanetsimal = c[4];
  nb.planetsimal = c[5];
  nb.testParticle = c[6];
  nb.total = c[0] + c[1] + c[2] + c[3] + c[4] + c[5] + c[6];
}

int class_index(int type) { return type - 1; }  // BodyType CentralBody = 1 ... TestParticle = 7

// Simulator::RemoveBody-style compaction (Simulator.cpp:737-771): shift the
// arrays over body k and decrement its class count.
void remove_body(BodyData& bd, int k) {
  const int n = bd.nBodies.total;
  int* ints[] = {bd.id, bd.type, bd.migType, bd.indexOfNN};
  double* dbls[] = {bd.migStopAt, bd.distanceOfNN, bd.mass,        bd.radius,
                    bd.density,   bd.cD,           bd.gammaStokes, bd.gammaEpstein};
  const int type = bd.type[k];
  for (int* a : ints) std::memmove(a + k, a + k + 1, sizeof(int) * (n - k - 1));
  for (double* a : dbls) std::memmove(a + k, a + k + 1, sizeof(double) * (n - k - 1));
  std::memmove(bd.y0 + 6 * k, bd.y0 + 6 * (k + 1), sizeof(double) * 6 * (n - k - 1));
  int* counts[] = {&bd.nBodies.centralBody,      &bd.nBodies.giantPlanet, &bd.nBodies.rockyPlanet,
                   &bd.nBodies.protoPlanet,      &bd.nBodies.superPlanetsimal, &bd.nBodies.planetsimal,
                   &bd.nBodies.testParticle};
  --*counts[class_index(type)];
  --bd.nBodies.total;
}

template <class Integrator>
int run_steps(Integrator& in, BodyData& bd, Acceleration& acc, TimeLine& tl, int n, const std::string& tag) {
  std::vector<double> times, hdid, hnext;
  int rc = 0;
  for (int s = 0; s < n && rc == 0; ++s) {
    rc = in.Driver(&bd, &acc, &tl);
    times.push_back(tl.time);
    hdid.push_back(tl.hDid);
    hnext.push_back(tl.hNext);
  }
  put_status(tag + "_status", rc);
  put(tag + "_time", times.data(), (int64_t)times.size());
  put(tag + "_h_did", hdid.data(), (int64_t)hdid.size());
  put(tag + "_h_next", hnext.data(), (int64_t)hnext.size());
  const int N = bd.nBodies.total;
  put(tag + "_y0", bd.y0, 6 * N);
  put(tag + "_y", bd.y, 6 * N);
  put(tag + "_accel", bd.accel, 6 * N);
  put(tag + "_yscale", bd.yscale, 6 * N);
  put(tag + "_error", bd.error, 6 * N);
  put(tag + "_rm3", acc.rm3, N);
  put(tag + "_nn_idx", bd.indexOfNN, N);
  put(tag + "_nn_dist", bd.distanceOfNN, N);
  put(tag + "_mig_type", bd.migType, N);
  double bh[2] = {bd.time, bd.h};
  put(tag + "_bd_time_h", bh, 2);
  int flags[3] = {acc.evaluateGasDrag, acc.evaluateTypeIMigration, acc.evaluateTypeIIMigration};
  put(tag + "_flags", flags, 3);
  return rc;
}

template <class Integrator>
void run(Integrator& in, BodyData& bd, Acceleration& acc, TimeLine& tl, int n1, int remove, int n2) {
  if (run_steps(in, bd, acc, tl, n1, "drv") != 0) return;
  if (remove >= 0) {
    remove_body(bd, remove);
    run_steps(in, bd, acc, tl, n2, "drv2");
  }
}

}  // namespace

int main(int argc, char** argv) {
  if (argc != 3) {
    std::fprintf(stderr, "usage: facade_program <input.bin> <output.bin>\n");
    return 2;
  }
  FILE* fi = std::fopen(argv[1], "rb");
  g_out = std::fopen(argv[2], "wb");
  if (!fi || !g_out) return 2;
  int32_t counts[7], hdr[5];
  sol_gas_component gas;
  double th[2];
  if (!get(fi, counts, 7) || !get(fi, hdr, 5) || !get(fi, &gas, 1) || !get(fi, th, 2)) return 2;
  const int integrator = hdr[0], n_steps = hdr[1], has_gas = hdr[2], remove = hdr[3], n_steps2 = hdr[4];

  BodyData bd;
  fill_counts(bd.nBodies, counts);
  if (bd.Allocate() != 0) return 3;
  const int N = bd.nBodies.total;
  bool ok = get(fi, bd.id, N) && get(fi, bd.type, N) && get(fi, bd.migType, N) && get(fi, bd.migStopAt, N) &&
            get(fi, bd.mass, N) && get(fi, bd.radius, N) && get(fi, bd.density, N) && get(fi, bd.cD, N) &&
            get(fi, bd.gammaStokes, N) && get(fi, bd.gammaEpstein, N) && get(fi, bd.y0, 6 * N);
  std::fclose(fi);
  if (!ok) return 2;

  Nebula nebula;
  if (has_gas) {
    GasComponent& g = nebula.gasComponent;
    g.alpha = gas.alpha;
    g.type = (GasDecreaseType)gas.decrease_type;
    g.timeScale = gas.time_scale;
    g.t0 = gas.t0;
    g.t1 = gas.t1;
    g.innerEdge = gas.inner_edge;
    g.meanMolecularWeight = gas.mean_molecular_weight;
    g.particleDiameter = gas.particle_diameter;
    g.eta = PowerLaw(gas.eta.c, gas.eta.index);
    g.tau = PowerLaw(gas.tau.c, gas.tau.index);
    g.scaleHeight = PowerLaw(gas.scale_height.c, gas.scale_height.index);
    g.density = PowerLaw(gas.density.c, gas.density.index);
    g.meanFreePath = PowerLaw(gas.mean_free_path.c, gas.mean_free_path.index);
  }
  Acceleration acc((IntegratorType)integrator, false, &bd, has_gas ? &nebula : nullptr);

  // Compute at the initial state, as a driver's first evaluation does
  std::vector<double> dydt(6 * (size_t)N);
  put_status("compute_status", acc.Compute(th[0], bd.y0, dydt.data()));
  put("compute_dydt", dydt.data(), 6 * N);
  put("compute_rm3", acc.rm3, N);
  put("compute_nn_idx", bd.indexOfNN, N);
  put("compute_nn_dist", bd.distanceOfNN, N);
  put("compute_mig_type", bd.migType, N);
  if (acc.accelGasDrag) put("compute_drag", acc.accelGasDrag, 3 * bd.nBodies.NOfPlAndSpl());

  // the individual terms
  std::vector<double> grav(6 * (size_t)N);
  put_status("gravity_status", acc.GravityAC(th[0], bd.y0, grav.data()));
  put("gravity", grav.data(), 6 * N);
  if (has_gas && bd.nBodies.NOfPlAndSpl() > 0) {
    std::vector<double> drag(3 * (size_t)bd.nBodies.NOfPlAndSpl());
    put_status("drag_status", acc.GasDragAC(th[0], bd.y0, drag.data()));
    put("drag", drag.data(), (int64_t)drag.size());
  }

  // single attempts from BodyData's y0 / accel, with the Driver's flags
  RungeKuttaFehlberg78 rkf;
  bd.time = th[0];
  bd.h = th[1];
  std::memcpy(bd.accel, dydt.data(), sizeof(double) * 6 * N);
  acc.evaluateTypeIMigration = false;
  acc.evaluateTypeIIMigration = false;
  put_status("step_status", rkf.Step(&bd, &acc));
  put("step_y", bd.y, 6 * N);
  put("step_error", bd.error, 6 * N);
  // GetErrorMax of the attempt's error against the Driver's yscale
  std::vector<double> yscale(6 * (size_t)N);
  for (int i = 0; i < 6 * N; ++i) yscale[i] = std::fabs(bd.y0[i]) + std::fabs(th[1] * dydt[i]) + 1.0e-30;
  double em = rkf.GetErrorMax(6 * N, bd.error, yscale.data());
  put("step_error_max", &em, 1);
  DormandPrince dp;
  double em_dp = dp.GetErrorMax(6 * N, bd.error);
  put("dp_error_max", &em_dp, 1);

  TimeLine tl;
  tl.time = th[0];
  tl.hNext = th[1];
  if (integrator == RUNGE_KUTTA_FEHLBERG78) {
    run(rkf, bd, acc, tl, n_steps, remove, n_steps2);
  } else if (integrator == RUNGE_KUTTA4) {
    RungeKutta4 rk4;
    run(rk4, bd, acc, tl, n_steps, remove, n_steps2);
  } else {
    run(dp, bd, acc, tl, n_steps, remove, n_steps2);
  }
  std::fclose(g_out);
  return 0;
}
