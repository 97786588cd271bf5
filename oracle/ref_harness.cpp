// Test infrastructure only: a direct-call driver for the reference Solaris CPU
// classes, linked against objects compiled from the reference's own sources
// (recipe: oracle/Makefile).  It never ships with the library and is never
// timed as the product.  It reads one case file, calls the reference's
// Acceleration / RungeKuttaFehlberg78 / RungeKutta4 / DormandPrince /
// Calculate / Ephemeris code exactly as Simulator::Integrate does
// (Solaris/Simulator.cpp:121-178), and writes named arrays to an output file.
//
// Case file (little endian):
//   i32 magic 'SOL1', i32 cmd, i32 counts[7] (central, giant, rocky, proto,
//   super-planetesimal, planetesimal, test particle), i32 barycentric,
//   i32 has_nebula, f64 nebula[16], f64 t, f64 h, i32 nsteps, i32 flags,
//   i32 id[N], i32 type[N], i32 migType[N], f64 migStopAt[N], f64 mass[N],
//   f64 radius[N], f64 density[N], f64 cD[N], f64 gammaStokes[N],
//   f64 gammaEpstein[N], f64 y0[6N], i32 n_extra, f64 extra[n_extra].
// Output file: repeated records {i32 name_len, name, i32 kind (0 f64, 1 i32),
//   i64 count, payload}.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cstdint>
#include <string>
#include <vector>

#include "Acceleration.h"
#include "BodyData.h"
#include "Calculate.h"
#include "Constants.h"
#include "DormandPrince.h"
#include "Ephemeris.h"
#include "IntegratorType.h"
#include "Nebula.h"
#include "OrbitalElement.h"
#include "Phase.h"
#include "RungeKutta4.h"
#include "RungeKuttaFehlberg78.h"
#include "TimeLine.h"

enum Cmd {
  CMD_ACCEL = 1, CMD_RKF78_STEP = 2, CMD_RKF78_DRIVER = 3, CMD_RK4_DRIVER = 4,
  CMD_DP_DRIVER = 5, CMD_INTEGRALS = 6, CMD_EPHEMERIS = 7, CMD_KEPLER = 8,
  CMD_TIME_ACCEL = 9, CMD_ORBITAL_ELEMENT = 10
};

static FILE* g_out = 0;

static void put(const char* name, int kind, const void* data, int64_t count) {
  int32_t len = (int32_t)strlen(name);
  fwrite(&len, 4, 1, g_out);
  fwrite(name, 1, len, g_out);
  int32_t k = kind;
  fwrite(&k, 4, 1, g_out);
  fwrite(&count, 8, 1, g_out);
  fwrite(data, kind == 0 ? 8 : 4, (size_t)count, g_out);
}
static void put_d(const char* name, const double* d, int64_t n) { put(name, 0, d, n); }
static void put_i(const char* name, const int* d, int64_t n) { put(name, 1, d, n); }

template <class T> static void rd(FILE* f, T* dst, size_t n) {
  if (fread(dst, sizeof(T), n, f) != n) { fprintf(stderr, "short read\n"); exit(2); }
}

int main(int argc, char** argv) {
  if (argc != 3) { fprintf(stderr, "usage: ref_harness <case> <out>\n"); return 2; }
  FILE* f = fopen(argv[1], "rb");
  if (!f) { perror("case"); return 2; }
  int32_t magic, cmd, counts[7], bary, has_neb, nsteps, flags;
  double neb[16], t, h;
  rd(f, &magic, 1); rd(f, &cmd, 1);
  if (magic != 0x534F4C31) { fprintf(stderr, "bad magic\n"); return 2; }
  rd(f, counts, 7); rd(f, &bary, 1); rd(f, &has_neb, 1); rd(f, neb, 16);
  rd(f, &t, 1); rd(f, &h, 1); rd(f, &nsteps, 1); rd(f, &flags, 1);

  BodyData bd;
  bd.nBodies.centralBody = counts[0]; bd.nBodies.giantPlanet = counts[1];
  bd.nBodies.rockyPlanet = counts[2]; bd.nBodies.protoPlanet = counts[3];
  bd.nBodies.superPlanetsimal = counts[4]; bd.nBodies.planetsimal = counts[5];
  bd.nBodies.testParticle = counts[6];
  int N = 0; for (int k = 0; k < 7; ++k) N += counts[k];
  bd.nBodies.total = N;
  if (bd.Allocate() != 0) return 3;
  rd(f, bd.id, N); rd(f, bd.type, N); rd(f, bd.migType, N);
  rd(f, bd.migStopAt, N); rd(f, bd.mass, N); rd(f, bd.radius, N); rd(f, bd.density, N);
  rd(f, bd.cD, N); rd(f, bd.gammaStokes, N); rd(f, bd.gammaEpstein, N);
  rd(f, bd.y0, 6 * N);
  int32_t n_extra = 0; rd(f, &n_extra, 1);
  std::vector<double> extra(n_extra > 0 ? n_extra : 1);
  if (n_extra > 0) rd(f, extra.data(), n_extra);
  fclose(f);
  memset(bd.y, 0, sizeof(double) * 6 * N);
  memset(bd.accel, 0, sizeof(double) * 6 * N);
  memset(bd.error, 0, sizeof(double) * 6 * N);
  memset(bd.yscale, 0, sizeof(double) * 6 * N);

  Nebula* nebula = 0;
  if (has_neb) {
    nebula = new Nebula();
    GasComponent& g = nebula->gasComponent;
    g.alpha = neb[0];
    g.type = (GasDecreaseType)(int)neb[1];
    g.timeScale = neb[2]; g.t0 = neb[3]; g.t1 = neb[4];
    g.eta = PowerLaw(neb[5], neb[6]);
    g.tau = PowerLaw(neb[7], neb[8]);
    g.scaleHeight = PowerLaw(neb[9], neb[10]);
    g.density = PowerLaw(neb[11], neb[12]);
    // meanFreePath, innerEdge and a keep their constructor values, as the
    // XML reader leaves them (Solaris/GasComponent.cpp:9-33).
  }

  g_out = fopen(argv[2], "wb");
  if (!g_out) { perror("out"); return 2; }

  IntegratorType itype = RUNGE_KUTTA_FEHLBERG78;
  if (cmd == CMD_RK4_DRIVER) itype = RUNGE_KUTTA4;
  if (cmd == CMD_DP_DRIVER) itype = DORMAND_PRINCE;
  Acceleration acc(itype, bary != 0, &bd, nebula);

  if (cmd == CMD_ACCEL) {
    acc.evaluateGasDrag = (flags & 1) != 0;
    acc.evaluateTypeIMigration = (flags & 2) != 0;
    acc.evaluateTypeIIMigration = (flags & 4) != 0;
    int r = acc.Compute(t, bd.y0, bd.accel);
    put_i("status", &r, 1);
    put_d("dydt", bd.accel, 6 * N);
    if (!bary) put_d("rm3", acc.rm3, N);
    put_i("nn_idx", bd.indexOfNN, N);
    put_d("nn_dist", bd.distanceOfNN, N);
    put_i("mig_type", bd.migType, N);
  } else if (cmd == CMD_TIME_ACCEL) {
    // Wall time of nsteps Compute calls (CPU baseline timing in this container).
    acc.evaluateGasDrag = (flags & 1) != 0;
    acc.evaluateTypeIMigration = (flags & 2) != 0;
    acc.evaluateTypeIIMigration = (flags & 4) != 0;
    struct timespec a, b;
    clock_gettime(CLOCK_MONOTONIC, &a);
    for (int s = 0; s < nsteps; ++s) acc.Compute(t, bd.y0, bd.accel);
    clock_gettime(CLOCK_MONOTONIC, &b);
    double sec = (b.tv_sec - a.tv_sec) + 1e-9 * (b.tv_nsec - a.tv_nsec);
    put_d("seconds", &sec, 1);
    put_d("dydt", bd.accel, 6 * N);
  } else if (cmd == CMD_RKF78_STEP) {
    // One attempt at fixed h, with the flag protocol of RungeKuttaFehlberg78::Driver
    // (Solaris/RungeKuttaFehlberg78.cpp:74-95) and its yscale (:87-89).
    RungeKuttaFehlberg78 rk;
    bd.time = t; bd.h = h;
    acc.evaluateGasDrag = true; acc.evaluateTypeIMigration = true; acc.evaluateTypeIIMigration = true;
    acc.Compute(t, bd.y0, bd.accel);
    for (int i = 0; i < 6 * N; ++i) bd.yscale[i] = fabs(bd.y0[i]) + fabs(bd.h * bd.accel[i]) + 1.0e-30;
    acc.evaluateTypeIMigration = false; acc.evaluateTypeIIMigration = false;
    int r = rk.Step(&bd, &acc);
    double em = rk.GetErrorMax(6 * N, bd.error, bd.yscale);
    put_i("status", &r, 1);
    put_d("f0", bd.accel, 6 * N);
    put_d("y", bd.y, 6 * N);
    put_d("error", bd.error, 6 * N);
    put_d("yscale", bd.yscale, 6 * N);
    put_d("error_max", &em, 1);
    if (!bary) put_d("rm3", acc.rm3, N);
    put_i("nn_idx", bd.indexOfNN, N);
    put_d("nn_dist", bd.distanceOfNN, N);
  } else if (cmd == CMD_RKF78_DRIVER || cmd == CMD_RK4_DRIVER || cmd == CMD_DP_DRIVER) {
    TimeLine tl;
    tl.time = t; tl.hNext = h; tl.hDid = 0.0;
    RungeKuttaFehlberg78 rkf; RungeKutta4 rk4; DormandPrince dp;
    std::vector<double> times, hdid, hnext, traj;
    int status = 0;
    for (int s = 0; s < nsteps; ++s) {
      int r;
      if (cmd == CMD_RKF78_DRIVER) r = rkf.Driver(&bd, &acc, &tl);
      else if (cmd == CMD_RK4_DRIVER) r = rk4.Driver(&bd, &acc, &tl);
      else r = dp.Driver(&bd, &acc, &tl);
      if (r != 0) { status = r; break; }
      times.push_back(tl.time); hdid.push_back(tl.hDid); hnext.push_back(tl.hNext);
      if (flags & 8) traj.insert(traj.end(), bd.y0, bd.y0 + 6 * N);
    }
    put_i("status", &status, 1);
    int ns = (int)times.size();
    put_i("n_steps", &ns, 1);
    put_d("time", times.data(), ns);
    put_d("h_did", hdid.data(), ns);
    put_d("h_next", hnext.data(), ns);
    put_d("y0", bd.y0, 6 * N);
    if (flags & 8) put_d("trajectory", traj.data(), (int64_t)traj.size());
    if (!bary) put_d("rm3", acc.rm3, N);
    put_i("nn_idx", bd.indexOfNN, N);
    put_d("nn_dist", bd.distanceOfNN, N);
    put_i("mig_type", bd.migType, N);
  } else if (cmd == CMD_INTEGRALS) {
    Calculate::Integrals(&bd);
    put_d("integrals", bd.integrals, 16);
  } else if (cmd == CMD_EPHEMERIS) {
    // extra = M records of {mu, a, e, i, peri, node, M}
    int M = n_extra / 7;
    std::vector<double> ph(6 * M);
    std::vector<int> st(M);
    for (int k = 0; k < M; ++k) {
      const double* x = &extra[7 * k];
      OrbitalElement oe;
      oe.semiMajorAxis = x[1]; oe.eccentricity = x[2]; oe.inclination = x[3];
      oe.argumentOfPericenter = x[4]; oe.longitudeOfNode = x[5]; oe.meanAnomaly = x[6];
      Phase p;
      st[k] = Ephemeris::CalculatePhase(x[0], &oe, &p);
      ph[6 * k + 0] = p.position.x; ph[6 * k + 1] = p.position.y; ph[6 * k + 2] = p.position.z;
      ph[6 * k + 3] = p.velocity.x; ph[6 * k + 4] = p.velocity.y; ph[6 * k + 5] = p.velocity.z;
    }
    put_i("status", st.data(), M);
    put_d("phase", ph.data(), 6 * M);
  } else if (cmd == CMD_ORBITAL_ELEMENT) {
    // extra = M records of {mu, x, y, z, vx, vy, vz} -> {a, e}
    int M = n_extra / 7;
    std::vector<double> ae(2 * M);
    std::vector<int> st(M);
    for (int k = 0; k < M; ++k) {
      const double* x = &extra[7 * k];
      Phase p;
      p.position = Vector(x[1], x[2], x[3]);
      p.velocity = Vector(x[4], x[5], x[6]);
      double a = 0, e = 0;
      st[k] = Ephemeris::CalculateOrbitalElement(x[0], &p, &a, &e);
      ae[2 * k] = a; ae[2 * k + 1] = e;
    }
    put_i("status", st.data(), M);
    put_d("a_e", ae.data(), 2 * M);
  } else if (cmd == CMD_KEPLER) {
    int M = n_extra / 2;
    std::vector<double> E(M);
    std::vector<int> st(M);
    for (int k = 0; k < M; ++k) st[k] = Ephemeris::KeplerEquationSolver(extra[2 * k], extra[2 * k + 1], 1.0e-14, E[k]);
    put_i("status", st.data(), M);
    put_d("E", E.data(), M);
  } else {
    fprintf(stderr, "unknown cmd %d\n", cmd);
    return 2;
  }
  fclose(g_out);
  return 0;
}
