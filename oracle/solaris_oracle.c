/*
 * solaris_oracle.c - CPU restatement of the Solaris force-and-integrate path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker): used by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg.  The GB300
 * library never links or calls it.
 *
 * Every function restates the reference function cited beside it, keeping
 * its operation order so that, built with -ffp-contract=off, it reproduces
 * the reference g++ build bit for bit (pinned by tests/test_oracle_golden.py
 * against fixtures made by the reference itself).  File references are
 * relative to the reference project root.
 */
#include "solaris_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ---- constants: Solaris/Constants.h:29-99 ------------------------------ */
#define K_GAUSS 1.720209895e-2
#define K_GAUSS2 2.959122082855911025e-4
#define K_PI 3.14159265358979323846
#define K_SQRT_TWO_PI 2.50662827463100024161
static const double K_SOLAR_TO_KILOGRAM = 1.98911e30;
static const double K_AU_TO_METER = 1.495978707e11;
static const double K_AU_TO_SOLAR_RADIUS = 215.094;
static const double K_DAY_TO_SECOND = 86400.0;
static const double K_BOLTZMAN_SI = 1.3806488e-23;
static const double K_PROTON_MASS_SI = 1.672621777e-27;

static double c_kilogram_to_solar(void) { return 1.0 / K_SOLAR_TO_KILOGRAM; }
static double c_meter_to_au(void) { return 1.0 / K_AU_TO_METER; }
static double c_gram_to_solar(void) { return 1.0 / (1.0e3 * K_SOLAR_TO_KILOGRAM); }
static double c_gram_per_cm3_to_solar_per_au3(void) {
  double l = 1.0e-2 * c_meter_to_au();
  return c_gram_to_solar() / (l * l * l);
}
static double c_proton_mass_cmu(void) { return K_PROTON_MASS_SI * c_kilogram_to_solar(); }
static double c_boltzman_cmu(void) {
  double m2au = c_meter_to_au();
  double s2d = 1.0 / K_DAY_TO_SECOND;
  return K_BOLTZMAN_SI * (c_kilogram_to_solar() * (m2au * m2au)) / (s2d * s2d);
}
static double c_proton_mass_boltzman_cmu(void) { return 1.0 / (c_boltzman_cmu() / c_proton_mass_cmu()); }

#define SQR(a) ((a) * (a))

struct orc_system {
  sol_nbodies n;
  int32_t total;
  int32_t barycentric;
  int32_t has_gas;
  sol_gas_component gas;
  /* body parameters (copies; mig_type is mutated by migration) */
  int32_t *id, *type, *mig_type;
  double *mig_stop_at, *mass, *radius, *density, *cd, *gamma_stokes, *gamma_epstein;
  /* Acceleration state (Solaris/Acceleration.h:364-377) */
  double* rm3;
  double *acc_drag, *acc_mig1, *acc_mig2;
  int32_t n_drag, n_mig1, n_mig2;
  int eval_drag, eval_mig1, eval_mig2;
  int32_t* nn_idx;
  double* nn_dist;
  /* function-local statics of GasComponent (GasComponent.cpp:223-241) */
  int thermal_init;
  double cvth, ctp, pt;
  double epsilon;
  /* integrator scratch */
  double *accel, *yscale, *error, *ytmp, *ybuf, *fk[13];
  /* host threads of the sink loops of GravityAC and of orc_jvp (default 1;
   * every sink's sum stays sequential, so the results do not depend on it) */
  int n_threads;
};

static int n_massive(const orc_system* s) {
  return s->n.central_body + s->n.giant_planet + s->n.rocky_planet + s->n.proto_planet;
}
static int n_pl_and_spl(const orc_system* s) { return s->n.super_planetesimal + s->n.planetesimal; }

static double* dup_d(const double* src, int n, double fill) {
  double* d = (double*)malloc(sizeof(double) * (n > 0 ? n : 1));
  for (int i = 0; i < n; ++i) d[i] = src ? src[i] : fill;
  return d;
}
static int32_t* dup_i(const int32_t* src, int n, int32_t fill) {
  int32_t* d = (int32_t*)malloc(sizeof(int32_t) * (n > 0 ? n : 1));
  for (int i = 0; i < n; ++i) d[i] = src ? src[i] : fill;
  return d;
}

orc_system* orc_create(const sol_body_data* b, const sol_gas_component* gas, int32_t barycentric) {
  orc_system* s = (orc_system*)calloc(1, sizeof(orc_system));
  s->n_threads = 1;
  s->n = b->n;
  s->total = b->n.central_body + b->n.giant_planet + b->n.rocky_planet + b->n.proto_planet +
             b->n.super_planetesimal + b->n.planetesimal + b->n.test_particle;
  int N = s->total;
  s->barycentric = barycentric;
  s->has_gas = gas != NULL;
  if (gas) s->gas = *gas;
  s->id = dup_i(b->id, N, 0);
  s->type = dup_i(b->type, N, 0);
  s->mig_type = dup_i(b->mig_type, N, 0);
  s->mig_stop_at = dup_d(b->mig_stop_at, N, 0.0);
  s->mass = dup_d(b->mass, N, 0.0);
  s->radius = dup_d(b->radius, N, 0.0);
  s->density = dup_d(b->density, N, 0.0);
  s->cd = dup_d(b->cd, N, 0.0);
  s->gamma_stokes = dup_d(b->gamma_stokes, N, 0.0);
  s->gamma_epstein = dup_d(b->gamma_epstein, N, 0.0);
  s->rm3 = NULL; /* allocated lazily and zeroed, Acceleration.cpp:65-69 */
  s->nn_idx = dup_i(NULL, N, -1);
  s->nn_dist = dup_d(NULL, N, 0.0);
  s->eval_drag = s->eval_mig1 = s->eval_mig2 = 1;
  s->epsilon = pow(10, -10.0); /* RungeKuttaFehlberg78.cpp:38-39 */
  int nv = 6 * N;
  s->accel = dup_d(NULL, nv, 0.0);
  s->yscale = dup_d(NULL, nv, 0.0);
  s->error = dup_d(NULL, nv, 0.0);
  s->ytmp = dup_d(NULL, nv, 0.0);
  s->ybuf = dup_d(NULL, nv, 0.0);
  for (int k = 0; k < 13; ++k) s->fk[k] = dup_d(NULL, nv, 0.0);
  return s;
}

void orc_destroy(orc_system* s) {
  if (!s) return;
  free(s->id); free(s->type); free(s->mig_type); free(s->mig_stop_at); free(s->mass);
  free(s->radius); free(s->density); free(s->cd); free(s->gamma_stokes); free(s->gamma_epstein);
  free(s->rm3); free(s->acc_drag); free(s->acc_mig1); free(s->acc_mig2);
  free(s->nn_idx); free(s->nn_dist);
  free(s->accel); free(s->yscale); free(s->error); free(s->ytmp); free(s->ybuf);
  for (int k = 0; k < 13; ++k) free(s->fk[k]);
  free(s);
}

int32_t orc_n_total(const orc_system* s) { return s->total; }

void orc_set_eval_flags(orc_system* s, uint32_t f) {
  s->eval_drag = (f & SOL_EVAL_GAS_DRAG) != 0;
  s->eval_mig1 = (f & SOL_EVAL_TYPE_I) != 0;
  s->eval_mig2 = (f & SOL_EVAL_TYPE_II) != 0;
}

void orc_set_epsilon(orc_system* s, double eps) { s->epsilon = eps; }

/* ---- GasComponent (Solaris/GasComponent.cpp) ---------------------------- */
static double power_law(const sol_power_law* p, double x) { return p->c * pow(x, p->index); } /* PowerLaw.cpp:17-20 */

static double reduction_factor(const sol_gas_component* g, double t) { /* GasComponent.cpp:36-61 */
  switch (g->decrease_type) {
    case SOL_GAS_CONSTANT: return 1.0;
    case SOL_GAS_LINEAR:
      if (t <= g->t0) return 1.0;
      else if (t > g->t0 && t <= g->t1) return 1.0 - (t - g->t0) / (g->t1 - g->t0);
      else return 0.0;
    case SOL_GAS_EXPONENTIAL: return exp(-t / g->time_scale);
    default: return 1.0;
  }
}

static double midplane_density(const sol_gas_component* g, double r) { /* GasComponent.cpp:63-69 */
  double a1 = power_law(&g->density, r);
  double a2 = power_law(&g->scale_height, r);
  return a1 * a2 * K_SQRT_TWO_PI;
}

static void circular_velocity(double mu, const double* rv, double* out) { /* GasComponent.cpp:97-126 */
  out[0] = out[1] = out[2] = 0.0;
  double r = sqrt(SQR(rv[0]) + SQR(rv[1]));
  double vc = sqrt(mu / r);
  double p;
  if (rv[0] == 0.0 && rv[1] == 0.0) {
    return;
  } else if (rv[1] == 0.0) {
    out[1] = rv[0] > 0.0 ? vc : -vc;
  } else if (rv[0] == 0.0) {
    out[0] = rv[1] > 0.0 ? -vc : vc;
  } else if (rv[0] >= rv[1]) {
    p = rv[1] / rv[0];
    out[1] = rv[0] >= 0 ? vc / sqrt(1.0 + SQR(p)) : -vc / sqrt(1.0 + SQR(p));
    out[0] = -out[1] * p;
  } else {
    p = rv[0] / rv[1];
    out[0] = rv[1] >= 0 ? -vc / sqrt(1.0 + SQR(p)) : vc / sqrt(1.0 + SQR(p));
    out[1] = -out[0] * p;
  }
}

static void gas_velocity(const sol_gas_component* g, double mu, const double* rv, double* out) { /* :128-138 */
  circular_velocity(mu, rv, out);
  double r = sqrt(SQR(rv[0]) + SQR(rv[1]));
  double v = sqrt(1.0 - 2.0 * power_law(&g->eta, r));
  out[0] *= v;
  out[1] *= v;
}

static double gas_density_at(const sol_gas_component* g, const double* rv) { /* :141-157 */
  double r = sqrt(SQR(rv[0]) + SQR(rv[1]));
  double h = power_law(&g->scale_height, r);
  double arg = SQR(rv[2] / h);
  if (g->inner_edge < r) {
    return power_law(&g->density, r) * exp(-arg);
  } else {
    double a = g->density.c * pow(g->inner_edge, g->density.index - 4.0);
    return a * SQR(SQR(r)) * exp(-arg);
  }
}

/* MeanThermalSpeed_CMU(mC, r) calls Temperature_CMU(r, mC) with the arguments
 * swapped (GasComponent.cpp:238-243, :221-229); both keep function-local
 * statics computed on the first call. */
static double mean_thermal_speed_cmu(orc_system* s, double mC, double r) {
  const sol_gas_component* g = &s->gas;
  if (!s->thermal_init) {
    s->cvth = sqrt((8.0 * c_boltzman_cmu()) / (K_PI * g->mean_molecular_weight * c_proton_mass_cmu()));
    s->ctp = K_GAUSS2 * c_proton_mass_boltzman_cmu();
    s->pt = 2.0 * g->scale_height.index - 3.0;
    s->thermal_init = 1;
  }
  /* Temperature_CMU(mC' = r, r' = mC) */
  double cT = SQR(g->scale_height.c) * r * g->mean_molecular_weight * s->ctp;
  double temperature = cT * pow(mC, s->pt);
  return s->cvth * sqrt(temperature);
}

/* ---- Ephemeris (Solaris/Ephemeris.cpp) ---------------------------------- */
/* The reference g++ build binds abs(double) to int abs(int) in this file. */
static double quirk_abs(double x, int32_t quirks) {
  if (quirks & SOL_QUIRK_INT_ABS) {
    int i = (int)x;
    return (double)(i < 0 ? -i : i);
  }
  return fabs(x);
}

int orc_calculate_orbital_element(double mu, const double ph[6], double* a, double* e, int32_t quirks) {
  /* Ephemeris::CalculateOrbitalElement(mu, phase, &a, &e), Ephemeris.cpp:10-41 */
  const double sq3 = 1.0e-14;
  double v2 = ph[3] * ph[3] + ph[4] * ph[4] + ph[5] * ph[5];
  double rl = sqrt(ph[0] * ph[0] + ph[1] * ph[1] + ph[2] * ph[2]);
  double h = v2 / 2.0 + (-mu / rl);
  if (h >= 0.0) return 1;
  double cx = ph[1] * ph[5] - ph[2] * ph[4];
  double cy = ph[2] * ph[3] - ph[0] * ph[5];
  double cz = ph[0] * ph[4] - ph[1] * ph[3];
  double c2 = cx * cx + cy * cy + cz * cz;
  double e2 = 1.0 + 2.0 * c2 * h / (mu * mu);
  if (quirk_abs(e2, quirks) < sq3) e2 = 0.0;
  *e = sqrt(e2);
  *a = -mu / (2.0 * h);
  return 0;
}

int orc_kepler_equation_solver(double e, double m, double eps, double* E) {
  /* Ephemeris::KeplerEquationSolver, Ephemeris.cpp:187-211 (abs binds to the
   * int overload in the reference build, so the loop ends once |E1-E| < 1). */
  if (e == 0.0 || m == 0.0 || m == K_PI) {
    *E = m;
    return 0;
  }
  double EE = m + e * (sin(m)) / (1.0 - sin(m + e) + sin(m));
  double E1 = 0.0, error;
  int step = 0;
  do {
    E1 = EE - (EE - e * sin(EE) - m) / (1.0 - e * cos(EE));
    error = quirk_abs(E1 - EE, SOL_QUIRK_INT_ABS);
    EE = E1;
    step++;
  } while (error > eps && step <= 25);
  *E = EE;
  if (step > 25) return 1;
  return 0;
}

int orc_calculate_phase(double mu, const double el[6], double ph[6]) {
  /* Ephemeris::CalculatePhase, Ephemeris.cpp:141-176.  el = {a, e, i, peri, node, M} */
  double e = el[1];
  double E = 0;
  if (orc_kepler_equation_solver(e, el[5], 1.0e-14, &E) == 1) return 1;
  double v = 2.0 * atan(sqrt((1.0 + e) / (1.0 - e)) * tan(E / 2.0));
  double a = el[0];
  double p = a * (1.0 - e * e);
  double r = p / (1.0 + e * cos(v));
  double kszi = r * cos(v);
  double eta = r * sin(v);
  double vKszi = -sqrt(mu / p) * sin(v);
  double vEta = sqrt(mu / p) * (e + cos(v));
  double peri = el[3], node = el[4], incl = el[2];
  double cw = cos(peri), sw = sin(peri), cO = cos(node), sO = sin(node), ci = cos(incl), si = sin(incl);
  double P[3] = {cw * cO - sw * sO * ci, cw * sO + sw * cO * ci, sw * si};
  double Q[3] = {-sw * cO - cw * sO * ci, -sw * sO + cw * cO * ci, cw * si};
  for (int k = 0; k < 3; ++k) {
    ph[k] = kszi * P[k] + eta * Q[k];
    ph[3 + k] = vKszi * P[k] + vEta * Q[k];
  }
  return 0;
}

/* ---- Acceleration (Solaris/Acceleration.cpp) ---------------------------- */
static void gravity_ac_sink(orc_system* s, const double* y, double* accel, int i, int NOfMassive0) {
  /* body of the i loop of GravityAC, Acceleration.cpp:268-326 */
  double rMin = 1.0e10;
  double ax = 0.0, ay = 0.0, az = 0.0;
  double mu = K_GAUSS2 * (s->mass[0] + s->mass[i]);
  int i0 = 6 * i;
  accel[i0 + 0] = y[i0 + 3];
  accel[i0 + 1] = y[i0 + 4];
  accel[i0 + 2] = y[i0 + 5];
  accel[i0 + 3] = -mu * s->rm3[i] * y[i0 + 0];
  accel[i0 + 4] = -mu * s->rm3[i] * y[i0 + 1];
  accel[i0 + 5] = -mu * s->rm3[i] * y[i0 + 2];
  int NOfMassive = s->type[i] <= SOL_PROTO_PLANET ? NOfMassive0 + s->n.super_planetesimal : NOfMassive0;
  for (int j = 1; j < NOfMassive; j++) {
    if (j == i) continue;
    int j0 = 6 * j;
    double xij = y[j0 + 0] - y[i0 + 0];
    double yij = y[j0 + 1] - y[i0 + 1];
    double zij = y[j0 + 2] - y[i0 + 2];
    double rij2 = SQR(xij) + SQR(yij) + SQR(zij);
    double rij = sqrt(rij2);
    double rijm3 = 1.0 / (rij2 * rij);
    if (rij < rMin) {
      rMin = rij;
      s->nn_idx[i] = j;
      s->nn_dist[i] = rij;
    }
    double Gmj = K_GAUSS2 * s->mass[j];
    ax += Gmj * (xij * rijm3 - y[j0 + 0] * s->rm3[j]);
    ay += Gmj * (yij * rijm3 - y[j0 + 1] * s->rm3[j]);
    az += Gmj * (zij * rijm3 - y[j0 + 2] * s->rm3[j]);
  }
  accel[i0 + 3] += ax;
  accel[i0 + 4] += ay;
  accel[i0 + 5] += az;
}

static void gravity_ac_prepass(orc_system* s, const double* y) {
  /* Acceleration.cpp:253-264 */
  s->nn_idx[0] = -1;
  s->nn_dist[0] = 0.0;
  for (int i = 1; i < s->total; i++) {
    int i0 = 6 * i;
    double r2 = SQR(y[i0 + 0]) + SQR(y[i0 + 1]) + SQR(y[i0 + 2]);
    double r = sqrt(r2);
    s->rm3[i] = 1.0 / (r2 * r);
    s->nn_idx[i] = -1;
    s->nn_dist[i] = 0.0;
  }
}

static void gravity_ac(orc_system* s, const double* y, double* accel) {
  /* Acceleration::GravityAC, Acceleration.cpp:248-329 */
  gravity_ac_prepass(s, y);
  accel[0] = accel[1] = accel[2] = accel[3] = accel[4] = accel[5] = 0.0;
  int nm = n_massive(s);
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(s->n_threads) if (s->n_threads > 1)
#endif
  for (int i = 1; i < s->total; i++) gravity_ac_sink(s, y, accel, i, nm);
}

void orc_set_threads(orc_system* s, int32_t n_threads) { s->n_threads = n_threads > 1 ? n_threads : 1; }

static void gravity_bc_range(orc_system* s, const double* y, double* accel, int lo, int hi) {
  /* GravityBC_SelfInteracting / _NonSelfInteracting, Acceleration.cpp:541-634 */
  int nMassive = n_massive(s);
  for (int i = lo; i < hi; i++) {
    double rMin = 1.0e10;
    int i0 = 6 * i;
    s->nn_idx[i] = -1;
    s->nn_dist[i] = 0.0;
    accel[i0 + 0] = y[i0 + 3];
    accel[i0 + 1] = y[i0 + 4];
    accel[i0 + 2] = y[i0 + 5];
    accel[i0 + 3] = accel[i0 + 4] = accel[i0 + 5] = 0.0;
    for (int j = nMassive - 1; j >= 0; j--) {
      if (j == i) continue;
      int j0 = 6 * j;
      double dxij = y[j0 + 0] - y[i0 + 0];
      double dyij = y[j0 + 1] - y[i0 + 1];
      double dzij = y[j0 + 2] - y[i0 + 2];
      double rij2 = SQR(dxij) + SQR(dyij) + SQR(dzij);
      double rij = sqrt(rij2);
      if (rij < rMin) {
        rMin = rij;
        s->nn_idx[i] = j;
        s->nn_dist[i] = rij;
      }
      double c = s->mass[j] * 1.0 / (rij2 * rij);
      accel[i0 + 3] += c * dxij;
      accel[i0 + 4] += c * dyij;
      accel[i0 + 5] += c * dzij;
    }
    accel[i0 + 3] *= K_GAUSS2;
    accel[i0 + 4] *= K_GAUSS2;
    accel[i0 + 5] *= K_GAUSS2;
  }
}

static void gas_drag(orc_system* s, double t, const double* y, double* accel) {
  /* Acceleration::GasDragAC, Acceleration.cpp:331-422 (GasDragBC is the same, :639-642) */
  const sol_gas_component* g = &s->gas;
  double factor = reduction_factor(g, t);
  int lower = n_massive(s);
  int upper = lower + s->n.planetesimal + s->n.super_planetesimal;
  for (int i = lower; i < upper; i++) {
    int i0 = 6 * i;
    int j0 = 3 * (i - lower);
    double r = sqrt(SQR(y[i0 + 0]) + SQR(y[i0 + 1]) + SQR(y[i0 + 2]));
    double C = 0.0;
    double rv[3] = {y[i0 + 0], y[i0 + 1], y[i0 + 2]};
    double vg[3];
    gas_velocity(g, K_GAUSS2 * s->mass[0], rv, vg);
    double u[3] = {y[i0 + 3] - vg[0], y[i0 + 4] - vg[1], y[i0 + 5] - vg[2]};
    double rhoGas = factor * gas_density_at(g, rv);
    double lambda = power_law(&g->mean_free_path, r);
    if (s->radius[i] <= 0.1 * lambda) {
      double vth = mean_thermal_speed_cmu(s, s->mass[0], r);
      C = s->gamma_epstein[i] * vth * rhoGas;
    } else if (s->radius[i] >= 10.0 * lambda) {
      double uLength = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
      C = s->gamma_stokes[i] * uLength * rhoGas;
    } else {
      double lambda1 = 0.1 * lambda;
      double lambda2 = 10.0 * lambda;
      double gammaE = 1.0 / (s->density[i] * lambda1);
      double gammaS = 3.0 / 8.0 * s->cd[i] / (s->density[i] * lambda2);
      double vth = mean_thermal_speed_cmu(s, s->mass[0], r);
      double ulen = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
      double K = gammaS * ulen / (gammaE * vth);
      double eta = lambda2 / lambda1;
      double kappa = log10(K) / log10(eta);
      double gamma = gammaE * vth * pow(lambda1, -kappa);
      C = gamma * pow(s->radius[i], kappa) * rhoGas;
    }
    accel[j0 + 0] = -C * u[0];
    accel[j0 + 1] = -C * u[1];
    accel[j0 + 2] = -C * u[2];
  }
}

static void orbital_a_e(orc_system* s, const double* yi, double mc, double m, double* a, double* e) {
  double mu = K_GAUSS2 * (mc + m);
  *a = 0.0;
  *e = 0.0;
  /* the reference ignores the status (Acceleration.cpp:452) */
  orc_calculate_orbital_element(mu, yi, a, e, s->gas.quirks);
}

static void migration_type1(orc_system* s, double t, const double* y, double* accel) {
  /* Acceleration::MigrationTypeIAC, Acceleration.cpp:424-485 (BC: :645-713,
   * where TransformToAC is a no-op, Calculate.cpp:17-19) */
  const sol_gas_component* g = &s->gas;
  double factor = reduction_factor(g, t);
  int lower = s->n.central_body + s->n.giant_planet;
  int upper = n_massive(s);
  double absidx = quirk_abs(g->density.index, g->quirks);
  for (int i = lower; i < upper; i++) {
    if (s->mig_type[i] != SOL_MIGRATION_TYPE_I) continue;
    int i0 = 6 * i;
    int j0 = 3 * (i - lower);
    double r2 = SQR(y[i0 + 0]) + SQR(y[i0 + 1]) + SQR(y[i0 + 2]);
    double r = sqrt(r2);
    if (r <= s->mig_stop_at[i]) {
      accel[j0 + 0] = accel[j0 + 1] = accel[j0 + 2] = 0.0;
      s->mig_type[i] = SOL_MIGRATION_NO;
      continue;
    }
    double m = s->mass[i];
    double mc = s->mass[0];
    double a = 0.0, e = 0.0;
    orbital_a_e(s, &y[i0], mc, m, &a, &e);
    double O = K_GAUSS * sqrt((mc + m) / (a * a * a));
    double C = SQR(mc) / (m * midplane_density(g, r) * a * a);
    double h = power_law(&g->scale_height, r);
    double ar = h / r;
    double er = e * r;
    double tm = 0.0;
    if (e < 1.1 * h / r) {
      /* TypeIMigrationTime, :766-777 */
      double Cm = 2.0 / (2.7 + 1.1 * absidx) / O;
      double er1 = er / (1.3 * h);
      double er2 = er / (1.1 * h);
      double frac = (1.0 + er1 * er1 * er1 * er1 * er1) / (1.0 - er2 * er2 * er2 * er2);
      tm = Cm * C * SQR(ar) * frac;
      tm = 1.0 / tm;
    }
    /* TypeIEccentricityDampingTime, :779-789 */
    double Ce = 0.1 / (0.78 * O);
    double q = er / h;
    double fr = 1.0 + 0.25 * (q * q * q);
    double te = Ce * C * (ar * ar * ar * ar) * fr;
    double ti = te;
    double vr = y[i0 + 0] * y[i0 + 3] + y[i0 + 1] * y[i0 + 4] + y[i0 + 2] * y[i0 + 5];
    te = 2.0 * vr / (r2 * te);
    ti = 2.0 / ti;
    accel[j0 + 0] = -factor * (tm * y[i0 + 3] + te * y[i0 + 0]);
    accel[j0 + 1] = -factor * (tm * y[i0 + 4] + te * y[i0 + 1]);
    accel[j0 + 2] = -factor * (tm * y[i0 + 5] + te * y[i0 + 2] + ti * y[i0 + 5]);
  }
}

static double tau_nu(const sol_gas_component* g, double r, double O) { /* :831-849 */
  double index = g->tau.index;
  double c = g->tau.c;
  double h = power_law(&g->scale_height, r);
  if (index == 2) return c * SQR(r / h) / (g->alpha * O);
  return c * pow(r / h, index) / (g->alpha * O);
}

static void migration_type2(orc_system* s, double t, const double* y, double* accel) {
  /* Acceleration::MigrationTypeIIAC, Acceleration.cpp:487-528 (BC :716-764) */
  const sol_gas_component* g = &s->gas;
  double factor = reduction_factor(g, t);
  int lower = s->n.central_body;
  int upper = s->n.central_body + s->n.giant_planet;
  for (int i = lower; i < upper; i++) {
    if (s->mig_type[i] != SOL_MIGRATION_TYPE_II) continue;
    int i0 = 6 * i;
    int j0 = 3 * (i - lower);
    double r2 = SQR(y[i0 + 0]) + SQR(y[i0 + 1]) + SQR(y[i0 + 2]);
    double r = sqrt(r2);
    if (r <= s->mig_stop_at[i]) {
      s->mig_type[i] = SOL_MIGRATION_NO;
      accel[j0 + 0] = accel[j0 + 1] = accel[j0 + 2] = 0.0;
      continue;
    }
    double m = s->mass[i];
    double mc = s->mass[0];
    double a = 0.0, e = 0.0;
    orbital_a_e(s, &y[i0], mc, m, &a, &e);
    double O = K_GAUSS * sqrt((mc + m) / (a * a * a));
    double c0 = (s->barycentric && (g->quirks & SOL_QUIRK_BC_TAU_NU)) ? tau_nu(g, r, O) : 1.0 / tau_nu(g, r, O);
    double vr = y[i0 + 3] * y[i0 + 0] + y[i0 + 4] * y[i0 + 1] + y[i0 + 5] * y[i0 + 2];
    double c1 = vr / r2;
    accel[j0 + 0] = -factor * (c0 * (0.5 * y[i0 + 3] + 50 * (c1 * y[i0 + 0])));
    accel[j0 + 1] = -factor * (c0 * (0.5 * y[i0 + 4] + 50 * (c1 * y[i0 + 1])));
    accel[j0 + 2] = -factor * (c0 * (0.5 * y[i0 + 5] + 50 * (c1 * y[i0 + 2]) + y[i0 + 5]));
  }
}

int orc_compute(orc_system* s, double t, const double* y, double* dydt) {
  /* Acceleration::Compute + ComputeAstroCentric / ComputeBaryCentric,
   * Acceleration.cpp:60-246 */
  int N = s->total;
  if (!s->rm3) s->rm3 = dup_d(NULL, N, 0.0);
  if (s->barycentric) {
    int nm = n_massive(s);
    gravity_bc_range(s, y, dydt, 0, nm);
    gravity_bc_range(s, y, dydt, nm, N);
  } else {
    gravity_ac(s, y, dydt);
  }
  if (!s->has_gas) return 0;
  int npl = n_pl_and_spl(s);
  if (!s->acc_drag && npl > 0) { s->acc_drag = dup_d(NULL, 3 * npl, 0.0); s->n_drag = npl; }
  if (s->eval_drag && s->acc_drag) gas_drag(s, t, y, s->acc_drag);
  int lower = n_massive(s);
  for (int i = lower; i < lower + npl; i++) {
    int i0 = 6 * i, j0 = 3 * (i - lower);
    dydt[i0 + 3] += s->acc_drag[j0 + 0];
    dydt[i0 + 4] += s->acc_drag[j0 + 1];
    dydt[i0 + 5] += s->acc_drag[j0 + 2];
  }
  /* The reference sizes this buffer by protoPlanet only but indexes it over
   * rocky + proto bodies; it is sized for both here. */
  int nrp = s->n.rocky_planet + s->n.proto_planet;
  if (!s->acc_mig1 && s->n.proto_planet > 0) { s->acc_mig1 = dup_d(NULL, 3 * nrp, 0.0); s->n_mig1 = nrp; }
  if (s->eval_mig1 && s->acc_mig1) migration_type1(s, t, y, s->acc_mig1);
  lower = s->n.central_body + s->n.giant_planet;
  for (int i = lower; i < n_massive(s); i++) {
    if (s->mig_type[i] == SOL_MIGRATION_NO || !s->acc_mig1) continue;
    int i0 = 6 * i, j0 = 3 * (i - lower);
    dydt[i0 + 3] += s->acc_mig1[j0 + 0];
    dydt[i0 + 4] += s->acc_mig1[j0 + 1];
    dydt[i0 + 5] += s->acc_mig1[j0 + 2];
  }
  if (!s->acc_mig2 && s->n.giant_planet > 0) { s->acc_mig2 = dup_d(NULL, 3 * s->n.giant_planet, 0.0); s->n_mig2 = s->n.giant_planet; }
  if (s->eval_mig2 && s->acc_mig2) migration_type2(s, t, y, s->acc_mig2);
  lower = s->n.central_body;
  for (int i = lower; i < s->n.central_body + s->n.giant_planet; i++) {
    if (s->mig_type[i] == SOL_MIGRATION_NO) continue;
    int i0 = 6 * i, j0 = 3 * (i - lower);
    dydt[i0 + 3] += s->acc_mig2[j0 + 0];
    dydt[i0 + 4] += s->acc_mig2[j0 + 1];
    dydt[i0 + 5] += s->acc_mig2[j0 + 2];
  }
  return 0;
}

void orc_get_last_eval(const orc_system* s, double* rm3, int32_t* nn_idx, double* nn_dist) {
  int N = s->total;
  for (int i = 0; i < N; ++i) {
    if (rm3) rm3[i] = s->rm3 ? s->rm3[i] : 0.0;
    if (nn_idx) nn_idx[i] = s->nn_idx[i];
    if (nn_dist) nn_dist[i] = s->nn_dist[i];
  }
}

void orc_get_mig_type(const orc_system* s, int32_t* mt) { memcpy(mt, s->mig_type, sizeof(int32_t) * s->total); }

/* ---- RungeKuttaFehlberg78 (Solaris/RungeKuttaFehlberg78.cpp) ------------ */
/* Coefficients, :41-56 */
static const double D1_0 = 41.0 / 840.0, D1_5 = 34.0 / 105.0, D1_6 = 9.0 / 35.0, D1_8 = 9.0 / 280.0,
                    D1_10 = 41.0 / 840.0;
static const double D_1_0 = 2.0 / 27.0, D_2_0 = 1.0 / 36.0, D_3_0 = 1.0 / 24.0, D_4_0 = 5.0 / 12.0,
                    D_5_0 = 1.0 / 20.0, D_6_0 = -25.0 / 108.0, D_7_0 = 31.0 / 300.0, D_8_0 = 2.0,
                    D_9_0 = -91.0 / 108.0, D_10_0 = 2383.0 / 4100.0, D_11_0 = 3.0 / 205.0,
                    D_12_0 = -1777.0 / 4100.0;
static const double D_2_1 = 1.0 / 12.0;
static const double D_3_2 = 1.0 / 8.0, D_4_2 = -25.0 / 16.0;
static const double D_4_3 = 25.0 / 16.0, D_5_3 = 1.0 / 4.0, D_6_3 = 125.0 / 108.0, D_8_3 = -53.0 / 6.0,
                    D_9_3 = 23.0 / 108.0, D_10_3 = -341.0 / 164.0, D_12_3 = -341.0 / 164.0;
static const double D_5_4 = 1.0 / 5.0, D_6_4 = -65.0 / 27.0, D_7_4 = 61.0 / 225.0, D_8_4 = 704.0 / 45.0,
                    D_9_4 = -976.0 / 135.0, D_10_4 = 4496.0 / 1025.0, D_12_4 = 4496.0 / 1025.0;
static const double D_6_5 = 125.0 / 54.0, D_7_5 = -2.0 / 9.0, D_8_5 = -107.0 / 9.0, D_9_5 = 311.0 / 54.0,
                    D_10_5 = -301.0 / 82.0, D_11_5 = -6.0 / 41.0, D_12_5 = -289.0 / 82.0;
static const double D_7_6 = 13.0 / 900.0, D_8_6 = 67.0 / 90.0, D_9_6 = -19.0 / 60.0, D_10_6 = 2133.0 / 4100.0,
                    D_11_6 = -3.0 / 205.0, D_12_6 = 2193.0 / 4100.0;
static const double D_8_7 = 3.0, D_9_7 = 17.0 / 6.0, D_10_7 = 45.0 / 82.0, D_11_7 = -3.0 / 41.0,
                    D_12_7 = 51.0 / 82.0;
static const double D_9_8 = -1.0 / 12.0, D_10_8 = 45.0 / 164.0, D_11_8 = 3.0 / 41.0, D_12_8 = 33.0 / 164.0;
static const double D_10_9 = 18.0 / 41.0, D_11_9 = 6.0 / 41.0, D_12_9 = 12.0 / 41.0;
static const double D_12_11 = 1.0;

static void rkf78_step(orc_system* s, double t, double h, const double* y0, double* y, double* err) {
  /* RungeKuttaFehlberg78::Step, :147-250.  fk[0] is the Driver's accel. */
  int nv = 6 * s->total;
  double** fk = s->fk;
  double* yt = s->ytmp;
  const double* f0 = s->accel;
  int i;
  for (i = 0; i < nv; i++) yt[i] = y0[i] + h * (D_1_0 * f0[i]);
  orc_compute(s, t, yt, fk[1]);
  for (i = 0; i < nv; i++) yt[i] = y0[i] + h * (D_2_0 * f0[i] + D_2_1 * fk[1][i]);
  orc_compute(s, t, yt, fk[2]);
  for (i = 0; i < nv; i++) yt[i] = y0[i] + h * (D_3_0 * f0[i] + D_3_2 * fk[2][i]);
  orc_compute(s, t, yt, fk[3]);
  for (i = 0; i < nv; i++) yt[i] = y0[i] + h * (D_4_0 * f0[i] + D_4_2 * fk[2][i] + D_4_3 * fk[3][i]);
  orc_compute(s, t, yt, fk[4]);
  for (i = 0; i < nv; i++) yt[i] = y0[i] + h * (D_5_0 * f0[i] + D_5_3 * fk[3][i] + D_5_4 * fk[4][i]);
  orc_compute(s, t, yt, fk[5]);
  for (i = 0; i < nv; i++)
    yt[i] = y0[i] + h * (D_6_0 * f0[i] + D_6_3 * fk[3][i] + D_6_4 * fk[4][i] + D_6_5 * fk[5][i]);
  orc_compute(s, t, yt, fk[6]);
  for (i = 0; i < nv; i++)
    yt[i] = y0[i] + h * (D_7_0 * f0[i] + D_7_4 * fk[4][i] + D_7_5 * fk[5][i] + D_7_6 * fk[6][i]);
  orc_compute(s, t, yt, fk[7]);
  for (i = 0; i < nv; i++)
    yt[i] = y0[i] + h * (D_8_0 * f0[i] + D_8_3 * fk[3][i] + D_8_4 * fk[4][i] + D_8_5 * fk[5][i] +
                         D_8_6 * fk[6][i] + D_8_7 * fk[7][i]);
  orc_compute(s, t, yt, fk[8]);
  for (i = 0; i < nv; i++)
    yt[i] = y0[i] + h * (D_9_0 * f0[i] + D_9_3 * fk[3][i] + D_9_4 * fk[4][i] + D_9_5 * fk[5][i] +
                         D_9_6 * fk[6][i] + D_9_7 * fk[7][i] + D_9_8 * fk[8][i]);
  orc_compute(s, t, yt, fk[9]);
  for (i = 0; i < nv; i++)
    yt[i] = y0[i] + h * (D_10_0 * f0[i] + D_10_3 * fk[3][i] + D_10_4 * fk[4][i] + D_10_5 * fk[5][i] +
                         D_10_6 * fk[6][i] + D_10_7 * fk[7][i] + D_10_8 * fk[8][i] + D_10_9 * fk[9][i]);
  orc_compute(s, t, yt, fk[10]);
  for (i = 0; i < nv; i++)
    yt[i] = y0[i] + h * (D_11_0 * f0[i] + D_11_5 * fk[5][i] + D_11_6 * fk[6][i] + D_11_7 * fk[7][i] +
                         D_11_8 * fk[8][i] + D_11_9 * fk[9][i]);
  orc_compute(s, t, yt, fk[11]);
  for (i = 0; i < nv; i++)
    yt[i] = y0[i] + h * (D_12_0 * f0[i] + D_12_3 * fk[3][i] + D_12_4 * fk[4][i] + D_12_5 * fk[5][i] +
                         D_12_6 * fk[6][i] + D_12_7 * fk[7][i] + D_12_8 * fk[8][i] + D_12_9 * fk[9][i] +
                         D_12_11 * fk[11][i]);
  orc_compute(s, t, yt, fk[12]);
  for (i = 0; i < nv; i++)
    y[i] = y0[i] + h * (D1_0 * f0[i] + D1_5 * fk[5][i] + D1_6 * (fk[6][i] + fk[7][i]) +
                        D1_8 * (fk[8][i] + fk[9][i]) + D1_10 * fk[10][i]);
  for (i = 0; i < nv; i++) err[i] = h * fabs(f0[i] + fk[10][i] - fk[11][i] - fk[12][i]) * 41.0 / 840.0;
}

static double rkf78_error_max(const orc_system* s, int n, const double* yerr, const double* yscale) {
  /* GetErrorMax, :252-262 */
  double errorMax = 0.0;
  for (int i = 0; i < n; i++) {
    double err = fabs(yerr[i] / yscale[i]);
    if (err > errorMax) errorMax = err;
  }
  return errorMax / s->epsilon;
}

int orc_rkf78_step(orc_system* s, double t, double h, const double* y0, double* y, double* error,
                   double* error_max) {
  int nv = 6 * s->total;
  s->eval_drag = s->eval_mig1 = s->eval_mig2 = 1;
  orc_compute(s, t, y0, s->accel);
  for (int i = 0; i < nv; i++) s->yscale[i] = fabs(y0[i]) + fabs(h * s->accel[i]) + 1.0e-30;
  s->eval_mig1 = s->eval_mig2 = 0;
  rkf78_step(s, t, h, y0, y, error);
  if (error_max) *error_max = rkf78_error_max(s, nv, error, s->yscale);
  return 0;
}

static int rkf78_driver(orc_system* s, double* y0, sol_time_line* tl, sol_step_stats* st) {
  /* RungeKuttaFehlberg78::Driver, :66-140 (SAFETY .9, PGROW -.2, PSHRNK -.25,
   * ERRCON 1.89e-4, TINY 1e-30) */
  int nv = 6 * s->total;
  double time = tl->time;
  double h = tl->h_next;
  s->eval_drag = s->eval_mig1 = s->eval_mig2 = 1;
  orc_compute(s, tl->time, y0, s->accel);
  if (st) st->evaluations++;
  for (int i = 0; i < nv; i++) s->yscale[i] = fabs(y0[i]) + fabs(h * s->accel[i]) + 1.0e-30;
  s->eval_mig1 = s->eval_mig2 = 0;
  double errorMax = 0.0;
  for (;;) {
    rkf78_step(s, time, h, y0, s->ybuf, s->error);
    if (st) st->evaluations += 12;
    errorMax = rkf78_error_max(s, nv, s->error, s->yscale);
    if (errorMax < 1.0) {
      tl->h_did = h;
      break;
    }
    if (st) st->rejected++;
    double hTemp = 0.9 * h * pow(errorMax, -0.25);
    h = fabs(hTemp) > fabs(0.1 * h) ? hTemp : 0.1 * h;
    double tNew = tl->time + h;
    if (tNew == tl->time) return SOL_ERR_UNDERFLOW;
  }
  tl->time += tl->h_did;
  tl->h_next = errorMax > 1.89e-4 ? (0.9 * h * pow(errorMax, -0.2)) : (5.0 * h);
  memcpy(y0, s->ybuf, sizeof(double) * nv); /* swap(y0, y) */
  if (st) st->accepted++;
  return 0;
}

static int rk4_driver(orc_system* s, double* y0, sol_time_line* tl, sol_step_stats* st) {
  /* RungeKutta4::Driver and Step, Solaris/RungeKutta4.cpp:20-129 */
  int nv = 6 * s->total;
  double h = tl->h_next;
  double t = tl->time;
  s->eval_drag = s->eval_mig1 = s->eval_mig2 = 1;
  orc_compute(s, tl->time, y0, s->accel);
  s->eval_mig1 = s->eval_mig2 = 0;
  const double a21 = 1.0 / 2.0, a32 = 1.0 / 2.0, a43 = 1.0;
  const double b1 = 1.0 / 6.0, b2 = 1.0 / 3.0, b3 = 1.0 / 3.0, b4 = 1.0 / 6.0;
  const double c2 = 1.0 / 2.0, c3 = 1.0 / 2.0, c4 = 1.0;
  double** fk = s->fk;
  double* yt = s->ytmp;
  const double* f0 = s->accel;
  int i;
  for (i = 0; i < nv; i++) yt[i] = y0[i] + h * (a21 * f0[i]);
  orc_compute(s, t + c2 * h, yt, fk[1]);
  for (i = 0; i < nv; i++) yt[i] = y0[i] + h * (a32 * fk[1][i]);
  orc_compute(s, t + c3 * h, yt, fk[2]);
  for (i = 0; i < nv; i++) yt[i] = y0[i] + h * (a43 * fk[2][i]);
  orc_compute(s, t + c4 * h, yt, fk[3]);
  for (i = 0; i < nv; i++) s->ybuf[i] = y0[i] + h * (b1 * f0[i] + b2 * fk[1][i] + b3 * fk[2][i] + b4 * fk[3][i]);
  if (st) { st->evaluations += 4; st->accepted++; }
  tl->h_did = h;
  tl->time += tl->h_did;
  tl->h_next = h;
  memcpy(y0, s->ybuf, sizeof(double) * nv);
  return 0;
}

/* Dormand-Prince RKN 7(6) tableau, Solaris/DormandPrince.cpp:37-124 */
typedef struct dp_tab { double b[9], bdh[9], c[9], a[9][8]; } dp_tab;
static void dp_init(dp_tab* T) {
  double sQ = sqrt(21.0);
  memset(T, 0, sizeof(*T));
  T->b[0] = 1.0 / 20.0; T->b[4] = 8.0 / 45.0; T->b[5] = 7.0 * (7.0 + sQ) / 360.0;
  T->b[6] = 7.0 * (7.0 - sQ) / 360.0; T->b[7] = -1.0 / 20.0; T->b[8] = 1.0 / 20.0;
  T->bdh[0] = 1.0 / 20.0; T->bdh[4] = 16.0 / 45.0; T->bdh[5] = 49.0 / 180.0; T->bdh[6] = 49.0 / 180.0;
  T->bdh[7] = 1.0 / 20.0;
  T->c[1] = 1.0 / 10.0; T->c[2] = 1.0 / 5.0; T->c[3] = 3.0 / 8.0; T->c[4] = 1.0 / 2.0;
  T->c[5] = (7.0 - sQ) / 14.0; T->c[6] = (7.0 + sQ) / 14.0; T->c[7] = 1.0; T->c[8] = 1.0;
  T->a[1][0] = 1.0 / 200.0;
  T->a[2][0] = 1.0 / 150.0; T->a[2][1] = 1.0 / 75.0;
  T->a[3][0] = 171.0 / 8192.0; T->a[3][1] = 45.0 / 4096.0; T->a[3][2] = 315.0 / 8192.0;
  T->a[4][0] = 5.0 / 288.0; T->a[4][1] = 25.0 / 528.0; T->a[4][2] = 25.0 / 672.0; T->a[4][3] = 16.0 / 693.0;
  T->a[5][0] = (1003.0 - 205.0 * sQ) / 12348.0; T->a[5][1] = -25.0 * (751.0 - 173.0 * sQ) / 90552.0;
  T->a[5][2] = 25.0 * (624.0 - 137.0 * sQ) / 43218.0; T->a[5][3] = -128.0 * (361.0 - 79.0 * sQ) / 237699.0;
  T->a[5][4] = (3411.0 - 745.0 * sQ) / 24696.0;
  T->a[6][0] = (793.0 + 187.0 * sQ) / 12348.0; T->a[6][1] = -25.0 * (331.0 + 113.0 * sQ) / 90552.0;
  T->a[6][2] = 25.0 * (1044.0 + 247.0 * sQ) / 43218.0; T->a[6][3] = -128.0 * (14885.0 + 3779.0 * sQ) / 9745659.0;
  T->a[6][4] = (3327.0 + 797.0 * sQ) / 24696.0; T->a[6][5] = -(581.0 + 127.0 * sQ) / 1722.0;
  T->a[7][0] = -(157.0 - 3.0 * sQ) / 378.0; T->a[7][1] = 25.0 * (143.0 - 10.0 * sQ) / 2772.0;
  T->a[7][2] = -25.0 * (876.0 + 55.0 * sQ) / 3969.0; T->a[7][3] = 1280.0 * (913.0 + 18.0 * sQ) / 596673.0;
  T->a[7][4] = -(1353.0 + 26.0 * sQ) / 2268.0; T->a[7][5] = 7.0 * (1777.0 + 377.0 * sQ) / 4428.0;
  T->a[7][6] = 7.0 * (5.0 - sQ) / 36.0;
  T->a[8][0] = 1.0 / 20.0; T->a[8][4] = 8.0 / 45.0; T->a[8][5] = 7.0 * (7.0 + sQ) / 360.0;
  T->a[8][6] = 7.0 * (7.0 - sQ) / 360.0;
}

static void dp_step2(orc_system* s, const dp_tab* T, double time, double h, const double* y0, double* y,
                     double* err) {
  /* DormandPrince::Step2, :246-491.  f[0] is the Driver's accel. */
  int N = s->total;
  double h2 = h * h;
  double* f[9];
  f[0] = s->accel;
  for (int k = 1; k < 9; ++k) f[k] = s->fk[k];
  double* yt = s->ytmp;
  for (int k = 1; k < 9; ++k) {
    double ttemp = time + T->c[k] * h;
    for (int i = 0; i < N; i++) {
      int i0 = 6 * i;
      for (int j = 0; j < 3; j++) {
        int n = i0 + j;
        double var;
        if (k == 8) {
          var = T->a[k][0] * f[0][n + 3] + T->a[k][4] * f[4][n + 3] + T->a[k][5] * f[5][n + 3] +
                T->a[k][6] * f[6][n + 3];
        } else {
          var = T->a[k][0] * f[0][n + 3];
          for (int l = 1; l < k; ++l) var = var + T->a[k][l] * f[l][n + 3];
        }
        yt[n] = y0[n] + T->c[k] * h * y0[n + 3] + h2 * (var);
        yt[n + 3] = y0[n + 3] + h * (var);
      }
    }
    orc_compute(s, ttemp, yt, f[k]);
  }
  for (int i = 0; i < N; i++) {
    int i0 = 6 * i;
    for (int j = 0; j < 3; j++) {
      int n = i0 + j;
      y[n] = y0[n] + h * y0[n + 3] +
             h2 * (T->b[0] * f[0][n + 3] + T->b[4] * f[4][n + 3] + T->b[5] * f[5][n + 3] +
                   T->b[6] * f[6][n + 3] + T->b[7] * f[7][n + 3] + T->b[8] * f[8][n + 3]);
      err[n] = h2 * fabs(f[7][n + 3] - f[8][n + 3]) / 20.0;
      y[n + 3] = y0[n + 3] + h * (T->bdh[0] * f[0][n + 3] + T->bdh[4] * f[4][n + 3] + T->bdh[5] * f[5][n + 3] +
                                  T->bdh[6] * f[6][n + 3] + T->bdh[7] * f[7][n + 3]);
      err[n + 3] = 0.0;
    }
  }
}

static int dp_driver(orc_system* s, double* y0, sol_time_line* tl, sol_step_stats* st) {
  /* DormandPrince::Driver, :126-170 (maxIter 10) */
  dp_tab T;
  dp_init(&T);
  int nv = 6 * s->total;
  double time = tl->time;
  s->eval_drag = s->eval_mig1 = s->eval_mig2 = 1;
  orc_compute(s, tl->time, y0, s->accel);
  if (st) st->evaluations++;
  s->eval_mig1 = s->eval_mig2 = 0;
  int iter = 0;
  double errorMax = 0.0;
  do {
    iter++;
    double h = tl->h_next;
    dp_step2(s, &T, time, h, y0, s->ybuf, s->error);
    if (st) st->evaluations += 8;
    errorMax = 0.0;
    for (int i = 0; i < nv; i++) {
      double e = fabs(s->error[i]);
      if (e > errorMax) errorMax = e;
    }
    tl->h_did = h;
    tl->h_next = errorMax < 1.0e-20 ? 2.0 * h : 0.9 * h * pow(s->epsilon / errorMax, 1.0 / 7.0);
    if (st && errorMax > s->epsilon) st->rejected++;
  } while (errorMax > s->epsilon && iter <= 10);
  if (iter > 10) return SOL_ERR_MAXITER;
  tl->time += tl->h_did;
  memcpy(y0, s->ybuf, sizeof(double) * nv);
  if (st) st->accepted++;
  return 0;
}

int orc_driver(orc_system* s, int32_t integrator, double* y0, sol_time_line* tl, int32_t n_steps,
               sol_step_stats* stats, double* times, double* h_did, double* h_next) {
  for (int k = 0; k < n_steps; ++k) {
    int r;
    if (integrator == SOL_RUNGE_KUTTA_FEHLBERG78) r = rkf78_driver(s, y0, tl, stats);
    else if (integrator == SOL_RUNGE_KUTTA4) r = rk4_driver(s, y0, tl, stats);
    else if (integrator == SOL_DORMAND_PRINCE) r = dp_driver(s, y0, tl, stats);
    else return SOL_ERR_ARG;
    if (r) return r;
    if (times) times[k] = tl->time;
    if (h_did) h_did[k] = tl->h_did;
    if (h_next) h_next[k] = tl->h_next;
  }
  return 0;
}

/* ---- events: Simulator::CheckEvent predicates (Simulator.cpp:626-645, 690-729) */
int orc_check_events(const orc_system* s, const double* y0, double ejection, double hit_centrum,
                     double collision_factor, sol_event* out, int32_t capacity, int32_t* n_out) {
  int n = 0;
  double e3 = ejection > 0 ? 1.0 / (ejection * ejection * ejection) : 0.0;
  double h3 = hit_centrum > 0 ? 1.0 / (hit_centrum * hit_centrum * hit_centrum) : 0.0;
  for (int i = 1; i < s->total; i++) {
    int i0 = 6 * i;
    double r = sqrt(SQR(y0[i0 + 0]) + SQR(y0[i0 + 1]) + SQR(y0[i0 + 2]));
    if (ejection > 0 && s->rm3 && s->rm3[i] < e3) {
      if (n < capacity) { out[n].kind = SOL_EVENT_EJECTION; out[n].idx1 = 0; out[n].idx2 = i; out[n].pad = 0; out[n].distance = r; }
      n++;
    }
    if (hit_centrum > 0 && s->rm3 && s->rm3[i] > h3) {
      if (n < capacity) { out[n].kind = SOL_EVENT_HIT_CENTRUM; out[n].idx1 = 0; out[n].idx2 = i; out[n].pad = 0; out[n].distance = r; }
      n++;
    }
  }
  if (collision_factor > 0) {
    for (int i = 0; i < s->total; i++) {
      int j = s->nn_idx[i];
      if (j >= 0 && collision_factor * (s->radius[i] + s->radius[j]) > s->nn_dist[i]) {
        if (n < capacity) { out[n].kind = SOL_EVENT_COLLISION; out[n].idx1 = i; out[n].idx2 = j; out[n].pad = 0; out[n].distance = s->nn_dist[i]; }
        n++;
      }
    }
  }
  *n_out = n;
  return 0;
}

/* ---- Calculate::Integrals (Solaris/Calculate.cpp:43-172) ----------------- */
void orc_integrals(const orc_system* s, const double* y0, double out[16]) {
  int N = s->total;
  int nm = n_massive(s);
  double M = 0.0;
  for (int i = 0; i < nm; i++) M += s->mass[i];
  out[0] = M;
  double bc[6] = {0, 0, 0, 0, 0, 0};
  for (int i = 0; i < N; i++)
    for (int j = 0; j < 6; j++) bc[j] += s->mass[i] * y0[6 * i + j];
  for (int j = 0; j < 6; j++) out[1 + j] = bc[j] / M;
  out[7] = sqrt(SQR(out[1]) + SQR(out[2]) + SQR(out[3]));
  out[8] = sqrt(SQR(out[4]) + SQR(out[5]) + SQR(out[6]));
  double cx = 0, cy = 0, cz = 0;
  for (int i = 0; i < N; i++) {
    const double* p = &y0[6 * i];
    double m = s->mass[i];
    double rx = p[1] * p[5] - p[2] * p[4];
    double ry = p[2] * p[3] - p[0] * p[5];
    double rz = p[0] * p[4] - p[1] * p[3];
    cx += m * rx;
    cy += m * ry;
    cz += m * rz;
  }
  out[9] = cx; out[10] = cy; out[11] = cz;
  out[12] = sqrt(cx * cx + cy * cy + cz * cz);
  double ke = 0.0;
  for (int i = 0; i < N; i++) {
    const double* p = &y0[6 * i];
    double v2 = SQR(p[3]) + SQR(p[4]) + SQR(p[5]);
    ke += 0.5 * s->mass[i] * v2;
  }
  out[13] = ke;
  double pe = 0.0;
  for (int i = 0; i < N; i++) {
    for (int j = 0; j < N; j++) {
      if (i == j) continue;
      double dx = y0[6 * j + 0] - y0[6 * i + 0];
      double dy = y0[6 * j + 1] - y0[6 * i + 1];
      double dz = y0[6 * j + 2] - y0[6 * i + 2];
      double rij = sqrt(dx * dx + dy * dy + dz * dz);
      pe += s->mass[i] * s->mass[j] / rij;
    }
  }
  pe *= 0.5 * K_GAUSS2;
  out[14] = pe;
  out[15] = out[13] - out[14];
}

/* ---- bounded CPU-baseline sample --------------------------------------- */
int64_t orc_gravity_ac_sample(orc_system* s, const double* y, int32_t i_begin, int32_t i_end, double* dydt,
                              int32_t n_threads) {
  if (!s->rm3) s->rm3 = dup_d(NULL, s->total, 0.0);
  gravity_ac_prepass(s, y);
  int nm = n_massive(s);
  if (i_begin < 1) i_begin = 1;
  if (i_end > s->total) i_end = s->total;
  int64_t pairs = 0;
#ifdef _OPENMP
  if (n_threads < 1) n_threads = 1;
#pragma omp parallel for schedule(dynamic, 16) num_threads(n_threads) reduction(+ : pairs)
#endif
  for (int i = i_begin; i < i_end; i++) {
    gravity_ac_sink(s, y, dydt, i, nm);
    int ns = s->type[i] <= SOL_PROTO_PLANET ? nm + s->n.super_planetesimal : nm;
    pairs += (ns - 1) - ((i >= 1 && i < ns) ? 1 : 0) + 1; /* Kepler term + direct terms */
  }
  return pairs;
}

/* ---- fixed-step RKF78 and its tangent-linear model ----------------------
 * Fixed-step integration: RungeKuttaFehlberg78::Step at constant h (no step
 * control), y_{n+1} = its 7th-order result (RungeKuttaFehlberg78.cpp:236-238).
 * Masses are variables of the tangent-linear model (the gradient with respect
 * to masses is part of the adjoint's output); gas terms are not included. */

/* T(x) v = v / |x|^3 - 3 x (x . v) / |x|^5 */
static void tensor_apply(const double* x, const double* v, double* out) {
  double r2 = x[0] * x[0] + x[1] * x[1] + x[2] * x[2];
  double r = sqrt(r2);
  double r3 = r2 * r;
  double r5 = r3 * r2;
  double xv = x[0] * v[0] + x[1] * v[1] + x[2] * v[2];
  for (int k = 0; k < 3; ++k) out[k] = v[k] / r3 - 3.0 * x[k] * xv / r5;
}

/* Jacobian-vector product of GravityAC (Acceleration.cpp:248-329):
 * d(dydt) for a perturbation (dy, dm) at state y. */
void orc_jvp(orc_system* s, const double* y, const double* dy, const double* dm, double* df) {
  int N = s->total, nm = n_massive(s), nspl = s->n.super_planetesimal;
  double m0 = s->mass[0], dm0 = dm ? dm[0] : 0.0;
  for (int k = 0; k < 6; ++k) df[k] = 0.0;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(s->n_threads) if (s->n_threads > 1)
#endif
  for (int i = 1; i < N; ++i) {
    const double* ri = &y[6 * i];
    const double* dri = &dy[6 * i];
    double* o = &df[6 * i];
    o[0] = dri[3];
    o[1] = dri[4];
    o[2] = dri[5];
    double r2 = ri[0] * ri[0] + ri[1] * ri[1] + ri[2] * ri[2];
    double rm3 = 1.0 / (r2 * sqrt(r2));
    double t[3];
    tensor_apply(ri, dri, t);
    double mu = K_GAUSS2 * (m0 + s->mass[i]);
    double dmu = K_GAUSS2 * (dm0 + (dm ? dm[i] : 0.0));
    for (int k = 0; k < 3; ++k) o[3 + k] = -dmu * ri[k] * rm3 - mu * t[k];
    int ns = s->type[i] <= SOL_PROTO_PLANET ? nm + nspl : nm;
    for (int j = 1; j < ns; ++j) {
      if (j == i) continue;
      const double* rj = &y[6 * j];
      const double* drj = &dy[6 * j];
      double d[3] = {rj[0] - ri[0], rj[1] - ri[1], rj[2] - ri[2]};
      double dd[3] = {drj[0] - dri[0], drj[1] - dri[1], drj[2] - dri[2]};
      double d2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
      double dm3 = 1.0 / (d2 * sqrt(d2));
      double rj2 = rj[0] * rj[0] + rj[1] * rj[1] + rj[2] * rj[2];
      double rjm3 = 1.0 / (rj2 * sqrt(rj2));
      double td[3], tr[3];
      tensor_apply(d, dd, td);
      tensor_apply(rj, drj, tr);
      double gm = K_GAUSS2 * s->mass[j];
      double gdm = K_GAUSS2 * (dm ? dm[j] : 0.0);
      for (int k = 0; k < 3; ++k) o[3 + k] += gdm * (d[k] * dm3 - rj[k] * rjm3) + gm * (td[k] - tr[k]);
    }
  }
}

static void rkf78_fixed_stages(orc_system* s, const double* y0, double h, double* ynew, double** Y, double** F) {
  /* stage states Y[0..12] and derivatives F[0..12] of one Step at fixed h */
  const int nv = 6 * s->total;
  const double A[13][13] = {
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
  const double B[13] = {41.0 / 840.0, 0, 0, 0, 0, 34.0 / 105.0, 9.0 / 35.0, 9.0 / 35.0, 9.0 / 280.0, 9.0 / 280.0,
                        41.0 / 840.0, 0, 0};
  for (int r = 0; r < 13; ++r) {
    for (int e = 0; e < nv; ++e) {
      double acc = 0.0;
      for (int l = 0; l < r; ++l) acc += A[r][l] * F[l][e];
      Y[r][e] = y0[e] + h * acc;
    }
    s->eval_drag = s->eval_mig1 = s->eval_mig2 = 0;
    orc_compute(s, 0.0, Y[r], F[r]);
  }
  for (int e = 0; e < nv; ++e) {
    double acc = 0.0;
    for (int k = 0; k < 13; ++k) acc += B[k] * F[k][e];
    ynew[e] = y0[e] + h * acc;
  }
}

/* n fixed steps from y0; with dy0/dm also the tangent-linear solution dy. */
int orc_rkf78_fixed(orc_system* s, const double* y0, double h, int32_t n_steps, double* y_out, const double* dy0,
                    const double* dm, double* dy_out) {
  const int nv = 6 * s->total;
  double *Y[13], *F[13], *dY[13], *dF[13];
  for (int k = 0; k < 13; ++k) {
    Y[k] = (double*)malloc(sizeof(double) * nv);
    F[k] = (double*)malloc(sizeof(double) * nv);
    dY[k] = (double*)malloc(sizeof(double) * nv);
    dF[k] = (double*)malloc(sizeof(double) * nv);
  }
  double* y = (double*)malloc(sizeof(double) * nv);
  double* yn = (double*)malloc(sizeof(double) * nv);
  double* dy = (double*)malloc(sizeof(double) * nv);
  memcpy(y, y0, sizeof(double) * nv);
  if (dy0) memcpy(dy, dy0, sizeof(double) * nv);
  const double A[13][13] = {
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
  const double B[13] = {41.0 / 840.0, 0, 0, 0, 0, 34.0 / 105.0, 9.0 / 35.0, 9.0 / 35.0, 9.0 / 280.0, 9.0 / 280.0,
                        41.0 / 840.0, 0, 0};
  for (int n = 0; n < n_steps; ++n) {
    rkf78_fixed_stages(s, y, h, yn, Y, F);
    if (dy0) {
      for (int r = 0; r < 13; ++r) {
        for (int e = 0; e < nv; ++e) {
          double acc = 0.0;
          for (int l = 0; l < r; ++l) acc += A[r][l] * dF[l][e];
          dY[r][e] = dy[e] + h * acc;
        }
        orc_jvp(s, Y[r], dY[r], dm, dF[r]);
      }
      for (int e = 0; e < nv; ++e) {
        double acc = 0.0;
        for (int k = 0; k < 13; ++k) acc += B[k] * dF[k][e];
        dy[e] = dy[e] + h * acc;
      }
    }
    memcpy(y, yn, sizeof(double) * nv);
  }
  memcpy(y_out, y, sizeof(double) * nv);
  if (dy0 && dy_out) memcpy(dy_out, dy, sizeof(double) * nv);
  for (int k = 0; k < 13; ++k) {
    free(Y[k]);
    free(F[k]);
    free(dY[k]);
    free(dF[k]);
  }
  free(y);
  free(yn);
  free(dy);
  return 0;
}

void orc_set_masses(orc_system* s, const double* mass) { memcpy(s->mass, mass, sizeof(double) * s->total); }

/* ---- events: Simulator::CheckEvent (Simulator.cpp:621-735), RemoveBody
 * (:737-771), HandleCollision (:773-935) ---------------------------------------
 * The reference's order and arithmetic, with bodies identified by identity
 * where the reference indexes arrays that earlier removals have shifted, and
 * every per-body array compacted (RemoveBody shifts only some of them): the
 * semantics the device implementation documents. */
static int ev_position(const char* removed, int b) {
  int p = 0;
  for (int q = 0; q < b; ++q) p += !removed[q];
  return p;
}

static void ev_log(orc_system* s, const double* y0, sol_affair* log, int cap, int* nl, int type, int idx1, int idx2,
                   int b1, int b2, double time) {
  if (*nl < cap) {
    sol_affair* f = &log[*nl];
    f->type = type;
    f->idx1 = idx1;
    f->idx2 = idx2;
    f->id1 = s->id[b1];
    f->id2 = s->id[b2];
    f->pad = 0;
    f->time = time;
    for (int q = 0; q < 6; ++q) {
      f->phase1[q] = y0[6 * b1 + q];
      f->phase2[q] = y0[6 * b2 + q];
    }
  }
  (*nl)++;
}

static void ev_survivor(const orc_system* s, int a, int b, int* sv, int* mg) {  /* :775-781 */
  if (s->mass[a] == s->mass[b]) {
    *sv = a < b ? a : b;
    *mg = a > b ? a : b;
  } else {
    *sv = s->mass[a] > s->mass[b] ? a : b;
    *mg = s->mass[a] < s->mass[b] ? a : b;
  }
}

static void ev_merge(orc_system* s, double* y0, int sv, int mg) {  /* :799-880 */
  double ms = s->mass[sv];
  double mm = s->type[mg] == SOL_SUPER_PLANETESIMAL
                  ? s->density[mg] * (4.0 / 3.0 * K_PI * (s->radius[mg] * s->radius[mg] * s->radius[mg]))
                  : s->mass[mg];
  double M = ms + mm;
  if (s->type[sv] != SOL_CENTRAL_BODY)
    for (int q = 0; q < 6; ++q) y0[6 * sv + q] = 1.0 / M * (ms * y0[6 * sv + q] + mm * y0[6 * mg + q]);
  s->mass[sv] = M;
  if (s->radius[sv] == 0.0) return;
  if (s->radius[mg] == 0.0) {
    s->density[mg] = s->density[sv];
    s->radius[mg] = pow(3.0 / (4.0 * K_PI) * s->mass[mg] / s->density[mg], 1.0 / 3.0);
  }
  double rs = s->radius[sv], rm = s->radius[mg];
  double vol = 4.0 / 3.0 * K_PI * (rs * rs * rs + rm * rm * rm);
  s->radius[sv] = pow(3.0 / (4.0 * K_PI) * vol, 1.0 / 3.0);
  s->density[sv] = M / vol;
}

static void compact_d(double* a, const char* removed, int n, int width) {
  int k = 0;
  for (int i = 0; i < n; ++i)
    if (!removed[i]) {
      if (k != i) memmove(a + (size_t)k * width, a + (size_t)i * width, sizeof(double) * width);
      k++;
    }
}
static void compact_i(int32_t* a, const char* removed, int n) {
  int k = 0;
  for (int i = 0; i < n; ++i)
    if (!removed[i]) a[k++] = a[i];
}
static void compact_rows(double* buf, const char* removed, int lo, int hi) {
  int k = 0;
  for (int i = lo; i < hi; ++i)
    if (!removed[i]) {
      if (k != i - lo) memmove(buf + 3 * k, buf + 3 * (i - lo), 3 * sizeof(double));
      k++;
    }
}

int orc_handle_events(orc_system* s, double time, double ejection, double hit_centrum, double factor, double* y0,
                      sol_affair* log, int32_t cap, int32_t* n_log) {
  const int n = s->total;
  char* removed = (char*)calloc(n > 0 ? n : 1, 1);
  double e3 = ejection > 0 ? 1.0 / (ejection * ejection * ejection) : 0.0;
  double h3 = hit_centrum > 0 ? 1.0 / (hit_centrum * hit_centrum * hit_centrum) : 0.0;
  int nl = 0;
  for (int i = 1; i < n; ++i)  /* ejections (:631-637, :648-659) */
    if (ejection > 0 && s->rm3[i] < e3) {
      ev_log(s, y0, log, cap, &nl, 0, 0, i, 0, i, time);
      removed[i] = 1;
    }
  for (int i = 1; i < n; ++i)  /* hit centrum (:639-645, :661-687) */
    if (!removed[i] && hit_centrum > 0 && s->rm3[i] > h3) {
      ev_log(s, y0, log, cap, &nl, 1, 0, i, 0, i, time);
      int sv, mg;
      ev_survivor(s, 0, i, &sv, &mg);
      if (s->type[mg] != SOL_TEST_PARTICLE) ev_merge(s, y0, sv, mg);
      removed[i] = 1;
    }
  if (factor > 0)  /* collisions (:689-732) */
    for (int i = 0; i < n; ++i) {
      if (removed[i]) continue;
      int j = s->nn_idx[i];
      if (j < 0 || removed[j] || !(factor * (s->radius[i] + s->radius[j]) > s->nn_dist[i])) continue;
      int sv, mg;
      ev_survivor(s, i, j, &sv, &mg);
      if (s->type[mg] == SOL_TEST_PARTICLE) {
        s->nn_idx[i] = -1;
        continue;
      }
      ev_log(s, y0, log, cap, &nl, 3, ev_position(removed, sv), ev_position(removed, mg), sv, mg, time);
      ev_merge(s, y0, sv, mg);
      removed[mg] = 1;
      s->nn_idx[mg] = -1;
    }
  int nr = 0;
  for (int i = 0; i < n; ++i) nr += removed[i];
  if (nr > 0) {
    const int nm_old = n_massive(s), nc_old = s->n.central_body, ng_old = s->n.giant_planet;
    const int hi_drag = nm_old + n_pl_and_spl(s);
    if (s->acc_drag) compact_rows(s->acc_drag, removed, nm_old, hi_drag);
    if (s->acc_mig1) compact_rows(s->acc_mig1, removed, nc_old + ng_old, nm_old);
    if (s->acc_mig2) compact_rows(s->acc_mig2, removed, nc_old, nc_old + ng_old);
    for (int i = 0; i < n; ++i) {
      if (!removed[i]) continue;
      switch (s->type[i]) {
        case SOL_CENTRAL_BODY: s->n.central_body--; break;
        case SOL_GIANT_PLANET: s->n.giant_planet--; break;
        case SOL_ROCKY_PLANET: s->n.rocky_planet--; break;
        case SOL_PROTO_PLANET: s->n.proto_planet--; break;
        case SOL_SUPER_PLANETESIMAL: s->n.super_planetesimal--; break;
        case SOL_PLANETESIMAL: s->n.planetesimal--; break;
        default: s->n.test_particle--; break;
      }
    }
    compact_i(s->id, removed, n);
    compact_i(s->type, removed, n);
    compact_i(s->mig_type, removed, n);
    double* per_body[] = {s->mig_stop_at, s->mass, s->radius, s->density, s->cd, s->gamma_stokes, s->gamma_epstein,
                          s->rm3};
    for (int k = 0; k < 8; ++k) compact_d(per_body[k], removed, n, 1);
    compact_d(y0, removed, n, 6);
    s->total = n - nr;
    for (int i = 0; i < s->total; ++i) {
      s->nn_idx[i] = -1;
      s->nn_dist[i] = 0.0;
    }
  }
  free(removed);
  *n_log = nl;
  return 0;
}

void orc_get_bodies(const orc_system* s, sol_nbodies* counts, int32_t* id, int32_t* type, double* mass,
                    double* radius, double* density) {
  const size_t n = (size_t)s->total;
  if (counts) *counts = s->n;
  if (id) memcpy(id, s->id, sizeof(int32_t) * n);
  if (type) memcpy(type, s->type, sizeof(int32_t) * n);
  if (mass) memcpy(mass, s->mass, sizeof(double) * n);
  if (radius) memcpy(radius, s->radius, sizeof(double) * n);
  if (density) memcpy(density, s->density, sizeof(double) * n);
}

/* ---- GasComponent helpers, for their known-answer tests ------------------- */
/* which: 0 circular_velocity(mu, r) -> out[3]; 1 gas_velocity(mu, r) -> out[3];
 * 2 gas_density_at(r); 3 MeanFreePath_CMU(rho); 4 SoundSpeed_CMU(T);
 * 5 Temperature_CMU(mC, r); 6 MeanThermalSpeed_CMU(mC, r) as the drag calls it
 * (GasComponent.cpp:97-157, :159-243). */
double orc_gas_probe(const sol_gas_component* g, int32_t which, const double* args, double* out3) {
  switch (which) {
    case 0: circular_velocity(args[0], args + 1, out3); return 0.0;
    case 1: gas_velocity(g, args[0], args + 1, out3); return 0.0;
    case 2: return gas_density_at(g, args);
    case 3: {  /* MeanFreePath_CMU (:170-188) */
      const double sqrt_two_pi = 4.4428829381583662470158809900607;  /* the value of the reference's constant */
      double a1 = g->mean_molecular_weight * c_proton_mass_cmu();
      double d2 = SQR(g->particle_diameter * c_meter_to_au());
      double result = a1 / sqrt_two_pi;
      return result / (d2 * args[0]);
    }
    case 4: {  /* SoundSpeed_CMU (:198-204) */
      double result = c_boltzman_cmu() * args[0];
      result /= g->mean_molecular_weight * c_proton_mass_cmu();
      return sqrt(result);
    }
    case 5: {  /* Temperature_CMU (:221-229) */
      double cTp = K_GAUSS2 * c_proton_mass_boltzman_cmu();
      double pT = 2.0 * g->scale_height.index - 3.0;
      double cT = SQR(g->scale_height.c) * args[0] * g->mean_molecular_weight * cTp;
      return cT * pow(args[1], pT);
    }
    case 6: {
      orc_system tmp;
      memset(&tmp, 0, sizeof(tmp));
      tmp.gas = *g;
      return mean_thermal_speed_cmu(&tmp, args[0], args[1]);
    }
    default: return 0.0;
  }
}

/* KeplerEquationSolver with the stopping rule selectable: SOL_QUIRK_INT_ABS
 * as the reference build, 0 with fabs (as the reference's CUDA prototypes). */
int orc_kepler_solve(double e, double m, double eps, int32_t quirks, double* E) {
  if (e == 0.0 || m == 0.0 || m == K_PI) {
    *E = m;
    return 0;
  }
  double EE = m + e * (sin(m)) / (1.0 - sin(m + e) + sin(m));
  double E1 = 0.0, error;
  int step = 0;
  do {
    E1 = EE - (EE - e * sin(EE) - m) / (1.0 - e * cos(EE));
    error = quirk_abs(E1 - EE, quirks);
    EE = E1;
    step++;
  } while (error > eps && step <= 25);
  *E = EE;
  return step > 25 ? 1 : 0;
}
