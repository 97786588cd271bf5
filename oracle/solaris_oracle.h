/*
 * solaris_oracle.h - CPU restatement of the Solaris force-and-integrate path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker for the GB300 kernels: it is
 * imported by tests/, by __graft_entry__.smoke() and by bench.py's CPU
 * baseline, never by the library.  Each function follows the reference
 * function named in its comment operation by operation (no contraction:
 * compile with -ffp-contract=off), so that on the same inputs it reproduces
 * the reference build bit for bit; tests/test_oracle_golden.py pins it
 * against fixtures produced by the reference itself.
 */
#ifndef SOLARIS_ORACLE_H_
#define SOLARIS_ORACLE_H_

#include "../include/solaris_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_system orc_system;

orc_system* orc_create(const sol_body_data* bodies, const sol_gas_component* gas_or_null,
                       int32_t barycentric);
void orc_destroy(orc_system* s);
int32_t orc_n_total(const orc_system* s);
void orc_set_eval_flags(orc_system* s, uint32_t flags);
void orc_set_epsilon(orc_system* s, double eps);
/* host threads of the sink loops of GravityAC and orc_jvp (default 1) */
void orc_set_threads(orc_system* s, int32_t n_threads);

/* Acceleration::Compute (Solaris/Acceleration.cpp:60-80). */
int orc_compute(orc_system* s, double t, const double* y, double* dydt);
/* Outputs of the last Compute: rm3, indexOfNN, distanceOfNN, migType. */
void orc_get_last_eval(const orc_system* s, double* rm3, int32_t* nn_idx, double* nn_dist);
void orc_get_mig_type(const orc_system* s, int32_t* mig_type);

/* One RKF78 attempt with the Driver's flag protocol and yscale. */
int orc_rkf78_step(orc_system* s, double t, double h, const double* y0, double* y,
                   double* error, double* error_max);
/* n_steps Driver calls (integrator = sol_integrator_type).  y0 in/out.
 * times/h_did/h_next (n_steps entries each) may be NULL. */
int orc_driver(orc_system* s, int32_t integrator, double* y0, sol_time_line* tl, int32_t n_steps,
               sol_step_stats* stats, double* times, double* h_did, double* h_next);

/* Simulator::CheckEvent predicates on the last evaluation. */
int orc_check_events(const orc_system* s, const double* y0, double ejection, double hit_centrum,
                     double collision_factor, sol_event* out, int32_t capacity, int32_t* n_out);

/* Calculate::Integrals (Solaris/Calculate.cpp:43-62). */
void orc_integrals(const orc_system* s, const double* y0, double out[16]);

/* Ephemeris helpers (Solaris/Ephemeris.cpp). */
int orc_kepler_equation_solver(double e, double m, double eps, double* E);
int orc_calculate_phase(double mu, const double elements[6], double phase[6]);
int orc_calculate_orbital_element(double mu, const double phase[6], double* a, double* e, int32_t quirks);

/* GravityAC restricted to sinks [i_begin, i_end), with n_threads OpenMP
 * threads: the bounded CPU-baseline sample.  Returns the pair count. */
int64_t orc_gravity_ac_sample(orc_system* s, const double* y, int32_t i_begin, int32_t i_end,
                              double* dydt, int32_t n_threads);

/* Jacobian-vector product of GravityAC for a perturbation (dy, dm). */
void orc_jvp(orc_system* s, const double* y, const double* dy, const double* dm, double* df);
/* n fixed-h RKF78 steps (7th-order result); with dy0 (and dm) also the
 * tangent-linear solution. */
int orc_rkf78_fixed(orc_system* s, const double* y0, double h, int32_t n_steps, double* y_out, const double* dy0,
                    const double* dm, double* dy_out);
void orc_set_masses(orc_system* s, const double* mass);

/* Simulator::CheckEvent with RemoveBody and HandleCollision (Simulator.cpp:
 * 621-935) on the last evaluation's rm3 and nearest neighbours: y0 and the
 * system are compacted in place; *n_log affairs (up to cap in log). */
int orc_handle_events(orc_system* s, double time, double ejection, double hit_centrum, double factor, double* y0,
                      sol_affair* log, int32_t cap, int32_t* n_log);
double orc_gas_probe(const sol_gas_component* g, int32_t which, const double* args, double* out3);
int orc_kepler_solve(double e, double m, double eps, int32_t quirks, double* E);
void orc_get_bodies(const orc_system* s, sol_nbodies* counts, int32_t* id, int32_t* type, double* mass,
                    double* radius, double* density);

#ifdef __cplusplus
}
#endif

#endif
