/*
 * solaris_gb300.h - C-ABI of the GB300 force-and-integrate engine for the
 * Solaris planetary N-body simulator.
 *
 * Every entry point returns an int status (SOL_OK == 0), mirroring the
 * reference's "return 0 = OK, 1 = error" convention (Solaris/Error.h,
 * HANDLE_RESULT in Solaris/Acceleration.cpp:24-28); the message of the last
 * failure on the calling thread is available from sol_last_error().  No C++
 * exception crosses this boundary.  All pointers are plain host pointers
 * unless the name says "_device"; host pointers are borrowed for the call
 * only.  Device buffers are owned by the context.
 *
 * State layout at the boundary is the reference's: y[6N] array-of-structs
 * (x, y, z, vx, vy, vz per body), bodies sorted by BodyType with the central
 * body at index 0 (Solaris/BodyData.h:37-42, Solaris/Simulator.cpp:449-483).
 */
#ifndef SOLARIS_GB300_H_
#define SOLARIS_GB300_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
enum sol_status {
  SOL_OK = 0,
  SOL_ERR_ARG = 1,        /* invalid argument (null pointer, bad count, ...)   */
  SOL_ERR_CUDA = 2,       /* CUDA runtime error                                */
  SOL_ERR_NAN = 3,        /* non-finite value detected on the device          */
  SOL_ERR_UNDERFLOW = 4,  /* step-size underflow (RungeKuttaFehlberg78.cpp:116-122) */
  SOL_ERR_TIMEOUT = 5,    /* a bounded device wait ran out                     */
  SOL_ERR_MAXITER = 6,    /* Dormand-Prince retry limit (DormandPrince.cpp:158-162) */
  SOL_ERR_NOMEM = 7,      /* device allocation failed                          */
  SOL_ERR_STATE = 8,      /* call not valid in the context's current state     */
  SOL_ERR_ORBIT = 9       /* unbound orbit where elements are required (Ephemeris.cpp:16-21) */
};

/* ---- body classes: numeric values of BodyType (Solaris/Body.h:231-241) -- */
enum sol_body_type {
  SOL_UNDEFINED_BODY_TYPE = 0,
  SOL_CENTRAL_BODY = 1,
  SOL_GIANT_PLANET = 2,
  SOL_ROCKY_PLANET = 3,
  SOL_PROTO_PLANET = 4,
  SOL_SUPER_PLANETESIMAL = 5,
  SOL_PLANETESIMAL = 6,
  SOL_TEST_PARTICLE = 7
};

/* MigrationType (Solaris/Body.h:252-256) */
enum sol_migration_type { SOL_MIGRATION_NO = 0, SOL_MIGRATION_TYPE_I = 1, SOL_MIGRATION_TYPE_II = 2 };

/* GasDecreaseType (Solaris/GasDecreaseType.h) */
enum sol_gas_decrease_type { SOL_GAS_CONSTANT = 0, SOL_GAS_LINEAR = 1, SOL_GAS_EXPONENTIAL = 2 };

/* IntegratorType (Solaris/IntegratorType.h) */
enum sol_integrator_type {
  SOL_DORMAND_PRINCE = 0,
  SOL_RUNGE_KUTTA4 = 1,
  SOL_RUNGE_KUTTA56 = 2, /* declared by the reference, never implemented */
  SOL_RUNGE_KUTTA_FEHLBERG78 = 3
};

/* Pair-force arithmetic.
 *  FP64:  plain FP64 in the reference's form: IEEE sqrt and division, no
 *         contraction, the operation order of GravityAC
 *         (Solaris/Acceleration.cpp:248-329).  Bit-identical to the reference
 *         CPU build.
 *  SPLIT: FP64 displacement and r^2; 1/r^3 from an FP32 rsqrt seed plus one
 *         FP64 Newton correction (carried to second order in the residual);
 *         per-tile partial sums folded with compensated two-sum.  Relative
 *         acceleration error against FP64 well below 1e-12.
 *  SPLIT_FF: the displacement stays FP64 (3 FP64 instructions per pair); r^2,
 *         the FP32 rsqrt seed with its Newton correction, G m r^-3 and the
 *         accumulation run in float-float (pairs of FP32 numbers, ~48-bit
 *         significand) on the FP32 pipe; tile sums are folded into FP64.
 *         Same 1e-12 relative bound; requires pair distances above 1e-12 AU
 *         for the float-float branch (closer pairs fall back to FP64).       */
enum sol_precision { SOL_PRECISION_FP64 = 0, SOL_PRECISION_SPLIT = 1, SOL_PRECISION_SPLIT_FF = 2 };

/* Acceleration::evaluate* switches (Solaris/Acceleration.h:375-377) */
#define SOL_EVAL_GAS_DRAG 1u
#define SOL_EVAL_TYPE_I 2u
#define SOL_EVAL_TYPE_II 4u
#define SOL_EVAL_ALL 7u

/* Behaviours of the reference g++ build that a faithful replacement must
 * reproduce.  sol_gas_component_init() sets SOL_QUIRKS_REFERENCE.
 *  INT_ABS:      abs(double) binds to int abs() (Acceleration.cpp:770 and
 *                Ephemeris.cpp:30): |index| and the e^2 clamp use the
 *                truncated integer value.
 *  BC_TAU_NU:    barycentric type-II damping uses TauNu, heliocentric uses
 *                1/TauNu (Acceleration.cpp:518 vs :754).                    */
#define SOL_QUIRK_INT_ABS 1u
#define SOL_QUIRK_BC_TAU_NU 2u
#define SOL_QUIRKS_REFERENCE (SOL_QUIRK_INT_ABS | SOL_QUIRK_BC_TAU_NU)

/* ---- data model --------------------------------------------------------- */

/* NBodies (Solaris/NBodies.h:62-88): counts per body class. */
typedef struct sol_nbodies {
  int32_t central_body;
  int32_t giant_planet;
  int32_t rocky_planet;
  int32_t proto_planet;
  int32_t super_planetesimal;
  int32_t planetesimal;
  int32_t test_particle;
} sol_nbodies;

/* Per-body parameters of BodyData (Solaris/BodyData.h:22-35).  Arrays have
 * total = sum of the counts entries; bodies are sorted by type.  Any of
 * radius/density/cd/gamma_* may be NULL when no nebula is used. */
typedef struct sol_body_data {
  sol_nbodies n;
  const int32_t* id;
  const int32_t* type;
  const int32_t* mig_type;
  const double* mig_stop_at;
  const double* mass;
  const double* radius;
  const double* density;
  const double* cd;
  const double* gamma_stokes;
  const double* gamma_epstein;
} sol_body_data;

/* PowerLaw (Solaris/PowerLaw.h): c * x^index. */
typedef struct sol_power_law {
  double c;
  double index;
} sol_power_law;

/* GasComponent (Solaris/GasComponent.h:251-295). */
typedef struct sol_gas_component {
  double alpha;
  int32_t decrease_type; /* sol_gas_decrease_type */
  int32_t quirks;        /* SOL_QUIRK_* bits */
  double time_scale;
  double t0;
  double t1;
  double inner_edge;
  double mean_molecular_weight;
  double particle_diameter;
  sol_power_law eta;
  sol_power_law tau;
  sol_power_law scale_height;
  sol_power_law density;
  sol_power_law mean_free_path;
} sol_gas_component;

/* TimeLine subset used by the integrator drivers (Solaris/TimeLine.h). */
typedef struct sol_time_line {
  double time;
  double h_next;
  double h_did;
} sol_time_line;

/* Counters of a driver call sequence. */
typedef struct sol_step_stats {
  int64_t accepted;   /* steps accepted (Counter::succededStep) */
  int64_t rejected;   /* attempts rejected by the error control */
  int64_t evaluations;/* force evaluations */
} sol_step_stats;

/* Event kinds of Simulator::CheckEvent (Solaris/Simulator.cpp:621-735). */
enum sol_event_kind { SOL_EVENT_EJECTION = 1, SOL_EVENT_HIT_CENTRUM = 2, SOL_EVENT_COLLISION = 3 };

typedef struct sol_event {
  int32_t kind;  /* sol_event_kind */
  int32_t idx1;  /* body index (0 = central body for ejection / hit-centrum) */
  int32_t idx2;  /* body index of the other body */
  int32_t pad;
  double distance; /* |r| for ejection / hit-centrum, NN distance for collision */
} sol_event;

typedef struct sol_ctx sol_ctx;

/* ---- utilities ---------------------------------------------------------- */
const char* sol_last_error(void);
int sol_version(void);
/* Fill a GasComponent with the constructor defaults of
 * GasComponent::GasComponent() (Solaris/GasComponent.cpp:9-34), including the
 * mean-free-path power law built from the default density. */
int sol_gas_component_init(sol_gas_component* gas);

/* ---- context: replaces `new Acceleration(type, baryCentric, &bodyData, nebula)`
 * (Solaris/Simulator.cpp:82, Solaris/Acceleration.cpp:35-50). ------------ */
int sol_create(const sol_body_data* bodies, const sol_gas_component* gas_or_null,
               int32_t barycentric, int32_t device, sol_ctx** out);
int sol_destroy(sol_ctx* ctx);
/* sol_precision; a barycentric context (GravityBC_*, FP64 only) rejects the
 * split forms with SOL_ERR_ARG. */
int sol_set_precision(sol_ctx* ctx, int32_t precision);
/* Acceleration::evaluateGasDrag / evaluateTypeIMigration / evaluateTypeIIMigration */
int sol_set_eval_flags(sol_ctx* ctx, uint32_t flags);
int sol_get_n_total(const sol_ctx* ctx, int32_t* n);

/* Acceleration::Compute(t, y, dydt) (Solaris/Acceleration.h:19,
 * Solaris/Acceleration.cpp:60-80) with host buffers.  rm3, nn_idx, nn_dist
 * (N entries each) receive Acceleration::rm3 and BodyData::indexOfNN /
 * distanceOfNN; any of them may be NULL.  Migration side effects on
 * BodyData::migType are kept in the context (sol_get_mig_type). */
int sol_accel_compute(sol_ctx* ctx, double t, const double* y, double* dydt,
                      double* rm3, int32_t* nn_idx, double* nn_dist);
int sol_get_mig_type(const sol_ctx* ctx, int32_t* mig_type);

/* Acceleration::Compute for the sinks [sink_begin, sink_end) only, on device
 * buffers (a rank's block of a system whose sinks are partitioned over
 * GPUs): d_y[6N] holds every body's state (every position is a source; a
 * sink's own velocity is read), rows [sink_begin, sink_end) of d_dydt[6N]
 * receive that sink's velocity and acceleration as Compute writes them, the
 * other rows are untouched; rm3 and the nearest neighbours of those sinks
 * are kept (sol_get_last_eval).  Enqueued on the context's stream
 * (sol_get_stream) without waiting.  Heliocentric contexts; the context's
 * precision and evaluate flags.  The reference evaluates every sink in one
 * call (Solaris/Acceleration.cpp:248-329, the loop over i); the result rows
 * are the same. */
int sol_accel_sinks_device(sol_ctx* ctx, double t, const double* d_y, int32_t sink_begin, int32_t sink_end,
                           double* d_dydt);

/* ---- integrators: RungeKuttaFehlberg78::Driver, RungeKutta4::Driver,
 * DormandPrince::Driver (Solaris/RungeKuttaFehlberg78.h:22, RungeKutta4.h:15,
 * DormandPrince.h:14).  Each call performs n_steps driver calls on the
 * context's resident state with device-side step control and no host
 * round trip per attempt. ---------------------------------------------- */
int sol_set_state(sol_ctx* ctx, const double* y0);   /* host y0[6N] -> device */
int sol_get_state(sol_ctx* ctx, double* y0);         /* device -> host y0[6N] */
int sol_set_tolerance(sol_ctx* ctx, double epsilon); /* RKF78/DP epsilon (1e-10 by default) */
/* RKF78 / DP driver calls run as one CUDA graph each, whose attempt loop is a
 * device-side conditional WHILE node (default, enable = 1), or with the host
 * reading the control block after every attempt (enable = 0).  Results are
 * identical. */
int sol_set_device_loop(sol_ctx* ctx, int32_t enable);
int sol_driver(sol_ctx* ctx, int32_t integrator, sol_time_line* tl, int32_t n_steps,
               sol_step_stats* stats);
/* Convenience: host y0 in, host y0 out around sol_driver. */
int sol_driver_host(sol_ctx* ctx, int32_t integrator, double* y0, sol_time_line* tl,
                    int32_t n_steps, sol_step_stats* stats);
/* One RKF78 attempt at fixed h from y0 (RungeKuttaFehlberg78::Step and
 * GetErrorMax, :147-262), with the Driver's evaluate-flag protocol (:74-95). */
int sol_rkf78_step(sol_ctx* ctx, double t, double h, const double* y0, double* y,
                   double* error, double* error_max);
/* Per-body outputs of the last force evaluation (rm3, NN arrays). */
int sol_get_last_eval(sol_ctx* ctx, double* rm3, int32_t* nn_idx, double* nn_dist);

/* ---- the remaining public members of Acceleration and the integrators ----
 * (Solaris/Acceleration.h:17-45, RungeKuttaFehlberg78.h:17-24,
 * RungeKutta4.h:11-17, DormandPrince.h:10-18), used by the C++ class facade
 * (solaris_gb300/facade). */
enum sol_term {
  SOL_TERM_GRAVITY = 0,  /* GravityAC / GravityBC (Acceleration.cpp:248-329, :541-634) */
  SOL_TERM_GAS_DRAG = 1, /* GasDragAC / GasDragBC (:331-422) */
  SOL_TERM_TYPE_I = 2,   /* MigrationTypeIAC / MigrationTypeIBC (:424-485) */
  SOL_TERM_TYPE_II = 3   /* MigrationTypeIIAC / MigrationTypeIIBC (:487-528) */
};
/* One term of Acceleration::Compute on host buffers, in the context's frame.
 * GRAVITY: out[6N] (velocities and gravity, no nebula terms); rm3 and the NN
 *   arrays are then those of this evaluation (sol_get_last_eval).
 * GAS_DRAG: out[3 (superPlanetesimal + planetesimal)], rows of the bodies
 *   from NOfMassive on.
 * TYPE_I: out[3 (rockyPlanet + protoPlanet)], rows of the bodies from
 *   centralBody + giantPlanet on; TYPE_II: out[3 giantPlanet], rows from
 *   centralBody on.  Rows of bodies whose migType is another type keep the
 *   caller's values; a body inside migStopAt gets zeros and migType No.
 * Requires a nebula except for GRAVITY. */
int sol_accel_term(sol_ctx* ctx, int32_t term, double t, const double* y, double* out);

enum sol_helper {
  SOL_HELPER_TYPE_I_MIGRATION_TIME = 0,   /* TypeIMigrationTime(C, O, ar, er, h), Acceleration.cpp:766-777 */
  SOL_HELPER_TYPE_I_ECC_DAMPING_TIME = 1, /* TypeIEccentricityDampingTime(C, O, ar, er, h), :779-789 */
  SOL_HELPER_TAU_NU = 2                   /* TauNu(r, O), :831-849 */
};
/* The scalar helpers of Acceleration with the context's nebula; args holds
 * the reference arguments in order (5, or 2 for TauNu). */
int sol_migration_helper(sol_ctx* ctx, int32_t which, const double* args, double* out);

/* RungeKuttaFehlberg78::GetErrorMax(n, yerr, yscale) = max |yerr/yscale| /
 * epsilon (RungeKuttaFehlberg78.cpp:252-262) or DormandPrince::GetErrorMax(n,
 * yerr) = max |yerr| (DormandPrince.cpp:493-503) on host arrays of n
 * entries (n <= 6N with a context; ctx may be NULL, as the reference's
 * GetErrorMax has no Acceleration: the current device is used); NaN entries
 * never become the maximum, as in the reference's comparison.  yscale and
 * epsilon are ignored for DormandPrince. */
int sol_error_max(sol_ctx* ctx, int32_t integrator, int32_t n, const double* yerr, const double* yscale,
                  double epsilon, double* out);

/* One attempt of RungeKuttaFehlberg78::Step (:147-250), RungeKutta4::Step
 * (RungeKutta4.cpp:58-129) or DormandPrince::Step2 (DormandPrince.cpp:246-491)
 * from host y0 at (t, h), with f0 = BodyData::accel given by the caller and,
 * for RKF78, BodyData::yscale (NULL: the Driver's yscale from y0, f0 and h).
 * The stage evaluations use the context's evaluate flags (sol_set_eval_flags).
 * Writes y[6N], error[6N] (RKF78 and DP; may be NULL) and error_max (the
 * integrator's GetErrorMax; 0 for RK4).  The context's resident state
 * becomes y0. */
int sol_integrator_attempt(sol_ctx* ctx, int32_t integrator, double t, double h, const double* y0,
                           const double* f0, const double* yscale, double* y, double* error, double* error_max);

/* What the last driver call or attempt leaves in BodyData: accel (f0 of the
 * step), yscale and error (of the last attempt), 6N entries each; NULL skips. */
int sol_get_driver_vectors(sol_ctx* ctx, double* accel, double* yscale, double* error);
/* Acceleration's persistent side buffers accelGasDrag[3 (superPlanetesimal +
 * planetesimal)], accelMigrationTypeI[3 (rockyPlanet + protoPlanet)] and
 * accelMigrationTypeII[3 giantPlanet] (Acceleration.cpp:176-243); NULL skips. */
int sol_get_side_buffers(sol_ctx* ctx, double* drag, double* mig1, double* mig2);

/* ---- events: predicates of Simulator::CheckEvent (Solaris/Simulator.cpp:626-645,
 * :690-729) evaluated on the device from the last force evaluation. ------ */
int sol_check_events(sol_ctx* ctx, double ejection, double hit_centrum, double collision_factor,
                     sol_event* out, int32_t capacity, int32_t* n_out);

/* ---- diagnostics: Calculate::Integrals (Solaris/Calculate.cpp:43-62). ---
 * The 16 values of the reference's integrals record for the context's state
 * (or y0_or_null).  Up to 1,024 bodies the potential energy is the
 * reference's single running sum over ordered pairs, bit for bit (on the
 * host); above, the device evaluates each unordered pair once (1/r from an
 * FP32 seed and an FP64 Newton step) into per-CTA partials that the host adds
 * in order: deterministic and within ~1e-13 relative of the exact sum, but
 * not the reference's rounding.  Coincident bodies give +inf (NaN where one
 * of the two masses is 0), as the reference's m_i m_j / 0. */
int sol_integrals(sol_ctx* ctx, const double* y0_or_null, double integrals[16]);

/* ---- output files: BinaryFileAdapter (Solaris/BinaryFileAdapter.cpp:107-219)
 * Phases: per record double time, int32 n, then per body int32 id and the 6
 * doubles of y0 (binary), or the reference's text layout (setw(15)
 * setprecision(10) time, setw(8) n, per body setw(8) id and setw(15)
 * setprecision(6) values, end of line).  Integrals: a length-prefixed header
 * at the start of the file, then per record int32 (n + 1), double time and
 * the 16 doubles of Calculate::Integrals.  Records are appended. ----------- */
typedef struct sol_output sol_output;
/* Either path may be NULL (that file is not written).  An integrals file
 * gets the header when it is empty at open. */
int sol_output_open(sol_ctx* ctx, const char* phases_path, const char* integrals_path, int32_t text,
                    sol_output** out);
/* Appends the context's resident state (Simulator: SavePhases(time, n, y0, id)).
 * Costs the compute stream one device copy; the host copy and the write run
 * on a copy stream and a writer thread while the integration continues. */
int sol_output_save_phases(sol_output* out, double time);
/* Calculate::Integrals of the resident state (O(N^2) potential on the device)
 * and SaveIntegrals(time, 16, integrals). */
int sol_output_save_integrals(sol_output* out, double time);
int sol_output_flush(sol_output* out); /* every queued record on disk */
int sol_output_close(sol_output* out);
/* The records themselves, host only (length = bytes; buf NULL asks for it). */
int sol_format_phases_record(double time, int32_t n, const double* y, const int32_t* id, int32_t text, char* buf,
                             int64_t capacity, int64_t* length);
int sol_format_integrals_record(double time, int32_t n, const double* integrals, int32_t header, char* buf,
                                int64_t capacity, int64_t* length);

/* ---- events on the device: Simulator::CheckEvent (Solaris/Simulator.cpp:
 * 621-735) with RemoveBody (:737-771) and HandleCollision (:773-935) --------- */
/* TwoBodyAffair (Solaris/TwoBodyAffair.h): type is the reference's EventType
 * (0 ejection, 1 hit centrum, 3 collision); idx1/idx2 the bodies' indices
 * (ejection and hit centrum: before any removal; collision: among the bodies
 * present at that moment, survivor first); phases before a merge. */
typedef struct sol_affair {
  int32_t type;
  int32_t idx1, idx2;
  int32_t id1, id2;
  int32_t pad;
  double time;
  double phase1[6];
  double phase2[6];
} sol_affair;
/* After a driver call (the last evaluation's rm3 and nearest neighbours):
 * every body with rm3 < 1/ejection^3 is logged and removed; every body with
 * rm3 > 1/hit_centrum^3 is merged into the central body and removed; then,
 * in body order, a body whose nearest neighbour j satisfies
 * collision_factor * (R_i + R_j) > distance merges with it (the lighter into
 * the heavier, equal masses into the lower index; mass and momentum add up,
 * radius from the summed volume) and the merger is removed.  A parameter <= 0
 * turns that event off.  The context's bodies are compacted on the device
 * (counts, parameters, state, side buffers); nearest neighbours are cleared
 * until the next evaluation.  log receives up to capacity affairs, *n_log
 * their number.  Bodies are identified by id where the reference uses
 * indices that earlier removals have shifted. */
int sol_handle_events(sol_ctx* ctx, double time, double ejection, double hit_centrum, double collision_factor,
                      sol_affair* log, int32_t capacity, int32_t* n_log);
/* The context's body set: counts, ids, types and the (possibly merged)
 * mass, radius and density; any pointer may be NULL. */
int sol_get_bodies(sol_ctx* ctx, sol_nbodies* counts, int32_t* id, int32_t* type, double* mass, double* radius,
                   double* density);
/* SaveTwoBodyAffair (Solaris/BinaryFileAdapter.cpp:244-261): appends n
 * records (int32 event id = first_event_id + k, int32 type, int32 body ids,
 * 6 + 6 doubles of phases, double time) to path. */
int sol_write_affairs(const char* path, const sol_affair* affairs, int32_t n, int32_t first_event_id);

/* ---- the Simulator's step loop between host work ---------------------------
 * Simulator::Integrate / DecisionMaking (Solaris/Simulator.cpp:121-250) for
 * the steps at which the host has nothing to do.  After each accepted driver
 * step: steps += 1, elapsed and last_save += h_did; then
 *   SOL_STOP_EVENT  when an event predicate of CheckEvent holds on the step's
 *                   last evaluation (rm3 < 1 / R_ej^3, rm3 > 1 / R_hc^3,
 *                   factor (R_i + R_NN) > d_NN; a parameter <= 0 is off):
 *                   the rest of DecisionMaking is the host's;
 *   SOL_STOP_LENGTH when |clock| >= |length| (clock: time, or elapsed when
 *                   relative_end != 0);
 * otherwise h_next is clamped to the end of the phase, then
 *   SOL_STOP_OUTPUT when |last_save| >= |output| (a record is due; the host
 *                   saves, sets last_save = 0 and clamps h_next to the next
 *                   output);
 * otherwise h_next is clamped to the next output and, every 100 steps of the
 * run (steps % 100 == 0), state components below 1e-50 are set to zero
 * (Tools::CheckAgainstSmallestNumber); after max_steps such steps
 * SOL_STOP_STEPS.  The stopping step's smallest-number flush is the host's. */
typedef struct sol_sim_line {
  double time, length, output;
  double h_next, h_did;
  double elapsed, last_save;
  int64_t steps;
  int32_t relative_end, pad;
} sol_sim_line;
enum { SOL_STOP_STEPS = 0, SOL_STOP_EVENT = 1, SOL_STOP_LENGTH = 2, SOL_STOP_OUTPUT = 3 };
int sol_run_until(sol_ctx* ctx, int32_t integrator, sol_sim_line* line, int32_t max_steps, double ejection,
                  double hit_centrum, double collision_factor, int32_t* reason, sol_step_stats* stats);
/* Tools::CheckAgainstSmallestNumber on the resident state: |y| < 1e-50 -> 0. */
int sol_flush_smallest(sol_ctx* ctx);
/* After sol_run_until with collision_factor > 0: the state at the start of
 * the last step (bodyData.y after the swap, which the reference's collision
 * records carry), 6N doubles. */
int sol_get_step_start(sol_ctx* ctx, double* y);

/* ---- initial conditions in bulk ------------------------------------------
 * Ephemeris::CalculatePhase with Ephemeris::KeplerEquationSolver
 * (Solaris/Ephemeris.cpp:141-211) for n bodies on the device, one thread per
 * body: elements[6n] = {a, e, i, argument of pericentre, longitude of node,
 * mean anomaly} per body, mu[n] = G (m0 + m), phases[6n] = x y z vx vy vz.
 * quirks: SOL_QUIRK_INT_ABS reproduces the reference build's stopping rule of
 * the Kepler iteration (|change| through int abs(), so it stops once below 1);
 * 0 iterates to 1e-14.  status[n] (may be NULL): SOL_OK or SOL_ERR_ORBIT where
 * the iteration did not converge in 25 steps. */
int sol_phases_from_elements(int32_t device, int32_t n, const double* mu, const double* elements, int32_t quirks,
                             double* phases, int32_t* status);

/* ---- discrete adjoint of fixed-step RKF78 --------------------------------
 * Forward: n_steps RungeKuttaFehlberg78::Step calls at constant h, each taking
 * the 7th-order result (RungeKuttaFehlberg78.cpp:147-250; heliocentric
 * gravity, no nebula), the state stored every `checkpoint_every` steps.
 * Backward: given dL/dy at the final state, dL/dy0 (6N) and dL/dmass (N) of
 * that discrete map, recomputing each segment from its checkpoint.  A
 * torch.autograd.Function-style pair: forward once, then backward. */
int sol_adjoint_forward(sol_ctx* ctx, double h, int32_t n_steps, int32_t checkpoint_every, const double* y0,
                        double* y_final);
int sol_adjoint_backward(sol_ctx* ctx, const double* dl_dy_final, double* dl_dy0, double* dl_dmass);
/* Replace the body masses (BodyData::mass) of a context. */
int sol_set_masses(sol_ctx* ctx, const double* mass);

/* ---- batched ensembles ---------------------------------------------------
 * Many independent systems (no nebula, heliocentric), each advanced by its
 * own adaptive RungeKuttaFehlberg78 driver calls (RungeKuttaFehlberg78.cpp:
 * 66-262) in one persistent launch: a CTA runs whole driver calls of one
 * system at a time, taking systems from a work queue.  State is the
 * concatenation of the systems' y[6N] arrays in the order given. */
typedef struct sol_ensemble sol_ensemble;
int sol_ensemble_create(const sol_body_data* systems, int32_t n_systems, int32_t device, sol_ensemble** out);
int sol_ensemble_destroy(sol_ensemble* ens);
/* SOL_PRECISION_FP64 (the reference's arithmetic) or SOL_PRECISION_SPLIT_FF */
int sol_ensemble_set_precision(sol_ensemble* ens, int32_t precision);
int sol_ensemble_set_tolerance(sol_ensemble* ens, double epsilon);
int sol_ensemble_set_state(sol_ensemble* ens, const double* y0_all, const sol_time_line* time_lines);
/* any output may be NULL; status[s] is SOL_OK or SOL_ERR_UNDERFLOW per system */
int sol_ensemble_get_state(sol_ensemble* ens, double* y0_all, sol_time_line* time_lines, int32_t* status);
/* n_steps driver calls for every system */
int sol_ensemble_advance(sol_ensemble* ens, int32_t n_steps, sol_step_stats* stats);
/* launch shape: threads per system (multiple of 32) and resident systems per SM */
int sol_ensemble_configure(sol_ensemble* ens, int32_t threads_per_system, int32_t systems_per_sm);
/* times `steps` driver calls for each candidate launch shape on a copy of the
 * state, restores the state and keeps the fastest shape */
int sol_ensemble_autotune(sol_ensemble* ens, int32_t steps, int32_t* threads_per_system, int32_t* systems_per_sm,
                          double* best_ms);

/* ---- caller-allocated force evaluation --------------------------------- */
/* GravityAC alone (no gas terms) for callers that cannot allocate device
 * memory: a host framework that owns every device byte, a plugin with a fixed
 * memory budget, or a real-time loop where cudaMalloc would stall.  This entry
 * point has no counterpart in the reference.  It calls no cudaMalloc,
 * cudaFree or allocating library routine: all inputs and outputs are device
 * pointers the caller owns (type[N], mass[N], y[6N] in; dydt[6N], rm3[N],
 * nn_idx[N], nn_dist[N] out), and its scratch is a fixed array inside the
 * library (about 1 MiB per device, kept until the process exits), so N is
 * limited to 16,384 bodies; larger N returns SOL_ERR_ARG.  The first call on
 * a device resolves that array's device address and should come before any
 * stream capture.  Work is enqueued on `stream` (a cudaStream_t, NULL for
 * the default stream) asynchronously.  Every call shares the one array:
 * calls whose work overlaps on the GPU (other streams, other host threads)
 * race and must be serialised by the caller. */
int sol_gravity_noalloc(const sol_nbodies* counts, const int32_t* d_type, const double* d_mass,
                        const double* d_y, double* d_dydt, double* d_rm3, int32_t* d_nn_idx,
                        double* d_nn_dist, int32_t precision, void* stream);

/* The status of the last sol_gravity_noalloc call on the current device,
 * read after the work queued on `stream` has finished (this call waits for
 * that stream): SOL_OK, or SOL_ERR_TIMEOUT when a bounded wait of that
 * evaluation ran out, in which case its outputs are incomplete.  *status
 * (may be NULL) receives the raw device status word.  Allocates nothing.
 * No counterpart in the reference. */
int sol_gravity_noalloc_status(void* stream, int32_t* status);

/* ---- failure-path test hooks --------------------------------------------
 * Every device wait (a bulk copy's mbarrier phase, the group driver's
 * barrier) polls at most a spin limit of times; a wait that runs out raises
 * SOL_DEV_TIMEOUT and the call returns SOL_ERR_TIMEOUT, leaving the context
 * usable.  This hook lets a test reach that path without faulting anything:
 * spin_limit bounds the waits (0: the default of 2^26 polls) and withhold >= 0
 * names a participant that never arrives (-1: none).
 *  ctx != NULL: the context's group driver (few-source RKF78 / RK4 systems in
 *    sol_driver and sol_run_until): CTA `withhold` skips its arrivals at the
 *    group barrier, so the other CTAs' waits run out.
 *  ctx == NULL: sol_gravity_noalloc, process-wide: source tile `withhold` of
 *    every CTA is never copied, so the wait for it runs out.
 * No counterpart in the reference. */
int sol_set_wait_test(sol_ctx* ctx, uint32_t spin_limit, int32_t withhold);

/* ---- measurement helpers ------------------------------------------------ */
/* Measured FP64 fused-multiply-add throughput of this GPU in FLOP/s (FMA = 2):
 * twice rates[0] of sol_measure_fp64_pipe. */
int sol_measure_fp64_peak(int32_t device, double* flops);
/* Measured FP64 pipe throughput in thread instructions per second:
 * rates[0] DFMA, rates[1] DADD, rates[2] DMUL, each from 16 independent
 * chains per thread on a grid of exactly the CTAs the SMs hold at once (best
 * of 5 launches of ~50 ms); sm_mhz (may be NULL) receives the SM clock during
 * the fastest DFMA launch (SM cycles over %globaltimer nanoseconds in one
 * CTA).  On the GB300 such chains reach 84% of the FP64 pipe's issue rate
 * (1/16 warp instruction per SM cycle). */
int sol_measure_fp64_pipe(int32_t device, double rates[3], double* sm_mhz);
/* Measured FP32 pipe throughput in FP32 lane operations per second (an FMA
 * is one): rates[0] scalar FFMA chains, rates[1] paired FFMA2 chains (two
 * lanes per instruction), set up as sol_measure_fp64_pipe's; sm_mhz (may be
 * NULL) the SM clock of the fastest FFMA2 launch. */
int sol_measure_fp32_pipe(int32_t device, double rates[2], double* sm_mhz);
/* Self-check of the reference-form pair arithmetic: the correctly rounded
 * sqrt(a) and 1 / (a sqrt(a)) that replace IEEE square root and division in
 * every FP64 GravityAC pair (Acceleration.cpp:294-317), and the integer-pipe
 * multiply of its terms, compared bit for bit with the FP64 instructions on
 * n seeded samples of one input family
 * (mode 0: a log-uniform over [2^-200, 2^200]; 1: square roots within
 * 2^-13 ulp of a midpoint; 2: squared distances in a 100 AU box; 3:
 * reciprocals within 2^-12 ulp of a midpoint from approximations up to 300
 * ulps off; 4: log-uniform reciprocals from such approximations; 5: square
 * roots and reciprocals next to powers of two; 6: the integer-pipe double
 * multiply of the pair terms against the FP64 instruction, random operands;
 * 7: the same next to the normalisation boundaries, zeros and squares;
 * 8, 9: the RKF78 step-size control's errorMax^-1/5 and errorMax^-1/4,
 * checked for correct rounding by the sign of em t^N - 1 at the midpoints
 * around each result).
 * result[0] = samples whose fast path disagrees (0 when correct),
 * result[1] = samples the fast path hands to IEEE sqrt and division,
 * result[2] = the first disagreeing sample's index, or -1. */
int sol_check_pair_math(int32_t device, int32_t mode, int64_t n, uint64_t seed, int64_t result[3]);
/* Number of kernels this library launched since load. */
int sol_kernel_launch_count(int64_t* count);
/* The CUDA stream (cudaStream_t) every kernel of this context is launched on. */
int sol_get_stream(sol_ctx* ctx, void** stream);
/* Average duration in milliseconds of one launch of the pair kernel alone
 * (no prepass), over `reps` launches on the context's resident state, timed
 * with CUDA events on the context's stream. */
int sol_bench_force(sol_ctx* ctx, int32_t precision, int32_t reps, double* ms_per_launch);
/* Average duration in milliseconds of the elementwise kernels of one RKF78
 * attempt alone (12 stage sums, the final sum with the error estimate and its
 * scaled norm, the norm reduction) over the context's stage vectors:
 * 8 * 6N * 93 bytes of algorithmic HBM traffic per attempt. */
int sol_bench_stages(sol_ctx* ctx, int32_t reps, double* ms_per_attempt);

#ifdef __cplusplus
}
#endif

#endif /* SOLARIS_GB300_H_ */
