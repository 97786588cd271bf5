// Shared machinery of the C++ class facade: the libsolaris_gb300 contexts
// behind each Acceleration object and the host read-back of everything the
// reference classes leave in host memory after a call.
#ifndef SOLARIS_GB300_FACADE_STATE_H_
#define SOLARIS_GB300_FACADE_STATE_H_

#include <cstdint>

#include "solaris_gb300.h"

class Acceleration;
class BodyData;
class TimeLine;

namespace solgb_facade {

// Registration of an Acceleration (its constructor / destructor).
void attach(const Acceleration* acc, bool barycentric);
void detach(const Acceleration* acc);
bool barycentric_of(const Acceleration* acc);

// Acceleration::Compute / ComputeAstroCentric / ComputeBaryCentric.
int compute(Acceleration* acc, bool barycentric, double t, const double* y, double* dydt);
// One term of Compute (sol_term) into out; for the gravity term only body
// rows [row_begin, row_end) of out and of the nearest-neighbour arrays are
// written (the split of GravityBC into its self- and non-self-interacting
// halves), -1 = all.
int term(Acceleration* acc, bool barycentric, int which, double t, const double* y, double* out, int row_begin = -1,
         int row_end = -1);
// TypeIMigrationTime / TypeIEccentricityDampingTime / TauNu.
double helper(Acceleration* acc, bool barycentric, int which, const double* args);

// RungeKuttaFehlberg78 / RungeKutta4 / DormandPrince ::Driver.
int driver(int integrator, double epsilon, BodyData* bd, Acceleration* acc, TimeLine* tl);
// RungeKuttaFehlberg78::Step, RungeKutta4::Step, DormandPrince::Step2.
int attempt(int integrator, double epsilon, BodyData* bd, Acceleration* acc);
// RungeKuttaFehlberg78::GetErrorMax, DormandPrince::GetErrorMax.
double error_max(int integrator, int n, const double* yerr, const double* yscale, double epsilon);

// Error::_errMsg = the library's message, the location pushed; returns 1.
int fail(const char* file, const char* function, long line);

}  // namespace solgb_facade

#endif
