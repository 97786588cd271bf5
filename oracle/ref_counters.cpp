// Counters around the reference program, linked with -Wl,--wrap so that the
// reference's own objects run unchanged: every call of
// RungeKuttaFehlberg78::Driver (one accepted step) and of
// Acceleration::Compute (one force evaluation) from another object file is
// counted, and the totals are printed to stderr at exit.  The reference keeps
// no count of rejected attempts (Counter::failedStep is never incremented);
// with RKF78's 13 evaluations per accepted and 12 per rejected attempt
// (RungeKuttaFehlberg78.cpp:66-250) they follow from these two counts.
#include <cstdio>
#include <cstdlib>

class BodyData;
class Acceleration;
class TimeLine;

static unsigned long long g_drivers = 0, g_evals = 0;

static void report() {
  std::fprintf(stderr, "ref_counters: driver_calls %llu force_evaluations %llu\n", g_drivers, g_evals);
}

static struct Reporter {
  Reporter() { std::atexit(report); }
} g_reporter;

extern "C" {
int __real__ZN12Acceleration7ComputeEdPdS0_(Acceleration* self, double t, double* y, double* dydt);
int __wrap__ZN12Acceleration7ComputeEdPdS0_(Acceleration* self, double t, double* y, double* dydt) {
  ++g_evals;
  return __real__ZN12Acceleration7ComputeEdPdS0_(self, t, y, dydt);
}
int __real__ZN20RungeKuttaFehlberg786DriverEP8BodyDataP12AccelerationP8TimeLine(void* self, BodyData* b,
                                                                               Acceleration* a, TimeLine* tl);
int __wrap__ZN20RungeKuttaFehlberg786DriverEP8BodyDataP12AccelerationP8TimeLine(void* self, BodyData* b,
                                                                               Acceleration* a, TimeLine* tl) {
  ++g_drivers;
  return __real__ZN20RungeKuttaFehlberg786DriverEP8BodyDataP12AccelerationP8TimeLine(self, b, a, tl);
}
}
