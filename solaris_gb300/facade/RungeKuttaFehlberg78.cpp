// RungeKuttaFehlberg78 (Solaris/RungeKuttaFehlberg78.h) on the GB300: Driver
// is one device-side driver call (first evaluation, attempts with the
// step-size control on the device, accept); Step is one attempt from the
// BodyData's y0 and accel; GetErrorMax reduces on the device.  BodyData and
// TimeLine are left as the reference leaves them (time, h, accel, yscale,
// error, y0 / y swapped; TimeLine time, hDid, hNext).
#include <cmath>

#include "BodyData.h"
#include "Error.h"
#include "RungeKuttaFehlberg78.h"
#include "facade_state.h"

namespace f = solgb_facade;

RungeKuttaFehlberg78::RungeKuttaFehlberg78() {
  name = "Runge-Kutta-Fehlberg 7(8), GB300 device driver";
  reference = "E. Fehlberg, NASA Technical Report R-287 / R-381";
  accuracy = -10.0;
  epsilon = std::pow(10.0, accuracy);
}

int RungeKuttaFehlberg78::Driver(BodyData* bodyData, Acceleration* acceleration, TimeLine* timeLine) {
  if (f::driver(SOL_RUNGE_KUTTA_FEHLBERG78, epsilon, bodyData, acceleration, timeLine) != 0)
    return f::fail(__FILE__, __func__, __LINE__);
  return 0;
}

int RungeKuttaFehlberg78::Step(BodyData* bodyData, Acceleration* acceleration) {
  if (f::attempt(SOL_RUNGE_KUTTA_FEHLBERG78, epsilon, bodyData, acceleration) != 0)
    return f::fail(__FILE__, __func__, __LINE__);
  return 0;
}

double RungeKuttaFehlberg78::GetErrorMax(const int n, const double* yerr, const double* yscale) {
  return f::error_max(SOL_RUNGE_KUTTA_FEHLBERG78, n, yerr, yscale, epsilon);
}
