// RungeKutta4 (Solaris/RungeKutta4.h) on the GB300: Driver is one device-side
// step at h = TimeLine::hNext; Step is one step from the BodyData's y0 and
// accel.
#include <cmath>

#include "BodyData.h"
#include "Error.h"
#include "RungeKutta4.h"
#include "facade_state.h"

namespace f = solgb_facade;

RungeKutta4::RungeKutta4() {
  name = "Classical Runge-Kutta 4, GB300 device driver";
  reference = "";
  accuracy = -10.0;
  epsilon = std::pow(10.0, accuracy);
}

int RungeKutta4::Driver(BodyData* bodyData, Acceleration* acceleration, TimeLine* timeLine) {
  if (f::driver(SOL_RUNGE_KUTTA4, epsilon, bodyData, acceleration, timeLine) != 0)
    return f::fail(__FILE__, __func__, __LINE__);
  return 0;
}

int RungeKutta4::Step(BodyData* bodyData, Acceleration* acceleration) {
  if (f::attempt(SOL_RUNGE_KUTTA4, epsilon, bodyData, acceleration) != 0) return f::fail(__FILE__, __func__, __LINE__);
  return 0;
}
