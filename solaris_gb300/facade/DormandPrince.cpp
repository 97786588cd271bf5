// DormandPrince (Solaris/DormandPrince.h) on the GB300: Driver is one
// device-side driver call (at most 10 attempts, as the reference's maxIter);
// Step2 is one attempt from the BodyData's y0 and accel.  Step, the
// reference's earlier arrangement of the same Runge-Kutta-Nystrom 7(6) stages
// (not called by its Driver), runs the Step2 attempt.
#include <cmath>

#include "BodyData.h"
#include "DormandPrince.h"
#include "Error.h"
#include "facade_state.h"

namespace f = solgb_facade;

DormandPrince::DormandPrince() {
  name = "Dormand-Prince Runge-Kutta-Nystrom 7(6), GB300 device driver";
  reference = "J. R. Dormand, P. J. Prince, Celestial Mechanics 18 (1978) 223-232";
  accuracy = -10.0;
  epsilon = std::pow(10.0, accuracy);
}

int DormandPrince::Driver(BodyData* bodyData, Acceleration* acceleration, TimeLine* timeLine) {
  if (f::driver(SOL_DORMAND_PRINCE, epsilon, bodyData, acceleration, timeLine) != 0)
    return f::fail(__FILE__, __func__, __LINE__);
  return 0;
}

int DormandPrince::Step(BodyData* bodyData, Acceleration* acceleration) { return Step2(bodyData, acceleration); }

int DormandPrince::Step2(BodyData* bodyData, Acceleration* acceleration) {
  if (f::attempt(SOL_DORMAND_PRINCE, epsilon, bodyData, acceleration) != 0)
    return f::fail(__FILE__, __func__, __LINE__);
  return 0;
}

double DormandPrince::GetErrorMax(int n, const double* yerr) {
  return f::error_max(SOL_DORMAND_PRINCE, n, yerr, nullptr, epsilon);
}
