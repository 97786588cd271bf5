// Acceleration (Solaris/Acceleration.h) on the GB300: every member function
// evaluates on the device through libsolaris_gb300; the members the
// reference leaves on the host (rm3, BodyData::indexOfNN / distanceOfNN /
// migType, the drag and migration side buffers) are filled after each call.
// Compiles against the reference's own headers or against
// solaris_gb300/facade/include.
#include <cstring>

#include "Acceleration.h"
#include "BodyData.h"
#include "Error.h"
#include "facade_state.h"

namespace f = solgb_facade;

#define SOL_FACADE_CHECK(expr)                                  \
  do {                                                          \
    if ((expr) != 0) return f::fail(__FILE__, __func__, __LINE__); \
  } while (0)

Acceleration::Acceleration(IntegratorType iType, bool baryCentric, BodyData* bD, Nebula* n) {
  _integratorType = iType;
  _baryCentric = baryCentric;
  evaluateGasDrag = true;
  evaluateTypeIMigration = true;
  evaluateTypeIIMigration = true;
  bodyData = bD;
  nebula = n;
  rm3 = 0;
  accelGasDrag = 0;
  accelMigrationTypeI = 0;
  accelMigrationTypeII = 0;
  f::attach(this, baryCentric);
}

Acceleration::~Acceleration() {
  f::detach(this);
  delete[] rm3;
  delete[] accelGasDrag;
  delete[] accelMigrationTypeI;
  delete[] accelMigrationTypeII;
}

int Acceleration::Compute(double t, double* y, double* totalAccel) {
  if (rm3 == 0) rm3 = new double[bodyData->nBodies.total]();
  SOL_FACADE_CHECK(_baryCentric ? ComputeBaryCentric(t, y, totalAccel) : ComputeAstroCentric(t, y, totalAccel));
  return 0;
}

int Acceleration::ComputeAstroCentric(double t, double* y, double* totalAccel) {
  SOL_FACADE_CHECK(f::compute(this, false, t, y, totalAccel));
  return 0;
}

int Acceleration::ComputeBaryCentric(double t, double* y, double* totalAccel) {
  SOL_FACADE_CHECK(f::compute(this, true, t, y, totalAccel));
  return 0;
}

int Acceleration::GravityAC(double t, double* y, double* a) {
  SOL_FACADE_CHECK(f::term(this, false, SOL_TERM_GRAVITY, t, y, a));
  return 0;
}

int Acceleration::GasDragAC(double t, double* y, double* a) {
  SOL_FACADE_CHECK(f::term(this, false, SOL_TERM_GAS_DRAG, t, y, a));
  return 0;
}

int Acceleration::MigrationTypeIAC(double t, double* y, double* a) {
  SOL_FACADE_CHECK(f::term(this, false, SOL_TERM_TYPE_I, t, y, a));
  return 0;
}

int Acceleration::MigrationTypeIIAC(double t, double* y, double* a) {
  SOL_FACADE_CHECK(f::term(this, false, SOL_TERM_TYPE_II, t, y, a));
  return 0;
}

int Acceleration::GravityBC(double t, double* y, double* a) {
  SOL_FACADE_CHECK(f::term(this, true, SOL_TERM_GRAVITY, t, y, a));
  return 0;
}

// The massive bodies' rows of GravityBC (Acceleration.cpp:541-588).
int Acceleration::GravityBC_SelfInteracting(double t, double* y, double* a) {
  SOL_FACADE_CHECK(f::term(this, true, SOL_TERM_GRAVITY, t, y, a, 0, bodyData->nBodies.NOfMassive()));
  return 0;
}

// The other bodies' rows (Acceleration.cpp:590-634); they start from zero
// here, where the reference adds onto whatever the caller's array held.
int Acceleration::GravityBC_NonSelfInteracting(double t, double* y, double* a) {
  SOL_FACADE_CHECK(f::term(this, true, SOL_TERM_GRAVITY, t, y, a, bodyData->nBodies.NOfMassive(),
                           bodyData->nBodies.total));
  return 0;
}

int Acceleration::GasDragBC(double t, double* y, double* a) {
  SOL_FACADE_CHECK(f::term(this, true, SOL_TERM_GAS_DRAG, t, y, a));
  return 0;
}

int Acceleration::MigrationTypeIBC(double t, double* y, double* a) {
  SOL_FACADE_CHECK(f::term(this, true, SOL_TERM_TYPE_I, t, y, a));
  return 0;
}

int Acceleration::MigrationTypeIIBC(double t, double* y, double* a) {
  SOL_FACADE_CHECK(f::term(this, true, SOL_TERM_TYPE_II, t, y, a));
  return 0;
}

double Acceleration::TypeIMigrationTime(const double C, const double O, const double ar, const double er,
                                        const double h) {
  const double args[5] = {C, O, ar, er, h};
  return f::helper(this, _baryCentric, SOL_HELPER_TYPE_I_MIGRATION_TIME, args);
}

double Acceleration::TypeIEccentricityDampingTime(const double C, const double O, const double ar, const double er,
                                                  const double h) {
  const double args[5] = {C, O, ar, er, h};
  return f::helper(this, _baryCentric, SOL_HELPER_TYPE_I_ECC_DAMPING_TIME, args);
}

double Acceleration::TauNu(double r, double O) {
  const double args[2] = {r, O};
  return f::helper(this, _baryCentric, SOL_HELPER_TAU_NU, args);
}
