// Standalone BodyData (arrays sized by nBodies.total, zero-initialised).
#include "BodyData.h"

#include <new>

#include "Error.h"

BodyData::BodyData()
    : time(0.0), h(0.0), id(0), type(0), migType(0), migStopAt(0), indexOfNN(0), distanceOfNN(0), mass(0), radius(0),
      density(0), cD(0), gammaStokes(0), gammaEpstein(0), y0(0), y(0), yBetterEst(0), yscale(0), accel(0), error(0) {
  for (int k = 0; k < 6; ++k) bc[k] = 0.0;
  for (int k = 0; k < 2; ++k) kineticEnergy[k] = potentialEnergy[k] = totalEnergy[k] = 0.0;
  for (int k = 0; k < 16; ++k) integrals[k] = 0.0;
}

BodyData::~BodyData() { Free(); }

int BodyData::Allocate() {
  const int n = nBodies.total;
  if (n <= 0) {
    Error::_errMsg = "BodyData::Allocate: no bodies";
    Error::PushLocation(__FILE__, __func__, __LINE__);
    return 1;
  }
  Free();
  const size_t nv = 6 * (size_t)n;
  id = new (std::nothrow) int[n]();
  type = new (std::nothrow) int[n]();
  migType = new (std::nothrow) int[n]();
  indexOfNN = new (std::nothrow) int[n]();
  double** per_body[] = {&migStopAt, &distanceOfNN, &mass, &radius, &density, &cD, &gammaStokes, &gammaEpstein};
  for (double** p : per_body) *p = new (std::nothrow) double[n]();
  double** per_var[] = {&y0, &y, &yBetterEst, &yscale, &accel, &error};
  for (double** p : per_var) *p = new (std::nothrow) double[nv]();
  bool ok = id && type && migType && indexOfNN;
  for (double** p : per_body) ok = ok && *p;
  for (double** p : per_var) ok = ok && *p;
  if (!ok) {
    Free();
    Error::_errMsg = "BodyData::Allocate: host memory allocation";
    Error::PushLocation(__FILE__, __func__, __LINE__);
    return 1;
  }
  return 0;
}

void BodyData::Free() {
  int** ints[] = {&id, &type, &migType, &indexOfNN};
  for (int** p : ints) {
    delete[] *p;
    *p = 0;
  }
  double** dbls[] = {&migStopAt, &distanceOfNN, &mass,   &radius, &density,    &cD,     &gammaStokes,
                     &gammaEpstein, &y0,       &y,      &yBetterEst, &yscale, &accel,  &error};
  for (double** p : dbls) {
    delete[] *p;
    *p = 0;
  }
}
