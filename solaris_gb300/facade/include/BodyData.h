// The arrays the integrators and Acceleration work on: per-body parameters
// (structure of arrays), the state y0 and the integrator's work vectors
// (array of structs, x y z vx vy vz per body), bodies sorted by class with the
// central body first.
#ifndef BODYDATA_H_
#define BODYDATA_H_

#include "NBodies.h"
#include "Phase.h"
#include "Vector.h"

class BodyData {
 public:
  BodyData();
  ~BodyData();

  int Allocate();  // all arrays for nBodies.total bodies, zeroed; 1 on failure
  void Free();

  NBodies nBodies;

  double time;
  double h;

  int* id;
  int* type;
  int* migType;
  double* migStopAt;
  int* indexOfNN;  // nearest neighbour of body j: index indexOfNN[j]
  double* distanceOfNN;

  double* mass;
  double* radius;
  double* density;
  double* cD;
  double* gammaStokes;
  double* gammaEpstein;

  double* y0;
  double* y;
  double* yBetterEst;
  double* yscale;
  double* accel;
  double* error;

  double bc[6];
  Phase phaseOfBC;
  Vector angularMomentum[2];
  double kineticEnergy[2];
  double potentialEnergy[2];
  double totalEnergy[2];
  double integrals[16];
};

#endif
