// Acceleration of the Solaris class interface, implemented on the GB300 by
// libsolaris_gb300 (solaris_gb300/facade/Acceleration.cpp).  Public members
// are those of the reference class: the evaluate* switches, the nearest-body
// outputs it leaves in BodyData, rm3 and the drag / migration side buffers
// are filled on the host after each call.
#ifndef ACCELERATION_H_
#define ACCELERATION_H_

#include "IntegratorType.h"

class BodyData;
class Nebula;

class Acceleration {
 public:
  Acceleration(IntegratorType iType, bool baryCentric, BodyData* bD, Nebula* n);
  ~Acceleration();

  int Compute(double t, double* y, double* totalAccel);
  int ComputeAstroCentric(double t, double* y, double* totalAccel);
  int ComputeBaryCentric(double t, double* y, double* totalAccel);

  int GravityAC(double t, double* y, double* a);
  int GasDragAC(double t, double* y, double* a);
  int MigrationTypeIAC(double t, double* y, double* a);
  int MigrationTypeIIAC(double t, double* y, double* a);

  int GravityBC(double t, double* y, double* a);
  int GravityBC_SelfInteracting(double t, double* y, double* a);
  int GravityBC_NonSelfInteracting(double t, double* y, double* a);
  int GasDragBC(double t, double* y, double* a);
  int MigrationTypeIBC(double t, double* y, double* a);
  int MigrationTypeIIBC(double t, double* y, double* a);

  double TypeIMigrationTime(const double C, const double O, const double ar, const double er, const double h);
  double TypeIEccentricityDampingTime(const double C, const double O, const double ar, const double er,
                                      const double h);
  double TauNu(double r, double O);

  BodyData* bodyData;
  Nebula* nebula;

  double* accelGasDrag;
  double* accelMigrationTypeI;
  double* accelMigrationTypeII;

  double* rm3;  // 1 / |r_i|^3 of the last heliocentric evaluation

  bool evaluateGasDrag;
  bool evaluateTypeIMigration;
  bool evaluateTypeIIMigration;

 private:
  IntegratorType _integratorType;
  bool _baryCentric;
};

#endif
