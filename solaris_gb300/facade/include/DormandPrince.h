// Dormand-Prince Runge-Kutta-Nystrom 7(6) driver of the Solaris class
// interface.
#ifndef DORMAND_PRINCE_H_
#define DORMAND_PRINCE_H_

#include <string>

class Acceleration;
class BodyData;
class TimeLine;

class DormandPrince {
 public:
  DormandPrince();

  int Driver(BodyData* bodyData, Acceleration* acceleration, TimeLine* timeLine);
  int Step(BodyData* bodyData, Acceleration* acceleration);
  int Step2(BodyData* bodyData, Acceleration* acceleration);
  double GetErrorMax(int n, const double* yerr);

  std::string name;
  std::string reference;
  double accuracy;
  double epsilon;
};

#endif
