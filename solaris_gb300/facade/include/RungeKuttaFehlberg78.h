// Runge-Kutta-Fehlberg 7(8) driver of the Solaris class interface; each
// Driver call is one device-side driver call of libsolaris_gb300.
#ifndef RUNGEKUTTAFEHLBERG78_H_
#define RUNGEKUTTAFEHLBERG78_H_

#include <string>

class Acceleration;
class BodyData;
class TimeLine;

class RungeKuttaFehlberg78 {
 public:
  RungeKuttaFehlberg78();

  int Driver(BodyData* bodyData, Acceleration* acceleration, TimeLine* timeLine);
  int Step(BodyData* bodyData, Acceleration* acceleration);
  double GetErrorMax(const int n, const double* yerr, const double* yscale);

  std::string name;
  std::string reference;
  double accuracy;
  double epsilon;
};

#endif
