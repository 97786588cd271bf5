// Integration clock: the drivers read time and hNext and set time, hDid and
// hNext.
#ifndef TIMELINE_H_
#define TIMELINE_H_

class TimeLine {
 public:
  TimeLine();

  bool Forward() { return length >= 0; }

  double start;
  double length;
  double output;
  double save;
  double time;
  int millenium;
  double hNext;
  double hDid;
  double elapsedTime;
  double lastSave;
  double lastNSteps;
  bool startTimeDefined;
};

#endif
