// Standalone TimeLine: everything starts at zero.
#include "TimeLine.h"

TimeLine::TimeLine()
    : start(0.0), length(0.0), output(0.0), save(0.0), time(0.0), millenium(0), hNext(0.0), hDid(0.0),
      elapsedTime(0.0), lastSave(0.0), lastNSteps(0.0), startTimeDefined(false) {}
