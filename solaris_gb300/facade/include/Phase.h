// Position and velocity of one body (BodyData::phaseOfBC).
#ifndef PHASE_H_
#define PHASE_H_

#include "Vector.h"

class Phase {
 public:
  Phase() : bodyId(0) {}
  explicit Phase(int id) : bodyId(id) {}
  int bodyId;
  Vector position;
  Vector velocity;
};

#endif
