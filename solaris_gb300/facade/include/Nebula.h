// The protoplanetary nebula; the force path reads its gas component.
#ifndef NEBULA_H_
#define NEBULA_H_

#include <string>

#include "GasComponent.h"

class Nebula {
 public:
  Nebula() : massFactor(1.0), gasToDustRatio(100.0), snowLine(2.7) {}

  std::string name;
  std::string description;
  std::string file;
  std::string fargoPath;

  double massFactor;
  double gasToDustRatio;
  double snowLine;

  GasComponent gasComponent;
};

#endif
