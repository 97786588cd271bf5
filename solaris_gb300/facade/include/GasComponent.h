// Gas of the nebula: the data members the force terms read (drag, type-I and
// type-II migration).  The constructor sets the defaults of the reference
// class, taken from sol_gas_component_init.
#ifndef GASCOMPONENT_H_
#define GASCOMPONENT_H_

#include "GasDecreaseType.h"
#include "PowerLaw.h"

class GasComponent {
 public:
  GasComponent();

  double alpha;
  double meanMolecularWeight;
  double particleDiameter;

  GasDecreaseType type;
  double timeScale;
  double t0;
  double t1;
  double innerEdge;
  double a;

  PowerLaw eta;
  PowerLaw tau;
  PowerLaw scaleHeight;
  PowerLaw density;
  PowerLaw meanFreePath;
  PowerLaw temperature;
};

#endif
