// Standalone GasComponent: the reference constructor's defaults, taken from
// the library (sol_gas_component_init), including the mean-free-path law
// built from the default density.
#include "GasComponent.h"

#include "solaris_gb300.h"

GasComponent::GasComponent() : a(0.0) {
  sol_gas_component g;
  sol_gas_component_init(&g);
  alpha = g.alpha;
  meanMolecularWeight = g.mean_molecular_weight;
  particleDiameter = g.particle_diameter;
  type = (GasDecreaseType)g.decrease_type;
  timeScale = g.time_scale;
  t0 = g.t0;
  t1 = g.t1;
  innerEdge = g.inner_edge;
  eta = PowerLaw(g.eta.c, g.eta.index);
  tau = PowerLaw(g.tau.c, g.tau.index);
  scaleHeight = PowerLaw(g.scale_height.c, g.scale_height.index);
  density = PowerLaw(g.density.c, g.density.index);
  meanFreePath = PowerLaw(g.mean_free_path.c, g.mean_free_path.index);
}
