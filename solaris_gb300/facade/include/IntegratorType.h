// Integrator selector of the Solaris class interface (same enumerators and
// order as the reference's IntegratorType.h; numeric values are part of the
// interface and match sol_integrator_type in solaris_gb300.h).
#ifndef INTEGRATORTYPE_H_
#define INTEGRATORTYPE_H_

enum IntegratorType { DORMAND_PRINCE, RUNGE_KUTTA4, RUNGE_KUTTA56, RUNGE_KUTTA_FEHLBERG78 };

#endif
