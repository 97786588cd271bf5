// The body-class enumerations of the Solaris class interface (the reference's
// Body.h also defines the Body class of its scenario model, which the
// force-and-integrate path does not use).  Values match sol_body_type and
// sol_migration_type in solaris_gb300.h.
#ifndef BODY_H_
#define BODY_H_

enum BodyType {
  UndefinedBodyType,
  CentralBody,
  GiantPlanet,
  RockyPlanet,
  ProtoPlanet,
  SuperPlanetesimal,
  Planetesimal,
  TestParticle,
  NOfBodyType
};

enum MigrationType { No, TypeI, TypeII };

#endif
