// Standalone NBodies.
#include "NBodies.h"

NBodies::NBodies()
    : centralBody(0), giantPlanet(0), rockyPlanet(0), protoPlanet(0), superPlanetsimal(0), planetsimal(0),
      testParticle(0), total(0), removed(0), threshold(0) {}

int NBodies::NOfMassive() { return centralBody + giantPlanet + rockyPlanet + protoPlanet; }

int NBodies::NOfPlAndSpl() { return superPlanetsimal + planetsimal; }

int NBodies::NOfVar() { return 6 * total; }
