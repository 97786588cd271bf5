// Number of bodies per class.  Bodies are stored sorted by class in this
// order; the massive classes (central body, giant, rocky and proto planets)
// attract every body, super-planetesimals attract the massive ones only.
#ifndef NBODIES_H_
#define NBODIES_H_

class NBodies {
 public:
  NBodies();

  int NOfMassive();   // centralBody + giantPlanet + rockyPlanet + protoPlanet
  int NOfPlAndSpl();  // superPlanetsimal + planetsimal
  int NOfVar();       // 6 * total

  int centralBody;
  int giantPlanet;
  int rockyPlanet;
  int protoPlanet;
  int superPlanetsimal;
  int planetsimal;
  int testParticle;
  int total;

  int removed;
  int threshold;
};

#endif
