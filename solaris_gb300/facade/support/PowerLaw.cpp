// Standalone PowerLaw.
#include "PowerLaw.h"

#include <cmath>

PowerLaw::PowerLaw() : c(0.0), index(0.0) {}

PowerLaw::PowerLaw(double c_, double index_) : c(c_), index(index_) {}

double PowerLaw::Evaluate(double x) { return c * std::pow(x, index); }
