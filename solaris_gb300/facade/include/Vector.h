// Three-component vector used by BodyData's diagnostic members.
#ifndef VECTOR_H_
#define VECTOR_H_

class Vector {
 public:
  Vector() : x(0.0), y(0.0), z(0.0) {}
  Vector(double a, double b, double c) : x(a), y(b), z(c) {}
  double x;
  double y;
  double z;
};

#endif
