// bodies.cuh -- device view of the rigid bodies of a system, shared by the
// body kernels (bodies.cu) and the fused Verlet step (verlet.cu).
#pragma once

#include "rigid.cuh"
#include "system.hpp"

namespace emdee {

struct BodyArgs {
  BodyState* b;
  int nb;
  const int* atom;     // flat body-atom indices (0-based)
  const double* M;     // flat masses
  const double* d;     // flat body-frame coordinates
  double* delta;       // flat space-frame offsets
};

inline BodyArgs body_args(System& s) {
  BodyArgs A;
  A.b = s.dBodies;
  A.nb = s.nbodies;
  A.atom = s.dBodyAtom;
  A.M = s.dBodyM;
  A.d = s.dBodyD;
  A.delta = s.dBodyDelta;
  return A;
}

}  // namespace emdee
