// One instantiation of the production MC kernel: double storage, 32 lanes per move.
#include "cg_spec.cuh"

CG_SPEC_INSTANTIATE(double, 32, d32)
