// One instantiation of the production MC kernel: float storage, 8 lanes per move.
#include "cg_spec.cuh"

CG_SPEC_INSTANTIATE(float, 8, f8)
