// One instantiation of the production MC kernel: float storage, 16 lanes per move.
#include "cg_spec.cuh"

CG_SPEC_INSTANTIATE(float, 16, f16)
