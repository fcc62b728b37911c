// One instantiation of the production MC kernel: float storage, 32 lanes per move.
#include "cg_spec.cuh"

CG_SPEC_INSTANTIATE(float, 32, f32)
