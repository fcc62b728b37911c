// The production MC kernel's cluster form: float storage, 32 lanes per move,
// a replica on a thread-block cluster of CTAs (workloads with fewer replicas
// than SMs).
#include "cg_spec.cuh"

CG_SPEC_INSTANTIATE_CLUSTER(float, 32, c32)
