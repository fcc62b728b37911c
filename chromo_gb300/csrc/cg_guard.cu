// cg_guard.cu -- on-device FP64 drift guard of the batched rounds.
//
// The MC kernels keep each replica's running sum of accepted dE in FP64
// (RepDev::run_dE) and the exchange kernel adds the energy change of every
// accepted chi or mu swap to RepDev::xch_dE.  Every `every`-th round of
// cg_run_batched ends with the replicas' full FP64 energies recomputed from
// the resident state (cg_energy.cuh: elastic + binding + field), and the
// change since the previous check is compared with the change of
// run_dE + xch_dE over the same rounds.  A difference beyond
// tol_abs + tol_rel * max(1, |E|) (or a non-finite one) sets the replica's
// E_DRIFT error bit, which the next cg_sync reports.  An interval whose end
// energies carry a 1e25 / 1e99 penalty is not compared (FP64 cannot resolve
// the soft energy next to it); its end becomes the next reference.  The recompute is split
// over chunk x replica blocks whose partial sums are added in chunk order, so
// it is deterministic and spreads over the GPU even for a few large replicas.
//
// Reference: the energies are chromo/polymers.pyx:1348-1538 and
// chromo/fields.pyx:1675-1875,1939-2316; the reference itself has no drift
// (it sums dE in FP64 on the CPU and never recomputes).
#include <cuda_runtime.h>

#include "cg_energy.cuh"

namespace cg {

// partial sums per (replica, chunk): el, bi, fe, dbl[0..2]
constexpr int kGuardParts = 3 + CG_MAX_BINDERS;

__device__ __forceinline__ bool guard_round(const GuardArgs& g) {
  return (g.counter[0] + 1) % (unsigned long long)g.every == 0;
}

template <typename Pos>
__global__ void guard_partial_kernel(KArgs a, GuardArgs g) {
  __shared__ double sh[32];
  if (!guard_round(g)) return;
  const int rep = blockIdx.y, chunk = blockIdx.x;
  const RepDev& rd = a.reps[rep];
  EnergyParts p{0.0, 0.0, 0.0, 0.0, {0, 0, 0}};
  const long long nb_per = (rd.n_beads + g.chunks - 1) / g.chunks;
  const long long b0 = chunk * nb_per, b1 = b0 + nb_per < rd.n_beads ? b0 + nb_per : rd.n_beads;
  for (long long i = b0 + threadIdx.x; i < b1; i += blockDim.x) bead_energy<Pos>(a, rd, i, p);
  if (rd.field_kind == 2) {
    const long long nv_per = (rd.n_vox + g.chunks - 1) / g.chunks;
    const long long v0 = chunk * nv_per, v1 = v0 + nv_per < rd.n_vox ? v0 + nv_per : rd.n_vox;
    for (long long v = v0 + threadIdx.x; v < v1; v += blockDim.x) voxel_energy(a, rd, v, p);
  }
  double vals[kGuardParts] = {p.el, p.bi, p.fe, (double)p.dbl[0], (double)p.dbl[1], (double)p.dbl[2]};
  double* out = g.partial + ((long long)rep * g.chunks + chunk) * kGuardParts;
  for (int k = 0; k < kGuardParts; k++) {
    const double t = block_total(vals[k], sh);
    if (threadIdx.x == 0) out[k] = t;
  }
}

// One thread per replica: the check (on a guard round), then the round counter.
__global__ void guard_check_kernel(KArgs a, GuardArgs g) {
  const bool check = guard_round(g);
  for (int rep = blockIdx.x * blockDim.x + threadIdx.x; rep < a.n_reps; rep += gridDim.x * blockDim.x) {
    if (!check) continue;
    RepDev& rd = a.reps[rep];
    double t[kGuardParts] = {0, 0, 0, 0, 0, 0};
    const double* in = g.partial + (long long)rep * g.chunks * kGuardParts;
    for (int c = 0; c < g.chunks; c++)
      for (int k = 0; k < kGuardParts; k++) t[k] += in[c * kGuardParts + k];
    double E = t[0] + t[1];
    if (rd.field_kind == 2) {
      double intra = 0;
      for (int b = 0; b < rd.nb; b++) intra += rd.intra[b] * t[3 + b];
      E += t[2] + intra;
    }
    const double run = rd.run_dE + rd.xch_dE;
    // an interval whose end energies carry a penalty (|E| >= kPenaltyFloor)
    // cannot be checked in FP64: the guard takes new references there
    if (g.init[rep] && fabs(E) < kPenaltyFloor && fabs(g.e_ref[rep]) < kPenaltyFloor) {
      const double d = (E - g.e_ref[rep]) - (run - g.run_ref[rep]);
      g.drift[rep] = d;
      const double bound = g.tol_abs + g.tol_rel * (fabs(E) > 1.0 ? fabs(E) : 1.0);
      if (!(fabs(d) <= bound)) rd.err |= E_DRIFT;
    }
    g.e_ref[rep] = E;
    g.run_ref[rep] = run;
    g.init[rep] = 1;
  }
  __syncthreads();
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    if (check) g.counter[1] += 1;
    g.counter[0] += 1;
  }
}

}  // namespace cg

void cg_launch_guard(const cg::KArgs& a, const cg::GuardArgs& g, bool fp64, cudaStream_t s) {
  const dim3 grid((unsigned)g.chunks, (unsigned)a.n_reps);
  if (fp64) cg::guard_partial_kernel<double><<<grid, 256, 0, s>>>(a, g);
  else cg::guard_partial_kernel<float><<<grid, 256, 0, s>>>(a, g);
  cg::guard_check_kernel<<<1, 256, 0, s>>>(a, g);
}
