// cg_energy.cuh -- FP64 energy terms of one bead and one voxel, shared by
// the per-replica energy kernel and the drift guard.
//
// The energy is the one whose differences are the per-move dE: SSWLC elastic
// energy (SSWLC.compute_E, chromo/polymers.pyx:1348-1381), the single-site
// binding free energy whose differences are binding_dE
// (chromo/polymers.pyx:1383-1538), and the field energy in the form whose
// differences are the per-move field dE (chromo/fields.pyx:1675-1875).
#pragma once
#include "cg_device.cuh"
#include "cg_kernels.h"
#include "cg_move.cuh"

namespace cg {

// Partial sums of one replica's energy over a range of beads and voxels.
struct EnergyParts {
  double el, bi, fe, sx;                // elastic, binding, field, chi-free sum S
  long long dbl[CG_MAX_BINDERS];        // doubly bound beads per binder
};

// Bond i - 1 -> i (i > 0) and the binding free energy of bead i.
template <typename Pos>
__device__ __forceinline__ void bead_energy(const KArgs& a, const RepDev& rd, long long i, EnergyParts& p) {
  const V4<Pos>* r4 = reinterpret_cast<const V4<Pos>*>(a.r4) + rd.bead_off;
  const V4<Pos>* t34 = reinterpret_cast<const V4<Pos>*>(a.t34) + rd.bead_off;
  const double* bonds = a.bonds + rd.bead_off * 6;
  if (i > 0) {
    double r0[3], r1[3], a0[3], a1[3], dr[3], dp[3], bend[3];
    ld3(r4, i - 1, r0); ld3(r4, i, r1); ld3(t34, i - 1, a0); ld3(t34, i, a1);
    Bond<double> b = load_bond<double>(bonds, i - 1);
    for (int j = 0; j < 3; j++) dr[j] = r1[j] - r0[j];
    double par = a0[0] * dr[0] + a0[1] * dr[1] + a0[2] * dr[2];
    for (int j = 0; j < 3; j++) dp[j] = dr[j] - a0[j] * par;
    for (int j = 0; j < 3; j++) bend[j] = a1[j] + (-a0[j] - b.eta * dp[j]);
    p.el += e_pair(b, bend, par, dp);
    if (rd.twist) {  // SSTWLC.compute_E, chromo/polymers.pyx:2250-2285
      const V4<Pos>* t24 = reinterpret_cast<const V4<Pos>*>(a.t24) + rd.bead_off;
      p.el += twist_bond_energy(a.twist + 2 * (rd.bead_off + i - 1), frame_of(t24[i - 1], t34[i - 1]),
                                frame_of(t24[i], t34[i]));
    }
  }
  const unsigned sw = a.states[rd.bead_off + i], mw = a.marks[rd.bead_off + i];
  int tot = 0;
  for (int b = 0; b < rd.nb; b++) {
    int s = (int)((sw >> (8 * b)) & 0xFF), nm = (int)((mw >> (8 * b)) & 0xFF);
    double me = rd.mu[b] > 0 ? rd.mu[b] * (-rd.mu_adjust + 2) : rd.mu[b] * rd.mu_adjust;
    p.bi += bind_f(rd, b, nm, s) - (double)s * me;
    tot += s;
    p.dbl[b] += s == 2;
  }
  if (rd.max_binders != -1 && tot > rd.max_binders) p.bi += kEHugePoly * (double)(tot - rd.max_binders);
}

// Field terms of voxel v (UniformDensityField only).
__device__ __forceinline__ void voxel_energy(const KArgs& a, const RepDev& rd, long long v, EnergyParts& p) {
  const long long* grid = a.grid + rd.vox_off * a.ncol;
  double V = rd.has_access ? a.access_vol[rd.vox_off + v] : rd.vol_bin;
  double rho[CG_MAX_BINDERS];
  for (int b = 0; b < rd.nb; b++) rho[b] = ((double)grid[v * a.ncol + 1 + b] * kFxInv) / V;
  for (int b = 0; b < rd.nb; b++) p.fe += rd.pref[b] * rho[b] * rho[b];
  for (int b = 0; b < rd.nb; b++)
    for (int e = 0; e < rd.nb; e++) p.fe += rd.xpref[b * CG_MAX_BINDERS + e] * rho[b] * rho[e];
  double vf = ((double)grid[v * a.ncol] * kFxInv) / V * rd.bead_vol;
  double sv = (V / rd.bead_vol) * vf * vf;
  // S: the chi-free sum over the voxels at or below vf_limit (a voxel above
  // it costs 1e99 vf, which does not depend on chi)
  if (!(vf > rd.vf_limit)) p.sx += sv;
  p.fe += vf > rd.vf_limit ? kEHugeField * vf : rd.chi * sv;
}

// one block; deterministic tree reduction, the total valid in warp 0
__device__ __forceinline__ double block_total(double v, double* sh) {
  v = warp_sum(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  double t = 0;
  if (threadIdx.x < 32) {
    t = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
    t = warp_sum(t);
  }
  return t;
}

}  // namespace cg
