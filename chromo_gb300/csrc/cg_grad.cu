// cg_grad.cu -- derivatives of the FP64 replica energy (no counterpart in the
// reference, which has no derivatives).
//
// The energy is the one cg_energy reports: SSWLC elastic energy
// (chromo/polymers.pyx:1348-1381), binding free energy (:1383-1538) and the
// field energy in the form whose differences are the per-move field dE
// (chromo/fields.pyx:1675-1875):
//   E_field = sum_v [ sum_b pref_b rho_b^2 + sum_bc xpref_bc rho_b rho_c
//                     + (vf > vf_limit ? 1e99 vf : chi (V / V_bead) vf^2) ]
//             + sum_b intra_b #(beads with state_b == 2),
// rho_b = (sum_i w_i(v) s_ib) / V and vf = (sum_i w_i(v)) V_bead / V, w_i(v)
// the trilinear weight of bead i at voxel v.
//
// gradient_kernel: dE/dr_i = elastic (the two bonds at bead i) + field
// (sum over the bead's eight voxels of dE_v/dw_i(v) dw_i(v)/dr_i).
// terms_kernel: the sums whose linear combinations are dE/d(chi, mu, eps)
// and the reweighting observables, optionally added (with their outer
// products) to per-replica running sums over sampled configurations.
#include <cuda_runtime.h>

#include "cg_device.cuh"
#include "cg_kernels.h"

namespace cg {

// d E_pair / d dr of bond (bead j -> bead j+1), dr = r_{j+1} - r_j, a0 / a1
// the t3 tangents at j / j+1.  With par = a0.dr, dp = P dr (P = I - a0 a0^T),
// bend = a1 - a0 - eta dp:
//   dE/ddr = -eta eb P bend + ep (par - gamma) a0 + epp P dp.
__device__ __forceinline__ void bond_grad(const Bond<double>& b, const double a0[3], const double a1[3],
                                          const double dr[3], double g[3]) {
  const double par = a0[0] * dr[0] + a0[1] * dr[1] + a0[2] * dr[2];
  double dp[3], bend[3];
  for (int j = 0; j < 3; j++) dp[j] = dr[j] - a0[j] * par;
  for (int j = 0; j < 3; j++) bend[j] = a1[j] + (-a0[j] - b.eta * dp[j]);
  const double ab = a0[0] * bend[0] + a0[1] * bend[1] + a0[2] * bend[2];
  const double ad = a0[0] * dp[0] + a0[1] * dp[1] + a0[2] * dp[2];
  for (int j = 0; j < 3; j++)
    g[j] = -b.eta * b.eb * (bend[j] - a0[j] * ab) + b.ep * (par - b.g) * a0[j] + b.epp * (dp[j] - a0[j] * ad);
}

// Trilinear weights of one position with their derivatives along x, y, z
// (the construction of voxel_weights; d(lower)/dx = -1/dx, d(upper)/dx = 1/dx).
__device__ __forceinline__ void weights_and_slopes(const RepDev& rd, const double pos[3], double w[8],
                                                   double dw[8][3], int v[8]) {
  const double width[3] = {rd.wx, rd.wy, rd.wz};
  const int n[3] = {rd.nx, rd.ny, rd.nz};
  double wl[3], inv[3];
  int lo[3], hi[3];
  for (int j = 0; j < 3; j++) {
    const double d = width[j] / (double)n[j];
    const double x = pymod(pos[j] + 0.5 * width[j], width[j]) - 0.5 * d;
    const long long ind = (long long)floor(x / d);
    const int li = ind == -1 ? n[j] - 1 : (int)ind;
    lo[j] = li < 0 ? 0 : (li >= n[j] ? n[j] - 1 : li);
    hi[j] = lo[j] + 1 == n[j] ? 0 : lo[j] + 1;
    wl[j] = 1 - (x / d - (double)ind);
    inv[j] = 1.0 / d;
  }
  for (int l = 0; l < 8; l++) {
    const int bx = l & 1, by = (l >> 1) & 1, bz = (l >> 2) & 1;
    const double f[3] = {bx ? 1 - wl[0] : wl[0], by ? 1 - wl[1] : wl[1], bz ? 1 - wl[2] : wl[2]};
    const double s[3] = {bx ? inv[0] : -inv[0], by ? inv[1] : -inv[1], bz ? inv[2] : -inv[2]};
    w[l] = f[0] * f[1] * f[2];
    dw[l][0] = s[0] * f[1] * f[2];
    dw[l][1] = f[0] * s[1] * f[2];
    dw[l][2] = f[0] * f[1] * s[2];
    v[l] = (bx ? hi[0] : lo[0]) + rd.nx * ((by ? hi[1] : lo[1]) + rd.ny * (bz ? hi[2] : lo[2]));
  }
}

// d E_pair / d a0 and d E_pair / d a1 of bond (j -> j+1) (the t3 tangents at
// j and j+1 taken as free vectors, as the energy's formula reads them):
//   dE/da1 = eb bend,
//   dE/da0 = eb (eta (par bend + (a0.bend) dr) - bend) + ep (par - gamma) dr
//            - epp (par dp + (a0.dp) dr).
__device__ __forceinline__ void bond_tangent_grad(const Bond<double>& b, const double a0[3], const double a1[3],
                                                  const double dr[3], double g0[3], double g1[3]) {
  const double par = a0[0] * dr[0] + a0[1] * dr[1] + a0[2] * dr[2];
  double dp[3], bend[3];
  for (int j = 0; j < 3; j++) dp[j] = dr[j] - a0[j] * par;
  for (int j = 0; j < 3; j++) bend[j] = a1[j] + (-a0[j] - b.eta * dp[j]);
  const double ab = a0[0] * bend[0] + a0[1] * bend[1] + a0[2] * bend[2];
  const double ad = a0[0] * dp[0] + a0[1] * dp[1] + a0[2] * dp[2];
  for (int j = 0; j < 3; j++) {
    g1[j] = b.eb * bend[j];
    g0[j] = b.eb * (b.eta * (par * bend[j] + ab * dr[j]) - bend[j]) + b.ep * (par - b.g) * dr[j] -
            b.epp * (par * dp[j] + ad * dr[j]);
  }
}

template <typename Pos, typename Out>
__global__ void gradient_kernel(KArgs a, Out* out, Out* out_t3) {
  const int rep = blockIdx.y;
  const RepDev& rd = a.reps[rep];
  const V4<Pos>* r4 = reinterpret_cast<const V4<Pos>*>(a.r4) + rd.bead_off;
  const V4<Pos>* t34 = reinterpret_cast<const V4<Pos>*>(a.t34) + rd.bead_off;
  const double* bonds = a.bonds + rd.bead_off * 6;
  const unsigned* st = a.states + rd.bead_off;
  const long long* grid = a.grid + rd.vox_off * a.ncol;
  const long long N = rd.n_beads;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N;
       i += (long long)gridDim.x * blockDim.x) {
    double ri[3], ai[3], gr[3] = {0, 0, 0}, gt[3] = {0, 0, 0};
    ld3(r4, i, ri);
    ld3(t34, i, ai);
    if (i > 0) {  // bond (i-1 -> i): + dE/ddr; dE/da1 for the tangent
      double rp[3], ap[3], dr[3], g[3];
      ld3(r4, i - 1, rp);
      ld3(t34, i - 1, ap);
      for (int j = 0; j < 3; j++) dr[j] = ri[j] - rp[j];
      const Bond<double> b = load_bond<double>(bonds, i - 1);
      bond_grad(b, ap, ai, dr, g);
      for (int j = 0; j < 3; j++) gr[j] += g[j];
      if (out_t3) {
        double g0[3], g1[3];
        bond_tangent_grad(b, ap, ai, dr, g0, g1);
        for (int j = 0; j < 3; j++) gt[j] += g1[j];
      }
    }
    if (i + 1 < N) {  // bond (i -> i+1): - dE/ddr; dE/da0 for the tangent
      double rn[3], an[3], dr[3], g[3];
      ld3(r4, i + 1, rn);
      ld3(t34, i + 1, an);
      for (int j = 0; j < 3; j++) dr[j] = rn[j] - ri[j];
      const Bond<double> b = load_bond<double>(bonds, i);
      bond_grad(b, ai, an, dr, g);
      for (int j = 0; j < 3; j++) gr[j] -= g[j];
      if (out_t3) {
        double g0[3], g1[3];
        bond_tangent_grad(b, ai, an, dr, g0, g1);
        for (int j = 0; j < 3; j++) gt[j] += g0[j];
      }
    }
    if (rd.field_kind == 2) {
      double w[8], dw[8][3];
      int v[8];
      weights_and_slopes(rd, ri, w, dw, v);
      const unsigned sw = st[i];
      for (int l = 0; l < 8; l++) {
        const long long* row = grid + (long long)v[l] * a.ncol;
        const double V = rd.has_access ? a.access_vol[rd.vox_off + v[l]] : rd.vol_bin;
        double rho[CG_MAX_BINDERS];
        for (int b = 0; b < rd.nb; b++) rho[b] = ((double)row[1 + b] * kFxInv) / V;
        const double vf = ((double)row[0] * kFxInv) / V * rd.bead_vol;
        double phi = vf > rd.vf_limit ? kEHugeField * rd.bead_vol / V : 2 * rd.chi * vf;
        for (int b = 0; b < rd.nb; b++) {
          const int s = (int)((sw >> (8 * b)) & 0xFF);
          if (!s) continue;
          double pb = 2 * rd.pref[b] * rho[b];
          for (int c = 0; c < rd.nb; c++)
            pb += (rd.xpref[b * CG_MAX_BINDERS + c] + rd.xpref[c * CG_MAX_BINDERS + b]) * rho[c];
          phi += (double)s * pb / V;
        }
        for (int j = 0; j < 3; j++) gr[j] += phi * dw[l][j];
      }
    }
    Out* o = out + 3 * (rd.bead_off + i);
    o[0] = (Out)gr[0];
    o[1] = (Out)gr[1];
    o[2] = (Out)gr[2];
    if (out_t3) {
      Out* ot = out_t3 + 3 * (rd.bead_off + i);
      ot[0] = (Out)gt[0];
      ot[1] = (Out)gt[1];
      ot[2] = (Out)gt[2];
    }
  }
}

__device__ double grad_block_sum(double v, double* sh) {
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
  return t;  // valid in warp 0
}

// Terms T[14] of one replica: [0] S = sum_(vf <= limit) (V / V_bead) vf^2,
// [1..3] sum_v rho_b^2, [4..6] sum_v rho_0 rho_1, rho_0 rho_2, rho_1 rho_2,
// [7..9] #(state_b == 2), [10..12] sum_i s_ib, [13] sum_v (W / V)^2 with W the
// bead weight of the voxel.  acc (or null): running sums [T, T T^T, count].
__global__ void terms_kernel(KArgs a, double* terms, double* acc) {
  __shared__ double sh[32];
  __shared__ double T[kTerms];
  const int rep = blockIdx.x;
  const RepDev& rd = a.reps[rep];
  double loc[kTerms];
  for (int k = 0; k < kTerms; k++) loc[k] = 0;
  const unsigned* st = a.states + rd.bead_off;
  for (long long i = threadIdx.x; i < rd.n_beads; i += blockDim.x) {
    const unsigned sw = st[i];
    for (int b = 0; b < rd.nb; b++) {
      const int s = (int)((sw >> (8 * b)) & 0xFF);
      loc[7 + b] += s == 2 ? 1.0 : 0.0;
      loc[10 + b] += (double)s;
    }
  }
  if (rd.field_kind == 2 && !rd.has_access) {
    // Uniform voxel volume V: every term is a sum of products of fixed-point
    // grid values times one constant, so the raw products are summed (no FP64
    // division per voxel; GB300 runs FP64 at 1/64 of the FP32 rate) and
    // scaled once.  vf <= vf_limit <=> g0 <= vf_limit / (2^-40 Vb / V).
    const long long* grid = a.grid + rd.vox_off * a.ncol;
    const double u = kFxInv / rd.vol_bin;          // density per fixed-point unit
    const double c = u * rd.bead_vol;              // volume fraction per unit
    const double gmax = rd.vf_limit / c;
    double s00 = 0, s00_lim = 0, sbb[CG_MAX_BINDERS] = {0, 0, 0}, sx[3] = {0, 0, 0};
    for (long long v = threadIdx.x; v < rd.n_vox; v += blockDim.x) {
      const double g0 = (double)grid[v * a.ncol];
      double gb[CG_MAX_BINDERS] = {0, 0, 0};
      for (int b = 0; b < rd.nb; b++) gb[b] = (double)grid[v * a.ncol + 1 + b];
      const double q = g0 * g0;
      s00 += q;
      if (g0 <= gmax) s00_lim += q;
      for (int b = 0; b < CG_MAX_BINDERS; b++) sbb[b] += gb[b] * gb[b];
      sx[0] += gb[0] * gb[1];
      sx[1] += gb[0] * gb[2];
      sx[2] += gb[1] * gb[2];
    }
    const double u2 = u * u;
    loc[0] += (rd.vol_bin / rd.bead_vol) * (c * c) * s00_lim;
    for (int b = 0; b < CG_MAX_BINDERS; b++) loc[1 + b] += u2 * sbb[b];
    for (int k = 0; k < 3; k++) loc[4 + k] += u2 * sx[k];
    loc[13] += u2 * s00;
  } else if (rd.field_kind == 2) {
    const long long* grid = a.grid + rd.vox_off * a.ncol;
    for (long long v = threadIdx.x; v < rd.n_vox; v += blockDim.x) {
      const double V = rd.has_access ? a.access_vol[rd.vox_off + v] : rd.vol_bin;
      double rho[CG_MAX_BINDERS] = {0, 0, 0};
      for (int b = 0; b < rd.nb; b++) rho[b] = ((double)grid[v * a.ncol + 1 + b] * kFxInv) / V;
      const double dens = ((double)grid[v * a.ncol] * kFxInv) / V;
      const double vf = dens * rd.bead_vol;
      if (vf <= rd.vf_limit) loc[0] += (V / rd.bead_vol) * vf * vf;
      for (int b = 0; b < CG_MAX_BINDERS; b++) loc[1 + b] += rho[b] * rho[b];
      loc[4] += rho[0] * rho[1];
      loc[5] += rho[0] * rho[2];
      loc[6] += rho[1] * rho[2];
      loc[13] += dens * dens;
    }
  }
  for (int k = 0; k < kTerms; k++) {
    const double t = grad_block_sum(loc[k], sh);
    if (threadIdx.x == 0) T[k] = t;
  }
  __syncthreads();
  if (terms && threadIdx.x < kTerms) terms[rep * kTerms + threadIdx.x] = T[threadIdx.x];
  if (acc) {
    double* A = acc + (long long)rep * kAccPerRep;
    if (threadIdx.x < kTerms) A[threadIdx.x] += T[threadIdx.x];
    for (int k = threadIdx.x; k < kTerms * kTerms; k += blockDim.x)
      A[kTerms + k] += T[k / kTerms] * T[k % kTerms];
    if (threadIdx.x == 0) A[kTerms + kTerms * kTerms] += 1.0;
  }
}

}  // namespace cg

static dim3 gradient_grid(const cg::KArgs& a, long long max_beads) {
  long long bx = (max_beads + 127) / 128;
  if (bx > 64) bx = 64;
  if (bx < 1) bx = 1;
  return dim3((unsigned)bx, (unsigned)a.n_reps);
}

void cg_launch_gradient(const cg::KArgs& a, bool fp64, float* out, long long max_beads, cudaStream_t s) {
  const dim3 grid = gradient_grid(a, max_beads);
  if (fp64) cg::gradient_kernel<double, float><<<grid, 128, 0, s>>>(a, out, nullptr);
  else cg::gradient_kernel<float, float><<<grid, 128, 0, s>>>(a, out, nullptr);
}

void cg_launch_gradient64(const cg::KArgs& a, bool fp64, double* out, double* out_t3, long long max_beads,
                          cudaStream_t s) {
  const dim3 grid = gradient_grid(a, max_beads);
  if (fp64) cg::gradient_kernel<double, double><<<grid, 128, 0, s>>>(a, out, out_t3);
  else cg::gradient_kernel<float, double><<<grid, 128, 0, s>>>(a, out, out_t3);
}

namespace cg {
// Global bead b (replicas concatenated) of FP64 [total_beads x 3] arrays into
// the resident 4-vector storage.
template <typename Pos>
__global__ void store_chains_kernel(KArgs a, long long total, const double* r, const double* t3) {
  V4<Pos>* r4 = reinterpret_cast<V4<Pos>*>(a.r4);
  V4<Pos>* t34 = reinterpret_cast<V4<Pos>*>(a.t34);
  for (long long b = blockIdx.x * (long long)blockDim.x + threadIdx.x; b < total;
       b += (long long)gridDim.x * blockDim.x) {
    if (r) r4[b] = V4<Pos>{(Pos)r[3 * b], (Pos)r[3 * b + 1], (Pos)r[3 * b + 2], (Pos)0};
    if (t3) t34[b] = V4<Pos>{(Pos)t3[3 * b], (Pos)t3[3 * b + 1], (Pos)t3[3 * b + 2], (Pos)0};
  }
}
}  // namespace cg

void cg_launch_store_chains(const cg::KArgs& a, bool fp64, long long total, const double* r, const double* t3,
                            cudaStream_t s) {
  long long blocks = (total + 255) / 256;
  if (blocks > 152 * 8) blocks = 152 * 8;
  if (blocks < 1) blocks = 1;
  if (fp64) cg::store_chains_kernel<double><<<(unsigned)blocks, 256, 0, s>>>(a, total, r, t3);
  else cg::store_chains_kernel<float><<<(unsigned)blocks, 256, 0, s>>>(a, total, r, t3);
}

void cg_launch_terms(const cg::KArgs& a, double* terms, double* acc, cudaStream_t s) {
  cg::terms_kernel<<<a.n_reps, 256, 0, s>>>(a, terms, acc);
}
