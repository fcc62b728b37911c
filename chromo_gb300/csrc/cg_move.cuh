// cg_move.cuh -- per-move building blocks shared by the MC kernels: the
// per-warp voxel hash (int64 fixed-point density deltas), the field dE over
// the touched voxels, commit of the touched voxels, confinement counts and
// the binding free-energy lookup.
#pragma once
#include "cg_device.cuh"
#include "cg_kernels.h"

namespace cg {

// FP32 copies of a replica's field and binding constants (one thread).
__device__ __forceinline__ void setup_f32(WarpShared& ws) {
  const RepDev& rd = ws.rd;
  make_gridf(rd, ws.gf);
  for (int b = 0; b < CG_MAX_BINDERS; b++) ws.f_pref[b] = (float)rd.pref[b];
  for (int b = 0; b < CG_MAX_BINDERS * CG_MAX_BINDERS; b++) ws.f_xpref[b] = (float)rd.xpref[b];
  ws.f_scale = (float)(kFxInv / rd.vol_bin);
  ws.f_vb = (float)rd.bead_vol;
  ws.f_k = (float)(rd.chi * (rd.vol_bin / rd.bead_vol));
  ws.f_lim = (float)rd.vf_limit;
  for (int i = 0; i < CG_MAX_BINDERS * (CG_MAX_MARK + 1) * (CG_MAX_MARK + 1); i++)
    ws.f_bind[i] = (float)rd.bind_f[i];
  for (int b = 0; b < CG_MAX_BINDERS; b++) {
    ws.f_me[b] = (float)(rd.mu[b] > 0 ? rd.mu[b] * (-rd.mu_adjust + 2) : rd.mu[b] * rd.mu_adjust);
    ws.f_intra[b] = (float)rd.intra[b];
  }
}

// ---------------------------------------------------------------- hash insert
// Add d to column `col` of a hash entry.  Global-memory tables take one 64-bit
// atomic.  Shared-memory tables (split = true) keep each column as two 32-bit
// counters, d = hi * 2^21 + lo with lo in [0, 2^21): 32-bit shared atomics are
// native and several times faster than 64-bit ones.  A shared table has at
// most 1,024 slots and serves moves of m <= slots / 16 beads, so a column gets
// at most 16 m <= 1,024 contributions of |d| < 2^42: |sum hi| < 2^10 * 3 * 2^19
// and sum lo < 2^10 * 2^21, both below 2^31.
__device__ __forceinline__ void add_delta(long long* vals, int ncol, int slot, int col, long long d,
                                          bool split = false) {
  if (d == 0) return;
  long long* cell = &vals[(long long)slot * ncol + col];
  if (split) {
    int* half = reinterpret_cast<int*>(cell);
    atomicAdd(half, (int)(d & 0x1FFFFF));
    atomicAdd(half + 1, (int)(d >> 21));
  } else {
    atomicAdd((unsigned long long*)cell, (unsigned long long)d);
  }
}

// Value of a hash column written by add_delta.
__device__ __forceinline__ long long hash_delta(const long long* cell, bool split) {
  if (!split) return *cell;
  const int* half = reinterpret_cast<const int*>(cell);
  return (long long)half[1] * 2097152LL + (long long)half[0];
}

// Linear probing for `key` after its home slot `start` was found taken by
// another key: the slot, plus 1 << 30 when the key claimed it new, or -1 when
// the table is full (out of line: the loop is rare and would be inlined at
// every claim).
static __device__ __noinline__ int hash_probe_packed(int* keys, int logH, int key, int start) {
  const unsigned mask = (1u << logH) - 1u;
  unsigned h = ((unsigned)start + 1u) & mask;
  for (unsigned it = 1; it <= mask; it++) {
    int prev = atomicCAS(&keys[h], -1, key);
    if (prev == -1) return (int)h | (1 << 30);
    if (prev == key) return (int)h;
    h = (h + 1) & mask;
  }
  return -1;
}
__device__ __forceinline__ int hash_probe(int* keys, int logH, int key, int start, bool& inserted,
                                          unsigned& err) {
  const int r = hash_probe_packed(keys, logH, key, start);
  if (r < 0) { err |= E_SPIN; return -1; }
  inserted = (r >> 30) & 1;
  return r & ((1 << 30) - 1);
}

// Claim (or find) the slot of `key`; a new slot is appended to the used list.
__device__ __forceinline__ int hash_slot(int* keys, int* used, int* nused, int logH, int key,
                                         unsigned& err) {
  const unsigned h = ((unsigned)key * 0x9E3779B1u) >> (32 - logH);
  int prev = atomicCAS(&keys[h], -1, key);
  int slot = (int)h;
  bool fresh = prev == -1;
  if (!fresh && prev != key) {
    const int r = hash_probe_packed(keys, logH, key, (int)h);
    if (r < 0) { err |= E_SPIN; return -1; }
    fresh = (r >> 30) & 1;
    slot = r & ((1 << 30) - 1);
  }
  if (fresh) used[atomicAdd(nused, 1)] = slot;
  return slot;
}

// Deposit +/- one bead's eight trilinear weights with binder states `st`
// (packed int8) into the hash.  The eight home-slot claims are issued back to
// back (independent shared-memory atomics in flight together); only a claim
// that meets another key probes on.  The lane appends its new slots to the
// used list with one counter update.
template <typename Real>
__device__ __forceinline__ void deposit_bead(const RepDev& rd, int ncol, int* keys, int* used,
                                             int* nused, long long* vals, int logH,
                                             const Real w[8], const int v[8], unsigned st,
                                             bool negate, unsigned& err, bool split = false) {
  int slot[8], prev[8];
#pragma unroll
  for (int l = 0; l < 8; l++) {
    slot[l] = (int)(((unsigned)v[l] * 0x9E3779B1u) >> (32 - logH));
    prev[l] = atomicCAS(&keys[slot[l]], -1, v[l]);
  }
  unsigned fresh = 0;
#pragma unroll
  for (int l = 0; l < 8; l++) {
    if (prev[l] == -1) {
      fresh |= 1u << l;
    } else if (prev[l] != v[l]) {
      bool inserted = false;
      slot[l] = hash_probe(keys, logH, v[l], slot[l], inserted, err);
      if (slot[l] < 0) return;
      if (inserted) fresh |= 1u << l;
    }
  }
  if (fresh) {
    int at = atomicAdd(nused, __popc(fresh));
#pragma unroll
    for (int l = 0; l < 8; l++)
      if ((fresh >> l) & 1u) used[at++] = slot[l];
  }
#pragma unroll
  for (int l = 0; l < 8; l++) {
    long long q = q40(w[l]);
    if (negate) q = -q;
    add_delta(vals, ncol, slot[l], 0, q, split);
    for (int b = 0; b < rd.nb; b++)
      add_delta(vals, ncol, slot[l], 1 + b, q * (long long)((st >> (8 * b)) & 0xFF), split);
  }
}

// Claim (or find) the slots of up to NQ voxels per lane (v[j] where
// want[j]) in a table shared by the lanes `peers` (this lane's bit set); the
// peers append their new slots to the used list with one counter update.
// Every lane's home-slot claims are issued back to back; only a claim that
// meets another key probes on.  A table that cannot take a new voxel (slot
// -1), or whose count of voxels passes `cap` (every peer), sets `full_bit` in
// err.  Called by the whole warp.
template <int NQ>
__device__ __forceinline__ void claim_slots(int* keys, int* used, int* nused, int logH, const int (&v)[NQ],
                                            const bool (&want)[NQ], int (&slot)[NQ], unsigned& err,
                                            int cap, unsigned full_bit, unsigned peers) {
  int prev[NQ];
  bool fresh[NQ];
#pragma unroll
  for (int j = 0; j < NQ; j++) {
    slot[j] = (int)(((unsigned)v[j] * 0x9E3779B1u) >> (32 - logH));
    prev[j] = want[j] ? atomicCAS(&keys[slot[j]], -1, v[j]) : v[j];
  }
#pragma unroll
  for (int j = 0; j < NQ; j++) {
    fresh[j] = prev[j] == -1;
    if (!fresh[j] && prev[j] != v[j]) {
      const int r = hash_probe_packed(keys, logH, v[j], slot[j]);
      if (r < 0) {
        err |= full_bit;
        slot[j] = -1;
      } else {
        fresh[j] = (r >> 30) & 1;
        slot[j] = r & ((1 << 30) - 1);
      }
    }
  }
  const unsigned lane = threadIdx.x & 31u, lt = (1u << lane) - 1u;
  const int leader = __ffs((int)peers) - 1;
  unsigned bal[NQ];
  int cnt = 0;
#pragma unroll
  for (int j = 0; j < NQ; j++) {
    bal[j] = __ballot_sync(kFull, fresh[j]) & peers;
    cnt += __popc(bal[j]);
  }
  int base = 0;
  if ((int)lane == leader && cnt) base = atomicAdd(nused, cnt);
  base = __shfl_sync(kFull, base, leader);
  int at = base;
#pragma unroll
  for (int j = 0; j < NQ; j++) {
    if (fresh[j]) used[at + __popc(bal[j] & lt)] = slot[j];
    at += __popc(bal[j]);
  }
  if (at > cap) err |= full_bit;
}

// The lanes of this lane's aligned group of G lanes.
template <int G>
__device__ __forceinline__ unsigned group_mask() {
  if (G == 32) return kFull;
  return ((1u << (G & 31)) - 1u) << ((threadIdx.x & 31u) & ~(unsigned)(G - 1));
}

// Add a corner's contribution q to a voxel-table slot: the bead column, and
// q times the bead's state for each binder column (states packed as bytes).
__device__ __forceinline__ void add_corner(long long* vals, int hcol, int slot, long long q, unsigned sw, int nb,
                                           bool split) {
  add_delta(vals, hcol, slot, 0, q, split);
  for (int b = 0; b < nb; b++) add_delta(vals, hcol, slot, 1 + b, q * (long long)((sw >> (8 * b)) & 0xFF), split);
}

// One voxel's grid row -- bead weight, then one column per binder -- with
// 16-byte loads (rows are 2 or 4 int64 columns, 16- or 32-byte aligned).
__device__ __forceinline__ void load_row(const long long* gv, int ncol, long long row[4]) {
  const longlong2 lo = *reinterpret_cast<const longlong2*>(gv);
  row[0] = lo.x;
  row[1] = lo.y;
  row[2] = row[3] = 0;
  if (ncol == 4) {
    const longlong2 hi = reinterpret_cast<const longlong2*>(gv)[1];
    row[2] = hi.x;
    row[3] = hi.y;
  }
}

// chi term of one voxel in FP64 (fields.pyx:1792-1875 with the vf_limit
// branch): `soft` is the FP64 part, `huge` the 1e99 penalty of the voxel
// above vf_limit in kHugeUnit units (after the move minus before it).
struct ChiSplit {
  double soft;
  long long huge;
};
static __device__ __noinline__ ChiSplit chi_term64(const RepDev& rd, double V, long long g0, long long d0) {
  double vf0 = ((double)g0 * kFxInv) / V * rd.bead_vol;
  double vf1 = ((double)(g0 + d0) * kFxInv) / V * rd.bead_vol;
  double k = rd.chi * (V / rd.bead_vol);
  ChiSplit t{0.0, 0};
  if (vf1 > rd.vf_limit || vf0 > rd.vf_limit) {
    const double u = rd.bead_vol / V;
    if (vf1 > rd.vf_limit) t.huge += huge_units(g0 + d0, u);
    else t.soft += k * vf1 * vf1;
    if (vf0 > rd.vf_limit) t.huge -= huge_units(g0, u);
    else t.soft -= k * vf0 * vf0;
    return t;
  }
  t.soft = k * ((vf1 - vf0) * (vf1 + vf0));
  return t;
}

// hard + huge * kHugeUnit: the FP64 part of a move's dE with its exact 1e99
// penalties added (out of line, the penalties are rare)
static __device__ __noinline__ double hard_with_huge(double hard, long long huge) {
  return hard + (double)huge * kHugeUnit;
}
__device__ __forceinline__ double with_huge(double hard, long long huge) {
  return huge != 0 ? hard_with_huge(hard, huge) : hard;
}

// Field dE over the touched voxels (fixed-point grid), FP64 arithmetic; also
// stores the post-move grid values into the hash values for the commit.  The
// sum is added to `hard` (the FP64 part of the move's dE), nothing to `soft`;
// the 1e99 penalties of voxels above vf_limit go to `huge` (kHugeUnit units).
// Called by the whole warp; lane gl of each group of G lanes takes voxels
// gl, gl + G, ... of its group's table.
template <int G = 32>
static __device__ void field_dE_voxels(const WarpShared& ws, const KArgs& a, int hcol, const int* keys,
                                  const int* used, long long* vals, int nused, int lane,
                                  long long& n_vox, double& soft, double& hard, long long& huge,
                                  bool split = false) {
  const RepDev& rd = ws.rd;
  double part = 0;
  long long hpart = 0;
  const long long* grid = a.grid + rd.vox_off * a.ncol;
  for (int i = lane; i < nused; i += G) {
    int slot = used[i];
    int v = keys[slot];
    long long* d = vals + (long long)slot * hcol;
    long long row[4];
    load_row(grid + (long long)v * a.ncol, a.ncol, row);
    long long g0 = row[0], d0 = hash_delta(d, split);
    double V = rd.has_access ? a.access_vol[rd.vox_off + v] : rd.vol_bin;
    double c = 0, rho[CG_MAX_BINDERS], dd[CG_MAX_BINDERS];
#pragma unroll
    for (int b = 0; b < CG_MAX_BINDERS; b++) {
      if (b >= rd.nb) break;
      long long gb = row[1 + b], db = hash_delta(d + 1 + b, split);
      rho[b] = ((double)gb * kFxInv) / V;
      dd[b] = ((double)db * kFxInv) / V;
      c += rd.pref[b] * (dd[b] * (2 * rho[b] + dd[b]));
      d[1 + b] = gb + db;
    }
#pragma unroll
    for (int b = 0; b < CG_MAX_BINDERS; b++)
#pragma unroll
      for (int e = 0; e < CG_MAX_BINDERS; e++)
        if (b < rd.nb && e < rd.nb)
          c += rd.xpref[b * CG_MAX_BINDERS + e] * (rho[b] * dd[e] + dd[b] * rho[e] + dd[b] * dd[e]);
    const ChiSplit t = chi_term64(rd, V, g0, d0);
    c += t.soft;
    hpart += t.huge;
    d[0] = g0 + d0;
    part += c;
  }
  n_vox = nused;
  (void)soft;
  hard += gsum<G>(part);
  if (__any_sync(kFull, hpart != 0)) huge += gsum<G>(hpart);  // warp vote: see gsum(Fx)
}

// An FP64 term of the FP32 path: in fixed point like the FP32 terms when it
// is below 2^20 kT (so that the sum stays independent of the order of the
// terms), else into the FP64 side sum.
__device__ __forceinline__ void acc_add_wide(Fx& s, double x) {
  if (fabs(x) < 1048576.0) s.q += __double2ll_rn(x * 1073741824.0);
  else s.hard = add_hard(s.hard, x);
}

// Field dE of one touched voxel v of the FP32 path (row `d` of a voxel table:
// the move's density deltas in, the voxel's post-move row out): FP32
// arithmetic, fixed-point accumulation into `part`; a voxel at or near the
// volume-fraction limit takes the FP64 branch (its chi term in fixed point or
// the side sum, the 1e99 penalties exactly into `huge`), so which side of the
// limit it lies on is decided as in FP64.
__device__ __forceinline__ void voxel_dE_f32(const WarpShared& ws, const KArgs& a, const long long* grid, int v,
                                             long long* d, bool split, Fx& part, long long& huge) {
  const RepDev& rd = ws.rd;
  long long row[4];
  load_row(grid + (long long)v * a.ncol, a.ncol, row);
  const long long g0 = row[0], d0 = hash_delta(d, split);
  float sc = ws.f_scale, k = ws.f_k;
  if (rd.has_access) {  // per-voxel factors precomputed from V (no FP64 division here)
    sc = a.access_sc[rd.vox_off + v];
    k = (float)(rd.chi * a.access_vb[rd.vox_off + v]);
  }
  float c = 0, rho[CG_MAX_BINDERS], dd[CG_MAX_BINDERS];
#pragma unroll
  for (int b = 0; b < CG_MAX_BINDERS; b++) {
    if (b >= rd.nb) break;
    long long gb = row[1 + b], db = hash_delta(d + 1 + b, split);
    rho[b] = (float)gb * sc;
    dd[b] = (float)db * sc;
    c += ws.f_pref[b] * (dd[b] * (2.0f * rho[b] + dd[b]));
    d[1 + b] = gb + db;
  }
#pragma unroll
  for (int b = 0; b < CG_MAX_BINDERS; b++)
#pragma unroll
    for (int e = 0; e < CG_MAX_BINDERS; e++)
      if (b < rd.nb && e < rd.nb)
        c += ws.f_xpref[b * CG_MAX_BINDERS + e] * (rho[b] * dd[e] + dd[b] * rho[e] + dd[b] * dd[e]);
  const float vf0 = (float)g0 * sc * ws.f_vb;
  const float dvf = (float)d0 * sc * ws.f_vb;
  if (vf0 > ws.f_lim - 1e-3f || vf0 + dvf > ws.f_lim - 1e-3f) {
    acc_add(part, c);
    const ChiSplit t = chi_term64(rd, rd.has_access ? a.access_vol[rd.vox_off + v] : rd.vol_bin, g0, d0);
    acc_add_wide(part, t.soft);
    huge += t.huge;
  } else {
    acc_add(part, c + k * (dvf * (2.0f * vf0 + dvf)));
  }
  d[0] = g0 + d0;
}

// FP32 arithmetic per voxel, fixed-point accumulation into `soft` (see
// voxel_dE_f32), over the voxels of one move's table by its G lanes.
template <int G = 32>
static __device__ void field_dE_voxels(const WarpShared& ws, const KArgs& a, int hcol, const int* keys,
                                  const int* used, long long* vals, int nused, int lane,
                                  long long& n_vox, Fx& soft, double& hard, long long& huge,
                                  bool split = false) {
  const RepDev& rd = ws.rd;
  Fx part = Fx{0, 0.0};
  long long hpart = 0;
  const long long* grid = a.grid + rd.vox_off * a.ncol;
  (void)hard;
  for (int i = lane; i < nused; i += G) {
    const int slot = used[i];
    voxel_dE_f32(ws, a, grid, keys[slot], vals + (long long)slot * hcol, split, part, hpart);
  }
  n_vox = nused;
  acc_add(soft, gsum<G>(part));
  if (__any_sync(kFull, hpart != 0)) huge += gsum<G>(hpart);  // warp vote: see gsum(Fx)
}

__device__ __forceinline__ void commit_grid(const RepDev& rd, const KArgs& a, int hcol, int* keys,
                                            const int* used, long long* vals, int nused, int lane,
                                            bool accept) {
  long long* grid = a.grid + rd.vox_off * a.ncol;
  for (int i = lane; i < nused; i += 32) {
    int slot = used[i];
    if (accept) {
      int v = keys[slot];
      for (int c = 0; c < hcol; c++) grid[(long long)v * a.ncol + c] = vals[(long long)slot * hcol + c];
    }
    keys[slot] = -1;
    for (int c = 0; c < hcol; c++) vals[(long long)slot * hcol + c] = 0;
  }
}

// confinement count of one position (chromo/fields.pyx:121-202); out of
// line: confinement is off in periodic boxes and its FP64 arithmetic would
// otherwise sit in the hot loop's code
static __device__ __noinline__ int out_of_bounds3(const RepDev& rd, double x, double y, double z, bool trial) {
  if (rd.confine_kind == 1) return sqrt(x * x + y * y + z * z) > rd.confine_length ? 1 : 0;
  if (rd.confine_kind == 2 && trial)
    return (fabs(x) > rd.confine_length / 2 ? 1 : 0) + (fabs(y) > rd.confine_length / 2 ? 1 : 0) +
           (fabs(z) > rd.confine_length / 2 ? 1 : 0);
  return 0;
}
template <typename Real>
__device__ __forceinline__ int out_of_bounds(const RepDev& rd, const Real q[3], bool trial) {
  return out_of_bounds3(rd, (double)q[0], (double)q[1], (double)q[2], trial);
}
// FP32 positions in a sphere: |q|^2 in FP32 (relative error below 2e-7)
// decides every position further than 1e-5 |q|^2 from the boundary, as the
// FP64 test would; the rest take the FP64 test.
__device__ __forceinline__ int out_of_bounds(const RepDev& rd, const float q[3], bool trial) {
  if (rd.confine_kind == 1) {
    const float s = q[0] * q[0] + q[1] * q[1] + q[2] * q[2];
    const float l2 = (float)(rd.confine_length * rd.confine_length);
    if (s < l2 * 0.99999f) return 0;
    if (s > l2 * 1.00001f) return 1;
  }
  return out_of_bounds3(rd, (double)q[0], (double)q[1], (double)q[2], trial);
}

__device__ __forceinline__ double bind_f(const RepDev& rd, int b, int nm, int s) {
  return rd.bind_f[(b * (CG_MAX_MARK + 1) + nm) * (CG_MAX_MARK + 1) + s];
}

// bead_binding_dE (chromo/polymers.pyx:1408-1538) of one bead whose binder
// `bsel` goes from its current state (packed in sw, marks in mw) to s_new.
// FP64 storage: the reference's FP64 arithmetic.
__device__ __forceinline__ double bead_bind_dE(const WarpShared& ws, unsigned sw, unsigned mw, int bsel,
                                               int s_new, double) {
  const RepDev& rd = ws.rd;
  double de = 0;
  if (rd.max_binders != -1) {
    int tot_t = 0, tot_c = 0;
    for (int h = 0; h < rd.nb; h++) {
      int shh = (int)((sw >> (8 * h)) & 0xFF);
      tot_c += shh;
      tot_t += h == bsel ? s_new : shh;
    }
    if (tot_t > rd.max_binders) de += kEHugePoly * (double)(tot_t - rd.max_binders);
    if (tot_c > rd.max_binders) de -= kEHugePoly * (double)(tot_c - rd.max_binders);
  }
  for (int b = 0; b < rd.nb; b++) {
    int sc = (int)((sw >> (8 * b)) & 0xFF);
    int stt = b == bsel ? s_new : sc;
    int nm = (int)((mw >> (8 * b)) & 0xFF);
    de += bind_f(rd, b, nm, stt);
    de -= bind_f(rd, b, nm, sc);
    if (rd.mu[b] > 0) {
      double me = rd.mu[b] * (-rd.mu_adjust + 2);
      de -= (double)stt * me;
      de += (double)sc * me;
    } else {
      de -= (double)stt * rd.mu[b] * rd.mu_adjust;
      de += (double)sc * rd.mu[b] * rd.mu_adjust;
    }
  }
  return de;
}

// FP32 storage: FP32 arithmetic on the FP32 copies of the table and of the
// effective chemical potentials (terms of order 1 kT; error ~1e-7 kT).
__device__ __forceinline__ float bead_bind_dE(const WarpShared& ws, unsigned sw, unsigned mw, int bsel,
                                              int s_new, float) {
  const RepDev& rd = ws.rd;
  float de = 0;
  if (rd.max_binders != -1) {
    int tot_t = 0, tot_c = 0;
    for (int h = 0; h < rd.nb; h++) {
      int shh = (int)((sw >> (8 * h)) & 0xFF);
      tot_c += shh;
      tot_t += h == bsel ? s_new : shh;
    }
    if (tot_t > rd.max_binders) de += (float)kEHugePoly * (float)(tot_t - rd.max_binders);
    if (tot_c > rd.max_binders) de -= (float)kEHugePoly * (float)(tot_c - rd.max_binders);
  }
  for (int b = 0; b < rd.nb; b++) {
    int sc = (int)((sw >> (8 * b)) & 0xFF);
    int stt = b == bsel ? s_new : sc;
    int nm = (int)((mw >> (8 * b)) & 0xFF);
    const float* tb = ws.f_bind + (b * (CG_MAX_MARK + 1) + nm) * (CG_MAX_MARK + 1);
    de += (tb[stt] - tb[sc]) - ws.f_me[b] * (float)(stt - sc);
  }
  return de;
}

// intranucleosome term of a binding move (fields.pyx:1920-1933): into the
// FP64 part for FP64 storage, into the FF part for FP32 storage
__device__ __forceinline__ void add_intra(const WarpShared& ws, int bsel, int ddb, double&, double& hard) {
  hard += ws.rd.intra[bsel] * (double)ddb;
}
__device__ __forceinline__ void add_intra(const WarpShared& ws, int bsel, int ddb, Fx& soft, double&) {
  acc_add(soft, ws.f_intra[bsel] * (float)ddb);
}

// dE = dEp + soft + hard and the Metropolis decision on it.  FP64 storage:
// dE = (0 + dEp) + hard in FP64, as the reference sums polymer and field dE
// (mc_sim.pyx:144-171).  FP32 storage: decided on the FF sum when the FP64
// part is empty.  *dE_out (if given) receives dE in FP64.
__device__ __forceinline__ bool decide(unsigned x, double dEp, double, double hard, double* dE_out) {
  double dE = 0;
  dE += dEp;
  dE += hard;
  if (dE_out) *dE_out = dE;
  return metropolis(x, -dE);
}
__device__ __forceinline__ bool decide(unsigned x, const Fx& dEp, const Fx& soft, double hard,
                                       double* dE_out) {
  const long long q = dEp.q + soft.q;
  if (!is_zero64(dEp.hard)) hard = add_hard(hard, dEp.hard);
  if (!is_zero64(soft.hard)) hard = add_hard(hard, soft.hard);
  const bool d = metropolis_fx(x, q, hard);
  if (dE_out) *dE_out = (double)q * kFxEInv + hard;
  return d;
}
}  // namespace cg
