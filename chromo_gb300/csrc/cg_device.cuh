// cg_device.cuh -- device-side building blocks of the GB300 MC inner loop.
//
// Everything here runs inside one warp per replica.  Scalars of a move
// (random draws, bead bounds, the rotation matrix, dE totals, the decision)
// are computed redundantly and identically by all 32 lanes, so the warp never
// diverges on them; per-bead and per-voxel work is spread over the lanes.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/chromo_gb300.h"
#include "cg_math32.h"

namespace cg {

constexpr double kFxScale = 1099511627776.0;          // 2^40 fixed-point units per unit weight
constexpr double kFxInv = 1.0 / 1099511627776.0;
constexpr double kEHugePoly = 1e25;                     // chromo/polymers.pyx:35
constexpr double kEHugeField = 1e99;                    // chromo/fields.pyx:32
constexpr double kRandMax = 2147483647.0;               // glibc RAND_MAX
// The 1e99 penalties of the field (a voxel above vf_limit, fields.pyx:1832-1840;
// a bead outside the confinement, fields.pyx:121-202) are summed exactly, in
// integer units of kHugeUnit = 1e99 * 2^-40: a voxel above the limit holding
// n fixed-point units of bead weight costs huge_units(n, Vb / V) = n Vb / V
// rounded once (1e99 vf = kHugeUnit * n Vb / V), a bead outside costs 2^40.
// A move's penalty is then independent of the order of its voxels and is
// exactly zero when the weight above the limit does not change, so the
// decisions in that regime are well defined.
constexpr double kHugeUnit = kEHugeField * kFxInv;
// The running sum of accepted dE (RepDev::run_dE) leaves out moves whose dE
// carries a penalty (|dE| >= kPenaltyFloor: the 1e25 max_binders term or the
// 1e99 field terms; soft energies of a chain are many orders below): one such
// term in an FP64 sum would absorb every later dE.  Such moves only leave a
// penalised state (a move into one is never accepted), so the energy at one
// end of their interval carries the penalty itself, and differences of the
// running sum over intervals whose energies carry none stay exact.
constexpr double kPenaltyFloor = 1e20;
__device__ __forceinline__ bool soft_dE(double dE) { return fabs(dE) < kPenaltyFloor; }
constexpr unsigned kFull = 0xffffffffu;
constexpr int kMaxIter = 4096;                          // cap on resampling loops

// device-side error bits (mapped to cg_status on the host)
enum : unsigned { E_WINDOW = 1u, E_STREAM = 2u, E_NONFINITE = 4u, E_SPIN = 8u, E_DRIFT = 32u };
// internal: a move's shared-memory voxel table filled up (the move is then
// evaluated again with its global-memory table; never reported)
constexpr unsigned E_OVF = 16u;

template <typename T> struct alignas(4 * sizeof(T)) V4 { T x, y, z, w; };

// Per-replica parameters (device global; copied into shared memory per warp).
struct RepDev {
  long long bead_off, n_beads, vox_off, n_vox;
  int nx, ny, nz, nb;
  double wx, wy, wz, dx, dy, dz, vol_bin;
  int field_kind, confine_kind, max_binders, has_access;
  double confine_length, chi, vf_limit, bead_vol;
  double pref[CG_MAX_BINDERS], intra[CG_MAX_BINDERS], xpref[CG_MAX_BINDERS * CG_MAX_BINDERS];
  int sites[CG_MAX_BINDERS], fast_n;  // fast_n: sub-bins per voxel of the move deposits (0: exact)
  double mu[CG_MAX_BINDERS], mu_adjust;
  double bind_f[CG_MAX_BINDERS * (CG_MAX_MARK + 1) * (CG_MAX_MARK + 1)];
  unsigned long long draw_pos, bstate_pos;
  double run_dE;
  double xch_dE;  // energy change of this replica's accepted chi / mu swaps
  int twist, pad2;  // twist: SSTWLC bond energy (KArgs::twist holds the bond parameters)
  unsigned err, pad1;
};

// ---------------------------------------------------------------- RNG

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), counter-based.
__device__ __forceinline__ uint4 philox(uint4 c, uint2 k) {
#pragma unroll
  for (int i = 0; i < 10; i++) {
    unsigned hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
    unsigned hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
    c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
    k.x += 0x9E3779B9u;
    k.y += 0xBB67AE85u;
  }
  return c;
}

__device__ __forceinline__ unsigned comp4(uint4 v, unsigned i) {
  return i == 0 ? v.x : i == 1 ? v.y : i == 2 ? v.z : v.w;
}

// Stream of 31-bit draws (the role of libc rand()) and of binding states (the
// role of np.random.randint(0, sites + 1)).  Both are indexed: draw j of the
// replica's stream is a pure function of j, so lanes can read ahead.
template <bool AUDIT> struct Rng;

template <> struct Rng<false> {
  uint2 key, keyb;
  unsigned long long pos, bpos;
  unsigned long long cctr;
  uint4 cache;
  bool fail;
  __device__ void init(unsigned long long seed, int rep, unsigned long long p, unsigned long long bp) {
    key = make_uint2((unsigned)seed ^ (unsigned)rep * 0x85EBCA6Bu, (unsigned)(seed >> 32));
    keyb = make_uint2(key.x ^ 0x68E31DA4u, key.y ^ 0xB5297A4Du);
    pos = p; bpos = bp; cctr = ~0ull; fail = false;
  }
  __device__ __forceinline__ unsigned at(unsigned long long j, bool& ok) const {
    ok = true;
    uint4 o = philox(make_uint4((unsigned)(j >> 2), (unsigned)(j >> 34), 0x2545F491u, 0u), key);
    return comp4(o, (unsigned)(j & 3)) >> 1;
  }
  __device__ __forceinline__ unsigned next() {
    unsigned long long j = pos++, c = j >> 2;
    if (c != cctr) {
      cache = philox(make_uint4((unsigned)c, (unsigned)(c >> 32), 0x2545F491u, 0u), key);
      cctr = c;
    }
    return comp4(cache, (unsigned)(j & 3)) >> 1;
  }
  __device__ __forceinline__ int state_at(unsigned long long j, int nt, bool& ok) const {
    ok = true;
    uint4 o = philox(make_uint4((unsigned)(j >> 2), (unsigned)(j >> 34), 0x7F4A7C15u, 0u), keyb);
    return (int)__umulhi(comp4(o, (unsigned)(j & 3)), (unsigned)(nt + 1));
  }
};

template <> struct Rng<true> {
  const unsigned* draws;
  long long n;
  const signed char* bs;
  long long nbs;
  unsigned long long pos, bpos;
  bool fail;
  __device__ __forceinline__ unsigned at(unsigned long long j, bool& ok) const {
    ok = j < (unsigned long long)n;
    return ok ? draws[j] : 0u;
  }
  __device__ __forceinline__ unsigned next() {
    bool ok;
    unsigned v = at(pos++, ok);
    if (!ok) fail = true;
    return v;
  }
  __device__ __forceinline__ int state_at(unsigned long long j, int nt, bool& ok) const {
    ok = j < (unsigned long long)nbs;
    return ok ? (int)bs[j] : 0;
  }
};

// x / (2^31 - 1) correctly rounded, as the reference's rand() / RAND_MAX, with
// one FMA instead of a double division: with a = x 2^-31 (exact),
// fma(a, 2^-31 + 2^-62, a) equals the quotient for every x in [0, 2^31 - 1]
// (checked exhaustively on the host).
__device__ __forceinline__ double unif(unsigned x) {
  double a = (double)x * 0x1p-31;
  return __fma_rn(a, 0x1.00000002p-31, a);
}
// x / (2^31 - 1) to within 2^-23 relative, in FP32 only: the fast paths below
// use it with margins far above that error and fall back to unif() near a
// decision boundary.
__device__ __forceinline__ float unif32(unsigned x) { return (float)x * 4.656612873077393e-10f; }

// floor(-log10(u + 1e-5) * window * 0.45 + 1.0001) (bead_selection.pyx:56-65)
// evaluated in FP32 when the result is unambiguous, else in FP64, so the
// integer equals the reference's FP64 value.
static __device__ __noinline__ long long sel_floor64(unsigned x, long long window) {
  return (long long)(-log10(unif(x) + 0.00001) * (double)window * 0.45 + 1.0001);
}
__device__ __forceinline__ long long sel_floor(unsigned x, long long window) {
  float y = -log10f(unif32(x) + 0.00001f) * (float)window * 0.45f + 1.0001f;
  float fl = floorf(y);
  float margin = 1e-3f + 1e-6f * y;
  if (y - fl > margin && fl + 1.0f - y > margin) return (long long)fl;
  return sel_floor64(x, window);
}

// int(unif(x) * n) (the bound_0 draw of crank_shaft, move_funcs.pyx:64): in
// FP32 when the product is clear of an integer by more than its rounding
// error (relative error below 2e-7), else in FP64; same integer either way.
static __device__ __noinline__ long long scaled_index64(unsigned x, long long n) {
  return (int)(unif(x) * (double)n);
}
__device__ __forceinline__ long long scaled_index(unsigned x, long long n) {
  float y = unif32(x) * (float)n;
  float fl = floorf(y);
  float margin = 1e-4f + 4e-7f * y;
  if (y - fl > margin && fl + 1.0f - y > margin) return (long long)fl;
  return scaled_index64(x, n);
}

// The Metropolis test u < exp(t) (mc_sim.pyx:164-171) with u = unif(x):
// decided in FP32 away from the boundary, in FP64 near it; same outcome as
// the FP64 comparison.
static __device__ __noinline__ bool metropolis(unsigned x, double t) {
  double u = unif(x);
  if (t != t) return false;
  if (t > 80.0) return true;
  if (t >= -80.0) {
    double e = (double)expf((float)t);
    if (u < e * (1.0 - 1e-4)) return true;
    if (u > e * (1.0 + 1e-4)) return false;
  } else if (u > 0.0) {
    return false;
  }
  return u < exp(t);
}

// ---------------------------------------------------------------- FP32 sums
// FF: unevaluated sum hi + lo of two binary32 numbers (Knuth's TwoSum with
// Dekker's renormalisation), for the three terms of one bond's energy.  Both
// operands enter symmetrically (the TwoSum error term is the exact rounding
// error).
struct FF { float hi, lo; };

__device__ __forceinline__ FF ff_add(FF a, FF b) {
  float s = a.hi + b.hi;
  float bb = s - a.hi;
  float e = (a.hi - (s - bb)) + (b.hi - bb);
  e += a.lo + b.lo;
  float hi = s + e;
  return FF{hi, e - (hi - s)};
}
__device__ __forceinline__ FF ff_add(FF a, float b) { return ff_add(a, FF{b, 0.0f}); }

// True when an FP64 value is +0 or -0 (integer test, no FP64 instruction)
__device__ __forceinline__ bool is_zero64(double v) { return (__double_as_longlong(v) << 1) == 0; }

// dE of the FP32 path in fixed point: every FP32 energy term is rounded to a
// multiple of 2^-30 kT (error at most 2^-31 kT per term) and the terms are
// summed exactly in int64.  The sum therefore does not depend on the order of
// the terms -- on how beads and voxels are spread over lanes, or on the order
// in which voxels were first touched -- and needs no FP64 instruction (FP64
// runs at 1/64 of the FP32 rate on GB300).  Terms of 2^20 kT or more, and
// non-finite ones, go to an FP64 side sum `hard` (rare: a 1e25 max_binders
// penalty, an extreme bond).
constexpr double kFxEInv = 1.0 / 1073741824.0;  // kT per fixed-point unit

// round(x * 2^30), ties to even, for |x| < 2^20, with 32-bit conversions only:
// a = |x| 2^10 < 2^30 is exact, floor(a) 2^20 is even, and (a - floor(a)) 2^20
// is exact, so rounding that fraction rounds the whole.
__device__ __forceinline__ long long q30(float x) {
  const float a = fabsf(x) * 1024.0f;
  const float fl = floorf(a);
  const long long q = (long long)(int)fl * 1048576LL + (long long)(int)rintf((a - fl) * 1048576.0f);
  return x < 0.0f ? -q : q;
}

struct Fx {
  long long q;  // sum of the terms in units of 2^-30 kT
  double hard;  // FP64 sum of the terms outside the fixed-point range
};

// Accumulator of the arithmetic of each storage type: FP64 storage sums in
// FP64 (the reference's arithmetic), FP32 storage in fixed point.
template <typename Real> struct AccOf { using type = double; };
template <> struct AccOf<float> { using type = Fx; };
__device__ __forceinline__ void acc_add(double& s, double v) { s += v; }
// a + b for the FP64 side sums, which are almost always zero: out of line,
// so that a guarded add stays a branch instead of becoming an FP64 add on
// every lane (FP64 issues at a small fraction of the FP32 rate here)
static __device__ __noinline__ double add_hard(double a, double b) { return a + b; }
__device__ __forceinline__ void acc_add(Fx& s, float x) {
  if (fabsf(x) < 1048576.0f) s.q += q30(x);
  else s.hard = add_hard(s.hard, (double)x);
}
__device__ __forceinline__ void acc_add(Fx& s, FF v) { acc_add(s, v.hi); acc_add(s, v.lo); }
__device__ __forceinline__ void acc_add(Fx& s, const Fx& v) {
  s.q += v.q;
  if (!is_zero64(v.hard)) s.hard = add_hard(s.hard, v.hard);
}
// An FP64 term (the twist part of a bond's dE): added as FP64 for FP64
// storage, rounded to FP32 and added in fixed point for FP32 storage (its
// relative error 6e-8 is far inside the path's 1e-5 bound).
__device__ __forceinline__ void acc_add_d(double& s, double v) { s += v; }
__device__ __forceinline__ void acc_add_d(Fx& s, double v) { acc_add(s, (float)v); }
__device__ __forceinline__ double acc_d(double v) { return v; }
__device__ __forceinline__ double acc_d(const Fx& v) { return (double)v.q * kFxEInv + v.hard; }
template <typename A> __device__ __forceinline__ A acc_zero();
template <> __device__ __forceinline__ double acc_zero<double>() { return 0.0; }
template <> __device__ __forceinline__ Fx acc_zero<Fx>() { return Fx{0, 0.0}; }

// The Metropolis test of the FP32 path on dE = q 2^-30 + hard: decided in
// FP32 when `hard` is empty and u and exp(-dE) differ by more than 1e-4
// relative (the FP32 errors of u, of exp and of converting q stay below 1e-5
// for |dE| <= 80), else by metropolis() on the FP64 value of dE.
__device__ __forceinline__ bool metropolis_fx(unsigned x, long long q, double hard) {
  if (is_zero64(hard)) {
    const float th = -(float)q * 9.313225746154785e-10f;
    if (th > 81.0f) return true;
    if (th < -81.0f && x != 0u) return false;
    if (th >= -80.0f && th <= 80.0f) {
      const float u = unif32(x), e = expf(th);
      if (u < e * 0.9999f) return true;
      if (u > e * 1.0001f) return false;
    }
  }
  return metropolis(x, -((double)q * kFxEInv + hard));
}

// ---------------------------------------------------------------- bead selection
// chromo/util/bead_selection.pyx:19-192

template <class R>
__device__ long long capped_exponential(R& g, long long window, long long cap, unsigned& err) {
  long long r = sel_floor(g.next(), window);
  int it = 0;
  while (r > cap) {
    if (g.fail) return cap;  // stream exhausted: reported by the caller
    if (++it > kMaxIter) { err |= E_SPIN; return cap; }
    r = sel_floor(g.next(), window);
  }
  return r;
}

template <class R>
__device__ long long from_left(R& g, long long window, long long n, unsigned& err) {
  if (window > n) { err |= E_WINDOW; return 0; }
  return capped_exponential(g, window, window, err);
}

template <class R>
__device__ long long from_point(R& g, long long window, long long n, long long ind0, unsigned& err) {
  if (window > n) { err |= E_WINDOW; return 0; }
  if (window < 1) return ind0;
  long long side = g.next() & 1u;
  if (side == 0) {
    long long ws = window < ind0 ? window : ind0;
    if (ws < 1) ws = 1;
    long long ub = ind0 > 1 ? ind0 : 1;
    return ub - from_left(g, ws, ub, err);
  }
  long long rem = n - ind0;
  long long ws = window < rem ? window : rem;
  if (ws < 1) ws = 1;
  long long ub = rem > 1 ? rem : 1;
  return from_left(g, ws, ub, err) + ind0;
}

__device__ __forceinline__ void check_bead_bounds(long long b0, long long b1, long long n,
                                                  long long& i0, long long& i1) {
  if (b0 > n) b0 = n;
  if (b0 < 0) b0 = 0;
  if (b1 > n) { i0 = b0; i1 = n; }
  else if (b1 < 0) { i0 = 0; i1 = b0 + 1; }
  else if (b0 == b1) { i0 = b0; i1 = b0 + 1; }
  else { i0 = b0 < b1 ? b0 : b1; i1 = b0 > b1 ? b0 : b1; }
}

// ---------------------------------------------------------------- geometry
// chromo/util/linalg.pyx:23-199

// Proposal math.  FP64 storage: the CUDA FP64 functions, as the reference
// uses libm.  FP32 storage: the deterministic binary32 functions of
// cg_math32.h, which the host oracle compiles from the same source.
__device__ __forceinline__ void rsincos(double x, double* sn, double* cs) { sincos(x, sn, cs); }
__device__ __forceinline__ void rsincos(float x, float* sn, float* cs) { cgm_sincosf(x, sn, cs); }
__device__ __forceinline__ double racos(double x) { return acos(x); }
__device__ __forceinline__ float racos(float x) { return cgm_acosf(x); }
__device__ __forceinline__ double rsqrt_(double x) { return sqrt(x); }
__device__ __forceinline__ float rsqrt_(float x) { return sqrtf(x); }

template <typename Real> __device__ __forceinline__ Real uni(unsigned x);
template <> __device__ __forceinline__ double uni<double>(unsigned x) { return unif(x); }
template <> __device__ __forceinline__ float uni<float>(unsigned x) { return cgm_unif24(x); }

// uniform_sample_unit_sphere from two draws (phi, theta)
template <typename Real>
__device__ __forceinline__ void sphere_from(unsigned xphi, unsigned xtheta, Real v[3]) {
  Real phi = uni<Real>(xphi) * (Real)(2.0 * 3.141592653589793);
  Real theta = racos(uni<Real>(xtheta) * 2 - 1);
  Real sp, cp, st, ct;
  rsincos(phi, &sp, &cp);
  rsincos(theta, &st, &ct);
  v[0] = cp * st;
  v[1] = sp * st;
  v[2] = ct;
}

template <typename Real, class R>
__device__ __forceinline__ void sphere(R& g, Real v[3]) {
  unsigned a = g.next();
  unsigned b = g.next();
  sphere_from<Real>(a, b, v);
}

// Rotation by `ang` (sine s, cosine c) about unit axis a through point p:
// x' = M[:, :3] x + M[:, 3].
template <typename Real>
__device__ __forceinline__ void axis_rotation_sc(const Real a[3], const Real p[3], Real s, Real c,
                                                 Real M[3][4]) {
  Real oc = 1 - c, a0 = a[0] * a[0], a1 = a[1] * a[1], a2 = a[2] * a[2];
  M[0][0] = a0 + (a1 + a2) * c;
  M[0][1] = a[0] * a[1] * oc - a[2] * s;
  M[0][2] = a[0] * a[2] * oc + a[1] * s;
  M[1][0] = a[0] * a[1] * oc + a[2] * s;
  M[1][1] = a1 + (a0 + a2) * c;
  M[1][2] = a[1] * a[2] * oc - a[0] * s;
  M[2][0] = a[0] * a[2] * oc - a[1] * s;
  M[2][1] = a[1] * a[2] * oc + a[0] * s;
  M[2][2] = a2 + (a0 + a1) * c;
  M[0][3] = (p[1] * a[2] - p[2] * a[1]) * s;
  M[1][3] = (p[2] * a[0] - p[0] * a[2]) * s;
  M[2][3] = (p[0] * a[1] - p[1] * a[0]) * s;
  M[0][3] += (p[0] * (1 - a0) - a[0] * (p[1] * a[1] + p[2] * a[2])) * oc;
  M[1][3] += (p[1] * (1 - a1) - a[1] * (p[0] * a[0] + p[2] * a[2])) * oc;
  M[2][3] += (p[2] * (1 - a2) - a[2] * (p[0] * a[0] + p[1] * a[1])) * oc;
}

template <typename Real>
__device__ __forceinline__ void axis_rotation(const Real a[3], const Real p[3], Real ang, Real M[3][4]) {
  Real s, c;
  rsincos(ang, &s, &c);
  axis_rotation_sc(a, p, s, c, M);
}

template <typename Pos, typename Real>
__device__ __forceinline__ void ld3(const V4<Pos>* a, long long i, Real v[3]) {
  V4<Pos> q = a[i];
  v[0] = (Real)q.x; v[1] = (Real)q.y; v[2] = (Real)q.z;
}

template <typename Pos>
__device__ __forceinline__ double rnd_pos(double x) { return (double)(Pos)x; }

// ---------------------------------------------------------------- SSWLC energy
// chromo/polymers.pyx:1148-1346

template <typename Real> struct Bond { Real eb, g, ep, epp, eta; };

template <typename Real>
__device__ __forceinline__ Bond<Real> load_bond(const double* bonds, long long i) {
  const double* b = bonds + 6 * i;
  return Bond<Real>{(Real)b[0], (Real)b[1], (Real)b[2], (Real)b[3], (Real)b[4]};
}

// Bond i of the storage type's arithmetic: FP64 parameters for FP64 storage,
// their FP32 copy (one 16-byte and one 4-byte load) for FP32 storage.
__device__ __forceinline__ Bond<double> bond_at(const double* b64, const float*, long long i, double) {
  return load_bond<double>(b64, i);
}
__device__ __forceinline__ Bond<float> bond_at(const double*, const float* b32, long long i, float) {
  const float4 q = *reinterpret_cast<const float4*>(b32 + 8 * i);
  return Bond<float>{q.x, q.y, q.z, q.w, b32[8 * i + 4]};
}

template <typename Real>
__device__ __forceinline__ Real e_pair(const Bond<Real>& b, const Real bend[3], Real par, const Real dp[3]) {
  Real x = par - b.g;
  return (Real)0.5 * b.eb * (bend[0] * bend[0] + bend[1] * bend[1] + bend[2] * bend[2])
       + (Real)0.5 * b.ep * (x * x)
       + (Real)0.5 * b.epp * (dp[0] * dp[0] + dp[1] * dp[1] + dp[2] * dp[2]);
}

// bond (0 -> 1) with bead 1 moved: bead_pair_dE_poly_forward (FP64 difference)
template <typename Real>
__device__ __forceinline__ double pair_dE_fwd(const Bond<Real>& b, const Real r0[3], const Real r1[3],
                                              const Real tr1[3], const Real t30[3],
                                              const Real t31[3], const Real tt31[3]) {
  Real drt[3], dr[3], dpt[3], dp[3], bt[3], bc[3];
  for (int i = 0; i < 3; i++) { drt[i] = tr1[i] - r0[i]; dr[i] = r1[i] - r0[i]; }
  Real pt = t30[0] * drt[0] + t30[1] * drt[1] + t30[2] * drt[2];
  Real pc = t30[0] * dr[0] + t30[1] * dr[1] + t30[2] * dr[2];
  for (int i = 0; i < 3; i++) {
    dpt[i] = drt[i] - t30[i] * pt;
    dp[i] = dr[i] - t30[i] * pc;
    bt[i] = tt31[i] - t30[i] - dpt[i] * b.eta;
    bc[i] = t31[i] - t30[i] - dp[i] * b.eta;
  }
  return (double)e_pair(b, bt, pt, dpt) - (double)e_pair(b, bc, pc, dp);
}

// bond (0 -> 1) with bead 0 moved: bead_pair_dE_poly_reverse (FP64 difference)
template <typename Real>
__device__ __forceinline__ double pair_dE_rev(const Bond<Real>& b, const Real r0[3], const Real tr0[3],
                                              const Real r1[3], const Real t30[3],
                                              const Real tt30[3], const Real t31[3]) {
  Real drt[3], dr[3], dpt[3], dp[3], bt[3], bc[3];
  for (int i = 0; i < 3; i++) { drt[i] = r1[i] - tr0[i]; dr[i] = r1[i] - r0[i]; }
  Real pt = tt30[0] * drt[0] + tt30[1] * drt[1] + tt30[2] * drt[2];
  Real pc = t30[0] * dr[0] + t30[1] * dr[1] + t30[2] * dr[2];
  for (int i = 0; i < 3; i++) {
    dpt[i] = drt[i] - tt30[i] * pt;
    dp[i] = dr[i] - t30[i] * pc;
    bt[i] = t31[i] - tt30[i] - dpt[i] * b.eta;
    bc[i] = t31[i] - t30[i] - dp[i] * b.eta;
  }
  return (double)e_pair(b, bt, pt, dpt) - (double)e_pair(b, bc, pc, dp);
}

// ---------------------------------------------------------------- SSTWLC twist
// E_pair_with_twist (chromo/polymers.pyx:2050-2102) adds 0.5 eps_twist dw^2 to
// the bond energy, dw = omega - omega0 wrapped into [-pi, pi), omega the
// twist angle of the two beads' (t2, t3) frames
// (compute_twist_angle_omega, :3427-3461): with t1 = t2 x t3,
// omega = atan2(t2_0 . t1_1 - t1_0 . t2_1, t1_0 . t1_1 + t2_0 . t2_1).
// Evaluated in FP64 for both storage types (a few bonds per move, twist
// chains only).
struct Frame {
  double t2[3], t3[3];
};
template <typename Real>
__device__ __forceinline__ Frame frame_of(const Real t2[3], const Real t3[3]) {
  return Frame{{(double)t2[0], (double)t2[1], (double)t2[2]}, {(double)t3[0], (double)t3[1], (double)t3[2]}};
}
template <typename Pos>
__device__ __forceinline__ Frame frame_of(const V4<Pos>& t2, const V4<Pos>& t3) {
  return Frame{{(double)t2.x, (double)t2.y, (double)t2.z}, {(double)t3.x, (double)t3.y, (double)t3.z}};
}
__device__ __forceinline__ double twist_energy(const double* tw, const Frame& a, const Frame& b) {
  const double t1a[3] = {a.t2[1] * a.t3[2] - a.t2[2] * a.t3[1], a.t2[2] * a.t3[0] - a.t2[0] * a.t3[2],
                         a.t2[0] * a.t3[1] - a.t2[1] * a.t3[0]};
  const double t1b[3] = {b.t2[1] * b.t3[2] - b.t2[2] * b.t3[1], b.t2[2] * b.t3[0] - b.t2[0] * b.t3[2],
                         b.t2[0] * b.t3[1] - b.t2[1] * b.t3[0]};
  const double y = (a.t2[0] * t1b[0] + a.t2[1] * t1b[1] + a.t2[2] * t1b[2]) -
                   (t1a[0] * b.t2[0] + t1a[1] * b.t2[1] + t1a[2] * b.t2[2]);
  const double x = (t1a[0] * t1b[0] + t1a[1] * t1b[1] + t1a[2] * t1b[2]) +
                   (a.t2[0] * b.t2[0] + a.t2[1] * b.t2[1] + a.t2[2] * b.t2[2]);
  const double kPi = 3.141592653589793;
  double dw = atan2(y, x) - tw[1];
  dw -= 2 * kPi * floor((dw + kPi) / (2 * kPi));
  return 0.5 * tw[0] * (dw * dw);
}
// twist part of a bond's dE: E(a_new, b_new) - E(a_cur, b_cur); tw = (eps_twist, omega0)
static __device__ __noinline__ double twist_pair_dE(const double* tw, Frame a_cur, Frame b_cur, Frame a_new,
                                                    Frame b_new) {
  return twist_energy(tw, a_new, b_new) - twist_energy(tw, a_cur, b_cur);
}
static __device__ __noinline__ double twist_bond_energy(const double* tw, Frame a, Frame b) {
  return twist_energy(tw, a, b);
}

// (x + y + z) / 2 as FF
__device__ __forceinline__ FF half_sum3(float x, float y, float z) {
  FF s = ff_add(FF{x, 0.0f}, y);
  s = ff_add(s, z);
  return FF{0.5f * s.hi, 0.5f * s.lo};
}

// FP32 evaluation of E_pair(trial) - E_pair(current) in difference form:
// |b_t|^2 - |b_c|^2 = sum (b_t - b_c)(b_t + b_c) and likewise for the other
// two terms, with the differences formed from the (small) input differences,
// so the rounding error scales with dE rather than with E.
// Forward bond (bead 1 moved; bead 0 and its tangent fixed).
__device__ __forceinline__ FF pair_dE_fwd(const Bond<float>& b, const float r0[3], const float r1[3],
                                              const float tr1[3], const float t30[3],
                                              const float t31[3], const float tt31[3]) {
  float drt[3], dr[3], ddr[3];
  for (int i = 0; i < 3; i++) { drt[i] = tr1[i] - r0[i]; dr[i] = r1[i] - r0[i]; ddr[i] = tr1[i] - r1[i]; }
  float pt = t30[0] * drt[0] + t30[1] * drt[1] + t30[2] * drt[2];
  float pc = t30[0] * dr[0] + t30[1] * dr[1] + t30[2] * dr[2];
  float dpar = t30[0] * ddr[0] + t30[1] * ddr[1] + t30[2] * ddr[2];
  float e_par = dpar * ((pt - b.g) + (pc - b.g));
  float e_perp = 0, e_bend = 0;
  for (int i = 0; i < 3; i++) {
    float dpt = drt[i] - t30[i] * pt, dp = dr[i] - t30[i] * pc;
    float ddp = ddr[i] - t30[i] * dpar;
    float bt = tt31[i] - t30[i] - dpt * b.eta, bc = t31[i] - t30[i] - dp * b.eta;
    float db = (tt31[i] - t31[i]) - ddp * b.eta;
    e_perp += ddp * (dpt + dp);
    e_bend += db * (bt + bc);
  }
  return half_sum3(b.eb * e_bend, b.ep * e_par, b.epp * e_perp);
}

// Reverse bond (bead 0 moved; bead 1 fixed).
__device__ __forceinline__ FF pair_dE_rev(const Bond<float>& b, const float r0[3], const float tr0[3],
                                              const float r1[3], const float t30[3],
                                              const float tt30[3], const float t31[3]) {
  float drt[3], dr[3], ddr[3], dt[3];
  for (int i = 0; i < 3; i++) {
    drt[i] = r1[i] - tr0[i]; dr[i] = r1[i] - r0[i]; ddr[i] = r0[i] - tr0[i]; dt[i] = tt30[i] - t30[i];
  }
  float pt = tt30[0] * drt[0] + tt30[1] * drt[1] + tt30[2] * drt[2];
  float pc = t30[0] * dr[0] + t30[1] * dr[1] + t30[2] * dr[2];
  float dpar = (tt30[0] * ddr[0] + tt30[1] * ddr[1] + tt30[2] * ddr[2])
             + (dt[0] * dr[0] + dt[1] * dr[1] + dt[2] * dr[2]);
  float e_par = dpar * ((pt - b.g) + (pc - b.g));
  float e_perp = 0, e_bend = 0;
  for (int i = 0; i < 3; i++) {
    float dpt = drt[i] - tt30[i] * pt, dp = dr[i] - t30[i] * pc;
    float ddp = ddr[i] - (dt[i] * pt + t30[i] * dpar);
    float bt = t31[i] - tt30[i] - dpt * b.eta, bc = t31[i] - t30[i] - dp * b.eta;
    float db = -dt[i] - ddp * b.eta;
    e_perp += ddp * (dpt + dp);
    e_bend += db * (bt + bc);
  }
  return half_sum3(b.eb * e_bend, b.ep * e_par, b.epp * e_perp);
}

// ---------------------------------------------------------------- density field
// chromo/fields.pyx:1430-1673: eight trilinear weights and periodic voxel indices.

__device__ __forceinline__ double pymod(double a, double b) {
  if (a >= 0 && a < b) return a;  // fmod(a, b) == a exactly here
  double m = fmod(a, b);
  if (m != 0 && ((m < 0) != (b < 0))) m += b;
  return m;
}
__device__ __forceinline__ float pymodf(float a, float b) {
  if (a >= 0 && a < b) return a;
  float m = fmodf(a, b);
  if (m != 0 && ((m < 0) != (b < 0))) m += b;
  return m;
}

// FP32 copies of the grid geometry, derived once per launch
struct GridF {
  float w[3], half_w[3], half_d[3], inv_d[3];
  float sw[3], inv_sw[3], nsub[3], half_np;  // fast_field sub-bins (FP32 storage)
  int n[3], nx, nxy;
};

__device__ __forceinline__ void make_gridf(const RepDev& rd, GridF& gf) {
  const double W[3] = {rd.wx, rd.wy, rd.wz};
  const int n[3] = {rd.nx, rd.ny, rd.nz};
  for (int j = 0; j < 3; j++) {
    double d = W[j] / (double)n[j];
    gf.w[j] = (float)W[j];
    gf.half_w[j] = (float)(0.5 * W[j]);
    gf.half_d[j] = (float)(0.5 * d);
    gf.inv_d[j] = (float)(1.0 / d);
    gf.n[j] = n[j];
    const int np = rd.fast_n > 0 ? rd.fast_n : 1;
    gf.sw[j] = (float)(d / (double)np);
    gf.inv_sw[j] = (float)((double)np / d);
    gf.nsub[j] = (float)((double)np * n[j]);
  }
  gf.half_np = (float)(0.5 * (rd.fast_n > 0 ? rd.fast_n : 1));
  gf.nx = rd.nx;
  gf.nxy = rd.nx * rd.ny;
}

// Per axis: the lower and upper voxel of a bead and the lower voxel's weight
// (fields.pyx:1524-1673).  Exact reference arithmetic (FP64 storage).
__device__ __forceinline__ void voxel_axes(const RepDev& rd, const GridF&, const double pos[3],
                                           double wl[3], int lo[3], int hi[3]) {
  const double width[3] = {rd.wx, rd.wy, rd.wz};
  const int n[3] = {rd.nx, rd.ny, rd.nz};
#pragma unroll
  for (int j = 0; j < 3; j++) {
    double d = width[j] / (double)n[j];
    double x = pymod(pos[j] + 0.5 * width[j], width[j]) - 0.5 * d;
    long long ind = (long long)floor(x / d);
    int li = ind == -1 ? n[j] - 1 : (int)ind;
    lo[j] = li < 0 ? 0 : (li >= n[j] ? n[j] - 1 : li);  // in range for finite x; guards the rest
    hi[j] = lo[j] + 1 == n[j] ? 0 : lo[j] + 1;
    wl[j] = 1 - (x / d - (double)ind);
  }
}

// FP32 arithmetic (FP32 storage): same construction, one reciprocal multiply.
__device__ __forceinline__ void voxel_axes(const RepDev&, const GridF& gf, const float pos[3],
                                           float wl[3], int lo[3], int hi[3]) {
#pragma unroll
  for (int j = 0; j < 3; j++) {
    float x = pymodf(pos[j] + gf.half_w[j], gf.w[j]) - gf.half_d[j];
    float t = x * gf.inv_d[j];
    float fl = floorf(t);
    int ind = (int)fl;
    int li = ind == -1 ? gf.n[j] - 1 : ind;
    lo[j] = li < 0 ? 0 : (li >= gf.n[j] ? gf.n[j] - 1 : li);
    hi[j] = lo[j] + 1 == gf.n[j] ? 0 : lo[j] + 1;
    wl[j] = 1 - (t - fl);
  }
}

// The sub-bin version of voxel_axes for per-move density changes with
// fast_field (get_change_in_density_quickly, fields.pyx:1235-1368, with the
// tables of init_fast_field, :577-671): each coordinate is moved to the lower
// edge of its sub-bin, floor((x + L/2) / w_sub) mod (n_points n), w_sub =
// d / n_points, and the voxel and weight are those of that edge, shifted by
// half a voxel.  FP64: the reference's arithmetic.
__device__ __forceinline__ void fast_axes(const RepDev& rd, const GridF&, const double pos[3],
                                          double wl[3], int lo[3], int hi[3]) {
  const double width[3] = {rd.wx, rd.wy, rd.wz};
  const int n[3] = {rd.nx, rd.ny, rd.nz};
  const double np = (double)rd.fast_n;
#pragma unroll
  for (int j = 0; j < 3; j++) {
    const double d = width[j] / (double)n[j];
    const double sw = d / np;
    const double sb = pymod(floor((pos[j] + 0.5 * width[j]) / sw), np * (double)n[j]);
    const double q = ((sb - np / 2) * sw) / d;
    const double ind = floor(q);
    const int li = ind == -1.0 ? n[j] - 1 : (int)ind;
    lo[j] = li < 0 ? 0 : (li >= n[j] ? n[j] - 1 : li);
    hi[j] = lo[j] + 1 == n[j] ? 0 : lo[j] + 1;
    wl[j] = 1 - (q - ind);
  }
}
// FP32 storage: the same construction in binary32.
__device__ __forceinline__ void fast_axes(const RepDev&, const GridF& gf, const float pos[3], float wl[3],
                                          int lo[3], int hi[3]) {
#pragma unroll
  for (int j = 0; j < 3; j++) {
    const float sb = pymodf(floorf((pos[j] + gf.half_w[j]) * gf.inv_sw[j]), gf.nsub[j]);
    const float q = ((sb - gf.half_np) * gf.sw[j]) * gf.inv_d[j];
    const float fl = floorf(q);
    const int ind = (int)fl;
    const int li = ind == -1 ? gf.n[j] - 1 : ind;
    lo[j] = li < 0 ? 0 : (li >= gf.n[j] ? gf.n[j] - 1 : li);
    hi[j] = lo[j] + 1 == gf.n[j] ? 0 : lo[j] + 1;
    wl[j] = 1 - (q - fl);
  }
}
// Per-axis voxels and weights of a move's density change: the sub-bin ones
// with fast_field, else the exact ones (full deposits always use the exact
// ones, as the reference's update_all_densities does).  Out of line for
// fast_field, which production runs leave off.
template <typename Real>
static __device__ __noinline__ void fast_axes_ool(const RepDev& rd, const GridF& gf, const Real pos[3],
                                                  Real wl[3], int lo[3], int hi[3]) {
  fast_axes(rd, gf, pos, wl, lo, hi);
}
template <typename Real>
__device__ __forceinline__ void move_axes(const RepDev& rd, const GridF& gf, const Real pos[3], Real wl[3],
                                          int lo[3], int hi[3]) {
  if (rd.fast_n > 0) fast_axes_ool(rd, gf, pos, wl, lo, hi);
  else voxel_axes(rd, gf, pos, wl, lo, hi);
}

// Corner l (bit 0: x, bit 1: y, bit 2: z upper) of the eight trilinear
// weights and its voxel index.
template <typename Real>
__device__ __forceinline__ void voxel_corner(const GridF& gf, const Real wl[3], const int lo[3],
                                             const int hi[3], int l, Real& w, int& v) {
  const int bx = l & 1, by = (l >> 1) & 1, bz = (l >> 2) & 1;
  const Real fx = bx ? (1 - wl[0]) : wl[0];
  const Real fy = by ? (1 - wl[1]) : wl[1];
  const Real fz = bz ? (1 - wl[2]) : wl[2];
  w = fx * fy * fz;
  v = (bx ? hi[0] : lo[0]) + gf.nx * (by ? hi[1] : lo[1]) + gf.nxy * (bz ? hi[2] : lo[2]);
}

template <typename Real>
__device__ __forceinline__ void voxel_weights(const RepDev& rd, const GridF& gf, const Real pos[3],
                                              Real w[8], int v[8]) {
  Real wl[3];
  int lo[3], hi[3];
  voxel_axes(rd, gf, pos, wl, lo, hi);
#pragma unroll
  for (int l = 0; l < 8; l++) voxel_corner(gf, wl, lo, hi, l, w[l], v[l]);
}

template <typename Real>
__device__ __forceinline__ void move_weights(const RepDev& rd, const GridF& gf, const Real pos[3],
                                             Real w[8], int v[8]) {
  Real wl[3];
  int lo[3], hi[3];
  move_axes(rd, gf, pos, wl, lo, hi);
#pragma unroll
  for (int l = 0; l < 8; l++) voxel_corner(gf, wl, lo, hi, l, w[l], v[l]);
}

__device__ __forceinline__ long long q40(double w) { return __double2ll_rn(w * kFxScale); }
// penalty units of a voxel above vf_limit (see kHugeUnit)
__device__ __forceinline__ long long huge_units(long long n, double vb_over_v) {
  return __double2ll_rn((double)n * vb_over_v);
}
__device__ __forceinline__ long long q40(float w) { return cgm_q40f(w); }

// ---------------------------------------------------------------- warp helpers

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}
// Reductions over aligned groups of G lanes (G = 8, 16, 32): every lane of a
// group ends with the group's total.  Must be called by the whole warp.
template <int G> __device__ __forceinline__ double gsum(double v) {
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}
template <int G> __device__ __forceinline__ long long gsum(long long v) {
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}
template <int G> __device__ __forceinline__ int gsum(int v) {
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}
template <int G> __device__ __forceinline__ unsigned gor(unsigned v) {
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) v |= __shfl_xor_sync(kFull, v, o);
  return v;
}
// The group's votes as G bits (lane gl of the group -> bit gl).
template <int G> __device__ __forceinline__ unsigned gballot(bool p) {
  const unsigned b = __ballot_sync(kFull, p);
  if (G == 32) return b;
  return (b >> ((threadIdx.x & 31u) & ~(unsigned)(G - 1))) & ((1u << (G & 31)) - 1u);
}
template <int G> __device__ __forceinline__ bool gany(bool p) { return gballot<G>(p) != 0u; }
// Fixed-point sums are exact; the FP64 side sum is reduced only when some
// lane of the warp holds one.  The test is a warp vote, not a group vote: the
// reduction's shuffles name all 32 lanes, so with G < 32 every group of the
// warp must take the branch together (a group that holds only zeros adds
// zeros).
template <int G> __device__ __forceinline__ Fx gsum(Fx v) {
  v.q = gsum<G>(v.q);
  if (__any_sync(kFull, !is_zero64(v.hard))) v.hard = gsum<G>(v.hard);
  return v;
}
__device__ __forceinline__ Fx warp_sum(Fx v) { return gsum<32>(v); }
__device__ __forceinline__ long long warp_sum_ll(long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

}  // namespace cg
