// cg_spec.cuh -- the production MC kernel: several moves of a replica in flight.
//
// One CTA per replica, W warps, each warp split into 32 / G groups of G lanes
// (G = 8, 16 or 32).  Every group evaluates one move, so S = W * 32 / G moves
// are in flight.  Within one controller's cycle (same move kind, fixed
// amplitudes) the next S attempted moves are evaluated at once, group s taking
// move t0 + s, all against the state before the batch.  Then:
//
//   * each move's read/write footprint -- the beads it reads or writes and
//     the voxels it touches -- is compared with the footprints of the earlier
//     moves of the batch (beads by index range, voxels through a block-wide
//     voxel -> move-bitmask table);
//   * walking the batch in order, move s stands iff no earlier *accepted*
//     move's footprint meets its own; the first move that fails, and every
//     later one, is evaluated again in the next batch on the updated state;
//   * the standing accepted moves are committed; their footprints are
//     disjoint, so the commits do not interact.
//
// The result is exactly that of applying the moves one after the other (a
// rejected move changes nothing; an accepted move only changes its own
// footprint), for every W and G: each attempted move takes its random numbers
// from its own Philox4x32-10 sub-stream, indexed by (replica, move number,
// draw number), and the FP32 path sums dE exactly in fixed point, so neither
// the spread of beads and voxels over lanes nor the order of hash claims
// changes a bit.  Acceptance statistics and the controllers' amplitude updates
// are applied in move order as in the one-move-at-a-time loop
// (chromo/mc/mc_sim.pyx:88-182).
//
// Several moves per warp: a move of a few beads (the mean segment of the
// benchmark's moves is 4-20 beads) leaves most of a warp's lanes idle, and the
// scalar part of a move (draws, bead selection, rotation, Metropolis) is
// computed redundantly by all lanes of its group; with G = 16 or 8 one warp
// instruction serves 2 or 4 moves.  Every warp-collective operation below is
// executed by the whole warp with per-group masks, so groups may diverge only
// in code without collectives.
#pragma once
#include <cuda_runtime.h>

#include "cg_device.cuh"
#include "cg_kernels.h"
#include "cg_move.cuh"

namespace cg {

// Draw j (>= kDrawCache) of a move's sub-stream: word j & 3 of Philox block
// j >> 2.  Out of line: few moves draw this many numbers, and inlined at every
// draw site the rounds would fill the instruction cache.
static __device__ __noinline__ unsigned move_draw_slow(uint2 key, unsigned tlo, unsigned thi,
                                                       unsigned long long j) {
  uint4 o = philox(make_uint4((unsigned)(j >> 2), tlo, thi, 0x2545F491u), key);
  return comp4(o, (unsigned)j & 3u) >> 1;
}

// Random numbers of one attempted move (its own counter space).  Draw j is
// word j & 3 of Philox block j >> 2.  The first kDrawCache draws are computed
// at init by the move's G lanes into its shared-memory buffer, so a move's
// draws cost one Philox latency instead of a chain of them; init() must be
// called by the whole warp.
struct MoveRng {
  uint2 key, keyb;
  unsigned tlo, thi;
  unsigned long long pos, bpos;
  const unsigned* buf;
  bool fail;
  template <int G>
  __device__ void init(unsigned long long seed, int rep, unsigned long long t, unsigned* draws, int gl) {
    key = make_uint2((unsigned)seed ^ (unsigned)rep * 0x85EBCA6Bu, (unsigned)(seed >> 32) ^ 0x1B873593u);
    keyb = make_uint2(key.x ^ 0x68E31DA4u, key.y ^ 0xB5297A4Du);
    tlo = (unsigned)t;
    thi = (unsigned)(t >> 32);
    pos = 0; bpos = 0; fail = false;
    for (int j = gl; j < kDrawCache / 4; j += G) {
      uint4 o = philox(make_uint4((unsigned)j, tlo, thi, 0x2545F491u), key);
      reinterpret_cast<uint4*>(draws)[j] = o;
    }
    __syncwarp();
    buf = draws;
  }
  __device__ __forceinline__ unsigned next() { return word(pos++); }
  // draw j, from the cache when it holds it
  __device__ __forceinline__ unsigned word(unsigned long long j) const {
    if (j < (unsigned long long)kDrawCache) return buf[j] >> 1;
    return move_draw_slow(key, tlo, thi, j);
  }
  __device__ __forceinline__ int state_at(unsigned long long k, int nt, bool& ok) const {
    ok = true;
    uint4 o = philox(make_uint4((unsigned)(k >> 2), tlo, thi, 0x7F4A7C15u), keyb);
    return (int)__umulhi(comp4(o, (unsigned)(k & 3)), (unsigned)(nt + 1));
  }
};

__device__ __forceinline__ int block_insert(int* bkeys, int logHB, int key) {
  const unsigned mask = (1u << logHB) - 1u;
  unsigned h = ((unsigned)key * 0x9E3779B1u) >> (32 - logHB);
  for (int it = 0; it < 64; it++) {
    int prev = atomicCAS(&bkeys[h], -1, key);
    if (prev == -1 || prev == key) return (int)h;
    h = (h + 1) & mask;
  }
  return -1;
}

// Scratch of one move slot: its shared-memory region, or the slot's global
// region for moves too large for shared memory.
struct SlotScratch {
  int* keys;
  int* used;
  int* bslot;
  long long* vals;
  int logH;
  void* stage;
  int* idx;
  unsigned* picked;
};

__device__ __forceinline__ void use_table(SlotScratch& S, const SlotScratch& from) {
  S.keys = from.keys; S.used = from.used; S.bslot = from.bslot; S.vals = from.vals; S.logH = from.logH;
}

// Drop the entries a move left in a voxel table (keys, values, block slots).
__device__ __forceinline__ void clear_table(const SlotScratch& T, int hcol, int nu, int gl, int G) {
  for (int i = gl; i < nu; i += G) {
    const int slot = T.used[i];
    T.keys[slot] = -1;
    for (int cc = 0; cc < hcol; cc++) T.vals[(long long)slot * hcol + cc] = 0;
    T.bslot[i] = -1;
  }
}

// A position move's bead data in global memory (one replica).
template <typename Pos>
struct ChainView {
  const V4<Pos>* r4;
  const V4<Pos>* t34;
  const V4<Pos>* t24;
  const unsigned* st;
  const double* bonds;
  const float* bonds32;
  const double* twist;  // (eps_twist, omega0) per bond, SSTWLC replicas only
  // lean: the caller's instantiation has no SSTWLC replica (twist stays null)
  __device__ ChainView(const KArgs& a, const RepDev& rd, bool lean)
      : r4(reinterpret_cast<const V4<Pos>*>(a.r4) + rd.bead_off),
        t34(reinterpret_cast<const V4<Pos>*>(a.t34) + rd.bead_off),
        t24(reinterpret_cast<const V4<Pos>*>(a.t24) + rd.bead_off),
        st(a.states + rd.bead_off), bonds(a.bonds + rd.bead_off * 6), bonds32(a.bonds32 + rd.bead_off * 8),
        twist(!lean && rd.twist ? a.twist + rd.bead_off * 2 : nullptr) {}
};

// Lanes per bead of the position-move deposit; each lane takes 8 / kLanesPerBead
// of the bead's trilinear corners.
// Largest position move of the pooled voxel table: an entry gets at most 2 m
// contributions of |d| < 2^42, which its two 32-bit split counters hold for
// m < 512.
constexpr int kPoolMaxBeads = 256;

constexpr int kLanesPerBead = 4;
constexpr int kCornersPerLane = 8 / kLanesPerBead;

// The bond to the fixed right neighbour of moved bead i (old r, t3, t2 and
// new tr, tt3, tt2), with its twist term: the second bond of a one-bead move
// when one lane takes the whole bead.
template <typename Pos, typename Acc>
static __device__ __noinline__ Acc right_bond_term(const ChainView<Pos>& cv, long long i, const Pos (&r)[3],
                                                   const Pos (&tr)[3], const Pos (&t3)[3], const Pos (&tt3)[3],
                                                   const Pos (&t2)[3], const Pos (&tt2)[3]) {
  const V4<Pos> RN = cv.r4[i + 1], TN = cv.t34[i + 1];
  const Bond<Pos> bn = bond_at(cv.bonds, cv.bonds32, i, (Pos)0);
  const Pos rn[3] = {RN.x, RN.y, RN.z}, tn[3] = {TN.x, TN.y, TN.z};
  Acc out = acc_zero<Acc>();
  acc_add(out, pair_dE_rev(bn, r, tr, rn, t3, tt3, tn));
  if (cv.twist) {
    const Frame nb = frame_of(cv.t24[i + 1], TN), cur = frame_of(t2, t3), nw = frame_of(tt2, tt3);
    acc_add_d(out, twist_pair_dE(cv.twist + 2 * i, cur, nb, nw, nb));
  }
  return out;
}

// Lane cl (0..kLanesPerBead-1) of bead k of a position move (transform M;
// segment [ind0, indf) of m beads of a chain of N): transforms the bead,
// stages its r, t3, t2 (lanes 0-2), takes the bond to a fixed left neighbour
// (lane 0 of the first bead, `left`) or to a fixed right neighbour (lane 1 of
// the last bead, `right`) into `pterm`, counts the confinement crossings
// (lane 0), and returns the voxel-table contributions of its corners c =
// cl * kCornersPerLane + j: q[2j] at vq[2j] (old weight removed; the weight
// change when the old and new weights lie in the same eight voxels) and
// q[2j+1] at vq[2j+1] (new weight otherwise), with the bead's binder states
// in sw.  The neighbour beads and bond parameters are loaded with the moved
// bead (in-range indices on every lane).
template <typename Pos, typename Acc>
__device__ __forceinline__ void bead_task(const RepDev& rd, const GridF& gf, const ChainView<Pos>& cv, int kind,
                                          const Pos (&M)[3][4], long long N, long long ind0, long long indf,
                                          long long m, long long k, int cl, V4<Pos>* stage, bool density,
                                          bool conf, int (&vq)[2 * kCornersPerLane],
                                          long long (&q)[2 * kCornersPerLane], unsigned& sw, unsigned& e,
                                          bool& left, bool& right, Acc& pterm, int& oob) {
  using Real = Pos;
  const long long i = ind0 + k;
  constexpr int kRightLane = kLanesPerBead > 1 ? 1 : 0;
  left = cl == 0 && k == 0 && ind0 != 0;
  right = cl == kRightLane && k == m - 1 && indf != N;
  // with one lane per bead, a one-bead move's lane takes both bonds; else a
  // lane takes at most one, and loads one neighbour
  const bool two = kLanesPerBead == 1 && left && right;
  const long long in = left ? i - 1 : (right ? i + 1 : i);
  const V4<Pos> RN = cv.r4[in], TN = cv.t34[in];
  const Bond<Real> bn = bond_at(cv.bonds, cv.bonds32, (right && !left) ? i : in, (Real)0);
  const V4<Pos> R = cv.r4[i], T3 = cv.t34[i], T2 = cv.t24[i];
  const unsigned swi = density ? cv.st[i] : 0u;
  const Real r[3] = {R.x, R.y, R.z}, t3[3] = {T3.x, T3.y, T3.z}, t2[3] = {T2.x, T2.y, T2.z};
  Real tr[3], tt3[3], tt2[3];
  if (kind == CG_SLIDE) {
    for (int j = 0; j < 3; j++) { tr[j] = r[j] + M[j][3]; tt3[j] = t3[j]; tt2[j] = t2[j]; }
  } else {
    for (int j = 0; j < 3; j++) {
      Real er = 0, e3 = 0, e2 = 0;
      for (int qq = 0; qq < 3; qq++) { er += M[j][qq] * r[qq]; e3 += M[j][qq] * t3[qq]; e2 += M[j][qq] * t2[qq]; }
      tr[j] = er + M[j][3]; tt3[j] = e3; tt2[j] = e2;
    }
  }
  const bool fin = isfinite(tr[0]) && isfinite(tr[1]) && isfinite(tr[2]);
  if (!fin) e |= E_NONFINITE;
#pragma unroll
  for (int w = cl; w < 3; w += kLanesPerBead) {  // lanes 0-2 stage r, t3, t2 (all three with fewer lanes)
    Real o[3];
    for (int j = 0; j < 3; j++) o[j] = w == 0 ? tr[j] : (w == 1 ? tt3[j] : tt2[j]);
    stage[3 * k + w] = V4<Pos>{(Pos)o[0], (Pos)o[1], (Pos)o[2], (Pos)0};
  }
  const Real rn[3] = {(Real)RN.x, (Real)RN.y, (Real)RN.z}, tn[3] = {(Real)TN.x, (Real)TN.y, (Real)TN.z};
  pterm = acc_zero<Acc>();
  if (left) acc_add(pterm, pair_dE_fwd(bn, rn, r, tr, tn, t3, tt3));
  if (right && !two) acc_add(pterm, pair_dE_rev(bn, r, tr, rn, t3, tt3, tn));
  if (cv.twist && (left || right) && !two) {  // SSTWLC: the bond's twist term
    const Frame nb = frame_of(cv.t24[in], TN), cur = frame_of(t2, t3), nw = frame_of(tt2, tt3);
    const double* tw = cv.twist + 2 * (left ? in : i);
    acc_add_d(pterm, left ? twist_pair_dE(tw, nb, cur, nb, nw) : twist_pair_dE(tw, cur, nb, nw, nb));
  }
  if (two) {  // the right bond of a one-bead move (one lane per bead), out of line
    acc_add(pterm, right_bond_term<Pos, Acc>(cv, i, r, tr, t3, tt3, t2, tt2));
    if (cv.twist) {
      const Frame nb = frame_of(cv.t24[in], TN), cur = frame_of(t2, t3), nw = frame_of(tt2, tt3);
      acc_add_d(pterm, twist_pair_dE(cv.twist + 2 * in, nb, cur, nb, nw));
    }
  }
  oob = 0;
  if (cl == 0 && conf) oob = out_of_bounds(rd, tr, true) * 65536 + out_of_bounds(rd, r, false);
  if (density && fin) {
    Real wl0[3], wl1[3];
    int lo0[3], hi0[3], lo1[3], hi1[3];
    move_axes(rd, gf, r, wl0, lo0, hi0);
    move_axes(rd, gf, tr, wl1, lo1, hi1);
    const bool same = lo0[0] == lo1[0] && lo0[1] == lo1[1] && lo0[2] == lo1[2];
#pragma unroll
    for (int j = 0; j < kCornersPerLane; j++) {
      const int c = cl * kCornersPerLane + j;
      Real w0, w1;
      voxel_corner(gf, wl0, lo0, hi0, c, w0, vq[2 * j]);
      voxel_corner(gf, wl1, lo1, hi1, c, w1, vq[2 * j + 1]);
      const long long q0 = q40(w0), q1 = q40(w1);
      q[2 * j] = same ? q1 - q0 : -q0;
      q[2 * j + 1] = same ? 0 : q1;
    }
    sw = swi;
  }
}

// A bond term kept in a move plan (fixed-point part and FP64 part).
__device__ __forceinline__ void store_acc(long long& q, double& h, const Fx& v) { q = v.q; h = v.hard; }
__device__ __forceinline__ void store_acc(long long& q, double& h, double v) { q = 0; h = v; }
template <typename Acc> __device__ __forceinline__ Acc load_acc(long long q, double h);
template <> __device__ __forceinline__ Fx load_acc<Fx>(long long q, double h) { return Fx{q, h}; }
template <> __device__ __forceinline__ double load_acc<double>(long long, double h) { return h; }

// Deposit of the batch's position moves that use a shared voxel table
// (plan.blk), by every thread of the CTA: the moves' bead corners, in move
// order, are dealt out to the threads (eight per bead), so a move of many
// beads no longer holds the batch back while the other warps wait.  The
// table is the CTA's pooled table (FP32 storage: keys voxel * 32 + slot, one
// used list, claims appended once per warp) or the slot's own table (claims
// appended once per warp and move).  The bond terms, confinement counts and
// error bits go to the move's plan.  A move whose optimistic table overflows
// (E_OVF: a pool or a table past 3/4 load) is skipped from then on; its
// group deposits it again in its global table.  Called by every thread.
template <typename Pos, bool LEAN>
__device__ void block_deposit(const KArgs& a, SpecShared& sh, int rep, int B, int kind) {
  using Acc = typename AccOf<Pos>::type;
  unsigned char* smem = reinterpret_cast<unsigned char*>(&sh);
  const RepDev& rd = sh.ws.rd;
  const GridF& gf = sh.ws.gf;
  const ChainView<Pos> cv(a, rd, LEAN);
  const long long N = rd.n_beads;
  const bool conf = rd.field_kind != 0 && rd.confine_kind;
  const int Hs = 1 << a.logH, hcol = a.hcol;
  const bool pool = a.pool_on != 0;
  // lane j of every warp holds the end of move j's tasks in the batch's
  // task list (kLanesPerBead per bead of the moves with plan.blk)
  const int lane = (int)(threadIdx.x & 31u);
  int end = (lane < B && sh.plan[lane].blk) ? kLanesPerBead * sh.plan[lane].m : 0;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(kFull, end, o);
    if (lane >= o) end += y;
  }
  const int total = __shfl_sync(kFull, end, 31);
  for (int t0 = 0; t0 < total; t0 += (int)blockDim.x) {
    const int t = t0 + (int)threadIdx.x;
    // the task's move: the number of moves whose tasks end at or before t
    int s = 0;
    for (int j = 0; j < B; j++) s += __shfl_sync(kFull, end, j) <= t ? 1 : 0;
    const int before = __shfl_sync(kFull, end, s > 0 ? s - 1 : 0);
    int base = s > 0 ? before : 0;
    if (t >= total) s = base = 0;
    MovePlan& P = sh.plan[s];
    const bool act = t < total && !(P.derr & E_OVF);
    const long long k = (t - base) / kLanesPerBead;
    const int cl = (t - base) % kLanesPerBead;
    unsigned char* wb = smem + a.spec_off_warps + (size_t)s * a.warp_smem;
    int vq[2 * kCornersPerLane] = {};
    long long q[2 * kCornersPerLane] = {};
    unsigned sw = 0, e = 0;
    if (act) {
      Pos M[3][4];
      const Pos* Mp = reinterpret_cast<const Pos*>(P.M);
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 4; j++) M[i][j] = Mp[4 * i + j];
      V4<Pos>* stage = P.gstage ? reinterpret_cast<V4<Pos>*>(a.g_stage) +
                                      ((long long)rep * a.spec_s + s) * a.g_stage_cap * 3
                                : reinterpret_cast<V4<Pos>*>(wb + a.off_stage);
      bool left, right;
      Acc pterm;
      int oob;
      bead_task<Pos, Acc>(rd, gf, cv, kind, M, N, P.ind0, P.indf, P.m, k, cl, stage, true, conf, vq, q, sw, e,
                          left, right, pterm, oob);
      if (left) store_acc(P.pq[0], P.ph[0], pterm);  // both bonds of a one-lane bead: in pq[0]
      if (right && !left) store_acc(P.pq[1], P.ph[1], pterm);
      if (oob) atomicAdd(&P.oob, oob);
    }
    // the pooled table (one used list for the whole CTA, keys voxel * 32 +
    // slot), or the move's own table (one used list per move)
    const unsigned peers = pool ? kFull : __match_any_sync(kFull, t < total ? s : -1);
    int* keys = reinterpret_cast<int*>(pool ? smem + a.off_pkeys : wb + a.off_keys);
    int* used = reinterpret_cast<int*>(pool ? smem + a.off_pused : wb + a.off_used);
    long long* vals = reinterpret_cast<long long*>(pool ? smem + a.off_pvals : wb + a.off_vals);
    bool want[2 * kCornersPerLane];
#pragma unroll
    for (int j = 0; j < 2 * kCornersPerLane; j++) {
      want[j] = q[j] != 0;
      if (pool) vq[j] = vq[j] * 32 + s;
    }
    const bool sure = P.sure && !pool;
    const unsigned full_bit = sure ? E_SPIN : E_OVF;
    const int lh = pool ? a.pool_logH : a.logH;
    int slot[2 * kCornersPerLane];
    claim_slots<2 * kCornersPerLane>(keys, used, pool ? &sh.npool : &sh.nused[s], lh, vq, want, slot, e,
                                     sure ? Hs : (3 << lh) / 4, full_bit, peers);
    if (!(e & full_bit)) {
#pragma unroll
      for (int j = 0; j < 2 * kCornersPerLane; j++)
        if (want[j]) add_corner(vals, hcol, slot[j], q[j], sw, rd.nb, true);
    }
    if (e) atomicOr(&P.derr, e);
  }
}

// Field dE and conflict registration of the batch's pooled voxel entries, by
// every thread of the CTA (FP32 storage): entry -> (voxel, move slot s);
// the voxel's FP32 field term (voxel_dE_f32, which also leaves the voxel's
// post-move row in the entry for the commit); its registration in the block
// voxel table, whose atomicOr returns the moves that registered the voxel
// first (an earlier one is a conflict of s, a later one learns of s through
// its plan's mask).  Per move, the fixed-point terms are summed exactly (a
// warp reduces each move's terms in three 21-bit limbs, one 64-bit atomic
// per warp and move), so the sum does not depend on which thread took which
// voxel.  Entries of moves that overflowed the pool are skipped (their
// groups redo them in their global tables).  Called by every thread.
static __device__ void block_field_pool(const KArgs& a, SpecShared& sh, unsigned char* smem, int* bkeys,
                                 unsigned* bmask) {
  const WarpShared& ws = sh.ws;
  const RepDev& rd = ws.rd;
  const int* pkeys = reinterpret_cast<const int*>(smem + a.off_pkeys);
  const int* pused = reinterpret_cast<const int*>(smem + a.off_pused);
  long long* pvals = reinterpret_cast<long long*>(smem + a.off_pvals);
  const long long* grid = a.grid + rd.vox_off * a.ncol;
  const int n = sh.npool;
  const int lane = (int)(threadIdx.x & 31u);
  for (int e0 = (int)(threadIdx.x & ~31u); e0 < n; e0 += (int)blockDim.x) {
    const int e = e0 + lane;
    int s = -1;
    Fx part = Fx{0, 0.0};
    long long hp = 0;
    if (e < n) {
      const int slot = pused[e];
      const int key = pkeys[slot];
      s = key & 31;
      const int v = key >> 5;
      MovePlan& P = sh.plan[s];
      if (P.derr & E_OVF) {
        s = -1;
      } else {
        voxel_dE_f32(ws, a, grid, v, pvals + (long long)slot * a.hcol, true, part, hp);
        const int b = block_insert(bkeys, a.spec_logHB, v);
        if (b < 0) {
          atomicOr(&P.freg, 1);
        } else {
          const unsigned prior = atomicOr(&bmask[b], 1u << s);
          const unsigned below = (1u << s) - 1u, above = ~((2u << s) - 1u);
          if (prior & below) atomicOr(&P.cmask, prior & below);
          for (unsigned later = prior & above; later; later &= later - 1)
            atomicOr(&sh.plan[__ffs((int)later) - 1].cmask, 1u << s);
        }
        if (!is_zero64(part.hard)) atomicAdd(&P.fh, part.hard);
        if (hp) atomicAdd(reinterpret_cast<unsigned long long*>(&P.fH), (unsigned long long)hp);
      }
    }
    // q = l2 2^42 + l1 2^21 + l0 with l0, l1 in [0, 2^21) (|q| < 2^50): each
    // limb's sum over a warp fits 32 bits
    unsigned todo = __ballot_sync(kFull, s >= 0);
    while (todo) {
      const int leader = __ffs((int)todo) - 1;
      const int sl = __shfl_sync(kFull, s, leader);
      const bool mine = s == sl;
      const long long q = mine ? part.q : 0;
      const unsigned l0 = __reduce_add_sync(kFull, (unsigned)(q & 0x1FFFFF));
      const unsigned l1 = __reduce_add_sync(kFull, (unsigned)((q >> 21) & 0x1FFFFF));
      const int l2 = __reduce_add_sync(kFull, (int)(q >> 42));
      const unsigned who = __ballot_sync(kFull, mine);
      if (lane == leader) {
        const long long sum = (long long)l2 * 4398046511104LL + (long long)l1 * 2097152LL + (long long)l0;
        atomicAdd(reinterpret_cast<unsigned long long*>(&sh.plan[sl].fq), (unsigned long long)sum);
        atomicAdd(&sh.plan[sl].fn, __popc(who));
      }
      todo &= ~who;
    }
  }
}

// Commit of the pooled entries after the batch is resolved, by every thread:
// the post-move rows of the standing accepted moves (the first `cut`, bits of
// `acc`) go to the grid with 16-byte stores; every entry is cleared, and so
// is the block voxel table.
static __device__ void block_commit_pool(const KArgs& a, SpecShared& sh, unsigned char* smem, int cut, unsigned acc,
                                  int* bkeys, unsigned* bmask) {
  const RepDev& rd = sh.ws.rd;
  int* pkeys = reinterpret_cast<int*>(smem + a.off_pkeys);
  const int* pused = reinterpret_cast<const int*>(smem + a.off_pused);
  long long* pvals = reinterpret_cast<long long*>(smem + a.off_pvals);
  long long* grid = a.grid + rd.vox_off * a.ncol;
  const int n = sh.npool, hcol = a.hcol, ncol = a.ncol;
  for (int e = (int)threadIdx.x; e < n; e += (int)blockDim.x) {
    const int slot = pused[e];
    const int key = pkeys[slot];
    const int s = key & 31;
    long long* src = pvals + (long long)slot * hcol;
    if (s < cut && ((acc >> s) & 1u) && !(sh.plan[s].derr & E_OVF)) {
      longlong2* dst = reinterpret_cast<longlong2*>(grid + (long long)(key >> 5) * ncol);
      dst[0] = make_longlong2(src[0], src[1]);
      if (ncol == 4) dst[1] = make_longlong2(hcol > 2 ? src[2] : 0, hcol > 3 ? src[3] : 0);
    }
    pkeys[slot] = -1;
    for (int cc = 0; cc < hcol; cc++) src[cc] = 0;
  }
  for (int i = (int)threadIdx.x; i < (1 << a.spec_logHB); i += (int)blockDim.x) {
    bkeys[i] = -1;
    bmask[i] = 0u;
  }
}

// Move-log terms of a plan (out of line: the log is off in production runs).
static __device__ __noinline__ void log_terms_d(MovePlan& P, double dEp, unsigned long long pos) {
  P.dEp = dEp;
  P.ndraw = (int)pos;
}
__device__ __forceinline__ void log_terms(MovePlan& P, double dEp, unsigned long long pos) {
  log_terms_d(P, dEp, pos);
}
__device__ __forceinline__ void log_terms(MovePlan& P, const Fx& dEp, unsigned long long pos) {
  log_terms_d(P, acc_d(dEp), pos);
}

// Record of move t (its plan) in the move log, when t is within the log.
static __device__ __noinline__ void log_move(const KArgs& a, int rep, unsigned long long k, const MovePlan& P) {
  if (k >= (unsigned long long)a.mlog_cap) return;
  cg_move_record rec;
  rec.kind = P.kind;
  rec.n_inds = P.empty ? 0 : P.m;
  rec.ind0 = P.ind0;
  rec.indf = P.indf;
  rec.dE_poly = P.empty ? 0.0 : P.dEp;
  rec.dE_field = P.empty ? 0.0 : P.dE - P.dEp;
  rec.accepted = P.empty ? -1 : P.dec;
  rec.n_draws = P.ndraw;
  a.mlog[(long long)rep * a.mlog_cap + (long long)k] = rec;
}

// The pooled pass's field terms of a move, added to its field dE.
__device__ __forceinline__ void add_pool_terms(Fx& s, const MovePlan& P) {
  s.q += P.fq;
  if (!is_zero64(P.fh)) s.hard = add_hard(s.hard, P.fh);
}
__device__ __forceinline__ void add_pool_terms(double& s, const MovePlan& P) {
  s += (double)P.fq * kFxEInv + P.fh;
}

// Evaluate move t of the batch in slot s (group lanes gl = 0..G-1); `live`
// is false for the groups of a partly filled batch and for the warps without
// a move, which run the collectives and block barriers with empty work.
// Every thread of the CTA calls it (position moves hold two block barriers
// around the block-wide deposit); B is the batch's number of moves.
template <typename Pos, int G, bool LEAN>
__device__ void evaluate_move(const KArgs& a, SpecShared& sh, int rep, int s, int gl, bool live, int kind,
                              const cg_move_ctl& c, unsigned long long t, unsigned* draws,
                              const SlotScratch& sm, const SlotScratch& gm, int* bkeys, unsigned* bmask,
                              int logHB, int B) {
  using Real = Pos;
  using Acc = typename AccOf<Real>::type;
  const RepDev& rd = sh.ws.rd;
  const GridF& gf = sh.ws.gf;
  const WarpShared& ws = sh.ws;
  const long long N = rd.n_beads;
  const int hcol = a.hcol;  // stride of the voxel-table values
  const V4<Pos>* r4 = reinterpret_cast<const V4<Pos>*>(a.r4) + rd.bead_off;
  const V4<Pos>* t34 = reinterpret_cast<const V4<Pos>*>(a.t34) + rd.bead_off;
  const V4<Pos>* t24 = reinterpret_cast<const V4<Pos>*>(a.t24) + rd.bead_off;
  const unsigned* st = a.states + rd.bead_off;
  const unsigned* mk = a.marks + rd.bead_off;
  const double* bonds = a.bonds + rd.bead_off * 6;
  const float* bonds32 = a.bonds32 + rd.bead_off * 8;
  MovePlan& P = sh.plan[s];
  MoveRng g;
  if (__any_sync(kFull, live)) g.init<G>(a.seed, rep, t, draws, gl);
  unsigned err = 0;
  const bool check_field = rd.field_kind != 0 && kind != CG_TANGENT_ROTATION;
  const bool density = rd.field_kind == 2;
  long long ind0 = 0, indf = 0, m = 0;
  // dE = dEp (polymer) + dEs (field; fixed point for FP32 storage) + dEh (the
  // FP64 part: confinement penalties, and the whole field dE for FP64 storage)
  Acc dEp = acc_zero<Acc>(), dEs = acc_zero<Acc>();
  double dEh = 0;
  long long dEH = 0;  // the exact 1e99 penalties, in kHugeUnit units
  long long nvox = 0;
  bool empty = !live;
  int gtab = 0, gstage = 0;
  unsigned cmb = 0;  // position moves: conflicts with earlier moves of the batch
  SlotScratch S = sm;
  int* nused = &sh.nused[s];
  const int Hs = 1 << sm.logH;
  const bool pool = a.pool_on != 0;
  bool pooled = false;  // a position move whose voxels the CTA's pooled pass evaluates
  if (threadIdx.x == 0) sh.npool = 0;  // every reader of the last batch's pool passed a barrier since

  if (kind <= CG_SLIDE) {
    const ChainView<Pos> cv(a, rd, LEAN);
    Real M[3][4];
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 4; j++) M[i][j] = i == j ? (Real)1 : (Real)0;
    if (live) {
      if (kind == CG_CRANK_SHAFT) {
        Real ang = (Real)c.amp_move * (uni<Real>(g.next()) - (Real)0.5);
        const unsigned xb0 = g.next();
        long long b0 = sizeof(Real) == 4 ? scaled_index(xb0, N) : (long long)(int)(unif(xb0) * (double)N);
        long long b1 = from_point(g, c.amp_bead, N, b0, err);
        if (b1 < 1) b1 = 1;
        check_bead_bounds(b0, b1, N, ind0, indf);
        long long ia, ib;
        if (ind0 == indf - 1 && ind0 == 0) { ia = indf; ib = ind0; }
        else if (ind0 == indf - 1 && ind0 == N - 1) { ia = ind0; ib = ind0 - 1; }
        else if (ind0 == 0 && indf == N) { ia = indf - 1; ib = ind0; }
        else if (ind0 == 0) { ia = indf; ib = ind0; }
        else if (indf == N) { ia = indf - 1; ib = ind0 - 1; }
        else { ia = indf; ib = ind0 - 1; }
        if (!err) {
          Real pa[3], pb[3], dir[3], p[3];
          long long ip;  // the fulcrum bead, loaded with the two axis beads
          if (ind0 == 0 && indf != N) ip = indf;
          else if (ind0 != 0 && indf == N) ip = ind0 - 1;
          else if (ind0 == 0 && indf == N) ip = ind0;
          else ip = ind0 - 1;
          ld3(r4, ia, pa); ld3(r4, ib, pb); ld3(r4, ip, p);
          for (int i = 0; i < 3; i++) dir[i] = pa[i] - pb[i];
          Real mag = rsqrt_(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
          if (mag < (Real)1E-5) sphere<Real>(g, dir);
          else { Real sc = (Real)1 / mag; for (int i = 0; i < 3; i++) dir[i] = dir[i] * sc; }
          axis_rotation(dir, p, ang, M);
        }
      } else if (kind == CG_END_PIVOT) {
        Real ang = (Real)c.amp_move * (uni<Real>(g.next()) - (Real)0.5);
        long long lhs = g.next() & 1u;
        if (lhs == 1) { ind0 = 0; indf = from_left(g, c.amp_bead, N, err) + 1; }
        else { ind0 = N - from_left(g, c.amp_bead, N, err); indf = N; }
        Real axis[3], p[3];
        sphere<Real>(g, axis);
        long long ip;
        if (ind0 == 0 && indf != N) ip = indf;
        else if (ind0 != 0 && indf == N) ip = ind0 - 1;
        else if (ind0 == 0 && indf == N && lhs == 1) ip = indf - 1;
        else ip = ind0;
        if (!err) {
          ld3(r4, ip, p);
          axis_rotation(axis, p, ang, M);
        }
      } else {
        Real amp = (Real)c.amp_move * uni<Real>(g.next()), d[3];
        sphere<Real>(g, d);
        for (int i = 0; i < 3; i++) M[i][3] = d[i] * amp;
        long long b0 = g.next() % (unsigned)N;
        long long b1 = from_point(g, c.amp_bead, N, b0, err);
        check_bead_bounds(b0, b1, N, ind0, indf);
      }
    }
    m = (!live || err) ? 0 : indf - ind0;
    if (live && !err && m == 0) empty = true;
    if (m > a.stage_cap) { S.stage = gm.stage; gstage = 1; }
    // voxel table: with the CTA's pooled table (FP32 storage), every move of
    // up to kPoolMaxBeads beads, optimistically (a pool past 3/4 load sends
    // the move to its global table); else the slot's own table when the
    // move's at most 16 m voxels surely fit, or optimistically up to m <=
    // slots / 4 with the same fallback; global beyond
    bool sure, blk;
    if (pool) {
      sure = false;
      blk = density && m > 0 && m <= kPoolMaxBeads;
      if (density && m > 0 && !blk) { use_table(S, gm); gtab = 1; }
    } else {
      sure = 16 * m <= Hs;
      if (!sure && 4 * m > Hs) { use_table(S, gm); gtab = 1; }
      blk = density && m > 0 && !gtab;  // moves with a shared table are deposited by the whole CTA
    }
    V4<Pos>* stage = reinterpret_cast<V4<Pos>*>(S.stage);  // r, t3, t2 of each moved bead
    if (gl == 0 && live) {
      P.blk = blk ? 1 : 0;
      P.sure = sure ? 1 : 0;
      P.m = (int)m;
      P.ind0 = (int)ind0;
      P.indf = (int)indf;
      P.gstage = gstage;
      P.oob = 0;
      P.derr = 0;
      P.cmask = 0;
      P.pq[0] = P.pq[1] = 0;
      P.ph[0] = P.ph[1] = 0;
      P.fq = P.fH = 0;
      P.fh = 0;
      P.fn = P.freg = 0;
      Pos* Mp = reinterpret_cast<Pos*>(P.M);  // in the position type: no conversions
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 4; j++) Mp[4 * i + j] = M[i][j];
    }
    __syncthreads();
    block_deposit<Pos, LEAN>(a, sh, rep, B, kind);
    // earlier moves u of the batch whose written beads [ind0, indf) meet the
    // beads this move reads (its segment and both neighbours); a move with no
    // beads (failed or empty) is never accepted, so it needs no exclusion
    for (int u0 = 0; u0 < B; u0 += G) {
      const int u = u0 + gl;
      bool hit = false;
      if (m > 0 && u < s) {
        const MovePlan& U = sh.plan[u];
        hit = U.m > 0 && (long long)U.ind0 <= indf && ind0 - 1 <= (long long)U.indf - 1;
      }
      cmb |= gballot<G>(hit) << u0;
    }
    __syncthreads();
    if (pool && density) block_field_pool(a, sh, reinterpret_cast<unsigned char*>(&sh), bkeys, bmask);
    Acc part = acc_zero<Acc>();
    int oob = 0;
    bool ovf = false;
    if (blk) {
      const unsigned eb = P.derr;
      ovf = (eb & E_OVF) != 0;
      pooled = pool && !ovf;
      err |= eb & ~E_OVF;
      if (gl == 0) {
        acc_add(part, load_acc<Acc>(P.pq[0], P.ph[0]));
        acc_add(part, load_acc<Acc>(P.pq[1], P.ph[1]));
        oob = P.oob;
      }
    }
    const unsigned peers = group_mask<G>();
    for (int pass = 0; pass < 2; pass++) {
      if (pass == 1) {
        if (!__any_sync(kFull, ovf)) break;
        if (ovf) clear_table(S, hcol, *nused, gl, G);
        __syncwarp();
        if (ovf) {
          if (gl == 0) *nused = 0;
          use_table(S, gm);
          gtab = 1;
          part = acc_zero<Acc>();
          oob = 0;
        }
        __syncwarp();
      }
      // pass 0: the moves the CTA did not deposit; pass 1: overflowed ones
      const bool run = pass == 0 ? !blk : ovf;
      const int cap = gtab ? (1 << gm.logH) : (sure ? Hs : (3 * Hs) / 4);
      const unsigned full_bit = (gtab || sure) ? E_SPIN : E_OVF;
      unsigned e = 0;
      // the group's own deposit: kLanesPerBead lanes per bead, lane gl
      // taking part gl % kLanesPerBead of bead gl / kLanesPerBead of a pass
      constexpr int BP = G / kLanesPerBead;
      const int kc = gl / kLanesPerBead, cl = gl % kLanesPerBead;
      for (long long kb = 0; __any_sync(kFull, run && kb < m && !(e & E_OVF)); kb += BP) {
        const long long k = kb + kc;
        const bool act = run && k < m && !(e & E_OVF);
        int vq[2 * kCornersPerLane] = {};
        long long q[2 * kCornersPerLane] = {};
        unsigned sw = 0;
        if (act) {
          bool left, right;
          Acc pterm;
          int ob;
          bead_task<Pos, Acc>(rd, gf, cv, kind, M, N, ind0, indf, m, k, cl, stage, density,
                              check_field && rd.confine_kind, vq, q, sw, e, left, right, pterm, ob);
          if (left || right) acc_add(part, pterm);
          oob += ob;
        }
        if (density) {
          bool want[2 * kCornersPerLane];
#pragma unroll
          for (int j = 0; j < 2 * kCornersPerLane; j++) want[j] = q[j] != 0;
          int slot[2 * kCornersPerLane];
          claim_slots<2 * kCornersPerLane>(S.keys, S.used, nused, S.logH, vq, want, slot, e, cap, full_bit, peers);
          if (!(e & full_bit)) {
#pragma unroll
            for (int j = 0; j < 2 * kCornersPerLane; j++)
              if (want[j]) add_corner(S.vals, hcol, slot[j], q[j], sw, rd.nb, !gtab);
          }
          e = gor<G>(e);  // a full table ends the group's passes together
        }
      }
      e = gor<G>(e);
      if (run) ovf = (e & E_OVF) != 0;
      err |= e & ~E_OVF;
    }
    err = gor<G>(err);
    dEp = gsum<G>(part);
    if (check_field && rd.confine_kind) {
      int oo = gsum<G>(oob);
      dEH += ((long long)(oo >> 16) - (long long)(oo & 0xFFFF)) << 40;
    }
    __syncwarp();
    if (density)
      field_dE_voxels<G>(ws, a, hcol, S.keys, S.used, S.vals, *nused, gl, nvox, dEs, dEh, dEH, !gtab);
  } else if (kind == CG_TANGENT_ROTATION) {
    Real ang = 0;
    long long n = 0;
    if (live) {
      ang = (Real)c.amp_move * (uni<Real>(g.next()) - (Real)0.5);
      n = (long long)(g.next() % (unsigned)c.amp_bead) + 1;
      if (n > N) err |= E_WINDOW;
    }
    m = (!live || err) ? 0 : n;
    if (m > a.stage_cap) { S.stage = gm.stage; S.idx = gm.idx; gstage = 1; }
    int* idx = S.idx;
    // n distinct random beads, drawn in order with redraws (get_inds): G
    // candidates per round, the first fresh ones taken in draw order.  Beads
    // taken in a round that another round follows are marked in the slot's
    // bitmap, which later rounds consult (a move of fewer beads than G
    // usually needs one round and touches no bitmap).
    long long got = 0;
    int it = 0, rounds = 0;
    const unsigned lt = (1u << gl) - 1u;
    const unsigned gmask = G == 32 ? kFull : ((1u << (G & 31)) - 1u) << ((threadIdx.x & 31u) & ~(unsigned)(G - 1));
    for (;;) {
      bool want = live && !err && got < m;
      if (want && ++it > kMaxIter) { err |= E_SPIN; want = false; }
      if (!__any_sync(kFull, want)) break;
      const unsigned x = g.word(g.pos + gl);
      const long long cand = want ? (long long)(x % (unsigned)N) : -1 - (long long)(threadIdx.x & 31u);
      const unsigned grp = __match_any_sync(kFull, cand) & gmask;
      const unsigned gshift = G == 32 ? 0u : ((threadIdx.x & 31u) & ~(unsigned)(G - 1));
      const bool first = ((grp >> gshift) & lt) == 0;
      const bool fresh = want && first && !(rounds > 0 && ((S.picked[cand >> 5] >> (cand & 31)) & 1u));
      const unsigned bal = gballot<G>(fresh);
      const long long need = m - got;
      const int cnt = __popc(bal);
      const int rank = __popc(bal & lt);
      if (fresh && rank < need) {
        idx[got + rank] = (int)cand;
        if (cnt < need) atomicOr(&S.picked[cand >> 5], 1u << (cand & 31));
      }
      if (want) {
        rounds++;
        long long consumed;
        if (cnt >= need) {
          unsigned b = bal;
          for (long long q = 1; q < need; q++) b &= b - 1;
          consumed = __ffs((int)b);
          got = m;
        } else {
          consumed = G;
          got += cnt;
        }
        g.pos += consumed;
      }
      __syncwarp();
    }
    err = gor<G>(err);
    const long long marked = rounds > 1 ? got : 0;  // beads whose marks are cleared below
    if (err) m = 0;
    const unsigned long long axis_base = g.pos;
    V4<Pos>* stage = reinterpret_cast<V4<Pos>*>(S.stage);
    Acc part = acc_zero<Acc>();
    Real sa, ca;
    rsincos(ang, &sa, &ca);
    for (long long k = gl; k < m; k += G) {
      const long long i = idx[k];
      // the bead, both neighbours and both bonds, loaded together (in-range
      // indices at the chain ends, where the term is skipped)
      const bool hl = i != 0, hr = i + 1 != N;
      const long long il = hl ? i - 1 : i, ir = hr ? i + 1 : i;
      Real r[3], t3[3], t2[3], tt3[3], tt2[3], r0[3], t30[3], r1[3], t31[3];
      ld3(r4, i, r); ld3(t34, i, t3); ld3(t24, i, t2);
      ld3(r4, il, r0); ld3(t34, il, t30); ld3(r4, ir, r1); ld3(t34, ir, t31);
      const Bond<Real> bl = bond_at(bonds, bonds32, il, (Real)0), br = bond_at(bonds, bonds32, i, (Real)0);
      const unsigned xa = g.word(axis_base + 2 * k), xb = g.word(axis_base + 2 * k + 1);
      Real axis[3];
      sphere_from<Real>(xa, xb, axis);
      const Real origin[3] = {0, 0, 0};
      Real M[3][4];
      axis_rotation_sc(axis, origin, sa, ca, M);
      for (int j = 0; j < 3; j++) {
        Real e3 = 0, e2 = 0;
        for (int q = 0; q < 3; q++) { e3 += M[j][q] * t3[q]; e2 += M[j][q] * t2[q]; }
        tt3[j] = e3; tt2[j] = e2;
      }
      stage[3 * k + 1] = V4<Pos>{(Pos)tt3[0], (Pos)tt3[1], (Pos)tt3[2], (Pos)0};
      stage[3 * k + 2] = V4<Pos>{(Pos)tt2[0], (Pos)tt2[1], (Pos)tt2[2], (Pos)0};
      Acc de = acc_zero<Acc>();
      if (hl) acc_add(de, pair_dE_fwd(bl, r0, r, r, t30, t3, tt3));
      if (hr) acc_add(de, pair_dE_rev(br, r, r, r1, t3, tt3, t31));
      if (!LEAN && rd.twist) {  // SSTWLC: twist terms of both bonds
        const double* tw = a.twist + rd.bead_off * 2;
        const Frame cur = frame_of(t2, t3), nw = frame_of(tt2, tt3);
        double dt = 0;
        if (hl) {
          const Frame l = frame_of(t24[il], t34[il]);
          dt += twist_pair_dE(tw + 2 * il, l, cur, l, nw);
        }
        if (hr) {
          const Frame rr = frame_of(t24[ir], t34[ir]);
          dt += twist_pair_dE(tw + 2 * i, cur, rr, nw, rr);
        }
        acc_add_d(de, dt);
      }
      acc_add(part, de);
    }
    g.pos = axis_base + 2 * (unsigned long long)m;
    dEp = gsum<G>(part);
    // the picked marks only serve the redraws of this move
    for (long long k = gl; k < marked; k += G) {
      int i = idx[k];
      atomicAnd(&S.picked[i >> 5], ~(1u << (i & 31)));
    }
    __syncwarp();
    if (m > 0) {
      ind0 = idx[0];
      indf = ind0 + 1;
    }
  } else {
    int bsel = 0;
    if (live) {
      bsel = (int)(g.next() % (unsigned)rd.nb);
      long long b0 = g.next() % (unsigned)N;
      long long b1 = from_point(g, c.amp_bead, N, b0, err);
      if (!err) check_bead_bounds(b0, b1, N, ind0, indf);
    }
    m = (!live || err) ? 0 : indf - ind0;
    const int nt = rd.sites[bsel];
    if (m > a.stage_cap) { S.idx = gm.idx; gstage = 1; }
    if (8 * m > Hs) { use_table(S, gm); gtab = 1; }
    int* idx = S.idx;
    Acc part = acc_zero<Acc>();
    int dbl = 0;
    // eight lanes per bead, one trilinear corner each: corner lane 0 takes
    // the binding free energy, each lane the change of its corner's binder
    // column
    constexpr int BP = G / 8;
    const int kc = gl >> 3, cl = gl & 7;
    for (long long kb = 0; __any_sync(kFull, kb < m); kb += BP) {
      const long long k = kb + kc;
      int vq[1] = {0};
      bool want[1] = {false};
      long long q = 0;
      if (k < m) {
        const long long i = ind0 + k;
        bool ok;
        int s_new = g.state_at(g.bpos + k, nt, ok);
        unsigned sw = st[i], mw = mk[i];
        int s_old = (int)((sw >> (8 * bsel)) & 0xFF);
        if (cl == 0) {
          acc_add(part, bead_bind_dE(ws, sw, mw, bsel, s_new, (Real)0));
          dbl += (s_new == 2 ? 1 : 0) - (s_old == 2 ? 1 : 0);
          idx[k] = s_new;
        }
        if (density && s_new != s_old) {
          Real p[3], wl[3], w;
          int lo[3], hi[3];
          ld3(r4, i, p);
          move_axes(rd, gf, p, wl, lo, hi);
          voxel_corner(gf, wl, lo, hi, cl, w, vq[0]);
          q = q40(w) * (long long)(s_new - s_old);
          want[0] = true;
        }
      }
      if (density) {
        int slot[1];
        claim_slots<1>(S.keys, S.used, nused, S.logH, vq, want, slot, err, 1 << S.logH, E_SPIN, group_mask<G>());
        if (want[0] && slot[0] >= 0) add_delta(S.vals, hcol, slot[0], 1 + bsel, q, !gtab);
      }
    }
    g.bpos += (unsigned long long)m;
    err = gor<G>(err);
    dEp = gsum<G>(part);
    const int ddb = gsum<G>(dbl);
    if (check_field && rd.field_kind == 1 && rd.confine_kind == 2) {
      int oob = 0;
      for (long long k = gl; k < m; k += G) {
        double p[3];
        ld3(r4, ind0 + k, p);
        oob += out_of_bounds(rd, p, true);
      }
      dEH += (long long)gsum<G>(oob) << 40;
    }
    __syncwarp();
    if (density) {
      field_dE_voxels<G>(ws, a, hcol, S.keys, S.used, S.vals, *nused, gl, nvox, dEs, dEh, dEH, !gtab);
      if (m > 0) add_intra(ws, bsel, ddb, dEs, dEh);
    }
    if (gl == 0 && live) P.bsel = bsel;
  }
  err = gor<G>(err);
  // register the touched voxels for the conflict test
  // (position moves: the moves that registered a voxel first are this
  // move's conflicts if earlier in the batch; a later move that registered
  // it first learns of this one through its plan's mask)
  int regfail = 0;
  if (density && check_field) {
    const int nu = (live && !err && !empty) ? *nused : 0;
    const unsigned below = (1u << s) - 1u, above = ~((2u << s) - 1u);
    for (int i = gl; i < nu; i += G) {
      int v = S.keys[S.used[i]];
      int b = block_insert(bkeys, logHB, v);
      S.bslot[i] = b;
      if (b < 0) {
        regfail = 1;
      } else {
        const unsigned prior = atomicOr(&bmask[b], 1u << s);
        if (kind <= CG_SLIDE) {
          cmb |= prior & below;
          for (unsigned later = prior & above; later; later &= later - 1)
            atomicOr(&sh.plan[__ffs((int)later) - 1].cmask, 1u << s);
        }
      }
    }
    regfail = (int)gor<G>((unsigned)regfail);
  }
  if (kind <= CG_SLIDE) {
    cmb = gor<G>(cmb);
    if (gl == 0 && live) atomicOr(&P.cmask, cmb);
  }
  if (kind <= CG_SLIDE && pool && density) {
    __syncthreads();  // the pooled field pass is complete
    if (pooled) {
      add_pool_terms(dEs, P);
      dEH += P.fH;
      nvox = P.fn;
      regfail |= P.freg;
    }
  }
  bool dec = false;
  if (live && !err && !empty) dec = decide(g.next(), dEp, dEs, with_huge(dEh, dEH), gl == 0 ? &P.dE : nullptr);
  if (gl == 0 && live) {
    P.kind = kind; P.m = (int)m; P.ind0 = (int)ind0; P.indf = (int)indf;
    P.empty = empty ? 1 : 0; P.err = (int)err; P.regfail = regfail; P.dec = dec ? 1 : 0;
    P.nvox = (int)nvox; P.gtab = gtab; P.gstage = gstage;
    if (!LEAN && a.mlog) log_terms(P, dEp, g.pos);
  }
}

// Bits of earlier moves of the batch (u < s) whose footprint meets move s's.
template <int G>
__device__ void conflict_mask(const KArgs& a, SpecShared& sh, unsigned char* smem, int rep, int s, int gl,
                              bool live, int kind, int B, const SlotScratch& sm, const SlotScratch& gm,
                              const unsigned* bmask) {
  MovePlan& P = sh.plan[s];
  const RepDev& rd = sh.ws.rd;
  const bool act = live && !P.err && !P.empty;
  unsigned cm = 0;
  if (rd.field_kind == 2 && kind != CG_TANGENT_ROTATION) {
    const int nu = act ? sh.nused[s] : 0;
    const int* bs = P.gtab ? gm.bslot : sm.bslot;
    for (int i = gl; i < nu; i += G) {
      int b = bs[i];
      if (b >= 0) cm |= bmask[b];
    }
    cm = gor<G>(cm);
  }
  cm &= (1u << s) - 1u;
  if (kind == CG_TANGENT_ROTATION) {
    // rotated beads of u against those of s and their neighbours
    const int* lw = P.gstage ? gm.idx : sm.idx;
    for (int u = 0; u < B; u++) {
      const MovePlan& U = sh.plan[u];
      int hit = 0;
      if (act && u < s && !U.err && !U.empty) {
        const int* lu = U.gstage ? a.g_idx + ((long long)rep * a.spec_s + u) * a.g_stage_cap
                                 : reinterpret_cast<const int*>(smem + a.spec_off_warps +
                                                                (size_t)u * a.warp_smem + a.off_idx);
        for (int k = gl; k < P.m && !hit; k += G) {
          int j = lw[k];
          for (int q = 0; q < U.m; q++) {
            int d = lu[q] - j;
            if (d >= -1 && d <= 1) { hit = 1; break; }
          }
        }
      }
      if (gany<G>(hit)) cm |= 1u << u;
    }
  } else {
    // lane gl takes the earlier moves u = u0 + gl: beads written by u,
    // [ind0, indf), against the beads read by s -- the segment and, for
    // position moves, its two neighbours
    for (int u0 = 0; u0 < B; u0 += G) {
      const int u = u0 + gl;
      bool hit = false;
      if (act && u < s) {
        const MovePlan& U = sh.plan[u];
        if (!U.err && !U.empty) {
          const long long wlo = U.ind0, whi = (long long)U.indf - 1;
          const long long rlo = P.kind == CG_CHANGE_BINDING_STATE ? P.ind0 : (long long)P.ind0 - 1;
          const long long rhi = P.kind == CG_CHANGE_BINDING_STATE ? (long long)P.indf - 1 : (long long)P.indf;
          hit = wlo <= rhi && rlo <= whi;
        }
      }
      cm |= gballot<G>(hit) << u0;
    }
  }
  if (gl == 0 && live) P.cmask = cm;
}

// SimpleControl.update_amplitudes (chromo/mc/mc_controller.py:126-189)
__device__ __forceinline__ void update_amplitudes(cg_move_ctl& c) {
  if (c.ctrl_kind != 1) return;
  double acc = c.acc_rate;
  if (acc < 0.5) {
    double prop = c.amp_move * 0.95;
    if (prop > c.move_lo) c.amp_move = prop;
    else {
      c.amp_move = c.move_hi;
      double nb = (double)(c.amp_bead - 1);
      c.amp_bead = (long long)(c.bead_lo > nb ? c.bead_lo : nb);
    }
  } else if (acc > 0.5) {
    double prop = c.amp_move / 0.95;
    if (prop < c.move_hi) c.amp_move = prop;
    else {
      c.amp_move = c.move_lo;
      double nb = (double)(c.amp_bead + 1);
      c.amp_bead = (long long)(c.bead_hi < nb ? c.bead_hi : nb);
    }
  }
}

template <typename Pos, int G>
__device__ void commit_and_clear(const KArgs& a, SpecShared& sh, int s, int gl, bool accept,
                                 const SlotScratch& sm, const SlotScratch& gm, int* bkeys, unsigned* bmask) {
  const MovePlan& P = sh.plan[s];
  const RepDev& rd = sh.ws.rd;
  const int ncol = a.ncol, hcol = a.hcol;
  V4<Pos>* r4w = reinterpret_cast<V4<Pos>*>(a.r4) + rd.bead_off;
  V4<Pos>* t34w = reinterpret_cast<V4<Pos>*>(a.t34) + rd.bead_off;
  V4<Pos>* t24w = reinterpret_cast<V4<Pos>*>(a.t24) + rd.bead_off;
  unsigned* st = a.states + rd.bead_off;
  const V4<Pos>* stage = reinterpret_cast<const V4<Pos>*>(P.gstage ? gm.stage : sm.stage);
  const int* idx = P.gstage ? gm.idx : sm.idx;
  int* keys = P.gtab ? gm.keys : sm.keys;
  int* used = P.gtab ? gm.used : sm.used;
  int* bslot = P.gtab ? gm.bslot : sm.bslot;
  long long* vals = P.gtab ? gm.vals : sm.vals;
  const int m = P.m;
  if (accept) {
    if (P.kind <= CG_SLIDE) {
      for (int k = gl; k < m; k += G) {
        const long long i = (long long)P.ind0 + k;
        r4w[i] = stage[3 * k];
        if (P.kind != CG_SLIDE) {
          t34w[i] = stage[3 * k + 1];
          t24w[i] = stage[3 * k + 2];
        }
      }
    } else if (P.kind == CG_TANGENT_ROTATION) {
      for (int k = gl; k < m; k += G) {
        const long long i = idx[k];
        t34w[i] = stage[3 * k + 1];
        t24w[i] = stage[3 * k + 2];
      }
    } else {
      for (int k = gl; k < m; k += G) {
        const long long i = (long long)P.ind0 + k;
        unsigned sw = st[i];
        sw = (sw & ~(0xFFu << (8 * P.bsel))) | ((unsigned)idx[k] << (8 * P.bsel));
        st[i] = sw;
      }
    }
  }
  const int nu = sh.nused[s];
  long long* grid = a.grid + rd.vox_off * ncol;
  for (int i = gl; i < nu; i += G) {
    int slot = used[i];
    if (accept) {  // the voxel's post-move row, stored with 16-byte stores (padding column stays 0)
      const int v = keys[slot];
      const long long* src = vals + (long long)slot * hcol;
      longlong2* dst = reinterpret_cast<longlong2*>(grid + (long long)v * ncol);
      dst[0] = make_longlong2(src[0], src[1]);
      if (ncol == 4) dst[1] = make_longlong2(hcol > 2 ? src[2] : 0, hcol > 3 ? src[3] : 0);
    }
    keys[slot] = -1;
    for (int cc = 0; cc < hcol; cc++) vals[(long long)slot * hcol + cc] = 0;
    int b = bslot[i];
    if (b >= 0) { bkeys[b] = -1; bmask[b] = 0u; }
    bslot[i] = -1;
  }
}

// 168 registers: two CTAs of 6 warps fit one SM's register file (measured
// faster than 128 registers with 8 warps, which spills).  LEAN: the
// instantiation for launches with no SSTWLC replica and no move log, whose
// code for those is left out (it holds the batch loop's state in registers
// without spills; the host picks it per launch, a.lean).
template <typename Pos, int G, bool LEAN>
__global__ void __maxnreg__(168) spec_kernel(KArgs a) {
  extern __shared__ __align__(32) unsigned char smem[];
  constexpr int GPW = 32 / G;  // move groups per warp
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int gl = lane & (G - 1);
  const int slot = warp * GPW + lane / G;
  const int Sn = a.spec_s;
  const int rep = blockIdx.x;
  if (rep >= a.n_reps) return;
  SpecShared& sh = *reinterpret_cast<SpecShared*>(smem);
  int* bkeys = reinterpret_cast<int*>(smem + a.spec_off_bkeys);
  unsigned* bmask = reinterpret_cast<unsigned*>(smem + a.spec_off_bmask);
  const int HB = 1 << a.spec_logHB;
  const int hcol = a.hcol;
  unsigned char* wb = smem + a.spec_off_warps + (size_t)slot * a.warp_smem;
  unsigned* draws = reinterpret_cast<unsigned*>(wb + a.off_draws);
  SlotScratch sm, gm;
  sm.keys = reinterpret_cast<int*>(wb + a.off_keys);
  sm.used = reinterpret_cast<int*>(wb + a.off_used);
  sm.bslot = reinterpret_cast<int*>(wb + a.off_bslot);
  sm.vals = reinterpret_cast<long long*>(wb + a.off_vals);
  sm.logH = a.logH;
  sm.stage = wb + a.off_stage;
  sm.idx = reinterpret_cast<int*>(wb + a.off_idx);
  const long long gi = (long long)rep * Sn + slot;
  const long long Hg = 1LL << a.g_logH;
  gm.keys = a.g_keys + gi * Hg;
  gm.used = a.g_used + gi * Hg;
  gm.bslot = a.g_bslot + gi * Hg;
  gm.vals = a.g_vals + gi * Hg * hcol;
  gm.logH = a.g_logH;
  gm.stage = reinterpret_cast<V4<Pos>*>(a.g_stage) + gi * a.g_stage_cap * 3;
  gm.idx = a.g_idx + gi * a.g_stage_cap;
  {
    const unsigned* src = reinterpret_cast<const unsigned*>(a.reps + rep);
    unsigned* dst = reinterpret_cast<unsigned*>(&sh.ws.rd);
    for (int i = tid; i < (int)(sizeof(RepDev) / 4); i += blockDim.x) dst[i] = src[i];
    const unsigned* cs = reinterpret_cast<const unsigned*>(a.ctl + (long long)rep * 5);
    unsigned* cd = reinterpret_cast<unsigned*>(sh.ws.ctl);
    for (int i = tid; i < (int)(5 * sizeof(cg_move_ctl) / 4); i += blockDim.x) cd[i] = cs[i];
    for (int i = tid; i < HB; i += blockDim.x) { bkeys[i] = -1; bmask[i] = 0u; }
    for (int i = tid; i < 30; i += blockDim.x) sh.ws.tally[i] = 0;
    for (int i = gl; i < (1 << a.logH); i += G) { sm.keys[i] = -1; sm.bslot[i] = -1; }
    for (int i = gl; i < (1 << a.logH) * hcol; i += G) sm.vals[i] = 0;
    if (gl == 0) sh.nused[slot] = 0;
    if (a.pool_on) {
      int* pk = reinterpret_cast<int*>(smem + a.off_pkeys);
      long long* pv = reinterpret_cast<long long*>(smem + a.off_pvals);
      for (int i = tid; i < (1 << a.pool_logH); i += blockDim.x) pk[i] = -1;
      for (int i = tid; i < (1 << a.pool_logH) * hcol; i += blockDim.x) pv[i] = 0;
    }
  }
  __syncthreads();
  if (tid == 0) {
    const RepDev& rd0 = sh.ws.rd;
    setup_f32(sh.ws);
    sh.t0 = rd0.draw_pos;
    sh.tlog = rd0.draw_pos;
    sh.run_dE = rd0.run_dE;
    sh.stop = 0;
    sh.cut = 0;
    sh.npool = 0;
  }
  __syncthreads();
  const long long words = (sh.ws.rd.n_beads + 31) / 32;
  sm.picked = gm.picked = a.picked + a.picked_off[rep] + slot * words;

  for (long long step = 0; step < a.n_steps; step++) {
    for (int ci = 0; ci < a.n_ctl; ci++) {
      cg_move_ctl& c = sh.ws.ctl[ci];
      const int kind = (int)c.move_kind;
      if (c.move_on == 1) {
        long long done = 0, batches = 0;
        while (done < c.num_per_cycle) {
          // every batch attempts at least one move or stops the run, so there
          // are at most num_per_cycle batches; the cap turns a stalled loop
          // into an error status instead of a spin
          if (++batches > c.num_per_cycle + 64) {
            if (tid == 0) sh.stop = E_SPIN;
            __syncthreads();
            break;
          }
          const int B = (int)(c.num_per_cycle - done < Sn ? c.num_per_cycle - done : Sn);
          const bool wlive = warp * GPW < B;  // the warp has a move of this batch
          const bool live = slot < B;
          evaluate_move<Pos, G, LEAN>(a, sh, rep, slot, gl, live, kind, c, sh.t0 + (unsigned long long)slot, draws,
                                sm, gm, bkeys, bmask, a.spec_logHB, B);
          __syncthreads();
          if (kind > CG_SLIDE) {  // position moves set their masks while evaluating
            if (wlive) conflict_mask<G>(a, sh, smem, rep, slot, gl, live, kind, B, sm, gm, bmask);
            __syncthreads();
          }
          // Resolve, computed by every warp from the plans (lane u reads move u):
          // the batch stands up to the first move that failed or meets an
          // earlier accepted move (everything before it stands, so "earlier
          // accepted" is the accepted moves below it), or up to and including
          // the first move whose voxels could not be registered.
          const bool valid = lane < B;
          const MovePlan& Pl = sh.plan[valid ? lane : 0];
          const bool p_err = valid && Pl.err != 0;
          const unsigned D = __ballot_sync(kFull, valid && !Pl.empty && Pl.dec);
          const unsigned F = __ballot_sync(kFull, p_err || (valid && (Pl.cmask & D & ((1u << lane) - 1u))));
          const unsigned RF = __ballot_sync(kFull, valid && Pl.regfail);
          const int first_fail = F ? __ffs((int)F) - 1 : B;
          int cut = first_fail;
          if (RF && __ffs((int)RF) < cut) cut = __ffs((int)RF);
          const unsigned acc = cut >= 32 ? D : (D & ((1u << cut) - 1u));
          if (warp == 0) {
            // bookkeeping of the standing moves, in move order where it is FP64
            const bool stand = lane < cut;
            const bool took = (acc >> lane) & 1u;
            const unsigned sm_m = __reduce_add_sync(kFull, stand ? (unsigned)Pl.m : 0u);
            const unsigned sm_v = __reduce_add_sync(kFull, stand ? (unsigned)Pl.nvox : 0u);
            const unsigned ac_m = __reduce_add_sync(kFull, took ? (unsigned)Pl.m : 0u);
            const unsigned ac_v = __reduce_add_sync(kFull, took ? (unsigned)Pl.nvox : 0u);
            if (lane == 0) {
              const unsigned n_acc = (unsigned)__popc(acc);
              c.num_attempt += cut;
              c.num_success += n_acc;
              unsigned long long* t = sh.ws.tally + kind * 6;
              t[0] += (unsigned long long)cut;
              t[1] += n_acc;
              t[2] += sm_m;
              t[3] += sm_v;
              t[4] += ac_m;
              t[5] += ac_v;
              // acc = alpha * x + (1 - alpha) * acc with x in {0, 1}, where
              // alpha * x is alpha or 0 exactly: one FP64 multiply-add chain
              double run = sh.run_dE, rate = c.acc_rate;
              const double alpha = c.alpha, beta = 1 - c.alpha;
              for (int w = 0; w < cut; w++) {
                const MovePlan& P = sh.plan[w];
                if (!LEAN && a.mlog) log_move(a, rep, sh.t0 + (unsigned long long)w - sh.tlog, P);
                if (P.empty) continue;
                if (P.dec && soft_dE(P.dE)) run += P.dE;
                rate = (P.dec ? alpha : 0.0) + beta * rate;
              }
              sh.run_dE = run;
              c.acc_rate = rate;
              sh.t0 += (unsigned long long)cut;
              if (cut == first_fail && first_fail < B && sh.plan[first_fail].err) sh.stop = sh.plan[first_fail].err;
            }
          }
          if (wlive && live)
            commit_and_clear<Pos, G>(a, sh, slot, gl, slot < cut && ((acc >> slot) & 1u), sm, gm, bkeys, bmask);
          __syncwarp();
          if (live && gl == 0) sh.nused[slot] = 0;
          if (kind <= CG_SLIDE && a.pool_on && sh.ws.rd.field_kind == 2)
            block_commit_pool(a, sh, smem, cut, acc, bkeys, bmask);
          __syncthreads();
          done += cut;
          if (sh.stop) break;
        }
      }
      if (sh.stop) break;
      if (tid == 0) update_amplitudes(c);
      __syncthreads();
    }
    if (sh.stop) break;
  }
  __syncthreads();
  {
    unsigned* cd = reinterpret_cast<unsigned*>(a.ctl + (long long)rep * 5);
    const unsigned* cs = reinterpret_cast<const unsigned*>(sh.ws.ctl);
    for (int i = tid; i < (int)(5 * sizeof(cg_move_ctl) / 4); i += blockDim.x) cd[i] = cs[i];
  }
  if (tid == 0) {
    RepDev* out = a.reps + rep;
    out->draw_pos = sh.t0;
    out->run_dE = sh.run_dE;
    out->err = (unsigned)sh.stop;
    unsigned long long* t = a.tally + (long long)rep * 30;
    for (int i = 0; i < 30; i++) t[i] += sh.ws.tally[i];
  }
}

}  // namespace cg

// Launch, shared-memory opt-in and register count of one storage / lanes
// pair (both its lean and full forms).
#define CG_SPEC_INSTANTIATE(Pos, G, NAME)                                                          \
  void cg_launch_spec_##NAME(const cg::KArgs& a, size_t smem, cudaStream_t s) {                    \
    if (a.lean)                                                                                    \
      cg::spec_kernel<Pos, G, true><<<a.n_reps, 32 * a.spec_w, smem, s>>>(a);                      \
    else                                                                                           \
      cg::spec_kernel<Pos, G, false><<<a.n_reps, 32 * a.spec_w, smem, s>>>(a);                     \
  }                                                                                                \
  cudaError_t cg_spec_smem_##NAME(int bytes) {                                                     \
    cudaError_t e = cudaFuncSetAttribute(cg::spec_kernel<Pos, G, false>,                           \
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);      \
    if (e != cudaSuccess) return e;                                                                \
    return cudaFuncSetAttribute(cg::spec_kernel<Pos, G, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                bytes);                                                            \
  }                                                                                                \
  int cg_spec_regs_##NAME() {                                                                      \
    cudaFuncAttributes at, bt;                                                                     \
    if (cudaFuncGetAttributes(&at, cg::spec_kernel<Pos, G, false>) != cudaSuccess) return 0;       \
    if (cudaFuncGetAttributes(&bt, cg::spec_kernel<Pos, G, true>) != cudaSuccess) return 0;        \
    return at.numRegs > bt.numRegs ? at.numRegs : bt.numRegs;                                      \
  }
