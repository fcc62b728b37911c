// cg_mc.cu -- the MC inner loop of chromo on GB300 (sm_103a), one warp per replica.
//
// One launch runs `n_steps` MC steps (chromo/mc/mc_sim.pyx:88-103) on every
// replica.  Warp w of the grid owns replica w: it keeps the replica's
// parameters and move controllers in shared memory, proposes each move
// (chromo/mc/move_funcs.pyx), evaluates the SSWLC elastic dE of the two
// boundary bonds or of each rotated bead (chromo/polymers.pyx:1024-1346), the
// binding dE from a precomputed single-site free-energy table
// (:1383-1538), re-deposits the moved beads into the voxel grid by trilinear
// weights and evaluates the chi / binder field dE over only the touched
// voxels (chromo/fields.pyx:1149-1875), applies the Metropolis test
// (chromo/mc/mc_sim.pyx:163-182) and commits.
//
// Touched voxels are deduplicated in a per-warp open-addressing hash in
// shared memory whose values are int64 fixed-point density deltas (2^-40 of a
// unit trilinear weight); the grid itself is int64 fixed point, so a deposit
// is exactly undone by the opposite deposit and the grid never depends on the
// order of updates.
#include <mutex>
#include <cuda_runtime.h>

#include "cg_device.cuh"
#include "cg_kernels.h"
#include "cg_move.cuh"
#include "cg_energy.cuh"

namespace cg {


// ---------------------------------------------------------------- the kernel

template <typename Pos, bool AUDIT>
__global__ void __launch_bounds__(128, 1) mc_kernel(KArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int rep = AUDIT ? a.audit_rep : blockIdx.x * a.wpb + warp;
  if (!AUDIT && rep >= a.n_reps) return;
  if (AUDIT && (blockIdx.x != 0 || warp != 0)) return;
  unsigned char* base = smem + a.spec_off_warps + (size_t)warp * a.warp_smem;
  WarpShared& ws = reinterpret_cast<SpecShared*>(smem)->ws;
  int* s_keys = reinterpret_cast<int*>(base + a.off_keys);
  int* s_used = reinterpret_cast<int*>(base + a.off_used);
  long long* s_vals = reinterpret_cast<long long*>(base + a.off_vals);
  Pos* s_stage = reinterpret_cast<Pos*>(base + a.off_stage);
  int* s_idx = reinterpret_cast<int*>(base + a.off_idx);
  const int ncol = a.hcol;  // stride of the voxel-hash values

  {  // load replica parameters and controllers into shared memory
    const unsigned* src = reinterpret_cast<const unsigned*>(a.reps + rep);
    unsigned* dst = reinterpret_cast<unsigned*>(&ws.rd);
    for (int i = lane; i < (int)(sizeof(RepDev) / 4); i += 32) dst[i] = src[i];
    const unsigned* cs = reinterpret_cast<const unsigned*>(a.ctl + (long long)rep * 5);
    unsigned* cd = reinterpret_cast<unsigned*>(ws.ctl);
    for (int i = lane; i < (int)(5 * sizeof(cg_move_ctl) / 4); i += 32) cd[i] = cs[i];
    for (int i = lane; i < (1 << a.logH); i += 32) s_keys[i] = -1;
    for (int i = lane; i < (1 << a.logH) * ncol; i += 32) s_vals[i] = 0;
    if (lane < 30) ws.tally[lane] = 0;
    if (lane == 0) ws.nused = 0;
  }
  __syncwarp();
  if (lane == 0) setup_f32(ws);
  __syncwarp();
  using Real = Pos;
  const RepDev& rd = ws.rd;
  const GridF& gf = ws.gf;
  const long long N = rd.n_beads;
  const V4<Pos>* r4 = reinterpret_cast<const V4<Pos>*>(a.r4) + rd.bead_off;
  const V4<Pos>* t34 = reinterpret_cast<const V4<Pos>*>(a.t34) + rd.bead_off;
  const V4<Pos>* t24 = reinterpret_cast<const V4<Pos>*>(a.t24) + rd.bead_off;
  V4<Pos>* r4w = reinterpret_cast<V4<Pos>*>(a.r4) + rd.bead_off;
  V4<Pos>* t34w = reinterpret_cast<V4<Pos>*>(a.t34) + rd.bead_off;
  V4<Pos>* t24w = reinterpret_cast<V4<Pos>*>(a.t24) + rd.bead_off;
  unsigned* st = a.states + rd.bead_off;
  const unsigned* mk = a.marks + rd.bead_off;
  const double* bonds = a.bonds + rd.bead_off * 6;
  const float* bonds32 = a.bonds32 + rd.bead_off * 8;
  // per-replica global scratch (used when a move is too large for shared memory)
  const long long gi = (long long)rep * a.spec_s;  // the replica's first move-slot region
  int* g_keys = a.g_keys + gi * (1 << a.g_logH);
  int* g_used = a.g_used + gi * (1 << a.g_logH);
  long long* g_vals = a.g_vals + gi * (1 << a.g_logH) * ncol;
  Pos* g_stage = reinterpret_cast<Pos*>(a.g_stage) + gi * a.g_stage_cap * 9;
  int* g_idx = a.g_idx + gi * a.g_stage_cap;
  unsigned* picked = a.picked + a.picked_off[rep];

  Rng<AUDIT> g;
  if constexpr (AUDIT) {
    g.draws = a.a_draws; g.n = a.a_n_draws; g.bs = a.a_bstates; g.nbs = a.a_n_bstates;
    g.pos = 0; g.bpos = 0; g.fail = false;
  } else {
    g.init(a.seed, rep, rd.draw_pos, rd.bstate_pos);
  }
  unsigned err = rd.err;
  double run_dE = rd.run_dE;
  long long nrec = 0;
  unsigned long long* tally = ws.tally;

  for (long long step = 0; step < a.n_steps && !err; step++) {
    for (int ci = 0; ci < a.n_ctl && !err; ci++) {
      cg_move_ctl& c = ws.ctl[ci];
      const int kind = (int)c.move_kind;
      if (c.move_on == 1) {
        for (long long jj = 0; jj < c.num_per_cycle && !err; jj++) {
          // ------------------------------------------------ one mc_step
          const unsigned long long draw0 = g.pos;
          const bool check_field = rd.field_kind != 0 && kind != CG_TANGENT_ROTATION;
          const bool density = rd.field_kind == 2;
          if (lane == 0) c.num_attempt += 1;  // moves.pyx:151
          long long ind0 = 0, indf = 0, m = 0;
          int bsel = -1;
          // dE = dEp (polymer) + dEs (field, FF for FP32 storage) + dEh (FP64 part)
          using Acc = typename AccOf<Real>::type;
          Acc dEp = acc_zero<Acc>(), dEs = acc_zero<Acc>();
          double dEh = 0;
          long long dEH = 0;  // the exact 1e99 penalties, in kHugeUnit units
          long long nvox = 0;
          bool empty = false;
          int* keys = s_keys; int* used = s_used; long long* vals = s_vals; int logH = a.logH;
          Pos* stage = s_stage;
          int* idx = s_idx;
          if (kind <= CG_SLIDE) {
            // ---------------- segment moves: crank_shaft / end_pivot / slide
            Real Md[3][4];
            if (kind == CG_CRANK_SHAFT) {  // move_funcs.pyx:39-101, 157-280
              Real ang = (Real)c.amp_move * (uni<Real>(g.next()) - (Real)0.5);
              const unsigned xb0 = g.next();
              long long b0 = sizeof(Real) == 4 ? scaled_index(xb0, N) : (long long)(int)(unif(xb0) * (double)N);
              long long b1 = from_point(g, c.amp_bead, N, b0, err);
              if (b1 < 1) b1 = 1;
              check_bead_bounds(b0, b1, N, ind0, indf);
              Real pa[3], pb[3], dir[3], p[3];
              long long ia, ib;
              if (ind0 == indf - 1 && ind0 == 0) { ia = indf; ib = ind0; }
              else if (ind0 == indf - 1 && ind0 == N - 1) { ia = ind0; ib = ind0 - 1; }
              else if (ind0 == 0 && indf == N) { ia = indf - 1; ib = ind0; }
              else if (ind0 == 0) { ia = indf; ib = ind0; }
              else if (indf == N) { ia = indf - 1; ib = ind0 - 1; }
              else { ia = indf; ib = ind0 - 1; }
              if (err) break;
              ld3(r4, ia, pa); ld3(r4, ib, pb);
              for (int i = 0; i < 3; i++) dir[i] = pa[i] - pb[i];
              Real mag = rsqrt_(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
              if (mag < (Real)1E-5) sphere<Real>(g, dir);
              else { Real sc = (Real)1 / mag; for (int i = 0; i < 3; i++) dir[i] = dir[i] * sc; }
              long long ip;
              if (ind0 == 0 && indf != N) ip = indf;
              else if (ind0 != 0 && indf == N) ip = ind0 - 1;
              else if (ind0 == 0 && indf == N) ip = ind0;
              else ip = ind0 - 1;
              ld3(r4, ip, p);
              axis_rotation(dir, p, ang, Md);
            } else if (kind == CG_END_PIVOT) {  // move_funcs.pyx:285-398
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
              if (err) break;
              ld3(r4, ip, p);
              axis_rotation(axis, p, ang, Md);
            } else {  // slide, move_funcs.pyx:403-465
              Real amp = (Real)c.amp_move * uni<Real>(g.next()), d[3];
              sphere<Real>(g, d);
              for (int i = 0; i < 3; i++) { Md[i][3] = d[i] * amp; }
              long long b0 = g.next() % (unsigned)N;
              long long b1 = from_point(g, c.amp_bead, N, b0, err);
              check_bead_bounds(b0, b1, N, ind0, indf);
            }
            if (err) break;
            // the matrix in the arithmetic of the storage type (exact for FP64)
            Real M[3][4];
            for (int i = 0; i < 3; i++)
              for (int j = 0; j < 4; j++) M[i][j] = (Real)Md[i][j];
            m = indf - ind0;
            if (m == 0) {
              empty = true;
            } else {
              if (m > a.stage_cap) { stage = g_stage; }
              const bool smem_hash = 16 * m * 2 <= (1LL << a.logH);
              if (!smem_hash) { keys = g_keys; used = g_used; vals = g_vals; logH = a.g_logH; }
              Acc part = acc_zero<Acc>();
              int oob = 0;
              for (long long k = lane; k < m; k += 32) {
                const long long i = ind0 + k;
                V4<Pos> R = r4[i], T3 = t34[i], T2 = t24[i];
                Real r[3] = {R.x, R.y, R.z};
                Real t3[3] = {T3.x, T3.y, T3.z};
                Real t2[3] = {T2.x, T2.y, T2.z};
                Real tr[3], tt3[3], tt2[3];
                if (kind == CG_SLIDE) {
                  for (int j = 0; j < 3; j++) { tr[j] = r[j] + M[j][3]; tt3[j] = t3[j]; tt2[j] = t2[j]; }
                } else {
                  for (int j = 0; j < 3; j++) {
                    Real er = 0, e3 = 0, e2 = 0;
                    for (int q = 0; q < 3; q++) { er += M[j][q] * r[q]; e3 += M[j][q] * t3[q]; e2 += M[j][q] * t2[q]; }
                    tr[j] = er + M[j][3];
                    tt3[j] = e3;
                    tt2[j] = e2;
                  }
                }
                const bool fin = isfinite(tr[0]) && isfinite(tr[1]) && isfinite(tr[2]);
                if (!fin) err |= E_NONFINITE;
                Pos* sg = stage + k * 9;
                for (int j = 0; j < 3; j++) { sg[j] = (Pos)tr[j]; sg[3 + j] = (Pos)tt3[j]; sg[6 + j] = (Pos)tt2[j]; }
                if (k == 0 && ind0 != 0) {  // continuous_dE_poly forward bond, polymers.pyx:1121-1131
                  Real r0[3], t30[3];
                  ld3(r4, i - 1, r0); ld3(t34, i - 1, t30);
                  acc_add(part, pair_dE_fwd(bond_at(bonds, bonds32, i - 1, (Real)0), r0, r, tr, t30, t3, tt3));
                  if (rd.twist) {  // SSTWLC twist term, polymers.pyx:2104-2175
                    const Frame l = frame_of(t24[i - 1], t34[i - 1]);
                    acc_add_d(part, twist_pair_dE(a.twist + 2 * (rd.bead_off + i - 1), l, frame_of(t2, t3), l,
                                                  frame_of(tt2, tt3)));
                  }
                }
                if (k == m - 1 && indf != N) {  // reverse bond, polymers.pyx:1132-1142
                  Real r1[3], t31[3];
                  ld3(r4, i + 1, r1); ld3(t34, i + 1, t31);
                  acc_add(part, pair_dE_rev(bond_at(bonds, bonds32, i, (Real)0), r, tr, r1, t3, tt3, t31));
                  if (rd.twist) {  // :2177-2248
                    const Frame rr = frame_of(t24[i + 1], t34[i + 1]);
                    acc_add_d(part, twist_pair_dE(a.twist + 2 * (rd.bead_off + i), frame_of(t2, t3), rr,
                                                  frame_of(tt2, tt3), rr));
                  }
                }
                if (check_field && rd.confine_kind) {
                  oob += out_of_bounds(rd, tr, true) * 65536 + out_of_bounds(rd, r, false);
                }
                if (density && fin) {
                  Real w0[8], w1[8];
                  int v0[8], v1[8];
                  move_weights(rd, gf, r, w0, v0);
                  move_weights(rd, gf, tr, w1, v1);
                  unsigned s = st[i];
                  deposit_bead(rd, ncol, keys, used, &ws.nused, vals, logH, w0, v0, s, true, err);
                  deposit_bead(rd, ncol, keys, used, &ws.nused, vals, logH, w1, v1, s, false, err);
                }
              }
              err = __reduce_or_sync(kFull, err);
              dEp = warp_sum(part);
              if (check_field && rd.confine_kind) {
                int oo = __reduce_add_sync(kFull, (unsigned)oob);
                dEH += ((long long)(oo >> 16) - (long long)(oo & 0xFFFF)) << 40;
              }
              __syncwarp();
              if (density) {
                int nu = ws.nused;
                field_dE_voxels(ws, a, ncol, keys, used, vals, nu, lane, nvox, dEs, dEh, dEH);
              }
            }
          } else if (kind == CG_TANGENT_ROTATION) {
            // ---------------- tangent_rotation, move_funcs.pyx:470-582
            Real ang = (Real)c.amp_move * (uni<Real>(g.next()) - (Real)0.5);
            long long n = (long long)(g.next() % (unsigned)c.amp_bead) + 1;
            if (n > N) { err |= E_WINDOW; break; }
            m = n;
            if (m > a.stage_cap) { stage = g_stage; idx = g_idx; }
            // distinct random beads, drawn in order with redraws (get_inds)
            long long got = 0;
            int it = 0;
            while (got < n) {
              if (++it > kMaxIter) { err |= E_SPIN; break; }
              bool ok;
              unsigned x = g.at(g.pos + lane, ok);
              long long cand = ok ? (long long)(x % (unsigned)N) : -1 - lane;
              unsigned grp = __match_any_sync(kFull, cand);
              bool first = (grp & ((1u << lane) - 1u)) == 0;
              bool fresh = ok && first && !((picked[cand >> 5] >> (cand & 31)) & 1u);
              unsigned bal = __ballot_sync(kFull, fresh);
              unsigned okb = __ballot_sync(kFull, ok);
              long long need = n - got;
              int cnt = __popc(bal);
              int rank = __popc(bal & ((1u << lane) - 1u));
              if (fresh && rank < need) {
                idx[got + rank] = (int)cand;
                atomicOr(&picked[cand >> 5], 1u << (cand & 31));
              }
              long long consumed;
              if (cnt >= need) {
                unsigned b = bal;
                for (long long q = 1; q < need; q++) b &= b - 1;
                consumed = __ffs(b);  // lane of the last needed candidate + 1
                got = n;
              } else {
                consumed = 32;
                got += cnt;
              }
              if ((okb & (consumed >= 32 ? kFull : ((1u << consumed) - 1u))) !=
                  (consumed >= 32 ? kFull : ((1u << consumed) - 1u))) {
                g.fail = true; err |= E_STREAM;
              }
              g.pos += consumed;
              __syncwarp();
            }
            if (err) break;
            const unsigned long long axis_base = g.pos;
            Acc part = acc_zero<Acc>();
            Real sa, ca;
            rsincos(ang, &sa, &ca);
            for (long long k = lane; k < m; k += 32) {
              const long long i = idx[k];
              bool ok1, ok2;
              unsigned xa = g.at(axis_base + 2 * k, ok1), xb = g.at(axis_base + 2 * k + 1, ok2);
              if (!(ok1 && ok2)) err |= E_STREAM;
              Real axis[3];
              sphere_from<Real>(xa, xb, axis);
              const Real origin[3] = {0, 0, 0};
              Real Md[3][4];
              axis_rotation_sc(axis, origin, sa, ca, Md);
              Real M[3][4];
              for (int ii = 0; ii < 3; ii++)
                for (int jj2 = 0; jj2 < 4; jj2++) M[ii][jj2] = (Real)Md[ii][jj2];
              Real r[3], t3[3], t2[3], tt3[3], tt2[3];
              ld3(r4, i, r); ld3(t34, i, t3); ld3(t24, i, t2);
              for (int j = 0; j < 3; j++) {
                Real e3 = 0, e2 = 0;
                for (int q = 0; q < 3; q++) { e3 += M[j][q] * t3[q]; e2 += M[j][q] * t2[q]; }
                tt3[j] = e3;
                tt2[j] = e2;
              }
              Pos* sg = stage + k * 9;
              for (int j = 0; j < 3; j++) { sg[3 + j] = (Pos)tt3[j]; sg[6 + j] = (Pos)tt2[j]; }
              Acc de = acc_zero<Acc>();
              if (i != 0) {
                Real r0[3], t30[3];
                ld3(r4, i - 1, r0); ld3(t34, i - 1, t30);
                acc_add(de, pair_dE_fwd(bond_at(bonds, bonds32, i - 1, (Real)0), r0, r, r, t30, t3, tt3));
              }
              if (i + 1 != N) {
                Real r1[3], t31[3];
                ld3(r4, i + 1, r1); ld3(t34, i + 1, t31);
                acc_add(de, pair_dE_rev(bond_at(bonds, bonds32, i, (Real)0), r, r, r1, t3, tt3, t31));
              }
              if (rd.twist) {  // SSTWLC twist terms of both bonds
                const double* tw = a.twist + 2 * rd.bead_off;
                const Frame cur = frame_of(t2, t3), nw = frame_of(tt2, tt3);
                double dt = 0;
                if (i != 0) {
                  const Frame l = frame_of(t24[i - 1], t34[i - 1]);
                  dt += twist_pair_dE(tw + 2 * (i - 1), l, cur, l, nw);
                }
                if (i + 1 != N) {
                  const Frame rr = frame_of(t24[i + 1], t34[i + 1]);
                  dt += twist_pair_dE(tw + 2 * i, cur, rr, nw, rr);
                }
                acc_add_d(de, dt);
              }
              acc_add(part, de);
            }
            g.pos = axis_base + 2 * (unsigned long long)m;
            err = __reduce_or_sync(kFull, err);
            dEp = warp_sum(part);
            ind0 = idx[0]; indf = ind0 + 1;
          } else {
            // ---------------- change_binding_state, move_funcs.pyx:717-820
            bsel = (int)(g.next() % (unsigned)rd.nb);
            long long b0 = g.next() % (unsigned)N;
            long long b1 = from_point(g, c.amp_bead, N, b0, err);
            if (err) break;
            check_bead_bounds(b0, b1, N, ind0, indf);
            m = indf - ind0;
            const int nt = rd.sites[bsel];
            if (m > a.stage_cap) idx = g_idx;
            const bool smem_hash = 8 * m * 2 <= (1LL << a.logH);
            if (!smem_hash) { keys = g_keys; used = g_used; vals = g_vals; logH = a.g_logH; }
            Acc part = acc_zero<Acc>();
            int dbl = 0;  // doubly-bound trial minus current, chosen binder (fields.pyx:1877-1937)
            for (long long k = lane; k < m; k += 32) {
              const long long i = ind0 + k;
              bool ok;
              int s_new = g.state_at(g.bpos + k, nt, ok);
              if (!ok) err |= E_STREAM;
              unsigned sw = st[i], mw = mk[i];
              int s_old = (int)((sw >> (8 * bsel)) & 0xFF);
              // bead_binding_dE, polymers.pyx:1408-1538
              acc_add(part, bead_bind_dE(ws, sw, mw, bsel, s_new, (Real)0));
              dbl += (s_new == 2 ? 1 : 0) - (s_old == 2 ? 1 : 0);
              idx[k] = s_new;
              if (density && s_new != s_old) {
                Real p[3], w[8];
                int v[8];
                ld3(r4, i, p);
                move_weights(rd, gf, p, w, v);
#pragma unroll
                for (int l = 0; l < 8; l++) {
                  int slot = hash_slot(keys, used, &ws.nused, logH, v[l], err);
                  if (slot < 0) break;
                  add_delta(vals, ncol, slot, 1 + bsel, q40(w[l]) * (long long)(s_new - s_old));
                }
              }
            }
            g.bpos += (unsigned long long)m;
            err = __reduce_or_sync(kFull, err);
            dEp = warp_sum(part);
            int ddb = __reduce_add_sync(kFull, (unsigned)dbl);
            if (check_field && rd.field_kind == 1 && rd.confine_kind == 2) {
              // NullField evaluates the (cubical) confinement on binding moves too
              int oob = 0;
              for (long long k = lane; k < m; k += 32) {
                double p[3];
                ld3(r4, ind0 + k, p);
                oob += out_of_bounds(rd, p, true);
              }
              dEH += (long long)__reduce_add_sync(kFull, (unsigned)oob) << 40;
            }
            __syncwarp();
            if (density) {
              int nu = ws.nused;
              field_dE_voxels(ws, a, ncol, keys, used, vals, nu, lane, nvox, dEs, dEh, dEH);
              add_intra(ws, bsel, ddb, dEs, dEh);
            }
          }
          if (AUDIT && g.fail) err |= E_STREAM;
          if (err) break;
          dEh = with_huge(dEh, dEH);
          // ------------------------------------------------ Metropolis + commit
          int accepted = -1;
          if (!empty) {
            double dE = 0;
            bool acc = decide(g.next(), dEp, dEs, dEh, &dE);
            if (AUDIT && g.fail) { err |= E_STREAM; break; }
            accepted = acc ? 1 : 0;
            if (acc) {
              if (kind <= CG_SLIDE) {
                for (long long k = lane; k < m; k += 32) {
                  const Pos* sg = stage + k * 9;
                  const long long i = ind0 + k;
                  r4w[i] = V4<Pos>{sg[0], sg[1], sg[2], (Pos)0};
                  if (kind != CG_SLIDE) {
                    t34w[i] = V4<Pos>{sg[3], sg[4], sg[5], (Pos)0};
                    t24w[i] = V4<Pos>{sg[6], sg[7], sg[8], (Pos)0};
                  }
                }
              } else if (kind == CG_TANGENT_ROTATION) {
                for (long long k = lane; k < m; k += 32) {
                  const Pos* sg = stage + k * 9;
                  const long long i = idx[k];
                  t34w[i] = V4<Pos>{sg[3], sg[4], sg[5], (Pos)0};
                  t24w[i] = V4<Pos>{sg[6], sg[7], sg[8], (Pos)0};
                }
              } else {
                for (long long k = lane; k < m; k += 32) {
                  const long long i = ind0 + k;
                  unsigned sw = st[i];
                  sw = (sw & ~(0xFFu << (8 * bsel))) | ((unsigned)idx[k] << (8 * bsel));
                  st[i] = sw;
                }
              }
              if (lane == 0) { c.num_success += 1; if (soft_dE(dE)) run_dE += dE; }
            }
            if (density && check_field) commit_grid(rd, a, ncol, keys, used, vals, ws.nused, lane, acc);
            if (kind == CG_TANGENT_ROTATION) {
              for (long long k = lane; k < m; k += 32) {
                int i = idx[k];
                atomicAnd(&picked[i >> 5], ~(1u << (i & 31)));
              }
            }
            if (lane == 0) {
              c.acc_rate = c.alpha * (acc ? 1.0 : 0.0) + (1 - c.alpha) * c.acc_rate;
              tally[kind * 6 + 1] += acc ? 1 : 0;
              tally[kind * 6 + 4] += acc ? (unsigned long long)m : 0;
              tally[kind * 6 + 5] += acc ? (unsigned long long)nvox : 0;
            }
          }
          if (lane == 0) {
            tally[kind * 6 + 0] += 1;
            tally[kind * 6 + 2] += (unsigned long long)m;
            tally[kind * 6 + 3] += (unsigned long long)nvox;
          }
          __syncwarp();
          if (lane == 0) ws.nused = 0;
          if (AUDIT && lane == 0 && nrec < a.a_max_recs) {
            cg_move_record rec;
            rec.kind = kind; rec.n_inds = (int)m; rec.ind0 = (int)ind0; rec.indf = (int)indf;
            rec.dE_poly = empty ? 0.0 : acc_d(dEp); rec.dE_field = empty ? 0.0 : acc_d(dEs) + dEh;
            rec.accepted = accepted; rec.n_draws = (int)(g.pos - draw0);
            a.a_recs[nrec] = rec;
          }
          nrec++;
          __syncwarp();
        }
      }
      // SimpleControl.update_amplitudes, mc_controller.py:126-189
      if (lane == 0 && c.ctrl_kind == 1) {
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
      __syncwarp();
    }
  }
  // ------------------------------------------------ write back
  __syncwarp();
  {
    unsigned* cd = reinterpret_cast<unsigned*>(a.ctl + (long long)rep * 5);
    const unsigned* cs = reinterpret_cast<const unsigned*>(ws.ctl);
    for (int i = lane; i < (int)(5 * sizeof(cg_move_ctl) / 4); i += 32) cd[i] = cs[i];
  }
  if (lane == 0) {
    RepDev* out = a.reps + rep;
    out->draw_pos = AUDIT ? rd.draw_pos : g.pos;
    out->bstate_pos = AUDIT ? rd.bstate_pos : g.bpos;
    out->run_dE = run_dE;
    out->err = err;
    if (AUDIT) {
      a.a_out[0] = nrec;
      a.a_out[1] = (long long)g.pos;
      a.a_out[2] = (long long)g.bpos;
    }
    unsigned long long* t = a.tally + (long long)rep * 30;
    for (int i = 0; i < 30; i++) t[i] += tally[i];
  }
}

// ---------------------------------------------------------------- re-deposit
// update_all_densities_for_all_polymers (chromo/fields.pyx:2041-2106): every
// bead adds its eight fixed-point weights; int64 atomics make the result
// independent of the order of the adds.
template <typename Pos>
__global__ void deposit_kernel(KArgs a, int rep_only) {
  const int rep = rep_only >= 0 ? rep_only : blockIdx.y;
  const RepDev& rd = a.reps[rep];
  if (rd.field_kind != 2) return;
  const V4<Pos>* r4 = reinterpret_cast<const V4<Pos>*>(a.r4) + rd.bead_off;
  long long* grid = a.grid + rd.vox_off * a.ncol;
  GridF gf;
  make_gridf(rd, gf);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < rd.n_beads;
       i += (long long)gridDim.x * blockDim.x) {
    Pos p[3], w[8];
    int v[8];
    ld3(r4, i, p);
    voxel_weights(rd, gf, p, w, v);
    unsigned s = a.states[rd.bead_off + i];
    for (int l = 0; l < 8; l++) {
      long long q = q40(w[l]);
      atomicAdd((unsigned long long*)&grid[(long long)v[l] * a.ncol], (unsigned long long)q);
      for (int b = 0; b < rd.nb; b++) {
        long long qb = q * (long long)((s >> (8 * b)) & 0xFF);
        if (qb) atomicAdd((unsigned long long*)&grid[(long long)v[l] * a.ncol + 1 + b], (unsigned long long)qb);
      }
    }
  }
}

// ---------------------------------------------------------------- FP64 energies
// one block per replica; deterministic block tree reduction.
__device__ double block_sum(double v, double* sh) {
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

template <typename Pos>
__global__ void energy_kernel(KArgs a, double* out) {
  __shared__ double sh[32];
  const int rep = blockIdx.x;
  const RepDev& rd = a.reps[rep];
  EnergyParts p{0.0, 0.0, 0.0, 0.0, {0, 0, 0}};
  for (long long i = threadIdx.x; i < rd.n_beads; i += blockDim.x) bead_energy<Pos>(a, rd, i, p);
  if (rd.field_kind == 2)
    for (long long v = threadIdx.x; v < rd.n_vox; v += blockDim.x) voxel_energy(a, rd, v, p);
  const double el = p.el, bi = p.bi, fe = p.fe, sx = p.sx;
  const long long* dbl = p.dbl;
  double t_el = block_sum(el, sh);
  double t_bi = block_sum(bi, sh);
  double t_fe = block_sum(fe, sh);
  double t_sx = block_sum(sx, sh);
  double t_db[CG_MAX_BINDERS];
  for (int b = 0; b < CG_MAX_BINDERS; b++) t_db[b] = block_sum((double)dbl[b], sh);
  if (threadIdx.x == 0) {
    double intra = 0;
    for (int b = 0; b < rd.nb; b++) intra += rd.intra[b] * t_db[b];
    out[rep * 5 + 0] = t_el;
    out[rep * 5 + 1] = t_bi;
    out[rep * 5 + 2] = rd.field_kind == 2 ? t_fe + intra : 0.0;
    out[rep * 5 + 3] = rd.run_dE;
    out[rep * 5 + 4] = t_sx;
  }
}

// The chi-free sums S_r alone (the input of the exchange): the same per-thread
// order and block reduction as energy_kernel's out[5 r + 4], so the values are
// identical, without the elastic, binding and binder-density terms.
__global__ void chi_sum_kernel(KArgs a, double* out) {
  __shared__ double sh[32];
  const int rep = blockIdx.x;
  const RepDev& rd = a.reps[rep];
  double sx = 0;
  if (rd.field_kind == 2 && !rd.has_access) {
    // uniform voxel volume: S = (V / Vb) c^2 sum g0^2 with c = 2^-40 Vb / V the
    // volume fraction per fixed-point unit (no FP64 division per voxel); a
    // voxel whose volume fraction may be above vf_limit takes the exact test
    // of energy_kernel and is left out of S when above it
    const long long* grid = a.grid + rd.vox_off * a.ncol;
    const double c = kFxInv / rd.vol_bin * rd.bead_vol;
    const double near = rd.vf_limit * (1.0 - 1e-9);
    double s00 = 0;
    for (long long v = threadIdx.x; v < rd.n_vox; v += blockDim.x) {
      const long long n = grid[v * a.ncol];
      const double g0 = (double)n;
      if (g0 * c > near && ((double)n * kFxInv) / rd.vol_bin * rd.bead_vol > rd.vf_limit) continue;
      s00 += g0 * g0;
    }
    sx = (rd.vol_bin / rd.bead_vol) * (c * c) * s00;
  } else if (rd.field_kind == 2) {
    const long long* grid = a.grid + rd.vox_off * a.ncol;
    for (long long v = threadIdx.x; v < rd.n_vox; v += blockDim.x) {
      double V = rd.has_access ? a.access_vol[rd.vox_off + v] : rd.vol_bin;
      double vf = ((double)grid[v * a.ncol] * kFxInv) / V * rd.bead_vol;
      if (!(vf > rd.vf_limit)) sx += (V / rd.bead_vol) * vf * vf;
    }
  }
  const double t = block_sum(sx, sh);
  if (threadIdx.x == 0) out[rep * 5 + 4] = t;
  if (a.mu_rungs > 1) {  // bound sites of the mu-ladder binder (exact integer sum)
    const unsigned* st = a.states + rd.bead_off;
    const int sh8 = 8 * a.mu_binder;
    long long nbl = 0;
    for (long long i = threadIdx.x; i < rd.n_beads; i += blockDim.x) nbl += (st[i] >> sh8) & 0xFFu;
    const double nbt = block_sum((double)nbl, sh);
    if (threadIdx.x == 0) a.nbound[rep] = nbt;
  }
}

// ---------------------------------------------------------------- replica exchange
// Swap chi between neighbouring rungs of each ladder (n_rungs consecutive
// rung slots per ladder).  eout[5 r + 4] holds S_r = sum over the voxels at
// or below vf_limit of (V/Vb) vf^2, the chi-free part of replica r's field
// energy (a voxel above the limit costs 1e99 vf whatever chi is), so that
// E_r = chi_r S_r + (chi-independent terms).  One block; round < 0 takes the
// round number from a device counter and advances it (graph replays).
__global__ void exchange_kernel(KArgs a, const double* eout, int n_rungs, long long round_in,
                                unsigned long long seed) {
  __shared__ long long round_sh;
  if (threadIdx.x == 0) round_sh = round_in >= 0 ? round_in : (long long)a.xround[0];
  __syncthreads();
  const long long round = round_sh;
  const int parity = (int)(round & 1);
  const int ladders = a.n_reps / n_rungs;
  const int per = n_rungs / 2;  // no chi pairs for n_rungs = 1 (a mu-only ladder)
  for (int t = threadIdx.x; t < ladders * per; t += blockDim.x) {
    const int ladder = t / per, pair = t % per;
    if (2 * pair + 1 + parity >= n_rungs) continue;
    const int ra = ladder * n_rungs + 2 * pair + parity, rb = ra + 1;
    const int ia = a.rep_of_rung[ra], ib = a.rep_of_rung[rb];
    const double ca = a.reps[ia].chi, cb = a.reps[ib].chi;
    const double x = (ca - cb) * (eout[5 * ia + 4] - eout[5 * ib + 4]);
    uint4 o = philox(make_uint4((unsigned)round, (unsigned)(round >> 32), (unsigned)ra, 0x3C6EF372u),
                     make_uint2((unsigned)seed ^ 0xA4093822u, (unsigned)(seed >> 32)));
    const double u = (double)(o.x >> 1) / kRandMax;
    if (u < exp(x)) {
      // E_r = chi_r S_r + (chi-free terms): the swap's energy change of each replica
      a.reps[ia].xch_dE += (cb - ca) * eout[5 * ia + 4];
      a.reps[ib].xch_dE += (ca - cb) * eout[5 * ib + 4];
      a.reps[ia].chi = cb;
      a.reps[ib].chi = ca;
      a.rep_of_rung[ra] = ib;
      a.rep_of_rung[rb] = ia;
      a.swaps[ra] += 1;
    }
    a.swap_attempts[ra] += 1;
  }
  __syncthreads();
  // mu swaps between neighbouring mu rungs (same chi rung) of each grid of
  // mu_rungs x n_rungs slots: the mu-dependent energy of replica r is
  // -m(mu_r) N_r with m(mu) = mu (2 - f) for mu > 0, mu f otherwise
  // (chromo/polymers.pyx:1520-1531), N_r its bound sites of the binder, so a
  // swap changes the energy by dE = m_a(mu_a) N_a + m_b(mu_b) N_b
  // - m_a(mu_b) N_a - m_b(mu_a) N_b and is accepted iff u < exp(-dE).
  if (a.mu_rungs > 1) {
    const int nm = a.mu_rungs, b = a.mu_binder;
    const int grids = a.n_reps / (nm * n_rungs);
    const int mper = nm / 2;
    for (int t = threadIdx.x; t < grids * n_rungs * mper; t += blockDim.x) {
      const int grid = t / (n_rungs * mper), rest = t % (n_rungs * mper);
      const int crung = rest / mper, pair = rest % mper;
      const int mr = 2 * pair + parity;
      if (mr + 1 >= nm) continue;
      const int sa = (grid * nm + mr) * n_rungs + crung, sb = sa + n_rungs;
      const int ia = a.rep_of_rung[sa], ib = a.rep_of_rung[sb];
      const double mua = a.reps[ia].mu[b], mub = a.reps[ib].mu[b];
      const double fa = a.reps[ia].mu_adjust, fb = a.reps[ib].mu_adjust;
      auto eff = [](double mu, double f) { return mu > 0 ? mu * (-f + 2) : mu * f; };
      const double na = a.nbound[ia], nb = a.nbound[ib];
      const double dE = eff(mua, fa) * na + eff(mub, fb) * nb - eff(mub, fa) * na - eff(mua, fb) * nb;
      uint4 o = philox(make_uint4((unsigned)round, (unsigned)(round >> 32), (unsigned)sa, 0x5BE0CD19u),
                       make_uint2((unsigned)seed ^ 0xA4093822u, (unsigned)(seed >> 32)));
      const double u = (double)(o.x >> 1) / kRandMax;
      if (u < exp(-dE)) {
        a.reps[ia].xch_dE += (eff(mua, fa) - eff(mub, fa)) * na;
        a.reps[ib].xch_dE += (eff(mub, fb) - eff(mua, fb)) * nb;
        a.reps[ia].mu[b] = mub;
        a.reps[ib].mu[b] = mua;
        a.rep_of_rung[sa] = ib;
        a.rep_of_rung[sb] = ia;
        a.mu_swaps[sa] += 1;
      }
      a.mu_swap_attempts[sa] += 1;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0 && round_in < 0) a.xround[0] += 1;
}

// ---------------------------------------------------------------- launchers

template <typename Pos>
static void launch_mc_t(const KArgs& a, bool audit, int blocks, cudaStream_t s) {
  const size_t shm = (size_t)a.spec_off_warps + (size_t)a.warp_smem * (audit ? 1 : a.wpb);
  const int threads = audit ? 32 : 32 * a.wpb;
  if (audit) mc_kernel<Pos, true><<<1, threads, shm, s>>>(a);
  else mc_kernel<Pos, false><<<blocks, threads, shm, s>>>(a);
}

template <typename Pos>
static cudaError_t set_smem_t(int bytes) {
  cudaError_t e = cudaFuncSetAttribute(mc_kernel<Pos, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(mc_kernel<Pos, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

}  // namespace cg

void cg_launch_mc(const cg::KArgs& a, bool fp64, bool audit, cudaStream_t s) {
  const int blocks = (a.n_reps + a.wpb - 1) / a.wpb;
  if (fp64) cg::launch_mc_t<double>(a, audit, blocks, s);
  else cg::launch_mc_t<float>(a, audit, blocks, s);
}

// Raised only (the attribute is shared by every simulation in the process;
// see cg_set_spec_smem).
cudaError_t cg_set_mc_smem(bool fp64, int bytes) {
  static std::mutex mu;
  static int cur[64][2];
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lock(mu);
  int* c = dev >= 0 && dev < 64 ? &cur[dev][fp64 ? 1 : 0] : nullptr;
  if (c && bytes <= *c) return cudaSuccess;
  e = fp64 ? cg::set_smem_t<double>(bytes) : cg::set_smem_t<float>(bytes);
  if (e == cudaSuccess && c) *c = bytes;
  return e;
}

void cg_launch_deposit(const cg::KArgs& a, bool fp64, int rep, int n_reps_launch, long long max_beads,
                       cudaStream_t s) {
  dim3 grid((unsigned)((max_beads + 255) / 256 < 1024 ? (max_beads + 255) / 256 : 1024),
            rep >= 0 ? 1 : (unsigned)n_reps_launch);
  if (grid.x == 0) grid.x = 1;
  if (fp64) cg::deposit_kernel<double><<<grid, 256, 0, s>>>(a, rep);
  else cg::deposit_kernel<float><<<grid, 256, 0, s>>>(a, rep);
}

void cg_launch_energy(const cg::KArgs& a, bool fp64, double* out, cudaStream_t s) {
  if (fp64) cg::energy_kernel<double><<<a.n_reps, 256, 0, s>>>(a, out);
  else cg::energy_kernel<float><<<a.n_reps, 256, 0, s>>>(a, out);
}

void cg_launch_chi_sum(const cg::KArgs& a, double* out, cudaStream_t s) {
  cg::chi_sum_kernel<<<a.n_reps, 256, 0, s>>>(a, out);
}

void cg_launch_exchange(const cg::KArgs& a, const double* eout, int n_rungs, long long round,
                        unsigned long long seed, cudaStream_t s) {
  cg::exchange_kernel<<<1, 256, 0, s>>>(a, eout, n_rungs, round, seed);
}
