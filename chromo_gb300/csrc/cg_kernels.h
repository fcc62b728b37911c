// cg_kernels.h -- arguments shared by the host C ABI and the kernels.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <string>

#include "cg_device.cuh"

namespace cg {

// Records msg as the calling thread's cg_last_error() and returns code.
int record_error(int code, const std::string& msg);

// Per-warp header at the start of the warp's shared-memory region.
struct WarpShared {
  RepDev rd;
  cg_move_ctl ctl[5];
  unsigned long long tally[30];
  GridF gf;
  // FP32 copies of the field constants (uniform accessible volume)
  float f_pref[CG_MAX_BINDERS], f_xpref[CG_MAX_BINDERS * CG_MAX_BINDERS];
  float f_scale;  // 2^-40 / vol_bin
  float f_vb;     // bead volume
  float f_k;      // chi * vol_bin / bead volume
  float f_lim;    // vf_limit
  // FP32 copies of the binding constants: free energy table, effective
  // chemical potential (mu (2 - f) for mu > 0, else mu f), intranucleosome term
  float f_bind[CG_MAX_BINDERS * (CG_MAX_MARK + 1) * (CG_MAX_MARK + 1)];
  float f_me[CG_MAX_BINDERS], f_intra[CG_MAX_BINDERS];
  int nused;
  int pad[3];
};

constexpr int kMaxW = 12;  // warps per replica CTA (12 x 32 threads x 168 registers fill one SM)
constexpr int kMaxS = 32;  // moves in flight per replica (one bit each in 32-bit masks)

// Outcome of one speculatively evaluated move.
struct MovePlan {
  int kind, m, ind0, indf;
  int empty, err, regfail, dec;
  unsigned cmask;
  int nvox, gtab, gstage, bsel, ndraw;
  double dE;
  double dEp;  // polymer part of dE (written only when the move log is on)
  // block-wide deposit of a position move (its beads' corners spread over
  // every thread of the CTA): the proposal's transform and table kind in,
  // the two boundary bond terms, the confinement counts and the error bits out
  int blk, sure, oob;
  unsigned derr;
  long long pq[2];
  double ph[2];
  double M[12];  // the 3 x 4 transform, stored in the position type
  // the CTA's pass over the pooled voxel table (FP32 position moves): the
  // move's field dE in fixed point, its FP64 side sum, its exact 1e99 units,
  // its touched voxels and a failed registration
  long long fq, fH;
  double fh;
  int fn, freg;
};

// Shared-memory header of one replica's CTA.
constexpr int kDrawCache = 64;  // first draws of each in-flight move, precomputed by its lanes

struct SpecShared {
  WarpShared ws;
  MovePlan plan[kMaxS];
  int nused[kMaxS];
  unsigned long long t0;   // move counter (selects each move's random sub-stream)
  unsigned long long tlog; // move counter at launch (index origin of the move log)
  double run_dE;
  int cut, stop;
  unsigned accmask;
  int npool;  // entries of the pooled voxel table in use
};

static_assert(sizeof(unsigned) * kDrawCache % 16 == 0, "the draw buffers are written with 16-byte stores");

struct KArgs {
  RepDev* reps;
  cg_move_ctl* ctl;
  int n_ctl, n_reps;
  unsigned long long* tally;  // [n_reps * 30]
  void* r4;                   // V4<Pos> per bead (all replicas concatenated)
  void* t34;
  void* t24;
  unsigned* states;           // packed int8 binding states per bead
  unsigned* marks;            // packed int8 chemical_mods per bead
  const double* bonds;        // 6 doubles per bead (bond i -> i+1)
  const float* bonds32;       // the same in FP32, 8 floats per bead (16-byte aligned rows)
  const double* twist;        // per bead: eps_twist, omega0 of bond i -> i+1 (null: no SSTWLC replica)
  long long* grid;            // ncol int64 per voxel
  const double* access_vol;   // per voxel, or null
  const float* access_sc;     // per voxel: (float)(2^-40 / V), with access_vol
  const double* access_vb;    // per voxel: V / bead volume, with access_vol
  int ncol;   // grid columns per voxel (2 or 4: rows padded to 16 or 32 bytes)
  int hcol;   // columns of a voxel-hash entry (n_binders + 1)
  // per-replica global scratch for moves too large for shared memory
  int* g_keys;
  int* g_used;
  int* g_bslot;
  long long* g_vals;
  int g_logH;
  void* g_stage;
  int* g_idx;
  long long g_stage_cap;
  unsigned* picked;           // tangent-rotation bitmaps
  const long long* picked_off;
  // launch shape and shared-memory layout (bytes within one move slot's
  // region; the audit kernel uses the first region for its single move)
  long long n_steps;
  int wpb, logH;
  long long stage_cap;
  int warp_smem, off_draws, off_keys, off_used, off_bslot, off_vals, off_stage, off_idx;
  // CTA layout: header, block voxel table, then one region per move slot;
  // spec_w warps of 32 / spec_g groups, spec_s = spec_w * 32 / spec_g slots
  int spec_w, spec_g, spec_s, spec_logHB, spec_off_bkeys, spec_off_bmask, spec_off_warps;
  // pooled voxel table of the CTA (FP32 storage): 2^pool_logH entries keyed by
  // voxel * 32 + move slot, shared by the position moves of a batch
  int pool_on, pool_logH, off_pkeys, off_pused, off_pvals;
  unsigned long long seed;
  // the MC kernel's lean form: no replica uses SSTWLC twist and the move log
  // is off
  int lean;
  // audit mode
  int audit_rep;
  const unsigned* a_draws;
  long long a_n_draws;
  const signed char* a_bstates;
  long long a_n_bstates;
  cg_move_record* a_recs;
  long long a_max_recs;
  long long* a_out;
  // production kernel's move log (null: off): records [n_reps x mlog_cap],
  // move k of the launch (k < mlog_cap) of replica r at r * mlog_cap + k
  cg_move_record* mlog;
  long long mlog_cap;
  // replica exchange
  int* rep_of_rung;            // parameter slot -> replica holding that slot's (chi, mu)
  unsigned long long* swaps;
  unsigned long long* swap_attempts;
  unsigned long long* xround;  // exchange rounds performed (graph replays)
  // mu ladder: mu_rungs > 1 arranges slots as [grid][mu rung][chi rung] and
  // also swaps mu of binder mu_binder between neighbouring mu rungs
  int mu_rungs, mu_binder;
  double* nbound;              // per replica: bound sites of binder mu_binder
  unsigned long long* mu_swaps;
  unsigned long long* mu_swap_attempts;
};

// Drift guard of the batched rounds (cg_guard.cu): every `every`-th round the
// full FP64 energies are recomputed in chunks x replicas blocks and checked
// against the running sums.
struct GuardArgs {
  int every, chunks;
  double tol_abs, tol_rel;
  double* partial;                // [n_reps x chunks x 6]
  double *e_ref, *run_ref, *drift;  // [n_reps]
  int* init;                      // [n_reps]: a reference energy is held
  unsigned long long* counter;    // [0] rounds seen, [1] checks made
};

}  // namespace cg

void cg_launch_guard(const cg::KArgs& a, const cg::GuardArgs& g, bool fp64, cudaStream_t s);
void cg_launch_steric(const cg::KArgs& a, bool fp64, int rep, long long n_rows, long long ind0, long long indf,
                      const double* trial, double e, double V0, double* rows, double* out, cudaStream_t s);
void cg_launch_mc(const cg::KArgs& a, bool fp64, bool audit, cudaStream_t s);
void cg_launch_spec(const cg::KArgs& a, bool fp64, size_t smem_bytes, cudaStream_t s);
cudaError_t cg_set_spec_smem(bool fp64, int lanes_per_move, int bytes);
// whether an MC kernel is built for (storage, lanes per move)
bool cg_spec_shape_ok(bool fp64, int lanes_per_move);
cudaError_t cg_set_mc_smem(bool fp64, int bytes);
void cg_launch_deposit(const cg::KArgs& a, bool fp64, int rep, int n_reps_launch, long long max_beads,
                       cudaStream_t s);
void cg_launch_energy(const cg::KArgs& a, bool fp64, double* out, cudaStream_t s);
void cg_launch_chi_sum(const cg::KArgs& a, double* out, cudaStream_t s);
// warps of the MC kernel that fit one SM's register file
int cg_spec_warps_per_sm(bool fp64, int lanes_per_move);

namespace cg {
constexpr int kTerms = 14;                                // energy terms per replica (cg_grad.cu)
constexpr int kAccPerRep = kTerms + kTerms * kTerms + 1;  // running sums of T, T T^T, count
}
void cg_launch_gradient(const cg::KArgs& a, bool fp64, float* out, long long max_beads, cudaStream_t s);
void cg_launch_gradient64(const cg::KArgs& a, bool fp64, double* out, double* out_t3, long long max_beads,
                          cudaStream_t s);
void cg_launch_host_load(const cg::KArgs& a, bool fp64, const void* tab, int R, long long max_beads, int nb,
                         unsigned* flag, int mode, cudaStream_t s);
void cg_launch_host_store(const cg::KArgs& a, bool fp64, const void* tab, int R, long long max_beads, int nb,
                          cudaStream_t s);
void cg_launch_stage_commit(const cg::KArgs& a, bool fp64, const void* tab, int R, long long max_beads,
                            const void* s_r, const void* s_t3, const void* s_t2, const unsigned* s_st,
                            cudaStream_t s);
void cg_launch_store_chains(const cg::KArgs& a, bool fp64, long long total, const double* r, const double* t3,
                            cudaStream_t s);
void cg_launch_terms(const cg::KArgs& a, double* terms, double* acc, cudaStream_t s);
void cg_launch_exchange(const cg::KArgs& a, const double* eout, int n_rungs, long long round,
                        unsigned long long seed, cudaStream_t s);
