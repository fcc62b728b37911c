/*
 * chromo_gb300.h -- C ABI of the GB300 Monte Carlo inner loop for chromo.
 *
 * One handle (cg_sim) holds R replicas resident in GPU memory.  A replica is
 * one polymer (SSWLC / Chromatin chain) in its own UniformDensityField (or a
 * NullField, or no field), with its five move controllers.  Everything is
 * plain pointers and sizes; host buffers are copied inside each call.
 *
 * Each entry point names the reference interface it replaces (paths inside
 * the chromo repository).  Return value: 0 on success, a negative cg_status
 * otherwise; cg_last_error() gives the message of the last failure on the
 * calling thread.
 */
#ifndef CHROMO_GB300_H
#define CHROMO_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CG_MAX_BINDERS 3
#define CG_MAX_MARK 3  /* marks (chemical_mods) and sites per bead in 0..3 */

typedef struct cg_sim cg_sim;

typedef enum {
    CG_OK = 0,
    CG_ERR_ARG = -1,          /* invalid argument (ValueError / TypeError in the reference) */
    CG_ERR_CUDA = -2,         /* CUDA runtime failure */
    CG_ERR_WINDOW = -3,       /* bead window larger than the chain (ValueError raised by
                                 chromo/util/bead_selection.pyx:86-89,138-141) */
    CG_ERR_STREAM = -4,       /* a supplied random stream ran out (audit mode) */
    CG_ERR_NONFINITE = -5,    /* NaN / Inf position produced by a move */
    CG_ERR_SPIN = -6,         /* an iteration cap was hit (bead-selection resampling,
                                 tangent-index redraws, hash probing) */
    CG_ERR_NOMEM = -7,
    CG_ERR_DRIFT = -8         /* the drift guard found the recomputed energy off the running
                                 sum of dE (cg_set_drift_guard) */
} cg_status;

/* Move kinds, in the order of chromo/mc/mc_controller.py:255-258. */
enum { CG_CRANK_SHAFT = 0, CG_END_PIVOT = 1, CG_SLIDE = 2, CG_TANGENT_ROTATION = 3,
       CG_CHANGE_BINDING_STATE = 4 };

/* State of one MC move and its controller: MCAdapter (chromo/mc/moves.pxd:14-25),
 * SimpleControl / NoControl (chromo/mc/mc_controller.py:74-189) and the EWMA
 * AcceptanceTracker (chromo/util/mc_stat.py:190-208). */
typedef struct {
    int64_t move_kind;     /* CG_* above */
    int64_t ctrl_kind;     /* 0: NoControl, 1: SimpleControl */
    int64_t num_per_cycle;
    int64_t move_on;
    double amp_move;
    int64_t amp_bead;
    double bead_lo, bead_hi, move_lo, move_hi;  /* controller bounds */
    double acc_rate;       /* EWMA acceptance rate */
    double alpha;          /* 2 / (moves_in_average + 1) */
    int64_t num_attempt, num_success;
} cg_move_ctl;

/* One attempted move in audit mode. accepted = -1 marks an empty move
 * (no beads selected), which returns before the energy evaluation
 * (chromo/mc/mc_sim.pyx:148-151). */
typedef struct {
    int32_t kind, n_inds, ind0, indf;
    double dE_poly, dE_field;
    int32_t accepted, n_draws;
} cg_move_record;

/* UniformDensityField / NullField description (chromo/fields.pyx:453-535,
 * 687-712; prefactors precomputed as there). */
typedef struct {
    int32_t field_kind;    /* 0: polymer in no field, 1: NullField, 2: UniformDensityField */
    int32_t confine_kind;  /* 0: none (periodic box), 1: "Spherical", 2: "Cubical" */
    double confine_length;
    int32_t nx, ny, nz, n_binders;
    double x_width, y_width, z_width;
    double chi, vf_limit, bead_vol;
    double pref[CG_MAX_BINDERS];    /* field_energy_prefactor */
    double intra[CG_MAX_BINDERS];   /* interaction_energy_intranucleosome */
    double xpref[CG_MAX_BINDERS * CG_MAX_BINDERS]; /* cross_talk_field_energy_prefactor[b][c] */
    int32_t fast_field;    /* 1: per-move density changes from sub-bin weights (init_fast_field,
                              chromo/fields.pyx:577-671, 1235-1368); full deposits stay exact */
    int32_t n_points;      /* sub-bins per voxel and axis when fast_field (rounded up to even) */
} cg_field_params;

/* Binding energetics of the polymer's beads (chromo/polymers.pyx:1408-1538). */
typedef struct {
    int32_t n_binders, max_binders;   /* max_binders = -1: no cap */
    int32_t sites[CG_MAX_BINDERS];    /* sites_per_bead */
    int32_t pad;
    double mu[CG_MAX_BINDERS];        /* chemical_potential */
    double mu_adjust_factor;
    /* bind_f[(b*(CG_MAX_MARK+1) + n_marked)*(CG_MAX_MARK+1) + n_bound] =
       -ln(single-site binding partition function) */
    double bind_f[CG_MAX_BINDERS * (CG_MAX_MARK + 1) * (CG_MAX_MARK + 1)];
} cg_binding_params;

typedef struct {
    int32_t n_replicas;
    int32_t pos_fp64;          /* 1: positions stored in FP64, 0: in FP32 */
    int32_t n_binders;         /* 1..CG_MAX_BINDERS (same for every replica) */
    int32_t warps_per_block;   /* 0: chosen by the library */
    const int64_t *n_beads;    /* [n_replicas] */
    const int32_t *grid_dims;  /* [n_replicas * 3] voxels in x, y, z (1,1,1 without a field) */
    int64_t max_segment;       /* largest bead amplitude of a segment move + 1 */
    int64_t max_tangent;       /* largest bead amplitude of tangent_rotation */
    int32_t nonuniform_access; /* 1: per-voxel accessible volumes are uploaded */
    int32_t lanes_per_move;    /* lanes evaluating one move: 8, 16 or 32 (FP64 storage: 32);
                                  0: chosen by the library */
} cg_config;

/* Allocate device state for R replicas.  Replaces constructing the reference's
 * PolymerBase / UniformDensityField objects (chromo/polymers.pyx:164-258,
 * chromo/fields.pyx:453-535) for the GPU. */
int cg_create(const cg_config *cfg, cg_sim **out);
void cg_destroy(cg_sim *sim);
const char *cg_last_error(void);

/* Upload one chain: r, t3, t2 [N*3], states and chemical_mods [N*n_binders],
 * bond parameters [(N-1)*5] = eps_bend, gamma, eps_par, eps_perp, eta per bond
 * (SSWLC._find_parameters, chromo/polymers.pyx:1545-1601). */
int cg_set_chain(cg_sim *sim, int32_t rep, const double *r, const double *t3, const double *t2,
                 const int64_t *states, const int64_t *marks, const double *bonds);
int cg_get_chain(cg_sim *sim, int32_t rep, double *r, double *t3, double *t2, int64_t *states);

/* cg_set_chain / cg_get_chain for every replica in one call: r[rep], t3[rep],
 * t2[rep] point to replica rep's [N_rep*3] arrays and states[rep] to its
 * [N_rep*n_binders] array (a NULL array list, or a NULL entry, skips that
 * array or replica).  Where the GPU can address pageable host memory
 * (cudaDevAttrPageableMemoryAccess: Grace-Blackwell NVLink-C2C) one kernel
 * reads or writes the caller's arrays directly (an upload is read once into
 * device staging arrays, checked, and copied into the resident state only if
 * it passed, so a rejected one changes nothing); elsewhere, or with the
 * environment variable CHROMO_GB300_STAGED_HOST_IO=1 at cg_create, the
 * host-side conversion runs on several threads into a pinned buffer and each
 * array crosses the bus in one copy.  This is how a batch of chains is moved
 * between the reference's per-polymer numpy arrays and the device. */
int cg_set_chains(cg_sim *sim, const double *const *r, const double *const *t3,
                  const double *const *t2, const int64_t *const *states);
int cg_get_chains(cg_sim *sim, double *const *r, double *const *t3, double *const *t2,
                  int64_t *const *states);
/* *direct = 1 when cg_set_chains / cg_get_chains access the host arrays from
 * the GPU, 0 when they stage through pinned memory (no counterpart in the
 * reference, which has no device). */
int cg_get_transfer_mode(cg_sim *sim, int32_t *direct);

/* SSTWLC twist for replica rep (chromo/polymers.pyx:1889-2320): per bond
 * i -> i+1 (N - 1 each) the twist modulus eps_twist = lt / bead_length and the
 * natural twist omega0 = bead_length * (2 pi / 10.5) / 0.332.  The bond
 * energy gains 0.5 eps_twist dw^2, dw = omega - omega0 wrapped into
 * [-pi, pi), omega the twist angle of the two beads' (t2, t3) frames
 * (compute_twist_angle_omega, :3427-3461), in every move's dE and in the
 * energies; FP64 arithmetic for both storage types.  eps_twist = NULL turns
 * it off.  cg_gradient_device refuses dE/dt3 while a replica has twist. */
int cg_set_twist(cg_sim *sim, int32_t rep, const double *eps_twist, const double *omega0);

/* Steric clashes of the detailed chromatin model (DetailedChromatinWithSterics,
 * chromo/polymers.pyx:2738-2938): every pair of beads of replica rep closer
 * than excluded_distance costs V0 ((e/d)^12 - 2 (e/d)^6 + 1).
 * cg_steric_energy: the clash energy of the resident chain
 * (eval_E_steric_clashes, :2900-2920).  cg_steric_delta: its change when
 * beads [ind0, indf) move to r_trial ((indf - ind0) x 3, host FP64)
 * (get_delta_distances + eval_delta_steric_clashes, :2827-2898), an O(m N)
 * pass over the chain.  Both blocking, deterministic (rows added in order). */
int cg_steric_energy(cg_sim *sim, int32_t rep, double excluded_distance, double V0, double *out);
int cg_steric_delta(cg_sim *sim, int32_t rep, int64_t ind0, int64_t indf, const double *r_trial,
                    double excluded_distance, double V0, double *out);

/* Field of one replica; access_vol [G] or NULL when every voxel is fully
 * accessible (get_accessible_volumes, chromo/fields.pyx:714-768). */
int cg_set_field(cg_sim *sim, int32_t rep, const cg_field_params *field, const double *access_vol);
int cg_set_binding(cg_sim *sim, int32_t rep, const cg_binding_params *bind);

/* Controllers of one replica, in the order they are cycled. */
int cg_set_controllers(cg_sim *sim, int32_t rep, const cg_move_ctl *ctl, int32_t n_ctl);
int cg_get_controllers(cg_sim *sim, int32_t rep, cg_move_ctl *ctl, int32_t n_ctl);

/* Re-deposit every bead into the density grid of one replica (rep = -1: all).
 * Replaces update_all_densities_for_all_polymers (chromo/fields.pyx:2041-2106).
 * The grid is int64 fixed point in units of 2^-40 of trilinear weight, so the
 * result does not depend on the order of the deposits. */
int cg_deposit(cg_sim *sim, int32_t rep);
/* Density grid of one replica as int64 fixed point [G * (n_binders+1)]. */
int cg_get_density(cg_sim *sim, int32_t rep, int64_t *grid);

/* Run mc_sim on every replica (chromo/mc/mc_sim.pyx:26-103): n_steps steps,
 * each cycling the controllers, each controller attempting num_per_cycle moves
 * (mc_step, chromo/mc/mc_sim.pyx:106-182) and then updating its amplitudes.
 * Random numbers come from counter-based Philox4x32-10 streams keyed by
 * (seed, replica).  stream: a cudaStream_t or NULL for the default stream.
 * Returns after the kernel has been enqueued; cg_sync() waits and reports
 * device-side errors. */
int cg_run(cg_sim *sim, int64_t n_steps, uint64_t seed, void *stream);
int cg_sync(cg_sim *sim, void *stream);

/* Audit mode for one replica: the same kernel, but every random number is
 * taken from the supplied arrays -- draws[] in [0, 2^31-1] where the reference
 * calls libc rand(), bstates[] where it calls np.random.randint for a new
 * binding state (chromo/mc/move_funcs.pyx:805-820) -- and every attempted move
 * is recorded.  Synchronous. */
int cg_run_audit(cg_sim *sim, int32_t rep, int64_t n_steps,
                 const uint32_t *draws, int64_t n_draws,
                 const int8_t *bstates, int64_t n_bstates,
                 cg_move_record *records, int64_t max_records, int64_t *n_records,
                 int64_t *draws_used, int64_t *bstates_used);

/* cg_run with a per-move log (blocking): the production kernel, at the sim's
 * launch shape, runs n_steps MC steps of every replica from the state and
 * move counters it holds, as cg_run does, and writes each attempted move's
 * record, in move order, to records[rep * max_records + k] for the first
 * max_records moves of each replica; n_records[rep] (R entries) receives the
 * number of moves the replica attempted.  dE_poly and dE_field are the move's
 * polymer and field dE, n_draws the number of draws it took from its own
 * random sub-stream, accepted = -1 marks an empty move.  This is the device
 * counterpart of the reference's per-move log (MCAdapter.accept / reject with
 * log_move, chromo/mc/moves.pyx:156-300, into AcceptanceTracker.log_move,
 * chromo/util/mc_stat.py:116-145); the parity tests replay the same moves on
 * the CPU from it. */
int cg_run_logged(cg_sim *sim, int64_t n_steps, uint64_t seed, cg_move_record *records,
                  int64_t max_records, int64_t *n_records);

/* FP64 energies of one replica, recomputed from the resident state:
 * out[0] elastic (SSWLC.compute_E, chromo/polymers.pyx:1348-1381),
 * out[1] binding free energy (sum of the single-site terms whose differences
 *        are binding_dE, chromo/polymers.pyx:1383-1538),
 * out[2] field energy in the form whose differences are the per-move field dE
 *        (chromo/fields.pyx:1675-1875),
 * out[3] running sum of accepted dE since the last cg_reset_running_energy,
 *        leaving out the moves whose dE carries a penalty (|dE| >= 1e20: the
 *        1e25 max_binders term, the 1e99 volume-fraction and confinement
 *        terms), which would absorb every later dE in an FP64 sum; such moves
 *        only leave a penalised state, so the running sum's changes equal the
 *        energy's over every interval whose end energies carry no penalty. */
int cg_energy(cg_sim *sim, int32_t rep, double *out);
int cg_reset_running_energy(cg_sim *sim);

/* cg_energy for every replica at once: out [n_replicas x 5] = elastic,
 * binding, field (as cg_energy), running sum of accepted dE, and the chi-free
 * part S = sum_v (V / V_bead) vf^2 of the field energy, over the voxels at or
 * below vf_limit (field = chi * S + terms that do not depend on chi; a voxel
 * above the limit costs 1e99 vf whatever chi is).  Work is enqueued on `stream`; the call
 * returns once out is filled. */
int cg_energies(cg_sim *sim, double *out, void *stream);

/* Derivatives of the energy cg_energy reports (elastic + binding + field in
 * the form whose differences are the move dE); no counterpart in the
 * reference, which has no derivatives.  dEdr [total beads x 3] FP32, replicas
 * concatenated in creation order: dE/dr of every bead (the two bonds at the
 * bead and the bead's eight trilinear weights), or NULL.  terms
 * [n_replicas x 14] FP64, or NULL: [0] S = sum over voxels with vf <= vf_limit
 * of (V/V_bead) vf^2 (= dE/dchi), [1..3] sum_v rho_b^2, [4..6] sum_v rho_0 rho_1,
 * rho_0 rho_2, rho_1 rho_2, [7..9] number of beads with state_b == 2,
 * [10..12] sum_i state_ib, [13] sum_v (bead density)^2; dE/d(mu_b) and
 * dE/d(eps) are linear in them (field_prefactor, intranucleosome and
 * cross-talk prefactors are linear in eps, chromo/fields.pyx:687-712).
 * Synchronous. */
int cg_gradient(cg_sim *sim, float *dEdr, double *terms);
/* Device-resident counterparts for callers whose data already lives on the
 * GPU (a torch.autograd.Function on CUDA tensors; no counterpart in the
 * reference, which has no device).  All arrays are DEVICE pointers with the
 * replicas' beads concatenated in replica order; all work is enqueued on
 * `stream` and nothing is copied to the host.
 * cg_set_chains_device: positions r and/or tangents t3 [total_beads x 3] FP64
 *   (either may be NULL) into the resident chains (rounded to the storage type);
 * cg_deposit_async: cg_deposit of every replica, on `stream`;
 * cg_energies_device: out [n_replicas x 5] as cg_energies;
 * cg_gradient_device: dE/dr and (dEdt3 != NULL) dE/dt3 [total_beads x 3] FP64
 *   of the cg_energy sum; t3 enters only the elastic energy, through the two
 *   bonds at each bead (chromo/polymers.pyx:1348-1381), taken as free vectors. */
int cg_set_chains_device(cg_sim *sim, const double *r, const double *t3, void *stream);
int cg_deposit_async(cg_sim *sim, void *stream);
int cg_energies_device(cg_sim *sim, double *out, void *stream);
int cg_gradient_device(cg_sim *sim, double *dEdr, double *dEdt3, void *stream);
/* Add every replica's 14 terms T and their products T T^T to running sums on
 * the device (enqueued on `stream`), for reweighting: the covariance of any
 * two linear combinations of the terms follows from the sums. */
int cg_sample_terms(cg_sim *sim, void *stream);
/* Running sums [n_replicas x (14 + 196 + 1)]: sum T, sum T T^T (row major),
 * number of samples; reset != 0 zeroes them after reading. */
int cg_get_samples(cg_sim *sim, double *out, int32_t reset);

/* Per-replica, per-move tallies [5 * 6]: attempts, accepts, beads moved,
 * voxels touched, beads moved in accepted moves, voxels touched in accepted
 * moves.  Used for the algorithmic-bytes roofline. */
int cg_get_tally(cg_sim *sim, int32_t rep, uint64_t *out);
int cg_reset_tally(cg_sim *sim);

/* Replica exchange across a chi ladder (no counterpart in the reference,
 * which has a single chain per run): replicas are grouped in ladders of
 * n_rungs consecutive replicas; in round `round` the rungs (2i+p, 2i+1+p),
 * p = round % 2, propose to swap chi with probability
 * min(1, exp((chi_a - chi_b) * (S_a - S_b))), S the chi-free part of the
 * field energy.  chi_of_rep is read and written [n_replicas]. */
int cg_exchange(cg_sim *sim, int32_t n_rungs, int64_t round, uint64_t seed, void *stream);
int cg_get_chi(cg_sim *sim, double *chi);

/* Two-dimensional ladder (no counterpart in the reference): with mu_rungs >= 2
 * the parameter slots form grids of mu_rungs x n_rungs (slot = (grid * mu_rungs
 * + mu rung) * n_rungs + chi rung, replica r starting in slot r), and every
 * exchange round after its chi swaps also proposes, for mu-rung pairs
 * (2i+p, 2i+1+p) at the same chi rung, to swap the chemical potential of
 * binder `binder`, accepted with probability min(1, exp(-dE)), dE the change
 * of sum_r -m(mu_r) N_r (m(mu) = mu (2 - f) for mu > 0, mu f otherwise, f the
 * annealing factor; N_r the replica's bound sites of that binder,
 * chromo/polymers.pyx:1520-1531).  n_rungs = 1 gives a mu-only ladder.
 * mu_rungs = 0 switches it off. */
int cg_set_mu_ladder(cg_sim *sim, int32_t mu_rungs, int32_t binder);
int cg_get_mu(cg_sim *sim, int32_t binder, double *mu);
/* Accepted and attempted swaps per lower slot of each pair [n_replicas] each
 * (any pointer may be NULL). */
int cg_get_swap_counts(cg_sim *sim, uint64_t *chi_swaps, uint64_t *chi_attempts, uint64_t *mu_swaps,
                       uint64_t *mu_attempts);

/* Batched run: n_rounds x (n_steps MC steps on every replica, then one
 * exchange round), captured once in a CUDA graph and replayed.  n_rungs = 0
 * disables exchange. */
int cg_run_batched(cg_sim *sim, int64_t n_rounds, int64_t n_steps, int32_t n_rungs,
                   uint64_t seed, void *stream);

/* Kernel launch shape currently in use, and the number of MC kernels the
 * library launched since creation. */
int cg_get_launch_info(cg_sim *sim, int32_t *warps_per_block, int32_t *hash_slots,
                       int64_t *kernels_launched);

/* Launch shape of the MC kernel: warps per replica CTA, lanes per move, moves
 * in flight per replica (warps * 32 / lanes) and shared voxel-table slots per
 * move.  No counterpart in the reference (its loop runs one move at a time);
 * the autotuner (chromo_gb300.autotune) reads it. */
int cg_get_launch_shape(cg_sim *sim, int32_t *warps_per_block, int32_t *lanes_per_move,
                        int32_t *moves_in_flight, int32_t *hash_slots);

/* On-device drift guard of cg_run_batched (no counterpart in the reference,
 * whose running energy is an exact-order FP64 sum on one CPU core): with
 * every_rounds > 0, every every_rounds-th captured round ends with every
 * replica's full FP64 energy (the cg_energy sum: elastic + binding + field)
 * recomputed from the resident state, and its change since the previous
 * check compared with the change, over the same rounds, of the running sum of
 * accepted dE plus the energy change of the replica's accepted chi / mu swaps.
 * A difference above tol_abs + tol_rel * max(1, |E|), or a non-finite one,
 * makes the next cg_sync return CG_ERR_DRIFT.  The first check takes the
 * reference energies; an interval with a penalised energy (|E| >= 1e20) at
 * either end is not compared, and its end becomes the next reference.  0
 * turns the guard off.  Drift has two sources: FP32
 * rounding of the per-move dE, and the reference's tangent-rotation rule for
 * adjacent beads (chromo/polymers.pyx:1074-1080), whose summed dE is not the
 * energy change; the tolerances must cover both. */
int cg_set_drift_guard(cg_sim *sim, int32_t every_rounds, double tol_abs, double tol_rel);
/* drift[rep] (R entries) = the difference measured at the last check of each
 * replica; *checks = the number of checks made.  Waits for the device. */
int cg_get_drift(cg_sim *sim, double *drift, int64_t *checks);

/* Checkpoint of the whole resident state (no counterpart in the reference,
 * whose resume restarts from a polymer CSV snapshot with fresh random streams,
 * chromo/mc/__init__.py:167-227): chains, binding states, bond parameters,
 * density grids, accessible volumes, controllers, tallies, every replica's
 * parameters (chi, mu), move counter (which selects each move's Philox
 * sub-stream) and running dE, the exchange slot map, round counter and swap
 * counts.  cg_load_state into a sim created with the same layout (checked)
 * continues the run exactly as if it had not stopped, given the same seeds.
 * cg_state_bytes: the image size; cg_save_state / cg_load_state: host buffer
 * of at least that size.  The drift guard takes new reference energies after
 * a load. */
int64_t cg_state_bytes(cg_sim *sim);
int cg_save_state(cg_sim *sim, void *buf, int64_t bytes);
int cg_load_state(cg_sim *sim, const void *buf, int64_t bytes);

/* Per-round timing of cg_run_batched (no counterpart in the reference, which
 * has no device): with capacity > 0 every captured round brackets its MC
 * kernel with two CUDA event-record nodes, pointed before each launch at the
 * next of `capacity` event pairs (a ring), so the kernel's duration is
 * measured on the device inside the replayed graph.  0 turns it off.  Either
 * way the next cg_run_batched captures its graph again. */
int cg_set_round_timing(cg_sim *sim, int32_t capacity);
/* Durations (ms) of the MC kernel of the last min(rounds run, capacity, max)
 * timed rounds, oldest first; *count receives how many.  Waits for them. */
int cg_get_round_times(cg_sim *sim, float *mc_ms, int32_t max, int32_t *count);

/* Warps of the MC kernel for (storage precision, lanes per move) that fit one
 * SM's register file, or -1 for a shape that is not built.  No counterpart in
 * the reference; the autotuner derives its candidate shapes from it. */
int cg_mc_warps_per_sm(int32_t pos_fp64, int32_t lanes_per_move);

/* Field energy of one chain, allocating nothing (no counterpart in the
 * reference).  Deposits the chain into a fixed-point density grid and writes
 * out[0] = the field energy in the form cg_energy reports in its out[2]
 * (chromo/fields.pyx:1939-2316, :1675-1875, re-deposit of :2041-2106) and
 * out[1] = the chi-free sum S = sum_v (V / V_bead) vf^2 over the voxels at or
 * below vf_limit; both are NaN when a position is not finite.  For callers that
 * must not allocate device memory (a server whose device memory belongs to its
 * own pool; code in which a cudaMalloc would stall work in flight).
 *
 * All array arguments are DEVICE pointers: r [n_beads x 3] FP64, states
 * [n_beads x n_binders] int64 in 0..3, access_vol [nx*ny*nz] FP64 or NULL for
 * the uniform voxel volume, out [2] FP64.  field->field_kind must be 2.  The
 * work is enqueued on `stream` (a cudaStream_t, NULL for the default stream);
 * read out after synchronising it.
 *
 * The grid lives in a static device array of 1,048,576 int64 cells (8 MiB):
 * nx*ny*nz*(n_binders+1) above that is rejected with CG_ERR_ARG.  Each call
 * zeroes the cells it uses on `stream` first, so nothing needs to start at
 * zero.  The first call on each device may load the library's device code
 * there (under CUDA's lazy module loading the module, with its 8 MiB array, is
 * created on first use) and looks up the array's address
 * (cudaGetSymbolAddress): make it in the set-up phase, before any stream
 * capture; from the second call on nothing is created.  Device pointers must
 * belong to the current device (or be managed memory).  There is
 * one array per device: calls that overlap in time on one device (different
 * streams or host threads) race on it; calls on one stream are ordered. */
int cg_field_energy_static(const cg_field_params *field, int64_t n_beads, const double *r,
                           const int64_t *states, const double *access_vol, double *out,
                           void *stream);

#ifdef __cplusplus
}
#endif
#endif /* CHROMO_GB300_H */
