/*
 * chromo_oracle.c -- CPU restatement of chromo's Monte Carlo inner loop.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the GPU path: it is
 * imported by tests/, by __graft_entry__.smoke() and by bench.py's CPU
 * baseline leg, never by the product package.
 *
 * It restates, function by function, the reference's hot path:
 *   mc_sim / mc_step                 chromo/mc/mc_sim.pyx:26-182
 *   MCAdapter accept / reject        chromo/mc/moves.pyx:137-286
 *   SimpleControl + EWMA tracker     chromo/mc/mc_controller.py:97-189,
 *                                    chromo/util/mc_stat.py:190-208
 *   five move proposals              chromo/mc/move_funcs.pyx:39-820
 *   bead selection                   chromo/util/bead_selection.pyx:19-192
 *   rotation / translation matrices  chromo/util/linalg.pyx:23-199
 *   SSWLC elastic + binding dE       chromo/polymers.pyx:1024-1538
 *   UniformDensityField dE / commit  chromo/fields.pyx:121-202,1149-1975
 *   full energies                    chromo/polymers.pyx:1348-1381,
 *                                    chromo/fields.pyx:1939-2316
 *
 * Randomness is an explicit input: the reference draws from libc rand()
 * (values in [0, RAND_MAX], RAND_MAX = 2^31-1) and from numpy's
 * np.random.randint for new binding states.  Here both are arrays that the
 * caller supplies ("draws" and "bstates"), consumed in the reference's order,
 * so the same arrays drive this oracle, the real reference (through srand())
 * and the GPU kernel's audit mode.
 *
 * Build twice: -DOR_POS=double (positions stored in FP64, the reference's
 * storage) and -DOR_POS=float (positions stored in FP32, the GPU storage).
 * Arithmetic is FP64 in both; trial positions are rounded to OR_POS before
 * any energy is evaluated, which is exactly what the GPU does.  Compile with
 * -ffp-contract=off so every operation is individually rounded.
 *
 * Density has two modes:
 *   fixed_density = 0: FP64 density with the reference's incremental update
 *                      and 1e-18 clamps (chromo/fields.pyx:1497-1520,
 *                      1740-1750, 2033-2039) -- for checking against the
 *                      reference itself;
 *   fixed_density = 1: int64 fixed point (2^-40 units of trilinear weight),
 *                      the GPU's storage; per-voxel dE uses the GPU formula.
 */
#include <math.h>
#include <stdint.h>

/* Deterministic binary32 sin / cos / acos shared with the GPU's FP32-storage
 * path (same source, so the emulation below is bit-identical to it). */
#include "../chromo_gb300/csrc/cg_math32.h"
#include <stdlib.h>
#include <string.h>

#ifndef OR_POS
#define OR_POS double
#endif

#define OR_RAND_MAX 2147483647.0
#define OR_E_HUGE_POLY 1e25 /* chromo/polymers.pyx:35 */
#define OR_E_HUGE_FIELD 1e99 /* chromo/fields.pyx:32 */
#define OR_FX_SCALE 1099511627776.0 /* 2^40 */
/* fixed_density = 1 (the GPU's formula): the 1e99 penalties are summed exactly
 * in integer units of OR_HUGE_UNIT = 1e99 * 2^-40 -- a voxel above vf_limit
 * holding n fixed-point units costs llrint(n * Vb / V) units (1e99 vf rounded
 * once), a bead outside the confinement 2^40 units -- so a move's penalty does
 * not depend on the order of its voxels. */
#define OR_HUGE_UNIT (OR_E_HUGE_FIELD / OR_FX_SCALE)
#define OR_MAXB 8

enum { MV_CRANK = 0, MV_END_PIVOT = 1, MV_SLIDE = 2, MV_TANGENT = 3, MV_BINDING = 4 };
enum {
    OR_OK = 0,
    OR_ERR_DRAWS = -1,     /* draw stream exhausted */
    OR_ERR_BSTATES = -2,   /* binding-state stream exhausted */
    OR_ERR_WINDOW = -3,    /* bead window larger than chain (ValueError in reference) */
    OR_ERR_ALLOC = -4,
    OR_ERR_ARGS = -5
};

typedef struct {
    int64_t n_beads, n_binders;
    OR_POS *r, *t3, *t2;        /* N x 3, row major */
    int64_t *states;            /* N x nb */
    const int64_t *marks;       /* N x nb (chemical_mods) */
    const double *eps_bend, *gamma, *eps_par, *eps_perp, *eta; /* N-1 each */
    /* binding: f[(b*(mark_max+1) + Nm)*(site_max+1) + s] = -ln(site partition fn) */
    const double *bind_f;
    int64_t mark_max, site_max;
    const int64_t *sites;       /* nb */
    const double *mu;           /* nb chemical potentials */
    double mu_adjust_factor;
    int64_t max_binders;
    /* field */
    int64_t field_kind;         /* 0: polymer not in a field, 1: NullField, 2: UniformDensityField */
    int64_t confine_kind;       /* 0: none (periodic), 1: Spherical, 2: Cubical */
    double confine_length;
    int64_t nx, ny, nz;
    double x_width, y_width, z_width;
    const double *access_vol;   /* G or NULL (every voxel fully accessible) */
    double vol_bin, chi, vf_limit, bead_vol;
    const double *pref;         /* nb   field_energy_prefactor */
    const double *intra;        /* nb   interaction_energy_intranucleosome */
    const double *xpref;        /* nb*nb cross_talk_field_energy_prefactor */
    int64_t fixed_density;
    double *density;            /* G x (nb+1), fixed_density == 0 */
    int64_t *density_fx;        /* G x (nb+1), fixed_density == 1 */
    /* per-move scratch (allocated by or_scratch_init) */
    double *density_trial;      /* G x (nb+1) */
    int64_t *dfx;               /* G x (nb+1) */
    int64_t *slot_of;           /* G, -1 when untouched */
    int64_t *found;             /* list of touched voxels, insertion order */
    int64_t n_found, found_cap;
    int64_t *inds;              /* N */
    double *trial;              /* N x 9 : r, t3, t2 of the moved beads (as OR_POS, widened) */
    int64_t *new_states;        /* N */
    unsigned char *picked;      /* N */
    int64_t fast_n;             /* fast_field: sub-bins per voxel and axis (0: exact weights) */
    /* SSTWLC twist (NULL: SSWLC): eps_twist = lt / bead_length and the natural
     * twist omega0 = bead_length * (2 pi / 10.5) / 0.332 per bond */
    const double *eps_twist, *omega0;
} or_system;

typedef struct {
    int64_t move_kind, ctrl_kind, num_per_cycle, move_on;
    double amp_move;
    int64_t amp_bead;
    double bead_lo, bead_hi, move_lo, move_hi;
    double acc_rate, alpha;
    int64_t num_attempt, num_success;
} or_ctl;

typedef struct {
    int32_t kind, n_inds, ind0, indf;
    double dE_poly, dE_field;
    int32_t accepted, n_draws;
} or_record;

typedef struct {
    const uint32_t *a;
    int64_t n, pos;
    const int64_t *b;
    int64_t nb_, bpos;
    int err;
    /* Philox mode (philox != 0): the GPU production kernel's random numbers.
     * Every attempted move t has its own sub-streams: draw j is word j & 3 of
     * Philox4x32-10 at counter (j >> 2, t_lo, t_hi, 0x2545F491) under `key`,
     * shifted right by one (31 bits, the role of rand()); binding state k is
     * umulhi(word k & 3 at counter (k >> 2, t_lo, t_hi, 0x7F4A7C15) under
     * `keyb`, sites + 1).  pos / bpos restart at 0 for every move. */
    int philox;
    uint32_t key[2], keyb[2];
    uint64_t t;
    int64_t ties;   /* decisions taken from the followed run in the tie band */
} or_rng;

/* ---------------- random stream ---------------------------------------- */

/* Philox4x32-10 (Salmon, Moraes, Dror and Shaw, SC'11): ten rounds of two
 * 32 x 32 -> 64-bit multiplies with the published multipliers and Weyl key
 * increments. */
static void or_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3], k0 = key[0], k1 = key[1];
    for (int i = 0; i < 10; i++) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0, n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        c1 = (uint32_t)p1;
        c3 = (uint32_t)p0;
        c0 = n0;
        c2 = n2;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

static uint32_t philox_word(const or_rng *g, const uint32_t key[2], uint32_t tag, uint64_t j)
{
    uint32_t ctr[4] = {(uint32_t)(j >> 2), (uint32_t)g->t, (uint32_t)(g->t >> 32), tag}, out[4];
    or_philox(ctr, key, out);
    return out[j & 3];
}

/* draws == NULL: take libc rand() itself, as the reference does (timing runs) */
static int64_t rnd(or_rng *g)
{
    if (g->philox) return (int64_t)(philox_word(g, g->key, 0x2545F491u, (uint64_t)g->pos++) >> 1);
    if (!g->a) { g->pos++; return (int64_t)rand(); }
    if (g->pos >= g->n) { g->err = OR_ERR_DRAWS; return 0; }
    return (int64_t)g->a[g->pos++];
}

static double rndu(or_rng *g) { return (double)rnd(g) / OR_RAND_MAX; }

static int64_t rnd_state(or_rng *g, int64_t n_tails)
{
    if (g->philox) {
        uint32_t w = philox_word(g, g->keyb, 0x7F4A7C15u, (uint64_t)g->bpos++);
        return (int64_t)(((uint64_t)w * (uint64_t)(n_tails + 1)) >> 32);
    }
    if (!g->b) { g->bpos++; return (int64_t)(rand() % (int)(n_tails + 1)); }
    if (g->bpos >= g->nb_) { g->err = OR_ERR_BSTATES; return 0; }
    return g->b[g->bpos++];
}

/* ---------------- bead selection: chromo/util/bead_selection.pyx ---------- */

/* capped_exponential, bead_selection.pyx:19-66 */
static int64_t capped_exponential(or_rng *g, int64_t window, int64_t cap)
{
    int64_t r = (int64_t)(-log10(rndu(g) + 0.00001) * (double)window * 0.45 + 1.0001);
    while (r > cap && !g->err)
        r = (int64_t)(-log10(rndu(g) + 0.00001) * (double)window * 0.45 + 1.0001);
    return r;
}

/* from_left, bead_selection.pyx:69-90 */
static int64_t from_left(or_rng *g, int64_t window, int64_t n_beads)
{
    if (window > n_beads) { g->err = OR_ERR_WINDOW; return 0; }
    return capped_exponential(g, window, window);
}

/* from_right, bead_selection.pyx:93-112 */
static int64_t from_right(or_rng *g, int64_t window, int64_t n_beads)
{
    return n_beads - from_left(g, window, n_beads);
}

/* from_point, bead_selection.pyx:115-154 */
static int64_t from_point(or_rng *g, int64_t window, int64_t n_beads, int64_t ind0)
{
    if (window > n_beads) { g->err = OR_ERR_WINDOW; return 0; }
    if (window < 1) return ind0;
    int64_t side = rnd(g) % 2;
    if (side == 0) {
        int64_t ws = window < ind0 ? window : ind0;
        if (ws < 1) ws = 1;
        int64_t ub = ind0 > 1 ? ind0 : 1;
        return from_right(g, ws, ub);
    } else {
        int64_t rem = n_beads - ind0;
        int64_t ws = window < rem ? window : rem;
        if (ws < 1) ws = 1;
        int64_t ub = rem > 1 ? rem : 1;
        return from_left(g, ws, ub) + ind0;
    }
}

/* check_bead_bounds, bead_selection.pyx:157-192 */
static void check_bead_bounds(int64_t b0, int64_t b1, int64_t n, int64_t *i0, int64_t *i1)
{
    if (b0 > n) b0 = n;
    if (b0 < 0) b0 = 0;
    if (b1 > n) { *i0 = b0; *i1 = n; }
    else if (b1 < 0) { *i0 = 0; *i1 = b0 + 1; }
    else if (b0 == b1) { *i0 = b0; *i1 = b0 + 1; }
    else { *i0 = b0 < b1 ? b0 : b1; *i1 = b0 > b1 ? b0 : b1; }
}

/* Squares.  Cython compiles the reference's "x**2" to pow(x, 2.0), and glibc's
 * pow(x, 2.0) differs from x*x by one ulp for ~0.1% of inputs; the
 * reference-semantics mode (refpow = 1) uses pow so that it reproduces the
 * reference bit for bit, the GPU-emulation mode uses x*x like the kernel. */
static inline double sq(double x, int refpow) { return refpow ? pow(x, 2.0) : x * x; }

/* ---------------- linear algebra: chromo/util/linalg.pyx ---------------- */

/* uniform_sample_unit_sphere(_inplace), linalg.pyx:23-59 */
static void sphere(or_rng *g, double v[3])
{
    double phi = rndu(g) * (2.0 * M_PI);
    double theta = acos(rndu(g) * 2 - 1);
    v[0] = cos(phi) * sin(theta);
    v[1] = sin(phi) * sin(theta);
    v[2] = cos(theta);
}

/* arbitrary_axis_rotation, linalg.pyx:62-143: M = [R | T] about axis a through p */
static void axis_rotation(const double a[3], const double p[3], double ang, double M[3][4],
                          int rp)
{
    double c = cos(ang), s = sin(ang), oc = 1 - c;
    double a0 = sq(a[0], rp), a1 = sq(a[1], rp), a2 = sq(a[2], rp);
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

/* FP32-storage proposal math, as on the GPU */
static void sphere_f32(or_rng *g, double v[3])
{
    unsigned xa = (unsigned)rnd(g), xb = (unsigned)rnd(g);
    float phi = cgm_unif24(xa) * 6.2831855f;
    float theta = cgm_acosf(cgm_unif24(xb) * 2.0f - 1.0f);
    float sp, cp, st, ct;
    cgm_sincosf(phi, &sp, &cp);
    cgm_sincosf(theta, &st, &ct);
    v[0] = (double)(cp * st);
    v[1] = (double)(sp * st);
    v[2] = (double)ct;
}

/* axis rotation in binary32 with the GPU's operation order; the result is
 * returned widened (exactly) to double */
static void axis_rotation_f32(const double ad[3], const double pd[3], float s, float c, double M[3][4])
{
    float a[3] = {(float)ad[0], (float)ad[1], (float)ad[2]};
    float p[3] = {(float)pd[0], (float)pd[1], (float)pd[2]};
    float oc = 1 - c, a0 = a[0] * a[0], a1 = a[1] * a[1], a2 = a[2] * a[2], m[3][4];
    m[0][0] = a0 + (a1 + a2) * c;
    m[0][1] = a[0] * a[1] * oc - a[2] * s;
    m[0][2] = a[0] * a[2] * oc + a[1] * s;
    m[1][0] = a[0] * a[1] * oc + a[2] * s;
    m[1][1] = a1 + (a0 + a2) * c;
    m[1][2] = a[1] * a[2] * oc - a[0] * s;
    m[2][0] = a[0] * a[2] * oc - a[1] * s;
    m[2][1] = a[1] * a[2] * oc + a[0] * s;
    m[2][2] = a2 + (a0 + a1) * c;
    m[0][3] = (p[1] * a[2] - p[2] * a[1]) * s;
    m[1][3] = (p[2] * a[0] - p[0] * a[2]) * s;
    m[2][3] = (p[0] * a[1] - p[1] * a[0]) * s;
    m[0][3] += (p[0] * (1 - a0) - a[0] * (p[1] * a[1] + p[2] * a[2])) * oc;
    m[1][3] += (p[1] * (1 - a1) - a[1] * (p[0] * a[0] + p[2] * a[2])) * oc;
    m[2][3] += (p[2] * (1 - a2) - a[2] * (p[0] * a[0] + p[1] * a[1])) * oc;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 4; j++) M[i][j] = (double)m[i][j];
}

/* ---------------- helpers ------------------------------------------------ */

static inline void ld3(const OR_POS *a, int64_t i, double v[3])
{
    v[0] = (double)a[3 * i]; v[1] = (double)a[3 * i + 1]; v[2] = (double)a[3 * i + 2];
}

static inline double rnd_pos(double x) { return (double)(OR_POS)x; }

/* FP32-storage emulation of the GPU (positions stored as float and a
 * fixed-point grid): the GPU applies the FP64 move matrix rounded to FP32 with
 * FP32 arithmetic and computes trilinear weights in FP32, so this mode does
 * the same to keep the state bit-identical; every energy difference is still
 * evaluated in FP64 here (the recomputation the GPU's dE is checked against). */
#define OR_F32 (sizeof(OR_POS) == 4)
static inline int emu32(const or_system *s) { return OR_F32 && s->fixed_density; }



/* transform_r_t3_t2, move_funcs.pyx:121-154: trial = round_to_storage(M * x) */
static void transform_bead(const or_system *s, int64_t i, double M[3][4], double out[9])
{
    double r[3], t3[3], t2[3];
    ld3(s->r, i, r); ld3(s->t3, i, t3); ld3(s->t2, i, t2);
    if (emu32(s)) {
        float Mf[3][4];
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 4; b++) Mf[a][b] = (float)M[a][b];
        for (int j = 0; j < 3; j++) {
            float er = 0, e3 = 0, e2 = 0;
            for (int k = 0; k < 3; k++) {
                er += Mf[j][k] * (float)r[k];
                e3 += Mf[j][k] * (float)t3[k];
                e2 += Mf[j][k] * (float)t2[k];
            }
            out[j] = (double)(er + Mf[j][3]);
            out[3 + j] = (double)e3;
            out[6 + j] = (double)e2;
        }
        return;
    }
    for (int j = 0; j < 3; j++) {
        double er = 0, e3 = 0, e2 = 0;
        for (int k = 0; k < 3; k++) {
            er += M[j][k] * r[k];
            e3 += M[j][k] * t3[k];
            e2 += M[j][k] * t2[k];
        }
        out[j] = rnd_pos(er + M[j][3]);
        out[3 + j] = rnd_pos(e3);
        out[6 + j] = rnd_pos(e2);
    }
}

/* ---------------- SSWLC elastic energy: chromo/polymers.pyx -------------- */

/* E_pair, polymers.pyx:1148-1175 */
static double e_pair(const or_system *s, const double bend[3], double dr_par,
                     const double dr_perp[3], int64_t b)
{
    return 0.5 * s->eps_bend[b] * (bend[0] * bend[0] + bend[1] * bend[1] + bend[2] * bend[2])
         + 0.5 * s->eps_par[b] * sq(dr_par - s->gamma[b], !s->fixed_density)
         + 0.5 * s->eps_perp[b] * (dr_perp[0] * dr_perp[0] + dr_perp[1] * dr_perp[1]
                                   + dr_perp[2] * dr_perp[2]);
}

/* compute_twist_angle_omega, polymers.pyx:3427-3461: with t1 = t2 x t3,
 * omega = atan2(t2_0 . t1_1 - t1_0 . t2_1, t1_0 . t1_1 + t2_0 . t2_1) */
static double twist_omega(const double t2a[3], const double t3a[3], const double t2b[3], const double t3b[3])
{
    double t1a[3] = {t2a[1] * t3a[2] - t2a[2] * t3a[1], t2a[2] * t3a[0] - t2a[0] * t3a[2],
                     t2a[0] * t3a[1] - t2a[1] * t3a[0]};
    double t1b[3] = {t2b[1] * t3b[2] - t2b[2] * t3b[1], t2b[2] * t3b[0] - t2b[0] * t3b[2],
                     t2b[0] * t3b[1] - t2b[1] * t3b[0]};
    double y = (t2a[0] * t1b[0] + t2a[1] * t1b[1] + t2a[2] * t1b[2])
             - (t1a[0] * t2b[0] + t1a[1] * t2b[1] + t1a[2] * t2b[2]);
    double x = (t1a[0] * t1b[0] + t1a[1] * t1b[1] + t1a[2] * t1b[2])
             + (t2a[0] * t2b[0] + t2a[1] * t2b[1] + t2a[2] * t2b[2]);
    return atan2(y, x);
}

/* E_pair_with_twist, polymers.pyx:2050-2102: the SSWLC bond energy plus
 * 0.5 eps_twist dw^2, dw = omega - omega0 wrapped into [-pi, pi) */
static double e_pair_twist(const or_system *s, const double bend[3], double dr_par, const double dr_perp[3],
                           double omega, int64_t b)
{
    double dw = omega - s->omega0[b];
    dw -= 2 * M_PI * floor((dw + M_PI) / (2 * M_PI));
    return e_pair(s, bend, dr_par, dr_perp, b) + 0.5 * s->eps_twist[b] * sq(dw, !s->fixed_density);
}

/* bead_pair_dE_poly_forward, polymers.pyx:1177-1277 (bead 1 moved); with
 * twist bead_pair_dE_poly_forward_with_twist, :2104-2175 (t2 of both beads) */
static double pair_dE_fwd(const or_system *s, const double r0[3], const double r1[3],
                          const double tr1[3], const double t30[3], const double t31[3],
                          const double tt31[3], int64_t b, const double t20[3], const double t21[3],
                          const double tt21[3])
{
    double drt[3], dr[3], dpt[3], dp[3], bt[3], bc[3];
    for (int i = 0; i < 3; i++) { drt[i] = tr1[i] - r0[i]; dr[i] = r1[i] - r0[i]; }
    double pt = t30[0] * drt[0] + t30[1] * drt[1] + t30[2] * drt[2];
    double pc = t30[0] * dr[0] + t30[1] * dr[1] + t30[2] * dr[2];
    for (int i = 0; i < 3; i++) {
        dpt[i] = drt[i] - t30[i] * pt;
        dp[i] = dr[i] - t30[i] * pc;
        bt[i] = tt31[i] - t30[i] - dpt[i] * s->eta[b];
        bc[i] = t31[i] - t30[i] - dp[i] * s->eta[b];
    }
    if (s->eps_twist)
        return e_pair_twist(s, bt, pt, dpt, twist_omega(t20, t30, tt21, tt31), b)
             - e_pair_twist(s, bc, pc, dp, twist_omega(t20, t30, t21, t31), b);
    return e_pair(s, bt, pt, dpt, b) - e_pair(s, bc, pc, dp, b);
}

/* bead_pair_dE_poly_reverse, polymers.pyx:1279-1346 (bead 0 moved); with
 * twist bead_pair_dE_poly_reverse_with_twist, :2177-2248 */
static double pair_dE_rev(const or_system *s, const double r0[3], const double tr0[3],
                          const double r1[3], const double t30[3], const double tt30[3],
                          const double t31[3], int64_t b, const double t20[3], const double tt20[3],
                          const double t21[3])
{
    double drt[3], dr[3], dpt[3], dp[3], bt[3], bc[3];
    for (int i = 0; i < 3; i++) { drt[i] = r1[i] - tr0[i]; dr[i] = r1[i] - r0[i]; }
    double pt = tt30[0] * drt[0] + tt30[1] * drt[1] + tt30[2] * drt[2];
    double pc = t30[0] * dr[0] + t30[1] * dr[1] + t30[2] * dr[2];
    for (int i = 0; i < 3; i++) {
        dpt[i] = drt[i] - tt30[i] * pt;
        dp[i] = dr[i] - t30[i] * pc;
        bt[i] = t31[i] - tt30[i] - dpt[i] * s->eta[b];
        bc[i] = t31[i] - t30[i] - dp[i] * s->eta[b];
    }
    if (s->eps_twist)
        return e_pair_twist(s, bt, pt, dpt, twist_omega(tt20, tt30, t21, t31), b)
             - e_pair_twist(s, bc, pc, dp, twist_omega(t20, t30, t21, t31), b);
    return e_pair(s, bt, pt, dpt, b) - e_pair(s, bc, pc, dp, b);
}

/* continuous_dE_poly, polymers.pyx:1084-1146.  tr0 / tr_last: trial (r,t3) of
 * beads ind0 and indf-1. */
static double continuous_dE(const or_system *s, int64_t ind0, int64_t indf,
                            const double *trial_first, const double *trial_last)
{
    double dE = 0, a[3], b[3], c[3], d[3], e[3], f[3];
    if (ind0 != 0) {
        ld3(s->r, ind0 - 1, a); ld3(s->r, ind0, b); ld3(s->t3, ind0 - 1, c); ld3(s->t3, ind0, d);
        ld3(s->t2, ind0 - 1, e); ld3(s->t2, ind0, f);
        dE += pair_dE_fwd(s, a, b, trial_first, c, d, trial_first + 3, ind0 - 1, e, f, trial_first + 6);
    }
    if (indf != s->n_beads) {
        ld3(s->r, indf - 1, a); ld3(s->r, indf, b); ld3(s->t3, indf - 1, c); ld3(s->t3, indf, d);
        ld3(s->t2, indf - 1, e); ld3(s->t2, indf, f);
        dE += pair_dE_rev(s, a, trial_last, b, c, trial_last + 3, d, indf - 1, e, trial_last + 6, f);
    }
    return dE;
}

/* SSWLC.compute_E, polymers.pyx:1348-1381 */
double or_elastic_E(const or_system *s)
{
    double E = 0;
    for (int64_t i = 1; i < s->n_beads; i++) {
        double r0[3], r1[3], a[3], b[3], dr[3], dp[3], bend[3];
        ld3(s->r, i - 1, r0); ld3(s->r, i, r1); ld3(s->t3, i - 1, a); ld3(s->t3, i, b);
        for (int j = 0; j < 3; j++) dr[j] = r1[j] - r0[j];
        double par = a[0] * dr[0] + a[1] * dr[1] + a[2] * dr[2];
        for (int j = 0; j < 3; j++) dp[j] = dr[j] - a[j] * par;
        for (int j = 0; j < 3; j++) bend[j] = b[j] + (-a[j] - s->eta[i - 1] * dp[j]);
        if (s->eps_twist) {  /* SSTWLC.compute_E, polymers.pyx:2250-2285 */
            double c2[3], d2[3];
            ld3(s->t2, i - 1, c2); ld3(s->t2, i, d2);
            E += e_pair_twist(s, bend, par, dp, twist_omega(c2, a, d2, b), i - 1);
        } else {
            E += e_pair(s, bend, par, dp, i - 1);
        }
    }
    return E;
}

/* ---------------- binding energy: polymers.pyx:1383-1538 ----------------- */

static double bind_f(const or_system *s, int64_t b, int64_t nm, int64_t st)
{
    return s->bind_f[(b * (s->mark_max + 1) + nm) * (s->site_max + 1) + st];
}

static double mu_eff(const or_system *s, int64_t b)
{
    /* polymers.pyx:1519-1537: annealing scales positive and negative mu differently */
    if (s->mu[b] > 0) return s->mu[b] * (-s->mu_adjust_factor + 2);
    return s->mu[b] * s->mu_adjust_factor;
}

/* bead_binding_dE, polymers.pyx:1408-1538; st_trial has nb entries */
static double bead_binding_dE(const or_system *s, int64_t ind, const int64_t *st_trial)
{
    int64_t nb = s->n_binders;
    const int64_t *st = s->states + ind * nb;
    const int64_t *mk = s->marks + ind * nb;
    double dE = 0;
    if (s->max_binders != -1) {
        int64_t tot = 0;
        for (int64_t h = 0; h < nb; h++) tot += st_trial[h];
        if (tot > s->max_binders) dE += OR_E_HUGE_POLY * (double)(tot - s->max_binders);
        tot = 0;
        for (int64_t h = 0; h < nb; h++) tot += st[h];
        if (tot > s->max_binders) dE -= OR_E_HUGE_POLY * (double)(tot - s->max_binders);
    }
    for (int64_t b = 0; b < nb; b++) {
        dE += bind_f(s, b, mk[b], st_trial[b]);
        dE -= bind_f(s, b, mk[b], st[b]);
        if (s->mu[b] > 0) {
            double me = s->mu[b] * (-s->mu_adjust_factor + 2);
            dE -= (double)st_trial[b] * me;
            dE += (double)st[b] * me;
        } else {
            /* (state * mu) * factor, left to right as at polymers.pyx:1532-1537 */
            dE -= (double)st_trial[b] * s->mu[b] * s->mu_adjust_factor;
            dE += (double)st[b] * s->mu[b] * s->mu_adjust_factor;
        }
    }
    return dE;
}

/* single-site free energies of the current states (the dE-consistent binding energy) */
double or_binding_E(const or_system *s)
{
    double E = 0;
    int64_t nb = s->n_binders;
    for (int64_t i = 0; i < s->n_beads; i++) {
        const int64_t *st = s->states + i * nb;
        const int64_t *mk = s->marks + i * nb;
        int64_t tot = 0;
        for (int64_t b = 0; b < nb; b++) {
            E += bind_f(s, b, mk[b], st[b]) - (double)st[b] * mu_eff(s, b);
            tot += st[b];
        }
        if (s->max_binders != -1 && tot > s->max_binders)
            E += OR_E_HUGE_POLY * (double)(tot - s->max_binders);
    }
    return E;
}

/* ---------------- density field: chromo/fields.pyx ----------------------- */

static inline double pymod(double a, double b)
{
    double m = fmod(a, b);
    if (m != 0 && ((m < 0) != (b < 0))) m += b;
    return m;
}

/* Eight trilinear weights and voxel super-indices of one position,
 * fields.pyx:1430-1458 (bin + lower weight), :1524-1598 (weights),
 * :1600-1673 (indices), :565-575 (periodic super-index table). */
static float pymodf_(float a, float b)
{
    if (a >= 0 && a < b) return a;
    float m = fmodf(a, b);
    if (m != 0 && ((m < 0) != (b < 0))) m += b;
    return m;
}

/* FP32 trilinear weights, the GPU's FP32-storage arithmetic */
static void voxel_weights_f32(const or_system *s, const double pos[3], double w[8], int64_t v[8])
{
    const double width[3] = {s->x_width, s->y_width, s->z_width};
    const int64_t n[3] = {s->nx, s->ny, s->nz};
    float wl[3];
    int64_t lo[3], hi[3];
    for (int j = 0; j < 3; j++) {
        double d = width[j] / (double)n[j];
        float fw = (float)width[j], hw = (float)(0.5 * width[j]), hd = (float)(0.5 * d);
        float inv = (float)(1.0 / d);
        float x = pymodf_((float)pos[j] + hw, fw) - hd;
        float t = x * inv;
        float fl = floorf(t);
        int ind = (int)fl;
        int64_t li = ind == -1 ? n[j] - 1 : ind;
        lo[j] = li < 0 ? 0 : (li >= n[j] ? n[j] - 1 : li);
        hi[j] = (lo[j] + 1) % n[j];
        wl[j] = 1 - (t - fl);
    }
    for (int l = 0; l < 8; l++) {
        int bx = l & 1, by = (l >> 1) & 1, bz = (l >> 2) & 1;
        float fx = bx ? (1 - wl[0]) : wl[0];
        float fy = by ? (1 - wl[1]) : wl[1];
        float fz = bz ? (1 - wl[2]) : wl[2];
        w[l] = (double)(fx * fy * fz);
        int64_t ix = bx ? hi[0] : lo[0], iy = by ? hi[1] : lo[1], iz = bz ? hi[2] : lo[2];
        v[l] = ix + s->nx * iy + s->nx * s->ny * iz;
    }
}

/* Eight weights and voxels from per-axis lower voxels and lower weights. */
static void corners(const or_system *s, const double wl[3], const int64_t lo[3], const int64_t hi[3],
                    double w[8], int64_t v[8])
{
    for (int l = 0; l < 8; l++) {
        int bx = l & 1, by = (l >> 1) & 1, bz = (l >> 2) & 1;
        double fx = bx ? (1 - wl[0]) : wl[0];
        double fy = by ? (1 - wl[1]) : wl[1];
        double fz = bz ? (1 - wl[2]) : wl[2];
        w[l] = fx * fy * fz;
        int64_t ix = bx ? hi[0] : lo[0], iy = by ? hi[1] : lo[1], iz = bz ? hi[2] : lo[2];
        v[l] = ix + s->nx * iy + s->nx * s->ny * iz;
    }
}

/* fast_field: the weights of a move's density change from sub-bins
 * (get_change_in_density_quickly, fields.pyx:1235-1368, with the tables of
 * init_fast_field, :577-671): a coordinate's sub-bin is
 * floor((x + L/2) / w_sub) mod (n_points n), w_sub = dx / n_points, and the
 * voxel and lower weight are those of the sub-bin's lower edge shifted by
 * half a voxel: q = ((i - n_points/2) w_sub) / dx, voxel floor(q) (-1 -> n-1),
 * lower weight 1 - (q - floor(q)).  Full deposits keep exact weights. */
static void fast_weights(const or_system *s, const double pos[3], double w[8], int64_t v[8])
{
    const double width[3] = {s->x_width, s->y_width, s->z_width};
    const int64_t n[3] = {s->nx, s->ny, s->nz};
    const double np = (double)s->fast_n;
    int64_t lo[3], hi[3];
    if (emu32(s)) {  /* the GPU's binary32 construction */
        float wl[3];
        for (int j = 0; j < 3; j++) {
            double d = width[j] / (double)n[j];
            float hw = (float)(0.5 * width[j]), inv_sw = (float)(np / d), sw = (float)(d / np);
            float nsub = (float)(np * (double)n[j]), inv_d = (float)(1.0 / d), hnp = (float)(0.5 * np);
            float sb = pymodf_(floorf(((float)pos[j] + hw) * inv_sw), nsub);
            float q = ((sb - hnp) * sw) * inv_d;
            float fl = floorf(q);
            int ind = (int)fl;
            int64_t li = ind == -1 ? n[j] - 1 : ind;
            lo[j] = li < 0 ? 0 : (li >= n[j] ? n[j] - 1 : li);
            hi[j] = (lo[j] + 1) % n[j];
            wl[j] = 1 - (q - fl);
        }
        for (int l = 0; l < 8; l++) {
            int bx = l & 1, by = (l >> 1) & 1, bz = (l >> 2) & 1;
            float fx = bx ? (1 - wl[0]) : wl[0];
            float fy = by ? (1 - wl[1]) : wl[1];
            float fz = bz ? (1 - wl[2]) : wl[2];
            w[l] = (double)(fx * fy * fz);
            int64_t ix = bx ? hi[0] : lo[0], iy = by ? hi[1] : lo[1], iz = bz ? hi[2] : lo[2];
            v[l] = ix + s->nx * iy + s->nx * s->ny * iz;
        }
        return;
    }
    double wl[3];
    for (int j = 0; j < 3; j++) {
        double d = width[j] / (double)n[j];
        double sw = d / np;
        double sb = pymod(floor((pos[j] + 0.5 * width[j]) / sw), np * (double)n[j]);
        double q = ((sb - np / 2) * sw) / d;
        double ind = floor(q);
        lo[j] = ind == -1.0 ? n[j] - 1 : (int64_t)ind;
        hi[j] = (lo[j] + 1) % n[j];
        wl[j] = 1 - (q - ind);
    }
    corners(s, wl, lo, hi, w, v);
}

static void voxel_weights(const or_system *s, const double pos[3], double w[8], int64_t v[8])
{
    if (emu32(s)) { voxel_weights_f32(s, pos, w, v); return; }
    const double width[3] = {s->x_width, s->y_width, s->z_width};
    const int64_t n[3] = {s->nx, s->ny, s->nz};
    double wl[3];
    int64_t lo[3], hi[3];
    for (int j = 0; j < 3; j++) {
        double d = width[j] / (double)n[j];
        double x = pymod(pos[j] + 0.5 * width[j], width[j]) - 0.5 * d;
        int64_t ind = (int64_t)floor(x / d);
        lo[j] = ind == -1 ? n[j] - 1 : ind;
        hi[j] = (lo[j] + 1) % n[j];
        wl[j] = 1 - (x / d - (double)ind);
    }
    for (int l = 0; l < 8; l++) {
        int bx = l & 1, by = (l >> 1) & 1, bz = (l >> 2) & 1;
        double fx = bx ? (1 - wl[0]) : wl[0];
        double fy = by ? (1 - wl[1]) : wl[1];
        double fz = bz ? (1 - wl[2]) : wl[2];
        w[l] = fx * fy * fz;
        int64_t ix = bx ? hi[0] : lo[0], iy = by ? hi[1] : lo[1], iz = bz ? hi[2] : lo[2];
        v[l] = ix + s->nx * iy + s->nx * s->ny * iz;
    }
}

static inline double avol(const or_system *s, int64_t v)
{
    return s->access_vol ? s->access_vol[v] : s->vol_bin;
}

static inline int64_t q40(double w) { return (int64_t)llrint(w * OR_FX_SCALE); }

/* update_all_densities_for_all_polymers, fields.pyx:2041-2106 (one polymer) */
void or_deposit_all(or_system *s)
{
    int64_t nc = s->n_binders + 1, G = s->nx * s->ny * s->nz;
    if (s->fixed_density) memset(s->density_fx, 0, sizeof(int64_t) * G * nc);
    else memset(s->density, 0, sizeof(double) * G * nc);
    for (int64_t i = 0; i < s->n_beads; i++) {
        double p[3], w[8];
        int64_t v[8];
        ld3(s->r, i, p);
        voxel_weights(s, p, w, v);
        for (int l = 0; l < 8; l++) {
            if (s->fixed_density) {
                int64_t q = q40(w[l]);
                s->density_fx[v[l] * nc] += q;
                for (int64_t m = 1; m < nc; m++)
                    s->density_fx[v[l] * nc + m] += q * s->states[i * s->n_binders + m - 1];
            } else {
                double d = w[l] / avol(s, v[l]);
                s->density[v[l] * nc] += d;
                for (int64_t m = 1; m < nc; m++)
                    s->density[v[l] * nc + m] += d * (double)s->states[i * s->n_binders + m - 1];
            }
        }
    }
    if (!s->fixed_density)
        for (int64_t i = 0; i < G * nc; i++)
            if (fabs(s->density[i]) < 1e-18) s->density[i] = 0;
}

/* get_confinement_dE, fields.pyx:121-202.  trial = 1 reads the moved beads'
 * trial positions.  The cubical branch for trial = 0 is nested under
 * "if trial == 1" in the reference and therefore always counts zero; that is
 * kept. */
static int64_t confinement_count(const or_system *s, int64_t n, int trial)
{
    if (s->confine_kind == 0) return 0;
    int64_t out = 0;
    for (int64_t k = 0; k < n; k++) {
        double p[3];
        if (trial) { p[0] = s->trial[9 * k]; p[1] = s->trial[9 * k + 1]; p[2] = s->trial[9 * k + 2]; }
        else ld3(s->r, s->inds[k], p);
        if (s->confine_kind == 1) {
            if (sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]) > s->confine_length) out++;
        } else if (trial) {
            for (int j = 0; j < 3; j++)
                if (fabs(p[j]) > s->confine_length / 2) out++;
        }
    }
    return out;
}

static double confinement_E(const or_system *s, int64_t n, int trial)
{
    return (double)confinement_count(s, n, trial) * OR_E_HUGE_FIELD;
}

static void touch(or_system *s, int64_t v, int *is_new)
{
    if (s->slot_of[v] < 0) {
        s->slot_of[v] = s->n_found;
        s->found[s->n_found++] = v;
        *is_new = 1;
    } else *is_new = 0;
}

/* Order in which a CPython set of small non-negative ints iterates.  The
 * reference collects the touched voxels in a Python set and sums over
 * np.array(list(bins_found)) (fields.pyx:1428,1522); in the regime where a
 * voxel crosses vf_limit the field dE is a difference of ~1e97 terms and its
 * rounding depends on that order.  This reproduces the open-addressing table
 * of CPython's set (hash(i) = i, 8 initial slots, 9 linear probes, perturbed
 * probing, resize to 4x used when 5*fill >= 3*mask) and rewrites s->found in
 * table order. */
static void pyset_order(or_system *s)
{
    int64_t n = s->n_found;
    size_t cap = 8;
    while (cap < (size_t)(4 * n + 8)) cap <<= 1;
    int64_t *tab = malloc(sizeof(int64_t) * cap * 2), *tmp = tab + cap;
    size_t mask = 7, fill = 0;
    for (size_t i = 0; i <= mask; i++) tab[i] = -1;
    for (int64_t e = 0; e < n; e++) {
        int64_t key = s->found[e];
        size_t perturb = (size_t)key, i = (size_t)key & mask;
        for (;;) {
            size_t probes = (i + 9 <= mask) ? 9 : 0, j = i;
            int done = 0;
            for (;;) {
                if (tab[j] == -1) { tab[j] = key; done = 1; break; }
                if (probes-- == 0) break;
                j++;
            }
            if (done) break;
            perturb >>= 5;
            i = (i * 5 + 1 + perturb) & mask;
        }
        fill++;
        if (fill * 5 >= mask * 3) {
            size_t newsize = 8, old = mask;
            while (newsize <= fill * 4) newsize <<= 1;
            for (size_t q = 0; q <= old; q++) tmp[q] = tab[q];
            mask = newsize - 1;
            for (size_t q = 0; q <= mask; q++) tab[q] = -1;
            for (size_t q = 0; q <= old; q++) {
                if (tmp[q] < 0) continue;
                int64_t k2 = tmp[q];
                size_t pt = (size_t)k2, ii = (size_t)k2 & mask;
                for (;;) {
                    if (tab[ii] == -1) { tab[ii] = k2; break; }
                    int placed = 0;
                    if (ii + 9 <= mask) {
                        for (size_t jj = 1; jj <= 9; jj++)
                            if (tab[ii + jj] == -1) { tab[ii + jj] = k2; placed = 1; break; }
                    }
                    if (placed) break;
                    pt >>= 5;
                    ii = (ii * 5 + 1 + pt) & mask;
                }
            }
        }
    }
    int64_t m = 0;
    for (size_t q = 0; q <= mask; q++)
        if (tab[q] >= 0) s->found[m++] = tab[q];
    free(tab);
}

/* get_change_in_density, fields.pyx:1370-1522 (FP64, reference semantics), or
 * the fixed-point equivalent.  n moved beads: s->inds[k], trial positions in
 * s->trial, trial states (state_change) in s->new_states for binder bsel. */
static void change_in_density(or_system *s, int64_t n, int state_change, int64_t bsel)
{
    int64_t nb = s->n_binders, nc = nb + 1;
    s->n_found = 0;
    for (int64_t k = 0; k < n; k++) {
        int64_t i = s->inds[k];
        double p0[3], p1[3], w[2][8];
        int64_t v[2][8];
        ld3(s->r, i, p0);
        if (state_change) { p1[0] = p0[0]; p1[1] = p0[1]; p1[2] = p0[2]; }
        else { p1[0] = s->trial[9 * k]; p1[1] = s->trial[9 * k + 1]; p1[2] = s->trial[9 * k + 2]; }
        if (s->fast_n > 0) {
            fast_weights(s, p0, w[0], v[0]);
            fast_weights(s, p1, w[1], v[1]);
        } else {
            voxel_weights(s, p0, w[0], v[0]);
            voxel_weights(s, p1, w[1], v[1]);
        }
        for (int c = 0; c < 2; c++) {
            for (int l = 0; l < 8; l++) {
                int is_new;
                int64_t vox = v[c][l];
                touch(s, vox, &is_new);
                for (int64_t m = 0; m < nc; m++) {
                    int64_t st = 1;
                    if (m > 0) {
                        st = s->states[i * nb + m - 1];
                        if (c == 1 && state_change && m - 1 == bsel) st = s->new_states[k];
                    }
                    if (s->fixed_density) {
                        int64_t q = q40(w[c][l]) * st;
                        if (c == 0) q = -q;
                        if (is_new) s->dfx[vox * nc + m] = q;
                        else s->dfx[vox * nc + m] += q;
                    } else {
                        double dt = w[c][l] / avol(s, vox);
                        if (m > 0) dt = dt * (double)st;
                        double temp = (c == 0 ? -1. : 1.) * dt;
                        if (is_new) s->density_trial[vox * nc + m] = fabs(temp) > 1e-18 ? temp : 0;
                        else if (fabs(temp) > 1e-18) s->density_trial[vox * nc + m] += temp;
                    }
                }
            }
        }
    }
}

/* count_doubly_bound, fields.pyx:1877-1937 */
static int64_t doubly_bound(const or_system *s, int64_t n, int64_t b, int trial,
                            int state_change, int64_t bsel)
{
    int64_t cnt = 0;
    for (int64_t k = 0; k < n; k++) {
        int64_t st = s->states[s->inds[k] * s->n_binders + b];
        if (trial && state_change && b == bsel) st = s->new_states[k];
        if (st == 2) cnt++;
    }
    return cnt;
}

/* get_dE_binders_and_beads + nonspecific_interact_dE, fields.pyx:1675-1875 */
static double dE_binders_and_beads(or_system *s, int64_t n, int state_change, int64_t bsel,
                                   int64_t *huge)
{
    int64_t nb = s->n_binders, nc = nb + 1;
    double dE = 0;
    if (!s->fixed_density) {
        /* reference order: per binder oligomerisation + intranucleosome, then
         * cross talk, then the nonspecific term (fields.pyx:1759-1790) */
        for (int64_t b = 0; b < nb; b++) {
            double tot = 0;
            for (int64_t j = 0; j < s->n_found; j++) {
                int64_t v = s->found[j];
                double rho = s->density[v * nc + b + 1], d = s->density_trial[v * nc + b + 1];
                double x = pow(rho + d, 2.0) - pow(rho, 2.0);
                if (fabs(x) < 1e-18) x = 0;
                tot += x;
            }
            dE += s->pref[b] * tot;
            int64_t dd = doubly_bound(s, n, b, 1, state_change, bsel)
                       - doubly_bound(s, n, b, 0, state_change, bsel);
            dE += s->intra[b] * (double)dd;
        }
        for (int64_t b = 0; b < nb; b++)
            for (int64_t c = 0; c < nb; c++) {
                double tot = 0;
                for (int64_t j = 0; j < s->n_found; j++) {
                    int64_t v = s->found[j];
                    double rb = s->density[v * nc + b + 1], db = s->density_trial[v * nc + b + 1];
                    double rc = s->density[v * nc + c + 1], dc = s->density_trial[v * nc + c + 1];
                    double x = (rb + db) * (rc + dc) - rb * rc;
                    if (fabs(x) < 1e-18) x = 0;
                    tot += x;
                }
                dE += s->xpref[b * nb + c] * tot;
            }
        double ns = 0;
        for (int64_t j = 0; j < s->n_found; j++) {
            int64_t v = s->found[j];
            double V = avol(s, v);
            double vf0 = s->density[v * nc] * s->bead_vol;
            double vf1 = vf0 + s->density_trial[v * nc] * s->bead_vol;
            if (vf1 > s->vf_limit) ns += OR_E_HUGE_FIELD * vf1;
            else ns += s->chi * (V / s->bead_vol) * pow(vf1, 2.0);
            if (vf0 > s->vf_limit) ns -= OR_E_HUGE_FIELD * vf0;
            else ns -= s->chi * (V / s->bead_vol) * pow(vf0, 2.0);
        }
        return dE + ns;
    }
    /* fixed-point grid: per-voxel contribution in the GPU's formula */
    for (int64_t j = 0; j < s->n_found; j++) {
        int64_t v = s->found[j];
        double V = avol(s, v);
        double c = 0, rho[OR_MAXB], d[OR_MAXB];
        for (int64_t b = 0; b < nb; b++) {
            rho[b] = ((double)s->density_fx[v * nc + b + 1] / OR_FX_SCALE) / V;
            d[b] = ((double)s->dfx[v * nc + b + 1] / OR_FX_SCALE) / V;
            c += s->pref[b] * (d[b] * (2 * rho[b] + d[b]));
        }
        for (int64_t b = 0; b < nb; b++)
            for (int64_t e = 0; e < nb; e++)
                c += s->xpref[b * nb + e] * (rho[b] * d[e] + d[b] * rho[e] + d[b] * d[e]);
        double vf0 = ((double)s->density_fx[v * nc] / OR_FX_SCALE) / V * s->bead_vol;
        double vf1 = ((double)(s->density_fx[v * nc] + s->dfx[v * nc]) / OR_FX_SCALE) / V * s->bead_vol;
        double k = s->chi * (V / s->bead_vol);
        if (vf1 > s->vf_limit || vf0 > s->vf_limit) {
            double u = s->bead_vol / V;
            if (vf1 > s->vf_limit)
                *huge += llrint((double)(s->density_fx[v * nc] + s->dfx[v * nc]) * u);
            else c += k * vf1 * vf1;
            if (vf0 > s->vf_limit) *huge -= llrint((double)s->density_fx[v * nc] * u);
            else c -= k * vf0 * vf0;
        } else {
            c += k * ((vf1 - vf0) * (vf1 + vf0));
        }
        dE += c;
    }
    for (int64_t b = 0; b < nb; b++) {
        int64_t dd = doubly_bound(s, n, b, 1, state_change, bsel)
                   - doubly_bound(s, n, b, 0, state_change, bsel);
        dE += s->intra[b] * (double)dd;
    }
    return dE;
}

/* UniformDensityField.compute_dE, fields.pyx:1149-1233 / NullField, :309-319 */
static double field_dE(or_system *s, int64_t n, int state_change, int64_t bsel)
{
    double dE = 0;
    if (s->fixed_density) {
        /* the GPU's formula: exact penalty units (OR_HUGE_UNIT) */
        int64_t huge = 0;
        if (s->field_kind == 1) {
            huge = (confinement_count(s, n, 1) - confinement_count(s, n, 0)) * (int64_t)OR_FX_SCALE;
            return (double)huge * OR_HUGE_UNIT;
        }
        if (!state_change)
            huge += (confinement_count(s, n, 1) - confinement_count(s, n, 0)) * (int64_t)OR_FX_SCALE;
        change_in_density(s, n, state_change, bsel);
        dE += dE_binders_and_beads(s, n, state_change, bsel, &huge);
        if (huge) dE += (double)huge * OR_HUGE_UNIT;
        return dE;
    }
    if (s->field_kind == 1) {
        /* NullField.compute_dE evaluates confinement for every move type */
        dE = confinement_E(s, n, 1);
        dE -= confinement_E(s, n, 0);
        return dE;
    }
    if (!state_change) {
        dE += confinement_E(s, n, 1);
        dE -= confinement_E(s, n, 0);
    }
    change_in_density(s, n, state_change, bsel);
    pyset_order(s);
    dE += dE_binders_and_beads(s, n, state_change, bsel, NULL);
    return dE;
}

/* update_affected_densities, fields.pyx:1968-1975 (+ reset of the touched set) */
static void field_commit(or_system *s, int accept)
{
    int64_t nc = s->n_binders + 1;
    for (int64_t j = 0; j < s->n_found; j++) {
        int64_t v = s->found[j];
        if (accept) {
            for (int64_t m = 0; m < nc; m++) {
                if (s->fixed_density) s->density_fx[v * nc + m] += s->dfx[v * nc + m];
                else {
                    s->density[v * nc + m] += s->density_trial[v * nc + m];
                    s->density_trial[v * nc + m] = 0;
                }
            }
        }
        s->slot_of[v] = -1;
    }
    s->n_found = 0;
}

/* dE-consistent field energy: the quantity whose differences are the per-move
 * field dE (fields.pyx:1675-1875), i.e. sum_b pref_b sum rho_b^2 +
 * sum_bc xpref_bc sum rho_b rho_c + chi (V/Vb) sum vf^2 (1e99 vf above the
 * limit) + intranucleosome * (#doubly bound). */
double or_field_E(const or_system *s)
{
    int64_t nb = s->n_binders, nc = nb + 1, G = s->nx * s->ny * s->nz;
    double E = 0;
    if (s->field_kind != 2) return 0;
    for (int64_t v = 0; v < G; v++) {
        double V = avol(s, v), rho[OR_MAXB], n0;
        for (int64_t b = 0; b < nb; b++)
            rho[b] = s->fixed_density ? ((double)s->density_fx[v * nc + b + 1] / OR_FX_SCALE) / V
                                      : s->density[v * nc + b + 1];
        n0 = s->fixed_density ? ((double)s->density_fx[v * nc] / OR_FX_SCALE) / V : s->density[v * nc];
        for (int64_t b = 0; b < nb; b++) E += s->pref[b] * rho[b] * rho[b];
        for (int64_t b = 0; b < nb; b++)
            for (int64_t c = 0; c < nb; c++) E += s->xpref[b * nb + c] * rho[b] * rho[c];
        double vf = n0 * s->bead_vol;
        E += vf > s->vf_limit ? OR_E_HUGE_FIELD * vf : s->chi * (V / s->bead_vol) * vf * vf;
    }
    for (int64_t b = 0; b < nb; b++) {
        int64_t cnt = 0;
        for (int64_t i = 0; i < s->n_beads; i++) cnt += s->states[i * nb + b] == 2;
        E += s->intra[b] * (double)cnt;
    }
    return E;
}

/* ---------------- scratch -------------------------------------------------- */

int or_scratch_init(or_system *s)
{
    int64_t nc = s->n_binders + 1, G = s->nx * s->ny * s->nz, N = s->n_beads;
    if (s->n_binders > OR_MAXB || N < 1) return OR_ERR_ARGS;
    if (G < 1) G = 1;
    s->density_trial = calloc((size_t)(G * nc), sizeof(double));
    s->dfx = calloc((size_t)(G * nc), sizeof(int64_t));
    s->slot_of = malloc(sizeof(int64_t) * (size_t)G);
    s->found_cap = G;
    s->found = malloc(sizeof(int64_t) * (size_t)G);
    s->inds = malloc(sizeof(int64_t) * (size_t)N);
    s->trial = malloc(sizeof(double) * 9 * (size_t)N);
    s->new_states = malloc(sizeof(int64_t) * (size_t)N);
    s->picked = calloc((size_t)N, 1);
    if (!s->density_trial || !s->dfx || !s->slot_of || !s->found || !s->inds || !s->trial
        || !s->new_states || !s->picked) return OR_ERR_ALLOC;
    for (int64_t v = 0; v < G; v++) s->slot_of[v] = -1;
    s->n_found = 0;
    return OR_OK;
}

void or_scratch_free(or_system *s)
{
    free(s->density_trial); free(s->dfx); free(s->slot_of); free(s->found);
    free(s->inds); free(s->trial); free(s->new_states); free(s->picked);
    s->density_trial = NULL; s->dfx = NULL; s->slot_of = NULL; s->found = NULL;
    s->inds = NULL; s->trial = NULL; s->new_states = NULL; s->picked = NULL;
}

/* ---------------- one MC step: chromo/mc/mc_sim.pyx:106-182 --------------- */

static void rot_axis_crank(const or_system *s, or_rng *g, int64_t ind0, int64_t indf, double dir[3])
{
    /* get_crank_shaft_axis, move_funcs.pyx:157-234 */
    int64_t N = s->n_beads;
    double a[3], b[3];
    if (ind0 == indf - 1 && ind0 == 0) { ld3(s->r, indf, a); ld3(s->r, ind0, b); }
    else if (ind0 == indf - 1 && ind0 == N - 1) { ld3(s->r, ind0, a); ld3(s->r, ind0 - 1, b); }
    else if (ind0 == 0 && indf == N) { ld3(s->r, indf - 1, a); ld3(s->r, ind0, b); }
    else if (ind0 == 0) { ld3(s->r, indf, a); ld3(s->r, ind0, b); }
    else if (indf == N) { ld3(s->r, indf - 1, a); ld3(s->r, ind0 - 1, b); }
    else { ld3(s->r, indf, a); ld3(s->r, ind0 - 1, b); }
    if (emu32(s)) {
        float d[3] = {(float)a[0] - (float)b[0], (float)a[1] - (float)b[1], (float)a[2] - (float)b[2]};
        float mag = sqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
        if (mag < 1E-5f) { sphere_f32(g, dir); return; }
        float sc = 1.0f / mag;
        for (int i = 0; i < 3; i++) dir[i] = (double)(d[i] * sc);
        return;
    }
    for (int i = 0; i < 3; i++) dir[i] = a[i] - b[i];
    int rp = !s->fixed_density;
    double mag = sqrt(sq(dir[0], rp) + sq(dir[1], rp) + sq(dir[2], rp));
    if (mag < 1E-5) sphere(g, dir);
    else {
        double sc = 1.0 / mag;
        for (int i = 0; i < 3; i++) dir[i] = dir[i] * sc;
    }
}

static void crank_fulcrum(const or_system *s, int64_t ind0, int64_t indf, double p[3])
{
    /* get_crank_shaft_fulcrum, move_funcs.pyx:237-280 */
    int64_t N = s->n_beads;
    if (ind0 == 0 && indf != N) ld3(s->r, indf, p);
    else if (ind0 != 0 && indf == N) ld3(s->r, ind0 - 1, p);
    else if (ind0 == 0 && indf == N) ld3(s->r, ind0, p);
    else ld3(s->r, ind0 - 1, p);
}

static void end_pivot_fulcrum(const or_system *s, int64_t ind0, int64_t indf, int64_t lhs, double p[3])
{
    /* get_end_pivot_fulcrum, move_funcs.pyx:349-398 */
    int64_t N = s->n_beads;
    if (ind0 == 0 && indf != N) ld3(s->r, indf, p);
    else if (ind0 != 0 && indf == N) ld3(s->r, ind0 - 1, p);
    else if (ind0 == 0 && indf == N && lhs == 1) ld3(s->r, indf - 1, p);
    else ld3(s->r, ind0, p);
}

/* Propose (move_funcs.pyx), evaluate dE (mc_sim.pyx:153-162), Metropolis
 * (:163-171), accept / reject (moves.pyx:156-286, fields.pyx:1968).
 * Returns n_inds (0: empty move, returned before dE as in mc_sim.pyx:150-151). */
/* One attempted move.  forced (0 / 1, or -1 for none) is the decision of a
 * run being followed: it replaces this move's own decision when the two
 * differ and dE lies in the tie band |dE + ln u| <= 1e-5 max(1, |dE|), where
 * the FP32 arithmetic of the followed run may legitimately decide otherwise. */
static int64_t mc_step(or_system *s, or_ctl *c, or_rng *g, or_record *rec, int forced)
{
    int64_t N = s->n_beads, nb = s->n_binders, n = 0, ind0 = 0, indf = 0, bsel = -1;
    int64_t draw0 = g->pos;
    int kind = (int)c->move_kind;
    int check_field = s->field_kind != 0 && kind != MV_TANGENT;
    double dEp = 0, dEf = 0;
    c->num_attempt += 1;                        /* moves.pyx:151 */
    if (kind == MV_CRANK || kind == MV_END_PIVOT || kind == MV_SLIDE) {
        double M[3][4];
        if (kind == MV_CRANK) {                 /* move_funcs.pyx:39-101 */
            int64_t xang = rnd(g);
            double ang = c->amp_move * ((double)xang / OR_RAND_MAX - 0.5);
            float angf = (float)c->amp_move * (cgm_unif24((unsigned)xang) - 0.5f);
            int64_t b0 = (int32_t)(rndu(g) * (double)N);
            int64_t b1 = from_point(g, c->amp_bead, N, b0);
            if (b1 < 1) b1 = 1;
            check_bead_bounds(b0, b1, N, &ind0, &indf);
            double dir[3], p[3];
            rot_axis_crank(s, g, ind0, indf, dir);
            crank_fulcrum(s, ind0, indf, p);
            if (emu32(s)) {
                float sn, cs;
                cgm_sincosf(angf, &sn, &cs);
                axis_rotation_f32(dir, p, sn, cs, M);
            } else axis_rotation(dir, p, ang, M, !s->fixed_density);
        } else if (kind == MV_END_PIVOT) {      /* move_funcs.pyx:285-346 */
            int64_t xang = rnd(g);
            double ang = c->amp_move * ((double)xang / OR_RAND_MAX - 0.5);
            float angf = (float)c->amp_move * (cgm_unif24((unsigned)xang) - 0.5f);
            int64_t lhs = rnd(g) % 2;
            if (lhs == 1) { ind0 = 0; indf = from_left(g, c->amp_bead, N) + 1; }
            else { ind0 = from_right(g, c->amp_bead, N); indf = N; }
            double axis[3], p[3];
            if (emu32(s)) sphere_f32(g, axis);
            else sphere(g, axis);
            end_pivot_fulcrum(s, ind0, indf, lhs, p);
            if (emu32(s)) {
                float sn, cs;
                cgm_sincosf(angf, &sn, &cs);
                axis_rotation_f32(axis, p, sn, cs, M);
            } else axis_rotation(axis, p, ang, M, !s->fixed_density);
        } else {                                /* move_funcs.pyx:403-465 */
            int64_t xamp = rnd(g);
            double amp = c->amp_move * ((double)xamp / OR_RAND_MAX), d[3];
            if (emu32(s)) {
                float ampf = (float)c->amp_move * cgm_unif24((unsigned)xamp);
                sphere_f32(g, d);
                for (int i = 0; i < 3; i++) d[i] = (double)((float)d[i] * ampf);
            } else {
                sphere(g, d);
                for (int i = 0; i < 3; i++) d[i] = d[i] * amp;
            }
            memset(M, 0, sizeof(M));
            M[0][0] = M[1][1] = M[2][2] = 1;
            M[0][3] = d[0]; M[1][3] = d[1]; M[2][3] = d[2];
            int64_t b0 = rnd(g) % N;
            int64_t b1 = from_point(g, c->amp_bead, N, b0);
            check_bead_bounds(b0, b1, N, &ind0, &indf);
        }
        if (g->err) return g->err;
        n = indf - ind0;
        for (int64_t k = 0; k < n; k++) {
            s->inds[k] = ind0 + k;
            if (kind == MV_SLIDE) {
                /* slide translates r only (move_funcs.pyx:458-463) */
                double r[3];
                ld3(s->r, ind0 + k, r);
                for (int j = 0; j < 3; j++) {
                    s->trial[9 * k + j] = emu32(s) ? (double)((float)r[j] + (float)M[j][3])
                                                   : rnd_pos(r[j] + M[j][3]);
                    s->trial[9 * k + 3 + j] = (double)s->t3[3 * (ind0 + k) + j];
                    s->trial[9 * k + 6 + j] = (double)s->t2[3 * (ind0 + k) + j];
                }
            } else transform_bead(s, ind0 + k, M, s->trial + 9 * k);
        }
        if (n == 0) goto empty;
        dEp = continuous_dE(s, ind0, indf, s->trial, s->trial + 9 * (n - 1));
        if (check_field) dEf = field_dE(s, n, 0, -1);
    } else if (kind == MV_TANGENT) {            /* move_funcs.pyx:470-582 */
        int64_t xang = rnd(g);
        double ang = c->amp_move * ((double)xang / OR_RAND_MAX - 0.5);
        float angf = (float)c->amp_move * (cgm_unif24((unsigned)xang) - 0.5f);
        float sang, cang;
        cgm_sincosf(angf, &sang, &cang);
        n = rnd(g) % c->amp_bead + 1;
        if (n > N) { g->err = OR_ERR_WINDOW; return g->err; }
        for (int64_t k = 0; k < n && !g->err; k++) {
            int64_t i;
            do { i = rnd(g) % N; } while (s->picked[i] && !g->err);
            s->picked[i] = 1;
            s->inds[k] = i;
        }
        for (int64_t k = 0; k < n; k++) s->picked[s->inds[k]] = 0;
        if (g->err) return g->err;
        static const double origin[3] = {0, 0, 0};
        for (int64_t k = 0; k < n; k++) {      /* rotate_select_beads, :517-549 */
            double axis[3], M[3][4], t3[3], t2[3];
            int64_t i = s->inds[k];
            if (emu32(s)) {
                sphere_f32(g, axis);
                axis_rotation_f32(axis, origin, sang, cang, M);
            } else {
                sphere(g, axis);
                axis_rotation(axis, origin, ang, M, !s->fixed_density);
            }
            ld3(s->t3, i, t3); ld3(s->t2, i, t2);
            for (int j = 0; j < 3; j++) {
                if (emu32(s)) {
                    float e3 = 0, e2 = 0;
                    for (int q = 0; q < 3; q++) {
                        e3 += (float)M[j][q] * (float)t3[q];
                        e2 += (float)M[j][q] * (float)t2[q];
                    }
                    s->trial[9 * k + 3 + j] = (double)e3;
                    s->trial[9 * k + 6 + j] = (double)e2;
                } else {
                    double e3 = 0, e2 = 0;
                    for (int q = 0; q < 3; q++) { e3 += M[j][q] * t3[q]; e2 += M[j][q] * t2[q]; }
                    s->trial[9 * k + 3 + j] = rnd_pos(e3);
                    s->trial[9 * k + 6 + j] = rnd_pos(e2);
                }
                s->trial[9 * k + j] = (double)s->r[3 * i + j];
            }
        }
        if (g->err) return g->err;
        /* SSWLC.compute_dE tangent branch, polymers.pyx:1074-1080 */
        for (int64_t k = 0; k < n; k++)
            dEp += continuous_dE(s, s->inds[k], s->inds[k] + 1, s->trial + 9 * k, s->trial + 9 * k);
        ind0 = s->inds[0]; indf = s->inds[0] + 1;
    } else {                                    /* change_binding_state, move_funcs.pyx:717-820 */
        bsel = rnd(g) % nb;
        int64_t b0 = rnd(g) % N;
        int64_t b1 = from_point(g, c->amp_bead, N, b0);
        if (g->err) return g->err;
        check_bead_bounds(b0, b1, N, &ind0, &indf);
        n = indf - ind0;
        for (int64_t k = 0; k < n; k++) {
            s->inds[k] = ind0 + k;
            s->new_states[k] = rnd_state(g, s->sites[bsel]);
            for (int j = 0; j < 3; j++) s->trial[9 * k + j] = (double)s->r[3 * (ind0 + k) + j];
        }
        if (g->err) return g->err;
        if (n == 0) goto empty;
        /* binding_dE, polymers.pyx:1383-1406 */
        for (int64_t k = 0; k < n; k++) {
            int64_t st[OR_MAXB];
            for (int64_t b = 0; b < nb; b++) st[b] = s->states[(ind0 + k) * nb + b];
            st[bsel] = s->new_states[k];
            dEp += bead_binding_dE(s, ind0 + k, st);
        }
        if (check_field) dEf = field_dE(s, n, 1, bsel);
    }
    {
        double dE = 0;
        dE += dEp;
        dE += dEf;
        double ex = exp(-dE);
        double u = rndu(g);
        int acc = u < ex;
        if (g->err) return g->err;
        if (forced >= 0 && forced != acc && fabs(dE + log(u)) <= 1e-5 * fmax(1.0, fabs(dE))) {
            acc = forced;
            g->ties++;
        }
        if (acc) {
            if (kind == MV_BINDING) {
                for (int64_t k = 0; k < n; k++) s->states[s->inds[k] * nb + bsel] = s->new_states[k];
            } else {
                for (int64_t k = 0; k < n; k++) {
                    int64_t i = s->inds[k];
                    for (int j = 0; j < 3; j++) {
                        if (kind != MV_TANGENT) s->r[3 * i + j] = (OR_POS)s->trial[9 * k + j];
                        if (kind != MV_SLIDE) {
                            s->t3[3 * i + j] = (OR_POS)s->trial[9 * k + 3 + j];
                            s->t2[3 * i + j] = (OR_POS)s->trial[9 * k + 6 + j];
                        }
                    }
                }
            }
            c->num_success += 1;
        }
        if (check_field && s->field_kind == 2) field_commit(s, acc);
        c->acc_rate = c->alpha * (acc ? 1.0 : 0.0) + (1 - c->alpha) * c->acc_rate;
        if (rec) {
            rec->kind = kind; rec->n_inds = (int32_t)n; rec->ind0 = (int32_t)ind0; rec->indf = (int32_t)indf;
            rec->dE_poly = dEp; rec->dE_field = dEf; rec->accepted = acc;
            rec->n_draws = (int32_t)(g->pos - draw0);
        }
        return n;
    }
empty:
    if (rec) {
        rec->kind = kind; rec->n_inds = 0; rec->ind0 = (int32_t)ind0; rec->indf = (int32_t)indf;
        rec->dE_poly = 0; rec->dE_field = 0; rec->accepted = -1;
        rec->n_draws = (int32_t)(g->pos - draw0);
    }
    return 0;
}

/* SimpleControl.update_move_amplitude / update_bead_amplitude,
 * mc_controller.py:126-189 (setpoint 0.5, factor 0.95, one bead) */
static void update_amplitudes(or_ctl *c)
{
    if (c->ctrl_kind != 1) return;
    double acc = c->acc_rate;
    if (acc < 0.5) {
        double prop = c->amp_move * 0.95;
        if (prop > c->move_lo) c->amp_move = prop;
        else {
            c->amp_move = c->move_hi;
            double nb = (double)(c->amp_bead - 1);
            c->amp_bead = (int64_t)(c->bead_lo > nb ? c->bead_lo : nb);
        }
    } else if (acc > 0.5) {
        double prop = c->amp_move / 0.95;
        if (prop < c->move_hi) c->amp_move = prop;
        else {
            c->amp_move = c->move_lo;
            double nb = (double)(c->amp_bead + 1);
            c->amp_bead = (int64_t)(c->bead_hi < nb ? c->bead_hi : nb);
        }
    }
}

/* The step loop of mc_sim, mc_sim.pyx:88-103 (one polymer); follow as in
 * mc_step, indexed by record. */
static int64_t mc_loop(or_system *s, or_ctl *ctl, int64_t n_ctl, int64_t n_steps, or_rng *g,
                       const int8_t *follow, int64_t n_follow, or_record *recs, int64_t max_recs)
{
    int64_t nrec = 0;
    for (int64_t k = 0; k < n_steps; k++) {
        for (int64_t ci = 0; ci < n_ctl; ci++) {
            or_ctl *c = &ctl[ci];
            if (c->move_on == 1) {
                for (int64_t j = 0; j < c->num_per_cycle; j++) {
                    or_record *rec = (recs && nrec < max_recs) ? &recs[nrec] : NULL;
                    int forced = (follow && nrec < n_follow) ? follow[nrec] : -1;
                    if (g->philox) { g->pos = 0; g->bpos = 0; }
                    int64_t r = mc_step(s, c, g, rec, forced);
                    if (r < 0) return r;
                    nrec++;
                    if (g->philox) g->t++;
                }
            }
            update_amplitudes(c);
        }
    }
    return nrec;
}

/* mc_sim, mc_sim.pyx:26-103 (one polymer).  Returns the number of records
 * written (attempted moves) or a negative error code. */
int64_t or_mc_sim(or_system *s, or_ctl *ctl, int64_t n_ctl, int64_t n_steps,
                  const uint32_t *draws, int64_t n_draws, int64_t *draw_pos,
                  const int64_t *bstates, int64_t n_bstates, int64_t *bstate_pos,
                  or_record *recs, int64_t max_recs)
{
    or_rng g;
    memset(&g, 0, sizeof g);
    g.a = draws; g.n = n_draws; g.pos = *draw_pos;
    g.b = bstates; g.nb_ = n_bstates; g.bpos = *bstate_pos;
    int64_t r = mc_loop(s, ctl, n_ctl, n_steps, &g, NULL, 0, recs, max_recs);
    *draw_pos = g.pos;
    *bstate_pos = g.bpos;
    return r;
}

/* mc_sim driven by the GPU production kernel's random numbers (see or_rng):
 * replica `rep` of a run seeded with `seed`, starting at move counter
 * *move_pos (advanced by the attempted moves).  follow (n_follow entries, or
 * NULL) holds the followed run's decisions per attempted move (1, 0, -1 for an
 * empty move); *ties receives how many tie-band decisions were taken from it. */
int64_t or_mc_sim_philox(or_system *s, or_ctl *ctl, int64_t n_ctl, int64_t n_steps, uint64_t seed,
                         int32_t rep, int64_t *move_pos, const int8_t *follow, int64_t n_follow,
                         int64_t *ties, or_record *recs, int64_t max_recs)
{
    or_rng g;
    memset(&g, 0, sizeof g);
    g.philox = 1;
    g.key[0] = (uint32_t)seed ^ ((uint32_t)rep * 0x85EBCA6Bu);
    g.key[1] = (uint32_t)(seed >> 32) ^ 0x1B873593u;
    g.keyb[0] = g.key[0] ^ 0x68E31DA4u;
    g.keyb[1] = g.key[1] ^ 0xB5297A4Du;
    g.t = (uint64_t)*move_pos;
    int64_t r = mc_loop(s, ctl, n_ctl, n_steps, &g, follow, n_follow, recs, max_recs);
    *move_pos = (int64_t)g.t;
    if (ties) *ties = g.ties;
    return r;
}

/* Known-answer hook: one Philox4x32-10 block (test infrastructure). */
void or_kat_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    or_philox(ctr, key, out);
}

/* size helpers for the ctypes wrapper */
/* Known-answer hooks (test infrastructure): the rotation about axis a through
 * p (arbitrary_axis_rotation, linalg.pyx:62-143) in the reference's
 * arithmetic, as the 3 x 4 matrix [R | T] row by row, and the transform of
 * bead i of s by such a matrix (transform_r_t3_t2, move_funcs.pyx:121-154):
 * out = r', t3', t2'. */
void or_kat_axis_rotation(const double a[3], const double p[3], double ang, double out[12])
{
    double M[3][4];
    axis_rotation(a, p, ang, M, 1);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 4; j++) out[4 * i + j] = M[i][j];
}

void or_kat_transform(const or_system *s, int64_t i, const double M12[12], double out[9])
{
    double M[3][4];
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 4; b++) M[a][b] = M12[4 * a + b];
    transform_bead(s, i, M, out);
}

int64_t or_sizeof_system(void) { return (int64_t)sizeof(or_system); }
int64_t or_sizeof_ctl(void) { return (int64_t)sizeof(or_ctl); }
int64_t or_sizeof_record(void) { return (int64_t)sizeof(or_record); }
int64_t or_pos_bytes(void) { return (int64_t)sizeof(OR_POS); }

/* ---------------- steric clashes: chromo/polymers.pyx:2738-2938 ----------- */

/* Clash energy of one pair at distance d: V0 ((e/d)^12 - 2 (e/d)^6 + 1)
 * when d < e (the excluded distance, twice the bead radius), else 0
 * (eval_delta_steric_clashes / eval_E_steric_clashes; Cython pow for **). */
static double clash(double d, double e, double V0)
{
    if (!(d < e)) return 0.0;
    double f = e / d;
    return V0 * (pow(f, 12.0) - 2 * pow(f, 6.0) + 1);
}

static double pair_dist(const double *a, const double *b)
{
    return sqrt(pow(a[0] - b[0], 2.0) + pow(a[1] - b[1], 2.0) + pow(a[2] - b[2], 2.0));
}

/* eval_E_steric_clashes, polymers.pyx:2900-2920: every pair i < j. r: N x 3. */
double or_steric_E(const double *r, int64_t n, double e, double V0)
{
    double E = 0;
    for (int64_t i = 0; i < n; i++)
        for (int64_t j = i + 1; j < n; j++) E += clash(pair_dist(r + 3 * i, r + 3 * j), e, V0);
    return E;
}

/* get_delta_distances + eval_delta_steric_clashes, polymers.pyx:2827-2898:
 * beads [ind0, indf) move to rt (m x 3); pairs (i moved, j any) counted once
 * (j >= i inside the moved range skipped); trial minus current. */
double or_steric_dE(const double *r, const double *rt, int64_t n, int64_t ind0, int64_t indf, double e,
                    double V0)
{
    double dE = 0;
    for (int64_t i = ind0; i < indf; i++) {
        const double *pi_t = rt + 3 * (i - ind0), *pi = r + 3 * i;
        for (int64_t j = 0; j < n; j++) {
            if (j >= i && j >= ind0 && j < indf) continue;
            const double *pj_t = (j >= ind0 && j < indf) ? rt + 3 * (j - ind0) : r + 3 * j;
            double dt = (i == j) ? 0.0 : pair_dist(pi_t, pj_t);
            double dc = (i == j) ? 0.0 : pair_dist(pi, r + 3 * j);
            dE += clash(dt, e, V0);
            dE -= clash(dc, e, V0);
        }
    }
    return dE;
}
