// cg_capi.cu -- host side of the C ABI declared in include/chromo_gb300.h.
//
// Owns the device buffers of a cg_sim, converts host FP64 / int64 arrays to
// the resident layout (V4 positions in FP32 or FP64, packed int8 binder
// states, int64 fixed-point grid), sizes the per-warp shared-memory region
// and launches the kernels of cg_mc.cu.
#include <cuda_runtime.h>
#include <cstdlib>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <atomic>
#include <string>
#include <thread>
#include <vector>

#include "cg_kernels.h"

using cg::KArgs;
using cg::RepDev;
template <typename T> using V4 = cg::V4<T>;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

#define CUDA_TRY(x)                                                                 \
  do {                                                                              \
    cudaError_t e_ = (x);                                                           \
    if (e_ != cudaSuccess)                                                          \
      return fail(CG_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_));    \
  } while (0)

size_t align16(size_t x) { return (x + 15) & ~size_t(15); }
size_t align32(size_t x) { return (x + 31) & ~size_t(31); }

int next_log2(long long x) {
  int l = 0;
  while ((1LL << l) < x) l++;
  return l;
}

}  // namespace

struct cg_sim {
  int R = 0, nb = 0, ncol = 0, fp64 = 0, wpb = 1, n_sm = 0, nonuniform = 0;
  std::vector<long long> n_beads, bead_off, n_vox, vox_off, picked_off;
  std::vector<int> dims;
  long long total_beads = 0, total_vox = 0, total_picked = 0;
  long long max_segment = 0, max_tangent = 0, max_beads = 0, max_vox = 0;
  int n_ctl = 5;
  long long kernels = 0;
  // device buffers
  RepDev* reps = nullptr;
  cg_move_ctl* ctl = nullptr;
  unsigned long long* tally = nullptr;
  void *r4 = nullptr, *t34 = nullptr, *t24 = nullptr;
  unsigned *states = nullptr, *marks = nullptr;
  double* bonds = nullptr;
  float* bonds32 = nullptr;  // FP32 copy, 8 floats per bead: eb, g, ep, epp, eta, pad
  long long* grid = nullptr;
  double* access_vol = nullptr;
  // per voxel, from the accessible volume V: the FP32 density scale
  // 2^-40 / V and V / bead volume (the chi term's factor without chi)
  float* access_sc = nullptr;
  double* access_vb = nullptr;
  int *g_keys = nullptr, *g_used = nullptr, *g_bslot = nullptr;
  long long* g_vals = nullptr;
  int g_logH = 0;
  void* g_stage = nullptr;
  int* g_idx = nullptr;
  long long g_stage_cap = 0;
  unsigned* picked = nullptr;
  long long* d_picked_off = nullptr;
  double* eout = nullptr;
  long long* aout = nullptr;
  int* rep_of_rung = nullptr;
  unsigned long long *swaps = nullptr, *swap_attempts = nullptr, *xround = nullptr;
  int mu_rungs = 0, mu_binder = 0;
  double* nbound = nullptr;
  unsigned long long *mu_swaps = nullptr, *mu_swap_attempts = nullptr;
  // shared-memory layout
  int logH = 0, warp_smem = 0, off_draws = 0, off_keys = 0, off_used = 0, off_bslot = 0, off_vals = 0, off_stage = 0,
      off_idx = 0;
  int spec_w = 1, spec_g = 32, spec_s = 1, spec_logHB = 11, spec_off_bkeys = 0, spec_off_bmask = 0, spec_off_warps = 0;
  int pool_on = 0, pool_logH = 0, off_pkeys = 0, off_pused = 0, off_pvals = 0;
  long long stage_cap = 0;
  size_t spec_bytes = 0;
  // captured batched graph
  cudaGraphExec_t graph = nullptr;
  cudaGraph_t graph_src = nullptr;  // kept while its timing nodes are re-pointed per launch
  long long graph_rounds = -1, graph_steps = -1;
  int graph_rungs = -1;
  unsigned long long graph_seed = 0;
  cudaStream_t graph_stream = nullptr;
  // per-round timing of the MC kernel inside the graph (cg_set_round_timing):
  // ring of timing_cap event pairs; each captured round's two event-record
  // nodes are pointed at the next pair before every launch
  int timing_cap = 0;
  long long timing_count = 0;
  std::vector<cudaEvent_t> tev_begin, tev_end;
  std::vector<cudaEvent_t> cap_begin, cap_end;  // events the nodes were captured with
  std::vector<cudaGraphNode_t> tnode_begin, tnode_end;

  void drop_graph() {
    if (graph) cudaGraphExecDestroy(graph);
    if (graph_src) cudaGraphDestroy(graph_src);
    graph = nullptr;
    graph_src = nullptr;
    for (cudaEvent_t e : cap_begin) cudaEventDestroy(e);
    for (cudaEvent_t e : cap_end) cudaEventDestroy(e);
    cap_begin.clear(); cap_end.clear(); tnode_begin.clear(); tnode_end.clear();
  }
  void drop_timing() {
    drop_graph();
    for (cudaEvent_t e : tev_begin) cudaEventDestroy(e);
    for (cudaEvent_t e : tev_end) cudaEventDestroy(e);
    tev_begin.clear(); tev_end.clear();
    timing_cap = 0;
    timing_count = 0;
  }
  double* twist = nullptr;  // SSTWLC bond parameters (cg_set_twist), allocated on first use
  double* steric_work = nullptr;  // steric clash rows, trial segment and total (allocated on first use)
  long long steric_cap = 0;
  // drift guard of the batched rounds (cg_set_drift_guard)
  int guard_every = 0, guard_chunks = 1;
  double guard_tol_abs = 0, guard_tol_rel = 0;
  double *guard_partial = nullptr, *guard_e_ref = nullptr, *guard_run_ref = nullptr, *guard_drift = nullptr;
  int* guard_init = nullptr;
  unsigned long long* guard_counter = nullptr;
  cg::GuardArgs guard_args() const {
    cg::GuardArgs g{};
    g.every = guard_every; g.chunks = guard_chunks; g.tol_abs = guard_tol_abs; g.tol_rel = guard_tol_rel;
    g.partial = guard_partial; g.e_ref = guard_e_ref; g.run_ref = guard_run_ref; g.drift = guard_drift;
    g.init = guard_init; g.counter = guard_counter;
    return g;
  }
  void free_guard() {
    void* ptrs[] = {guard_partial, guard_e_ref, guard_run_ref, guard_drift, guard_init, guard_counter};
    for (void* p : ptrs)
      if (p) cudaFree(p);
    guard_partial = guard_e_ref = guard_run_ref = guard_drift = nullptr;
    guard_init = nullptr;
    guard_counter = nullptr;
    guard_every = 0;
  }
  // derivatives: per-bead gradient, per-replica terms, running sums (allocated on first use)
  float* grad = nullptr;
  double* terms = nullptr;
  double* acc = nullptr;
  // pinned host staging for chain uploads / downloads
  void* pinned = nullptr;
  size_t pinned_bytes = 0;
  // direct host access (cudaDevAttrPageableMemoryAccess): cg_set_chains /
  // cg_get_chains read and write the caller's arrays from the GPU; the
  // replica table of host pointers and the upload check flag live here
  int direct_host = 0;
  void* hio_tab = nullptr;
  unsigned* hio_flag = nullptr;
  // replicas using SSTWLC twist (the MC kernel's full form); with none,
  // launches take its lean form
  std::vector<unsigned char> full_of;
  long long n_full = 0;
  void note_features(int rep, const RepDev& d) {
    const unsigned char f = d.twist != 0;
    if (f == full_of[rep]) return;
    const bool was_lean = n_full == 0;
    n_full += f ? 1 : -1;
    full_of[rep] = f;
    if (was_lean != (n_full == 0)) drop_graph();  // the captured launches' form changes
  }
  // device staging arrays of a direct upload (resident layout; allocated on
  // the first upload, hio_stage_failed when there was no room)
  void *hio_r4 = nullptr, *hio_t34 = nullptr, *hio_t24 = nullptr;
  unsigned* hio_states = nullptr;
  int hio_stage_failed = 0;
  bool upload_stage() {
    if (hio_r4) return true;
    if (hio_stage_failed) return false;
    const size_t pb = pos_bytes() * (size_t)total_beads;
    void* p[4] = {nullptr, nullptr, nullptr, nullptr};
    const size_t bytes[4] = {pb, pb, pb, 4 * (size_t)total_beads};
    bool ok = true;
    for (int k = 0; k < 4 && ok; k++) ok = cudaMalloc(&p[k], bytes[k] == 0 ? 16 : bytes[k]) == cudaSuccess;
    for (int k = 0; k < 4 && ok; k++) ok = cudaMemset(p[k], 0, bytes[k] == 0 ? 16 : bytes[k]) == cudaSuccess;
    if (!ok) {
      for (void* q : p)
        if (q) cudaFree(q);
      cudaGetLastError();  // the failed allocation is not an error of a later call
      hio_stage_failed = 1;
      return false;
    }
    hio_r4 = p[0]; hio_t34 = p[1]; hio_t24 = p[2]; hio_states = static_cast<unsigned*>(p[3]);
    return true;
  }

  unsigned char* staging(size_t bytes) {
    if (bytes > pinned_bytes) {
      if (pinned) cudaFreeHost(pinned);
      pinned = nullptr;
      pinned_bytes = 0;
      if (cudaHostAlloc(&pinned, bytes, cudaHostAllocDefault) != cudaSuccess) return nullptr;
      pinned_bytes = bytes;
    }
    return static_cast<unsigned char*>(pinned);
  }

  size_t pos_bytes() const { return fp64 ? sizeof(V4<double>) : sizeof(V4<float>); }
  size_t scal_bytes() const { return fp64 ? 8 : 4; }

  KArgs args() const {
    KArgs a{};
    a.reps = reps; a.ctl = ctl; a.n_ctl = n_ctl; a.n_reps = R; a.tally = tally;
    a.r4 = r4; a.t34 = t34; a.t24 = t24; a.states = states; a.marks = marks; a.bonds = bonds;
    a.bonds32 = bonds32;
    a.twist = twist;
    a.grid = grid; a.access_vol = access_vol; a.access_sc = access_sc; a.access_vb = access_vb;
    a.ncol = ncol; a.hcol = nb + 1;
    a.g_keys = g_keys; a.g_used = g_used; a.g_bslot = g_bslot; a.g_vals = g_vals; a.g_logH = g_logH;
    a.g_stage = g_stage; a.g_idx = g_idx; a.g_stage_cap = g_stage_cap;
    a.picked = picked; a.picked_off = d_picked_off;
    a.wpb = wpb; a.logH = logH; a.stage_cap = stage_cap; a.warp_smem = warp_smem; a.off_draws = off_draws;
    a.off_keys = off_keys; a.off_used = off_used; a.off_vals = off_vals; a.off_stage = off_stage;
    a.off_idx = off_idx; a.off_bslot = off_bslot;
    a.spec_w = spec_w; a.spec_g = spec_g; a.spec_s = spec_s; a.spec_logHB = spec_logHB; a.spec_off_bkeys = spec_off_bkeys;
    a.spec_off_bmask = spec_off_bmask; a.spec_off_warps = spec_off_warps;
    a.pool_on = pool_on; a.pool_logH = pool_logH; a.off_pkeys = off_pkeys; a.off_pused = off_pused;
    a.off_pvals = off_pvals;
    a.rep_of_rung = rep_of_rung; a.swaps = swaps; a.swap_attempts = swap_attempts;
    a.xround = xround;
    a.mu_rungs = mu_rungs; a.mu_binder = mu_binder; a.nbound = nbound;
    a.mu_swaps = mu_swaps; a.mu_swap_attempts = mu_swap_attempts;
    a.lean = n_full == 0 ? 1 : 0;
    return a;
  }

  // Region of one move slot for voxel-table capacity 2^lh and staging
  // capacity sc (offsets within the region; the draw buffer first, 16-byte
  // aligned; the staged 4-vectors 32-byte aligned); returns the region size,
  // a multiple of 32 bytes.
  int layout(int lh, long long sc) {
    size_t H = size_t(1) << lh;
    size_t o = 0;
    off_draws = (int)o; o += 4 * cg::kDrawCache;
    off_keys = (int)o; o += 4 * H;
    off_used = (int)o; o += 4 * H;
    off_bslot = (int)o; o += 4 * H;
    o = align16(o);
    off_vals = (int)o; o += 8 * H * (nb + 1);
    o = align32(o);  // staged 4-vectors: 16 bytes (FP32) or 32 bytes (FP64) each
    off_stage = (int)o; o += sc * 12 * scal_bytes();
    o = align16(o);
    off_idx = (int)o; o += 4 * sc;
    o = align32(o);
    logH = lh; stage_cap = sc; warp_smem = (int)o;
    return warp_smem;
  }
  // CTA layout: header, block voxel table (2^lhb entries), the pooled voxel
  // table (2^lhp entries: keys, used list, nb + 1 split int64 values; none
  // for lhp = 0), one region per move slot (W warps of 32 / G slots).
  size_t cta_layout(int lhb, int W, int G, int lhp = 0) {
    size_t o = align16(sizeof(cg::SpecShared));
    spec_off_bkeys = (int)o; o += 4 * (size_t(1) << lhb);
    spec_off_bmask = (int)o; o += 4 * (size_t(1) << lhb);
    o = align32(o);
    pool_on = lhp > 0 ? 1 : 0;
    pool_logH = lhp;
    off_pkeys = off_pused = off_pvals = 0;
    if (lhp > 0) {
      const size_t HP = size_t(1) << lhp;
      off_pkeys = (int)o; o += 4 * HP;
      off_pused = (int)o; o += 4 * HP;
      o = align16(o);
      off_pvals = (int)o; o += 8 * HP * (nb + 1);
      o = align32(o);
    }
    spec_off_warps = (int)o;
    spec_logHB = lhb;
    spec_w = W;
    spec_g = G;
    spec_s = W * (32 / G);
    return o + (size_t)spec_s * warp_smem;
  }
};

template <typename P>
static void pack_pos(const double* src, long long n, unsigned char* out) {
  V4<P>* o = reinterpret_cast<V4<P>*>(out);
  for (long long i = 0; i < n; i++) o[i] = V4<P>{(P)src[3 * i], (P)src[3 * i + 1], (P)src[3 * i + 2], (P)0};
}
template <typename P>
static void unpack_pos(const unsigned char* in, long long n, double* dst) {
  const V4<P>* o = reinterpret_cast<const V4<P>*>(in);
  for (long long i = 0; i < n; i++) {
    dst[3 * i] = (double)o[i].x; dst[3 * i + 1] = (double)o[i].y; dst[3 * i + 2] = (double)o[i].z;
  }
}

// Run f(rep) for every replica on up to hardware_concurrency() host threads
// (replicas taken in turn from a shared counter).
template <class F>
static void for_each_replica(int R, const F& f) {
  unsigned nt = std::thread::hardware_concurrency();
  if (nt < 1) nt = 1;
  if (nt > 32) nt = 32;
  if ((int)nt > R) nt = (unsigned)R;
  std::atomic<int> next(0);
  auto work = [&]() {
    for (int r = next.fetch_add(1); r < R; r = next.fetch_add(1)) f(r);
  };
  std::vector<std::thread> pool;
  for (unsigned t = 1; t < nt; t++) pool.emplace_back(work);
  work();
  for (auto& t : pool) t.join();
}

extern "C" {

const char* cg_last_error(void) { return g_err.c_str(); }

void cg_destroy(cg_sim* s) {
  if (!s) return;
  s->drop_timing();
  s->free_guard();
  if (s->pinned) cudaFreeHost(s->pinned);
  if (s->twist) cudaFree(s->twist);
  if (s->steric_work) cudaFree(s->steric_work);
  if (s->hio_tab) cudaFree(s->hio_tab);
  if (s->hio_flag) cudaFree(s->hio_flag);
  {
    void* stage[] = {s->hio_r4, s->hio_t34, s->hio_t24, s->hio_states};
    for (void* p : stage)
      if (p) cudaFree(p);
  }
  void* ptrs[] = {s->reps, s->ctl, s->tally, s->r4, s->t34, s->t24, s->states, s->marks, s->bonds,
                  s->bonds32, s->grid, s->access_vol, s->access_sc, s->access_vb, s->g_keys, s->g_used, s->g_bslot, s->g_vals, s->g_stage, s->g_idx,
                  s->picked, s->d_picked_off, s->eout, s->aout, s->rep_of_rung, s->swaps,
                  s->swap_attempts, s->xround, s->grad, s->terms, s->acc, s->nbound, s->mu_swaps,
                  s->mu_swap_attempts};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  delete s;
}

// Lanes per move when the caller leaves it to the library: 32 (the fastest
// shape measured on the batched benchmark workload; the autotuner picks
// others where they win), and always 32 for FP64 storage.
static int default_lanes(const cg_sim* s, int g_req) {
  if (s->fp64) return 32;
  return g_req > 0 ? g_req : 32;
}

// Warps per replica: the largest W <= kMaxW for which every replica's CTA is
// resident at once (ceil(R / SMs) CTAs per SM, W warps each, within the
// register file), and at most 32 moves in flight.
static int default_warps(const cg_sim* s, int G) {
  const long long ctas = (s->R + s->n_sm - 1) / std::max(1, s->n_sm);
  const long long W = cg_spec_warps_per_sm(s->fp64 != 0, G) / std::max(1LL, ctas);
  const long long wmax = std::min<long long>(cg::kMaxW, cg::kMaxS / (32 / G));
  return (int)std::min<long long>(wmax, std::max<long long>(1, W));
}

static int choose_shape(cg_sim* s, int w_req, int g_req) {
  // One CTA per replica with W warps of 32 / G moves each.  The CTAs that can
  // be resident per SM -- those every replica needs to run at once, or fewer
  // when the register file holds fewer CTAs of W warps (the replicas then run
  // in waves) -- share the SM's shared memory; each move slot gets the
  // largest voxel table that then fits.
  const size_t smem_per_sm = 227 * 1024;
  long long ctas_per_sm = (s->R + s->n_sm - 1) / std::max(1, s->n_sm);
  if (ctas_per_sm < 1) ctas_per_sm = 1;
  const int G = default_lanes(s, g_req);
  int W = w_req > 0 ? w_req : default_warps(s, G);
  if (W > cg::kMaxW) W = cg::kMaxW;
  if (W * (32 / G) > cg::kMaxS) W = cg::kMaxS / (32 / G);
  const long long reg_ctas = std::max(1, cg_spec_warps_per_sm(s->fp64 != 0, G) / W);
  if (ctas_per_sm > reg_ctas) ctas_per_sm = reg_ctas;
  const size_t budget = std::min<size_t>(smem_per_sm / ctas_per_sm - 1024, 220 * 1024);
  const int lhb = 10;
  const long long sc = G == 32 ? 48 : 32;
  // FP32 storage: the position moves of a batch share one pooled voxel table
  // (keys voxel * 32 + slot: grids below 2^26 voxels), as large as fits (up
  // to 4,096 entries); the slots keep 64-entry tables for binding moves
  int lhp = 0;
  if (!s->fp64 && s->max_vox < (1LL << 26)) {
    s->layout(6, sc);
    for (int t = 12; t >= 8 && lhp == 0; t--)
      if (s->cta_layout(lhb, W, G, t) <= budget) lhp = t;
  }
  int lh = 6;
  if (lhp == 0) {
    lh = 10;  // at most 1,024 slots: the 32-bit split counters of a shared table cannot overflow
    for (; lh > 6; lh--) {
      s->layout(lh, sc);
      if (s->cta_layout(lhb, W, G) <= budget) break;
    }
  }
  s->layout(lh, sc);
  s->spec_bytes = s->cta_layout(lhb, W, G, lhp);
  s->wpb = 1;
  cudaError_t e = cg_set_spec_smem(s->fp64 != 0, G, (int)s->spec_bytes);
  if (e == cudaSuccess) e = cg_set_mc_smem(s->fp64 != 0, (int)(s->spec_off_warps + s->warp_smem));
  if (e != cudaSuccess) return fail(CG_ERR_CUDA, std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(e));
  return CG_OK;
}

int cg_create(const cg_config* cfg, cg_sim** out) {
  if (!cfg || !out) return fail(CG_ERR_ARG, "null argument");
  if (cfg->n_replicas < 1) return fail(CG_ERR_ARG, "n_replicas must be >= 1");
  if (cfg->n_binders < 1 || cfg->n_binders > CG_MAX_BINDERS)
    return fail(CG_ERR_ARG, "n_binders must be in 1..3");
  cg_sim* s = new cg_sim();
  s->R = cfg->n_replicas;
  s->full_of.assign(s->R, 0);
  s->nb = cfg->n_binders;
  s->ncol = cfg->n_binders + 1 <= 2 ? 2 : 4;
  s->fp64 = cfg->pos_fp64 ? 1 : 0;
  s->nonuniform = cfg->nonuniform_access ? 1 : 0;
  s->max_segment = std::max<long long>(cfg->max_segment, 2);
  s->max_tangent = std::max<long long>(cfg->max_tangent, 1);
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&s->n_sm, cudaDevAttrMultiProcessorCount, dev);
  for (int r = 0; r < s->R; r++) {
    long long n = cfg->n_beads[r];
    if (n < 2) { cg_destroy(s); return fail(CG_ERR_ARG, "every chain needs at least 2 beads"); }
    if (n > 2000000000LL) { cg_destroy(s); return fail(CG_ERR_ARG, "chains are limited to 2e9 beads"); }
    int nx = cfg->grid_dims[3 * r], ny = cfg->grid_dims[3 * r + 1], nz = cfg->grid_dims[3 * r + 2];
    if (nx < 1 || ny < 1 || nz < 1) { cg_destroy(s); return fail(CG_ERR_ARG, "grid dims must be >= 1"); }
    if ((long long)nx * ny * nz > (1LL << 30)) { cg_destroy(s); return fail(CG_ERR_ARG, "grid too large"); }
    s->n_beads.push_back(n);
    s->bead_off.push_back(s->total_beads);
    s->total_beads += n;
    s->dims.insert(s->dims.end(), {nx, ny, nz});
    s->n_vox.push_back((long long)nx * ny * nz);
    s->vox_off.push_back(s->total_vox);
    s->total_vox += (long long)nx * ny * nz;
    s->picked_off.push_back(s->total_picked);
    s->total_picked += (n + 31) / 32;
    s->max_beads = std::max(s->max_beads, n);
    s->max_vox = std::max(s->max_vox, (long long)nx * ny * nz);
  }
  s->g_logH = next_log2(32 * s->max_segment);
  s->g_stage_cap = std::max(s->max_segment, s->max_tangent);
  const long long Hg = 1LL << s->g_logH;
  if (cfg->lanes_per_move != 0 && !cg_spec_shape_ok(s->fp64 != 0, cfg->lanes_per_move)) {
    cg_destroy(s);
    return fail(CG_ERR_ARG, "lanes_per_move must be 8, 16 or 32 (32 with FP64 storage)");
  }
  if (cfg->warps_per_block < 0 || cfg->warps_per_block > cg::kMaxW) {
    cg_destroy(s);
    return fail(CG_ERR_ARG, "warps_per_block must be in 0..12");
  }
  {
    const int G = default_lanes(s, cfg->lanes_per_move);
    int W = cfg->warps_per_block > 0 ? cfg->warps_per_block : default_warps(s, G);
    if (W * (32 / G) > cg::kMaxS) W = cg::kMaxS / (32 / G);
    s->spec_w = W;
    s->spec_g = G;
    s->spec_s = W * (32 / G);
  }
  const long long RW = (long long)s->R * s->spec_s;
  // tangent-rotation bitmaps: one per (replica, move slot)
  s->total_picked = 0;
  for (int r = 0; r < s->R; r++) {
    s->picked_off[r] = s->total_picked;
    s->total_picked += (long long)s->spec_s * ((s->n_beads[r] + 31) / 32);
  }
  auto M = [&](void** p, size_t bytes) { return cudaMalloc(p, bytes == 0 ? 16 : bytes); };
  cudaError_t e = cudaSuccess;
#define ALLOC(ptr, bytes) if (e == cudaSuccess) e = M((void**)&(ptr), (bytes))
  ALLOC(s->reps, sizeof(RepDev) * s->R);
  ALLOC(s->ctl, sizeof(cg_move_ctl) * 5 * s->R);
  ALLOC(s->tally, sizeof(unsigned long long) * 30 * s->R);
  ALLOC(s->r4, s->pos_bytes() * s->total_beads);
  ALLOC(s->t34, s->pos_bytes() * s->total_beads);
  ALLOC(s->t24, s->pos_bytes() * s->total_beads);
  ALLOC(s->states, 4 * s->total_beads);
  ALLOC(s->marks, 4 * s->total_beads);
  ALLOC(s->bonds, 6 * 8 * s->total_beads);
  ALLOC(s->bonds32, 8 * 4 * s->total_beads);
  ALLOC(s->grid, 8 * s->ncol * s->total_vox);
  if (s->nonuniform) ALLOC(s->access_vol, 8 * s->total_vox);
  if (s->nonuniform) ALLOC(s->access_sc, 4 * s->total_vox);
  if (s->nonuniform) ALLOC(s->access_vb, 8 * s->total_vox);
  ALLOC(s->g_keys, 4 * Hg * RW);
  ALLOC(s->g_used, 4 * Hg * RW);
  ALLOC(s->g_bslot, 4 * Hg * RW);
  ALLOC(s->g_vals, 8 * Hg * (s->nb + 1) * RW);
  ALLOC(s->g_stage, s->scal_bytes() * 12 * s->g_stage_cap * RW);
  ALLOC(s->g_idx, 4 * s->g_stage_cap * RW);
  ALLOC(s->picked, 4 * s->total_picked);
  ALLOC(s->d_picked_off, 8 * s->R);
  ALLOC(s->eout, 8 * 5 * s->R);
  ALLOC(s->aout, 8 * 4);
  ALLOC(s->rep_of_rung, 4 * s->R);
  ALLOC(s->swaps, 8 * s->R);
  ALLOC(s->swap_attempts, 8 * s->R);
  ALLOC(s->xround, 8);
  ALLOC(s->nbound, 8 * s->R);
  ALLOC(s->mu_swaps, 8 * s->R);
  ALLOC(s->mu_swap_attempts, 8 * s->R);
  {
    // chains move between the caller's arrays and the device in one kernel
    // pass where the GPU can address pageable host memory (Grace-Blackwell
    // NVLink-C2C); CHROMO_GB300_STAGED_HOST_IO=1 keeps the staged path
    int pageable = 0;
    cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev);
    const char* env = std::getenv("CHROMO_GB300_STAGED_HOST_IO");
    s->direct_host = pageable == 1 && s->R <= 65535 && !(env && env[0] == '1');
  }
  if (s->direct_host) ALLOC(s->hio_tab, 4 * sizeof(void*) * s->R);
  if (s->direct_host) ALLOC(s->hio_flag, sizeof(unsigned));
#undef ALLOC
  if (e != cudaSuccess) {
    cg_destroy(s);
    return fail(CG_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  }
  cudaMemset(s->reps, 0, sizeof(RepDev) * s->R);
  cudaMemset(s->ctl, 0, sizeof(cg_move_ctl) * 5 * s->R);
  cudaMemset(s->tally, 0, 8 * 30 * s->R);
  cudaMemset(s->r4, 0, s->pos_bytes() * s->total_beads);
  cudaMemset(s->t34, 0, s->pos_bytes() * s->total_beads);
  cudaMemset(s->t24, 0, s->pos_bytes() * s->total_beads);
  cudaMemset(s->states, 0, 4 * s->total_beads);
  cudaMemset(s->marks, 0, 4 * s->total_beads);
  cudaMemset(s->bonds, 0, 48 * s->total_beads);
  cudaMemset(s->bonds32, 0, 32 * s->total_beads);
  cudaMemset(s->grid, 0, 8 * s->ncol * s->total_vox);
  cudaMemset(s->g_keys, 0xFF, 4 * Hg * RW);
  cudaMemset(s->g_bslot, 0xFF, 4 * Hg * RW);
  cudaMemset(s->g_vals, 0, 8 * Hg * (s->nb + 1) * RW);
  cudaMemset(s->picked, 0, 4 * s->total_picked);
  cudaMemset(s->swaps, 0, 8 * s->R);
  cudaMemset(s->swap_attempts, 0, 8 * s->R);
  cudaMemset(s->xround, 0, 8);
  cudaMemset(s->nbound, 0, 8 * s->R);
  cudaMemset(s->mu_swaps, 0, 8 * s->R);
  cudaMemset(s->mu_swap_attempts, 0, 8 * s->R);
  cudaMemcpy(s->d_picked_off, s->picked_off.data(), 8 * s->R, cudaMemcpyHostToDevice);
  std::vector<int> ror(s->R);
  for (int r = 0; r < s->R; r++) ror[r] = r;
  cudaMemcpy(s->rep_of_rung, ror.data(), 4 * s->R, cudaMemcpyHostToDevice);
  std::vector<RepDev> rd(s->R);
  for (int r = 0; r < s->R; r++) {
    RepDev& d = rd[r];
    memset(&d, 0, sizeof(d));
    d.bead_off = s->bead_off[r];
    d.n_beads = s->n_beads[r];
    d.vox_off = s->vox_off[r];
    d.n_vox = s->n_vox[r];
    d.nx = s->dims[3 * r]; d.ny = s->dims[3 * r + 1]; d.nz = s->dims[3 * r + 2];
    d.nb = s->nb;
    d.wx = d.wy = d.wz = 1.0;
    d.dx = d.dy = d.dz = 1.0;
    d.vol_bin = 1.0;
    d.max_binders = -1;
    d.vf_limit = 0.5;
    d.mu_adjust = 1.0;
  }
  cudaMemcpy(s->reps, rd.data(), sizeof(RepDev) * s->R, cudaMemcpyHostToDevice);
  e = cudaGetLastError();
  if (e != cudaSuccess) { cg_destroy(s); return fail(CG_ERR_CUDA, cudaGetErrorString(e)); }
  int rc = choose_shape(s, s->spec_w, s->spec_g);
  if (rc) { cg_destroy(s); return rc; }
  *out = s;
  return CG_OK;
}

static int check_rep(cg_sim* s, int rep) {
  if (!s) return fail(CG_ERR_ARG, "null sim");
  if (rep < 0 || rep >= s->R) return fail(CG_ERR_ARG, "replica index out of range");
  return CG_OK;
}

static int get_rep(cg_sim* s, int rep, RepDev* d) {
  CUDA_TRY(cudaMemcpy(d, s->reps + rep, sizeof(RepDev), cudaMemcpyDeviceToHost));
  return CG_OK;
}
static int put_rep(cg_sim* s, int rep, const RepDev* d) {
  CUDA_TRY(cudaMemcpy(s->reps + rep, d, sizeof(RepDev), cudaMemcpyHostToDevice));
  s->note_features(rep, *d);
  return CG_OK;
}

int cg_set_chain(cg_sim* s, int rep, const double* r, const double* t3, const double* t2,
                 const int64_t* states, const int64_t* marks, const double* bonds) {
  if (int rc = check_rep(s, rep)) return rc;
  const long long n = s->n_beads[rep], off = s->bead_off[rep];
  const double* src[3] = {r, t3, t2};
  void* dst[3] = {s->r4, s->t34, s->t24};
  unsigned char* buf = s->staging(s->pos_bytes() * n * 3 + 4 * n);
  if (!buf) return fail(CG_ERR_NOMEM, "pinned staging allocation failed");
  for (int k = 0; k < 3; k++) {
    if (!src[k]) continue;
    for (long long i = 0; i < 3 * n; i++)
      if (!std::isfinite(src[k][i])) return fail(CG_ERR_NONFINITE, "non-finite position or tangent");
    unsigned char* b = buf + s->pos_bytes() * n * k;
    if (s->fp64) pack_pos<double>(src[k], n, b);
    else pack_pos<float>(src[k], n, b);
    CUDA_TRY(cudaMemcpy((char*)dst[k] + s->pos_bytes() * off, b, s->pos_bytes() * n, cudaMemcpyHostToDevice));
  }
  unsigned* pk = reinterpret_cast<unsigned*>(buf + s->pos_bytes() * n * 3);
  const int64_t* sm[2] = {states, marks};
  unsigned* dsm[2] = {s->states, s->marks};
  for (int k = 0; k < 2; k++) {
    if (!sm[k]) continue;
    for (long long i = 0; i < n; i++) {
      unsigned w = 0;
      for (int b = 0; b < s->nb; b++) {
        int64_t v = sm[k][i * s->nb + b];
        if (v < 0 || v > CG_MAX_MARK)
          return fail(CG_ERR_ARG, k == 0 ? "binding states must be in 0..3" : "chemical_mods must be in 0..3");
        w |= (unsigned)v << (8 * b);
      }
      pk[i] = w;
    }
    CUDA_TRY(cudaMemcpy(dsm[k] + off, pk, 4 * n, cudaMemcpyHostToDevice));
  }
  if (bonds) {
    std::vector<double> bb(6 * n, 0.0);
    for (long long i = 0; i + 1 < n; i++)
      for (int j = 0; j < 5; j++) bb[6 * i + j] = bonds[5 * i + j];
    CUDA_TRY(cudaMemcpy(s->bonds + 6 * off, bb.data(), 8 * 6 * n, cudaMemcpyHostToDevice));
    std::vector<float> bf(8 * n, 0.0f);
    for (long long i = 0; i + 1 < n; i++)
      for (int j = 0; j < 5; j++) bf[8 * i + j] = (float)bonds[5 * i + j];
    CUDA_TRY(cudaMemcpy(s->bonds32 + 8 * off, bf.data(), 4 * 8 * n, cudaMemcpyHostToDevice));
  }
  return CG_OK;
}

int cg_set_twist(cg_sim* s, int rep, const double* eps_twist, const double* omega0) {
  if (int rc = check_rep(s, rep)) return rc;
  RepDev d;
  if (int rc = get_rep(s, rep, &d)) return rc;
  if (!eps_twist) {
    d.twist = 0;
    return put_rep(s, rep, &d);
  }
  if (!omega0) return fail(CG_ERR_ARG, "omega0 is required with eps_twist");
  const long long n = s->n_beads[rep], off = s->bead_off[rep];
  for (long long i = 0; i + 1 < n; i++)
    if (!(eps_twist[i] > 0) || !std::isfinite(omega0[i]))
      return fail(CG_ERR_ARG, "twist moduli must be positive and natural twists finite");
  if (!s->twist) {
    CUDA_TRY(cudaMalloc(&s->twist, 16 * std::max(1LL, s->total_beads)));
    CUDA_TRY(cudaMemset(s->twist, 0, 16 * std::max(1LL, s->total_beads)));
    s->drop_graph();  // the kernels' arguments changed
  }
  std::vector<double> tw(2 * n, 0.0);
  for (long long i = 0; i + 1 < n; i++) { tw[2 * i] = eps_twist[i]; tw[2 * i + 1] = omega0[i]; }
  CUDA_TRY(cudaMemcpy(s->twist + 2 * off, tw.data(), 16 * n, cudaMemcpyHostToDevice));
  d.twist = 1;
  return put_rep(s, rep, &d);
}

static int steric_run(cg_sim* s, int rep, long long ind0, long long indf, const double* r_trial, double e,
                      double V0, double* out) {
  if (int rc = check_rep(s, rep)) return rc;
  if (!out) return fail(CG_ERR_ARG, "null out");
  if (!(e > 0) || !std::isfinite(V0)) return fail(CG_ERR_ARG, "excluded distance must be > 0, V0 finite");
  const long long n = s->n_beads[rep];
  const long long m = r_trial ? indf - ind0 : 0;
  if (r_trial && (ind0 < 0 || indf > n || m < 1)) return fail(CG_ERR_ARG, "need 0 <= ind0 < indf <= n_beads");
  const long long need = n + 3 * m + 1;
  if (need > s->steric_cap) {
    if (s->steric_work) cudaFree(s->steric_work);
    s->steric_work = nullptr;
    s->steric_cap = 0;
    CUDA_TRY(cudaMalloc(&s->steric_work, 8 * need));
    s->steric_cap = need;
  }
  double* rows = s->steric_work;
  double* trial = r_trial ? rows + n : nullptr;
  double* total = rows + n + 3 * m;
  if (trial) CUDA_TRY(cudaMemcpy(trial, r_trial, 8 * 3 * m, cudaMemcpyHostToDevice));
  cg_launch_steric(s->args(), s->fp64 != 0, rep, r_trial ? m : n, ind0, indf, trial, e, V0, rows, total, 0);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaMemcpy(out, total, 8, cudaMemcpyDeviceToHost));
  return CG_OK;
}

int cg_steric_energy(cg_sim* s, int32_t rep, double excluded_distance, double V0, double* out) {
  return steric_run(s, rep, 0, 0, nullptr, excluded_distance, V0, out);
}

int cg_steric_delta(cg_sim* s, int32_t rep, int64_t ind0, int64_t indf, const double* r_trial,
                    double excluded_distance, double V0, double* out) {
  if (!r_trial) return fail(CG_ERR_ARG, "null r_trial");
  return steric_run(s, rep, ind0, indf, r_trial, excluded_distance, V0, out);
}

int cg_get_chain(cg_sim* s, int rep, double* r, double* t3, double* t2, int64_t* states) {
  if (int rc = check_rep(s, rep)) return rc;
  const long long n = s->n_beads[rep], off = s->bead_off[rep];
  unsigned char* buf = s->staging(s->pos_bytes() * n * 3 + 4 * n);
  if (!buf) return fail(CG_ERR_NOMEM, "pinned staging allocation failed");
  double* dst[3] = {r, t3, t2};
  void* src[3] = {s->r4, s->t34, s->t24};
  for (int k = 0; k < 3; k++) {
    if (!dst[k]) continue;
    CUDA_TRY(cudaMemcpy(buf, (char*)src[k] + s->pos_bytes() * off, s->pos_bytes() * n, cudaMemcpyDeviceToHost));
    if (s->fp64) unpack_pos<double>(buf, n, dst[k]);
    else unpack_pos<float>(buf, n, dst[k]);
  }
  if (states) {
    unsigned* pk = reinterpret_cast<unsigned*>(buf + s->pos_bytes() * n * 3);
    CUDA_TRY(cudaMemcpy(pk, s->states + off, 4 * n, cudaMemcpyDeviceToHost));
    for (long long i = 0; i < n; i++)
      for (int b = 0; b < s->nb; b++) states[i * s->nb + b] = (pk[i] >> (8 * b)) & 0xFF;
  }
  return CG_OK;
}

// The replica table of host pointers for the direct-access kernels.
static int put_host_table(cg_sim* s, const double* const* r, const double* const* t3, const double* const* t2,
                          const int64_t* const* states) {
  std::vector<const void*> tab(4 * (size_t)s->R, nullptr);
  for (int rep = 0; rep < s->R; rep++) {
    tab[4 * rep] = r ? r[rep] : nullptr;
    tab[4 * rep + 1] = t3 ? t3[rep] : nullptr;
    tab[4 * rep + 2] = t2 ? t2[rep] : nullptr;
    tab[4 * rep + 3] = states ? states[rep] : nullptr;
  }
  CUDA_TRY(cudaMemcpy(s->hio_tab, tab.data(), tab.size() * sizeof(void*), cudaMemcpyHostToDevice));
  return CG_OK;
}

int cg_set_chains(cg_sim* s, const double* const* r, const double* const* t3, const double* const* t2,
                  const int64_t* const* states) {
  if (!s) return fail(CG_ERR_ARG, "null sim");
  if (s->direct_host) {
    if (int rc = put_host_table(s, r, t3, t2, states)) return rc;
    CUDA_TRY(cudaMemset(s->hio_flag, 0, sizeof(unsigned)));
    if (s->upload_stage()) {
      // one pass over the host arrays into the staging arrays, checked; then
      // the given arrays are copied into the resident state on the device
      KArgs st = s->args();
      st.r4 = s->hio_r4; st.t34 = s->hio_t34; st.t24 = s->hio_t24; st.states = s->hio_states;
      cg_launch_host_load(st, s->fp64 != 0, s->hio_tab, s->R, s->max_beads, s->nb, s->hio_flag, 2, 0);
      CUDA_TRY(cudaGetLastError());
      unsigned bad = 0;
      CUDA_TRY(cudaMemcpy(&bad, s->hio_flag, sizeof(unsigned), cudaMemcpyDeviceToHost));
      if (bad & 1u) return fail(CG_ERR_NONFINITE, "non-finite position or tangent");
      if (bad & 2u) return fail(CG_ERR_ARG, "binding states must be in 0..3");
      cg_launch_stage_commit(s->args(), s->fp64 != 0, s->hio_tab, s->R, s->max_beads, s->hio_r4, s->hio_t34,
                             s->hio_t24, s->hio_states, 0);
      CUDA_TRY(cudaGetLastError());
      CUDA_TRY(cudaStreamSynchronize(0));
      return CG_OK;
    }
    cg_launch_host_load(s->args(), s->fp64 != 0, s->hio_tab, s->R, s->max_beads, s->nb, s->hio_flag, 0, 0);
    CUDA_TRY(cudaGetLastError());
    unsigned bad = 0;
    CUDA_TRY(cudaMemcpy(&bad, s->hio_flag, sizeof(unsigned), cudaMemcpyDeviceToHost));
    if (bad & 1u) return fail(CG_ERR_NONFINITE, "non-finite position or tangent");
    if (bad & 2u) return fail(CG_ERR_ARG, "binding states must be in 0..3");
    cg_launch_host_load(s->args(), s->fp64 != 0, s->hio_tab, s->R, s->max_beads, s->nb, s->hio_flag, 1, 0);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaStreamSynchronize(0));
    return CG_OK;
  }
  const long long N = s->total_beads;
  const size_t pb = s->pos_bytes();
  unsigned char* buf = s->staging(pb * N * 3 + 4 * N);
  if (!buf) return fail(CG_ERR_NOMEM, "pinned staging allocation failed");
  const double* const* src[3] = {r, t3, t2};
  unsigned* pk = reinterpret_cast<unsigned*>(buf + pb * N * 3);
  std::atomic<int> bad(0);
  for_each_replica(s->R, [&](int rep) {
    const long long n = s->n_beads[rep], off = s->bead_off[rep];
    for (int k = 0; k < 3; k++) {
      if (!src[k] || !src[k][rep]) continue;
      const double* a = src[k][rep];
      for (long long i = 0; i < 3 * n; i++)
        if (!std::isfinite(a[i])) { bad.store(1); return; }
      unsigned char* b = buf + pb * (N * k + off);
      if (s->fp64) pack_pos<double>(a, n, b);
      else pack_pos<float>(a, n, b);
    }
    if (states && states[rep]) {
      for (long long i = 0; i < n; i++) {
        unsigned w = 0;
        for (int b = 0; b < s->nb; b++) {
          const int64_t v = states[rep][i * s->nb + b];
          if (v < 0 || v > CG_MAX_MARK) { bad.store(2); return; }
          w |= (unsigned)v << (8 * b);
        }
        pk[off + i] = w;
      }
    }
  });
  if (bad.load() == 1) return fail(CG_ERR_NONFINITE, "non-finite position or tangent");
  if (bad.load() == 2) return fail(CG_ERR_ARG, "binding states must be in 0..3");
  // every replica given for an array, or none: one copy of the whole array
  void* dst[3] = {s->r4, s->t34, s->t24};
  for (int k = 0; k < 3; k++) {
    if (!src[k]) continue;
    bool all = true;
    for (int rep = 0; rep < s->R; rep++) all = all && src[k][rep];
    if (all) {
      CUDA_TRY(cudaMemcpy(dst[k], buf + pb * N * k, pb * N, cudaMemcpyHostToDevice));
    } else {
      for (int rep = 0; rep < s->R; rep++)
        if (src[k][rep])
          CUDA_TRY(cudaMemcpy((char*)dst[k] + pb * s->bead_off[rep], buf + pb * (N * k + s->bead_off[rep]),
                              pb * s->n_beads[rep], cudaMemcpyHostToDevice));
    }
  }
  if (states) {
    bool all = true;
    for (int rep = 0; rep < s->R; rep++) all = all && states[rep];
    if (all) {
      CUDA_TRY(cudaMemcpy(s->states, pk, 4 * N, cudaMemcpyHostToDevice));
    } else {
      for (int rep = 0; rep < s->R; rep++)
        if (states[rep])
          CUDA_TRY(cudaMemcpy(s->states + s->bead_off[rep], pk + s->bead_off[rep], 4 * s->n_beads[rep],
                              cudaMemcpyHostToDevice));
    }
  }
  return CG_OK;
}

int cg_get_chains(cg_sim* s, double* const* r, double* const* t3, double* const* t2, int64_t* const* states) {
  if (!s) return fail(CG_ERR_ARG, "null sim");
  if (s->direct_host) {
    if (int rc = put_host_table(s, (const double* const*)r, (const double* const*)t3, (const double* const*)t2,
                                (const int64_t* const*)states))
      return rc;
    cg_launch_host_store(s->args(), s->fp64 != 0, s->hio_tab, s->R, s->max_beads, s->nb, 0);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaStreamSynchronize(0));
    return CG_OK;
  }
  const long long N = s->total_beads;
  const size_t pb = s->pos_bytes();
  unsigned char* buf = s->staging(pb * N * 3 + 4 * N);
  if (!buf) return fail(CG_ERR_NOMEM, "pinned staging allocation failed");
  double* const* dst[3] = {r, t3, t2};
  void* src[3] = {s->r4, s->t34, s->t24};
  for (int k = 0; k < 3; k++)
    if (dst[k]) CUDA_TRY(cudaMemcpy(buf + pb * N * k, src[k], pb * N, cudaMemcpyDeviceToHost));
  unsigned* pk = reinterpret_cast<unsigned*>(buf + pb * N * 3);
  if (states) CUDA_TRY(cudaMemcpy(pk, s->states, 4 * N, cudaMemcpyDeviceToHost));
  for_each_replica(s->R, [&](int rep) {
    const long long n = s->n_beads[rep], off = s->bead_off[rep];
    for (int k = 0; k < 3; k++) {
      if (!dst[k] || !dst[k][rep]) continue;
      const unsigned char* b = buf + pb * (N * k + off);
      if (s->fp64) unpack_pos<double>(b, n, dst[k][rep]);
      else unpack_pos<float>(b, n, dst[k][rep]);
    }
    if (states && states[rep])
      for (long long i = 0; i < n; i++)
        for (int b = 0; b < s->nb; b++) states[rep][i * s->nb + b] = (pk[off + i] >> (8 * b)) & 0xFF;
  });
  return CG_OK;
}

int cg_set_field(cg_sim* s, int rep, const cg_field_params* f, const double* access_vol) {
  if (int rc = check_rep(s, rep)) return rc;
  if (!f) return fail(CG_ERR_ARG, "null field");
  if (f->field_kind < 0 || f->field_kind > 2) return fail(CG_ERR_ARG, "field_kind must be 0, 1 or 2");
  if (f->confine_kind < 0 || f->confine_kind > 2) return fail(CG_ERR_ARG, "confine_kind must be 0, 1 or 2");
  if (f->field_kind == 2) {
    if (f->nx != s->dims[3 * rep] || f->ny != s->dims[3 * rep + 1] || f->nz != s->dims[3 * rep + 2])
      return fail(CG_ERR_ARG, "field grid differs from the grid given at creation");
    if (f->n_binders != s->nb) return fail(CG_ERR_ARG, "field binder count differs from the polymer's");
    if (!(f->x_width > 0 && f->y_width > 0 && f->z_width > 0)) return fail(CG_ERR_ARG, "box widths must be > 0");
  }
  if (access_vol && !s->nonuniform)
    return fail(CG_ERR_ARG, "per-voxel accessible volumes need nonuniform_access at creation");
  RepDev d;
  if (int rc = get_rep(s, rep, &d)) return rc;
  d.field_kind = f->field_kind;
  d.confine_kind = f->confine_kind;
  d.confine_length = f->confine_length;
  if (f->field_kind == 2) {
    d.wx = f->x_width; d.wy = f->y_width; d.wz = f->z_width;
    d.dx = f->x_width / f->nx; d.dy = f->y_width / f->ny; d.dz = f->z_width / f->nz;
    d.vol_bin = f->x_width * f->y_width * f->z_width / (double)(d.n_vox);
  }
  d.chi = f->chi; d.vf_limit = f->vf_limit; d.bead_vol = f->bead_vol;
  for (int b = 0; b < CG_MAX_BINDERS; b++) { d.pref[b] = f->pref[b]; d.intra[b] = f->intra[b]; }
  for (int b = 0; b < CG_MAX_BINDERS * CG_MAX_BINDERS; b++) d.xpref[b] = f->xpref[b];
  d.has_access = access_vol ? 1 : 0;
  if (f->fast_field && f->field_kind == 2) {
    if (f->n_points < 1 || f->n_points > (1 << 20)) return fail(CG_ERR_ARG, "n_points must be in 1..2^20");
    d.fast_n = f->n_points + (f->n_points % 2);  // init_fast_field rounds up to even
  } else {
    d.fast_n = 0;
  }
  if (access_vol) {
    // the factors the MC kernel's FP32 field terms need per voxel, in the
    // same FP64 arithmetic the kernel would do per touched voxel
    const long long nv = s->n_vox[rep];
    std::vector<float> sc(nv);
    std::vector<double> vb(nv);
    for (long long v = 0; v < nv; v++) {
      sc[v] = (float)((1.0 / 1099511627776.0) / access_vol[v]);
      vb[v] = access_vol[v] / f->bead_vol;
    }
    CUDA_TRY(cudaMemcpy(s->access_vol + s->vox_off[rep], access_vol, 8 * nv, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(s->access_sc + s->vox_off[rep], sc.data(), 4 * nv, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(s->access_vb + s->vox_off[rep], vb.data(), 8 * nv, cudaMemcpyHostToDevice));
  }
  return put_rep(s, rep, &d);
}

int cg_set_binding(cg_sim* s, int rep, const cg_binding_params* b) {
  if (int rc = check_rep(s, rep)) return rc;
  if (!b || b->n_binders != s->nb) return fail(CG_ERR_ARG, "binding parameters do not match n_binders");
  for (int i = 0; i < s->nb; i++)
    if (b->sites[i] < 0 || b->sites[i] > CG_MAX_MARK) return fail(CG_ERR_ARG, "sites_per_bead must be in 0..3");
  RepDev d;
  if (int rc = get_rep(s, rep, &d)) return rc;
  d.max_binders = b->max_binders;
  for (int i = 0; i < CG_MAX_BINDERS; i++) { d.sites[i] = b->sites[i]; d.mu[i] = b->mu[i]; }
  d.mu_adjust = b->mu_adjust_factor;
  for (int i = 0; i < CG_MAX_BINDERS * (CG_MAX_MARK + 1) * (CG_MAX_MARK + 1); i++) d.bind_f[i] = b->bind_f[i];
  return put_rep(s, rep, &d);
}

int cg_set_controllers(cg_sim* s, int rep, const cg_move_ctl* c, int n_ctl) {
  if (int rc = check_rep(s, rep)) return rc;
  if (!c || n_ctl < 1 || n_ctl > 5) return fail(CG_ERR_ARG, "between 1 and 5 controllers");
  for (int i = 0; i < n_ctl; i++) {
    if (c[i].move_kind < 0 || c[i].move_kind > 4) return fail(CG_ERR_ARG, "unknown move kind");
    double top = c[i].ctrl_kind == 1 ? std::max<double>((double)c[i].amp_bead, c[i].bead_hi) : (double)c[i].amp_bead;
    if (c[i].move_kind == CG_TANGENT_ROTATION) {
      if (top > (double)s->max_tangent)
        return fail(CG_ERR_ARG, "tangent_rotation bead amplitude exceeds max_tangent given at creation");
      if (c[i].move_on && c[i].amp_bead < 1) return fail(CG_ERR_ARG, "tangent_rotation needs amp_bead >= 1");
      if (top > 2e9) return fail(CG_ERR_ARG, "bead amplitude too large");
    } else if (top + 1 > (double)s->max_segment) {
      return fail(CG_ERR_ARG, "bead amplitude exceeds max_segment given at creation");
    }
  }
  if (rep == 0) s->n_ctl = n_ctl;
  else if (n_ctl != s->n_ctl) return fail(CG_ERR_ARG, "every replica needs the same number of controllers");
  CUDA_TRY(cudaMemcpy(s->ctl + 5LL * rep, c, sizeof(cg_move_ctl) * n_ctl, cudaMemcpyHostToDevice));
  return CG_OK;
}

int cg_get_controllers(cg_sim* s, int rep, cg_move_ctl* c, int n_ctl) {
  if (int rc = check_rep(s, rep)) return rc;
  if (!c || n_ctl < 1 || n_ctl > 5) return fail(CG_ERR_ARG, "between 1 and 5 controllers");
  CUDA_TRY(cudaMemcpy(c, s->ctl + 5LL * rep, sizeof(cg_move_ctl) * n_ctl, cudaMemcpyDeviceToHost));
  return CG_OK;
}

int cg_deposit(cg_sim* s, int rep) {
  if (!s) return fail(CG_ERR_ARG, "null sim");
  if (rep >= s->R) return fail(CG_ERR_ARG, "replica index out of range");
  KArgs a = s->args();
  if (rep < 0) {
    CUDA_TRY(cudaMemset(s->grid, 0, 8 * s->ncol * s->total_vox));
    cg_launch_deposit(a, s->fp64, -1, s->R, s->max_beads, 0);
  } else {
    CUDA_TRY(cudaMemset(s->grid + s->ncol * s->vox_off[rep], 0, 8 * s->ncol * s->n_vox[rep]));
    cg_launch_deposit(a, s->fp64, rep, 1, s->n_beads[rep], 0);
  }
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaDeviceSynchronize());
  return CG_OK;
}

int cg_get_density(cg_sim* s, int rep, int64_t* grid) {
  if (int rc = check_rep(s, rep)) return rc;
  const long long G = s->n_vox[rep];
  std::vector<long long> buf(G * s->ncol);
  CUDA_TRY(cudaMemcpy(buf.data(), s->grid + s->ncol * s->vox_off[rep], 8 * G * s->ncol, cudaMemcpyDeviceToHost));
  for (long long v = 0; v < G; v++)
    for (int c = 0; c <= s->nb; c++) grid[v * (s->nb + 1) + c] = buf[v * s->ncol + c];
  return CG_OK;
}

static int device_errors(cg_sim* s) {
  std::vector<RepDev> rd(s->R);
  CUDA_TRY(cudaMemcpy(rd.data(), s->reps, sizeof(RepDev) * s->R, cudaMemcpyDeviceToHost));
  unsigned any = 0;
  int first = -1;
  for (int r = 0; r < s->R; r++)
    if (rd[r].err) { any |= rd[r].err; if (first < 0) first = r; }
  if (!any) return CG_OK;
  // leave the replicas and the global scratch clean for the caller
  for (int r = 0; r < s->R; r++) rd[r].err = 0;
  cudaMemcpy(s->reps, rd.data(), sizeof(RepDev) * s->R, cudaMemcpyHostToDevice);
  const long long Hg = 1LL << s->g_logH;
  const long long RW = (long long)s->R * s->spec_s;
  cudaMemset(s->g_keys, 0xFF, 4 * Hg * RW);
  cudaMemset(s->g_bslot, 0xFF, 4 * Hg * RW);
  cudaMemset(s->g_vals, 0, 8 * Hg * (s->nb + 1) * RW);
  cudaMemset(s->picked, 0, 4 * s->total_picked);
  char msg[160];
  snprintf(msg, sizeof msg, "device error bits 0x%x (first at replica %d)", any, first);
  if (any & cg::E_WINDOW) return fail(CG_ERR_WINDOW, std::string(msg) + ": bead selection window must be less than polymer length");
  if (any & cg::E_STREAM) return fail(CG_ERR_STREAM, std::string(msg) + ": supplied random stream exhausted");
  if (any & cg::E_NONFINITE) return fail(CG_ERR_NONFINITE, std::string(msg) + ": non-finite position");
  if (any & cg::E_DRIFT)
    return fail(CG_ERR_DRIFT, std::string(msg) + ": recomputed energy left the running sum of dE by more than "
                              "the drift guard's bound (cg_get_drift)");
  return fail(CG_ERR_SPIN, std::string(msg) + ": iteration cap reached");
}

int cg_run(cg_sim* s, int64_t n_steps, uint64_t seed, void* stream) {
  if (!s) return fail(CG_ERR_ARG, "null sim");
  if (n_steps < 0) return fail(CG_ERR_ARG, "n_steps must be >= 0");
  if (n_steps == 0) return CG_OK;
  KArgs a = s->args();
  a.n_steps = n_steps;
  a.seed = seed;
  cg_launch_spec(a, s->fp64, s->spec_bytes, (cudaStream_t)stream);
  s->kernels++;
  CUDA_TRY(cudaGetLastError());
  return CG_OK;
}

int cg_run_logged(cg_sim* s, int64_t n_steps, uint64_t seed, cg_move_record* records, int64_t max_records,
                  int64_t* n_records) {
  if (!s) return fail(CG_ERR_ARG, "null sim");
  if (n_steps < 0 || max_records < 0) return fail(CG_ERR_ARG, "negative size");
  if (max_records > 0 && !records) return fail(CG_ERR_ARG, "null records");
  std::vector<RepDev> rd0(s->R), rd1(s->R);
  CUDA_TRY(cudaDeviceSynchronize());
  CUDA_TRY(cudaMemcpy(rd0.data(), s->reps, sizeof(RepDev) * s->R, cudaMemcpyDeviceToHost));
  cg_move_record* d_log = nullptr;
  const long long cap = std::max<int64_t>(max_records, 1);
  cudaError_t e = cudaMalloc(&d_log, sizeof(cg_move_record) * cap * s->R);
  if (e == cudaSuccess && n_steps > 0) {
    KArgs a = s->args();
    a.n_steps = n_steps;
    a.seed = seed;
    a.mlog = d_log;
    a.mlog_cap = max_records;
    a.lean = 0;  // the move log is in the full form only
    cg_launch_spec(a, s->fp64, s->spec_bytes, 0);
    s->kernels++;
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
  }
  if (e == cudaSuccess) e = cudaMemcpy(rd1.data(), s->reps, sizeof(RepDev) * s->R, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && max_records > 0)
    e = cudaMemcpy(records, d_log, sizeof(cg_move_record) * max_records * s->R, cudaMemcpyDeviceToHost);
  cudaFree(d_log);
  if (e != cudaSuccess) return fail(CG_ERR_CUDA, cudaGetErrorString(e));
  if (n_records)
    for (int r = 0; r < s->R; r++) n_records[r] = (int64_t)(rd1[r].draw_pos - rd0[r].draw_pos);
  return device_errors(s);
}

int cg_sync(cg_sim* s, void* stream) {
  if (!s) return fail(CG_ERR_ARG, "null sim");
  CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
  return device_errors(s);
}

int cg_run_audit(cg_sim* s, int rep, int64_t n_steps, const uint32_t* draws, int64_t n_draws,
                 const int8_t* bstates, int64_t n_bstates, cg_move_record* records,
                 int64_t max_records, int64_t* n_records, int64_t* draws_used, int64_t* bstates_used) {
  if (int rc = check_rep(s, rep)) return rc;
  if (n_steps < 0 || n_draws < 0 || n_bstates < 0 || max_records < 0) return fail(CG_ERR_ARG, "negative size");
  for (int64_t i = 0; i < n_draws; i++)
    if (draws[i] > 2147483647u) return fail(CG_ERR_ARG, "draws must be in [0, 2^31-1]");
  for (int64_t i = 0; i < n_bstates; i++)
    if (bstates[i] < 0 || bstates[i] > CG_MAX_MARK) return fail(CG_ERR_ARG, "binding-state draws must be in 0..3");
  unsigned* d_draws = nullptr;
  signed char* d_bs = nullptr;
  cg_move_record* d_rec = nullptr;
  cudaError_t e = cudaMalloc(&d_draws, 4 * std::max<int64_t>(n_draws, 1));
  if (e == cudaSuccess) e = cudaMalloc(&d_bs, std::max<int64_t>(n_bstates, 1));
  if (e == cudaSuccess) e = cudaMalloc(&d_rec, sizeof(cg_move_record) * std::max<int64_t>(max_records, 1));
  if (e == cudaSuccess && n_draws) e = cudaMemcpy(d_draws, draws, 4 * n_draws, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && n_bstates) e = cudaMemcpy(d_bs, bstates, n_bstates, cudaMemcpyHostToDevice);
  int rc = CG_OK;
  if (e == cudaSuccess) {
    KArgs a = s->args();
    a.n_steps = n_steps;
    a.audit_rep = rep;
    a.a_draws = d_draws; a.a_n_draws = n_draws;
    a.a_bstates = d_bs; a.a_n_bstates = n_bstates;
    a.a_recs = d_rec; a.a_max_recs = max_records;
    a.a_out = s->aout;
    cg_launch_mc(a, s->fp64, true, 0);
    s->kernels++;
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
  }
  long long out[3] = {0, 0, 0};
  if (e == cudaSuccess) e = cudaMemcpy(out, s->aout, sizeof out, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && records && max_records)
    e = cudaMemcpy(records, d_rec, sizeof(cg_move_record) * std::min<long long>(out[0], max_records),
                   cudaMemcpyDeviceToHost);
  cudaFree(d_draws); cudaFree(d_bs); cudaFree(d_rec);
  if (e != cudaSuccess) return fail(CG_ERR_CUDA, cudaGetErrorString(e));
  if (n_records) *n_records = out[0];
  if (draws_used) *draws_used = out[1];
  if (bstates_used) *bstates_used = out[2];
  rc = device_errors(s);
  return rc;
}

int cg_energy(cg_sim* s, int rep, double* out) {
  if (int rc = check_rep(s, rep)) return rc;
  KArgs a = s->args();
  cg_launch_energy(a, s->fp64, s->eout, 0);
  CUDA_TRY(cudaGetLastError());
  double buf[5];
  CUDA_TRY(cudaMemcpy(buf, s->eout + 5 * rep, sizeof buf, cudaMemcpyDeviceToHost));
  for (int i = 0; i < 4; i++) out[i] = buf[i];
  return CG_OK;
}

int cg_energies(cg_sim* s, double* out, void* stream) {
  if (!s || !out) return fail(CG_ERR_ARG, "null argument");
  cudaStream_t st = (cudaStream_t)stream;
  KArgs a = s->args();
  cg_launch_energy(a, s->fp64, s->eout, st);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaMemcpyAsync(out, s->eout, sizeof(double) * 5 * s->R, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  return CG_OK;
}

static int ensure_derivative_buffers(cg_sim* s) {
  if (!s->grad) CUDA_TRY(cudaMalloc(&s->grad, sizeof(float) * 3 * std::max(1LL, s->total_beads)));
  if (!s->terms) CUDA_TRY(cudaMalloc(&s->terms, sizeof(double) * cg::kTerms * s->R));
  if (!s->acc) {
    CUDA_TRY(cudaMalloc(&s->acc, sizeof(double) * cg::kAccPerRep * s->R));
    CUDA_TRY(cudaMemset(s->acc, 0, sizeof(double) * cg::kAccPerRep * s->R));
  }
  return CG_OK;
}

int cg_gradient(cg_sim* s, float* dEdr, double* terms) {
  if (!s) return fail(CG_ERR_ARG, "null sim");
  if (int rc = ensure_derivative_buffers(s)) return rc;
  KArgs a = s->args();
  if (dEdr) cg_launch_gradient(a, s->fp64 != 0, s->grad, s->max_beads, 0);
  if (terms) cg_launch_terms(a, s->terms, nullptr, 0);
  CUDA_TRY(cudaGetLastError());
  if (dEdr) CUDA_TRY(cudaMemcpy(dEdr, s->grad, sizeof(float) * 3 * s->total_beads, cudaMemcpyDeviceToHost));
  if (terms) CUDA_TRY(cudaMemcpy(terms, s->terms, sizeof(double) * cg::kTerms * s->R, cudaMemcpyDeviceToHost));
  return CG_OK;
}

int cg_set_chains_device(cg_sim* s, const double* r, const double* t3, void* stream) {
  if (!s) return fail(CG_ERR_ARG, "null sim");
  if (!r && !t3) return CG_OK;
  cg_launch_store_chains(s->args(), s->fp64 != 0, s->total_beads, r, t3, (cudaStream_t)stream);
  CUDA_TRY(cudaGetLastError());
  return CG_OK;
}

int cg_deposit_async(cg_sim* s, void* stream) {
  if (!s) return fail(CG_ERR_ARG, "null sim");
  cudaStream_t st = (cudaStream_t)stream;
  CUDA_TRY(cudaMemsetAsync(s->grid, 0, 8 * s->ncol * s->total_vox, st));
  cg_launch_deposit(s->args(), s->fp64, -1, s->R, s->max_beads, st);
  CUDA_TRY(cudaGetLastError());
  return CG_OK;
}

int cg_energies_device(cg_sim* s, double* out, void* stream) {
  if (!s || !out) return fail(CG_ERR_ARG, "null argument");
  cg_launch_energy(s->args(), s->fp64, out, (cudaStream_t)stream);
  CUDA_TRY(cudaGetLastError());
  return CG_OK;
}

int cg_gradient_device(cg_sim* s, double* dEdr, double* dEdt3, void* stream) {
  if (!s) return fail(CG_ERR_ARG, "null sim");
  if (!dEdr) return fail(CG_ERR_ARG, "dEdr is required");
  if (dEdt3 && s->twist) return fail(CG_ERR_ARG, "dE/dt3 does not include SSTWLC twist terms");
  cg_launch_gradient64(s->args(), s->fp64 != 0, dEdr, dEdt3, s->max_beads, (cudaStream_t)stream);
  CUDA_TRY(cudaGetLastError());
  return CG_OK;
}

int cg_sample_terms(cg_sim* s, void* stream) {
  if (!s) return fail(CG_ERR_ARG, "null sim");
  if (int rc = ensure_derivative_buffers(s)) return rc;
  cg_launch_terms(s->args(), nullptr, s->acc, (cudaStream_t)stream);
  CUDA_TRY(cudaGetLastError());
  return CG_OK;
}

int cg_get_samples(cg_sim* s, double* out, int reset) {
  if (!s || !out) return fail(CG_ERR_ARG, "null argument");
  if (int rc = ensure_derivative_buffers(s)) return rc;
  CUDA_TRY(cudaMemcpy(out, s->acc, sizeof(double) * cg::kAccPerRep * s->R, cudaMemcpyDeviceToHost));
  if (reset) CUDA_TRY(cudaMemset(s->acc, 0, sizeof(double) * cg::kAccPerRep * s->R));
  return CG_OK;
}

int cg_reset_running_energy(cg_sim* s) {
  if (!s) return fail(CG_ERR_ARG, "null sim");
  std::vector<RepDev> rd(s->R);
  CUDA_TRY(cudaMemcpy(rd.data(), s->reps, sizeof(RepDev) * s->R, cudaMemcpyDeviceToHost));
  for (auto& d : rd) d.run_dE = 0;
  CUDA_TRY(cudaMemcpy(s->reps, rd.data(), sizeof(RepDev) * s->R, cudaMemcpyHostToDevice));
  return CG_OK;
}

int cg_get_tally(cg_sim* s, int rep, uint64_t* out) {
  if (int rc = check_rep(s, rep)) return rc;
  CUDA_TRY(cudaMemcpy(out, s->tally + 30LL * rep, 30 * 8, cudaMemcpyDeviceToHost));
  return CG_OK;
}

int cg_reset_tally(cg_sim* s) {
  if (!s) return fail(CG_ERR_ARG, "null sim");
  CUDA_TRY(cudaMemset(s->tally, 0, 8 * 30 * s->R));
  return CG_OK;
}

static int enqueue_exchange(cg_sim* s, int n_rungs, long long round, uint64_t seed, cudaStream_t st) {
  KArgs a = s->args();
  cg_launch_chi_sum(a, s->eout, st);
  cg_launch_exchange(a, s->eout, n_rungs, round, seed, st);
  return CG_OK;
}

// chi rungs per row (n_rungs) against the replica count and the mu ladder
static int check_rungs(const cg_sim* s, long long n_rungs) {
  if (s->mu_rungs > 1) {
    if (n_rungs < 1 || s->R % (n_rungs * s->mu_rungs))
      return fail(CG_ERR_ARG, "with a mu ladder, n_rungs * mu_rungs must divide n_replicas");
    return CG_OK;
  }
  if (n_rungs < 2 || s->R % n_rungs) return fail(CG_ERR_ARG, "n_rungs must be >= 2 and divide n_replicas");
  return CG_OK;
}

int cg_set_mu_ladder(cg_sim* s, int32_t mu_rungs, int32_t binder) {
  if (!s) return fail(CG_ERR_ARG, "null sim");
  if (mu_rungs != 0 && (mu_rungs < 2 || s->R % mu_rungs))
    return fail(CG_ERR_ARG, "mu_rungs must be 0 or >= 2 and divide n_replicas");
  if (binder < 0 || binder >= s->nb) return fail(CG_ERR_ARG, "binder index out of range");
  s->mu_rungs = mu_rungs;
  s->mu_binder = binder;
  s->drop_graph();  // arguments are baked into it
  return CG_OK;
}

int cg_get_mu(cg_sim* s, int32_t binder, double* mu) {
  if (!s || !mu) return fail(CG_ERR_ARG, "null argument");
  if (binder < 0 || binder >= s->nb) return fail(CG_ERR_ARG, "binder index out of range");
  std::vector<RepDev> rd(s->R);
  CUDA_TRY(cudaMemcpy(rd.data(), s->reps, sizeof(RepDev) * s->R, cudaMemcpyDeviceToHost));
  for (int r = 0; r < s->R; r++) mu[r] = rd[r].mu[binder];
  return CG_OK;
}

int cg_get_swap_counts(cg_sim* s, uint64_t* chi_swaps, uint64_t* chi_attempts, uint64_t* mu_swaps,
                       uint64_t* mu_attempts) {
  if (!s) return fail(CG_ERR_ARG, "null sim");
  uint64_t* dst[4] = {chi_swaps, chi_attempts, mu_swaps, mu_attempts};
  unsigned long long* src[4] = {s->swaps, s->swap_attempts, s->mu_swaps, s->mu_swap_attempts};
  for (int k = 0; k < 4; k++)
    if (dst[k]) CUDA_TRY(cudaMemcpy(dst[k], src[k], 8 * s->R, cudaMemcpyDeviceToHost));
  return CG_OK;
}

int cg_exchange(cg_sim* s, int n_rungs, int64_t round, uint64_t seed, void* stream) {
  if (!s) return fail(CG_ERR_ARG, "null sim");
  if (int rc = check_rungs(s, n_rungs)) return rc;
  enqueue_exchange(s, n_rungs, round, seed, (cudaStream_t)stream);
  CUDA_TRY(cudaGetLastError());
  return CG_OK;
}

int cg_get_chi(cg_sim* s, double* chi) {
  if (!s) return fail(CG_ERR_ARG, "null sim");
  std::vector<RepDev> rd(s->R);
  CUDA_TRY(cudaMemcpy(rd.data(), s->reps, sizeof(RepDev) * s->R, cudaMemcpyDeviceToHost));
  for (int r = 0; r < s->R; r++) chi[r] = rd[r].chi;
  return CG_OK;
}

int cg_run_batched(cg_sim* s, int64_t n_rounds, int64_t n_steps, int32_t n_rungs, uint64_t seed,
                   void* stream) {
  if (!s) return fail(CG_ERR_ARG, "null sim");
  if (n_rounds < 1 || n_steps < 1) return fail(CG_ERR_ARG, "n_rounds and n_steps must be >= 1");
  if (n_rungs)
    if (int rc = check_rungs(s, n_rungs)) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  const bool timed = s->timing_cap > 0;
  if (!(s->graph && s->graph_rounds == n_rounds && s->graph_steps == n_steps && s->graph_rungs == n_rungs &&
        s->graph_seed == seed && s->graph_stream == st && (long long)s->tnode_begin.size() == (timed ? n_rounds : 0))) {
    s->drop_graph();
    if (timed) {
      s->cap_begin.assign(n_rounds, nullptr);
      s->cap_end.assign(n_rounds, nullptr);
      for (long long k = 0; k < n_rounds; k++) {
        CUDA_TRY(cudaEventCreate(&s->cap_begin[k]));
        CUDA_TRY(cudaEventCreate(&s->cap_end[k]));
      }
    }
    cudaStream_t cap;
    CUDA_TRY(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    cudaGraph_t gr;
    CUDA_TRY(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
    for (long long k = 0; k < n_rounds; k++) {
      KArgs a = s->args();
      a.n_steps = n_steps;
      a.seed = seed;
      if (timed) cudaEventRecordWithFlags(s->cap_begin[k], cap, cudaEventRecordExternal);
      cg_launch_spec(a, s->fp64, s->spec_bytes, cap);
      if (timed) cudaEventRecordWithFlags(s->cap_end[k], cap, cudaEventRecordExternal);
      if (n_rungs) enqueue_exchange(s, n_rungs, -1, seed, cap);
      if (s->guard_every) cg_launch_guard(a, s->guard_args(), s->fp64, cap);
    }
    cudaError_t e = cudaStreamEndCapture(cap, &gr);
    cudaStreamDestroy(cap);
    if (e != cudaSuccess) return fail(CG_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    if (timed) {  // the event-record nodes of each round, found by the events they were captured with
      size_t n = 0;
      cudaGraphGetNodes(gr, nullptr, &n);
      std::vector<cudaGraphNode_t> nodes(n);
      if (n) cudaGraphGetNodes(gr, nodes.data(), &n);
      s->tnode_begin.assign(n_rounds, nullptr);
      s->tnode_end.assign(n_rounds, nullptr);
      for (cudaGraphNode_t nd : nodes) {
        cudaGraphNodeType ty;
        if (cudaGraphNodeGetType(nd, &ty) != cudaSuccess || ty != cudaGraphNodeTypeEventRecord) continue;
        cudaEvent_t ev = nullptr;
        cudaGraphEventRecordNodeGetEvent(nd, &ev);
        for (long long k = 0; k < n_rounds; k++) {
          if (ev == s->cap_begin[k]) s->tnode_begin[k] = nd;
          if (ev == s->cap_end[k]) s->tnode_end[k] = nd;
        }
      }
      for (long long k = 0; k < n_rounds; k++)
        if (!s->tnode_begin[k] || !s->tnode_end[k]) {
          cudaGraphDestroy(gr);
          s->tnode_begin.clear();
          return fail(CG_ERR_CUDA, "graph capture: round timing nodes not found");
        }
    }
    e = cudaGraphInstantiate(&s->graph, gr, 0);
    s->graph_src = gr;
    if (e != cudaSuccess) { s->drop_graph(); return fail(CG_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e)); }
    s->graph_rounds = n_rounds; s->graph_steps = n_steps; s->graph_rungs = n_rungs;
    s->graph_seed = seed; s->graph_stream = st;
  }
  if (timed)
    for (long long k = 0; k < n_rounds; k++) {
      const long long slot = (s->timing_count + k) % s->timing_cap;
      CUDA_TRY(cudaGraphExecEventRecordNodeSetEvent(s->graph, s->tnode_begin[k], s->tev_begin[slot]));
      CUDA_TRY(cudaGraphExecEventRecordNodeSetEvent(s->graph, s->tnode_end[k], s->tev_end[slot]));
    }
  CUDA_TRY(cudaGraphLaunch(s->graph, st));
  if (timed) s->timing_count += n_rounds;
  s->kernels += n_rounds;
  return CG_OK;
}

int cg_set_drift_guard(cg_sim* s, int32_t every_rounds, double tol_abs, double tol_rel) {
  if (!s) return fail(CG_ERR_ARG, "null sim");
  if (every_rounds < 0) return fail(CG_ERR_ARG, "every_rounds must be >= 0");
  if (!(tol_abs >= 0) || !(tol_rel >= 0)) return fail(CG_ERR_ARG, "tolerances must be >= 0");
  CUDA_TRY(cudaDeviceSynchronize());
  s->drop_graph();  // the guard's launches are part of the captured round
  s->free_guard();
  if (every_rounds == 0) return CG_OK;
  // enough chunk x replica blocks to spread one recompute over the GPU
  const int chunks = (int)std::max<long long>(1, std::min<long long>(64, (4LL * std::max(s->n_sm, 1) + s->R - 1) / s->R));
  const size_t R = (size_t)s->R;
  cudaError_t e = cudaMalloc(&s->guard_partial, sizeof(double) * R * chunks * 6);
  if (e == cudaSuccess) e = cudaMalloc(&s->guard_e_ref, sizeof(double) * R);
  if (e == cudaSuccess) e = cudaMalloc(&s->guard_run_ref, sizeof(double) * R);
  if (e == cudaSuccess) e = cudaMalloc(&s->guard_drift, sizeof(double) * R);
  if (e == cudaSuccess) e = cudaMalloc(&s->guard_init, sizeof(int) * R);
  if (e == cudaSuccess) e = cudaMalloc(&s->guard_counter, sizeof(unsigned long long) * 2);
  if (e == cudaSuccess) e = cudaMemset(s->guard_drift, 0, sizeof(double) * R);
  if (e == cudaSuccess) e = cudaMemset(s->guard_init, 0, sizeof(int) * R);
  if (e == cudaSuccess) e = cudaMemset(s->guard_counter, 0, sizeof(unsigned long long) * 2);
  if (e != cudaSuccess) {
    s->free_guard();
    return fail(CG_ERR_NOMEM, std::string("drift guard buffers: ") + cudaGetErrorString(e));
  }
  s->guard_every = every_rounds;
  s->guard_chunks = chunks;
  s->guard_tol_abs = tol_abs;
  s->guard_tol_rel = tol_rel;
  return CG_OK;
}

int cg_get_drift(cg_sim* s, double* drift, int64_t* checks) {
  if (!s) return fail(CG_ERR_ARG, "null sim");
  if (!s->guard_every) return fail(CG_ERR_ARG, "the drift guard is off (cg_set_drift_guard)");
  CUDA_TRY(cudaDeviceSynchronize());
  if (drift) CUDA_TRY(cudaMemcpy(drift, s->guard_drift, sizeof(double) * s->R, cudaMemcpyDeviceToHost));
  if (checks) {
    unsigned long long c[2];
    CUDA_TRY(cudaMemcpy(c, s->guard_counter, sizeof c, cudaMemcpyDeviceToHost));
    *checks = (int64_t)c[1];
  }
  return CG_OK;
}

// ---------------------------------------------------------------- checkpoint
// The whole resident state of a sim, as one byte image: a header naming the
// layout, then every device buffer whose contents carry over between calls.
namespace {
struct StateHeader {
  unsigned long long magic, version;
  long long R, nb, ncol, fp64, total_beads, total_vox, n_ctl, mu_rungs, mu_binder, twist;
};
constexpr unsigned long long kStateMagic = 0x31534D4F52484343ULL;  // "CCHROMS1"

struct StatePart {
  void* dev;
  size_t bytes;
};

std::vector<StatePart> state_parts(cg_sim* s) {
  const size_t R = (size_t)s->R, B = (size_t)s->total_beads;
  std::vector<StatePart> p = {
      {s->reps, sizeof(RepDev) * R},        {s->ctl, sizeof(cg_move_ctl) * 5 * R},
      {s->tally, 8 * 30 * R},               {s->r4, s->pos_bytes() * B},
      {s->t34, s->pos_bytes() * B},         {s->t24, s->pos_bytes() * B},
      {s->states, 4 * B},                   {s->marks, 4 * B},
      {s->bonds, 48 * B},                   {s->bonds32, 32 * B},
      {s->grid, 8 * (size_t)s->ncol * (size_t)s->total_vox},
      {s->rep_of_rung, 4 * R},              {s->swaps, 8 * R},
      {s->swap_attempts, 8 * R},            {s->xround, 8},
      {s->mu_swaps, 8 * R},                 {s->mu_swap_attempts, 8 * R}};
  if (s->twist) p.push_back({s->twist, 16 * B});
  if (s->nonuniform) {
    p.push_back({s->access_vol, 8 * (size_t)s->total_vox});
    p.push_back({s->access_sc, 4 * (size_t)s->total_vox});
    p.push_back({s->access_vb, 8 * (size_t)s->total_vox});
  }
  return p;
}

StateHeader state_header(const cg_sim* s) {
  StateHeader h{kStateMagic, 1, s->R, s->nb, s->ncol, s->fp64, s->total_beads, s->total_vox, s->n_ctl,
                s->mu_rungs, s->mu_binder, s->twist ? 1 : 0};
  return h;
}
}  // namespace

int64_t cg_state_bytes(cg_sim* s) {
  if (!s) return fail(CG_ERR_ARG, "null sim");
  size_t n = sizeof(StateHeader);
  for (const StatePart& p : state_parts(s)) n += p.bytes;
  return (int64_t)n;
}

int cg_save_state(cg_sim* s, void* buf, int64_t bytes) {
  if (!s || !buf) return fail(CG_ERR_ARG, "null argument");
  if (bytes < cg_state_bytes(s)) return fail(CG_ERR_ARG, "buffer smaller than cg_state_bytes()");
  CUDA_TRY(cudaDeviceSynchronize());
  unsigned char* out = static_cast<unsigned char*>(buf);
  const StateHeader h = state_header(s);
  memcpy(out, &h, sizeof h);
  size_t off = sizeof h;
  for (const StatePart& p : state_parts(s)) {
    CUDA_TRY(cudaMemcpy(out + off, p.dev, p.bytes, cudaMemcpyDeviceToHost));
    off += p.bytes;
  }
  return CG_OK;
}

int cg_load_state(cg_sim* s, const void* buf, int64_t bytes) {
  if (!s || !buf) return fail(CG_ERR_ARG, "null argument");
  if (bytes < (int64_t)sizeof(StateHeader)) return fail(CG_ERR_ARG, "state image too short");
  StateHeader h, want = state_header(s);
  memcpy(&h, buf, sizeof h);
  if (h.magic != kStateMagic || h.version != want.version)
    return fail(CG_ERR_ARG, "not a state image of this library");
  if (memcmp(&h, &want, sizeof h) != 0)
    return fail(CG_ERR_ARG, "state image of a simulation with another layout (replicas, beads, grids, "
                            "binders, precision, controllers or mu ladder differ)");
  if (bytes < cg_state_bytes(s)) return fail(CG_ERR_ARG, "state image truncated");
  CUDA_TRY(cudaDeviceSynchronize());
  const unsigned char* in = static_cast<const unsigned char*>(buf);
  size_t off = sizeof h;
  for (const StatePart& p : state_parts(s)) {
    CUDA_TRY(cudaMemcpy(p.dev, in + off, p.bytes, cudaMemcpyHostToDevice));
    off += p.bytes;
  }
  if (s->guard_every) CUDA_TRY(cudaMemset(s->guard_init, 0, sizeof(int) * s->R));  // new reference energies
  {  // the restored replicas' twist chooses the MC kernel's form
    std::vector<RepDev> rd(s->R);
    CUDA_TRY(cudaMemcpy(rd.data(), s->reps, sizeof(RepDev) * s->R, cudaMemcpyDeviceToHost));
    for (int r = 0; r < s->R; r++) s->note_features(r, rd[r]);
  }
  return CG_OK;
}

int cg_set_round_timing(cg_sim* s, int32_t capacity) {
  if (!s) return fail(CG_ERR_ARG, "null sim");
  if (capacity < 0 || capacity > (1 << 20)) return fail(CG_ERR_ARG, "capacity must be in 0..2^20");
  CUDA_TRY(cudaDeviceSynchronize());
  s->drop_timing();
  s->tev_begin.assign(capacity, nullptr);
  s->tev_end.assign(capacity, nullptr);
  for (int k = 0; k < capacity; k++) {
    CUDA_TRY(cudaEventCreate(&s->tev_begin[k]));
    CUDA_TRY(cudaEventCreate(&s->tev_end[k]));
  }
  s->timing_cap = capacity;
  return CG_OK;
}

int cg_get_round_times(cg_sim* s, float* mc_ms, int32_t max, int32_t* count) {
  if (!s) return fail(CG_ERR_ARG, "null sim");
  if (max < 0 || (max > 0 && !mc_ms)) return fail(CG_ERR_ARG, "bad output buffer");
  long long n = std::min<long long>(std::min<long long>(s->timing_count, s->timing_cap), max);
  for (long long i = 0; i < n; i++) {
    const long long slot = (s->timing_count - n + i) % s->timing_cap;
    CUDA_TRY(cudaEventSynchronize(s->tev_end[slot]));
    CUDA_TRY(cudaEventElapsedTime(&mc_ms[i], s->tev_begin[slot], s->tev_end[slot]));
  }
  if (count) *count = (int32_t)n;
  return CG_OK;
}

int cg_get_launch_shape(cg_sim* s, int32_t* wpb, int32_t* lanes, int32_t* in_flight, int32_t* hash_slots) {
  if (!s) return fail(CG_ERR_ARG, "null sim");
  if (wpb) *wpb = s->spec_w;
  if (lanes) *lanes = s->spec_g;
  if (in_flight) *in_flight = s->spec_s;
  if (hash_slots) *hash_slots = s->pool_on ? 1 << s->pool_logH : 1 << s->logH;
  return CG_OK;
}

int cg_mc_warps_per_sm(int32_t pos_fp64, int32_t lanes) {
  if (!cg_spec_shape_ok(pos_fp64 != 0, lanes)) return -1;
  return cg_spec_warps_per_sm(pos_fp64 != 0, lanes);
}

int cg_get_transfer_mode(cg_sim* s, int32_t* direct) {
  if (!s || !direct) return fail(CG_ERR_ARG, "null argument");
  *direct = s->direct_host;
  return CG_OK;
}

int cg_get_launch_info(cg_sim* s, int32_t* wpb, int32_t* hash_slots, int64_t* kernels) {
  if (!s) return fail(CG_ERR_ARG, "null sim");
  if (wpb) *wpb = s->spec_w;
  if (hash_slots) *hash_slots = 1 << s->logH;
  if (kernels) *kernels = s->kernels;
  return CG_OK;
}

}  // extern "C"

int cg::record_error(int code, const std::string& msg) { return fail(code, msg); }
