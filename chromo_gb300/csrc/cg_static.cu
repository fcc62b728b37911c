// cg_static.cu -- field energy of one chain with no memory allocation.
//
// cg_field_energy_static() deposits a chain into an int64 fixed-point density
// grid and evaluates the UniformDensityField energy of that grid, the same
// numbers that cg_deposit followed by cg_energy give for a replica.  It takes
// device pointers and needs no cg_sim, and it allocates nothing: the grid is
// the file-scope device array below, whose size is fixed when the library is
// built.  It is meant for callers that must not allocate device memory: a
// server whose device memory belongs to its own pool and may not grow, or code
// in which a cudaMalloc (which can synchronise the whole device) would stall
// work already in flight.  Everything else is better served by the cg_sim path.
//
// Shared state: one scratch array per device, so two calls that overlap in
// time on the same device (on different streams, or from different host
// threads) race on it and give wrong results.  Calls on one stream are
// ordered and safe.  The scratch does not need to start at zero: each call
// clears the cells it uses on its stream before depositing.
//
// The first call on a device may load this library's device code there (with
// CUDA's lazy module loading the module, and with it the 8 MiB array, is
// created on first use): that call belongs in the caller's set-up phase, and
// from the second call on nothing is created.
#include <cuda_runtime.h>

#include <atomic>
#include <cstring>
#include <string>

#include "cg_kernels.h"

namespace {

using cg::GridF;
using cg::RepDev;

// 2^20 int64 cells (8 MiB) of grid, then the doubly-bound counters and a
// flag word set when a position is not finite.  Enough for a 64^3 grid with
// three binders (262,144 voxels x 4 columns) or 80^3 with one binder
// (512,000 voxels x 2 columns).
constexpr long long kStaticCells = 1LL << 20;
constexpr long long kStaticFlags = CG_MAX_BINDERS + 1;
constexpr long long kStaticTotal = kStaticCells + kStaticFlags;
__device__ __align__(256) long long g_static_scratch[kStaticTotal];

// Device address of g_static_scratch, looked up once per device by the first
// call made on that device (cudaGetSymbolAddress can load the module, so that
// first call belongs before any stream capture).
constexpr int kMaxDevices = 64;
std::atomic<long long*> g_scratch_addr[kMaxDevices];

int scratch_on_device(long long** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cg::record_error(CG_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return cg::record_error(CG_ERR_CUDA, "device ordinal beyond 63");
  long long* p = g_scratch_addr[dev].load();
  if (!p) {
    e = cudaGetSymbolAddress((void**)&p, g_static_scratch);
    if (e != cudaSuccess)
      return cg::record_error(CG_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    g_scratch_addr[dev].store(p);
  }
  *out = p;
  return CG_OK;
}

// Device memory of the current device, or managed memory.  Memory of another
// device is refused: the kernels run on the current device and would fault
// on it without peer access.
int device_pointer(const void* p, const char* name) {
  cudaPointerAttributes at;
  cudaError_t e = cudaPointerGetAttributes(&at, p);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return cg::record_error(CG_ERR_ARG, std::string(name) + " is not a device pointer");
  }
  if (at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged)
    return cg::record_error(CG_ERR_ARG, std::string(name) + " must point to device memory");
  if (at.type == cudaMemoryTypeDevice) {
    int dev = -1;
    e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cg::record_error(CG_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (at.device != dev)
      return cg::record_error(CG_ERR_ARG, std::string(name) + " is memory of device " + std::to_string(at.device) +
                                              ", not of the current device " + std::to_string(dev));
  }
  return CG_OK;
}

// Every bead adds its eight fixed-point trilinear weights to the total-density
// column and, times its bound count, to each binder's column
// (update_all_densities_for_all_polymers, chromo/fields.pyx:2041-2106).  A bead
// whose position is not finite deposits nothing and sets doubly[CG_MAX_BINDERS].
__global__ void static_deposit_kernel(RepDev rd, const double* r, const long long* states,
                                      long long* grid, unsigned long long* doubly) {
  const int ncol = rd.nb + 1;
  GridF gf;
  cg::make_gridf(rd, gf);
  unsigned n2[CG_MAX_BINDERS] = {0, 0, 0};
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < rd.n_beads;
       i += (long long)gridDim.x * blockDim.x) {
    const double p[3] = {r[3 * i], r[3 * i + 1], r[3 * i + 2]};
    if (!(isfinite(p[0]) && isfinite(p[1]) && isfinite(p[2]))) {
      atomicOr(doubly + CG_MAX_BINDERS, 1ull);
      continue;
    }
    double w[8];
    int v[8];
    cg::voxel_weights(rd, gf, p, w, v);
    long long s[CG_MAX_BINDERS];
    for (int b = 0; b < rd.nb; b++) {
      s[b] = states[i * rd.nb + b];
      n2[b] += s[b] == 2;
    }
    for (int l = 0; l < 8; l++) {
      const long long q = cg::q40(w[l]);
      long long* cell = grid + (long long)v[l] * ncol;
      atomicAdd((unsigned long long*)cell, (unsigned long long)q);
      for (int b = 0; b < rd.nb; b++)
        if (s[b]) atomicAdd((unsigned long long*)(cell + 1 + b), (unsigned long long)(q * s[b]));
    }
  }
  for (int b = 0; b < CG_MAX_BINDERS; b++) {
    unsigned t = __reduce_add_sync(cg::kFull, n2[b]);
    if ((threadIdx.x & 31) == 0 && t) atomicAdd(doubly + b, (unsigned long long)t);
  }
}

__device__ double static_block_sum(double v, double* sh) {
  v = cg::warp_sum(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  double t = 0;
  if (threadIdx.x < 32) {
    t = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
    t = cg::warp_sum(t);
  }
  return t;
}

// One block: the field energy of the grid in the consistent form
// (chromo/fields.pyx:1939-2316 with the per-voxel terms of :1675-1875), plus
// the intra-bead term of doubly bound beads; out[1] is the chi-free sum
// S = sum_v (V / V_bead) vf^2 over the voxels at or below vf_limit.
__global__ void static_energy_kernel(RepDev rd, const long long* grid, const unsigned long long* doubly,
                                     const double* access_vol, double* out) {
  __shared__ double sh[32];
  const int ncol = rd.nb + 1;
  double fe = 0, sx = 0;
  for (long long v = threadIdx.x; v < rd.n_vox; v += blockDim.x) {
    const double V = access_vol ? access_vol[v] : rd.vol_bin;
    double rho[CG_MAX_BINDERS];
    for (int b = 0; b < rd.nb; b++) rho[b] = ((double)grid[v * ncol + 1 + b] * cg::kFxInv) / V;
    for (int b = 0; b < rd.nb; b++) fe += rd.pref[b] * rho[b] * rho[b];
    for (int b = 0; b < rd.nb; b++)
      for (int e = 0; e < rd.nb; e++) fe += rd.xpref[b * CG_MAX_BINDERS + e] * rho[b] * rho[e];
    const double vf = ((double)grid[v * ncol] * cg::kFxInv) / V * rd.bead_vol;
    const double sv = (V / rd.bead_vol) * vf * vf;
    if (!(vf > rd.vf_limit)) sx += sv;  // above vf_limit the term is 1e99 vf, free of chi
    fe += vf > rd.vf_limit ? cg::kEHugeField * vf : rd.chi * sv;
  }
  const double t_fe = static_block_sum(fe, sh);
  const double t_sx = static_block_sum(sx, sh);
  if (threadIdx.x == 0) {
    double intra = 0;
    for (int b = 0; b < rd.nb; b++) intra += rd.intra[b] * (double)doubly[b];
    const bool bad = doubly[CG_MAX_BINDERS] != 0;  // a position was not finite
    out[0] = bad ? __longlong_as_double(0x7FF8000000000000LL) : t_fe + intra;
    out[1] = bad ? __longlong_as_double(0x7FF8000000000000LL) : t_sx;
  }
}

}  // namespace

extern "C" int cg_field_energy_static(const cg_field_params* f, int64_t n_beads, const double* r,
                                      const int64_t* states, const double* access_vol, double* out,
                                      void* stream) {
  if (!f || !out) return cg::record_error(CG_ERR_ARG, "null argument");
  if (f->field_kind != 2) return cg::record_error(CG_ERR_ARG, "field_kind must be 2 (UniformDensityField)");
  if (f->n_binders < 1 || f->n_binders > CG_MAX_BINDERS)
    return cg::record_error(CG_ERR_ARG, "n_binders must be in 1..3");
  if (f->nx < 1 || f->ny < 1 || f->nz < 1) return cg::record_error(CG_ERR_ARG, "grid dims must be >= 1");
  if (!(f->x_width > 0 && f->y_width > 0 && f->z_width > 0))
    return cg::record_error(CG_ERR_ARG, "box widths must be > 0");
  if (n_beads < 0 || n_beads > 2000000000LL) return cg::record_error(CG_ERR_ARG, "n_beads must be in 0..2e9");
  if (n_beads > 0 && (!r || !states)) return cg::record_error(CG_ERR_ARG, "null chain arrays");
  if (f->nx > kStaticCells || f->ny > kStaticCells || f->nz > kStaticCells)
    return cg::record_error(CG_ERR_ARG, "grid larger than the static scratch (1048576 cells)");
  const long long n_vox = (long long)f->nx * f->ny * f->nz;
  const long long cells = n_vox * (f->n_binders + 1);
  if (n_vox > kStaticCells || cells > kStaticCells)
    return cg::record_error(CG_ERR_ARG, "grid needs " + std::to_string(n_vox) + " voxels x " +
                                            std::to_string(f->n_binders + 1) +
                                            " columns; the static scratch holds 1048576 cells");
  if (n_beads > 0) {
    if (int rc = device_pointer(r, "r")) return rc;
    if (int rc = device_pointer(states, "states")) return rc;
  }
  if (access_vol)
    if (int rc = device_pointer(access_vol, "access_vol")) return rc;
  if (int rc = device_pointer(out, "out")) return rc;

  long long* scratch = nullptr;
  if (int rc = scratch_on_device(&scratch)) return rc;
  long long* grid = scratch;
  unsigned long long* doubly = reinterpret_cast<unsigned long long*>(scratch + kStaticCells);

  RepDev rd;
  memset(&rd, 0, sizeof rd);
  rd.n_beads = n_beads;
  rd.n_vox = n_vox;
  rd.nx = f->nx; rd.ny = f->ny; rd.nz = f->nz; rd.nb = f->n_binders;
  rd.wx = f->x_width; rd.wy = f->y_width; rd.wz = f->z_width;
  rd.dx = f->x_width / f->nx; rd.dy = f->y_width / f->ny; rd.dz = f->z_width / f->nz;
  rd.vol_bin = f->x_width * f->y_width * f->z_width / (double)n_vox;
  rd.field_kind = 2;
  rd.chi = f->chi; rd.vf_limit = f->vf_limit; rd.bead_vol = f->bead_vol;
  for (int b = 0; b < CG_MAX_BINDERS; b++) { rd.pref[b] = f->pref[b]; rd.intra[b] = f->intra[b]; }
  for (int b = 0; b < CG_MAX_BINDERS * CG_MAX_BINDERS; b++) rd.xpref[b] = f->xpref[b];
  rd.has_access = access_vol ? 1 : 0;

  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemsetAsync(grid, 0, sizeof(long long) * cells, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(doubly, 0, sizeof(unsigned long long) * kStaticFlags, s);
  if (e != cudaSuccess) return cg::record_error(CG_ERR_CUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));
  if (n_beads > 0) {
    long long blocks = (n_beads + 255) / 256;
    if (blocks > 152 * 8) blocks = 152 * 8;
    static_deposit_kernel<<<(unsigned)blocks, 256, 0, s>>>(rd, r, reinterpret_cast<const long long*>(states),
                                                           grid, doubly);
  }
  static_energy_kernel<<<1, 256, 0, s>>>(rd, grid, doubly, access_vol, out);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cg::record_error(CG_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
  return CG_OK;
}
