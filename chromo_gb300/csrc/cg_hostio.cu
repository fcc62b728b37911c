// cg_hostio.cu -- chain transfers that read and write the caller's host
// arrays from the GPU itself.
//
// On a Grace-Blackwell node the GPU reaches pageable host memory through
// NVLink-C2C with the host's page tables (cudaDevAttrPageableMemoryAccess).
// cg_set_chains / cg_get_chains then move every replica's FP64 positions,
// tangents and int64 binding states in one kernel pass: the kernel reads the
// caller's numpy arrays where they lie and writes the resident 4-vectors (or
// the reverse), with no host-side conversion into a pinned buffer and no
// separate DMA.  The replica table (one host pointer per array and replica,
// NULL to skip) is copied to the device first.  Uploads are checked in a
// first pass (non-finite coordinates, states outside 0..3) and written in a
// second, so a rejected upload leaves the resident state unchanged, as the
// staged path does.
#include <cuda_runtime.h>

#include "cg_kernels.h"

namespace cg {

struct HostRow {  // one replica's host arrays (NULL: not transferred)
  double* r;
  double* t3;
  double* t2;
  long long* st;
};

// The host arrays are walked flat (element j of replica rep's [n x 3] or
// [n x nb] array on thread j), so every warp reads or writes 32 consecutive
// 8-byte words of host memory: whole 256-byte lines over the link.  The
// resident side takes the scattered accesses (HBM / L2).
//
// mode 0: check only (flag bit 1: non-finite coordinate, bit 2: state out of
// range); mode 1: write the resident storage.
template <typename Pos>
__global__ void host_load_kernel(KArgs a, const HostRow* tab, int nb, unsigned* flag, int mode) {
  const int rep = blockIdx.y;
  const RepDev& rd = a.reps[rep];
  const long long n = rd.n_beads, off = rd.bead_off;
  const HostRow row = tab[rep];
  const double* src[3] = {row.r, row.t3, row.t2};
  Pos* dst[3] = {reinterpret_cast<Pos*>(reinterpret_cast<V4<Pos>*>(a.r4) + off),
                 reinterpret_cast<Pos*>(reinterpret_cast<V4<Pos>*>(a.t34) + off),
                 reinterpret_cast<Pos*>(reinterpret_cast<V4<Pos>*>(a.t24) + off)};
  const long long stride = (long long)gridDim.x * blockDim.x;
  unsigned bad = 0;
  for (int k = 0; k < 3; k++) {
    if (!src[k]) continue;
    for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < 3 * n; j += stride) {
      const double x = src[k][j];
      if (mode == 0) {
        if (!isfinite(x)) bad |= 1u;
      } else {
        dst[k][4 * (j / 3) + j % 3] = (Pos)x;  // the 4-vector's pad stays 0
      }
    }
  }
  if (row.st) {
    unsigned char* sb = reinterpret_cast<unsigned char*>(a.states + off);
    for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < n * nb; j += stride) {
      const long long v = row.st[j];
      if (v < 0 || v > CG_MAX_MARK) bad |= 2u;
      else if (mode == 1) sb[4 * (j / nb) + j % nb] = (unsigned char)v;  // byte b of bead i's word
    }
  }
  if (bad) atomicOr(flag, bad);
}

template <typename Pos>
__global__ void host_store_kernel(KArgs a, const HostRow* tab, int nb) {
  const int rep = blockIdx.y;
  const RepDev& rd = a.reps[rep];
  const long long n = rd.n_beads, off = rd.bead_off;
  const HostRow row = tab[rep];
  double* dst[3] = {row.r, row.t3, row.t2};
  const Pos* src[3] = {reinterpret_cast<const Pos*>(reinterpret_cast<const V4<Pos>*>(a.r4) + off),
                       reinterpret_cast<const Pos*>(reinterpret_cast<const V4<Pos>*>(a.t34) + off),
                       reinterpret_cast<const Pos*>(reinterpret_cast<const V4<Pos>*>(a.t24) + off)};
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (int k = 0; k < 3; k++) {
    if (!dst[k]) continue;
    for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < 3 * n; j += stride)
      dst[k][j] = (double)src[k][4 * (j / 3) + j % 3];
  }
  if (row.st) {
    const unsigned char* sb = reinterpret_cast<const unsigned char*>(a.states + off);
    for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < n * nb; j += stride)
      row.st[j] = (long long)sb[4 * (j / nb) + j % nb];
  }
}

}  // namespace cg

static dim3 hostio_grid(int R, long long max_beads) {
  long long bx = (3 * max_beads + 255) / 256;
  if (bx > 64) bx = 64;
  if (bx < 1) bx = 1;
  return dim3((unsigned)bx, (unsigned)R);
}

void cg_launch_host_load(const cg::KArgs& a, bool fp64, const void* tab, int R, long long max_beads, int nb,
                         unsigned* flag, int mode, cudaStream_t s) {
  const auto* t = static_cast<const cg::HostRow*>(tab);
  if (fp64) cg::host_load_kernel<double><<<hostio_grid(R, max_beads), 256, 0, s>>>(a, t, nb, flag, mode);
  else cg::host_load_kernel<float><<<hostio_grid(R, max_beads), 256, 0, s>>>(a, t, nb, flag, mode);
}

void cg_launch_host_store(const cg::KArgs& a, bool fp64, const void* tab, int R, long long max_beads, int nb,
                          cudaStream_t s) {
  const auto* t = static_cast<const cg::HostRow*>(tab);
  if (fp64) cg::host_store_kernel<double><<<hostio_grid(R, max_beads), 256, 0, s>>>(a, t, nb);
  else cg::host_store_kernel<float><<<hostio_grid(R, max_beads), 256, 0, s>>>(a, t, nb);
}
