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

// mode 0: check only (flag bit 1: non-finite coordinate, bit 2: state out of
// range); mode 1: write the resident storage.
template <typename Pos>
__global__ void host_load_kernel(KArgs a, const HostRow* tab, int nb, unsigned* flag, int mode) {
  const int rep = blockIdx.y;
  const RepDev& rd = a.reps[rep];
  const long long n = rd.n_beads, off = rd.bead_off;
  const HostRow row = tab[rep];
  const double* src[3] = {row.r, row.t3, row.t2};
  V4<Pos>* dst[3] = {reinterpret_cast<V4<Pos>*>(a.r4) + off, reinterpret_cast<V4<Pos>*>(a.t34) + off,
                     reinterpret_cast<V4<Pos>*>(a.t24) + off};
  unsigned bad = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
      if (!src[k]) continue;
      const double x = src[k][3 * i], y = src[k][3 * i + 1], z = src[k][3 * i + 2];
      if (mode == 0) {
        if (!(isfinite(x) && isfinite(y) && isfinite(z))) bad |= 1u;
      } else {
        dst[k][i] = V4<Pos>{(Pos)x, (Pos)y, (Pos)z, (Pos)0};
      }
    }
    if (row.st) {
      unsigned w = 0;
      for (int b = 0; b < nb; b++) {
        const long long v = row.st[i * nb + b];
        if (v < 0 || v > CG_MAX_MARK) bad |= 2u;
        w |= (unsigned)(v & 0xFF) << (8 * b);
      }
      if (mode == 1) a.states[off + i] = w;
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
  const V4<Pos>* src[3] = {reinterpret_cast<const V4<Pos>*>(a.r4) + off,
                           reinterpret_cast<const V4<Pos>*>(a.t34) + off,
                           reinterpret_cast<const V4<Pos>*>(a.t24) + off};
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
      if (!dst[k]) continue;
      const V4<Pos> v = src[k][i];
      dst[k][3 * i] = (double)v.x;
      dst[k][3 * i + 1] = (double)v.y;
      dst[k][3 * i + 2] = (double)v.z;
    }
    if (row.st) {
      const unsigned w = a.states[off + i];
      for (int b = 0; b < nb; b++) row.st[i * nb + b] = (long long)((w >> (8 * b)) & 0xFF);
    }
  }
}

}  // namespace cg

static dim3 hostio_grid(int R, long long max_beads) {
  long long bx = (max_beads + 255) / 256;
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
