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
// NULL to skip) is copied to the device first.  An upload is read once from
// the host, checked (non-finite coordinates, states outside 0..3) and written
// into device staging arrays of the resident layout; only an upload that
// passed is then copied into the resident state (device to device), so a
// rejected upload leaves the resident state unchanged, as the host-staged
// path does.  Without room for the device staging arrays, the upload is
// checked in a first pass over the host arrays and written in a second.
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
// range); mode 1: write a's storage; mode 2: check and write.
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
      if (mode != 1 && !isfinite(x)) bad |= 1u;
      if (mode != 0) dst[k][4 * (j / 3) + j % 3] = (Pos)x;  // the 4-vector's pad stays 0
    }
  }
  if (row.st) {
    unsigned char* sb = reinterpret_cast<unsigned char*>(a.states + off);
    for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < n * nb; j += stride) {
      const long long v = row.st[j];
      if (v < 0 || v > CG_MAX_MARK) bad |= 2u;
      else if (mode != 0) sb[4 * (j / nb) + j % nb] = (unsigned char)v;  // byte b of bead i's word
    }
  }
  if (bad) atomicOr(flag, bad);
}

// Copy the arrays an upload gave (the table's non-NULL entries) from the
// staging arrays (same layout) into the resident state.
template <typename Pos>
__global__ void stage_commit_kernel(KArgs a, const HostRow* tab, const V4<Pos>* s_r, const V4<Pos>* s_t3,
                                    const V4<Pos>* s_t2, const unsigned* s_st) {
  const int rep = blockIdx.y;
  const RepDev& rd = a.reps[rep];
  const long long n = rd.n_beads, off = rd.bead_off;
  const HostRow row = tab[rep];
  const bool give[3] = {row.r != nullptr, row.t3 != nullptr, row.t2 != nullptr};
  const V4<Pos>* src[3] = {s_r + off, s_t3 + off, s_t2 + off};
  V4<Pos>* dst[3] = {reinterpret_cast<V4<Pos>*>(a.r4) + off, reinterpret_cast<V4<Pos>*>(a.t34) + off,
                     reinterpret_cast<V4<Pos>*>(a.t24) + off};
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (int k = 0; k < 3; k++) {
    if (!give[k]) continue;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += stride) dst[k][i] = src[k][i];
  }
  if (row.st)
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += stride)
      a.states[off + i] = s_st[off + i];
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

void cg_launch_stage_commit(const cg::KArgs& a, bool fp64, const void* tab, int R, long long max_beads,
                            const void* s_r, const void* s_t3, const void* s_t2, const unsigned* s_st,
                            cudaStream_t s) {
  const auto* t = static_cast<const cg::HostRow*>(tab);
  const dim3 grid = hostio_grid(R, (max_beads + 2) / 3);  // one thread per bead
  if (fp64)
    cg::stage_commit_kernel<double><<<grid, 256, 0, s>>>(a, t, static_cast<const cg::V4<double>*>(s_r),
                                                         static_cast<const cg::V4<double>*>(s_t3),
                                                         static_cast<const cg::V4<double>*>(s_t2), s_st);
  else
    cg::stage_commit_kernel<float><<<grid, 256, 0, s>>>(a, t, static_cast<const cg::V4<float>*>(s_r),
                                                        static_cast<const cg::V4<float>*>(s_t3),
                                                        static_cast<const cg::V4<float>*>(s_t2), s_st);
}

void cg_launch_host_store(const cg::KArgs& a, bool fp64, const void* tab, int R, long long max_beads, int nb,
                          cudaStream_t s) {
  const auto* t = static_cast<const cg::HostRow*>(tab);
  if (fp64) cg::host_store_kernel<double><<<hostio_grid(R, max_beads), 256, 0, s>>>(a, t, nb);
  else cg::host_store_kernel<float><<<hostio_grid(R, max_beads), 256, 0, s>>>(a, t, nb);
}
