// cg_steric.cu -- steric clash energy of bead pairs on the device.
//
// The detailed chromatin model with sterics (DetailedChromatinWithSterics,
// chromo/polymers.pyx:2738-2938) adds, for every pair of beads closer than
// the excluded distance e (twice the bead radius), V0 ((e/d)^12 - 2 (e/d)^6 + 1).
// The reference keeps an N x N distance matrix and refreshes the rows of the
// moved beads each move (get_delta_distances); here distances are computed on
// the fly from the resident positions, one CTA per row (a moved bead against
// every bead: the O(m N) update of one move), and the rows' partial sums are
// added in row order, so the results are deterministic.
#include <cuda_runtime.h>

#include "cg_kernels.h"

namespace cg {

__device__ __forceinline__ double clash_energy(double d, double e, double V0) {
  if (!(d < e)) return 0.0;
  const double f = e / d;
  return V0 * (pow(f, 12.0) - 2 * pow(f, 6.0) + 1);
}

__device__ __forceinline__ double dist3(const double a[3], const double b[3]) {
  const double x = a[0] - b[0], y = a[1] - b[1], z = a[2] - b[2];
  return sqrt(x * x + y * y + z * z);
}

__device__ __forceinline__ double row_total(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  double t = 0;
  if (threadIdx.x < 32) {
    t = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(kFull, t, o);
  }
  return t;
}

// Row i of the clash energy (pairs i < j), or with trial != null the change of
// moved bead i = ind0 + blockIdx.x: trial positions of [ind0, indf) in trial
// (m x 3), pairs with a moved j >= i skipped (counted once).
template <typename Pos>
__global__ void steric_rows_kernel(KArgs a, int rep, long long ind0, long long indf, const double* trial,
                                   double e, double V0, double* rows) {
  __shared__ double sh[32];
  const RepDev& rd = a.reps[rep];
  const V4<Pos>* r4 = reinterpret_cast<const V4<Pos>*>(a.r4) + rd.bead_off;
  const long long N = rd.n_beads;
  const long long i = trial ? ind0 + blockIdx.x : (long long)blockIdx.x;
  double ri[3];
  ld3(r4, i, ri);
  double part = 0;
  if (!trial) {
    for (long long j = i + 1 + threadIdx.x; j < N; j += blockDim.x) {
      double rj[3];
      ld3(r4, j, rj);
      part += clash_energy(dist3(ri, rj), e, V0);
    }
  } else {
    const double* ti = trial + 3 * (i - ind0);
    for (long long j = threadIdx.x; j < N; j += blockDim.x) {
      const bool moved = j >= ind0 && j < indf;
      if (moved && j >= i) continue;
      double rj[3], tj[3];
      ld3(r4, j, rj);
      if (moved) { tj[0] = trial[3 * (j - ind0)]; tj[1] = trial[3 * (j - ind0) + 1]; tj[2] = trial[3 * (j - ind0) + 2]; }
      else { tj[0] = rj[0]; tj[1] = rj[1]; tj[2] = rj[2]; }
      part += clash_energy(dist3(ti, tj), e, V0) - clash_energy(dist3(ri, rj), e, V0);
    }
  }
  const double t = row_total(part, sh);
  if (threadIdx.x == 0) rows[blockIdx.x] = t;
}

// out[0] = the rows added in order (one thread: deterministic)
__global__ void steric_sum_kernel(const double* rows, long long n, double* out) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    double s = 0;
    for (long long k = 0; k < n; k++) s += rows[k];
    out[0] = s;
  }
}

}  // namespace cg

void cg_launch_steric(const cg::KArgs& a, bool fp64, int rep, long long n_rows, long long ind0, long long indf,
                      const double* trial, double e, double V0, double* rows, double* out, cudaStream_t s) {
  if (fp64) cg::steric_rows_kernel<double><<<(unsigned)n_rows, 256, 0, s>>>(a, rep, ind0, indf, trial, e, V0, rows);
  else cg::steric_rows_kernel<float><<<(unsigned)n_rows, 256, 0, s>>>(a, rep, ind0, indf, trial, e, V0, rows);
  cg::steric_sum_kernel<<<1, 32, 0, s>>>(rows, n_rows, out);
}
