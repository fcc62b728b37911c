// cg_spec.cu -- dispatch of the production MC kernel (cg_spec.cuh) over its
// instantiations: FP32 storage with 8, 16 or 32 lanes per move, FP64 storage
// with 32 (the reference-arithmetic mode, where speed is secondary).  Each
// instantiation is compiled in its own translation unit (cg_spec_*.cu).
#include <mutex>

#include "cg_kernels.h"

void cg_launch_spec_f8(const cg::KArgs& a, size_t smem, cudaStream_t s);
void cg_launch_spec_f16(const cg::KArgs& a, size_t smem, cudaStream_t s);
void cg_launch_spec_f32(const cg::KArgs& a, size_t smem, cudaStream_t s);
void cg_launch_spec_d32(const cg::KArgs& a, size_t smem, cudaStream_t s);
cudaError_t cg_spec_smem_f8(int bytes);
cudaError_t cg_spec_smem_f16(int bytes);
cudaError_t cg_spec_smem_f32(int bytes);
cudaError_t cg_spec_smem_d32(int bytes);
int cg_spec_regs_f8();
int cg_spec_regs_f16();
int cg_spec_regs_f32();
int cg_spec_regs_d32();

bool cg_spec_shape_ok(bool fp64, int g) { return fp64 ? g == 32 : (g == 8 || g == 16 || g == 32); }

void cg_launch_spec(const cg::KArgs& a, bool fp64, size_t smem_bytes, cudaStream_t s) {
  if (fp64) cg_launch_spec_d32(a, smem_bytes, s);
  else if (a.spec_g == 8) cg_launch_spec_f8(a, smem_bytes, s);
  else if (a.spec_g == 16) cg_launch_spec_f16(a, smem_bytes, s);
  else cg_launch_spec_f32(a, smem_bytes, s);
}

// The dynamic shared-memory limit is an attribute of the kernel (per device),
// shared by every simulation in the process: it is only ever raised, so that
// creating a simulation with a smaller layout never breaks the launches of a
// live one with a larger layout.
namespace {
constexpr int kMaxDevices = 64;
std::mutex g_smem_mu;
int g_spec_smem[kMaxDevices][4];
}  // namespace

cudaError_t cg_set_spec_smem(bool fp64, int g, int bytes) {
  const int k = fp64 ? 3 : g == 8 ? 0 : g == 16 ? 1 : 2;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lock(g_smem_mu);
  int* cur = dev >= 0 && dev < kMaxDevices ? &g_spec_smem[dev][k] : nullptr;
  if (cur && bytes <= *cur) return cudaSuccess;
  if (fp64) e = cg_spec_smem_d32(bytes);
  else if (g == 8) e = cg_spec_smem_f8(bytes);
  else if (g == 16) e = cg_spec_smem_f16(bytes);
  else e = cg_spec_smem_f32(bytes);
  if (e == cudaSuccess && cur) *cur = bytes;
  return e;
}

int cg_spec_warps_per_sm(bool fp64, int g) {
  const int regs = fp64 ? cg_spec_regs_d32()
                 : g == 8 ? cg_spec_regs_f8() : g == 16 ? cg_spec_regs_f16() : cg_spec_regs_f32();
  if (regs <= 0) return cg::kMaxW;
  const int per_warp = (regs * 32 + 255) / 256 * 256;  // allocation unit: 256 registers
  return 65536 / per_warp;
}
