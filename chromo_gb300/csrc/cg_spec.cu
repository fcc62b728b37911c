// cg_spec.cu -- dispatch of the production MC kernel (cg_spec.cuh) over its
// instantiations: FP32 storage with 8, 16 or 32 lanes per move, FP64 storage
// with 32 (the reference-arithmetic mode, where speed is secondary).  Each
// instantiation is compiled in its own translation unit (cg_spec_*.cu).
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

cudaError_t cg_set_spec_smem(bool fp64, int g, int bytes) {
  if (fp64) return cg_spec_smem_d32(bytes);
  if (g == 8) return cg_spec_smem_f8(bytes);
  if (g == 16) return cg_spec_smem_f16(bytes);
  return cg_spec_smem_f32(bytes);
}

int cg_spec_warps_per_sm(bool fp64, int g) {
  const int regs = fp64 ? cg_spec_regs_d32()
                 : g == 8 ? cg_spec_regs_f8() : g == 16 ? cg_spec_regs_f16() : cg_spec_regs_f32();
  if (regs <= 0) return cg::kMaxW;
  const int per_warp = (regs * 32 + 255) / 256 * 256;  // allocation unit: 256 registers
  return 65536 / per_warp;
}
