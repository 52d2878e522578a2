// Diagnostics reduction and the storage dispatch of the update kernels.
#include <cfloat>

#include "solver.h"

namespace mcb {

cudaError_t launch_phi_f32(int variant, const StepArgs& a, cudaStream_t s);
cudaError_t launch_phi_f16(int variant, const StepArgs& a, cudaStream_t s);
cudaError_t launch_phi_bf16(int variant, const StepArgs& a, cudaStream_t s);
cudaError_t launch_collide_f32(int variant, bool bgk, const StepArgs& a, cudaStream_t s);
cudaError_t launch_collide_f16(int variant, bool bgk, const StepArgs& a, cudaStream_t s);
cudaError_t launch_collide_bf16(int variant, bool bgk, const StepArgs& a, cudaStream_t s);
cudaError_t launch_init_f32(const InitArgs& a, int nx, int ny, int nz, cudaStream_t s);
cudaError_t launch_init_f16(const InitArgs& a, int nx, int ny, int nz, cudaStream_t s);
cudaError_t launch_init_bf16(const InitArgs& a, int nx, int ny, int nz, cudaStream_t s);

namespace {

// ----------------------------------------------------------- diagnostics reduction --

__device__ __forceinline__ void diag_zero(DiagPartial& d) {
  d.mass = d.ke = d.umax = d.rho_in = d.n_in = d.rho_out = d.n_out = d.vol_half = 0.0;
  d.phi_min = DBL_MAX;
  d.phi_max = -DBL_MAX;
  d.mass_q30 = 0;
  d.nonfinite = 0;
}
__device__ __forceinline__ void diag_merge(DiagPartial& a, const DiagPartial& b) {
  a.mass += b.mass;
  a.ke += b.ke;
  a.umax = fmax(a.umax, b.umax);
  a.rho_in += b.rho_in;
  a.n_in += b.n_in;
  a.rho_out += b.rho_out;
  a.n_out += b.n_out;
  a.vol_half += b.vol_half;
  a.phi_min = fmin(a.phi_min, b.phi_min);
  a.phi_max = fmax(a.phi_max, b.phi_max);
  a.mass_q30 += b.mass_q30;
  a.nonfinite += b.nonfinite;
}
__device__ __forceinline__ void diag_shfl(DiagPartial& d, int off) {
  DiagPartial o;
  o.mass = __shfl_down_sync(0xffffffffu, d.mass, off);
  o.ke = __shfl_down_sync(0xffffffffu, d.ke, off);
  o.umax = __shfl_down_sync(0xffffffffu, d.umax, off);
  o.rho_in = __shfl_down_sync(0xffffffffu, d.rho_in, off);
  o.n_in = __shfl_down_sync(0xffffffffu, d.n_in, off);
  o.rho_out = __shfl_down_sync(0xffffffffu, d.rho_out, off);
  o.n_out = __shfl_down_sync(0xffffffffu, d.n_out, off);
  o.vol_half = __shfl_down_sync(0xffffffffu, d.vol_half, off);
  o.phi_min = __shfl_down_sync(0xffffffffu, d.phi_min, off);
  o.phi_max = __shfl_down_sync(0xffffffffu, d.phi_max, off);
  o.mass_q30 = __shfl_down_sync(0xffffffffu, d.mass_q30, off);
  o.nonfinite = __shfl_down_sync(0xffffffffu, d.nonfinite, off);
  diag_merge(d, o);
}

// FP64 sums over one case with a fixed grid and a fixed reduction tree, so the result is
// the same on every run.
__global__ void __launch_bounds__(kDiagThreads) k_diag(const DiagArgs a) {
  const CaseDesc* cd = a.cases + a.case_index;
  const int nx = cd->nx, ny = cd->ny, nz = cd->nz;
  const bool ref = cd->bc == kBcRef;
  const long long n = cd->ncell, co = cd->cell_off, T = a.cells_total;
  DiagPartial d;
  diag_zero(d);
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  for (long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += stride) {
    if (ref) {
      const int x = static_cast<int>(i % nx);
      const int y = static_cast<int>((i / nx) % ny);
      const int z = static_cast<int>(i / (static_cast<long long>(nx) * ny));
      if (x == 0 || x == nx - 1 || y == 0 || y == ny - 1 || z == 0 || z == nz - 1) continue;
    }
    const float phi = a.macros[co + i];
    const float rho = a.macros[T + co + i];
    const float ux = a.macros[2 * T + co + i];
    const float uy = a.macros[3 * T + co + i];
    const float uz = a.macros[4 * T + co + i];
    const int P = a.p[co + i];
    d.mass_q30 += P;
    const double u2 = static_cast<double>(ux) * ux + static_cast<double>(uy) * uy +
                      static_cast<double>(uz) * uz;
    d.ke += 0.5 * static_cast<double>(rho) * u2;
    d.umax = fmax(d.umax, sqrt(u2));
    if (phi > 0.99f) { d.rho_in += rho; d.n_in += 1.0; }
    if (phi < 0.01f) { d.rho_out += rho; d.n_out += 1.0; }
    if (phi > 0.5f) d.vol_half += 1.0;
    d.phi_min = fmin(d.phi_min, static_cast<double>(phi));
    d.phi_max = fmax(d.phi_max, static_cast<double>(phi));
    if (!isfinite(phi) || !isfinite(rho) || !isfinite(ux) || !isfinite(uy) || !isfinite(uz))
      d.nonfinite += 1;
  }
  for (int off = 16; off > 0; off >>= 1) diag_shfl(d, off);
  __shared__ DiagPartial warp_part[kDiagThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) warp_part[warp] = d;
  __syncthreads();
  if (threadIdx.x == 0) {
    DiagPartial b = warp_part[0];
    for (int w = 1; w < kDiagThreads / 32; ++w) diag_merge(b, warp_part[w]);
    a.partials[blockIdx.x] = b;
  }
}

__global__ void k_diag_final(const DiagArgs a, int nparts) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  DiagPartial r = a.partials[0];
  for (int i = 1; i < nparts; ++i) diag_merge(r, a.partials[i]);
  r.mass = static_cast<double>(r.mass_q30) * (1.0 / 1073741824.0);
  *a.result = r;
}

}  // namespace

cudaError_t launch_phi(int storage, int variant, const StepArgs& a, cudaStream_t s) {
  switch (storage) {
    case kStF32: return launch_phi_f32(variant, a, s);
    case kStF16: return launch_phi_f16(variant, a, s);
    case kStBF16: return launch_phi_bf16(variant, a, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_collide(int storage, int variant, bool bgk, const StepArgs& a,
                           cudaStream_t s) {
  switch (storage) {
    case kStF32: return launch_collide_f32(variant, bgk, a, s);
    case kStF16: return launch_collide_f16(variant, bgk, a, s);
    case kStBF16: return launch_collide_bf16(variant, bgk, a, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_init(int storage, const InitArgs& a, int nx, int ny, int nz,
                        cudaStream_t s) {
  switch (storage) {
    case kStF32: return launch_init_f32(a, nx, ny, nz, s);
    case kStF16: return launch_init_f16(a, nx, ny, nz, s);
    case kStBF16: return launch_init_bf16(a, nx, ny, nz, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_diag(const DiagArgs& a, cudaStream_t s) {
  k_diag<<<kDiagBlocks, kDiagThreads, 0, s>>>(a);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_diag_final<<<1, 32, 0, s>>>(a, kDiagBlocks);
  return cudaGetLastError();
}

}  // namespace mcb
