// Diagnostics reduction and the storage dispatch of the update kernels.
#include <cfloat>
#include <climits>
#include <cstdint>
#include <cstdio>

#include "mcb.h"
#include "solver.h"

namespace mcb {

cudaError_t launch_phi_f32(int variant, int gmode, const StepArgs& a, cudaStream_t s);
cudaError_t launch_phi_f16(int variant, int gmode, const StepArgs& a, cudaStream_t s);
cudaError_t launch_phi_bf16(int variant, int gmode, const StepArgs& a, cudaStream_t s);
cudaError_t launch_collide_f32(int variant, int gmode, const StepArgs& a, const void* tmap,
                               cudaStream_t s);
cudaError_t prepare_tma_f32();
size_t tma_smem_f32();
cudaError_t launch_collide_f16(int variant, int gmode, const StepArgs& a, const void* tmap,
                               cudaStream_t s);
cudaError_t prepare_tma_f16();
size_t tma_smem_f16();
cudaError_t launch_collide_bf16(int variant, int gmode, const StepArgs& a, const void* tmap,
                               cudaStream_t s);
cudaError_t prepare_tma_bf16();
size_t tma_smem_bf16();
cudaError_t occupancy_f32(int variant, int gmode, int qf, int ratio, int wide,
                          int* phi_blocks, int* collide_blocks);
cudaError_t occupancy_f16(int variant, int gmode, int qf, int ratio, int wide,
                          int* phi_blocks, int* collide_blocks);
cudaError_t occupancy_bf16(int variant, int gmode, int qf, int ratio, int wide,
                          int* phi_blocks, int* collide_blocks);
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
    // with a density ratio the rho field holds p / cs^2; the energy takes the density
    const double rk = cd->drho != 0.f ? static_cast<double>(cd->rho_out) +
                                            static_cast<double>(cd->drho) * phi
                                      : static_cast<double>(rho);
    d.ke += 0.5 * rk * u2;
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

// ------------------------------------------------- initial-field scan (set_fields) --

// Sum and first non-finite index of n floats, on a fixed grid with a fixed reduction order
// (the same result on every run): block b writes partial b, one thread then merges the
// partials in block order.
__global__ void __launch_bounds__(kDiagThreads)
    k_field_scan(const float* v, long long n, double* psum, long long* pbad) {
  double sum = 0.0;
  long long bad = LLONG_MAX;
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  for (long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += stride) {
    const float x = v[i];
    if (isfinite(x)) sum += x;
    else bad = min(bad, i);
  }
  for (int off = 16; off > 0; off >>= 1) {
    sum += __shfl_down_sync(0xffffffffu, sum, off);
    bad = min(bad, __shfl_down_sync(0xffffffffu, bad, off));
  }
  __shared__ double wsum[kDiagThreads / 32];
  __shared__ long long wbad[kDiagThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    wsum[warp] = sum;
    wbad[warp] = bad;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = wsum[0];
    long long b = wbad[0];
    for (int w = 1; w < kDiagThreads / 32; ++w) {
      s += wsum[w];
      b = min(b, wbad[w]);
    }
    psum[blockIdx.x] = s;
    pbad[blockIdx.x] = b;
  }
}

__global__ void k_field_scan_final(const double* psum, const long long* pbad, int nparts,
                                   double* out_sum, long long* out_bad) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double s = 0.0;
  long long b = LLONG_MAX;
  for (int i = 0; i < nparts; ++i) {
    s += psum[i];
    b = min(b, pbad[i]);
  }
  *out_sum = s;
  *out_bad = b;
}

// ------------------------------------------ allocation-free diagnostics (new kernels) --

// The reduction of k_diag over caller-owned device fields, with sizes by value. P may be
// null, in which case the Q2.30 sum is taken from phi.
__global__ void __launch_bounds__(kDiagThreads)
    k_diag_fields(int nx, int ny, int nz, int ref, const float* phi_a, const float* rho_a,
                  const float* ux_a, const float* uy_a, const float* uz_a, const int* p_a,
                  DiagPartial* partials) {
  const long long n = static_cast<long long>(nx) * ny * nz;
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
    const float phi = phi_a[i];
    const float rho = rho_a[i];
    const float ux = ux_a[i];
    const float uy = uy_a[i];
    const float uz = uz_a[i];
    d.mass_q30 += p_a ? p_a[i] : __float2int_rn(phi * 1073741824.0f);
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
    partials[blockIdx.x] = b;
  }
}

// Merges the partials in block order into partials[nparts].
__global__ void k_diag_fields_final(DiagPartial* partials, int nparts) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  DiagPartial r = partials[0];
  for (int i = 1; i < nparts; ++i) diag_merge(r, partials[i]);
  r.mass = static_cast<double>(r.mass_q30) * (1.0 / 1073741824.0);
  partials[nparts] = r;
}

}  // namespace

cudaError_t launch_phi(int storage, int variant, int gmode, const StepArgs& a,
                       cudaStream_t s) {
  switch (storage) {
    case kStF32: return launch_phi_f32(variant, gmode, a, s);
    case kStF16: return launch_phi_f16(variant, gmode, a, s);
    case kStBF16: return launch_phi_bf16(variant, gmode, a, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_collide(int storage, int variant, int gmode, const StepArgs& a,
                           const void* tmap_in, cudaStream_t s) {
  switch (storage) {
    case kStF32: return launch_collide_f32(variant, gmode, a, tmap_in, s);
    case kStF16: return launch_collide_f16(variant, gmode, a, tmap_in, s);
    case kStBF16: return launch_collide_bf16(variant, gmode, a, tmap_in, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t prepare_tma(int storage) {
  switch (storage) {
    case kStF32: return prepare_tma_f32();
    case kStF16: return prepare_tma_f16();
    case kStBF16: return prepare_tma_bf16();
    default: return cudaErrorInvalidValue;
  }
}

size_t tma_smem_bytes(int storage) {
  switch (storage) {
    case kStF32: return tma_smem_f32();
    case kStF16: return tma_smem_f16();
    case kStBF16: return tma_smem_bf16();
    default: return 0;
  }
}

cudaError_t occupancy(int storage, int variant, int gmode, int qf, int ratio, int wide,
                      int* phi_blocks, int* collide_blocks) {
  switch (storage) {
    case kStF32: return occupancy_f32(variant, gmode, qf, ratio, wide, phi_blocks, collide_blocks);
    case kStF16: return occupancy_f16(variant, gmode, qf, ratio, wide, phi_blocks, collide_blocks);
    case kStBF16: return occupancy_bf16(variant, gmode, qf, ratio, wide, phi_blocks, collide_blocks);
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

cudaError_t launch_field_scan(const float* v, long long n, void* partials, void* result,
                              cudaStream_t s) {
  double* psum = static_cast<double*>(partials);
  long long* pbad = reinterpret_cast<long long*>(psum + kDiagBlocks);
  double* out_sum = static_cast<double*>(result);
  long long* out_bad = reinterpret_cast<long long*>(out_sum + 1);
  k_field_scan<<<kDiagBlocks, kDiagThreads, 0, s>>>(v, n, psum, pbad);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_field_scan_final<<<1, 32, 0, s>>>(psum, pbad, kDiagBlocks, out_sum, out_bad);
  return cudaGetLastError();
}

cudaError_t launch_diag(const DiagArgs& a, cudaStream_t s) {
  k_diag<<<kDiagBlocks, kDiagThreads, 0, s>>>(a);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_diag_final<<<1, 32, 0, s>>>(a, kDiagBlocks);
  return cudaGetLastError();
}

}  // namespace mcb

// ------------------------------------------------------ mcb_diagnostics_device (C ABI) --
//
// Some callers cannot call cudaMalloc. A host code that owns every byte of device memory
// through its own pool, sized once at start-up, forbids later allocations. So does a
// driver loop that must not risk the device-wide synchronisation cudaFree can imply.
// mcb_diagnostics_device serves them:
//   - its only scratch is the file-scope array below;
//   - the caller passes the fields and receives the result;
//   - nothing is allocated on the device or the host.

// One partial record per reduction block plus the merged result: (304 + 1) records of 96
// bytes, about 29 KB. It is the maximum, whatever the lattice size, because the reduction
// grid is fixed. Every GPU that loads this library holds the array until the process
// exits. All calls share it.
static __device__ __align__(256) mcb::DiagPartial g_diag_scratch[mcb::kDiagBlocks + 1];

namespace {

thread_local char g_dev_err[256];

int dev_fail(int code, const char* msg, cudaError_t e = cudaSuccess) {
  std::snprintf(g_dev_err, sizeof g_dev_err, "%s%s%s", msg, e != cudaSuccess ? ": " : "",
                e != cudaSuccess ? cudaGetErrorString(e) : "");
  mcb::report_error(code, g_dev_err);
  return code;
}

// Device address of the scratch array in the current context. In host code the array's name
// is only a host-side stand-in, so the address comes from cudaGetSymbolAddress. It is looked
// up on every call, not cached: it is not a stream operation, it costs far less than the
// reduction, and a context torn down and created again (cudaDeviceReset, for one) may load the
// module at another address, which a cached pointer would miss.
int scratch_in_current_context(mcb::DiagPartial** out) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_diag_scratch);
  if (e != cudaSuccess || !p)
    return dev_fail(MCB_ERR_CUDA, "cudaGetSymbolAddress of the diagnostics scratch failed", e);
  *out = static_cast<mcb::DiagPartial*>(p);
  return MCB_OK;
}

}  // namespace

extern "C" int mcb_diagnostics_device(const float* phi, const float* rho, const float* ux,
                                      const float* uy, const float* uz,
                                      const int32_t* phi_q30, int nx, int ny, int nz, int bc,
                                      void* stream, mcb_diag* out) {
  if (!out || !phi || !rho || !ux || !uy || !uz)
    return dev_fail(MCB_ERR_INVALID, "mcb_diagnostics_device: NULL field or output pointer");
  if (nx < 1 || ny < 1 || nz < 1)
    return dev_fail(MCB_ERR_INVALID, "mcb_diagnostics_device: sizes must be >= 1");
  if (static_cast<long long>(nx) * ny * nz > MCB_DIAG_DEVICE_MAX_CELLS)
    return dev_fail(MCB_ERR_INVALID,
                    "mcb_diagnostics_device: more than 2^31-1 cells (MCB_DIAG_DEVICE_MAX_CELLS)");
  if (bc != MCB_BC_REF && bc != MCB_BC_PERIODIC && bc != MCB_BC_WALLS_Z)
    return dev_fail(MCB_ERR_INVALID, "mcb_diagnostics_device: unknown boundary mode");
  mcb::DiagPartial* scratch = nullptr;
  const int rc = scratch_in_current_context(&scratch);
  if (rc != MCB_OK) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  mcb::k_diag_fields<<<mcb::kDiagBlocks, mcb::kDiagThreads, 0, s>>>(
      nx, ny, nz, bc == MCB_BC_REF, phi, rho, ux, uy, uz, phi_q30, scratch);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return dev_fail(MCB_ERR_CUDA, "diagnostics launch failed", e);
  mcb::k_diag_fields_final<<<1, 32, 0, s>>>(scratch, mcb::kDiagBlocks);
  e = cudaGetLastError();
  if (e != cudaSuccess) return dev_fail(MCB_ERR_CUDA, "diagnostics launch failed", e);
  mcb::DiagPartial r;
  e = cudaMemcpyAsync(&r, scratch + mcb::kDiagBlocks, sizeof r, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return dev_fail(MCB_ERR_CUDA, "diagnostics read-back failed", e);
  out->mass = r.mass;
  out->mass_q30 = r.mass_q30;
  out->kinetic = r.ke;
  out->umax = r.umax;
  out->n_in = r.n_in;
  out->n_out = r.n_out;
  out->rho_in = r.n_in > 0 ? r.rho_in / r.n_in : 0.0;
  out->rho_out = r.n_out > 0 ? r.rho_out / r.n_out : 0.0;
  out->dp = (r.n_in > 0 && r.n_out > 0) ? (out->rho_in - out->rho_out) / 3.0 : 0.0;
  out->vol_half = r.vol_half;
  out->phi_min = r.phi_min;
  out->phi_max = r.phi_max;
  out->finite = r.nonfinite == 0;
  out->update = -1;
  if (!out->finite) return dev_fail(MCB_ERR_NUMERIC, "mcb_diagnostics_device: non-finite values");
  return MCB_OK;
}
