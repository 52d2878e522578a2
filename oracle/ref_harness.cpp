// TEST INFRASTRUCTURE ONLY: runs the reference's own CUDA kernels on the GPU.
//
// The kernels are the unmodified src/var.cu, src/init.cu and src/lbm.cu of
// kreeyto/MULTIC-BUBBLE-CUDA, compiled for sm_103a into a cubin by oracle/Makefile. This
// file holds none of that source. It loads the cubin with the CUDA driver API and finds
// the kernels by name. It then plays the role of the reference's initializeVars
// (src/var.cu:57-114) and main loop (src/main.cu:56-182):
//   - allocate the 22 arrays and memset them the same way;
//   - upload the __constant__ symbols;
//   - run initTensor; write a host-provided phi in place of initPhase; run initDist;
//   - run the ten step kernels in their intended order, on one stream.
// The reference issues collisionFluid and collisionPhase on two more streams with no
// dependency on the first, which is a race; this harness keeps them on one stream. Its
// outputs pin the CPU oracle and serve as the parity target for the solver.
#include <cuda.h>

#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace {

std::string g_err;

int fail(const char* what, CUresult r) {
  const char* s = nullptr;
  cuGetErrorString(r, &s);
  g_err = std::string(what) + ": " + (s ? s : "unknown CUDA error");
  return 1;
}

#define RH(call)                          \
  do {                                    \
    const CUresult r_ = (call);           \
    if (r_ != CUDA_SUCCESS) return fail(#call, r_); \
  } while (0)

enum K {
  kInitTensor, kInitPhase, kInitDist, kPhiCalc, kGradCalc, kCurvatureCalc, kMomentiCalc,
  kCollisionFluid, kCollisionPhase, kStreamingCalc, kFgBoundary, kBoundaryConditions,
  kMovingWallBC, kNumK
};
// Itanium-mangled name prefixes ("_Z" + length + name) of the reference's kernels.
const char* kNames[kNumK] = {
    "_Z10initTensor", "_Z9initPhase", "_Z8initDist", "_Z7phiCalc", "_Z8gradCalc",
    "_Z13curvatureCalc", "_Z11momentiCalc", "_Z14collisionFluid", "_Z14collisionPhase",
    "_Z13streamingCalc", "_Z10fgBoundary", "_Z18boundaryConditions", "_Z12movingWallBC"};

enum A {
  aRho, aPhi, aUx, aUy, aUz, aNx, aNy, aNz, aCurv, aInd, aFfx, aFfy, aFfz, aPxx, aPyy, aPzz,
  aPxy, aPxz, aPyz, aF, aG, aGout, kNumA
};

struct Ref {
  CUdevice dev = 0;
  CUcontext ctx = nullptr;
  CUmodule mod = nullptr;
  CUfunction k[kNumK] = {};
  CUdeviceptr a[kNumA] = {};
  CUstream stream = nullptr;
  // The reference's own stream layout (src/main.cu:49-52): collisionFluid and
  // collisionPhase on two more streams, created with default flags, not ordered after the
  // kernels of the main stream (src/main.cu:127-141). Only ref_run_streams(..., 3) uses them.
  CUstream coll_fluid = nullptr, coll_phase = nullptr;
  CUevent e0 = nullptr, e1 = nullptr;
  int NX = 0, NY = 0, NZ = 0;
  int moving_wall = 1;

  int launch(K which, std::vector<void*> args, CUstream on = nullptr) {
    const unsigned bx = 8, by = 8, bz = 8;
    const unsigned gx = (NX + 7) / 8, gy = (NY + 7) / 8, gz = (NZ + 7) / 8;
    RH(cuLaunchKernel(k[which], gx, gy, gz, bx, by, bz, 0, on ? on : stream, args.data(),
                      nullptr));
    return 0;
  }
};

}  // namespace

extern "C" {

const char* ref_error(void) { return g_err.c_str(); }

void* ref_open(const char* cubin_path, int device) {
  Ref* r = new Ref;
  auto bad = [&](const char* what, CUresult e) {
    fail(what, e);
    delete r;
    return static_cast<void*>(nullptr);
  };
  CUresult e;
  if ((e = cuInit(0)) != CUDA_SUCCESS) return bad("cuInit", e);
  if ((e = cuDeviceGet(&r->dev, device)) != CUDA_SUCCESS) return bad("cuDeviceGet", e);
  if ((e = cuDevicePrimaryCtxRetain(&r->ctx, r->dev)) != CUDA_SUCCESS)
    return bad("cuDevicePrimaryCtxRetain", e);
  if ((e = cuCtxSetCurrent(r->ctx)) != CUDA_SUCCESS) return bad("cuCtxSetCurrent", e);
  if ((e = cuModuleLoad(&r->mod, cubin_path)) != CUDA_SUCCESS) return bad("cuModuleLoad", e);
  unsigned count = 0;
  if ((e = cuModuleGetFunctionCount(&count, r->mod)) != CUDA_SUCCESS)
    return bad("cuModuleGetFunctionCount", e);
  std::vector<CUfunction> fs(count);
  if ((e = cuModuleEnumerateFunctions(fs.data(), count, r->mod)) != CUDA_SUCCESS)
    return bad("cuModuleEnumerateFunctions", e);
  for (CUfunction f : fs) {
    const char* name = nullptr;
    if (cuFuncGetName(&name, f) != CUDA_SUCCESS || !name) continue;
    for (int i = 0; i < kNumK; ++i)
      if (std::strncmp(name, kNames[i], std::strlen(kNames[i])) == 0) r->k[i] = f;
  }
  for (int i = 0; i < kNumK; ++i)
    if (!r->k[i]) {
      g_err = std::string("kernel not found in cubin: ") + kNames[i];
      delete r;
      return nullptr;
    }
  if ((e = cuStreamCreate(&r->stream, CU_STREAM_NON_BLOCKING)) != CUDA_SUCCESS)
    return bad("cuStreamCreate", e);
  if ((e = cuEventCreate(&r->e0, CU_EVENT_DEFAULT)) != CUDA_SUCCESS) return bad("cuEventCreate", e);
  if ((e = cuEventCreate(&r->e1, CU_EVENT_DEFAULT)) != CUDA_SUCCESS) return bad("cuEventCreate", e);
  return r;
}

// initializeVars (src/var.cu:57-114) with the size and the four scalars as parameters.
// The velocity set and weights are the D3Q19 tables of src/var.cu:29-45.
int ref_setup(void* h, int nx, int ny, int nz, float tau, float sigma, float sharp_c,
              int moving_wall) {
  Ref* r = static_cast<Ref*>(h);
  if (!r) return 1;
  // streamingCalc wraps with "& (N-1)" (src/lbm.cu:350-352): powers of two only.
  auto pow2 = [](int v) { return v >= 8 && (v & (v - 1)) == 0; };
  if (!pow2(nx) || !pow2(ny) || !pow2(nz)) {
    g_err = "reference kernels need power-of-two sizes >= 8";
    return 1;
  }
  const long long cells = static_cast<long long>(nx) * ny * nz;
  if (cells * 19 >= (1LL << 31)) {
    g_err = "reference kernels index with int: 19*nx*ny*nz must stay below 2^31";
    return 1;
  }
  RH(cuCtxSetCurrent(r->ctx));
  r->NX = nx;
  r->NY = ny;
  r->NZ = nz;
  r->moving_wall = moving_wall;
  const size_t S = static_cast<size_t>(cells) * sizeof(float);
  for (int i = 0; i < kNumA; ++i) {
    if (r->a[i]) cuMemFree(r->a[i]);
    r->a[i] = 0;
    RH(cuMemAlloc(&r->a[i], (i == aF || i == aG || i == aGout) ? S * 19 : S));
  }
  const int zeroed[] = {aPhi, aUx, aUy, aUz, aF, aG, aNx, aNy, aNz, aCurv, aInd, aFfx, aFfy, aFfz};
  for (int i : zeroed)
    RH(cuMemsetD8Async(r->a[i], 0, (i == aF || i == aG) ? S * 19 : S, r->stream));
  const float cssq = 1.0f / 3.0f, omega = 1.0f / tau;
  float w[19];
  w[0] = 1.0f / 3.0f;
  for (int l = 1; l <= 6; ++l) w[l] = 1.0f / 18.0f;
  for (int l = 7; l < 19; ++l) w[l] = 1.0f / 36.0f;
  const int cix[19] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0};
  const int ciy[19] = {0, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 1, -1};
  const int ciz[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, -1, 1, -1, 1};
  auto put = [&](const char* name, const void* src, size_t bytes) -> int {
    CUdeviceptr p = 0;
    size_t sz = 0;
    RH(cuModuleGetGlobal(&p, &sz, r->mod, name));
    if (sz != bytes) {
      g_err = std::string("unexpected size of symbol ") + name;
      return 1;
    }
    RH(cuMemcpyHtoD(p, src, bytes));
    return 0;
  };
  if (put("CSSQ", &cssq, 4) || put("OMEGA", &omega, 4) || put("SHARP_C", &sharp_c, 4) ||
      put("SIGMA", &sigma, 4) || put("W", w, sizeof w) || put("CIX", cix, sizeof cix) ||
      put("CIY", ciy, sizeof ciy) || put("CIZ", ciz, sizeof ciz))
    return 1;
  RH(cuStreamSynchronize(r->stream));
  return 0;
}

// initTensor, then phi from the host instead of initPhase, then initDist (src/main.cu:56-68).
int ref_set_phi(void* h, const float* phi) {
  Ref* r = static_cast<Ref*>(h);
  if (!r || !phi || !r->NX) return 1;
  RH(cuCtxSetCurrent(r->ctx));
  int NX = r->NX, NY = r->NY, NZ = r->NZ;
  CUdeviceptr* a = r->a;
  if (r->launch(kInitTensor, {&a[aPxx], &a[aPyy], &a[aPzz], &a[aPxy], &a[aPxz], &a[aPyz],
                              &a[aRho], &NX, &NY, &NZ}))
    return 1;
  const size_t S = static_cast<size_t>(NX) * NY * NZ * sizeof(float);
  RH(cuMemcpyHtoDAsync(a[aPhi], phi, S, r->stream));
  if (r->launch(kInitDist, {&a[aRho], &a[aPhi], &a[aF], &a[aG], &NX, &NY, &NZ})) return 1;
  RH(cuStreamSynchronize(r->stream));
  return 0;
}

// The body of the step loop (src/main.cu:79-178) nsteps times, timed with events around
// the launches. streams = 1: every kernel on one stream, in the intended order. streams = 3:
// the reference's own layout, collisionFluid and collisionPhase on two more streams with no
// dependency on momentiCalc, then both streams synchronised from the host
// (src/main.cu:127-141). That order races; its results vary from run to run, which sets the
// noise floor of any comparison with the reference.
int ref_run_streams(void* h, int nsteps, int streams, float* ms) {
  Ref* r = static_cast<Ref*>(h);
  if (!r || !r->NX || nsteps < 0 || (streams != 1 && streams != 3)) return 1;
  RH(cuCtxSetCurrent(r->ctx));
  if (streams == 3 && !r->coll_fluid) {
    RH(cuStreamCreate(&r->coll_fluid, CU_STREAM_DEFAULT));
    RH(cuStreamCreate(&r->coll_phase, CU_STREAM_DEFAULT));
  }
  CUstream sf = streams == 3 ? r->coll_fluid : nullptr;
  CUstream sp = streams == 3 ? r->coll_phase : nullptr;
  int NX = r->NX, NY = r->NY, NZ = r->NZ;
  CUdeviceptr* a = r->a;
  RH(cuEventRecord(r->e0, r->stream));
  for (int s = 0; s < nsteps; ++s) {
    if (r->launch(kPhiCalc, {&a[aPhi], &a[aG], &NX, &NY, &NZ}) ||
        r->launch(kGradCalc, {&a[aPhi], &a[aNx], &a[aNy], &a[aNz], &a[aInd], &NX, &NY, &NZ}) ||
        r->launch(kCurvatureCalc, {&a[aCurv], &a[aInd], &a[aNx], &a[aNy], &a[aNz], &a[aFfx],
                                   &a[aFfy], &a[aFfz], &NX, &NY, &NZ}) ||
        r->launch(kMomentiCalc, {&a[aUx], &a[aUy], &a[aUz], &a[aRho], &a[aFfx], &a[aFfy],
                                 &a[aFfz], &a[aF], &a[aPxx], &a[aPyy], &a[aPzz], &a[aPxy],
                                 &a[aPxz], &a[aPyz], &NX, &NY, &NZ}) ||
        r->launch(kCollisionFluid, {&a[aF], &a[aUx], &a[aUy], &a[aUz], &a[aFfx], &a[aFfy],
                                    &a[aFfz], &a[aRho], &a[aPxx], &a[aPyy], &a[aPzz],
                                    &a[aPxy], &a[aPxz], &a[aPyz], &NX, &NY, &NZ}, sf) ||
        r->launch(kCollisionPhase, {&a[aG], &a[aUx], &a[aUy], &a[aUz], &a[aPhi], &a[aNx],
                                    &a[aNy], &a[aNz], &NX, &NY, &NZ}, sp))
      return 1;
    if (streams == 3) {
      RH(cuStreamSynchronize(sf));
      RH(cuStreamSynchronize(sp));
    }
    if (r->moving_wall && r->launch(kMovingWallBC, {&a[aF], &a[aRho], &NX, &NY, &NZ})) return 1;
    if (r->launch(kStreamingCalc, {&a[aG], &a[aGout], &NX, &NY, &NZ})) return 1;
    std::swap(a[aG], a[aGout]);
    if (r->launch(kFgBoundary, {&a[aF], &a[aRho], &a[aG], &a[aPhi], &NX, &NY, &NZ}) ||
        r->launch(kBoundaryConditions, {&a[aPhi], &NX, &NY, &NZ}))
      return 1;
    // src/main.cu:180 waits for the device after every update
    if (streams == 3) RH(cuCtxSynchronize());
  }
  RH(cuEventRecord(r->e1, r->stream));
  RH(cuEventSynchronize(r->e1));
  float t = 0.f;
  RH(cuEventElapsedTime(&t, r->e0, r->e1));
  if (ms) *ms = t;
  return 0;
}

int ref_run(void* h, int nsteps, float* ms) { return ref_run_streams(h, nsteps, 1, ms); }

// which: 0 phi, 1 rho, 2 ux, 3 uy, 4 uz
int ref_get(void* h, int which, float* host) {
  Ref* r = static_cast<Ref*>(h);
  if (!r || !host || !r->NX || which < 0 || which > 4) return 1;
  RH(cuCtxSetCurrent(r->ctx));
  const int map[5] = {aPhi, aRho, aUx, aUy, aUz};
  const size_t S = static_cast<size_t>(r->NX) * r->NY * r->NZ * sizeof(float);
  RH(cuMemcpyDtoHAsync(host, r->a[map[which]], S, r->stream));
  RH(cuStreamSynchronize(r->stream));
  return 0;
}

void ref_close(void* h) {
  Ref* r = static_cast<Ref*>(h);
  if (!r) return;
  cuCtxSetCurrent(r->ctx);
  if (r->stream) cuStreamSynchronize(r->stream);
  for (CUdeviceptr p : r->a)
    if (p) cuMemFree(p);
  if (r->e0) cuEventDestroy(r->e0);
  if (r->e1) cuEventDestroy(r->e1);
  if (r->stream) cuStreamDestroy(r->stream);
  if (r->coll_fluid) cuStreamDestroy(r->coll_fluid);
  if (r->coll_phase) cuStreamDestroy(r->coll_phase);
  if (r->mod) cuModuleUnload(r->mod);
  cuDevicePrimaryCtxRelease(r->dev);
  delete r;
}

}  // extern "C"
