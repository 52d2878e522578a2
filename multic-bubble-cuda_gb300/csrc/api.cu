// C ABI of the solver (include/mcb.h): handle and batch life cycle, stepping, field
// read-back, diagnostics, dumps and the tile autotuner.
//
// Reference counterparts:
//   - state: src/var.cu:57-114 (initializeVars), src/auxFunctions.cu:4-10 (freeMemory);
//   - init: src/init.cu:3-80;
//   - step loop: src/main.cu:74-190;
//   - output: src/auxFunctions.cu:12-67.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <climits>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <cuda.h>  // CUtensorMap, cuTensorMapEncodeTiled (through the runtime entry point)

#include "mcb.h"
#include "lattice.h"
#include "solver.h"

namespace {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

#define MCB_CU(call)                                                                     \
  do {                                                                                   \
    const cudaError_t e_ = (call);                                                       \
    if (e_ != cudaSuccess)                                                               \
      return fail(e_ == cudaErrorMemoryAllocation ? MCB_ERR_ALLOC : MCB_ERR_CUDA,        \
                  "%s failed: %s", #call, cudaGetErrorString(e_));                       \
  } while (0)

#define MCB_TRY(expr)          \
  do {                         \
    const int r_ = (expr);     \
    if (r_ != MCB_OK) return r_; \
  } while (0)

// Balanced work decomposition (zchunk = -w): w resident waves of equal-work blocks per
// kernel.
constexpr int kMaxWaves = 16;
constexpr int kMinCollidePlanes = 8;

size_t pop_bytes(int storage) { return storage == mcb::kStF32 ? 4 : 2; }

int validate(const mcb_config& c, int index) {
  if (c.nx < 4 || c.ny < 4 || c.nz < 4)
    return fail(MCB_ERR_INVALID, "case %d: lattice %dx%dx%d is below 4 cells per axis", index,
                c.nx, c.ny, c.nz);
  if (c.nx > 65535 || c.ny > 65535 || c.nz > 65535)
    return fail(MCB_ERR_INVALID, "case %d: an axis exceeds 65535 cells", index);
  const long long n = static_cast<long long>(c.nx) * c.ny * c.nz;
  if (n > 0x7fffffffLL)
    return fail(MCB_ERR_INVALID, "case %d: %lld cells exceed 2^31-1 per case", index, n);
  if (c.bc != MCB_BC_REF && c.bc != MCB_BC_PERIODIC && c.bc != MCB_BC_WALLS_Z)
    return fail(MCB_ERR_INVALID, "case %d: unknown boundary mode %d", index, c.bc);
  if (c.bc == MCB_BC_REF && (c.nx < 8 || c.ny < 8 || c.nz < 8))
    return fail(MCB_ERR_INVALID, "case %d: reference boundary mode needs >= 8 cells per axis",
                index);
  if (c.storage != MCB_STORE_F32 && c.storage != MCB_STORE_F16 && c.storage != MCB_STORE_BF16)
    return fail(MCB_ERR_INVALID, "case %d: unknown storage %d", index, c.storage);
  if (!(c.tau > 0.5f) || !std::isfinite(c.tau))
    return fail(MCB_ERR_INVALID, "case %d: tau must be > 0.5 (got %g)", index, c.tau);
  if (!(c.tau_g > 0.5f) || !std::isfinite(c.tau_g))
    return fail(MCB_ERR_INVALID, "case %d: tau_g must be > 0.5 (got %g)", index, c.tau_g);
  if (c.bc == MCB_BC_REF && c.tau_g != 1.0f)
    return fail(MCB_ERR_INVALID,
                "case %d: reference boundary mode relaxes g fully; tau_g must be 1", index);
  if (!(c.width > 0.f) || !std::isfinite(c.width))
    return fail(MCB_ERR_INVALID, "case %d: width must be > 0", index);
  if (!std::isfinite(c.sigma) || !std::isfinite(c.gravity) || !std::isfinite(c.sharp_c))
    return fail(MCB_ERR_INVALID, "case %d: non-finite parameter", index);
  if (c.variant < -1 || c.variant >= mcb::kNumVariants)
    return fail(MCB_ERR_INVALID, "case %d: variant %d out of range", index, c.variant);
  if (c.velocity_set != 19 && c.velocity_set != 27)
    return fail(MCB_ERR_INVALID, "case %d: velocity_set must be 19 or 27 (got %d)", index,
                c.velocity_set);
  if (!(c.rho_in > 0.f) || !(c.rho_out > 0.f) || !std::isfinite(c.rho_in) ||
      !std::isfinite(c.rho_out))
    return fail(MCB_ERR_INVALID, "case %d: rho_in and rho_out must be > 0", index);
  if (c.rho_in != c.rho_out && c.bc == MCB_BC_REF)
    return fail(MCB_ERR_INVALID,
                "case %d: the reference boundary mode is density-matched (rho_in == rho_out)",
                index);
  if (c.zchunk < -kMaxWaves)
    return fail(MCB_ERR_INVALID, "case %d: zchunk must be >= -%d", index, kMaxWaves);
  if (c.g_mode != MCB_G_AUTO && c.g_mode != MCB_G_POPULATIONS)
    return fail(MCB_ERR_INVALID, "case %d: unknown g_mode %d", index, c.g_mode);
  return MCB_OK;
}

float sharp_of(const mcb_config& c) {
  return c.sharp_c > 0.f ? c.sharp_c : (c.tau_g - 0.5f) * 4.0f / c.width;
}

}  // namespace

// One set of device buffers holding one or more cases.
struct Solver {
  int storage = 0, variant = 0, zchunk_req = 0, use_graph = 1, device = 0;
  std::vector<mcb_config> cfg;
  std::vector<mcb::CaseDesc> cases;
  long long cells_total = 0, max_cells = 0;
  long long f_cells_total = 0, max_f_cells = 0;  // cells of the f layout (x rounded up to 32)
  bool bgk = false;
  int gmode = mcb::kGPop;
  int qf = 19;             // velocity set of f
  int ratio = 0;           // density-ratio model
  int wide = 0;            // some case needs 64-bit f offsets
  bool padded = false;     // f in the padded layout of the TMA collide
  bool pair_ok = false;    // the two-cells-per-thread kernel can run these cases
  bool wide_blocked = false;  // 64-bit f offsets on the blocked layout: the pair kernel only
  bool push = false;       // the collide kernel writes the next phi (all but the TMA kernel)
  CUtensorMap fmap[2];     // TMA descriptors of f[0], f[1] (padded only)
  int* err = nullptr;      // device error flag of bounded waits
  mcb::CaseDesc* d_cases = nullptr;
  void* jbuf = nullptr;
  void* f[2] = {nullptr, nullptr};
  void* g[2] = {nullptr, nullptr};
  // g rest population: stored g without push; with push only the first update's phi
  // kernel reads one (the init's)
  int* rest[2] = {nullptr, nullptr};
  // phi, Q2.30: two buffers alternate; the push mode rotates three (current, next, cleared
  // for the one after) or, with stored g, four (the previous one, whose split the 16-bit g
  // decode needs)
  int* p[4] = {nullptr, nullptr, nullptr, nullptr};
  float* macros = nullptr;
  float* stage = nullptr;
  mcb::DiagPartial* partials = nullptr;
  mcb::DiagPartial* result = nullptr;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaGraphExec_t graph[8] = {};  // per (f parity, phi slot) at the start of the graph
  int graph_steps = 16;
  // Launch groups: the cases of each group run one phi and one collide launch per update,
  // with the group's tile variant. A single case, and a batch until mcb_batch_autotune
  // splits it, is one group of every case with the handle's variant and z chunk request.
  struct Group {
    int variant = 0, zchunk_req = 0;
    std::vector<int> members;  // case indices, in launch order
    std::vector<int> zc_case;  // per member: > 0 fixed z chunk overriding the group's split
    int ntiles = 0, zchunk = 16, balanced = 1, phi_balanced = 0, planes = 0;
    int grid_phi = 0, grid_collide = 0;
    int table = 0;  // first entry of the group's case table in d_gcases
  };
  std::vector<Group> groups;
  bool grouped = false;  // groups set by the batch autotuner (else one group, rebuilt)
  mcb::CaseDesc* d_gcases = nullptr;  // the case tables of the groups, back to back
  std::vector<mcb::CaseDesc> gtab;    // host image of d_gcases
  int parity = 0, first = 1, latest_p = 1;
  int pk = 0;  // current phi buffer; advances by one per update, modulo nphi()
  long long update = -1;
  std::vector<char> fields_set;
  std::vector<cudaEvent_t> prof_events;
  bool stepped = false, timed = false;

  int set_device() {
    MCB_CU(cudaSetDevice(device));
    return MCB_OK;
  }

  int nphi() const { return push ? (gmode == mcb::kGEquil ? 3 : 4) : 2; }
  int graph_key() const { return parity * 4 + pk; }

  void drop_graphs() {
    for (auto& ge : graph)
      if (ge) {
        cudaGraphExecDestroy(ge);
        ge = nullptr;
      }
  }

  void release() {
    if (stream) cudaStreamSynchronize(stream);
    drop_graphs();
    for (int i = 0; i < 2; ++i) {
      cudaFree(f[i]);
      cudaFree(g[i]);
      cudaFree(rest[i]);
      cudaFree(p[i]);
      f[i] = g[i] = nullptr;
      rest[i] = p[i] = nullptr;
    }
    for (int i = 2; i < 4; ++i) {
      cudaFree(p[i]);
      p[i] = nullptr;
    }
    cudaFree(macros);
    cudaFree(err);
    err = nullptr;
    cudaFree(jbuf);
    jbuf = nullptr;
    cudaFree(stage);
    cudaFree(partials);
    cudaFree(result);
    cudaFree(d_cases);
    cudaFree(d_gcases);
    d_gcases = nullptr;
    macros = stage = nullptr;
    partials = result = nullptr;
    d_cases = nullptr;
    for (cudaEvent_t e : prof_events) cudaEventDestroy(e);
    prof_events.clear();
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (stream) cudaStreamDestroy(stream);
    ev0 = ev1 = nullptr;
    stream = nullptr;
  }

  // Work decomposition of the cases of one group for its variant and z chunk request:
  //   zchunk_req > 0: fixed chunks of that many planes, one block each;
  //   zchunk_req < 0: balanced ranges, -zchunk_req resident waves of equal-work blocks
  //   per kernel;
  //   zchunk_req == 0: fixed chunks chosen below.
  // A member's own fixed chunk (zc_case > 0) overrides the group's unless it is balanced.
  int build_group(Group& g, int nsm) {
    const mcb::Variant v = mcb::kVariants[g.variant];
    long long plane_total = 0;
    for (int ci : g.members) {
      mcb::CaseDesc& d = cases[ci];
      d.tiles_x = (d.nx + v.bx - 1) / v.bx;
      d.tiles_y = (d.ny + v.by - 1) / v.by;
      d.plane0 = static_cast<int>(plane_total);
      plane_total += static_cast<long long>(d.tiles_x) * d.tiles_y * d.nz;
      if (plane_total > 0x7fffffffLL) return fail(MCB_ERR_INVALID, "too many tile planes");
    }
    g.planes = static_cast<int>(plane_total);
    g.balanced = g.zchunk_req < 0;
    int occ_phi = 0, occ_col = 0;
    MCB_CU(mcb::occupancy(storage, g.variant, gmode, qf, ratio, wide, &occ_phi, &occ_col));
    if (occ_phi <= 0 || occ_col <= 0)
      return fail(MCB_ERR_CUDA, "no resident blocks for tile variant %d", g.variant);
    int zc = g.zchunk_req;
    if (zc <= 0) {
      // Default split, from sweeps on GB300: when one case's tile columns fit in one
      // resident wave of collide blocks, cut every column into the same number of chunks so
      // that the whole case is one wave whose blocks march neighbouring columns in step
      // (128x128x256: 37 planes, 2 % faster than 16-plane chunks, 2.4 % faster than
      // balanced runs at FP32). Otherwise 32-plane chunks (512^3: 13 % faster than balanced
      // runs, 2.5 % faster than 16). A chunk keeps at least 4 planes: on the 64^3 static
      // bubble 4-plane chunks (256 blocks) run 20.6 us per update against 25.2 with 8 and
      // 23.6 with 2 (FP32, relaxed g), 14.6 against 17.6 with 8 (FP16, pair kernel,
      // equilibrium g).
      const long long wave = 1LL * occ_col * nsm;
      long long cols = 0;
      int nzmax = 1;
      for (int ci : g.members) {
        cols += static_cast<long long>(cases[ci].tiles_x) * cases[ci].tiles_y;
        nzmax = std::max(nzmax, cases[ci].nz);
      }
      if (g.members.size() == 1 && cols <= wave) {
        const long long m = std::max<long long>(1, std::min<long long>(wave / cols, nzmax / 4));
        zc = static_cast<int>((nzmax + m - 1) / m);
      } else {
        zc = 32;
      }
    }
    long long tile0 = 0;
    for (size_t k = 0; k < g.members.size(); ++k) {
      mcb::CaseDesc& d = cases[g.members[k]];
      const int own = k < g.zc_case.size() ? g.zc_case[k] : 0;
      d.zchunk = (own > 0 && !g.balanced) ? own : zc;
      d.tiles_z = (d.nz + d.zchunk - 1) / d.zchunk;
      d.tile0 = static_cast<int>(tile0);
      tile0 += static_cast<long long>(d.tiles_x) * d.tiles_y * d.tiles_z;
      if (tile0 > 0x7fffffffLL) return fail(MCB_ERR_INVALID, "too many tiles (%lld)", tile0);
    }
    g.ntiles = static_cast<int>(tile0);
    g.zchunk = g.balanced ? g.zchunk_req : zc;
    g.phi_balanced = 0;
    if (g.balanced) {
      const int waves = -g.zchunk;
      g.grid_phi = static_cast<int>(std::min<long long>(g.planes, 1LL * occ_phi * nsm * waves));
      // A collide piece re-reads four phi planes and recomputes two normal planes before
      // its first plane: give each block at least kMinCollidePlanes.
      g.grid_collide = static_cast<int>(std::min<long long>(
          std::max(1, g.planes / kMinCollidePlanes), 1LL * occ_col * nsm * waves));
    } else {
      g.grid_phi = g.grid_collide = g.ntiles;
      // When the collide chunks leave part of a phi wave idle, the record phi kernel (no
      // halo to prime) takes one resident wave of equal runs instead: 128x128x256 57 us
      // against 59, with the D3Q27 chunks 57 against 87. Larger cases keep the chunks
      // (512^3: 1.47 ms against 1.74 balanced).
      g.phi_balanced = gmode == mcb::kGEquil && g.ntiles < 1LL * occ_phi * nsm;
      if (g.phi_balanced)
        g.grid_phi = static_cast<int>(std::min<long long>(g.planes, 1LL * occ_phi * nsm));
    }
    return MCB_OK;
  }

  // Rebuilds the work decomposition of every group (one group of every case with the
  // handle's variant and z chunk request, unless the batch autotuner set the groups).
  int build_tiles() {
    if (!grouped) {
      groups.assign(1, Group{});
      groups[0].variant = variant;
      groups[0].zchunk_req = zchunk_req;
      for (int i = 0; i < static_cast<int>(cases.size()); ++i) groups[0].members.push_back(i);
    }
    int nsm = 0;
    MCB_CU(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device));
    if (nsm <= 0) return fail(MCB_ERR_CUDA, "no multiprocessors");
    for (auto& g : groups) MCB_TRY(build_group(g, nsm));
    drop_graphs();
    MCB_TRY(upload_tables());
    MCB_CU(cudaStreamSynchronize(stream));
    return MCB_OK;
  }

  // The case table in case order (init, diagnostics) and the groups' launch tables.
  int upload_tables() {
    gtab.clear();
    for (auto& g : groups) {
      g.table = static_cast<int>(gtab.size());
      for (int ci : g.members) gtab.push_back(cases[ci]);
    }
    MCB_CU(cudaMemcpyAsync(d_cases, cases.data(), sizeof(mcb::CaseDesc) * cases.size(),
                           cudaMemcpyHostToDevice, stream));
    MCB_CU(cudaMemcpyAsync(d_gcases, gtab.data(), sizeof(mcb::CaseDesc) * gtab.size(),
                           cudaMemcpyHostToDevice, stream));
    return MCB_OK;
  }

  // The schedule of case ci: its group's variant, and its z chunk setting (the group's
  // request, or the case's own fixed chunk).
  void schedule_of(int ci, int* v, int* zc) const {
    for (const auto& g : groups)
      for (size_t k = 0; k < g.members.size(); ++k)
        if (g.members[k] == ci) {
          *v = g.variant;
          const int own = k < g.zc_case.size() ? g.zc_case[k] : 0;
          *zc = (own > 0 && !g.balanced) ? own : g.zchunk;
          return;
        }
    *v = variant;
    *zc = zchunk_req;
  }

  int create(const mcb_config* cs, int n) {
    if (!cs || n <= 0) return fail(MCB_ERR_INVALID, "no cases");
    for (int i = 0; i < n; ++i) MCB_TRY(validate(cs[i], i));
    storage = cs[0].storage;
    device = cs[0].device;
    qf = cs[0].velocity_set;
    ratio = cs[0].rho_in != cs[0].rho_out;
    for (int i = 1; i < n; ++i)
      if (cs[i].storage != storage || cs[i].device != device || cs[i].velocity_set != qf ||
          (cs[i].rho_in != cs[i].rho_out) != (ratio != 0))
        return fail(MCB_ERR_INVALID,
                    "all cases of a batch must share storage, device, velocity set and "
                    "density model");
    // The one-cell default tile, 32x8 (measured sweeps on GB300, either storage); the pair
    // kernel replaces it below where it applies.
    variant = cs[0].variant >= 0 ? cs[0].variant : 0;
    zchunk_req = cs[0].zchunk;
    use_graph = cs[0].use_graph;
    cfg.assign(cs, cs + n);
    cases.resize(n);
    long long off = 0;
    for (int i = 0; i < n; ++i) {
      const mcb_config& c = cs[i];
      mcb::CaseDesc& d = cases[i];
      std::memset(&d, 0, sizeof d);
      d.nx = c.nx;
      d.ny = c.ny;
      d.nz = c.nz;
      d.bc = c.bc;
      d.ncell = static_cast<long long>(c.nx) * c.ny * c.nz;
      d.cell_off = off;
      d.g_off = off * 18;
      d.omega = 1.0f / c.tau;
      d.omega_g = 1.0f / c.tau_g;
      d.sigma = c.sigma;
      d.sharp_c = sharp_of(c);
      d.gravity = c.gravity;
      d.phi_mean = 0.f;
      d.rho_out = ratio ? c.rho_out : 1.0f;
      d.drho = ratio ? c.rho_in - c.rho_out : 0.0f;
      off += d.ncell;
      max_cells = std::max(max_cells, d.ncell);
      if (c.tau_g != 1.0f) bgk = true;
    }
    cells_total = off;
    fields_set.assign(n, 0);
    bool force_pop = false;
    for (int i = 0; i < n; ++i) force_pop = force_pop || cs[i].g_mode == MCB_G_POPULATIONS;
    gmode = bgk ? mcb::kGBgk : (force_pop ? mcb::kGPop : mcb::kGEquil);
    // The TMA collide, on request only (measured slower than the plain tiles on GB300):
    // one case, (P, J) records, rows a multiple of 16 bytes. Elsewhere a request for it
    // runs the plain 32x8 tile.
    // Ghost columns: 32 bytes on each side keep every row's cells on 32-byte sectors.
    const int gxe = 32 / static_cast<int>(pop_bytes(storage));
    padded = n == 1 && qf == 19 && !ratio && gmode == mcb::kGEquil &&
             cs[0].nx % (gxe / 2) == 0 &&
             cs[0].variant == mcb::kTmaVariant && encode_fn() != nullptr;
    // 32-bit f offsets need qf * cells < 2^31 in every case (cells of the blocked layout,
    // x rounded up to 32); larger cases run the 32x8 tile with 64-bit offsets.
    // MCB_WIDE_OFFSETS=1 forces those on any size (the tests compare the two).
    long long max_blocked = 0;
    for (auto& d : cases)
      max_blocked = std::max(max_blocked, ((d.nx + 31) / 32) * 32LL * d.ny * d.nz);
    const char* force_wide = std::getenv("MCB_WIDE_OFFSETS");
    wide = max_blocked * qf >= (1LL << 31) || (force_wide && force_wide[0] == '1');
    // The two-cells-per-thread kernel: D3Q19 f at density ratio 1, an even nx in every case.
    // It addresses f per plane with 64-bit plane offsets, so with equilibrium g it also runs
    // the cases that need 64-bit f offsets, on the blocked layout. Stored g: periodic and
    // wall modes, 32-bit g offsets (18 * cells < 2^31).
    pair_ok = qf == 19 && !ratio && !padded;
    for (auto& d : cases) {
      pair_ok = pair_ok && d.nx % 2 == 0 &&
                (d.nx + 31LL) / 32 * 32 * d.ny * qf * static_cast<long long>(pop_bytes(storage)) <
                    (1LL << 32);  // a plane of f under 2^32 bytes
      if (gmode != mcb::kGEquil)
        pair_ok = pair_ok && d.bc != mcb::kBcRef && 18LL * d.ncell < (1LL << 31);
    }
    if (mcb::is_pair_variant(variant) && !pair_ok) variant = 0;
    // Default tile: the pair kernel where it applies, else 32x8. Measured on GB300, collide
    // kernel of the 128x128x256 walls-and-gravity workload (FP32 / FP16 / BF16 storage):
    //   - equilibrium g: 133 us against 137 at FP32, 120 against 138 at FP16;
    //   - g stored at full relaxation: 163 / 147 / 156 us against 174 / 171 / 198;
    //   - relaxed g (tau_g 0.8): 16-bit storage with the L2 prefetch variant, 275 / 303 us
    //     against 298 / 313; at FP32 the one-cell tile stays (233 us against 286).
    // Where nx leaves the pair kernel's 64-cell-wide tiles emptier than the one-cell
    // kernel's 32-wide ones, the one-cell tile stays: 96^3, equilibrium g, 35.6 us against
    // 41.0 (FP32); 80^3 27.9 against 31.9. 200x200x100 (tiles 78 % full, against 89 %)
    // still runs the pair kernel faster, 157 us against 175. Stored g takes the pair kernel
    // from 64^3 (there 16.6 us against 17.8 for the populations at FP32, 25.1 against 26.0
    // relaxed at FP16); 32^3 and 96^3 run faster one cell per thread.
    auto x_fill = [&](int w) {  // share of the tiles' thread columns that hold cells
      double c = 0, t = 0;
      for (auto& d : cases) {
        c += static_cast<double>(d.nx) * d.ny * d.nz;
        t += static_cast<double>((d.nx + w - 1) / w) * w * d.ny * d.nz;
      }
      return c / t;
    };
    const bool pair_fills = x_fill(mcb::kVariants[mcb::kPairVariant].bx) >=
                            0.85 * x_fill(mcb::kVariants[0].bx);
    if (cs[0].variant < 0 && pair_ok && pair_fills) {
      if (gmode == mcb::kGEquil) variant = mcb::kPairVariant;
      else if (cells_total >= (1LL << 18) && gmode == mcb::kGPop) variant = mcb::kPairVariant;
      else if (cells_total >= (1LL << 18) && storage != MCB_STORE_F32)
        variant = mcb::kPairVariant + 1;
    }
    // f layout: blocked with equilibrium g and 32-bit offsets (x rounded up to whole 32-cell
    // blocks), or with the pair kernel at any size; plain otherwise (the 64-bit one-cell
    // kernels and the stored-g ones measured slower blocked: they spill the extra per-thread
    // offsets, so they run the plain layout only). The padded TMA layout is set below.
    const bool blocked = mcb::is_pair_variant(variant) || (gmode == mcb::kGEquil && !wide);
    wide_blocked = wide && blocked;
    f_cells_total = max_f_cells = 0;
    for (auto& d : cases) {
      d.fxb = blocked ? (d.nx + 31) / 32 : 0;
      const long long fc = blocked ? static_cast<long long>(d.fxb) * 32 * d.ny * d.nz : d.ncell;
      d.f_off = f_cells_total * qf;
      f_cells_total += fc;
      max_f_cells = std::max(max_f_cells, fc);
    }
    if (wide) padded = false;
    if (padded) variant = mcb::kTmaVariant;
    else if (variant == mcb::kTmaVariant || qf == 27 || ratio || (wide && !wide_blocked))
      variant = 0;
    for (auto& d : cases) {
      if (padded) {
        d.fgx = gxe;
        d.fpx = d.nx + 2 * gxe;
        d.fpy = d.ny + 2;
        d.fn = static_cast<long long>(d.fpx) * d.fpy * d.nz;
        d.f_off = 0;
        d.fxb = 0;
      } else {
        d.fgx = 0;
        d.fpx = d.nx;
        d.fpy = d.ny;
        d.fn = d.ncell;
      }
    }
    MCB_TRY(set_device());
    MCB_CU(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    MCB_CU(cudaEventCreate(&ev0));
    MCB_CU(cudaEventCreate(&ev1));
    const size_t fb = f_bytes();
    const size_t gb = static_cast<size_t>(cells_total) * 18 * pop_bytes(storage);
    const size_t cb = static_cast<size_t>(cells_total) * sizeof(int);
    // Every collide kernel but the TMA one writes the next phi itself; the TMA one keeps
    // (phi, J) records and the phi kernel.
    push = !padded;
    for (int i = 0; i < 2; ++i) {
      MCB_CU(cudaMalloc(&f[i], fb));
      if (padded) MCB_CU(cudaMemset(f[i], 0, fb));  // ghost columns nothing reads stay 0
      if (gmode != mcb::kGEquil) {
        MCB_CU(cudaMalloc(&g[i], gb));
        if (!push || i == 0) MCB_CU(cudaMalloc(&rest[i], cb));
      }
    }
    for (int i = 0; i < nphi(); ++i) MCB_CU(cudaMalloc(&p[i], cb));
    if (gmode == mcb::kGEquil && !push)
      MCB_CU(cudaMalloc(&jbuf, static_cast<size_t>(cells_total) * sizeof(float4)));
    MCB_CU(cudaMalloc(&macros, static_cast<size_t>(cells_total) * 5 * sizeof(float)));
    MCB_CU(cudaMalloc(&stage, static_cast<size_t>(max_cells) * 4 * sizeof(float)));
    MCB_CU(cudaMalloc(&partials, sizeof(mcb::DiagPartial) * mcb::kDiagBlocks));
    MCB_CU(cudaMalloc(&result, sizeof(mcb::DiagPartial)));
    MCB_CU(cudaMalloc(&d_cases, sizeof(mcb::CaseDesc) * n));
    MCB_CU(cudaMalloc(&d_gcases, sizeof(mcb::CaseDesc) * n));
    MCB_CU(cudaMalloc(&err, sizeof(int)));
    MCB_CU(cudaMemset(err, 0, sizeof(int)));
    if (padded) {
      MCB_CU(mcb::prepare_tma(storage));
      for (int i = 0; i < 2; ++i) MCB_TRY(encode_fmap(i));
    }
    return build_tiles();
  }

  // Whether tile variant v can run these cases on the f layout fixed at creation: the TMA
  // variant alone on the padded layout; D3Q27 f and the density-ratio model on the 32x8
  // tile; the pair kernel where it applies, and alone on a blocked layout with 64-bit
  // offsets. Stored g: the pair kernel on the blocked layout, the one-cell tiles on the
  // plain one.
  bool variant_fits(int v) const {
    if ((v == mcb::kTmaVariant) != padded) return false;
    if ((qf == 27 || ratio) && v != 0) return false;
    if (mcb::is_pair_variant(v) && !pair_ok) return false;
    if (wide_blocked && !mcb::is_pair_variant(v)) return false;
    if (gmode != mcb::kGEquil && mcb::is_pair_variant(v) != (cases[0].fxb > 0)) return false;
    return true;
  }

  // Runs 2 updates to warm up (graph captures included), then nsteps timed ones; reports
  // the MLUPS of the cases the groups hold.
  int time_updates(int nsteps, double* mlups) {
    MCB_TRY(step(2));
    MCB_TRY(step(nsteps));
    float ms = 0.f;
    MCB_TRY(last_ms(&ms));
    long long cells = 0;
    for (const auto& gr : groups)
      for (int ci : gr.members) cells += cases[ci].ncell;
    *mlups = static_cast<double>(cells) * nsteps / (ms * 1e-3) / 1e6;
    return MCB_OK;
  }

  size_t f_bytes() const {
    const long long per = padded ? cases[0].fn : f_cells_total;
    return static_cast<size_t>(per) * qf * pop_bytes(storage);
  }

  // cuTensorMapEncodeTiled from the driver, through the runtime (no libcuda link).
  using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                   const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                   const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion,
                                   CUtensorMapFloatOOBfill);
  static EncodeTiled encode_fn() {
    static EncodeTiled fn = [] {
      void* p = nullptr;
      cudaDriverEntryPointQueryResult q;
      if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                           cudaEnableDefault, &q) != cudaSuccess ||
          q != cudaDriverEntryPointSuccess)
        p = nullptr;
      return reinterpret_cast<EncodeTiled>(p);
    }();
    return fn;
  }

  // 4-D map of f[i]: (x, y, z, population) over the padded layout; box 32 + ghost width
  // by 8 rows by 1 plane by 1 population. Out-of-range boxes read zeros.
  int encode_fmap(int i) {
    const mcb::CaseDesc& d = cases[0];
    const size_t e = pop_bytes(storage);
    const cuuint64_t dims[4] = {static_cast<cuuint64_t>(d.fpx), static_cast<cuuint64_t>(d.fpy),
                                static_cast<cuuint64_t>(d.nz), 19};
    const cuuint64_t strides[3] = {d.fpx * e, static_cast<cuuint64_t>(d.fpx) * d.fpy * e,
                                   static_cast<cuuint64_t>(d.fn) * e};
    const cuuint32_t box[4] = {static_cast<cuuint32_t>(32 + d.fgx / 2), 8, 1, 1};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    const CUresult r = encode_fn()(
        &fmap[i], e == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_UINT16, 4,
        f[i], dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
        CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(MCB_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", r);
    return MCB_OK;
  }

  // Error flag of the kernels' bounded waits; read at every synchronisation point.
  int check_err() {
    int h = 0;
    MCB_CU(cudaMemcpy(&h, err, sizeof h, cudaMemcpyDeviceToHost));
    if (h != 0) {
      cudaMemset(err, 0, sizeof(int));
      return fail(MCB_ERR_CUDA, "a TMA wait in the collide kernel gave up (code %d)", h);
    }
    return MCB_OK;
  }

  int set_fields(int ci, const float* phi, const float* ux, const float* uy, const float* uz) {
    if (ci < 0 || ci >= static_cast<int>(cases.size()))
      return fail(MCB_ERR_INVALID, "case index %d out of range", ci);
    if (!phi) return fail(MCB_ERR_INVALID, "phi is NULL");
    const bool has_u = ux || uy || uz;
    if (has_u && !(ux && uy && uz))
      return fail(MCB_ERR_INVALID, "ux, uy, uz must be all NULL or all non-NULL");
    if (stepped && cases.size() > 1)
      return fail(MCB_ERR_STATE, "batch fields can only be set before the first step");
    MCB_TRY(set_device());
    mcb::CaseDesc& d = cases[ci];
    const size_t n = static_cast<size_t>(d.ncell);
    // The fields go to the staging buffer first; the device scans phi (its mean is the
    // buoyancy reference, and a non-finite value rejects the call before any state
    // changes). The one synchronisation also releases the caller's buffers.
    MCB_CU(cudaMemcpyAsync(stage, phi, n * sizeof(float), cudaMemcpyHostToDevice, stream));
    if (has_u) {
      MCB_CU(cudaMemcpyAsync(stage + n, ux, n * sizeof(float), cudaMemcpyHostToDevice, stream));
      MCB_CU(cudaMemcpyAsync(stage + 2 * n, uy, n * sizeof(float), cudaMemcpyHostToDevice,
                             stream));
      MCB_CU(cudaMemcpyAsync(stage + 3 * n, uz, n * sizeof(float), cudaMemcpyHostToDevice,
                             stream));
    }
    MCB_CU(mcb::launch_field_scan(stage, static_cast<long long>(n), partials, result, stream));
    struct {
      double sum;
      long long bad;
    } scan{};
    MCB_CU(cudaMemcpyAsync(&scan, result, sizeof scan, cudaMemcpyDeviceToHost, stream));
    MCB_CU(cudaStreamSynchronize(stream));
    if (scan.bad != LLONG_MAX)
      return fail(MCB_ERR_INVALID, "phi[%lld] is not finite", scan.bad);
    d.phi_mean = static_cast<float>(scan.sum / static_cast<double>(n));
    MCB_TRY(upload_tables());
    // A single case restarts from update 0 in buffer set 0.
    if (cases.size() == 1 || !stepped) {
      parity = 0;
      pk = 0;
      first = 1;
      latest_p = nphi() - 1;
      update = -1;
      stepped = false;
    }
    mcb::InitArgs a{};
    a.cases = d_cases;
    a.case_index = ci;
    a.phi = stage;
    a.ux = has_u ? stage + n : nullptr;
    a.uy = has_u ? stage + 2 * n : nullptr;
    a.uz = has_u ? stage + 3 * n : nullptr;
    a.f0 = f[0];
    a.f1 = f[1];
    a.g0 = g[0];
    a.rest0 = rest[0];
    // phi into the current buffer and the one diagnostics read; push: the next one cleared
    a.p0 = p[pk];
    a.p1 = p[(pk + nphi() - 1) % nphi()];
    a.p_zero = push ? p[(pk + 1) % nphi()] : nullptr;
    a.macros = macros;
    a.cells_total = cells_total;
    a.gmode = gmode;
    a.qf = qf;
    // Stream-ordered: the next call on the handle follows the init.
    MCB_CU(mcb::launch_init(storage, a, d.nx, d.ny, d.nz, stream));
    fields_set[ci] = 1;
    return MCB_OK;
  }

  mcb::StepArgs args(const Group& gr, bool with_macros) const {
    mcb::StepArgs a{};
    a.cases = d_gcases + gr.table;
    a.ncases = static_cast<int>(gr.members.size());
    for (int ci : gr.members) a.has_ref = a.has_ref || cases[ci].bc == mcb::kBcRef;
    a.ntiles = gr.ntiles;
    a.balanced = gr.balanced;
    a.phi_balanced = gr.balanced || gr.phi_balanced;
    a.planes = gr.planes;
    a.grid_phi = gr.grid_phi;
    a.grid_collide = gr.grid_collide;
    a.err = err;
    a.qf = qf;
    a.ratio = ratio;
    a.wide = wide;
    a.f_in = f[parity];
    a.f_out = f[parity ^ 1];
    a.g_in = g[parity];
    a.g_out = g[parity ^ 1];
    a.rest_in = rest[parity];
    a.rest_out = rest[parity ^ 1];
    a.p_prev = p[(pk + nphi() - 1) % nphi()];
    a.p_cur = p[pk];
    a.p_next = push ? p[(pk + 1) % nphi()] : nullptr;
    a.p_zero = push ? p[(pk + 2) % nphi()] : nullptr;
    a.macros = with_macros ? macros : nullptr;
    a.j = jbuf;
    a.cells_total = cells_total;
    a.first = first;
    return a;
  }

  // Equilibrium storage has no populations before the first collision: its first update
  // takes phi from the init and runs only the collide kernel.
  // The phi kernel: equilibrium g runs it only without push and after the first update
  // (the init's phi starts it); stored g without push on every update, with push on the
  // first one only (its phi is the pulled sum of the init's populations, as every later
  // phi is the pushed sum of the collided ones).
  bool skips_phi() const {
    return gmode == mcb::kGEquil ? (push || first) : (push && !first);
  }

  // The phi stage of an update: the phi kernels of the groups, or nothing (push, first
  // equilibrium update).
  int launch_phi_stage(bool with_macros) {
    if (skips_phi()) return MCB_OK;
    for (const auto& gr : groups)
      MCB_CU(mcb::launch_phi(storage, gr.variant, gmode, args(gr, with_macros), stream));
    return MCB_OK;
  }

  // The collide kernels of the groups.
  int launch_collide_stage(bool with_macros) {
    for (const auto& gr : groups)
      MCB_CU(mcb::launch_collide(storage, gr.variant, gmode, args(gr, with_macros),
                                 padded ? &fmap[parity] : nullptr, stream));
    return MCB_OK;
  }

  // Moves to the next update's buffers.
  void advance() {
    latest_p = pk;
    pk = (pk + 1) % nphi();
    parity ^= 1;
    first = 0;
    ++update;
  }

  int launch_update(bool with_macros) {
    MCB_TRY(launch_phi_stage(with_macros));
    MCB_TRY(launch_collide_stage(with_macros));
    advance();
    return MCB_OK;
  }

  // A graph of graph_steps updates (even) starting from the current buffers.
  int ensure_graph() {
    const int key = graph_key();
    if (graph[key]) return MCB_OK;
    const int save_par = parity, save_pk = pk, save_first = first, save_latest = latest_p;
    const long long save_update = update;
    first = 0;
    cudaGraph_t gr = nullptr;
    MCB_CU(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    int rc = MCB_OK;
    for (int i = 0; i < graph_steps && rc == MCB_OK; ++i) rc = launch_update(false);
    const cudaError_t ec = cudaStreamEndCapture(stream, &gr);
    parity = save_par;
    pk = save_pk;
    first = save_first;
    latest_p = save_latest;
    update = save_update;
    if (rc != MCB_OK) {
      if (gr) cudaGraphDestroy(gr);
      return rc;
    }
    if (ec != cudaSuccess)
      return fail(MCB_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(ec));
    const cudaError_t ei = cudaGraphInstantiate(&graph[key], gr, 0);
    cudaGraphDestroy(gr);
    if (ei != cudaSuccess)
      return fail(MCB_ERR_CUDA, "graph instantiate failed: %s", cudaGetErrorString(ei));
    return MCB_OK;
  }

  int step(int nsteps) {
    if (nsteps < 0) return fail(MCB_ERR_INVALID, "nsteps must be >= 0");
    for (size_t i = 0; i < fields_set.size(); ++i)
      if (!fields_set[i]) return fail(MCB_ERR_STATE, "fields of case %zu are not set", i);
    if (nsteps == 0) return MCB_OK;
    MCB_TRY(set_device());
    MCB_CU(cudaEventRecord(ev0, stream));
    int remaining = nsteps;
    while (remaining > 0) {
      const bool eager = first || !use_graph || remaining - 1 < graph_steps;
      if (eager) {
        MCB_TRY(launch_update(remaining == 1));
        --remaining;
      } else {
        MCB_TRY(ensure_graph());
        MCB_CU(cudaGraphLaunch(graph[graph_key()], stream));
        // The graph leaves the f parity unchanged (even length) and moves the phi slot on.
        pk = (pk + graph_steps) % nphi();
        latest_p = (pk + nphi() - 1) % nphi();
        update += graph_steps;
        remaining -= graph_steps;
      }
    }
    MCB_CU(cudaEventRecord(ev1, stream));
    stepped = true;
    timed = true;
    return MCB_OK;
  }

  // nsteps updates with an event after every kernel: ev[0] | phi ev[2i+1] collide ev[2i+2].
  int step_profiled(int nsteps, float* total_ms, float* phi_ms, float* collide_ms) {
    if (nsteps <= 0) return fail(MCB_ERR_INVALID, "nsteps must be > 0");
    for (size_t i = 0; i < fields_set.size(); ++i)
      if (!fields_set[i]) return fail(MCB_ERR_STATE, "fields of case %zu are not set", i);
    MCB_TRY(set_device());
    const size_t need = 2 * static_cast<size_t>(nsteps) + 1;
    while (prof_events.size() < need) {
      cudaEvent_t e;
      MCB_CU(cudaEventCreate(&e));
      prof_events.push_back(e);
    }
    MCB_CU(cudaEventRecord(prof_events[0], stream));
    MCB_CU(cudaEventRecord(ev0, stream));
    for (int i = 0; i < nsteps; ++i) {
      MCB_TRY(launch_phi_stage(i == nsteps - 1));
      MCB_CU(cudaEventRecord(prof_events[2 * i + 1], stream));
      MCB_TRY(launch_collide_stage(i == nsteps - 1));
      MCB_CU(cudaEventRecord(prof_events[2 * i + 2], stream));
      advance();
    }
    MCB_CU(cudaEventRecord(ev1, stream));
    stepped = true;
    timed = true;
    MCB_CU(cudaEventSynchronize(ev1));
    MCB_TRY(check_err());
    float tp = 0.f, tc = 0.f, tt = 0.f;
    for (int i = 0; i < nsteps; ++i) {
      float a = 0.f, b = 0.f;
      MCB_CU(cudaEventElapsedTime(&a, prof_events[2 * i], prof_events[2 * i + 1]));
      MCB_CU(cudaEventElapsedTime(&b, prof_events[2 * i + 1], prof_events[2 * i + 2]));
      tp += a;
      tc += b;
    }
    MCB_CU(cudaEventElapsedTime(&tt, prof_events[0], prof_events[2 * nsteps]));
    if (total_ms) *total_ms = tt;
    if (phi_ms) *phi_ms = tp;
    if (collide_ms) *collide_ms = tc;
    return MCB_OK;
  }

  // ---- checkpoint: header + raw device buffers ----
  struct CkptHeader {
    char magic[8];
    int abi, nx, ny, nz, bc, storage, gmode, parity, first, latest_p, pad, qf, ratio, pk;
    long long update;
    float tau, tau_g, sigma, sharp_c, gravity, phi_mean;
  };

  // (device pointer, bytes) of every buffer the next update reads, in file order.
  std::vector<std::pair<void*, size_t>> ckpt_buffers() {
    const size_t n = static_cast<size_t>(cells_total);
    std::vector<std::pair<void*, size_t>> v;
    v.push_back({f[parity], f_bytes()});
    if (gmode == mcb::kGEquil) {
      if (jbuf) v.push_back({jbuf, n * sizeof(float4)});
    } else {
      v.push_back({g[parity], n * 18 * pop_bytes(storage)});
      if (rest[parity]) v.push_back({rest[parity], n * sizeof(int)});
    }
    for (int i = 0; i < nphi(); ++i) v.push_back({p[i], n * sizeof(int)});
    v.push_back({macros, n * 5 * sizeof(float)});
    return v;
  }

  // f layout of the checkpoint header: the ghost width of the padded layout, -1 blocked,
  // 0 plain.
  int layout_code() const {
    return padded ? cases[0].fgx : (cases[0].fxb > 0 ? -1 : 0);
  }

  int ckpt_save(const char* path) {
    if (!path) return fail(MCB_ERR_INVALID, "path is NULL");
    if (cases.size() != 1) return fail(MCB_ERR_INVALID, "checkpoints hold one case");
    if (!fields_set[0]) return fail(MCB_ERR_STATE, "fields are not set");
    MCB_TRY(set_device());
    MCB_CU(cudaStreamSynchronize(stream));
    CkptHeader hd{};
    std::memcpy(hd.magic, "MCBCKPT1", 8);
    const mcb::CaseDesc& d = cases[0];
    hd.abi = MCB_ABI_VERSION;
    hd.nx = d.nx;
    hd.ny = d.ny;
    hd.nz = d.nz;
    hd.bc = d.bc;
    hd.storage = storage;
    hd.gmode = gmode;
    hd.parity = parity;
    hd.first = first;
    hd.latest_p = latest_p;
    hd.pk = pk;
    hd.pad = layout_code();  // f layout
    hd.qf = qf;
    hd.ratio = ratio;
    hd.update = update;
    hd.tau = cfg[0].tau;
    hd.tau_g = cfg[0].tau_g;
    hd.sigma = d.sigma;
    hd.sharp_c = d.sharp_c;
    hd.gravity = d.gravity;
    hd.phi_mean = d.phi_mean;
    FILE* fp = std::fopen(path, "wb");
    if (!fp) return fail(MCB_ERR_IO, "cannot open %s for writing", path);
    bool ok = std::fwrite(&hd, sizeof hd, 1, fp) == 1;
    std::vector<char> buf(64 << 20);
    for (auto& b : ckpt_buffers()) {
      for (size_t off = 0; ok && off < b.second; off += buf.size()) {
        const size_t len = std::min(buf.size(), b.second - off);
        if (cudaMemcpy(buf.data(), static_cast<char*>(b.first) + off, len,
                       cudaMemcpyDeviceToHost) != cudaSuccess) {
          std::fclose(fp);
          return fail(MCB_ERR_CUDA, "checkpoint read-back failed");
        }
        ok = std::fwrite(buf.data(), 1, len, fp) == len;
      }
    }
    if (std::fclose(fp) != 0) ok = false;
    if (!ok) return fail(MCB_ERR_IO, "short write to %s", path);
    return MCB_OK;
  }

  int ckpt_load(const char* path) {
    if (!path) return fail(MCB_ERR_INVALID, "path is NULL");
    if (cases.size() != 1) return fail(MCB_ERR_INVALID, "checkpoints hold one case");
    MCB_TRY(set_device());
    FILE* fp = std::fopen(path, "rb");
    if (!fp) return fail(MCB_ERR_IO, "cannot open %s", path);
    CkptHeader hd{};
    if (std::fread(&hd, sizeof hd, 1, fp) != 1 || std::memcmp(hd.magic, "MCBCKPT1", 8) != 0) {
      std::fclose(fp);
      return fail(MCB_ERR_INVALID, "%s is not a solver checkpoint", path);
    }
    mcb::CaseDesc& d = cases[0];
    if (hd.nx != d.nx || hd.ny != d.ny || hd.nz != d.nz || hd.bc != d.bc ||
        hd.storage != storage || hd.gmode != gmode || hd.pad != layout_code() ||
        hd.qf != qf || hd.ratio != ratio) {
      std::fclose(fp);
      return fail(MCB_ERR_INVALID,
                  "checkpoint %s was written for another size, boundary mode, storage, g mode, "
                  "f layout, velocity set or density model",
                  path);
    }
    MCB_CU(cudaStreamSynchronize(stream));
    parity = hd.parity;
    std::vector<char> buf(64 << 20);
    bool ok = true;
    for (auto& b : ckpt_buffers()) {
      for (size_t off = 0; ok && off < b.second; off += buf.size()) {
        const size_t len = std::min(buf.size(), b.second - off);
        ok = std::fread(buf.data(), 1, len, fp) == len;
        if (ok && cudaMemcpy(static_cast<char*>(b.first) + off, buf.data(), len,
                             cudaMemcpyHostToDevice) != cudaSuccess) {
          std::fclose(fp);
          return fail(MCB_ERR_CUDA, "checkpoint upload failed");
        }
      }
    }
    std::fclose(fp);
    if (!ok) return fail(MCB_ERR_IO, "%s is truncated", path);
    // Reference-mode shells keep f = W_l in both buffers: the other buffer takes the same.
    MCB_CU(cudaMemcpy(f[parity ^ 1], f[parity], f_bytes(), cudaMemcpyDeviceToDevice));
    first = hd.first;
    latest_p = hd.latest_p;
    pk = push ? hd.pk : parity;
    update = hd.update;
    d.phi_mean = hd.phi_mean;
    MCB_TRY(upload_tables());
    MCB_CU(cudaStreamSynchronize(stream));
    drop_graphs();
    fields_set[0] = 1;
    stepped = update >= 0;
    return MCB_OK;
  }

  int sync() {
    MCB_TRY(set_device());
    MCB_CU(cudaStreamSynchronize(stream));
    return check_err();
  }

  int get_field(int ci, int which, float* host) {
    if (ci < 0 || ci >= static_cast<int>(cases.size()))
      return fail(MCB_ERR_INVALID, "case index %d out of range", ci);
    if (!host) return fail(MCB_ERR_INVALID, "host pointer is NULL");
    if (which < MCB_FIELD_PHI || which > MCB_FIELD_P)
      return fail(MCB_ERR_INVALID, "unknown field %d", which);
    if (!fields_set[ci]) return fail(MCB_ERR_STATE, "fields of case %d are not set", ci);
    MCB_TRY(set_device());
    const mcb::CaseDesc& d = cases[ci];
    const int slot = which == MCB_FIELD_P ? 1 : which;
    const float* src = macros + static_cast<size_t>(slot) * cells_total + d.cell_off;
    MCB_CU(cudaMemcpyAsync(host, src, static_cast<size_t>(d.ncell) * sizeof(float),
                           cudaMemcpyDeviceToHost, stream));
    MCB_CU(cudaStreamSynchronize(stream));
    MCB_TRY(check_err());
    const long long n = d.ncell;
    if (which == MCB_FIELD_P)
      for (long long i = 0; i < n; ++i) host[i] *= (1.0f / 3.0f);
    if (which == MCB_FIELD_PHI && d.bc == mcb::kBcRef && update >= 0) {
      // Zero-gradient shell copy (boundaryConditions, src/lbm.cu:403-425), applied as if
      // the three face copies ran one after another: every shell cell takes the value of
      // the nearest interior cell.
      const int nx = d.nx, ny = d.ny, nz = d.nz;
      for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
          for (int i = 0; i < nx; ++i) {
            if (i > 0 && i < nx - 1 && j > 0 && j < ny - 1 && k > 0 && k < nz - 1) continue;
            const int ic = std::min(std::max(i, 1), nx - 2);
            const int jc = std::min(std::max(j, 1), ny - 2);
            const int kc = std::min(std::max(k, 1), nz - 2);
            host[i + nx * (j + static_cast<long long>(ny) * k)] =
                host[ic + nx * (jc + static_cast<long long>(ny) * kc)];
          }
    }
    return MCB_OK;
  }

  // The exact Q2.30 phi of the latest update (the integers the diagnostics sum).
  int get_phi_q30(int ci, int32_t* host) {
    if (ci < 0 || ci >= static_cast<int>(cases.size()))
      return fail(MCB_ERR_INVALID, "case index %d out of range", ci);
    if (!host) return fail(MCB_ERR_INVALID, "host pointer is NULL");
    if (!fields_set[ci]) return fail(MCB_ERR_STATE, "fields of case %d are not set", ci);
    MCB_TRY(set_device());
    const mcb::CaseDesc& d = cases[ci];
    MCB_CU(cudaMemcpyAsync(host, p[latest_p] + d.cell_off,
                           static_cast<size_t>(d.ncell) * sizeof(int32_t),
                           cudaMemcpyDeviceToHost, stream));
    MCB_CU(cudaStreamSynchronize(stream));
    return check_err();
  }

  int diagnostics(int ci, mcb_diag* out) {
    if (ci < 0 || ci >= static_cast<int>(cases.size()))
      return fail(MCB_ERR_INVALID, "case index %d out of range", ci);
    if (!out) return fail(MCB_ERR_INVALID, "out is NULL");
    if (!fields_set[ci]) return fail(MCB_ERR_STATE, "fields of case %d are not set", ci);
    MCB_TRY(set_device());
    mcb::DiagArgs a{};
    a.cases = d_cases;
    a.case_index = ci;
    a.macros = macros;
    a.p = p[latest_p];
    a.cells_total = cells_total;
    a.partials = partials;
    a.result = result;
    MCB_CU(mcb::launch_diag(a, stream));
    mcb::DiagPartial r;
    MCB_CU(cudaMemcpyAsync(&r, result, sizeof r, cudaMemcpyDeviceToHost, stream));
    MCB_CU(cudaStreamSynchronize(stream));
    MCB_TRY(check_err());
    std::memset(out, 0, sizeof *out);
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
    out->update = static_cast<int>(update);
    if (!out->finite) return fail(MCB_ERR_NUMERIC, "%lld non-finite values", r.nonfinite);
    return MCB_OK;
  }

  int last_ms(float* ms) {
    if (!ms) return fail(MCB_ERR_INVALID, "ms is NULL");
    if (!timed) return fail(MCB_ERR_STATE, "no step has been timed");
    MCB_TRY(set_device());
    MCB_CU(cudaEventSynchronize(ev1));
    MCB_CU(cudaEventElapsedTime(ms, ev0, ev1));
    return MCB_OK;
  }
};

namespace mcb {
int report_error(int code, const char* msg) {
  g_err = msg ? msg : "";
  return code;
}
}  // namespace mcb

// A copy of the state the next update reads, so that timing trials can run on the live
// fields and leave them as they were. Owns its device copies.
struct StateCopy {
  Solver& s;
  void *fs = nullptr, *gs = nullptr, *rs = nullptr, *ps = nullptr, *ms = nullptr;
  size_t n = 0, fb = 0, gb = 0;
  int par = 0, first = 0, latest = 0, pk = 0;
  long long update = -1;
  bool eq = false;

  explicit StateCopy(Solver& solver) : s(solver) {}
  ~StateCopy() {
    cudaFree(fs);
    cudaFree(gs);
    cudaFree(rs);
    cudaFree(ps);
    cudaFree(ms);
  }

  int copy(bool back) {
    auto cp = [&](void* dst, const void* src, size_t b) {
      return cudaMemcpyAsync(dst, src, b, cudaMemcpyDeviceToDevice, s.stream);
    };
    cudaError_t e = cudaSuccess;
    if (!back) {
      if (e == cudaSuccess) e = cp(fs, s.f[par], fb);
      if (e == cudaSuccess && gb) e = cp(gs, eq ? s.jbuf : s.g[par], gb);
      if (e == cudaSuccess && s.rest[par]) e = cp(rs, s.rest[par], n * 4);
      for (int i = 0; i < s.nphi(); ++i)
        if (e == cudaSuccess) e = cp(static_cast<char*>(ps) + i * n * 4, s.p[i], n * 4);
      if (e == cudaSuccess) e = cp(ms, s.macros, n * 20);
    } else {
      if (e == cudaSuccess) e = cp(s.f[par], fs, fb);
      if (e == cudaSuccess && gb) e = cp(eq ? s.jbuf : s.g[par], gs, gb);
      if (e == cudaSuccess && s.rest[par]) e = cp(s.rest[par], rs, n * 4);
      for (int i = 0; i < s.nphi(); ++i)
        if (e == cudaSuccess) e = cp(s.p[i], static_cast<char*>(ps) + i * n * 4, n * 4);
      if (e == cudaSuccess) e = cp(s.macros, ms, n * 20);
      // Reference-mode shells keep f = W_l in both buffers; the other buffer's interior
      // is rewritten by the next update.
      if (e == cudaSuccess) e = cp(s.f[par ^ 1], fs, fb);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s.stream);
    if (e != cudaSuccess) return fail(MCB_ERR_CUDA, "autotune copy: %s", cudaGetErrorString(e));
    return MCB_OK;
  }

  int take() {
    par = s.parity;
    n = static_cast<size_t>(s.cells_total);
    eq = s.gmode == mcb::kGEquil;
    fb = s.f_bytes();
    // g state: stored populations, or with equilibrium g the (phi, J) records of the TMA
    // variant (none in push mode).
    gb = eq ? (s.jbuf ? n * sizeof(float4) : 0) : n * 18 * pop_bytes(s.storage);
    if (cudaMalloc(&fs, fb) != cudaSuccess || (gb && cudaMalloc(&gs, gb) != cudaSuccess) ||
        cudaMalloc(&rs, n * 4) != cudaSuccess || cudaMalloc(&ps, n * 16) != cudaSuccess ||
        cudaMalloc(&ms, n * 20) != cudaSuccess)
      return fail(MCB_ERR_ALLOC, "autotune: no room for a state copy");
    first = s.first;
    latest = s.latest_p;
    pk = s.pk;
    update = s.update;
    return copy(false);
  }

  int restore() {
    MCB_TRY(copy(true));
    s.parity = par;
    s.pk = pk;
    s.first = first;
    s.latest_p = latest;
    s.update = update;
    return MCB_OK;
  }
};

struct mcb_handle {
  Solver s;
};
struct mcb_batch {
  Solver s;
};

extern "C" {

const char* mcb_last_error(void) { return g_err.c_str(); }
int mcb_abi_version(void) { return MCB_ABI_VERSION; }

int mcb_config_default(mcb_config* c) {
  if (!c) return fail(MCB_ERR_INVALID, "cfg is NULL");
  std::memset(c, 0, sizeof *c);
  c->nx = 64;
  c->ny = 64;
  c->nz = 256;
  c->bc = MCB_BC_REF;
  c->storage = MCB_STORE_F32;
  c->tau = 0.505f;
  c->tau_g = 1.0f;
  c->sigma = 0.1f;
  c->width = 3.0f;
  c->sharp_c = 0.15f * 3.0f;
  c->gravity = 0.0f;
  c->device = 0;
  c->variant = -1;
  c->zchunk = 0;
  c->use_graph = 1;
  c->g_mode = MCB_G_AUTO;
  c->velocity_set = 19;
  c->rho_in = 1.0f;
  c->rho_out = 1.0f;
  return MCB_OK;
}

int mcb_create(const mcb_config* cfg, mcb_handle** out) {
  if (!out) return fail(MCB_ERR_INVALID, "out is NULL");
  *out = nullptr;
  if (!cfg) return fail(MCB_ERR_INVALID, "cfg is NULL");
  mcb_handle* h = new (std::nothrow) mcb_handle;
  if (!h) return fail(MCB_ERR_ALLOC, "host allocation failed");
  const int rc = h->s.create(cfg, 1);
  if (rc != MCB_OK) {
    h->s.release();
    delete h;
    return rc;
  }
  *out = h;
  return MCB_OK;
}

int mcb_destroy(mcb_handle* h) {
  if (!h) return MCB_OK;
  cudaSetDevice(h->s.device);
  h->s.release();
  delete h;
  return MCB_OK;
}

int mcb_set_fields(mcb_handle* h, const float* phi, const float* ux, const float* uy,
                   const float* uz) {
  if (!h) return fail(MCB_ERR_INVALID, "handle is NULL");
  return h->s.set_fields(0, phi, ux, uy, uz);
}

int mcb_step(mcb_handle* h, int nsteps) {
  if (!h) return fail(MCB_ERR_INVALID, "handle is NULL");
  return h->s.step(nsteps);
}

int mcb_synchronize(mcb_handle* h) {
  if (!h) return fail(MCB_ERR_INVALID, "handle is NULL");
  return h->s.sync();
}

int mcb_get_field(mcb_handle* h, int which, float* host) {
  if (!h) return fail(MCB_ERR_INVALID, "handle is NULL");
  return h->s.get_field(0, which, host);
}

int mcb_get_phi_q30(mcb_handle* h, int32_t* host) {
  if (!h) return fail(MCB_ERR_INVALID, "handle is NULL");
  return h->s.get_phi_q30(0, host);
}

int mcb_diagnostics(mcb_handle* h, mcb_diag* out) {
  if (!h) return fail(MCB_ERR_INVALID, "handle is NULL");
  return h->s.diagnostics(0, out);
}

int mcb_write_phi_file(const char* dir, const char* id, const char* name, int step,
                       const float* data, size_t n) {
  if (!dir || !id || !name || (!data && n)) return fail(MCB_ERR_INVALID, "NULL argument");
  if (step < 0) return fail(MCB_ERR_INVALID, "step must be >= 0");
  char tail[64];
  std::snprintf(tail, sizeof tail, "%06d.bin", step);
  const std::string path = std::string(dir) + id + "_" + name + tail;
  FILE* fp = std::fopen(path.c_str(), "wb");
  if (!fp) return fail(MCB_ERR_IO, "cannot open %s for writing", path.c_str());
  const size_t w = n ? std::fwrite(data, sizeof(float), n, fp) : 0;
  const int cl = std::fclose(fp);
  if (w != n || cl != 0) return fail(MCB_ERR_IO, "short write to %s", path.c_str());
  return MCB_OK;
}

int mcb_write_info_file(const char* dir, const char* id, const char* velocity_set, int nx,
                        int ny, int nz, double tau, double umax, double fx, double fy,
                        double fz, int save_every, int nsteps, double mlups) {
  if (!dir || !id || !velocity_set) return fail(MCB_ERR_INVALID, "NULL argument");
  const std::string path = std::string(dir) + id + "_info.txt";
  FILE* fp = std::fopen(path.c_str(), "w");
  if (!fp) return fail(MCB_ERR_IO, "cannot open %s for writing", path.c_str());
  // One "key: value" line per item, the value last on its line: post/fileTreat.py:37-124
  // splits each line on spaces and takes the last token.
  const char* pad = "                           ";
  std::fprintf(fp, "---------------------------- SIMULATION INFORMATION ----------------------------\n");
  std::fprintf(fp, "%sSimulation ID: %s\n", pad, id);
  std::fprintf(fp, "%sVelocity set: %s\n", pad, velocity_set);
  std::fprintf(fp, "%sPrecision: float\n", pad);
  std::fprintf(fp, "%sNX: %d\n", pad, nx);
  std::fprintf(fp, "%sNY: %d\n", pad, ny);
  std::fprintf(fp, "%sNZ: %d\n", pad, nz);
  std::fprintf(fp, "%sNZ_TOTAL: %d\n", pad, nz);
  std::fprintf(fp, "%sTau: %g\n", pad, tau);
  std::fprintf(fp, "%sUmax: %e\n", pad, umax);
  std::fprintf(fp, "%sFX: %e\n", pad, fx);
  std::fprintf(fp, "%sFY: %e\n", pad, fy);
  std::fprintf(fp, "%sFZ: %e\n", pad, fz);
  std::fprintf(fp, "%sSave steps: %d\n", pad, save_every);
  std::fprintf(fp, "%sNsteps: %d\n", pad, nsteps);
  std::fprintf(fp, "%sMLUPS: %e\n", pad, mlups > 0 ? mlups : 0.0);
  std::fprintf(fp, "--------------------------------------------------------------------------------\n");
  if (std::fclose(fp) != 0) return fail(MCB_ERR_IO, "cannot write %s", path.c_str());
  return MCB_OK;
}

int mcb_dump_phi(mcb_handle* h, const char* dir, const char* id, int step) {
  if (!h || !dir || !id) return fail(MCB_ERR_INVALID, "NULL argument");
  if (step < 0) return fail(MCB_ERR_INVALID, "step must be >= 0");
  const mcb::CaseDesc& d = h->s.cases[0];
  std::vector<float> buf(static_cast<size_t>(d.ncell));
  MCB_TRY(h->s.get_field(0, MCB_FIELD_PHI, buf.data()));
  return mcb_write_phi_file(dir, id, "phi", step, buf.data(), buf.size());
}

int mcb_dump_field(mcb_handle* h, const char* dir, const char* id, int which, int step) {
  static const char* const kNames[] = {"phi", "rho", "ux", "uy", "uz", "pres"};
  if (!h || !dir || !id) return fail(MCB_ERR_INVALID, "NULL argument");
  if (which < MCB_FIELD_PHI || which > MCB_FIELD_P)
    return fail(MCB_ERR_INVALID, "unknown field %d", which);
  if (step < 0) return fail(MCB_ERR_INVALID, "step must be >= 0");
  const mcb::CaseDesc& d = h->s.cases[0];
  std::vector<float> buf(static_cast<size_t>(d.ncell));
  MCB_TRY(h->s.get_field(0, which, buf.data()));
  return mcb_write_phi_file(dir, id, kNames[which], step, buf.data(), buf.size());
}

int mcb_write_info(const mcb_handle* h, const char* dir, const char* id,
                   const char* velocity_set, int save_every, int nsteps, double mlups) {
  if (!h || !dir || !id || !velocity_set) return fail(MCB_ERR_INVALID, "NULL argument");
  const mcb_config& c = h->s.cfg[0];
  double umax = 0.0;
  if (h->s.update >= 0) {
    mcb_diag dg;
    if (const_cast<mcb_handle*>(h)->s.diagnostics(0, &dg) == MCB_OK) umax = dg.umax;
  }
  return mcb_write_info_file(dir, id, velocity_set, c.nx, c.ny, c.nz, c.tau, umax, 0.0, 0.0,
                             c.gravity, save_every, nsteps, mlups);
}

int mcb_checkpoint_save(mcb_handle* h, const char* path) {
  if (!h) return fail(MCB_ERR_INVALID, "handle is NULL");
  return h->s.ckpt_save(path);
}

int mcb_checkpoint_load(mcb_handle* h, const char* path) {
  if (!h) return fail(MCB_ERR_INVALID, "handle is NULL");
  return h->s.ckpt_load(path);
}

int mcb_get_schedule(const mcb_handle* h, int* variant, int* zchunk) {
  if (!h || !variant || !zchunk) return fail(MCB_ERR_INVALID, "NULL argument");
  *variant = h->s.variant;
  *zchunk = h->s.groups.empty() ? h->s.zchunk_req : h->s.groups[0].zchunk;
  return MCB_OK;
}

int mcb_get_update(const mcb_handle* h, int* update) {
  if (!h || !update) return fail(MCB_ERR_INVALID, "NULL argument");
  *update = static_cast<int>(h->s.update);
  return MCB_OK;
}

int mcb_get_dims(const mcb_handle* h, int* nx, int* ny, int* nz) {
  if (!h || !nx || !ny || !nz) return fail(MCB_ERR_INVALID, "NULL argument");
  *nx = h->s.cfg[0].nx;
  *ny = h->s.cfg[0].ny;
  *nz = h->s.cfg[0].nz;
  return MCB_OK;
}

int mcb_last_step_ms(mcb_handle* h, float* ms) {
  if (!h) return fail(MCB_ERR_INVALID, "handle is NULL");
  return h->s.last_ms(ms);
}

int mcb_step_profiled(mcb_handle* h, int nsteps, float* total_ms, float* phi_ms,
                      float* collide_ms) {
  if (!h) return fail(MCB_ERR_INVALID, "handle is NULL");
  return h->s.step_profiled(nsteps, total_ms, phi_ms, collide_ms);
}

int mcb_variant_count(void) { return mcb::kNumVariants; }

int mcb_variant_shape(int variant, int* bx, int* by) {
  if (variant < 0 || variant >= mcb::kNumVariants || !bx || !by)
    return fail(MCB_ERR_INVALID, "bad variant or NULL argument");
  *bx = mcb::kVariants[variant].bx;
  *by = mcb::kVariants[variant].by;
  return MCB_OK;
}

int mcb_autotune(mcb_handle* h, int nsteps, int* best_variant, int* best_zchunk,
                 double* best_mlups) {
  if (!h) return fail(MCB_ERR_INVALID, "handle is NULL");
  if (nsteps < 2) return fail(MCB_ERR_INVALID, "nsteps must be >= 2");
  Solver& s = h->s;
  if (!s.fields_set[0]) return fail(MCB_ERR_STATE, "fields are not set");
  MCB_TRY(s.set_device());
  StateCopy snap(s);
  int rc = snap.take();
  const int save_variant = s.variant, save_zreq = s.zchunk_req;
  double best = -1.0;
  int bv = save_variant, bz = s.zchunk_req;
  // The default split, balanced ranges of 1..4 resident waves, then fixed chunks.
  const int zc_list[] = {0, -1, -2, -3, -4, 8, 16, 32};
  for (int v = 0; v < mcb::kNumVariants && rc == MCB_OK; ++v) {
    if (!s.variant_fits(v)) continue;
    for (int zc : zc_list) {
      if (zc > s.cfg[0].nz) continue;
      s.variant = v;
      s.zchunk_req = zc;
      double mlups = 0.0;
      rc = s.build_tiles();
      if (rc == MCB_OK) rc = s.time_updates(nsteps, &mlups);
      if (rc != MCB_OK) break;
      if (mlups > best) {
        best = mlups;
        bv = v;
        bz = zc;
      }
      rc = snap.restore();
      if (rc != MCB_OK) break;
    }
  }
  s.variant = (rc == MCB_OK) ? bv : save_variant;
  s.zchunk_req = (rc == MCB_OK) ? bz : save_zreq;
  const int rb = s.build_tiles();
  if (rc != MCB_OK) return rc;
  if (rb != MCB_OK) return rb;
  if (best_variant) *best_variant = bv;
  if (best_zchunk) *best_zchunk = bz;
  if (best_mlups) *best_mlups = best;
  return MCB_OK;
}

// ---- batch ----

int mcb_batch_create(const mcb_config* cases, int ncases, mcb_batch** out) {
  if (!out) return fail(MCB_ERR_INVALID, "out is NULL");
  *out = nullptr;
  mcb_batch* b = new (std::nothrow) mcb_batch;
  if (!b) return fail(MCB_ERR_ALLOC, "host allocation failed");
  const int rc = b->s.create(cases, ncases);
  if (rc != MCB_OK) {
    b->s.release();
    delete b;
    return rc;
  }
  *out = b;
  return MCB_OK;
}

int mcb_batch_destroy(mcb_batch* b) {
  if (!b) return MCB_OK;
  cudaSetDevice(b->s.device);
  b->s.release();
  delete b;
  return MCB_OK;
}

int mcb_batch_set_fields(mcb_batch* b, int ci, const float* phi, const float* ux,
                         const float* uy, const float* uz) {
  if (!b) return fail(MCB_ERR_INVALID, "batch is NULL");
  return b->s.set_fields(ci, phi, ux, uy, uz);
}

int mcb_batch_step(mcb_batch* b, int nsteps) {
  if (!b) return fail(MCB_ERR_INVALID, "batch is NULL");
  return b->s.step(nsteps);
}

int mcb_batch_get_field(mcb_batch* b, int ci, int which, float* host) {
  if (!b) return fail(MCB_ERR_INVALID, "batch is NULL");
  return b->s.get_field(ci, which, host);
}

int mcb_batch_diagnostics(mcb_batch* b, int ci, mcb_diag* out) {
  if (!b) return fail(MCB_ERR_INVALID, "batch is NULL");
  return b->s.diagnostics(ci, out);
}

int mcb_batch_last_step_ms(mcb_batch* b, float* ms) {
  if (!b) return fail(MCB_ERR_INVALID, "batch is NULL");
  return b->s.last_ms(ms);
}

int mcb_batch_get_schedule(const mcb_batch* b, int case_index, int* variant, int* zchunk) {
  if (!b || !variant || !zchunk) return fail(MCB_ERR_INVALID, "NULL argument");
  if (case_index < 0 || case_index >= static_cast<int>(b->s.cases.size()))
    return fail(MCB_ERR_INVALID, "case index %d out of range", case_index);
  b->s.schedule_of(case_index, variant, zchunk);
  return MCB_OK;
}

int mcb_batch_autotune(mcb_batch* b, int nsteps, double* default_mlups, double* tuned_mlups) {
  if (!b) return fail(MCB_ERR_INVALID, "batch is NULL");
  if (nsteps < 2) return fail(MCB_ERR_INVALID, "nsteps must be >= 2");
  Solver& s = b->s;
  for (size_t i = 0; i < s.fields_set.size(); ++i)
    if (!s.fields_set[i]) return fail(MCB_ERR_STATE, "fields of case %zu are not set", i);
  MCB_TRY(s.set_device());
  using Group = Solver::Group;
  StateCopy snap(s);
  MCB_TRY(snap.take());
  // The untuned schedule: one launch of every case with the batch's variant and split.
  const std::vector<Group> before = s.groups;
  const bool before_grouped = s.grouped;
  s.grouped = false;
  double base = 0.0;
  int rc = s.build_tiles();
  if (rc == MCB_OK) rc = s.time_updates(nsteps, &base);
  if (rc == MCB_OK) rc = snap.restore();
  // Size classes: the cases of one lattice size.
  std::vector<std::vector<int>> classes;
  std::vector<std::array<int, 3>> keys;
  for (int i = 0; i < static_cast<int>(s.cases.size()); ++i) {
    const std::array<int, 3> k{s.cases[i].nx, s.cases[i].ny, s.cases[i].nz};
    size_t c = 0;
    while (c < keys.size() && keys[c] != k) ++c;
    if (c == keys.size()) {
      keys.push_back(k);
      classes.emplace_back();
    }
    classes[c].push_back(i);
  }
  // Each class alone: every variant that fits, with the group's default split or a fixed
  // chunk (fixed chunks can differ per case inside one launch; balanced runs cannot).
  const int zc_list[] = {0, 8, 16, 24, 32, 48, 64};
  std::vector<int> best_v(classes.size(), s.variant), best_z(classes.size(), 0);
  for (size_t c = 0; c < classes.size() && rc == MCB_OK; ++c) {
    double best = -1.0;
    for (int v = 0; v < mcb::kNumVariants && rc == MCB_OK; ++v) {
      if (!s.variant_fits(v)) continue;
      for (int zc : zc_list) {
        if (zc > keys[c][2]) continue;
        Group g;
        g.variant = v;
        g.zchunk_req = zc;
        g.members = classes[c];
        s.groups.assign(1, g);
        s.grouped = true;
        double m = 0.0;
        rc = s.build_tiles();
        if (rc == MCB_OK) rc = s.time_updates(nsteps, &m);
        if (rc == MCB_OK) rc = snap.restore();
        if (rc != MCB_OK) break;
        if (m > best) {
          best = m;
          best_v[c] = v;
          best_z[c] = zc;
        }
      }
    }
  }
  // Two ways to combine the choices: one launch per chosen variant, each case with its
  // class's chunk; or one launch of every case with the variant that covers the most cells.
  std::vector<std::vector<Group>> plans;
  if (rc == MCB_OK) {
    std::vector<Group> per_variant;
    std::vector<long long> cells_of(mcb::kNumVariants, 0);
    for (size_t c = 0; c < classes.size(); ++c) {
      size_t gi = 0;
      while (gi < per_variant.size() && per_variant[gi].variant != best_v[c]) ++gi;
      if (gi == per_variant.size()) {
        per_variant.emplace_back();
        per_variant.back().variant = best_v[c];
      }
      for (int ci : classes[c]) {
        per_variant[gi].members.push_back(ci);
        per_variant[gi].zc_case.push_back(best_z[c]);
        cells_of[best_v[c]] += s.cases[ci].ncell;
      }
    }
    plans.push_back(per_variant);
    if (per_variant.size() > 1) {
      Group one;
      one.variant = static_cast<int>(
          std::max_element(cells_of.begin(), cells_of.end()) - cells_of.begin());
      for (size_t c = 0; c < classes.size(); ++c)
        for (int ci : classes[c]) {
          one.members.push_back(ci);
          one.zc_case.push_back(best_z[c]);
        }
      plans.push_back({one});
    }
  }
  double tuned = base;
  std::vector<Group> chosen;
  for (const auto& plan : plans) {
    if (rc != MCB_OK) break;
    s.groups = plan;
    s.grouped = true;
    double m = 0.0;
    rc = s.build_tiles();
    if (rc == MCB_OK) rc = s.time_updates(nsteps, &m);
    if (rc == MCB_OK) rc = snap.restore();
    if (rc == MCB_OK && m > tuned) {
      tuned = m;
      chosen = plan;
    }
  }
  // Keep the fastest measured schedule; the untuned one if nothing beat it.
  if (rc == MCB_OK) {
    s.grouped = !chosen.empty();
    if (s.grouped) s.groups = chosen;
  } else {
    s.grouped = before_grouped;
    s.groups = before;
  }
  const int rb = s.build_tiles();
  if (rc != MCB_OK) return rc;
  if (rb != MCB_OK) return rb;
  if (default_mlups) *default_mlups = base;
  if (tuned_mlups) *tuned_mlups = tuned;
  return MCB_OK;
}

int mcb_batch_cells(const mcb_batch* b, int64_t* cells) {
  if (!b || !cells) return fail(MCB_ERR_INVALID, "NULL argument");
  *cells = b->s.cells_total;
  return MCB_OK;
}

}  // extern "C"
