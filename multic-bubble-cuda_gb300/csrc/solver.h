// Device-side case table and kernel arguments shared by the kernels and the host API.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace mcb {

enum Bc : int { kBcRef = 0, kBcPeriodic = 1, kBcWallsZ = 2 };
enum Storage : int { kStF32 = 0, kStF16 = 1, kStBF16 = 2 };

// How g crosses from one update to the next. Every collide kernel but the TMA one adds
// the post-collision populations, as exact Q2.30 integers, into the next update's phi.
//   kGPop:   the 18 moving populations are also stored, full relaxation (g* = geq).
//   kGBgk:   they are stored, and the next update pulls and relaxes them (tau_g != 1).
//   kGEquil: full relaxation, nothing stored: each post-collision population is the
//            equilibrium W_l (phi + c_l . J), J = 3 phi u + sharp_c phi (1 - phi) n, of its
//            source cell. The TMA collide keeps phi and J as one 16-byte record per cell,
//            from which its phi kernel rebuilds the populations.
enum GMode : int { kGPop = 0, kGBgk = 1, kGEquil = 2 };

// One case of a launch. A single-case handle has one entry. A batch has one entry per case,
// and every case keeps its own offsets into the shared population buffers.
struct CaseDesc {
  int nx, ny, nz, bc;
  int tiles_x, tiles_y, tiles_z, zchunk;  // tile decomposition of this launch
  int tile0;                              // first tile (block) index of this case
  int plane0;                             // first tile-plane index of this case
  long long ncell;     // nx*ny*nz
  long long cell_off;  // offset of the case's cells in per-cell arrays (phi, rest, macros)
  long long f_off;     // element offset of the case's f values
  long long g_off;     // element offset of the case's 18*ncell moving g values
  // f layout, blocked (fxb > 0: equilibrium g with 32-bit offsets, not the TMA update): fxb
  // blocks of 32 cells in x per row, each holding its Q populations as runs of 32 values:
  //   element (l, x, y, z) at f_off + ((z*ny + y)*fxb + x/32)*Q*32 + l*32 + x%32,
  // so population l of a cell sits a fixed l*32 elements after its population 0.
  // Otherwise element (l, x, y, z) at f_off + l*fn + (z*fpy + y + (fgx ? 1 : 0))*fpx + x +
  // fgx. Plain (stored g, 64-bit offsets): fgx 0, fpx nx, fpy ny, fn ncell. Padded (the
  // TMA update): fgx ghost columns (32 bytes) on each side of a row and one ghost row on
  // each side of a plane, which hold the periodic images of the opposite edge.
  long long fn;
  int fgx, fpx, fpy, fxb;
  float omega;         // 1/tau
  float omega_g;       // 1/tau_g
  float sigma;
  float sharp_c;
  float gravity;
  float phi_mean;      // mean phi of the initial field (buoyancy reference)
  float rho_out;       // density of phi = 0
  float drho;          // rho_in - rho_out; nonzero selects the density-ratio model
};

// Buffers of one update. Populations are stored post-collision at the cell that
// collided them ("pull" layout): an update gathers f*(x - c_l, l).
// Work of a launch: tile-planes, one BX x BY tile of one z plane, numbered case by case,
// column tile by column tile, z fastest. A block takes a contiguous range and marches each
// column piece of it in z.
//   - fixed chunks (balanced == 0): block b takes z chunk b of the tile table (tile0,
//     tiles_x, tiles_y, tiles_z, zchunk); grid = ntiles.
//   - balanced (balanced == 1): block b of G takes [b P / G, (b+1) P / G) of the P planes,
//     so every block has the same work and G is a whole number of resident waves.
struct StepArgs {
  const CaseDesc* cases;
  int ncases;
  int ntiles;
  int balanced;
  int phi_balanced;    // the record phi kernel always takes balanced ranges
  int planes;          // P, tile-planes of all cases
  int grid_phi;        // blocks of the phi kernel
  int grid_collide;    // blocks of the collide kernel
  int* err;            // set to a nonzero code when a bounded wait of a kernel gives up
  int qf;              // velocity set of f: 19 or 27 (every case of a launch)
  int ratio;           // 1: the density-ratio model (every case of a launch)
  int wide;            // 1: some case has QF * ncell >= 2^31 (64-bit f offsets)
  const void* f_in;   // 19 arrays per case
  void* f_out;
  const void* g_in;   // 18 moving g arrays per case (l = 1..18)
  void* g_out;
  const int* rest_in;  // g rest population, Q2.30 (per cell)
  int* rest_out;
  const int* p_prev;   // phi of the previous update, Q2.30
  int* p_cur;          // phi of this update, Q2.30
  int* p_next;         // phi of the next update, accumulated by the collide kernel
                       // (records not stored; zero before the launch), else nullptr
  int* p_zero;         // with p_next: the phi buffer of the update after the next one,
                       // cleared by the collide kernel (three buffers rotate)
  float* macros;       // nullptr, or [5][cells_total]: phi, rho, ux, uy, uz
  void* j;             // kGEquil: 16-byte (P bits, Jx, Jy, Jz) per cell, at cell_off per case
  long long cells_total;
  int first;           // 1 on the first update after fields were set
  int has_ref;         // 1: some case of the launch is in reference mode (MCB_BC_REF)
};

struct InitArgs {
  const CaseDesc* cases;
  int case_index;
  const float* phi;   // host-provided initial fields of this case (device copies)
  const float* ux;    // may be nullptr (rest)
  const float* uy;
  const float* uz;
  void* f0;
  void* f1;
  void* g0;
  int* rest0;
  int* p0;
  int* p1;
  int* p_zero;        // nullptr, or a phi buffer to clear (the next phi of the push mode)
  float* macros;
  long long cells_total;
  int gmode;
  int qf;  // velocity set of f
};

// Per-block partial sums of the diagnostics reduction.
struct DiagPartial {
  double mass, ke, umax, rho_in, n_in, rho_out, n_out, vol_half, phi_min, phi_max;
  long long mass_q30;
  long long nonfinite;
};

struct DiagArgs {
  const CaseDesc* cases;
  int case_index;
  const float* macros;
  const int* p;        // latest phi, Q2.30
  long long cells_total;
  DiagPartial* partials;  // gridDim.x entries
  DiagPartial* result;    // one entry
};

constexpr int kNumVariants = 7;
struct Variant { int bx, by; };
// Cell tiles of the variants. Variant 4 is the 32x8 collide that stages f through the tensor
// memory accelerator (TMA) on the padded f layout; it needs one case, (phi, J) records and nx
// a multiple of 16 bytes. Variants 5 and 6 take two neighbouring cells in x per thread (64x4
// cells, 32x4 threads; three and four blocks per SM); they need equilibrium g, D3Q19 f at
// density ratio 1 and an even nx in every case.
constexpr Variant kVariants[kNumVariants] = {{32, 8}, {16, 16}, {64, 4}, {16, 8}, {32, 8},
                                             {64, 4}, {64, 4}};
constexpr int kTmaVariant = 4;
constexpr int kPairVariant = 5;
constexpr int kPairBY = 4;  // thread rows of the pair kernel's block
constexpr bool is_pair_variant(int v) { return v == kPairVariant || v == kPairVariant + 1; }
constexpr int kErrTmaWait = 1;  // StepArgs::err: a TMA wait timed out
constexpr int kDiagBlocks = 304;   // fixed grid: the reduction order never changes
constexpr int kDiagThreads = 256;

// Kernel launchers (kernels.cu). Each returns the launch status.
cudaError_t launch_phi(int storage, int variant, int gmode, const StepArgs& a,
                       cudaStream_t s);
// tmap_in: the CUtensorMap of f_in for the TMA variant (nullptr otherwise).
cudaError_t launch_collide(int storage, int variant, int gmode, const StepArgs& a,
                           const void* tmap_in, cudaStream_t s);
// Raises the dynamic shared memory limit of the TMA collide kernels (call once per device
// before the first launch or occupancy query).
cudaError_t prepare_tma(int storage);
// Dynamic shared memory of the TMA collide kernel for a storage.
size_t tma_smem_bytes(int storage);
// Resident blocks per SM of the phi and collide kernels of a tile variant.
cudaError_t occupancy(int storage, int variant, int gmode, int qf, int ratio, int wide,
                      int* phi_blocks, int* collide_blocks);
cudaError_t launch_init(int storage, const InitArgs& a, int nx, int ny, int nz,
                        cudaStream_t s);
cudaError_t launch_diag(const DiagArgs& a, cudaStream_t s);
// Sum (FP64, fixed order) and first non-finite index (LLONG_MAX if none) of n device floats:
// partials needs 2 * kDiagBlocks * 8 bytes, result receives {double sum, long long index}.
cudaError_t launch_field_scan(const float* v, long long n, void* partials, void* result,
                              cudaStream_t s);

// Records msg as the calling thread's mcb_last_error() text; returns code.
int report_error(int code, const char* msg);

}  // namespace mcb
