// Fused sm_103a kernels of one lattice update.
//
// The reference runs ten launches per update (src/main.cu:79-178):
//   phiCalc, gradCalc, curvatureCalc, momentiCalc, collisionFluid, collisionPhase,
//   movingWallBC, streamingCalc, fgBoundary, boundaryConditions.
// Between them it keeps 22 full-grid arrays in HBM. Here one update is one kernel:
//
//   k_collide  marches a BX x BY column of cells through a z chunk. It keeps a 5-plane
//              ring of phi (halo 2) and a 4-plane ring of normals (halo 1) in shared
//              memory, the normals computed one plane ahead so that each plane takes one
//              block barrier. For every cell it computes:
//                - the isotropic normals and |grad phi| (gradCalc, src/lbm.cu:34-72);
//                - the curvature and interfacial force (curvatureCalc, src/lbm.cu:80-125);
//                - the moments (momentiCalc, src/lbm.cu:133-225);
//                - the regularized f collision with He forcing (collisionFluid,
//                  src/lbm.cu:233-288);
//                - the g collision (collisionPhase, src/lbm.cu:290-329).
//              f is stored post-collision at the colliding cell; the next update gathers
//              it from x - c_l (pull streaming). The g populations, as exact Q2.30
//              integers, are added straight into the next update's phi at x + c_l
//              (streamingCalc + phiCalc, src/lbm.cu:337-357, 5-26), through a shared ring
//              and integer atomics. In reference mode the shell cells write the
//              rest-equilibrium inflow of fgBoundary (src/lbm.cu:365-401) and their next
//              phi, the lagged copy of boundaryConditions (src/lbm.cu:403-425).
//   k_phi      pull-gathers the 19 stored g populations of every cell and sums them into
//              phi: the first update with stored g only (its phi comes from the init).
//   k_phi_eq   the same when g is kept as one (phi, J) record per cell: the opt-in TMA
//              variant only.
//
// HBM traffic per lattice update: f read and written once and 12 bytes of phi (read, the
// next one accumulated, the one after cleared); with stored g, g written (and read when
// it relaxes with tau_g != 1). Nothing else reaches HBM: normals, curvature, force and
// moments live in registers and shared memory.
//
// phi is carried as Q2.30 fixed point. Every g collision makes the rest population the
// exact integer remainder, so the 19 integers a cell sends add up to its phi exactly,
// and streaming and bounce-back only move them. So the lattice sum of phi is invariant to
// the last bit in periodic and walled domains.
#pragma once

#include <cuda.h>  // CUtensorMap
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <cfloat>
#include <type_traits>
#include <cstring>

#include "lattice.h"
#include "solver.h"

namespace mcb {
namespace {

// ------------------------------------------------------------------ storage policies --

// Integer weight split of a cell's phi (face and edge parts) and the same parts as floats.
// The 16-bit g encoding stores each population relative to its part.
struct GSplit {
  int wf, we;
  float ff, fe;
};

// f float32 absolute, g Q2.30 absolute (32-bit storage).
struct StF32 {
  using FT = float;
  using GT = int;
  static constexpr bool kDev = false;   // g decode needs the source cell's phi
  static constexpr bool kFDev = false;  // f stored as f_l - W_l
  static __device__ __forceinline__ FT fload(const FT* p) { return __ldg(p); }
  static __device__ __forceinline__ GT gload(const GT* p) { return __ldg(p); }
  template <int L> static __device__ __forceinline__ float f_raw(FT v) { return v; }
  template <int L> static __device__ __forceinline__ FT f_put(float f) { return f; }
  template <int L> static __device__ __forceinline__ int g_dec(GT v, int) { return v; }
  static __device__ __forceinline__ GSplit g_split(int) { return GSplit{0, 0, 0.f, 0.f}; }
  template <int L>
  static __device__ __forceinline__ GT g_put(float g, const GSplit&, int& q) {
    q = __float2int_rn(g * kQ30);
    return q;
  }
  template <int L> static __device__ __forceinline__ GT g_shell(int p) { return wsplit<L>(p); }
  static __device__ __forceinline__ int rest_store(int p, int sumq) { return p - sumq; }
  static __device__ __forceinline__ int rest_dec(int stored, int) { return stored; }
  static __device__ __forceinline__ int rest_shell(int p) { return wsplit_rest(p); }
  static __device__ __forceinline__ int rest_init(float g0, int) {
    return __float2int_rn(g0 * kQ30);
  }
};

struct HalfOps {
  using T = __half;
  static __device__ __forceinline__ float tof(T v) { return __half2float(v); }
  static __device__ __forceinline__ T fromf(float f) { return __float2half_rn(f); }
  // Every finite half is a multiple of 2^-24, hence an exact Q2.30 integer. Out-of-range
  // values saturate the same way on encode and decode, so the phi sum stays exact.
  static __device__ __forceinline__ T enc_exact(float d) { return __float2half_rn(d); }
};

struct Bf16Ops {
  using T = __nv_bfloat16;
  static __device__ __forceinline__ float tof(T v) { return __bfloat162float(v); }
  static __device__ __forceinline__ T fromf(float f) { return __float2bfloat16_rn(f); }
  // bfloat16 values below 2^-22 are not multiples of 2^-30. Small deviations are therefore
  // rounded to k * 2^-30 with |k| <= 256 first; that value is exact in bfloat16. Larger
  // ones round to a multiple of 2^-29.
  static __device__ __forceinline__ T enc_exact(float d) {
    const int k = __float2int_rn(d * kQ30);
    if (k <= 256 && k >= -256) return __float2bfloat16_rn(static_cast<float>(k) * kInvQ30);
    return __float2bfloat16_rn(d);
  }
};

// 16-bit deviation form: f_l - W_l, and g_l - w_l(phi of the cell that collided it).
// w_l is the exact integer split of that phi. The g rest population is a Q2.30 integer
// holding the exact remainder.
template <class O>
struct St16 {
  using FT = typename O::T;
  using GT = typename O::T;
  static constexpr bool kDev = true;
  static constexpr bool kFDev = true;
  static __device__ __forceinline__ FT fload(const FT* p) { return __ldg(p); }
  static __device__ __forceinline__ GT gload(const GT* p) { return __ldg(p); }
  template <int L> static __device__ __forceinline__ float f_raw(FT v) { return O::tof(v); }
  template <int L> static __device__ __forceinline__ FT f_put(float dev) {
    return O::fromf(dev);
  }
  template <int L> static __device__ __forceinline__ int g_dec(GT v, int psrc) {
    return wsplit<L>(psrc) + __float2int_rn(O::tof(v) * kQ30);
  }
  static __device__ __forceinline__ GSplit g_split(int p) {
    const int wf = wsplit_face(p), we = wsplit_edge_of_face(wf);
    return GSplit{wf, we, __int2float_rn(wf) * kInvQ30, __int2float_rn(we) * kInvQ30};
  }
  template <int L>
  static __device__ __forceinline__ GT g_put(float g, const GSplit& sp, int& q) {
    const int w = L <= 6 ? sp.wf : sp.we;
    const GT h = O::enc_exact(g - (L <= 6 ? sp.ff : sp.fe));
    q = w + __float2int_rn(O::tof(h) * kQ30);
    return h;
  }
  template <int L> static __device__ __forceinline__ GT g_shell(int) { return O::fromf(0.0f); }
  static __device__ __forceinline__ int rest_store(int p, int sumq) {
    return p - sumq - wsplit_rest(p);
  }
  static __device__ __forceinline__ int rest_dec(int stored, int p) {
    return wsplit_rest(p) + stored;
  }
  static __device__ __forceinline__ int rest_shell(int) { return 0; }
  static __device__ __forceinline__ int rest_init(float g0, int p) {
    return __float2int_rn(g0 * kQ30) - wsplit_rest(p);
  }
};

using StH16 = St16<HalfOps>;
using StB16 = St16<Bf16Ops>;

// ------------------------------------------------------------------------- helpers --

// Value for the source cell x - c (C = +1 takes the minus neighbour).
template <int C, class T>
__device__ __forceinline__ T src_of(T m, T o, T p) {
  if constexpr (C == 1) return m;
  else if constexpr (C == -1) return p;
  else return o;
}
// Value for the neighbour x + c.
template <int C, class T>
__device__ __forceinline__ T nbr_of(T m, T o, T p) {
  if constexpr (C == 1) return p;
  else if constexpr (C == -1) return m;
  else return o;
}

__device__ __forceinline__ int wrap1(int v, int n) {
  return v < 0 ? v + n : (v >= n ? v - n : v);
}
__device__ __forceinline__ int clampi(int v, int lo, int hi) { return min(max(v, lo), hi); }

__device__ __forceinline__ void l2_prefetch(const void* p) {
  asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

// L2 prefetch of one plane of a BX x BY tile in narr arrays: the first and the last
// element of every row, which covers each row's one or two 128-byte lines. A later update
// loop iteration then finds these populations in L2. That keeps DRAM busy regardless of
// how many warps are resident. Every address lies inside the arrays.
template <int NT, int BX, int BY>
__device__ __forceinline__ void prefetch_rows(int tid, const char* base, long long arr_bytes,
                                              int narr, int elem, long long plane_elems,
                                              int xt, int yt, int nx, int ny) {
  const int x_last = min(xt + BX, nx) - 1;
  const int total = narr * BY * 2;
  for (int j = tid; j < total; j += NT) {
    const int side = j & 1, r = (j >> 1) % BY, arr = (j >> 1) / BY;
    const int y = yt + r;
    if (y >= ny) continue;
    const int x = side ? x_last : xt;
    l2_prefetch(base + arr * arr_bytes +
                (plane_elems + static_cast<long long>(y) * nx + x) * elem);
  }
}

// Last case whose first index (tile0 or plane0) is <= key.
template <bool kPlanes>
__device__ __forceinline__ int find_case(const CaseDesc* cs, int n, int key) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if ((kPlanes ? __ldg(&cs[mid].plane0) : __ldg(&cs[mid].tile0)) <= key) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

struct Tile {
  int nx, ny, nz, bc, zb, ze, xt, yt, ci;
  int fgx, fpx, fpy, fxb;
  long long ncell, cell_off, f_off, g_off, fn;
};

// The tile-planes [p0, p1) of this block.
__device__ __forceinline__ int2 block_range(const StepArgs& a, bool balanced) {
  const int b = static_cast<int>(blockIdx.x);
  if (balanced) {
    const long long P = a.planes, G = gridDim.x;
    return make_int2(static_cast<int>(b * P / G), static_cast<int>((b + 1) * P / G));
  }
  const CaseDesc* cd = a.cases + find_case<false>(a.cases, a.ncases, b);
  const int cols = __ldg(&cd->tiles_x) * __ldg(&cd->tiles_y);
  const int r = b - __ldg(&cd->tile0);
  const int nz = __ldg(&cd->nz), zc = __ldg(&cd->zchunk);
  const int base = __ldg(&cd->plane0) + (r % cols) * nz;
  const int z0 = (r / cols) * zc;
  return make_int2(base + z0, base + min(z0 + zc, nz));
}

// The column piece that starts at tile-plane p and ends at p1 or at the column's top.
template <int BX, int BY>
__device__ __forceinline__ Tile segment_tile(const StepArgs& a, int p, int p1) {
  const int c = find_case<true>(a.cases, a.ncases, p);
  const CaseDesc* cd = a.cases + c;
  Tile t;
  t.ci = c;
  t.nx = __ldg(&cd->nx);
  t.ny = __ldg(&cd->ny);
  t.nz = __ldg(&cd->nz);
  t.bc = __ldg(&cd->bc);
  const int tiles_x = __ldg(&cd->tiles_x);
  const int r = p - __ldg(&cd->plane0);
  const int col = r / t.nz;
  t.zb = r - col * t.nz;
  t.ze = min(t.nz, t.zb + (p1 - p));
  t.xt = (col % tiles_x) * BX;
  t.yt = (col / tiles_x) * BY;
  t.ncell = __ldg(&cd->ncell);
  t.cell_off = __ldg(&cd->cell_off);
  t.f_off = __ldg(&cd->f_off);
  t.g_off = __ldg(&cd->g_off);
  t.fn = __ldg(&cd->fn);
  t.fgx = __ldg(&cd->fgx);
  t.fpx = __ldg(&cd->fpx);
  t.fpy = __ldg(&cd->fpy);
  t.fxb = __ldg(&cd->fxb);
  return t;
}

// Runs body(tile) over the column pieces of this block's range. sync: a block barrier
// between pieces, for kernels whose pieces reuse shared memory.
template <int BX, int BY, bool kSync, class Body>
__device__ __forceinline__ void for_each_segment(const StepArgs& a, Body&& body,
                                                 bool balanced) {
  const int2 r = block_range(a, balanced);
  for (int p = r.x; p < r.y;) {
    const Tile t = segment_tile<BX, BY>(a, p, r.y);
    if (kSync && p != r.x) __syncthreads();
    body(t);
    p += t.ze - t.zb;
  }
}

// Register budgets, the largest warp counts per SM that compile without spills: 24 for
// k_collide (80 registers); for k_phi, 32 with 32-bit storage (64 registers) and 24 with
// the 16-bit decode (80 registers). Both kernels wait on loads, so resident warps hide
// latency.
constexpr int kCollideWarpsPerSM = 24;
template <class S>
constexpr int phi_warps_per_sm() { return S::kDev ? 24 : 32; }

// ---------------------------------------------------------------- k_phi: g -> phi --

template <class S, int BX, int BY>
__device__ __forceinline__ void phi_segment(const StepArgs& a, const Tile& t) {
  using GT = typename S::GT;
  const int nx = t.nx, ny = t.ny, nz = t.nz;
  const int x = t.xt + static_cast<int>(threadIdx.x);
  const int y = t.yt + static_cast<int>(threadIdx.y);
  if (x >= nx || y >= ny) return;
  const long long n = t.ncell;
  const GT* __restrict__ gin = static_cast<const GT*>(a.g_in) + t.g_off;
  const int* __restrict__ rest = a.rest_in + t.cell_off;
  const int* __restrict__ pprev = a.p_prev + t.cell_off;
  int* __restrict__ pcur = a.p_cur + t.cell_off;
  const int nxy = nx * ny;
  const bool ref = t.bc == kBcRef, walls = t.bc == kBcWallsZ;
  const int xm = x == 0 ? nx - 1 : x - 1, xp = x == nx - 1 ? 0 : x + 1;
  const int ym = (y == 0 ? ny - 1 : y - 1) * nx, yo = y * nx;
  const int yp = (y == ny - 1 ? 0 : y + 1) * nx;
  const bool shell_xy = ref && (x == 0 || x == nx - 1 || y == 0 || y == ny - 1);
  const int tid = threadIdx.x + BX * threadIdx.y;
  auto prefetch = [&](int zpl) {
    const long long po = static_cast<long long>(zpl) * nxy;
    prefetch_rows<BX * BY, BX, BY>(tid, reinterpret_cast<const char*>(gin), n * sizeof(GT),
                                   kQ - 1, sizeof(GT), po, t.xt, t.yt, nx, ny);
    prefetch_rows<BX * BY, BX, BY>(tid, reinterpret_cast<const char*>(rest), 0, 1, 4, po,
                                   t.xt, t.yt, nx, ny);
    if (S::kDev)
      prefetch_rows<BX * BY, BX, BY>(tid, reinterpret_cast<const char*>(pprev), 0, 1, 4, po,
                                     t.xt, t.yt, nx, ny);
  };
  if (t.zb + 1 < nz) prefetch(t.zb + 1);

  for (int z = t.zb; z < t.ze; ++z) {
    if (z + 2 < nz && z + 2 <= t.ze) prefetch(z + 2);
    const int zo = z * nxy;
    const int idx = x + yo + zo;
    int P;
    if (ref && (shell_xy || z == 0 || z == nz - 1)) {
      // Shell: zero-gradient copy of the previous update's interior phi; zero on the
      // first update (the reference's memset, src/var.cu:86).
      if (a.first) {
        P = 0;
      } else {
        const int xc = clampi(x, 1, nx - 2), yc = clampi(y, 1, ny - 2);
        const int zc = clampi(z, 1, nz - 2);
        P = __ldg(pprev + xc + yc * nx + zc * nxy);
      }
    } else {
      const int zm = (z == 0 ? nz - 1 : z - 1) * nxy;
      const int zp = (z == nz - 1 ? 0 : z + 1) * nxy;
      const bool blo = walls && z == 0, bhi = walls && z == nz - 1;
      const int pself = S::kDev ? __ldg(pprev + idx) : 0;
      P = S::rest_dec(__ldg(rest + idx), pself);
      static_for<1, kQ>([&](auto LC) {
        constexpr int L = decltype(LC)::value;
        constexpr int O = opp(L);
        const bool bounce = (cz(L) == 1) ? blo : ((cz(L) == -1) ? bhi : false);
        if (bounce) {
          P += S::template g_dec<O>(S::gload(gin + (O - 1) * n + idx), pself);
        } else {
          const int s = src_of<cz(L)>(zm, zo, zp) + src_of<cy(L)>(ym, yo, yp) +
                        src_of<cx(L)>(xm, x, xp);
          const int ps = S::kDev ? __ldg(pprev + s) : 0;
          P += S::template g_dec<L>(S::gload(gin + (L - 1) * n + s), ps);
        }
      });
    }
    pcur[idx] = P;
  }
}

template <class S, int BX, int BY>
__global__ void __launch_bounds__(BX * BY, phi_warps_per_sm<S>() * 32 / (BX * BY))
    k_phi(const StepArgs a) {
  for_each_segment<BX, BY, false>(
      a, [&](const Tile& t) { phi_segment<S, BX, BY>(a, t); }, a.balanced != 0);
}

// ------------------------------------- k_phi_eq: g -> phi when g is stored as (phi, J) --
//
// With full g relaxation, the post-collision population l of a cell is the equilibrium
//   g*_l = W_l (phi + c_l . J),  J = 3 phi u + SHARP_C phi (1 - phi) n
// (src/lbm.cu:319-326). Its Q2.30 value is stored implicitly as two parts:
//   - the exact integer weight split w_l(P) of the cell's phi, which sums to P over l;
//   - q_J(l) = m_l c_l.J', with J' = rn(J 2^30 / 36) per component (integers) and
//     m_l = 2 on the faces (W = 1/18), 1 on the edges (W = 1/36): W_l c_l.J 2^30 to within
//     one unit per component. Opposite directions are exact negatives.
// The 18 moving parts of a cell therefore add up to P - w_0(P): the rest population is
// exactly w_0(P), and the lattice sum of phi is invariant. Each cell keeps one 16-byte
// record of the update: (P, J'x, J'y, J'z) as int bits.

// J' of a cell.
struct JQ {
  int x, y, z;
};
__device__ __forceinline__ JQ jq_of(float jx, float jy, float jz) {
  constexpr float k = 1073741824.0f / 36.0f;
  return JQ{__float2int_rn(jx * k), __float2int_rn(jy * k), __float2int_rn(jz * k)};
}

// q_J for direction L (its opposite is the exact negative).
template <int L>
__device__ __forceinline__ int qj(const JQ& j) {
  int cj = 0;
  if constexpr (cx(L) != 0) cj += cx(L) > 0 ? j.x : -j.x;
  if constexpr (cy(L) != 0) cj += cy(L) > 0 ? j.y : -j.y;
  if constexpr (cz(L) != 0) cj += cz(L) > 0 ? j.z : -j.z;
  return L <= 6 ? 2 * cj : cj;
}

// Q2.30 population L of a cell record (P, J'x, J'y, J'z).
template <int L>
__device__ __forceinline__ int q_rec(float4 r) {
  return wsplit<L>(__float_as_int(r.x)) +
         qj<L>(JQ{__float_as_int(r.y), __float_as_int(r.z), __float_as_int(r.w)});
}

template <class S, int BX, int BY>
__device__ __forceinline__ void phi_eq_segment(const StepArgs& a, const Tile& t) {
  const int nx = t.nx, ny = t.ny, nz = t.nz;
  const int x = t.xt + static_cast<int>(threadIdx.x);
  const int y = t.yt + static_cast<int>(threadIdx.y);
  if (x >= nx || y >= ny) return;
  const float4* __restrict__ rec = static_cast<const float4*>(a.j) + t.cell_off;
  const int* __restrict__ pprev = a.p_prev + t.cell_off;
  int* __restrict__ pcur = a.p_cur + t.cell_off;
  const int nxy = nx * ny;
  const bool ref = t.bc == kBcRef, walls = t.bc == kBcWallsZ;
  const int xm = x == 0 ? nx - 1 : x - 1, xp = x == nx - 1 ? 0 : x + 1;
  const int ym = (y == 0 ? ny - 1 : y - 1) * nx, yo = y * nx;
  const int yp = (y == ny - 1 ? 0 : y + 1) * nx;
  const bool shell_xy = ref && (x == 0 || x == nx - 1 || y == 0 || y == ny - 1);

  auto cell = [&](int z) -> int {
    const int zo = z * nxy;
    const int idx = x + yo + zo;
    if (ref && (shell_xy || z == 0 || z == nz - 1)) {
      // Shell: zero-gradient copy of the previous update's interior phi.
      const int xc = clampi(x, 1, nx - 2), yc = clampi(y, 1, ny - 2);
      const int zc = clampi(z, 1, nz - 2);
      return __ldg(pprev + xc + yc * nx + zc * nxy);
    }
    const int zm = (z == 0 ? nz - 1 : z - 1) * nxy;
    const int zp = (z == nz - 1 ? 0 : z + 1) * nxy;
    const bool blo = walls && z == 0, bhi = walls && z == nz - 1;
    const float4 r0 = __ldg(rec + idx);
    int P = wsplit_rest(__float_as_int(r0.x));
    auto pull = [&](auto LC) {
      constexpr int L = decltype(LC)::value;
      constexpr int O = opp(L);
      const bool bounce = (cz(L) == 1) ? blo : ((cz(L) == -1) ? bhi : false);
      if (bounce) {
        P += q_rec<O>(r0);  // across a z wall the cell's own opposite population returns
      } else {
        const int src = src_of<cz(L)>(zm, zo, zp) + src_of<cy(L)>(ym, yo, yp) +
                        src_of<cx(L)>(xm, x, xp);
        P += q_rec<L>(__ldg(rec + src));
      }
    };
    // Nine records in flight at a time: the compiler may not hoist the second half of the
    // loads above the first half's arithmetic, which keeps the kernel within its registers.
    static_for<1, 10>(pull);
    asm volatile("" ::: "memory");
    static_for<10, kQ>(pull);
    return P;
  };
  for (int z = t.zb; z < t.ze; ++z) pcur[x + yo + z * nxy] = cell(z);
}

template <class S, int BX, int BY>
__global__ void __launch_bounds__(BX * BY, 32 * 32 / (BX * BY)) k_phi_eq(const StepArgs a) {
  for_each_segment<BX, BY, false>(
      a, [&](const Tile& t) { phi_eq_segment<S, BX, BY>(a, t); }, a.phi_balanced != 0);
}

// ------------------------------------------- TMA staging of f for the collide kernel --
//
// The TMA variant loads, for every plane a block collides, the 19 pulled population boxes
// of its 32x8 tile with cp.async.bulk.tensor (one instruction per box, issued by one
// thread) into a two-stage shared-memory ring, completed on an mbarrier per stage. The
// threads then read f_l(x - c_l) from shared memory at a fixed offset. Each box is the
// tile widened by 16 bytes in x, so that its x origin stays 16-byte aligned whatever the
// direction's x shift; periodic images come from the ghost columns (32 bytes a side) and
// rows of the padded layout, which the collide kernel rewrites with every update.

constexpr int kTmaBX = 32, kTmaBY = 8;
constexpr int kTmaMaxSpin = 1 << 20;  // try_wait rounds before a wait gives up

template <class FT>
struct TmaBox {
  static constexpr int kGX = 16 / static_cast<int>(sizeof(FT));  // x slop: 16 bytes
  static constexpr int kW = kTmaBX + kGX;                         // box width (elements)
  static constexpr int kBytes = kW * kTmaBY * static_cast<int>(sizeof(FT));
  static_assert(kBytes % 128 == 0, "TMA boxes must keep 128-byte shared-memory alignment");
  static constexpr int kStageBytes = kQ * kBytes;
  static constexpr int kSmem = 2 * kStageBytes + 128;  // two stages + alignment slack
};

struct TmaPipe {
  unsigned char* buf;        // 2 stages x 19 boxes
  unsigned long long* mbar;  // one mbarrier per stage
  const CUtensorMap* map;    // f_in
  unsigned it;               // planes consumed by this block so far (stage = it & 1)
  bool failed;
};

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(unsigned long long* m, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(m)), "r"(count)
               : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long* m, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(m)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long* m, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(m)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Waits for the given phase parity; false after kTmaMaxSpin rounds.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* m, unsigned parity) {
  for (int i = 0; i < kTmaMaxSpin; ++i)
    if (mbar_try_wait(m, parity)) return true;
  return false;
}

__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map, int c0, int c1,
                                            int c2, int c3, unsigned long long* m) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3),
      "r"(smem_u32(m))
      : "memory");
}

// Issues the 19 boxes that plane zt of a tile pulls into stage buffer dst (one thread).
// Box l covers padded x [x0, x0 + kW), rows yt - cy .. yt - cy + 7, plane zt - cz (wrapped
// when periodic; its own plane and population opp(l) across a z wall).
template <class FT>
__device__ __forceinline__ void tma_issue_plane(const TmaPipe& p, unsigned char* dst,
                                                unsigned long long* m, int xt, int yt,
                                                int zt, int nz, int bc, int gxl) {
  constexpr int GX = TmaBox<FT>::kGX;
  mbar_expect_tx(m, TmaBox<FT>::kStageBytes);
  static_for<0, kQ>([&](auto LC) {
    constexpr int L = decltype(LC)::value;
    int zs = zt - cz(L), pop = L, y0 = yt + 1 - cy(L);
    int x0 = gxl + xt - (cx(L) == 1 ? GX : 0);
    if (cz(L) != 0 && (zs < 0 || zs >= nz)) {
      if (bc == kBcWallsZ) {
        zs = zt;
        pop = opp(L);
        x0 = gxl + xt;
        y0 = yt + 1;
      } else if (bc == kBcPeriodic) {
        zs = zs < 0 ? zs + nz : zs - nz;
      }  // reference mode: only shell planes reach past z; the box reads the fill value
    }
    tma_load_4d(dst + L * TmaBox<FT>::kBytes, p.map, x0, y0, zs, pop, m);
  });
}

// Ghost copies of a freshly collided population of cell (x, y): the periodic images that
// consumers across the x and y edges pull (padded layout, periodic x and y only).
template <int L, class FT>
__device__ __forceinline__ void f_ghosts(FT* f, long long fn, int x, int y, int z, int nx,
                                         int ny, int gx, int px, int py, FT v) {
  int gxp = -1, gyp = -1;
  if (cx(L) == -1 && x == 0) gxp = nx + gx;
  else if (cx(L) == 1 && x == nx - 1) gxp = gx - 1;
  if (cy(L) == -1 && y == 0) gyp = ny + 1;
  else if (cy(L) == 1 && y == ny - 1) gyp = 0;
  if (gxp < 0 && gyp < 0) return;
  FT* fl = f + L * fn + static_cast<long long>(z) * py * px;
  if (gxp >= 0) fl[static_cast<long long>(y + 1) * px + gxp] = v;
  if (gyp >= 0) fl[static_cast<long long>(gyp) * px + x + gx] = v;
  if (gxp >= 0 && gyp >= 0) fl[static_cast<long long>(gyp) * px + gxp] = v;
}

// ------------------------------------------------------- k_collide: the fused update --

// QF: velocity set of f (19 or 27); g and the phi stencils are D3Q19 either way.
// kRatio: the density-ratio model (f carries p* = p / (rho cs^2); see DensityRatio below).
// kWide: 64-bit f offsets, for cases with QF * ncell >= 2^31; otherwise the offsets
// l * ncell + cell are 32-bit signed integers (measured 9-12 % fewer instructions).
template <class S, int GM, int BX, int BY, bool kTma = false, int QF = kQ, bool kRatio = false,
          bool kWide = false>
__device__ __forceinline__ void collide_segment(const StepArgs& a, const Tile& t,
                                                TmaPipe* pipe = nullptr) {
  static_assert((QF == kQ && !kRatio) || !kTma, "the TMA collide is D3Q19, density-matched");
  constexpr bool BGK = GM == kGBgk;
  constexpr bool EQ = GM == kGEquil;
  using FT = typename S::FT;
  using GT = typename S::GT;
  constexpr int NT = BX * BY;
  constexpr int PX = BX + 4, PY = BY + 4, PP = PX * PY;  // phi plane, halo 2
  constexpr int HX = BX + 2, HY = BY + 2, HP = HX * HY;  // normals plane, halo 1
  constexpr int KPF = (PP + NT - 1) / NT;                // phi values per thread per plane
  static_assert(PX % 2 == 0 && HX % 2 == 0, "normals are computed for pairs of points in x");
  __shared__ __align__(16) float sphi[5][PP];
  __shared__ __align__(16) float snrm[4][4][HP];  // nx, ny, nz, |grad phi| of four planes

  const int nx = t.nx, ny = t.ny, nz = t.nz;
  const int nxy = nx * ny;
  const bool ref = t.bc == kBcRef, walls = t.bc == kBcWallsZ;
  const int tx = threadIdx.x, ty = threadIdx.y, tid = tx + BX * ty;
  const int x = t.xt + tx, y = t.yt + ty;
  const bool active = x < nx && y < ny;
  using IT = typename std::conditional<kWide, long long, int>::type;
  const IT n = static_cast<IT>(t.ncell);
  const long long ng = t.ncell;  // g offsets stay 64-bit (measured: 32-bit ones spill in BGK)

  const CaseDesc* cd = a.cases + t.ci;
  const float omega = __ldg(&cd->omega), omega_g = __ldg(&cd->omega_g);
  const float sigma = __ldg(&cd->sigma), sharp_c = __ldg(&cd->sharp_c);
  const float gravity = __ldg(&cd->gravity), phi_mean = __ldg(&cd->phi_mean);
  const float rho_out = kRatio ? __ldg(&cd->rho_out) : 1.f, drho = kRatio ? __ldg(&cd->drho) : 0.f;

  const int* __restrict__ pcur = a.p_cur + t.cell_off;

  // Halo cells of a phi plane handled by this thread: their in-plane offsets are fixed.
  int hoff[KPF];
#pragma unroll
  for (int k = 0; k < KPF; ++k) {
    const int i = tid + k * NT;
    if (i < PP) {
      int gx = t.xt - 2 + i % PX, gy = t.yt - 2 + i / PX;
      if (!ref) {
        gx = wrap1(gx, nx);
        gy = wrap1(gy, ny);
      }
      hoff[k] = clampi(gx, 0, nx - 1) + clampi(gy, 0, ny - 1) * nx;
    } else {
      hoff[k] = 0;
    }
  }
  auto zmap = [&](int z) -> int {
    if (t.bc == kBcPeriodic) z = wrap1(z, nz);
    else if (walls) z = z < 0 ? -1 - z : (z >= nz ? 2 * nz - 1 - z : z);  // mirror
    return clampi(z, 0, nz - 1);
  };
  int pre[KPF];
  auto issue = [&](int zpl) {
    const int* base = pcur + static_cast<long long>(zmap(zpl)) * nxy;
#pragma unroll
    for (int k = 0; k < KPF; ++k)
      if (tid + k * NT < PP) pre[k] = __ldg(base + hoff[k]);
  };
  auto commit = [&](int zpl) {
    float* d = sphi[(zpl + 5) % 5];
#pragma unroll
    for (int k = 0; k < KPF; ++k)
      if (tid + k * NT < PP) d[tid + k * NT] = __int2float_rn(pre[k]) * kInvQ30;
  };
  // kPush (every kernel but the TMA one): the collide kernel writes the next update's phi
  // itself. Each cell s pushes its 19 exact Q2.30 populations to their consumers s + c_l:
  // with equilibrium g q_l = w_l(P_s) + m_l c_l.J'_s (the integers the record rebuild
  // pulls), with stored g the integers it stores and the rest part P_s - sum q. Inside the
  // tile they go through a 4-plane shared ring of integer sums (tile + halo 1), flushed to
  // global memory with integer atomic adds once a target plane is complete. Integer sums do
  // not depend on the order, so the next phi is the pulled sum, bit for bit, with no phi
  // kernel.
  constexpr bool kPush = !kTma;
  __shared__ int sacc[kPush ? 4 : 1][kPush ? HP : 1];
  int* __restrict__ pnext = kPush ? a.p_next + t.cell_off : nullptr;
  int* __restrict__ pzero = kPush ? a.p_zero + t.cell_off : nullptr;
  // Global in-plane offsets of this thread's two accumulator positions (-1: none).
  int aoff[2] = {-1, -1};
  if constexpr (kPush) {
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      const int i = tid + k * NT;
      if (i >= HP) continue;
      int gx = t.xt - 1 + i % HX, gy = t.yt - 1 + i / HX;
      if (ref) {
        // outside the lattice, or a shell cell (its phi is the lagged copy): no target
        if (gx <= 0 || gx >= nx - 1 || gy <= 0 || gy >= ny - 1) continue;
      } else {
        gx = wrap1(gx, nx);
        gy = wrap1(gy, ny);
        if (gx < 0 || gx >= nx || gy < 0 || gy >= ny) continue;
      }
      aoff[k] = gx + gy * nx;
    }
    for (int i = tid; i < 4 * HP; i += NT) (&sacc[0][0])[i] = 0;
  }
  // Adds the integer sums of target plane q to the next phi and clears the ring slot.
  auto flush = [&](int q) {
    if constexpr (kPush) {
      int* slot = sacc[(q + 8) % 4];
      int qz = q;
      if (t.bc == kBcPeriodic) qz = wrap1(q, nz);
      const bool plane_ok = ref ? (qz > 0 && qz < nz - 1) : (qz >= 0 && qz < nz);
#pragma unroll
      for (int k = 0; k < 2; ++k) {
        const int i = tid + k * NT;
        if (i >= HP) continue;
        const int v = slot[i];
        slot[i] = 0;
        if (v != 0 && plane_ok && aoff[k] >= 0)
          atomicAdd(pnext + aoff[k] + static_cast<long long>(qz) * nxy, v);
      }
    }
  };

  // Phi-plane offset c of normals point i (the same on every plane), stored as -c - 1
  // where (reference mode) the point is on or beyond the shell in x or y and its normal
  // is 0: a table filled here, once per run (the rings fill after the barrier that
  // follows).
  __shared__ int scen[HP];
  for (int i = tid; i < HP; i += NT) {
    const int hx = i % HX, hy = i / HX;
    const int gx = t.xt - 1 + hx, gy = t.yt - 1 + hy;
    const bool zero = ref && (gx <= 0 || gx >= nx - 1 || gy <= 0 || gy >= ny - 1);
    const int c = (hy + 1) * PX + hx + 1;
    scen[i] = zero ? -c - 1 : c;
  }
  // Normals and |grad phi| of plane zp on the halo-1 region (gradCalc, src/lbm.cu:34-72).
  // A thread takes two neighbouring points in x and computes both with packed FP32 pairs
  // (each lane the same fused operations in the same order as one point alone). Their
  // first point sits at an odd phi-plane offset, so the neighbours at x -+ 1 of the pair
  // are aligned pairs in shared memory.
  auto normals = [&](int zp) {
    const float* pm = sphi[(zp + 4) % 5];
    const float* p0 = sphi[(zp + 5) % 5];
    const float* pp = sphi[(zp + 6) % 5];
    float(*dst)[HP] = snrm[(zp + 4) % 4];
    const bool zshell = ref && (zp <= 0 || zp >= nz - 1);
    // 16-bit relaxed g (the heaviest per-cell work, its g decode) hands the pairs out from
    // the last thread down, away from the threads that take the second phi points of
    // commit and the second ring positions of flush: 15 % faster there, 1-2 % slower in
    // the other forms.
    constexpr bool kTopDown = BGK && S::kDev;
    for (int j = kTopDown ? NT - 1 - tid : tid; 2 * j < HP; j += NT) {
      const int e0 = scen[2 * j], e1 = scen[2 * j + 1];
      const int c = e0 >= 0 ? e0 : -e0 - 1;  // the pair's first point; the second is c + 1
      float2 gx = make_float2(0.f, 0.f), gy = gx, gz = gx;
      static_for<1, kQ>([&](auto LC) {
        constexpr int L = decltype(LC)::value;
        constexpr float w3 = 3.0f * wf(L);
        const float* q = nbr_of<cz(L)>(pm, p0, pp) + c + cy(L) * PX + cx(L);
        const float2 v =
            cx(L) != 0 ? *reinterpret_cast<const float2*>(q) : make_float2(q[0], q[1]);
        if constexpr (cx(L) != 0) gx = __ffma2_rn(make_float2(cx(L) * w3, cx(L) * w3), v, gx);
        if constexpr (cy(L) != 0) gy = __ffma2_rn(make_float2(cy(L) * w3, cy(L) * w3), v, gy);
        if constexpr (cz(L) != 0) gz = __ffma2_rn(make_float2(cz(L) * w3, cz(L) * w3), v, gz);
      });
      const float2 g2 = __ffma2_rn(gz, gz, __ffma2_rn(gy, gy, __fmul2_rn(gx, gx)));
      float2 fac = make_float2(rsqrtf(fmaxf(g2.x, 1e-9f)), rsqrtf(fmaxf(g2.y, 1e-9f)));
      // zero normals on the reference shell
      if (zshell || e0 < 0) fac.x = 0.f;
      if (zshell || e1 < 0) fac.y = 0.f;
      reinterpret_cast<float2*>(dst[0])[j] = __fmul2_rn(gx, fac);
      reinterpret_cast<float2*>(dst[1])[j] = __fmul2_rn(gy, fac);
      reinterpret_cast<float2*>(dst[2])[j] = __fmul2_rn(gz, fac);
      reinterpret_cast<float2*>(dst[3])[j] = __fmul2_rn(g2, fac);
    }
  };

  // Per-thread neighbour offsets in x and y (periodic wrap; reference-mode interior cells
  // never reach past the shell).
  const int xm = x == 0 ? nx - 1 : x - 1, xp = x == nx - 1 ? 0 : x + 1;
  const int ym = (y == 0 ? ny - 1 : y - 1) * nx, yo = y * nx;
  const int yp = (y == ny - 1 ? 0 : y + 1) * nx;
  const bool shell_xy = ref && (x == 0 || x == nx - 1 || y == 0 || y == ny - 1);

  const FT* __restrict__ fin = static_cast<const FT*>(a.f_in) + t.f_off;
  FT* __restrict__ fout = static_cast<FT*>(a.f_out) + t.f_off;
  // f layout. Blocked (equilibrium g, all but the TMA kernel): population l of cell
  // (x, y, z) at fz(z) + fy(y) + fx(x) + l*32, with fz = z*PS, fy = y*RS,
  // fx = (x/32)*Q*32 + x%32. Per thread the x and y terms of a cell and of its pull sources
  // (x -+ 1, y -+ 1, with periodic wrap) are fixed; per plane the z terms are uniform.
  // Plain (stored g, and 64-bit offsets: those kernels have no registers to spare for the
  // terms): population l at l*n + cell index.
  constexpr bool kBlocked = EQ && !kTma && !kWide;
  const IT RS = static_cast<IT>(t.fxb) * (QF * 32);
  const IT PS = RS * ny;
  auto fxof = [](int xs) -> IT { return static_cast<IT>(xs >> 5) * (QF * 32) + (xs & 31); };
  const IT fx0 = kBlocked ? fxof(x) : 0, fxm = kBlocked ? fxof(xm) : 0;
  const IT fxp = kBlocked ? fxof(xp) : 0;
  const IT fy0 = kBlocked ? static_cast<IT>(y) * RS : 0;
  const IT fym = kBlocked ? static_cast<IT>(y == 0 ? ny - 1 : y - 1) * RS : 0;
  const IT fyp = kBlocked ? static_cast<IT>(y == ny - 1 ? 0 : y + 1) * RS : 0;
  const GT* __restrict__ gin = static_cast<const GT*>(a.g_in) + t.g_off;
  GT* __restrict__ gout = static_cast<GT*>(a.g_out) + t.g_off;
  const int* __restrict__ rest_in = (EQ || kPush) ? nullptr : a.rest_in + t.cell_off;
  int* __restrict__ rest_out = (EQ || kPush) ? nullptr : a.rest_out + t.cell_off;
  float4* __restrict__ jout = EQ ? static_cast<float4*>(a.j) + t.cell_off : nullptr;
  const int* __restrict__ pprev = a.p_prev + t.cell_off;

  // 16-bit relaxed g decodes every pulled population against the weight split of its source
  // cell's previous phi. A 4-plane ring of that previous phi (tile + halo 1, exact integers)
  // serves the 18 sources of a cell from shared memory instead of 18 global loads. Plane q
  // sits in slot q & 3; the slot of plane z + 2 is written after the barrier of plane z,
  // when every thread has finished plane z - 1, the last to read plane z - 2 there.
  // (Only where the block's static shared memory stays within 48 KB: not the 64x4 tile.)
  constexpr int kSmemNoRing = (5 * PP + 16 * HP + 4 * HP + HP) * 4;
  constexpr bool kPRing = BGK && S::kDev && !kTma && kSmemNoRing + 16 * HP <= 48 * 1024;
  constexpr int KPR = kPRing ? (HP + NT - 1) / NT : 1;
  __shared__ int sprev[kPRing ? 4 : 1][kPRing ? HP : 1];
  int proff[KPR], ppre[KPR];
  if constexpr (kPRing) {
#pragma unroll
    for (int k = 0; k < KPR; ++k) {
      const int i = tid + k * NT;
      int gx = t.xt - 1 + i % HX, gy = t.yt - 1 + i / HX;  // reference mode has no BGK g
      gx = ((gx % nx) + nx) % nx;
      gy = ((gy % ny) + ny) % ny;
      proff[k] = i < HP ? gx + gy * nx : 0;
    }
  }
  auto prev_issue = [&](int q) {
    if constexpr (kPRing) {
      const int zq = t.bc == kBcPeriodic ? wrap1(q, nz) : clampi(q, 0, nz - 1);
      const int* base = pprev + static_cast<long long>(zq) * nxy;
#pragma unroll
      for (int k = 0; k < KPR; ++k)
        if ((k + 1) * NT <= HP || tid + k * NT < HP) ppre[k] = __ldg(base + proff[k]);
    }
  };
  auto prev_commit = [&](int q) {
    if constexpr (kPRing) {
#pragma unroll
      for (int k = 0; k < KPR; ++k)
        if ((k + 1) * NT <= HP || tid + k * NT < HP) sprev[q & 3][tid + k * NT] = ppre[k];
    }
  };

  // f layout of the stores: plain (fn = n, cell index) or padded (TMA variant).
  const long long fn = kTma ? t.fn : n;
  const bool ghosts = kTma && !ref;
  using Box = TmaBox<FT>;
  const unsigned it0 = kTma ? pipe->it : 0u;
  if constexpr (kTma) {
    // Planes zb and zb+1 into the two stages; each later plane is issued when the stage
    // it reuses has been read.
    if (tid == 0) {
      for (int k = 0; k < 2 && t.zb + k < t.ze; ++k) {
        const unsigned st = (it0 + k) & 1u;
        tma_issue_plane<FT>(*pipe, pipe->buf + st * Box::kStageBytes, pipe->mbar + st, t.xt,
                            t.yt, t.zb + k, nz, t.bc, t.fgx);
      }
    }
  }

  // Pushes the populations of source cell (x, y, z), phi P and integer flux J', into the
  // shared ring: q_l to target plane z + cz(l), the rest part and populations bounced at a
  // z wall to the cell itself.
  // Adds population L of the cell, value(L), to its consumer in the ring: L = 1..18 first,
  // then the rest part (value(0)), so a value may depend on the ones before it.
  auto push_values = [&](int z, auto&& value) {
    if constexpr (kPush) {
      const int o = (ty + 1) * HX + tx + 1;
      int* s0 = &sacc[(z + 8) & 3][o];
      int* sm = &sacc[(z + 7) & 3][o];
      int* sp = &sacc[(z + 9) & 3][o];
      if (walls && (z == 0 || z == nz - 1)) {
        // A wall plane: what leaves through the wall returns to the cell itself.
        const bool blo = z == 0, bhi = z == nz - 1;
        static_for<1, kQ>([&](auto LC) {
          constexpr int L = decltype(LC)::value;
          constexpr int D = cy(L) * HX + cx(L);
          const int q = value(LC);
          const bool bounce = cz(L) < 0 ? blo : (cz(L) > 0 ? bhi : false);
          int* tgt = cz(L) < 0 ? sm + D : (cz(L) > 0 ? sp + D : s0 + D);
          atomicAdd(bounce ? s0 : tgt, q);
        });
      } else {
        // Every other plane: fixed shared offsets (immediates of the atomics).
        static_for<1, kQ>([&](auto LC) {
          constexpr int L = decltype(LC)::value;
          constexpr int D = cy(L) * HX + cx(L);
          int* b = cz(L) < 0 ? sm : (cz(L) > 0 ? sp : s0);
          atomicAdd(b + D, value(LC));
        });
      }
      atomicAdd(s0, value(std::integral_constant<int, 0>{}));
    }
  };
  // Equilibrium g of phi P and integer flux J'.
  auto push = [&](int z, int P, const JQ& jq) {
    const int wfc = wsplit_face(P), wed = wsplit_edge_of_face(wfc);
    push_values(z, [&](auto LC) {
      constexpr int L = decltype(LC)::value;
      if constexpr (L == 0) return P - 6 * wfc - 12 * wed;  // the rest part
      else return (L <= 6 ? wfc : wed) + qj<L>(jq);
    });
  };

  // Normals one plane ahead: each plane takes one barrier, after which the normals of
  // plane z+2 go into the fourth ring slot while the collision of plane z reads planes
  // z-1 .. z+1.
  // Prologue: phi planes zb-2 .. zb+2, normals zb-1 .. zb+1.
  for (int zpl = t.zb - 2; zpl <= t.zb + 2; ++zpl) {
    issue(zpl);
    commit(zpl);
  }
  issue(t.zb + 3);
  for (int q = t.zb - 1; q <= t.zb + 1; ++q) {
    prev_issue(q);
    prev_commit(q);
  }
  prev_issue(t.zb + 2);
  __syncthreads();
  for (int zpl = t.zb - 1; zpl <= t.zb + 1; ++zpl) normals(zpl);
  __syncthreads();

  for (int z = t.zb; z < t.ze; ++z) {
    commit(z + 3);
    if (z + 4 <= t.ze + 1) issue(z + 4);

    const int zo = z * nxy;
    const int idx = x + yo + zo;
    const bool shell = shell_xy || (ref && (z == 0 || z == nz - 1));
    const bool work = active && !shell;
    const int zm = (z == 0 ? nz - 1 : z - 1) * nxy;
    const int zp = (z == nz - 1 ? 0 : z + 1) * nxy;
    const bool blo = walls && z == 0, bhi = walls && z == nz - 1;

    // This cell's phi (read now, used after the barrier).
    const int pc = active ? __ldg(pcur + idx) : 0;
    // Pull the 19 f populations (issued before the barriers to overlap their latency).
    FT fr[QF];
    if constexpr (kTma) {
      const unsigned k = it0 + static_cast<unsigned>(z - t.zb);
      const unsigned st = k & 1u;
      const bool ok = mbar_wait_bounded(pipe->mbar + st, (k >> 1) & 1u);
      if (work && ok) {
        const FT* box = reinterpret_cast<const FT*>(pipe->buf + st * Box::kStageBytes);
        static_for<0, kQ>([&](auto LC) {
          constexpr int L = decltype(LC)::value;
          // Column of x - c_l in the box of l (its origin is 16-byte aligned); across a
          // z wall the box holds the cell's own column.
          constexpr int RX = cx(L) == 1 ? Box::kGX - 1 : (cx(L) == -1 ? 1 : 0);
          const bool bounce = (cz(L) == 1) ? blo : ((cz(L) == -1) ? bhi : false);
          const int rx = (RX != 0 && bounce) ? 0 : RX;
          fr[L] = box[L * (Box::kBytes / static_cast<int>(sizeof(FT))) + ty * Box::kW + tx + rx];
        });
      }
      if (__syncthreads_or(!ok)) {
        // A box never arrived: flag it, let the copies in flight land, leave the launch.
        if (tid == 0) {
          atomicExch(a.err, kErrTmaWait);
          for (int q = 0; q < 2; ++q) {
            const unsigned kk = k + q;
            if (t.zb + static_cast<int>(kk - it0) < t.ze)
              mbar_wait_bounded(pipe->mbar + (kk & 1u), (kk >> 1) & 1u);
          }
        }
        __syncthreads();
        pipe->failed = true;
        return;
      }
      // Every thread has read stage st: refill it with plane z + 2.
      if (tid == 0 && z + 2 < t.ze)
        tma_issue_plane<FT>(*pipe, pipe->buf + st * Box::kStageBytes, pipe->mbar + st, t.xt,
                            t.yt, z + 2, nz, t.bc, t.fgx);
    } else if (work) {
      const IT fz0 = static_cast<IT>(z) * PS;
      // this cell's population 0
      const FT* __restrict__ fc = kBlocked ? fin + (fz0 + fy0 + fx0) : fin + idx;
      // the stride between populations
      constexpr int kLS = kBlocked ? 32 : 0;
      const IT ls = kBlocked ? static_cast<IT>(kLS) : n;
      fr[0] = S::fload(fc);
      // Population L of source cell x - c_L. Blocked: its x, y and z terms, then L*32 as an
      // immediate offset. Plain: L*n + cell (32-bit: one signed offset; 64-bit: the base
      // pointer first, cheaper there).
      auto pull = [&](auto LC, IT fzm, IT fzp) {
        constexpr int L = decltype(LC)::value;
        if constexpr (kBlocked) {
          const IT s = src_of<cz(L)>(fzm, fz0, fzp) + src_of<cy(L)>(fym, fy0, fyp) +
                       src_of<cx(L)>(fxm, fx0, fxp);
          fr[L] = S::fload(fin + s + L * kLS);
        } else {
          const int s = src_of<cz(L)>(zm, zo, zp) + src_of<cy(L)>(ym, yo, yp) +
                        src_of<cx(L)>(xm, x, xp);
          if constexpr (kWide) fr[L] = S::fload(fin + L * n + s);
          else fr[L] = S::fload(fin + (L * n + s));
        }
      };
      const IT fzm = static_cast<IT>(z == 0 ? nz - 1 : z - 1) * PS;
      const IT fzp = static_cast<IT>(z == nz - 1 ? 0 : z + 1) * PS;
      if (blo || bhi) {
        // A wall plane: what left through the wall returns as the cell's own opposite
        // population.
        static_for<1, QF>([&](auto LC) {
          constexpr int L = decltype(LC)::value;
          constexpr int O = opp(L);
          const bool bounce = (cz(L) == 1) ? blo : ((cz(L) == -1) ? bhi : false);
          if (bounce) fr[L] = S::fload(fc + O * ls);
          else pull(LC, fzm, fzp);
        });
      } else {
        static_for<1, QF>([&](auto LC) { pull(LC, fzm, fzp); });
      }
    }
    if constexpr (!kTma) __syncthreads();  // the TMA path synchronised in its wait
    if constexpr (kPRing) {
      prev_commit(z + 2);
      if (z + 3 <= t.ze + 1) prev_issue(z + 3);
    }
    if (kPush && z - 2 >= t.zb - 1) flush(z - 2);  // complete: sources z-3 .. z-1 are in
    if (z + 2 <= t.ze) normals(z + 2);
    if (!active) continue;

    if constexpr (kPush) pzero[idx] = 0;  // the next update accumulates into it
    if (shell) {
      // Reference shell cell: rest-equilibrium inflow g = W_l * phi_b
      // (fgBoundary, src/lbm.cu:391-400); its f stays at W_l (rho_b = 1) from the init.
      if constexpr (kPush) {
        // no flux; the shell's own next phi is the lagged copy of its nearest interior cell
        push(z, pc, JQ{0, 0, 0});
        pnext[idx] = __ldg(pcur + clampi(x, 1, nx - 2) + clampi(y, 1, ny - 2) * nx +
                           clampi(z, 1, nz - 2) * nxy);
      } else if constexpr (EQ) {
        jout[idx] = make_float4(__int_as_float(pc), __int_as_float(0), __int_as_float(0),
                                __int_as_float(0));
      }
      if constexpr (!EQ) {
        static_for<1, kQ>([&](auto LC) {
          constexpr int L = decltype(LC)::value;
          gout[(L - 1) * ng + idx] = S::template g_shell<L>(pc);
        });
        if constexpr (!kPush) rest_out[idx] = S::rest_shell(pc);
      }
      if (a.macros) {
        const long long T = a.cells_total, o = t.cell_off + idx;
        a.macros[o] = __int2float_rn(pc) * kInvQ30;
        a.macros[T + o] = 1.0f;
        a.macros[2 * T + o] = 0.0f;
        a.macros[3 * T + o] = 0.0f;
        a.macros[4 * T + o] = 0.0f;
      }
      continue;
    }

    // Curvature and interfacial force (curvatureCalc, src/lbm.cu:80-125). Each neighbour
    // contributes c.n, so only the components along its nonzero c are read.
    const float(*nm)[HP] = snrm[(z + 3) % 4];
    const float(*n0)[HP] = snrm[(z + 4) % 4];
    const float(*np)[HP] = snrm[(z + 5) % 4];
    const int hc = (ty + 1) * HX + tx + 1;
    const float4 nc = make_float4(n0[0][hc], n0[1][hc], n0[2][hc], n0[3][hc]);
    float kap = 0.f;
    static_for<1, kQ>([&](auto LC) {
      constexpr int L = decltype(LC)::value;
      constexpr float w3 = 3.0f * wf(L);
      const float(*pl)[HP] = nbr_of<cz(L)>(nm, n0, np);
      const int o = hc + cy(L) * HX + cx(L);
      float cn = 0.f;
      if constexpr (cx(L) != 0) cn += cx(L) * pl[0][o];
      if constexpr (cy(L) != 0) cn += cy(L) * pl[1][o];
      if constexpr (cz(L) != 0) cn += cz(L) * pl[2][o];
      kap -= w3 * cn;
    });
    const float phi = sphi[(z + 5) % 5][(ty + 2) * PX + tx + 2];
    const float mult = sigma * kap;
    float Fx = mult * nc.x * nc.w;
    float Fy = mult * nc.y * nc.w;
    float Fz = mult * nc.z * nc.w;
    if (gravity != 0.f) Fz += gravity * (phi - phi_mean);

    // Moments (momentiCalc, src/lbm.cu:133-225). The non-equilibrium second moment is
    // sum c c (f - feq + HeF). For the D3Q19 second-order equilibrium its equilibrium
    // and forcing parts reduce in closed form:
    //   sum c_a c_b feq = rho (cs^2 d_ab + u_a u_b)
    //   sum c_a c_b HeF = (u_a F_b + u_b F_a)/2 - 3/2 (u.F) u_a u_b
    // This uses the 4th-order isotropy of D3Q19 and D3Q27.
    // 16-bit storage holds f_l - W_l: its moments start from those of the weights
    // (sum W = 1, sum W c_a c_b = d_ab / 3, odd moments 0).
    float f[QF];
    static_for<0, QF>([&](auto LC) {
      constexpr int L = decltype(LC)::value;
      f[L] = S::template f_raw<L>(fr[L]);
    });
    // The density-ratio f is small (p* starts at 0) and is stored as it is.
    constexpr bool kDevF = S::kFDev && !kRatio;
    constexpr float m0 = kDevF ? 1.0f : 0.0f, m2 = kDevF ? 1.0f / 3.0f : 0.0f;
    float rho = m0, jx = 0.f, jy = 0.f, jz = 0.f;
    float sxx = m2, syy = m2, szz = m2, sxy = 0.f, sxz = 0.f, syz = 0.f;
    if constexpr (EQ) {
      // Opposite pairs (l odd, l + 1): their sum feeds rho and the second moments, their
      // difference the momentum (about 30 % fewer adds than population by population).
      rho += f[0];
      static_for<0, (QF - 1) / 2>([&](auto KC) {
        constexpr int L = 2 * decltype(KC)::value + 1;
        const float sp = f[L] + f[L + 1], dm = f[L] - f[L + 1];
        rho += sp;
        if constexpr (cx(L) != 0) { jx += cx(L) * dm; sxx += sp; }
        if constexpr (cy(L) != 0) { jy += cy(L) * dm; syy += sp; }
        if constexpr (cz(L) != 0) { jz += cz(L) * dm; szz += sp; }
        if constexpr (cx(L) * cy(L) != 0) sxy += (cx(L) * cy(L)) * sp;
        if constexpr (cx(L) * cz(L) != 0) sxz += (cx(L) * cz(L)) * sp;
        if constexpr (cy(L) * cz(L) != 0) syz += (cy(L) * cz(L)) * sp;
      });
    } else {
      static_for<0, QF>([&](auto LC) {
        constexpr int L = decltype(LC)::value;
        const float v = f[L];
        rho += v;
        if constexpr (cx(L) != 0) { jx += cx(L) * v; sxx += v; }
        if constexpr (cy(L) != 0) { jy += cy(L) * v; syy += v; }
        if constexpr (cz(L) != 0) { jz += cz(L) * v; szz += v; }
        if constexpr (cx(L) * cy(L) != 0) sxy += (cx(L) * cy(L)) * v;
        if constexpr (cx(L) * cz(L) != 0) sxz += (cx(L) * cz(L)) * v;
        if constexpr (cy(L) * cz(L) != 0) syz += (cy(L) * cz(L)) * v;
      });
    }
    float ux, uy, uz, pxx, pyy, pzz, pxy, pxz, pyz, inv_rp = 0.f, rp = 1.f;
    if constexpr (kRatio) {
      // DensityRatio: velocity-based pressure formulation (Zu and He 2013; Fakhari et al.
      // 2017) with rho = rho_out + drho phi and grad rho = drho grad phi, grad phi being
      // n |grad phi| of the isotropic stencil.
      //   p* = sum f, u* = sum c f, Pi* = sum c c f - p*/3 I - u* u*,
      //   F += -p*/3 grad rho - (1 - omega/2) Pi* . grad rho,   u = u* + F / (2 rho).
      rp = rho_out + drho * phi;
      inv_rp = 1.0f / rp;
      const float gx = drho * nc.x * nc.w, gy = drho * nc.y * nc.w, gz = drho * nc.z * nc.w;
      const float p3 = rho * (1.0f / 3.0f);
      const float qxx = sxx - p3 - jx * jx, qyy = syy - p3 - jy * jy, qzz = szz - p3 - jz * jz;
      const float qxy = sxy - jx * jy, qxz = sxz - jx * jz, qyz = syz - jy * jz;
      const float cm = 1.0f - 0.5f * omega;
      Fx = Fx - p3 * gx - cm * (qxx * gx + qxy * gy + qxz * gz);
      Fy = Fy - p3 * gy - cm * (qxy * gx + qyy * gy + qyz * gz);
      Fz = Fz - p3 * gz - cm * (qxz * gx + qyz * gy + qzz * gz);
      ux = jx + 0.5f * Fx * inv_rp;
      uy = jy + 0.5f * Fy * inv_rp;
      uz = jz + 0.5f * Fz * inv_rp;
      pxx = sxx - p3 - ux * ux;
      pyy = syy - p3 - uy * uy;
      pzz = szz - p3 - uz * uz;
      pxy = sxy - ux * uy;
      pxz = sxz - ux * uz;
      pyz = syz - uy * uz;
    } else {
      const float inv_rho = 1.0f / rho;
      ux = (jx + 0.5f * Fx) * inv_rho;
      uy = (jy + 0.5f * Fy) * inv_rho;
      uz = (jz + 0.5f * Fz) * inv_rho;
      const float uF = ux * Fx + uy * Fy + uz * Fz;
      const float h = 1.5f * uF;
      pxx = sxx - rho * (1.0f / 3.0f + ux * ux) + ux * Fx - h * ux * ux;
      pyy = syy - rho * (1.0f / 3.0f + uy * uy) + uy * Fy - h * uy * uy;
      pzz = szz - rho * (1.0f / 3.0f + uz * uz) + uz * Fz - h * uz * uz;
      pxy = sxy - rho * ux * uy + 0.5f * (ux * Fy + uy * Fx) - h * ux * uy;
      pxz = sxz - rho * ux * uz + 0.5f * (ux * Fz + uz * Fx) - h * ux * uz;
      pyz = syz - rho * uy * uz + 0.5f * (uy * Fz + uz * Fy) - h * uy * uz;
    }
    const float uF = ux * Fx + uy * Fy + uz * Fz;
    const float u2 = ux * ux + uy * uy + uz * uz;
    const float h = 1.5f * uF;
    const float tr3 = (pxx + pyy + pzz) * (1.0f / 3.0f);

    // Regularized collision with He forcing (collisionFluid, src/lbm.cu:233-288):
    //   f*_l = feq_l + (1 - omega) W_l/(2 cs^4) Q_l:Pi + HeF_l
    //        = W_l [E_l (rho + 3/2 (c_l.F - u.F)) + 9/2 (1 - omega) Q_l:Pi]
    // with E_l = 1 + 3 c.u + 9/2 (c.u)^2 - 3/2 u^2. Opposite pairs share Q_l:Pi and flip
    // c.u and c.F.
    const float om = (1.0f - omega) * 4.5f;
    // Deviation storage writes f*_l - W_l: the -1 folds into the shared term of each pair.
    constexpr float fshift = kDevF ? -1.0f : 0.0f;
    const float R = rho - h;
    // DensityRatio: f*_l = W_l [p* + 3 c.u + 9/2 (c.u)^2 - 3/2 u^2 + 9/2 (1 - omega) Q_l:Pi
    //                          + (1 - omega/2) 3 c.F / rho].
    const float base = kRatio ? rho - 1.5f * u2 : 1.0f - 1.5f * u2;
    const float cf = kRatio ? (1.0f - 0.5f * omega) * 3.0f * inv_rp : 0.f;
    // g collision (collisionPhase, src/lbm.cu:290-329):
    //   geq_l = W_l [phi (1 + 3 c.u) + sharp_c phi (1 - phi) c.n]
    // tau_g = 1 takes g* = geq as the reference does; otherwise BGK with omega_g.
    const float A = sharp_c * phi * (1.0f - phi);
    const float phi3 = 3.0f * phi;

    float fo[QF];
    float go[kQ];
    if constexpr (kRatio) fo[0] = wfq<QF>(0) * (base - om * tr3);
    else fo[0] = wfq<QF>(0) * (base * R - om * tr3 + fshift);
    static_for<0, (QF - 1) / 2>([&](auto KC) {
      constexpr int L = 2 * decltype(KC)::value + 1;
      constexpr int O = L + 1;
      constexpr float W = wfq<QF>(L);
      float cu = 0.f, cF = 0.f, cn = 0.f, qp = -tr3;
      if constexpr (cx(L) != 0) { cu += cx(L) * ux; cF += cx(L) * Fx; cn += cx(L) * nc.x; qp += pxx; }
      if constexpr (cy(L) != 0) { cu += cy(L) * uy; cF += cy(L) * Fy; cn += cy(L) * nc.y; qp += pyy; }
      if constexpr (cz(L) != 0) { cu += cz(L) * uz; cF += cz(L) * Fz; cn += cz(L) * nc.z; qp += pzz; }
      if constexpr (cx(L) * cy(L) != 0) qp += (2 * cx(L) * cy(L)) * pxy;
      if constexpr (cx(L) * cz(L) != 0) qp += (2 * cx(L) * cz(L)) * pxz;
      if constexpr (cy(L) * cz(L) != 0) qp += (2 * cy(L) * cz(L)) * pyz;
      const float q = om * qp + fshift;
      const float e0 = base + 4.5f * cu * cu, e1 = 3.0f * cu;
      if constexpr (kRatio) {
        const float fe = cf * cF;
        fo[L] = W * (e0 + q + (e1 + fe));
        fo[O] = W * (e0 + q - (e1 + fe));
      } else {
        // The weight stays outside the bracket. Folding it into the terms (W base + ...)
        // changed the rounding of the small non-equilibrium part enough to shift the D3Q27
        // shear-wave viscosity by 4 %; summing opposite pairs first in the moments moved
        // the 2000-update static bubble 1.4e-4 from the FP64 oracle (1.5 % faster).
        const float rf = 1.5f * cF;
        fo[L] = W * ((e0 + e1) * (R + rf) + q);
        fo[O] = W * ((e0 - e1) * (R - rf) + q);
      }
      if constexpr (L < kQ) {
        constexpr float WG = wf(L);  // g is D3Q19
        const float dg = phi3 * cu + A * cn;
        go[L] = WG * (phi + dg);
        go[O] = WG * (phi - dg);
      }
    });

    if constexpr (kTma) {
      const long long pidx = (static_cast<long long>(z) * t.fpy + y + 1) * t.fpx + x + t.fgx;
      static_for<0, kQ>([&](auto LC) {
        constexpr int L = decltype(LC)::value;
        const FT v = S::template f_put<L>(fo[L]);
        fout[L * fn + pidx] = v;
        if (ghosts) f_ghosts<L>(fout, fn, x, y, z, nx, ny, t.fgx, t.fpx, t.fpy, v);
      });
    } else {
      if constexpr (kBlocked) {
        FT* __restrict__ fc = fout + (static_cast<IT>(z) * PS + fy0 + fx0);
        static_for<0, QF>([&](auto LC) {
          constexpr int L = decltype(LC)::value;
          fc[L * 32] = S::template f_put<L>(fo[L]);
        });
      } else {
        static_for<0, QF>([&](auto LC) {
          constexpr int L = decltype(LC)::value;
          fout[L * n + idx] = S::template f_put<L>(fo[L]);
        });
      }
    }

    if constexpr (BGK) {
      // Incoming g (pull), decoded, then relaxed towards geq.
      const int hcp = (ty + 1) * HX + tx + 1;  // this cell in the previous-phi ring
      int pself = 0;
      if constexpr (kPRing) pself = sprev[z & 3][hcp];
      else if constexpr (S::kDev) pself = __ldg(pprev + idx);
      static_for<1, kQ>([&](auto LC) {
        constexpr int L = decltype(LC)::value;
        constexpr int O = opp(L);
        const bool bounce = (cz(L) == 1) ? blo : ((cz(L) == -1) ? bhi : false);
        int gi;
        if (bounce) {
          gi = S::template g_dec<O>(S::gload(gin + (O - 1) * ng + idx), pself);
        } else {
          const int s = src_of<cz(L)>(zm, zo, zp) + src_of<cy(L)>(ym, yo, yp) +
                        src_of<cx(L)>(xm, x, xp);
          int ps = 0;  // the source x - c_l: plane z - cz, row ty - cy, column tx - cx
          if constexpr (kPRing) ps = sprev[(z - cz(L)) & 3][hcp - cy(L) * HX - cx(L)];
          else if constexpr (S::kDev) ps = __ldg(pprev + s);
          gi = S::template g_dec<L>(S::gload(gin + (L - 1) * ng + s), ps);
        }
        const float gf = __int2float_rn(gi) * kInvQ30;
        go[L] = gf + omega_g * (go[L] - gf);
      });
    } else {
      (void)omega_g;
      (void)gin;
      (void)rest_in;
    }
    if constexpr (EQ) {
      // Equilibrium storage: the 18 populations are W_l (phi + c_l . J), J = 3 phi u + A n.
      const JQ jq = jq_of(phi3 * ux + A * nc.x, phi3 * uy + A * nc.y, phi3 * uz + A * nc.z);
      if constexpr (kPush) push(z, pc, jq);
      else
        jout[idx] = make_float4(__int_as_float(pc), __int_as_float(jq.x), __int_as_float(jq.y),
                                __int_as_float(jq.z));
    } else {
      // Stored g: the 18 moving populations as stored (exact Q2.30 integers q) and the rest
      // part, the exact remainder P - sum q. In push mode they also go to their consumers'
      // next phi, and the rest part is not stored (no phi kernel reads it).
      int sumq = 0;
      const GSplit sp = S::g_split(pc);
      auto gval = [&](auto LC) {
        constexpr int L = decltype(LC)::value;
        if constexpr (L == 0) {
          return pc - sumq;
        } else {
          int q;
          gout[(L - 1) * ng + idx] = S::template g_put<L>(go[L], sp, q);
          sumq += q;
          return q;
        }
      };
      if constexpr (kPush) {
        push_values(z, gval);
      } else {
        static_for<1, kQ>(gval);
        rest_out[idx] = S::rest_store(pc, sumq);
      }
    }

    if (a.macros) {
      const long long T = a.cells_total, o = t.cell_off + idx;
      a.macros[o] = phi;
      a.macros[T + o] = kRatio ? rho * rp : rho;  // density-ratio model: p / cs^2
      a.macros[2 * T + o] = ux;
      a.macros[3 * T + o] = uy;
      a.macros[4 * T + o] = uz;
    }
  }
  if constexpr (kPush) {
    // The last target planes of the run.
    __syncthreads();
    for (int q = max(t.ze - 2, t.zb - 1); q <= t.ze; ++q) flush(q);
  }
}

// 24 resident warps per SM (80 registers) for every form. 16-bit relaxed g spills a little
// there; at 16 warps (128 registers, no spills) it measured 2 % slower.
template <class S, int GM, int BX, int BY>
__global__ void __launch_bounds__(BX * BY, kCollideWarpsPerSM * 32 / (BX * BY))
    k_collide(const StepArgs a) {
  for_each_segment<BX, BY, true>(a,
                                 [&](const Tile& t) { collide_segment<S, GM, BX, BY>(a, t); }, a.balanced != 0);
}

// Cases of 2^31 / 19 cells or more: 64-bit f offsets, 32x8 tiles.
template <class S, int GM>
__global__ void __launch_bounds__(256, kCollideWarpsPerSM / 8) k_collide_wide(const StepArgs a) {
  for_each_segment<32, 8, true>(
      a, [&](const Tile& t) { collide_segment<S, GM, 32, 8, false, kQ, false, true>(a, t); }, a.balanced != 0);
}

// The TMA variant: 32x8 tiles, f staged through shared memory (one case, (P, J) records).
template <class S>
__global__ void __launch_bounds__(kTmaBX * kTmaBY, kCollideWarpsPerSM * 32 / (kTmaBX * kTmaBY))
    k_collide_tma(const StepArgs a, const __grid_constant__ CUtensorMap fmap) {
  extern __shared__ __align__(1024) unsigned char tma_smem[];
  __shared__ __align__(8) unsigned long long mbar[2];
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    mbar_init(&mbar[0], 1);
    mbar_init(&mbar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  // Boxes start on 128-byte boundaries of the shared window.
  unsigned char* buf = tma_smem + ((128u - (smem_u32(tma_smem) & 127u)) & 127u);
  TmaPipe pipe{buf, mbar, &fmap, 0u, false};
  for_each_segment<kTmaBX, kTmaBY, true>(a, [&](const Tile& t) {
    if (pipe.failed) return;
    collide_segment<S, kGEquil, kTmaBX, kTmaBY, true>(a, t, &pipe);
    pipe.it += static_cast<unsigned>(t.ze - t.zb);
  }, a.balanced != 0);
}

// D3Q27 f: 32x8 tiles, 27 populations in flight: two blocks of eight warps per SM
// (128 registers). With equilibrium g, 16-bit storage and 32-bit offsets three blocks
// (80 registers, a small spill) measured 9 % faster at 128 x 128 x 256; at FP32 they
// measured 3 % slower, and the other forms spill three to five times as much.
template <class S, int GM, bool kWide>
constexpr int collide27_blocks() {
  return (!std::is_same<typename S::FT, float>::value && GM == kGEquil && !kWide) ? 3 : 2;
}
template <class S, int GM, bool kWide>
__global__ void __launch_bounds__(256, collide27_blocks<S, GM, kWide>())
    k_collide27(const StepArgs a) {
  for_each_segment<32, 8, true>(
      a, [&](const Tile& t) { collide_segment<S, GM, 32, 8, false, kQ27, false, kWide>(a, t); }, a.balanced != 0);
}

// Density-ratio model: 32x8 tiles; two blocks per SM for D3Q27 f, three for D3Q19.
template <class S, int GM, int QF, bool kWide>
__global__ void __launch_bounds__(256, QF == kQ27 ? 2 : kCollideWarpsPerSM / 8)
    k_collide_ratio(const StepArgs a) {
  for_each_segment<32, 8, true>(
      a, [&](const Tile& t) { collide_segment<S, GM, 32, 8, false, QF, true, kWide>(a, t); }, a.balanced != 0);
}

// ------------------------------------------------------------------ k_init: fields --

// Writes the stored populations so that the first update gathers the equilibria of the
// given fields: f_l(x) = feq_l(rho = 1, u(x)), g_l(x) = W_l phi(x) (1 + 3 c_l.u(x)).
// In pull layout the value stored at y for direction l is the one its consumer y + c_l
// reads; with bounce-back the consumer is y itself, as direction opp(l).
// (initDist, src/init.cu:51-80.)
template <class S, int QF>
__global__ void k_init(const InitArgs a) {
  using FT = typename S::FT;
  using GT = typename S::GT;
  const CaseDesc* cd = a.cases + a.case_index;
  const int nx = cd->nx, ny = cd->ny, nz = cd->nz, bc = cd->bc;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  if (x >= nx || y >= ny || z >= nz) return;
  const long long n = cd->ncell, co = cd->cell_off;
  const int idx = x + nx * (y + ny * z);
  const bool ref = bc == kBcRef, walls = bc == kBcWallsZ;
  const bool shell = ref && (x == 0 || x == nx - 1 || y == 0 || y == ny - 1 || z == 0 ||
                             z == nz - 1);
  const bool eq = a.gmode == kGEquil;
  const float phi_self = a.phi[idx];
  // Equilibrium g: the first update takes its phi from here (no phi kernel runs before
  // it); the reference's shell phi starts at 0 (src/var.cu:86). Stored g: the first
  // update's phi kernel sums the populations written below.
  const int P = (eq && shell) ? 0 : __float2int_rn(phi_self * kQ30);
  a.p0[co + idx] = P;
  a.p1[co + idx] = P;
  if (a.p_zero) a.p_zero[co + idx] = 0;
  const float ux_s = a.ux ? a.ux[idx] : 0.f;
  const float uy_s = a.uy ? a.uy[idx] : 0.f;
  const float uz_s = a.uz ? a.uz[idx] : 0.f;
  if (a.macros) {
    const long long T = a.cells_total;
    a.macros[co + idx] = phi_self;
    a.macros[T + co + idx] = 1.0f;
    a.macros[2 * T + co + idx] = ux_s;
    a.macros[3 * T + co + idx] = uy_s;
    a.macros[4 * T + co + idx] = uz_s;
  }
  FT* f0 = static_cast<FT*>(a.f0) + cd->f_off;
  FT* f1 = static_cast<FT*>(a.f1) + cd->f_off;
  // f layout: blocked (population stride 32 within a 32-cell x block), or padded (ghost
  // columns and rows, kept periodic; the TMA update).
  const int fxb = cd->fxb;
  const long long fn = fxb ? 32 : cd->fn;
  const long long fidx =
      fxb ? ((static_cast<long long>(z) * ny + y) * fxb + (x >> 5)) * (QF * 32) + (x & 31)
          : (static_cast<long long>(z) * cd->fpy + y + (cd->fgx ? 1 : 0)) * cd->fpx + x +
                cd->fgx;
  const bool fghost = cd->fgx != 0 && !ref;
  const bool ratio = cd->drho != 0.f;
  GT* g0 = static_cast<GT*>(a.g0) + cd->g_off;
  static_for<0, QF>([&](auto LC) {
    constexpr int L = decltype(LC)::value;
    int xc = x + cx(L), yc = y + cy(L), zc = z + cz(L);
    bool bounce = false;
    if (ref) {
      if (xc < 0 || xc >= nx || yc < 0 || yc >= ny || zc < 0 || zc >= nz) {
        xc = x;
        yc = y;
        zc = z;
      }
    } else {
      xc = wrap1(xc, nx);
      yc = wrap1(yc, ny);
      if (walls && (zc < 0 || zc >= nz)) {
        // Half-way bounce-back: the population returns to the cell it left.
        bounce = true;
        xc = x;
        yc = y;
        zc = z;
      } else {
        zc = wrap1(zc, nz);
      }
    }
    const int ci = xc + nx * (yc + ny * zc);
    const float ux = a.ux ? a.ux[ci] : 0.f;
    const float uy = a.uy ? a.uy[ci] : 0.f;
    const float uz = a.uz ? a.uz[ci] : 0.f;
    // Direction as seen by the consumer: opp(L) after a bounce.
    const float sx = bounce ? -cx(L) : cx(L), sy = bounce ? -cy(L) : cy(L);
    const float sz = bounce ? -cz(L) : cz(L);
    const float cu = sx * ux + sy * uy + sz * uz;
    const float u2 = ux * ux + uy * uy + uz * uz;
    constexpr float W = wfq<QF>(L);
    // density-ratio model: p* = 0 at the start, stored without the weight shift
    float feq = W * ((ratio ? 0.0f : 1.0f) + 3.0f * cu + 4.5f * cu * cu - 1.5f * u2);
    if (shell) feq = W;
    const float fst = (S::kFDev && !ratio) ? feq - W : feq;
    const FT v = S::template f_put<L>(fst);
    f0[L * fn + fidx] = v;
    // The first update writes every cell of the other buffer, except the reference-mode
    // shell, whose f stays W_l in both buffers.
    if (ref) f1[L * fn + fidx] = v;
    if (fghost) f_ghosts<L>(f0, fn, x, y, z, nx, ny, cd->fgx, cd->fpx, cd->fpy, v);
    if (eq) {
      // no g populations are stored
    } else if constexpr (L == 0) {
      if (a.rest0) a.rest0[co + idx] = S::rest_init(wf(0) * phi_self, P);
    } else if constexpr (L < kQ) {  // g is D3Q19
      const float geq = wf(L) * a.phi[ci] * (1.0f + 3.0f * cu);
      int q;
      g0[(L - 1) * n + idx] = S::template g_put<L>(geq, S::g_split(P), q);
    }
  });
}

}  // namespace
}  // namespace mcb

#include "kernels_pair.cuh"

namespace mcb {
namespace {

// ------------------------------------------------------------------------ dispatch --

// Kernel entry and block shape of each tile variant (kVariants order).
template <class S, int BX, int BY>
const void* phi_kernel_of(bool eq) {
  return eq ? reinterpret_cast<const void*>(k_phi_eq<S, BX, BY>)
            : reinterpret_cast<const void*>(k_phi<S, BX, BY>);
}

template <class S>
const void* phi_kernel(int variant, bool eq, dim3* block) {
  switch (variant) {
    case 0:
    case kTmaVariant: *block = dim3(32, 8); return phi_kernel_of<S, 32, 8>(eq);
    case 1: *block = dim3(16, 16); return phi_kernel_of<S, 16, 16>(eq);
    // the pair variants' tiles are 64 x 4 cells (stored g runs this kernel on the first
    // update of a push run)
    case kPairVariant:
    case kPairVariant + 1:
    case 2: *block = dim3(64, 4); return phi_kernel_of<S, 64, 4>(eq);
    case 3: *block = dim3(16, 8); return phi_kernel_of<S, 16, 8>(eq);
    default: return nullptr;
  }
}

template <class S, int GM>
const void* collide_kernel(int variant, dim3* block) {
  switch (variant) {
    case 0: *block = dim3(32, 8); return reinterpret_cast<const void*>(k_collide<S, GM, 32, 8>);
    case 1: *block = dim3(16, 16); return reinterpret_cast<const void*>(k_collide<S, GM, 16, 16>);
    case 2: *block = dim3(64, 4); return reinterpret_cast<const void*>(k_collide<S, GM, 64, 4>);
    case 3: *block = dim3(16, 8); return reinterpret_cast<const void*>(k_collide<S, GM, 16, 8>);
    case kPairVariant:
    case kPairVariant + 1:
      // two cells per thread (the instance without the reference-mode shell; launches pick
      // by StepArgs::has_ref)
      *block = dim3(kPairTX, kPairBY);
      return pair_kernel<S>(variant, false, GM);
    default: return nullptr;
  }
}

template <class S, int GM, bool kWide>
const void* collide_32x8_of(int qf, bool ratio) {
  if (ratio) {
    return qf == kQ27 ? reinterpret_cast<const void*>(k_collide_ratio<S, GM, kQ27, kWide>)
                      : reinterpret_cast<const void*>(k_collide_ratio<S, GM, kQ, kWide>);
  }
  if (qf == kQ27) return reinterpret_cast<const void*>(k_collide27<S, GM, kWide>);
  return kWide ? reinterpret_cast<const void*>(k_collide_wide<S, GM>) : nullptr;
}

template <class S, int GM>
const void* collide_32x8_kernel(int qf, bool ratio, bool wide) {
  return wide ? collide_32x8_of<S, GM, true>(qf, ratio)
              : collide_32x8_of<S, GM, false>(qf, ratio);
}

// The 32x8 collide kernels outside the tile variants: D3Q27 f, the density-ratio model and
// cases that need 64-bit f offsets.
template <class S>
const void* collide27_kernel(int gmode, int qf, bool ratio, bool wide) {
  switch (gmode) {
    case kGPop: return collide_32x8_kernel<S, kGPop>(qf, ratio, wide);
    case kGBgk: return collide_32x8_kernel<S, kGBgk>(qf, ratio, wide);
    case kGEquil: return collide_32x8_kernel<S, kGEquil>(qf, ratio, wide);
    default: return nullptr;
  }
}

template <class S>
const void* collide_kernel_gm(int variant, int gmode, dim3* block) {
  switch (gmode) {
    case kGPop: return collide_kernel<S, kGPop>(variant, block);
    case kGBgk: return collide_kernel<S, kGBgk>(variant, block);
    case kGEquil: return collide_kernel<S, kGEquil>(variant, block);
    default: return nullptr;
  }
}

inline cudaError_t launch_on(const void* fn, int grid, dim3 block, const StepArgs& a,
                             cudaStream_t s, int dyn_smem = 0) {
  if (!fn || grid <= 0) return cudaErrorInvalidValue;
  void* args[] = {const_cast<StepArgs*>(&a)};
  return cudaLaunchKernel(fn, dim3(grid), block, args, static_cast<size_t>(dyn_smem), s);
}

template <class S>
cudaError_t launch_collide_tma(const StepArgs& a, const void* tmap, cudaStream_t s) {
  if (!tmap || a.grid_collide <= 0) return cudaErrorInvalidValue;
  CUtensorMap map;
  memcpy(&map, tmap, sizeof map);
  k_collide_tma<S><<<a.grid_collide, dim3(kTmaBX, kTmaBY), TmaBox<typename S::FT>::kSmem, s>>>(
      a, map);
  return cudaGetLastError();
}

template <class S>
cudaError_t prepare_tma_kernel() {
  return cudaFuncSetAttribute(k_collide_tma<S>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              TmaBox<typename S::FT>::kSmem);
}

// Resident blocks per SM of the phi and collide kernels of a variant.
template <class S>
cudaError_t occupancy_of(int variant, int gmode, int qf, int ratio, int wide, int* phi_blocks,
                         int* collide_blocks) {
  if (!is_pair_variant(variant) && (qf == kQ27 || ratio || wide)) {
    dim3 bp;
    const void* fp = phi_kernel<S>(0, gmode == kGEquil, &bp);
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        phi_blocks, fp, static_cast<int>(bp.x * bp.y), 0);
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        collide_blocks, collide27_kernel<S>(gmode, qf, ratio != 0, wide != 0), 256, 0);
  }
  if (variant == kTmaVariant) {
    if (gmode != kGEquil) return cudaErrorInvalidValue;
    dim3 bp;
    const void* fp = phi_kernel<S>(0, true, &bp);
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        phi_blocks, fp, static_cast<int>(bp.x * bp.y), 0);
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        collide_blocks, k_collide_tma<S>, kTmaBX * kTmaBY, TmaBox<typename S::FT>::kSmem);
  }
  dim3 bp, bc;
  const void* fp = phi_kernel<S>(variant, gmode == kGEquil, &bp);
  const void* fc = collide_kernel_gm<S>(variant, gmode, &bc);
  if (!fp || !fc) return cudaErrorInvalidValue;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      phi_blocks, fp, static_cast<int>(bp.x * bp.y), 0);
  if (e != cudaSuccess) return e;
  int dyn = 0;
  if (is_pair_variant(variant)) {
    // Every launch of a solver follows this call on its device: the opt-in above 48 KB of
    // shared memory per block is set here.
    dyn = pair_dyn_smem<S>(gmode);
    if (dyn > 0) {
      e = cudaFuncSetAttribute(fc, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn);
      if (e != cudaSuccess) return e;
    }
  }
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(collide_blocks, fc,
                                                       static_cast<int>(bc.x * bc.y), dyn);
}

template <class S>
cudaError_t init_storage(const InitArgs& a, int nx, int ny, int nz, cudaStream_t s) {
  const dim3 block(32, 8);
  const dim3 grid((nx + 31) / 32, (ny + 7) / 8, nz);
  if (a.qf == kQ27) k_init<S, kQ27><<<grid, block, 0, s>>>(a);
  else k_init<S, kQ><<<grid, block, 0, s>>>(a);
  return cudaGetLastError();
}

// One storage format per translation unit, so the formats compile in parallel.
#define MCB_STORAGE_LAUNCHERS(S, suffix)                                                   \
  cudaError_t launch_phi_##suffix(int variant, int gmode, const StepArgs& a,               \
                                  cudaStream_t s) {                                        \
    dim3 block;                                                                            \
    const void* fn = phi_kernel<S>(variant, gmode == kGEquil, &block);                     \
    return launch_on(fn, a.grid_phi, block, a, s);                                         \
  }                                                                                        \
  cudaError_t launch_collide_##suffix(int variant, int gmode, const StepArgs& a,           \
                                      const void* tmap, cudaStream_t s) {                  \
    if (variant == kTmaVariant)                                                            \
      return gmode == kGEquil ? launch_collide_tma<S>(a, tmap, s) : cudaErrorInvalidValue; \
    if (is_pair_variant(variant))                                                          \
      return launch_on(pair_kernel<S>(variant, a.has_ref != 0, gmode), a.grid_collide,     \
                       dim3(kPairTX, kPairBY), a, s, pair_dyn_smem<S>(gmode));             \
    if (a.qf == kQ27 || a.ratio || a.wide)                                                 \
      return launch_on(collide27_kernel<S>(gmode, a.qf, a.ratio != 0, a.wide != 0),        \
                       a.grid_collide, dim3(32, 8), a, s);                                 \
    dim3 block;                                                                            \
    const void* fn = collide_kernel_gm<S>(variant, gmode, &block);                         \
    return launch_on(fn, a.grid_collide, block, a, s);                                     \
  }                                                                                        \
  cudaError_t prepare_tma_##suffix() { return prepare_tma_kernel<S>(); }                   \
  size_t tma_smem_##suffix() { return TmaBox<typename S::FT>::kSmem; }                     \
  cudaError_t occupancy_##suffix(int variant, int gmode, int qf, int ratio, int wide,      \
                                 int* phi_blocks, int* collide_blocks) {                   \
    return occupancy_of<S>(variant, gmode, qf, ratio, wide, phi_blocks, collide_blocks);   \
  }                                                                                        \
  cudaError_t launch_init_##suffix(const InitArgs& a, int nx, int ny, int nz,              \
                                   cudaStream_t s) {                                       \
    return init_storage<S>(a, nx, ny, nz, s);                                              \
  }

}  // namespace
}  // namespace mcb
