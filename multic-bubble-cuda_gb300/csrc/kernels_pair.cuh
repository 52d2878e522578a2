// k_collide_pair: the update of k_collide with two neighbouring cells in x per thread, for
// D3Q19 f at density ratio 1 (the reference's model) on the blocked f layout, with every g
// form (equilibrium g pushed; g populations stored, at full relaxation or relaxed with
// tau_g != 1; the stored forms without the reference-mode shell).
//
// It computes what k_collide computes (gradCalc, curvatureCalc, momentiCalc, collisionFluid,
// collisionPhase, streamingCalc and phiCalc of src/lbm.cu, fgBoundary and
// boundaryConditions in reference mode), in the same order per cell. What changes is the
// shape of the work:
//   - a thread owns cells x0 = xt + 2 tx and x0 + 1 of one row, so every arithmetic step of
//     the moments, the curvature, the force and the collisions runs once for both cells in
//     packed FP32 (FFMA2, FADD2, FMUL2: each lane the IEEE single-precision operation);
//   - the populations that do not move in x (9 of 19) are gathered for both cells with one
//     aligned 64-bit (FP32) or 32-bit (16-bit storage) load, and all 19 post-collision
//     populations are stored for both cells with one such store each; 16-bit storage packs
//     the pair with one conversion;
//   - equilibrium g: the 19 integer g populations of the two cells are summed per target
//     before the shared atomics where their targets coincide (28 atomics for the pair
//     instead of 38);
//   - relaxed g: the 18 pulled populations of a plane and their sources' previous phi are
//     staged in shared memory by asynchronous copies one plane ahead (cp.async), so that no
//     register holds them across the plane's barrier;
//   - the per-plane and per-segment work (phi ring, offsets, loop) is shared by two cells.
// Arithmetic and the exact integer push of phi are those of k_collide, so results agree with
// it to FP32 rounding (the fused multiply-adds are placed explicitly here). Requires an even
// nx in every case, so that a pair never straddles the lattice edge.
#pragma once

namespace pk {

__device__ __forceinline__ float2 dup(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma(float2 a, float2 b, float2 c) {
  return __ffma2_rn(a, b, c);
}
// a - b, exactly rounded: b * (-1) is exact, so the fused operation rounds once.
__device__ __forceinline__ float2 sub(float2 a, float2 b) {
  return __ffma2_rn(b, make_float2(-1.0f, -1.0f), a);
}
__device__ __forceinline__ float2 scale(float2 a, float c) { return __fmul2_rn(a, dup(c)); }
// s * a + b for a compile-time sign s = +1 or -1.
template <int Sg>
__device__ __forceinline__ float2 addsg(float2 b, float2 a) {
  if constexpr (Sg > 0) return add(b, a);
  else return sub(b, a);
}

// Sx x + Sy y + Sz z for compile-time signs in {-1, 0, 1}, starting from the first nonzero
// term, which must be +1 (true of every odd population, the first of its opposite pair):
// no add to a zero start, and the same value as that sum.
template <int Sx, int Sy, int Sz>
__device__ __forceinline__ float2 cdot(float2 x, float2 y, float2 z) {
  if constexpr (Sx != 0) {
    static_assert(Sx == 1, "the first term is positive");
    float2 r = x;
    if constexpr (Sy != 0) r = addsg<Sy>(r, y);
    if constexpr (Sz != 0) r = addsg<Sz>(r, z);
    return r;
  } else if constexpr (Sy != 0) {
    static_assert(Sy == 1, "the first term is positive");
    return Sz != 0 ? addsg<Sz>(y, z) : y;
  } else {
    static_assert(Sz == 1, "the first term is positive");
    return z;
  }
}
// An accumulator's next term: the term itself when it is the first (kFirst; then Sg = +1).
template <bool kFirst, int Sg>
__device__ __forceinline__ float2 acc(float2 a, float2 v) {
  if constexpr (kFirst) {
    static_assert(Sg == 1, "the first term is positive");
    return v;
  } else {
    return addsg<Sg>(a, v);
  }
}

// Asynchronous B-byte copy (B = 4 or 8) from global to shared memory: the value goes
// through no register, and cp_async_wait_all waits for this thread's copies.
template <int B>
__device__ __forceinline__ void cp_async(void* sdst, const void* gsrc) {
  static_assert(B == 4 || B == 8, "cp.async.ca copies 4, 8 or 16 bytes");
  const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(sdst));
  const size_t g = __cvta_generic_to_global(gsrc);
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(d), "l"(g), "n"(B)
               : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;\n" ::: "memory");
}

// Pair loads and stores of the storage formats. Deviation storage (16-bit) returns the
// stored f - W; the moments add the weights' moments.
template <class S>
struct PairIO;
template <>
struct PairIO<mcb::StF32> {
  using FT = float;
  // Raw loaded values: kept as loaded until the moments convert them, so that no
  // instruction waits on a load before the plane's barrier.
  using R2 = float2;
  using R1 = float;
  static __device__ __forceinline__ R2 raw2(const float* p) {
    return __ldg(reinterpret_cast<const float2*>(p));
  }
  static __device__ __forceinline__ R1 raw1(const float* p) { return __ldg(p); }
  static __device__ __forceinline__ float2 cvt2(R2 v) { return v; }
  static __device__ __forceinline__ float cvt1(R1 v) { return v; }
  static __device__ __forceinline__ R1 lo(R2 v) { return v.x; }
  static __device__ __forceinline__ R1 hi(R2 v) { return v.y; }
  static __device__ __forceinline__ float2 ld2(const float* p) {
    return __ldg(reinterpret_cast<const float2*>(p));
  }
  static __device__ __forceinline__ float ld1(const float* p) { return __ldg(p); }
  static __device__ __forceinline__ void st2(float* p, float2 v) {
    *reinterpret_cast<float2*>(p) = v;
  }
};
template <>
struct PairIO<mcb::StH16> {
  using FT = __half;
  using R2 = __half2;
  using R1 = __half;
  static __device__ __forceinline__ R2 raw2(const __half* p) {
    return __ldg(reinterpret_cast<const __half2*>(p));
  }
  static __device__ __forceinline__ R1 raw1(const __half* p) { return __ldg(p); }
  static __device__ __forceinline__ float2 cvt2(R2 v) { return __half22float2(v); }
  static __device__ __forceinline__ float cvt1(R1 v) { return __half2float(v); }
  static __device__ __forceinline__ R1 lo(R2 v) { return __low2half(v); }
  static __device__ __forceinline__ R1 hi(R2 v) { return __high2half(v); }
  static __device__ __forceinline__ float2 ld2(const __half* p) {
    return __half22float2(__ldg(reinterpret_cast<const __half2*>(p)));
  }
  static __device__ __forceinline__ float ld1(const __half* p) { return __half2float(__ldg(p)); }
  static __device__ __forceinline__ void st2(__half* p, float2 v) {
    *reinterpret_cast<__half2*>(p) = __float22half2_rn(v);
  }
};
template <>
struct PairIO<mcb::StB16> {
  using FT = __nv_bfloat16;
  using R2 = __nv_bfloat162;
  using R1 = __nv_bfloat16;
  static __device__ __forceinline__ R2 raw2(const __nv_bfloat16* p) {
    return __ldg(reinterpret_cast<const __nv_bfloat162*>(p));
  }
  static __device__ __forceinline__ R1 raw1(const __nv_bfloat16* p) { return __ldg(p); }
  static __device__ __forceinline__ float2 cvt2(R2 v) { return __bfloat1622float2(v); }
  static __device__ __forceinline__ float cvt1(R1 v) { return __bfloat162float(v); }
  static __device__ __forceinline__ R1 lo(R2 v) { return __low2bfloat16(v); }
  static __device__ __forceinline__ R1 hi(R2 v) { return __high2bfloat16(v); }
  static __device__ __forceinline__ float2 ld2(const __nv_bfloat16* p) {
    return __bfloat1622float2(__ldg(reinterpret_cast<const __nv_bfloat162*>(p)));
  }
  static __device__ __forceinline__ float ld1(const __nv_bfloat16* p) {
    return __bfloat162float(__ldg(p));
  }
  static __device__ __forceinline__ void st2(__nv_bfloat16* p, float2 v) {
    *reinterpret_cast<__nv_bfloat162*>(p) = __float22bfloat162_rn(v);
  }
};

// Stored g of a pair of cells: raw loads, and the store of both cells' encoded values.
template <class S>
struct GPairIO;
template <>
struct GPairIO<mcb::StF32> {
  using GT = int;  // Q2.30
  using R2 = int2;
  using R1 = int;
  static __device__ __forceinline__ R2 raw2(const int* p) {
    return __ldg(reinterpret_cast<const int2*>(p));
  }
  static __device__ __forceinline__ R1 raw1(const int* p) { return __ldg(p); }
  static __device__ __forceinline__ R1 lo(R2 v) { return v.x; }
  static __device__ __forceinline__ R1 hi(R2 v) { return v.y; }
  static __device__ __forceinline__ void st2(int* p, int a, int b) {
    *reinterpret_cast<int2*>(p) = make_int2(a, b);
  }
};
template <>
struct GPairIO<mcb::StH16> {
  using GT = __half;
  using R2 = __half2;
  using R1 = __half;
  static __device__ __forceinline__ R2 raw2(const __half* p) {
    return __ldg(reinterpret_cast<const __half2*>(p));
  }
  static __device__ __forceinline__ R1 raw1(const __half* p) { return __ldg(p); }
  static __device__ __forceinline__ R1 lo(R2 v) { return __low2half(v); }
  static __device__ __forceinline__ R1 hi(R2 v) { return __high2half(v); }
  static __device__ __forceinline__ void st2(__half* p, __half a, __half b) {
    *reinterpret_cast<__half2*>(p) = __halves2half2(a, b);
  }
};
template <>
struct GPairIO<mcb::StB16> {
  using GT = __nv_bfloat16;
  using R2 = __nv_bfloat162;
  using R1 = __nv_bfloat16;
  static __device__ __forceinline__ R2 raw2(const __nv_bfloat16* p) {
    return __ldg(reinterpret_cast<const __nv_bfloat162*>(p));
  }
  static __device__ __forceinline__ R1 raw1(const __nv_bfloat16* p) { return __ldg(p); }
  static __device__ __forceinline__ R1 lo(R2 v) { return __low2bfloat16(v); }
  static __device__ __forceinline__ R1 hi(R2 v) { return __high2bfloat16(v); }
  static __device__ __forceinline__ void st2(__nv_bfloat16* p, __nv_bfloat16 a,
                                             __nv_bfloat16 b) {
    *reinterpret_cast<__nv_bfloat162*>(p) = __halves2bfloat162(a, b);
  }
};

}  // namespace pk

namespace mcb {
namespace {

constexpr int kPairTX = 32;  // threads in x; a tile is 2 * kPairTX = 64 cells wide

// Ring slot of a non-negative plane index in the 5-plane phi ring (unsigned: no sign fix-up).
__device__ __forceinline__ unsigned slot5(int v) { return static_cast<unsigned>(v) % 5u; }

// Dynamic shared memory of the relaxed-g pair kernel: two planes of staged g (18
// populations x kPairBY rows x 34 words of two cells) and, for the 16-bit deviation form, a
// ring of four planes of staged previous phi (kPairBY + 2 rows x 34 words).
template <class S>
__host__ __device__ constexpr int pair_gbuf_bytes() {
  return 2 * (kQ - 1) * kPairBY * 2 * (kPairTX + 2) * static_cast<int>(sizeof(typename S::GT));
}
template <class S>
__host__ __device__ constexpr int pair_bgk_smem() {
  return pair_gbuf_bytes<S>() + (S::kDev ? 4 * (kPairBY + 2) * 2 * (kPairTX + 2) * 4 : 0);
}

// kRef: some case of the launch is in reference mode (frozen shell); the shell handling is
// compiled only into that instance, which also runs the other modes.
// kL2: prefetch into L2 the f rows of plane z + 2 while plane z collides.
// GM: how g crosses the update (kGEquil: pushed equilibrium populations, nothing stored;
// kGPop: stored at full relaxation; kGBgk: stored, pulled and relaxed with tau_g != 1). The
// stored forms run periodic and wall modes only (no reference shell) and need 18 * cells
// below 2^31 (checked on the host).
template <class S, int BY, bool kRef, bool kL2, int GM>
__device__ __forceinline__ void collide_pair_segment(const StepArgs& a, const Tile& t) {
  constexpr bool EQ = GM == kGEquil;
  constexpr bool BGK = GM == kGBgk;
  using GIO = pk::GPairIO<S>;
  using GT = typename GIO::GT;
  using FT = typename S::FT;
  using IO = pk::PairIO<S>;
  using pk::add;
  using pk::dup;
  using pk::fma;
  using pk::mul;
  using pk::scale;
  using pk::sub;
  constexpr int TX = kPairTX, BX = 2 * TX, NT = TX * BY;
  constexpr int PX = BX + 4, PY = BY + 4, PP = PX * PY;  // phi plane, halo 2
  constexpr int PH = PX / 2, PP2 = PP / 2;              // the same in pairs of values
  constexpr int KP2 = (PP2 + NT - 1) / NT;              // phi pairs per thread per plane
  constexpr int HX = BX + 2, HY = BY + 2, HP = HX * HY;  // normals plane, halo 1
  constexpr int KFL = (HP + NT - 1) / NT;                // ring positions per thread
  constexpr bool kDevF = S::kFDev;
  constexpr int QF = kQ;
  __shared__ __align__(16) float sphi[5][PP];
  __shared__ __align__(16) float snrm[4][4][HP];  // nx, ny, nz, |grad phi| of four planes
  __shared__ __align__(16) int sacc[4][HP];       // push ring: integer sums of the next phi

  const int nx = t.nx, ny = t.ny, nz = t.nz;
  const int nxy = nx * ny;
  const bool ref = kRef && t.bc == kBcRef;
  const bool walls = t.bc == kBcWallsZ;
  const int tx = threadIdx.x, ty = threadIdx.y, tid = tx + TX * ty;
  const int x0 = t.xt + 2 * tx, y = t.yt + ty;
  const bool active = x0 < nx && y < ny;  // nx is even: x0 + 1 < nx with x0

  const CaseDesc* cd = a.cases + t.ci;
  const float omega = __ldg(&cd->omega), omega_g = __ldg(&cd->omega_g);
  const float sigma = __ldg(&cd->sigma), sharp_c = __ldg(&cd->sharp_c);
  const float gravity = __ldg(&cd->gravity), phi_mean = __ldg(&cd->phi_mean);

  const int* __restrict__ pcur = a.p_cur + t.cell_off;
  int* __restrict__ pnext = a.p_next + t.cell_off;
  int* __restrict__ pzero = a.p_zero + t.cell_off;

  // Halo pairs of a phi plane handled by this thread (in-plane offsets, even: the pair is
  // one aligned 64-bit load). Periodic axes wrap; in reference mode x clamps to the lattice
  // (the values beyond the shell only feed normals that are zero there).
  int hoff[KP2];
#pragma unroll
  for (int k = 0; k < KP2; ++k) {
    const int i = tid + k * NT;
    hoff[k] = 0;
    if (i < PP2) {
      int gx = t.xt - 2 + 2 * (i % PH), gy = t.yt - 2 + i / PH;
      if (ref) {
        gx = clampi(gx, 0, nx - 2);
        gy = clampi(gy, 0, ny - 1);
      } else {
        gx = ((gx % nx) + nx) % nx;
        gy = ((gy % ny) + ny) % ny;
      }
      hoff[k] = gx + gy * nx;
    }
  }
  auto zmap = [&](int z) -> int {
    if (t.bc == kBcPeriodic) z = wrap1(z, nz);
    else if (walls) z = z < 0 ? -1 - z : (z >= nz ? 2 * nz - 1 - z : z);  // mirror
    return clampi(z, 0, nz - 1);
  };
  int2 pre[KP2];
  auto issue = [&](int zpl) {
    const int* base = pcur + static_cast<long long>(zmap(zpl)) * nxy;
#pragma unroll
    for (int k = 0; k < KP2; ++k)
      if ((k + 1) * NT <= PP2 || tid + k * NT < PP2)  // whole rounds need no test
        pre[k] = __ldg(reinterpret_cast<const int2*>(base + hoff[k]));
  };
  auto commit = [&](int zpl) {
    float2* d = reinterpret_cast<float2*>(sphi[slot5(zpl + 5)]);
#pragma unroll
    for (int k = 0; k < KP2; ++k)
      if ((k + 1) * NT <= PP2 || tid + k * NT < PP2)
        d[tid + k * NT] = scale(make_float2(__int2float_rn(pre[k].x), __int2float_rn(pre[k].y)),
                                kInvQ30);
  };

  // Push ring: the global in-plane offsets of this thread's ring positions (-1: none).
  int aoff[KFL];
#pragma unroll
  for (int k = 0; k < KFL; ++k) {
    const int i = tid + k * NT;
    aoff[k] = -1;
    if (i >= HP) continue;
    int gx = t.xt - 1 + i % HX, gy = t.yt - 1 + i / HX;
    if (ref) {
      if (gx <= 0 || gx >= nx - 1 || gy <= 0 || gy >= ny - 1) continue;
    } else {
      gx = ((gx % nx) + nx) % nx;
      gy = ((gy % ny) + ny) % ny;
    }
    aoff[k] = gx + gy * nx;
  }
  for (int i = tid; i < 4 * HP; i += NT) (&sacc[0][0])[i] = 0;
  auto flush = [&](int q) {
    int* slot = sacc[(q + 8) & 3];
    int qz = q;
    if (t.bc == kBcPeriodic) qz = wrap1(q, nz);
    const bool plane_ok = ref ? (qz > 0 && qz < nz - 1) : (qz >= 0 && qz < nz);
#pragma unroll
    for (int k = 0; k < KFL; ++k) {
      const int i = tid + k * NT;
      if ((k + 1) * NT > HP && i >= HP) continue;
      const int v = slot[i];
      slot[i] = 0;
      if (v != 0 && plane_ok && aoff[k] >= 0)
        atomicAdd(pnext + aoff[k] + static_cast<long long>(qz) * nxy, v);
    }
  };

  // Normals: this thread's point pairs of a normals plane, the same on every plane. Round k
  // takes pair j = tid + k NT, points 2j and 2j + 1 (hx even, so both lie in one row); ncen
  // is the phi-plane offset of the first point, and nzero flags (reference mode) the points
  // whose normal is zero: on the shell or beyond it.
  constexpr int NPR = HP / 2, KN = (NPR + NT - 1) / NT;  // point pairs, rounds
  int ncen[KN];
  int nzero[KN];
#pragma unroll
  for (int k = 0; k < KN; ++k) {
    const int i = 2 * (tid + k * NT);
    const int hx = i % HX, hy = i / HX;
    ncen[k] = (hy + 1) * PX + hx + 1;
    nzero[k] = 0;
    if (ref) {
      const int gx = t.xt - 1 + hx, gy = t.yt - 1 + hy;
      const bool yz = gy <= 0 || gy >= ny - 1;
      nzero[k] = ((yz || gx <= 0 || gx >= nx - 1) ? 1 : 0) |
                 ((yz || gx + 1 <= 0 || gx + 1 >= nx - 1) ? 2 : 0);
    }
  }
  // Normals and |grad phi| of plane zp on the halo-1 region (gradCalc, src/lbm.cu:34-72), two
  // points in x per thread in packed FP32, as k_collide computes them. The first point of a
  // pair sits at an odd phi-plane offset, so its x -+ 1 neighbours are aligned pairs.
  auto normals = [&](int zp) {
    const float* pm = sphi[slot5(zp + 4)];
    const float* p0 = sphi[slot5(zp + 5)];
    const float* pp = sphi[slot5(zp + 6)];
    float(*dst)[HP] = snrm[(zp + 4) & 3];
    const bool zshell = ref && (zp <= 0 || zp >= nz - 1);
#pragma unroll
    for (int k = 0; k < KN; ++k) {
      const int j = tid + k * NT;
      if ((k + 1) * NT > NPR && j >= NPR) break;  // whole rounds need no test
      const int c = ncen[k];
      float2 gx = dup(0.f), gy = gx, gz = gx;
      static_for<1, kQ>([&](auto LC) {
        constexpr int L = decltype(LC)::value;
        constexpr float w3 = 3.0f * wf(L);
        const float* q = nbr_of<cz(L)>(pm, p0, pp) + c + cy(L) * PX + cx(L);
        const float2 v =
            cx(L) != 0 ? *reinterpret_cast<const float2*>(q) : make_float2(q[0], q[1]);
        if constexpr (cx(L) != 0) gx = fma(dup(cx(L) * w3), v, gx);
        if constexpr (cy(L) != 0) gy = fma(dup(cy(L) * w3), v, gy);
        if constexpr (cz(L) != 0) gz = fma(dup(cz(L) * w3), v, gz);
      });
      const float2 g2 = fma(gz, gz, fma(gy, gy, mul(gx, gx)));
      float2 fac = make_float2(rsqrtf(fmaxf(g2.x, 1e-9f)), rsqrtf(fmaxf(g2.y, 1e-9f)));
      if (kRef && ref) {  // zero normals on the reference shell
        if (zshell || (nzero[k] & 1)) fac.x = 0.f;
        if (zshell || (nzero[k] & 2)) fac.y = 0.f;
      }
      reinterpret_cast<float2*>(dst[0])[j] = mul(gx, fac);
      reinterpret_cast<float2*>(dst[1])[j] = mul(gy, fac);
      reinterpret_cast<float2*>(dst[2])[j] = mul(gz, fac);
      reinterpret_cast<float2*>(dst[3])[j] = mul(g2, fac);
    }
  };

  // Blocked f layout: population l of cell (x, y, z) at z*PS + y*RS + fx(x) + 32 l, with
  // fx(x) = (x / 32) * 19 * 32 + x % 32. x0 is even, so x0 and x0 + 1 share a 32-cell block.
  const FT* __restrict__ fin = static_cast<const FT*>(a.f_in) + t.f_off;
  FT* __restrict__ fout = static_cast<FT*>(a.f_out) + t.f_off;
  const int RS = t.fxb * (QF * 32);
  const long long PS = static_cast<long long>(RS) * ny;
  auto fxof = [](int xs) -> int { return (xs >> 5) * (QF * 32) + (xs & 31); };
  const int xw = active ? x0 : 0;
  const int fx0 = fxof(xw);                                     // x0 (and x0 + 1 at +1)
  const int fxm = fxof(xw == 0 ? nx - 1 : xw - 1);              // x0 - 1
  const int fxp = fxof(xw + 2 >= nx ? xw + 2 - nx : xw + 2);    // x0 + 2
  const int yw = active ? y : 0;
  const int fy0 = yw * RS;
  const int fym = (yw == 0 ? ny - 1 : yw - 1) * RS;
  const int fyp = (yw == ny - 1 ? 0 : yw + 1) * RS;
  const int yo = yw * nx;

  // Byte offsets in a plane of the pull sources: rows y - 1, y, y + 1 (the sources of
  // cy = +1, 0, -1) by x terms x0 - 1, x0, x0 + 2. A plane holds under 2^32 bytes (checked
  // on the host).
  unsigned boff[3][3];
  {
    const int fys[3] = {fym, fy0, fyp}, fxs[3] = {fxm, fx0, fxp};
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = 0; c < 3; ++c)
        boff[r][c] = static_cast<unsigned>(fys[r] + fxs[c]) * static_cast<unsigned>(sizeof(FT));
  }

  // The gathered populations of both cells (values of x0 and x0 + 1), as loaded: a pair for
  // the populations that do not move in x (one aligned load), two values for the others.
  typename IO::R2 r2[QF] = {};
  typename IO::R1 r1a[QF] = {}, r1b[QF] = {};
  // Population L of both cells in FP32.
  auto fval = [&](auto LC) -> float2 {
    constexpr int L = decltype(LC)::value;
    if constexpr (cx(L) == 0) return IO::cvt2(r2[L]);
    else return make_float2(IO::cvt1(r1a[L]), IO::cvt1(r1b[L]));
  };
  // Stored g.
  const GT* __restrict__ gin = static_cast<const GT*>(a.g_in) + t.g_off;
  GT* __restrict__ gout = static_cast<GT*>(a.g_out) + t.g_off;
  const int* __restrict__ pprev = a.p_prev + t.cell_off;
  const int ng = static_cast<int>(t.ncell);
  // Relaxed g pulls the 18 stored populations of its sources; the 16-bit form decodes each
  // against its source's previous phi. Both are staged in shared memory with asynchronous
  // copies one plane ahead, so that no register holds them across the plane's barrier:
  //   - g of plane z: per population and tile row, the source row's words (2 cells each)
  //     from x = xt - 2 to xt + 64 (words 0 .. TX + 1), in two buffers (z & 1);
  //   - previous phi: rows yt - 1 .. yt + BY of a plane, the same x range, in a ring of
  //     four planes (q & 3): planes z - 1 .. z + 1 are read while z + 2 arrives.
  // Element 2 tx + 2 - cx of a staged row is the source x0 - cx of the pair's first cell.
  constexpr int GW = TX + 2, GR = 2 * GW;  // words and elements of a staged row
  constexpr int PR = BY + 2;               // staged previous-phi rows
  extern __shared__ __align__(16) unsigned char pair_dyn[];
  GT* const gbuf = reinterpret_cast<GT*>(pair_dyn);
  int* const pring = reinterpret_cast<int*>(pair_dyn + pair_gbuf_bytes<S>());
  // A staged coordinate one step or so past the lattice edge, wrapped (the reads that use
  // it); coordinates further out are never read and take 0.
  auto wrap_st = [](int v, int n) {
    return v < 0 ? v + n : (v < n ? v : (v - n < n ? v - n : 0));
  };
  constexpr int KPJ = (PR * GW + NT - 1) / NT;  // previous-phi words per thread and plane
  auto gplane = [&](int q) {  // the stored plane of plane index q (walls: clamped, unread)
    if (t.bc == kBcPeriodic) q = wrap1(q, nz);
    return clampi(q, 0, nz - 1) * nxy;
  };
  constexpr int kGW = 2 * static_cast<int>(sizeof(GT));  // bytes of a g word
  // Copies the g words of collision plane zq into buffer zq & 1.
  // Each thread copies, for its row y, the word at x0 of the rows y - 1, y, y + 1 (the
  // first thread past the lattice edge in x: the wrapped word at x = 0); thread 0 adds the
  // left halo word, thread TX - 1 the right one. Rows past the edge are never read.
  auto stage_g = [&](int zq) {
    const int zs[3] = {gplane(zq - 1), gplane(zq), gplane(zq + 1)};  // cz = 1, 0, -1
    const int yr = y < ny ? y : 0;
    const int rows[3] = {(yr == 0 ? ny - 1 : yr - 1) * nx, yr * nx,  // cy = 1, 0, -1
                         (yr == ny - 1 ? 0 : yr + 1) * nx};
    const int xo = x0 < nx ? x0 : 0;
    const int xh = wrap_st(tx == 0 ? t.xt - 2 : t.xt + 2 * TX, nx);
    GT* b = gbuf + (zq & 1) * ((kQ - 1) * BY * GR) + ty * GR;
    static_for<1, kQ>([&](auto LC) {
      constexpr int L = decltype(LC)::value;
      const GT* src = gin + (L - 1) * ng + zs[1 - cz(L)] + rows[1 - cy(L)];
      GT* dst = b + (L - 1) * (BY * GR);
      pk::cp_async<kGW>(dst + 2 + 2 * tx, src + xo);
      if constexpr (cx(L) == 1) {
        if (tx == 0) pk::cp_async<kGW>(dst, src + xh);
      } else if constexpr (cx(L) == -1) {
        if (tx == TX - 1) pk::cp_async<kGW>(dst + 2 * (TX + 1), src + xh);
      }
    });
  };
  // Copies the previous phi of plane q into ring slot q & 3.
  auto stage_p = [&](int q) {
    const int* src = pprev + gplane(q);
    int* dst = pring + (q & 3) * (PR * GR);
#pragma unroll
    for (int k = 0; k < KPJ; ++k) {
      const int j = tid + k * NT;
      if ((k + 1) * NT <= PR * GW || j < PR * GW)
        pk::cp_async<8>(dst + 2 * j, src + wrap_st(t.yt - 1 + j / GW, ny) * nx +
                                          wrap_st(t.xt - 2 + 2 * (j % GW), nx));
    }
  };

  // Gathers the 19 populations of both cells of plane z and their Q2.30 phi.
  auto gather = [&](int z, int2& pcv) {
    const bool blo = walls && z == 0, bhi = walls && z == nz - 1;
    pcv = __ldg(reinterpret_cast<const int2*>(pcur + x0 + yo + z * nxy));
    // Plane bases (the same for the whole block) plus this thread's byte offsets in the
    // plane, fixed for the segment; the population index is an immediate.
    const char* pz0 = reinterpret_cast<const char*>(fin + static_cast<long long>(z) * PS);
    const char* pzm =
        reinterpret_cast<const char*>(fin + static_cast<long long>(z == 0 ? nz - 1 : z - 1) * PS);
    const char* pzp =
        reinterpret_cast<const char*>(fin + static_cast<long long>(z == nz - 1 ? 0 : z + 1) * PS);
    auto at = [](const char* base, unsigned off, int elems) {
      return reinterpret_cast<const FT*>(base + off) + elems;
    };
    auto pull = [&](auto LC) {
      constexpr int L = decltype(LC)::value;
      const char* pl = src_of<cz(L)>(pzm, pz0, pzp);
      constexpr int yi = cy(L) == 1 ? 0 : (cy(L) == 0 ? 1 : 2);  // source row y - cy
      if constexpr (cx(L) == 0) {
        r2[L] = IO::raw2(at(pl, boff[yi][1], L * 32));
      } else if constexpr (cx(L) == 1) {  // sources x0 - 1 and x0
        r1a[L] = IO::raw1(at(pl, boff[yi][0], L * 32));
        r1b[L] = IO::raw1(at(pl, boff[yi][1], L * 32));
      } else {  // sources x0 + 1 and x0 + 2
        r1a[L] = IO::raw1(at(pl, boff[yi][1], L * 32 + 1));
        r1b[L] = IO::raw1(at(pl, boff[yi][2], L * 32));
      }
    };
    r2[0] = IO::raw2(at(pz0, boff[1][1], 0));
    if (blo || bhi) {
      // A wall plane: what left through the wall returns as the cell's own opposite
      // population.
      static_for<1, QF>([&](auto LC) {
        constexpr int L = decltype(LC)::value;
        const bool bounce = (cz(L) == 1) ? blo : ((cz(L) == -1) ? bhi : false);
        if (bounce) {
          const typename IO::R2 v = IO::raw2(at(pz0, boff[1][1], opp(L) * 32));
          if constexpr (cx(L) == 0) {
            r2[L] = v;
          } else {
            r1a[L] = IO::lo(v);
            r1b[L] = IO::hi(v);
          }
        } else {
          pull(LC);
        }
      });
    } else {
      static_for<1, QF>(pull);
    }
  };

  // Prologue: phi planes zb-2 .. zb+2, normals zb-1 .. zb+1.
  for (int zpl = t.zb - 2; zpl <= t.zb + 2; ++zpl) {
    issue(zpl);
    commit(zpl);
  }
  issue(t.zb + 3);
  int2 pc = make_int2(0, 0);
  __syncthreads();
  for (int zpl = t.zb - 1; zpl <= t.zb + 1; ++zpl) normals(zpl);
  if constexpr (BGK) {
    stage_g(t.zb);
    if constexpr (S::kDev)
      for (int q = t.zb - 1; q <= t.zb + 1; ++q) stage_p(q);
  }
  __syncthreads();

  for (int z = t.zb; z < t.ze; ++z) {
    commit(z + 3);
    if (z + 4 <= t.ze + 1) issue(z + 4);

    const int idx = x0 + yo + z * nxy;
    const bool zshell = ref && (z == 0 || z == nz - 1);
    const bool blo = walls && z == 0, bhi = walls && z == nz - 1;
    // The gathered values stay as loaded until the moments use them, after the barrier and
    // the normals: no instruction waits on these loads before then.
    if (active) gather(z, pc);
    if constexpr (BGK) pk::cp_async_wait_all();  // this plane's staged g and previous phi
    __syncthreads();
    if constexpr (BGK) {
      // The next plane's: its buffers were last read by plane z - 1, which every thread
      // has finished.
      if (z + 1 < t.ze) {
        stage_g(z + 1);
        if constexpr (S::kDev) stage_p(z + 2);
      }
    }
    if (z - 2 >= t.zb - 1) flush(z - 2);  // complete: sources z-3 .. z-1 are in
    if (z + 2 <= t.ze) normals(z + 2);
    if constexpr (kL2) {
      // Plane z + 2 (the source plane of the next update's cz = -1 populations): rows
      // yt - 1 .. yt + BY of the tile's two 32-cell blocks, each a contiguous run of
      // 19 x 32 values, in 128-byte lines spread over the block's threads.
      if (z + 2 < t.ze + 1) {
        const int zq = t.bc == kBcPeriodic ? wrap1(z + 2, nz) : min(z + 2, nz - 1);
        constexpr int kRunBytes = QF * 32 * static_cast<int>(sizeof(FT));
        constexpr int kLines = (kRunBytes + 127) / 128;
        constexpr int kJobs = (BY + 2) * 2 * kLines;
        const char* pl = reinterpret_cast<const char*>(fin + static_cast<long long>(zq) * PS);
        const int xb0 = t.xt >> 5;
        for (int j = tid; j < kJobs; j += NT) {
          const int line = j % kLines, rb = j / kLines;
          const int row = rb >> 1, xb = xb0 + (rb & 1);
          int yq = t.yt - 1 + row;
          yq = yq < 0 ? yq + ny : (yq >= ny ? yq - ny : yq);
          if (xb < t.fxb && yq >= 0 && yq < ny)
            l2_prefetch(pl + (static_cast<long long>(yq) * RS + xb * (QF * 32)) * sizeof(FT) +
                        line * 128);
        }
      }
    }
    if (!active) continue;

    *reinterpret_cast<int2*>(pzero + idx) = make_int2(0, 0);  // next update accumulates here
    // Reference-mode shell cells of this pair (never collide; rest-equilibrium inflow).
    const bool sh0 = ref && (zshell || x0 == 0 || y == 0 || y == ny - 1);
    const bool sh1 = ref && (zshell || x0 + 1 == nx - 1 || y == 0 || y == ny - 1);

    // Curvature (curvatureCalc, src/lbm.cu:80-125): kappa = -3 sum_l W_l c_l.n(x + c_l). The
    // pair sits at normals offsets h0 (odd) and h0 + 1, so its x-1 and x+1 neighbours are
    // aligned pairs; the x+0 neighbours are read as two values.
    const float(*nm)[HP] = snrm[(z + 3) & 3];
    const float(*n0)[HP] = snrm[(z + 4) & 3];
    const float(*np)[HP] = snrm[(z + 5) & 3];
    const int h0 = (ty + 1) * HX + 2 * tx + 1;
    auto nrm2 = [&](const float(*pl)[HP], int comp, int o) -> float2 {
      const float* q = &pl[comp][h0 + o];
      return (o & 1) ? *reinterpret_cast<const float2*>(q) : make_float2(q[0], q[1]);
    };
    const float2 ncx = nrm2(n0, 0, 0), ncy = nrm2(n0, 1, 0), ncz = nrm2(n0, 2, 0);
    const float2 ncw = nrm2(n0, 3, 0);
    // Per opposite pair (l, l + 1): W_l c_l . (n(x + c_l) - n(x - c_l)).
    float2 kap = dup(0.f);
    static_for<0, (kQ - 1) / 2>([&](auto KC) {
      constexpr int L = 2 * decltype(KC)::value + 1;
      constexpr float w3 = 3.0f * wf(L);
      const float(*pp)[HP] = nbr_of<cz(L)>(nm, n0, np);   // x + c_l
      const float(*pq)[HP] = nbr_of<-cz(L)>(nm, n0, np);  // x - c_l
      constexpr int o = cy(L) * HX + cx(L);
      const float2 cp = pk::cdot<cx(L), cy(L), cz(L)>(
          cx(L) ? nrm2(pp, 0, o) : dup(0.f), cy(L) ? nrm2(pp, 1, o) : dup(0.f),
          cz(L) ? nrm2(pp, 2, o) : dup(0.f));
      const float2 cm = pk::cdot<cx(L), cy(L), cz(L)>(
          cx(L) ? nrm2(pq, 0, -o) : dup(0.f), cy(L) ? nrm2(pq, 1, -o) : dup(0.f),
          cz(L) ? nrm2(pq, 2, -o) : dup(0.f));
      if constexpr (L == 1) kap = mul(dup(-w3), sub(cp, cm));
      else kap = fma(dup(-w3), sub(cp, cm), kap);
    });
    const float2 phi = *reinterpret_cast<const float2*>(&sphi[slot5(z + 5)][(ty + 2) * PX + 2 * tx + 2]);
    const float2 mult = scale(kap, sigma);
    const float2 mw = mul(mult, ncw);
    float2 Fx = mul(mw, ncx), Fy = mul(mw, ncy), Fz = mul(mw, ncz);
    if (gravity != 0.f) Fz = fma(dup(gravity), sub(phi, dup(phi_mean)), Fz);

    // Moments (momentiCalc, src/lbm.cu:133-225), from opposite-pair sums; deviation storage
    // starts from the weights' moments.
    constexpr float m0 = kDevF ? 1.0f : 0.0f, m2 = kDevF ? 1.0f / 3.0f : 0.0f;
    // Accumulators start from their first term (the first odd population with the component:
    // x 1, y 3, z 5, xy 7, xz 9, yz 11, each with sign +1), not from an add to zero.
    float2 rho = fval(std::integral_constant<int, 0>{});
    if constexpr (kDevF) rho = add(dup(m0), rho);
    float2 jx = dup(0.f), jy = jx, jz = jx;
    float2 sxx = dup(m2), syy = sxx, szz = sxx, sxy = dup(0.f), sxz = sxy, syz = sxy;
    static_for<0, (QF - 1) / 2>([&](auto KC) {
      constexpr int L = 2 * decltype(KC)::value + 1;
      const float2 fa = fval(std::integral_constant<int, L>{});
      const float2 fb = fval(std::integral_constant<int, L + 1>{});
      const float2 sp = add(fa, fb), dm = sub(fa, fb);
      rho = add(rho, sp);
      if constexpr (cx(L) != 0) {
        jx = pk::acc<L == 1, cx(L)>(jx, dm);
        sxx = pk::acc<!kDevF && L == 1, 1>(sxx, sp);
      }
      if constexpr (cy(L) != 0) {
        jy = pk::acc<L == 3, cy(L)>(jy, dm);
        syy = pk::acc<!kDevF && L == 3, 1>(syy, sp);
      }
      if constexpr (cz(L) != 0) {
        jz = pk::acc<L == 5, cz(L)>(jz, dm);
        szz = pk::acc<!kDevF && L == 5, 1>(szz, sp);
      }
      if constexpr (cx(L) * cy(L) != 0) sxy = pk::acc<L == 7, cx(L) * cy(L)>(sxy, sp);
      if constexpr (cx(L) * cz(L) != 0) sxz = pk::acc<L == 9, cx(L) * cz(L)>(sxz, sp);
      if constexpr (cy(L) * cz(L) != 0) syz = pk::acc<L == 11, cy(L) * cz(L)>(syz, sp);
    });
    const float2 inv_rho = make_float2(__frcp_rn(rho.x), __frcp_rn(rho.y));
    const float2 ux = mul(fma(dup(0.5f), Fx, jx), inv_rho);
    const float2 uy = mul(fma(dup(0.5f), Fy, jy), inv_rho);
    const float2 uz = mul(fma(dup(0.5f), Fz, jz), inv_rho);
    const float2 uF = fma(uz, Fz, fma(uy, Fy, mul(ux, Fx)));
    const float2 nh = scale(uF, -1.5f);  // -h
    const float2 nrho = scale(rho, -1.0f);
    const float2 uxx = mul(ux, ux), uyy = mul(uy, uy), uzz = mul(uz, uz);
    const float2 uxy = mul(ux, uy), uxz = mul(ux, uz), uyz = mul(uy, uz);
    // p_ab = s_ab - rho (d_ab / 3 + u_a u_b) + (u_a F_b + u_b F_a) / 2 - h u_a u_b
    const float2 pxx = fma(nh, uxx, fma(ux, Fx, fma(nrho, add(dup(1.0f / 3.0f), uxx), sxx)));
    const float2 pyy = fma(nh, uyy, fma(uy, Fy, fma(nrho, add(dup(1.0f / 3.0f), uyy), syy)));
    const float2 pzz = fma(nh, uzz, fma(uz, Fz, fma(nrho, add(dup(1.0f / 3.0f), uzz), szz)));
    const float2 pxy = fma(nh, uxy, fma(dup(0.5f), fma(ux, Fy, mul(uy, Fx)), fma(nrho, uxy, sxy)));
    const float2 pxz = fma(nh, uxz, fma(dup(0.5f), fma(ux, Fz, mul(uz, Fx)), fma(nrho, uxz, sxz)));
    const float2 pyz = fma(nh, uyz, fma(dup(0.5f), fma(uy, Fz, mul(uz, Fy)), fma(nrho, uyz, syz)));
    const float2 u2 = add(add(uxx, uyy), uzz);
    const float2 tr3 = scale(add(add(pxx, pyy), pzz), 1.0f / 3.0f);

    // Regularized collision with He forcing (collisionFluid, src/lbm.cu:233-288):
    //   f*_l = W_l [E_l (rho + 3/2 (c_l.F - u.F)) + 9/2 (1 - omega) Q_l:Pi]
    // per opposite pair, with E_l = 1 + 3 c.u + 9/2 (c.u)^2 - 3/2 u^2.
    // g: A and 3 phi for the equilibrium W_l (phi + 3 phi c.u + A c.n)
    const float2 A = mul(scale(phi, sharp_c), fma(dup(-1.0f), phi, dup(1.0f)));
    const float2 phi3 = scale(phi, 3.0f);
    // Ring offsets of the pair's own row in the three target planes of the push.
    int* s0 = &sacc[(z + 8) & 3][h0];
    int* sm = &sacc[(z + 7) & 3][h0];
    int* sp = &sacc[(z + 9) & 3][h0];
    // Stored g: each population is encoded, stored and pushed as the collision makes it
    // (collisionPhase, src/lbm.cu:290-329; BGK with omega_g when tau_g != 1). The 16-bit
    // form stores it relative to the split of this cell's phi.
    const GSplit gsp0 = S::g_split(pc.x), gsp1 = S::g_split(pc.y);
    int sumq0 = 0, sumq1 = 0;
    auto emit = [&](auto LC, float2 g) {
      constexpr int L = decltype(LC)::value;
      int qa, qb;
      const GT ha = S::template g_put<L>(g.x, gsp0, qa);
      const GT hb = S::template g_put<L>(g.y, gsp1, qb);
      GIO::st2(gout + (L - 1) * ng + idx, ha, hb);
      sumq0 += qa;
      sumq1 += qb;
      constexpr int D = cy(L) * HX + cx(L);
      const bool bounce = cz(L) < 0 ? blo : (cz(L) > 0 ? bhi : false);
      int* tgt = bounce ? s0 : (cz(L) < 0 ? sm : (cz(L) > 0 ? sp : s0)) + D;
      atomicAdd(tgt, qa);
      atomicAdd(tgt + 1, qb);
    };
    // The decoded incoming population L of both cells (relaxed g): staged, or across a z
    // wall the cell's own opposite population.
    auto gdec = [&](auto LC) -> float2 {
      constexpr int L = decltype(LC)::value;
      constexpr int O = opp(L);
      const bool bounce = (cz(L) == 1) ? blo : ((cz(L) == -1) ? bhi : false);
      int ia, ib;
      if (bounce) {
        const typename GIO::R2 v = GIO::raw2(gin + (O - 1) * ng + idx);
        int2 ps = make_int2(0, 0);
        if constexpr (S::kDev) ps = __ldg(reinterpret_cast<const int2*>(pprev + idx));
        ia = S::template g_dec<O>(GIO::lo(v), ps.x);
        ib = S::template g_dec<O>(GIO::hi(v), ps.y);
      } else {
        constexpr int e = 2 - cx(L);  // the first cell's source, less 2 tx
        const GT* gr = gbuf + ((z & 1) * (kQ - 1) + (L - 1)) * (BY * GR) + ty * GR + 2 * tx + e;
        GT va, vb;
        if constexpr (cx(L) == 0) {
          const typename GIO::R2 w = *reinterpret_cast<const typename GIO::R2*>(gr);
          va = GIO::lo(w);
          vb = GIO::hi(w);
        } else {
          va = gr[0];
          vb = gr[1];
        }
        int pa = 0, pb = 0;
        if constexpr (S::kDev) {
          const int* pr = pring + ((z - cz(L)) & 3) * (PR * GR) + (ty + 1 - cy(L)) * GR + 2 * tx + e;
          if constexpr (cx(L) == 0) {
            const int2 w = *reinterpret_cast<const int2*>(pr);
            pa = w.x;
            pb = w.y;
          } else {
            pa = pr[0];
            pb = pr[1];
          }
        }
        ia = S::template g_dec<L>(va, pa);
        ib = S::template g_dec<L>(vb, pb);
      }
      return scale(make_float2(__int2float_rn(ia), __int2float_rn(ib)), kInvQ30);
    };
    const float2 om = dup((1.0f - omega) * 4.5f);
    constexpr float fshift = kDevF ? -1.0f : 0.0f;
    const float2 R = add(rho, nh);
    const float2 base = fma(dup(-1.5f), u2, dup(1.0f));
    FT* __restrict__ fo_base = fout + static_cast<long long>(z) * PS + fy0 + fx0;
    // The shell lanes keep the value the init wrote: f = W (0 in deviation form).
    auto put = [&](int L, float2 v) {
      if (kRef && (sh0 || sh1)) {
        const float wv = kDevF ? 0.0f : wf(L);
        if (sh0) v.x = wv;
        if (sh1) v.y = wv;
      }
      IO::st2(fo_base + L * 32, v);
    };
    {
      const float2 v = scale(fma(base, R, fma(scale(om, -1.0f), tr3, dup(fshift))), wf(0));
      put(0, v);
    }
    static_for<0, (QF - 1) / 2>([&](auto KC) {
      constexpr int L = 2 * decltype(KC)::value + 1;
      constexpr int O = L + 1;
      constexpr float W = wf(L);
      const float2 cu = pk::cdot<cx(L), cy(L), cz(L)>(ux, uy, uz);
      const float2 cF = pk::cdot<cx(L), cy(L), cz(L)>(Fx, Fy, Fz);
      float2 qp = scale(tr3, -1.0f);
      if constexpr (cx(L) != 0) qp = add(qp, pxx);
      if constexpr (cy(L) != 0) qp = add(qp, pyy);
      if constexpr (cz(L) != 0) qp = add(qp, pzz);
      if constexpr (cx(L) * cy(L) != 0) qp = fma(dup(2.0f * cx(L) * cy(L)), pxy, qp);
      if constexpr (cx(L) * cz(L) != 0) qp = fma(dup(2.0f * cx(L) * cz(L)), pxz, qp);
      if constexpr (cy(L) * cz(L) != 0) qp = fma(dup(2.0f * cy(L) * cz(L)), pyz, qp);
      const float2 q = fma(om, qp, dup(fshift));
      const float2 e0 = fma(scale(cu, 4.5f), cu, base), e1 = scale(cu, 3.0f);
      const float2 rf = scale(cF, 1.5f);
      put(L, scale(fma(add(e0, e1), add(R, rf), q), W));
      put(O, scale(fma(sub(e0, e1), sub(R, rf), q), W));
    });
    if constexpr (!EQ) {
      // Stored g, after the f collision (fewer values live at once): W_l (phi +- dg),
      // dg = 3 phi c.u + A c.n, relaxed against the pulled populations (tau_g != 1).
      static_for<0, (kQ - 1) / 2>([&](auto KC) {
        constexpr int L = 2 * decltype(KC)::value + 1;
        constexpr int O = L + 1;
        constexpr float WG = wf(L);
        const float2 cu = pk::cdot<cx(L), cy(L), cz(L)>(ux, uy, uz);
        const float2 cn = pk::cdot<cx(L), cy(L), cz(L)>(ncx, ncy, ncz);
        const float2 dg = fma(phi3, cu, mul(A, cn));
        float2 gL = scale(add(phi, dg), WG), gO = scale(sub(phi, dg), WG);
        if constexpr (BGK) {
          const float2 fL = gdec(std::integral_constant<int, L>{});
          const float2 fO = gdec(std::integral_constant<int, O>{});
          gL = fma(dup(omega_g), sub(gL, fL), fL);
          gO = fma(dup(omega_g), sub(gO, fO), fO);
        }
        emit(std::integral_constant<int, L>{}, gL);
        emit(std::integral_constant<int, O>{}, gO);
      });
      // the rest population: the exact remainder of each cell's phi
      atomicAdd(s0, pc.x - sumq0);
      atomicAdd(s0 + 1, pc.y - sumq1);
    }

    if constexpr (EQ) {
      // g (collisionPhase, src/lbm.cu:290-329), full relaxation: the populations are the
      // equilibrium W_l (phi + c_l.J), J = 3 phi u + sharp_c phi (1 - phi) n, pushed as exact
      // Q2.30 integers into the next phi (streamingCalc + phiCalc).
      constexpr float kj = 1073741824.0f / 36.0f;
      const float2 Jx = scale(fma(phi3, ux, mul(A, ncx)), kj);
      const float2 Jy = scale(fma(phi3, uy, mul(A, ncy)), kj);
      const float2 Jz = scale(fma(phi3, uz, mul(A, ncz)), kj);
      // shell lanes push their phi with no flux
      JQ j0{__float2int_rn(Jx.x), __float2int_rn(Jy.x), __float2int_rn(Jz.x)};
      JQ j1{__float2int_rn(Jx.y), __float2int_rn(Jy.y), __float2int_rn(Jz.y)};
      if (kRef) {
        if (sh0) j0 = JQ{0, 0, 0};
        if (sh1) j1 = JQ{0, 0, 0};
      }
      {
        const int wf0 = wsplit_face(pc.x), we0 = wsplit_edge_of_face(wf0);
        const int wf1 = wsplit_face(pc.y), we1 = wsplit_edge_of_face(wf1);
        auto q0 = [&](auto LC) -> int {
          constexpr int L = decltype(LC)::value;
          if constexpr (L == 0) return pc.x - 6 * wf0 - 12 * we0;
          else return (L <= 6 ? wf0 : we0) + qj<L>(j0);
        };
        auto q1 = [&](auto LC) -> int {
          constexpr int L = decltype(LC)::value;
          if constexpr (L == 0) return pc.y - 6 * wf1 - 12 * we1;
          else return (L <= 6 ? wf1 : we1) + qj<L>(j1);
        };
        if (walls && (blo || bhi)) {
          // A wall plane: what leaves through the wall returns to the cell itself.
          static_for<0, kQ>([&](auto LC) {
            constexpr int L = decltype(LC)::value;
            constexpr int D = cy(L) * HX + cx(L);
            const bool bounce = cz(L) < 0 ? blo : (cz(L) > 0 ? bhi : false);
            int* tgt = cz(L) < 0 ? sm : (cz(L) > 0 ? sp : s0);
            atomicAdd(bounce ? s0 : tgt + D, q0(LC));
            atomicAdd(bounce ? s0 + 1 : tgt + D + 1, q1(LC));
          });
        } else {
          // Targets of the pair in one (cy, cz) row: cell x0 reaches h0 - 1 .. h0 + 1, cell
          // x0 + 1 reaches h0 .. h0 + 2. The two middle targets take one atomic each for
          // both cells.
          auto row = [&](int* b, auto LM, auto L0, auto LP) {
            constexpr int Z = decltype(L0)::value;
            // LM: cx = -1, L0: cx = 0, LP: cx = +1 (each of the same cy, cz)
            atomicAdd(b - 1, q0(LM));
            atomicAdd(b, q0(std::integral_constant<int, Z>{}) + q1(LM));
            atomicAdd(b + 1, q0(LP) + q1(std::integral_constant<int, Z>{}));
            atomicAdd(b + 2, q1(LP));
          };
          // rest, +x, -x in the cell's own row and plane
          row(s0, std::integral_constant<int, 2>{}, std::integral_constant<int, 0>{},
              std::integral_constant<int, 1>{});
          // rows y+1 and y-1 in the plane: (-1,+1,0) 14, (0,+1,0) 3, (+1,+1,0) 7;
          // (-1,-1,0) 8, (0,-1,0) 4, (+1,-1,0) 13
          row(s0 + HX, std::integral_constant<int, 14>{}, std::integral_constant<int, 3>{},
              std::integral_constant<int, 7>{});
          row(s0 - HX, std::integral_constant<int, 8>{}, std::integral_constant<int, 4>{},
              std::integral_constant<int, 13>{});
          // planes z+1 and z-1: (-1,0,+1) 16, (0,0,+1) 5, (+1,0,+1) 9;
          // (-1,0,-1) 10, (0,0,-1) 6, (+1,0,-1) 15
          row(sp, std::integral_constant<int, 16>{}, std::integral_constant<int, 5>{},
              std::integral_constant<int, 9>{});
          row(sm, std::integral_constant<int, 10>{}, std::integral_constant<int, 6>{},
              std::integral_constant<int, 15>{});
          // the four (0, +-1, +-1) edges: one target per cell
          static_for<0, 4>([&](auto KC) {
            constexpr int K = decltype(KC)::value;
            constexpr int L = K == 0 ? 11 : (K == 1 ? 12 : (K == 2 ? 17 : 18));
            constexpr int D = cy(L) * HX;
            int* b = (cz(L) > 0 ? sp : sm) + D;
            atomicAdd(b, q0(std::integral_constant<int, L>{}));
            atomicAdd(b + 1, q1(std::integral_constant<int, L>{}));
          });
        }
      }
    }
    if (kRef && (sh0 || sh1)) {
      // The shell's own next phi is the lagged copy of its nearest interior cell
      // (boundaryConditions, src/lbm.cu:403-425).
      const int zc = clampi(z, 1, nz - 2) * nxy, yc = clampi(y, 1, ny - 2) * nx;
      if (sh0) pnext[idx] = __ldg(pcur + clampi(x0, 1, nx - 2) + yc + zc);
      if (sh1) pnext[idx + 1] = __ldg(pcur + clampi(x0 + 1, 1, nx - 2) + yc + zc);
    }

    if (a.macros) {
      const long long T = a.cells_total, o = t.cell_off + idx;
      float2 mphi = phi, mrho = rho, mx = ux, my = uy, mz = uz;
      if (kRef && sh0) { mphi.x = __int2float_rn(pc.x) * kInvQ30; mrho.x = 1.f; mx.x = my.x = mz.x = 0.f; }
      if (kRef && sh1) { mphi.y = __int2float_rn(pc.y) * kInvQ30; mrho.y = 1.f; mx.y = my.y = mz.y = 0.f; }
      *reinterpret_cast<float2*>(a.macros + o) = mphi;
      *reinterpret_cast<float2*>(a.macros + T + o) = mrho;
      *reinterpret_cast<float2*>(a.macros + 2 * T + o) = mx;
      *reinterpret_cast<float2*>(a.macros + 3 * T + o) = my;
      *reinterpret_cast<float2*>(a.macros + 4 * T + o) = mz;
    }
  }
  // The last target planes of the run.
  __syncthreads();
  for (int q = max(t.ze - 2, t.zb - 1); q <= t.ze; ++q) flush(q);
}

template <class S, int BY, bool kRef, int kMinBlocks, bool kL2, int GM>
__global__ void __launch_bounds__(kPairTX * BY, kMinBlocks)
    k_collide_pair(const StepArgs a) {
  for_each_segment<2 * kPairTX, BY, true>(
      a, [&](const Tile& t) { collide_pair_segment<S, BY, kRef, kL2, GM>(a, t); },
      a.balanced != 0);
}

// The pair kernel of a tile variant, with or without the reference-mode shell handling.
// Variant 5: three blocks of four warps per SM (168 registers: no spills, and more
// independent work per warp; two blocks per SM measured 12 % slower at FP16 storage and 26 %
// at FP32, four blocks at 128 registers 6 % and 18 %). Variant 6: the same with an L2
// prefetch of the f rows of the plane after next.
template <class S, int GM>
const void* pair_kernel_gm(int variant, bool with_ref) {
  if constexpr (GM != kGEquil) {
    // stored g: periodic and wall modes only (the host sees to it)
    // relaxed FP32 g: its staged planes leave room for two blocks per SM
    constexpr int MB = (GM == kGBgk && !S::kDev) ? 2 : 3;
    return variant == kPairVariant
               ? reinterpret_cast<const void*>(k_collide_pair<S, kPairBY, false, MB, false, GM>)
               : reinterpret_cast<const void*>(k_collide_pair<S, kPairBY, false, MB, true, GM>);
  } else if (variant == kPairVariant) {
    return with_ref ? reinterpret_cast<const void*>(k_collide_pair<S, kPairBY, true, 3, false, GM>)
                    : reinterpret_cast<const void*>(k_collide_pair<S, kPairBY, false, 3, false, GM>);
  } else {
    return with_ref ? reinterpret_cast<const void*>(k_collide_pair<S, kPairBY, true, 3, true, GM>)
                    : reinterpret_cast<const void*>(k_collide_pair<S, kPairBY, false, 3, true, GM>);
  }
}

// Dynamic shared memory of a pair-kernel launch.
template <class S>
int pair_dyn_smem(int gmode) {
  return gmode == kGBgk ? pair_bgk_smem<S>() : 0;
}

template <class S>
const void* pair_kernel(int variant, bool with_ref, int gmode) {
  switch (gmode) {
    case kGEquil: return pair_kernel_gm<S, kGEquil>(variant, with_ref);
    case kGBgk: return pair_kernel_gm<S, kGBgk>(variant, with_ref);
    case kGPop: return pair_kernel_gm<S, kGPop>(variant, with_ref);
    default: return nullptr;
  }
}

}  // namespace
}  // namespace mcb
