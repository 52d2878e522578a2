// TEST INFRASTRUCTURE ONLY: CPU oracle for the phase-field LBM update.
//
// This is a restatement, kernel by kernel, of the reference's update (kreeyto/MULTIC-BUBBLE-CUDA):
//   src/lbm.cu:5-461, src/init.cu:51-80, constants src/var.cu:21-53, order src/main.cu:74-190.
// It keeps the reference's data flow:
//   - full-grid arrays for phi, the normals, the indicator, the curvature, the force, u,
//     rho and Pi;
//   - in-place push streaming for f;
//   - a separate pull streaming pass for g.
// It is templated on the arithmetic type:
//   - double: the accuracy oracle;
//   - float: follows the reference's float expressions term by term.
// Only the tests, the smoke check and the CPU baseline of the benchmark use it. The product
// (the CUDA library) never calls it.
//
// Boundary modes:
//   0 "ref": the reference's frozen one-cell shell:
//       - rest-equilibrium inflow from the shell (fgBoundary, src/lbm.cu:365-401);
//       - zero-gradient shell phi lagged by one update (boundaryConditions,
//         src/lbm.cu:403-425), applied as three sequential face copies;
//       - the dead shell writes of movingWallBC (src/lbm.cu:430-461) when asked.
//   1 periodic in x, y, z.
//   2 periodic in x, y with half-way bounce-back walls in z. phi is mirrored across the
//     walls for the stencils.
// Modes 1 and 2, BGK g relaxation with tau_g != 1 and the Boussinesq force have no
// reference counterpart. They restate the same update with those additions.
//
// f on D3Q27 (qf = 27) uses the tables of src/var.cu:33-35,47-52. The reference's D3Q27
// moments are unfinished (src/lbm.cu:174-218 keep D3Q19 index sums), so for it the moments
// are taken from their definitions: rho = sum f, rho u = sum c f + F/2, and
// Pi = sum c c (f - feq + F_l/2). g and the phi stencils stay on D3Q19.
//
// Density ratio (rho_in != rho_out; periodic and wall modes): f carries the normalised
// pressure p* = p / (rho cs^2) of the velocity-based formulation (Zu and He 2013; Fakhari,
// Mitchell, Leonardi and Bolster 2017), with rho = rho_out + (rho_in - rho_out) phi:
//   p* = sum f, u* = sum c f, Pi* = sum c c f - p* cs^2 I - u* u*,
//   F = F_s + F_b - p* cs^2 grad rho - (1 - omega/2) Pi* . grad rho,
//   u = u* + F / (2 rho),
//   f*_l = W_l [p* + 3 c.u + 9/2 (c.u)^2 - 3/2 u^2] + (1 - omega) W_l 9/2 Q_l : Pi
//          + (1 - omega/2) 3 W_l c.F / rho,   Pi = sum c c f - p* cs^2 I - u u,
// with grad rho = (rho_in - rho_out) grad phi from the isotropic stencil. The start is
// p* = 0 at the given u. The rho field reports p / cs^2 = p* rho.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// D3Q19 in the reference's order (src/var.cu:29-31).
const int CIX[19] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0};
const int CIY[19] = {0, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 1, -1};
const int CIZ[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, -1, 1, -1, 1};
int OPP(int l) { return l == 0 ? 0 : ((l & 1) ? l + 1 : l - 1); }
// f lattice: D3Q19 followed by the eight D3Q27 corners (src/var.cu:33-35).
const int FCX[27] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0,
                     1, -1, 1, -1, 1, -1, -1, 1};
const int FCY[27] = {0, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 1, -1,
                     1, -1, 1, -1, -1, 1, 1, -1};
const int FCZ[27] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, -1, 1, -1, 1,
                     1, -1, -1, 1, 1, -1, 1, -1};

struct Params {
  int nx, ny, nz, bc;
  double tau, tau_g, sigma, sharp_c, gravity;
  int threads;
  int moving_wall;  // ref mode: also run movingWallBC's shell writes
  int qf;           // velocity set of f: 19 or 27
  double rho_in, rho_out;  // densities of phi = 1 and phi = 0 (equal: the reference model)
};

template <class T>
struct Oracle {
  Params p;
  long long n;
  T W[19];
  T FW[27];  // f weights (D3Q19 or D3Q27)
  int QF;
  T CSSQ, OMEGA, OMEGA_G, SHARP_C, SIGMA;
  std::vector<T> f, g, g_out, phi, nx_, ny_, nz_, ind, curv, ffx, ffy, ffz;
  std::vector<T> ux, uy, uz, rho, pxx, pyy, pzz, pxy, pxz, pyz, pst;
  T phi_mean = 0;
  long long update = -1;

  explicit Oracle(const Params& q) : p(q) {
    n = static_cast<long long>(p.nx) * p.ny * p.nz;
    W[0] = T(1) / T(3);
    for (int l = 1; l <= 6; ++l) W[l] = T(1) / T(18);
    for (int l = 7; l < 19; ++l) W[l] = T(1) / T(36);
    QF = p.qf == 27 ? 27 : 19;
    if (QF == 19) {
      for (int l = 0; l < 19; ++l) FW[l] = W[l];
    } else {
      FW[0] = T(8) / T(27);
      for (int l = 1; l <= 6; ++l) FW[l] = T(2) / T(27);
      for (int l = 7; l < 19; ++l) FW[l] = T(1) / T(54);
      for (int l = 19; l < 27; ++l) FW[l] = T(1) / T(216);
    }
    CSSQ = T(1) / T(3);
    OMEGA = T(1) / T(p.tau);
    OMEGA_G = T(1) / T(p.tau_g);
    SHARP_C = T(p.sharp_c);
    SIGMA = T(p.sigma);
    const size_t N = static_cast<size_t>(n);
    f.assign(static_cast<size_t>(QF) * N, 0);
    g.assign(19 * N, 0);
    g_out.assign(19 * N, 0);
    for (auto* v : {&phi, &nx_, &ny_, &nz_, &ind, &curv, &ffx, &ffy, &ffz, &ux, &uy, &uz, &rho,
                    &pxx, &pyy, &pzz, &pxy, &pxz, &pyz, &pst})
      v->assign(N, 0);
  }

  long long I3(int i, int j, int k) const {
    return i + static_cast<long long>(p.nx) * (j + static_cast<long long>(p.ny) * k);
  }
  long long I4(int i, int j, int k, int l) const { return I3(i, j, k) + n * l; }
  bool ref() const { return p.bc == 0; }
  bool ratio() const { return p.rho_in != p.rho_out; }
  bool walls() const { return p.bc == 2; }
  bool shell(int i, int j, int k) const {
    return i == 0 || i == p.nx - 1 || j == 0 || j == p.ny - 1 || k == 0 || k == p.nz - 1;
  }
  // Cells the update acts on: the interior in ref mode, every cell otherwise.
  bool acts(int i, int j, int k) const { return !ref() || !shell(i, j, k); }
  static int wrap(int v, int m) { return ((v % m) + m) % m; }

  template <class F>
  void for_cells(F&& body) {
    const int nz = p.nz;
#pragma omp parallel for schedule(static) num_threads(p.threads)
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < p.ny; ++j)
        for (int i = 0; i < p.nx; ++i) body(i, j, k);
  }

  // phi at a stencil neighbour: wrap in periodic directions, mirror across z walls.
  T phi_at(int i, int j, int k) const {
    if (!ref()) {
      i = wrap(i, p.nx);
      j = wrap(j, p.ny);
      if (walls()) k = k < 0 ? -1 - k : (k >= p.nz ? 2 * p.nz - 1 - k : k);
      else k = wrap(k, p.nz);
    }
    return phi[I3(i, j, k)];
  }
  // normal at a stencil neighbour; across a z wall it is the mirror image (n_z flips).
  void n_at(int i, int j, int k, T& a, T& b, T& c) const {
    T s = 1;
    if (!ref()) {
      i = wrap(i, p.nx);
      j = wrap(j, p.ny);
      if (walls()) {
        if (k < 0) { k = -1 - k; s = -1; }
        else if (k >= p.nz) { k = 2 * p.nz - 1 - k; s = -1; }
      } else {
        k = wrap(k, p.nz);
      }
    }
    const long long o = I3(i, j, k);
    a = nx_[o];
    b = ny_[o];
    c = s * nz_[o];
  }

  void set_fields(const float* ph, const float* u, const float* v, const float* w) {
    double sum = 0;
    for (int k = 0; k < p.nz; ++k)
      for (int j = 0; j < p.ny; ++j)
        for (int i = 0; i < p.nx; ++i) {
          const long long o = I3(i, j, k);
          // Ref mode: the shell starts at 0 (cudaMemset, src/var.cu:86); initPhase writes
          // the interior only (src/init.cu:37).
          phi[o] = (ref() && shell(i, j, k)) ? T(0) : T(ph[o]);
          sum += ph[o];
          ux[o] = u ? T(u[o]) : T(0);
          uy[o] = v ? T(v[o]) : T(0);
          uz[o] = w ? T(w[o]) : T(0);
          rho[o] = ratio() ? T(0) : T(1);  // initTensor, src/init.cu:3-25 (p* = 0)
        }
    phi_mean = T(sum / static_cast<double>(n));
    // initDist (src/init.cu:51-80), generalised to f at the equilibrium of u and
    // g = W phi (1 + 3 c.u).
    for_cells([&](int i, int j, int k) {
      const long long o = I3(i, j, k);
      const T a = ux[o], b = uy[o], c = uz[o];
      const T uu = T(1.5) * (a * a + b * b + c * c);
      for (int l = 0; l < QF; ++l) {
        const T cu = T(3) * (a * FCX[l] + b * FCY[l] + c * FCZ[l]);
        // density ratio: p* = 0 at the start
        f[I4(i, j, k, l)] = FW[l] * ((ratio() ? T(0) : rho[o]) + cu + T(0.5) * cu * cu - uu);
      }
      for (int l = 0; l < 19; ++l) {
        const T cu = T(3) * (a * CIX[l] + b * CIY[l] + c * CIZ[l]);
        g[I4(i, j, k, l)] = W[l] * phi[o] * (T(1) + cu);
      }
    });
    for (int k = 0; k < p.nz; ++k)
      for (int j = 0; j < p.ny; ++j)
        for (int i = 0; i < p.nx; ++i)
          if (ref() && shell(i, j, k)) {
            ux[I3(i, j, k)] = uy[I3(i, j, k)] = uz[I3(i, j, k)] = 0;
          }
    update = -1;
  }

  // phiCalc, src/lbm.cu:5-26.
  void phi_calc() {
    for_cells([&](int i, int j, int k) {
      if (!acts(i, j, k)) return;
      T s = 0;
      for (int l = 0; l < 19; ++l) s += g[I4(i, j, k, l)];
      phi[I3(i, j, k)] = s;
    });
  }

  // gradCalc, src/lbm.cu:34-72.
  void grad_calc() {
    for_cells([&](int i, int j, int k) {
      if (!acts(i, j, k)) return;
      T gx = 0, gy = 0, gz = 0;
      for (int l = 0; l < 19; ++l) {
        const T v = phi_at(i + CIX[l], j + CIY[l], k + CIZ[l]);
        const T coef = T(3) * W[l];
        gx += coef * CIX[l] * v;
        gy += coef * CIY[l] * v;
        gz += coef * CIZ[l] * v;
      }
      const T g2 = gx * gx + gy * gy + gz * gz;
      const T fac = T(1) / std::sqrt(std::max(g2, T(1e-9)));
      const long long o = I3(i, j, k);
      nx_[o] = gx * fac;
      ny_[o] = gy * fac;
      nz_[o] = gz * fac;
      ind[o] = g2 * fac;
    });
  }

  // curvatureCalc, src/lbm.cu:80-125, plus the Boussinesq force on z.
  void curvature_calc() {
    for_cells([&](int i, int j, int k) {
      if (!acts(i, j, k)) return;
      const long long o = I3(i, j, k);
      T c = 0;
      for (int l = 0; l < 19; ++l) {
        T a, b, d;
        n_at(i + CIX[l], j + CIY[l], k + CIZ[l], a, b, d);
        c -= T(3) * W[l] * (CIX[l] * a + CIY[l] * b + CIZ[l] * d);
      }
      const T mult = SIGMA * c;
      curv[o] = c;
      ffx[o] = mult * nx_[o] * ind[o];
      ffy[o] = mult * ny_[o] * ind[o];
      ffz[o] = mult * nz_[o] * ind[o];
      if (p.gravity != 0) ffz[o] += T(p.gravity) * (phi[o] - phi_mean);
    });
  }

  // Moments of D3Q27 f from their definitions (see the header).
  void moments_q27() {
    for_cells([&](int i, int j, int k) {
      if (!acts(i, j, k)) return;
      const long long o = I3(i, j, k);
      T fv[27];
      for (int l = 0; l < 27; ++l) fv[l] = f[I4(i, j, k, l)];
      T r = 0, jx = 0, jy = 0, jz = 0;
      for (int l = 0; l < 27; ++l) {
        r += fv[l];
        jx += FCX[l] * fv[l];
        jy += FCY[l] * fv[l];
        jz += FCZ[l] * fv[l];
      }
      const T inv = T(1) / r;
      const T fx = ffx[o], fy = ffy[o], fz = ffz[o];
      const T a = (jx + T(0.5) * fx) * inv, b = (jy + T(0.5) * fy) * inv;
      const T c = (jz + T(0.5) * fz) * inv;
      const T ic = T(1) / CSSQ;
      const T uu = T(0.5) * (a * a + b * b + c * c) * ic;
      const T irc = T(1) / (r * CSSQ);
      T sxx = 0, syy = 0, szz = 0, sxy = 0, sxz = 0, syz = 0;
      for (int l = 0; l < 27; ++l) {
        const T udc = (a * FCX[l] + b * FCY[l] + c * FCZ[l]) * ic;
        const T common = FW[l] * (r + r * (udc + T(0.5) * udc * udc - uu));
        const T hef = T(0.5) * common *
                      ((FCX[l] - a) * fx + (FCY[l] - b) * fy + (FCZ[l] - c) * fz) * irc;
        const T fneq = fv[l] - (common - hef);
        sxx += FCX[l] * FCX[l] * fneq;
        syy += FCY[l] * FCY[l] * fneq;
        szz += FCZ[l] * FCZ[l] * fneq;
        sxy += FCX[l] * FCY[l] * fneq;
        sxz += FCX[l] * FCZ[l] * fneq;
        syz += FCY[l] * FCZ[l] * fneq;
      }
      pxx[o] = sxx;
      pyy[o] = syy;
      pzz[o] = szz;
      pxy[o] = sxy;
      pxz[o] = sxz;
      pyz[o] = syz;
      ux[o] = a;
      uy[o] = b;
      uz[o] = c;
      rho[o] = r;
    });
  }

  // Moments, total force and velocity of the density-ratio model (see the header).
  void moments_ratio() {
    const T drho = T(p.rho_in - p.rho_out), r_out = T(p.rho_out);
    for_cells([&](int i, int j, int k) {
      const long long o = I3(i, j, k);
      T ps = 0, jx = 0, jy = 0, jz = 0, sxx = 0, syy = 0, szz = 0, sxy = 0, sxz = 0, syz = 0;
      for (int l = 0; l < QF; ++l) {
        const T v = f[I4(i, j, k, l)];
        const T X = FCX[l], Y = FCY[l], Z = FCZ[l];
        ps += v;
        jx += X * v;
        jy += Y * v;
        jz += Z * v;
        sxx += X * X * v;
        syy += Y * Y * v;
        szz += Z * Z * v;
        sxy += X * Y * v;
        sxz += X * Z * v;
        syz += Y * Z * v;
      }
      const T rp = r_out + drho * phi[o];
      const T gx = drho * nx_[o] * ind[o], gy = drho * ny_[o] * ind[o];
      const T gz = drho * nz_[o] * ind[o];
      const T p3 = ps * CSSQ;
      const T qxx = sxx - p3 - jx * jx, qyy = syy - p3 - jy * jy, qzz = szz - p3 - jz * jz;
      const T qxy = sxy - jx * jy, qxz = sxz - jx * jz, qyz = syz - jy * jz;
      const T cm = T(1) - T(0.5) * OMEGA;
      const T fx = ffx[o] - p3 * gx - cm * (qxx * gx + qxy * gy + qxz * gz);
      const T fy = ffy[o] - p3 * gy - cm * (qxy * gx + qyy * gy + qyz * gz);
      const T fz = ffz[o] - p3 * gz - cm * (qxz * gx + qyz * gy + qzz * gz);
      const T a = jx + T(0.5) * fx / rp, b = jy + T(0.5) * fy / rp, c = jz + T(0.5) * fz / rp;
      pxx[o] = sxx - p3 - a * a;
      pyy[o] = syy - p3 - b * b;
      pzz[o] = szz - p3 - c * c;
      pxy[o] = sxy - a * b;
      pxz[o] = sxz - a * c;
      pyz[o] = syz - b * c;
      ffx[o] = fx;
      ffy[o] = fy;
      ffz[o] = fz;
      ux[o] = a;
      uy[o] = b;
      uz[o] = c;
      pst[o] = ps;
      rho[o] = ps * rp;  // p / cs^2
    });
  }

  // momentiCalc, src/lbm.cu:133-225.
  void momenti_calc() {
    if (ratio()) {
      moments_ratio();
      return;
    }
    if (QF == 27) {
      moments_q27();
      return;
    }
    for_cells([&](int i, int j, int k) {
      if (!acts(i, j, k)) return;
      const long long o = I3(i, j, k);
      T fv[19], fneq[19];
      for (int l = 0; l < 19; ++l) fv[l] = f[I4(i, j, k, l)];
      T r = 0;
      for (int l = 0; l < 19; ++l) r += fv[l];
      const T inv = T(1) / r;
      const T sx = inv * (fv[1] - fv[2] + fv[7] - fv[8] + fv[9] - fv[10] + fv[13] - fv[14] +
                          fv[15] - fv[16]);
      const T sy = inv * (fv[3] - fv[4] + fv[7] - fv[8] + fv[11] - fv[12] + fv[14] - fv[13] +
                          fv[17] - fv[18]);
      const T sz = inv * (fv[5] - fv[6] + fv[9] - fv[10] + fv[11] - fv[12] + fv[16] - fv[15] +
                          fv[18] - fv[17]);
      const T fx = ffx[o], fy = ffy[o], fz = ffz[o];
      const T a = sx + fx * T(0.5) * inv, b = sy + fy * T(0.5) * inv, c = sz + fz * T(0.5) * inv;
      const T ic = T(1) / CSSQ;
      const T uu = T(0.5) * (a * a + b * b + c * c) * ic;
      const T irc = T(1) / (r * CSSQ);
      for (int l = 0; l < 19; ++l) {
        const T udc = (a * CIX[l] + b * CIY[l] + c * CIZ[l]) * ic;
        const T eq = r * (udc + T(0.5) * udc * udc - uu);
        const T common = W[l] * (r + eq);
        const T hef = T(0.5) * common *
                      ((CIX[l] - a) * fx + (CIY[l] - b) * fy + (CIZ[l] - c) * fz) * irc;
        fneq[l] = fv[l] - (common - hef);
      }
      pxx[o] = fneq[1] + fneq[2] + fneq[7] + fneq[8] + fneq[9] + fneq[10] + fneq[13] + fneq[14] +
               fneq[15] + fneq[16];
      pyy[o] = fneq[3] + fneq[4] + fneq[7] + fneq[8] + fneq[11] + fneq[12] + fneq[13] +
               fneq[14] + fneq[17] + fneq[18];
      pzz[o] = fneq[5] + fneq[6] + fneq[9] + fneq[10] + fneq[11] + fneq[12] + fneq[15] +
               fneq[16] + fneq[17] + fneq[18];
      pxy[o] = fneq[7] - fneq[13] + fneq[8] - fneq[14];
      pxz[o] = fneq[9] - fneq[15] + fneq[10] - fneq[16];
      pyz[o] = fneq[11] - fneq[17] + fneq[12] - fneq[18];
      ux[o] = a;
      uy[o] = b;
      uz[o] = c;
      rho[o] = r;
    });
  }

  // Target of a push along direction l from (i,j,k): false if the link leaves through a
  // z wall (the population bounces back into (i,j,k) as opp(l)).
  bool push_target(int i, int j, int k, int l, int& ti, int& tj, int& tk) const {
    ti = i + FCX[l];
    tj = j + FCY[l];
    tk = k + FCZ[l];
    if (ref()) return true;  // interior cells always land inside
    ti = wrap(ti, p.nx);
    tj = wrap(tj, p.ny);
    if (walls() && (tk < 0 || tk >= p.nz)) return false;
    tk = wrap(tk, p.nz);
    return true;
  }

  // Collision of the density-ratio model (see the header), pushed like collisionFluid.
  void collision_ratio() {
    const T drho = T(p.rho_in - p.rho_out), r_out = T(p.rho_out);
    for_cells([&](int i, int j, int k) {
      const long long o = I3(i, j, k);
      const T a = ux[o], b = uy[o], c = uz[o], ps = pst[o];
      const T rp = r_out + drho * phi[o];
      const T fx = ffx[o], fy = ffy[o], fz = ffz[o];
      const T uu = T(1.5) * (a * a + b * b + c * c);
      const T tr = (pxx[o] + pyy[o] + pzz[o]) * CSSQ;
      for (int l = 0; l < QF; ++l) {
        const int X = FCX[l], Y = FCY[l], Z = FCZ[l];
        const T cu = T(3) * (a * X + b * Y + c * Z);
        const T feq = FW[l] * (ps + cu + T(0.5) * cu * cu - uu);
        const T qpi = X * X * pxx[o] + Y * Y * pyy[o] + Z * Z * pzz[o] +
                      T(2) * (X * Y * pxy[o] + X * Z * pxz[o] + Y * Z * pyz[o]) - tr;
        const T post = feq + (T(1) - OMEGA) * FW[l] * T(4.5) * qpi +
                       (T(1) - T(0.5) * OMEGA) * T(3) * FW[l] * (X * fx + Y * fy + Z * fz) / rp;
        int ti, tj, tk;
        if (push_target(i, j, k, l, ti, tj, tk)) f[I4(ti, tj, tk, l)] = post;
        else f[I4(i, j, k, OPP(l))] = post;
      }
    });
  }

  // collisionFluid, src/lbm.cu:233-288 (in-place push; collision reads only the moments).
  void collision_fluid() {
    if (ratio()) {
      collision_ratio();
      return;
    }
    for_cells([&](int i, int j, int k) {
      if (!acts(i, j, k)) return;
      const long long o = I3(i, j, k);
      const T a = ux[o], b = uy[o], c = uz[o], r = rho[o];
      const T fx = ffx[o], fy = ffy[o], fz = ffz[o];
      const T uu = T(0.5) * (a * a + b * b + c * c) / CSSQ;
      const T irc = T(1) / (r * CSSQ);
      const T ic = T(1) / CSSQ;
      for (int l = 0; l < QF; ++l) {
        const int X = FCX[l], Y = FCY[l], Z = FCZ[l];
        const T udc = (a * X + b * Y + c * Z) * ic;
        const T feq = FW[l] * (r + r * (udc + T(0.5) * udc * udc - uu));
        const T hef = T(0.5) * feq * ((X - a) * fx + (Y - b) * fy + (Z - c) * fz) * irc;
        const T fneq = (FW[l] / (T(2) * CSSQ * CSSQ)) *
                       ((X * X - CSSQ) * pxx[o] + (Y * Y - CSSQ) * pyy[o] +
                        (Z * Z - CSSQ) * pzz[o] + T(2) * X * Y * pxy[o] +
                        T(2) * X * Z * pxz[o] + T(2) * Y * Z * pyz[o]);
        const T post = feq + (T(1) - OMEGA) * fneq + hef;
        int ti, tj, tk;
        if (push_target(i, j, k, l, ti, tj, tk)) f[I4(ti, tj, tk, l)] = post;
        else f[I4(i, j, k, OPP(l))] = post;
      }
    });
  }

  // collisionPhase, src/lbm.cu:290-329 (in place). With tau_g != 1 the post-collision
  // value relaxes from the incoming g towards the same equilibrium.
  void collision_phase() {
    const bool full = p.tau_g == 1.0;
    for_cells([&](int i, int j, int k) {
      if (!acts(i, j, k)) return;
      const long long o = I3(i, j, k);
      const T a = ux[o], b = uy[o], c = uz[o], ph = phi[o];
      const T na = nx_[o], nb = ny_[o], nc = nz_[o];
      const T ic = T(1) / CSSQ;
      const T pn = SHARP_C * ph * (T(1) - ph);
      for (int l = 0; l < 19; ++l) {
        const T udc = (a * CIX[l] + b * CIY[l] + c * CIZ[l]) * ic;
        const T geq = W[l] * ph * (T(1) + udc);
        const T ai = pn * (CIX[l] * na + CIY[l] * nb + CIZ[l] * nc);
        const T eq = geq + W[l] * ai;
        T& gv = g[I4(i, j, k, l)];
        gv = full ? eq : gv + OMEGA_G * (eq - gv);
      }
    });
  }

  // movingWallBC, src/lbm.cu:430-461: writes f on the j = 0 and j = ny-1 shell planes only.
  // It is launched on the 3-D grid, so k only reaches 8 * ceil(ny/8). Nothing reads those
  // values afterwards.
  void moving_wall() {
    const int kmax = std::min(p.nz, 8 * ((p.ny + 7) / 8));
    const T uw = T(0.03);
    for (int k = 0; k < kmax; ++k)
      for (int i = 0; i < p.nx; ++i)
        for (int l = 0; l < QF; ++l) {
          const T rb = rho[I3(i, 0, k)];
          f[I4(i, 0, k, l)] = rb * FW[l] * (T(1) + (FCX[l] * (-uw)) / CSSQ);
          const T rt = rho[I3(i, p.ny - 1, k)];
          f[I4(i, p.ny - 1, k, l)] = rt * FW[l] * (T(1) + (FCX[l] * uw) / CSSQ);
        }
  }

  // streamingCalc, src/lbm.cu:337-357 (pull with periodic wrap; modulo instead of the
  // power-of-two mask). Walls bounce g back so phi cannot leave through them.
  void streaming() {
    for_cells([&](int i, int j, int k) {
      for (int l = 0; l < 19; ++l) {
        int si = wrap(i - CIX[l], p.nx), sj = wrap(j - CIY[l], p.ny);
        int sk = k - CIZ[l];
        if (walls() && (sk < 0 || sk >= p.nz)) {
          g_out[I4(i, j, k, l)] = g[I4(i, j, k, OPP(l))];
          continue;
        }
        sk = wrap(sk, p.nz);
        g_out[I4(i, j, k, l)] = g[I4(si, sj, sk, l)];
      }
    });
    std::swap(g, g_out);
  }

  // fgBoundary, src/lbm.cu:365-401.
  void fg_boundary() {
    for (int k = 0; k < p.nz; ++k)
      for (int j = 0; j < p.ny; ++j)
        for (int i = 0; i < p.nx; ++i) {
          if (!shell(i, j, k)) continue;
          const long long o = I3(i, j, k);
          for (int l = 0; l < QF; ++l) {
            const int a = i + FCX[l], b = j + FCY[l], c = k + FCZ[l];
            if (a >= 0 && a < p.nx && b >= 0 && b < p.ny && c >= 0 && c < p.nz)
              f[I4(a, b, c, l)] = rho[o] * FW[l];
          }
          for (int l = 0; l < 19; ++l) {
            const int a = i + CIX[l], b = j + CIY[l], c = k + CIZ[l];
            if (a >= 0 && a < p.nx && b >= 0 && b < p.ny && c >= 0 && c < p.nz)
              g[I4(a, b, c, l)] = phi[o] * W[l];
          }
        }
  }

  // boundaryConditions, src/lbm.cu:403-425, as the three face copies run in order (z, y,
  // x). The reference runs them concurrently from every thread, so its edges are racy.
  void boundary_conditions() {
    const int X = p.nx, Y = p.ny, Z = p.nz;
    for (int j = 0; j < Y; ++j)
      for (int i = 0; i < X; ++i) {
        phi[I3(i, j, 0)] = phi[I3(i, j, 1)];
        phi[I3(i, j, Z - 1)] = phi[I3(i, j, Z - 2)];
      }
    for (int k = 0; k < Z; ++k)
      for (int i = 0; i < X; ++i) {
        phi[I3(i, 0, k)] = phi[I3(i, 1, k)];
        phi[I3(i, Y - 1, k)] = phi[I3(i, Y - 2, k)];
      }
    for (int k = 0; k < Z; ++k)
      for (int j = 0; j < Y; ++j) {
        phi[I3(0, j, k)] = phi[I3(1, j, k)];
        phi[I3(X - 1, j, k)] = phi[I3(X - 2, j, k)];
      }
  }

  // One update in the order of src/main.cu:79-178, on one stream.
  void step() {
    phi_calc();
    grad_calc();
    curvature_calc();
    momenti_calc();
    collision_fluid();
    collision_phase();
    if (ref() && p.moving_wall) moving_wall();
    streaming();
    if (ref()) {
      fg_boundary();
      boundary_conditions();
    }
    ++update;
  }
};

struct Any {
  int prec;
  void* impl;
};

template <class T>
Oracle<T>* as(Any* a) {
  return static_cast<Oracle<T>*>(a->impl);
}

}  // namespace

extern "C" {

typedef struct orc_params {
  int nx, ny, nz, bc;
  double tau, tau_g, sigma, sharp_c, gravity;
  int threads;
  int moving_wall;
  int qf;  // velocity set of f: 19 (or 0) or 27
  double rho_in, rho_out;  // phase densities (0, 0 or equal: density-matched model)
} orc_params;

void* orc_create(const orc_params* q, int precision) {
  if (!q || q->nx < 3 || q->ny < 3 || q->nz < 3 || q->bc < 0 || q->bc > 2) return nullptr;
  if (precision != 32 && precision != 64) return nullptr;
  if (q->qf != 0 && q->qf != 19 && q->qf != 27) return nullptr;
  const bool ratio = q->rho_in > 0 && q->rho_out > 0 && q->rho_in != q->rho_out;
  if (ratio && q->bc == 0) return nullptr;  // the frozen shell is density-matched only
  Params p{q->nx, q->ny, q->nz, q->bc, q->tau, q->tau_g, q->sigma, q->sharp_c, q->gravity,
           q->threads > 0 ? q->threads : 1, q->moving_wall, q->qf == 27 ? 27 : 19,
           ratio ? q->rho_in : 1.0, ratio ? q->rho_out : 1.0};
  Any* a = new Any{precision, nullptr};
  if (precision == 64) a->impl = new Oracle<double>(p);
  else a->impl = new Oracle<float>(p);
  return a;
}

void orc_destroy(void* h) {
  Any* a = static_cast<Any*>(h);
  if (!a) return;
  if (a->prec == 64) delete as<double>(a);
  else delete as<float>(a);
  delete a;
}

int orc_set_fields(void* h, const float* phi, const float* ux, const float* uy,
                   const float* uz) {
  Any* a = static_cast<Any*>(h);
  if (!a || !phi) return 1;
  if (a->prec == 64) as<double>(a)->set_fields(phi, ux, uy, uz);
  else as<float>(a)->set_fields(phi, ux, uy, uz);
  return 0;
}

int orc_step(void* h, int nsteps) {
  Any* a = static_cast<Any*>(h);
  if (!a || nsteps < 0) return 1;
  for (int s = 0; s < nsteps; ++s) {
    if (a->prec == 64) as<double>(a)->step();
    else as<float>(a)->step();
  }
  return 0;
}

// which: 0 phi, 1 rho, 2 ux, 3 uy, 4 uz, 5 p = rho/3
int orc_get(void* h, int which, double* out) {
  Any* a = static_cast<Any*>(h);
  if (!a || !out || which < 0 || which > 5) return 1;
  auto copy = [&](auto* o) {
    const auto& src = which == 0 ? o->phi : which == 1 || which == 5 ? o->rho
                    : which == 2 ? o->ux : which == 3 ? o->uy : o->uz;
    for (long long i = 0; i < o->n; ++i)
      out[i] = which == 5 ? static_cast<double>(src[i]) / 3.0 : static_cast<double>(src[i]);
  };
  if (a->prec == 64) copy(as<double>(a));
  else copy(as<float>(a));
  return 0;
}

// out: mass, ke, umax, rho_in, rho_out, dp, n_in, n_out, vol_half (interior for ref mode)
int orc_diag(void* h, double* out) {
  Any* a = static_cast<Any*>(h);
  if (!a || !out) return 1;
  auto run = [&](auto* o) {
    double mass = 0, ke = 0, umax = 0, rin = 0, rout = 0, nin = 0, nout = 0, vh = 0;
    for (int k = 0; k < o->p.nz; ++k)
      for (int j = 0; j < o->p.ny; ++j)
        for (int i = 0; i < o->p.nx; ++i) {
          if (o->ref() && o->shell(i, j, k)) continue;
          const long long c = o->I3(i, j, k);
          const double ph = o->phi[c], r = o->rho[c];
          // kinetic energy with the density (the rho field is p / cs^2 with a ratio)
          const double rk = o->ratio() ? o->p.rho_out + (o->p.rho_in - o->p.rho_out) * ph : r;
          const double u2 = double(o->ux[c]) * o->ux[c] + double(o->uy[c]) * o->uy[c] +
                            double(o->uz[c]) * o->uz[c];
          mass += ph;
          ke += 0.5 * rk * u2;
          umax = std::max(umax, std::sqrt(u2));
          if (ph > 0.99) { rin += r; nin += 1; }
          if (ph < 0.01) { rout += r; nout += 1; }
          if (ph > 0.5) vh += 1;
        }
    out[0] = mass;
    out[1] = ke;
    out[2] = umax;
    out[3] = nin > 0 ? rin / nin : 0;
    out[4] = nout > 0 ? rout / nout : 0;
    out[5] = (nin > 0 && nout > 0) ? (out[3] - out[4]) / 3.0 : 0;
    out[6] = nin;
    out[7] = nout;
    out[8] = vh;
  };
  if (a->prec == 64) run(as<double>(a));
  else run(as<float>(a));
  return 0;
}

int orc_threads_available(void) {
#ifdef _OPENMP
  return omp_get_num_procs();
#else
  return 1;
#endif
}

}  // extern "C"
