// Host-side initial fields: the reference's single centred bubble (src/init.cu:27-49) and the
// seeded multi-bubble scenarios of the benchmark set. Every random draw comes from
// splitmix64, so the GPU path and the CPU oracle receive identical float32 arrays.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "mcb.h"

namespace {

struct Rng {
  uint64_t s;
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double uniform() { return static_cast<double>(next() >> 11) * (1.0 / 9007199254740992.0); }
  double uniform(double a, double b) { return a + (b - a) * uniform(); }
  double normal() {  // Box-Muller
    double u1 = uniform();
    if (u1 < 1e-300) u1 = 1e-300;
    const double u2 = uniform();
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
  }
};

double profile(double R, double d, double width) {
  return 0.5 + 0.5 * std::tanh(2.0 * (R - d) / width);
}

// Signed nearest-image offset along a periodic axis.
double image(double d, int n, bool periodic) {
  if (!periodic) return d;
  const double h = 0.5 * n;
  while (d > h) d -= n;
  while (d < -h) d += n;
  return d;
}

int axis_index(int v, int n, bool periodic) {
  if (periodic) return ((v % n) + n) % n;
  return (v < 0 || v >= n) ? -1 : v;
}

// Associated Legendre P_l^m(x), m >= 0, by the standard three-term recurrence.
double legendre(int l, int m, double x) {
  double pmm = 1.0;
  const double s = std::sqrt(std::max(0.0, 1.0 - x * x));
  for (int i = 1; i <= m; ++i) pmm *= -(2.0 * i - 1.0) * s;
  if (l == m) return pmm;
  double pm1 = x * (2.0 * m + 1.0) * pmm;
  if (l == m + 1) return pm1;
  double pl = 0.0;
  for (int ll = m + 2; ll <= l; ++ll) {
    pl = ((2.0 * ll - 1.0) * x * pm1 - (ll + m - 1.0) * pmm) / (ll - m);
    pmm = pm1;
    pm1 = pl;
  }
  return pl;
}

// Real spherical harmonic shape (unnormalised): P_l^|m|(cos t) * (cos m p | sin |m| p).
double ylm(int l, int m, double t, double p) {
  const double leg = legendre(l, std::abs(m), std::cos(t));
  return m >= 0 ? leg * std::cos(m * p) : leg * std::sin(-m * p);
}

struct Mode {
  int l, m;
  double amp, norm;
};

void fill_bubbles(int nx, int ny, int nz, int bc, double width, const mcb_bubble* b, int nb,
                  float* phi) {
  const bool px = bc != MCB_BC_REF, py = bc != MCB_BC_REF, pz = bc == MCB_BC_PERIODIC;
  const size_t n = static_cast<size_t>(nx) * ny * nz;
  std::vector<double> acc(n, 0.0);
  for (int k = 0; k < nb; ++k) {
    const mcb_bubble& q = b[k];
    const double ax = q.ax > 0 ? q.ax : 1.0, ay = q.ay > 0 ? q.ay : 1.0;
    const double az = q.az > 0 ? q.az : 1.0;
    const double reach = q.r * std::max(ax, std::max(ay, az)) + 5.0 * width;
    const int x0 = static_cast<int>(std::floor(q.cx - reach)), x1 = static_cast<int>(std::ceil(q.cx + reach));
    const int y0 = static_cast<int>(std::floor(q.cy - reach)), y1 = static_cast<int>(std::ceil(q.cy + reach));
    const int z0 = static_cast<int>(std::floor(q.cz - reach)), z1 = static_cast<int>(std::ceil(q.cz + reach));
    // Visit each lattice cell at most once per bubble even when the box wraps.
    std::vector<int> xs, ys, zs;
    for (int v = x0; v <= x1 && static_cast<int>(xs.size()) < nx; ++v) {
      const int i = axis_index(v, nx, px);
      if (i >= 0) xs.push_back(i);
    }
    for (int v = y0; v <= y1 && static_cast<int>(ys.size()) < ny; ++v) {
      const int j = axis_index(v, ny, py);
      if (j >= 0) ys.push_back(j);
    }
    for (int v = z0; v <= z1 && static_cast<int>(zs.size()) < nz; ++v) {
      const int kk = axis_index(v, nz, pz);
      if (kk >= 0) zs.push_back(kk);
    }
    for (int kk : zs)
      for (int j : ys)
        for (int i : xs) {
          const double dx = image(i - q.cx, nx, px) / ax;
          const double dy = image(j - q.cy, ny, py) / ay;
          const double dz = image(kk - q.cz, nz, pz) / az;
          const double d = std::sqrt(dx * dx + dy * dy + dz * dz);
          const size_t idx = i + static_cast<size_t>(nx) * (j + static_cast<size_t>(ny) * kk);
          acc[idx] = std::max(acc[idx], profile(q.r, d, width));
        }
  }
  for (size_t i = 0; i < n; ++i) phi[i] = static_cast<float>(acc[i]);
  if (bc == MCB_BC_REF) {
    // The reference's init writes the interior only; the shell stays 0 (src/init.cu:37).
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i)
          if (i == 0 || i == nx - 1 || j == 0 || j == ny - 1 || k == 0 || k == nz - 1)
            phi[i + static_cast<size_t>(nx) * (j + static_cast<size_t>(ny) * k)] = 0.0f;
  }
}

// Places nb non-overlapping bubbles (gap >= width) with radii in [rlo, rhi] and centres in
// [lo, hi] per axis. Returns false if the domain is too crowded.
bool place(Rng& rng, int nb, double rlo, double rhi, const double lo[3], const double hi[3],
           const int dims[3], const bool per[3], double width, std::vector<mcb_bubble>& out) {
  out.clear();
  for (int k = 0; k < nb; ++k) {
    bool ok = false;
    for (int tries = 0; tries < 20000 && !ok; ++tries) {
      mcb_bubble q{};
      q.r = rng.uniform(rlo, rhi);
      q.ax = q.ay = q.az = 1.0;
      double c[3];
      for (int a = 0; a < 3; ++a) {
        const double l = per[a] ? lo[a] : std::max(lo[a], q.r + 2.0);
        const double h = per[a] ? hi[a] : std::min(hi[a], dims[a] - 1.0 - q.r - 2.0);
        if (h < l) break;
        c[a] = rng.uniform(l, h);
      }
      q.cx = c[0];
      q.cy = c[1];
      q.cz = c[2];
      ok = true;
      for (const auto& o : out) {
        const double dx = image(q.cx - o.cx, dims[0], per[0]);
        const double dy = image(q.cy - o.cy, dims[1], per[1]);
        const double dz = image(q.cz - o.cz, dims[2], per[2]);
        if (std::sqrt(dx * dx + dy * dy + dz * dz) < q.r + o.r + width) {
          ok = false;
          break;
        }
      }
      if (ok) out.push_back(q);
    }
    if (!ok) return false;
  }
  return true;
}

int scaled(double e, double s) { return std::max(8, static_cast<int>(std::lround(e * s))); }

}  // namespace

extern "C" {

int mcb_fill_phi_reference(int nx, int ny, int nz, float r, float width, float* phi) {
  if (!phi || nx < 3 || ny < 3 || nz < 3 || !(width > 0.f)) return MCB_ERR_INVALID;
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        float v = 0.0f;
        if (i > 0 && i < nx - 1 && j > 0 && j < ny - 1 && k > 0 && k < nz - 1) {
          const float dx = i - nx * 0.5f, dy = j - ny * 0.5f, dz = k - nz * 0.5f;
          const float ri = std::sqrt(dx * dx + dy * dy + dz * dz);
          v = 0.5f + 0.5f * std::tanh(2.0f * (r - ri) / width);
        }
        phi[i + static_cast<size_t>(nx) * (j + static_cast<size_t>(ny) * k)] = v;
      }
  return MCB_OK;
}

int mcb_fill_phi_bubbles(int nx, int ny, int nz, int bc, float width, const mcb_bubble* bubbles,
                         int nbubbles, float* phi) {
  if (!phi || nx < 1 || ny < 1 || nz < 1 || nbubbles < 0 || (nbubbles > 0 && !bubbles) ||
      !(width > 0.f))
    return MCB_ERR_INVALID;
  fill_bubbles(nx, ny, nz, bc, width, bubbles, nbubbles, phi);
  return MCB_OK;
}

int mcb_workload(int scenario, int case_index, uint64_t seed, double scale, mcb_config* cfg,
                 float* phi, float* ux, float* uy, float* uz) {
  if (!cfg || !(scale > 0.0) || scale > 4.0) return MCB_ERR_INVALID;
  mcb_config_default(cfg);
  Rng rng{seed * 0x2545F4914F6CDD1Dull + static_cast<uint64_t>(scenario) * 0x9E37ull +
          static_cast<uint64_t>(case_index) * 0xD1B54A32D192ED03ull};
  const double W = 4.0;
  cfg->width = static_cast<float>(W);
  cfg->sharp_c = 0.0f;  // derived from tau_g and width
  cfg->gravity = 0.0f;
  cfg->tau_g = 1.0f;
  std::vector<mcb_bubble> bubbles;
  int modes_l = 0;
  std::vector<Mode> modes;
  double noise = 0.0;
  switch (scenario) {
    case 0: {  // reference parity case: frozen shell, 64^3, R 12, W 4, tau 0.8, sigma 0.1
      const int e = scaled(64, scale);
      cfg->nx = cfg->ny = cfg->nz = e;
      cfg->bc = MCB_BC_REF;
      cfg->tau = 0.8f;
      cfg->sigma = 0.1f;
      if (phi) mcb_fill_phi_reference(e, e, e, static_cast<float>(12.0 * scale), 4.0f, phi);
      break;
    }
    case 1: {  // static bubble, 64^3 periodic, R 12, W 4, tau 0.8, sigma 0.1, tau_g 0.8
      const int e = scaled(64, scale);
      cfg->nx = cfg->ny = cfg->nz = e;
      cfg->bc = MCB_BC_PERIODIC;
      cfg->tau = 0.8f;
      cfg->tau_g = 0.8f;
      cfg->sigma = 0.1f;
      // The geometric centre of the node set, (e-1)/2, is off the nodes.
      const double c = 0.5 * (e - 1);
      mcb_bubble q{c, c, c, 12.0 * scale, 1, 1, 1};
      bubbles.push_back(q);
      break;
    }
    case 2: {  // rising perturbed bubble, 128x128x256, walls in z, g 1e-5
      cfg->nx = scaled(128, scale);
      cfg->ny = scaled(128, scale);
      cfg->nz = scaled(256, scale);
      cfg->bc = MCB_BC_WALLS_Z;
      cfg->tau = 0.7f;
      cfg->sigma = 0.05f;
      cfg->gravity = 1e-5f;
      mcb_bubble q{0.5 * (cfg->nx - 1), 0.5 * (cfg->ny - 1), 48.0 * scale, 16.0 * scale, 1, 1, 1};
      bubbles.push_back(q);
      for (int l = 2; l <= 6; ++l) {
        Mode md;
        md.l = l;
        md.m = static_cast<int>(std::floor(rng.uniform() * (2 * l + 1))) - l;
        if (md.m > l) md.m = l;
        md.amp = rng.uniform(0.0, 0.5) * scale;
        double mx = 0.0;  // normalise the mode to a unit crest
        for (int a = 0; a <= 180; ++a)
          for (int c = 0; c < 360; ++c)
            mx = std::max(mx, std::fabs(ylm(l, md.m, a * M_PI / 180.0, c * M_PI / 180.0)));
        md.norm = mx > 0 ? 1.0 / mx : 0.0;
        modes.push_back(md);
      }
      modes_l = 1;
      break;
    }
    case 3: {  // 32 bubbles, 256^3 periodic, Gaussian velocity noise
      const int e = scaled(256, scale);
      cfg->nx = cfg->ny = cfg->nz = e;
      cfg->bc = MCB_BC_PERIODIC;
      cfg->tau = 0.6f;
      cfg->sigma = 0.05f;
      const double lo[3] = {0, 0, 0}, hi[3] = {1.0 * e, 1.0 * e, 1.0 * e};
      const int dims[3] = {e, e, e};
      const bool per[3] = {true, true, true};
      if (!place(rng, 32, 6.0 * scale, 16.0 * scale, lo, hi, dims, per, W, bubbles))
        return MCB_ERR_INVALID;
      noise = 1e-4;
      break;
    }
    case 4: {  // one case of the batched set
      if (case_index < 0) return MCB_ERR_INVALID;
      static const int edges[5] = {32, 48, 64, 80, 96};
      const int e = scaled(edges[static_cast<int>(rng.uniform() * 5) % 5], scale);
      cfg->nx = cfg->ny = cfg->nz = e;
      cfg->bc = MCB_BC_PERIODIC;
      cfg->storage = MCB_STORE_F16;
      const double R = rng.uniform(0.15, 0.3) * e;
      cfg->sigma = static_cast<float>(rng.uniform(0.01, 0.1));
      cfg->tau = static_cast<float>(rng.uniform(0.55, 1.0));
      const double asp = rng.uniform(1.0, 1.3);
      // Volume-preserving prolate ellipsoid along x.
      const double c = 0.5 * (e - 1);
      mcb_bubble q{c, c, c, R, std::pow(asp, 2.0 / 3.0),
                   std::pow(asp, -1.0 / 3.0), std::pow(asp, -1.0 / 3.0)};
      bubbles.push_back(q);
      break;
    }
    case 5: {  // 512 bubbles in the lower half of 512^3, walls in z, g 5e-6
      const int e = scaled(512, scale);
      cfg->nx = cfg->ny = cfg->nz = e;
      cfg->bc = MCB_BC_WALLS_Z;
      cfg->storage = MCB_STORE_F16;
      cfg->tau = 0.6f;
      cfg->sigma = 0.03f;
      cfg->gravity = 5e-6f;
      const double lo[3] = {0, 0, 0}, hi[3] = {1.0 * e, 1.0 * e, 0.5 * e};
      const int dims[3] = {e, e, e};
      const bool per[3] = {true, true, false};
      if (!place(rng, 512, 5.0 * scale, 10.0 * scale, lo, hi, dims, per, W, bubbles))
        return MCB_ERR_INVALID;
      break;
    }
    case 6: {  // 64^3 periodic rerun of the multi-bubble precision study (4 bubbles)
      const int e = scaled(64, scale);
      cfg->nx = cfg->ny = cfg->nz = e;
      cfg->bc = MCB_BC_PERIODIC;
      cfg->tau = 0.6f;
      cfg->sigma = 0.05f;
      const double lo[3] = {0, 0, 0}, hi[3] = {1.0 * e, 1.0 * e, 1.0 * e};
      const int dims[3] = {e, e, e};
      const bool per[3] = {true, true, true};
      if (!place(rng, 4, 6.0 * scale, 12.0 * scale, lo, hi, dims, per, W, bubbles))
        return MCB_ERR_INVALID;
      noise = 1e-4;
      break;
    }
    default:
      return MCB_ERR_INVALID;
  }
  if (!phi) return MCB_OK;
  const int nx = cfg->nx, ny = cfg->ny, nz = cfg->nz;
  const size_t n = static_cast<size_t>(nx) * ny * nz;
  if (scenario != 0) {
    if (modes_l) {
      // Perturbed sphere: R(theta, p) = R0 + sum_l a_l Y_l^m(theta, p) / max|Y_l^m|.
      const mcb_bubble& q = bubbles[0];
      std::vector<double> acc(n, 0.0);
      for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
          for (int i = 0; i < nx; ++i) {
            const double dx = image(i - q.cx, nx, true), dy = image(j - q.cy, ny, true);
            const double dz = k - q.cz;
            const double d = std::sqrt(dx * dx + dy * dy + dz * dz);
            double R = q.r;
            if (d > 1e-12) {
              const double t = std::acos(std::max(-1.0, std::min(1.0, dz / d)));
              const double p = std::atan2(dy, dx);
              for (const Mode& md : modes) R += md.amp * md.norm * ylm(md.l, md.m, t, p);
            }
            acc[i + static_cast<size_t>(nx) * (j + static_cast<size_t>(ny) * k)] =
                profile(R, d, W);
          }
      for (size_t i = 0; i < n; ++i) phi[i] = static_cast<float>(acc[i]);
    } else {
      fill_bubbles(nx, ny, nz, cfg->bc, W, bubbles.data(), static_cast<int>(bubbles.size()),
                   phi);
    }
  }
  if (ux && uy && uz) {
    for (size_t i = 0; i < n; ++i) {
      ux[i] = noise > 0 ? static_cast<float>(noise * rng.normal()) : 0.0f;
      uy[i] = noise > 0 ? static_cast<float>(noise * rng.normal()) : 0.0f;
      uz[i] = noise > 0 ? static_cast<float>(noise * rng.normal()) : 0.0f;
    }
  }
  return MCB_OK;
}

}  // extern "C"
