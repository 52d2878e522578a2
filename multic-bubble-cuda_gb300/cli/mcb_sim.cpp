// mcb_sim: command-line driver that replaces the reference's src/main.cu.
//
//   mcb_sim <velocity_set> <id> [options]      velocity_set: D3Q19 or D3Q27 (for f)
//
// With no options it runs the reference's hard-coded case (src/var.cu:3-25,
// src/init.cu:27-49, src/main.cu:35):
//   - 64x64x256, tau 0.505, sigma 0.1, sharp_c 0.45;
//   - one bubble, R 20, width 3;
//   - 25000 updates, saved every 100.
// Output goes to ../bin/<velocity_set>/<id>/ relative to the working directory
// (src/main.cu:14-21): <id>_info.txt and <id>_phiNNNNNN.bin, which post/fileTreat.py reads.
// Update STEP is dumped after it has run, for STEP = 0, save, 2*save, ... up to the step
// count (src/main.cu:74-190 runs NSTEPS+1 updates).
//
// Options:
//   --steps N       updates after update 0 (default 25000)
//   --save N        dump every N updates (default 100; 0 = no dumps)
//   --out DIR       output directory instead of ../bin/<vs>/<id>/
//   --scenario K    seeded benchmark scenario 0..5 instead of the reference case
//   --scale S       length scale of the scenario (default 1)
//   --seed N        scenario seed (default 1)
//   --storage f32|f16|bf16
//   --autotune      pick the fastest tile variant before running
//   --fields LIST   comma-separated fields to dump: phi,rho,ux,uy,uz,pres (default phi)
//   --checkpoint F  write a checkpoint of the full solver state to F after the last update
//   --restart F     resume from checkpoint F (same case options) instead of the initial
//                   fields; updates already run are not repeated
#include <sys/stat.h>

#include <algorithm>
#include <cerrno>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "mcb.h"

namespace {

int die(const char* what, int rc) {
  std::fprintf(stderr, "mcb_sim: %s failed (%d): %s\n", what, rc, mcb_last_error());
  return 1;
}

bool make_dirs(const std::string& path) {
  std::string cur;
  for (size_t i = 0; i < path.size(); ++i) {
    cur += path[i];
    if ((path[i] == '/' || i + 1 == path.size()) && !cur.empty() && cur != "/") {
      if (mkdir(cur.c_str(), 0755) != 0 && errno != EEXIST) return false;
    }
  }
  return true;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: %s <velocity set> <ID> [options]\n", argv[0]);
    return 1;
  }
  const std::string vs = argv[1], id = argv[2];
  if (vs != "D3Q19" && vs != "D3Q27") {
    std::fprintf(stderr, "mcb_sim: velocity set must be D3Q19 or D3Q27 (f; g is D3Q19)\n");
    return 1;
  }
  int nsteps = 25000, save = 100, scenario = -1, autotune = 0;
  double scale = 1.0;
  unsigned long long seed = 1;
  int storage = -1;
  std::string out = "../bin/" + vs + "/" + id + "/";
  std::string checkpoint, restart;
  std::vector<int> fields = {MCB_FIELD_PHI};
  for (int i = 3; i < argc; ++i) {
    const std::string a = argv[i];
    auto next = [&]() -> const char* {
      if (i + 1 >= argc) {
        std::fprintf(stderr, "mcb_sim: %s needs a value\n", a.c_str());
        std::exit(1);
      }
      return argv[++i];
    };
    if (a == "--steps") nsteps = std::atoi(next());
    else if (a == "--save") save = std::atoi(next());
    else if (a == "--out") out = next();
    else if (a == "--scenario") scenario = std::atoi(next());
    else if (a == "--scale") scale = std::atof(next());
    else if (a == "--seed") seed = std::strtoull(next(), nullptr, 10);
    else if (a == "--autotune") autotune = 1;
    else if (a == "--checkpoint") checkpoint = next();
    else if (a == "--restart") restart = next();
    else if (a == "--fields") {
      static const char* const names[] = {"phi", "rho", "ux", "uy", "uz", "pres"};
      fields.clear();
      std::string list = next();
      size_t pos = 0;
      while (pos <= list.size()) {
        const size_t end = std::min(list.find(',', pos), list.size());
        const std::string name = list.substr(pos, end - pos);
        int k = -1;
        for (int j = 0; j < 6; ++j)
          if (name == names[j]) k = j;
        if (k < 0) {
          std::fprintf(stderr, "mcb_sim: unknown field %s\n", name.c_str());
          return 1;
        }
        fields.push_back(k);
        pos = end + 1;
      }
    }
    else if (a == "--storage") {
      const std::string s = next();
      storage = s == "f32" ? MCB_STORE_F32 : s == "f16" ? MCB_STORE_F16
              : s == "bf16" ? MCB_STORE_BF16 : -2;
      if (storage == -2) {
        std::fprintf(stderr, "mcb_sim: unknown storage %s\n", s.c_str());
        return 1;
      }
    } else if (a == "1") {
      // pipeline.sh passes a third argument that the reference ignores.
    } else {
      std::fprintf(stderr, "mcb_sim: unknown option %s\n", a.c_str());
      return 1;
    }
  }
  if (nsteps < 0 || save < 0) {
    std::fprintf(stderr, "mcb_sim: --steps and --save must be >= 0\n");
    return 1;
  }
  if (!out.empty() && out.back() != '/') out += '/';
  if (!make_dirs(out)) {
    std::fprintf(stderr, "mcb_sim: cannot create %s\n", out.c_str());
    return 1;
  }

  mcb_config cfg;
  std::vector<float> phi, ux, uy, uz;
  int rc;
  if (scenario < 0) {
    mcb_config_default(&cfg);
    phi.resize(static_cast<size_t>(cfg.nx) * cfg.ny * cfg.nz);
    rc = mcb_fill_phi_reference(cfg.nx, cfg.ny, cfg.nz, 20.0f, 3.0f, phi.data());
    if (rc) return die("mcb_fill_phi_reference", rc);
  } else {
    rc = mcb_workload(scenario, 0, seed, scale, &cfg, nullptr, nullptr, nullptr, nullptr);
    if (rc) return die("mcb_workload", rc);
    const size_t n = static_cast<size_t>(cfg.nx) * cfg.ny * cfg.nz;
    phi.resize(n);
    ux.resize(n);
    uy.resize(n);
    uz.resize(n);
    rc = mcb_workload(scenario, 0, seed, scale, &cfg, phi.data(), ux.data(), uy.data(),
                      uz.data());
    if (rc) return die("mcb_workload", rc);
  }
  if (storage >= 0) cfg.storage = storage;
  cfg.velocity_set = vs == "D3Q27" ? 27 : 19;

  mcb_handle* h = nullptr;
  if ((rc = mcb_create(&cfg, &h))) return die("mcb_create", rc);
  if ((rc = mcb_set_fields(h, phi.data(), ux.empty() ? nullptr : ux.data(),
                           uy.empty() ? nullptr : uy.data(), uz.empty() ? nullptr : uz.data())))
    return die("mcb_set_fields", rc);
  int done = -1;  // last update run
  if (!restart.empty()) {
    if ((rc = mcb_checkpoint_load(h, restart.c_str()))) return die("mcb_checkpoint_load", rc);
    if ((rc = mcb_get_update(h, &done))) return die("mcb_get_update", rc);
    std::printf("restart: %s after update %d\n", restart.c_str(), done);
  }
  if (autotune) {
    int v = 0, zc = 0;
    double ml = 0;
    if ((rc = mcb_autotune(h, 20, &v, &zc, &ml))) return die("mcb_autotune", rc);
    std::printf("autotune: variant %d, zchunk %d, %.1f MLUPS\n", v, zc, ml);
  }
  if ((rc = mcb_write_info(h, out.c_str(), id.c_str(), vs.c_str(), save, nsteps, 0.0)))
    return die("mcb_write_info", rc);

  double device_ms = 0.0;
  const auto t0 = std::chrono::steady_clock::now();
  const int first_update = done + 1;
  auto advance = [&](int target) -> int {
    const int n = target - done;
    if (n <= 0) return 0;
    int r = mcb_step(h, n);
    if (r) return r;
    float ms = 0.f;
    if ((r = mcb_last_step_ms(h, &ms))) return r;
    device_ms += ms;
    done = target;
    return 0;
  };
  // First dump point after a restart: the next multiple of save past the restored update.
  int s0 = 0;
  if (done >= 0) s0 = save > 0 ? std::min((done / save + 1) * save, nsteps) : nsteps;
  for (int s = s0; s <= nsteps && done < nsteps;) {
    if ((rc = advance(s))) return die("mcb_step", rc);
    if (save > 0 && s % save == 0) {
      for (int k : fields)
        if ((rc = mcb_dump_field(h, out.c_str(), id.c_str(), k, s)))
          return die("mcb_dump_field", rc);
    }
    if (s == nsteps) break;
    const int nxt = save > 0 ? (s / save + 1) * save : nsteps;
    s = nxt < nsteps ? nxt : nsteps;
  }
  const double wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  const double cells = static_cast<double>(cfg.nx) * cfg.ny * cfg.nz;
  const double updates = static_cast<double>(nsteps + 1 - first_update);
  const double mlups_dev = device_ms > 0 ? cells * updates / (device_ms * 1e-3) / 1e6 : 0.0;
  const double mlups_wall = wall > 0 ? cells * updates / wall / 1e6 : 0.0;
  mcb_diag d;
  rc = mcb_diagnostics(h, &d);
  if (rc && rc != MCB_ERR_NUMERIC) return die("mcb_diagnostics", rc);
  if ((rc = mcb_write_info(h, out.c_str(), id.c_str(), vs.c_str(), save, nsteps, mlups_dev)))
    return die("mcb_write_info", rc);
  if (!checkpoint.empty() && (rc = mcb_checkpoint_save(h, checkpoint.c_str())))
    return die("mcb_checkpoint_save", rc);
  std::printf("updates %d  cells %.0f  device %.3f s  %.1f MLUPS (device)  %.1f MLUPS (wall)\n",
              static_cast<int>(updates), cells, device_ms * 1e-3, mlups_dev, mlups_wall);
  std::printf("mass %.12e  kinetic %.6e  umax %.6e  dp %.6e  finite %d\n", d.mass, d.kinetic,
              d.umax, d.dp, d.finite);
  mcb_destroy(h);
  return d.finite ? 0 : 2;
}
