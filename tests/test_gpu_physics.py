"""Physics known-answers of the CUDA solver, and its 16-bit storage against the FP64 oracle.

The static bubble is the first benchmark config: 64^3 periodic, R 12 at the domain centre,
W 4, tau 0.8, sigma 0.1, tau_g 0.8, 2000 updates. It checks:
  - the Laplace law dp = 2 sigma / R, with R the radius of the phi > 1/2 volume;
  - exact phi-mass conservation;
  - FP16/BF16 storage against the FP64 oracle: Laplace dp within 2 %; max phi error <= 1e-3
    for FP16 and <= 5e-3 for BF16.
The precision-study rerun is a 64^3 periodic box with 4 bubbles and velocity noise. It
compares every storage with the oracle in phi, u and p after 200 and 1000 updates.
"""
import json
import math
import os

import numpy as np
import pytest

import mcb
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

STORAGES = {"f32": mcb.STORE_F32, "f16": mcb.STORE_F16, "bf16": mcb.STORE_BF16}
RESULTS = os.environ.get("MCB_PHYSICS_RESULTS")  # optional JSON dump of the measured numbers


def _run_gpu(cfg, fields, steps, storage):
    cfg.storage = storage
    with mcb.Solver(cfg) as s:
        s.set_fields(*fields)
        s.step(1)
        m0 = s.diagnostics()["mass_q30"]
        s.step(steps - 1)
        d = s.diagnostics()
        out = {k: s.get(k).astype(np.float64) for k in ("phi", "ux", "uy", "uz", "p")}
    return out, d, m0


def _run_oracle(cfg, fields, steps):
    o = Oracle.from_config(cfg)
    o.set_fields(*fields)
    o.step(steps)
    return {k: o.get(k) for k in ("phi", "ux", "uy", "uz", "p")}, o.diagnostics()


def _dump(name, data):
    if RESULTS:
        path = f"{RESULTS}_{name}.json"
        with open(path, "w") as fp:
            json.dump(data, fp, indent=1)


def test_laplace_law_and_16bit_storage_on_the_static_bubble():
    cfg, phi, ux, uy, uz = mcb.workload(1)
    fields = (phi, ux, uy, uz)
    steps = 2000
    ref, dref = _run_oracle(cfg, fields, steps)
    r_ref = (3 * dref["vol_half"] / (4 * math.pi)) ** (1 / 3)
    report = {"oracle": {"dp": dref["dp"], "R_half": r_ref,
                         "laplace_err": dref["dp"] * r_ref / (2 * cfg.sigma) - 1}}
    for name, st in STORAGES.items():
        g, d, m0 = _run_gpu(cfg, fields, steps, st)
        r = (3 * d["vol_half"] / (4 * math.pi)) ** (1 / 3)
        report[name] = {
            "dp": d["dp"], "R_half": r,
            "laplace_err": d["dp"] * r / (2 * cfg.sigma) - 1,
            "dp_err_vs_oracle": d["dp"] / dref["dp"] - 1,
            "max_phi_err": float(np.max(np.abs(g["phi"] - ref["phi"]))),
            "max_u_err": float(max(np.max(np.abs(g[k] - ref[k])) for k in ("ux", "uy", "uz"))),
            "max_p_err": float(np.max(np.abs(g["p"] - ref["p"]))),
            "mass_drift_q30": int(d["mass_q30"] - m0),
        }
    _dump("laplace", report)
    print(json.dumps(report))
    # Bounds: FP32 follows FP64 closely. FP16 meets the 1e-3 phi and 2 % Laplace targets.
    # BF16 (8-bit mantissa) meets the Laplace target at a looser phi bound.
    phi_bound = {"f32": 1e-4, "f16": 1e-3, "bf16": 5e-3}
    for name, rep in report.items():
        if name == "oracle":
            continue
        assert rep["mass_drift_q30"] == 0, name
        assert abs(rep["dp_err_vs_oracle"]) <= 0.02, (name, rep)
        assert abs(rep["laplace_err"]) <= 0.02, (name, rep)
        assert rep["max_phi_err"] <= phi_bound[name], (name, rep)


def test_precision_study_rerun_against_the_oracle():
    """The bounds apply at 200 updates. Later, the flow amplifies rounding: the FP32 and FP64
    oracles alone part by 3e-3 in phi by update 1000. The 1000-update errors are reported
    beside, not bounded."""
    cfg, phi, ux, uy, uz = mcb.workload(6, seed=3)
    fields = (phi, ux, uy, uz)
    report = {}
    for steps in (200, 1000):
        ref, dref = _run_oracle(cfg, fields, steps)
        for name, st in STORAGES.items():
            g, d, m0 = _run_gpu(cfg, fields, steps, st)
            report[f"{name}@{steps}"] = {
                "max_phi_err": float(np.max(np.abs(g["phi"] - ref["phi"]))),
                "max_u_err": float(max(np.max(np.abs(g[k] - ref[k]))
                                       for k in ("ux", "uy", "uz"))),
                "max_p_err": float(np.max(np.abs(g["p"] - ref["p"]))),
                "mass_drift_q30": int(d["mass_q30"] - m0),
                "mass_rel_vs_oracle": d["mass"] / dref["mass"] - 1,
            }
    _dump("precision", report)
    print(json.dumps(report))
    for k, rep in report.items():
        assert rep["mass_drift_q30"] == 0, k
    assert report["f32@200"]["max_phi_err"] <= 1e-4, report
    assert report["f16@200"]["max_phi_err"] <= 1e-3, report
    assert report["bf16@200"]["max_phi_err"] <= 5e-3, report
    assert report["f16@200"]["max_u_err"] <= 1e-4, report


def test_command_line_driver_writes_reference_style_output(tmp_path):
    """mcb_sim keeps the reference's argv (<velocity set> <ID>) and output files."""
    import subprocess

    exe = mcb.LIB_PATH.parent / "mcb_sim"
    out = str(tmp_path) + "/"
    r = subprocess.run([str(exe), "D3Q19", "042", "--scenario", "1", "--scale", "0.25",
                        "--steps", "20", "--save", "10", "--out", out],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    names = sorted(p.name for p in tmp_path.iterdir())
    assert names == ["042_info.txt", "042_phi000000.bin", "042_phi000010.bin",
                     "042_phi000020.bin"]
    n = 16 ** 3
    for nm in names[1:]:
        a = np.fromfile(tmp_path / nm, np.float32)
        assert a.size == n and np.all(np.isfinite(a)) and 0.3 < a.max() <= 1.1
    info = (tmp_path / "042_info.txt").read_text()
    assert "NX: 16" in info and "Precision: float" in info and "MLUPS:" in info


def test_command_line_restart_continues_bitwise(tmp_path):
    """A run stopped after update 10 with --checkpoint and resumed with --restart dumps the
    same update-20 fields, bit for bit, as the uninterrupted run."""
    import subprocess

    exe = mcb.LIB_PATH.parent / "mcb_sim"
    base = [str(exe), "D3Q19", "007", "--scenario", "2", "--scale", "0.125", "--save", "10",
            "--fields", "phi,rho,uz,pres"]
    ck = str(tmp_path / "s.ckpt")
    runs = {"whole": ["--steps", "20"], "first": ["--steps", "10", "--checkpoint", ck],
            "rest": ["--steps", "20", "--restart", ck]}
    for name, extra in runs.items():
        (tmp_path / name).mkdir()
        r = subprocess.run(base + extra + ["--out", str(tmp_path / name) + "/"],
                           capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, (name, r.stdout + r.stderr)
    rest = sorted(p.name for p in (tmp_path / "rest").iterdir())
    assert rest == ["007_info.txt", "007_phi000020.bin", "007_pres000020.bin",
                    "007_rho000020.bin", "007_uz000020.bin"]
    for nm in rest[1:]:
        assert (tmp_path / "rest" / nm).read_bytes() == (tmp_path / "whole" / nm).read_bytes()
    rho = np.fromfile(tmp_path / "whole" / "007_rho000020.bin", np.float32)
    pres = np.fromfile(tmp_path / "whole" / "007_pres000020.bin", np.float32)
    np.testing.assert_allclose(pres, rho / 3, rtol=1e-6)
