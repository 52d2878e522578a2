"""The solver against the reference's own kernels at the static-bubble scale, and the noise
floor of the reference's own stream order.

tests/golden/ref64.npz holds the reference's kernels (unmodified src/lbm.cu, compiled for
sm_103a, run by oracle/ref_harness.cpp on a GB300) after 2000 updates of its own init: 64^3,
the node-centred bubble of src/init.cu:27-49 with R 12 and width 4, tau 0.8, sigma 0.1,
SHARP_C 0.5, frozen shell (src/main.cu:74-190). The solver runs the same case in its
reference mode (MCB_BC_REF) and is compared on the stored plane z = 32 and on whole-field
statistics.

The reference issues collisionFluid and collisionPhase on their own streams, unordered after
momentiCalc (src/main.cu:49-52, 127-141). The harness runs that order too; how far it moves
the reference's own result from the one-stream order is the floor of any parity bound.
"""
import json
import os

import numpy as np
import pytest

import mcb
from oracle.oracle import ReferenceKernels, harness_available

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
FIELDS = ("phi", "rho", "ux", "uy", "uz")
RESULTS = os.environ.get("MCB_PHYSICS_RESULTS")

# Max |solver FP32 - reference FP32| on the plane z = 32 after 2000 updates, shell rows
# excluded (the reference's shell edges race). Both are FP32; the node-centred init turns
# rounding noise at the centre node into ~1e-3 differences within ten updates, which decay
# after that. Measured: phi 1.3e-4, rho 6.0e-6, u 2.7e-7 (the FP64 oracle sits 1.6e-4,
# 7.8e-6 and 3.1e-7 from the reference). The bounds are about 1.5 times that.
PLANE_TOL = {"phi": 2e-4, "rho": 2e-5, "ux": 2e-6, "uy": 2e-6, "uz": 2e-6}


def _stats(a):
    a = a.astype(np.float64)
    return np.array([a.sum(), np.abs(a).max(), (a * a).sum()])


def test_reference_mode_64_cubed_2000_updates_matches_the_reference_kernels():
    g = np.load(os.path.join(GOLDEN, "ref64.npz"))
    meta = json.loads(str(g["meta"]))
    n, upd = meta["n"], meta["updates"]
    cfg, *_ = mcb.workload(0, fields=False)
    assert (cfg.nx, cfg.bc, cfg.tau, cfg.sigma, cfg.width) == (
        n, mcb.BC_REF, np.float32(meta["tau"]), np.float32(meta["sigma"]), meta["width"])
    phi = mcb.fill_phi_reference(n, n, n, meta["r"], meta["width"])
    with mcb.Solver(cfg) as s:
        s.set_fields(phi)
        s.step(upd)
        d = s.diagnostics()
        mine = {k: s.get(k).astype(np.float64) for k in FIELDS}
    report = {}
    for k in FIELDS:
        want = g[f"{k}_plane"].astype(np.float64)
        diff = np.abs(mine[k][32] - want)[1:-1, 1:-1]
        st, st_ref = _stats(mine[k]), g[f"{k}_stats"]
        report[k] = {"plane_max": float(diff.max()),
                     "sum_rel": float(abs(st[0] - st_ref[0]) / max(abs(st_ref[0]), 1e-30)),
                     "maxabs": float(abs(st[1] - st_ref[1]))}
    report["mass_drift_q30_note"] = "reference mode: the shell is open, mass is not invariant"
    report["finite"] = bool(d["finite"])
    if RESULTS:
        with open(f"{RESULTS}_ref64.json", "w") as fp:
            json.dump(report, fp, indent=1)
    print(json.dumps(report))
    for k, tol in PLANE_TOL.items():
        assert report[k]["plane_max"] <= tol, (k, report[k])
        assert report[k]["maxabs"] <= tol, (k, report[k])
    # Whole-field sums. The reference's FP32 populations do not keep the phi sum (its FP32
    # weights sum to 1 + 1.5e-8, src/var.cu:40-45); the solver's integer phi and the FP64
    # oracle do. Both end 3.4e-5 (measured) from the reference's total after 2000 updates.
    assert report["phi"]["sum_rel"] <= 1e-4, report["phi"]
    assert report["rho"]["sum_rel"] <= 1e-6, report["rho"]


@pytest.mark.skipif(not harness_available(), reason="reference cubin not built")
def test_reference_three_stream_order_floor():
    """The reference's own stream order against its one-stream order (same kernels, same
    inputs): the gap, if any, is race noise in the reference itself. The solver's gap to the
    one-stream reference is reported beside it."""
    n, steps = 32, 300
    cfg, *_ = mcb.workload(0, scale=n / 64, fields=False)
    phi = mcb.fill_phi_bubbles(n, n, n, mcb.BC_REF, 4.0,
                               [(n / 2 - 0.3, n / 2 + 0.35, n / 2 + 0.45, 8.0)])
    sharp = (cfg.tau_g - 0.5) * 4.0 / cfg.width
    runs = {}
    for streams in (1, 3, 3):
        rk = ReferenceKernels(n, n, n, cfg.tau, cfg.sigma, sharp)
        rk.set_phi(phi)
        rk.run(steps, streams=streams)
        runs.setdefault(streams, []).append({k: rk.get(k).astype(np.float64) for k in FIELDS})
        rk.close()
    with mcb.Solver(cfg) as s:
        s.set_fields(phi)
        s.step(steps)
        mine = {k: s.get(k).astype(np.float64) for k in FIELDS}
    inner = (slice(1, -1),) * 3
    one = runs[1][0]
    report = {}
    for k in FIELDS:
        report[k] = {
            "three_vs_one_stream": max(float(np.max(np.abs(r[k][inner] - one[k][inner])))
                                       for r in runs[3]),
            "three_vs_three": float(np.max(np.abs(runs[3][0][k][inner] - runs[3][1][k][inner]))),
            "solver_vs_one_stream": float(np.max(np.abs(mine[k][inner] - one[k][inner])))}
    if RESULTS:
        with open(f"{RESULTS}_three_stream.json", "w") as fp:
            json.dump(report, fp, indent=1)
    print(json.dumps(report))
    for k in FIELDS:
        for r in runs[3]:
            assert np.all(np.isfinite(r[k])), k
    # the solver's own parity bound (tests/test_gpu_parity.py) on the same case
    assert report["phi"]["solver_vs_one_stream"] < 2e-5, report
