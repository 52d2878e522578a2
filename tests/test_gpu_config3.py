"""The precision study of the multi-bubble field: its 64^3 crop rerun against the FP64 oracle.

The full field is 256^3 periodic with 32 non-overlapping bubbles, R ~ U[6, 16], velocity
noise N(0, 1e-4), tau 0.6, sigma 0.05, W 4 (mcb_workload scenario 3; the reference hard-codes
one bubble on one grid, src/var.cu:3-4 and src/init.cu:27-49). The oracle cannot run 256^3
for 5000 updates on the host, so a 64^3 crop of that initial field (phi and u) is rerun on
both sides, periodic, with the same parameters: FP32, FP16 and BF16 population storage on
the GPU against the FP64 oracle. The crop is placed where its faces are free of bubbles, so
the periodic seams cut no interface.

The flow amplifies rounding: the FP32 oracle itself parts from the FP64 one as the run goes
on. The errors of every storage are reported and bounded at 200 and 5000 updates as
multiples of that FP32-oracle floor; the phi mass stays exact throughout.
"""
import json
import os

import numpy as np
import pytest

import mcb
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

STORAGES = {"f32": mcb.STORE_F32, "f16": mcb.STORE_F16, "bf16": mcb.STORE_BF16}
RESULTS = os.environ.get("MCB_PHYSICS_RESULTS")
EDGE = 64


def crop_origin(phi, edge=EDGE, tries=3000, seed=7):
    """Seeded search for the crop origin whose six faces stay below phi 1e-3 (no interface
    crosses a periodic seam) and that holds the most bubble volume."""
    n = phi.shape[0]
    rng = np.random.default_rng(seed)
    best, best_vol = None, -1.0
    idx = np.arange(edge)
    for _ in range(tries):
        o = rng.integers(0, n, 3)
        zs, ys, xs = (o[0] + idx) % n, (o[1] + idx) % n, (o[2] + idx) % n
        faces = (phi[zs[0]][np.ix_(ys, xs)], phi[zs[-1]][np.ix_(ys, xs)],
                 phi[np.ix_(zs, ys[[0, -1]], xs)], phi[np.ix_(zs, ys, xs[[0, -1]])])
        if max(float(f.max()) for f in faces) >= 1e-3:
            continue
        vol = float(phi[np.ix_(zs, ys, xs)].sum())
        if vol > best_vol:
            best, best_vol = tuple(int(v) for v in o), vol
    assert best is not None, "no crop with bubble-free faces"
    return best


def cut(a, o, edge=EDGE):
    n = a.shape[0]
    idx = np.arange(edge)
    zs, ys, xs = (o[0] + idx) % n, (o[1] + idx) % n, (o[2] + idx) % n
    return np.ascontiguousarray(a[np.ix_(zs, ys, xs)])


def test_config3_crop_rerun_against_the_oracle():
    cfg3, phi, ux, uy, uz = mcb.workload(3, seed=1)
    assert (cfg3.nx, cfg3.bc, cfg3.tau, cfg3.sigma) == (256, mcb.BC_PERIODIC,
                                                         np.float32(0.6), np.float32(0.05))
    o = crop_origin(phi)
    fields = tuple(cut(a, o) for a in (phi, ux, uy, uz))
    assert fields[0].max() > 0.99  # the crop holds at least one bubble core
    cfg = mcb.default_config(nx=EDGE, ny=EDGE, nz=EDGE, bc=mcb.BC_PERIODIC, tau=cfg3.tau,
                             tau_g=cfg3.tau_g, sigma=cfg3.sigma, width=cfg3.width,
                             sharp_c=cfg3.sharp_c)
    horizons = (200, 5000)
    ref = {}
    for prec in (64, 32):
        orc = Oracle.from_config(cfg, precision=prec)
        orc.set_fields(*fields)
        done = 0
        for h in horizons:
            orc.step(h - done)
            done = h
            ref[(prec, h)] = {k: orc.get(k) for k in ("phi", "ux", "uy", "uz", "p")}
        orc.close()
    report = {"crop_origin_zyx": o, "phi_max": float(fields[0].max())}

    def errs(a, b):
        return {"max_phi_err": float(np.max(np.abs(a["phi"] - b["phi"]))),
                "rms_phi_err": float(np.sqrt(np.mean((a["phi"] - b["phi"]) ** 2))),
                "max_u_err": float(max(np.max(np.abs(a[k] - b[k])) for k in ("ux", "uy", "uz"))),
                "max_p_err": float(np.max(np.abs(a["p"] - b["p"])))}

    for h in horizons:
        report[f"oracle_f32@{h}"] = errs(ref[(32, h)], ref[(64, h)])
    for name, st in STORAGES.items():
        cfg.storage = st
        with mcb.Solver(cfg) as s:
            s.set_fields(*fields)
            s.step(1)
            m0 = s.diagnostics()["mass_q30"]
            done = 1
            for h in horizons:
                s.step(h - done)
                done = h
                g = {k: s.get(k).astype(np.float64) for k in ("phi", "ux", "uy", "uz", "p")}
                e = errs(g, ref[(64, h)])
                e["mass_drift_q30"] = int(s.diagnostics()["mass_q30"] - m0)
                report[f"{name}@{h}"] = e
    if RESULTS:
        with open(f"{RESULTS}_config3_crop.json", "w") as fp:
            json.dump(report, fp, indent=1)
    print(json.dumps(report))
    for name in STORAGES:
        for h in horizons:
            assert report[f"{name}@{h}"]["mass_drift_q30"] == 0, (name, h)
    # This multi-bubble flow amplifies rounding: the FP32 oracle, a faithful FP32 restatement,
    # parts from the FP64 one by 6.5e-4 in phi after 200 updates and 8.5e-3 after 5000
    # (measured). Each storage is bounded against that floor at both horizons. The ratios
    # move with FP32-level changes of the arithmetic (the one-cell and the two-cell collide,
    # measured in phi at 200 and 5000 updates): FP32 1.1 and 1.0, or 0.3 and 0.5; FP16 2.3
    # and 2.9, or 3.9 and 7.0; BF16 5.8 and 11.2, or 7.4 and 15.2.
    mult = {"f32": 1.5, "f16": 10.0, "bf16": 25.0}
    for name, m in mult.items():
        for h in horizons:
            floor = report[f"oracle_f32@{h}"]
            for e in ("max_phi_err", "max_u_err", "max_p_err"):
                assert report[f"{name}@{h}"][e] <= m * floor[e], (name, h, e, report)
