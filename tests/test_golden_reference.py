"""The CPU oracle against golden outputs of the reference's own kernels.

The fixtures under tests/golden/ come from the unmodified src/var.cu, src/init.cu and
src/lbm.cu of kreeyto/MULTIC-BUBBLE-CUDA. They were compiled for sm_103a and run on a GB300
by tests/golden/make_golden.py. They pin the oracle, which restates those kernels in FP64;
the reference itself has no tests or fixtures.
"""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

import mcb
from oracle.oracle import Oracle

GOLDEN = Path(__file__).resolve().parent / "golden"
FIELDS = ("phi", "rho", "ux", "uy", "uz")
# Max |FP64 oracle - reference (FP32, GPU)| on interior cells of the stored slab. Measured:
# phi 6e-6, rho 1e-6, u 1.5e-7 after 200 updates.
TOL = {"phi": 2e-5, "rho": 3e-6, "ux": 5e-7, "uy": 5e-7, "uz": 5e-7}


def _load(name):
    g = np.load(GOLDEN / f"{name}.npz")
    return g, json.loads(str(g["meta"]))


def _initial_phi(meta):
    n, r, w = meta["n"], meta["r"], meta["width"]
    if meta.get("off_centre"):
        return mcb.fill_phi_bubbles(n, n, n, mcb.BC_REF, w,
                                    [(n / 2 - 0.3, n / 2 + 0.35, n / 2 + 0.45, r)])
    return mcb.fill_phi_reference(n, n, n, r, w)


@pytest.mark.parametrize("name", ["ref32", "ref32c"])
def test_oracle_matches_reference_kernels(built, name):
    g, meta = _load(name)
    phi = _initial_phi(meta)
    assert hashlib.sha256(phi.tobytes()).hexdigest() == str(g["phi0_sha256"])
    n = meta["n"]
    o = Oracle(n, n, n, mcb.BC_REF, meta["tau"], 1.0, meta["sigma"], meta["sharp_c"])
    o.set_fields(phi)
    z0, z1 = meta["slab"]
    done = 0
    for u in meta["updates"]:
        o.step(u + 1 - done)
        done = u + 1
        for k in FIELDS:
            mine = o.get(k)
            want = g[f"u{u}_{k}_slab"].astype(np.float64)
            inner = (slice(None), slice(1, -1), slice(1, -1))  # slab rows off the shell
            d = float(np.max(np.abs(mine[z0:z1][inner] - want[inner])))
            assert d < TOL[k], (u, k, d)
            s_ref = g[f"u{u}_{k}_stats"]
            # whole-field sum, shell included (its racy edges are within float noise): the
            # mean difference per cell stays below half the pointwise bound
            assert abs(mine.sum() - s_ref[0]) <= 0.5 * TOL[k] * n**3, (u, k)
            assert abs(np.abs(mine).max() - s_ref[1]) <= TOL[k], (u, k)


@pytest.mark.slow
def test_oracle_matches_reference_kernels_at_64_cubed_over_2000_updates(built):
    """ref64.npz: the reference's kernels on their own node-centred init at the static-bubble
    scale (64^3, R 12, width 4, tau 0.8, sigma 0.1, SHARP_C 0.5), plane z = 32 and
    whole-field statistics after 2000 updates. The oracle in FP32 follows the reference's
    FP32 arithmetic to rounding over the whole run. Measured: phi 2.0e-5, rho 1.1e-6, u
    1.5e-7 on the plane. (In FP64 the gap is phi 1.6e-4, rho 7.8e-6, u 3.1e-7: the
    node-centred start amplifies FP32 rounding, then it decays.)"""
    g, meta = _load("ref64")
    n = meta["n"]
    phi = mcb.fill_phi_reference(n, n, n, meta["r"], meta["width"])
    assert hashlib.sha256(phi.tobytes()).hexdigest() == str(g["phi0_sha256"])
    o = Oracle(n, n, n, mcb.BC_REF, meta["tau"], 1.0, meta["sigma"], meta["sharp_c"],
               precision=32)
    o.set_fields(phi)
    o.step(meta["updates"])
    tol = {"phi": 6e-5, "rho": 4e-6, "ux": 5e-7, "uy": 5e-7, "uz": 5e-7}
    for k in FIELDS:
        mine = o.get(k)
        want = g[f"{k}_plane"].astype(np.float64)
        d = float(np.max(np.abs(mine[32] - want)[1:-1, 1:-1]))
        assert d < tol[k], (k, d)
        s_ref = g[f"{k}_stats"]
        assert abs(np.abs(mine).max() - s_ref[1]) <= tol[k], k
    for k, rel in (("phi", 1e-5), ("rho", 1e-7)):
        s_ref = g[f"{k}_stats"]
        assert abs(o.get(k).sum() - s_ref[0]) <= rel * abs(s_ref[0]), k
