"""Generates the golden fixtures of the reference's own kernels (needs the GB300).

The reference (kreeyto/MULTIC-BUBBLE-CUDA) has no tests or golden vectors. These fixtures
are outputs of its unmodified kernels, in one configuration each:
  - src/var.cu, src/init.cu and src/lbm.cu, compiled for sm_103a into oracle/_ref/ref_lbm.cubin;
  - run by oracle/ref_harness.cpp in the order of src/main.cu:79-178, on one stream.
  ref32.npz  32^3, bubble R 8, width 4, tau 0.8, sigma 0.1, SHARP_C 0.5, its centre
             off the lattice nodes at (15.7, 16.35, 16.45): fields after update 0 and after
             update 199, as a central slab z in [12, 20), plus whole-field sums and max-abs
             values. The reference's node-centred init turns rounding noise into ~1e-3
             differences within ten updates (grad phi = 0 at that node). The off-node centre
             keeps two correct implementations within float noise.
  ref32c.npz the reference's node-centred init, the same parameters: updates 0 and 3.
  ref64.npz  64^3, R 12, width 4 (the same parameters): the plane z = 32 after update 1999,
             whole-field statistics, and the reference's device time.
The initial phi is mcb.fill_phi_reference (initPhase's formula with R and width as
parameters); its SHA-256 is stored so a test can check it is unchanged.

Usage (on the GPU machine): python tests/golden/make_golden.py OUT_DIR
"""
import hashlib
import json
import sys
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(REPO))
sys.path.insert(0, str(REPO / "multic-bubble-cuda_gb300"))

import mcb  # noqa: E402
from oracle.oracle import ReferenceKernels  # noqa: E402

FIELDS = ("phi", "rho", "ux", "uy", "uz")
PARAMS = dict(tau=0.8, sigma=0.1, sharp_c=0.5, width=4.0)


def stats(a):
    a = a.astype(np.float64)
    return [float(a.sum()), float(np.abs(a).max()), float((a * a).sum())]


def run(n, r, snaps, off_centre=False):
    if off_centre:
        phi = mcb.fill_phi_bubbles(n, n, n, mcb.BC_REF, PARAMS["width"],
                                   [(n / 2 - 0.3, n / 2 + 0.35, n / 2 + 0.45, r)])
    else:
        phi = mcb.fill_phi_reference(n, n, n, r, PARAMS["width"])
    rk = ReferenceKernels(n, n, n, PARAMS["tau"], PARAMS["sigma"], PARAMS["sharp_c"])
    rk.set_phi(phi)
    done, out, ms_total = 0, {}, 0.0
    for s in snaps:
        ms_total += rk.run(s + 1 - done)
        done = s + 1
        out[s] = {k: rk.get(k) for k in FIELDS}
    rk.close()
    return phi, out, ms_total, done


def main(out_dir):
    out_dir = Path(out_dir)
    out_dir.mkdir(parents=True, exist_ok=True)
    z0, z1 = 12, 20
    for name, off, ups in (("ref32", True, [0, 199]), ("ref32c", False, [0, 3])):
        phi, snaps, _, _ = run(32, 8.0, ups, off_centre=off)
        data = {"phi0_sha256": np.array(hashlib.sha256(phi.tobytes()).hexdigest())}
        meta = {"n": 32, "r": 8.0, **PARAMS, "slab": [z0, z1], "updates": ups,
                "off_centre": off}
        for s, fields in snaps.items():
            for k, a in fields.items():
                data[f"u{s}_{k}_slab"] = a[z0:z1].copy()
                data[f"u{s}_{k}_stats"] = np.array(stats(a))
        data["meta"] = np.array(json.dumps(meta))
        np.savez_compressed(out_dir / f"{name}.npz", **data)

    phi, snaps, ms, done = run(64, 12.0, [1999])
    f = snaps[1999]
    data = {"phi0_sha256": np.array(hashlib.sha256(phi.tobytes()).hexdigest())}
    for k, a in f.items():
        data[f"{k}_plane"] = a[32].copy()
        data[f"{k}_stats"] = np.array(stats(a))
    meta = {"n": 64, "r": 12.0, **PARAMS, "updates": done, "device_ms": ms,
            "mlups": 64 ** 3 * done / (ms * 1e-3) / 1e6}
    data["meta"] = np.array(json.dumps(meta))
    np.savez_compressed(out_dir / "ref64.npz", **data)
    print(json.dumps(meta))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else Path(__file__).resolve().parent)
