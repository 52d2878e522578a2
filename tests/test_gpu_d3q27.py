"""D3Q27 for f (src/var.cu:33-35, 47-52) on the GPU, against the FP64 oracle's D3Q27 update.

The reference builds D3Q27 tables but leaves its moments on D3Q19 index sums
(src/lbm.cu:174-218), so there is no reference run to compare with: the oracle restates
the update with D3Q27 f and moments from their definitions. g and the phi stencils stay
D3Q19, so phi mass stays exact.
"""
import numpy as np
import pytest

import mcb
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

FIELDS = ("phi", "rho", "ux", "uy", "uz")
TOL = {"phi": 2e-5, "rho": 2e-5, "ux": 2e-6, "uy": 2e-6, "uz": 2e-6}


def case(bc, n=(24, 20, 28), tau_g=1.0, gravity=0.0, noise=0.0, seed=0):
    nx, ny, nz = n
    cfg = mcb.default_config(nx=nx, ny=ny, nz=nz, bc=bc, tau=0.7, tau_g=tau_g, sigma=0.05,
                             width=4.0, sharp_c=0.0, gravity=gravity, velocity_set=27)
    if bc == mcb.BC_REF:
        cfg.tau_g = 1.0
        phi = mcb.fill_phi_bubbles(nx, ny, nz, bc, 4.0, [(nx * 0.47, ny * 0.52, nz * 0.49, 6.0)])
    else:
        phi = mcb.fill_phi_bubbles(nx, ny, nz, bc, 4.0, [(nx * 0.45, ny * 0.5, nz * 0.4, 5.0),
                                                         (nx * 0.8, ny * 0.2, nz * 0.8, 3.0)])
    u = None
    if noise:
        rng = np.random.default_rng(seed)
        u = tuple((noise * rng.standard_normal(phi.shape)).astype(np.float32) for _ in range(3))
    return cfg, phi, u


def run_gpu(cfg, phi, u, steps):
    with mcb.Solver(cfg) as s:
        s.set_fields(phi, *(u if u is not None else (None, None, None)))
        s.step(steps)
        return {k: s.get(k).astype(np.float64) for k in FIELDS}, s.diagnostics()


def run_oracle(cfg, phi, u, steps):
    o = Oracle.from_config(cfg)
    o.set_fields(phi, *(u if u is not None else (None, None, None)))
    o.step(steps)
    out = {k: o.get(k) for k in FIELDS}
    o.close()
    return out


@pytest.mark.parametrize("bc,tau_g,gravity,noise", [
    (mcb.BC_PERIODIC, 1.0, 0.0, 1e-3),
    (mcb.BC_PERIODIC, 0.8, 0.0, 1e-3),
    (mcb.BC_WALLS_Z, 1.0, 1e-4, 0.0),
    (mcb.BC_WALLS_Z, 0.8, 1e-4, 1e-3),
    (mcb.BC_REF, 1.0, 0.0, 0.0),
])
def test_d3q27_f32_matches_fp64_oracle(bc, tau_g, gravity, noise):
    cfg, phi, u = case(bc, tau_g=tau_g, gravity=gravity, noise=noise)
    g, _ = run_gpu(cfg, phi, u, 30)
    o = run_oracle(cfg, phi, u, 30)
    for k, tol in TOL.items():
        d = float(np.max(np.abs(g[k] - o[k])))
        assert d < tol, (k, d)


@pytest.mark.parametrize("storage,tol", [(mcb.STORE_F16, 1e-3), (mcb.STORE_BF16, 2e-3)])
def test_d3q27_16bit_storage_stays_close_to_fp64(storage, tol):
    cfg, phi, u = case(mcb.BC_PERIODIC, n=(32, 32, 32), noise=1e-4)
    o = run_oracle(cfg, phi, u, 200)
    cfg.storage = storage
    g, _ = run_gpu(cfg, phi, u, 200)
    assert np.max(np.abs(g["phi"] - o["phi"])) < tol
    assert np.max(np.abs(g["ux"] - o["ux"])) < 1e-4


@pytest.mark.parametrize("storage", [mcb.STORE_F32, mcb.STORE_F16])
def test_d3q27_keeps_phi_mass_exact_and_restarts_bitwise(tmp_path, storage):
    cfg, phi, u = case(mcb.BC_WALLS_Z, gravity=1e-4, noise=1e-3)
    cfg.storage = storage
    ck = str(tmp_path / "q27.ckpt")
    with mcb.Solver(cfg) as s:
        assert s.schedule[0] == 0
        s.set_fields(phi, *u)
        s.step(1)
        m0 = s.diagnostics()["mass_q30"]
        s.step(40)
        s.checkpoint_save(ck)
        s.step(25)
        assert s.diagnostics()["mass_q30"] == m0
        want = {k: s.get(k) for k in FIELDS}
    with mcb.Solver(cfg) as s2:
        s2.checkpoint_load(ck)
        s2.step(25)
        for k in FIELDS:
            assert np.array_equal(s2.get(k), want[k]), k
    cfg19 = case(mcb.BC_WALLS_Z)[0]
    cfg19.velocity_set = 19
    cfg19.storage = storage
    with mcb.Solver(cfg19) as s3:
        with pytest.raises(mcb.McbError):
            s3.checkpoint_load(ck)


def test_d3q27_shear_wave_decays_at_the_lattice_viscosity():
    """u_x = A sin(2 pi z / 64) in a single phase decays as exp(-nu k^2 t),
    nu = (tau - 1/2) / 3."""
    nx, ny, nz, tau, amp, steps = 8, 8, 64, 0.8, 1e-4, 400
    cfg = mcb.default_config(nx=nx, ny=ny, nz=nz, bc=mcb.BC_PERIODIC, tau=tau, tau_g=1.0,
                             sigma=0.0, width=4.0, sharp_c=0.0, velocity_set=27)
    z = np.arange(nz)
    prof = np.sin(2 * np.pi * z / nz)
    ux = np.broadcast_to((amp * prof)[:, None, None], (nz, ny, nx)).astype(np.float32)
    zero = np.zeros((nz, ny, nx), np.float32)
    with mcb.Solver(cfg) as s:
        s.set_fields(zero, ux, zero, zero)
        s.step(steps + 1)  # fields of update `steps`
        got = s.get("ux")[:, 0, 0].astype(np.float64)
    a = np.dot(got, prof) / np.dot(prof, prof)
    rate = -np.log(a / amp) / steps
    want = (tau - 0.5) / 3 * (2 * np.pi / nz) ** 2
    assert rate == pytest.approx(want, rel=5e-3)


def test_d3q27_batch_matches_single_cases_bitwise():
    cfgs, fields = [], []
    for i, n in enumerate([(24, 20, 28), (16, 24, 20)]):
        c, phi, u = case(mcb.BC_PERIODIC, n=n, noise=1e-3, seed=i)
        cfgs.append(c)
        fields.append((phi, u))
    singles = [run_gpu(c, phi, u, 13)[0] for c, (phi, u) in zip(cfgs, fields)]
    with mcb.Batch(cfgs) as b:
        for i, (phi, u) in enumerate(fields):
            b.set_fields(i, phi, *u)
        b.step(13)
        for i in range(len(cfgs)):
            for k in FIELDS:
                assert np.array_equal(b.get(i, k).astype(np.float64), singles[i][k]), (i, k)
