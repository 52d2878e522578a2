"""The CPU oracle on its own: known answers of the restated reference update.

The reference has no tests, fixtures or golden vectors. These checks are the physics
known-answers, plus the algebra the fused kernel relies on.
"""
import numpy as np
import pytest

import mcb
from oracle.oracle import Oracle

CX = np.array([0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0])
CY = np.array([0, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 1, -1])
CZ = np.array([0, 0, 0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, -1, 1, -1, 1])
W = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)
C = np.stack([CX, CY, CZ], 1).astype(np.float64)


def test_d3q19_isotropy_used_by_the_closed_form_moments():
    """The fused kernel replaces the per-population sums of momentiCalc (src/lbm.cu:201-218)
    by closed forms. Those hold because D3Q19 is isotropic to 4th order."""
    rng = np.random.default_rng(3)
    cs2 = 1 / 3
    assert np.isclose(W.sum(), 1)
    assert np.allclose(np.einsum("l,la,lb->ab", W, C, C), cs2 * np.eye(3))
    for _ in range(20):
        rho = 1 + 0.05 * rng.standard_normal()
        u = 0.05 * rng.standard_normal(3)
        F = 1e-3 * rng.standard_normal(3)
        cu = C @ u
        E = 1 + 3 * cu + 4.5 * cu**2 - 1.5 * u @ u
        feq = W * rho * E
        hef = 0.5 * feq * ((C - u) @ F) * 3 / rho
        m_eq = np.einsum("l,la,lb->ab", feq, C, C)
        m_he = np.einsum("l,la,lb->ab", hef, C, C)
        assert np.allclose(m_eq, rho * (cs2 * np.eye(3) + np.outer(u, u)), atol=1e-14)
        want = 0.5 * (np.outer(u, F) + np.outer(F, u)) - 1.5 * (u @ F) * np.outer(u, u)
        assert np.allclose(m_he, want, atol=1e-15)
        # regularised post-collision population in the kernel's pair form
        Pi = rng.standard_normal((3, 3)) * 1e-3
        Pi = Pi + Pi.T
        om = 1 / 0.7
        Q = np.einsum("la,lb->lab", C, C) - cs2 * np.eye(3)
        ref = feq + (1 - om) * W / (2 * cs2**2) * np.einsum("lab,ab->l", Q, Pi) + hef
        R = rho - 1.5 * (u @ F)
        qp = np.einsum("lab,ab->l", Q, Pi)
        mine = W * (E * (R + 1.5 * (C @ F)) + 4.5 * (1 - om) * qp)
        assert np.allclose(mine, ref, atol=1e-15)


def test_isotropic_gradient_is_exact_on_quadratics():
    """gradCalc's stencil (src/lbm.cu:51-63): sum 3 W_l c_l phi(x + c_l) is exact for
    polynomials of degree <= 2."""
    rng = np.random.default_rng(1)
    for _ in range(10):
        a = rng.standard_normal(3)
        B = rng.standard_normal((3, 3))
        B = B + B.T
        x0 = rng.standard_normal(3)
        phi = lambda x: a @ x + 0.5 * x @ B @ x
        grad = sum(3 * W[l] * C[l] * phi(x0 + C[l]) for l in range(19))
        assert np.allclose(grad, a + B @ x0, atol=1e-12)


def _bubble(n, bc=mcb.BC_PERIODIC, r=None, width=4.0):
    return mcb.fill_phi_bubbles(n, n, n, bc, width, [(n / 2, n / 2, n / 2, r or n / 5)])


@pytest.mark.parametrize("phi0", [0.0, 0.3, 1.0])
def test_uniform_rest_state_stays_fixed(built, phi0):
    n = 12
    o = Oracle(n, n, n, mcb.BC_PERIODIC, 0.7, 1.0, 0.1, 0.5)
    o.set_fields(np.full((n, n, n), phi0, np.float32))
    o.step(20)
    assert np.max(np.abs(o.get("phi") - float(np.float32(phi0)))) < 1e-13
    assert np.max(np.abs(o.get("rho") - 1.0)) < 1e-13
    for k in ("ux", "uy", "uz"):
        assert np.max(np.abs(o.get(k))) < 1e-15


@pytest.mark.parametrize("bc,gravity,tau_g", [(mcb.BC_PERIODIC, 0.0, 1.0),
                                              (mcb.BC_PERIODIC, 0.0, 0.8),
                                              (mcb.BC_WALLS_Z, 1e-4, 1.0)])
def test_phi_mass_is_conserved_in_closed_domains(built, bc, gravity, tau_g):
    n = 16
    phi = mcb.fill_phi_bubbles(n, n, n, bc, 4.0, [(8, 8, 6, 4), (4, 3, 12, 2.5)])
    o = Oracle(n, n, n, bc, 0.7, tau_g, 0.05, (tau_g - 0.5), gravity)
    o.set_fields(phi)
    o.step(1)
    m0 = o.diagnostics()["mass"]
    o.step(60)
    m1 = o.diagnostics()["mass"]
    assert abs(m1 - m0) / m0 < 1e-12


def test_centred_bubble_keeps_mirror_symmetry(built):
    """Symmetric in exact arithmetic. Round-off breaks it, and the sharpening flux
    sharp_c phi (1 - phi) n amplifies that wherever |grad phi| is tiny next to phi (1 - phi):
    in the tanh tails and between periodic images. So the check uses a short horizon."""
    n = 24
    phi = _bubble(n, r=6)
    o = Oracle(n, n, n, mcb.BC_PERIODIC, 0.8, 1.0, 0.1, 0.5)
    o.set_fields(phi)
    o.step(6)
    p = o.get("phi")
    ux = o.get("ux")
    # cell i mirrors cell (n - i) mod n about the centre n/2
    idx = (-np.arange(n)) % n
    assert np.max(np.abs(p - p[:, :, idx])) < 1e-12
    assert np.max(np.abs(p - p.transpose(0, 2, 1))) < 1e-12
    assert np.max(np.abs(ux + ux[:, :, idx])) < 1e-13


def test_moving_wall_writes_have_no_effect(built):
    """movingWallBC (src/lbm.cu:430-461) writes f only on shell cells, which nothing reads:
    the solver leaves it out."""
    n = 16
    phi = mcb.fill_phi_reference(n, n, n, 4.0, 4.0)
    runs = []
    for mw in (True, False):
        o = Oracle(n, n, n, mcb.BC_REF, 0.8, 1.0, 0.1, 0.5, moving_wall=mw)
        o.set_fields(phi)
        o.step(25)
        runs.append({k: o.get(k) for k in ("phi", "rho", "ux", "uy", "uz")})
    for k in runs[0]:
        assert np.array_equal(runs[0][k], runs[1][k]), k


def off_centre_reference_phi(n, r=8.0):
    """A reference-mode bubble whose centre is not a lattice node (shell left at 0)."""
    return mcb.fill_phi_bubbles(n, n, n, mcb.BC_REF, 4.0,
                                [(n / 2 - 0.3, n / 2 + 0.35, n / 2 + 0.45, r)])


def test_fp32_restatement_tracks_fp64(built):
    """Off-centre bubble: the float restatement stays within float noise of FP64."""
    n = 32
    res = []
    for prec in (64, 32):
        o = Oracle(n, n, n, mcb.BC_REF, 0.8, 1.0, 0.1, 0.5, precision=prec)
        o.set_fields(off_centre_reference_phi(n))
        o.step(100)
        res.append({k: o.get(k) for k in ("phi", "ux", "rho")})
    assert np.max(np.abs(res[0]["phi"] - res[1]["phi"])) < 5e-5
    assert np.max(np.abs(res[0]["rho"] - res[1]["rho"])) < 1e-5
    assert np.max(np.abs(res[0]["ux"] - res[1]["ux"])) < 2e-6


def test_node_centred_bubble_amplifies_rounding(built):
    """The reference's init (src/init.cu:27-49) centres the bubble on a lattice node.
    There grad phi = 0, and the normal grad phi * rsqrt(max(|grad phi|^2, 1e-9))
    (src/lbm.cu:65-70) scales the rounding noise of grad phi by up to 3e4. Float and double
    therefore part by ~1e-3 at that node within 10 updates. They agree to rounding for
    the first few updates."""
    n = 32
    phi = mcb.fill_phi_reference(n, n, n, 8.0, 4.0)
    runs = [Oracle(n, n, n, mcb.BC_REF, 0.8, 1.0, 0.1, 0.5, precision=p) for p in (64, 32)]
    for o in runs:
        o.set_fields(phi)
        o.step(4)
    assert np.max(np.abs(runs[0].get("phi") - runs[1].get("phi"))) < 2e-6
    for o in runs:
        o.step(6)
    assert np.max(np.abs(runs[0].get("phi") - runs[1].get("phi"))) > 1e-4


# D3Q27 f (src/var.cu:33-35, 47-52): the D3Q19 set followed by the eight corners.
CX27 = np.concatenate([CX, [1, -1, 1, -1, 1, -1, -1, 1]])
CY27 = np.concatenate([CY, [1, -1, 1, -1, -1, 1, 1, -1]])
CZ27 = np.concatenate([CZ, [1, -1, -1, 1, 1, -1, 1, -1]])
W27 = np.array([8 / 27] + [2 / 27] * 6 + [1 / 54] * 12 + [1 / 216] * 8)
C27 = np.stack([CX27, CY27, CZ27], 1).astype(np.float64)


def test_d3q27_tables_are_a_symmetric_isotropic_lattice():
    """Opposite pairs (2k-1, 2k) and 4th-order isotropy: the closed-form moments of the
    fused kernel hold for D3Q27 as for D3Q19."""
    for l in range(1, 27, 2):
        assert np.array_equal(C27[l], -C27[l + 1])
    assert len({tuple(c) for c in C27}) == 27
    cs2 = 1 / 3
    assert np.isclose(W27.sum(), 1)
    assert np.allclose(np.einsum("l,la,lb->ab", W27, C27, C27), cs2 * np.eye(3))
    m4 = np.einsum("l,la,lb,lc,ld->abcd", W27, C27, C27, C27, C27)
    d = np.eye(3)
    want = cs2**2 * (np.einsum("ab,cd->abcd", d, d) + np.einsum("ac,bd->abcd", d, d)
                     + np.einsum("ad,bc->abcd", d, d))
    assert np.allclose(m4, want)
    assert np.allclose(np.einsum("l,la,lb,lc->abc", W27, C27, C27, C27), 0)


def _shear_wave(velocity_set, tau=0.8, n=32, amp=1e-4, steps=300):
    """u_x = amp sin(2 pi z / n) in a single phase; returns the fitted decay rate and the
    analytic nu k^2, nu = cs^2 (tau - 1/2)."""
    nx, ny, nz = 4, 4, n
    z = np.arange(nz)
    ux = np.broadcast_to((amp * np.sin(2 * np.pi * z / nz))[:, None, None],
                         (nz, ny, nx)).astype(np.float32)
    zero = np.zeros((nz, ny, nx), np.float32)
    o = Oracle(nx, ny, nz, mcb.BC_PERIODIC, tau, 1.0, 0.0, 0.0, velocity_set=velocity_set)
    o.set_fields(zero, ux, zero, zero)
    o.step(steps)
    got = o.get("ux")[:, 0, 0]
    o.close()
    # the initial profile is u at update 0's start; steps updates decay it steps times
    a = np.dot(got, np.sin(2 * np.pi * z / nz)) / np.dot(np.sin(2 * np.pi * z / nz),
                                                       np.sin(2 * np.pi * z / nz))
    rate = -np.log(a / amp) / steps
    nu = (tau - 0.5) / 3
    return rate, nu * (2 * np.pi / nz) ** 2


@pytest.mark.parametrize("velocity_set", [19, 27])
def test_shear_wave_decays_at_the_lattice_viscosity(built, velocity_set):
    rate, want = _shear_wave(velocity_set)
    assert rate == pytest.approx(want, rel=2e-3)


def test_d3q27_rest_state_stays_fixed_and_conserves_mass(built):
    n = 12
    phi = np.full((n, n, n), 0.3, np.float32)
    o = Oracle(n, n, n, mcb.BC_PERIODIC, 0.7, 1.0, 0.05, 0.5, velocity_set=27)
    o.set_fields(phi)
    o.step(20)
    assert np.max(np.abs(o.get("ux"))) < 1e-15
    assert np.max(np.abs(o.get("rho") - 1)) < 1e-14
    assert np.max(np.abs(o.get("phi") - np.float32(0.3))) < 1e-14
    o.close()
    cfg, phi, *_ = mcb.workload(1, scale=0.25)  # 16^3 static bubble, periodic
    cfg.velocity_set = 27
    o = Oracle.from_config(cfg)
    o.set_fields(phi)
    o.step(1)
    r0, m0 = o.get("rho").sum(), o.diagnostics()["mass"]
    o.step(40)
    assert o.get("rho").sum() == pytest.approx(r0, rel=1e-12)
    assert o.diagnostics()["mass"] == pytest.approx(m0, rel=1e-12)
    o.close()


def test_density_ratio_oracle_static_bubble_obeys_laplace(built):
    """The oracle's density-ratio model (ratio 10) on a 32^3 periodic static bubble:
    dp = 2 sigma / R within 2 % and conserved phi mass."""
    import math

    n, r, sigma = 32, 8.0, 0.01
    c = (n - 1) / 2
    phi = mcb.fill_phi_bubbles(n, n, n, mcb.BC_PERIODIC, 4.0, [(c, c, c, r)])
    o = Oracle(n, n, n, mcb.BC_PERIODIC, 0.8, 1.0, sigma, 0.5, rho_in=10.0, rho_out=1.0)
    o.set_fields(phi)
    o.step(1)
    m0 = o.diagnostics()["mass"]
    o.step(600)
    d = o.diagnostics()
    o.close()
    rh = (3 * d["vol_half"] / (4 * math.pi)) ** (1 / 3)
    assert abs(d["dp"] * rh / (2 * sigma) - 1) < 0.02
    assert d["mass"] == pytest.approx(m0, rel=1e-12)
    assert d["umax"] < 2e-5


def test_density_ratio_is_refused_in_reference_mode(built):
    c = mcb.default_config(rho_in=10.0, rho_out=1.0)
    with pytest.raises(mcb.McbError, match="density-matched"):
        mcb.Solver(c)


@pytest.mark.parametrize("scale", [0.25, 0.5])
def test_oracle_side_generator_matches_the_solver_workload(built, scale):
    """The benchmark's CPU reference arm builds the rising-bubble field without the solver
    library (oracle/workload_port.py). It must be the field the solver generates."""
    from oracle.workload_port import rising_bubble

    cfg, phi, ux, uy, uz = mcb.workload(2, seed=1, scale=scale)
    mine, p = rising_bubble(seed=1, scale=scale)
    assert mine.shape == phi.shape == (cfg.nz, cfg.ny, cfg.nx)
    assert (p["nx"], p["ny"], p["nz"], p["bc"]) == (cfg.nx, cfg.ny, cfg.nz, cfg.bc)
    assert np.float32(p["tau"]) == cfg.tau and np.float32(p["sigma"]) == cfg.sigma
    assert np.float32(p["gravity"]) == cfg.gravity and p["width"] == cfg.width
    # libm and numpy may round a transcendental differently in the last double bit. That
    # can move a float32 value by one unit in the last place, or, deep in the tanh tail,
    # leave 1e-16 where the other rounds to exactly 0.
    d = np.abs(mine.astype(np.float64) - phi)
    assert d.max() <= 1e-15 or d.max() <= 2 * np.finfo(np.float32).eps, d.max()
    big = np.maximum(mine, phi) > 1e-6
    ulps = np.abs(mine.view(np.int32).astype(np.int64) - phi.view(np.int32).astype(np.int64))
    assert ulps[big].max() <= 2, ulps[big].max()
    assert not ux.any() and not uy.any() and not uz.any()
