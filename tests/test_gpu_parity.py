"""Parity of the CUDA solver (through the C ABI) with the FP64 CPU oracle and with the
reference's own kernels, plus its exact invariants. All of these need the GB300."""
import numpy as np
import pytest

import mcb
from oracle.oracle import Oracle, ReferenceKernels, harness_available

pytestmark = pytest.mark.gpu

FIELDS = ("phi", "rho", "ux", "uy", "uz")


def gpu_run(cfg, phi, u=None, steps=10, **over):
    for k, v in over.items():
        setattr(cfg, k, v)
    with mcb.Solver(cfg) as s:
        s.set_fields(phi, *(u if u is not None else (None, None, None)))
        s.step(steps)
        out = {k: s.get(k).astype(np.float64) for k in FIELDS}
        out["diag"] = s.diagnostics()
    return out


def oracle_run(cfg, phi, u=None, steps=10, precision=64):
    o = Oracle.from_config(cfg, precision=precision)
    o.set_fields(phi, *(u if u is not None else (None, None, None)))
    o.step(steps)
    out = {k: o.get(k) for k in FIELDS}
    out["diag"] = o.diagnostics()
    return out


def maxdiff(a, b, k):
    return float(np.max(np.abs(a[k] - b[k])))


def small_case(bc, n=(24, 20, 28), tau_g=1.0, gravity=0.0, noise=0.0, seed=0):
    nx, ny, nz = n
    cfg = mcb.default_config(nx=nx, ny=ny, nz=nz, bc=bc, tau=0.7, tau_g=tau_g, sigma=0.05,
                             width=4.0, sharp_c=0.0, gravity=gravity)
    phi = mcb.fill_phi_bubbles(nx, ny, nz, bc, 4.0, [(nx * 0.45, ny * 0.5, nz * 0.4, 5.0),
                                                     (nx * 0.8, ny * 0.2, nz * 0.8, 3.0)])
    u = None
    if noise:
        rng = np.random.default_rng(seed)
        u = tuple((noise * rng.standard_normal(phi.shape)).astype(np.float32) for _ in range(3))
    return cfg, phi, u


# Max |GPU FP32 - FP64 oracle| after 30 updates on the small cases. The float32 rounding
# of one update is ~1e-7 relative; 30 updates of this dissipative system stay well below
# these bounds.
TOL = {"phi": 2e-5, "rho": 2e-5, "ux": 2e-6, "uy": 2e-6, "uz": 2e-6}


@pytest.mark.parametrize("bc,tau_g,gravity,noise", [
    (mcb.BC_PERIODIC, 1.0, 0.0, 0.0),
    (mcb.BC_PERIODIC, 0.8, 0.0, 1e-3),
    (mcb.BC_PERIODIC, 1.0, 1e-4, 1e-3),
    (mcb.BC_WALLS_Z, 1.0, 0.0, 0.0),
    (mcb.BC_WALLS_Z, 1.0, 1e-4, 0.0),
    (mcb.BC_WALLS_Z, 0.8, 1e-4, 1e-3),
])
def test_f32_matches_fp64_oracle(bc, tau_g, gravity, noise):
    cfg, phi, u = small_case(bc, tau_g=tau_g, gravity=gravity, noise=noise)
    g = gpu_run(cfg, phi, u, steps=30)
    o = oracle_run(cfg, phi, u, steps=30)
    for k, tol in TOL.items():
        assert maxdiff(g, o, k) < tol, (k, maxdiff(g, o, k))


@pytest.mark.parametrize("storage", [mcb.STORE_F32, mcb.STORE_F16, mcb.STORE_BF16])
@pytest.mark.parametrize("bc", [mcb.BC_REF, mcb.BC_PERIODIC, mcb.BC_WALLS_Z])
def test_first_update_reproduces_the_initial_field(bc, storage):
    """phi of update 0 is the sum of the initial populations, i.e. the initial phi. This
    checks the stored-population layout of the init, bounced links included."""
    cfg, phi, u = small_case(bc if bc != mcb.BC_REF else mcb.BC_PERIODIC, noise=1e-3)
    if bc == mcb.BC_REF:
        cfg.bc = mcb.BC_REF
        phi = mcb.fill_phi_bubbles(cfg.nx, cfg.ny, cfg.nz, mcb.BC_REF, 4.0,
                                   [(10.3, 9.6, 12.2, 5.0)])
        u = None
    cfg.storage = storage
    g = gpu_run(cfg, phi, u, steps=1)
    want = phi.astype(np.float64)
    if bc == mcb.BC_REF:  # interior only: the shell shows the zero-gradient copy
        sl = (slice(1, -1),) * 3
        g["phi"], want = g["phi"][sl], want[sl]
    # float32 rounding; 16-bit storage rounds each stored deviation (11 or 8 bits)
    tol = {mcb.STORE_F32: 3e-7, mcb.STORE_F16: 2e-5, mcb.STORE_BF16: 2e-4}[storage]
    assert np.max(np.abs(g["phi"] - want)) < tol


def off_centre_reference_phi(n, r=8.0):
    """Reference-mode bubble whose centre is not a lattice node (shell left at 0)."""
    return mcb.fill_phi_bubbles(n, n, n, mcb.BC_REF, 4.0,
                                [(n / 2 - 0.3, n / 2 + 0.35, n / 2 + 0.45, r)])


def reference_cfg(n):
    cfg, *_ = mcb.workload(0, scale=n / 64, fields=False)  # tau 0.8, sigma 0.1, W 4
    assert (cfg.nx, cfg.bc, cfg.tau_g) == (n, mcb.BC_REF, 1.0)
    return cfg


def test_reference_mode_matches_fp64_oracle():
    n = 32
    cfg = reference_cfg(n)
    phi = off_centre_reference_phi(n)
    g = gpu_run(cfg, phi, steps=100)
    o = oracle_run(cfg, phi, steps=100)
    for k, tol in TOL.items():
        assert maxdiff(g, o, k) < tol, (k, maxdiff(g, o, k))
    # the shell of phi holds the zero-gradient copy, as in the reference's dumps
    assert np.array_equal(g["phi"][0, 1:-1, 1:-1], g["phi"][1, 1:-1, 1:-1])


def test_reference_init_short_horizon_matches_fp64_oracle():
    """The reference's own node-centred bubble (src/init.cu:27-49). Its centre node makes
    the run sensitive to rounding after a few updates, so the horizon is short."""
    n = 32
    cfg = reference_cfg(n)
    phi = mcb.fill_phi_reference(n, n, n, 8.0, 4.0)
    g = gpu_run(cfg, phi, steps=4)
    o = oracle_run(cfg, phi, steps=4)
    for k in FIELDS:
        assert maxdiff(g, o, k) < 2e-6, (k, maxdiff(g, o, k))


def _reference_kernels(cfg, phi, steps):
    n = cfg.nx
    sharp = (cfg.tau_g - 0.5) * 4.0 / cfg.width
    rk = ReferenceKernels(n, n, n, cfg.tau, cfg.sigma, sharp)
    rk.set_phi(phi)
    rk.run(steps)
    out = {k: rk.get(k).astype(np.float64) for k in FIELDS}
    rk.close()
    return out


@pytest.mark.skipif(not harness_available(), reason="reference cubin not built")
@pytest.mark.parametrize("init,steps,tol", [("off_centre", 300, TOL),
                                            ("reference", 4, {k: 2e-6 for k in FIELDS})])
def test_reference_mode_matches_reference_kernels(init, steps, tol):
    """The reference's own kernels (unmodified src/lbm.cu for sm_103a) and the fused solver,
    from the same initial phi, 32^3. The comparison excludes the shell, whose edges the
    reference writes racily (src/lbm.cu:411-424)."""
    n = 32
    cfg = reference_cfg(n)
    phi = off_centre_reference_phi(n) if init == "off_centre" else \
        mcb.fill_phi_reference(n, n, n, 8.0, 4.0)
    ref = _reference_kernels(cfg, phi, steps)
    g = gpu_run(cfg, phi, steps=steps)
    inner = (slice(1, -1),) * 3
    for k in FIELDS:
        d = float(np.max(np.abs(g[k][inner] - ref[k][inner])))
        assert d < tol[k], (k, d)


@pytest.mark.parametrize("storage", [mcb.STORE_F32, mcb.STORE_F16, mcb.STORE_BF16])
@pytest.mark.parametrize("bc", [mcb.BC_PERIODIC, mcb.BC_WALLS_Z])
def test_phi_mass_is_exactly_conserved(storage, bc):
    cfg, phi, u = small_case(bc, tau_g=0.8 if bc == mcb.BC_PERIODIC else 1.0,
                             gravity=1e-4, noise=1e-3)
    cfg.storage = storage
    with mcb.Solver(cfg) as s:
        s.set_fields(phi, *u)
        s.step(1)
        m0 = s.diagnostics()["mass_q30"]
        for _ in range(5):
            s.step(37)
            assert s.diagnostics()["mass_q30"] == m0


@pytest.mark.parametrize("storage,tol", [(mcb.STORE_F16, 1e-3), (mcb.STORE_BF16, 1e-3)])
def test_16bit_storage_stays_close_to_fp64(storage, tol):
    cfg, phi, u = small_case(mcb.BC_PERIODIC, n=(32, 32, 32), noise=1e-4)
    o = oracle_run(cfg, phi, u, steps=200)
    g = gpu_run(cfg, phi, u, steps=200, storage=storage)
    assert maxdiff(g, o, "phi") < tol
    assert maxdiff(g, o, "ux") < 1e-4


def test_tile_variants_graphs_and_chunks_agree_bitwise():
    cfg, phi, u = small_case(mcb.BC_WALLS_Z, n=(40, 36, 30), tau_g=0.8, gravity=1e-4,
                             noise=1e-3)
    # the one-cell tiles against the 32x8 one, the pair variants against each other
    base = {0: gpu_run(cfg, phi, u, steps=41, variant=0, use_graph=0, zchunk=0),
            PAIR: gpu_run(cfg, phi, u, steps=41, variant=PAIR, use_graph=0, zchunk=0)}
    for v in range(mcb.lib().mcb_variant_count()):
        for g in (0, 1):
            for zc in (0, -3, 4, 7):
                r = gpu_run(cfg, phi, u, steps=41, variant=v, use_graph=g, zchunk=zc)
                want = base[PAIR if v in PAIRS else 0]
                for k in FIELDS:
                    assert np.array_equal(r[k], want[k]), (v, g, zc, k)


@pytest.mark.parametrize("storage", [mcb.STORE_F32, mcb.STORE_F16, mcb.STORE_BF16])
@pytest.mark.parametrize("bc", [mcb.BC_PERIODIC, mcb.BC_WALLS_Z, mcb.BC_REF])
def test_tma_collide_matches_the_plain_tile_bitwise(bc, storage):
    """The TMA-staged collide (padded f layout with periodic ghost columns and rows) gives
    the fields of the plain 32x8 tile, bit for bit: partial tiles in x and y, walls,
    periodic images, reference shells."""
    if bc == mcb.BC_REF:
        cfg, u = reference_cfg(32), None
        cfg.nx, cfg.ny, cfg.nz = 48, 40, 36
        phi = mcb.fill_phi_bubbles(48, 40, 36, bc, 4.0, [(20.3, 18.6, 17.1, 8.0)])
    else:
        cfg, phi, u = small_case(bc, n=(48, 20, 30), gravity=1e-4, noise=1e-3)
    cfg.storage = storage
    runs = {}
    for v in (4, 0):
        cfg.variant = v
        with mcb.Solver(cfg) as s:
            s.set_fields(phi, *(u if u is not None else (None, None, None)))
            runs[v] = s.schedule[0]
            s.step(37)
            runs[(v, "f")] = {k: s.get(k) for k in FIELDS}
    assert runs[4] == 4 and runs[0] == 0
    for k in FIELDS:
        assert np.array_equal(runs[(4, "f")][k], runs[(0, "f")][k]), k


def test_tma_collide_is_skipped_where_it_does_not_apply():
    # rows not a multiple of 16 bytes, stored g populations: the plain 32x8 tile runs
    cfg, phi, u = small_case(mcb.BC_PERIODIC, n=(42, 20, 30))
    cfg.variant = 4
    with mcb.Solver(cfg) as s:
        assert s.schedule[0] == 0
    cfg, phi, u = small_case(mcb.BC_PERIODIC, n=(48, 20, 30), tau_g=0.8)
    cfg.variant = 4
    with mcb.Solver(cfg) as s:
        assert s.schedule[0] == 0
    # The default is the two-cells-per-thread tile where it applies and its 64-wide tiles
    # fill x nearly as well as 32-wide ones, else the 32x8 tile. Stored g takes it from 2^18
    # cells (relaxed g: with the L2 prefetch at 16-bit storage, not at all at FP32).
    big = (64, 64, 64)
    for n, tau_g, g_mode, storage, want in (
            ((48, 20, 30), 1.0, mcb.G_AUTO, mcb.STORE_F32, PAIR),
            ((96, 20, 30), 1.0, mcb.G_AUTO, mcb.STORE_F32, 0),
            ((200, 20, 30), 1.0, mcb.G_AUTO, mcb.STORE_F16, PAIR),
            ((48, 20, 30), 1.0, mcb.G_POPULATIONS, mcb.STORE_F16, 0),
            ((48, 20, 30), 0.8, mcb.G_AUTO, mcb.STORE_F16, 0),
            (big, 1.0, mcb.G_POPULATIONS, mcb.STORE_F32, PAIR),
            (big, 1.0, mcb.G_POPULATIONS, mcb.STORE_F16, PAIR),
            (big, 0.8, mcb.G_AUTO, mcb.STORE_F32, 0),
            (big, 0.8, mcb.G_AUTO, mcb.STORE_F16, PAIR + 1),
            (big, 0.8, mcb.G_AUTO, mcb.STORE_BF16, PAIR + 1)):
        cfg = mcb.default_config(nx=n[0], ny=n[1], nz=n[2], bc=mcb.BC_PERIODIC, tau_g=tau_g)
        cfg.g_mode, cfg.storage = g_mode, storage
        with mcb.Solver(cfg) as s:
            assert s.schedule[0] == want, (n, tau_g, g_mode, storage)
    cfg, phi, u = small_case(mcb.BC_PERIODIC, n=(47, 20, 30), tau_g=0.8)
    cfg.storage = mcb.STORE_F16
    with mcb.Solver(cfg) as s:
        assert s.schedule[0] == 0


PAIR = 5  # the two-cells-per-thread tile variants: 5 (three blocks per SM) and 6 (four)
PAIRS = (5, 6)


@pytest.mark.parametrize("storage", [mcb.STORE_F32, mcb.STORE_F16])
def test_work_splits_agree_bitwise_with_equilibrium_g(storage):
    """Balanced ranges (pieces that start mid-column and span columns) and fixed chunks
    give the same fields, bit for bit: every one-cell tile variant, and the pair kernel
    against itself."""
    cfg, phi, u = small_case(mcb.BC_WALLS_Z, n=(72, 40, 96), gravity=1e-4, noise=1e-3)
    cfg.storage = storage
    base = {0: gpu_run(cfg, phi, u, steps=23, variant=0, zchunk=5),
            PAIR: gpu_run(cfg, phi, u, steps=23, variant=PAIR, zchunk=5)}
    for v in range(mcb.lib().mcb_variant_count()):
        for zc in (0, -1, -2, -7, 16):
            r = gpu_run(cfg, phi, u, steps=23, variant=v, zchunk=zc)
            want = base[PAIR if v in PAIRS else 0]
            for k in FIELDS:
                assert np.array_equal(r[k], want[k]), (v, zc, k)


# |pair kernel - one-cell kernel| after 31 updates. FP32: the same arithmetic with the fused
# multiply-adds placed differently and the curvature summed per opposite pair, so the fields
# part at FP32 rounding (the FP32 and FP64 oracles part by 5e-7 in phi and 1e-6 in rho on
# these cases; the reference-mode case, whose shell amplifies rounding, parts by 3.0e-6 in
# phi). 16-bit storage rounds every stored population, and a last-bit difference before the
# rounding moves it by one 16-bit unit: the bounds are those of the storage itself (measured:
# FP16 2.1e-5 in rho and 6.4e-6 in u, BF16 5.1e-5 in u; BF16 in reference mode 1.03e-3 in
# phi, where the shell amplifies those units).
PAIR_TOL = {mcb.STORE_F32: {"phi": 5e-6, "rho": 4e-6, "ux": 4e-7, "uy": 4e-7, "uz": 4e-7},
            mcb.STORE_F16: {"phi": 2e-4, "rho": 2e-4, "ux": 4e-5, "uy": 4e-5, "uz": 4e-5},
            mcb.STORE_BF16: {"phi": 2e-3, "rho": 1e-3, "ux": 2e-4, "uy": 2e-4, "uz": 2e-4}}


@pytest.mark.parametrize("storage", [mcb.STORE_F32, mcb.STORE_F16, mcb.STORE_BF16])
@pytest.mark.parametrize("bc", [mcb.BC_PERIODIC, mcb.BC_WALLS_Z, mcb.BC_REF])
def test_pair_kernel_matches_the_one_cell_kernel(bc, storage):
    """The two-cells-per-thread collide against the one-cell collide: partial tiles in x
    (the 64-cell tile against nx = 72 and 32) and y, walls with gravity, periodic images,
    reference shells (pairs that hold a shell cell and an interior cell)."""
    if bc == mcb.BC_REF:
        # the off-node bubble the reference-kernel parity uses (well conditioned in FP32)
        cfg, phi, u = reference_cfg(32), off_centre_reference_phi(32), None
    else:
        cfg, phi, u = small_case(bc, n=(72, 22, 30), gravity=1e-4, noise=1e-3)
    cfg.storage = storage
    runs = {}
    for v in PAIRS + (0,):
        cfg.variant = v
        with mcb.Solver(cfg) as s:
            s.set_fields(phi, *(u if u is not None else (None, None, None)))
            assert s.schedule[0] == v
            s.step(1)
            m0 = s.diagnostics()["mass_q30"]
            s.step(30)
            runs[v] = {k: s.get(k).astype(np.float64) for k in FIELDS}
            if bc != mcb.BC_REF:
                assert s.diagnostics()["mass_q30"] == m0, v
    for k, tol in PAIR_TOL[storage].items():
        assert maxdiff(runs[PAIR], runs[0], k) < tol, (k, maxdiff(runs[PAIR], runs[0], k))
        assert np.array_equal(runs[5][k], runs[6][k]), k  # the same arithmetic


@pytest.mark.parametrize("storage", [mcb.STORE_F32, mcb.STORE_F16, mcb.STORE_BF16])
@pytest.mark.parametrize("bc", [mcb.BC_PERIODIC, mcb.BC_WALLS_Z])
@pytest.mark.parametrize("g_form", ["relaxed", "populations"])
def test_pair_kernel_with_stored_g_matches_the_one_cell_kernel(g_form, bc, storage):
    """Stored g populations (relaxed with tau_g != 1, or stored at full relaxation): the
    pair kernel on the blocked f layout against the one-cell kernel on the plain one. The
    phi mass stays exact on both."""
    cfg, phi, u = small_case(bc, n=(72, 22, 30), tau_g=0.8 if g_form == "relaxed" else 1.0,
                             gravity=1e-4, noise=1e-3)
    if g_form == "populations":
        cfg.g_mode = mcb.G_POPULATIONS
    cfg.storage = storage
    runs = {}
    for v in PAIRS + (0,):
        cfg.variant = v
        with mcb.Solver(cfg) as s:
            s.set_fields(phi, *u)
            assert s.schedule[0] == v
            s.step(1)
            m0 = s.diagnostics()["mass_q30"]
            s.step(30)
            runs[v] = {k: s.get(k).astype(np.float64) for k in FIELDS}
            assert s.diagnostics()["mass_q30"] == m0, v
    for k, tol in PAIR_TOL[storage].items():
        assert maxdiff(runs[PAIR], runs[0], k) < tol, (k, maxdiff(runs[PAIR], runs[0], k))
        assert np.array_equal(runs[5][k], runs[6][k]), k


@pytest.mark.parametrize("bc,gravity,noise,tau_g", [(mcb.BC_PERIODIC, 0.0, 0.0, 1.0),
                                                    (mcb.BC_PERIODIC, 1e-4, 1e-3, 1.0),
                                                    (mcb.BC_WALLS_Z, 1e-4, 1e-3, 1.0),
                                                    (mcb.BC_PERIODIC, 0.0, 1e-3, 0.8),
                                                    (mcb.BC_WALLS_Z, 1e-4, 1e-3, 0.8)])
def test_pair_kernel_matches_fp64_oracle(bc, gravity, noise, tau_g):
    cfg, phi, u = small_case(bc, gravity=gravity, noise=noise, tau_g=tau_g)
    g = gpu_run(cfg, phi, u, steps=30, variant=PAIR)
    o = oracle_run(cfg, phi, u, steps=30)
    for k, tol in TOL.items():
        assert maxdiff(g, o, k) < tol, (k, maxdiff(g, o, k))


def test_pair_kernel_in_reference_mode_matches_reference_kernels():
    if not harness_available():
        pytest.skip("reference cubin not built")
    n = 32
    cfg = reference_cfg(n)
    phi = off_centre_reference_phi(n)
    ref = _reference_kernels(cfg, phi, 300)
    g = gpu_run(cfg, phi, steps=300, variant=PAIR)
    inner = (slice(1, -1),) * 3
    for k in FIELDS:
        d = float(np.max(np.abs(g[k][inner] - ref[k][inner])))
        assert d < TOL[k], (k, d)


def test_pair_kernel_is_skipped_where_it_does_not_apply():
    # odd nx, stored g populations in reference mode, D3Q27 f, a density ratio: the
    # one-cell 32x8 tile runs
    for over in ({"n": (23, 20, 28)}, {"g_mode": mcb.G_POPULATIONS, "bc": mcb.BC_REF},
                 {"velocity_set": 27}, {"rho_in": 10.0}):
        kw = {k: v for k, v in over.items() if k in ("n", "tau_g")}
        cfg, phi, u = small_case(over.get("bc", mcb.BC_PERIODIC), **kw)
        for k, v in over.items():
            if k not in ("n", "tau_g", "bc"):
                setattr(cfg, k, v)
        cfg.variant = PAIR
        with mcb.Solver(cfg) as s:
            assert s.schedule[0] == 0, over


def test_pair_kernel_with_64bit_plane_offsets_agrees_bitwise(monkeypatch):
    """The pair kernel addresses f per plane with 64-bit offsets, so cases that need 64-bit
    f offsets run it on the blocked layout. MCB_WIDE_OFFSETS=1 forces that path on a small
    case: the fields must not change."""
    cfg, phi, u = small_case(mcb.BC_WALLS_Z, gravity=1e-4, noise=1e-3)
    base = gpu_run(cfg, phi, u, steps=23, variant=PAIR)
    monkeypatch.setenv("MCB_WIDE_OFFSETS", "1")
    cfg.variant = PAIR
    with mcb.Solver(cfg) as s:
        assert s.schedule[0] == PAIR
    wide = gpu_run(cfg, phi, u, steps=23, variant=PAIR)
    for k in FIELDS:
        assert np.array_equal(wide[k], base[k]), k


@pytest.mark.parametrize("velocity_set,ratio,tau_g", [(19, 1.0, 1.0), (19, 1.0, 0.8),
                                                     (27, 1.0, 1.0), (19, 10.0, 1.0)])
def test_64bit_population_offsets_agree_bitwise(monkeypatch, velocity_set, ratio, tau_g):
    """Cases of 2^31 / Q cells or more address f with 64-bit offsets; every other case with
    32-bit ones. MCB_WIDE_OFFSETS=1 forces the 64-bit kernels on a small case: the fields
    must not change."""
    cfg, phi, u = small_case(mcb.BC_WALLS_Z, tau_g=tau_g, gravity=1e-4, noise=1e-3)
    cfg.velocity_set = velocity_set
    cfg.rho_in = ratio
    base = gpu_run(cfg, phi, u, steps=23)
    monkeypatch.setenv("MCB_WIDE_OFFSETS", "1")
    wide = gpu_run(cfg, phi, u, steps=23)
    for k in FIELDS:
        assert np.array_equal(wide[k], base[k]), k


def test_steps_split_across_calls_agree_bitwise():
    cfg, phi, u = small_case(mcb.BC_PERIODIC, tau_g=0.8, noise=1e-3)
    one = gpu_run(cfg, phi, u, steps=50)
    with mcb.Solver(cfg) as s:
        s.set_fields(phi, *u)
        for n in (1, 17, 3, 29):
            s.step(n)
        assert s.update == 49
        for k in FIELDS:
            assert np.array_equal(s.get(k).astype(np.float64), one[k]), k


def test_batch_matches_single_cases_bitwise():
    cases = []
    for i, (n, bc, storage) in enumerate([((16, 16, 16), mcb.BC_PERIODIC, mcb.STORE_F16),
                                          ((24, 20, 28), mcb.BC_WALLS_Z, mcb.STORE_F16),
                                          ((32, 32, 32), mcb.BC_PERIODIC, mcb.STORE_F16)]):
        cfg, phi, u = small_case(bc, n=n, noise=1e-3, seed=i, gravity=1e-4 * (i == 1))
        cfg.storage = storage
        cfg.tau = 0.6 + 0.1 * i
        cases.append((cfg, phi, u))
    with mcb.Batch([c for c, _, _ in cases]) as b:
        for i, (c, phi, u) in enumerate(cases):
            b.set_fields(i, phi, *u)
        b.step(33)
        got = [{k: b.get(i, k) for k in FIELDS} for i in range(len(cases))]
        dg = [b.diagnostics(i) for i in range(len(cases))]
    for i, (c, phi, u) in enumerate(cases):
        single = gpu_run(c, phi, u, steps=33)
        for k in FIELDS:
            assert np.array_equal(got[i][k].astype(np.float64), single[k]), (i, k)
        assert dg[i]["mass_q30"] == single["diag"]["mass_q30"]


@pytest.mark.parametrize("storage", [mcb.STORE_F32, mcb.STORE_F16])
def test_batch_with_relaxed_g_on_the_pair_kernel_matches_single_cases_bitwise(storage):
    """Stored, relaxed g on the pair kernel in one launch over uneven cases: the staged
    pulls and the push address each case's own g and phi arrays."""
    cases = []
    for i, (n, bc) in enumerate([((16, 16, 16), mcb.BC_PERIODIC), ((24, 20, 28), mcb.BC_WALLS_Z),
                                 ((72, 22, 30), mcb.BC_PERIODIC)]):
        cfg, phi, u = small_case(bc, n=n, tau_g=0.8, noise=1e-3, seed=i,
                                 gravity=1e-4 * (i == 1))
        cfg.storage = storage
        cfg.tau = 0.6 + 0.1 * i
        cfg.variant = PAIR
        cases.append((cfg, phi, u))
    with mcb.Batch([c for c, _, _ in cases]) as b:
        for i, (c, phi, u) in enumerate(cases):
            b.set_fields(i, phi, *u)
            assert b.schedule(i)[0] == PAIR
        b.step(33)
        got = [{k: b.get(i, k) for k in FIELDS} for i in range(len(cases))]
        dg = [b.diagnostics(i) for i in range(len(cases))]
    for i, (c, phi, u) in enumerate(cases):
        single = gpu_run(c, phi, u, steps=33)
        for k in FIELDS:
            assert np.array_equal(got[i][k].astype(np.float64), single[k]), (i, k)
        assert dg[i]["mass_q30"] == single["diag"]["mass_q30"]


@pytest.mark.parametrize("storage", [mcb.STORE_F32, mcb.STORE_F16])
@pytest.mark.parametrize("bc", [mcb.BC_PERIODIC, mcb.BC_WALLS_Z, mcb.BC_REF])
def test_equilibrium_g_storage_matches_stored_populations(bc, storage):
    """With tau_g = 1 the solver stores J instead of the 19 g populations (g_mode auto).
    Forcing the populations must give the same update up to rounding, with the phi sum
    exact either way."""
    if bc == mcb.BC_REF:
        cfg = reference_cfg(32)
        phi, u = off_centre_reference_phi(32), None
    else:
        cfg, phi, u = small_case(bc, gravity=1e-4, noise=1e-3)
    cfg.storage = storage
    runs = {}
    for mode in (mcb.G_AUTO, mcb.G_POPULATIONS):
        cfg.g_mode = mode
        with mcb.Solver(cfg) as s:
            s.set_fields(phi, *(u if u is not None else (None, None, None)))
            s.step(1)
            m0 = s.diagnostics()["mass_q30"]
            s.step(59)
            d = s.diagnostics()
            runs[mode] = {k: s.get(k).astype(np.float64) for k in FIELDS}
            if bc != mcb.BC_REF:
                assert d["mass_q30"] == m0, mode
    tol = {mcb.STORE_F32: 1e-5, mcb.STORE_F16: 1e-3}[storage]
    for k in FIELDS:
        assert maxdiff(runs[mcb.G_AUTO], runs[mcb.G_POPULATIONS], k) < tol, k


def test_rest_state_is_a_fixed_point():
    n = 16
    cfg = mcb.default_config(nx=n, ny=n, nz=n, bc=mcb.BC_PERIODIC, tau=0.7, tau_g=1.0,
                             width=4.0, sharp_c=0.0)
    for storage in (mcb.STORE_F32, mcb.STORE_F16, mcb.STORE_BF16):
        g = gpu_run(cfg, np.full((n, n, n), 0.25, np.float32), steps=20, storage=storage)
        assert np.max(np.abs(g["phi"] - 0.25)) < 1e-6
        assert np.max(np.abs(g["rho"] - 1.0)) < 1e-6
        assert np.max(np.abs(g["ux"])) < 1e-7


def test_dump_files_hold_the_phi_field(tmp_path):
    cfg, phi, u = small_case(mcb.BC_PERIODIC)
    d = str(tmp_path) + "/"
    with mcb.Solver(cfg) as s:
        s.set_fields(phi)
        s.step(5)
        s.dump_phi(d, "001", 4)
        s.write_info(d, "001", nsteps=4)
        want = s.get("phi")
    raw = np.fromfile(tmp_path / "001_phi000004.bin", np.float32)
    assert np.array_equal(raw.reshape(want.shape), want)
    text = (tmp_path / "001_info.txt").read_text()
    assert "Precision: float" in text and "NZ_TOTAL: 28" in text


def test_field_dumps_are_read_by_post_file_treat_names(tmp_path):
    cfg, phi, u = small_case(mcb.BC_WALLS_Z, gravity=1e-4)
    d = str(tmp_path) + "/"
    with mcb.Solver(cfg) as s:
        s.set_fields(phi)
        s.step(3)
        for name in ("phi", "rho", "ux", "uy", "uz", "p"):
            s.dump_field(name, d, "002", 2)
        want = {k: s.get(k) for k in ("phi", "rho", "ux", "uy", "uz", "p")}
        with pytest.raises(mcb.McbError):
            lib = mcb.lib()
            mcb._check(lib.mcb_dump_field(s._h, d.encode(), b"002", 9, 2))
    for name, fname in (("phi", "phi"), ("rho", "rho"), ("ux", "ux"), ("uy", "uy"),
                        ("uz", "uz"), ("p", "pres")):
        raw = np.fromfile(tmp_path / f"002_{fname}000002.bin", np.float32)
        assert np.array_equal(raw.reshape(want[name].shape), want[name]), name


@pytest.mark.parametrize("tau_g,storage", [(1.0, mcb.STORE_F32), (0.8, mcb.STORE_F32),
                                           (0.8, mcb.STORE_F16)])
def test_autotune_restores_the_state(tau_g, storage):
    """Stored g keeps four phi buffers (the previous one is the base of the 16-bit g
    decode): every one of them must come back after the trials."""
    cfg, phi, u = small_case(mcb.BC_PERIODIC, n=(32, 32, 32), tau_g=tau_g, noise=1e-3)
    cfg.storage = storage
    ref = gpu_run(cfg, phi, u, steps=20)
    with mcb.Solver(cfg) as s:
        s.set_fields(phi, *u)
        s.step(10)
        before = {k: s.get(k) for k in FIELDS}
        v0 = s.schedule[0]
        v, zc, ml = s.autotune(nsteps=4)
        # zc > 0: fixed chunks; zc < 0: balanced over -zc waves; 0: the default split.
        assert 0 <= v < mcb.lib().mcb_variant_count() and -16 <= zc <= 64 and ml > 0
        assert s.schedule[0] == v
        for k in FIELDS:  # the trials left the fields as they were
            assert np.array_equal(s.get(k), before[k]), k
        s.step(10)
        for k in FIELDS:
            got = s.get(k).astype(np.float64)
            if (v in PAIRS) == (v0 in PAIRS):  # the same arithmetic: bit for bit
                assert np.array_equal(got, ref[k]), k
            else:  # the other collide family: FP32 rounding apart
                assert np.max(np.abs(got - ref[k])) < PAIR_TOL[storage][k], k


@pytest.mark.parametrize("storage", [mcb.STORE_F32, mcb.STORE_F16])
@pytest.mark.parametrize("bc,tau_g,variant", [(mcb.BC_PERIODIC, 1.0, -1),
                                              (mcb.BC_WALLS_Z, 0.8, -1),
                                              (mcb.BC_WALLS_Z, 0.8, PAIR + 1),
                                              (mcb.BC_REF, 1.0, -1)])
def test_checkpoint_restart_continues_bitwise(tmp_path, bc, tau_g, variant, storage):
    """Default tiles, and relaxed g on the pair kernel (blocked f layout, stored g)."""
    if bc == mcb.BC_REF:
        cfg, phi, u = reference_cfg(32), off_centre_reference_phi(32), None
    else:
        cfg, phi, u = small_case(bc, tau_g=tau_g, gravity=1e-4, noise=1e-3)
    cfg.storage = storage
    cfg.variant = variant
    ck = str(tmp_path / "state.ckpt")
    with mcb.Solver(cfg) as s:
        s.set_fields(phi, *(u if u is not None else (None, None, None)))
        s.step(31)
        s.checkpoint_save(ck)
        s.step(23)
        want = {k: s.get(k) for k in FIELDS}
        want_d = s.diagnostics()
    with mcb.Solver(cfg) as s2:
        if variant >= 0:
            assert s2.schedule[0] == variant
        s2.checkpoint_load(ck)
        assert s2.update == 30
        s2.step(23)
        assert s2.update == 53
        for k in FIELDS:
            assert np.array_equal(s2.get(k), want[k]), k
        assert s2.diagnostics()["mass_q30"] == want_d["mass_q30"]
    other = mcb.default_config(nx=cfg.nx + 2, ny=cfg.ny, nz=cfg.nz, bc=cfg.bc, tau=cfg.tau,
                               tau_g=cfg.tau_g, width=4.0, storage=storage)
    with mcb.Solver(other) as s3:
        with pytest.raises(mcb.McbError) as e:
            s3.checkpoint_load(ck)
        assert e.value.code == mcb.ERR_INVALID
    if variant >= 0:  # stored g on the pair kernel's blocked f: not loadable into plain f
        cfg.variant = 0
        with mcb.Solver(cfg) as s4:
            with pytest.raises(mcb.McbError) as e:
                s4.checkpoint_load(ck)
            assert e.value.code == mcb.ERR_INVALID


def test_errors_come_back_as_status_codes():
    cfg, phi, _ = small_case(mcb.BC_PERIODIC)
    with mcb.Solver(cfg) as s:
        with pytest.raises(mcb.McbError) as e:
            s.step(1)  # fields not set
        assert e.value.code == mcb.ERR_STATE
        s.set_fields(phi)
        with pytest.raises(mcb.McbError) as e:
            s.get(17)
        assert e.value.code == mcb.ERR_INVALID
        bad = phi.copy()
        bad[3, 3, 3] = np.nan
        with pytest.raises(mcb.McbError) as e:
            s.set_fields(bad)
        assert e.value.code == mcb.ERR_INVALID


def test_batch_autotune_restores_the_fields_and_matches_single_cases(tmp_path):
    """mcb_batch_autotune picks a tile variant and z chunk per size class. Afterwards the
    batch continues from the fields it had, and each case matches, bit for bit, a single
    handle run with that case's schedule."""
    cases = []
    for i, n in enumerate([(32, 32, 32), (48, 48, 48), (32, 32, 32), (64, 64, 64),
                           (48, 48, 48)]):
        cfg, phi, u = small_case(mcb.BC_PERIODIC, n=n, noise=1e-3, seed=i)
        cfg.storage = mcb.STORE_F16
        cfg.tau = 0.6 + 0.05 * i
        cases.append((cfg, phi, u))
    with mcb.Batch([c for c, _, _ in cases]) as b:
        for i, (c, phi, u) in enumerate(cases):
            b.set_fields(i, phi, *u)
        b.step(3)
        before = [{k: b.get(i, k) for k in FIELDS} for i in range(len(cases))]
        first = [b.schedule(i) for i in range(len(cases))]
        base, tuned = b.autotune(nsteps=4)
        assert tuned >= base > 0
        # the fields are those before the trials
        for i in range(len(cases)):
            for k in FIELDS:
                assert np.array_equal(b.get(i, k), before[i][k]), (i, k)
        sched = [b.schedule(i) for i in range(len(cases))]
        # cases of one size class share a schedule
        assert sched[0] == sched[2] and sched[1] == sched[4], sched
        b.step(20)
        got = [{k: b.get(i, k) for k in FIELDS} for i in range(len(cases))]
    # A single handle replays the case: 3 updates with the batch's first schedule, then (from
    # a checkpoint) 20 with the tuned one.
    for i, (c, phi, u) in enumerate(cases):
        ck = str(tmp_path / f"case{i}.ckpt")
        c.variant, c.zchunk = first[i]
        with mcb.Solver(c) as s:
            s.set_fields(phi, *u)
            s.step(3)
            s.checkpoint_save(ck)
        c.variant, c.zchunk = sched[i]
        with mcb.Solver(c) as s:
            s.checkpoint_load(ck)
            s.step(20)
            for k in FIELDS:
                assert np.array_equal(got[i][k], s.get(k)), (i, first[i], sched[i], k)
