"""Host-side checks of the C ABI that need no GPU: exported symbols, configuration
defaults and validation, initial-field generators, and the dump/info file format."""
import ctypes
import importlib.util
import re
from pathlib import Path

import numpy as np
import pytest

import mcb

from conftest import REFERENCE_POST, REPO


def _header_functions():
    text = (REPO / "include" / "mcb.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mcb_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(built):
    names = _header_functions()
    assert len(names) >= 30
    L = ctypes.CDLL(str(mcb.LIB_PATH))
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert sorted(mcb.EXPORTS) == names
    assert L.mcb_abi_version() == 4


def test_config_default_is_the_reference_case(built):
    c = mcb.default_config()
    assert (c.nx, c.ny, c.nz) == (64, 64, 256)  # src/var.cu:3-4
    assert c.tau == pytest.approx(0.505)  # src/var.cu:21
    assert c.sigma == pytest.approx(0.1)  # src/var.cu:25
    assert c.sharp_c == pytest.approx(0.45)  # src/var.cu:24
    assert c.bc == mcb.BC_REF and c.storage == mcb.STORE_F32 and c.tau_g == 1.0


@pytest.mark.parametrize("field,value,needle", [
    ("nx", 2, "below 4"), ("tau", 0.4, "tau must"), ("tau_g", 0.5, "tau_g must"),
    ("bc", 7, "boundary"), ("storage", 9, "storage"), ("width", 0.0, "width"),
    ("variant", 99, "variant"), ("zchunk", -17, "zchunk"), ("velocity_set", 15, "velocity_set"),
    ("rho_in", 0.0, "rho_in")])
def test_invalid_configs_are_rejected_before_touching_the_gpu(built, field, value, needle):
    c = mcb.default_config(bc=mcb.BC_PERIODIC, tau_g=1.0)
    setattr(c, field, value)
    with pytest.raises(mcb.McbError) as e:
        mcb.Solver(c)
    assert e.value.code == mcb.ERR_INVALID
    assert needle in str(e.value)


def test_reference_mode_requires_full_g_relaxation(built):
    c = mcb.default_config(tau_g=0.8)
    with pytest.raises(mcb.McbError, match="tau_g must be 1"):
        mcb.Solver(c)


def test_oversized_case_is_rejected(built):
    c = mcb.default_config(nx=2048, ny=2048, nz=1024, bc=mcb.BC_PERIODIC)
    with pytest.raises(mcb.McbError, match="2\\^31"):
        mcb.Solver(c)


def test_fill_phi_reference_is_init_phase(built):
    """initPhase (src/init.cu:27-49) in float32: centred tanh bubble, shell left at 0."""
    nx, ny, nz, r, w = 20, 16, 24, 5.0, 3.0
    got = mcb.fill_phi_reference(nx, ny, nz, r, w)
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    f32 = np.float32
    dx = i.astype(f32) - f32(nx) * f32(0.5)
    dy = j.astype(f32) - f32(ny) * f32(0.5)
    dz = k.astype(f32) - f32(nz) * f32(0.5)
    ri = np.sqrt(dx * dx + dy * dy + dz * dz)
    want = f32(0.5) + f32(0.5) * np.tanh(f32(2.0) * (f32(r) - ri) / f32(w))
    shell = (i == 0) | (i == nx - 1) | (j == 0) | (j == ny - 1) | (k == 0) | (k == nz - 1)
    want[shell] = 0
    assert np.max(np.abs(got - want)) <= 2e-7


def test_workloads_are_seeded_and_well_formed(built):
    c1, p1, *_ = mcb.workload(3, seed=7, scale=0.25)
    c2, p2, *_ = mcb.workload(3, seed=7, scale=0.25)
    c3, p3, *_ = mcb.workload(3, seed=8, scale=0.25)
    assert np.array_equal(p1, p2) and not np.array_equal(p1, p3)
    assert (c1.nx, c1.ny, c1.nz) == (64, 64, 64) and c1.bc == mcb.BC_PERIODIC
    assert 0.0 <= p1.min() and p1.max() <= 1.0
    c, phi, ux, uy, uz = mcb.workload(3, seed=7, scale=0.25)
    assert 0.5e-4 < ux.std() < 2e-4  # N(0, 1e-4) velocity noise
    c, phi, *_ = mcb.workload(2, seed=1, scale=0.25)
    assert (c.nx, c.ny, c.nz) == (32, 32, 64) and c.bc == mcb.BC_WALLS_Z
    assert c.gravity == pytest.approx(1e-5)
    cases = [mcb.workload(4, case_index=i, seed=3, fields=False)[0] for i in range(64)]
    edges = {c.nx for c in cases}
    assert edges <= {32, 48, 64, 80, 96} and len(edges) >= 4
    assert all(c.storage == mcb.STORE_F16 and 0.55 <= c.tau <= 1.0 for c in cases)
    c5, *_ = mcb.workload(5, fields=False)
    assert (c5.nx, c5.nz, c5.storage) == (512, 512, mcb.STORE_F16)


def _load_file_treat():
    path = REFERENCE_POST / "fileTreat.py"
    if not path.exists():
        pytest.skip("the reference's post/ scripts are not on this machine")
    spec = importlib.util.spec_from_file_location("fileTreat_ref", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_dump_and_info_round_trip_through_post_file_treat(built, tmp_path):
    """The files the solver writes are read back by the reference's post/fileTreat.py."""
    ft = _load_file_treat()
    nx, ny, nz = 6, 5, 7
    d = str(tmp_path) + "/"
    mcb.write_info_file(d, "007", "D3Q19", nx, ny, nz, 0.8, umax=1e-3, save_every=100,
                        nsteps=200)
    rng = np.random.default_rng(0)
    fields = {s: rng.random((nz, ny, nx), dtype=np.float32) for s in (0, 100, 200)}
    for s, a in fields.items():
        mcb.write_phi_file(d, "007", "phi", s, a)
    assert sorted(p.name for p in tmp_path.iterdir())[0] == "007_info.txt"
    info = ft.getSimInfo(d)
    assert (info["NX"], info["NY"], info["NZ"], info["NZ_TOTAL"]) == (nx, ny, nz, nz)
    assert info["Prc"] == "float" and info["ID"] == "007" and info["Nsteps"] == 200
    assert info["Tau"] == pytest.approx(0.8) and info["Umax"] == pytest.approx(1e-3)
    assert ft.getMacrSteps(d) == [0, 100, 200]
    for s, a in fields.items():
        got = ft.getMacrsFromStep(s, d)["phi"]  # (x, y, z) after fileTreat's swapaxes
        assert np.array_equal(got, np.swapaxes(a, 0, 2))


def test_extra_field_dumps_are_told_apart_by_post_file_treat(built, tmp_path):
    """With the dumped names added to __macr_names__ (post/fileTreat.py:8), the reader
    matches each file to its field by substring; "pres" is not a substring of another
    name, where "p" would be of "phi"."""
    ft = _load_file_treat()
    names = ["phi", "rho", "ux", "uy", "uz", "pres"]
    nx, ny, nz = 4, 3, 5
    d = str(tmp_path) + "/"
    mcb.write_info_file(d, "009", "D3Q19", nx, ny, nz, 0.7, nsteps=10)
    rng = np.random.default_rng(1)
    data = {k: rng.random((nz, ny, nx), dtype=np.float32) for k in names}
    for k, a in data.items():
        mcb.write_phi_file(d, "009", k, 10, a)
    ft.__macr_names__ = names
    got = ft.getMacrsFromStep(10, d)
    assert sorted(got) == sorted(names)
    for k in names:
        assert np.array_equal(got[k], np.swapaxes(data[k], 0, 2)), k


def test_writers_report_io_errors(built, tmp_path):
    with pytest.raises(mcb.McbError) as e:
        mcb.write_phi_file(str(tmp_path / "missing") + "/", "x", "phi", 0, np.zeros(4))
    assert e.value.code == mcb.ERR_IO
