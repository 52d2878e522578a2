"""Python binding of the solver's C ABI (include/mcb.h), through ctypes.

The CUDA library ``_lib/libmcb.so`` is the only compute path. Importing this module does
not load it; the first call does, and raises ``McbError`` if the library is missing. There
is no CPU fallback.

Arrays follow the reference's layout (src/header.cuh:20-27): float32, x fastest. Python
returns them as ``(nz, ny, nx)`` arrays, which is how post/fileTreat.py:146-149 reshapes a
dump.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libmcb.so"

OK, ERR_INVALID, ERR_CUDA, ERR_ALLOC, ERR_IO, ERR_STATE, ERR_NUMERIC = range(7)
BC_REF, BC_PERIODIC, BC_WALLS_Z = 0, 1, 2
STORE_F32, STORE_F16, STORE_BF16 = 0, 1, 2
FIELD_PHI, FIELD_RHO, FIELD_UX, FIELD_UY, FIELD_UZ, FIELD_P = range(6)
FIELDS = {"phi": FIELD_PHI, "rho": FIELD_RHO, "ux": FIELD_UX, "uy": FIELD_UY, "uz": FIELD_UZ,
          "p": FIELD_P}
STORAGES = {"f32": STORE_F32, "f16": STORE_F16, "bf16": STORE_BF16}
G_AUTO, G_POPULATIONS = 0, 1

# Every symbol include/mcb.h declares.
EXPORTS = [
    "mcb_last_error", "mcb_abi_version", "mcb_config_default", "mcb_create", "mcb_destroy",
    "mcb_set_fields", "mcb_step", "mcb_synchronize", "mcb_get_field", "mcb_diagnostics",
    "mcb_dump_phi", "mcb_write_info", "mcb_write_phi_file", "mcb_write_info_file",
    "mcb_get_update", "mcb_get_dims", "mcb_last_step_ms", "mcb_step_profiled",
    "mcb_variant_count", "mcb_variant_shape", "mcb_autotune", "mcb_fill_phi_reference",
    "mcb_fill_phi_bubbles", "mcb_workload", "mcb_batch_create", "mcb_batch_destroy",
    "mcb_batch_set_fields", "mcb_batch_step", "mcb_batch_get_field", "mcb_batch_diagnostics",
    "mcb_batch_last_step_ms", "mcb_batch_cells", "mcb_diagnostics_device",
    "mcb_checkpoint_save", "mcb_checkpoint_load", "mcb_dump_field", "mcb_get_schedule",
    "mcb_get_phi_q30", "mcb_batch_autotune", "mcb_batch_get_schedule",
]


class McbError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


class Config(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("bc", C.c_int),
                ("storage", C.c_int), ("tau", C.c_float), ("tau_g", C.c_float),
                ("sigma", C.c_float), ("width", C.c_float), ("sharp_c", C.c_float),
                ("gravity", C.c_float), ("device", C.c_int), ("variant", C.c_int),
                ("zchunk", C.c_int), ("use_graph", C.c_int), ("g_mode", C.c_int),
                ("velocity_set", C.c_int), ("rho_in", C.c_float), ("rho_out", C.c_float)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class Diag(C.Structure):
    _fields_ = [("mass", C.c_double), ("mass_q30", C.c_int64), ("kinetic", C.c_double),
                ("umax", C.c_double), ("rho_in", C.c_double), ("rho_out", C.c_double),
                ("dp", C.c_double), ("n_in", C.c_double), ("n_out", C.c_double),
                ("vol_half", C.c_double), ("phi_min", C.c_double), ("phi_max", C.c_double),
                ("finite", C.c_int), ("update", C.c_int)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class Bubble(C.Structure):
    _fields_ = [("cx", C.c_double), ("cy", C.c_double), ("cz", C.c_double), ("r", C.c_double),
                ("ax", C.c_double), ("ay", C.c_double), ("az", C.c_double)]


_lib = None
_FP = C.POINTER(C.c_float)


def lib() -> C.CDLL:
    """Loads libmcb.so (once). Raises McbError when it has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise McbError(ERR_STATE, f"{LIB_PATH} is missing; run __graft_entry__.build()")
        L = C.CDLL(str(LIB_PATH))
        L.mcb_last_error.restype = C.c_char_p
        vp = C.c_void_p
        sigs = {
            "mcb_config_default": [C.POINTER(Config)],
            "mcb_create": [C.POINTER(Config), C.POINTER(vp)],
            "mcb_destroy": [vp],
            "mcb_set_fields": [vp, _FP, _FP, _FP, _FP],
            "mcb_step": [vp, C.c_int],
            "mcb_synchronize": [vp],
            "mcb_get_field": [vp, C.c_int, _FP],
            "mcb_get_phi_q30": [vp, C.POINTER(C.c_int32)],
            "mcb_diagnostics": [vp, C.POINTER(Diag)],
            "mcb_dump_phi": [vp, C.c_char_p, C.c_char_p, C.c_int],
            "mcb_write_info": [vp, C.c_char_p, C.c_char_p, C.c_char_p, C.c_int, C.c_int,
                               C.c_double],
            "mcb_write_phi_file": [C.c_char_p, C.c_char_p, C.c_char_p, C.c_int, _FP,
                                   C.c_size_t],
            "mcb_write_info_file": [C.c_char_p, C.c_char_p, C.c_char_p, C.c_int, C.c_int,
                                    C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                    C.c_double, C.c_int, C.c_int, C.c_double],
            "mcb_dump_field": [vp, C.c_char_p, C.c_char_p, C.c_int, C.c_int],
            "mcb_get_schedule": [vp, C.POINTER(C.c_int), C.POINTER(C.c_int)],
            "mcb_checkpoint_save": [vp, C.c_char_p],
            "mcb_checkpoint_load": [vp, C.c_char_p],
            "mcb_get_update": [vp, C.POINTER(C.c_int)],
            "mcb_get_dims": [vp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)],
            "mcb_last_step_ms": [vp, _FP],
            "mcb_step_profiled": [vp, C.c_int, _FP, _FP, _FP],
            "mcb_variant_shape": [C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)],
            "mcb_autotune": [vp, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                             C.POINTER(C.c_double)],
            "mcb_fill_phi_reference": [C.c_int, C.c_int, C.c_int, C.c_float, C.c_float, _FP],
            "mcb_fill_phi_bubbles": [C.c_int, C.c_int, C.c_int, C.c_int, C.c_float,
                                     C.POINTER(Bubble), C.c_int, _FP],
            "mcb_workload": [C.c_int, C.c_int, C.c_uint64, C.c_double, C.POINTER(Config), _FP,
                             _FP, _FP, _FP],
            "mcb_batch_create": [C.POINTER(Config), C.c_int, C.POINTER(vp)],
            "mcb_batch_destroy": [vp],
            "mcb_batch_set_fields": [vp, C.c_int, _FP, _FP, _FP, _FP],
            "mcb_batch_step": [vp, C.c_int],
            "mcb_batch_get_field": [vp, C.c_int, C.c_int, _FP],
            "mcb_batch_diagnostics": [vp, C.c_int, C.POINTER(Diag)],
            "mcb_batch_last_step_ms": [vp, _FP],
            "mcb_batch_cells": [vp, C.POINTER(C.c_int64)],
            "mcb_batch_autotune": [vp, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)],
            "mcb_batch_get_schedule": [vp, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)],
            "mcb_diagnostics_device": [vp, vp, vp, vp, vp, vp, C.c_int, C.c_int, C.c_int,
                                       C.c_int, vp, C.POINTER(Diag)],
        }
        for name, args in sigs.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = C.c_int
        L.mcb_variant_count.restype = C.c_int
        L.mcb_abi_version.restype = C.c_int
        _lib = L
    return _lib


def _check(rc: int) -> None:
    if rc != OK:
        raise McbError(rc, lib().mcb_last_error().decode(errors="replace"))


def _fptr(a):
    return None if a is None else a.ctypes.data_as(_FP)


def _as_f32(a, n: int):
    if a is None:
        return None
    a = np.ascontiguousarray(a, dtype=np.float32).reshape(-1)
    if a.size != n:
        raise ValueError(f"expected {n} values, got {a.size}")
    return a


def default_config(**kw) -> Config:
    c = Config()
    _check(lib().mcb_config_default(C.byref(c)))
    for k, v in kw.items():
        if isinstance(v, str) and k == "storage":
            v = STORAGES[v]
        setattr(c, k, v)
    return c


def fill_phi_reference(nx: int, ny: int, nz: int, r: float, width: float) -> np.ndarray:
    out = np.empty(nx * ny * nz, np.float32)
    _check(lib().mcb_fill_phi_reference(nx, ny, nz, r, width, _fptr(out)))
    return out.reshape(nz, ny, nx)


def fill_phi_bubbles(nx, ny, nz, bc, width, bubbles) -> np.ndarray:
    arr = (Bubble * max(1, len(bubbles)))()
    for i, b in enumerate(bubbles):
        vals = list(b) + [1.0] * (7 - len(b))
        arr[i] = Bubble(*vals)
    out = np.empty(nx * ny * nz, np.float32)
    _check(lib().mcb_fill_phi_bubbles(nx, ny, nz, bc, width, arr, len(bubbles), _fptr(out)))
    return out.reshape(nz, ny, nx)


def write_phi_file(directory: str, sim_id: str, name: str, step: int, data) -> None:
    """Raw float32 dump "<dir><id>_<name>%06d.bin" (host data, no GPU)."""
    a = np.ascontiguousarray(data, np.float32).reshape(-1)
    _check(lib().mcb_write_phi_file(directory.encode(), sim_id.encode(), name.encode(), step,
                                    _fptr(a), a.size))


def write_info_file(directory: str, sim_id: str, velocity_set: str, nx: int, ny: int, nz: int,
                    tau: float, umax: float = 0.0, fx: float = 0.0, fy: float = 0.0,
                    fz: float = 0.0, save_every: int = 100, nsteps: int = 0,
                    mlups: float = 0.0) -> None:
    _check(lib().mcb_write_info_file(directory.encode(), sim_id.encode(), velocity_set.encode(),
                                     nx, ny, nz, tau, umax, fx, fy, fz, save_every, nsteps,
                                     mlups))


def diagnostics_device(phi, rho, ux, uy, uz, nx: int, ny: int, nz: int, bc: int,
                       phi_q30=None, stream=None, allow_nonfinite: bool = False) -> dict:
    """mcb_diagnostics_device over caller-owned device arrays, given as raw device
    addresses (ints). The call allocates nothing; see include/mcb.h."""
    d = Diag()
    rc = lib().mcb_diagnostics_device(phi, rho, ux, uy, uz, phi_q30, nx, ny, nz, bc, stream,
                                      C.byref(d))
    if rc != OK and not (allow_nonfinite and rc == ERR_NUMERIC):
        _check(rc)
    return d.as_dict()


def workload(scenario: int, case_index: int = 0, seed: int = 1, scale: float = 1.0,
             fields: bool = True):
    """Seeded scenario: returns (Config, phi, ux, uy, uz) with arrays shaped (nz, ny, nx)."""
    c = Config()
    _check(lib().mcb_workload(scenario, case_index, seed, scale, C.byref(c), None, None, None,
                              None))
    if not fields:
        return c, None, None, None, None
    n = c.nx * c.ny * c.nz
    phi, ux, uy, uz = (np.empty(n, np.float32) for _ in range(4))
    _check(lib().mcb_workload(scenario, case_index, seed, scale, C.byref(c), _fptr(phi),
                              _fptr(ux), _fptr(uy), _fptr(uz)))
    shp = (c.nz, c.ny, c.nx)
    return c, phi.reshape(shp), ux.reshape(shp), uy.reshape(shp), uz.reshape(shp)


class Solver:
    """One case: mcb_create ... mcb_destroy."""

    def __init__(self, cfg: Config):
        self._h = C.c_void_p()
        _check(lib().mcb_create(C.byref(cfg), C.byref(self._h)))
        self.cfg = cfg
        self.shape = (cfg.nz, cfg.ny, cfg.nx)
        self.n = cfg.nx * cfg.ny * cfg.nz

    def close(self) -> None:
        if self._h:
            lib().mcb_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_fields(self, phi, ux=None, uy=None, uz=None) -> None:
        phi = _as_f32(phi, self.n)
        ux, uy, uz = (_as_f32(a, self.n) for a in (ux, uy, uz))
        _check(lib().mcb_set_fields(self._h, _fptr(phi), _fptr(ux), _fptr(uy), _fptr(uz)))

    def step(self, n: int = 1) -> None:
        _check(lib().mcb_step(self._h, n))

    def synchronize(self) -> None:
        _check(lib().mcb_synchronize(self._h))

    def get(self, field: str | int, out: np.ndarray | None = None) -> np.ndarray:
        which = FIELDS[field] if isinstance(field, str) else field
        if out is None:
            out = np.empty(self.n, np.float32)
        _check(lib().mcb_get_field(self._h, which, _fptr(out)))
        return out.reshape(self.shape)

    def get_phi_q30(self) -> np.ndarray:
        """The exact Q2.30 phi of the latest update (int32, 1.0 = 2^30)."""
        out = np.empty(self.n, np.int32)
        _check(lib().mcb_get_phi_q30(self._h, out.ctypes.data_as(C.POINTER(C.c_int32))))
        return out.reshape(self.shape)

    def diagnostics(self, allow_nonfinite: bool = False) -> dict:
        d = Diag()
        rc = lib().mcb_diagnostics(self._h, C.byref(d))
        if rc != OK and not (allow_nonfinite and rc == ERR_NUMERIC):
            _check(rc)
        return d.as_dict()

    def dump_phi(self, directory: str, sim_id: str, step: int) -> None:
        _check(lib().mcb_dump_phi(self._h, directory.encode(), sim_id.encode(), step))

    def dump_field(self, name: str, directory: str, sim_id: str, step: int) -> None:
        """Writes <directory><sim_id>_<name>%06d.bin; name is a FIELDS key ("p" is
        written as "pres")."""
        _check(lib().mcb_dump_field(self._h, directory.encode(), sim_id.encode(),
                                    FIELDS[name], step))

    def write_info(self, directory: str, sim_id: str, velocity_set: str = "D3Q19",
                   save_every: int = 100, nsteps: int = 0, mlups: float = 0.0) -> None:
        _check(lib().mcb_write_info(self._h, directory.encode(), sim_id.encode(),
                                    velocity_set.encode(), save_every, nsteps, mlups))

    @property
    def schedule(self) -> tuple[int, int]:
        """(tile variant, z chunk setting) the handle runs; variant 4 is the TMA collide."""
        v, z = C.c_int(), C.c_int()
        _check(lib().mcb_get_schedule(self._h, C.byref(v), C.byref(z)))
        return v.value, z.value

    def checkpoint_save(self, path: str) -> None:
        _check(lib().mcb_checkpoint_save(self._h, str(path).encode()))

    def checkpoint_load(self, path: str) -> None:
        _check(lib().mcb_checkpoint_load(self._h, str(path).encode()))

    @property
    def update(self) -> int:
        u = C.c_int()
        _check(lib().mcb_get_update(self._h, C.byref(u)))
        return u.value

    def last_step_ms(self) -> float:
        ms = C.c_float()
        _check(lib().mcb_last_step_ms(self._h, C.byref(ms)))
        return ms.value

    def step_profiled(self, n: int):
        """Runs n updates with an event after every kernel; returns
        (total_ms, phi_kernel_ms, collide_kernel_ms)."""
        t, a, b = C.c_float(), C.c_float(), C.c_float()
        _check(lib().mcb_step_profiled(self._h, n, C.byref(t), C.byref(a), C.byref(b)))
        return t.value, a.value, b.value

    def autotune(self, nsteps: int = 20):
        v, z, m = C.c_int(), C.c_int(), C.c_double()
        _check(lib().mcb_autotune(self._h, nsteps, C.byref(v), C.byref(z), C.byref(m)))
        return v.value, z.value, m.value


class Batch:
    """Many independent cases in one set of launches (mcb_batch_*)."""

    def __init__(self, cfgs):
        arr = (Config * len(cfgs))(*cfgs)
        self._h = C.c_void_p()
        _check(lib().mcb_batch_create(arr, len(cfgs), C.byref(self._h)))
        self.cfgs = list(cfgs)

    def close(self) -> None:
        if self._h:
            lib().mcb_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _n(self, i):
        c = self.cfgs[i]
        return c.nx * c.ny * c.nz, (c.nz, c.ny, c.nx)

    def set_fields(self, i, phi, ux=None, uy=None, uz=None) -> None:
        n, _ = self._n(i)
        phi = _as_f32(phi, n)
        ux, uy, uz = (_as_f32(a, n) for a in (ux, uy, uz))
        _check(lib().mcb_batch_set_fields(self._h, i, _fptr(phi), _fptr(ux), _fptr(uy),
                                          _fptr(uz)))

    def step(self, n: int = 1) -> None:
        _check(lib().mcb_batch_step(self._h, n))

    def get(self, i, field) -> np.ndarray:
        n, shp = self._n(i)
        which = FIELDS[field] if isinstance(field, str) else field
        out = np.empty(n, np.float32)
        _check(lib().mcb_batch_get_field(self._h, i, which, _fptr(out)))
        return out.reshape(shp)

    def diagnostics(self, i) -> dict:
        d = Diag()
        _check(lib().mcb_batch_diagnostics(self._h, i, C.byref(d)))
        return d.as_dict()

    def last_step_ms(self) -> float:
        ms = C.c_float()
        _check(lib().mcb_batch_last_step_ms(self._h, C.byref(ms)))
        return ms.value

    @property
    def cells(self) -> int:
        c = C.c_int64()
        _check(lib().mcb_batch_cells(self._h, C.byref(c)))
        return c.value

    def autotune(self, nsteps: int = 20) -> tuple[float, float]:
        """Per-size-class tile choice (mcb_batch_autotune): (untuned, tuned) MLUPS."""
        a, b = C.c_double(), C.c_double()
        _check(lib().mcb_batch_autotune(self._h, nsteps, C.byref(a), C.byref(b)))
        return a.value, b.value

    def schedule(self, i) -> tuple[int, int]:
        """(tile variant, z chunk setting) case i runs."""
        v, z = C.c_int(), C.c_int()
        _check(lib().mcb_batch_get_schedule(self._h, i, C.byref(v), C.byref(z)))
        return v.value, z.value
