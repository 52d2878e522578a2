"""TEST INFRASTRUCTURE ONLY: ctypes wrappers of the CPU oracle (liborc.so) and of the
reference-kernel harness (libref_harness.so + _ref/ref_lbm.cubin).

Oracle: FP64 (or FP32) restatement of the reference update, src/lbm.cu:5-461 in the order of
src/main.cu:79-178. Harness: the reference's own kernels on the GPU.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ORC_LIB = HERE / "_build" / "liborc.so"
HARNESS_LIB = HERE / "_build" / "libref_harness.so"
CUBIN = HERE / "_ref" / "ref_lbm.cubin"

FIELDS = {"phi": 0, "rho": 1, "ux": 2, "uy": 3, "uz": 4, "p": 5}


class OrcParams(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("bc", C.c_int),
                ("tau", C.c_double), ("tau_g", C.c_double), ("sigma", C.c_double),
                ("sharp_c", C.c_double), ("gravity", C.c_double), ("threads", C.c_int),
                ("moving_wall", C.c_int), ("qf", C.c_int), ("rho_in", C.c_double),
                ("rho_out", C.c_double)]


_orc = None
_FP = C.POINTER(C.c_float)
_DP = C.POINTER(C.c_double)


def _orc_lib():
    global _orc
    if _orc is None:
        if not ORC_LIB.exists():
            raise RuntimeError(f"{ORC_LIB} missing: run oracle/build.py")
        L = C.CDLL(str(ORC_LIB))
        L.orc_create.argtypes = [C.POINTER(OrcParams), C.c_int]
        L.orc_create.restype = C.c_void_p
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_set_fields.argtypes = [C.c_void_p, _FP, _FP, _FP, _FP]
        L.orc_step.argtypes = [C.c_void_p, C.c_int]
        L.orc_get.argtypes = [C.c_void_p, C.c_int, _DP]
        L.orc_diag.argtypes = [C.c_void_p, _DP]
        L.orc_threads_available.restype = C.c_int
        _orc = L
    return _orc


def threads_available() -> int:
    return int(_orc_lib().orc_threads_available())


def sharp_of(cfg) -> float:
    """The solver's sharpening coefficient: sharp_c, or (tau_g - 1/2) * 4 / width."""
    return float(cfg.sharp_c) if cfg.sharp_c > 0 else (float(cfg.tau_g) - 0.5) * 4.0 / float(cfg.width)


class Oracle:
    """CPU restatement of the update. precision 64 (default) or 32."""

    def __init__(self, nx, ny, nz, bc, tau, tau_g, sigma, sharp_c, gravity=0.0,
                 precision=64, threads=None, moving_wall=True, velocity_set=19, rho_in=1.0,
                 rho_out=1.0):
        p = OrcParams(nx, ny, nz, bc, tau, tau_g, sigma, sharp_c, gravity,
                      threads or max(1, os.cpu_count() or 1), int(moving_wall),
                      int(velocity_set), float(rho_in), float(rho_out))
        self._h = _orc_lib().orc_create(C.byref(p), precision)
        if not self._h:
            raise ValueError("orc_create rejected the parameters")
        self.shape = (nz, ny, nx)
        self.n = nx * ny * nz

    @classmethod
    def from_config(cls, cfg, precision=64, threads=None, moving_wall=True):
        # The solver stores tau etc. as float32; the oracle takes those exact values.
        f = lambda v: float(np.float32(v))
        return cls(cfg.nx, cfg.ny, cfg.nz, cfg.bc, f(cfg.tau), f(cfg.tau_g), f(cfg.sigma),
                   f(np.float32(sharp_of(cfg))), f(cfg.gravity), precision, threads, moving_wall,
                   getattr(cfg, "velocity_set", 19) or 19, f(getattr(cfg, "rho_in", 1.0) or 1.0),
                   f(getattr(cfg, "rho_out", 1.0) or 1.0))

    def close(self):
        if self._h:
            _orc_lib().orc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_fields(self, phi, ux=None, uy=None, uz=None):
        def ptr(a):
            if a is None:
                return None
            a = np.ascontiguousarray(a, np.float32).reshape(-1)
            self._keep.append(a)
            return a.ctypes.data_as(_FP)
        self._keep = []
        rc = _orc_lib().orc_set_fields(self._h, ptr(phi), ptr(ux), ptr(uy), ptr(uz))
        self._keep = []
        if rc:
            raise RuntimeError("orc_set_fields failed")

    def step(self, n=1):
        if _orc_lib().orc_step(self._h, n):
            raise RuntimeError("orc_step failed")

    def get(self, field) -> np.ndarray:
        out = np.empty(self.n, np.float64)
        if _orc_lib().orc_get(self._h, FIELDS[field], out.ctypes.data_as(_DP)):
            raise RuntimeError("orc_get failed")
        return out.reshape(self.shape)

    def diagnostics(self) -> dict:
        out = np.zeros(9, np.float64)
        _orc_lib().orc_diag(self._h, out.ctypes.data_as(_DP))
        keys = ["mass", "kinetic", "umax", "rho_in", "rho_out", "dp", "n_in", "n_out", "vol_half"]
        return dict(zip(keys, out.tolist()))


# ---------------------------------------------------------------- reference harness --

_ref = None


def harness_available() -> bool:
    return HARNESS_LIB.exists() and CUBIN.exists()


def _ref_lib():
    global _ref
    if _ref is None:
        L = C.CDLL(str(HARNESS_LIB))
        L.ref_error.restype = C.c_char_p
        L.ref_open.argtypes = [C.c_char_p, C.c_int]
        L.ref_open.restype = C.c_void_p
        L.ref_setup.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_float, C.c_float,
                                C.c_float, C.c_int]
        L.ref_set_phi.argtypes = [C.c_void_p, _FP]
        L.ref_run.argtypes = [C.c_void_p, C.c_int, _FP]
        L.ref_run_streams.argtypes = [C.c_void_p, C.c_int, C.c_int, _FP]
        L.ref_get.argtypes = [C.c_void_p, C.c_int, _FP]
        L.ref_close.argtypes = [C.c_void_p]
        _ref = L
    return _ref


class ReferenceKernels:
    """The reference's CUDA kernels (cubin) driven in their intended order on one stream."""

    def __init__(self, nx, ny, nz, tau, sigma, sharp_c, device=0, moving_wall=True):
        L = _ref_lib()
        self._h = L.ref_open(str(CUBIN).encode(), device)
        if not self._h:
            raise RuntimeError(L.ref_error().decode())
        if L.ref_setup(self._h, nx, ny, nz, tau, sigma, sharp_c, int(moving_wall)):
            raise RuntimeError(L.ref_error().decode())
        self.shape = (nz, ny, nx)
        self.n = nx * ny * nz

    def set_phi(self, phi):
        a = np.ascontiguousarray(phi, np.float32).reshape(-1)
        if _ref_lib().ref_set_phi(self._h, a.ctypes.data_as(_FP)):
            raise RuntimeError(_ref_lib().ref_error().decode())

    def run(self, nsteps, streams=1) -> float:
        """nsteps updates; streams=3 issues the two collisions on their own streams, as the
        reference's main loop does (src/main.cu:127-141). Returns the device milliseconds."""
        ms = C.c_float()
        if _ref_lib().ref_run_streams(self._h, nsteps, streams, C.byref(ms)):
            raise RuntimeError(_ref_lib().ref_error().decode())
        return ms.value

    def get(self, field) -> np.ndarray:
        idx = {"phi": 0, "rho": 1, "ux": 2, "uy": 3, "uz": 4}[field]
        out = np.empty(self.n, np.float32)
        if _ref_lib().ref_get(self._h, idx, out.ctypes.data_as(_FP)):
            raise RuntimeError(_ref_lib().ref_error().decode())
        return out.reshape(self.shape)

    def close(self):
        if self._h:
            _ref_lib().ref_close(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
