"""TEST INFRASTRUCTURE ONLY: build recipe for the checkers under oracle/.

Builds three things:
  _build/liborc.so          the CPU oracle (oracle.cpp), plain g++ with OpenMP.
  _build/libref_harness.so  the driver-API runner of the reference's kernels (ref_harness.cpp).
  _ref/ref_lbm.cubin        the reference's own kernels: src/var.cu, src/init.cu and
                            src/lbm.cu of kreeyto/MULTIC-BUBBLE-CUDA, unmodified, compiled for
                            sm_103a as one translation unit. The flags are those of
                            src/compile.sh:17-20 except the target architecture: -DD3Q19,
                            --restrict. No device link is needed, because the three files
                            form one unit. Built only where the reference checkout exists
                            (REF_ROOT, default /root/reference). Elsewhere the prebuilt cubin
                            is used as is.
"""
from __future__ import annotations

import os
import platform
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
REF_OUT = HERE / "_ref"
DEFAULT_REF_ROOT = Path(os.environ.get("REF_ROOT", "/root/reference"))
CUDA = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))


def _run(cmd):
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"command failed: {' '.join(map(str, cmd))}\n{res.stdout}\n{res.stderr}")


def _stale(out: Path, deps) -> bool:
    return not out.exists() or any(Path(d).stat().st_mtime > out.stat().st_mtime for d in deps)


def oracle_cmd() -> list:
    src = HERE / "oracle.cpp"
    # -ffp-contract=off: the same float/double results on x86_64 and aarch64 hosts.
    return ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
            str(src), "-o", str(BUILD / "liborc.so")]


def harness_cmd() -> list:
    src = HERE / "ref_harness.cpp"
    return ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", f"-I{CUDA / 'include'}", str(src),
            "-o", str(BUILD / "libref_harness.so"), f"-L{CUDA / 'lib64' / 'stubs'}", "-lcuda"]


def cubin_cmd(ref_root: Path) -> list:
    REF_OUT.mkdir(parents=True, exist_ok=True)
    unit = REF_OUT / "ref_all.cu"
    src = ref_root / "src"
    unit.write_text("".join(f'#include "{src / f}"\n' for f in ("var.cu", "init.cu", "lbm.cu")))
    # the unit is deleted after the compile (see build): only the cubin stays
    return [str(CUDA / "bin" / "nvcc"), "-cubin", "-gencode", "arch=compute_103a,code=sm_103a",
            "-DD3Q19", "--restrict", "-O3", str(unit), "-o", str(REF_OUT / "ref_lbm.cubin")]


def build(ref_root: Path | None = None) -> dict:
    """Builds what is stale; returns the paths that exist afterwards."""
    stamp = BUILD / "ARCH"
    if stamp.exists() and stamp.read_text().strip() != platform.machine():
        shutil.rmtree(BUILD)  # built on another host architecture
    BUILD.mkdir(parents=True, exist_ok=True)
    stamp.write_text(platform.machine() + "\n")
    ref_root = Path(ref_root) if ref_root else DEFAULT_REF_ROOT
    jobs = []
    if _stale(BUILD / "liborc.so", [HERE / "oracle.cpp"]):
        jobs.append(oracle_cmd())
    if _stale(BUILD / "libref_harness.so", [HERE / "ref_harness.cpp"]):
        jobs.append(harness_cmd())
    ref_srcs = [ref_root / "src" / f for f in ("var.cu", "init.cu", "lbm.cu", "header.cuh",
                                                "var.cuh", "kernels.cuh")]
    if all(p.exists() for p in ref_srcs) and _stale(REF_OUT / "ref_lbm.cubin", ref_srcs):
        jobs.append(cubin_cmd(ref_root))
    if jobs:
        with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            for f in [ex.submit(_run, j) for j in jobs]:
                f.result()
    unit = REF_OUT / "ref_all.cu"
    if unit.exists():
        unit.unlink()
    return {
        "oracle": BUILD / "liborc.so",
        "harness": BUILD / "libref_harness.so",
        "cubin": REF_OUT / "ref_lbm.cubin" if (REF_OUT / "ref_lbm.cubin").exists() else None,
    }


if __name__ == "__main__":
    print(build())
