"""Builds the solver library (libmcb.so) and the command-line driver in-tree.

Every CUDA translation unit is compiled for sm_103a only. The units are compiled in
parallel, then linked with nvcc. Outputs go to ``mcb/_lib`` next to this file.
"""
from __future__ import annotations

import os
import platform
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent            # .../multic-bubble-cuda_gb300/mcb
ROOT = PKG_DIR.parent                                # .../multic-bubble-cuda_gb300
CSRC = ROOT / "csrc"
CLI = ROOT / "cli"
LIB_DIR = PKG_DIR / "_lib"
OBJ_DIR = LIB_DIR / "obj"
REPO = ROOT.parent
INCLUDE = REPO / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
              "-diag-suppress", "177", f"-I{INCLUDE}"]
CU_SOURCES = ["kern_f32.cu", "kern_f16.cu", "kern_bf16.cu", "kern_common.cu", "api.cu"]
CPP_SOURCES = ["workload.cpp"]


def nvcc() -> str:
    cand = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "bin" / "nvcc"
    return str(cand) if cand.exists() else "nvcc"


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"command failed ({res.returncode}): {' '.join(cmd)}\n"
                           f"{res.stdout}\n{res.stderr}")


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, jobs: int | None = None) -> Path:
    """Compiles libmcb.so and mcb_sim; returns the library path."""
    stamp = LIB_DIR / "ARCH"
    if stamp.exists() and stamp.read_text().strip() != platform.machine():
        shutil.rmtree(LIB_DIR)  # built on another host architecture
    OBJ_DIR.mkdir(parents=True, exist_ok=True)
    stamp.write_text(platform.machine() + "\n")
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))
    cmds, objs = [], []
    for src in CU_SOURCES:
        obj = OBJ_DIR / (src + ".o")
        objs.append(obj)
        if _stale(obj, [CSRC / src] + headers):
            cmds.append([nvcc(), *ARCH, *NVCC_FLAGS, "-c", str(CSRC / src), "-o", str(obj)])
    for src in CPP_SOURCES:
        obj = OBJ_DIR / (src + ".o")
        objs.append(obj)
        if _stale(obj, [CSRC / src] + headers):
            cmds.append(["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", f"-I{INCLUDE}", "-c",
                         str(CSRC / src), "-o", str(obj)])
    if cmds:
        with ThreadPoolExecutor(max_workers=jobs or min(len(cmds), os.cpu_count() or 4)) as ex:
            for f in [ex.submit(_run, c) for c in cmds]:
                f.result()
    lib = LIB_DIR / "libmcb.so"
    if cmds or _stale(lib, objs):
        _run([nvcc(), *ARCH, "-shared", "-o", str(lib), *map(str, objs)])
    exe = LIB_DIR / "mcb_sim"
    cli_src = CLI / "mcb_sim.cpp"
    if cli_src.exists() and _stale(exe, [cli_src, lib]):
        _run(["g++", "-O2", "-std=c++17", "-Wall", f"-I{INCLUDE}", str(cli_src), "-o", str(exe),
              f"-L{LIB_DIR}", "-lmcb", f"-Wl,-rpath,{LIB_DIR}"])
    if verbose:
        print(f"built {lib}", file=sys.stderr)
    return lib


if __name__ == "__main__":
    build(verbose=True)
