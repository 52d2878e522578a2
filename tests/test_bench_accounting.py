"""The algorithmic bytes per lattice update that bench.py divides by the kernel time
(roofline.achieved), per g storage, velocity set and storage precision."""
import importlib.util
import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(REPO / "multic-bubble-cuda_gb300"))
import mcb  # noqa: E402

_spec = importlib.util.spec_from_file_location("bench_under_test", REPO / "bench.py")
bench = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(bench)


def rising_bubble(**over):
    cfg, *_ = mcb.workload(2, seed=1)
    for k, v in over.items():
        setattr(cfg, k, v)
    return cfg


@pytest.mark.parametrize("over,variant,gs,f32,f16", [
    # push: f in and out, phi in, the next phi, the phi after next cleared
    ({}, -1, "push", (0, 164, 164), (0, 88, 88)),
    ({"velocity_set": 27}, -1, "push", (0, 228, 228), (0, 120, 120)),
    # the TMA variant keeps (phi, J) records and their phi kernel
    ({}, bench.TMA_VARIANT, "records", (20, 172, 192), (20, 96, 116)),
    # stored populations: as push, and the 18 moving g written
    ({"g_mode": mcb.G_POPULATIONS}, -1, "populations", (0, 236, 236), (0, 124, 124)),
    # relaxed g: written and read; 16-bit also reads the previous phi
    ({"tau_g": 0.8}, -1, "bgk", (0, 308, 308), (0, 164, 164)),
])
def test_bytes_per_lattice_update(over, variant, gs, f32, f16):
    cfg = rising_bubble(**over)
    assert bench.g_storage(cfg, variant) == gs
    assert bench.bytes_per_lu(cfg, "f32", variant) == f32
    assert bench.bytes_per_lu(cfg, "f16", variant) == f16
    assert bench.bytes_per_lu(cfg, "bf16", variant) == f16


def test_swarm_footprint_fits_the_gpu():
    cells = 512 ** 3
    gb = bench.footprint_bytes(cells, "f16", "push") / 1e9
    assert 16.0 < gb < 17.0  # f ping-pong 10.2 GB, three phi buffers, fields, staging
