"""Benchmark of the fused phase-field LBM update on GB300 (one JSON line on rank 0).

Workload: the rising perturbed bubble:
  - 128x128x256 cells, periodic in x and y, bounce-back walls in z;
  - gravity 1e-5, R 16 at z 48, spherical-harmonic modes l = 2..6;
  - tau 0.7, sigma 0.05, W 4;
  - FP32 storage, seeded synthetic initial field.
A step is one lattice update of the whole lattice. Inputs exceed L2: the f populations one
update reads and writes hold 638 MB.

  value     MLUPS with the state resident in HBM: cells * K / device time of K updates as
            the library runs them (CUDA-graph replay), CUDA events on the solver's stream,
            max over ranks. Before the timed region: W warm-up updates and 34 untimed
            updates that capture the graphs. A second pass of K updates with an event after
            every kernel gives the per-kernel times of the roofline.
  e2e       the same metric through the C ABI with host buffers, timed on the host:
            upload of the initial fields from pinned memory, K updates, and a phi read-back
            every 100 updates (the reference's dump cadence, src/main.cu:184-189).
  roofline  the fused collide kernel: algorithmic bytes per launch / average launch time,
            against the measured HBM copy bandwidth.
  cpu_baseline  the FP64 oracle (a restatement of the reference update) on the host cores.

--impl reference times the reference path on the host cores, on the same full-size workload.
The reference has no CPU implementation, so that path is the oracle port; its initial field
comes from the oracle-side generator (oracle/workload_port.py), so that arm loads no solver
code. --gpus N > 1 runs N independent replicas,
one per GPU; the path has no exchange step between cases.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO))
sys.path.insert(0, str(REPO / "multic-bubble-cuda_gb300"))

METRIC = "MLUPS and % HBM roofline; FP16-store vs FP32 at fixed Laplace-law error"
SCENARIO, SEED = 2, 1
TMA_VARIANT = 4
# Population storage: the arithmetic is FP32 whatever the storage ("dtype" of the line).
STORAGE_WORDS = {"f32": "FP32", "f16": "FP16 deviation-form", "bf16": "BF16 deviation-form"}


def g_storage(cfg, variant: int = -1) -> str:
    """How the phase field crosses an update.
      push         g at equilibrium (tau_g = 1, the default): the collide kernel adds each
                   cell's integer populations into the next phi; no g is stored
      records      the same g, with a 16-byte (P, J) record per cell and the phi kernel
                   (the TMA-staged collide)
      populations  g stored (MCB_G_POPULATIONS at tau_g = 1) and pushed into the next phi
      bgk          g stored and relaxed with tau_g != 1 (pulled and stored), pushed likewise"""
    import mcb

    if cfg.tau_g != 1.0:
        return "bgk"
    if cfg.g_mode == mcb.G_POPULATIONS:
        return "populations"
    return "records" if variant == TMA_VARIANT else "push"


def bytes_per_lu(cfg, storage: str, variant: int = -1) -> tuple[int, int, int]:
    """(phi kernel, collide kernel, whole update) algorithmic bytes per lattice update:
    each array a kernel reads or writes, once per cell.
      push         collide: f in and out (Q populations), phi in, the next phi (integer
                   atomics into L2, counted once), the phi buffer after next cleared (4 B)
      records      phi kernel: the record in, phi out; collide: f in and out, phi in, record out
      populations  collide: as push, and the 18 moving g out
      bgk          collide: as push, the 18 moving g in and out, and with 16-bit storage the
                   previous phi in (the base of the deviation form)"""
    pb = 4 if storage == "f32" else 2
    q = 27 if cfg.velocity_set == 27 else 19
    f = 2 * q * pb
    push = f + 4 + 4 + 4
    gs = g_storage(cfg, variant)
    if gs == "push":
        ph, col = 0, push
    elif gs == "records":
        ph, col = 16 + 4, f + 4 + 16
    elif gs == "populations":
        ph, col = 0, push + 18 * pb
    else:
        ph, col = 0, push + 2 * 18 * pb + (4 if storage != "f32" else 0)
    return ph, col, ph + col


def footprint_bytes(cells: int, storage: str, gs: str, q: int = 19) -> int:
    """Device bytes of one solver handle: f ping-pong, g state, phi buffers, macros,
    host-upload staging."""
    pb = 4 if storage == "f32" else 2
    g = {"push": 3 * cells * 4, "records": cells * 16 + 2 * cells * 4}.get(
        gs, 2 * cells * 18 * pb + cells * 4 + 4 * cells * 4)
    return 2 * cells * q * pb + g + cells * 5 * 4 + cells * 4 * 4


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return ws, rank, local


def init_dist(ws, backend):
    if ws <= 1:
        return None
    import torch.distributed as dist

    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group(backend=backend)
    return dist


def reduce_max(dist, value: float, device=None) -> float:
    """Max over ranks (identity without a process group)."""
    if dist is None:
        return value
    import torch

    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


def peaks():
    p = REPO / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class Clocks:
    """nvidia-smi samples of the SM clock and throttle reasons during a timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        self.out = ""
        if self.proc:
            time.sleep(0.2)
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out, _ = self.proc.communicate()

    def summary(self):
        rows = [r.split(",") for r in (self.out or "").strip().splitlines() if r.count(",") >= 8]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in rows for n, v in zip(names, r[5:9]) if "Active" in v
                          and "Not" not in v})
        loaded = sorted(sm)[len(sm) // 2:] if sm else []
        return {"sm_mhz": statistics.median(loaded) if loaded else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons, "samples": len(rows)}


SCALE = 1.0
G_POPULATIONS = False
VARIANT, ZCHUNK = -1, 0


def make_solver(storage: str, device: int, tau_g: float | None = None):
    import mcb

    cfg, phi, ux, uy, uz = mcb.workload(SCENARIO, seed=SEED, scale=SCALE)
    cfg.storage = mcb.STORAGES[storage]
    cfg.device = device
    if G_POPULATIONS:
        cfg.g_mode = mcb.G_POPULATIONS
    if tau_g is not None:
        cfg.tau_g = tau_g
    cfg.variant, cfg.zchunk = VARIANT, ZCHUNK
    s = mcb.Solver(cfg)
    return s, cfg, (phi, ux, uy, uz)


def pinned_like(a):
    import torch

    t = torch.empty(a.size, dtype=torch.float32, pin_memory=True)
    v = t.numpy()
    v[:] = a.reshape(-1)
    return t, v


PAIR_VARIANTS = (5, 6)  # the two-cells-per-thread collide (k_collide_pair)
KERNEL_OF = {}  # (storage, tau_g) -> name of the collide kernel the device leg ran


def collide_name(variant: int) -> str:
    return "k_collide_pair" if variant in PAIR_VARIANTS else "k_collide"


GRAPH_PREP = 2 * 16 + 2  # untimed updates that capture both graph parities of 16 updates


def device_run(storage, device, steps, warmup, dist, tau_g=None):
    """Device-resident timing. The timed region is K updates as the library runs them
    (graph replay, CUDA events on the solver's stream); a second pass of K updates with an
    event after every kernel gives the per-kernel times of the roofline."""
    s, cfg, fields = make_solver(storage, device, tau_g)
    KERNEL_OF[(storage, tau_g)] = collide_name(s.schedule[0])
    s.set_fields(*fields)
    s.step(warmup)
    s.step(GRAPH_PREP)
    s.synchronize()
    barrier(dist)
    s.step(steps)
    s.synchronize()
    total = s.last_step_ms()
    barrier(dist)
    _, t_phi, t_col = s.step_profiled(steps)
    s.synchronize()
    d = s.diagnostics(allow_nonfinite=True)
    s.close()
    return cfg, total, t_phi, t_col, d


def e2e_run(device, steps, save=100):
    """Host-timed run through the C ABI with host buffers."""
    import mcb

    cfg, phi, ux, uy, uz = mcb.workload(SCENARIO, seed=SEED)
    cfg.device = device
    s = mcb.Solver(cfg)
    keep = [pinned_like(a) for a in (phi, ux, uy, uz)]
    host = [v for _, v in keep]
    out_t, out = pinned_like(np.zeros(s.n, np.float32))
    # warm the graphs and the copy path once (not timed)
    s.set_fields(*host)
    s.step(2 * 16 + 2)
    s.get("phi", out)
    s.synchronize()
    t0 = time.perf_counter()
    s.set_fields(*host)
    done, reads = 0, 0
    while done < steps:
        n = min(save, steps - done)
        s.step(n)
        done += n
        s.get("phi", out)
        reads += 1
    t1 = time.perf_counter()
    s.close()
    cells = cfg.nx * cfg.ny * cfg.nz
    return {"value": cells * steps / (t1 - t0) / 1e6, "unit": "MLUPS",
            "h2d_bytes_per_step": 4 * 4 * cells / steps,
            "d2h_bytes_per_step": 4 * cells * reads / steps,
            "steps": steps,
            "note": f"H2D of phi,u from pinned host once; D2H of phi every {save} updates"}


def reference_cuda_run(device, steps):
    """The reference's own kernels (unmodified src/lbm.cu, sm_103a cubin) on the same GPU, at
    the same cell count (128x128x256, its frozen-shell mode: it has no walls or gravity)."""
    from oracle.oracle import ReferenceKernels, harness_available
    import mcb

    if not harness_available():
        return {"unavailable": "reference cubin not present (built only where the reference "
                               "checkout exists)"}
    nx, ny, nz = 128, 128, 256
    phi = mcb.fill_phi_reference(nx, ny, nz, 16.0, 4.0)
    rk = ReferenceKernels(nx, ny, nz, 0.7, 0.05, 0.5, device=device)
    rk.set_phi(phi)
    rk.run(5)
    ms = rk.run(steps)
    rk.close()
    return {"value": nx * ny * nz * steps / (ms * 1e-3) / 1e6, "unit": "MLUPS",
            "config": "128x128x256 frozen-shell mode, one stream, 10 launches per update",
            "steps": steps}


def storage_leg(device, steps, warmup, storage, tau_g=None):
    """One device leg of the bench workload: MLUPS and the collide kernel's roofline at the
    given storage (and g relaxation time)."""
    cfg, total, t_phi, t_col, d = device_run(storage, device, steps, warmup, None, tau_g)
    cells = cfg.nx * cfg.ny * cfg.nz
    hbm, peak_kind = peaks()
    _, col_b, upd_b = bytes_per_lu(cfg, storage)
    col_s = t_col * 1e-3 / steps
    return {"storage": storage, "tau_g": cfg.tau_g, "g_storage": g_storage(cfg),
            "kernel": KERNEL_OF[(storage, tau_g)],
            "value": cells * steps / (total * 1e-3) / 1e6, "unit": "MLUPS", "steps": steps,
            "kernel_ms": {"phi_stage": t_phi / steps, "k_collide": t_col / steps},
            "roofline": {"bytes_per_lu": col_b, "achieved": col_b * cells / col_s / 1e9,
                         "peak": hbm, "unit": "GB/s",
                         "frac": col_b * cells / col_s / 1e9 / hbm,
                         "peak_kind": f"{peak_kind} HBM copy bandwidth",
                         "update_bytes_per_lu": upd_b},
            "finite": bool(d["finite"])}


def reference_mode_run(device, steps, nx=128, ny=128, nz=256, tau=0.7, sigma=0.05, r=16.0,
                       width=4.0, sharp_c=None):
    """The solver in the reference's frozen-shell mode (MCB_BC_REF) on the reference
    kernels' own setting: one centred bubble (initPhase's formula), tau_g = 1."""
    import mcb

    cfg = mcb.default_config(nx=nx, ny=ny, nz=nz, bc=mcb.BC_REF, tau=tau, tau_g=1.0,
                             sigma=sigma, width=width, device=device,
                             sharp_c=sharp_c if sharp_c is not None else 0.0)
    phi = mcb.fill_phi_reference(nx, ny, nz, r, width)
    cells = nx * ny * nz
    with mcb.Solver(cfg) as s:
        s.set_fields(phi)
        s.step(34)
        total, _, t_col = s.step_profiled(steps)
    return {"value": cells * steps / (total * 1e-3) / 1e6, "unit": "MLUPS", "steps": steps,
            "config": f"{nx}x{ny}x{nz} frozen-shell mode, tau {tau}, sigma {sigma}, "
                      f"R {r}, W {width}, FP32",
            "k_collide_ms": t_col / steps}


def reference_cuda_stock(device, steps, nx=64, ny=64, nz=256, tau=0.505, sigma=0.1,
                         sharp_c=0.45, r=20.0, width=3.0, label="stock constants"):
    """The reference's own kernels at the reference's stock setting: 64x64x256, tau 0.505,
    sigma 0.1, SHARP_C 0.45 (src/var.cu:3-25), R 20 and width 3 (src/init.cu:39,46); or at
    another size and setting (the static bubble: 64^3, tau 0.8, sigma 0.1, SHARP_C 0.5, R 12,
    width 4)."""
    from oracle.oracle import ReferenceKernels, harness_available
    import mcb

    if not harness_available():
        return {"unavailable": "reference cubin not present"}
    phi = mcb.fill_phi_reference(nx, ny, nz, r, width)
    rk = ReferenceKernels(nx, ny, nz, tau, sigma, sharp_c, device=device)
    rk.set_phi(phi)
    rk.run(5)
    ms = rk.run(steps)
    rk.close()
    return {"value": nx * ny * nz * steps / (ms * 1e-3) / 1e6, "unit": "MLUPS",
            "config": f"{nx}x{ny}x{nz} {label}, one stream, 10 launches per update",
            "steps": steps}


CONFIG3_UPDATES = 5000


def config3_run(device, updates=CONFIG3_UPDATES):
    """The precision study as configured: 256^3 periodic, 32 bubbles R ~ U[6, 16], velocity
    noise 1e-4, tau 0.6, sigma 0.05, W 4, run for the full number of updates with FP32,
    FP16 and BF16 population storage. Reports device MLUPS and the exact phi-mass drift of
    each, and how far the 16-bit runs end from the FP32 run. The errors against the FP64
    oracle come from the 64^3 crop rerun in the GPU tests."""
    import mcb

    cfg, phi, ux, uy, uz = mcb.workload(3, seed=SEED)
    cfg.device = device
    cells = cfg.nx * cfg.ny * cfg.nz
    out, last = {}, {}
    for st in ("f32", "f16", "bf16"):
        cfg.storage = mcb.STORAGES[st]
        with mcb.Solver(cfg) as s:
            s.set_fields(phi, ux, uy, uz)
            s.step(1)
            m0 = s.diagnostics()["mass_q30"]
            s.step(updates - 1)
            ms = s.last_step_ms()
            d = s.diagnostics(allow_nonfinite=True)
            last[st] = {k: s.get(k) for k in ("phi", "ux", "uy", "uz")}
        out[st] = {"mlups": cells * (updates - 1) / (ms * 1e-3) / 1e6,
                   "mass_drift_q30": int(d["mass_q30"] - m0), "finite": bool(d["finite"]),
                   "kinetic": d["kinetic"]}
    for st in ("f16", "bf16"):
        out[st]["max_phi_diff_vs_f32"] = float(np.max(np.abs(last[st]["phi"] - last["f32"]["phi"])))
        out[st]["max_u_diff_vs_f32"] = float(max(np.max(np.abs(last[st][k] - last["f32"][k]))
                                                 for k in ("ux", "uy", "uz")))
    out["cells"] = cells
    out["updates"] = updates
    out["ratio_f16_vs_f32"] = out["f16"]["mlups"] / out["f32"]["mlups"]
    out["ratio_bf16_vs_f32"] = out["bf16"]["mlups"] / out["f32"]["mlups"]
    return out


def laplace_run(device, updates=2000):
    """The static bubble (64^3 periodic, R 12, W 4, tau 0.8, sigma 0.1, tau_g 0.8): the
    Laplace-law error dp R / (2 sigma) - 1 after the full run, per storage, with R the radius
    of the phi > 1/2 volume. The lattice fits in L2, so its MLUPS are not a roofline figure."""
    import math

    import mcb

    cfg, phi, ux, uy, uz = mcb.workload(1, seed=SEED)
    cfg.device = device
    cells = cfg.nx * cfg.ny * cfg.nz
    out = {}
    for st in ("f32", "f16", "bf16"):
        cfg.storage = mcb.STORAGES[st]
        with mcb.Solver(cfg) as s:
            s.set_fields(phi, ux, uy, uz)
            s.step(updates)
            ms = s.last_step_ms()
            d = s.diagnostics()
        r = (3 * d["vol_half"] / (4 * math.pi)) ** (1 / 3)
        out[st] = {"laplace_err": d["dp"] * r / (2 * cfg.sigma) - 1, "dp": d["dp"],
                   "R_half": r, "mlups": cells * updates / (ms * 1e-3) / 1e6}
    out["updates"] = updates
    return out


def batch_run(device, steps, ncases=64):
    """64 uneven static/oscillating cases (edges 32..96, FP16 storage) in one launch per
    phase over the packed case table, graph-replayed. Compared with the same cases run one
    after another, each with its own handle."""
    import mcb

    cases = [mcb.workload(4, case_index=i, seed=SEED) for i in range(ncases)]
    cfgs = []
    for c, *_ in cases:
        c.device = device
        cfgs.append(c)
    warm = 2 * 16 + 2  # builds both graph parities outside the timed call
    with mcb.Batch(cfgs) as b:
        for i, (_, phi, *_r) in enumerate(cases):
            b.set_fields(i, phi)
        b.step(warm)
        b.step(steps)
        ms_batch = b.last_step_ms()
        cells = b.cells
        # per-size-class tile choice, then the same timing with the chosen schedule
        at_default, at_tuned = b.autotune(nsteps=20)
        b.step(warm)
        b.step(steps)
        ms_tuned = b.last_step_ms()
        classes = {}
        for i, c in enumerate(cfgs):
            classes.setdefault(f"{c.nx}", list(b.schedule(i)))
    ms_seq = 0.0
    for c, (_, phi, *_r) in zip(cfgs, cases):
        with mcb.Solver(c) as s:
            s.set_fields(phi)
            s.step(warm)
            s.step(steps)
            ms_seq += s.last_step_ms()
    return {"cases": ncases, "cells": cells, "storage": "f16", "steps": steps,
            "batch_mlups": cells * steps / (ms_batch * 1e-3) / 1e6,
            "batch_tuned_mlups": cells * steps / (ms_tuned * 1e-3) / 1e6,
            "autotune_trials_mlups": {"default": at_default, "tuned": at_tuned},
            "tuned_schedule_by_edge": classes,
            "sequential_mlups": cells * steps / (ms_seq * 1e-3) / 1e6,
            "speedup": ms_seq / ms_batch, "speedup_tuned": ms_seq / ms_tuned}


def d3q27_run(device, steps, storage="f32"):
    """The same workload with f on D3Q27 (27 populations): device MLUPS."""
    import mcb

    cfg, phi, ux, uy, uz = mcb.workload(SCENARIO, seed=SEED, scale=SCALE)
    cfg.storage = mcb.STORAGES[storage]
    cfg.velocity_set = 27
    cfg.device = device
    cells = cfg.nx * cfg.ny * cfg.nz
    with mcb.Solver(cfg) as s:
        s.set_fields(phi, ux, uy, uz)
        s.step(20)
        total, t_phi, t_col = s.step_profiled(steps)
    col_bytes = bytes_per_lu(cfg, storage)[1]
    return {"storage": storage, "steps": steps, "mlups": cells * steps / (total * 1e-3) / 1e6,
            "kernel_ms": {"phi_stage": t_phi / steps, "k_collide": t_col / steps},
            "collide_bytes_per_lu": col_bytes,
            "collide_gbs_algorithmic": col_bytes * cells / (t_col * 1e-3 / steps) / 1e9}


def swarm_run(device, steps):
    """The large swarm: 512^3, FP16 storage, walls in z, gravity 5e-6, 512 bubbles."""
    import mcb

    cfg, phi, *_ = mcb.workload(5, seed=SEED)
    cfg.device = device
    cells = cfg.nx * cfg.ny * cfg.nz
    with mcb.Solver(cfg) as s:
        s.set_fields(phi)
        s.step(2)
        m0 = s.diagnostics()["mass_q30"]
        total, t_phi, t_col = s.step_profiled(steps)
        d = s.diagnostics()
    per_update = total * 1e-3 / steps
    gs = g_storage(cfg)
    return {"cells": cells, "storage": "f16", "g_storage": gs, "steps": steps,
            "mlups": cells / per_update / 1e6,
            "hbm_gbs_algorithmic": bytes_per_lu(cfg, "f16")[2] * cells / per_update / 1e9,
            "mass_drift_q30": int(d["mass_q30"] - m0),
            "footprint_gb": footprint_bytes(cells, "f16", gs) / 1e9,
            "kernel_ms": {"phi_stage": t_phi / steps, "k_collide": t_col / steps}}


def cpu_baseline(seconds=10.0, threads=None):
    """FP64 oracle on the host cores: the bench workload at full size, as many updates as
    fit in the given seconds."""
    import mcb
    from oracle.oracle import Oracle

    threads = threads or os.cpu_count() or 1
    cfg, phi, ux, uy, uz = mcb.workload(SCENARIO, seed=SEED, scale=SCALE)
    o = Oracle.from_config(cfg, threads=threads)
    o.set_fields(phi, ux, uy, uz)
    o.step(1)
    n, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        o.step(1)
        n += 1
    dt = time.perf_counter() - t0
    cells = cfg.nx * cfg.ny * cfg.nz
    return {"value": cells * n / dt / 1e6, "unit": "MLUPS", "cores": threads, "kind": "port",
            "sample": f"FP64 oracle, the bench workload ({cfg.nx}x{cfg.ny}x{cfg.nz}),"
                      f" {n} updates in {dt:.1f} s"}


def traffic_per_launch(cells, storage="f32", gs="push"):
    """DRAM bytes per collide launch, from the committed ncu capture of this workload
    (profiles/traffic.json, bytes per cell), times the cells of one launch."""
    p = REPO / "profiles" / "traffic.json"
    if not p.exists():
        return None
    d = json.loads(p.read_text())
    try:
        return float(d[gs][f"collide_{storage}_dram_bytes_per_cell"]) * cells
    except KeyError:
        return None


def run_reference_arm(args, ws, rank):
    """The reference path on the host cores: the FP64 oracle port of the reference update
    (the reference has no CPU implementation) on the full 128x128x256 rising bubble. The
    initial field comes from the oracle-side generator, so this arm loads no solver code."""
    if rank != 0:
        return
    steps, warmup = args.steps, args.warmup
    from oracle.oracle import Oracle
    from oracle.workload_port import rising_bubble

    threads = os.cpu_count() or 1
    phi, p = rising_bubble(seed=SEED, scale=SCALE)
    f32 = lambda v: float(np.float32(v))
    sharp = (p["tau_g"] - 0.5) * 4.0 / p["width"]
    o = Oracle(p["nx"], p["ny"], p["nz"], p["bc"], f32(p["tau"]), f32(p["tau_g"]),
               f32(p["sigma"]), f32(sharp), f32(p["gravity"]), threads=threads)
    o.set_fields(phi)
    o.step(warmup)
    t0 = time.perf_counter()
    o.step(steps)
    dt = time.perf_counter() - t0
    cells = p["nx"] * p["ny"] * p["nz"]
    v = cells * steps / dt / 1e6
    sample = (f"FP64 oracle port of the reference update (the reference has no CPU path) on "
              f"the full {p['nx']}x{p['ny']}x{p['nz']} rising bubble, {steps} updates after "
              f"{warmup} warm-up updates, {threads} threads")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": "MLUPS", "n_gpus": ws,
        "steps": steps, "warmup": warmup, "ms_per_step": dt * 1e3 / max(steps, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": f"rising perturbed bubble {p['nx']}x{p['ny']}x{p['nz']}, walls "
                               "z, gravity 1e-5, Y_lm l=2..6, tau 0.7, sigma 0.05, W 4",
                   "cells": cells, "same_config": True, "seed": SEED},
        "cpu_baseline": {"value": v, "unit": "MLUPS", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": v, "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="solver", choices=["solver", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--scale", type=float, default=1.0,
                    help="length scale of the workload (profiling runs use a smaller case)")
    ap.add_argument("--storage", default="f32", choices=["f32", "f16", "bf16"],
                    help="population storage of the device leg (the headline is f32)")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the batched-cases and 512^3 swarm legs")
    ap.add_argument("--g-populations", action="store_true",
                    help="store the 18 moving g populations (the phi kernel reads them)")
    ap.add_argument("--variant", type=int, default=-1,
                    help="tile variant of the device leg (-1 default; 4 the TMA-staged collide)")
    ap.add_argument("--zchunk", type=int, default=0,
                    help="work split of the device leg (0 default, >0 fixed chunks, -w waves)")
    ap.add_argument("--tau-g", type=float, default=None,
                    help="g relaxation time of the device leg (1: equilibrium g, the workload's)")
    ap.add_argument("--only-device", action="store_true",
                    help="time the device loop only (no fp16, e2e, reference or CPU legs)")
    args = ap.parse_args()
    global SCALE, G_POPULATIONS, VARIANT, ZCHUNK
    SCALE = args.scale
    G_POPULATIONS = args.g_populations
    VARIANT, ZCHUNK = args.variant, args.zchunk
    ws, rank, local = dist_env()
    if args.impl == "reference":
        run_reference_arm(args, ws, rank)
        return
    if args.warmup < 3:
        raise SystemExit("--warmup must be >= 3")

    import __graft_entry__
    import mcb

    if not mcb.LIB_PATH.exists():
        __graft_entry__.build()
    dist = init_dist(ws, "nccl")
    import torch

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    with Clocks(local) as clk:
        cfg, total_ms, phi_ms, col_ms, diag = device_run(args.storage, local, args.steps,
                                                         args.warmup, dist, args.tau_g)
    t_max = reduce_max(dist, total_ms, dev)
    cells = cfg.nx * cfg.ny * cfg.nz
    value = ws * cells * args.steps / (t_max * 1e-3) / 1e6
    hbm, peak_kind = peaks()
    col_avg_s = col_ms * 1e-3 / args.steps
    st = args.storage
    gs = g_storage(cfg, VARIANT)
    _, col_b, upd_b = bytes_per_lu(cfg, st, VARIANT)
    achieved = col_b * cells / col_avg_s / 1e9
    update_achieved = upd_b * cells / (total_ms * 1e-3 / args.steps) / 1e9
    # The roofline MLUPS of the metric as first stated for this path: an update that stores
    # f and g moves 2 x 19 populations in and out, 304 B/LU at FP32 (152 at 16 bits). This
    # update stores no g, so it can run above that figure.
    mb = 2 * 2 * 19 * (4 if st == "f32" else 2)
    metric_roofline = {"bytes_per_lu": mb, "mlups": hbm * 1e3 / mb,
                       "frac": (value / ws) / (hbm * 1e3 / mb)}
    result = {
        "metric": METRIC, "value": value, "unit": "MLUPS", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "storage": st,
        "data": "synthetic",
        "config": {"workload": f"rising perturbed bubble {cfg.nx}x{cfg.ny}x{cfg.nz}, walls z, "
                               "gravity 1e-5, Y_lm l=2..6, tau 0.7, sigma 0.05, W 4, "
                               f"{STORAGE_WORDS[st]} population storage",
                   "cells": cells,
                   "l2": f"inputs larger than L2 (f in and out: "
                         f"{2 * 19 * (4 if st == 'f32' else 2) * cells / 1e6:.0f} MB per update)",
                   "parallelism": f"replicas x{ws}", "seed": SEED,
                   "graph_prep_updates": GRAPH_PREP},
        "roofline": {"bound": "hbm", "kernel": KERNEL_OF[(st, args.tau_g)], "achieved": achieved,
                     "peak": hbm,
                     "unit": "GB/s", "frac": achieved / hbm,
                     "peak_kind": f"{peak_kind} HBM copy bandwidth",
                     "bytes_per_lu": col_b, "g_storage": gs,
                     "traffic": traffic_per_launch(cells, st, gs),
                     "update_achieved": update_achieved, "update_frac": update_achieved / hbm,
                     "update_bytes_per_lu": upd_b,
                     "kernel_ms": {"phi_stage": phi_ms / args.steps, "k_collide": col_ms / args.steps}},
        "roofline_mlups_fg": metric_roofline,
        # one collide launch per update, but with the TMA records: the phi kernel and the
        # collide kernel
        "gpu_launches": (2 if gs == "records" else 1) * args.steps,
        "clocks": clk.summary(),
        "mass_q30_finite": bool(diag["finite"]),
    }
    if rank == 0 and args.only_device:
        print(json.dumps(result))
    elif rank == 0:
        legs = {k: storage_leg(local, args.steps, args.warmup, k) for k in ("f16", "bf16")}
        v32 = value / ws
        for k, leg in legs.items():
            leg["ratio_vs_f32"] = leg["value"] / v32
        result["fp16"], result["bf16"] = legs["f16"], legs["bf16"]
        # stored, relaxed g (tau_g = 0.8, the static-bubble setting) on the same workload
        result["stored_g"] = [storage_leg(local, args.steps, args.warmup, k, tau_g=0.8)
                              for k in ("f32", "f16")]
        result["e2e"] = e2e_run(local, args.steps)
        result["e2e_500"] = e2e_run(local, 500)
        if not args.no_extras:
            result["config3"] = config3_run(local)
            result["laplace"] = laplace_run(local)
            result["batch"] = batch_run(local, min(args.steps, 200))
            result["swarm"] = swarm_run(local, min(args.steps, 50))
            result["d3q27"] = [d3q27_run(local, min(args.steps, 200), st) for st in ("f32", "f16")]
        nref = min(max(args.steps, 20), 200)
        rc = reference_cuda_run(local, nref)
        mine = reference_mode_run(local, nref)
        if "value" in rc:
            mine["ratio_vs_reference_cuda"] = mine["value"] / rc["value"]
        result["reference_cuda"] = rc
        result["reference_mode"] = mine
        stock = reference_cuda_stock(local, nref)
        mine_stock = reference_mode_run(local, nref, 64, 64, 256, 0.505, 0.1, 20.0, 3.0, 0.45)
        if "value" in stock:
            mine_stock["ratio_vs_reference_cuda"] = mine_stock["value"] / stock["value"]
        result["reference_cuda_stock"] = stock
        result["reference_mode_stock"] = mine_stock
        # the static bubble (64^3, the reference's frozen shell at tau 0.8, sigma 0.1)
        sb = reference_cuda_stock(local, nref, 64, 64, 64, 0.8, 0.1, 0.5, 12.0, 4.0,
                                  "static bubble R 12, tau 0.8, sigma 0.1, SHARP_C 0.5")
        mine_sb = reference_mode_run(local, nref, 64, 64, 64, 0.8, 0.1, 12.0, 4.0, 0.5)
        if "value" in sb:
            mine_sb["ratio_vs_reference_cuda"] = mine_sb["value"] / sb["value"]
        result["reference_cuda_static_bubble"] = sb
        result["reference_mode_static_bubble"] = mine_sb
        result["cpu_baseline"] = cpu_baseline(args.cpu_seconds)
        print(json.dumps(result))
    barrier(dist)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
