"""Benchmark of the Steinbach multi-phase-field time step on GB300.

Workload (default): the large 3D production configuration -- 512^3 cells,
1000 Voronoi ferrite grains + 20000 austenite nuclei (radius 2 cells), up to 4
active grains per cell (uint16 ids, FP32 fractions), C 0.10 / Mn 1.5 wt%,
T = 1023 K.  One "step" is one full time step: the phase sweep plus n_sub
diffusion sub-steps.  ``--workload 3d256`` selects the 256^3 configuration.

Printed JSON (rank 0, one line):
  value    cell-updates/s of the FP32-compensated step with the state resident
           in HBM, timed with CUDA events on the launching stream.
  e2e      the same metric through the C ABI with host buffers: upload of the
           reference-layout state from pinned memory, K x (step + statistics
           read-back), download of the state, all inside the timed region.
  roofline the diffusion sub-step kernel (the dominant one): algorithmic bytes
           per launch / mean launch time (CUDA events around each launch).
  fp64     the plain FP64 step (reference layout) on the same workload.
  cpu_baseline  the FP64 CPU oracle (bit-for-bit equal to the reference's own
           CPU code on the golden cases) on a bounded sample of the workload: a
           slab of the same initial state.

--impl reference times the reference's CPU algorithm (the FP64 oracle) on all
host cores over the same workload and configuration, one bounded sample per
step (a z slab of the same seeded state, generated by the oracle library's own
copy of the input generator; the product library is not loaded).

Multi-GPU (--gpus N under torchrun): one domain is not decomposed across GPUs,
so each rank advances an independent replica (different seed);
value = all ranks' cells x steps / max-over-ranks time ("scaling": "weak").
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import shutil
import statistics
import subprocess
import sys
import tempfile
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "cell-updates/s & % HBM roofline: FP32 vs FP64 step; batch; adjoint/fwd ratio"
_T0 = time.perf_counter()


def _log(msg: str) -> None:
    """Progress of the legs on stderr (the JSON line goes to stdout)."""
    print(f"[bench {time.perf_counter() - _T0:7.1f}s] {msg}", file=sys.stderr, flush=True)
UNIT = "cell-updates/s"


def _peaks() -> dict:
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 50 ms during a region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []
        self.t = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "50",
                 "-i", str(self.device)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            if self.t:
                self.t.join(timeout=2)

    def summary(self) -> dict:
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def _workload(name: str):
    from phasefield_gb300 import workloads as W

    return W.WORKLOADS[name]


def _model_for(wl, grid=None, tmp=None):
    import phasefield_gb300 as pf
    from phasefield_gb300 import workloads as W

    d = tmp or tempfile.mkdtemp(prefix="pfbench_")
    cfg = W.write_config(os.path.join(d, wl.name + ".txt"), grid=grid or wl.grid, dx=wl.dx, T=wl.T,
                         num_grain=(wl.n_grains, 0, 0), num_nuclei=wl.n_nuclei, directory=d)
    W.write_thermo(os.path.join(d, "thermo_steel.txt"))
    return cfg, pf.read_model(cfg)


def _scaled_spec(wl, grid):
    """Spec for a sub-box of the workload keeping grain and nucleus densities."""
    s = wl.spec()
    frac = (grid[0] * grid[1] * grid[2]) / float(wl.N)
    s.n_grains = max(2, int(round(wl.n_grains * frac)))
    s.n_nuclei = int(round(wl.n_nuclei * frac))
    s.n_particles = int(round(wl.n_particles * frac))
    return s


def _config(wl, grid, n_sub: int, nsol: int) -> dict:
    """The workload description both arms print (identical by construction)."""
    return {"workload": f"{wl.name}: {grid[0]}x{grid[1]}x{grid[2]} cells, {wl.n_grains} grains, "
                        f"{wl.n_nuclei} nuclei r={wl.nucleus_radius}, C/Mn {wl.C0} +-{wl.C_noise[0]} wt%, "
                        f"T={wl.T} K, n_sub={n_sub}",
            "grid": list(grid), "n_sub": n_sub, "solutes": nsol,
            "l2": f"inputs larger than L2 (FP32 state {grid[0] * grid[1] * grid[2] * 52 / 1e9:.2f} GB, L2 0.13 GB)"}


SLAB_PLANES = 32


def cpu_sample(wl, grid):
    """A bounded sample of the workload for the FP64 CPU oracle, built without
    the product library: planes [z0, z0 + SLAB_PLANES) of the workload's own
    seeded initial state (the oracle library carries the same input
    generator), stepped as a periodic box.  Returns (oracle model, state,
    cells per step, n_sub, label)."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import build_oracle
    import pyoracle as po
    from phasefield_gb300 import workloads as W

    build_oracle.build_oracle()
    d = tempfile.mkdtemp(prefix="pfcpu_")
    W.write_thermo(os.path.join(d, "thermo_steel.txt"))
    full_cfg = W.write_config(os.path.join(d, "full.txt"), grid=grid, dx=wl.dx, T=wl.T, directory=d)
    om_full = po.load_model(full_cfg)
    nz = min(SLAB_PLANES, grid[2])
    z0 = (grid[2] - nz) // 2
    spec = wl.spec() if tuple(grid) == tuple(wl.grid) else _scaled_spec(wl, grid)
    st = po.init_state(om_full, spec, 0.0, z0=z0, nz=nz)
    slab_cfg = W.write_config(os.path.join(d, "slab.txt"), grid=(grid[0], grid[1], nz), dx=wl.dx, T=wl.T,
                              directory=d)
    om = po.load_model(slab_cfg)
    n_sub = po.params_at(om_full, 0.0).n_sub
    cells = grid[0] * grid[1] * nz
    label = (f"planes {z0}..{z0 + nz - 1} of the {wl.name} seeded initial state ({grid[0]}x{grid[1]}x{nz} cells, "
             f"same state as the GPU arm), stepped as a periodic box; one full FP64 time step (phase sweep + "
             f"n_sub={n_sub} diffusion sub-steps) per sample")
    return om, st, cells, n_sub, label


def run_reference(args) -> dict:
    """--impl reference: the reference's CPU algorithm (FP64 oracle) on the host
    cores, over the same workload and configuration as the GPU arm."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import pyoracle as po

    wl = _workload(args.workload)
    grid = tuple(args.grid) if args.grid else wl.grid
    om, st, cells, n_sub, label = cpu_sample(wl, grid)
    t = 0.0
    for _ in range(args.warmup):
        t = po.run(om, st, t, 1)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        t = po.run(om, st, t, 1)
    dt = time.perf_counter() - t0
    v = cells * args.steps / dt
    return {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded Voronoi grains + nuclei)",
        "config": _config(wl, grid, n_sub, om.nsol),
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": po.num_threads(), "kind": "port", "sample": label},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def run_batch(args, rank: int) -> dict:
    """Batched ensemble: 64 square 2D domains (sides 128..512 in steps of 32),
    T ~ U[993,1053] K, C ~ U[0.05,0.20] wt%, per-domain grain and nucleus
    densities, FP32 compensated, advanced by one persistent launch replayed from
    a CUDA graph."""
    import torch

    import phasefield_gb300 as pf
    from phasefield_gb300 import workloads as W

    doms = W.ensemble(64, seed=rank)
    paths = W.ensemble_inputs(tempfile.mkdtemp(prefix="pfens_"), doms)
    models = [pf.read_model(p) for p in paths]
    B = pf.Batch(models)
    for d, (m, dom) in enumerate(zip(models, doms)):
        B.upload(d, pf.init_microstructure(m, W.ensemble_spec(dom), 0.0), 0.0)
    from phasefield_gb300 import replicas

    tuned = B.autotune(50)  # tile shape of the persistent kernel (states restored)
    st = B.run(args.warmup)
    torch.cuda.synchronize()
    replicas.barrier()
    t0 = time.perf_counter()
    st2 = B.run(args.batch_steps)
    dt = replicas.max_over_ranks(time.perf_counter() - t0, device="cuda" if replicas.world()[1] > 1 else None)
    info = B.info()
    info["cells"] = sum(replicas.gather([info["cells"]]))  # every rank advances its own ensemble
    fr = [float(B.reduce(d)[1] / (m.ix * m.iy)) for d, m in enumerate(models[:4])]
    B.close()
    return {"domains": len(models), "cells": info["cells"], "steps": args.batch_steps, "resident_blocks": info["blocks"],
            "n_sub_max": info["n_sub_max"], "ok": st == pf.PF_OK and st2 == pf.PF_OK,
            "value": info["cells"] * args.batch_steps / dt, "unit": UNIT, "seconds": dt,
            "launch": "one persistent cooperative kernel per run, replayed from a CUDA graph",
            "tile": tuned,
            "austenite_fraction_first_domains": fr}


def run_adjoint(args) -> dict:
    """Adjoint calibration: 2D 512^2, ferrite + austenite + cementite particles
    (radius 2, 0.5% area), FP32 with FP64 reductions.  Two modes: record (the
    forward keeps every step's record in HBM, the gradient only sweeps
    backwards) and checkpoints every 100 steps (the gradient recomputes each
    segment).  Ratio = gradient time / forward time of the same mode; both
    also against the production FP32C forward."""
    import numpy as np

    import phasefield_gb300 as pf
    from phasefield_gb300 import workloads as W

    wl = W.WORKLOADS["2d512cem"]
    cfg, m = _model_for(wl)
    st = pf.init_microstructure(m, wl.spec(), 0.0)

    def mode(K):
        A = pf.Adjoint(m, pf.PF_PREC_FP32C, K)
        A.upload(st, 0.0)
        # Warm-up: captures the graphs reused below (record mode: one per step count).
        A.forward(args.adjoint_steps if K == 0 else min(args.adjoint_steps, 200))
        A.gradient(0)
        J = A.forward(args.adjoint_steps)
        g = A.gradient(0)
        t = A.timings()
        A.close()
        return J, g, t

    J, g, t = mode(0)
    Jc, gc, tc = mode(100)
    # The production FP32C forward on the same state, for scale.
    import torch

    F = pf.PhaseField(m, pf.PF_PREC_FP32C)
    F.upload(st, 0.0)
    F.update(10)
    F.synchronize()
    t0 = time.perf_counter()
    F.update(args.adjoint_steps)
    F.synchronize()
    prod_ms = (time.perf_counter() - t0) * 1e3
    F.close()
    torch.cuda.synchronize()
    N = wl.grid[0] * wl.grid[1] * wl.grid[2]
    n_sub = pf.params_at(m, 0.0).n_sub
    return {"grid": list(wl.grid), "steps": args.adjoint_steps, "mode": "record",
            "record_bytes": (72 + 4 * n_sub) * N * args.adjoint_steps,
            "production_forward_ms": prod_ms, "adjoint_over_production_forward": t["gradient_ms"] / prod_ms,
            "J_ferrite_fraction": float(J[0]), "J_austenite_carbon": float(J[1]),
            "dJ0_ds": [float(x) for x in g], "forward_ms": t["forward_ms"], "gradient_ms": t["gradient_ms"],
            "adjoint_over_forward": t["gradient_ms"] / t["forward_ms"],
            "forward_and_gradient_over_production_forward": (t["forward_ms"] + t["gradient_ms"]) / prod_ms,
            "checkpointed": {"checkpoint_every": 100, "forward_ms": tc["forward_ms"], "gradient_ms": tc["gradient_ms"],
                             "adjoint_over_forward": tc["gradient_ms"] / tc["forward_ms"],
                             "adjoint_over_production_forward": tc["gradient_ms"] / prod_ms,
                             "J_max_rel_diff": float(np.max(np.abs(np.array(J) - np.array(Jc)) / np.abs(np.array(Jc)))),
                             "gradient_max_rel_diff": float(np.max(np.abs(np.array(g) - np.array(gc)) /
                                                                   np.maximum(np.abs(np.array(gc)), 1e-300)))},
            "note": "record: the forward stores every step's record, the gradient is the reverse sweep alone; "
                    "checkpointed: the gradient recomputes each 100-step segment, then sweeps it backwards"}


def run_precision(args) -> dict:
    """Error of the FP32-compensated path against FP64 on the 3D FP32-vs-FP64
    configuration (3d256: 256^3, 200 grains, 2000 nuclei, T = 1013 K, 2000
    steps; --precision-grid scales the box keeping grain and nucleus densities):
    against the four-slot model in FP64 (the workload's own model -- up to 4
    grains per cell -- so the difference is FP32 rounding alone), and, on a
    --six-slot-grid box, against the six-slot FP64 reference path (which adds
    the model change of keeping four grains per cell)."""
    import numpy as np

    import phasefield_gb300 as pf
    from phasefield_gb300 import workloads as W

    wl = W.WORKLOADS["3d256"]
    S = args.precision_steps

    def setup(g):
        grid = (g, g, g)
        cfg, m = _model_for(wl, grid)
        spec = wl.spec() if grid == wl.grid else _scaled_spec(wl, grid)
        return m, pf.init_microstructure(m, spec, 0.0), g * g * g

    def fp32(m, st):
        F = pf.PhaseField(m, pf.PF_PREC_FP32C)
        F.upload(st, 0.0)
        F.update(S)
        out = F.download(conc=False)
        out["reduce"] = F.reduce()
        F.close()
        return out

    def err(a32, ref_phase, ref_C, N):
        d = np.abs(a32["phase"][:3 * N] - ref_phase)
        fr32 = a32["phase"].reshape(N, 3).mean(0)
        frr = ref_phase.reshape(N, 3).mean(0)
        return {"phase_max_abs": float(d.max()), "phase_mean_abs": float(d.mean()),
                "cells_phase_err_gt_1e-5": int((d.reshape(N, 3).max(1) > 1e-5).sum()),
                "carbon_max_rel": float(np.max(np.abs(a32["C"][:N] - ref_C) / np.abs(ref_C))),
                "carbon_mean_rel": float(np.mean(np.abs(a32["C"][:N] - ref_C) / np.abs(ref_C))),
                "phase_fraction_abs": [float(x) for x in np.abs(fr32 - frr)]}

    t0 = time.perf_counter()
    m, st, N = setup(args.precision_grid)
    a32 = fp32(m, st)
    A = pf.Adjoint(m, pf.PF_PREC_FP64, max(S, 1))
    A.upload(st, 0.0)
    A.forward(S)
    a4 = A.final_state()
    A.close()
    C0 = st["C"][:N].sum()
    out = {"grid": [args.precision_grid] * 3, "steps": S, "cells": N,
           "vs_fp64_four_slot": err(a32, a4["phase"], a4["C"], N),
           "carbon_mass_rel_drift_fp32": float(abs(a32["reduce"][4] - C0) / C0)}
    if args.sensitivity_grid > 0:
        # How far the FP64 four-slot model itself moves when only its input is
        # rounded: phi rounded to FP32 (what the compact layout stores), or
        # perturbed by a few FP64 ulps.  Pointwise differences of this size are
        # a property of the model's discrete decisions (clamps at 0 / 1 and the
        # cutoff, top-four choice), not of the arithmetic precision.
        ms, sts, Ns = setup(args.sensitivity_grid)

        def fp64_four_slot(state):
            A = pf.Adjoint(ms, pf.PF_PREC_FP64, max(S, 1))
            A.upload(state, 0.0)
            A.forward(S)
            out = A.final_state()
            A.close()
            return out

        base = fp64_four_slot(sts)
        r32 = dict(sts, phi=sts["phi"].astype(np.float32).astype(np.float64))
        ulp = dict(sts, phi=sts["phi"] * (1.0 + 4.0 * np.finfo(np.float64).eps))
        c32 = fp32(ms, sts)
        out["sensitivity_fp64_four_slot"] = {
            "grid": [args.sensitivity_grid] * 3,
            "fp64_input_rounded_to_fp32": err(fp64_four_slot(r32), base["phase"], base["C"], Ns),
            "fp64_input_times_1p4ulp": err(fp64_four_slot(ulp), base["phase"], base["C"], Ns),
            "fp32c": err(c32, base["phase"], base["C"], Ns),
        }
    if args.six_slot_grid > 0:
        m6, st6, N6 = setup(args.six_slot_grid)
        b32 = fp32(m6, st6)
        F64 = pf.PhaseField(m6, pf.PF_PREC_FP64)
        F64.upload(st6, 0.0)
        F64.update(S)
        a64 = F64.download(conc=False)
        F64.close()
        out["vs_fp64_six_slot"] = dict(err(b32, a64["phase"], a64["C"][:N6], N6), grid=[args.six_slot_grid] * 3)
    out["seconds"] = time.perf_counter() - t0
    return out


def run_ours(args, rank: int, world: int, local_rank: int) -> dict | None:
    import numpy as np
    import torch

    import phasefield_gb300 as pf

    torch.cuda.set_device(local_rank)
    dev = torch.cuda.current_device()
    wl = _workload(args.workload)
    grid = tuple(args.grid) if args.grid else wl.grid
    cfg, m = _model_for(wl, grid)
    spec = wl.spec() if tuple(grid) == tuple(wl.grid) else _scaled_spec(wl, grid)
    spec.seed = wl.seed + rank
    N = grid[0] * grid[1] * grid[2]
    P = pf.params_at(m, 0.0)
    nsol = m.nsol
    # A dedicated stream: every context launches on it and the CUDA events are
    # recorded on it (torch's default stream has handle 0, which the C ABI
    # reads as "use the context's own stream").
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    def max_over_ranks(x: float) -> float:
        if world == 1:
            return x
        t = torch.tensor([x], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        return float(t.item())

    # ---- initial state, generated on the device (pf_init_device) ---------
    # The reference-layout context also serves the FP64 leg, and its download
    # is the host state of the e2e leg.
    _log(f"initial state {grid} on the device")
    G = pf.PhaseField(m, pf.PF_PREC_FP64)
    G.set_stream(stream.cuda_stream)
    G.construct_on_device(spec, 0.0)  # warm-up (module load, first allocations)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    G.construct_on_device(spec, 0.0)
    torch.cuda.synchronize()
    init_dev_s = time.perf_counter() - t0
    st0 = {k: v for k, v in G.download().items() if isinstance(v, np.ndarray)} if not args.no_e2e else None
    _log("initial state done")

    # ---- value: FP32-compensated step, state resident in HBM -------------
    F = pf.PhaseField(m, pf.PF_PREC_FP32C)
    F.set_stream(stream.cuda_stream)
    F.construct_on_device(spec, 0.0)
    tuned = F.autotune() if not args.no_tune else None
    F.update(args.warmup)
    F.enable_kernel_timing(True)
    barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev) as clk:
        e0.record(stream)
        F.update(args.steps)
        e1.record(stream)
        torch.cuda.synchronize()
    barrier()
    ms = max_over_ranks(e0.elapsed_time(e1))
    kt = F.kernel_times()
    # A phase sweep is two kernels (register-list cells, then the deferred
    # cells with longer stencil lists); a diffusion sub-step is one.
    launches = 2 * kt["phase"][1] + kt["diffusion"][1]
    value = world * N * args.steps / (ms / 1e3)
    fr_end = F.fractions()
    F.enable_kernel_timing(False)
    # Binary microstructure files written from the device state while two
    # more steps run (pf_write_vti_binary): time to enqueue, and until written.
    out_dir = tempfile.mkdtemp(prefix="pfvti_")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    F.write_vti_binary(out_dir, 0, 16)
    t_enq = time.perf_counter() - t0
    F.update(2)
    torch.cuda.synchronize()
    t_steps = time.perf_counter() - t0
    F.write_wait()
    t_all = time.perf_counter() - t0
    vti_bytes = sum(os.path.getsize(os.path.join(out_dir, f)) for f in os.listdir(out_dir))
    shutil.rmtree(out_dir, ignore_errors=True)
    output = {"pieces": 16, "bytes": vti_bytes, "enqueue_ms": t_enq * 1e3, "two_steps_after_ms": t_steps * 1e3,
              "written_s": t_all, "note": "fields formed on the device, copied on a side stream and written by "
                                          "host threads while the two steps ran"}
    F.close()

    _log("FP32C leg done")
    # ---- FP64 plain step on the same workload ----------------------------
    fp64 = None
    if args.fp64_steps > 0:
        k64 = max(1, min(args.steps, args.fp64_steps))
        G.update(1)
        G.enable_kernel_timing(True)
        torch.cuda.synchronize()
        g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        g0.record(stream)
        G.update(k64)
        g1.record(stream)
        torch.cuda.synchronize()
        ms64 = max_over_ranks(g0.elapsed_time(g1))
        kt64 = G.kernel_times()
        value64 = world * N * k64 / (ms64 / 1e3)
        fp64 = {"value": value64, "unit": UNIT, "steps": k64, "ms_per_step": ms64 / k64,
                "phase_ms": kt64["phase"][0] / max(1, kt64["phase"][1]),
                "diffusion_ms": kt64["diffusion"][0] / max(1, kt64["diffusion"][1])}
    G.close()
    extra = {"init": {"device_s": init_dev_s, "how": "pf_init_device: the seeded generator run one cell per GPU "
                                                    "thread into the FP64 reference-layout context"},
             "output": output}
    if args.no_e2e:
        return _result(args, wl, grid, N, P, nsol, world, rank, ms, value, kt, launches, fr_end, fp64, None, clk, tuned,
                       extra)

    _log("FP64 leg done")
    # ---- e2e: through the C ABI with pinned host buffers -----------------
    keep_alive = []

    def pinned(arr: np.ndarray) -> np.ndarray:
        t = torch.empty(arr.size, dtype={np.int32: torch.int32, np.float64: torch.float64}[arr.dtype.type],
                        pin_memory=True)
        keep_alive.append(t)
        out = t.numpy()
        out[:] = arr
        return out

    host = {k: pinned(v) for k, v in st0.items()}
    back = {k: pinned(np.zeros_like(v)) for k, v in st0.items()}
    H = pf.PhaseField(m, pf.PF_PREC_FP32C)
    H.set_stream(stream.cuda_stream)
    H.upload(host, 0.0)   # warm the path (allocations, module load) and tune once
    if not args.no_tune:
        H.autotune()
    H.update(1)
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    H.upload(host, 0.0)
    for _ in range(args.steps):
        H.update(1)
        H.fractions()  # device -> host read of the step's statistics (64 bytes)
    tt = ctypes.c_double()
    pf.check(pf.lib().pf_download_state(H._ctx, pf._ptr(back["ids"]), pf._ptr(back["phi"]), pf._ptr(back["phase"]),
                                        pf._ptr(back["conc"]), pf._ptr(back["C"]), ctypes.byref(tt)), "download")
    e2e_s = max_over_ranks(time.perf_counter() - t0)
    H.close()
    state_bytes = sum(int(v.nbytes) for k, v in st0.items() if k in ("ids", "phi", "phase", "C"))
    down_bytes = sum(int(v.nbytes) for v in st0.values())
    e2e = {"value": world * N * args.steps / e2e_s, "unit": UNIT,
           "h2d_bytes_per_step": int(state_bytes / args.steps),
           "d2h_bytes_per_step": int(64 + down_bytes / args.steps)}
    return _result(args, wl, grid, N, P, nsol, world, rank, ms, value, kt, launches, fr_end, fp64, e2e, clk, tuned,
                   extra)


def _diffusion_kernel(tuned):
    """Name of the FP32 diffusion kernel the timed steps launched."""
    if not tuned:
        return "k_diffuse_tma (library default where the grid allows TMA, else k_diffuse)"
    return "k_diffuse_tma" if tuned.get("variant") == 1 else "k_diffuse"


def _result(args, wl, grid, N, P, nsol, world, rank, ms, value, kt, launches, fr_end, fp64, e2e, clk, tuned=None,
            extra=None):
    if rank != 0:
        return None
    pk = _peaks()
    diff_bytes = N * (12 + 16 * nsol)           # algorithmic bytes per diffusion sub-step
    phase_bytes = N * (60 + 8 * nsol)           # algorithmic bytes per phase sweep
    t_diff = kt["diffusion"][0] / max(1, kt["diffusion"][1]) / 1e3
    t_phase = kt["phase"][0] / max(1, kt["phase"][1]) / 1e3
    ach = diff_bytes / t_diff / 1e9
    step_bytes = phase_bytes + P.n_sub * diff_bytes

    _log("e2e leg done")
    # ---- CPU baseline (oracle, bounded sample) ----------------------------
    cpu = None
    if not args.no_cpu:
        sys.path.insert(0, os.path.join(REPO, "oracle"))
        import pyoracle as po

        g0 = time.perf_counter()
        om, cst, cells, _, label = cpu_sample(wl, grid)
        gen_s = time.perf_counter() - g0  # the slab's state from the host generator (plus set-up)
        if extra is not None and "init" in extra:
            extra["init"]["host_s_estimate"] = gen_s * grid[2] / (cells / (grid[0] * grid[1]))
            extra["init"]["host_cores"] = po.num_threads()
            extra["init"]["host_sample"] = ("the same generator on the host (oracle library copy, all cores) for the "
                                            "CPU sample's slab, scaled by planes")
        tcur = po.run(om, cst, 0.0, 1)
        c0 = time.perf_counter()
        nst = 2
        po.run(om, cst, tcur, nst)
        cdt = time.perf_counter() - c0
        cpu = {"value": cells * nst / cdt, "unit": UNIT, "cores": po.num_threads(), "kind": "port",
               "sample": label + f", {nst} steps"}

    ms_step = ms / args.steps
    # DRAM traffic of the diffusion kernel: bytes per cell from the committed ncu
    # capture of a smaller box of the same workload (profiles/ncu_traffic.json),
    # scaled to this launch by its cell count.
    traffic, traffic_src = None, None
    tpath = os.path.join(REPO, "profiles", "ncu_traffic.json")
    if os.path.exists(tpath):
        with open(tpath) as f:
            tj = json.load(f).get("k_diffuse")
        if tj:
            traffic = tj["dram_bytes_per_cell"] * N
            traffic_src = f"ncu dram__bytes_read+write on {tj['case']}, scaled by cell count"
    return {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32 (Kahan-compensated solutes, fp64 reductions)",
        "data": "synthetic (seeded Voronoi grains + nuclei, uniform noise)",
        "config": _config(wl, grid, P.n_sub, nsol),
        "roofline": {"bound": "hbm", "achieved": ach, "peak": pk["hbm_gbs"], "unit": "GB/s",
                     "frac": ach / pk["hbm_gbs"], "traffic": traffic, "traffic_source": traffic_src,
                     "kernel": _diffusion_kernel(tuned),
                     "algorithmic_bytes_per_launch": diff_bytes, "mean_launch_ms": t_diff * 1e3,
                     "peak_source": pk["source"] + " (MEASURED_PEAKS.json hbm_gbs)"},
        "kernels": {
            "phase_sweep_f32": {"kernels": "k_phase_f32 + k_phase_f32_rest", "launches": kt["phase"][1],
                                "mean_ms": t_phase * 1e3,
                                "gbs": phase_bytes / t_phase / 1e9, "bytes_per_launch": phase_bytes},
            "diffusion_f32": {"launches": kt["diffusion"][1], "mean_ms": t_diff * 1e3, "gbs": ach,
                              "bytes_per_launch": diff_bytes},
            "step_gbs_effective": step_bytes * args.steps / (ms / 1e3) / 1e9,
            "diffusion_tile": tuned,
        },
        "fp64": fp64,
        "fp32_over_fp64": (value / fp64["value"]) if fp64 else None,
        "fractions_end": [float(x) for x in fr_end[:3]],
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
        **(extra or {}),
    }


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="3d512")
    ap.add_argument("--fp64-steps", type=int, default=3)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="skip the diffusion tile autotuner")
    ap.add_argument("--batch-steps", type=int, default=5000, help="steps of the 64-domain ensemble (0 = skip)")
    ap.add_argument("--adjoint-steps", type=int, default=2000, help="steps of the adjoint calibration run (0 = skip)")
    ap.add_argument("--precision-steps", type=int, default=2000, help="steps of the FP32-vs-FP64 error run (0 = skip)")
    ap.add_argument("--precision-grid", type=int, default=256, help="cube side of the FP32-vs-FP64 error run")
    ap.add_argument("--sensitivity-grid", type=int, default=128,
                    help="cube side of the FP64 self-sensitivity comparison (0 = skip)")
    ap.add_argument("--six-slot-grid", type=int, default=128,
                    help="cube side of the FP32C-vs-six-slot-FP64 comparison (0 = skip)")
    ap.add_argument("--grid", type=int, nargs=3, default=None, help="override the workload grid")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(run_reference(args)), flush=True)
        return

    import __graft_entry__

    if rank == 0 or world == 1:
        __graft_entry__.build()
    if world > 1:
        import torch

        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        torch.distributed.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
        torch.distributed.barrier()
        if rank != 0:
            __graft_entry__.build()
    out = run_ours(args, rank, world, local_rank)
    _log("main leg done")
    if args.batch_steps > 0:
        b = run_batch(args, rank)
        _log("batch done")
        if out is not None:
            out["batch"] = b
    if args.adjoint_steps > 0 and out is not None:
        out["adjoint"] = run_adjoint(args)
        _log("adjoint done")
    if args.precision_steps > 0 and out is not None:
        out["precision"] = run_precision(args)
        _log("precision done")
    if out is not None:
        print(json.dumps(out), flush=True)
    if world > 1:
        import torch

        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
