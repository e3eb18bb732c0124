#!/usr/bin/env python3
"""FFNO3D forward + input-VJP throughput on GB300 (voxels/s).

Workload (the scaled configuration): FFNO3D width 64, 8 blocks, height operator with M = 32 modes
(z_min_wavelength = 40/31), H + Ca II level-fraction head (12 levels), one cube [1, 6, 256, 128, 128] = 4.19 M voxels,
synthetic seeded inputs with the reference's channel distributions, random-init weights of that architecture.

A step is one forward pass plus one input VJP over the cube (each block's intermediates kept from the forward when
they fit in half the free HBM, else recomputed block by block in the backward), inputs resident in HBM (value), in
the BF16 tensor-core form by default; the plain FP32 drop-in runs on the same cube for the speed-up and the BF16 error.
e2e is the same step through the service backend's vjp_local with host numpy buffers (host<->device copies inside the
timed region). The cube (GBs of activations) is far larger than L2, so no flush is needed between steps. The serving
stream (256 mixed-size PREDICT requests, Poisson arrivals at 40 per second) reports p50 / p99 latency.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference] [--precision fp32|bf16]

--impl reference times the reference algorithm's CPU implementation (the oracle port of the reference FFNO3D, float32
torch on the host cores) on a bounded sub-cube per step, same metric and unit.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WIDTH, LAYERS, MODES = 64, 8, 32
SHAPE = (256, 128, 128)
ATOMS = ["H", "CA"]
DXY = 48e3
MEAN_X = np.array([4.75, 0.0, 0.0, 0.0, 17.5, -8.0], np.float32)
STD_X = np.array([2.5 / math.sqrt(12), 5.0, 5.0, 5.0, 7.0 / math.sqrt(12), 8.0 / math.sqrt(12)], np.float32)
CPU_SAMPLE = (64, 32, 32)       # sub-cube per step of the reference arm and of cpu_baseline (same C, L, M)
CONFIG4 = (496, 252, 252)       # the full-volume inversion step (31.5 M voxels)
CONFIG0 = (64, 32, 32)          # the CPU-runnable forward: width 32, 4 blocks, M = 16, H
CONFIG3 = (256, 96, 96)         # the differentiation case: the width-64 model's fwd+VJP
STREAM_CHUNKS = (32, 16)        # depth planes / column rows per device slab of the host-RAM streaming forward
KERNELS_PER_CALL = {"ffno_column_info": 3, "ffno_outer": 2, "ffno_outer_tc": 2, "ffno_outer_tc_ld": 2}
METRIC = "FFNO3D voxels/s fwd & fwd+VJP, BF16 vs FP32 @ |\u0394log n|\u22642e-3; p50/p99 latency"


def model_config():
    return dict(width=WIDTH, n_layers=LAYERS, z_min_wavelength=40.0 / (MODES - 1))


def build_model(seed=0, **overrides):
    import torch
    from ffnoml_gb300 import create_ffno3d
    torch.manual_seed(seed)
    m = create_ffno3d(6, 12, atoms=ATOMS, **dict(model_config(), **overrides))
    with torch.no_grad():
        for name, p in m.named_parameters():
            if ".freq_u." in name:
                p.normal_(0.0, 0.1)
        c = 0
        for lv in m.species_levels:
            m.proj2.weight[c + lv].normal_(0.0, 0.3)
            m.proj2.bias[c + lv].normal_(0.0, 0.3)
            c += lv + 1
    m.set_normalization(MEAN_X, STD_X, np.zeros(12), np.ones(12))
    return m.eval()


def synthetic_si(shape, seed=1):
    """SI features (6, D, H, W), heights (D, H, W) in metres, as the service receives them."""
    D, H, W = shape
    g = np.random.default_rng(seed)
    f = np.empty((6, D, H, W), np.float32)
    f[0] = 10.0 ** g.uniform(3.5, 6.0, (D, H, W))
    f[1:4] = g.normal(0.0, 5e3, (3, D, H, W))
    f[4] = g.uniform(14.0, 21.0, (D, H, W))
    f[5] = g.uniform(-12.0, -4.0, (D, H, W))
    z = np.broadcast_to(np.linspace(14.0, -1.0, D, dtype=np.float32)[:, None, None] * 1e6, (D, H, W)).copy()
    return f, z


def per_column_heights(z):
    """Heights [1, D, H, W] (Mm) of the same span with every column's grid its own: each column stretched by up to
    +-2 % and shifted, so that no two columns share their tables."""
    import torch
    _, D, H, W = z.shape
    hh = torch.arange(H, dtype=torch.float32, device=z.device)[:, None]
    ww = torch.arange(W, dtype=torch.float32, device=z.device)[None, :]
    stretch = 1.0 + 0.02 * torch.sin(0.37 * hh + 0.23 * ww)
    shift = 0.05 * torch.cos(0.11 * hh - 0.19 * ww)
    return (z * stretch[None, None] + shift[None, None]).contiguous()


def per_column_run(model, x, z, cot, dev, world, timed):
    """fwd+VJP with per-column heights, and the time to build the per-column tables (device kernels, host prep)."""
    import torch
    ex = model.executor()
    zc = per_column_heights(z)
    geo = ex.geometry(zc)
    pk = ex.packed(dev)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    hgt = ex.height_percol(pk, geo, 0, dev)
    torch.cuda.synchronize(dev)
    build_s = time.perf_counter() - t0
    ms, _ = timed(lambda: ex.backward(ex.forward(x, zc, DXY, DXY, keep=True)[1], cot), 2, 1)
    V = x.shape[2] * x.shape[3] * x.shape[4]
    out = {"value": job_rate(V, world, ms / 1e3), "unit": "voxels/s", "ms_per_step": ms, "pass": "fwd+vjp",
           "columns": int(x.shape[3] * x.shape[4]), "live_modes": int(hgt["live"]),
           "tables_build_ms": 1e3 * build_s, "tables": "device (ffno_percol_tables), gradient ffno_percol_tables_vjp"}
    del hgt
    for key in [key for key in ex._height if key[0] == "percol"]:
        del ex._height[key]
    torch.cuda.empty_cache()
    return out


def normalised(f, z):
    """Model-unit, normalised inputs [1, 6, D, H, W] and z [1, D, H, W] in Mm (ffno_fsdp_runtime._model_inputs)."""
    m = f.astype(np.float64).copy()
    m[0] = np.log10(m[0])
    m[1:4] /= 1e3
    x = (m - MEAN_X[:, None, None, None]) / STD_X[:, None, None, None]
    return x[None].astype(np.float32), (z / 1e6)[None].astype(np.float32)


def dist_info():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def max_over_ranks(value, world, device):
    """The largest of every rank's value (a time: the job ends when its slowest replica does)."""
    if world <= 1:
        return float(value)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t)


def job_rate(units_per_rank, world, seconds):
    """Whole-job throughput of `world` replicas that each processed units_per_rank in (max-over-ranks) seconds."""
    return world * units_per_rank / seconds


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.out = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.out = [line.split(",") for line in out.strip().splitlines() if line.strip()]

    def summary(self):
        rows = [[c.strip() for c in r] for r in self.out if len(r) >= 9]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ---------------------------------------------------------------------------------------------------- CPU arms
def cpu_rate(model_state, shape, steps=1, warmup=0):
    """fwd+VJP voxels/s of the oracle port (float32 torch on the host cores) on a sub-cube."""
    import torch
    from ffnoml_gb300.config import species_of
    from oracle.ffno_oracle import OracleFFNO3D
    cfg = dict(model_config(), species=species_of(ATOMS), in_channels=6, out_channels=12)
    oracle = OracleFFNO3D(model_state, cfg, torch.float32, checkpoint_blocks=True)
    f, z = synthetic_si(shape, seed=3)
    x, zz = normalised(f, z)
    x = torch.from_numpy(x)
    zz = torch.from_numpy(zz)
    cot = torch.from_numpy(np.random.default_rng(4).normal(size=(1, 12) + shape).astype(np.float32))

    def step():
        xr = x.clone().requires_grad_(True)
        zr = zz.clone().requires_grad_(True)
        y = oracle.forward(xr, zr, DXY, DXY)
        torch.autograd.backward(y, cot)

    for _ in range(warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(steps):
        step()
    dt = time.perf_counter() - t0
    vox = shape[0] * shape[1] * shape[2]
    return vox * steps / dt, dt, torch.get_num_threads()


def cpu_forward_rate(model_state, cfg, shape, steps=1):
    """Forward voxels/s of the oracle port (float32 torch on the host cores, no autograd) on a whole cube."""
    import torch
    from oracle.ffno_oracle import OracleFFNO3D
    oracle = OracleFFNO3D(model_state, cfg, torch.float32, checkpoint_blocks=True)
    f, z = synthetic_si(shape, seed=3)
    x, zz = normalised(f, z)
    x, zz = torch.from_numpy(x), torch.from_numpy(zz)
    with torch.no_grad():
        t0 = time.perf_counter()
        for _ in range(steps):
            oracle.forward(x, zz, DXY, DXY)
        dt = time.perf_counter() - t0
    return shape[0] * shape[1] * shape[2] * steps / dt, dt, torch.get_num_threads()


def run_reference(args):
    import torch
    rank, world, _ = dist_info()
    if rank != 0:
        return
    torch.set_num_threads(len(os.sched_getaffinity(0)))
    model = build_model()
    state = {k: v.detach().clone() for k, v in model.state_dict().items()}
    rate, dt, cores = cpu_rate(state, CPU_SAMPLE, steps=args.steps, warmup=args.warmup)
    sample = (f"{CPU_SAMPLE[0]}x{CPU_SAMPLE[1]}x{CPU_SAMPLE[2]} sub-cube of the same model per step, fwd+VJP; "
              "the full cube's rate is extrapolated as this per-voxel rate")
    line = {"impl": "reference", "metric": METRIC, "value": rate, "unit": "voxels/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * dt / max(args.steps, 1), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "FFNO3D w64 L8 M32 H+CaII, [1,6,256,128,128], per-step sample " + sample,
                       "parallelism": "cpu"},
            "cpu_baseline": {"value": rate, "unit": "voxels/s", "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": rate, "unit": "voxels/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------------------------------- GPU arm
def algorithmic_flops_per_voxel(C, L, D, H, W, M, levels, species, r=8):
    """Forward MACs x 2 per voxel of the path (shared grid), the per-unit figure of the whole-step rate."""
    Wf = W // 2 + 1
    per_block = (31 * C * C + C + (4 * C * C + 4 * r * C) * Wf / W + 4 * M * C + (4 * C * C + 4 * r * C) * M / D)
    head = 6 * C + 2 * C * C + 2 * C * (levels + species)
    return 2 * (L * per_block + head)


def algorithmic(name, args):
    """(bytes, flops) one launch of entry point `name` must move and compute, from its own arguments: FP32 tensors read
    once and written once (weights and statistics omitted), GEMM flops counted once (the split-BF16 form issues three
    BF16 MMAs per product; that is not counted). None when the entry point has no formula here."""
    base = name.split(":")[0]
    nz = lambda a: 1 if a else 0
    if base in ("ffno_spectral_mix", "ffno_spectral_mix_tc"):
        F, nb, C, rank = args[2], args[3], args[7], args[12]
        rows = F * nb
        return 2 * rows * 2 * C * 4, rows * (8 * C * C + 8 * rank * C)
    if base in ("ffno_xform", "ffno_xform_tc"):
        d = args[3]
        batches = d.nb
        return 4 * batches * (d.K + d.M) * d.N, 2 * batches * d.M * d.K * d.N
    if base == "ffno_xform_tcr":
        d = args[5]
        return 4 * d.nb * (d.K + d.M) * d.N, 2 * d.nb * d.M * d.K * d.N
    if base == "ffno_xform_pt":
        d = args[4]
        batches = d.nb
        return 4 * batches * ((d.K + d.M) * d.N + d.M * d.K), 2 * batches * d.M * d.K * d.N
    if base == "ffno_mlp2_fwd_tc":
        V, C = args[6], args[7]
        return 4 * V * C * (1 + nz(args[2]) + 1 + nz(args[5])), 8 * V * C * C
    if base == "ffno_gate_fwd_tc":
        V, C = args[1], args[2]
        return 4 * V * C * 2 + 4 * V * nz(args[4]), 4 * V * C * C
    if base == "ffno_fuse1_tc":
        V, C = args[5], args[6]
        return 4 * V * C * (3 + 2 + nz(args[10])), 10 * V * C * C
    if base == "ffno_fuse2_tc":
        V, C = args[5], args[6]
        return 4 * V * C * (4 + 1), 12 * V * C * C
    if base == "ffno_mlp2_bwd_tc":
        V, C = args[3], args[4]
        return 4 * V * C * (2 + nz(args[2]) + 1), 12 * V * C * C
    if base == "ffno_gate_bwd_tc":
        V, C = args[3], args[4]
        return 4 * V * C * (2 + nz(args[2]) + 1) + 4 * V * 2 * nz(args[6]), 8 * V * C * C
    if base == "ffno_fuse_bwd_a_tc":
        V, C = args[6], args[7]
        return 4 * V * C * (5 + 2), 12 * V * C * C
    if base == "ffno_fuse_bwd_b_tc":
        V, C = args[9], args[10]
        return 4 * V * C * (9 + 3), 18 * V * C * C
    if base == "ffno_outer":
        R1, R2, N = args[2], args[5], args[6]
        return 4 * N * (R1 + R2), 2 * N * R1 * R2
    return None


def roofline_rows(per, peaks):
    """Achieved algorithmic GB/s and TFLOP/s of every entry point with a formula, its bound (the larger of bytes at
    the HBM peak and flops at the sustained BF16 peak) and the fraction of that peak."""
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    tf = float(peaks.get("bf16_tflops_sustained", 1700.0))
    rows = {}
    for name, (t_ms, n, nbytes, nflops) in per.items():
        if nbytes is None:
            continue
        sec = t_ms / 1e3
        gbs, tfs = nbytes / sec / 1e9, nflops / sec / 1e12
        hbm_bound = nbytes / (hbm * 1e9) >= nflops / (tf * 1e12)
        rows[name] = {"bound": "hbm" if hbm_bound else "tensor", "GB/s": round(gbs, 1), "TFLOP/s": round(tfs, 2),
                      "frac": round(gbs / hbm if hbm_bound else tfs / tf, 4), "avg_launch_ms": round(t_ms / n, 4),
                      "launches": n, "bytes_per_launch": int(nbytes / n), "flops_per_launch": int(nflops / n)}
    return rows


def dram_traffic(kernel, nbytes_per_launch):
    """DRAM bytes per launch of `kernel` at the benchmark's size: the ratio of ncu's dram__bytes_read + write to the
    algorithmic bytes measured on a smaller capture (profiles/dram_traffic.json), times this launch's algorithmic
    bytes (the traffic of these kernels grows in proportion to the rows they process). None without a capture."""
    try:
        with open(os.path.join(ROOT, "profiles", "dram_traffic.json")) as fh:
            table = json.load(fh)
    except (OSError, ValueError):
        return None, None
    rec = table.get(kernel.split(":")[0])
    if not rec:
        return None, None
    ratio = rec["dram_bytes"] / rec["algorithmic_bytes"]
    return ratio * nbytes_per_launch, rec.get("case")


def population_mesh_rate(dev, nz=95, nx=256, ny=256, levels=12, reps=5):
    """Columns per second of the population-mesh features map plus the back-map (and of their VJP) on a synthetic
    log-tau cube: nz points per column (log tau500 -6 .. 1.4), heights varying by column, the default fixed mesh."""
    import torch
    from ffnoml_gb300.population_mesh import MeshMaps, PopulationMeshConfig, population_mesh
    g = np.random.default_rng(11)
    ncol = nx * ny
    tau = 10.0 ** np.linspace(-6.0, 1.4, nz)
    scale = 1 + 0.05 * g.random(ncol)
    z = -1.2e5 * np.log(tau)[None, :] * scale[:, None] + 2e4 * g.random(ncol)[:, None]
    atm = np.empty((6, ncol, nz))
    atm[0] = (4300 + 1700 * tau ** 0.25)[None] * scale[:, None]
    atm[1:4] = g.normal(0, 3e3, (3, ncol, nz))
    atm[4] = 19 + 0.6 * np.log10(tau)[None] + 0.01 * g.random((ncol, nz))
    atm[5] = -3.5 + 0.45 * np.log10(tau)[None] + 0.01 * g.random((ncol, nz))
    mesh = population_mesh(PopulationMeshConfig())
    maps = MeshMaps(z, mesh, dev)
    at = torch.as_tensor(atm, device=dev)
    pm = torch.exp(torch.randn(levels, ncol, len(mesh), dtype=torch.float64, device=dev))
    pb = torch.randn(levels, ncol, nz, dtype=torch.float64, device=dev)

    def fwd():
        f, _ = maps.features(at)
        return f, maps.backmap(pm)

    def vjp(f):
        maps.backmap_vjp(pm, pb)
        maps.features_vjp(at, f, torch.ones_like(f))

    f, _ = fwd()
    vjp(f)
    torch.cuda.synchronize()
    a, b, c = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    a.record()
    for _ in range(reps):
        fwd()
    b.record()
    for _ in range(reps):
        vjp(f)
    c.record()
    torch.cuda.synchronize()
    tf, tv = a.elapsed_time(b) / reps, b.elapsed_time(c) / reps
    return {"value": ncol / (tf / 1e3), "unit": "columns/s", "ms_per_step": tf, "vjp_ms": tv, "columns": ncol,
            "column_points": nz, "mesh_points": len(mesh), "levels": levels, "dtype": "f64",
            "workload": f"{nx}x{ny} log-tau columns of {nz} points onto the default fixed mesh and back"}


def run_gb300(args):
    import torch
    import torch.distributed as dist
    from ffnoml_gb300 import _native as nat
    from ffnoml_gb300.runtime import GB300Backend

    rank, world, local = dist_info()
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    model = build_model().to(dev).set_precision(args.precision)
    D, H, W = args.shape
    V = D * H * W
    f_np, z_np = synthetic_si((D, H, W), seed=1 + rank)
    x_np, z_mm = normalised(f_np, z_np)
    x = torch.from_numpy(x_np).to(dev)
    z = torch.from_numpy(z_mm).to(dev)
    cot = torch.from_numpy(np.random.default_rng(2 + rank).normal(size=(1, 12, D, H, W)).astype(np.float32)).to(dev)
    ex = model.executor()

    def fwd_vjp():
        y, st = ex.forward(x, z, DXY, DXY, keep=True)
        ex.backward(st, cot)

    def fwd():
        ex.forward(x, z, DXY, DXY)

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    def timed(fn, steps, warmup):
        for _ in range(warmup):
            fn()
        barrier()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        calls0 = nat.counter.calls
        a.record()
        for _ in range(steps):
            fn()
        b.record()
        barrier()
        ms = max_over_ranks(a.elapsed_time(b), world, dev)
        return ms / steps, nat.counter.calls - calls0

    # fwd+VJP at the headline precision, device-resident (--fwd-only: the forward alone, a profiling case)
    step = fwd if args.fwd_only else fwd_vjp
    torch.cuda.reset_peak_memory_stats(dev)
    with ClockSampler(local) as clk:
        ms_step, calls = timed(step, args.steps, args.warmup)
    clocks = clk.summary()
    cached_states = ex.last_cached
    memory = {"peak_allocated_gib": torch.cuda.max_memory_allocated(dev) / 2 ** 30,
              "device_total_gib": torch.cuda.get_device_properties(dev).total_memory / 2 ** 30}
    ms_fwd = ms_step if args.fwd_only else timed(fwd, max(args.steps, 3), 1)[0]

    # kernel breakdown of one step (CUDA events around every entry point on the launching stream)
    nat.counter.timing = []
    step()
    torch.cuda.synchronize()
    per = {}
    for name, e0, e1, cargs in nat.counter.timing:
        t, n, nb, nf = per.get(name, (0.0, 0, 0, 0))
        alg = algorithmic(name, cargs)
        per[name] = (t + e0.elapsed_time(e1), n + 1, None if alg is None or nb is None else nb + alg[0],
                     None if alg is None or nf is None else nf + alg[1])
    nat.counter.timing = None
    launches = sum(KERNELS_PER_CALL.get(k.split(":")[0], 1) * v[1] for k, v in per.items())
    total = sum(v[0] for v in per.values())
    breakdown = {k: {"ms": round(v[0], 3), "launches": v[1], "share": round(v[0] / total, 4)}
                 for k, v in sorted(per.items(), key=lambda kv: -kv[1][0])}

    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            peaks = json.load(fh)
    except OSError:
        pass
    rows = roofline_rows(per, peaks)
    top = max(rows, key=lambda k: per[k][0])
    r = rows[top]
    hbm_b = r["bound"] == "hbm"
    traffic, traffic_case = dram_traffic(top, r["bytes_per_launch"])
    roof = {"kernel": top, "bound": r["bound"], "achieved": r["GB/s"] if hbm_b else r["TFLOP/s"],
            "peak": float(peaks.get("hbm_gbs", 6800.0)) if hbm_b else float(peaks.get("bf16_tflops_sustained", 1700.0)),
            "unit": "GB/s" if hbm_b else "TFLOP/s", "frac": r["frac"], "traffic": traffic,
            "traffic_source": traffic_case, "algorithmic_bytes_per_launch": r["bytes_per_launch"],
            "avg_launch_ms": r["avg_launch_ms"],
            "peak_source": ("of measured (hbm_gbs)" if hbm_b else "of measured (bf16_tflops_sustained)")
            if peaks else "of fallback"}

    # the plain FP32 drop-in on the same cube, and the BF16 error against it
    fp32 = None
    if args.fwd_only:
        args.no_fp32 = args.no_e2e = args.no_cpu_baseline = args.no_serve = True
    if args.precision == "bf16" and not args.no_fp32:
        with torch.no_grad():
            y16 = ex.forward(x, z, DXY, DXY)[0]
            model.set_precision("fp32")
            y32 = ex.forward(x, z, DXY, DXY)[0]
            dlog = float((y16 - y32).abs().max())
        del y16, y32
        ms32, _ = timed(fwd_vjp, max(2, args.steps // 2), 1)
        ms32f, _ = timed(fwd, max(2, args.steps // 2), 1)
        model.set_precision("bf16")
        fp32 = {"fwd+vjp": {"value": job_rate(V, world, ms32 / 1e3), "unit": "voxels/s", "ms_per_step": ms32},
                "fwd": {"value": job_rate(V, world, ms32f / 1e3), "unit": "voxels/s", "ms_per_step": ms32f},
                "bf16_speedup_fwd+vjp": ms32 / ms_step, "bf16_speedup_fwd": ms32f / ms_fwd,
                "max_abs_dlog10n_bf16_vs_fp32": dlog}

    # forward-mode derivative (JVP, FP32 tangent kernels) along a seeded input tangent, inputs resident
    jvp = None
    if not args.no_jvp and not args.fwd_only:
        xdot = torch.from_numpy(np.random.default_rng(6 + rank).normal(size=x.shape).astype(np.float32)).to(dev)
        ms_jvp, _ = timed(lambda: ex.jvp(x, z, DXY, DXY, xdot), 2, 1)
        jvp = {"value": job_rate(V, world, ms_jvp / 1e3), "unit": "voxels/s", "ms_per_step": ms_jvp,
               "dtype": "f32"}

    # e2e through the service backend with host buffers
    e2e = None
    if not args.no_e2e:
        backend = GB300Backend(model, [f"l{i}" for i in range(12)], device=dev)
        cot_np = np.random.default_rng(5).normal(size=(D, H, W, 12)).astype(np.float32)
        for _ in range(max(1, min(args.warmup, 2))):
            backend.vjp_local(f_np, z_np, DXY, DXY, cot_np)
        barrier()
        t0 = time.perf_counter()
        n_e2e = max(1, min(args.steps, 3))
        for _ in range(n_e2e):
            backend.vjp_local(f_np, z_np, DXY, DXY, cot_np)
        barrier()
        e2e_s = max_over_ranks((time.perf_counter() - t0) / n_e2e, world, dev)
        e2e = {"value": job_rate(V, world, e2e_s), "unit": "voxels/s", "h2d_bytes_per_step": int(f_np.nbytes + z_np.nbytes +
                                                                                            cot_np.nbytes),
               "d2h_bytes_per_step": int(f_np.nbytes + z_np.nbytes), "ms_per_step": 1e3 * e2e_s}

    # the host-RAM streaming forward on the same cube (hidden states in pinned host memory, slabs on the device)
    streaming = None
    if not args.no_streaming and not args.fwd_only:
        from ffnoml_gb300.streaming import StreamingForward
        sfw = StreamingForward(model, chunk_depth=STREAM_CHUNKS[0], chunk_rows=STREAM_CHUNKS[1])
        sfw(f_np, z_np, DXY, DXY)
        barrier()
        t0 = time.perf_counter()
        n_s = max(1, min(args.steps, 2))
        for _ in range(n_s):
            sfw(f_np, z_np, DXY, DXY)
        barrier()
        st = max_over_ranks((time.perf_counter() - t0) / n_s, world, dev)
        streaming = {"value": job_rate(V, world, st), "unit": "voxels/s", "ms_per_step": 1e3 * st, "pass": "forward",
                     "chunk_depth": STREAM_CHUNKS[0], "chunk_rows": STREAM_CHUNKS[1], "slabs_per_step": sfw.slabs,
                     "host_hidden_bytes": 4 * V * WIDTH * 4, "h2d_bytes_per_step": int(f_np.nbytes + z_np.nbytes),
                     "d2h_bytes_per_step": int(V * 12 * 4)}
        del sfw

    # population-mesh maps (FP64): a log-tau cube's columns onto the default fixed mesh and the populations back
    mesh_maps = None
    if not args.fwd_only:
        mesh_maps = population_mesh_rate(dev)

    # production variant P: the same model with the height operator at its production band limit (M = 1001, 340
    # live modes at D = 256), fwd+VJP at the headline precision on the same cube
    variant_p = None
    if not args.no_variant_p and not args.fwd_only:
        mp = build_model(z_min_wavelength=0.04).to(dev).set_precision(args.precision)
        exp = mp.executor()
        ms_p, _ = timed(lambda: exp.backward(exp.forward(x, z, DXY, DXY, keep=True)[1], cot), 2, 1)
        hp = exp.height(exp.packed(dev), exp.geometry(z), dev)
        variant_p = {"value": job_rate(V, world, ms_p / 1e3), "unit": "voxels/s", "ms_per_step": ms_p,
                     "modes": mp.blocks[0].vertical.modes, "live_modes": int(hp["live"]), "pass": "fwd+vjp"}
        del mp, exp, hp
        torch.cuda.empty_cache()

    # the production model (width 96, 4 blocks, hidden 128, M = 1001, H: the reference's MODEL_CONFIG defaults) on the
    # same cube, fwd+VJP in both precisions: at width 96 the "bf16" form runs every kernel family on the tensor cores
    # (width-96 forms of the channel kernels)
    production = None
    if not args.no_production and not args.fwd_only:
        production = production_run(x, z, dev, world, timed)

    # per-column height grids (every column its own heights: the height operator's non-shared path) on the same
    # cube: the per-column tables built on the device once (timed alone), then fwd+VJP steps with them, the tables'
    # gradient for every column included
    per_column = None
    if not args.no_per_column and not args.fwd_only:
        per_column = per_column_run(model, x, z, cot, dev, world, timed)

    # config 4: the full-volume inversion step [1,6,496,252,252] on this GPU (block states recomputed), with the BF16
    # forward against the FP32 forward on the whole cube
    config4 = None
    if not args.no_config4 and not args.fwd_only:
        config4 = config4_run(model, ex, dev, world, rank, timed)

    # configs 0 and 3 of the benchmark table: the small width-32 forward (with the oracle port's forward of the same
    # cube on the host cores) and the width-64 model's fwd+VJP on [1,6,256,96,96]
    configs = None
    if not args.no_configs and not args.fwd_only:
        configs = configs_run(model, dev, world, rank, timed, with_cpu=not args.no_cpu_baseline)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        torch.set_num_threads(len(os.sched_getaffinity(0)))
        state = {k: v.detach().cpu().clone() for k, v in model.state_dict().items()}
        S = CPU_SAMPLE
        rate, dt, cores = cpu_rate(state, S, steps=1, warmup=0)
        cpu = {"value": rate, "unit": "voxels/s", "cores": cores, "kind": "port",
               "sample": f"{S[0]}x{S[1]}x{S[2]} sub-cube of the same model, one fwd+VJP "
                         f"({dt:.1f} s), oracle port of the reference FFNO3D in float32 torch; the full cube's rate "
                         "is extrapolated as this per-voxel rate"}

    serving = None
    if rank == 0 and not args.no_serve:
        serving = serving_stream(model, args.serve_requests, 40.0)
        # inversion requests are VJPs: the same size mix at a rate the device can follow
        serving["vjp_stream"] = serving_stream(model, max(16, args.serve_requests // 4), 5.0, seed=17, op="VJP")

    flops_vox = algorithmic_flops_per_voxel(WIDTH, LAYERS, D, H, W, MODES, 12, 2)
    if rank == 0:
        line = {
            "metric": METRIC, "value": job_rate(V, world, ms_step / 1e3), "unit": "voxels/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32" if args.precision == "fp32" else "bf16", "data": "synthetic",
            "config": {"workload": f"FFNO3D w{WIDTH} L{LAYERS} M{MODES} H+CaII, [1,6,{D},{H},{W}] " +
                                   ("forward only" if args.fwd_only else "fwd + input VJP (block states " +
                                    ("kept from the forward)" if cached_states else "recomputed per block)")),
                       "voxels_per_step": V, "parallelism": f"replicas{world}",
                       "l2": "working set (GBs) >> L2; no flush needed", "precision": args.precision},
            "fwd": {"value": job_rate(V, world, ms_fwd / 1e3), "unit": "voxels/s", "ms_per_step": ms_fwd},
            "fp32": fp32, "jvp": jvp,
            "algorithmic_tflops": {"fwd+vjp": 2 * flops_vox * V / (ms_step / 1e3) / 1e12,
                                   "fwd": flops_vox * V / (ms_fwd / 1e3) / 1e12},
            "roofline": roof, "roofline_by_entry": dict(sorted(rows.items(), key=lambda kv: -per[kv[0]][0])[:12]),
            "kernel_breakdown_ms": breakdown,
            "clocks": clocks, "memory": memory, "gpu_launches": launches * args.steps, "e2e": e2e,
            "cpu_baseline": cpu,
            "serving": serving, "streaming": streaming, "population_mesh": mesh_maps,
            "variant_p": variant_p, "per_column": per_column, "config4": config4, "production": production,
            "configs": configs,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def entry_breakdown(step, top):
    """CUDA-event milliseconds per entry point (tagged per call site) over one run of step(): the `top` largest."""
    import torch
    from ffnoml_gb300 import _native as nat
    nat.counter.timing = []
    step()
    torch.cuda.synchronize()
    per = {}
    for name, e0, e1, _ in nat.counter.timing:
        per[name] = per.get(name, 0.0) + e0.elapsed_time(e1)
    nat.counter.timing = None
    return {k: round(v, 2) for k, v in sorted(per.items(), key=lambda kv: -kv[1])[:top]}


def production_run(x, z, dev, world, timed):
    """fwd+VJP of the production model (create_ffno3d defaults: width 96, 4 blocks, M = 1001, H atom) on the cube
    x, z, 2 timed steps in FP32 and in "bf16" (every kernel family on tensor cores, the channel kernels in their
    width-96 forms), with the largest |d log10 n| between the two forwards."""
    import torch
    from ffnoml_gb300 import create_ffno3d
    torch.manual_seed(5)
    m = create_ffno3d(6, 6).to(dev).eval()
    with torch.no_grad():
        for name, p in m.named_parameters():
            if ".freq_u." in name:
                p.normal_(0.0, 0.1)
    m.set_normalization(MEAN_X, STD_X, np.zeros(6), np.ones(6))
    D, H, W = x.shape[2:]
    V = D * H * W
    cot = torch.randn((1, 6, D, H, W), generator=torch.Generator(dev).manual_seed(21), device=dev)
    ex = m.executor()
    out = {"model": "width 96, 4 blocks, hidden 128, M = 1001, H (6 levels)", "shape": [D, H, W]}
    ys = {}
    step = lambda: ex.backward(ex.forward(x, z, DXY, DXY, keep=True)[1], cot)
    for prec in ("fp32", "bf16"):
        m.set_precision(prec)
        ms, _ = timed(step, 2, 1)
        out[prec] = {"value": job_rate(V, world, ms / 1e3), "unit": "voxels/s", "ms_per_step": ms, "pass": "fwd+vjp",
                     "top_entries_ms": entry_breakdown(step, 8)}
        with torch.no_grad():
            ys[prec] = ex.forward(x, z, DXY, DXY)[0]
    hp = ex.height(ex.packed(dev), ex.geometry(z), dev)
    out["live_modes"] = int(hp["live"])
    m.set_precision("bf16")
    out["tensor_cores"] = {"width_16_64_kernels": bool(ex.packed(dev).tc), "width_96_kernels": bool(ex._tc_fuse96()),
                           "transforms": bool(ex._tc_xf())}
    out["bf16_speedup"] = out["fp32"]["ms_per_step"] / out["bf16"]["ms_per_step"]
    out["max_abs_dlog10n_bf16_vs_fp32"] = float((ys["bf16"] - ys["fp32"]).abs().max())
    del m, ex, ys, hp, cot
    torch.cuda.empty_cache()
    return out


def configs_run(model, dev, world, rank, timed, with_cpu):
    """Config 0 (width 32, 4 blocks, M = 16, H; [1,6,64,32,32]): the forward on this GPU in FP32 and BF16 (20 timed
    steps) and, on rank 0, the oracle port's FP32 forward of the same whole cube on the host cores. Config 3 (the
    headline model on [1,6,256,96,96], cotangent N(0, 1)): fwd+VJP at the model's precision (3 timed steps)."""
    import torch
    from ffnoml_gb300 import create_ffno3d
    from ffnoml_gb300.config import species_of
    cfg0 = dict(width=32, n_layers=4, z_min_wavelength=40.0 / 15)
    torch.manual_seed(20)
    m0 = create_ffno3d(6, 6, atoms=["H"], **cfg0)
    with torch.no_grad():
        for name, p in m0.named_parameters():
            if ".freq_u." in name:
                p.normal_(0.0, 0.1)
    m0.set_normalization(MEAN_X, STD_X, np.zeros(6), np.ones(6))
    state0 = {k: v.detach().clone() for k, v in m0.state_dict().items()}
    m0 = m0.eval().to(dev)
    ex0 = m0.executor()
    V0 = CONFIG0[0] * CONFIG0[1] * CONFIG0[2]
    f_np, z_np = synthetic_si(CONFIG0, seed=21 + rank)
    x_np, z_mm = normalised(f_np, z_np)
    x0, z0 = torch.from_numpy(x_np).to(dev), torch.from_numpy(z_mm).to(dev)
    c0 = {"shape": list(CONFIG0), "model": "width 32, 4 blocks, M = 16, H (6 levels)", "pass": "forward"}
    for prec in ("fp32", "bf16"):
        m0.set_precision(prec)
        ms, _ = timed(lambda: ex0.forward(x0, z0, DXY, DXY), 20, 3)
        c0[prec] = {"value": job_rate(V0, world, ms / 1e3), "unit": "voxels/s", "ms_per_step": ms}
    if with_cpu and rank == 0:
        torch.set_num_threads(len(os.sched_getaffinity(0)))
        cfg = dict(cfg0, species=species_of(["H"]), in_channels=6, out_channels=6)
        rate, dt, cores = cpu_forward_rate(state0, cfg, CONFIG0, steps=2)
        c0["cpu"] = {"value": rate, "unit": "voxels/s", "cores": cores, "kind": "port", "seconds": dt,
                     "sample": "the whole cube, two forwards, oracle port of the reference FFNO3D in float32 torch"}
    del m0, ex0, x0, z0
    D, H, W = CONFIG3
    V3 = D * H * W
    f_np, z_np = synthetic_si(CONFIG3, seed=31 + rank)
    x_np, z_mm = normalised(f_np, z_np)
    x3, z3 = torch.from_numpy(x_np).to(dev), torch.from_numpy(z_mm).to(dev)
    cot3 = torch.randn((1, 12, D, H, W), generator=torch.Generator(dev).manual_seed(32 + rank), device=dev)
    ex = model.executor()
    ms, _ = timed(lambda: ex.backward(ex.forward(x3, z3, DXY, DXY, keep=True)[1], cot3), 3, 1)
    c3 = {"shape": list(CONFIG3), "model": f"width {WIDTH}, {LAYERS} blocks, M = {MODES}, H + Ca II",
          "pass": "fwd+vjp", "precision": model.precision, "value": job_rate(V3, world, ms / 1e3), "unit": "voxels/s",
          "ms_per_step": ms}
    del x3, z3, cot3
    torch.cuda.empty_cache()
    return {"config0": c0, "config3": c3}


def config4_run(model, ex, dev, world, rank, timed):
    """fwd+VJP of the full-volume cube at the model's precision (2 timed steps), its peak device memory, and the
    largest |d log10 n| between the BF16 and the FP32 forward on the whole cube."""
    import torch
    D, H, W = CONFIG4
    V = D * H * W
    torch.cuda.empty_cache()
    f_np, z_np = synthetic_si(CONFIG4, seed=11 + rank)
    x_np, z_mm = normalised(f_np, z_np)
    del f_np, z_np
    x = torch.from_numpy(x_np).to(dev)
    z = torch.from_numpy(z_mm).to(dev)
    del x_np, z_mm
    cot = torch.randn((1, 12, D, H, W), generator=torch.Generator(dev).manual_seed(12 + rank), device=dev)
    precision = model.precision
    out = {"shape": list(CONFIG4), "voxels": V}
    try:
        torch.cuda.reset_peak_memory_stats(dev)
        ms, _ = timed(lambda: ex.backward(ex.forward(x, z, DXY, DXY, keep=True)[1], cot), 2, 1)
        out.update({"value": job_rate(V, world, ms / 1e3), "unit": "voxels/s", "ms_per_step": ms,
                    "pass": "fwd+vjp", "precision": precision, "block_states": "kept" if ex.last_cached else
                    "recomputed per block", "peak_allocated_gib": torch.cuda.max_memory_allocated(dev) / 2 ** 30})
        if precision == "bf16":
            with torch.no_grad():
                y16 = ex.forward(x, z, DXY, DXY)[0]
                model.set_precision("fp32")
                try:
                    y32 = ex.forward(x, z, DXY, DXY)[0]
                finally:
                    model.set_precision(precision)
                out["max_abs_dlog10n_bf16_vs_fp32"] = float((y16 - y32).abs().max())
            del y16, y32
    except torch.cuda.OutOfMemoryError as e:
        out["error"] = "out of device memory: " + str(e).splitlines()[0]
    del x, z, cot
    torch.cuda.empty_cache()
    return out


def serving_stream(model, n_requests, rate, seed=7, slots=4, connections=8, op="PREDICT"):
    """The mixed-size request stream: Poisson arrivals at `rate` per second, D in {128, 192, 256}, H = W in
    {32, 64, 96, 128}, PREDICT (or VJP, with a seeded population cotangent) over the protocol-v2 service (each request
    on one of `connections` client connections). Returns p50 / p99 latency (send to reply), aggregate voxels/s, and
    the server's mean queue wait and service time per request."""
    import threading
    import queue as q

    from ffnoml_gb300.runtime import GB300Backend
    from ffnoml_gb300.service import Client, Server

    backend = GB300Backend(model, [f"l{i}" for i in range(12)])
    srv = Server({"HCA": backend}, "bench", slots=slots)
    srv.start()
    g = np.random.default_rng(seed)
    sizes = [(int(g.choice([128, 192, 256])), int(s), int(s)) for s in g.choice([32, 64, 96, 128], n_requests)]
    gaps = g.exponential(1.0 / rate, n_requests)
    inputs = {}
    for sh in set(sizes):
        f, z = synthetic_si(sh, seed=11)
        extra = ()
        if op == "VJP":
            extra = (np.random.default_rng(13).normal(size=sh + (12,)).astype(np.float32) * np.float32(1e-15),)
        inputs[sh] = (f, z) + extra
    # warm every shape once (tables and packs are built on first use)
    c = Client(srv.port, "bench")
    for sh in set(sizes):
        c.request(op, "HCA", inputs[sh][0], inputs[sh][1], DXY, DXY, 12, *inputs[sh][2:])
    c.close()
    srv.scheduler.completed.clear()
    work = q.Queue()
    lat = [None] * n_requests

    # each shape's request bytes are encoded once: the clients (threads of this process, like the server) only send
    # bytes and read the reply's bytes, so that the measured time is the server's
    encoded = {sh: Client.encode(op, "HCA", a[0], a[1], DXY, DXY, 12, *a[2:]) for sh, a in inputs.items()}
    reply_floats = {sh: (7 if op == "VJP" else 12) * sh[0] * sh[1] * sh[2] for sh in inputs}

    def client_loop():
        cl = Client(srv.port, "bench")
        into = bytearray(4 * max(reply_floats.values()))
        while True:
            item = work.get()
            if item is None:
                break
            i, t_send = item
            wait = t_send - time.perf_counter()
            if wait > 0:
                time.sleep(wait)
            t0 = time.perf_counter()
            cl.request_raw(encoded[sizes[i]], 4 * reply_floats[sizes[i]], into)
            lat[i] = time.perf_counter() - t0
        cl.close()

    threads = [threading.Thread(target=client_loop) for _ in range(connections)]
    for t in threads:
        t.start()
    t_begin = time.perf_counter()
    t = t_begin
    for i in range(n_requests):
        t += gaps[i]
        work.put((i, t))
    for _ in threads:
        work.put(None)
    for t_ in threads:
        t_.join()
    elapsed = time.perf_counter() - t_begin
    done = list(srv.scheduler.completed)
    srv.shutdown()
    vox = sum(d * h * w for d, h, w in sizes)
    lat_ms = np.array(lat) * 1e3
    wait_ms = [1e3 * (r.t_start - r.t_arrive) for r in done if r.t_start]
    serve_ms = [1e3 * (r.t_done - r.t_start) for r in done if r.t_start]
    return {"requests": n_requests, "rate_per_s": rate, "slots": slots, "op": op,
            "p50_ms": float(np.percentile(lat_ms, 50)), "p99_ms": float(np.percentile(lat_ms, 99)),
            "voxels_per_s": vox / elapsed, "wall_s": elapsed,
            "offered_voxels_per_s": vox / float(np.sum(gaps)),
            "server_mean_queue_ms": float(np.mean(wait_ms)) if wait_ms else None,
            "server_mean_service_ms": float(np.mean(serve_ms)) if serve_ms else None,
            "server_busy_slot_s": float(np.sum(serve_ms)) / 1e3 if serve_ms else None}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="bf16", choices=["fp32", "bf16"])
    ap.add_argument("--no-fp32", action="store_true", help="skip the FP32 comparison run")
    ap.add_argument("--fwd-only", action="store_true", help="time the forward pass alone (profiling cases)")
    ap.add_argument("--no-jvp", action="store_true", help="skip the forward-mode derivative timing")
    ap.add_argument("--shape", default="256,128,128")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--no-streaming", action="store_true", help="skip the host-RAM streaming forward")
    ap.add_argument("--no-config4", action="store_true", help="skip the full-volume [1,6,496,252,252] step")
    ap.add_argument("--no-variant-p", action="store_true", help="skip the production band limit (M = 1001) step")
    ap.add_argument("--no-production", action="store_true",
                    help="skip the production model (width 96, M = 1001) steps")
    ap.add_argument("--no-per-column", action="store_true", help="skip the per-column height grid step")
    ap.add_argument("--no-configs", action="store_true", help="skip the config 0 forward and the config 3 fwd+VJP")
    ap.add_argument("--serve-requests", type=int, default=256)
    args = ap.parse_args()
    args.shape = tuple(int(v) for v in args.shape.split(","))
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
