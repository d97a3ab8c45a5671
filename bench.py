"""Benchmark of the exodus box path on GB300: Mparticles/s at 512^3.

One step is the whole path over one box: CIC deposit, density contrast,
chain-mesh build, and the finder over the 19-rung ladder (per rung: filter +
C2R, candidate scan, pre-filter, sphere growth, commit), ending with the
catalogue on the host.

- ``value``: the step on particles already resident in HBM
  (sifg_box_device), timed with CUDA events on the library's own stream.
- ``e2e``: the same step through sif's C API with host buffers
  (sif_grid_assign_cic, sif_grid_to_density_contrast, sif_chain_mesh_alloc,
  sif_finder_exodus_raw), every host<->device copy inside the timed region.
- ``cpu_baseline``: the CPU restatement of the reference's path (oracle/,
  its release-flags build) with all host cores, on the same 512^3 workload:
  one whole-path run, and the same with the FFT stage taken out.

- ``fp64_form``: the same step in the FP64 form (sifg_box_device_f64: the
  reference's SIF_USE_DOUBLE arithmetic), the form the float path is
  measured against.
- ``batched_form``: 64 boxes of 64^3-256^3 particles through
  sifg_box_batch_device (engines run concurrently, their count autotuned).
- ``adjoint``: the differentiation workload (256^3 particles, box 500,
  grid 256^3, Gaussian R = 5): forward (deposit + contrast + smoothing) and
  backward (smoothing of the gradient + the deposit's adjoint) times.

``--impl reference`` times that CPU path alone (the reference arm), on the
same workload.
Under torchrun every rank runs its own replica (the path does not shard).
"""
import argparse
import ctypes as C
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
sys.path.insert(0, os.path.join(ROOT, "oracle"))

METRIC = "exodus Mparticles/s at 512^3"
UNIT = "Mparticles/s"

# The 512^3 workload: Zel'dovich lattice, box 1000 Mpc/h, rms displacement 5,
# seed 1002; grid 512^3; mesh cells of 8 Mpc/h; ladder(4, 24, 0.10);
# threshold -0.8; excursion-set variant.
WORKLOAD = dict(name="B", n=512, box=1000.0, rms=5.0, seed=1002, grid=512, mesh=125, r0=4.0,
                threshold=-0.8)


WORKLOAD_NAME = ("512^3 particles, box 1000 Mpc/h, grid 512^3, mesh 125^3 (8 Mpc/h), "
                 "ladder(4, 24, 0.10) 19 rungs, threshold -0.8, excursion-set")


def radii_of(w):
    from sif_gb300 import synth

    return synth.ladder(w["r0"], 6.0 * w["r0"], 0.10).astype(np.float32)


def small_workload():
    return dict(name="A-small", n=128, box=500.0, rms=4.0, seed=1001, grid=128, mesh=50, r0=5.0,
                threshold=-0.8)


# --------------------------------------------------------------------------
# clocks
# --------------------------------------------------------------------------

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        import tempfile

        try:
            fd, self.path = tempfile.mkstemp(prefix="sif_gb300_clocks_", suffix=".csv")
            self.f = os.fdopen(fd, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.path:
            self.f.close()
            with open(self.path) as f:
                self.lines = f.readlines()
            os.unlink(self.path)

    def summary(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": sorted(reasons),
                "samples": len(sm)}


# --------------------------------------------------------------------------
# the GPU arm
# --------------------------------------------------------------------------

def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profiled_traffic(kernel):
    """DRAM bytes per launch of `kernel` from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", f"{kernel}.md")
    try:
        for line in open(path):
            if line.startswith("dram_bytes_per_launch_full_size:"):
                return float(line.split(":", 1)[1].split()[0])
    except OSError:
        pass
    return None


def gpu_arm(args, rank, world):
    import torch

    from sif_gb300 import abi, build, device, pysif, synth

    build.build()
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    pysif.system_init(log_level="error")
    w = small_workload() if args.small else WORKLOAD
    radii = radii_of(w)
    x, y, z = synth.zeldovich(w["n"], w["box"], w["rms"], w["seed"], backend="torch")
    n = len(x)
    xs = [torch.from_numpy(a).cuda() for a in (x, y, z)]
    torch.cuda.synchronize()
    stream = device.stream()

    def step():
        return device.box(*xs, w["grid"], w["box"], w["mesh"], radii, w["threshold"])

    for _ in range(args.warmup):
        cat = step()
    n_voids = len(cat[0])
    launches0 = device.launch_count()
    timings = []
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    with ClockSampler(torch.cuda.current_device()) as clocks:
        start.record(stream)
        for _ in range(args.steps):
            step()
        end.record(stream)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
    ms = start.elapsed_time(end) / args.steps
    launches = (device.launch_count() - launches0) // args.steps
    # The last step's kernel timings, read after the timed region.
    timings.append(device.last_timings())
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    value = world * n / (ms / 1e3) / 1e6

    # Roofline of the dominant kernel of the step, from the last step's events.
    tm = timings[-1]
    peak, peak_kind = peaks()
    kernels = {
        "growth_kernel": (tm["growth_ms"], tm["growth_launches"],
                          12.0 * tm["growth_particles"] + 16.0 * tm["growth_cells"]),
        "tile_deposit_kernel": (tm["cic_ms"], tm["cic_launches"],
                                12.0 * n + 4.0 * w["grid"] ** 3),
        # The whole deposit stage (tile count, scan, tile scatter, deposit,
        # faces' fix-up) on the same algorithmic bytes.
        "cic_stage": (tm["cic_stage_ms"], 1 if tm["cic_stage_ms"] > 0 else 0,
                      12.0 * n + 4.0 * w["grid"] ** 3),
        # The kernel that applies the filter: at a 512^3 grid the first pass of
        # the float form's own inverse transform (filter + kx FFT), else the
        # filter kernel ahead of cuFFT's C2R. Either reads the spectrum once
        # and writes the transform's input once: 16 B per mode.
        ("colfft512_kernel" if w["grid"] == 512 else "filter_kernel"): (
            tm["filter_ms"], tm["filter_launches"],
            tm["filter_launches"] * 16.0 * w["grid"] ** 2 * (w["grid"] // 2 + 1)),
    }
    dom = max((k for k in kernels if k != "cic_stage"), key=lambda k: kernels[k][0])
    rooflines = {}
    for k, (kms, kl, kbytes) in kernels.items():
        if kl == 0 or kms <= 0:
            continue
        per_launch = kbytes / kl
        achieved = per_launch / (kms / kl / 1e3) / 1e9
        traffic = profiled_traffic(k)
        rooflines[k] = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak,
                        "unit": "GB/s", "frac": round(achieved / peak, 4),
                        "traffic": traffic, "ms_per_launch": round(kms / kl, 4),
                        "launches_per_step": kl,
                        "algorithmic_bytes_per_launch": per_launch,
                        "peak_kind": peak_kind}

    # e2e: sif's C API on host buffers.
    e2e = None
    if not args.no_e2e:
        e2e = e2e_run(args, w, x, y, z, radii)

    fp64 = adj = batch = None
    if not args.no_forms and not args.small:
        fp64 = fp64_run(args, w, x, y, z, radii)
        adj = adjoint_run(args)
        batch = batch_run(args)

    precision = precision_run(args) if not (args.no_precision or args.small) else None

    cpu = None
    if rank == 0 and not args.no_cpu and not args.small:
        cpu = cpu_run(x, y, z, w, radii, steps=3, warmup=1)

    line = {
        "metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic Zel'dovich lattice (seeded), no dataset",
        "config": {"workload": WORKLOAD_NAME if not args.small
                   else "128^3 particles, box 500, grid 128^3, mesh 50^3",
                   "n_particles": n, "n_voids": n_voids, "l2": "inputs larger than L2 (1.6 GB of particles)",
                   "parallelism": f"replicas x{world}" if world > 1 else "1 GPU",
                   "window_bins": 8},
        "roofline": dict(rooflines.get(dom, {}), kernel=dom),
        "rooflines": rooflines,
        "gpu_launches": int(launches),
        "clocks": clocks.summary(),
        "e2e": e2e,
        "fp64_form": fp64,
        "adjoint": adj,
        "batched_form": batch,
        "precision_1024": precision,
        "cpu_baseline": cpu,
        "stages_ms_last_step": {"growth": round(tm["growth_ms"], 3), "cic_deposit": round(tm["cic_ms"], 3),
                                "mesh": round(tm["mesh_ms"], 3), "filter": round(tm["filter_ms"], 3),
                                "wall": round(tm["wall_ms"], 3)},
        "rungs_last_step": device.last_rung_stats() if args.verbose else None,
    }
    return line


def fp64_run(args, w, x, y, z, radii):
    """The step in the FP64 form on the same particles (as double), device-resident."""
    import torch

    from sif_gb300 import device

    xs = [torch.from_numpy(a.astype(np.float64)).cuda() for a in (x, y, z)]
    r64 = radii.astype(np.float64)
    stream = device.stream()

    def step():
        return device.box(*xs, w["grid"], w["box"], w["mesh"], r64, float(w["threshold"]))

    for _ in range(2):
        cat = step()
    steps = max(1, min(args.steps, 3))
    torch.cuda.synchronize()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for _ in range(steps):
        step()
    end.record(stream)
    torch.cuda.synchronize()
    ms = start.elapsed_time(end) / steps
    del xs
    torch.cuda.empty_cache()
    return {"value": round(len(x) / (ms / 1e3) / 1e6, 2), "unit": UNIT, "ms_per_step": round(ms, 3),
            "steps": steps, "n_voids": len(cat[0]), "dtype": "f64"}


# The differentiation workload: 256^3 particles, box 500, grid 256^3, rms
# displacement 4, seed 1005, Gaussian R = 5; the loss is the sum of the squared
# smoothed contrast over the cells within 2R of the voids the finder returns
# (ladder(5, 30, 0.10), threshold -0.8), centres held fixed.
ADJOINT = dict(n=256, box=500.0, rms=4.0, seed=1005, grid=256, radius=5.0, mesh=62)


def adjoint_run(args):
    import torch

    from sif_gb300 import autograd, device, synth

    a = ADJOINT
    x, y, z = synth.zeldovich(a["n"], a["box"], a["rms"], a["seed"], backend="torch")
    xs = [torch.from_numpy(v).cuda() for v in (x, y, z)]
    radii = synth.ladder(a["radius"], 6 * a["radius"], 0.10).astype(np.float32)
    cx, cy, cz, _ = device.box(*xs, a["grid"], a["box"], a["mesh"], radii, -0.8)
    n = a["grid"]
    cell = a["box"] / n
    reach = 2.0 * a["radius"]
    span = int(reach / cell) + 1
    off = torch.arange(-span, span + 1, device="cuda")
    ox, oy, oz = torch.meshgrid(off, off, off, indexing="ij")
    ox, oy, oz = ox.reshape(-1), oy.reshape(-1), oz.reshape(-1)
    mask = torch.zeros(n ** 3, dtype=torch.bool, device="cuda")
    cs = torch.from_numpy(np.stack([cx, cy, cz], 1).astype(np.float64)).cuda()
    for chunk in torch.split(cs, 512):
        base = torch.floor(chunk / cell).long()
        idx = [(base[:, k, None] + o[None, :]) for k, o in enumerate((ox, oy, oz))]
        d2 = sum(((i.double() * cell - chunk[:, k, None] + a["box"] / 2) % a["box"] - a["box"] / 2) ** 2
                 for k, i in enumerate(idx))
        flat = ((idx[0] % n) * n + (idx[1] % n)) * n + (idx[2] % n)
        mask[flat[d2 <= reach * reach]] = True
    stream = device.stream()
    fwd, bwd = [], []
    for it in range(3 + 5):
        xg = [v.clone().requires_grad_(True) for v in xs]
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        torch.cuda.synchronize()
        e0.record(stream)
        s_field = autograd.smoothed_contrast(*xg, n, a["box"], a["radius"], filter="gaussian")
        e1.record(stream)
        loss = (s_field[mask] ** 2).sum()
        loss.backward()
        e2.record(stream)
        torch.cuda.synchronize()
        if it >= 3:
            fwd.append(e0.elapsed_time(e1))
            bwd.append(e1.elapsed_time(e2))
    f, b = statistics.median(fwd), statistics.median(bwd)
    return {"config": "256^3 particles, box 500 Mpc/h, grid 256^3, Gaussian R=5, loss over "
                      f"{int(mask.sum())} cells within 2R of {len(cx)} void centres",
            "forward_ms": round(f, 3), "adjoint_ms": round(b, 3), "ratio": round(b / f, 3),
            "steps": len(fwd)}


# The batching workload: 64 independent boxes, particles per side drawn
# log-uniform in [64, 256], box sides uniform in [200, 1000] Mpc/h, grid =
# particles per side, rms displacement 4, seed 2000 + box; ladder(R, 6R, 0.10)
# with R twice the mean separation; threshold -0.8; mesh from
# sif_finder_suggest_mesh_cells.
BATCH = dict(boxes=64, n_lo=64, n_hi=256, box_lo=200.0, box_hi=1000.0, rms=4.0, seed=2000)


def batch_run(args):
    import torch

    from sif_gb300 import device, synth

    b = BATCH
    rng = np.random.default_rng(b["seed"])
    boxes = []
    total = 0
    for k in range(b["boxes"]):
        n = int(round(math.exp(rng.uniform(math.log(b["n_lo"]), math.log(b["n_hi"])))))
        n += n % 2
        L = float(rng.uniform(b["box_lo"], b["box_hi"]))
        x, y, z = synth.zeldovich(n, L, b["rms"], b["seed"] + k, backend="torch")
        r0 = 2.0 * L / n
        boxes.append(dict(x=torch.from_numpy(x).cuda(), y=torch.from_numpy(y).cuda(),
                          z=torch.from_numpy(z).cuda(), n_grid=n, box=L, mesh_cells=0,
                          radii=synth.ladder(r0, 6 * r0, 0.10).astype(np.float32),
                          threshold=-0.8))
        total += n ** 3
    stream = device.stream()

    def timed(engines):
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        start.record(stream)
        cats, used = device.box_batch(boxes, engines=engines)
        end.record(stream)
        torch.cuda.synchronize()
        return start.elapsed_time(end), used, sum(len(c[0]) for c in cats)

    timed(0)  # the autotuner's trial runs (and warm-up)
    seq_ms, _, nv1 = timed(1)
    ms, used, nv = timed(0)
    assert nv == nv1, "catalogues depend on the engine count"
    del boxes
    torch.cuda.empty_cache()
    return {"config": f"{b['boxes']} boxes, {b['n_lo']}^3-{b['n_hi']}^3 particles (log-uniform), "
                      f"box {b['box_lo']:.0f}-{b['box_hi']:.0f} Mpc/h, grid = lattice, "
                      "ladder(2 sep, 12 sep, 0.10), threshold -0.8, suggested mesh",
            "value": round(total / (ms / 1e3) / 1e6, 2), "unit": UNIT, "ms": round(ms, 2),
            "engines": used, "one_engine_ms": round(seq_ms, 2),
            "speedup_vs_one_engine": round(seq_ms / ms, 3), "n_particles": total, "n_voids": nv}


# The precision workload: 1024^3 particles in a 2000 Mpc/h box (rms
# displacement 4, seed 1003), grid 1024^3. The float form's smoothed fields
# (top-hat R = 4 with the CIC window correction, the finder's smoothing;
# Gaussian R = 5), from its own CIC and contrast, against the whole chain in
# FP64 on the CPU (the oracle: FP64 CIC, contrast, transforms) and against the
# GPU's FP64 form; then the float finder on the whole box (ladder(4, 24, 0.10),
# threshold -0.8, suggested mesh).
PRECISION = dict(n=1024, box=2000.0, rms=4.0, seed=1003, grid=1024, r_tophat=4.0, r_gauss=5.0)
# Host memory the CPU FP64 chain at 1024^3 needs at its peak (positions,
# density, spectrum, a filtered copy, a field, the two float fields).
PRECISION_HOST_GB = 64.0


def host_available_gb():
    try:
        for line in open("/proc/meminfo"):
            if line.startswith("MemAvailable:"):
                return int(line.split()[1]) / 2 ** 20
    except OSError:
        pass
    return 0.0


def rel_err(got, want, chunk=1 << 26):
    """Relative L2 and max-norm (both over the rms of want) of two n^3
    arrays, in chunks (no full-size temporaries)."""
    se = sw = mx = 0.0
    for a in range(0, len(want), chunk):
        g = np.asarray(got[a:a + chunk], np.float64)
        w = np.asarray(want[a:a + chunk], np.float64)
        d = g - w
        se += float(np.dot(d, d))
        sw += float(np.dot(w, w))
        mx = max(mx, float(np.abs(d).max()))
    rms = math.sqrt(sw / len(want))
    return math.sqrt(se / len(want)) / rms, mx / rms


def precision_run(args):
    import torch

    from sif_gb300 import device, pysif, synth

    c = PRECISION
    n = c["grid"]
    x, y, z = synth.zeldovich(c["n"], c["box"], c["rms"], c["seed"], backend="torch")
    xs = [torch.from_numpy(v).cuda() for v in (x, y, z)]

    def rel(a, b):
        d = (a.double() - b)
        rms = torch.sqrt((b * b).mean())
        return float(torch.sqrt((d * d).mean()) / rms), float(d.abs().max() / rms)

    g32 = device.cic(*xs, n, c["box"])
    device.density_contrast(g32)
    fields32 = {"tophat": device.smooth(g32, n, c["box"], c["r_tophat"]),
                "gauss": device.smooth(g32, n, c["box"], c["r_gauss"], filter="gaussian")}
    out = {"config": "1024^3 particles, box 2000 Mpc/h, grid 1024^3; the float form's fields "
                     "(its CIC, contrast, top-hat R=4 and Gaussian R=5 smoothing) against the "
                     "whole chain in FP64"}
    # Against the GPU's FP64 form on the same positions.
    xs64 = [v.double() for v in xs]
    g64 = device.cic(*xs64, n, c["box"])
    del xs64
    device.density_contrast(g64)
    out["fp64_form"] = {}
    out["fp64_form"]["contrast_rel_l2"], out["fp64_form"]["contrast_rel_max"] = rel(g32, g64)
    for key, r, filt in (("tophat_r4", c["r_tophat"], "top-hat"), ("gauss_r5", c["r_gauss"], "gaussian")):
        f64 = device.smooth(g64, n, c["box"], r, filter=filt)
        out["fp64_form"][f"{key}_rel_l2"], out["fp64_form"][f"{key}_rel_max"] = rel(
            fields32["tophat" if key.startswith("top") else "gauss"], f64)
        del f64
    del g64, g32
    host32 = {k: v.cpu().numpy() for k, v in fields32.items()}
    del fields32
    torch.cuda.empty_cache()
    # Against the CPU FP64 oracle, where the host has the memory for it.
    avail = host_available_gb()
    if avail >= PRECISION_HOST_GB:
        import oracle_ctypes as O

        O.build()
        t0 = time.perf_counter()
        d64 = O.cic_f64(x, y, z, n, c["box"])
        O.density_contrast_f64(d64, inplace=True)
        spec = O.Spectrum(d64, n, c["box"])
        del d64
        oracle = {}
        for key, r, code in (("tophat_r4", c["r_tophat"], 1), ("gauss_r5", c["r_gauss"], 2)):
            f64 = spec.smooth(r, code)
            oracle[f"{key}_rel_l2"], oracle[f"{key}_rel_max"] = rel_err(
                host32["tophat" if code == 1 else "gauss"], f64)
            del f64
        spec.free()
        oracle["cpu_s"] = round(time.perf_counter() - t0, 1)
        out["fp64_oracle"] = oracle
        out["tophat_r4_rel_l2"] = oracle["tophat_r4_rel_l2"]
        out["gauss_r5_rel_l2"] = oracle["gauss_r5_rel_l2"]
        out["reference"] = "FP64 oracle (CPU)"
    else:
        out["fp64_oracle"] = (f"not run: {avail:.0f} GB of host memory available, the CPU FP64 "
                              f"chain at 1024^3 needs about {PRECISION_HOST_GB:.0f}")
        out["tophat_r4_rel_l2"] = out["fp64_form"]["tophat_r4_rel_l2"]
        out["gauss_r5_rel_l2"] = out["fp64_form"]["gauss_r5_rel_l2"]
        out["reference"] = "the GPU's FP64 form"
    del host32, x, y, z
    radii = synth.ladder(4.0, 24.0, 0.10).astype(np.float32)
    mesh = pysif.finders.suggest_mesh_cells(c["n"] ** 3, c["box"], float(radii.max()))
    stream = device.stream()
    cat = device.box(*xs, n, c["box"], mesh, radii, -0.8)
    torch.cuda.synchronize()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record(stream)
    cat = device.box(*xs, n, c["box"], mesh, radii, -0.8)
    end.record(stream)
    torch.cuda.synchronize()
    ms = start.elapsed_time(end)
    out.update({"finder_ms": round(ms, 2), "finder_mparticles_s": round(c["n"] ** 3 / ms / 1e3, 2),
                "mesh_cells": mesh, "n_voids": len(cat[0])})
    del xs
    torch.cuda.empty_cache()
    return out


def e2e_run(args, w, x, y, z, radii):
    """The step through sif's C API on host buffers: the positions live in a
    sif_field_t (host memory), and each step runs sif_grid_assign_cic,
    sif_grid_to_density_contrast, sif_chain_mesh_alloc and
    sif_finder_exodus_raw, each returning its result in its struct's host
    arrays. Timed on the host clock around the whole step.

    With the library's host mirrors on (sifg_set_host_mirrors: a call reuses
    the device copy an earlier call made of an array instead of copying it
    up again), the step first declares the field's positions new
    (sifg_host_modified), so they are copied up every step as a new input
    would be; the grid and the mesh the step itself made are not copied back
    up. The bytes each step copied are the library's own count
    (sifg_copy_bytes). `copy_all` is the same step with mirrors off: every
    call copies its inputs up and its results down."""
    from sif_gb300 import _lib, abi

    lib = _lib.load()
    n = len(x)
    P = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))  # noqa: E731
    field = lib.sif_field_alloc(n)
    assert lib.sif_field_assign_positions(field, P(x), P(y), P(z)) == 0
    grid = lib.sif_grid_alloc(w["grid"], w["box"])
    r = np.ascontiguousarray(radii, np.float32)
    opt = abi.SIF_FINDER_NO_CHECKPOINT
    positions = C.cast(field.contents.x, C.c_void_p)

    def step():
        lib.sifg_host_modified(positions)  # this step's input
        grid.contents.content = abi.SIF_GRID_EMPTY
        assert lib.sif_grid_assign_cic(grid, field) == 0
        assert lib.sif_grid_to_density_contrast(grid) == 0
        mesh = lib.sif_chain_mesh_alloc(w["mesh"], w["box"], field, abi.SIF_MESH_DROP_INDICES)
        assert mesh
        cat = lib.sif_finder_exodus_raw(grid, mesh, P(r), len(r), w["threshold"], 0.0, opt, None)
        assert cat
        nv = cat.contents.n_voids
        lib.sif_catalogue_free(cat)
        lib.sif_chain_mesh_free(mesh)
        return nv

    def copied():
        h2d, d2h = C.c_uint64(0), C.c_uint64(0)
        lib.sifg_copy_bytes(C.byref(h2d), C.byref(d2h))
        return h2d.value, d2h.value

    def timed(mirrors):
        lib.sifg_set_host_mirrors(1 if mirrors else 0)
        steps = max(1, min(args.steps, args.e2e_steps))
        # The first step allocates the structs' host blocks and the mirrors
        # (a few hundred ms); the warm-up steps take that out of the timing.
        for _ in range(max(1, args.warmup)):
            step()
        b0 = copied()
        each = []
        t0 = time.perf_counter()
        for _ in range(steps):
            t = time.perf_counter()
            nv = step()
            each.append(time.perf_counter() - t)
        dt = (time.perf_counter() - t0) / steps
        b1 = copied()
        return {"value": round(n / dt / 1e6, 2), "unit": UNIT,
                "h2d_bytes_per_step": (b1[0] - b0[0]) // steps,
                "d2h_bytes_per_step": (b1[1] - b0[1]) // steps,
                "ms_per_step": round(dt * 1e3, 2), "each_ms": [round(e * 1e3, 2) for e in each],
                "steps": steps, "n_voids": nv}

    try:
        out = timed(True)
        out["host_mirrors"] = True
        out["copy_all"] = timed(False)
    finally:
        lib.sifg_set_host_mirrors(0)
    lib.sif_grid_free(grid)
    lib.sif_field_free(field)
    return out


# --------------------------------------------------------------------------
# the CPU path (the oracle port of the reference)
# --------------------------------------------------------------------------

def cpu_step(O, x, y, z, w, radii, threads):
    """One whole path through the port's release-flags build, as the
    reference's caller runs it: float CIC, contrast, chain mesh, the finder
    with its own smoothing (and the restore of the grid). Returns the seconds
    per stage and the voids found."""
    cat, t = O.pipeline(x, y, z, w["grid"], w["box"], w["mesh"], radii, w["threshold"], threads,
                        fast=True)
    return t, len(cat[0])


def cpu_run(x, y, z, w, radii, steps=1, warmup=0, budget_s=150.0):
    """The CPU baseline on the workload itself: `warmup` untimed runs, then up
    to `steps` timed ones (at least one; no more once budget_s has gone by);
    the median, and the same with the finder's FFT stage (its transforms,
    timed alone on the same contrast) taken out."""
    import oracle_ctypes as O

    O.build()
    threads = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(threads))
    for _ in range(warmup):
        cpu_step(O, x, y, z, w, radii, threads)
    runs = []
    t_start = time.perf_counter()
    nv = 0
    while len(runs) < max(1, steps):
        t, nv = cpu_step(O, x, y, z, w, radii, threads)
        runs.append(t)
        if time.perf_counter() - t_start >= budget_s:
            break
    total = statistics.median(sum(t.values()) for t in runs)
    stages = {k: round(statistics.median(t[k] for t in runs) * 1e3, 1) for k in runs[0]}
    delta = O.density_contrast(O.cic_float(x, y, z, w["grid"], w["box"]))
    fft = O.smoothing_seconds(delta, w["grid"], w["box"], radii, fast=True)
    n = len(x)
    sample = (f"the whole workload ({w['n']}^3 particles, box {w['box']:.0f}, grid {w['grid']}^3, "
              f"mesh {w['mesh']}^3, {len(radii)} rungs), the port's release-flags build, median of "
              f"{len(runs)} run(s)")
    return {"value": round(n / total / 1e6, 3), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": sample, "ms_per_step": round(total * 1e3, 1), "stages_ms": stages,
            "fft_stage_ms": round(fft * 1e3, 1),
            "value_excluding_fft": round(n / max(total - fft, 1e-9) / 1e6, 3),
            "n_voids": nv, "steps": len(runs)}


def reference_arm(args):
    """The reference's path on the host cores (the port: the reference
    sources are not on the GPU machines), on the GPU arm's own workload and
    inputs: W untimed runs (at most 1), then up to K timed ones within a few
    minutes."""
    from sif_gb300 import synth

    w = WORKLOAD
    try:
        import torch

        backend = "torch" if torch.cuda.is_available() else "numpy"
    except ImportError:
        backend = "numpy"
    x, y, z = synth.zeldovich(w["n"], w["box"], w["rms"], w["seed"], backend=backend)
    cpu = cpu_run(x, y, z, w, radii_of(w), steps=args.steps, warmup=min(args.warmup, 1),
                  budget_s=150.0)
    return {
        "impl": "reference", "metric": METRIC, "value": cpu["value"], "unit": UNIT, "n_gpus": 1,
        "steps": cpu["steps"], "warmup": min(args.warmup, 1), "ms_per_step": cpu["ms_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic Zel'dovich lattice (seeded), no dataset",
        "config": {"workload": WORKLOAD_NAME, "n_particles": len(x),
                   "timed_on": f"{cpu['cores']} host cores"},
        "cpu_baseline": cpu,
        "e2e": {"value": cpu["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--small", action="store_true", help="a 128^3 box, for quick checks")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-forms", action="store_true", help="skip the FP64-form and adjoint runs")
    ap.add_argument("--no-precision", action="store_true",
                    help="skip the 1024^3 float-vs-FP64 field error and the 1024^3 finder")
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--verbose", action="store_true")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        if rank != 0:
            return 0
        print(json.dumps(reference_arm(args)))
        return 0
    if world > 1:
        import torch

        torch.distributed.init_process_group("nccl")
    line = gpu_arm(args, rank, world)
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        import torch

        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
