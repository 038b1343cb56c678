"""Benchmark: AOpticsManager::TraceNonSequential on the Schwarzschild-Couder
telescope (two 8-term AGeoAsphericDisk mirrors, 1e7 rays at 400 nm over
0-4 deg field), one GB300.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                  [--workload NAME] [--rays N]

A step traces the whole batch to termination.  `value` is rays/s with the
batch already in HBM (the 1e7-ray inputs, 560 MB, exceed L2; smaller
batches get a 256 MB L2 flush between timed steps); `e2e` is the same
through the host-buffer C ABI call rbg_trace_host (host->device copy of the
rays, trace, device->host copy of fates, points and directions inside the
timed region).  The CPU baseline is the FP64 oracle (the restatement of the
reference algorithm) on all host cores over a bounded sample.  With
--impl reference only that CPU path runs.  --workload selects one of the
other telescope configurations (paraboloid, davies_cotton, light_guide,
schmidt_cassegrain) at its own size; --workload corsika and thinfilm time
the stages either side of the trace (CORSIKA bunch -> ray expansion, the
20-layer thin-film stack) with their own metric.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

METRIC = "Mrays/s & grad-evals/s: chosen form vs plain GPU tracer at equal PSF d80 error"
UNIT = "rays/s"
CPU_SAMPLE = 200_000
# algorithmic bytes (per ray: 40 B in + 48 B out; per segment 52 B read + 52 B write)
BYTES_PER_RAY = 88
BYTES_PER_SEGMENT = 104
# DRAM bytes per ray of the mixed tracer on the Schwarzschild-Couder batch:
# dram__bytes_read.sum + dram__bytes_write.sum of one ncu-captured launch
# over 3e6 rays (364.1 MB + 339.1 MB: the rays read in take-up order, the
# results written back to each ray's own index); traffic grows with the ray
# count (every byte is ray I/O), so a launch's traffic is this times its rays
DRAM_BYTES_PER_RAY_SC = (364.103424e6 + 339.134976e6) / 3e6


# workload name -> (default rays, description); Schwarzschild-Couder is the
# configuration the headline metric is quoted on, the others are the
# remaining telescope configurations at their own sizes
WORKLOADS = {
    "schwarzschild_couder": (10_000_000, {
        "field_deg": [0, 1, 2, 3, 4], "lambda_nm": 400,
        "mirrors": "AGeoAsphericDisk x2, 8 coefficients, N(0,1e-3) rel perturbation"}),
    "paraboloid": (1_000_000, {
        "field_deg": [0, 0.5, 1, 2], "lambda_nm": 400, "mirrors": "TGeoParaboloid shell f=8 m, R=1"}),
    "davies_cotton": (10_000_000, {
        "field_deg": "11 steps 0-2.5", "lambda_nm": "U(300,600)",
        "mirrors": "380 hexagonal sphere-cap facets (CSG), tilt N(0,0.5 mrad), roughness 1 mrad, R=0.85"}),
    "light_guide": (10_000_000, {
        "incidence_deg": "0-40", "lambda_nm": "U(300,600)",
        "optics": "64 variants of a 7x7 AGeoWinstonConePoly array (R=0.9) behind a 5 mm Sellmeier window, Fresnel"}),
    "schmidt_cassegrain": (100_000_000, {
        "samples": 256, "optics": "corrector + spherical mirrors with a 20-layer TiO2/SiO2 stack (per-ray TMM)"}),
}


def workload_config(name, n, precision):
    cfg = {"workload": name, "rays": n}
    cfg.update(WORKLOADS[name][1])
    cfg.update({"precision": precision, "l2": f"inputs {n * 56 / 1e6:.0f} MB" +
                (" > L2 (no flush)" if n * 56 > 129e6 else " (L2 flushed between steps)"),
                "parallelism": "replicas"})
    return cfg


def build_workload(name, n):
    from robast_gb300 import configs

    return configs.CONFIGS[name](n_rays=n)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.rows = []
        self.proc = None
        self.gpu = gpu_index

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for i, nm in enumerate(names):
                if len(r) > 5 + i and r[5 + i].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def grad_bench(batch, rays, steps, device, N, torch):
    """Gradient evaluations per second of the summed per-field RMS spot
    radius w.r.t. the 22 Schwarzschild-Couder parameters: adjoint (mixed
    forward with hit records + one backward) vs central finite differences
    (2 x 22 traces) with the plain FP64 tracer and with the mixed tracer,
    same rays.  The losses run over the rays whose fate is the same in all
    89 traces: a ray that turns from focused to obscured between the +h and
    -h traces is a jump that finite differences see and a derivative does
    not.  The FP64 differences are the accuracy reference."""
    from robast_gb300 import adjoint as A

    build = A.sc_builder()
    p0 = A.sc_parameters()
    group = rays["group"]
    n_groups = int(batch["group"].max()) + 1
    TF = A.make_trace_function()

    def loss_of(x, y, keep):
        return A.rms_spot_groups(x, y, keep, group, n_groups)

    h = A.fd_steps(p0)
    res = device.alloc_result(rays["x"].numel(), rays["x"].device)
    outs = []

    def fd(precision):
        def trace(p):
            man, _ = build(p)
            device.trace(man, rays, res, precision=precision)
            outs.append(res["status"] == N.RBG_FOCUS)
            return res["x"].clone(), res["y"].clone()

        torch.cuda.synchronize()
        t0 = time.perf_counter()
        pts = []
        for k in range(len(p0)):
            pp, pm = p0.copy(), p0.copy()
            pp[k] += h[k]
            pm[k] -= h[k]
            pts.append((trace(pp), trace(pm)))
        torch.cuda.synchronize()
        return pts, time.perf_counter() - t0

    pts64, t_fd64 = fd(N.PREC_FP64)
    ptsmx, t_fdmx = fd(N.PREC_MIXED)
    stable = outs[0].clone()
    for f in outs[1:]:
        stable &= f

    # hit records: a Schwarzschild-Couder ray has at most 4 points (start,
    # primary, secondary, focal surface); a longer path would be skipped
    # and counted in adjoint_skipped
    def adjoint_eval():
        params = torch.tensor(p0, dtype=torch.float64, requires_grad=True)
        x, y, f = TF.apply(params, build, rays, N.PREC_MIXED, 4)[:3]
        loss_of(x, y, f & stable).backward()
        return params.grad.clone()

    g_adj = adjoint_eval()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        g_adj = adjoint_eval()
    torch.cuda.synchronize()
    t_adj = (time.perf_counter() - t0) / steps

    def central(pts):
        return np.array([(float(loss_of(*a, stable)) - float(loss_of(*b, stable))) / (2 * h[k])
                         for k, (a, b) in enumerate(pts)])

    fd64, fdmx = central(pts64), central(ptsmx)
    ga = g_adj.cpu().numpy()
    # relative error per parameter in the loss change over one FD step
    # (d loss/d p * h), floored at 1e-3 of the largest such change, and the
    # plain relative error beside it
    scale = np.abs(fd64 * h).max()
    rel = np.abs((ga - fd64) * h) / np.maximum(np.abs(fd64 * h), 1e-3 * scale)
    # plain relative error where the derivative is not zero by symmetry
    # (the secondary's rotation about the optical axis moves no ray)
    nonzero = np.abs(fd64 * h) > 1e-9 * scale
    rel_plain = np.where(nonzero, np.abs(ga - fd64) / np.where(nonzero, np.abs(fd64), 1.0), np.nan)
    return {"unit": "grad-evals/s", "params": len(p0), "rays": int(rays["x"].numel()),
            "rays_in_loss": int(stable.sum().item()), "adjoint_skipped": int(TF.last_skipped),
            "hit_records_per_ray": 4,
            "adjoint": 1.0 / t_adj, "finite_differences_fp64": 1.0 / t_fd64,
            "finite_differences_mixed": 1.0 / t_fdmx,
            "speedup_vs_fd_fp64": t_fd64 / t_adj, "speedup_vs_fd_mixed": t_fdmx / t_adj,
            "max_rel_err_vs_fd": float(rel.max()), "rel_err_vs_fd": [float(v) for v in rel],
            "max_plain_rel_err_vs_fd": float(np.nanmax(rel_plain)),
            "plain_rel_err_vs_fd": [None if np.isnan(v) else float(v) for v in rel_plain],
            "abs_err_where_fd_is_zero": [float(abs(ga[k])) for k in np.nonzero(~nonzero)[0]],
            "fd_mixed_vs_fd_fp64_max_rel": float(np.max(np.abs(fdmx - fd64) * h) / scale),
            "loss": "sum over the 5 field angles of the RMS spot radius, rays with a stable fate"}


def cpu_baseline(man, batch, sample):
    import oracle_ref

    from robast_gb300 import configs

    sample = min(sample, len(batch["x"]))
    idx = np.linspace(0, len(batch["x"]) - 1, sample).astype(np.int64)
    sub = {k: v[idx] for k, v in batch.items()}
    arr = configs.to_array(sub)
    cores = os.cpu_count() or 1
    t0 = time.perf_counter()
    st, _ = oracle_ref.trace(man, arr, threads=cores)
    dt = time.perf_counter() - t0
    return {"value": sample / dt, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{sample} rays spread evenly over the {len(batch['x'])}-ray batch (every group), oracle FP64, "
                      f"{cores} threads, contiguous chunks"}, st


def fma_peaks(N, torch):
    """FP64 and FP32 FMA rates (FLOP/s) of this GPU from the library's
    microbenchmark (independent FMA chains timed with CUDA events)."""
    import ctypes as C

    out = {}
    st = torch.cuda.current_stream().cuda_stream
    for bits in (64, 32):
        v = C.c_double()
        N.check(N.lib().rbg_measure_fma_peak(bits, C.byref(v), C.c_void_p(st)), "rbg_measure_fma_peak")
        out[bits] = v.value
    return out


def roofline(man, rays, n, seg, kernel_ms, prec, workload, device, N, torch):
    """The tracer kernel against its three ceilings: HBM (algorithmic ray
    bytes), the FP64 pipe and the FP32 pipe (algorithmic flops from the
    counting build's events, rbg_trace_count_events, for scenes it counts);
    the bound is the largest fraction.  Peaks: HBM from the measured copy
    bandwidth, FMA rates measured here."""
    hbm, how = peaks()
    alg_bytes = n * BYTES_PER_RAY + seg * BYTES_PER_SEGMENT
    t = kernel_ms / 1e3
    fr = {"hbm": {"achieved": alg_bytes / t / 1e9, "peak": hbm, "unit": "GB/s", "peak_source": how}}
    fr["hbm"]["frac"] = fr["hbm"]["achieved"] / hbm
    counts = None
    if prec == N.PREC_MIXED:
        try:
            counts, f64, f32 = device.count_events(man, rays)
        except Exception:
            counts = None
    if counts is not None:
        pk = fma_peaks(N, torch)
        for key, fl, bits in (("fp64", f64, 64), ("fp32", f32, 32)):
            fr[key] = {"achieved": fl / t / 1e12, "peak": pk[bits] / 1e12, "unit": "TFLOP/s",
                       "frac": fl / t / pk[bits], "peak_source": "measured here (FMA microbenchmark)",
                       "flops_per_launch": fl}
    bound = max(fr, key=lambda k: fr[k]["frac"])
    out = {"bound": bound, "achieved": fr[bound]["achieved"], "peak": fr[bound]["peak"], "unit": fr[bound]["unit"],
           "frac": fr[bound]["frac"],
           "traffic": (DRAM_BYTES_PER_RAY_SC * n if workload == "schwarzschild_couder" and prec == N.PREC_MIXED
                       else None),
           "kernel_ms": kernel_ms, "fractions": fr,
           "note": "achieved = algorithmic work per launch / the tracer kernel's own duration (CUDA events "
                   "around its launch); bytes = 88 B per ray + 104 B per segment; flops = counted events x "
                   "flops per event kind (rbg_event_flops)"}
    if counts is not None:
        out["event_counts"] = counts
    return out


def spot_r80(device, res, group, g, lims, nbins=500):
    """r80 of group g's focused rays: the device histogram through the
    device ContainmentRadius."""
    h = device.focal_histogram(res, nbins, lims[0], lims[1], nbins, lims[2], lims[3], mask=group == g)
    return device.containment_radius(h, lims[0], lims[1], lims[2], lims[3], 0.8)[0]


def oracle_r80(x, y, lims, nbins=500):
    """r80 from host focal points: TH2D::Fill's bins, the oracle's search."""
    import oracle_ref

    fx = (x - lims[0]) / (lims[1] - lims[0]) * nbins
    fy = (y - lims[2]) / (lims[3] - lims[2]) * nbins
    ok = (fx >= 0) & (fy >= 0) & (fx < nbins) & (fy < nbins)
    h = np.zeros((nbins, nbins))
    np.add.at(h, (fx[ok].astype(np.int64), fy[ok].astype(np.int64)), 1.0)
    return oracle_ref.containment_radius(h, lims[0], lims[1], lims[2], lims[3], 0.8)[0]


def field_limits(x, y, focus, group, n_groups):
    """Per field: a histogram window of +-6 sigma about the spot centroid."""
    lims = []
    for g in range(n_groups):
        sel = focus & (group == g)
        if sel.sum() < 10:
            lims.append(None)
            continue
        mx, my = x[sel].mean(), y[sel].mean()
        hw = 6 * max(np.sqrt(x[sel].var() + y[sel].var()), 1e-6)
        lims.append((mx - hw, mx + hw, my - hw, my + hw))
    return lims


def parity_vs_oracle(man, batch, res, device, N, cores):
    """The whole batch traced by the FP64 oracle on all host cores: ray by
    ray agreement of the GPU result (fates, point counts and last nodes
    exactly; positions and directions), and r80 of every field from the GPU
    (device histogram + device ContainmentRadius) against r80 from the
    oracle's own focal points (oracle ContainmentRadius).  The oracle's wall
    time is the CPU baseline."""
    import oracle_ref

    from robast_gb300 import configs

    arr = configs.to_array(batch)
    t0 = time.perf_counter()
    st, ref = oracle_ref.trace(man, arr, threads=cores)
    dt = time.perf_counter() - t0
    gpu = {k: res[k].cpu().numpy() for k in ("status", "npoints", "last_node", "x", "y", "z", "dx", "dy", "dz")}
    same = (gpu["status"] == ref["status"]) & (gpu["npoints"] == ref["npoints"]) & \
           (gpu["last_node"] == ref["last_node"])
    bad = np.nonzero(~same)[0]
    pos = max(float(np.max(np.abs(gpu[k][same] - ref[k][same]) / np.maximum(1.0, np.abs(ref[k][same])),
                           initial=0)) for k in ("x", "y", "z"))
    dirs = max(float(np.max(np.abs(gpu[k][same] - ref[k][same]), initial=0)) for k in ("dx", "dy", "dz"))
    group = batch["group"]
    n_groups = int(group.max()) + 1
    focus = ref["status"] == N.RBG_FOCUS
    lims = field_limits(ref["x"], ref["y"], focus, group, n_groups)
    import torch

    gdev = torch.as_tensor(np.ascontiguousarray(group, dtype=np.int32)).to(res["x"].device)
    r_gpu, r_orc = [], []
    for g, lm in enumerate(lims):
        if lm is None:
            continue
        r_gpu.append(spot_r80(device, res, gdev, g, lm))
        sel = focus & (group == g)
        r_orc.append(oracle_r80(ref["x"][sel], ref["y"][sel], lm))
    rel = [abs(a - b) / b for a, b in zip(r_gpu, r_orc) if b > 0]
    block = {"rays": int(len(same)), "oracle_status": int(st),
             "fate_mismatches": int(bad.size), "fate_mismatch_rays": [int(i) for i in bad[:10]],
             "max_pos_rel_err": pos, "max_dir_abs_err": dirs,
             "r80_cm_gpu": r_gpu, "r80_cm_oracle": r_orc, "r80_max_rel_diff": max(rel) if rel else None,
             "compared": "status, npoints and last_node exactly; x, y, z relative to max(1, |x|); "
                         "r80 = 80 % containment radius (AGeoUtil::ContainmentRadius) of each field's "
                         "500 x 500 focal-plane histogram over +-6 sigma"}
    cb = {"value": len(same) / dt, "unit": UNIT, "cores": cores, "kind": "port",
          "sample": f"the whole {len(same)}-ray batch, oracle FP64, {cores} threads, contiguous chunks "
                    "(the trace the parity check uses)"}
    return block, cb


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from robast_gb300 import build, configs

    build.build_library()
    build.build_oracle()
    n = args.rays or WORKLOADS[args.workload][0]
    man, batch = build_workload(args.workload, n)
    sample = args.cpu_sample
    vals = []
    for i in range(args.warmup + args.steps):
        cb, st = cpu_baseline(man, batch, sample)
        if i >= args.warmup:
            vals.append(cb["value"])
    v = float(np.median(vals))
    cb["value"] = v
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": sample / v * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": workload_config(args.workload, n, "fp64-cpu"), "cpu_baseline": cb,
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "reference = CPU FP64 restatement (ROOT, which the reference needs, is not installable)"}
    print(json.dumps(line))


# ---------------------------------------------------------------------------
# the stages either side of the trace: CORSIKA bunch expansion (upstream)
# and thin-film stacks (per-hit physics / coating design), one JSON line each
# ---------------------------------------------------------------------------
STAGES = {
    "corsika": (10_000_000, "bunches"),
    "thinfilm": (10_000_000, "(angle, wavelength) pairs"),
}


def synthetic_bunches(n, seed=11):
    """Photon bunches with the value ranges of a CORSIKA IACT event at a
    telescope: positions within 6 m, downward directions within 5 deg of the
    zenith, 0.5-5 photons per bunch, half of them without a wavelength."""
    g = np.random.default_rng(seed)
    th = np.radians(5) * np.sqrt(g.uniform(0, 1, n))
    ph = g.uniform(0, 2 * np.pi, n)
    b = {"x": g.uniform(-600, 600, n), "y": g.uniform(-600, 600, n), "zem": g.uniform(5e5, 1.5e6, n),
         "time": g.uniform(0, 30, n), "cx": np.sin(th) * np.cos(ph), "cy": np.sin(th) * np.sin(ph),
         "cz": -np.cos(th), "lambda": np.where(g.uniform(0, 1, n) < 0.5, 0.0, g.uniform(300, 550, n)),
         "photons": g.uniform(0.5, 5.0, n)}
    return {k: v.astype(np.float32) for k, v in b.items()}


def stage_line(args, name, n, metric, unit, value, ms, alg_bytes, launches, clocks, e2e, cb, extra):
    hbm, how = peaks()
    achieved = alg_bytes / (ms / 1e3) / 1e9
    line = {"metric": metric, "value": value, "unit": unit, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": name, "units": n, "l2": "inputs and outputs > L2 (no flush)"},
            "gpu_launches": launches * args.steps,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                         "traffic": None, "peak_source": how},
            "e2e": e2e, "clocks": clocks, "cpu_baseline": cb}
    line.update(extra)
    print(json.dumps(line))


def time_events(fn, steps, warmup, torch):
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    ev = lambda: torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as ck:
        e0, e1 = ev(), ev()
        e0.record()
        for _ in range(steps):
            fn()
        e1.record()
        torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps, ck.summary()


def run_corsika(args):
    """ACorsikaIACTFile::GetRayArray (src/ACorsikaIACTFile.cxx:71-133) on
    synthetic bunches: rays per second out of rbg_bunches_to_rays."""
    import torch

    import oracle_ref

    from robast_gb300 import _native as N
    from robast_gb300 import build
    from robast_gb300.corsika import BUNCH_FIELDS
    from robast_gb300.device import _ptr

    build.build_library()
    build.build_oracle()
    nb = args.rays or STAGES["corsika"][0]
    hb = synthetic_bunches(nb)
    dev = {f: torch.as_tensor(hb[f]).cuda() for f in BUNCH_FIELDS}
    fp, dp = C.POINTER(C.c_float), C.POINTER(C.c_double)

    def bunches(src, ptr):
        b = N.Bunches()
        b.n = nb
        for f in BUNCH_FIELDS:
            setattr(b, "lambda_" if f == "lambda" else f, C.cast(ptr(src[f]), fp))
        return b

    db = bunches(dev, _ptr)
    ws = torch.empty(int(N.lib().rbg_bunches_workspace_bytes(nb)), dtype=torch.uint8, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    z, tel_z, nidx, lmin, lmax, seed = 1500.0, 0.0, 1.0, 300.0, 550.0, 7
    total = C.c_int64()
    N.check(N.lib().rbg_bunches_to_rays(C.byref(db), z, tel_z, nidx, lmin, lmax, seed, _ptr(ws), None, 0,
                                        C.byref(total), C.c_void_p(st)), "count")
    m = total.value
    names = ("x", "y", "z", "t", "dx", "dy", "dz", "lam")
    out = {f: torch.empty(m, dtype=torch.float64, device="cuda") for f in names}
    rs = N.Rays(m, *(C.cast(_ptr(out[f]), dp) for f in names))

    def step():
        N.check(N.lib().rbg_bunches_to_rays(C.byref(db), z, tel_z, nidx, lmin, lmax, seed, _ptr(ws), C.byref(rs), m,
                                            C.byref(total), C.c_void_p(st)), "rbg_bunches_to_rays")

    ms, clocks = time_events(step, args.steps, args.warmup, torch)
    # end to end: bunches from pinned host memory, rays back to pinned host
    # memory (ACorsikaIACTFile::GetRayArray returns host rays)
    hpin = {f: torch.as_tensor(hb[f]).pin_memory() for f in BUNCH_FIELDS}
    hout = {f: torch.empty(m, dtype=torch.float64).pin_memory() for f in names}

    def e2e_step():
        for f in BUNCH_FIELDS:
            dev[f].copy_(hpin[f], non_blocking=True)
        step()
        for f in names:
            hout[f].copy_(out[f], non_blocking=True)
        torch.cuda.synchronize()

    e2e_step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    t_e2e = (time.perf_counter() - t0) / args.steps
    # CPU: the oracle restatement, one thread, on the first 2e6 bunches
    k = min(nb, 2_000_000)
    sub = {f: hb[f][:k] for f in hb}
    t0 = time.perf_counter()
    ref = oracle_ref.bunches_to_rays(sub, z, tel_z, nidx, lmin, lmax, seed)
    dt = time.perf_counter() - t0
    n_cpu = len(ref["x"])
    # parity of the first rays (the same Philox draws)
    got = {f: out[f][:n_cpu].cpu().numpy() for f in names}
    worst = max(float(np.max(np.abs(got[f] - ref[f]) / np.maximum(1.0, np.abs(ref[f])))) for f in names)
    cb = {"value": n_cpu / dt, "unit": "rays/s", "cores": 1, "kind": "port",
          "sample": f"first {k} of the {nb} bunches ({n_cpu} rays), oracle restatement, 1 thread"}
    e2e = {"value": m / t_e2e, "unit": "rays/s", "h2d_bytes_per_step": nb * 4 * len(BUNCH_FIELDS),
           "d2h_bytes_per_step": m * 8 * len(names)}
    alg = nb * 32 + m * 64
    stage_line(args, "corsika_bunches_to_rays", nb, "CORSIKA bunch -> ray expansion (ACorsikaIACTFile::GetRayArray)",
               "rays/s", m / (ms / 1e3), ms, alg, 3, clocks, e2e, cb,
               {"rays_per_step": m, "max_rel_diff_vs_oracle": worst,
                "roofline_note": "algorithmic bytes = 32 B per bunch read + 64 B per ray written"})


def run_thinfilm(args):
    """AMultilayer::CoherentTMMMixed (src/AMultilayer.cxx:240-481) of the
    20-layer TiO2/SiO2 quarter-wave stack of the Schmidt-Cassegrain
    configuration over (angle, wavelength) pairs, and its
    PreCalculateCoherentTMM table (include/AMultilayer.h:243-262)."""
    import torch

    import oracle_ref

    from robast_gb300 import _native as N
    from robast_gb300 import build, configs

    build.build_library()
    build.build_oracle()
    n = args.rays or STAGES["thinfilm"][0]
    man, _ = configs.schmidt_cassegrain(n_rays=16, n_samples=1)
    scene = man._ensure_scene()
    ml = 0
    nm = 1e-7
    g = np.random.default_rng(5)
    th_h = g.uniform(0, np.radians(60), n)
    lam_h = g.uniform(300 * nm, 700 * nm, n)
    th = torch.as_tensor(th_h).cuda()
    lam = torch.as_tensor(lam_h).cuda()
    R_, T_ = torch.empty_like(th), torch.empty_like(th)
    st = torch.cuda.current_stream().cuda_stream

    def step():
        N.check(N.lib().rbg_multilayer_rt(scene.handle, ml, 0, 2, n, th.data_ptr(), None, lam.data_ptr(),
                                          R_.data_ptr(), T_.data_ptr(), C.c_void_p(st)), "rbg_multilayer_rt")

    ms, clocks = time_events(step, args.steps, args.warmup, torch)
    hin = {"th": torch.as_tensor(th_h).pin_memory(), "lam": torch.as_tensor(lam_h).pin_memory()}
    hout = {"R": torch.empty(n, dtype=torch.float64).pin_memory(), "T": torch.empty(n, dtype=torch.float64).pin_memory()}

    def e2e_step():
        th.copy_(hin["th"], non_blocking=True)
        lam.copy_(hin["lam"], non_blocking=True)
        step()
        hout["R"].copy_(R_, non_blocking=True)
        hout["T"].copy_(T_, non_blocking=True)
        torch.cuda.synchronize()

    e2e_step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    t_e2e = (time.perf_counter() - t0) / args.steps
    k = 20_000
    t0 = time.perf_counter()
    ref = [oracle_ref.tmm(scene, ml, "mixed", th_h[i], lam_h[i]) for i in range(k)]
    dt = time.perf_counter() - t0
    r_gpu = R_[:k].cpu().numpy()
    worst = float(np.max(np.abs(r_gpu - np.array([r for r, _ in ref]))))
    cb = {"value": k / dt, "unit": "evaluations/s", "cores": 1, "kind": "port",
          "sample": f"first {k} of the {n} pairs, oracle restatement through ctypes, 1 thread"}
    e2e = {"value": n / t_e2e, "unit": "evaluations/s", "h2d_bytes_per_step": n * 16, "d2h_bytes_per_step": n * 16}
    stage_line(args, "thinfilm_20layer_coherent_mixed", n,
               "AMultilayer::CoherentTMMMixed evaluations (20-layer stack, s and p)", "evaluations/s",
               n / (ms / 1e3), ms, n * 32, 1, clocks, e2e, cb,
               {"max_abs_diff_R_vs_oracle": worst, "layers": 20,
                "roofline_note": "algorithmic bytes = 16 B in + 16 B out per evaluation; the kernel is bound "
                                 "by the FP64 pipe (complex transfer matrices), not by HBM"})


def run_kernels(args):
    """One small pass over every kernel of the library, for profilers (the
    command of the ncu captures under profiles/): the Schwarzschild-Couder
    batch traced by both tracers (with the take-up order's kernels), the
    adjoint of its RMS spot, the focal-plane moments, histogram and
    ContainmentRadius, and a device ray source; with --workload another
    configuration, traced by its mixed-tracer instance and the FP64 tracer.
    Prints a one-line summary; no timing."""
    import torch

    from robast_gb300 import _native as N
    from robast_gb300 import adjoint as A
    from robast_gb300 import build, configs, device

    build.build_library()
    if args.workload != "schwarzschild_couder":
        # another scene class: its mixed-tracer instance and the FP64 tracer
        man, batch = build_workload(args.workload, args.rays or 1_000_000)
        rays = device.to_device(batch)
        res = device.alloc_result(len(batch["x"]))
        device.reserve(man, len(batch["x"]))
        for _ in range(max(1, args.warmup)):
            device.trace(man, rays, res, precision=N.PREC_MIXED)
        device.trace(man, rays, res, precision=N.PREC_FP64)
        torch.cuda.synchronize()
        print(json.dumps({"kernels": "ok", "workload": args.workload, "rays": len(batch["x"]),
                          "focused": int((res["status"] == N.RBG_FOCUS).sum().item())}))
        return
    n = args.rays or 3_000_000
    _, batch = configs.schwarzschild_couder(n_rays=n)
    rays = device.to_device(batch)
    man, specs = A.sc_builder()(A.sc_parameters())
    for _ in range(max(1, args.warmup)):
        device.trace(man, rays, precision=N.PREC_MIXED)
    device.trace(man, rays, precision=N.PREC_FP64)
    res, st = A.trace_with_history(man, rays)
    f = res["status"] == N.RBG_FOCUS
    gx = torch.where(f, 2 * res["x"], torch.zeros_like(res["x"]))
    gy = torch.where(f, 2 * res["y"], torch.zeros_like(res["y"]))
    g, skipped = A.vjp(man, res, specs, gx, gy)
    group = rays["group"]
    mom = device.focal_moments(res, group, 5)
    h = device.focal_histogram(res, 500, -2.0, 2.0, 500, -2.0, 2.0, mask=group == 0)
    r80 = device.containment_radius(h, -2.0, 2.0, -2.0, 2.0, 0.8)[0]
    shot = device.shoot(N.RBG_SHOOT_RANDOM_CIRCLE, [500.0], n, 400e-7, None, None, (0.0, 0.0, -1.0))
    torch.cuda.synchronize()
    print(json.dumps({"kernels": "ok", "rays": n, "focused": int(f.sum().item()), "adjoint_skipped": skipped,
                      "r80_cm": r80, "shot": int(shot["x"].numel()), "moments_rays": float(mom[:, 0].sum())}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300")
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--no-compare", action="store_true", help="skip the plain FP64 comparison run")
    ap.add_argument("--no-grad", action="store_true", help="skip the gradient benchmark")
    ap.add_argument("--workload", default="schwarzschild_couder", choices=sorted(WORKLOADS) + sorted(STAGES))
    ap.add_argument("--rays", type=int, default=0, help="rays per step (default: the workload's size)")
    ap.add_argument("--cpu-sample", type=int, default=CPU_SAMPLE)
    ap.add_argument("--compaction", type=int, default=0, help="mixed tracer refill threshold (0: tuned)")
    ap.add_argument("--no-parity", dest="parity", action="store_false",
                    help="skip the whole-batch oracle trace (the CPU baseline then times a sample)")
    ap.add_argument("--kernels", action="store_true",
                    help="one small pass over every kernel (for profilers), no timing")
    args = ap.parse_args()
    if args.kernels:
        return run_kernels(args)
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "corsika":
        return run_corsika(args)
    if args.workload == "thinfilm":
        return run_thinfilm(args)

    import torch

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    from robast_gb300 import _native as N
    from robast_gb300 import build, configs, device

    build.build_library()
    build.build_oracle()
    prec = N.PREC_MIXED if args.precision == "mixed" else N.PREC_FP64
    n_req = args.rays or WORKLOADS[args.workload][0]
    man, batch = build_workload(args.workload, n_req)
    n = len(batch["x"])
    man.ray_id_offset = rank * n
    man.compaction = args.compaction
    rays = device.to_device(batch, f"cuda:{local}")
    res = device.alloc_result(n, f"cuda:{local}")
    stream = torch.cuda.current_stream()

    def barrier():
        if ws > 1:
            import torch.distributed as dist

            dist.barrier()

    # inputs smaller than twice the 129 MB L2: write a 256 MB buffer between
    # timed steps and time each step on its own
    flush = torch.empty(64 << 20, dtype=torch.float32, device=f"cuda:{local}") if n * 56 < 2 * 129e6 else None

    kernel_ms = []

    def timed(p, out):
        for _ in range(args.warmup):
            device.trace(man, rays, out, precision=p)
        torch.cuda.synchronize()
        nl = N.lib().rbg_last_launch_count(man.scene.handle)
        barrier()
        torch.cuda.synchronize()
        ev = lambda: torch.cuda.Event(enable_timing=True)
        kernel_ms.clear()
        with ClockSampler(local) as ck:
            if flush is None:
                e0, e1 = ev(), ev()
                e0.record(stream)
                for _ in range(args.steps):
                    device.trace(man, rays, out, precision=p)
                    # the tracer kernel's own duration (events on its
                    # stream around the launch, read after the call's sync)
                    kernel_ms.append(N.lib().rbg_last_kernel_ms(man.scene.handle))
                e1.record(stream)
                torch.cuda.synchronize()
                t = e0.elapsed_time(e1) / args.steps
            else:
                pairs = []
                for _ in range(args.steps):
                    flush.zero_()
                    a, b = ev(), ev()
                    a.record(stream)
                    device.trace(man, rays, out, precision=p)
                    b.record(stream)
                    pairs.append((a, b))
                    kernel_ms.append(N.lib().rbg_last_kernel_ms(man.scene.handle))
                torch.cuda.synchronize()
                t = sum(a.elapsed_time(b) for a, b in pairs) / args.steps
        barrier()
        if ws > 1:
            import torch.distributed as dist

            tt = torch.tensor([t], device=f"cuda:{local}")
            dist.all_reduce(tt, op=dist.ReduceOp.MAX)
            t = float(tt.item())
        return t, nl, ck.summary()

    # every device allocation of the trace made up front (scene tables,
    # take-up order workspace, host pipeline slots)
    device.reserve(man, n)
    N.check(N.lib().rbg_scene_set_timing(man.scene.handle, 1), "rbg_scene_set_timing")
    # autotune the mixed tracer's compaction threshold on this batch (outside
    # the timed region, like the warm-up) unless one was given
    tuned = None
    if prec == N.PREC_MIXED and args.compaction == 0:
        tuned = device.autotune(man, rays, res)
    block_used = device.tuning(man)[0] if prec == N.PREC_MIXED else 128
    ms, launches, clocks = timed(prec, res)
    kms = float(np.mean(kernel_ms)) if kernel_ms and min(kernel_ms) > 0 else None
    seg = int((res["npoints"].to(torch.int64) - 1).sum().item())
    value = n * ws / (ms / 1e3)
    group = rays["group"]
    n_groups = int(batch["group"].max()) + 1
    compare = None
    if not args.no_compare and prec != N.PREC_FP64:
        # the plain FP64 tracer: one thread per ray in input order (the
        # metric's denominator), and the same tracer in the chosen form's
        # take-up order, which separates the precision gain from the order's
        res64 = device.alloc_result(n, f"cuda:{local}")
        man.ray_order = N.ORDER_INPUT
        ms64, _, _ = timed(N.PREC_FP64, res64)
        man.ray_order = N.ORDER_SPATIAL
        ms64o, _, _ = timed(N.PREC_FP64, res64)
        same = (res64["status"] == res["status"]) & (res64["npoints"] == res["npoints"]) & \
               (res64["last_node"] == res["last_node"])
        agree = float(same.double().mean().item())
        h64 = {k: res64[k].cpu().numpy() for k in ("status", "x", "y")}
        lims = field_limits(h64["x"], h64["y"], h64["status"] == N.RBG_FOCUS, batch["group"], n_groups)
        r80 = {"chosen": [], "fp64": []}
        for g, lm in enumerate(lims):
            if lm is None:
                continue
            r80["chosen"].append(spot_r80(device, res, group, g, lm))
            r80["fp64"].append(spot_r80(device, res64, group, g, lm))
        rel = [abs(a - b) / b for a, b in zip(r80["chosen"], r80["fp64"]) if b > 0]
        compare = {"plain_fp64_rays_per_s": n * ws / (ms64 / 1e3), "plain_fp64_ms_per_step": ms64,
                   "speedup_vs_plain_fp64": ms64 / ms,
                   "plain_fp64_ordered_rays_per_s": n * ws / (ms64o / 1e3),
                   "speedup_vs_plain_fp64_ordered": ms64o / ms,
                   "fate_agreement": agree, "fate_mismatches": int((~same).sum().item()),
                   "r80_cm_chosen": r80["chosen"], "r80_cm_fp64": r80["fp64"],
                   "r80_max_rel_diff": max(rel) if rel else None}
        del res64

    # end to end through the host-buffer C ABI call
    from robast_gb300.manager import make_result

    arr = configs.to_array(batch)
    pinned = {}
    for f in ("x", "y", "z", "t", "dx", "dy", "dz", "lam"):
        pt = torch.empty(n, dtype=torch.float64).pin_memory()
        pt.numpy()[:] = getattr(arr, f)
        pinned[f] = pt
    dp = C.POINTER(C.c_double)
    rs = N.Rays(n, *(C.cast(C.c_void_p(pinned[f].data_ptr()), dp) for f in ("x", "y", "z", "t", "dx", "dy",
                                                                             "dz", "lam")))
    host_out = {f: torch.empty(n, dtype=torch.float64).pin_memory() for f in ("x", "y", "z", "t", "dx", "dy",
                                                                              "dz")}
    host_out["status"] = torch.empty(n, dtype=torch.uint8).pin_memory()
    host_out["npoints"] = torch.empty(n, dtype=torch.int32).pin_memory()
    host_out["last_node"] = torch.empty(n, dtype=torch.int32).pin_memory()
    rr = N.Result()
    rr.status = C.cast(C.c_void_p(host_out["status"].data_ptr()), C.POINTER(C.c_uint8))
    rr.npoints = C.cast(C.c_void_p(host_out["npoints"].data_ptr()), C.POINTER(C.c_int32))
    rr.last_node = C.cast(C.c_void_p(host_out["last_node"].data_ptr()), C.POINTER(C.c_int32))
    for f in ("x", "y", "z", "t", "dx", "dy", "dz"):
        setattr(rr, f, C.cast(C.c_void_p(host_out[f].data_ptr()), dp))
    opts = man.trace_options(prec)
    for _ in range(max(1, args.warmup)):
        N.lib().rbg_trace_host(man.scene.handle, C.byref(rs), C.byref(rr), C.byref(opts))
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        N.lib().rbg_trace_host(man.scene.handle, C.byref(rs), C.byref(rr), C.byref(opts))
    t_e2e = (time.perf_counter() - t0) / args.steps
    barrier()
    e2e = {"value": n * ws / t_e2e, "unit": UNIT, "h2d_bytes_per_step": n * 8 * 8,
           "d2h_bytes_per_step": n * (7 * 8 + 4 + 4 + 1)}

    if rank != 0:
        return
    roof = roofline(man, rays, n, seg, kms if kms else ms, prec, args.workload, device, N, torch)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if prec == N.PREC_FP64 else "f32+f64", "data": "synthetic",
            "config": workload_config(args.workload, n, args.precision), "gpu_launches": launches * args.steps,
            "segments_per_step": seg,
            "compaction": args.compaction or tuned,
            "block_size": block_used,
            "tracer_kernel_ms": kms,
            "roofline": roof,
            "e2e": e2e, "clocks": clocks, "vs_plain_fp64": compare}
    if not args.no_grad and ws == 1 and args.workload == "schwarzschild_couder":
        line["grad"] = grad_bench(batch, rays, max(1, min(args.steps, 3)), device, N, torch)
    if args.parity and ws == 1:
        block, cb = parity_vs_oracle(man, batch, res, device, N, os.cpu_count() or 1)
        line["parity_vs_oracle"] = block
    else:
        cb, _ = cpu_baseline(man, batch, args.cpu_sample)
    line["cpu_baseline"] = cb
    print(json.dumps(line))


if __name__ == "__main__":
    main()
