"""Benchmark of the D3Q19 time step on one GB300 (and the reference CPU arm).

Workload: the lid-driven cavity of the headline metric -- 256^3 fluid sites,
TRT with tau+ = 0.56 (nu = 0.02) and magic parameter 1/4, Zou-He velocity lid
u = (0.05, 0, 0) on the +y face, bounce-back on the other five faces,
rho0 = 1, u0 = 0.  A step is one lattice update of all 16.8 M fluid sites.

Our arm (default) prints one JSON line with
  value        MLUPS of the FP32-shifted fused AA kernel, inputs resident in HBM,
               CUDA events around exactly --steps steps after --warmup steps;
  e2e          MLUPS through the public API Solver.evolve(1) per step, with the
               per-call host->device inputs and the device->host den/vel
               download inside the timed region;
  roofline     HBM roofline of the step kernel: 152 algorithmic bytes per fluid
               site (19 FP32 loads + 19 FP32 stores) per launch / launch time;
  fp64         the same for the FP64 plain path (304 B per site);
  fp16         the same for FP16 storage with FP32 arithmetic (76 B per site);
  error        relative L2 velocity errors of FP32 and FP16 against FP64 after
               --err-steps (10000) steps of the same cavity;
  cpu_baseline the reference's own OpenMP solver on this host's cores;
  porous       the 384x256x256 regularized porous channel: FP64 / FP32 / FP16
               MLUPS and roofline over 5000 steps, Darcy flux error vs FP64;
  ensemble     512 channels in one launch per step: MLUPS, roofline, error of
               sampled domains vs FP64 single-domain runs after 2000 steps;
  adjoint      the 256x64x64 inverse problem: backward/forward device-time
               ratio over 2000 steps (checkpoints every 50), reverse-sweep
               roofline, gradients vs central differences of the FP64 model.
The three workload blocks run on one GPU only (--blocks none skips them);
each has its own clocks, roofline and error.
`--impl reference` times only the reference's CPU solver on the same config.
Inputs (1.3 GB of FP32 populations) exceed the 129 MB L2, so no flush is used.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
for p in (os.path.join(ROOT, "jyu-lb_gb300"), os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

N_DEFAULT = 256
KVISC = (0.56 - 0.5) / 3.0
MAGIC = 0.25
LID = 0.05
BYTES_FP32 = 152
BYTES_FP64 = 304


def cavity_metric(n):
    return f"D3Q19 MLUPS (lid-driven cavity {n}^3, TRT)"


def cavity_config(n):
    """The workload description both arms print, so that their lines compare."""
    return {"workload": f"lid-driven cavity {n}^3, TRT tau+=0.56 magic 1/4, Zou-He lid u=(0.05,0,0) on +y, "
                        "bounce-back elsewhere, rho0=1, u0=0",
            "fluid_sites": n ** 3,
            "l2_policy": f"no flush: inputs larger than L2 ({76 * n ** 3 / 1e9:.2f} GB of FP32 populations "
                         "against the 129 MB L2)" if 76 * n ** 3 > 129e6 else "no flush (a case that fits in L2)",
            "multi_gpu": "replicas only"}


def cavity(n, precision, stream=None):
    from jyulb.defs import FIXED_VEL, TRT, WALL
    from jyulb.isothermal import Solver

    bc = np.array([WALL, WALL, WALL, FIXED_VEL, WALL, WALL], dtype=np.int32)
    s = Solver(np.array([n, n, n], dtype=np.int32), TRT, KVISC, np.zeros(3), bc,
               precision=precision, trt_magic=MAGIC, stream=stream)
    s.get_phase()[:] = 1
    s.get_vel()[:, -1, :, 0] = LID
    nf = s.finalize_init()
    return s, nf


class ClockSampler:
    """nvidia-smi samples (every 20 ms) of SM clocks and throttle reasons
    during a region; summary(window) keeps the samples taken inside a
    wall-clock window (the timed steps), when there are any."""

    FIELDS = ("timestamp,clocks.sm,clocks.max.sm,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    _count = 0

    def __init__(self, index=0):
        self.proc = None
        ClockSampler._count += 1
        self.out = os.path.join("/tmp", f"jlb_clocks_{os.getpid()}_{ClockSampler._count}.csv")
        self.index = index

    def __enter__(self):
        try:
            self.fh = open(self.out, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "20"], stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def summary(self, window=None):
        if self.proc is None or not os.path.exists(self.out):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        import datetime

        rows = []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.out):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                ts = datetime.datetime.strptime(parts[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
            except ValueError:
                ts = None  # unknown timestamp format: the sample is kept, unplaced
            try:
                rows.append((ts, float(parts[1]), float(parts[2]),
                             [nm for nm, v in zip(names, parts[4:8]) if v.lower().startswith("active")]))
            except ValueError:
                continue
        os.remove(self.out)
        inside = [r for r in rows if window and r[0] is not None and window[0] <= r[0] <= window[1]]
        sel = inside or rows
        reasons = sorted({nm for r in sel for nm in r[3]})
        out = {"sm_mhz": statistics.median(r[1] for r in sel) if sel else None,
               "sm_max_mhz": max(r[2] for r in sel) if sel else None, "samples": len(sel), "reasons": reasons}
        if window:
            out["samples_in_timed_region"] = len(inside)
        return out


def measured_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profile_traffic(name):
    """DRAM bytes per launch from the committed ncu summary, if present."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as fh:
            return json.load(fh).get(name)
    except Exception:
        return None


def time_device(s, nf, steps, warmup, torch, st):
    """MLUPS and mean launch time of the step kernel, inputs in HBM; the
    events are recorded on the stream the solver launches on."""
    lib, h = s._lib, s._h
    assert lib.jlb_step(h, warmup, 0) == 0
    torch.cuda.synchronize()
    l0 = s.kernel_launches
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    w0 = time.time()
    e0.record(st)
    assert lib.jlb_step(h, steps, 0) == 0
    e1.record(st)
    torch.cuda.synchronize()
    time_device.window = (w0, time.time())
    ms = e0.elapsed_time(e1)
    launches = s.kernel_launches - l0
    return nf * steps / (ms * 1e-3) / 1e6, ms / steps, launches


def over_ranks(ms, units, world, dist=None, device="cpu"):
    """Whole-job time and MLUPS of `world` replicas: each rank processed
    `units` site updates in its own `ms`, and the job took as long as the
    slowest rank."""
    if dist is not None and world > 1:
        import torch

        t = torch.tensor([ms], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    return ms, units * world / (ms * 1e-3) / 1e6


def time_e2e(s, nf, steps, warmup):
    """MLUPS through Solver.evolve(1): per-call inputs uploaded, den/vel
    downloaded into the host arrays every step.  Also returns the median
    per-call time, which a stray slow call on the host does not move."""
    for _ in range(warmup):
        s.evolve(1)
    b0 = s.transfer_bytes
    calls = []
    t0 = time.perf_counter()
    for _ in range(steps):
        c0 = time.perf_counter()
        s.evolve(1)
        calls.append(time.perf_counter() - c0)
    dt = time.perf_counter() - t0
    b1 = s.transfer_bytes
    time_e2e.median_ms = statistics.median(calls) * 1e3
    return (nf * steps / dt / 1e6, dt * 1e3 / steps, (b1[0] - b0[0]) // steps, (b1[1] - b0[1]) // steps)


def l2_error(n, steps, stream):
    """Relative L2 velocity errors of FP32 and FP16 storage against FP64
    after `steps` steps of the cavity."""
    from jyulb.defs import FP16, FP32, FP64

    s64, nf = cavity(n, FP64, stream)
    s64.evolve(steps)
    v64 = np.array(s64.get_vel())
    del s64
    errs = []
    for prec in (FP32, FP16):
        s, _ = cavity(n, prec, stream)
        s.evolve(steps)
        v = np.array(s.get_vel())
        del s
        errs.append(float(np.linalg.norm(v - v64) / np.linalg.norm(v64)))
    return errs


def reference_mlups(n, steps, warmup, threads=None, budget_s=20.0):
    """Times the reference's own OpenMP solver (oracle/_ref) on the cavity."""
    if threads:
        os.environ["OMP_NUM_THREADS"] = str(threads)
    code = f"""
import sys, time, json, numpy as np
sys.path.insert(0, {os.path.join(ROOT, 'oracle', '_ref')!r})
from jyulb.isothermal import Solver
n = {n}
s = Solver(np.array([n, n, n], dtype=np.int32), 1, {KVISC!r}, np.zeros(3),
           np.array([0, 0, 0, 3, 0, 0], dtype=np.int32))
s.get_phase()[:] = 1
vel = s.get_vel(); np.asarray(vel)[:, -1, :, 0] = {LID!r}
nf = s.finalize_init()
s.evolve({max(warmup, 1)})
t0 = time.perf_counter(); s.evolve(1); t1 = time.perf_counter() - t0
k = max(1, min({steps}, int({budget_s} / max(t1, 1e-6))))
t0 = time.perf_counter(); s.evolve(k); dt = time.perf_counter() - t0
print(json.dumps({{"mlups": nf * k / dt / 1e6, "steps": k, "sec": dt}}))
"""
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stderr[-2000:])
    return json.loads(r.stdout.strip().splitlines()[-1])


def ensure_reference():
    import build_ref

    if not build_ref.available():
        build_ref.build()
    return build_ref.available()


def cpu_baseline(n):
    cores = os.cpu_count() or 1
    try:
        if ensure_reference():
            r = reference_mlups(n, steps=20, warmup=1, threads=cores, budget_s=15.0)
            return {"value": round(r["mlups"], 3), "unit": "MLUPS", "cores": cores, "kind": "reference",
                    "sample": f"reference jyulb OpenMP solver, {n}^3 cavity TRT, {r['steps']} steps "
                              f"({r['sec']:.1f} s) after 1 warm-up step"}
    except Exception as e:  # fall back to the single-threaded oracle port
        print(f"reference baseline failed: {e}", file=sys.stderr)
    import pyoracle

    m = 64
    o = pyoracle.Oracle((m, m, m), 1, KVISC, None, [0, 0, 0, 3, 0, 0])
    o.get_phase()[:] = 1
    o.get_vel()[:, -1, :, 0] = LID
    nf = o.finalize_init()
    o.evolve(1)
    t0 = time.perf_counter()
    o.evolve(10)
    dt = time.perf_counter() - t0
    return {"value": round(nf * 10 / dt / 1e6, 3), "unit": "MLUPS", "cores": 1, "kind": "port",
            "sample": f"C oracle, {m}^3 cavity TRT, 10 steps"}


def ensemble_domains(n, seed=2024, scale=1.0):
    """The batched-ensemble workload: n channels with nx~U[32,256],
    ny~U[16,128], nz~U[8,64], tau~U[0.55,1.5], gx~U[1e-7,1e-5]; solid rows at
    the y ends, periodic x/z; every other channel has a moving top wall with
    u~U[0.01,0.05] along x (Couette-Poiseuille)."""
    from jyulb.ensemble import Domain

    rng = np.random.default_rng(seed)
    doms = []
    for d in range(n):
        nx = max(4, int(rng.integers(32, 257) * scale))
        ny = max(4, int(rng.integers(16, 129) * scale))
        nz = max(2, int(rng.integers(8, 65) * scale))
        tau = float(rng.uniform(0.55, 1.5))
        gx = float(rng.uniform(1e-7, 1e-5))
        uw = float(rng.uniform(0.01, 0.05))
        phase = np.ones((nx, ny, nz), np.uint8)
        phase[:, 0, :] = 0
        phase[:, -1, :] = 0
        vel = None
        if d % 2 == 1:
            vel = np.zeros((nx, ny, nz, 3))
            vel[:, -1, :, 0] = uw
        doms.append(Domain(phase, None, vel, (tau - 0.5) / 3.0, [gx, 0.0, 0.0]))
    return doms


def ensemble_block(args):
    """The batched ensemble: `--ens-steps` steps in all (a few untimed
    warm-up steps, the rest timed with CUDA events), then a sample of domains
    re-run as FP64 single domains for the same number of steps."""
    import torch
    from jyulb.defs import BGK, FP64
    from jyulb.ensemble import Ensemble
    from jyulb.isothermal import Solver

    torch.cuda.set_device(0)
    t0 = time.perf_counter()
    doms = ensemble_domains(args.domains)
    st = torch.cuda.Stream()
    ens = Ensemble(doms, BGK, stream=st.cuda_stream)
    setup_s = time.perf_counter() - t0
    info = ens.info()
    nf = info["fluid_sites"]
    total = max(args.ens_steps, args.warmup + 1)
    warm = min(args.warmup, total - 1)
    steps = total - warm
    ens.evolve(warm)
    torch.cuda.synchronize()
    l0 = ens.info()["launches"]
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as clk:
        w0 = time.time()
        e0.record(st)
        ens.evolve(steps)
        e1.record(st)
        torch.cuda.synchronize()
        window = (w0, time.time())
    dt = e0.elapsed_time(e1) * 1e-3
    launches = ens.info()["launches"] - l0
    mlups = nf * steps / dt / 1e6
    # per-domain check: FP64 single-domain runs of a sample of domains, same
    # total step count
    errs = []
    sample = range(0, len(doms), max(1, len(doms) // max(1, args.check_domains)))[: args.check_domains]
    for d in sample:
        dom = doms[d]
        s = Solver(np.array(dom.phase.shape, dtype=np.int32), BGK, dom.kvisc, dom.g, None, precision=FP64)
        s.get_phase()[:] = dom.phase
        if dom.vel is not None:
            s.get_vel()[:] = dom.vel
        s.finalize_init()
        s.evolve(total)
        _, v = ens.moments(d)
        fl = dom.phase != 0
        v64 = np.asarray(s.get_vel())
        errs.append(float(np.linalg.norm(v[fl] - v64[fl]) / np.linalg.norm(v64[fl])))
        del s
    del ens
    torch.cuda.empty_cache()
    peak, peak_kind = measured_peak()
    ach = nf * BYTES_FP32 / (dt / steps) / 1e9
    return {
        "metric": "D3Q19 MLUPS, batched ensemble of channels (FP32 shifted, one launch per step)",
        "value": round(mlups, 3), "unit": "MLUPS", "steps": steps, "warmup": warm,
        "ms_per_step": round(dt * 1e3 / steps, 4), "dtype": "f32",
        "config": {"workload": f"{len(doms)} channels nx~U[32,256] ny~U[16,128] nz~U[8,64], tau~U[0.55,1.5], "
                               "gx~U[1e-7,1e-5], half with moving top wall u~U[0.01,0.05]; BGK",
                   "domains": len(doms), "packed_sites": info["sites"], "fluid_sites": nf,
                   "setup_s": round(setup_s, 1), "autotuned_block": info["block"],
                   "autotune_us_per_step": info["tune_us_per_step"],
                   "l2_policy": "no flush: 14.5 GB of FP32 populations against the 129 MB L2"},
        "roofline": {"bound": "hbm", "achieved": round(ach, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(ach / peak, 4), "peak_kind": peak_kind, "bytes_per_site": BYTES_FP32},
        "error": {"domains_checked": len(errs), "vel_rel_l2_vs_fp64_max": max(errs) if errs else None,
                  "vel_rel_l2_vs_fp64_median": statistics.median(errs) if errs else None, "steps": total},
        "gpu_launches": launches, "clocks": clk.summary(window),
    }


def run_ensemble(args):
    line = ensemble_block(args)
    line.update({"n_gpus": 1, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                 "data": "synthetic"})
    print(json.dumps(line))
    return 0


POROUS_SHAPE = (384, 256, 256)


def porous_geometry(seed=2025, shape=POROUS_SHAPE, r=8, porosity=0.6):
    """Seeded non-overlapping spheres of radius r until the porosity first
    drops to `porosity`.  Random sequential addition of equal spheres jams
    near a 38% solid fraction, short of 40%, so the candidate centres are a
    lattice of spacing 2r+1 with a seeded jitter of +-1/2 site per axis (no
    two spheres overlap) and spheres are added in a seeded random order.
    Periodic in x and z (spheres wrap), whole spheres inside the y walls."""
    nx, ny, nz = shape
    rng = np.random.default_rng(seed)
    sp = 2 * r + 1
    cs = [np.arange(n // sp) * sp + sp / 2.0 for n in (nx, ny, nz)]
    C = np.stack(np.meshgrid(*cs, indexing="ij"), -1).reshape(-1, 3)
    C = C + rng.uniform(-0.5, 0.5, C.shape)
    C = C[rng.permutation(len(C))]
    solid = np.zeros(shape, bool)
    off = np.arange(-r - 1, r + 2)
    target = (1.0 - porosity) * solid.size
    nsolid = 0
    for c in C:
        base = np.floor(c).astype(int)
        X, Y, Z = np.meshgrid(base[0] + off, base[1] + off, base[2] + off, indexing="ij")
        inside = (X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2 <= r * r
        xi, yi, zi = X[inside] % nx, Y[inside], Z[inside] % nz
        nsolid += int((~solid[xi, yi, zi]).sum())
        solid[xi, yi, zi] = True
        if nsolid >= target:
            break
    phase = np.where(solid, 0, 1).astype(np.uint8)
    return phase, float(phase.mean())


def porous_block(args):
    """Porous channel: FP64, FP32-shifted and FP16-storage runs of the same
    steps; MLUPS, roofline and the Darcy flux error against FP64."""
    import torch
    from jyulb.defs import FP16, FP32, FP64, PERIODIC, REGULARIZATION, WALL
    from jyulb.isothermal import Solver

    torch.cuda.set_device(0)
    st = torch.cuda.Stream()
    t0 = time.perf_counter()
    shape = tuple(max(32, int(n * args.porous_scale)) for n in POROUS_SHAPE)
    phase, por = porous_geometry(shape=shape)
    geom_s = time.perf_counter() - t0
    steps = args.porous_steps
    bc = np.array([PERIODIC, PERIODIC, WALL, WALL, PERIODIC, PERIODIC], dtype=np.int32)
    peak, peak_kind = measured_peak()
    res, vel = {}, {}
    nsites = phase.size
    runs = [r for r in (("fp32", FP32, BYTES_FP32), ("fp16", FP16, 76), ("fp64", FP64, BYTES_FP64))
            if r[0] in args.porous_precisions.split(",")]
    for name, prec, bps in runs:
        s = Solver(np.array(shape, dtype=np.int32), REGULARIZATION, (0.7 - 0.5) / 3.0,
                   np.array([5e-6, 0.0, 0.0]), bc, precision=prec, stream=st.cuda_stream)
        s.get_phase()[:] = phase
        nf = s.finalize_init()
        lib, h = s._lib, s._h
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with ClockSampler(0) as clk:
            w0 = time.time()
            e0.record(st)
            assert lib.jlb_step(h, steps - 1, 0) == 0
            assert lib.jlb_step(h, 1, 1) == 0
            e1.record(st)
            torch.cuda.synchronize()
            window = (w0, time.time())
        ms = e0.elapsed_time(e1)
        red = s.reduce()
        assert lib.jlb_download_moments(h, s.den.ctypes.data_as(lib.jlb_download_moments.argtypes[1]),
                                        s.vel.ctypes.data_as(lib.jlb_download_moments.argtypes[2])) == 0
        vel[name] = np.array(s.get_vel())
        ach = nf * bps / (ms * 1e-3 / steps) / 1e9
        res[name] = {"mlups": round(nf * steps / (ms * 1e-3) / 1e6, 1), "ms_per_step": round(ms / steps, 4),
                     "bytes_per_site": bps, "achieved_gbs": round(ach, 1), "roofline_frac": round(ach / peak, 4),
                     "darcy_flux": red["vel_sum"][0] / nsites, "clocks": clk.summary(window)}
        del s
        torch.cuda.empty_cache()
    fl = phase != 0
    for name in ("fp32", "fp16"):
        if name not in res or "fp64" not in res:
            continue
        d64 = res["fp64"]["darcy_flux"]
        res[name]["darcy_rel_err_vs_fp64"] = abs(res[name]["darcy_flux"] - d64) / abs(d64)
        res[name]["vel_rel_l2_vs_fp64"] = float(np.linalg.norm(vel[name][fl] - vel["fp64"][fl]) /
                                                np.linalg.norm(vel["fp64"][fl]))
    return {
        "metric": "D3Q19 MLUPS, porous channel 384x256x256 (regularized), FP32 shifted",
        "value": res["fp32"]["mlups"], "unit": "MLUPS", "steps": steps, "warmup": 0,
        "ms_per_step": res["fp32"]["ms_per_step"], "dtype": "f32",
        "config": {"workload": f"porous channel {shape[0]}x{shape[1]}x{shape[2]}, regularized tau=0.7, gx=5e-6, seeded spheres r=8 "
                               "(jittered lattice, random order) to porosity 0.6, periodic x/z, walls at the y ends",
                   "porosity": round(por, 5), "fluid_sites": int(fl.sum()), "geometry_s": round(geom_s, 1),
                   "l2_policy": "inputs larger than L2 (FP16 populations 1.9 GB), no flush"},
        "roofline": {"bound": "hbm", "achieved": res["fp32"]["achieved_gbs"], "peak": peak, "unit": "GB/s",
                     "frac": res["fp32"]["roofline_frac"], "peak_kind": peak_kind, "bytes_per_site": BYTES_FP32},
        "precisions": res,
        "gpu_launches": 3 * steps,
        "clocks": res["fp32"]["clocks"],
    }


def run_porous(args):
    line = porous_block(args)
    line.update({"n_gpus": 1, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                 "data": "synthetic"})
    print(json.dumps(line))
    return 0


ADJ_SHAPE = (256, 64, 64)
ADJ_PLANE = 200
BYTES_ADJ_FP32 = 228  # reverse sweep: adjoint populations read + written, state before the step read
BYTES_RECOMP_FP32 = 152  # recompute: one out-of-place forward step (K-1 of every K steps)


def adjoint_case(precision, stream=None, K=50):
    """The inverse-problem channel: 256x64x64, a cylinder of radius 8 along z
    at a seeded position, Zou-He velocity inlet on x=0 with one u_x per inlet
    site, density outlet rho=1 on the last x layer, walls on the y and z faces;
    TRT with magic parameter 1/4; loss on the plane x=200."""
    from jyulb.adjoint import ChannelProblem
    from jyulb.defs import FIXED_DEN, FIXED_VEL, TRT, WALL

    nx, ny, nz = ADJ_SHAPE
    rng = np.random.default_rng(7)
    cx, cy = int(rng.integers(56, 73)), ny // 2 + int(rng.integers(-3, 4))
    X, Y = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    phase = np.ones(ADJ_SHAPE, np.uint8)
    phase[(X - cx) ** 2 + (Y - cy) ** 2 <= 64] = 0
    return ChannelProblem(phase, bc=[FIXED_VEL, FIXED_DEN, WALL, WALL, WALL, WALL], rlx_scheme=TRT,
                          precision=precision, trt_magic=0.25, loss_plane=ADJ_PLANE, checkpoint_every=K,
                          stream=stream), phase


def adjoint_params():
    """Hidden parameters (they make the target) and the starting guess."""
    _, ny, nz = ADJ_SHAPE
    rng = np.random.default_rng(11)
    yy = (np.arange(ny) + 0.5) / ny
    zz = (np.arange(nz) + 0.5) / nz
    prof = 16.0 * np.outer(yy * (1 - yy), zz * (1 - zz))
    hidden = (0.6 + 0.05 * float(rng.random()), np.array([2e-6 * (1 + 0.2 * float(rng.random())), 0.0, 0.0]),
              0.04 * prof * (1 + 0.1 * rng.standard_normal((ny, nz))))
    guess = (0.58, np.array([1e-6, 0.0, 0.0]), 0.035 * prof)
    return hidden, guess


def adjoint_block(args):
    """Adjoint workload: forward and backward device times of the FP32
    problem, and its gradients against central differences of the FP64
    forward model."""
    import torch
    from jyulb.defs import FP32, FP64

    torch.cuda.set_device(0)
    steps = args.adj_steps
    st = torch.cuda.Stream()
    K = args.adj_ckpt
    (tau_h, g_h, uin_h), (tau0, g0, uin0) = adjoint_params()
    # the target is data: the FP64 model's velocity at the hidden parameters
    p64, phase = adjoint_case(FP64, None, K)
    _, target = p64.forward(tau_h, g_h, uin_h, steps)
    p32, _ = adjoint_case(FP32, st.cuda_stream, K)
    nf = int((phase != 0).sum())
    for _ in range(max(1, args.warmup // 5)):
        p32.forward(tau0, g0, uin0, steps, target)
        p32.backward()
    recs = []
    walls = []
    with ClockSampler(0) as clk:
        w0 = time.time()
        for _ in range(args.adj_reps):
            t0 = time.perf_counter()
            L, _ = p32.forward(tau0, g0, uin0, steps, target)
            dtau, dg, duin = p32.backward()
            walls.append(time.perf_counter() - t0)
            recs.append(p32.timers())
        window = (w0, time.time())
    med = {k: statistics.median(r[k] for r in recs) for k in recs[0]}
    ratio = med["backward"] / med["forward"]
    # central differences of the FP64 forward model
    L64, _ = p64.forward(tau0, g0, uin0, steps, target)
    a64 = p64.backward()

    def loss64(tau, g, uin):
        return p64.forward(tau, g, uin, steps, target)[0]

    rng = np.random.default_rng(3)
    v = rng.choice([-1.0, 1.0], size=uin0.shape) * (phase[0] != 0)
    big = np.unravel_index(np.argsort(np.abs(duin).ravel())[-2:], duin.shape)
    checks = []

    def fd(name, h, plus, minus, adj32, adj64):
        # central differences of the FP64 model; a parameter whose influence
        # has not reached the loss plane yet has d = 0
        d = (loss64(*plus(h)) - loss64(*minus(h))) / (2 * h)
        checks.append({"param": name, "fd_fp64": d, "adjoint_fp32": adj32, "adjoint_fp64": adj64,
                       "rel_err_fp32": abs(adj32 - d) / abs(d) if d else None,
                       "rel_err_fp64": abs(adj64 - d) / abs(d) if d else None,
                       "rel_diff_fp32_vs_fp64_adjoint": abs(adj32 - adj64) / abs(adj64) if adj64 else None})

    ex = np.array([1.0, 0.0, 0.0])
    fd("tau", 1e-4, lambda h: (tau0 + h, g0, uin0), lambda h: (tau0 - h, g0, uin0), dtau, a64[0])
    fd("gx", 1e-9, lambda h: (tau0, g0 + h * ex, uin0), lambda h: (tau0, g0 - h * ex, uin0), dg[0],
       a64[1][0])
    fd("uin.v (random +-1 direction over the inlet)", 1e-6, lambda h: (tau0, g0, uin0 + h * v),
       lambda h: (tau0, g0, uin0 - h * v), float((duin * v).sum()), float((a64[2] * v).sum()))
    for j, k in zip(*big):
        du = np.zeros_like(uin0)
        du[j, k] = 1.0
        fd(f"uin[{j},{k}]", 1e-6, lambda h: (tau0, g0, uin0 + h * du), lambda h: (tau0, g0, uin0 - h * du),
           float(duin[j, k]), float(a64[2][j, k]))
    peak, peak_kind = measured_peak()
    rev_ms = med["reverse"] / steps
    rec_steps = steps - (steps + K - 1) // K
    rec_ms = med["recompute"] / max(rec_steps, 1)
    bwd_bytes = nf * (BYTES_ADJ_FP32 * steps + BYTES_RECOMP_FP32 * rec_steps)
    del p64, p32
    torch.cuda.empty_cache()
    return {
        "metric": "adjoint backward / forward device-time ratio, D3Q19 TRT channel 256x64x64, FP32 shifted",
        "value": round(ratio, 3), "unit": "x", "steps": steps, "warmup": max(1, args.warmup // 5),
        "ms_per_step": round(med["forward"] / steps, 5), "higher_is_better": False, "dtype": "f32",
        "config": {"workload": "channel 256x64x64, seeded cylinder r=8 along z, Zou-He u_x inlet per site, "
                               "outlet rho=1, walls y/z, TRT magic 1/4; loss |u-target|^2 on x=200, target "
                               "from the FP64 model at hidden seeded (tau, gx, uin)",
                   "fluid_sites": nf, "checkpoint_every": K, "repetitions": args.adj_reps,
                   "l2": "80 MB lattice; 3.1 GB of checkpoints and 7.9 GB of recompute states per run exceed the 129 MB L2"},
        "forward_ms": round(med["forward"], 3), "backward_ms": round(med["backward"], 3),
        "recompute_ms": round(med["recompute"], 3), "reverse_ms": round(med["reverse"], 3),
        "reverse_step_vs_forward_step": round(med["reverse"] / med["forward"], 3),
        "forward_mlups": round(nf * steps / med["forward"] / 1e3, 1),
        "reverse_sweep_mlups": round(nf * steps / med["reverse"] / 1e3, 1),
        "roofline": {"bound": "hbm", "kernel": "adjoint reverse sweep", "achieved": round(
            nf * BYTES_ADJ_FP32 / (rev_ms * 1e-3) / 1e9, 1), "peak": peak, "unit": "GB/s",
            "frac": round(nf * BYTES_ADJ_FP32 / (rev_ms * 1e-3) / 1e9 / peak, 4), "peak_kind": peak_kind,
            "bytes_per_site": BYTES_ADJ_FP32, "recompute_gbs": round(nf * BYTES_RECOMP_FP32 / (rec_ms * 1e-3) / 1e9, 1),
            "recompute_bytes_per_site": BYTES_RECOMP_FP32,
            "backward_gbs": round(bwd_bytes / (med["backward"] * 1e-3) / 1e9, 1),
            "note": "recompute (second stream) overlaps the reverse sweep; kernel times are measured while overlapped"},
        "loss": {"fp32": L, "fp64": L64},
        "gradient_check": checks,
        "max_rel_err_fp32_vs_fd": max((c["rel_err_fp32"] for c in checks if c["rel_err_fp32"] is not None),
                                      default=None),
        "max_rel_err_fp64_vs_fd": max((c["rel_err_fp64"] for c in checks if c["rel_err_fp64"] is not None),
                                      default=None),
        "gradient_note": "rel_err_fp32 compares the FP32 adjoint with differences of the FP64 model, so it "
                         "includes the FP32 model's own rounding (its loss differs from the FP64 model's by "
                         "the relative amount in loss_rel_diff); rel_diff_fp32_vs_fp64_adjoint is that gap "
                         "between the two adjoints",
        "loss_rel_diff": abs(L - L64) / abs(L64),
        "e2e": {"value": round(statistics.median(walls) * 1e3, 2), "unit": "ms per forward+backward through "
                "jyulb.adjoint (host parameters in, gradients out)",
                "h2d_bytes_per_step": int(8 * (uin0.size + target.size + 4)),
                "d2h_bytes_per_step": int(8 * (uin0.size + 4 + target.size))},
        "clocks": clk.summary(window),
    }


def run_adjoint(args):
    line = adjoint_block(args)
    line.update({"n_gpus": 1, "scaling": "weak", "vs_baseline": None, "data": "synthetic"})
    print(json.dumps(line))
    return 0


def run_reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    n = args.size
    cores = os.cpu_count() or 1
    try:
        ok = ensure_reference()
    except Exception as e:
        ok = False
        err = str(e)
    if not ok:
        print(json.dumps({"impl": "reference", "unavailable": "reference solver could not be built here"}))
        return 0
    r = reference_mlups(n, steps=max(args.steps, 1), warmup=args.warmup, threads=cores, budget_s=60.0)
    line = {
        "impl": "reference", "metric": cavity_metric(n),
        "path": f"reference jyulb OpenMP solver (FP64), {cores} host threads; its TRT magic parameter is "
                "fixed at 3/16, which costs the same as 1/4",
        "value": round(r["mlups"], 3), "unit": "MLUPS", "n_gpus": args.gpus, "steps": r["steps"],
        "warmup": args.warmup, "ms_per_step": round(r["sec"] * 1e3 / r["steps"], 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": cavity_config(n),
        "cpu_baseline": {"value": round(r["mlups"], 3), "unit": "MLUPS", "cores": cores,
                         "kind": "reference",
                         "sample": f"{r['steps']} steps of the {n}^3 cavity after {args.warmup} warm-up"},
        "e2e": {"value": round(r["mlups"], 3), "unit": "MLUPS", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--size", type=int, default=N_DEFAULT)
    ap.add_argument("--err-steps", type=int, default=10000)
    ap.add_argument("--e2e-steps", type=int, default=100)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--workload", default="cavity", choices=["cavity", "ensemble", "adjoint", "porous"])
    ap.add_argument("--porous-steps", type=int, default=5000)
    ap.add_argument("--porous-scale", type=float, default=1.0)
    ap.add_argument("--porous-precisions", default="fp32,fp16,fp64")
    ap.add_argument("--adj-steps", type=int, default=2000)
    ap.add_argument("--adj-reps", type=int, default=3)
    ap.add_argument("--adj-ckpt", type=int, default=50)
    ap.add_argument("--domains", type=int, default=512)
    ap.add_argument("--check-domains", type=int, default=6)
    ap.add_argument("--ens-steps", type=int, default=2000)
    ap.add_argument("--blocks", default="porous,ensemble,adjoint",
                    help="workloads added to the default (cavity) line on one GPU; 'none' for the cavity alone")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference_arm(args)
    if args.workload == "ensemble":
        return run_ensemble(args)
    if args.workload == "adjoint":
        return run_adjoint(args)
    if args.workload == "porous":
        return run_porous(args)

    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    from jyulb.defs import FP16, FP32, FP64, FP64_FAST

    n = args.size
    tstream = torch.cuda.Stream()
    stream = tstream.cuda_stream
    # replicas only: every rank advances its own cavity (the path has no
    # exchange step on one domain per GPU)
    s32, nf = cavity(n, FP32, stream)
    assert nf == n ** 3, "every interior site of the cavity is fluid"
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        mlups, ms_launch, launches = time_device(s32, nf, args.steps, args.warmup, torch, tstream)
    win32 = time_device.window
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    ms_launch, mlups = over_ranks(ms_launch, nf, world, dist, "cuda")
    clocks = clk.summary(win32)
    e2e_mlups, e2e_ms, h2d, d2h = 0, 0, 0, 0
    if args.e2e_steps > 0:
        if dist:
            dist.barrier()
        e2e_mlups, e2e_ms, h2d, d2h = time_e2e(s32, nf, args.e2e_steps, 3)
        e2e_ms, e2e_mlups = over_ranks(e2e_ms, nf, world, dist, "cuda")
    del s32
    torch.cuda.empty_cache()
    s64, _ = cavity(n, FP64, stream)
    with ClockSampler(local) as clk64:
        mlups64, ms64, _ = time_device(s64, nf, max(args.steps // 4, 20), args.warmup, torch, tstream)
    win64 = time_device.window
    del s64
    torch.cuda.empty_cache()
    s64f, _ = cavity(n, FP64_FAST, stream)
    with ClockSampler(local) as clk64f:
        mlups64f, ms64f, _ = time_device(s64f, nf, max(args.steps // 4, 20), args.warmup, torch, tstream)
    win64f = time_device.window
    del s64f
    torch.cuda.empty_cache()
    s16, _ = cavity(n, FP16, stream)
    with ClockSampler(local) as clk16:
        mlups16, ms16, _ = time_device(s16, nf, args.steps, args.warmup, torch, tstream)
    win16 = time_device.window
    del s16
    torch.cuda.empty_cache()
    err, err16 = l2_error(n, args.err_steps, stream) if args.err_steps > 0 else (None, None)
    peak, peak_kind = measured_peak()
    ach = nf * BYTES_FP32 / (ms_launch * 1e-3) / 1e9
    ach64 = nf * BYTES_FP64 / (ms64 * 1e-3) / 1e9
    line = {
        "metric": cavity_metric(n),
        "value": round(mlups, 3),
        "unit": "MLUPS",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms_launch, 5),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "path": "FP32-shifted fused AA step kernels (jlb_evolve)",
        "config": cavity_config(n),
        "roofline": {"bound": "hbm", "achieved": round(ach, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(ach / peak, 4), "peak_kind": peak_kind,
                     "bytes_per_site": BYTES_FP32, "traffic": profile_traffic("step_fp32")},
        "fp64": {"value": round(mlups64, 3), "unit": "MLUPS", "ms_per_step": round(ms64, 5),
                 "roofline_frac": round(ach64 / peak, 4), "achieved_gbs": round(ach64, 1),
                 "bytes_per_site": BYTES_FP64, "fp32_over_fp64": round(mlups / mlups64, 3),
                 "clocks": clk64.summary(win64)},
        "fp64_fast": {"value": round(mlups64f, 3), "unit": "MLUPS", "ms_per_step": round(ms64f, 5),
                      "roofline_frac": round(nf * BYTES_FP64 / (ms64f * 1e-3) / 1e9 / peak, 4),
                      "achieved_gbs": round(nf * BYTES_FP64 / (ms64f * 1e-3) / 1e9, 1),
                      "bytes_per_site": BYTES_FP64, "over_fp64": round(mlups64f / mlups64, 3),
                      "note": "FP64 state, regrouped FMA-contracted arithmetic; within 1e-12 relative of the "
                              "bitwise FP64 path on the parity cases",
                      "clocks": clk64f.summary(win64f)},
        "fp16": {"value": round(mlups16, 3), "unit": "MLUPS", "ms_per_step": round(ms16, 5),
                 "roofline_frac": round(nf * 76 / (ms16 * 1e-3) / 1e9 / peak, 4),
                 "achieved_gbs": round(nf * 76 / (ms16 * 1e-3) / 1e9, 1), "bytes_per_site": 76,
                 "clocks": clk16.summary(win16)},
        "error": {"vel_rel_l2_fp32_vs_fp64": err, "vel_rel_l2_fp16_vs_fp64": err16, "steps": args.err_steps},
        "e2e": {"value": round(e2e_mlups, 3), "unit": "MLUPS", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": round(e2e_ms, 4),
                "median_ms_per_call": round(getattr(time_e2e, "median_ms", 0.0), 4), "steps": args.e2e_steps,
                "api": "Solver.evolve(1) with page-locked host den/vel"},
        "gpu_launches": launches,
        "clocks": clocks,
    }
    if rank == 0 and world == 1 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(n)
    if world == 1:
        # the other configurations of the metric, each with its own clocks,
        # roofline and error (one GPU only: replicas would only repeat them)
        blocks = {"porous": porous_block, "ensemble": ensemble_block, "adjoint": adjoint_block}
        for name in [b for b in args.blocks.split(",") if b in blocks]:
            t0 = time.perf_counter()
            line[name] = blocks[name](args)
            line[name]["wall_s"] = round(time.perf_counter() - t0, 1)
    if rank == 0:
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
