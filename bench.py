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
  error        relative L2 velocity error of FP32 against FP64 after
               --err-steps steps of the same cavity;
  cpu_baseline the reference's own OpenMP solver on this host's cores.
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

METRIC = "D3Q19 MLUPS (lid-driven cavity 256^3, TRT), FP32-shifted fused AA kernel"
N_DEFAULT = 256
KVISC = (0.56 - 0.5) / 3.0
MAGIC = 0.25
LID = 0.05
BYTES_FP32 = 152
BYTES_FP64 = 304


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
    """nvidia-smi samples of SM clocks and throttle reasons during a region."""

    FIELDS = ("clocks.sm,clocks.max.sm,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.proc = None
        self.out = os.path.join("/tmp", f"jlb_clocks_{os.getpid()}.csv")
        self.index = index

    def __enter__(self):
        try:
            self.fh = open(self.out, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.fh, stderr=subprocess.DEVNULL)
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

    def summary(self):
        if self.proc is None or not os.path.exists(self.out):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.out):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.remove(self.out)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "samples": len(sm), "reasons": sorted(reasons)}


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
    e0.record(st)
    assert lib.jlb_step(h, steps, 0) == 0
    e1.record(st)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    launches = s.kernel_launches - l0
    return nf * steps / (ms * 1e-3) / 1e6, ms / steps, launches


def time_e2e(s, nf, steps, warmup):
    """MLUPS through Solver.evolve(1): per-call inputs uploaded, den/vel
    downloaded into the host arrays every step."""
    for _ in range(warmup):
        s.evolve(1)
    b0 = s.transfer_bytes
    t0 = time.perf_counter()
    for _ in range(steps):
        s.evolve(1)
    dt = time.perf_counter() - t0
    b1 = s.transfer_bytes
    return (nf * steps / dt / 1e6, dt * 1e3 / steps, (b1[0] - b0[0]) // steps, (b1[1] - b0[1]) // steps)


def l2_error(n, steps, stream):
    from jyulb.defs import FP32, FP64

    s64, nf = cavity(n, FP64, stream)
    s64.evolve(steps)
    v64 = np.array(s64.get_vel())
    del s64
    s32, _ = cavity(n, FP32, stream)
    s32.evolve(steps)
    v32 = np.array(s32.get_vel())
    del s32
    return float(np.linalg.norm(v32 - v64) / np.linalg.norm(v64))


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


def run_ensemble(args):
    import torch
    from jyulb.defs import BGK, FP64
    from jyulb.ensemble import Ensemble
    from jyulb.isothermal import Solver

    torch.cuda.set_device(0)
    t0 = time.perf_counter()
    doms = ensemble_domains(args.domains)
    ens = Ensemble(doms, BGK)
    setup_s = time.perf_counter() - t0
    info = ens.info()
    nf = info["fluid_sites"]
    ens.evolve(args.warmup)
    torch.cuda.synchronize()
    l0 = ens.info()["launches"]
    with ClockSampler(0) as clk:
        t0 = time.perf_counter()
        ens.evolve(args.steps)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
    launches = ens.info()["launches"] - l0
    mlups = nf * args.steps / dt / 1e6
    # per-domain check: FP64 single-domain runs of a sample of domains, same
    # total step count
    errs = []
    total = args.warmup + args.steps
    for d in range(0, len(doms), max(1, len(doms) // args.check_domains))[: args.check_domains]:
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
    peak, peak_kind = measured_peak()
    ach = nf * BYTES_FP32 / (dt / args.steps) / 1e9
    line = {
        "metric": "D3Q19 MLUPS, batched ensemble of channels (FP32 shifted, one launch per step)",
        "value": round(mlups, 3), "unit": "MLUPS", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(dt * 1e3 / args.steps, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"{len(doms)} channels nx~U[32,256] ny~U[16,128] nz~U[8,64], tau~U[0.55,1.5], "
                               "gx~U[1e-7,1e-5], half with moving top wall u~U[0.01,0.05]; BGK",
                   "domains": len(doms), "packed_sites": info["sites"], "fluid_sites": nf,
                   "setup_s": round(setup_s, 1), "autotuned_block": info["block"],
                   "autotune_ns_per_step": info["tune_ns_per_step"]},
        "roofline": {"bound": "hbm", "achieved": round(ach, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(ach / peak, 4), "peak_kind": peak_kind, "bytes_per_site": BYTES_FP32},
        "error": {"domains_checked": len(errs), "vel_rel_l2_vs_fp64_max": max(errs) if errs else None,
                  "vel_rel_l2_vs_fp64_median": statistics.median(errs) if errs else None, "steps": total},
        "gpu_launches": launches, "clocks": clk.summary(),
    }
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
        "impl": "reference", "metric": METRIC.replace("FP32-shifted fused AA kernel", "reference CPU solver"),
        "value": round(r["mlups"], 3), "unit": "MLUPS", "n_gpus": args.gpus, "steps": r["steps"],
        "warmup": args.warmup, "ms_per_step": round(r["sec"] * 1e3 / r["steps"], 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": {"workload": f"lid-driven cavity {n}^3 TRT, Zou-He lid on +y",
                                        "threads": cores},
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
    ap.add_argument("--err-steps", type=int, default=1000)
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--workload", default="cavity", choices=["cavity", "ensemble"])
    ap.add_argument("--domains", type=int, default=512)
    ap.add_argument("--check-domains", type=int, default=6)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference_arm(args)
    if args.workload == "ensemble":
        return run_ensemble(args)

    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    from jyulb.defs import FP32, FP64

    n = args.size
    tstream = torch.cuda.Stream()
    stream = tstream.cuda_stream
    # replicas only: every rank advances its own cavity (the path has no
    # exchange step on one domain per GPU)
    s32, nf = cavity(n, FP32, stream)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        mlups, ms_launch, launches = time_device(s32, nf, args.steps, args.warmup, torch, tstream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
        t = torch.tensor([ms_launch], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_launch = float(t.item())
        mlups = nf * world / (ms_launch * 1e-3) / 1e6
    clocks = clk.summary()
    e2e_mlups, e2e_ms, h2d, d2h = time_e2e(s32, nf, args.e2e_steps, 3) if args.e2e_steps > 0 else (0, 0, 0, 0)
    del s32
    torch.cuda.empty_cache()
    s64, _ = cavity(n, FP64, stream)
    with ClockSampler(local) as clk64:
        mlups64, ms64, _ = time_device(s64, nf, max(args.steps // 4, 20), args.warmup, torch, tstream)
    del s64
    torch.cuda.empty_cache()
    err = l2_error(n, args.err_steps, stream) if args.err_steps > 0 else None
    peak, peak_kind = measured_peak()
    ach = nf * BYTES_FP32 / (ms_launch * 1e-3) / 1e9
    ach64 = nf * BYTES_FP64 / (ms64 * 1e-3) / 1e9
    line = {
        "metric": METRIC,
        "value": round(mlups * (1 if dist is None else 1), 3),
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
        "config": {"workload": f"lid-driven cavity {n}^3, TRT tau+=0.56 magic 1/4, Zou-He lid u=(0.05,0,0) on +y, "
                               "bounce-back elsewhere", "fluid_sites": nf, "precision": "FP32 shifted",
                   "l2_policy": "inputs larger than L2 (1.3 GB populations), no flush",
                   "multi_gpu": "replicas only"},
        "roofline": {"bound": "hbm", "achieved": round(ach, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(ach / peak, 4), "peak_kind": peak_kind,
                     "bytes_per_site": BYTES_FP32, "traffic": profile_traffic("step_fp32")},
        "fp64": {"value": round(mlups64, 3), "unit": "MLUPS", "ms_per_step": round(ms64, 5),
                 "roofline_frac": round(ach64 / peak, 4), "achieved_gbs": round(ach64, 1),
                 "bytes_per_site": BYTES_FP64, "fp32_over_fp64": round(mlups / mlups64, 3),
                 "clocks": clk64.summary()},
        "error": {"vel_rel_l2_fp32_vs_fp64": err, "steps": args.err_steps},
        "e2e": {"value": round(e2e_mlups, 3), "unit": "MLUPS", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": round(e2e_ms, 4),
                "api": "Solver.evolve(1) with page-locked host den/vel"},
        "gpu_launches": launches,
        "clocks": clocks,
    }
    if rank == 0 and world == 1 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(n)
    if rank == 0:
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
