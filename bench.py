"""Benchmark of the GB300 DEM step (prints one JSON line on rank 0).

A bench "step" is one frame of the reference's compute(): `frame` simulation
steps of LOM + Simulation over the whole scene (WGPUComputeProg::compute with
gen_per_frame steps, src/wgpu_prog.rs:1420-1473; the reference default is
105, src/settings.rs:322).  The metric is particle-steps/s = particles x
simulation steps / device time.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload c3_batch|c4_serve|c1_chains|c0_settle|c2_impact|dense_bed] [--frame F]

  python bench.py --profile-steps K [--workload ...] [knobs] -- a profiling
  target, not a bench: K steps of the workload with plain kernel launches
  (profilers cannot see kernels inside graphs with conditional nodes) and
  the given knobs, then exit; nothing is timed.

--impl reference times the reference's algorithm on the host cores: the CPU
restatement under oracle/ (the reference's own WGSL-through-wgpu step cannot
run without a graphics stack), with every host thread, on a bounded sample of
the same workload.  Under torchrun only rank 0 runs it.
"""
import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in ("physics-sim_gb300", "oracle"):
    _q = os.path.join(ROOT, _p)
    if _q not in sys.path:
        sys.path.insert(0, _q)

import numpy as np  # noqa: E402

L2_BYTES = 129 * 1024 * 1024
FLUSH_BYTES = 2 * L2_BYTES


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=0)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c3_batch")
    ap.add_argument("--frame", type=int, default=0)
    ap.add_argument("--scenes", type=int, default=512)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--horizon", type=int, default=5000,
                    help="c3: simulation steps per scene the timed frames cover from the initial states")
    ap.add_argument("--settle-steps", type=int, default=20000,
                    help="c3: also time two frames after the mix has run this many steps (0: skip)")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--serve-rate", type=float, default=200.0)
    ap.add_argument("--serve-seconds", type=float, default=60.0)
    ap.add_argument("--serve-min", type=int, default=2000)
    ap.add_argument("--serve-max", type=int, default=256000)
    ap.add_argument("--serve-hmin", type=int, default=1000)
    ap.add_argument("--serve-hmax", type=int, default=20000)
    ap.add_argument("--serve-pool", type=int, default=48)
    ap.add_argument("--serve-budget-gb", type=float, default=150.0)
    ap.add_argument("--serve-active", type=int, default=16 << 20)
    ap.add_argument("--serve-timeout", type=float, default=900.0)
    ap.add_argument("--no-tune", action="store_true", help="library defaults instead of the autotuner's picks")
    ap.add_argument("--profile-steps", type=int, default=0,
                    help="profiling target: run this many steps with plain launches and exit (nothing timed)")
    ap.add_argument("--particles", type=int, default=0, help="dense_bed: particles")
    ap.add_argument("--c2-cols", type=int, default=1024, help="c2_impact: lattice columns (a crop when < 1024)")
    ap.add_argument("--c2-rows", type=int, default=4096, help="c2_impact: lattice rows (a crop when < 4096)")
    ap.add_argument("--cell-factor", type=float, default=0.0, help="--profile-steps: search_cell_factor")
    ap.add_argument("--skin", type=float, default=0.0, help="--profile-steps: list_skin")
    ap.add_argument("--block", type=int, default=0, help="--profile-steps: block_size")
    ap.add_argument("--graph-steps", type=int, default=35, help="--profile-steps: reorder_interval")
    ap.add_argument("--split", action="store_true", help="--profile-steps: k_narrow + k_forces")
    ap.add_argument("--reorder-every", type=int, default=0,
                    help="rebuilds per reorder into cell order (dem_ext.reorder_every; 0: library default)")
    ap.add_argument("--unfused", action="store_true", help="--profile-steps: a LOM kernel every step")
    ap.add_argument("--plain", action="store_true",
                    help="plain kernel launches instead of CUDA graphs, so that ncu can list every "
                         "launch (a profiling aid, not a bench configuration)")
    return ap.parse_args()


def build_workload(name, args=None):
    import dem_scenes
    if name == "c1_chains":
        sc, p, ext = dem_scenes.c1_chains()
        desc = {"workload": "c1 bonded chain tensile test", "chains": 64, "chain_length": 256,
                "particles": 64 * 256, "bond_model": "parallel (bonds=3)", "bond_radius_factor": 0.8,
                "bond_strengths": "Weibull(8, 5e3) per bond", "dt": 1e-4}
    elif name == "c0_settle":
        sc, p, ext = dem_scenes.c0_settle()
        desc = {"workload": "c0 granular settle", "particles": 4096, "box": [128, 256], "dt": 1e-4}
    elif name == "dense_bed":
        n = (args.particles if args is not None and args.particles > 0 else 0) or (1 << 20)
        sc, p, ext = dem_scenes.dense_bed(n=n)
        desc = {"workload": "dense bed (c0 particle model, packed)", "particles": n, "dt": 1e-4}
    elif name == "c2_impact":
        cols, rows = (args.c2_cols, args.c2_rows) if args is not None else (1024, 4096)
        sc, p, ext = dem_scenes.c2_impact(cols=cols, rows=rows)
        nb = int(sc["bonds"].shape[0] // 3)
        desc = {"workload": "c2 single large impact scene" + ("" if (cols, rows) == (1024, 4096) else " (crop)"),
                "particles": int(sc["radii"].shape[0]),
                "bed": [2 * cols, 2 * rows], "lattice": "%d x %d, pitch 2" % (cols, rows),
                "radii": "log-normal, median 1, sigma 0.15",
                "bonded_fraction": 0.3, "clusters": "horizontal runs of 4-32", "bonds": nb,
                "bond_model": "parallel (bonds=3), factor 0.8, Weibull(8, 5e3) strengths",
                "projectile": {"radius": 40, "speed": 50}, "dt": 5e-5}
    else:
        raise SystemExit("unknown workload %s" % name)
    return sc, p, ext, desc


def cpu_sample_workload(name, sc, p, ext):
    """The scene the CPU arms time.  For c2 a 128 x 256 crop of the same bed
    model with the same r = 40 projectile: the reference's bucket side is set
    by the largest radius (80), so each particle scans as many bucket members
    as in the full scene and the per-particle cost is the same."""
    if name == "c2_impact":
        import dem_scenes
        s2, p2, e2 = dem_scenes.c2_impact(cols=128, rows=256)
        return s2, p2, e2, "c2 crop: 128 x 256 bed + r=40 projectile (%d particles)" % s2["radii"].shape[0]
    return sc, p, ext, None


def build_batch_workload(n_scenes, seed):
    import dem_scenes
    items = dem_scenes.c3_batch(n_scenes=n_scenes, seed=seed)
    ns = [int(it[0]["radii"].shape[0]) for it in items]
    nb = [int(it[0]["bonds"].shape[0] // 3) if it[0]["bonds"].shape[0] >= 3 else 0 for it in items]
    desc = {"workload": "c3 batched uneven scenes", "scenes": n_scenes,
            "particles": int(sum(ns)), "particles_per_scene": "log-uniform [1000, 64000] (min %d, max %d)"
            % (min(ns), max(ns)), "bond_fraction": "uniform [0, 0.5]", "bonds": int(sum(nb)),
            "scene_model": "loose c0 disks + bonded chains of 32 (parallel bonds, factor 0.8, Weibull strengths)",
            "dt": 1e-4, "seed": seed}
    return items, desc


def job_rate(units, dev_ms, ws, device):
    """Whole-job throughput of the replicas: the units every rank processed
    (summed over ranks) over the slowest rank's device time (max over ranks).
    Returns (units per second, max ms, total units)."""
    if ws > 1:
        import torch
        import torch.distributed as dist
        u = torch.tensor([float(units)], dtype=torch.float64, device=device)
        m = torch.tensor([float(dev_ms)], dtype=torch.float64, device=device)
        dist.all_reduce(u, op=dist.ReduceOp.SUM)
        dist.all_reduce(m, op=dist.ReduceOp.MAX)
        units, dev_ms = float(u.item()), float(m.item())
    return units / (dev_ms / 1e3), dev_ms, units


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 100 ms."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.f = tempfile.NamedTemporaryFile(mode="w+", suffix=".csv", delete=False)
        self.p = None
        self.marks = []

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.QUERY,
                                       "--format=csv,noheader,nounits", "-lms", "100"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def mark(self):
        self.f.flush()
        try:
            self.marks.append(sum(1 for _ in open(self.f.name)))
        except OSError:
            self.marks.append(0)

    def stop(self):
        if self.p is not None:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.p.kill()
        self.f.flush()

    def summary(self):
        try:
            lines = [l.strip() for l in open(self.f.name) if l.strip()]
        except OSError:
            lines = []
        if len(self.marks) >= 2 and self.marks[1] > self.marks[0]:
            window = lines[self.marks[0]:self.marks[1]]
        else:
            window = lines
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in window:
            c = [x.strip() for x in l.split(",")]
            if len(c) < 9:
                continue
            try:
                sm.append(float(c[1]))
                mx = float(c[2])
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if c[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        try:
            os.unlink(self.f.name)
        except OSError:
            pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(path))
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profiled_traffic(workload):
    """dram bytes per k_interact launch recorded from an ncu capture under profiles/."""
    path = os.path.join(ROOT, "profiles", "k_interact_%s.md" % workload)
    try:
        txt = open(path).read()
    except OSError:
        return None
    m = re.search(r"dram_bytes_per_launch:\s*([0-9.eE+]+)", txt)
    return float(m.group(1)) if m else None


def interact_bytes(s_u, s_b, n, fused):
    """Algorithmic bytes of one Simulation-kernel launch (the per-step byte
    model of the workload definition): 12 per unbonded and 36 per bonded
    directed slot, plus per
    particle the force pass's 56 (pos, r, del_pos, del_rot, material,
    external force read; acc, rot_acc, vel, rot_vel written) or, when the
    kernel also carries the next step's LOM pass, the whole 120-byte state
    round trip of a step."""
    return 12 * s_u + 36 * s_b + (120 if fused else 56) * n


def slot_counts(st):
    c = st["contacts"].reshape(-1, 6)
    occ = c[:, 1] != -1
    bonded = occ & (c[:, 5] >= 0)
    return int((occ & ~bonded).sum()), int(bonded.sum())


def fp64_twin_error(samples, device):
    """Error of the FP32 path against the FP64 transcription of the same step
    (the oracle's twin, a checker run on the host): for each sampled state,
    one step through the library (a Context on that state) and one step of
    the twin; per particle |a32 - a64| / scale with scale = (|data[0]| +
    m g) / m, i.e. the particle's normal-force total (data[0] = sum of F_n)
    plus its weight, as an acceleration.  `samples` are (state, params, ext)."""
    import dem
    import oracle
    errs = []
    for st, p, ext in samples:
        with dem.Context({k: (v.copy() if hasattr(v, "copy") else v) for k, v in st.items()}, p,
                         device=device, **ext) as ctx:
            ctx.step(1)
            s1 = ctx.download()
        twin = oracle.step_f64(st, p, 1, **_okw(ext))
        r = st["radii"].astype(np.float64)
        dens = st["materials"].reshape(-1, 6)[st["material_pointers"], 3].astype(np.float64)
        mass = dens * np.pi * r * r
        live = r > 0
        a32 = s1["acc"].reshape(-1, 2).astype(np.float64)[live]
        a64 = twin["acc"].reshape(-1, 2)[live]
        fsum = np.abs(s1["data"].reshape(-1, 7)[live, 0].astype(np.float64))
        g = 9.81 * float(p.get("gravity_acc", 1.0)) if p.get("gravity", 0) else 0.0
        scale = (fsum + mass[live] * g) / mass[live]
        ok = scale > 0
        errs.append(np.linalg.norm(a32 - a64, axis=1)[ok] / scale[ok])
    e = np.concatenate(errs) if errs else np.zeros(1)
    return {"max": float(e.max()), "median": float(np.median(e)), "p99": float(np.percentile(e, 99)),
            "particles": int(e.size), "states": len(samples),
            "scale": "per particle (|sum F_n| + m g) / m: one FP32 step of the library vs one step of the "
                     "oracle's FP64 twin from the same state"}


def cpu_baseline(sc, p, ext, seconds, frame):
    """The oracle (reference-mode FP32 CPU restatement) on a bounded sample of
    the same workload, all host threads."""
    import oracle
    okw = {}
    if "bond_lambda" in ext:
        okw["bond_lambda"] = ext["bond_lambda"]
    if "bond_sn" in ext:
        okw["bond_sn"], okw["bond_ss"] = ext["bond_sn"], ext["bond_ss"]
    s = {k: (v.copy() if hasattr(v, "copy") else v) for k, v in sc.items()}
    n = int(s["radii"].shape[0])
    t0 = time.perf_counter()
    oracle.step(s, p, 1, **okw)
    t1 = time.perf_counter()
    per = max(t1 - t0, 1e-6)
    k = int(max(1, min(seconds / per, 50 * frame)))
    t0 = time.perf_counter()
    oracle.step(s, p, k, step_base=1, **okw)
    dt = time.perf_counter() - t0
    cores = os.cpu_count() or 1
    return {"value": n * k / dt, "unit": "particle-steps/s", "cores": cores, "kind": "port",
            "sample": "%d consecutive steps of the %d-particle scene from its initial state "
                      "(%.1f s, OpenMP over particles)" % (k, n, dt)}, n * k / dt


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    sc, p, ext, desc = build_workload(args.workload, args)
    sc, p, ext, crop = cpu_sample_workload(args.workload, sc, p, ext)
    if crop:
        desc = dict(desc)
        desc["cpu_sample_scene"] = crop
    import oracle
    okw = {}
    if "bond_lambda" in ext:
        okw["bond_lambda"] = ext["bond_lambda"]
    if "bond_sn" in ext:
        okw["bond_sn"], okw["bond_ss"] = ext["bond_sn"], ext["bond_ss"]
    n = int(sc["radii"].shape[0])
    s = {k: (v.copy() if hasattr(v, "copy") else v) for k, v in sc.items()}
    # bounded sample per bench step: enough simulation steps for ~1 s of CPU work
    t0 = time.perf_counter()
    oracle.step(s, p, 1, **okw)
    per = max(time.perf_counter() - t0, 1e-6)
    sub = int(max(1, min(args.frame, 1.0 / per)))
    step_base = 1
    for _ in range(args.warmup):
        oracle.step(s, p, sub, step_base=step_base, **okw)
        step_base += sub
    t0 = time.perf_counter()
    for _ in range(args.steps):
        oracle.step(s, p, sub, step_base=step_base, **okw)
        step_base += sub
    dt = time.perf_counter() - t0
    value = n * sub * args.steps / dt
    cores = os.cpu_count() or 1
    cfg = dict(desc)
    cfg.update({"frame_steps": args.frame, "sample_steps_per_bench_step": sub})
    line = {"metric": "particle-steps/s", "value": value, "unit": "particle-steps/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "impl": "reference", "config": cfg,
            "cpu_baseline": {"value": value, "unit": "particle-steps/s", "cores": cores, "kind": "port",
                             "sample": "%d steps per bench step, %d bench steps, all host threads" % (sub, args.steps)},
            "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def scene_bytes(sc):
    keys = ("pos", "radii", "vel", "acc", "rot", "rot_vel", "rot_acc", "forces", "fixity", "del_pos",
            "del_rot", "bonds", "contacts", "material_pointers", "materials", "data")
    return int(sum(sc[k].nbytes for k in keys))


def run_ours(args):
    import torch
    import build_lib
    import dem
    build_lib.build()
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    sc, p, ext, desc = build_workload(args.workload, args)
    n = int(sc["radii"].shape[0])
    F = args.frame
    # autotuner (cell size, skin, block size, steps per graph, one or two
    # Simulation kernels) on the scene itself, before anything is timed
    knobs, tune_info = {"reorder_interval": 21}, None
    if not args.no_tune and not args.plain:
        knobs, tune_info = dem.autotune([(sc, p, ext)], device=local)
    g = knobs["reorder_interval"]
    F = args.frame if args.frame_given else g * max(1, -(-105 // g))
    if args.reorder_every > 0:
        knobs = dict(knobs, reorder_every=args.reorder_every)
    ctx = dem.Context(sc, p, device=local, plain_launches=args.plain, **knobs, **ext)
    stream = torch.cuda.ExternalStream(ctx.stream(), device=dev)
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device=dev)

    def barrier():
        torch.cuda.synchronize(dev)
        ctx.synchronize()
        if ws > 1:
            torch.distributed.barrier()

    for _ in range(args.warmup):
        ctx.step(F)
    barrier()
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    launches0 = ctx.stats()["kernel_launches"]
    sampler.mark()
    barrier()
    evs = []
    wall0 = time.perf_counter()
    for k in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(float(k))          # L2 flush between frames, outside the events
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ctx.step(F)
        e1.record(stream)
        evs.append((e0, e1))
    barrier()
    wall = time.perf_counter() - wall0
    sampler.mark()
    launches = ctx.stats()["kernel_launches"] - launches0
    sampler.stop()
    dev_ms = sum(a.elapsed_time(b) for a, b in evs)
    value, max_ms, _ = job_rate(n * F * args.steps, dev_ms, ws, dev)
    clocks = sampler.summary()

    # roofline pass: events around every k_interact launch, same stream, plain launches
    ctx.kernel_timing(True)
    ctx.step(2 * F)
    int_ms, int_n = ctx.kernel_time("interact")
    lom_ms, lom_n = ctx.kernel_time("lom")
    bp_ms, bp_n = ctx.kernel_time("broad_phase")
    ctx.kernel_timing(False)
    st = ctx.download()
    s_u, s_b = slot_counts(st)
    fused = not knobs.get("unfused_lom", 0)
    alg_bytes = interact_bytes(s_u, s_b, n, fused)
    avg_s = (int_ms / max(int_n, 1)) / 1e3
    peak, peak_kind = measured_peaks()
    achieved = alg_bytes / avg_s / 1e9
    traffic = profiled_traffic(args.workload)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
                "kernel": "k_interact + next step's LOM pass" if fused else "k_interact",
                "launch_us": avg_s * 1e6,
                "algorithmic_bytes_per_launch": alg_bytes,
                "slots_unbonded": s_u, "slots_bonded": s_b,
                "lom_us": lom_ms / max(lom_n, 1) * 1e3, "broad_phase_us": bp_ms / max(bp_n, 1) * 1e3}

    # end to end through the public API: restore from host arrays, one frame, update_state
    import dem as _dem
    host = {k: (v.copy() if hasattr(v, "copy") else v) for k, v in st.items()}
    h2d = scene_bytes(host)
    d2h = h2d
    e2e_n = max(1, args.e2e_steps)
    ctx.upload(host)
    ctx.step(F)
    out = ctx.download()          # the caller's arrays, allocated once (State owns its vectors)
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_n):
        ctx.upload(host)
        ctx.step(F)
        ctx.download(out)
    barrier()
    e2e_s = time.perf_counter() - t0
    del out, _dem
    e2e = {"value": job_rate(n * F * e2e_n, e2e_s * 1e3, ws, dev)[0], "unit": "particle-steps/s",
           "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": d2h,
           "note": "dem_upload (restore) of the whole scene + dem_step(frame) + dem_download (update_state)"}

    base = None
    fp64 = None
    if rank == 0 and ws == 1:
        csc, cp, cext, crop = cpu_sample_workload(args.workload, sc, p, ext)
        base, _ = cpu_baseline(csc, cp, cext, args.cpu_seconds, F)
        if crop:
            base["sample"] = crop + "; " + base["sample"]
        fp64 = fp64_twin_error([(st, p, ext)], local)
        fp64["state"] = "the scene after the timed frames and the roofline pass"
    cfg = dict(desc)
    cfg.update({"frame_steps": F, "parallelism": "replicas" if ws > 1 else "single",
                "l2": "flushed between frames (write of %d MiB on the stream, untimed)" % (FLUSH_BYTES >> 20),
                "knobs": knobs, "autotune": tune_info, "graphs": True})
    line = {"metric": "particle-steps/s", "value": value, "unit": "particle-steps/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": max_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": cfg, "clocks": clocks, "roofline": roofline,
            "e2e": e2e, "gpu_launches": int(launches), "wall_s": wall}
    if fp64 is not None:
        line["fp64_error"] = fp64
    if base is not None:
        line["cpu_baseline"] = base
    ctx.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


def _okw(ext):
    kw = {}
    if "bond_lambda" in ext:
        kw["bond_lambda"] = ext["bond_lambda"]
    if "bond_sn" in ext:
        kw["bond_sn"], kw["bond_ss"] = ext["bond_sn"], ext["bond_ss"]
    return kw


def run_reference_batch(args):
    """The CPU restatement of the reference step over the batched mix: each
    bench step advances one scene of the mix (cycling through them) by a
    bounded number of steps, all host threads."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    import oracle
    items, desc = build_batch_workload(args.scenes, args.seed)
    states = [{k: (v.copy() if hasattr(v, "copy") else v) for k, v in it[0].items()} for it in items]
    done = [0] * len(items)

    def one(k, steps):
        sc, p, ext = items[k]
        oracle.step(states[k], p, steps, step_base=done[k], **_okw(ext))
        done[k] += steps
        return int(sc["radii"].shape[0]) * steps

    sub = args.frame if args.frame_given else max(1, args.horizon // max(args.steps, 1))
    for w in range(args.warmup):
        one(w % len(items), 1)
    tot = 0
    t0 = time.perf_counter()
    for k in range(args.steps):
        tot += one(k % len(items), sub)
    dt = time.perf_counter() - t0
    value = tot / dt
    cores = os.cpu_count() or 1
    cfg = dict(desc)
    cfg.update({"frame_steps": sub, "horizon": "%d steps per scene from the initial states" % args.horizon,
                "sample": "scene k mod %d advanced %d steps per bench step from its initial state"
                % (len(items), sub)})
    line = {"metric": "particle-steps/s", "value": value, "unit": "particle-steps/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "impl": "reference", "config": cfg,
            "cpu_baseline": {"value": value, "unit": "particle-steps/s", "cores": cores, "kind": "port",
                             "sample": "%d bench steps of %d steps on scenes of the mix, all host threads"
                             % (args.steps, sub)},
            "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours_batch(args):
    """c3: the 512-scene mix in one batch.  The timed frames run every scene
    from its initial state over the configured horizon (frames of F steps, F
    a multiple of the autotuned graph length, K frames covering at least
    --horizon steps); warm-up frames run first on the same batch, which is
    then restored to the initial states (dem_batch_upload_many) before the
    timed region."""
    import torch
    import build_lib
    import dem
    build_lib.build()
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    items, desc = build_batch_workload(args.scenes, args.seed + rank)
    ntot = sum(int(it[0]["radii"].shape[0]) for it in items)
    # autotuner: cell size, list skin (re-sort interval), block size and steps
    # per graph, picked on a sample of the scenes before anything is timed
    knobs, tune_info = {"reorder_interval": 35}, None
    if not args.no_tune and not args.plain:
        knobs, tune_info = dem.autotune(items, device=local)
    g = knobs["reorder_interval"]
    if args.frame_given:
        F = args.frame
    else:
        F = g * max(1, -(-args.horizon // (args.steps * g)))
    if args.reorder_every > 0:
        knobs = dict(knobs, reorder_every=args.reorder_every)
    batch = dem.Batch(items, device=local, plain_launches=args.plain, **knobs)
    stream = torch.cuda.ExternalStream(batch.stream(), device=dev)
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    initial = dem.SceneTable([(k, it[0]) for k, it in enumerate(items)])

    def barrier():
        torch.cuda.synchronize(dev)
        batch.synchronize()
        if ws > 1:
            torch.distributed.barrier()

    def slots_now():
        su = sb = 0
        for k in range(len(items)):
            a, b2 = slot_counts(batch.download(k))
            su += a
            sb += b2
        return su, sb

    for _ in range(args.warmup):
        batch.step(F)
    barrier()
    batch.upload_many(initial)        # back to the initial states: the timed frames cover the horizon
    barrier()
    slots_start = slots_now()
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    launches0 = batch.stats()["kernel_launches"]
    rebuilds0 = batch.stats()["reorders"]
    sampler.mark()
    barrier()
    evs = []
    wall0 = time.perf_counter()
    for k in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(float(k))
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        batch.step(F)
        e1.record(stream)
        evs.append((e0, e1))
    barrier()
    wall = time.perf_counter() - wall0
    sampler.mark()
    st = batch.stats()
    launches = st["kernel_launches"] - launches0
    sampler.stop()
    dev_ms = sum(a.elapsed_time(b) for a, b in evs)
    frame_ms = [a.elapsed_time(b) for a, b in evs]
    value, max_ms, _ = job_rate(ntot * F * args.steps, dev_ms, ws, dev)
    clocks = sampler.summary()
    states = [batch.download(k) for k in range(len(items))]
    s_u = s_b = 0
    for stt in states:
        a, b2 = slot_counts(stt)
        s_u += a
        s_b += b2

    # roofline of the Simulation kernel on the state at the end of the
    # horizon (plain launches with events around every launch)
    fused = not knobs.get("unfused_lom", 0)
    alg_bytes = interact_bytes(s_u, s_b, ntot, fused)
    peak, peak_kind = measured_peaks()
    roofline = {"bound": "hbm", "peak": peak, "unit": "GB/s", "peak_source": peak_kind,
                "kernel": "k_interact + next step's LOM pass" if fused else "k_interact",
                "state": "end of the timed horizon (step %d)" % (F * args.steps),
                "algorithmic_bytes_per_launch": alg_bytes,
                "slots_unbonded": s_u, "slots_bonded": s_b, "traffic": profiled_traffic(args.workload)}
    try:
        kt = BatchKernelTimer(batch)
        kt.run(2 * F)
        roofline.update(kt.figures(alg_bytes, peak))
    except Exception as exc:  # timing is diagnostic; the value above stands
        roofline["error"] = str(exc)
    states = [batch.download(k) for k in range(len(items))]

    # the same scenes through the plain single-scene path, one after another,
    # each from its state at the end of the horizon (F steps)
    plain_ms = 0.0
    plain_ps = 0
    for (sc, p, ext), stt in zip(items, states):
        ctx = dem.Context(stt, p, device=local, reorder_interval=35, plain_launches=args.plain, **ext)
        cst = torch.cuda.ExternalStream(ctx.stream(), device=dev)
        ctx.step(35)
        ctx.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(cst)
        ctx.step(F)
        e1.record(cst)
        e1.synchronize()
        plain_ms += e0.elapsed_time(e1)
        plain_ps += int(sc["radii"].shape[0]) * F
        ctx.close()
    plain_value = plain_ps / (plain_ms / 1e3)

    # end to end through the batch API: restore every scene from host arrays,
    # one frame, read every scene back
    # (host arrays are the caller's, allocated once, as State owns its vectors)
    h2d = sum(scene_bytes(x) for x in states)
    outs = [batch.download(k) for k in range(len(items))]
    # the callers' scene structs are built once, as a C caller keeps its
    # dem_scene table; one untimed cycle first (it allocates the staging the
    # bulk calls keep, as the warm-up steps do for the device buffers)
    up_tab = dem.SceneTable(list(enumerate(states)))
    down_tab = dem.SceneTable(list(enumerate(outs)))
    batch.upload_many(up_tab)
    batch.step(F)
    batch.download_many(down_tab)
    barrier()
    e2e_n = max(1, args.e2e_steps)
    t0 = time.perf_counter()
    for _ in range(e2e_n):
        batch.upload_many(up_tab)
        batch.step(F)
        batch.download_many(down_tab)
    barrier()
    e2e_s = time.perf_counter() - t0
    # one more cycle, each call waited for, for the breakdown (not in the value)
    parts = {}
    for name, fn in (("upload_ms", lambda: batch.upload_many(up_tab)), ("frame_ms", lambda: batch.step(F)),
                     ("download_ms", lambda: batch.download_many(down_tab))):
        barrier()
        t1 = time.perf_counter()
        fn()
        barrier()
        parts[name] = (time.perf_counter() - t1) * 1e3
    del up_tab, down_tab
    single = {"value": job_rate(ntot * F * e2e_n, e2e_s * 1e3, ws, dev)[0], "cycle_ms": e2e_s * 1e3 / e2e_n,
              "breakdown_ms": parts}

    # The same cycle with the mix held as two batches (alternate scenes), so
    # that one half's transfers overlap the other half's frame: upload A and
    # step it, read B's previous frame back, upload B and step it, read A
    # back.  Every cycle still moves every scene in and out once.  The halves
    # move their arrays with host threads through page-locked blocks and the
    # copy engines (dem_ext.host_copies), which leaves the SMs to the other
    # half's frame (measured on the mix: 121 ms per cycle against 136 ms
    # with the device's own copy kernels, and 140 ms for one batch).
    halves = [list(range(0, len(items), 2)), list(range(1, len(items), 2))]
    hb = [dem.Batch([items[k] for k in idx], device=local, plain_launches=args.plain, host_copies=1, **knobs)
          for idx in halves]
    h_up = [dem.SceneTable([(j, states[k]) for j, k in enumerate(idx)]) for idx in halves]
    h_down = [dem.SceneTable([(j, outs[k]) for j, k in enumerate(idx)]) for idx in halves]

    def pipelined(n):
        A, B = hb
        for c in range(n):
            A.upload_many(h_up[0])
            A.step(F)
            if c > 0:
                B.download_many(h_down[1])
            B.upload_many(h_up[1])
            B.step(F)
            A.download_many(h_down[0])
        B.download_many(h_down[1])

    pipelined(1)                      # untimed: staging and graphs of both halves
    for b in hb:
        b.synchronize()
    barrier()
    t0 = time.perf_counter()
    pipelined(e2e_n)
    for b in hb:
        b.synchronize()
    barrier()
    pipe_s = time.perf_counter() - t0
    for b in hb:
        b.close()
    del outs, hb, h_up, h_down
    e2e = {"value": job_rate(ntot * F * e2e_n, pipe_s * 1e3, ws, dev)[0], "unit": "particle-steps/s",
           "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": h2d,
           "cycle_ms": pipe_s * 1e3 / e2e_n,
           "single_batch": single,
           "note": "per cycle every scene is restored from the caller's host arrays (dem_batch_upload_many), "
                   "advanced one frame (dem_batch_step) and read back into the caller's arrays "
                   "(dem_batch_download_many), from the states at the end of the horizon; the mix is held as "
                   "two batches of alternate scenes so that one half's transfers overlap the other half's "
                   "frame, each half moving its arrays through page-locked blocks by host threads and the copy "
                   "engines (dem_ext.host_copies = 1); single_batch: the same cycle on one batch whose copy "
                   "kernels read and write the callers' arrays, calls in sequence (its breakdown_ms: one extra "
                   "cycle with each call waited for)"}

    # settled states: the mix run on (untimed) to --settle-steps, then frames timed there
    settled = None
    if args.settle_steps > F * args.steps:
        batch.upload_many(dem.SceneTable(list(enumerate(states))))
        left = args.settle_steps - F * args.steps - F
        batch.step(max(left - left % g, 0))
        barrier()
        su2, sb2 = slots_now()
        sev = []
        for k in range(2):
            with torch.cuda.stream(stream):
                flush.fill_(float(k))
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            batch.step(F)
            e1.record(stream)
            sev.append((e0, e1))
        barrier()
        sms = sum(a.elapsed_time(b) for a, b in sev)
        alg2 = interact_bytes(su2, sb2, ntot, fused)
        settled = {"after_steps": int(args.settle_steps), "particle_steps_per_s": ntot * F * 2 / (sms / 1e3),
                   "slots_unbonded": su2, "slots_bonded": sb2, "frames": 2, "frame_steps": F}
        try:
            kt = BatchKernelTimer(batch)
            kt.run(2 * F)
            fig = kt.figures(alg2, peak)
            settled.update({"interact_launch_us": fig["launch_us"], "interact_frac": fig["frac"],
                            "algorithmic_bytes_per_launch": alg2})
        except Exception as exc:
            settled["error"] = str(exc)
        states = [batch.download(k) for k in range(len(items))]

    base = None
    fp64 = None
    if rank == 0 and ws == 1:
        base = cpu_baseline_batch(items, args.cpu_seconds)
        pick = sorted(set(np.linspace(0, len(items) - 1, 8).astype(int).tolist()))
        fp64 = fp64_twin_error([(states[k], items[k][1], items[k][2]) for k in pick], local)
        fp64["sampled_scenes"] = pick
    cfg = dict(desc)
    cfg.update({"frame_steps": F, "horizon": "%d steps per scene from the initial states (%d frames of %d)"
                % (F * args.steps, args.steps, F),
                "frame_ms": {"first": frame_ms[0], "last": frame_ms[-1], "min": min(frame_ms),
                             "max": max(frame_ms)},
                "slots_at_start": {"unbonded": slots_start[0], "bonded": slots_start[1]},
                "slots_at_end": {"unbonded": s_u, "bonded": s_b},
                "parallelism": "replicas" if ws > 1 else "single",
                "l2": "inputs larger than L2 (and a %d MiB write between frames, untimed)" % (FLUSH_BYTES >> 20),
                "graph_steps": g, "knobs": knobs, "autotune": tune_info,
                "plain_path_particle_steps_per_s": plain_value,
                "plain_path_sample": "each scene alone (dem_create per scene), one frame from its end-of-horizon "
                                     "state",
                "batched_over_plain": value / plain_value if plain_value else None,
                "rebuilds": st["reorders"] - rebuilds0, "list_overflows": st["list_overflows"],
                "settled": settled})
    line = {"metric": "particle-steps/s", "value": value, "unit": "particle-steps/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": max_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": cfg, "clocks": clocks, "roofline": roofline,
            "e2e": e2e, "gpu_launches": int(launches), "wall_s": wall}
    if fp64 is not None:
        line["fp64_error"] = fp64
    if base is not None:
        line["cpu_baseline"] = base
    batch.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


class BatchKernelTimer:
    """k_interact launch times of a batch, CUDA events on the batch's stream."""

    def __init__(self, batch):
        import ctypes as C
        import dem
        self.L = dem.lib()
        self.b = batch
        self.C = C
        self.L.dem_batch_kernel_timing.argtypes = [C.c_void_p, C.c_int32]
        self.L.dem_batch_kernel_time.argtypes = [C.c_void_p, C.c_char_p, C.POINTER(C.c_double),
                                                 C.POINTER(C.c_int64)]

    def run(self, steps):
        self.L.dem_batch_kernel_timing(self.b.h, 1)
        self.b.step(steps)
        self.b.synchronize()

    def figures(self, alg_bytes, peak):
        C = self.C
        out = {}
        for k in ("interact", "lom", "broad_phase"):
            ms = C.c_double(0.0)
            n = C.c_int64(0)
            self.L.dem_batch_kernel_time(self.b.h, k.encode(), C.byref(ms), C.byref(n))
            out[k] = (ms.value, n.value)
        self.L.dem_batch_kernel_timing(self.b.h, 0)
        ims, inn = out["interact"]
        avg_s = ims / max(inn, 1) / 1e3
        achieved = alg_bytes / avg_s / 1e9
        return {"achieved": achieved, "frac": achieved / peak, "launch_us": avg_s * 1e6,
                "lom_us": out["lom"][0] / max(out["lom"][1], 1) * 1e3,
                "rebuild_body_us": out["broad_phase"][0] / max(out["broad_phase"][1], 1) * 1e3}


def cpu_baseline_batch(items, seconds):
    """The oracle on a sample of the mix: consecutive scenes advanced 35 steps
    each until about `seconds` of CPU time, all host threads."""
    import oracle
    done_ps = 0
    t0 = time.perf_counter()
    k = 0
    while time.perf_counter() - t0 < seconds and k < len(items):
        sc, p, ext = items[k]
        s = {key: (v.copy() if hasattr(v, "copy") else v) for key, v in sc.items()}
        oracle.step(s, p, 35, **_okw(ext))
        done_ps += int(sc["radii"].shape[0]) * 35
        k += 1
    dt = time.perf_counter() - t0
    return {"value": done_ps / dt, "unit": "particle-steps/s", "cores": os.cpu_count() or 1, "kind": "port",
            "sample": "first %d scenes of the mix, 35 steps each from their initial states (%.1f s)" % (k, dt)}


def run_serve(args):
    """c4: Poisson arrivals of scene requests (sizes log-uniform, horizons
    uniform) served by continuous batching; reports aggregate particle-steps/s
    and completion-latency percentiles (arrival to completion) of every
    request that arrived in the window, with the queue depth over time.
    Scene contents come from a seeded pool of pre-built scenes (the cost of
    building 12k scenes on the host is not part of serving); requests refer
    to the pool's arrays (dem_server_submit_borrowed), so a queued request
    holds no host copy."""
    import torch
    import build_lib
    import dem
    import dem_scenes
    build_lib.build()
    ws, rank, local = dist_env()
    if rank != 0:
        return
    torch.cuda.set_device(local)
    rng = np.random.default_rng(args.seed)
    rate, window = args.serve_rate, args.serve_seconds
    arrivals = np.cumsum(rng.exponential(1.0 / rate, size=int(rate * window * 2) + 16))
    arrivals = arrivals[arrivals < window]
    pool_n = np.exp(rng.uniform(np.log(args.serve_min), np.log(args.serve_max), args.serve_pool)).astype(int)
    pool = [dem_scenes.c3_mix_scene(int(n), float(rng.uniform(0, 0.5)), 7919 * k + args.seed)
            for k, n in enumerate(pool_n)]
    pick = rng.integers(0, len(pool), size=len(arrivals))
    horizons = rng.integers(args.serve_hmin, args.serve_hmax + 1, size=len(arrivals))
    offered = float(sum(int(pool[pick[k]][0]["radii"].shape[0]) * int(horizons[k]) for k in range(len(arrivals))))
    sv = dem.Server(device=local, memory_budget_bytes=int(args.serve_budget_gb * (1 << 30)),
                    max_active_particles=args.serve_active, reorder_interval=35)
    sampler = ClockSampler(local)
    sampler.start()
    sampler.mark()
    t0 = time.perf_counter()
    nxt = 0
    submitted = {}
    done = {}
    finals = []  # (final state, params, ext) of the first completed requests, for the FP64-twin error
    max_queue = max_running = 0
    series = []
    next_sample = 0.0
    chunk = 35
    limit = t0 + args.serve_timeout
    while len(done) < len(arrivals) and time.perf_counter() < limit:
        now = time.perf_counter() - t0
        while nxt < len(arrivals) and arrivals[nxt] <= now:
            sc, p, ext = pool[pick[nxt]]
            rid = sv.submit(sc, p, int(horizons[nxt]), borrow=True, **ext)
            submitted[rid] = (nxt, int(sc["radii"].shape[0]) * int(horizons[nxt]))
            nxt += 1
        sv.advance(chunk)
        st = sv.stats()
        max_queue = max(max_queue, st["queued"])
        max_running = max(max_running, st["running"])
        tp = time.perf_counter() - t0
        if tp >= next_sample:
            series.append([round(tp, 2), int(st["queued"]), int(st["running"]), int(st["active_particles"])])
            next_sample = tp + 1.0
        for rid in sv.poll():
            k, work = submitted[rid]
            if len(finals) < 4:
                out, _, _ = sv.fetch(rid)
                finals.append((out, pool[pick[k]][1], pool[pick[k]][2]))
            else:
                sv.finish(rid)
            done[rid] = (k, tp - arrivals[k], work)
        if st["running"] == 0 and st["queued"] == 0 and nxt < len(arrivals):
            time.sleep(max(0.0, arrivals[nxt] - (time.perf_counter() - t0)))
    elapsed = time.perf_counter() - t0
    sampler.mark()
    sampler.stop()
    st = sv.stats()
    sv.close()
    fp64 = fp64_twin_error(finals, local) if finals else None
    if fp64 is not None:
        fp64["state"] = "the final states of the first %d completed requests" % len(finals)
    lat = np.array([v[1] for v in done.values()]) if done else np.zeros(1)
    in_window = [v[1] for v in done.values() if arrivals[v[0]] < window]
    value = st["particle_steps"] / elapsed
    step_every = max(1, len(series) // 60)
    line = {"metric": "particle-steps/s", "value": value, "unit": "particle-steps/s", "n_gpus": 1,
            "steps": int(st["steps"]), "warmup": 0, "ms_per_step": elapsed / max(st["steps"], 1) * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": "c4 served stream", "arrival_rate_per_s": rate, "arrival_window_s": window,
                       "requests": int(len(arrivals)), "completed": int(len(done)),
                       "offered_particle_steps": offered,
                       "offered_particle_steps_per_s_over_window": offered / window,
                       "particles_per_request": "log-uniform [%d, %d] (pool of %d seeded scenes)"
                       % (args.serve_min, args.serve_max, args.serve_pool),
                       "horizon_steps": "uniform [%d, %d]" % (args.serve_hmin, args.serve_hmax),
                       "memory_budget_gb": args.serve_budget_gb, "max_active_particles": args.serve_active,
                       "capacity_particles": st["capacity_particles"], "device_bytes": st["device_bytes"],
                       "admission_waits": {"on_max_active_particles": int(st["waits_active"]),
                                           "on_device_ranges": int(st["waits_memory"])},
                       "max_queue": int(max_queue), "max_running": int(max_running),
                       "queue_depth_series": {"columns": ["t_s", "queued", "running", "active_particles"],
                                              "rows": series[::step_every]},
                       "advance_chunk_steps": chunk, "elapsed_s": elapsed,
                       "drained": bool(len(done) == len(arrivals))},
            "latency_s": {"p50": float(np.percentile(lat, 50)), "p95": float(np.percentile(lat, 95)),
                          "p99": float(np.percentile(lat, 99)), "max": float(lat.max()),
                          "of": "arrival to completion, every completed request (%d)" % len(in_window)},
            "clocks": sampler.summary()}
    if fp64 is not None:
        line["fp64_error"] = fp64
    print(json.dumps(line), flush=True)


def run_profile_target(args):
    """K steps of the workload with plain launches and the given knobs (the
    target of an ncu capture); prints the stats and exits."""
    import build_lib
    import dem
    build_lib.build()
    knobs = {"split_narrow": int(args.split), "unfused_lom": int(args.unfused),
             "search_cell_factor": args.cell_factor, "list_skin": args.skin, "block_size": args.block,
             "reorder_interval": args.graph_steps, "plain_launches": True, "reorder_every": args.reorder_every}
    if args.workload == "c3_batch":
        items, _ = build_batch_workload(args.scenes, args.seed)
        with dem.Batch(items, **knobs) as b:
            b.step(args.profile_steps)
            b.synchronize()
            print("ok", len(items), "scenes", args.profile_steps, "steps", b.stats(), flush=True)
        return
    sc, p, ext, desc = build_workload(args.workload, args)
    with dem.Context(sc, p, **knobs, **ext) as ctx:
        ctx.step(args.profile_steps)
        ctx.synchronize()
        print("ok", desc["workload"], desc["particles"], "particles", args.profile_steps, "steps", ctx.stats(),
              flush=True)


def main():
    args = parse_args()
    if args.profile_steps > 0:
        run_profile_target(args)
        return
    if args.workload == "c4_serve":
        run_serve(args)
        return
    batch = args.workload == "c3_batch"
    args.frame_given = args.frame > 0
    if args.frame <= 0:
        args.frame = 35 if batch else 105
    if args.steps <= 0:
        args.steps = 20 if batch else 200
    if args.impl == "reference":
        if batch:
            run_reference_batch(args)
        else:
            run_reference(args)
    else:
        if batch:
            run_ours_batch(args)
        else:
            run_ours(args)


if __name__ == "__main__":
    main()
