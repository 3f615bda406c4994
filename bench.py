"""Benchmark of the GB300 PCA sweep-and-prune broadphase.

Workload (one "step" = one broadphase call): 1,048,576 fp32 AABBs whose
centres follow an anisotropic Gaussian with std (100, 20, 5) along a seeded
random rotation, half-extents exp(N(-1, 0.5^2)) clipped to [0.05, 2]; 64
jittered copies of the centres (N(0, 0.05^2) per axis) are made up front and
the timed calls cycle through them (64 x 32 MiB of distinct inputs, larger
than L2).  Every call returns the sorted (i < j) uint32 pair list, as the
reference's Sap::collision canonicalises its output.  Synthetic data, seeded.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line (rank 0): the device-timed throughput (value), the
same metric end to end through the public API with host copies (e2e), the
dominant kernel against the measured HBM peak (roofline, with the L1 and
DRAM throughput of its committed ncu summary), the whole call against
156 n + 8 P bytes, per-stage times, the restated reference on the host
cores (cpu_baseline), kernel launches, sampled clocks, and extras (the
16,384-box case against the O(n^2) brute force, a 16,777,216-box scene,
4096 batched scenes, the rigid-body step).  --impl reference times the
reference algorithm restated on the CPU (oracle/, the checker) on all host
cores: each step one call whose sweeps start from one slice of each sorted
group, slices in turn, reported as the full-call time they add up to.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_OBJ = 1 << 20
N_JITTER = 64
FALLBACK_HBM_GBS = 6800.0


def algorithmic_bytes(n: int, P: int) -> dict:
    """Algorithmic HBM bytes of one broadphase call, per stage:
    PCA reads 24n; projection reads 24n and writes key + id 8n; the sort
    (4 passes, histograms fused) reads 4n plus 16n per pass; the sweep reads
    8n keys/ids and 24n bounds and writes 8P.  Total 156 n + 8 P."""
    return {"pca": 24 * n, "project": 32 * n, "sort": (4 + 16 * 4) * n, "sweep": 32 * n + 8 * P,
            "canonical": 0, "total": 156 * n + 8 * P}


def rb_algorithmic_bytes(nb: int, np_: int, Pc: int, Pb: int) -> int:
    """Rigid-body step: 276 n_b + 96 n_p + 8 P_c + B_bp(n_b, P_b)."""
    return 276 * nb + 96 * np_ + 8 * Pc + algorithmic_bytes(nb, Pb)["total"]


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(path))
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def traffic_table():
    """dram bytes per launch from committed ncu summaries (profiles/ncu_traffic.txt)."""
    out = {}
    path = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    if os.path.exists(path):
        for line in open(path):
            line = line.strip()
            if not line or line.startswith("#"):
                continue
            parts = line.split()
            if len(parts) >= 3:
                out[(parts[0], parts[1])] = float(parts[2])
    return out


def profile_metric(kernel: str, name: str):
    """A percentage from a committed ncu summary (profiles/<kernel>_gauss1m.md
    table row `| name | value % |`), as a fraction, or None."""
    path = os.path.join(ROOT, "profiles", f"{kernel}_gauss1m.md")
    if not os.path.exists(path):
        return None
    for line in open(path):
        cells = [c.strip() for c in line.strip().strip("|").split("|")]
        if len(cells) == 2 and cells[0] == name and cells[1].endswith("%"):
            return round(float(cells[1].rstrip("%").strip()) / 100.0, 4)
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
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

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            p = [x.strip() for x in l.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for k, name in enumerate(names):
                if p[5 + k].lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def workload_config(args, world: int) -> dict:
    """The `config` of the JSON line, the same for both arms."""
    return {"workload": "gauss1m: 1,048,576 AABBs, anisotropic Gaussian std (100,20,5) under a seeded "
                        "rotation, log-normal half-extents, 64 jittered copies cycled",
            "n": args.n, "l2": f"inputs cycled over {args.jitter_sets} x {2 * args.n * 16 >> 20} MiB",
            "output": "sorted (i<j) uint32 pairs", "parallelism": f"replicas x{world}"}


def make_inputs(rank: int, n: int, sets_wanted: int = N_JITTER):
    """n objects; for n != 1,048,576 the spread is scaled by (n / 2^20)^(1/3)
    so the object density (and so the work per object) stays that of the
    1M workload."""
    from gsap_gb300 import scenes
    f = (n / N_OBJ) ** (1.0 / 3.0)
    c, h, R = scenes.aabb_gauss_parts(n, seed=rank, std=(100.0 * f, 20.0 * f, 5.0 * f))
    sets = []
    for k in range(sets_wanted):
        cj = scenes.jitter(c, seed=1000 * (rank + 1) + k) if k else c
        mn = np.empty((n, 4), np.float32)
        mx = np.empty((n, 4), np.float32)
        mn[:, :3] = cj - h
        mx[:, :3] = cj + h
        mn[:, 3] = 0.0
        mx[:, 3] = 0.0
        sets.append((mn, mx))
    return sets, R


# ----------------------------------------------------------------- our arm

def run_ours(args, world, rank, local):
    import torch
    import torch.distributed as dist

    import gsap_gb300
    from gsap_gb300 import Sap, _lib

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    gsap_gb300.load()
    n = args.n
    host_sets, R = make_inputs(rank, n, args.jitter_sets)
    dsets = [(torch.from_numpy(mn).to(dev), torch.from_numpy(mx).to(dev)) for mn, mx in host_sets]
    fixed = (args.cell_factor is not None or args.sort_bits is not None or args.sort is not None
             or args.sort_tile is not None or args.no_tune)
    sort_mode = {"radix": 0, "bucket": 1}[args.sort or "radix"]
    sap = Sap(n, cell_factor=args.cell_factor or 2.0, sort_bits=args.sort_bits or 32, sort_mode=sort_mode,
              sort_tile=args.sort_tile or 4096)
    cap = 16 * n
    pairs = torch.empty((cap, 2), dtype=torch.int32, device=dev)
    d_count = torch.zeros(1, dtype=torch.int64, device=dev)
    stream = torch.cuda.current_stream()
    # autotuner (set-up, untimed): sort (and radix tile), key width and cell factor for this input
    tuned = None if fixed else sap.autotune(*dsets[0], pairs=pairs, sorted=True, graph=True, reps=10, stream=stream)
    passes = (tuned["sort_bits"] if tuned else (args.sort_bits or 32)) // 8
    if tuned:
        sort_mode = 0 if tuned["sort"] == "radix" else 1

    def call(k, sorted_=True, graph=True):
        mn, mx = dsets[k % len(dsets)]
        sap.broadphase_async(mn, mx, pairs, d_count, sorted=sorted_, graph=graph, stream=stream)

    # warm-up (also captures the per-input graphs)
    for k in range(args.warmup):
        call(k)
    for k in range(min(len(dsets), args.steps)):
        call(k)
    torch.cuda.synchronize()
    sap.check()
    P0 = int(d_count.item())
    stats = sap.stats()

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with ClockSampler(local) as clk:
        barrier()
        t0 = time.perf_counter()
        for k in range(args.steps):
            ev[k][0].record(stream)
            call(k)
            ev[k][1].record(stream)
        barrier()
        wall = time.perf_counter() - t0
    sap.check()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    ms = float(np.mean(step_ms))
    total_ms = float(np.sum(step_ms))
    if world > 1:
        t = torch.tensor([total_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    value = world * n * args.steps / (total_ms / 1e3) / 1e6  # Mobjects/s, whole job

    # per-stage breakdown (events on the launching stream, no graph)
    sap.enable_timing(True)
    stages = []
    for k in range(8):
        sap.broadphase(*dsets[k % len(dsets)], pairs=pairs, sorted=True, stream=stream)
        stages.append(sap.stage_times())
    sap.enable_timing(False)
    names = ["pca", "project", "sort", "sweep", "canonical"]
    st_ms = {nm: float(np.mean([s[i] for s in stages])) for i, nm in enumerate(names)}
    alg = algorithmic_bytes(n, P0)
    peak, peak_kind = peaks()
    dom = max(("pca", "project", "sort", "sweep"), key=lambda s: st_ms[s])
    achieved = alg[dom] / (st_ms[dom] / 1e3) / 1e9
    traffic = traffic_table().get((f"stage_{dom}", "gauss1m"))
    pipe_gbs = alg["total"] / (ms / 1e3) / 1e9

    # temporal mode (GSAP_FLAG_TEMPORAL): each call sweeps with the previous
    # call's grid while its own PCA runs beside it; same inputs, same pairs
    for k in range(min(len(dsets), args.steps) + 2):
        sap.broadphase_async(*dsets[k % len(dsets)], pairs, d_count, sorted=True, graph=True, temporal=True,
                             stream=stream)
    torch.cuda.synchronize()
    sap.check()
    assert int(d_count.item()) > 0
    et0, et1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    et0.record(stream)
    for k in range(args.steps):
        sap.broadphase_async(*dsets[k % len(dsets)], pairs, d_count, sorted=True, graph=True, temporal=True,
                             stream=stream)
    et1.record(stream)
    torch.cuda.synchronize()
    sap.check()
    temporal_ms = et0.elapsed_time(et1) / args.steps

    # unsorted pair set (no canonicalisation), for reference
    for k in range(16):
        call(k, sorted_=False)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for k in range(16):
        call(k, sorted_=False)
    e1.record(stream)
    torch.cuda.synchronize()
    unsorted_ms = e0.elapsed_time(e1) / 16

    # Graph mode with new buffers on every call: windows of larger buffers at
    # a new offset each call (same shape, new pointers).  Once the handle
    # holds 64 graphs of this shape, each call re-captures its launches and
    # updates a cached graph in place (cudaGraphExecUpdate).
    KF = 100
    big_mn = torch.empty((n + 2 * KF + 160, 4), dtype=torch.float32, device=dev)
    big_mx = torch.empty_like(big_mn)
    big_mn[:n] = dsets[0][0]
    big_mn[n:] = dsets[0][0][: big_mn.shape[0] - n]
    big_mx[:n] = dsets[0][1]
    big_mx[n:] = dsets[0][1][: big_mx.shape[0] - n]
    big_pairs = torch.empty((cap + 2 * KF + 160, 2), dtype=torch.int32, device=dev)

    def fresh(k):
        sap.broadphase_async(big_mn[k:k + n], big_mx[k:k + n], big_pairs[k:k + cap], d_count, sorted=True,
                             graph=True, stream=stream)

    for k in range(80):  # fills the per-shape quota (instantiations), then updates
        fresh(k)
    torch.cuda.synchronize()
    sap.check()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    h0 = time.perf_counter()
    for k in range(80, 80 + KF):
        fresh(k)
    host_s = time.perf_counter() - h0
    f1.record(stream)
    torch.cuda.synchronize()
    sap.check()
    fresh_ms = f0.elapsed_time(f1) / KF
    del big_mn, big_mx, big_pairs

    # End to end through the public API with host buffers, as a streaming
    # user runs it: every call copies its inputs from pinned host memory and
    # reads back its pair count and pair list.  Two slots: the copies of one
    # call overlap the compute of the next (copy streams + events); the host
    # reads call k's count only once call k has finished.
    pin = [(torch.from_numpy(mn).pin_memory(), torch.from_numpy(mx).pin_memory()) for mn, mx in host_sets[:4]]
    slots = []
    for _ in range(2):
        slots.append({"mn": torch.empty_like(dsets[0][0]), "mx": torch.empty_like(dsets[0][1]),
                      "pairs": torch.empty((cap, 2), dtype=torch.int32, device=dev),
                      "cnt": torch.zeros(1, dtype=torch.int64, device=dev),
                      "hcnt": torch.zeros(1, dtype=torch.int64).pin_memory(),
                      "hpairs": torch.empty((cap, 2), dtype=torch.int32).pin_memory()})
    s_in, s_out = torch.cuda.Stream(), torch.cuda.Stream()
    h2d = 2 * n * 16
    d2h = []
    K_e2e = max(8, min(args.steps, 64))

    def e2e_run(K):
        ev_in = [torch.cuda.Event() for _ in range(K)]
        ev_done = [torch.cuda.Event() for _ in range(K)]
        ev_out = [torch.cuda.Event() for _ in range(K)]
        sizes = []

        def drain(j):
            sl = slots[j % 2]
            ev_done[j].synchronize()  # call j finished: its count is on the host
            c = int(sl["hcnt"].item())
            with torch.cuda.stream(s_out):
                s_out.wait_event(ev_done[j])
                sl["hpairs"][:c].copy_(sl["pairs"][:c], non_blocking=True)
                ev_out[j].record(s_out)
            sizes.append(8 + 8 * c)

        for k in range(K):
            sl = slots[k % 2]
            pm, px = pin[k % len(pin)]
            with torch.cuda.stream(s_in):
                if k >= 2:
                    s_in.wait_event(ev_done[k - 2])  # slot inputs free
                sl["mn"].copy_(pm, non_blocking=True)
                sl["mx"].copy_(px, non_blocking=True)
                ev_in[k].record(s_in)
            stream.wait_event(ev_in[k])
            if k >= 2:
                stream.wait_event(ev_out[k - 2])  # slot pair buffer drained
            sap.broadphase_async(sl["mn"], sl["mx"], sl["pairs"], sl["cnt"], sorted=True, graph=True, stream=stream)
            sl["hcnt"].copy_(sl["cnt"], non_blocking=True)
            ev_done[k].record(stream)
            if k >= 1:
                drain(k - 1)
        drain(K - 1)
        torch.cuda.synchronize()
        return sizes

    e2e_run(4)  # warm-up: graphs for both slots
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    d2h = e2e_run(K_e2e)
    e2e_s = (time.perf_counter() - t0) / K_e2e
    e2e_val = world * n / e2e_s / 1e6

    # CPU baseline: the reference algorithm restated (oracle port), full calls
    cpu = None
    if rank == 0 and not args.no_cpu:
        import oracle
        mn, mx = host_sets[0]
        oracle.build()
        cap = len(oracle.sap_ref(0, mn, mx))  # untimed: sizes the output so each timed call runs once
        t0 = time.perf_counter()
        reps = 2
        for _ in range(reps):
            oracle.sap_ref(0, mn, mx, cap=cap)
        t = (time.perf_counter() - t0) / reps
        cores = os.cpu_count()
        cpu = {"value": round(n / t / 1e6, 4), "unit": "Mobjects/s", "cores": cores, "kind": "port",
               "sample": f"{reps} full calls of the {n}-AABB scene after one untimed: max-variance axis, "
                         f"quadrant sweeps, cross pass, sort+unique (oracle/bp.c orc_sap_ref, OpenMP over {cores} threads)"}

    extras = {}
    if not args.no_extras:
        extras = run_extras(args, dev, stream)

    # pca + finish, project, the sort (bucket: count sums, offsets, scatter,
    # local sort; radix: one per pass), sweep, row sums + row scan, scatter,
    # rank, long rows
    launches_per_call = 9 + (4 if sort_mode == 1 else passes)
    clocks = clk.summary()
    line = {
        "metric": "1M-AABB PCA sweep-and-prune broadphase throughput (sorted i<j pair set)",
        "value": round(value, 3), "unit": "Mobjects/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": workload_config(args, world),
        "pairs_per_call": P0,
        "settings": dict(tuned, autotuned=True) if tuned else
        {"sort_bits": args.sort_bits or 32, "cell_factor": args.cell_factor or 2.0, "sort": args.sort or "radix",
         "sort_tile": args.sort_tile or 4096, "autotuned": False},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": traffic, "kernel": f"stage:{dom}",
                     "peak_kind": peak_kind,
                     "traffic_source": "from the committed ncu capture of this kernel on this workload "
                                       "(profiles/ncu_traffic.txt), not measured in this run",
                     # what limits it instead: the L1 data path (one ncu --set full capture)
                     "limiter": {"l1tex_throughput_frac": profile_metric(f"k_{dom}", "L1/TEX Cache Throughput"),
                                 "dram_throughput_frac": profile_metric(f"k_{dom}", "DRAM Throughput"),
                                 "source": f"profiles/k_{dom}_gauss1m.md (from the committed capture, "
                                           "not measured in this run)"}},
        "pipeline_roofline": {"bytes_alg": alg["total"], "achieved_gbs": round(pipe_gbs, 1),
                              "frac": round(pipe_gbs / peak, 4), "formula": "156 n + 8 P"},
        "stage_ms": {k: round(v, 4) for k, v in st_ms.items()},
        "sweep_stats": {"entries": stats["entries"], "tests": stats["tests"], "buckets": stats["buckets"],
                        "qbits": stats["qbits"], "warp_iters": stats["iters"],
                        "lane_efficiency": round(stats["tests"] / max(1, 32 * stats["iters"]), 3),
                        "tests_per_pair": round(stats["tests"] / max(1, P0), 2)},
        "unsorted_ms_per_step": round(unsorted_ms, 4),
        "new_buffers_every_call": {"ms_per_step": round(fresh_ms, 4), "host_ms_per_call": round(host_s / KF * 1e3, 4),
                                   "calls": KF, "cached_ms_per_step": round(ms, 4),
                                   "mode": "graph mode, new input and output pointers each call: the launches "
                                           "are captured again and a cached graph of the shape is updated in "
                                           "place (cudaGraphExecUpdate)"},
        "temporal": {"ms_per_step": round(temporal_ms, 4), "value": round(n / (temporal_ms / 1e3) / 1e6, 3),
                     "unit": "Mobjects/s",
                     "mode": "GSAP_FLAG_TEMPORAL: grid of the previous call, this call's PCA beside the sweep"},
        "e2e": {"value": round(e2e_val, 3), "unit": "Mobjects/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": int(np.mean(d2h)), "calls": K_e2e,
                "mode": "pinned H2D of inputs + D2H of count and pairs every call; copies of one call overlap "
                        "the compute of the next (two slots)"},
        "cpu_baseline": cpu,
        "gpu_launches": launches_per_call * args.steps,
        "clocks": clocks,
        "wall_s_timed": round(wall, 4),
    }
    if extras:
        line["extras"] = extras
    return line


def fixed_settings(args):
    """Sap settings from the command line (--no-tune): key width, cell
    factor, sort and radix tile, with the untuned defaults."""
    kw = dict(sort_bits=args.sort_bits or 32, cell_factor=args.cell_factor or 2.0,
              sort_mode={"radix": 0, "bucket": 1}[args.sort or "radix"], sort_tile=args.sort_tile or 4096)
    desc = {"sort_bits": kw["sort_bits"], "cell_factor": kw["cell_factor"], "sort": args.sort or "radix",
            "sort_tile": kw["sort_tile"], "autotuned": False}
    return kw, desc


def _extra_small(args, dev, stream, out):
    import torch

    from gsap_gb300 import CONTACT_CONFIG, ParticleRigidBody, Sap, scenes
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    peak, _ = peaks()
    dt = 1.0 / 600.0
    cfgp = dict(k=2e4, eta=50.0, kt=0.1, gravity_y=-9.81, box_lo=(0.0, 0.0, 0.0), box_hi=(200.0, 200.0, 200.0))
    gstream = torch.cuda.Stream()
    # --- small case: 16,384 AABBs, centres U[0,100]^3, half-extents U[0.1,0.5];
    # the reference's own CPU path for it is the O(n^2) brute force
    smn, smx = scenes.aabb_uniform(16384, 0)
    dsmn, dsmx = torch.from_numpy(smn).to(dev), torch.from_numpy(smx).to(dev)
    skw, sdesc = fixed_settings(args)
    ssap = Sap(16384, **skw) if args.no_tune else Sap(16384)
    spairs = torch.empty((16 * 16384, 2), dtype=torch.int32, device=dev)
    scnt = torch.zeros(1, dtype=torch.int64, device=dev)
    # autotuner (set-up, untimed), as for the 1M workload
    stuned = None if args.no_tune else ssap.autotune(dsmn, dsmx, pairs=spairs, sorted=True, graph=True, reps=20,
                                                     stream=stream)
    for _ in range(5):
        ssap.broadphase_async(dsmn, dsmx, spairs, scnt, sorted=True, graph=True, stream=stream)
    torch.cuda.synchronize()
    ssap.check()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(200):
        ssap.broadphase_async(dsmn, dsmx, spairs, scnt, sorted=True, graph=True, stream=stream)
    e1.record(stream)
    torch.cuda.synchronize()
    ssap.check()
    small = {"n": 16384, "pairs": int(scnt.item()), "ms_per_call": round(e0.elapsed_time(e1) / 200, 4),
             "settings": dict(stuned, autotuned=True) if stuned else sdesc}
    if not args.no_cpu:
        import oracle
        oracle.build()
        t0 = time.perf_counter()
        bf = oracle.bf_aabb(smn, smx)
        small["cpu_brute_force_ms"] = round((time.perf_counter() - t0) * 1e3, 2)
        small["cpu_cores"] = os.cpu_count()
        small["equal_to_brute_force"] = bool(np.array_equal(spairs[: len(bf)].cpu().numpy().astype(np.uint32), bf)
                                             and int(scnt.item()) == len(bf))
    out["small_16k"] = small
    del ssap, spairs


def _extra_demo(args, dev, stream, out):
    import torch

    from gsap_gb300 import CONTACT_CONFIG, ParticleRigidBody, Sap, scenes
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    peak, _ = peaks()
    dt = 1.0 / 600.0
    cfgp = dict(k=2e4, eta=50.0, kt=0.1, gravity_y=-9.81, box_lo=(0.0, 0.0, 0.0), box_hi=(200.0, 200.0, 200.0))
    gstream = torch.cuda.Stream()
    # --- the reference's own call: Sap::collision on the particles of the
    # headless demo scene (4096 hexagon bodies x 6 particles = 24,576 spheres,
    # demoParticles.h:403, :898-903), both-direction list + pairEntries
    from gsap_gb300 import demo
    # the scene after 300 demo steps (the bodies have fallen and pile up, so
    # the particles touch as in the demo's later frames)
    dsc = demo.demo_scene(4096, n_row=16, seed=0)
    dd = demo.Demo(dsc)
    dd.run(300, stream=stream)
    torch.cuda.synchronize()
    dd.sap.check()
    dprb = dd.system
    dsph = torch.from_numpy(dprb.get_particles()["p_pos"]).to(dev)
    nsp = dsph.shape[0]
    ckw, cdesc = fixed_settings(args)
    csap = Sap(nsp, mode=1, **ckw) if args.no_tune else Sap(nsp, mode=1)
    cpairs = torch.empty((40 * nsp, 2), dtype=torch.int32, device=dev)
    cent = torch.empty(nsp + 1, dtype=torch.int32, device=dev)
    # autotuner (set-up, untimed) on the same spheres; the collision calls use its settings
    ctuned = None if args.no_tune else csap.autotune(dsph, None, pairs=cpairs, sorted=True, graph=True, reps=20,
                                                     stream=stream)
    for _ in range(5):
        npc, nec = csap.collision(0.0, dsph, cpairs, cent, stream=stream)
    h0 = time.perf_counter()
    e0.record(stream)
    for _ in range(100):
        npc, nec = csap.collision(0.0, dsph, cpairs, cent, stream=stream)
    e1.record(stream)
    torch.cuda.synchronize()
    coll = {"spheres": nsp, "pairs_both_directions": npc, "pair_entries": nec,
            "ms_per_call": round((time.perf_counter() - h0) * 10, 4),
            "device_ms_per_call": round(e0.elapsed_time(e1) / 100, 4),
            "note": "gsap_sap_collision blocks for the host counts each call, as Sap::collision does",
            "settings": dict(ctuned, autotuned=True) if ctuned else cdesc}
    if not args.no_cpu:
        import oracle
        sp = dsph.cpu().numpy()
        wp, we = oracle.both_directions(oracle.bf_sphere(sp))
        coll["equal_to_brute_force"] = bool(npc == len(wp) and nec == len(we) and
                                            np.array_equal(cpairs[:npc].cpu().numpy(), wp) and
                                            np.array_equal(cent[:nec].cpu().numpy(), we))
    out["demo_collision_24k"] = coll
    del dprb, dd, csap, cpairs, cent


def _extra_large(args, dev, stream, out):
    import torch

    from gsap_gb300 import CONTACT_CONFIG, ParticleRigidBody, Sap, scenes
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    peak, _ = peaks()
    dt = 1.0 / 600.0
    cfgp = dict(k=2e4, eta=50.0, kt=0.1, gravity_y=-9.81, box_lo=(0.0, 0.0, 0.0), box_hi=(200.0, 200.0, 200.0))
    gstream = torch.cuda.Stream()
    # --- large case: 16,777,216 AABBs at the 1M workload's object density
    # (spread scaled by 16^(1/3)); one input set of 512 MiB, larger than L2
    nl = 1 << 24
    (lmn, lmx), = make_inputs(0, nl, 1)[0]
    dlmn, dlmx = torch.from_numpy(lmn).to(dev), torch.from_numpy(lmx).to(dev)
    del lmn, lmx
    lsap = Sap(nl, sort_bits=args.sort_bits or 32, cell_factor=args.cell_factor or 2.0)
    lcfg = (dict(sort_bits=args.sort_bits or 32, cell_factor=args.cell_factor or 2.0, autotuned=False)
            if args.no_tune else lsap.autotune(dlmn, dlmx, reps=5))
    lpairs = torch.empty((8 * nl, 2), dtype=torch.int32, device=dev)
    lcnt = torch.zeros(1, dtype=torch.int64, device=dev)
    for _ in range(3):
        lsap.broadphase_async(dlmn, dlmx, lpairs, lcnt, sorted=True, graph=True, stream=stream)
    torch.cuda.synchronize()
    lsap.check()
    e0.record(stream)
    for _ in range(10):
        lsap.broadphase_async(dlmn, dlmx, lpairs, lcnt, sorted=True, graph=True, stream=stream)
    e1.record(stream)
    torch.cuda.synchronize()
    lsap.check()
    l_ms = e0.elapsed_time(e1) / 10
    out["large_16m"] = {"n": nl, "pairs": int(lcnt.item()), "ms_per_call": round(l_ms, 4),
                        "mobjects_per_s": round(nl / (l_ms / 1e3) / 1e6, 1), "settings": lcfg,
                        "sample": "one seeded 16,777,216-AABB scene, 10 graph calls after the autotuner"}
    lsap.close()
    del lsap, lpairs, dlmn, dlmx


def _extra_batched(args, dev, stream, out):
    import torch

    from gsap_gb300 import CONTACT_CONFIG, ParticleRigidBody, Sap, scenes
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    peak, _ = peaks()
    dt = 1.0 / 600.0
    cfgp = dict(k=2e4, eta=50.0, kt=0.1, gravity_y=-9.81, box_lo=(0.0, 0.0, 0.0), box_hi=(200.0, 200.0, 200.0))
    gstream = torch.cuda.Stream()
    # --- batched broadphase: 4096 scenes, sizes log-uniform in [64, 65536]
    S = args.scenes
    mn, mx, off = scenes.batched_aabb(S=S, seed=7)
    n = len(mn)
    dmn, dmx = torch.from_numpy(mn).to(dev), torch.from_numpy(mx).to(dev)
    doff = torch.from_numpy(off.astype(np.int32)).to(dev)
    bsap = Sap(n, max_scenes=S, pair_factor=2, sort_tile=args.sort_tile or 0)
    cap = 2 * n
    pairs = torch.empty((cap, 2), dtype=torch.int32, device=dev)
    cnt = torch.zeros(1, dtype=torch.int64, device=dev)
    import ctypes as C

    from gsap_gb300 import _lib
    L = _lib.load()
    btuned = (dict(sort_bits=32, cell_factor=2.0, sort="radix", sort_tile=args.sort_tile or 4096, autotuned=False)
              if args.no_tune else
              dict(bsap.autotune(dmn, dmx, offsets=doff, pairs=pairs, sorted=True, graph=True, reps=3, stream=stream),
                   autotuned=True))

    def batched_call():
        st = L.gsap_broadphase_batched(bsap.handle, dmn.data_ptr(), dmx.data_ptr(), doff.data_ptr(), S, n,
                                       pairs.data_ptr(), cap, C.c_void_p(cnt.data_ptr()), None, 1 | 2,
                                       C.c_void_p(stream.cuda_stream))
        _lib.check(st)

    for _ in range(3):
        batched_call()
    torch.cuda.synchronize()
    bsap.check()
    Pb = int(cnt.item())
    equal = None
    if not args.no_cpu:
        import oracle
        want = oracle.pairs_batched(mn, mx, off, bf_max=8192)
        got = pairs[:Pb].cpu().numpy().astype(np.uint32)
        equal = bool(len(got) == len(want) and np.array_equal(got, want))
    reps = 5
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        batched_call()
    e1.record(stream)
    torch.cuda.synchronize()
    batched_ms = e0.elapsed_time(e1) / reps
    # plain pipeline: one scene per call sequence, same flags, same GPU
    psap = Sap(int((off[1:] - off[:-1]).max()))
    views = [(dmn[off[s]:off[s + 1]], dmx[off[s]:off[s + 1]]) for s in range(S)]
    pc = torch.zeros(1, dtype=torch.int64, device=dev)

    def plain_pass():
        for a, b in views:
            psap.broadphase_async(a, b, pairs, pc, sorted=True, graph=False, stream=stream)

    plain_pass()
    torch.cuda.synchronize()
    e0.record(stream)
    plain_pass()
    e1.record(stream)
    torch.cuda.synchronize()
    plain_ms = e0.elapsed_time(e1)
    peak, _ = peaks()
    bbytes = sum(algorithmic_bytes(int(off[s + 1] - off[s]), 0)["total"] for s in range(S)) + 8 * Pb
    out["batched"] = {"scenes": S, "objects": n, "pairs": Pb, "ms_per_batch": round(batched_ms, 3),
                      "scenes_per_s": round(S / (batched_ms / 1e3), 1),
                      "plain_ms_per_pass": round(plain_ms, 3),
                      "plain_scenes_per_s": round(S / (plain_ms / 1e3), 1),
                      "speedup_vs_plain": round(plain_ms / batched_ms, 2),
                      "achieved_gbs": round(bbytes / (batched_ms / 1e3) / 1e9, 1),
                      "frac": round(bbytes / (batched_ms / 1e3) / 1e9 / peak, 4),
                      "settings": btuned,
                      "equal_to_reference": equal,
                      "reference": "oracle per scene: O(n^2) Aabb::overlaps for scenes <= 8192 objects, the same "
                                   "predicate on x-overlapping pairs above (untimed check of the timed output)"}
    del bsap, psap, pairs, dmn, dmx
    torch.cuda.empty_cache()


def _extra_rigid(args, dev, stream, out):
    import torch

    from gsap_gb300 import CONTACT_CONFIG, ParticleRigidBody, Sap, scenes
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    peak, _ = peaks()
    dt = 1.0 / 600.0
    cfgp = dict(k=2e4, eta=50.0, kt=0.1, gravity_y=-9.81, box_lo=(0.0, 0.0, 0.0), box_hi=(200.0, 200.0, 200.0))
    gstream = torch.cuda.Stream()
    # --- rigid body: 65,536 cubes of 2x2x2 particles in a 200^3 box, 1000 steps
    dt = 1.0 / 600.0
    nb = args.bodies
    sc = scenes.cubes_in_box(nb, box=200.0, seed=3)
    cfgp = dict(k=2e4, eta=50.0, kt=0.1, gravity_y=-9.81, box_lo=(0.0, 0.0, 0.0), box_hi=(200.0, 200.0, 200.0))
    prb = ParticleRigidBody(nb, sc["n_particles"], 16)
    prb.load_scene(sc)
    prb.set_contact(model=CONTACT_CONFIG, **cfgp)
    init = {k: np.ascontiguousarray(sc[k], np.float32) for k in ("pos", "quat", "lin_vel", "ang_vel")}
    rkw, rdesc = fixed_settings(args)
    rkw["sort_bits"] = rdesc["sort_bits"] = args.sort_bits or 24
    rsap = Sap(nb, **rkw)
    # autotuner (set-up, untimed) on the body AABBs of the initial pose
    rtuned = None
    if not args.no_tune:
        bmn, bmx = scenes.body_aabbs(sc)
        rtuned = rsap.autotune(torch.from_numpy(bmn).to(dev), torch.from_numpy(bmx).to(dev), reps=20, stream=stream)
    rb = {"bodies": nb, "particles": sc["n_particles"],
          "broadphase_settings": dict(rtuned, autotuned=True) if rtuned else rdesc}
    if not args.no_cpu:
        import oracle
        from oracle.trajectory import fp64_errors
        st64 = scenes.to_f64(sc)
        t0 = time.perf_counter()
        oracle.rb_step_cfg_f64(st64, dict(cfgp, dt=dt))
        cpu_rb_s = time.perf_counter() - t0
        t0 = time.perf_counter()
        e = fp64_errors(prb, rsap, sc, dict(cfgp, dt=dt), steps=args.rb_check_steps, stream=stream)
        rb["fp64_error"] = {"steps": e["steps"], "per_step_max": e["per_step_max"],
                            "per_step_max_all_bodies": e["per_step_max_all_bodies"],
                            "bodies_left_out_max": e["bodies_left_out_max"], "worst": e["worst"],
                            "free_running": e["free_running"], "check_s": round(time.perf_counter() - t0, 1),
                            "definition": "max |gpu - fp64| / max |fp64| over xyz; per step: each GPU step "
                                          "taken from the FP64 state rounded to FP32; free running: the GPU's "
                                          "own trajectory after all steps"}
        rb["cpu_baseline"] = {"value": round(nb / cpu_rb_s / 1e6, 4), "unit": "Mbody_steps/s",
                              "cores": os.cpu_count(), "kind": "port",
                              "sample": "one config-model step of the same scene, FP64 oracle "
                                        "(oracle/rb.c orc_rb_step_cfg_f64, OpenMP)"}
    prb.set_state(init)
    for _ in range(5):
        prb.step(rsap, dt, stream=stream)
    torch.cuda.synchronize()
    rsap.check()
    # step split: broadphase stages (CUDA events inside the step) against the whole step, eager launches
    rsap.enable_timing(True)
    split = []
    for _ in range(10):
        s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s0.record(stream)
        prb.step(rsap, dt, stream=stream)
        s1.record(stream)
        torch.cuda.synchronize()
        split.append((s0.elapsed_time(s1), sum(rsap.stage_times())))
    rsap.enable_timing(False)
    prb.set_state(init)
    prb.step(rsap, dt, stream=stream)
    torch.cuda.synchronize()
    Pb_rb = int(rsap.stats()["pairs"])
    # one step captured as a CUDA graph (the step makes no host synchronisation)
    gstream = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=gstream):
        prb.step(rsap, dt, stream=gstream)
    for _ in range(3):
        graph.replay()
    torch.cuda.synchronize()
    rsap.check()
    prb.contacts(reset=True)
    steps = args.rb_steps
    e0.record(stream)
    for _ in range(steps):
        graph.replay()
    e1.record(stream)
    torch.cuda.synchronize()
    rsap.check()
    rb_ms = e0.elapsed_time(e1) / steps
    Pc = prb.contacts() / (2.0 * steps)  # contact pairs per step (each contact is counted from both sides)
    npart = sc["n_particles"]
    b_rb = rb_algorithmic_bytes(nb, npart, int(Pc), Pb_rb)
    step_ms, bp_ms = float(np.median([a for a, _ in split])), float(np.median([b for _, b in split]))
    rb.update({"steps": steps, "ms_per_step": round(rb_ms, 4),
               "launch": "one step captured as a CUDA graph, replayed",
               "body_steps_per_s": round(nb / (rb_ms / 1e3), 1), "body_pairs": Pb_rb,
               "contact_pairs_per_step": round(Pc, 1),
               "bytes_alg": b_rb, "achieved_gbs": round(b_rb / (rb_ms / 1e3) / 1e9, 1),
               "frac": round(b_rb / (rb_ms / 1e3) / 1e9 / peak, 4),
               "formula": "276 n_b + 96 n_p + 8 P_c + B_bp(n_b, P_b), P_c = particle contact pairs per step "
                          "(device counter of the force kernel)",
               "step_split_eager_ms": {"step": round(step_ms, 4), "broadphase": round(bp_ms, 4),
                                       "rigid_kernels_and_gaps": round(step_ms - bp_ms, 4),
                                       "note": "10 eager steps, CUDA events; the timed graph replay has no gaps"}})
    out["rigid"] = rb
    del prb, rsap, graph
    torch.cuda.empty_cache()


def _extra_rigid_batched(args, dev, stream, out):
    import torch

    from gsap_gb300 import CONTACT_CONFIG, ParticleRigidBody, Sap, scenes
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    peak, _ = peaks()
    dt = 1.0 / 600.0
    cfgp = dict(k=2e4, eta=50.0, kt=0.1, gravity_y=-9.81, box_lo=(0.0, 0.0, 0.0), box_hi=(200.0, 200.0, 200.0))
    gstream = torch.cuda.Stream()
    # --- batched dynamics: 1024 scenes of 256..8192 bodies (cubes, rods, L shapes) in a 100^3 box
    ms_ = scenes.mixed_scenes(S=args.rb_scenes, seed=4)
    bo = ms_["body_offsets"]
    nbb = int(bo[-1])
    cfgb = dict(cfgp, box_hi=(100.0, 100.0, 100.0))
    bprb = ParticleRigidBody(nbb, ms_["n_particles"], 16)
    bprb.load_scene(ms_)
    bprb.set_contact(model=CONTACT_CONFIG, **cfgb)
    bprb.set_scenes(bo)
    binit = {k: np.ascontiguousarray(ms_[k], np.float32) for k in ("pos", "quat", "lin_vel", "ang_vel")}
    bsap2 = Sap(nbb, max_scenes=args.rb_scenes)
    # autotuner (set-up, untimed) on the body AABBs of the initial pose
    rbtuned = None
    if not args.no_tune:
        bmn, bmx = scenes.body_aabbs(ms_)
        rbtuned = bsap2.autotune(torch.from_numpy(bmn).to(dev), torch.from_numpy(bmx).to(dev),
                                 offsets=torch.from_numpy(np.asarray(bo, np.int32)).to(dev), reps=5, stream=stream)
    rbb = {"scenes": args.rb_scenes, "bodies": nbb, "particles": ms_["n_particles"],
           "broadphase_settings": dict(rbtuned, autotuned=True) if rbtuned else {"autotuned": False}}
    if not args.no_cpu:
        from oracle.trajectory import fp64_errors
        t0 = time.perf_counter()
        e = fp64_errors(bprb, bsap2, ms_, dict(cfgb, dt=dt), steps=args.rb_check_steps,
                        check_scenes=min(args.rb_check_scenes, args.rb_scenes), stream=stream)
        rbb["fp64_error"] = {"steps": e["steps"], "checked_scenes": min(args.rb_check_scenes, args.rb_scenes),
                             "checked_bodies": e["checked_bodies"], "per_step_max": e["per_step_max"],
                             "per_step_max_all_bodies": e["per_step_max_all_bodies"],
                             "bodies_left_out_max": e["bodies_left_out_max"], "worst": e["worst"],
                             "free_running": e["free_running"], "check_s": round(time.perf_counter() - t0, 1),
                             "definition": "as rigid.fp64_error, over the bodies of the first checked_scenes "
                                           "scenes of the batch (scenes never interact, so the oracle run on "
                                           "them alone gives their whole-batch result)"}
    bprb.set_state(binit)
    for _ in range(3):
        bprb.step(bsap2, dt, stream=stream)
    torch.cuda.synchronize()
    bsap2.check()
    bgraph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(bgraph, stream=gstream):
        bprb.step(bsap2, dt, stream=gstream)
    for _ in range(3):
        bgraph.replay()
    torch.cuda.synchronize()
    bsap2.check()
    bprb.contacts(reset=True)
    bsteps = args.rb_batched_steps
    e0.record(stream)
    for _ in range(bsteps):
        bgraph.replay()
    e1.record(stream)
    torch.cuda.synchronize()
    bsap2.check()
    b_ms = e0.elapsed_time(e1) / bsteps
    bPc = bprb.contacts() / (2.0 * bsteps)
    del bgraph
    # plain: the first 32 scenes, one system per scene, stepped one after another (eager launches)
    nplain = 32
    plain = []
    for s in range(nplain):
        a, z = int(bo[s]), int(bo[s + 1])
        sub = scenes.subset_bodies(ms_, a, z)
        p = ParticleRigidBody(z - a, sub["n_particles"], 16)
        p.load_scene(sub)
        p.set_contact(model=CONTACT_CONFIG, **cfgb)
        plain.append((p, Sap(z - a)))
    for p, sp in plain:
        p.step(sp, dt, stream=stream)
    torch.cuda.synchronize()
    psteps = 20
    e0.record(stream)
    for _ in range(psteps):
        for p, sp in plain:
            p.step(sp, dt, stream=stream)
    e1.record(stream)
    torch.cuda.synchronize()
    p_ms = e0.elapsed_time(e1) / psteps
    rbb.update({"ms_per_step": round(b_ms, 4), "launch": "one batched step captured as a CUDA graph, replayed",
                "scene_steps_per_s": round(args.rb_scenes / (b_ms / 1e3), 1),
                "contact_pairs_per_step": round(bPc, 1),
                "plain_scene_steps_per_s": round(nplain / (p_ms / 1e3), 1),
                "plain_sample": f"first {nplain} scenes, one system each, stepped in turn (eager launches)",
                "speedup_vs_plain": round((args.rb_scenes / b_ms) / (nplain / p_ms), 2)})
    out["rigid_batched"] = rbb



EXTRAS = ("small", "demo", "large", "batched", "rigid", "rigid_batched")


def run_extras(args, dev, stream, which=EXTRAS):
    """The other workloads, each measured on its own: the 16,384-box case
    against the O(n^2) brute force, Sap::collision on the demo's 24,576
    spheres, a 16,777,216-box scene, 4096 batched scenes against the plain
    per-scene pipeline, the 65,536-cube rigid-body step and the batched
    dynamics."""
    import torch
    out = {}
    for name in which:
        globals()[f"_extra_{name}"](args, dev, stream, out)
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
    return out


# ------------------------------------------------------------ reference arm

def run_reference(args, world, rank):
    """The reference algorithm on the host cores (oracle port).  A full call
    on 1M objects takes seconds, so each step is one call whose sweeps start
    from one of `parts` contiguous slices of each sorted group, the slices
    taken in turn; the call splits its time into the fixed stages (centres,
    axis choice, partition, group sorts) and the stages that scale with the
    sweep starts (the sweeps and the sort + unique of their pairs).  Over the
    steps, mean(fixed) + parts * mean(scaled) is the time of one full call;
    one full call, timed before the warm-up, checks it."""
    import oracle
    oracle.build()
    n = args.n
    host_sets, _ = make_inputs(0, n, args.jitter_sets)
    mn, mx = host_sets[0]
    t0 = time.perf_counter()
    _, f1, v1 = oracle.sap_ref_sampled(0, mn, mx, 1, 0)
    full_s = time.perf_counter() - t0
    # the fewest slices (a power of two, at most 256) that end W+K steps in ~150 s
    budget = 150.0 / max(1, args.steps + args.warmup)
    parts = 1
    while parts < 256 and f1 + v1 / parts > budget:
        parts *= 2
    for k in range(args.warmup):
        oracle.sap_ref_sampled(0, *host_sets[k % len(host_sets)], parts, (parts - args.warmup + k) % parts)
    fixed, scaled, wall = [], [], []
    for k in range(args.steps):
        a, b = host_sets[k % len(host_sets)]
        t0 = time.perf_counter()
        _, f, v = oracle.sap_ref_sampled(0, a, b, parts, k % parts)
        wall.append(time.perf_counter() - t0)
        fixed.append(f)
        scaled.append(v)
    ms = (float(np.mean(fixed)) + parts * float(np.mean(scaled))) * 1e3
    value = n / (ms / 1e3) / 1e6
    cores = os.cpu_count()
    sample = (f"reference SaP restated (oracle/bp.c orc_sap_ref_sampled, OpenMP over {cores} threads): each "
              f"step one call with the sweeps started from one of {parts} contiguous slices of each sorted group, "
              f"slices in turn ({np.mean(wall) * 1e3:.1f} ms wall per step); full-call time = mean fixed stages + "
              f"{parts} x mean sweep-proportional stages = {ms:.0f} ms; one full call measured {full_s * 1e3:.0f} ms "
              f"({n / full_s / 1e6:.3f} Mobjects/s)")
    line = {
        "impl": "reference",
        "metric": "1M-AABB PCA sweep-and-prune broadphase throughput (sorted i<j pair set)",
        "value": round(value, 4), "unit": "Mobjects/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": workload_config(args, world),
        "cpu_baseline": {"value": round(value, 4), "unit": "Mobjects/s", "cores": cores, "kind": "port",
                         "sample": sample, "fixed_ms": round(float(np.mean(fixed)) * 1e3, 3),
                         "scaled_ms": round(parts * float(np.mean(scaled)) * 1e3, 3),
                         "split": "fixed = centres, axis choice, partition, group sorts; scaled = the sweeps "
                                  "and the sort + unique of their pairs (all OpenMP-parallel)"},
        "e2e": {"value": round(value, 4), "unit": "Mobjects/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    return line


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1024)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=N_OBJ)
    ap.add_argument("--scenes", type=int, default=4096)
    ap.add_argument("--bodies", type=int, default=65536)
    ap.add_argument("--rb-scenes", type=int, default=1024)
    ap.add_argument("--rb-steps", type=int, default=1000, help="timed steps of the 65,536-cube rigid-body step")
    ap.add_argument("--rb-batched-steps", type=int, default=100, help="timed steps of the batched dynamics")
    ap.add_argument("--rb-check-steps", type=int, default=100,
                    help="steps of the FP64 trajectory checks of the rigid-body extras")
    ap.add_argument("--rb-check-scenes", type=int, default=128,
                    help="scenes of the batched dynamics checked against the FP64 oracle")
    ap.add_argument("--no-extras", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cell-factor", type=float, default=None,
                    help="sweep cell size / mean projected width (default: autotuned)")
    ap.add_argument("--sort-bits", type=int, default=None, choices=[16, 24, 32], help="radix key width (default: autotuned)")
    ap.add_argument("--sort", default=None, choices=["bucket", "radix"],
                    help="how the sweep entries are sorted (default: autotuned)")
    ap.add_argument("--sort-tile", type=int, default=None, choices=[2048, 4096],
                    help="keys per radix tile (default: autotuned)")
    ap.add_argument("--no-tune", action="store_true", help="skip the autotuner (defaults: 32 bits, cell factor 2.0)")
    ap.add_argument("--jitter-sets", type=int, default=N_JITTER,
                    help="distinct jittered inputs cycled by the timed calls (64 = the workload)")
    ap.add_argument("--only", default=None,
                    help="run only these extras (comma-separated: " + ",".join(EXTRAS) + ") and print them, "
                         "for profiling one workload")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    world, rank, local = dist_setup()
    if args.only:
        import torch
        import gsap_gb300
        torch.cuda.set_device(local)
        gsap_gb300.load()
        which = [w for w in args.only.split(",") if w]
        bad = [w for w in which if w not in EXTRAS]
        if bad:
            raise SystemExit(f"unknown extras {bad}; choose from {EXTRAS}")
        out = run_extras(args, torch.device("cuda", local), torch.cuda.current_stream(), which)
        print(json.dumps({"extras": out}), flush=True)
        return
    if args.impl == "reference":
        if rank != 0:
            return
        print(json.dumps(run_reference(args, world, rank)), flush=True)
        return
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    line = run_ours(args, world, rank, local)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
