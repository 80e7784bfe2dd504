"""Spatial-join benchmark: join pairs/s and probe rows/s on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload 2] [--impl ours|reference]

Workload (default 2): 2M building polygons (4-12 vertices, GMM-clustered)
probing 50k star zones (32-256 vertices) with ST_Intersects; both sides FP64
WKB in Arrow binary layout, seeded synthetic data.  A step is one pass of the
probe phase over the whole probe column: WKB decode -> f32 filter boxes ->
LBVH count / scan / scatter -> refine -> compaction, with the probe column
resident in HBM at the start of the timed region (value) or staged from
pinned host memory through the C ABI with the pairs copied back (e2e).
The probe column (>300 MB) exceeds the 129 MB L2, so no flush is needed
between steps.  The chosen form (banded FP32 filter + FP64 escalation) is the
headline; the plain FP64 form is timed beside it.

--impl reference times the reference CPU join restated in C (oracle/, the
reference's Rust binary cannot be built here) on the host cores, on a
bounded sample of the same workload.
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
for _p in (ROOT, os.path.join(ROOT, "sedona-db_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "join pairs/s & probe rows/s on 1 GB300 (exact pair set): chosen vs plain GPU form"


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


def make_inputs(workload: int, scale: float):
    from sedona_gpuspatial import datagen
    if workload == 1:
        return datagen.workload1(n_points=int(1_000_000 * scale), n_polys=int(10_000 * scale))
    if workload == 2:
        return datagen.workload2(n_buildings=int(2_000_000 * scale), n_zones=int(50_000 * scale))
    if workload == 3:
        return datagen.workload3(n_points=int(10_000_000 * scale), n_zones=int(50_000 * scale))
    if workload == 4:
        return datagen.workload4(n_probe=int(20_000_000 * scale), n_build=int(1_000_000 * scale))
    raise SystemExit(f"unknown workload {workload}")


WORKLOAD_NAMES = {
    1: "pip_uniform_1m_points_x_10k_star_polygons_st_intersects",
    2: "polygon_polygon_2m_buildings_x_50k_zones_st_intersects",
    3: "contains_10m_gmm_points_x_50k_zones_st_contains",
    4: "dwithin25_20m_x_1m_gmm_points",
}


class ClockSampler:
    """nvidia-smi sampling during the timed region (SM clock + throttle reasons)."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except FileNotFoundError:
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
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup(backend: str = "nccl"):
    """Replicas only: every rank runs the whole workload on its own GPU; the
    process group is used for the barrier around the timed region and the
    max-over-ranks time, never on the data path."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group(backend=backend)
        pg = dist
    return world, rank, local, pg


def barrier_max(pg, value: float, device) -> float:
    """Max of a per-rank time over all ranks (the job's time)."""
    if pg is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def aggregate_value(pairs_per_rank: int, world: int, ms_max: float) -> float:
    """Whole-job pairs/s: every replica processes the same workload."""
    return pairs_per_rank * world / (ms_max * 1e-3)


def to_device(col):
    """Uploads a WKB column into torch-owned device buffers; returns the
    SpjDeviceWkb view and the tensors keeping it alive."""
    import torch
    from sedona_gpuspatial import capi
    off = torch.from_numpy(np.ascontiguousarray(col.offsets)).cuda()
    data = torch.from_numpy(np.ascontiguousarray(col.data)).cuda()
    d = capi.SpjDeviceWkb(length=len(col), offsets=off.data_ptr(),
                          offsets_are_64bit=int(col.offsets.dtype == np.int64),
                          data=data.data_ptr(), data_length=len(col.data), validity=None,
                          validity_offset=0)
    return d, (off, data)


def probe_vertices_per_row(col) -> float:
    """Average stored vertices per probe row: 1 for a point column; for the
    single-ring polygon columns the generators make, (bytes - 13 per row) / 16."""
    if len(col) == 0:
        return 0.0
    if int(col.data[1]) == 1:  # WKB type of row 0 (little endian): Point
        return 1.0
    return (len(col.data) - 13 * len(col)) / 16.0 / len(col)


def algorithmic_refine_bytes(stats, probe_vertices_per_row: float, build_vertex_bytes: int):
    """8 B per candidate (ids) + the probe geometry's FP64 vertices per
    candidate + the build side's FP64 vertices once + 1 B flag per candidate."""
    m = stats["candidates"]
    return m * (8 + 16 * probe_vertices_per_row + 1) + build_vertex_bytes


def run_ours(args, world, rank, local, pg, light=False, workload=None, pred_override=None):
    """Workloads 1, 2 and 4 through SpjJoin.  light (the per-workload entries
    beside the headline): fewer steps, no option variants."""
    import torch
    from sedona_gpuspatial import capi

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    workload = workload or args.workload
    inp = make_inputs(workload, args.scale)
    pred = pred_override or {"knn": "dwithin"}.get(inp.predicate, inp.predicate)
    run_steps = min(args.steps, 3) if light else args.steps
    run_warmup = min(args.warmup, 2) if light else args.warmup
    distance = float(inp.params.get("distance", 0.0))
    rt = capi.Runtime.get(local)

    def make_join(form, opts=None):
        # the chosen form takes --join-options; a variant's options go on top
        opts = {**(args.join_options if form == 1 else {}), **(opts or {})}
        leaf = opts.pop("leaf_size", 0)
        j = capi.SpatialJoin(rt, leaf_size=leaf, refine_form=form, profile=True)
        for k, v in (opts or {}).items():
            j.set_option(k, v)
        j.build(inp.build)
        return j

    dcol, keep = to_device(inp.probe)
    n_rows = len(inp.probe)
    results = {}
    for form, name, steps in ((1, "chosen", run_steps), (0, "plain", max(1, args.plain_steps))):
        j = make_join(form)
        stream = torch.cuda.ExternalStream(j.stream())
        for _ in range(run_warmup):
            j.probe_device(dcol, pred, distance)
        j.reset_stats()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        if pg:
            pg.barrier()
        sampler = ClockSampler(local) if name == "chosen" else None
        if sampler:
            sampler.__enter__()
        with torch.cuda.stream(stream):
            e0.record(stream)
        npairs = 0
        for _ in range(steps):
            _, _, npairs = j.probe_device(dcol, pred, distance)
        with torch.cuda.stream(stream):
            e1.record(stream)
        torch.cuda.synchronize()
        if sampler:
            sampler.__exit__()
        ms = e0.elapsed_time(e1) / steps
        ms = barrier_max(pg, ms, dev)
        st = j.stats()
        results[name] = {"ms": ms, "pairs": npairs, "stats": st,
                         "clocks": sampler.summary() if sampler else None, "join": j}
    chosen = results["chosen"]
    st = chosen["stats"]
    steps = run_steps

    # e2e: host (pinned) WKB -> C ABI -> host pairs, copies inside the timed region
    # (page-locked host buffers from cudaHostAlloc, through torch's pinned
    # allocator; the column is copied in before the timed region)
    j = chosen["join"]
    from sedona_gpuspatial.wkb import WkbColumn

    def pinned_like(a):
        t = torch.empty(a.nbytes, dtype=torch.uint8, pin_memory=True)
        v = t.numpy().view(a.dtype)
        v[:] = a
        return t, v

    t_off, off = pinned_like(np.ascontiguousarray(inp.probe.offsets))
    t_data, data = pinned_like(np.ascontiguousarray(inp.probe.data))
    hcol = WkbColumn(off, data, inp.probe.validity)
    cap = int(chosen["pairs"] * 1.01) + 16
    t_ob = torch.empty(cap, dtype=torch.int32, pin_memory=True)
    t_op = torch.empty(cap, dtype=torch.int32, pin_memory=True)
    ob = t_ob.numpy().view(np.uint32)
    op = t_op.numpy().view(np.uint32)
    for _ in range(run_warmup):
        j.probe_host(hcol, pred, distance, ob, op)
    stream = torch.cuda.ExternalStream(j.stream())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        e0.record(stream)
    n_e2e = 0
    for _ in range(steps):
        n_e2e = j.probe_host(hcol, pred, distance, ob, op)
    with torch.cuda.stream(stream):
        e1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = barrier_max(pg, e0.elapsed_time(e1) / steps, dev)
    assert n_e2e == chosen["pairs"], (n_e2e, chosen["pairs"])
    del t_ob, t_op, ob, op
    torch.cuda.synchronize()

    # parity of the full-size run, outside the timed region: one more call of
    # the chosen form, its pair list against the oracle (the whole set, or a
    # seeded sample of probe rows where the oracle would take minutes)
    parity = None
    if args.parity:
        db, dp, n = j.probe_device(dcol, pred, distance)
        torch.cuda.synchronize()
        assert n == chosen["pairs"], (n, chosen["pairs"])
        if workload in (1, 2) and pred == "intersects":
            hb, hp = host_pairs(db, dp, n)
            parity = parity_full(inp.build, inp.probe, pred, distance, hb, hp)
            del hb, hp
        else:
            parity = parity_sample(inp.build, inp.probe, pred, distance, db, dp, n,
                                   frac=0.02 if workload == 2 else 0.01)

    # execution options of the chosen form, each timed on its own join
    # (they change speed only; the pair count is checked)
    variants = {}
    option_sets = [] if light else [{"candidate_order": 0}, {"refine_min_blocks": 4},
                                     {"cell_grid": 0}, {"grid_rings": 1},
                                     {"probe_order": -1},
                                     {"refine_split": 1}, {"refine_split": 3},
                                     {"candidate_order": 0, "refine_split": 0}]
    if pred == "dwithin" and not light:
        option_sets += [{"fuse_dwithin": 0}, {"dwithin_slots": 0}, {"dwithin_slots": 128},
                        {"dwithin_arena": 1}, {"dwithin_slots": 32},
                        {"probe_order": -1, "dwithin_arena": 0},
                        {"leaf_size": 4}, {"leaf_size": 32}]
    for opts in option_sets:
        jv = make_join(1, opts)
        for _ in range(2):
            jv.probe_device(dcol, pred, distance)
        sv = torch.cuda.ExternalStream(jv.stream())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        with torch.cuda.stream(sv):
            e0.record(sv)
        nv = 0
        for _ in range(max(1, min(steps, 3))):
            _, _, nv = jv.probe_device(dcol, pred, distance)
        with torch.cuda.stream(sv):
            e1.record(sv)
        torch.cuda.synchronize()
        assert nv == chosen["pairs"], (opts, nv, chosen["pairs"])
        name = ",".join(f"{k}={v}" for k, v in opts.items())
        variants[name] = e0.elapsed_time(e1) / max(1, min(steps, 3))
        del jv


    # roofline of the dominant kernel (refine) over the timed steps
    hbm_peak, peak_kind = load_peaks()
    probe_vpr = probe_vertices_per_row(inp.probe)
    build_vbytes = int(st["build_vertices"]) * 16
    ref_bytes = algorithmic_refine_bytes({"candidates": st["candidates"] / steps}, probe_vpr,
                                         build_vbytes)
    ref_ms = st["ms_refine"] / steps
    achieved = ref_bytes / (ref_ms * 1e-3) / 1e9 if ref_ms > 0 else 0.0
    kernel = "k_dwithin<fast>" if pred == "dwithin" else "k_refine<fast>"
    if pred == "dwithin" and st["ms_compact"] == 0:
        # point-point ST_DWithin is decided inside the traversal (count pass +
        # scatter pass, no candidate pairs): per probe row its point and box
        # (32 B) and a count (4 B), 8 B per result pair, the build points
        # (FP64 + FP32 splits, 32 B) once
        kernel = "k_dwithin_fused (count + scatter passes)"
        ref_bytes = n_rows * 36 + 8 * chosen["pairs"] + 32 * len(inp.build)
        ref_ms = (st["ms_filter"] + st["ms_refine"]) / steps
        achieved = ref_bytes / (ref_ms * 1e-3) / 1e9 if ref_ms > 0 else 0.0
    traffic = None
    traffic_note = None
    tf = os.path.join(ROOT, "profiles", f"refine_traffic_workload{workload}.json")
    if os.path.exists(tf) and pred == "intersects":
        with open(tf) as f:
            tj = json.load(f)
        traffic = tj.get("bytes_per_launch")
        traffic_note = tj.get("scaled_from")

    pairs_total = chosen["pairs"] * world
    value = pairs_total / (chosen["ms"] * 1e-3)
    plain = results["plain"]
    out = {
        "metric": METRIC,
        "value": value,
        "unit": "pairs/s",
        "n_gpus": world,
        "steps": steps,
        "warmup": run_warmup,
        "ms_per_step": chosen["ms"],
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64 (f32 filter)",
        "data": "synthetic (seeded; SpatialBench data not available)",
        "config": {"workload": WORKLOAD_NAMES[workload] if pred_override is None
                   else WORKLOAD_NAMES[workload].replace("st_intersects", "st_" + pred),
                   "probe_rows": n_rows,
                   "build_rows": len(inp.build), "predicate": pred, "scale": args.scale,
                   "pairs_per_step": chosen["pairs"], "l2": "probe column > L2, no flush",
                   "parallelism": f"replicas x{world}", **join_opts_cfg(args)},
        "probe_rows_per_s": n_rows * world / (chosen["ms"] * 1e-3),
        "plain_f64_form": {"pairs_per_s": plain["pairs"] * world / (plain["ms"] * 1e-3),
                           "ms_per_step": plain["ms"], "pairs": plain["pairs"],
                           "steps": max(1, args.plain_steps),
                           "speedup_chosen_vs_plain": plain["ms"] / chosen["ms"]},
        "phases_ms_per_step": {k: st[k] / steps for k in
                               ("ms_decode", "ms_filter", "ms_refine", "ms_compact")},
        "fp64_escalated_fraction": st["escalations"] / max(1, st["pairs_evaluated"]),
        "candidates_per_step": st["candidates"] / steps,
        "gpu_launches": int(st["kernel_launches"]),
        "option_variants_ms_per_step": variants,
        "e2e": {"value": pairs_total / (e2e_ms * 1e-3), "unit": "pairs/s",
                "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": int(off.nbytes + data.nbytes),
                "d2h_bytes_per_step": int(8 * n_e2e)},
        "roofline": {"bound": "hbm", "kernel": kernel, "achieved": achieved,
                     "peak": hbm_peak, "peak_kind": peak_kind, "unit": "GB/s",
                     "frac": achieved / hbm_peak, "traffic": traffic,
                     "algorithmic_bytes_per_launch": ref_bytes},
        "clocks": chosen["clocks"],
    }
    if traffic_note:
        out["roofline"]["traffic_note"] = traffic_note
    if parity is not None:
        out["parity"] = parity
    if workload == 4:
        out["knn"] = run_knn(inp, local, run_steps, run_warmup, args.parity)
    return out, inp


def dev_i32(ptr: int, n: int):
    """A torch view of n int32 values at a device pointer the library owns."""
    import torch

    class _A:
        __cuda_array_interface__ = {"shape": (n,), "typestr": "<i4", "data": (ptr, False),
                                    "version": 3, "strides": None}
    return torch.as_tensor(_A(), device="cuda")


def host_pairs(db: int, dp: int, n: int):
    """A device pair list (the library's buffers) copied to host arrays."""
    if n == 0:
        return np.zeros(0, np.uint32), np.zeros(0, np.uint32)
    return (dev_i32(db, n).cpu().numpy().view(np.uint32),
            dev_i32(dp, n).cpu().numpy().view(np.uint32))


def device_keys(db: int, dp: int, n: int):
    """Sorted (probe << 32 | build) keys of a device pair list, on the device."""
    import torch
    if n == 0:
        return torch.zeros(0, dtype=torch.int64, device="cuda")
    k = (dev_i32(dp, n).long() << 32) | (dev_i32(db, n).long() & 0xFFFFFFFF)
    return torch.sort(k).values


def sorted_keys(b, p):
    """(probe << 32 | build) keys of a pair list, sorted: equal arrays mean
    equal pair sets."""
    k = (np.asarray(p).astype(np.uint64) << np.uint64(32)) | np.asarray(b).astype(np.uint64)
    k.sort()
    return k


def parity_full(build_col, probe_col, pred, distance, b, p):
    """The whole pair set of a full-size run against the oracle's (the C
    restatement of the reference CPU join) on all host cores."""
    import oracle
    oracle.build(with_ref=False)
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    ob, op = oracle.join(oracle.Geoms(build_col), oracle.Geoms(probe_col), pred, distance,
                         nthreads=threads)
    oracle_s = time.perf_counter() - t0
    eq = len(ob) == len(b) and np.array_equal(sorted_keys(b, p), sorted_keys(ob, op))
    return {"pairs_equal": bool(eq), "pairs": int(len(b)), "oracle_pairs": int(len(ob)),
            "oracle_cores": threads, "oracle_s": round(oracle_s, 2),
            "kind": "full sorted (probe, build) pair set vs the oracle"}


def parity_sample(build_col, probe_col, pred, distance, db, dp, n, frac=0.01, seed=20260301):
    """The pair list of a full-size run, restricted on the device to a seeded
    sample of probe rows, against the oracle on those rows (every pair of
    every sampled row: the per-row lists must be equal)."""
    import torch
    import oracle
    oracle.build(with_ref=False)
    threads = os.cpu_count() or 1
    nrows = len(probe_col)
    rng = np.random.default_rng(seed)
    rows = np.sort(rng.choice(nrows, size=max(1, int(nrows * frac)), replace=False))
    pos = torch.full((nrows,), -1, dtype=torch.int32, device="cuda")
    pos[torch.from_numpy(rows).cuda()] = torch.arange(len(rows), dtype=torch.int32,
                                                       device="cuda")
    keys = []
    if n:
        dbt, dpt = dev_i32(db, n), dev_i32(dp, n)
        step = 1 << 27
        for s in range(0, n, step):
            pc, bc = dpt[s:s + step], dbt[s:s + step]
            sp = pos.index_select(0, pc)
            m = sp >= 0
            keys.append(((sp[m].long() << 32) | (bc[m].long() & 0xFFFFFFFF)).cpu().numpy())
    gk = np.sort(np.concatenate(keys)).astype(np.uint64) if keys else np.zeros(0, np.uint64)
    del pos
    t0 = time.perf_counter()
    ob, op = oracle.join(oracle.Geoms(build_col), oracle.Geoms(probe_col.take(rows)), pred,
                         distance, nthreads=threads)
    oracle_s = time.perf_counter() - t0
    eq = len(gk) == len(ob) and np.array_equal(gk, sorted_keys(ob, op))
    return {"pairs_equal": bool(eq), "pairs": int(n), "sampled_rows": int(len(rows)),
            "sampled_pairs": int(len(gk)), "oracle_pairs": int(len(ob)), "oracle_cores": threads,
            "oracle_s": round(oracle_s, 2),
            "kind": f"{frac:.0%} of probe rows (seed {seed}): every pair of those rows from the "
                    "full-size run vs the oracle"}


def join_opts_cfg(args):
    return {"join_options": args.join_options} if args.join_options else {}


def run_stream(args, world, rank, local, pg):
    """Workload 3: the probe column arrives as uneven record batches.  Chosen
    form: the batched stream (one CUDA-graph replay of the persistent
    work-queue kernels over every batch, parameters autotuned).  Plain form:
    one probe call per batch with the FP64 refine."""
    import torch
    from sedona_gpuspatial import capi

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    inp = make_inputs(args.workload, args.scale)
    rt = capi.Runtime.get(local)
    sizes = inp.batches
    dcols, keep = [], []
    start = 0
    for n in sizes:
        part = inp.probe.slice(start, start + n)
        d, k = to_device(part)
        dcols.append(d)
        keep.append(k)
        start += n
    j = capi.SpatialJoin(rt, refine_form=1, profile=True)
    for k, v in args.join_options.items():
        j.set_option(k, v)
    j.build(inp.build)
    st = capi.StreamProbe(j)
    st.set_batches(dcols)
    cache = os.environ.get("SPJ_AUTOTUNE_CACHE", "")
    t0 = time.perf_counter()
    tuned = st.autotune(inp.predicate, cache or None)
    tune_s = time.perf_counter() - t0
    for _ in range(args.warmup):
        st.run(inp.predicate)
    stream = torch.cuda.ExternalStream(st.stream())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.__enter__()
    with torch.cuda.stream(stream):
        e0.record(stream)
    npairs = 0
    for _ in range(args.steps):
        _, _, npairs = st.run(inp.predicate)
    with torch.cuda.stream(stream):
        e1.record(stream)
    torch.cuda.synchronize()
    sampler.__exit__()
    ms = barrier_max(pg, e0.elapsed_time(e1) / args.steps, dev)
    sstats = st.stats()

    # e2e: every step copies each batch's WKB (offsets + bytes) from pinned
    # host memory into the stream's device batches, replays, and copies the
    # pairs back into pinned host memory, all on the stream's own CUDA stream
    host_parts = []
    for (d, k) in zip(dcols, keep):
        host_parts.append([torch.empty(t.numel() * t.element_size(), dtype=torch.uint8,
                                       pin_memory=True).view(t.dtype) for t in k])
        for h_, t_ in zip(host_parts[-1], k):
            h_.copy_(t_.cpu())
    h2d = sum(t.numel() * t.element_size() for k in keep for t in k)
    cap = int(npairs * 1.01) + 16
    hb = torch.empty(cap, dtype=torch.int32, pin_memory=True)
    hpr = torch.empty(cap, dtype=torch.int32, pin_memory=True)

    def e2e_step():
        with torch.cuda.stream(stream):
            for hp, k in zip(host_parts, keep):
                for h, t in zip(hp, k):
                    t.copy_(h, non_blocking=True)
        db, dp, n = st.run(inp.predicate)
        if n:
            with torch.cuda.stream(stream):
                hb[:n].copy_(dev_i32(db, n), non_blocking=True)
                hpr[:n].copy_(dev_i32(dp, n), non_blocking=True)
        return n

    for _ in range(args.warmup):
        e2e_step()
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        e0.record(stream)
    for _ in range(args.steps):
        n_e2e = e2e_step()
    with torch.cuda.stream(stream):
        e1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = barrier_max(pg, e0.elapsed_time(e1) / args.steps, dev)
    assert n_e2e == npairs, (n_e2e, npairs)
    # torch's pinned allocator records an event on the stream a pinned block
    # was copied on when the block is freed: free them while the stream
    # probe (and its stream) still exists
    torch.cuda.synchronize()
    del host_parts, hb, hpr, h_, t_
    torch.cuda.synchronize()
    parity = None
    if args.parity:
        db, dp, n = st.run(inp.predicate)
        torch.cuda.synchronize()
        parity = parity_sample(inp.build, inp.probe, inp.predicate, 0.0, db, dp, n, frac=0.01)

    # plain form: per-batch calls, FP64 refine
    jp = capi.SpatialJoin(rt, refine_form=0, profile=True)
    jp.build(inp.build)
    for d in dcols[:3]:
        jp.probe_device(d, inp.predicate, 0.0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    base, plain_pairs = 0, 0
    for d, n in zip(dcols, sizes):
        _, _, m = jp.probe_device(d, inp.predicate, 0.0, base)
        plain_pairs += m
        base += n
    torch.cuda.synchronize()
    plain_ms = (time.perf_counter() - t0) * 1e3
    assert plain_pairs == npairs, (plain_pairs, npairs)
    # per-batch calls with the chosen refine (batching ablation)
    jb = capi.SpatialJoin(rt, refine_form=1)
    jb.build(inp.build)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    base = 0
    for d, n in zip(dcols, sizes):
        jb.probe_device(d, inp.predicate, 0.0, base)
        base += n
    torch.cuda.synchronize()
    per_batch_ms = (time.perf_counter() - t0) * 1e3

    n_rows = len(inp.probe)
    hbm_peak, peak_kind = load_peaks()
    # algorithmic bytes of one replay: WKB + offsets read once (two passes
    # read them twice), 4 B count + 8 B offset per row, 8 B per pair out,
    # the build side's vertices once
    wkb_bytes = len(inp.probe.data) + 4 * (n_rows + len(sizes))
    alg = 2 * wkb_bytes + 12 * n_rows + 8 * npairs + 16 * int(j.stats()["build_vertices"])
    achieved = alg / (ms * 1e-3) / 1e9
    out = {
        "metric": METRIC, "value": aggregate_value(npairs, world, ms), "unit": "pairs/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64 (f32 filter)", "data": "synthetic (seeded; SpatialBench data not available)",
        "config": {"workload": WORKLOAD_NAMES[args.workload], "probe_rows": n_rows,
                   "batches": len(sizes), "build_rows": len(inp.build),
                   "predicate": inp.predicate, "scale": args.scale, "pairs_per_step": npairs,
                   "autotuned": {"block": tuned[0], "chunk_rows": tuned[1], "leaf_size": tuned[2],
                                 "seconds": tune_s},
                   "l2": "probe batches > L2, no flush", "parallelism": f"replicas x{world}",
                   **join_opts_cfg(args)},
        "probe_rows_per_s": n_rows * world / (ms * 1e-3),
        "plain_f64_form": {"pairs_per_s": npairs / (plain_ms * 1e-3), "ms_per_step": plain_ms,
                           "form": "one probe call per batch, FP64 refine",
                           "speedup_chosen_vs_plain": plain_ms / ms},
        "per_batch_calls_f32_ms": per_batch_ms,
        "e2e": {"value": npairs * world / (e2e_ms * 1e-3), "unit": "pairs/s",
                "ms_per_step": e2e_ms, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(8 * npairs)},
        "gpu_launches": int(sstats["launches_per_replay"] * args.steps),
        "fp64_escalations_per_replay": sstats["escalations"] / max(1, args.steps + args.warmup + 2),
        "roofline": {"bound": "hbm", "kernel": "stream replay (decode, traversal, refine, compact)",
                     "achieved": achieved, "peak": hbm_peak, "peak_kind": peak_kind,
                     "unit": "GB/s", "frac": achieved / hbm_peak, "traffic": None,
                     "algorithmic_bytes_per_launch": alg},
        "clocks": sampler.summary(),
    }
    if parity is not None:
        out["parity"] = parity
    return out, inp


def run_knn(inp, local, steps: int, warmup: int, parity: bool = False):
    """KNN k=8 over the workload-4 points: 20M probes x 1M build, probe
    coordinates resident in HBM; chosen form (split-FP32 traversal proving
    the k-set, FP64 keys for the k results only, unproven probes through the
    exact kernel) vs the plain FP64 form."""
    import torch
    from sedona_gpuspatial import capi
    k = int(inp.params["k"])
    bx, by = inp.params["build_xy"]
    px, py = inp.params["probe_xy"]
    d_xy = torch.from_numpy(np.ascontiguousarray(np.stack([px, py], 1))).cuda()
    n = len(px)
    d_idx = torch.empty(n * k, dtype=torch.int32, device="cuda")
    d_dist = torch.empty(n * k, dtype=torch.float64, device="cuda")
    res = {}
    for form, name in ((1, "chosen"), (0, "plain")):
        kj = capi.KnnJoin(capi.Runtime.get(local), refine_form=form)
        kj.build(bx, by)
        reps = steps if name == "chosen" else 1
        for _ in range(warmup if name == "chosen" else 1):
            kj.query_device(d_xy.data_ptr(), n, k, d_idx.data_ptr(), d_dist.data_ptr())
        stream = torch.cuda.ExternalStream(kj.stream())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            e0.record(stream)
        for _ in range(reps):
            kj.query_device(d_xy.data_ptr(), n, k, d_idx.data_ptr(), d_dist.data_ptr())
        with torch.cuda.stream(stream):
            e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        res[name] = {"ms_per_step": ms, "probe_rows_per_s": n / (ms * 1e-3),
                     "pairs_per_s": n * k / (ms * 1e-3)}
        st = kj.stats()
        res[name]["exact_evals_per_probe"] = st["exact_evals"] / max(1, st["queries"])
        res[name]["redone_frac"] = st["redone"] / max(1, st["queries"])
    # algorithmic bytes: 16 B per probe in, k * (4 + 8) B out
    alg = n * (16 + 12 * k)
    hbm_peak, peak_kind = load_peaks()
    ach = alg / (res["chosen"]["ms_per_step"] * 1e-3) / 1e9
    res["speedup_chosen_vs_plain"] = res["plain"]["ms_per_step"] / res["chosen"]["ms_per_step"]
    res["k"] = k
    res["roofline"] = {"bound": "hbm", "kernel": "k_knn_split<8>", "achieved": ach,
                       "peak": hbm_peak, "unit": "GB/s", "frac": ach / hbm_peak,
                       "algorithmic_bytes_per_launch": alg}
    if parity:
        # the chosen form's k-lists of a seeded 1% of the probes against the
        # oracle's: build rows exactly, distances to 1e-12 relative
        import oracle
        from sedona_gpuspatial import wkb
        kj = capi.KnnJoin(capi.Runtime.get(local), refine_form=1)
        kj.build(bx, by)
        kj.query_device(d_xy.data_ptr(), n, k, d_idx.data_ptr(), d_dist.data_ptr())
        torch.cuda.synchronize()
        rng = np.random.default_rng(20260302)
        rows = np.sort(rng.choice(n, size=max(1, n // 100), replace=False))
        trows = torch.from_numpy(rows).cuda()
        gi = d_idx.view(n, k).index_select(0, trows).cpu().numpy().view(np.uint32)
        gd = d_dist.view(n, k).index_select(0, trows).cpu().numpy()
        threads = os.cpu_count() or 1
        t0 = time.perf_counter()
        oi, od = oracle.knn(oracle.Geoms(wkb.points_column(bx, by)),
                            oracle.Geoms(wkb.points_column(px[rows], py[rows])), k,
                            nthreads=threads)
        fin = np.isfinite(od)
        res["parity"] = {
            "ids_equal": bool(np.array_equal(gi, oi)),
            "dist_max_rel_err": float(np.max(np.abs(gd[fin] - od[fin]) /
                                             np.maximum(np.abs(od[fin]), 1e-300)))
            if fin.any() else 0.0,
            "dist_tolerance": 1e-12, "sampled_rows": int(len(rows)), "oracle_cores": threads,
            "oracle_s": round(time.perf_counter() - t0, 2),
            "kind": "1% of probes (seed 20260302): k build rows (ties by row id) and distances "
                    "vs the oracle"}
        res["parity"]["pairs_equal"] = bool(res["parity"]["ids_equal"] and
                                            res["parity"]["dist_max_rel_err"] <= 1e-12)
    return res


def run_learned(args, world, rank, local, pg):
    """Workload 5: 100M GMM build points, 10M range boxes + 10M exact-point
    lookups (ST_Intersects).  Chosen form: the learned index (trained on the
    GPU).  Plain form: the LBVH join with the FP64 refine on the same inputs,
    which is also the arbiter of the pair set."""
    import torch
    from sedona_gpuspatial import capi, datagen

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    s = args.scale
    build, boxes, lookups, _ = datagen.workload5(n_build=int(100_000_000 * s),
                                                 n_boxes=int(10_000_000 * s),
                                                 n_lookups=int(10_000_000 * s))
    rt = capi.Runtime.get(local)
    db_, kb = to_device(build)
    dbox, kbox = to_device(boxes)
    dlk, klk = to_device(lookups)
    li = capi.LearnedIndex(rt, leaves=4096)
    li.build_device(db_)
    st_build = li.stats()
    # window autotuned on a sample (a tenth of each probe column)
    ns = max(1, len(boxes) // 10)
    sb, ksb = to_device(boxes.slice(0, ns))
    sl, ksl = to_device(lookups.slice(0, max(1, len(lookups) // 10)))
    t0 = time.perf_counter()
    window = li.autotune_window([sb, sl], "intersects")
    tune_ms = (time.perf_counter() - t0) * 1e3
    del ksb, ksl

    def step(obj, method):
        n = 0
        for d in (dbox, dlk):
            _, _, m = getattr(obj, method)(d, "intersects")
            n += m
        return n

    stream = torch.cuda.ExternalStream(li.stream())
    for _ in range(args.warmup):
        step(li, "query_device")
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.__enter__()
    before = li.stats()
    with torch.cuda.stream(stream):
        e0.record(stream)
    npairs = 0
    for _ in range(args.steps):
        npairs = step(li, "query_device")
    with torch.cuda.stream(stream):
        e1.record(stream)
    torch.cuda.synchronize()
    sampler.__exit__()
    after = li.stats()
    ms = barrier_max(pg, e0.elapsed_time(e1) / args.steps, dev)
    lookups_n = after["lookups"] - before["lookups"]
    phases = {k: (after[k] - before[k]) / args.steps for k in ("ms_order", "ms_ranges", "ms_eval")}
    launches = int(after["kernel_launches"] - before["kernel_launches"])
    steps_per_lookup = (after["search_steps"] - before["search_steps"]) / max(1, lookups_n)

    # e2e: every step copies both probe columns (offsets + WKB) from pinned
    # host memory into their device buffers, queries, and copies the pairs
    # into pinned host memory, all on the index's stream (stream order keeps
    # a column's pair copies ahead of the next query, which reuses the
    # index's output buffers)
    host_parts = []
    for k in (kbox, klk):
        host_parts.append([torch.empty(t.numel() * t.element_size(), dtype=torch.uint8,
                                       pin_memory=True).view(t.dtype) for t in k])
        for h_, t_ in zip(host_parts[-1], k):
            h_.copy_(t_.cpu())
    h2d = sum(t.numel() * t.element_size() for k in (kbox, klk) for t in k)
    cap = int(npairs * 1.01) + 16
    hb = torch.empty(cap, dtype=torch.int32, pin_memory=True)
    hpr = torch.empty(cap, dtype=torch.int32, pin_memory=True)

    def e2e_step():
        n = 0
        for d, hps, k in zip((dbox, dlk), host_parts, (kbox, klk)):
            with torch.cuda.stream(stream):
                for h, t in zip(hps, k):
                    t.copy_(h, non_blocking=True)
            dbp, dpp, m = li.query_device(d, "intersects")
            if m:
                with torch.cuda.stream(stream):
                    hb[n:n + m].copy_(dev_i32(dbp, m), non_blocking=True)
                    hpr[n:n + m].copy_(dev_i32(dpp, m), non_blocking=True)
            n += m
        return n

    for _ in range(args.warmup):
        e2e_step()
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        e0.record(stream)
    for _ in range(args.steps):
        n_e2e = e2e_step()
    with torch.cuda.stream(stream):
        e1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = barrier_max(pg, e0.elapsed_time(e1) / args.steps, dev)
    assert n_e2e == npairs, (n_e2e, npairs)
    # torch's pinned allocator records an event on the stream a pinned block
    # was copied on when the block is freed: free them while the index (and
    # its stream) still exists
    del host_parts, hb, hpr, h_, t_
    torch.cuda.synchronize()

    # ablation: the untrained model (line through each leaf's end keys)
    li.set_trained(False)
    st_untrained = li.stats()
    step(li, "query_device")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    b0 = li.stats()
    n_untrained = step(li, "query_device")
    torch.cuda.synchronize()
    untrained_ms = (time.perf_counter() - t0) * 1e3
    b1 = li.stats()
    untrained_steps = (b1["search_steps"] - b0["search_steps"]) / max(1, b1["lookups"] - b0["lookups"])
    li.set_trained(True)
    assert n_untrained == npairs

    # plain form / arbiter: the LBVH join, FP64 refine, same inputs
    # (leaf size 4: measured best for range boxes and lookups over points)
    jp = capi.SpatialJoin(rt, leaf_size=4, refine_form=0)
    jp.build_device(db_)
    step(jp, "probe_device")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    n_plain = step(jp, "probe_device")
    torch.cuda.synchronize()
    plain_ms = (time.perf_counter() - t0) * 1e3
    assert n_plain == npairs, (n_plain, npairs)
    # the LBVH join in its chosen form (FP32 filter, Morton-ordered probes)
    jf = capi.SpatialJoin(rt, leaf_size=4, refine_form=1)
    jf.build_device(db_)
    step(jf, "probe_device")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    n_fast = step(jf, "probe_device")
    torch.cuda.synchronize()
    fast_ms = (time.perf_counter() - t0) * 1e3
    assert n_fast == npairs, (n_fast, npairs)
    # parity: the learned index's full pair set against the LBVH join with
    # the FP64 refine (the arbiter), per probe column, compared on the device
    parity = None
    if args.parity:
        equal = True
        for d in (dbox, dlk):
            ka = device_keys(*li.query_device(d, "intersects"))
            kb = device_keys(*jp.probe_device(d, "intersects"))
            equal = equal and ka.shape == kb.shape and bool(torch.equal(ka, kb))
            del ka, kb
        parity = {"pairs_equal": equal, "pairs": int(npairs),
                  "kind": "full sorted pair sets, learned index vs the LBVH join with the "
                          "FP64 refine (the arbiter; both probe columns)"}
    n_rows = len(boxes) + len(lookups)
    hbm_peak, peak_kind = load_peaks()
    # algorithmic bytes per step: probe WKB + offsets once, per lookup the
    # key / point reads (4 B key + 16 B point per scanned build point are
    # not counted: re-reads), 8 B per pair out
    alg = len(boxes.data) + len(lookups.data) + 4 * (n_rows + 2) + 8 * npairs
    achieved = alg / (ms * 1e-3) / 1e9
    out = {
        "metric": METRIC, "value": aggregate_value(npairs, world, ms), "unit": "pairs/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64 (f32 filter)", "data": "synthetic (seeded; SpatialBench data not available)",
        "config": {"workload": "learned_index_100m_points_10m_boxes_10m_lookups_st_intersects",
                   "build_rows": len(build), "probe_rows": n_rows, "scale": s,
                   "pairs_per_step": npairs, "leaves": 4096,
                   "l2": "probe columns > L2, no flush", "parallelism": f"replicas x{world}"},
        "probe_rows_per_s": n_rows * world / (ms * 1e-3),
        "learned_index": {"build_ms": st_build["ms_build"], "window": window,
                          "window_box": after["window_box"],
                          "window_autotune_ms": tune_ms,
                          "phases_ms_per_step": phases,
                          "leaves_over_window_after_tuning": after["leaves_over_window"],
                          "max_err": st_build["max_err"],
                          "mean_err": st_build["mean_err"],
                          "leaves_over_window": st_build["leaves_over_window"],
                          "lbvh_fallback_rows_per_step":
                              (after["lbvh_fallbacks"] - before["lbvh_fallbacks"]) / args.steps,
                          "window_misses_per_step":
                              (after["window_misses"] - before["window_misses"]) / args.steps,
                          "ranges_per_step": (after["ranges"] - before["ranges"]) / args.steps,
                          "search_steps_per_lookup": steps_per_lookup,
                          "untrained": {"ms_per_step": untrained_ms,
                                        "max_err": st_untrained["max_err"],
                                        "mean_err": st_untrained["mean_err"],
                                        "search_steps_per_lookup": untrained_steps}},
        "plain_f64_form": {"pairs_per_s": npairs / (plain_ms * 1e-3), "ms_per_step": plain_ms,
                           "form": "LBVH join, FP64 refine (also the pair-set arbiter)",
                           "speedup_chosen_vs_plain": plain_ms / ms},
        "lbvh_fast_form": {"ms_per_step": fast_ms, "pairs_per_s": npairs / (fast_ms * 1e-3),
                           "form": "LBVH join, FP32-filtered refine, Morton-ordered probes",
                           "speedup_learned_vs_lbvh_fast": fast_ms / ms},
        "roofline": {"bound": "hbm", "kernel": "k_learned_ranges + k_learned_eval (all passes)",
                     "achieved": achieved, "peak": hbm_peak, "peak_kind": peak_kind,
                     "unit": "GB/s", "frac": achieved / hbm_peak, "traffic": None,
                     "algorithmic_bytes_per_launch": alg},
        "gpu_launches": launches,
        "e2e": {"value": npairs * world / (e2e_ms * 1e-3), "unit": "pairs/s",
                "ms_per_step": e2e_ms, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(8 * npairs)},
        "clocks": sampler.summary(),
    }
    if parity is not None:
        out["parity"] = parity
    from types import SimpleNamespace
    return out, SimpleNamespace(build=build, probe=boxes, predicate="intersects", params={})


def cpu_baseline(inp, seconds_budget: float = 15.0, pred=None):
    """The oracle (C restatement of the reference CPU join) on a bounded
    sample of the probe side with all host threads."""
    import oracle
    oracle.build(with_ref=False)
    threads = os.cpu_count() or 1
    B = oracle.Geoms(inp.build)
    pred = pred or {"knn": "dwithin"}.get(inp.predicate, inp.predicate)
    distance = float(inp.params.get("distance", 0.0))
    n = len(inp.probe)
    # each oracle call builds its grid over the build side first: that is the
    # reference's build phase, so it is timed alone (one probe row) and taken
    # out of every call's time
    P1 = oracle.Geoms(inp.probe.slice(0, 1))
    t0 = time.perf_counter()
    oracle.join(B, P1, pred, distance, nthreads=threads)
    t_build = time.perf_counter() - t0
    rows = min(n, 20000)
    el = 0.0
    npairs = 0
    done = 0
    while True:
        P = oracle.Geoms(inp.probe.slice(done % n, min(n, done % n + rows)))
        t0 = time.perf_counter()
        b, p = oracle.join(B, P, pred, distance, nthreads=threads)
        el += max(time.perf_counter() - t0 - t_build, 1e-9)
        npairs += len(b)
        done += len(P._keep)
        if el > seconds_budget or done >= n:
            break
        rows = min(n - done, int(rows * 2))
    return {"value": npairs / el, "unit": "pairs/s", "cores": threads, "kind": "port",
            "probe_rows_per_s": done / el,
            "sample": f"first {done} probe rows of the workload against the full build side "
                      f"(probe phase: the oracle's per-call grid build, {t_build:.2f} s, "
                      "timed alone and subtracted)"}


def run_reference(args, world, rank):
    if rank != 0:
        return None
    inp = make_inputs(args.workload, args.scale)
    vals = []
    for _ in range(args.warmup):
        pass  # the CPU join has no warm-up state worth priming beyond the first sample
    for _ in range(args.steps):
        vals.append(cpu_baseline(inp, seconds_budget=args.ref_seconds))
    v = float(np.median([x["value"] for x in vals]))
    base = vals[-1]
    return {
        "impl": "reference",
        "metric": METRIC, "value": v, "unit": "pairs/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD_NAMES[args.workload], "probe_rows": len(inp.probe),
                   "build_rows": len(inp.build), "scale": args.scale},
        "cpu_baseline": {"value": v, "unit": "pairs/s", "cores": base["cores"],
                         "kind": "port", "sample": base["sample"]},
        "e2e": {"value": v, "unit": "pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "restatement of the reference CPU SpatialJoinExec (tg predicates) in C; "
                "the reference's Rust binary cannot be built here",
    }


def run_geoparquet(args, local):
    """GeoParquet -> device: the 2M-building probe column of the polygon
    workload written as a GeoParquet file (SNAPPY, data page v1, 1 MiB pages,
    1M-row row groups), then read onto the device column the join takes.
    value: rows/s over the device phases (Snappy, page decode, value copy)
    with the chunk bytes in HBM; e2e: rows/s of open + read from the file
    (page cache) through the H2D copy to the finished device column."""
    import shutil
    import tempfile

    import torch
    from sedona_gpuspatial import geoparquet as gp
    inp = make_inputs(2, args.scale)
    col = inp.probe
    tmp = tempfile.mkdtemp(prefix="spj_gpq_")
    try:
        path = os.path.join(tmp, "buildings.parquet")
        t0 = time.perf_counter()
        gp.write_wkb(path, col, compression="snappy", page_version=1,
                     row_group_rows=1 << 20, page_bytes=1 << 20)
        t_write = time.perf_counter() - t0
        n = len(col)
        steps, warmup = args.steps, max(3, args.warmup)
        t0 = time.perf_counter()
        f = gp.GeoParquetFile(path)
        t_open = time.perf_counter() - t0
        for _ in range(warmup):
            f.read_wkb(device=local)
        dev_ms, ph_sum, wall = 0.0, None, 0.0
        sampler = ClockSampler(local)
        with sampler:
            for _ in range(steps):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                d = f.read_wkb(device=local)
                wall += time.perf_counter() - t0
                st, ph = f.stats(), f.phases()
                dev_ms += ph["decompress"] + ph["decode"] + ph["values"]
                ph_sum = ph if ph_sum is None else {k: ph_sum[k] + ph[k] for k in ph}
        ms = dev_ms / steps
        e2e_ms = wall * 1e3 / steps
        ph_avg = {k: v / steps for k, v in ph_sum.items()}
        # parity: the device column against the written column, every byte
        got = gp.device_to_host(d)
        parity = {"rows": n, "bytes_equal": bool(
            np.array_equal(got.offsets, col.offsets.astype(np.int64)) and
            np.array_equal(got.data, col.data) and got.validity is None),
            "checked": "every offset and byte of the device column against the column written"}
        f.close()
        # roofline of the slowest device phase, by its algorithmic bytes
        vb, fb, pb = st["value_bytes"], st["file_bytes"], st["page_bytes"]
        alg = {"decompress": fb + pb,        # compressed pages read, raw pages written
               "decode": 41 * n,             # length word, validity, value spans (tmp + row)
               "values": 2 * vb + 28 * n}    # value bytes read + written, spans, offsets
        kernels = {"decompress": "k_snappy_frags (+ k_snappy_pages; host block index)",
                   "decode": "k_data_pages",
                   "values": "k_copy_values (+ k_offsets64)"}
        dom = max(alg, key=lambda k: ph_avg[k])
        hbm_peak, peak_kind = load_peaks()
        achieved = alg[dom] / (ph_avg[dom] * 1e-3) / 1e9
        # CPU: the oracle's reader (one thread) on the same file
        import oracle
        oracle.build(with_ref=False)
        t0 = time.perf_counter()
        o_off, o_data, o_valid = oracle.parquet_read(path)
        t_cpu = time.perf_counter() - t0
        cpu_equal = bool(np.array_equal(o_data, col.data) and o_valid.all())
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    return {
        "metric": "GeoParquet WKB column read to a device column (rows/s)",
        "value": n / (ms * 1e-3), "unit": "rows/s", "ms_per_step": ms, "steps": steps,
        "warmup": warmup,
        "phases_ms_per_step": ph_avg,
        "e2e": {"value": n / (e2e_ms * 1e-3), "unit": "rows/s", "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": int(fb), "d2h_bytes_per_step": 24,
                "open_ms": t_open * 1e3,
                "note": "SpjParquetReadWkb on an open file: chunk reads from the page cache "
                        "into page-locked memory, H2D, decode (the footer parse at open is "
                        "open_ms, once per file)"},
        "roofline": {"bound": "hbm", "kernel": kernels[dom], "achieved": achieved,
                     "peak": hbm_peak, "peak_kind": peak_kind, "unit": "GB/s",
                     "frac": achieved / hbm_peak, "traffic": None,
                     "algorithmic_bytes_per_launch": alg[dom]},
        "gpu_launches": 8 * steps,
        "parity": {**parity, "oracle_bytes_equal": cpu_equal},
        "cpu_baseline": {"value": n / t_cpu, "unit": "rows/s", "cores": 1, "kind": "port",
                         "sample": f"the whole file ({n} rows, {fb} bytes) read by the "
                                   "oracle's C Parquet reader on one thread"},
        "clocks": sampler.summary(),
        "config": {"workload": "geoparquet_read_2m_building_polygons_snappy_v1",
                   "rows": n, "file_bytes": int(fb), "page_bytes": int(pb),
                   "value_bytes": int(vb), "write_seconds": round(t_write, 2),
                   "l2": "column > L2, no flush"},
    }


def run_materialize(args, local):
    """Joined-batch materialisation on the device for the polygon workload's
    81M result pairs: the build and probe id columns (int64) and the probe
    WKB column gathered per pair, plus a left join's visited bitmap (mark,
    then collect the unmatched build rows).  The build WKB is not gathered
    (each pair would copy a ~2.3 KB zone: 190 GB); a query projecting it
    gathers it with the same call."""
    import torch
    from sedona_gpuspatial import capi
    from sedona_gpuspatial import materialize as mat
    inp = make_inputs(2, args.scale)
    join = capi.SpatialJoin()
    join.build(inp.build)
    dcol, keep = to_device(inp.probe)
    db, dp, npairs = join.probe_device(dcol, "intersects")
    torch.cuda.synchronize()
    bi = torch.as_tensor(_DevI32(db, npairs), device="cuda")
    pi = torch.as_tensor(_DevI32(dp, npairs), device="cuda")
    nb, npb = len(inp.build), len(inp.probe)
    build_ids = mat.DeviceColumn(nb, values=torch.arange(nb, dtype=torch.int64, device="cuda"))
    probe_ids = mat.DeviceColumn(npb, values=torch.arange(npb, dtype=torch.int64, device="cuda"))
    probe_wkb = mat.DeviceColumn(npb, offsets=keep[0], data=keep[1])
    steps, warmup = min(args.steps, 5), max(3, args.warmup)

    def step():
        cols = mat.build_joined_columns([build_ids], [probe_ids, probe_wkb], bi, pi)
        vb = mat.VisitedBitmap(nb)
        vb.mark(bi)
        un = vb.collect(False)
        return cols, un

    for _ in range(warmup):
        out = step()
        del out
    s = torch.cuda.current_stream()
    e0, e1, eb0, eb1 = (torch.cuda.Event(enable_timing=True) for _ in range(4))
    sampler = ClockSampler(local)
    bin_ms = 0.0
    with sampler:
        torch.cuda.synchronize()
        e0.record(s)
        for _ in range(steps):
            cols, un = step()
            if _ < steps - 1:
                del cols, un
        e1.record(s)
        torch.cuda.synchronize()
        for _ in range(steps):
            eb0.record(s)
            off, data = mat.take_binary(probe_wkb.offsets, probe_wkb.data, pi)
            eb1.record(s)
            torch.cuda.synchronize()
            bin_ms += eb0.elapsed_time(eb1)
            del off, data
    ms = e0.elapsed_time(e1) / steps
    bin_ms /= steps
    out_bytes = int(cols[2].data.numel())
    # parity: fixed columns exactly (torch gather), the binary column's
    # lengths exactly and 2000 sampled values byte for byte, the unmatched
    # build rows against a bincount
    ok_ids = bool(torch.equal(cols[0].values, bi.long()) and torch.equal(cols[1].values, pi.long()))
    poff = keep[0].long()
    lens = (poff[1:] - poff[:-1])[pi.long()]
    ok_len = bool(torch.equal(cols[2].offsets[1:] - cols[2].offsets[:-1], lens))
    rng = np.random.default_rng(20260301)
    sample = rng.integers(0, npairs, 2000)
    o = cols[2].offsets.cpu().numpy()
    pis = pi.cpu().numpy().view(np.uint32)
    ok_val = all(cols[2].data[o[i]:o[i + 1]].cpu().numpy().tobytes() == inp.probe.value(int(pis[i]))
                 for i in sample)
    seen = torch.bincount(bi.long(), minlength=nb) > 0
    ok_vis = bool(torch.equal(un.long(), torch.nonzero(~seen).flatten()))
    # roofline of the binary gather (k_bin_lengths + scan + k_bin_copy, run
    # twice by take_binary: a sizing call, then the copy): value bytes read
    # and written, per pair its index and the source offsets (12 B) and the
    # output offset (8 B), twice for the sizing pass
    alg = 2 * out_bytes + 2 * npairs * 20
    hbm_peak, peak_kind = load_peaks()
    achieved = alg / (bin_ms * 1e-3) / 1e9
    # CPU: numpy takes of the same columns over a sample of the pairs
    bnp, pnp = bi[:2_000_000].cpu().numpy().view(np.uint32), pis[:2_000_000]
    ids_b, ids_p = np.arange(nb, dtype=np.int64), np.arange(npb, dtype=np.int64)
    t0 = time.perf_counter()
    np.take(ids_b, bnp)
    np.take(ids_p, pnp)
    inp.probe.take(pnp.astype(np.int64))
    t_cpu = time.perf_counter() - t0
    del cols, un, join
    return {
        "metric": "joined-batch materialisation on the device (result pairs/s)",
        "value": npairs / (ms * 1e-3), "unit": "pairs/s", "ms_per_step": ms, "steps": steps,
        "warmup": warmup,
        "phases_ms_per_step": {"probe_wkb_take_binary": bin_ms},
        "roofline": {"bound": "hbm", "kernel": "k_bin_copy (+ k_bin_lengths, scan)",
                     "achieved": achieved, "peak": hbm_peak, "peak_kind": peak_kind,
                     "unit": "GB/s", "frac": achieved / hbm_peak, "traffic": None,
                     "algorithmic_bytes_per_launch": alg},
        "gpu_launches": 26 * steps,
        "parity": {"id_columns_equal": ok_ids, "wkb_lengths_equal": ok_len,
                   "wkb_sampled_values_equal": bool(ok_val), "unmatched_rows_equal": ok_vis,
                   "pairs": npairs},
        "cpu_baseline": {"value": len(bnp) / t_cpu, "unit": "pairs/s", "cores": 1,
                         "kind": "port",
                         "sample": f"numpy takes (build ids, probe ids, probe WKB) for the "
                                   f"first {len(bnp)} pairs"},
        "clocks": sampler.summary(),
        "config": {"workload": "materialize_2m_buildings_x_50k_zones_result_pairs",
                   "pairs": npairs, "probe_wkb_bytes_out": out_bytes,
                   "columns": "build id (int64), probe id (int64), probe WKB; visited bitmap",
                   "l2": "columns > L2, no flush"},
    }


def run_outofcore(args, local):
    """The partitioned (out-of-core) join on the learned-index workload's
    data: its 100M points are the build side, held in host memory and split
    into KDB partitions by a device budget of a quarter of their decoded
    size, and its 10M boxes probe every partition they meet (ST_Intersects).
    value: pairs/s of SpjJoinPartitioned from the host columns to the pairs
    on the host (its inputs live in host memory by design, so value and e2e
    coincide); the one-pass join of the same host columns is timed beside it."""
    from types import SimpleNamespace

    import torch
    from sedona_gpuspatial import capi, datagen
    n_build = int(100_000_000 * args.scale)
    n_boxes = int(10_000_000 * args.scale)
    build, probe, _, _ = datagen.workload5(n_build=n_build, n_boxes=n_boxes, n_lookups=1)
    budget = int(build.nbytes * 5 // 2 // 4)
    steps, warmup = min(args.steps, 3), 1
    j = capi.SpatialJoin(profile=True)
    for _ in range(warmup):
        j.join_partitioned(build, probe, "intersects", build_budget_bytes=budget, seed=1)
    j.reset_stats()
    sampler = ClockSampler(local)
    wall = 0.0
    with sampler:
        for _ in range(steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            b, p, st = j.join_partitioned(build, probe, "intersects", build_budget_bytes=budget,
                                          seed=1)
            wall += time.perf_counter() - t0
    ms = wall * 1e3 / steps
    js = j.stats()
    npairs = len(b)
    # parity: the same pair set as the one-pass join of the same host columns
    one = capi.SpatialJoin()
    t0 = time.perf_counter()
    one.build(build)
    ob, op = one.probe(probe, "intersects")
    one_ms = (time.perf_counter() - t0) * 1e3
    keys = np.sort(p.astype(np.uint64) * np.uint64(n_build) + b.astype(np.uint64))
    okeys = np.sort(op.astype(np.uint64) * np.uint64(n_build) + ob.astype(np.uint64))
    parity = {"pairs": npairs, "pairs_equal_one_pass": bool(np.array_equal(keys, okeys)),
              "unique": bool(len(keys) == 0 or (np.diff(keys) > 0).all()),
              "checked": "sorted pair set against the one-pass GPU join of the same columns"}
    del ob, op, okeys
    sample = np.random.default_rng(20260301).integers(0, max(1, npairs), 2000)
    import oracle
    oracle.build(with_ref=False)
    G = oracle.Geoms(probe.take(p[sample].astype(np.int64)))
    Bg = oracle.Geoms(build.take(b[sample].astype(np.int64)))
    parity["sampled_pairs_hold_in_oracle"] = bool(all(
        oracle.predicate(Bg, i, G, i, "intersects") == 1 for i in range(len(sample))))
    # roofline: the refine over all passes (point-in-box tests: per candidate
    # the two ids, the probe ring's 5 vertices and the build point)
    hbm_peak, peak_kind = load_peaks()
    cand = js["candidates"] / steps
    ref_bytes = cand * (8 + 16 * 5 + 16 + 1)
    ref_ms = js["ms_refine"] / steps
    achieved = ref_bytes / (ref_ms * 1e-3) / 1e9 if ref_ms > 0 else 0.0
    cpu = cpu_baseline(SimpleNamespace(build=build, probe=probe, predicate="intersects",
                                       params={}), seconds_budget=args.config_ref_seconds)
    return {
        "metric": "partitioned join pairs/s from host columns (build side in KDB partitions)",
        "value": npairs / (ms * 1e-3), "unit": "pairs/s", "ms_per_step": ms, "steps": steps,
        "warmup": warmup,
        "phases_ms_per_step": {"boxes": st["ms_boxes"], "partition": st["ms_partition"],
                               "passes": st["ms_passes"],
                               "refine_device": js["ms_refine"] / steps,
                               "filter_device": js["ms_filter"] / steps,
                               "decode_device": js["ms_decode"] / steps},
        "partitions": {k: st[k] for k in ("partitions", "passes", "build_rows_max",
                                          "probe_rows_multi", "probe_rows_none",
                                          "probe_rows_probed", "direct_host_reads")},
        "one_pass_e2e_ms": one_ms,
        "e2e": {"value": npairs / (ms * 1e-3), "unit": "pairs/s", "ms_per_step": ms,
                "h2d_bytes_per_step": int(build.nbytes + probe.nbytes),
                "d2h_bytes_per_step": int(8 * npairs),
                "note": "both columns in host memory; every pass reads its rows from there"},
        "roofline": {"bound": "hbm", "kernel": "k_refine<fast> (all passes)",
                     "achieved": achieved, "peak": hbm_peak, "peak_kind": peak_kind,
                     "unit": "GB/s", "frac": achieved / hbm_peak, "traffic": None,
                     "algorithmic_bytes_per_launch": ref_bytes},
        "gpu_launches": int(js["kernel_launches"] / max(1, steps)),
        "parity": parity,
        "cpu_baseline": cpu,
        "clocks": sampler.summary(),
        "config": {"workload": "outofcore_100m_points_build_x_10m_boxes_probe_kdb_partitions",
                   "build_rows": n_build, "probe_rows": n_boxes, "build_budget_bytes": budget,
                   "predicate": "intersects", "l2": "columns > L2, no flush"},
    }


class _DevI32:
    def __init__(self, ptr, n):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": "<i4", "data": (ptr, False),
                                         "version": 3, "strides": None}


NESTED_KEYS = ("value", "unit", "ms_per_step", "steps", "warmup", "probe_rows_per_s",
               "partitions", "one_pass_e2e_ms",
               "plain_f64_form", "phases_ms_per_step", "fp64_escalated_fraction",
               "fp64_escalations_per_replay", "roofline", "e2e", "gpu_launches", "parity",
               "knn", "learned_index", "lbvh_fast_form", "per_batch_calls_f32_ms", "clocks",
               "config")


def run_configs(args, world, rank, local, pg, names):
    """One entry per workload beside the headline (fewer steps, no option
    variants): its own timing, plain FP64 form, roofline, e2e, parity of the
    full-size run and CPU baseline."""
    import copy

    import torch
    res = {}
    for name in names:
        a = copy.copy(args)
        a.steps, a.warmup = min(args.steps, 3), min(args.warmup, 2)
        t0 = time.perf_counter()
        pred = None
        if name == "1":
            out, inp = run_ours(a, world, rank, local, pg, light=True, workload=1)
        elif name == "2contains":
            pred = "contains"
            out, inp = run_ours(a, world, rank, local, pg, light=True, workload=2,
                                pred_override="contains")
        elif name == "3":
            a.workload = 3
            out, inp = run_stream(a, world, rank, local, pg)
        elif name == "4":
            out, inp = run_ours(a, world, rank, local, pg, light=True, workload=4)
        elif name == "5":
            a.workload = 5
            out, inp = run_learned(a, world, rank, local, pg)
        elif name == "geoparquet":
            out, inp = run_geoparquet(a, local), None
        elif name == "materialize":
            out, inp = run_materialize(a, local), None
        elif name == "outofcore":
            out, inp = run_outofcore(a, local), None
        else:
            raise SystemExit(f"unknown config {name}")
        entry = {k: out[k] for k in NESTED_KEYS + ("metric", "cpu_baseline") if k in out}
        if rank == 0 and not args.no_cpu_baseline and inp is not None:
            entry["cpu_baseline"] = cpu_baseline(inp, seconds_budget=args.config_ref_seconds,
                                                 pred=pred)
        entry["seconds"] = round(time.perf_counter() - t0, 1)
        res[out["config"]["workload"]] = entry
        if rank == 0:
            print(f"[bench] {out['config']['workload']}: {entry['ms_per_step']:.2f} ms/step, "
                  f"parity {entry.get('parity', {}).get('pairs_equal')}, "
                  f"{entry['seconds']} s", file=sys.stderr, flush=True)
        del out, inp
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--plain-steps", type=int, default=2)
    ap.add_argument("--workload", type=int, default=2)
    ap.add_argument("--scale", type=float, default=1.0)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--ref-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-parity", dest="parity", action="store_false",
                    help="skip the parity check of the full-size run against the oracle")
    ap.add_argument("--configs", default="1,2contains,3,4,5,geoparquet,materialize,outofcore",
                    help="workload entries timed beside the headline (empty: none)")
    ap.add_argument("--config-ref-seconds", type=float, default=5.0)
    ap.add_argument("--join-options", type=json.loads, default={},
                    help='execution options of the chosen form, e.g. \'{"refine_min_blocks": 6}\'')
    args = ap.parse_args()
    world, rank, local, pg = (1, 0, 0, None)
    if args.impl == "reference":
        world = int(os.environ.get("WORLD_SIZE", "1"))
        rank = int(os.environ.get("RANK", "0"))
        out = run_reference(args, world, rank)
        if out is not None:
            print(json.dumps(out))
        return
    world, rank, local, pg = dist_setup()
    if args.workload == 3:
        out, inp = run_stream(args, world, rank, local, pg)
    elif args.workload == 5:
        out, inp = run_learned(args, world, rank, local, pg)
    else:
        out, inp = run_ours(args, world, rank, local, pg)
    if rank == 0 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(inp, seconds_budget=args.ref_seconds)
    if rank == 0:
        print(f"[bench] headline: {out['ms_per_step']:.2f} ms/step, parity "
              f"{out.get('parity', {}).get('pairs_equal')}", file=sys.stderr, flush=True)
    del inp
    names = [c for c in args.configs.split(",") if c] if args.workload == 2 else []
    if names:
        import torch
        torch.cuda.empty_cache()
        out["configs"] = run_configs(args, world, rank, local, pg, names)
    if rank == 0:
        out.pop("_", None)
        print(json.dumps(out))
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
