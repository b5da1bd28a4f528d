"""FindNccModel throughput on one GB300 (or N replicas under torchrun).

Workload "find_2048_t128_5x": 2048x2048 uint8 scenes, one 128x128 template
pasted at 5 poses each (rotation U[-30 deg, 30 deg], sub-pixel shifts), model
AngleStart -30 deg, AngleExtent 60 deg, automatic angle step, NumLevels 4;
FindNccModel MinScore 0.7, NumMatches 5, MaxOverlap 0.5, SubPixel true.
A step is one find on each of `--batch` distinct scenes.

value: images/s with the scenes resident in HBM, through the batched operator
(mvg_find_ncc_models_batch: 32 finds in flight on the library's host
threads, each launching its own kernels; --cohorts k merges their
tensor-core launches), CUDA events around each step's call, L2 flushed
between steps.  e2e: the same calls on page-locked host images, wall clock
around each step (upload, the finds and the result read-back inside the
timed region).  roofline: the correlation kernel's algorithmic
multiply-adds over its event time in a profiled pass of the same steps
(per-find stage events on the find streams), or over the merged launches'
event time when the value pass merges; beside it the other launch policy
and the same finds one at a time.
cpu_baseline: the FP64 oracle restatement of the reference on this host's
cores (one scene per thread); its matches are the parity check of the value
pass's poses.

--impl reference: the reference's CPU implementation of the path (the oracle
port here; the reference itself when it was compiled on this machine), all
host threads, one scene per thread per step.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import re
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

D = math.radians
WORKLOAD = "find_2048_t128_5x"
GEN = dict(height=2048, width=2048, tsize=128, n_poses=5, angle_range=(-D(30), D(30)))
CREATE = dict(num_levels=4, angle_start=-D(30), angle_extent=D(60), angle_step="auto", metric="use_polarity")
FIND = dict(angle_start=-D(30), angle_extent=D(60), min_score=0.7, num_matches=5, max_overlap=0.5, subpixel="true",
            num_levels=4)
METRIC = "FindNccModel images/s at <=0.05px/0.05deg pose error; tensor-core vs plain GPU"


def peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return dict(hbm=d["hbm_gbs"], tflops=d["bf16_tflops"], tflops_sustained=d["bf16_tflops_sustained"],
                    source="measured")
    return dict(hbm=6800.0, tflops=1900.0, tflops_sustained=1700.0, source="fallback")


def scenes(n: int, template_seed: int = 1):
    """n distinct seeded scenes sharing one template (generated on host threads)."""
    from concurrent.futures import ThreadPoolExecutor

    from mvkit_gb300 import workloads as W
    with ThreadPoolExecutor(max(1, min(n, os.cpu_count() or 1))) as ex:
        return list(ex.map(lambda i: W.make_workload(1000 + i, template_seed=template_seed, **GEN), range(n)))


class ClockSampler:
    """nvidia-smi clock/throttle samples while running (20 ms period)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def traffic_from_profiles(kernel: str):
    """DRAM bytes per launch recorded by the committed ncu summary, if any."""
    for p in sorted((ROOT / "profiles").glob(f"{kernel}*.md")):
        m = re.search(r"dram_bytes_per_launch:\s*([0-9.eE+]+)", p.read_text())
        if m:
            return float(m.group(1))
    return None


def cpu_baseline(images, threads: int):
    """The oracle on this host's cores, one scene per thread (the first
    `threads` scenes); returns the baseline and each scene's matches."""
    from concurrent.futures import ThreadPoolExecutor

    import oracle_lib
    orc = oracle_lib.oracle()
    wl = images[0]
    model = orc.create(wl.template, levels=CREATE["num_levels"], angle_start=CREATE["angle_start"],
                       angle_extent=CREATE["angle_extent"])
    sample = [images[i % len(images)].image for i in range(threads)]

    def one(im):  # the ctypes call releases the GIL: the finds run in parallel
        return orc.find(model, im, FIND["angle_start"], FIND["angle_extent"], FIND["min_score"],
                        FIND["num_matches"], FIND["max_overlap"], True, 4, 1)

    with ThreadPoolExecutor(threads) as ex:
        t0 = time.perf_counter()
        results = list(ex.map(one, sample))
        dt = time.perf_counter() - t0
    n = sum(len(r) for r in results)
    base = {"value": len(sample) / dt, "unit": "images/s", "cores": threads, "kind": "port",
            "sample": f"{len(sample)} scenes of {WORKLOAD}, one per thread, FP64 oracle restatement "
                      f"of the reference scalar path ({n} matches)", "seconds": dt}
    return base, [oracle_lib.to_halcon(r) for r in results[:min(threads, len(images))]]


def halcon(row, col, angle):
    """The operator's edge-centred pose of a matcher pose (ncc_matching_api.cpp:171-176)."""
    c, s = math.cos(angle), math.sin(angle)
    return row + .5 * (1 - c + s), col + .5 * (1 - c - s)


def pose_error(found, images, oracle=None) -> dict:
    """Pose errors of the timed finds: against each scene's pasted poses (the
    generator's ground truth, nearest match per pose) and, on the oracle's
    sample, against the FP64 oracle (same count and order required)."""
    dr, dc, da, missing = [], [], [], 0
    for (rows, cols, angles, scores), wl in zip(found, images):
        got = np.stack([rows, cols, angles], axis=1) if len(rows) else np.zeros((0, 3))
        for p in wl.poses:
            r, c = halcon(p.row, p.column, p.angle)
            if not len(got):
                missing += 1
                continue
            k = int(np.argmin(np.hypot(got[:, 0] - r, got[:, 1] - c)))
            if math.hypot(got[k, 0] - r, got[k, 1] - c) > 2.0:
                missing += 1
                continue
            dr.append(abs(got[k, 0] - r))
            dc.append(abs(got[k, 1] - c))
            da.append(abs(math.degrees(got[k, 2] - p.angle)))
    out = {"vs_truth": {"scenes": len(images), "poses": sum(len(w.poses) for w in images), "unmatched": missing,
                        "max_drow": max(dr, default=None), "max_dcol": max(dc, default=None),
                        "max_dangle_deg": max(da, default=None),
                        "note": "nearest match per pasted pose: the NCC optimum of a noisy bilinear paste lies "
                                "off the pasted pose, for the FP64 oracle as well (oracle_on_its_sample)"}}
    if oracle is not None:
        o = pose_error([(r[:, 0], r[:, 1], r[:, 2], r[:, 3]) for r in oracle], images[:len(oracle)])["vs_truth"]
        out["vs_truth"]["oracle_on_its_sample"] = {k: o[k] for k in ("scenes", "unmatched", "max_drow", "max_dcol",
                                                                     "max_dangle_deg")}
    if oracle is not None:
        same, d = True, np.zeros(4)
        for (rows, cols, angles, scores), want in zip(found, oracle):
            got = np.stack([rows, cols, angles, scores], axis=1) if len(rows) else np.zeros((0, 4))
            if got.shape != want.shape:
                same = False
                continue
            if len(got):
                d = np.maximum(d, np.abs(got - want).max(axis=0))
        out["vs_oracle"] = {"scenes": len(oracle), "count_and_order_equal": same, "max_drow": float(d[0]),
                            "max_dcol": float(d[1]), "max_dangle_deg": math.degrees(float(d[2])),
                            "max_dscore": float(d[3]),
                            "within_tolerance": bool(same and d[0] <= .05 and d[1] <= .05 and
                                                     math.degrees(d[2]) <= .05 and d[3] <= 1e-4)}
    return out


def same_results(a, b) -> bool:
    """Two passes' per-scene (Row, Column, Angle, Score) are bit-identical."""
    return bool(len(a) == len(b) and
                all(all(np.array_equal(u, v) for u, v in zip(x[:4], y[:4])) for x, y in zip(a, b)))


def max_over_ranks(x: float, device: str = "cuda") -> float:
    """The largest x over the replicas (all-reduce MAX); x itself on one."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return x
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(images_per_rank: int, world: int, slowest_ms: float) -> float:
    """Whole-job images/s: every replica's images over the slowest replica's time."""
    return images_per_rank * world / (slowest_ms / 1e3)


def run_reference(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    images = scenes(min(threads, 8))
    import oracle_lib
    orc = oracle_lib.oracle()
    model = orc.create(images[0].template, levels=4, angle_start=CREATE["angle_start"],
                       angle_extent=CREATE["angle_extent"])
    sample = [images[i % len(images)].image for i in range(threads)]

    def step():
        return orc.find_many(model, sample, threads, FIND["angle_start"], FIND["angle_extent"], FIND["min_score"],
                             FIND["num_matches"], FIND["max_overlap"], True, 4, 1)

    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    dt = time.perf_counter() - t0
    value = args.steps * len(sample) / dt
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "images/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "scenes_per_step": len(sample), "threads": threads},
            "cpu_baseline": {"value": value, "unit": "images/s", "cores": threads, "kind": "port",
                             "sample": f"{len(sample)} scenes per step, one per host thread"},
            "e2e": {"value": value, "unit": "images/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# The other configurations at their stated sizes, run in extended mode (the
# reference refuses them under its budgets).  Selected with --workload; the
# headline line stays find_2048_t128_5x.
FULL_CIRCLE = (-math.pi, 2 * math.pi)
CONFIG_WORKLOADS = {
    # 64 scenes of sizes {512x512, 1280x1024, 2448x2048, 4096x3000}, 8 templates
    # {32..256}^2 each pasted 1-10 times over a full circle (as many as fit
    # without overlap on the smaller scenes), contrast +-10 %, noise sigma 5;
    # automatic levels, MinScore 0.6, NumMatches 10 per template (at most 10
    # pastes), MaxOverlap 0.5.  A step searches the batch once per template
    # (one single-model batched call each, selection on the device): a
    # FindNccModels with per-model quotas selects on the host and refines
    # candidate after candidate until every quota is met
    "batch_64_t32_256_360": dict(
        kind="batch", gen=dict(seed=3, n_images=64, sizes=((512, 512), (1024, 1280), (2048, 2448), (3000, 4096)),
                               tsizes=(32, 48, 64, 96, 128, 160, 192, 256), max_pastes=10,
                               angle_range=(-math.pi, math.pi), contrast=0.1, noise_sigma=5, fit=True),
        levels="auto", find=(FULL_CIRCLE[0], FULL_CIRCLE[1], 0.6, 10, 0.5, "true", 0), per_model=True,
        budgets=dict(samples=600_000_000, pixels=1 << 30, candidates=1 << 21), workers=8),
    # 5120x5120 uint8, 4 templates {128, 160, 192, 256}^2 pasted at 256 poses
    # (subpixel row/column, angle U[0, 360 deg), scale U[0.95, 1.05]): a
    # full-circle FindNccModels (rigid, the reference's refinement) and the
    # adjoint-driven Gauss-Newton on (row, column, angle, scale) from its
    # poses; the quadratic peak fit of the discrete poses beside them
    "similarity_5120_t128_256_256x": dict(
        kind="similarity", gen=dict(seed=7, height=5120, width=5120, tsizes=(128, 160, 192, 256), n_poses=256),
        levels=4, find=(FULL_CIRCLE[0], FULL_CIRCLE[1], 0.4, [64] * 4, 0.5, "true", 4),
        budgets=dict(samples=600_000_000, pixels=1 << 30, candidates=1 << 21), workers=1),
    # 8192x8192 uint16 (12-bit, noise sigma 20), one 512^2 template pasted 20
    # times over a full circle; NumLevels 6, MinScore 0.5, NumMatches 20,
    # MaxOverlap 0.3
    "u16_8192_t512_20x": dict(
        kind="single", gen=dict(height=8192, width=8192, tsize=512, n_poses=20, angle_range=(-math.pi, math.pi),
                                maxval=4095, noise_sigma=20),
        scenes=2, levels=6, find=(FULL_CIRCLE[0], FULL_CIRCLE[1], 0.5, 20, 0.3, "true", 6),
        budgets=dict(samples=600_000_000, pixels=1 << 30, candidates=1 << 18), workers=2),
}


def run_config(args) -> None:
    """One configuration workload: a step is the whole batch (or the scenes)
    through the batched operator in extended mode; value with the images in
    HBM (CUDA events around each call), e2e from page-locked host images
    (wall clock); roofline of the tensor-core correlation from a profiled
    pass on per-find host threads; pose error against the pasted poses;
    cpu_baseline: the FP64 oracle with the same budgets on a sample."""
    import torch
    import mvkit_gb300 as mg
    from mvkit_gb300 import build
    from mvkit_gb300 import workloads as W

    cfg = CONFIG_WORKLOADS[args.workload]
    if cfg["kind"] == "similarity":
        run_similarity(args, cfg)
        return
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    procs = max(1, min(16, os.cpu_count() or 1))
    t_gen = time.perf_counter()
    if cfg["kind"] == "batch":
        scenes_ = W.make_batch_workloads(**cfg["gen"], processes=procs)
        templates = scenes_[0].templates
        truth = [[(k, p) for k, ps in enumerate(s_.poses) for p in ps] for s_ in scenes_]
    else:
        scenes_ = [W.make_workload(5000 + i, template_seed=5000, **cfg["gen"]) for i in range(cfg["scenes"])]
        templates = [scenes_[0].template]
        assert all(np.array_equal(x.template, templates[0]) for x in scenes_)
        truth = [[(0, p) for p in s_.poses] for s_ in scenes_]
    t_gen = time.perf_counter() - t_gen
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    build.build()
    mg.load()
    mg.set_budgets(**cfg["budgets"])
    t0 = time.perf_counter()
    models = [mg.create_ncc_model(t, cfg["levels"], FULL_CIRCLE[0], FULL_CIRCLE[1], "auto", "use_polarity")
              for t in templates]
    t_models = time.perf_counter() - t0
    images = [x.image for x in scenes_]
    dev = [mg.DeviceImage(im) for im in images]
    pinned, pinned_bufs = [], []  # the buffers own the page-locked memory the arrays view
    for im in images:
        pb = mg.PinnedBuffer(im.shape, im.dtype)
        pb.array[...] = im
        pinned_bufs.append(pb)
        pinned.append(pb.array)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    workers = min(cfg["workers"], len(images))
    st = torch.cuda.Stream()

    def step(imgs):
        if not cfg.get("per_model"):
            return mg.find_ncc_models_batch(imgs, models, *cfg["find"], workers=workers, raise_errors=False)
        # one batched call per model; image i's matches of every model, model
        # index k (a failed image keeps its first error)
        per = [mg.find_ncc_models_batch(imgs, [m], *cfg["find"], workers=workers, raise_errors=False)
               for m in models]
        out = []
        for i in range(len(imgs)):
            errs = [p_[i] for p_ in per if isinstance(p_[i], mg.MvError)]
            if errs:
                out.append(errs[0])
                continue
            parts = [p_[i] for p_ in per]
            out.append(tuple(np.concatenate([q[j] for q in parts]) for j in range(4)) +
                       (np.concatenate([np.full(len(q[0]), k, np.int64) for k, q in enumerate(parts)]),))
        return out

    def timed(imgs, events: bool):
        total, out = 0.0, None
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            if world > 1:
                torch.distributed.barrier()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            w0 = time.perf_counter()
            e0.record(st)
            out = step(imgs)
            e1.record(st)
            torch.cuda.synchronize()
            total += e0.elapsed_time(e1) if events else (time.perf_counter() - w0) * 1e3
        return total, out

    for _ in range(args.warmup):
        step(dev)
    step(pinned)
    with ClockSampler(local) as clocks:
        dev_ms, found = timed(dev, True)
    host_ms, found_host = timed(pinned, False)

    # per-find host threads with stage events: one find per scene per model
    from concurrent.futures import ThreadPoolExecutor

    def prof_worker(j):
        torch.cuda.set_device(local)
        mg.set_budgets(**cfg["budgets"])
        mg.profile_reset()
        mg.profile_enable(True)
        for im in dev[j::workers]:
            for m in models:
                mg.find_ncc_model(im, m, *cfg["find"])
        mg.profile_enable(False)
        return mg.profile_read()

    with ThreadPoolExecutor(workers) as ex:
        profs = list(ex.map(prof_worker, range(workers)))
    stages, finds = {}, 0
    for p_ in profs:
        finds += p_["finds"]
        for k, v in p_.items():
            if isinstance(v, dict):
                acc = stages.setdefault(k, dict(ms=0.0, launches=0, work=0.0))
                for f in ("ms", "launches", "work"):
                    acc[f] += v[f]
    if world > 1:
        dev_ms, host_ms = max_over_ranks(dev_ms), max_over_ranks(host_ms)
    value = replica_value(args.steps * len(images), world, dev_ms)
    e2e = replica_value(args.steps * len(images), world, host_ms)
    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return
    pk = peaks()
    tc = stages.get("track_tc", {"ms": 0.0, "work": 0.0, "launches": 0})
    cc = stages.get("track", {"ms": 0.0, "work": 0.0, "launches": 0})
    on_tc = tc["work"] > 0
    d = tc if on_tc else cc
    ach = 2.0 * d["work"] / (d["ms"] / 1e3) / 1e12 if d["ms"] else None
    roof = {"bound": "tensor", "achieved": ach, "peak": pk["tflops_sustained"], "unit": "TFLOP/s",
            "frac": ach / pk["tflops_sustained"] if ach else None, "traffic": None,
            "kernel": "tc_track_kernel" if on_tc else "track_kernel",
            "ms_per_launch": d["ms"] / max(1, d["launches"]),
            "cuda_core_tracking": {"achieved": 2.0 * cc["work"] / (cc["ms"] / 1e3) / 1e12 if cc["ms"] else None,
                                   "algorithmic_macs": cc["work"], "ms": cc["ms"]},
            "tensor_core_tracking": {"achieved": 2.0 * tc["work"] / (tc["ms"] / 1e3) / 1e12 if tc["ms"] else None,
                                     "algorithmic_macs": tc["work"], "ms": tc["ms"]},
            "note": f"profiled pass: one find per scene and model on {workers} host threads, algorithmic "
                    f"correlation FLOPs over the kernel's event time; peak = {pk['source']} dense bf16 sustained"
                    + ("" if on_tc else "; no tracking group of this workload is on the tensor cores (uint16 "
                       "levels above 1, level windows beyond shared memory): the FP32 CUDA-core tracking "
                       "kernel, against the tensor peak for comparison")}
    # pose error against the pasted poses: nearest match of the paste's model
    failed = [(i, r.status, r.message) for i, r in enumerate(found) if isinstance(r, mg.MvError)]
    dr, dc, da, unmatched = [], [], [], 0
    for res, tr in zip(found, truth):
        if isinstance(res, mg.MvError):
            unmatched += len(tr)
            continue
        rows, cols, angles, _, mids = res
        for k, p in tr:
            r, c = halcon(p.row, p.column, p.angle)
            sel = np.nonzero(mids == k)[0]
            if not len(sel):
                unmatched += 1
                continue
            dist_ = np.hypot(rows[sel] - r, cols[sel] - c)
            j = sel[int(np.argmin(dist_))]
            if dist_.min() > 2.0:
                unmatched += 1
                continue
            dr.append(abs(rows[j] - r))
            dc.append(abs(cols[j] - c))
            da.append(abs(math.degrees(math.remainder(angles[j] - p.angle, 2 * math.pi))))
    pose = {"vs_truth": {"poses": sum(len(t) for t in truth), "unmatched": unmatched,
                         "max_drow": max(dr, default=None), "max_dcol": max(dc, default=None),
                         "max_dangle_deg": max(da, default=None),
                         "median_drow": float(np.median(dr)) if dr else None,
                         "median_dcol": float(np.median(dc)) if dc else None},
            "e2e_equals_value_pass": same_results([r for r in found_host if not isinstance(r, mg.MvError)],
                                                  [r for r in found if not isinstance(r, mg.MvError)]),
            "failed_images": failed}
    line = {
        "metric": METRIC, "value": value, "unit": "images/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u16" if images[0].dtype == np.uint16 else "u8", "data": "synthetic",
        "config": {"workload": args.workload, "images_per_step": len(images), "templates": [t.shape[0] for t in templates],
                   "controls": list(cfg["find"]), "num_levels": cfg["levels"], "budgets": cfg["budgets"],
                   "mode": "extended (the reference's budgets lifted)", "finds_in_flight": workers,
                   "l2": "flushed (256 MiB write) between steps", "parallelism": f"replicas x{world}",
                   "generation_s": round(t_gen, 1), "model_build_s": round(t_models, 2)},
        "e2e": {"value": e2e, "unit": "images/s", "h2d_bytes_per_step": int(sum(im.nbytes for im in images)),
                "d2h_bytes_per_step": int(sum(5 * 8 * len(r[0]) + 16 for r in found if not isinstance(r, mg.MvError))),
                "api": "find_ncc_models_batch on pinned host images; wall clock per step"},
        "roofline": roof,
        "gpu_launches": int(sum(v["launches"] for v in stages.values()) * args.steps),
        "clocks": clocks.summary(),
        "matches_per_image": [None if isinstance(r, mg.MvError) else len(r[0]) for r in found],
        # event time per stage, summed over the profiled pass's finds on all
        # its host threads (finds overlap, so the sum exceeds a step's time)
        "stages_ms_profiled_pass": {k: round(v["ms"], 1) for k, v in stages.items()},
        "profiled_finds": finds,
        "pose_error": pose,
    }
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = config_cpu_baseline(cfg, scenes_, templates)
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def matcher_pose(r, c, a):
    """The matcher's pixel-centre pose of the operator's edge-centred one."""
    ca, sa = np.cos(a), np.sin(a)
    return r - .5 * (1 - ca + sa), c - .5 * (1 - ca - sa)


def similarity_errors(poses, model_of, truth) -> dict:
    """Pose errors against the pasted similarity poses (nearest pose of the
    paste's model within 3 px): median and max per degree of freedom, and the
    share within 0.05 px (row and column) and 0.05 deg."""
    err, missing = [], 0
    for t in truth:
        sel = np.nonzero(model_of == t.model)[0]
        d = np.hypot(poses[sel, 0] - t.row, poses[sel, 1] - t.column) if len(sel) else np.zeros(0)
        if not len(sel) or d.min() > 3:
            missing += 1
            continue
        p = poses[sel[int(np.argmin(d))]]
        err.append((abs(p[0] - t.row), abs(p[1] - t.column), abs(math.degrees(math.remainder(p[2] - t.angle,
                                                                                                 2 * math.pi))),
                    abs(p[3] - t.scale)))
    e = np.array(err) if err else np.zeros((0, 4))
    names = ("row_px", "col_px", "angle_deg", "scale")
    return {"found": len(err), "missing": missing,
            "median": dict(zip(names, np.median(e, axis=0).tolist())) if len(e) else None,
            "max": dict(zip(names, e.max(axis=0).tolist())) if len(e) else None,
            "within_0.05px_0.05deg": float(np.mean((e[:, 0] <= .05) & (e[:, 1] <= .05) & (e[:, 2] <= .05)))
            if len(e) else None}


def run_similarity(args, cfg) -> None:
    """The differentiable-refinement configuration: a step is the full-circle
    FindNccModels of the scene (extended mode) plus the adjoint Gauss-Newton
    refinement of every match; pose errors of the rigid, quadratic-fit and
    adjoint forms against the pasted poses."""
    import torch
    import mvkit_gb300 as mg
    from mvkit_gb300 import build
    from mvkit_gb300 import workloads as W

    local = int(os.environ.get("LOCAL_RANK", "0"))
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    t0 = time.perf_counter()
    wl = W.make_similarity_workload(**cfg["gen"])
    t_gen = time.perf_counter() - t0
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    build.build()
    mg.load()
    mg.set_budgets(**cfg["budgets"])
    t0 = time.perf_counter()
    models = [mg.create_ncc_model(t, cfg["levels"], FULL_CIRCLE[0], FULL_CIRCLE[1], "auto", "use_polarity")
              for t in wl.templates]
    t_models = time.perf_counter() - t0
    dev = mg.DeviceImage(wl.image)
    pb = mg.PinnedBuffer(wl.image.shape, np.uint8)
    pb.array[...] = wl.image
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    f = cfg["find"]
    st = torch.cuda.Stream()

    def step(img, subpixel="true"):
        r, c, a, sc, m = mg.find_ncc_models(img, models, f[0], f[1], f[2], f[3], f[4], subpixel, f[6])
        mr, mc = matcher_pose(r, c, a)
        poses = np.stack([mr, mc, a, np.ones_like(a)], axis=1)
        refined = poses.copy()
        for k, model in enumerate(models):
            if (m == k).any():
                refined[m == k], _ = mg.ncc_refine_similarity(img, model, poses[m == k], iterations=40)
        return poses, refined, m

    def timed(img, events):
        total, out = 0.0, None
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            w0 = time.perf_counter()
            e0.record(st)
            out = step(img)
            e1.record(st)
            torch.cuda.synchronize()
            total += e0.elapsed_time(e1) if events else (time.perf_counter() - w0) * 1e3
        return total, out

    for _ in range(args.warmup):
        step(dev)
    step(pb.array)
    with ClockSampler(local) as clocks:
        dev_ms, (rigid, adjoint, m) = timed(dev, True)
    host_ms, (rigid_h, adjoint_h, _) = timed(pb.array, False)
    # the quadratic peak fit of the discrete (SubPixel "false") poses
    r, c, a, _, md = mg.find_ncc_models(dev, models, f[0], f[1], f[2], f[3], f[4], "false", f[6])
    mr, mc = matcher_pose(r, c, a)
    discrete = np.stack([mr, mc, a, np.ones_like(a)], axis=1)
    quad = discrete.copy()
    for k, model in enumerate(models):
        if (md == k).any():
            quad[md == k], _ = mg.ncc_quadratic_peak_fit(dev, model, discrete[md == k],
                                                         (1.0, 1.0, mg.get_ncc_model_params(model)[3], 0.02))
    # stage profile of the finds (one per model) on this thread
    mg.profile_reset()
    mg.profile_enable(True)
    for model in models:
        mg.find_ncc_model(dev, model, f[0], f[1], f[2], f[3][0], f[4], "true", f[6])
    mg.profile_enable(False)
    prof = mg.profile_read()
    if rank != 0:
        return
    pk = peaks()
    tc = prof.get("track_tc", {"ms": 0.0, "work": 0.0, "launches": 0})
    ach = 2.0 * tc["work"] / (tc["ms"] / 1e3) / 1e12 if tc["ms"] else None
    value = replica_value(args.steps, world, dev_ms)
    line = {
        "metric": METRIC, "value": value, "unit": "images/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": {"workload": args.workload, "image": f"{wl.image.shape[1]}x{wl.image.shape[0]} u8",
                   "templates": [t.shape[0] for t in wl.templates], "poses": len(wl.poses),
                   "controls": list(f), "num_levels": cfg["levels"], "budgets": cfg["budgets"],
                   "mode": "extended (the reference's budgets lifted)",
                   "step": "FindNccModels (rigid Gauss-Newton) + adjoint Gauss-Newton on (row, column, angle, "
                           "scale) of every match, 40 iterations at most",
                   "l2": "flushed (256 MiB write) between steps", "generation_s": round(t_gen, 1),
                   "model_build_s": round(t_models, 2)},
        "e2e": {"value": replica_value(args.steps, world, host_ms), "unit": "images/s",
                "h2d_bytes_per_step": int(2 * wl.image.nbytes),
                "d2h_bytes_per_step": int(len(rigid) * 8 * 9),
                "api": "find_ncc_models and ncc_refine_similarity on the page-locked host image (each call "
                       "uploads it); wall clock per step"},
        "roofline": {"bound": "tensor", "achieved": ach, "peak": pk["tflops_sustained"], "unit": "TFLOP/s",
                     "frac": ach / pk["tflops_sustained"] if ach else None, "traffic": None,
                     "kernel": "tc_track_kernel", "ms_per_launch": tc["ms"] / max(1, tc["launches"]),
                     "note": "profiled pass: one find per model on one stream"},
        "gpu_launches": int(sum(v["launches"] for v in prof.values() if isinstance(v, dict)) * args.steps),
        "clocks": clocks.summary(),
        "pose_error": {"rigid_gauss_newton": similarity_errors(rigid, m, wl.poses),
                       "quadratic_peak_fit": similarity_errors(quad, md, wl.poses),
                       "adjoint_gauss_newton": similarity_errors(adjoint, m, wl.poses),
                       "e2e_equals_value_pass": bool(np.array_equal(adjoint_h, adjoint))},
    }
    if not args.no_cpu_baseline:
        import oracle_lib
        b = cfg["budgets"]
        oracle_lib.set_oracle_budgets(b["samples"], b["pixels"], b["candidates"])
        orc = oracle_lib.oracle()
        crop = np.ascontiguousarray(wl.image[:1280, :1280])
        om = orc.create(wl.templates[0], levels=cfg["levels"], angle_start=FULL_CIRCLE[0],
                        angle_extent=FULL_CIRCLE[1])
        t0 = time.perf_counter()
        n = len(orc.find(om, crop, f[0], f[1], f[2], f[3][0], f[4], True, f[6], 1))
        dt = time.perf_counter() - t0
        oracle_lib.set_oracle_budgets()
        share = crop.size / wl.image.size / len(models)  # of one step's work, by pixels and models
        line["cpu_baseline"] = {"value": share / dt, "unit": "images/s", "cores": 1, "kind": "port",
                                "sample": f"the FP64 oracle's rigid find of the {wl.templates[0].shape[0]}^2 model "
                                          f"on a 1280x1280 crop of the scene ({n} matches, {dt:.1f} s), scaled to "
                                          f"a whole image and {len(models)} models by pixels x models",
                                "seconds": dt}
    print(json.dumps(line), flush=True)


def config_cpu_baseline(cfg, scenes_, templates) -> dict:
    """The FP64 oracle with the workload's budgets on a bounded sample: one
    scene per host thread (the smallest scenes of a batch), every template
    searched by its own single-model find; model build excluded."""
    from concurrent.futures import ThreadPoolExecutor

    import oracle_lib
    b = cfg["budgets"]
    oracle_lib.set_oracle_budgets(b["samples"], b["pixels"], b["candidates"])
    orc = oracle_lib.oracle()
    f = cfg["find"]
    lv = 0 if cfg["levels"] == "auto" else cfg["levels"]
    oms = [orc.create(t, levels=lv, angle_start=FULL_CIRCLE[0], angle_extent=FULL_CIRCLE[1]) for t in templates]
    threads = max(1, min(os.cpu_count() or 1, 16))
    order = sorted(range(len(scenes_)), key=lambda i: scenes_[i].image.size)
    sample = [scenes_[i].image for i in order[:threads]]

    quota = f[3][0] if isinstance(f[3], list) else f[3]

    def one(im):
        return sum(len(orc.find(om, im, f[0], f[1], f[2], quota, f[4], True, f[6], 1)) for om in oms)

    with ThreadPoolExecutor(threads) as ex:
        t0 = time.perf_counter()
        n = sum(ex.map(one, sample))
        dt = time.perf_counter() - t0
    oracle_lib.set_oracle_budgets()
    px = sum(im.size for im in sample)
    return {"value": len(sample) / dt, "unit": "images/s", "cores": min(threads, len(sample)), "kind": "port",
            "sample": f"{len(sample)} of the workload's scenes ({px / 1e6:.1f} M pixels), one per thread, each "
                      f"searched by {len(oms)} single-model FP64 oracle finds with the same budgets ({n} matches)",
            "seconds": dt}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--batch", type=int, default=32, help="scenes per step")
    ap.add_argument("--streams", type=int, default=32, help="finds in flight (host threads, one stream each)")
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--path", default="tensor", choices=["tensor", "plain"],
                    help="correlation path of the headline line (tensor cores or FP32 CUDA cores)")
    ap.add_argument("--no-compare", action="store_true", help="skip timing the other correlation path")
    ap.add_argument("--cohorts", type=int, default=0,
                    help="groups of finds in flight whose tensor-core launches are merged (0: per find)")
    ap.add_argument("--tc-lookahead", type=int, default=None,
                    help="grid rows of tensor-core weights in flight (launch shape; default: the library's)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default=WORKLOAD, choices=[WORKLOAD, *CONFIG_WORKLOADS],
                    help="the headline workload or a configuration workload (extended mode)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.workload != WORKLOAD:
        args.warmup = max(args.warmup, 3)
        run_config(args)
        return
    args.warmup = max(args.warmup, 3)

    import torch
    import mvkit_gb300 as mg
    from mvkit_gb300 import build

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    build.build()
    mg.load()

    wls = scenes(args.batch)
    model = mg.create_ncc_model(wls[0].template, **CREATE)
    ctl = (FIND["angle_start"], FIND["angle_extent"], FIND["min_score"], FIND["num_matches"], FIND["max_overlap"],
           FIND["subpixel"], FIND["num_levels"])
    threads = max(1, min(args.streams, args.batch))
    streams = [torch.cuda.Stream() for _ in range(threads)]
    dev = [mg.DeviceImage(w.image) for w in wls]
    pinned = []
    for w in wls:
        pb = mg.PinnedBuffer(w.image.shape, np.uint8)
        pb.array[...] = w.image
        pinned.append(pb)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MiB > L2
    found = []

    from concurrent.futures import ThreadPoolExecutor
    pool = ThreadPoolExecutor(threads)
    profiles = []

    path = [args.path]

    def thread_settings():
        mg.set_correlation_path(path[0])
        if args.tc_lookahead is not None:
            mg.ncc.set_tc_weight_lookahead(args.tc_lookahead)

    def worker(j, images, location_host: bool, ends, profile: bool):
        # each host thread owns one stream and the library's per-thread workspace
        torch.cuda.set_device(local)
        thread_settings()
        st = streams[j]
        if profile:
            mg.profile_reset()
            mg.profile_enable(True)
        out = []
        for im in images[j::threads]:
            arg = im.array if location_host else im
            out.append(mg.find_ncc_model(arg, model, *ctl, stream=st.cuda_stream))
        if ends is not None:
            ends[j].record(st)
        if profile:
            mg.profile_enable(False)
            profiles.append(mg.profile_read())
        return out

    def one_step(images, location_host: bool, ends=None, profile=False):
        futs = [pool.submit(worker, j, images, location_host, ends, profile) for j in range(threads)]
        res = [f.result() for f in futs]
        out = []
        for i in range(len(images)):
            out.append(res[i % threads][i // threads])
        return out

    def timed(images, host: bool, steps: int, profile=False):
        total = 0.0
        for _ in range(steps):
            flush.zero_()
            torch.cuda.synchronize()
            if world > 1:
                torch.distributed.barrier()
            e0 = torch.cuda.Event(enable_timing=True)
            ends = [torch.cuda.Event(enable_timing=True) for _ in range(threads)]
            e0.record(streams[0])
            torch.cuda.synchronize()
            found[:] = one_step(images, host, ends, profile)
            torch.cuda.synchronize()
            total += max(e0.elapsed_time(e) for e in ends)
        return total

    def aggregate():
        prof = {"finds": 0, "tensor_issued_macs": 0.0}
        for p in profiles:
            for k, v in p.items():
                if k in ("finds", "tensor_issued_macs"):
                    prof[k] += v
                    continue
                acc = prof.setdefault(k, dict(ms=0.0, launches=0, work=0.0))
                for f in ("ms", "launches", "work"):
                    acc[f] += v[f]
        profiles.clear()
        return prof

    host_images = [pb.array for pb in pinned]

    def batch_step(images, merge=None):
        # the batched operator: finds on the library's host threads (one
        # stream each, the calling thread's correlation path), tensor-core
        # launches merged across the finds in flight; results read back
        thread_settings()
        mg.set_batch_merge(args.cohorts if merge is None else merge)
        return mg.find_ncc_models_batch(images, [model], *ctl, workers=threads)

    batch_found = []

    def timed_batch(images, steps: int, merge=None, events=True):
        """Per step: L2 flush, then one batched call between CUDA events
        (device-resident images) or wall-clock stamps (host images); the call
        returns once its results are on the host."""
        total = 0.0
        st = streams[0]
        for _ in range(steps):
            flush.zero_()
            torch.cuda.synchronize()
            if world > 1:
                torch.distributed.barrier()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            t0 = time.perf_counter()
            e0.record(st)
            out = batch_step(images, merge)
            e1.record(st)
            torch.cuda.synchronize()
            total += e0.elapsed_time(e1) if events else (time.perf_counter() - t0) * 1e3
        batch_found[:] = out
        return total

    # the other correlation path, device-resident scenes, same protocol
    other = None
    if not args.no_compare:
        path[0] = "plain" if args.path == "tensor" else "tensor"
        for _ in range(args.warmup):
            batch_step(dev)
        torch.cuda.synchronize()
        other_ms = timed_batch(dev, args.steps)
        timed(dev, False, args.steps, profile=True)
        oprof = aggregate()
        other = {"path": path[0], "ms": other_ms,
                 "stages_ms_per_find": {k: round(v["ms"] / max(1, oprof["finds"]), 4) for k, v in oprof.items()
                                        if isinstance(v, dict)}}
        path[0] = args.path

    for _ in range(args.warmup):
        batch_step(dev)
        batch_step(host_images)
    torch.cuda.synchronize()

    mg.batch_profile_reset()
    with ClockSampler(local) as clocks:
        dev_ms = timed_batch(dev, args.steps)
    merged = mg.batch_profile_read()
    value_found = [r[:4] for r in batch_found]
    # ablation: the same steps with the other launch policy (merged within
    # one cohort of all finds in flight, or one launch per find)
    alt_cohorts = (1 if args.cohorts == 0 else 0) if args.path == "tensor" else None
    alt_ms, alt_same, alt_merged = None, None, None
    if alt_cohorts is not None:
        mg.batch_profile_reset()
        alt_ms = timed_batch(dev, args.steps, merge=alt_cohorts)
        alt_merged = mg.batch_profile_read()
        alt_same = same_results(batch_found, value_found)
    # the same steps again from per-find host threads with CUDA events around
    # each kernel group on the find streams: stage times and launch counts
    # (the events stay out of the value pass)
    timed(dev, False, args.steps, profile=True)
    prof = aggregate()
    host_ms = timed_batch(host_images, args.steps, events=False)

    # the same finds one at a time (untimed): per-kernel event times without
    # other streams' kernels interleaved
    def isolated():
        thread_settings()
        mg.profile_reset()
        mg.profile_enable(True)
        st = streams[0]
        for im in dev:
            mg.find_ncc_model(im, model, *ctl, stream=st.cuda_stream)
        mg.profile_enable(False)
        return mg.profile_read()

    iso = pool.submit(isolated).result()

    maxed = max_over_ranks
    dev_ms, host_ms = maxed(dev_ms), maxed(host_ms)
    if other is not None:
        other["value"] = replica_value(args.steps * args.batch, world, maxed(other.pop("ms")))
    value = replica_value(args.steps * args.batch, world, dev_ms)
    e2e = replica_value(args.steps * args.batch, world, host_ms)
    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return

    stages = {k: v for k, v in prof.items() if isinstance(v, dict)}
    pk = peaks()
    launches_total = sum(v["launches"] for v in stages.values())
    kernel_names = {"track": "track_kernel", "track_tc": "tc_track_kernel", "coarse": "coarse_kernel",
                    "score": "score_kernel", "refine": "refine_kernel", "sort": "sort_kernel",
                    "select": "select_kernel"}
    # roofline of the correlation kernel of the chosen path: tensor-core
    # tracking (its event time also covers three small grouping launches) or
    # the CUDA-core tracking kernel
    rstage = "track_tc" if args.path == "tensor" and stages.get("track_tc", {}).get("ms") else "track"
    d = stages[rstage]
    achieved_sep = 2.0 * d["work"] / (d["ms"] / 1e3) / 1e12 if d["ms"] else None
    di = iso[rstage]
    achieved_iso = 2.0 * di["work"] / (di["ms"] / 1e3) / 1e12 if di["ms"] else None
    peak = pk["tflops_sustained"]
    def merged_roof(m):
        a = 2.0 * m["macs"] / (m["ms"] / 1e3) / 1e12
        return {"achieved": a, "frac": a / peak, "launches": m["launches"], "find_jobs": m["jobs"],
                "ms_per_launch": m["ms"] / max(1, m["launches"]), "ms_per_find_job": m["ms"] / max(1, m["jobs"])}

    if rstage == "track_tc" and merged["ms"] > 0:
        # the value pass's merged launches: all finds' tensor-core work over
        # the launches' event time on the batcher's stream
        achieved = 2.0 * merged["macs"] / (merged["ms"] / 1e3) / 1e12
        note = (f"value pass: algorithmic correlation FLOPs (2 x MACs) of all finds over the event time of the "
                f"merged tc_track_kernel launches ({merged['launches']} launches, {merged['jobs']} find jobs); "
                f"peak = {pk['source']} dense bf16 sustained; fp16 operands (exact integer halves), FP32 "
                f"accumulation in tensor memory; issued/algorithmic MACs = "
                f"{merged['issued'] / max(1.0, merged['macs']):.2f}")
        ms_per_launch = merged["ms"] / max(1, merged["launches"])
    else:
        achieved = achieved_sep
        note = (f"algorithmic correlation FLOPs (2 x MACs) over the stage's event time; peak = {pk['source']} "
                f"dense bf16 sustained; "
                + ("fp16 operands (exact integer digits), FP32 accumulation in tensor memory; issued/algorithmic "
                   f"MACs = {prof.get('tensor_issued_macs', 0.0) / max(1.0, d['work']):.2f}"
                   if rstage == "track_tc" else "FP32 CUDA cores"))
        ms_per_launch = d["ms"] / max(1, d["launches"])
    roof = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": achieved / peak if achieved else None,
            "traffic": traffic_from_profiles(kernel_names[rstage]),
            "kernel": kernel_names[rstage],
            "ms_per_launch": ms_per_launch,
            "per_find_launches": {"achieved": achieved_sep, "frac": achieved_sep / peak if achieved_sep else None,
                                  "note": "each find launching its own tc_track_kernel, 32 finds in flight "
                                          "(stage events on the find streams)"},
            "merged_launches": (dict(merged_roof(alt_merged), cohorts=alt_cohorts,
                                     note="ablation pass: the finds' launches merged, one launch per step for the "
                                          "cohort; event time on the batcher's stream")
                                if alt_merged and alt_merged["ms"] > 0 else None),
            "isolated": {"achieved": achieved_iso,
                         "frac": achieved_iso / peak if achieved_iso else None,
                         "ms_per_launch": di["ms"] / max(1, di["launches"]),
                         "note": "same finds one at a time on one stream, one launch per find step (untimed pass)"},
            "note": note}
    matches = [len(r[0]) for r in value_found]
    line = {
        "metric": METRIC, "value": value, "unit": "images/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": {"workload": WORKLOAD, "image": "2048x2048 u8", "template": "128x128", "poses": 5,
                   "angle_range_deg": [-30, 30], "num_levels": 4, "min_score": 0.7, "num_matches": 5,
                   "max_overlap": 0.5, "scenes_per_step": args.batch, "l2": "flushed (256 MiB write) between steps",
                   "finds_in_flight": threads, "merge_cohorts": args.cohorts,
                   **({"tc_weight_lookahead": args.tc_lookahead} if args.tc_lookahead is not None else {}),
                   "parallelism": f"replicas x{world}",
                   "path": ("tensor-core (tcgen05) tracking correlation" if args.path == "tensor"
                            else "plain FP32 CUDA-core correlation")},
        "e2e": {"value": e2e, "unit": "images/s",
                "h2d_bytes_per_step": int(sum(w.image.nbytes for w in wls)),
                "d2h_bytes_per_step": int(args.batch * (4 * 8 * FIND["num_matches"] + 128)),
                "api": "find_ncc_models_batch (mvg_find_ncc_models_batch) on pinned host images, "
                       f"{threads} library host threads; wall clock per step, synchronized on both sides"},
        "roofline": roof,
        # kernels of the value pass: every find's own launches, its tensor-core
        # launches replaced by the merged ones
        "gpu_launches": int(launches_total - stages.get("track_tc", {}).get("launches", 0) + merged["launches"]
                            if merged["launches"] else launches_total),
        "clocks": clocks.summary(),
        "stages_ms_per_find": {k: round(v["ms"] / max(1, prof["finds"]), 4) for k, v in stages.items()},
        "stages_ms_per_find_isolated": {k: round(v["ms"] / max(1, iso["finds"]), 4) for k, v in iso.items()
                                        if isinstance(v, dict)},
        "matches_per_scene": matches,
    }
    if other is not None:
        line["compare"] = other
    if alt_ms is not None:
        line["merge_ablation"] = {
            "value_pass_cohorts": args.cohorts, "value_images_per_s": value,
            "other_cohorts": alt_cohorts,
            "other_images_per_s": replica_value(args.steps * args.batch, world, maxed(alt_ms)),
            "note": "cohorts 0: every find launches its own tensor-core kernels; k > 0: the finds in flight "
                    "form k groups whose launches are merged"}
    oracle = None
    if not args.no_cpu_baseline:
        line["cpu_baseline"], oracle = cpu_baseline(wls, os.cpu_count() or 1)
    line["pose_error"] = pose_error(value_found, wls, oracle)
    # the other passes return the value pass's matches bit for bit
    line["pose_error"]["e2e_equals_value_pass"] = same_results(batch_found, value_found)
    line["pose_error"]["per_find_threads_equal_value_pass"] = same_results(found, value_found)
    if alt_same is not None:
        line["pose_error"]["ablation_equals_value_pass"] = alt_same
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
