#!/usr/bin/env python
"""Benchmark: 4096x4096 frames of 20,000 mixed paths (seed 1), pixel mode.

One step renders one frame of the scene (curves -> intersections -> sort ->
winding -> spans/fragments -> RGBA8) on one GB300.  Prints ONE JSON line.

  value       frames/s with the scene resident in HBM, CUDA events on the
              render stream around each frame, L2 flushed (256 MiB memset)
              between timed frames.
  e2e         frames/s through the C ABI with host buffers: every step copies
              the scene from pinned host memory (sr_load_scene) and reads the
              RGBA8 frame back into pinned host memory (sr_render).  Three
              renderer contexts on three streams, each driven by its own host
              thread, keep three frames in flight, so one frame's copies and
              its chain stage's idle tail overlap the other frames' kernels.
  roofline    the dominant stage's algorithmic bytes / its CUDA-event time
              against the measured HBM copy bandwidth.
  cpu_baseline  the C++ oracle (the CPU restatement of the reference shaders)
              rendering the same frame with every host thread.

--impl reference times that CPU restatement as the reference arm (the
reference itself is a Windows/Vulkan program with no CPU path).
Under torchrun (N>1) every rank renders its own replica of the frame
("replicas only"; no collective on the data path).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

WORKLOADS = {
    # name: (preset, seed, width, height, paths)
    "frame4096": (1, 1, 4096, 4096, 20000),
    "frame1024": (0, 0, 1024, 1024, 500),
    "mixed2048": (1, 1, 2048, 2048, 5000),
}
L2_FLUSH_BYTES = 256 << 20
# GPU images kept (as SHA-256) for the oracle check in the CPU-baseline leg:
# "batch" holds (scene index, hash) of a seeded sample of the batch workload,
# "served" (scene index, hash) of served requests
CHECKS = {"batch": [], "served": []}
ORACLE_SAMPLE = 64
# What bounds each stage's main kernel (profiles/ncu_top_kernels_frame4096.md):
# the HBM fraction is the roofline only for the stages that move bytes.
LIMITS = {
    "resolve": "latency of each segment's walk back to its collapse cut and of the record gathers",
    "chains": "the dependent bisection steps of the longest crossing chains",
    "wide": "the longest chain's bisection rounds (lane exchange latency), beside the rest of the frame",
    "sort": "shared-memory ranking latency of the tile sort and merge rounds",
    "winding_emit": "latency of each tile's flag, look-back and emission phases at 4-5 CTAs per SM, DRAM ~14%",
}
STAGE_NAMES = ["transform", "count", "offset_scan", "chains", "merge", "fragment", "sort", "winding_emit",
               "row_sort", "resolve", "wide"]


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="frame4096", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--e2e-streams", type=int, default=3,
                    help="frames in flight in the end-to-end leg (one context, stream and host thread each)")
    ap.add_argument("--batch-scenes", type=int, default=4096,
                    help="scenes of the batched workload (0 skips it)")
    ap.add_argument("--batch-size", type=int, default=512, help="scenes per resident batch")
    ap.add_argument("--batch-streams", type=int, default=3,
                    help="streams the resident batches' frames are spread over (frames in flight)")
    ap.add_argument("--plain-scenes", type=int, default=512,
                    help="scenes the plain per-scene renderer is timed on")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-sizing configuration")
    ap.add_argument("--train-epochs", type=int, default=30)
    ap.add_argument("--small-batch", type=int, default=32,
                    help="scenes per batch in the learned-vs-exact sizing stream")
    ap.add_argument("--serve-requests", type=int, default=2048, help="requests of the serving configuration")
    ap.add_argument("--serve-rate", type=float, default=2000.0, help="Poisson arrival rate (requests/s)")
    ap.add_argument("--serve-overload", type=float, default=8000.0,
                    help="a second arrival rate above the plain renderer's capacity (0 skips it)")
    ap.add_argument("--serve-batch", type=int, default=256, help="largest batch the server forms")
    return ap.parse_args()


def dist_env():
    from vkscanlinepr_gb300.replicas import dist_env as env
    return env()


def metric_name(workload):
    """The metric both arms report for a workload."""
    if workload == "frame4096":
        return "frames/s (4096x4096, 20000 paths, 1 spp, bit-exact)"
    return "frames/s (%s)" % workload


def measured_peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_traffic():
    """DRAM bytes per launch of each stage's kernel from the committed ncu
    summary (lines 'traffic <stage> <bytes> <records>'), or {}."""
    p = os.path.join(REPO, "profiles", "traffic.md")
    out = {}
    if os.path.exists(p):
        for line in open(p):
            parts = line.strip().strip("|").split()
            if len(parts) == 4 and parts[0] == "traffic":
                out[parts[1]] = (float(parts[2]), float(parts[3]))
    return out


class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.tmp = tempfile.NamedTemporaryFile(prefix="clk", suffix=".csv", delete=False)

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=self.tmp, stderr=subprocess.DEVNULL)
        except (OSError, ValueError):
            self.proc = None
        time.sleep(0.3)

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.tmp.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.tmp.name) as f:
            for line in f:
                cols = [c.strip() for c in line.split(",")]
                if len(cols) < 7:
                    continue
                try:
                    sm.append(float(cols[0]))
                    mx.append(float(cols[1]))
                except ValueError:
                    continue
                for n, v in zip(names, cols[3:7]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
        os.unlink(self.tmp.name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "samples": len(sm),
                "reasons": sorted(reasons)}


def stage_bytes(st, n_curves, n_points, W, H):
    """Algorithmic bytes per stage for one frame."""
    N = st["n_intersections"]
    O = st["n_draw_records"]
    passes = st["sort_passes"]
    rows_bits = max(1, int(np.ceil(np.log2(H + 1))))
    row_passes = (rows_bits + 7) // 8
    return {
        "transform": n_points * (8 + 4 + 8),
        "count": n_curves * (12 + 32 + 20 + 4),
        "offset_scan": n_curves * 8,
        "chains": n_curves * (12 + 80 + 32) + N * 4,
        "merge": n_curves * (8 + 80) + N * (4 + 8),
        "fragment": N * (8 + 8),                       # record in, key (with winding bits) out
        # the per-path segmented sort: one read and one write of each 8-byte
        # key (the least any sort moves; large paths' merge rounds come on top)
        "sort": N * 2 * 8,
        # sorted keys in; draw records (16 B) and their cell rows (4 B) out
        "winding_emit": N * 8 + O * (16 + 4),
        "row_sort": O * 4 + row_passes * O * 2 * (4 + 4),
        # a latency walk to each segment's collapse cut bounds it, and the
        # records it reads depend on where the cuts fall: no byte count
        # comparable with the streaming stages (its time is reported)
        "resolve": 0,
        # the wide chains and their curves' merge and fragments, on a second
        # stream beside chains, merge and fragment (their bytes are counted there)
        "wide": 0,
    }


def run_cpu_baseline(scene_oracle, W, H, budget_s=20.0):
    import oracle
    threads = oracle.hw_threads()
    times = []
    img = None
    t_all = time.perf_counter()
    while True:
        t0 = time.perf_counter()
        f = oracle.Frame(scene_oracle, width=W, height=H, mode=oracle.MODE_PIXEL, threads=threads)
        times.append(time.perf_counter() - t0)
        if img is None:
            img = f.get("image")
        del f
        if time.perf_counter() - t_all > budget_s * 0.5 or len(times) >= 5:
            break
    v = len(times) / sum(times)
    return {"value": round(v, 4), "unit": "frames/s", "cores": threads, "kind": "port",
            "sample": "%d full frame(s) of the same scene by the oracle (C++ restatement, %d threads)"
                      % (len(times), threads)}, img


def run_batched(sr, args, sptr, steps):
    """Configuration 2: uneven scenes (side 256..2048, lognormal path
    counts), rendered as resident batches replaying captured CUDA graphs,
    against the plain renderer (load + render per scene)."""
    total, per = args.batch_scenes, args.batch_size
    seed = 2
    t0 = time.perf_counter()
    batches = []
    for k in range((total + per - 1) // per):
        n = min(per, total - k * per)
        b = sr.SceneBatch(mode=sr.MODE_PIXEL)
        b.add_synth(2, seed, n, scene_index=k * per)
        b.commit()
        batches.append(b)
    build_s = time.perf_counter() - t0
    # launch shapes for this size class: timed on the first batch, cached in
    # JSON, applied to the batches of the same class
    tpath = os.path.join(tempfile.mkdtemp(prefix="srtune"), "tuning.json")
    t0 = time.perf_counter()
    tuning = batches[0].autotune(tpath, stream=sptr)
    tune_s = time.perf_counter() - t0
    tclass = batches[0].tuning_class()
    with open(tpath) as f:
        tune_cache = json.load(f)
    for b in batches[1:]:
        b.set_tuning(**tuning)
    caps, records = [], 0
    for b in batches:           # exact frame: learns each batch's record count
        b.render(stream=sptr)
        st = b.stats()
        caps.append(st["n_intersections"])
        records += st["n_intersections"]
    for b, c in zip(batches, caps):
        b.render(capacity=c, graph=True, stream=sptr)   # capture
    # the batches' frames are independent: spread them over a few streams so
    # one frame's tail (its longest bisection chains) overlaps the next ones
    import ctypes as _ct
    import torch
    nst = max(1, args.batch_streams)
    streams = [torch.cuda.Stream() for _ in range(nst)]
    sps = [_ct.c_void_p(x.cuda_stream) for x in streams]
    torch.cuda.synchronize()
    times = []
    for _ in range(steps):
        t1 = time.perf_counter()
        for i, (b, c) in enumerate(zip(batches, caps)):
            b.enqueue(c, graph=True, stream=sps[i % nst])
        for b in batches:
            b.finish()
        times.append(time.perf_counter() - t1)
    overflows = sum(b.stats()["overflows"] for b in batches)
    batched_sps = total / (sum(times) / len(times))
    # a seeded sample of the timed frames' images, checked against the oracle later
    sample = sorted(np.random.default_rng(11).choice(total, min(ORACLE_SAMPLE, total), replace=False).tolist())
    CHECKS["batch"] = [(i, image_hash(batches[i // per].image(i % per))) for i in sample]
    # plain per-scene renderer on the first scenes of the same set
    nplain = min(args.plain_scenes, total)
    ctx = None
    plain_t = 0.0
    exact = 0
    checked = 0
    for i in range(nplain):
        sc = sr.synth_scene(2, seed, scene_index=i)
        if ctx is None or (ctx.width, ctx.height) != (sc.width, sc.height):
            if ctx is not None:
                ctx.close()
            ctx = sr.ScanlineVGRasterizer(mode=sr.MODE_PIXEL)
            ctx.initialize(None, sc.width, sc.height)
            ctx.loadVG(sc)
            ctx.render_device(stream=sptr)   # warm the context's buffers
        t1 = time.perf_counter()
        ctx.loadVG(sc)
        ctx.render_device(stream=sptr)
        plain_t += time.perf_counter() - t1
        if i < 24:
            img = ctx.render()
            checked += 1
            exact += int(np.array_equal(img, batches[i // per].image(i % per)))
    if ctx is not None:
        ctx.close()
    plain_sps = nplain / plain_t
    n_resident = len(batches)
    learned = serving = None
    if not args.no_learned:
        sz, margins, learned = run_learned(sr, args, sptr, batches)
        for b in batches:
            b.close()
        batches = []
        serving = run_serving(sr, args, sz, margins)
        sz.close()
    for b in batches:
        b.close()
    return learned, serving, {"scenes": total, "records": int(records), "resident_batches": n_resident,
            "scenes_per_s": round(batched_sps, 1), "ms_per_batch_of_all": round(1000 * sum(times) / len(times), 2),
            "sizing": "record capacity from the previous exact frame, frame replayed as a CUDA graph",
            "streams": nst,
            "overflows": int(overflows), "plain_scenes_per_s": round(plain_sps, 1),
            "plain_sample": nplain, "speedup_vs_plain": round(batched_sps / plain_sps, 2),
            "bit_exact_vs_plain": "%d/%d" % (exact, checked), "build_s": round(build_s, 2),
            "autotune": {"class": tclass, "chosen": tuning, "seconds": round(tune_s, 2),
                         "cache": tune_cache}}


def _labels_of(sr, batches_spec, sptr):
    """Features, exact-count labels and scene path ranges of the paths of
    several synthetic batches: [(preset, seed, count, first_scene_index), ...]."""
    xs, ts, ranges, paths = [], [], [0], 0
    for preset, seed, count, first in batches_spec:
        b = sr.SceneBatch(mode=sr.MODE_PIXEL)
        b.add_synth(preset, seed, count, scene_index=first)
        b.commit()
        xs.append(b.features(stream=sptr))
        ts.append(b.labels(stream=sptr))
        ranges.extend(int(v) + paths for v in b.path_ranges()[1:])
        paths += xs[-1].shape[0]
        b.close()
    return sr.concat_device(xs), sr.concat_device(ts), np.array(ranges), paths


def run_learned(sr, args, sptr, batches):
    """Configuration 3: the sizing network trained on ~200k paths of the
    4096^2 and batch generators (labels from the exact count pass), margins
    calibrated on held-out scenes, evaluated on the batched workload's
    scenes: per-path overflow, over-allocation, and the time sizing from the
    network saves against waiting for the exact count."""
    import ctypes as _ct
    import torch
    t0 = time.perf_counter()
    x, t, _, n_train = _labels_of(sr, [(1, 101 + i, 1, 0) for i in range(4)] + [(2, 102, 384, 0)], sptr)
    label_s = time.perf_counter() - t0
    xv, tv, val_ranges, n_val = _labels_of(sr, [(2, 103, 96, 0)], sptr)
    sz = sr.Sizer(seed=1)
    sz.set_norm(sr.sizer_norm(x.numpy(), t.numpy()))
    t0 = time.perf_counter()
    loss = sz.train(x, t, epochs=args.train_epochs, batch=4096, lr=1e-3, seed=7, stream=sptr)
    train_s = time.perf_counter() - t0
    steps = sz.state()["step"]
    pv = sz.predict(xv).numpy()
    margins = sr.calibrate_margins(pv, tv.numpy(), val_ranges)
    val_loss, _ = sz.loss_grad(xv, tv)
    # evaluation on the batched workload's scenes (seed 2), one resident
    # batch at a time so only one holds planned-size buffers
    for b in batches:
        b.release()
    paths = over_r = over_d = 0
    acc = {k: 0 for k in ("records", "draws", "path_records", "path_draws", "exact_r", "exact_d")}
    plan_ms, overflows = [], 0
    t_exact = t_learned = 0.0
    for b in batches:
        t1 = time.perf_counter()
        pl = b.plan(sz, margins, stream=sptr)
        plan_ms.append(1000 * (time.perf_counter() - t1))
        j = b.judge(stream=sptr)
        paths += j["paths"]
        over_r += j["paths_over_records"]
        over_d += j["paths_over_draws"]
        for k in ("records", "draws", "path_records", "path_draws"):
            acc[k] += pl[k]
        acc["exact_r"] += j["records"]
        acc["exact_d"] += j["draws"]
        # the batch rendered once: waiting for the exact count against a
        # plan plus a pre-sized frame; both warmed first
        b.render(capacity=pl["records"], draw_capacity=pl["draws"], stream=sptr)
        b.render(stream=sptr)
        t1 = time.perf_counter()
        b.render(stream=sptr)
        t_exact += time.perf_counter() - t1
        o0 = b.stats()["overflows"]
        t1 = time.perf_counter()
        pl = b.plan(sz, margins, stream=sptr)
        b.render(capacity=pl["records"], draw_capacity=pl["draws"], stream=sptr)
        t_learned += time.perf_counter() - t1
        overflows += b.stats()["overflows"] - o0
        b.release()
    # a stream of serving-sized batches of new scenes: each is assembled on
    # the host, uploaded, sized and rendered.  With exact sizing the host
    # waits inside every frame for its count, so it cannot assemble the next
    # batch while the GPU renders; planned frames are enqueued whole and the
    # host moves on to the next batch.
    sb = args.small_batch
    nsb = max(2, min(48, args.batch_scenes // max(1, sb)))
    scenes = [sr.synth_scene(2, 2, scene_index=i) for i in range(nsb * sb)]
    rs, ss = torch.cuda.Stream(), torch.cuda.Stream()
    rsp, ssp = _ct.c_void_p(rs.cuda_stream), _ct.c_void_p(ss.cuda_stream)
    objs = [sr.SceneBatch(mode=sr.MODE_PIXEL) for _ in range(2)]

    def fill(b, k):
        b.clear()
        for sc in scenes[k * sb:(k + 1) * sb]:
            b.add_scene(sc)
        b.commit()

    def exact_stream():
        for k in range(nsb):
            b = objs[k % 2]
            fill(b, k)
            b.render(stream=rsp)

    def learned_stream():
        prev = None
        for k in range(nsb):
            b = objs[k % 2]
            fill(b, k)
            pl = b.plan(sz, margins, stream=ssp)
            b.enqueue(pl["records"], draw_capacity=pl["draws"], stream=rsp)
            if prev is not None:
                prev.finish()
            prev = b
        prev.finish()
    exact_stream()
    learned_stream()
    torch.cuda.synchronize()
    o0 = sum(b.stats()["overflows"] for b in objs)
    t1 = time.perf_counter()
    exact_stream()
    t_small_exact = time.perf_counter() - t1
    t1 = time.perf_counter()
    learned_stream()
    t_small_learned = time.perf_counter() - t1
    small_over = sum(b.stats()["overflows"] for b in objs) - o0
    for b in objs:
        b.close()
    return sz, margins, {
        "train_paths": int(n_train), "val_paths": int(n_val), "label_s": round(label_s, 2),
        "train_steps": int(steps), "train_s": round(train_s, 3), "train_mse": round(loss, 5),
        "val_mse": round(val_loss, 5), "margins": [round(m, 4) for m in margins],
        "eval_paths": int(paths),
        "overflow_paths_records": round(over_r / max(paths, 1), 5),
        "overflow_paths_draws": round(over_d / max(paths, 1), 5),
        "path_allot_over_exact": [round(acc["path_records"] / max(acc["exact_r"], 1), 3),
                                  round(acc["path_draws"] / max(acc["exact_d"], 1), 3)],
        "frame_capacity_over_exact": [round(acc["records"] / max(acc["exact_r"], 1), 3),
                                      round(acc["draws"] / max(acc["exact_d"], 1), 3)],
        "plan_ms_per_batch": round(statistics.median(plan_ms), 3),
        "batch_frames_overflowed": int(overflows),
        "big_batches": {"scenes_per_batch": args.batch_size, "exact_s": round(t_exact, 4),
                        "learned_s": round(t_learned, 4), "saved_frac": round(1 - t_learned / t_exact, 4)},
        "stream": {"scenes_per_batch": sb, "batches": nsb, "exact_s": round(t_small_exact, 4),
                   "learned_s": round(t_small_learned, 4),
                   "saved_frac": round(1 - t_small_learned / t_small_exact, 4),
                   "scenes_per_s_exact": round(nsb * sb / t_small_exact, 1),
                   "scenes_per_s_learned": round(nsb * sb / t_small_learned, 1),
                   "overflowed": int(small_over)},
    }


def _serve(sr, srv, scenes, arrivals, check_every=0):
    """Submits scenes[i % len] at arrivals[i] (seconds from the start, None:
    all at once) from a client thread and collects them in order; returns
    per-request (submit, done) times on the server clock and the images of
    every check_every-th request."""
    import queue
    import threading
    q = queue.Queue()
    n = len(arrivals)

    def client():
        t0 = time.perf_counter()
        for i in range(n):
            if arrivals[i] is not None:
                d = t0 + arrivals[i] - time.perf_counter()
                if d > 0:
                    time.sleep(d)
            q.put((i, srv.submit(scenes[i % len(scenes)])))
    th = threading.Thread(target=client)
    th.start()
    times, imgs = [], {}
    for _ in range(n):
        i, tk = q.get()
        fetch = check_every > 0 and i % check_every == 0
        img, info = srv.wait(tk, fetch=fetch)
        times.append((info["submit_s"], info["done_s"], info["batch_scenes"]))
        if fetch:
            imgs[i] = img
    th.join()
    return np.array(times), imgs


def _lat_summary(sub, done):
    lat = 1000.0 * (done - sub)
    span = done.max() - sub.min()
    return {"p50_ms": round(float(np.percentile(lat, 50)), 2), "p99_ms": round(float(np.percentile(lat, 99)), 2),
            "scenes_per_s": round(len(lat) / span, 1)}


def run_serving(sr, args, sz, margins):
    """Configuration 4: requests of batch-workload sizes arriving as a
    Poisson stream, served by the continuous-batching server (learned
    sizing, 120 GB budget) against the exact-sizing server and the plain
    per-request renderer; every image bit-exact."""
    n = args.serve_requests
    pool = [sr.synth_scene(2, 2, scene_index=i) for i in range(min(n, 1024))]
    rng = np.random.default_rng(4)
    arrivals = list(np.cumsum(rng.exponential(1.0 / args.serve_rate, n)))
    warm_n = min(512, max(len(pool) - 64, 0))
    warm = list(np.cumsum(np.random.default_rng(3).exponential(1.0 / args.serve_rate, warm_n)))
    out = {"requests": n, "rate_per_s": args.serve_rate, "scene_pool": len(pool), "budget_bytes": int(120e9),
           "warmup": "64 requests at once, then %d arrivals at the same rate (untimed)" % warm_n,
           "slots": {"learned": 2, "exact": 1}}
    # two batches in flight: at 2,000 requests/s the tail was shortest with
    # two (three let the largest scenes' frames share the GPU longer)
    for name, sizer, slots in (("learned", sz, 2), ("exact", None, 1)):
        srv = sr.RenderServer(sizer=sizer, slots=slots, max_batch_scenes=args.serve_batch, memory_budget=120e9,
                              margins=margins)
        # untimed warm-up: a burst, then a stream of the same rate with
        # images fetched as in the timed run, so that every slot's buffers
        # have grown to the batches a stream forms and the fetch path has run
        _serve(sr, srv, pool[:64], [None] * 64)
        _serve(sr, srv, pool[64:64 + warm_n], warm, check_every=32)
        t, imgs = _serve(sr, srv, pool, arrivals,
                         check_every=max(1, n // ORACLE_SAMPLE) if name == "learned" else 0)
        res = _lat_summary(t[:, 0], t[:, 1])
        res["mean_batch"] = round(float(t[:, 2].mean()), 1)
        ts, _ = _serve(sr, srv, pool, [None] * n)                     # saturation: all at once
        res["saturated_scenes_per_s"] = _lat_summary(ts[:, 0], ts[:, 1])["scenes_per_s"]
        if args.serve_overload > 0:
            over = list(np.cumsum(np.random.default_rng(5).exponential(1.0 / args.serve_overload, n)))
            to, _ = _serve(sr, srv, pool, over)
            res["at_%d_per_s" % int(args.serve_overload)] = _lat_summary(to[:, 0], to[:, 1])
        st = srv.stats()
        res.update({"batches": int(st["batches"]), "overflows": int(st["overflows"]),
                    "refits": int(st["refits"]), "peak_bytes": int(st["peak_bytes"])})
        srv.close()
        out[name] = res
        if name == "learned":
            checked = imgs
    # the plain renderer, one request at a time in arrival order
    ctx = None
    done = []
    t_free = 0.0
    exact = 0
    for i in range(n):
        sc = pool[i % len(pool)]
        if ctx is None or (ctx.width, ctx.height) != (sc.width, sc.height):
            if ctx is not None:
                ctx.close()
            ctx = sr.ScanlineVGRasterizer(mode=sr.MODE_PIXEL)
            ctx.initialize(None, sc.width, sc.height)
            ctx.loadVG(sc)
            ctx.render_device()
        t1 = time.perf_counter()
        ctx.loadVG(sc)
        ctx.render_device()
        svc = time.perf_counter() - t1
        start = max(arrivals[i], t_free)
        t_free = start + svc
        done.append(t_free)
        if i in checked:
            exact += int(np.array_equal(ctx.render(), checked[i]))
    if ctx is not None:
        ctx.close()
    CHECKS["served"] = [(i % len(pool), image_hash(img)) for i, img in sorted(checked.items())]
    out["plain"] = _lat_summary(np.array(arrivals), np.array(done))
    out["bit_exact_vs_plain"] = "%d/%d" % (exact, len(checked))
    out["speedup_vs_plain"] = round(out["learned"]["scenes_per_s"] / out["plain"]["scenes_per_s"], 2)
    out["saturated_speedup_vs_plain"] = round(out["learned"]["saturated_scenes_per_s"] /
                                              out["plain"]["scenes_per_s"], 2)
    return out


def image_hash(img):
    import hashlib
    return hashlib.sha256(np.ascontiguousarray(img).tobytes()).hexdigest()


def check_against_oracle(threads):
    """The kept batch and served images against the oracle's frames of the
    same scenes (pixel mode), and their samples that flip against the FP64
    oracle.  Returns ({"batch": "k/n", "served": "k/n"}, flips summary)."""
    import oracle
    exact, flips = {}, []
    for key, items in CHECKS.items():
        ok = 0
        for idx, h in items:
            sc = oracle.synth(2, 2, scene_index=idx)
            img = oracle.Frame(sc, mode=oracle.MODE_PIXEL, threads=threads).get("image")
            ok += int(image_hash(img) == h)
            if key == "batch":
                flips.append(oracle.fp64_flips(sc, oracle.MODE_PIXEL, threads=threads, image=img))
        exact[key] = "%d/%d" % (ok, len(items))
    fl = None
    if flips:
        fl = {"scenes": len(flips), "total": int(sum(flips)), "max": int(max(flips)),
              "scenes_with_flips": int(sum(1 for f in flips if f))}
    return exact, fl


def oracle_scene(preset, seed, W, H, P):
    import oracle
    return oracle.synth(preset, seed, width=W, height=H, n_paths=P)


def main():
    args = parse_args()
    rank, world, local = dist_env()
    wl = WORKLOADS[args.workload]
    preset, seed, W, H, P = wl
    workload_desc = "%dx%d frame, %d paths (preset %d, seed %d), pixel mode, 1 sample/px" % (W, H, P, preset, seed)

    if args.impl == "reference":
        if rank != 0:
            return 0
        import oracle
        oracle.build()
        sc = oracle_scene(preset, seed, W, H, P)
        threads = oracle.hw_threads()
        for _ in range(args.warmup):
            oracle.Frame(sc, mode=oracle.MODE_PIXEL, threads=threads)
        t = []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            oracle.Frame(sc, mode=oracle.MODE_PIXEL, threads=threads)
            t.append(time.perf_counter() - t0)
        v = len(t) / sum(t)
        line = {"metric": metric_name(args.workload), "value": round(v, 4), "unit": "frames/s",
                "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": round(1000 * sum(t) / len(t), 3), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "impl": "reference",
                "config": {"workload": workload_desc, "l2": "n/a (CPU)"},
                "cpu_baseline": {"value": round(v, 4), "unit": "frames/s", "cores": threads, "kind": "port",
                                 "sample": "one full frame per step (C++ restatement of the reference "
                                           "shaders, %d threads)" % threads},
                "e2e": {"value": round(v, 4), "unit": "frames/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return 0

    import torch
    import vkscanlinepr_gb300 as sr
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    sr.lib()
    stream = torch.cuda.current_stream()
    sptr = ctypes_stream(stream)

    scene = sr.synth_scene(preset, seed, width=W, height=H, n_paths=P)
    r = sr.ScanlineVGRasterizer(mode=sr.MODE_PIXEL, device=local, profile=True)
    r.initialize(None, W, H)
    r.loadVG(scene)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")

    clk = ClockSampler(local)
    clk.start()
    for _ in range(max(args.warmup, 3)):
        r.render_device(stream=sptr)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    step_ms, stage_acc, launches = [], {k: 0.0 for k in STAGE_NAMES}, 0
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    for _ in range(args.steps):
        flush.zero_()
        e0.record(stream)
        r.render_device(stream=sptr)
        e1.record(stream)
        e1.synchronize()
        step_ms.append(e0.elapsed_time(e1))
        st = r.stats()
        launches += st["kernel_launches"]
        for k in STAGE_NAMES:
            stage_acc[k] += st["stage_ms"][k]
    torch.cuda.synchronize()
    clocks = clk.stop()
    from vkscanlinepr_gb300 import replicas
    total_ms = replicas.max_over_ranks(sum(step_ms))            # the slowest replica
    value = world * args.steps / (total_ms / 1000.0)
    st = r.stats()

    # ---- end to end through the C ABI with pinned host buffers
    arrs = scene.arrays()
    pinned = {}
    h2d = 0
    for k, a in arrs.items():
        pb = sr.PinnedBuffer(max(a.nbytes, 4))
        view = pb.array[:a.nbytes].view(a.dtype)
        view[:] = a
        pinned[k] = (pb, view)
        h2d += a.nbytes
    pscene = sr.VGContainer.from_arrays(W, H, *[pinned[k][1] for k in
                                                ("position", "pos_path_idx", "curve_pos_map", "curve_type",
                                                 "curve_path_idx", "fill_rule", "fill_info")])
    # one renderer context, stream, pinned output and host thread per frame in flight
    n_fly = max(1, args.e2e_streams)
    e2e_streams = [torch.cuda.Stream() for _ in range(n_fly)]   # kept alive for the leg
    legs = [(r, ctypes_stream(e2e_streams[0]), sr.PinnedBuffer(W * H * 4))]
    for k in range(1, n_fly):
        rk = sr.ScanlineVGRasterizer(mode=sr.MODE_PIXEL, device=local)
        rk.initialize(None, W, H)
        legs.append((rk, ctypes_stream(e2e_streams[k]), sr.PinnedBuffer(W * H * 4)))
    per_leg = max(3, min(args.steps, 10))
    e2e_steps = per_leg * n_fly

    def leg(k, n):
        rk, sk, pb = legs[k]
        img = pb.array.reshape(H, W, 4)
        for _ in range(n):
            rk.loadVG(pscene)
            rk.render(out=img, stream=sk)

    for k in range(n_fly):   # warm every context (allocations, first launches)
        leg(k, 1)
    import threading
    if world > 1:
        dist.barrier()
    t0 = time.perf_counter()
    threads = [threading.Thread(target=leg, args=(k, per_leg)) for k in range(n_fly)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    e2e_s = replicas.max_over_ranks(time.perf_counter() - t0)
    e2e = {"value": round(world * e2e_steps / e2e_s, 4), "unit": "frames/s", "h2d_bytes_per_step": int(h2d),
           "d2h_bytes_per_step": int(W * H * 4), "frames_in_flight": n_fly}
    out_img = legs[0][2].array.reshape(H, W, 4)
    gpu_img = out_img.copy()
    for rk, _, _ in legs[1:]:
        rk.close()
    r.close()

    learned, serving, batched = (run_batched(sr, args, sptr, max(2, min(args.steps, 5))) if args.batch_scenes > 0
                                 else (None, None, None))

    # ---- roofline of the dominant stage
    peak, peak_kind = measured_peaks()
    sb = stage_bytes(st, scene.n_curves, scene.n_points, W, H)
    stage_ms = {k: stage_acc[k] / args.steps for k in STAGE_NAMES}
    dom = max((k for k in stage_ms if sb[k]), key=lambda k: stage_ms[k])
    stages = {}
    for k in STAGE_NAMES:
        ms = stage_ms[k]
        stages[k] = {"ms": round(ms, 4), "algo_bytes": int(sb[k]),
                     "gbs": round(sb[k] / (ms * 1e6), 1) if ms > 0 and sb[k] else None,
                     "frac": round(sb[k] / (ms * 1e6) / peak, 4) if ms > 0 and sb[k] else None}
    traffic = None
    tr = profile_traffic()
    if dom in tr and tr[dom][1] > 0:
        traffic = int(tr[dom][0] / tr[dom][1] * st["n_intersections"])
    achieved = sb[dom] / (stage_ms[dom] * 1e6)
    roofline = {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak,
                "peak_kind": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else peak_kind,
                "unit": "GB/s", "frac": round(achieved / peak, 4), "traffic": traffic,
                "limited_by": LIMITS.get(dom, "")}

    line = {"metric": metric_name(args.workload),
            "value": round(value, 4), "unit": "frames/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": workload_desc, "width": W, "height": H, "paths": P,
                       "n_intersections": int(st["n_intersections"]), "n_draw_records": int(st["n_draw_records"]),
                       "sort_key_bits": int(st["key_bits"]), "sort_passes": int(st["sort_passes"]),
                       "l2": "flushed between timed frames (256 MiB memset)",
                       "parallelism": "replicas" if world > 1 else "single"},
            "samples_per_s": round(value * W * H, 1),
            "roofline": roofline, "stages": stages, "e2e": e2e, "clocks": clocks,
            "gpu_launches": int(launches)}
    if batched is not None:
        line["batched"] = batched
    if learned is not None:
        line["learned"] = learned
    if serving is not None:
        line["serving"] = serving

    if rank == 0 and not args.no_cpu_baseline:
        so = oracle_scene(preset, seed, W, H, P)
        cpu, ref_img = run_cpu_baseline(so, W, H)
        line["cpu_baseline"] = cpu
        line["bit_exact"] = bool(np.array_equal(ref_img, gpu_img))
        import oracle
        th = oracle.hw_threads()
        flips = {"frame": oracle.fp64_flips(so, oracle.MODE_PIXEL, threads=th, image=gpu_img),
                 "what": "pixels whose colour differs from the FP64 oracle (double arithmetic, 52 bisection "
                         "steps); the GPU image is bit-exact to the FP32 oracle"}
        exact, batch_flips = check_against_oracle(th)
        if batch_flips is not None:
            flips["batch_sample"] = batch_flips
        line["fp64_flips"] = flips
        if batched is not None:
            line["batched"]["bit_exact_vs_oracle"] = exact["batch"]
        if serving is not None:
            line["serving"]["bit_exact_vs_oracle"] = exact["served"]
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def ctypes_stream(stream):
    import ctypes
    return ctypes.c_void_p(stream.cuda_stream)


if __name__ == "__main__":
    sys.exit(main())
