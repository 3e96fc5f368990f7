#!/usr/bin/env python3
"""Benchmark of the GB300 traversal path: Mrays/s closest-hit.

Workload (the raw-traversal configuration): a 1,048,576-triangle float32 soup
(seed 2; centroids uniform in the unit cube, vertices at centroid + 0.005 x a
direction uniform on the sphere) in the reference-built QBVH (binned SAH,
leafMax 16), and 4,194,304 incoherent rays (origins uniform in the cube,
directions uniform on the sphere, tmax = +inf).  A step = one closest-hit
trace of all 4M rays.  Inputs are generated from seeds (no scene files ship
with the reference).

  value  : rays / device time of the trace kernel, rays already in HBM, L2
           flushed (256 MB write) before every timed step
  e2e    : the same trace through the C ABI with pinned host buffers: the
           host->device copy of the rays and device->host copy of the hits
           are inside the timed region
  roofline: algorithmic bytes per launch = rays * 44 + 128 * node visits +
           48 * triangle tests (visit counts from the kernel's counters, which
           equal the oracle's), over the kernel's average duration, against
           the measured HBM copy bandwidth

`--impl reference` times the reference algorithm on the host cores: the C++
restatement in oracle/ (the Go reference does not build here: no Go
toolchain, and its assembly is amd64-only).
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_TRIS = 1 << 20
N_RAYS = 1 << 22
SEED = 2
METRIC = "Mrays/s closest-hit"
CONFIG = {"workload": "raw traversal: 1,048,576-triangle soup (seed 2), 4,194,304 incoherent rays, closest-hit",
          "triangles": N_TRIS, "rays_per_step": N_RAYS, "leaf_max": 16,
          "l2": "flushed between timed steps (256 MB write); scene data (~55 MB) is L2-resident by design"}


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
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
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def measured_l2_gbs(dev):
    """L2 bandwidth on this GPU: a device copy of a 24 MiB buffer into
    another (48 MiB read + write, resident in the 126 MB L2 after the first
    pass), timed with CUDA events over 64 copies, best of 5.  The traversal's
    working set (nodes + triangles, about 57 MB) is L2-resident too, so its
    algorithmic bytes are reported against this as well as against HBM."""
    import torch
    n = (24 << 20) // 4
    a = torch.ones(n, dtype=torch.float32, device=dev)
    b = torch.empty_like(a)
    for _ in range(8):
        b.copy_(a)
    best = 0.0
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(64):
            b.copy_(a)
        e1.record()
        torch.cuda.synchronize()
        best = max(best, 2 * 4 * n * 64 / (e0.elapsed_time(e1) / 1e3) / 1e9)
    return round(best, 1)


def profiled_traffic():
    """DRAM bytes per launch of the traversal kernel from the committed ncu
    summary (profiles/traverse_soup1m_incoherent.md), or None."""
    p = os.path.join(ROOT, "profiles", "traverse_soup1m_incoherent.md")
    if not os.path.exists(p):
        return None
    for ln in open(p):
        if ln.startswith("traffic_bytes_per_launch:"):
            try:
                return float(ln.split(":", 1)[1].strip())
            except ValueError:
                return None
    return None


def launches_per_step(ctx, n):
    """Kernels of ours per trace call: the traversal, plus the three
    ray-reordering kernels when the tuning enables them (n >= 65536)."""
    t = ctx.get_tuning()
    return 1 + (3 if (t["kernel"] & 8) and n >= (1 << 16) else 0)


def max_over_ranks(values, world, device):
    """The timed durations of a step loop as the job sees them: with N
    replicas (one rank per GPU, no data-path collective) the slowest rank's
    (an all-reduce MAX); one rank: unchanged."""
    if world <= 1:
        return list(values)
    import torch
    import torch.distributed as dist
    t = torch.tensor(list(values), device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.tolist()


def job_value(units_per_rank_step, steps, world, seconds):
    """Whole-job throughput in millions of units per second: every rank
    processes its own units (weak scaling) in the max-over-ranks time."""
    return units_per_rank_step * steps * world / seconds / 1e6


def make_workload():
    from vermeer_gb300 import scenes
    v, ip = scenes.triangle_soup(N_TRIS, SEED)
    rays = scenes.incoherent_rays(N_RAYS, SEED)
    return v, ip, rays


def cpu_baseline(v, ip, rays, threads, sample, min_seconds=0.0, mesh=None):
    """The oracle port on the host cores over a bounded sample of the rays,
    traced again until min_seconds of work (at most 16 passes); returns
    (Mrays/s, seconds, the sample's closest hits, passes, the oracle mesh)."""
    from oracle import orc
    m = mesh if mesh is not None else orc.Mesh(v, ip)
    sub = rays[:sample]
    m.trace(sub[:4096], nthreads=threads)  # warm the caches / thread pool
    t0 = time.perf_counter()
    hits = m.trace(sub, nthreads=threads)
    passes = 1
    while time.perf_counter() - t0 < min_seconds and passes < 16:
        m.trace(sub, nthreads=threads)
        passes += 1
    dt = time.perf_counter() - t0
    return sample * passes / dt / 1e6, dt, hits, passes, m


REF_WORKERS = 5  # core.Render's workers: min(Globals.MaxGoRoutines (default 5), 10) (core/render.go:190)


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    v, ip, rays = make_workload()
    threads = cpu_threads()
    from oracle import orc
    m = orc.Mesh(v, ip)
    m.trace(rays[:1 << 16], nthreads=threads)  # warm the caches / thread pool
    for _ in range(args.warmup):
        m.trace(rays[:1 << 18], nthreads=threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        m.trace(rays, nthreads=threads)  # the whole configured step: all 4,194,304 rays
    dt = time.perf_counter() - t0
    value = N_RAYS * args.steps / dt / 1e6
    w_sample = 1 << 18
    t0 = time.perf_counter()
    m.trace(rays[:w_sample], nthreads=REF_WORKERS)
    wval = w_sample / (time.perf_counter() - t0) / 1e6
    line = {"metric": METRIC, "value": round(value, 4), "unit": "Mrays/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(dt / args.steps * 1e3, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": dict(CONFIG), "impl": "reference",
            "cpu_baseline": {"value": round(value, 4), "unit": "Mrays/s", "cores": threads, "kind": "port",
                             "sample": f"all {N_RAYS} incoherent rays per step, {threads} threads; C++ restatement "
                                       "of qbvh.Trace + PolyMesh.TraceElems (oracle/)",
                             "reference_workers": {"threads": REF_WORKERS, "value": round(wval, 4),
                                                   "sample": f"{w_sample} rays, the reference's default worker "
                                                             "count (core/render.go:190)"}},
            "e2e": {"value": round(value, 4), "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def run_gpu(args):
    import torch
    import torch.distributed as dist
    rank, world, local = dist_env()
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    import vermeer_gb300 as vg
    from vermeer_gb300 import _lib

    global N_RAYS
    N_RAYS = args.rays
    CONFIG["rays_per_step"] = N_RAYS
    v, ip, rays = make_workload()
    ctx = vg.Context(local)
    # A dedicated stream: the kernels and the CUDA events share it.
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    geom = ctx.mesh_build(v, ip)
    soa = np.ascontiguousarray(rays[:, :7].T)  # px py pz dx dy dz tmax
    d_rays = torch.from_numpy(soa).to(dev)
    out = {k: torch.empty(N_RAYS, dtype=torch.int32 if k == "prim" else torch.float32, device=dev)
           for k in ("prim", "t", "u", "v", "w")}
    P = ctypes.c_void_p
    r = _lib.Rays(*[P(d_rays[k].data_ptr()) for k in range(7)], None)
    h = _lib.Hits(P(out["prim"].data_ptr()), None, *[P(out[k].data_ptr()) for k in ("t", "u", "v", "w")])
    L = ctx.L

    def trace(flags):
        st = _lib.TraceStats()
        rc = L.vmr_trace_mesh(ctx.h, geom, ctypes.byref(r), N_RAYS, flags, ctypes.byref(h), ctypes.byref(st))
        if rc != 0:
            raise vg.VmrError(rc, L.vmr_last_error(ctx.h).decode())
        return st

    # Visit counts for the algorithmic byte count: one untimed host-buffer
    # pass with the counters on (they equal the oracle's NodesT/LeafsT sums).
    host_soa = [np.ascontiguousarray(soa[k]) for k in range(7)]
    hr = _lib.Rays(*[h_.ctypes.data_as(P) for h_ in host_soa], None)
    hbuf = {k: np.empty(N_RAYS, np.int32 if k == "prim" else np.float32) for k in ("prim", "t", "u", "v", "w")}
    hh = _lib.Hits(hbuf["prim"].ctypes.data_as(P), None, *[hbuf[k].ctypes.data_as(P) for k in ("t", "u", "v", "w")])
    cst = _lib.TraceStats()
    rc = L.vmr_trace_mesh(ctx.h, geom, ctypes.byref(hr), N_RAYS, 4, ctypes.byref(hh), ctypes.byref(cst))
    if rc != 0:
        raise vg.VmrError(rc, L.vmr_last_error(ctx.h).decode())
    alg_bytes = N_RAYS * 44.0 + 128.0 * cst.node_visits + 48.0 * cst.tri_tests

    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    for _ in range(args.warmup):
        flush.zero_()
        trace(2)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    traverse_ms = []
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        for i in range(args.steps):
            flush.zero_()
            ev[i][0].record(stream)
            trace(2)
            ev[i][1].record(stream)
            traverse_ms.append(ctx.trace_timing()[1])  # the traversal kernel alone
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    ctx.sync()
    kernel_ms = [a.elapsed_time(b) for a, b in ev]
    dev_s = sum(kernel_ms) / 1e3
    dev_s, wall = max_over_ranks([dev_s, wall], world, dev)
    value = job_value(N_RAYS, args.steps, world, dev_s)
    avg_launch_s = sum(traverse_ms) / len(traverse_ms) / 1e3  # dominant kernel

    peak, peak_kind = measured_peaks()
    achieved = alg_bytes / avg_launch_s / 1e9
    l2_gbs = measured_l2_gbs(dev)
    traffic = profiled_traffic()
    clocks = clk.summary()
    e2e, e2e_hits = None, None
    if not args.no_e2e:
        e2e, e2e_hits = measure_e2e(args, ctx, geom, host_soa, hbuf, flush, world)
    line = {"metric": METRIC, "value": round(value, 3), "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(wall / args.steps * 1e3, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": CONFIG, "e2e": e2e,
            "gpu_launches": args.steps * launches_per_step(ctx, N_RAYS),
            "step_ms_device": round(dev_s / args.steps * 1e3, 4),
            "kernel_ms_mean": round(avg_launch_s * 1e3, 4),
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "traffic": traffic,
                         "peak_source": f"{peak_kind} hbm_gbs", "algorithmic_bytes_per_launch": alg_bytes,
                         "node_visits_per_ray": round(cst.node_visits / N_RAYS, 3),
                         "tri_tests_per_ray": round(cst.tri_tests / N_RAYS, 3),
                         "l2": {"achieved": round(achieved, 1), "peak": l2_gbs, "unit": "GB/s",
                                "frac": round(achieved / l2_gbs, 4),
                                "peak_source": "measured in this run: device copy of a 24 MiB buffer (L2-resident), "
                                               "best of 5 x 64 copies"}},
            "clocks": clocks}
    if rank == 0 and not args.no_cpu_baseline:
        threads = cpu_threads()
        sample = N_RAYS
        cval, cdt, chits, cpasses, om = cpu_baseline(v, ip, rays, threads, sample, min_seconds=10.0)
        wsample = min(1 << 20, N_RAYS)
        wval, _, _, _, _ = cpu_baseline(v, ip, rays, REF_WORKERS, wsample, mesh=om)
        line["cpu_baseline"] = {"value": round(cval, 4), "unit": "Mrays/s", "cores": threads, "kind": "port",
                                "sample": f"all {N_RAYS} incoherent rays, {cpasses} passes ({cdt:.1f} s), "
                                          "C++ restatement of qbvh.Trace + PolyMesh.TraceElems (oracle/)",
                                "reference_workers": {"threads": REF_WORKERS, "value": round(wval, 4),
                                                      "sample": f"{wsample} rays, the reference's default "
                                                                "worker count (core/render.go:190)"}}
        if e2e is not None:  # the end-to-end hits against the oracle on the sample
            ok = all(np.array_equal(np.asarray(chits[k]).view(np.uint32), np.asarray(e2e_hits[k][:sample]).view(np.uint32))
                     for k in ("prim", "t", "u", "v", "w"))
            e2e["hits_match_oracle_sample"] = bool(ok)
    if rank == 0 and not args.no_render:
        line["traversal_queries"] = traversal_queries(ctx, geom, d_rays, flush, stream, args)
        line["render"] = render_extras(ctx, args)
    if rank == 0:
        print(json.dumps(line))
    ctx.close()
    if world > 1:
        dist.destroy_process_group()
    return 0


def traversal_queries(ctx, geom, d_incoherent, flush, stream, args):
    """The raw-traversal configuration's other queries on the same soup and
    QBVH: closest hit for the 4,194,304 coherent primaries of a 2048x2048
    pinhole looking at the cube, and any hit (shadow rays) for both ray sets;
    device-timed over 5 steps each, L2 flushed before every step."""
    import torch
    import vermeer_gb300 as vg
    from vermeer_gb300 import _lib, scenes
    P = ctypes.c_void_p
    L = ctx.L
    coh = scenes.coherent_rays(2048)
    d_coh = torch.from_numpy(np.ascontiguousarray(coh[:, :7].T)).to(d_incoherent.device)
    n = coh.shape[0]
    out = {k: torch.empty(n, dtype=torch.int32 if k == "prim" else torch.float32, device=d_incoherent.device)
           for k in ("prim", "t", "u", "v", "w")}
    h = _lib.Hits(P(out["prim"].data_ptr()), None, *[P(out[k].data_ptr()) for k in ("t", "u", "v", "w")])
    res = {}
    for name, dr, flags in (("coherent_closest_hit", d_coh, 2), ("incoherent_any_hit", d_incoherent, 3),
                            ("coherent_any_hit", d_coh, 3)):
        r = _lib.Rays(*[P(dr[k].data_ptr()) for k in range(7)], None)
        st = _lib.TraceStats()

        def step():
            rc = L.vmr_trace_mesh(ctx.h, geom, ctypes.byref(r), n, flags, ctypes.byref(h), ctypes.byref(st))
            if rc != 0:
                raise vg.VmrError(rc, L.vmr_last_error(ctx.h).decode())
        for _ in range(3):
            flush.zero_()
            step()
        ms = []
        for _ in range(5):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            step()
            b.record(stream)
            torch.cuda.synchronize()
            ms.append(a.elapsed_time(b))
        hits = int((out["prim"] >= 0).sum().item())
        res[name] = {"mrays_per_s": round(n * len(ms) / (sum(ms) / 1e3) / 1e6, 2), "ms_per_step": round(sum(ms) / len(ms), 4),
                     "rays": n, "hits": hits}
    return res


def _relmse(a, ref):
    return float(np.mean((a - ref) ** 2 / (ref ** 2 + 1e-2)))


def _median_rel(a, ref):
    return float(np.median((a - ref) ** 2 / (ref ** 2 + 1e-2)))


# The guided arm's configuration on the slit-light room (see guided_slit).
GUIDE = dict(depth=2, alpha_max=0.5, lr=1e-2, train_batches=32, train_steps=32, batch_spp=8)


def guided_slit(ctx, width=1024, plain_spp=256):
    """Equal-time relMSE, guided against plain, on the slit-light room at
    width x width: the 4096-spp float64 plain reference first (untimed), then
    each arm in 8-spp batches with its relMSE after every batch (computed
    outside the timed region) -> a relMSE-versus-wall-time curve per arm.
    The plain arm runs plain_spp samples; the guided arm trains online on
    one-sample batches (GUIDE), then renders with the frozen guide until it
    has used the plain arm's wall time.  guided_time_to_plain_relmse: the
    guided arm's time to reach the plain arm's final relMSE over the plain
    arm's time (null if it does not within that time); plain_time_to_guided
    : the plain time that reaches the guided arm's final relMSE, by
    interpolating the plain curve (relMSE ~ 1/spp beyond its end)."""
    from vermeer_gb300 import scenes
    W = H = width
    sc = scenes.slit_room(200_000, width=W, height=H)
    ctx.load_scene(sc)
    t0 = time.perf_counter()
    ref = np.zeros((H, W, 3), np.float64)
    for k in range(16):
        ctx.render_path(W, H, 256 * k, 256, 99, max_depth=8, fb64=ref)
    t_ref = time.perf_counter() - t0
    ctx.render_path(W, H, 0, 4, 1, max_depth=8)  # warm the graphs
    bs = GUIDE["batch_spp"]

    def curve_point(img, t, spp):
        return {"spp": spp, "wall_s": round(t, 4), "relmse": round(_relmse(img, ref), 5),
                "median_rel_sq_err": round(_median_rel(img, ref), 6)}

    plain = np.zeros((H, W, 3), np.float32)
    tp, pc = 0.0, []
    for k in range(plain_spp // bs):
        t0 = time.perf_counter()
        plain, _ = ctx.render_path(W, H, bs * k, bs, 1, max_depth=8, fb=plain)
        tp += time.perf_counter() - t0
        pc.append(curve_point(plain, tp, bs * (k + 1)))
    # guided: warm its graphs (untimed), then train and render from scratch
    kw = dict(max_depth=8, guided=True, guide_fraction=GUIDE["alpha_max"], guide_depth=GUIDE["depth"])
    ctx.guide_init(7)
    ctx.render_path(W, H, 0, 1, 2, train=True, train_steps=1, **kw)
    ctx.render_path(W, H, 0, 1, 2, **kw)
    ctx.guide_init(7)
    g = np.zeros((H, W, 3), np.float32)
    gc, spp, tg, t_train = [], 0, 0.0, 0.0
    for k in range(GUIDE["train_batches"]):
        t0 = time.perf_counter()
        g, _ = ctx.render_path(W, H, spp, 1, 1, fb=g, train=True, train_steps=GUIDE["train_steps"],
                               train_batch=65536, train_lr=GUIDE["lr"], **kw)
        tg += time.perf_counter() - t0
        spp += 1
    t_train = tg
    gc.append(curve_point(g, tg, spp))
    while tg < tp:
        t0 = time.perf_counter()
        g, _ = ctx.render_path(W, H, spp, bs, 1, fb=g, **kw)
        tg += time.perf_counter() - t0
        spp += bs
        gc.append(curve_point(g, tg, spp))
    target = pc[-1]["relmse"]
    t_hit = next((c["wall_s"] for c in gc if c["relmse"] <= target), None)
    # plain time to the guided arm's final relMSE (relMSE ~ 1/time past the curve's end)
    gfin = gc[-1]["relmse"]
    hit = next((c["wall_s"] for c in pc if c["relmse"] <= gfin), None)
    t_plain_eq = hit if hit is not None else tp * target / gfin
    return {
        "workload": f"slit-light room, 200,000 diffuse triangles, {W}x{H}, depth 8; plain {plain_spp} spp in "
                    f"{bs}-spp batches vs the guided tracer for the same wall time: online training on "
                    f"{GUIDE['train_batches']} one-sample batches ({GUIDE['train_steps']} Adam steps of up to "
                    f"65,536 records each, learning rate {GUIDE['lr']}), then the frozen guide in {bs}-spp batches; "
                    f"the first {GUIDE['depth']} vertices of each path guided, learned selection probability "
                    f"(at most {GUIDE['alpha_max']}); every image keeps all its samples; relMSE = mean over pixels "
                    "and channels of (a - r)^2 / (r^2 + 0.01) against the 4096-spp float64 plain render",
        "reference_spp": 4096, "reference_render_s": round(t_ref, 2),
        "plain": pc[-1], "guided": dict(gc[-1], train_s=round(t_train, 3)),
        "guided_time_to_plain_relmse": None if t_hit is None else round(t_hit / tp, 3),
        "plain_time_to_guided_relmse_over_guided_time": round(t_plain_eq / tg, 3),
        "curve": {"plain": pc, "guided": gc},
    }


def render_extras(ctx, args):
    """The render configurations, measured on the same GPU after the
    headline (each on its own seeded synthetic scene):
      reference_small_room   reference-mode core.Render (direct light, hero
                             wavelength), 256x256 x 16 iterations, bit-parity
                             with the oracle on a 64x64 sample, and the oracle's
                             C++ restatement of the Go renderer timed on the
                             host cores
      extended_sphere_grid   the extended path tracer on the 2,097,152-triangle
                             sphere grid, 1920x1080, depth 8, 64 spp
      batched_jobs           64 uneven static/motion jobs traced in one launch,
                             against one launch per job (default and
                             autotuned launch parameters)
      batched_path_jobs      64 uneven static/motion soups path traced as
                             one batched render (each job its own scene),
                             256x256, 32 spp, depth 5, against one render
                             call per job
      guided_slit            equal-wall-time relMSE (mean and median over
                             pixels) on the slit-light room at 1024x1024
                             against a 4096-spp float64 plain render, with a
                             relMSE-versus-wall-time curve for each arm
      qbvh_build             the 2,097,152-triangle QBVH build (BuildAccel,
                             leafMax 16) by the device builder and by the host
                             builder, with the oracle's single-threaded
                             restatement of the reference builder timed beside
                             them; the two product builds must be identical"""
    from oracle import orc
    from vermeer_gb300 import scenes
    import vermeer_gb300 as vg
    out = {}
    # QBVH build
    bv, bip = scenes.triangle_soup(1 << 21, 3)
    res = {}
    for b, name in ((vg.BUILD_DEVICE, "device"), (vg.BUILD_HOST, "host")):
        ctx.set_builder(b)
        ts = []
        for _ in range(3):
            t0 = time.perf_counter()
            g = ctx.mesh_build(bv, bip)
            ctx.sync()
            ts.append(time.perf_counter() - t0)
        res[name] = (min(ts), ctx.mesh_export(g)["nodes"].tobytes())
    ctx.set_builder(vg.BUILD_AUTO)
    t0 = time.perf_counter()
    orc.Mesh(bv, bip)
    odt = time.perf_counter() - t0
    out["qbvh_build"] = {
        "workload": "2,097,152-triangle soup (seed 3), QBVH leafMax 16, wall time of vmr_mesh_build (upload, build, "
                    "device tables)",
        "device_ms": round(res["device"][0] * 1e3, 2), "host_ms": round(res["host"][0] * 1e3, 2),
        "host_threads": cpu_threads(), "identical": res["device"][1] == res["host"][1],
        "cpu_baseline": {"ms": round(odt * 1e3, 2), "cores": 1, "kind": "port",
                         "sample": "the whole build, oracle/orc_core.cpp (C++ restatement of qbvh.BuildAccel)"}}
    # reference mode, small room, as configured
    sc = scenes.small_room(16384, seed=1)
    ctx.load_scene(sc)
    ctx.render(256, 256, 0, 2, 7)
    fb, st = ctx.render(256, 256, 0, 16, 7)
    ctx.render(256, 256, 0, 2, 7, f32=True)
    fb32, st32 = ctx.render(256, 256, 0, 16, 7, f32=True)
    rel32 = np.abs(fb32 - fb).sum(-1) / np.maximum(np.abs(fb).sum(-1), 1e-3)
    r = orc.Render(sc)
    threads = cpu_threads()
    t0 = time.perf_counter()
    ref = r.run(256, 256, 0, 16, 7, nthreads=threads)  # the whole configured image on the host cores
    cdt = time.perf_counter() - t0
    t0 = time.perf_counter()
    r.run(64, 64, 0, 4, 7, nthreads=REF_WORKERS)
    wdt = time.perf_counter() - t0
    out["reference_small_room"] = {
        "workload": "small room, 16,384-triangle soup + 10-triangle box, 2 TriLights, 256x256, 16 iterations",
        "samples_per_s": round(256 * 256 * 16 / (st["ms"] / 1e3), 1), "device_ms": round(st["ms"], 3),
        "camera_rays": st["camera_rays"], "shadow_rays": st["shadow_rays"],
        "bit_equal_to_oracle_frac": float((fb.view(np.uint32) == ref.view(np.uint32)).all(-1).mean()),
        "float32_shading": {"samples_per_s": round(256 * 256 * 16 / (st32["ms"] / 1e3), 1),
                            "device_ms": round(st32["ms"], 3),
                            "mean_rel_pixel_err_vs_float64": float(rel32.mean()),
                            "p99_rel_pixel_err_vs_float64": float(np.percentile(rel32, 99))},
        "cpu_baseline": {"samples_per_s": round(256 * 256 * 16 / cdt, 1), "cores": threads, "kind": "port",
                         "sample": "the whole 256x256 x 16 image, oracle/orc_render.cpp (C++ restatement of "
                                   "core.Render)",
                         "reference_workers": {"threads": REF_WORKERS, "samples_per_s": round(64 * 64 * 4 / wdt, 1),
                                               "sample": "64x64 x 4 iterations, the reference's default worker "
                                                         "count (core/render.go:190)"}}}
    # extended mode, sphere grid
    sc = scenes.sphere_grid()
    ctx.load_scene(sc)
    W, H = sc["width"], sc["height"]
    ctx.render_path(W, H, 0, 2, 3, max_depth=8)
    fb, st = ctx.render_path(W, H, 0, 64, 3, max_depth=8)
    out["extended_sphere_grid"] = {
        "workload": "16x16 displaced spheres x 8,192 tris + ground, 4 quad lights + environment, 1920x1080, "
                    "depth 8, RR from 3, 64 spp; the scene traced flattened (one mesh over all triangles)",
        "samples_per_s": round(W * H * 64 / (st["ms"] / 1e3), 1),
        "mrays_per_s": round((st["rays"] + st["shadow_rays"]) / (st["ms"] / 1e3) / 1e6, 2),
        "device_ms": round(st["ms"], 3), "rays": st["rays"], "shadow_rays": st["shadow_rays"],
        "graph_replays": st["graph_replays"]}
    # bounce and shadow queues traced in ray-key order (VMR_PATH_SORT_QUEUES)
    # against queue order, 16 spp each
    qs = {}
    for srt in (False, True):
        ctx.render_path(W, H, 0, 2, 3, max_depth=8, sort_queues=srt)
        _, s16 = ctx.render_path(W, H, 0, 16, 3, max_depth=8, sort_queues=srt)
        qs["sorted" if srt else "queue_order"] = round(W * H * 16 / (s16["ms"] / 1e3), 1)
    out["extended_sphere_grid"]["queue_sort_samples_per_s_16spp"] = qs
    # the two-level traversal (VMR_PATH_TWO_LEVEL) against the flattened
    # scene the renders above trace, 16 spp each
    ctx.render_path(W, H, 0, 2, 3, max_depth=8, two_level=True)
    _, s16 = ctx.render_path(W, H, 0, 16, 3, max_depth=8, two_level=True)
    out["extended_sphere_grid"]["two_level_samples_per_s_16spp"] = round(W * H * 16 / (s16["ms"] / 1e3), 1)
    # queue capacity chosen by the path autotuner (8 spp per candidate)
    t0 = time.perf_counter()
    best, table = ctx.autotune_path(W, H, 8, seed=3, max_depth=8)
    tune_s = time.perf_counter() - t0
    _, s16 = ctx.render_path(W, H, 0, 16, 3, max_depth=8)
    ctx.set_path_batch(0)
    out["extended_sphere_grid"]["queue_capacity_autotune"] = {
        "candidates_ms_8spp": {str(k): round(v, 2) for k, v in table.items()}, "best_paths": best,
        "autotune_s": round(tune_s, 2), "tuned_samples_per_s_16spp": round(W * H * 16 / (s16["ms"] / 1e3), 1)}
    # batched uneven jobs: one launch vs one launch per job
    import torch
    rng_sizes = np.exp(np.log(1000) + (np.log(200000) - np.log(1000)) * scenes.uniform(4, 64, 0)).astype(int)
    cam = scenes.coherent_rays(256)
    jobs, host_jobs = [], []
    for j, nt in enumerate(rng_sizes):
        motion = j % 2 == 1
        if motion:
            v, ip = scenes.motion_soup(int(nt), 400 + j, velocity=0.05)
        else:
            v, ip = scenes.triangle_soup(int(nt), 400 + j)
        g = ctx.mesh_build(v, ip, keys=2 if motion else 1, motion_mode=1)
        rays = cam.copy()
        rays[:, 7] = scenes.uniform(500 + j, rays.shape[0], 7).astype(np.float32) if motion else 0.0
        jobs.append((g, torch.from_numpy(np.ascontiguousarray(rays.T)).cuda()))
        host_jobs.append((v, ip, motion, rays))
    nrays = sum(r.shape[1] for _, r in jobs)
    ctx.trace_jobs(jobs)
    _, jst = ctx.trace_jobs(jobs)

    def per_job_ms():
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(torch.cuda.current_stream())
        for g, r in jobs:
            ctx.trace_mesh(g, r)
        b.record(torch.cuda.current_stream())
        torch.cuda.synchronize()
        return a.elapsed_time(b)
    per_job_ms()
    seq_default = per_job_ms()
    t0 = time.perf_counter()
    for g, r in jobs:
        ctx.autotune(g, r)
    tune_s = time.perf_counter() - t0
    seq_tuned = per_job_ms()
    for g, _ in jobs:
        ctx.clear_tuning(g)
    # the reference algorithm on the host: the oracle's restatement of
    # qbvh.Trace / motion traversal, every job's rays one job at a time
    # (traces timed, builds not), on all host threads and on the reference's
    # default worker count
    cpu = {}
    meshes = [(orc.Mesh(v, ip, keys=2 if motion else 1, motion_fixed=motion), rays)
              for v, ip, motion, rays in host_jobs]
    for label, nt in (("all_threads", 0), ("reference_workers", REF_WORKERS)):
        sample = meshes if nt == 0 else meshes[:8]
        t0 = time.perf_counter()
        nr = 0
        for m, rays in sample:
            m.trace(rays, nthreads=nt)
            nr += rays.shape[0]
        cpu[label] = {"mrays_per_s": round(nr / (time.perf_counter() - t0) / 1e6, 3),
                      "threads": cpu_threads() if nt == 0 else nt, "jobs": len(sample), "rays": nr}
    del meshes
    out["batched_jobs"] = {
        "workload": "64 triangle soups, sizes log-uniform in [1k, 200k] (seed 4), every other one with two-key "
                    "linear motion (velocity in a 0.05 ball), 256x256 camera rays each (times uniform in [0, 1) "
                    "for the motion jobs), closest hit",
        "triangles": int(rng_sizes.sum()), "rays": int(nrays),
        "one_launch_mrays_per_s": round(nrays / (jst["kernel_ms"] / 1e3) / 1e6, 2),
        "per_job_launches_mrays_per_s": round(nrays / (seq_default / 1e3) / 1e6, 2),
        "per_job_autotuned_mrays_per_s": round(nrays / (seq_tuned / 1e3) / 1e6, 2),
        "autotune_s": round(tune_s, 2),
        "cpu_baseline": dict(cpu, kind="port",
                             sample="all 64 jobs on all host threads; the first 8 jobs (4 static, 4 motion) on the "
                                    "reference's default worker count; oracle/orc_core.cpp, C++ restatement of "
                                    "qbvh.Trace and the motion traversal, one job after another")}
    # batched path-traced jobs: one launch per stage for all jobs, against one
    # vmr_render_path call per job (each job its own one-mesh scene)
    bj = scenes.batched_jobs()
    ids = [ctx.mesh_build(m["verts"], m["idxp"], keys=m.get("keys", 1), motion_mode=m.get("motion_mode", 0))
           for m in bj["meshes"]]
    ctx.set_shaders(bj["shaders"])
    for g in ids:
        ctx.mesh_set_shading(g, [0])
    ctx.set_lights([])
    ctx.set_disk_lights([])
    ctx.set_sphere_lights([])
    ctx.set_quad_lights([])
    ctx.set_env_light(bj["env"])
    ctx.set_pixel_filter(vg.FILTER_BOX)
    W, H = bj["width"], bj["height"]
    jobs = [dict(geom=g, width=W, height=H, camera=c) for g, c in zip(ids, bj["cameras"])]
    ctx.render_path_jobs(jobs, 0, 1, 5, max_depth=5)
    t0 = time.perf_counter()
    _, jst = ctx.render_path_jobs(jobs, 0, 32, 5, max_depth=5)
    jwall = time.perf_counter() - t0
    t0 = time.perf_counter()
    sep_ms = 0.0
    for g, c in zip(ids, bj["cameras"]):
        ctx.scene_build([g])
        ctx.set_camera(c)
        _, s1 = ctx.render_path(W, H, 0, 32, 5, max_depth=5)
        sep_ms += s1["ms"]
    sep_wall = time.perf_counter() - t0
    n_samp = len(jobs) * W * H * 32
    out["batched_path_jobs"] = {
        "workload": "64 jobs: triangle soups of log-uniform [1k, 200k] triangles (seed 4), every other one with "
                    "two-key linear motion (velocity in a 0.05 ball, shutter [0, 1]); each job 256x256, 32 spp, "
                    "depth 5, RR from 3, Lambert 0.7 under a constant white environment",
        "triangles": int(np.sum(bj["sizes"])),
        "one_call": {"samples_per_s": round(n_samp / (jst["ms"] / 1e3), 1),
                     "mrays_per_s": round((jst["rays"] + jst["shadow_rays"]) / (jst["ms"] / 1e3) / 1e6, 2),
                     "device_ms": round(jst["ms"], 2), "wall_s": round(jwall, 3)},
        "per_job_calls": {"samples_per_s": round(n_samp / (sep_ms / 1e3), 1), "device_ms": round(sep_ms, 2),
                          "wall_s": round(sep_wall, 3)}}
    out["guided_slit"] = guided_slit(ctx)
    return out


def measure_e2e(args, ctx, geom, host_soa, hbuf, flush, world):
    """End to end through the C ABI: pinned host rays in, pinned hits out,
    both copies inside the timed region."""
    import torch
    import vermeer_gb300 as vg
    from vermeer_gb300 import _lib
    P = ctypes.c_void_p
    L = ctx.L
    pin_rays = [torch.from_numpy(host_soa[k]).pin_memory() for k in range(7)]
    pin_out = {k: torch.empty(N_RAYS, dtype=torch.int32 if k == "prim" else torch.float32).pin_memory()
               for k in ("prim", "t", "u", "v", "w")}
    er = _lib.Rays(*[P(t_.data_ptr()) for t_ in pin_rays], None)
    eh = _lib.Hits(P(pin_out["prim"].data_ptr()), None, *[P(pin_out[k].data_ptr()) for k in ("t", "u", "v", "w")])
    est = _lib.TraceStats()

    def e2e_step():
        rc_ = L.vmr_trace_mesh(ctx.h, geom, ctypes.byref(er), N_RAYS, 0, ctypes.byref(eh), ctypes.byref(est))
        if rc_ != 0:
            raise vg.VmrError(rc_, L.vmr_last_error(ctx.h).decode())

    for _ in range(args.warmup):
        e2e_step()
    torch.cuda.synchronize()
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    e2e_s = 0.0
    for _ in range(args.steps):
        flush.zero_()  # L2 flush, outside the timed region
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2e_step()  # synchronous: returns once the hits are in the pinned buffers
        e2e_s += time.perf_counter() - t0
    e2e_s = max_over_ranks([e2e_s], world, torch.device("cuda", torch.cuda.current_device()))[0]
    e2e_value = job_value(N_RAYS, args.steps, world, e2e_s)
    ok = np.array_equal(pin_out["prim"].numpy(), hbuf["prim"])
    hits = {k: pin_out[k].numpy().copy() for k in ("prim", "t", "u", "v", "w")}
    return ({"value": round(e2e_value, 3), "unit": "Mrays/s", "h2d_bytes_per_step": N_RAYS * 7 * 4,
             "d2h_bytes_per_step": N_RAYS * 5 * 4, "hits_match_device_path": bool(ok)}, hits)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-render", action="store_true", help="skip the render configurations")
    ap.add_argument("--rays", type=int, default=N_RAYS, help="rays per step (profiling runs use fewer)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
