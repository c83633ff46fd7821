"""Benchmark of the ray-batch intersection path (one JSON line on rank 0).

Workload (default, --workload path): the 1M-triangle path-tracing frame --
1024x1024, 8 spp (2x4 jittered), 800 displaced icospheres (1,024,000
triangles) through Accelerator "ray-bvh", path integrator to depth 5
(Russian roulette after bounce 3, integrators/path.cpp:43-157) with one
area-light shadow ray per vertex; every camera, bounce and shadow batch of
the frame runs on the device (pbg_render).  One step = one frame.

value     nearest-hit + any-hit rays per second of the frame with the plain
          cluster order, CUDA-event time of the whole frame on the device
          (ray generation, traversal, shading, queue compaction, film).
learned_vs_plain  the same frames with the learned ordering on (online
          training and inference inside each frame's time), their ratio, the
          work counters per ray of both, and whether the images are equal.
e2e       the same frame through the host call pbg_render: camera, light and
          parameters in, the RGB image read back; wall time of the call.
roofline  the traversal launches: algorithmic bytes against the measured HBM
          copy peak, and algorithmic FP32 work (box and triangle tests
          counted by the kernels' counting variants on one extra frame)
          against the nominal FP32 rate.
cpu_baseline  the oracle's restatement of the same frame (same samples,
          SAH BVH + pbrt's triangle test) on all host cores and on one, a
          bounded strided sample of the frame's paths.
parity    the whole frame against the oracle's render of the same seed.

Other workloads: --workload frame (the rayhierarchy direct-lighting frame,
181,250 triangles, 1 camera + 4 shadow batches through the per-batch C ABI)
and --workload batch (64 scenes, one persistent launch per step).

--impl reference runs the reference's CPU path on the same workload (the
oracle port: the reference's own build needs its source tree, which the GPU
host lacks) on all host cores and prints the same line with
"impl": "reference".
--gpus N under torchrun: one replica per GPU ("replicas only": rays are
independent, nothing is exchanged).
"""
from __future__ import annotations

import argparse
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
import pbg_import  # noqa: E402

pbg_import.load()

METRIC = "Mrays/s nearest+any-hit at exact hit-ID match: plain vs learned-ordered, 1 GB300"
# dram__bytes_read.sum + dram__bytes_write.sum of one trace step of the
# 64-scene batch per set walk (walk 2: ncu --set full, the warm-up launch
# after autotuning; walk 4: its nearest-hit and any-hit launches at 7 CTAs
# per SM, ncu DRAM counters on the autotuner's trial runs)
BATCH_STEP_DRAM_BYTES = {2: 1_604_272_000, 4: 1_658_600_000}
# dram__bytes_read.sum + dram__bytes_write.sum of the traversal stage of one
# batch call of the terrain frame (every traversal kernel of the warm-up
# frame's nearest batch and four shadow batches, averaged over the five)
FRAME_TRAVERSAL_DRAM_BYTES = {"rayhierarchy": 148_000_000, "ray-bvh": 116_000_000}
# The traversal is bound by instruction issue, not by HBM: ncu's issue-active
# fraction of the dominant kernel (smsp__issue_active, --set full capture of
# the frame's camera and first shadow batch)
# dram__bytes_read.sum + dram__bytes_write.sum per traversal launch of the
# path frame: the average over the 12 traversal launches of one full-size
# frame (ncu, the walks the autotuner picked, the timed frame of the run)
PATH_LAUNCH_DRAM_BYTES = 175_686_955
# smsp__issue_active of the bounce walks (ncu --set full, bounce 1 of the
# first frame of a 256x256 frame of the same scene: nearest, any-hit)
PATH_ISSUE_ACTIVE = {"walk 6 (nearest)": 0.67, "walk 6 (any-hit)": 0.58, "walk 5 (nearest)": 0.71,
                     "walk 5 (any-hit)": 0.59, "walk 2 (nearest)": 0.72, "walk 2 (any-hit)": 0.50}
FRAME_ISSUE_ACTIVE = {"rayhierarchy": {"rh_split_test_kernel<0,0> (camera, nearest)": 0.72,
                                       "rh_split_test_kernel<1,0> (shadow, any-hit)": 0.73}}
# the kernel of each ray-bvh walk (pbg_params.walk)
WALK_KERNEL = {1: "bvh_kernel", 2: "bvh_persistent_kernel", 3: "bvh_packet_kernel (sorted)",
               4: "bvh_packet_kernel", 5: "wide_walk_kernel", 6: "wide_walk_kernel (warp-spread triangle tests)"}
L2_BYTES = 129 * 1024 * 1024
CAMERA = dict(eye=(0.0, 9.0, -14.0), target=(0.0, 0.0, 0.0), fov=50.0)


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}",
                 "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
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
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx = float(f[1])
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[4 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def max_over_ranks(value: float, world: int) -> float:
    """The slowest rank's time: all-reduce MAX over the process group (a
    CUDA tensor under NCCL, a CPU tensor under gloo)."""
    if world <= 1:
        return float(value)
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank: float, world: int, ms_max: float) -> float:
    """Whole-job throughput in millions of units per second: every replica
    processes units_per_rank, the job takes the slowest rank's time."""
    return units_per_rank * world / (ms_max * 1e-3) / 1e6


def rank_barrier(world: int) -> None:
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def make_workload(scale: float = 1.0):
    from pbrt_gb300 import scenes as S
    sc = S.terrain_icospheres(seed=2)
    res = int(1024 * scale)
    rays = S.pinhole_rays(res, res, CAMERA["eye"], CAMERA["target"], CAMERA["fov"], spp=4,
                          jitter_seed=7)
    return sc, rays


def shadow_batches(rays, prim, t, light_quad, nsamples=4, seed=13):
    """Shadow segments from each hit point to seeded points on the quad light,
    one batch per light sample (core/integrator.cpp:358-455); rays that
    missed are invalid in every batch.  mint = rayEpsilon = 1e-3 t
    (shapes/trianglemesh.cpp:190), maxt = dist (1 - 1e-3) (core/light.h:79-84)."""
    g = np.random.default_rng(seed)
    n = rays.shape[1]
    hit = prim >= 0
    p = rays[0:3] + rays[3:6] * np.where(hit, t, 0)[None]
    q0, q1, q3 = light_quad[0].astype(np.float64), light_quad[1].astype(np.float64), light_quad[3].astype(np.float64)
    out = []
    for _ in range(nsamples):
        u, v = g.random(n), g.random(n)
        lp = q0[:, None] + (q1 - q0)[:, None] * u[None] + (q3 - q0)[:, None] * v[None]
        d = lp - p
        dist = np.sqrt((d ** 2).sum(0))
        dist = np.where(dist > 0, dist, 1.0)
        r = np.empty((8, n), np.float32)
        r[0:3] = p
        r[3:6] = d / dist[None]
        r[6] = np.where(hit, 1e-3 * t, 0.0)
        r[7] = dist * (1 - 1e-3)
        out.append(r)
    return out, hit.astype(np.uint8)


def to_dev(rays):
    import torch
    o = torch.from_numpy(np.ascontiguousarray(np.stack([rays[0], rays[1], rays[2], rays[6]], 1)))
    d = torch.from_numpy(np.ascontiguousarray(np.stack([rays[3], rays[4], rays[5], rays[7]], 1)))
    return o.cuda(), d.cuda()


def run_gpu(args, rank, world, dev):
    import torch
    from pbrt_gb300 import accel as A
    torch.cuda.set_device(dev)
    sc, rays = make_workload()
    tris = sc["tris"]
    n = rays.shape[1]
    acc = A.MakeAccelerator(args.accel, tris, {"device": dev, "clusterLevels": args.rh_cluster_levels,
                                               "walk": args.walk})
    # the breadth-first renderer's ray image: one tile of 1024 x 1024 pixels x 4 spp
    acc.Preprocess(None, 4, 1, 1, xres=1024, yres=1024)
    stream = torch.cuda.Stream()
    o4, d4 = to_dev(rays)
    prim = torch.empty(n, dtype=torch.int32, device="cuda")
    tt, b1, b2 = (torch.empty(n, device="cuda") for _ in range(3))
    with torch.cuda.stream(stream):
        acc.intersect_device(o4, d4, prim, tt, b1, b2, stream=stream)
    stream.synchronize()
    hp, ht = prim.cpu().numpy(), tt.cpu().numpy()
    shadows, hitmask = shadow_batches(rays, hp, ht, sc["area_light_quad"])
    sdev = [to_dev(s) for s in shadows]
    valid = torch.from_numpy(hitmask).cuda()
    occ = torch.empty(n, dtype=torch.uint8, device="cuda")
    nhit = int(hitmask.sum())
    rays_per_step = n + len(shadows) * nhit
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")
    tuned = None
    if not args.no_tune:  # launch shapes for the camera batch and the shadow batches
        tuned = {"camera (nearest)": acc.autotune(o4, d4, stream=stream),
                 "shadow (any-hit)": acc.autotune(sdev[0][0], sdev[0][1], anyhit=True, valid=valid,
                                                  stream=stream)}
        stream.synchronize()

    def step():
        acc.intersect_device(o4, d4, prim, tt, b1, b2, stream=stream)
        for so, sd in sdev:
            acc.occluded_device(so, sd, occ, valid=valid, stream=stream)

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            step()
    stream.synchronize()
    acc.stats()
    launches0 = acc.stats()["kernel_launches"]
    acc.profile(True)
    times = []
    rank_barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(dev) as clk:
        for _ in range(args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(1.0)  # evict L2 between steps, outside the timed region
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                step()
                e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
    torch.cuda.synchronize()
    rank_barrier(world)
    st = acc.stats()
    acc.profile(False)
    launches = st["kernel_launches"] - launches0
    step_ms = sum(times) / len(times)
    step_ms = max_over_ranks(step_ms, world)

    # dominant kernel: the traversal stage (event-timed inside the library)
    trav_ms = st["stage_ms"]["traverse"]
    trav_launches = st["timed_launches"]["traverse"]
    valid_shadow = nhit
    # algorithmic bytes per traversal launch (averaged over the step's five):
    # rays read once (32 B), scene records read once (48 B + 16 B sphere),
    # results written once (8 B key nearest, 1 bit any-hit)
    step_bytes = (n * 32 + n * 8 + len(shadows) * (valid_shadow * 32 + valid_shadow / 8)
                  + (1 + len(shadows)) * len(tris) * 64)
    # one unit = the traversal stage of one batch call (one launch for
    # ray-bvh and naive; seed, expand, split + leaf tests, leaf sort and leaf
    # tests for rayhierarchy), event-timed inside the library
    calls = (1 + len(shadows)) * args.steps
    per_launch_bytes = step_bytes / (1 + len(shadows))
    avg_launch_ms = trav_ms / max(calls, 1)
    hbm, peak_kind = peaks()
    achieved = per_launch_bytes / (avg_launch_ms * 1e-3) / 1e9
    traffic = FRAME_TRAVERSAL_DRAM_BYTES.get(args.accel)

    # parity sample: hit IDs of a ray sample against the oracle port (CPU)
    parity = None
    if rank == 0 and not args.no_parity:
        from oracle import oracle as O
        sel = np.arange(0, n, max(1, n // 8192))
        got = prim.cpu().numpy()[sel]
        B = O.BVH(tris)
        want = B.nearest(rays[:, sel])[0]
        occ_got = occ.cpu().numpy()[sel]
        occ_want = B.anyhit(shadows[-1][:, sel], valid=hitmask[sel])
        parity = {"sample_rays": int(2 * len(sel)),
                  "hit_id_mismatches": int((got != want).sum()),
                  "occlusion_mismatches": int((occ_got != occ_want).sum())}

    e2e = run_e2e(args, acc, rays, shadows, hitmask, rays_per_step) if rank == 0 else None
    cpu = cpu_baseline(tris, rays, shadows, hitmask) if (rank == 0 and world == 1 and not args.no_cpu) else None
    if rank == 0:
        clocks = clk.summary()
        value = job_rate(rays_per_step, world, step_ms)
        line = {
            "metric": METRIC, "value": round(value, 2), "unit": "Mrays/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(step_ms, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded terrain + icospheres, seeded jitter and light samples)",
            "config": {"workload": "rayhierarchy direct lighting 1024x1024x4spp, 181,250 triangles, "
                                   "1 nearest + 4 shadow batches per frame",
                       "accelerator": args.accel, "rays_per_step": rays_per_step,
                       "primary_rays": n, "shadow_rays": len(shadows) * nhit,
                       "triangles": int(len(tris)), "parallelism": f"replicas x{world}",
                       "l2": "flushed between steps (256 MB write), outside the timed region",
                       "autotune": {k: v["best"] for k, v in tuned.items()} if tuned else None},
            "autotune": tuned,
            "e2e": e2e,
            "roofline": {"bound": "hbm", "achieved": round(achieved, 2), "peak": hbm,
                         "unit": "GB/s", "frac": round(achieved / hbm, 5),
                         "traffic": traffic, "kernel": "traversal stage of one batch call",
                         "launches_per_unit": round(trav_launches / max(calls, 1), 2),
                         "algorithmic_bytes_per_launch": int(per_launch_bytes),
                         "avg_launch_ms": round(avg_launch_ms, 4), "peak_source": peak_kind,
                         "issue_active": FRAME_ISSUE_ACTIVE.get(args.accel)},
            "stage_ms_per_step": {k: round(v / args.steps, 4) for k, v in st["stage_ms"].items()},
            "gpu_launches": int(launches),
            "cpu_baseline": cpu,
            "parity": parity,
            "clocks": clocks,
        }
        print(json.dumps(line), flush=True)


PATH_CAMERA = dict(eye=(0.0, 6.0, -62.0), look=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0), fov=42.0)
PATH_LIGHT = np.array([[-12, 32, -12], [12, 32, -12], [12, 32, 12], [-12, 32, 12]], np.float32)
PATH_LIGHT_L = (12.0, 12.0, 12.0)
PATH_RES, PATH_SPP, PATH_DEPTH = 1024, (2, 4), 5
PATH_WORKLOAD = ("ray-bvh path tracing 1024x1024x8spp (2x4 jittered), 1,024,000 triangles "
                 "(800 displaced icospheres), depth 5, one area-light sample per vertex, "
                 "whole frame on device")
# Algorithmic FP32 work per counted unit (an FMA counts as 2 FLOP): a slab
# test of one child box with the ray's reciprocal direction precomputed is
# 6 subtractions + 6 multiplications; a ray/triangle test by Moller-Trumbore
# stage is 24 FLOP (s1 = d x e2, divisor, 1/divisor, o - p1, b1), then 15
# (s2 = v x e1, b2) and 6 (t); pbrt's exact test is all three stages.
FLOP_BOX, FLOP_STAGE1, FLOP_STAGE23, FLOP_EXACT = 12, 24, 21, 45


def fp32_peak_tflops(sm_mhz):
    """Nominal dense FP32 rate: SMs x 128 FP32 lanes x 2 FLOP (FMA) x clock."""
    import torch
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    return sms * 128 * 2 * sm_mhz * 1e6 / 1e12, sms


def cpu_model():
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.startswith("Model name:"):
                return ln.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        for ln in open("/proc/cpuinfo"):
            if ln.lower().startswith("model name"):
                return ln.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform
    return platform.machine()


def path_setup():
    from pbrt_gb300 import render as R
    from pbrt_gb300 import scenes as S
    sc = S.displaced_icospheres(seed=3)
    r2c, c2w = R.perspective_camera(PATH_RES, PATH_RES, PATH_CAMERA["eye"], PATH_CAMERA["look"],
                                    PATH_CAMERA["up"], PATH_CAMERA["fov"])
    return sc, r2c, c2w


def path_cpu_counter(tris, r2c, c2w, seed):
    from oracle import oracle as O
    lights = [{"type": "quad", "quad": PATH_LIGHT, "L": PATH_LIGHT_L, "nsamples": 1}]
    return O.RenderCounter(tris, r2c, c2w, PATH_RES, PATH_RES, lights, "path", PATH_SPP, True,
                           PATH_DEPTH, seed)


def timed_cpu_sample(rc, threads, target_s, seed):
    """Traces a strided subset of the frame's samples sized to about target_s
    seconds on `threads` host threads; returns (rays, seconds, stride)."""
    # the probe traces about 65,536 samples: enough that thread start-up
    # does not dominate its time
    probe = max(1, rc.samples // 65536)
    t0 = time.perf_counter()
    n0, s0 = rc.count(0, probe, threads, seed)
    dt = max(time.perf_counter() - t0, 1e-4)
    per_sample = dt / max(1, (rc.samples + probe - 1) // probe)
    stride = max(1, int(rc.samples * per_sample / target_s))
    t0 = time.perf_counter()
    n, s = rc.count(1, stride, threads, seed)
    return n + s, time.perf_counter() - t0, stride


def ordering_study(acc, reps=5):
    """What a cluster ordering can gain on the path scene.  Any-hit: shadow
    segments from the camera hits of a 1024x1024 image (1 spp) to random
    points on the area light; nearest-hit: those camera rays.  Times (CUDA
    events on the launch stream) and counted work per ray of the plain walk,
    of the walk with perfect hints (each ray's own occluder or first-hit
    cluster: the ceiling of any ordering), and of the learned ordering when
    the scene has a trained network (its inference and record collection
    included)."""
    import torch
    from pbrt_gb300 import scenes as S
    rays = S.pinhole_rays(PATH_RES, PATH_RES, PATH_CAMERA["eye"], PATH_CAMERA["look"], PATH_CAMERA["fov"], spp=1,
                          jitter_seed=21)
    n = rays.shape[1]
    o4, d4 = to_dev(rays)
    prim = torch.empty(n, dtype=torch.int32, device="cuda")
    tt, b1, b2 = (torch.empty(n, device="cuda") for _ in range(3))
    acc.intersect_device(o4, d4, prim, tt, b1, b2)
    torch.cuda.synchronize()
    hp, ht = prim.cpu().numpy(), tt.cpu().numpy()
    shadows, hit = shadow_batches(rays, hp, ht, PATH_LIGHT, nsamples=1, seed=23)
    so, sd = to_dev(shadows[0])
    valid = torch.from_numpy(hit).cuda()
    occ = torch.empty(n, dtype=torch.uint8, device="cuda")
    occluder = torch.empty(n, dtype=torch.int32, device="cuda")
    hint = torch.empty(n, dtype=torch.int16, device="cuda")
    stream = torch.cuda.Stream()

    def timed(fn, nrays):
        with torch.cuda.stream(stream):
            fn()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(reps):
                fn()
            e1.record(stream)
        e1.synchronize()
        acc.profile(2)
        with torch.cuda.stream(stream):
            fn()
        stream.synchronize()
        w = acc.stats()["work"]
        acc.profile(False)
        nv = max(int(nrays), 1)
        return {"ms": round(e0.elapsed_time(e1) / reps, 4),
                "node_tests_per_ray": round(w["node_tests"] / nv, 3),
                "triangle_tests_per_ray": round(w["filter_tests"] / nv, 3)}

    learner_on = acc.learn_stats()["trained_steps"] > 0
    if learner_on:
        acc.learn_enable(True, queries=2)
        learned = timed(lambda: acc.occluded_device(so, sd, occ, valid=valid, stream=stream), hit.sum())
        occ_l = occ.clone()
        acc.learn_enable(False)
    # the plain legs pass "no cluster" for every ray, so that plain and
    # hinted walks run the same kernel
    none = torch.full((n,), -1, dtype=torch.int16, device="cuda")
    plain = timed(lambda: acc.occluded_hinted_device(so, sd, none, occ, occluder, valid=valid, stream=stream),
                  hit.sum())
    occ_p = occ.clone()
    acc.clusters_of_device(occluder, hint, stream=stream)
    perfect = timed(lambda: acc.occluded_hinted_device(so, sd, hint, occ, valid=valid, stream=stream), hit.sum())
    same = bool(torch.equal(occ, occ_p)) and (not learner_on or bool(torch.equal(occ_l, occ_p)))
    out = {"shadow_rays": int(hit.sum()), "occluded_fraction": round(float(occ_p.float().sum()) / max(int(hit.sum()), 1), 4),
           "plain": plain, "perfect_hints": perfect,
           "perfect_over_plain_time": round(plain["ms"] / perfect["ms"], 3), "results_identical": same}
    if learner_on:
        out["learned"] = learned
        out["learned_over_plain_time"] = round(plain["ms"] / learned["ms"], 3)
    # nearest hit: the camera rays themselves, hinted with their own first hit
    nhint = torch.empty(n, dtype=torch.int16, device="cuda")
    p2, t2, c1, c2 = (torch.empty_like(x) for x in (prim, tt, b1, b2))
    nplain = timed(lambda: acc.intersect_hinted_device(o4, d4, none, p2, t2, c1, c2, stream=stream), n)
    acc.clusters_of_device(prim, nhint, stream=stream)
    nperfect = timed(lambda: acc.intersect_hinted_device(o4, d4, nhint, p2, t2, c1, c2, stream=stream), n)
    out["nearest"] = {"camera_rays": n, "plain": nplain, "perfect_hints": nperfect,
                      "perfect_over_plain_time": round(nplain["ms"] / nperfect["ms"], 3),
                      "results_identical": bool(torch.equal(p2, prim) and torch.equal(t2, tt))}
    return out


def path_tuning(acc, tris):
    """pbg_autotune on batches shaped like the path frame's own, one per
    batch class: the camera rays (8 jittered samples per pixel, consecutive)
    and the shadow rays from their hits to the light (coherent), and bounce
    rays (cosine-weighted directions from 2 M of the camera hits) with the
    shadow rays from their hits (incoherent).  Queues are compacted as the
    renderer compacts them (no validity masks)."""
    import torch
    from pbrt_gb300 import scenes as S

    def nearest(o4, d4):
        n = o4.shape[0]
        prim = torch.empty(n, dtype=torch.int32, device="cuda")
        t, b1, b2 = (torch.empty(n, device="cuda") for _ in range(3))
        acc.intersect_device(o4, d4, prim, t, b1, b2)
        torch.cuda.synchronize()
        return prim.cpu().numpy(), t.cpu().numpy()

    def shadow_queue(rays, prim, t, seed):
        sh, hit = shadow_batches(rays, prim, t, PATH_LIGHT, nsamples=1, seed=seed)
        return to_dev(np.ascontiguousarray(sh[0][:, hit == 1]))

    cam = S.pinhole_rays(PATH_RES, PATH_RES, PATH_CAMERA["eye"], PATH_CAMERA["look"], PATH_CAMERA["fov"],
                         spp=PATH_SPP[0] * PATH_SPP[1], jitter_seed=5)
    co4, cd4 = to_dev(cam)
    hp, ht = nearest(co4, cd4)
    so4, sd4 = shadow_queue(cam, hp, ht, 29)
    tuned = {"coherent nearest": acc.autotune(co4, cd4), "coherent any-hit": acc.autotune(so4, sd4, anyhit=True)}
    del co4, cd4, so4, sd4
    g = np.random.default_rng(31)
    idx = np.flatnonzero(hp >= 0)
    idx = idx[:: max(1, len(idx) // (1 << 21))][: 1 << 21]
    v = tris[hp[idx]].reshape(-1, 3, 3).astype(np.float64)
    nrm = np.cross(v[:, 1] - v[:, 0], v[:, 2] - v[:, 0])
    nrm /= np.maximum(np.linalg.norm(nrm, axis=1, keepdims=True), 1e-30)
    nrm *= np.where((nrm * cam[3:6, idx].T).sum(1, keepdims=True) > 0, -1.0, 1.0)
    b = np.empty((8, len(idx)), np.float32)
    b[0:3] = cam[0:3, idx] + cam[3:6, idx] * ht[idx][None]
    b[3:6] = S._cosine_dirs(nrm, g).T
    b[6] = 1e-3 * ht[idx]
    b[7] = np.inf
    bo4, bd4 = to_dev(b)
    bp, bt = nearest(bo4, bd4)
    bso4, bsd4 = shadow_queue(b, bp, bt, 37)
    tuned["incoherent nearest"] = acc.autotune(bo4, bd4, incoherent=True)
    tuned["incoherent any-hit"] = acc.autotune(bso4, bsd4, anyhit=True, incoherent=True)
    torch.cuda.synchronize()
    return tuned


def run_gpu_path(args, rank, world, dev):
    """The ray-bvh path-tracing frame: 1024x1024 x 8 spp (2x4 jittered) on
    800 displaced icospheres (1,024,000 triangles), path integrator to depth
    5 with Russian roulette after bounce 3, one area-light shadow ray per
    vertex; the whole frame runs on the device (pbg_render).  value = the
    plain ordering; the learned ordering is measured on the same frames."""
    import torch
    from pbrt_gb300 import accel as A
    from pbrt_gb300 import render as R
    torch.cuda.set_device(dev)
    sc, r2c, c2w = path_setup()
    tris = sc["tris"]
    t0 = time.perf_counter()
    acc = A.MakeAccelerator("ray-bvh", tris, {"device": dev, "raySort": int(args.ray_sort), "walk": args.walk,
                                              "bvhBuild": args.bvh_build, "maxBVHPrim": args.max_leaf})
    build_s = time.perf_counter() - t0
    cam = R.camera_struct(r2c, c2w, PATH_RES, PATH_RES)
    light = R.quad_light(PATH_LIGHT, PATH_LIGHT_L, 1)
    prm = R.render_params("path", spp=PATH_SPP, jitter=True, max_depth=PATH_DEPTH, seed=17)
    tuned = path_tuning(acc, tris) if not args.no_tune else None

    def measure():
        for k in range(args.warmup):
            prm.seed = 500 + k
            R.render(acc, cam, [light], prm)
        torch.cuda.synchronize()
        l0 = acc.stats()["kernel_launches"]
        acc.profile(True)
        frames, walls = [], []
        rank_barrier(world)
        torch.cuda.synchronize()
        with ClockSampler(dev) as clk:
            for k in range(args.steps):
                prm.seed = 1000 + k  # the same frames in every mode
                w0 = time.perf_counter()
                img, st = R.render(acc, cam, [light], prm)
                walls.append(time.perf_counter() - w0)
                frames.append(st)
        torch.cuda.synchronize()
        rank_barrier(world)
        stt = acc.stats()
        acc.profile(False)
        return frames, walls, stt, clk.summary(), stt["kernel_launches"] - l0, img

    def count_work(seed):
        """One more frame with the counting kernels (profiling level 2)."""
        acc.profile(2)
        prm.seed = seed
        _, st = R.render(acc, cam, [light], prm)
        w = acc.stats()["work"]
        acc.profile(False)
        return w, st

    def rate(frames):
        rays = sum(f["nearest_rays"] + f["shadow_rays"] for f in frames) / len(frames)
        ms = sum(f["ms_total"] for f in frames) / len(frames)
        return rays, ms

    frames, walls, stt, clocks, launches, img_plain = measure()
    rays, frame_ms = rate(frames)
    work, wst = count_work(1000)
    learned_line = None
    if args.learned:
        acc.learn_enable(True, seed=5, steps_per_train=args.learn_steps, lr=args.learn_lr,
                         margin=args.learn_margin, queries=args.learn_queries)
        lf, lw, lstt, lclocks, llaunch, img_learned = measure()
        lwork, _ = count_work(1000)
        ls = acc.learn_stats()
        l_rays, l_ms = rate(lf)
        learned_line = {
            "plain_mrays_s": round(rays / (frame_ms * 1e-3) / 1e6, 2),
            "learned_mrays_s": round(l_rays / (l_ms * 1e-3) / 1e6, 2),
            "learned_over_plain": round((l_rays / l_ms) / (rays / frame_ms), 3),
            "learned_traversal_ms_per_step": round(lstt["stage_ms"]["traverse"] / args.steps, 3),
            "plain_traversal_ms_per_step": round(stt["stage_ms"]["traverse"] / args.steps, 3),
            "images_identical": bool(np.array_equal(img_plain, img_learned)),
            "work_per_ray": {
                "plain": {k: round(v / (wst["nearest_rays"] + wst["shadow_rays"]), 3) for k, v in work.items()},
                "learned": {k: round(v / (wst["nearest_rays"] + wst["shadow_rays"]), 3) for k, v in lwork.items()}},
            "mlp": {"trained_steps": ls["trained_steps"], "records": ls["records"],
                    "last_loss": round(ls["last_loss"], 4), "top1_accuracy": round(ls["last_accuracy"], 4),
                    "train_ms_total": round(ls["train_ms"], 2), "infer_ms_total": round(ls["infer_ms"], 2)},
        }
        learned_line["ordering_ceiling"] = ordering_study(acc)
        if args.learned == 1:  # the learned-ordered form as the value
            frames, walls, stt, clocks, launches = lf, lw, lstt, lclocks, llaunch
            rays, frame_ms = l_rays, l_ms
            work = lwork
    frame_ms = max_over_ranks(frame_ms, world)
    if rank != 0:
        return
    trav_ms = stt["stage_ms"]["traverse"] / args.steps
    hbm, peak_kind = peaks()
    n_launch = max(stt["timed_launches"]["traverse"], 1)
    launches_per_frame = n_launch / args.steps
    # HBM: every traced ray read once (32 B) and its result written once
    # (16 B nearest, 1 B any-hit), the triangle records read once per launch
    near_rays = sum(f["nearest_rays"] for f in frames) / len(frames)
    sh_rays = sum(f["shadow_rays"] for f in frames) / len(frames)
    per_launch_bytes = (near_rays * 48 + sh_rays * 33) / launches_per_frame + len(tris) * 48
    avg_launch_ms = stt["stage_ms"]["traverse"] / n_launch
    achieved = per_launch_bytes / (avg_launch_ms * 1e-3) / 1e9
    # FP32: the counted frame's work over its own traversal share of the frame
    flops_frame = (work["node_tests"] * FLOP_BOX + work["filter_tests"] * FLOP_STAGE1
                   + work["filter_stage2"] * FLOP_STAGE23 + work["exact_tests"] * FLOP_EXACT)
    flops_per_launch = flops_frame / launches_per_frame
    fp32_achieved = flops_per_launch / (avg_launch_ms * 1e-3) / 1e12
    fp32_peak, sms = fp32_peak_tflops(clocks.get("sm_max_mhz") or 2070.0)
    # CPU baseline: the oracle's restatement of the same frame (same seed,
    # same samples) on the host cores, a bounded strided sample
    cpu = None
    if not args.no_cpu and world == 1:
        rc = path_cpu_counter(tris, r2c, c2w, 1000)
        threads = os.cpu_count() or 1
        r_all, s_all, stride_all = timed_cpu_sample(rc, threads, 10.0, 1000)
        r_one, s_one, stride_one = timed_cpu_sample(rc, 1, 3.0, 1000)
        cpu = {"value": round(r_all / s_all / 1e6, 3), "unit": "Mrays/s", "cores": threads, "kind": "port",
               "seconds": round(s_all, 2), "cpu_model": cpu_model(),
               "sample": (f"every {stride_all}th sample of the same frame" if stride_all > 1 else "the whole frame")
                         + f" ({r_all} nearest + shadow rays), depth-first path per sample, "
                           "SAH BVH + pbrt's triangle test (oracle/render_oracle.c)",
               "single_core": {"value": round(r_one / s_one / 1e6, 3), "cores": 1, "seconds": round(s_one, 2),
                               "sample": f"every {stride_one}th sample ({r_one} rays)"}}
        del rc
    parity = None
    if not args.no_parity and world == 1:
        # the whole frame against the oracle's render of the same seed
        from oracle import oracle as O
        lights = [{"type": "quad", "quad": PATH_LIGHT, "L": PATH_LIGHT_L, "nsamples": 1}]
        prm.seed = 1000
        img_gpu, _ = R.render(acc, cam, [light], prm)
        c0 = time.perf_counter()
        img_cpu = O.render(tris, r2c, c2w, PATH_RES, PATH_RES, lights, "path", PATH_SPP, True, PATH_DEPTH,
                           1000)
        diff = img_gpu.astype(np.float64) - img_cpu.astype(np.float64)
        parity = {"image": f"{PATH_RES}x{PATH_RES}x{PATH_SPP[0] * PATH_SPP[1]}spp frame, seed 1000",
                  "rmse_vs_oracle": float(np.sqrt(np.mean(diff ** 2))),
                  "pixels_differing": int(np.count_nonzero(np.any(diff != 0, axis=2))),
                  "tolerance": "RMSE <= 1e-4", "oracle_seconds": round(time.perf_counter() - c0, 2)}
    line = {
        "metric": METRIC, "value": round(job_rate(rays, world, frame_ms), 2), "unit": "Mrays/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(frame_ms, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded displaced icospheres, counter-hash samples)",
        "config": {"workload": PATH_WORKLOAD, "accelerator": "ray-bvh",
                   "ordering": "learned" if args.learned == 1 else "plain",
                   "rays_per_step": int(rays), "nearest_rays": int(near_rays), "shadow_rays": int(sh_rays),
                   "triangles": int(len(tris)), "bvh_build_s": round(build_s, 2),
                   "bvh_nodes": int(acc.stats()["bvh_nodes"]),
                   "wide_nodes": int(acc.stats()["wide_nodes"]),
                   "wide_build_s": round(acc.stats()["wide_build_ms"] * 1e-3, 3),
                   "ray_sort": bool(args.ray_sort), "walk": args.walk,
                   "bvh_build": "host" if args.bvh_build == 1 else "device", "parallelism": f"replicas x{world}",
                   "l2": "inputs > L2 (8.4M paths x 32 B rays per bounce)",
                   "autotune": {k: v["best"] for k, v in tuned.items()} if tuned else None},
        "autotune": tuned,
        "traversal_mrays_s": round(rays / (trav_ms * 1e-3) / 1e6, 2),
        "e2e": {"value": round(rays / (sum(walls) / len(walls)) / 1e6, 2), "unit": "Mrays/s",
                "ms_per_step": round(sum(walls) / len(walls) * 1e3, 3),
                "h2d_bytes_per_step": 256 + 112, "d2h_bytes_per_step": PATH_RES * PATH_RES * 12,
                "api": "pbg_render (camera, light and parameters in, RGB image out; wall time of the host call)"},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 2), "peak": hbm, "unit": "GB/s",
                     "frac": round(achieved / hbm, 5), "traffic": PATH_LAUNCH_DRAM_BYTES,
                     "kernel": "traversal launch (" + ", ".join(
                         f"{k}: {WALK_KERNEL.get(v['best'].get('walk'), 'walk %s' % v['best'].get('walk'))}"
                         for k, v in tuned.items()) + ")" if tuned else
                     "traversal launch (the automatic walks: bvh_kernel on bounce 0, bvh_persistent_kernel after)",
                     "launches_per_step": round(launches_per_frame, 2),
                     "algorithmic_bytes_per_launch": int(per_launch_bytes),
                     "avg_launch_ms": round(avg_launch_ms, 4), "peak_source": peak_kind + " (of measured copy)",
                     "fp32": {"achieved_tflops": round(fp32_achieved, 3), "peak_tflops": round(fp32_peak, 1),
                              "frac": round(fp32_achieved / fp32_peak, 5),
                              "flops_per_launch": int(flops_per_launch),
                              "peak_source": f"nominal: {sms} SMs x 128 FP32 lanes x 2 x max SM clock",
                              "counted": {k: int(v) for k, v in work.items()},
                              "flop_per_unit": {"box_test": FLOP_BOX, "tri_stage1": FLOP_STAGE1,
                                                "tri_stage2_3": FLOP_STAGE23, "exact_test": FLOP_EXACT}},
                     "issue_active": PATH_ISSUE_ACTIVE},
        "stage_ms_per_step": {k: round(v / args.steps, 4) for k, v in stt["stage_ms"].items()},
        "gpu_launches": int(launches),
        "learned_vs_plain": learned_line,
        "cpu_baseline": cpu,
        "parity": parity,
        "clocks": clocks,
    }
    print(json.dumps(line), flush=True)


NAIVE_WORKLOAD = ("naive direct lighting 256x256x1spp at pixel centres, UV sphere + ground quad "
                  "(4,034 triangles), point light, whole frame on device")


def flush_l2(buf):
    """Overwrites a buffer larger than L2 (129 MB) so the next frame starts
    with a cold cache."""
    buf.add_(1.0)


def run_gpu_naive(args, rank, world, dev):
    """Accelerator "naive" on its small workload: 256x256 at pixel centres,
    one camera ray and one point-light shadow ray per pixel, every ray
    against all 4,034 triangles; the whole frame runs on the device
    (pbg_render).  The inputs fit in L2, so L2 is flushed before every
    frame.  The camera matrices and the light come from the reference's own
    render of this scene (tests/golden/render_small.npz), and the image is
    compared with that render."""
    import torch
    from pbrt_gb300 import accel as A
    from pbrt_gb300 import render as R
    from pbrt_gb300 import scenes as S
    torch.cuda.set_device(dev)
    g = dict(np.load(os.path.join(ROOT, "tests", "golden", "render_small.npz")))
    tris = S.config_small_naive()["tris"]
    acc = A.MakeAccelerator("naive", tris, {"device": dev})
    acc.Preprocess(None, 1, 1, 1, xres=256, yres=256)
    cam = R.camera_struct(g["r2c"], g["c2w"], 256, 256)
    light = R.point_light(g["light_pos"], g["light_I"])
    prm = R.render_params("directlighting")
    flush = torch.zeros(64 << 20, dtype=torch.float32, device="cuda")  # 256 MB
    tuned = None
    if not args.no_tune:  # the splits' launch shape, on the frame's camera rays and its shadow rays
        cr = S.config_small_naive()["rays"]
        o4, d4 = to_dev(cr)
        tuned = {"camera (nearest)": acc.autotune(o4, d4)}
        n0 = cr.shape[1]
        prim = torch.empty(n0, dtype=torch.int32, device="cuda")
        tt, b1, b2 = (torch.empty(n0, device="cuda") for _ in range(3))
        acc.intersect_device(o4, d4, prim, tt, b1, b2)
        torch.cuda.synchronize()
        hp, ht = prim.cpu().numpy(), tt.cpu().numpy()
        hit = hp >= 0
        p = cr[0:3, hit] + cr[3:6, hit] * ht[hit][None]
        dl = g["light_pos"].astype(np.float32)[:, None] - p
        dist = np.sqrt((dl ** 2).sum(0))
        sh = np.empty((8, int(hit.sum())), np.float32)
        sh[0:3] = p
        sh[3:6] = dl / dist[None]
        sh[6] = 1e-3 * ht[hit]
        sh[7] = dist * (1 - 1e-3)
        so4, sd4 = to_dev(sh)
        tuned["shadow (any-hit)"] = acc.autotune(so4, sd4, anyhit=True)
        torch.cuda.synchronize()
    for _ in range(args.warmup):
        flush_l2(flush)
        R.render(acc, cam, [light], prm)
    torch.cuda.synchronize()
    l0 = acc.stats()["kernel_launches"]
    acc.profile(True)
    frames, walls = [], []
    rank_barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(dev) as clk:
        for _ in range(args.steps):
            flush_l2(flush)
            torch.cuda.synchronize()
            w0 = time.perf_counter()
            img, st = R.render(acc, cam, [light], prm)
            walls.append(time.perf_counter() - w0)
            frames.append(st)
    torch.cuda.synchronize()
    rank_barrier(world)
    stt = acc.stats()
    acc.profile(False)
    launches = stt["kernel_launches"] - l0
    clocks = clk.summary()
    acc.profile(2)
    flush_l2(flush)
    _, wst = R.render(acc, cam, [light], prm)
    work = acc.stats()["work"]
    acc.profile(False)
    rays = sum(f["nearest_rays"] + f["shadow_rays"] for f in frames) / len(frames)
    near_rays = sum(f["nearest_rays"] for f in frames) / len(frames)
    sh_rays = sum(f["shadow_rays"] for f in frames) / len(frames)
    frame_ms = max_over_ranks(sum(f["ms_total"] for f in frames) / len(frames), world)
    if rank != 0:
        return
    hbm, peak_kind = peaks()
    n_launch = max(stt["timed_launches"]["traverse"], 1)
    launches_per_frame = n_launch / args.steps
    avg_launch_ms = stt["stage_ms"]["traverse"] / n_launch
    per_launch_bytes = (near_rays * 48 + sh_rays * 33) / launches_per_frame + len(tris) * 48
    achieved = per_launch_bytes / (avg_launch_ms * 1e-3) / 1e9
    flops_frame = (work["filter_tests"] * FLOP_STAGE1 + work["filter_stage2"] * FLOP_STAGE23
                   + work["exact_tests"] * FLOP_EXACT)
    flops_per_launch = flops_frame / launches_per_frame
    fp32_achieved = flops_per_launch / (avg_launch_ms * 1e-3) / 1e12
    fp32_peak, sms = fp32_peak_tflops(clocks.get("sm_max_mhz") or 2070.0)
    cpu = None
    lights = [{"type": "point", "pos": g["light_pos"], "I": g["light_I"]}]
    if not args.no_cpu and world == 1:
        from oracle import oracle as O
        rc = O.RenderCounter(tris, g["r2c"], g["c2w"], 256, 256, lights, "directlighting", (1, 1), False, 5, 1)
        threads = os.cpu_count() or 1
        r_all, s_all, stride_all = timed_cpu_sample(rc, threads, 5.0, 1)
        r_one, s_one, stride_one = timed_cpu_sample(rc, 1, 3.0, 1)
        cpu = {"value": round(r_all / s_all / 1e6, 3), "unit": "Mrays/s", "cores": threads, "kind": "port",
               "seconds": round(s_all, 2), "cpu_model": cpu_model(),
               "sample": ("the whole frame" if stride_all == 1 else f"every {stride_all}th pixel of the frame")
                         + f" ({r_all} camera + shadow rays), SAH BVH + pbrt's triangle test "
                           "(oracle/render_oracle.c)",
               "single_core": {"value": round(r_one / s_one / 1e6, 3), "cores": 1, "seconds": round(s_one, 2),
                               "sample": f"every {stride_one}th pixel ({r_one} rays)"}}
        del rc
    parity = None
    if not args.no_parity and world == 1:
        diff = img.astype(np.float64) - g["image"].astype(np.float64)
        parity = {"image": "256x256 frame against the reference's own render of it",
                  "rmse_vs_reference": float(np.sqrt(np.mean(diff ** 2))),
                  "pixels_differing": int(np.count_nonzero(np.any(diff != 0, axis=2))),
                  "tolerance": "bit-exact"}
    line = {
        "metric": METRIC, "value": round(job_rate(rays, world, frame_ms), 2), "unit": "Mrays/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(frame_ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (UV sphere + ground quad; the reference's camera and light)",
        "config": {"workload": NAIVE_WORKLOAD, "accelerator": "naive", "rays_per_step": int(rays),
                   "nearest_rays": int(near_rays), "shadow_rays": int(sh_rays), "triangles": int(len(tris)),
                   "parallelism": f"replicas x{world}", "l2": "flushed before every frame (256 MB write)",
                   "autotune": {k: v["best"] for k, v in tuned.items()} if tuned else None},
        "autotune": tuned,
        "e2e": {"value": round(rays / (sum(walls) / len(walls)) / 1e6, 2), "unit": "Mrays/s",
                "ms_per_step": round(sum(walls) / len(walls) * 1e3, 4),
                "h2d_bytes_per_step": 256 + 112, "d2h_bytes_per_step": 256 * 256 * 12,
                "api": "pbg_render (camera, light and parameters in, RGB image out; wall time of the host call)"},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 2), "peak": hbm, "unit": "GB/s",
                     "frac": round(achieved / hbm, 5), "traffic": None,
                     "kernel": "naive_kernel (one nearest-hit and one any-hit launch per frame)",
                     "launches_per_step": round(launches_per_frame, 2),
                     "algorithmic_bytes_per_launch": int(per_launch_bytes),
                     "avg_launch_ms": round(avg_launch_ms, 4), "peak_source": peak_kind + " (of measured copy)",
                     "fp32": {"achieved_tflops": round(fp32_achieved, 3), "peak_tflops": round(fp32_peak, 1),
                              "frac": round(fp32_achieved / fp32_peak, 5),
                              "flops_per_launch": int(flops_per_launch),
                              "peak_source": f"nominal: {sms} SMs x 128 FP32 lanes x 2 x max SM clock",
                              "counted": {k: int(v) for k, v in work.items()},
                              "flop_per_unit": {"tri_stage1": FLOP_STAGE1, "tri_stage2_3": FLOP_STAGE23,
                                                "exact_test": FLOP_EXACT}}},
        "stage_ms_per_step": {k: round(v / args.steps, 4) for k, v in stt["stage_ms"].items()},
        "gpu_launches": int(launches),
        "cpu_baseline": cpu,
        "parity": parity,
        "clocks": clocks,
    }
    print(json.dumps(line), flush=True)


def run_reference_naive(args):
    """The reference's CPU path for the naive workload's frame on all host
    cores: the oracle's restatement of the breadth-first direct-lighting
    render (camera ray and point-light shadow ray per pixel) over its SAH
    BVH and pbrt's triangle test; each step renders the whole frame."""
    from oracle import oracle as O
    from pbrt_gb300 import scenes as S
    g = dict(np.load(os.path.join(ROOT, "tests", "golden", "render_small.npz")))
    tris = S.config_small_naive()["tris"]
    lights = [{"type": "point", "pos": g["light_pos"], "I": g["light_I"]}]
    rc = O.RenderCounter(tris, g["r2c"], g["c2w"], 256, 256, lights, "directlighting", (1, 1), False, 5, 1)
    threads = os.cpu_count() or 1
    times, nrays = [], 0
    for it in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        a, b = rc.count(0, 1, threads, 1)
        dt = time.perf_counter() - t0
        if it >= args.warmup:
            times.append(dt)
            nrays += a + b
    value = nrays / sum(times) / 1e6
    line = {"metric": METRIC, "value": round(value, 3), "unit": "Mrays/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(sum(times) / len(times) * 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (UV sphere + ground quad; the reference's camera and light)", "impl": "reference",
            "config": {"workload": NAIVE_WORKLOAD, "accelerator": "naive", "sample": "the whole frame per step"},
            "cpu_baseline": {"value": round(value, 3), "unit": "Mrays/s", "cores": threads, "kind": "port",
                             "cpu_model": cpu_model(), "sample": "the whole frame per step (oracle/render_oracle.c)"},
            "e2e": {"value": round(value, 3), "unit": "Mrays/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _o4d4(rays):
    o4 = np.ascontiguousarray(np.stack([rays[0], rays[1], rays[2], rays[6]], 1).astype(np.float32))
    d4 = np.ascontiguousarray(np.stack([rays[3], rays[4], rays[5], rays[7]], 1).astype(np.float32))
    return o4, d4


def run_gpu_batch(args, rank, world, dev):
    """64 independent terrain + icosphere scenes (log-normal triangle counts,
    median 20k) with 4k..1M mixed rays each (primary and path rays nearest
    hit, shadow segments any hit), all answered by one persistent launch per
    step (pbg_sceneset_trace, CUDA graph replay, autotuned shape)."""
    import torch
    from pbrt_gb300 import accel as A
    from pbrt_gb300 import scenes as S
    from pbrt_gb300.batch import SceneSet
    torch.cuda.set_device(dev)
    scs = S.many_scenes(seed=5)
    tris_total = sum(len(s["tris"]) for s in scs)
    t0 = time.perf_counter()
    sset = SceneSet([s["tris"] for s in scs], device=dev)
    build_s = time.perf_counter() - t0
    near_off = np.concatenate([[0], np.cumsum([s["near"].shape[1] for s in scs])]).astype(np.int64)
    occ_off = np.concatenate([[0], np.cumsum([s["shadow"].shape[1] for s in scs])]).astype(np.int64)
    on, dn = _o4d4(np.concatenate([s["near"] for s in scs], 1))
    os_, ds = _o4d4(np.concatenate([s["shadow"] for s in scs], 1))
    nn, ns = int(near_off[-1]), int(occ_off[-1])
    rays_per_step = nn + ns

    def pinned(a):
        h = torch.empty(a.shape, dtype=torch.from_numpy(a[:0]).dtype, pin_memory=True)
        h.numpy()[...] = a
        return h

    h_on, h_dn, h_os, h_ds = (pinned(a) for a in (on, dn, os_, ds))
    o4n, d4n, o4s, d4s = (h.to("cuda") for h in (h_on, h_dn, h_os, h_ds))
    prim = torch.empty(nn, dtype=torch.int32, device="cuda")
    tt, b1, b2 = (torch.empty(nn, device="cuda") for _ in range(3))
    occ = torch.empty(ns, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.Stream()
    dev_args = dict(o4n=o4n, d4n=d4n, near_offsets=near_off, prim=prim, t=tt, b1=b1, b2=b2, o4s=o4s,
                    d4s=d4s, occ_offsets=occ_off, occ=occ)
    t0 = time.perf_counter()
    with torch.cuda.stream(stream):
        tuned = sset.autotune(**dev_args, stream=stream)
    tune_s = time.perf_counter() - t0
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            sset.trace(**dev_args, stream=stream)
    stream.synchronize()
    times = []
    rank_barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(dev) as clk:
        for _ in range(args.steps):
            with torch.cuda.stream(stream):
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                sset.trace(**dev_args, stream=stream)
                e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
    torch.cuda.synchronize()
    step_ms = sum(times) / len(times)
    step_ms = max_over_ranks(step_ms, world)
    # per-scene completion: three synchronising calls with the stamps read back
    lat = []
    for _ in range(3):
        st, per = sset.trace(**dev_args, stats=True, stream=stream)
        lat.append(st)
    p50 = statistics.median(x["scene_ms_p50"] for x in lat)
    p99 = statistics.median(x["scene_ms_p99"] for x in lat)
    if rank != 0:
        return
    got_prim, got_t, got_occ = prim.cpu().numpy(), tt.cpu().numpy(), occ.cpu().numpy()

    # the plain per-scene kernels: one ray-bvh scene per call, same device arrays
    accs = [A.MakeAccelerator("ray-bvh", s["tris"], {"device": dev}) for s in scs]
    pprim = torch.empty_like(prim)
    pt, pb1, pb2 = (torch.empty_like(tt) for _ in range(3))
    pocc = torch.empty_like(occ)

    def per_scene_step():
        for k, acc in enumerate(accs):
            a, b = int(near_off[k]), int(near_off[k + 1])
            if b > a:
                acc.intersect_device(o4n[a:b], d4n[a:b], pprim[a:b], pt[a:b], pb1[a:b], pb2[a:b],
                                     stream=stream)
            a, b = int(occ_off[k]), int(occ_off[k + 1])
            if b > a:
                acc.occluded_device(o4s[a:b], d4s[a:b], pocc[a:b], stream=stream)

    with torch.cuda.stream(stream):
        per_scene_step()
        stream.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(3):
            per_scene_step()
        e1.record(stream)
    e1.synchronize()
    per_scene_ms = e0.elapsed_time(e1) / 3
    check = {"rays": rays_per_step,
             "hit_id_mismatches": int((pprim.cpu().numpy() != got_prim).sum()),
             "t_bit_mismatches": int((pt.cpu().numpy().view(np.uint32) != got_t.view(np.uint32)).sum()),
             "occlusion_mismatches": int((pocc.cpu().numpy() != got_occ).sum())}

    # e2e: pinned host rays in, results out, through the public SceneSet call
    h_prim = torch.empty(nn, dtype=torch.int32, pin_memory=True)
    h_t, h_b1, h_b2 = (torch.empty(nn, dtype=torch.float32, pin_memory=True) for _ in range(3))
    h_occ = torch.empty(ns, dtype=torch.uint8, pin_memory=True)

    copy_stream = torch.cuda.Stream(priority=-1)
    host = dict(o4n=h_on, d4n=h_dn, o4s=h_os, d4s=h_ds, prim=h_prim, t=h_t, b1=h_b1, b2=h_b2, occ=h_occ)
    dev = dict(o4n=o4n, d4n=d4n, o4s=o4s, d4s=d4s, prim=prim, t=tt, b1=b1, b2=b2, occ=occ)

    def e2e_step():
        # two halves of the scenes: one half's copies overlap the other's trace
        sset.trace_host(host, dev, near_off, occ_off, stream, copy_stream)

    e2e_step()
    w0 = time.perf_counter()
    for _ in range(max(1, args.steps)):
        e2e_step()
    e2e_ms = (time.perf_counter() - w0) * 1e3 / max(1, args.steps)
    h2d = nn * 32 + ns * 32
    d2h = nn * 16 + ns

    # oracle parity on a ray sample of every scene, and the CPU baseline
    parity, cpu = None, None
    if not args.no_parity or not args.no_cpu:
        from oracle import oracle as O
        threads = os.cpu_count() or 1
        bvhs = [O.BVH(s["tris"]) for s in scs]

        def cpu_pass(stride, check):
            nrays, secs, mism, occ_mism = 0, 0.0, 0, 0
            for k, (s, B) in enumerate(zip(scs, bvhs)):
                sel_n = np.arange(0, s["near"].shape[1], stride)
                sel_s = np.arange(0, s["shadow"].shape[1], stride)
                c0 = time.perf_counter()
                wp = B.nearest(np.ascontiguousarray(s["near"][:, sel_n]), threads=threads)[0]
                wo = B.anyhit(np.ascontiguousarray(s["shadow"][:, sel_s]), threads=threads)
                secs += time.perf_counter() - c0
                nrays += len(sel_n) + len(sel_s)
                if check:
                    mism += int((got_prim[near_off[k] + sel_n] != wp).sum())
                    occ_mism += int((got_occ[occ_off[k] + sel_s] != wo).sum())
            return nrays, secs, mism, occ_mism

        sampled, sec97, mism, occ_mism = cpu_pass(97, True)
        parity = {"sample_rays": sampled, "hit_id_mismatches": mism, "occlusion_mismatches": occ_mism,
                  "oracle": "SAH BVH + pbrt triangle test (oracle/pbrt_oracle.c)"}
        if not args.no_cpu and world == 1:
            # a bounded sample of about 12 s of CPU work
            stride = max(1, int(round(97 * sec97 / 12.0)))
            cpu_rays, cpu_s, reps = 0, 0.0, 0
            while cpu_s < 9.6 and (reps == 0 or stride == 1):
                r_, s_, _, _ = cpu_pass(stride, False)
                cpu_rays += r_
                cpu_s += s_
                reps += 1
            cpu = {"value": round(cpu_rays / cpu_s / 1e6, 3), "unit": "Mrays/s", "cores": threads,
                   "kind": "port", "seconds": round(cpu_s, 2),
                   "sample": f"every {stride}th nearest and shadow ray of each of the 64 scenes, "
                             f"one scene at a time, {reps} pass(es), {cpu_rays} rays"}

    hbm, peak_kind = peaks()
    # algorithmic bytes of one trace launch: rays read once (32 B), results
    # written once (16 B nearest, 1 B any-hit), every scene's triangle
    # records read once (48 B)
    launch_bytes = nn * (32 + 16) + ns * (32 + 1) + tris_total * 48
    achieved = launch_bytes / (step_ms * 1e-3) / 1e9
    value = job_rate(rays_per_step, world, step_ms)
    line = {
        "metric": METRIC, "value": round(value, 2), "unit": "Mrays/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(step_ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded terrain + icosphere scenes, seeded camera, path and shadow rays)",
        "config": {"workload": "batched many-scene: 64 scenes (log-normal triangle counts, median 20k), "
                               "4k-1M mixed rays each, one persistent launch per step",
                   "accelerator": "ray-bvh scene set", "scenes": len(scs), "rays_per_step": rays_per_step,
                   "nearest_rays": nn, "shadow_rays": ns, "triangles": int(tris_total),
                   "build_s": round(build_s, 2), "autotune_s": round(tune_s, 2), "tuned": tuned,
                   "parallelism": f"replicas x{world}",
                   "l2": "inputs > L2 (%.2f GB of rays per step)" % (rays_per_step * 32 / 1e9)},
        "scene_ms_p50": round(p50, 3), "scene_ms_p99": round(p99, 3),
        "per_scene_kernels": {"mrays_s": round(rays_per_step / (per_scene_ms * 1e-3) / 1e6, 2),
                              "ms_per_step": round(per_scene_ms, 3), "launches_per_step": 2 * len(scs)},
        "check_vs_per_scene_kernels": check,
        "e2e": {"value": round(rays_per_step / (e2e_ms * 1e-3) / 1e6, 2), "unit": "Mrays/s",
                "ms_per_step": round(e2e_ms, 3), "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h),
                "api": "SceneSet.trace_host: two pbg_sceneset_trace calls over halves of the scenes, pinned host rays in and results out, copies overlapping the other half's trace"},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 2), "peak": hbm, "unit": "GB/s",
                     "frac": round(achieved / hbm, 5), "traffic": BATCH_STEP_DRAM_BYTES.get(tuned.get("walk")),
                     "kernel": {1: "batch_trace_kernel", 2: "batch_persistent_kernel",
                                3: "wide_walk_kernel (set walk 3, one launch per query kind)",
                                4: "wide_walk_kernel (set walk 4, one launch per query kind)"}.get(
                         tuned.get("walk"), "walk %s" % tuned.get("walk")) + " (tuned walk)",
                     "algorithmic_bytes_per_launch": int(launch_bytes),
                     "avg_launch_ms": round(step_ms, 4), "peak_source": peak_kind},
        "gpu_launches": 2 * args.steps,
        "cpu_baseline": cpu,
        "parity": parity,
        "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)


def run_e2e(args, acc, rays, shadows, hitmask, rays_per_step):
    """Host-buffer frame through the C ABI: pinned arrays in and out."""
    import torch
    n = rays.shape[1]

    def pinned(shape, dtype):
        return torch.empty(shape, dtype=dtype, pin_memory=True).numpy()

    hr = pinned((8, n), torch.float32)
    hr[...] = rays
    hs = []
    for s in shadows:
        a = pinned((8, n), torch.float32)
        a[...] = s
        hs.append(a)
    hv = pinned((n,), torch.uint8)
    hv[...] = hitmask
    out_p = pinned((n,), torch.int32)
    out_t, out_b1, out_b2 = (pinned((n,), torch.float32) for _ in range(3))
    out_o = pinned((n,), torch.uint8)
    import ctypes as C
    from pbrt_gb300 import _lib as L
    lib = L.lib()

    def rays_struct(a, valid):
        return acc._rays_struct(a, valid)

    def frame():
        h = L.Hits(out_p.ctypes.data_as(C.POINTER(C.c_int32)), out_t.ctypes.data_as(C.POINTER(C.c_float)),
                   out_b1.ctypes.data_as(C.POINTER(C.c_float)), out_b2.ctypes.data_as(C.POINTER(C.c_float)))
        rs = rays_struct(hr, None)
        L.check(lib.pbg_intersect(acc.handle, C.byref(rs), n, C.byref(h)), "pbg_intersect")
        for a in hs:
            rs2 = rays_struct(a, hv)
            L.check(lib.pbg_occluded(acc.handle, C.byref(rs2), n, out_o.ctypes.data), "pbg_occluded")

    for _ in range(max(1, args.warmup)):
        frame()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    k = max(1, args.steps)
    for _ in range(k):
        frame()
    torch.cuda.synchronize()
    ms = (time.perf_counter() - t0) * 1e3 / k
    # bytes that cross the host link: a shadow batch's invalid rays are not
    # read (only their validity byte), the results of every ray are written
    nvalid = int(np.count_nonzero(hitmask))
    h2d = n * 32 + len(shadows) * (nvalid * 32 + n)
    d2h = n * 16 + len(shadows) * n
    return {"value": round(rays_per_step / (ms * 1e-3) / 1e6, 2), "unit": "Mrays/s",
            "ms_per_step": round(ms, 3), "h2d_bytes_per_step": int(h2d),
            "d2h_bytes_per_step": int(d2h), "api": "pbg_intersect + 4 x pbg_occluded (host buffers)"}


def cpu_sample(rays, shadows, hitmask, frac):
    n = rays.shape[1]
    sel = np.arange(0, n, max(1, int(round(1 / frac))))
    return sel


def cpu_baseline(tris, rays, shadows, hitmask, target_s: float = 12.0, threads=None):
    """Oracle port of pbrt's CPU BVH path, all host cores: a stride sample of
    the frame sized to about target_s seconds, or whole frames repeated until
    target_s when one frame takes less."""
    from oracle import oracle as O
    threads = threads or os.cpu_count() or 1
    B = O.BVH(tris)
    n = rays.shape[1]

    def run(sel):
        B.nearest(rays[:, sel], threads=threads)
        nr = len(sel)
        for s in shadows:
            B.anyhit(s[:, sel], valid=hitmask[sel], threads=threads)
            nr += int(hitmask[sel].sum())
        return nr

    sel = np.arange(0, n, 512)
    t0 = time.perf_counter()
    run(sel)
    dt = max(time.perf_counter() - t0, 1e-3)
    stride = max(1, int(512 * dt / target_s))
    sel = np.arange(0, n, stride)
    nr, reps = 0, 0
    t0 = time.perf_counter()
    while True:
        nr += run(sel)
        reps += 1
        if time.perf_counter() - t0 >= 0.8 * target_s or stride > 1:
            break
    dt = time.perf_counter() - t0
    what = (f"every {stride}th camera ray of the frame ({len(sel)} rays) and its 4 shadow rays"
            if stride > 1 else f"the whole frame ({n} camera rays + 4 shadow batches) x {reps}")
    return {"value": round(nr / dt / 1e6, 3), "unit": "Mrays/s", "cores": int(threads),
            "kind": "port", "seconds": round(dt, 2),
            "sample": what + "; SAH BVH + pbrt's triangle test (oracle/pbrt_oracle.c)"}


def run_reference_frame(args):
    """The reference's CPU path for the rayhierarchy frame on the host cores:
    the shadow batches come from the CPU path's own hits, generated once
    before the timed steps; each step traces a strided subset of the GPU
    frame's rays (camera rays and their 4 shadow rays)."""
    sc, rays = make_workload()
    tris = sc["tris"]
    from oracle import oracle as O
    B = O.BVH(tris)
    n = rays.shape[1]
    threads = os.cpu_count() or 1
    prim, t, _, _ = B.nearest(rays, threads=threads)
    shadows, hit = shadow_batches(rays, prim, t, sc["area_light_quad"])
    stride = 8
    times, nrays = [], 0
    for it in range(args.warmup + args.steps):
        sel = np.arange(it % stride, n, stride)
        sub = np.ascontiguousarray(rays[:, sel])
        subs = [np.ascontiguousarray(sh[:, sel]) for sh in shadows]
        hv = np.ascontiguousarray(hit[sel])
        t0 = time.perf_counter()
        B.nearest(sub, threads=threads)
        nr = sub.shape[1]
        for sh in subs:
            B.anyhit(sh, valid=hv, threads=threads)
            nr += int(hv.sum())
        dt = time.perf_counter() - t0
        if it >= args.warmup:
            times.append(dt)
            nrays += nr
    value = nrays / sum(times) / 1e6
    line = {"metric": METRIC, "value": round(value, 3), "unit": "Mrays/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(sum(times) / len(times) * 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded terrain + icospheres)", "impl": "reference",
            "config": {"workload": "rayhierarchy direct lighting 1024x1024x4spp, 181,250 triangles, "
                                   "1 nearest + 4 shadow batches per frame",
                       "sample": f"1/{stride} of the camera rays per step (a different eighth each step) "
                                 "and their 4 shadow rays"},
            "cpu_baseline": {"value": round(value, 3), "unit": "Mrays/s", "cores": threads, "kind": "port",
                             "cpu_model": cpu_model(),
                             "sample": f"1/{stride} of the frame's rays per step"},
            "e2e": {"value": round(value, 3), "unit": "Mrays/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_reference_path(args):
    """The reference's CPU path for the path-tracing frame on all host cores:
    the oracle's restatement of the breadth-first path integrator over its
    SAH BVH and pbrt's triangle test, the same frame and samples as the GPU
    arm; each step traces every fourth path of the frame (a different
    quarter each step), timed whole (camera rays, shading, bounce and shadow
    rays).  With smaller samples the last of each step's 409,600-sample
    tasks (the reference's MaxRaysPerCall) left host threads idle."""
    from pbrt_gb300 import scenes  # noqa: F401  (package import for the scene generator)
    sc, r2c, c2w = path_setup()
    rc = path_cpu_counter(sc["tris"], r2c, c2w, 1000)
    threads = os.cpu_count() or 1
    stride = 4
    times, nrays = [], 0
    for it in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        a, b = rc.count(it % stride, stride, threads, 1000)
        dt = time.perf_counter() - t0
        if it >= args.warmup:
            times.append(dt)
            nrays += a + b
    value = nrays / sum(times) / 1e6
    line = {"metric": METRIC, "value": round(value, 3), "unit": "Mrays/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(sum(times) / len(times) * 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded displaced icospheres, counter-hash samples)", "impl": "reference",
            "config": {"workload": PATH_WORKLOAD, "accelerator": "ray-bvh",
                       "sample": f"1/{stride} of the frame's paths per step"},
            "cpu_baseline": {"value": round(value, 3), "unit": "Mrays/s", "cores": threads, "kind": "port",
                             "cpu_model": cpu_model(),
                             "sample": f"every {stride}th sample of the frame per step, seed 1000 "
                                       "(oracle/render_oracle.c)"},
            "e2e": {"value": round(value, 3), "unit": "Mrays/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--accel", default="rayhierarchy", choices=["naive", "rayhierarchy", "ray-bvh"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-parity", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="keep the default launch shapes (no pbg_autotune)")
    ap.add_argument("--workload", default="path", choices=["path", "frame", "batch", "naive"])
    ap.add_argument("--path-res", type=int, default=PATH_RES,
                    help="path workload: image width and height (profiler captures use a smaller frame)")
    ap.add_argument("--max-leaf", type=int, default=0,
                    help="path workload: triangles per BVH leaf at most (0 = the library's default, 4)")
    ap.add_argument("--bvh-build", type=int, default=0,
                    help="path workload: 0 build the BVH on the device, 1 on the host cores")
    ap.add_argument("--ray-sort", type=int, default=0)
    ap.add_argument("--rh-cluster-levels", type=int, default=0,
                    help="rayhierarchy: levels walked by 32-triangle clusters (0 = down to the leaves' parents, <0 = off)")
    ap.add_argument("--walk", type=int, default=0,
                    help="ray-bvh: 0 automatic (or tuned), 1 one thread per ray, 2 persistent warps, "
                         "3 warp packets over the ray hierarchy's leaves, 4 warp packets in the caller's order, "
                         "5 persistent warps over the eight-wide tree, 6 the same with warp-spread triangle tests")
    ap.add_argument("--learn-steps", type=int, default=0, help="SGD steps per frame (0 = 8)")
    ap.add_argument("--learn-lr", type=float, default=0.0, help="learning rate (0 = 0.05)")
    ap.add_argument("--learn-margin", type=float, default=0.0,
                    help="logit lead needed to walk the predicted cluster first (0 = 1.0)")
    ap.add_argument("--learn-queries", type=int, default=2,
                    help="batches the learned ordering serves: 1 nearest-hit, 2 any-hit (default: the ordering "
                         "ceiling of nearest-hit batches is 1.03x, of any-hit batches 1.44x), 3 both")
    ap.add_argument("--learned", type=int, default=2,
                    help="path workload: 0 plain ordering, 1 learned ordering as the value, "
                         "2 plain as the value with the learned comparison attached")
    args = ap.parse_args()
    if args.path_res != PATH_RES:  # a smaller frame of the same scene, for profiler captures
        global PATH_WORKLOAD
        PATH_WORKLOAD = PATH_WORKLOAD.replace(f"{PATH_RES}x{PATH_RES}", f"{args.path_res}x{args.path_res}")
        globals()["PATH_RES"] = args.path_res
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        if rank == 0:
            if args.workload == "path":
                run_reference_path(args)
            elif args.workload == "frame":
                run_reference_frame(args)
            elif args.workload == "naive":
                run_reference_naive(args)
            else:
                print(json.dumps({"impl": "reference", "unavailable": "the 64-scene batch has no reference arm; "
                                  "its CPU baseline is in the GPU line"}), flush=True)
        return
    if world > 1:
        import torch
        torch.cuda.set_device(local)
        torch.distributed.init_process_group("nccl")
    if args.workload == "path":
        run_gpu_path(args, rank, world, local)
    elif args.workload == "batch":
        run_gpu_batch(args, rank, world, local)
    elif args.workload == "naive":
        run_gpu_naive(args, rank, world, local)
    else:
        run_gpu(args, rank, world, local)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
