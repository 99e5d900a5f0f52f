"""Benchmark: Lantern's path-tracing loop on one GB300 (workloads named by scene and size).

Default workload ("icosphere-1.3M"): the displaced icosphere scene --
1,310,720 + 4 triangles, Lambert / mirror / dielectric meshes, 1024x1024,
64 samples per pixel, max depth 10, roulette after bounce 3. One step = one
complete render of that frame (67,108,864 path samples) through
Integrator.RenderFrame (lt_render on device film buffers).

Reported (one JSON line on rank 0):
  value        Msamples/s over the K timed steps (device time, CUDA events on
               the stream lt_render runs on; L2 flushed between steps by
               writing a 256 MiB buffer outside the timed region)
  e2e          the same metric through the C ABI with HOST film buffers: the
               film is copied in, rendered and copied out every step
  mrays        Mrays/s (path segments + light-sample + BSDF-MIS rays)
  roofline     trace kernel: algorithmic bytes (32 B ray + 16 B hit + 32 B per
               child-box test + 40 B per triangle test, node/triangle counts
               from the oracle's BVH2 on a pixel-subsampled render of the same
               frame) / trace-kernel device time, against measured HBM GB/s
  cpu_baseline the reference integrator (oracle/_ref) on the host cores, whole
               frames of the same scene for about 10 s (the oracle's
               restatement for medium-c2, whose HG phase and RGB sigma_s the
               reference's scene JSON cannot state)
--impl reference runs only that CPU path (its own arm).
Other workloads (--workload): nine-spheres (256x256, 16 spp, depth 8),
medium-c2r and medium-c2 (the medium sphere, 512x512, 256 spp, depth 32).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Msamples/s & Mrays/s on 1 GB300 vs host CPU at matched RMSE; adjoint grads/s"
SCENES = os.path.join(ROOT, "_scenes")
# DRAM bytes (read + write) per ray traced by k_trace on the icosphere workload, measured
# with ncu dram__bytes_{read,write}.sum over the 11 k_trace launches of one render of this
# workload (11.34 GB for 171,793,118 traced rays; profiles/k_trace_k_shade_icosphere-1.3M.md)
TRACE_DRAM_BYTES_PER_RAY = 66.0
# L2 throughput of k_trace as a fraction of the L2's peak (ncu
# lts__throughput.avg.pct_of_peak_sustained_elapsed of iterations 0 and 1 of a
# 4-spp render of the same scene; profiles/k_trace_k_shade_icosphere-1.3M.md)
TRACE_L2_FRAC = 0.105


def max_over_ranks(value: float, dist=None, device="cpu") -> float:
    """The largest of every rank's `value` (a time): the whole job is as slow as
    its slowest replica. Without a process group, `value` itself."""
    if dist is None:
        return value
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: float, world: int, seconds: float) -> float:
    """Units all replicas processed per second, in millions (weak scaling: each
    of the `world` ranks renders the same workload)."""
    return units_per_rank * world / seconds / 1e6


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            p = json.load(fh)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def make_scene(name: str):
    import lantern_gb300.scenes as S
    if name == "icosphere-1.3M":
        sc = S.displaced_icosphere_scene(width=1024, height=1024, spp=64, max_depth=10, rr_depth=3,
                                         name="bench_icosphere")
        return sc, {"spp": 64, "max_depth": 10, "rr_depth": 3}
    if name == "nine-spheres":
        sc = S.nine_spheres(width=256, height=256, spp=16, max_depth=8, rr_depth=3, name="bench_nine")
        return sc, {"spp": 16, "max_depth": 8, "rr_depth": 3}
    if name == "medium-c2r":  # the reference-expressible medium scene (isotropic, scalar sigma_s)
        sc = S.medium_sphere_scene(width=512, height=512, spp=256, max_depth=32, rr_depth=3,
                                   reference_expressible=True, name="bench_c2r")
        return sc, {"spp": 256, "max_depth": 32, "rr_depth": 3}
    if name == "medium-c2":  # the full medium scene: RGB sigma_s, Henyey-Greenstein g = 0.3
        sc = S.medium_sphere_scene(width=512, height=512, spp=256, max_depth=32, rr_depth=3, name="bench_c2")
        return sc, {"spp": 256, "max_depth": 32, "rr_depth": 3}
    raise SystemExit(f"unknown workload {name}")


# Workloads whose scene the reference's JSON cannot state (its media have an
# isotropic phase and a scalar sigma_s): their CPU baseline is the oracle's C
# restatement of the same estimator, run on every host core.
PORT_ONLY = {"medium-c2"}


def cpu_renderer(path, workload):
    """The CPU implementation a workload is timed with: the reference integrator
    (oracle/_ref) or, for PORT_ONLY workloads, the oracle. Returns (render,
    width, height, kind, cores) with render(frames, first_frame, max_depth,
    rr_depth) -> (seconds, rays), or None when the reference is not built."""
    from oracle import oracle as O
    cores = int(os.environ.get("LT_REF_THREADS", os.cpu_count()))
    if workload in PORT_ONLY:
        sc = O.OracleScene(path)

        def render(frames, first, max_depth, rr_depth):
            t0 = time.perf_counter()
            r = sc.render(frames, first_frame=first, max_depth=max_depth, rr_depth=rr_depth, threads=cores)
            return time.perf_counter() - t0, sum(r["rays"])
        return render, sc.width, sc.height, "port", cores
    if not os.path.exists(O.REF_SO):
        O.build_reference()
    if not os.path.exists(O.REF_SO):
        return None
    ref = O.ReferenceScene(path)

    def render(frames, first, max_depth, rr_depth):
        r = ref.render(frames, first_frame=first, max_depth=max_depth, rr_depth=rr_depth)
        return r["seconds"], r["rays"]
    return render, ref.width, ref.height, "reference", cores


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 50 ms (a default timed
    region is a quarter of a second)."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int = 0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(2)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = max(mx, float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(n)
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def bytes_per_ray(scene_path: str, width: int, height: int, max_depth: int, rr_depth: int):
    """Oracle BVH2 node/triangle counts per ray on a pixel-subsampled 1-spp render."""
    from oracle import oracle as O
    import numpy as np
    orc = O.OracleScene(scene_path)
    # camera rays + bounce rays: trace the oracle's own path segments on a subsample
    # of pixels by rendering at the full resolution's camera through a strided grid
    rng = np.random.default_rng(0)
    xs = rng.integers(0, width, 4096)
    ys = rng.integers(0, height, 4096)
    rays = []
    import ctypes as C
    L = O.lib()
    for x, y in zip(xs, ys):
        d, o = np.zeros(3, np.float32), np.zeros(3, np.float32)
        L.orc_camera_ray(orc.h, int(x), int(y), C.c_float(0.0), C.c_float(0.0), O.fptr(d), O.fptr(o))
        rays.append(np.concatenate([o, [0.0], d, [np.inf]]).astype(np.float32))
    rays = np.stack(rays)
    hits, cnt = orc.intersect(rays, counters=True)
    # secondary rays: cosine-ish directions from the primary hit points
    hit = hits[:, 3] != 0xFFFFFFFF
    t = hits[hit, 0].view(np.float32)
    d = rays[hit, 4:7] / np.linalg.norm(rays[hit, 4:7], axis=1, keepdims=True)
    p = rays[hit, 0:3] + d * t[:, None]
    dd = rng.normal(size=p.shape)
    dd /= np.linalg.norm(dd, axis=1, keepdims=True)
    dd = np.where((dd * -d).sum(1, keepdims=True) > 0, dd, -dd)
    sec = np.concatenate([p, np.full((p.shape[0], 1), 0.001), dd, np.full((p.shape[0], 1), np.inf)], 1)
    _, cnt2 = orc.intersect(sec.astype(np.float32), counters=True)
    allc = np.concatenate([cnt, cnt2]).astype(np.float64)
    n_node, n_tri = allc[:, 0].mean(), allc[:, 1].mean()
    return 48.0 + 32.0 * n_node + 40.0 * n_tri, float(n_node), float(n_tri)


def run_reference(args, workload):
    """The reference CPU integrator (oracle/_ref) on this host's cores (the
    oracle's restatement for PORT_ONLY workloads)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    sc, rp = make_scene(workload)
    path = __import__("lantern_gb300.scenes", fromlist=["x"]).ensure_written(sc, SCENES)
    try:
        cr = cpu_renderer(path, workload)
    except RuntimeError as e:
        print(json.dumps({"impl": "reference", "unavailable": f"reference build failed: {str(e)[:200]}"}))
        return
    if cr is None:
        print(json.dumps({"impl": "reference", "unavailable": "reference sources not staged (oracle/_ref/src)"}))
        return
    render, width, height, kind, cores = cr
    t1 = 1.0
    for _ in range(args.warmup):
        t1 = render(1, 0, rp["max_depth"], rp["rr_depth"])[0]
    # each step: a bounded sample of about 2 s of CPU work (whole frames)
    frames_per_step = int(max(1, min(64, round(2.0 / max(t1, 1e-6)))))
    secs, rays = 0.0, 0
    for k in range(args.steps):
        s, r = render(frames_per_step, 1000 + k, rp["max_depth"], rp["rr_depth"])
        secs += s
        rays += r
    samples = width * height * frames_per_step * args.steps
    v = samples / secs / 1e6
    line = {"impl": "reference", "metric": METRIC, "value": round(v, 4), "unit": "Msamples/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(1e3 * secs / args.steps, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene)",
            "config": {"workload": workload, "width": width, "height": height, "spp_per_step": frames_per_step,
                       "max_depth": rp["max_depth"], "rr_depth": rp["rr_depth"], "triangles": sc.num_triangles},
            "mrays": round(rays / secs / 1e6, 4),
            "cpu_baseline": {"value": round(v, 4), "unit": "Msamples/s", "cores": cores, "kind": kind,
                             "sample": f"{args.steps} x {frames_per_step} frame(s) of {width}x{height}"},
            "e2e": {"value": round(v, 4), "unit": "Msamples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="icosphere-1.3M")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--microbench", action=argparse.BooleanOptionalAction, default=True,
                    help="also time lt_intersect on 16,777,216 random rays of the same mesh")
    ap.add_argument("--adjoint", action=argparse.BooleanOptionalAction, default=True,
                    help="also time the path-replay adjoint on the differentiable workload")
    ap.add_argument("--adjoint-spp", type=int, default=32,
                    help="samples per pixel of the differentiable workload (small cases for profiling)")
    ap.add_argument("--fd-check", action=argparse.BooleanOptionalAction, default=True,
                    help="with --adjoint: check 64 gradients against central differences (after the timings)")
    ap.add_argument("--spp", type=int, default=None,
                    help="override the workload's samples per pixel (small cases for profiling)")
    ap.add_argument("--paths-in-flight", type=int, default=None,
                    help="wavefront path slots (lt_tuning.paths_in_flight); default: the whole render, "
                         "up to 67,108,864")
    ap.add_argument("--bvh-width", type=int, default=2, choices=[2, 4, 8],
                    help="BVH width of the traversal (lt_tuning.bvh_width)")
    ap.add_argument("--trace-threads", type=int, default=0, choices=[0, 64, 128, 256],
                    help="threads per block of the trace kernel (lt_tuning.trace_threads; 0 = the library's)")
    ap.add_argument("--shade-threads", type=int, default=0, choices=[0, 64, 128, 256, 512],
                    help="threads per block of the shade kernel (lt_tuning.shade_threads; 0 = the library's)")
    ap.add_argument("--stage-timing", action=argparse.BooleanOptionalAction, default=True,
                    help="events around every launch in the timed region (the roofline's kernel time); "
                         "without them lt_render runs as the library does by default")
    ap.add_argument("--batch", action=argparse.BooleanOptionalAction, default=True,
                    help="also time the 64-scene batch: one lt_render_batch vs one lt_render per scene")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3

    if args.impl == "reference":
        run_reference(args, args.workload)
        return

    import numpy as np
    import torch

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    import lantern_gb300.scenes as S
    from lantern_gb300.integrator import FrameBuffer, Integrator, Scene, render_host

    sc, rp = make_scene(args.workload)
    if args.spp:
        rp["spp"] = args.spp
    path = S.ensure_written(sc, SCENES) if rank == 0 or world == 1 else None
    if dist:
        dist.barrier()
        path = os.path.join(SCENES, f"{sc.name}.json")
    scene = Scene(local)
    scene.LoadSceneFromJSON(path)
    paths_in_flight = args.paths_in_flight or min(scene.width * scene.height * rp["spp"], 1 << 26)
    scene.ctx.set_tuning(bvh_width=args.bvh_width, paths_in_flight=paths_in_flight,
                         **({"trace_threads": args.trace_threads} if args.trace_threads else {}),
                         **({"shade_threads": args.shade_threads} if args.shade_threads else {}))
    info = scene.info()
    fb = FrameBuffer(scene.width, scene.height, f"cuda:{local}")
    integ = Integrator(scene, fb, max_depth=rp["max_depth"], rr_depth=rp["rr_depth"])
    spp = rp["spp"]
    stream = torch.cuda.current_stream()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")
    # events around every launch in the timed region: the roofline's kernel
    # time (lt_render is a little faster without them, the library default)
    scene.ctx.set_stage_timing(args.stage_timing)

    for _ in range(args.warmup):
        integ.RenderFrame(spp)
    torch.cuda.synchronize()

    clocks = ClockSampler(local)
    clocks.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    total_ms, trace_ms, shade_ms, init_ms, idle_ms, rays, launches = 0.0, 0.0, 0.0, 0.0, 0.0, 0, 0
    main_rays, conn_traced, trace_launches = 0, 0, 0
    for _ in range(args.steps):
        flush.fill_(1)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        integ.RenderFrame(spp)
        e1.record(stream)
        e1.synchronize()
        total_ms += e0.elapsed_time(e1)
        st = integ.stats()
        trace_ms += st.trace_ms
        shade_ms += st.shade_ms
        init_ms += st.init_ms
        idle_ms += st.idle_ms
        rays += st.main_rays + st.light_rays + st.bsdf_rays
        main_rays += st.main_rays
        conn_traced += st.light_traversals
        launches += st.kernel_launches
        trace_launches += st.iterations
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clk = clocks.stop()
    samples = scene.width * scene.height * spp * args.steps
    t_ms = max_over_ranks(total_ms, dist, f"cuda:{local}")
    value = whole_job_rate(samples, world, t_ms / 1e3)
    mrays = whole_job_rate(rays, world, t_ms / 1e3)

    scene.ctx.set_stage_timing(False)  # the library default, for the end-to-end calls
    e2e = None
    if not args.no_e2e:
        import numpy as np
        npix = scene.width * scene.height
        host = {"rgb": np.zeros((scene.height, scene.width, 3), np.float32),
                "bounces": np.zeros((scene.height, scene.width), np.uint32),
                "counts": np.zeros((scene.height, scene.width), np.uint32)}
        host = {k: torch.from_numpy(v).pin_memory().numpy() for k, v in host.items()}
        render_host(scene.ctx, scene.width, scene.height, spp, 0, rp["max_depth"], rp["rr_depth"], host)
        t0 = time.perf_counter()
        for k in range(args.steps):
            render_host(scene.ctx, scene.width, scene.height, spp, 7 + k, rp["max_depth"], rp["rr_depth"], host)
        e2e_s = max_over_ranks(time.perf_counter() - t0, dist, f"cuda:{local}")
        e2e = {"value": round(whole_job_rate(samples, world, e2e_s), 3), "unit": "Msamples/s",
               "h2d_bytes_per_step": npix * 20, "d2h_bytes_per_step": npix * 20}

    # the wavefront's queue lengths per iteration, from one more render after the
    # timed ones (lt_set_queue_trace): (path rays, camera rays, connection records)
    scene.ctx.set_queue_trace(1024)
    integ.RenderFrame(spp)
    torch.cuda.synchronize()
    queue_lengths = scene.ctx.queue_trace().tolist()
    scene.ctx.set_queue_trace(0)

    micro = None
    if args.microbench and args.workload == "icosphere-1.3M":
        micro = microbench(scene, path, local)
    scene.ctx.trim()  # the headline render's buffers (the whole render in flight) go back
    adjoint = adjoint_bench(local, args.fd_check, args.adjoint_spp) if args.adjoint else None
    batch = batch_bench(local) if args.batch else None

    line = None
    if rank == 0:
        peak, peak_kind = _peaks()
        roof = None
        try:
            bpr, n_node, n_tri = bytes_per_ray(path, scene.width, scene.height, rp["max_depth"], rp["rr_depth"])
            # k_trace traces the path rays and the connection rays that needed a
            # query; both are charged the closest-hit bytes of one ray
            if trace_ms <= 0.0:
                raise ValueError("no stage times (--no-stage-timing): no kernel time for the roofline")
            achieved = (main_rays + conn_traced) * bpr / (trace_ms / 1e3) / 1e9
            traced_per_launch = (main_rays + conn_traced) / max(trace_launches, 1)
            roof = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                    "frac": round(achieved / peak, 4), "kernel": "k_trace",
                    # DRAM bytes per launch: ncu-measured bytes per traced ray x rays per launch
                    "traffic": (round(TRACE_DRAM_BYTES_PER_RAY * traced_per_launch)
                                if args.workload == "icosphere-1.3M" else None),
                    "algorithmic_bytes_per_launch": round(bpr * traced_per_launch),
                    "l2_frac": TRACE_L2_FRAC if args.workload == "icosphere-1.3M" else None,
                    "bytes_per_ray": round(bpr, 1), "node_tests_per_ray": round(n_node, 2),
                    "tri_tests_per_ray": round(n_tri, 2), "peak_kind": peak_kind,
                    "rays_traced_per_step": (main_rays + conn_traced) // args.steps,
                    # kernel time of each stage (events around every launch) and the
                    # time between the render's kernels, as shares of the step
                    "trace_share": round(trace_ms / max(total_ms, 1e-9), 3),
                    "shade_share": round(shade_ms / max(total_ms, 1e-9), 3),
                    "init_share": round(init_ms / max(total_ms, 1e-9), 3),
                    "idle_share": round(idle_ms / max(total_ms, 1e-9), 3)}
            # the whole render against the same bandwidth: bytes per sample = rays
            # per sample (path, light-sample and BSDF-sample rays, the reference's
            # count) x bytes per ray + 20 B of film update; above 1 where the
            # caches serve what the model charges to HBM
            b_sample = rays / samples * bpr + 20.0
            roof["bytes_per_sample"] = round(b_sample, 1)
            roof["sample_roofline"] = round(peak * 1e3 / b_sample, 1)  # Msamples/s
            roof["sample_frac"] = round(value / world / (peak * 1e3 / b_sample), 4)
        except Exception as e:  # the oracle is a checker; report its absence
            roof = {"error": str(e)[:200]}
        cpu = None
        if not args.no_cpu_baseline:
            cpu = cpu_baseline(path, rp, args.workload)
        line = {"metric": METRIC, "value": round(value, 3), "unit": "Msamples/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(t_ms / args.steps, 3),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (seeded procedural scene, written as Lantern JSON + LMF)",
                "config": {"workload": args.workload, "width": scene.width, "height": scene.height, "spp": spp,
                           "max_depth": rp["max_depth"], "rr_depth": rp["rr_depth"],
                           "triangles": info.num_triangles, "bvh_nodes": info.num_bvh_nodes,
                           "bvh_width": args.bvh_width, "paths_in_flight": paths_in_flight,
                           "trace_threads": scene.ctx.tuning().trace_threads,
                           "shade_threads": scene.ctx.tuning().shade_threads,
                           "l2": "flushed between steps (256 MiB write)", "parallelism": "replicas" if world > 1
                           else "single GPU"},
                "mrays": round(mrays, 2), "gpu_launches": launches,
                "clocks": clk, "e2e": e2e, "roofline": roof, "cpu_baseline": cpu,
                "queue_lengths": {"columns": ["path_rays", "camera_rays", "connection_records"],
                                  "per_iteration": queue_lengths},
                "intersect_microbench": micro, "adjoint": adjoint, "batch": batch}
        print(json.dumps(line))
    if dist:
        dist.barrier()
        dist.destroy_process_group()


def adjoint_bench(local, fd_check=True, spp=32):
    """Differentiable workload: nine spheres + HG medium sphere, 512x512, `spp` (32),
    depth 8. Times the plain forward render (wavefront), the differentiable
    forward that keeps per-sample radiance, and the path-replay adjoint of the
    L2 loss to the true-parameter image; grads/s = full gradients per second."""
    import torch
    import lantern_gb300.scenes as S
    from lantern_gb300.diff import DiffScene, render_image
    from lantern_gb300.integrator import FrameBuffer, Integrator, Scene
    path = S.ensure_written(S.differentiable_scene(), SCENES)
    ds = DiffScene(path, local)
    a0, e0, sa0, ss0 = ds.defaults()
    true, init = S.differentiable_targets(ds.num_triangles)
    dev = ds.device
    sc = Scene(local)
    sc.LoadSceneFromJSON(path)
    fb = FrameBuffer(sc.width, sc.height, f"cuda:{local}")
    it = Integrator(sc, fb, max_depth=8, rr_depth=3)
    th = [torch.from_numpy(init["albedo"]).to(dev), e0, torch.from_numpy(init["sigma_a"]).to(dev),
          torch.from_numpy(init["sigma_s"]).to(dev)]
    with torch.no_grad():
        target = render_image(ds, torch.from_numpy(true["albedo"]).to(dev), e0,
                              torch.from_numpy(true["sigma_a"]).to(dev), torch.from_numpy(true["sigma_s"]).to(dev),
                              spp, 0, 8, 3)

    def timed(f, n=3):
        f()
        torch.cuda.synchronize()
        st = torch.cuda.current_stream()
        e0_, e1_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0_.record(st)
        for _ in range(n):
            f()
        e1_.record(st)
        e1_.synchronize()
        return e0_.elapsed_time(e1_) / n

    fwd = timed(lambda: it.RenderFrame(spp))
    out = {}
    dfw = timed(lambda: out.update(r=ds.render(*th, spp, 0, 8, 3, keep_samples=True)))
    rgb, _, _, samples = out["r"]
    dI = (2.0 * (rgb / spp - target) / spp).contiguous()
    adj = timed(lambda: ds.adjoint(*th, dI, spp, 0, 8, 3, samples=samples))
    nparams = 6 * ds.num_triangles + 6 * ds.num_media
    # acceptance check of the gradients (outside the timings): 64 parameters
    # (seed 4) against central differences, h = 1e-3
    fdc = None
    if fd_check:
        from lantern_gb300.diff import finite_difference_check
        fdc = finite_difference_check(ds, th, target, spp, max_depth=8, count=64, seed=4, h=1e-3)
    step = dfw + adj
    return {"config": f"differentiable scene 512x512, {spp} spp, depth 8", "parameters": nparams,
            "forward_ms": round(fwd, 3), "diff_forward_ms": round(dfw, 3), "adjoint_ms": round(adj, 3),
            "adjoint_over_forward": round(adj / fwd, 3), "grads_per_s": round(1e3 / adj, 2),
            "step_ms": round(step, 3), "step_over_forward": round(step / fwd, 3),
            "grads_per_s_step": round(1e3 / step, 2),
            "ratios": "adjoint_over_forward: adjoint pass / plain forward render; step_over_forward: "
                      "(differentiable forward + adjoint) / plain forward render",
            "fd_check": None if fdc is None else {
                "parameters": fdc["parameters"], "checked": fdc["checked"],
                "max_rel_err": round(fdc["max_rel_err"], 5), "h": 1e-3, "seed": 4,
                "within_2pct": not fdc["failures"]}}


def batch_bench(local, count=64, reps=3):
    """Batched workload: 64 seeded scenes (seed 5; 128^2..1024^2, 1k..500k
    triangles, 4/16/64 spp, 30% with the fog medium; depth 10). Times every
    scene rendered by its own Integrator.RenderFrame (lt_render, one after the
    other: the sequential baseline, with the default and with the tuned launch
    configuration) against one RenderBatch (lt_render_batch: one captured
    graph launch for the scenes below the wavefront size, the ones that fill
    it alone after it) after lt_autotune_batch. Device time on the stream, best of
    `reps`; films accumulate across repetitions (additive, like RenderFrame)."""
    import torch
    import lantern_gb300.scenes as S
    from lantern_gb300.integrator import FrameBuffer, Integrator, RenderBatch, Scene
    gen = S.batch_scenes(count=count)
    sdir = os.path.join(SCENES, "batch")
    scenes = []
    for sc in gen:
        s = Scene(local)
        s.LoadSceneFromJSON(S.ensure_written(sc, sdir))
        scenes.append(s)
    fbs = [FrameBuffer(s.width, s.height, f"cuda:{local}") for s in scenes]
    spps = [sc.render["spp"] for sc in gen]
    depth = [sc.render["max_depth"] for sc in gen]
    samples = sum(s.width * s.height * n for s, n in zip(scenes, spps))
    stream = torch.cuda.current_stream()

    def integrators():
        return [Integrator(s, fb, max_depth=d, rr_depth=3) for s, fb, d in zip(scenes, fbs, depth)]

    def sequential():
        for it, n in zip(integrators(), spps):
            it.RenderFrame(n)

    def batched():
        RenderBatch(integrators(), spps)

    def timed(f):
        f()
        torch.cuda.synchronize()
        best = 1e30
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            f()
            e1.record(stream)
            e1.synchronize()
            best = min(best, e0.elapsed_time(e1))
        return best

    seq_default = timed(sequential)
    # the ceiling of batching: in one more sequential pass, the kernel time of
    # every render (events around each launch), the time each render's stream
    # waited for the host between its batches of iterations, and the rest of the
    # wall time (between renders)
    busy = idle = inside = 0.0
    for s in scenes:
        s.ctx.set_stage_timing(True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for it, n in zip(integrators(), spps):
        it.RenderFrame(n)
        st_ = it.stats()
        busy += st_.init_ms + st_.trace_ms + st_.shade_ms
        idle += st_.idle_ms
        inside += st_.gpu_ms
    e1.record(stream)
    e1.synchronize()
    seq_wall = e0.elapsed_time(e1)
    for s in scenes:
        s.ctx.set_stage_timing(False)
    owner = scenes[0].ctx
    owner.set_stream(stream.cuda_stream)
    t0 = time.perf_counter()
    tune = owner.autotune_batch([s.ctx for s in scenes], [(n, 0, d, 3) for n, d in zip(spps, depth)], spp_cap=1)
    tune_s = time.perf_counter() - t0
    bat = timed(batched)
    st = owner.stats()
    tuned = tune.as_dict()
    for s in scenes[1:]:
        s.ctx.set_tuning(**{k: v for k, v in tuned.items() if k != "ms"})
    seq_tuned = timed(sequential)
    seq = min(seq_default, seq_tuned)
    # where batching pays: the scenes that do not fill the wavefront by
    # themselves (lt_render_batch renders the others alone), batched vs one by one
    limit = tuned["paths_in_flight"] or (1 << 24)
    small = [k for k in range(len(scenes)) if scenes[k].width * scenes[k].height * spps[k] < limit]

    def small_sequential():
        its = integrators()
        for k in small:
            its[k].RenderFrame(spps[k])

    def small_batched():
        its = integrators()
        RenderBatch([its[k] for k in small], [spps[k] for k in small])

    small_seq = timed(small_sequential) if small else 0.0
    small_bat = timed(small_batched) if small else 0.0
    # every context keeps its wavefront until trimmed: give the plain renders'
    # buffers back before the differentiable part allocates its own
    for s in scenes:
        s.ctx.trim()

    # the scenes marked for the adjoint: differentiable forward (keeping every
    # sample's radiance) and the adjoint of loss = sum(image^2), per scene vs batched
    from lantern_gb300.diff import DiffScene, adjoint_batch, render_batch
    marked = [k for k, sc in enumerate(gen) if sc.render.get("adjoint")]
    dss = [DiffScene(ctx=scenes[k].ctx) for k in marked]
    prm = [ds.defaults() for ds in dss]
    asp = [spps[k] for k in marked]
    adep = [depth[k] for k in marked]

    def adj_sequential():
        for ds, p, n, d in zip(dss, prm, asp, adep):
            rgb, _, _, smp = ds.render(*p, n, 0, d, 3, keep_samples=True)
            ds.adjoint(*p, (2.0 * rgb / n) / n, n, 0, d, 3, samples=smp)
            del smp

    def adj_batched():
        outs = render_batch(dss, prm, asp, 0, adep, 3, keep_samples=True)
        adjoint_batch(dss, prm, [(2.0 * o[0] / n) / n for o, n in zip(outs, asp)], asp, 0, adep, 3,
                      samples=[o[3] for o in outs])

    adj_samples = sum(ds.width * ds.height * n for ds, n in zip(dss, asp))
    adj_seq = timed(adj_sequential)
    adj_bat = timed(adj_batched)

    # the two passes apart (one more run of each, events between the passes):
    # differentiable forwards, then adjoints from their samples
    def split(run):
        evs = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        run(evs)
        evs[2].synchronize()
        return evs[0].elapsed_time(evs[1]), evs[1].elapsed_time(evs[2])

    def seq_split(evs):
        evs[0].record(stream)
        fw, bw = 0.0, 0.0
        for ds, p, n, d in zip(dss, prm, asp, adep):
            a, b, c = (torch.cuda.Event(enable_timing=True) for _ in range(3))
            a.record(stream)
            rgb, _, _, smp = ds.render(*p, n, 0, d, 3, keep_samples=True)
            b.record(stream)
            ds.adjoint(*p, (2.0 * rgb / n) / n, n, 0, d, 3, samples=smp)
            c.record(stream)
            c.synchronize()
            fw += a.elapsed_time(b)
            bw += b.elapsed_time(c)
            del smp
        evs[1].record(stream)
        evs[2].record(stream)
        seq_split.ms = (fw, bw)

    def bat_split(evs):
        evs[0].record(stream)
        outs = render_batch(dss, prm, asp, 0, adep, 3, keep_samples=True)
        evs[1].record(stream)
        adjoint_batch(dss, prm, [(2.0 * o[0] / n) / n for o, n in zip(outs, asp)], asp, 0, adep, 3,
                      samples=[o[3] for o in outs])
        evs[2].record(stream)

    split(seq_split)
    fwd_seq, bwd_seq = seq_split.ms
    fwd_bat, bwd_bat = split(bat_split)
    return {"workload": f"{count} scenes (seed 5): 128^2-1024^2, 1k-500k triangles, 4/16/64 spp, 30% medium; "
                        f"{len(marked)} also run the adjoint",
            "samples": samples, "triangles": sum(s.info().num_triangles for s in scenes),
            "sequential_ms": round(seq_default, 2), "sequential_tuned_ms": round(seq_tuned, 2),
            "batched_ms": round(bat, 2), "batched_msamples_per_s": round(samples / bat / 1e3, 2),
            "speedup_vs_sequential": round(seq / bat, 3), "tuning": tuned, "tune_s": round(tune_s, 2),
            "sequential_ceiling": {"wall_ms": round(seq_wall, 2), "kernel_ms": round(busy, 2),
                                   "idle_in_renders_ms": round(idle, 2),
                                   "between_renders_ms": round(max(seq_wall - inside, 0.0), 2),
                                   "max_speedup": round(seq_default / max(busy, 1e-9), 3),
                                   "note": "kernel_ms, idle and wall_ms from one more sequential pass with "
                                           "events around every launch; max_speedup = sequential_ms (without "
                                           "them) / kernel time: what batching reaches if it removes every gap "
                                           "and runs the same kernels as fast"},
            "batched_iterations": st.iterations, "batched_kernel_launches": st.kernel_launches,
            "scenes_below_wavefront": {"count": len(small),
                                       "samples": sum(scenes[k].width * scenes[k].height * spps[k] for k in small),
                                       "sequential_ms": round(small_seq, 2), "batched_ms": round(small_bat, 2),
                                       "speedup": round(small_seq / small_bat, 3) if small else None,
                                       "note": "the scenes with fewer samples than the wavefront holds, rendered "
                                               "one by one vs in one lt_render_batch"},
            "adjoint_scenes": len(marked), "adjoint_samples": adj_samples,
            "adjoint_sequential_ms": round(adj_seq, 2), "adjoint_batched_ms": round(adj_bat, 2),
            "adjoint_speedup": round(adj_seq / adj_bat, 3),
            "adjoint_passes_ms": {"forward_sequential": round(fwd_seq, 2), "forward_batched": round(fwd_bat, 2),
                                  "adjoint_sequential": round(bwd_seq, 2), "adjoint_batched": round(bwd_bat, 2)},
            "total_sequential_ms": round(seq + adj_seq, 2), "total_batched_ms": round(bat + adj_bat, 2),
            "total_speedup": round((seq + adj_seq) / (bat + adj_bat), 3)}


def microbench(scene, path, local, n=1 << 24):
    """lt_intersect on n rays: origins uniform in the mesh bounds, directions
    uniform on the sphere (seed 2), tnear 0, tfar inf. Device Mrays/s over 5
    launches (inputs 512 MiB, larger than L2), plus the oracle's BVH2 on a
    bounded CPU sample with all host cores."""
    import numpy as np
    import torch
    import lantern_gb300.scenes as S
    from lantern_gb300.integrator import intersect
    with open(path) as fh:
        j = json.load(fh)
    lo, hi = np.full(3, np.inf), np.full(3, -np.inf)
    from oracle import oracle as O
    for p in j["primitives"]:
        if p["name"].startswith("ico_"):
            pos = O.read_lmf(os.path.join(os.path.dirname(path), p["file_path"]))["positions"]
            lo, hi = np.minimum(lo, pos.min(0)), np.maximum(hi, pos.max(0))
    rays = S.random_rays(n, lo, hi, seed=2)
    dr = torch.from_numpy(rays).to(f"cuda:{local}")
    intersect(scene.ctx, dr)  # warm-up
    torch.cuda.synchronize()
    st = torch.cuda.current_stream()
    ms = 0.0
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        hits = intersect(scene.ctx, dr)
        e1.record(st)
        e1.synchronize()
        ms += e0.elapsed_time(e1)
    hit_frac = float((hits[:, 3].view(torch.int32) != -1).float().mean())
    out = {"rays": n, "mrays": round(5 * n / (ms / 1e3) / 1e6, 1), "hit_fraction": round(hit_frac, 4)}
    try:
        orc = O.OracleScene(path)
        sample = rays[: 1 << 18]
        t0 = time.perf_counter()
        orc.intersect(sample, threads=os.cpu_count())
        dt = time.perf_counter() - t0
        out["cpu_oracle_mrays"] = round(sample.shape[0] / dt / 1e6, 2)
        out["cpu_oracle_sample"] = f"{sample.shape[0]} rays, {os.cpu_count()} threads, oracle BVH2"
    except Exception as e:
        out["cpu_oracle_error"] = str(e)[:200]
    return out


def cpu_baseline(path, rp, workload):
    """The workload's CPU implementation (cpu_renderer) on this host, whole
    frames of the same scene for about 10 s."""
    try:
        cr = cpu_renderer(path, workload)
        if cr is None:
            return None
        render, width, height, kind, cores = cr
        t1 = render(1, 98, rp["max_depth"], rp["rr_depth"])[0]
        frames = int(max(1, min(256, round(10.0 / max(t1, 1e-6)))))  # about 10 s of CPU work
        secs, rays = render(frames, 99, rp["max_depth"], rp["rr_depth"])
        n = width * height * frames
        return {"value": round(n / secs / 1e6, 4), "unit": "Msamples/s", "cores": cores, "kind": kind,
                "sample": f"{frames} frame(s) (1 spp each) of {width}x{height}, {secs:.1f} s",
                "mrays": round(rays / secs / 1e6, 3)}
    except Exception as e:
        return {"error": str(e)[:200]}


if __name__ == "__main__":
    main()
