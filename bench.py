"""Benchmark: closest-hit Mrays/s on the BVH stress workload.

Workload (one "step" = one closest-hit launch, 1 spp): a seeded icosphere
subdivided to 1,310,720 triangles, displaced by 3-octave value noise,
instanced 64 times with seeded rigid transforms inside a 100^3 cube; rays =
1920x1080 jittered pinhole primaries + one cosine-weighted diffuse bounce per
primary hit, cast together through the C ABI (``mrg_cast_closest``).  Inputs
(rays 32 B + hits 16 B + meta hits 8 B per ray, ~230 MB) exceed the 129 MB L2,
so no flush is needed between steps; each step restores the rays' tMax first.

``value``: rays per step / device time per step (CUDA events on the launching
stream, K timed steps after W warm-ups, max over ranks).  ``e2e``: the same
metric through the host-buffer entry point ``mrg_cast_closest_host`` with
pinned host buffers (H2D + cast + D2H + sync inside the timed region).
``--impl reference``: the CPU restatement of MRay's host-backend LBVH cast
(oracle/) on all host cores over a bounded sample of the same rays.
"""
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

METRIC = "Mrays/s closest-hit"
UNIT = "Mrays/s"
WIDTH, HEIGHT = 1920, 1080
WORKLOAD = "bvh-stress: 1,310,720-tri displaced icosphere x 64 rigid instances, 1920x1080 primary + 1 diffuse bounce"


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def l2_copy_peak(dev, reps=50):
    """Measured L2 bandwidth: a 24 MiB -> 24 MiB device copy that stays in
    the 129 MB L2 (read + write bytes over the CUDA-event time of the best
    of `reps` copies).  The denominator of the L2 roofline fraction."""
    import torch
    n = 24 << 20
    a = torch.empty(n, dtype=torch.uint8, device=dev)
    b = torch.empty(n, dtype=torch.uint8, device=dev)
    a.fill_(1)
    for _ in range(5):
        b.copy_(a)
    best = None
    for _ in range(reps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        b.copy_(a)
        e1.record()
        torch.cuda.synchronize(dev)
        ms = e0.elapsed_time(e1)
        best = ms if best is None else min(best, ms)
    return 2.0 * n / (best * 1e-3) / 1e9


def profile_figures():
    """Per-launch counters of k_trace<closest> on this workload from the
    committed ncu summary: lines 'name: value' (DRAM traffic, L2 bytes, warp
    instructions)."""
    out = {}
    tp = os.path.join(ROOT, "profiles", "k_trace_closest_bvh_stress.md")
    if os.path.exists(tp):
        for ln in open(tp):
            for key in ("traffic_bytes_per_launch", "l2_bytes_per_launch", "warp_instructions_per_launch"):
                if ln.startswith(key + ":"):
                    try:
                        out[key] = int(ln.split(":", 1)[1].strip())
                    except ValueError:
                        pass
    return out


def pt_profile_figures():
    """DRAM and L2 bytes of one render call of the C0 / C2 path-tracing
    workloads (every kernel of the call summed) from the committed ncu
    summary: lines '<w>_dram_bytes_per_call: value' and
    '<w>_l2_bytes_per_call: value'."""
    out = {}
    tp = os.path.join(ROOT, "profiles", "pt_workloads_roofline.md")
    if os.path.exists(tp):
        for ln in open(tp):
            for w in ("c0", "c2"):
                for key in ("dram_bytes_per_call", "l2_bytes_per_call"):
                    if ln.startswith("%s_%s:" % (w, key)):
                        try:
                            out.setdefault(w, {})[key] = int(ln.split(":", 1)[1].strip())
                        except ValueError:
                            pass
    return out


def pt_roofline(extra, hbm_peak, l2_peak):
    """Roofline lines of the C0 and C2 render calls: the profiled DRAM and L2
    bytes of one call over the call's live time (CUDA events, streams
    overlapped), against the measured HBM and L2 copy peaks."""
    prof = pt_profile_figures()
    out = {}
    for w, ms_key, paths in (("c0", "box_pt_ms_per_16spp", 256 * 256 * 16),
                             ("c2", "c2_ms_per_4spp_1080p", 1920 * 1080 * 4)):
        ms = extra.get(ms_key)
        f = prof.get(w)
        if not ms or not f:
            continue
        sec = ms * 1e-3
        line = {"ms_per_call": ms, "paths_per_call": paths, "mpaths_per_s": round(paths / sec / 1e6, 1)}
        if "dram_bytes_per_call" in f:
            gbs = f["dram_bytes_per_call"] / sec / 1e9
            line.update(dram_bytes_per_path=round(f["dram_bytes_per_call"] / paths, 1), dram_gbs=round(gbs, 1),
                        dram_frac_of_measured_hbm=round(gbs / hbm_peak, 3))
        if "l2_bytes_per_call" in f:
            gbs = f["l2_bytes_per_call"] / sec / 1e9
            line.update(l2_bytes_per_path=round(f["l2_bytes_per_call"] / paths, 1), l2_gbs=round(gbs, 1),
                        l2_frac_of_measured_l2=round(gbs / l2_peak, 3))
        out[w] = line
    return out


def make_workload(seed=0):
    from mray_gb300 import scenes
    pos, idx, m = scenes.bvh_stress_scene(seed=seed)
    prim = scenes.primary_rays(WIDTH, HEIGHT, seed)
    return pos, idx, m, prim


def gpu_arm(args):
    import torch
    import torch.distributed as dist
    from mray_gb300 import Accelerator, scenes
    from mray_gb300 import build as B
    B.build()

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev)

    pos, idx, m, prim = make_workload(seed=rank)
    acc = Accelerator(local)
    mesh = acc.upload_mesh(pos, idx, prim_key_base=0x10000000)
    for i in range(m.shape[0]):
        acc.add_instance(mesh, m[i], light_or_mat_key=i, trans_key=(1 << 24) | i, accel_key=(2 << 20) | i)
    t0 = time.perf_counter()
    acc.construct()
    build_s = time.perf_counter() - t0
    st = acc.stats()

    # primary hits -> bounce rays (one diffuse bounce per primary hit)
    pr = torch.from_numpy(prim).to(dev)
    ph = torch.zeros((prim.shape[0], 4), dtype=torch.int32, device=dev)
    pm = torch.zeros((prim.shape[0], 2), dtype=torch.float32, device=dev)
    acc.cast_rays(pr, ph, pm, stream=stream)
    acc.sync_status(stream)
    prh = pr.cpu().numpy()
    phh = ph.cpu().numpy().view(np.uint32)
    hit = prh[:, 7] < 3e38
    inst = np.where(hit, phh[:, 2] & 0xFFFFFF, 0xFFFFFFFF).astype(np.uint32)
    primk = (phh[:, 0] - 0x10000000).astype(np.uint32)
    bounce, _ = scenes.bounce_rays(prim, inst, primk, prh[:, 7], pos, idx, m, seed=rank + 1)
    rays_np = np.vstack([prim, bounce]).astype(np.float32)
    n = rays_np.shape[0]

    pristine = torch.from_numpy(rays_np).to(dev)
    rays = pristine.clone()
    hits = torch.zeros((n, 4), dtype=torch.int32, device=dev)
    meta = torch.zeros((n, 2), dtype=torch.float32, device=dev)

    # traversal counts over the whole ray set (algorithmic bytes per ray)
    counts = acc.traversal_counts(pristine, stream=stream)

    def step():
        rays.copy_(pristine)
        acc.cast_rays(rays, hits, meta, stream=stream)

    for _ in range(args.warmup):
        step()
    acc.sync_status(stream)

    # kernel-only timing (events around the cast launch alone)
    kev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    sampler = ClockSampler(local)
    sampler.start()
    if ws > 1:
        dist.barrier()
    torch.cuda.synchronize(dev)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for k in range(args.steps):
        rays.copy_(pristine)
        kev[k][0].record(stream)
        acc.cast_rays(rays, hits, meta, stream=stream)
        kev[k][1].record(stream)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    if ws > 1:
        dist.barrier()
    clocks = sampler.stop()
    acc.sync_status(stream)
    total_ms = e0.elapsed_time(e1)
    kernel_ms = sum(a.elapsed_time(b) for a, b in kev) / args.steps
    if ws > 1:
        t = torch.tensor([total_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    ms_per_step = total_ms / args.steps
    value = (n * ws) / (ms_per_step * 1e-3) / 1e6

    # e2e: host buffers through mrg_cast_closest_host (pinned)
    h_rays = torch.from_numpy(rays_np).pin_memory()
    h_hits = torch.zeros((n, 4), dtype=torch.int32).pin_memory()
    h_meta = torch.zeros((n, 2), dtype=torch.float32).pin_memory()
    hr, hh, hm = h_rays.numpy(), h_hits.numpy().view(np.uint32), h_meta.numpy()
    acc.cast_rays_host(hr, hh, hm)           # grow staging buffers (untimed)
    e2e_times = []
    for _ in range(max(3, min(args.steps, 10))):
        hr[:] = rays_np
        t0 = time.perf_counter()
        acc.cast_rays_host(hr, hh, hm)
        e2e_times.append(time.perf_counter() - t0)
    e2e_s = statistics.median(e2e_times)
    e2e_val = n / e2e_s / 1e6
    if ws > 1:
        t = torch.tensor([e2e_s], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_val = n * ws / float(t.item()) / 1e6

    # any-hit (shadow rays from the bounce origins to a point light)
    shadow = torch.from_numpy(scenes.shadow_rays(bounce, (0.0, 80.0, -60.0))).to(dev)
    vis = torch.zeros(((shadow.shape[0] + 31) // 32,), dtype=torch.int32, device=dev)
    for _ in range(2):
        acc.cast_visibility_rays(vis, shadow, stream=stream)
    a0 = torch.cuda.Event(enable_timing=True)
    a1 = torch.cuda.Event(enable_timing=True)
    a0.record(stream)
    for _ in range(args.steps):
        acc.cast_visibility_rays(vis, shadow, stream=stream)
    a1.record(stream)
    torch.cuda.synchronize(dev)
    any_ms = a0.elapsed_time(a1) / args.steps
    any_val = shadow.shape[0] / (any_ms * 1e-3) / 1e6

    # the opt-in watertight triangle test on the same scene and rays:
    # closest-hit rate and how many rays it answers differently from MT
    wt = Accelerator(local, watertight=True)
    wmesh = wt.upload_mesh(pos, idx, prim_key_base=0x10000000)
    for i in range(m.shape[0]):
        wt.add_instance(wmesh, m[i], light_or_mat_key=i, trans_key=(1 << 24) | i, accel_key=(2 << 20) | i)
    wt.construct()
    wrays = pristine.clone()
    whits = torch.zeros_like(hits)
    wmeta = torch.zeros_like(meta)
    for _ in range(3):
        wrays.copy_(pristine)
        wt.cast_rays(wrays, whits, wmeta, stream=stream)
    wsteps = max(3, min(args.steps, 50))
    w0 = torch.cuda.Event(enable_timing=True)
    w1 = torch.cuda.Event(enable_timing=True)
    w0.record(stream)
    for _ in range(wsteps):
        wrays.copy_(pristine)
        wt.cast_rays(wrays, whits, wmeta, stream=stream)
    w1.record(stream)
    torch.cuda.synchronize(dev)
    wt.sync_status(stream)
    wt_val = n / (w0.elapsed_time(w1) / wsteps * 1e-3) / 1e6
    mt_t = rays[:, 7].cpu().numpy().view(np.uint32)
    wt_t = wrays[:, 7].cpu().numpy().view(np.uint32)
    mt_k = hits.cpu().numpy().view(np.uint32)[:, [0, 2]]
    wt_k = whits.cpu().numpy().view(np.uint32)[:, [0, 2]]
    mt_hit = rays[:, 7].cpu().numpy() < 3e38
    wt_hit = wrays[:, 7].cpu().numpy() < 3e38
    diff_prim = int(((mt_k != wt_k).any(axis=1) & mt_hit & wt_hit).sum())
    diff_status = int((mt_hit != wt_hit).sum())
    diff_t = int(((mt_t != wt_t) & mt_hit & wt_hit).sum())
    wt.close()

    peak, peak_kind = load_peaks()
    per_ray = (32 + 28 + 80.0 * counts["node_visits"] / counts["rays"] +
               48.0 * counts["tri_tests"] / counts["rays"] + 96.0 * counts["instance_entries"] / counts["rays"])
    achieved = per_ray * n / (kernel_ms * 1e-3) / 1e9
    # DRAM bytes, L2 bytes and warp instructions of one k_trace<closest>
    # launch from the committed ncu summary; fractions of the live kernel time
    prof = profile_figures()
    traffic = prof.get("traffic_bytes_per_launch")
    l2_peak = l2_copy_peak(dev)
    ksec = kernel_ms * 1e-3
    sm_mhz = clocks.get("sm_mhz") or 2070.0
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    fractions = {}
    if traffic:
        fractions["dram"] = round(traffic / ksec / 1e9 / peak, 3)
    if prof.get("l2_bytes_per_launch"):
        fractions["l2"] = round(prof["l2_bytes_per_launch"] / ksec / 1e9 / l2_peak, 3)
    if prof.get("warp_instructions_per_launch"):
        # 4 warp schedulers per SM, one issue each per cycle
        fractions["issue_slots"] = round(prof["warp_instructions_per_launch"] / (sms * 4 * sm_mhz * 1e6 * ksec), 3)

    line = {
        "metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_per_step, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded scene and rays)",
        "config": {"workload": WORKLOAD, "rays_per_step": n, "primary_rays": int(prim.shape[0]),
                   "bounce_rays": int(bounce.shape[0]), "triangles_per_instance": int(idx.shape[0]),
                   "instances": int(m.shape[0]), "l2": "inputs larger than L2 (~%d MB per step)" % (n * 56 // 2**20),
                   "parallelism": "replicas" if ws > 1 else "single GPU"},
        "e2e": {"value": round(e2e_val, 2), "unit": UNIT, "h2d_bytes_per_step": n * 56,
                "d2h_bytes_per_step": n * 56},
        "gpu_launches": args.steps,
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 3), "traffic": traffic,
                     "peak_source": "%s (MEASURED_PEAKS.json hbm_gbs)" % peak_kind if peak_kind == "measured" else "fallback",
                     # what actually binds: the algorithmic bytes are served from L2 /
                     # L1 (DRAM moves ~9% of them); the kernel is issue-bound
                     "limiter": "issue slots (ALU pipe, divergent warps)",
                     "fractions_of_measured": fractions,
                     "l2_copy_peak_gbs": round(l2_peak, 1),
                     "kernel": "k_trace<closest>", "kernel_ms": round(kernel_ms, 4),
                     "algorithmic_bytes_per_ray": round(per_ray, 1),
                     "node_visits_per_ray": round(counts["node_visits"] / counts["rays"], 2),
                     "tlas_node_visits_per_ray": round(counts["tlas_node_visits"] / counts["rays"], 2),
                     "tri_tests_per_ray": round(counts["tri_tests"] / counts["rays"], 2),
                     "instance_entries_per_ray": round(counts["instance_entries"] / counts["rays"], 2)},
        "clocks": clocks,
        "extra": {"anyhit_mrays_s": round(any_val, 1), "shadow_rays": int(shadow.shape[0]),
                  "watertight_mrays_s": round(wt_val, 1),
                  "watertight_vs_mt": {"rays": n, "hit_status_differs": diff_status,
                                       "primitive_differs": diff_prim, "t_bits_differ": diff_t,
                                       "primitive_differs_frac": round(diff_prim / n, 7)},
                  "build_ms": round(st["buildMs"], 1), "build_wall_s": round(build_s, 3),
                  "bvh_device_mb": round(st["deviceBytes"] / 2**20, 1),
                  "blas_nodes": st["blasNodes"]},
    }
    line["extra"].update(box_scene_pt(args, dev))
    if not args.no_pt_extras:
        line["extra"].update(c2_scene_pt(args, dev))
        line["extra"].update(c3_adjoint(args, dev))
        line["extra"].update(c4_equal_time(args, dev))
    line["extra"]["pt_roofline"] = pt_roofline(line["extra"], peak, l2_peak)
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(pos, idx, m, rays_np, budget_s=args.cpu_seconds)
        if not args.no_pt_extras:
            line["extra"]["pt_cpu_baselines"] = pt_cpu_baselines()
    if ws > 1:
        dist.barrier()
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(line))


def box_scene_pt(args, dev):
    """Box-scene path tracing (256x256, 16 spp, depth 8, RR from depth 3,
    NEE + MIS): samples per second and paths per second on the device."""
    import torch
    from mray_gb300.pt import PathTracer, load_box_scene
    from mray_gb300 import scenes
    pt = PathTracer(dev.index or 0)
    load_box_scene(pt, 0)
    cam = scenes.box_camera()
    reps = max(3, min(args.steps, 20))

    if getattr(args, "single_call", False):
        pt.render(PathTracer.params(256, 256, 16, cam, max_depth=8, rr_start=3, seed=0))
        torch.cuda.synchronize(dev)
        pt.close()
        return {"single_call": True}

    def timed(sampler):
        # the ZSobol group's initial sample count covers every timed call
        p = PathTracer.params(256, 256, 16, cam, max_depth=8, rr_start=3, seed=0, sampler=sampler,
                              sampler_max_spp=16 * (reps + 1))
        img = pt.render(p)
        torch.cuda.synchronize(dev)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for r in range(reps):
            p.sampleStart = 16 * (r + 1)
            pt.render(p, image=img)
        e1.record()
        torch.cuda.synchronize(dev)
        return e0.elapsed_time(e1) / reps

    ms = timed("independent")
    ms_zs = timed("zsobol-owen")

    # guided path tracing on the same workload: the grid learns across the calls
    pt.guide_create()
    p = PathTracer.params(256, 256, 16, cam, max_depth=8, rr_start=3, seed=0, samples_per_pass=16)
    img = pt.render_guided(p)
    torch.cuda.synchronize(dev)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for r in range(reps):
        p.sampleStart = 16 * (r + 1)
        pt.render_guided(p, image=img)
    e1.record()
    torch.cuda.synchronize(dev)
    ms_g = e0.elapsed_time(e1) / reps
    used, size = pt.guide_stats()
    pt.close()
    return {"box_pt_ms_per_16spp": round(ms, 3),
            "box_pt_spp_per_s": round(16.0 / (ms * 1e-3), 1),
            "box_pt_mpaths_per_s": round(256 * 256 * 16 / (ms * 1e-3) / 1e6, 1),
            "box_pt_zsobol_ms_per_16spp": round(ms_zs, 3),
            "box_guided_ms_per_16spp": round(ms_g, 3),
            "box_guided_mpaths_per_s": round(256 * 256 * 16 / (ms_g * 1e-3) / 1e6, 1),
            "box_guided_grid_entries": int(used), "box_guided_grid_table": int(size)}


def box_guided(args, dev):
    """Guided path tracing on the box workload alone (256x256, 16 spp per
    call, depth 8, RR from 3): with --single-call, two calls (the second on
    a grid the first filled), untimed."""
    import torch
    from mray_gb300.pt import PathTracer, load_box_scene
    from mray_gb300 import scenes
    pt = PathTracer(dev.index or 0)
    load_box_scene(pt, 0)
    pt.guide_create()
    p = PathTracer.params(256, 256, 16, scenes.box_camera(), max_depth=8, rr_start=3, seed=0, samples_per_pass=16)
    img = pt.render_guided(p)
    calls = 1 if getattr(args, "single_call", False) else max(3, min(args.steps, 20))
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for r in range(calls):
        p.sampleStart = 16 * (r + 1)
        pt.render_guided(p, image=img)
    e1.record()
    torch.cuda.synchronize(dev)
    ms = e0.elapsed_time(e1) / calls
    used, _ = pt.guide_stats()
    pt.close()
    return {"box_guided_ms_per_16spp": round(ms, 3), "box_guided_grid_entries": int(used)}


def _spectral_inputs():
    from mray_gb300 import spectral
    gold = os.path.join(ROOT, "tests", "golden")
    res, lut = spectral.read_mrspectra(os.path.join(gold, "REC_709_r32.mrspectra"))
    return res, lut, spectral.load_tables(os.path.join(gold, "spectral_rec709.npz"))


def c2_scene_pt(args, dev):
    """Spectral production scene (199,778 triangles, 509 surfaces, textured
    Lambert / GGX metal / glass, 8 area lights + a 1024x512 sky): 1920x1080,
    4 wavelengths per path, depth 12, RR from 3, NEE + MIS; samples per
    second (the configuration's 64 spp frame is timed in 4-spp steps)."""
    import torch
    from mray_gb300.pt import PathTracer, load_box_scene
    from mray_gb300 import scenes
    surf, cam = scenes.c2_scene(0)
    pt = PathTracer(dev.index or 0)
    load_box_scene(pt, surf)
    build_ms = pt.acc.stats()["buildMs"]        # all 509 BLASes + TLAS, wall clock of mrg_build
    pt.set_env(scenes.sky_map(1024, 512, seed=0))
    pt.set_spectral(*_spectral_inputs())
    spp = 4
    p = PathTracer.params(1920, 1080, spp, cam, max_depth=12, rr_start=3, seed=0)
    img = pt.render(p)
    torch.cuda.synchronize(dev)
    if getattr(args, "single_call", False):
        pt.close()
        return {"single_call": True}
    reps = max(3, min(args.steps // 20, 16))
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for r in range(reps):
        p.sampleStart = spp * (r + 1)
        pt.render(p, image=img)
    e1.record()
    torch.cuda.synchronize(dev)
    ms = e0.elapsed_time(e1) / reps
    pt.close()
    return {"c2_build_ms": round(float(build_ms), 2),
            "c2_ms_per_4spp_1080p": round(ms, 2), "c2_spp_per_s_1080p": round(spp / (ms * 1e-3), 1),
            "c2_mpaths_per_s": round(1920 * 1080 * spp / (ms * 1e-3) / 1e6, 1),
            "c2_ms_per_64spp_frame": round(ms * 16, 1)}


def c3_adjoint(args, dev):
    """Differentiable workload: box + 65,024-triangle textured sphere, 512^2
    f32 albedo texture, 512^2 image, 32 spp, depth 6; one path-replay adjoint
    (primal + replay) per step giving d(loss)/d(texture) and d(loss)/d(area-light
    emission)."""
    import torch
    from mray_gb300.pt import PathTracer
    from mray_gb300 import scenes
    tex = torch.from_numpy(scenes.value_noise_texture(512, seed=0, dtype=np.float32)).to(dev)
    surf = scenes.adjoint_scene(None)
    pt = PathTracer(dev.index or 0)
    for s in surf:
        inst = pt.add_surface(s["pos"], s["idx"], s["m34"], cull=s.get("cull", True), uv=s.get("uv"))
        if s["kind"] == "light":
            pt.set_area_light(inst, s["radiance"])
        else:
            pt.set_lambert(inst, s["albedo"])
        if "uv" in s:
            sphere = inst
    tid = pt.add_texture(tex)
    pt.set_albedo_texture(sphere, tid)
    pt.build()
    p = PathTracer.params(512, 512, 32, scenes.box_camera(), max_depth=6, rr_start=6, seed=0)
    delta = torch.full((512, 512, 4), 1e-6, dtype=torch.float32, device=dev)
    grad = torch.zeros((512, 512, 4), dtype=torch.float32, device=dev)
    grad_em = torch.zeros((pt.n_instances, 4), dtype=torch.float32, device=dev)
    pt.adjoint(p, tid, delta, grad=grad, grad_emission=grad_em)
    torch.cuda.synchronize(dev)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    reps = 3
    e0.record()
    for _ in range(reps):
        pt.adjoint(p, tid, delta, grad=grad, grad_emission=grad_em)
    e1.record()
    torch.cuda.synchronize(dev)
    ms = e0.elapsed_time(e1) / reps
    pt.close()
    return {"c3_adjoint_ms_512sq_32spp": round(ms, 2)}


def c4_equal_time(args, dev, spp_per_frame=8):
    """Radiance cache on the spectral production scene (config C2: 1920x1080,
    4 wavelengths, depth 12; 16 levels x 2 x 2^19 hash grid, 5 hidden 64-wide
    layers, lr 1e-2, about 32,768 training paths = up to 65,536 training
    samples per frame, paths end in the cache after one bounce), relMSE
    against a 4096-spp plain render:
    - cold start: from an untrained cache, T one-sample training frames
      (T = 4, 8, 16, 32, 64), then one cache-assisted frame of 1, 2, 4 or 8
      spp that does not train; the cheapest total (training frames included)
      whose frame reaches the 16-spp plain render's relMSE, and the plain
      render's time over it;
    - steady state (after the 64 training frames): equal-time relMSE of
      cache-assisted frames of spp_per_frame samples in the plain render's
      time, and the cheapest single cached frame (1, 2, 4 or 8 spp) that
      reaches the plain render's relMSE, training not counted."""
    import torch
    from mray_gb300.pt import PathTracer, load_box_scene
    from mray_gb300.cache import RadianceCache
    from mray_gb300 import scenes
    surf, cam = scenes.c2_scene(0)
    pt = PathTracer(dev.index or 0)
    load_box_scene(pt, surf)
    pt.set_env(scenes.sky_map(1024, 512, seed=0))
    pt.set_spectral(*_spectral_inputs())
    aabb = tuple(float(v) for v in pt.acc.scene_aabb())
    w, h = 1920, 1080

    def P(spp, seed, start=0, spp_pass=0):
        return PathTracer.params(w, h, spp, cam, max_depth=12, rr_start=3, seed=seed, sample_start=start,
                                 samples_per_pass=spp_pass)

    ref = pt.render(P(4096, 1, spp_pass=16))
    ref = (ref[..., :3] / ref[..., 3:]).double()

    def relmse(img):
        im = (img[..., :3] / img[..., 3:]).double()
        return float(torch.mean((im - ref) ** 2 / (ref ** 2 + 1e-2)))

    def timed(fn):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize(dev)
        e0.record()
        out = fn()
        e1.record()
        torch.cuda.synchronize(dev)
        return out, e0.elapsed_time(e1)

    pt.render(P(16, 7))
    plain, t_plain = timed(lambda: pt.render(P(16, 2)))
    plain_rel = relmse(plain)
    k = spp_per_frame
    out = {"c4_plain_16spp_ms": round(t_plain, 2), "c4_plain_relmse": round(plain_rel, 5)}

    # cold start: a fresh cache, training frames counted
    cache = RadianceCache(owner=pt, aabb=aabb, max_batch=65536)
    trained, t_train, cold = 0, 0.0, []
    for target in (4, 8, 16, 32, 64):
        def train():
            for f in range(trained, target):
                pt.render_cached(P(1, 100 + f, start=f), train_paths=32768)
        _, dt = timed(train)
        t_train += dt
        trained = target
        out["c4_cold_%dtrain_ms" % target] = round(t_train, 2)
        for spp in (1, 2, 4, 8):
            one, t_one = timed(lambda: pt.render_cached(P(spp, 5000 + target, start=0), train_paths=0)[0])
            rel = relmse(one)
            out["c4_cold_%dtrain_%dspp_relmse" % (target, spp)] = round(rel, 5)
            if rel <= plain_rel:
                cold.append((t_train + t_one, target, spp))
                break
    if cold:
        tt, n, spp = min(cold)
        out["c4_cold_start_time_to_plain_quality_ms"] = round(tt, 2)
        out["c4_cold_start_training_frames"] = n
        out["c4_cold_start_frame_spp"] = spp
        out["c4_cold_start_speedup"] = round(t_plain / tt, 3)

    # steady state (the cache trained on the 64 frames above)
    _, t_frame = timed(lambda: pt.render_cached(P(k, 300, start=0), train_paths=32768))
    frames = max(1, int(t_plain // t_frame))

    def run_frames():
        img = None
        for f in range(frames):
            img, _ = pt.render_cached(P(k, 1000 + f, start=k * f), image=img, train_paths=32768)
        return img
    img, t_cached = timed(run_frames)
    out.update({"c4_cached_frame_ms": round(t_frame, 3), "c4_cached_frames": frames,
                "c4_cached_spp_per_frame": k, "c4_cached_ms": round(t_cached, 2),
                "c4_cached_relmse": round(relmse(img), 5)})
    best = None
    for spp in (1, 2, 4, 8):
        one, t_one = timed(lambda: pt.render_cached(P(spp, 2000 + spp, start=0), train_paths=32768)[0])
        rel = relmse(one)
        out["c4_cached_%dspp_ms" % spp] = round(t_one, 3)
        out["c4_cached_%dspp_relmse" % spp] = round(rel, 5)
        if best is None and rel <= plain_rel:
            best = (spp, t_one)
    if best is not None:
        out["c4_steady_time_to_plain_quality_ms"] = round(best[1], 3)
        out["c4_steady_time_to_plain_quality_speedup"] = round(t_plain / best[1], 2)
    out["c4_workload"] = ("spectral production scene 1920x1080 (4 wavelengths) depth 12, reference 4096 spp plain; "
                          "cold start counts the training frames, steady state does not")
    cache.close()
    out.update(guided_equal_time(pt, P, relmse, timed, t_plain, plain_rel))
    # the same with zero-weight lobes falling back to the material sample
    fixed = guided_equal_time(pt, P, relmse, timed, t_plain, plain_rel, fix_zero_weight=True)
    out.update({k.replace("guided_", "guided_fixed_"): v for k, v in fixed.items() if "relmse" in k or "_ms" in k})
    pt.close()
    return out


def guided_equal_time(pt, P, relmse, timed, t_plain, plain_rel, spp=2, fix_zero_weight=False):
    """Guided path tracing (GuidedPTRenderer, default options) on the same
    scene and reference: from an empty grid, frames of `spp` samples per
    pixel accumulated for the plain 16-spp render's time (learning included),
    then, the grid trained, one more 16-spp guided frame against the plain
    16-spp render."""
    import torch
    pt.guide_create(fix_zero_weight=fix_zero_weight)
    pt.render_guided(P(spp, 900, spp_pass=spp))         # allocations, first launches
    pt.guide_clear()
    img, spent, frames = None, 0.0, 0
    while spent < t_plain:
        img, dt = timed(lambda: pt.render_guided(P(spp, 1000, start=spp * frames, spp_pass=spp), image=img))
        spent += dt
        frames += 1
    used, size = pt.guide_stats()
    one, t_one = timed(lambda: pt.render_guided(P(16, 3000, spp_pass=spp)))
    rel_one = relmse(one)
    return {"guided_equal_time_frames": frames, "guided_equal_time_spp": frames * spp,
            "guided_equal_time_ms": round(spent, 2), "guided_equal_time_relmse": round(relmse(img), 5),
            "guided_16spp_ms": round(t_one, 2), "guided_16spp_relmse": round(rel_one, 5),
            "guided_16spp_vs_plain_relmse": round(rel_one / plain_rel, 3),
            "guided_16spp_mpaths_per_s": round(1920 * 1080 * 16 / (t_one * 1e-3) / 1e6, 1),
            "guided_grid_entries": int(used), "guided_grid_table": int(size)}


def cache_micro(args, dev):
    """Radiance cache alone (16 levels x 2^19 x 2 hash grid, 5 x 64-wide MLP):
    one optimisation step on 65,536 (input, target) samples (forward,
    backward, tensor-core weight gradient, Adam) and a 2,073,600-sample query
    (one 1080p frame), device-timed with CUDA events."""
    import torch
    from mray_gb300.cache import RadianceCache
    rng = np.random.default_rng(0)

    def batch(n):
        x = np.zeros((n, 16), np.float32)
        x[:, 0:3] = rng.random((n, 3)) * 4 - 2
        x[:, 3] = rng.random(n)
        d = rng.standard_normal((n, 3))
        x[:, 4:7] = d / np.linalg.norm(d, axis=1, keepdims=True)
        x[:, 8:11] = x[:, 4:7]
        x[:, 12:15] = rng.random((n, 3))
        return torch.from_numpy(x).to(dev)

    def timed(fn, reps):
        for _ in range(3):
            fn()
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize(dev)
        return e0.elapsed_time(e1) / reps

    c = RadianceCache(device=dev.index or 0, aabb=(-2, -2, -2, 2, 2, 2), max_batch=65536)
    xb, tb = batch(65536), torch.rand((65536, 4), device=dev)
    reps = max(3, min(args.steps, 50))
    train_ms = timed(lambda: c.train(xb, tb, loss=False), reps)
    xq = batch(2073600)
    out = torch.empty((2073600, 4), dtype=torch.float32, device=dev)
    query_ms = timed(lambda: c.query(xq, out=out), reps)
    c.close()
    return {"cache_train_step_ms_65536": round(train_ms, 4), "cache_query_ms_2073600": round(query_ms, 4),
            "cache_query_msamples_per_s": round(2073600 / (query_ms * 1e-3) / 1e6, 1)}


def oracle_scene(pos, idx, m):
    import oracle
    S = oracle.Scene()
    mid = S.add_mesh(pos, idx, prim_key_base=0x10000000)
    for i in range(m.shape[0]):
        S.add_instance(mid, m[i], lm_key=i, trans_key=(1 << 24) | i, accel_key=(2 << 20) | i)
    S.build()
    return S


def sample_rays(rays, k):
    stride = max(1, rays.shape[0] // k)
    return np.ascontiguousarray(rays[::stride][:k])


def cpu_baseline(pos, idx, m, rays_np, budget_s=15.0):
    """The oracle (C restatement of MRay's host-backend LBVH cast) on every
    host core over a stride sample of the same ray set."""
    import oracle
    S = oracle_scene(pos, idx, m)
    threads = oracle.default_threads()
    k = 65536
    s = sample_rays(rays_np, k)
    t0 = time.perf_counter()
    S.cast_closest(s, threads=threads)
    dt = time.perf_counter() - t0
    rate = s.shape[0] / dt
    # grow the sample to roughly the time budget
    k2 = int(min(rays_np.shape[0], max(k, rate * budget_s)))
    s2 = sample_rays(rays_np, k2)
    t0 = time.perf_counter()
    S.cast_closest(s2, threads=threads)
    dt2 = time.perf_counter() - t0
    return {"value": round(s2.shape[0] / dt2 / 1e6, 3), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "%d of %d rays (stride sample of primary+bounce set), %.1f s" % (s2.shape[0], rays_np.shape[0], dt2)}


def pt_cpu_baselines(budget_s=10.0):
    """The path-tracer oracle (the C restatement of MRay's host-backend path
    tracer over its LBVH) on every host core: C0 (box scene, 256x256, depth 8,
    RR from 3, NEE + MIS) in samples per second over the full film, and C2
    (the spectral production scene, 1080p, depth 12) for one sample of every
    pixel.  The GPU numbers are
    box_pt_spp_per_s and c2_spp_per_s_1080p."""
    import oracle
    from mray_gb300 import scenes
    threads = oracle.default_threads()
    out = {}
    S = oracle.PtScene(scenes.box_scene(0))
    cam = scenes.box_camera()
    t0 = time.perf_counter()
    S.render(S.params(256, 256, 1, cam, max_depth=8, rr_start=3, seed=0), threads=threads)
    t1 = time.perf_counter() - t0
    spp = max(1, min(16, int(budget_s / max(t1, 1e-3))))
    t0 = time.perf_counter()
    S.render(S.params(256, 256, spp, cam, max_depth=8, rr_start=3, seed=0), threads=threads)
    dt = time.perf_counter() - t0
    out["c0"] = {"value": round(spp / dt, 2), "unit": "spp/s (256x256)", "cores": threads, "kind": "port",
                 "mpaths_per_s": round(256 * 256 * spp / dt / 1e6, 3),
                 "sample": "256x256 x %d spp, depth 8, NEE+MIS, %.1f s" % (spp, dt)}
    surf, ccam = scenes.c2_scene(0)
    sky = scenes.sky_map(1024, 512, seed=0)
    gold = os.path.join(ROOT, "tests", "golden")
    spec = oracle.Spectral(os.path.join(gold, "REC_709_r32.mrspectra"), os.path.join(gold, "spectral_rec709.npz"))
    t0 = time.perf_counter()
    S2 = oracle.PtScene(surf, env={"texels": sky}, spectral=spec)
    build_s = time.perf_counter() - t0
    # one sample of every pixel of the 1080p film
    p = S2.params(1920, 1080, 1, ccam, max_depth=12, rr_start=3, seed=0)
    t0 = time.perf_counter()
    S2.render(p, threads=threads)
    dt = time.perf_counter() - t0
    out["c2"] = {"value": round(1.0 / dt, 4), "unit": "spp/s (1080p)", "cores": threads, "kind": "port",
                 "mpaths_per_s": round(1920 * 1080 / dt / 1e6, 3),
                 "sample": "1920x1080 x 1 spp, spectral, depth 12, %.1f s; scene build %.1f s" % (dt, build_s)}
    return out


def reference_arm(args):
    """CPU restatement of MRay's host-backend cast (no reference CUDA path runs
    here: the reference's GPU backend needs OptiX or its own CUDA build)."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from mray_gb300 import build as B
    from mray_gb300 import scenes
    import oracle
    B.build_scenes()
    pos, idx, m, prim = make_workload()
    S = oracle_scene(pos, idx, m)
    threads = oracle.default_threads()
    # same primary+bounce mix as the GPU arm: sample primaries, bounce from their hits
    ps = sample_rays(prim, 32768)
    r, h, _, inst = S.cast_closest(ps, threads=threads)
    bounce, _ = scenes.bounce_rays(ps, inst, (h[:, 0] - 0x10000000).astype(np.uint32), r[:, 7], pos, idx, m, seed=1)
    sample = np.vstack([ps, bounce]).astype(np.float32)
    for _ in range(args.warmup):
        S.cast_closest(sample[:4096], threads=threads)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        S.cast_closest(sample, threads=threads)
        times.append(time.perf_counter() - t0)
    tot = sum(times)
    value = sample.shape[0] * args.steps / tot / 1e6
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(tot / args.steps * 1e3, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene and rays)",
        "impl": "reference",
        "config": {"workload": WORKLOAD, "rays_per_step": int(sample.shape[0]),
                   "sample": "32768 stride-sampled primaries + their diffuse bounces",
                   "parallelism": "host threads"},
        "cpu_baseline": {"value": round(value, 3), "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": "%d rays per step" % sample.shape[0]},
        "e2e": {"value": round(value, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def only_workload(args):
    import torch
    from mray_gb300 import build as B
    B.build()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    fn = {"c0": box_scene_pt, "c2": c2_scene_pt, "c3": c3_adjoint, "c4": c4_equal_time, "cache": cache_micro,
          "gbox": box_guided}[args.only]
    print(json.dumps({"workload": args.only, **fn(args, dev)}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-pt-extras", action="store_true",
                    help="skip the production-scene and adjoint path-tracing lines")
    ap.add_argument("--only", choices=["c0", "c2", "c3", "c4", "cache", "gbox"], default=None,
                    help="run one path-tracing workload alone and print its line (for profiling)")
    ap.add_argument("--single-call", action="store_true",
                    help="with --only c0 / c2: build the scene and render exactly one call, untimed "
                         "(the case the path-tracing roofline profile captures)")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl != "reference":
        args.warmup = 3
    if args.impl == "reference":
        reference_arm(args)
    elif args.only:
        only_workload(args)
    else:
        gpu_arm(args)


if __name__ == "__main__":
    main()
