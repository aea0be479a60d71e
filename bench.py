"""Benchmark of the GB300 ray-query path.

Default workload ("wavefront"): heightfield on a 1024x1024 vertex grid
(2,093,058 triangles, SAH build with <= 4 primitives per leaf), 1920x1080
pinhole primary rays from (0.5,-0.5,0.8) aimed at the grid centre, then per hit
one any-hit shadow ray to a point light at (0.2,0.2,2.0) and one
cosine-weighted diffuse bounce ray. One step = one frame of the wavefront
executor (rdn_wavefront_shadow_bounce). Metric: Mrays/s over all rays traced.

Further legs, each a key of the same JSON line (skipped with --no-<leg>):
  parity           every ray of the timed frame (and of the plain soup, and of
                   the watertight frame) classified against the oracle:
                   identical / exact-distance tie / NaN-exposed / edge / other;
  watertight       the frame with the watertight triangle test;
  plain_soup10k    the plain closest-hit configuration (10k soup, 256^2 rays);
  accuracy_vs_fp64 FP32 results against FP64 (same triangle, brute force);
  ao, task_graph   the AO renderer and the device task graph;
  batched          256 triangle soups, up to 4 diffuse bounces with Russian
                   roulette, one persistent launch per bounce in a CUDA graph,
                   against the plain per-scene launch loop (same tuned knobs);
  adjoint          256x256 heightfield, 512x512 rays, attribute loss: forward
                   and forward + adjoint, gradient error against FP64;
  batched_adjoint  64 heightfields, primaries + 2 bounces, forward + adjoint in
                   one graph, gradient error against FP64;
  cpu_baseline     the oracle's pipeline on the host cores (rank 0 only);
  headline         the metric's figures in one place.

--impl reference times the reference's CPU path for the same workload: the
oracle (a C++ restatement of the reference's CPU traversal, the Rust reference
cannot be built here) on all host cores over a bounded sample of the frame.

Multi-GPU (rendiation_gb300.partition): the frame is split into row bands, one
per GPU (strong scaling: `value` is one frame's rays over the slowest rank's
time); the batched legs split their scenes across GPUs balanced by triangles x
rays; the single-scene adjoint splits its rays and sums the vertex gradients
with one all-reduce after the backward. No other collective touches the data
path; the timed regions are bracketed by barriers and the max over ranks is
reported.
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

LIGHT = (0.2, 0.2, 2.0)
METRIC = "Mrays/s closest-hit: batched & fwd+adjoint vs plain, at stated FP64 error"


def algorithmic_roofline(alg_bytes: float, ms: float, basis: str) -> dict:
    """The HBM roofline figure of one launch (or graph): algorithmic bytes over
    its device time, against the measured HBM peak."""
    peak, kind = measured_peak_gbs()
    gbs = alg_bytes / (ms / 1e3) / 1e9
    return {"bound": "hbm", "achieved": round(gbs, 1), "peak": peak, "unit": "GB/s", "frac": round(gbs / peak, 4),
            "algorithmic_bytes": int(alg_bytes), "ms": round(ms, 4), "peak_kind": kind, "basis": basis}


def node_bytes_per_ray(counts: dict, n: int) -> float:
    """Algorithmic bytes per ray: 32 (ray in) + 16 (hit out) + 48 per node visit
    + 36 per triangle test, visits and tests counted in the reference's traversal
    order on the reference-built BVH."""
    return 32.0 + 16.0 + 48.0 * counts["node_visits"] / n + 36.0 * counts["tri_tests"] / n


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
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

    def summary(self) -> dict:
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for name, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(seconds: float, ws: int, device) -> float:
    """The slowest rank's time: every replica's timed region must have ended."""
    if ws == 1:
        return seconds
    import torch

    t = torch.tensor([seconds], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(count: int, ws: int) -> int:
    """Sum of an integer over the ranks (the rank's own value when alone)."""
    if ws <= 1:
        return int(count)
    import torch

    t = torch.tensor([int(count)], dtype=torch.int64, device="cuda" if torch.cuda.is_available() else "cpu")
    torch.distributed.all_reduce(t)
    return int(t.item())


def replicas_value(rays_per_step: int, steps: int, ws: int, seconds: float) -> float:
    """Whole-job Mrays/s of ws replicas that each traced steps x rays_per_step."""
    return rays_per_step * steps * ws / seconds / 1e6


def measured_peak_gbs():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_entry(workload: str, kernel: str) -> dict:
    """The committed ncu figures of one kernel (profiles/traffic.json), or {}."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(p):
        return {}
    with open(p) as f:
        return json.load(f).get(workload, {}).get(kernel, {})


def traffic_from_profile(workload: str, kernel: str):
    """Per-launch DRAM bytes of the dominant kernel from the committed ncu summary, if any."""
    e = profile_entry(workload, kernel)
    return float(e["dram_bytes_per_launch"]) if "dram_bytes_per_launch" in e else None


def measured_limits(workload: str, kernel: str, kernel_ms: float, peak_gbs: float, clocks: dict) -> dict:
    """What the counters of the committed ncu capture say bounds the kernel:
    dram_frac = measured DRAM bytes per launch over the live launch time, against
    the measured HBM peak; issue_frac = warp instructions per launch against the
    issue capacity of the launch (152 SMs x 4 schedulers x one instruction per
    clock at the sampled median SM clock); simt = threads per warp instruction."""
    e = profile_entry(workload, kernel)
    if not e:
        return {}
    out = {}
    if "dram_bytes_per_launch" in e:
        out["dram_frac"] = round(e["dram_bytes_per_launch"] / (kernel_ms / 1e3) / 1e9 / peak_gbs, 4)
    mhz = clocks.get("sm_mhz") or clocks.get("sm_max_mhz") or 2070.0
    if "warp_instructions_per_launch" in e:
        cap = 152 * 4 * float(mhz) * 1e6 * (kernel_ms / 1e3)
        out["issue_frac"] = round(e["warp_instructions_per_launch"] / cap, 4)
    if "threads_per_warp_instruction" in e:
        out["simt_lanes_per_warp_instruction"] = e["threads_per_warp_instruction"]
        out["limiter"] = (f"instruction issue with divergent lanes: {e['threads_per_warp_instruction']} of 32 lanes "
                          f"per warp instruction, issue active {round(100 * e['issue_active'], 1)} %, DRAM "
                          f"{e.get('dram_throughput_pct', '?')} % of peak (ncu, {e.get('source', 'profiles/')})")
    return out


# --------------------------------------------------------------------------- workloads

def build_heightfield_system(n_grid: int):
    """The heightfield scene, built on the host and on the GPU (kept); returns
    (mesh, system, build comparison)."""
    from rendiation_gb300 import raytracing as rt
    from rendiation_gb300 import scenes

    mesh = scenes.heightfield(n_grid, seed=1)
    P = rt.AccelerationStructureSystem(device=0)
    b = P.create_bottom_level_acceleration_structure([rt.BottomLevelAccelerationStructureBuildSource(
        mesh.positions, mesh.indices)])
    t = P.create_top_level_acceleration_structure([rt.TopLevelAccelerationStructureSourceInstance(b)])
    P.bind_tlas([t])
    return mesh, P, compare_builds(P)


def reference_counts_of_queues(P, wf, n_secondary):
    """Reference-order node visits / triangle tests of the rays one frame traced:
    the primaries (regenerated on the host, bit-identical to the kernel's camera
    rays) and the shadow and bounce queues read back from the scratch."""
    import torch

    from rendiation_gb300 import raytracing as rt
    from rendiation_gb300 import scenes

    prim = scenes.pinhole_rays(wf.camera)
    d_prim = torch.from_numpy(prim.view(np.float32).reshape(-1, 8).copy()).cuda()
    hits = torch.empty((prim.shape[0], 4), dtype=torch.float32, device="cuda")
    c_prim = P.trace_counted(d_prim, hits, traversal=rt.TRAVERSAL_REFERENCE)
    n = wf.n
    base = wf.scratch_ptr - wf.scratch.data_ptr()
    up = lambda b: (b + 255) & ~255  # noqa: E731
    sh = wf.scratch[base + 256: base + 256 + n_secondary * 32].view(torch.float32).reshape(-1, 8)
    # bounce rays: the grazing bin from the queue's front, the steep bin at its back
    n_front, n_back = (int(c) for c in wf.scratch[base + 8: base + 16].view(torch.int32).cpu().tolist())
    assert n_front + n_back == n_secondary
    bo_off = base + 256 + up(n * 32)
    bo_all = wf.scratch[bo_off: bo_off + n * 32].view(torch.float32).reshape(-1, 8)
    bo = torch.cat([bo_all[:n_front], bo_all[n - n_back:]])
    h2 = torch.empty((max(1, n_secondary), 4), dtype=torch.float32, device="cuda")
    c_sh = P.trace_counted(sh.contiguous(), h2, traversal=rt.TRAVERSAL_REFERENCE,
                           ray_flags=rt.RAY_FLAG_ACCEPT_FIRST_HIT_AND_END_SEARCH)
    c_bo = P.trace_counted(bo.contiguous(), h2, traversal=rt.TRAVERSAL_REFERENCE)
    return c_prim, c_sh, c_bo


def bench_wavefront(args, ws, rank):
    import torch

    from rendiation_gb300 import raytracing as rt
    from rendiation_gb300 import scenes

    W, H = args.width, args.height
    mesh, P, build = build_heightfield_system(args.grid)
    cam = scenes.heightfield_camera(W, H)
    traversal = {"reference": rt.TRAVERSAL_REFERENCE, "wide": rt.TRAVERSAL_ORDERED_WIDE}.get(
        args.traversal, rt.TRAVERSAL_ORDERED)
    # N GPUs split the frame into row bands (rendiation_gb300.partition): each
    # rank traces its band with the whole frame's rays and samplers
    from rendiation_gb300.partition import row_bands

    band = row_bands(H, ws)[rank]
    wf = rt.Wavefront(P, cam, LIGHT, traversal=traversal, block_size=args.block, rows=band)
    stream = torch.cuda.current_stream()
    tuned = None
    if args.tune and args.traversal == "ordered":
        from rendiation_gb300.autotune import Autotuner, grid

        tuner = Autotuner(args.tune_cache)
        # traversal stack in shared memory (local 0) or in local memory (1)
        orders = [rt.TRAVERSAL_ORDERED, rt.TRAVERSAL_ORDERED_WIDE]
        # register tier (regs) applies to the local-stack kernels
        cands = (grid(traversal=orders, block=[32, 64, 128], local=[0])
                 + grid(traversal=orders, block=[32, 64, 128], local=[1], regs=[0, 1, 2]))
        # secondary schedule: batches of 32 rays per warp (refill 0) or dynamic fetch
        cands2 = (grid(traversal=orders, block=[32, 64, 128], refill=[0], local=[0])
                  + grid(traversal=orders, block=[32, 64, 128], refill=[0], local=[1], regs=[0, 1, 2])
                  + grid(traversal=orders, block=[64], refill=[8, 16], local=[0]))

        def run_phase(ph):
            def run(c):
                wf.desc.traversal, wf.desc.block_size = c["traversal"], c["block"]
                wf.desc.refill, wf.desc.local_stack = c.get("refill", 0), c.get("local", 0)
                wf.desc.register_tier, wf.desc.speculation = c.get("regs", 0), c.get("spec", 0)
                wf.run(7, phases=ph)
            return run

        wf.run(7)
        torch.cuda.synchronize()
        t1 = tuner.tune("wavefront-primary", cands, run_phase(1))
        t2 = tuner.tune("wavefront-secondary", cands2, run_phase(2))
        # second stage: leaf-postponement threshold of the speculative walk
        b1, b2 = dict(t1.best), dict(t2.best)
        s1 = tuner.tune("wavefront-primary-speculation", [dict(b1, spec=k) for k in (0, 2, 4, 8, 16)],
                        run_phase(1))
        s2 = tuner.tune("wavefront-secondary-speculation", [dict(b2, spec=k) for k in (0, 2, 4, 8, 16)],
                        run_phase(2))
        b1, b2 = s1.best, s2.best
        wf.configure((b1["traversal"], b1["block"], b1.get("local", 0), b1.get("regs", 0), b1.get("spec", 0)),
                     (b2["traversal"], b2["block"], b2.get("local", 0), b2.get("regs", 0), b2.get("spec", 0)),
                     refill=b2.get("refill", 0))
        tuned = {"primary": b1, "secondary": b2}

    # one frame to learn the ray counts, then the reference-order visit counts of those rays
    wf.run(0)
    torch.cuda.synchronize()
    n_prim, n_sh, n_bo = wf.rays_traced()
    rays_per_step = n_prim + n_sh + n_bo
    c_prim, c_sh, c_bo = reference_counts_of_queues(P, wf, n_sh)
    bytes_primary = n_prim * node_bytes_per_ray(c_prim, n_prim)
    bytes_secondary = n_sh * node_bytes_per_ray(c_sh, max(1, n_sh)) + n_bo * node_bytes_per_ray(c_bo, max(1, n_bo))

    for s in range(args.warmup):
        wf.run(1 + s)
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()

    # device-timed region: K frames, events around every kernel launch pair
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(torch.cuda.current_device()) as clk:
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()
        start.record(stream)
        for s in range(args.steps):
            ev[s][0].record(stream)
            wf.run(100 + s)
            ev[s][1].record(stream)
        stop.record(stream)
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()
    total_ms = start.elapsed_time(stop)

    # per-kernel split of a frame, outside the timed region: events on the
    # launching stream around the primary kernel and the secondary kernel
    import ctypes as C

    k_prim, k_sec = [], []
    for s in range(max(3, min(args.steps, 10))):
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))  # noqa: B007
        e0.record(stream)
        wf.run(200 + s, phases=1)
        e1.record(stream)
        wf.run(200 + s, phases=2)
        e2.record(stream)
        torch.cuda.synchronize()
        k_prim.append(e0.elapsed_time(e1))
        k_sec.append(e1.elapsed_time(e2))
    prim_ms, sec_ms = float(np.mean(k_prim)), float(np.mean(k_sec))
    frame_ms = total_ms / args.steps
    elapsed = total_ms / 1000.0
    elapsed = max_over_ranks(elapsed, ws, "cuda")
    # whole-job rays of one frame: the bands' rays summed over ranks
    frame_rays = sum_over_ranks(rays_per_step, ws)
    value = frame_rays * args.steps / elapsed / 1e6

    # e2e through the C ABI: every step launches its frame and reads all of its
    # pixel records back into pinned host memory. Two output buffers: the copy
    # of frame k (copy stream) overlaps frame k+1 (compute stream); frame k+2
    # waits for that copy before it overwrites the buffer.
    wf2 = rt.Wavefront(P, cam, LIGHT, traversal=traversal, block_size=args.block, rows=band)
    if wf.phase_config is not None:
        wf2.configure(*wf.phase_config, refill=wf.desc.refill)
    else:
        same = (wf.desc.traversal, wf.desc.block_size, wf.desc.local_stack, wf.desc.register_tier,
                wf.desc.speculation)
        wf2.configure(same, same, refill=wf.desc.refill)
    frames = (wf, wf2)
    host_out = [torch.empty(wf.out.shape, dtype=wf.out.dtype, pin_memory=True) for _ in range(2)]
    copy_stream = torch.cuda.Stream()
    done_frame = [torch.cuda.Event() for _ in range(2)]
    done_copy = [torch.cuda.Event() for _ in range(2)]

    def e2e_steps(k0, count):
        for s in range(count):
            b = s % 2
            if s >= 2:
                stream.wait_event(done_copy[b])
            frames[b].run(k0 + s)
            done_frame[b].record(stream)
            copy_stream.wait_event(done_frame[b])
            with torch.cuda.stream(copy_stream):
                host_out[b].copy_(frames[b].out, non_blocking=True)
            done_copy[b].record(copy_stream)
        torch.cuda.synchronize()

    e2e_steps(300, 4)
    t0 = time.perf_counter()
    e2e_steps(400, args.steps)
    e2e_s = time.perf_counter() - t0
    e2e_s = max_over_ranks(e2e_s, ws, "cuda")
    e2e_value = frame_rays * args.steps / e2e_s / 1e6
    d2h = int(wf.out.numel() * 4)
    h2d = C.sizeof(wf.desc)

    peak, peak_kind = measured_peak_gbs()
    if sec_ms >= prim_ms:
        dom_name, dom_bytes, dom_ms = "secondary_kernel (shadow + bounce queues)", bytes_secondary, sec_ms
    else:
        dom_name, dom_bytes, dom_ms = "primary_kernel (raygen + trace + shade + enqueue)", bytes_primary, prim_ms
    achieved = dom_bytes / (dom_ms / 1000.0) / 1e9
    out = {
        "metric": METRIC,
        "value": round(value, 3),
        "unit": "Mrays/s",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(frame_ms, 4),
        "higher_is_better": True,
        "scaling": "strong",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded heightfield, PCG64 seed 1)",
        "config": {
            "workload": f"wavefront primary+shadow+bounce, heightfield {args.grid}^2 "
                        f"({mesh.triangle_count} tris, SAH <=4/leaf), {W}x{H} primaries",
            "rays_per_step": frame_rays,
            "partition": f"{ws} row band(s) of the frame, one per GPU (strong scaling: one frame per step)",
            "rays_primary": n_prim, "rays_shadow": n_sh, "rays_bounce": n_bo,
            "traversal": args.traversal,
            "autotuned": tuned,
            "l2": f"no flush: acceleration structure {P.device_bytes() / 1e6:.0f} MB on device > 129 MB L2",
        },
        "e2e": {"value": round(e2e_value, 3), "unit": "Mrays/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h,
                "pipelining": "pixel records of frame k copied to pinned host memory while frame k+1 runs"},
        "gpu_launches": 2 * args.steps,
        "roofline": {
            "bound": "hbm",
            "achieved": round(achieved, 1),
            "peak": peak,
            "unit": "GB/s",
            "frac": round(achieved / peak, 4),
            "achieved_basis": ("algorithmic: per ray the reference order's node (48 B) and triangle (36 B) fetches "
                               "plus ray and hit, over the launch; the ordered walk does that work with far fewer "
                               "fetches, so frac can exceed 1 and does not measure bandwidth use"),
            "traffic": traffic_from_profile("wavefront", dom_name.split()[0]),
            "kernel": dom_name,
            "kernel_ms": round(dom_ms, 4),
            "kernel_ms_split": {"primary": round(prim_ms, 4), "secondary": round(sec_ms, 4)},
            "algorithmic_bytes_per_launch": int(dom_bytes),
            "bytes_per_ray": {"primary": round(node_bytes_per_ray(c_prim, n_prim), 1),
                              "shadow": round(node_bytes_per_ray(c_sh, max(1, n_sh)), 1),
                              "bounce": round(node_bytes_per_ray(c_bo, max(1, n_bo)), 1)},
            "peak_kind": peak_kind,
            **measured_limits("wavefront", dom_name.split()[0], dom_ms, peak, clk.summary()),
        },
        "clocks": clk.summary(),
        "build": build,
    }
    return out, P, mesh, cam, wf


def watertight_twin(P, wf, cam):
    """A frame with wf's launch knobs and the watertight triangle test."""
    from rendiation_gb300 import raytracing as rt

    wt = rt.Wavefront(P, cam, LIGHT)
    if wf.phase_config is not None:
        (p1, p2) = wf.phase_config
        wt.configure((p1[0] | rt.INTERSECT_WATERTIGHT,) + tuple(p1[1:]),
                     (p2[0] | rt.INTERSECT_WATERTIGHT,) + tuple(p2[1:]), refill=wf.desc.refill)
    else:
        same = (wf.desc.traversal | rt.INTERSECT_WATERTIGHT, wf.desc.block_size, wf.desc.local_stack,
                wf.desc.register_tier, wf.desc.speculation)
        wt.configure(same, same, refill=wf.desc.refill)
    return wt


def parity_report(P, S_field, wf, cam, threads: int) -> dict:
    """Parity of the timed configuration with the oracle (the CPU restatement
    of the reference's path), every ray classified (oracle.parity): identical,
    exact-distance tie, NaN-exposed, edge, other; `other` must be 0.
      frame      the whole 1920x1080 frame of the wavefront leg with the
                 autotuned knobs it was timed with, against the oracle's
                 pipeline over the same frame;
      soup10k    the plain closest-hit configuration: 10,000-triangle soup,
                 256x256 pinhole rays, rdn_trace with the cfg0 leg's knobs;
      watertight the frame's primary rays traced with the watertight test,
                 against the reference's formula (near ties and edge cases
                 only), and the watertight frame against the oracle's
                 watertight pipeline."""
    import torch

    from oracle import orc
    from oracle import parity
    from rendiation_gb300 import raytracing as rt
    from rendiation_gb300 import scenes

    W, H = cam.width, cam.height
    out = {}
    sample = 77
    wf.run(sample)
    torch.cuda.synchronize()
    got = wf.results()
    t0 = time.perf_counter()
    exp, _, sec = orc.wavefront_shadow_bounce(S_field, cam.as_floats(), W, H, LIGHT, sample, threads=threads)
    out["frame"] = parity.classify_wavefront(S_field, cam, W, H, LIGHT, got, exp, sample, threads=threads)
    out["frame"]["oracle_seconds"] = round(sec, 3)

    # the plain closest-hit configuration
    soup = scenes.triangle_soup(10_000, seed=0)
    Ps = rt.AccelerationStructureSystem(device=0)
    b = Ps.create_bottom_level_acceleration_structure([rt.BottomLevelAccelerationStructureBuildSource(soup.positions)])
    Ps.bind_tlas([Ps.create_top_level_acceleration_structure([rt.TopLevelAccelerationStructureSourceInstance(b)])])
    Ps.build(blas_bin_size=4, device_build=True)
    Ss = orc.OracleSystem()
    sb = Ss.create_blas([(soup.positions, None, 1)])
    Ss.bind_tlas([Ss.create_tlas([{"blas": sb}])])
    Ss.build(blas_bin_size=4)
    srays = scenes.pinhole_rays(scenes.soup_camera())
    d = torch.from_numpy(srays.view(np.float32).reshape(-1, 8).copy()).cuda()
    hits = torch.empty((srays.shape[0], 4), device="cuda")
    ext = torch.empty((srays.shape[0], 4), dtype=torch.int32, device="cuda")
    Ps.trace(d, hits, ext, traversal=rt.TRAVERSAL_ORDERED_WIDE, local_stack=1)
    torch.cuda.synchronize()
    e_soup, _ = Ss.trace(srays, threads=threads)
    _, out["soup10k"] = parity.classify_trace(Ss, srays, rt.hits_to_numpy(hits), ext.cpu().numpy().view(np.uint32),
                                              e_soup, exact=True, threads=threads)
    Ps.close()

    # the watertight test against the reference's formula, on the frame's primary rays
    prim = scenes.pinhole_rays(cam)
    dp = torch.from_numpy(prim.view(np.float32).reshape(-1, 8).copy()).cuda()
    hp = torch.empty((prim.shape[0], 4), device="cuda")
    xp = torch.empty((prim.shape[0], 4), dtype=torch.int32, device="cuda")
    P.trace(dp, hp, xp, traversal=rt.TRAVERSAL_ORDERED_WIDE | rt.INTERSECT_WATERTIGHT, local_stack=1)
    torch.cuda.synchronize()
    e_ref, _ = S_field.trace(prim, threads=threads)
    g_wt = rt.hits_to_numpy(hp)
    _, c = parity.classify_trace(S_field, prim, g_wt, xp.cpu().numpy().view(np.uint32), e_ref, exact=False,
                                 threads=threads)
    c["hits_reference_formula"] = int((e_ref["prim"] != orc.MISS).sum())
    c["hits_watertight"] = int((g_wt["prim"] != orc.MISS).sum())
    same = (g_wt["prim"] == e_ref["prim"]) & (e_ref["prim"] != orc.MISS)
    c["max_rel_t_difference_same_triangle"] = float(np.max(np.abs(g_wt["t"][same].astype(np.float64) - e_ref["t"][same])
                                                           / e_ref["t"][same])) if same.any() else 0.0
    out["watertight_primaries_vs_reference_formula"] = c
    # the watertight frame against the oracle's watertight pipeline
    wt_frame = watertight_twin(P, wf, cam)
    wt_frame.run(sample)
    torch.cuda.synchronize()
    exp_wt, _, _ = orc.wavefront_shadow_bounce(S_field, cam.as_floats(), W, H, LIGHT, sample, threads=threads,
                                               watertight=True)
    out["watertight_frame"] = parity.classify_wavefront(S_field, cam, W, H, LIGHT, wt_frame.results(), exp_wt, sample,
                                                        watertight=True, threads=threads)
    out["other_total"] = (out["frame"]["other"] + out["soup10k"]["other"]
                          + out["watertight_primaries_vs_reference_formula"]["other"]
                          + out["watertight_frame"]["other"])
    out["seconds"] = round(time.perf_counter() - t0, 2)
    out["threads"] = threads
    return out


def bench_watertight(args, P, wf, cam) -> dict:
    """The wavefront frame with the watertight triangle test (same tuned knobs,
    RDN_INTERSECT_WATERTIGHT OR-ed into both kernels' traversal), device-timed
    like the main leg, against the reference's formula."""
    import torch

    from rendiation_gb300 import raytracing as rt

    wt = watertight_twin(P, wf, cam)
    stream = torch.cuda.current_stream()
    res = {}
    for name, frame in (("reference_formula", wf), ("watertight", wt)):
        for s in range(args.warmup):
            frame.run(500 + s)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        reps = max(5, min(args.steps, 20))
        e0.record(stream)
        for s in range(reps):
            frame.run(600 + s)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        rays = sum(frame.rays_traced())
        res[name] = {"frame_ms": round(ms, 4), "mrays": round(rays / (ms / 1e3) / 1e6, 2), "rays_per_frame": rays}
    res["watertight_over_reference_formula_time"] = round(res["watertight"]["frame_ms"]
                                                          / res["reference_formula"]["frame_ms"], 4)
    return res


def bench_plain_soup(args) -> dict:
    """The plain closest-hit configuration: 10,000-triangle soup (seeded;
    centroids U[0,1]^3, vertex offsets U[-0.02,0.02]^3), SAH <= 4 per leaf,
    256x256 pinhole rays from (0.5,0.5,-1.5) along +z, 60 degree vertical field
    of view; rdn_trace per step. The structure (about 1.3 MB) is L2-resident, so
    the bound is L2, not HBM: `l2_gbs` is the algorithmic bytes (reference-order
    node and triangle fetches, rays and hits) over the device time. e2e: the
    same query through the C ABI from pinned host rays to pinned host hits."""
    import torch

    from rendiation_gb300 import raytracing as rt
    from rendiation_gb300 import scenes

    soup = scenes.triangle_soup(10_000, seed=0)
    P = rt.AccelerationStructureSystem(device=0)
    b = P.create_bottom_level_acceleration_structure([rt.BottomLevelAccelerationStructureBuildSource(soup.positions)])
    P.bind_tlas([P.create_top_level_acceleration_structure([rt.TopLevelAccelerationStructureSourceInstance(b)])])
    P.build(blas_bin_size=4, device_build=True)
    rays = scenes.pinhole_rays(scenes.soup_camera())
    n = rays.shape[0]
    d = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).cuda()
    hits = torch.empty((n, 4), device="cuda")
    stream = torch.cuda.current_stream()
    cands = [(trav, block, local) for trav in (rt.TRAVERSAL_ORDERED, rt.TRAVERSAL_ORDERED_WIDE)
             for block in (32, 64, 128) for local in (0, 1)]

    def time_ms(trav, block, local, reps=200):
        for _ in range(5):
            P.trace(d, hits, traversal=trav, block_size=block, local_stack=local)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            P.trace(d, hits, traversal=trav, block_size=block, local_stack=local)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    timings = {c: time_ms(*c, reps=50) for c in cands}
    best = min(timings, key=timings.get)
    ms = time_ms(*best, reps=max(200, args.steps * 10))
    c_ref = P.trace_counted(d, hits, traversal=rt.TRAVERSAL_REFERENCE)
    alg_bytes = n * node_bytes_per_ray(c_ref, n)
    # e2e: pinned host rays in, pinned host hits out, every step
    h_rays = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).pin_memory()
    h_hits = torch.empty((n, 4), dtype=torch.float32).pin_memory()
    for _ in range(5):
        d.copy_(h_rays, non_blocking=True)
        P.trace(d, hits, traversal=best[0], block_size=best[1], local_stack=best[2])
        h_hits.copy_(hits, non_blocking=True)
    torch.cuda.synchronize()
    steps = max(50, args.steps)
    t0 = time.perf_counter()
    for _ in range(steps):
        d.copy_(h_rays, non_blocking=True)
        P.trace(d, hits, traversal=best[0], block_size=best[1], local_stack=best[2])
        h_hits.copy_(hits, non_blocking=True)
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / steps
    P.close()
    return {
        "workload": "soup 10,000 tris, 256x256 pinhole primaries, rdn_trace closest hit",
        "knobs": {"traversal": best[0], "block": best[1], "local_stack": best[2]},
        "device_ms": round(ms, 5),
        "mrays": round(n / (ms / 1e3) / 1e6, 2),
        "algorithmic_bytes_per_launch": int(alg_bytes),
        "bytes_per_ray": round(node_bytes_per_ray(c_ref, n), 1),
        "l2_gbs": round(alg_bytes / (ms / 1e3) / 1e9, 1),
        "bound": "L2 (structure about 1.3 MB, L2-resident)",
        "hbm_frac_algorithmic": round(alg_bytes / (ms / 1e3) / 1e9 / measured_peak_gbs()[0], 4),
        "e2e": {"mrays": round(n / e2e_s / 1e6, 2), "ms": round(e2e_s * 1e3, 4), "h2d_bytes_per_step": n * 32,
                "d2h_bytes_per_step": n * 16},
    }


def compare_builds(P, bin_size=4) -> dict:
    """Builds P's structure on the host, then on the GPU (the one kept), and
    checks that the reference-layout arrays of both builds are identical."""
    t0 = time.perf_counter()
    P.build(blas_bin_size=bin_size)
    host_s = time.perf_counter() - t0
    host = {name: P.built_array(name) for name in ("tri_bvh_forest", "indices_redirect", "tri_bvh_root")}
    P.build(blas_bin_size=bin_size, device_build=True)  # warm (context, allocator)
    t0 = time.perf_counter()
    P.build(blas_bin_size=bin_size, device_build=True)
    dev_s = time.perf_counter() - t0
    st = P.build_stats()
    same = all(P.built_array(name) == data for name, data in host.items())
    del host
    return {"host_s": round(host_s, 4), "host_threads": os.cpu_count(), "device_s": round(dev_s, 4),
            "device_gpu_span_s": round(st["device_seconds"], 5), "speedup": round(host_s / dev_s, 1),
            "triangles": st["triangles"], "nodes": st["nodes"], "arrays_identical": bool(same),
            "compared": "tri_bvh_forest, indices_redirect, tri_bvh_root (byte equality)"}


def accuracy_vs_fp64(P, S, cam, sample=65536):
    """Errors of the product's FP32 closest hits against FP64, the figure the
    metric is stated at: (1) a sample of the frame's primary rays, each hit
    re-evaluated in FP64 on the same triangle (the oracle's evaluator); (2) a
    10,000-triangle soup with 64x64 pinhole rays against an FP64 brute-force
    closest hit over every triangle (no BVH)."""
    import torch

    from oracle import orc
    from rendiation_gb300 import raytracing as rt
    from rendiation_gb300 import scenes

    def product_hits(system, rays):
        d = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).cuda()
        hits = torch.empty((rays.shape[0], 4), device="cuda")
        ext = torch.empty((rays.shape[0], 4), dtype=torch.int32, device="cuda")
        system.trace(d, hits, ext, traversal=rt.TRAVERSAL_ORDERED_WIDE, local_stack=1)
        torch.cuda.synchronize()
        h = rt.hits_to_numpy(hits)
        out = np.zeros(rays.shape[0], orc.HIT_DTYPE)
        for k in ("t", "u", "v", "prim"):
            out[k] = h[k]
        e = ext.cpu().numpy().view(np.uint32)
        out["geometry"], out["instance"] = e[:, 0], e[:, 1]
        return out

    rays = scenes.pinhole_rays(cam)
    pick = np.random.default_rng(5).choice(rays.shape[0], min(sample, rays.shape[0]), replace=False)
    r = np.ascontiguousarray(rays[pick])
    got = product_hits(P, r)
    f64 = S.eval_fp64(r, got)
    hit = got["prim"] != orc.MISS
    rel_t = np.abs(got["t"][hit] - f64[hit, 0]) / np.maximum(np.abs(f64[hit, 0]), 1e-30)
    bary = np.maximum(np.abs(got["u"][hit] - f64[hit, 1]), np.abs(got["v"][hit] - f64[hit, 2]))

    soup = scenes.triangle_soup(10_000, seed=0)
    Ps = rt.AccelerationStructureSystem(device=0)
    b = Ps.create_bottom_level_acceleration_structure([rt.BottomLevelAccelerationStructureBuildSource(soup.positions)])
    Ps.bind_tlas([Ps.create_top_level_acceleration_structure([rt.TopLevelAccelerationStructureSourceInstance(b)])])
    Ps.build(blas_bin_size=4, device_build=True)
    Ss = orc.OracleSystem()
    sb = Ss.create_blas([(soup.positions, None, 1)])
    Ss.bind_tlas([Ss.create_tlas([{"blas": sb}])])
    Ss.build(blas_bin_size=4)
    srays = scenes.pinhole_rays(scenes.soup_camera(64, 64))
    sg = product_hits(Ps, srays)
    truth = Ss.bruteforce_fp64(srays, threads=os.cpu_count() or 1)
    t_hit = np.isfinite(truth[:, 0])
    g_hit = sg["prim"] != orc.MISS
    both = t_hit & g_hit
    Ps.close()
    return {
        "heightfield_primary_rays_sampled": int(r.shape[0]),
        "max_rel_t_error_vs_fp64_same_triangle": float(rel_t.max()) if rel_t.size else 0.0,
        "max_abs_barycentric_error_vs_fp64": float(bary.max()) if bary.size else 0.0,
        "soup10k_rays": int(srays.shape[0]),
        "soup_hit_miss_disagreements_vs_fp64_bruteforce": int(np.sum(t_hit != g_hit)),
        "soup_closest_triangle_disagreements_vs_fp64_bruteforce": int(np.sum(sg["prim"][both]
                                                                            != truth[both, 3].astype(np.uint32))),
        "soup_max_rel_t_error_vs_fp64_bruteforce": float(np.max(np.abs(sg["t"][both] - truth[both, 0])
                                                                / truth[both, 0])) if both.any() else 0.0,
        "note": ("u, v follow the reference's projected-barycentric formula bit for bit; its error grows as "
                 "1/cos of the angle between the ray and the triangle plane (the differentiable kernels "
                 "re-solve u, v in float-float)"),
    }


def oracle_heightfield(mesh):
    from oracle import orc

    S = orc.OracleSystem()
    b = S.create_blas([(mesh.positions, mesh.indices, 1)])
    t = S.create_tlas([{"blas": b}])
    S.bind_tlas([t])
    S.build(blas_bin_size=4)
    return S


def bench_ao(args, P, S_field):
    """Ray-traced ambient occlusion of the reference (feature/ao.rs) on the
    1024^2 heightfield: a 512x512 frame (the reference clamps AO frames to
    512^2 pixels), one jittered camera ray per pixel and one occlusion ray per
    hit, progressive average into RGBA8. The fused kernel against the
    reference's pipeline as a device task graph (5 task groups, 8 rounds),
    issued as plain launches and replayed from a captured CUDA graph. The
    sample index advances every frame."""
    import ctypes as C

    import torch

    from rendiation_gb300 import native
    from rendiation_gb300 import raytracing as rt
    from rendiation_gb300 import task_graph as tg

    L = native.lib()
    W = H = 512
    eye = (0.5, -0.5, 0.8)
    vp = tg.look_at_view_projection_inv(eye, (0.5, 0.5, 0.0), (0, 0, 1), 20.0, 1.0, 0.01, 100.0)
    # coherent camera rays: the four-child walk unless the reference order is asked for
    traversal = rt.TRAVERSAL_REFERENCE if args.traversal == "reference" else rt.TRAVERSAL_ORDERED_WIDE
    stream = torch.cuda.current_stream()
    sp = C.c_void_p(stream.cuda_stream)
    counts = torch.zeros(2, dtype=torch.int32, device="cuda")
    images = {m: torch.zeros(W * H * 4, dtype=torch.uint8, device="cuda") for m in ("fused", "graph")}
    descs = {m: tg.ao_desc(W, H, vp, eye, images[m], 0, 0, traversal) for m in images}
    for d in descs.values():
        d.ray_counts = counts.data_ptr()
    h = C.c_void_p()
    assert L.rdn_ao_pipeline_create(P._h, W, H, sp, C.byref(h)) == 0

    def frame(mode, s):
        d = descs[mode]
        d.sample_count = s % 256
        if mode == "fused":
            assert L.rdn_ao_render(P._h, C.byref(d), sp) == 0
        else:
            assert L.rdn_ao_render_graph(h, C.byref(d), sp) == 0

    # one frame each from a zero image: the two forms must write the same bytes
    frame("fused", 0)
    frame("graph", 0)
    torch.cuda.synchronize()
    out = {"images_equal": bool(torch.equal(images["fused"], images["graph"]))}
    reps = 20

    def timed(fn):
        for k in range(args.warmup):
            fn(k)
        counts.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for k in range(reps):
            fn(args.warmup + k)
        e1.record(stream)
        torch.cuda.synchronize()
        c = counts.cpu().numpy()
        return e0.elapsed_time(e1) / reps, (int(c[0]) + int(c[1])) / reps

    # launch shape of the fused kernel: block size and node layout, timed on the frame
    shapes = {}
    for trav in (rt.TRAVERSAL_ORDERED, rt.TRAVERSAL_ORDERED_WIDE) if traversal != rt.TRAVERSAL_REFERENCE else (traversal,):
        for block in (32, 64, 128):
            descs["fused"].traversal, descs["fused"].block_size = trav, block
            shapes[(trav, block)] = timed(lambda k: frame("fused", k))[0]
    best = min(shapes, key=shapes.get)
    descs["fused"].traversal, descs["fused"].block_size = best
    out["fused_shape"] = {"traversal": {0: "binary", 1: "reference", 2: "wide"}[best[0]], "block": best[1]}
    # leaf postponement threshold of the ordered walks, per form, timed on the frame
    if traversal != rt.TRAVERSAL_REFERENCE:
        for mode in ("fused", "graph"):
            spec_ms = {}
            for k in (0, 2, 4, 8, 16):
                descs[mode].speculation = k
                spec_ms[k] = timed(lambda i: frame(mode, i))[0]
            descs[mode].speculation = min(spec_ms, key=spec_ms.get)
            out[mode + "_speculation"] = descs[mode].speculation
            out[mode + "_speculation_ms"] = {str(k): round(v, 4) for k, v in spec_ms.items()}
    ms, rays = timed(lambda k: frame("fused", k))
    out["rays_per_frame"] = rays
    out["fused_ms"], out["fused_mrays"] = round(ms, 4), round(rays / ms / 1e3, 1)
    ms, rays_g = timed(lambda k: frame("graph", k))
    out["graph_ms"], out["graph_mrays"] = round(ms, 4), round(rays_g / ms / 1e3, 1)
    # each form captured once (rdn_ao_capture) and replayed; the frame reads and
    # advances a device sample counter, so every replay draws the next sample
    counter = torch.zeros(1, dtype=torch.int32, device="cuda")
    for mode, pipe in (("fused", None), ("graph", h)):
        d = descs[mode]
        d.sample_counter = counter.data_ptr()
        ge = C.c_void_p()
        assert L.rdn_ao_capture(P._h, pipe, C.byref(d), C.byref(ge)) == 0
        ms, rays_c = timed(lambda k: L.rdn_graph_launch(ge, sp))
        L.rdn_graph_destroy(ge)
        d.sample_counter = None
        out[mode + "_captured_ms"], out[mode + "_captured_mrays"] = round(ms, 4), round(rays_c / ms / 1e3, 1)
    out["graph_over_fused"] = round(out["graph_ms"] / out["fused_ms"], 2)
    out["graph_launches_per_frame"] = 3 + 8 * (1 + 5 * 2)  # per round: drain, then a poll and a bookkeep per group
    out["captured"] = "rdn_ao_capture: one CUDA graph per frame, sample index read from a device counter"
    st, flags = P.check_errors()
    assert st == 0 and flags == 0
    L.rdn_task_graph_destroy(h)
    if S_field is not None:
        from oracle import orc

        img = np.zeros(W * H, np.uint32)
        rows = (0, 64)
        n, sec = orc.ao_render(S_field, vp, eye, W, H, img, sample_count=0, rows=rows, threads=os.cpu_count() or 1)
        out["cpu_mrays"] = round((n[0] + n[1]) / sec / 1e6, 2)
        out["cpu_threads"] = os.cpu_count() or 1
        out["cpu_sample"] = f"rows {rows[0]}..{rows[1]} of the frame"
    out["traversal"] = {rt.TRAVERSAL_REFERENCE: "reference", rt.TRAVERSAL_ORDERED_WIDE: "wide"}.get(traversal, "ordered")
    out["workload"] = (f"heightfield 1024^2 (2093058 tris), AO {W}x{H}: camera ray + occlusion ray per hit "
                       "(ACCEPT_FIRST_HIT_AND_END_SEARCH, [0.01, 100])")
    return out


def bench_path_tracing(args, P, S_field):
    """The reference path tracer (feature/path_tracing) on the 1024^2
    heightfield: one sample per pixel, max_path_depth 3, one directional light,
    the default physical material, ACES tone map, progressive RGBA8 average.
    Timed at the reference's own render size for a 1920x1080 frame
    (clamp_size_by_area to 512^2 pixels: 682x384) and at the full 1920x1080.
    Rays = core + shadow rays traced by the frame. A band of rows of the
    clamped frame in the reference traversal order is compared with the
    oracle bit for bit."""
    import torch

    from rendiation_gb300 import path_tracing as pt
    from rendiation_gb300 import raytracing as rt
    from rendiation_gb300 import task_graph as tg

    lights = [pt.directional_light((3.0, 2.8, 2.5), (0.35, 0.25, -1.0))]
    eye = (0.5, -0.35, 0.55)
    stream = torch.cuda.current_stream()
    out = {}
    for name, (W, H) in (("clamped", pt.clamp_size_by_area(1920, 1080)), ("full_1080p", (1920, 1080))):
        vp = tg.look_at_view_projection_inv(eye, (0.5, 0.5, 0.0), (0, 0, 1), 45.0, W / H, 0.01, 100.0)
        R = pt.DeviceReferencePathTracingRenderer(P, W, H, vp, eye, lights=lights, background_color=(0.4, 0.5, 0.7),
                                                  count_rays=True)
        reps = 20

        def timed(trav, block, sched, tier=0, spec=0):
            R.traversal, R.block_size, R.schedule, R.register_tier, R.speculation = trav, block, sched, tier, spec
            for _ in range(args.warmup):
                R.render()
            R.ray_counts.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(reps):
                R.render()
            e1.record(stream)
            torch.cuda.synchronize()
            c = R.ray_counts.cpu().numpy().view(np.uint32)
            return e0.elapsed_time(e1) / reps, (int(c[0]) / reps, int(c[1]) / reps)

        shapes = {}
        travs = (rt.TRAVERSAL_REFERENCE,) if args.traversal == "reference" else (rt.TRAVERSAL_ORDERED,
                                                                                  rt.TRAVERSAL_ORDERED_WIDE)
        for sched in (pt.SCHEDULE_PIXEL, pt.SCHEDULE_REFILL, pt.SCHEDULE_WAVEFRONT):
            for trav in travs:
                for block in (32, 64, 128):
                    shapes[(trav, block, sched)] = timed(trav, block, sched)[0]
        best = min(shapes, key=shapes.get)
        tiers = {0: shapes[best]}
        if best[2] != pt.SCHEDULE_PIXEL and best[0] != rt.TRAVERSAL_REFERENCE:
            for tier in (1, 2):
                tiers[tier] = timed(*best, tier)[0]
        tier = min(tiers, key=tiers.get)
        specs = {0: tiers[tier]}
        if best[0] != rt.TRAVERSAL_REFERENCE:
            for k in (2, 4, 8, 16):
                specs[k] = timed(*best, tier, k)[0]
        spec = min(specs, key=specs.get)
        ms, (core, shadow) = timed(*best, tier, spec)
        leg = {"size": [W, H], "ms_per_sample": round(ms, 4), "core_rays": core, "shadow_rays": shadow,
               "mrays": round((core + shadow) / ms / 1e3, 1),
               "shape": {"traversal": {0: "binary", 1: "reference", 2: "wide"}[best[0]], "block": best[1],
                         "schedule": ("pixel", "refill", "wavefront")[best[2]], "register_tier": tier,
                         "speculation": spec},
               "shapes_ms": {f"{('pixel', 'refill', 'wavefront')[k[2]]}/{k[0]}/{k[1]}": round(v, 4)
                             for k, v in shapes.items()},
               "register_tiers_ms": {str(k): round(v, 4) for k, v in tiers.items()},
               "speculation_ms": {str(k): round(v, 4) for k, v in specs.items()}}
        # the same sample captured once (rdn_pt_capture) and replayed: it reads and advances a device
        # sample counter, so every replay draws the next sample without host work
        counter = torch.zeros(1, dtype=torch.int32, device="cuda")
        frame = R.capture(counter)
        for _ in range(args.warmup):
            frame()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            frame()
        e1.record(stream)
        torch.cuda.synchronize()
        cms = e0.elapsed_time(e1) / reps
        leg["captured_ms_per_sample"] = round(cms, 4)
        leg["captured_mrays"] = round((core + shadow) / cms / 1e3, 1)
        del frame
        if name == "clamped" and S_field is not None:
            from oracle import orc

            band = (H // 2 - 16, H // 2 + 16)
            R2 = pt.DeviceReferencePathTracingRenderer(P, W, H, vp, eye, lights=lights,
                                                       background_color=(0.4, 0.5, 0.7),
                                                       traversal=rt.TRAVERSAL_REFERENCE, keep_radiance=True)
            R2.render()
            torch.cuda.synchronize()
            img = np.zeros(W * H, np.uint32)
            rad = np.zeros(W * H * 4, np.float32)
            n, sec = orc.pt_render(S_field, vp, eye, W, H, img, lights=lights, bg=(0.4, 0.5, 0.7), rows=band,
                                   radiance=rad, threads=os.cpu_count() or 1)
            g = R2.result().reshape(-1, 4).astype(np.uint32)
            gp = (g[:, 0] | (g[:, 1] << 8) | (g[:, 2] << 16) | (g[:, 3] << 24)).reshape(H, W)[band[0]:band[1]]
            gr = R2.radiance.cpu().numpy().reshape(H, W, 4)[band[0]:band[1]]
            wr = rad.reshape(H, W, 4)[band[0]:band[1]]
            leg["parity_band_rows"] = list(band)
            leg["parity_texels_identical"] = float(np.mean(gp == img.reshape(H, W)[band[0]:band[1]]))
            leg["parity_radiance_bit_identical"] = float(np.mean((gr.view(np.uint32) == wr.view(np.uint32)).all(-1)))
            leg["cpu_mrays"] = round((n[0] + n[1]) / sec / 1e6, 2)
            leg["cpu_threads"] = os.cpu_count() or 1
            leg["cpu_sample"] = f"rows {band[0]}..{band[1]} of the {W}x{H} frame (oracle, reference order)"
        out[name] = leg
    st, flags = P.check_errors()
    assert st == 0 and flags == 0
    out["workload"] = ("heightfield 1024^2 (2093058 tris), reference path tracer: max_path_depth 3, one "
                       "directional light with a shadow ray per hit, default physical material (Lambertian + "
                       "GGX), ACES tone map, running RGBA8 average; rays = core + shadow")
    return out


def bench_task_graph(args, P):
    """Throughput of the device task graph alone (no tracing): one million root
    tasks of a chain future that spawns and awaits a child in group 1 (which
    spawns and awaits one in group 2), then one more in group 2 - four tasks
    per root, each spawned, polled, woken and cleaned up by the executor. One
    dispatch plus its device-ended round loop, captured once and replayed."""
    import torch

    from rendiation_gb300 import task_graph as tg

    roots = 1_000_000
    src = tg.DeviceTaskGraphBuildSource(capacity=roots)
    src.define_task(tg.BaseShaderFuture().then_spawn_task(1).then_spawn_task(2).map(), 1)
    src.define_task(tg.BaseShaderFuture().then_spawn_task(2).map(), 1)
    src.define_task(tg.BaseShaderFuture(), 1)
    exe = src.build(P)
    launch = exe.capture_until_empty(roots, 0, max_rounds=64)
    for _ in range(args.warmup):
        launch()
    torch.cuda.synchronize()
    assert exe.read_back_execution_states().is_empty() and exe.check_errors() == 0
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 10
    e0.record(stream)
    for _ in range(reps):
        launch()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    tasks = 4 * roots
    # the same work as plain launches: dispatch, then the number of rounds that
    # drains the graph (counted once from the host), issued by execute(rounds)
    exe.dispatch_allocate_init_task(roots, 0)
    rounds = 0
    while not exe.read_back_execution_states().is_empty():
        exe.execute(1)
        rounds += 1
    for _ in range(args.warmup):
        exe.dispatch_allocate_init_task(roots, 0)
        exe.execute(rounds)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        exe.dispatch_allocate_init_task(roots, 0)
        exe.execute(rounds)
    e1.record(stream)
    torch.cuda.synchronize()
    assert exe.read_back_execution_states().is_empty() and exe.check_errors() == 0
    plain_ms = e0.elapsed_time(e1) / reps
    exe.close()
    return {"workload": "1,000,000 roots x 4 tasks (chain futures over 3 groups), dispatch + device-ended round loop",
            "ms": round(ms, 3), "mtasks_per_s": round(tasks / ms / 1e3, 1), "rounds": rounds,
            "plain_launches_ms": round(plain_ms, 3), "plain_launches_mtasks_per_s": round(tasks / plain_ms / 1e3, 1)}


def bench_batched(args, ws=1, rank=0):
    """Batched multi-scene paths: 256 soups (log-uniform 1k..200k triangles),
    log-uniform 4k..256k rays per scene, <= 4 diffuse bounces with Russian
    roulette from bounce 2. One persistent launch per bounce for all scenes,
    captured in a CUDA graph, against the plain per-scene launch loop (the same
    executor called once per scene)."""
    import ctypes as C

    import torch

    from rendiation_gb300 import native
    from rendiation_gb300 import raytracing as rt
    from rendiation_gb300 import scenes

    b = scenes.batched_soups(n_scenes=args.scenes)
    if ws > 1:  # each GPU takes a share of the scenes balanced by triangles x rays
        from rendiation_gb300 import partition

        costs = partition.scene_costs([m.triangle_count for m in b.meshes], np.diff(b.ray_offsets))
        b = partition.batch_subset(b, partition.balanced_scenes(costs, ws)[rank])
    P = rt.AccelerationStructureSystem(device=0)
    for m in b.meshes:
        P.create_bottom_level_acceleration_structure([rt.BottomLevelAccelerationStructureBuildSource(m.positions)])
    handles = [P.create_top_level_acceleration_structure([rt.TopLevelAccelerationStructureSourceInstance(s)])
               for s in range(len(b.meshes))]
    P.bind_tlas(handles)
    build = compare_builds(P)
    build_s = build["host_s"]
    rays = torch.from_numpy(b.rays.view(np.float32).reshape(-1, 8).copy()).cuda()
    tidx = torch.from_numpy(b.tlas_idx.astype(np.int32)).cuda()
    traversal = {"reference": rt.TRAVERSAL_REFERENCE, "wide": rt.TRAVERSAL_ORDERED_WIDE}.get(
        args.traversal, rt.TRAVERSAL_ORDERED)
    stream = torch.cuda.current_stream()

    batched = rt.Paths(P, rays, tidx, max_bounces=4, rr_start=2, seed=1, traversal=traversal)
    tuned = None
    if args.tune and args.traversal == "ordered":
        from rendiation_gb300.autotune import Autotuner, grid

        orders = [rt.TRAVERSAL_ORDERED, rt.TRAVERSAL_ORDERED_WIDE]
        cands = (grid(traversal=orders, block=[64, 128], sort_key=[rt.SORT_NONE], refill=[0], local=[0, 1])
                 + grid(traversal=orders, block=[64], sort_key=[rt.SORT_SCENE_OCTANT], refill=[0], local=[0, 1])
                 + grid(traversal=orders, block=[64], sort_key=[rt.SORT_NONE], refill=[8, 16], local=[0]))

        def run(c):
            batched.configure(c["traversal"], c["block"], c["sort_key"], c["refill"], c["local"])
            batched.run()

        res = Autotuner().tune("batched-paths", cands, run, reps=2)
        best = dict(res.best)

        def run_spec(c):
            batched.configure(speculation=c["spec"])
            batched.run()

        batched.configure(best["traversal"], best["block"], best["sort_key"], best["refill"], best["local"])
        res2 = Autotuner().tune("batched-paths-speculation", [dict(best, spec=k) for k in (0, 2, 4, 8)], run_spec,
                                reps=2)
        batched.configure(speculation=res2.best["spec"])
        res.best, res.timings_ms = res2.best, res.timings_ms + res2.timings_ms
        tuned = {"best": res.best, "timings_ms": res.timings_ms}
    batched.capture()
    for _ in range(args.warmup):
        batched.launch_graph()
    torch.cuda.synchronize()
    segs = batched.segments()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = max(3, args.batched_steps)
    e0.record(stream)
    for _ in range(reps):
        batched.launch_graph()
    e1.record(stream)
    torch.cuda.synchronize()
    batched_ms = e0.elapsed_time(e1) / reps
    res_batched = batched.results()

    # plain per-scene loop: the same executor, one scene per call, with the
    # launch knobs the batched graph was tuned to (node width, block, stack
    # placement, leaf postponement, secondary schedule, sort key)
    L = native.lib()
    max_n = int(np.max(np.diff(b.ray_offsets)))
    knobs = batched.desc
    size = C.c_size_t()
    L.rdn_paths_scratch_size(max_n, 4, knobs.sort_key, C.byref(size))
    scratch = torch.empty(size.value + 256, dtype=torch.uint8, device="cuda")
    sptr = (scratch.data_ptr() + 255) & ~255
    out = torch.empty((b.rays.shape[0], 2), dtype=torch.float32, device="cuda")
    desc = native.PathDesc()
    desc.max_bounces, desc.rr_start, desc.albedo, desc.rr_survive, desc.seed = 4, 2, 0.5, 0.5, 1
    desc.traversal, desc.scratch, desc.scratch_bytes = knobs.traversal, sptr, size.value
    desc.block_size, desc.sort_key, desc.refill = knobs.block_size, knobs.sort_key, knobs.refill
    desc.local_stack, desc.speculation = knobs.local_stack, knobs.speculation
    plain_knobs = {"traversal": int(desc.traversal), "block": int(desc.block_size), "sort_key": int(desc.sort_key),
                   "refill": int(desc.refill), "local": int(desc.local_stack), "spec": int(desc.speculation)}

    def plain_loop():
        for sidx in range(len(b.meshes)):
            o0, o1 = int(b.ray_offsets[sidx]), int(b.ray_offsets[sidx + 1])
            desc.rays = rays.data_ptr() + o0 * 32
            desc.tlas_idx = None
            desc.count = o1 - o0
            desc.tlas_uniform = sidx
            desc.out = out.data_ptr() + o0 * 8
            st = L.rdn_trace_paths(P._h, C.byref(desc), C.c_void_p(stream.cuda_stream))
            if st != native.RDN_OK:
                raise native.RdnError(st, L.rdn_last_error(P._h).decode())

    plain_loop()
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        plain_loop()
    e1.record(stream)
    torch.cuda.synchronize()
    plain_ms = e0.elapsed_time(e1) / reps
    # per-scene seeds equal the batched ones only when ids match: compare statistics, not records
    total = int(sum(segs))
    # roofline estimate: the primaries' reference-order fetches per ray (the
    # path executor records no bounce rays), applied to every segment
    h4 = torch.empty((rays.shape[0], 4), device="cuda")
    c_prim = P.trace_counted(rays, h4, tlas_idx=tidx, traversal=rt.TRAVERSAL_REFERENCE)
    b_prim = node_bytes_per_ray(c_prim, rays.shape[0])
    del h4
    if ws > 1:  # whole-job figures: segments of every rank's scenes over the slowest rank
        total = sum_over_ranks(total, ws)
        batched_ms = max_over_ranks(batched_ms / 1e3, ws, "cuda") * 1e3
        plain_ms = max_over_ranks(plain_ms / 1e3, ws, "cuda") * 1e3
    return {
        "ranks": ws,
        "workload": f"{len(b.meshes)} soups, {sum(m.triangle_count for m in b.meshes)} tris, "
                    f"{b.rays.shape[0]} primaries, <=4 bounces, roulette p=0.5 from bounce 2",
        "segments_per_step": total,
        "segments_per_bounce": segs,
        "batched_graph_mrays": round(total / (batched_ms / 1e3) / 1e6, 2),
        "batched_ms": round(batched_ms, 3),
        "plain_loop_mrays": round(total / (plain_ms / 1e3) / 1e6, 2),
        "plain_loop_ms": round(plain_ms, 3),
        "speedup_vs_plain_loop": round(plain_ms / batched_ms, 3),
        "roofline": {"batched_graph": algorithmic_roofline(
            total * b_prim, batched_ms, "estimate: every segment costed at the primaries' mean reference-order fetches "
            f"({b_prim:.0f} B per ray)")},
        "plain_loop_knobs": plain_knobs,
        "build": build,
        "escaped_fraction": round(float(np.mean(res_batched["depth_flags"] >> 31)), 4),
        "autotuned": tuned,
    }


def bench_adjoint(args, ws=1, rank=0):
    """Differentiable closest hit: heightfield 256^2 (130,050 tris) with a
    per-vertex attribute uniform in [0,1], 512x512 primary rays, loss =
    sum (interpolated attribute - target)^2 with the target rendered from a
    copy whose heights are jittered by N(0, 0.005). Forward alone against
    forward + adjoint, the adjoint differentiating the hits the forward
    recorded (and, for comparison, tracing them again)."""
    import ctypes as C

    import torch

    from rendiation_gb300 import native
    from rendiation_gb300 import raytracing as rt
    from rendiation_gb300 import scenes

    n_grid, res = 256, 512
    L = native.lib()
    mesh = scenes.heightfield(n_grid, seed=1)
    jit = scenes.heightfield(n_grid, seed=1, jitter_sigma=0.005, jitter_seed=4242)
    rng = np.random.Generator(np.random.PCG64(17))
    attr = torch.from_numpy(rng.random(mesh.positions.shape[0]).astype(np.float32)).cuda()
    cam = scenes.PinholeCamera.look_at((0.5, -0.5, 0.8), (0.5, 0.5, 0.0), 20.0, res, res)
    rays_np = scenes.pinhole_rays(cam)
    if ws > 1:  # each GPU takes a row band of the rays; vertex gradients are summed across GPUs
        from rendiation_gb300.partition import row_bands

        r0, r1 = row_bands(res, ws)[rank]
        rays_np = np.ascontiguousarray(rays_np[r0 * res:r1 * res])
    rays = torch.from_numpy(rays_np.view(np.float32).reshape(-1, 8).copy()).cuda()
    n = rays_np.shape[0]
    traversal = {"reference": rt.TRAVERSAL_REFERENCE, "wide": rt.TRAVERSAL_ORDERED_WIDE}.get(
        args.traversal, rt.TRAVERSAL_ORDERED)

    def system(m):
        P = rt.AccelerationStructureSystem(device=0)
        b = P.create_bottom_level_acceleration_structure([rt.BottomLevelAccelerationStructureBuildSource(
            m.positions, m.indices)])
        P.bind_tlas([P.create_top_level_acceleration_structure([rt.TopLevelAccelerationStructureSourceInstance(b)])])
        P.build(blas_bin_size=4, device_build=True)
        return P

    Pt = system(jit)
    target = torch.zeros(n, device="cuda")
    d = native.AttrLossDesc(rays.data_ptr(), n, 0, attr.data_ptr(), None, target.data_ptr(), None, None, None, None,
                            None, 1.0, traversal, 0, 0)
    assert L.rdn_attr_loss_forward(Pt._h, C.byref(d), None) == 0
    torch.cuda.synchronize()
    Pt.close()
    P = system(mesh)
    loss = torch.zeros(1, dtype=torch.float64, device="cuda")
    grad = torch.zeros((mesh.positions.shape[0], 4), device="cuda")
    hit_tri = torch.zeros(n, dtype=torch.int32, device="cuda")
    hit_inst = torch.zeros(n, dtype=torch.int32, device="cuda")
    fwd = native.AttrLossDesc(rays.data_ptr(), n, 0, attr.data_ptr(), target.data_ptr(), None, None,
                              loss.data_ptr(), None, None, None, 1.0, traversal, 0, 0)
    fwd_rec = native.AttrLossDesc(rays.data_ptr(), n, 0, attr.data_ptr(), target.data_ptr(), None, None,
                                  loss.data_ptr(), None, None, None, 1.0, traversal, 0, 0, hit_tri.data_ptr(),
                                  hit_inst.data_ptr())
    adj = native.AttrLossDesc(rays.data_ptr(), n, 0, attr.data_ptr(), target.data_ptr(), None, None, None,
                              grad.data_ptr(), None, None, 1.0, traversal, 0, 0)
    adj_rec = native.AttrLossDesc(rays.data_ptr(), n, 0, attr.data_ptr(), target.data_ptr(), None, None, None,
                                  grad.data_ptr(), None, None, 1.0, traversal, 0, 1, hit_tri.data_ptr(),
                                  hit_inst.data_ptr())
    stream = torch.cuda.current_stream()
    sp = C.c_void_p(stream.cuda_stream)

    # traversal stacks in shared or local memory: the faster forward decides
    def fwd_ms(ls, sp_, reps=20):
        fwd.local_stack, fwd.speculation = ls, sp_
        for _ in range(3):
            assert L.rdn_attr_loss_forward(P._h, C.byref(fwd), sp) == 0
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            assert L.rdn_attr_loss_forward(P._h, C.byref(fwd), sp) == 0
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    stack_ms = {(ls, sp_): fwd_ms(ls, sp_) for ls in (0, 1) for sp_ in (0, 4)}
    local, spec = min(stack_ms, key=stack_ms.get)
    for dsc in (fwd, fwd_rec, adj, adj_rec):
        dsc.local_stack, dsc.speculation = local, spec

    def run(mode):
        loss.zero_()
        assert L.rdn_attr_loss_forward(P._h, C.byref(fwd_rec if mode == "tape" else fwd), sp) == 0
        if mode != "forward":
            grad.zero_()
            assert L.rdn_attr_loss_adjoint(P._h, C.byref(adj_rec if mode == "tape" else adj), sp) == 0
            if ws > 1:
                from rendiation_gb300.partition import sum_gradients

                sum_gradients(grad)  # one all-reduce after the backward

    out = {}
    for name, w in (("forward", "forward"), ("forward_adjoint", "tape"), ("forward_adjoint_retrace", "retrace")):
        for _ in range(args.warmup):
            run(w)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        reps = 50
        e0.record(stream)
        for _ in range(reps):
            run(w)
        e1.record(stream)
        torch.cuda.synchronize()
        out[name + "_ms"] = round(e0.elapsed_time(e1) / reps, 4)
        out[name + "_mrays"] = round(n / (e0.elapsed_time(e1) / reps / 1e3) / 1e6, 2)
    out["fwd_adjoint_over_fwd"] = round(out["forward_adjoint_ms"] / out["forward_ms"], 3)
    out["fwd_adjoint_retrace_over_fwd"] = round(out["forward_adjoint_retrace_ms"] / out["forward_ms"], 3)
    out["adjoint"] = "from the forward's recorded hits (8 B per ray); _retrace: hits traced again"
    # gradient error at this configuration: one forward (recording the hits) and one adjoint
    loss.zero_()
    grad.zero_()
    assert L.rdn_attr_loss_forward(P._h, C.byref(fwd_rec), sp) == 0
    assert L.rdn_attr_loss_adjoint(P._h, C.byref(adj_rec), sp) == 0
    torch.cuda.synchronize()
    # roofline: the reference order's fetches for these rays; the adjoint adds
    # the 48 B float4 atomic scatter to three corners per hit
    hits4 = torch.empty((n, 4), device="cuda")
    c_ref = P.trace_counted(rays, hits4, traversal=rt.TRAVERSAL_REFERENCE)
    b_ray = node_bytes_per_ray(c_ref, n) + 4.0  # + the attribute read
    n_hit = int((hit_tri.cpu().numpy().view(np.uint32) != 0xFFFFFFFF).sum())
    out["roofline"] = {
        "forward": algorithmic_roofline(n * b_ray, out["forward_ms"],
                                        "per ray 32 + 16 + 48 x node visits + 36 x triangle tests of the reference "
                                        "order, + 4 B attribute"),
        "forward_adjoint_retrace": algorithmic_roofline(2 * n * b_ray + 48.0 * n_hit, out["forward_adjoint_retrace_ms"],
                                                        "forward twice (the adjoint traces again) + 48 B of atomic "
                                                        "scatter per hit"),
        "bytes_per_ray": round(b_ray, 1),
    }
    if ws == 1:  # (with several GPUs the gradient is the sum over every rank's rays)
        out["gradient_error"] = attr_loss_gradient_error(
            mesh, attr.cpu().numpy(), rays_np, target.cpu().numpy(), hit_tri.cpu().numpy().view(np.uint32),
            grad.cpu().numpy())
    out["local_stack"], out["speculation"] = local, spec
    out["loss"] = float(loss.item())
    out["workload"] = f"heightfield {n_grid}^2 ({mesh.triangle_count} tris), {res}x{res} rays, attribute loss"
    P.close()
    return out


def attr_loss_gradient_error(mesh, attr, rays, targets, tri, grad, n_vertices=64, seed=23):
    """Gradient error of the attribute loss at frozen visibility against FP64:
    (1) the FP64 analytic gradient over every vertex some ray sees; (2) FP64
    central differences on `n_vertices` random seen vertices (positions and
    attribute), plain with h = 1e-4 as the configuration states, and
    Richardson-extrapolated from h and h/2; (3) for every vertex whose plain
    h = 1e-4 difference is off by more than 1e-3, the central difference at
    h = 1e-4 .. 1e-7, showing it converge to the kernel's gradient (grazing rays
    make u, v strongly nonlinear in the vertex positions, so the truncation
    error of the h = 1e-4 difference is what disagrees)."""
    idx = mesh.indices.reshape(-1, 3)
    hit = tri != 0xFFFFFFFF
    r = rays[hit]
    tv = idx[tri[hit]]
    tg = targets[hit].astype(np.float64)
    pos = mesh.positions.astype(np.float64)
    a = attr.astype(np.float64)
    o = r["org"].astype(np.float64)
    d = r["dir"].astype(np.float64)

    def solve(p_, sel):
        v = p_[tv[sel]]
        M = np.stack([-d[sel], v[:, 1] - v[:, 0], v[:, 2] - v[:, 0]], axis=2)
        x = np.linalg.solve(M, (o[sel] - v[:, 0])[..., None])[..., 0]
        return x, M

    def loss(p_, a_, sel):
        x, _ = solve(p_, sel)
        u, v = x[:, 1], x[:, 2]
        t = tv[sel]
        val = (1 - u - v) * a_[t[:, 0]] + u * a_[t[:, 1]] + v * a_[t[:, 2]]
        return float(np.sum((val - tg[sel]) ** 2))

    allr = np.arange(r.shape[0])
    x, M = solve(pos, allr)
    u, v = x[:, 1], x[:, 2]
    val = (1 - u - v) * a[tv[:, 0]] + u * a[tv[:, 1]] + v * a[tv[:, 2]]
    res = 2 * (val - tg)
    G = np.stack([np.zeros_like(res), res * (a[tv[:, 1]] - a[tv[:, 0]]), res * (a[tv[:, 2]] - a[tv[:, 0]])], 1)
    lam = np.linalg.solve(np.transpose(M, (0, 2, 1)), G[..., None])[..., 0]
    ga, gp = np.zeros(a.shape[0]), np.zeros((a.shape[0], 3))
    for k, wk in enumerate([1 - u - v, u, v]):
        np.add.at(ga, tv[:, k], res * wk)
        np.add.at(gp, tv[:, k], -wk[:, None] * lam)
    g_pos, g_attr = grad[:, :3].astype(np.float64), grad[:, 3].astype(np.float64)
    seen = np.unique(tv.reshape(-1))
    norm_p = np.linalg.norm(gp[seen], axis=1)
    floor_p = 1e-2 * np.median(norm_p[norm_p > 0])
    floor_a = 1e-2 * np.median(np.abs(ga[seen][ga[seen] != 0]))
    rel_p = np.linalg.norm(g_pos[seen] - gp[seen], axis=1) / np.maximum(norm_p, floor_p)
    rel_a = np.abs(g_attr[seen] - ga[seen]) / np.maximum(np.abs(ga[seen]), floor_a)

    rng = np.random.default_rng(seed)
    pick = rng.choice(seen, size=min(n_vertices, seen.size), replace=False)

    def central(vi, c, hh, sel):
        if c < 3:
            pp, pm = pos.copy(), pos.copy()
            pp[vi, c] += hh
            pm[vi, c] -= hh
            return (loss(pp, a, sel) - loss(pm, a, sel)) / (2 * hh)
        ap, am = a.copy(), a.copy()
        ap[vi] += hh
        am[vi] -= hh
        return (loss(pos, ap, sel) - loss(pos, am, sel)) / (2 * hh)

    plain, rich, conv = [], [], []
    for vi in pick:
        sel = np.nonzero(np.any(tv == vi, axis=1))[0]
        got = np.array([*g_pos[vi], g_attr[vi]])
        fd1 = np.array([central(vi, c, 1e-4, sel) for c in range(4)])
        fd2 = np.array([central(vi, c, 5e-5, sel) for c in range(4)])
        ri = (4 * fd2 - fd1) / 3
        den = max(np.linalg.norm(ri[:3]), floor_p)
        e_plain = np.linalg.norm(got[:3] - fd1[:3]) / den
        e_rich = np.linalg.norm(got[:3] - ri[:3]) / den
        e_attr = abs(got[3] - ri[3]) / max(abs(ri[3]), floor_a)
        plain.append(float(e_plain))
        rich.append(float(max(e_rich, e_attr)))
        if e_plain > 1e-3:
            series = {}
            for hh in (1e-4, 1e-5, 1e-6, 1e-7):
                f = np.array([central(vi, c, hh, sel) for c in range(3)])
                series[f"{hh:.0e}"] = float(np.linalg.norm(got[:3] - f) / den)
            conv.append({"vertex": int(vi), "rays": int(sel.size), "rel_error_by_h": series})
    return {
        "vertices_seen": int(seen.size),
        "max_rel_vs_fp64_analytic_positions": float(rel_p.max()),
        "max_rel_vs_fp64_analytic_attributes": float(rel_a.max()),
        "fd_vertices": int(len(pick)),
        "max_rel_vs_fp64_fd_h1e-4": float(max(plain)),
        "median_rel_vs_fp64_fd_h1e-4": float(np.median(plain)),
        "vertices_within_1e-3_of_fd_h1e-4": int(sum(e <= 1e-3 for e in plain)),
        "max_rel_vs_fp64_fd_richardson": float(max(rich)),
        "fd_convergence_of_vertices_over_1e-3": conv,
    }


def bench_batched_adjoint(args, ws=1, rank=0):
    """Batched differentiable paths: 64 heightfields with vertex grids
    log-uniform in [64^2, 512^2] (octaves seeded per scene), each with a
    per-vertex attribute and 64k..1M primary rays (log-uniform) plus 2 diffuse
    bounces; targets are the same paths' values on copies with heights jittered
    by N(0, 0.005). Forward + adjoint of all scenes in one captured CUDA graph,
    the adjoint differentiating the segments the forward recorded (and, for
    comparison, tracing the paths again). Gradient error per scene against FP64 on a
    sample of 2048 paths per scene (analytic FP64 gradient over the sample, and
    FP64 central differences, h = 1e-4 with Richardson extrapolation, on 2
    vertices per scene)."""
    import ctypes as C

    import torch

    from rendiation_gb300 import native
    from rendiation_gb300 import raytracing as rt
    from rendiation_gb300 import scenes

    L = native.lib()
    n_scenes, seg = args.diff_scenes, 3
    grids = np.sqrt(scenes.log_uniform_ints(n_scenes, 64 * 64, 512 * 512, 31)).astype(np.int64)
    nrays = scenes.log_uniform_ints(n_scenes, 64_000, 1_000_000, 32)
    ids = list(range(n_scenes))
    if ws > 1:  # each GPU takes a share of the scenes balanced by triangles x rays
        from rendiation_gb300 import partition

        ids = partition.balanced_scenes(partition.scene_costs(2 * (grids - 1) ** 2, nrays), ws)[rank]
    meshes = [scenes.heightfield(int(grids[k]), seed=100 + k) for k in ids]
    jitter = [scenes.heightfield(int(grids[k]), seed=100 + k, jitter_sigma=0.005, jitter_seed=7000 + k) for k in ids]
    grids, nrays, n_scenes = grids[ids], nrays[ids], len(ids)

    def system(ms):
        P = rt.AccelerationStructureSystem(device=0)
        for m in ms:
            P.create_bottom_level_acceleration_structure([rt.BottomLevelAccelerationStructureBuildSource(
                m.positions, m.indices)])
        P.bind_tlas([P.create_top_level_acceleration_structure([rt.TopLevelAccelerationStructureSourceInstance(s)])
                     for s in range(len(ms))])
        P.build(blas_bin_size=4, device_build=True)
        return P

    rays, tidx = [], []
    for k in range(n_scenes):
        w = int(np.sqrt(nrays[k] * 16 / 9))
        h = max(1, int(nrays[k]) // w)
        cam = scenes.PinholeCamera.look_at((0.5, -0.5, 0.8), (0.5, 0.5, 0.0), 20.0, w, h)
        r = scenes.pinhole_rays(cam)
        rays.append(r)
        tidx.append(np.full(r.shape[0], k, np.uint32))
    rays = np.concatenate(rays)
    tidx = np.concatenate(tidx)
    n = rays.shape[0]
    nv = sum(m.positions.shape[0] for m in meshes)
    attr = torch.from_numpy(np.random.Generator(np.random.PCG64(33)).random(nv).astype(np.float32)).cuda()
    d_rays = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).cuda()
    d_tidx = torch.from_numpy(tidx.astype(np.int32)).cuda()
    torch.cuda.reset_peak_memory_stats()

    def desc(**kw):
        d = native.AttrPathDesc()
        d.rays, d.tlas_idx, d.count, d.segments, d.seed, d.grad_scale = d_rays.data_ptr(), d_tidx.data_ptr(), n, seg, 5, 1.0
        d.attributes = attr.data_ptr()
        for k, v in kw.items():
            setattr(d, k, v)
        return d

    Pj = system(jitter)
    targets = torch.zeros(n * seg, device="cuda")
    assert L.rdn_attr_paths_forward(Pj._h, C.byref(desc(values=targets.data_ptr())), None) == 0
    torch.cuda.synchronize()
    Pj.close()
    P = system(meshes)
    as_bytes = P.device_bytes()
    loss = torch.zeros(1, dtype=torch.float64, device="cuda")
    grad = torch.zeros((nv, 4), device="cuda")
    # device memory of the configuration's own form (hits recomputed in the backward, no tape)
    peak_recompute = int(torch.cuda.max_memory_allocated() + as_bytes)
    # the forward's record of every segment (triangle, instance, ray): 40 B per segment
    tape_tri = torch.zeros(n * seg, dtype=torch.int32, device="cuda")
    tape_inst = torch.zeros(n * seg, dtype=torch.int32, device="cuda")
    tape_rays = torch.zeros((n * seg, 8), device="cuda")
    tape = dict(seg_tri=tape_tri.data_ptr(), seg_inst=tape_inst.data_ptr(), seg_rays=tape_rays.data_ptr())
    stream = torch.cuda.current_stream()
    sp = C.c_void_p(stream.cuda_stream)

    def graph_ms(dsc, reps=3):
        h = C.c_void_p()
        assert L.rdn_attr_paths_graph(P._h, C.byref(dsc), nv, C.byref(h)) == 0
        L.rdn_graph_launch(h, sp)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            L.rdn_graph_launch(h, sp)
        e1.record(stream)
        torch.cuda.synchronize()
        L.rdn_graph_destroy(h)
        return e0.elapsed_time(e1) / reps

    # traversal stacks in shared or local memory and the leaf-postponement
    # threshold: the faster forward decides
    stack_ms = {(ls, sp_): graph_ms(desc(targets=targets.data_ptr(), loss_sum=loss.data_ptr(), local_stack=ls,
                                         speculation=sp_))
                for ls in (0, 1) for sp_ in (0, 4)}
    local, spec = min(stack_ms, key=stack_ms.get)
    knobs = dict(local_stack=local, speculation=spec)
    both = desc(targets=targets.data_ptr(), loss_sum=loss.data_ptr(), grad_vertices=grad.data_ptr(), from_record=1,
                **knobs, **tape)
    retrace = desc(targets=targets.data_ptr(), loss_sum=loss.data_ptr(), grad_vertices=grad.data_ptr(), **knobs)
    fwd = desc(targets=targets.data_ptr(), loss_sum=loss.data_ptr(), **knobs)
    g = C.c_void_p()
    assert L.rdn_attr_paths_graph(P._h, C.byref(both), nv, C.byref(g)) == 0
    gr = C.c_void_p()
    assert L.rdn_attr_paths_graph(P._h, C.byref(retrace), nv, C.byref(gr)) == 0
    gf = C.c_void_p()
    assert L.rdn_attr_paths_graph(P._h, C.byref(fwd), nv, C.byref(gf)) == 0
    out = {"local_stack": local, "speculation": spec,
           "forward_ms_by_knobs": {f"{'local' if k[0] else 'shared'}/spec{k[1]}": round(v, 3)
                                   for k, v in stack_ms.items()}}
    for name, handle in (("forward", gf), ("forward_adjoint", g), ("forward_adjoint_retrace", gr)):
        for _ in range(args.warmup):
            L.rdn_graph_launch(handle, sp)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(5):
            L.rdn_graph_launch(handle, sp)
        e1.record(stream)
        torch.cuda.synchronize()
        out[name + "_ms"] = round(e0.elapsed_time(e1) / 5, 3)
    L.rdn_graph_destroy(g)
    L.rdn_graph_destroy(gr)
    L.rdn_graph_destroy(gf)
    del tape_tri, tape_inst, tape_rays
    # device memory of the timed forms (before the counting below allocates its own buffers)
    peak_timed = int(torch.cuda.max_memory_allocated() + as_bytes)
    # segments traced per step (one forward pass records the segment triangles)
    seg_tri = torch.zeros(n * seg, dtype=torch.int32, device="cuda")
    seg_rays = torch.zeros((n * seg, 8), device="cuda")
    assert L.rdn_attr_paths_forward(P._h, C.byref(desc(seg_tri=seg_tri.data_ptr(), seg_rays=seg_rays.data_ptr())),
                                    None) == 0
    torch.cuda.synchronize()
    tri_all = seg_tri.cpu().numpy().view(np.uint32).reshape(-1, seg)
    # a segment is traced when every earlier one hit
    traced = int(n + np.sum(tri_all[:, 0] != 0xFFFFFFFF) + np.sum((tri_all[:, 0] != 0xFFFFFFFF) & (tri_all[:, 1] != 0xFFFFFFFF)))
    out["segments_per_step"] = traced
    # roofline: the reference order's fetches for every traced segment ray
    live = np.ones((n, seg), bool)
    live[:, 1] = tri_all[:, 0] != 0xFFFFFFFF
    live[:, 2] = live[:, 1] & (tri_all[:, 1] != 0xFFFFFFFF)
    sel = torch.from_numpy(np.nonzero(live.reshape(-1))[0]).cuda()
    s_rays = seg_rays[sel].contiguous()
    s_tidx = d_tidx.repeat_interleave(seg)[sel].contiguous()
    h4 = torch.empty((s_rays.shape[0], 4), device="cuda")
    c_seg = P.trace_counted(s_rays, h4, tlas_idx=s_tidx, traversal=rt.TRAVERSAL_REFERENCE)
    b_seg = node_bytes_per_ray(c_seg, s_rays.shape[0]) + 4.0
    del seg_rays, s_rays, h4
    out["forward_mrays"] = round(traced / (out["forward_ms"] / 1e3) / 1e6, 2)
    out["forward_adjoint_mrays"] = round(traced / (out["forward_adjoint_ms"] / 1e3) / 1e6, 2)
    out["fwd_adjoint_over_fwd"] = round(out["forward_adjoint_ms"] / out["forward_ms"], 3)
    out["forward_adjoint_retrace_mrays"] = round(traced / (out["forward_adjoint_retrace_ms"] / 1e3) / 1e6, 2)
    out["fwd_adjoint_retrace_over_fwd"] = round(out["forward_adjoint_retrace_ms"] / out["forward_ms"], 3)
    out["adjoint"] = ("from the forward's record of every segment (triangle, instance, ray; 40 B per segment), "
                      "one graph for forward + adjoint; _retrace: the adjoint traces the paths again")
    out["peak_hbm_bytes"] = peak_timed
    # the configuration asks for hits recomputed in the backward pass, not stored per bounce
    out["roofline"] = {
        "forward": algorithmic_roofline(traced * b_seg, out["forward_ms"],
                                        "per traced segment the reference order's fetches (counted on the recorded "
                                        "segment rays) + 4 B attribute"),
        "forward_adjoint_retrace": algorithmic_roofline(2 * traced * b_seg + 48.0 * traced,
                                                        out["forward_adjoint_retrace_ms"],
                                                        "forward twice + 48 B of atomic scatter per segment"),
        "bytes_per_segment": round(b_seg, 1),
    }
    out["config_conforming"] = {
        "form": "hits recomputed by tracing the paths again in the adjoint (no tape)",
        "fwd_adjoint_over_fwd": out["fwd_adjoint_retrace_over_fwd"],
        "forward_adjoint_mrays": out["forward_adjoint_retrace_mrays"],
        "peak_hbm_bytes": peak_recompute,
    }
    out["workload"] = (f"{n_scenes} heightfields {int(grids.min())}^2..{int(grids.max())}^2 "
                       f"({sum(m.triangle_count for m in meshes)} tris), {n} primaries, 2 bounces")
    out["gradient_error"] = batched_gradient_error(P, meshes, rays, tidx, attr, targets, seg)
    P.close()
    return out


def batched_gradient_error(P, meshes, rays, tidx, attr, targets, seg, sample=2048):
    """Per scene: the kernel gradient of a loss over `sample` paths against FP64
    (analytic over every vertex, central differences on 2 random vertices)."""
    import ctypes as C

    import torch

    from rendiation_gb300 import native

    L = native.lib()
    pos = np.concatenate([m.positions for m in meshes]).astype(np.float64)
    offs = np.cumsum([0] + [m.positions.shape[0] for m in meshes])
    idx = np.concatenate([m.indices + offs[k] for k, m in enumerate(meshes)]).astype(np.int64)
    a = attr.cpu().numpy().astype(np.float64)
    tg_all = targets.cpu().numpy().reshape(-1, seg)
    worst_analytic, worst_fd, worst_fd_plain, worst_unc = [], [], [], []
    p99_analytic, worst_cond, worst_off_edge, edge_hits = [], [], [], []
    worst_detail = {}
    rng = np.random.default_rng(8)
    for s in range(len(meshes)):
        sel = np.nonzero(tidx == s)[0]
        sel = sel[rng.choice(sel.shape[0], min(sample, sel.shape[0]), replace=False)]
        sr = np.ascontiguousarray(rays[sel])
        m = sr.shape[0]
        d_r = torch.from_numpy(sr.view(np.float32).reshape(-1, 8).copy()).cuda()
        d_t = torch.from_numpy(tidx[sel].astype(np.int32)).cuda()
        d_tg = torch.from_numpy(np.ascontiguousarray(tg_all[sel]).reshape(-1)).cuda()
        seg_tri = torch.zeros(m * seg, dtype=torch.int32, device="cuda")
        seg_rays = torch.zeros((m * seg, 8), device="cuda")
        grad = torch.zeros((pos.shape[0], 4), device="cuda")
        d = native.AttrPathDesc()
        d.rays, d.tlas_idx, d.count, d.segments, d.seed, d.grad_scale = d_r.data_ptr(), d_t.data_ptr(), m, seg, 5, 1.0
        d.attributes, d.targets = attr.data_ptr(), d_tg.data_ptr()
        d.seg_tri, d.seg_rays = seg_tri.data_ptr(), seg_rays.data_ptr()
        seg_inst = torch.zeros(m * seg, dtype=torch.int32, device="cuda")
        seg_val = torch.zeros(m * seg, device="cuda")
        d.seg_inst, d.values = seg_inst.data_ptr(), seg_val.data_ptr()
        assert L.rdn_attr_paths_forward(P._h, C.byref(d), None) == 0
        d.grad_vertices, d.from_record = grad.data_ptr(), 1
        assert L.rdn_attr_paths_adjoint(P._h, C.byref(d), None) == 0
        torch.cuda.synchronize()
        tri = seg_tri.cpu().numpy().view(np.uint32)
        alive = tri != 0xFFFFFFFF
        seg_vals = seg_val.cpu().numpy().astype(np.float64)
        rr = seg_rays.cpu().numpy().reshape(-1, 8)[alive].astype(np.float64)
        t_ = tri[alive].astype(np.int64)
        tg = d_tg.cpu().numpy().astype(np.float64)[alive]
        tv = idx.reshape(-1, 3)[t_]
        dd = rr[:, 4:7] / np.linalg.norm(rr[:, 4:7], axis=1, keepdims=True)

        def bary(P64):
            v = P64[tv]
            e1, e2 = v[:, 1] - v[:, 0], v[:, 2] - v[:, 0]
            M = np.stack([-dd, e1, e2], axis=2)
            x = np.linalg.solve(M, (rr[:, 0:3] - v[:, 0])[..., None])[..., 0]
            return x[:, 1], x[:, 2], M

        def loss_of(P64, sel_rows=None):
            u, v, _ = bary(P64)
            val = (1 - u - v) * a[tv[:, 0]] + u * a[tv[:, 1]] + v * a[tv[:, 2]]
            return np.sum((val - tg) ** 2)

        u, v, M = bary(pos)
        val = (1 - u - v) * a[tv[:, 0]] + u * a[tv[:, 1]] + v * a[tv[:, 2]]
        r = 2 * (val - tg)
        gvec = np.stack([np.zeros_like(r), r * (a[tv[:, 1]] - a[tv[:, 0]]), r * (a[tv[:, 2]] - a[tv[:, 0]])], 1)
        lam = np.linalg.solve(np.transpose(M, (0, 2, 1)), gvec[..., None])[..., 0]
        gp = np.zeros((pos.shape[0], 3))
        gabs = np.zeros(pos.shape[0])  # sum of |per-ray contribution|: scale of the FP32 atomic sum's rounding
        for k, wk in enumerate([1 - u - v, u, v]):
            np.add.at(gp, tv[:, k], -wk[:, None] * lam)
            np.add.at(gabs, tv[:, k], np.linalg.norm(wk[:, None] * lam, axis=1))
        gg = grad.cpu().numpy().astype(np.float64)[:, :3]
        norm = np.linalg.norm(gp, axis=1)
        live = norm > 0
        floor = 1e-2 * np.median(norm[live]) if live.any() else 1.0
        rel = np.linalg.norm(gg - gp, axis=1)[live] / np.maximum(norm[live], floor)
        if float(np.max(rel)) > worst_detail.get("rel", -1.0):
            wv = np.nonzero(live)[0][int(np.argmax(rel))]
            contrib = np.sum(tv == wv)
            vals = np.array(seg_vals)[alive] if seg_vals is not None else None
            worst_detail.update({"rel": float(np.max(rel)), "scene": s, "segments_at_vertex": int(contrib),
                                 "grad_norm_over_floor": float(norm[wv] / floor),
                                 "abs_sum_over_grad_norm": float(gabs[wv] / max(norm[wv], 1e-300)),
                                 "max_value_error_of_scene": (float(np.max(np.abs(vals - val)))
                                                              if vals is not None else None)})
        worst_analytic.append(float(np.max(rel)))
        p99_analytic.append(float(np.percentile(rel, 99)))
        worst_cond.append(float(np.max(np.linalg.norm(gg - gp, axis=1)[live] / gabs[live])))
        # a segment that hits an edge shared by two triangles (a barycentric ~ 0)
        # has two valid closest hits at the same distance; forward and adjoint
        # may pick different ones (the ordered walks keep either), which moves
        # that ray's contribution to another triangle's corners
        edge = np.minimum(np.minimum(u, v), 1 - u - v) < 1e-6
        near_edge = np.zeros(pos.shape[0], bool)
        near_edge[tv[edge].reshape(-1)] = True
        off = live & ~near_edge
        edge_hits.append(int(edge.sum()))
        if off.any():
            worst_off_edge.append(float(np.max(np.linalg.norm(gg - gp, axis=1)[off] / np.maximum(norm[off], floor))))
        # FP64 central differences on 2 random vertices some sampled ray sees; the
        # difference between the Richardson extrapolations from h and h/2 is the
        # differences' own error, reported beside the result
        fd_err, fd_plain, fd_unc = 0.0, 0.0, 0.0
        seen = np.unique(tv.reshape(-1))
        for vi in rng.choice(seen, size=min(2, seen.size), replace=False):
            fd, fd2, fdp = np.zeros(3), np.zeros(3), np.zeros(3)
            for c in range(3):
                def cd(h):
                    pp, pm = pos.copy(), pos.copy()
                    pp[vi, c] += h
                    pm[vi, c] -= h
                    return (loss_of(pp) - loss_of(pm)) / (2 * h)
                c1, c2, c4 = cd(1e-4), cd(5e-5), cd(2.5e-5)
                fdp[c] = c1
                fd[c] = (4 * c2 - c1) / 3
                fd2[c] = (4 * c4 - c2) / 3
            den = max(np.linalg.norm(fd2), floor)
            fd_err = max(fd_err, float(np.linalg.norm(gg[vi] - fd2) / den))
            fd_plain = max(fd_plain, float(np.linalg.norm(gg[vi] - fdp) / den))
            fd_unc = max(fd_unc, float(np.linalg.norm(fd - fd2) / den))
        worst_unc.append(fd_unc)
        worst_fd.append(fd_err)
        worst_fd_plain.append(fd_plain)
    return {"sample_paths_per_scene": sample,
            "max_rel_vs_fp64_analytic": max(worst_analytic),
            "p99_rel_vs_fp64_analytic": max(p99_analytic),
            "max_err_over_contribution_abs_sum": max(worst_cond),
            "max_rel_vs_fp64_analytic_off_edge_hits": max(worst_off_edge) if worst_off_edge else None,
            "edge_hit_segments": int(sum(edge_hits)),
            "worst_vertex": worst_detail,
            "max_rel_vs_fp64_fd_richardson": max(worst_fd),
            "max_rel_vs_fp64_fd_h1e-4": max(worst_fd_plain),
            "max_fd_own_uncertainty": max(worst_unc),
            "median_rel_vs_fp64_fd_richardson": float(np.median(worst_fd)),
            "scenes_within_1e-3_of_fd": int(sum(1 for e, u in zip(worst_fd, worst_unc) if e <= 1e-3 + 2 * u)),
            "per_scene_rel_vs_fp64_fd_richardson": [round(x, 7) for x in worst_fd]}


def cpu_baseline_wavefront(S, cam, threads: int, budget_s: float, steps: int = 1):
    """The oracle's pipeline on host cores over a bounded band of rows (BVH built beforehand)."""
    from oracle import orc

    W, H = cam.width, cam.height
    # calibrate on a small band around the image centre, then size the sample
    r0 = H // 2 - 4
    _, rays, sec = orc.wavefront_shadow_bounce(S, cam.as_floats(), W, H, LIGHT, 0, row0=r0, row1=r0 + 8,
                                               threads=threads)
    rate = sum(rays) / max(sec, 1e-6)
    rows = int(max(8, min(H, budget_s * rate / max(1.0, sum(rays) / 8.0))))
    r0 = max(0, H // 2 - rows // 2)
    results = []
    for s in range(steps):
        _, rays, sec = orc.wavefront_shadow_bounce(S, cam.as_floats(), W, H, LIGHT, s, row0=r0, row1=r0 + rows,
                                                   threads=threads)
        results.append((sum(rays), sec))
    total_rays = sum(r for r, _ in results)
    total_s = sum(s for _, s in results)
    return {"value": round(total_rays / total_s / 1e6, 3), "unit": "Mrays/s", "cores": threads, "kind": "port",
            "sample": f"rows {r0}..{r0 + rows} of the {W}x{H} frame ({total_rays // steps} rays per step)"}, total_s


def run_reference(args, ws, rank):
    """--impl reference: the oracle port of the reference's CPU path on all host threads."""
    if rank != 0:
        return None
    from rendiation_gb300 import scenes

    threads = os.cpu_count() or 1
    mesh = scenes.heightfield(args.grid, seed=1)
    cam = scenes.heightfield_camera(args.width, args.height)
    S = oracle_heightfield(mesh)
    for _ in range(args.warmup):
        cpu_baseline_wavefront(S, cam, threads, budget_s=1.0)
    cb, total_s = cpu_baseline_wavefront(S, cam, threads, budget_s=args.cpu_budget / max(1, args.steps),
                                         steps=args.steps)
    return {
        "impl": "reference",
        "metric": METRIC,
        "value": cb["value"],
        "unit": "Mrays/s",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(total_s * 1000.0 / args.steps, 3),
        "higher_is_better": True,
        "scaling": "strong",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded heightfield, PCG64 seed 1)",
        "config": {"workload": f"wavefront primary+shadow+bounce, heightfield {args.grid}^2, "
                               f"{args.width}x{args.height} primaries (bounded row sample per step)"},
        "cpu_baseline": cb,
        "e2e": {"value": cb["value"], "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def headline(out: dict) -> dict:
    """The metric's three figures in one place: the plain wavefront Mrays/s,
    batched against the plain per-scene loop, forward + adjoint against forward
    (the configuration's own form: hits recomputed in the backward), each at its
    stated FP64 error and oracle parity."""
    h = {"wavefront_mrays": out.get("value"), "wavefront_e2e_mrays": out.get("e2e", {}).get("value")}
    if "batched" in out:
        h["batched_over_plain_loop"] = out["batched"]["speedup_vs_plain_loop"]
        h["batched_graph_mrays"] = out["batched"]["batched_graph_mrays"]
    if "batched_adjoint" in out:
        cc = out["batched_adjoint"].get("config_conforming", {})
        h["fwd_adjoint_over_fwd_recompute"] = cc.get("fwd_adjoint_over_fwd")
        h["fwd_adjoint_over_fwd_tape"] = out["batched_adjoint"].get("fwd_adjoint_over_fwd")
    if "adjoint" in out and "gradient_error" in out["adjoint"]:
        ge = out["adjoint"]["gradient_error"]
        h["gradient_max_rel_vs_fp64_fd_h1e-4"] = ge["max_rel_vs_fp64_fd_h1e-4"]
        h["gradient_max_rel_vs_fp64_fd_richardson"] = ge["max_rel_vs_fp64_fd_richardson"]
        h["gradient_max_rel_vs_fp64_analytic"] = ge["max_rel_vs_fp64_analytic_positions"]
    if "accuracy_vs_fp64" in out:
        h["t_max_rel_error_vs_fp64"] = out["accuracy_vs_fp64"]["max_rel_t_error_vs_fp64_same_triangle"]
    if "parity" in out:
        fr = out["parity"]["frame"]
        h["parity_other"] = out["parity"]["other_total"]
        h["parity_frame_ties"] = {"primary": fr["primary"]["tie"], "bounce": fr["bounce"]["tie"]}
        h["parity_frame_nan_exposed"] = {"primary": fr["primary"]["nan"], "shadow": fr["shadow"]["nan"],
                                         "bounce": fr["bounce"]["nan"]}
    if "path_tracing" in out:
        ptl = out["path_tracing"]
        h["path_tracer_mrays"] = {k: ptl[k]["mrays"] for k in ("clamped", "full_1080p") if k in ptl}
        if "parity_texels_identical" in ptl.get("clamped", {}):
            h["path_tracer_parity_texels_identical"] = ptl["clamped"]["parity_texels_identical"]
    return h


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="wavefront", choices=["wavefront"])
    ap.add_argument("--grid", type=int, default=1024)
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--traversal", default="ordered", choices=["ordered", "wide", "reference"])
    ap.add_argument("--block", type=int, default=0)
    ap.add_argument("--cpu-budget", type=float, default=12.0, help="seconds of CPU work for the CPU baseline")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-tune", dest="tune", action="store_false", help="skip the launch autotuner")
    ap.add_argument("--tune-cache", default=None, help="JSON file that keeps the autotuner's choices between runs")
    ap.add_argument("--no-batched-adjoint", action="store_true")
    ap.add_argument("--no-ao", action="store_true", help="skip the ambient-occlusion leg")
    ap.add_argument("--no-task-graph", action="store_true", help="skip the task-graph throughput leg")
    ap.add_argument("--no-path-tracing", action="store_true", help="skip the reference path-tracer leg")
    ap.add_argument("--no-accuracy", action="store_true", help="skip the FP32-vs-FP64 accuracy check")
    ap.add_argument("--no-parity", action="store_true", help="skip the oracle parity report")
    ap.add_argument("--no-watertight", action="store_true", help="skip the watertight-test frame timing")
    ap.add_argument("--no-plain-soup", action="store_true", help="skip the plain 10k-soup closest-hit leg")
    ap.add_argument("--diff-scenes", type=int, default=64)
    ap.add_argument("--scenes", type=int, default=256)
    ap.add_argument("--batched-steps", type=int, default=5)
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)

    ws, rank, local = dist_env()
    if args.impl == "reference":
        out = run_reference(args, ws, rank)
        if out is not None:
            print(json.dumps(out), flush=True)
        return

    import torch

    torch.cuda.set_device(local)
    if ws > 1:
        torch.distributed.init_process_group("nccl")
    out, P, mesh, cam, wf = bench_wavefront(args, ws, rank)
    # the oracle's copy of the heightfield (CPU), for the accuracy and parity checks and the CPU baseline
    need_oracle = not (args.no_accuracy and args.no_cpu_baseline and args.no_parity)
    S_field = oracle_heightfield(mesh) if rank == 0 and need_oracle else None
    if S_field is not None and not args.no_accuracy:
        out["accuracy_vs_fp64"] = accuracy_vs_fp64(P, S_field, cam)
    if not args.no_watertight:
        out["watertight"] = bench_watertight(args, P, wf, cam)
    if S_field is not None and not args.no_parity:
        out["parity"] = parity_report(P, S_field, wf, cam, os.cpu_count() or 1)
    if not args.no_plain_soup:
        out["plain_soup10k"] = bench_plain_soup(args)
    if not args.no_ao:
        out["ao"] = bench_ao(args, P, S_field if not args.no_cpu_baseline else None)
    if not args.no_task_graph:
        out["task_graph"] = bench_task_graph(args, P)
    if not args.no_path_tracing:
        out["path_tracing"] = bench_path_tracing(args, P, S_field if not args.no_cpu_baseline else None)
    if not args.no_batched:
        P.close()
        out["batched"] = bench_batched(args, ws, rank)
    if not args.no_adjoint:
        out["adjoint"] = bench_adjoint(args, ws, rank)
    if not args.no_batched_adjoint:
        out["batched_adjoint"] = bench_batched_adjoint(args, ws, rank)
    if rank == 0:
        if not args.no_cpu_baseline:
            cb, _ = cpu_baseline_wavefront(S_field, cam, os.cpu_count() or 1, budget_s=args.cpu_budget)
            out["cpu_baseline"] = cb
        out["headline"] = headline(out)
        print(json.dumps(out), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
