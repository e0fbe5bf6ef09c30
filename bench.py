#!/usr/bin/env python
"""Forward + backward throughput of the differentiable rasteriser.

Workload (one step = one forward and one backward over one batch):
  35,002 V / 70,000 F displaced sphere (mm), 1024^2 texture, textured +
  SH-shaded, 8 ring views at 1024x1024 (8,388,608 pixels), upstream image
  gradient N(0,1), no target-image gradient.  Seeded synthetic inputs.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gvr|reference]

One JSON line on rank 0.  `value` is device time with inputs resident in
HBM (L2 flushed between steps by a 256 MiB memset outside the timed events);
`e2e` goes through the C ABI with pinned host buffers and the host<->device
copies inside the timed region: every step copies its inputs in and its
render and gradients out, on copy streams that overlap the kernels of the
neighbouring steps (the serial form, one stream, is reported beside it).
Under torchrun every rank renders its own
replica (the path needs no cross-GPU exchange), `value` is the total pixels
of all ranks / the slowest rank's time.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

REPO = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(REPO, "gvv-differentiable-cuda-renderer_gb300")
for _p in (PKG, REPO):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "fwd+bwd Mpix/s (8×1024², 70k faces)"
UNIT = "Mpix/s"
WORKLOAD = ("multiview_textured: 35,002 V / 70,000 F displaced sphere (mm), textured 1024^2 + SH shaded, "
            "8 ring views at 1024x1024, fwd+bwd w.r.t. vertices, texture and SH")
FLUSH_BYTES = 256 << 20


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", choices=["gvr", "reference"], default="gvr")
    ap.add_argument("--cpu-seconds", type=float, default=10.0, help="bound of the CPU-baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer pass (profiling runs)")
    ap.add_argument("--views", type=int, default=8, help="views of the workload (profiling runs use fewer)")
    ap.add_argument("--workload", choices=["multiview", "batched", "fit", "learned", "gemm", "atomics"],
                    default="multiview",
                    help="multiview: the fwd+bwd step above (default); batched: 64 uneven meshes through one "
                         "plan (forward + backward), against the same jobs as one call each; fit: plain "
                         "analysis-by-synthesis fits of the morphable model; learned: train the proposal "
                         "network, then fit from its proposals against the plain fit; gemm: the proposal "
                         "network's GEMM shapes on the tcgen05 kernel and on torch.matmul; atomics: the L2's "
                         "FP32 reduction rate, the peak the scatter kernels' atomics are read against")
    ap.add_argument("--meshes", type=int, default=64, help="meshes of the batched workload")
    ap.add_argument("--fits", type=int, default=1000, help="held-out seeds of the fit / learned workloads")
    ap.add_argument("--train-renders", type=int, default=1_000_000, help="renders the proposal network trains on")
    ap.add_argument("--fit-batch", type=int, default=50, help="fits run together")
    ap.add_argument("--gemm-shapes", default="", help="gemm workload: comma-separated shape names to run (default all)")
    return ap.parse_args()


def algorithmic_bytes(P, C, N, F, Ht, Wt, textured, vertex_color):
    """Bytes one fwd+bwd call must move: per pixel the render, face id,
    barycentrics, upstream gradient and their reads (64 B); per view the
    vertex normals, face records and (textured) UVs; the texture and its
    gradient; vertex positions and their gradient; SH and its gradient."""
    return (P * 64 + C * (12 * N + 12 * F + 24 * F * textured + 12 * N) + 12 * N * vertex_color +
            24 * Ht * Wt * textured + 24 * N + 216 * C)


def kernel_bytes(name, P, C, N, F, Ht, Wt, textured, target):
    """Algorithmic bytes of one launch of the two pixel kernels."""
    if name == "k_raster":    # render 12 + face 4 + bary 8 per pixel; vertex normals, faces, uvs, texture read
        return P * 24 + C * (12 * N + 12 * F + 24 * F * textured) + 12 * Ht * Wt * textured
    if name == "k_bwd_pixels":  # grad_render 12 + face 4 + bary 8 (+ target and its grad) per pixel; texture grad written
        return P * (24 + 24 * target) + C * (12 * N + 12 * F + 24 * F * textured) + 24 * Ht * Wt * textured
    return None


class ClockSampler:
    """nvidia-smi samples (200 ms) of SM clock and throttle reasons while running."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        self.t0 = time.time()

    def stop(self):
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        rows = []
        if self.path and os.path.exists(self.path):
            for line in open(self.path):
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
            os.remove(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        mx = [num(r[2]) for r in rows if num(r[2]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in rows for n, v in zip(names, r[5:9]) if v.strip().lower() == "active"})
        load = [s for s in sm if mx and s >= 0.5 * max(mx)] or sm
        return {"sm_mhz": statistics.median(load) if load else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def dist_setup():
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    return world, rank, local


def reduce_max(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def cpu_reference(scene, seconds, max_reps=None):
    """The oracle port (CPU restatement of the reference kernels) on all host
    cores: full fwd+bwd of the workload, repeated up to `seconds`."""
    from oracle import oracle
    from oracle.oracle import OracleScene
    s = scene
    o = OracleScene(s["faces"], s["uvs"], s["vertex_pos"][0], s["vertex_color"][0], s["texture"][0],
                    s["sh_coeff"][0], s["extrinsics"][0], s["intrinsics"][0], s["width"], s["height"],
                    s["albedo_mode"], s["shading_mode"])
    reps, t0 = 0, time.perf_counter()
    while True:
        out = o.forward()
        o.backward(out["face"], out["bary"], out["vertex_normal"], s["grad_render"][0], s["target_image"][0],
                   s["grad_target"][0])
        reps += 1
        el = time.perf_counter() - t0
        if el >= seconds or (max_reps and reps >= max_reps):
            break
    P = s["num_views"] * s["width"] * s["height"]
    return {"value": P * reps / el / 1e6, "unit": UNIT, "cores": oracle.num_threads(), "kind": "port",
            "sample": f"{reps} x the full workload (fwd+bwd, 8 views 1024^2), {el:.1f} s"}


def run_reference(args):
    """The reference has no CPU implementation of this path (its kernels are
    CUDA only), so this arm times the oracle port of those kernels on every
    host core.  Each step is a bounded sample of the workload: one of the 8
    views (cycling) at full resolution, forward + backward."""
    world, rank, _ = dist_setup()
    if rank != 0:
        return
    from gvr import scenes
    from oracle import oracle
    from oracle.oracle import OracleScene
    oracle.build()
    s = scenes.multiview_textured(seed=0)
    P1 = s["width"] * s["height"]

    def one_view(c):
        sl = slice(c, c + 1)
        o = OracleScene(s["faces"], s["uvs"], s["vertex_pos"][0], s["vertex_color"][0], s["texture"][0],
                        s["sh_coeff"][0][sl], s["extrinsics"][0][sl], s["intrinsics"][0][sl], s["width"],
                        s["height"], s["albedo_mode"], s["shading_mode"])
        out = o.forward()
        o.backward(out["face"], out["bary"], out["vertex_normal"], s["grad_render"][0][sl], s["target_image"][0][sl],
                   s["grad_target"][0][sl])

    for k in range(args.warmup):
        one_view(k % s["num_views"])
    times = []
    for k in range(args.steps):
        t0 = time.perf_counter()
        one_view(k % s["num_views"])
        times.append(time.perf_counter() - t0)
    ms = 1e3 * sum(times) / len(times)
    value = P1 / (ms / 1e3) / 1e6
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "fp64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "batch": 1, "views": 8, "resolution": 1024, "faces": 70000,
                       "vertices": 35002, "texture": 1024, "parallelism": "replicas"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": oracle.num_threads(), "kind": "port",
                             "sample": "each step: one of the 8 views (cycling) at 1024^2, fwd+bwd, on the CPU "
                                       "oracle (the reference has no CPU path; its kernels are CUDA only)"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    gpu = reference_kernels_gpu(s)
    if gpu is not None:
        line["reference_kernels_gpu"] = gpu
    print(json.dumps(line), flush=True)


def reference_kernels_gpu(s, reps=3):
    """The reference's own CUDA kernels (cpp/src/Renderer/CUDABasedRasterization{,Grad}.cu,
    compiled unmodified for sm_103a with nvcc's default flags into
    oracle/_ref) on the same workload and GPU: mean forward and backward ms
    of `reps` calls after one warm-up (the reference's kernel timing, CUDA
    events around its launch sequence).  None where no GPU or no build."""
    try:
        import torch
        if not torch.cuda.is_available():
            return None
        from oracle import refcore
        if not refcore.available():
            return None
        ref = refcore.Refcore(fmad=True)
        fwd = ref.forward(s)
        ref.backward(s, fwd)
        f_ms, b_ms = [], []
        for _ in range(reps):
            fwd = ref.forward(s)
            f_ms.append(fwd["ms"])
            b_ms.append(ref.backward(s, fwd)["ms"])
        ref.close()
    except Exception as exc:  # a measurement beside the line, never a failure of it
        return {"unavailable": f"{type(exc).__name__}: {exc}"}
    P = s["num_views"] * s["width"] * s["height"]
    f, b = sum(f_ms) / reps, sum(b_ms) / reps
    return {"fwd_ms": f, "bwd_ms": b, "value": P / ((f + b) / 1e3) / 1e6, "unit": UNIT, "reps": reps,
            "build": "reference kernels from their sources, nvcc defaults, sm_103a; one GPU, same workload",
            "gpu": torch.cuda.get_device_name(0)}


def run_gvr(args):
    import numpy as np
    import torch

    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from gvr import _lib, native_build, renderer, scenes
    native_build.build()
    L = _lib.load()

    s = scenes.multiview_textured(seed=rank, num_views=args.views)
    B, C, H, W = 1, s["num_views"], s["height"], s["width"]
    N, F = s["num_vertices"], s["faces"].shape[0]
    Ht, Wt = s["texture"].shape[1], s["texture"].shape[2]
    P = B * C * H * W
    h = renderer.get_handle(s["faces"], s["uvs"], N, C, W, H, s["albedo_mode"], s["shading_mode"], device=dev)
    host = {k: torch.from_numpy(np.ascontiguousarray(s[k])).pin_memory()
            for k in ("vertex_pos", "vertex_color", "texture", "sh_coeff", "extrinsics", "intrinsics", "grad_render")}
    d = {k: v.to(dev) for k, v in host.items()}
    out = dict(bary=torch.empty((B, C, H, W, 2), device=dev), face=torch.empty((B, C, H, W), dtype=torch.int32, device=dev),
               render=torch.empty((B, C, H, W, 3), device=dev), vnorm=torch.empty((B, C, N, 3), device=dev),
               gpos=torch.empty((B, N, 3), device=dev), gcol=torch.empty((B, N, 3), device=dev),
               gtex=torch.empty((B, Ht, Wt, 3), device=dev), gsh=torch.empty((B, C, 27), device=dev))
    fws = torch.empty(h.forward_workspace_size(B), dtype=torch.uint8, device=dev)
    bws = torch.empty(h.backward_workspace_size(B), dtype=torch.uint8, device=dev)
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    fa = _lib.GvrForwardArgs(B, Ht, Wt, p(d["vertex_pos"]), p(d["vertex_color"]), p(d["texture"]), p(d["sh_coeff"]),
                             None, p(d["extrinsics"]), p(d["intrinsics"]), p(out["bary"]), p(out["face"]),
                             p(out["render"]), p(out["vnorm"]), None, None, p(fws), fws.numel())
    ba = _lib.GvrBackwardArgs(B, Ht, Wt, p(d["grad_render"]), p(d["vertex_pos"]), p(d["vertex_color"]), p(d["texture"]),
                              p(d["sh_coeff"]), None, p(out["vnorm"]), p(out["bary"]), p(out["face"]), None, p(d["extrinsics"]),
                              p(d["intrinsics"]), p(out["gpos"]), p(out["gcol"]), p(out["gtex"]), p(out["gsh"]),
                              p(bws), bws.numel())
    stream = torch.cuda.current_stream(dev)
    sp = ctypes.c_void_p(stream.cuda_stream)

    def step():
        _lib.check(L.gvr_forward(h.ptr, ctypes.byref(fa), sp))
        _lib.check(L.gvr_backward(h.ptr, ctypes.byref(ba), sp))

    flush = torch.empty(FLUSH_BYTES, dtype=torch.uint8, device=dev)
    clocks = ClockSampler(local)
    clocks.start()
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    # ---- timed region: K steps, device time per step between events
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    barrier(world)
    torch.cuda.synchronize()
    n0 = L.gvr_launch_count()
    t_wall = time.perf_counter()
    for a, b in evs:
        flush.zero_()
        a.record(stream)
        step()
        b.record(stream)
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall
    barrier(world)
    launches = L.gvr_launch_count() - n0
    ms = sum(a.elapsed_time(b) for a, b in evs) / args.steps
    ms = reduce_max(ms, world)
    value = world * P / (ms / 1e3) / 1e6

    # ---- per-kernel time of the same steps (events around each launch, on the launching stream)
    L.gvr_profile_enable(1)
    for _ in range(args.steps):
        flush.zero_()
        step()
    torch.cuda.synchronize()
    prof = _lib.profile_read()
    L.gvr_profile_enable(0)
    clk = clocks.stop()
    dom = max(prof.items(), key=lambda kv: kv[1][1])
    dom_name, (dom_n, dom_ms) = dom[0], dom[1]
    dom_avg = dom_ms / max(dom_n, 1)
    textured = s["albedo_mode"] == "textured"
    kb = kernel_bytes(dom_name, P, C, N, F, Ht, Wt, textured, 0)
    peaks = {}
    pk_path = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(pk_path):
        peaks = json.load(open(pk_path))
    peak = peaks.get("hbm_gbs") or 6800.0
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    traffic = None
    tf_path = os.path.join(REPO, "profiles", "dram_traffic.json")
    if os.path.exists(tf_path):
        traffic = json.load(open(tf_path)).get(dom_name)
    achieved = (kb / (dom_avg / 1e3) / 1e9) if kb else None
    roofline = {"bound": "hbm", "kernel": dom_name, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                "bytes_per_launch": kb, "avg_launch_ms": dom_avg, "peak_source": peak_src}
    step_bytes = algorithmic_bytes(P, C, N, F, Ht, Wt, int(textured), int(s["albedo_mode"] == "vertexColor"))

    # ---- end to end through the C ABI with host buffers.  Every step copies
    # its inputs in from pinned host memory and its render and gradients out.
    # Pipelined: two buffer sets; inputs go in on one copy stream, results
    # out on another, the forward and backward run on the compute stream, so
    # step i's copies overlap the kernels of steps i-1 and i+1 (and the
    # upstream gradient's copy overlaps the step's own forward).  The serial
    # form (copy in, compute, copy out on one stream) is reported beside it.
    hres = [{k: torch.empty(out[k].shape, dtype=out[k].dtype).pin_memory() for k in ("render", "gpos", "gtex", "gsh")}
            for _ in range(2)]
    h2d = sum(v.numel() * v.element_size() for v in host.values())
    d2h = sum(v.numel() * v.element_size() for v in hres[0].values())
    small = [k for k in host if k != "grad_render"]
    dsets = [d, {k: torch.empty_like(v) for k, v in d.items()}]
    osets = [out, {k: torch.empty_like(v) for k, v in out.items()}]
    fas, bas = [], []
    for dd, oo in zip(dsets, osets):
        fas.append(_lib.GvrForwardArgs(B, Ht, Wt, p(dd["vertex_pos"]), p(dd["vertex_color"]), p(dd["texture"]),
                                       p(dd["sh_coeff"]), None, p(dd["extrinsics"]), p(dd["intrinsics"]), p(oo["bary"]),
                                       p(oo["face"]), p(oo["render"]), p(oo["vnorm"]), None, None, p(fws), fws.numel()))
        bas.append(_lib.GvrBackwardArgs(B, Ht, Wt, p(dd["grad_render"]), p(dd["vertex_pos"]), p(dd["vertex_color"]),
                                        p(dd["texture"]), p(dd["sh_coeff"]), None, p(oo["vnorm"]), p(oo["bary"]), p(oo["face"]),
                                        None, p(dd["extrinsics"]), p(dd["intrinsics"]), p(oo["gpos"]), p(oo["gcol"]),
                                        p(oo["gtex"]), p(oo["gsh"]), p(bws), bws.numel()))
    s_in, s_out = torch.cuda.Stream(dev), torch.cuda.Stream(dev)
    ev = lambda: torch.cuda.Event()
    comp_done, out_done = [ev(), ev()], [ev(), ev()]
    for e_ in comp_done + out_done:
        e_.record(stream)

    def e2e_pipelined(i):
        j = i & 1
        dd, oo, hh = dsets[j], osets[j], hres[j]
        in_small, in_grad, fwd_done = ev(), ev(), ev()
        s_in.wait_event(comp_done[j])              # step i-2's kernels are done with these inputs
        with torch.cuda.stream(s_in):
            for k in small:
                dd[k].copy_(host[k], non_blocking=True)
            in_small.record(s_in)
            dd["grad_render"].copy_(host["grad_render"], non_blocking=True)
            in_grad.record(s_in)
        stream.wait_event(in_small)
        stream.wait_event(out_done[j])             # step i-2's results are copied out of these outputs
        _lib.check(L.gvr_forward(h.ptr, ctypes.byref(fas[j]), sp))
        fwd_done.record(stream)
        stream.wait_event(in_grad)
        _lib.check(L.gvr_backward(h.ptr, ctypes.byref(bas[j]), sp))
        comp_done[j].record(stream)
        s_out.wait_event(fwd_done)
        with torch.cuda.stream(s_out):
            hh["render"].copy_(oo["render"], non_blocking=True)
            s_out.wait_event(comp_done[j])
            for k in ("gpos", "gtex", "gsh"):
                hh[k].copy_(oo[k], non_blocking=True)
            out_done[j].record(s_out)

    def e2e_serial():
        for k, v in host.items():
            d[k].copy_(v, non_blocking=True)
        step()
        for k, v in hres[0].items():
            v.copy_(out[k], non_blocking=True)

    e2e_ms = e2e_serial_ms = float("nan")
    if not args.no_e2e:
        torch.cuda.synchronize()
        for i in range(max(2, args.warmup)):
            e2e_pipelined(i)
        torch.cuda.synchronize()
        barrier(world)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        s_in.wait_event(e0)
        for i in range(args.steps):
            e2e_pipelined(i)
        stream.wait_stream(s_out)
        e1.record(stream)
        torch.cuda.synchronize()
        e2e_ms = reduce_max(e0.elapsed_time(e1) / args.steps, world)
        # every step's results reached the host: the last two buffer sets match a serial step
        for k in ("render", "gtex"):
            if not torch.equal(hres[(args.steps - 1) & 1][k], osets[(args.steps - 1) & 1][k].cpu()):
                raise RuntimeError(f"pipelined e2e: host copy of {k} differs from the device result")
        for _ in range(max(1, args.warmup)):
            e2e_serial()
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.steps):
            e2e_serial()
        e1.record(stream)
        torch.cuda.synchronize()
        e2e_serial_ms = reduce_max(e0.elapsed_time(e1) / args.steps, world)
        barrier(world)

    if rank != 0:
        return
    cpu = None
    if world == 1 and not args.no_cpu_baseline:
        try:
            cpu = cpu_reference(s, args.cpu_seconds)
        except Exception as exc:  # the checker is optional for the GPU number
            cpu = {"value": None, "unit": UNIT, "cores": None, "kind": "port", "sample": f"failed: {exc}"}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "fp32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "batch": B, "views": C, "resolution": W, "faces": F, "vertices": N,
                       "texture": Wt, "l2": "flushed between steps (256 MiB memset outside the timed events)",
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "faces_per_s": world * B * C * F / (ms / 1e3),
            "step_roofline": {"bytes": step_bytes, "achieved": step_bytes / (ms / 1e3) / 1e9, "peak": peak,
                              "unit": "GB/s", "frac": step_bytes / (ms / 1e3) / 1e9 / peak},
            "roofline": roofline,
            "kernels_ms_per_step": {k: round(v[1] / args.steps, 5) for k, v in sorted(prof.items(), key=lambda kv: -kv[1][1])},
            "e2e": {"value": world * P / (e2e_ms / 1e3) / 1e6, "unit": UNIT, "ms_per_step": e2e_ms,
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "pipeline": "2 buffer sets; copies in and out on their own streams overlap the kernels",
                    "serial_ms_per_step": e2e_serial_ms,
                    "serial_value": world * P / (e2e_serial_ms / 1e3) / 1e6},
            "gpu_launches": launches, "timed_wall_s": t_wall,
            "clocks": clk, "cpu_baseline": cpu}
    print(json.dumps(line), flush=True)


def run_batched(args):
    """Uneven batch: `--meshes` displaced spheres with 1k..200k faces, 1..8
    views each at 256^2/512^2/1024^2, mixed modes, 512^2 textures (views of a
    mesh sharing a resolution form one job).  One step = the forward and the
    backward (upstream gradients N(0, 1)) of every job.  Timed three ways on
    the same buffers: the plan's forward and backward replayed as CUDA graphs
    (autotuned tiles; the value), the plan launched eagerly, and one
    gvr_forward + gvr_backward call per job (the per-mesh loop); the
    forward alone is reported beside them."""
    import torch
    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from gvr import _lib, native_build, renderer, scenes
    from gvr.batch import BatchPlan
    native_build.build()
    L = _lib.load()
    specs = scenes.uneven_batch(seed=rank, num_meshes=args.meshes)
    jobs = []
    for s in specs:
        h = renderer.get_handle(s["faces"], s["uvs"], s["num_vertices"], s["num_views"], s["width"], s["height"],
                                s["albedo_mode"], s["shading_mode"], device=dev)
        jobs.append(dict(handle=h, vertex_pos=s["vertex_pos"], vertex_color=s["vertex_color"], texture=s["texture"],
                         sh_coeff=s["sh_coeff"], extrinsics=s["extrinsics"], intrinsics=s["intrinsics"]))
    t0 = time.perf_counter()
    plan = BatchPlan(jobs, autotune=True)
    tune_s = time.perf_counter() - t0
    P = sum(s["num_views"] * s["width"] * s["height"] for s in specs)
    faces = sum(s["num_views"] * s["faces"].shape[0] for s in specs)
    stream = torch.cuda.Stream(dev)
    flush = torch.empty(FLUSH_BYTES, dtype=torch.uint8, device=dev)

    def timed(fn):
        with torch.cuda.stream(stream):
            for _ in range(max(3, args.warmup)):
                fn()
            stream.synchronize()
            barrier(world)
            total = 0.0
            for _ in range(args.steps):
                flush.fill_(1)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                fn()
                e1.record(stream)
                e1.synchronize()
                total += e0.elapsed_time(e1)
        return reduce_max(total / args.steps, world)

    # upstream gradients N(0, 1) for every job, bound once (the buffers stay)
    import numpy as np
    rng = np.random.default_rng(rank)
    plan.forward(stream=stream)
    plan.bind_backward([rng.normal(0, 1, (1, s["num_views"], s["height"], s["width"], 3)).astype(np.float32)
                        for s in specs])
    stream.synchronize()

    def graph_step():
        plan.forward(stream=stream, graph=True)
        plan.backward(stream=stream, graph=True)

    def eager_step():
        plan.forward(stream=stream)
        plan.backward(stream=stream)

    def per_call_step():
        plan.forward_per_call(stream=stream)
        plan.backward_per_call(stream=stream)

    reps = max(3, args.warmup) + args.steps
    graph_ms = timed(graph_step)
    n0 = L.gvr_launch_count()
    eager_ms = timed(eager_step)
    n1 = L.gvr_launch_count()
    per_call_ms = timed(per_call_step)
    per_call_launches = (L.gvr_launch_count() - n1) / reps
    eager_launches = (n1 - n0) / reps  # graph replays add none here
    fwd_graph_ms = timed(lambda: plan.forward(stream=stream, graph=True))
    fwd_per_call_ms = timed(lambda: plan.forward_per_call(stream=stream))
    # the same jobs with the one persistent raster kernel instead of per-job lanes
    plan_p = BatchPlan(jobs, autotune=True, persistent=True)
    fwd_persistent_ms = timed(lambda: plan_p.forward(stream=stream, graph=True))
    plan_p.close()
    cfgs = {}
    for j in range(len(jobs)):
        cfgs.setdefault("%dx%d/%d" % plan.tile_config(j), 0)
        cfgs["%dx%d/%d" % plan.tile_config(j)] += 1
    if rank != 0:
        return
    value = world * P / (graph_ms / 1e3) / 1e6
    line = {"metric": "batched fwd+bwd Mpix/s (64 uneven meshes)", "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": graph_ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "fp32", "data": "synthetic",
            "config": {"workload": f"uneven_batch: {args.meshes} displaced spheres, faces log-uniform 1k..200k, "
                                   "1..8 views at 256/512/1024^2, mixed albedo x shading modes, 512^2 textures",
                       "jobs": len(jobs), "views": sum(s["num_views"] for s in specs), "pixels": P,
                       "view_faces": faces, "l2": "flushed between steps (256 MiB fill outside the timed events)",
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "faces_per_s": world * faces / (graph_ms / 1e3),
            "plan_graph_ms": graph_ms, "plan_eager_ms": eager_ms, "per_call_ms": per_call_ms,
            "per_call_mpix_s": P / (per_call_ms / 1e3) / 1e6,
            "forward_only": {"plan_graph_ms": fwd_graph_ms, "per_call_ms": fwd_per_call_ms,
                             "plan_graph_mpix_s": P / (fwd_graph_ms / 1e3) / 1e6,
                             "persistent_plan_graph_ms": fwd_persistent_ms},
            "launches_per_step": {"plan": eager_launches, "per_call": per_call_launches},
            "autotune_s": tune_s, "tile_configs": cfgs}
    print(json.dumps(line), flush=True)


def _fit_summary(ev, batch):
    """Per-seed figures of a proposal.evaluate result.  A fit that never
    reaches the goal counts with its whole run; times are per fit (the
    batch's GPU time shared by its `batch` fits)."""
    import numpy as np
    steps = ev["steps_to_goal"]
    ok = [s is not None for s in steps]
    n = len(steps)
    per_fit_total = ev["total_gpu_ms"] / n
    ms = [m / batch if m is not None else None for m in ev["gpu_ms_to_goal"]]
    solved = [m for m in ms if m is not None]
    return {"seeds": n, "reached": int(sum(ok)), "reached_frac": sum(ok) / n,
            "median_steps_to_goal": float(np.median([s for s in steps if s is not None])) if any(ok) else None,
            "median_gpu_ms_to_goal_per_fit": float(np.median(solved)) if solved else None,
            "mean_gpu_ms_to_solution_per_fit": float(np.mean([m if m is not None else per_fit_total for m in ms])),
            "final_rmse_median": float(np.median(ev["final_rmse"])), "total_gpu_ms": ev["total_gpu_ms"],
            # the whole run's GPU time per fit that reaches the goal: what one solved fit costs
            "gpu_ms_per_fit_reaching_goal": ev["total_gpu_ms"] / sum(ok) if any(ok) else None}


def run_fit_bench(args):
    """Analysis-by-synthesis fitting of the morphable model (28,000 vertices,
    80 shape + 80 albedo bases, pose, 27 SH; 4 views at 512^2; 200 Adam
    steps on photometric L2) on `--fits` held-out seeds.  `learned` first
    trains the proposal network on `--train-renders` renders from this
    rasteriser, then fits from its proposals (plain fit from the mean as
    fallback when the RMSE is above 0.05 after 20 steps) and from the mean."""
    import torch
    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from gvr import fitting, native_build, proposal, tc
    native_build.build()
    clocks = ClockSampler(local)
    clocks.start()
    model = fitting.MorphableModel(num_vertices=28000, seed=0, device=dev)
    fitter = fitting.Fitter(model, num_views=4, size=512, silhouette=fitting.Fitter.SILHOUETTE)
    seeds = list(range(1_000_000, 1_000_000 + args.fits))
    line = {"n_gpus": world, "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
            "data": "synthetic", "unit": "ms"}
    plain = proposal.evaluate(fitter, None, seeds, batch=args.fit_batch)
    ps = _fit_summary(plain, args.fit_batch)
    cfg = {"workload": "morphable-model fit: 28,000 V displaced-sphere mean + 80 shape + 80 albedo smooth bases, "
                       "pose 6, SH 27; 4 views at 512^2; 200 Adam steps on photometric L2 + silhouette term "
                       "(distance field to the target outline through the model-to-data gradient); goal RMSE <= 0.01",
           "fits": args.fits, "fit_batch": args.fit_batch}
    if args.workload == "fit":
        line.update(metric="fit GPU ms to RMSE<=0.01 (plain, per fit)", value=ps["mean_gpu_ms_to_solution_per_fit"],
                    config=cfg, plain=ps)
    else:
        net = proposal.ProposalNet(dev, seed=0)
        batch = 256
        trainer = proposal.Trainer(model, net, batch=batch, lr=1e-3, seed=7)
        steps = max(1, args.train_renders // batch)
        losses, secs = trainer.train(steps, log_every=max(1, steps // 20))
        learned = proposal.evaluate(fitter, net, seeds, batch=args.fit_batch)
        ls = _fit_summary(learned, args.fit_batch)
        t_l, t_p = proposal.time_to_match(learned, plain)
        ls["mean_gpu_ms_to_plain_final_rmse_per_fit"] = float(t_l.mean())
        ps["mean_gpu_ms_full_fit_per_fit"] = float(t_p.mean())
        cfg.update(train_renders=steps * batch, train_batch=batch,
                   network="5 conv 3x3/2 (3-32-64-128-256-256) + MLP 16384-1024-193, BF16 tcgen05 GEMMs, FP32 accum")
        line.update(metric="fit GPU ms to RMSE<=0.01 (learned proposal, per fit)",
                    value=ls["mean_gpu_ms_to_solution_per_fit"], config=cfg, learned=ls, plain=ps,
                    speedup_vs_plain=ps["mean_gpu_ms_to_solution_per_fit"] / ls["mean_gpu_ms_to_solution_per_fit"],
                    speedup_to_plain_final_rmse=float(t_p.mean() / t_l.mean()),
                    speedup_per_fit_reaching_goal=(ps["gpu_ms_per_fit_reaching_goal"] / ls["gpu_ms_per_fit_reaching_goal"]
                                                   if ps["gpu_ms_per_fit_reaching_goal"] and
                                                   ls["gpu_ms_per_fit_reaching_goal"] else None),
                    training={"steps": steps, "seconds": secs, "loss": losses, "tc_error": tc.tc_error()})
    line["clocks"] = clocks.stop()
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_gemm_bench(args):
    """The proposal network's matrix products at its real shapes (training
    batch 256, 256x256 input): the five im2col convolutions (forward, input
    gradient, weight gradient), the two MLP layers, and the first MLP
    layer's gradients.  Each on the tcgen05 GEMM (gvr_gemm_bf16 through
    gvr.tc.gemm, which splits K for the weight gradients as the network's
    calls do; BF16 operands, FP32 accumulate, operands already K-padded) and
    on torch.matmul (cuBLAS) with the same BF16 operands and output type;
    CUDA events, median of `--steps` launches after warm-up.  Reports
    TFLOP/s (2 M N K / t) and the GB/s of the minimal traffic (both operands
    read once, the output written once) against the measured peaks."""
    import torch
    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from gvr import native_build, tc
    native_build.build()
    B = 256
    shapes = []  # (name, M, N, K, output type)
    chans = (3, 32, 64, 128, 256, 256)
    hw = 256
    for i, (ci, co) in enumerate(zip(chans[:-1], chans[1:])):
        hw //= 2
        K = (9 * ci + 63) // 64 * 64
        M = B * hw * hw
        shapes.append((f"conv{i + 1} fwd", M, co, K, torch.bfloat16))
        shapes.append((f"conv{i + 1} dgrad", M, K, co if co % 64 == 0 else 64, torch.float32))
        shapes.append((f"conv{i + 1} wgrad", co, K, M, torch.float32))
    shapes += [("fc1 fwd", B, 1024, 16384, torch.float32), ("fc1 dgrad", B, 16384, 1024, torch.float32),
               ("fc1 wgrad", 1024, 16384, B, torch.float32), ("fc2 fwd", B, 193, 1024, torch.float32)]
    if args.gemm_shapes:
        keep = {x.strip() for x in args.gemm_shapes.split(",")}
        shapes = [sh for sh in shapes if sh[0] in keep]
    peaks = {}
    pk = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(pk):
        peaks = json.load(open(pk))
    rows = []
    gen = torch.Generator(device=dev).manual_seed(0)

    def timed(fn, reps):
        for _ in range(max(3, args.warmup)):
            fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            e1.synchronize()
            ts.append(e0.elapsed_time(e1))
        return statistics.median(ts)

    for name, M, N, K, odt in shapes:
        A = (torch.randn((M, K), generator=gen, device=dev) * 0.1).to(torch.bfloat16)
        Bm = (torch.randn((N, K), generator=gen, device=dev) * 0.1).to(torch.bfloat16)
        ours = timed(lambda: tc.gemm(A, Bm, out_dtype=odt), args.steps)
        ref = timed(lambda: torch.matmul(A, Bm.t()).to(odt), args.steps)
        exact = torch.matmul(A.float(), Bm.float().t())
        err = float((tc.gemm(A, Bm, out_dtype=torch.float32) - exact).abs().max() / exact.abs().max())
        flops = 2.0 * M * N * K
        byts = 2.0 * (M * K + N * K) + M * N * (2 if odt == torch.bfloat16 else 4)
        rows.append({"gemm": name, "M": M, "N": N, "K": K, "ours_ms": ours, "ours_tflops": flops / ours / 1e9,
                     "ours_gbs": byts / ours / 1e6, "torch_ms": ref, "torch_tflops": flops / ref / 1e9,
                     "torch_gbs": byts / ref / 1e6, "rel_err_vs_fp32": err})
        del A, Bm, exact
    tot_ours = sum(r["ours_ms"] for r in rows)
    tot_ref = sum(r["torch_ms"] for r in rows)
    line = {"metric": "proposal-network GEMM shape set, total ms (tcgen05 GEMM; cuBLAS beside it)",
            "value": tot_ours, "unit": "ms", "n_gpus": 1, "steps": args.steps, "warmup": max(3, args.warmup),
            "higher_is_better": False, "scaling": "none", "vs_baseline": None, "dtype": "bf16 (fp32 accumulate)",
            "data": "synthetic N(0, 0.01) operands",
            "config": {"workload": "proposal network GEMM shapes, batch 256, 256^2 input", "shapes": len(rows)},
            "torch_matmul_ms": tot_ref, "ratio_torch_over_ours": tot_ref / tot_ours,
            "peaks": {"bf16_tflops": peaks.get("bf16_tflops"), "hbm_gbs": peaks.get("hbm_gbs")}, "shapes": rows}
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_atomics_bench(args):
    """The L2's rate of fire-and-forget FP32 reductions on this GPU: the peak
    that the scatter kernels' reduction requests are read against.  Every
    addition of gvr_probe_reductions goes to its own pseudo-random 32-byte
    sector of a 64 MiB buffer (it stays in L2), so one addition is one L2
    reduction request; scalar and 16-byte (float4) additions, at 1 to 16
    resident blocks of 256 threads per SM.  CUDA events, median of
    `--steps` launches after warm-up."""
    import torch
    from gvr import _lib
    L = _lib.load()
    dev = torch.device("cuda", 0)
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    words = 16 << 20
    buf = torch.zeros(words, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    sp = ctypes.c_void_p(stream.cuda_stream)
    rounds = 64
    rows = []
    for vec in (0, 1):
        for per_sm in (1, 2, 4, 8, 16):
            grid = sms * per_sm

            def launch():
                _lib.check(L.gvr_probe_reductions(ctypes.c_void_p(buf.data_ptr()), words, vec, rounds, grid, sp))

            for _ in range(max(3, args.warmup)):
                launch()
            ts = []
            for _ in range(max(5, args.steps)):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                launch()
                e1.record(stream)
                e1.synchronize()
                ts.append(e0.elapsed_time(e1))
            ms = statistics.median(ts)
            n = grid * 256 * rounds
            rows.append({"bytes_per_addition": 16 if vec else 4, "blocks_per_sm": per_sm, "additions": n, "ms": ms,
                         "g_reductions_per_s": n / ms / 1e6, "gb_per_s": n * (16 if vec else 4) / ms / 1e6})
    best = {b: max(r["g_reductions_per_s"] for r in rows if r["bytes_per_addition"] == b) for b in (4, 16)}
    line = {"metric": "L2 FP32 reduction rate, random 32-byte sectors (peak for the scatter kernels)",
            "value": best[16], "unit": "G reductions/s (16-byte)", "n_gpus": 1, "steps": max(5, args.steps),
            "warmup": max(3, args.warmup), "higher_is_better": True, "scaling": "none", "vs_baseline": None,
            "dtype": "fp32", "data": "synthetic",
            "config": {"workload": "gvr_probe_reductions over a 64 MiB buffer, 64 additions per thread", "sms": sms},
            "g_reductions_per_s_4byte": best[4], "g_reductions_per_s_16byte": best[16], "rows": rows}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batched":
        run_batched(args)
    elif args.workload in ("fit", "learned"):
        run_fit_bench(args)
    elif args.workload == "gemm":
        run_gemm_bench(args)
    elif args.workload == "atomics":
        run_atomics_bench(args)
    else:
        run_gvr(args)
    if int(os.environ.get("WORLD_SIZE", "1")) > 1:
        import torch.distributed as dist
        if dist.is_initialized():
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
