#!/usr/bin/env python3
"""Benchmark: Dual Marching Cubes + non-manifold repair on GB300.

One step = one pass of the reference's DMC entry point over one grid: grid
refinement (UniformGridHost::readFromFile's refine, minus file IO), then
DualMarchingCubes::run with the reference's default flags (vertex-to-surface
iteration, non-manifold split with all steps, non-manifold vertex detection).

Default workload ("blobs129_refine4"): a 129^3 fp32 grid of 64 seeded Gaussian
blobs (sigma 3-12 cells) refined x4 to 513^3 samples = 512^3 cells, iso 0.4.
Metric: Mcells/s = processed cells / step time.  `value` is timed with the
input already resident in HBM; `e2e` goes through the C ABI from pinned host
memory (upload of the 129^3 input, then mdmc_run_to_host: the run with the whole mesh copied into
pinned host arrays, the copies overlapping the later stages).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--config NAME]

With --gpus N > 1 (launched under torch.distributed.run) every rank runs an
independent replica on its own grid (different seed); value = all ranks' cells
/ the slowest rank's time ("replicas only": the path has no exchange step).
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

PEAKS_FILE = ROOT / "MEASURED_PEAKS.json"
L2_FLUSH_BYTES = 256 << 20  # > 129 MB L2


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default 100 for this library, 10 CPU runs for --impl reference)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--config", default="blobs129_refine4")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-noise", action="store_true")
    ap.add_argument("--no-fit", action="store_true",
                    help="skip the 200 Adam steps of the sphere-to-torus fit (the differentiable workload)")
    args = ap.parse_args()
    if args.steps is None:
        # ~0.1 s of timed GPU work, long enough for the clock samples to land in it
        args.steps = 100 if args.impl == "ours" else 10
    return args


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def peaks():
    try:
        p = json.loads(PEAKS_FILE.read_text())
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled while the timed loop runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.dev = device_index
        self.proc = None
        self.lines = []

    INTERVAL_MS = 20

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", str(self.INTERVAL_MS)],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            # the timed steps start once the sampler is delivering
            t0 = time.time()
            while not self.lines and time.time() - t0 < 5.0 and self.proc.poll() is None:
                time.sleep(0.005)
            self.first = len(self.lines)
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            # one sample after the timed steps, so that they lie between samples
            n, t0 = len(self.lines), time.time()
            while len(self.lines) <= n and time.time() - t0 < 1.0 and self.proc.poll() is None:
                time.sleep(0.002)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = max(smax, float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm),
                "window": "nvidia-smi every %d ms from just before to just after the timed steps" % self.INTERVAL_MS}


def algorithmic_bytes(kernel, s):
    """Bytes a kernel must move to or from HBM, per launch (each datum once).
    Refined grids are evaluated on demand from the coarse input, so the passes
    over them read only the coarse samples (S_in)."""
    S_in, rows = s["samples_in"], s["rows"]
    S = s["samples_in"] if s["refined"] else s["samples"]
    A, V, Q = s["active"], s["dmc_vertices"], s["dmc_quads"]
    if kernel == "refine":  # coarse-cell pre-pass: coarse samples read, one bit per coarse cell written
        return 4 * S_in + S_in // 8
    words = s["mask_words"]
    if kernel == "count":  # grid read once; active-cell mask words and their first-cell offsets written
        return 4 * S + 8 * words
    if kernel == "emit":  # mask + offsets read; records and {contours, quads} counts written, counts scanned in place
        return 8 * words + 16 * A + 8 * A + 16 * A
    if kernel == "vertices":  # records read; positions + normals (24 B), the vertex pass's degree (4 B) and the
        # quad pass's starting flags (1 B) and smallest-outgoing-halfedge seed (4 B) written per vertex
        return 16 * A + (24 + 4 + 1 + 4) * V
    if kernel == "quads":  # read: each active cell's record (16 B) and the mask word and first-cell offset
        # that find it (8 B), each quad's owner (4 B); written: halfedges with twins (64 B), valences (4 B),
        # face first halfedge (4 B), attributes (2 B), output quad (16 B) per quad, and each vertex's
        # smallest outgoing halfedge (4 B)
        return (16 + 8) * A + 4 * Q + (64 + 4 + 4 + 2 + 16) * Q + 4 * V
    raise KeyError(kernel)


def survey_bytes(s):
    """Whole-step algorithmic bytes as the headline roofline defines them:
    input once, processed grid once, mesh out (positions + normals, quads,
    halfedges, faces, attributes, vertex maps and flags)."""
    V, Q = s["dmc_vertices"], s["dmc_quads"]
    return 4 * s["samples_in"] + 4 * s["samples"] + 24 * V + (16 + 64 + 4 + 2) * Q + 5 * V


def run_ours(args, rank, world, local):
    import torch

    import manifolddmc_gb300 as mdmc
    from manifolddmc_gb300.workloads import CONFIGS

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    desc, gen, iso, refine, pad = CONFIGS[args.config]
    vol = gen() if rank == 0 else gen(seed=100 + rank)  # replicas get their own grid
    dims_in = [vol.shape[2], vol.shape[1], vol.shape[0]]
    origin = np.zeros(3, np.float32)
    spacing = np.ones(3, np.float32)
    lib = mdmc.library()
    ctx = ctypes.c_void_p()
    assert lib.mdmc_create(ctypes.byref(ctx), None) == 0
    stream = torch.cuda.current_stream(dev)
    sh = ctypes.c_void_p(stream.cuda_stream)
    d_in = torch.from_numpy(vol).to(dev)
    dims_c = np.asarray(dims_in, np.int32)
    grid = mdmc.Grid()
    stats = mdmc.Stats()
    mesh = mdmc.Mesh()

    def check(st):
        if st != 0:
            raise RuntimeError(lib.mdmc_last_error(ctx).decode())

    def step(host=None, out=None):
        src, on_host = (host.data_ptr(), 1) if host is not None else (d_in.data_ptr(), 0)
        check(lib.mdmc_prepare_grid(ctx, ctypes.c_void_p(src), on_host, dims_c.ctypes.data_as(ctypes.c_void_p),
                                    origin.ctypes.data_as(ctypes.c_void_p), spacing.ctypes.data_as(ctypes.c_void_p),
                                    refine, int(pad), ctypes.byref(grid), sh))
        if out is None:
            st = lib.mdmc_run(ctx, ctypes.byref(grid), ctypes.c_float(iso), ctypes.byref(mesh), ctypes.byref(stats), sh)
        else:
            st = lib.mdmc_run_to_host(ctx, ctypes.byref(grid), ctypes.c_float(iso), ctypes.byref(out),
                                      ctypes.byref(mesh), ctypes.byref(stats), sh)
        if st not in (0, 4):
            check(st)

    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    # warm-up: every kernel and stage timed (event records on the stream), for
    # the per-kernel breakdown; the timed steps record only the dominant
    # kernel's pair, for the roofline (no stage times: ~1.7 us per record)
    kernels = ("refine", "count", "emit", "vertices", "quads")
    check(lib.mdmc_set_kernel_timing(ctx, mdmc.TIME_ALL))
    warm_ms = {k: [] for k in kernels}
    for i in range(max(args.warmup, 3)):
        flush.zero_()
        step()
        torch.cuda.synchronize(dev)
        if i:
            for k in kernels:
                warm_ms[k].append(getattr(stats, mdmc.KERNEL_TIMING[k][1]))
    breakdown = {k: float(np.mean(v)) for k, v in warm_ms.items()}
    dominant = max(breakdown, key=breakdown.get)
    check(lib.mdmc_set_kernel_timing(ctx, mdmc.KERNEL_TIMING[dominant][0]))
    cells = (grid.dims[0] - 1) * (grid.dims[1] - 1) * (grid.dims[2] - 1)
    samples = grid.dims[0] * grid.dims[1] * grid.dims[2]

    per_step, kernel_ms, launches = [], {dominant: []}, 0
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            flush.zero_()  # L2 flush between timed steps (outside the step's events)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step()
            e1.record(stream)
            e1.synchronize()
            per_step.append(e0.elapsed_time(e1))
            kernel_ms[dominant].append(getattr(stats, mdmc.KERNEL_TIMING[dominant][1]))
            launches += int(stats.kernel_launches)
    torch.cuda.synchronize(dev)
    if world > 1:
        torch.distributed.barrier()
    ms = float(np.mean(per_step))
    if world > 1:
        t = torch.tensor([ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    value = world * cells / (ms / 1e3) / 1e6

    sizes = {"samples_in": int(np.prod(dims_in)), "samples": samples, "rows": (grid.dims[1] - 1) * (grid.dims[2] - 1),
             "mask_words": (grid.dims[1] - 1) * (grid.dims[2] - 1) * ((grid.dims[0] - 1 + 31) // 32),
             "refined": bool(refine or pad),
             "active": int(stats.num_active_cells), "dmc_vertices": int(stats.num_dmc_vertices),
             "dmc_quads": int(stats.num_dmc_quads)}
    dominant_ms = float(np.mean(kernel_ms[dominant]))
    peak, peak_kind = peaks()
    ab = algorithmic_bytes(dominant, sizes)
    achieved = ab / (dominant_ms / 1e3) / 1e9
    traffic = None
    tf = ROOT / "profiles" / "traffic.json"
    if tf.exists():
        try:
            traffic = json.loads(tf.read_text()).get(args.config, {}).get(dominant)
        except Exception:
            traffic = None
    roofline = {"bound": "hbm", "kernel": dominant, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "peak_kind": peak_kind, "traffic": traffic,
                "algorithmic_bytes": ab, "kernel_ms_timed": round(dominant_ms, 4),
                "kernel_ms": {k: round(v, 4) for k, v in breakdown.items()},
                "kernel_ms_source": "warm-up steps with every kernel timed (the timed steps time only the dominant one)",
                "by_kernel": {k: {"ms": round(v, 4), "algorithmic_bytes": algorithmic_bytes(k, sizes),
                                  "achieved": round(algorithmic_bytes(k, sizes) / (v / 1e3) / 1e9, 1) if v > 0 else None,
                                  "frac": round(algorithmic_bytes(k, sizes) / (v / 1e3) / 1e9 / peak, 4) if v > 0 else None}
                              for k, v in breakdown.items()},
                "whole_step_bytes": survey_bytes(sizes),
                "whole_step_gbs": round(survey_bytes(sizes) / (ms / 1e3) / 1e9, 1),
                "whole_step_frac": round(survey_bytes(sizes) / (ms / 1e3) / 1e9 / peak, 4)}

    e2e = None
    if not args.no_e2e:
        check(lib.mdmc_set_kernel_timing(ctx, 0))  # the user's call: no kernel timing
        host_in = torch.from_numpy(vol).pin_memory()
        V, F, H = int(mesh.num_vertices), int(mesh.num_faces), int(mesh.num_halfedges)
        bufs = {"positions": torch.empty((V, 3), dtype=torch.float32).pin_memory(),
                "normals": torch.empty((V, 3), dtype=torch.float32).pin_memory(),
                "quads": torch.empty((F, 4), dtype=torch.int32).pin_memory(),
                "halfedges": torch.empty((H, 4), dtype=torch.int32).pin_memory(),
                "face_first": torch.empty(F, dtype=torch.int32).pin_memory(),
                "face_attr": torch.empty(F, dtype=torch.int16).pin_memory(),
                "vertex_he": torch.empty(V, dtype=torch.int32).pin_memory(),
                "vertex_flags": torch.empty(V, dtype=torch.uint8).pin_memory()}
        d2h = sum(b.numel() * b.element_size() for b in bufs.values())
        out = mdmc.HostMeshArrays(V, F, *[b.data_ptr() for b in bufs.values()])
        e2e_ms = []
        for i in range(args.steps + 1):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step(host=host_in, out=out)  # mdmc_run_to_host: the mesh lands in the pinned host arrays
            if int(mesh.num_vertices) != V or int(mesh.num_faces) != F:
                raise RuntimeError("mesh size changed between runs")
            e1.record(stream)
            e1.synchronize()
            if i:
                e2e_ms.append(e0.elapsed_time(e1))
        m = float(np.mean(e2e_ms))
        if world > 1:
            t = torch.tensor([m], device=dev)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            m = float(t.item())
        e2e = {"value": round(world * cells / (m / 1e3) / 1e6, 2), "unit": "Mcells/s", "ms_per_step": round(m, 4),
               "h2d_bytes_per_step": int(host_in.numel() * 4), "d2h_bytes_per_step": int(d2h)}

    noise = None
    if rank == 0 and not args.no_noise:
        noise = measure_noise(args, dev, stream, flush)
    batched = None
    if rank == 0 and not args.no_batch:
        batched = measure_batch(args, dev)
    adjoint = None
    if rank == 0 and not args.no_adjoint:
        adjoint = measure_adjoint(args, dev, stream, flush)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(args.config)
    lib.mdmc_destroy(ctx)
    if rank == 0:
        line = {
            "metric": "Mcells/s (DMC + manifold repair, 512^3-cell refined grid)",
            "value": round(value, 2), "unit": "Mcells/s", "n_gpus": world, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": round(ms, 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded numpy default_rng fields of the workload's shape; no dataset)",
            "config": workload_config(args.config),
            "parallelism": "replicas" if world > 1 else "single GPU",
            "l2": "flushed between timed steps (256 MB write)",
            "mesh": {"dmc_vertices": int(stats.num_dmc_vertices), "dmc_quads": int(stats.num_dmc_quads),
                     "final_vertices": int(mesh.num_vertices), "final_faces": int(mesh.num_faces),
                     "split_iterations": int(stats.split_iterations), "edges4": int(stats.num_edges4)},
            "roofline": roofline,
            "cpu_baseline": cpu,
            "e2e": e2e,
            "adjoint": adjoint,
            "batch": batched,
            "noise": noise,
            "gpu_launches": launches,
            "clocks": clocks.summary(),
        }
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


def measure_adjoint(args, dev, stream, flush):
    """Forward (surface iteration off) and forward + adjoint on the 128^3
    sphere SDF with the grid resident in HBM; CUDA events on the run's stream,
    L2 flushed before every timed pass.  The gradient's accuracy is checked by
    tests/test_gpu_adjoint.py, not here."""
    import torch

    import manifolddmc_gb300 as mdmc
    from manifolddmc_gb300.workloads import CONFIGS
    name = "sphere128_sdf"
    desc, gen, iso, refine, pad = CONFIGS[name]
    vol = gen()
    d_in = torch.from_numpy(vol).to(dev)
    dmc = mdmc.DualMarchingCubes(enable_surface_to_vertex_iteration=0)
    grid = mdmc.UniformGrid(d_in, [vol.shape[2], vol.shape[1], vol.shape[0]], stream=stream)
    dmc.run(iso, grid, stream=stream)
    V = int(dmc.mesh.num_vertices)
    dl = torch.randn((V, 3), device=dev, generator=torch.Generator(device=dev).manual_seed(0))
    dgrid = torch.empty_like(d_in)
    fwd, both = [], []
    for i in range(max(args.warmup, 3) + args.steps):
        for with_adjoint in (False, True):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            dmc.run(iso, grid, stream=stream)
            if with_adjoint:
                dmc.backward(dl, dgrid, stream=stream)
            e1.record(stream)
            e1.synchronize()
            if int(dmc.mesh.num_vertices) != V:
                raise RuntimeError("mesh size changed between runs")
            if i >= max(args.warmup, 3):
                (both if with_adjoint else fwd).append(e0.elapsed_time(e1))
    f, b = float(np.mean(fwd)), float(np.mean(both))
    # the adjoint accumulates with float atomics: the spread between two
    # backward passes of the same run, relative to the gradient's scale
    dmc.run(iso, grid, stream=stream)
    g1 = torch.empty_like(d_in)
    g2 = torch.empty_like(d_in)
    dmc.backward(dl, g1, stream=stream)
    dmc.backward(dl, g2, stream=stream)
    stream.synchronize()
    scale = float(g1.abs().max())
    spread = float((g1 - g2).abs().max()) / scale if scale > 0 else 0.0
    fit = None
    if not args.no_fit:
        # 200 Adam steps of forward + adjoint + one-sided Chamfer to 200k points
        # on a torus (R = 40, r = 15 cells) around the grid's centre; the
        # nearest points come from the library's point index
        from manifolddmc_gb300.optimize import fit_to_points
        from manifolddmc_gb300.workloads import torus_points
        c = (vol.shape[0] - 1) / 2.0
        pts = torch.from_numpy(torus_points(200000, 40.0, 15.0, (c, c, c), seed=5)).to(dev)
        fit_to_points(d_in, pts, iso, steps=5, lr=0.1)  # warm-up (buffers, index build path)
        split = {}
        _, losses, seconds = fit_to_points(d_in, pts, iso, steps=200, lr=0.1, timing=split)
        fit = {"steps": 200, "points": 200000, "seconds": round(seconds, 3), "ms_per_step": round(1e3 * seconds / 200, 3),
               "loss_first": round(losses[0], 4), "loss_last": round(losses[-1], 4),
               "step_split_ms": {k: round(v, 4) for k, v in split.items()},
               "note": "wall clock of the whole loop (Python, autograd and Adam included); step_split_ms from CUDA "
                       "events: DMC forward, nearest points + loss, adjoint backward + Adam"}
    return {"workload": name, "description": desc, "vertices": V, "fwd_ms": round(f, 4), "fit": fit,
            "fwd_adjoint_ms": round(b, 4), "ratio": round(b / f, 3),
            "run_to_run_spread": spread,
            "run_to_run_note": "max |g1 - g2| / max |g1| over two backward passes of one run (float atomics)",
            "gradient_check": "max |gpu - FP64 oracle| <= 1e-5 * max |FP64| (tests/test_gpu_adjoint.py); "
                              "FP64 oracle vs FP64 central differences h=1e-4 (tests/test_adjoint_oracle.py)"}


def measure_noise(args, dev, stream, flush):
    """The uniform-noise workloads, the worst case for ambiguous cells and
    non-manifold edges (every non-manifold edge goes through the splitter):
    256^3 samples (iso 0.5) and 513^3 samples = 512^3 cells, the headline cell
    count.  Grid resident in HBM, one mdmc_run per step with the stage times
    (CUDA events inside the library) and the step time (CUDA events around
    the call), L2 flushed before every step; the 512^3 grid needs about 150 GB
    of device memory and is skipped on smaller devices."""
    import torch

    import manifolddmc_gb300 as mdmc
    from manifolddmc_gb300.workloads import CONFIGS
    peak, peak_kind = peaks()
    out = {}
    for name, steps in (("noise256", 5), ("noise513", 3)):
        desc, gen, iso, refine, pad = CONFIGS[name]
        free, total = torch.cuda.mem_get_info(dev)
        if name == "noise513" and total < 200e9:
            out[name] = {"skipped": "needs a device with 200 GB or more"}
            continue
        vol = gen()
        d_in = torch.from_numpy(vol).to(dev)
        del vol
        dims = [d_in.shape[2], d_in.shape[1], d_in.shape[0]]
        dmc = mdmc.DualMarchingCubes()
        grid = mdmc.UniformGrid(d_in, dims, stream=stream)
        ms, stages = [], {"dmc": [], "halfedge": [], "repair": [], "detect": []}
        for i in range(1 + steps):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            dmc.run(iso, grid, stream=stream)
            e1.record(stream)
            e1.synchronize()
            if i:
                ms.append(e0.elapsed_time(e1))
                st = dmc.stats
                for k, f in (("dmc", "ms_dmc"), ("halfedge", "ms_halfedge"), ("repair", "ms_repair"),
                             ("detect", "ms_detect")):
                    stages[k].append(float(getattr(st, f)))
        st = dmc.stats
        cells = (dims[0] - 1) * (dims[1] - 1) * (dims[2] - 1)
        t = float(np.mean(ms))
        sizes = {"samples_in": dims[0] * dims[1] * dims[2], "samples": dims[0] * dims[1] * dims[2],
                 "dmc_vertices": int(st.num_dmc_vertices), "dmc_quads": int(st.num_dmc_quads)}
        b = survey_bytes(sizes)
        out[name] = {"description": desc, "steps": steps, "ms_per_step": round(t, 3),
                     "mcells_s": round(cells / (t / 1e3) / 1e6, 1),
                     "stage_ms": {k: round(float(np.mean(v)), 3) for k, v in stages.items()},
                     "whole_step_bytes": b, "whole_step_gbs": round(b / (t / 1e3) / 1e9, 1),
                     "whole_step_frac": round(b / (t / 1e3) / 1e9 / peak, 4), "peak_kind": peak_kind,
                     "dmc_vertices": int(st.num_dmc_vertices), "dmc_quads": int(st.num_dmc_quads),
                     "final_vertices": int(dmc.mesh.num_vertices), "final_faces": int(dmc.mesh.num_faces),
                     "split_iterations": int(st.split_iterations), "edges4": int(st.num_edges4),
                     "non_manifold_vertices": int(st.num_non_manifold_vertices)}
        del dmc, grid, d_in
        torch.cuda.synchronize(dev)
        torch.cuda.empty_cache()
    return out


def measure_batch(args, dev):
    """The batched workload (96 seeded grids of uneven dims, blobs or noise,
    iso in [0.3, 0.7]), resident in HBM: one mdmc_run_batch call (workers
    autotuned on the warm-up call) against 96 sequential mdmc_run calls on one
    context.  Both calls are synchronous; wall-clock over each whole call.
    Inputs total far more than L2."""
    import torch

    import manifolddmc_gb300 as mdmc
    from manifolddmc_gb300.workloads import batch_grids
    items = batch_grids(96, seed=4)
    tensors = [torch.from_numpy(v).to(dev) for v, _ in items]
    grids = [mdmc.UniformGrid(t, [t.shape[2], t.shape[1], t.shape[0]]) for t in tensors]
    isos = [iso for _, iso in items]
    cells = sum((g.grid.dims[0] - 1) * (g.grid.dims[1] - 1) * (g.grid.dims[2] - 1) for g in grids)
    torch.cuda.synchronize(dev)
    batch = mdmc.BatchedDualMarchingCubes(streams=0)
    batch.run(grids, isos)  # warm-up: grows the slots and picks the worker count
    single = mdmc.DualMarchingCubes()
    for g, iso in zip(grids, isos):
        single.run(iso, g)
    # each grid's stream time (the run's first to last CUDA event inside the
    # library, gaps while the host reads counts back included), summed
    busy = 0.0
    for g, iso in zip(grids, isos):
        single.run(iso, g)
        busy += float(single.stats.ms_total)
    seq, bat = [], []
    for _ in range(max(1, min(args.steps, 3))):
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        for g, iso in zip(grids, isos):
            single.run(iso, g)
        torch.cuda.synchronize(dev)
        seq.append(time.perf_counter() - t0)
        t0 = time.perf_counter()
        batch.run(grids, isos)
        torch.cuda.synchronize(dev)
        bat.append(time.perf_counter() - t0)
    s, b = float(np.mean(seq)), float(np.mean(bat))
    return {"workload": "96 grids, dims uniform in [24,192] per axis, 4-32 Gaussian blobs or uniform noise (50/50), "
                        "iso uniform in [0.3,0.7], seed 4",
            "cells": int(cells), "streams": batch.streams, "sequential_ms": round(1e3 * s, 3),
            "batch_ms": round(1e3 * b, 3), "speedup": round(s / b, 3), "gpu_busy_ms": round(busy, 3),
            "gpu_busy_note": "sum over the 96 grids of each run's stream time (ms_total: first to last CUDA event "
                             "of the run, including the short gaps while the host reads counts back)",
            "batch_mcells_s": round(cells / b / 1e6, 1), "sequential_mcells_s": round(cells / s / 1e6, 1)}


def workload_config(config):
    """The workload descriptor both arms print (inputs only, no results)."""
    from manifolddmc_gb300.workloads import CONFIGS
    desc, gen, iso, refine, pad = CONFIGS[config]
    shape = {"blobs64_pad": [64] * 3, "noise128": [128] * 3, "noise256": [256] * 3, "blobs129_refine4": [129] * 3, "blobs65_refine4": [65] * 3,
             "noise513": [513] * 3, "sphere128_sdf": [128] * 3}[config]
    proc = [d + (d - 1) * refine + (2 if pad else 0) for d in shape]
    return {"workload": config, "description": desc, "cells": (proc[0] - 1) * (proc[1] - 1) * (proc[2] - 1),
            "grid_in": shape, "grid_processed": proc, "iso": iso, "refinement": refine, "pad": bool(pad)}


def cpu_sample(config, fraction=1):
    """The workload for the CPU timings: the whole input (fraction 1), or its
    first 1/fraction of the z-planes, refined as in the GPU workload."""
    from manifolddmc_gb300.workloads import CONFIGS
    desc, gen, iso, refine, pad = CONFIGS[config]
    vol = gen()
    nz = vol.shape[0] if fraction <= 1 else max(2, vol.shape[0] // fraction + 1)
    sub = np.ascontiguousarray(vol[:nz])
    return sub, [sub.shape[2], sub.shape[1], sub.shape[0]], iso, refine, pad


def cpu_threads():
    """Host threads the oracle's OpenMP regions use (OMP_NUM_THREADS, else every core)."""
    env = os.environ.get("OMP_NUM_THREADS")
    return int(env) if env and env.isdigit() else (os.cpu_count() or 1)


def time_oracle(sub, dims, iso, refine, pad):
    """One run of the FP64 build of the oracle (refinement and the whole
    path in double) on the sample; returns (cells, seconds, result)."""
    sys.path.insert(0, str(ROOT / "tests"))
    from _support import oracle_run_refined
    o = np.zeros(3, np.float32)
    s = np.ones(3, np.float32)
    t0 = time.perf_counter()
    r = oracle_run_refined(sub.reshape(-1), dims, o, s, refine, pad, iso, f64=True)
    dt = time.perf_counter() - t0
    d = [x + (x - 1) * refine + (2 if pad else 0) for x in dims]
    cells = (d[0] - 1) * (d[1] - 1) * (d[2] - 1)
    return cells, dt, r


CPU_BASELINE_WHAT = ("the FP64 build of the CPU oracle (the C++ restatement of the reference's algorithm compiled "
                     "with double arithmetic; the reference has no CPU path): refinement and the DMC cell loop run "
                     "with OpenMP over z-slabs on %d host threads, the halfedge build, the repair and the fan "
                     "detection are serial")


def cpu_baseline(config):
    """Median of 5 runs after 1 warm-up, on the whole workload."""
    sub, dims, iso, refine, pad = cpu_sample(config)
    times = []
    cells = 0
    for i in range(6):
        cells, dt, _ = time_oracle(sub, dims, iso, refine, pad)
        if i:
            times.append(dt)
    dt = float(np.median(times))
    return {"value": round(cells / dt / 1e6, 3), "unit": "Mcells/s", "cores": cpu_threads(), "kind": "port",
            "sample": (CPU_BASELINE_WHAT % cpu_threads()) + "; the whole workload (%d of %d input z-planes, %d "
                      "cells), median of 5 runs after 1 warm-up: %.2f s (runs %s s)"
                      % (dims[2], dims[2], cells, dt, ", ".join("%.2f" % t for t in times))}


def run_reference(args, rank, world):
    if rank != 0:
        return
    sub, dims, iso, refine, pad = cpu_sample(args.config)
    times = []
    cells = 0
    for i in range(max(args.warmup, 3) + args.steps):
        cells, dt, _ = time_oracle(sub, dims, iso, refine, pad)
        if i >= max(args.warmup, 3):
            times.append(dt)
    ms = float(np.median(times)) * 1e3
    value = cells / (ms / 1e3) / 1e6
    sample = ((CPU_BASELINE_WHAT % cpu_threads()) + "; each step one run over the whole workload (%d input z-planes, "
              "%d cells); value from the median step" % (dims[2], cells))
    line = {"impl": "reference", "metric": "Mcells/s (DMC + manifold repair, 512^3-cell refined grid)",
            "value": round(value, 3), "unit": "Mcells/s", "n_gpus": world, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": round(ms, 2), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded numpy default_rng fields of the workload's shape; no dataset)",
            "config": workload_config(args.config), "parallelism": "%d host threads" % cpu_threads(),
            "cpu_baseline": {"value": round(value, 3), "unit": "Mcells/s", "cores": cpu_threads(), "kind": "port",
                             "sample": sample},
            "e2e": {"value": round(value, 3), "unit": "Mcells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world, local)


if __name__ == "__main__":
    main()
