#!/usr/bin/env python3
"""Benchmark of the GB300 skeleton hot path.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME] [--impl ours|reference]

Workloads (seeded synthetic inputs; shapes and value distributions of the
reference's examples):
  stencil_suite (default) -- the radius sweep and 3-D stencils: DM<float>
      8192^2 box mean at r = 1, 2, 4, 6, 8, 10 (one sweep each), DM<int> 8192^2
      Game of Life (200 steps), DC<float> 512^3 heat3D (100 steps). One step is
      one pass over all three parts. Metric: stencil GCUPS (cell updates / s).
  jacobi -- plain 2-D Jacobi, DM<float> 1024^2, 100 sweeps + FP64 residual.
  mapzipfold -- DA<float> 2^28 map/zip/fold(+) and DA<int> 2^28 mapIndex/fold(+).
      Metric: GB/s of algorithmic traffic.
  box / life / heat -- one part of the suite alone.

Prints one JSON line (rank 0). `value` is measured with device-resident inputs
(CUDA events on the library stream around K steps, max over ranks); `e2e` is
the same metric through the C ABI with host buffers, the host->device copy of
every step's inputs and the device->host copy of its results inside the timed
region. `roofline` is the dominant kernel's algorithmic bytes per launch over
its average launch time (events on the same stream) against the measured HBM
copy bandwidth. `cpu_baseline` is the CPU oracle (a restatement of the
reference's OpenMP loops) timed on a bounded sample on this host's cores.
--impl reference times that CPU implementation alone on the same workload.
"""
from __future__ import annotations

import argparse
import gc
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

HBM_FALLBACK_GBS = 6800.0


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return HBM_FALLBACK_GBS, "fallback"


# ---- distributed plumbing (replicas only: no data-path collective) ------------------
class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local_rank = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo")
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, v: float) -> float:
        if not self.pg:
            return v
        import torch
        t = torch.tensor([v], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def sum(self, v: float) -> float:
        if not self.pg:
            return v
        import torch
        t = torch.tensor([v], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


# ---- clocks sampled during the timed region ------------------------------------------
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()
        time.sleep(0.3)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return None
        time.sleep(0.15)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
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
            for nm, v in zip(names, parts[3:7]):
                if v.lower() in ("active", "1"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


# ---- timing helpers on the library stream -------------------------------------------
class Events:
    """CUDA events recorded on libmsl_gb300's stream (via torch's external-stream view)."""

    def __init__(self, abi):
        import torch
        self.torch = torch
        self.stream = torch.cuda.ExternalStream(abi.stream_handle())

    def record(self):
        e = self.torch.cuda.Event(enable_timing=True)
        e.record(self.stream)
        return e

    @staticmethod
    def ms(a, b) -> float:
        return a.elapsed_time(b)


def pinned(shape, dtype):
    import torch
    tdt = {np.dtype(np.float32): torch.float32, np.dtype(np.int32): torch.int32,
           np.dtype(np.float64): torch.float64, np.dtype(np.uint16): torch.int16}[np.dtype(dtype)]
    t = torch.empty(shape, dtype=tdt, pin_memory=True)
    return t, t.numpy().view(dtype)


# ---- workloads ------------------------------------------------------------------------
BOX_RADII = (1, 2, 4, 6, 8, 10)


class Part:
    """One stencil part of a workload: device buffers, host mirrors, step and oracle sample."""

    def __init__(self, name, updates, launches, bytes_per_launch, dtype):
        self.name, self.updates, self.launches = name, updates, launches
        self.bytes_per_launch, self.dtype = bytes_per_launch, dtype
        # one read and one write of the grid: what a launch that runs several
        # sweeps (temporal blocking) must move at least
        self.compulsory_bytes = bytes_per_launch
        self.ms = 0.0


class StencilSuite:
    name = "stencil_suite"
    metric = "stencil GCUPS"
    unit = "GCUPS"
    dtype = "f32+i32"

    def __init__(self, abi, parts=("box", "life", "heat"), life_steps=200, heat_steps=100, side=8192, cube=512):
        self.A = abi
        self.which = parts
        self.life_steps, self.heat_steps, self.side, self.cube = life_steps, heat_steps, side, cube
        self.parts = {}
        n2, n3 = side * side, cube ** 3
        if "box" in parts:
            self.parts["box"] = Part("box_mean_r1-10", n2 * len(BOX_RADII), len(BOX_RADII), 8 * n2, "f32")
        if "life" in parts:
            self.parts["life"] = Part("life", n2 * life_steps, life_steps, 8 * n2, "i32")
            self.parts["life"].compulsory_bytes = 8 * n2
        if "heat" in parts:
            self.parts["heat"] = Part("heat3d", n3 * heat_steps, heat_steps, 8 * n3, "f32")

    def config(self):
        c = {"workload": "stencil radius sweep + 3-D stencils (" + "+".join(p.name for p in self.parts.values()) + ")",
             "l2": "inputs larger than L2 (every grid >= 256 MiB)"}
        if "box" in self.parts:
            c["box"] = f"DM<float> {self.side}^2, U[0,255], mean over (2r+1)^2, r in {list(BOX_RADII)}, 1 sweep each"
        if "life" in self.parts:
            c["life"] = f"DM<int> {self.side}^2, Bernoulli(0.3), {self.life_steps} steps, dead border"
        if "heat" in self.parts:
            c["heat"] = f"DC<float> {self.cube}^3, U[0,1), 7-point heat3D, {self.heat_steps} steps, Dirichlet 0"
        return c

    def setup(self):
        from muesli4_gb300 import workloads as W
        A = self.A
        s, m = self.side, self.cube
        self.host_in, self.host_out, self.dev = {}, {}, {}
        if "box" in self.parts:
            img = W.blur_image(s, s, 42)
            t, h = pinned(img.shape, np.float32)
            h[...] = img
            self.host_in["box"] = (t, h)
            self.host_out["box"] = pinned(img.shape, np.float32)
            self.dev["box"] = (A.DeviceArray.from_host(img), A.DeviceArray(img.shape, np.float32))
        if "life" in self.parts:
            board = W.life_board(s, s, 42)
            t, h = pinned(board.shape, np.int32)
            h[...] = board
            self.host_in["life"] = (t, h)
            self.host_out["life"] = pinned(board.shape, np.int32)
            self.dev["life"] = [A.DeviceArray.from_host(board), A.DeviceArray(board.shape, np.int32)]
        if "heat" in self.parts:
            cube = W.heat_cube(m, m, m, 42)
            t, h = pinned(cube.shape, np.float32)
            h[...] = cube
            self.host_in["heat"] = (t, h)
            self.host_out["heat"] = pinned(cube.shape, np.float32)
            self.dev["heat"] = [A.DeviceArray.from_host(cube), A.DeviceArray(cube.shape, np.float32)]
        self.h2d = sum(h.nbytes for _, h in self.host_in.values())
        self.d2h = sum(h.nbytes for _, h in self.host_out.values())
        # The autotuner picks the temporal depth (sweeps per launch) for the
        # iterated 2-D part; its records are used by the timed iterate calls.
        self.tuned = {}
        if "heat" in self.parts:
            # heat3D runs `k` sweeps per launch (msl_set_stencil3d_depth): the
            # algorithmic bytes of a launch are those of its k sweeps, its
            # compulsory bytes one read and one write of the cube
            k = max(1, getattr(self, "heat_sweeps_per_launch", 1))
            p = self.parts["heat"]
            p.launches = heat_launches(self.heat_steps, k)
            p.bytes_per_launch = 8 * m ** 3 * self.heat_steps // p.launches
            p.sweeps_per_launch = k
            self.tuned["heat_sweeps_per_launch"] = k
        if "life" in self.parts:
            d = getattr(self, "fixed_depth", 0)
            if d <= 0:
                d, rate = A.autotune_stencil2d(A.MSL_ST2_LIFE, A.MSL_I32, s, s, 1, 64)
            self.tuned["life_temporal_depth"] = d
            p = self.parts["life"]
            p.launches = life_launches(self.life_steps, d)
            p.bytes_per_launch = 8 * s * s * self.life_steps // p.launches  # algorithmic, averaged over launches

    def updates(self):
        return sum(p.updates for p in self.parts.values())

    def run_part(self, k):
        """Enqueue one part on the library stream (no host synchronisation)."""
        A = self.A
        if k == "box":
            src, dst = self.dev["box"]
            for r in BOX_RADII:
                A.stencil2d(A.MSL_ST2_BOXMEAN, src, dst, r, 0.0)
        elif k == "life":
            a, b = self.dev["life"]
            last, _ = A.stencil2d_iterate(A.MSL_ST2_LIFE, a, b, 1, 0, self.life_steps, residual=False)
            if last is b:
                self.dev["life"] = [b, a]
        else:
            a, b = self.dev["heat"]
            last, _ = A.stencil3d_iterate(A.MSL_ST3_HEAT7, a, b, 1, 0.0, self.heat_steps, residual=False)
            if last is b:
                self.dev["heat"] = [b, a]

    def result_of(self, k):
        return self.dev[k][1] if k == "box" else self.dev[k][0]

    def step(self, ev=None, marks=None):
        """One pass over the parts on the device. With `ev`, records an event
        after each part into `marks`."""
        for k in ("box", "life", "heat"):
            if k in self.parts:
                self.run_part(k)
                if ev is not None:
                    marks.append((k, ev.record()))

    def e2e_step(self):
        """Host buffers in, host buffers out, through the C ABI, pipelined:
        every part's input goes up on an upload stream and its result comes
        down on a download stream, so transfers overlap the other parts'
        kernels (the library stream waits for each part's upload; each
        download waits for its part's kernels)."""
        import torch
        A = self.A
        if not hasattr(self, "_streams"):
            self._streams = (torch.cuda.Stream(), torch.cuda.Stream(), torch.cuda.ExternalStream(A.stream_handle()))
        up, down, lib = self._streams
        # the long heat3D part in the middle: only the first upload (box) and
        # the last download (Life), 256 MiB each, are not hidden behind kernels
        order = [k for k in ("box", "heat", "life") if k in self.parts]
        ev_up, ev_done = {}, {}
        for k in order:
            _, h = self.host_in[k]
            A.check(A.load().msl_upload_async(self.dev[k][0].ptr, h.ctypes.data, h.nbytes, up.cuda_stream),
                    "msl_upload_async")
            ev_up[k] = torch.cuda.Event()
            ev_up[k].record(up)
        for k in order:
            lib.wait_event(ev_up[k])
            self.run_part(k)
            ev_done[k] = torch.cuda.Event()
            ev_done[k].record(lib)
        for k in order:
            down.wait_event(ev_done[k])
            _, h = self.host_out[k]
            A.check(A.load().msl_download_async(h.ctypes.data, self.result_of(k).ptr, h.nbytes, down.cuda_stream),
                    "msl_download_async")
        down.synchronize()

    # CPU sample: per-part rates measured on bounded samples, combined in the
    # workload's own mix of cell updates.
    def cpu_sample(self, O, threads, min_seconds: float = 0.0):
        """Per-part CPU rates on bounded samples (repeated until min_seconds),
        combined in this workload's own mix of cell updates."""
        from muesli4_gb300 import workloads as W
        O.set_threads(threads)
        done = {k: 0.0 for k in self.parts}
        spent = {k: 0.0 for k in self.parts}
        desc = []
        img = W.blur_image(512, self.side, 42) if "box" in self.parts else None
        board = W.life_board(2048, self.side, 42) if "life" in self.parts else None
        cube = W.heat_cube(64, self.cube, self.cube, 42) if "heat" in self.parts else None
        if img is not None:
            desc.append(f"box r=1..10 on {img.shape[0]}x{self.side}")
        if board is not None:
            desc.append(f"life 4 steps on {board.shape[0]}x{self.side}")
        if cube is not None:
            desc.append(f"heat3d 4 steps on {cube.shape[0]}x{self.cube}x{self.cube}")
        t_begin = time.perf_counter()
        while True:
            if img is not None:
                for r in BOX_RADII:
                    t0 = time.perf_counter()
                    O.stencil2d(2, img, r, 0.0)
                    spent["box"] += time.perf_counter() - t0
                done["box"] += img.size * len(BOX_RADII)
            if board is not None:
                t0 = time.perf_counter()
                O.stencil2d_iterate(4, board, 1, 0, 4)
                spent["life"] += time.perf_counter() - t0
                done["life"] += 4 * board.size
            if cube is not None:
                t0 = time.perf_counter()
                O.stencil3d_iterate(0, cube, 1, 0.0, 4)
                spent["heat"] += time.perf_counter() - t0
                done["heat"] += 4 * cube.size
            if time.perf_counter() - t_begin >= min_seconds:
                break
        total_t = sum(self.parts[k].updates * spent[k] / done[k] for k in self.parts)
        return self.updates() / total_t / 1e9, "; ".join(desc) + f" ({time.perf_counter() - t_begin:.1f} s)"


class Jacobi:
    name = "jacobi"
    metric = "stencil GCUPS"
    unit = "GCUPS"
    dtype = "f32"

    def __init__(self, abi, side=1024, iters=100):
        self.A, self.side, self.iters = abi, side, iters
        self.parts = {"jacobi": Part("jacobi5", side * side * iters, iters, 8 * side * side, "f32")}

    def config(self):
        return {"workload": f"plain Jacobi DM<float> {self.side}^2, 5-point, {self.iters} sweeps + FP64 residual",
                "l2": "grid (8 MiB) is L2-resident: the HBM fraction is effective bandwidth"}

    def setup(self):
        from muesli4_gb300 import workloads as W
        A = self.A
        g = W.jacobi_grid(self.side, self.side, 42)
        t, h = pinned(g.shape, np.float32)
        h[...] = g
        self.host_in = {"jacobi": (t, h)}
        self.host_out = {"jacobi": pinned(g.shape, np.float32)}
        self.dev = {"jacobi": [A.DeviceArray.from_host(g), A.DeviceArray(g.shape, np.float32)]}
        self.h2d, self.d2h = h.nbytes, h.nbytes + 8
        self.residual = None
        d = getattr(self, "fixed_depth", 0)
        rows = getattr(self, "fixed_tile_rows", 0) or 32
        if d <= 0:
            d, rows, _ = A.autotune_stencil2d_shape(A.MSL_ST2_JACOBI5, A.MSL_F32, self.side, self.side, 1, self.iters)
        tiles = ((self.side + 63) // 64) * ((self.side + rows - 1) // rows)
        self.tuned = {"temporal_depth": d, "tile": f"64x{rows}" if d > 1 else "64x32 (one sweep per launch)",
                      "threads_per_cta": rows * 8 if d > 1 else 256, "ctas": tiles}
        p = self.parts["jacobi"]
        p.launches = (self.iters + d - 1) // d
        p.bytes_per_launch = 8 * self.side * self.side * self.iters // p.launches
        p.compulsory_bytes = 8 * self.side * self.side

    def updates(self):
        return self.parts["jacobi"].updates

    def step(self, ev=None, marks=None):
        A = self.A
        a, b = self.dev["jacobi"]
        last, self.residual = A.stencil2d_iterate(A.MSL_ST2_JACOBI5, a, b, 1, 0.0, self.iters, residual=True)
        if ev is not None:
            marks.append(("jacobi", ev.record()))

    def e2e_step(self):
        A = self.A
        _, h = self.host_in["jacobi"]
        a, b = self.dev["jacobi"]
        A.check(A.load().msl_upload(a.ptr, h.ctypes.data, h.nbytes), "msl_upload")
        last, self.residual = A.stencil2d_iterate(A.MSL_ST2_JACOBI5, a, b, 1, 0.0, self.iters, residual=True)
        _, ho = self.host_out["jacobi"]
        A.check(A.load().msl_download(ho.ctypes.data, last.ptr, ho.nbytes), "msl_download")

    def cpu_sample(self, O, threads, min_seconds: float = 0.0):
        from muesli4_gb300 import workloads as W
        O.set_threads(threads)
        g = W.jacobi_grid(self.side, self.side, 42)
        t0 = time.perf_counter()
        O.stencil2d_iterate(0, g, 1, 0.0, 20)
        return 20 * self.side * self.side / (time.perf_counter() - t0) / 1e9, f"20 sweeps on {self.side}^2"


class MapZipFold:
    name = "mapzipfold"
    metric = "map/zip/fold GB/s"
    unit = "GB/s"
    dtype = "f32+i32"

    def __init__(self, abi, n=1 << 28):
        self.A, self.n = abi, n
        b = 4 * n
        # algorithmic bytes: map 8 B/elem, zip 12, fold 4; int mapIndex 8, fold 4
        self.parts = {"map": Part("map_f32", n, 1, 2 * b, "f32"), "zip": Part("zip_f32", n, 1, 3 * b, "f32"),
                      "fold": Part("fold_f32", n, 1, b, "f32"), "mapindex": Part("mapindex_i32", n, 1, 2 * b, "i32"),
                      "ifold": Part("fold_i32", n, 1, b, "i32")}

    def config(self):
        return {"workload": f"DA<float> {self.n} map 2.5x+1 / zip a*b+a / fold(+); DA<int> mapIndex x^(i&1023) / fold(+)",
                "l2": "inputs larger than L2 (1 GiB arrays)"}

    def bytes(self):
        return sum(p.bytes_per_launch for p in self.parts.values())

    def setup(self):
        from muesli4_gb300 import workloads as W
        A = self.A
        a = W.uniform_f32(self.n, -1, 1, 42)
        b = W.uniform_f32(self.n, -1, 1, 43)
        x = W.uniform_i32(self.n, 0, 1000, 44)
        self.host_in = {}
        for k, v in (("a", a), ("b", b), ("x", x)):
            t, h = pinned(v.shape, v.dtype)
            h[...] = v
            self.host_in[k] = (t, h)
        self.host_out = {"z": pinned(a.shape, np.float32), "y": pinned(x.shape, np.int32)}
        self.dev = {"a": A.DeviceArray.from_host(a), "b": A.DeviceArray.from_host(b), "x": A.DeviceArray.from_host(x),
                    "m": A.DeviceArray(a.shape, np.float32), "z": A.DeviceArray(a.shape, np.float32),
                    "y": A.DeviceArray(x.shape, np.int32)}
        self.h2d = sum(h.nbytes for _, h in self.host_in.values())
        self.d2h = sum(h.nbytes for _, h in self.host_out.values()) + 8

    def updates(self):
        return self.bytes()

    def step(self, ev=None, marks=None):
        A, d = self.A, self.dev
        A.map(A.MSL_MAP_AFFINE, d["a"], d["m"], (2.5, 1.0))
        if ev is not None:
            marks.append(("map", ev.record()))
        A.zip(A.MSL_ZIP_MULADD, d["m"], d["b"], d["z"])
        if ev is not None:
            marks.append(("zip", ev.record()))
        self.fsum = A.fold(A.MSL_FOLD_SUM, d["z"])
        if ev is not None:
            marks.append(("fold", ev.record()))
        A.map_index(A.MSL_IDX_XOR_MASK, d["x"], d["y"], (1023,))
        if ev is not None:
            marks.append(("mapindex", ev.record()))
        self.isum = A.fold(A.MSL_FOLD_SUM, d["y"])
        if ev is not None:
            marks.append(("ifold", ev.record()))

    def e2e_step(self):
        A, d = self.A, self.dev
        for k in ("a", "b", "x"):
            _, h = self.host_in[k]
            A.check(A.load().msl_upload(d[k].ptr, h.ctypes.data, h.nbytes), "msl_upload")
        self.step()
        for k in ("z", "y"):
            _, h = self.host_out[k]
            A.check(A.load().msl_download(h.ctypes.data, d[k].ptr, h.nbytes), "msl_download")

    def fold_kernel_rates(self, ev, launches=10):
        """GB/s of the fold kernel alone: msl_fold returns its value to the
        host, so its part time above includes the host's wait for the kernel;
        the same kernel through the asynchronous msl_fold_noalloc, timed with
        CUDA events on the library stream, shows the device time."""
        import ctypes
        A, d = self.A, self.dev
        res = A.DeviceArray((1,), np.float64)
        out = {}
        st = ctypes.c_void_p(A.stream_handle())
        for key, arr, code in (("fold_f32", d["z"], A.MSL_F32), ("fold_i32", d["y"], A.MSL_I32)):
            for _ in range(2):
                A.check(A.load().msl_fold_noalloc(code, A.MSL_FOLD_SUM, arr.ptr, self.n, res.ptr, st))
            A.sync()
            e0 = ev.record()
            for _ in range(launches):
                A.check(A.load().msl_fold_noalloc(code, A.MSL_FOLD_SUM, arr.ptr, self.n, res.ptr, st))
            e1 = ev.record()
            A.sync()
            t = ev.ms(e0, e1) / 1e3 / launches
            out[key] = {"us_per_launch": t * 1e6, "GB_per_s": 4 * self.n / t / 1e9}
        return out

    def cpu_sample(self, O, threads, min_seconds: float = 0.0):
        from muesli4_gb300 import workloads as W
        n = 1 << 25
        a = W.uniform_f32(n, -1, 1, 42)
        b = W.uniform_f32(n, -1, 1, 43)
        x = W.uniform_i32(n, 0, 1000, 44)
        O.set_threads(threads)
        t = {}
        t0 = time.perf_counter(); m = O.map(0, a, (2.5, 1.0)); t["map"] = time.perf_counter() - t0
        t0 = time.perf_counter(); z = O.zip(3, m, b); t["zip"] = time.perf_counter() - t0
        t0 = time.perf_counter(); y = O.map_index(2, x, (1023,)); t["mapindex"] = time.perf_counter() - t0
        O.set_threads(1)  # the reference's parallel fold is a data race; its correct form is sequential
        t0 = time.perf_counter(); O.fold(0, z); t["fold"] = time.perf_counter() - t0
        t0 = time.perf_counter(); O.fold(0, y); t["ifold"] = time.perf_counter() - t0
        O.set_threads(threads)
        scale = self.n / n
        total_t = sum(v * scale for v in t.values())
        return self.bytes() / total_t / 1e9, f"2^25-element arrays ({threads} threads; folds on 1 thread)"


def side_class(n):
    return "64-127" if n < 128 else "128-255" if n < 256 else "256-511" if n < 512 else "512-1023" if n < 1024 \
        else "1024-2048"


class BatchSolve:
    """Batched plain-Jacobi solves: 256 grids, sides log-uniform in [64, 2048]
    rounded to multiples of 32 (seed 7), initialised as the plain-Jacobi grid
    (per-grid seed 7000 + g), iterated to an FP64 residual <= 1e-4 or the
    sweep cap. One step = one batched solve of all grids from their initial
    values. Metric: solves per second, counting only the grids that reached
    the residual (a grid stopped by the cap is not a solve).

    storage "f32": FP32 iterates, residual max |u_k - u_(k-1)| every 100
    sweeps. storage "bf16dc": FP32 solution with bfloat16-stored corrections
    (defect correction), residual max |J(u) - u| every 20-sweep cycle."""
    metric = "batched Jacobi solves/s"
    unit = "solves/s"

    def __init__(self, abi, count=256, storage="f32", cap=20_000, tol=1e-4, check_every=None):
        self.A = abi
        self.count, self.storage, self.cap, self.tol = count, storage, cap, tol
        self.check_every = check_every or (100 if storage == "f32" else 20)
        self.dtype = "f32" if storage == "f32" else "bf16-storage corrections/f32-compute (defect correction)"
        rng = np.random.default_rng(7)
        u = rng.uniform(np.log(64), np.log(2048), count)
        self.sides = [int(min(2048, max(64, round(np.exp(v) / 32) * 32))) for v in u]
        self.parts = {}

    @property
    def code(self):
        return self.A.MSL_F32 if self.storage == "f32" else self.A.MSL_BF16_DC

    def config(self):
        how = ("FP32 iterates, residual max|u_k - u_(k-1)|" if self.storage == "f32" else
               "FP32 solution + bfloat16 corrections (defect correction), residual max|J(u) - u|")
        return {"workload": f"{self.count} plain-Jacobi grids, sides log-uniform [64, 2048] (multiple of 32, seed 7), "
                            f"{how} in FP64 every {self.check_every} sweeps, tol {self.tol}, cap {self.cap} sweeps; "
                            f"solves/s counts only grids that reached the tolerance",
                "cells": int(sum(n * n for n in self.sides)), "sweep_cap": self.cap, "check_every": self.check_every}

    def setup(self):
        from muesli4_gb300 import workloads as W
        A = self.A
        self.grids = [W.jacobi_grid(n, n, 7000 + g) for g, n in enumerate(self.sides)]
        self.batch = A.Batch([(n, n) for n in self.sides], storage=self.code)
        self.info = self.batch.info()
        self.load_all()
        tuned_dtype = A.MSL_F32 if self.storage == "f32" else A.MSL_BF16
        self.depth, _ = A.autotune_stencil2d(A.MSL_ST2_JACOBI5, tuned_dtype, 1024, 1024, 1, 100)
        if self.storage == "f32":
            while self.check_every % self.depth:
                self.depth -= 1
        self.tuned = {"temporal_depth": self.depth, "resident_grids": self.info["resident"],
                      "worklist_tiles": self.info["tiles"]}
        self.h2d = sum(g.nbytes for g in self.grids)
        self.d2h = self.h2d

    def updates(self):
        return self.count

    def load_all(self):
        for i, g in enumerate(self.grids):
            self.batch.set_grid(i, g)

    def solve(self, batch, cap=None):
        batch.solve(self.tol, cap or self.cap, self.check_every, self.depth)

    def step(self, ev=None, marks=None):
        self.batch.reset()  # initial values from their device copies
        self.solve(self.batch)

    def e2e_step(self):
        self.load_all()
        self.solve(self.batch)
        self.results = [self.batch.get_grid(i) for i in range(self.count)]

    def summary(self):
        res = [self.batch.get_grid(i) for i in range(self.count)]
        iters = [r[1] for r in res]
        conv = [r[2] <= self.tol for r in res]
        sweeps = sum(it * n * n for it, n in zip(iters, self.sides))
        by_side = {}
        for n, c in zip(self.sides, conv):
            k = side_class(n)
            by_side.setdefault(k, [0, 0])
            by_side[k][0] += int(c)
            by_side[k][1] += 1
        return res, {"converged": int(sum(conv)), "count": self.count, "sweep_cap": self.cap,
                     "converged_by_side": {k: f"{a}/{b}" for k, (a, b) in sorted(by_side.items())},
                     "max_sweeps": int(max(iters)), "median_sweeps": float(np.median(iters)),
                     "cell_updates": int(sweeps)}

    def plain_seconds(self):
        """The one-grid-at-a-time GPU path over every grid: FP32 through the
        stencil skeleton (msl_stencil2d_iterate, a residual check every
        check_every sweeps), defect correction as a batch of one grid. Returns
        the summed solve time (allocation and upload outside the timing)."""
        A = self.A
        t = 0.0
        self.plain_by_side = {}
        for g, n in enumerate(self.sides):
            t_before = t
            if self.storage == "f32":
                a, b = A.DeviceArray.from_host(self.grids[g]), A.DeviceArray((n, n), np.float32)
                A.sync()
                t0 = time.perf_counter()
                A.solve_plain(A.MSL_ST2_JACOBI5, a, b, self.tol, self.cap, self.check_every)
                A.sync()
                t += time.perf_counter() - t0
                del a, b
            else:
                one = A.Batch([(n, n)], storage=self.code)
                one.set_grid(0, self.grids[g])
                A.sync()
                t0 = time.perf_counter()
                self.solve(one)
                A.sync()
                t += time.perf_counter() - t0
                one.close()
            k = side_class(n)
            self.plain_by_side[k] = self.plain_by_side.get(k, 0.0) + (t - t_before)
        return t

    def fp64_errors(self, results):
        """Every grid's max |u - u64| against FP64 Jacobi sweeps of the same
        count, computed on the GPU (msl_stencil2d_iterate in FP64)."""
        A = self.A
        errs = []
        for g, n in enumerate(self.sides):
            got, it, _ = results[g]
            a = A.DeviceArray.from_host(self.grids[g].astype(np.float64))
            b = A.DeviceArray((n, n), np.float64)
            last, _ = A.stencil2d_iterate(A.MSL_ST2_JACOBI5, a, b, 1, 0.0, int(it), residual=False) if it else (a, None)
            errs.append(float(np.max(np.abs(got.astype(np.float64) - last.download()))))
            del a, b
        return errs

    def cpu_sample(self, O, threads, min_seconds: float = 0.0):
        return None, "not measured"


WORKLOADS = {
    "stencil_suite": lambda A: StencilSuite(A),
    "box": lambda A: StencilSuite(A, parts=("box",)),
    "life": lambda A: StencilSuite(A, parts=("life",)),
    "heat": lambda A: StencilSuite(A, parts=("heat",)),
    "jacobi": lambda A: Jacobi(A),
    "mapzipfold": lambda A: MapZipFold(A),
    "batch": lambda A: BatchSolve(A),
    "batch_bf16": lambda A: BatchSolve(A, storage="bf16dc"),
}


def value_of(w, seconds: float) -> float:
    return w.updates() / seconds / 1e9


def cpu_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def run_reference(args, dist: Dist):
    """Reference arm: the CPU implementation of the path (the oracle, a
    restatement of the reference's OpenMP loops) on this host's cores."""
    if dist.rank != 0:
        return
    from oracle import pyoracle as O
    O.build()
    w = WORKLOADS[args.workload](None)
    threads = cpu_threads()
    vals = []
    for i in range(args.warmup + args.steps):
        v, sample = w.cpu_sample(O, threads)
        if i >= args.warmup:
            vals.append(v)
    v = statistics.median(vals)
    line = {"metric": w.metric, "value": v, "unit": w.unit, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": w.dtype, "data": "synthetic", "impl": "reference",
            "config": w.config() if hasattr(w, "config") else {"workload": args.workload},
            "cpu_baseline": {"value": v, "unit": w.unit, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": w.unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def serve_requests(count: int, seed: int = 11):
    """Request stream of the served-solves workload: half 2-D plain-Jacobi
    grids n x n with n log-uniform in [64, 4096], half 3-D heat cubes m^3 with
    m log-uniform in [32, 256]; U[0,1) initial values from a per-request seed."""
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(count):
        if rng.random() < 0.5:
            n = int(round(np.exp(rng.uniform(np.log(64), np.log(4096)))))
            reqs.append(("2d", (n, n), seed * 100000 + i))
        else:
            m = int(round(np.exp(rng.uniform(np.log(32), np.log(256)))))
            reqs.append(("3d", (m, m, m), seed * 100000 + i))
    return reqs


def run_serve(args, dist: Dist):
    """Served stencil solves (Jacobi and heat3D requests of mixed sizes): Poisson
    arrivals at rates swept around the plain path's capacity; p50/p99 latency
    and solves/s of the continuously batching server against the plain
    one-request-at-a-time GPU path fed the same arrivals (a FIFO queue served
    for real in the same process: each request waits for its arrival time and
    for the requests before it, then runs alone through the stencil skeleton)."""
    from muesli4_gb300 import abi as A
    A.init(dist.local_rank)
    tol, cap, check = 1e-4, 5000, 100
    reqs = serve_requests(args.serve_requests)
    cache = {}

    def init_of(i):
        if i not in cache:
            kind, shape, sd = reqs[i]
            cache[i] = np.random.default_rng(sd).random(shape, dtype=np.float32)
        return cache[i]

    # The autotuner picks the 2-D launch shape per grid-size class; the plain
    # path and the server both use its records.
    tuned = {}
    for c in range(12, 25):  # every grid-size class of the 2-D requests (64^2 .. 4096^2 cells)
        n = int(round(2 ** (c / 2)))
        d, rows, _ = A.autotune_stencil2d_shape(A.MSL_ST2_JACOBI5, A.MSL_F32, n, n, 1, 100)
        tuned[n] = f"depth {d}, 64x{rows}"

    def plain_solve(i):
        x = init_of(i)
        kind = A.MSL_ST3_HEAT7 if x.ndim == 3 else A.MSL_ST2_JACOBI5
        a, b = A.DeviceArray.from_host(x), A.DeviceArray(x.shape, np.float32)
        out, _, _ = A.solve_plain(kind, a, b, tol, cap, check)
        out.download()

    # plain capacity: service time of a sample of requests, one at a time
    rng = np.random.default_rng(5)
    sample = sorted(rng.choice(len(reqs), size=min(args.serve_plain_sample, len(reqs)), replace=False).tolist())
    t0 = time.perf_counter()
    for i in sample:
        plain_solve(i)
    plain_capacity = len(sample) / (time.perf_counter() - t0)

    def plain_queue(arrivals):
        """The plain path served for real: FIFO, one request at a time."""
        t0, lat = time.perf_counter(), []
        for i, a in enumerate(arrivals):
            now = time.perf_counter() - t0
            if a > now:
                time.sleep(a - now)
            plain_solve(i)
            lat.append(time.perf_counter() - t0 - a)
        return len(arrivals) / (time.perf_counter() - t0), lat

    sweep = []
    for factor in args.serve_rates:
        lam = factor * plain_capacity
        arr = np.cumsum(np.random.default_rng(11).exponential(1.0 / lam, len(reqs)))
        arr -= arr[0]
        srv = A.Server(hbm_budget=120 << 30, tol=tol, max_iters=cap, check_every=check)
        t0 = time.perf_counter()
        ids = []
        for i, a in enumerate(arr):
            now = time.perf_counter() - t0
            if a > now:
                time.sleep(a - now)
            ids.append(srv.submit(init_of(i)))
        lat, queued, sweeps = [], [], 0
        for rid in ids:
            srv.wait(rid, -1.0)
            _, it, _, l, q = srv.result(rid)
            lat.append(l)
            queued.append(q)
            sweeps += it
            srv.release(rid)
        wall = time.perf_counter() - t0
        st = srv.stats()
        srv.stop()
        p_rate, p_lat = plain_queue(arr)
        sweep.append({"rate_factor": factor, "offered_per_s": lam, "served_solves_per_s": len(reqs) / wall,
                      "served_p50_s": float(np.percentile(lat, 50)), "served_p99_s": float(np.percentile(lat, 99)),
                      "served_queue_p99_s": float(np.percentile(queued, 99)), "intervals": st["intervals"],
                      "plain_solves_per_s": p_rate, "plain_p50_s": float(np.percentile(p_lat, 50)),
                      "plain_p99_s": float(np.percentile(p_lat, 99))})
        print(json.dumps(sweep[-1]), file=sys.stderr, flush=True)
    top = sweep[-1]
    if dist.rank == 0:
        line = {"metric": "served stencil solves/s", "value": top["served_solves_per_s"], "unit": "solves/s",
                "n_gpus": dist.world, "steps": 1, "warmup": 0, "ms_per_step": None, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": f"{len(reqs)} requests: half 2-D Jacobi n^2 (n log-uniform [64,4096]), half "
                                       f"3-D heat m^3 (m log-uniform [32,256]); U[0,1) init; residual <= {tol} "
                                       f"every {check} sweeps or {cap} sweeps; HBM budget 120 GB; Poisson arrivals",
                           "plain_capacity_per_s": plain_capacity, "plain_capacity_sample": len(sample),
                           "plain_path": "served for real, FIFO, same arrivals",
                           "jacobi_launch_shape_by_side": tuned},
                "sweep": sweep, "served_over_plain_at_top_rate": top["served_solves_per_s"] / top["plain_solves_per_s"]}
        print(json.dumps(line), flush=True)


def run_batch(args, dist: Dist):
    """Batched solves (configs 3): timed batched solves, then -- outside the
    timed region -- the end-to-end solve with host grids, the plain path over
    every grid and every grid's FP64 error."""
    from muesli4_gb300 import abi as A
    A.init(dist.local_rank)
    w = WORKLOADS[args.workload](A)
    if args.batch_cap or args.batch_grids:
        cap = args.batch_cap or w.cap
        w.__init__(A, count=args.batch_grids or w.count, storage=w.storage,
                   cap=max(w.check_every, cap // w.check_every * w.check_every))
    w.setup()
    if args.temporal_depth > 0:  # a fixed depth instead of the autotuner's
        w.depth = args.temporal_depth
        w.tuned["temporal_depth"] = w.depth
    ev = Events(A)
    # Warm-up: short solves (a tenth of the cap) so that every kernel and the
    # round graph have run before the timed solves.
    for _ in range(args.warmup):
        w.batch.reset()
        w.solve(w.batch, max(w.check_every, w.cap // 10 // w.check_every * w.check_every))
    A.sync()
    dist.barrier()
    sampler = ClockSampler(dist.local_rank)
    sampler.start()
    launches0 = A.launch_count()
    e0 = ev.record()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        w.step()
    e1 = ev.record()
    A.sync()
    wall = time.perf_counter() - t0
    clocks = sampler.stop()
    launches = A.launch_count() - launches0
    dev_s = max(ev.ms(e0, e1) / 1e3, 1e-9)
    t_max = dist.max(max(dev_s, wall))
    results, summ = w.summary()
    solved = summ["converged"]
    value = dist.sum(solved * args.steps) / t_max
    # end to end: host grids in, results out
    t0 = time.perf_counter()
    w.e2e_step()
    A.sync()
    e2e_s = dist.max(time.perf_counter() - t0)
    plain_s = w.plain_seconds() if not args.batch_timing_only else float("nan")
    errs = w.fp64_errors(results) if not args.batch_timing_only else [float("nan")]
    if dist.rank == 0:
        gcups = summ["cell_updates"] / (t_max / args.steps) / 1e9
        plain_rate = solved / plain_s
        line = {
            "metric": w.metric, "value": value, "unit": w.unit, "n_gpus": dist.world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_max * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": w.dtype, "data": "synthetic",
            "config": dict(w.config(), parallelism=f"replicas x{dist.world}", **w.tuned,
                           warmup_note="warm-up solves use a tenth of the sweep cap"),
            "solved": f"{solved}/{w.count}",
            "e2e": {"value": solved / e2e_s, "unit": w.unit, "h2d_bytes_per_step": w.h2d, "d2h_bytes_per_step": w.d2h},
            "plain_path": {"value": plain_rate, "unit": w.unit, "seconds_all_grids": plain_s,
                           "seconds_by_side": getattr(w, "plain_by_side", None),
                           "grids": "all, one at a time", "batched_over_plain": value / plain_rate},
            "convergence": summ, "effective_GCUPS": gcups,
            "max_error_vs_fp64": {"grids": f"all {w.count}, FP64 Jacobi of the same sweep count on the GPU",
                                  "max_abs": max(errs), "median_abs": float(np.median(errs)),
                                  "max_abs_converged": max([e for e, r in zip(errs, results) if r[2] <= w.tol],
                                                           default=None)},
            "gpu_launches": launches, "clocks": clocks,
        }
        print(json.dumps(line), flush=True)


def heat_launches(steps, sweeps_per_launch):
    """Launches of a heat3D iteration: `sweeps_per_launch` sweeps per launch
    (the z-marching kernel's two), an odd last sweep on its own."""
    k = max(1, sweeps_per_launch)
    return steps // k + steps % k


def life_launches(steps, depth):
    """Launches of a Life iteration on a width that is a multiple of 4: one
    generation cell by cell, then `depth` packed generations per launch."""
    return 1 + (steps - 1 + depth - 1) // depth


DRAM_TRAFFIC_PER_LAUNCH = {
    "heat3d": 1090.23e6,         # profiles/heat7_zmarch_512.md (two sweeps of 512^3 per launch)
    "heat3d/1": 1026.96e6,       # profiles/heat7_stencil3d_512.md (one sweep of 512^3)
    "life": 479.4e6,             # profiles/life_bits_stencil2d_8192.md (32 generations of 8192^2)
    "box_mean_r1-10": 495.08e6,  # profiles/boxmean_r10_box2d_pair_8192.md (r = 10)
}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--workload", default="stencil_suite", choices=sorted(WORKLOADS) + ["serve"])
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--batch-cap", type=int, default=0, help="sweep cap of the batch workloads")
    ap.add_argument("--batch-grids", type=int, default=0, help="number of grids of the batch workloads")
    ap.add_argument("--batch-timing-only", action="store_true",
                    help="batch workloads: skip the plain path and the FP64 errors (for sweeps of settings)")
    ap.add_argument("--serve-requests", type=int, default=400, help="requests of the serve workload (the full stream: 10000)")
    ap.add_argument("--serve-plain-sample", type=int, default=40)
    ap.add_argument("--serve-rates", type=float, nargs="+", default=[0.25, 0.5, 1.0, 2.0])
    ap.add_argument("--temporal-depth", type=int, default=0,
                    help="sweeps per launch of the iterated 2-D stencils (0: the autotuner's choice)")
    ap.add_argument("--tile-rows", type=int, default=0, choices=[0, 16, 32, 64],
                    help="tile height of the 2-D temporal-blocking kernel with --temporal-depth (0: 32)")
    ap.add_argument("--stencil3d-depth", type=int, default=2, choices=[1, 2],
                    help="heat3D sweeps per launch: 2 the z-marching kernel (default), 1 one sweep")
    ap.add_argument("--stencil3d-persistent", type=int, default=-1, choices=[-1, 0, 1],
                    help="3-D stencil kernel: 1 persistent, 0 one CTA per block, -1 library default")
    ap.add_argument("--elements", type=int, default=0,
                    help="array length of the mapzipfold workload (default 2^28; smaller for profiler captures)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    dist = Dist()
    if args.impl == "reference":
        run_reference(args, dist)
        dist.close()
        return

    if args.workload.startswith("batch"):
        run_batch(args, dist)
        dist.close()
        return
    if args.workload == "serve":
        run_serve(args, dist)
        dist.close()
        return

    from muesli4_gb300 import abi as A
    A.init(dist.local_rank)
    A.set_stencil3d_persistent(args.stencil3d_persistent)
    A.set_stencil3d_depth(args.stencil3d_depth)
    w = MapZipFold(A, args.elements) if args.workload == "mapzipfold" and args.elements > 0 \
        else WORKLOADS[args.workload](A)
    w.fixed_depth = args.temporal_depth  # > 0: no autotuning of the Life depth
    w.fixed_tile_rows = args.tile_rows
    w.heat_sweeps_per_launch = args.stencil3d_depth
    w.setup()
    if args.temporal_depth > 0:  # after setup: overrides the autotuner's record
        A.set_temporal_depth(args.temporal_depth)
        if args.tile_rows:
            A.set_tile_rows(args.tile_rows)
    ev = Events(A)
    for _ in range(args.warmup):
        w.step()
    A.sync()

    # ---- device-resident timed region ----
    # (the host's garbage collector stays off inside both timed regions: a
    # collection pass would be host noise, not the library's time)
    gc.collect()
    gc.disable()
    dist.barrier()
    A.sync()
    sampler = ClockSampler(dist.local_rank)
    sampler.start()
    launches0 = A.launch_count()
    step_marks = []
    e0 = ev.record()
    for _ in range(args.steps):
        start, marks = ev.record(), []
        w.step(ev, marks)
        step_marks.append((start, marks))
    e1 = ev.record()
    A.sync()
    launches = A.launch_count() - launches0
    clocks = sampler.stop()
    dist.barrier()
    total_ms = ev.ms(e0, e1)
    # per-part device time: from the event before each part to the event after it
    per_part = {k: 0.0 for k in w.parts}
    for start, marks in step_marks:
        prev = start
        for k, e in marks:
            per_part[k] += ev.ms(prev, e)
            prev = e
    t_max = dist.max(total_ms / 1e3)
    total_updates = dist.sum(w.updates() * args.steps)
    value = total_updates / t_max / 1e9

    # ---- end to end through the C ABI with host buffers (warm-up as for the device loop) ----
    for _ in range(args.warmup):
        w.e2e_step()
    A.sync()
    dist.barrier()
    t0 = time.perf_counter()
    e_a = ev.record()
    e2e_steps_ms = []
    for _ in range(args.steps):
        t_s = time.perf_counter()
        w.e2e_step()
        e2e_steps_ms.append((time.perf_counter() - t_s) * 1e3)
    e_b = ev.record()
    A.sync()
    e2e_s = max(time.perf_counter() - t0, ev.ms(e_a, e_b) / 1e3)
    gc.enable()
    e2e_s = dist.max(e2e_s)
    e2e_value = dist.sum(w.updates() * args.steps) / e2e_s / 1e9
    # the pipelined downloads must have read the finished results
    for k, (_, h) in w.host_out.items():
        if hasattr(w, "result_of") and not np.array_equal(w.result_of(k).download(), h):
            raise RuntimeError(f"end-to-end result of {k} differs from the device result")

    kernel_only = w.fold_kernel_rates(ev) if hasattr(w, "fold_kernel_rates") else None

    # ---- roofline of the dominant kernel ----
    peak, peak_kind = measured_peaks()
    dom = max(w.parts, key=lambda k: per_part[k])
    p = w.parts[dom]
    avg_launch_s = per_part[dom] / 1e3 / (args.steps * p.launches)
    achieved = p.bytes_per_launch / avg_launch_s / 1e9
    parts_out = {}
    for k, pp in w.parts.items():
        t = per_part[k] / 1e3 / args.steps
        parts_out[pp.name] = {"ms_per_step": t * 1e3, "launches_per_step": pp.launches,
                              "GB_per_s": pp.bytes_per_launch * pp.launches / t / 1e9 if t > 0 else None}
        if w.unit == "GCUPS":
            parts_out[pp.name]["GCUPS"] = pp.updates / t / 1e9 if t > 0 else None
    # DRAM bytes per launch of the dominant kernel (dram__bytes_read.sum +
    # dram__bytes_write.sum) from the ncu captures summarised in profiles/.
    traffic = DRAM_TRAFFIC_PER_LAUNCH.get(p.name if getattr(p, "sweeps_per_launch", 2) != 1 else p.name + "/1")
    if p.name == "life" and getattr(w, "tuned", {}).get("life_temporal_depth") != 32:
        traffic = None  # captured at temporal depth 32

    cpu = None
    if dist.rank == 0 and not args.no_cpu_baseline:
        try:
            from oracle import pyoracle as O
            O.build()
            threads = cpu_threads()
            v, sample = w.cpu_sample(O, threads, min_seconds=10.0)
            cpu = {"value": v, "unit": w.unit, "cores": threads, "kind": "port", "sample": sample}
        except Exception as exc:  # the CPU baseline is reported, never required
            cpu = {"value": None, "unit": w.unit, "cores": 0, "kind": "port", "sample": f"failed: {exc}"}

    if dist.rank == 0:
        line = {
            "metric": w.metric, "value": value, "unit": w.unit, "n_gpus": dist.world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_max * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": w.dtype, "data": "synthetic",
            "config": dict(w.config(), parallelism=f"replicas x{dist.world}", **getattr(w, "tuned", {})),
            "e2e": {"value": e2e_value, "unit": w.unit, "h2d_bytes_per_step": w.h2d, "d2h_bytes_per_step": w.d2h,
                    # host-clock time of each end-to-end step: single slow steps (the host link is
                    # shared) move the whole-run value, which is total updates over total time
                    "step_ms_median": statistics.median(e2e_steps_ms), "step_ms_max": max(e2e_steps_ms)},
            "roofline": {"bound": "hbm", "kernel": p.name, "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": peak_kind, "traffic": traffic,
                         "bytes_per_launch": p.bytes_per_launch,
                         # several sweeps per launch: the grid's one read and write per launch
                         "compulsory_bytes_per_launch": p.compulsory_bytes,
                         "compulsory_frac": p.compulsory_bytes / avg_launch_s / 1e9 / peak,
                         **({"sweeps_per_launch": p.sweeps_per_launch} if hasattr(p, "sweeps_per_launch") else {})},
            "parts": parts_out,
            **({"fold_kernel_only": {k: dict(v, frac=v["GB_per_s"] / peak) for k, v in kernel_only.items()}}
               if kernel_only else {}),
            "cpu_baseline": cpu,
            "gpu_launches": launches,
            "clocks": clocks,
        }
        print(json.dumps(line), flush=True)
    dist.close()


if __name__ == "__main__":
    main()
