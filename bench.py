#!/usr/bin/env python3
"""Benchmark of the dense-CRF mean-field hot path on GB300.

Workload ("plain_vga"): DenseCRF2D 640x480, 21 labels, smooth-random-field
unary, 40-cell Voronoi image, addPairwiseGaussian(sxy=3, compat=3) +
addPairwiseBilateral(sxy=80, srgb=13, compat=10) with Potts compatibility,
10 mean-field iterations, float32.  Seeded synthetic inputs
(pydensecrf_gb300.synthetic.plain_vga); no dataset is involved.

One STEP is one complete solve of that image: both lattice builds and
normalisations plus the 10 iterations.  Metric: MPix*label*iter/s =
W*H*M*T / step time (higher is better).

* value -- inputs resident in HBM (unary and image on the device), the C ABI
  with device pointers; CUDA events on the engine's stream around each step;
  L2 flushed (a 512 MiB write) between timed steps, outside the events.
* e2e   -- the public Python API (DenseCRF2D / setUnaryEnergy /
  addPairwise* / inference) with the unary and image in pinned host memory:
  every step copies them host->device and reads the marginals back.
* cpu_baseline -- the CPU oracle (a C restatement of the reference's
  algorithm, oracle/dcrf_oracle.c) on a bounded sample of the same workload,
  one solve per host thread in parallel.
* accuracy -- the marginals of the last timed end-to-end solve against the
  oracle on the same inputs, in float and in float64.
* --impl reference -- the reference's CPU path for this workload on the host
  cores (the oracle port: the reference itself is not built on this machine),
  same metric and step definition.

Under torchrun (--gpus N > 1) every rank solves its own image: replicas, no
collective on the data path (scaling "weak"); value = all ranks' work / the
slowest rank's time.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

W, H, M, T = 640, 480, 21, 10
UNITS_PER_STEP = W * H * M * T / 1e6  # MPix*label*iter per solve
METRIC = "MPix*label*iter/s, 640x480x21, 10 iterations (Gaussian+bilateral), full solve incl. lattice build"
WORKLOAD = "DenseCRF2D 640x480 M=21 T=10, Gaussian(sxy=3,c=3)+bilateral(sxy=80,srgb=13,c=10) Potts"


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def whole_job_rate(local_time, steps, world, dist=None, device="cpu", per_second=1.0):
    """Whole-job throughput of `world` replicas that each ran `steps` solves:
    every rank's work over the slowest rank's time (max over ranks; `dist`
    None on one rank).  `local_time` is this rank's time in units of
    1/per_second seconds (per_second=1e3 for milliseconds).  Returns (rate,
    slowest time)."""
    import torch

    t = torch.tensor([float(local_time)], dtype=torch.float64, device=device)
    if dist is not None:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    slowest = float(t.item())
    return world * steps * UNITS_PER_STEP / (slowest / per_second), slowest


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "20"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
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
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx = float(p[2])
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def profiled_traffic():
    """DRAM bytes (read + write) of one point-pass launch on this workload and
    where they come from: the ncu capture recorded in
    profiles/pointpass_plain_vga.json (dram__bytes_read.sum +
    dram__bytes_write.sum of one launch, with the command that took it).
    Returns (bytes or None, source text)."""
    try:
        with open(os.path.join(ROOT, "profiles", "pointpass_plain_vga.json")) as fh:
            rec = json.load(fh)
        return int(rec["traffic_bytes_per_launch"]), rec.get("traffic_source", "ncu capture")
    except Exception:
        return None, None


def measured_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ----------------------------------------------------------------------------
def _oracle():
    """The CPU oracle module (test infrastructure: used here only for the CPU
    reference figures), built on first use."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    O.build()
    return O


def host_variant(O) -> int:
    """The lattice build the reference compiles on this host: its SSE path on
    x86-64, its scalar path elsewhere (e.g. aarch64), selected by the
    reference's own #ifdef __SSE__ (permutohedral.cpp:36-39)."""
    import platform

    return O.VARIANT_SSE if platform.machine().lower() in ("x86_64", "amd64", "i686", "i386") else O.VARIANT_SCALAR


def host_variant_name() -> str:
    import platform

    x86 = platform.machine().lower() in ("x86_64", "amd64", "i686", "i386")
    return "SSE lattice build and filter (x86)" if x86 else "scalar lattice build and filter (non-x86)"


def cpu_oracle_rate(cfg, threads: int, solves_per_thread: int = 1):
    """Throughput of the CPU oracle on full solves of the workload, `threads` in parallel."""
    O = _oracle()
    U = np.ascontiguousarray(cfg["U"].T)
    fg = O.features_gaussian_2d(W, H, 3.0, 3.0)
    fb = O.features_bilateral_2d(cfg["img"], 80, 80, 13, 13, 13)

    def solve():
        c = O.OracleCRF(W * H, M, host_variant(O))
        c.set_unary(U)
        c.add_pairwise(fg, 3.0)
        c.add_pairwise(fb, 10.0)
        c.inference(T)

    def worker():
        for _ in range(solves_per_thread):
            solve()

    t0 = time.perf_counter()
    ths = [threading.Thread(target=worker) for _ in range(threads)]
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    dt = time.perf_counter() - t0
    n = threads * solves_per_thread
    return n * UNITS_PER_STEP / dt, dt, n


def cpu_single_core(cfg, reps: int = 1):
    """The reference's own setting: one solve on one host thread (its sources
    have no threading), with the lattice builds (the two addPairwise calls)
    and the T iterations timed apart; the fastest of `reps` solves."""
    O = _oracle()
    U = np.ascontiguousarray(cfg["U"].T)
    fg = O.features_gaussian_2d(W, H, 3.0, 3.0)
    fb = O.features_bilateral_2d(cfg["img"], 80, 80, 13, 13, 13)
    best = None
    for _ in range(max(1, reps)):
        t0 = time.perf_counter()
        c = O.OracleCRF(W * H, M, host_variant(O))
        c.set_unary(U)
        c.add_pairwise(fg, 3.0)
        c.add_pairwise(fb, 10.0)
        t1 = time.perf_counter()
        c.inference(T)
        t2 = time.perf_counter()
        del c
        if best is None or t2 - t0 < best[0] + best[1]:
            best = (t1 - t0, t2 - t1)
    build_s, inf_s = best
    return {"value": round(UNITS_PER_STEP / (build_s + inf_s), 3), "unit": "MPix*label*iter/s", "cores": 1,
            "kind": "port", "variant": host_variant_name(), "build_ms": round(1e3 * build_s, 1),
            "iteration_ms": round(1e3 * inf_s / T, 2),
            "sample": f"one full solve on one thread (fastest of {max(1, reps)})"}


def solve_accuracy(cfg, Q_gpu: np.ndarray):
    """Error of the benchmarked solve's own marginals (M x N, from the timed
    end-to-end steps) against the oracle on the same inputs, in float (the
    reference's arithmetic, x86 lattice variant like the engine's default) and
    in float64 (the exact-arithmetic limit over the same lattices)."""
    O = _oracle()
    c = O.OracleCRF(W * H, M, O.VARIANT_SSE)
    c.set_unary(np.ascontiguousarray(cfg["U"].T))
    c.add_pairwise(O.features_gaussian_2d(W, H, 3.0, 3.0), 3.0)
    c.add_pairwise(O.features_bilateral_2d(cfg["img"], 80, 80, 13, 13, 13), 10.0)
    q32, q64 = c.inference(T), c.inference_f64(T)
    q = np.asarray(Q_gpu, np.float32).reshape(M, W * H).T
    return {"max_abs_vs_oracle": float(np.abs(q - q32).max()), "max_abs_vs_fp64": float(np.abs(q - q64).max()),
            "oracle_vs_fp64": float(np.abs(q32 - q64).max()),
            "argmax_agreement_vs_oracle": float((q.argmax(1) == q32.argmax(1)).mean()),
            "sample": "the marginals of the last timed end-to-end solve"}


def cpu_oracle_problems(problems, threads: int):
    """Wall-clock throughput of the CPU oracle on full solves of `problems`, one
    per host thread (`threads` at a time).  A problem is (N, M, T, unary as
    (N, M), [(features as (N, d), compatibility, kernel type)]); the oracle's C
    calls release the GIL, so the threads run in parallel.  Returns (MPix * label
    * iter/s, seconds, solves)."""
    O = _oracle()

    def solve(p):
        N, Mp, Tp, U, terms = p
        c = O.OracleCRF(N, Mp, host_variant(O))
        c.set_unary(U)
        for f, compat, ktype in terms:
            c.add_pairwise(f, compat, ktype=ktype)
        c.inference(Tp)

    import concurrent.futures as cf

    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(max_workers=max(1, threads)) as ex:
        list(ex.map(solve, problems))
    dt = time.perf_counter() - t0
    units = sum(p[0] * p[1] * p[2] for p in problems) / 1e6
    return units / dt, dt, len(problems)


def cpu_batched_baseline(threads: int):
    """The batched workload's CPU reference point: the oracle on the first
    `threads` images of the 64-image batch, one per host thread."""
    from pydensecrf_gb300 import synthetic as S

    O = _oracle()
    # the generator's first images are those of the 64-image batch (only the
    # shared compatibility, drawn after the images, differs)
    cfg = S.batch_uneven(0, B=min(threads, 64))
    probs = []
    for b in range(len(cfg["sizes"])):
        Wb, Hb = cfg["sizes"][b]
        probs.append((Wb * Hb, cfg["M"], cfg["T"], np.ascontiguousarray(cfg["U"][b].T),
                      [(O.features_gaussian_2d(Wb, Hb, 3.0, 3.0), cfg["compat"], 1),
                       (O.features_bilateral_2d(cfg["img"][b], 80, 80, 13, 13, 13), cfg["compat"], 1)]))
    rate, dt, n = cpu_oracle_problems(probs, threads)
    px = sum(p[0] for p in probs)
    return {"value": round(rate, 3), "unit": "MPix*label*iter/s", "cores": threads, "kind": "port",
            "variant": host_variant_name(),
            "sample": f"{n} of the 64 images ({px} px), one full solve per host thread, {dt:.1f} s"}


def cpu_volumes_baseline(threads: int):
    """The volume workload's CPU reference point: the oracle's forward on the 8
    volumes, one per host thread."""
    from pydensecrf_gb300 import synthetic as S

    cfg = S.volume_96(0)
    Sz = cfg["S"]
    n = Sz ** 3
    zz, yy, xx = np.mgrid[0:Sz, 0:Sz, 0:Sz].astype(np.float32)
    pos = np.ascontiguousarray(np.stack([xx / np.float32(3), yy / np.float32(3), zz / np.float32(3)]).reshape(3, -1).T)
    probs = [(n, cfg["M"], cfg["T"], np.ascontiguousarray(u.T),
              [(np.ascontiguousarray(f.T), cfg["compat"], 2), (pos, 1.0, 1)]) for u, f in zip(cfg["U"], cfg["feat"])]
    rate, dt, k = cpu_oracle_problems(probs, threads)
    return {"value": round(rate, 3), "unit": "MVoxel*label*iter/s (forward incl. lattice builds)", "cores": threads,
            "kind": "port", "variant": host_variant_name(),
            "sample": f"the {k} volumes' forward solves, one per host thread, {dt:.1f} s"}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    from pydensecrf_gb300 import synthetic as S

    cfg = S.plain_vga(0)
    cores = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_oracle_rate(cfg, cores)
    times = []
    for _ in range(args.steps):
        _, dt, n = cpu_oracle_rate(cfg, cores)
        times.append(dt)
    total = sum(times)
    value = args.steps * cores * UNITS_PER_STEP / total
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "MPix*label*iter/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * total / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded plain_vga generator)", "impl": "reference",
        "config": {"workload": WORKLOAD, "step": f"{cores} full solves in parallel (one per host thread)"},
        "cpu_baseline": {"value": round(value, 3), "unit": "MPix*label*iter/s", "cores": cores, "kind": "port",
                         "variant": host_variant_name(),
                         "sample": f"{cores} concurrent full solves per step, {args.steps} steps"},
        "e2e": {"value": round(value, 3), "unit": "MPix*label*iter/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


# ----------------------------------------------------------------------------
def learning_step_times(lib, _lib, dev, stream, reps: int = 2, profile_one: bool = False):
    """Forward and forward+backward of the differentiable mean-field on the
    training workload (512x512, 21 labels, 5 iterations, Gaussian Potts with
    a CONST kernel + bilateral with a 21x21 Matrix compatibility and DIAG
    kernel; loss =
    cross-entropy against a 30-region label map), per image over 8 images.

    forward  = both lattice builds + 5 checkpointed iterations;
    backward = the adjoint: dL/dU, dL/d(compatibility) and dL/d(bilateral
               kernel parameters).  CUDA events on the engine's stream."""
    import torch

    from pydensecrf_gb300 import synthetic as S

    cfg = S.train_512(0)
    Wt, Ht, Mt, Tt = cfg["W"], cfg["H"], cfg["M"], cfg["T"]
    Nt = Wt * Ht
    Us = [torch.from_numpy(u).to(dev) for u in cfg["U"]]
    imgs = [torch.from_numpy(im).to(dev) for im in cfg["img"]]
    gts = [torch.from_numpy(g).to(dev) for g in cfg["gt"]]
    cg = np.array([3.0], np.float32)
    cm = np.ascontiguousarray(cfg["compat"], np.float32)
    Q = torch.empty((Mt, Nt), dtype=torch.float32, device=dev)
    dU = torch.empty_like(Q)
    h = ctypes.c_void_p()
    _lib.check(lib.dcrf_create_2d(Wt, Ht, Mt, ctypes.byref(h)))
    _lib.check(lib.dcrf_set_stream(h, ctypes.c_void_p(stream.cuda_stream)))
    _lib.check(lib.dcrf_set_autotune(h, 1))
    cols = torch.arange(Nt, device=dev)
    grads = {}

    def grad_buffers():
        # sized from the terms' parameter counts (Gaussian: Potts 1; bilateral: 21x21 + DIAG 5)
        if not grads:
            nc = nk = 0
            for term in range(2):
                c, k = ctypes.c_int(), ctypes.c_int()
                _lib.check(lib.dcrf_param_counts(h, term, ctypes.byref(c), ctypes.byref(k)))
                nc += c.value
                nk += k.value
            grads["c"] = np.zeros(max(1, nc), np.float64)
            grads["k"] = np.zeros(max(1, nk), np.float64)
        return grads["c"], grads["k"]

    def fwd(i):
        _lib.check(lib.dcrf_clear_pairwise(h))
        _lib.check(lib.dcrf_set_unary(h, ctypes.c_void_p(Us[i].data_ptr()), _lib.LAYOUT_LM, _lib.DEVICE))
        # CONST kernel: the Gaussian bandwidth is not learned here
        _lib.check(lib.dcrf_add_pairwise_gaussian(h, 3.0, 3.0, _lib.COMPAT_POTTS, cg.ctypes.data, 0, 3, None))
        _lib.check(lib.dcrf_add_pairwise_bilateral(h, 80.0, 80.0, 13.0, 13.0, 13.0, ctypes.c_void_p(imgs[i].data_ptr()),
                                                   _lib.DEVICE, _lib.COMPAT_MATRIX, cm.ctypes.data, 1, 3, None))
        _lib.check(lib.dcrf_inference_checkpointed(h, Tt, ctypes.c_void_p(Q.data_ptr()), _lib.LAYOUT_LM, _lib.DEVICE))

    def bwd(i):
        with torch.cuda.stream(stream):
            dQ = torch.zeros_like(Q)
            dQ[gts[i], cols] = -1.0 / (Nt * Q[gts[i], cols].clamp_min(1e-20))
        dcomp, dkern = grad_buffers()
        _lib.check(lib.dcrf_backward(h, ctypes.c_void_p(dQ.data_ptr()), _lib.LAYOUT_LM, _lib.DEVICE,
                                     ctypes.c_void_p(dU.data_ptr()), dcomp.ctypes.data, dkern.ctypes.data))

    fwd(0)
    bwd(0)
    torch.cuda.synchronize()
    if profile_one:  # one forward + backward between cudaProfilerStart/Stop (ncu --profile-from-start off)
        fwd(1)
        bwd(1)
        torch.cuda.synchronize()
        torch.cuda.profiler.start()
        fwd(2)
        bwd(2)
        torch.cuda.synchronize()
        torch.cuda.profiler.stop()
    f_ms, b_ms = [], []
    for _ in range(reps):
        for i in range(len(Us)):
            e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
            e0.record(stream)
            fwd(i)
            e1.record(stream)
            bwd(i)
            e2.record(stream)
            torch.cuda.synchronize()
            f_ms.append(e0.elapsed_time(e1))
            b_ms.append(e1.elapsed_time(e2))
    lib.dcrf_destroy(h)
    f, b = float(np.median(f_ms)), float(np.median(b_ms))
    return {"workload": "512x512 M=21 T=5, Gaussian Potts + bilateral Matrix(21x21) DIAG, CE loss, 8 images",
            "fwd_ms_per_img": round(f, 3), "bwd_ms_per_img": round(b, 3),
            "fwd_plus_bwd_over_fwd": round((f + b) / f, 3),
            "grads": "dU, dcompat (Potts + 21x21), dkernel (bilateral 5 scales)"}


PHASES = ((0, "point"), (1, "reduce"), (2, "blur"), (3, "lattice"), (4, "other"), (5, "norm"))


def phase_ms(handles, lib, _lib):
    """Device milliseconds per kernel class recorded by the handles' profiling
    mode, summed over the handles (profiling must be on while they ran)."""
    out = {}
    for cls, name in PHASES:
        tot = 0.0
        for h in handles:
            ms, n = ctypes.c_double(), ctypes.c_longlong()
            _lib.check(lib.dcrf_profile(h, cls, ctypes.byref(ms), ctypes.byref(n)))
            tot += ms.value
        out[name] = round(tot, 3)
    return out


def batched_vs_loop(lib, _lib, dev, stream, reps: int = 2, n_images: int = 64):
    """The batched form against a per-image loop on 64 uneven images
    (W, H ~ U[256, 1024], M=21, T=10, Gaussian sxy=3 + bilateral sxy=80
    srgb=13, both with one random symmetric 21x21 Matrix compatibility,
    entries U(0, 2), zero diagonal).  Inputs resident in HBM; per image the
    loop uses its own pre-created handle (lattice builds and inference in the
    timed region, handle creation outside), the batch one handle for all.
    Both solve the full problem: lattice builds, normalisations, 10 iterations."""
    import torch

    from pydensecrf_gb300 import synthetic as S

    cfg = S.batch_uneven(0, B=n_images)
    Mb, Tb = cfg["M"], cfg["T"]
    sizes = cfg["sizes"]
    Ns = [w * h for w, h in sizes]
    Ntot = sum(Ns)
    cm = np.ascontiguousarray(cfg["compat"], np.float32)
    U_all = torch.from_numpy(np.concatenate([u.reshape(-1) for u in cfg["U"]])).to(dev)
    img_all = torch.from_numpy(np.concatenate([im.reshape(-1) for im in cfg["img"]])).to(dev)
    Q_all = torch.empty(Mb * Ntot, dtype=torch.float32, device=dev)
    offs = np.concatenate([[0], np.cumsum(Ns)])

    def ptr(t, off=0):
        return ctypes.c_void_p(int(t.data_ptr() + int(off) * t.element_size()))

    def solve(h, u, img, q):
        _lib.check(lib.dcrf_clear_pairwise(h))
        _lib.check(lib.dcrf_set_unary(h, u, _lib.LAYOUT_LM, _lib.DEVICE))
        _lib.check(lib.dcrf_add_pairwise_gaussian(h, 3.0, 3.0, _lib.COMPAT_MATRIX, cm.ctypes.data, 1, 3, None))
        _lib.check(lib.dcrf_add_pairwise_bilateral(h, 80.0, 80.0, 13.0, 13.0, 13.0, img, _lib.DEVICE,
                                                   _lib.COMPAT_MATRIX, cm.ctypes.data, 1, 3, None))
        _lib.check(lib.dcrf_inference(h, Tb, q, _lib.LAYOUT_LM, _lib.DEVICE))

    Wa = np.ascontiguousarray([w for w, _ in sizes], np.int32)
    Ha = np.ascontiguousarray([h for _, h in sizes], np.int32)
    hb = ctypes.c_void_p()
    _lib.check(lib.dcrf_create_batch_2d(len(sizes), Wa.ctypes.data, Ha.ctypes.data, Mb, ctypes.byref(hb)))
    _lib.check(lib.dcrf_set_stream(hb, ctypes.c_void_p(stream.cuda_stream)))
    _lib.check(lib.dcrf_set_autotune(hb, 1))

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        ms = []
        for _ in range(reps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            torch.cuda.synchronize()
            ms.append(a.elapsed_time(b))
        return float(np.median(ms))

    batch_ms = timed(lambda: solve(hb, ptr(U_all), ptr(img_all), ptr(Q_all)))
    # per-phase device time of one solve (profiling mode: events around every launch)
    _lib.check(lib.dcrf_set_profiling(hb, 1))
    solve(hb, ptr(U_all), ptr(img_all), ptr(Q_all))
    batch_phases = phase_ms([hb], lib, _lib)
    _lib.check(lib.dcrf_set_profiling(hb, 0))
    c0, c1 = ctypes.c_ulonglong(), ctypes.c_ulonglong()
    lib.dcrf_launch_count(ctypes.byref(c0))
    solve(hb, ptr(U_all), ptr(img_all), ptr(Q_all))
    torch.cuda.synchronize()
    lib.dcrf_launch_count(ctypes.byref(c1))
    batch_launches = c1.value - c0.value
    Qb = Q_all.clone()
    knobs = [ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_float(), ctypes.c_int()]
    _lib.check(lib.dcrf_get_tuning(hb, *[ctypes.byref(k) for k in knobs]))
    lib.dcrf_destroy(hb)

    # the per-image handles run with the batch's tuned knobs (same arithmetic)
    hs = []
    for w, h_ in sizes:
        h = ctypes.c_void_p()
        _lib.check(lib.dcrf_create_2d(w, h_, Mb, ctypes.byref(h)))
        _lib.check(lib.dcrf_set_stream(h, ctypes.c_void_p(stream.cuda_stream)))
        _lib.check(lib.dcrf_set_tuning(h, *[k.value for k in knobs]))
        hs.append(h)

    def loop():
        for i, h in enumerate(hs):
            solve(h, ptr(U_all, Mb * offs[i]), ptr(img_all, 3 * offs[i]), ptr(Q_all, Mb * offs[i]))

    loop_ms = timed(loop)
    for h in hs:
        _lib.check(lib.dcrf_set_profiling(h, 1))
    loop()
    loop_phases = phase_ms(hs, lib, _lib)
    for h in hs:
        lib.dcrf_destroy(h)
    same = bool(torch.equal(Qb, Q_all))
    units = Ntot * Mb * Tb / 1e6
    return {"workload": f"{len(sizes)} images W,H~U[256,1024] (sum {Ntot} px) M=21 T=10, Gaussian+bilateral, "
                        "21x21 Matrix compat", "batched_ms": round(batch_ms, 3), "loop_ms": round(loop_ms, 3),
            "speedup": round(loop_ms / batch_ms, 3),
            "batched_value": round(units / (batch_ms / 1e3), 1), "loop_value": round(units / (loop_ms / 1e3), 1),
            "unit": "MPix*label*iter/s", "batched_launches": int(batch_launches),
            "batched_equals_loop": same,
            # device time per kernel class of one solve, summed over the handles (profiling mode);
            # the per-pixel classes (point, reduce, blur) bound what batching can remove
            "breakdown_ms": {"batched": batch_phases, "loop": loop_phases},
            "tuning": {"split": knobs[0].value, "smem_kb": knobs[1].value, "task_len": knobs[2].value,
                       "hash_load": round(knobs[3].value, 2), "coop_blur": knobs[4].value}}


def volumes_fwd_bwd(lib, _lib, dev, stream, reps: int = 2):
    """Generic (non-2D) batched forward + backward on 8 volumes of 96^3 voxels:
    features (x/5, y/5, z/5, I/0.1) with a FULL kernel and a random symmetric
    4x4 Matrix compatibility, plus a DIAG Gaussian on (x/3, y/3, z/3) with
    Potts 1; M=4, T=8; gradients w.r.t. unary and compatibility.  One batched
    handle, inputs resident in HBM."""
    import torch

    from pydensecrf_gb300 import synthetic as S

    cfg = S.volume_96(0)
    Sz, Mv, Tv = cfg["S"], cfg["M"], cfg["T"]
    B = len(cfg["U"])
    n = Sz ** 3
    Ntot = B * n
    zz, yy, xx = np.mgrid[0:Sz, 0:Sz, 0:Sz].astype(np.float32)
    pos = np.ascontiguousarray(np.stack([xx / np.float32(3), yy / np.float32(3), zz / np.float32(3)]).reshape(3, -1))
    U_all = torch.from_numpy(np.concatenate([u.reshape(-1) for u in cfg["U"]])).to(dev)
    F4 = torch.from_numpy(np.ascontiguousarray(np.concatenate(cfg["feat"], axis=1))).to(dev)
    F3 = torch.from_numpy(np.ascontiguousarray(np.concatenate([pos] * B, axis=1))).to(dev)
    Q = torch.empty(Mv * Ntot, dtype=torch.float32, device=dev)
    dQ = torch.randn(Mv * Ntot, generator=torch.Generator(device=dev).manual_seed(0), device=dev) / Ntot
    dU = torch.empty_like(Q)
    cm = np.ascontiguousarray(cfg["compat"], np.float32)
    cp = np.array([1.0], np.float32)
    Ns = np.full(B, n, np.int32)
    h = ctypes.c_void_p()
    _lib.check(lib.dcrf_create_batch(B, Ns.ctypes.data, Mv, ctypes.byref(h)))
    _lib.check(lib.dcrf_set_stream(h, ctypes.c_void_p(stream.cuda_stream)))
    _lib.check(lib.dcrf_set_autotune(h, 1))
    dc = np.zeros(Mv * Mv + 1, np.float64)

    def fwd():
        _lib.check(lib.dcrf_clear_pairwise(h))
        _lib.check(lib.dcrf_set_unary(h, ctypes.c_void_p(U_all.data_ptr()), _lib.LAYOUT_LM, _lib.DEVICE))
        _lib.check(lib.dcrf_add_pairwise(h, ctypes.c_void_p(F4.data_ptr()), 4, _lib.DEVICE, _lib.COMPAT_MATRIX,
                                         cm.ctypes.data, 2, 3, None))
        _lib.check(lib.dcrf_add_pairwise(h, ctypes.c_void_p(F3.data_ptr()), 3, _lib.DEVICE, _lib.COMPAT_POTTS,
                                         cp.ctypes.data, 1, 3, None))
        _lib.check(lib.dcrf_inference_checkpointed(h, Tv, ctypes.c_void_p(Q.data_ptr()), _lib.LAYOUT_LM,
                                                   _lib.DEVICE))

    def bwd():
        _lib.check(lib.dcrf_backward(h, ctypes.c_void_p(dQ.data_ptr()), _lib.LAYOUT_LM, _lib.DEVICE,
                                     ctypes.c_void_p(dU.data_ptr()), dc.ctypes.data, None))

    fwd()
    bwd()
    torch.cuda.synchronize()
    f_ms, b_ms = [], []
    for _ in range(reps):
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        e0.record(stream)
        fwd()
        e1.record(stream)
        bwd()
        e2.record(stream)
        torch.cuda.synchronize()
        f_ms.append(e0.elapsed_time(e1))
        b_ms.append(e1.elapsed_time(e2))
    lib.dcrf_destroy(h)
    f, b = float(np.median(f_ms)), float(np.median(b_ms))
    units = Ntot * Mv * Tv / 1e6
    return {"workload": f"{B} volumes of {Sz}^3 (N={Ntot}) M=4 T=8, FULL kernel on (x,y,z,I) + DIAG Gaussian, "
                        "Matrix compat, one batched handle",
            "fwd_ms": round(f, 3), "bwd_ms": round(b, 3), "fwd_plus_bwd_over_fwd": round((f + b) / f, 3),
            "fwd_value": round(units / (f / 1e3), 1), "unit": "MVoxel*label*iter/s (forward incl. lattice builds)",
            "grads": "dU, dcompat"}


def run_gpu(args):
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist_mod

        dist_mod.init_process_group("nccl")
        dist = dist_mod
    dev = torch.device("cuda", local)

    from pydensecrf_gb300 import _lib, synthetic as S
    from pydensecrf_gb300 import densecrf as dcrf

    lib = _lib.load()
    cfg = S.plain_vga(rank)
    U_d = torch.from_numpy(cfg["U"]).to(dev)
    img_d = torch.from_numpy(cfg["img"]).to(dev)
    Q_d = torch.empty((M, W * H), dtype=torch.float32, device=dev)
    h = ctypes.c_void_p()
    _lib.check(lib.dcrf_create_2d(W, H, M, ctypes.byref(h)))
    stream = torch.cuda.current_stream(dev)
    _lib.check(lib.dcrf_set_stream(h, ctypes.c_void_p(stream.cuda_stream)))
    if not args.fixed_knobs:
        _lib.check(lib.dcrf_set_autotune(h, 1))  # tuned during the first warm-up step
    cg = np.array([3.0], np.float32)
    cb = np.array([10.0], np.float32)

    def step_device():
        _lib.check(lib.dcrf_clear_pairwise(h))
        _lib.check(lib.dcrf_set_unary(h, ctypes.c_void_p(U_d.data_ptr()), _lib.LAYOUT_LM, _lib.DEVICE))
        _lib.check(lib.dcrf_add_pairwise_gaussian(h, 3.0, 3.0, _lib.COMPAT_POTTS, cg.ctypes.data, 1, 3, None))
        _lib.check(lib.dcrf_add_pairwise_bilateral(h, 80.0, 80.0, 13.0, 13.0, 13.0, ctypes.c_void_p(img_d.data_ptr()),
                                                   _lib.DEVICE, _lib.COMPAT_POTTS, cb.ctypes.data, 1, 3, None))
        _lib.check(lib.dcrf_inference(h, T, ctypes.c_void_p(Q_d.data_ptr()), _lib.LAYOUT_LM, _lib.DEVICE))

    flush = torch.empty(128 * 1024 * 1024, dtype=torch.float32, device=dev)  # 512 MiB > L2

    def barrier():
        if dist:
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        step_device()
    cnt0 = ctypes.c_ulonglong()
    cnt1 = ctypes.c_ulonglong()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    barrier()
    lib.dcrf_launch_count(ctypes.byref(cnt0))
    with ClockSampler(local) as clk:
        for k in range(args.steps):
            flush.zero_()
            ev[k][0].record(stream)
            step_device()
            ev[k][1].record(stream)
        barrier()
    lib.dcrf_launch_count(ctypes.byref(cnt1))
    step_ms = [a.elapsed_time(b) for a, b in ev]
    value, total_ms = whole_job_rate(float(sum(step_ms)), args.steps, world, dist, dev, per_second=1e3)
    launches = int(cnt1.value - cnt0.value)

    tk = [ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_float(), ctypes.c_int()]
    _lib.check(lib.dcrf_get_tuning(h, *[ctypes.byref(k) for k in tk]))
    tuning = {"split": tk[0].value, "smem_kb": tk[1].value, "task_len": tk[2].value,
              "hash_load": round(tk[3].value, 2), "coop_blur": tk[4].value}

    # ---- breakdown and roofline: a profiled pass (events around every launch)
    _lib.check(lib.dcrf_set_profiling(h, 1))
    nprof = 3
    for _ in range(nprof):
        flush.zero_()
        step_device()
    prof = {}
    for cls, name in PHASES:
        ms, n = ctypes.c_double(), ctypes.c_longlong()
        _lib.check(lib.dcrf_profile(h, cls, ctypes.byref(ms), ctypes.byref(n)))
        prof[name] = {"ms_per_step": ms.value / nprof, "launches_per_step": n.value // nprof,
                      "avg_us": 1e3 * ms.value / max(1, n.value)}
    _lib.check(lib.dcrf_set_profiling(h, 0))
    Ls, Ps = [], []
    for term in range(2):
        L, P, nt = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _lib.check(lib.dcrf_term_stats(h, term, ctypes.byref(L), ctypes.byref(P), ctypes.byref(nt)))
        Ls.append(L.value)
        Ps.append(P.value)
    N = W * H
    MP = 24
    d_terms = (2, 5)
    # algorithmic bytes of one mean-field point pass (slice + compatibility + softmax + tile splat):
    # unary read, per term: corner offsets + slice weights, norm, every vertex row once, tile member
    # lists (uint16 point + float weight), partial rows written; plus the slot map.
    pp_bytes = N * M * 4 + N * 4 + sum(N * (d + 1) * 8 + N * 4 + L * MP * 4 + N * (d + 1) * 6 + P * MP * 4
                                       for d, L, P in zip(d_terms, Ls, Ps))
    # the lattice builds (Permutohedral::init + the kernel normalisation): algorithmic bytes
    # per term N*d*4 (features) + N*(d+1)*8 (offsets + weights) + L*d*2 (keys) + (d+1)*L*8 (neighbours)
    build_bytes = sum(N * d * 4 + N * (d + 1) * 8 + L * d * 2 + (d + 1) * L * 8 for d, L in zip(d_terms, Ls))
    peak, peak_kind = measured_peak()
    if args.traffic is not None:
        traffic, traffic_src = args.traffic, "--traffic argument"
    else:
        traffic, traffic_src = profiled_traffic()
    avg_s = prof["point"]["avg_us"] / 1e6
    achieved = pp_bytes / avg_s / 1e9
    roofline = {"bound": "hbm", "kernel": "pointpass_kernel<24>", "achieved": round(achieved, 1),
                "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 3), "traffic": traffic, "traffic_source": traffic_src,
                "algorithmic_bytes_per_launch": int(pp_bytes), "avg_launch_us": round(prof["point"]["avg_us"], 2),
                "peak_kind": peak_kind}
    lat_s = prof["lattice"]["ms_per_step"] / 1e3
    lattice_roofline = {"bound": "latency (dependent launches, one host wait per term)",
                        "scope": "the two lattice builds (Permutohedral::init); their normalisation is 'norm'",
                        "algorithmic_bytes_per_step": int(build_bytes), "ms_per_step": round(1e3 * lat_s, 4),
                        "achieved": round(build_bytes / lat_s / 1e9, 1), "peak": peak, "unit": "GB/s",
                        "frac": round(build_bytes / lat_s / 1e9 / peak, 4)}

    # ---- end to end through the public Python API, pinned host buffers
    U_h = torch.from_numpy(cfg["U"]).pin_memory().numpy()
    img_h = torch.from_numpy(cfg["img"]).pin_memory().numpy()

    def step_e2e():
        d = dcrf.DenseCRF2D(W, H, M)
        d.setUnaryEnergy(U_h)
        d.addPairwiseGaussian(sxy=3, compat=3)
        d.addPairwiseBilateral(sxy=80, srgb=13, rgbim=img_h, compat=10)
        Q = d.inference(T)
        return Q

    for _ in range(max(1, args.warmup)):
        step_e2e()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        Q = step_e2e()
    torch.cuda.synchronize()
    e2e_value, e2e_s = whole_job_rate(time.perf_counter() - t0, args.steps, world, dist, dev)

    # ---- CPU baseline (rank 0, single GPU runs only)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        try:
            rate, dt, n = cpu_oracle_rate(cfg, threads)
            cpu = {"value": round(rate, 3), "unit": "MPix*label*iter/s", "cores": threads, "kind": "port",
                   "variant": host_variant_name(),
                   "sample": f"{n} full solves of the same workload, one per thread, {dt:.1f} s"}
        except Exception as e:  # a CPU sample that cannot run is reported; the GPU line still prints
            cpu = {"unavailable": f"{type(e).__name__}: {e}"}
        else:
            try:
                cpu["single_core"] = cpu_single_core(cfg)
            except Exception as e:
                cpu["single_core"] = {"unavailable": f"{type(e).__name__}: {e}"}

    # ---- accuracy of the timed solve itself against the oracle (float and FP64)
    accuracy = None
    if rank == 0 and world == 1 and not args.no_cpu:
        try:
            accuracy = solve_accuracy(cfg, np.array(Q))
        except Exception as e:  # reported, not fatal
            accuracy = {"unavailable": f"{type(e).__name__}: {e}"}

    lib.dcrf_destroy(h)
    learning = learning_step_times(lib, _lib, dev, stream) if (rank == 0 and not args.no_learning) else None
    batched = batched_vs_loop(lib, _lib, dev, stream) if (rank == 0 and not args.no_batch) else None
    volumes = volumes_fwd_bwd(lib, _lib, dev, stream) if (rank == 0 and not args.no_batch) else None
    # CPU reference points of the batched and volume workloads (the oracle port,
    # one solve per host thread); reported only, never the target
    if rank == 0 and world == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        for obj, fn in ((batched, cpu_batched_baseline), (volumes, cpu_volumes_baseline)):
            if obj is not None:
                try:
                    obj["cpu_baseline"] = fn(threads)
                except Exception as e:  # a baseline that cannot run is reported, not fatal
                    obj["cpu_baseline"] = {"unavailable": f"{type(e).__name__}: {e}"}
    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": "MPix*label*iter/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded plain_vga generator)",
            "config": {"workload": WORKLOAD, "step": "one full solve: 2 lattice builds + norms + 10 iterations",
                       "l2": "flushed between timed steps (512 MiB write)", "parallelism": f"replicas x{world}"},
            "e2e": {"value": round(e2e_value, 3), "unit": "MPix*label*iter/s",
                    "h2d_bytes_per_step": int(cfg["U"].nbytes + cfg["img"].nbytes),
                    "d2h_bytes_per_step": int(N * M * 4), "ms_per_step": round(1e3 * e2e_s / args.steps, 3)},
            "gpu_launches": launches,
            "breakdown_ms_per_step": {k: round(v["ms_per_step"], 4) for k, v in prof.items()},
            "iteration_ms": round((prof["point"]["ms_per_step"] + prof["reduce"]["ms_per_step"]
                                   + prof["blur"]["ms_per_step"]) / T, 4),
            "lattice": {"L": Ls, "partials": Ps},
            "tuning": tuning,
            "roofline": roofline,
            "lattice_roofline": lattice_roofline,
            "cpu_baseline": cpu,
            "accuracy": accuracy,
            "learning": learning,
            "batched": batched,
            "volumes": volumes,
            "clocks": clk.summary(),
        }
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline sample")
    ap.add_argument("--no-learning", action="store_true", help="skip the forward+backward timing")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-vs-loop timing")
    ap.add_argument("--learning-only", action="store_true",
                    help="only the forward+backward timing, one step of it between cudaProfilerStart/Stop "
                         "(for ncu --profile-from-start off); prints its JSON object")
    ap.add_argument("--fixed-knobs", action="store_true",
                    help="no autotuning of the main solve (the default knobs; a fixed launch sequence for profilers)")
    ap.add_argument("--traffic", type=float, default=None,
                    help="DRAM bytes per point-pass launch from an ncu capture (reported as roofline.traffic)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.learning_only:
        import torch

        from pydensecrf_gb300 import _lib

        dev = torch.device("cuda", 0)
        torch.cuda.set_device(dev)
        r = learning_step_times(_lib.load(), _lib, dev, torch.cuda.current_stream(dev), profile_one=True)
        print(json.dumps(r))
        return 0
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
