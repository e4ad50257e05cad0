#!/usr/bin/env python
"""FlOF on GB300: 4D flow solves/s at 64^4 to a fixed CG residual.

One step is the whole two-way workload at one resolution:
  * both deformations (data 0 -> 1 and 1 -> 0) with opticalFlowMultiscale4d
    at 64^4 float32, flof.py's parameters with cgAccuracy 1e-4;
  * the mode-2 two-way apply (deform4d) at alpha 0.25 / 0.5 / 0.75 on the
    64^4 grid;
  * the mode-3 two-way apply (loadAdvectTimeSlice_OptRun for both
    directions plus the blend) of every frame of a 128^3 x 64 hi-res SDF
    series at the same three alphas.
Inputs are the seeded synthetic drop/pool SDFs of ofblend_gb300.synth.

value: solves/s with inputs resident in HBM (2 solves per step, summed over
ranks); e2e: the same through the C ABI with host buffers, copies included.
`--impl reference` times the CPU oracle (a restatement of the reference's
CPU path) on a bounded sample of the same workload.
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

os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "4D flow solves/s at 64^4 to fixed residual: learned warm-start vs plain CG"
NFRAMEBUF = 4  # device frame buffers of the e2e pipeline
REF_MAX_STEPS = 1  # whole CPU steps of the reference arm (minutes each)
UNIT = "solves/s"
ALPHAS = (0.25, 0.5, 0.75)


def args_():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--res", type=int, default=64)
    ap.add_argument("--hires", type=int, default=128)
    ap.add_argument("--cg-accuracy", type=float, default=1e-4)
    ap.add_argument("--blur-type", type=int, default=1)
    ap.add_argument("--e2e-steps", type=int, default=8)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-oracle64", action="store_true",
                    help="--workload mixed: skip the FP64 oracle solve (minutes on the host)")
    ap.add_argument("--no-learned", action="store_true",
                    help="skip the learned-mode record of the default line")
    ap.add_argument("--train-pairs", type=int, default=256)
    ap.add_argument("--train-epochs", type=int, default=20)
    ap.add_argument("--workload", default="flof",
                    choices=["flof", "batch", "mixed", "learned", "net"],
                    help="flof: the two-way 64^4 workload (default); batch: 64 independent solves of "
                         "uneven sizes, concurrent against sequential; mixed: the 96^4 solve in mixed "
                         "precision against FP32; learned: train the warm start and solve with it; "
                         "net: the network's training step alone")
    ap.add_argument("--net-batch", type=int, default=16)
    ap.add_argument("--batch-pairs", type=int, default=64)
    ap.add_argument("--batch-workers", type=int, default=0)
    return ap.parse_args()


def flof_params(acc, blur_type):
    # scenes/flof.py:913-915 with ofsd defaults, except the CG accuracy
    return dict(wSmooth=0.001, wEnergy=0.0001, cgAccuracy=acc, postVelBlur=4, cfl=999, multiStep=3,
                minGridSize=20, doFinalProject=True, resetBndWidth=0.1, blurType=blur_type)


def dist():
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local = int(os.environ.get("LOCAL_RANK", 0))
    return rank, world, local


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    Q = ("index,uuid,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, uuid: str | None):
        self.uuid = uuid
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                                         text=True)
        except (OSError, ValueError):
            self.proc = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=5)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            if self.uuid and self.uuid not in f[1]:
                continue
            try:
                sm.append(float(f[2]))
                mx.append(float(f[3]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() in ("active", "1"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def measured_bf16_tflops():
    """Burst cuBLAS bf16 TFLOP/s of this GPU (the tensor roofline)."""
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        if "bf16_tflops" in d:
            return float(d["bf16_tflops"]), "measured"
    return 1900.0, "fallback"


def step_hbm(recs, steps, ms, peak, peak_kind):
    """HBM rate of the whole step on one GPU: the algorithmic bytes of every
    launch (each kernel class's per-cell bytes; kernels bound by arithmetic
    count their compulsory bytes only) over the untraced step time."""
    b = sum(r[2] for r in recs) / steps
    gbs = b / (ms / steps * 1e-3) / 1e9
    return {"bytes_per_step": round(b), "achieved": round(gbs, 1), "peak": peak, "unit": "GB/s",
            "frac": round(gbs / peak, 4), "peak_source": f"hbm_gbs of {peak_kind}"}


def ncu_traffic():
    """Per-launch DRAM bytes (read + write) of the kernel classes measured by
    ncu at 64^4, from the committed summary's table (profiles/)."""
    p = os.path.join(ROOT, "profiles", "dram_traffic_cg_64.md")
    out = {}
    if os.path.exists(p):
        with open(p) as f:
            for ln in f:
                cells = [c.strip() for c in ln.strip().strip("|").split("|")]
                if len(cells) >= 4 and cells[0].startswith("cg_"):
                    try:
                        out[cells[0]] = float(cells[3]) * 1e6
                    except ValueError:
                        pass
    return out


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
class Workload:
    def __init__(self, F, synth, R, H, acc, blur_type, ctx):
        self.F = F
        self.R, self.H = R, H
        self.Tf = R  # hi-res frames = t extent of the deformation
        dims = (R, R, R, R)
        self.dims = dims
        s0, s1 = synth.scene_for(0), synth.scene_for(1)
        self.h_i0 = synth.flow_input(s0, dims)
        self.h_i1 = synth.flow_input(s1, dims)
        self.h_s0 = synth.sdf4d(s0, dims)
        self.h_s1 = synth.sdf4d(s1, dims)
        hd = (H, H, H, self.Tf)
        self.h_hi0 = synth.sdf4d(s0, hd)
        self.h_hi1 = synth.sdf4d(s1, hd)
        self.params = flof_params(acc, blur_type)
        mk = lambda cls, d: cls(dims=d, ctx=ctx)  # noqa: E731
        self.g_i0, self.g_i1 = mk(F.Grid4Real, dims), mk(F.Grid4Real, dims)
        self.g_s0, self.g_s1 = mk(F.Grid4Real, dims), mk(F.Grid4Real, dims)
        self.g_hi0, self.g_hi1 = mk(F.Grid4Real, hd), mk(F.Grid4Real, hd)
        self.v01, self.v10 = mk(F.Grid4Vec4, dims), mk(F.Grid4Vec4, dims)
        self.out4 = mk(F.Grid4Real, dims)
        self.dst = mk(F.RealGrid, (H, H, H, 1))
        # further frame buffers of the e2e pipeline (downloads in flight)
        self.dsts = [self.dst] + [mk(F.RealGrid, (H, H, H, 1)) for _ in range(NFRAMEBUF - 1)]
        self.factor = (H / R, H / R, H / R, self.Tf / R)
        self.bord = int(H * 0.1)
        self.stats = []

    def upload(self):
        for name in ("i0", "i1", "s0", "s1", "hi0", "hi1"):
            getattr(self, "g_" + name).from_numpy(getattr(self, "h_" + name))

    def h2d_bytes(self):
        return sum(getattr(self, "h_" + n).nbytes for n in ("i0", "i1", "s0", "s1", "hi0", "hi1"))

    def step(self):
        """One step on inputs resident in HBM."""
        F = self.F
        self.v01.clear()
        self.v10.clear()
        F.opticalFlowMultiscale4d(self.v01, self.g_i0, self.g_i1, **self.params)
        self.stats.append(F.last_solve_stats())
        F.opticalFlowMultiscale4d(self.v10, self.g_i1, self.g_i0, **self.params)
        self.stats.append(F.last_solve_stats())
        for a in ALPHAS:
            F.deform4d(self.out4, self.g_s0, self.g_s1, self.v01, self.v10, alpha=a, twoway=1)
        F.loadAdvectTimeSlice_OptInit(1, self.v01)
        F.loadAdvectTimeSlice_OptInit(2, self.v10)
        H, Tf = self.H, self.Tf
        for a in ALPHAS:
            for t in range(Tf):
                F.loadAdvectTimeSlice_OptRunTwoway(1, 2, self.dst, self.g_hi0, self.g_hi1, t + 0.5, a, 1.0,
                                                   (0, 0, 0, 0), (1, 1, 1, Tf / Tf), self.factor,
                                                   overrideSize=(H, H, H, Tf), overrideTimeOff=0.0,
                                                   bordSkip=self.bord)
        F.loadAdvectTimeSlice_Finish(1)
        F.loadAdvectTimeSlice_Finish(2)

    def step_e2e(self, pinned, sink, ctx):
        """One step through the C ABI from and to host buffers, with the
        transfers pipelined on the context's copy stream: the solves wait only
        for their own inputs (the mode-2 and hi-res inputs upload meanwhile),
        results download while later work runs, and frames rotate through
        NFRAMEBUF device buffers.  Ends when every result is in host memory."""
        F = self.F
        for n in ("i0", "i1", "s0", "s1", "hi0", "hi1"):
            getattr(self, "g_" + n).upload_async(pinned[n])
        for g in (self.g_i0, self.g_i1, self.v01, self.v10):
            g.copy_wait()
        self.v01.clear()
        self.v10.clear()
        F.opticalFlowMultiscale4d(self.v01, self.g_i0, self.g_i1, **self.params)
        self.stats.append(F.last_solve_stats())
        F.opticalFlowMultiscale4d(self.v10, self.g_i1, self.g_i0, **self.params)
        self.stats.append(F.last_solve_stats())
        self.v01.download_async(sink["v01"])
        self.v10.download_async(sink["v10"])
        self.g_s0.copy_wait()
        self.g_s1.copy_wait()
        for k, a in enumerate(ALPHAS):
            self.out4.copy_wait()
            F.deform4d(self.out4, self.g_s0, self.g_s1, self.v01, self.v10, alpha=a, twoway=1)
            self.out4.download_async(sink["out4"][k])
        F.loadAdvectTimeSlice_OptInit(1, self.v01)
        F.loadAdvectTimeSlice_OptInit(2, self.v10)
        self.g_hi0.copy_wait()
        self.g_hi1.copy_wait()
        H, Tf = self.H, self.Tf
        n = 0
        for a in ALPHAS:
            for t in range(Tf):
                d = self.dsts[n % NFRAMEBUF]
                d.copy_wait()
                F.loadAdvectTimeSlice_OptRunTwoway(1, 2, d, self.g_hi0, self.g_hi1, t + 0.5, a, 1.0,
                                                   (0, 0, 0, 0), (1, 1, 1, Tf / Tf), self.factor,
                                                   overrideSize=(H, H, H, Tf), overrideTimeOff=0.0,
                                                   bordSkip=self.bord)
                d.download_async(sink["frame"][n % NFRAMEBUF])
                n += 1
        F.loadAdvectTimeSlice_Finish(1)
        F.loadAdvectTimeSlice_Finish(2)
        ctx.copies_sync()

    def d2h_bytes(self):
        return (2 * self.v01.dims[0] ** 4 * 16 + len(ALPHAS) * self.h_s0.nbytes
                + len(ALPHAS) * self.Tf * self.H ** 3 * 4)


def roofline(records, R, peak, peak_kind, traffic):
    """Roofline of the kernel class with the most device time at the full
    grid size R, and the device time of every class over all sizes (the
    pyramid levels and the hi-res frames included)."""
    per, every = {}, {}
    for name, sx, nb, ms in records:
        e = every.setdefault(name, [0, 0.0, 0.0])
        e[0] += 1
        e[1] += nb
        e[2] += ms
        if sx != R:
            continue
        e = per.setdefault(name, [0, 0.0, 0.0])
        e[0] += 1
        e[1] += nb
        e[2] += ms
    if not per:
        return None, {}
    dom = max(per, key=lambda k: per[k][2])
    n, nb, ms = per[dom]
    achieved = (nb / n) / ((ms / n) * 1e-3) / 1e9
    tr = traffic.get(dom) if R == 64 else None  # the summary was captured at 64^4
    rl = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
          "frac": round(achieved / peak, 4), "traffic": tr, "kernel": dom,
          "launches": n, "bytes_per_launch": nb / n, "ms_per_launch": ms / n,
          "peak_source": f"hbm_gbs of {peak_kind}"}
    share = {k: {"launches": v[0], "ms": round(v[2], 3),
                 "GBps": round(v[1] / (v[2] * 1e-3) / 1e9, 1) if v[2] > 0 else None}
             for k, v in sorted(every.items(), key=lambda kv: -kv[1][2])}
    return rl, share


def cpu_step_seconds(R, H, acc):
    """One whole two-way step of the workload at grid R and hi-res H on the
    host with the CPU oracle (CpuWorkload); returns (seconds, parts)."""
    W = CpuWorkload(R, H, acc)
    t = W.step()
    return t, W.parts


CPU_BASELINE_RES = 32  # the GPU line's bounded CPU sample: the same workload at 32^4


# ---------------------------------------------------------------------------
# ranks: one process per GPU, replicas of the whole workload (no data-path
# collective); these helpers run on any torch.distributed backend
# ---------------------------------------------------------------------------
def init_ranks(world, local, backend="nccl"):
    """Join the process group of a multi-rank run (NCCL between GPUs; the
    tests use gloo on CPU)."""
    if world <= 1:
        return
    import torch
    import torch.distributed as td
    if backend == "nccl":
        td.init_process_group("nccl", device_id=torch.device("cuda", local))
    else:
        td.init_process_group(backend)


def barrier(world):
    if world > 1:
        import torch.distributed as td
        td.barrier()


def max_over_ranks(x, world, device="cuda"):
    """The slowest rank's time: the whole job ends when it does."""
    if world <= 1:
        return float(x)
    import torch
    import torch.distributed as td
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    td.all_reduce(t, op=td.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank, world, seconds):
    """Whole-job throughput: the units all ranks processed over the slowest
    rank's time."""
    return units_per_rank * world / seconds


LEARNED_VARIANTS = (
    ("mg", {"solver": "mg"}),
    ("mg_separable", {"solver": "mg", "blurType": 2}),
    ("mg_separable_warm", {"solver": "mg", "blurType": 2, "warmStart": True}),
)
WARM_TRAIN_PAIRS, WARM_TRAIN_EPOCHS = 64, 5  # the default line's warm-start network


def learned_record(W, a, ctx, stream):
    """The learned solve mode beside the plain one on the same two-way step.

    Variants: "mg" is the multigrid-preconditioned PCG (solver="mg": the same
    stop rule on the same residual; the plain operator judges each result and
    the plain PCG finishes when needed); "mg_separable" adds blurType 2, the
    separable Gaussian blur and extrapolation box sums (equal to the direct
    stencils up to rounding); "mg_separable_warm" starts the coarsest level
    from the learned network's prediction (trained here on plain-solver
    outputs of WARM_TRAIN_PAIRS seeded pairs at 32^4).  The record's value is
    the "mg_separable" variant's.

    Accuracy is measured against a tightly converged plain solve (cgAccuracy
    1e-7): at cgAccuracy 1e-4 the plain result itself is only that close to
    the converged deformation, so every variant is judged by the same
    yardstick (relative L2 of the deformation and max-abs cells of the SDF
    deformed at alpha 0.5), with and without the final projection."""
    import torch
    from ofblend_gb300 import warmstart
    F = W.F
    plain = dict(W.params)
    steps = max(1, a.steps)
    sdf = F.Grid4Real(dims=W.dims, ctx=ctx)
    # the warm-start network, trained on the GPU from plain-solver outputs
    t0 = time.perf_counter()
    samples = warmstart.make_samples(WARM_TRAIN_PAIRS, base_seed=10000,
                                     solve_params=dict(flof_params(0.01, a.blur_type)), ctx=ctx)
    t_data = time.perf_counter() - t0
    model = F.Model(16, ctx=ctx, seed=1)
    t0 = time.perf_counter()
    hist = warmstart.train(model, samples, epochs=WARM_TRAIN_EPOCHS, batch=16, lr=2e-3)
    ctx.synchronize()
    t_train = time.perf_counter() - t0
    del samples
    model.attach()

    def deformed(v):
        sdf.from_numpy(W.h_s0)
        F.advect4d(v, sdf, 0.5)
        return sdf.to_numpy()

    def accuracy(base):
        fields = {}
        for key, prm in [("plain", base), ("converged", dict(base, cgAccuracy=1e-7))] + \
                [(k, dict(base, **extra)) for k, extra in LEARNED_VARIANTS]:
            v = F.Grid4Vec4(dims=W.dims, ctx=ctx)
            F.opticalFlowMultiscale4d(v, W.g_i0, W.g_i1, **prm)
            fields[key] = v
        ref = fields.pop("converged")
        refv = ref.to_numpy().astype(np.float64)
        ref_sdf = deformed(ref)
        out = {}
        for key, v in fields.items():
            x = v.to_numpy().astype(np.float64)
            out[key] = {"rel_l2_vs_converged": float(np.linalg.norm(x - refv) / np.linalg.norm(refv)),
                        "sdf_cells_vs_converged": float(np.abs(deformed(v) - ref_sdf).max())}
        return out

    rec = {"accuracy": accuracy(plain),
           "accuracy_without_projection": accuracy(dict(plain, doFinalProject=False)),
           "variants": {}}
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    for key, extra in LEARNED_VARIANTS:
        W.params = dict(plain, **extra)
        f0 = ctx.mg_fallbacks()
        for _ in range(2):
            W.step()
        W.stats.clear()
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(steps):
            W.step()
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        it = [[x[1] for x in st["solves"] if x[0] == a.res] for st in W.stats[:2]]
        ctx.profile(True)
        W.step()
        torch.cuda.synchronize()
        recs = ctx.profile_records()
        ctx.profile(False)
        share = {}
        for name, sx, nb, kms in recs:
            e = share.setdefault(name, [0, 0.0])
            e[0] += 1
            e[1] += kms
        rec["variants"][key] = {
            "params": extra, "value": round(2 * steps / (ms * 1e-3), 4), "unit": UNIT,
            "steps": steps, "ms_per_step": round(ms / steps, 3), "cg_iterations_level0": it,
            "cg_iterations_total": [st["cg_total_iterations"] for st in W.stats[:2]],
            "warm_start_used": [st["warm_start"] for st in W.stats[:2]],
            "plain_finishes": ctx.mg_fallbacks() - f0,
            "kernel_ms_per_step": {k: {"launches": v[0], "ms": round(v[1], 3)}
                                   for k, v in sorted(share.items(), key=lambda kv: -kv[1][1])}}
    W.params = plain
    model.detach()
    model.free()
    rec["warm_start_training"] = {"pairs": WARM_TRAIN_PAIRS, "epochs": WARM_TRAIN_EPOCHS,
                                  "data_seconds": round(t_data, 2), "train_seconds": round(t_train, 2),
                                  "loss_first_last": [round(hist[0], 6), round(hist[-1], 6)]}
    last = rec["variants"]["mg_separable"]
    rec.update({
        "solver": "multigrid-preconditioned PCG (V-cycle over 2^4 aggregates, block-Jacobi "
                  "smoothing, parameters fitted on solver-generated systems) with separable "
                  "stencils; same stop rule on the same residual; the plain operator judges, "
                  "the plain PCG finishes",
        "value": last["value"], "unit": UNIT, "ms_per_step": last["ms_per_step"],
        "cg_iterations_level0": last["cg_iterations_level0"]})
    return rec


def run_gpu(a):
    import torch
    rank, world, local = dist()
    init_ranks(world, local)
    torch.cuda.set_device(local)
    import ofblend_gb300 as F
    from ofblend_gb300 import synth
    ctx = F.Context(local)
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream.cuda_stream)
    W = Workload(F, synth, a.res, a.hires, a.cg_accuracy, a.blur_type, ctx)
    W.upload()
    # The end-to-end run's pinned host buffers (3.7 GB) are allocated and
    # filled here, seconds before they are used: on some hosts copies from
    # freshly pinned memory ran at a tenth of the usual rate for a while.
    pinned = {}
    for n in ("i0", "i1", "s0", "s1", "hi0", "hi1"):
        h = getattr(W, "h_" + n)
        tt = torch.empty(h.shape, dtype=torch.float32, pin_memory=True)
        tt.numpy()[...] = h
        pinned[n] = tt.numpy()
    pin = lambda shape: torch.empty(shape, dtype=torch.float32, pin_memory=True).numpy()  # noqa: E731
    sink = {"v01": pin(W.v01.shape), "v10": pin(W.v10.shape),
            "out4": [pin(W.out4.shape) for _ in ALPHAS],
            "frame": [pin(W.dst.shape) for _ in range(NFRAMEBUF)]}
    for _ in range(max(a.warmup, 0)):
        W.step()
    torch.cuda.synchronize()
    barrier(world)
    uuid = None
    try:
        uuid = str(torch.cuda.get_device_properties(local).uuid)
    except Exception:
        pass
    clocks = ClockSampler(uuid)
    clocks.start()
    W.stats.clear()
    l0 = ctx.kernel_launches()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(a.steps):
        W.step()
    e1.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    launches = ctx.kernel_launches() - l0
    ms = e0.elapsed_time(e1)
    # A second pass of the same steps with a CUDA event pair around every
    # launch (on the context's stream) gives the per-kernel times of the
    # roofline and the shares.  The events sit between dependent launches and
    # cost a few percent, so the first pass alone gives the throughput.
    ctx.profile(True)
    e0.record(stream)
    for _ in range(a.steps):
        W.step()
    e1.record(stream)
    torch.cuda.synchronize()
    ms_prof = e0.elapsed_time(e1)
    clk = clocks.stop()
    recs = ctx.profile_records()
    ctx.profile(False)
    ms_max = max_over_ranks(ms, world)
    if a.steps <= 0:
        raise SystemExit("--steps must be positive")
    value = job_rate(2 * a.steps, world, ms_max * 1e-3)
    peak, peak_kind = measured_peaks()
    rl, share = roofline(recs, a.res, peak, peak_kind, ncu_traffic())
    rl["region"] = "profiled pass of the same steps, one CUDA event pair per launch"

    # e2e: through the C ABI with the pinned host buffers allocated above,
    # copies inside
    def copy_rates():
        """GB/s of one hi-res input up and back down on the copy stream."""
        g = W.g_hi0
        torch.cuda.synchronize()
        ctx.synchronize()
        tc = time.perf_counter()
        g.upload_async(pinned["hi0"])
        g.copy_wait()
        ctx.synchronize()
        up = time.perf_counter() - tc
        tc = time.perf_counter()
        g.download_async(pinned["hi0"])
        g.copy_wait()
        ctx.synchronize()
        down = time.perf_counter() - tc
        nb = pinned["hi0"].nbytes
        return round(nb / up / 1e9, 1), round(nb / down / 1e9, 1)

    e2e_val = None
    e2e_extra = {}
    if a.e2e_steps > 0:
        rates_before = copy_rates()
        W.step_e2e(pinned, sink, ctx)
        torch.cuda.synchronize()
        rates_warm = copy_rates()
        barrier(world)
        per = []
        t0 = time.perf_counter()
        for _ in range(a.e2e_steps):
            ts = time.perf_counter()
            W.step_e2e(pinned, sink, ctx)
            per.append(time.perf_counter() - ts)
        torch.cuda.synchronize()
        e2e_s = max_over_ranks(time.perf_counter() - t0, world)
        e2e_val = round(job_rate(2 * a.e2e_steps, world, e2e_s), 4)
        # the copy rates the transfers run at, before and after the e2e steps
        rates_after = copy_rates()
        e2e_extra = {"ms_per_step": round(e2e_s * 1e3 / a.e2e_steps, 3),
                     "ms_per_step_min": round(min(per) * 1e3, 3),
                     "ms_each": [round(t * 1e3, 1) for t in per],
                     "h2d_GBps": rates_after[0], "d2h_GBps": rates_after[1],
                     "h2d_d2h_GBps_before": list(rates_before),
                     "h2d_d2h_GBps_after_warmup_step": list(rates_warm)}

    st = list(W.stats)
    iters = [s["solves"] for s in st]
    learned = None
    if not a.no_learned:
        learned = learned_record(W, a, ctx, stream)
        learned["speedup_vs_plain"] = round(learned["value"] / value, 3)
    line = {
        "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": round(ms_max / a.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded drop/pool SDFs)",
        "config": flof_config(a, world),
        "roofline": rl,
        "e2e": dict({"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": W.h2d_bytes(),
                     "d2h_bytes_per_step": W.d2h_bytes(), "steps": a.e2e_steps}, **e2e_extra),
        "gpu_launches": launches,
        "clocks": clk,
        "kernel_share": share,
        "hbm_step": step_hbm(recs, a.steps, ms_max, peak, peak_kind),
        "kernel_ms_per_step": round(sum(r[3] for r in recs) / a.steps, 3),
        "ms_per_step_profiled": round(ms_prof / a.steps, 3),
        "cg_iterations_level0": [[x[1] for x in s if x[0] == a.res] for s in iters[:2]],
    }
    if learned is not None:
        line["learned"] = learned
    if rank == 0 and not a.no_cpu_baseline:
        # A whole 64^4 step takes minutes on the host (the reference arm times
        # it); this line carries a bounded sample: the same two-way step at
        # 32^4, measured whole and not scaled, since the cost grows faster
        # than the cell count (more PCG iterations and sweeps at 64^4).
        rc = CPU_BASELINE_RES
        t_cpu, parts = cpu_step_seconds(rc, 2 * rc, a.cg_accuracy)
        line["cpu_baseline"] = {
            "value": round(2.0 / t_cpu, 6), "unit": UNIT, "cores": int(os.environ["OMP_NUM_THREADS"]),
            "kind": "port", "grid": [rc] * 4,
            "sample": f"one whole two-way step of this workload at {rc}^4 with {2 * rc}^3x{rc} hi-res "
                      f"frames (both deformations, deform4d at 3 alphas, all frames), not scaled to "
                      f"64^4; --impl reference times the 64^4 step whole",
            "seconds": round(t_cpu, 3), "parts": parts}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def flof_config(a, world):
    """The workload of the default line; both arms report it."""
    return {"workload": f"two-way FlOF at {a.res}^4: both deformations (flof parameters, "
                        f"cgAccuracy {a.cg_accuracy}, blurType {a.blur_type}) + deform4d and "
                        f"{a.hires}^3x{a.res} hi-res frames at alpha 0.25/0.5/0.75",
            "grid": [a.res] * 4, "hires": [a.hires] * 3 + [a.res], "frames_per_step": 3 * a.res,
            "solver": "plain multiscale Jacobi-PCG", "l2": "inputs larger than L2 (no flush)",
            "parallelism": f"replicas x{world}"}


class CpuWorkload:
    """The two-way workload of `Workload`, on the host with the CPU oracle:
    both deformations (opticalFlowMultiscale4d), deform4d at the three
    alphas and every hi-res frame of both directions plus the blend, with
    the same inputs and parameters.  The oracle runs its per-cell loops on
    OpenMP threads (the reference's KERNEL(fourd) loops do the same) and
    keeps the PCG's dot products serial, as the reference does."""

    def __init__(self, R, H, acc):
        import oracle
        from ofblend_gb300 import synth
        self.o = oracle.get(False)
        self.R, self.H, self.Tf = R, H, R
        dims = (R,) * 4
        s0, s1 = synth.scene_for(0), synth.scene_for(1)
        self.i0, self.i1 = synth.flow_input(s0, dims), synth.flow_input(s1, dims)
        self.s0, self.s1 = synth.sdf4d(s0, dims), synth.sdf4d(s1, dims)
        hd = (H, H, H, self.Tf)
        self.h0, self.h1 = synth.sdf4d(s0, hd), synth.sdf4d(s1, hd)
        p = flof_params(acc, 1)
        p.pop("blurType")
        self.params = p
        self.parts = {}

    def step(self):
        o, R, H, Tf = self.o, self.R, self.H, self.Tf
        zv = np.zeros(self.i0.shape + (4,), np.float32)
        t = time.perf_counter()
        v01, _, _ = o.opticalFlowMultiscale4d(zv, self.i0, self.i1, **self.params)
        v10, _, _ = o.opticalFlowMultiscale4d(zv, self.i1, self.i0, **self.params)
        t1 = time.perf_counter()
        for a in ALPHAS:
            o.deform4d(v01, v10, self.s0, self.s1, np.float32(a), twoway=1)
        t2 = time.perf_counter()
        kw = dict(loadTimeScale=1.0, defoOffset=(0, 0, 0, 0), defoScale=(1, 1, 1, 1),
                  defoFactor=(H / R, H / R, H / R, Tf / R), overrideSize=(H, H, H, Tf),
                  overrideTimeOff=0.0, bordSkip=int(H * 0.1))
        dst = np.zeros((H, H, H), np.float32)
        for a in ALPHAS:
            ai = np.float32(1.0 - a)
            for f in range(Tf):
                d0 = o.optRunFrame(v01, dst, self.h0, time=f + 0.5, blendAlpha=a, **kw)
                d1 = o.optRunFrame(v10, dst, self.h1, time=f + 0.5, blendAlpha=ai, **kw)
                o.addScaled(o.multConst(d0[None], ai), d1[None], np.float32(a))
        t3 = time.perf_counter()
        self.parts = {"solves_s": round(t1 - t, 2), "deform4d_s": round(t2 - t1, 2),
                      "frames_s": round(t3 - t2, 2)}
        return t3 - t


def run_reference(a):
    """The reference arm: the CPU oracle (the restatement of the reference's
    CPU path; the reference itself is not built here) runs the same two-way
    step whole.  One step takes minutes on the host, so the arm times
    min(steps, REF_MAX_STEPS) whole steps without warm-up and reports the
    steps it ran."""
    rank, world, _ = dist()
    if rank != 0:
        return
    W = CpuWorkload(a.res, a.hires, a.cg_accuracy)
    steps = max(1, min(a.steps, REF_MAX_STEPS))
    times = [W.step() for _ in range(steps)]
    t_step = sum(times) / len(times)
    v = 2.0 / t_step
    cores = int(os.environ["OMP_NUM_THREADS"])
    line = {
        "metric": METRIC, "value": round(v, 6), "unit": UNIT, "n_gpus": world, "steps": steps,
        "warmup": 0, "ms_per_step": round(t_step * 1e3, 1), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded drop/pool SDFs)",
        "impl": "reference",
        "config": flof_config(a, world),
        "cpu_baseline": {"value": round(v, 6), "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{steps} whole two-way step(s) of the workload in config: both "
                                   "deformations, deform4d at 3 alphas, all hi-res frames of both "
                                   "directions and the blend",
                         "parts_last_step": W.parts},
        "e2e": {"value": round(v, 6), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "steps_requested": a.steps, "warmup_requested": a.warmup,
    }
    print(json.dumps(line), flush=True)


def run_batch(a):
    """64 independent deformation solves of uneven sizes (S in 24..64, T in
    16..48, 1-3 drops): the batched entry point (concurrent worker streams,
    autotuned PCG launch shapes) against the same solves one after another."""
    import torch
    import ofblend_gb300 as F
    from ofblend_gb300 import _lib, synth
    torch.cuda.set_device(0)
    ctx = F.Context(0)
    ctx.set_option(_lib.FLOF_OPT_AUTOTUNE, 1)
    ps = synth.batch_pairs(a.batch_pairs)
    vs, i0s, i1s = [], [], []
    for dims, s0, s1 in ps:
        vs.append(F.Grid4Vec4(dims=dims, ctx=ctx))
        i0s.append(F.Grid4Real(dims=dims, ctx=ctx).from_numpy(synth.flow_input(s0, dims)))
        i1s.append(F.Grid4Real(dims=dims, ctx=ctx).from_numpy(synth.flow_input(s1, dims)))
    p = flof_params(a.cg_accuracy, a.blur_type)

    def reset():
        for v in vs:
            v.setConst(0.0)

    def batched():
        reset()
        F.opticalFlowMultiscale4d_batch(vs, i0s, i1s, workers=a.batch_workers, **p)

    def sequential():
        reset()
        for v, x, y in zip(vs, i0s, i1s):
            F.opticalFlowMultiscale4d(v, x, y, **p)

    def timed(fn, steps):
        ctx.synchronize()
        t0 = time.perf_counter()
        for _ in range(steps):
            fn()
        ctx.synchronize()
        return (time.perf_counter() - t0) / steps

    for _ in range(max(a.warmup, 1)):
        batched()
    sequential()  # warm the main context's pool and tuning table
    tb = timed(batched, a.steps)
    ts = timed(sequential, 1)
    n = len(ps)
    cells = int(sum(np.prod(d) for d, _, _ in ps))
    line = {
        "metric": f"batched 4D flow solves/s, {n} pairs of uneven sizes", "value": round(n / tb, 3),
        "unit": UNIT, "n_gpus": 1, "steps": a.steps, "warmup": a.warmup, "ms_per_step": round(tb * 1e3, 2),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded multi-drop pairs, seeds 1000+k)",
        "config": {"workload": f"{n} pairs, S in {list(synth.BATCH_SIZES)}, T in {list(synth.BATCH_T)}, "
                               f"1-3 drops r~U(3,8); flof parameters, cgAccuracy {a.cg_accuracy}",
                   "cells_total": cells, "workers": a.batch_workers or "auto", "autotune": True},
        "sequential": {"value": round(n / ts, 3), "ms_per_step": round(ts * 1e3, 2)},
        "speedup_vs_sequential": round(ts / tb, 3),
    }
    print(json.dumps(line), flush=True)
    ctx.close()


def run_mixed(a):
    """Mixed precision (BF16 gradient, FP64 residuals, iterative refinement)
    against the FP32 solve at 96^4 with two drops per data set, and the FP32
    solve of the inputs rounded to BF16 (the SDFs stored in BF16).  Each
    deformation, and the SDF it deforms at alpha 0.5, is compared with the
    FP64 CPU oracle's solve of the same inputs."""
    import torch
    import ofblend_gb300 as F
    from ofblend_gb300 import synth
    torch.cuda.set_device(0)
    ctx = F.Context(0)
    p = dict(flof_params(a.cg_accuracy, a.blur_type), doFinalProject=False)

    def scenes():
        return (synth.make_scene(11, ndrops=2, radius_range=(4.0, 6.0)),
                synth.make_scene(12, ndrops=2, radius_range=(4.0, 6.0)))

    s0, s1 = scenes()
    R = 96
    dims = (R, R, R, R)
    g0 = F.Grid4Real(dims=dims, ctx=ctx).from_numpy(synth.flow_input(s0, dims))
    g1 = F.Grid4Real(dims=dims, ctx=ctx).from_numpy(synth.flow_input(s1, dims))
    v = F.Grid4Vec4(dims=dims, ctx=ctx)
    res = {}
    for prec in ("fp32", "mixed"):
        for _ in range(max(a.warmup, 1)):
            v.setConst(0.0)
            F.opticalFlowMultiscale4d(v, g0, g1, precision=prec, **p)
        times = []
        for _ in range(max(a.steps, 1)):
            v.setConst(0.0)
            ctx.synchronize()
            t0 = time.perf_counter()
            F.opticalFlowMultiscale4d(v, g0, g1, precision=prec, **p)
            ctx.synchronize()
            times.append(time.perf_counter() - t0)
        st = F.last_solve_stats()
        res[prec] = {"s": min(times), "vel": v.to_numpy(), "stats": st}
    d96 = float(np.linalg.norm(res["mixed"]["vel"] - res["fp32"]["vel"]) /
                np.linalg.norm(res["fp32"]["vel"]))
    # The SDF inputs stored in BF16: the same FP32 solve on inputs rounded to
    # BF16 (round to nearest even), to measure what the data term makes of it.
    h0, h1 = g0.to_numpy(), g1.to_numpy()

    def bf16(x):
        u = x.view(np.uint32).astype(np.uint64)
        u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
        return u.astype(np.uint32).view(np.float32)
    b0 = F.Grid4Real(dims=dims, ctx=ctx).from_numpy(bf16(h0))
    b1 = F.Grid4Real(dims=dims, ctx=ctx).from_numpy(bf16(h1))
    v.setConst(0.0)
    F.opticalFlowMultiscale4d(v, b0, b1, **p)
    res["bf16_sdf"] = {"vel": v.to_numpy()}
    del b0, b1
    errors = None
    if not a.no_oracle64:
        # the FP64 CPU oracle (the reference's -DDOUBLEPRECISION build restated)
        # on the same inputs; deformed SDFs at alpha 0.5 in cells
        import oracle
        o64, o32 = oracle.get(True), oracle.get(False)
        t0 = time.perf_counter()
        ref, _, _ = o64.opticalFlowMultiscale4d(np.zeros(h0.shape + (4,), np.float64),
                                                h0.astype(np.float64), h1.astype(np.float64),
                                                **{k: v_ for k, v_ in p.items() if k != "blurType"})
        t64 = time.perf_counter() - t0
        sdf0 = synth.sdf4d(s0, dims)
        ref_sdf = o64.advect4d(ref, sdf0.astype(np.float64), 0.5)
        errors = {"oracle_fp64_seconds": round(t64, 1)}
        for key in ("fp32", "mixed", "bf16_sdf"):
            x = res[key]["vel"]
            errors[key] = {
                "rel_l2_vs_fp64": float(np.linalg.norm(x.astype(np.float64) - ref) / np.linalg.norm(ref)),
                "sdf_cells_vs_fp64": float(np.abs(o32.advect4d(x, sdf0, 0.5).astype(np.float64)
                                                  - ref_sdf).max())}

    m = res["mixed"]["stats"]
    line = {
        "metric": "4D flow solves/s at 96^4, mixed precision (BF16 gradient, FP64 refinement)",
        "value": round(1.0 / res["mixed"]["s"], 4), "unit": UNIT, "n_gpus": 1, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": round(res["mixed"]["s"] * 1e3, 2), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "bf16/f32/f64",
        "data": "synthetic (two drops per data set)",
        "config": {"workload": "one deformation 96^4, flof parameters without the final projection, "
                               f"cgAccuracy {a.cg_accuracy}", "grid": [96] * 4},
        "fp32": {"value": round(1.0 / res["fp32"]["s"], 4), "ms": round(res["fp32"]["s"] * 1e3, 2),
                 "cg_iterations": res["fp32"]["stats"]["cg_total_iterations"]},
        "mixed_cg_iterations": m["cg_total_iterations"],
        "mixed_true_residual_finest": m["true_residual"][-1] if m["true_residual"] else None,
        "mixed_vs_fp32_rel_l2_96": d96,
        "errors_vs_fp64_oracle": errors,
    }
    print(json.dumps(line), flush=True)
    ctx.close()


def net_flops(res: int) -> float:
    """Forward FLOPs of the warm start network at coarse extent res:
    2 * taps * cin * cout per output voxel and layer."""
    layers = [(2, 16, 81, 1), (16, 32, 81, 2), (32, 32, 81, 2), (32, 64, 81, 4), (64, 64, 81, 4),
              (96, 32, 81, 2), (48, 16, 81, 1), (16, 4, 1, 1)]
    return float(sum(2 * taps * ci * co * (res // div) ** 4 for ci, co, taps, div in layers))


def net_train_flops(res: int) -> float:
    """FLOPs of one training sample: forward, weight gradients, and input
    gradients of every layer but the first."""
    return 3.0 * net_flops(res) - 2.0 * 81 * 2 * 16 * res ** 4


def run_learned(a):
    """The learned warm start: trained on the GPU from plain-solver outputs of
    seeded 1-3 drop pairs at 32^4, then the two-way deformations of the
    standard inputs at --res solved cold and warm-started."""
    import torch
    import ofblend_gb300 as F
    from ofblend_gb300 import synth, warmstart
    torch.cuda.set_device(0)
    ctx = F.Context(0)
    t0 = time.perf_counter()
    samples = warmstart.make_samples(a.train_pairs, base_seed=10000,
                                     solve_params=dict(flof_params(0.01, a.blur_type)), ctx=ctx)
    t_data = time.perf_counter() - t0
    m = F.Model(16, ctx=ctx, seed=1)
    t0 = time.perf_counter()
    hist = warmstart.train(m, samples, epochs=a.train_epochs, batch=16, lr=2e-3)
    ctx.synchronize()
    t_train = time.perf_counter() - t0
    m.attach()
    R = a.res
    dims = (R, R, R, R)
    s0, s1 = synth.scene_for(0), synth.scene_for(1)
    g0 = F.Grid4Real(dims=dims, ctx=ctx).from_numpy(synth.flow_input(s0, dims))
    g1 = F.Grid4Real(dims=dims, ctx=ctx).from_numpy(synth.flow_input(s1, dims))
    v = F.Grid4Vec4(dims=dims, ctx=ctx)
    p = flof_params(a.cg_accuracy, a.blur_type)
    res = {}
    for mode in ("plain", "warm"):
        def step():
            st = []
            for x, y in ((g0, g1), (g1, g0)):
                v.setConst(0.0)
                F.opticalFlowMultiscale4d(v, x, y, warmStart=(mode == "warm"), **p)
                st.append(F.last_solve_stats())
            return st
        for _ in range(max(a.warmup, 1)):
            step()
        ctx.synchronize()
        tt = time.perf_counter()
        for _ in range(max(a.steps, 1)):
            st = step()
        ctx.synchronize()
        sec = (time.perf_counter() - tt) / max(a.steps, 1)
        res[mode] = {"solves_per_s": round(2.0 / sec, 4), "ms_per_step": round(sec * 1e3, 2),
                     "cg_iterations": [x["cg_total_iterations"] for x in st],
                     "warm_start": [x["warm_start"] for x in st],
                     "coarse_err_zero_vs_pred": [x["warm_start_err"] for x in st]}
    nsamp = a.train_pairs * a.train_epochs
    line = {
        "metric": f"4D flow solves/s at {R}^4 to fixed residual: learned warm-start vs plain CG",
        "value": res["warm"]["solves_per_s"], "unit": UNIT, "n_gpus": 1, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": res["warm"]["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 (network: tcgen05 bf16 MMAs, activations and gradients as bf16 hi/lo pairs, "
                 "f32 accumulation in tensor memory)",
        "data": "synthetic (training: seeded 1-3 drop pairs at 32^4; evaluation: data 0 <-> 1)",
        "config": {"workload": f"both deformations at {R}^4, flof parameters, cgAccuracy {a.cg_accuracy}",
                   "train_pairs": a.train_pairs, "train_epochs": a.train_epochs},
        "plain": res["plain"], "warm": res["warm"],
        "speedup_vs_plain": round(res["warm"]["solves_per_s"] / res["plain"]["solves_per_s"], 4),
        "training": {"data_seconds": round(t_data, 2), "train_seconds": round(t_train, 2),
                     "loss_first_last": [round(hist[0], 6), round(hist[-1], 6)],
                     "samples_per_s": round(nsamp / t_train, 1),
                     "net_tflops_fwd_bwd": round(net_train_flops(16) * nsamp / t_train / 1e12, 3)},
    }
    pk, pk_kind = measured_bf16_tflops()
    ach = net_train_flops(16) * nsamp / t_train / 1e12
    # training throughput in useful network FLOPs (2 x 81 x cin x cout per
    # output voxel and 3^4 layer; forward, weight and input gradients)
    # against the bf16 tensor peak
    line["roofline"] = {"bound": "tensor", "region": "network training (whole train loop)",
                        "achieved": round(ach, 3), "peak": pk, "unit": "TFLOP/s",
                        "frac": round(ach / pk, 5), "traffic": None,
                        "peak_source": f"bf16_tflops of {pk_kind}"}
    print(json.dumps(line), flush=True)
    m.detach()
    ctx.close()


def run_net(a):
    """The warm-start network's training step alone: Adam steps of a batch of
    --net-batch seeded random samples at the coarse extent 16^4 (the
    tcgen05 convolutions, their gradients and the update)."""
    import numpy as np
    import torch
    import ofblend_gb300 as F
    torch.cuda.set_device(0)
    ctx = F.Context(0)
    R = 16
    m = F.Model(R, ctx=ctx, seed=1)
    rng = np.random.default_rng(0)
    d = (R,) * 4
    samples = [(F.Grid4Real(dims=d, ctx=ctx).from_numpy((rng.standard_normal(d) * 0.004).astype(np.float32)),
                F.Grid4Real(dims=d, ctx=ctx).from_numpy((rng.standard_normal(d) * 0.004).astype(np.float32)),
                F.Grid4Vec4(dims=d, ctx=ctx).from_numpy((rng.standard_normal(d + (4,)) * 0.5).astype(np.float32)))
               for _ in range(max(a.net_batch, 1))]
    for _ in range(a.warmup):
        m.train_step(samples, 1e-3)
    ctx.synchronize()
    t0 = time.perf_counter()
    for _ in range(a.steps):
        m.train_step(samples, 1e-3)  # returns after the step has finished
    sec = (time.perf_counter() - t0) / max(a.steps, 1)
    sps = len(samples) / sec
    ach = net_train_flops(R) * sps / 1e12
    pk, pk_kind = measured_bf16_tflops()
    print(json.dumps({
        "metric": "warm-start network training samples/s at 16^4", "value": round(sps, 2),
        "unit": "samples/s", "n_gpus": 1, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": round(sec * 1e3, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None,
        "dtype": "bf16 tcgen05 MMAs (activations and gradients as bf16 hi/lo pairs), f32 accumulation",
        "data": "synthetic (seeded normal inputs and targets)",
        "config": {"workload": f"Adam steps of {len(samples)} samples at 16^4", "batch": len(samples)},
        "roofline": {"bound": "tensor", "region": "whole training step", "achieved": round(ach, 3),
                     "peak": pk, "unit": "TFLOP/s", "frac": round(ach / pk, 5), "traffic": None,
                     "peak_source": f"bf16_tflops of {pk_kind}"}}), flush=True)
    m.free()
    ctx.close()


if __name__ == "__main__":
    a = args_()
    if a.impl == "reference":
        run_reference(a)
    elif a.workload == "batch":
        run_batch(a)
    elif a.workload == "mixed":
        run_mixed(a)
    elif a.workload == "learned":
        run_learned(a)
    elif a.workload == "net":
        run_net(a)
    else:
        run_gpu(a)
