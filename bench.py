"""Chunk-generation benchmark: batched GB300 build vs one-chunk-per-launch vs CPU.

Workload (one step): build every chunk of the uniform grid -- 16x16x16 = 4096
chunks of 12^3 cells (13^3 = 2197 f32 samples each, 9.0M samples), 4-octave
fBm (base frequency 0.04, lacunarity 2, persistence 0.5) minus 0.03*(z-128),
iso-level 0 -- with permutation seed (step % 10), producing VertColor
vertices, unit normals and u32 indices per chunk plus per-chunk records.

  value    chunks/s of the batched persistent build (fast build, FMA on),
           inputs resident in HBM, CUDA events on the context stream, L2
           flushed (256 MiB write) before every timed step.  The outputs are
           every chunk's; the build skips the noise of the chunks its depth
           bias and the fBm bound decide (the roofline counts only the noise
           it evaluates).
  e2e      chunks/s through uww_build_chunks_host with pinned host buffers:
           descriptor upload, build, record/vertex/normal/index download.
  plain    chunks/s of the plain form: one launch per chunk (the drop-in of
           Chunk::build_full), same kernel code.
  exact    chunks/s of the parity build (reference f32 order, no FMA).

``--impl reference`` times the reference algorithm on the host cores instead:
the CPU oracle in reference semantics (f64 noise, O(V) linear dedup search,
powf colours), with all host threads, on the same workload: exactly --steps
timed steps, each a bounded slice of the grid, about 30 s in all.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import numpy as np  # noqa: E402

METRIC = "chunks/s (noise+MC, batched vs per-chunk) & fwd+adjoint Mvox/s on 1 GB300"
UNIT = "chunks/s"
N_SEEDS = 10

# Algorithmic FP32 work, counted on the parity kernel's formulation (one flop
# per add/sub/mul/div/floor, an FMA as 2), independent of how the fast kernel
# factors it:
FLOPS_PER_OCTAVE = 83          # one Perlin evaluation + fBm accumulate
FLOPS_PER_SAMPLE_EXTRA = 16    # world coordinates, normalisation, linear bias
FLOPS_PER_OCTAVE_GRAD = 254    # Perlin value + analytic gradient + accumulate (normals)
FLOPS_PER_VERTEX_EXTRA = 60    # interpolation, colour ramp, normalisation

# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one launch of
# the step's dominant kernel, front_kernel, on this workload, from a
# single-kernel ncu capture of this script's own step (-k regex:front_kernel
# -s 12 -c 1 of `bench.py --steps 5 --warmup 3 --quick --no-cpu
# --clock-window 0`, caches flushed before the launch): 186.4 KB read,
# 0.3 KB written.  Its staged output stays in L2 for the emission kernel, so this is
# far below the algorithmic output bytes.
NCU_DRAM_BYTES_PER_LAUNCH = 186_624
NCU_TRAFFIC_SOURCE = ("ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum -k regex:front_kernel -s 12 -c 1, "
                      "python bench.py --steps 5 --warmup 3 --quick --no-cpu --clock-window 0")
# FP32 flops the noise-stage kernel executes per launch of this workload
# (2 x FFMA + FADD + FMUL thread instructions, ncu sm__sass_thread_inst_executed_op_*_pred_on.sum,
# -k regex:sample_kernel_fast -s 3 -c 1 of the same command): the column form
# runs 4.3x fewer flops than the reference formulation counted above.
NCU_SAMPLE_EXECUTED_FLOPS = 728_236_800


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--plain-steps", type=int, default=2)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--quick", action="store_true", help="skip plain/exact/e2e legs (profiling runs)")
    ap.add_argument("--threads", type=int, default=0, help="threads per CTA (0: tuned/automatic)")
    ap.add_argument("--bps", type=int, default=0, help="resident CTAs per SM (0: tuned/automatic)")
    ap.add_argument("--no-fit", action="store_true", help="skip the terrain-fitting leg")
    ap.add_argument("--fit-steps", type=int, default=200, help="Adam steps of the terrain-fitting leg")
    ap.add_argument("--leg", default="", choices=["", "mixed_lod", "adjoint", "queries", "terrain_fit"],
                    help="with --quick: also run this one leg (profiling runs)")
    ap.add_argument("--clock-window", type=float, default=CLOCK_WINDOW_S,
                    help="seconds nvidia-smi watches the build (untimed steps fill what the timed ones leave); "
                         "0 for profiling runs that must launch few kernels")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in Path(self.path).read_text().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_model():
    try:
        for line in Path("/proc/cpuinfo").read_text().splitlines():
            if line.lower().startswith(("model name", "cpu model")):
                return line.split(":", 1)[1].strip()
        out = subprocess.run(["lscpu"], capture_output=True, text=True).stdout
        for line in out.splitlines():
            if line.startswith("Model name"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


def rank_seeds(rank: int):
    """The permutation seeds one rank cycles through: with N GPUs every rank
    builds the full grid with its own seeds (weak scaling, no exchange)."""
    return [(s + rank * N_SEEDS) % 1000 for s in range(N_SEEDS)]


def config_dict(n: int, l2: str = "flushed (256 MiB write) before each timed step") -> dict:
    """The workload both arms run; identical between them but for the L2 note."""
    return {"workload": "uniform grid: 16x16x16 = 4096 chunks of 12^3 cells (13^3 f32 samples), "
                        "4-oct fBm f=0.04 lac 2 pers 0.5, bias -0.03(z-128), iso 0; "
                        "outputs VertColor + normals + u32 indices",
            "chunks_per_step": n, "cells_per_step": n * 12 ** 3, "samples_per_step": n * 13 ** 3, "l2": l2}


def workload(seed):
    from underwaterworld_gb300 import layout, workloads
    return workloads.uniform_grid(seed=seed, outputs=layout.UWW_OUT_COLOR | layout.UWW_OUT_NORMALS)


def bias_decided_mask(params, descs) -> np.ndarray:
    """Which chunks the build decides from the depth bias alone (without their
    noise): a float32 restatement of the kernel's test (fBm bound
    1.11 * |norm| * sum|amp|, margin 1e-3 (1 + B + |bias|)), for the linear
    bias of the measured workloads; all False for the other bias modes."""
    f32 = np.float32
    amps = np.array([params.amplitude * params.persistence ** k for k in range(params.octaves)], np.float64)
    scale = f32(1.1547005383792515)
    norm = scale / f32(amps.sum()) if params.normalize else scale
    B = f32(1.11) * abs(norm) * f32(np.abs(amps).sum())
    cells = descs["cells"].astype(np.int64)
    oz = descs["pos"][:, 2].astype(np.int64) * 16
    s = (f32(16) / cells.astype(f32)).astype(f32)
    if params.bias_mode != 2:
        return np.zeros(len(descs), bool)
    b0 = f32(params.bias_a) * (oz.astype(f32) - f32(params.bias_b))
    b1 = f32(params.bias_a) * ((cells.astype(f32) * s + oz.astype(f32)).astype(f32) - f32(params.bias_b))
    lo, hi = np.minimum(b0, b1), np.maximum(b0, b1)
    m = f32(1e-3) * (f32(1) + B + np.maximum(np.abs(lo), np.abs(hi)))
    iso = f32(params.iso_level)
    return (lo - B - m > iso) | (hi + B + m < iso)


def bias_decided(params, descs) -> int:
    """How many chunks the depth bias decides; used to count the noise flops
    the build actually performs."""
    return int(bias_decided_mask(params, descs).sum())


def cpu_reference(descs, seeds, threads, budget_s=20.0):
    """The reference algorithm on the host: oracle in f64 reference semantics with
    the O(V) dedup search and colours (no normals, like the reference).  Whole
    grids, one seed each, until budget_s has passed.  Loads no GPU library."""
    from oracle import oracle as O
    from underwaterworld_gb300 import layout
    O.build()
    done, t0, i = 0, time.perf_counter(), 0
    while True:
        p, _ = workload(seeds[i % len(seeds)])
        p.outputs = layout.UWW_OUT_COLOR
        O.build_chunks(p, descs, precision=O.F64, search=O.SEARCH_LINEAR, threads=threads)
        done += len(descs)
        i += 1
        el = time.perf_counter() - t0
        if el > budget_s or i >= len(seeds):
            return done / el, done, el


REF_BUDGET_S = 150.0        # upper bound on the reference arm's timed steps
REF_ONE_THREAD_S = 10.0     # the single-threaded figure beside it


def run_reference(args):
    """The reference arm: the reference's algorithm (the CPU oracle in f64
    reference semantics, with its O(V) dedup search and colours) on every host
    core, for this arm's workload and metric.  It times exactly --steps steps;
    each step builds the whole 4096-chunk grid with the next seed, unless
    --steps whole grids would take longer than REF_BUDGET_S (measured on the
    warm-up steps), in which case each step builds a rotating slice of the
    grid sized to fit.  The reference itself is single-threaded
    (README.md:19), so a single-thread figure on whole grids is reported
    beside it.  Under torchrun, rank 0 alone runs it.  Nothing here loads the
    GPU library: the parameters and struct layouts come from
    underwaterworld_gb300.layout."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from oracle import oracle as O
    from underwaterworld_gb300 import layout
    O.build()
    _, descs = workload(0)
    n = len(descs)
    threads = os.cpu_count() or 1
    params = []
    for seed in range(N_SEEDS):
        p, _ = workload(seed)
        p.outputs = layout.UWW_OUT_COLOR
        params.append(p)

    def build(p, d, th=threads):
        O.build_chunks(p, d, precision=O.F64, search=O.SEARCH_LINEAR, threads=th)

    def step_slice(s, size):
        if size >= n:
            return descs
        idx = (s * size + np.arange(size)) % n
        return layout.make_descs(descs["pos"][idx], descs["cells"][idx])

    steps = max(1, args.steps)
    wt = []
    for w in range(max(args.warmup, 1)):
        t0 = time.perf_counter()
        build(params[w % N_SEEDS], descs)
        wt.append(time.perf_counter() - t0)
    grid_s = min(wt)
    per_step = n if steps * grid_s <= REF_BUDGET_S else int(max(32, n * REF_BUDGET_S / (steps * grid_s)))
    elapsed = 0.0
    for s in range(steps):
        d = step_slice(s, per_step)
        t0 = time.perf_counter()
        build(params[s % N_SEEDS], d)
        elapsed += time.perf_counter() - t0
    value = steps * per_step / elapsed
    one_v, one_n, one_el = cpu_reference(descs, list(range(N_SEEDS)), 1, budget_s=REF_ONE_THREAD_S)
    cpu = cpu_model()
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * elapsed / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config_dict(n, l2="n/a (host CPU)"),
        "build": "CPU oracle, reference semantics (f64 noise, O(V) dedup search)", "threads": threads, "device": f"host CPU cores, no GPU used ({cpu})",
        "chunks_per_timed_step": per_step,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{per_step} chunks per step ({'the whole 4096-chunk grid' if per_step >= n else 'a rotating slice of the 4096-chunk grid'}, "
                                   f"seeds cycling), {steps} steps in {elapsed:.1f} s, {threads} threads, CPU: {cpu}"},
        "single_thread": {"value": one_v, "unit": UNIT, "cores": 1,
                          "sample": f"{one_n} chunks ({one_n // n} whole grids, seeds 0..) in {one_el:.1f} s, 1 thread "
                                    f"(the reference is single-threaded)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def timed(stream, fn, flush=None):
    """Device time of fn() on stream, in seconds (L2 flushed first if given)."""
    import torch
    if flush is not None:
        flush.zero_()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    fn()
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1) * 1e-3


CLOCK_WINDOW_S = 2.0   # nvidia-smi watches the timed build at least this long


def probe_lib():
    """The benchmark's measurement kernels (libuww_bench_probe.so)."""
    from underwaterworld_gb300 import build as B
    L = C.CDLL(str(B.build_probe()))
    L.bench_probe_fma.argtypes = [C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p, C.POINTER(C.c_double)]
    L.bench_probe_fma.restype = C.c_int
    L.bench_probe_host_write.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_uint32, C.c_void_p]
    L.bench_probe_host_write.restype = C.c_int
    return L


def leg_fp32_peak(stream, dev, sms, gpu_index, window_s=1.0):
    """FP32 peak: the FMA probe (8 CTAs of 256 threads per SM, 8 independent
    FMA chains per thread), timed launch by launch for about window_s with
    nvidia-smi sampling the clocks; reported as measured (the fastest launch)
    and as SMs x 128 lanes x 2 flops x the median SM clock under the probe."""
    import torch
    PL = probe_lib()
    blocks = sms * 8
    sink = torch.empty(blocks * 256, dtype=torch.float32, device=dev)
    fl = C.c_double()
    h = C.c_void_p(stream.cuda_stream)
    for _ in range(3):
        assert PL.bench_probe_fma(blocks, 4096, C.c_void_p(sink.data_ptr()), h, C.byref(fl)) == 0
    torch.cuda.synchronize()
    clk = ClockSampler(gpu_index)
    clk.start()
    rates, t0 = [], time.perf_counter()
    while time.perf_counter() - t0 < window_s or len(rates) < 5:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        PL.bench_probe_fma(blocks, 4096, C.c_void_p(sink.data_ptr()), h, C.byref(fl))
        e1.record(stream)
        e1.synchronize()
        rates.append(fl.value / (e0.elapsed_time(e1) * 1e-3))
    c = clk.stop()
    mhz = c.get("sm_mhz")
    return {"measured_tflops": max(rates) / 1e12, "median_tflops": statistics.median(rates) / 1e12,
            "launches": len(rates), "sm_mhz_median": mhz, "clock_samples": c.get("samples"),
            "reasons": c.get("reasons"), "sms": sms,
            "clock_peak_tflops": sms * 128 * 2 * mhz * 1e6 / 1e12 if mhz else None,
            "kernel": "bench_probe_fma (libuww_bench_probe.so)"}


def leg_host_link(stream, dev, sms, nbytes, steps=20):
    """Device-to-host bandwidth for one step's output size: a pinned
    cudaMemcpyAsync (copy engine) and SM stores into the same pinned buffer
    (how the streamed host output of the batched build moves)."""
    import torch
    PL = probe_lib()
    nbytes = (nbytes + 15) // 16 * 16
    d = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    h = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    hs = C.c_void_p(stream.cuda_stream)

    def ce():
        h.copy_(d, non_blocking=True)

    def sm():
        assert PL.bench_probe_host_write(C.c_void_p(d.data_ptr()), C.c_void_p(h.data_ptr()), nbytes, sms * 4, hs) == 0

    res = {"bytes": nbytes}
    for name, fn in (("copy_engine_gbs", ce), ("sm_store_gbs", sm)):
        for _ in range(3):
            fn()
        t = statistics.median([timed(stream, fn) for _ in range(steps)])
        res[name] = nbytes / t / 1e9
    return res


def leg_no_shortcut(ctx, L, d_desc, n, out, out_t, params, flush, stream, steps, tuning):
    """The batched build with the depth-bias shortcut off
    (UWW_TUNE_NO_DEPTH_SHORTCUT): every chunk evaluates its noise, as every
    chunk of the reference samples its grid before the blank check
    (chunk.rs:131-133).  Same output; its per-chunk cost and FP32 roofline."""
    from underwaterworld_gb300 import abi
    ctx.set_tuning(*tuning, options=abi.UWW_TUNE_NO_DEPTH_SHORTCUT)
    ts, vs = [], []
    for i in range(steps + 3):
        ctx.set_params(params[i % N_SEEDS])

        def run():
            abi.check(L.uww_build_chunks(ctx.h, C.c_void_p(d_desc.data_ptr()), n, 12, C.byref(out)), "build")

        t = timed(stream, run, flush)
        tot = out_t["totals"].cpu().numpy()
        assert int(tot[2]) == 0 and int(tot[3]) == 0, tot
        if i >= 3:
            ts.append(t)
            vs.append(int(tot[0]))
    ctx.set_tuning(*tuning, options=0)
    mean = statistics.mean(ts)
    K = params[0].octaves
    flops = n * 13 ** 3 * (K * FLOPS_PER_OCTAVE + FLOPS_PER_SAMPLE_EXTRA) + \
        statistics.mean(vs) * (K * FLOPS_PER_OCTAVE_GRAD + FLOPS_PER_VERTEX_EXTRA)
    return {"chunks_per_s": n / mean, "us_per_step": mean * 1e6, "steps": steps, "flops_per_step": flops,
            "tflops": flops / mean / 1e12}


def leg_fast_vs_f64(params, descs, seeds):
    """Accuracy of the fast build (the one `value` times) against the F64
    oracle -- the reference's f64 noise (perlin_util.rs:6-29) -- on the whole
    grid for each seed, outside every timed region: flipped cells (case
    indices that differ) and the vertex position error over the chunks with
    identical index buffers."""
    from oracle import oracle as O
    from underwaterworld_gb300 import abi
    from underwaterworld_gb300.chunk import Context
    rows = []
    for seed in seeds:
        p = params[seed % len(params)].copy()
        p.outputs = abi.UWW_OUT_CASES
        p.math_mode = abi.UWW_MATH_FAST
        ref_p = p.copy()
        ref_p.math_mode = abi.UWW_MATH_EXACT
        ref = O.build_chunks(ref_p, descs, precision=O.F64, threads=os.cpu_count() or 1)
        with Context(p) as c:
            got = c.build_chunks_device(descs, int(ref.totals[0]) + 4096, int(ref.totals[1]) + 16384)
        assert got.status == abi.UWW_OK, got.status
        rows.append(O.fast_vs_reference(got, ref))
    return {"seeds": list(seeds), "cells": sum(r["cells"] for r in rows),
            "flipped_cells": sum(r["flipped_cells"] for r in rows),
            "max_vertex_err": max(r["max_vertex_err"] for r in rows),
            "median_vertex_err": float(np.median([r["median_vertex_err"] for r in rows])),
            "vertices_compared": sum(r["vertices_compared"] for r in rows),
            "unit": "world units (a cell is 16/12)", "oracle": "F64 CPU oracle (reference semantics)"}


def leg_noise_stage(ctx, stream, flush, params, descs, steps, warmup):
    """The noise stage alone: uww_sample_chunks (Chunk::build_iso for the batch)
    on the uniform grid, samples written to HBM; FP32 roofline of the algorithmic
    count (FLOPS_PER_OCTAVE per sample-octave + FLOPS_PER_SAMPLE_EXTRA)."""
    import torch
    from underwaterworld_gb300 import abi
    n = len(descs)
    ctx.set_params(params)
    ns = n * 13 ** 3
    out = torch.empty(ns, dtype=torch.float32, device=stream.device)
    d_desc = torch.from_numpy(descs.view(np.uint8).copy()).to(stream.device)
    L = abi.lib()

    def run():
        abi.check(L.uww_sample_chunks(ctx.h, C.c_void_p(d_desc.data_ptr()), n, 12, C.c_void_p(out.data_ptr()), ns),
                  "sample")

    for _ in range(warmup):
        run()
    ts = [timed(stream, run, flush) for _ in range(steps)]
    t = statistics.median(ts)
    flops = ns * (params.octaves * FLOPS_PER_OCTAVE + FLOPS_PER_SAMPLE_EXTRA)
    return {"us": t * 1e6, "samples": ns, "msamples_per_s": ns / t / 1e6, "tflops": flops / t / 1e12,
            "flops_per_step": flops, "bytes_written": ns * 4}


def leg_frame_graph(ctx, params, descs, steps, warmup):
    """Uniform grid as a per-frame CUDA graph: descriptor + count upload, build,
    record + totals download, one graph launch per frame; host wall time."""
    from underwaterworld_gb300.frame import FrameBuilder
    n = len(descs)
    ctx.set_params(params)
    fb = FrameBuilder(ctx, n, 12, 1 << 20, 1 << 22)
    for _ in range(warmup):
        fb.build(descs)
    t = []
    for _ in range(steps):
        t0 = time.perf_counter()
        fb.build(descs)
        t.append(time.perf_counter() - t0)
    fb.close()
    return {"chunks_per_s": n / statistics.median(t), "ms_per_frame": 1e3 * statistics.median(t),
            "h2d_bytes_per_frame": n * 32 + 4, "d2h_bytes_per_frame": n * 32 + 32,
            "note": "uww_frame_launch + sync, host wall clock, median"}


def leg_mixed_lod(stream, flush, steps, warmup):
    """Uneven LOD batch (2048 chunks, 12^3/24^3/48^3 at 50/35/15 %, 6-octave fBm)
    in one build call (the split build: its 24^3 and 48^3 chunks as x slabs),
    autotuned (cached per config); p50/p99 latency."""
    import torch
    from underwaterworld_gb300 import abi, workloads
    from underwaterworld_gb300.chunk import Context
    from underwaterworld_gb300.frame import autotune
    p, d = workloads.mixed_lod(seed=0, outputs=abi.UWW_OUT_COLOR | abi.UWW_OUT_NORMALS)
    p.math_mode = abi.UWW_MATH_FAST
    n = len(d)
    ctx = Context(p, stream=stream.cuda_stream)
    dev = torch.device("cuda", torch.cuda.current_device())
    vcap, icap = 1 << 23, 1 << 25
    bufs = {k: torch.empty(b, dtype=torch.uint8, device=dev) for k, b in
            (("v", vcap * 24), ("nrm", vcap * 12), ("i", icap * 4), ("r", n * 32), ("t", 32))}
    d_desc = torch.from_numpy(d.view(np.uint8).copy()).to(dev)
    out = abi.MeshOut(bufs["v"].data_ptr(), bufs["nrm"].data_ptr(), bufs["i"].data_ptr(), None, None,
                      bufs["r"].data_ptr(), bufs["t"].data_ptr(), vcap, icap, 0, 0)
    cache = ROOT / "underwaterworld_gb300" / "_build" / "tune_cache.txt"
    tun, tuned_us = autotune(ctx, d_desc.data_ptr(), n, 48, out, str(cache))
    shape = ctx.launch_shape(n, 48)
    L = abi.lib()

    def step():
        abi.check(L.uww_build_chunks(ctx.h, C.c_void_p(d_desc.data_ptr()), n, 48, C.byref(out)), "mixed build")

    for _ in range(warmup):
        step()
    lat = [timed(stream, step, flush) for _ in range(steps)]
    tot = bufs["t"].view(torch.int64).cpu().numpy()
    assert int(tot[2]) == 0 and int(tot[3]) == 0, tot
    cells = int((d["cells"].astype(np.int64) ** 3).sum())
    samples = int(((d["cells"].astype(np.int64) + 1) ** 3).sum())
    ctx.close()
    lat_ms = np.array(lat) * 1e3
    mean = float(np.mean(lat))
    return {"chunks": n, "cells": cells, "samples": samples, "chunks_per_s": n / mean,
            "mvoxels_per_s": cells / mean / 1e6, "p50_ms": float(np.percentile(lat_ms, 50)),
            "p99_ms": float(np.percentile(lat_ms, 99)), "steps": steps,
            "tuning": {"threads": tun.threads, "blocks_per_sm": tun.blocks_per_sm, "smem_cells": tun.smem_cells,
                       "tuned_us": tuned_us},
            "build": {"kind": "split" if shape.build == abi.UWW_BUILD_SPLIT else "pipelined",
                      "slabs_per_chunk": shape.slabs_per_chunk, "threads": shape.threads, "grid": shape.grid,
                      "blocks_per_sm": shape.blocks_per_sm},
            "verts": int(tot[0]), "inds": int(tot[1])}


def leg_adjoint(stream, flush, steps, warmup):
    """Adjoint batch: 512 chunks of 24^3 cells, 4-octave fBm; forward (build +
    edge ids) then backward (dL/dtheta, dL/dsamples) with seeded cotangents."""
    from underwaterworld_gb300 import abi, workloads
    from underwaterworld_gb300.adjoint import Adjoint
    from underwaterworld_gb300.chunk import Context
    p, d = workloads.adjoint_batch(seed=0)
    p.math_mode = abi.UWW_MATH_FAST
    ctx = Context(p, stream=stream.cuda_stream)
    a = Adjoint(ctx, d, 1 << 21, 1 << 23, sample_grad=True)
    a.forward()
    f = a.fetch_forward()
    a.set_pos_grad(workloads.cotangents(f["records"], f["edge_ids"], seed=0))

    def fb():
        a.forward()
        a.backward()

    for _ in range(warmup):
        fb()
    tf = [timed(stream, a.forward, flush) for _ in range(steps)]
    tb = [timed(stream, a.backward, flush) for _ in range(steps)]
    tfb = [timed(stream, fb, flush) for _ in range(steps)]
    g = a.theta_grad()
    cells = len(d) * 24 ** 3
    ctx.close()
    m = statistics.mean(tfb)
    return {"chunks": len(d), "cells": cells, "verts": int(f["totals"][0]),
            "fwd_ms": 1e3 * statistics.mean(tf), "bwd_ms": 1e3 * statistics.mean(tb), "fwd_bwd_ms": 1e3 * m,
            "fwd_adjoint_mvoxels_per_s": cells / m / 1e6, "theta_grad_finite": bool(np.all(np.isfinite(g)))}


def leg_terrain_fit(stream, steps=200):
    """Terrain fitting: 512^3 cells as 32^3 chunks of 16^3, 8-octave fBm; Adam
    (lr 1e-2) on theta for `steps` steps toward an 8-Gaussian heightmap."""
    import torch
    from underwaterworld_gb300.adjoint import TerrainFit, gaussian_heightmap, terrain_volume
    from underwaterworld_gb300.chunk import Context
    p, d = terrain_volume(chunks_per_edge=32, cells=16, octaves=8, seed=0)
    free0, total = torch.cuda.mem_get_info()
    ctx = Context(p, stream=stream.cuda_stream)
    target = gaussian_heightmap(16, 32.0, n_bumps=8, seed=0, base=128.0)
    fit = TerrainFit(ctx, d, target, 32.0, vert_capacity=1 << 23, ind_capacity=1 << 25, lr=1e-2)
    min_free = torch.cuda.mem_get_info()[0]
    losses, t0 = [], time.perf_counter()
    for _ in range(steps):
        loss, _ = fit.step()
        losses.append(loss)
        min_free = min(min_free, torch.cuda.mem_get_info()[0])
    el = time.perf_counter() - t0
    # device time of one forward+backward at the final theta
    def fb():
        fit.adj.forward()
        fit.adj.backward()
    fb()
    tfb = statistics.mean([timed(stream, fb) for _ in range(5)])
    cells = len(d) * 16 ** 3
    rmse0, rmse1 = float(np.sqrt(losses[0])), float(np.sqrt(losses[-1]))
    g = fit.last_grad
    ctx.close()
    tail = losses[-20:]
    return {"cells": cells, "steps": steps, "seconds": el, "step_ms": 1e3 * el / steps,
            "fwd_bwd_ms": 1e3 * tfb, "fwd_adjoint_mvoxels_per_s": cells / tfb / 1e6,
            "loss_first": losses[0], "loss_last": losses[-1], "rms_height_error_first": rmse0,
            "rms_height_error_last": rmse1, "peak_device_bytes": int(free0 - min_free),
            "final_grad_norm": float(np.linalg.norm(g)),
            "final_scaled_grad_norm": float(np.linalg.norm(g * fit.scale)),
            "loss_change_last_20_steps": float((tail[-1] - tail[0]) / tail[0])}


def leg_queries(stream, flush, steps):
    """The callers around the build (§8f rows): point density queries
    (perlin_util::iso_at for 1M points), boid wall rays (100k boids x 18 rays
    against the reference grid's mesh), the scheduler feed (update_nearby), and
    the terrain shading pass over the uniform grid's vertices."""
    import torch
    from underwaterworld_gb300 import abi, workloads
    from underwaterworld_gb300.chunk import Context, DeviceArray
    from underwaterworld_gb300.query import RayScene
    from underwaterworld_gb300.schedule import Scheduler, schedule_params
    res = {}
    L = abi.lib()
    dev = stream.device
    # point queries on the uniform grid's density
    p, d = workloads.uniform_grid(seed=0, outputs=abi.UWW_OUT_COLOR)
    p.math_mode = abi.UWW_MATH_FAST
    ctx = Context(p, stream=stream.cuda_stream)
    npts = 1 << 20
    g = torch.Generator(device="cpu").manual_seed(0)
    xyz = (torch.rand(npts, 3, generator=g) * 256.0).to(dev)
    dens = torch.empty(npts, device=dev)
    run = lambda: abi.check(L.uww_density_at(ctx.h, C.c_void_p(xyz.data_ptr()), npts, C.c_void_p(dens.data_ptr())))
    run()
    t = statistics.median([timed(stream, run, flush) for _ in range(steps)])
    res["density_at"] = {"points": npts, "us": t * 1e6, "mpoints_per_s": npts / t / 1e6}
    ctx.close()
    # boid wall rays against the reference grid (iso -0.1, exact build)
    p, d = workloads.reference_grid(outputs=abi.UWW_OUT_CASES)
    ctx = Context(p, stream=stream.cuda_stream)
    sc = RayScene(ctx, d)
    b = sc.batch()
    nq, nr = 100_000, 18
    rng = np.random.default_rng(0)
    origins = (b.verts["pos"][rng.integers(0, len(b.verts), nq)] + rng.normal(0, 1.5, (nq, 3))).astype(np.float32)
    dirs = rng.normal(size=(nq, nr, 3)).astype(np.float32)
    dirs /= np.linalg.norm(dirs, axis=-1, keepdims=True)
    d_o, d_d = ctx.upload(origins), ctx.upload(dirs.astype(np.float32))
    d_t = DeviceArray(nq * nr * 4)
    run = lambda: abi.check(L.uww_ray_query(ctx.h, C.byref(sc.scene), C.c_void_p(d_o.ptr), nq, C.c_void_p(d_d.ptr),
                                            nr, 3, C.c_void_p(d_t.ptr)))
    run()
    t = statistics.median([timed(stream, run, flush) for _ in range(steps)])
    res["ray_query"] = {"boids": nq, "rays_per_boid": nr, "us": t * 1e6, "mrays_per_s": nq * nr / t / 1e6}
    # scheduler feed with the reference grid as the known chunks
    size = 1 << int(2 * len(d) - 1).bit_length()
    d_tab = DeviceArray(size * 4)
    abi.check(L.uww_chunk_index(ctx.h, C.c_void_p(sc.d_desc.ptr), len(d), C.c_void_p(d_tab.ptr), size))
    sch = Scheduler(ctx)
    sp = schedule_params(np.array([3.0, -2.0, 1.0], np.float32), np.array([-3.0, -2.0, 2.0], np.float32),
                         np.array([4.0, -2.0, 1.0], np.float32))
    known = (sc.d_desc.ptr, sc.d_rec.ptr, d_tab.ptr, size)
    run = lambda: sch.run(sp, known)
    run()
    t = statistics.median([timed(stream, run) for _ in range(steps)])
    gen, ren, counts = sch.fetch()
    res["schedule"] = {"us": t * 1e6, "candidates": 10 * 10 * 5, "generate": int(counts[0]), "render": int(counts[1])}
    ctx.close()
    # terrain shading over the uniform grid's mesh
    p, d = workloads.uniform_grid(seed=0, outputs=abi.UWW_OUT_COLOR)
    p.math_mode = abi.UWW_MATH_FAST
    ctx = Context(p, stream=stream.cuda_stream)
    vcap = 1 << 20
    d_desc = ctx.upload(d)
    bufs = [DeviceArray(vcap * 24), DeviceArray(4 << 22), DeviceArray(len(d) * 32), DeviceArray(32)]
    out = abi.MeshOut(bufs[0].ptr, None, bufs[1].ptr, None, None, bufs[2].ptr, bufs[3].ptr, vcap, 1 << 22, 0, 0)
    abi.check(L.uww_build_chunks(ctx.h, C.c_void_p(d_desc.ptr), len(d), 12, C.byref(out)))
    ctx.sync()
    nv = int(ctx.download(bufs[3], (4,), np.uint64)[0])
    cam = abi.CameraUniform()
    for i in range(16):
        cam.view_proj[i] = 1.0 if i % 5 == 0 else 0.0
    for i in range(3):
        cam.sub_pos[i], cam.sub_forward[i], cam.fog_color[i] = 128.0, (1.0, 0.0, 0.0)[i], 0.1
    d_clip, d_rgb = DeviceArray(vcap * 16), DeviceArray(vcap * 12)
    run = lambda: abi.check(L.uww_shade_vertices(ctx.h, C.byref(cam), C.c_void_p(bufs[0].ptr), C.c_void_p(bufs[3].ptr),
                                                 0, vcap, C.c_void_p(d_clip.ptr), C.c_void_p(d_rgb.ptr), None))
    run()
    t = statistics.median([timed(stream, run, flush) for _ in range(steps)])
    res["shade"] = {"vertices": nv, "us": t * 1e6, "mverts_per_s": nv / t / 1e6}
    ctx.close()
    return res


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    rank, world, local = dist_env()
    import torch
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)

    from underwaterworld_gb300 import abi, build as B
    from underwaterworld_gb300.chunk import Context, HostArray
    B.build()
    L = abi.lib()
    # One explicit stream for everything: the library's launches, torch's own
    # work (L2 flush, copies) and the timing events.  (The default stream's
    # handle is 0, which would make the library create a stream of its own.)
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)
    assert stream.cuda_stream != 0

    params, descs = [], None
    for s in rank_seeds(rank):
        p, d = workload(s)
        p.math_mode = abi.UWW_MATH_FAST
        params.append(p)
        descs = d
    n = len(descs)
    ctx = Context(params[0], stream=stream.cuda_stream)
    if args.threads or args.bps:
        ctx.set_tuning(threads=args.threads, blocks_per_sm=args.bps)

    d_desc = torch.from_numpy(descs.view(np.uint8).copy()).to(dev)
    # capacity: one sizing pass per seed
    vcap, icap = 1 << 20, 1 << 22
    out_t = {}

    def alloc(vc, ic):
        out_t["verts"] = torch.empty(vc * 24, dtype=torch.uint8, device=dev)
        out_t["normals"] = torch.empty(vc * 12, dtype=torch.uint8, device=dev)
        out_t["inds"] = torch.empty(ic * 4, dtype=torch.uint8, device=dev)
        out_t["records"] = torch.empty(n * 32, dtype=torch.uint8, device=dev)
        out_t["totals"] = torch.zeros(4, dtype=torch.int64, device=dev)
        return abi.MeshOut(out_t["verts"].data_ptr(), out_t["normals"].data_ptr(), out_t["inds"].data_ptr(), None,
                           None, out_t["records"].data_ptr(), out_t["totals"].data_ptr(), vc, ic)

    out = alloc(vcap, icap)
    maxv = maxi = 0
    for p in params:
        ctx.set_params(p)
        abi.check(L.uww_build_chunks(ctx.h, C.c_void_p(d_desc.data_ptr()), n, 12, C.byref(out)), "build")
        tot = out_t["totals"].cpu().numpy()
        maxv, maxi = max(maxv, int(tot[0])), max(maxi, int(tot[1]))
    vcap, icap = int(maxv * 1.1) + 1024, int(maxi * 1.1) + 4096
    out = alloc(vcap, icap)

    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def step(i, o=None):
        ctx.set_params(params[i % N_SEEDS])
        abi.check(L.uww_build_chunks(ctx.h, C.c_void_p(d_desc.data_ptr()), n, 12, C.byref(o or out)), "build")

    for i in range(args.warmup):
        step(i)
    torch.cuda.synchronize()
    tot = out_t["totals"].cpu().numpy()
    assert int(tot[2]) == 0 and int(tot[3]) == 0, tot

    # ---- timed batched steps ----
    clocks = ClockSampler(local)
    clocks.start()
    t_window = time.perf_counter()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    times, verts_sum, inds_sum = [], 0, 0
    for i in range(args.steps):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step(i)
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1) * 1e-3)
        tot = out_t["totals"].cpu().numpy()
        # a step that overflowed or timed out is not counted as built
        assert int(tot[2]) == 0 and int(tot[3]) == 0, ("timed step", i, tot)
        verts_sum += int(tot[0])
        inds_sum += int(tot[1])
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    # the timed steps of a short run end before nvidia-smi's first samples:
    # keep running the same step, untimed, until the sampler has watched it
    # for CLOCK_WINDOW_S
    extra_steps = 0
    while time.perf_counter() - t_window < args.clock_window:
        flush.zero_()
        step(args.steps + extra_steps)
        extra_steps += 1
        if extra_steps % 16 == 0:
            torch.cuda.synchronize()
    torch.cuda.synchronize()
    clk = clocks.stop()
    clk["window_s"] = round(time.perf_counter() - t_window, 2)
    clk["note"] = (f"sampled every 100 ms over the {args.steps} timed steps and {extra_steps} more untimed steps "
                   f"of the same build")
    t_total = sum(times)
    if world > 1:
        tt = torch.tensor([t_total], device=dev, dtype=torch.float64)
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        t_total = float(tt.item())
    value = world * n * args.steps / t_total
    ms_step = 1e3 * t_total / args.steps

    extra = {}
    if not args.quick:
        # ---- exact (parity) build ----
        ex_times = []
        for i in range(max(3, args.steps // 2)):
            q = params[i % N_SEEDS].copy()
            q.math_mode = abi.UWW_MATH_EXACT
            ctx.set_params(q)
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            abi.check(L.uww_build_chunks(ctx.h, C.c_void_p(d_desc.data_ptr()), n, 12, C.byref(out)), "build")
            e1.record(stream)
            e1.synchronize()
            ex_times.append(e0.elapsed_time(e1) * 1e-3)
            tot = out_t["totals"].cpu().numpy()
            assert int(tot[2]) == 0 and int(tot[3]) == 0, ("exact step", i, tot)
        extra["exact_chunks_per_s"] = n / statistics.mean(ex_times)

        # ---- plain: one launch per chunk, each into its own slot ----
        ctx.set_params(params[0])
        per = 15 * 12 ** 3
        pv = torch.empty(n * per * 24, dtype=torch.uint8, device=dev)
        pn = torch.empty(n * per * 12, dtype=torch.uint8, device=dev)
        pi = torch.empty(n * per * 4, dtype=torch.uint8, device=dev)
        pr = torch.empty(n * 32, dtype=torch.uint8, device=dev)
        pt = torch.empty(n * 32, dtype=torch.uint8, device=dev)
        outs = [abi.MeshOut(pv.data_ptr() + k * per * 24, pn.data_ptr() + k * per * 12, pi.data_ptr() + k * per * 4,
                            None, None, pr.data_ptr() + 32 * k, pt.data_ptr() + 32 * k, per, per) for k in range(n)]
        base = d_desc.data_ptr()
        fn = L.uww_build_chunk_plain
        for k in range(64):
            fn(ctx.h, C.c_void_p(base + 32 * k), 12, C.byref(outs[k]))
        torch.cuda.synchronize()
        pl = []
        for _ in range(args.plain_steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for k in range(n):
                fn(ctx.h, C.c_void_p(base + 32 * k), 12, C.byref(outs[k]))
            e1.record(stream)
            e1.synchronize()
            pl.append(e0.elapsed_time(e1) * 1e-3)
        extra["plain_chunks_per_s"] = n / statistics.mean(pl)
        del pv, pn, pi

        # ---- e2e through the host-buffer API with pinned buffers ----
        h_desc = HostArray((n,), abi.CHUNK_DESC_DTYPE)
        h_desc.array[:] = descs
        h_rec = HostArray((n,), abi.CHUNK_RECORD_DTYPE)
        h_v = HostArray((vcap,), abi.VERT_COLOR_DTYPE)
        h_n = HostArray((vcap, 3), np.float32)
        h_i = HostArray((icap,), np.uint32)
        h_t = np.zeros(4, np.uint64)
        hout = abi.MeshOut(h_v.ptr, h_n.ptr, h_i.ptr, None, None, h_rec.ptr, h_t.ctypes.data, vcap, icap)
        e2e_t, h2d, d2h = [], 0, 0
        for i in range(args.warmup + args.steps):
            ctx.set_params(params[i % N_SEEDS])
            t0 = time.perf_counter()
            abi.check(L.uww_build_chunks_host(ctx.h, C.c_void_p(h_desc.ptr), n, C.byref(hout)), "host build")
            t1 = time.perf_counter()
            if i >= args.warmup:
                e2e_t.append(t1 - t0)
                h2d += n * 32
                d2h += n * 32 + 32 + int(h_t[0]) * (24 + 12) + int(h_t[1]) * 4
        k = len(e2e_t)
        extra["e2e"] = {"value": world * n / statistics.mean(e2e_t), "unit": UNIT,
                        "h2d_bytes_per_step": h2d // k, "d2h_bytes_per_step": d2h // k}

    extra["noise_stage"] = leg_noise_stage(ctx, stream, flush, params[0], descs, max(10, min(args.steps, 200)), 3)
    if args.quick and args.leg:
        if args.leg == "mixed_lod":
            extra["mixed_lod"] = leg_mixed_lod(stream, flush, max(5, min(args.steps, 200)), 3)
        elif args.leg == "adjoint":
            extra["adjoint"] = leg_adjoint(stream, flush, max(5, min(args.steps, 50)), 3)
        elif args.leg == "queries":
            extra["queries"] = leg_queries(stream, flush, max(5, min(args.steps, 50)))
        else:
            extra["terrain_fit"] = leg_terrain_fit(stream, args.fit_steps)
    tuning = (args.threads, args.bps)
    if not args.quick:
        extra["no_depth_shortcut"] = leg_no_shortcut(ctx, L, d_desc, n, out, out_t, params, flush, stream,
                                                     max(5, min(args.steps, 200)), tuning)
        extra["host_link"] = leg_host_link(stream, dev, torch.cuda.get_device_properties(dev).multi_processor_count,
                                           extra["e2e"]["d2h_bytes_per_step"])
        extra["frame_graph"] = leg_frame_graph(ctx, params[0], descs, max(5, min(args.steps, 50)), 3)
        extra["mixed_lod"] = leg_mixed_lod(stream, flush, max(10, min(args.steps, 200)), 3)
        extra["adjoint"] = leg_adjoint(stream, flush, max(5, min(args.steps, 50)), 3)
        extra["queries"] = leg_queries(stream, flush, max(5, min(args.steps, 50)))
        if not args.no_fit:
            extra["terrain_fit"] = leg_terrain_fit(stream, args.fit_steps)

    # ---- FP32 peak probe (roofline denominator) ----
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    peak = leg_fp32_peak(stream, dev, sms, local)
    fp32_peak = peak["measured_tflops"]
    extra["fp32_peak"] = peak

    # the noise flops the build performs: chunks decided by the depth bias
    # alone evaluate none
    decided = bias_decided(params[0], descs)
    samples = (n - decided) * 13 ** 3
    mean_v, mean_i = verts_sum / args.steps, inds_sum / args.steps
    oct_ = params[0].octaves
    flops = samples * (oct_ * FLOPS_PER_OCTAVE + FLOPS_PER_SAMPLE_EXTRA) + \
        mean_v * (oct_ * FLOPS_PER_OCTAVE_GRAD + FLOPS_PER_VERTEX_EXTRA)
    achieved = flops / (t_total / args.steps) / 1e12
    # algorithmic bytes of the mesh emission: VertColor + normal per vertex, u32
    # per index, the record per chunk written; the descriptor per chunk read
    out_bytes = mean_v * (24 + 12) + mean_i * 4 + n * (32 + 32)
    hbm_peak, hbm_src = 6800.0, "fallback"
    try:
        hbm_peak = float(json.loads((ROOT / "MEASURED_PEAKS.json").read_text())["hbm_gbs"])
        hbm_src = "measured (copy bandwidth)"
    except (OSError, ValueError, KeyError):
        pass

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded chunk grid; seeds 0-9 cycle per step)",
        "config": config_dict(n),
        "build": "fast (FMA), split build: depth-bias planning into cost-ranked work queues (chunks it decides "
                 "settled without their noise), persistent front kernel (noise, classification, chunk-local "
                 "pass 1 staged), emission kernel as its programmatic dependent (records, colour/normal "
                 "blocks, index blocks)",
        "mean_verts_per_step": mean_v, "mean_inds_per_step": mean_i, "chunks_decided_by_depth_bias": decided,
        "mvoxels_per_s": value * 12 ** 3 / 1e6,
        "msamples_per_s": value * 13 ** 3 / 1e6,
        # per step: the planning kernel, the front kernel, the emission kernel
        "gpu_launches": args.steps * 3,
        "clocks": clk,
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": achieved / fp32_peak, "traffic": NCU_DRAM_BYTES_PER_LAUNCH,
                     "peak_source": f"measured live: FMA probe kernel, {sms}x8 CTAs, at a median "
                                    f"{peak['sm_mhz_median']} MHz (SMs x 128 x 2 x clock = "
                                    f"{peak['clock_peak_tflops']} TFLOP/s); the measured-peaks file has no FP32 entry",
                     "traffic_source": NCU_TRAFFIC_SOURCE,
                     "kernel": "front_kernel (the noise of the evaluated chunks); achieved over the whole step "
                               "(planning + front + emission), a lower bound on the front kernel's own rate",
                     "flops_per_step": flops,
                     "emission": {"bound": "hbm", "achieved": out_bytes / (t_total / args.steps) / 1e9,
                                  "peak": hbm_peak, "unit": "GB/s",
                                  "frac": out_bytes / (t_total / args.steps) / 1e9 / hbm_peak,
                                  "bytes_per_step": out_bytes, "peak_source": hbm_src}},
    }
    ns_leg = extra.get("noise_stage")
    if ns_leg:
        ns_leg["frac_of_fp32_peak"] = ns_leg["tflops"] / fp32_peak
        executed = NCU_SAMPLE_EXECUTED_FLOPS / (ns_leg["us"] * 1e-6) / 1e12
        line["roofline"]["noise_stage"] = {"bound": "fp32", "achieved": ns_leg["tflops"], "peak": fp32_peak,
                                           "unit": "TFLOP/s", "frac": ns_leg["tflops"] / fp32_peak,
                                           "flops": "algorithmic: the reference formulation's 348 per sample",
                                           "executed_tflops": executed, "executed_frac": executed / fp32_peak,
                                           "executed_flops_source": "ncu FP32 instruction counts of one launch "
                                                                    "(profiles/sample_kernel_fast_uniform_grid_4096.md)",
                                           "kernel": "sample_kernel_fast (uww_sample_chunks), 4096 x 13^3 samples"}
    line.update({k: v for k, v in extra.items() if k != "e2e"})
    if "adjoint" in extra:
        line["fwd_adjoint_mvoxels_per_s"] = extra["adjoint"]["fwd_adjoint_mvoxels_per_s"]
    if "e2e" in extra:
        line["e2e"] = extra["e2e"]
    if "plain_chunks_per_s" in extra:
        line["batched_over_plain"] = value / world / extra["plain_chunks_per_s"]

    nsc = extra.get("no_depth_shortcut")
    if nsc:
        nsc["frac_of_fp32_peak"] = nsc["tflops"] / fp32_peak
    if rank == 0 and not args.quick:
        # accuracy of the fast build against the f64 oracle, outside the timed region
        line["fast_vs_f64"] = leg_fast_vs_f64(params, descs, range(N_SEEDS))
    if rank == 0 and not args.no_cpu and not args.quick:
        cv, cn, cel = cpu_reference(descs, list(range(N_SEEDS)), 1, budget_s=12.0)
        line["cpu_baseline"] = {"value": cv, "unit": UNIT, "cores": 1, "kind": "port",
                                "sample": f"{cn} chunks ({cn // n} full 4096-chunk grids, seeds 0..) in {cel:.1f} s, "
                                          f"oracle f64 reference semantics with linear dedup search, 1 thread, "
                                          f"CPU: {cpu_model()}"}
    if rank == 0:
        print(json.dumps(line))
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
