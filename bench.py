"""Benchmark of the ZFP fixed-rate codec on one GB300 (or N replicas).

Workload: a 512^3 float64 field (1 GiB; sum of 16 random-phase sinusoids
with integer wavevectors, |k| in 1..32, amplitude 1/|k|^2), fixed rate 16
bits/value.  One step = compress the field, then decompress the stream, so
both kernels run once per step; inputs (1 GiB field, 256 MiB stream) are far
larger than the 129 MB L2, so no flush is needed between steps.

Reported (one JSON line on rank 0):
  value      uncompressed GB/s through compress + decompress (2 x 1 GiB per
             step / step time), device-resident buffers, CUDA-event timed;
  e2e        the same through the public C ABI with pinned host buffers
             (host->device and device->host copies inside the timed region);
  roofline   the dominant kernel's algorithmic bytes per launch / its
             average duration against the measured HBM copy bandwidth;
  cpu_baseline  the oracle's CPU restatement of zfp 0.5.0 on this host.
`--impl reference` times that CPU implementation alone on the same metric.

Multi-GPU: the path has no exchange step, so --gpus N runs N independent
replicas (one per rank, weak scaling); value = all ranks' bytes / the
slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

GiB = 1 << 30
SHAPE = (512, 512, 512)
RATE = 16.0
WORKLOAD = "3d_f64_512cube_sinusoids16_rate16"
FALLBACK_HBM_GBS = 6800.0


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="gzfp", choices=["gzfp", "reference"])
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-batched", action="store_true",
                   help="plain3d: leave out the batched workload's summary")
    p.add_argument("--no-serving", action="store_true",
                   help="plain3d: leave out the serving workload's summary")
    p.add_argument("--edge", type=int, default=512,
                   help="cube edge of the field (smaller cases for profiling)")
    p.add_argument("--rate", type=float, default=16.0)
    p.add_argument("--workload", default="plain3d",
                   choices=["plain3d", "batched", "serving", "accuracy", "edges"],
                   help="plain3d: the 1 GiB 3D float64 field (default); batched: 512 mixed "
                        "3D arrays in one graph-captured batch vs 512 plain launches; serving: "
                        "Poisson request arrivals through the request server; accuracy: the "
                        "plain3d field in zfp's fixed-accuracy mode; edges: the 1D and 2D "
                        "fields with partial edge blocks at rates 4, 12 and 24")
    p.add_argument("--tolerance", type=float, default=1e-6,
                   help="accuracy workload: absolute error tolerance")
    p.add_argument("--edges-fields", default="1d_f32_walk,2d_f32_16381x16383,2d_f64_8191x8190",
                   help="edges workload: the fields to run (for profiling one of them)")
    p.add_argument("--edges-scale", type=float, default=1.0,
                   help="edges workload: values per field x this (for small profiling cases)")
    p.add_argument("--arrays", type=int, default=512, help="batched workload: array count")
    p.add_argument("--requests", type=int, default=20000, help="serving workload: requests")
    p.add_argument("--inflight", type=int, default=3, help="serving workload: batches in flight")
    p.add_argument("--max-batch", type=int, default=256, help="serving workload: requests per batch")
    p.add_argument("--load", type=float, default=0.7,
                   help="serving workload: arrival rate as a fraction of plain-path capacity")
    p.add_argument("--batch-compress-config", default="",
                   help="batched workload: threads,ctas_per_sm,blocks_per_thread,claim_ahead of "
                        "the compress plan instead of the autotuner's choice")
    p.add_argument("--batch-decompress-config", default="",
                   help="batched workload: the same for the decompress plan")
    args = p.parse_args()
    global SHAPE, RATE, WORKLOAD
    SHAPE = (args.edge,) * 3
    RATE = args.rate
    WORKLOAD = f"3d_f64_{args.edge}cube_sinusoids16_rate{args.rate:g}"
    return args


def dist_env():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def max_over_ranks(value: float, world: int, device=None) -> float:
    """The largest of every rank's `value` (the slowest rank's time); the
    value itself when there is one rank."""
    if world <= 1:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            m = json.load(f)
        return float(m["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons while running."""

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            # the timed region starts only once nvidia-smi is answering
            t0 = time.time()
            while not self.rows and self.proc.poll() is None and time.time() - t0 < 5:
                time.sleep(0.01)
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def __exit__(self, *exc):
        if self.proc:
            n = len(self.rows)
            t0 = time.time()
            while len(self.rows) == n and self.proc.poll() is None and time.time() - t0 < 1:
                time.sleep(0.01)  # one sample taken after the region ends
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
                for i, nm in enumerate(names):
                    if r[5 + i].lower().startswith("active"):
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


# --------------------------------------------------------------- CPU side

def load_synth():
    """cuzfp_gb300/synth.py loaded by path.  Importing it through the package
    would run the package's __init__, which loads the CUDA codec; the CPU
    reference arm must not load it."""
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "gzfp_synth", os.path.join(ROOT, "cuzfp_gb300", "synth.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def plain_config(maxbits: int, sbytes: int, world: int) -> dict:
    """The `config` of the plain 3D workload, the same on both arms."""
    return {"workload": WORKLOAD, "shape": list(SHAPE), "rate": RATE, "maxbits": maxbits,
            "stream_bytes": sbytes,
            "l2": ("inputs larger than L2" if SHAPE[0] * SHAPE[1] * SHAPE[2] * 8 > 129e6
                   else "field smaller than L2 (a profiling size)") +
                  f" ({(SHAPE[0] * SHAPE[1] * SHAPE[2] * 8) >> 20} MiB field, "
                  f"{sbytes >> 20} MiB stream)",
            "parallelism": f"replicas x{world}"}

def cpu_measure(field_np, rate: float, threads: int, reps: int = 1):
    """Oracle (CPU restatement of zfp 0.5.0) compress+decompress throughput:
    (GB/s both ways, compress GB/s, decompress GB/s, the stream, the
    decompressed array)."""
    from oracle import oracle
    nbytes = field_np.nbytes
    best = None
    for _ in range(reps):
        t0 = time.perf_counter()
        s = oracle.compress(field_np, rate, threads)
        t1 = time.perf_counter()
        d = oracle.decompress(s, field_np.shape, field_np.dtype, rate, threads)
        t2 = time.perf_counter()
        gbs = 2 * nbytes / (t2 - t0) / 1e9
        if best is None or gbs > best[0]:
            best = (gbs, nbytes / (t1 - t0) / 1e9, nbytes / (t2 - t1) / 1e9)
    return best + (s, d)


def run_reference(args, rank, world):
    """--impl reference: zfp 0.5.0's CPU path (the oracle port, pinned bit for
    bit to the reference's own zfp build) on all host cores, one step = the
    whole field compressed and decompressed."""
    import numpy as np
    if rank != 0:
        return
    from oracle import oracle
    synth = load_synth()
    lib = oracle.port()
    threads = os.cpu_count() or 1
    field = synth.sinusoids(SHAPE, 16, 32, seed=0, dtype=np.float64)
    maxbits = int(lib.gzo_maxbits(oracle.DOUBLE, 3, RATE))
    sbytes = int(lib.gzo_stream_bytes(oracle.DOUBLE, SHAPE[2], SHAPE[1], SHAPE[0], RATE))
    for _ in range(max(args.warmup, 0)):
        cpu_measure(field, RATE, threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        st = oracle.compress(field, RATE, threads)
        oracle.decompress(st, field.shape, field.dtype, RATE, threads)
    dt = time.perf_counter() - t0
    value = 2 * field.nbytes * args.steps / dt / 1e9
    sample = f"the whole {field.nbytes >> 20} MiB field, compress+decompress, every step"
    out = {
        "impl": "reference", "metric": "zfp fixed-rate compress+decompress throughput",
        "value": round(value, 4), "unit": "GB/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(1e3 * dt / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": plain_config(maxbits, sbytes, args.gpus),
        "cpu_baseline": {"value": round(value, 4), "unit": "GB/s", "cores": threads,
                         "kind": "port", "sample": sample},
        "e2e": {"value": round(value, 4), "unit": "GB/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


# ------------------------------------------------------------ batched path

def batched_arrays(n_arrays: int, seed: int = 0):
    """Shapes, dtypes and rates of the mixed batch: 3D, per-axis size
    uniform in 17..257, float32 / float64 50/50, rate from {4, 8, 16, 32}."""
    import numpy as np
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(n_arrays):
        shape = tuple(int(v) for v in rng.integers(17, 258, 3))
        dt = "float32" if rng.random() < 0.5 else "float64"
        rate = float(rng.choice([4.0, 8.0, 16.0, 32.0]))
        specs.append((shape, dt, rate, 1000 + i))
    return specs


def batch_launches(gz, specs, cfg, decompress: bool) -> int:
    """Kernels one batch launches: the chunk table, and per kind present one
    persistent kernel (ctas_per_sm > 0) or one grid kernel per non-empty
    range of its items, those staged in shared memory (whole 64-bit words,
    at most 32 per block to decode, 16 to encode) and the others."""
    ranges = set()
    for _, dt, r, _ in specs:
        t = gz._type_of(dt)
        mb = gz._lib.gzfp_rate_to_maxbits(int(t), 3, r)
        staged = mb % 64 == 0 and mb // 64 <= (32 if decompress else 16)
        ranges.add((dt, staged if cfg.ctas_per_sm == 0 else None))
    return 1 + len(ranges)


def run_batched(args, rank, world, local, emit=True):
    """512 mixed arrays: one graph-captured batch per direction against 512
    plain launches per direction (same stream, device buffers).
    Prints the result line when `emit`, and returns it (on rank 0)."""
    import torch

    import cuzfp_gb300 as gz
    from cuzfp_gb300 import synth

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    specs = batched_arrays(args.arrays, seed=rank)
    fields = [synth.sinusoids_device(sh, 16, 32, seed=sd,
                                     dtype=torch.float32 if dt == "float32" else torch.float64,
                                     device=dev) for sh, dt, _, sd in specs]
    rates = [r for _, _, r, _ in specs]
    nbytes = sum(f.numel() * f.element_size() for f in fields)
    plain_s = gz.batch_stream_buffers(fields, rates)
    batch_s = gz.batch_stream_buffers(fields, rates)
    sbytes = sum(s.numel() * 8 for s in plain_s)
    plain_o = [torch.empty_like(f) for f in fields]
    batch_o = [torch.empty_like(f) for f in fields]
    torch.cuda.synchronize()

    # the plain leg: one gzfp_compress_bits / gzfp_decompress_bits call per
    # array through the C ABI, arguments built once
    lib, sh = gz._lib, stream.cuda_stream
    cargs, dargs = [], []
    for f, r, w, o in zip(fields, rates, plain_s, plain_o):
        t = int(gz._type_of(f.dtype))
        nx, ny, nz = gz._dims_of(f.shape)
        mb = lib.gzfp_rate_to_maxbits(t, len(f.shape), float(r))
        nb = w.numel() * 8
        cargs.append((t, nx, ny, nz, mb, f.data_ptr(), w.data_ptr(), nb, None, sh))
        dargs.append((t, nx, ny, nz, mb, w.data_ptr(), nb, o.data_ptr(), sh))

    def plain_step():
        for a in cargs:
            if lib.gzfp_compress_bits(*a) != 0:
                raise RuntimeError(lib.gzfp_last_error().decode())
        for a in dargs:
            if lib.gzfp_decompress_bits(*a) != 0:
                raise RuntimeError(lib.gzfp_last_error().decode())

    def launch_shape(spec, decompress, out):
        # a fixed shape (so that a profiler's run codes with the kernels the
        # timed run chose), or the autotuner's
        if spec:
            return gz.BatchConfig(*[int(v) for v in spec.split(",")]), None
        return gz.autotune_batch(fields if not decompress else out, batch_s, rates,
                                 decompress=decompress, repeats=2, cuda_stream=stream)

    t0 = time.perf_counter()
    cfg_c, ms_c = launch_shape(args.batch_compress_config, False, None)
    cfg_d, ms_d = launch_shape(args.batch_decompress_config, True, batch_o)
    tune_s = time.perf_counter() - t0
    cplan = gz.BatchPlan(fields, batch_s, rates, decompress=False, config=cfg_c)
    dplan = gz.BatchPlan(batch_o, batch_s, rates, decompress=True, config=cfg_d)

    def batch_step():
        cplan.launch(stream)
        dplan.launch(stream)

    def timed(fn, steps):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            for _ in range(max(args.warmup, 3)):
                fn()
            stream.synchronize()
            if world > 1:
                torch.distributed.barrier()
            a.record(stream)
            for _ in range(steps):
                fn()
            b.record(stream)
        b.synchronize()
        ms = a.elapsed_time(b) / steps
        ms = max_over_ranks(ms, world, dev)
        return ms

    with ClockSampler(local) as clk:
        batch_ms = timed(batch_step, args.steps)
    plain_ms = timed(plain_step, max(2, args.steps // 2))
    # the two paths must agree bit for bit on every array
    torch.cuda.synchronize()
    same_streams = all(torch.equal(a, b) for a, b in zip(plain_s, batch_s))
    same_fields = all(torch.equal(a.view(torch.int32 if a.dtype == torch.float32 else torch.int64),
                                  b.view(torch.int32 if b.dtype == torch.float32 else torch.int64))
                      for a, b in zip(plain_o, batch_o))
    cplan.close()
    dplan.close()
    if rank != 0:
        return
    peak, peak_kind = peaks()
    arrays = len(fields) * world
    res = {
        "metric": "batched zfp compress+decompress throughput (arrays/s)",
        "value": round(arrays / (batch_ms * 1e-3), 2), "unit": "arrays/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(batch_ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic",
        "config": {"workload": f"batched_{args.arrays}_3d_mixed", "arrays": args.arrays,
                   "uncompressed_bytes": nbytes, "stream_bytes": sbytes,
                   "l2": f"inputs larger than L2 ({nbytes / 1e9:.1f} GB of fields per step)",
                   "compress_config": cfg_c.as_dict(), "decompress_config": cfg_d.as_dict(),
                   "autotune_seconds": round(tune_s, 2)},
        "batched_gbs": round(2 * nbytes * world / (batch_ms * 1e-3) / 1e9, 2),
        "plain": {"ms_per_step": round(plain_ms, 4),
                  "arrays_per_s": round(arrays / (plain_ms * 1e-3), 2),
                  "gbs": round(2 * nbytes * world / (plain_ms * 1e-3) / 1e9, 2),
                  "launches_per_step": 2 * len(fields)},
        "speedup_vs_plain": round(plain_ms / batch_ms, 3),
        "bit_identical": bool(same_streams and same_fields),
        "roofline": {"bound": "hbm",
                     "achieved": round((2 * nbytes + 2 * sbytes) * world / (batch_ms * 1e-3) / 1e9, 2),
                     "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
                     "frac": round((2 * nbytes + 2 * sbytes) / (batch_ms * 1e-3) / 1e9 / peak, 4),
                     "traffic": None},
        # per step and direction: the chunk-table kernel, and per kind (all
        # arrays are 3D: one kind per scalar type) one persistent kernel or a
        # grid kernel per non-empty range (staged items, the others)
        "gpu_launches": (batch_launches(gz, specs, cfg_c, False) +
                         batch_launches(gz, specs, cfg_d, True)) * args.steps,
        "clocks": clk.summary(),
    }
    if emit:
        print(json.dumps(res), flush=True)
    return res


# ------------------------------------------------------------ serving loop

def serving_requests(n: int, seed: int = 0):
    """(op, edge, dtype, rate) of the request mix: cubic arrays with edge
    log-uniform in 32..384, float32 / float64 50/50, rate from {8, 16, 32},
    compress / decompress 50/50."""
    import numpy as np
    rng = np.random.default_rng(seed)
    edges = np.rint(np.exp(rng.uniform(np.log(32), np.log(384), n))).astype(int)
    f32 = rng.random(n) < 0.5
    rates = rng.choice([8.0, 16.0, 32.0], n)
    comp = rng.random(n) < 0.5
    return [(0 if comp[i] else 1, int(edges[i]), "float32" if f32[i] else "float64",
             float(rates[i])) for i in range(n)]


def run_serving(args, rank, world, local, emit=True):
    """Poisson arrivals at 70% of the plain path's capacity through the
    request server (device-queue mode, and the slot mode beside it), against
    serial plain calls on the same requests.  Prints the result line when
    `emit`, and returns it (on rank 0)."""
    import numpy as np
    import torch

    import cuzfp_gb300 as gz
    from cuzfp_gb300 import synth

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    n = args.requests
    specs = serving_requests(n, seed=rank)
    dts = {"float32": torch.float32, "float64": torch.float64}
    # resident inputs: one 384^3 field per dtype (a request of edge e reads
    # its first e^3 values as an e^3 cube) and, for decompression, the stream
    # of every (edge, dtype, rate) that a decompress request names
    pool = {k: synth.sinusoids_device((384, 384, 384), 16, 32, seed=rank, dtype=v, device=dev)
            for k, v in dts.items()}

    def field(e, dt):
        return pool[dt].view(-1)[: e ** 3].view(e, e, e)

    streams = {}
    for op, e, dt, r in specs:
        if op == 1 and (e, dt, r) not in streams:
            streams[(e, dt, r)] = gz.compress_tensor(field(e, dt), r)
    torch.cuda.synchronize()
    lib = gz._lib
    maxf = 384 ** 3 * 8
    scratch = torch.empty(maxf // 8, dtype=torch.int64, device=dev)
    nbytes = np.array([e ** 3 * (4 if dt == "float32" else 8) for _, e, dt, _ in specs], float)

    def plain_args(i):
        op, e, dt, r = specs[i]
        t = int(gz._type_of(dts[dt]))
        mb = lib.gzfp_rate_to_maxbits(t, 3, r)
        sb = gz.stream_size(gz._type_of(dts[dt]), e, e, e, mb)
        if op == 0:
            return lib.gzfp_compress_bits, (t, e, e, e, mb, field(e, dt).data_ptr(),
                                            scratch.data_ptr(), maxf, None, stream.cuda_stream)
        return lib.gzfp_decompress_bits, (t, e, e, e, mb, streams[(e, dt, r)].data_ptr(), sb,
                                          scratch.data_ptr(), stream.cuda_stream)

    # serial plain calls: each request's device time = its service time
    calls = [plain_args(i) for i in range(n)]
    for fn, a in calls[:50]:
        fn(*a)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2 * n)]
    torch.cuda.synchronize()
    for i, (fn, a) in enumerate(calls):
        ev[2 * i].record(stream)
        if fn(*a) != 0:
            raise RuntimeError(lib.gzfp_last_error().decode())
        ev[2 * i + 1].record(stream)
    torch.cuda.synchronize()
    service = np.array([ev[2 * i].elapsed_time(ev[2 * i + 1]) * 1e-3 for i in range(n)])
    plain_gbs = nbytes.sum() / service.sum() / 1e9
    capacity = n / service.sum()  # requests/s, device time only
    lam = args.load * capacity
    rng = np.random.default_rng(1000 + rank)
    arrivals = np.cumsum(rng.exponential(1.0 / lam, n))
    # the plain path under the same arrivals: one FIFO server
    fin, lat_plain = 0.0, np.empty(n)
    for i in range(n):
        fin = max(arrivals[i], fin) + service[i]
        lat_plain[i] = fin - arrivals[i]

    # sampled requests are checked bit for bit against their plain result
    sample = list(range(0, n, 97))
    check, expect = {}, {}
    for i in sample:
        op, e, dt, r = specs[i]
        if op == 0:
            ref = gz.compress_tensor(field(e, dt), r)
        else:
            ref = gz.decompress_tensor(streams[(e, dt, r)], (e, e, e), dts[dt], r)
        expect[i] = ref
        check[i] = torch.empty_like(ref)
    torch.cuda.synchronize()

    def requests(arr):
        out = []
        for i, (op, e, dt, r) in enumerate(specs):
            cp = check.get(i)
            if op == 0:
                out.append(gz.serve_request(0, field(e, dt), r, float(arr[i]), copy_to=cp))
            else:
                out.append(gz.serve_request(1, streams[(e, dt, r)], r, float(arr[i]),
                                            shape=(e, e, e), dtype=dts[dt], copy_to=cp))
        return out

    # the device-queue server (a persistent scheduler drains published
    # requests and launches each from the device) and, beside it, the slot
    # server (a batch per free slot)
    qcfg = gz.default_serve_config()
    qcfg.budget_bytes = 40 << 30
    qcfg.max_batch = args.max_batch
    qcfg.device_queue = 1
    cfg = gz.default_serve_config()
    cfg.device_queue = 0  # slots
    cfg.budget_bytes = 40 << 30
    cfg.max_inflight = args.inflight
    cfg.max_batch = args.max_batch
    with ClockSampler(local) as clk:
        res, stats = gz.serve(requests(arrivals), qcfg)
    lat = np.array([r.completed - arrivals[i] for i, r in enumerate(res)])
    ok = all(r.status == 0 for r in res)
    # saturation: every request queued at time zero
    sres, sstats = gz.serve(requests(np.zeros(n)), qcfg)
    torch.cuda.synchronize()
    bit_q = ok and all(_same_bits(expect[i], check[i]) for i in sample)
    res_s, stats_s = gz.serve(requests(arrivals), cfg)
    lat_s = np.array([r.completed - arrivals[i] for i, r in enumerate(res_s)])
    ssres, ssstats = gz.serve(requests(np.zeros(n)), cfg)
    torch.cuda.synchronize()
    ok = ok and all(r.status == 0 for r in res_s)

    bit_identical = bit_q and ok and all(_same_bits(expect[i], check[i]) for i in sample)

    # one 384^3 rate-16 request alone, per kind: the device queue's grid
    # (device-clock span of its CTAs, median of 3 runs) against the plain
    # call (CUDA events, mean of 5)
    lone = {}
    for dt in ("float32", "float64"):
        x = field(384, dt)
        w = gz.compress_tensor(x, 16.0)
        w_out, x_out = torch.empty_like(w), torch.empty_like(x)
        for op, name in ((0, "compress"), (1, "decompress")):
            def plain():
                if op == 0:
                    gz.compress_tensor(x, 16.0, out=w_out, cuda_stream=stream)
                else:
                    gz.decompress_tensor(w, x.shape, dts[dt], 16.0, out=x_out, cuda_stream=stream)
            plain()
            torch.cuda.synchronize()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            for _ in range(5):
                plain()
            b.record(stream)
            b.synchronize()
            spans = []
            for _ in range(3):
                rq = (gz.serve_request(0, x, 16.0, 0.0) if op == 0 else
                      gz.serve_request(1, w, 16.0, 0.0, shape=x.shape, dtype=dts[dt]))
                r1, _ = gz.serve([rq], qcfg)
                spans.append(r1[0].device_end - r1[0].device_start)
            lone[f"{name}_{dt}"] = {"plain_ms": round(a.elapsed_time(b) / 5, 4),
                                    "queue_ms": round(float(np.median(spans)) * 1e3, 4)}
    if rank != 0:
        return
    p50, p99 = np.percentile(lat, 50), np.percentile(lat, 99)
    res_line = {
        "metric": f"serving p99 latency at {round(100 * args.load)}% of plain-path capacity",
        "value": round(p99 * 1e3, 4), "unit": "ms", "n_gpus": world, "steps": 1,
        "warmup": 50, "ms_per_step": round(stats.wall * 1e3, 3), "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": {"workload": f"serving_{n}_requests_cubic_32to384_poisson{round(100 * args.load)}",
                   "requests": n, "budget_gb": 40, "arrival_rate_per_s": round(lam, 2),
                   "uncompressed_bytes": float(nbytes.sum()),
                   "l2": "inputs larger than L2 (a 384^3 field per dtype, ~2 GB of streams "
                         "per second of arrivals)",
                   "server": "device queue (a persistent scheduler kernel drains published requests and launches each as its own grid from the device)"},
        "latency_ms": {"p50": round(p50 * 1e3, 4), "p99": round(p99 * 1e3, 4),
                       "mean": round(float(lat.mean()) * 1e3, 4)},
        "plain_serial_latency_ms": {"p50": round(np.percentile(lat_plain, 50) * 1e3, 4),
                                    "p99": round(np.percentile(lat_plain, 99) * 1e3, 4)},
        "served_gbs": round(nbytes.sum() / stats.wall / 1e9, 2),
        "saturated_gbs": round(nbytes.sum() / sstats.wall / 1e9, 2),
        "plain_serial_gbs": round(plain_gbs, 2),
        "saturated_vs_plain": round(nbytes.sum() / sstats.wall / 1e9 / plain_gbs, 3),
        "stats": stats.as_dict(), "saturated_stats": sstats.as_dict(),
        "slots": {"max_batch": cfg.max_batch, "max_inflight": cfg.max_inflight,
                  "latency_ms": {"p50": round(np.percentile(lat_s, 50) * 1e3, 4),
                                 "p99": round(np.percentile(lat_s, 99) * 1e3, 4)},
                  "saturated_gbs": round(nbytes.sum() / ssstats.wall / 1e9, 2),
                  "stats": stats_s.as_dict()},
        "lone_384cube_rate16": lone,
        "bit_identical_sample": bool(bit_identical), "checked": len(sample),
        "gpu_launches": int(stats.kernels), "clocks": clk.summary(),
    }
    if not emit:
        return res_line
    print(json.dumps(res_line), flush=True)
    return res_line


def _same_bits(a, b):
    """Two tensors equal bit for bit."""
    import torch
    if a.dtype in (torch.float32, torch.float64):
        it = torch.int32 if a.dtype == torch.float32 else torch.int64
        return torch.equal(a.view(it), b.view(it))
    return torch.equal(a, b)


def run_edges(args, rank, world, local):
    """The 1D and 2D fields whose last blocks are partial: 1D float32 of
    2^28 - 3 values (random walk), 2D float32 16381 x 16383 and float64
    8191 x 8190 (8 sinusoids, |k| up to 64), each at 4, 12 and 24 bits per
    value, compress and decompress kernels timed with CUDA events."""
    import torch

    import cuzfp_gb300 as gz
    from cuzfp_gb300 import synth

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    peak, peak_kind = peaks()
    cases, tot_bytes, tot_ms = [], 0, 0.0
    sc = args.edges_scale
    side = lambda n: max(1, int(round(n * sc ** 0.5)))  # noqa: E731
    fields = [("1d_f32_walk", lambda: synth.random_walk_device(
                  max(1, int((1 << 28) * sc) - 3), seed=2 + rank, dtype=torch.float32,
                  device=dev)),
              ("2d_f32_16381x16383", lambda: synth.sinusoids_device(
                  (side(16383), side(16381)), 8, 64, seed=3 + rank, dtype=torch.float32,
                  device=dev)),
              ("2d_f64_8191x8190", lambda: synth.sinusoids_device(
                  (side(8190), side(8191)), 8, 64, seed=4 + rank, dtype=torch.float64,
                  device=dev))]
    keep = set(args.edges_fields.split(","))
    fields = [f for f in fields if f[0] in keep]
    with ClockSampler(local) as clk:
        for name, make in fields:
            x = make()
            nbytes = x.numel() * x.element_size()
            for rate in (4.0, 12.0, 24.0):
                words = gz.compress_tensor(x, rate)
                out = torch.empty_like(x)
                sbytes = words.numel() * 8
                for _ in range(max(args.warmup, 3)):
                    gz.compress_tensor(x, rate, out=words, cuda_stream=stream)
                    gz.decompress_tensor(words, x.shape, x.dtype, rate, out=out, cuda_stream=stream)
                ev = [torch.cuda.Event(enable_timing=True) for _ in range(3 * args.steps)]
                torch.cuda.synchronize()
                if world > 1:
                    torch.distributed.barrier()
                with torch.cuda.stream(stream):
                    for i in range(args.steps):
                        ev[3 * i].record(stream)
                        gz.compress_tensor(x, rate, out=words, cuda_stream=stream)
                        ev[3 * i + 1].record(stream)
                        gz.decompress_tensor(words, x.shape, x.dtype, rate, out=out,
                                             cuda_stream=stream)
                        ev[3 * i + 2].record(stream)
                stream.synchronize()
                enc = sum(ev[3 * i].elapsed_time(ev[3 * i + 1]) for i in range(args.steps)) / args.steps
                dec = sum(ev[3 * i + 1].elapsed_time(ev[3 * i + 2]) for i in range(args.steps)) / args.steps
                enc = max_over_ranks(enc, world, dev)
                dec = max_over_ranks(dec, world, dev)
                alg = nbytes + sbytes
                cases.append({"field": name, "rate": rate, "encode_ms": round(enc, 4),
                              "decode_ms": round(dec, 4),
                              "gbs": round(2 * nbytes / ((enc + dec) * 1e-3) / 1e9, 2),
                              "encode_frac": round(alg / (enc * 1e-3) / 1e9 / peak, 4),
                              "decode_frac": round(alg / (dec * 1e-3) / 1e9 / peak, 4)})
                tot_bytes += 2 * nbytes
                tot_ms += enc + dec
                del words, out
            del x
            torch.cuda.empty_cache()
    if rank != 0:
        return
    worst = max(cases, key=lambda c: c["encode_ms"] + c["decode_ms"])
    res = {
        "metric": "zfp fixed-rate compress+decompress throughput, 1D/2D fields with partial edge blocks",
        "value": round(tot_bytes * world / (tot_ms * 1e-3) / 1e9, 3), "unit": "GB/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(tot_ms, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": {"workload": "edges_1d_f32_2d_f32_2d_f64_rates_4_12_24",
                   "fields": [f[0] for f in fields], "scale": sc,
                   "l2": "inputs larger than L2 (0.5-1 GiB fields)" if sc >= 1 else
                         f"fields scaled by {sc}",
                   "parallelism": f"replicas x{world}"},
        "cases": cases,
        "roofline": {"bound": "hbm", "kernel": f"slowest case {worst['field']} rate {worst['rate']}",
                     "frac": min(worst["encode_frac"], worst["decode_frac"]), "peak": peak,
                     "peak_kind": peak_kind, "unit": "GB/s", "traffic": None},
        "gpu_launches": 2 * args.steps * len(cases),
        "clocks": clk.summary(),
    }
    print(json.dumps(res), flush=True)


def run_accuracy(args, rank, world, local):
    """The plain3d field in zfp's fixed-accuracy mode: variable-length blocks,
    compressed on the device with their start bits and decompressed from
    them (each call ends when its result is complete).  Also times the
    serial block walk that decoding needs without start bits, on a 64^3
    field."""
    import torch

    import cuzfp_gb300 as gz
    from cuzfp_gb300 import synth

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    field = synth.sinusoids_device(SHAPE, 16, 32, seed=rank, dtype=torch.float64, device=dev)
    nbytes = field.numel() * field.element_size()
    mode = gz.mode_accuracy(gz.zfp_type.double, args.tolerance)
    out = torch.empty_like(field)
    words, offs = gz.compress_mode(field, mode, with_offsets=True, cuda_stream=stream)
    sbytes = words.numel() * 8
    for _ in range(max(args.warmup, 3)):
        words, offs = gz.compress_mode(field, mode, with_offsets=True, cuda_stream=stream)
        gz.decompress_mode(words, SHAPE, torch.float64, mode, offsets=offs, out=out,
                           cuda_stream=stream)
    torch.cuda.synchronize()
    err = float((out - field).abs().max())
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3 * args.steps)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        for i in range(args.steps):
            ev[3 * i].record(stream)
            words, offs = gz.compress_mode(field, mode, with_offsets=True, cuda_stream=stream)
            ev[3 * i + 1].record(stream)
            gz.decompress_mode(words, SHAPE, torch.float64, mode, offsets=offs, out=out,
                               cuda_stream=stream)
            ev[3 * i + 2].record(stream)
        stream.synchronize()
    torch.cuda.synchronize()
    enc_ms = sum(ev[3 * i].elapsed_time(ev[3 * i + 1]) for i in range(args.steps)) / args.steps
    dec_ms = sum(ev[3 * i + 1].elapsed_time(ev[3 * i + 2]) for i in range(args.steps)) / args.steps
    ms_per_step = max_over_ranks(enc_ms + dec_ms, world, dev)
    # the serial walk, on a small field (15^3 = 3,375 blocks: too few for
    # the parallel index, which starts at 4,096), and the parallel index of
    # the whole stream, checked against the compressor's start bits
    small = synth.sinusoids_device((60, 60, 60), 16, 32, seed=rank, dtype=torch.float64,
                                   device=dev)
    sw = gz.compress_mode(small, mode, cuda_stream=stream)
    gz.index_blocks(sw, small.shape, torch.float64, mode, cuda_stream=stream)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    gz.index_blocks(sw, small.shape, torch.float64, mode, cuda_stream=stream)
    b.record(stream)
    b.synchronize()
    walk_us = a.elapsed_time(b) * 1e3 / (15 ** 3)
    idx = gz.index_blocks(words, SHAPE, torch.float64, mode, cuda_stream=stream)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    idx = gz.index_blocks(words, SHAPE, torch.float64, mode, cuda_stream=stream)
    torch.cuda.synchronize()
    index_ms = (time.perf_counter() - t0) * 1e3
    index_ok = bool(torch.equal(idx, offs))
    if rank != 0:
        return
    peak, peak_kind = peaks()
    alg = nbytes + sbytes
    res = {
        "metric": "zfp fixed-accuracy compress+decompress throughput",
        "value": round(2 * nbytes * world / (ms_per_step * 1e-3) / 1e9, 3), "unit": "GB/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(ms_per_step, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"3d_f64_{args.edge}cube_sinusoids16_accuracy{args.tolerance:g}",
                   "shape": list(SHAPE), "mode": list(mode.as_tuple()), "stream_bytes": sbytes,
                   "bits_per_value": round(8 * sbytes / field.numel(), 3),
                   "max_abs_error": err,
                   "l2": "inputs larger than L2 (1 GiB field)",
                   "parallelism": f"replicas x{world}"},
        "compress_gbs": round(nbytes / (enc_ms * 1e-3) / 1e9, 3),
        "decompress_gbs": round(nbytes / (dec_ms * 1e-3) / 1e9, 3),
        "calls": {"compress_ms": round(enc_ms, 4), "decompress_ms": round(dec_ms, 4),
                  "compress_alg_gbs": round(alg / (enc_ms * 1e-3) / 1e9, 2),
                  "decompress_alg_gbs": round(alg / (dec_ms * 1e-3) / 1e9, 2)},
        "roofline": {"bound": "hbm", "kernel": "compress+decompress calls",
                     "achieved": round(2 * alg / (ms_per_step * 1e-3) / 1e9, 2), "peak": peak,
                     "peak_kind": peak_kind, "unit": "GB/s",
                     "frac": round(2 * alg / (ms_per_step * 1e-3) / 1e9 / peak, 4),
                     "traffic": None},
        "block_walk_us_per_block": round(walk_us, 3),
        "parallel_index": {"ms": round(index_ms, 3), "blocks": int(offs.numel()),
                           "equal_to_compressor_offsets": index_ok,
                           "serial_walk_estimate_ms": round(walk_us * offs.numel() / 1e3, 1)},
        "gpu_launches": 6 * args.steps,
        "clocks": clk.summary(),
    }
    print(json.dumps(res), flush=True)


# --------------------------------------------------------------- GPU side

def main():
    args = parse()
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if args.impl == "gzfp" else "gloo"
        dist.init_process_group(backend)
    try:
        run(args, rank, world, local)
    finally:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


def run(args, rank, world, local):
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if args.workload == "batched":
        run_batched(args, rank, world, local)
        return
    if args.workload == "serving":
        run_serving(args, rank, world, local)
        return
    if args.workload == "accuracy":
        run_accuracy(args, rank, world, local)
        return
    if args.workload == "edges":
        run_edges(args, rank, world, local)
        return
    import numpy as np
    import torch

    import cuzfp_gb300 as gz
    from cuzfp_gb300 import synth

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    field = synth.sinusoids_device(SHAPE, 16, 32, seed=rank, dtype=torch.float64, device=dev)
    nbytes = field.numel() * field.element_size()
    zfp = gz.zfp_stream()
    gz.stream_set_rate(zfp, RATE, gz.zfp_type.double, 3)
    sbytes = gz.stream_size(gz.zfp_type.double, SHAPE[2], SHAPE[1], SHAPE[0], zfp.maxbits)
    words = torch.empty(sbytes // 8, dtype=torch.int64, device=dev)
    out = torch.empty_like(field)
    torch.cuda.synchronize()

    def step():
        gz.compress_tensor(field, RATE, out=words, cuda_stream=stream)
        gz.decompress_tensor(words, SHAPE, torch.float64, RATE, out=out, cuda_stream=stream)

    # warm-up, then per-kernel timing on the launching stream
    with torch.cuda.stream(stream):
        for _ in range(max(args.warmup, 3)):
            step()
    stream.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3 * args.steps)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        with torch.cuda.stream(stream):
            t_start = torch.cuda.Event(enable_timing=True)
            t_end = torch.cuda.Event(enable_timing=True)
            t_start.record(stream)
            for i in range(args.steps):
                ev[3 * i].record(stream)
                gz.compress_tensor(field, RATE, out=words, cuda_stream=stream)
                ev[3 * i + 1].record(stream)
                gz.decompress_tensor(words, SHAPE, torch.float64, RATE, out=out,
                                     cuda_stream=stream)
                ev[3 * i + 2].record(stream)
            t_end.record(stream)
        stream.synchronize()
    torch.cuda.synchronize()
    total_ms = t_start.elapsed_time(t_end)
    enc_ms = sum(ev[3 * i].elapsed_time(ev[3 * i + 1]) for i in range(args.steps)) / args.steps
    dec_ms = sum(ev[3 * i + 1].elapsed_time(ev[3 * i + 2]) for i in range(args.steps)) / args.steps
    total_ms = max_over_ranks(total_ms, world, dev)
    ms_per_step = total_ms / args.steps
    value = 2 * nbytes * world / (ms_per_step * 1e-3) / 1e9

    # rate-distortion of the decoded field against the original, for
    # information (the zfp tool's statistics, zfp-0.5.0/utils/zfp.c:29-57)
    err = (out - field).abs()
    erms = float(torch.sqrt((err * err).mean()))
    frange = float(field.max() - field.min())
    distortion = {"maxe": float(err.max()), "rmse": erms,
                  "nrmse": erms / frange if frange > 0 else 0.0,
                  "psnr": 20 * math.log10(frange / (2 * erms)) if erms > 0 and frange > 0
                  else float("inf")}
    del err
    dev_stream = words.cpu().numpy().view(np.uint64)
    dev_out = out.cpu().numpy()

    # e2e through the C ABI with pinned host buffers
    e2e = None
    if not args.no_e2e:
        h_in = field.cpu().pin_memory()
        h_stream = torch.empty(sbytes // 8, dtype=torch.int64).pin_memory()
        h_out = torch.empty(SHAPE, dtype=torch.float64).pin_memory()
        zf = gz.zfp_field_3d(h_in, gz.zfp_type.double, SHAPE[2], SHAPE[1], SHAPE[0])
        zo = gz.zfp_field_3d(h_out, gz.zfp_type.double, SHAPE[2], SHAPE[1], SHAPE[0])
        zs = gz.zfp_stream(stream=h_stream)
        gz.stream_set_rate(zs, RATE, gz.zfp_type.double, 3)

        def e2e_step():
            gz.compress(zs, zf, cuda_stream=stream)
            gz.decompress(zs, zo, cuda_stream=stream)

        for _ in range(max(args.warmup, 3)):
            e2e_step()
        torch.cuda.synchronize()
        e_steps = max(3, args.steps // 2)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(e_steps):
            e2e_step()
        b.record(stream)
        b.synchronize()
        e_ms = a.elapsed_time(b) / e_steps
        e_ms = max_over_ranks(e_ms, world, dev)
        e2e = {"value": round(2 * nbytes * world / (e_ms * 1e-3) / 1e9, 3), "unit": "GB/s",
               "ms_per_step": round(e_ms, 3),
               "h2d_bytes_per_step": nbytes + sbytes, "d2h_bytes_per_step": sbytes + nbytes}

    # the batched workload's summary (512 mixed arrays, graph-captured batch
    # launches against plain launches), so that one run records it
    batched = None
    if not args.no_batched:
        bargs = argparse.Namespace(**vars(args))
        bargs.steps, bargs.warmup = 5, 3
        b = run_batched(bargs, rank, world, local, emit=False)
        if b is not None:
            batched = {"workload": b["config"]["workload"], "ms_per_step": b["ms_per_step"],
                       "arrays_per_s": b["value"], "batched_gbs": b["batched_gbs"],
                       "plain_ms_per_step": b["plain"]["ms_per_step"],
                       "speedup_vs_plain": b["speedup_vs_plain"],
                       "bit_identical": b["bit_identical"], "steps": bargs.steps,
                       "compress_config": b["config"]["compress_config"],
                       "decompress_config": b["config"]["decompress_config"]}
        torch.cuda.empty_cache()
    # the serving workload's summary (Poisson arrivals at 70% of plain-path
    # capacity through the device-queue server)
    serving = None
    if not args.no_serving:
        s = run_serving(argparse.Namespace(**vars(args)), rank, world, local, emit=False)
        if s is not None:
            serving = {"workload": s["config"]["workload"], "server": s["config"]["server"],
                       "latency_ms": s["latency_ms"],
                       "plain_serial_latency_ms": s["plain_serial_latency_ms"],
                       "slots_latency_ms": s["slots"]["latency_ms"],
                       "served_gbs": s["served_gbs"], "saturated_vs_plain": s["saturated_vs_plain"],
                       "mean_inflight": round(s["stats"]["mean_inflight"], 3),
                       "lone_384cube_rate16": s["lone_384cube_rate16"],
                       "bit_identical_sample": s["bit_identical_sample"]}
        torch.cuda.empty_cache()

    if rank != 0:
        return
    peak, peak_kind = peaks()
    alg = nbytes + sbytes  # algorithmic bytes per launch (same for both kernels)
    enc_gbs = alg / (enc_ms * 1e-3) / 1e9
    dec_gbs = alg / (dec_ms * 1e-3) / 1e9
    dominant = ("encode", enc_ms, enc_gbs) if enc_ms >= dec_ms else ("decode", dec_ms, dec_gbs)
    traffic = None
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            traffic = json.load(f).get(WORKLOAD, {}).get(dominant[0])
    except Exception:
        traffic = None
    cpu = None
    parity = {"checked": False}
    # the CPU leg (baseline and whole-field parity) runs at N = 1 only: with
    # more ranks, rank 0 would hold the others' GPUs idle while it codes
    if not args.no_cpu and world == 1:
        from oracle import oracle
        oracle.port()
        host = field.cpu().numpy()
        threads = os.cpu_count() or 1
        gbs, c_gbs, d_gbs, ref_s, ref_d = cpu_measure(host, RATE, threads, reps=2)
        cpu = {"value": round(gbs, 4), "unit": "GB/s", "cores": threads, "kind": "port",
               "sample": f"the whole {nbytes >> 20} MiB field, compress+decompress, best of 2",
               "compress_gbs": round(c_gbs, 4), "decompress_gbs": round(d_gbs, 4)}
        # zfp 0.5.0 as shipped is serial: one thread on the first 64 z-planes
        part = host[: min(64, host.shape[0])]
        g1, c1, d1, _, _ = cpu_measure(part, RATE, 1)
        cpu["single_thread"] = {"value": round(g1, 4), "compress_gbs": round(c1, 4),
                                "decompress_gbs": round(d1, 4), "cores": 1,
                                "sample": f"the first {part.shape[0]} z-planes "
                                          f"({part.nbytes >> 20} MiB), compress+decompress"}
        # the CPU leg coded the very field the GPU coded: compare the whole
        # stream and the whole decoded array bit for bit, for the timed
        # device-buffer run and for the host-buffer (e2e) run
        parity = {"checked": True, "compared": "whole field",
                  "stream": bool(np.array_equal(dev_stream, ref_s)),
                  "output": bool(np.array_equal(dev_out.view(np.uint64), ref_d.view(np.uint64)))}
        if e2e is not None:
            parity["e2e_stream"] = bool(np.array_equal(h_stream.numpy().view(np.uint64), ref_s))
            parity["e2e_output"] = bool(np.array_equal(h_out.numpy().view(np.uint64),
                                                       ref_d.view(np.uint64)))
        del ref_s, ref_d, host
    res = {
        "metric": "zfp fixed-rate compress+decompress throughput",
        "value": round(value, 3), "unit": "GB/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_per_step, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": plain_config(zfp.maxbits, sbytes, world),
        "compress_gbs": round(nbytes / (enc_ms * 1e-3) / 1e9, 3),
        "decompress_gbs": round(nbytes / (dec_ms * 1e-3) / 1e9, 3),
        "kernels": {"encode": {"ms": round(enc_ms, 4), "alg_gbs": round(enc_gbs, 2),
                               "frac": round(enc_gbs / peak, 4)},
                    "decode": {"ms": round(dec_ms, 4), "alg_gbs": round(dec_gbs, 2),
                               "frac": round(dec_gbs / peak, 4)}},
        "roofline": {"bound": "hbm", "kernel": dominant[0], "achieved": round(dominant[2], 2),
                     "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
                     "frac": round(dominant[2] / peak, 4), "traffic": traffic},
        "gpu_launches": 2 * args.steps,
        "clocks": clk.summary(),
        "e2e": e2e,
        "cpu_baseline": cpu,
        "parity": parity,
        "rate_distortion": distortion,
        "batched": batched,
        "serving": serving,
    }
    print(json.dumps(res), flush=True)


if __name__ == "__main__":
    main()
