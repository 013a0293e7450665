"""Benchmark of the batched 2x2 Hermitian EVD (VecJac's dbjac2_/zbjac2_/sbjac2_/cbjac2_).

Workload ("bjac2", default): the batched-EVD configuration -- 2^28 real symmetric FP64
triples, 2^27 complex Hermitian FP64, 2^28 real FP32 and 2^27 complex FP32, SoA arrays,
entries +-2^e*u with e uniform in [-300, 300] (FP64) / [-40, 40] (FP32), u uniform in
[1, 2), generated on the GPU from a seed (synthetic data; the reference publishes no
data set). One step = one pass of all four batches (n < 0: cosines and sines).

Metric: GB/s of algorithmic HBM traffic (56.5 / 72.5 / 28.25 / 36.25 bytes per element for
d / z / s / c: inputs, outputs and the permutation bitmask), whole job. The inputs
(37 GB) exceed the 129 MB L2 many times over, so no L2 flush is needed between steps.
The same line carries the SVD half of the metric in its "svd" object (--no-svd leaves it
out): dvjsvd 1024x1024 FP64 and zvjsvd 4096x2048 FP64 complex, mixed-precision and plain,
in matrices/s with sweeps, the mixed/plain ratio and the errors against the exact singular
values and against the FP64 oracle (the plain path, the reference's algorithm bit for bit);
the plain 4096x2048 run takes about a minute (--svd-plain-steps 0 skips it).

Other workloads (--workload): "svd1024" (dvjsvd_ on a 1024x1024 FP64 matrix, matrices/s),
"zsvd" (zvjsvd_ on 4096x2048 FP64 complex), "zsvd_mixed"/"dsvd_mixed" (the same matrix
through the mixed-precision path, with the plain FP64 arm timed beside it), "batch_d"/
"batch_s" (20,000 uneven real matrices in one persistent launch), "diff" (4096 FP32
matrices 128x64: batched SVD forward and the hand-written adjoint, matrices/s).

Timing follows the harness contract: W untimed warm-up steps, then K steps between CUDA
events on the launching stream with a barrier and a device synchronize on both sides,
max over ranks; the e2e figure goes through the C ABI with host buffers (copies in the
timed region). With --gpus N > 1 (torchrun, one process per GPU) every rank runs an
independent replica ("replicas only": the batch shards without any exchange).
"""
import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

BPE = {"d": 56.5, "z": 72.5, "s": 28.25, "c": 36.25}
LG = {"d": 28, "z": 27, "s": 28, "c": 27}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    def __init__(self, dev=0):
        self.dev = dev
        self.proc = None
        self.rows = []

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(2)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[0]))
                mx.append(float(r[1]))
                for k, v in zip(names, r[3:7]):
                    if v.lower().startswith("active"):
                        reasons.add(k)
            except (ValueError, IndexError):
                pass
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_init(gpus):
    import torch
    if gpus > 1 or "RANK" in os.environ:
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        dist.init_process_group(backend)
        rank = dist.get_rank()
        world = dist.get_world_size()
        if torch.cuda.is_available():
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", rank)))
        return dist, rank, world
    return None, 0, 1


def barrier(dist):
    if dist is not None:
        dist.barrier()


def allmax(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------- GPU inputs
def gen_pairs_gpu(kind, n, seed):
    """SoA inputs on the GPU with the distribution of vecjac_gb300.workloads.pairs2x2"""
    import torch
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    dt = torch.float64 if kind in "dz" else torch.float32
    lo, hi = (-300, 300) if kind in "dz" else (-40, 40)
    out = []
    for _ in range(4 if kind in "zc" else 3):
        e = torch.randint(lo, hi + 1, (n,), generator=g, device="cuda", dtype=torch.int32)
        u = torch.rand(n, generator=g, device="cuda", dtype=dt) + 1.0
        s = torch.randint(0, 2, (n,), generator=g, device="cuda", dtype=torch.int32).to(dt) * 2 - 1
        out.append(torch.ldexp(s * u, e.to(dt)).to(dt))
        del e, u, s
    return out


class Batch:
    def __init__(self, kind, n, seed):
        import torch
        self.kind, self.n = kind, n
        self.ins = gen_pairs_gpu(kind, n, seed)
        dt = self.ins[0].dtype
        self.outs = [torch.empty(n, dtype=dt, device="cuda") for _ in range(5 if kind in "zc" else 4)]
        self.p = torch.empty(n // (8 if kind in "dz" else 16), dtype=torch.int32, device="cuda")

    def launch(self, vj, stream):
        k, i, o = self.kind, self.ins, self.outs
        if k in "zc":
            r = vj.bjac2_dev(k, -self.n, i[0], i[1], i[2], i[3], o[0], o[1], o[2], o[3], o[4], self.p, stream=stream)
        else:
            r = vj.bjac2_dev(k, -self.n, i[0], i[1], i[2], None, o[0], o[1], None, o[2], o[3], self.p, stream=stream)
        if r != 1:
            raise RuntimeError("bjac2 %s failed: %d" % (k, r))

    def bytes(self):
        return BPE[self.kind] * self.n


# thread instructions per element of k_bjac2 (ncu smsp__inst_executed.sum x 32 / elements,
# issue slots: 2^24 real and 2^23 complex launches; the profile summary k_bjac2_fp64_pipe_2e24)
BJAC2_INST_PER_ELEM = {"d": 1278.0, "z": 1979.0}
# thread instructions per element that execute on the FP64 pipe (ncu
# smsp__inst_executed_pipe_fp64.sum x 32 / elements; profile summary k_bjac2_fp64_pipe_2e24)
BJAC2_FP64_PIPE_PER_ELEM = {"d": 25.0, "z": 50.0}
# DRAM bytes (read + write) of one 2^24-element real FP64 launch, from the same capture
BJAC2_D_DRAM_2E24 = 402.788096e6 + 495.165696e6
# the reference's own AVX-512 dbjac2_/zbjac2_ (src/dbjac2.c, src/zbjac2.c, compiled from its
# sources) on an x86-64 host with AVX-512, 8 threads, 2^24 elements of the same distribution,
# best of 5; it cannot be built on this Arm host (src/vec.h:11), so the figure is not measured
# in this run
X86_REFERENCE_BJAC2 = {"dbjac2_": {"gbs": 50.6, "threads": 8}, "zbjac2_": {"gbs": 50.5, "threads": 8},
                       "host": "x86-64 Sapphire Rapids (AVX-512), gcc 13.3 -O3 -march=native -fopenmp"}


def device_info():
    """SM count (from the device) and the measured FMA rates of its FP64 and FP32 pipes
    (vj_measure_fma_rate: a kernel of independent FMA chains on every SM)."""
    import ctypes as C
    import torch
    import vecjac_gb300 as vj
    props = torch.cuda.get_device_properties(torch.cuda.current_device())
    out = {"sms": int(props.multi_processor_count), "name": props.name}
    L = vj.lib()
    for key, f64 in (("fp64_fma_per_s", 1), ("fp32_fma_per_s", 0)):
        v = C.c_double(0.0)
        r = L.vj_measure_fma_rate(C.c_int(f64), C.byref(v), None)
        out[key] = float(v.value) if r == 0 else None
    return out


def bench_fma_probe(args, vj):
    """The FMA pipes in several shapes (vj_measure_fma_shape): throughput per active lane
    with 32, 16 and 8 active lanes per warp, and the latency of one dependent chain. On
    GB300 the FP64 pipe completes about one warp instruction per 77 cycles per
    sub-partition whatever the number of active lanes, and a dependent DFMA takes about as
    long: one warp of one serial chain per sub-partition keeps it busy, and lanes left
    idle are lost."""
    import ctypes as C
    import torch
    props = torch.cuda.get_device_properties(torch.cuda.current_device())
    sms = int(props.multi_processor_count)
    L = vj.lib()
    rows = []
    for f64 in (1, 0):
        for wps, lanes, ch in ((4, 32, 8), (4, 16, 8), (4, 8, 8), (8, 32, 8), (8, 16, 8), (16, 16, 8),
                               (64, 32, 8), (4, 32, 1), (8, 32, 1), (16, 32, 1)):
            v = C.c_double(0.0)
            r = L.vj_measure_fma_shape(C.c_int(f64), C.c_int(wps), C.c_int(lanes), C.c_int(ch), C.byref(v), None)
            if r != 0:
                continue
            per_sm = v.value / sms
            rows.append({"pipe": "fp64" if f64 else "fp32", "warps_per_sm": wps, "lanes": lanes, "chains": ch,
                         "active_lane_fma_per_s": v.value, "per_sm_per_ns": round(per_sm * 1e-9, 3),
                         "ns_per_dependent_fma": (round(1e9 * wps * lanes * sms / v.value, 3) if ch == 1
                                                  else None)})
    return {"metric": "FMA pipe probe (active-lane FMAs per second)", "value": rows[0]["active_lane_fma_per_s"],
            "unit": "FMA/s", "n_gpus": 1, "steps": 3, "warmup": 1, "higher_is_better": True,
            "data": "synthetic", "dtype": "f64+f32", "config": {"workload": "FMA chains on every SM, %d SMs" % sms},
            "shapes": rows}


def issue_bound(kind, sm_mhz, sms):
    """Element-rate bound of the FP64 2x2 from instruction issue: each SM issues at most one
    warp instruction per clock on each of its 4 sub-partitions (128 thread instructions per
    clock), and the kernel executes BJAC2_INST_PER_ELEM[kind] thread instructions per
    element (correctly rounded divisions as integer long division, square roots and FMAs
    on the FP64 pipe, exponent handling on the integer pipes)."""
    return sms * 128.0 * sm_mhz * 1e6 / BJAC2_INST_PER_ELEM[kind]


def bench_bjac2(args, vj, dist, rank, world):
    import torch
    kinds = "dzsc"
    shift = args.scale
    batches = [Batch(k, 1 << (LG[k] - shift), seed=100 + i + 17 * rank) for i, k in enumerate(kinds)]
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    sh = stream.cuda_stream
    for _ in range(args.warmup):
        for b in batches:
            b.launch(vj, sh)
    torch.cuda.synchronize()
    # per-kernel durations (events on the launching stream), one extra step
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in batches]
    for b, (e0, e1) in zip(batches, ev):
        e0.record(stream)
        b.launch(vj, sh)
        e1.record(stream)
    torch.cuda.synchronize()
    per_ms = {b.kind: e0.elapsed_time(e1) for b, (e0, e1) in zip(batches, ev)}
    barrier(dist)
    torch.cuda.synchronize()
    with Clocks(torch.cuda.current_device()) as clk:
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for _ in range(args.steps):
            for b in batches:
                b.launch(vj, sh)
        t1.record(stream)
        torch.cuda.synchronize()
    barrier(dist)
    ms = allmax(dist, t0.elapsed_time(t1)) / args.steps
    total_bytes = sum(b.bytes() for b in batches)
    value = world * total_bytes / (ms * 1e-3) / 1e9
    clocks = clk.summary()
    pk, pk_src = peaks()
    dev = device_info()
    # dominant kernel: the FP64 real batch
    dom = batches[0]
    dom_gbs = dom.bytes() / (per_ms["d"] * 1e-3) / 1e9
    sm_mhz = clocks["sm_mhz"] or pk.get("sm_max_mhz", 2070.0)
    fb = issue_bound("d", sm_mhz, dev["sms"])
    per_kernel = {k: {"ms": round(per_ms[k], 4), "elements": b.n,
                      "gbs": round(b.bytes() / (per_ms[k] * 1e-3) / 1e9, 1),
                      "hbm_frac": round(b.bytes() / (per_ms[k] * 1e-3) / 1e9 / pk["hbm_gbs"], 4)}
                  for k, b in zip(kinds, batches)}
    # the FP64 kinds are bound by the FP64 pipe: FP64-pipe instructions per element (ncu) x
    # elements/s against the measured DFMA rate of this GPU
    for k in "dz":
        if BJAC2_FP64_PIPE_PER_ELEM[k] and dev["fp64_fma_per_s"]:
            eps_ = per_kernel[k]["elements"] / (per_kernel[k]["ms"] * 1e-3)
            per_kernel[k]["fp64_pipe_frac"] = round(eps_ * BJAC2_FP64_PIPE_PER_ELEM[k] / dev["fp64_fma_per_s"], 4)
    if BJAC2_FP64_PIPE_PER_ELEM["d"] and dev["fp64_fma_per_s"]:
        ach = dom.n / (per_ms["d"] * 1e-3) * BJAC2_FP64_PIPE_PER_ELEM["d"]
        roof = {"bound": "fp64_pipe", "kernel": "k_bjac2<double,real,sine>", "achieved": round(ach / 1e12, 5),
                "peak": round(dev["fp64_fma_per_s"] / 1e12, 5), "unit": "Tinst/s",
                "frac": round(ach / dev["fp64_fma_per_s"], 4),
                "peak_source": "measured live: vj_measure_fma_rate (DFMA chains on all %d SMs)" % dev["sms"],
                "achieved_source": "%.1f FP64-pipe thread instructions per element (ncu) x elements/s"
                                   % BJAC2_FP64_PIPE_PER_ELEM["d"]}
    else:
        roof = {"bound": "fp64_pipe", "kernel": "k_bjac2<double,real,sine>", "achieved": None, "peak": None,
                "unit": "Tinst/s", "frac": None}
    roof["hbm"] = {"achieved": round(dom_gbs, 1), "peak": pk["hbm_gbs"], "unit": "GB/s",
                   "frac": round(dom_gbs / pk["hbm_gbs"], 4), "peak_source": pk_src,
                   "traffic": round(BJAC2_D_DRAM_2E24 * dom.n / 2 ** 24),
                   "traffic_source": "ncu dram__bytes_read+write of a 2^24-element launch, scaled to this launch"}
    roof["issue"] = {"elements_per_s": round(dom.n / (per_ms["d"] * 1e-3), 1),
                     "bound_elements_per_s": round(fb, 1),
                     "frac": round(dom.n / (per_ms["d"] * 1e-3) / fb, 4),
                     "note": "%d thread instructions per element (ncu), 128 per clock per SM, %d SMs"
                             % (BJAC2_INST_PER_ELEM["d"], dev["sms"])}
    out = {
        "metric": "batched 2x2 Hermitian EVD throughput (GB/s of HBM traffic)",
        "value": round(value, 2), "unit": "GB/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(ms, 4), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64+f32", "data": "synthetic (seeded, GPU-generated; +-2^e*u distribution)",
        "config": {"workload": "bjac2: dbjac2_ 2^%d + zbjac2_ 2^%d + sbjac2_ 2^%d + cbjac2_ 2^%d elements, n<0 (sines)"
                   % tuple(LG[k] - shift for k in kinds),
                   "bytes_per_step": total_bytes, "l2": "inputs larger than L2 (no flush)",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "per_kernel": per_kernel,
        "roofline": roof,
        "device": dev,
        "clocks": clocks,
        "gpu_launches": args.steps * len(batches),
    }
    for b in batches:
        del b.ins, b.outs, b.p
    torch.cuda.empty_cache()
    if args.e2e:
        out["e2e"] = e2e_bjac2(args, vj, dist, world)
    if rank == 0 and args.cpu_baseline:
        out["cpu_baseline"] = cpu_baseline_bjac2(args.cpu_elems)
        out["cpu_baseline"]["x86_reference"] = X86_REFERENCE_BJAC2
    if args.svd:
        out["svd"] = bench_svd_suite(args, vj, dist, rank, world)
    return out


def e2e_bjac2(args, vj, dist, world):
    """The same workload through the reference-facing C ABI (dbjac2_ ... with host
    buffers; the library stages chunks through the GPU), copies inside the timed region."""
    import torch
    shift = args.scale + args.e2e_shift
    kinds = "dzsc"
    # host buffers of the full workload need ~2x its 37 GB of RAM (inputs, outputs, staging
    # of the generator); shrink the e2e batches when the host has less
    try:
        with open("/proc/meminfo") as f:
            avail = {l.split(":")[0]: int(l.split()[1]) for l in f}["MemAvailable"] * 1024
    except (OSError, KeyError, ValueError):
        avail = 1 << 40
    need = sum(BPE[k] * (1 << (LG[k] - shift)) for k in kinds) * 1.6
    while need > 0.6 * avail and shift < 8:
        shift += 1
        need /= 2
    # pinned (page-locked) host buffers, as an application feeding a GPU library keeps them;
    # pageable ones when the host refuses to pin that much
    pinned = True

    def host_like(t):
        nonlocal pinned
        if pinned:
            try:
                h = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
                return h.copy_(t).numpy() if t.is_cuda else h.numpy()
            except RuntimeError:
                pinned = False
        return t.cpu().numpy() if t.is_cuda else np.empty(tuple(t.shape), t.numpy().dtype)

    bufs = {}
    h2d = d2h = 0
    for i, k in enumerate(kinds):
        n = 1 << (LG[k] - shift)
        ins = [host_like(t) for t in gen_pairs_gpu(k, n, 300 + i)]
        tdt = torch.float64 if k in "dz" else torch.float32
        outs = [host_like(torch.empty(n, dtype=tdt)) for _ in range(5 if k in "zc" else 4)]
        p = host_like(torch.empty(n // (8 if k in "dz" else 16), dtype=torch.int32)).view(np.uint32)
        bufs[k] = (n, ins, outs, p)
        h2d += sum(a.nbytes for a in ins)
        d2h += sum(a.nbytes for a in outs) + p.nbytes
    total = sum(BPE[k] * bufs[k][0] for k in kinds)

    def step():
        for k in kinds:
            n, ins, outs, p = bufs[k]
            a21i = ins[3] if k in "zc" else None
            if k in "zc":
                r = vj.bjac2(k, -n, ins[0], ins[1], ins[2], a21i, c=outs[0], at=outs[1], sat=outs[2], l1=outs[3],
                             l2=outs[4], p=p)
            else:
                r = vj.bjac2(k, -n, ins[0], ins[1], ins[2], c=outs[0], at=outs[1], l1=outs[2], l2=outs[3], p=p)
            if r[0] != 1:
                raise RuntimeError("host bjac2 failed")

    for _ in range(max(1, min(args.warmup, 2))):
        step()
    steps = max(1, min(args.steps, 3))
    barrier(dist)
    torch.cuda.synchronize()
    t = time.perf_counter()
    for _ in range(steps):
        step()
    torch.cuda.synchronize()
    el = allmax(dist, time.perf_counter() - t) / steps
    return {"value": round(world * total / el / 1e9, 2), "unit": "GB/s", "h2d_bytes_per_step": int(h2d),
            "d2h_bytes_per_step": int(d2h), "steps": steps,
            "elements": {k: bufs[k][0] for k in kinds},
            "path": "C ABI dbjac2_/zbjac2_/sbjac2_/cbjac2_ on %s host buffers" % ("pinned" if pinned else "pageable")}


def cpu_baseline_bjac2(elems_lg, threads=None, warmup=1, steps=None, target_s=10.0):
    """The oracle port (oracle/vjo.c, the reference's algorithm in portable C) on the host
    cores, all threads, on a bounded sample of 2^elems_lg elements per precision: `warmup`
    untimed passes, then `steps` timed passes (None: as many as fill about target_s
    seconds, at most 64). One pass = d, z, s and c batches of the sample, n < 0."""
    from concurrent.futures import ThreadPoolExecutor

    from oracle import oracle as O
    from vecjac_gb300 import workloads as W
    O.build()
    R = O.Restatement()
    threads = threads or os.cpu_count()
    n = 1 << elems_lg
    data = {k: W.pairs2x2(k, n, 7) for k in "dzsc"}
    outs = {k: [np.empty(n, data[k][0].dtype) for _ in range(5)] for k in "dzsc"}
    perm = {k: np.empty(n // 8, np.uint32) for k in "dzsc"}
    chunk = n // threads
    chunk -= chunk % 16

    def run_kind(k, ex):
        ins, out, p = data[k], outs[k], perm[k]
        f = R.fn(k + "bjac2_")
        f.restype = C.c_longlong
        lanes = 8 if k in "dz" else 16

        def part(off):
            cnt = min(chunk, n - off)
            nn = C.c_longlong(-cnt)
            ptr = lambda a: C.c_void_p(a.ctypes.data + off * a.itemsize)
            if k in "zc":
                f(C.byref(nn), ptr(ins[0]), ptr(ins[1]), ptr(ins[2]), ptr(ins[3]), ptr(out[0]), ptr(out[1]),
                  ptr(out[2]), ptr(out[3]), ptr(out[4]), C.c_void_p(p.ctypes.data + (off // lanes) * 4))
            else:
                f(C.byref(nn), ptr(ins[0]), ptr(ins[1]), ptr(ins[2]), ptr(out[0]), ptr(out[1]), ptr(out[2]),
                  ptr(out[3]), C.c_void_p(p.ctypes.data + (off // lanes) * 4))

        list(ex.map(part, range(0, n, chunk)))

    with ThreadPoolExecutor(threads) as ex:
        def one_pass():
            t0 = time.perf_counter()
            for k in "dzsc":
                run_kind(k, ex)
            return time.perf_counter() - t0

        t1 = 0.0
        for _ in range(max(1, warmup)):
            t1 = one_pass()
        if steps is None:
            steps = int(min(64, max(1, round(target_s / max(t1, 1e-3)))))
        el = sum(one_pass() for _ in range(steps))
    total = sum(BPE[k] * n for k in "dzsc")
    return {"value": round(total * steps / el / 1e9, 3), "unit": "GB/s", "cores": threads, "kind": "port",
            "sample": "2^%d elements each of d/z/s/c (n<0) per pass, %d timed passes, oracle/vjo.c on %d host "
                      "threads" % (elems_lg, steps, threads),
            "seconds": round(el, 2), "steps": steps, "ms_per_step": round(el / steps * 1e3, 3)}


def reference_arm(args, dist, rank):
    """The reference's CPU implementation of the path on this host's cores. VecJac's own
    AVX-512 code cannot be compiled on this (Arm) host, so its portable restatement in C
    (oracle/vjo.c) is timed: W untimed and K timed steps, each step one pass over a
    bounded sample of the same workload (2^cpu_elems elements per precision)."""
    if rank != 0:
        return None
    base = cpu_baseline_bjac2(args.cpu_elems, warmup=args.warmup, steps=max(1, args.steps))
    v = base["value"]
    return {"metric": "batched 2x2 Hermitian EVD throughput (GB/s of HBM traffic)", "value": v, "unit": "GB/s",
            "n_gpus": 1, "steps": base["steps"], "warmup": args.warmup, "ms_per_step": base["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64+f32",
            "data": "synthetic (seeded)",
            "config": {"workload": "bjac2: d/z/s/c 2x2 EVD, bounded CPU sample 2^%d each" % args.cpu_elems},
            "impl": "reference",
            "cpu_baseline": {"value": v, "unit": "GB/s", "cores": base["cores"], "kind": "port",
                             "sample": base["sample"]},
            "e2e": {"value": v, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


# ---------------------------------------------------------------- SVD workloads
def svd_roofline(flops_per_s, fp64, kernel, dev=None):
    """Roofline object for the Jacobi SVD workloads: algorithmic FLOP rate (12m + 6n real,
    36m + 20n complex per pair and sweep) against the FMA pipe's peak, measured live on this
    GPU (vj_measure_fma_rate; 2 flops per FMA)."""
    dev = dev or device_info()
    fma = dev["fp64_fma_per_s" if fp64 else "fp32_fma_per_s"]
    peak = 2.0 * fma / 1e12 if fma else None
    ach = flops_per_s / 1e12
    return {"bound": "fp64_pipe" if fp64 else "fp32_pipe", "kernel": kernel, "achieved": round(ach, 5),
            "peak": round(peak, 3) if peak else None, "unit": "TFLOP/s",
            "frac": round(ach / peak, 4) if peak else None, "traffic": None,
            "peak_source": "measured live: vj_measure_fma_rate (FMA chains on all %d SMs)" % dev["sms"],
            "note": "algorithmic FLOPs; the reference's scaled compensated dot product executes ~9 operations "
                    "per element and accumulator chain, so the pipe is busier than this fraction"}


def svd_case(args, vj, dist, kind, m, n, lo, mixed_steps, plain_steps, warmup, seed=2024):
    """One SVD configuration timed through the device entry points (CUDA events on the
    launching stream): the mixed-precision path (FP32 presweeps, FP64 finish) and the plain
    FP64 path (the reference's algorithm, bit-identical to the compiled reference and the
    oracle). Errors: singular values against the exact ones of the construction, mixed
    against plain (the FP64 oracle's result), and ||U^H U - I||_F, ||V^H V - I||_F in units
    of n eps."""
    import torch
    from vecjac_gb300 import workloads as W
    cx = kind == "z"
    A, s = W.svd_matrix(m, n, seed=seed, lo=lo, complex_=cx)
    js, stp = vj.pjs(args.pivot, n)
    Gt = torch.tensor(np.ascontiguousarray(A.real.T), dtype=torch.float64, device="cuda")
    Git = torch.tensor(np.ascontiguousarray(A.imag.T), dtype=torch.float64, device="cuda") if cx else None
    G, Gi = torch.empty_like(Gt), (torch.empty_like(Gt) if cx else None)
    V = torch.empty((n, n), dtype=torch.float64, device="cuda")
    Vi = torch.empty_like(V) if cx else None
    eS = torch.empty(n, dtype=torch.float64, device="cuda")
    fS = torch.empty_like(eS)
    djs = torch.tensor(js.astype(np.int32), device="cuda")
    stream = torch.cuda.current_stream()
    eps = float(np.finfo(np.float64).eps)

    def reset():
        G.copy_(Gt)
        if cx:
            Gi.copy_(Git)

    def mixed():
        reset()
        return vj.vjsvd_mixed_dev(kind, m, n, G, m, V, n, eS, fS, djs, stp, Gi=Gi, ldGi=m, Vi=Vi, ldVi=n,
                                  stream=stream.cuda_stream)

    def plain():
        reset()
        return vj.vjsvd_dev(kind, m, n, G, m, V, n, eS, fS, djs, stp, Gi=Gi, ldGi=m, Vi=Vi, ldVi=n,
                            stream=stream.cuda_stream)

    def timed(fn, k):
        torch.cuda.synchronize()
        barrier(dist)
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for _ in range(k):
            r = fn()
        t1.record(stream)
        torch.cuda.synchronize()
        return allmax(dist, t0.elapsed_time(t1)) / k, r

    def results():
        sig = (fS * torch.exp2(eS)).cpu().numpy()
        U = torch.complex(G, Gi) if cx else G
        Vm = torch.complex(V, Vi) if cx else V
        # stored column-major: row j of the tensor is column j of the matrix
        ou = float(torch.linalg.norm(U.conj() @ U.T - torch.eye(n, dtype=U.dtype, device="cuda")))
        ov = float(torch.linalg.norm(Vm.conj() @ Vm.T - torch.eye(n, dtype=Vm.dtype, device="cuda")))
        srt = np.sort(sig)[::-1]
        # the stated orthogonality bound is ||U^H U - I||_F, ||V^H V - I||_F <= 16 n eps; the
        # reference's own algorithm (the plain path, bit for bit) can exceed it for V, and
        # the flag says so per configuration rather than loosening the bound
        return sig, {"max_rel_sigma_err_vs_exact": float(np.max(np.abs(srt - s) / s)),
                     "max_sigma_err_over_sigma_max": float(np.max(np.abs(srt - s)) / s[0]),
                     "orth_U_fro_over_n_eps": round(ou / (n * eps), 3),
                     "orth_V_fro_over_n_eps": round(ov / (n * eps), 3),
                     "orth_within_16_n_eps": bool(max(ou, ov) <= 16 * n * eps)}

    per_pair = (36 * m + 20 * n) if cx else (12 * m + 6 * n)
    out = {"config": "%svjsvd %dx%d, sigma log-uniform in [1e%d, 1], pivot strategy id %d" % (kind, m, n, lo, args.pivot),
           "bound_64_n_eps": 64 * n * eps, "condition": 10.0 ** (-lo),
           # 64 n eps relative to each sigma is the bound for column-scaled condition <= 1e3;
           # these matrices have Haar factors, so their column-scaled condition is their
           # condition, and the bound that applies is 64 n eps relative to sigma_max
           "relative_bound_applies": bool(10.0 ** (-lo) <= 1e3)}
    for _ in range(warmup):
        mixed()
    ms, (sw, sw32, swf) = timed(mixed, mixed_steps)
    ph = vj.last_mixed_phases()
    sig_m, err_m = results()
    out["mixed"] = dict({"ms_per_matrix": round(ms, 2), "matrices_per_s": round(1000.0 / ms, 4),
                         "steps": mixed_steps, "sweeps_fp32": int(sw32), "sweeps_fp64_plain_dot": int(swf),
                         "sweeps_fp64_reference": int(sw), "fp32_block_sweeps": ph.get("fp32_block_sweeps"),
                         "phases_ms": {k: round(v, 1) for k, v in ph.items() if k.endswith("_ms")},
                         "fp32_roofline": mixed_fp32_roofline(ph, kind, m, n, int(sw32))}, **err_m)
    if plain_steps > 0:
        pms, psw = timed(plain, plain_steps)
        sig_p, err_p = results()
        out["plain"] = dict({"ms_per_matrix": round(pms, 2), "matrices_per_s": round(1000.0 / pms, 5),
                             "steps": plain_steps, "sweeps": int(psw),
                             "flops_per_s": psw * (n * (n - 1) / 2) * per_pair / (pms * 1e-3)}, **err_p)
        rel = float(np.max(np.abs(np.sort(sig_m) - np.sort(sig_p)) / np.sort(sig_p)))
        nrm = float(np.max(np.abs(np.sort(sig_m) - np.sort(sig_p))) / np.max(sig_p))
        out["mixed"]["max_rel_sigma_err_vs_fp64_oracle"] = rel
        out["mixed"]["within_64_n_eps_of_fp64_oracle"] = bool(rel <= 64 * n * eps)
        out["mixed"]["max_sigma_err_vs_fp64_oracle_over_sigma_max"] = nrm
        out["mixed"]["within_64_n_eps_sigma_max_of_fp64_oracle"] = bool(nrm <= 64 * n * eps)
        out["mixed_over_plain"] = round(pms / ms, 3)
    return out


def bench_svd_suite(args, vj, dist, rank, world):
    """The SVD half of the metric beside the 2x2 line: dvjsvd 1024x1024 FP64 (sigma in
    [1e-6, 1]) and zvjsvd 4096x2048 FP64 complex (sigma in [1e-8, 1]), each mixed-precision
    and plain, with matrices/s, sweeps, the mixed/plain ratio and the errors against the
    exact singular values and the FP64 oracle (the plain path, which is the reference's
    algorithm bit for bit)."""
    import torch
    with Clocks(torch.cuda.current_device()) as clk:
        d = svd_case(args, vj, dist, "d", 1024, 1024, -6, mixed_steps=3, plain_steps=1, warmup=1, seed=2024 + rank)
        z = svd_case(args, vj, dist, "z", 4096, 2048, -8, mixed_steps=1, plain_steps=args.svd_plain_steps,
                     warmup=1, seed=2024 + rank)
    dev = device_info()
    for c, cx in ((d, False), (z, True)):
        if "plain" in c:
            c["plain"]["roofline"] = svd_roofline(c["plain"]["flops_per_s"], True,
                                                  "k_step<double,%s>" % ("cplx" if cx else "real"), dev)
    return {"metric": "Jacobi SVD matrices/s at FP64 accuracy, mixed vs plain", "unit": "matrices/s",
            "timing": "CUDA events on the launching stream around each call (inputs resident on the GPU)",
            "dvjsvd_1024x1024": d, "zvjsvd_4096x2048": z, "clocks": clk.summary()}


def cpu_baseline_svd(kind, A, js, stp, sweeps, budget_s=10.0):
    """The oracle's restatement of the reference's ?vjsvd_ (oracle/vjo.c, one host thread)
    on the same matrix: a sweep restricted to the first s pivot steps is timed (s chosen to
    fill about budget_s), and scaled to the full run (stp steps per sweep, sweeps + 1
    sweeps including the converged one)."""
    from oracle import oracle as O
    O.build()
    R = O.Restatement()
    cx = kind in "zc"

    def run(s_):
        t0 = time.perf_counter()
        if cx:
            R.vjsvd(kind, A.real, js[:s_], s_, swp=1, Gi=A.imag)
        else:
            R.vjsvd(kind, A, js[:s_], s_, swp=1)
        return time.perf_counter() - t0

    t1 = run(1)
    s_ = int(max(1, min(stp, budget_s / max(t1, 1e-6))))
    t = run(s_)
    per_sweep = t * stp / s_
    total = per_sweep * (sweeps + 1)
    return {"value": round(1.0 / total, 6), "unit": "matrices/s", "cores": 1, "kind": "port",
            "sample": "%svjsvd_ restatement (oracle/vjo.c), one sweep of %d of %d pivot steps on the same matrix "
                      "(%.1f s), scaled to %d sweeps" % (kind, s_, stp, t, sweeps + 1),
            "seconds_per_matrix": round(total, 1)}


def bench_svd(args, vj, dist, rank, world, kind, m, n):
    import torch
    from vecjac_gb300 import workloads as W
    cx = kind in "zc"
    A, s = W.svd_matrix(m, n, seed=2024 + rank, lo=(-8.0 if cx else -6.0), complex_=cx)
    js, stp = vj.pjs(args.pivot, n)
    dt = np.float64 if kind in "dz" else np.float32
    Gt = torch.tensor(np.ascontiguousarray(A.real.T, dt), device="cuda")
    Git = torch.tensor(np.ascontiguousarray(A.imag.T, dt), device="cuda") if cx else None
    G = torch.empty_like(Gt)
    Gi = torch.empty_like(Gt) if cx else None
    V = torch.empty((n, n), dtype=Gt.dtype, device="cuda")
    Vi = torch.empty_like(V) if cx else None
    eS = torch.empty(n, dtype=Gt.dtype, device="cuda")
    fS = torch.empty_like(eS)
    djs = torch.tensor(js.astype(np.int32), device="cuda")
    stream = torch.cuda.current_stream()

    def one():
        G.copy_(Gt)
        if cx:
            Gi.copy_(Git)
        r = vj.vjsvd_dev(kind, m, n, G, m, V, n, eS, fS, djs, stp, Gi=Gi, ldGi=m, Vi=Vi, ldVi=n,
                         stream=stream.cuda_stream)
        return r

    for _ in range(args.warmup):
        sweeps = one()
    torch.cuda.synchronize()
    barrier(dist)
    with Clocks(torch.cuda.current_device()) as clk:
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for _ in range(args.steps):
            sweeps = one()
        t1.record(stream)
        torch.cuda.synchronize()
    ms = allmax(dist, t0.elapsed_time(t1)) / args.steps
    sig = fS.double().cpu().numpy() * np.exp2(eS.double().cpu().numpy())
    err = float(np.max(np.abs(np.sort(sig)[::-1] - s) / s))
    per_pair = (36 * m + 20 * n) if cx else (12 * m + 6 * n)
    flops = sweeps * (n * (n - 1) / 2) * per_pair
    out = {"metric": "Jacobi SVD matrices/s (%svjsvd_)" % kind, "value": round(world * 1000.0 / ms, 4),
            "unit": "matrices/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(ms, 3), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if kind in "dz" else "f32", "data": "synthetic (Haar factors, log-uniform sigma)",
            "config": {"workload": "%svjsvd_ %dx%d, pivot strategy id %d (modulus ordering; libpvn tables unavailable)"
                       % (kind, m, n, args.pivot),
                       "sweeps": int(sweeps), "max_rel_sigma_err_vs_exact": err},
            "flops_per_s": flops / (ms * 1e-3), "clocks": clk.summary(),
            "gpu_launches": int(sweeps + 1) * stp}
    out["roofline"] = svd_roofline(out["flops_per_s"], kind in "dz",
                                   "k_step<%s,%s>" % ("double" if kind in "dz" else "float",
                                                      "cplx" if cx else "real"))
    if rank == 0 and args.cpu_baseline:
        out["cpu_baseline"] = cpu_baseline_svd(kind, A, js, stp, int(sweeps))
    return out


def bench_mixed(args, vj, dist, rank, world, kind, m, n):
    """Mixed-precision SVD (FP32 presweeps, FP64 finish) against the plain FP64 SVD of the
    same matrix: the mixed path is timed over K steps after W warm-ups, the plain one over
    --plain-steps runs (it is the slow arm); both sigma sets are compared with the exact
    sigma of the synthetic matrix."""
    import torch
    from vecjac_gb300 import workloads as W
    cx = kind == "z"
    A, s = W.svd_matrix(m, n, seed=2024 + rank, lo=(-8.0 if cx else -6.0), complex_=cx)
    js, stp = vj.pjs(args.pivot, n)
    Gt = torch.tensor(np.ascontiguousarray(A.real.T), dtype=torch.float64, device="cuda")
    Git = torch.tensor(np.ascontiguousarray(A.imag.T), dtype=torch.float64, device="cuda") if cx else None
    G = torch.empty_like(Gt)
    Gi = torch.empty_like(Gt) if cx else None
    V = torch.empty((n, n), dtype=torch.float64, device="cuda")
    Vi = torch.empty_like(V) if cx else None
    eS = torch.empty(n, dtype=torch.float64, device="cuda")
    fS = torch.empty_like(eS)
    djs = torch.tensor(js.astype(np.int32), device="cuda")
    stream = torch.cuda.current_stream()

    def reset():
        G.copy_(Gt)
        if cx:
            Gi.copy_(Git)

    def mixed():
        reset()
        return vj.vjsvd_mixed_dev(kind, m, n, G, m, V, n, eS, fS, djs, stp, Gi=Gi, ldGi=m, Vi=Vi, ldVi=n,
                                  stream=stream.cuda_stream, stages=args.stages)

    def plain():
        reset()
        return vj.vjsvd_dev(kind, m, n, G, m, V, n, eS, fS, djs, stp, Gi=Gi, ldGi=m, Vi=Vi, ldVi=n,
                            stream=stream.cuda_stream)

    def sigma_err():
        sig = fS.cpu().numpy() * np.exp2(eS.cpu().numpy())
        srt = np.sort(sig)[::-1]
        return srt, float(np.max(np.abs(srt - s) / s)), float(np.max(np.abs(srt - s)) / s[0])

    def timed(fn, k):
        torch.cuda.synchronize()
        barrier(dist)
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for _ in range(k):
            r = fn()
        t1.record(stream)
        torch.cuda.synchronize()
        return allmax(dist, t0.elapsed_time(t1)) / k, r

    for _ in range(args.warmup):
        mixed()
    with Clocks(torch.cuda.current_device()) as clk:
        ms, (sw64, sw32, swf) = timed(mixed, args.steps)
    rot64 = vj.last_trace()["rotations"]
    phases = vj.last_mixed_phases()
    sig_m, rel_m, nrm_m = sigma_err()
    out = {"metric": "Jacobi SVD matrices/s (%svjsvd mixed FP32->FP64)" % kind,
           "value": round(world * 1000.0 / ms, 5), "unit": "matrices/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic (Haar factors, log-uniform sigma in [%g, 1])" % (1e-8 if cx else 1e-6),
           "config": {"workload": "%svjsvd_ %dx%d mixed precision (FP32 block-sweep rounds, each with Newton-Schulz "
                                  "steps, then FP64 finishing sweeps), pivot strategy id %d" % (kind, m, n, args.pivot),
                      "stages": args.stages or 2,
                      "sweeps_fp32": int(sw32), "sweeps_fp64_plain_dot": int(swf), "sweeps_fp64": int(sw64),
                      "fp64_rotations_per_sweep": rot64,
                      "max_rel_sigma_err_vs_exact": rel_m, "max_sigma_err_over_sigma_max": nrm_m},
           "phases_ms": {k: round(v, 1) for k, v in phases.items() if k.endswith("_ms")},
           "clocks": clk.summary()}
    out["roofline"] = mixed_fp32_roofline(phases, kind, m, n, int(sw32))
    if args.plain_steps > 0:
        pms, psw = timed(plain, args.plain_steps)
        sig_p, rel_p, nrm_p = sigma_err()
        out["plain"] = {"ms_per_step": round(pms, 3), "steps": args.plain_steps, "sweeps": int(psw),
                        "max_rel_sigma_err_vs_exact": rel_p, "max_sigma_err_over_sigma_max": nrm_p,
                        "max_rel_sigma_diff_mixed_vs_plain": float(np.max(np.abs(sig_m - sig_p) / sig_p))}
        out["speedup_vs_plain"] = round(pms / ms, 3)
        if rank == 0 and args.cpu_baseline:
            out["cpu_baseline"] = cpu_baseline_svd(kind, A, js, stp, int(psw))
    return out


def mixed_fp32_roofline(phases, kind, m, n, sweeps32):
    """Tensor-pipe roofline of the FP32 stages of the mixed SVD when they ran as block sweeps:
    the split-BF16x3 products of every block step (per block pair: the 128 x 128 Gram matrix
    over m rows, and the rotation of m + n rows of 128 columns, each 2 x 128 x 128 flops per
    row and term) over the whole FP32 phase time (which includes the pair eigenproblems on
    the CUDA cores), against the measured BF16 peak. None for column-pair sweeps (their
    operands live in L2: no HBM or tensor roofline applies)."""
    if not (phases.get("fp32_block_sweeps") and phases["fp32_ms"] > 0 and sweeps32 > 0):
        return None
    pk, src = peaks()
    terms = 3 if os.environ.get("VJ_BLOCK_TERMS") == "3" else 6
    nb = n // (32 if kind == "z" else 64)
    flops = sweeps32 * (nb - 1) * (nb // 2) * 2.0 * 128 * 128 * (2 * m + n) * terms
    ach = flops / (phases["fp32_ms"] * 1e-3) / 1e12
    peak = pk.get("bf16_tflops_sustained") or pk["bf16_tflops"]
    return {"bound": "tensor", "kernel": "k_gram + k_apply (split-BF16x3 tcgen05, %d terms)" % terms,
            "achieved": round(ach, 2), "peak": peak, "unit": "TFLOP/s", "frac": round(ach / peak, 4),
            "traffic": None, "peak_source": src + " (bf16 sustained)",
            "note": "BF16 tensor flops of the Gram and rotation products over the whole FP32 phase, pair "
                    "eigenproblems and launch gaps included"}


def bench_diff(args, vj, dist, rank, world):
    """Differentiable batched SVD: 4096 FP32 matrices 128x64, sigma uniform in [0.1, 10] with
    relative gaps >= 1e-3, loss = sum_i w_i s_i + <G_U, U_k> + <G_V, V_k>, k = 16. One step =
    forward (batched SVD in one persistent launch, sort, sign fix, loss) + backward (the
    adjoint kernel). The adjoint launch is also timed alone (its own CUDA events)."""
    import torch
    from vecjac_gb300 import autodiff as AD
    count, m, n, k = args.diff_count, 128, 64, 16
    A64, _ = AD.spaced_sigma_matrices(count, m, n, seed=91 + rank)
    rng = np.random.default_rng(92 + rank)
    w, GU, GV = rng.standard_normal((count, n)), rng.standard_normal((count, m, k)), rng.standard_normal((count, n, k))
    t32 = lambda x: torch.tensor(x, dtype=torch.float32, device="cuda")
    A, w32, GU32, GV32 = t32(A64), t32(w), t32(GU), t32(GV)

    def step():
        X = A.clone().requires_grad_(True)
        S, Uk, Vk = AD.svd_k(X, k)
        L = (w32 * S).sum() + (GU32 * Uk).sum() + (GV32 * Vk).sum()
        L.backward()
        return X.grad

    for _ in range(args.warmup):
        g = step()
    torch.cuda.synchronize()
    barrier(dist)
    with Clocks(torch.cuda.current_device()) as clk:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            g = step()
        e1.record()
        torch.cuda.synchronize()
    ms = allmax(dist, e0.elapsed_time(e1)) / args.steps
    # the adjoint kernel alone, on the saved factors of one forward
    with torch.no_grad():
        S, U, V, _ = AD.svd_batch_dev(A)
        S, U, V = AD._sort_and_fix(S, U, V)
    Uc, Vc = U.contiguous(), V.contiguous()
    for _ in range(3):
        AD.adjoint(Uc, S, Vc, w32, GU32, GV32)
    torch.cuda.synchronize()
    a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 20
    a0.record()
    for _ in range(reps):
        AD.adjoint(Uc, S, Vc, w32, GU32, GV32)
    a1.record()
    torch.cuda.synchronize()
    adj_ms = a0.elapsed_time(a1) / reps
    adj_bytes = count * 4.0 * (m * n + n * n + m * k + n * k + 2 * n + m * n)
    adj_flops = count * 2.0 * (m * n * k + n * n * k + n ** 3 + m * n * (n + k))
    pk, src = peaks()
    achieved = adj_bytes / (adj_ms * 1e-3) / 1e9
    # gradient error vs torch.linalg.svd (FP64 on the GPU) on a sample of the batch; torch's
    # GPU SVD loads its own linear-algebra library, which can be missing (then: reported)
    ns = min(count, 256)
    t64 = lambda x: torch.tensor(x, dtype=torch.float64, device="cuda")
    try:
        At = torch.tensor(A64[:ns], dtype=torch.float64, device="cuda", requires_grad=True)
        Ut, St, Vht = torch.linalg.svd(At, full_matrices=False)
        Vt = Vht.mT
        with torch.no_grad():
            piv = torch.argmax(Vt.abs(), dim=1, keepdim=True)
            sg = torch.sign(torch.gather(Vt, 1, piv))
        Ut, Vt = Ut * sg, Vt * sg
        Lt = (t64(w[:ns]) * St).sum() + (t64(GU[:ns]) * Ut[:, :, :k]).sum() + (t64(GV[:ns]) * Vt[:, :, :k]).sum()
        Lt.backward()
        ref = At.grad
        err_torch = float(torch.max(torch.amax((g[:ns].double() - ref).abs(), dim=(1, 2)) /
                                    torch.amax(ref.abs(), dim=(1, 2))))
    except RuntimeError as e:
        err_torch = "torch.linalg.svd unavailable: %s" % str(e).splitlines()[-1][:120]
    # FP64 path against central finite differences (h = 1e-6) on 8 matrices, 2 directions
    nf = 8
    A8 = torch.tensor(A64[:nf], dtype=torch.float64, device="cuda", requires_grad=True)
    w8, GU8, GV8 = t64(w[:nf]), t64(GU[:nf]), t64(GV[:nf])
    S8, U8, V8 = AD.svd_k(A8, k)
    ((w8 * S8).sum() + (GU8 * U8).sum() + (GV8 * V8).sum()).backward()

    def losses(X):
        with torch.no_grad():
            S_, U_, V_ = AD.svd_k(X, k)
            return ((w8 * S_).sum(1) + (GU8 * U_).sum((1, 2)) + (GV8 * V_).sum((1, 2))).cpu().numpy()

    h, err_fd = 1e-6, 0.0
    for _ in range(2):
        E = torch.tensor(rng.standard_normal((nf, m, n)), dtype=torch.float64, device="cuda")
        fd = (losses(A8.detach() + h * E) - losses(A8.detach() - h * E)) / (2 * h)
        an = (A8.grad * E).sum((1, 2)).cpu().numpy()
        err_fd = max(err_fd, float(np.max(np.abs(fd - an) / np.maximum(1.0, np.abs(an)))))
    out = {"metric": "differentiable batched SVD matrices/s (forward + adjoint)", "value": round(world * count * 1000.0 / ms, 1),
           "unit": "matrices/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": round(ms, 3), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32", "data": "synthetic (Haar factors, sigma uniform in [0.1, 10], relative gaps >= 1e-3)",
           "config": {"workload": "%d FP32 matrices %dx%d, loss sum w s + <G_U,U_k> + <G_V,V_k>, k=%d" % (count, m, n, k),
                      "l2": "inputs larger than L2 (A alone is %d MB), no flush" % (count * m * n * 4 // 10 ** 6)},
           "adjoint": {"ms": round(adj_ms, 4), "gflops": round(adj_flops / (adj_ms * 1e-3) / 1e9, 1),
                       "max_rel_grad_err_vs_torch_fp64": err_torch, "max_rel_grad_err_fp64_vs_fd": err_fd},
           "roofline": {"kernel": "k_svd_adjoint<float>", "bound": "hbm", "achieved": round(achieved, 1),
                        "peak": pk["hbm_gbs"], "unit": "GB/s", "frac": round(achieved / pk["hbm_gbs"], 4),
                        "traffic": None, "peak_source": src},
           "clocks": clk.summary(), "gpu_launches": 2 * args.steps}
    if rank == 0 and args.cpu_baseline:
        torch.set_num_threads(8)
        nc = 256
        Ac = torch.tensor(A64[:nc], dtype=torch.float32, requires_grad=True)
        wc, GUc, GVc = [torch.tensor(x[:nc], dtype=torch.float32) for x in (w, GU, GV)]
        t0 = time.perf_counter()
        Uc_, Sc_, Vhc_ = torch.linalg.svd(Ac, full_matrices=False)
        ((wc * Sc_).sum() + (GUc * Uc_[:, :, :k]).sum() + (GVc * Vhc_.mT[:, :, :k]).sum()).backward()
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": round(nc / dt, 1), "unit": "matrices/s", "cores": 8, "kind": "torch",
                               "sample": "torch.linalg.svd forward + backward, %d of the FP32 matrices, CPU" % nc}
    return out


def gen_uneven(count, seed, kind):
    """The uneven-batch workload: m ~ U{16..512}, n ~ U{8..m}, A = Q1 diag(sigma) Q2^T with
    Q1, Q2 from QR of Gaussian matrices and sigma = 10^U(-4, 0) per matrix (host threads)."""
    from concurrent.futures import ThreadPoolExecutor
    rng = np.random.default_rng(seed)
    m = rng.integers(16, 513, count)
    n = np.array([rng.integers(8, int(mm) + 1) for mm in m])
    seeds = rng.integers(0, 2 ** 63 - 1, count)

    def one(i):
        r = np.random.default_rng(int(seeds[i]))
        q1, _ = np.linalg.qr(r.standard_normal((int(m[i]), int(n[i]))))
        q2, _ = np.linalg.qr(r.standard_normal((int(n[i]), int(n[i]))))
        s = 10.0 ** r.uniform(-4.0, 0.0, int(n[i]))
        return ((q1 * s) @ q2.T).astype(np.float64 if kind == "d" else np.float32)

    with ThreadPoolExecutor(os.cpu_count()) as ex:
        return list(ex.map(one, range(count)))


def bench_batch(args, vj, dist, rank, world, kind):
    import torch
    from vecjac_gb300 import batch as B
    mats = gen_uneven(args.batch_count, 77 + rank, kind)
    b = B.Batch(mats, kind)
    blk, occ = B.autotune(b, args.pivot)
    g = B.capture(b, args.pivot, block=blk, occupancy=occ)
    for _ in range(max(0, args.warmup - 1)):
        g.replay()
    torch.cuda.synchronize()
    barrier(dist)
    with Clocks(torch.cuda.current_device()) as clk:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            g.replay()
        e1.record()
        torch.cuda.synchronize()
    ms = allmax(dist, e0.elapsed_time(e1)) / args.steps
    info = b.info.cpu().numpy()
    flops = b.flops(np.maximum(info, 0))
    # the same matrices one launch sequence per matrix (vj_?vjsvd_dev) on a sample
    sample = min(args.batch_sample, len(mats))
    idx = np.random.default_rng(5).choice(len(mats), sample, replace=False)
    t = 0.0
    for i in idx:
        A = mats[i]
        m2, n2 = B.padded_shape(A.shape[0], A.shape[1], kind)
        P = np.zeros((m2, n2), A.dtype)
        P[:A.shape[0], :A.shape[1]] = A
        js, stp = vj.pjs(args.pivot, n2)
        Gd = torch.tensor(P.T.copy(), device="cuda")
        Vd = torch.empty((n2, n2), dtype=Gd.dtype, device="cuda")
        eS = torch.empty(n2, dtype=Gd.dtype, device="cuda")
        fS = torch.empty_like(eS)
        dj = torch.tensor(js.astype(np.int32), device="cuda")
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        vj.vjsvd_dev(kind, m2, n2, Gd, m2, Vd, n2, eS, fS, dj, stp)
        torch.cuda.synchronize()
        t += time.perf_counter() - t0
    per_launch = len(mats) * (t / sample)
    out = {"metric": "batched Jacobi SVD matrices/s (%svjsvd_, uneven sizes)" % kind,
            "value": round(world * len(mats) / (ms * 1e-3), 2), "unit": "matrices/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 2), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64" if kind == "d" else "f32",
            "data": "synthetic (m~U[16,512], n~U[8,m], Q1 diag(sigma) Q2^T, sigma=10^U(-4,0))",
            "config": {"workload": "%d matrices in one persistent launch (CUDA graph), pivot id %d, block %d, "
                       "register bound for %d CTAs of 256 threads per SM (autotuned)"
                       % (len(mats), args.pivot, blk, occ), "errors": int((info < 0).sum()),
                       "mean_sweeps": float(info[info >= 0].mean())},
            "flops_per_s": flops / (ms * 1e-3),
            "one_launch_per_matrix_s_estimate": round(per_launch, 2),
            "speedup_vs_per_matrix_launches": round(per_launch / (ms * 1e-3), 2),
            "clocks": clk.summary(), "gpu_launches": 2 * args.steps}
    out["roofline"] = svd_roofline(out["flops_per_s"], kind == "d",
                                   "k_batch<%s>" % ("double" if kind == "d" else "float"))
    if rank == 0 and args.cpu_baseline:
        out["cpu_baseline"] = cpu_baseline_batch(mats, kind, args.pivot)
    return out


def cpu_baseline_batch(mats, kind, pivot, budget_s=10.0):
    """The oracle's restatement of ?vjsvd_ (oracle/vjo.c) on every host thread, one matrix per
    task, over a random sample of the batch (zero-padded like the GPU batch) sized to fill
    about budget_s; reported as whole-batch matrices/s."""
    from concurrent.futures import ThreadPoolExecutor

    from oracle import oracle as O
    from vecjac_gb300 import batch as B
    O.build()
    R = O.Restatement()
    threads = os.cpu_count()
    rng = np.random.default_rng(6)
    order = rng.permutation(len(mats))

    def one(i):
        A = mats[i]
        m2, n2 = B.padded_shape(A.shape[0], A.shape[1], kind)
        P = np.zeros((m2, n2), A.dtype)
        P[:A.shape[0], :A.shape[1]] = A
        js, stp = R.pjs(pivot, n2)
        R.vjsvd(kind, P, js, stp)

    done, t0 = 0, time.perf_counter()
    with ThreadPoolExecutor(threads) as ex:
        while time.perf_counter() - t0 < budget_s and done < len(mats):
            chunk = order[done:done + threads]
            list(ex.map(one, chunk))
            done += len(chunk)
    el = time.perf_counter() - t0
    return {"value": round(done / el, 2), "unit": "matrices/s", "cores": threads, "kind": "port",
            "sample": "%d random matrices of the batch through the %svjsvd_ restatement (oracle/vjo.c), one per host "
                      "thread, %.1f s" % (done, kind, el)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="bjac2", choices=["bjac2", "fma_probe", "svd1024", "zsvd", "zsvd_mixed", "dsvd_mixed",
                                                             "batch_d", "batch_s", "diff"])
    ap.add_argument("--diff-count", type=int, default=4096, help="matrices of the differentiable batch")
    ap.add_argument("--svd-m", type=int, default=0, help="rows of the SVD workloads (0: the workload's own)")
    ap.add_argument("--svd-n", type=int, default=0, help="columns of the SVD workloads (0: the workload's own)")
    ap.add_argument("--plain-steps", type=int, default=1, help="timed runs of the plain FP64 arm of *_mixed")
    ap.add_argument("--stages", type=int, default=0, help="FP32 preconditioning rounds of *_mixed (0: library default)")
    ap.add_argument("--batch-count", type=int, default=20000)
    ap.add_argument("--batch-sample", type=int, default=40)
    ap.add_argument("--scale", type=int, default=0, help="shrink the 2x2 batches by 2^scale")
    ap.add_argument("--e2e-shift", type=int, default=0, help="further shrink of the e2e batches")
    ap.add_argument("--no-e2e", dest="e2e", action="store_false")
    ap.add_argument("--no-cpu", dest="cpu_baseline", action="store_false")
    ap.add_argument("--no-svd", dest="svd", action="store_false",
                    help="leave the SVD object (dvjsvd 1024^2 and zvjsvd 4096x2048) out of the default line")
    ap.add_argument("--svd-plain-steps", type=int, default=1,
                    help="timed runs of the plain zvjsvd 4096x2048 in the SVD object (0: skip, ~1 min each)")
    ap.add_argument("--cpu-elems", type=int, default=24)
    ap.add_argument("--pivot", type=int, default=4, help="pivot strategy id for the SVD workloads")
    args = ap.parse_args()
    if args.impl == "reference":
        rank = int(os.environ.get("RANK", "0"))
        out = reference_arm(args, None, rank)
        if out is not None:
            print(json.dumps(out))
        return
    import torch
    dist, rank, world = dist_init(args.gpus)
    from vecjac_gb300 import build
    build.build()
    import vecjac_gb300 as vj
    if args.workload == "bjac2":
        out = bench_bjac2(args, vj, dist, rank, world)
    elif args.workload == "fma_probe":
        out = bench_fma_probe(args, vj)
    elif args.workload == "svd1024":
        out = bench_svd(args, vj, dist, rank, world, "d", 1024, 1024)
    elif args.workload.startswith("batch_"):
        out = bench_batch(args, vj, dist, rank, world, args.workload[-1])
    elif args.workload == "diff":
        out = bench_diff(args, vj, dist, rank, world)
    elif args.workload == "zsvd_mixed":
        out = bench_mixed(args, vj, dist, rank, world, "z", args.svd_m or 4096, args.svd_n or 2048)
    elif args.workload == "dsvd_mixed":
        out = bench_mixed(args, vj, dist, rank, world, "d", args.svd_m or 4096, args.svd_n or 2048)
    else:
        out = bench_svd(args, vj, dist, rank, world, "z", args.svd_m or 4096, args.svd_n or 2048)
    if rank == 0:
        print(json.dumps(out))
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
