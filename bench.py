#!/usr/bin/env python
"""Throughput of extract_pore_network on GB300 (Gvoxel/s), one JSON line on rank 0.

Workload (one "step"): extract_pore_network on a 512^3 float32 SDF of polydisperse overlapping
spheres (log-normal radii, mean 10 voxels, sigma 0.25, porosity 0.4, periodic min-image distance),
seeded synthetic data generated on the device; outputs pores, int32 labels and connections.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

value  : voxels / device time per step, SDF resident in HBM, results left on the device
         (pnm_extract_pore_network_dev), timed with CUDA events on the library's stream.
e2e    : the same metric through the host C ABI (pnm_extract_pore_network) from pinned host
         memory: H2D of the SDF and D2H of labels, pores and pairs inside every timed step.
roofline: the whole pipeline against the 64 B/voxel algorithmic model of the extraction path
         (pores 4, markers+CCL 8, flood 12, gradient roots 8, renumbering 28, topology 4) and the
         measured HBM copy bandwidth.
N > 1  : independent replicas, one volume per rank (the path does not shard): scaling "weak".
--impl reference: the reference's CPU implementation on this host's cores (the reference header
         built against the Kokkos shim where its checkout exists, otherwise the project's C++
         restatement of it), each step one extract_pore_network of the same 512^3 volume. This
         arm never loads the product library: the volume comes from the generator module loaded
         by path (torch on the GPU when present, numpy otherwise).
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Gvoxel/s extract_pore_network, batched vs plain on same GB300; p50/p99 latency"
ALG_BYTES_PER_VOXEL = 64  # extract_pore_network algorithmic bytes per voxel
FALLBACK_HBM_GBS = 6800.0


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--size", type=int, default=512, help="cube edge of the benchmark volume")
    ap.add_argument("--cpu-sample", type=int, default=0,
                    help="cube edge of the CPU baseline sample (0: the whole benchmark volume)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true",
                    help="skip the ragged 96-volume batched-vs-plain measurement")
    ap.add_argument("--no-served", action="store_true",
                    help="skip the Poisson serving measurement")
    ap.add_argument("--no-flow", action="store_true",
                    help="skip the 256^3 float64 extract_network_flow measurement")
    ap.add_argument("--profile", choices=["plain", "flow"], default=None,
                    help="run one call of a leg inside an NVTX range named 'profiled_call' "
                         "(after warm-up calls) and exit: the target of an ncu launch list")
    ap.add_argument("--batch-volumes", type=int, default=96)
    ap.add_argument("--serve-requests", type=int, default=400,
                    help="requests per arrival rate of the serving sweep")
    return ap.parse_args()


def measured_hbm_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        return float(json.load(open(p))["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def profile_traffic():
    """(DRAM bytes per pipeline call, the commit the ncu capture was taken at) from the committed
    launch-list summary under profiles/; (None, None) without it."""
    p = os.path.join(ROOT, "profiles", "extract_pore_network_512_launches.txt")
    traffic = commit = None
    try:
        for line in open(p):
            if line.startswith("dram_bytes_per_call:"):
                traffic = int(float(line.split(":")[1]))
            elif line.startswith("taken_at_commit:"):
                commit = line.split(":")[1].strip()
    except OSError:
        pass
    return traffic, commit


def workload_config(n_edge):
    return {"workload": f"extract_pore_network {n_edge}^3 float32 polydisperse sphere packing",
            "voxels": n_edge ** 3, "radius": "log-normal mean 10 voxels sigma 0.25",
            "porosity": 0.4, "sdf": "periodic min-image, negative in solid", "seed": 2,
            "l2": "SDF (4 B/voxel) and labels exceed the 129 MB L2 every step; no flush needed",
            "parallelism": "replicas (one volume per GPU)"}


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.path = tempfile.mktemp(suffix=".csv")
        self.proc = None
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(gpu_index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"], stdout=self.f,
                stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[3:7]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def replica_seed(rank: int) -> int:
    """Each rank extracts its own volume (replicas: the path does not shard one volume)."""
    return 2 + rank


def whole_job_rate(local_value: float, voxels_per_rank: int, world: int, device) -> tuple:
    """(max over ranks of a per-rank step time, whole-job Gvoxel/s = all ranks' voxels / that
    time). Rank timings are combined with an all-reduce MAX when a process group is up."""
    import torch

    t = torch.tensor([float(local_value)], dtype=torch.float64, device=device)
    if world > 1 and torch.distributed.is_initialized():
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    worst = float(t.item())
    return worst, voxels_per_rank * world / worst / 1e9


def load_synthetic():
    """peclet_pnm_gb300/synthetic.py loaded by path: numpy / torch only, so the reference arm
    gets the benchmark volume without importing the package (which loads the CUDA library)."""
    import importlib.util

    spec = importlib.util.spec_from_file_location(
        "pnm_synthetic", os.path.join(ROOT, "peclet_pnm_gb300", "synthetic.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def gen_volume(n_edge, seed, device):
    return load_synthetic().packing((n_edge, n_edge, n_edge), 0.4, seed=seed, device=device)


def cpu_sample_run(n_edge, threads, kind, sdf_np):
    from oracle import Oracle

    o = Oracle(kind, threads=threads, openmp_ref=True) if kind == "reference" else \
        Oracle("port", threads=threads)
    t = time.perf_counter()
    o.extract_pore_network(sdf_np, [0.0] * 3, [1.0] * 3)
    return time.perf_counter() - t


def sample_volume(n_edge, seed):
    try:
        import torch

        if torch.cuda.is_available():
            return gen_volume(n_edge, seed, "cuda").cpu().numpy()
    except Exception:
        pass
    return gen_volume(n_edge, seed, None)


def reference_arm(args, rank):
    if rank != 0:
        return
    from oracle import reference_available

    kind = "reference" if reference_available() else "port"
    threads = os.cpu_count() or 1
    # the volume `ours` times at N=1 (rank 0's replica seed), whole, every step
    sdf = sample_volume(args.size, replica_seed(0))
    vox = sdf.size
    for _ in range(args.warmup):
        cpu_sample_run(args.size, threads, kind, sdf)
    ts = [cpu_sample_run(args.size, threads, kind, sdf) for _ in range(args.steps)]
    t = sum(ts) / len(ts)
    value = vox / t / 1e9
    impl = ("the reference's src/pore_extraction.hpp built against the project's Kokkos-compat "
            "OpenMP shim" if kind == "reference" else
            "the project's C++ restatement of the reference algorithm (OpenMP); the reference "
            "checkout is absent on this host")
    sample = (f"the whole {args.size}^3 benchmark volume (seed {replica_seed(0)}) per step, "
              f"one extract_pore_network on {threads} host threads: {impl}")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": "Gvoxel/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "config": workload_config(args.size),
        "cpu_baseline": {"value": value, "unit": "Gvoxel/s", "cores": threads, "kind": kind,
                         "sample": sample},
        "e2e": {"value": value, "unit": "Gvoxel/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0}}), flush=True)


def batched_bench(args, dev):
    """Ragged batch: 96 packings, edges drawn per axis from {48,...,192} (seed 5+i), porosity
    U[0.3,0.6]. Batched (one launch per stage, graph replay) vs the plain per-volume path in a loop,
    both with the SDFs resident; e2e adds the H2D of every SDF from pinned memory and the D2H of
    every result (labels, pores, pairs)."""
    import torch

    import peclet_pnm_gb300 as pnm
    from peclet_pnm_gb300 import _capi
    from peclet_pnm_gb300 import synthetic as syn

    shapes = syn.batch_shapes(args.batch_volumes)
    vols = [syn.packing(sh, phi, seed=sd, device=dev) for sh, phi, sd in shapes]
    torch.cuda.synchronize(dev)
    nvox = sum(int(v.numel()) for v in vols)
    ctx = pnm.Context(dev.index)
    stream = torch.cuda.current_stream(dev)
    ctx.set_stream(stream.cuda_stream)
    o = np.zeros(3, np.float32)
    s = np.ones(3, np.float32)
    maxn = max(int(v.numel()) for v in vols)
    d_seg = torch.empty(maxn, dtype=torch.int32, device=dev)
    d_pores = torch.empty((1_000_000, 4), dtype=torch.float32, device=dev)
    pair_cap = 8_000_000
    d_pairs = torch.empty((pair_cap, 2), dtype=torch.int32, device=dev)
    npo, npa = _capi._i64(), _capi._i64()

    def plain_all():
        for v in vols:
            nz, ny, nx = v.shape
            ctx.check(_capi.pnm_extract_pore_network_dev(
                ctx.h, v.data_ptr(), nx, ny, nz, _capi.as_ptr(o), _capi.as_ptr(s),
                d_pores.data_ptr(), 1_000_000, ctypes.byref(npo), d_seg.data_ptr(),
                d_pairs.data_ptr(), pair_cap, ctypes.byref(npa)))

    for _ in range(args.warmup):
        plain_all()
    torch.cuda.synchronize(dev)
    l0 = ctx.stats()["launches"]
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        plain_all()
    e1.record(stream)
    torch.cuda.synchronize(dev)
    plain_ms = e0.elapsed_time(e1) / args.steps
    plain_launches = (ctx.stats()["launches"] - l0) // args.steps

    b = pnm.Batch([tuple(v.shape) for v in vols])
    for i, v in enumerate(vols):
        b.check(_capi.pnm_batch_set_sdf(b.h, i, ctypes.c_void_p(v.data_ptr())))
    # launch shape for this size class (timed on this data; not part of the timed region)
    t_tune = time.perf_counter()
    tuned = b.autotune(cache=os.path.join(tempfile.mkdtemp(), "tune.txt"), reps=2)
    t_tune = time.perf_counter() - t_tune
    bstream = torch.cuda.ExternalStream(b.stream, device=dev)
    for _ in range(args.warmup):
        b.run()
    e0.record(bstream)
    for _ in range(args.steps):
        b.launch()
        b.wait()
    e1.record(bstream)
    torch.cuda.synchronize(dev)
    batch_ms = e0.elapsed_time(e1) / args.steps

    # e2e: pinned host SDFs in, every volume's labels, pores and pairs out, each step
    hs = [torch.empty(v.shape, dtype=torch.float32, pin_memory=True) for v in vols]
    for h, v in zip(hs, vols):
        h.copy_(v)
    infos = [b.volume(i) for i in range(len(vols))]
    tot_p = sum(v["n_pores"] for v in infos)
    tot_q = sum(v["n_pairs"] for v in infos)
    hseg = torch.empty(nvox + 1, dtype=torch.int32, pin_memory=True)
    hpores = torch.empty(4 * tot_p + 4, dtype=torch.float32, pin_memory=True)
    hpairs = torch.empty(2 * tot_q + 2, dtype=torch.int32, pin_memory=True)

    def e2e_step():
        for i, h in enumerate(hs):
            b.check(_capi.pnm_batch_set_sdf(b.h, i, ctypes.c_void_p(h.data_ptr())))
        b.run()
        so = po = qo = 0
        for i in range(len(hs)):
            b.check(_capi.pnm_batch_copy_out(
                b.h, i, ctypes.c_void_p(hpores.data_ptr() + 16 * po),
                ctypes.c_void_p(hseg.data_ptr() + 4 * so),
                ctypes.c_void_p(hpairs.data_ptr() + 8 * qo)))
            so += infos[i]["nx"] * infos[i]["ny"] * infos[i]["nz"]
            po += infos[i]["n_pores"]
            qo += infos[i]["n_pairs"]
        return 4 * so, 4 * so + 16 * po + 8 * qo

    e2e_step()
    t0 = time.perf_counter()
    k = max(3, min(args.steps, 5))
    for _ in range(k):
        h2d, d2h = e2e_step()
    t_e2e = (time.perf_counter() - t0) / k
    st = b.stats()
    out = {
        "workload": f"{len(vols)} ragged float32 packings, edges per axis from "
                    "{48,64,96,128,160,192}, porosity U[0.3,0.6], seeds 5+i",
        "voxels": nvox,
        "batched": {"value": nvox / (batch_ms * 1e-3) / 1e9, "unit": "Gvoxel/s",
                    "ms_per_step": batch_ms, "gpu_launches": int(st["launches"]),
                    "cuda_graph": b.uses_graph,
                    "tuning": {k: v for k, v in tuned.items() if k != "ms"},
                    "autotune_s": t_tune},
        "plain": {"value": nvox / (plain_ms * 1e-3) / 1e9, "unit": "Gvoxel/s",
                  "ms_per_step": plain_ms, "gpu_launches": int(plain_launches)},
        "batched_over_plain": plain_ms / batch_ms,
        "e2e": {"value": nvox / t_e2e / 1e9, "unit": "Gvoxel/s", "ms_per_step": t_e2e * 1e3,
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
        "outputs": {"pores": int(st["n_pores"]), "pairs": int(st["n_pairs"]),
                    "flood_sweeps": int(st["flood_sweeps"])},
    }
    b.close()
    ctx.close()
    del vols
    torch.cuda.empty_cache()
    return out


FLOW_BYTES_PER_VOXEL = 164  # extract_network_flow algorithmic bytes per voxel (60 + 104)


def flow_inputs(dev, n=256):
    """The 256^3 float64 packing (seed 3) and its Fourier fields (seed 4), on the device."""
    from peclet_pnm_gb300 import synthetic as syn

    sdf = syn.packing((n, n, n), 0.4, seed=3, dtype=np.float64, device=dev)
    return sdf, syn.fourier_fields_device(sdf)


def flow_bench(args, dev):
    """extract_network_flow on a 256^3 float64 packing (seed 3) with u, v, w, p = 32 random Fourier
    modes (|k| <= 8, amplitude 1e-3, seed 4) zeroed in solid, openness clamp(0.5 + face SDF, 0, 1),
    grad_p_zyx = [0, 0, -1e-4].

    `device`: pnm_extract_network_flow_dev on device-resident inputs (a solver's fields handed over
    in place), CUDA events on the context's stream; its roofline is the 164 B/voxel model against
    the measured HBM peak. `e2e`: the host C ABI call (host SDF and fields in, host results out,
    the reference binding's call). `h2d`: the pinned host-to-device copy of the same 1.07 GB of
    inputs alone, which bounds the host call from below. Check: the pore residuals of a closed
    periodic network sum to zero. `cpu_baseline`: the oracle port on all host cores, one call."""
    import torch

    import peclet_pnm_gb300 as pnm
    from peclet_pnm_gb300 import _capi

    n = 256
    sdf, fields = flow_inputs(dev, n)
    o = np.zeros(3, np.float32)
    s = np.ones(3, np.float32)
    g = np.array([0.0, 0.0, -1e-4], np.float64)[::-1].copy()  # xyz
    # device-resident leg
    d_sdf = sdf.to(torch.float32).contiguous()
    d_f = [f.contiguous() for f in fields]
    ctx = pnm.Context(dev.index)
    stream = torch.cuda.Stream(dev)
    ctx.set_stream(stream.cuda_stream)
    rd = _capi.PnmFlowResultDev()

    def call_dev():
        ctx.check(_capi.pnm_extract_network_flow_dev(
            ctx.h, ctypes.c_void_p(d_sdf.data_ptr()), n, n, n, _capi.as_ptr(o), _capi.as_ptr(s),
            *[ctypes.c_void_p(f.data_ptr()) for f in d_f], _capi.as_ptr(g), ctypes.byref(rd)))

    for _ in range(3):
        call_dev()
    stream.synchronize()
    reps = 10
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        call_dev()
    e1.record(stream)
    e1.synchronize()
    t_dev = e0.elapsed_time(e1) / 1e3 / reps
    dev_counts = (int(rd.n_pores), int(rd.n_throats))
    ctx.set_timing(True)
    call_dev()
    stage_ms = ctx.stats()["stage_ms"]
    ctx.set_timing(False)
    ctx.set_stream(None)
    # pinned host copies of the inputs; the H2D of all of them alone, for scale
    h_sdf = torch.empty((n, n, n), dtype=torch.float32, pin_memory=True)
    h_sdf.copy_(d_sdf)
    hf = []
    for f in fields:
        h = torch.empty((n, n, n), dtype=torch.float64, pin_memory=True)
        h.copy_(f)
        hf.append(h)
    h2d_bytes = 4 * n ** 3 + 7 * 8 * n ** 3
    with torch.cuda.stream(stream):
        for _ in range(2):
            d_sdf.copy_(h_sdf, non_blocking=True)
            for h, d in zip(hf, d_f):
                d.copy_(h, non_blocking=True)
        e0.record(stream)
        d_sdf.copy_(h_sdf, non_blocking=True)
        for h, d in zip(hf, d_f):
            d.copy_(h, non_blocking=True)
        e1.record(stream)
    e1.synchronize()
    t_h2d = e0.elapsed_time(e1) / 1e3
    sdf_np = sdf.cpu().numpy()
    fields_np = None if args.no_cpu_baseline else [f.cpu().numpy() for f in fields]
    del sdf, fields, d_sdf, d_f
    torch.cuda.empty_cache()
    res = _capi._P(_capi.PnmFlowResult)()

    def call():
        ctx.check(_capi.pnm_extract_network_flow(
            ctx.h, ctypes.c_void_p(h_sdf.data_ptr()), n, n, n, _capi.as_ptr(o), _capi.as_ptr(s),
            *[ctypes.c_void_p(h.data_ptr()) for h in hf], _capi.as_ptr(g), ctypes.byref(res)))

    for _ in range(2):
        call()
        _capi.pnm_flow_result_free(res)
    ts = []
    for _ in range(5):
        t0 = time.perf_counter()
        call()
        ts.append(time.perf_counter() - t0)
        r = res.contents
        npo, nth = int(r.n_pores), int(r.n_throats)
        resid = np.ctypeslib.as_array(r.pore_residual, (npo,)).copy() if npo else np.zeros(0)
        flow = np.ctypeslib.as_array(r.throat_flow, (nth,)).copy() if nth else np.zeros(0)
        _capi.pnm_flow_result_free(res)
    t = float(np.median(ts))
    scale = float(np.abs(flow).sum()) or 1.0
    ctx.close()
    peak, peak_src = measured_hbm_peak()
    achieved = FLOW_BYTES_PER_VOXEL * n ** 3 / t_dev / 1e9
    out = {"workload": "extract_network_flow 256^3 float64 packing (seed 3), 32-mode Fourier "
                       "u,v,w,p (seed 4), openness from face SDF, grad_p_zyx [0,0,-1e-4]",
           "device": {"value": n ** 3 / t_dev / 1e9, "unit": "Gvoxel/s",
                      "ms_per_step": t_dev * 1e3, "h2d_bytes_per_step": 0,
                      "same_counts": dev_counts == (npo, nth),
                      "stage_ms": {k: round(v, 4) for k, v in stage_ms.items() if v > 0}},
           "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                        "frac": achieved / peak, "model_bytes_per_voxel": FLOW_BYTES_PER_VOXEL,
                        "kernel": "extract_network_flow device pipeline (all kernels of one "
                                  "call, SDF and fields resident)",
                        "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)"},
           "e2e": {"value": n ** 3 / t / 1e9, "unit": "Gvoxel/s", "ms_per_step": t * 1e3,
                   "ms_min": min(ts) * 1e3, "h2d_bytes_per_step": h2d_bytes,
                   "d2h_bytes_per_step": 16 * npo + 16 * npo + nth * (8 + 24)},
           "h2d": {"ms": t_h2d * 1e3, "gb_per_s": h2d_bytes / t_h2d / 1e9,
                   "what": "pinned H2D of the SDF and the seven float64 fields alone"},
           "pores": npo, "throats": nth,
           "residual_sum_over_flux": float(abs(resid.sum())) / scale}
    if fields_np is not None:
        from oracle import Oracle

        threads = os.cpu_count() or 1
        t0 = time.perf_counter()
        Oracle("port", threads=threads).extract_network_flow(
            sdf_np, [0.0] * 3, [1.0] * 3, *fields_np[:4], ox=fields_np[4], oy=fields_np[5],
            oz=fields_np[6], grad_p_zyx=[0.0, 0.0, -1e-4])
        t_cpu = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": n ** 3 / t_cpu / 1e9, "unit": "Gvoxel/s",
                               "cores": threads, "kind": "port",
                               "sample": f"the whole 256^3 flow workload, one call ({t_cpu:.1f} s,"
                                         " the project's C++ restatement, OpenMP)"}
    return out


def profile_call(args, dev):
    """Warm-up calls of one leg, then one call inside the NVTX range 'profiled_call' (ncu:
    --nvtx --nvtx-include "profiled_call/"); prints the call's figures."""
    import torch

    import peclet_pnm_gb300 as pnm
    from peclet_pnm_gb300 import _capi

    ctx = pnm.Context(dev.index)
    stream = torch.cuda.current_stream(dev)
    ctx.set_stream(stream.cuda_stream)
    o = np.zeros(3, np.float32)
    s = np.ones(3, np.float32)
    if args.profile == "flow":
        n = 256
        sdf, fields = flow_inputs(dev, n)
        d_sdf = sdf.to(torch.float32).contiguous()
        del sdf
        g = np.array([-1e-4, 0.0, 0.0], np.float64)
        rd = _capi.PnmFlowResultDev()

        def call():
            ctx.check(_capi.pnm_extract_network_flow_dev(
                ctx.h, ctypes.c_void_p(d_sdf.data_ptr()), n, n, n, _capi.as_ptr(o),
                _capi.as_ptr(s), *[ctypes.c_void_p(f.data_ptr()) for f in fields],
                _capi.as_ptr(g), ctypes.byref(rd)))
    else:
        n = args.size
        sdf = gen_volume(n, replica_seed(0), dev)
        d_seg = torch.empty(sdf.numel(), dtype=torch.int32, device=dev)
        d_pores = torch.empty((1_000_000, 4), dtype=torch.float32, device=dev)
        d_pairs = torch.empty((4_000_000, 2), dtype=torch.int32, device=dev)
        npo, npa = _capi._i64(), _capi._i64()

        def call():
            ctx.check(_capi.pnm_extract_pore_network_dev(
                ctx.h, sdf.data_ptr(), n, n, n, _capi.as_ptr(o), _capi.as_ptr(s),
                d_pores.data_ptr(), 1_000_000, ctypes.byref(npo), d_seg.data_ptr(),
                d_pairs.data_ptr(), 4_000_000, ctypes.byref(npa)))
    for _ in range(max(1, args.warmup)):
        call()
    torch.cuda.synchronize(dev)
    l0 = ctx.stats()["launches"]
    torch.cuda.nvtx.range_push("profiled_call")
    call()
    torch.cuda.nvtx.range_pop()
    torch.cuda.synchronize(dev)
    print(json.dumps({"profile": args.profile, "edge": n,
                      "launches": ctx.stats()["launches"] - l0}), flush=True)
    ctx.close()


SERVE_RATES = (200, 500, 1000, 3000)  # Poisson arrival rates of the sweep, requests/s
SERVE_P99_LIMIT_MS = 100.0       # latency limit of the "highest sustainable rate" figure


def served_bench(args, dev):
    """Serving under Poisson arrivals at 200, 500, 1000 and 3000 requests/s (seed 6 + rate). Requests
    are cubic SDFs with edges log-uniform in [32, 384]: 64 distinct request volumes cut at seeded
    offsets from two seeded 384^3 packings (porosity 0.45, seeds 60 and 61), drawn for each
    request by a seeded uniform choice; SDFs sit in pinned host memory. For each rate, two paths:

    * served: the server (continuous batching over concurrent streams, 120 GB budget);
    * plain: one request at a time in arrival order (H2D + pnm_extract_pore_network_dev).

    Latency is measured from the arrival time to (a) results resident on the device and (b) the
    labels, pores and pairs copied back to pinned host memory (the served path copies each result
    out in completion order on one consumer thread). Reported per rate: p50 / p99 of both, the
    delivered Gvoxel/s, and per path the highest rate whose p99 (to the host) stays under
    SERVE_P99_LIMIT_MS. A saturating burst of 200 requests shows the capacity of each path."""
    import threading

    import torch

    import peclet_pnm_gb300 as pnm
    from peclet_pnm_gb300 import _capi
    from peclet_pnm_gb300 import synthetic as syn

    rng = np.random.default_rng(6)
    big = [syn.packing((384, 384, 384), 0.45, seed=60 + k, device=dev) for k in range(2)]
    pool = []
    for i in range(64):
        e = int(round(np.exp(rng.uniform(np.log(32), np.log(384)))))
        src = big[i % 2]
        oz, oy, ox = (int(rng.integers(0, 385 - e)) for _ in range(3))
        h = torch.empty((e, e, e), dtype=torch.float32, pin_memory=True)
        h.copy_(src[oz:oz + e, oy:oy + e, ox:ox + e])
        pool.append(h)
    del big
    torch.cuda.empty_cache()
    n_req = args.serve_requests
    maxn = max(int(r.numel()) for r in pool)
    # pinned host destinations of the results (the largest request's size)
    h_seg = torch.empty(maxn, dtype=torch.int32, pin_memory=True)
    h_pores = torch.empty((1_000_000, 4), dtype=torch.float32, pin_memory=True)
    h_pairs = torch.empty((8_000_000, 2), dtype=torch.int32, pin_memory=True)

    ctx = pnm.Context(dev.index)
    stream = torch.cuda.Stream(dev)
    ctx.set_stream(stream.cuda_stream)
    d_sdf = torch.empty(maxn, dtype=torch.float32, device=dev)
    d_seg = torch.empty(maxn, dtype=torch.int32, device=dev)
    d_pores = torch.empty((1_000_000, 4), dtype=torch.float32, device=dev)
    d_pairs = torch.empty((8_000_000, 2), dtype=torch.int32, device=dev)
    npo, npa = _capi._i64(), _capi._i64()
    o = np.zeros(3, np.float32)
    s = np.ones(3, np.float32)

    def plain_one(h):
        """One request through the plain path; returns (resident, host) completion times."""
        e = h.shape[0]
        with torch.cuda.stream(stream):
            d_sdf[:h.numel()].copy_(h.view(-1), non_blocking=True)
        ctx.check(_capi.pnm_extract_pore_network_dev(
            ctx.h, d_sdf.data_ptr(), e, e, e, _capi.as_ptr(o), _capi.as_ptr(s),
            d_pores.data_ptr(), 1_000_000, ctypes.byref(npo), d_seg.data_ptr(),
            d_pairs.data_ptr(), 8_000_000, ctypes.byref(npa)))
        stream.synchronize()
        t_res = time.perf_counter()
        with torch.cuda.stream(stream):
            h_seg[:h.numel()].copy_(d_seg[:h.numel()], non_blocking=True)
            h_pores[:npo.value].copy_(d_pores[:npo.value], non_blocking=True)
            h_pairs[:npa.value].copy_(d_pairs[:npa.value], non_blocking=True)
        stream.synchronize()
        return t_res, time.perf_counter()

    for h in pool[:8]:
        plain_one(h)
    srv = pnm.Server(max_inflight=2)
    for t in [srv.submit(h) for h in pool[:8]]:
        srv.wait(t)
        srv.release(t)

    def pct(a, q):
        return float(np.percentile(a, q)) if len(a) else None

    def run_plain(arrivals, reqs):
        res, hst = [], []
        t0 = time.perf_counter()
        for j, h in enumerate(reqs):
            wait = arrivals[j] - (time.perf_counter() - t0)
            if wait > 0:
                time.sleep(wait)
            tr, th = plain_one(h)
            res.append(tr - t0 - arrivals[j])
            hst.append(th - t0 - arrivals[j])
        span = time.perf_counter() - t0
        return np.array(res) * 1e3, np.array(hst) * 1e3, span

    def run_served(arrivals, reqs):
        tickets, submitted, hst, errors = [], [], [], []

        def reaper(n):
            k = 0
            while k < n:
                if k >= len(tickets):
                    time.sleep(0.0002)
                    continue
                rc = srv.wait(tickets[k])
                if rc != 0:
                    errors.append(rc)
                else:
                    _capi.pnm_server_copy_out(
                        srv.h, tickets[k], ctypes.c_void_p(h_pores.data_ptr()),
                        ctypes.c_void_p(h_seg.data_ptr()), ctypes.c_void_p(h_pairs.data_ptr()))
                hst.append(time.perf_counter() - t0 - arrivals[k])
                srv.release(tickets[k])
                k += 1

        srv.reset_stats()
        th = threading.Thread(target=reaper, args=(len(reqs),))
        t0 = time.perf_counter()
        th.start()
        for j, h in enumerate(reqs):
            wait = arrivals[j] - (time.perf_counter() - t0)
            if wait > 0:
                time.sleep(wait)
            tickets.append(srv.submit(h))
        th.join()
        span = time.perf_counter() - t0
        if errors:
            raise RuntimeError(f"served requests failed: {errors[:5]}")
        return srv.stats(), np.array(hst) * 1e3, span

    sweep = []
    for rate in SERVE_RATES:
        rr = np.random.default_rng(6 + rate)
        arrivals = np.cumsum(rr.exponential(1.0 / rate, size=n_req))
        reqs = [pool[int(j)] for j in rr.integers(0, len(pool), size=n_req)]
        vox = sum(int(r.numel()) for r in reqs)
        pr, ph, pspan = run_plain(arrivals, reqs)
        sp, sh, sspan = run_served(arrivals, reqs)
        sweep.append({
            "rate_per_s": rate, "requests": n_req, "offered_gvoxel_per_s": vox / arrivals[-1] / 1e9,
            "served": {"p50_ms": sp["p50_ms"], "p99_ms": sp["p99_ms"],
                       "p50_host_ms": pct(sh, 50), "p99_host_ms": pct(sh, 99),
                       "gvoxel_per_s": vox / sspan / 1e9, "batches": int(sp["batches"]),
                       "batch_reuse": int(sp["cache_hits"]),
                       "peak_device_gb": sp["peak_bytes"] / 1e9},
            "plain": {"p50_ms": pct(pr, 50), "p99_ms": pct(pr, 99),
                      "p50_host_ms": pct(ph, 50), "p99_host_ms": pct(ph, 99),
                      "gvoxel_per_s": vox / pspan / 1e9}})
    # saturating burst: 200 requests submitted at once
    reqs = [pool[j % len(pool)] for j in range(200)]
    burst_vox = sum(int(h.numel()) for h in reqs)
    t0 = time.perf_counter()
    for h in reqs:
        plain_one(h)
    plain_burst = burst_vox / (time.perf_counter() - t0) / 1e9
    sb, _, bspan = run_served(np.zeros(len(reqs)), reqs)
    srv.close()
    ctx.close()

    def best_rate(path):
        ok = [r["rate_per_s"] for r in sweep
              if r[path]["p99_host_ms"] is not None and r[path]["p99_host_ms"] <= SERVE_P99_LIMIT_MS]
        return max(ok) if ok else None

    return {
        "workload": f"{n_req} Poisson requests per rate (rates {list(SERVE_RATES)}/s, seed 6 + "
                    "rate), cubic edges log-uniform in [32,384] from 64 volumes cut from two "
                    "seeded 384^3 packings, pinned host SDFs, 120 GB budget",
        "sweep": sweep,
        "p99_limit_ms": SERVE_P99_LIMIT_MS,
        "max_rate_within_limit": {"served": best_rate("served"), "plain": best_rate("plain")},
        "burst_200": {"served_gvoxel_per_s": burst_vox / bspan / 1e9,
                      "served_batches": int(sb["batches"]), "served_p50_ms": sb["p50_ms"],
                      "served_p99_ms": sb["p99_ms"], "plain_gvoxel_per_s": plain_burst},
    }


def ours(args, rank, world, local_rank):
    import torch

    import peclet_pnm_gb300 as pnm
    from peclet_pnm_gb300 import _capi

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    n_edge = args.size
    sdf = gen_volume(n_edge, replica_seed(rank), dev)
    nvox = sdf.numel()
    ctx = pnm.Context(local_rank)
    stream = torch.cuda.current_stream(dev)
    ctx.set_stream(stream.cuda_stream)
    o = np.zeros(3, np.float32)
    s = np.ones(3, np.float32)
    pore_cap = 1_000_000
    d_seg = torch.empty(nvox, dtype=torch.int32, device=dev)
    d_pores = torch.empty((pore_cap, 4), dtype=torch.float32, device=dev)
    npo, npa = _capi._i64(), _capi._i64()
    pair_cap = 1 << 20
    d_pairs = torch.empty((pair_cap, 2), dtype=torch.int32, device=dev)

    def step():
        rc = _capi.pnm_extract_pore_network_dev(
            ctx.h, sdf.data_ptr(), n_edge, n_edge, n_edge, _capi.as_ptr(o), _capi.as_ptr(s),
            d_pores.data_ptr(), pore_cap, ctypes.byref(npo), d_seg.data_ptr(),
            d_pairs.data_ptr(), pair_cap, ctypes.byref(npa))
        ctx.check(rc)

    # size the pair buffer for this volume
    rc = _capi.pnm_extract_pore_network_dev(
        ctx.h, sdf.data_ptr(), n_edge, n_edge, n_edge, _capi.as_ptr(o), _capi.as_ptr(s),
        d_pores.data_ptr(), pore_cap, ctypes.byref(npo), d_seg.data_ptr(), d_pairs.data_ptr(),
        pair_cap, ctypes.byref(npa))
    if rc == _capi.PNM_ERR_CAPACITY:
        pair_cap = int(npa.value * 1.25) + 1024
        d_pairs = torch.empty((pair_cap, 2), dtype=torch.int32, device=dev)
    for _ in range(args.warmup):
        step()
    dist = world > 1
    if dist:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    clocks = ClockSampler(local_rank)
    launches0 = ctx.stats()["launches"]
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize(dev)
    if dist:
        torch.distributed.barrier()
    clk = clocks.stop()
    launches = ctx.stats()["launches"] - launches0
    ms = e0.elapsed_time(e1) / args.steps
    st = ctx.stats()
    # one more call outside the timed region with per-stage device timing on
    ctx.set_timing(True)
    step()
    stage_ms = ctx.stats()["stage_ms"]
    ctx.set_timing(False)
    s_max, value = whole_job_rate(ms * 1e-3, nvox, world, dev)
    ms_max = s_max * 1e3

    # e2e through the host C ABI from pinned memory
    h_sdf = torch.empty(sdf.shape, dtype=torch.float32, pin_memory=True)
    h_sdf.copy_(sdf.cpu())
    h_seg = torch.empty(nvox, dtype=torch.int32, pin_memory=True)
    pp = _capi._P(_capi.PnmPore)()
    pr = _capi._P(ctypes.c_int32)()
    npp, npr = _capi._i64(), _capi._i64()

    def e2e_step():
        ctx.check(_capi.pnm_extract_pore_network(
            ctx.h, ctypes.c_void_p(h_sdf.data_ptr()), n_edge, n_edge, n_edge, _capi.as_ptr(o),
            _capi.as_ptr(s), ctypes.byref(pp), ctypes.byref(npp),
            ctypes.c_void_p(h_seg.data_ptr()), ctypes.byref(pr), ctypes.byref(npr)))
        _capi.pnm_free(ctypes.cast(pp, ctypes.c_void_p))
        _capi.pnm_free(ctypes.cast(pr, ctypes.c_void_p))

    ctx.set_stream(None)
    for _ in range(2):
        e2e_step()
    k_e2e = max(3, min(args.steps, 10))
    if dist:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    e2e_each = []  # per-call times beside the mean (host-link throughput varies between runs)
    for _ in range(k_e2e):
        t1 = time.perf_counter()
        e2e_step()
        e2e_each.append(time.perf_counter() - t1)
    t_e2e = (time.perf_counter() - t0) / k_e2e
    _, e2e_value = whole_job_rate(t_e2e, nvox, world, dev)

    peak, peak_src = measured_hbm_peak()
    achieved = ALG_BYTES_PER_VOXEL * nvox / (ms * 1e-3) / 1e9
    traffic, traffic_commit = profile_traffic()
    result = {
        "metric": METRIC, "value": value, "unit": "Gvoxel/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "config": workload_config(n_edge),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one "
                                       "call, profiles/extract_pore_network_512_launches.txt "
                                       f"(taken at commit {traffic_commit})",
                     "kernel": "extract_pore_network device pipeline (all kernels of one call)",
                     "model_bytes_per_voxel": ALG_BYTES_PER_VOXEL,
                     "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)"},
        "e2e": {"value": e2e_value, "unit": "Gvoxel/s", "ms_per_step": t_e2e * 1e3,
                "ms_min": min(e2e_each) * 1e3,
                "ms_median": float(np.median(e2e_each)) * 1e3,
                "h2d_bytes_per_step": 4 * nvox,
                "d2h_bytes_per_step": 4 * nvox + 16 * int(npp.value) + 8 * int(npr.value)},
        "gpu_launches": launches,
        "stage_ms": {k: round(v, 4) for k, v in stage_ms.items() if v > 0},
        "clocks": clk,
        "outputs": {"pores": int(st["n_pores"]), "pairs": int(st["n_pairs"]),
                    "pore_labels": int(st["n_pore_labels"]),
                    "solid_labels": int(st["n_solid_labels"]),
                    "flood_sweeps": int(st["flood_sweeps"]), "ccl_edges": int(st["ccl_edges"])},
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        e = args.cpu_sample or n_edge
        samp = sdf.cpu().numpy()[:e, :e, :e].copy()
        t_cpu = cpu_sample_run(e, threads, "port", samp)
        what = (f"the whole {e}^3 benchmark volume" if e == n_edge else
                f"{e}^3 corner of the benchmark volume")
        result["cpu_baseline"] = {
            "value": samp.size / t_cpu / 1e9, "unit": "Gvoxel/s", "cores": threads,
            "kind": "port",
            "sample": f"{what}, one extract_pore_network ({t_cpu:.1f} s, the project's C++ "
                      f"restatement of the reference algorithm, OpenMP on {threads} threads)"}
    ctx.close()
    del sdf
    torch.cuda.empty_cache()
    if rank == 0 and world == 1 and not args.no_batched:
        result["batched"] = batched_bench(args, dev)
    if rank == 0 and world == 1 and not args.no_served:
        result["served"] = served_bench(args, dev)
    if rank == 0 and world == 1 and not args.no_flow:
        result["flow"] = flow_bench(args, dev)
    if rank == 0:
        print(json.dumps(result), flush=True)


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        reference_arm(args, rank)
        return
    if args.profile:
        import torch

        torch.cuda.set_device(local_rank)
        profile_call(args, torch.device("cuda", local_rank))
        return
    if world > 1:
        import torch

        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        torch.cuda.set_device(local_rank)
        torch.distributed.init_process_group("nccl")
    try:
        ours(args, rank, world, local_rank)
    finally:
        if world > 1:
            import torch

            torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
