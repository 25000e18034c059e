#!/usr/bin/env python
"""Throughput of the TNMMAP decoder on a GB300: rotated surface code d=7,
code-capacity depolarising noise p=0.05 (X, Y, Z each p/3), batches of
65,536 seeded syndromes.

One step = decoding one batch: the float32 contraction of every syndrome
plus the float64 recheck of low-margin syndromes (and, when a surrogate
checkpoint is given, the gated surrogate in front of them).  ``value`` times
the decode with syndromes already in HBM; ``e2e`` times the same call through
the C ABI with pinned host buffers, copies included.  ``--impl reference``
times the CPU restatement of the reference's per-syndrome float64
contraction on the host cores instead.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "d=7 syndromes/s: gated surrogate+batched TN vs plain TN, ≤1e-4 decision diff"
D, P, BATCH = 7, 0.05, 65536
SEED = 0x7E5A0001


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--batch", type=int, default=BATCH)
    ap.add_argument("--cpu-sample", type=int, default=12000)
    ap.add_argument("--profile", action="store_true",
                    help="one float32 contraction launch of --batch syndromes (for ncu), no timing")
    ap.add_argument("--no-autotune", action="store_true")
    return ap.parse_args()


def workload(pkg, rank, nbatches, batch):
    t = pkg.tanner_graph(pkg.SurfaceCode(D, D))
    em = pkg.depolarizing(P, t.nq)
    rng = np.random.default_rng(SEED + rank)
    bits = []
    for _ in range(nbatches):
        ep = pkg.random_error_pattern(em, rng, nsamples=batch)
        s = pkg.syndrome_extraction(ep, t)
        bits.append(np.concatenate([s.sx, s.sz], axis=1))
    return t, em, bits


def config(batch):
    return {"workload": f"rotated surface code d={D} (49 data qubits, 48 checks), code-capacity depolarizing "
                        f"p={P} (X/Y/Z p/3 each), {batch} seeded syndromes per step",
            "batch": batch, "code": f"SurfaceCode({D},{D})", "p": P,
            "l2": "256 MB buffer written between timed steps (inputs are smaller than L2)",
            "parallelism": "replicas (independent syndromes per GPU)"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = os.path.join(ROOT, "gpurun_out", f"clocks_rank{gpu_index}.csv")

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def read_traffic():
    """Per-launch DRAM bytes of the dominant kernel from the committed ncu
    summary (profiles/roofline_traffic.txt: 'key value' lines)."""
    path = os.path.join(ROOT, "profiles", "roofline_traffic.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        parts = line.split()
        if len(parts) >= 2 and parts[0] == f"tn_contract_f32_d{D}_bytes_per_launch_{BATCH}":
            return float(parts[1])
    return None


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            m = json.load(f)
        return m.get("bf16_tflops"), m.get("hbm_gbs"), "measured"
    return 1900.0, 6800.0, "fallback"


def cpu_baseline(pkg, ct, bits, sample):
    """The oracle's float64 per-syndrome contraction on all host cores."""
    from oracle.c_oracle import CContractor, max_threads

    g = ct.graph
    cc = CContractor(g.ixs, [np.asarray(x) for x in g.tensors], g.iy, g.syndrome_positions, ct.steps)
    sub = bits[:sample]
    packed = pkg.pack_syndromes(sub)
    cc.contract(packed[:64])
    t0 = time.perf_counter()
    marg, cls = cc.contract(packed)
    dt = time.perf_counter() - t0
    return {"value": len(sub) / dt, "unit": "syndromes/s", "cores": max_threads(), "kind": "port",
            "sample": f"{len(sub)} syndromes of the same workload, float64 tree contraction per syndrome "
                      f"(CPU restatement of TNMMAP; the reference Julia package is not runnable here)",
            "seconds": dt}, cls


def run_reference(args):
    import __graft_entry__ as G

    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    pkg = G.load_package()
    from oracle.c_oracle import CContractor, max_threads

    t, em, bits = workload(pkg, 0, 1, max(args.cpu_sample, 256))
    lx, lz = pkg.logical_operator(t)
    g = pkg.tnmmap_css_graph(t, em, lx, lz)
    steps = pkg.optimize_code(g, pkg.TreeSA())
    cc = CContractor(g.ixs, [np.asarray(x) for x in g.tensors], g.iy, g.syndrome_positions, steps)
    per = max(64, args.cpu_sample // max(args.steps, 1))
    packed = pkg.pack_syndromes(bits[0])
    for w in range(args.warmup):
        cc.contract(packed[:min(per, 256)])
    times = []
    for s in range(args.steps):
        lo = (s * per) % max(len(packed) - per, 1)
        t0 = time.perf_counter()
        cc.contract(packed[lo:lo + per])
        times.append(time.perf_counter() - t0)
    total = sum(times)
    value = per * args.steps / total
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "syndromes/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded depolarizing errors)", "config": dict(config(per), batch=per),
            "cpu_baseline": {"value": value, "unit": "syndromes/s", "cores": max_threads(), "kind": "port",
                             "sample": f"{per} syndromes per step, float64 per-syndrome tree contraction "
                                       f"(CPU restatement; Julia/OMEinsum not runnable here)"},
            "e2e": {"value": value, "unit": "syndromes/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch

    import __graft_entry__ as G

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    pkg = G.load_package()
    W, K, B = args.warmup, args.steps, args.batch
    t, em, bits = workload(pkg, rank, W + K, B)
    ct = pkg.compile(pkg.TNMMAP(precision="f32", device=local), t, em)
    if not args.no_autotune:
        ct.program.autotune(16384)
    info = ct.program.info
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream
    packed = [pkg.pack_syndromes(b) for b in bits]
    d_syn = [torch.from_numpy(p).cuda() for p in packed]
    d_cls = torch.empty(B, dtype=torch.int32, device="cuda")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def flush_l2():
        flush.fill_(1.0)

    # warm-up (also the first-call allocations inside the library)
    for i in range(W):
        ct.program.decode_ptrs(d_syn[i].data_ptr(), B, d_cls.data_ptr(), None, None, sptr)
    torch.cuda.synchronize()

    # ---- value: device-resident decode ------------------------------------
    clocks = ClockSampler(local)
    clocks.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    rechecks = 0
    for i in range(K):
        flush_l2()
        ev[i][0].record(stream)
        ct.program.decode_ptrs(d_syn[W + i].data_ptr(), B, d_cls.data_ptr(), None, None, sptr)
        ev[i][1].record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clk = clocks.stop()
    ms = [a.elapsed_time(b) for a, b in ev]
    step_ms = sum(ms) / K
    rechecks = ct.program.last_recheck_count()

    # ---- roofline: the float32 contraction kernel alone --------------------
    d_lp = torch.empty((B, info["n_classes"]), dtype=torch.float64, device="cuda")
    kms = []
    for i in range(min(K, 5)):
        flush_l2()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        ct.program.contract_ptrs(d_syn[W + i].data_ptr(), B, pkg.native.TQEC_F32, d_lp.data_ptr(), sptr)
        b.record(stream)
        torch.cuda.synchronize()
        kms.append(a.elapsed_time(b))
    kernel_ms = statistics.median(kms)
    flops = info["flops_per_syndrome"]
    achieved_tflops = flops * B / (kernel_ms / 1e3) / 1e12
    bf16_peak, hbm_peak, peak_kind = peaks()

    # ---- e2e: pinned host in, pinned host out, through the C ABI -----------
    h_syn = [torch.from_numpy(p).pin_memory() for p in packed]
    h_cls = torch.empty(B, dtype=torch.int32).pin_memory()
    ct.program.decode_ptrs(h_syn[0].data_ptr(), B, h_cls.data_ptr(), None, None, sptr)
    torch.cuda.synchronize()
    e2e_ms = []
    for i in range(K):
        flush_l2()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        ct.program.decode_ptrs(h_syn[W + i].data_ptr(), B, h_cls.data_ptr(), None, None, sptr)
        b.record(stream)
        torch.cuda.synchronize()
        e2e_ms.append(a.elapsed_time(b))
    e2e_step = sum(e2e_ms) / K

    # ---- plain float64 form: one launch per syndrome (drop-in baseline) ----
    plain = pkg.compile(pkg.TNMMAP(precision="f64", plain=True, device=local), t, em)
    m = 128
    plain.program.decode_ptrs(d_syn[0].data_ptr(), 8, d_cls.data_ptr(), None, None, sptr)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    plain.program.decode_ptrs(d_syn[0].data_ptr(), m, d_cls.data_ptr(), None, None, sptr)
    b.record(stream)
    torch.cuda.synchronize()
    plain_rate = m / (a.elapsed_time(b) / 1e3)
    plain.close()

    # max over ranks
    if dist:
        tt = torch.tensor([step_ms, e2e_step], dtype=torch.float64, device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        step_ms, e2e_step = tt.tolist()
    value = world * B / (step_ms / 1e3)
    e2e_value = world * B / (e2e_step / 1e3)

    line = None
    if rank == 0:
        cpu, cpu_cls = cpu_baseline(pkg, ct, bits[W], args.cpu_sample)
        gpu_cls = ct.decode_batch(bits[W][:args.cpu_sample])
        mismatch = float(np.mean(gpu_cls != cpu_cls))
        traffic = read_traffic()
        line = {
            "metric": METRIC, "value": value, "unit": "syndromes/s", "n_gpus": world, "steps": K, "warmup": W,
            "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded depolarizing errors, numpy PCG64)", "config": config(B),
            "e2e": {"value": e2e_value, "unit": "syndromes/s", "h2d_bytes_per_step": int(packed[0].nbytes),
                    "d2h_bytes_per_step": int(B * 4)},
            "roofline": {"bound": "tensor", "achieved": achieved_tflops, "peak": bf16_peak, "unit": "TFLOP/s",
                         "frac": achieved_tflops / bf16_peak, "traffic": traffic,
                         "kernel": "tn_contract_kernel<float> (SIMT float32; peak is the measured bf16 "
                                   f"tensor rate, {peak_kind})",
                         "flops_per_syndrome": flops, "kernel_ms": kernel_ms},
            "cpu_baseline": cpu,
            "clocks": clk,
            "gpu_launches": 2 * K,
            "plain_f64_gpu_syn_per_s": plain_rate,
            "speedup_vs_plain_f64_gpu": value / plain_rate,
            "decision_mismatch_vs_f64_oracle": mismatch,
            "recheck_fraction": rechecks / B,
        }
        print(json.dumps(line), flush=True)
    ct.close()
    if dist:
        dist.barrier()
        dist.destroy_process_group()


def run_profile(args):
    """W warm-up launches then one float32 contraction launch of the d=7
    workload: the case the ncu captures profile."""
    import torch

    import __graft_entry__ as G

    pkg = G.load_package()
    t, em, bits = workload(pkg, 0, 1, args.batch)
    ct = pkg.compile(pkg.TNMMAP(precision="f32"), t, em)
    d_syn = torch.from_numpy(pkg.pack_syndromes(bits[0])).cuda()
    d_lp = torch.empty((args.batch, ct.n_classes), dtype=torch.float64, device="cuda")
    sptr = torch.cuda.current_stream().cuda_stream
    for _ in range(args.warmup + 1):
        ct.program.contract_ptrs(d_syn.data_ptr(), args.batch, pkg.native.TQEC_F32, d_lp.data_ptr(), sptr)
    torch.cuda.synchronize()
    print(json.dumps({"profile_case": config(args.batch), "program": ct.program.info}), flush=True)
    ct.close()


def main():
    args = parse()
    if args.profile:
        run_profile(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
