#!/usr/bin/env python
"""Benchmark of the GFAz transform hot path on GB300.

A step is one pass of the path over the chromosome-scale workload: seeded
synthetic graph of the cfg2 shape (90 haplotype P-lines of ~5.7M steps,
~513M int32 steps, ~4.5 GB of P-line text), compressed on the GPU (delta
coding + 8 grammar rounds) and decompressed again (expansion + inverse
delta + P-line text emission).

  value  GB/s of GFA P-line text per (compress + decompress) step, inputs
         resident in HBM, text left in HBM, CUDA events on the library's
         stream; total over all ranks.
  e2e    the same through the C ABI with host buffers: pinned host steps in,
         encoded stream + rulebook out to the host (what the entropy stage
         consumes), loaded back from the host and decoded to pinned host
         text; every copy inside the timed region; three such jobs in flight
         at once (--e2e-jobs), each on its own context and stream.

`--impl reference` times the reference algorithm's CPU implementation on
the host cores (the oracle port: the reference is not built on the GPU
host) on the whole workload, every timed step all 90 P-lines; the port's
speed relative to the reference CLI's own code is recorded in
oracle/calibration.json (made by oracle/calibrate_ref.py) and reported
beside it.

Multi-GPU (torchrun): independent replicas, one per rank (the transform has
no cross-rank exchange); a barrier and the max over ranks bracket the timed
region.
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "GFA GB/s compress+decompress, batched vs plain GPU vs CPU; extract p50/p99 ms"
UNIT = "GB/s"
HBM_FALLBACK = 6800.0


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--scale", type=float, default=1.0, help="fraction of the cfg2 workload (testing)")
    ap.add_argument("--cpu-sample-paths", type=int, default=90,
                    help="P-lines of the CPU port's timed pass (all 90 by default)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--e2e-jobs", type=int, default=3, help="end-to-end jobs in flight at once")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--no-plain", action="store_true", help="skip the one-traversal-per-launch GPU baseline")
    ap.add_argument("--serve-rate", type=float, default=5000.0, help="extract requests per second")
    ap.add_argument("--serve-seconds", type=float, default=1.0)
    ap.add_argument("--serve-sweep", default="100,1000,10000,20000",
                    help="further request rates to report (comma separated; empty for none)")
    return ap.parse_args()


def workload(scale: float):
    from gfaz_gb300 import synthetic
    n_paths = max(2, int(round(90 * min(1.0, scale * 4)))) if scale < 1 else 90
    nseg = int(8_000_000 * scale) if scale < 1 else 8_000_000
    steps, off, nseg = synthetic.cfg2_stream(seed=2, n_segments=max(nseg, 10_000), n_paths=n_paths)
    return steps, off, nseg


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return float(d.get("hbm_gbs", HBM_FALLBACK)), "measured"
    return HBM_FALLBACK, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        """Starts sampling every 50 ms and waits (up to 3 s) for the first
        sample, so that the timed region that follows is covered."""
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            t0 = time.perf_counter()
            while not self.lines and time.perf_counter() - t0 < 3.0:
                time.sleep(0.01)
        except OSError:
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append((time.perf_counter(), ln.strip()))

    def begin(self):
        self.t_begin = time.perf_counter()

    def end(self):
        self.t_end = time.perf_counter()

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        lo, hi = getattr(self, "t_begin", 0.0), getattr(self, "t_end", float("inf"))
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for t, ln in self.lines:
            if not lo <= t <= hi:
                continue
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "samples": len(sm),
                "reasons": sorted(reasons)}


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def run_cpu_port(steps, off, sample_paths, threads, grammar=False):
    """Times the oracle port (reference algorithm on the CPU) on the first
    `sample_paths` traversals; returns (GB/s, seconds, text bytes, sample,
    grammar or None).  With grammar set, the port's encoded stream, offsets
    and rulebook come back too (copied out after its timed phases)."""
    from oracle import oracle
    k = min(sample_paths, len(off) - 1)
    s = steps[:int(off[k])]
    o = off[:k + 1].copy()
    oracle.lib()
    t0 = time.perf_counter()
    r = oracle.roundtrip_p(s, o, 8, 1, threads, grammar=grammar)
    dt = time.perf_counter() - t0
    nbytes = r[0]
    return (nbytes / dt / 1e9, dt, nbytes, f"{k} of {len(off) - 1} P-lines ({int(o[-1])} steps)",
            r[3] if grammar else None)


def _cpu_leg_child(base, sample_paths, threads, q, passes, warmup_paths, grammar):
    """Spawned child of run_cpu_port_isolated: an untimed pass on the first
    warmup_paths traversals (when any), then `passes` timed passes on the
    steps saved at base; the last pass's grammar saved beside them."""
    steps = np.load(base + ".steps.npy")
    off = np.load(base + ".off.npy")
    if warmup_paths:
        run_cpu_port(steps, off, warmup_paths, threads)
    res = []
    for k in range(passes):
        last = grammar and k == passes - 1
        v, dt, nb, sample, gram = run_cpu_port(steps, off, sample_paths, threads, grammar=last)
        if last:
            np.savez(base + ".gram.npz", enc=gram[0], off=gram[1], rules=gram[2])
        res.append((v, dt, nb, sample))
    q.put((res, len(os.sched_getaffinity(0))))


def run_cpu_port_isolated(steps, off, sample_paths, threads, passes=1, warmup_paths=0, grammar=True):
    """run_cpu_port in a freshly spawned process, so that the port's OpenMP
    threads start from a clean process: inside the bench process (after its
    CUDA work, or after the workload generator's numpy calls) the same pass
    ran up to 5x slower.  Returns ([(GB/s, seconds, text bytes, sample) per
    pass], cpus usable, grammar of the last pass or None)."""
    import multiprocessing as mp
    import tempfile
    with tempfile.TemporaryDirectory() as td:
        base = os.path.join(td, "cpu_leg")
        np.save(base + ".steps.npy", steps)
        np.save(base + ".off.npy", off)
        mpc = mp.get_context("spawn")
        q = mpc.Queue()
        p = mpc.Process(target=_cpu_leg_child,
                        args=(base, sample_paths, threads, q, passes, warmup_paths, grammar))
        p.start()
        res, usable = q.get()
        p.join()
        gram = None
        if grammar:
            z = np.load(base + ".gram.npz")
            gram = (z["enc"], z["off"], z["rules"])
    return res, usable, gram


def calibration():
    """The port's time relative to the reference CLI's on the same input
    (oracle/calibration.json), or None."""
    p = os.path.join(ROOT, "oracle", "calibration.json")
    if not os.path.exists(p):
        return None
    with open(p) as fh:
        c = json.load(fh)
    return {"port_over_reference_time": c["ratio_port_over_reference_time"]["total"],
            "compress": c["ratio_port_over_reference_time"]["compress"],
            "decompress": c["ratio_port_over_reference_time"]["decompress"],
            "measured_on": f"{c['input']}, {c['threads']} threads of the build host "
                           "(oracle/calibrate_ref.py against the reference CLI built from its sources)"}


def serving_setup(ctx, seed: int = 5):
    """The serving graph: the config-1 generator on a 600k-segment backbone
    whose 64 P-lines are lognormal windows (median 200k steps) of its
    traversals, compressed into a container.  Config-1 paths are ~22k
    steps, so the longer windows keep the serving config's lengths."""
    import tempfile
    import gfaz_gb300 as gz
    from gfaz_gb300 import synthetic
    steps, off, names, nseg, links = synthetic.serve_paths(seed=seed)
    nt = len(off) - 1
    g = gz.encode(steps, off, rounds=8, delta_round=1, ctx=ctx)
    ptext = g.text(0, nt, names=names, overlaps=["*"] * nt)
    del g
    lines = ptext.split(b"\n")[:-1]
    body = [b"H\tVN:Z:1.1\n", b"".join(b"S\t%d\t*\n" % i for i in range(1, nseg + 1)),
            b"".join(b"L\t%d\t+\t%d\t+\t0M\n" % (a, b) for a, b in links.tolist()), ptext]
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "serve.gfa")
        with open(path, "wb") as fh:
            fh.write(b"".join(body))
        data = gz.compress_file(path)
    return {"data": data, "steps": steps, "off": off, "names": names, "lines": lines}


def serving_run(S, rate: float, duration: float, seed: int = 5, append_every: int = 1000, workers: int = 4,
                trace: list = None) -> dict:
    """Poisson-arriving extract-path requests at `rate` req/s for `duration`
    s against gfaz_gb300.Server holding the serving graph, with an append of
    1-8 new P-lines every `append_every` requests."""
    import queue
    import gfaz_gb300 as gz
    data, names, lines = S["data"], S["names"], S["lines"]
    nt = len(names)
    rng = np.random.default_rng(seed)
    n_req = max(1, int(rate * duration))
    arrivals = np.cumsum(rng.exponential(1.0 / rate, n_req))
    picks = rng.integers(0, nt, n_req)
    lat, qms, sms, bsz, nbytes = [], [], [], [], [0]
    with gz.Server(data, hbm_budget=40 << 30, workers=workers) as srv:
        for n in names:
            srv.wait(srv.submit_path(n))
        q = queue.Queue()

        def waiter():
            while True:
                item = q.get()
                if item is None:
                    return
                kind, k, t = item
                size, ms, q_ms, s_ms, b = srv.wait_detail(t)
                if kind == "x":
                    lat.append(ms)
                    qms.append(q_ms)
                    sms.append(s_ms)
                    bsz.append(b)
                    nbytes[0] += size
                if trace is not None:
                    trace.append((kind, k, float(arrivals[k]), ms, q_ms, s_ms, b))

        th = threading.Thread(target=waiter)
        th.start()
        appended = 0
        t0 = time.perf_counter()
        for k in range(n_req):
            target = t0 + arrivals[k]
            while True:
                d = target - time.perf_counter()
                if d <= 0:
                    break
                if d > 4e-4:
                    time.sleep(d - 3e-4)  # leave the interpreter to the waiter thread
            if append_every and k % append_every == append_every // 2:
                m = int(rng.integers(1, 9))
                new = []
                for j in range(m):
                    src = lines[int(rng.integers(0, len(lines)))].split(b"\t")
                    new.append(b"\t".join([src[0], b"app%d_%d" % (appended, j)] + src[2:]) + b"\n")
                appended += 1
                q.put(("a", k, srv.submit_append(b"".join(new))))
            q.put(("x", k, srv.submit_path(names[int(picks[k])])))
        q.put(None)
        th.join()
        wall = time.perf_counter() - t0
        st = srv.stats()
    return {"rate_req_s": rate, "requests": len(lat), "appends": appended, "seconds": wall,
            "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "queue_p50_ms": float(np.percentile(qms, 50)), "queue_p99_ms": float(np.percentile(qms, 99)),
            "service_p50_ms": float(np.percentile(sms, 50)), "service_p99_ms": float(np.percentile(sms, 99)),
            "mean_batch": float(np.mean(bsz)), "gbps": nbytes[0] / wall / 1e9, "batches": st["batches"],
            "max_batch": st["max_batch"], "workers": workers}


def serving_bench(ctx, rate: float, duration: float, cpu: bool, sweep=(), seed: int = 5) -> dict:
    """Serving (config 5): the headline rate, a sweep of other rates, and
    beside them the same requests one per launch through the non-resident
    extraction API (whole-container decode, like the reference's
    extract-path) and the oracle's CPU expansion + formatting of one path."""
    import gfaz_gb300 as gz
    S = serving_setup(ctx, seed)
    out = serving_run(S, rate, duration, seed)
    out.update({"hbm_budget_gb": 40,
                "graph": "config-1 bubble graph, 600k-segment backbone, 64 P-lines of lognormal length "
                         "(median 200k steps), %d steps" % len(S["steps"])})
    keep = ("rate_req_s", "p50_ms", "p99_ms", "queue_p99_ms", "service_p99_ms", "mean_batch", "gbps")
    out["sweep"] = [{k: v for k, v in serving_run(S, r, duration, seed).items() if k in keep} for r in sweep]
    data, names, off = S["data"], S["names"], S["off"]
    nt = len(names)
    rng = np.random.default_rng(seed + 1)
    plain = []
    for i in rng.integers(0, nt, 10).tolist():
        a = time.perf_counter()
        gz.extract_path_line(data, names[i], ctx=ctx)
        plain.append((time.perf_counter() - a) * 1e3)
    out["plain_gpu"] = {"p50_ms": float(np.percentile(plain, 50)), "requests": len(plain),
                        "form": "one request per launch, whole-container decode (non-resident extract API)"}
    if cpu:
        from oracle import oracle
        enc = oracle.compress(S["steps"], off, 8, 1)
        oo = off.astype(np.uint64)
        cpu_ms = []
        for i in rng.integers(0, nt, 5).tolist():
            a = time.perf_counter()
            e0, e1 = int(enc["enc_offsets"][i]), int(enc["enc_offsets"][i + 1])
            x = oracle.expand(enc["encoded"][e0:e1], np.array([0, e1 - e0], np.uint64), enc["rules_first"],
                              enc["rules_second"], enc["layer_start"], 1,
                              np.array([0, int(oo[i + 1] - oo[i])], np.uint64))
            oracle.format_p(x, np.array([0, len(x)], np.uint64), [names[i]], ["*"])
            cpu_ms.append((time.perf_counter() - a) * 1e3)
        out["cpu"] = {"p50_ms": float(np.percentile(cpu_ms, 50)), "requests": len(cpu_ms), "kind": "port",
                      "form": "oracle expansion + P-line formatting of one path from a preloaded grammar"}
    return out


def reference_arm(args):
    ws, rank, _ = dist_init()
    if rank != 0:
        return 0
    steps, off, _ = workload(args.scale)
    threads = os.cpu_count() or 1
    # in one spawned process: warm-up passes page the port's code and buffers
    # in on a 12-line sample (untimed); every timed step is the whole workload
    warm = min(12, args.cpu_sample_paths) if args.warmup else 0
    res, usable, _ = run_cpu_port_isolated(steps, off, args.cpu_sample_paths, threads, passes=args.steps,
                                           warmup_paths=warm, grammar=False)
    secs = [r[1] for r in res]
    nbytes, sample = res[-1][2], res[-1][3]
    value = nbytes * len(secs) / sum(secs) / 1e9
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(secs) / len(secs),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
           "data": "synthetic (seeded cfg2-shape generator)",
           "config": {"workload": "chromosome-scale cfg2: 90 P-lines, %d steps; the whole workload per timed step"
                                   % len(steps),
                      "rounds": 8, "delta_round": 1, "threshold": 2},
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                            "sample": sample + f" per step, in a spawned process ({usable} CPUs usable); "
                                               "oracle/gfaz_oracle.c (OpenMP), reference CLI not buildable on "
                                               "the GPU host",
                            "calibration": calibration()},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)
    return 0


def e2e_bench(args, steps, off, names, overlaps, ginfo, text_bytes, device, ws):
    """End to end through the C ABI with host buffers.  One job = pinned host
    steps uploaded and compressed (gfz_encode), the encoded stream and rule
    columns copied to pinned host memory (what the entropy stage consumes),
    loaded back from there (gfz_grammar_load) and decoded to P-line text in a
    pinned host buffer (gfz_decode_text; the library stages the text in HBM
    and a copy engine moves it).  args.e2e_jobs jobs are in flight at once,
    each on its own context, CUDA stream and host buffers (host threads; the
    library calls release the interpreter lock), so one job's upload and
    kernels overlap another's text download over the chip-to-chip link.  Every step is one whole job with all of its copies;
    the time is the wall clock from the first job's start to the last one's
    end, with the device synchronised on both sides."""
    import ctypes
    import torch
    import gfaz_gb300 as gz
    from gfaz_gb300._ffi import lib as L, check
    ntrav = len(off) - 1
    offa = np.ascontiguousarray(off, np.uint64)
    h_steps = torch.from_numpy(steps).pin_memory()
    rules_cap = max(1, ginfo["num_rules"] * 2 + 1024)
    jobs = max(1, args.e2e_jobs)

    class Slot:
        def __init__(self):
            # above the lowest priority, which the library gives the text
            # it writes into host memory
            self.stream = torch.cuda.Stream(device=device, priority=-1)
            self.ctx = gz.Context(device, self.stream.cuda_stream)
            self.enc = torch.empty(max(1, int(ginfo["encoded_len"] * 1.5) + 1024), dtype=torch.int32).pin_memory()
            self.f = torch.empty(rules_cap, dtype=torch.int32).pin_memory()
            self.s = torch.empty(rules_cap, dtype=torch.int32).pin_memory()
            self.text = torch.empty(int(text_bytes * 1.1) + 4096, dtype=torch.uint8).pin_memory()

        def run(self):
            ctx = self.ctx
            h = ctypes.c_void_p()
            check(L().gfz_encode(ctx.handle, ctypes.c_void_p(h_steps.data_ptr()), offa.ctypes.data, ntrav, 8, 2, 1,
                                 gz.WHERE_HOST, ctypes.byref(h)))
            g = gz.Grammar(h, ctx)
            info = g.info()
            eoff = np.zeros(ntrav + 1, np.uint64)
            check(L().gfz_grammar_copy(ctx.handle, g.handle, ctypes.c_void_p(self.enc.data_ptr()), eoff.ctypes.data,
                                       None, gz.WHERE_HOST))
            check(L().gfz_grammar_rule_columns(ctx.handle, g.handle, ctypes.c_void_p(self.f.data_ptr()),
                                               ctypes.c_void_p(self.s.data_ptr()), gz.WHERE_HOST))
            del g
            h2 = ctypes.c_void_p()
            check(L().gfz_grammar_load(ctx.handle, ctypes.c_void_p(self.enc.data_ptr()), eoff.ctypes.data, ntrav,
                                       ctypes.c_void_p(self.f.data_ptr()), ctypes.c_void_p(self.s.data_ptr()),
                                       info["num_rules"], info["layer_start"], 1, gz.WHERE_HOST, ctypes.byref(h2)))
            g2 = gz.Grammar(h2, ctx)
            n = g2.decode_text(0, ntrav, names=names, overlaps=overlaps, out_ptr=self.text.data_ptr(),
                               cap=self.text.numel(), where=gz.WHERE_HOST)
            del g2
            return info, n

    slots = [Slot() for _ in range(jobs)]
    for sl in slots:  # warm-up one after the other: each context tunes alone
        for _ in range(max(1, args.warmup // 2)):
            sl.run()
    errors = []

    def worker(j, count, results):
        try:
            for i in range(j, count, jobs):
                results[i] = slots[j].run()
        except Exception as e:  # reported after the join
            errors.append(e)

    def in_flight(count, results):
        ths = [threading.Thread(target=worker, args=(j, count, results)) for j in range(jobs)]
        for t in ths:
            t.start()
        for t in ths:
            t.join()
        if errors:
            raise errors[0]

    # and once all at once: the device memory pool grows to what the jobs
    # hold together now, not inside the timed region
    in_flight(jobs, [None] * jobs)
    k2 = jobs * max(1, -(-args.steps // jobs))  # the timed steps rounded up to whole rounds of the jobs
    results = [None] * k2
    torch.cuda.synchronize()
    w0 = time.perf_counter()
    in_flight(k2, results)
    torch.cuda.synchronize()
    wall = time.perf_counter() - w0
    e2e_ms = wall * 1e3 / k2
    info, n = results[-1]
    heads_ok = all(bytes(sl.text[:64].numpy().tobytes()).startswith(b"P\thap0\t") for sl in slots)
    h2d = 4 * len(steps) + 4 * info["encoded_len"] + 8 * info["num_rules"] + 8 * (ntrav + 1) * 2
    d2h = 4 * info["encoded_len"] + 8 * info["num_rules"] + n
    out = {"value": ws * n / (e2e_ms / 1e3) / 1e9, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
           "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_ms, "jobs_in_flight": jobs, "steps": k2,
           "text_head_ok": heads_ok}
    del slots
    return out


def main():
    args = parse_args()
    if args.impl == "reference":
        return reference_arm(args)
    import torch
    import gfaz_gb300 as gz

    ws, rank, local = dist_init()
    if ws > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    steps, off, nseg = workload(args.scale)
    ntrav = len(off) - 1
    names = [f"hap{i}" for i in range(ntrav)]
    overlaps = ["*"] * ntrav

    stream = torch.cuda.Stream(device=dev)
    ctx = gz.Context(local, stream.cuda_stream)
    d_steps = torch.from_numpy(steps).to(dev)
    torch.cuda.synchronize()

    def step():
        g = gz.encode(None, off, rounds=8, delta_round=1, ctx=ctx, device_ptr=d_steps.data_ptr())
        n = g.decode_text(0, ntrav, names=names, overlaps=overlaps)
        return g, n

    for _ in range(args.warmup):
        g, text_bytes = step()
        del g
    # parity: decode(encode(x)) == x on the device-resident input
    g, text_bytes = step()
    x, xoff = g.decode()
    parity_ok = bool(np.array_equal(xoff, off) and np.array_equal(x, steps))
    ginfo = g.info()
    gpu_grammar = g.arrays() if not args.no_cpu_baseline and rank == 0 else None
    del g, x

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()

    clocks = ClockSampler(local)
    ctx.set_timing(True)
    ctx.kernel_stats(reset=True)
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3 * args.steps)]
    with torch.cuda.stream(stream):
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        clocks.begin()
        t0.record(stream)
        for i in range(args.steps):
            ev[3 * i].record(stream)
            g = gz.encode(None, off, rounds=8, delta_round=1, ctx=ctx, device_ptr=d_steps.data_ptr())
            ev[3 * i + 1].record(stream)
            g.decode_text(0, ntrav, names=names, overlaps=overlaps)
            ev[3 * i + 2].record(stream)
            del g
        t1.record(stream)
    torch.cuda.synchronize()
    clocks.end()
    barrier()
    clk = clocks.stop()
    ms = t0.elapsed_time(t1) / args.steps
    comp_ms = sum(ev[3 * i].elapsed_time(ev[3 * i + 1]) for i in range(args.steps)) / args.steps
    dec_ms = sum(ev[3 * i + 1].elapsed_time(ev[3 * i + 2]) for i in range(args.steps)) / args.steps
    kstats = ctx.kernel_stats(reset=True)
    ctx.set_timing(False)
    launches = int(kstats.pop("_launches", 0)) // max(1, args.steps)
    if ws > 1:
        import torch.distributed as dist
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = ws * text_bytes / (ms / 1e3) / 1e9

    # roofline of the dominant kernel (algorithmic bytes / measured time)
    peak, peak_kind = peaks()
    top = max(kstats.items(), key=lambda kv: kv[1]["ms"])
    kname, kst = top
    achieved = kst["bytes"] / (kst["ms"] / 1e3) / 1e9 if kst["ms"] > 0 else 0.0
    traffic = None
    tp = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if os.path.exists(tp):
        with open(tp) as fh:
            tj = json.load(fh)
        if kname in tj and tj[kname].get("bytes_per_algorithmic_byte"):
            traffic = tj[kname]["bytes_per_algorithmic_byte"] * kst["bytes"] / max(1, kst["launches"])
    kernels = {k: {"ms_per_step": v["ms"] / args.steps, "launches_per_step": v["launches"] / args.steps,
                   "gbps": (v["bytes"] / (v["ms"] / 1e3) / 1e9) if v["ms"] > 0 else None}
               for k, v in sorted(kstats.items(), key=lambda kv: -kv[1]["ms"])}

    cpu = None
    grammar_parity = "not compared"
    grammar_ok = True
    if not args.no_cpu_baseline and rank == 0:
        threads = os.cpu_count() or 1
        res, usable, cpu_grammar = run_cpu_port_isolated(steps, off, args.cpu_sample_paths, threads)
        v, dt, nb, sample = res[-1]
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{sample}, one compress+decompress transform pass in {dt:.2f} s in a spawned process "
                         f"({usable} CPUs usable; oracle/gfaz_oracle.c, OpenMP)", "calibration": calibration()}
        if args.cpu_sample_paths >= ntrav:
            # the GPU grammar of the parity step against the port's, element by element
            grammar_ok = all(np.array_equal(a, b) for a, b in zip(gpu_grammar, cpu_grammar))
            grammar_parity = "identical to the CPU port's" if grammar_ok else "MISMATCH with the CPU port's"

    # end to end through the C ABI with host buffers (after the CPU leg: the
    # jobs' page-locked buffers stay with the process)
    e2e = None
    if not args.no_e2e:
        e2e = e2e_bench(args, steps, off, names, overlaps, ginfo, text_bytes, local, ws)

    # plain GPU form: the same kernels with one traversal per launch sequence
    # (compression encodes each P-line as its own stream, so its rulebooks
    # are per path: a throughput baseline; decompression decodes the shared
    # grammar one path at a time and gives identical text)
    plain = None
    if not args.no_plain:
        with torch.cuda.stream(stream):
            torch.cuda.synchronize()
            c0 = time.perf_counter()
            grams = []
            for t in range(ntrav):
                o = np.array([0, int(off[t + 1] - off[t])], np.uint64)
                grams.append(gz.encode(None, o, rounds=8, delta_round=1, ctx=ctx,
                                       device_ptr=d_steps.data_ptr() + 4 * int(off[t])))
            torch.cuda.synchronize()
            pc = time.perf_counter() - c0
            del grams
            g = gz.encode(None, off, rounds=8, delta_round=1, ctx=ctx, device_ptr=d_steps.data_ptr())
            torch.cuda.synchronize()
            d0 = time.perf_counter()
            pbytes = 0
            for t in range(ntrav):
                pbytes += g.decode_text(t, t + 1, names=names[t:t + 1], overlaps=overlaps[t:t + 1])
            torch.cuda.synchronize()
            pd = time.perf_counter() - d0
            del g
        plain = {"value": ws * text_bytes / (pc + pd) / 1e9, "compress_gbps": ws * text_bytes / pc / 1e9,
                 "decompress_gbps": ws * pbytes / pd / 1e9, "compress_ms": pc * 1e3, "decompress_ms": pd * 1e3,
                 "text_identical_size": pbytes == text_bytes,
                 "form": "one traversal per launch sequence (%d sequences), wall clock" % ntrav}

    extract = None
    if not args.no_serving and rank == 0:
        sweep = [float(x) for x in args.serve_sweep.split(",") if x]
        extract = serving_bench(ctx, args.serve_rate, args.serve_seconds, not args.no_cpu_baseline, sweep)

    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic (seeded cfg2-shape generator; published datasets unavailable)",
        "config": {"workload": "chromosome-scale cfg2: 90 P-lines, %d steps, %d segments" % (len(steps), nseg),
                   "rounds": 8, "delta_round": 1, "threshold": 2, "text_bytes_per_replica": int(text_bytes),
                   "encoded_len": int(ginfo["encoded_len"]), "rules": int(ginfo["num_rules"]),
                   "rounds_done": int(ginfo["rounds_done"]),
                   "l2": "inputs larger than L2 (%.2f GB stream per step)" % (4 * len(steps) / 1e9),
                   "parallelism": "replicas" if ws > 1 else "single GPU"},
        "compress_gbps": ws * text_bytes / (comp_ms / 1e3) / 1e9,
        "decompress_gbps": ws * text_bytes / (dec_ms / 1e3) / 1e9,
        "compress_ms": comp_ms, "decompress_ms": dec_ms,
        "parity": {"roundtrip": "decode(encode(x)) == x: %s" % ("exact" if parity_ok else "MISMATCH"),
                   "grammar": "encoded stream, offsets and rulebook of the whole workload " + grammar_parity},
        "roofline": {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind, "traffic": traffic},
        "kernels": kernels,
        "gpu_launches": launches,
        "clocks": clk,
        "e2e": e2e,
        "cpu_baseline": cpu,
        "plain_gpu": plain,
        "extract": extract,
    }
    if rank == 0:
        print(json.dumps(out), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0 if parity_ok and grammar_ok else 1


if __name__ == "__main__":
    sys.exit(main())
