"""Benchmark: frequent patterns per second of the GB300 gSpan miner.

Workload (default): generator configuration 2 -- 100,000 graphs, Poisson(30)
edges per graph, 5 vertex / 5 edge labels, 50 embedded seed patterns --
mined at minsup 1% (1000 graphs).  One step = one complete mining pass at
that support (every frequent pattern of the database enumerated, supports
counted, canonicality checked, patterns emitted to the host).

value      : patterns / second with the database already resident in HBM
e2e        : same metric through the C ABI from host arrays: the reference's
             cudabin arrays copied to the GPU and converted there
             (gs_db_from_arrays_device), mined, every pattern written to the
             host buffer -- all inside the timed step
roofline   : the count kernel (k_wave_count, the dominant kernel): algorithmic
             bytes per launch / kernel time, both measured inside the library on
             its own stream with CUDA events, against the measured HBM peak
cpu_baseline: the oracle (C restatement of the reference's sequential gSpan) on
             one host core, time-bounded sample of the same workload

--impl reference times the reference's CPU implementation (the oracle port,
since the reference's own sources are not present on the GPU host) on all host
cores, one process per core over disjoint root subtrees, time-bounded.

Multi-GPU (torchrun, N > 1): every rank mines a disjoint set of root subtrees
of the same database (no data exchange); the step time is the max over ranks.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

WORLD = int(os.environ.get("WORLD_SIZE", "1"))
RANK = int(os.environ.get("RANK", "0"))
LOCAL_RANK = int(os.environ.get("LOCAL_RANK", "0"))
if WORLD > 1:
    # one GPU per rank: the native library sees only this rank's device
    os.environ["CUDA_VISIBLE_DEVICES"] = str(LOCAL_RANK)

L2_BYTES = 129 * 1024 * 1024


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--config", type=int, default=2)
    p.add_argument("--scale", type=float, default=1.0)
    p.add_argument("--minsup-frac", type=float, default=0.01)
    p.add_argument("--wave-nodes", type=int, default=None)
    p.add_argument("--launch-mode", type=int, default=0, help="0: per-wave CUDA graphs, 1: direct launches")
    p.add_argument("--extension", default="rmpath", choices=["rmpath", "lists"],
                   help="extension strategy: rmpath scans every right-most-path vertex (default); lists joins "
                        "the parent's per-row lists (the reference's gspan_cuda_lists)")
    p.add_argument("--cpu-seconds", type=float, default=15.0)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--workload", default="mine", choices=["mine", "batch", "serving"],
                   help="mine: one database (the default line); batch: 64 databases mined together vs one at "
                        "a time; serving: Poisson request streams against 8 resident databases")
    p.add_argument("--requests", type=float, default=1.0, help="serving: scale of the request counts")
    return p.parse_args()


def peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """Samples nvidia-smi SM clocks and throttle reasons while running."""

    def __init__(self):
        self.samples = []
        self.proc = None
        self.max_mhz = None

    def start(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        idx = os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0] if WORLD > 1 else "0"
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", idx, "--query-gpu=" + q, "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 7:
                self.samples.append(parts)

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.t.join(timeout=2)
        mhz, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in self.samples:
            try:
                mhz.append(float(s[0]))
                mx = float(s[1])
            except ValueError:
                continue
            for n, v in zip(names, s[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        mhz.sort()
        med = mhz[len(mhz) // 2] if mhz else None
        return {"sm_mhz": med, "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(mhz)}


def count_traffic(a, alg_bytes_per_step, launches_per_step):
    """DRAM bytes per count-kernel launch from the committed ncu capture
    (profiles/k_wave_count_traffic_config2.json): as captured for the same
    workload, else scaled by this run's algorithmic bytes per launch."""
    try:
        with open(os.path.join(REPO, "profiles", "k_wave_count_traffic_config2.json")) as f:
            p = json.load(f)
    except Exception:
        return None, None
    if launches_per_step <= 0:
        return None, None
    per_launch = alg_bytes_per_step / launches_per_step
    if a.config == 2 and a.scale == 1.0 and abs(a.minsup_frac - 0.01) < 1e-12:
        return float(p["dram_bytes_per_launch"]), "ncu capture of this workload: " + p["command"]
    ratio = p["dram_bytes_per_pass"] / p["algorithmic_bytes_per_pass"]
    return ratio * per_launch, ("scaled from the configuration-2 capture by algorithmic bytes per launch "
                                "(traffic/algorithmic = %.3f)" % ratio)


def cudabin_arrays(db, tmpdir):
    """The reference's flat cudabin arrays of a database (host memory)."""
    import numpy as np
    p = os.path.join(tmpdir, "db.cudabin")
    db.write(p, "cudabin")
    raw = np.fromfile(p, dtype=np.int32)
    os.remove(p)
    n, esz, maxv, vc = (int(x) for x in raw[:4])
    o = 4
    arrs = {}
    arrs["edges"] = raw[o:o + esz].copy(); o += esz
    arrs["edges_labels"] = raw[o:o + esz].copy(); o += esz
    arrs["vertex_labels"] = raw[o:o + n * maxv].copy(); o += n * maxv
    arrs["vertex_offsets"] = raw[o:o + n * maxv + 1].copy()
    return n, esz, maxv, vc, arrs


def run_oracle_sample(db_txt, minsup, seconds, part=None):
    oracle = os.path.join(REPO, "oracle", "_build", "gspan_oracle")
    if not os.path.exists(oracle):
        subprocess.check_call(["make", "-s", "-C", os.path.join(REPO, "oracle")])
    cmd = [oracle, "txt", db_txt, str(minsup), "-", "--time-limit", str(seconds)]
    if part is not None:
        cmd += ["--roots", "%d/%d" % part]
    return subprocess.Popen(cmd, stdout=subprocess.DEVNULL, stderr=subprocess.PIPE, text=True)


def parse_oracle(stderr):
    d = {}
    for tok in stderr.split():
        if "=" in tok:
            k, v = tok.split("=", 1)
            d[k] = v
    return float(d.get("total_time", "nan")), int(float(d.get("total_frequent_graphs", "0"))), "stopped" in d


def cpu_oracle(db_txt, minsup, seconds, cores):
    t0 = time.time()
    procs = [run_oracle_sample(db_txt, minsup, seconds, (i, cores) if cores > 1 else None) for i in range(cores)]
    res = [parse_oracle(p.communicate()[1]) for p in procs]
    wall = time.time() - t0
    elapsed = max(r[0] for r in res)
    pats = sum(r[1] for r in res)
    stopped = any(r[2] for r in res)
    return pats, elapsed, stopped, wall


def _timed(fn):
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    r = fn()
    torch.cuda.synchronize()
    return r, (time.perf_counter() - t0) * 1000.0


def bench_batch(a, g):
    """64 databases (generator configuration 3, seeds 1000..1063: 1,000-50,000
    graphs log-uniform, 2-20 vertex and edge labels, 10-40 mean edges) at
    minsup 5%: all mined in shared waves by one gs_mine_batch call, against the
    same 64 mined one at a time (batched engine, and the plain one-node-per-
    launch form).  No pattern output in any arm (patterns are counted)."""
    import torch
    dbs = [g.Database.generate(3, seed=1000 + i, scale=a.scale) for i in range(64)]
    sups = [max(1, int(round(0.05 * len(d)))) for d in dbs]
    for d in dbs:
        d.upload()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.int32, device="cuda:0")
    for _ in range(max(3, a.warmup)):
        g.mine_batch(dbs, sups, collect=False)
    # untimed: the autotuner picks the wave options for this workload
    t0 = time.perf_counter()
    tuned, report = g.autotune(dbs, sups)
    tune_s = time.perf_counter() - t0
    for _ in range(2):
        g.mine_batch(dbs, sups, collect=False, **tuned)
        g.mine_batch(dbs, sups, collect=False, extension="lists", **tuned)
    clocks = Clocks()
    clocks.start()
    tb, st_b, td, tl = [], None, [], []
    for _ in range(a.steps):
        flush.fill_(1)
        (_, st_b), ms = _timed(lambda: g.mine_batch(dbs, sups, collect=False, **tuned))
        tb.append(ms)
        flush.fill_(1)
        _, ms = _timed(lambda: g.mine_batch(dbs, sups, collect=False))
        td.append(ms)
        # the lists extension strategy on the same batch and options
        flush.fill_(1)
        (_, st_l), ms = _timed(lambda: g.mine_batch(dbs, sups, collect=False, extension="lists", **tuned))
        tl.append(ms)
    clk = clocks.stop()
    pats = st_b["patterns"]
    assert st_l["patterns"] == pats, (st_l["patterns"], pats)

    def one_at_a_time(**kw):
        tot, n = 0.0, 0
        for d, s in zip(dbs, sups):
            flush.fill_(1)
            (_, st), ms = _timed(lambda: g.mine(d, s, collect=False, **kw))
            tot += ms
            n += st["patterns"]
        return tot, n
    one_at_a_time()  # warm-up
    t_solo, n_solo = one_at_a_time()
    t_plain, n_plain = one_at_a_time(wave_nodes=1)
    assert n_solo == pats == n_plain, (n_solo, pats, n_plain)
    ms = sum(tb) / len(tb)
    line = {"metric": "frequent patterns/sec", "value": pats / (ms / 1000.0), "unit": "patterns/s", "n_gpus": 1,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "strong",
            "vs_baseline": None, "dtype": "int32", "data": "synthetic",
            "config": {"workload": "batch: 64 databases of generator configuration 3 (seeds 1000-1063), minsup 5%, "
                                   "one gs_mine_batch call with autotuned wave options",
                       "graphs": sum(len(d) for d in dbs),
                       "l2": "flushed between steps (256 MiB write)"},
            "patterns_per_step": pats,
            "autotuned": {"options": tuned, "report": report, "tuning_s": tune_s,
                          "default_options_ms": sum(td) / len(td)},
            "lists_strategy": {"ms": sum(tl) / len(tl), "patterns_per_s": pats / (sum(tl) / len(tl) / 1000.0),
                               "count_ms": st_l["count_ms"], "mat_ms": st_l["mat_ms"],
                               "list_entries": st_l["list_entries"], "join_nodes": st_l["join_nodes"]},
            "one_at_a_time": {"ms": t_solo, "patterns_per_s": pats / (t_solo / 1000.0)},
            "plain_one_at_a_time": {"ms": t_plain, "patterns_per_s": pats / (t_plain / 1000.0)},
            "speedup_vs_one_at_a_time": t_solo / ms, "speedup_vs_plain": t_plain / ms,
            "clocks": clk, "gpu_launches": int(st_b["launches"]) * a.steps, "stats_last_step": st_b}
    print(json.dumps(line))


def bench_serving(a, g):
    """8 resident databases (generator configuration 4, seeds 2000..2007:
    10,000-200,000 graphs); Poisson request streams at 5, 20, 50 and 200
    requests/s (seed 7), each request = (database uniform, minsup uniform from
    1/2/5/10%, max pattern edges uniform 4..8).  Latency = submission to
    completion; throughput = patterns of the stream / (first submission to
    last completion).  The same requests are then mined serially, one at a
    time, by the plain one-node-per-launch form and by the batched engine."""
    import random
    dbs = [g.Database.generate(4, seed=2000 + i, scale=a.scale) for i in range(8)]
    for d in dbs:
        d.upload()
    rng = random.Random(7)
    plan = [(5, 30), (20, 60), (50, 100), (200, 200)]
    out = {}
    with g.Server(max_active=64) as srv:
        ids = [srv.add_db(d) for d in dbs]
        # warm-up with the largest request shape (minsup 1%, 8 edges): every
        # kernel variant and CUDA graph the streams use is loaded and built, and
        # the pool has grown, before the timed streams
        for i in range(8):
            srv.result(srv.submit(ids[i], max(1, int(round(0.01 * len(dbs[i])))), 8), decode=False)
        clocks = Clocks()
        clocks.start()
        last_reqs = None
        for lam, n in plan:
            n = max(4, int(n * a.requests))
            reqs = []
            for _ in range(n):
                d = rng.randrange(8)
                reqs.append((d, max(1, int(round(rng.choice([0.01, 0.02, 0.05, 0.10]) * len(dbs[d])))),
                             rng.randint(4, 8)))
            gaps = [rng.expovariate(lam) for _ in range(n)]
            t0 = time.perf_counter()
            t, rids = t0, []
            for (d, s, me), gap in zip(reqs, gaps):
                t += gap
                now = time.perf_counter()
                if t > now:
                    time.sleep(t - now)
                rids.append(srv.submit(ids[d], s, me))
            infos = [srv.result(r, decode=False)[1] for r in rids]
            wall = time.perf_counter() - t0
            lat = sorted(i["latency_ms"] for i in infos)
            rank = lambda q: lat[max(1, int(-(-q * len(lat) // 1))) - 1]  # noqa: E731 nearest rank
            pats = sum(i["patterns"] for i in infos)
            out[str(lam)] = {"requests": n, "p50_ms": rank(0.5), "p99_ms": rank(0.99),
                             "mean_ms": sum(lat) / len(lat), "patterns": pats, "wall_s": wall,
                             "patterns_per_s": pats / wall, "offered_s": t - t0}
            last_reqs = reqs
        clk = clocks.stop()
        sst = srv.stats()

    def serial(**kw):
        tot, n = 0.0, 0
        for d, s, me in last_reqs:
            (_, st), ms = _timed(lambda: g.mine(dbs[d], s, max_edges=me, collect=False, **kw))
            tot += ms
            n += st["patterns"]
        return tot, n
    serial()  # warm-up
    t_b, n_b = serial()
    t_p, n_p = serial(wave_nodes=1)
    top = out[str(plan[-1][0])]
    assert n_b == n_p == top["patterns"], (n_b, n_p, top["patterns"])
    line = {"metric": "frequent patterns/sec (served)", "value": top["patterns_per_s"], "unit": "patterns/s",
            "n_gpus": 1, "higher_is_better": True, "scaling": "strong", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic",
            "config": {"workload": "serving: 8 databases of generator configuration 4 (seeds 2000-2007), Poisson "
                                   "arrivals (seed 7), minsup 1/2/5/10%, max edges 4-8; value at 200 req/s",
                       "graphs": [len(d) for d in dbs]},
            "streams": out,
            "serial_plain_at_200": {"ms": t_p, "patterns_per_s": n_p / (t_p / 1000.0)},
            "serial_batched_at_200": {"ms": t_b, "patterns_per_s": n_b / (t_b / 1000.0)},
            "server": {"max_running": sst["max_running"], "completed": sst["completed"], "waves": sst["waves"],
                       "peak_pool_bytes": sst["peak_pool_bytes"]},
            "clocks": clk}
    print(json.dumps(line))


def main():
    a = parse()
    import gpu_graph_mining_gb300 as g
    if not os.path.exists(g.LIB_PATH):
        from gpu_graph_mining_gb300 import build as b
        b.build()
    if a.workload != "mine" and a.impl == "gb300":
        if RANK == 0:
            (bench_batch if a.workload == "batch" else bench_serving)(a, g)
        return

    workload = "config%d: generator configuration %d x%.3g, minsup %.2f%%" % (a.config, a.config, a.scale,
                                                                             100 * a.minsup_frac)
    metric = "frequent patterns/sec"
    unit = "patterns/s"
    db = g.Database.generate(a.config, scale=a.scale)
    minsup = max(1, int(round(a.minsup_frac * len(db))))
    info = db.info()
    config = {"workload": workload, "graphs": info["graphs"], "vertices": info["vertices"],
              "adjacency_entries": info["adjacency_entries"], "minsup": minsup,
              "l2": "flushed between steps (256 MiB write)"}

    if a.impl == "reference":
        if RANK != 0:
            return
        cores = os.cpu_count() or 1
        with tempfile.TemporaryDirectory() as td:
            p = os.path.join(td, "db.txt")
            db.write(p, "txt")
            for _ in range(a.warmup):  # short warm-up samples (page cache, CPU clocks)
                cpu_oracle(p, minsup, 1.0, cores)
            vals = []
            t_all = 0.0
            for _ in range(a.steps):
                pats, el, stopped, wall = cpu_oracle(p, minsup, a.cpu_seconds, cores)
                vals.append(pats / el if el > 0 else 0.0)
                t_all += el
        v = sum(vals) / len(vals)
        line = {"impl": "reference", "metric": metric, "value": v, "unit": unit, "n_gpus": 0, "steps": a.steps,
                "warmup": a.warmup, "ms_per_step": 1000 * t_all / a.steps, "higher_is_better": True,
                "scaling": "strong", "vs_baseline": None, "dtype": "int32", "data": "synthetic", "config": config,
                "cpu_baseline": {"value": v, "unit": unit, "cores": cores, "kind": "port",
                                 "sample": "oracle (C restatement of src/gspan) on the full database at the same "
                                           "minsup, one process per core over disjoint root subtrees, each stopped "
                                           "after %.0f s; patterns found / elapsed" % a.cpu_seconds},
                "e2e": {"value": v, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    import torch
    dist = None
    if WORLD > 1:
        import torch.distributed as dist
        torch.cuda.set_device(0)
        dist.init_process_group("nccl")
    dev = torch.device("cuda:0")
    flush_buf = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.int32, device=dev)

    def barrier():
        if dist:
            dist.barrier()
        torch.cuda.synchronize()

    part = dict(root_part=RANK, root_parts=WORLD) if WORLD > 1 else {}
    db.upload()
    kw = dict(part)
    if a.wave_nodes is not None:
        kw["wave_nodes"] = a.wave_nodes
    if a.launch_mode:
        kw["launch_mode"] = a.launch_mode
    if a.extension != "rmpath":
        kw["extension"] = a.extension
        config["extension"] = a.extension
    # warm-up (also creates the engine's pool and scratch)
    for _ in range(max(3, a.warmup)):
        g.mine_collect(db, minsup, decode=False, **kw)

    # ---- resident-database timing
    clocks = Clocks()
    clocks.start()
    times, stats_all = [], []
    n_patterns = None
    for _ in range(a.steps):
        flush_buf.fill_(1)
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        # every pattern lands in a host buffer (gs_mine_collect), freed after timing
        n_patterns, st = g.mine_collect(db, minsup, decode=False, **kw)
        e1.record()
        barrier()
        times.append(e0.elapsed_time(e1))
        stats_all.append(st)
    clk = clocks.stop()
    ms = sum(times) / len(times)
    pats_local = n_patterns
    if dist:
        t = torch.tensor([ms, float(pats_local)], device=dev)
        mx = t.clone()
        dist.all_reduce(mx, op=dist.ReduceOp.MAX)
        sm = t.clone()
        dist.all_reduce(sm, op=dist.ReduceOp.SUM)
        ms_job, pats_job = float(mx[0]), int(sm[1])
    else:
        ms_job, pats_job = ms, pats_local
    value = pats_job / (ms_job / 1000.0)

    # roofline of the count kernel (mean over timed steps)
    cb = sum(s["count_bytes"] for s in stats_all) / len(stats_all)
    cms = sum(s["count_ms"] for s in stats_all) / len(stats_all)
    mb = sum(s["mat_bytes"] for s in stats_all) / len(stats_all)
    mms = sum(s["mat_ms"] for s in stats_all) / len(stats_all)
    peak, peak_kind = peaks()
    waves = sum(s["waves"] for s in stats_all) / len(stats_all)
    count_gbps = (cb / (cms / 1000.0)) / 1e9 if cms > 0 else 0.0
    mat_gbps = (mb / (mms / 1000.0)) / 1e9 if mms > 0 else 0.0
    # the dominant kernel is the one with more device time per step
    if mms > cms:
        dom, achieved, dom_bytes, dom_ms, other = "k_wave materialise", mat_gbps, mb, mms, ("k_wave count", count_gbps)
    else:
        dom, achieved, dom_bytes, dom_ms, other = "k_wave count", count_gbps, cb, cms, ("k_wave materialise", mat_gbps)
    launches_per_step = sum(s["launches"] for s in stats_all) / len(stats_all)
    traffic, traffic_note = count_traffic(a, cb, waves) if dom == "k_wave count" else (None, None)

    # ---- end-to-end through the C ABI from host arrays
    e2e_times, h2d, d2h = [], 0, 0
    with tempfile.TemporaryDirectory() as td:
        n, esz, maxv, vc, arrs = cudabin_arrays(db, td)
        import ctypes
        import numpy as np
        P = ctypes.POINTER(ctypes.c_int32)

        def ptr(x):
            return x.ctypes.data_as(P)
        for i in range(a.steps + 1):
            flush_buf.fill_(1)
            barrier()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            st = ctypes.c_int32(0)
            # the reference's set_database(graph_database_cuda&) path: host arrays in,
            # converted and indexed on the GPU
            h = g.lib().gs_db_from_arrays_device(n, esz, maxv, vc, ptr(arrs["edges"]), ptr(arrs["edges_labels"]),
                                                 ptr(arrs["vertex_labels"]), ptr(arrs["vertex_offsets"]),
                                                 ctypes.byref(st))
            if not h:
                raise RuntimeError(g.lib().gs_last_error().decode())
            d = g.Database(h)
            _, s = g.mine_collect(d, minsup, decode=False, **kw)
            d.free()
            e1.record()
            barrier()
            if i > 0:  # the first pass is a warm-up
                e2e_times.append(e0.elapsed_time(e1))
                # the cudabin arrays uploaded by the ingest, plus the miner's own copies
                raw = sum(int(x.nbytes) for x in arrs.values())
                h2d, d2h = s["h2d_bytes"] + raw, s["d2h_bytes"]
    e2e_ms = sum(e2e_times) / len(e2e_times)
    if dist:
        t = torch.tensor([e2e_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_ms = float(t[0])
    e2e = pats_job / (e2e_ms / 1000.0)

    if RANK != 0:
        dist.destroy_process_group() if dist else None
        return

    cpu = None
    if not a.no_cpu_baseline and WORLD == 1:
        with tempfile.TemporaryDirectory() as td:
            p = os.path.join(td, "db.txt")
            db.write(p, "txt")
            pats, el, stopped, _ = cpu_oracle(p, minsup, a.cpu_seconds, 1)
        cpu = {"value": pats / el if el > 0 else None, "unit": unit, "cores": 1, "kind": "port",
               "sample": "oracle (C restatement of src/gspan, pinned to the reference) on the full database at "
                         "minsup %d, %s after %.1f s: %d patterns" % (minsup, "stopped" if stopped else "finished",
                                                                      el, pats)}

    line = {
        "metric": metric, "value": value, "unit": unit, "n_gpus": WORLD, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": ms_job, "higher_is_better": True, "scaling": "strong", "vs_baseline": None,
        "dtype": "int32", "data": "synthetic", "config": config,
        "patterns_per_step": pats_job,
        "e2e": {"value": e2e, "unit": unit, "ms_per_step": e2e_ms, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak if peak else None, "peak_kind": peak_kind, "traffic": traffic,
                     "traffic_source": traffic_note,
                     "algorithmic_bytes_per_step": dom_bytes, "kernel_ms_per_step": dom_ms,
                     "launches_per_step": waves, "other_kernel": {"kernel": other[0], "achieved": other[1]}},
        "cpu_baseline": cpu,
        "clocks": clk,
        "gpu_launches": int(launches_per_step * a.steps),
        "stats_last_step": stats_all[-1],
    }
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
