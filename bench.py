"""Benchmark: frequent patterns per second of the GB300 gSpan miner.

Workload (default): generator configuration 5 -- 1,000,000 graphs, Poisson(40)
edges per graph, 10 Zipf(1.2) vertex labels, 3 edge labels, 200 embedded
seed patterns of 3-8 edges (80 M adjacency entries, about 1 GB, far beyond
the 129 MB L2) -- mined at minsup 0.5% (5000 graphs).  One step = one
complete mining pass at that support (every frequent pattern of the database
enumerated, supports counted, canonicality checked, patterns written to the
host).

value      : patterns / second with the database already resident in HBM
e2e        : same metric through the C ABI from host arrays: the reference's
             cudabin arrays copied to the GPU and converted there
             (gs_db_from_arrays_device), mined, every pattern written to the
             host buffer -- all inside the timed step
roofline   : the count kernel (k_wave count, the dominant kernel): algorithmic
             bytes / kernel time, both measured inside the library on its own
             stream with CUDA events, against the measured HBM peak; the
             materialise and selection kernels beside it
cpu_baseline: the oracle (C restatement of the reference's sequential gSpan) on
             one host core, a time-bounded sample of the same workload
Nested, same line: configuration 2 (100,000 graphs) at minsup 1/2/5%, the
64-database batch (configuration 3) against the same databases mined one at
a time, and the serving streams (configuration 4) with p50/p99 latency.

--impl reference times the reference's CPU implementation -- the oracle port,
since the reference's sources are not present on the GPU host -- on all host
cores (one process per core over disjoint root subtrees), without loading
anything of this package: the oracle generates the same seeded database
itself.

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

ORACLE = os.path.join(REPO, "oracle", "_build", "gspan_oracle")
METRIC = "frequent patterns/sec"
UNIT = "patterns/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--config", type=int, default=5)
    p.add_argument("--scale", type=float, default=1.0)
    p.add_argument("--minsup-frac", type=float, default=None,
                   help="default: 0.5%% for configuration 5, 1%% otherwise")
    p.add_argument("--wave-nodes", type=int, default=None)
    p.add_argument("--launch-mode", type=int, default=0, help="0: per-wave CUDA graphs, 1: direct launches")
    p.add_argument("--extension", default="rmpath", choices=["rmpath", "lists", "auto"],
                   help="extension strategy: rmpath scans every right-most-path vertex (default); lists joins the "
                        "parent's per-row lists (the reference's gspan_cuda_lists); auto joins in waves whose "
                        "databases do not stay in L2")
    p.add_argument("--cpu-seconds", type=float, default=15.0, help="cpu_baseline: the oracle's time bound")
    p.add_argument("--ref-seconds", type=float, default=3.0,
                   help="--impl reference: each step's time bound per process")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-extras", action="store_true",
                   help="the headline workload only (no configuration-2 sweep, batch or serving keys)")
    p.add_argument("--workload", default="mine", choices=["mine", "batch", "serving"],
                   help="mine: one database (the default line); batch: 64 databases mined together vs one at "
                        "a time; serving: Poisson request streams against 8 resident databases")
    p.add_argument("--requests", type=float, default=1.0, help="serving: scale of the request counts")
    a = p.parse_args()
    if a.minsup_frac is None:
        a.minsup_frac = 0.005 if a.config == 5 else 0.01
    return a


def peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def workload_name(config, scale, minsup_frac):
    return "config%d: generator configuration %d x%.3g, minsup %.2f%%" % (config, config, scale, 100 * minsup_frac)


def gen_spec(config, scale, seed=0):
    return "%d,%d,%r" % (config, seed, float(scale))


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


# ---------------------------------------------------------------- reference arm

def ensure_oracle():
    if not os.path.exists(ORACLE):
        subprocess.check_call(["make", "-s", "-C", os.path.join(REPO, "oracle")])


def oracle_intervals(spec, minsup, win, nint, cores):
    """Runs the oracle on a generated database as `cores` processes over
    disjoint root subtrees.  Each builds the root map once (untimed: on
    1,000,000 graphs it is a sort of 40 M root edges, about half a minute),
    then mines for `nint` consecutive windows of `win` seconds, its traversal
    restarting whenever it completes, and reports the patterns found by the
    end of each window.  Consecutive windows sample the whole traversal, deep
    subtrees included, not only its first seconds near the roots.  Returns
    the load lines and the patterns found by all processes in each window."""
    ensure_oracle()
    procs = []
    for i in range(cores):
        cmd = [ORACLE, "gen", spec, str(minsup), "-", "--roots-once", "--intervals", str(nint), str(win)]
        if cores > 1:
            cmd += ["--roots", "%d/%d" % (i, cores)]
        procs.append(subprocess.Popen(cmd, stdout=subprocess.DEVNULL, stderr=subprocess.PIPE, text=True))
    load, cum, passes, roots_s = {}, [0.0] * nint, 0, 0.0
    for k, p in enumerate(procs):
        err = p.communicate()[1]
        if p.returncode != 0:
            raise RuntimeError("oracle failed (%d): %s" % (p.returncode, err[-500:]))
        for line in err.splitlines():
            d = dict(tok.split("=", 1) for tok in line.split() if "=" in tok)
            if "intervals" in d:
                c = [float(x) for x in d["intervals"].split(",")]
                cum = [a + b for a, b in zip(cum, c)]
                passes += int(d.get("passes_completed", "0"))
            if "roots_time" in d:
                roots_s = max(roots_s, float(d["roots_time"]))
            if k == 0 and "load_time" in d:
                load.update(d)
    per = [cum[0]] + [cum[j] - cum[j - 1] for j in range(1, nint)]
    load["passes_completed"] = passes
    load["roots_time"] = roots_s
    return load, per


def config_from_load(a, load, minsup):
    return {"workload": workload_name(a.config, a.scale, a.minsup_frac), "graphs": int(load["graphs"]),
            "vertices": int(load["vertices"]), "adjacency_entries": int(load["adjacency_entries"]),
            "minsup": minsup, "l2": "flushed between steps (256 MiB write)"}


def bench_reference(a):
    """The reference's sequential gSpan (src/gspan/gspan.cpp:281-351, restated
    by the oracle) on all host cores.  Nothing of the GPU package is loaded:
    the oracle generates the seeded database itself (a CPU test checks that it
    is byte for byte the one the GPU arm mines)."""
    if RANK != 0:
        return
    cores = os.cpu_count() or 1
    spec = gen_spec(a.config, a.scale)
    ensure_oracle()
    n_graphs = int(subprocess.check_output([ORACLE, "--gen-count", spec], text=True))
    minsup = max(1, int(round(a.minsup_frac * n_graphs)))
    load, per = oracle_intervals(spec, minsup, a.ref_seconds, a.warmup + a.steps, cores)
    timed = per[a.warmup:]
    v = sum(timed) / (len(timed) * a.ref_seconds)
    ms = 1000.0 * a.ref_seconds
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": 0, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "strong",
            "vs_baseline": None, "dtype": "int32", "data": "synthetic", "config": config_from_load(a, load, minsup),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": "oracle (C restatement of src/gspan, pinned to the reference binary) on the "
                                       "full generated database at minsup %d, one process per core over disjoint "
                                       "root subtrees; each process builds the root map once (%.1f s, untimed), "
                                       "then mines continuously, restarting whenever its traversal completes "
                                       "(%d completions); a step is one %.1f s window of that run (the first %d "
                                       "windows are the warm-up): patterns found by all processes in the window / "
                                       "its length" % (minsup, load["roots_time"], load["passes_completed"],
                                                       a.ref_seconds, a.warmup),
                             "root_map_s": load["roots_time"]},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "patterns_per_step": timed}
    print(json.dumps(line))


# ---------------------------------------------------------------- GPU arm

def count_traffic(tag, alg_bytes_per_step, launches_per_step):
    """DRAM bytes per count-kernel launch from the committed ncu capture of this
    workload (profiles/k_wave_count_traffic_<tag>.json), scaled by this run's
    algorithmic bytes per launch when the capture saw a different amount."""
    path = os.path.join(REPO, "profiles", "k_wave_count_traffic_%s.json" % tag)
    try:
        with open(path) as f:
            p = json.load(f)
    except Exception:
        return None, None
    if launches_per_step <= 0:
        return None, None
    per_launch = alg_bytes_per_step / launches_per_step
    ratio = p["dram_bytes_per_pass"] / p["algorithmic_bytes_per_pass"]
    return ratio * per_launch, ("ncu capture %s (DRAM / algorithmic bytes = %.3f, applied to this run's "
                                "algorithmic bytes per launch): %s" % (os.path.basename(path), ratio, p["command"]))


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


def cpu_oracle_sample(spec, minsup, seconds):
    """cpu_baseline: the oracle on one core for three windows of seconds/3
    (the root map built before them, untimed); the first window is a
    warm-up.  Returns patterns, seconds and the root-map time."""
    load, per = oracle_intervals(spec, minsup, seconds / 3.0, 3, 1)
    return sum(per[1:]), 2.0 * seconds / 3.0, load["roots_time"]


class Timer:
    """Barrier + synchronize on both sides; CUDA events on torch's stream
    bracket the call (the library's own stream work is ordered inside it by
    the call's synchronous return)."""

    def __init__(self, torch, dist, flush):
        self.torch, self.dist, self.flush = torch, dist, flush

    def barrier(self):
        if self.dist:
            self.dist.barrier()
        self.torch.cuda.synchronize()

    def run(self, fn):
        torch = self.torch
        self.flush.fill_(1)
        self.barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        r = fn()
        e1.record()
        self.barrier()
        return r, e0.elapsed_time(e1)


def roofline(stats_all, peak, peak_kind, traffic, traffic_note, serial_stats=None):
    """Achieved GB/s of the count, materialise and selection kernels: their
    algorithmic bytes (counted inside the kernels) / their device time (CUDA
    events on the wave contexts' streams), averaged over the timed steps.
    In the timed steps the contexts' streams overlap: one wave's selection and
    materialise passes share the GPU with another wave's count, so their event
    spans include time spent sharing it.  serial_stats (untimed passes with
    every context on one stream, gs_mine_opts.serial) give each kernel's
    exclusive time: "kernels_one_stream"."""
    n = len(stats_all)

    def avg(k):
        return sum(s[k] for s in stats_all) / n

    def kern(bytes_key, ms_key):
        b, ms = avg(bytes_key), avg(ms_key)
        gbps = (b / (ms / 1000.0)) / 1e9 if ms > 0 else 0.0
        return {"achieved": gbps, "frac": gbps / peak if peak else None, "algorithmic_bytes_per_step": b,
                "kernel_ms_per_step": ms}
    count = kern("count_bytes", "count_ms")
    mat = kern("mat_bytes", "mat_ms")
    sel = kern("sel_bytes", "sel_ms")
    waves = avg("waves")
    return {"bound": "hbm", "kernel": "k_wave count", "achieved": count["achieved"], "peak": peak, "unit": "GB/s",
            "frac": count["frac"], "peak_kind": peak_kind, "traffic": traffic, "traffic_source": traffic_note,
            "algorithmic_bytes_per_step": count["algorithmic_bytes_per_step"],
            "kernel_ms_per_step": count["kernel_ms_per_step"], "launches_per_step": waves,
            "kernels": {"k_wave count": count, "materialise (k_mat_records, k_wave materialise)": mat,
                        "selection (k_screen_keys + k_count_listed)": sel,
                        "k_is_min": {"kernel_ms_per_step": avg("min_ms"), "note": "shared memory only"}},
            "kernels_note": "event spans on overlapping streams (a pass sharing the GPU with another wave's count)",
            "kernels_one_stream": roofline(serial_stats, peak, peak_kind, None, None)["kernels"] if serial_stats
            else None}


def mine_timed(g, tm, db, minsup, steps, warmup, kw):
    for _ in range(warmup):
        g.mine_collect(db, minsup, decode=False, **kw)
    times, stats_all, n = [], [], None
    for _ in range(steps):
        # every pattern lands in a host buffer (gs_mine_collect), freed after timing
        (n, st), ms = tm.run(lambda: g.mine_collect(db, minsup, decode=False, **kw))
        times.append(ms)
        stats_all.append(st)
    return times, stats_all, n


def e2e_timed(g, tm, db, minsup, steps, kw, warmup=3):
    """The reference's set_database(graph_database_cuda&) path: host cudabin
    arrays in, converted and indexed on the GPU, mined, patterns to the host.
    warmup untimed passes first (the first ingest of new host arrays pays for
    their first translations and the ingest pool; a later one in some runs
    too), then steps timed passes."""
    import ctypes
    times, h2d, d2h, ingest = [], 0, 0, []
    with tempfile.TemporaryDirectory() as td:
        n, esz, maxv, vc, arrs = cudabin_arrays(db, td)
        P = ctypes.POINTER(ctypes.c_int32)

        def ptr(x):
            return x.ctypes.data_as(P)

        def step():
            st = ctypes.c_int32(0)
            t0 = time.perf_counter()
            h = g.lib().gs_db_from_arrays_device(n, esz, maxv, vc, ptr(arrs["edges"]), ptr(arrs["edges_labels"]),
                                                 ptr(arrs["vertex_labels"]), ptr(arrs["vertex_offsets"]),
                                                 ctypes.byref(st))
            ingest.append(1e3 * (time.perf_counter() - t0))
            if not h:
                raise RuntimeError(g.lib().gs_last_error().decode())
            d = g.Database(h)
            _, s = g.mine_collect(d, minsup, decode=False, **kw)
            d.free()
            return s
        raw = sum(int(x.nbytes) for x in arrs.values())
        for i in range(warmup + steps):
            s, ms = tm.run(step)
            if i >= warmup:
                times.append(ms)
                # the cudabin arrays uploaded by the ingest, plus the miner's own copies
                h2d, d2h = s["h2d_bytes"] + raw, s["d2h_bytes"]
    # host-timed ingest call (gs_db_from_arrays_device returns with the database ready) per timed step
    return times, h2d, d2h, ingest[warmup:]


def config2_sweep(a, g, tm):
    """Configuration 2 (100,000 graphs) at minsup 1, 2 and 5%: resident
    patterns/s, the three kernels' GB/s at 1%, and end to end at 1%."""
    peak, peak_kind = peaks()
    db = g.Database.generate(2)
    db.upload()
    steps = max(3, min(a.steps, 10))
    out = {"workload": "generator configuration 2 (100,000 graphs)", "graphs": len(db), "steps": steps}
    for frac in (0.01, 0.02, 0.05):
        ms_ = max(1, int(round(frac * len(db))))
        times, stats_all, n = mine_timed(g, tm, db, ms_, steps, 3, {})
        ms = sum(times) / len(times)
        r = {"minsup": ms_, "patterns": n, "ms_per_step": ms, "value": n / (ms / 1000.0)}
        if frac == 0.01:
            cb = sum(s["count_bytes"] for s in stats_all) / len(stats_all)
            w = sum(s["waves"] for s in stats_all) / len(stats_all)
            traffic, note = count_traffic("config2", cb, w)
            r["roofline"] = roofline(stats_all, peak, peak_kind, traffic, note)
            et, h2d, d2h, _ = e2e_timed(g, tm, db, ms_, steps, {}, max(3, a.warmup))
            e = sum(et) / len(et)
            r["e2e"] = {"value": n / (e / 1000.0), "ms_per_step": e, "h2d_bytes_per_step": h2d,
                        "d2h_bytes_per_step": d2h}
        out["minsup_%g%%" % (100 * frac)] = r
    db.free()
    return out


def bench_batch(a, g, tm, steps):
    """64 databases (generator configuration 3, seeds 1000..1063: 1,000-50,000
    graphs log-uniform, 2-20 vertex and edge labels, 10-40 mean edges) at
    minsup 5%: all mined in shared waves by one gs_mine_batch call, against the
    same 64 mined one at a time (batched engine, and the plain one-node-per-
    launch form).  No pattern output in any arm (patterns are counted)."""
    dbs = [g.Database.generate(3, seed=1000 + i, scale=a.scale) for i in range(64)]
    sups = [max(1, int(round(0.05 * len(d)))) for d in dbs]
    for d in dbs:
        d.upload()
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
    for _ in range(steps):
        (_, st_b), ms = tm.run(lambda: g.mine_batch(dbs, sups, collect=False, **tuned))
        tb.append(ms)
        _, ms = tm.run(lambda: g.mine_batch(dbs, sups, collect=False))
        td.append(ms)
        # the lists extension strategy on the same batch and options
        (_, st_l), ms = tm.run(lambda: g.mine_batch(dbs, sups, collect=False, extension="lists", **tuned))
        tl.append(ms)
    clk = clocks.stop()
    pats = st_b["patterns"]
    assert st_l["patterns"] == pats, (st_l["patterns"], pats)

    def one_at_a_time(**kw):
        tot, n = 0.0, 0
        for d, s in zip(dbs, sups):
            (_, st), ms = tm.run(lambda: g.mine(d, s, collect=False, **kw))
            tot += ms
            n += st["patterns"]
        return tot, n
    one_at_a_time()  # warm-up
    t_default, n_solo = one_at_a_time()
    # the same 64 one at a time with the batch's tuned options too: the faster of the two is the comparison
    one_at_a_time(**tuned)
    t_tuned, n_tuned = one_at_a_time(**tuned)
    t_solo = min(t_default, t_tuned)
    t_plain, n_plain = one_at_a_time(wave_nodes=1)
    assert n_solo == pats == n_plain == n_tuned, (n_solo, pats, n_plain, n_tuned)
    ms = sum(tb) / len(tb)
    line = {"metric": "frequent patterns/sec", "value": pats / (ms / 1000.0), "unit": "patterns/s", "n_gpus": 1,
            "steps": steps, "warmup": a.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "strong",
            "vs_baseline": None, "dtype": "int32", "data": "synthetic",
            "config": {"workload": "batch: 64 databases of generator configuration 3 (seeds 1000-1063), minsup 5%, "
                                   "one gs_mine_batch call with autotuned wave options (the batch split over "
                                   "the autotuned number of schedulers, each on its own host thread)",
                       "graphs": sum(len(d) for d in dbs),
                       "l2": "flushed between steps (256 MiB write)"},
            "patterns_per_step": pats,
            "autotuned": {"options": tuned, "report": report, "tuning_s": tune_s,
                          "default_options_ms": sum(td) / len(td)},
            "lists_strategy": {"ms": sum(tl) / len(tl), "patterns_per_s": pats / (sum(tl) / len(tl) / 1000.0),
                               "count_ms": st_l["count_ms"], "mat_ms": st_l["mat_ms"],
                               "list_entries": st_l["list_entries"], "join_nodes": st_l["join_nodes"]},
            "one_at_a_time": {"ms": t_solo, "patterns_per_s": pats / (t_solo / 1000.0),
                              "default_options_ms": t_default, "tuned_options_ms": t_tuned},
            "plain_one_at_a_time": {"ms": t_plain, "patterns_per_s": pats / (t_plain / 1000.0)},
            "speedup_vs_one_at_a_time": t_solo / ms, "speedup_vs_plain": t_plain / ms,
            "clocks": clk, "gpu_launches": int(st_b["launches"]) * steps, "stats_last_step": st_b}
    for d in dbs:
        d.free()
    return line


def bench_serving(a, g, tm):
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
            (_, st), ms = tm.run(lambda: g.mine(dbs[d], s, max_edges=me, collect=False, **kw))
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
    for d in dbs:
        d.free()
    return line


def main():
    a = parse()
    if a.impl == "reference":
        bench_reference(a)
        return
    import gpu_graph_mining_gb300 as g
    if not os.path.exists(g.LIB_PATH):
        from gpu_graph_mining_gb300 import build as b
        b.build()
    import torch
    dist = None
    if WORLD > 1:
        import torch.distributed as dist
        torch.cuda.set_device(0)
        dist.init_process_group("nccl")
    dev = torch.device("cuda:0")
    # written between timed steps: larger than the 129 MB L2
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.int32, device=dev)
    tm = Timer(torch, dist, flush)
    if a.workload != "mine":
        if RANK == 0:
            line = bench_batch(a, g, tm, a.steps) if a.workload == "batch" else bench_serving(a, g, tm)
            print(json.dumps(line))
        return

    db = g.Database.generate(a.config, scale=a.scale)
    minsup = max(1, int(round(a.minsup_frac * len(db))))
    info = db.info()
    config = {"workload": workload_name(a.config, a.scale, a.minsup_frac), "graphs": info["graphs"],
              "vertices": info["vertices"], "adjacency_entries": info["adjacency_entries"], "minsup": minsup,
              "l2": "flushed between steps (256 MiB write)"}
    part = dict(root_part=RANK, root_parts=WORLD) if WORLD > 1 else {}
    kw = dict(part)
    if a.wave_nodes is not None:
        kw["wave_nodes"] = a.wave_nodes
    if a.launch_mode:
        kw["launch_mode"] = a.launch_mode
    if a.extension != "rmpath":
        kw["extension"] = a.extension
        config["extension"] = a.extension
    db.upload()

    # ---- resident-database timing (the warm-up also creates the engine's pool and scratch)
    clocks = Clocks()
    for _ in range(max(3, a.warmup)):
        g.mine_collect(db, minsup, decode=False, **kw)
    clocks.start()
    times, stats_all, pats_local = mine_timed(g, tm, db, minsup, a.steps, 0, kw)
    clk = clocks.stop()
    ms = sum(times) / len(times)
    config_ms_range = [min(times), max(times)]
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
    peak, peak_kind = peaks()
    cb = sum(s["count_bytes"] for s in stats_all) / len(stats_all)
    waves = sum(s["waves"] for s in stats_all) / len(stats_all)
    tag = "config%d" % a.config if a.scale == 1.0 and a.extension == "rmpath" else "none"
    traffic, traffic_note = count_traffic(tag, cb, waves)
    # each kernel's exclusive time: untimed passes with the wave contexts on one stream
    _, serial_stats, _ = mine_timed(g, tm, db, minsup, 2, 1, dict(kw, serial=1))
    roof = roofline(stats_all, peak, peak_kind, traffic, traffic_note, serial_stats)
    launches_per_step = sum(s["launches"] for s in stats_all) / len(stats_all)

    # ---- end to end through the C ABI from host arrays
    e2e_times, h2d, d2h, ingest_ms = e2e_timed(g, tm, db, minsup, a.steps, kw, max(3, a.warmup))
    e2e_ms = sum(e2e_times) / len(e2e_times)
    if dist:
        t = torch.tensor([e2e_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_ms = float(t[0])
    e2e = pats_job / (e2e_ms / 1000.0)

    if RANK != 0:
        dist.destroy_process_group() if dist else None
        return

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": WORLD, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": ms_job, "higher_is_better": True, "scaling": "strong", "vs_baseline": None,
        "dtype": "int32", "data": "synthetic", "config": config,
        "patterns_per_step": pats_job, "ms_per_step_range": config_ms_range,
        "e2e": {"value": e2e, "unit": UNIT, "ms_per_step": e2e_ms, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "steps": len(e2e_times),
                "ms_min": min(e2e_times), "ms_max": max(e2e_times), "ms_steps": e2e_times,
                "ingest_ms_steps": ingest_ms},
        "roofline": roof,
        "cpu_baseline": None,
        "clocks": clk,
        "gpu_launches": int(launches_per_step * a.steps),
        "stats_last_step": stats_all[-1],
    }
    db.free()
    if not a.no_cpu_baseline and WORLD == 1:
        pats, el, roots_s = cpu_oracle_sample(gen_spec(a.config, a.scale), minsup, a.cpu_seconds)
        line["cpu_baseline"] = {
            "value": pats / el if el > 0 else None, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": "oracle (C restatement of src/gspan, pinned to the reference binary) on the full generated "
                      "database at minsup %d, one core: the root map built first (%.1f s, untimed), then mining "
                      "for three windows of %.1f s (the traversal restarting if it completes); patterns of the "
                      "last two windows / their length: %d patterns in %.1f s" %
                      (minsup, roots_s, a.cpu_seconds / 3.0, pats, el),
            "root_map_s": roots_s}
    if not a.no_extras and WORLD == 1 and a.config == 5:
        # the other workloads, each timed the same way (flush, barrier, CUDA events)
        line["config2"] = config2_sweep(a, g, tm)
        nb = max(3, min(a.steps, 5))
        bl = bench_batch(a, g, tm, nb)
        line["batch"] = {k: bl[k] for k in ("value", "ms_per_step", "steps", "patterns_per_step", "config",
                                            "autotuned", "lists_strategy", "one_at_a_time", "plain_one_at_a_time",
                                            "speedup_vs_one_at_a_time", "speedup_vs_plain", "clocks")}
        sl = bench_serving(a, g, tm)
        line["serving"] = {k: sl[k] for k in ("value", "config", "streams", "serial_plain_at_200",
                                              "serial_batched_at_200", "server", "clocks")}
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
