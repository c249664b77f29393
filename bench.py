"""Benchmark: MaxCut QAOA <Z_i Z_j> terms/s on one GB300.

Workload (the reference's QAOA objective, src/maxcut.cpp:162-204): a seeded
random 4-regular graph with 30 vertices (60 edges), QAOA depth p=1, every edge
term's light-cone circuit as src/maxcut.h:105-233 writes it, contracted under
this build's line-graph (min-fill) ordering.  One step evaluates all 60 terms
at one (gamma, beta) point.

  value      mixed-precision terms/s with the inputs resident in HBM (one grouped
             launch per step, per-step CUDA events on the launching stream, L2
             flushed between steps)
  e2e        the same through the public API with host buffers: every step hands
             the rotation angles of a new (gamma, beta) point to the batch (one
             pinned H2D copy of the angles; the gate tensors are built on the
             device), runs, and reads the 60 values back
  fp64       the plain complex128 path (bit-exact with the reference) for the
             mixed/FP64 ratio; error = |mixed - fp64| per term
  batched    64 (gamma, beta) points x every edge term of 16 random 3-regular
             graphs (20-40 vertices, p = 1 and 2) in one grouped launch per step,
             mixed vs FP64
  serving    Poisson arrivals of QAOA / random-circuit / QFT requests through the
             continuous-batching server under a 150 GB budget: p50/p99 latency
  cpu_baseline / --impl reference: the CPU oracle port (a C restatement of the
             reference's ContractIndices loop, QASM parse included per term, as
             the reference pays it) on the host cores

python bench.py [--gpus N --steps K --warmup W] [--impl reference]
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "QAOA <ZZ> terms/s (mixed vs FP64 GPU, err<=1e-6); serve p50/p99 latency"
NODES, DEGREE, P = 30, 4, 1
WORKLOAD = "MaxCut QAOA p=1, seeded random 4-regular graph, 30 nodes, 60 edge terms, line-graph (min-fill) ordering"
L2_FLUSH_BYTES = 256 << 20


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(values, world, device):
    """Element-wise max of per-rank timings (the slowest rank sets the job time)."""
    if world <= 1:
        return list(values)
    import torch
    import torch.distributed as dist
    t = torch.tensor(list(values), dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.tolist()


def angle_points(seed, n):
    rng = np.random.default_rng(seed)
    return [list(rng.uniform(0.0, math.pi, 2)) for _ in range(n)]   # [beta, gamma], U[0, pi)


def term_rotation_angles(qasm_text):
    """Angles of the rotation gates of a term in node order, as the parser reads them."""
    out = []
    for line in qasm_text.split("\n"):
        t = line.split(" ")
        if t and t[0] in ("Rx", "Rz"):
            out.append(float(t[1]))
    return out


def build_terms(dgf, point):
    import qtorch_gb300 as qg
    n = qg.qaoa_num_edges(dgf)
    return [qg.qaoa_term_text(dgf, P, point, e) for e in range(n)]


# ---------------------------------------------------------------------------
# CPU side (oracle port): the checker / baseline, never the product

def _cpu_worker(job):
    """One term on the oracle port: (value, parse seconds, contraction seconds)."""
    from oracle import port
    qasm, meas, seq = job
    t0 = time.perf_counter()
    net = port.Net(qasm, meas)
    t1 = time.perf_counter()
    net.replay(seq)
    return net.final_value, t1 - t0, time.perf_counter() - t1


def cpu_terms_per_s(jobs, workers, min_seconds=0.0):
    """Oracle port over (qasm, measure, sequence) jobs on `workers` processes
    (spawn): (terms/s, terms, seconds, share of the workers' time spent parsing)."""
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    parse_s = contract_s = 0.0
    with ctx.Pool(workers) as pool:
        pool.map(_cpu_worker, jobs[:workers])          # warm the workers
        done, t0 = 0, time.perf_counter()
        while True:
            for _, tp, tc in pool.map(_cpu_worker, jobs):
                parse_s += tp
                contract_s += tc
            done += len(jobs)
            el = time.perf_counter() - t0
            if el >= min_seconds:
                break
    return done / el, done, el, parse_s / max(parse_s + contract_s, 1e-30)


def sequences_for(terms):
    """Line-graph orderings of the terms (computed by the host planner, no GPU)."""
    import qtorch_gb300 as qg
    return [qg.Plan(q, m, ordering="linegraph", symbolic=True).sequence() for q, m in terms]


# ---------------------------------------------------------------------------

class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled during the timed region."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.rows = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index),
                 "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap", "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
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
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[0]))
                mx = float(r[1])
                for n, v in zip(names, r[3:7]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return d["hbm_gbs"], "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


# sources whose change invalidates an ncu capture of the grouped interpreter:
# the kernel and the plan block it reads
KERNEL_SOURCES = ["kernels.cu", "engine.cuh", "plan.cpp", "plan.h"]


def kernel_source_hash():
    import hashlib
    h = hashlib.sha256()
    for name in KERNEL_SOURCES:
        with open(os.path.join(HERE, "qtorch_gb300", "csrc", name), "rb") as f:
            h.update(f.read())
    return h.hexdigest()[:16]


def profiled_traffic():
    """Per-launch DRAM bytes of the grouped kernel from the committed ncu
    summary, only when that capture was taken of the current kernel sources
    (its 'kernel_sources_sha16' line); (bytes or None, note)."""
    path = os.path.join(HERE, "profiles", "plan_kernel_mixed_qaoa_p1_30node.txt")
    fields = {}
    try:
        with open(path) as f:
            for line in f:
                if "=" in line:
                    k, v = line.split("=", 1)
                    fields[k.strip()] = v.strip()
    except OSError:
        return None, "no ncu summary"
    if fields.get("kernel_sources_sha16") != kernel_source_hash():
        return None, "the committed ncu capture predates the current kernel sources"
    try:
        return float(fields["dram_bytes_per_launch"].split()[0]), "ncu capture of the current kernel sources"
    except (KeyError, ValueError, IndexError):
        return None, "no DRAM figure in the ncu summary"


def time_steps(run, steps, warmup, stream, flush):
    """Per-step CUDA events on the launching stream; L2 flushed between steps.
    The timed steps sit in an NVTX range "timed" (for ncu --nvtx-include)."""
    import torch
    for _ in range(warmup):
        run()
    torch.cuda.synchronize()
    with torch.cuda.nvtx.range("timed"):
        times = timed_loop(run, steps, stream, flush)
    torch.cuda.synchronize()
    return times


def timed_loop(run, steps, stream, flush):
    import torch
    times = []
    for _ in range(steps):
        flush()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        run()
        e.record(stream)
        e.synchronize()
        times.append(s.elapsed_time(e) / 1e3)
    return times


def term_layer_shape(qasm_text, p):
    """(edges per layer, qubits) of a light-cone term: rotations come as
    [Rz(-gamma_i) x E, Rx(2 beta_i) x n] for i = 1..p (src/maxcut.h:205-233)."""
    n = int(qasm_text.split("\n", 1)[0])
    n_rz = sum(1 for line in qasm_text.split("\n") if line.startswith("Rz "))
    return n_rz // p, n


def rotation_vector(shapes, point, p):
    """Rotation angles of every term at one point, as the parser reads the reference's text."""
    betas, gammas = point[:p], point[p:]
    out = []
    for e, n in shapes:
        for i in range(p):
            out += [float("%g" % -gammas[i])] * e + [float("%g" % (betas[i] * 2.0))] * n
    return out


def run_batched(ctx, args, stream, flush):
    """Config 4: 64 seeded (gamma, beta) points x all edge terms of 16 random
    3-regular graphs with 20-40 vertices, p = 1 or 2, in one grouped launch."""
    import qtorch_gb300 as qg
    rng = np.random.default_rng(4242)
    graphs = []
    for g in range(16):
        n = int(rng.integers(10, 21)) * 2
        p = 1 + (g % 2)
        graphs.append((qg.random_regular_graph(n, 3, seed=100 + g), p))
    n_points = args.batched_points
    plans, shapes, ps = [], [], []
    for dgf, p in graphs:
        pt0 = [0.3] * p + [0.7] * p
        for e in range(qg.qaoa_num_edges(dgf)):
            q, m = qg.qaoa_term_text(dgf, p, pt0, e)
            plans.append(qg.Plan(q, m, ordering="linegraph", ctx=ctx))
            shapes.append(term_layer_shape(q, p))
            ps.append(p)
    points = [list(rng.uniform(0.0, math.pi, 4)) for _ in range(n_points)]   # beta1, beta2, gamma1, gamma2
    angles = []
    for pt in points:
        for sh, p in zip(shapes, ps):
            angles += rotation_vector([sh], pt[:p] + pt[2:2 + p], p)
    res = {}
    for prec in (qg.MIXED, qg.FP64):
        b = qg.Batch(ctx)
        for _ in points:
            for pl in plans:
                b.add(pl)
        b.set_rotations(np.array(angles))
        b.prepare(prec)
        b.use_graph(True)
        policy = b.autotune()[0] if args.autotune else b.launch_policy
        vals = b.execute(prec)
        t = time_steps(b.run, args.batched_steps, 3, stream, flush)
        res[prec] = (vals, sum(t) / len(t), len(b), b.launches_per_run, policy, b.launch_info())
        b._release()
    n_inst = res[qg.MIXED][2]
    err = np.abs(res[qg.MIXED][0] - res[qg.FP64][0])
    mixed_rate = n_inst / res[qg.MIXED][1]
    fp64_rate = n_inst / res[qg.FP64][1]
    return {"workload": "64 seeded (gamma,beta) points x all edge terms of 16 random 3-regular graphs, "
                        "20-40 vertices, p=1 (8 graphs) and p=2 (8 graphs), one grouped launch per step",
            "terms_per_step": n_inst, "distinct_plans": len(plans), "mixed_terms_per_s": mixed_rate,
            "fp64_terms_per_s": fp64_rate, "mixed_over_fp64": mixed_rate / fp64_rate,
            "mixed_ms_per_step": 1e3 * res[qg.MIXED][1], "fp64_ms_per_step": 1e3 * res[qg.FP64][1],
            "error_vs_fp64": {"max_abs": float(err.max()), "mean_abs": float(err.mean())},
            "launches_per_step": res[qg.MIXED][3],
            "launch_policy": {"autotuned": bool(args.autotune), "mixed": res[qg.MIXED][4],
                              "fp64": res[qg.FP64][4],
                              "mixed_grid": res[qg.MIXED][5]["grid"],
                              "mixed_smem_bytes": res[qg.MIXED][5]["smem_bytes"]}}


SERVE_BUDGET = 150 << 30
# Work cap of one request: ~2-3 s of the GPU at the ~1e13 complex MAC/s the
# large steps run at.  Requests above it are refused at submission.
SERVE_MAX_MACS = int(3e13)
# Distinct requests whose FP64 value is computed for the error bound (FP64 runs
# at ~4e10 complex MAC/s on this part: ~2.5 s at the limit)
SERVE_FP64_CHECK_MACS = int(1e11)
SERVE_RAND_QUBITS = (10, 14, 18, 22, 26, 30)
SERVE_RAND_DEPTHS = (8, 12, 16, 20)
SERVE_QFT_QUBITS = tuple(range(8, 25, 2))


SERVE_QUEUED = {}   # per class: seconds each request of the last serve() waited before admission


def zipf(n, a=1.2):
    w = np.array([(i + 1.0) ** -a for i in range(n)])
    return w / w.sum()


def run_serving(args):
    """Config 5: Poisson arrivals of contraction requests against a 150 GB
    device-memory budget.  The mix: QAOA edge terms (p=1 and p=2), random
    Rx/Ry/Rz + CZ circuits of 10-30 qubits and depth 8-20, QFT circuits of 8-24
    qubits on a random basis input; within each class the sizes are drawn from
    a Zipf distribution (exponent 1.2) over the class's circuits ordered by
    complex MACs, so the largest are rare but present.  Every circuit is
    planned with the automatic ordering; one whose largest intermediate is
    beyond the engine (more than 24 wires) is refused at planning, one above
    the work cap at submission, and both are counted."""
    import qtorch_gb300 as qg
    from qtorch_gb300.circuits import qft_measure_text, qft_text, random_circuit_text
    ctx = qg.Context(0)
    ctx.set_memory_budget(SERVE_BUDGET)
    qaoa = []
    dgf = qg.random_regular_graph(NODES, DEGREE, seed=args.graph_seed)
    for e in range(qg.qaoa_num_edges(dgf)):
        q, m = qg.qaoa_term_text(dgf, 1, [0.4, 1.1], e)
        qaoa.append(qg.Plan(q, m, ordering="linegraph", ctx=ctx))
    dgf2 = qg.random_regular_graph(30, 3, seed=5)
    for e in range(0, qg.qaoa_num_edges(dgf2), 3):
        q, m = qg.qaoa_term_text(dgf2, 2, [0.3, 0.8, 0.6, 0.2], e)
        qaoa.append(qg.Plan(q, m, ordering="linegraph", ctx=ctx))
    t_plan = time.perf_counter()
    plan_s = []

    def build(name, text, meas):
        """(name, plan or None, macs): None when planning refuses it"""
        t0 = time.perf_counter()
        try:
            p = qg.Plan(text, meas, ordering="auto", ctx=ctx)
            out = (name, p, p.flops)
        except qg.InvalidFunctionInput:
            out = (name, None, float("inf"))
        plan_s.append(time.perf_counter() - t0)
        return out

    rand = [build(f"rand{n}x{d}", random_circuit_text(n, d, 7 + i), "Z")
            for i, (n, d) in enumerate((n, d) for n in SERVE_RAND_QUBITS for d in SERVE_RAND_DEPTHS)]
    qft = [build(f"qft{n}", qft_text(n, 3 + i), qft_measure_text(n)) for i, n in enumerate(SERVE_QFT_QUBITS)]
    t_plan = time.perf_counter() - t_plan
    rand.sort(key=lambda r: r[2])
    qft.sort(key=lambda r: r[2])
    # FP64 value of every distinct request up to the check size: the error bound
    ref = {}
    for p in qaoa + [r[1] for r in rand + qft if r[1] is not None and r[2] <= SERVE_FP64_CHECK_MACS]:
        ref[id(p)] = p.execute(qg.FP64)
    rng = np.random.default_rng(2024)
    p_rand, p_qft = zipf(len(rand)), zipf(len(qft))
    reqs = []   # (class, name, plan or None)
    for _ in range(args.serve_requests):
        u = rng.uniform()
        if u < 0.80:
            reqs.append(("qaoa", "qaoa", qaoa[int(rng.integers(len(qaoa)))]))
        elif u < 0.92:
            r = rand[int(rng.choice(len(rand), p=p_rand))]
            reqs.append(("random", r[0], r[1]))
        else:
            r = qft[int(rng.choice(len(qft), p=p_qft))]
            reqs.append(("qft", r[0], r[1]))

    # one server for both phases: the saturation phase also warms its lanes'
    # device and pinned-memory caches and the plans' device blocks
    srv = qg.Server(max_inflight=256, precision=qg.MIXED, ctx=ctx, max_macs=SERVE_MAX_MACS)
    classes = ("qaoa", "random", "qft")

    def serve(gaps):
        """Submit every request at its arrival time (gaps None: all at once);
        latencies by class, wall time, max error against FP64, refusals."""
        tickets = []
        refused = {k: {} for k in classes}
        t0 = time.perf_counter()
        t_next = t0
        for k, (cls, name, plan) in enumerate(reqs):
            if gaps is not None:
                t_next += gaps[k]
                while True:
                    now = time.perf_counter()
                    if now >= t_next:
                        break
                    time.sleep(min(t_next - now, 0.0005))
            if plan is None:
                refused[cls][name] = refused[cls].get(name, 0) + 1   # beyond the engine at planning
                tickets.append(None)
                continue
            try:
                tickets.append(srv.submit(plan))
            except (qg.Refused, qg.OutOfMemory):
                refused[cls][name] = refused[cls].get(name, 0) + 1
                tickets.append(None)
        srv.drain()
        wall = time.perf_counter() - t0
        lat = {k: [] for k in classes}
        queued = {k: [] for k in classes}
        err = {k: 0.0 for k in classes}
        checked = {k: 0 for k in classes}
        served_names = {k: set() for k in classes}
        for (cls, name, plan), t in zip(reqs, tickets):
            if t is None:
                continue
            try:
                v, l, qd, _ = srv.poll_detail(t)
            except qg.QtError as e:
                raise RuntimeError(f"request {name} failed: {e}; {ctx.last_error}") from e
            lat[cls].append(l)
            queued[cls].append(qd)
            served_names[cls].add(name)
            if id(plan) in ref:
                err[cls] = max(err[cls], abs(v - ref[id(plan)]))
                checked[cls] += 1
        SERVE_QUEUED.clear()
        SERVE_QUEUED.update(queued)
        return lat, wall, err, checked, refused, served_names

    def pct(xs, f):
        xs = sorted(xs)
        return 1e3 * xs[min(len(xs) - 1, max(0, int(math.ceil(f * len(xs))) - 1))] if xs else None

    # saturation: everything at once gives the server's throughput on this mix;
    # the measured stream then offers a stated fraction of it as Poisson arrivals
    _, wall_sat, err_sat, _, _, _ = serve(None)
    n_served = sum(1 for r in reqs if r[2] is not None and r[2].flops <= SERVE_MAX_MACS)
    capacity = n_served / wall_sat
    rate = args.serve_rate if args.serve_rate > 0 else args.serve_load * capacity
    gaps = rng.exponential(1.0 / rate, len(reqs))
    st0 = srv.stats()
    lat, wall, err, checked, refused, served_names = serve(gaps)
    st1 = srv.stats()
    srv.close()
    waves = st1["waves"] - st0["waves"]
    wave_reqs = st1["wave_requests"] - st0["wave_requests"]
    wave_s = st1["lane_seconds"] - st0["lane_seconds"]
    all_lat = [x for v in lat.values() for x in v]
    largest = {cls: max((r for r in pool if r[0] in served_names[cls]), key=lambda r: r[2], default=None)
               for cls, pool in (("random", rand), ("qft", qft))}
    out = {
        "workload": f"{len(reqs)} requests, Poisson arrivals at {rate:.0f}/s ({rate / capacity:.2f} of the "
                    f"saturation throughput): 80% QAOA edge terms (30-vertex 4-regular p=1, 30-vertex 3-regular "
                    f"p=2), 12% random Rx/Ry/Rz+CZ circuits of {SERVE_RAND_QUBITS} qubits x depth "
                    f"{SERVE_RAND_DEPTHS}, 8% QFT of {SERVE_QFT_QUBITS} qubits on a random basis input; sizes "
                    "Zipf(1.2) over each class's circuits ordered by complex MACs; <Z_0> measured (<X> of the "
                    "last qubit for QFT); automatic ordering (greedy or min-fill), plans built before the stream "
                    "(requests carry a plan); refused: beyond 24-wire intermediates at planning, above the work "
                    "cap at submission",
        "precision": "mixed", "memory_budget_bytes": SERVE_BUDGET, "work_cap_complex_macs": SERVE_MAX_MACS,
        "planning_s": {"total": t_plan, "max": max(plan_s), "circuits": len(plan_s)},
        "saturation_requests_per_s": capacity, "arrival_rate_per_s": rate,
        "p50_ms": pct(all_lat, 0.50), "p99_ms": pct(all_lat, 0.99),
        "p50_ms_by_class": {k: pct(v, 0.50) for k, v in lat.items()},
        "p99_ms_by_class": {k: pct(v, 0.99) for k, v in lat.items()},
        "queued_p50_ms_by_class": {k: pct(v, 0.50) for k, v in SERVE_QUEUED.items()},
        "queued_p99_ms_by_class": {k: pct(v, 0.99) for k, v in SERVE_QUEUED.items()},
        "requests_per_s": len(all_lat) / wall, "completed": len(all_lat),
        "refused": sum(sum(v.values()) for v in refused.values()), "refused_by_circuit": refused,
        "largest_served": {k: (v[0], float(v[2])) if v else None for k, v in largest.items()},
        "waves": waves, "mean_requests_per_wave": wave_reqs / max(waves, 1),
        "oom_retries": st1["oom_retries"],
        "mean_wave_ms": 1e3 * wave_s / max(waves, 1),
        "error_vs_fp64_max_abs": max(max(err.values()), max(err_sat.values())),
        "error_vs_fp64_max_abs_by_class": {k: max(err[k], err_sat[k]) for k in err},
        "fp64_checked_requests": checked,
        "fp64_check": f"every served request of at most {SERVE_FP64_CHECK_MACS:.0e} complex MACs",
        "error_bound": 1e-6,
    }
    ctx.close()
    return out


# Config 3's terms at their stated size: (edge, seed) of the 50-vertex 3-regular
# p=2 light-cone terms whose seeded stochastic ordering (ContractionTools.h:
# 219-388 restated with a seed) reaches a qTorch rank-13 or rank-14
# intermediate (2^26-2^28 complex64 elements = 0.5-2 GiB, "rank 26-28" in
# dimension-2 legs).  Rule: for every edge, the first seed in 1..600 whose plan
# peaks at rank 14, else the first at rank 13 (29 of the 75 edges have one);
# bench.py --rescan-config3 recomputes the list.
CONFIG3_GRAPH = (50, 3, 3)          # vertices, degree, graph seed
CONFIG3_ANGLES = [0.3, 0.8, 0.6, 0.2]   # beta_1, beta_2, gamma_1, gamma_2
CONFIG3_TERMS = [(1, 533), (4, 224), (5, 533), (9, 515), (11, 485), (16, 11), (17, 162), (18, 402), (21, 201),
                 (25, 515), (29, 206), (30, 288), (32, 299), (35, 404), (36, 348), (37, 387), (45, 569), (46, 201),
                 (48, 560), (52, 138), (53, 595), (57, 210), (58, 20), (59, 572), (62, 370), (65, 358), (69, 222),
                 (70, 275), (72, 542), (74, 542)]


def config3_scan(max_seed=600):
    import qtorch_gb300 as qg
    dgf = qg.random_regular_graph(*CONFIG3_GRAPH[:2], seed=CONFIG3_GRAPH[2])
    out = []
    for e in range(qg.qaoa_num_edges(dgf)):
        q, m = qg.qaoa_term_text(dgf, 2, CONFIG3_ANGLES, e)
        best = None
        for s in range(1, max_seed + 1):
            r = qg.Plan(q, m, ordering="stochastic", seed=s, symbolic=True).peak_rank
            if r == 14:
                best = (e, s)
                break
            if r == 13 and best is None:
                best = (e, s)
        if best:
            out.append(best)
    return out


def run_config3(args):
    """Config 3: MaxCut QAOA p=2 on a seeded 3-regular 50-vertex graph, the
    light-cone terms whose seeded stochastic plans reach rank 13-14, run step by
    step (the tcgen05 3xTF32 GEMM takes the GEMM-shaped steps); mixed vs the
    bit-exact FP64 form per term.  Also every term under the line-graph
    ordering in one grouped launch, and two GEMM-shaped circuits (a 16-qubit
    random circuit, a 14-qubit QFT with <X> of its last qubit: every <Z> is 0)."""
    import qtorch_gb300 as qg
    from qtorch_gb300.circuits import qft_measure_text, qft_text, random_circuit_text
    ctx = qg.Context(0)
    dgf = qg.random_regular_graph(*CONFIG3_GRAPH[:2], seed=CONFIG3_GRAPH[2])
    out = {"workload": "MaxCut QAOA p=2, seeded random 3-regular graph, 50 vertices"}
    # --- the rank 13-14 terms, one plan each, step by step
    plans = []
    for e, seed in CONFIG3_TERMS:
        q, m = qg.qaoa_term_text(dgf, 2, CONFIG3_ANGLES, e)
        pl = qg.Plan(q, m, ordering="stochastic", seed=seed, ctx=ctx)
        if pl.peak_rank >= 13:
            plans.append(pl)
    v64 = [pl.execute(qg.FP64) for pl in plans]
    tc0, st0 = ctx.tensor_core_steps, ctx.stream_steps
    vmx = [pl.execute(qg.MIXED) for pl in plans]
    tc_steps, st_steps = ctx.tensor_core_steps - tc0, ctx.stream_steps - st0
    ctx.synchronize()

    def timed(prec, reps):
        best = None
        for _ in range(reps):
            t0 = time.perf_counter()
            for pl in plans:
                pl.execute(prec)
            el = time.perf_counter() - t0
            best = el if best is None else min(best, el)
        return best

    t_mx = timed(qg.MIXED, 3)
    t_64 = timed(qg.FP64, 1)
    err = np.array([abs(a - b) for a, b in zip(vmx, v64)])
    mag = np.array([abs(v) for v in v64])
    out["rank13_14"] = {
        "terms": len(plans), "peak_ranks": {str(r): sum(1 for p in plans if p.peak_rank == r) for r in (13, 14)},
        "ordering": "seeded stochastic (ContractionTools.h:219-388), per-term seeds in bench.py CONFIG3_TERMS",
        "complex_macs": int(sum(p.flops for p in plans)),
        "mixed_terms_per_s": len(plans) / t_mx, "fp64_terms_per_s": len(plans) / t_64,
        "mixed_over_fp64": t_64 / t_mx,
        "mixed_complex_macs_per_s": sum(p.flops for p in plans) / t_mx,
        "error_vs_fp64": {"max_abs": float(err.max()), "mean_abs": float(err.mean()), "bound": 1e-6},
        "value_fp64_abs": {"min": float(mag.min()), "max": float(mag.max())},
        "tensor_core_steps_per_pass": tc_steps, "stream_steps_per_pass": st_steps,
        "timing": "host clock around Plan.execute per term (synchronous), best of 3 passes (FP64: 1)"}
    # --- every edge term under the line-graph ordering, one grouped launch
    lg = []
    for e in range(qg.qaoa_num_edges(dgf)):
        q, m = qg.qaoa_term_text(dgf, 2, CONFIG3_ANGLES, e)
        lg.append(qg.Plan(q, m, ordering="linegraph", ctx=ctx))
    res = {}
    for prec in (qg.MIXED, qg.FP64):
        b = qg.Batch(ctx)
        for pl in lg:
            b.add(pl)
        b.prepare(prec)
        b.use_graph(True)
        policy = b.autotune()[0] if args.autotune else b.launch_policy
        vals = b.execute(prec)
        for _ in range(3):
            b.run()
        ctx.synchronize()
        t0 = time.perf_counter()
        for _ in range(20):
            b.run()
        b.fetch()
        res[prec] = (vals, (time.perf_counter() - t0) / 20, policy)
        b._release()
    err = np.abs(res[qg.MIXED][0] - res[qg.FP64][0])
    out["linegraph_all_terms"] = {"terms": len(lg), "peak_rank_max": max(p.peak_rank for p in lg),
                                  "complex_macs": int(sum(p.flops for p in lg)),
                                  "mixed_terms_per_s": len(lg) / res[qg.MIXED][1],
                                  "fp64_terms_per_s": len(lg) / res[qg.FP64][1],
                                  "error_vs_fp64": {"max_abs": float(err.max()), "mean_abs": float(err.mean())},
                                  "timing": "host clock over 20 graph launches after 3 warm-up launches"}
    gemm = []
    for name, text, meas in (("random 16 qubits depth 12, <Z_0>", random_circuit_text(16, 12, 1), "Z"),
                             ("QFT 14 qubits, <X_13>", qft_text(14, 5), qft_measure_text(14))):
        pl = qg.Plan(text, meas, ordering="linegraph", ctx=ctx)
        t0 = time.perf_counter()
        v64 = pl.execute(qg.FP64)
        t64 = time.perf_counter() - t0
        pl.execute(qg.MIXED)
        t0 = time.perf_counter()
        vmx = pl.execute(qg.MIXED)
        tmx = time.perf_counter() - t0
        gemm.append({"circuit": name, "peak_rank": pl.peak_rank, "complex_macs": int(pl.flops),
                     "mixed_s": tmx, "fp64_s": t64, "mixed_over_fp64": t64 / tmx, "error_abs": abs(vmx - v64),
                     "value_fp64": [v64.real, v64.imag]})
    out["gemm_shaped"] = gemm
    ctx.close()
    return out


CONFIG1_FIXTURE = os.path.join(HERE, "tests", "golden", "config1.json")


def run_config1(args):
    """Config 1: seeded 6-qubit depth-10 circuits (Rx(theta), theta ~ U[0, 2 pi),
    on every qubit, then CZ on 2 random disjoint pairs, per layer), <Z_0> by
    full contraction of the complex128 network under a fixed-seed stochastic
    ordering.  The fixtures hold, per seed, the circuit, the recorded ordering
    and the unmodified reference's value for it; the GPU runs the same
    ordering (FP64: checked equal to the reference bit for bit; mixed), and
    the reference itself (oracle/_ref, -O2 and as shipped) replays it on one
    host core (parse + contraction per evaluation, its ContractGivenSequence)."""
    import tempfile

    import qtorch_gb300 as qg
    with open(CONFIG1_FIXTURE) as f:
        cases = json.load(f)
    ctx = qg.Context(0)
    rows = []
    have_ref = ensure_reference_harness()
    for c in cases:
        plan = qg.Plan(c["qasm"], c["measure"], ordering="stochastic", seed=c["seed"], ctx=ctx)
        assert [list(p) for p in plan.sequence()] == c["sequence"]
        want = complex(*c["value"])
        row = {"seed": c["seed"], "complex_macs": plan.flops}
        for name, prec in (("fp64", qg.FP64), ("mixed", qg.MIXED)):
            v = plan.execute(prec)
            n, t0 = 0, time.perf_counter()
            while time.perf_counter() - t0 < 0.2 or n < 20:
                v = plan.execute(prec)
                n += 1
            row[f"gpu_{name}_us"] = 1e6 * (time.perf_counter() - t0) / n
            row[f"{name}_value"] = [v.real, v.imag]
        row["fp64_equals_reference"] = complex(*row["fp64_value"]) == want
        row["mixed_error_abs"] = abs(complex(*row["mixed_value"]) - want)
        if have_ref:
            with tempfile.TemporaryDirectory(prefix="qt_c1_") as wd:
                paths = [os.path.join(wd, x) for x in ("c.qasm", "c.meas", "c.seq")]
                for p, text in zip(paths, (c["qasm"], c["measure"],
                                           "\n".join(f"{a} {b}" for a, b in c["sequence"]) + "\n")):
                    with open(p, "w") as f:
                        f.write(text)
                for key, exe in (("reference_O2_us", REF_HARNESS), ("reference_as_shipped_us", REF_HARNESS_G)):
                    r = subprocess.run([exe, "seqtime", *paths, "1.0"], capture_output=True, text=True, timeout=600)
                    kv = {ln.split()[0]: ln.split()[1:] for ln in r.stdout.splitlines() if ln.split()}
                    row[key] = 1e6 * float(kv["seconds_per_rep"][0]) if r.returncode == 0 else None
                    if r.returncode == 0:
                        row[key.replace("_us", "_value_equal")] = complex(float(kv["value"][0]),
                                                                          float(kv["value"][1])) == want
        rows.append(row)
    ctx.close()
    return {"workload": "seeded 6-qubit depth-10 Rx + CZ(2 disjoint pairs) circuits, <Z_0>, this build's seeded "
                        "stochastic ordering (recorded in tests/golden/config1.json with the reference's value); "
                        "GPU: Plan.execute per evaluation (host wall clock, plan built once); reference: its "
                        "ContractGivenSequence on one host core, parse + contraction per evaluation",
            "reference_available": have_ref, "cases": rows}


def run_gemm_case(args):
    """--gemm-case qft14|rand16: one GEMM-shaped circuit of config 3 (QFT-14,
    <X_13>; random 16 qubits depth 12, <Z_0>), mixed form, executed three
    times (a case for ncu launch lists and captures); prints the last time."""
    import qtorch_gb300 as qg
    from qtorch_gb300.circuits import qft_measure_text, qft_text, random_circuit_text
    text, meas = {"qft14": (qft_text(14, 5), qft_measure_text(14)),
                  "rand16": (random_circuit_text(16, 12, 1), "Z")}[args.gemm_case]
    ctx = qg.Context(0)
    pl = qg.Plan(text, meas, ordering="linegraph", ctx=ctx)
    ts = []
    for _ in range(3):
        t0 = time.perf_counter()
        v = pl.execute(qg.MIXED)
        ts.append(time.perf_counter() - t0)
    print(json.dumps({"circuit": args.gemm_case, "mixed_s": ts, "value": [v.real, v.imag],
                      "tensor_core_steps": ctx.tensor_core_steps, "stream_steps": ctx.stream_steps}), flush=True)
    ctx.close()


def run_config3_mixed_only(args):
    """The first --config3-terms terms of config 3's rank 13-14 set, mixed form
    only, two passes (a small case for ncu launch lists and captures)."""
    import qtorch_gb300 as qg
    ctx = qg.Context(0)
    dgf = qg.random_regular_graph(*CONFIG3_GRAPH[:2], seed=CONFIG3_GRAPH[2])
    plans = []
    for e, seed in CONFIG3_TERMS[:args.config3_terms]:
        q, m = qg.qaoa_term_text(dgf, 2, CONFIG3_ANGLES, e)
        plans.append(qg.Plan(q, m, ordering="stochastic", seed=seed, ctx=ctx))
    out = []
    for _ in range(2):
        t0 = time.perf_counter()
        vals = [pl.execute(qg.MIXED) for pl in plans]
        out.append(time.perf_counter() - t0)
    print(json.dumps({"terms": len(plans), "seconds_per_pass": out, "values": [[v.real, v.imag] for v in vals]}))
    ctx.close()


def measure_permute(rank=13, dtype=1, kinds=("reverse", "random", "identity"), launches=20):
    """The tiled index permutation (qt_permute_device) on one tensor of `rank`
    wires (complex64: 537 MB at rank 13, larger than L2): CUDA events around
    each launch on the context stream, after 3 warm-up launches.  Algorithmic
    bytes per launch: the tensor read once and written once."""
    import ctypes

    import torch

    import qtorch_gb300 as qg
    stream = torch.cuda.Stream()
    ctx = qg.Context(0, stream=stream.cuda_stream)
    lib = qg._capi.load()
    elem = 8 if dtype == 1 else 16
    n = 4 ** rank
    x = torch.empty(n * elem // 4, dtype=torch.float32, device="cuda")
    y = torch.empty_like(x)
    x.normal_()
    torch.cuda.synchronize()
    rng = np.random.default_rng(3)
    out = {}
    for kind in kinds:
        perm = {"reverse": list(range(rank))[::-1], "identity": list(range(rank)),
                "random": [int(v) for v in rng.permutation(rank)]}[kind]
        pa = np.array(perm, dtype=np.int32)
        pp = pa.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
        times = []
        for i in range(launches + 3):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            assert lib.qt_permute_device(ctx.handle, ctypes.c_void_p(x.data_ptr()), rank, dtype, pp,
                                         ctypes.c_void_p(y.data_ptr())) == 0
            e1.record(stream)
            e1.synchronize()
            if i >= 3:
                times.append(e0.elapsed_time(e1) / 1e3)
        t = sum(times) / len(times)
        alg = 2 * n * elem
        out[kind] = {"perm": perm, "us": 1e6 * t, "alg_bytes": alg, "gb_per_s": alg / t / 1e9,
                     "frac_of_hbm_peak": alg / t / 1e9 / measured_peaks()[0]}
    ctx.close()
    del x, y
    torch.cuda.empty_cache()
    return {"tensor": f"rank {rank} {'complex64' if dtype == 1 else 'complex128'} ({n * elem / 1e6:.0f} MB)",
            "launches_timed": launches, "cases": out}


def run_permute_case(args):
    """--permute-case rank[,dtype]: the permutation measurement alone (a case for ncu)."""
    f = [int(x) for x in args.permute_case.split(",")]
    print(json.dumps(measure_permute(f[0], f[1] if len(f) > 1 else 1)), flush=True)


def run_stream_case(args):
    """One complex64 contraction step of ranks (rA, rB) summed over K wires --
    --stream-case rA,rB,K[,seed] -- with seeded random wires, through
    qt_contract_pair on device tensors (C's free wires in ContractNodes order),
    20 timed launches (CUDA events on the context stream, inputs larger than
    L2): a small case for ncu captures of the step kernels.  Prints the step's
    average time and algorithmic GB/s."""
    import ctypes

    import torch

    import qtorch_gb300 as qg
    f = [int(x) for x in args.stream_case.split(",")]
    ra, rb, k = f[:3]
    rng = np.random.default_rng(f[3] if len(f) > 3 else 1)
    wa, wb = rng.permutation(ra), rng.permutation(rb)
    sa, sb = [int(x) for x in wa[:k]], [int(x) for x in wb[:k]]
    ffa = np.array([1] * (ra - k) + [0] * (rb - k), dtype=np.uint8)
    fi = np.array([w for w in range(ra) if w not in sa] + [w for w in range(rb) if w not in sb], dtype=np.int32)
    sa_a, sb_a = np.array(sa, dtype=np.int32), np.array(sb, dtype=np.int32)
    stream = torch.cuda.Stream()
    ctx = qg.Context(0, stream=stream.cuda_stream)
    lib = qg._capi.load()
    ta, tb = ctypes.c_void_p(), ctypes.c_void_p()
    for r, t in ((ra, ta), (rb, tb)):
        assert lib.qt_tensor_create(ctx.handle, r, 1, ctypes.byref(t)) == 0
        host = rng.standard_normal(2 * 4 ** r).astype(np.float32)
        assert lib.qt_tensor_upload(ctx.handle, t, host.ctypes.data_as(ctypes.c_void_p), host.nbytes) == 0
    P8, P32 = ctypes.POINTER(ctypes.c_uint8), ctypes.POINTER(ctypes.c_int32)
    ctx.synchronize()
    n0 = (ctx.stream_steps, ctx.tensor_core_steps)
    times = []
    for i in range(23):
        tc = ctypes.c_void_p()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        assert lib.qt_contract_pair(ctx.handle, ta, tb, len(fi), ffa.ctypes.data_as(P8), fi.ctypes.data_as(P32),
                                    k, sa_a.ctypes.data_as(P32), sb_a.ctypes.data_as(P32), ctypes.byref(tc)) == 0
        e1.record(stream)
        e1.synchronize()
        lib.qt_tensor_free(ctx.handle, tc)
        if i >= 3:
            times.append(e0.elapsed_time(e1) / 1e3)
    lib.qt_tensor_free(ctx.handle, ta)
    lib.qt_tensor_free(ctx.handle, tb)
    t = sum(times) / len(times)
    alg = 8 * (4 ** ra + 4 ** rb + 4 ** (ra + rb - 2 * k))
    print(json.dumps({"step": [ra, rb, k], "sum_a": sa, "sum_b": sb, "us": 1e6 * t, "alg_bytes": alg,
                      "gb_per_s": alg / t / 1e9, "stream_steps": ctx.stream_steps - n0[0],
                      "tensor_core_steps": ctx.tensor_core_steps - n0[1]}))
    ctx.close()


def run_only_serving(args):
    print(json.dumps(run_serving(args)), flush=True)


def run_only_config3(args):
    print(json.dumps(run_config3(args)), flush=True)


def run_only_batched(args):
    import torch

    import qtorch_gb300 as qg
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx = qg.Context(0, stream=stream.cuda_stream)
    flush_buf = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    print(json.dumps(run_batched(ctx, args, stream, lambda: flush_buf.fill_(1))), flush=True)
    ctx.close()


def run_engine(args):
    import torch

    import qtorch_gb300 as qg

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    # a non-default stream: the engine captures its launches into a CUDA graph there
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx = qg.Context(local, stream=stream.cuda_stream)

    dgf = qg.random_regular_graph(NODES, DEGREE, seed=args.graph_seed)
    points = angle_points(1000 + rank, args.warmup + args.steps + 1)
    terms = build_terms(dgf, points[0])
    plans = [qg.Plan(q, m, ordering="linegraph", ctx=ctx) for q, m in terms]
    n_terms = len(plans)

    batches = {}
    for prec in (qg.FP64, qg.MIXED):
        b = qg.Batch(ctx)
        for p in plans:
            b.add(p)
        b.prepare(prec)
        b.use_graph(True)
        batches[prec] = b
    # launch policies (shared-memory regions, CTAs per SM, schedule) chosen by
    # timing candidates on this batch; part of the setup, not the timed region
    policies = {prec: (batches[prec].autotune()[0] if args.autotune else batches[prec].launch_policy)
                for prec in batches}

    flush_buf = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")

    def flush():
        flush_buf.fill_(1)

    # accuracy of the mixed form against the FP64 form at the first point
    v64 = batches[qg.FP64].execute(qg.FP64)
    vmx = batches[qg.MIXED].execute(qg.MIXED)
    err = np.abs(vmx - v64)

    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t_mixed = time_steps(batches[qg.MIXED].run, args.steps, args.warmup, stream, flush)
    t_fp64 = time_steps(batches[qg.FP64].run, args.steps, args.warmup, stream, flush)

    # end to end through the public API: new angles -> H2D -> run -> D2H, every step
    rot = [term_rotation_angles(q) for q, _ in terms]
    n_rot = [len(r) for r in rot]
    for p, n in zip(plans, n_rot):
        assert p.num_rotations == n

    def angles_for(point):
        # Rz(-gamma) per light-cone edge, then Rx(2 beta) per qubit (maxcut.h:205-233), 6 significant digits
        beta, gamma = point
        out = []
        for q, _ in terms:
            for line in q.split("\n"):
                t = line.split(" ")
                if t[0] == "Rz":
                    out.append(float("%g" % -gamma))
                elif t[0] == "Rx":
                    out.append(float("%g" % (beta * 2.0)))
        return np.array(out)

    # (only the angles travel; the interpreter builds the gate tensors on the device)
    bm = batches[qg.MIXED]
    # the end-to-end calls are short (tens of microseconds): at least 200 timed
    # calls, so one slow call (the host thread descheduled) does not decide the mean
    e2e_steps = max(args.steps, 200)
    step_angles = [angles_for(points[1 + (j % (len(points) - 1))]) for j in range(args.warmup + e2e_steps)]

    def e2e_loop(name):
        times = []
        torch.cuda.synchronize()
        for j, a in enumerate(step_angles):
            if j == args.warmup:
                torch.cuda.nvtx.range_push(name)
            t0 = time.perf_counter()
            v = bm.evaluate(a)
            t1 = time.perf_counter()
            if j >= args.warmup:
                times.append(t1 - t0)
        torch.cuda.nvtx.range_pop()
        return times, v

    # one captured graph launch per call (angles read from, values written to pinned memory)
    graph_times, vals_graph = e2e_loop("e2e_graph")
    # the resident engine: no launch per call, plans staged in shared memory across calls
    bm.use_resident(1.0)
    e2e_times, vals = e2e_loop("e2e")
    engine_starts = bm.resident_starts
    bm.use_resident(0)
    a = step_angles[-1]
    assert np.array_equal(vals, vals_graph)
    # the last point again through the FP64 form with host-built leaves
    bf = batches[qg.FP64]
    bf.set_rotations(a)
    bf.upload()
    bf.run()
    e2e_err = np.abs(vals - bf.fetch())
    assert np.all(np.isfinite(vals))

    sum_mixed, sum_fp64, sum_e2e, sum_graph = max_over_ranks(
        [sum(t_mixed), sum(t_fp64), sum(e2e_times), sum(graph_times)], world, "cuda")
    total_terms = n_terms * args.steps * world
    e2e_terms = n_terms * e2e_steps * world
    value = total_terms / sum_mixed
    fp64_value = total_terms / sum_fp64
    e2e_value = e2e_terms / sum_e2e

    peak, peak_kind = measured_peaks()
    alg_bytes = sum(p.algorithmic_bytes(qg.MIXED) for p in plans)
    achieved = alg_bytes / (sum_mixed / args.steps) / 1e9
    cmacs = sum(p.flops for p in plans)
    traffic, traffic_note = profiled_traffic()

    line = {
        "metric": METRIC, "value": value, "unit": "terms/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * sum_mixed / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "complex64/fp32 (compensated twice-fp32 final reductions, complex128 values)",
        "data": "synthetic",
        "config": shared_config(args.graph_seed),
        "timing": {"l2": "flushed between steps (256 MiB write), per-step CUDA events on the launching stream",
                   "parallelism": f"weak: each rank evaluates its own {n_terms} terms per step",
                   "launch_policy": {"autotuned": bool(args.autotune), "mixed": policies[qg.MIXED],
                                     "fp64": policies[qg.FP64]}},
        "fp64": {"value": fp64_value, "unit": "terms/s", "ms_per_step": 1e3 * sum_fp64 / args.steps,
                 "parity": "bit-exact with the reference CPU loop under the same ordering"},
        "mixed_over_fp64": value / fp64_value,
        "error_vs_fp64": {"max_abs": float(err.max()), "mean_abs": float(err.mean()), "bound": 1e-6},
        "e2e": {"value": e2e_value, "unit": "terms/s", "h2d_bytes_per_step": bm.h2d_bytes,
                "d2h_bytes_per_step": bm.d2h_bytes, "ms_per_step": 1e3 * sum_e2e / e2e_steps,
                "steps": e2e_steps, "engine_starts": engine_starts,
                "path": "Batch.evaluate(angles) = qt_batch_evaluate with the resident engine (qt_batch_use_resident): "
                        "angles written to pinned host memory and read by the resident CTAs over the CPU-GPU "
                        "link, gate tensors built on the device, values and done flags written back to pinned "
                        "memory; host clock around each call",
                "error_vs_fp64_max_abs": float(e2e_err.max()),
                "median_ms_per_step": 1e3 * float(np.median(e2e_times)),
                "slowest_calls_ms": sorted(round(1e3 * t, 4) for t in e2e_times)[-5:],
                "graph_path": {"value": e2e_terms / sum_graph, "ms_per_step": 1e3 * sum_graph / e2e_steps,
                               "median_ms_per_step": 1e3 * float(np.median(graph_times)),
                               "path": "qt_batch_evaluate without the resident engine: one captured graph launch "
                                       "per call plus a stream synchronisation"}},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "traffic_source": traffic_note, "peak_source": peak_kind,
                     "kernel": "plan_kernel<mixed>",
                     "algorithmic_bytes_per_launch": alg_bytes, "complex_macs_per_launch": cmacs},
        "gpu_launches": int(args.steps * batches[qg.MIXED].launches_per_run),
        "clocks": clk.summary(),
    }
    if not args.no_batched:
        bm._release()
        line["batched"] = run_batched(ctx, args, stream, flush)
    if not args.no_permute:
        line["permute"] = measure_permute()
    if not args.no_config1:
        line["config1"] = run_config1(args)
    if not args.no_serving:
        line["serving"] = run_serving(args)
    if not args.no_config3:
        line["config3"] = run_config3(args)
    # the reference arm replays the committed orderings: they must be this run's
    with open(REF_FIXTURE) as f:
        fx_seqs = json.load(f)["sequences"]
    line["reference_orderings_match"] = fx_seqs == [[x for pr in p.sequence() for x in pr] for p in plans]
    if rank == 0 and world == 1 and not args.no_cpu:
        cores = os.cpu_count() or 1
        seqs = sequences_for(terms)
        jobs = [(q, m, s) for (q, m), s in zip(terms, seqs)]
        prate, pdone, pel, parse_share = cpu_terms_per_s(jobs, cores, min_seconds=args.cpu_seconds / 2)
        port = {"value": prate, "unit": "terms/s", "cores": cores, "kind": "port",
                "sample": f"{pdone} terms in {pel:.1f} s on the C restatement (oracle/qt_oracle.c)",
                "parse_share": parse_share}
        if ensure_reference_harness():
            rate, n, el = reference_cpu_sample(args.cpu_seconds, cores)
            share, rate_ex = reference_parse_split(REF_HARNESS, rate)
            line["cpu_baseline"] = {"value": rate, "unit": "terms/s", "cores": cores, "kind": "reference",
                                    "sample": f"{n} steps of 60 terms in {el:.1f} s: the unmodified reference "
                                              "(g++ -O2) writing, parsing and contracting every term "
                                              "(maxcut.cpp:166-196) under the recorded orderings, "
                                              f"{cores} forked workers",
                                    "parse_share": share, "terms_per_s_excluding_parse": rate_ex,
                                    "port": port}
        else:
            line["cpu_baseline"] = port
    line["summary"] = bench_summary(line)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    del batches, plans
    ctx.close()


def bench_summary(line):
    """The secondary numbers in a few hundred characters, last in the line."""
    def r(x, d=4):
        return None if x is None else float(f"{x:.{d}g}")
    s = {"config2": {"mixed_terms_per_s": r(line["value"]), "fp64_terms_per_s": r(line["fp64"]["value"]),
                     "mixed_over_fp64": r(line["mixed_over_fp64"], 3),
                     "e2e_terms_per_s": r(line["e2e"]["value"]),
                     "max_err": r(line["error_vs_fp64"]["max_abs"], 2)}}
    if "batched" in line:
        b = line["batched"]
        s["config4_batched"] = {"mixed_terms_per_s": r(b["mixed_terms_per_s"]),
                                "fp64_terms_per_s": r(b["fp64_terms_per_s"]),
                                "mixed_over_fp64": r(b["mixed_over_fp64"], 3),
                                "max_err": r(b["error_vs_fp64"]["max_abs"], 2)}
    if "config3" in line and "rank13_14" in line["config3"]:
        c = line["config3"]["rank13_14"]
        s["config3_rank13_14"] = {"terms": c["terms"], "mixed_terms_per_s": r(c["mixed_terms_per_s"]),
                                  "fp64_terms_per_s": r(c["fp64_terms_per_s"]),
                                  "mixed_over_fp64": r(c["mixed_over_fp64"], 3),
                                  "max_err": r(c["error_vs_fp64"]["max_abs"], 2),
                                  "mean_err": r(c["error_vs_fp64"]["mean_abs"], 2),
                                  "tensor_core_steps": c["tensor_core_steps_per_pass"],
                                  "stream_steps": c["stream_steps_per_pass"]}
    if "serving" in line:
        v = line["serving"]
        s["config5_serving"] = {"p50_ms": r(v["p50_ms"], 3), "p99_ms": r(v["p99_ms"], 3),
                                "offered_per_s": r(v["arrival_rate_per_s"]),
                                "saturation_per_s": r(v["saturation_requests_per_s"]),
                                "p99_ms_by_class": {k: r(x, 3) for k, x in v["p99_ms_by_class"].items()
                                                    if x is not None},
                                "max_err": r(v["error_vs_fp64_max_abs"], 2), "refused": v["refused"],
                                "completed": v["completed"]}
    if "config1" in line:
        cs = line["config1"]["cases"]
        s["config1"] = {"fp64_equals_reference": all(c["fp64_equals_reference"] for c in cs),
                        "gpu_fp64_us": r(sum(c["gpu_fp64_us"] for c in cs) / len(cs), 3),
                        "reference_O2_us": r(sum(c.get("reference_O2_us") or 0 for c in cs) / len(cs), 3)}
    if "permute" in line:
        s["permute_rank13_c64"] = {k: {"gb_per_s": r(v["gb_per_s"]), "frac": r(v["frac_of_hbm_peak"], 3)}
                                   for k, v in line["permute"]["cases"].items()}
    if "cpu_baseline" in line:
        c = line["cpu_baseline"]
        s["cpu"] = {"kind": c["kind"], "terms_per_s": r(c["value"]), "cores": c["cores"]}
    return s


REF_FIXTURE = os.path.join(HERE, "tests", "golden", "bench_qaoa_p1_30node.json")
REF_HARNESS = os.path.join(HERE, "oracle", "_ref", "qt_ref_harness")      # the reference at -O2
REF_HARNESS_G = os.path.join(HERE, "oracle", "_ref", "qt_ref_harness_g")  # as its Makefile builds it (-g)


def shared_config(graph_seed):
    """The workload description both arms print (same dict, so the lines compare)."""
    return {"workload": WORKLOAD, "graph_seed": graph_seed, "terms_per_step": 60,
            "angles": "beta,gamma ~ U[0,pi) seeded, a new point every step",
            "ordering": "line-graph (min-fill) sequences recorded once, replayed every step"}


def reference_inputs(workdir, steps):
    """Files the reference harness reads: the graph, one recorded ordering per
    term, one (beta, gamma) line per step.  No import of this build's package:
    the orderings come from the committed fixture (tests/golden/make_bench_inputs.py)."""
    with open(REF_FIXTURE) as f:
        fx = json.load(f)
    dgf = os.path.join(workdir, "graph.dgf")
    with open(dgf, "w") as f:
        f.write(fx["dgf"])
    seq = os.path.join(workdir, "sequences.txt")
    with open(seq, "w") as f:
        f.write("\n".join(" ".join(map(str, s)) for s in fx["sequences"]) + "\n")
    pts = angle_points(1000, steps)
    ang = os.path.join(workdir, "angles.txt")
    with open(ang, "w") as f:
        f.write("\n".join(f"{float(b)!r} {float(g)!r}" for b, g in pts) + "\n")
    return fx, dgf, seq, ang


def run_reference_harness(exe, steps, workers):
    """Per-step seconds of the reference's own QAOA objective (maxcut.cpp:166-196:
    write each term's QASM and measurement files, parse them, contract them with
    ContractGivenSequence under the recorded ordering) on `workers` forked
    processes, and the 60 values of the first step."""
    import tempfile
    with tempfile.TemporaryDirectory(prefix="qt_ref_bench_") as wd:
        fx, dgf, seq, ang = reference_inputs(wd, steps)
        r = subprocess.run([exe, "bench", dgf, str(fx["p"]), seq, ang, str(workers), wd],
                           capture_output=True, text=True, timeout=1800)
    if r.returncode != 0:
        raise RuntimeError(f"{os.path.basename(exe)} rc={r.returncode}: {r.stderr.strip()[:200]}")
    times, values = [], {}
    for line in r.stdout.splitlines():
        t = line.split()
        if t and t[0] == "step":
            times.append(float(t[2]))
        elif t and t[0] == "value":
            values[int(t[1])] = complex(float(t[2]), float(t[3]))
        elif t and t[0] == "split":
            # worker seconds writing + parsing the terms' files, and contracting them
            REF_SPLIT[os.path.basename(exe)] = (float(t[1]), float(t[2]))
    return times, [values[k] for k in sorted(values)]


REF_SPLIT = {}   # harness name -> (file write + parse seconds, contraction seconds) of its last run


def ensure_reference_harness():
    """Build oracle/_ref from the staged reference headers if it is not there yet."""
    if not (os.path.exists(REF_HARNESS) and os.path.exists(REF_HARNESS_G)):
        subprocess.run(["make", "-s", "-C", os.path.join(HERE, "oracle"), "ref"], check=False,
                       stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    return os.path.exists(REF_HARNESS) and os.path.exists(REF_HARNESS_G)


def reference_cpu_sample(seconds, workers):
    """The reference (-O2) on a bounded sample: enough steps for about `seconds`."""
    t1, _ = run_reference_harness(REF_HARNESS, 3, workers)
    per = max(min(t1[1:]), 1e-4)
    n = int(min(max(seconds / per, 5), 20000))
    t, _ = run_reference_harness(REF_HARNESS, n + 2, workers)
    t = t[2:]
    return 60 * len(t) / sum(t), len(t), sum(t)


def reference_parse_split(exe, rate):
    """(share of the workers' time spent writing and parsing the term files,
    terms/s with that share taken out) of the harness's last run."""
    prep, contract = REF_SPLIT.get(os.path.basename(exe), (0.0, 0.0))
    if prep + contract <= 0:
        return None, None
    share = prep / (prep + contract)
    return share, rate / max(1e-12, 1.0 - share)


def run_reference(args):
    """--impl reference: the unmodified reference (oracle/_ref, built from its
    own headers) timed on all host cores, on the engine arm's workload.  This
    process never imports this build's package."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    parse_share = None
    if ensure_reference_harness():
        times, _ = run_reference_harness(REF_HARNESS, args.warmup + args.steps, cores)
        times = times[args.warmup:]
        kind = "reference"
        sample = (f"{args.steps} steps of 60 terms after {args.warmup} warm-up steps: the reference's F_p body "
                  "(maxcut.cpp:166-196) per term -- write the QASM and measurement files, parse them "
                  "(Network.h:246-304), ContractGivenSequence (ContractionTools.h:392-411) over the recorded "
                  f"ordering -- unmodified reference headers built with g++ -O2, {cores} forked workers, one term "
                  "at a time")
        parse_share, _ = reference_parse_split(REF_HARNESS, 1.0)
        gsteps = max(3, min(args.steps, 10))
        gt, _ = run_reference_harness(REF_HARNESS_G, 2 + gsteps, cores)
        g_rate = 60 * gsteps / sum(gt[2:])
        g_share, g_ex = reference_parse_split(REF_HARNESS_G, g_rate)
        as_shipped = {"value": g_rate, "unit": "terms/s", "steps": gsteps,
                      "build": "g++ -g -std=c++11 -pthread, no -O (the reference's Makefile:34)",
                      "parse_share": g_share, "terms_per_s_excluding_parse": g_ex}
    else:
        # no staged reference headers on this machine: the C restatement instead
        import multiprocessing as mp

        from oracle import qaoa_terms
        with open(REF_FIXTURE) as f:
            fx = json.load(f)
        seqs = [[(s[2 * i], s[2 * i + 1]) for i in range(len(s) // 2)] for s in fx["sequences"]]
        points = angle_points(1000, args.warmup + args.steps)
        pool = mp.get_context("spawn").Pool(cores)
        times = []
        chunk = max(1, -(-len(seqs) // cores))
        for j in range(args.warmup + args.steps):
            pt = points[j]
            t0 = time.perf_counter()
            terms = qaoa_terms.all_terms(fx["dgf"], P, [pt[0], pt[1]])
            pool.map(_cpu_worker, [(q, m, s) for (_, q, m), s in zip(terms, seqs)], chunksize=chunk)
            if j >= args.warmup:
                times.append(time.perf_counter() - t0)
        pool.close()
        kind = "port"
        sample = f"{args.steps} steps of 60 terms on the C restatement of src/Network.h:876-971 (no reference build here)"
        as_shipped = None
    value = 60 * args.steps / sum(times)
    line = {
        "metric": METRIC, "value": value, "unit": "terms/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "complex128", "data": "synthetic",
        "config": shared_config(args.graph_seed),
        "impl": "reference",
        "cpu_baseline": {"value": value, "unit": "terms/s", "cores": cores, "kind": kind, "sample": sample},
        "parse_share": parse_share if kind == "reference" else None,
        "e2e": {"value": value, "unit": "terms/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    if as_shipped:
        line["as_shipped"] = as_shipped
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--graph-seed", type=int, default=1)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batched", action="store_true", help="skip the 64-point x 16-graph batched workload")
    ap.add_argument("--batched-points", type=int, default=64)
    ap.add_argument("--batched-steps", type=int, default=5)
    ap.add_argument("--no-serving", action="store_true", help="skip the request-serving workload")
    ap.add_argument("--serve-requests", type=int, default=3000)
    ap.add_argument("--serve-rate", type=float, default=0.0,
                    help="Poisson arrival rate, requests/s (0: --serve-load x the measured saturation throughput)")
    ap.add_argument("--serve-load", type=float, default=0.7)
    ap.add_argument("--no-config3", action="store_true", help="skip the p=2 50-vertex and GEMM-shaped cases")
    ap.add_argument("--only-config3", action="store_true", help="run only the config-3 cases (for profiling)")
    ap.add_argument("--config3-terms", type=int, default=0,
                    help="run only the first N rank 13-14 terms of config 3, mixed form (for profiling)")
    ap.add_argument("--no-permute", action="store_true", help="skip the index-permutation measurement")
    ap.add_argument("--no-config1", action="store_true", help="skip the 6-qubit config-1 circuits")
    ap.add_argument("--only-config1", action="store_true", help="run only the config-1 circuits")
    ap.add_argument("--gemm-case", default="", choices=["", "qft14", "rand16"],
                    help="run one GEMM-shaped circuit of config 3 three times (for profiling)")
    ap.add_argument("--permute-case", default="",
                    help="rank[,dtype]: time the tiled index permutation on one tensor (dtype 1: complex64, 0: complex128)")
    ap.add_argument("--stream-case", default="",
                    help="rA,rB,K[,seed]: time one complex64 step of these ranks (for profiling)")
    ap.add_argument("--rescan-config3", action="store_true",
                    help="print the (edge, seed) list of config 3's rank 13-14 terms and exit")
    ap.add_argument("--only-serving", action="store_true", help="run only the serving workload")
    ap.add_argument("--only-batched", action="store_true",
                    help="run only the batched workload and print its numbers (a small case for profiling)")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the default launch policies instead of timing candidates (qt_batch_autotune)")
    args = ap.parse_args()
    args.autotune = not args.no_autotune
    if args.warmup < 3:
        args.warmup = 3
    from oracle import port
    port.build()
    if args.impl == "reference":
        run_reference(args)
        return
    from qtorch_gb300 import build as qbuild
    qbuild.build()
    if args.rescan_config3:
        print(config3_scan())
    elif args.config3_terms > 0:
        run_config3_mixed_only(args)
    elif args.stream_case:
        run_stream_case(args)
    elif args.permute_case:
        run_permute_case(args)
    elif args.gemm_case:
        run_gemm_case(args)
    elif args.only_config1:
        print(json.dumps(run_config1(args)), flush=True)
    elif args.only_batched:
        run_only_batched(args)
    elif args.only_config3:
        run_only_config3(args)
    elif args.only_serving:
        run_only_serving(args)
    else:
        run_engine(args)


if __name__ == "__main__":
    main()
