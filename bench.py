"""Benchmark of the explicit C3D4 step on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (the large plain-FP64 configuration): unit cube meshed as 100^3 hexes,
each split into 6 tets -> 6,000,000 C3D4 elements and 1,030,301 nodes; interior
nodes jittered by a seeded +-0.1 h; 3D-Compressible-Neo-Hookean E=1e6 Pa,
nu=0.3, rho=1000; bottom face fixed; top face z velocity ramped linearly to
0.1 m/s over 200 steps; dt = 0.5 x CFL recomputed every step.  One "step" is
one explicit time step over the whole mesh.  Synthetic, seeded data.

Prints one JSON line: value = element-steps/s of the plain FP64 path with the
mesh resident in HBM (device time of K steps), e2e = the same through the C ABI
from host buffers (mesh upload, set-up, K steps and the read-back of u, v, a),
plus the mixed-precision and reference-order variants, the element kernel's
roofline and the CPU baseline.  --impl reference times the CPU implementation
of the path (the oracle's C restatement on all host cores) on a bounded sample.
Under torchrun each rank runs an independent replica ("replicas only").
"""
import argparse
import csv
import io
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "v.1.1_gb300"))

N_CUBE = 100
RAMP_STEPS = 200
V_TOP = 0.1
SEED = 1234
MATERIAL = (1, 1e6, 0.3, 1000.0)   # 3D-Compressible-Neo-Hookean
METRIC = "element-steps/s on 1 GB300 (plain FP64 vs mixed/batched); p50/p99 solve latency"
WORKLOAD = ("cube 100^3 hexes -> 6,000,000 C3D4 tets / 1,030,301 nodes, +-0.1h seeded jitter, "
            "3D-Compressible-Neo-Hookean E=1e6 nu=0.3 rho=1000, bottom fixed, top z-velocity ramped "
            "to 0.1 m/s over 200 steps, dt=0.5 CFL per step")


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profiled(key, kernel="pool_elem_kernel<FP64>"):
    """A per-element figure of a kernel from the committed ncu captures
    (profiles/ncu_figures.json: DRAM bytes per element from one --set full
    capture on the 64^3 cube, FP64 instructions per element, the FP64 peak
    measured with a DFMA loop), or None."""
    try:
        with open(os.path.join(ROOT, "profiles", "ncu_figures.json")) as f:
            return float(json.load(f)[kernel][key])
    except (OSError, KeyError, ValueError, TypeError):
        return None


def fp64_peak():
    """The FP64 pipe's DFMA rate on this GPU in G op/s, measured now by the
    library's probe (v.1.1_gb300/_build/msx_fp64_peak, built with the library),
    else the figure in profiles/ncu_figures.json; and which of the two."""
    exe = os.path.join(ROOT, "v.1.1_gb300", "_build", "msx_fp64_peak")
    try:
        r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
        for line in r.stdout.splitlines():
            if r.returncode == 0 and line.startswith("fp64_dfma_gops"):
                return float(line.split()[1]), "measured"
    except (OSError, subprocess.SubprocessError, ValueError):
        pass
    return profiled("fp64_peak_gops"), "recorded"


class Clocks:
    """nvidia-smi samples during a timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.proc:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        rows = [r for r in csv.reader(io.StringIO(self.out or "")) if len(r) >= 9]
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = max(float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit())
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].strip() == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(rows)}


def make_case(n):
    import msx
    X, conn = msx.mesh_cube(n, SEED, 0.1)
    bcs = msx.cube_bcs(n, V_TOP, msx.BC_VEL_RAMP, RAMP_STEPS)
    return X, conn, bcs


def run_variant(X, conn, bcs, precision, steps, warmup, device, keep_u=False):
    """Create, warm up, then time exactly `steps` steps with the mesh resident.
    With keep_u, also return u after the run (warm-up + steps + the 6 profiled
    steps), to compare the precision modes at the same step."""
    import msx
    S = msx.Solver(X, conn, [MATERIAL], bcs, 0.0, 1e30, 0.5, max_steps=0, precision=precision)
    S.run(warmup)
    with Clocks(device) as ck:
        rep = S.run(steps)
    assert rep.steps == steps, rep
    prof = S.profile(6)
    u = S.state()[0] if keep_u else None
    S.close()
    return (rep, prof, ck.summary(), u) if keep_u else (rep, prof, ck.summary())


def mixed_roofline(ne, nn, prof, ms_per_step):
    """HBM roofline of the mixed step: per element conn 16 + FP32 dphi/dX 48 + wJ 4 + length 4
    = 72 B, per node 176 B as in the FP64 step."""
    peak, peak_kind = peaks()
    alg_elem, alg_step = 72.0 * ne, 72.0 * ne + 176.0 * nn
    ach = alg_elem / (prof.element_ms * 1e-3) / 1e9
    step = alg_step / (ms_per_step * 1e-3) / 1e9
    tr = profiled("dram_bytes_per_element", "pool_elem_kernel<MIXED>")
    return {"bound": "hbm", "kernel": "pool_elem_kernel<MIXED>", "achieved": ach, "peak": peak, "unit": "GB/s",
            "frac": ach / peak, "peak_kind": peak_kind, "traffic": tr * ne if tr else None,
            "alg_bytes_per_launch": alg_elem,
            "step": {"alg_bytes": alg_step, "achieved": step, "frac": step / peak}}


def dword_roofline(ne, nn, prof, ms_per_step):
    """HBM roofline of the double-word step: per element conn 16 + dphi/dX as (hi, lo) 72 +
    wJ 8 + FP32 length 4 = 100 B, per node 176 B (the FP64 step's nodal data)."""
    peak, peak_kind = peaks()
    alg_elem, alg_step = 100.0 * ne, 100.0 * ne + 176.0 * nn
    ach = alg_elem / (prof.element_ms * 1e-3) / 1e9
    step = alg_step / (ms_per_step * 1e-3) / 1e9
    tr = profiled("dram_bytes_per_element", "pool_elem_kernel<DW>")
    return {"bound": "hbm", "kernel": "pool_elem_kernel<DW>", "achieved": ach, "peak": peak, "unit": "GB/s",
            "frac": ach / peak, "peak_kind": peak_kind, "traffic": tr * ne if tr else None,
            "alg_bytes_per_launch": alg_elem,
            "step": {"alg_bytes": alg_step, "achieved": step, "frac": step / peak},
            "note": "FP64's algebra in double-word FP32 arithmetic; rel. L2 of u vs the reference <= 6e-13 "
                    "on the golden decks (tests/test_gpu_parity.py)"}


def run_e2e(X, conn, bcs, steps):
    """Whole job through the C ABI from host buffers: upload, set-up, K steps,
    read back u, v, a.  The mesh is in page-locked host memory and the BCs in
    the C ABI's msx_bc array before the clock starts (a caller hands the
    library its own arrays; converting Python tuples is harness work), and the
    state is read back into page-locked buffers."""
    import msx
    import torch

    def pinned(shape, dtype):
        return torch.empty(shape, dtype=dtype, pin_memory=True).numpy()

    Xp, cp = pinned(X.shape, torch.float64), pinned(conn.shape, torch.int32)
    Xp[...] = X
    cp[...] = conn
    barr = msx.bc_array(bcs)   # the C ABI's msx_bc array, as the caller holds its BCs
    out = tuple(pinned((X.size,), torch.float64) for _ in range(3))
    t0 = time.perf_counter()
    S = msx.Solver(Xp, cp, [MATERIAL], barr, 0.0, 1e30, 0.5, max_steps=0, precision=msx.FP64)
    rep = S.run(steps)
    u, v, a = S.state(out)
    wall = time.perf_counter() - t0
    S.close()
    h2d = X.nbytes + conn.nbytes + len(bcs) * 24
    d2h = u.nbytes + v.nbytes + a.nbytes
    return wall, rep, h2d, d2h


def cpu_baseline(X, conn, bcs, target_s=10.0):
    """The oracle's C restatement (OpenMP, all host cores) on a bounded number
    of steps of the same mesh."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build()
    mesh = O.Mesh(X, conn)
    cores = os.cpu_count() or 1
    mat = [O.Material(*MATERIAL)]
    probe = O.run(mesh, mat, [O.Solver(0.0, 1e30, 0.5, bcs, max_steps=1)], nthreads=cores)
    per_step = max(probe.loop_seconds, 1e-3)
    nsteps = int(max(2, min(200, target_s / per_step)))
    r = O.run(mesh, mat, [O.Solver(0.0, 1e30, 0.5, bcs, max_steps=nsteps)], nthreads=cores)
    value = mesh.ne * r.steps / r.loop_seconds
    return {"value": value, "unit": "element-steps/s", "cores": cores, "kind": "port",
            "sample": "%d steps of the 6M-tet FP64 workload, oracle C restatement (OpenMP, %d threads), "
                      "set-up excluded; %.2f s" % (r.steps, cores, r.loop_seconds)}


def reference_arm(args):
    """The CPU implementation of the path (the oracle's C restatement of the
    reference, OpenMP over all host cores) on the same workload: W warm-up
    steps, then up to K timed steps bounded to about a minute."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build()
    mesh = O.cube_mesh(N_CUBE, SEED, 0.1)
    bcs = O.cube_bcs(N_CUBE, V_TOP, O.BC_VEL_RAMP, RAMP_STEPS)
    cores = os.cpu_count() or 1
    mat = [O.Material(*MATERIAL)]
    w = O.run(mesh, mat, [O.Solver(0.0, 1e30, 0.5, bcs, max_steps=min(args.warmup, 3))], nthreads=cores)
    per_step = max(w.loop_seconds / max(w.steps, 1), 1e-3)
    k = int(max(1, min(args.steps, 60.0 / per_step)))
    r = O.run(mesh, mat, [O.Solver(0.0, 1e30, 0.5, bcs, max_steps=k)], nthreads=cores)
    value = mesh.ne * r.steps / r.loop_seconds
    sample = ("%d of %d steps of the 6M-tet FP64 workload (bounded to ~60 s), oracle C restatement of the "
              "reference path, OpenMP %d threads, set-up excluded" % (r.steps, args.steps, cores))
    return {"impl": "reference", "metric": METRIC, "value": value, "unit": "element-steps/s", "n_gpus": args.gpus,
            "steps": r.steps, "warmup": w.steps, "ms_per_step": 1e3 * r.loop_seconds / r.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": WORKLOAD, "num_elems": mesh.ne, "num_nodes": mesh.nn,
                                            "precision": "FP64", "parallelism": "host cores (OpenMP)"},
            "cpu_baseline": {"value": value, "unit": "element-steps/s", "cores": cores, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": "element-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def accuracy_sample(ns, nus, k=8, seed=0):
    """Indices of the solves whose results are checked against FP64: the
    largest and the smallest cube, the highest and the lowest nu, then seeded
    picks up to k."""
    pick = [int(np.argmax(ns)), int(np.argmin(ns)), int(np.argmax(nus)), int(np.argmin(nus))]
    for i in np.random.default_rng(seed).permutation(len(ns)):
        if len(set(pick)) >= k:
            break
        pick.append(int(i))
    return sorted(set(pick))


def fp64_alone(X, conn, material, bcs, steps):
    """u after `steps` steps of one solve run by itself in the plain FP64 path."""
    import msx
    S = msx.Solver(X, conn, [material], bcs, 0.0, 1e30, 0.5, max_steps=steps, precision=msx.FP64)
    rep = S.run()
    u = S.state()[0]
    S.close()
    assert rep.steps == steps and rep.status == 0, rep
    return u


def accuracy_summary(cases, bar):
    e = [c["rel_l2_u_vs_fp64"] for c in cases]
    return {"solves_checked": len(e), "max_rel_l2_u_vs_fp64": max(e), "median_rel_l2_u_vs_fp64": float(np.median(e)),
            "bar": bar, "within_bar": bool(max(e) <= bar),
            "how": "each sampled solve re-run alone in the plain FP64 path for the same steps; relative L2 of u",
            "cases": cases}


def batched_variant(seed=7, count=256, steps=1000, warmup=3, precision=None, cache=None):
    """256 independent solves (cube side n log-uniform in [8, 48], E log-uniform
    in [1e5, 1e7], nu uniform in [0.25, 0.45], top velocity uniform in
    [0.01, 0.2]) stepped together by the pool, 1000 steps each: mixed (FP32
    elements, double-word nodes) by default, or another pool precision.  The
    timed region starts after admission, autotuning and warm-up and ends when
    the last solve's result is in host memory.  Afterwards a sample of the
    solves (largest and smallest n, extreme nu, seeded picks) runs alone in
    FP64 and the fetched displacements are compared with it."""
    import msx
    precision = msx.MIXED if precision is None else precision
    rng = np.random.default_rng(seed)
    ns = np.floor(np.exp(rng.uniform(np.log(8), np.log(49), count))).astype(int)
    Es = np.exp(rng.uniform(np.log(1e5), np.log(1e7), count))
    nus = rng.uniform(0.25, 0.45, count)
    vs = rng.uniform(0.01, 0.2, count)
    sample = accuracy_sample(ns, nus)

    def case(k):
        X, conn = msx.mesh_cube(int(ns[k]), SEED + k, 0.1)
        return X, conn, (1, float(Es[k]), float(nus[k]), 1000.0), \
            msx.cube_bcs(int(ns[k]), float(vs[k]), msx.BC_VEL_RAMP, RAMP_STEPS)

    cache = cache or TUNE_CACHE
    if os.path.exists(cache):
        os.remove(cache)
    P = msx.Pool(max_slots=count, precision=precision, steps_per_launch=32, tune_cache=cache)
    total_elems, owner = 0, {}
    t0 = time.perf_counter()
    for k in range(count):
        X, conn, mat, bcs = case(k)
        t = P.submit(X, conn, mat, bcs, steps)
        assert t is not None, "batched workload does not fit"
        owner[t] = k
        total_elems += conn.shape[0]
    admit_s = time.perf_counter() - t0
    P.step(warmup)   # autotunes the schedule on the resident work, then warms up
    before = P.stats()
    t1 = time.perf_counter()
    res, kept = [], {}
    while len(res) < count:
        P.step(steps)
        for r in P.poll():   # every result is read back to the host inside the timed region
            u = P.fetch(r["ticket"])[0]
            if owner[r["ticket"]] in sample:
                kept[owner[r["ticket"]]] = u
            res.append(r)
    wall = time.perf_counter() - t1
    after = P.stats()
    P.close()
    timed = after["element_steps"] - before["element_steps"]
    cases = []
    for k in sample:
        X, conn, mat, bcs = case(k)
        ref = fp64_alone(X, conn, mat, bcs, steps)
        cases.append({"solve": k, "n": int(ns[k]), "num_elems": int(conn.shape[0]), "E": float(Es[k]),
                      "nu": float(nus[k]), "v_top": float(vs[k]),
                      "rel_l2_u_vs_fp64": float(np.linalg.norm(kept[k] - ref) / max(np.linalg.norm(ref), 1e-300))})
    bar = 1e-10 if precision == msx.DOUBLE_WORD else 1e-5
    return {"value": timed / wall, "unit": "element-steps/s", "solves": count, "total_elems": int(total_elems),
            "steps_per_solve": steps, "wall_s": wall, "admit_s": admit_s,
            "all_ok": all(r["status"] == 0 and r["steps"] == steps for r in res),
            "accuracy": accuracy_summary(cases, bar),
            "schedule": {"threads": before["threads"], "tile_elems": before["tile_elems"],
                         "ctas_per_sm": before["ctas_per_sm"], "steps_per_graph": before["steps_per_launch"]}}


TUNE_CACHE = os.path.join(os.environ.get("TMPDIR", "/tmp"), "msx_pool_schedule.txt")


def serving_requests(lam, count, seed=11):
    """The seeded request stream of the serving configuration: Poisson
    arrivals at rate lam per second; cube side n log-uniform in [8, 64];
    compressible neo-Hookean with E log-uniform in [1e5, 1e7] and nu uniform
    in [0.25, 0.45]; top velocity uniform in [0.01, 0.2]; a step count uniform
    in [200, 2000]."""
    rng = np.random.default_rng(seed + int(lam))
    arrivals = np.cumsum(rng.exponential(1.0 / lam, count))
    ns = np.floor(np.exp(rng.uniform(np.log(8), np.log(65), count))).astype(int)
    steps = rng.integers(200, 2001, count)
    Es = np.exp(rng.uniform(np.log(1e5), np.log(1e7), count))
    nus = rng.uniform(0.25, 0.45, count)
    vs = rng.uniform(0.01, 0.2, count)
    return arrivals, ns, steps, Es, nus, vs


def serving_variant(lam, count=64, seed=11, max_slots=64, capacity=None):
    """Requests of serving_requests() arriving in real time are admitted into
    the pool as slots and HBM free up (continuous batching) while the pool's
    serving thread steps the resident solves.  Latency runs from a request's
    arrival to its result in host memory and is split into the wait before
    admission (the client building the request, then waiting for a slot) and
    the time in the pool (admission to completion, sharing the GPU).  The
    offered load is the requests' element-steps over their arrival span; with
    `capacity` (the batched rate of the same kernels) it is also given as a
    fraction of it, and a rate above it is marked saturated: its latencies
    then measure how fast the backlog drains.  A sample of the requests
    (largest n, extreme nu, seeded picks) is re-run alone in FP64."""
    import msx
    arrivals, ns, steps, Es, nus, vs = serving_requests(lam, count, seed)
    work = sum(6 * int(n) ** 3 * int(st) for n, st in zip(ns, steps))
    sample = accuracy_sample(ns, nus, seed=int(lam))

    def request(k):
        X, conn = msx.mesh_cube(int(ns[k]), SEED + 1000 + k, 0.1)
        return X, conn, (1, float(Es[k]), float(nus[k]), 1000.0), \
            msx.cube_bcs(int(ns[k]), float(vs[k]), msx.BC_VEL_RAMP, RAMP_STEPS), int(steps[k])

    # continuous batching in the pool: the library's serving thread steps it
    # while this thread builds and admits the arriving requests
    P = msx.Pool(max_slots=max_slots, precision=msx.MIXED, steps_per_launch=16, tune_cache=TUNE_CACHE)
    P.serve(True)
    start = time.perf_counter()
    nxt, owner, wait, inpool, kept, ready = 0, {}, {}, {}, {}, None
    while len(inpool) < count:
        if ready is None and nxt < count and arrivals[nxt] <= time.perf_counter() - start:
            ready = (nxt, request(nxt))
            nxt += 1
        admitted = False
        if ready is not None:
            t = P.submit(*ready[1])
            if t is not None:
                k = ready[0]
                owner[t] = k
                wait[k] = time.perf_counter() - start - arrivals[k]
                ready, admitted = None, True
        for r in P.poll():
            k = owner.pop(r["ticket"])
            inpool[k] = 1e-3 * r["latency_ms"]   # the pool's own admission-to-completion time
            u = P.fetch(r["ticket"])[0]
            if k in sample:
                kept[k] = u
        if not admitted:
            w = 0.001 if ready is not None or nxt >= count else arrivals[nxt] - (time.perf_counter() - start)
            time.sleep(max(0.0, min(0.001, w)))
    wall = time.perf_counter() - start
    P.close()
    W = np.array([wait[k] for k in range(count)]) * 1e3
    G = np.array([inpool[k] for k in range(count)]) * 1e3
    L = W + G
    offered = work / arrivals[-1]
    out = {"lambda_per_s": lam, "requests": count, "value": work / wall, "unit": "element-steps/s",
           "p50_ms": float(np.percentile(L, 50)), "p99_ms": float(np.percentile(L, 99)), "wall_s": wall,
           "arrival_span_s": float(arrivals[-1]), "offered_element_steps_per_s": offered,
           "wait_p50_ms": float(np.percentile(W, 50)), "wait_p99_ms": float(np.percentile(W, 99)),
           "in_pool_p50_ms": float(np.percentile(G, 50)), "in_pool_p99_ms": float(np.percentile(G, 99))}
    if capacity:
        out.update({"capacity_element_steps_per_s": capacity, "offered_fraction_of_capacity": offered / capacity,
                    "utilisation": (work / wall) / capacity, "saturated": bool(offered > capacity),
                    "capacity_note": "capacity = the batched mixed rate of the same kernels (variants.batched)"})
    cases = []
    for k in sample:
        X, conn, mat, bcs, st = request(k)
        ref = fp64_alone(X, conn, mat, bcs, st)
        cases.append({"request": k, "n": int(ns[k]), "num_elems": int(conn.shape[0]), "steps": st,
                      "nu": float(nus[k]), "E": float(Es[k]),
                      "rel_l2_u_vs_fp64": float(np.linalg.norm(kept[k] - ref) / max(np.linalg.norm(ref), 1e-300))})
    out["accuracy"] = accuracy_summary(cases, 1e-5)
    return out


def serving_sequential_fp64(lam, count=64, seed=11):
    """The same request stream served one solve at a time by the plain FP64 path."""
    import msx
    arrivals, ns, steps, Es, nus, vs = serving_requests(lam, count, seed)
    work = sum(6 * int(n) ** 3 * int(st) for n, st in zip(ns, steps))
    start = time.perf_counter()
    lat = []
    for k in range(count):
        now = time.perf_counter() - start
        if arrivals[k] > now:
            time.sleep(arrivals[k] - now)
        X, conn = msx.mesh_cube(int(ns[k]), SEED + 1000 + k, 0.1)
        S = msx.Solver(X, conn, [(1, float(Es[k]), float(nus[k]), 1000.0)],
                       msx.cube_bcs(int(ns[k]), float(vs[k]), msx.BC_VEL_RAMP, RAMP_STEPS), 0.0, 1e30, 0.5,
                       max_steps=int(steps[k]), precision=msx.FP64)
        S.run()
        S.state()
        S.close()
        lat.append((time.perf_counter() - start) - arrivals[k])
    wall = time.perf_counter() - start
    L = np.array(lat) * 1e3
    return {"lambda_per_s": lam, "requests": count, "value": work / wall, "unit": "element-steps/s",
            "p50_ms": float(np.percentile(L, 50)), "p99_ms": float(np.percentile(L, 99)), "wall_s": wall}


def precision_sweep(cube=N_CUBE, steps=5000, every=100):
    """Precision variant: the 6M-tet cube with St-Venant-Kirchhoff and
    compressible neo-Hookean, nu in {0.3, 0.45, 0.49}, 5000 steps, run side by
    side in the plain FP64 path and the mixed path (FP32 element kinematics,
    stress and B^T P; double-word nodal state; FP64 stable dt).  Every `every`
    steps: the relative L2 displacement error of the mixed run against the FP64
    run, and the largest von Mises difference over the largest von Mises
    stress.  The FP64 path stands in for the oracle here (it equals the oracle
    to ~1e-15 on this mesh after 2000 steps, tests/test_gpu_large.py; the CPU
    oracle needs ~0.1 s per step at this size)."""
    import msx
    X, conn = msx.mesh_cube(cube, SEED, 0.1)
    bcs = msx.cube_bcs(cube, V_TOP, msx.BC_VEL_RAMP, RAMP_STEPS)
    runs = []
    t0 = time.perf_counter()
    for law, lname in ((msx.STVK, "St-Venant-Kirchhoff"), (msx.COMPRESSIBLE_NH, "3D-Compressible-Neo-Hookean")):
        for nu in (0.3, 0.45, 0.49):
            mat = (law, 1e6, nu, 1000.0)
            A = msx.Solver(X, conn, [mat], bcs, 0.0, 1e30, 0.5, max_steps=steps, precision=msx.FP64)
            B = msx.Solver(X, conn, [mat], bcs, 0.0, 1e30, 0.5, max_steps=steps, precision=msx.MIXED)
            eu, ev, done, same_t = [], [], 0, True
            while done < steps:
                k = min(every, steps - done)
                ra, rb = A.run(k), B.run(k)
                assert ra.steps == k and rb.steps == k and ra.status == 0 and rb.status == 0, (ra, rb)
                done += k
                same_t &= abs(ra.t - rb.t) <= 1e-9 * abs(ra.t)
                ua, ub = A.state()[0], B.state()[0]
                eu.append(float(np.linalg.norm(ub - ua) / max(np.linalg.norm(ua), 1e-300)))
                va, vb = A.von_mises(), B.von_mises()
                ev.append(float(np.abs(vb - va).max() / max(np.abs(va).max(), 1e-300)))
            A.close()
            B.close()
            runs.append({"law": lname, "nu": nu, "max_rel_l2_u": max(eu), "final_rel_l2_u": eu[-1],
                         "max_rel_vms": max(ev), "final_rel_vms": ev[-1], "times_agree_1e-9": bool(same_t),
                         "rel_l2_u_every": [float("%.3g" % x) for x in eu],
                         "rel_vms_every": [float("%.3g" % x) for x in ev]})
    return {"num_elems": int(conn.shape[0]), "steps": steps, "every": every, "bar": 1e-5,
            "worst_rel_l2_u": max(r["max_rel_l2_u"] for r in runs),
            "worst_rel_vms": max(r["max_rel_vms"] for r in runs),
            "within_bar": bool(max(max(r["max_rel_l2_u"], r["max_rel_vms"]) for r in runs) <= 1e-5),
            "wall_s": time.perf_counter() - t0,
            "vms_metric": "max over elements |vm_mixed - vm_fp64| / max over elements |vm_fp64|",
            "runs": runs}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def reduce_max(x, ws):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-variants", action="store_true")
    ap.add_argument("--no-pool", action="store_true", help="skip the batched and serving variants")
    ap.add_argument("--no-sweep", action="store_true", help="skip the precision sweep (6 x 5000 steps)")
    ap.add_argument("--sweep-steps", type=int, default=5000)
    ap.add_argument("--cube", type=int, default=N_CUBE, help="hexes per cube edge (profiling runs only)")
    ap.add_argument("--only", choices=["fp64", "mixed", "fp64_exact", "dword"], default=None,
                    help="time a single variant (profiling runs only)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")

    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(reference_arm(args)))
        return
    import msx

    msx.load()
    msx.set_device(local)
    X, conn, bcs = make_case(args.cube)
    ne, nn = conn.shape[0], X.shape[1]

    barrier(ws)
    first = {"mixed": msx.MIXED, "fp64_exact": msx.FP64_EXACT, "dword": msx.DOUBLE_WORD}.get(args.only, msx.FP64)
    rep, prof, clocks, u_first = run_variant(X, conn, bcs, first, args.steps, args.warmup, local, keep_u=True)
    secs = reduce_max(rep.device_ms / 1e3, ws)
    value = ws * ne * args.steps / secs

    variants = {}
    if not args.no_variants and args.only is None:
        for name, prec in (("mixed", msx.MIXED), ("double_word", msx.DOUBLE_WORD), ("fp64_exact", msx.FP64_EXACT)):
            r2, p2, c2, u2 = run_variant(X, conn, bcs, prec, args.steps, args.warmup, local, keep_u=True)
            s2 = reduce_max(r2.device_ms / 1e3, ws)
            variants[name] = {"value": ws * ne * args.steps / s2, "ms_per_step": 1e3 * s2 / args.steps,
                              "element_kernel_ms": p2.element_ms, "node_kernel_ms": p2.node_ms,
                              "clocks": c2,
                              # error against the plain FP64 run at the same step (FP64 equals the
                              # oracle to ~1e-15 on this mesh: tests/test_gpu_large.py)
                              "rel_l2_u_vs_fp64": float(np.linalg.norm(u2 - u_first) /
                                                        max(np.linalg.norm(u_first), 1e-300))}
            if name == "mixed":
                variants[name]["roofline"] = mixed_roofline(ne, nn, p2, 1e3 * s2 / args.steps)
            if name == "double_word":
                variants[name]["roofline"] = dword_roofline(ne, nn, p2, 1e3 * s2 / args.steps)
    if not args.no_pool and args.only is None and args.cube == N_CUBE:
        variants["batched"] = batched_variant()
        variants["batched_double_word"] = batched_variant(precision=msx.DOUBLE_WORD, cache=TUNE_CACHE + ".dw")
        cap = variants["batched"]["value"]
        # lambda = 50 per s is below the pool's capacity: 500 requests (~10 s of
        # arrivals) give steady-state latencies; 200 and 800 per s exceed it
        variants["serving"] = [serving_variant(50, count=500, capacity=cap)] + \
            [serving_variant(lam, capacity=cap) for lam in (200, 800)]
        variants["serving_one_at_a_time_fp64"] = serving_sequential_fp64(200)
    if not args.no_sweep and args.only is None and args.cube == N_CUBE:
        variants["precision_sweep"] = precision_sweep(steps=args.sweep_steps)
    e2e = None
    if not args.no_e2e and args.only is None:
        # three whole jobs; the median wall time (one job is a few tens of ms,
        # so a single sample carries the host's scheduling noise)
        walls = []
        for _ in range(3):
            wall, r3, h2d, d2h = run_e2e(X, conn, bcs, args.steps)
            walls.append(reduce_max(wall, ws))
        wall = statistics.median(walls)
        e2e = {"value": ws * ne * args.steps / wall, "unit": "element-steps/s",
               "h2d_bytes_per_step": h2d / args.steps, "d2h_bytes_per_step": d2h / args.steps,
               "h2d_bytes_total": h2d, "d2h_bytes_total": d2h, "wall_s": wall, "wall_s_runs": walls,
               "note": "msx_create (mesh upload + set-up) + msx_run(K) + msx_get_state, host buffers; "
                       "median of 3 jobs"}
    if rank != 0:
        return
    peak, peak_kind = peaks()
    # algorithmic bytes: per element conn 16 + dphi/dX 96 + wJ 8 + reference length 8 = 128 B;
    # per node X, u, v, a, m read and u, v, a written = 176 B
    alg_elem = 128.0 * ne
    alg_step = 128.0 * ne + 176.0 * nn
    achieved = alg_elem / (prof.element_ms * 1e-3) / 1e9
    tr = profiled("dram_bytes_per_element")
    ops = profiled("fp64_ops_per_element")
    opk, opk_kind = fp64_peak()
    step_gbs = alg_step / (secs / args.steps) / 1e9
    roofline = {"bound": "hbm", "kernel": "pool_elem_kernel<FP64>", "achieved": achieved, "peak": peak,
                "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
                "traffic": tr * ne if tr else None,
                "alg_bytes_per_launch": alg_elem, "element_kernel_ms": prof.element_ms,
                "node_kernel_ms": prof.node_ms,
                "step": {"alg_bytes": alg_step, "achieved": step_gbs, "frac": step_gbs / peak,
                         "note": "whole step (element + node kernel): 128 B per element + 176 B per node"},
                "fp64_pipe": None if not ops else {
                    "achieved_gops": ops * ne / (prof.element_ms * 1e-3) / 1e9, "peak_gops": opk,
                    "frac": ops * ne / (prof.element_ms * 1e-3) / 1e9 / opk, "ops_per_element": ops,
                    "peak_kind": opk_kind,
                    "note": "FP64 ops/element from ncu counters (profiles/ncu_figures.json); peak: DFMA "
                            "rate with eight independent chains per thread on this GPU (msx_fp64_peak)"},
                "note": "the kernel is bound by the FP64 pipe, not by HBM; both fractions are reported"}
    # a profiling run of one other precision reports that precision's kernel
    if args.only == "mixed":
        roofline = mixed_roofline(ne, nn, prof, 1e3 * secs / args.steps)
    elif args.only == "dword":
        roofline = dword_roofline(ne, nn, prof, 1e3 * secs / args.steps)
    elif args.only == "fp64_exact":
        roofline = dict(roofline, kernel="elem_kernel_exact_screened", traffic=None, fp64_pipe=None,
                        note="reference operation order; no ncu figures for this kernel")
    dtype = {"mixed": "f32 elements, f32x2 nodes", "dword": "f32x2"}.get(args.only, "f64")
    line = {"metric": METRIC, "value": value, "unit": "element-steps/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": dtype, "data": "synthetic",
            "config": {"workload": WORKLOAD, "num_elems": ne, "num_nodes": nn,
                       "precision": {"mixed": "MIXED", "fp64_exact": "FP64_EXACT", "dword": "DOUBLE_WORD"}.get(
                           args.only, "FP64"),
                       "parallelism": "replicas" if ws > 1 else "single", "l2": "inputs larger than L2 "
                       "(element arrays %.2f GB resident)" % (ne * 128 / 1e9)},
            "roofline": roofline, "gpu_launches": rep.kernel_launches, "clocks": clocks, "e2e": e2e,
            "variants": variants}
    if not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(X, conn, bcs)
    print(json.dumps(line))


if __name__ == "__main__":
    main()
