#!/usr/bin/env python3
"""Benchmark of the GPU Voronoi vertex search (HighVoronoi.jl hot path).

Workload (one "step"): the full vertex search of a 4D mesh of N=20,000 points
i.i.d. uniform in [0,1]^4 (seed 1), cuboid(4, periodic=[]) boundary, no
integrator -- the configuration of the reference's 4D table
(docs/src/index.md:93).  Metric: Voronoi vertices per second.

  value      vertices/s with the points already resident in HBM
             (hv_mesh_build_device; sort, tree, candidate lists, seeds,
             wavefront and canonical renumbering all inside the step);
             L2 is flushed (256 MiB write) before every timed step.
  e2e        the same metric through the C ABI with host buffers: pinned
             host points -> hv_mesh_build -> hv_mesh_counts -> hv_mesh_vertices
             into pinned host arrays (signatures + coordinates).
  roofline   the dominant kernel (wavefront expansion), timed by the library
             with CUDA events on its own stream.
  --impl reference  the reference's algorithm on the host cores (the C++
             restatement in oracle/, since the Julia reference cannot run here).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "highvoronoi.jl_gb300"))

import numpy as np  # noqa: E402

METRIC = "Voronoi vertices/s"
UNIT = "vertices/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--method", choices=["fast", "plain"], default="fast")
    ap.add_argument("--workload", default="4d_uniform_20k")
    ap.add_argument("--n", type=int, default=0, help="override the point count (profiling cases)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--cpu-cells", type=int, default=0, help="cells per CPU sample (0 = all)")
    ap.add_argument("--serve", action="store_true", help="only the served-stream measurement")
    ap.add_argument("--serve-requests", type=int, default=2000)
    ap.add_argument("--serve-rate", type=float, default=200.0)
    ap.add_argument("--serve-slots", type=int, default=8)
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--no-serve-capacity", action="store_true", help="skip the unbounded-rate serving run")
    ap.add_argument("--no-autotune", action="store_true", help="skip the autotuned 5D clustered build")
    ap.add_argument("--serve-integrator", choices=["polygon", "none"], default="polygon")
    ap.add_argument("--no-integrators", action="store_true")
    ap.add_argument("--knn", type=int, default=0, help="candidate list length (0 = library default)")
    ap.add_argument("--leaf-size", type=int, default=0, help="tree leaf size (0 = library default)")
    ap.add_argument("--seed-stride", type=int, default=0, help="one descent seed per this many generators (0 = default)")
    ap.add_argument("--mc-dirs", type=int, default=1000, help="directions per cell of VI_HEURISTIC_MC")
    ap.add_argument("--no-c3", action="store_true", help="skip the 5D clustered 50k, 2D 1k and 6D 10k measurements")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain FP64 arm of the 5D measurement")
    ap.add_argument("--no-lattice", action="store_true", help="skip the 3D lattice (co-spherical generators)")
    return ap.parse_args()


def workload(args):
    from hvgpu import datasets as D
    w = dict(D.WORKLOADS[args.workload])
    if args.n:
        w["n"] = args.n
    if w["kind"] == "uniform":
        pts = D.uniform_points(w["d"], w["n"], w["seed"])
    else:
        pts = D.clustered_points(w["d"], w["n"], w["seed"])
    cfg = {"workload": f"{w['d']}d_{w['kind']}_{w['n']}_vertex_search", "d": w["d"], "n_points": w["n"],
           "seed": w["seed"], "boundary": "cuboid(d, periodic=[])", "integrator": None}
    return pts, cfg


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def aggregate_over_ranks(tot_ms, units, device):
    """Whole-job numbers of the replicas: the MAX over ranks of the timed
    milliseconds and the SUM of the units (vertices) they processed, over the
    default process group (nccl on the GPUs, gloo in the CPU tests)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(tot_ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    u = torch.tensor([float(units)], dtype=torch.float64, device=device)
    dist.all_reduce(u)
    return float(t.item()), int(round(u.item()))


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.flush()
        self.f.seek(0)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.f.name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def ncu_traffic_per_vertex():
    """Per-vertex DRAM traffic of the expansion kernel from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "ncu_expand_fast_traffic.json")
    try:
        with open(p) as f:
            return json.load(f)
    except Exception:
        return None


def cpu_baseline(pts, cells, threads):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    own, rays, sec = O.sample_cells(pts, cells, nthreads=threads)
    return own, rays, sec


def serve_requests(count, seed=2000):
    """The served stream (hvgpu.datasets.served_stream): request r has d uniform
    in {2,3,4,5}, N log-uniform in [200, 20000] and points uniform in the unit
    cube drawn with seed r; arrival gaps are exponential with unit mean."""
    from hvgpu import datasets as D
    return D.served_stream(count, seed)


def run_serve(args, device):
    """The served stream twice: once at the offered Poisson rate (latency
    percentiles of that load) and once with every request queued at the start
    (the sustainable rate of the device, meshes per second)."""
    from hvgpu import datasets as D
    from hvgpu.serve import Server
    reqs, gaps = serve_requests(args.serve_requests)
    pts = [D.uniform_points(d, n, r) for d, n, r in reqs]
    integ = None if args.serve_integrator == "none" else args.serve_integrator

    def stream(arrivals):
        with Server(device=device, slots=args.serve_slots) as srv:
            for d in (2, 3, 4, 5):  # warm-up: one request per dimension
                srv.result(srv.submit(D.uniform_points(d, 500, 10 ** 6 + d), integrator=integ))
            t0 = time.perf_counter()
            tickets, t_sub = [], []
            for p, ta in zip(pts, arrivals):
                now = time.perf_counter() - t0
                if ta > now:
                    time.sleep(ta - now)
                tickets.append(srv.submit(p, integrator=integ))
                t_sub.append(time.perf_counter() - t0)
            # the results are copied out after the stream; each request's completion
            # is its submission plus its latency on the server's clock
            lat, svc, fails, verts, t_end = [], [], 0, 0, 0.0
            for t, ts in zip(tickets, t_sub):
                r = srv.result(t)
                if r["status"] != 0:
                    fails += 1
                    continue
                lat.append(r["latency_ms"])
                svc.append(r["service_ms"])
                verts += len(r["sig"])
                t_end = max(t_end, ts + r["latency_ms"] / 1e3)
        return np.array(lat), np.array(svc), fails, verts, t_end

    lat, svc, fails, verts, t_end = stream(np.cumsum(gaps / args.serve_rate))
    out = {"requests": len(reqs), "rate_per_s": args.serve_rate, "slots": args.serve_slots, "failures": fails,
           "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
           "mean_ms": float(lat.mean()), "meshes_per_s": len(lat) / t_end, "vertices": int(verts),
           "service_p50_ms": float(np.percentile(svc, 50)), "service_p99_ms": float(np.percentile(svc, 99)),
           "service_max_ms": float(svc.max()),
           "config": "d uniform {2,3,4,5}, N log-uniform [200,20000], uniform points seed=request id, "
                     "cuboid(d, periodic=[]), " + ("VI_POLYGON" if integ else "no integrator") +
                     ", Poisson arrivals"}
    if not args.no_serve_capacity:
        clat, _, cfails, _, ct = stream(np.zeros(len(pts)))
        cap = len(clat) / ct
        out["capacity"] = {"meshes_per_s": cap, "failures": cfails, "seconds": ct,
                           "note": "all requests queued at t=0: the sustainable rate (to the last completion)"}
        # the same stream offered at 85% of that rate: latencies of the service, not of a growing queue
        rate = 0.85 * cap
        slat, ssvc, sfails, _, st_end = stream(np.cumsum(gaps / rate))
        out["at_85pct_capacity"] = {"rate_per_s": rate, "p50_ms": float(np.percentile(slat, 50)),
                                    "p99_ms": float(np.percentile(slat, 99)), "mean_ms": float(slat.mean()),
                                    "meshes_per_s": len(slat) / st_end, "failures": sfails,
                                    "service_p99_ms": float(np.percentile(ssvc, 99)),
                                    "service_max_ms": float(ssvc.max())}
    return out


def fp32_peak_tflops(local, clocks):
    """Nominal FP32 rate: SMs x 128 FP32 lanes x 2 flops x max SM clock."""
    import torch
    prop = torch.cuda.get_device_properties(local)
    fmax = (clocks or {}).get("sm_max_mhz") or 2070.0
    return prop.multi_processor_count * 128 * 2 * fmax * 1e6 / 1e12


FP64_PEAK_TFLOPS = 1.25  # nominal GB300 FP64 rate; no measured FP64 peak exists for this machine


def run_lattice(ctx, flush):
    """Co-spherical generators: a 3D lattice of 32^3 points (8 on every interior
    vertex's sphere) -- the search meets the ties and walks the vertex graph
    with vertices of any size; build and VI_POLYGON times, CUDA events."""
    import torch
    import hvgpu
    k, d = 32, 3
    g = (np.arange(k) + 0.5) / k
    pts = np.ascontiguousarray(np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, d))
    lo, hi = np.zeros(d), np.ones(d)
    prm = hvgpu.make_params(hvgpu.HV_METHOD_FAST)
    hvgpu.Mesh(ctx, pts, lo, hi, prm).free()  # warm-up
    times, ptimes = [], []
    for _ in range(3):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        m = hvgpu.Mesh(ctx, pts, lo, hi, prm)
        times.append((time.perf_counter() - t0) * 1e3)
        t1 = time.perf_counter()
        vol, _ = m.polygon()
        ptimes.append((time.perf_counter() - t1) * 1e3)
        V = m.counts()[0]
        mx = m.max_signature()
        m.free()
    ms = statistics.median(times)
    return {"workload": "3d_lattice_32", "n_points": int(len(pts)), "vertices": int(V), "max_signature": int(mx),
            "ms_build": ms, "vertices_per_s": V / (ms / 1e3), "ms_polygon": statistics.median(ptimes),
            "volume_sum": float(vol.sum()), "timing": "host wall clock of hv_mesh_build (fast search until the "
            "first tie, then the generic walk) and of hv_integrate_polygon"}


def run_c3(args, ctx, local, flush, clocks):
    """The 5D clustered N=50,000 mesh (seed 2): the batched split-precision
    search against the plain one-ray-per-thread FP64 search and the host CPU,
    then VI_POLYGON and VI_HEURISTIC_MC (1,000 directions per cell) on the GPU
    and the same phases in the CPU oracle."""
    import torch
    import hvgpu
    from hvgpu import datasets as D
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    name = "5d_clustered_50k"
    w = D.WORKLOADS[name]
    pts = D.workload_points(name)
    n, d = pts.shape
    lo, hi = np.zeros(d), np.ones(d)
    dev_pts = torch.from_numpy(np.ascontiguousarray(pts)).cuda()
    stream = torch.cuda.ExternalStream(ctx.stream())
    out = {"workload": f"{d}d_clustered_{n}", "d": d, "n_points": n, "seed": w["seed"],
           "boundary": "cuboid(d, periodic=[])", "l2": "flushed (256 MiB write) before every timed step"}

    def timed(params, steps, warm):
        for _ in range(warm):
            hvgpu.Mesh(ctx, np.array([n, d]), lo, hi, params, device_ptr=dev_pts.data_ptr()).free()
        tot, verts, sts = 0.0, 0, []
        for _ in range(steps):
            flush.zero_()
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            m = hvgpu.Mesh(ctx, np.array([n, d]), lo, hi, params, device_ptr=dev_pts.data_ptr())
            e1.record(stream)
            torch.cuda.synchronize()
            tot += e0.elapsed_time(e1)
            st = m.stats()
            sts.append(st)
            verts += st["vertices"]
            m.free()
        return verts / (tot / 1e3), tot / steps, sts

    steps = max(1, min(args.steps, 5))
    fv, fms, fst = timed(hvgpu.make_params(hvgpu.HV_METHOD_FAST), steps, max(args.warmup, 3))
    st0 = fst[-1]
    V = st0["vertices"]
    out["fast"] = {"vertices_per_s": fv, "ms_per_step": fms, "steps": steps, "vertices": V,
                   "rays_per_s": st0["rays"] / (fms / 1e3), "levels": st0["levels"],
                   "breakdown_ms": {k: statistics.mean(s[k] for s in fst) for k in
                                    ("ms_prepare", "ms_knn", "ms_descent", "ms_expand", "ms_fallback",
                                     "ms_centers", "ms_canonical")}}
    if not args.no_autotune:
        # hv_autotune on these points (candidate-list length, leaf size, seed stride), then the
        # same timed build with the winner; the vertex set does not depend on the knobs
        tuned = ctx.autotune(d, n, pts=pts, lo=lo, hi=hi)
        tv, tms, tst = timed(hvgpu.make_params(**tuned), steps, 2)
        assert tst[-1]["vertices"] == V
        out["autotuned"] = {"vertices_per_s": tv, "ms_per_step": tms, "steps": steps,
                            "params": {k: tuned[k] for k in ("knn", "leaf_size", "seed_stride")},
                            "over_defaults": tv / fv}
    if not args.no_plain:
        pv, pms, pst = timed(hvgpu.make_params(hvgpu.HV_METHOD_PLAIN), 1, 0)
        assert pst[-1]["vertices"] == V
        out["plain"] = {"vertices_per_s": pv, "ms_per_step": pms, "steps": 1,
                        "method": "one ray per thread, FP64 shrinking-ball tree search from the root"}
        out["fast_over_plain"] = fv / pv
    # roofline: FP32 issue pipe for the candidate scan, FP64 pipe for the centres
    m = hvgpu.Mesh(ctx, np.array([n, d]), lo, hi, hvgpu.make_params(hvgpu.HV_METHOD_FAST),
                   device_ptr=dev_pts.data_ptr())
    offs, nbr = m.neighbors()
    nbar = len(nbr) / n
    p32 = fp32_peak_tflops(local, clocks)
    exp_ms = out["fast"]["breakdown_ms"]["ms_expand"]
    f32 = V * nbar * (5 * d + 3)
    cen_ms = out["fast"]["breakdown_ms"]["ms_centers"]
    f64 = V * ((2.0 / 3.0) * d ** 3 + 4 * d * d)
    out["roofline"] = {
        "k_expand_fast": {"bound": "fp32", "unit": "TFLOP/s", "algorithmic_flops_per_vertex": nbar * (5 * d + 3),
                          "achieved": f32 / (exp_ms / 1e3) / 1e12, "peak": p32,
                          "frac": f32 / (exp_ms / 1e3) / 1e12 / p32, "peak_source": "nominal"},
        "k_centers": {"bound": "fp64", "unit": "TFLOP/s", "algorithmic_flops_per_vertex": (2.0 / 3.0) * d ** 3 + 4 * d * d,
                      "achieved": f64 / (cen_ms / 1e3) / 1e12, "peak": FP64_PEAK_TFLOPS,
                      "frac": f64 / (cen_ms / 1e3) / 1e12 / FP64_PEAK_TFLOPS, "peak_source": "nominal"}}
    # integrators on the same mesh, outputs in HBM (hv_integrate_*_device)
    dvol = torch.empty(n, dtype=torch.float64, device="cuda")
    darea = torch.empty(max(len(nbr), 1), dtype=torch.float64, device="cuda")
    integ = {}
    for key, fn in (("polygon", lambda: m.polygon_device(dvol.data_ptr(), darea.data_ptr())),
                    ("heuristic_mc", lambda: m.heuristic_mc_device(args.mc_dirs, 7, dvol.data_ptr(),
                                                                    darea.data_ptr()))):
        fn()
        ts = []
        for _ in range(max(1, min(args.steps, 3))):
            flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            fn()
            ts.append(time.perf_counter() - t0)
        integ[key] = {"ms": 1e3 * statistics.mean(ts), "cells_per_s": n / statistics.mean(ts)}
    st = m.stats()
    poly_dev_ms = st["ms_poly_incidence"] + st["ms_poly_facets"] + st["ms_poly_big"]
    integ["polygon"].update({"device_ms": poly_dev_ms, "ms_lattice_build": st["ms_poly_incidence"],
                             "ms_terms": st["ms_poly_facets"], "faces": st["poly_faces"],
                             "terms": st["poly_terms"]})
    # the reference decomposition's flag count (sum over cells of E_cell (d-1)! 2 d^2,
    # E_cell = d V_cell / 2, sum V_cell = (d+1) V): the work the reference's
    # integrator would do, per second of this one
    ref_flops = d * (d + 1) * V / 2.0 * math.factorial(d - 1) * 2 * d * d
    integ["polygon"]["reference_flag_flops"] = ref_flops
    integ["polygon"]["reference_equivalent_tflops"] = ref_flops / (poly_dev_ms / 1e3) / 1e12
    tf = st["poly_term_flops"]
    out["roofline"]["k_lat_terms"] = {
        "bound": "fp64", "unit": "TFLOP/s", "algorithmic_flops": tf,
        "achieved": tf / (st["ms_poly_facets"] / 1e3) / 1e12, "peak": FP64_PEAK_TFLOPS,
        "frac": tf / (st["ms_poly_facets"] / 1e3) / 1e12 / FP64_PEAK_TFLOPS, "peak_source": "nominal",
        "note": "one term per face and sub-face of the mesh-wide face lattice (pulling decomposition), "
                "FP64 operations counted per term, over the term kernels' device time"}
    integ["heuristic_mc"]["directions_per_cell"] = args.mc_dirs
    m.free()
    # the host CPU on the same phases (the oracle, OpenMP on every host core)
    if not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        cells = np.arange(0, n, 20)
        own, rays, sec = O.sample_cells(pts, cells, nthreads=threads)
        out["cpu_baseline"] = {"value": own / sec, "unit": UNIT, "cores": threads, "kind": "port",
                               "sample": f"per-cell search of {len(cells)} of the {n} cells (every 20th), vertices "
                                         f"owned per second (C++ restatement of the reference algorithm, OpenMP)"}
        out["fast_over_cpu"] = fv / (own / sec)
        pc = np.arange(0, n, 100)
        t0 = time.perf_counter()
        O.polygon_cells(pts, pc, nthreads=threads)
        tp = time.perf_counter() - t0
        integ["polygon"]["cpu"] = {"cells_per_s": len(pc) / tp, "cores": threads, "kind": "port",
                                   "sample": f"{len(pc)} of the {n} cells (every 100th), each cell's search and "
                                             f"flag-decomposition integral"}
        ref = O.OracleMesh(pts, csr=(offs, nbr))
        t0 = time.perf_counter()
        ref.heuristic_mc(args.mc_dirs, 7, nthreads=threads)
        tm = time.perf_counter() - t0
        integ["heuristic_mc"]["cpu"] = {"cells_per_s": n / tm, "ms": 1e3 * tm, "cores": threads, "kind": "port",
                                        "sample": f"all {n} cells on the GPU's neighbour lists, "
                                                  f"{args.mc_dirs} directions per cell"}
    out["integrators"] = integ
    return out


def run_small(args, ctx, flush, name, integrator):
    """A contract workload beside the headline (2D uniform 1k with VI_POLYGON,
    6D uniform 10k with VI_HEURISTIC_MC at --mc-dirs directions): the build
    (CUDA events, L2 flushed), its integrator (host wall clock through the C
    ABI, outputs copied) and the CPU oracle on bounded samples of both phases."""
    import torch
    import hvgpu
    from hvgpu import datasets as D
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    w = D.WORKLOADS[name]
    pts = D.workload_points(name)
    n, d = pts.shape
    lo, hi = np.zeros(d), np.ones(d)
    dev_pts = torch.from_numpy(np.ascontiguousarray(pts)).cuda()
    stream = torch.cuda.ExternalStream(ctx.stream())
    prm = hvgpu.make_params(hvgpu.HV_METHOD_FAST)
    out = {"workload": name, "d": d, "n_points": n, "seed": w["seed"], "boundary": "cuboid(d, periodic=[])",
           "l2": "flushed (256 MiB write) before every timed build"}
    for _ in range(max(args.warmup, 3)):
        hvgpu.Mesh(ctx, np.array([n, d]), lo, hi, prm, device_ptr=dev_pts.data_ptr()).free()
    steps = max(1, min(args.steps, 10))
    tot, V = 0.0, 0
    for _ in range(steps):
        flush.zero_()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        m = hvgpu.Mesh(ctx, np.array([n, d]), lo, hi, prm, device_ptr=dev_pts.data_ptr())
        e1.record(stream)
        torch.cuda.synchronize()
        tot += e0.elapsed_time(e1)
        V = m.stats()["vertices"]
        m.free()
    gv = V * steps / (tot / 1e3)
    out["build"] = {"vertices": V, "ms_per_step": tot / steps, "vertices_per_s": gv, "steps": steps}
    m = hvgpu.Mesh(ctx, np.array([n, d]), lo, hi, prm, device_ptr=dev_pts.data_ptr())
    fn = (lambda: m.polygon()) if integrator == "polygon" else (lambda: m.heuristic_mc(args.mc_dirs, 7))
    for _ in range(3):
        fn()
    ts = []
    for _ in range(steps):
        t0 = time.perf_counter()
        fn()
        ts.append(time.perf_counter() - t0)
    out[integrator] = {"ms": 1e3 * statistics.mean(ts), "cells_per_s": n / statistics.mean(ts)}
    if integrator == "heuristic_mc":
        out[integrator]["directions_per_cell"] = args.mc_dirs
    offs, nbr = m.neighbors()
    m.free()
    if not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        every = max(1, n // 200)
        cells = np.arange(0, n, every)
        own, rays, sec = O.sample_cells(pts, cells, nthreads=threads)
        out["build"]["cpu"] = {"value": own / sec, "unit": UNIT, "cores": threads, "kind": "port",
                               "sample": f"per-cell search of {len(cells)} of the {n} cells (every {every}th), "
                                         f"vertices owned per second"}
        out["build"]["gpu_over_cpu"] = gv / (own / sec)
        if integrator == "polygon":
            t0 = time.perf_counter()
            O.polygon_cells(pts, cells, nthreads=threads)
            tp = time.perf_counter() - t0
            out[integrator]["cpu"] = {"cells_per_s": len(cells) / tp, "cores": threads, "kind": "port",
                                      "sample": f"{len(cells)} of the {n} cells, each cell's search and "
                                                f"flag-decomposition integral"}
        else:
            # the sampled cells keep their neighbour lists (the GPU's), the others none
            keep = np.zeros(n, dtype=bool)
            keep[cells] = True
            cnt = np.where(keep, np.diff(offs), 0)
            soffs = np.concatenate([[0], np.cumsum(cnt)]).astype(offs.dtype)
            snbr = np.concatenate([nbr[offs[i]:offs[i + 1]] for i in cells]).astype(nbr.dtype)
            ref = O.OracleMesh(pts, csr=(soffs, snbr))
            t0 = time.perf_counter()
            ref.heuristic_mc(args.mc_dirs, 7, nthreads=threads)
            tm = time.perf_counter() - t0
            out[integrator]["cpu"] = {"cells_per_s": len(cells) / tm, "cores": threads, "kind": "port",
                                      "sample": f"{len(cells)} of the {n} cells (every {every}th) on the GPU's "
                                                f"neighbour lists, {args.mc_dirs} directions per cell"}
        out[integrator]["gpu_over_cpu"] = out[integrator]["cells_per_s"] / out[integrator]["cpu"]["cells_per_s"]
    return out


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    pts, cfg = workload(args)
    n = pts.shape[0]
    threads = os.cpu_count() or 1
    ncell = args.cpu_cells or min(n, 4000)
    cells = np.arange(0, n, max(1, n // ncell))[:ncell]
    for _ in range(args.warmup):
        cpu_baseline(pts, cells, threads)
    tot_v, tot_s = 0, 0.0
    for _ in range(args.steps):
        own, rays, sec = cpu_baseline(pts, cells, threads)
        tot_v += own
        tot_s += sec
    value = tot_v / tot_s
    sample = (f"per-cell search of {len(cells)} of the {n} cells (every {max(1, n // ncell)}th), vertices owned "
              f"by the sampled cells per second; C++ restatement of the reference algorithm, OpenMP")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot_s / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": cfg,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch
    import hvgpu
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    ctx = hvgpu.Context(local)
    pts, cfg = workload(args)
    n, d = pts.shape
    lo, hi = np.zeros(d), np.ones(d)
    method = hvgpu.HV_METHOD_FAST if args.method == "fast" else hvgpu.HV_METHOD_PLAIN
    knobs = {k: v for k, v in (("knn", args.knn), ("leaf_size", args.leaf_size), ("seed_stride", args.seed_stride)) if v}
    params = hvgpu.make_params(method, **knobs)
    if knobs:
        cfg["params"] = knobs
    dev_pts = torch.from_numpy(np.ascontiguousarray(pts)).cuda()
    stream = torch.cuda.ExternalStream(ctx.stream())
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def build_dev():
        return hvgpu.Mesh(ctx, np.array([n, d]), lo, hi, params, device_ptr=dev_pts.data_ptr())

    for _ in range(max(args.warmup, 3)):
        m = build_dev()
        V = m.stats()["vertices"]
        m.free()
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    clk = ClockSampler(local)
    clk.start()
    tot_ms, verts, stats = 0.0, 0, []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        m = build_dev()
        e1.record(stream)
        torch.cuda.synchronize()
        tot_ms += e0.elapsed_time(e1)
        st = m.stats()
        stats.append(st)
        verts += st["vertices"]
        m.free()
    clocks = clk.stop()
    if ws > 1:
        torch.distributed.barrier()
        tot_ms, verts = aggregate_over_ranks(tot_ms, verts, "cuda")
    value = verts / (tot_ms / 1e3)
    # ---- the two integrators on the same mesh (host wall clock through the C ABI, outputs copied back)
    integ = None
    if not args.no_integrators and ws == 1:
        m = build_dev()
        integ = {}
        for name, fn in (("polygon", lambda: m.polygon()),
                         ("heuristic_mc", lambda: m.heuristic_mc(args.mc_dirs, 7))):
            for _ in range(max(args.warmup, 3)):
                fn()
            ts = []
            for _ in range(args.steps):
                flush.zero_()
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                fn()
                ts.append(time.perf_counter() - t0)
            t = statistics.mean(ts)
            integ[name] = {"ms": 1e3 * t, "cells_per_s": n / t}
        st = m.stats()
        integ["polygon"].update({"ms_lattice_build": st["ms_poly_incidence"], "ms_terms": st["ms_poly_facets"],
                                 "faces": st["poly_faces"], "terms": st["poly_terms"]})
        integ["heuristic_mc"]["directions_per_cell"] = args.mc_dirs
        m.free()
    # ---- end to end through the C ABI with host buffers
    e2e = None
    if not args.no_e2e:
        host_pts = torch.from_numpy(np.ascontiguousarray(pts)).pin_memory().numpy()
        sig_buf = torch.empty((V, d + 1), dtype=torch.int64).pin_memory().numpy()
        r_buf = torch.empty((V, d), dtype=torch.float64).pin_memory().numpy()
        L = hvgpu.load()
        e2e_s, e2e_v = 0.0, 0
        for it in range(args.warmup + args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            m = hvgpu.Mesh(ctx, host_pts, lo, hi, params)
            nv, _ = m.counts()
            if nv > sig_buf.shape[0]:
                sig_buf = np.zeros((nv, d + 1), dtype=np.int64)
                r_buf = np.zeros((nv, d))
            ctx.check(L.hv_mesh_vertices(m._h, hvgpu._lib.iptr(sig_buf), hvgpu._lib.dptr(r_buf)), "vertices")
            t1 = time.perf_counter()
            m.free()
            if it >= args.warmup:
                e2e_s += t1 - t0
                e2e_v += nv
        e2e = {"value": e2e_v / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(n * d * 8),
               "d2h_bytes_per_step": int(V * (d + 1) * 8 + V * d * 8),
               "ms_per_step": 1e3 * e2e_s / args.steps}
    if rank != 0:
        return
    # ---- roofline of the dominant kernel (wavefront expansion)
    peaks, peak_kind = measured_peaks()
    st0 = stats[-1]
    exp_ms = statistics.mean(s["ms_expand"] for s in stats)
    launches = max(1, st0["levels"])
    Vs = st0["vertices"]
    alg_bytes = Vs * (4 * (d + 1) + 8 * d + 2 * 16)  # record + two hash slots per vertex
    achieved = alg_bytes / (exp_ms / 1e3) / 1e9
    tr = ncu_traffic_per_vertex()
    traffic = None
    if tr and tr.get("d") == d:
        traffic = tr["dram_bytes_per_vertex"] * Vs / launches
    kernel = "k_expand_fast" if method == hvgpu.HV_METHOD_FAST else "k_expand_plain"
    hbm = {"bound": "hbm", "kernel": kernel, "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
           "frac": achieved / peaks["hbm_gbs"], "traffic": traffic, "peak_source": peak_kind,
           "traffic_note": "ncu DRAM bytes with its default cache flush before every launch: the candidate lists "
                           "are re-read from DRAM at every wavefront level, which L2 holds in an unprofiled run",
           "alg_bytes_per_launch": alg_bytes / launches, "ms_per_launch": exp_ms / launches,
           "launches_per_step": launches}
    # The binding roof of the candidate scan is the FP32 issue pipe (the working set lives in L2):
    # n_bar (5d+3) flops per vertex, n_bar = mean neighbour count of the mesh; peak = SMs x 128 FP32
    # lanes x 2 x max SM clock (nominal; no measured FP32 peak exists for this machine)
    mm = build_dev()
    _, nnbr = mm.counts(neighbors=True)
    mm.free()
    nbar = nnbr / n
    fp32_peak = fp32_peak_tflops(local, clocks)
    fl = Vs * nbar * (5 * d + 3)
    ach = fl / (exp_ms / 1e3) / 1e12
    roof = {"bound": "fp32", "kernel": kernel, "achieved": ach, "peak": fp32_peak, "unit": "TFLOP/s",
            "frac": ach / fp32_peak, "traffic": traffic, "peak_source": "nominal",
            "algorithmic_flops_per_vertex": nbar * (5 * d + 3), "mean_neighbours": nbar,
            "ms_per_launch": exp_ms / launches, "launches_per_step": launches, "hbm": hbm}
    # FP64 view of the circumcentre solves: (2/3)d^3 + 4d^2 flops per vertex against the nominal
    # GB300 FP64 rate (1.25 TFLOP/s; no measured FP64 peak exists for this machine)
    cen_ms = statistics.mean(s["ms_centers"] for s in stats)
    f64 = Vs * ((2.0 / 3.0) * d ** 3 + 4 * d * d)
    roof["fp64"] = {"kernel": "k_centers", "algorithmic_flops_per_vertex": (2.0 / 3.0) * d ** 3 + 4 * d * d,
                    "achieved_tflops": f64 / (cen_ms / 1e3) / 1e12, "peak_tflops_nominal": FP64_PEAK_TFLOPS,
                    "frac": f64 / (cen_ms / 1e3) / 1e12 / FP64_PEAK_TFLOPS}
    # ---- CPU baseline on the host cores
    cpu = None
    if not args.no_cpu_baseline and ws == 1:
        threads = os.cpu_count() or 1
        ncell = args.cpu_cells or n
        cells = np.arange(0, n, max(1, n // ncell))[:ncell]
        own, rays, sec = cpu_baseline(pts, cells, threads)
        cpu = {"value": own / sec, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"per-cell search of {len(cells)} of the {n} cells, vertices owned per second "
                         f"(C++ restatement of the reference algorithm, OpenMP)"}
    c3 = None
    if not args.no_c3 and ws == 1:
        try:
            c3 = run_c3(args, ctx, local, flush, clocks)
        except Exception as e:  # the headline line must still print
            c3 = {"error": repr(e)}
    c1 = c4 = None
    if not args.no_c3 and ws == 1:  # the other contract workloads, with their CPU baselines
        try:
            c1 = run_small(args, ctx, flush, "2d_uniform_1k", "polygon")
        except Exception as e:  # the headline line must still print
            c1 = {"error": repr(e)}
        try:
            c4 = run_small(args, ctx, flush, "6d_uniform_10k_mc", "heuristic_mc")
        except Exception as e:
            c4 = {"error": repr(e)}
    lattice = None
    if not args.no_lattice and ws == 1:
        try:
            lattice = run_lattice(ctx, flush)
        except Exception as e:  # the headline line must still print
            lattice = {"error": repr(e)}
    serving = None
    if not args.no_serve and ws == 1:
        try:
            serving = run_serve(args, local)
        except Exception as e:  # the headline line must still print
            serving = {"error": str(e)}
    cfg.update({"method": args.method, "l2": "flushed (256 MiB write) before every timed step",
                "vertices_per_step": Vs, "levels": st0["levels"], "parallelism": f"replicas x{ws}"})
    breakdown = {k: statistics.mean(s[k] for s in stats) for k in
                 ("ms_prepare", "ms_search", "ms_knn", "ms_descent", "ms_expand", "ms_fallback", "ms_centers",
                  "ms_canonical")}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": tot_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic", "config": cfg,
            "e2e": e2e, "roofline": roof, "cpu_baseline": cpu, "clocks": clocks, "integrators": integ,
            "gpu_launches": int(sum(s["launches"] for s in stats)),
            "stats": {k: st0[k] for k in ("rays", "fallback_rays", "uncertified", "insecure", "dd_rescores",
                                          "degenerate", "descents", "levels", "fallback_tree_rays",
                                          "fallback_nodes", "fallback_leaves", "fallback_points",
                                          "ambiguous_sets")},
            "rays_per_s": st0["rays"] / (tot_ms / 1e3 / args.steps),
            "breakdown_ms": breakdown, "c1_2d_uniform_1k": c1, "c3_5d_clustered_50k": c3,
            "c4_6d_uniform_10k": c4, "lattice": lattice, "serving": serving}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.serve:
        import torch
        torch.cuda.set_device(0)
        print(json.dumps({"serving": run_serve(args, 0)}), flush=True)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
