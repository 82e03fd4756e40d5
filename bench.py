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
    ap.add_argument("--serve-integrator", choices=["polygon", "none"], default="polygon")
    ap.add_argument("--no-integrators", action="store_true")
    ap.add_argument("--knn", type=int, default=0, help="candidate list length (0 = library default)")
    ap.add_argument("--leaf-size", type=int, default=0, help="tree leaf size (0 = library default)")
    ap.add_argument("--seed-stride", type=int, default=0, help="one descent seed per this many generators (0 = default)")
    ap.add_argument("--mc-dirs", type=int, default=1000, help="directions per cell of VI_HEURISTIC_MC")
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
    import hvgpu
    from hvgpu import datasets as D
    from hvgpu.serve import Server
    reqs, gaps = serve_requests(args.serve_requests)
    pts = [D.uniform_points(d, n, r) for d, n, r in reqs]
    arrivals = np.cumsum(gaps / args.serve_rate)
    integ = None if args.serve_integrator == "none" else args.serve_integrator
    with Server(device=device, slots=args.serve_slots) as srv:
        # warm-up: one request per dimension
        for d in (2, 3, 4, 5):
            srv.result(srv.submit(D.uniform_points(d, 500, 10 ** 6 + d), integrator=integ))
        t0 = time.perf_counter()
        tickets = []
        for k, (p, ta) in enumerate(zip(pts, arrivals)):
            now = time.perf_counter() - t0
            if ta > now:
                time.sleep(ta - now)
            tickets.append(srv.submit(p, integrator=integ))
        lat, fails, verts = [], 0, 0
        for t in tickets:
            r = srv.result(t)
            if r["status"] != 0:
                fails += 1
                continue
            lat.append(r["latency_ms"])
            verts += r["sig"].shape[0]
        t_end = time.perf_counter() - t0
    lat = np.array(lat)
    return {"requests": len(reqs), "rate_per_s": args.serve_rate, "slots": args.serve_slots, "failures": fails,
            "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "mean_ms": float(lat.mean()), "meshes_per_s": len(lat) / t_end, "vertices": int(verts),
            "config": "d uniform {2,3,4,5}, N log-uniform [200,20000], uniform points seed=request id, "
                      "cuboid(d, periodic=[]), " + ("VI_POLYGON" if integ else "no integrator") +
                      ", Poisson arrivals"}


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
        integ["polygon"].update({k: st[k] for k in ("poly_big_facets", "ms_poly_incidence", "ms_poly_facets",
                                                    "ms_poly_big")})
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
    roof = {"bound": "hbm", "kernel": "k_expand_fast" if method == hvgpu.HV_METHOD_FAST else "k_expand_plain",
            "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"],
            "traffic": traffic, "peak_source": peak_kind,
            "traffic_note": "ncu DRAM bytes with its default cache flush before every launch: the candidate lists "
                            "are re-read from DRAM at every wavefront level, which L2 holds in an unprofiled run",
            "alg_bytes_per_launch": alg_bytes / launches, "ms_per_launch": exp_ms / launches,
            "launches_per_step": launches}
    # FP32 view (the binding pipe of the candidate scan): n_bar (5d+3) flops per vertex, n_bar = mean
    # neighbour count of the mesh; peak = SMs x 128 FP32 lanes x 2 x max SM clock (nominal)
    try:
        mm = build_dev()
        _, nnbr = mm.counts(neighbors=True)
        mm.free()
        nbar = nnbr / n
        prop = torch.cuda.get_device_properties(local)
        fmax = (clocks or {}).get("sm_max_mhz") or 2070.0
        fp32_peak = prop.multi_processor_count * 128 * 2 * fmax * 1e6 / 1e12
        fl = Vs * nbar * (5 * d + 3)
        ach = fl / (exp_ms / 1e3) / 1e12
        roof["fp32"] = {"algorithmic_flops_per_vertex": nbar * (5 * d + 3), "mean_neighbours": nbar,
                        "achieved_tflops": ach, "peak_tflops_nominal": fp32_peak, "frac": ach / fp32_peak}
    except Exception as ex:  # noqa: BLE001
        roof["fp32"] = {"error": str(ex)}
    # FP64 view of the circumcentre solves: (2/3)d^3 + 4d^2 flops per vertex against the nominal
    # GB300 FP64 rate (1.25 TFLOP/s; no measured FP64 peak exists for this machine)
    cen_ms = statistics.mean(s["ms_centers"] for s in stats)
    f64 = Vs * ((2.0 / 3.0) * d ** 3 + 4 * d * d)
    roof["fp64"] = {"kernel": "k_centers", "algorithmic_flops_per_vertex": (2.0 / 3.0) * d ** 3 + 4 * d * d,
                    "achieved_tflops": f64 / (cen_ms / 1e3) / 1e12, "peak_tflops_nominal": 1.25,
                    "frac": f64 / (cen_ms / 1e3) / 1e12 / 1.25}
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
            "breakdown_ms": breakdown, "serving": serving}
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
