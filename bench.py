#!/usr/bin/env python3
"""Benchmark of the petgem forward-modelling hot path on GB300.

Workload (configuration the metric is quoted on): mixed-precision CSEM,
Nedelec p=2 on a box [-1000,1000]^3 m split into 32^3 cubes x 6 Kuhn
tetrahedra (196,608 tets, 1,276,096 DOFs, 54,751,616 stored entries),
interior nodes jittered by U(+-0.15h) (seed 0), per-element conductivity
log-uniform in [0.01, 3.3] S/m (seed 1), x-directed HED at (0,0,50) m, 1 Hz.
Seeded synthetic inputs with these shapes stand in for any dataset.

One step = one pass of the assembly over the whole mesh with inputs
resident in HBM: element geometry coefficients -> fused elemental
matrices + deterministic CSR value assembly -> point-dipole RHS -> PEC.
`value` is Melem/s = elements / step time (the metric's "p=2 Melem/s
assembled"); the pattern build (once per mesh) is reported separately.
The "ms/RHS to 1e-8 residual, FP64 vs mixed-precision batched" half of the
metric is measured in `solve` (true FP64 residual <= 1e-8 ||b||).

`--impl reference` times the reference's algorithm on the host CPU (the
numpy oracle port of petgem's hvfem elemental matrices + COO assembly), on
bounded samples of the same workload, with all host cores.
"""
import argparse
import json
import math
import multiprocessing as mp
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "p=2 Melem/s assembled; ms/RHS to 1e-8 residual, FP64 vs mixed-prec batched"
WORKLOAD = "csem_p2_32cubed_jittered_logsigma (196,608 tets, 1,276,096 DOFs)"


def workload(n):
    return WORKLOAD if n == 32 else f"csem_p2_{n}cubed_jittered_logsigma ({6 * n ** 3:,} tets)"


def workload_config(n, tets, dofs, nnz):
    """`config` of both arms (the same keys and values for the same workload)."""
    return {"workload": workload(n), "p": 2, "tets": int(tets), "dofs": int(dofs), "nnz": int(nnz),
            "l2": "working set per step > 129 MB L2 (A values alone 16 B x nnz)"}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=32, help="cubes per axis (32 = the metric's configuration)")
    ap.add_argument("--solve", default="all", choices=["all", "none"])
    ap.add_argument("--max-it", type=int, default=40000)
    ap.add_argument("--nrhs", type=int, default=16)
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="target CPU time of a baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--assembly", default="fp64", choices=["df64", "fp64"],
                    help="arithmetic of the headline assembly (fp64, the reference's arithmetic; df64: "
                         "double-float on the FP32 pipes, reported beside it as assembly_df64)")
    ap.add_argument("--config", type=int, default=1, choices=[0, 1, 2, 3, 4],
                    help="1: the metric's workload (default); 0: plain FP64 CSEM p=1 16^3 with petgem's "
                         "GMRES(30)+Jacobi, checked against the oracle; 2: the batched workload (12 systems x 16 RHS "
                         "in one solve); 3: the adjoint gradient (24^3) with finite-difference checks; 4: the MT "
                         "configuration (p=3, 40^3)")
    ap.add_argument("--no-records", action="store_true",
                    help="assemble from the item list instead of the per-mesh assembly records")
    ap.add_argument("--solve-iters", type=int, default=0,
                    help="profiling mode: run each solver form for exactly this many iterations")
    ap.add_argument("--profile-only", default="",
                    help="profiling mode: comma-separated solver forms to run (default: all)")
    return ap.parse_args()


# ----------------------------------------------------------------------------- CPU (oracle) leg
def _cpu_worker(args):
    """Elemental matrices + COO->CSR assembly of a slice of elements with the
    oracle (numpy restatement of petgem/hvfem.py:223-316, solver.py:182-235)."""
    coords, eo, fo, sigma, dofs, p, N = args
    from oracle import fem
    M, K = fem.element_matrices_batch(coords, eo, fo, sigma, p)
    A = fem.assemble(M, K, dofs, N, 1.0)
    return A.nnz


def cpu_prepare(model):
    """Per-mesh oracle topology (not timed): per-element coordinates, orientations, DOFs."""
    from oracle import topology
    tets = model.tets
    eE, eN = topology.compute_edges(tets)
    eF, fN = topology.compute_faces(tets)
    fE = topology.compute_faces_edges(eF, eE, fN.shape[0])
    eo, fo = topology.element_orientation(tets, eE, eN, eF, fE)
    dofs, _, _, _, N = topology.compute_connectivity_dofs(eE, eF, model.p)
    return {"coords": model.nodes[tets], "eo": eo, "fo": fo, "dofs": dofs, "N": N,
            "nnz": pattern_nnz(eE, eF, model.p)}


def pattern_nnz(elemsE, elemsF, p):
    """Stored entries of A before PEC: every pair of mesh entities (edge,
    face, volume) that share an element couples all their DOFs."""
    T = elemsE.shape[0]
    nE, nF = int(elemsE.max()) + 1, int(elemsF.max()) + 1
    ents = [elemsE.astype(np.int64), nE + elemsF.astype(np.int64)]
    nd = [np.full(6, p), np.full(4, p * (p - 1))]
    if p >= 3:
        ents.append((nE + nF + np.arange(T, dtype=np.int64))[:, None])
        nd.append(np.array([p * (p - 1) * (p - 2) // 2]))
    ent = np.concatenate(ents, axis=1)
    ndof = np.concatenate(nd)
    keep = ndof > 0
    ent, ndof = ent[:, keep], ndof[keep]
    n_ent = nE + nF + T
    keys = (ent[:, :, None] * n_ent + ent[:, None, :]).reshape(-1)
    w = (ndof[:, None] * ndof[None, :]).reshape(-1)
    uk, first = np.unique(keys, return_index=True)
    return int(np.tile(w, T)[first].sum())


def cpu_assembly_rate(model, seconds, cores, prep=None, pool=None):
    """Melem/s of the oracle assembly on a bounded sample; returns (rate, sample_elems, wall).
    pool: a spawn-context Pool of `cores` workers (made here when None)."""
    prep = prep or cpu_prepare(model)
    tets = model.tets
    coords, eo, fo, dofs, N = prep["coords"], prep["eo"], prep["fo"], prep["dofs"], prep["N"]

    def job(idx):
        return (coords[idx], eo[idx], fo[idx], model.sigma[idx], dofs[idx], model.p, N)

    # calibrate on one core
    t = time.time()
    _cpu_worker(job(np.arange(64)))
    per_elem = (time.time() - t) / 64
    n_el = int(min(len(tets), max(cores * 64, seconds * cores / max(per_elem, 1e-6))))
    idx = np.arange(n_el)
    parts = np.array_split(idx, cores * 4)
    own = pool is None
    if own:
        pool = mp.get_context("spawn").Pool(cores)
    try:
        pool.map(_cpu_worker, [job(parts[0][:8])] * cores)     # warm the workers
        t = time.time()
        pool.map(_cpu_worker, [job(pp) for pp in parts])
        wall = time.time() - t
    finally:
        if own:
            pool.close()
            pool.join()
    return n_el / wall / 1e6, n_el, wall


# ----------------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 20 ms from a reader
    thread that stamps each line on arrival; summary() keeps the samples that
    arrived between mark_start() and mark_end() (plus one interval of grace)."""

    INTERVAL_MS = 20

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.rows = []
        self.t0 = self.t1 = None

    def __enter__(self):
        import threading
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", str(self.INTERVAL_MS)],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, stdin=subprocess.DEVNULL,
                                         text=True)
        except Exception:
            self.proc = None
            return self
        self.started = threading.Event()

        def reader():
            for ln in self.proc.stdout:
                self.rows.append((time.time(), ln))
                self.started.set()
        self.thread = threading.Thread(target=reader, daemon=True)
        self.thread.start()
        self.started.wait(timeout=5.0)            # sampling is live before the timed region
        return self

    def mark_start(self):
        self.t0 = time.time()

    def mark_end(self):
        self.t1 = time.time()
        time.sleep(2 * self.INTERVAL_MS / 1e3)

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows or self.t0 is None or self.t1 is None:
            return None
        grace = self.INTERVAL_MS / 1e3
        rows = [ln for t, ln in self.rows if self.t0 <= t <= self.t1 + grace]
        rows = [[c.strip() for c in r.split(",")] for r in rows]
        rows = [r for r in rows if len(r) >= 9]
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows), "window_ms": round((self.t1 - self.t0) * 1e3, 1)}


# ----------------------------------------------------------------------------- GPU leg
def fp64_peak(torch, lib):
    import ctypes
    out = torch.empty(152 * 16 * 256, dtype=torch.float64, device="cuda")
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    blocks, iters = 152 * 16, 2048
    for _ in range(2):
        lib.pg_fp64_probe(ctypes.c_void_p(out.data_ptr()), blocks, iters, s)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(5):
        lib.pg_fp64_probe(ctypes.c_void_p(out.data_ptr()), blocks, iters, s)
    e1.record()
    torch.cuda.synchronize()
    return 5 * lib.pg_fp64_probe_flops(blocks, iters) / (e0.elapsed_time(e1) * 1e-3) / 1e12


def measured_hbm():
    """HBM copy bandwidth from MEASURED_PEAKS.json, else the 6.8 TB/s fallback."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "of measured (MEASURED_PEAKS.json hbm_gbs)"
    except (OSError, KeyError, ValueError):
        return 6800.0, "of fallback (6.8 TB/s)"


def read_traffic(name):
    """dram bytes per launch recorded in a committed ncu summary, if present."""
    if name is None:
        return None
    path = os.path.join(ROOT, "profiles", name)
    try:
        for ln in open(path):
            if ln.startswith("traffic_bytes_per_launch:"):
                return float(ln.split(":")[1])
    except OSError:
        pass
    return None


def replica_throughput(ms_local, steps, units_per_rank, world, dist=None, device="cpu"):
    """Replicas (one mesh per rank, no data-path collective): the slowest
    rank's time sets the step time; value = all ranks' elements / that time,
    in Melem/s.  Returns (ms per step, value)."""
    import torch
    ms_max = float(ms_local)
    if dist is not None and world > 1:
        tt = torch.tensor([ms_max], dtype=torch.float64, device=device)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        ms_max = float(tt.item())
    ms_per_step = ms_max / steps
    return ms_per_step, world * units_per_rank / (ms_per_step * 1e-3) / 1e6


def run_gpu(args, rank, world, local_rank):
    import torch
    from petgem_gb300 import _lib, synthetic
    from petgem_gb300.engine import DeviceMesh
    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    lib = _lib.load()
    model = synthetic.config1(args.n)
    freq = model.source["frequency"]
    torch.zeros(1, device="cuda")          # CUDA context exists before the setup is timed
    torch.cuda.synchronize()

    t0 = time.time()
    mesh = DeviceMesh(model.nodes, model.tets, model.p, device=f"cuda:{local_rank}")
    if not args.no_records:
        mesh.records()
        mesh.tables_entry_major(args.assembly)
    torch.cuda.synchronize()
    setup_ms = (time.time() - t0) * 1e3
    T = mesh.T
    sigma = mesh.sigma_tensor(model.sigma)
    df = args.assembly == "df64"
    if df:
        coef = torch.empty((T, 12, 2), dtype=torch.float32, device="cuda")
    else:
        coef = torch.empty((T, 12), dtype=torch.float64, device="cuda")
    vals = torch.empty(mesh.nnz, dtype=torch.complex128, device="cuda")
    b = torch.zeros(mesh.N, dtype=torch.complex128, device="cuda")
    src_elem = mesh.locate_source(model.source)
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    launches_per_step = 4   # coefficients, fused assembly + PEC rows/columns, source, PEC on b

    def assemble(v=None, ar=None, cf=None):
        mesh.assemble(sigma, freq, out=vals if v is None else v, coef=coef if cf is None else cf,
                      arithmetic=ar or args.assembly, pec=True, records=not args.no_records)

    side = torch.cuda.Stream()

    def step(v=None, bv=None, ar=None, cf=None):
        # the RHS (zero, point dipole, PEC rows of b) runs on a second stream
        # beside the matrix pass; the step ends when both have finished
        bv = b if bv is None else bv
        main = torch.cuda.current_stream()
        side.wait_stream(main)
        with torch.cuda.stream(side):
            bv.zero_()
            mesh.source_rhs(model.source, src_elem, bv, status=status)
            mesh.pec_rhs(bv)
        mesh.element_coefficients(sigma, freq, out=coef if cf is None else cf, check=False,
                                  arithmetic=ar or args.assembly)
        assemble(v, ar, cf)
        main.wait_stream(side)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if status.item() != 0:
        raise RuntimeError("source RHS failed")

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    with ClockSampler(local_rank) as clk:
        clk.mark_start()
        e0.record()
        for _ in range(args.steps):
            step()
        e1.record()
        barrier()
        clk.mark_end()
    ms_per_step, value = replica_throughput(e0.elapsed_time(e1), args.steps, T, world, dist, "cuda")

    # dominant kernel: fused assembly, timed alone on the launching stream
    k0, k1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    k0.record()
    for _ in range(args.steps):
        assemble()
    k1.record()
    torch.cuda.synchronize()
    k_ms = k0.elapsed_time(k1) / args.steps
    nd = mesh.nd
    flops = T * (nd * (nd + 1) // 2) * 12 * 2          # 12 multiply-adds per unique elemental entry
    # algorithmic bytes: A values written once; per item its record (or item
    # word) read once; per element its 12 coefficients and tuple id; every
    # member of an upper pair (a <= b) once
    nl = {1: 6, 2: 10}.get(mesh.p, 11)
    work_bytes = mesh.n_items * (8 if args.no_records else _lib.query("pg_assembly_record_bytes", mesh.nnz))
    nbytes = int(mesh.nnz * 16 + work_bytes + T * (12 * 8 + 4) + T * (nl * (nl + 1) // 2) * 4)
    peak64 = fp64_peak(torch, lib)
    if df:
        hbm = measured_hbm()
        achieved = nbytes / (k_ms * 1e-3) / 1e9
        roofline = {"bound": "hbm", "kernel": ("k_values_rec<2, df>" if not args.no_records else "k_values_sym_df<2>")
                    + " (fused elemental + CSR assembly + PEC, double-float)",
                    "achieved": round(achieved, 1), "peak": hbm[0], "unit": "GB/s", "frac": round(achieved / hbm[0], 4),
                    "peak_source": hbm[1],
                    "traffic": read_traffic("assembly_records_df64_p2_ncu.md" if not args.no_records else None),
                    "algorithmic_bytes_per_launch": nbytes, "ms_per_launch": round(k_ms, 4),
                    "fp64_equivalent_tflops": round(flops / (k_ms * 1e-3) / 1e12, 4),
                    "fp64_peak_tflops": round(peak64, 4)}
    else:
        achieved = flops / (k_ms * 1e-3) / 1e12
        roofline = {"bound": "fp64", "kernel": ("k_values_rec<2, fp64>" if not args.no_records else "k_values_sym<2>")
                    + " (fused elemental + CSR assembly + PEC)",
                    "achieved": round(achieved, 4), "peak": round(peak64, 4), "unit": "TFLOP/s",
                    "frac": round(achieved / peak64, 4), "peak_source": "measured live (FP64 FMA probe)",
                    "traffic": read_traffic("assembly_records_fp64_p2_ncu.md" if not args.no_records else None),
                    "algorithmic_flops_per_launch": flops, "ms_per_launch": round(k_ms, 4),
                    "algorithmic_bytes_per_launch": nbytes}

    # the double-float form beside the FP64 headline: same step, (hi, lo)
    # FP32-pair products on the FP32 pipes; its dominant kernel is bound by
    # load traffic, so its roofline is the HBM copy rate
    assembly_df64 = None
    if not df and not args.no_records:
        mesh.tables_entry_major("df64")
        coef_df = torch.empty((T, 12, 2), dtype=torch.float32, device="cuda")
        vals_df = torch.empty_like(vals)
        for _ in range(args.warmup):
            step(vals_df, None, "df64", coef_df)
        barrier()
        e0.record()
        for _ in range(args.steps):
            step(vals_df, None, "df64", coef_df)
        e1.record()
        barrier()
        ms_df = e0.elapsed_time(e1) / args.steps
        k0.record()
        for _ in range(args.steps):
            assemble(vals_df, "df64", coef_df)
        k1.record()
        torch.cuda.synchronize()
        kdf = k0.elapsed_time(k1) / args.steps
        hbm = measured_hbm()
        ach = nbytes / (kdf * 1e-3) / 1e9
        # entrywise against the FP64 values, relative to each row's largest entry
        rowmax = torch.zeros(mesh.N, dtype=torch.float64, device="cuda")
        rows = torch.repeat_interleave(torch.arange(mesh.N, device="cuda"), mesh.rowptr[1:] - mesh.rowptr[:-1])
        rowmax.scatter_reduce_(0, rows, vals.abs(), reduce="amax")
        dev_rel = float(((vals_df - vals).abs() / rowmax[rows]).max())
        del rows, rowmax
        assembly_df64 = {"Melem_per_s": round(world * T / (ms_df * 1e-3) / 1e6, 3), "ms_per_step": round(ms_df, 4),
                         "dtype": "df64 (f32 pairs) -> f64",
                         "kernel": "k_values_rec<2, df> (fused elemental + CSR assembly + PEC, double-float)",
                         "ms_per_launch": round(kdf, 4),
                         "roofline": {"bound": "hbm", "achieved": round(ach, 1), "peak": hbm[0], "unit": "GB/s",
                                      "frac": round(ach / hbm[0], 4), "peak_source": hbm[1],
                                      "traffic": read_traffic("assembly_records_df64_p2_ncu.md"),
                                      "algorithmic_bytes_per_launch": nbytes},
                         "max_entry_dev_vs_fp64_over_row_max": dev_rel}
        del vals_df, coef_df

    # end to end: host buffers in (pinned), A values and b back to the host.
    # Two device / host buffer pairs: the read-back of step k (host link,
    # ~190 GB/s on GB300) overlaps the assembly of step k + 1.
    nodes_h = torch.from_numpy(np.ascontiguousarray(model.nodes)).pin_memory()
    sigma_h = torch.from_numpy(np.ascontiguousarray(model.sigma)).pin_memory()
    vals2 = [vals, torch.empty_like(vals)]
    b2 = [b, torch.empty_like(b)]
    vals_h = [torch.empty(mesh.nnz, dtype=torch.complex128).pin_memory() for _ in range(2)]
    b_h = [torch.empty(mesh.N, dtype=torch.complex128).pin_memory() for _ in range(2)]
    copier = torch.cuda.Stream()
    copied = [None, None]

    def e2e_step(k):
        i = k % 2
        main = torch.cuda.current_stream()
        if copied[i] is not None:
            main.wait_event(copied[i])              # buffer pair i has reached the host
        mesh.nodes.copy_(nodes_h, non_blocking=True)
        sigma.copy_(sigma_h, non_blocking=True)
        step(vals2[i], b2[i])
        ready = torch.cuda.Event()
        ready.record(main)
        copier.wait_event(ready)
        with torch.cuda.stream(copier):
            vals_h[i].copy_(vals2[i], non_blocking=True)
            b_h[i].copy_(b2[i], non_blocking=True)
            copied[i] = torch.cuda.Event()
            copied[i].record(copier)

    def e2e_drain():
        torch.cuda.current_stream().wait_stream(copier)

    for k in range(2):
        e2e_step(k)
    e2e_drain()
    barrier()
    e0.record()
    for k in range(args.steps):
        e2e_step(k)
    e2e_drain()
    e1.record()
    barrier()
    e2e_ms = e0.elapsed_time(e1) / args.steps
    if not torch.equal(vals_h[(args.steps - 1) % 2][:1024], vals[:1024].cpu()):
        raise RuntimeError("end-to-end read-back does not match the device values")
    # the host link itself: one device -> host copy of the A values into pinned memory
    link0, link1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    link0.record()
    vals_h[0].copy_(vals, non_blocking=True)
    link1.record()
    torch.cuda.synchronize()
    link_gbs = vals.numel() * 16 / (link0.elapsed_time(link1) * 1e-3) / 1e9
    e2e = {"value": round(world * T / (e2e_ms * 1e-3) / 1e6, 3), "unit": "Melem/s",
           "link_d2h_gbs": round(link_gbs, 1),
           "h2d_bytes_per_step": int(nodes_h.numel() * 8 + sigma_h.numel() * 8),
           "d2h_bytes_per_step": int(vals.numel() * 16 + b.numel() * 16), "ms_per_step": round(e2e_ms, 3),
           "pipelined": "read-back of step k overlaps step k + 1 (two buffer pairs)"}
    del vals2[1], b2[1]

    cpu_solve = None
    if rank == 0 and not args.no_cpu_baseline and args.solve == "all":
        cpu_solve = cpu_solve_rate(mesh, vals, b)

    solve = None
    if args.solve_iters > 0 and rank == 0:
        solve = profile_solves(args, torch, mesh, vals, b)
    elif args.solve == "all" and rank == 0:
        solve = run_solves(args, torch, mesh, model, vals, b)

    line = None
    if rank == 0:
        line = {"metric": METRIC, "value": round(value, 3), "unit": "Melem/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_per_step, 4),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f64" if not df else "df64 (f32 pairs) -> f64", "data": "synthetic (seeded Kuhn-cube mesh, jittered; log-uniform sigma)",
                "config": workload_config(args.n, T, mesh.N, mesh.nnz),
                "setup": {"parallelism": "replicas" if world > 1 else "single GPU",
                          "pattern_setup_ms": round(setup_ms, 1), "orientation_tuples": mesh.n_tuples},
                "roofline": roofline, "e2e": e2e, "gpu_launches": launches_per_step * args.steps,
                "clocks": clk.summary(), "assembly_df64": assembly_df64, "solve": solve}
        if cpu_solve is not None:
            if solve and "fp64_diagonal_jacobi" in solve:
                n_it = solve["fp64_diagonal_jacobi"]["iterations"]
                cpu_solve["ms_per_rhs_extrapolated"] = round(cpu_solve["ms_per_iteration"] * n_it, 1)
                cpu_solve["iterations_from"] = f"the GPU FP64 COCG + diagonal Jacobi count ({n_it}, same algorithm)"
                cpu_solve["gpu_fp64_speedup_per_rhs"] = round(cpu_solve["ms_per_rhs_extrapolated"] /
                                                              solve["fp64"]["ms_per_rhs"], 1)
                cpu_solve["gpu_df64_batched_speedup_per_rhs"] = round(cpu_solve["ms_per_rhs_extrapolated"] /
                                                                      solve["df64_batched"]["ms_per_rhs"], 1)
            line["cpu_baseline_solve"] = cpu_solve
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    return line


def cpu_solve_rate(mesh, vals, b, iters=150):
    """FP64 COCG (same algorithm, symmetric Jacobi) on all host cores, compiled
    C + OpenMP (oracle/csrc/cpu_cocg.c): ms per iteration on a bounded run of
    `iters` iterations of the workload's system."""
    from oracle import build_cpu
    rp, col = mesh.rowptr.cpu().numpy(), mesh.col.cpu().numpy()
    v, bh = vals.cpu().numpy(), b.cpu().numpy()
    build_cpu.cocg(rp, col, v, bh, 2, 1e-30)          # warm-up (page-in, thread pool)
    t = time.time()
    _, its, rel, st = build_cpu.cocg(rp, col, v, bh, iters, 1e-30)
    dt = time.time() - t
    return {"ms_per_iteration": round(dt * 1e3 / max(its, 1), 3), "sample_iterations": its,
            "threads": os.cpu_count() or 1, "kind": "port (compiled C + OpenMP, FP64 COCG + Jacobi)"}


def run_solves(args, torch, mesh, model, vals, b):
    """ms/RHS to a 1e-8 true relative residual for the plain FP64 form and the
    mixed-precision batched form (COCG with Jacobi scaling; restarted GMRES(30)
    per iteration cost as the PETSc-default reference point)."""
    from petgem_gb300 import synthetic
    out = {"criterion": "||b - A x|| <= 1e-8 ||b|| (FP64 true residual)"}

    def timed(ksp, prec, rhs, max_it, precond="block", inner_rtol=None):
        torch.cuda.synchronize()
        t = time.time()
        x, info = mesh.solve(vals, rhs, rtol=1e-8, precision=prec, max_it=max_it, raise_on_fail=False, ksp=ksp,
                             precond=precond, inner_rtol=inner_rtol)
        torch.cuda.synchronize()
        dt = time.time() - t
        k = 1 if rhs.ndim == 1 else rhs.shape[1]
        out = {"ksp": ksp, "precision": prec, "precond": precond, "nrhs": k,
               "seconds": round(dt, 3),
               "ms_per_rhs": round(dt * 1e3 / k, 2), "iterations": info.iterations,
               "ms_per_iteration": round(dt * 1e3 / max(info.iterations, 1), 4),
               "relres": info.relres, "converged": info.status == 0}
        if prec == "ir32":
            out["refinement_steps"] = info.restarts
            out["inner_rtol"] = inner_rtol if inner_rtol is not None else (1e-4 if precond == "grad" else 1e-2)
            out["iterations_are"] = "complex64 inner iterations (max over RHS)"
        return x, out

    # column 0: the workload's own HED; columns 1..: x-HEDs of the batched configuration
    srcs = [model.source] + synthetic.config2_sources(count=args.nrhs - 1)
    B = torch.zeros((mesh.N, len(srcs)), dtype=torch.complex128, device="cuda")
    for k, s in enumerate(srcs):
        bk = torch.zeros(mesh.N, dtype=torch.complex128, device="cuda")
        mesh.source_rhs(s, mesh.locate_source(s), bk)
        B[:, k] = bk
    mesh.pec_rhs(B)
    if not bool((torch.linalg.norm(B, dim=0) > 0).all()):
        raise RuntimeError("a batched source was not located in the mesh (zero right-hand side)")
    x64, r64 = timed("cocg", "fp64", b, args.max_it)
    _, r64j = timed("cocg", "fp64", b, args.max_it, precond="jacobi")
    # Jacobi plus the auxiliary-space correction D^-1 + B diag(B^T A B)^-1 B^T
    # (B = [G P], the discrete gradient and the vector P1 fields; the map is
    # built once per mesh and timed on its own)
    torch.cuda.synchronize()
    t = time.time()
    gmap = mesh.gradient_map()
    torch.cuda.synchronize()
    out["gradient_map"] = {"ms": round((time.time() - t) * 1e3, 2), "columns": gmap.n_cols, "entries": gmap.nnz}
    xg, rgr = timed("cocg", "fp64", b, args.max_it, precond="grad")
    Xgb, rgb = timed("cocg", "fp64", B.contiguous(), args.max_it, precond="grad")
    xgm, rgm = timed("gmres", "fp64", b, args.max_it, precond="grad")
    xgmm, rgmm = timed("gmres", "mixed", b, args.max_it, precond="grad")
    xgd, rgd = timed("cocg", "df64", b, args.max_it, precond="grad")
    Xgdb, rgdb = timed("cocg", "df64", B.contiguous(), args.max_it, precond="grad")
    xdf, rdf = timed("cocg", "df64", b, args.max_it)
    Xdb, rdb = timed("cocg", "df64", B.contiguous(), args.max_it)
    # complex64 inner solves + FP64 iterative refinement (one RHS, then the
    # 16-RHS batch); a stall would be recorded, not raised
    from petgem_gb300 import _lib
    def timed_ir(rhs, precond="block", inner_rtol=None):
        try:
            return timed("cocg", "ir32", rhs, args.max_it, precond=precond, inner_rtol=inner_rtol)
        except _lib.PetgemError as exc:
            return None, {"ksp": "cocg", "precision": "ir32", "converged": False, "status": exc.status,
                          "error": str(exc)}
    xir, rir = timed_ir(b)
    Xib, rib = timed_ir(B.contiguous())
    xgi, rgi = timed_ir(b, precond="grad")
    Xgib, rgib = timed_ir(B.contiguous(), precond="grad", inner_rtol=1e-5)
    # several frequencies in one solve: 4 frequencies x 8 sources (32 columns)
    freqs = [0.25, 0.5, 1.0, 2.0]
    f0 = model.source["frequency"]
    cols, fcol = [], []
    for f in freqs:
        for s in srcs[:8]:
            s = dict(s, frequency=f)
            bk = torch.zeros(mesh.N, dtype=torch.complex128, device="cuda")
            mesh.source_rhs(s, mesh.locate_source(s), bk)
            cols.append(bk)
            fcol.append(f)
    Bf = torch.stack(cols, 1).contiguous()
    mesh.pec_rhs(Bf)
    if not bool((torch.linalg.norm(Bf, dim=0) > 0).all()):
        raise RuntimeError("a multi-frequency source was not located in the mesh (zero right-hand side)")
    torch.cuda.synchronize()
    t = time.time()
    Xf, inf = mesh.solve_frequencies(vals, f0, Bf, fcol, rtol=1e-8, max_it=args.max_it, raise_on_fail=False)
    torch.cuda.synchronize()
    dtf = time.time() - t
    rmf = {"ksp": "cocg", "precision": "df64", "nrhs": len(fcol), "frequencies_hz": freqs, "sources": 8,
           "seconds": round(dtf, 3), "ms_per_rhs": round(dtf * 1e3 / len(fcol), 2), "iterations": inf.iterations,
           "ms_per_iteration": round(dtf * 1e3 / max(inf.iterations, 1), 4), "relres": inf.relres,
           "converged": inf.status == 0}
    torch.cuda.synchronize()
    t = time.time()
    Xfg, infg = mesh.solve_frequencies(vals, f0, Bf, fcol, precond="grad", rtol=1e-8, max_it=args.max_it,
                                       raise_on_fail=False)
    torch.cuda.synchronize()
    dtg = time.time() - t
    rmfg = {"ksp": "cocg", "precision": "df64", "precond": "grad", "nrhs": len(fcol), "frequencies_hz": freqs,
            "sources": 8, "seconds": round(dtg, 3), "ms_per_rhs": round(dtg * 1e3 / len(fcol), 2),
            "iterations": infg.iterations, "ms_per_iteration": round(dtg * 1e3 / max(infg.iterations, 1), 4),
            "relres": infg.relres, "converged": infg.status == 0}
    # the FP32-operator form stalls above 1e-8 at this conditioning: capped, per-iteration cost reported
    xmx, rmx = timed("cocg", "mixed", b, 3000)
    _, rg = timed("gmres", "mixed", b, 300)
    # receiver-field error of each form against a tight FP64 solve
    # reference solution for the receiver errors: FP64 COCG two decades tighter
    # (at 1e-11 the FP64 recurrence can stall near its attainable accuracy)
    xt, it_ = mesh.solve(vals, b, rtol=1e-10, precision="fp64", max_it=3 * args.max_it, raise_on_fail=False, ksp="cocg")
    out["reference_solve"] = {"rtol": 1e-10, "iterations": it_.iterations, "relres": it_.relres, "status": it_.status}
    Ft, _ = mesh.receiver_fields(xt, model.receivers, model.source["frequency"])
    j1 = fcol.index(f0)      # the workspace source at the workload frequency
    for x, r in ((x64, r64), (xdf, rdf), (xmx, rmx), (Xdb[:, 0].contiguous(), rdb), (Xf[:, j1].contiguous(), rmf),
                 (xir, rir), (None if Xib is None else Xib[:, 0].contiguous(), rib), (xg, rgr),
                 (Xgb[:, 0].contiguous(), rgb), (xgm, rgm), (xgd, rgd), (Xgdb[:, 0].contiguous(), rgdb),
                 (Xfg[:, j1].contiguous(), rmfg), (xgi, rgi), (xgmm, rgmm),
                 (None if Xgib is None else Xgib[:, 0].contiguous(), rgib)):
        if x is None:
            continue
        F, _ = mesh.receiver_fields(x, model.receivers, model.source["frequency"])
        r["receiver_rel_err_vs_fp64_1e-10"] = float(torch.linalg.norm(F - Ft) / torch.linalg.norm(Ft))
    out["fp64"] = r64
    out["fp64_diagonal_jacobi"] = r64j
    out["fp64_grad"] = rgr
    out["fp64_grad_batched"] = rgb
    out["gmres30_fp64_grad"] = rgm
    out["gmres30_mixed_grad"] = rgmm
    out["df64_grad"] = rgd
    out["ir32_grad"] = rgi
    out["ir32_grad_batched"] = rgib
    out["df64_grad_batched"] = rgdb
    out["speedup_df64_grad_batched_vs_fp64_per_rhs"] = round(r64["ms_per_rhs"] / max(rgdb["ms_per_rhs"], 1e-9), 2)
    out["speedup_fp64_grad_vs_fp64_per_rhs"] = round(r64["ms_per_rhs"] / max(rgr["ms_per_rhs"], 1e-9), 2)
    out["speedup_fp64_grad_batched_vs_fp64_per_rhs"] = round(r64["ms_per_rhs"] / max(rgb["ms_per_rhs"], 1e-9), 2)
    out["df64"] = rdf
    out["df64_batched"] = rdb
    out["mixed"] = rmx
    out["df64_multifrequency"] = rmf
    out["df64_multifrequency_grad"] = rmfg
    out["ir32"] = rir
    out["ir32_batched"] = rib
    if rib.get("converged"):
        out["speedup_ir32_batched_vs_fp64_per_rhs"] = round(r64["ms_per_rhs"] / max(rib["ms_per_rhs"], 1e-9), 2)
    out["gmres30_mixed_300its"] = rg
    out["note_grad"] = ("grad = diagonal Jacobi plus the auxiliary-space correction D^-1 + B diag(B^T A B)^-1 B^T "
                        "(B = [G P]: the discrete gradient of the quadratic H1 space and the vector P1 fields, "
                        "built on the device from the mesh); gmres30_fp64_grad is petgem's KSP, GMRES(30), "
                        "right-preconditioned with it")
    out["note"] = ("df64 = double-float (FP64-class, 48-bit mantissa) arithmetic on the FP32 pipes; ir32 = complex64 "
                   "inner COCG solves (matrix, vectors, products in FP32), each restarted from the FP64 true residual, "
                   "inside FP64 iterative refinement (each inner solve to a 100x residual drop, capped); at this "
                   "conditioning (eps32 * kappa ~ 1) its inner solves contract slowly and unevenly; mixed = complex64 "
                   "matrix/SpMV + FP64 recurrence with reliable updates, which stalls at this conditioning (capped)")
    out["speedup_df64_batched_vs_fp64_per_rhs"] = round(r64["ms_per_rhs"] / max(rdb["ms_per_rhs"], 1e-9), 2)

    return out


def profile_solves(args, torch, mesh, vals, b):
    """Fixed iteration counts of every solver form (for kernel launch lists)."""
    out = {}
    B = torch.stack([b] * args.nrhs, 1).contiguous()
    for name, ksp, prec, rhs, pc in (("cocg_fp64", "cocg", "fp64", b, "block"), ("cocg_df64", "cocg", "df64", b, "block"),
                                     ("cocg_df64_batched", "cocg", "df64", B, "block"),
                                     ("cocg_mixed", "cocg", "mixed", b, "block"), ("cocg_ir32", "cocg", "ir32", b, "block"),
                                     ("cocg_mixed_batched", "cocg", "mixed", B, "block"),
                                     ("gmres_mixed", "gmres", "mixed", b, "block"), ("gmres_fp64", "gmres", "fp64", b, "block"),
                                     ("cocg_fp64_grad", "cocg", "fp64", b, "grad"),
                                     ("cocg_df64_grad_batched", "cocg", "df64", B, "grad"),
                                     ("cocg_ir32_grad_batched", "cocg", "ir32", B, "grad")):
        if args.profile_only and name not in args.profile_only.split(","):
            continue
        torch.cuda.synchronize()
        t = time.time()
        _, info = mesh.solve(vals, rhs, rtol=1e-30, precision=prec, max_it=args.solve_iters, raise_on_fail=False,
                             ksp=ksp, check_every=args.solve_iters, precond=pc)
        torch.cuda.synchronize()
        dt = time.time() - t
        out[name] = {"iterations": info.iterations, "ms_per_iteration": round(dt * 1e3 / max(info.iterations, 1), 4)}
    return out


def run_reference(args, rank):
    """The reference's algorithm (oracle port) on the host CPU, bounded samples."""
    if rank != 0:
        return None
    from petgem_gb300 import synthetic
    model = synthetic.config1(args.n)
    cores = os.cpu_count() or 1
    prep = cpu_prepare(model)
    rates = []
    samples = []
    # each step a bounded sample; the whole K-step run stays within a few minutes
    per_step = max(0.5, min(args.cpu_seconds / 4, 120.0 / max(args.steps, 1)))
    with mp.get_context("spawn").Pool(cores) as pool:
        for _ in range(max(args.steps, 1)):
            rate, n_el, wall = cpu_assembly_rate(model, per_step, cores, prep, pool)
            rates.append(rate)
            samples.append(n_el)
    v = float(np.median(rates))
    sample = (f"oracle elemental matrices + COO/CSR assembly of the first {samples[0]} of {len(model.tets)} "
              f"elements per step, {cores} processes")
    return {"metric": METRIC, "value": round(v, 6), "unit": "Melem/s", "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "vs_baseline": None,
            "dtype": "f64", "data": "synthetic",
            "config": workload_config(args.n, len(model.tets), prep["N"], prep["nnz"]),
            "cpu_baseline": {"value": round(v, 6), "unit": "Melem/s", "cores": cores, "kind": "port",
                             "sample": sample},
            "e2e": {"value": round(v, 6), "unit": "Melem/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def run_config0(args):
    """Plain FP64 CSEM, Nedelec p = 1: 16^3 cubes x 6 tets (24,576 tets,
    31,024 DOFs), seawater 3.3 / sediment 1.0 S/m with a 0.01 S/m block,
    x-HED at (0,0,50) m, 1 Hz, 20 receivers on z = 0.  Times the FP64
    assembly (coefficients + fused elemental/CSR assembly + PEC) and petgem's
    own KSP, restarted GMRES(30) with Jacobi in complex128, to a 1e-8 true
    relative residual (ms per RHS).  The CPU leg builds the same system with
    the oracle (petgem's elemental loop and COO assembly restated), times
    scipy's GMRES(30) + Jacobi on it (the PETSc KSP stand-in), and checks the
    GPU's matrix, right-hand side and receiver fields against it and against
    a direct solve."""
    import torch
    from petgem_gb300 import synthetic
    from petgem_gb300.engine import DeviceMesh
    model = synthetic.config0()
    f = model.source["frequency"]
    pool = None
    if not args.no_cpu_baseline:                     # spawn workers before the first GPU call
        pool = mp.get_context("spawn").Pool(os.cpu_count() or 1)
    t0 = time.time()
    mesh = DeviceMesh(model.nodes, model.tets, 1)
    mesh.records()
    mesh.tables_entry_major("fp64")
    torch.cuda.synchronize()
    setup_ms = (time.time() - t0) * 1e3
    sigma = mesh.sigma_tensor(model.sigma)
    coef = torch.empty((mesh.T, 12), dtype=torch.float64, device="cuda")
    vals = torch.empty(mesh.nnz, dtype=torch.complex128, device="cuda")

    def step():
        mesh.element_coefficients(sigma, f, out=coef, check=False)
        mesh.assemble(sigma, f, out=vals, coef=coef, pec=True)
    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    steps = max(args.steps, 1)
    e0.record()
    for _ in range(steps):
        step()
    e1.record()
    torch.cuda.synchronize()
    asm_ms = e0.elapsed_time(e1) / steps
    b, _ = mesh.source_vector(model.source)
    mesh.pec_rhs(b)

    def solve(ksp, precond, prec="fp64"):
        mesh.solve(vals, b, rtol=1e-8, ksp=ksp, precond=precond, precision=prec, max_it=60, raise_on_fail=False)
        torch.cuda.synchronize()                     # warm-up: workspace, autotuning
        t = time.time()
        x, info = mesh.solve(vals, b, rtol=1e-8, ksp=ksp, precond=precond, precision=prec, restart=30,
                             max_it=args.max_it, raise_on_fail=False)
        torch.cuda.synchronize()
        dt = time.time() - t
        F, _ = mesh.receiver_fields(x, model.receivers, f)
        return x, F, {"ksp": ksp, "precond": precond, "precision": prec, "ms_per_rhs": round(dt * 1e3, 2),
                      "iterations": info.iterations, "relres": info.relres, "converged": info.status == 0}
    x, F, gm = solve("gmres", "jacobi")
    gm["restart"] = 30
    others = {}
    for name, ksp, pc, prec in (("cocg_fp64_block", "cocg", "block", "fp64"),
                                ("cocg_df64_block", "cocg", "block", "df64"),
                                ("gmres30_fp64_block", "gmres", "block", "fp64"),
                                ("gmres30_fp64_grad", "gmres", "grad", "fp64"),
                                ("cocg_fp64_grad", "cocg", "grad", "fp64")):
        _, Fo, r = solve(ksp, pc, prec)
        r["receiver_E_rel_diff_vs_gmres"] = float(torch.linalg.norm(Fo[:, :3] - F[:, :3]) /
                                                  torch.linalg.norm(F[:, :3]))
        others[name] = r
    cpu = None
    if pool is not None:
        from oracle import solve as osolve
        from oracle import system
        try:
            t = time.time()
            S = system.csem_system(model.nodes, model.tets, model.sigma, 1, model.source, pool=pool)
            t_asm = time.time() - t
        finally:
            pool.close()
            pool.join()
        A = S["A"]
        rp, cl = mesh.rowptr.cpu().numpy(), mesh.col.cpu().numpy()
        same_pattern = bool(np.array_equal(rp, A.indptr) and np.array_equal(cl, A.indices))
        v = vals.cpu().numpy()
        t = time.time()
        xc, its, rel = osolve.gmres_jacobi(A, S["b"], 1e-8, 30)
        t_gm = time.time() - t
        # the same GMRES(30) + Jacobi compiled as C + OpenMP on every host core
        # (oracle/csrc/cpu_gmres.c), the PETSc-class CPU point
        compiled = None
        try:
            from oracle import build_cpu
            build_cpu.gmres(A.indptr, A.indices, A.data, S["b"], 30, 5, 1e-8)      # warm-up (threads, page-in)
            t = time.time()
            xg, its_g, rel_g, st_g = build_cpu.gmres(A.indptr, A.indices, A.data, S["b"], 30, 20000, 1e-8)
            t_cg = time.time() - t
            compiled = {"ms_per_rhs": round(t_cg * 1e3, 1), "iterations": its_g, "relres": rel_g,
                        "converged": st_g == 0, "threads": os.cpu_count() or 1,
                        "x_rel_diff_vs_scipy": float(np.linalg.norm(xg - xc) / np.linalg.norm(xc))}
        except Exception as exc:   # the CPU point is reported, not required
            compiled = {"error": str(exc)[:200]}
        xd = osolve.direct(A, S["b"])
        Fd, _ = system.receiver_fields(S, xd, model.nodes, model.tets, 1, model.receivers, f)
        Fc, _ = system.receiver_fields(S, xc, model.nodes, model.tets, 1, model.receivers, f)
        Fg = F.cpu().numpy()
        rel_e = lambda a, r: float(np.linalg.norm(a[:, :3] - r[:, :3]) / np.linalg.norm(r[:, :3]))
        cpu = {"kind": "port", "cores": os.cpu_count() or 1,
               "sample": "the whole system: oracle elemental matrices (all cores) + COO assembly + PEC, then "
                         "scipy GMRES(30) + Jacobi (PETSc KSP stand-in, one core); compiled_gmres: the same "
                         "GMRES(30) + Jacobi in C + OpenMP on every host core",
               "assembly_seconds": round(t_asm, 3), "gmres_ms_per_rhs": round(t_gm * 1e3, 1),
               "gmres_iterations": its, "gmres_relres": rel,
               "compiled_gmres": compiled,
               "check": {"pattern_bit_exact": same_pattern,
                         "values_rel_diff": float(np.linalg.norm(v - A.data) / np.linalg.norm(A.data))
                         if same_pattern else None,
                         "b_rel_diff": float(np.linalg.norm(b.cpu().numpy() - S["b"]) / np.linalg.norm(S["b"])),
                         "gpu_receiver_E_rel_err_vs_oracle_direct": rel_e(Fg, Fd),
                         "gpu_receiver_EH_rel_err_vs_oracle_direct": float(np.linalg.norm(Fg - Fd) /
                                                                           np.linalg.norm(Fd)),
                         "cpu_gmres_receiver_E_rel_err_vs_oracle_direct": rel_e(Fc, Fd)}}
    return {"metric": "ms/RHS to 1e-8 residual, plain FP64 GMRES(30)+Jacobi (p=1 CSEM)", "value": gm["ms_per_rhs"],
            "unit": "ms/RHS", "n_gpus": 1, "steps": steps, "warmup": max(args.warmup, 3),
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded Kuhn-cube mesh, two layers and a resistive block)",
            "config": {"workload": "csem_p1_16cubed_two_layer_block (24,576 tets, 31,024 DOFs)", "p": 1,
                       "tets": mesh.T, "dofs": mesh.N, "nnz": mesh.nnz, "receivers": len(model.receivers)},
            "setup_ms": round(setup_ms, 1),
            "assembly": {"ms_per_step": round(asm_ms, 4), "Melem_per_s": round(mesh.T / asm_ms / 1e3, 2),
                         "arithmetic": "fp64"},
            "solve": gm, "other_solvers": others, "cpu_baseline": cpu}


def run_config3(args):
    """Adjoint gradient workload: 24^3 cubes (82,944 tets, p = 2), m = log10
    sigma per element, 100 receivers, misfit sum |E - d|^2 with d = E(m) plus
    10 % complex Gaussian noise (seed 4).  Times the gradient (forward solve,
    G^T conj(E - d), adjoint solve, per-element contraction) at rtol 1e-8, then
    checks it against central differences (step 1e-6) on 20 random elements
    (seed 7) and on the 4 elements of largest gradient, with solves at 1e-11."""
    import torch
    from petgem_gb300 import synthetic
    from petgem_gb300.adjoint import ReceiverMisfit
    from petgem_gb300.engine import DeviceMesh
    n = args.n if args.n != 32 else 24
    model = synthetic.config3(n)
    mesh = DeviceMesh(model.nodes, model.tets, 2)
    m = torch.as_tensor(model.m, dtype=torch.float64, device="cuda")
    # observed data: the model's own fields with 10 % complex noise
    probe = ReceiverMisfit(mesh, model.source, model.receivers, np.zeros((len(model.receivers), 3), complex),
                           rtol=1e-11, precision="df64", precond="grad")
    _, (_, _, u, r, keep) = probe.evaluate(m)
    E = r.cpu().numpy()                                   # E - 0 at the kept receivers
    rng = np.random.default_rng(4)
    noisy = E * (1.0 + 0.1 * (rng.standard_normal(E.shape) + 1j * rng.standard_normal(E.shape)))
    d = np.zeros((len(model.receivers), 3), complex)
    d[keep.cpu().numpy()] = noisy
    out = {}
    prob = ReceiverMisfit(mesh, model.source, model.receivers, d, rtol=1e-8, precision="df64", precond="grad")
    prob.value_and_gradient(m)                            # warm-up (autotuning, allocations)
    torch.cuda.synchronize()
    t = time.time()
    phi, g = prob.value_and_gradient(m)
    torch.cuda.synchronize()
    t_grad = time.time() - t
    its = [i.iterations for i in prob.last_info[-2:]]
    torch.cuda.synchronize()
    t = time.time()
    prob.evaluate(m)
    torch.cuda.synchronize()
    t_fwd = time.time() - t
    out["gradient_seconds"] = round(t_grad, 3)
    out["forward_seconds"] = round(t_fwd, 3)
    out["solve_iterations_forward_adjoint"] = its
    # central differences with tight solves
    tight = ReceiverMisfit(mesh, model.source, model.receivers, d, rtol=1e-11, precision="df64", max_it=400000,
                             precond="grad")
    phi_t, g_t = tight.value_and_gradient(m)
    g_np = g_t.cpu().numpy()
    h = 1e-6
    rnd = np.random.default_rng(7).choice(mesh.T, 20, replace=False)
    top = np.argsort(-np.abs(g_np))[:4]

    def fd(e):
        mp, mm = m.clone(), m.clone()
        mp[e] += h
        mm[e] -= h
        return (tight.evaluate(mp)[0].item() - tight.evaluate(mm)[0].item()) / (2 * h)
    fd_rnd = np.array([fd(int(e)) for e in rnd])
    fd_top = np.array([fd(int(e)) for e in top])
    # directional derivative along a seeded random direction over all
    # elements: grad . v against (phi(m + h v) - phi(m - h v)) / 2h
    v = torch.as_tensor(np.random.default_rng(8).standard_normal(mesh.T), device="cuda")
    dphi = float(torch.dot(g_t, v))
    directional = {"direction": "v ~ N(0, 1) per element, seed 8", "grad_dot_v": dphi}
    for hd in (1e-4, 1e-5):
        fdd = (tight.evaluate(m + hd * v)[0].item() - tight.evaluate(m - hd * v)[0].item()) / (2 * hd)
        directional[f"rel_err_h{hd:g}"] = abs(fdd - dphi) / abs(dphi)
    directional["passed_1e-5"] = bool(min(directional["rel_err_h0.0001"], directional["rel_err_h1e-05"]) <= 1e-5)
    out["directional_check"] = directional
    err_rnd = float(np.linalg.norm(fd_rnd - g_np[rnd]) / np.linalg.norm(g_np[rnd]))
    err_top = float(np.max(np.abs(fd_top - g_np[top]) / np.abs(g_np[top])))
    gmax = float(np.max(np.abs(g_np)))
    out["fd_check"] = {"step": h, "solve_rtol": 1e-11, "random_elements": 20,
                       "rel_err_random_normwise": err_rnd,
                       # the random elements' gradients lie far below the largest: a step of 1e-6 moves phi
                       # less than the solves' own error there, so their differences are measured against
                       # the gradient's scale
                       "max_abs_err_random_over_max_gradient": float(np.max(np.abs(fd_rnd - g_np[rnd]))) / gmax,
                       "max_abs_gradient_random_over_max_gradient": float(np.max(np.abs(g_np[rnd]))) / gmax,
                       "top_gradient_elements": 4,
                       "rel_err_top_max": err_top,
                       "gradient_at_1e-8_vs_1e-11": float(torch.linalg.norm(g - g_t) / torch.linalg.norm(g_t))}
    return {"metric": "seconds per adjoint gradient (forward + adjoint solve + contraction), p = 2",
            "value": round(t_grad, 3), "unit": "s", "n_gpus": 1, "steps": 1, "warmup": 1,
            "ms_per_step": round(t_grad * 1e3, 1), "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "df64 solves (f32 pairs; Jacobi + gradient correction), FP64 contraction",
            "data": "synthetic",
            "config": {"workload": f"adjoint_p2_{n}cubed (m = log10 sigma ~ U[-2, 0.5], seed 3; 100 receivers; "
                                   f"d = E(m) with 10 % complex noise, seed 4)", "tets": mesh.T, "dofs": mesh.N,
                       "phi": float(phi)},
            "detail": out}


def run_config4(args):
    """p = 3 MT configuration: 40^3 cubes (384,000 tets, 7.2 M DOFs, 611 M
    stored entries): mesh setup, assembly (double-float and FP64), the MT
    right-hand side of both polarisations, and their solve at 1 Hz and 0.1 Hz:
    one batched FP64 COCG per frequency with Jacobi plus the gradient
    correction (no PEC: the boundary DOFs are unknowns, so every gradient
    column is kept), aiming at a 1e-8 true residual; with air at 1e-8 S/m
    the true residual has an FP64 floor (~eps |A| |x| / |b|, reported), and a
    solve that reaches it first stops with status -7 (attainable accuracy);
    receivers' apparent resistivity and phase as petgem's computeImpedance."""
    import torch
    from petgem_gb300 import synthetic
    from petgem_gb300.engine import DeviceMesh
    n = args.n if args.n != 32 else 40
    model = synthetic.config4(n)
    t0 = time.time()
    mesh = DeviceMesh(model.nodes, model.tets, 3)
    mesh.records()
    mesh.tables_entry_major("df64")
    torch.cuda.synchronize()
    setup_ms = (time.time() - t0) * 1e3
    sigma = mesh.sigma_tensor(model.sigma)
    out = {}
    for ar in ("df64", "fp64"):
        coef = torch.empty((mesh.T, 12, 2) if ar == "df64" else (mesh.T, 12),
                           dtype=torch.float32 if ar == "df64" else torch.float64, device="cuda")
        vals = torch.empty(mesh.nnz, dtype=torch.complex128, device="cuda")

        def step():
            mesh.element_coefficients(sigma, 1.0, out=coef, check=False, arithmetic=ar)
            mesh.assemble(sigma, 1.0, out=vals, coef=coef, arithmetic=ar)
        for _ in range(max(args.warmup, 1)):
            step()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        steps = max(1, min(args.steps, 20))
        e0.record()
        for _ in range(steps):
            step()
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        out[ar] = {"ms_per_step": round(ms, 3), "Melem_per_s": round(mesh.T / ms / 1e3, 2)}
        del coef, vals
    mesh.mt_rhs(model.sigma, 1.0, ("x", "y"))         # boundary setup + first use
    torch.cuda.synchronize()
    t = time.time()
    mesh.mt_rhs(model.sigma, 1.0, ("x", "y"))
    torch.cuda.synchronize()
    out["mt_rhs_two_polarizations_ms"] = round((time.time() - t) * 1e3, 1)
    if args.solve == "all":
        from petgem_gb300.engine import MU0
        from petgem_gb300.pipeline import computeImpedance
        torch.cuda.synchronize()
        t = time.time()
        gmap = mesh.gradient_map(pec=False)
        torch.cuda.synchronize()
        out["gradient_map"] = {"ms": round((time.time() - t) * 1e3, 1), "columns": gmap.n_cols, "entries": gmap.nnz}
        solves = {}
        for f in model.frequencies:
            vals = mesh.assemble(sigma, f, arithmetic="fp64")
            B = mesh.mt_rhs(model.sigma, f, ("x", "y"))
            torch.cuda.synchronize()
            t = time.time()
            X, info = mesh.solve(vals, B, rtol=1e-8, ksp="cocg", precond="grad", pec=False, max_it=args.max_it,
                                 raise_on_fail=False)
            # the FP64 floor of the true residual: b - A x cannot be evaluated
            # below ~eps |A| |x| (the air's gradient components of x are huge)
            amax = float(vals.abs().max())
            floor = [2.0 ** -52 * amax * float(torch.linalg.norm(X[:, j])) / float(torch.linalg.norm(B[:, j]))
                     for j in range(2)]
            torch.cuda.synchronize()
            dt = time.time() - t
            Fs = [mesh.receiver_fields(X[:, k].contiguous(), model.receivers, f)[0].cpu().numpy() for k in range(2)]
            rho, phase, _, _ = computeImpedance(Fs, 2.0 * np.pi * f, MU0)
            solves[f"{f:g}Hz"] = {
                "ksp": "cocg", "precision": "fp64", "precond": "grad", "nrhs": 2, "seconds": round(dt, 3),
                "s_per_polarization": round(dt / 2, 3), "iterations": info.iterations,
                "ms_per_iteration": round(dt * 1e3 / max(info.iterations, 1), 3),
                "relres_per_polarization": info.relres_per_rhs, "converged": info.status == 0,
                "status": info.status, "fp64_residual_floor_eps_Amax_x_over_b": floor,
                "receivers": len(Fs[0]),
                "apparent_resistivity_xy_ohm_m": [float(np.min(rho[1])), float(np.median(rho[1])), float(np.max(rho[1]))],
                "phase_xy_deg": [float(np.min(phase[1])), float(np.median(phase[1])), float(np.max(phase[1]))],
                "stats_are": "min, median, max over the receivers"}
            del vals, B, X
        out["solve"] = solves
    return {"metric": "p=3 Melem/s assembled (MT configuration)", "value": out["df64"]["Melem_per_s"],
            "unit": "Melem/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "dtype": "df64 (f32 pairs) -> f64", "data": "synthetic",
            "config": {"workload": f"mt_p3_{n}cubed (box [-5000,5000]^2 x [-5000,2000] m, air / 2 layers / "
                                   f"3 ellipsoids)", "tets": mesh.T, "dofs": mesh.N, "nnz": mesh.nnz,
                       "setup_ms": round(setup_ms, 1), "orientation_tuples": mesh.n_tuples,
                       "device_memory_gb": round(torch.cuda.max_memory_allocated() / 1e9, 1)},
            "detail": out}


def run_config2(args):
    """Batched workload: the 24^3 two-layer mesh at 4 frequencies (one matrix
    each) x 16 x-HEDs, plus 8 extra meshes of 8^3..20^3 cubes (sizes drawn by
    seed 2) x 16 x-HEDs at 1 Hz: 12 systems x 16 right-hand sides, p = 2, to a
    1e-8 FP64 true residual.  Timed as one several-systems double-float COCG
    (every launch serves all systems) and, for comparison, as one batched COCG
    per system run back to back (same arithmetic and preconditioner), with
    Jacobi plus the gradient correction (the value) and with entity
    block-Jacobi."""
    import torch
    from petgem_gb300 import synthetic
    from petgem_gb300.engine import DeviceMesh, solve_csr_segments
    n = args.n if args.n != 32 else 24
    k = 16
    srcs = synthetic.config2_sources()                       # 64 x-HEDs, x in [-800, 800]
    freqs = [0.25, 0.5, 1.0, 2.0]
    entries = []                                             # (mesh, vals, b, label)

    def rhs(mesh, group, f):
        B = torch.zeros((mesh.N, k), dtype=torch.complex128, device="cuda")
        for j, s in enumerate(group):
            s = dict(s, frequency=f)
            bj = torch.zeros(mesh.N, dtype=torch.complex128, device="cuda")
            mesh.source_rhs(s, mesh.locate_source(s), bj)
            B[:, j] = bj
        mesh.pec_rhs(B)
        if not bool((torch.linalg.norm(B, dim=0) > 0).all()):
            raise RuntimeError("a source was not located in the mesh (zero right-hand side)")
        return B
    main_model = synthetic.config2(n)
    main = DeviceMesh(main_model.nodes, main_model.tets, 2)
    for i, f in enumerate(freqs):
        entries.append((main, main.assemble(main_model.sigma, f, pec=True), rhs(main, srcs[i::4], f),
                        f"{n}^3 at {f} Hz"))
    extra_sizes = synthetic.config2_extra_sizes()
    for ne in extra_sizes:
        em = synthetic.config2_extra(ne)
        mesh = DeviceMesh(em.nodes, em.tets, 2)
        entries.append((mesh, mesh.assemble(em.sigma, 1.0, pec=True), rhs(mesh, srcs[::4], 1.0), f"{ne}^3 at 1 Hz"))
    systems = [(m.rowptr, m.col, v, b) for m, v, b, _ in entries]
    blocks = (2, [(m.nE, m.nF, m.T) for m, _, _, _ in entries])
    rows = sum(m.N for m, _, _, _ in entries)
    nnz = sum(m.nnz for m, _, _, _ in entries)
    torch.cuda.synchronize()
    # warm-up: autotuning, graph capture paths and allocator (short, capped solves)
    solve_csr_segments(systems, blocks=blocks, rtol=1e-8, max_it=64, raise_on_fail=False)
    torch.cuda.synchronize()
    t = time.time()
    xs, info = solve_csr_segments(systems, blocks=blocks, rtol=1e-8, max_it=args.max_it, raise_on_fail=False)
    torch.cuda.synchronize()
    t_seg = time.time() - t
    per_system = []
    t_sep = 0.0
    for j, (m, v, b, label) in enumerate(entries):
        torch.cuda.synchronize()
        t = time.time()
        x1, i1 = m.solve(v, b, rtol=1e-8, ksp="cocg", precision="df64", max_it=args.max_it, raise_on_fail=False)
        torch.cuda.synchronize()
        dt = time.time() - t
        t_sep += dt
        r = b - m.spmv(v, xs[j])
        rr = (torch.linalg.norm(r, dim=0) / torch.linalg.norm(b, dim=0)).max().item()
        per_system.append({"system": label, "dofs": m.N, "iterations_batched": max(info.its_per_rhs[j]),
                           "iterations_alone": i1.iterations, "seconds_alone": round(dt, 3),
                           "true_relres_batched": rr, "converged_alone": i1.status == 0})
    n_rhs = len(entries) * k
    ms_rhs_bj = t_seg * 1e3 / n_rhs
    # the same batch with the gradient correction (one map per mesh, built once)
    grads = [m.gradient_map() for m, _, _, _ in entries]
    solve_csr_segments(systems, rtol=1e-8, max_it=64, raise_on_fail=False, gradients=grads)
    torch.cuda.synchronize()
    t = time.time()
    xg, info_g = solve_csr_segments(systems, rtol=1e-8, max_it=args.max_it, raise_on_fail=False, gradients=grads)
    torch.cuda.synchronize()
    t_seg_g = time.time() - t
    t_sep_g = 0.0
    for j, (m, v, b, label) in enumerate(entries):
        torch.cuda.synchronize()
        t = time.time()
        _, ig1 = m.solve(v, b, rtol=1e-8, ksp="cocg", precision="df64", precond="grad", max_it=args.max_it,
                         raise_on_fail=False)
        torch.cuda.synchronize()
        t_sep_g += time.time() - t
        r = b - m.spmv(v, xg[j])
        per_system[j]["grad"] = {"iterations_batched": max(info_g.its_per_rhs[j]),
                                 "iterations_alone": ig1.iterations,
                                 "true_relres_batched": (torch.linalg.norm(r, dim=0)
                                                         / torch.linalg.norm(b, dim=0)).max().item()}
    ms_rhs = t_seg_g * 1e3 / n_rhs
    # the extra meshes alone: small systems, where one solve per system is launch-latency bound
    n_main = len(freqs)
    torch.cuda.synchronize()
    t = time.time()
    _, info_x = solve_csr_segments(systems[n_main:], blocks=(2, blocks[1][n_main:]), rtol=1e-8, max_it=args.max_it,
                                   raise_on_fail=False)
    torch.cuda.synchronize()
    t_seg_x = time.time() - t
    t_sep_x = sum(p["seconds_alone"] for p in per_system[n_main:])
    # the same small meshes with one source each: latency-bound when solved one by one
    one = [(rp, c, v, b[:, 0].contiguous()) for rp, c, v, b in systems[n_main:]]
    torch.cuda.synchronize()
    t = time.time()
    _, info_1 = solve_csr_segments(one, blocks=(2, blocks[1][n_main:]), rtol=1e-8, max_it=args.max_it,
                                   raise_on_fail=False)
    torch.cuda.synchronize()
    t_seg_1 = time.time() - t
    t_sep_1 = 0.0
    for (m, v, b, _), (_, _, _, b1) in zip(entries[n_main:], one):
        torch.cuda.synchronize()
        t = time.time()
        m.solve(v, b1, rtol=1e-8, ksp="cocg", precision="df64", max_it=args.max_it, raise_on_fail=False)
        torch.cuda.synchronize()
        t_sep_1 += time.time() - t
    return {"metric": "ms/RHS to 1e-8, batched workload (several meshes and frequencies in one solve)",
            "value": round(ms_rhs, 2), "unit": "ms/RHS", "n_gpus": 1, "steps": 1, "warmup": 1,
            "ms_per_step": round(t_seg_g * 1e3, 1), "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "df64 (f32 pairs), FP64 true residual", "data": "synthetic",
            "config": {"workload": f"csem_p2_{n}cubed two-layer at {freqs} Hz + extra meshes {extra_sizes}^3 at 1 Hz, "
                                   f"{k} x-HEDs each (x in [-800, 800] m, z = 50 m)",
                       "systems": len(entries), "rhs_per_system": k, "rows": rows, "nnz": nnz,
                       "preconditioner": "Jacobi + gradient correction per system (value); entity block-Jacobi "
                                         "per system beside it"},
            "batched": {"seconds": round(t_seg_g, 3), "iterations": info_g.iterations, "status": info_g.status,
                        "worst_relres": info_g.relres},
            "one_solve_per_system": {"seconds": round(t_sep_g, 3), "ms_per_rhs": round(t_sep_g * 1e3 / n_rhs, 2)},
            "speedup_batched_vs_one_per_system": round(t_sep_g / max(t_seg_g, 1e-9), 2),
            "block_jacobi": {"ms_per_rhs": round(ms_rhs_bj, 2), "batched_seconds": round(t_seg, 3),
                             "iterations": info.iterations, "status": info.status, "worst_relres": info.relres,
                             "one_solve_per_system_seconds": round(t_sep, 3),
                             "speedup_batched_vs_one_per_system": round(t_sep / max(t_seg, 1e-9), 2)},
            "speedup_grad_vs_block_jacobi": round(t_seg / max(t_seg_g, 1e-9), 2),
            "extra_meshes_only": {"systems": len(entries) - n_main, "batched_seconds": round(t_seg_x, 3),
                                  "one_solve_per_system_seconds": round(t_sep_x, 3),
                                  "speedup": round(t_sep_x / max(t_seg_x, 1e-9), 2), "status": info_x.status},
            "extra_meshes_one_rhs": {"systems": len(one), "batched_seconds": round(t_seg_1, 3),
                                     "one_solve_per_system_seconds": round(t_sep_1, 3),
                                     "speedup": round(t_sep_1 / max(t_seg_1, 1e-9), 2), "status": info_1.status},
            "per_system": per_system}


def main():
    args = parse()
    if args.config == 0:
        if int(os.environ.get("RANK", 0)) == 0:
            print(json.dumps(run_config0(args)), flush=True)
        return
    if args.config == 2:
        if int(os.environ.get("RANK", 0)) == 0:
            print(json.dumps(run_config2(args)), flush=True)
        return
    if args.config == 3:
        if int(os.environ.get("RANK", 0)) == 0:
            print(json.dumps(run_config3(args)), flush=True)
        return
    if args.config == 4:
        if int(os.environ.get("RANK", 0)) == 0:
            print(json.dumps(run_config4(args)), flush=True)
        return
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local_rank = int(os.environ.get("LOCAL_RANK", 0))
    if args.impl == "reference":
        line = run_reference(args, rank)
        if line is not None:
            print(json.dumps(line), flush=True)
        return
    line = run_gpu(args, rank, world, local_rank)
    if rank == 0 and line is not None:
        if not args.no_cpu_baseline:
            from petgem_gb300 import synthetic
            cores = os.cpu_count() or 1
            rate, n_el, wall = cpu_assembly_rate(synthetic.config1(args.n), args.cpu_seconds, cores)
            line["cpu_baseline"] = {"value": round(rate, 6), "unit": "Melem/s", "cores": cores, "kind": "port",
                                    "sample": f"oracle assembly of {n_el} elements of the same mesh, "
                                              f"{cores} processes, {wall:.1f} s"}
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
