"""Benchmark: elasticity assembly + block-Jacobi preconditioner of the 100^3-node
jittered, node-permuted Kuhn cube (1,000,000 nodes, 5,821,794 tets,
14,761,198 CSR entries of 3x3 blocks) with per-element E and nu, one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

A step is one assembly + prec_init + prec_inversion of the whole mesh (what one
iteration of the reference's FEM loop times, src/FEM.cc:177-234).  `value` is
the FP32 path (FP32 arithmetic and values, Kahan-compensated sums, FP64
slivers and block inversion) with inputs resident in HBM; the plain FP64
bit-exact path is reported beside it (`fp64_plain`).  `e2e` runs the same FP32
step through the C ABI with host buffers: coordinates and coefficients copied
in, values and preconditioner copied out, every step -- pipelined
(mfem_step_async: step k's copy-out overlaps step k+1's copy-in and assembly),
with the synchronous form (one call after the other) reported beside it.  The L2 cache (129 MB) is
flushed before every timed step by writing a 512 MB buffer; each step is timed
alone with CUDA events on the library's stream.

--impl reference times the oracle port of the reference's CPU path (serial, as
the reference's REF build is) on the same mesh; it is the reported baseline.
With N > 1 (torchrun) every rank assembles its own mesh (weak scaling, no
exchange: the preconditioner halo sum is a no-op at one rank per domain).
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

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "mini-fem_gb300"))

import numpy as np  # noqa: E402

N_SIDE = 100      # nodes per side of the benchmark cube (--side changes it for small cases)
SEED = 2024
WORKLOAD = "ela_cube100_5.8M_tets"
METRIC = "ela assembly Melem/s @5.8M tets: FP32-batched vs FP64-plain; % HBM roofline"


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for nme, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nme)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def step_bytes(E, N, nnz, fp32):
    """Algorithmic bytes of one assembly + preconditioner step (ela):
    16E connectivity + 3N coordinates + E coefficients + 64E (16 CSR positions
    per element) + nnz*9 values + N*9*8 preconditioner."""
    w = 4 if fp32 else 8
    c = 8 if fp32 else 16
    return 16 * E + 3 * N * w + c * E + 64 * E + nnz * 9 * w + N * 9 * 8


def kernel_bytes(name, E, N, nnz, n_edge_units, fp32):
    """Algorithmic bytes of one launch of the named kernel: its inputs read once
    and its outputs written once."""
    rec = 64 if fp32 else 128
    w = 4 if fp32 else 8
    contrib_edge = 6 * E
    if name.startswith("edge_units"):
        return (n_edge_units * (8 + 8) + 4 * contrib_edge + rec * E
                + 2 * n_edge_units * 9 * w)
    if name.startswith("diag_units"):
        b = N * (4 + 8) + 4 * 4 * E + rec * E + N * 9 * w
        if "prec" in name:
            b += N * 9 * 8 + N
        return b
    if name.startswith("tile32"):
        # the tile kernel is the whole step but the coordinate split: the step's bytes
        return step_bytes(E, N, nnz, fp32)
    if name.startswith("grad"):
        coordb = 32 * N if fp32 else 24 * N
        return 16 * E + coordb + (8 if fp32 else 16) * E + rec * E
    return None


# DRAM bytes per element of one launch, from `ncu --set full` captures of the 60^3
# cube (profiles/tile32_ela_cube60.md, profiles/fp64_units_ela_cube60.md:
# dram__bytes_read.sum + dram__bytes_write.sum divided by its 1,232,274 tets);
# traffic grows in proportion to the mesh, so the full launch's traffic is this
# times E.
TRAFFIC_PER_ELEM = {"tile32+prec": (145.482752e6 + 94.085376e6) / 1232274,
                    "edge_units64": (282.084864e6 + 198.790656e6) / 1232274}

# FP64-pipe thread instructions per element of each FP64 gather kernel (ela with
# coefficients), from one ncu capture of the 60^3 cube
# (sm__thread_inst_executed_pipe_fp64_pred_on.sum / 1,232,274 tets;
# profiles/fp64_pipe_ela_cube60.md).  Every count is a fixed number per element,
# per contribution or per node, so it grows in proportion to the mesh.
FP64_OPS_PER_ELEM = {"grad64": 42221856 / 1232274,
                     "diag_units64+prec": 91199200 / 1232274,
                     "edge_units64": 143159136 / 1232274}


_MESHGEN = None


def meshgen():
    """The mesh generator (minifem/meshgen.py, numpy only) loaded as a standalone
    module by file path: the reference arm must not import the minifem package,
    whose __init__ loads the GPU library."""
    global _MESHGEN
    if _MESHGEN is None:
        import importlib.util
        path = os.path.join(ROOT, "mini-fem_gb300", "minifem", "meshgen.py")
        spec = importlib.util.spec_from_file_location("minifem_meshgen_standalone", path)
        mod = importlib.util.module_from_spec(spec)
        sys.modules[spec.name] = mod    # dataclasses resolve their module through sys.modules
        spec.loader.exec_module(mod)
        _MESHGEN = mod
    return _MESHGEN


def make_mesh(rank):
    return meshgen().cube_mesh(N_SIDE, seed=SEED + rank, op="ela")


def workload_name():
    return WORKLOAD if N_SIDE == 100 else f"ela_cube{N_SIDE}_{meshgen().cube_sizes(N_SIDE)[0]}_tets"


def bench_config(E, N, nnz, world):
    """The workload, identical on both arms (ours and --impl reference)."""
    return {"workload": workload_name(), "nbElem": E, "nbNodes": N, "nbEdges": nnz,
            "operator": "ela", "coefficients": "per element: E log-uniform [1e9,2e11], "
                                             "nu U[0.2,0.35]",
            "l2": "GPU arm: the 129 MB L2 flushed (512 MB write) before every timed "
                  "device step; end-to-end steps move 720 MB+ through the host link",
            "parallelism": f"replicas x{world}"}


def native_libs_loaded():
    """Shared objects of this repository mapped into this process."""
    try:
        with open("/proc/self/maps") as f:
            maps = f.read()
    except OSError:
        return []
    return sorted({ln.split()[-1] for ln in maps.splitlines()
                   if ln.split() and ln.split()[-1].endswith(".so") and ROOT in ln.split()[-1]})


def max_over_ranks(values, world, device):
    """Each timing's maximum over the ranks (all_reduce MAX; every rank gets it).
    `device` is where the reduction tensor lives: the rank's GPU under NCCL,
    "cpu" under gloo."""
    if world == 1:
        return list(values)
    import torch
    t = torch.tensor(values, device=device, dtype=torch.float64)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return t.tolist()


def run_ours(args, rank, world, local_rank):
    import torch
    import minifem
    import pyoracle as O  # noqa: F401  (only for checkBounds + the CPU baseline leg)

    torch.cuda.set_device(local_rank)
    mesh = make_mesh(rank)
    E, N = mesh.nbElem, mesh.nbNodes
    # setup, once per mesh (host wall time, each step synchronised): mesh upload,
    # CSR pattern, FP32 tile plan, FP64 gather plan (inside the first FP64
    # assembly, less a steady one), colouring
    setup = {}
    a = minifem.Assembler(local_rank)
    t0 = time.perf_counter()
    a.set_mesh(mesh.coord, mesh.elemToNode)
    a.synchronize()
    setup["set_mesh_s"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    row, col = a.create_nodeToNode("sorted")
    setup["create_nodeToNode_s"] = time.perf_counter() - t0
    nnz = len(col)
    a.set_coefficients("ela", mesh.coef)
    markf = O.checkbounds(mesh.boundNodesCode)
    a.set_check_bounds(markf)
    t0 = time.perf_counter()
    a.tile_info()
    setup["tile_plan_s"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    a.assembly("ela", "fp64", "gather", prec=True)
    a.synchronize()
    first64 = time.perf_counter() - t0
    t0 = time.perf_counter()
    a.assembly("ela", "fp64", "gather", prec=True)
    a.synchronize()
    setup["gather_plan_s"] = first64 - (time.perf_counter() - t0)
    t0 = time.perf_counter()
    ncolors = a.coloring_creation(seed=1)[1].size - 1
    setup["coloring_s"] = time.perf_counter() - t0
    setup = {k: round(v, 4) for k, v in setup.items()}
    setup["colours"] = ncolors
    stream = torch.cuda.ExternalStream(a.stream)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local_rank}")

    def timed(precision, steps, warmup, e2e=False, hostbuf=None):
        for _ in range(warmup):
            one(precision, e2e, hostbuf)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        evs = []
        t0 = time.perf_counter()
        for _ in range(steps):
            with torch.cuda.stream(stream):
                flush.fill_(1.0)
                s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                s.record(stream)
            one(precision, e2e, hostbuf)
            with torch.cuda.stream(stream):
                e.record(stream)
            evs.append((s, e))
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        if world > 1:
            torch.distributed.barrier()
        ms = [s.elapsed_time(e) for s, e in evs]
        return ms, wall

    def one(precision, e2e, hb):
        if not e2e:
            a.assembly("ela", precision, "gather", prec=True)
            return
        # host buffers in, host buffers out, through the C ABI
        a.update_coords(hb["coord"])
        a.set_coefficients("ela", hb["coef"])
        a.assembly("ela", precision, "gather", prec=True)
        minifem._native.lib.mfem_get_values_f32(a._h, hb["vals"].ctypes.data_as(minifem.api.C.c_void_p))
        minifem._native.lib.mfem_get_prec(a._h, hb["prec"].ctypes.data_as(minifem.api.C.c_void_p))

    # pinned host buffers for the end-to-end leg
    pin = lambda arr: torch.from_numpy(arr).pin_memory().numpy()  # noqa: E731
    hb = {"coord": pin(np.ascontiguousarray(mesh.coord)), "coef": pin(np.ascontiguousarray(mesh.coef)),
          "vals": pin(np.empty(nnz * 9, np.float32)), "prec": pin(np.empty(N * 9, np.float64))}

    with ClockSampler(local_rank) as clk:
        ms32, _ = timed("fp32", args.steps, args.warmup)
        ms64, _ = timed("fp64", args.steps, args.warmup)
    e2e_ms, e2e_wall = timed("fp32", args.steps, max(1, args.warmup // 2), e2e=True, hostbuf=hb)

    # end to end, pipelined (mfem_step_async / mfem_wait): step k's results are
    # copied out while step k+1's inputs are copied in and assembled; two pinned
    # host buffer sets, each step still copies its own inputs in and results out
    hbs = [{"vals": pin(np.empty(nnz * 9, np.float32)), "prec": pin(np.empty(N * 9, np.float64))}
           for _ in range(2)]

    def pipelined(steps):
        tickets = []
        for k in range(steps):
            if k >= 2:
                a.wait(tickets[k - 2])
            h = hbs[k % 2]
            tickets.append(a.step_async("ela", "fp32", h["vals"], h["prec"],
                                        coord=hb["coord"], coef=hb["coef"]))
        for t in tickets[-2:]:
            a.wait(t)

    def timed_pipelined(steps, warmup):
        pipelined(max(3, warmup))
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        with torch.cuda.stream(stream):
            ps, pe = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ps.record(stream)
        pipelined(steps)
        with torch.cuda.stream(stream):
            pe.record(stream)
        torch.cuda.synchronize()
        return ps.elapsed_time(pe) / steps

    pipe_ms = timed_pipelined(args.steps, args.warmup)
    d2h32 = int(hbs[0]["vals"].nbytes + hbs[0]["prec"].nbytes)

    # the same end-to-end steps with the bit-exact FP64 path (FP64 values out):
    # the like-for-like counterpart of the reference's FP64 CPU step
    e2e_prec = "fp64"
    hbs = [{"vals": pin(np.empty(nnz * 9, np.float64)), "prec": pin(np.empty(N * 9, np.float64))}
           for _ in range(2)]

    def pipelined(steps):  # noqa: F811  (same loop, FP64 values)
        tickets = []
        for k in range(steps):
            if k >= 2:
                a.wait(tickets[k - 2])
            h = hbs[k % 2]
            tickets.append(a.step_async("ela", e2e_prec, h["vals"], h["prec"],
                                        coord=hb["coord"], coef=hb["coef"]))
        for t in tickets[-2:]:
            a.wait(t)

    pipe64_ms = timed_pipelined(args.steps, args.warmup)
    d2h64 = int(hbs[0]["vals"].nbytes + hbs[0]["prec"].nbytes)
    del hbs

    # per-kernel durations (a separate, untimed pass with events per launch)
    prof = {}
    for prec in ("fp32", "fp64"):
        a.profile(True)
        for _ in range(3):
            with torch.cuda.stream(stream):
                flush.fill_(1.0)
            a.assembly("ela", prec, "gather", prec=True)
        rec = a.profile_read()
        a.profile(False)
        agg = {}
        for nme, t in rec:
            agg.setdefault(nme, []).append(t)
        prof[prec] = {k: sum(v) / len(v) for k, v in agg.items()}
    flagged = a.flagged()
    fp64_peak = a.fp64_rate("add")

    # accuracy of the FP32 step against the FP64 one (the FP64 gather equals the
    # oracle bit for bit), untimed
    from minifem import metrics
    a.assembly("ela", "fp64", "gather", prec=True)
    v64, p64 = a.values(), a.prec()
    a.assembly("ela", "fp32", "gather", prec=True)
    v32, p32 = a.values(), a.prec()
    errors = metrics.entry_errors(row, col, v64, v32, 9)
    errors["preconditioned_operator_rel"] = metrics.operator_error(row, col, v64, p64, v32, p32, 9)
    del v64, p64, v32, p32

    # FP32 after reverse Cuthill-McKee renumbering of the nodes
    from minifem.meshgen import renumber_nodes
    rmesh = renumber_nodes(mesh, a.rcm_permutation())
    ar = minifem.Assembler(local_rank)
    ar.set_mesh(rmesh.coord, rmesh.elemToNode)
    ar.create_nodeToNode("sorted")
    ar.set_coefficients("ela", rmesh.coef)
    ar.set_check_bounds(O.checkbounds(rmesh.boundNodesCode))
    rstream = torch.cuda.ExternalStream(ar.stream)
    for _ in range(args.warmup):
        ar.assembly("ela", "fp32", "gather", prec=True)
    rms = []
    for _ in range(args.steps):
        with torch.cuda.stream(rstream):
            flush.fill_(1.0)
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record(rstream)
        ar.assembly("ela", "fp32", "gather", prec=True)
        with torch.cuda.stream(rstream):
            e.record(rstream)
        rms.append((s, e))
    torch.cuda.synchronize()
    t_rcm = statistics.mean(x.elapsed_time(y) for x, y in rms)
    # its accuracy against the FP64 assembly of the same renumbered mesh
    rrow, rcol = ar.create_nodeToNode("sorted")
    ar.assembly("ela", "fp32", "gather", prec=True)
    rv32 = ar.values()
    ar.assembly("ela", "fp64", "gather", prec=True)
    rcm_errors = metrics.entry_errors(rrow, rcol, ar.values(), rv32, 9, raw=False)
    del rv32
    ar.close()

    # the batched FP32 form on the same mesh: 8 coefficient sets per iteration,
    # one CUDA graph replay (coordinate split, weights, one persistent tile
    # kernel that computes each tile's gradients once for all sets)
    from minifem.meshgen import coefficient_set
    n_sets = 8
    coefs = np.stack([mesh.coef] + [coefficient_set("ela", E, SEED + 100 * s) for s in range(1, n_sets)])
    bt = minifem.Batch(local_rank)
    bt.add(a, "ela", coefs)
    t_batch = _timer(torch, torch.cuda.ExternalStream(bt.stream), flush)(
        lambda: bt.assemble("fp32", prec=True), args.steps, args.warmup)
    # accuracy of three of the sets against their FP64 assemblies
    bt.assemble("fp32", prec=True)
    bt.synchronize()
    batch_errors = {}
    for s in (0, n_sets // 2, n_sets - 1):
        a.set_coefficients("ela", coefs[s])
        a.assembly("ela", "fp64", "gather", prec=True)
        batch_errors[f"set_{s}"] = metrics.entry_errors(row, col, a.values(),
                                                        bt.values(0, s, "fp32"), 9, raw=False)
    a.set_coefficients("ela", mesh.coef)
    bt.close()

    # maximum over ranks
    t32, t64, te2e, pipe_ms, pipe64_ms, t_batch = max_over_ranks(
        [statistics.mean(ms32), statistics.mean(ms64), statistics.mean(e2e_ms), pipe_ms, pipe64_ms,
         t_batch], world, f"cuda:{local_rank}")
    if rank != 0:
        return None

    hbm, peak_kind = peaks()
    # edge units: upper off-diagonal entries
    n_edge = (nnz - N) // 2

    def roofline(prec, step_ms):
        fp32 = prec == "fp32"
        ks = prof[prec]
        # the longest region among the kernels with an algorithmic byte count
        known = [k for k in ks if kernel_bytes(k, E, N, nnz, n_edge, fp32) is not None]
        dom = max(known, key=ks.get)
        kb = kernel_bytes(dom, E, N, nnz, n_edge, fp32)
        ach = kb / (ks[dom] * 1e-3) / 1e9
        sb = step_bytes(E, N, nnz, fp32)
        tr = TRAFFIC_PER_ELEM.get(dom)
        return ({"bound": "hbm", "kernel": dom, "achieved": round(ach, 1), "peak": hbm,
                 "unit": "GB/s", "frac": round(ach / hbm, 4),
                 "traffic": round(tr * E) if tr else None,
                 "algorithmic_bytes": kb, "launch_ms": round(ks[dom], 4),
                 "peak_kind": peak_kind},
                {"algorithmic_bytes": sb, "GB/s": round(sb / (step_ms * 1e-3) / 1e9, 1),
                 "frac": round(sb / (step_ms * 1e-3) / 1e9 / hbm, 4)})

    r32, s32 = roofline("fp32", t32)
    r64, s64 = roofline("fp64", t64)
    # the FP64 step against the FP64 pipe, its actual bound: FP64-pipe operations
    # of the dominant kernel and of the whole step against the measured rate
    ks64 = prof["fp64"]
    ops = {k: FP64_OPS_PER_ELEM[k] * E for k in FP64_OPS_PER_ELEM if k in ks64}
    dom64 = max(ops, key=lambda k: ks64[k])
    r64["fp64_pipe"] = {
        "bound": "fp64", "kernel": dom64,
        "achieved": round(ops[dom64] / (ks64[dom64] * 1e-3) / 1e9, 1),
        "peak": round(fp64_peak / 1e9, 1), "unit": "Gop/s",
        "frac": round(ops[dom64] / (ks64[dom64] * 1e-3) / fp64_peak, 4),
        "ops_per_launch": round(ops[dom64]), "launch_ms": round(ks64[dom64], 4),
        "step": {"ops": round(sum(ops.values())),
                 "achieved": round(sum(ops.values()) / (t64 * 1e-3) / 1e9, 1),
                 "frac": round(sum(ops.values()) / (t64 * 1e-3) / fp64_peak, 4)},
        "peak_kind": "measured on this GPU by mfem_fp64_rate (independent FP64 additions "
                     "on every SM, best of 3 launches)",
        "ops_source": "FP64-pipe thread instructions per element from ncu at 60^3, times E"}
    melem = lambda ms: world * E / (ms * 1e-3) / 1e6  # noqa: E731
    out = {
        "metric": METRIC, "value": round(melem(t32), 1), "unit": "Melem/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(t32, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: jittered (+-0.2h), node-permuted 100^3 Kuhn cube, E log-uniform "
                "[1e9,2e11], nu U[0.2,0.35], seeded",
        "config": bench_config(E, N, nnz, world),
        "precision": "fp32 (Kahan-compensated sums, fp64 slivers + fp64 block inverse); the "
                     "bit-exact fp64 path is `fp64_plain`, with its own end-to-end figure",
        "strategy": "gather",
        "roofline": r32, "step_roofline": s32,
        "fp64_plain": {"value": round(melem(t64), 1), "unit": "Melem/s", "ms_per_step": round(t64, 4),
                       "bit_exact": "gather, -fmad=false", "roofline": r64, "step_roofline": s64,
                       "e2e": {"value": round(melem(pipe64_ms), 1), "unit": "Melem/s",
                               "ms_per_step": round(pipe64_ms, 4),
                               "h2d_bytes_per_step": int(hb["coord"].nbytes + hb["coef"].nbytes),
                               "d2h_bytes_per_step": d2h64,
                               "path": "C ABI: mfem_step_async(MFEM_FP64) + mfem_wait, pinned host "
                                       "buffers, FP64 values and preconditioner out, pipelined as "
                                       "`e2e`"}},
        "fp32_over_fp64": round(t64 / t32, 2),
        "fp32_errors_vs_fp64": errors,
        "fp32_rcm": {"value": round(melem(t_rcm), 1), "unit": "Melem/s", "ms_per_step": round(t_rcm, 4),
                     "renumbering": "reverse Cuthill-McKee (mfem_rcm_permutation)",
                     "errors_vs_fp64": rcm_errors},
        "fp32_batched": {"value": round(n_sets * melem(t_batch), 1), "unit": "Melem/s",
                         "ms_per_step": round(t_batch, 4), "coefficient_sets": n_sets,
                         "counts": "element-assemblies: elements x coefficient sets",
                         "launch": "mfem_batch_assemble: one CUDA graph replay, one persistent tile "
                                   "kernel over every tile x 8 sets",
                         "errors_vs_fp64": batch_errors},
        "kernels_ms": prof,
        "setup": setup,
        "sliver_gradient_evaluations": flagged,
        "e2e": {"value": round(melem(pipe_ms), 1), "unit": "Melem/s", "ms_per_step": round(pipe_ms, 4),
                "h2d_bytes_per_step": int(hb["coord"].nbytes + hb["coef"].nbytes),
                "d2h_bytes_per_step": d2h32,
                "path": "C ABI: mfem_step_async + mfem_wait, pinned host buffers; the copy-out of "
                        "step k overlaps the copy-in and assembly of step k+1 (CUDA events around "
                        f"{args.steps} steps, last copy-out included)",
                "l2": "not flushed: every step copies 720 MB in and out, more than the 129 MB L2",
                "synchronous": {"value": round(melem(te2e), 1), "unit": "Melem/s",
                                "ms_per_step": round(te2e, 4),
                                "path": "C ABI: mfem_update_coords + mfem_set_coefficients + "
                                        "mfem_assemble_prec + mfem_get_values_f32 + mfem_get_prec"}},
        "gpu_launches": None,
        "clocks": clk.summary(),
    }
    # own kernels launched per timed FP32 step: coordinate split + weights, tile kernel
    out["gpu_launches"] = 2 * args.steps
    if args.cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(mesh, markf, args.cpu_iters)
    a.close()
    return out


def time_port(mesh, row, col, markf, iters, threads):
    """Seconds per full iteration (assembly + prec_init + prec_inversion) of the
    oracle port on `threads` host threads."""
    import pyoracle as O
    E, N = mesh.nbElem, mesh.nbNodes
    nnz = int(row[-1])
    O.set_threads(threads)
    t = []
    for _ in range(iters):
        t0 = time.perf_counter()
        vals = O.assembly(mesh.coord, row, col, mesh.elemToNode, nnz, "ela", mesh.coef)
        O.prec(vals, row, col, markf, N, "ela")
        t.append(time.perf_counter() - t0)
    return statistics.mean(t)


def host_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_baseline(mesh, markf, iters):
    """Oracle port of the reference's path (bit-identical to the reference's own
    operators), timed on this host as its two CPU builds run it
    (src/assembly.cc:647-673): `ref` -- every loop serial, one core;
    `coloring` -- the matrix reset and the preconditioner loops on every host
    core, the element loop serial (its per-element pragma is disabled in the
    shipped source, src/assembly.cc:362,516).  `value` is the faster of the two."""
    import pyoracle as O
    E, N = mesh.nbElem, mesh.nbNodes
    # the port's own pattern (reference column order), as the reference builds it
    prow, pcol = O.pattern(mesh.elemToNode, N)
    cores = host_cores()
    builds = {}
    for name, thr in (("ref", 1), ("coloring", cores)):
        sec = time_port(mesh, prow, pcol, markf, iters, thr)
        builds[name] = {"value": round(E / sec / 1e6, 3), "unit": "Melem/s", "cores": thr,
                        "s_per_iteration": round(sec, 3)}
    best = max(builds, key=lambda b: builds[b]["value"])
    return {"value": builds[best]["value"], "unit": "Melem/s", "cores": builds[best]["cores"],
            "kind": "port", "build": best, "builds": builds,
            "sample": f"{iters} full iterations (assembly + prec_init + prec_inversion) of the "
                      f"same {E}-tet mesh per build; ref: 1 core, coloring: {cores} cores for "
                      f"the reset and preconditioner loops, element loop serial"}


def run_reference(args, rank, world):
    """The reference's CPU path (the oracle port, bit-identical to the reference's
    own operators) on this host, as its COLORING/OMP build runs it: element loop
    serial, matrix reset and preconditioner loops on every host core.  Loads no
    library of the GB300 implementation (checked before timing)."""
    if rank != 0:
        return None
    import pyoracle as O
    mesh = make_mesh(0)
    E, N = mesh.nbElem, mesh.nbNodes
    row, col = O.pattern(mesh.elemToNode, N)
    nnz = int(row[-1])
    markf = O.checkbounds(mesh.boundNodesCode)
    cores = host_cores()
    O.set_threads(cores)
    libs = native_libs_loaded()
    if any("libminifem_gb300" in x for x in libs):
        raise RuntimeError(f"reference arm has the GPU library loaded: {libs}")

    def step():
        vals = O.assembly(mesh.coord, row, col, mesh.elemToNode, nnz, "ela", mesh.coef)
        O.prec(vals, row, col, markf, N, "ela")

    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    sec = (time.perf_counter() - t0) / args.steps
    v = round(E / sec / 1e6, 3)
    return {"metric": METRIC, "value": v, "unit": "Melem/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(sec * 1e3, 2), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": bench_config(E, N, nnz, world),
            "impl": "reference",
            "native_libs_loaded": native_libs_loaded(),
            "cpu_baseline": {"value": v, "unit": "Melem/s", "cores": cores, "kind": "port",
                             "build": "coloring",
                             "sample": "full mesh per step; element loop serial as in every "
                                       "reference build on this path (the COLORING build "
                                       "disables the per-element pragma, src/assembly.cc:362,"
                                       "516), matrix reset and preconditioner loops on every "
                                       "host core as in the reference's OMP builds"},
            "e2e": {"value": v, "unit": "Melem/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


# ---- supplementary workloads (--workload): the other benchmark configurations ----

def _timer(torch, stream, flush):
    def run(fn, steps, warmup):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        evs = []
        for _ in range(steps):
            with torch.cuda.stream(stream):
                flush.fill_(1.0)
                s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                s.record(stream)
            fn()
            with torch.cuda.stream(stream):
                e.record(stream)
            evs.append((s, e))
        torch.cuda.synchronize()
        return statistics.mean(x.elapsed_time(y) for x, y in evs)
    return run


def run_cube30(args, op, side=30):
    """side^3 cube (30^3: 146,334 tets), lap or ela: FP64 gather (bit-exact), colour
    scatter, atomics and FP32, with the oracle port timed beside them; the scatter
    and atomic results against the gather (max entry difference over the diagonal
    scale)."""
    import torch
    import minifem
    import pyoracle as O
    from minifem import metrics
    from minifem.meshgen import cube_mesh
    mesh = cube_mesh(side, seed=SEED, op=op)
    E, N = mesh.nbElem, mesh.nbNodes
    a = minifem.Assembler(0)
    a.set_mesh(mesh.coord, mesh.elemToNode)
    row, col = a.create_nodeToNode("reference")
    a.set_coefficients(op, mesh.coef)
    markf = O.checkbounds(mesh.boundNodesCode)
    a.set_check_bounds(markf)
    ncol = a.coloring_creation(seed=1)[1].size - 1
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda:0")
    timed = _timer(torch, torch.cuda.ExternalStream(a.stream), flush)
    res = {}
    dim = 1 if op == "lap" else 9
    a.assembly(op, "fp64", "gather", prec=True)
    gathered = a.values()
    for name, prec, strat in (("fp64_gather", "fp64", "gather"), ("fp64_scatter", "fp64", "scatter"),
                              ("fp64_atomic", "fp64", "atomic"), ("fp32_tiles", "fp32", "gather")):
        ms = timed(lambda: a.assembly(op, prec, strat, prec=True), args.steps, args.warmup)
        res[name] = {"ms_per_step": round(ms, 4), "value": round(E / (ms * 1e-3) / 1e6, 1)}
        if strat != "gather":
            res[name]["max_rel_diag_scaled_vs_gather"] = metrics.entry_errors(
                row, col, gathered, a.values(), dim)["max_rel_diag_scaled"]
    a.assembly(op, "fp64", "gather", prec=True)
    ref = O.full(mesh, op=op)
    bit_exact = (a.values().tobytes() == ref["values"].tobytes()
                 and a.prec().tobytes() == ref["prec"].tobytes())
    t = []
    for _ in range(max(3, args.cpu_iters)):
        t0 = time.perf_counter()
        v = O.assembly(mesh.coord, ref["row"], ref["col"], mesh.elemToNode, int(ref["row"][-1]), op,
                       mesh.coef)
        O.prec(v, ref["row"], ref["col"], markf, N, op)
        t.append(time.perf_counter() - t0)
    cpu = E / statistics.mean(t) / 1e6
    return {"metric": f"{op} assembly + preconditioner Melem/s @{E // 1000}k tets (FP64 gather)",
            "value": res["fp64_gather"]["value"], "unit": "Melem/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": res["fp64_gather"]["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"{op}_cube{side}_{E // 1000}k_tets", "nbElem": E, "nbNodes": N,
                       "nbEdges": len(col), "colours": ncol},
            "variants": res, "bit_exact_vs_oracle": bit_exact,
            "cpu_baseline": {"value": round(cpu, 3), "unit": "Melem/s", "cores": 1, "kind": "port",
                             "sample": f"{len(t)} iterations of the same mesh"}}


def run_stress(args):
    """60^3 stress cube (1,232,274 tets): jitter 0.45h, 5% slivers, E jump 1e6,
    nu up to 0.45; FP32 with double-float sliver gradients and an FP64 block inverse
    against all-FP64."""
    import torch
    import minifem
    import pyoracle as O
    from minifem import metrics
    from minifem.meshgen import cube_mesh
    mesh = cube_mesh(60, seed=SEED, op="ela", jitter=0.45, sliver_fraction=0.05, jump=1e6,
                     nu_max=0.45)
    E, N = mesh.nbElem, mesh.nbNodes
    a = minifem.Assembler(0)
    a.set_mesh(mesh.coord, mesh.elemToNode)
    row, col = a.create_nodeToNode("sorted")
    a.set_coefficients("ela", mesh.coef)
    a.set_check_bounds(O.checkbounds(mesh.boundNodesCode))
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda:0")
    timed = _timer(torch, torch.cuda.ExternalStream(a.stream), flush)
    t32 = timed(lambda: a.assembly("ela", "fp32", "gather", prec=True), args.steps, args.warmup)
    flagged = a.flagged()
    slots = a.tile_info()["tile_elems"]
    v32, p32 = a.values(), a.prec()
    # the threshold the tuner picks for a 1e-6 error target (the lowest that
    # meets it: fewest FP64 gradient evaluations)
    from minifem import autotune
    tuned = autotune.tune_sliver_threshold(a, "ela", row, col, target=1e-6)
    t32q = timed(lambda: a.assembly("ela", "fp32", "gather", prec=True), args.steps, args.warmup)
    flaggedq = a.flagged()
    v32q, p32q = a.values(), a.prec()
    a.set_sliver_threshold(0.1)
    t64 = timed(lambda: a.assembly("ela", "fp64", "gather", prec=True), args.steps, args.warmup)
    v64, p64 = a.values(), a.prec()
    err = metrics.entry_errors(row, col, v64, v32, 9)
    err["preconditioned_operator_rel"] = metrics.operator_error(row, col, v64, p64, v32, p32, 9)
    errq = metrics.entry_errors(row, col, v64, v32q, 9)
    errq["preconditioned_operator_rel"] = metrics.operator_error(row, col, v64, p64, v32q, p32q, 9)
    return {"metric": "ela stress mesh Melem/s @1.23M tets (FP32, double-float slivers, FP64 block inverse)",
            "value": round(E / (t32 * 1e-3) / 1e6, 1), "unit": "Melem/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(t32, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic: jitter 0.45h, slivers (aspect up to 1e4), E jump 1e6, nu <= 0.45",
            "config": {"workload": "ela_stress60_1.23M_tets", "nbElem": E, "nbNodes": N,
                       "nbEdges": len(col), "slivers_made": mesh.meta.get("slivers_made")},
            "quality_threshold": 0.1,
            "sliver_gradients": {"evaluations": flagged, "tile_element_slots": slots,
                                 "fraction": round(flagged / slots, 4),
                                 "note": "elements below the quality threshold, in double-float "
                                         "(FP64 below quality 1e-4); an element is evaluated once "
                                         "per tile that holds it"},
            "fp64_plain": {"value": round(E / (t64 * 1e-3) / 1e6, 1), "ms_per_step": round(t64, 4)},
            "fp32_errors_vs_fp64": err,
            "tuned_threshold": {"threshold": tuned["choice"], "target": tuned["target"],
                                "errors_by_threshold": tuned["errors"],
                                "value": round(E / (t32q * 1e-3) / 1e6, 1),
                                "ms_per_step": round(t32q, 4),
                                "sliver_gradient_fraction": round(flaggedq / slots, 4),
                                "fp32_errors_vs_fp64": errq}}


def run_solve(args):
    """Consumer of the 100^3 ela assembly: block-CSR SpMV (FP64 and FP32 values,
    FP64 vectors) with its bytes against the HBM peak, and block-Jacobi PCG to a
    relative residual of 1e-8 on the Dirichlet-constrained system."""
    import torch
    import minifem
    import pyoracle as O
    mesh = make_mesh(0)
    E, N = mesh.nbElem, mesh.nbNodes
    a = minifem.Assembler(0)
    a.set_mesh(mesh.coord, mesh.elemToNode)
    row, col = a.create_nodeToNode("sorted")
    nnz = len(col)
    a.set_coefficients("ela", mesh.coef)
    a.set_check_bounds(O.checkbounds(mesh.boundNodesCode))
    stream = torch.cuda.ExternalStream(a.stream)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda:0")
    timed = _timer(torch, stream, flush)
    x = torch.randn(3 * N, dtype=torch.float64, device="cuda:0")
    y = torch.empty_like(x)
    torch.cuda.synchronize()
    hbm, peak_kind = peaks()
    out = {}
    b = np.random.default_rng(SEED).standard_normal(3 * N)
    for prec in ("fp64", "fp32"):
        a.assembly("ela", prec, "gather", prec=True)
        a.synchronize()
        ms = timed(lambda: a.spmv(x.data_ptr(), y.data_ptr(), True), args.steps, args.warmup)
        w = 8 if prec == "fp64" else 4
        # values and columns once, row pointers, x once (gathers hit L2), y written
        byts = nnz * (9 * w + 4) + (N + 1) * 4 + 24 * N + 24 * N + N
        sol, it, rel = a.pcg(b, rtol=1e-8, max_iter=5000)
        t0 = time.perf_counter()
        sol, it, rel = a.pcg(b, rtol=1e-8, max_iter=5000)
        wall = time.perf_counter() - t0
        out[prec] = {"spmv_ms": round(ms, 4), "spmv_GBs": round(byts / (ms * 1e-3) / 1e9, 1),
                     "spmv_hbm_frac": round(byts / (ms * 1e-3) / 1e9 / hbm, 4),
                     "spmv_bytes": byts,
                     "spmv_arithmetic": "FP64 FMA chain, 9 per block" if prec == "fp64" else
                     "FP32 double-float (exact hi products, sums within 15 x 2^-48 of sum|a x|), "
                     "x split into hi/lo FP32 by one extra pass inside the timed call",
                     "pcg_iterations": it, "pcg_relres": rel, "pcg_s": round(wall, 4),
                     "pcg_ms_per_iteration": round(wall * 1e3 / max(it, 1), 4)}
    return {"metric": "ela 100^3 operator apply GB/s and block-Jacobi PCG (consumer of the assembly)",
            "value": out["fp32"]["spmv_GBs"], "unit": "GB/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": out["fp32"]["spmv_ms"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 values, f64 vectors",
            "data": "synthetic 100^3 ela cube as the benchmark line; b seeded N(0,1)",
            "config": {"workload": "ela_cube100_spmv_pcg", "nbNodes": N, "nbEdges": nnz,
                       "constrained": "check bounds as homogeneous Dirichlet",
                       "l2": "flushed before every timed SpMV"},
            "peak_GBs": hbm, "peak_kind": peak_kind, "fp64_values": out["fp64"],
            "fp32_values": out["fp32"]}


def run_renumber(args):
    """The 100^3 ela cube under each node renumbering the tuner compares:
    identity (the random numbering of the generator), reverse Cuthill-McKee,
    Morton and recursive coordinate bisection; FP32 and FP64 steps."""
    from minifem import autotune
    mesh = make_mesh(0)
    E = mesh.nbElem
    out = {}
    for prec in ("fp32", "fp64"):
        r = autotune.tune_renumbering(mesh, "ela", prec, repeats=max(3, args.steps))
        out[prec] = {"choice": r["choice"],
                     "ms_per_step": {n: round(t, 4) for n, t in r["timings"]},
                     "Melem_s": {n: round(E / (t * 1e-3) / 1e6, 1) for n, t in r["timings"]}}
    best = min(out["fp32"]["ms_per_step"].values())
    return {"metric": "ela 100^3 Melem/s per node renumbering (tuner candidates)",
            "value": round(E / (best * 1e-3) / 1e6, 1), "unit": "Melem/s", "n_gpus": 1,
            "steps": max(3, args.steps), "warmup": 1, "ms_per_step": best, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic 100^3 ela cube as the benchmark line",
            "config": {"workload": "ela_cube100_renumberings", "timing": "median of the library's "
                       "per-launch CUDA events, L2 not flushed"},
            "fp32": out["fp32"], "fp64": out["fp64"]}


def run_batch(args):
    """64 meshes, n ~ U{12..60} nodes per side (seeded), half lap half ela, 8
    coefficient sets each, re-assembled per iteration by one graph replay."""
    import torch
    import minifem
    import pyoracle as O
    from minifem.meshgen import cube_mesh, rng_u64
    from minifem import autotune, metrics
    sides = 12 + (rng_u64(SEED, 99, 64) % np.uint64(49)).astype(int)
    batch = minifem.Batch(0)
    asms, patterns, coefs, pending = [], [], [], []
    total_e = total_asm = 0
    for i, n in enumerate(sides):
        op = "lap" if i % 2 == 0 else "ela"
        meshes = [cube_mesh(int(n), seed=SEED + 1000 * i + s, op=op) for s in range(8)]
        m = meshes[0]
        a = minifem.Assembler(0)
        a.set_mesh(m.coord, m.elemToNode)
        patterns.append(a.create_nodeToNode("sorted"))
        a.set_check_bounds(O.checkbounds(m.boundNodesCode))
        a.set_coefficients(op, m.coef)
        coefs.append(np.stack([mm.coef for mm in meshes]))
        pending.append((a, op, coefs[-1]))
        asms.append((a, op))
        total_e += m.nbElem
        total_asm += 8 * m.nbElem
    # one tile size for the whole batch, timed on the batch
    t0 = time.perf_counter()
    tuned = autotune.tune_batch(pending, repeats=3)
    tune_s = time.perf_counter() - t0
    for (a, op), cs in zip(asms, coefs):
        batch.add(a, op, cs)
    info = batch.info()
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda:0")
    timed = _timer(torch, torch.cuda.ExternalStream(batch.stream), flush)
    t32 = timed(lambda: batch.assemble("fp32", prec=True), args.steps, args.warmup)
    t64 = timed(lambda: batch.assemble("fp64", prec=True), max(1, args.steps // 2), 1)
    batch.synchronize()
    # accuracy: FP32 sets of a sample of meshes against the FP64 batch (whose
    # gather is bit-exact against the oracle), every set of each sampled mesh
    batch.assemble("fp64", prec=True)
    batch.synchronize()
    v64 = {(i, s): batch.values(i, s, "fp64") for i in (0, 1, 62, 63) for s in range(8)}
    batch.assemble("fp32", prec=True)
    batch.synchronize()
    worst = {}
    for (i, s), ref in v64.items():
        row, col = patterns[i]
        e = metrics.entry_errors(row, col, ref, batch.values(i, s, "fp32"), O.op_dim(asms[i][1]),
                                 raw=False)
        w = worst.setdefault(f"mesh_{i}_{asms[i][1]}_n{int(sides[i])}", {"max_rel_diag_scaled": 0.0,
                                                                       "frobenius_rel": 0.0})
        for k in w:
            w[k] = max(w[k], e[k])
    return {"metric": "batched assembly + preconditioner, element-assemblies/s (64 meshes x 8 sets)",
            "value": round(total_asm / (t32 * 1e-3) / 1e6, 1), "unit": "Melem/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(t32, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic: 64 jittered permuted cubes, n ~ U{12..60}, half lap half ela, "
                    "8 coefficient sets each",
            "config": {"workload": "batch64x8", "meshes": len(sides), "sets": 8,
                       "elements": total_e, "element_assemblies": total_asm,
                       "tiles": info["work"], "persistent_grid": info["grid"],
                       "tuning": {"tile_size": tuned["choice"],
                                  "candidates_ms": [[f"{c['tile_rows']}x{c['tile_elems']}", round(t, 3)]
                                                    for c, t in tuned["timings"]],
                                  "seconds": round(tune_s, 2)},
                       "launch": "one CUDA graph per iteration; FP32 = one persistent kernel"},
            "fp64_plain": {"value": round(total_asm / (t64 * 1e-3) / 1e6, 1),
                           "ms_per_step": round(t64, 4)},
            "fp32_errors_vs_fp64": {"worst_over_8_sets": worst}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-baseline", type=int, default=1)
    ap.add_argument("--cpu-iters", type=int, default=3)
    ap.add_argument("--workload", default="ela100",
                    choices=["ela100", "ela30", "lap30", "strategies100", "stress60", "batch64",
                             "solve100", "renumber100"],
                    help="ela100: the benchmark line; the others: the remaining configurations")
    ap.add_argument("--side", type=int, default=N_SIDE,
                    help="nodes per cube side (100 = the benchmark mesh; smaller for profiling)")
    args = ap.parse_args()
    globals()["N_SIDE"] = args.side
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup
    sys.path.insert(0, os.path.join(ROOT, "oracle"))

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        backend = "nccl" if args.impl == "ours" else "gloo"
        if args.impl == "ours":
            torch.cuda.set_device(local_rank)
        torch.distributed.init_process_group(backend)
    try:
        if args.impl == "reference":
            out = run_reference(args, rank, world)
        elif args.workload == "ela100":
            out = run_ours(args, rank, world, local_rank)
        elif rank != 0:
            out = None
        elif args.workload in ("ela30", "lap30"):
            out = run_cube30(args, args.workload[:3])
        elif args.workload == "strategies100":
            out = run_cube30(args, "ela", side=100)
        elif args.workload == "stress60":
            out = run_stress(args)
        elif args.workload == "solve100":
            out = run_solve(args)
        elif args.workload == "renumber100":
            out = run_renumber(args)
        else:
            out = run_batch(args)
        if out is not None:
            print(json.dumps(out), flush=True)
    finally:
        if world > 1:
            import torch
            torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
