"""Autotuner: picks the assembly variant of a mesh by timing the candidates.

Candidates (all produce results within the stated tolerances; the FP64 gather is
the only bit-exact one, so a caller that needs bit-exactness keeps it):

* FP32: kernel 0 (per-element gradient records + one thread per entry) or kernel 1
  (spatial row tiles, gradients in shared memory) with tile sizes
  (rows, elements) from TILE_CANDIDATES;
* FP64: strategy gather / atomic / scatter (colour-ordered);
* node numbering: identity, reverse Cuthill-McKee, Morton or recursive coordinate
  bisection (`tune_renumbering`; the caller applies the permutation, since it
  renumbers the output);
* FP32 sliver threshold (`tune_sliver_threshold`): the lowest quality threshold
  (fewest FP64 gradient evaluations, so the fastest) whose assembly meets an
  error target against the mesh's own FP64 assembly;
* batches (`tune_batch`): one FP32 tile size for all meshes of a batch, timed on
  the whole batch (its persistent kernel sizes shared memory for the largest
  tile of any mesh).

Each candidate runs `repeats` times after one warm-up; the median of the per-step
device times (CUDA events recorded by the library around its launches) decides.
Choices are cached in a JSON file keyed by the mesh sizes, operator, precision
and device name, so a re-run on the same mesh reuses them without timing.
"""
from __future__ import annotations

import json
import os
import statistics

TILE_CANDIDATES = [(40, 448), (48, 512), (48, 544), (56, 576), (64, 640), (96, 960)]


def _device_name(device: int) -> str:
    try:
        import torch
        return torch.cuda.get_device_name(device)
    except Exception:
        return "cuda"


def _time(asm, op, precision, strategy, repeats):
    asm.assembly(op, precision, strategy, prec=True)   # warm-up (and plan build)
    asm.synchronize()
    times = []
    for _ in range(repeats):
        asm.profile(True)
        asm.assembly(op, precision, strategy, prec=True)
        rec = asm.profile_read()
        asm.profile(False)
        times.append(sum(t for _, t in rec))
    return statistics.median(times)


def tune(asm, op: str, precision: str, repeats: int = 3, cache: str | None = None,
         device: int = 0, strategies=None, kernels=(0, 1)) -> dict:
    """Time the candidates on `asm` (mesh, pattern, coefficients already set),
    apply the fastest and return {"choice": ..., "ms": ..., "timings": [...]}.
    `kernels` restricts the FP32 kernels tried (the batch runs tiles only)."""
    key = f"{asm.nbElem}:{asm.nbNodes}:{asm.nbEdges}:{op}:{precision}:{_device_name(device)}"
    db = {}
    if cache and os.path.exists(cache):
        with open(cache) as f:
            db = json.load(f)
        if key in db:
            _apply(asm, db[key]["choice"])
            return db[key]
    timings = []
    if precision == "fp32":
        if 0 in kernels:
            asm.set_option("fp32_kernel", 0)
            timings.append(({"fp32_kernel": 0, "strategy": "gather"},
                            _time(asm, op, "fp32", "gather", repeats)))
        for rows, elems in (TILE_CANDIDATES if 1 in kernels else ()):
            asm.set_option("fp32_kernel", 1)
            asm.set_option("tile_rows", rows)
            asm.set_option("tile_elems", elems)
            try:
                t = _time(asm, op, "fp32", "gather", repeats)
            except Exception:
                continue   # a tile that cannot hold one row's elements
            timings.append(({"fp32_kernel": 1, "tile_rows": rows, "tile_elems": elems,
                             "strategy": "gather"}, t))
    else:
        for s in (strategies or ("gather", "atomic", "scatter")):
            if s == "scatter":
                asm.coloring_creation(seed=0)
            timings.append(({"strategy": s}, _time(asm, op, "fp64", s, repeats)))
    choice, ms = min(timings, key=lambda x: x[1])
    _apply(asm, choice)
    out = {"choice": choice, "ms": ms, "timings": [[c, t] for c, t in timings]}
    if cache:
        db[key] = out
        tmp = cache + ".tmp"
        with open(tmp, "w") as f:
            json.dump(db, f, indent=1)
        os.replace(tmp, cache)
    return out


def _apply(asm, choice: dict):
    for k in ("fp32_kernel", "tile_rows", "tile_elems"):
        if k in choice:
            asm.set_option(k, choice[k])


THRESHOLDS = (0.05, 0.1, 0.15, 0.2, 0.3, 0.4)


def tune_sliver_threshold(asm, op: str, row, col, target: float = 1e-6, repeats: int = 3,
                          candidates=THRESHOLDS) -> dict:
    """The lowest FP32 quality threshold whose assembly is within `target` of
    the FP64 assembly (max entry error relative to the diagonal scale, the
    measure of minifem.metrics.entry_errors), for the mesh, pattern (row, col as
    create_nodeToNode returned them) and coefficients already set on `asm`.
    Applies and returns {"choice", "ms", "errors": {threshold: error}}; if no
    candidate meets the target, the most accurate one."""
    from . import metrics
    dim = 1 if op == "lap" else 9
    asm.assembly(op, "fp64", "gather", prec=True)
    ref = asm.values()
    errors, times = {}, {}
    for q in sorted(candidates):
        asm.set_sliver_threshold(q)
        times[q] = _time(asm, op, "fp32", "gather", repeats)
        asm.assembly(op, "fp32", "gather", prec=True)
        errors[q] = metrics.entry_errors(row, col, ref, asm.values(), dim)["max_rel_diag_scaled"]
        if errors[q] <= target:
            break
    ok = [q for q in errors if errors[q] <= target]
    choice = min(ok) if ok else min(errors, key=errors.get)
    asm.set_sliver_threshold(choice)
    return {"choice": choice, "ms": times[choice], "target": target,
            "errors": {str(q): e for q, e in errors.items()},
            "timings": {str(q): t for q, t in times.items()}}


BATCH_TILE_CANDIDATES = [(40, 448), (48, 512), (48, 544), (56, 576)]


def tune_batch(items, repeats: int = 3, device: int = 0,
               candidates=BATCH_TILE_CANDIDATES) -> dict:
    """One FP32 tile size (rows, elements) for every mesh of a batch: the batch's
    persistent kernel lays its shared memory out for the largest tile of any of
    its meshes, so a size that suits one mesh alone can cost every other tile an
    SM slot; the candidates are therefore timed on the whole batch.  `items` are
    (Assembler, op, coefSets) as Batch.add takes them; for each candidate the size
    is applied to every context, a batch is built and its FP32 replay timed (host
    wall time around replay + synchronise, median of `repeats` after one
    warm-up).  Applies the fastest to the contexts and returns {"choice",
    "timings"}; the caller builds its batch afterwards."""
    import time
    from .api import Batch
    timings = []
    for rows, elems in candidates:
        for asm, _, _ in items:
            asm.set_option("fp32_kernel", 1)
            asm.set_option("tile_rows", rows)
            asm.set_option("tile_elems", elems)
        b = Batch(device)
        try:
            for asm, op, cs in items:
                b.add(asm, op, cs)
            b.assemble("fp32", prec=True)
            b.synchronize()
            ts = []
            for _ in range(repeats):
                t0 = time.perf_counter()
                b.assemble("fp32", prec=True)
                b.synchronize()
                ts.append(time.perf_counter() - t0)
            timings.append(({"fp32_kernel": 1, "tile_rows": rows, "tile_elems": elems},
                            statistics.median(ts) * 1e3))
        except Exception:
            continue   # a tile that cannot hold one row's elements
        finally:
            b.close()
    choice, ms = min(timings, key=lambda x: x[1])
    for asm, _, _ in items:
        _apply(asm, choice)
    return {"choice": choice, "ms": ms, "timings": [[c, t] for c, t in timings]}


RENUMBERINGS = ("identity", "rcm", "morton", "bisection")


def tune_renumbering(mesh, op: str, precision: str = "fp32", repeats: int = 3, device: int = 0,
                     candidates=RENUMBERINGS) -> dict:
    """Time one assembly (+ preconditioner) of `mesh` (a meshgen.Mesh) under each
    node renumbering and return {"choice", "newOfOld" (None for identity), "ms",
    "timings"}; every candidate is assembled on its own context."""
    from .api import Assembler
    from .meshgen import renumber_nodes
    base = Assembler(device)
    base.set_mesh(mesh.coord, mesh.elemToNode)
    base.create_nodeToNode("sorted")
    perms = {"identity": None}
    if "rcm" in candidates:
        perms["rcm"] = base.rcm_permutation()
    for kind in ("morton", "bisection"):
        if kind in candidates:
            perms[kind] = base.locality_permutation(kind)
    base.close()
    timings = []
    for name in candidates:
        p = perms[name]
        m = mesh if p is None else renumber_nodes(mesh, p)
        a = Assembler(device)
        try:
            a.set_mesh(m.coord, m.elemToNode)
            a.create_nodeToNode("sorted")
            if m.coef is not None:
                a.set_coefficients(op, m.coef)
            timings.append((name, _time(a, op, precision, "gather", repeats)))
        finally:
            a.close()
    choice, ms = min(timings, key=lambda x: x[1])
    return {"choice": choice, "newOfOld": perms[choice], "ms": ms,
            "timings": [[n, t] for n, t in timings]}
