"""Pipelined steps (mfem_step_async / mfem_wait): host inputs in, host results
out on a second stream, two device result slots.  Every step's results must be
bit-identical to a synchronous assembly of the same inputs, whatever the
overlap with the steps around it."""
import numpy as np
import pytest

import pyoracle as O
from minifem.meshgen import cube_mesh

pytestmark = pytest.mark.gpu


def _inputs(m, k):
    """Step k's inputs: the mesh moved by a small seeded displacement and
    rescaled coefficients, so that every step has different results."""
    rng = np.random.default_rng(100 + k)
    coord = np.ascontiguousarray(m.coord + 1e-3 * rng.standard_normal(m.coord.shape) / 10)
    coef = np.ascontiguousarray(m.coef * (1.0 + 0.1 * k))
    return coord, coef


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_pipelined_steps_equal_synchronous(gpu, precision):
    m = cube_mesh(10, seed=21, op="ela")
    dt = np.float32 if precision == "fp32" else np.float64
    a = gpu(0)
    a.set_mesh(m.coord, m.elemToNode)
    a.create_nodeToNode("sorted")
    a.set_check_bounds(O.checkbounds(m.boundNodesCode))
    a.set_coefficients("ela", m.coef)
    nnz9, n9 = a.nbEdges * 9, a.nbNodes * 9
    steps = 5
    inputs = [_inputs(m, k) for k in range(steps)]
    # two host buffer sets, reused every second step as the API allows
    vals = [np.empty(nnz9, dt) for _ in range(2)]
    precs = [np.empty(n9) for _ in range(2)]
    got = []
    tickets = []
    for k in range(steps):
        if k >= 2:
            a.wait(tickets[k - 2])
            got.append((vals[k % 2].copy(), precs[k % 2].copy()))
        coord, coef = inputs[k]
        tickets.append(a.step_async("ela", precision, vals[k % 2], precs[k % 2], coord=coord, coef=coef))
    for k in range(steps - 2, steps):
        a.wait(tickets[k])
        got.append((vals[k % 2].copy(), precs[k % 2].copy()))
    # the synchronous getters read the latest step
    last = a.values_f32() if precision == "fp32" else a.values()
    assert last.tobytes() == got[-1][0].tobytes()

    # reference: one synchronous assembly per step's inputs on a fresh context
    b = gpu(0)
    b.set_mesh(m.coord, m.elemToNode)
    b.create_nodeToNode("sorted")
    b.set_check_bounds(O.checkbounds(m.boundNodesCode))
    for k in range(steps):
        coord, coef = inputs[k]
        b.update_coords(coord)
        b.set_coefficients("ela", coef)
        b.assembly("ela", precision, "gather", prec=True)
        v = b.values_f32() if precision == "fp32" else b.values()
        assert v.tobytes() == got[k][0].tobytes(), f"values of step {k}"
        assert b.prec().tobytes() == got[k][1].tobytes(), f"preconditioner of step {k}"
    # steps differ from one another (the test would be vacuous otherwise)
    assert got[0][0].tobytes() != got[1][0].tobytes()


def test_synchronous_call_after_pipelined_steps(gpu):
    """A synchronous assembly after pipelined steps writes the current slot only
    after its copy-out finished; the copied-out results stay intact."""
    m = cube_mesh(8, seed=5, op="ela")
    a = gpu(0)
    a.set_mesh(m.coord, m.elemToNode)
    a.create_nodeToNode("sorted")
    a.set_check_bounds(O.checkbounds(m.boundNodesCode))
    a.set_coefficients("ela", m.coef)
    v = np.empty(a.nbEdges * 9)
    t = a.step_async("ela", "fp64", v)
    a.set_coefficients("ela", m.coef * 2.0)
    a.assembly("ela", "fp64", "gather", prec=True)
    a.wait(t)
    a.set_coefficients("ela", m.coef)
    a.assembly("ela", "fp64", "gather", prec=True)
    assert a.values().tobytes() == v.tobytes()
    with pytest.raises(Exception):
        a.wait(5)          # unknown ticket


def test_pipelined_precision_switch(gpu):
    """FP32, FP64, FP32 steps back to back: the slot that grows for FP64 values is
    reallocated only after its copy-out, and every step's results stay exact."""
    m = cube_mesh(8, seed=9, op="ela")
    a = gpu(0)
    a.set_mesh(m.coord, m.elemToNode)
    a.create_nodeToNode("sorted")
    a.set_check_bounds(O.checkbounds(m.boundNodesCode))
    a.set_coefficients("ela", m.coef)
    n9 = a.nbEdges * 9
    outs = [np.empty(n9, np.float32), np.empty(n9), np.empty(n9, np.float32)]
    precs = [np.empty(a.nbNodes * 9) for _ in range(3)]
    kinds = ["fp32", "fp64", "fp32"]
    tickets = [a.step_async("ela", k, v, p) for k, v, p in zip(kinds, outs, precs)]
    for t in tickets:
        a.wait(t)
    for k, v, p in zip(kinds, outs, precs):
        a.assembly("ela", k, "gather", prec=True)
        ref = a.values_f32() if k == "fp32" else a.values()
        assert ref.tobytes() == v.tobytes()
        assert a.prec().tobytes() == p.tobytes()
