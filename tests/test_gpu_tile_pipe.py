"""The persistent, software-pipelined FP32 tile kernel (fp32_kernel 2) against
the one-CTA-per-tile kernel (fp32_kernel 1): the same tiles, contribution order
and arithmetic, so the same bits; the unit order grouped by store alignment
(unit_order 1) changes no bit either; and the pipelined kernel's bounded waits."""
import numpy as np
import pytest

import pyoracle as O
from minifem.meshgen import cube_mesh

pytestmark = pytest.mark.gpu


def _run(a, op, kernel, order=0):
    a.set_option("fp32_kernel", kernel)
    a.set_option("unit_order", order)
    a.assembly(op, "fp32", "gather", prec=True)
    return a.values_f32(), a.prec(), a.flagged()


@pytest.mark.parametrize("op,n,kw", [
    ("ela", 12, {}), ("lap", 12, {}), ("ela", 31, {}), ("lap", 4, {}),
    ("ela", 18, {"jitter": 0.45, "sliver_fraction": 0.05, "jump": 1e6, "nu_max": 0.45}),
])
def test_pipelined_equals_per_tile_kernel(gpu, op, n, kw):
    m = cube_mesh(n, seed=n, op=op, **kw)
    a = gpu(0)
    a.set_mesh(m.coord, m.elemToNode)
    a.create_nodeToNode("sorted")
    a.set_coefficients(op, m.coef)
    a.set_check_bounds(O.checkbounds(m.boundNodesCode))
    v1, p1, f1 = _run(a, op, 1)
    v2, p2, f2 = _run(a, op, 2)
    assert v2.tobytes() == v1.tobytes()
    assert p2.tobytes() == p1.tobytes()
    assert f2 == f1
    for kernel in (1, 2):
        v3, p3, _ = _run(a, op, kernel, order=1)
        assert v3.tobytes() == v1.tobytes() and p3.tobytes() == p1.tobytes()


def test_pipelined_small_tiles_many_per_cta(gpu):
    """Tiles much smaller than the default: every CTA walks many tiles."""
    m = cube_mesh(24, seed=3, op="ela")
    a = gpu(0)
    a.set_mesh(m.coord, m.elemToNode)
    a.create_nodeToNode("sorted")
    a.set_coefficients("ela", m.coef)
    a.set_option("tile_rows", 8)
    a.set_option("tile_elems", 160)
    v1, p1, _ = _run(a, "ela", 1)
    v2, p2, _ = _run(a, "ela", 2)
    assert v2.tobytes() == v1.tobytes() and p2.tobytes() == p1.tobytes()
    assert a.tile_info()["tiles"] > 152 * 4


def test_pipelined_bounded_wait(gpu):
    """A barrier that expects bytes that never arrive: the wait gives up, the
    next read reports MFEM_ERR_TIMEOUT, and the context assembles correctly
    afterwards.  No fault, no trap, no hang."""
    import minifem
    m = cube_mesh(6, seed=2, op="ela")
    a = gpu(0)
    a.set_mesh(m.coord, m.elemToNode)
    a.create_nodeToNode("reference")
    a.set_coefficients("ela", m.coef)
    a.set_option("fp32_kernel", 2)
    a.set_option("wait_limit", 200)
    a.set_option("test_missing_bytes", 16)
    a.assembly("ela", "fp32", "gather", prec=True)
    with pytest.raises(minifem.MfemError) as ei:
        a.values_f32()
    assert ei.value.code == -8
    a.set_option("test_missing_bytes", 0)
    a.set_option("wait_limit", 1 << 22)
    a.assembly("ela", "fp32", "gather", prec=True)
    v = a.values_f32().astype(np.float64)
    ref = O.full(m, op="ela")
    assert np.abs(v - ref["values"]).max() / np.abs(ref["values"]).max() < 1e-6
