"""The device halo sum (mfem_set_interfaces / mfem_halo_pack / mfem_halo_add)
against the oracle's restatement of the reference's domain-decomposed flow
(src/FEM.cc:177-234 with MPI_halo_exchange, src/halo.cc:39-122): every
sub-domain assembled on the GPU, packed, exchanged (loopback: all sub-domains
in this process, on one GPU), summed and inverted."""
import numpy as np
import pytest

import pyoracle as O
from halo_common import oracle_flow
from minifem.meshgen import cube_mesh, split_domains

pytestmark = pytest.mark.gpu


def _rank(dom, op, precision):
    import minifem
    from minifem.halo import DeviceBlocks, HaloExchange
    m = dom.mesh
    a = minifem.Assembler(0)
    a.set_mesh(m.coord, m.elemToNode)
    a.create_nodeToNode("sorted")
    a.set_coefficients(op, m.coef)
    a.set_check_bounds(O.checkbounds(m.boundNodesCode))
    a.assembly(op, precision, "gather")
    a.prec_init()
    x = HaloExchange(DeviceBlocks(a, dom.intfIndex, dom.intfNodes), dom.neighbors, O.op_dim(op))
    return a, x


@pytest.mark.parametrize("op", ["lap", "ela"])
@pytest.mark.parametrize("nb", [2, 4])
def test_device_halo_sum_bit_exact(op, nb):
    from minifem.halo import loopback_exchange
    doms = split_domains(cube_mesh(10, seed=4, op=op), nb)
    ranks = [_rank(d, op, "fp64") for d in doms]
    loopback_exchange([x for _, x in ranks], [d.rank for d in doms])
    expect = oracle_flow(doms, op)
    for d, (a, _) in zip(doms, ranks):
        a.prec_inversion()
        assert a.prec().tobytes() == expect[d.rank].tobytes(), f"rank {d.rank}"
        a.close()


def test_device_halo_fp32_blocks():
    """FP32 assembly: the blocks are the FP32 diagonal values widened to FP64;
    after the sum and the FP64 inversion they agree with the FP64 flow within
    the FP32 tolerance of the preconditioner."""
    from minifem.halo import loopback_exchange
    op = "ela"
    doms = split_domains(cube_mesh(10, seed=6, op=op), 4)
    ranks = [_rank(d, op, "fp32") for d in doms]
    loopback_exchange([x for _, x in ranks], [d.rank for d in doms])
    expect = oracle_flow(doms, op)
    for d, (a, _) in zip(doms, ranks):
        a.prec_inversion()
        got, ref = a.prec().reshape(-1, 9), expect[d.rank].reshape(-1, 9)
        scale = np.abs(ref).max(axis=1, keepdims=True)
        assert np.all(np.abs(got - ref) <= 1e-4 * scale)
        a.close()


def test_halo_needs_blocks_before_inversion():
    import minifem
    op = "lap"
    d = split_domains(cube_mesh(6, seed=1, op=op), 2)[0]
    a, x = _rank(d, op, "fp64")
    a.prec_inversion()           # blocks already inverted: the sum would be wrong
    with pytest.raises(minifem.MfemError, match="prec_init"):
        x.blocks.pack(1)
    a.close()
