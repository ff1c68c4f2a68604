"""Shared helpers of the halo tests: the reference's domain-decomposed flow
(per-rank assembly, prec_init, MPI_halo_exchange, prec_inversion; src/FEM.cc:177-234,
src/halo.cc:39-122) restated serially on the oracle."""
import numpy as np

import pyoracle as O


class OracleBlocks:
    """pack / add of the oracle's restatement of src/halo.cc on numpy blocks,
    exposed as torch CPU tensors (for the gloo transport)."""

    def __init__(self, p, intfIndex, intfNodes, op):
        import torch
        self.torch = torch
        self.p, self.op = p, op
        self.intfIndex = np.ascontiguousarray(intfIndex, np.int32)
        self.intfNodes = np.ascontiguousarray(intfNodes, np.int32)

    def pack(self, dim):
        return self.torch.from_numpy(O.halo_pack(self.p, self.intfIndex, self.intfNodes, self.op).copy())

    def empty_like(self, buf):
        return self.torch.empty_like(buf)

    def add(self, recv):
        O.halo_add(self.p, self.intfIndex, self.intfNodes, recv.numpy(), self.op)


def rank_blocks(dom, op):
    """One rank's oracle assembly and prec_init: (row, col, values, prec blocks, markf)."""
    m = dom.mesh
    row, col = O.pattern(m.elemToNode, m.nbNodes)
    vals = O.assembly(m.coord, row, col, m.elemToNode, int(row[-1]), op, m.coef)
    p = O.prec_blocks(vals, row, col, m.nbNodes, op)
    return row, col, vals, p, O.checkbounds(m.boundNodesCode)


def oracle_flow(domains, op, invert=True):
    """Every rank's preconditioner after the reference's halo sum (and inversion)."""
    per = [rank_blocks(d, op) for d in domains]
    sends = [O.halo_pack(b[3], d.intfIndex, d.intfNodes, op) for d, b in zip(domains, per)]
    dim = O.op_dim(op)
    out = []
    for d, b in zip(domains, per):
        recv = np.zeros_like(sends[d.rank])
        for i, q in enumerate(d.neighbors):
            nq = domains[int(q)]
            k = int(np.nonzero(nq.neighbors == d.rank)[0][0])
            recv[d.intfIndex[i] * dim:d.intfIndex[i + 1] * dim] = \
                sends[int(q)][nq.intfIndex[k] * dim:nq.intfIndex[k + 1] * dim]
        p = b[3].copy()
        O.halo_add(p, d.intfIndex, d.intfNodes, recv, op)
        if invert:
            O.prec_invert(p, b[0], b[1], b[4], d.mesh.nbNodes, op)
        out.append(p)
    return out
