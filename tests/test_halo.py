"""The halo sum of the domain-decomposed path on the CPU (src/halo.cc:39-122,
src/IO.cc:61-96): the domain split and its per-rank input files, the oracle's
restatement of MPI_halo_exchange against the undivided mesh, and the exchange
code path (minifem.halo.HaloExchange + TorchTransport) run by two and four gloo
ranks."""
import os
import socket

import numpy as np
import pytest

import pyoracle as O
from halo_common import OracleBlocks, oracle_flow, rank_blocks
from minifem.meshgen import cube_mesh, read_reference_input, split_domains, write_reference_tree


def _mesh(op, n=7, seed=3):
    return cube_mesh(n, seed=seed, op=op)


@pytest.mark.parametrize("nb", [2, 3, 4])
def test_split_is_a_partition_with_matching_interfaces(nb):
    m = _mesh("ela")
    doms = split_domains(m, nb)
    ge = np.sort(np.concatenate([d.globalElem for d in doms]))
    assert np.array_equal(ge, np.arange(m.nbElem))
    for d in doms:
        assert np.all(np.diff(d.globalElem) > 0) and np.all(np.diff(d.globalNode) > 0)
        # local connectivity maps back to the global one
        assert np.array_equal(d.globalNode[d.mesh.elemToNode - 1], m.elemToNode[d.globalElem] - 1)
        for i, q in enumerate(d.neighbors):
            o = doms[int(q)]
            k = int(np.nonzero(o.neighbors == d.rank)[0][0])
            mine = d.globalNode[d.intfNodes[d.intfIndex[i]:d.intfIndex[i + 1]] - 1]
            theirs = o.globalNode[o.intfNodes[o.intfIndex[k]:o.intfIndex[k + 1]] - 1]
            assert np.array_equal(mine, theirs) and mine.size > 0


def test_per_rank_input_files_round_trip(tmp_path):
    m = _mesh("lap")
    for d in split_domains(m, 3):
        path = write_reference_tree(d.mesh, str(tmp_path), "LM6", "lap", domain=d)
        assert path.endswith(f"lap_3_{d.rank}")
        r = read_reference_input(path)
        assert np.array_equal(r.elemToNode, d.mesh.elemToNode)
        assert np.array_equal(r.meta["intfIndex"], d.intfIndex)
        assert np.array_equal(r.meta["intfNodes"], d.intfNodes)
        assert np.array_equal(r.meta["neighborsList"], d.neighborsList)
        assert r.nbEdges == d.mesh.nbEdges == O.pattern(d.mesh.elemToNode, d.mesh.nbNodes)[0][-1]


@pytest.mark.parametrize("op", ["lap", "ela"])
@pytest.mark.parametrize("nb", [2, 4])
def test_oracle_halo_sum_against_undivided_mesh(op, nb):
    m = _mesh(op)
    doms = split_domains(m, nb)
    full = O.full(m, op=op)
    whole = O.prec_blocks(full["values"], full["row"], full["col"], m.nbNodes, op)
    summed = oracle_flow(doms, op, invert=False)
    d = O.op_dim(op)
    multi = 0
    for dom, p in zip(doms, summed):
        ref = whole.reshape(-1, d)[dom.globalNode]
        got = p.reshape(-1, d)
        intf = np.zeros(dom.mesh.nbNodes, bool)
        intf[dom.intfNodes - 1] = True
        multi += int((np.bincount(dom.intfNodes - 1, minlength=dom.mesh.nbNodes) > 1).sum())
        # interior nodes: the same contributions in the same order -> the same bits
        assert got[~intf].tobytes() == ref[~intf].tobytes()
        # interface nodes: partial sums added; equal up to rounding
        scale = np.abs(ref[intf]).max(axis=1, keepdims=True)
        assert np.all(np.abs(got[intf] - ref[intf]) <= 1e-14 * scale)
    if nb == 4:
        assert multi > 0, "no node on more than one interface: the split does not exercise the order"


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, op, nb_mesh, out_dir):
    import torch.distributed as dist
    from minifem.halo import HaloExchange, TorchTransport
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    try:
        m = cube_mesh(nb_mesh, seed=3, op=op)
        dom = split_domains(m, world)[rank]
        row, col, vals, p, markf = rank_blocks(dom, op)
        blocks = OracleBlocks(p, dom.intfIndex, dom.intfNodes, op)
        HaloExchange(blocks, dom.neighbors, O.op_dim(op), TorchTransport())()
        O.prec_invert(p, row, col, markf, dom.mesh.nbNodes, op)
        np.save(os.path.join(out_dir, f"prec_{rank}.npy"), p)
        dist.barrier()
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("op,world", [("ela", 2), ("lap", 2), ("ela", 4)])
def test_exchange_code_path_over_gloo(tmp_path, op, world):
    import torch.multiprocessing as mp
    n = 7
    mp.spawn(_rank_main, args=(world, _free_port(), op, n, str(tmp_path)), nprocs=world, join=True)
    expect = oracle_flow(split_domains(cube_mesh(n, seed=3, op=op), world), op)
    for r in range(world):
        got = np.load(os.path.join(tmp_path, f"prec_{r}.npy"))
        assert got.tobytes() == expect[r].tobytes(), f"rank {r}"
