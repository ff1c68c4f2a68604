"""Halo exchange of the preconditioner blocks between sub-domains: the device
form of MPI_halo_exchange (src/halo.cc:39-122), called between prec_init and
prec_inversion (src/FEM.cc:211-222).

Each rank assembles its own sub-domain (minifem.meshgen.split_domains or the
reference's <op>_<nbBlocks>_<rank> input files) on its own GPU.  One exchange:

1. pack   -- the blocks of every interface entry into a send buffer
             (mfem_halo_pack on the device; src/halo.cc:66-77);
2. move   -- interface i's slice to neighbour i, the neighbour's slice into
             the same place of the receive buffer (a Transport: torch.distributed
             point-to-point -- NCCL between GPUs, gloo on CPU -- or a loopback
             for several sub-domains in one process);
3. add    -- the received blocks onto the local ones, in interface order
             (mfem_halo_add; src/halo.cc:96-112), so that every rank ends with
             the same bits the reference computes.

The sum is the one data exchange of the reference's domain decomposition;
values (the CSR matrix) are never exchanged.
"""
from __future__ import annotations

import numpy as np


class DeviceBlocks:
    """The preconditioner blocks of an Assembler's latest mfem_prec_init, packed
    and summed on its GPU.  Buffers are torch CUDA tensors of float64."""

    def __init__(self, asm, intfIndex, intfNodes):
        import ctypes as C
        import torch
        from . import _native as N
        self._N, self._C, self.torch = N, C, torch
        self.asm = asm
        self.intfIndex = np.ascontiguousarray(intfIndex, np.int32)
        self.intfNodes = np.ascontiguousarray(intfNodes, np.int32)
        self.nbIntf = int(self.intfIndex.size - 1)
        asm._check(N.lib.mfem_set_interfaces(asm._h, self.nbIntf,
                                             self.intfIndex.ctypes.data_as(C.c_void_p),
                                             self.intfNodes.ctypes.data_as(C.c_void_p)))
        self.device = torch.device("cuda", asm.device)

    def pack(self, dim: int):
        n = int(self.intfIndex[-1]) * dim if self.nbIntf else 0
        send = self.torch.empty(max(n, 1), dtype=self.torch.float64, device=self.device)[:n]
        self.asm._check(self._N.lib.mfem_halo_pack(self.asm._h, self._C.c_void_p(send.data_ptr())))
        self.asm.synchronize()        # the transport reads it on another stream
        return send

    def empty_like(self, buf):
        return self.torch.empty_like(buf)

    def add(self, recv):
        self.torch.cuda.synchronize(self.device)   # the transport wrote it on another stream
        self.asm._check(self._N.lib.mfem_halo_add(self.asm._h, self._C.c_void_p(recv.data_ptr())))


class TorchTransport:
    """Point-to-point moves with torch.distributed (NCCL for CUDA tensors, gloo
    for CPU tensors).  Rank r sends its slice of interface i to
    neighbour neighbors[i] and receives that neighbour's slice; every pair
    exchanges one message each way per halo sum."""

    def __init__(self, group=None):
        import torch.distributed as dist
        self.dist, self.group = dist, group

    def move(self, send, recv, intfIndex, neighbors, dim):
        reqs = []
        for i, q in enumerate(neighbors):
            a, b = int(intfIndex[i]) * dim, int(intfIndex[i + 1]) * dim
            if b > a:
                reqs.append(self.dist.irecv(recv[a:b], src=int(q), group=self.group))
        for i, q in enumerate(neighbors):
            a, b = int(intfIndex[i]) * dim, int(intfIndex[i + 1]) * dim
            if b > a:
                reqs.append(self.dist.isend(send[a:b].contiguous(), dst=int(q), group=self.group))
        for r in reqs:
            r.wait()


class HaloExchange:
    """One rank's halo sum: blocks (DeviceBlocks, or any object with pack / add /
    empty_like) and a transport."""

    def __init__(self, blocks, neighbors, dim: int, transport=None):
        self.blocks = blocks
        self.neighbors = np.asarray(neighbors, np.int64)
        self.dim = dim
        self.transport = transport

    def __call__(self):
        if len(self.neighbors) == 0:       # one domain: a no-op (src/halo.cc:44)
            return
        send = self.blocks.pack(self.dim)
        recv = self.blocks.empty_like(send)
        self.transport.move(send, recv, self.blocks.intfIndex, self.neighbors, self.dim)
        self.blocks.add(recv)


def loopback_exchange(exchanges, ranks):
    """The halo sums of several sub-domains held by one process (ranks[k] is the
    rank of exchanges[k]): every rank packs, then each receives its neighbours'
    slices, then each adds -- the message pattern of the reference without a
    network."""
    by_rank = {r: x for r, x in zip(ranks, exchanges)}
    sends = {r: x.blocks.pack(x.dim) for r, x in by_rank.items()}
    for r, x in by_rank.items():
        recv = x.blocks.empty_like(sends[r])
        idx = x.blocks.intfIndex
        for i, q in enumerate(x.neighbors):
            y = by_rank[int(q)]
            # the neighbour's interface towards r
            k = int(np.nonzero(y.neighbors == r)[0][0])
            a, b = int(idx[i]) * x.dim, int(idx[i + 1]) * x.dim
            c, d = int(y.blocks.intfIndex[k]) * y.dim, int(y.blocks.intfIndex[k + 1]) * y.dim
            if b - a != d - c:
                raise ValueError(f"interface {r}<->{q} lists differ in length")
            recv[a:b] = sends[int(q)][c:d]
        x.blocks.add(recv)
