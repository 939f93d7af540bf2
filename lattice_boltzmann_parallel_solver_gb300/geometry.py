"""Boundary compiler: the reference's boundary closures, applied in order,
turned into one per-node descriptor the CUDA kernels read.

For every node and direction the post-streaming population has exactly one
source, set by the LAST closure that writes it (the reference applies its
closures one after another, boundary_utils.py:51-52, 103-106, 165-201, and
every closure reads f_pre, f_prev or a constant, never another closure's
output):

  PULL    periodic streaming                      (lattice_boltzmann_method.py:156-157)
  BOUNCE  f_pre(x, opp i) - k                     (boundary_conditions.py:108-109, 156, 162, 207-210)
  CONST   a fixed population                      (boundary_conditions.py:250-251)
  OUTLET  f_prev(x - 1, i)                        (boundary_conditions.py:279-280)

The descriptor is a uint32 per node ([ny][nx], x fastest) plus a bit mask
[ny][ceil(nx/32)] marking the nodes that have one; the constants k and the
fixed populations go into two small tables passed by value to the kernels.
"""
from __future__ import annotations

import copy
import ctypes

import numpy as np
import torch

from . import _lib

PULL, BOUNCE, CONST, OUTLET = _lib.SRC_PULL, _lib.SRC_BOUNCE, _lib.SRC_CONST, _lib.SRC_OUTLET


def dir_mask(dirs) -> int:
    m = 0
    for i in dirs:
        m |= 1 << int(i)
    return m


class CompiledGeometry:
    """Device-resident descriptor of one boundary composition on an nx x ny lattice.

    The compile works on the nodes that some source writes (gathered from the
    masks), not on dense per-direction arrays of the whole lattice, so its
    host cost grows with the boundary, not with nx * ny (a 2048 x 512
    Poiseuille lattice: a 4 MB descriptor array and two rows of sources)."""

    def __init__(self, nx: int, ny: int, sources=(), pressure=None, device="cuda"):
        self.nx, self.ny = int(nx), int(ny)
        # linear indices y * nx + x of the nodes each source writes
        lins = []
        for mask, i, kind, value in sources:
            mask = np.asarray(mask, dtype=bool)
            assert mask.shape == (nx, ny), "boundary mask shape %s does not match the lattice %s" % (
                mask.shape, (nx, ny))
            lins.append(np.flatnonzero(mask.T))
        nodes = np.unique(np.concatenate(lins)) if lins else np.zeros(0, dtype=np.int64)
        src = np.zeros((nodes.size, 9), dtype=np.uint32)
        kv = np.zeros((nodes.size, 9))
        cv = np.zeros((nodes.size, 9))
        for (mask, i, kind, value), lin in zip(sources, lins):
            pos = np.searchsorted(nodes, lin)
            src[pos, i] = kind
            kv[pos, i] = value if kind == BOUNCE else 0.0
            cv[pos, i] = value if kind == CONST else 0.0
        keep = (src != PULL).any(axis=-1)
        nodes, src, kv, cv = nodes[keep], src[keep], kv[keep], cv[keep]
        self.n_special = int(nodes.size)
        outlet_cols = np.unique(nodes[(src == OUTLET).any(axis=-1)] % nx)
        self.outlet = bool(outlet_cols.size)
        # the fused kernels keep the outlet's previous populations for column nx-1 only
        self.fusable = bool(np.all(outlet_cols == nx - 1))

        g = _lib.Geometry()
        g.nx, g.ny = self.nx, self.ny
        g.outlet = int(self.outlet)
        if self.n_special:
            ktab, kidx = np.unique(kv, axis=0, return_inverse=True)
            ctab, cidx = np.unique(cv, axis=0, return_inverse=True)
            if len(ktab) > _lib.MAX_SETS or len(ctab) > _lib.MAX_SETS:
                raise NotImplementedError("more than %d distinct boundary constant sets" % _lib.MAX_SETS)
            packed = np.zeros(nodes.size, dtype=np.uint32)
            for i in range(9):
                packed |= src[:, i] << np.uint32(2 * i)
            packed |= (kidx.reshape(-1).astype(np.uint32) << np.uint32(_lib.KSET_SHIFT)) | \
                (cidx.reshape(-1).astype(np.uint32) << np.uint32(_lib.CSET_SHIFT))
            desc = np.zeros(ny * nx, dtype=np.uint32)
            desc[nodes] = packed
            words = (nx + 31) // 32
            x, y = nodes % nx, nodes // nx
            bcmask = np.zeros(ny * words, dtype=np.uint32)
            np.bitwise_or.at(bcmask, y * words + (x >> 5), (np.uint32(1) << (x & 31).astype(np.uint32)))
            self.desc = torch.from_numpy(desc.reshape(ny, nx)).to(device)
            self.bcmask = torch.from_numpy(bcmask.reshape(ny, words)).to(device)
            g.desc = self.desc.data_ptr()
            g.bcmask = self.bcmask.data_ptr()
            # plain inlet / outlet columns: the batched boundary-free step applies
            # them itself, its boundary-node pass skips them
            edge = np.zeros(nodes.size, dtype=bool)
            g.edge_inlet_desc, g.edge_outlet_desc = self._edge_desc(nx, ny, nodes, src, packed, edge)
            # linear indices y*nx + x of the boundary nodes, for the boundary-node
            # pass: the other boundary nodes first, then the plain edge nodes
            order = np.concatenate([nodes[~edge], nodes[edge]]).astype(np.int32)
            self.bcnodes = torch.from_numpy(order).to(device)
            g.bcnodes = self.bcnodes.data_ptr()
            g.n_bcnodes = int(order.size)
            g.n_bcnodes_edge = int(edge.sum())
            g.n_kset, g.n_cset = len(ktab), len(ctab)
            for s_ in range(len(ktab)):
                for i in range(9):
                    g.kconst[s_][i] = float(ktab[s_, i])
            for s_ in range(len(ctab)):
                for i in range(9):
                    g.cconst[s_][i] = float(ctab[s_, i])
        else:
            self.desc = self.bcmask = self.bcnodes = None
        if pressure is not None:
            pin, pout, rho_in, rho_out = pressure
            g.pressure = 1
            g.pressure_in_dirs = dir_mask(pin)
            g.pressure_out_dirs = dir_mask(pout)
            g.rho_in, g.rho_out = float(rho_in), float(rho_out)
            assert nx >= 2
        self.pressure = pressure
        self.struct = g

    @staticmethod
    def _edge_desc(nx, ny, nodes, src, packed, edge):
        """(inlet, outlet) descriptors of the plain edge nodes, 0 for none; marks
        those nodes in ``edge`` (over the boundary nodes ``nodes``).  Plain inlet:
        all nine sources CONST (the most common such descriptor of column 0);
        plain outlet: directions 3, 6, 7 OUTLET and the others PULL (column
        nx-1).  A column qualifies only when every node of it has a descriptor,
        so that a kernel may apply the form to the whole column and leave the
        other nodes to the pass."""
        out = []
        x = nodes % nx
        for col, want in ((0, np.full(9, CONST)),
                          (nx - 1, np.array([OUTLET if i in (3, 6, 7) else PULL for i in range(9)]))):
            on = x == col
            if nx < 2 or int(on.sum()) != ny:
                out.append(0)
                continue
            plain = on & (src == want.astype(np.uint32)).all(axis=-1)
            if not plain.any():
                out.append(0)
                continue
            vals, counts = np.unique(packed[plain], return_counts=True)
            d = int(vals[np.argmax(counts)])
            edge |= plain & (packed == d)
            out.append(d)
        return out[0], out[1]

    @property
    def ref(self):
        return ctypes.byref(self.struct)

    def with_dev_ref(self, ux: float, uy: float) -> "CompiledGeometry":
        """This geometry with the reference velocity of the reference-shifted
        16-bit storages ("f16r", "bf16r") set to (ux, uy): a copy of the
        descriptor struct that shares the device arrays."""
        assert abs(ux) < 0.5 and abs(uy) < 0.5, "the reference velocity must lie inside (-0.5, 0.5)"
        g = copy.copy(self)
        g.struct = _lib.Geometry.from_buffer_copy(self.struct)
        g.struct.dev_ref_ux, g.struct.dev_ref_uy = float(ux), float(uy)
        return g


_EMPTY = {}


def empty_geometry(nx: int, ny: int) -> CompiledGeometry:
    """Fully periodic lattice: every node streams."""
    key = (int(nx), int(ny))
    if key not in _EMPTY:
        _EMPTY[key] = CompiledGeometry(nx, ny)
    return _EMPTY[key]
