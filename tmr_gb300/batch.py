"""Many independent forests as one.

A batch of forests becomes one ``OctForest`` over the disjoint union of
their blocks (node numbers offset per forest).  Trees of different forests
share no node, edge or face, so refine, balance, createNodes,
createInterpolation and the applies treat them independently, and every
kernel of the pipeline runs once for the whole batch instead of once per
forest.  Each forest's octants are the octants of its blocks (contiguous:
the block number leads the octant order), its nodes are contiguous in the
numbering (nodes are numbered in owner-block order), and its P is a
diagonal block of the batch's P.
"""
import numpy as np

from . import TMR
from ._lib import call


class ForestBatch:
    """Forests given by their block connectivities, held as one forest."""

    def __init__(self, conns, order=2, interp=TMR.GAUSS_LOBATTO_POINTS, stream=None):
        import torch
        blocks, first, off = [], [0], 0
        for c in conns:
            c = np.asarray(c, dtype=np.intc)
            blocks.append(c + off)
            off += int(c.max()) + 1
            first.append(first[-1] + c.shape[0])
        self.num_forests = len(conns)
        self.first_block = np.array(first, dtype=np.intc)
        self.forest = TMR.OctForest(order=order, interp=interp, stream=stream)
        self.forest.setConnectivity(np.vstack(blocks))
        bf = np.repeat(np.arange(self.num_forests, dtype=np.intc), np.diff(self.first_block))
        self._d_first = torch.tensor(self.first_block, device="cuda")
        self._d_block_forest = torch.tensor(bf, device="cuda")
        self._d_start = torch.zeros(self.num_forests + 1, dtype=torch.int64, device="cuda")

    def octant_starts(self, forest=None):
        """First octant of every forest (num_forests + 1 entries) in
        `forest` (default: the batch forest)."""
        f = self.forest if forest is None else forest
        o = f.getOctantsDevice()
        import torch
        return torch.searchsorted(o["block"], self._d_first).cpu().numpy()

    def random_refinement(self, seed, pass_, probs, active):
        """Per-forest seeded refinement array: forest k's octant j draws
        U(seed, k * 1024 + pass_, j) < probs[k] where active[k], else 0;
        the same flags TMR.random_refinement(n_k, seed, k*1024 + pass_,
        probs[k]) gives forest k alone."""
        import ctypes

        import torch
        _vp = ctypes.c_void_p
        n = self.forest.getNumOctants()
        out = torch.empty(max(n, 1), dtype=torch.int32, device="cuda")
        p = torch.as_tensor(np.asarray(probs, np.float64), device="cuda")
        a = torch.as_tensor(np.asarray(active, np.intc), device="cuda")
        call("tmrg_batch_refinement_device", self.forest.ptr, self.num_forests,
             _vp(self._d_first.data_ptr()), _vp(self._d_block_forest.data_ptr()),
             _vp(p.data_ptr()), _vp(a.data_ptr()), int(seed), int(pass_),
             _vp(self._d_start.data_ptr()), _vp(out.data_ptr()))
        return out[:n]

    def split_octants(self, octs, starts):
        """Per-forest (n_k, 7) octant arrays (block ids rebased, tags
        renumbered) from the batch's (n, 7) octants and octant starts."""
        out = []
        for k in range(self.num_forests):
            a = octs[starts[k]:starts[k + 1]].copy()
            a[:, 0] -= self.first_block[k]
            a[:, 4] = np.arange(len(a))
            out.append(a)
        return out
