"""Ghost-cell oracle (TEST INFRASTRUCTURE ONLY).

With one process every neighbour of gcell/gcells_sendrecv.c is the process
itself, so pfft_exchange is a periodic wrap of the compact block into the box
of extent gc_below + n + gc_above (doc/reference.tex:568-586), and pfft_reduce
is its adjoint: the sum over all periodic images, truncated back to the block
(gcell/gcells_plan.c:401-486).  `tuple` counts reals per cell.
"""
import numpy as np


def box_index(n, gcb, gca):
    idx = []
    for t in range(len(n)):
        k = np.arange(gcb[t] + n[t] + gca[t]) - gcb[t]
        idx.append(np.mod(k, n[t]))
    return idx


def exchange(block, n, gcb, gca):
    """block: array of shape n + (tuple,) -> box of shape ngc + (tuple,)."""
    ix = box_index(n, gcb, gca)
    return block[np.ix_(*ix)]


def reduce(box, n, gcb, gca):
    ix = box_index(n, gcb, gca)
    out = np.zeros(tuple(n) + box.shape[len(n):], dtype=box.dtype)
    grids = np.meshgrid(*ix, indexing="ij")
    np.add.at(out, tuple(g for g in grids), box)
    return out
