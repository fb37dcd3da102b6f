"""Refinement indicator restated on the CPU (test infrastructure: only tests
import it, as the checker).

Follows AdaptiveInversion::indicator_calculator (src/Inversion/
AdaptiveInversion.cpp:108-204): for each leaf cell the sum over its face
neighbours of (m_neighbour - m_cell)^2 times a face area, added in the order
of the (neighbour, area) list and rounded after every operation (separate
FP64 multiplies and adds).  Pinned bitwise to the compiled reference by
tests/golden/ref_indicator.npz.
"""
import numpy as np


def indicator(m, rowptr, neighbour, area) -> np.ndarray:
    m = np.asarray(m, dtype=np.float64)
    out = np.zeros(m.size)
    for i in range(m.size):
        acc = 0.0
        for k in range(int(rowptr[i]), int(rowptr[i + 1])):
            d = m[int(neighbour[k])] - m[i]
            acc = acc + (d * d) * float(area[k])
        out[i] = acc
    return out
