"""1-D base-state helpers used when building stage inputs.

``cell_to_edge`` follows Maestro::CelltoEdge (Source/MaestroCelltoEdge.cpp:5-55) for one
radial level: fourth-order interpolation clamped to the neighbouring cell values, second
order next to the ends, one-sided at the ends.
"""
import numpy as np


def cell_to_edge(c):
    c = np.asarray(c, dtype=np.float64)
    nr = c.shape[0]
    e = np.zeros(nr + 1)
    for r in range(nr + 1):
        if r == 0:
            e[r] = c[r]
        elif r == 1:
            e[r] = 0.5 * (c[r - 1] + c[r])
        elif r == nr:
            e[r] = c[r - 1]
        elif r == nr - 1:
            e[r] = 0.5 * (c[r] + c[r - 1])
        else:
            tmp = 7.0 / 12.0 * (c[r] + c[r - 1]) - 1.0 / 12.0 * (c[r + 1] + c[r - 2])
            lo = c[r - 1] if c[r - 1] < c[r] else c[r]
            hi = c[r - 1] if c[r] < c[r - 1] else c[r]
            t = lo if tmp < lo else tmp
            e[r] = hi if hi < t else t
    return e
