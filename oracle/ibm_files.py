"""ORACLE (test infrastructure): the IBM table files of BCM_Immersed_boundary.

IBM_minus<rank>.dat / IBM_plus<rank>.dat as BCM_Immersed_boundary.cpp
:989-1047 writes them and BCM_Reading_IBM.cpp:19-56 / main.cpp:848-876 read
them: per entry the ghost cell "c\\ti\\tj\\tk\\n", the image point's base cell
"c\\ti\\tj\\tk\\n" and the eight weights "%f\\t...%f\\n" (six decimals), then
"Number of Boundary Cells\\n" and the count.
"""
from __future__ import annotations

import numpy as np


def text(gc, ip, w) -> str:
    out = []
    for g, p, ww in zip(gc, ip, w):
        out.append("%d\t%d\t%d\t%d\n" % tuple(int(x) for x in g))
        out.append("%d\t%d\t%d\t%d\n" % tuple(int(x) for x in p))
        out.append("\t".join("%f" % float(x) for x in ww) + "\n")
    out.append("Number of Boundary Cells\n%d" % len(gc))
    return "".join(out)


def read(path: str):
    """(GCindex[m,4], IPsur[m,4], weight[m,8]) of one file, weights as the
    reference reads them back (six-decimal values)."""
    lines = open(path).read().split("\n")
    m = int(lines[-1])
    gc = np.array([[int(x) for x in lines[3 * e].split("\t")] for e in range(m)], np.int32)
    ip = np.array([[int(x) for x in lines[3 * e + 1].split("\t")] for e in range(m)], np.int32)
    w = np.array([[float(x) for x in lines[3 * e + 2].split("\t")] for e in range(m)])
    return gc.reshape(m, 4), ip.reshape(m, 4), w.reshape(m, 8)
