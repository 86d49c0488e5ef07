"""Writes tests/golden/blis_ref_outputs.npz: outputs of the reference BLIS itself.

The reference BLIS is compiled from its own sources by oracle/ref_blis.py (run
`python -m oracle.ref_blis` first); this script calls its typed API
(bli_dgemm, bli_dtrsm, bli_dgemv, bli_daxpyv, bli_ddotv) on inputs drawn from the
oracle's seeded generators (oracle/pyoracle.py: uniform on [-1, 1] and the
testsuite's "narrow powers of two") and stores only the outputs; the inputs are
regenerated from the seeds.  tests/test_oracle_blis.py checks the oracle against
them.  Re-run after changing a case below:

    python -m oracle.ref_blis && python tests/golden/make_blis_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import blis_ctypes as bc  # noqa: E402
from oracle import pyoracle as po  # noqa: E402

OUT = os.path.join(HERE, "blis_ref_outputs.npz")

GEMM = [  # (m, n, k, transa, transb, alpha, beta, gen)
    (64, 48, 80, 0, 0, 1.0, 0.0, "pow2"), (64, 48, 80, 0, 0, 1.0, 1.0, "pow2"),
    (64, 48, 80, 8, 8, 1.0, 1.0, "pow2"), (33, 17, 129, 8, 0, 1.0, 0.0, "pow2"),
    (64, 48, 80, 0, 0, 1.0, 0.5, "uniform"), (64, 48, 80, 8, 0, -0.7, 1.3, "uniform"),
    (31, 45, 200, 0, 8, 0.5, 0.0, "uniform"),
]
TRSM = [(s, u, t, d) for s in (0, 1) for u in (0xC0, 0x60) for t in (0, 8) for d in (0, 0x100)]
GEMV = [(0, 40, 56, 1.0, 0.0, "pow2"), (8, 40, 56, 1.0, 1.0, "pow2"), (0, 40, 56, 0.8, -0.5, "uniform"),
        (8, 57, 33, -1.2, 0.25, "uniform")]
VEC_N = 1000


def gen(kind, shape, seed):
    return po.narrow_pow2(shape, seed) if kind == "pow2" else po.uniform(shape, seed)


def trsm_inputs(side, m, n, seed):
    na = m if side == 0 else n
    a = po.uniform((na, na), seed)
    a = np.asfortranarray(a + np.diag(na + np.abs(np.diag(a))))  # well conditioned
    b = po.uniform((m, n), seed + 1)
    return a, b


def main():
    out = {"arch": np.array(bc.arch_name())}
    for i, (m, n, k, ta, tb, al, be, g) in enumerate(GEMM):
        s = 100 + 10 * i
        a = gen(g, (k, m) if ta else (m, k), s)
        b = gen(g, (n, k) if tb else (k, n), s + 1)
        c = gen(g, (m, n), s + 2)
        bc.dgemm(ta, tb, al, a, b, be, c)
        out["gemm%d" % i] = c
    for i, (sd, up, t, dg) in enumerate(TRSM):
        a, b = trsm_inputs(sd, 32, 24, 300 + 10 * i)
        bc.dtrsm(sd, up, t, dg, 0.75, a, b)
        out["trsm%d" % i] = b
    for i, (t, m, n, al, be, g) in enumerate(GEMV):
        s = 500 + 10 * i
        a = gen(g, (m, n), s)
        x = gen(g, ((m if t else n),), s + 1)
        y = gen(g, ((n if t else m),), s + 2)
        bc.dgemv(t, al, a, x, be, y)
        out["gemv%d" % i] = y
    for i, g in enumerate(("pow2", "uniform")):
        x = gen(g, (VEC_N,), 700 + i)
        y = gen(g, (VEC_N,), 710 + i)
        out["dotv%d" % i] = np.array(bc.ddotv(x, y))
        bc.daxpyv(0.625 if g == "pow2" else -0.3, x, y)
        out["axpyv%d" % i] = y
    np.savez_compressed(OUT, **out)
    print(OUT, len(out), "arrays")


if __name__ == "__main__":
    main()
