"""Test-side restatements of the reference's own checking machinery.

* DBEG / DMAKE: the deterministic matrix generator of the netlib level-3
  test driver (blastest/src/dblat3.c:3965-4108, 4458-4505).
* DMMCH: its test ratio, |ct - cc| / eps / gauge (dblat3.c:4109-4290),
  threshold 16.0 from blastest/input/dblat3.in.
* The BLIS testsuite residual of testsuite/src/test_gemm.c:303-414 (and the
  trsm/gemv variants), with operands normalised by a power of two at least
  their 1-norm (testsuite/src/test_libblis.c:2525-2580).
"""
import numpy as np


class DBeg:
    """Uniform (-0.5, 0.5) pseudo-random numbers of the netlib test drivers."""

    def __init__(self):
        self.reset()

    def reset(self):
        self.mi, self.i, self.ic = 891, 7, 0

    def __call__(self):
        self.ic += 1
        while True:
            self.i = self.i * self.mi
            self.i -= (self.i // 1000) * 1000
            if self.ic >= 5:
                self.ic = 0
                continue
            break
        return (self.i - 500) / 1001.0


def dmake_ge(gen, m, n, transl=0.0):
    """DMAKE('GE'): column by column; column n/2 zeroed off the diagonal when n > 3."""
    a = np.zeros((m, n), order="F")
    jz = n // 2 - 1  # Fortran column n/2 (1-based)
    for j in range(n):
        for i in range(m):
            v = gen() + transl
            if i != j and n > 3 and j == jz:
                v = 0.0
            a[i, j] = v
    return a


def dmake_tr(gen, n, lower, unit):
    """DMAKE('TR'): triangle from DBEG, opposite triangle zero, diagonal + 1."""
    a = np.zeros((n, n), order="F")
    for j in range(n):
        for i in range(n):
            if (lower and i >= j) or ((not lower) and i <= j):
                v = gen()
                if i != j and n > 3 and j == n // 2 - 1:
                    v = 0.0
                a[i, j] = v
        a[j, j] += 1.0
        if unit:
            a[j, j] = 1.0
    return a


EPS = np.finfo(np.float64).eps


def dmmch_ratio(alpha, a_op, b_op, beta, c0, cc):
    """Largest DMMCH test ratio over all entries (a_op, b_op already op()'d)."""
    ct = alpha * (a_op @ b_op) + beta * c0
    g = abs(alpha) * (np.abs(a_op) @ np.abs(b_op)) + abs(beta) * np.abs(c0)
    err = np.abs(ct - cc) / EPS
    nz = g != 0
    err[nz] = err[nz] / g[nz]
    return float(err.max()) if err.size else 0.0


def ceil_pow2(x):
    return 2.0 ** np.ceil(np.log2(x)) if x > 0 else 1.0


def normalize(a):
    """Divide by the smallest power of two >= the 1-norm (testsuite convention)."""
    nrm = np.abs(a).sum(axis=0).max() if a.size else 0.0
    return a / ceil_pow2(nrm)


def gemm_residual(alpha, a_op, b_op, beta, c0, c, seed=7):
    """||C t - (beta C0 t + alpha A (B t))||_2 for a random t."""
    rng = np.random.default_rng(seed)
    t = rng.uniform(-1.0, 1.0, size=c.shape[1])
    v = c @ t
    w = b_op @ t
    z = alpha * (a_op @ w) + beta * (c0 @ t)
    return float(np.linalg.norm(v - z))


def trsm_residual(side, alpha, a_op, b0, x, seed=7):
    """Residual of op(A) X = alpha B0 (left) or X op(A) = alpha B0 (right)."""
    rng = np.random.default_rng(seed)
    t = rng.uniform(-1.0, 1.0, size=x.shape[1])
    if side == 0:
        v = a_op @ (x @ t)
        z = alpha * (b0 @ t)
    else:
        v = x @ (a_op @ t)
        z = alpha * (b0 @ t)
    return float(np.linalg.norm(v - z))


def op(x, trans):
    return x.T if trans & 0x08 else x
