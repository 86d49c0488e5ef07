"""The CRT form's CPU model (oracle/gb_oracle.c orc_ozaki_crt_dgemm), without a GPU.

The model is exact integer arithmetic on the scaled operands plus one rounding; these
tests pin its parameters (the integer bits t the moduli afford) and its accuracy against
the double-double evaluator and the digit form's model.
"""
import numpy as np
import pytest

from oracle import pyoracle as po

MODULI = [257, 256, 255, 253, 251, 247, 241, 239, 233, 229, 227, 223, 217, 211, 199, 197]


def test_moduli_pairwise_coprime_and_bits():
    from math import gcd
    for i in range(16):
        for j in range(i):
            assert gcd(MODULI[i], MODULI[j]) == 1
    for n in (2, 8, 12, 16):
        M = 1
        for p in MODULI[:n]:
            M *= p
        for k in (1, 64, 1000, 16384, 100000):
            t = po.ozaki_crt_bits(n, k)
            if t < 1:
                continue
            kb = max(0, (k - 1).bit_length())
            # the product bound the reconstruction needs, and t is the largest that meets it
            assert k * 2 ** (2 * t) <= (8 * M) // 17 and 2 * t + kb <= 126
            assert k * 2 ** (2 * t + 2) > (8 * M) // 17 or 2 * (t + 1) + kb > 126 or t == 62
    assert po.ozaki_crt_bits(16, 16384) == 55


@pytest.mark.parametrize("k", [300, 4096])
def test_crt_model_accuracy(k):
    """At the same operand precision the CRT form is at least as accurate as the digit form
    (it drops no cross terms), and its error obeys the representation bound."""
    m, n = 60, 50
    a = po.expspread((m, k), 5)
    b = po.expspread((k, n), 6)
    ii, jj = np.meshgrid(np.arange(m), np.arange(n), indexing="ij")
    ii, jj = ii.ravel(), jj.ravel()
    hi, lo = po.dd_gemm_entries(0, 0, 1.0, a, b, 0.0, np.zeros((m, n), order="F"), ii, jj)
    c16 = np.zeros((m, n), order="F")
    assert po.ozaki_crt_dgemm(0, 0, 1.0, a, b, 0.0, c16, 16) == 0
    c7 = np.zeros((m, n), order="F")
    po.ozaki_dgemm(0, 0, 1.0, a, b, 0.0, c7, 7)
    e16 = po.componentwise_error(c16[ii, jj], hi, lo)
    e7 = po.componentwise_error(c7[ii, jj], hi, lo)
    assert e16 <= e7
    # |error| <= 2^-(t+1) (2^e_i |B_j|_1 + |A_i|_1 2^e_j) + 2^-(2t+2) k 2^(e_i+e_j) + 1 ulp
    t = po.ozaki_crt_bits(16, k)
    ea = 2.0 ** (np.floor(np.log2(np.abs(a).max(axis=1))) + 2)
    eb = 2.0 ** (np.floor(np.log2(np.abs(b).max(axis=0))) + 2)
    bound = 2.0 ** -(t + 1) * (np.outer(ea, np.abs(b).sum(0)) + np.outer(np.abs(a).sum(1), eb)) \
        + 2.0 ** -(2 * t + 2) * k * np.outer(ea, eb)
    exact = (hi + lo).reshape(m, n)
    assert np.all(np.abs(c16 - exact) <= bound + np.spacing(np.abs(exact)))


def test_crt_model_alpha_beta_and_exact_inputs():
    """Narrow powers of two are exact at 8 moduli; alpha and beta as in the digit form."""
    m, n, k = 40, 30, 64
    a = po.narrow_pow2((m, k), 7)
    b = po.narrow_pow2((k, n), 8)
    c0 = po.uniform((m, n), 9)
    ref = np.asfortranarray(c0.copy())
    po.dgemm(0, 0, 1.0, a, b, 1.0, ref)
    c = np.asfortranarray(c0.copy())
    po.ozaki_crt_dgemm(0, 0, 1.0, a, b, 1.0, c, 8)
    assert np.array_equal(c, ref)
