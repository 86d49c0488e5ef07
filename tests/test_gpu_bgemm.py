"""BF16 GEMM (A, B bf16; C and arithmetic fp32): the tcgen05 kernel (config
0, operands by TMA from the caller's K-contiguous rows or from a packed
copy) and the 64 x 64 engine with bf16 loads (configs 1..5), against an FP64
product of the same bf16 values."""
import numpy as np
import pytest

from blis_gb300 import dev

pytestmark = pytest.mark.gpu

N, T = 0, 8


def _bf16(shape, seed, pow2=False):
    import torch
    g = torch.Generator(device="cpu").manual_seed(seed)
    if pow2:
        # {0, +-2^s}, s in -6..0: every product and partial sum is exact in fp32 for k < 2^12
        e = torch.randint(-6, 1, shape, generator=g).double()
        sgn = torch.randint(0, 3, shape, generator=g).double() - 1.0
        x = sgn * torch.pow(2.0, e)
    else:
        x = torch.rand(shape, generator=g, dtype=torch.float64) * 2 - 1
    return x.to(torch.bfloat16)


def _colmajor(t):
    # a column-major device copy (storage of t.T, row-major)
    return t.t().contiguous().cuda().t()


def _run(config, ta, tb, m, n, k, alpha, beta, pow2=False, lda_pad=0):
    import torch
    a = _bf16((k, m) if ta else (m, k), 1, pow2)
    b = _bf16((n, k) if tb else (k, n), 2, pow2)
    c0 = torch.rand((m, n), generator=torch.Generator().manual_seed(3), dtype=torch.float64).float()
    if lda_pad:
        big = torch.zeros((a.shape[0] + lda_pad, a.shape[1]), dtype=torch.bfloat16)
        big[: a.shape[0]] = a
        ad = _colmajor(big)[: a.shape[0]]
    else:
        ad = _colmajor(a)
    bd = _colmajor(b)
    cd = _colmajor(c0)
    dev.bgemm(T if ta else N, T if tb else N, alpha, ad, bd, beta, cd, config=config)
    torch.cuda.synchronize()
    A = (a.t() if ta else a).double()
    B = (b.t() if tb else b).double()
    ref = alpha * (A @ B) + beta * c0.double()
    bound = abs(alpha) * (A.abs() @ B.abs()) * (k + 2) * 2.0 ** -24 + abs(beta) * c0.double().abs() * 2.0 ** -23
    return cd.cpu().double(), ref, bound


@pytest.mark.parametrize("config", [0, 1, 3, 5])
@pytest.mark.parametrize("ta", [0, 1])
@pytest.mark.parametrize("tb", [0, 1])
@pytest.mark.parametrize("m,n,k", [(300, 260, 200), (129, 65, 77), (256, 256, 128)])
def test_bgemm_against_fp64(config, ta, tb, m, n, k):
    got, ref, bound = _run(config, ta, tb, m, n, k, 1.5, 0.5)
    assert ((got - ref).abs() <= bound + 1e-30).all()


@pytest.mark.parametrize("config", [0, 2])
@pytest.mark.parametrize("ta,tb", [(0, 0), (1, 0), (0, 1), (1, 1)])
def test_bgemm_exact_on_powers_of_two(config, ta, tb):
    # both tensor-core operand routes (TMA from the caller's rows: A transposed, B not; packed copy
    # otherwise) and the FMA engine give the exact product
    got, ref, _ = _run(config, ta, tb, 200, 300, 500, 1.0, 0.0, pow2=True)
    assert (got == ref).all()


def test_bgemm_padded_leading_dimension_and_beta():
    # lda = k + 8 keeps the TMA route (16-byte rows); lda = k + 3 forces the packed copy
    for pad in (8, 3):
        got, ref, bound = _run(0, 1, 0, 150, 170, 96, -2.0, 1.25, lda_pad=pad)
        assert ((got - ref).abs() <= bound + 1e-30).all()


def test_bgemm_library_choice_and_edges():
    import torch
    got, ref, bound = _run(None, 0, 0, 700, 600, 400, 1.0, 0.0)
    assert ((got - ref).abs() <= bound + 1e-30).all()
    # k = 0: C := beta C
    c = _colmajor(torch.ones((5, 7)))
    z = torch.zeros((5, 1), dtype=torch.bfloat16).cuda()
    dev.bgemm(N, N, 1.0, z[:, :0], torch.zeros((0, 7), dtype=torch.bfloat16).cuda(), 3.0, c)
    torch.cuda.synchronize()
    assert torch.equal(c.cpu(), torch.full((5, 7), 3.0))
