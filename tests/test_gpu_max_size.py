"""The largest sizes the plans accept (the reference puts no upper bound on
unordered::Plan or fft128::Plan; here unordered n <= 2^28, fft128 n <= 2^24,
u64 products N <= 2^29, u128 products N <= 2^25), checked through properties
that hold at any size: forward then inverse returns n times the input; the
forward transform of the monomial X^d, in standard order, is exp(-2 pi i k d / n);
the product with the monomial X is the negacyclic shift.  Bit-exact parity
with the oracle at 2^22 points (unordered), 2^20 (fft128) and N = 2^22 / 2^21
(products) is in the other GPU test files."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def gen(torch, seed):
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    return g


def test_unordered_max_size(cuda):
    import concrete_fft as cf
    torch = cuda
    n = 1 << 28
    plan = cf.unordered.Plan(n, cf.unordered.Method.UserProvided(cf.FftAlgo.Dif16, 1024))
    u = torch.rand((n, 2), dtype=torch.float64, device="cuda", generator=gen(torch, 28))
    x = torch.view_as_complex(u * 2 - 1)
    del u
    d = x.clone()
    plan.fwd(d)
    plan.inv(d)
    assert float((d / n - x).abs().max()) < 1e-11
    del d, x
    deg = 123456789
    buf = torch.empty(n, dtype=torch.complex128, device="cuda")
    plan.fwd_monomial(deg, buf)
    std = torch.empty_like(buf)
    plan.to_standard(buf, std)
    k = np.random.default_rng(5).integers(0, n, 4096)
    got = std[torch.from_numpy(k).cuda()].cpu().numpy()
    want = np.exp(-2j * np.pi * (((k * deg) % n).astype(np.float64) / n))
    assert np.abs(got - want).max() < 1e-13
    back = torch.empty_like(buf)
    plan.from_standard(std, back)
    assert torch.equal(back, buf)
    del buf, std, back, plan
    torch.cuda.empty_cache()


def test_fft128_max_size(cuda):
    import concrete_fft as cf
    torch = cuda
    n = 1 << 24
    plan = cf.fft128.Plan(n)
    g = gen(torch, 24)
    hi = [torch.rand(n, dtype=torch.float64, device="cuda", generator=g) * 2 - 1 for _ in range(2)]
    x = [hi[0], hi[0] * 2.0 ** -60, hi[1], hi[1] * 2.0 ** -60]
    d = [t.clone() for t in x]
    plan.fwd(*d)
    plan.inv(*d)
    for k in (0, 2):  # the double-double error of n * x, scaled back by n
        err = ((d[k] - n * x[k]) + (d[k + 1] - n * x[k + 1])).abs().max() / n
        assert float(err) < 1e-26, k
    del d, x, hi, plan
    torch.cuda.empty_cache()


def test_u64_product_max_size(cuda):
    import concrete_fft as cf
    torch = cuda
    N = 1 << 29
    plan = cf.product.U64ProductPlan(N, cf.FftAlgo.Dif4, 1024)
    b = torch.zeros((1, N), dtype=torch.int64, device="cuda")
    b[0, 1] = 1
    bhat = torch.empty((1, N // 2), dtype=torch.complex128, device="cuda")
    plan.prepare_operand(b, bhat)
    del b
    a = torch.randint(-2 ** 8, 2 ** 8, (1, N), dtype=torch.int64, device="cuda", generator=gen(torch, 29))
    out = torch.empty_like(a)
    plan.product(a, bhat, out)
    assert torch.equal(out[:, 1:], a[:, :-1])
    assert torch.equal(out[:, :1], -a[:, -1:])
    del a, out, bhat, plan
    torch.cuda.empty_cache()


def test_u128_product_max_size(cuda):
    import concrete_fft as cf
    torch = cuda
    N = 1 << 25
    plan = cf.product.U128ProductPlan(N)
    b = torch.zeros((1, N), dtype=torch.int64, device="cuda")
    b[0, 1] = 1
    bhat = torch.empty((1, 4, N // 2), dtype=torch.float64, device="cuda")
    plan.prepare_operand(b, bhat)
    lo = torch.randint(-2 ** 40, 2 ** 40, (1, N), dtype=torch.int64, device="cuda", generator=gen(torch, 25))
    a = torch.stack([lo, (lo < 0).to(torch.int64).neg()], dim=-1)  # i128: sign-extended high word
    out = torch.empty_like(a)
    plan.product(a, bhat, out)
    shifted = torch.cat([-lo[:, -1:], lo[:, :-1]], dim=1)
    want = torch.stack([shifted, (shifted < 0).to(torch.int64).neg()], dim=-1)
    assert torch.equal(out, want)
    del a, out, bhat, plan
    torch.cuda.empty_cache()
