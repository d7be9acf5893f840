"""Parity at the benchmark configurations' full sizes.

Every product of the headline launch (8192 products of N = 2048, one operand
each) and of the u128 launches (2048 products, N = 1024 and 4096) is compared
with the oracle bit for bit.  The 100,000-item mixed batch is checked in full
through a size-independent property (forward then inverse returns n times the
input, for every item) and bit for bit on a random sample of items.
"""
import numpy as np
import pytest

from conftest import bits

pytestmark = pytest.mark.gpu


def test_headline_launch_every_product_bit_exact(cuda, oracle):
    """N = 2048, 8192 products per launch, A uniform u64, B digits in [-2^7, 2^7)."""
    import concrete_fft as cf
    torch = cuda
    N, count = 2048, 8192
    rng = np.random.default_rng(2)
    a = rng.integers(0, 2 ** 64, (count, N), dtype=np.uint64)
    b = rng.integers(-2 ** 7, 2 ** 7, (count, N))
    plan = cf.product.U64ProductPlan(N, cf.FftAlgo.Dif4, 1024)
    bhat = torch.empty((count, N // 2), dtype=torch.complex128, device="cuda")
    plan.prepare_operand(torch.from_numpy(b).cuda(), bhat)
    want_bhat = oracle.u64_prepare(N, 2, 1024, b)
    assert np.array_equal(bits(bhat.cpu().numpy()), bits(want_bhat))
    da = torch.from_numpy(a.view(np.int64)).cuda()
    out = torch.empty_like(da)
    plan.product(da, bhat, out)
    want = oracle.u64_product(N, 2, 1024, a, want_bhat, nthreads=0)
    assert np.array_equal(out.cpu().numpy().view(np.uint64), want)
    host = np.zeros_like(a)  # the host entry point, pipelined, on the same launch
    plan.product(a, bhat, host)
    assert np.array_equal(host, want)


@pytest.mark.parametrize("N", [1024, 4096])
def test_u128_launch_every_product_bit_exact(cuda, oracle, N):
    """2048 products per launch, A uniform u128, B digits in [-2^15, 2^15)."""
    import concrete_fft as cf
    torch = cuda
    count = 2048
    rng = np.random.default_rng(4)
    a = rng.integers(0, 2 ** 64, (count, N, 2), dtype=np.uint64)
    b = rng.integers(-2 ** 15, 2 ** 15, (count, N))
    plan = cf.product.U128ProductPlan(N)
    bhat = torch.empty((count, 4, N // 2), dtype=torch.float64, device="cuda")
    plan.prepare_operand(torch.from_numpy(b).cuda(), bhat)
    want_bhat = oracle.u128_prepare(N, b)
    assert np.array_equal(bhat.cpu().numpy().view(np.uint64), want_bhat.view(np.uint64))
    da = torch.from_numpy(a.view(np.int64)).cuda()
    out = torch.empty_like(da)
    plan.product(da, bhat, out)
    want = oracle.u128_product(N, a, want_bhat, nthreads=0)
    assert np.array_equal(out.cpu().numpy().view(np.uint64), want)


def test_mixed_batch_full_size(cuda, oracle):
    """100,000 transforms, n = 2^8..2^16, half ordered (n <= 1024) and half unordered,
    forward then inverse in one persistent launch: every item returns n times its input
    (relative error below 1e-12), and a sample of 64 items equals the oracle bit for bit."""
    import concrete_fft as cf
    torch = cuda
    count = 100_000
    rng = np.random.default_rng(3)
    log2n = rng.integers(8, 17, count)
    kind = np.where(log2n > 10, 1, rng.integers(0, 2, count))
    sizes = (1 << log2n).astype(np.int64)
    offs = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.uint64)
    items = np.zeros(count, dtype=cf.batch.ITEM_DTYPE)
    items["offset"], items["log2n"], items["kind"], items["direction"] = offs, log2n, kind, 3
    total = int(sizes.sum())
    b = cf.batch.Batch(items)
    g = torch.Generator(device="cuda")
    g.manual_seed(3)
    x = torch.rand((total, 2), dtype=torch.float64, device="cuda", generator=g) * 2 - 1
    data = x.clone()
    b.run(data)
    torch.cuda.synchronize()
    # every item: out / n == x within 1e-12 of the item's largest input
    scale = torch.repeat_interleave(torch.from_numpy(sizes.astype(np.float64)).cuda(),
                                    torch.from_numpy(sizes).cuda())
    err = (data / scale[:, None] - x).abs().amax(dim=1)
    item_of_point = torch.repeat_interleave(torch.arange(count, device="cuda"), torch.from_numpy(sizes).cuda())
    worst = torch.zeros(count, dtype=torch.float64, device="cuda").scatter_reduce(0, item_of_point, err, "amax")
    assert float(worst.max()) < 1e-12
    del scale, err, item_of_point, worst
    sample = rng.choice(count, 64, replace=False)
    for i in sample:  # only the sampled items are copied to the host
        o, n = int(offs[i]), int(sizes[i])
        xs = x[o:o + n].cpu().numpy()
        xi = xs[:, 0] + 1j * xs[:, 1]
        algo, base, _ = b.schedule(int(kind[i]), int(log2n[i]), 3)
        if kind[i] == 0:
            want = oracle.ordered_inv(int(algo), oracle.ordered_fwd(int(algo), xi))
        else:
            want = oracle.unordered_inv(int(algo), base, oracle.unordered_fwd(int(algo), base, xi))
        gs = data[o:o + n].cpu().numpy()
        gi = gs[:, 0] + 1j * gs[:, 1]
        assert np.array_equal(bits(gi), bits(want)), (i, n, kind[i])
