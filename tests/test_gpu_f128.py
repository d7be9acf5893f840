"""GPU fft128 (double-double negacyclic FFT) vs the oracle: bit-identical."""
import numpy as np
import pytest

from conftest import bits

pytestmark = pytest.mark.gpu
RNG = np.random.default_rng(11)


@pytest.mark.parametrize("n", [32, 64, 128, 256, 512, 1024, 2048, 4096, 8192, 16384, 32768, 1 << 20])
def test_f128_fwd_inv_bit_exact(cuda, oracle, n):
    import concrete_fft as cf
    torch = cuda
    batch = 3 if n <= 8192 else 1
    arrs = [RNG.standard_normal((batch, n)) for _ in range(2)]
    lo = [a * 2.0 ** -60 for a in (RNG.standard_normal((batch, n)), RNG.standard_normal((batch, n)))]
    host = [arrs[0], lo[0], arrs[1], lo[1]]
    plan = cf.fft128.Plan(n)
    assert plan.fft_size() == n
    dev = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in host]
    plan.fwd(*dev)
    want = oracle.f128_fwd(*host)
    for d, w in zip(dev, want):
        assert np.array_equal(bits(d.cpu().numpy()), bits(w)), n
    plan.inv(*dev)
    want = oracle.f128_inv(*want)
    for d, w in zip(dev, want):
        assert np.array_equal(bits(d.cpu().numpy()), bits(w)), n
    want = oracle.f128_fwd(*host)
    hb = [np.array(a, copy=True) for a in host]
    plan.fwd(*hb)  # host entry point
    for h, w in zip(hb, want):
        assert np.array_equal(bits(h), bits(w))


@pytest.mark.parametrize("n,batch", [(32, 1), (512, 3), (4096, 2), (16384, 1)])
def test_f128_host_entry_page_locked(cuda, oracle, n, batch):
    """Host entry points on page-locked arrays: up to 4096 points one kernel works on them
    in place; larger transforms take the staged copies.  Bits equal the oracle's."""
    import concrete_fft as cf
    torch = cuda
    hi = [RNG.standard_normal((batch, n)) for _ in range(2)]
    host = [hi[0], hi[0] * 2.0 ** -60, hi[1], hi[1] * 2.0 ** -60]
    plan = cf.fft128.Plan(n)
    bufs = [torch.from_numpy(np.ascontiguousarray(a)).pin_memory() for a in host]
    plan.fwd(*bufs)
    want = oracle.f128_fwd(*host)
    for b, w in zip(bufs, want):
        assert np.array_equal(bits(b.numpy()), bits(w)), n
    plan.inv(*bufs)
    want = oracle.f128_inv(*want)
    for b, w in zip(bufs, want):
        assert np.array_equal(bits(b.numpy()), bits(w)), n


@pytest.mark.parametrize("n", [1024, 4096, 16384])
def test_f128_block_points_bit_exact(cuda, oracle, n):
    """Every shared-memory block size (the stages above it in global memory) gives the
    oracle's bits, for the plan and for a u128 product plan's transforms."""
    import concrete_fft as cf
    torch = cuda
    hi = [RNG.standard_normal((4, n)) for _ in range(2)]
    host = [hi[0], hi[0] * 2.0 ** -60, hi[1], hi[1] * 2.0 ** -60]
    want_f = oracle.f128_fwd(*host)
    want_i = oracle.f128_inv(*want_f)
    plan = cf.fft128.Plan(n)
    for pts in (256, 512, 1024, 2048, 4096, 0):
        if pts > n:
            continue
        plan.set_block_points(pts)
        assert plan.block_points() == pts
        d = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in host]
        plan.fwd(*d)
        for x, w in zip(d, want_f):
            assert np.array_equal(bits(x.cpu().numpy()), bits(w)), (n, pts)
        plan.inv(*d)
        for x, w in zip(d, want_i):
            assert np.array_equal(bits(x.cpu().numpy()), bits(w)), (n, pts)
    with pytest.raises(cf.CfftError):
        plan.set_block_points(8192)


@pytest.mark.parametrize("n", [2, 4, 16, 64, 1024, 8192, 65536])
def test_f128_raw_negacyclic_functions(cuda, oracle, n):
    """negacyclic_fwd_fft / negacyclic_inv_fft with caller-owned twiddle arrays
    (src/fft128/mod.rs:1041-1104), batched, against the oracle."""
    import concrete_fft as cf
    torch = cuda
    tw = [np.zeros(n) for _ in range(4)]
    cf.fft128.init_negacyclic_twiddles(*tw)
    dtw = [torch.from_numpy(t).cuda() for t in tw]
    rng = np.random.default_rng(n)
    hi = [rng.uniform(-1, 1, (3, n)) for _ in range(2)]
    data = [hi[0], hi[0] * 2.0 ** -60, hi[1], hi[1] * 2.0 ** -60]
    d = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in data]
    cf.fft128.negacyclic_fwd_fft(*d, *dtw)
    want = oracle.f128_fwd(*data)
    for k in range(4):
        assert np.array_equal(d[k].cpu().numpy().view(np.uint64), want[k].view(np.uint64)), (n, k)
    cf.fft128.negacyclic_inv_fft(*d, *dtw)
    want_i = oracle.f128_inv(*want)
    for k in range(4):
        assert np.array_equal(d[k].cpu().numpy().view(np.uint64), want_i[k].view(np.uint64)), (n, k)
    # the reference's slice form: host arrays in place, same bits
    h = [np.ascontiguousarray(x).copy() for x in data]
    cf.fft128.negacyclic_fwd_fft(*h, *tw)
    for k in range(4):
        assert np.array_equal(h[k].view(np.uint64), want[k].view(np.uint64)), (n, k)
    cf.fft128.negacyclic_inv_fft(*h, *tw)
    for k in range(4):
        assert np.array_equal(h[k].view(np.uint64), want_i[k].view(np.uint64)), (n, k)


def test_f128_invalid_size(cuda):
    import concrete_fft as cf
    with pytest.raises(cf.CfftError):
        cf.fft128.Plan(16)
