"""GPU fft128 (double-double negacyclic FFT) vs the oracle: bit-identical."""
import numpy as np
import pytest

from conftest import bits

pytestmark = pytest.mark.gpu
RNG = np.random.default_rng(11)


@pytest.mark.parametrize("n", [32, 64, 256, 512, 2048, 4096, 8192, 32768])
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


def test_f128_invalid_size(cuda):
    import concrete_fft as cf
    with pytest.raises(cf.CfftError):
        cf.fft128.Plan(16)
