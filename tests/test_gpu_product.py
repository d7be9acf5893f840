"""Fused negacyclic products on the GPU: bit-identical to the oracle's CPU
pipeline, and torus error against the exact wrapping-integer schoolbook."""
import numpy as np
import pytest

from conftest import bits

pytestmark = pytest.mark.gpu
RNG = np.random.default_rng(3)


def torus_err_bits(got, exact):
    d = (got - exact).view(np.int64).astype(np.float64)
    m = np.abs(d).max()
    return 0.0 if m == 0 else float(np.log2(m))


@pytest.mark.parametrize("N,base_algo,base_n", [(2048, 6, 1024), (2048, 2, 512), (2048, 7, 32), (64, 0, 32),
                                                (1024, 5, 512), (4096, 6, 1024), (8192, 4, 1024)])
def test_u64_product_bit_exact(cuda, oracle, N, base_algo, base_n):
    import concrete_fft as cf
    torch = cuda
    count = 9
    plan = cf.product.U64ProductPlan(N, base_algo, base_n)
    assert plan.algo() == (base_algo, base_n)
    a = RNG.integers(0, 2 ** 64, (count, N), dtype=np.uint64)
    b = RNG.integers(-2 ** 7, 2 ** 7, (count, N))
    db = torch.from_numpy(b).cuda()
    bhat = torch.empty((count, N // 2), dtype=torch.complex128, device="cuda")
    plan.prepare_operand(db, bhat)
    want_bhat = oracle.u64_prepare(N, base_algo, base_n, b)
    assert np.array_equal(bhat.cpu().numpy().view(np.uint64), want_bhat.view(np.uint64))
    da = torch.from_numpy(a.view(np.int64)).cuda()
    out = torch.empty_like(da)
    plan.product(da, bhat, out)
    got = out.cpu().numpy().view(np.uint64)
    want = oracle.u64_product(N, base_algo, base_n, a, want_bhat, nthreads=0)
    assert np.array_equal(got, want)
    exact = oracle.u64_schoolbook(a[:2], b[:2])
    assert torus_err_bits(got[:2], exact) <= torus_err_bits(want[:2], exact)


@pytest.mark.parametrize("algo", [2, 3])
def test_u64_product_int_adds_bit_exact(cuda, oracle, algo):
    """Every integer-pipe addition level gives the same bits as the oracle."""
    import concrete_fft as cf
    torch = cuda
    N, count = 2048, 5
    a = RNG.integers(0, 2 ** 64, (count, N), dtype=np.uint64)
    b = RNG.integers(-2 ** 7, 2 ** 7, (count, N))
    for base in (1024, 512):
        plan = cf.product.U64ProductPlan(N, algo, base)
        bhat = torch.empty((count, N // 2), dtype=torch.complex128, device="cuda")
        plan.prepare_operand(torch.from_numpy(b).cuda(), bhat)
        want = oracle.u64_product(N, algo, base, a, oracle.u64_prepare(N, algo, base, b), nthreads=0)
        for e in (0, 4):
            plan.set_int_adds(e)
            assert plan.int_adds() == e
            out = torch.empty((count, N), dtype=torch.int64, device="cuda")
            plan.product(torch.from_numpy(a.view(np.int64)).cuda(), bhat, out)
            assert np.array_equal(out.cpu().numpy().view(np.uint64), want), (algo, base, e)


def test_u64_product_exact_when_small(cuda, oracle):
    """Bit-exact against the schoolbook wherever the exact sums fit in 53 bits."""
    import concrete_fft as cf
    torch = cuda
    N = 2048
    plan = cf.product.U64ProductPlan(N, 6, 1024)
    a = RNG.integers(-2 ** 30, 2 ** 30, (4, N)).astype(np.int64)
    b = RNG.integers(-2 ** 7, 2 ** 7, (4, N))
    bhat = torch.empty((4, N // 2), dtype=torch.complex128, device="cuda")
    plan.prepare_operand(torch.from_numpy(b).cuda(), bhat)
    out = torch.empty((4, N), dtype=torch.int64, device="cuda")
    plan.product(torch.from_numpy(a).cuda(), bhat, out)
    assert np.array_equal(out.cpu().numpy().view(np.uint64), oracle.u64_schoolbook(a.view(np.uint64), b))


def test_u64_product_shared_operand_and_host(cuda, oracle):
    import concrete_fft as cf
    torch = cuda
    N = 2048
    plan = cf.product.U64ProductPlan(N, 6, 1024)
    a = RNG.integers(0, 2 ** 64, (6, N), dtype=np.uint64)
    b = RNG.integers(-2 ** 7, 2 ** 7, (1, N))
    bhat = torch.empty((1, N // 2), dtype=torch.complex128, device="cuda")
    plan.prepare_operand(torch.from_numpy(b).cuda(), bhat)
    out = np.zeros_like(a)
    plan.product(a, bhat, out, shared_operand=True)  # host entry point
    want = oracle.u64_product(N, 6, 1024, a, oracle.u64_prepare(N, 6, 1024, b))
    assert np.array_equal(out, want)


def test_u64_product_host_pipeline_chunks(cuda, oracle):
    """Host entry point over many chunks: more chunks than copy/compute streams, a
    ragged last chunk, one distinct operand per product."""
    import concrete_fft as cf
    torch = cuda
    N, count = 2048, 2000
    plan = cf.product.U64ProductPlan(N, 2, 1024)
    a = RNG.integers(0, 2 ** 64, (count, N), dtype=np.uint64)
    b = RNG.integers(-2 ** 7, 2 ** 7, (count, N))
    bhat = torch.empty((count, N // 2), dtype=torch.complex128, device="cuda")
    plan.prepare_operand(torch.from_numpy(b).cuda(), bhat)
    out = np.zeros_like(a)
    plan.product(a, bhat, out)  # host entry point
    want = oracle.u64_product(N, 2, 1024, a, bhat.cpu().numpy(), nthreads=0)
    assert np.array_equal(out, want)


@pytest.mark.parametrize("N,count", [(2048, 2000), (65536, 80)])
def test_u64_product_host_page_locked_out(cuda, oracle, N, count):
    """Host entry point with page-locked host buffers: the kernels store the results
    into host memory themselves (no copy out).  Same bits as the copy path."""
    import concrete_fft as cf
    torch = cuda
    plan = cf.product.U64ProductPlan(N, 2, 1024)
    a = RNG.integers(0, 2 ** 64, (count, N), dtype=np.uint64)
    b = RNG.integers(-2 ** 7, 2 ** 7, (count, N))
    bhat = torch.empty((count, N // 2), dtype=torch.complex128, device="cuda")
    plan.prepare_operand(torch.from_numpy(b).cuda(), bhat)
    ha = torch.from_numpy(a.view(np.int64)).pin_memory()
    hout = torch.full_like(ha, -1).pin_memory()
    plan.product(ha, bhat, hout)
    copied = np.zeros_like(a)
    plan.product(a, bhat, copied)  # pageable: copies in and out
    assert np.array_equal(hout.numpy().view(np.uint64), copied)
    sel = [0, count // 2, count - 1]
    want = oracle.u64_product(N, 2, 1024, a[sel], bhat[sel].cpu().numpy(), nthreads=0)
    assert np.array_equal(copied[sel], want)


@pytest.mark.parametrize("N,count", [(1024, 700), (16384, 100)])
def test_u128_product_host_page_locked_out(cuda, oracle, N, count):
    import concrete_fft as cf
    torch = cuda
    plan = cf.product.U128ProductPlan(N)
    a = RNG.integers(0, 2 ** 64, (count, N, 2), dtype=np.uint64)
    b = RNG.integers(-2 ** 15, 2 ** 15, (count, N))
    bhat = torch.empty((count, 4, N // 2), dtype=torch.float64, device="cuda")
    plan.prepare_operand(torch.from_numpy(b).cuda(), bhat)
    ha = torch.from_numpy(a.view(np.int64)).pin_memory()
    hout = torch.full_like(ha, -1).pin_memory()
    plan.product(ha, bhat, hout)
    copied = np.zeros_like(a)
    plan.product(a, bhat, copied)
    assert np.array_equal(hout.numpy().view(np.uint64), copied)
    sel = [0, count - 1]
    want = oracle.u128_product(N, a[sel], bhat[sel].cpu().numpy(), nthreads=0)
    assert np.array_equal(copied[sel], want)


def negacyclic_shift(c, d):
    """c * X^d mod (X^N + 1) for integer rows c (int64, wrapping)."""
    N = c.shape[-1]
    d %= 2 * N
    out = np.roll(c, d % N, axis=-1)
    j = np.arange(N)
    flip = (j < d % N) ^ (d >= N)
    return np.where(flip, -out, out)


@pytest.mark.parametrize("N,algo,base", [(2048, 2, 1024), (2048, 6, 256), (16384, 2, 1024), (131072, 2, 1024)])
def test_u64_fourier_mul_monomial(cuda, oracle, N, algo, base):
    """Fourier-domain multiplication by X^d (the blind-rotation step): bit-identical to the
    oracle's prepared monomial times the operand, and a product with the rotated operand is
    the rotated product, exactly, for small inputs."""
    import concrete_fft as cf
    torch = cuda
    plan = cf.product.U64ProductPlan(N, algo, base)
    count = 2
    b = RNG.integers(-2 ** 7, 2 ** 7, (count, N))
    bhat = torch.empty((count, N // 2), dtype=torch.complex128, device="cuda")
    plan.prepare_operand(torch.from_numpy(b).cuda(), bhat)
    a = RNG.integers(-2 ** 10, 2 ** 10, (count, N)).astype(np.int64)
    base_out = torch.empty((count, N), dtype=torch.int64, device="cuda")
    plan.product(torch.from_numpy(a).cuda(), bhat, base_out)
    base_out = base_out.cpu().numpy()
    for d in (0, 1, N - 1, N, N + 7, 2 * N - 1, 5 * N + 3):
        z = bhat.clone()
        plan.fourier_mul_monomial(d, z)
        dm = d % (2 * N)
        digits = np.zeros((1, N), dtype=np.int64)
        digits[0, dm % N] = -1 if dm >= N else 1
        mono = oracle.u64_prepare(N, algo, base, digits)[0]
        want = oracle.c64_pointwise(mono, bhat.cpu().numpy())
        assert np.array_equal(bits(z.cpu().numpy()), bits(want)), (N, d)
        out = torch.empty((count, N), dtype=torch.int64, device="cuda")
        plan.product(torch.from_numpy(a).cuda(), z, out)
        assert np.array_equal(out.cpu().numpy(), negacyclic_shift(base_out, d)), (N, d)


def test_u64_measure_plan(cuda, oracle):
    import concrete_fft as cf
    plan = cf.product.U64ProductPlan(2048, measure_seconds=0.001)
    algo, base = plan.algo()
    assert base in (512, 1024) and 0 <= int(algo) <= 7


@pytest.mark.parametrize("N", [64, 128, 256, 512, 1024, 2048, 4096, 8192])
def test_u128_product_bit_exact(cuda, oracle, N):
    """A few products: the one-CTA kernel (N = 64), a cluster of 1-8 CTAs
    (N = 128..2048) or of 16 (N = 4096, 8192; five launches where such a cluster
    does not fit); the oracle's bits."""
    import concrete_fft as cf
    torch = cuda
    count = 3
    plan = cf.product.U128ProductPlan(N)
    a = RNG.integers(0, 2 ** 64, (count, N, 2), dtype=np.uint64)
    b = RNG.integers(-2 ** 15, 2 ** 15, (count, N))
    bhat = torch.empty((count, 4, N // 2), dtype=torch.float64, device="cuda")
    plan.prepare_operand(torch.from_numpy(b).cuda(), bhat)
    want_bhat = oracle.u128_prepare(N, b)
    assert np.array_equal(bhat.cpu().numpy().view(np.uint64), want_bhat.view(np.uint64))
    da = torch.from_numpy(a.view(np.int64)).cuda()
    out = torch.empty_like(da)
    plan.product(da, bhat, out)
    got = out.cpu().numpy().view(np.uint64)
    assert np.array_equal(got, oracle.u128_product(N, a, want_bhat, nthreads=0))
    small = RNG.integers(-2 ** 40, 2 ** 40, (1, N)).astype(np.int64)
    a2 = np.stack([small.view(np.uint64), np.where(small < 0, np.uint64(2 ** 64 - 1), np.uint64(0))], -1)
    da2 = torch.from_numpy(a2.view(np.int64)).cuda()
    out2 = torch.empty_like(da2)
    plan.product(da2, bhat[:1], out2)
    assert np.array_equal(out2.cpu().numpy().view(np.uint64), oracle.u128_schoolbook(a2, b[:1]))


@pytest.mark.parametrize("N,algo,base", [(64, 2, 32), (128, 6, 64), (128, 3, 32)])
def test_u64_product_small_N_packed(cuda, oracle, N, algo, base):
    """N <= 128: several products per CTA iteration (512 points); 1003 products, so the
    last group is ragged.  Every product equals the oracle's."""
    import concrete_fft as cf
    torch = cuda
    count = 1003
    plan = cf.product.U64ProductPlan(N, algo, base)
    a = RNG.integers(0, 2 ** 64, (count, N), dtype=np.uint64)
    b = RNG.integers(-2 ** 7, 2 ** 7, (count, N))
    bhat = torch.empty((count, N // 2), dtype=torch.complex128, device="cuda")
    plan.prepare_operand(torch.from_numpy(b).cuda(), bhat)
    want_bhat = oracle.u64_prepare(N, algo, base, b)
    da = torch.from_numpy(a.view(np.int64)).cuda()
    out = torch.empty_like(da)
    plan.product(da, bhat, out)
    assert np.array_equal(out.cpu().numpy().view(np.uint64), oracle.u64_product(N, algo, base, a, want_bhat, nthreads=0))
    shared = torch.empty_like(da)
    plan.product(da, bhat[:1], shared, shared_operand=True)
    want = oracle.u64_product(N, algo, base, a, np.repeat(want_bhat[:1], count, axis=0), nthreads=0)
    assert np.array_equal(shared.cpu().numpy().view(np.uint64), want)


@pytest.mark.parametrize("N,algo,base", [(16384, 2, 1024), (16384, 5, 512), (32768, 2, 1024), (65536, 6, 1024),
                                         (131072, 2, 1024), (1 << 22, 6, 1024)])
def test_u64_product_large_N(cuda, oracle, N, algo, base):
    """N > 8192: a thread-block cluster per product up to 65536, five launches above;
    bit-exact against the CPU pipeline, exact against the schoolbook when the sums fit
    in 53 bits."""
    import concrete_fft as cf
    torch = cuda
    plan = cf.product.U64ProductPlan(N, algo, base)
    count = 3
    a = RNG.integers(0, 2 ** 64, (count, N), dtype=np.uint64)
    b = RNG.integers(-2 ** 7, 2 ** 7, (count, N))
    bhat = torch.empty((count, N // 2), dtype=torch.complex128, device="cuda")
    plan.prepare_operand(torch.from_numpy(b).cuda(), bhat)
    da = torch.from_numpy(a.view(np.int64)).cuda()
    out = torch.empty_like(da)
    plan.product(da, bhat, out)
    want = oracle.u64_product(N, algo, base, a, bhat.cpu().numpy(), nthreads=0)
    assert np.array_equal(out.cpu().numpy().view(np.uint64), want)
    if N == 16384:
        small = RNG.integers(-2 ** 20, 2 ** 20, (1, N)).astype(np.int64)
        out1 = torch.empty((1, N), dtype=torch.int64, device="cuda")
        plan.product(torch.from_numpy(small).cuda(), bhat[:1], out1)
        exact = oracle.u64_schoolbook(small.view(np.uint64), b[:1])
        assert np.array_equal(out1.cpu().numpy().view(np.uint64), exact)


@pytest.mark.parametrize("N,base", [(4096, 1024), (8192, 1024), (8192, 256), (2048, 64), (16384, 1024)])
def test_u64_product_cluster_sizes_bit_identical(cuda, N, base):
    """Small batches on clusters of 2/4/8 CTAs give the one-CTA kernel's bits."""
    import concrete_fft as cf
    torch = cuda
    for algo in (2, 3, 4):
        plan = cf.product.U64ProductPlan(N, algo, base)
        count = 5
        a = torch.from_numpy(RNG.integers(0, 2 ** 64, (count, N), dtype=np.uint64).view(np.int64)).cuda()
        b = torch.from_numpy(RNG.integers(-2 ** 7, 2 ** 7, (count, N))).cuda()
        bhat = torch.empty((count, N // 2), dtype=torch.complex128, device="cuda")
        plan.prepare_operand(b, bhat)
        ref = torch.empty_like(a)
        plan.set_cluster_size(1)
        plan.product(a, bhat, ref)
        for ctas in (2, 4, 8, 0):
            plan.set_cluster_size(ctas)
            out = torch.zeros_like(a)
            plan.product(a, bhat, out)
            assert torch.equal(out, ref), (N, base, algo, ctas)


@pytest.mark.parametrize("N,base", [(2048, 1024), (1024, 512), (256, 128)])
def test_u64_product_no_level_clusters_bit_exact(cuda, oracle, N, base):
    """Plans whose transform has no outer level (n = base_n) on clusters of 2/4/8 CTAs
    (the residue classes of the base algorithm's passes), for all eight base
    algorithms, DIF and DIT: the oracle's bits at every cluster size."""
    import concrete_fft as cf
    torch = cuda
    count = 3
    for algo in range(8):
        plan = cf.product.U64ProductPlan(N, algo, base)
        assert plan.algo() == (algo, base)
        a = RNG.integers(0, 2 ** 64, (count, N), dtype=np.uint64)
        b = RNG.integers(-2 ** 7, 2 ** 7, (count, N))
        bhat = torch.empty((count, N // 2), dtype=torch.complex128, device="cuda")
        plan.prepare_operand(torch.from_numpy(b).cuda(), bhat)
        want_bhat = oracle.u64_prepare(N, algo, base, b)
        want = oracle.u64_product(N, algo, base, a, want_bhat, nthreads=0)
        da = torch.from_numpy(a.view(np.int64)).cuda()
        for ctas in (1, 2, 4, 8, 0):
            plan.set_cluster_size(ctas)
            out = torch.zeros_like(da)
            plan.product(da, bhat, out)
            assert np.array_equal(out.cpu().numpy().view(np.uint64), want), (N, algo, ctas)


def test_u64_product_no_level_clusters_up_to_one_per_sm(cuda):
    """Up to one product per SM on a radix-4 base runs on clusters by default: the
    same bits as one CTA per product, at 120 and 152 products."""
    import concrete_fft as cf
    torch = cuda
    plan = cf.product.U64ProductPlan(2048, 2, 1024)
    for count in (120, 152):
        a = torch.from_numpy(RNG.integers(0, 2 ** 64, (count, 2048), dtype=np.uint64).view(np.int64)).cuda()
        b = torch.from_numpy(RNG.integers(-2 ** 7, 2 ** 7, (count, 2048))).cuda()
        bhat = torch.empty((count, 1024), dtype=torch.complex128, device="cuda")
        plan.prepare_operand(b, bhat)
        out0 = torch.zeros_like(a)
        plan.set_cluster_size(0)
        plan.product(a, bhat, out0)
        out1 = torch.zeros_like(a)
        plan.set_cluster_size(1)
        plan.product(a, bhat, out1)
        plan.set_cluster_size(0)
        assert torch.equal(out0, out1), count


@pytest.mark.parametrize("N,base", [(4096, 1024), (8192, 1024), (4096, 512), (2048, 512), (16384, 1024)])
def test_u64_product_one_level_clusters_bit_exact(cuda, oracle, N, base):
    """A few products of a plan with one outer level (radix 2, 4 or 8) run on a cluster
    of level-0 slices times classes of the base, 16 CTAs where such a cluster fits
    (DIF bases; DIT bases take another path): the oracle's bits, and the same bits on
    one CTA per product."""
    import concrete_fft as cf
    torch = cuda
    count = 3
    for algo in range(8):
        plan = cf.product.U64ProductPlan(N, algo, base)
        a = RNG.integers(0, 2 ** 64, (count, N), dtype=np.uint64)
        b = RNG.integers(-2 ** 7, 2 ** 7, (count, N))
        bhat = torch.empty((count, N // 2), dtype=torch.complex128, device="cuda")
        plan.prepare_operand(torch.from_numpy(b).cuda(), bhat)
        want = oracle.u64_product(N, algo, base, a, oracle.u64_prepare(N, algo, base, b), nthreads=0)
        da = torch.from_numpy(a.view(np.int64)).cuda()
        for ctas in (0, 1):
            plan.set_cluster_size(ctas)
            out = torch.zeros_like(da)
            plan.product(da, bhat, out)
            assert np.array_equal(out.cpu().numpy().view(np.uint64), want), (N, base, algo, ctas)


@pytest.mark.parametrize("N", [16384, 32768, 1 << 21])
def test_u128_product_large_N(cuda, oracle, N):
    """N > 8192: five launches around the fft128 plan, bit-exact against the CPU pipeline
    (operand preparation included), exact against the schoolbook for small inputs."""
    import concrete_fft as cf
    torch = cuda
    count = 2
    plan = cf.product.U128ProductPlan(N)
    a = RNG.integers(0, 2 ** 64, (count, N, 2), dtype=np.uint64)
    b = RNG.integers(-2 ** 15, 2 ** 15, (count, N))
    bhat = torch.empty((count, 4, N // 2), dtype=torch.float64, device="cuda")
    plan.prepare_operand(torch.from_numpy(b).cuda(), bhat)
    want_bhat = oracle.u128_prepare(N, b)
    assert np.array_equal(bhat.cpu().numpy().view(np.uint64), want_bhat.view(np.uint64))
    da = torch.from_numpy(a.view(np.int64)).cuda()
    out = torch.empty_like(da)
    plan.product(da, bhat, out)
    assert np.array_equal(out.cpu().numpy().view(np.uint64), oracle.u128_product(N, a, want_bhat, nthreads=0))
    if N == 16384:
        small = RNG.integers(-2 ** 40, 2 ** 40, (1, N)).astype(np.int64)
        a2 = np.stack([small.view(np.uint64), np.where(small < 0, np.uint64(2 ** 64 - 1), np.uint64(0))], -1)
        out2 = torch.empty((1, N, 2), dtype=torch.int64, device="cuda")
        plan.product(torch.from_numpy(a2.view(np.int64)).cuda(), bhat[:1], out2)
        assert np.array_equal(out2.cpu().numpy().view(np.uint64), oracle.u128_schoolbook(a2, b[:1]))


def test_u128_product_host_pipeline(cuda, oracle):
    """Host entry point for u128 products over several pipelined chunks, one operand per
    product, against the device entry point (itself checked against the oracle above)."""
    import concrete_fft as cf
    torch = cuda
    N, count = 1024, 700
    plan = cf.product.U128ProductPlan(N)
    a = RNG.integers(0, 2 ** 64, (count, N, 2), dtype=np.uint64)
    b = RNG.integers(-2 ** 15, 2 ** 15, (count, N))
    bhat = torch.empty((count, 4, N // 2), dtype=torch.float64, device="cuda")
    plan.prepare_operand(torch.from_numpy(b).cuda(), bhat)
    host_out = np.zeros_like(a)
    plan.product(a, bhat, host_out)
    da = torch.from_numpy(a.view(np.int64)).cuda()
    out = torch.empty_like(da)
    plan.product(da, bhat, out)
    assert np.array_equal(host_out, out.cpu().numpy().view(np.uint64))
    sel = [0, 299, 699]
    want = oracle.u128_product(N, a[sel], bhat[sel].cpu().numpy(), nthreads=0)
    assert np.array_equal(host_out[sel], want)


@pytest.mark.parametrize("N,algo,base,terms", [(2048, 2, 1024, 8), (1024, 4, 512, 3), (4096, 6, 1024, 1),
                                               (8192, 3, 1024, 2), (16384, 2, 1024, 3), (32768, 6, 1024, 2),
                                               (1 << 18, 2, 1024, 3), (2048, 6, 1024, 4), (2048, 0, 1024, 2),
                                               (2048, 3, 1024, 3), (512, 2, 256, 2), (4096, 2, 1024, 3),
                                               (8192, 4, 1024, 2), (4096, 0, 1024, 2), (8192, 6, 1024, 2),
                                               (16384, 4, 1024, 2), (16384, 6, 1024, 2), (8192, 2, 1024, 3)])
def test_u64_product_sum_bit_exact(cuda, oracle, N, algo, base, terms):
    """Fourier-domain accumulation of `terms` products, one inverse per group (4 groups:
    a cluster per group for plans on a DIF base without an outer level or with one of
    radix 2, 4 or 8)."""
    import concrete_fft as cf
    torch = cuda
    count = 4
    plan = cf.product.U64ProductPlan(N, algo, base)
    a = RNG.integers(0, 2 ** 64, (count, terms, N), dtype=np.uint64)
    b = RNG.integers(-2 ** 7, 2 ** 7, (count * terms, N))
    bhat = torch.empty((count, terms, N // 2), dtype=torch.complex128, device="cuda")
    plan.prepare_operand(torch.from_numpy(b).cuda(), bhat)
    out = torch.empty((count, N), dtype=torch.int64, device="cuda")
    plan.product_sum(torch.from_numpy(a.view(np.int64)).cuda(), bhat, out)
    want_bhat = oracle.u64_prepare(N, algo, base, b).reshape(count, terms, N // 2)
    want = oracle.u64_product_sum(N, algo, base, a, want_bhat, nthreads=0)
    assert np.array_equal(out.cpu().numpy().view(np.uint64), want)
    if N <= 32768:  # the schoolbook is quadratic in N
        exact = sum(oracle.u64_schoolbook(a[0, t], b[t]) for t in range(terms))
        assert torus_err_bits(want[0], exact.astype(np.uint64)) < 30


def test_u64_product_sum_unfused_chunks(cuda, oracle):
    """Above N = 65536 the sum runs unfused, its groups in chunks within a 1 GiB
    workspace: N = 2^21, 2 terms (96 MiB a group), 23 groups -> chunks of 21 and 2."""
    import concrete_fft as cf
    torch = cuda
    N, terms, count = 1 << 21, 2, 23
    plan = cf.product.U64ProductPlan(N, 2, 1024)
    a = RNG.integers(0, 2 ** 64, (count, terms, N), dtype=np.uint64)
    b = RNG.integers(-2 ** 7, 2 ** 7, (count * terms, N))
    bhat = torch.empty((count, terms, N // 2), dtype=torch.complex128, device="cuda")
    plan.prepare_operand(torch.from_numpy(b).cuda(), bhat)
    out = torch.empty((count, N), dtype=torch.int64, device="cuda")
    plan.product_sum(torch.from_numpy(a.view(np.int64)).cuda(), bhat, out)
    sel = [0, 20, 21, 22]  # both sides of the chunk boundary
    want_bhat = oracle.u64_prepare(N, 2, 1024, b.reshape(count, terms, N)[sel].reshape(-1, N))
    want_bhat = want_bhat.reshape(len(sel), terms, N // 2)
    assert np.array_equal(bhat[sel].cpu().numpy().view(np.uint64), want_bhat.view(np.uint64))
    want = oracle.u64_product_sum(N, 2, 1024, a[sel], want_bhat, nthreads=0)
    assert np.array_equal(out.cpu().numpy().view(np.uint64)[sel], want)
