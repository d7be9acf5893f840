"""GPU ordered/unordered c64 transforms vs the oracle: bit-identical results."""
import os

import numpy as np
import pytest

from conftest import bits

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
RNG = np.random.default_rng(7)


def rand_c64(*shape):
    return RNG.uniform(-1, 1, shape) + 1j * RNG.uniform(-1, 1, shape)


def on_gpu(torch, x):
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


@pytest.mark.parametrize("algo", range(8))
def test_ordered_all_sizes_bit_exact(cuda, oracle, algo):
    import concrete_fft as cf
    torch = cuda
    for e in range(0, 11):
        n = 1 << e
        plan = cf.ordered.Plan(n, cf.ordered.Method.UserProvided(algo))
        assert plan.fft_size() == n and plan.algo() == algo and plan.fft_scratch() == 0
        batch = 3 if n > 64 else 37  # ragged: not a multiple of transforms per CTA
        x = rand_c64(batch, n)
        d = on_gpu(torch, x)
        plan.fwd(d)
        want = oracle.ordered_fwd(algo, x) if n > 1 else x
        assert np.array_equal(bits(d.cpu().numpy()), bits(want)), (algo, n)
        plan.inv(d)
        want_inv = oracle.ordered_inv(algo, want) if n > 1 else x
        assert np.array_equal(bits(d.cpu().numpy()), bits(want_inv)), (algo, n)


def test_ordered_batch_256_n1024(cuda, oracle):
    """The N = 1024, batch 256 fwd-then-inv workload."""
    import concrete_fft as cf
    torch = cuda
    x = rand_c64(256, 1024)
    for algo in (6, 7, 2):
        plan = cf.ordered.Plan(1024, cf.ordered.Method.UserProvided(algo))
        d = on_gpu(torch, x)
        plan.fwd(d)
        plan.inv(d)
        want = oracle.ordered_inv(algo, oracle.ordered_fwd(algo, x))
        assert np.array_equal(bits(d.cpu().numpy()), bits(want))
        rel = np.linalg.norm(d.cpu().numpy() / 1024 - x) / np.linalg.norm(x)
        assert rel < 1e-13


@pytest.mark.parametrize("algo", [2, 3])
def test_int_adds_levels_bit_exact(cuda, oracle, algo):
    """Ordered and unordered transforms at every integer-pipe addition level."""
    import concrete_fft as cf
    torch = cuda
    for n in (16, 256, 1024):
        plan = cf.ordered.Plan(n, cf.ordered.Method.UserProvided(algo))
        x = rand_c64(7, n)
        want_f = oracle.ordered_fwd(algo, x)
        want_i = oracle.ordered_inv(algo, want_f)
        for e in (0, 4):
            plan.set_int_adds(e)
            d = on_gpu(torch, x)
            plan.fwd(d)
            assert np.array_equal(bits(d.cpu().numpy()), bits(want_f)), (n, e)
            plan.inv(d)
            assert np.array_equal(bits(d.cpu().numpy()), bits(want_i)), (n, e)
    for n, base in ((2048, 512), (8192, 1024), (65536, 64)):
        plan = cf.unordered.Plan(n, cf.unordered.Method.UserProvided(algo, base))
        x = rand_c64(2, n)
        want = oracle.unordered_fwd(algo, base, x, nthreads=0)
        for e in (0, 4):
            plan.set_int_adds(e)
            d = on_gpu(torch, x)
            plan.fwd(d)
            assert np.array_equal(bits(d.cpu().numpy()), bits(want)), (n, base, e)


def test_unordered_golden_vector_on_gpu(cuda):
    """The reference's exact golden vector (src/unordered.rs:1176-9395) reproduced by the GPU."""
    import concrete_fft as cf
    torch = cuda
    inp = np.load(os.path.join(GOLDEN, "unordered_fwd_n2048_dif4_base32_input.npy"))
    exp = np.load(os.path.join(GOLDEN, "unordered_fwd_n2048_dif4_base32_expected.npy"))
    plan = cf.unordered.Plan(2048, cf.unordered.Method.UserProvided(cf.FftAlgo.Dif4, 32))
    d = on_gpu(torch, inp.copy())
    plan.fwd(d)
    assert np.array_equal(bits(d.cpu().numpy()), bits(exp))
    h = inp.copy()
    plan.fwd(h)  # host entry point
    assert np.array_equal(bits(h), bits(exp))


CASES = [(32, 32), (64, 32), (256, 32), (1024, 32), (1024, 512), (1024, 1024), (2048, 1024), (4096, 64),
         (8192, 1024), (16384, 512), (65536, 1024), (65536, 32), (1 << 20, 1024), (1 << 22, 1024), (1 << 22, 32)]


@pytest.mark.parametrize("batch", [1, 5, 64])
def test_host_entry_page_locked_in_place(cuda, oracle, batch):
    """Host entry points on page-locked buffers: one-kernel transforms read and write
    the caller's memory in place (split over a cluster below 16 transforms, one CTA
    per transform above).  Bits equal the oracle's."""
    import concrete_fft as cf
    torch = cuda
    for algo in (2, 3, 6):
        plan = cf.ordered.Plan(1024, cf.ordered.Method.UserProvided(algo))
        x = rand_c64(batch, 1024)
        h = torch.from_numpy(x.copy()).pin_memory()
        plan.fwd(h)
        want = oracle.ordered_fwd(algo, x)
        assert np.array_equal(bits(h.numpy()), bits(want)), (algo, batch)
        plan.inv(h)
        assert np.array_equal(bits(h.numpy()), bits(oracle.ordered_inv(algo, want))), (algo, batch)
    plan = cf.unordered.Plan(2048, cf.unordered.Method.UserProvided(2, 256))
    x = rand_c64(batch, 2048)
    h = torch.from_numpy(x.copy()).pin_memory()
    plan.fwd(h)
    assert np.array_equal(bits(h.numpy()), bits(oracle.unordered_fwd(2, 256, x, nthreads=0)))


def test_host_mapping_seen_from_any_thread(cuda):
    """The zero-copy host paths engage for page-locked memory, from the main thread and
    from other threads, and not for device or pageable memory."""
    import ctypes
    import threading
    import concrete_fft as cf
    torch = cuda
    L = cf.load()

    def mapped(ptr, n):
        d = ctypes.c_void_p()
        cf.check(L.cfft_diag_host_mapping(ctypes.c_void_p(ptr), n, ctypes.byref(d)))
        return d.value is not None

    pinned = torch.zeros(1 << 16, dtype=torch.int64).pin_memory()
    dev = torch.zeros(1 << 16, dtype=torch.int64, device="cuda")
    pageable = np.zeros(1 << 16, dtype=np.int64)
    assert mapped(pinned.data_ptr(), pinned.numel() * 8)
    assert mapped(pinned.data_ptr() + 4096, 4096)
    assert not mapped(dev.data_ptr(), 8)
    assert not mapped(pageable.ctypes.data, 8)
    seen = []
    t = threading.Thread(target=lambda: seen.append(mapped(pinned.data_ptr(), pinned.numel() * 8)))
    t.start()
    t.join()
    assert seen == [True]


def test_host_entry_registered_memory(cuda, oracle):
    """Host memory page-locked by cudaHostRegister (its device address is looked up,
    not assumed equal to the host pointer): in-place transforms and product results."""
    import concrete_fft as cf
    torch = cuda
    rt = torch.cuda.cudart()
    x = rand_c64(40, 1024)
    h = np.ascontiguousarray(x.copy())
    assert int(rt.cudaHostRegister(h.ctypes.data, h.nbytes, 0)) == 0
    try:
        plan = cf.ordered.Plan(1024, cf.ordered.Method.UserProvided(2))
        plan.fwd(h)
        assert np.array_equal(bits(h), bits(oracle.ordered_fwd(2, x)))
    finally:
        rt.cudaHostUnregister(h.ctypes.data)
    N, count = 2048, 300
    pp = cf.product.U64ProductPlan(N, 2, 1024)
    a = RNG.integers(0, 2 ** 64, (count, N), dtype=np.uint64)
    b = RNG.integers(-2 ** 7, 2 ** 7, (count, N))
    bhat = torch.empty((count, N // 2), dtype=torch.complex128, device="cuda")
    pp.prepare_operand(torch.from_numpy(b).cuda(), bhat)
    out = np.zeros_like(a)
    assert int(rt.cudaHostRegister(out.ctypes.data, out.nbytes, 0)) == 0
    try:
        pp.product(a, bhat, out)
    finally:
        rt.cudaHostUnregister(out.ctypes.data)
    want = oracle.u64_product(N, 2, 1024, a[[0, 299]], bhat[[0, 299]].cpu().numpy(), nthreads=0)
    assert np.array_equal(out[[0, 299]], want)


@pytest.mark.parametrize("n,base", CASES)
def test_unordered_bit_exact(cuda, oracle, n, base):
    import concrete_fft as cf
    torch = cuda
    batch = max(1, min(5, (1 << 18) // n))
    algos = (6, 3) if n < (1 << 18) else (6,)
    for algo in algos:
        plan = cf.unordered.Plan(n, cf.unordered.Method.UserProvided(algo, base))
        x = rand_c64(batch, n)
        d = on_gpu(torch, x)
        plan.fwd(d)
        want = oracle.unordered_fwd(algo, base, x, nthreads=0)
        assert np.array_equal(bits(d.cpu().numpy()), bits(want)), (n, base, algo)
        plan.inv(d)
        want = oracle.unordered_inv(algo, base, want, nthreads=0)
        assert np.array_equal(bits(d.cpu().numpy()), bits(want)), (n, base, algo)
        assert np.abs(d.cpu().numpy() / n - x).max() < 1e-12


@pytest.mark.parametrize("n,base", [(4096, 1024), (4096, 512), (32768, 1024), (16384, 64), (1 << 18, 1024)])
def test_block_points_bit_exact(cuda, oracle, n, base):
    """Every shared-memory block size a plan allows (its level sizes of at most 4096
    points; the levels above run in global memory) gives the oracle's bits."""
    import concrete_fft as cf
    torch = cuda
    plan = cf.unordered.Plan(n, cf.unordered.Method.UserProvided(6, base))
    auto = plan.block_points()
    x = rand_c64(2, n)
    want_f = oracle.unordered_fwd(6, base, x, nthreads=0)
    want_i = oracle.unordered_inv(6, base, want_f, nthreads=0)
    sizes, cur = [n], n
    while cur > base:
        cur //= 2 if cur == 2 * base else (4 if cur == 4 * base else 8)
        sizes.append(cur)
    for pts in [s for s in sizes if s <= 4096]:
        plan.set_block_points(pts)
        assert plan.block_points() == pts
        d = on_gpu(torch, x)
        plan.fwd(d)
        assert np.array_equal(bits(d.cpu().numpy()), bits(want_f)), (n, base, pts)
        plan.inv(d)
        assert np.array_equal(bits(d.cpu().numpy()), bits(want_i)), (n, base, pts)
    with pytest.raises(cf.CfftError):
        plan.set_block_points(2 * n if n <= 2048 else 8192)
    plan.set_block_points(0)
    assert plan.block_points() == auto


@pytest.mark.parametrize("ctas", [1, 2, 4, 8, 0])
def test_cluster_sizes_bit_exact(cuda, oracle, ctas):
    """One transform spread over a thread-block cluster (distributed shared memory)
    gives the same bits as one CTA per transform, for every algorithm and size."""
    import concrete_fft as cf
    torch = cuda
    for algo in range(8):
        for e in (6, 7, 9, 10):
            n = 1 << e
            plan = cf.ordered.Plan(n, cf.ordered.Method.UserProvided(algo))
            plan.set_cluster_size(ctas)
            x = rand_c64(3, n)
            d = on_gpu(torch, x)
            plan.fwd(d)
            want = oracle.ordered_fwd(algo, x)
            assert np.array_equal(bits(d.cpu().numpy()), bits(want)), (algo, n, ctas)
            plan.inv(d)
            want = oracle.ordered_inv(algo, want)
            assert np.array_equal(bits(d.cpu().numpy()), bits(want)), (algo, n, ctas)
    # with one outer level of radix 2, 4 or 8 over a DIF base, clusters of up to 16 CTAs
    # (automatic, for a small batch) take level 0's slices times the base's classes
    for n, base in [(256, 32), (1024, 64), (2048, 1024), (2048, 512), (4096, 1024), (4096, 512), (8192, 1024),
                    (16384, 512), (32768, 1024)]:
        for algo in ((0, 2, 4, 6, 7) if n in (2048, 4096, 8192) else (2, 7)):
            plan = cf.unordered.Plan(n, cf.unordered.Method.UserProvided(algo, base))
            plan.set_cluster_size(ctas)
            x = rand_c64(2, n)
            d = on_gpu(torch, x)
            plan.fwd(d)
            want = oracle.unordered_fwd(algo, base, x)
            assert np.array_equal(bits(d.cpu().numpy()), bits(want)), (n, base, algo, ctas)
            plan.inv(d)
            want = oracle.unordered_inv(algo, base, want)
            assert np.array_equal(bits(d.cpu().numpy()), bits(want)), (n, base, algo, ctas)


@pytest.mark.parametrize("n,base", [(16384, 1024), (16384, 512), (32768, 1024), (65536, 1024), (1 << 17, 1024)])
def test_levels_then_clusters_bit_exact(cuda, oracle, n, base):
    """A few transforms with two or more outer levels over a DIF base: the levels above
    the last in global memory, then every sub-transform on a cluster of level-0 slices
    times base classes.  Bits equal the oracle's, in both directions."""
    import concrete_fft as cf
    torch = cuda
    for algo in (0, 2, 4, 6):
        plan = cf.unordered.Plan(n, cf.unordered.Method.UserProvided(algo, base))
        for batch in (1, 3):
            x = rand_c64(batch, n)
            d = on_gpu(torch, x)
            plan.fwd(d)
            want = oracle.unordered_fwd(algo, base, x, nthreads=0)
            assert np.array_equal(bits(d.cpu().numpy()), bits(want)), (n, base, algo, batch)
            plan.inv(d)
            want = oracle.unordered_inv(algo, base, want, nthreads=0)
            assert np.array_equal(bits(d.cpu().numpy()), bits(want)), (n, base, algo, batch)


@pytest.mark.parametrize("batch", [1, 256])
def test_plan_calls_capture_into_a_cuda_graph(cuda, oracle, batch):
    """fwd and inv enqueue only kernels on the caller's stream, so a caller can capture
    them into a CUDA graph and replay it; replays give the oracle's bits."""
    import concrete_fft as cf
    torch = cuda
    for algo in (2, 3):
        plan = cf.ordered.Plan(1024, cf.ordered.Method.UserProvided(algo))
        x = rand_c64(batch, 1024)
        d = on_gpu(torch, x)
        plan.fwd(d)  # first calls outside the capture (kernel attributes are set once)
        plan.inv(d)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            plan.fwd(d)
            plan.inv(d)
        d.copy_(on_gpu(torch, x))
        g.replay()
        want = oracle.ordered_inv(algo, oracle.ordered_fwd(algo, x))
        assert np.array_equal(bits(d.cpu().numpy()), bits(want)), (algo, batch)
        d.copy_(on_gpu(torch, x))
        g.replay()
        g.replay()
        want = oracle.ordered_inv(algo, oracle.ordered_fwd(algo, want))
        assert np.array_equal(bits(d.cpu().numpy()), bits(want)), (algo, batch)


@pytest.mark.parametrize("n", [256, 1024, 4096])
def test_monomial_and_serde_order(cuda, oracle, n):
    import concrete_fft as cf
    torch = cuda
    for base in {32, n // 4, min(n, 1024)}:
        plan = cf.unordered.Plan(n, cf.unordered.Method.UserProvided(2, base))
        for d in RNG.integers(0, n, 3):
            buf = torch.zeros(n, dtype=torch.complex128, device="cuda")
            plan.fwd_monomial(int(d), buf)
            assert np.array_equal(bits(buf.cpu().numpy()), bits(oracle.fwd_monomial(n, base, int(d))))
        x = rand_c64(2, n)
        d = on_gpu(torch, x)
        std = torch.empty_like(d)
        plan.to_standard(d, std)
        assert np.array_equal(bits(std.cpu().numpy()), bits(oracle.to_standard(n, base, x)))
        back = torch.empty_like(d)
        plan.from_standard(std, back)
        assert np.array_equal(bits(back.cpu().numpy()), bits(x))


@pytest.mark.parametrize("batch", [1, 3, 8, 24])
def test_serde_tiles_and_batches(cuda, oracle, batch):
    """Standard-order conversion at every size class (shared-memory tiles of one or
    several transforms for n = 64..4096, global gather otherwise) and ragged batches."""
    import concrete_fft as cf
    torch = cuda
    for n, base in [(32, 32), (64, 32), (128, 64), (1024, 32), (1024, 512), (2048, 1024), (4096, 64), (8192, 1024)]:
        plan = cf.unordered.Plan(n, cf.unordered.Method.UserProvided(2, base))
        x = rand_c64(batch, n)
        d = on_gpu(torch, x)
        std = torch.empty_like(d)
        plan.to_standard(d, std)
        assert np.array_equal(bits(std.cpu().numpy()), bits(oracle.to_standard(n, base, x))), (n, base, batch)
        back = torch.empty_like(d)
        plan.from_standard(std, back)
        assert np.array_equal(bits(back.cpu().numpy()), bits(x)), (n, base, batch)


@pytest.mark.parametrize("pinned", [False, True])
def test_serde_host_device_in_one_call(cuda, oracle, pinned):
    """Serialized (standard-order) host data straight into device Fourier buffers and
    back, page-locked (read and written by the permutation kernel) or pageable (staged)."""
    import concrete_fft as cf
    torch = cuda
    for n, base in [(64, 32), (1024, 32), (2048, 1024), (8192, 1024), (65536, 64)]:
        plan = cf.unordered.Plan(n, cf.unordered.Method.UserProvided(2, base))
        x = rand_c64(3, n)
        std = torch.from_numpy(x.copy())
        if pinned:
            std = std.pin_memory()
        dev = torch.empty((3, n), dtype=torch.complex128, device="cuda")
        plan.from_standard(std, dev)
        torch.cuda.synchronize()
        assert np.array_equal(bits(dev.cpu().numpy()), bits(oracle.from_standard(n, base, x))), (n, base)
        back = torch.zeros_like(std)
        if pinned:
            back = back.pin_memory()
        plan.to_standard(dev, back)
        torch.cuda.synchronize()
        assert np.array_equal(bits(back.numpy()), bits(x)), (n, base)
    # a serialized product operand loads straight into the product plan's Fourier layout
    L = cf.load()
    N = 4096
    pp = cf.product.U64ProductPlan(N, 2, 512)
    b = RNG.integers(-2 ** 7, 2 ** 7, (2, N))
    want = oracle.u64_prepare(N, 2, 512, b)
    wire = torch.from_numpy(oracle.to_standard(N // 2, 512, want))
    if pinned:
        wire = wire.pin_memory()
    bhat = torch.empty((2, N // 2), dtype=torch.complex128, device="cuda")
    cf.check(L.cfft_unordered_from_standard_h2d(L.cfft_u64_product_fft(pp._h), wire.data_ptr(), bhat.data_ptr(), 2,
                                                torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    assert np.array_equal(bits(bhat.cpu().numpy()), bits(want))


def test_serde_roundtrip_across_bases(cuda, oracle):
    """src/unordered.rs:9399-9466 on the GPU: base-32 forward, standard order, base-64 inverse."""
    import concrete_fft as cf
    torch = cuda
    for n in (64, 128, 256, 512, 1024):
        p1 = cf.unordered.Plan(n, cf.unordered.Method.UserProvided(2, 32))
        p2 = cf.unordered.Plan(n, cf.unordered.Method.UserProvided(2, 64))
        x = rand_c64(n)
        d = on_gpu(torch, x)
        p1.fwd(d)
        std = p1.serialize_fourier_buffer(d)
        back = torch.empty_like(d)
        p2.deserialize_fourier_buffer(std, back)
        p2.inv(back)
        assert np.abs(back.cpu().numpy() / n - x).max() < 1e-12
    with pytest.raises(cf.CfftError):
        p2.deserialize_fourier_buffer(torch.zeros(n - 1, dtype=torch.complex128, device="cuda"), back)


def test_measure_plans(cuda, oracle):
    import concrete_fft as cf
    torch = cuda
    p = cf.ordered.Plan(1024, cf.ordered.Method.Measure(0.002))
    x = rand_c64(4, 1024)
    d = on_gpu(torch, x)
    p.fwd(d)
    assert np.array_equal(bits(d.cpu().numpy()), bits(oracle.ordered_fwd(int(p.algo()), x)))
    u = cf.unordered.Plan(4096, cf.unordered.Method.Measure(0.002))
    algo, base = u.algo()
    assert base in (512, 1024)
    d = on_gpu(torch, x.reshape(1, 4096))
    u.fwd(d)
    assert np.array_equal(bits(d.cpu().numpy()), bits(oracle.unordered_fwd(int(algo), base, x.reshape(1, 4096))))


def test_measure_results_are_persisted(cuda, oracle, tmp_path):
    """A second Measure plan of the same size reuses the stored choice (no re-timing);
    after save / clear / load it is reused again."""
    import time
    import concrete_fft as cf
    L = cf.load()
    L.cfft_tune_clear()
    t0 = time.perf_counter()
    p1 = cf.unordered.Plan(2048, cf.unordered.Method.Measure(0.002))
    t_measure = time.perf_counter() - t0
    assert L.cfft_tune_entries() == 1
    path = str(tmp_path / "tune.txt").encode()
    cf.check(L.cfft_tune_save(path))
    L.cfft_tune_clear()
    cf.check(L.cfft_tune_load(path))
    t0 = time.perf_counter()
    p2 = cf.unordered.Plan(2048, cf.unordered.Method.Measure(0.002))
    t_cached = time.perf_counter() - t0
    assert p2.algo() == p1.algo() and p2.int_adds() == p1.int_adds()
    assert t_cached < t_measure / 5
    L.cfft_tune_clear()


def test_invalid_calls_raise(cuda):
    import concrete_fft as cf
    torch = cuda
    p = cf.ordered.Plan(64, cf.ordered.Method.UserProvided(0))
    with pytest.raises(ValueError):
        p.fwd(torch.zeros(65, dtype=torch.complex128, device="cuda"))
    with pytest.raises(cf.CfftError):
        cf.ordered.Plan(2048, cf.ordered.Method.UserProvided(0))
    u = cf.unordered.Plan(64, cf.unordered.Method.UserProvided(0, 64))
    with pytest.raises(cf.CfftError):
        u.fwd_monomial(64, torch.zeros(64, dtype=torch.complex128, device="cuda"))
