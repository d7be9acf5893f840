"""Mixed-size product engine, the unfused pipeline, and the continuous-batching
server: bit-identical to the oracle, and every served result equal to the same
request computed alone."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
RNG = np.random.default_rng(17)
SIZES = [10, 11, 12, 13, 14]


@pytest.fixture(scope="module")
def engine(cuda):
    import concrete_fft as cf
    return cf.serving.ProductEngine(SIZES)


def test_engine_mixed_sizes_bit_exact(cuda, oracle, engine):
    import concrete_fft as cf
    torch = cuda
    items, keep = [], []
    for lN in SIZES + SIZES[::-1]:
        N = 1 << lN
        count = 2
        a = RNG.integers(0, 2 ** 64, (count, N), dtype=np.uint64)
        b = RNG.integers(-2 ** 7, 2 ** 7, (count, N))
        bhat = torch.empty((count, N // 2), dtype=torch.complex128, device="cuda")
        engine.prepare_operand(lN, torch.from_numpy(b).cuda(), bhat)
        da = torch.from_numpy(a.view(np.int64)).cuda()
        out = torch.zeros_like(da)
        for p in range(count):
            items.append((da[p].data_ptr(), bhat[p].data_ptr(), out[p].data_ptr(), lN, 0))
        keep.append((lN, a, b, bhat, da, out))
    arr = np.array(items, dtype=cf.serving.ITEM_DTYPE)
    d_items = torch.from_numpy(arr.view(np.uint8)).cuda()
    counter = torch.zeros(4, dtype=torch.int32, device="cuda")
    ws_bytes = engine.workspace_bytes()
    assert ws_bytes > 0  # N = 8192 and 16384 use the workspace
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device="cuda")
    engine.run(d_items, len(arr), counter, ws, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    for lN, a, b, bhat, da, out in keep:
        N = 1 << lN
        algo, base = engine.algo(lN)
        want_bhat = oracle.u64_prepare(N, algo, base, b)
        assert np.array_equal(bhat.cpu().numpy().view(np.uint64), want_bhat.view(np.uint64)), lN
        want = oracle.u64_product(N, algo, base, a, want_bhat, nthreads=0)
        assert np.array_equal(out.cpu().numpy().view(np.uint64), want), lN


@pytest.mark.parametrize("lN", [11, 14])
def test_unfused_pipeline_equals_fused(cuda, oracle, engine, lN):
    import concrete_fft as cf
    torch = cuda
    L = cf.load()
    N, count = 1 << lN, 3
    plan = engine.plan(lN)
    fft = ctypes.c_void_p(L.cfft_u64_product_fft(plan))
    a = RNG.integers(0, 2 ** 64, (count, N), dtype=np.uint64)
    b = RNG.integers(-2 ** 7, 2 ** 7, (count, N))
    bhat = torch.empty((count, N // 2), dtype=torch.complex128, device="cuda")
    engine.prepare_operand(lN, torch.from_numpy(b).cuda(), bhat)
    da = torch.from_numpy(a.view(np.int64)).cuda()
    z = torch.empty((count, N // 2), dtype=torch.complex128, device="cuda")
    out = torch.empty_like(da)
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    cf.check(L.cfft_u64_fold_twist(plan, p(da), p(z), count, s))
    cf.check(L.cfft_unordered_fwd(fft, p(z), count, s))
    cf.check(L.cfft_c64_pointwise(p(bhat), N // 2, p(z), N // 2, count, s))
    cf.check(L.cfft_unordered_inv(fft, p(z), count, s))
    cf.check(L.cfft_u64_untwist_round(plan, p(z), p(out), count, s))
    algo, base = engine.algo(lN)
    want = oracle.u64_product(N, algo, base, a, oracle.u64_prepare(N, algo, base, b), nthreads=0)
    assert np.array_equal(out.cpu().numpy().view(np.uint64), want)


@pytest.mark.parametrize("staged_io,via_queue,cluster_log2N", [(False, False, 0), (True, False, 0), (False, True, 0),
                                                               (False, False, 10), (False, True, 10)])
def test_server_results_same_alone_and_in_the_mix(cuda, oracle, engine, staged_io, via_queue, cluster_log2N):
    """Every recorded result of the batched loop equals the request run alone, with the
    kernels reading item records from and storing results into page-locked host memory
    (default) and with per-launch copies (staged_io); cluster_log2N = 10 puts every size
    on thread-block clusters (N = 1024 and 2048, whose plans have no outer level,
    included)."""
    import concrete_fft as cf
    srv = cf.serving.Server(engine, SIZES, operand_bytes=64 << 20, ring_bytes=256 << 20, seed=9)
    cfg = srv.config(rate=20000, duration_s=0.05, record_every=1, staged_io=staged_io, via_queue=via_queue,
                     cluster_log2N=cluster_log2N)
    stats = srv.run(cfg)
    assert stats["requests"] > 100 and stats["launches"] < stats["requests"]  # batching happened (the
    # queue counts its own launches: 0 here)
    ids = srv.recorded_ids()
    assert len(ids) == stats["requests"]
    for rid in ids[:: max(1, len(ids) // 40)]:
        mixed = srv.recorded_output(cfg, rid)
        alone = srv.run_alone(cfg, rid)
        assert np.array_equal(mixed, alone), rid
    for rid in ids[:3]:
        digits, bhat = srv.inputs(cfg, rid)
        lN, npd = srv.shape(cfg, rid)
        algo, base = engine.algo(lN)
        want = oracle.u64_product(1 << lN, algo, base, digits.view(np.uint64), bhat, nthreads=0)
        assert np.array_equal(srv.recorded_output(cfg, rid), want)


def test_plain_server_same_results(cuda, engine):
    import concrete_fft as cf
    srv = cf.serving.Server(engine, SIZES, operand_bytes=64 << 20, ring_bytes=256 << 20, seed=9)
    cfg = srv.config(rate=2000, duration_s=0.02, record_every=1, plain=True)
    stats = srv.run(cfg)
    assert stats["launches"] == 5 * stats["products"]
    for rid in srv.recorded_ids()[:10]:
        assert np.array_equal(srv.recorded_output(cfg, rid), srv.run_alone(cfg, rid))


def test_server_memory_gate(cuda, engine):
    """A ring that holds only a couple of requests still serves everything (admission waits)."""
    import concrete_fft as cf
    srv = cf.serving.Server(engine, [12], operand_bytes=16 << 20, ring_bytes=3 * 16 * (1 << 12) * 8, seed=3)
    cfg = srv.config(rate=50000, duration_s=0.01, log2N_min=12, log2N_max=12, record_every=1)
    stats = srv.run(cfg)
    assert stats["deferred_admissions"] > 0
    assert len(srv.recorded_ids()) == stats["requests"]
    with pytest.raises(cf.CfftError):
        srv.run(srv.config(rate=100, duration_s=0.01, log2N_min=12, log2N_max=14))  # sizes without pools


@pytest.mark.parametrize("staged_io,via_queue", [(False, False), (True, False), (False, True)])
def test_server_device_memory_gate(cuda, engine, staged_io, via_queue):
    """Admission is gated on the device's free memory, read during the run: with a faked free
    memory of 1.5 MiB (the output of the largest request, 12 products at N = 2^14) requests are
    held back by the gate, every request is still served, and every recorded result equals the
    request run alone.  A generous reserve against the real free
    memory defers as well; none does with the real reading and no reserve."""
    import concrete_fft as cf
    srv = cf.serving.Server(engine, SIZES, operand_bytes=64 << 20, ring_bytes=256 << 20, seed=4)
    cfg = srv.config(rate=40000, duration_s=0.03, record_every=1, staged_io=staged_io, via_queue=via_queue,
                     mem_free_override=3 << 19)
    stats = srv.run(cfg)
    assert stats["memory_deferrals"] > 0
    assert 0 < stats["min_memory_budget_mib"] <= 1.5
    ids = srv.recorded_ids()
    assert len(ids) == stats["requests"] > 100
    assert stats["output_bytes"] == sum(srv.shape(cfg, int(r))[1] << (srv.shape(cfg, int(r))[0] + 3) for r in ids)
    for rid in ids[:: max(1, len(ids) // 30)]:
        assert np.array_equal(srv.recorded_output(cfg, rid), srv.run_alone(cfg, rid)), rid
    free = cuda.cuda.mem_get_info()[0]
    tight = srv.run(srv.config(rate=40000, duration_s=0.01, mem_reserve_bytes=free - (1 << 20)))
    assert tight["memory_deferrals"] > 0 and tight["min_memory_budget_mib"] < 8
    loose = srv.run(srv.config(rate=40000, duration_s=0.01))
    assert loose["memory_deferrals"] == 0 and loose["min_memory_budget_mib"] > 1024


def _queue_requests(torch, engine, rng, nreq, host_out=False):
    """nreq requests of 1..6 products of random configured sizes, each with its own
    operand; returns (items per request, buffers to keep, expected results)."""
    import concrete_fft as cf
    reqs = []
    for _ in range(nreq):
        lN = int(rng.choice(SIZES))
        N = 1 << lN
        k = int(rng.integers(1, 7))
        a = rng.integers(0, 2 ** 64, (k, N), dtype=np.uint64)
        b = rng.integers(-2 ** 7, 2 ** 7, (k, N))
        bhat = torch.empty((k, N // 2), dtype=torch.complex128, device="cuda")
        engine.prepare_operand(lN, torch.from_numpy(b).cuda(), bhat)
        da = torch.from_numpy(a.view(np.int64)).cuda()
        out = torch.full((k, N), -1, dtype=torch.int64)
        out = out.pin_memory() if host_out else out.cuda()
        items = np.array([(da[p].data_ptr(), bhat[p].data_ptr(), out[p].data_ptr(), lN, 0) for p in range(k)],
                         dtype=cf.serving.ITEM_DTYPE)
        reqs.append((items, (lN, da, bhat, out)))
    return reqs


@pytest.mark.parametrize("host_out", [False, True])
def test_product_queue_threads(cuda, engine, host_out):
    """The submit / poll / wait API: four threads submit requests concurrently; every
    result equals the same products run alone through cfft_u64_product."""
    import threading
    import concrete_fft as cf
    torch = cuda
    q = cf.serving.ProductQueue(engine)
    rng = np.random.default_rng(31)
    per_thread = [_queue_requests(torch, engine, rng, 40, host_out) for _ in range(4)]
    torch.cuda.synchronize()
    errors = []

    def worker(reqs):
        try:
            tickets = [q.submit(items) for items, _ in reqs]
            for t in tickets[::2]:
                q.wait(t)
            for t in tickets[1::2]:
                while not q.poll(t):
                    pass
            assert all(q.poll(t) for t in tickets)  # done tickets stay done
        except Exception as e:  # reported by the main thread
            errors.append(repr(e))

    ts = [threading.Thread(target=worker, args=(r,)) for r in per_thread]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert not errors, errors
    for reqs in per_thread:
        for items, (lN, da, bhat, out) in reqs:
            want = torch.empty_like(da)
            cf.check(cf.load().cfft_u64_product(engine.plan(lN), da.data_ptr(), bhat.data_ptr(), (1 << lN) // 2,
                                                want.data_ptr(), len(items), torch.cuda.current_stream().cuda_stream))
            torch.cuda.synchronize()
            assert torch.equal(out.cpu(), want.cpu()), lN
    q.close()


def test_product_queue_errors_and_shutdown(cuda, engine):
    """Unconfigured sizes and pageable buffers are refused at submit; unknown tickets
    fail; closing the queue runs everything submitted first."""
    import concrete_fft as cf
    torch = cuda
    q = cf.serving.ProductQueue(engine, max_inflight=1)
    rng = np.random.default_rng(32)
    reqs = _queue_requests(torch, engine, rng, 30)
    torch.cuda.synchronize()
    bad = reqs[0][0].copy()
    bad["log2N"] = 20
    with pytest.raises(cf.CfftError):
        q.submit(bad)
    pageable = np.zeros((1, 1 << SIZES[0]), dtype=np.uint64)
    bad = reqs[0][0][:1].copy()
    bad["log2N"] = SIZES[0]
    bad["out"] = pageable.ctypes.data
    with pytest.raises(cf.CfftError):
        q.submit(bad)
    with pytest.raises(cf.CfftError):
        q.poll(10 ** 9)
    assert q.poll(q.submit(np.zeros(0, dtype=cf.serving.ITEM_DTYPE)))  # an empty group is done at once
    for items, _ in reqs:
        q.submit(items)
    q.close()  # returns after the 30 requests ran
    for items, (lN, da, bhat, out) in reqs:
        assert int((out == -1).all(dim=1).sum()) == 0, lN
