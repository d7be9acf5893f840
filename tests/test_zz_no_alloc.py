"""The product engine's no-allocation entry point.

Some callers cannot allocate device memory on their call path (their host
framework's allocator has reserved the device budget, or the loop is too
latency-critical for cudaMalloc/cudaFree, which synchronise the device).
cfft_product_engine_run_static serves them: it takes its work-queue counter and
its large-N workspace from a static device array instead of caller buffers.
This checks that it returns the same bits as cfft_product_engine_run (with a
caller-provided workspace) on two calls in a row, and that sizes beyond its
24 MiB workspace limit are rejected.  It lives in its own file, collected
last, and passes alone in a fresh process as well as after the other tests.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _items(torch, cf, engine, sizes, rng, count=3):
    items, outs, keep = [], [], []
    for lN in sizes:
        N = 1 << lN
        a = torch.from_numpy(rng.integers(0, 2 ** 64, (count, N), dtype=np.uint64).view(np.int64)).cuda()
        b = torch.from_numpy(rng.integers(-2 ** 7, 2 ** 7, (count, N))).cuda()
        bhat = torch.empty((count, N // 2), dtype=torch.complex128, device="cuda")
        engine.prepare_operand(lN, b, bhat)
        out = torch.zeros_like(a)
        for p in range(count):
            items.append((a[p].data_ptr(), bhat[p].data_ptr(), out[p].data_ptr(), lN, 0))
        outs.append(out)
        keep.append((a, bhat))
    arr = np.array(items, dtype=cf.serving.ITEM_DTYPE)
    return torch.from_numpy(arr.view(np.uint8)).cuda(), len(arr), outs, keep


def test_no_alloc_entry_point_matches_regular_run(cuda):
    import concrete_fft as cf
    torch = cuda
    sizes = [11, 13, 14]  # N = 8192 and 16384 use the workspace
    engine = cf.serving.ProductEngine(sizes)
    rng = np.random.default_rng(123)
    d_items, count, outs, keep = _items(torch, cf, engine, sizes, rng)
    stream = torch.cuda.current_stream().cuda_stream

    counter = torch.zeros(4, dtype=torch.int32, device="cuda")
    ws = torch.empty(engine.workspace_bytes(), dtype=torch.uint8, device="cuda")
    engine.run(d_items, count, counter, ws, stream)
    torch.cuda.synchronize()
    ref = [o.clone() for o in outs]

    for _ in range(2):  # two calls in a row share the static array
        for o in outs:
            o.zero_()
        engine.run_static(d_items, count, stream)
        torch.cuda.synchronize()
        for got, want in zip(outs, ref):
            assert torch.equal(got, want)


def test_no_alloc_entry_point_caps_its_grid_to_the_static_workspace(cuda):
    """320 products of N = 16384 (128 KiB of workspace each) and 64 of N = 2048: more CTAs
    than the 24 MiB array holds slices for (192), so the call runs on the capped grid, and
    the small items of the same call share it."""
    import concrete_fft as cf
    torch = cuda
    engine = cf.serving.ProductEngine([11, 14])
    rng = np.random.default_rng(321)
    d_big, n_big, outs_big, keep_big = _items(torch, cf, engine, [14], rng, count=320)
    d_small, n_small, outs_small, keep_small = _items(torch, cf, engine, [11], rng, count=64)
    d_items = torch.cat([d_big, d_small])
    count = n_big + n_small
    outs = outs_big + outs_small
    stream = torch.cuda.current_stream().cuda_stream
    counter = torch.zeros(4, dtype=torch.int32, device="cuda")
    ws = torch.empty(engine.workspace_bytes(), dtype=torch.uint8, device="cuda")
    engine.run(d_items, count, counter, ws, stream)
    torch.cuda.synchronize()
    ref = [o.clone() for o in outs]
    for _ in range(2):
        for o in outs:
            o.zero_()
        engine.run_static(d_items, count, stream)
        torch.cuda.synchronize()
        for got, want in zip(outs, ref):
            assert torch.equal(got, want)


def test_no_alloc_entry_point_rejects_sizes_beyond_its_limit(cuda):
    import concrete_fft as cf
    torch = cuda
    engine = cf.serving.ProductEngine([15])  # N = 32768: 256 KiB of workspace per CTA
    dummy = torch.zeros(64, dtype=torch.uint8, device="cuda")
    with pytest.raises(cf.CfftError) as err:
        engine.run_static(dummy, 1, torch.cuda.current_stream().cuda_stream)
    assert err.value.status == -1
    assert "24 MiB" in str(err.value) and "16384" in str(err.value)
