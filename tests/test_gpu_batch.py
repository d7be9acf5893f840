"""Mixed-size persistent batches: every item bit-identical to its plan's oracle result."""
import numpy as np
import pytest

from conftest import bits

pytestmark = pytest.mark.gpu
RNG = np.random.default_rng(21)


def make_items(count, max_log2=16, seed=0):
    rng = np.random.default_rng(seed)
    items, off = [], 0
    for _ in range(count):
        kind = int(rng.integers(0, 2))
        log2n = int(rng.integers(1, (10 if kind == 0 else max_log2) + 1))
        direction = int(rng.integers(1, 4))
        items.append((off, log2n, kind, direction))
        off += 1 << log2n
    perm = rng.permutation(len(items))  # items are not stored in queue order
    return [items[i] for i in perm], off


def expected(oracle, b, items, data):
    out = data.copy()
    for off, log2n, kind, direction in items:
        n = 1 << log2n
        algo, base, _ = b.schedule(kind, log2n, direction)
        x = data[off:off + n]
        if kind == 0:
            if direction & 1:
                x = oracle.ordered_fwd(int(algo), x)
            if direction & 2:
                x = oracle.ordered_inv(int(algo), x)
        else:
            if direction & 1:
                x = oracle.unordered_fwd(int(algo), base, x)
            if direction & 2:
                x = oracle.unordered_inv(int(algo), base, x)
        out[off:off + n] = x
    return out


@pytest.mark.parametrize("tune", [0.0, 0.0005])
def test_mixed_batch_bit_exact(cuda, oracle, tune):
    import concrete_fft as cf
    torch = cuda
    items, total = make_items(120 if tune == 0 else 40, seed=int(tune * 1e4))
    data = RNG.uniform(-1, 1, total) + 1j * RNG.uniform(-1, 1, total)
    b = cf.batch.Batch(items, tune_seconds=tune)
    assert b.units() > 0
    d = torch.from_numpy(data.copy()).cuda()
    b.run(d)
    assert np.array_equal(bits(d.cpu().numpy()), bits(expected(oracle, b, items, data)))


def test_graph_replay_and_default_stream(cuda, oracle):
    import concrete_fft as cf
    torch = cuda
    items, total = make_items(60, max_log2=13, seed=5)
    data = RNG.uniform(-1, 1, total) + 1j * RNG.uniform(-1, 1, total)
    want = None
    b = cf.batch.Batch(items)
    d = torch.from_numpy(data.copy()).cuda()
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        for _ in range(3):  # capture on the first run, replay on the next two
            d.copy_(torch.from_numpy(data))
            b.run(d)
            torch.cuda.current_stream().synchronize()
            got = d.cpu().numpy()
            want = expected(oracle, b, items, data) if want is None else want
            assert np.array_equal(bits(got), bits(want))
    d.copy_(torch.from_numpy(data))
    b.run(d, stream=0)  # the legacy stream: direct launch, no graph
    torch.cuda.synchronize()
    assert np.array_equal(bits(d.cpu().numpy()), bits(want))


def test_host_pipelined_run_bit_exact(cuda, oracle):
    """cfft_batch_run_host: items with gaps between them, in shuffled order, split into
    chunks and pipelined; every item equals the oracle, gaps stay untouched on the host."""
    import concrete_fft as cf
    torch = cuda
    rng = np.random.default_rng(5)
    items, off = [], 0
    for _ in range(90):
        kind = int(rng.integers(0, 2))
        log2n = int(rng.integers(4, (10 if kind == 0 else 14) + 1))
        items.append((off, log2n, kind, int(rng.integers(1, 4))))
        off += (1 << log2n) + int(rng.integers(0, 3)) * 8  # gaps of 0, 8 or 16 points
    items = [items[i] for i in rng.permutation(len(items))]
    data = rng.uniform(-1, 1, off) + 1j * rng.uniform(-1, 1, off)
    b = cf.batch.Batch(items)
    host = torch.from_numpy(data.copy()).pin_memory()
    dev = torch.zeros(off, dtype=torch.complex128, device="cuda")
    for _ in range(2):  # second call reuses the chunk tables
        host.copy_(torch.from_numpy(data))
        b.run_host(host, dev)
        torch.cuda.synchronize()
        got = host.numpy()
        assert np.array_equal(bits(got), bits(expected(oracle, b, items, data)))


def test_batch_rejects_bad_items(cuda):
    import concrete_fft as cf
    with pytest.raises(cf.CfftError):
        cf.batch.Batch([(0, 11, 0, 1)])  # ordered above 1024 points (src/ordered.rs:244)
    with pytest.raises(cf.CfftError):
        cf.batch.Batch([(0, 17, 1, 1)])
    with pytest.raises(cf.CfftError):
        cf.batch.Batch([(0, 4, 1, 0)])
