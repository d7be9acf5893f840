"""Plans shared by several host threads at once (the reference's Plan is Send + Sync):
device calls on per-thread streams and the pipelined host entry points, each thread's
results equal to the same calls made alone."""
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_threads_share_plans(cuda):
    import concrete_fft as cf
    torch = cuda
    N = 2048
    ordered = cf.ordered.Plan(1024, cf.ordered.Method.UserProvided(cf.FftAlgo.Dif4))
    unordered = cf.unordered.Plan(4096, cf.unordered.Method.UserProvided(cf.FftAlgo.Dit8, 512))
    prod = cf.product.U64ProductPlan(N, cf.FftAlgo.Dif4, 1024)
    rng = np.random.default_rng(17)
    nthreads, iters = 4, 10
    xs = [rng.uniform(-1, 1, (37, 1024)) + 1j * rng.uniform(-1, 1, (37, 1024)) for _ in range(nthreads)]
    us = [rng.uniform(-1, 1, (3, 4096)) + 1j * rng.uniform(-1, 1, (3, 4096)) for _ in range(nthreads)]
    a = [rng.integers(0, 2 ** 64, (300, N), dtype=np.uint64) for _ in range(nthreads)]
    b = rng.integers(-2 ** 7, 2 ** 7, (300, N))
    bhat = torch.empty((300, N // 2), dtype=torch.complex128, device="cuda")
    prod.prepare_operand(torch.from_numpy(b).cuda(), bhat)
    torch.cuda.synchronize()

    def alone(i):
        d = torch.from_numpy(xs[i]).cuda()
        ordered.fwd(d)
        u = torch.from_numpy(us[i]).cuda()
        unordered.fwd(u)
        unordered.inv(u)
        out = np.zeros_like(a[i])
        prod.product(a[i], bhat, out)
        torch.cuda.synchronize()
        return d.cpu().numpy(), u.cpu().numpy(), out

    want = [alone(i) for i in range(nthreads)]
    errors = []

    def worker(i):
        try:
            s = torch.cuda.Stream()
            for _ in range(iters):
                with torch.cuda.stream(s):
                    d = torch.from_numpy(xs[i]).cuda()
                    ordered.fwd(d)
                    u = torch.from_numpy(us[i]).cuda()
                    unordered.fwd(u)
                    unordered.inv(u)
                s.synchronize()
                out = np.zeros_like(a[i])
                prod.product(a[i], bhat, out)  # host entry point: this thread's own pipeline
                got = (d.cpu().numpy(), u.cpu().numpy(), out)
                for g, w in zip(got, want[i]):
                    if not np.array_equal(np.asarray(g).view(np.uint64), np.asarray(w).view(np.uint64)):
                        errors.append(i)
                        return
        except Exception as e:  # reported by the main thread
            errors.append(repr(e))

    ts = [threading.Thread(target=worker, args=(i,)) for i in range(nthreads)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert not errors, errors
