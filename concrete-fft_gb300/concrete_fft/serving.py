"""Continuous-batching request loop for negacyclic u64 products of mixed N.

A request is a set of (k+1)*l products: digit polynomials (small signed
integers, N coefficients each) times Fourier-domain operands that stay
resident on the device (the shape of a TFHE external product).  The server
admits requests as they arrive while device memory is available, copies their
inputs in, batches everything admitted since the last launch into one
persistent product-engine launch, and lets up to `max_inflight` launches run
at once on separate streams, so requests that arrive while others are on the
GPU overlap with them.  Completed requests are detected per launch and their
latency (arrival to result in host memory) is recorded.

`PlainServer` is the comparator: the reference API's usage pattern, one
request at a time, each product through the unfused pipeline with one launch
per step (fold+twist, forward transform, pointwise, inverse transform,
untwist+round).
"""
import ctypes
import time
from collections import deque

import numpy as np
import torch

from . import _buffers as B
from ._lib import check, load

ITEM_DTYPE = np.dtype([("a", np.uint64), ("bhat", np.uint64), ("out", np.uint64), ("log2N", np.uint32),
                       ("reserved", np.uint32)])


class ProductEngine:
    """cfft_product_engine_* of include/cfft.h."""

    def __init__(self, log2Ns):
        self._lib = load()
        arr = (ctypes.c_uint32 * len(log2Ns))(*log2Ns)
        h = ctypes.c_void_p()
        check(self._lib.cfft_product_engine_create(arr, len(log2Ns), ctypes.byref(h)))
        self._h = h
        self.log2Ns = sorted(set(int(x) for x in log2Ns))

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.cfft_product_engine_destroy(self._h)
            self._h = None

    def workspace_bytes(self):
        return self._lib.cfft_product_engine_workspace_bytes(self._h)

    def plan(self, log2N):
        return self._lib.cfft_product_engine_plan(self._h, log2N)

    def prepare_operand(self, log2N, b, bhat, stream):
        """b: (count, N) int64 device tensor -> bhat (count, N/2) complex128 device tensor."""
        count = b.numel() >> log2N
        check(self._lib.cfft_u64_prepare_operand(ctypes.c_void_p(self.plan(log2N)), B.ptr(b), B.ptr(bhat), count,
                                                 ctypes.c_void_p(stream.cuda_stream)))

    def run(self, d_items, count, counter, workspace, stream):
        check(self._lib.cfft_product_engine_run(self._h, ctypes.c_void_p(d_items.data_ptr()), count,
                                                ctypes.c_void_p(counter.data_ptr()),
                                                ctypes.c_void_p(workspace.data_ptr()) if workspace is not None else None,
                                                ctypes.c_void_p(stream.cuda_stream)))


class Ring:
    """Byte ring on one device buffer: allocations in admission order, released in
    completion order (oldest first).  Capacity is the admission gate."""

    def __init__(self, nbytes):
        self.cap = int(nbytes)
        self.head = 0  # next free byte (monotonic)
        self.tail = 0  # oldest live byte (monotonic)
        self.live = deque()  # (start, end) in allocation order, with a done flag
        self.done = {}

    def alloc(self, nbytes):
        nbytes = (int(nbytes) + 255) & ~255
        pos = self.head % self.cap
        pad = self.cap - pos if pos + nbytes > self.cap else 0  # never split across the wrap
        if self.head + pad + nbytes - self.tail > self.cap:
            return None
        start = self.head + pad
        self.head = start + nbytes
        self.live.append((start, self.head))
        self.done[start] = False
        return start % self.cap

    def release(self, start_mod_list):
        for s in start_mod_list:
            for st, en in self.live:
                if st % self.cap == s and not self.done[st]:
                    self.done[st] = True
                    break
        while self.live and self.done[self.live[0][0]]:
            st, en = self.live.popleft()
            del self.done[st]
            self.tail = en


class Request:
    __slots__ = ("rid", "arrival", "log2N", "nprod", "digits", "operands", "out", "t_done", "in_off", "out_off")

    def __init__(self, rid, arrival, log2N, digits, operands):
        self.rid, self.arrival, self.log2N = rid, arrival, log2N
        self.digits = digits      # host (nprod, N) int64, pinned slice
        self.operands = operands  # operand indices into the resident set of this N
        self.nprod = digits.shape[0]
        self.out = None
        self.t_done = None


class ResidentOperands:
    """Fourier-domain operands of each N, resident on the device."""

    def __init__(self, engine, total_bytes, seed=0, device="cuda"):
        self.bhat = {}
        rng = np.random.default_rng(seed)
        per = total_bytes // len(engine.log2Ns)
        s = torch.cuda.Stream()
        for lN in engine.log2Ns:
            N = 1 << lN
            count = max(1, per // (N // 2 * 16))
            bh = torch.empty((count, N // 2), dtype=torch.complex128, device=device)
            chunk = max(1, (1 << 26) // (N * 8))
            for c0 in range(0, count, chunk):
                c = min(chunk, count - c0)
                src = torch.from_numpy(rng.integers(0, 2 ** 64, (c, N), dtype=np.uint64).view(np.int64)).to(device)
                with torch.cuda.stream(s):
                    engine.prepare_operand(lN, src, bh[c0:c0 + c], s)
                s.synchronize()
            self.bhat[lN] = bh

    def count(self, lN):
        return self.bhat[lN].shape[0]

    def ptr(self, lN, idx):
        t = self.bhat[lN]
        return t.data_ptr() + int(idx) * t.stride(0) * 16


class Server:
    """Continuous batching over the product engine."""

    def __init__(self, engine, operands, mem_bytes=None, max_inflight=3, mem_fraction=0.5):
        self.engine, self.ops = engine, operands
        if mem_bytes is None:
            free, _ = torch.cuda.mem_get_info()
            mem_bytes = int(free * mem_fraction)
        self.ring = Ring(mem_bytes)
        self.mem = torch.empty(self.ring.cap, dtype=torch.uint8, device="cuda")
        self.base = self.mem.data_ptr()
        self.max_inflight = max_inflight
        self.streams = [torch.cuda.Stream() for _ in range(max_inflight)]
        ws = engine.workspace_bytes()
        self.ws = [torch.empty(max(ws, 16), dtype=torch.uint8, device="cuda") if ws else None
                   for _ in range(max_inflight)]
        self.counters = torch.zeros(max_inflight * 64, dtype=torch.int32, device="cuda")
        self.item_host = [torch.empty(0, dtype=torch.uint8).pin_memory() for _ in range(max_inflight)]
        self.item_dev = [torch.empty(0, dtype=torch.uint8, device="cuda") for _ in range(max_inflight)]
        self.inflight = deque()  # (slot, event, requests, out_host_views)
        self.slot_busy = [False] * max_inflight
        self.launches = 0

    def _admit(self, req):
        N = 1 << req.log2N
        nbytes = req.nprod * N * 8
        a_off = self.ring.alloc(nbytes)
        if a_off is None:
            return False
        o_off = self.ring.alloc(nbytes)
        if o_off is None:
            self.ring.release([a_off])
            return False
        req.in_off, req.out_off = a_off, o_off
        return True

    def _launch(self, reqs):
        slot = self.slot_busy.index(False)
        s = self.streams[slot]
        n_items = sum(r.nprod for r in reqs)
        items = np.zeros(n_items, dtype=ITEM_DTYPE)
        i = 0
        outs = []
        with torch.cuda.stream(s):
            for r in reqs:
                N = 1 << r.log2N
                nb = r.nprod * N * 8
                dst = self.mem[r.in_off:r.in_off + nb]
                dst.copy_(r.digits.view(-1).view(torch.uint8), non_blocking=True)
                a0 = self.base + r.in_off
                o0 = self.base + r.out_off
                k = np.arange(r.nprod, dtype=np.uint64)
                items["a"][i:i + r.nprod] = a0 + k * np.uint64(N * 8)
                items["out"][i:i + r.nprod] = o0 + k * np.uint64(N * 8)
                items["bhat"][i:i + r.nprod] = [self.ops.ptr(r.log2N, j) for j in r.operands]
                items["log2N"][i:i + r.nprod] = r.log2N
                i += r.nprod
            raw = torch.from_numpy(items.view(np.uint8))
            if self.item_host[slot].numel() < raw.numel():
                self.item_host[slot] = torch.empty(raw.numel() * 2, dtype=torch.uint8).pin_memory()
                self.item_dev[slot] = torch.empty(raw.numel() * 2, dtype=torch.uint8, device="cuda")
            self.item_host[slot][:raw.numel()].copy_(raw)
            self.item_dev[slot][:raw.numel()].copy_(self.item_host[slot][:raw.numel()], non_blocking=True)
            self.engine.run(self.item_dev[slot], n_items, self.counters[slot * 64:slot * 64 + 1], self.ws[slot], s)
            for r in reqs:
                N = 1 << r.log2N
                nb = r.nprod * N * 8
                r.out = torch.empty((r.nprod, N), dtype=torch.int64).pin_memory() if r.out is None else r.out
                r.out.view(-1).view(torch.uint8).copy_(self.mem[r.out_off:r.out_off + nb], non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(s)
        self.slot_busy[slot] = True
        self.inflight.append((slot, ev, reqs))
        self.launches += 1

    def _poll(self, block=False):
        done = []
        while self.inflight:
            slot, ev, reqs = self.inflight[0]
            if block:
                ev.synchronize()
            elif not ev.query():
                break
            self.inflight.popleft()
            t = time.perf_counter()
            for r in reqs:
                r.t_done = t
                self.ring.release([r.in_off, r.out_off])
            self.slot_busy[slot] = False
            done.extend(reqs)
        return done

    def serve(self, requests, t_start=None):
        """Serve `requests` (sorted by arrival, seconds relative to t_start) in real time."""
        pending = deque(requests)
        admitted = []
        waiting = deque()
        finished = []
        t0 = time.perf_counter() if t_start is None else t_start
        while pending or waiting or admitted or self.inflight:
            now = time.perf_counter() - t0
            while pending and pending[0].arrival <= now:
                waiting.append(pending.popleft())
            while waiting and self._admit(waiting[0]):
                admitted.append(waiting.popleft())
            if admitted and not all(self.slot_busy):
                self._launch(admitted)
                admitted = []
            finished.extend(self._poll(block=all(self.slot_busy) and bool(admitted)))
            if not admitted and not waiting and pending and not self.inflight:
                # idle until the next arrival
                dt = pending[0].arrival - (time.perf_counter() - t0)
                if dt > 0:
                    time.sleep(min(dt, 1e-4))
        for r in finished:
            r.t_done = r.t_done - t0
        return finished


class PlainServer:
    """One request at a time, one launch per pipeline step and product (the
    reference API's call pattern on the GPU Plan path)."""

    def __init__(self, engine, operands):
        self.engine, self.ops = engine, operands
        self._lib = load()
        self.s = torch.cuda.Stream()

    def serve(self, requests, t_start=None):
        L = self._lib
        pending = deque(requests)
        finished = []
        t0 = time.perf_counter() if t_start is None else t_start
        sp = ctypes.c_void_p(self.s.cuda_stream)
        while pending:
            r = pending.popleft()
            now = time.perf_counter() - t0
            if r.arrival > now:
                time.sleep(r.arrival - now)
            N = 1 << r.log2N
            plan = ctypes.c_void_p(self.engine.plan(r.log2N))
            fft = ctypes.c_void_p(L.cfft_u64_product_fft(plan))
            with torch.cuda.stream(self.s):
                a = r.digits.to("cuda", non_blocking=True)
                z = torch.empty((N // 2,), dtype=torch.complex128, device="cuda")
                out = torch.empty((r.nprod, N), dtype=torch.int64, device="cuda")
                for p in range(r.nprod):
                    check(L.cfft_u64_fold_twist(plan, ctypes.c_void_p(a[p].data_ptr()), B.ptr(z), 1, sp))
                    check(L.cfft_unordered_fwd(fft, B.ptr(z), 1, sp))
                    check(L.cfft_c64_pointwise(ctypes.c_void_p(self.ops.ptr(r.log2N, r.operands[p])), 0, B.ptr(z),
                                               N // 2, 1, sp))
                    check(L.cfft_unordered_inv(fft, B.ptr(z), 1, sp))
                    check(L.cfft_u64_untwist_round(plan, B.ptr(z), ctypes.c_void_p(out[p].data_ptr()), 1, sp))
                r.out = out.cpu()
            r.t_done = time.perf_counter() - t0
            finished.append(r)
        return finished


def poisson_requests(count, rate, seed, operands, log2Ns=(10, 11, 12, 13, 14), pool_per_size=32):
    """Seeded request stream: exponential inter-arrivals at `rate` req/s; each request is
    (k+1)*l products, k in {1,2}, l in {1..4}, N uniform over log2Ns, digits uniform in
    [-2^(b-1), 2^(b-1)) with b uniform in 4..10, operands drawn from the resident set."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, count))
    pools = {}
    for lN in log2Ns:
        N = 1 << lN
        b = rng.integers(4, 11, (pool_per_size, 1))
        lo = -(1 << (b - 1))
        digits = (rng.integers(0, 1 << 10, (pool_per_size, N)) % (1 << b)) + lo
        pools[lN] = torch.from_numpy(digits.astype(np.int64)).pin_memory()
    reqs = []
    for i in range(count):
        lN = int(rng.choice(log2Ns))
        nprod = (int(rng.integers(1, 3)) + 1) * int(rng.integers(1, 5))
        idx = rng.integers(0, pool_per_size, nprod)
        digits = pools[lN][torch.from_numpy(idx)].pin_memory() if nprod > 1 else pools[lN][int(idx[0]):int(idx[0]) + 1]
        ops = rng.integers(0, operands.count(lN), nprod)
        reqs.append(Request(i, float(t[i]), lN, digits, ops))
    return reqs


def latency_stats(finished):
    lat = np.array([r.t_done - r.arrival for r in finished])
    prods = sum(r.nprod for r in finished)
    span = max(r.t_done for r in finished) - min(r.arrival for r in finished)
    return {"requests": len(finished), "products": int(prods), "products_per_s": prods / span,
            "p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
            "max_ms": float(lat.max() * 1e3), "span_s": span}
