"""Negacyclic-product serving: the mixed-size product engine and the native
continuous-batching request loop (cfft_product_engine_* / cfft_server_* of
include/cfft.h)."""
import ctypes

import numpy as np

from . import _buffers as B
from ._lib import check, load

ITEM_DTYPE = np.dtype([("a", np.uint64), ("bhat", np.uint64), ("out", np.uint64), ("log2N", np.uint32),
                       ("reserved", np.uint32)])


class ProductEngine:
    """One persistent launch over products of any configured N (2^6..2^17)."""

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
        """Handle of the engine's cfft_u64_product_plan for size 2^log2N."""
        return ctypes.c_void_p(self._lib.cfft_product_engine_plan(self._h, log2N))

    def algo(self, log2N):
        a, b = ctypes.c_int(), ctypes.c_size_t()
        self._lib.cfft_u64_product_algo(self.plan(log2N), ctypes.byref(a), ctypes.byref(b))
        return a.value, b.value

    def prepare_operand(self, log2N, b, bhat):
        """b: int64 device tensor (count, N) -> bhat: complex128 device tensor (count, N/2)."""
        count = B.batch_of(b, 1 << log2N, 8)
        check(self._lib.cfft_u64_prepare_operand(self.plan(log2N), B.ptr(b), B.ptr(bhat), count, B.stream_of(b)))
        return bhat

    def run(self, items_dev, count, counter, workspace, stream):
        """items_dev: device tensor holding `count` ITEM_DTYPE records; counter: device int32 tensor."""
        ws = ctypes.c_void_p(workspace.data_ptr()) if workspace is not None else None
        check(self._lib.cfft_product_engine_run(self._h, ctypes.c_void_p(items_dev.data_ptr()), count,
                                                ctypes.c_void_p(counter.data_ptr()), ws, ctypes.c_void_p(stream)))

    def run_static(self, items_dev, count, stream):
        """The no-allocation run: counter and workspace from the library's static device array
        (largest N 16384; calls that overlap on the GPU race, so serialise them)."""
        check(self._lib.cfft_product_engine_run_static(self._h, ctypes.c_void_p(items_dev.data_ptr()), count,
                                                       ctypes.c_void_p(stream)))


class QueueConfig(ctypes.Structure):
    _fields_ = [("max_inflight", ctypes.c_uint32), ("cluster_log2N", ctypes.c_uint32)]


class ProductQueue:
    """The engine behind a work queue: submit groups of products from any thread, then poll or
    wait on the returned ticket.  Item buffers are device tensors or page-locked host tensors."""

    def __init__(self, engine, max_inflight=0, cluster_log2N=0):
        self._lib = load()
        self.engine = engine  # keep the engine alive
        h = ctypes.c_void_p()
        cfg = QueueConfig(max_inflight, cluster_log2N)
        check(self._lib.cfft_product_queue_create(engine._h, ctypes.byref(cfg), ctypes.byref(h)))
        self._h = h

    def close(self):
        """Runs everything submitted, then releases the queue."""
        if getattr(self, "_h", None):
            self._lib.cfft_product_queue_destroy(self._h)
            self._h = None

    __del__ = close

    def submit(self, items):
        """items: numpy array of ITEM_DTYPE records (a, bhat, out addresses, log2N); returns a ticket."""
        arr = np.ascontiguousarray(items, dtype=ITEM_DTYPE)
        t = ctypes.c_uint64()
        check(self._lib.cfft_product_queue_submit(self._h, ctypes.c_void_p(arr.ctypes.data), len(arr),
                                                  ctypes.byref(t)))
        return t.value

    def poll(self, ticket):
        """True when the ticket's products are complete (raises if its launch failed)."""
        r = self._lib.cfft_product_queue_poll(self._h, ticket)
        if r < 0:
            check(r)
        return r == 1

    def wait(self, ticket):
        check(self._lib.cfft_product_queue_wait(self._h, ticket))


class ServeConfig(ctypes.Structure):
    _fields_ = [("rate", ctypes.c_double), ("duration_s", ctypes.c_double), ("log2N_min", ctypes.c_uint32),
                ("log2N_max", ctypes.c_uint32), ("k_max", ctypes.c_uint32), ("l_max", ctypes.c_uint32),
                ("plain", ctypes.c_uint32), ("max_inflight", ctypes.c_uint32), ("record_every", ctypes.c_uint32),
                ("cluster_log2N", ctypes.c_uint32), ("staged_io", ctypes.c_uint32), ("via_queue", ctypes.c_uint32),
                ("mem_reserve_bytes", ctypes.c_uint64), ("mem_free_override", ctypes.c_uint64)]


class ServeStats(ctypes.Structure):
    _fields_ = [("requests", ctypes.c_uint64), ("products", ctypes.c_uint64), ("launches", ctypes.c_uint64),
                ("deferred_admissions", ctypes.c_uint64), ("products_per_s", ctypes.c_double),
                ("p50_ms", ctypes.c_double), ("p99_ms", ctypes.c_double), ("max_ms", ctypes.c_double),
                ("mean_batch", ctypes.c_double), ("span_s", ctypes.c_double),
                ("memory_deferrals", ctypes.c_uint64), ("input_bytes", ctypes.c_uint64),
                ("output_bytes", ctypes.c_uint64), ("min_memory_budget_mib", ctypes.c_double)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class Server:
    """Resident digit pools and Fourier operands plus the request loop."""

    def __init__(self, engine, log2Ns, operand_bytes, ring_bytes=0, seed=0):
        self._lib = load()
        self.engine = engine  # keep the engine alive
        arr = (ctypes.c_uint32 * len(log2Ns))(*log2Ns)
        h = ctypes.c_void_p()
        check(self._lib.cfft_server_create(engine._h, arr, len(log2Ns), int(operand_bytes), int(ring_bytes),
                                           int(seed), ctypes.byref(h)))
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.cfft_server_destroy(self._h)
            self._h = None

    @staticmethod
    def config(rate, duration_s, log2N_min=10, log2N_max=14, k_max=2, l_max=4, plain=False, max_inflight=3,
               record_every=0, cluster_log2N=0, staged_io=False, via_queue=False, mem_reserve_bytes=0,
               mem_free_override=0):
        """mem_reserve_bytes: device memory the admission gate leaves free; mem_free_override: a
        stand-in for the device's free bytes (tests fake a small device with it)."""
        return ServeConfig(rate, duration_s, log2N_min, log2N_max, k_max, l_max, int(plain), max_inflight,
                           record_every, cluster_log2N, int(staged_io), int(via_queue), int(mem_reserve_bytes),
                           int(mem_free_override))

    def run(self, cfg):
        st = ServeStats()
        check(self._lib.cfft_server_run(self._h, ctypes.byref(cfg), ctypes.byref(st)))
        return st.as_dict()

    def recorded_ids(self):
        n = self._lib.cfft_server_recorded(self._h)
        ids = np.zeros(n, dtype=np.uint64)
        if n:
            check(self._lib.cfft_server_recorded_ids(self._h, ctypes.c_void_p(ids.ctypes.data), n))
        return ids

    def shape(self, cfg, rid):
        lN, npd = ctypes.c_uint32(), ctypes.c_uint32()
        check(self._lib.cfft_server_request_shape(self._h, ctypes.byref(cfg), int(rid), ctypes.byref(lN),
                                                  ctypes.byref(npd)))
        return lN.value, npd.value

    def recorded_output(self, cfg, rid):
        lN, npd = self.shape(cfg, rid)
        out = np.zeros((npd, 1 << lN), dtype=np.uint64)
        check(self._lib.cfft_server_recorded_output(self._h, int(rid), ctypes.c_void_p(out.ctypes.data), out.size))
        return out

    def run_alone(self, cfg, rid):
        lN, npd = self.shape(cfg, rid)
        out = np.zeros((npd, 1 << lN), dtype=np.uint64)
        check(self._lib.cfft_server_run_alone(self._h, ctypes.byref(cfg), int(rid), ctypes.c_void_p(out.ctypes.data),
                                              out.size))
        return out

    def inputs(self, cfg, rid):
        lN, npd = self.shape(cfg, rid)
        N = 1 << lN
        digits = np.zeros((npd, N), dtype=np.int64)
        bhat = np.zeros((npd, N // 2), dtype=np.complex128)
        check(self._lib.cfft_server_request_inputs(self._h, ctypes.byref(cfg), int(rid),
                                                   ctypes.c_void_p(digits.ctypes.data),
                                                   ctypes.c_void_p(bhat.ctypes.data)))
        return digits, bhat
