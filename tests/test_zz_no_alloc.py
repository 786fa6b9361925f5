"""gbpx_generate_contacts_device_noalloc: the narrowphase over caller-owned device
arrays for callers that cannot allocate device memory during a call, with its
bucketing scratch in a fixed device array.

Checked against the allocating host entry point gbpx_generate_contacts and the
CPU oracle on two calls in a row (the shared scratch is reused), on a stream of
the caller's own, with the free device memory unchanged across calls of
different sizes, and the size limit.  This file sorts last so that a run that
stops at the first failure has run every other test first."""
import ctypes

import numpy as np
import pytest

from oracle_libs import run_contacts
from scenarios import np_pairs

pytestmark = pytest.mark.gpu

MAX_PAIRS = 262144
TOL = 1e-6   # device contacts against the host entry point and the oracle (the other contact tests' bar)
KEYS = ("type0", "geom0", "type1", "geom1", "pose0", "pose1")
DTYPES = (np.int32, np.float32, np.int32, np.float32, np.float32, np.float32)


def _noalloc():
    from physx_gb300 import lib
    L = lib()
    f = L.gbpx_generate_contacts_device_noalloc
    f.argtypes = [ctypes.c_void_p] * 6 + [ctypes.c_uint32, ctypes.c_float, ctypes.c_float, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f


class DeviceBatch:
    """One batch of pairs and its output arrays, all on the device (allocated by the test, not by the call)."""

    def __init__(self, pairs):
        import torch
        dev = torch.device("cuda:0")
        self.ins = [torch.from_numpy(np.ascontiguousarray(pairs[k], d)).to(dev) for k, d in zip(KEYS, DTYPES)]
        self.n = len(pairs["type0"])
        self.out = torch.zeros((self.n, 4, 8), dtype=torch.float32, device=dev)
        self.cnt = torch.zeros(self.n, dtype=torch.int32, device=dev)

    def launch(self, stream, cd=0.04, tl=1.0):
        rc = _noalloc()(*[t.data_ptr() for t in self.ins], self.n, cd, tl, self.out.data_ptr(), self.cnt.data_ptr(),
                        ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0, rc

    def result(self):
        return self.cnt.cpu().numpy().astype(np.uint32), self.out.cpu().numpy()


def _run_device(pairs, stream=None):
    import torch
    b = DeviceBatch(pairs)
    s = stream or torch.cuda.current_stream()
    b.launch(s)
    s.synchronize()
    return b.result()


def _same(cnt, out, ref_cnt, ref_out):
    assert np.array_equal(cnt, ref_cnt)
    for i in np.flatnonzero(ref_cnt):
        assert np.abs(out[i, :ref_cnt[i], :7] - ref_out[i, :ref_cnt[i], :7]).max() <= TOL


def test_noalloc_matches_allocating_entry_point_and_oracle_twice(cuda_device):
    from physx_gb300.contacts import generate_contacts
    for seed, n in ((91, 3000), (92, 5000)):
        pairs = np_pairs(seed, n)
        ref_cnt, ref_out = generate_contacts(pairs, max_per_pair=4)
        orc_cnt, orc_out = run_contacts("orc", pairs, max_per_pair=4)
        cnt, out = _run_device(pairs)
        _same(cnt, out, ref_cnt, ref_out)
        _same(cnt, out, orc_cnt, orc_out)


def test_noalloc_convex_core_pairs(cuda_device):
    """Primitive and convex-core pairs in one device batch: the host does not know
    the split, both generators cover the batch and skip each other's pairs."""
    from physx_gb300.workloads import convex_core_pairs
    a, b = np_pairs(93, 2000), convex_core_pairs(94, 2000)
    order = np.random.default_rng(95).permutation(4000)
    pairs = {k: np.concatenate([a[k], b[k]])[order] for k in a}
    orc_cnt, orc_out = run_contacts("orc", pairs, max_per_pair=4)
    cnt, out = _run_device(pairs)
    _same(cnt, out, orc_cnt, orc_out)


def test_noalloc_on_a_caller_stream(cuda_device):
    import torch
    pairs = np_pairs(93, 4000)
    orc_cnt, orc_out = run_contacts("orc", pairs, max_per_pair=4)
    side = torch.cuda.Stream()
    cnt, out = _run_device(pairs, stream=side)
    _same(cnt, out, orc_cnt, orc_out)


def test_noalloc_calls_leave_free_device_memory_unchanged(cuda_device):
    import torch
    batches = [DeviceBatch(np_pairs(94 + k, n)) for k, n in enumerate((1000, 7000, 20000, 300))]
    s = torch.cuda.current_stream()
    batches[0].launch(s)   # the first call on the device looks up the scratch address; kernels load
    s.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(2):
        for b in batches:
            b.launch(s)
    s.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, "the call changed free device memory by %d bytes" % (free0 - free1)
    cnt, out = batches[2].result()
    orc_cnt, orc_out = run_contacts("orc", np_pairs(96, 20000), max_per_pair=4)
    _same(cnt, out, orc_cnt, orc_out)


def test_noalloc_rejects_batches_above_scratch_capacity(cuda_device):
    f = _noalloc()
    fake = ctypes.c_void_p(256)   # never dereferenced: the size check comes first
    rc = f(fake, fake, fake, fake, fake, fake, MAX_PAIRS + 1, 0.04, 1.0, fake, fake, None)
    assert rc == -3   # GBPX_ERR_CAPACITY
