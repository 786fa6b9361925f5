"""gbpx_generate_contacts_device_noalloc: the narrowphase over caller-owned device
arrays with a fixed device scratch array (no allocation inside the call),
against the allocating host entry point gbpx_generate_contacts, two calls in a
row (the shared scratch is reused), plus the size limit."""
import ctypes

import numpy as np
import pytest

from scenarios import np_pairs

pytestmark = pytest.mark.gpu

MAX_PAIRS = 262144


def _noalloc():
    from physx_gb300 import lib
    L = lib()
    f = L.gbpx_generate_contacts_device_noalloc
    f.argtypes = [ctypes.c_void_p] * 6 + [ctypes.c_uint32, ctypes.c_float, ctypes.c_float, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f


def _run_device(pairs, cd=0.04, tl=1.0):
    import torch
    f = _noalloc()
    dev = torch.device("cuda:0")
    keys = ("type0", "geom0", "type1", "geom1", "pose0", "pose1")
    dts = (np.int32, np.float32, np.int32, np.float32, np.float32, np.float32)
    ins = [torch.from_numpy(np.ascontiguousarray(pairs[k], d)).to(dev) for k, d in zip(keys, dts)]
    n = len(pairs["type0"])
    out = torch.zeros((n, 4, 8), dtype=torch.float32, device=dev)
    cnt = torch.zeros(n, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream()
    rc = f(*[t.data_ptr() for t in ins], n, cd, tl, out.data_ptr(), cnt.data_ptr(), ctypes.c_void_p(stream.cuda_stream))
    assert rc == 0, rc
    stream.synchronize()
    return cnt.cpu().numpy().astype(np.uint32), out.cpu().numpy()


def test_noalloc_matches_allocating_entry_point_twice(cuda_device):
    from physx_gb300.contacts import generate_contacts
    for seed, n in ((91, 3000), (92, 5000)):
        pairs = np_pairs(seed, n)
        ref_cnt, ref_out = generate_contacts(pairs, max_per_pair=4)
        cnt, out = _run_device(pairs)
        assert np.array_equal(cnt, ref_cnt)
        for i in np.flatnonzero(ref_cnt):
            assert np.abs(out[i, :ref_cnt[i]] - ref_out[i, :ref_cnt[i]]).max() <= 1e-6


def test_noalloc_rejects_batches_above_scratch_capacity(cuda_device):
    f = _noalloc()
    fake = ctypes.c_void_p(256)   # never dereferenced: the size check comes first
    rc = f(fake, fake, fake, fake, fake, fake, MAX_PAIRS + 1, 0.04, 1.0, fake, fake, None)
    assert rc == -3   # GBPX_ERR_CAPACITY
