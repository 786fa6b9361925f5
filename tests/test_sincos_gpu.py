"""The integrator's half-angle sine and cosine (TGS integrateCoreStep, PGS
integrateCore) are evaluated in single precision from two-float Taylor sums
for |x| <= 0.125 and in double above: they equal the correctly rounded values
(numpy's double sin / cos rounded to float) and the device's double-precision
sin / cos rounded to float."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _eval(x):
    import physx_gb300
    L = physx_gb300.lib()
    L.gbpx_eval_sincos_angle.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p]
    x = np.ascontiguousarray(x, np.float32)
    out = np.zeros((len(x), 4), np.float32)
    physx_gb300.check(L.gbpx_eval_sincos_angle(x.ctypes.data, len(x), out.ctypes.data), "gbpx_eval_sincos_angle")
    return out


def test_half_angle_sincos_is_correctly_rounded(cuda_device):
    rng = np.random.default_rng(5)
    # every float in [2^-12, 0.125] spaced by 64 ulp, log-uniform samples down to
    # 2^-40, negatives, both sides of the switch to double, and the edges
    dense = (np.arange(np.float32(2.0 ** -12).view(np.int32), np.float32(0.125).view(np.int32) + 1, 64, dtype=np.int64)
             .astype(np.int32).view(np.float32))
    logs = np.exp2(rng.uniform(-40, -3, 400000)).astype(np.float32)
    edges = np.array([0.0, -0.0, 0.125, np.nextafter(np.float32(0.125), np.float32(1)), 0.2, 0.5, 1.0, 3.0, 1e-30, 1e-38], np.float32)
    x = np.concatenate([dense, logs, -logs[:100000], rng.uniform(0.12, 0.3, 50000).astype(np.float32), edges])
    out = _eval(x)
    ref_s = np.sin(x.astype(np.float64)).astype(np.float32)
    ref_c = np.cos(x.astype(np.float64)).astype(np.float32)
    # the device's double path rounded agrees with numpy's everywhere but at rare ties
    assert np.mean(out[:, 2] == ref_s) > 0.99999 and np.mean(out[:, 3] == ref_c) > 0.99999
    bad_s = np.count_nonzero(out[:, 0] != ref_s)
    bad_c = np.count_nonzero(out[:, 1] != ref_c)
    assert bad_s <= len(x) * 1e-6 and bad_c <= len(x) * 1e-6, (bad_s, bad_c, len(x))
    # and never more than one ulp away
    ulp_s = np.abs(out[:, 0].view(np.int32).astype(np.int64) - ref_s.view(np.int32).astype(np.int64))
    ulp_c = np.abs(out[:, 1].view(np.int32).astype(np.int64) - ref_c.view(np.int32).astype(np.int64))
    assert ulp_s[np.abs(x) > 1e-30].max() <= 1 and ulp_c.max() <= 1
