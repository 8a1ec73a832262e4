"""sf3d_field_maxabs_noalloc: the max-norm reduction of sf3d_check_stability with
its scratch memory in a fixed device array (no allocation in any call).

Collected last (file name), so it runs both alone and after every other GPU
test in the same process.  Two calls in a row on the same field give exactly
the maximum that sf3d_check_stability reports (a maximum does not depend on the
reduction order); NaN is reported as NaN; sizes beyond the fixed scratch are
rejected with an argument error."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(L, ptr, n):
    m = ctypes.c_float(-1.0)
    rc = L.sf3d_field_maxabs_noalloc(ctypes.c_void_p(ptr), ctypes.c_long(n), None, ctypes.byref(m))
    return rc, m.value


def test_noalloc_maxabs_matches_check_stability(gpulib):
    from specfem3d_gb300 import abi, configs, meshgen
    from specfem3d_gb300.solver import GPUSolver
    L = abi.load()
    L.sf3d_field_maxabs_noalloc.restype = ctypes.c_int
    L.sf3d_field_maxabs_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_long, ctypes.c_void_p,
                                            ctypes.POINTER(ctypes.c_float)]
    cfg = configs.small_layered(nx=7, ny=6, counts=(2, 2, 3), nstep=4, attenuation=False)
    db = meshgen.build_database(cfg)
    g = GPUSolver(db, cfg)
    n = 3 * int(db["nglob"])
    rng = np.random.default_rng(3)
    d = rng.standard_normal(n).astype(np.float32)
    d[12345 % n] = -7.25
    g.set_fields(d, np.zeros(n, np.float32), np.zeros(n, np.float32))
    ptr = L.sf3d_device_ptr(g.mp, b"displ")
    assert ptr
    rc0, ref = g.check_stability(1e30)
    assert rc0 == 0 and ref == 7.25
    for _ in range(2):
        rc, m = _noalloc(L, ptr, n)
        assert rc == 0 and m == ref
    # a prefix of the field: the maximum of that prefix
    rc, m = _noalloc(L, ptr, 1000)
    assert rc == 0 and m == np.abs(d[:1000]).max()
    # NaN propagates
    d[n // 2] = np.nan
    g.set_fields(d, np.zeros(n, np.float32), np.zeros(n, np.float32))
    rc, m = _noalloc(L, ptr, n)
    assert rc == 0 and np.isnan(m)
    # beyond the fixed scratch: rejected before any launch
    rc, _ = _noalloc(L, ptr, 536854528 + 1)
    assert rc == 1
    with pytest.raises(abi.SF3DError, match="256 KB scratch"):
        abi.check()
    g.close()


def test_noalloc_maxabs_many_blocks_and_at_the_limit(gpulib):
    """Device buffers of 6,000,000 values (367 partials: the final pass strides over
    more than 256 of them) and of exactly the documented maximum, 536,854,528 values
    (2.1 GB, 32,767 partials); the maximum equals the buffer's true max |x|, twice in
    a row, and a NaN in the last block of the large buffer is reported as NaN."""
    torch = pytest.importorskip("torch")
    from specfem3d_gb300 import abi
    L = abi.load()
    L.sf3d_field_maxabs_noalloc.restype = ctypes.c_int
    L.sf3d_field_maxabs_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_long, ctypes.c_void_p,
                                            ctypes.POINTER(ctypes.c_float)]
    torch.cuda.synchronize()
    gen = torch.Generator(device="cuda").manual_seed(11)
    for n, spot in ((6_000_000, 5_999_001), (536_854_528, 536_854_000)):
        x = torch.randn(n, device="cuda", generator=gen)
        x[spot] = -123.5                       # the maximum sits in the last partial
        torch.cuda.synchronize()
        ref = float(x.abs().max().item())
        assert ref == 123.5
        for _ in range(2):
            rc, m = _noalloc(L, x.data_ptr(), n)
            assert rc == 0 and m == ref
        x[spot] = float("nan")
        torch.cuda.synchronize()
        rc, m = _noalloc(L, x.data_ptr(), n)
        assert rc == 0 and np.isnan(m)
        del x
        torch.cuda.empty_cache()
