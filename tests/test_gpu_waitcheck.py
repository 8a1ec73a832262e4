"""The bounded mbarrier wait that guards the bulk copies of the stiffness, C-PML
and adjoint kernels gives up after its limit, records the kernel error word and
returns, leaving the context usable (sf3d_check_bounded_wait: a wait on an
mbarrier whose announced bytes no copy delivers; nothing faults, nothing spins
without bound, no copy is in flight).  After it, a stiffness run with the
bulk-copy build still matches the oracle."""
import ctypes
import os

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def test_bounded_wait_times_out_and_reports(gpulib):
    from specfem3d_gb300 import abi
    L = abi.load()
    flag = ctypes.c_int(0)
    waited = ctypes.c_double(0.0)
    assert L.sf3d_check_bounded_wait(0.2, ctypes.addressof(flag), ctypes.addressof(waited)) == 0
    assert flag.value == 1
    assert 0.2 <= waited.value < 2.0, waited.value
    # a limit outside (0, 2] s is refused on the host, and reported
    assert L.sf3d_check_bounded_wait(5.0, ctypes.addressof(flag), None) != 0
    with pytest.raises(abi.SF3DError, match="limit"):
        abi.check()


def test_context_usable_after_the_timeout(gpulib):
    from oracle import oracle as O
    from specfem3d_gb300 import abi, configs, meshgen
    from specfem3d_gb300.solver import GPUSolver
    L = abi.load()
    flag = ctypes.c_int(0)
    assert L.sf3d_check_bounded_wait(0.05, ctypes.addressof(flag), None) == 0 and flag.value == 1
    cfg = configs.small_layered(nstep=4, attenuation=True)
    db = meshgen.build_database(cfg)
    rng = np.random.default_rng(3)
    n3 = 3 * db["nglob"]
    d = rng.standard_normal(n3).astype(np.float32) * 1e-3
    v = rng.standard_normal(n3).astype(np.float32) * 1e-2
    g = GPUSolver(db, cfg)
    g.set_stiffness_variant(14)          # memory variables by bulk copy, bounded waits
    g.set_fields(d, v, np.zeros(n3, np.float32))
    g.forces_only()
    acc = g.fields()[2]
    g.close()
    sim = O.make_sim(db, cfg, "f32", nthreads=os.cpu_count() or 1)
    sim.get("displ")[:] = d
    sim.get("veloc")[:] = v
    sim.forces()
    assert rel_l2(acc, sim.get("accel")) < 2e-6
