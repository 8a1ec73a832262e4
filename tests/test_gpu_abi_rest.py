"""The debugging norms, single-field transfers and acoustic MPI pack/assembly
entry points (check_fields_cuda.cu, transfer_fields_cuda.cu,
assemble_MPI_scalar_cuda.cu) on the GPU: round trips through the device give
back what was sent, norms equal the host maxima, and the interface buffers
hold potential_dot_dot at the interface points (pack) and add the neighbours'
contributions once per interface (assembly)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _adjoint_solver():
    from specfem3d_gb300 import adjoint as ADJ, configs, meshgen
    from specfem3d_gb300.solver import GPUSolver
    cfg = configs.small_layered(nstep=20, attenuation=True)
    db = meshgen.build_database(cfg)
    g = GPUSolver(db, cfg, simulation_type=3)
    ADJ._prepare_adjoint(g, db, cfg["nstep"])
    return g


def test_backward_field_transfers_and_norms(gpulib, capfd):
    from specfem3d_gb300 import abi
    L = gpulib
    g = _adjoint_solver()
    A = abi.Args()
    n3 = 3 * g.nglob
    rng = np.random.default_rng(5)
    d, v, a = (rng.standard_normal(n3).astype(np.float32) for _ in range(3))
    L.transfer_b_fields_to_device_(A.i(n3), A.af(d), A.af(v), A.af(a), g.mp)
    out = np.zeros(n3, np.float32)
    L.transfer_b_accel_from_device_(A.i(n3), out.ctypes.data, g.mp)
    assert np.array_equal(out, a)
    L.transfer_b_veloc_from_device_(A.i(n3), out.ctypes.data, g.mp)
    assert np.array_equal(out, v)
    a2, v2 = 2 * a, 3 * v
    L.transfer_b_accel_to_device_(A.i(n3), A.af(a2), g.mp)
    L.transfer_b_veloc_to_device_(A.i(n3), A.af(v2), g.mp)
    bd, bv, ba = (np.zeros(n3, np.float32) for _ in range(3))
    L.transfer_b_fields_from_device_(A.i(n3), bd.ctypes.data, bv.ctypes.data, ba.ctypes.data, g.mp)
    assert np.array_equal(bd, d) and np.array_equal(bv, v2) and np.array_equal(ba, a2)
    abi.check()
    # norms of the device fields
    fd = rng.standard_normal(n3).astype(np.float32)
    g.set_fields(fd, np.zeros(n3, np.float32), 5 * fd)
    norm = np.zeros(1, np.float32)
    L.get_norm_elastic_from_device_(norm.ctypes.data, g.mp, A.i(1))
    assert norm[0] == np.abs(fd).max()
    L.get_norm_elastic_from_device_(norm.ctypes.data, g.mp, A.i(3))
    assert norm[0] == np.abs(d).max()
    L.check_max_norm_b_veloc_gpu_(A.i(n3), out.ctypes.data, g.mp, A.i(4))
    L.get_max_accel_(A.i(9), A.i(n3), g.mp)
    abi.check()
    txt = capfd.readouterr().out
    assert f"{np.abs(v2).max():e}" in txt and f"{5 * np.abs(fd).max():e}" in txt
    free, used, total = (np.zeros(1, np.float32) for _ in range(3))
    L.get_free_device_memory_(free.ctypes.data, used.ctypes.data, total.ctypes.data)
    assert total[0] > 1000 and 0 < used[0] < total[0]
    # a wrong size is an error, nothing is copied
    L.transfer_b_accel_from_device_(A.i(n3 - 3), out.ctypes.data, g.mp)
    with pytest.raises(abi.SF3DError, match="NDIM"):
        abi.check()
    g.close()


def test_backward_strain_and_memory_variable_uploads(gpulib):
    """transfer_b_strain_to_device takes the host layout (5,5,5,NSPEC): the strain
    comes back through transfer_compute_kernel_fields_from_device.  The layout
    (N_SLS,5,5,5,NSPEC) of transfer_b_rmemory_to_device is checked by the
    undo-attenuation restart (a snapshot's memory variables continue the forward
    trajectory); here its size check."""
    from specfem3d_gb300 import abi
    from specfem3d_gb300.solver import N_SLS
    L = gpulib
    g = _adjoint_solver()
    A = abi.Args()
    ne = 125 * g.nspec
    rng = np.random.default_rng(7)
    eps = [rng.standard_normal(ne).astype(np.float32) for _ in range(6)]
    L.transfer_b_strain_to_device_(g.mp, *(A.af(e) for e in eps), A.i(ne))
    abi.check()
    n3 = 3 * g.nglob
    acc, bdis = np.zeros(n3, np.float32), np.zeros(n3, np.float32)
    fe = [np.zeros(ne, np.float32) for _ in range(5)]
    be = [np.zeros(ne, np.float32) for _ in range(5)]
    kl = [np.zeros(ne, np.float32) for _ in range(3)]
    tr, btr = np.zeros(ne, np.float32), np.zeros(ne, np.float32)
    L.transfer_compute_kernel_fields_from_device_(
        g.mp, acc.ctypes.data, A.i(n3), bdis.ctypes.data, A.i(n3), *(x.ctypes.data for x in fe), A.i(ne),
        *(x.ctypes.data for x in be), A.i(ne), kl[0].ctypes.data, A.i(ne), kl[1].ctypes.data, A.i(ne),
        kl[2].ctypes.data, A.i(ne), tr.ctypes.data, btr.ctypes.data, A.i(ne))
    abi.check()
    for c in range(5):
        assert np.array_equal(be[c], eps[c]), c
    assert all(not k.any() for k in kl)
    # the memory variables
    nR = N_SLS * ne
    R = [rng.standard_normal(nR).astype(np.float32) for _ in range(6)]
    L.transfer_b_rmemory_to_device_(g.mp, *(A.af(r) for r in R), A.i(nR))
    abi.check()
    L.transfer_b_rmemory_to_device_(g.mp, *(A.af(r) for r in R), A.i(nR - 1))
    with pytest.raises(abi.SF3DError, match="size_R"):
        abi.check()
    g.close()


def test_acoustic_interfaces_and_potential_transfers(gpulib):
    from specfem3d_gb300 import abi, configs, meshgen
    from specfem3d_gb300.solver import GPUSolver
    L = gpulib
    cfg = configs.small_coupled(nstep=10)
    db = dict(meshgen.build_database(cfg))
    nglob = int(db["nglob"])
    rng = np.random.default_rng(11)
    # two synthetic interfaces, 1-based points, (max_nibool, num_interfaces) in Fortran order
    mxn, nib = 9, np.array([9, 6], np.int32)
    ibif = np.zeros((mxn, 2), np.int32)
    ibif[:, 0] = rng.choice(nglob, mxn, replace=False) + 1
    ibif[:6, 1] = np.concatenate([ibif[:3, 0], rng.choice(nglob, 3, replace=False) + 1])
    db.update(num_interfaces=2, max_nibool_interfaces=mxn, nibool_interfaces=nib,
              ibool_interfaces=ibif.reshape(-1, order="F"))
    g = GPUSolver(db, cfg)
    A = abi.Args()
    pdd = rng.standard_normal(nglob).astype(np.float32)
    L.transfer_dot_dot_to_device_(A.i(nglob), A.af(pdd), g.mp)
    back = np.zeros(nglob, np.float32)
    L.transfer_dot_dot_from_device_(A.i(nglob), back.ctypes.data, g.mp)
    assert np.array_equal(back, pdd)
    L.transfer_potential_ac_from_device_(A.i(nglob), back.ctypes.data, g.mp)
    assert np.array_equal(back, g.potentials()[0])
    norm = np.zeros(1, np.float32)
    L.get_norm_acoustic_from_device_(norm.ctypes.data, g.mp, A.i(1))
    assert norm[0] == np.abs(pdd).max()
    abi.check()
    send = np.zeros((2, mxn), np.float32)
    L.transfer_boun_pot_from_device_(g.mp, send.ctypes.data, A.i(1))
    abi.check()
    for i in range(2):
        assert np.array_equal(send[i, :nib[i]], pdd[ibif[:nib[i], i] - 1])
    recv = rng.standard_normal((2, mxn)).astype(np.float32)
    L.transfer_asmbl_pot_to_device_(g.mp, recv.ctypes.data, A.i(1))
    abi.check()
    want = pdd.astype(np.float64)
    for i in range(2):
        np.add.at(want, ibif[:nib[i], i] - 1, recv[i, :nib[i]])
    L.transfer_dot_dot_from_device_(A.i(nglob), back.ctypes.data, g.mp)
    assert np.allclose(back, want, rtol=0, atol=1e-6)
    # the backward potentials exist only after prepare_fields_acoustic_adj_dev
    L.transfer_boun_pot_from_device_(g.mp, send.ctypes.data, A.i(3))
    with pytest.raises(abi.SF3DError, match="not prepared"):
        abi.check()
    g.close()
