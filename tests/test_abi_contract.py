"""C-ABI contract (CPU): the header matches the reference's GPU entry points,
the library builds for sm_103a, loads, and exports every declared symbol."""
import ctypes
import json
import os
import re

import numpy as np

import pytest

from conftest import ROOT

FIXTURE = os.path.join(ROOT, "tests", "golden", "reference_gpu_abi.json")


def _norm(t):
    return t.replace("realw", "float").replace("field", "float").replace(" ", "")


def test_header_matches_reference_signatures():
    from specfem3d_gb300 import abi
    ref = json.load(open(FIXTURE))
    ours = abi.header_signatures()
    fc = {n[:-1]: a for n, (r, a) in ours.items() if n.endswith("_")}
    assert len(fc) >= 30
    for name, args in fc.items():
        assert name in ref, f"{name} is not an entry point of the reference GPU layer"
        types = [_norm(re.sub(r"\w+$", "", a)) for a in args]
        assert len(args) == len(ref[name]["types"]), name
        assert types == [_norm(t) for t in ref[name]["types"]], name


def test_hot_path_entry_points_present():
    from specfem3d_gb300 import abi
    ours = abi.header_signatures()
    for n in ["prepare_constants_device", "prepare_fields_elastic_device", "update_displacement_cuda",
              "compute_forces_viscoelastic_cuda", "compute_stacey_viscoelastic_cuda", "compute_add_sources_el_cuda",
              "kernel_3_a_cuda", "compute_seismograms_cuda", "transfer_fields_el_to_device",
              "transfer_fields_el_from_device", "prepare_cleanup_device", "compute_kernels_elastic_cuda",
              "prepare_fields_elastic_adj_dev", "add_sources_el_sim_type_2_or_3"]:
        assert n + "_" in ours, n


def test_library_builds_loads_and_exports(gpulib):
    from specfem3d_gb300 import abi, build
    path = build.lib_path()
    assert os.path.exists(path)
    for name in abi.exported_symbols():
        assert hasattr(gpulib, name), name
    assert gpulib.sf3d_version() >= 10000


def test_library_is_sm103a_only():
    # the fatbinary of the library must hold sm_103a code (cuobjdump is not used:
    # the build command line is the record); check the build flags
    from specfem3d_gb300 import build
    assert build.GENCODE == "-gencode=arch=compute_103a,code=sm_103a"


def test_error_status_without_abort(gpulib):
    """Argument validation runs before any CUDA call: an invalid NGLLX is reported
    through sf3d_last_error and the process keeps running."""
    from specfem3d_gb300 import abi
    L = gpulib
    L.sf3d_clear_error()
    A = abi.Args()
    mesh = ctypes.c_long(0)
    args = [ctypes.addressof(mesh), A.i(4)] + [A.i(0)] * 63
    L.prepare_constants_device_(*args)
    with pytest.raises(abi.SF3DError, match="NGLLX"):
        abi.check()
    assert mesh.value == 0
    L.sf3d_clear_error()


def test_null_handle_is_an_error(gpulib):
    from specfem3d_gb300 import abi
    L = gpulib
    L.sf3d_clear_error()
    A = abi.Args()
    mesh = ctypes.c_long(0)
    L.kernel_3_a_cuda_(ctypes.addressof(mesh), A.f(0.1), A.f(0.0), A.i(0), A.i(1))
    with pytest.raises(abi.SF3DError, match="not prepared"):
        abi.check()


def test_every_reference_entry_point_is_declared_and_exported(gpulib):
    """The library links into the reference program in place of its GPU layer:
    each of the entry points of the reference's stub file is declared in the
    header and exported by the library."""
    from specfem3d_gb300 import abi
    ref = json.load(open(FIXTURE))
    ours = abi.header_signatures()
    missing = [n for n in ref if n + "_" not in ours]
    assert not missing, missing
    for n in ref:
        assert hasattr(gpulib, n + "_"), n
    assert len(ref) == 124


@pytest.mark.parametrize("name,nargs", [("fault_solver_gpu_", 4), ("transfer_surface_to_host_", 2),
                                        ("compute_coupling_ocean_cuda_", 2),
                                        ("noise_read_add_surface_movie_cu_", 3)])
def test_unsupported_feature_is_an_error_status(gpulib, name, nargs):
    """Entry points of features the library does not provide return with
    SF3D_ERR_UNSUPPORTED (5) recorded and touch no argument."""
    from specfem3d_gb300 import abi
    gpulib.sf3d_clear_error()
    getattr(gpulib, name)(*([None] * nargs))
    buf = ctypes.create_string_buffer(512)
    assert gpulib.sf3d_last_error(buf, 512) == 5
    assert b"not supported" in buf.value
    gpulib.sf3d_clear_error()
    abi.check()


def test_gravity_off_and_no_damping_are_accepted(gpulib):
    from specfem3d_gb300 import abi
    A = abi.Args()
    gpulib.sf3d_clear_error()
    gpulib.prepare_fields_gravity_device_(None, A.i(0), None, None, None, None)
    gpulib.prepare_fault_device_(None, A.i(0), None)
    abi.check()
    gpulib.prepare_fields_gravity_device_(None, A.i(1), None, None, None, None)
    with pytest.raises(abi.SF3DError, match="gravity"):
        abi.check()


def test_host_vector_checks(gpulib, capfd):
    """check_error_vectors / check_max_norm_vector (check_fields_cuda.cu) reduce host
    arrays and print the result; no CUDA call."""
    from specfem3d_gb300 import abi
    A = abi.Args()
    a = np.array([1.0, -3.0, 2.0], np.float32)
    b = np.array([1.0, -1.0, 2.5], np.float32)
    gpulib.check_error_vectors_(A.i(3), A.af(a), A.af(b))
    gpulib.check_max_norm_vector_(A.i(3), A.af(a), A.i(7))
    out = capfd.readouterr().out
    assert "2.000000e+00" in out and "7: maximum norm of vector = 3.000000e+00" in out
