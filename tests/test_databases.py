"""proc######_external_mesh.bin / attenuation.bin (specfem3d_gb300.databases): the
Fortran record layer, and write -> read -> solver set-up round trips that must
give back every array the time loop takes, bit for bit (FP32; source and
receiver interpolants to 1e-5, as the files hold the mesh coordinates in
single precision), for a layered
viscoelastic block with Stacey faces, a fluid-over-solid block, a block of
regular elements (empty metric records) and one slice of a partitioned mesh
(MPI interfaces, outer/inner phases)."""
import os

import numpy as np
import pytest

import partition_block

KEYS_INT = ["ibool", "irregular_element_number", "ispec_is_acoustic", "abs_boundary_ispec", "abs_boundary_ijk",
            "free_surface_ispec", "free_surface_ijk", "coupling_ac_el_ispec", "coupling_ac_el_ijk",
            "ispec_selected_source"]
KEYS_REAL = ["xix", "xiy", "xiz", "etax", "etay", "etaz", "gammax", "gammay", "gammaz", "jacobian", "rhostore",
             "kappastore", "mustore", "rho_vp", "rho_vs", "rmassx", "rmassy", "rmassz", "rmass_acoustic",
             "abs_boundary_jacobian2Dw", "abs_boundary_normal", "coupling_ac_el_jacobian2Dw", "coupling_ac_el_normal",
             "sourcearrays", "stf", "factor_common", "factor_common_kappa", "alphaval", "betaval", "gammaval"]


def _receiver_positions(db, xyz):
    """Physical positions the receivers' elements and interpolants point at (a
    receiver on a face shared by two elements may be placed in either of them)."""
    ib = np.asarray(db["ibool"]).reshape(-1, 125) - 1
    out = []
    for r, e in enumerate(np.asarray(db["ispec_selected_rec"]) - 1):
        h = [np.asarray(db[k]).reshape(-1, 5)[r] for k in ("hxir", "hetar", "hgammar")]
        w = (h[2][:, None, None] * h[1][None, :, None] * h[0][None, None, :]).reshape(-1)
        out.append(w @ xyz[ib[e]])
    return np.asarray(out)


def _roundtrip(tmp_path, db, cfg, xyz, att):
    from specfem3d_gb300 import databases as D
    p = os.path.join(tmp_path, "proc000000_external_mesh.bin")
    D.write_external_mesh(p, db, xyz)
    a = None
    if att:
        pa = os.path.join(tmp_path, "proc000000_attenuation.bin")
        D.write_attenuation(pa, db)
        a = D.read_attenuation(pa, db["nspec"])
    raw = D.read_external_mesh(p, stacey=bool(db.get("stacey", 0)))
    return raw, D.solver_database(raw, cfg, a)


def _same(a, b):
    for k in ("nspec", "nglob", "nspec_irregular", "num_abs_boundary_faces", "num_free_surface_faces",
              "num_coupling_ac_el_faces", "stacey", "attenuation"):
        assert int(a.get(k, 0)) == int(b.get(k, 0)), k
    assert np.float32(a["xix_regular"]) == np.float32(b["xix_regular"])
    for k in KEYS_INT:
        if k in b:
            assert np.array_equal(np.asarray(a[k]).reshape(-1), np.asarray(b[k]).reshape(-1)), k
    for k in KEYS_REAL:
        if k in b:
            x, y = np.asarray(a[k]).reshape(-1), np.asarray(b[k]).reshape(-1)
            if k in ("sourcearrays", "hxir", "hetar", "hgammar", "stf"):
                # the files keep the point coordinates in CUSTOM_REAL, so the
                # located local coordinates move by float32 rounding of the mesh
                assert np.abs(x - y).max() <= 1e-5 * np.abs(y).max(), k
            else:
                assert np.array_equal(x.astype(np.float32), y.astype(np.float32)), k


@pytest.mark.parametrize("case", ["layered_att", "coupled", "regular"])
def test_database_roundtrip(tmp_path, case):
    from specfem3d_gb300 import configs, meshgen
    if case == "layered_att":
        cfg = configs.small_layered(nstep=20, attenuation=True)
    elif case == "coupled":
        cfg = configs.small_coupled(nstep=20)
    else:
        cfg = configs.small_adjoint(nstep=20, nshots=1, n=6)      # 312.5 m cubes
    db = meshgen.build_database(cfg)
    if case == "regular":
        assert db["nspec_irregular"] == 0
    from specfem3d_gb300 import databases as D
    xyz = D.global_coordinates(db["ibool"], meshgen.element_coordinates(cfg), db["nglob"])
    raw, back = _roundtrip(str(tmp_path), db, cfg, xyz, case == "layered_att")
    assert np.allclose(np.stack([raw["xstore"], raw["ystore"], raw["zstore"]], 1), xyz.astype(np.float32))
    _same(back, db)
    span = float(np.abs(xyz).max())
    assert np.abs(_receiver_positions(back, xyz) - _receiver_positions(db, xyz)).max() <= 1e-6 * span


def test_partition_slice_roundtrip(tmp_path):
    """A slice of a 3-way partitioned block keeps its MPI interfaces and its
    outer-element phase list through the files."""
    from specfem3d_gb300 import configs, meshgen, databases as D
    cfg = configs.small_layered(nstep=20, attenuation=False)
    db = meshgen.build_database(cfg)
    parts = partition_block.split_x(db, cfg, 3)
    d = parts[1]
    gl = np.asarray(d["global_points"]) - 1
    for c in "xyz":
        d["rmass" + c + "_stacey"] = db["rmass" + c + "_stacey"][gl]
    d["num_free_surface_faces"] = 0              # the slicer keeps only what the elastic step uses
    xyz = D.global_coordinates(db["ibool"], meshgen.element_coordinates(cfg), db["nglob"])[gl]
    p = os.path.join(str(tmp_path), "proc000001_external_mesh.bin")
    D.write_external_mesh(p, d, xyz)
    raw = D.read_external_mesh(p, stacey=True)
    assert raw["num_interfaces"] == d["num_interfaces"]
    assert np.array_equal(raw["nibool_interfaces"], np.asarray(d["nibool_interfaces"]))
    assert np.array_equal(raw["ibool_interfaces"], np.asarray(d["ibool_interfaces"]).reshape(-1))
    outer = raw["phase_ispec_inner_elastic"][:raw["nspec_outer_elastic"], 0]
    assert np.array_equal(np.sort(outer), np.sort(np.asarray(d["phase_outer"])))
    assert not raw["ispec_is_inner"][np.asarray(d["phase_outer"]) - 1].any()


def test_record_layer_subrecords(tmp_path, monkeypatch):
    """Records longer than the subrecord limit are split gfortran-style (leading
    marker negative while more follow, trailing marker negative after the first)
    and read back whole."""
    from specfem3d_gb300 import databases as D
    monkeypatch.setattr(D, "_MAX_SUB", 40)
    p = os.path.join(str(tmp_path), "r.bin")
    w = D.RecordWriter(p)
    a = np.arange(25, dtype=np.int32)          # 100 bytes: subrecords of 40, 40, 20
    w.write(a)
    w.write(np.array([7], np.int32))
    w.close()
    raw = open(p, "rb").read()
    marks = np.frombuffer(raw[:4], np.int32)[0], np.frombuffer(raw[44:48], np.int32)[0]
    assert marks == (-40, 40)
    r = D.RecordReader(p)
    assert np.array_equal(r.ints(), a)
    assert r.int() == 7
    with pytest.raises(EOFError):
        r.raw()
    r.close()


def test_reader_rejects_wrong_check_values(tmp_path):
    from specfem3d_gb300 import configs, meshgen, databases as D
    cfg = configs.small_layered(nstep=5, attenuation=False)
    db = meshgen.build_database(cfg)
    xyz = D.global_coordinates(db["ibool"], meshgen.element_coordinates(cfg), db["nglob"])
    p = os.path.join(str(tmp_path), "m.bin")
    D.write_external_mesh(p, db, xyz)
    with pytest.raises(ValueError, match="check value|expected"):
        D.read_external_mesh(p, stacey=False)          # the Stacey records are then read as the next ones


@pytest.mark.gpu
def test_database_files_run_like_the_original(gpulib, tmp_path):
    """A layered viscoelastic block written to the reference's database files, read
    back and set up as the solver does, steps like the database it came from:
    seismograms within 1e-5 relative L2 after 400 steps (the files keep the mesh
    coordinates in single precision, which moves the receiver interpolants by
    ~1e-6)."""
    from conftest import rel_l2
    from specfem3d_gb300 import configs, meshgen, databases as D
    from specfem3d_gb300.solver import GPUSolver
    cfg = configs.small_layered(nstep=400, attenuation=True)
    db = meshgen.build_database(cfg)
    xyz = D.global_coordinates(db["ibool"], meshgen.element_coordinates(cfg), db["nglob"])
    _, back = _roundtrip(str(tmp_path), db, cfg, xyz, True)
    out = []
    for d in (db, back):
        g = GPUSolver(d, cfg)
        g.run(cfg["nstep"], steps_per_graph=50)
        out.append(g.seismograms())
        g.close()
    assert np.abs(out[0]).max() > 0
    assert rel_l2(out[1], out[0]) < 1e-5


def _reference_sequence(flags: dict):
    """Variables save_arrays_solver_mesh writes under the given switches, in order
    (tests/golden/reference_database_records.json, extracted from the reference's
    save_arrays_solver.F90 by tests/golden/make_database_fixture.py)."""
    import json
    from conftest import ROOT
    fx = json.load(open(os.path.join(ROOT, "tests", "golden", "reference_database_records.json")))
    out = []
    for rec in fx["records"]:
        if all(flags.get(g, False) for g in rec["guards"]):
            out.append(rec["name"])
    return out


@pytest.mark.parametrize("case", ["layered_stacey", "coupled", "partition_colored"])
def test_record_sequence_follows_reference_writer(tmp_path, case):
    """The records written are those of the reference's save_arrays_solver_mesh for
    the same switches, in the same order and under the same variable names; the
    reader consumes exactly that many records."""
    from specfem3d_gb300 import configs, meshgen, databases as D
    colors = None
    if case == "layered_stacey":
        cfg = configs.small_layered(nstep=20, attenuation=True)
        db = meshgen.build_database(cfg)
    elif case == "coupled":
        cfg = configs.small_coupled(nstep=20)
        db = meshgen.build_database(cfg)
    else:
        cfg = configs.small_layered(nstep=20, attenuation=False)
        full = meshgen.build_database(cfg)
        db = partition_block.split_x(full, cfg, 3)[1]
        gl = np.asarray(db["global_points"]) - 1
        for c in "xyz":
            db["rmass" + c + "_stacey"] = full["rmass" + c + "_stacey"][gl]
        db["num_free_surface_faces"] = 0
        colors = np.arange(int(db["nspec"])) % 8
    xyz_all = meshgen.element_coordinates(cfg)
    if case == "partition_colored":
        xyz = D.global_coordinates(full["ibool"], xyz_all, full["nglob"])[gl]
    else:
        xyz = D.global_coordinates(db["ibool"], xyz_all, db["nglob"])
    p = os.path.join(str(tmp_path), "proc000000_external_mesh.bin")
    names = D.write_external_mesh(p, db, xyz, colors=colors)
    isac = np.asarray(db.get("ispec_is_acoustic", np.zeros(int(db["nspec"]))), bool)
    nif = int(db.get("num_interfaces", 0))
    flags = {
        "ACOUSTIC_SIMULATION": bool(isac.any()), "ELASTIC_SIMULATION": bool((~isac).any()),
        "num_abs_boundary_faces > 0": int(db["num_abs_boundary_faces"]) > 0,
        "STACEY_ABSORBING_CONDITIONS .and. (.not. PML_CONDITIONS)": bool(db.get("stacey", 0)),
        "num_free_surface_faces > 0": int(db.get("num_free_surface_faces", 0)) > 0,
        "num_coupling_ac_el_faces > 0": int(db.get("num_coupling_ac_el_faces", 0)) > 0,
        "num_interfaces_ext_mesh > 0": nif > 0,
        "num_phase_ispec_acoustic > 0": bool(isac.any()), "num_phase_ispec_elastic > 0": bool((~isac).any()),
        "USE_MESH_COLORING_GPU": colors is not None,
    }
    assert names == _reference_sequence(flags)
    raw = D.read_external_mesh(p, stacey=bool(db.get("stacey", 0)), coloring=colors is not None)
    assert raw["nspec"] == db["nspec"]
