"""Inter-slice assembly (transfer_boun_accel_from_device / transfer_asmbl_accel_to_device)
on the GPU: a block split into three slices along x, each slice a separate
Mesh driven through the per-call ABI in the reference's order (outer elements,
pack and exchange, inner elements, assembly, corrector), gives the seismograms
and wavefield of the undivided block (FP32; atomic summation order differs, so
<= 1e-5 relative)."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("att", [False, True])
def test_three_slices_match_single_mesh(gpulib, att):
    from specfem3d_gb300 import configs, meshgen
    from specfem3d_gb300.solver import GPUSolver
    from partition_block import receive_buffers, split_x
    cfg = configs.small_layered(nx=9, ny=5, counts=(2, 2, 3), nstep=300, attenuation=att)
    cfg["receivers"] = [(cfg["x1"] * f, cfg["y1"] * 0.4, 0.0) for f in (0.1, 0.3, 0.5, 0.7, 0.9)]
    db = meshgen.build_database(cfg)
    whole = GPUSolver(db, cfg)
    whole.run_per_call(cfg["nstep"])
    ref_seis = whole.seismograms()
    ref_d = whole.fields()[0].reshape(-1, 3)
    whole.close()
    parts = split_x(db, cfg, 3)
    assert all(p["num_interfaces"] >= 1 for p in parts) and len(parts[0]["phase_outer"]) > 0
    slices = [GPUSolver(p, cfg) for p in parts]
    for _ in range(cfg["nstep"]):
        for g in slices:
            g.step_predict()
        for g in slices:
            g.step_forces(1)
        sent = [g.pack_interfaces() for g in slices]
        for g in slices:
            g.step_forces(2)
        for g, recv in zip(slices, receive_buffers(parts, sent)):
            g.assemble_interfaces(recv)
        for g in slices:
            g.step_finish()
    seis = np.zeros_like(ref_seis)
    disp = np.zeros_like(ref_d)
    for g, p in zip(slices, parts):
        if p["nrec"]:
            seis[p["receiver_index"]] = g.seismograms()
        disp[p["global_points"] - 1] = g.fields()[0].reshape(-1, 3)
        g.close()
    e_s, e_d = rel_l2(seis, ref_seis), rel_l2(disp, ref_d)
    print(f"3 slices vs single mesh, {cfg['nstep']} steps: seismograms {e_s:.2e}, displacement {e_d:.2e}")
    assert np.abs(ref_seis).max() > 0
    assert e_s < 1e-5 and e_d < 1e-5
