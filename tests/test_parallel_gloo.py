"""Multi-process host logic on CPU (gloo): replica aggregation and the MPI
exchange of inter-slice assembly, with 2 and 3 ranks.  The device pack/add of
transfer_boun_accel_from_device / transfer_asmbl_accel_to_device is played by
numpy here; the GPU test of those entry points is test_gpu_partition.py."""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, result_dir):
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch.distributed as dist
    from specfem3d_gb300 import configs, meshgen
    from specfem3d_gb300.parallel_host import exchange_interfaces, replica_throughput
    from partition_block import split_x
    dist.init_process_group("gloo", rank=rank, world_size=world)
    # replicas: rank r processes (r + 1) * 1e6 units in (r + 1) * 10 ms
    v = replica_throughput((rank + 1) * 1e6, (rank + 1) * 10.0)
    expected = sum((r + 1) * 1e6 for r in range(world)) / (world * 10.0 / 1000.0)
    ok_rep = abs(v - expected) <= 1e-9 * expected
    # slices of one block, each holding its own contribution at its points
    cfg = configs.small_layered(nx=9, ny=4, counts=(1, 1, 2), nstep=4, attenuation=False)
    db = meshgen.build_database(cfg)
    parts = split_x(db, cfg, world)
    P = parts[rank]
    gl = P["global_points"]  # 1-based global index of each local point

    def contrib(g, r):
        return np.stack([np.sin(0.1 * g + r), np.cos(0.07 * g - r), 0.001 * g * (r + 1)], -1).astype(np.float32)

    accel = contrib(gl.astype(np.float64), rank)
    ni, mx = P["num_interfaces"], P["max_nibool_interfaces"]
    ibi = P["ibool_interfaces"].reshape(ni, mx) - 1
    send = np.zeros((ni, mx, 3), np.float32)
    for i in range(ni):
        send[i, :P["nibool_interfaces"][i]] = accel[ibi[i, :P["nibool_interfaces"][i]]]
    recv = exchange_interfaces(send, P["neighbours"])
    for i in range(ni):
        n = P["nibool_interfaces"][i]
        np.add.at(accel, ibi[i, :n], recv[i, :n])
    # expected: the sum over all slices that hold the point
    owners = [set(p["global_points"].tolist()) for p in parts]
    exp = np.zeros_like(accel)
    for r, own in enumerate(owners):
        m = np.array([g in own for g in gl])
        exp[m] += contrib(gl[m].astype(np.float64), r)
    ok_asm = np.allclose(accel, exp, rtol=1e-6, atol=1e-6)
    with open(os.path.join(result_dir, f"rank{rank}.txt"), "w") as f:
        f.write(f"{int(ok_rep)} {int(ok_asm)} {ni}\n")
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_gloo_replicas_and_interface_exchange(tmp_path, world):
    import torch.multiprocessing as mp
    mp.spawn(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    for r in range(world):
        ok_rep, ok_asm, ni = open(tmp_path / f"rank{r}.txt").read().split()
        assert ok_rep == "1" and ok_asm == "1", (r, ok_rep, ok_asm)
        assert int(ni) >= 1
