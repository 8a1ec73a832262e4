"""Host-side multi-process logic (torch.distributed), one process per GPU.

* ``replica_throughput``: independent replicas of a workload (the reference's
  process-level analogue is NUMBER_OF_SIMULTANEOUS_RUNS,
  src/shared/parallel.f90:2171-2260): whole-job units per second from every
  rank's units and the slowest rank's time.
* ``exchange_interfaces``: the MPI part of the inter-slice assembly
  (assemble_MPI_vector.f90:243-384, assemble_MPI_vector_send_cuda /
  assemble_MPI_vector_write_cuda): every slice sends, for each interface, its
  packed accel values to the neighbour and receives the neighbour's; the
  device side packs (transfer_boun_accel_from_device) and adds
  (transfer_asmbl_accel_to_device).
"""
from __future__ import annotations

import numpy as np


def replica_throughput(units_local: float, ms_local: float) -> float:
    """Sum of units over ranks / max of times over ranks (units per second)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return units_local / (ms_local / 1000.0)
    t_ms = torch.tensor([ms_local], dtype=torch.float64)
    units = torch.tensor([units_local], dtype=torch.float64)
    dist.all_reduce(t_ms, op=dist.ReduceOp.MAX)
    dist.all_reduce(units, op=dist.ReduceOp.SUM)
    return float(units.item()) / (float(t_ms.item()) / 1000.0)


def exchange_interfaces(send: np.ndarray, neighbours, tag: int = 0) -> np.ndarray:
    """send: (num_interfaces, max_nibool, 3) float32, row i for the interface with
    rank neighbours[i]; returns the receive buffer of the same layout, row i
    holding neighbour i's values for its interface with this rank."""
    import torch
    import torch.distributed as dist
    send_t = torch.from_numpy(np.ascontiguousarray(send, np.float32))
    recv_t = torch.zeros_like(send_t)
    reqs = []
    for i, q in enumerate(neighbours):
        reqs.append(dist.isend(send_t[i].contiguous(), dst=int(q), tag=tag))
    for i, q in enumerate(neighbours):
        buf = torch.zeros_like(send_t[i])
        dist.recv(buf, src=int(q), tag=tag)
        recv_t[i] = buf
    for r in reqs:
        r.wait()
    return recv_t.numpy()
