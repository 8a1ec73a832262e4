"""General hexahedral test meshes: a block with its interior nodes moved at random,
and a block turned by a rotation with its sources, receivers and moment tensors
turned alike.  Used by the CPU set-up parity tests and the GPU parity tests."""
import numpy as np


def distorted(cfg: dict, amplitude: float = 0.2, seed: int = 5) -> dict:
    """Block mesh of cfg with every node off the block's outer faces moved by up to
    amplitude x the smallest element edge along each axis (seeded)."""
    from specfem3d_gb300 import hexmesh
    mesh = hexmesh.block_mesh(cfg)
    nodes = mesh["nodes"].copy()
    lo, hi = nodes.min(axis=0), nodes.max(axis=0)
    inner = ((nodes > lo + 1e-6) & (nodes < hi - 1e-6)).all(axis=1)
    h = min(float(np.diff(np.unique(np.round(nodes[:, d], 6))).min()) for d in range(3))
    rng = np.random.default_rng(seed)
    nodes[inner] += rng.uniform(-amplitude * h, amplitude * h, size=(int(inner.sum()), 3))
    mesh["nodes"] = nodes
    return mesh


def rotation(a: float = 0.4, b: float = -0.7, c: float = 1.1) -> np.ndarray:
    """Proper rotation matrix from three angles (z, y, x)."""
    cz, sz, cy, sy, cx, sx = np.cos(a), np.sin(a), np.cos(b), np.sin(b), np.cos(c), np.sin(c)
    Rz = np.array([[cz, -sz, 0], [sz, cz, 0], [0, 0, 1]])
    Ry = np.array([[cy, 0, sy], [0, 1, 0], [-sy, 0, cy]])
    Rx = np.array([[1, 0, 0], [0, cx, -sx], [0, sx, cx]])
    return Rz @ Ry @ Rx


def rotated(cfg: dict, R: np.ndarray, mesh=None):
    """(mesh, cfg) of the same problem turned by R: nodes, source and receiver
    positions x -> R x; moment tensors M -> R M R^T; forces F -> R F."""
    from specfem3d_gb300 import hexmesh
    mesh = dict(mesh if mesh is not None else hexmesh.block_mesh(cfg))
    mesh["nodes"] = mesh["nodes"] @ R.T
    out = dict(cfg)
    srcs = []
    for s in cfg["sources"]:
        s = dict(s)
        p = R @ np.array([s["x"], s["y"], s["z"]])
        s["x"], s["y"], s["z"] = (float(v) for v in p)
        if s.get("type", "cmt") == "cmt":
            Mxx, Myy, Mzz, Mxy, Mxz, Myz = s["M"]
            M = np.array([[Mxx, Mxy, Mxz], [Mxy, Myy, Myz], [Mxz, Myz, Mzz]])
            Mr = R @ M @ R.T
            s["M"] = [Mr[0, 0], Mr[1, 1], Mr[2, 2], Mr[0, 1], Mr[0, 2], Mr[1, 2]]
        else:
            s["F"] = list(R @ np.asarray(s["F"], float))
        s.pop("octant", None)
        srcs.append(s)
    out["sources"] = srcs
    out["receivers"] = [tuple(float(v) for v in R @ np.asarray(r, float)) for r in cfg["receivers"]]
    return mesh, out
