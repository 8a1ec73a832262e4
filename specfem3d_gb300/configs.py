"""Workload definitions: the synthetic meshes, models, sources and receivers.

A configuration is a plain dict (the schema read by :mod:`specfem3d_gb300.meshgen`):

``nx, ny``            elements along x and y
``x0, x1, y0, y1``    horizontal extent (m)
``zlev``              vertical node levels of the element layers, bottom to top (m)
``elem_layer``        material layer of each element (len nx*ny*nz), or None
``layers``            list of {rho, vp, vs[, Qmu, Qkappa]} per material layer
``absorbing``         faces with Stacey conditions (free surface on the others)
``sources``           list of {type: cmt|force, x, y, z, M: [Mxx,Myy,Mzz,Mxy,Mxz,Myz] (N.m)
                      | F: [fx,fy,fz], stf: ricker|heaviside|gaussian, f0|hdur, tshift}
``receivers``         list of (x, y, z)
``dt, nstep``         time step and number of steps
``attenuation``       bool (N_SLS = 3 standard linear solids)

The named workloads follow the benchmark definitions of the project:
``refex``  the reference's example homogeneous_halfspace_HEX8_elastic_absorbing_Stacey_5sides
           (36x36x16 hexes over 134x134x60 km, DT 0.05, CMT with Heaviside stf);
``homogeneous_block``     homogeneous elastic block 10x10x5 km, 24x24x12 hexes, Ricker 2 Hz
                          CMT, 25 receivers (the CPU-runnable plain forward);
``layered_viscoelastic``  three-layer viscoelastic block 20x20x10 km, 128x128x64 hexes
                          (~67.6 M points), N_SLS = 3, 400 receivers;
``coupled_fluid_solid``   96x96x48 hexes, top sixth water over a perturbed elastic solid,
                          pressure source, 256 hydrophones;
``batched_shots``         64x64x32 hexes of the layered domain without attenuation, 32 CMT shots.
"""
from __future__ import annotations

import math

import numpy as np

COURANT_SUGGESTED = 0.5
GLL_MIN_SPACING = (1.0 - math.sqrt(3.0 / 7.0)) / 2.0  # smallest GLL gap / element edge, NGLL=5


def significant_dt(dt: float) -> float:
    """Cut a suggested time step to two significant digits with the half-digit
    rule of get_timestep_limit_significant_digit (shared/read_parameter_file.F90:1456-1497)."""
    lpow = int(2.0 - math.log10(dt))
    fac = 10.0 ** lpow
    ival = int(fac * dt)
    if fac * dt - ival >= 0.5:
        return (ival + 0.5) / fac
    return ival / fac


def cfl_dt(cfg: dict) -> float:
    """dt = COURANT_SUGGESTED * min GLL distance / vmax per element, minimum over
    elements, rounded (shared/check_mesh_resolution.f90:278-300)."""
    nx, ny = cfg["nx"], cfg["ny"]
    dx = (cfg["x1"] - cfg["x0"]) / nx
    dy = (cfg["y1"] - cfg["y0"]) / ny
    zlev = np.asarray(cfg["zlev"])
    best = math.inf
    lay_of_ez = _layer_of_ez(cfg)
    for ez in range(len(zlev) - 1):
        dz = zlev[ez + 1] - zlev[ez]
        lay = cfg["layers"][lay_of_ez[ez]]
        vmax = max(lay["vp"], lay["vs"]) * cfg.get("vmax_factor", 1.0)
        dmin = GLL_MIN_SPACING * min(dx, dy, dz)
        best = min(best, significant_dt(COURANT_SUGGESTED * dmin / vmax))
    return best


def _layer_of_ez(cfg):
    nz = len(cfg["zlev"]) - 1
    if cfg.get("layer_counts"):
        out = []
        for li, n in enumerate(cfg["layer_counts"]):
            out += [li] * n
        return out
    return [0] * nz


def layered_zlev(z_bottom: float, interfaces_top_down, counts_top_down):
    """Node levels for conforming layers: interfaces given top-down (z values,
    first = top surface), element counts per layer top-down."""
    tops = list(interfaces_top_down) + [z_bottom]
    levels = []
    for li in reversed(range(len(counts_top_down))):
        za, zb, n = tops[li + 1], tops[li], counts_top_down[li]
        seg = [za + (zb - za) * q / n for q in range(n)]
        levels += seg
    levels.append(tops[0])
    return levels


def random_moment_tensor(rng: np.random.Generator):
    """Seeded N(0,1) symmetric 3x3 tensor normalised to unit Frobenius norm (N.m):
    returns [Mxx, Myy, Mzz, Mxy, Mxz, Myz]."""
    a = rng.standard_normal((3, 3))
    m = 0.5 * (a + a.T)
    m /= np.linalg.norm(m)
    return [float(m[0, 0]), float(m[1, 1]), float(m[2, 2]), float(m[0, 1]), float(m[0, 2]), float(m[1, 2])]


def finish(cfg: dict) -> dict:
    """Fill derived fields (elem_layer, dt) of a configuration."""
    nz = len(cfg["zlev"]) - 1
    lay = _layer_of_ez(cfg)
    if cfg.get("elem_layer") is None:
        cfg["elem_layer"] = np.repeat(np.asarray(lay, np.int32), cfg["nx"] * cfg["ny"])
    if cfg.get("dt") is None:
        cfg["dt"] = cfl_dt(cfg)
    cfg.setdefault("absorbing", ["xmin", "xmax", "ymin", "ymax", "bottom"])
    cfg.setdefault("stacey", True)
    cfg.setdefault("attenuation", False)
    assert len(cfg["elem_layer"]) == cfg["nx"] * cfg["ny"] * nz
    return cfg


def refex(nstep: int = 5000) -> dict:
    """The reference example homogeneous_halfspace_HEX8_elastic_absorbing_Stacey_5sides:
    CMTSOLUTION (dyne.cm, r/t/p) mapped to x/y/z N.m (get_cmt.f90:424,
    locate_source.F90:210-223); STATIONS lat -> y, lon -> x."""
    Mrr, Mtt, Mpp, Mrt, Mrp, Mtp = -7.6e27, 7.7e27, -2.0e26, -2.5e28, 4.0e26, -2.5e27
    s = 1e-7
    M = [Mpp * s, Mtt * s, Mrr * s, -Mtp * s, Mrp * s, -Mrt * s]
    cfg = dict(nx=36, ny=36, x0=0.0, x1=134000.0, y0=0.0, y1=134000.0,
               zlev=list(np.linspace(-60000.0, 0.0, 17)), elem_layer=None,
               layers=[dict(rho=2300.0, vp=2800.0, vs=1500.0)], dt=0.05, nstep=nstep,
               sources=[dict(type="cmt", x=67000.0, y=67000.0, z=-30000.0, M=M, stf="heaviside", hdur=5.0)],
               # the REF_SEIS run located its stations at the coordinates printed in its
               # output_solver.txt (22732.0996, 34696.3984, ...): STATIONS values kept to
               # six significant digits
               receivers=[(x, 67000.0, 0.0) for x in (22732.1, 34696.4, 46660.7, 58625.0)],
               station_names=["X20", "X30", "X40", "X50"])
    # the source sits on a mesh vertex shared by 8 elements; the REF_SEIS run put
    # it in the element below, in front of and left of it (its output_solver.txt:
    # element 2772 of slice 0, local coordinates (1, 1, 1) of the CUBIT mesh)
    cfg["sources"][0]["octant"] = (-1, -1, -1)
    return finish(cfg)


def refex_no_absorbing(nstep: int = 5000) -> dict:
    """The reference example homogeneous_halfspace_HEX8_elastic_no_absorbing: the
    same block, source and stations without Stacey faces.  Its REF_SEIS run (4
    slices) placed the source, a vertex of 8 elements, in element 4905 of slice 0
    at local coordinates (-1, -1, 1) (REF_SEIS/output_solver.txt), which in its
    CUBIT mesh (MESH-default) is the element on the -x, +y, -z side of the vertex."""
    cfg = refex(nstep)
    cfg["stacey"] = False
    cfg["sources"][0]["octant"] = (-1, 1, -1)
    return cfg


def refex_cpml(nstep: int = 2400) -> dict:
    """The reference example CPML_examples/homogeneous_halfspace_HEX8_elastic_absorbing_CPML_5sides:
    the 36 x 36 x 16 block of the Stacey example with C-PML layers of three
    elements on the four sides and the bottom (absorbing_cpml_file: 9036 CPML
    elements, widths 11166.667 / 11166.667 / 11250 m), f0_FOR_PML 0.05555 Hz,
    no Stacey; FORCESOLUTION: a point force of 1e10 N along (E, N, Z_UP) =
    (1, -2, -1), normalised (setup_sources_receivers.f90:1132-1143), with a
    0.128 Hz Ricker at (67, 67, -30) km, a mesh vertex, where a point force lands
    on the vertex's one global point whichever element holds it; dt 0.11 s.
    The layers themselves come from ``pml.setup(db, cfg, nel=3, f0=cfg["pml_f0"])``."""
    cfg = refex(nstep)
    cfg["dt"] = 0.11
    f = np.array([1.0, -2.0, -1.0])
    f = 1e10 * f / np.sqrt(np.sum(f * f))
    cfg["sources"] = [dict(type="force", x=67000.0, y=67000.0, z=-30000.0, F=[float(v) for v in f],
                           stf="ricker", f0=0.128)]
    cfg["pml_f0"] = 0.05555
    cfg["pml_elements"] = 3
    return cfg


def refex_acoustic(nstep: int = 1000) -> dict:
    """The reference example homogeneous_acoustic: the 36 x 36 x 16 block of the
    Stacey example (134 x 134 x 60 km) filled with one fluid (rho 2300, vp 2800:
    nummaterial_velocity_file), Stacey faces on the five sides and a free surface
    on top; the CMTSOLUTION explosion (Mrr = Mtt = Mpp = 7.7e27 dyne.cm, half
    duration 2 s) at (67, 67, -30) km, a mesh vertex (its REF_SEIS run logged
    element 2772, local (1, 1, 1)); in a fluid element the reference takes a
    Gaussian time function and t0 = 3 half durations = 6 s; four hydrophones 50 m
    below the surface record pressure; dt 0.1136 s."""
    cfg = refex(nstep)
    M0 = 7.7e27 * 1e-7
    cfg["layers"] = [dict(rho=2300.0, vp=2800.0, vs=0.0)]
    cfg["dt"] = 0.1136
    cfg["sources"] = [dict(type="cmt", x=67000.0, y=67000.0, z=-30000.0, M=[M0, M0, M0, 0.0, 0.0, 0.0],
                           stf="heaviside", hdur=2.0, octant=(-1, -1, -1))]
    cfg["receivers"] = [(x, 67000.0, -50.0) for x in (22732.14, 34696.43, 46660.71, 58625.0)]
    cfg["record"] = ("pressure",)
    return cfg


def attenuation_benchmark(nstep: int = 1300) -> dict:
    """The reference benchmark EXAMPLES/benchmarks/attenuation/viscoelastic: an
    80 x 80 x 80 regular mesh of 37.5 m cubes spanning [-1500, 1500]^3 m
    (Mesh_Par_file, interfaces.dat), rho 2000, vp 3297.849, vs 2222.536,
    Q_kappa 10, Q_mu 20 with N_SLS = 3 around f0_REFERENCE 18 Hz; free surfaces,
    no Stacey; a vertical unit point force with an 18 Hz Ricker at (10, 10, 10)
    and one station at (510, 510, 510) (USE_SOURCES_RECEIVERS_Z); dt 5e-4."""
    lev = [float(v) for v in np.linspace(-1500.0, 1500.0, 81)]
    cfg = dict(nx=80, ny=80, x0=-1500.0, x1=1500.0, y0=-1500.0, y1=1500.0, zlev=lev,
               elem_layer=np.zeros(80 ** 3, np.int32),
               layers=[dict(rho=2000.0, vp=3297.849, vs=2222.536, Qkappa=10.0, Qmu=20.0)],
               dt=0.0005, nstep=nstep, stacey=False, absorbing=[], attenuation=True,
               sources=[dict(type="force", x=10.0, y=10.0, z=10.0, F=[0.0, 0.0, 1.0], stf="ricker", f0=18.0)],
               receivers=[(510.0, 510.0, 510.0)], station_names=["CE.1"])
    return finish(cfg)


def analytic_elastic(nstep: int = 14000) -> dict:
    """The reference benchmark EXAMPLES/benchmarks/analytic_examples/analytic_solution_elastic:
    16 x 16 x 16 regular elements of 2 km spanning [-16, 16]^3 km, rho 2300,
    vp 2800, vs 1500; Stacey on all six faces (STACEY_INSTEAD_OF_FREE_SURFACE);
    the CMTSOLUTION double couple Mrp = 1e23 dyne.cm (Heaviside, half duration
    2 s) at the origin (USE_SOURCES_RECEIVERS_Z), a vertex of 8 elements, which
    its REF_SEIS run placed at local (1, 1, 1) of its element 512, the element on
    the -x, -y, -z side; six stations; dt 1e-3."""
    s = 1e-7
    M = [0.0, 0.0, 0.0, 0.0, 1e23 * s, 0.0]          # Mxz = Mrp
    lev = [float(v) for v in np.linspace(-16000.0, 16000.0, 17)]
    stations = [("Z1", 3000.0, 1000.0, 4000.0), ("Z2", 1000.0, 3000.0, 4000.0), ("Z3", 6000.0, 1000.0, 4000.0),
                ("Z4", 1000.0, 6000.0, 4000.0), ("Z5", 6000.0, 1000.0, 2000.0), ("Z6", 1000.0, 6000.0, 2000.0)]
    cfg = dict(nx=16, ny=16, x0=-16000.0, x1=16000.0, y0=-16000.0, y1=16000.0, zlev=lev,
               elem_layer=np.zeros(16 ** 3, np.int32), layers=[dict(rho=2300.0, vp=2800.0, vs=1500.0)],
               dt=0.001, nstep=nstep, stacey=True, absorbing=["xmin", "xmax", "ymin", "ymax", "bottom", "top"],
               sources=[dict(type="cmt", x=0.0, y=0.0, z=0.0, M=M, stf="heaviside", hdur=2.0, octant=(-1, -1, -1))],
               receivers=[(x, y, z) for _, x, y, z in stations], station_names=[n for n, _, _, _ in stations])
    return finish(cfg)


# the 22 stations of EXAMPLES/applications/waterlayered_halfspace/DATA/STATIONS:
# (name, x = longitude column, y = latitude column, burial)
WATERLAYERED_STATIONS = [
    ("X10", 10767.86, 67000.0, 100.0), ("X20", 22732.14, 67000.0, 100.0), ("X30", 34696.43, 67000.0, 100.0),
    ("X40", 46660.71, 67000.0, 100.0), ("X50", 58625.00, 67000.0, 100.0), ("X55", 67000.00, 67000.0, 100.0),
    ("X60", 75375.00, 67000.0, 100.0), ("X70", 87339.29, 67000.0, 100.0), ("X80", 99303.57, 67000.0, 100.0),
    ("X90", 111269.86, 67000.0, 100.0), ("X1", 0.0, 67000.0, 100.0), ("X2", 67000.0, 67000.0, 25000.0),
    ("X3", 134000.0, 67000.0, 100.0), ("X4", 67000.0, 67000.0, 3500.0), ("X5", 67000.0, 67000.0, 3000.2),
    ("X6", 67000.0, 67000.0, 3000.1), ("X7", 67000.0, 67000.0, 2999.9), ("X8", 67000.0, 67000.0, 2999.8),
    ("Y1", 58625.0, 67000.0, 2999.9), ("Y2", 58625.0, 67000.0, 3000.1), ("Y3", 46660.71, 67000.0, 2999.9),
    ("Y4", 46660.71, 67000.0, 3000.1)]


def waterlayered(nstep: int = 4500) -> dict:
    """The reference example waterlayered_halfspace: a 45 x 45 x 20 element block
    of 134 x 134 x 60 km (its MESH-default grid), the top element row water
    (rho 1028, vp 1480) over a solid (3200, 7500, 4300) given as two materials
    of equal properties as in its nummaterial_velocity_file; Stacey on the five
    sides, free surface on top; the CMTSOLUTION explosion (Mrr = Mtt = Mpp =
    1e23 dyne.cm, half duration 2 s) 1 km deep in the water at (66999.9, 67000);
    the STATIONS list buried below the surface; dt 0.005 s.  The source lies in
    a fluid element, so the reference takes a Gaussian time function and t0 = 6 s;
    seismograms in fluid elements are (1/rho) grad of the potential."""
    M0 = 1e23 * 1e-7
    zlev = [float(z) for z in np.linspace(-60000.0, 0.0, 21)]
    rows = [2] * 16 + [1] * 3 + [0]           # bottom-up: material 3, material 2, water
    cfg = dict(nx=45, ny=45, x0=0.0, x1=134000.0, y0=0.0, y1=134000.0, zlev=zlev,
               elem_layer=np.repeat(np.asarray(rows, np.int32), 45 * 45),
               layers=[dict(rho=1028.0, vp=1480.0, vs=0.0), dict(rho=3200.0, vp=7500.0, vs=4300.0),
                       dict(rho=3200.0, vp=7500.0, vs=4300.0)],
               dt=0.005, nstep=nstep,
               sources=[dict(type="cmt", x=66999.9, y=67000.0, z=-1000.0, M=[M0, M0, M0, 0.0, 0.0, 0.0],
                             stf="heaviside", hdur=2.0)],
               receivers=[(x, y, -b) for _, x, y, b in WATERLAYERED_STATIONS],
               station_names=[n for n, _, _, _ in WATERLAYERED_STATIONS],
               record=("displ", "veloc", "accel"))
    return finish(cfg)


def homogeneous_block(nstep: int = 2000, seed: int = 2024) -> dict:
    rng = np.random.default_rng(seed)
    g = np.linspace(1000.0, 9000.0, 5)
    cfg = dict(nx=24, ny=24, x0=0.0, x1=10000.0, y0=0.0, y1=10000.0,
               zlev=list(np.linspace(-5000.0, 0.0, 13)), elem_layer=None,
               layers=[dict(rho=2300.0, vp=2800.0, vs=1500.0)], dt=None, nstep=nstep,
               sources=[dict(type="cmt", x=5000.0, y=5000.0, z=-2500.0, M=random_moment_tensor(rng),
                             stf="ricker", f0=2.0)],
               receivers=[(float(x), float(y), 0.0) for y in g for x in g])
    return finish(cfg)


def layered_viscoelastic(nstep: int = 4000, seed: int = 2025, nx: int = 128, ny: int = 128, counts=(13, 26, 25)) -> dict:
    """Layered viscoelastic block; conforming vertical counts 13/26/25 (top-down)
    make every element a non-cube box, i.e. the irregular-element path."""
    rng = np.random.default_rng(seed)
    zlev = layered_zlev(-10000.0, [0.0, -2000.0, -6000.0], list(counts))
    layers = [dict(rho=2000.0, vp=2000.0, vs=1000.0, Qmu=40.0, Qkappa=9999.0),
              dict(rho=2500.0, vp=4000.0, vs=2300.0, Qmu=150.0, Qkappa=9999.0),
              dict(rho=2800.0, vp=6000.0, vs=3460.0, Qmu=400.0, Qkappa=9999.0)]
    # layer index per element row, bottom to top
    lay_bottom_up = []
    for li in reversed(range(3)):
        lay_bottom_up += [li] * counts[li]
    g = np.linspace(500.0, 19500.0, 20)
    cfg = dict(nx=nx, ny=ny, x0=0.0, x1=20000.0, y0=0.0, y1=20000.0, zlev=zlev,
               layer_counts=None, elem_layer=np.repeat(np.asarray(lay_bottom_up, np.int32), nx * ny),
               layers=layers, dt=None, nstep=nstep, attenuation=True,
               sources=[dict(type="cmt", x=10000.0, y=10000.0, z=-8000.0, M=random_moment_tensor(rng),
                             stf="ricker", f0=2.0)],
               receivers=[(float(x), float(y), 0.0) for y in g for x in g])
    cfg["dt"] = _cfl_dt_by_rows(cfg, lay_bottom_up)
    return finish(cfg)


def _cfl_dt_by_rows(cfg, lay_rows):
    dx = (cfg["x1"] - cfg["x0"]) / cfg["nx"]
    dy = (cfg["y1"] - cfg["y0"]) / cfg["ny"]
    zlev = cfg["zlev"]
    best = math.inf
    for ez, li in enumerate(lay_rows):
        dz = zlev[ez + 1] - zlev[ez]
        lay = cfg["layers"][li]
        dmin = GLL_MIN_SPACING * min(dx, dy, dz)
        best = min(best, significant_dt(COURANT_SUGGESTED * dmin / max(lay["vp"], lay["vs"])))
    return best


def small_layered(nx=6, ny=5, counts=(2, 2, 3), nstep=200, attenuation=True, seed=7) -> dict:
    """Small irregular (non-cube) layered block for parity tests (layered_viscoelastic physics)."""
    cfg = layered_viscoelastic(nstep=nstep, seed=seed, nx=nx, ny=ny, counts=counts)
    cfg["x1"] = 20000.0 * nx / 128
    cfg["y1"] = 20000.0 * ny / 128
    z1 = -2000.0 * counts[0] / 13
    z2 = z1 - 4000.0 * counts[1] / 26
    cfg["zlev"] = layered_zlev(z2 - 4000.0 * counts[2] / 25, [0.0, z1, z2], list(counts))
    lay_bottom_up = []
    for li in reversed(range(3)):
        lay_bottom_up += [li] * counts[li]
    cfg["elem_layer"] = np.repeat(np.asarray(lay_bottom_up, np.int32), nx * ny)
    cfg["attenuation"] = attenuation
    cx, cy = cfg["x1"] / 2, cfg["y1"] / 2
    cfg["sources"][0].update(x=cx + 37.0, y=cy - 21.0, z=0.55 * cfg["zlev"][0])
    cfg["receivers"] = [(cx * 0.5, cy * 0.5, 0.0), (cx * 1.3, cy * 0.7, 0.0), (cx, cy, 0.5 * cfg["zlev"][0])]
    cfg["dt"] = _cfl_dt_by_rows(cfg, lay_bottom_up)
    return finish(cfg)


def batched_shots(nstep: int = 3000, nshots: int = 32, seed: int = 2026, nx: int = 64) -> dict:
    """nx x nx x nx/2 elements on the 20x20x10 km block (64 in the benchmark
    definition; smaller nx for profiling), shots and receivers unchanged."""
    rng = np.random.default_rng(seed)
    zlev = list(np.linspace(-10000.0, 0.0, nx // 2 + 1))
    g = np.linspace(1000.0, 19000.0, 5)
    shots = []
    for _ in range(nshots):
        shots.append(dict(type="cmt", x=float(rng.uniform(1000, 19000)), y=float(rng.uniform(1000, 19000)),
                          z=-float(rng.uniform(2000, 8000)), M=random_moment_tensor(rng), stf="ricker", f0=2.0))
    cfg = dict(nx=nx, ny=nx, x0=0.0, x1=20000.0, y0=0.0, y1=20000.0, zlev=zlev, elem_layer=None,
               layers=[dict(rho=2400.0, vp=3000.0, vs=1700.0)], dt=None, nstep=nstep,
               perturbation=dict(corr_len=1000.0, seed=2027),
               sources=shots[:1], shots=shots,
               receivers=[(float(x), float(y), 0.0) for y in g for x in g], vmax_factor=1.05)
    cfg = finish(cfg)
    # CFL with the +-5 % perturbation bound on vp
    cfg["dt"] = significant_dt(COURANT_SUGGESTED * GLL_MIN_SPACING * (20000.0 / nx) / (3000.0 * 1.05))
    return cfg


def adjoint_gradient(nstep: int = 3000, nshots: int = 8, checkpoint_every: int = 200) -> dict:
    """Misfit-gradient workload: the batched-shots mesh and background model with
    its first ``nshots`` shots; observed data come from the true model, the
    background with a Gaussian blob of +3 % vs (1.5 km radius) at the block
    centre, 5 km deep."""
    cfg = batched_shots(nstep=nstep, nshots=32)
    cfg["shots"] = cfg["shots"][:nshots]
    cfg["sources"] = cfg["shots"][:1]
    cfg["blob"] = dict(center=(10000.0, 10000.0, -5000.0), radius=1500.0, dlnvs=0.03)
    cfg["checkpoint_every"] = checkpoint_every
    return cfg


def small_adjoint(nstep: int = 600, nshots: int = 2, n: int = 12, seed: int = 31) -> dict:
    """Scaled-down misfit-gradient workload for tests: n x n x n/2 elements of the
    batched-shots element size (312.5 m), same background physics and blob
    (radius scaled to the block), ``nshots`` Ricker 2 Hz CMT shots."""
    rng = np.random.default_rng(seed)
    h = 20000.0 / 64
    nz = max(2, n // 2)
    L, D = n * h, nz * h
    shots = [dict(type="cmt", x=float(rng.uniform(0.25, 0.75) * L), y=float(rng.uniform(0.25, 0.75) * L),
                  z=-float(rng.uniform(0.3, 0.7) * D), M=random_moment_tensor(rng), stf="ricker", f0=2.0)
             for _ in range(nshots)]
    g = np.linspace(0.1 * L, 0.9 * L, 5)
    cfg = dict(nx=n, ny=n, x0=0.0, x1=L, y0=0.0, y1=L, zlev=[float(-D + q * h) for q in range(nz + 1)],
               elem_layer=None, layers=[dict(rho=2400.0, vp=3000.0, vs=1700.0)], dt=None, nstep=nstep,
               perturbation=dict(corr_len=1000.0, seed=2027), sources=shots[:1], shots=shots,
               receivers=[(float(x), float(y), 0.0) for y in g for x in g])
    cfg = finish(cfg)
    cfg["dt"] = significant_dt(COURANT_SUGGESTED * GLL_MIN_SPACING * h / (3000.0 * 1.05))
    cfg["blob"] = dict(center=(0.5 * L, 0.5 * L, -0.5 * D), radius=0.15 * L, dlnvs=0.03)
    cfg["checkpoint_every"] = max(1, nstep // 7)
    return cfg


def coupled_fluid_solid(nstep: int = 3000, nx: int = 96, ny: int = 96, nz: int = 48, fluid_layers: int = 8, seed: int = 2027) -> dict:
    """Coupled fluid/solid block: the top sixth of the depth is water
    (vp 1500, rho 1020), the rest a solid of (3000, 1700, 2400) carrying a seeded
    +-5 % Gaussian-correlated perturbation (1 km correlation length); pressure
    source (3 Hz Ricker) in the water; hydrophones at mid water depth.  The
    domain is the 20x20x10 km block of the layered workload."""
    zlev = list(np.linspace(-10000.0, 0.0, nz + 1))
    rows = [1] * (nz - fluid_layers) + [0] * fluid_layers
    zf = zlev[nz - fluid_layers]
    g = np.linspace(20000.0 / 32, 20000.0 - 20000.0 / 32, 16)
    x1 = 20000.0 * nx / 96
    y1 = 20000.0 * ny / 96
    g = np.linspace(x1 / 32, x1 - x1 / 32, 16)
    cfg = dict(nx=nx, ny=ny, x0=0.0, x1=x1, y0=0.0, y1=y1, zlev=[float(z) for z in zlev],
               elem_layer=np.repeat(np.asarray(rows, np.int32), nx * ny),
               layers=[dict(rho=1020.0, vp=1500.0, vs=0.0), dict(rho=2400.0, vp=3000.0, vs=1700.0)],
               dt=None, nstep=nstep, perturbation=dict(corr_len=1000.0, seed=seed),
               sources=[dict(type="force", x=x1 / 2 + 13.0, y=y1 / 2 - 7.0, z=zf / 2, F=[1.0, 1.0, 1.0],
                             stf="ricker", f0=3.0)],
               receivers=[(float(x), float(y), float(zf / 2)) for y in g for x in g], record=("pressure",),
               vmax_factor=1.05)
    cfg["dt"] = _cfl_dt_by_rows(cfg, rows) if False else None
    cfg = finish(cfg)
    # CFL over both materials with the perturbation bound
    dx = x1 / nx
    dz = 10000.0 / nz
    dmin = GLL_MIN_SPACING * min(dx, dz)
    cfg["dt"] = significant_dt(COURANT_SUGGESTED * dmin / (3000.0 * 1.05))
    return cfg


def small_coupled(nx: int = 5, ny: int = 4, nz: int = 6, fluid_layers: int = 2, nstep: int = 300) -> dict:
    """Small coupled block with the coupled_fluid_solid physics for parity tests."""
    cfg = coupled_fluid_solid(nstep=nstep, nx=nx, ny=ny, nz=nz, fluid_layers=fluid_layers)
    h = 20000.0 / 96
    cfg["x1"], cfg["y1"] = nx * h, ny * h
    cfg["zlev"] = [float(-nz * h + q * h) for q in range(nz + 1)]
    zf = cfg["zlev"][nz - fluid_layers]
    cfg["sources"][0].update(x=cfg["x1"] / 2 + 13.0, y=cfg["y1"] / 2 - 7.0, z=zf / 2)
    cfg["receivers"] = [(cfg["x1"] * 0.3, cfg["y1"] * 0.4, zf / 2), (cfg["x1"] * 0.7, cfg["y1"] * 0.6, zf / 2),
                        (cfg["x1"] * 0.5, cfg["y1"] * 0.5, zf / 2 - 3.0)]
    return cfg
