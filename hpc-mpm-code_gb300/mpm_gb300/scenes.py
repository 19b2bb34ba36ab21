"""Seeded synthetic scenes for the MPM transfer path.

A scene holds exactly what the reference reads from its input decks for one
rank: the grid header of ``InputParaGriddata`` (module/data_io.cpp:31-125),
the particle table of ``SolidMaterialPointBase::InputPointData``
(module/solid/solid_data_io.cpp:13-36: coord, matid, mass, vol0, F = I,
vol = vol0), the material table of ``datain_para``
(work/src_solid/explicit/datain_para.cpp:63-82: iprop, E, nu) and the
``BoundaryCondition`` node lists (module/bc.h:7-21).

Particles are seeded at the ``GaussianDistribution`` offsets
(module/mesh.cpp:12-54) inside each cell of a block, plus a seeded uniform
jitter, as ``MaterialPoint::BuildGaussianPoint`` (module/material_point.cpp:16)
places them.  Every generator takes a seed; ``seed = 12345 + config_id`` by
default.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

PIC, FLIP, TPIC, APIC = 0, 1, 2, 3   # MapScheme order, module/dataset.h:19
BC_U, BC_V, BC_W = 0, 1, 2


@dataclass
class Scene:
    xyelem: tuple            # cells per direction
    xymin: tuple             # grid origin
    dxy: tuple               # cell size per direction
    idimc: tuple             # shape-function order per direction (1 linear, 2 quadratic B-spline)
    npxye: tuple             # particles per cell per direction used by MakNodalVol
    dt: float
    mtol: float
    gravity: tuple
    iprop: np.ndarray        # (nmat,) int32: -1 rigid, 0 linear elastic, 1 Neo-Hookean
    mat_prop: np.ndarray     # (nmat, 3) float64: E, nu, spare
    coord: np.ndarray        # (n, 3) float64
    vel: np.ndarray          # (n, 3) float64
    mass: np.ndarray         # (n,) float64
    vol0: np.ndarray         # (n,) float64
    matid: np.ndarray        # (n,) int32
    scheme: int = PIC
    bcs: list = field(default_factory=list)   # [(comp, nodes int32, values float64)]
    name: str = "scene"

    @property
    def num(self) -> int:
        return int(self.mass.shape[0])

    @property
    def xynodec(self) -> tuple:
        return tuple(int(self.xyelem[i] + self.idimc[i]) for i in range(3))

    @property
    def nodec(self) -> int:
        nx, ny, nz = self.xynodec
        return nx * ny * nz

    def node_id(self, i, j, k):
        nx, ny, _ = self.xynodec
        return i + nx * j + nx * ny * k


def gaussian_offsets(npc: int, d: float) -> np.ndarray:
    """Particle offsets from the cell centre, module/mesh.cpp:16-51."""
    table = {
        1: [0.0],
        2: [-0.25, 0.25],
        3: [-1.0 / 3.0, 0.0, 1.0 / 3.0],
        4: [-0.375, -0.125, 0.125, 0.375],
        5: [-0.4, -0.2, 0.0, 0.2, 0.4],
        6: [-5.0 / 12.0, -3.0 / 12.0, -1.0 / 12.0, 1.0 / 12.0, 3.0 / 12.0, 5.0 / 12.0],
    }
    return np.asarray(table[npc], dtype=np.float64) * d


def block_particles(cell_lo, cell_hi, xymin, dxy, npc, jitter, rng):
    """Particles of a block of cells [cell_lo, cell_hi) at npc^3 per cell."""
    offs = [gaussian_offsets(npc[i], dxy[i]) for i in range(3)]
    ci = [np.arange(cell_lo[i], cell_hi[i]) for i in range(3)]
    # cell-major ordering like BuildGaussianPoint: cell loop outside, z/y/x offsets inside
    kz, jy, ix = np.meshgrid(ci[2], ci[1], ci[0], indexing="ij")
    centres = np.stack([xymin[d] + dxy[d] * ((ix, jy, kz)[d].ravel() + 0.5) for d in range(3)], axis=1)
    oz, oy, ox = np.meshgrid(offs[2], offs[1], offs[0], indexing="ij")
    local = np.stack([ox.ravel(), oy.ravel(), oz.ravel()], axis=1)
    pts = (centres[:, None, :] + local[None, :, :]).reshape(-1, 3)
    if jitter > 0.0:
        pts = pts + rng.uniform(-jitter, jitter, size=pts.shape) * np.asarray(dxy)[None, :]
    return pts


def face_nodes(xynodec, axis, index):
    nx, ny, nz = xynodec
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    ijk = (i, j, k)
    mask = ijk[axis] == index
    return (i[mask] + nx * j[mask] + nx * ny * k[mask]).astype(np.int32)


def elastic_block(grid=(32, 32, 32), dx=1.0e-2, cell_lo=(6, 6, 0), cell_hi=(26, 26, 20), npc=2,
                  jitter=0.1, E=1.0e6, nu=0.3, rho=1000.0, dt=1.0e-5, gravity=(0.0, 0.0, -9.81),
                  fix_bottom=True, scheme=PIC, idimc=(1, 1, 1), iprop=0, seed=12346, mtol=1.0e-12,
                  name="elastic_block"):
    """Linear-elastic block under gravity with a fixed bottom face.

    The defaults are the 64,000-particle FP64 CPU case: 32^3 cells,
    dx = 1e-2 m, a 20^3-cell block at 2x2x2 particles per cell, +-0.1 dx jitter,
    E = 1e6 Pa, nu = 0.3, rho = 1000 kg/m^3, dt = 1e-5 s, fixed bottom face.
    """
    rng = np.random.default_rng(seed)
    xymin = (0.0, 0.0, 0.0)
    dxy = (dx, dx, dx)
    pts = block_particles(cell_lo, cell_hi, xymin, dxy, (npc, npc, npc), jitter, rng)
    n = pts.shape[0]
    vp = dx ** 3 / npc ** 3
    scene = Scene(
        xyelem=tuple(grid), xymin=xymin, dxy=dxy, idimc=tuple(idimc), npxye=(npc, npc, npc),
        dt=dt, mtol=mtol, gravity=tuple(gravity),
        iprop=np.array([iprop], dtype=np.int32), mat_prop=np.array([[E, nu, 0.0]]),
        coord=pts, vel=np.zeros((n, 3)), mass=np.full(n, rho * vp), vol0=np.full(n, vp),
        matid=np.zeros(n, dtype=np.int32), scheme=scheme, name=name)
    if fix_bottom:
        nodes = face_nodes(scene.xynodec, 2, 0)
        for comp in (BC_U, BC_V, BC_W):
            scene.bcs.append((comp, nodes, np.zeros(nodes.shape[0])))
    return scene


def spinning_block(grid=(128, 128, 128), dx=4.0e-3, cell_lo=(24, 24, 24), cells=(80, 80, 80), npc=2,
                   compress_quarter=True, jitter=0.1, E=1.0e6, nu=0.3, rho=1000.0, dt=2.0e-6,
                   gravity=(0.0, 0.0, -9.81), vel_sigma=0.5, omega=10.0, scheme=PIC, seed=12347,
                   mtol=1.0e-12, name="spinning_block"):
    """The 4,096,000-particle FP32 explicit case (defaults).

    80^3 cells at 2x2x2 particles per cell on a 128^3 grid, dx = 4e-3 m.
    Velocities are N(0, vel_sigma^2) per component plus a rigid rotation
    omega about z through the block centre.  With ``compress_quarter`` the
    top quarter of the block (its upper cells[2]/4 layers) is squeezed along
    z by 8/27 into a slab at 27 particles per cell with vol0 = dx^3/27 and
    mass = rho * vol0, so that the P2G scatter sees 3.4x the particle density
    there; the particle count is unchanged.
    """
    rng = np.random.default_rng(seed)
    xymin = (0.0, 0.0, 0.0)
    dxy = (dx, dx, dx)
    cell_hi = tuple(cell_lo[i] + cells[i] for i in range(3))
    pts = block_particles(cell_lo, cell_hi, xymin, dxy, (npc, npc, npc), jitter, rng)
    n = pts.shape[0]
    vp = np.full(n, dx ** 3 / npc ** 3)
    if compress_quarter:
        z_lo = xymin[2] + dx * cell_lo[2]
        z0 = z_lo + dx * (cells[2] - cells[2] // 4)
        top = pts[:, 2] >= z0
        factor = float(npc ** 3) / 27.0
        pts[top, 2] = z0 + (pts[top, 2] - z0) * factor
        vp[top] = dx ** 3 / 27.0
    centre = np.array([xymin[d] + dx * (cell_lo[d] + 0.5 * cells[d]) for d in range(3)])
    vel = rng.normal(0.0, vel_sigma, size=(n, 3))
    rel = pts - centre[None, :]
    vel[:, 0] += -omega * rel[:, 1]
    vel[:, 1] += omega * rel[:, 0]
    return Scene(
        xyelem=tuple(grid), xymin=xymin, dxy=dxy, idimc=(1, 1, 1), npxye=(npc, npc, npc),
        dt=dt, mtol=mtol, gravity=tuple(gravity),
        iprop=np.array([0], dtype=np.int32), mat_prop=np.array([[E, nu, 0.0]]),
        coord=pts, vel=vel, mass=rho * vp, vol0=vp.copy(),
        matid=np.zeros(n, dtype=np.int32), scheme=scheme, name=name)


def cantilever(grid=(64, 64, 64), dx=1.0e-2, cell_lo=(0, 2, 2), cells=(60, 60, 60), npc=2, jitter=0.0,
               E=1.0e7, nu=0.3, rho=1000.0, dt=1.0e-3, gravity=(0.0, 0.0, -9.81), iprop=0,
               scheme=PIC, seed=12348, mtol=1.0e-12, idimc=(1, 1, 1), name="cantilever"):
    """Implicit-solid cantilever: cells[0] x cells[1] x cells[2] block clamped at x = 0.

    Defaults: 64^3 grid, 60^3 cells at 2x2x2 particles per cell = 1,728,000
    particles, E = 1e7 Pa, nu = 0.3, dt = 1e-3 s.  All three displacement
    components are fixed on the nodes of the x = 0 face.
    """
    rng = np.random.default_rng(seed)
    xymin = (0.0, 0.0, 0.0)
    dxy = (dx, dx, dx)
    cell_hi = tuple(cell_lo[i] + cells[i] for i in range(3))
    pts = block_particles(cell_lo, cell_hi, xymin, dxy, (npc, npc, npc), jitter, rng)
    n = pts.shape[0]
    vp = dx ** 3 / npc ** 3
    scene = Scene(
        xyelem=tuple(grid), xymin=xymin, dxy=dxy, idimc=tuple(idimc), npxye=(npc, npc, npc),
        dt=dt, mtol=mtol, gravity=tuple(gravity),
        iprop=np.array([iprop], dtype=np.int32), mat_prop=np.array([[E, nu, 0.0]]),
        coord=pts, vel=np.zeros((n, 3)), mass=np.full(n, rho * vp), vol0=np.full(n, vp),
        matid=np.zeros(n, dtype=np.int32), scheme=scheme, name=name)
    nodes = face_nodes(scene.xynodec, 0, cell_lo[0])
    for comp in (BC_U, BC_V, BC_W):
        scene.bcs.append((comp, nodes, np.zeros(nodes.shape[0])))
    return scene


def dam_break(grid=(256, 128, 128), dx=4.0e-3, cells=(128, 128, 96), npc=2, jitter=0.0, c0=30.0, gamma=7.0,
              mu=1.0e-3, rho=1000.0, dt=5.0e-6, gravity=(0.0, 0.0, -9.81), scheme=PIC, seed=12350,
              mtol=1.0e-12, name="dam_break"):
    """Weakly compressible water column (Tait fluid, material model 4).

    Defaults: 256 x 128 x 128-cell grid, dx = 4e-3 m, a 128 x 128 x 96-cell
    column in the x = 0 corner at 2x2x2 particles per cell = 12,582,912
    particles, c0 = 30 m/s, gamma = 7, rho0 = 1000 kg/m^3, mu = 1e-3 Pa s,
    dt = 5e-6 s.  Slip walls on every face of the box: the normal velocity
    component is fixed to zero on the boundary nodes.  mat_prop holds
    {c0, gamma, mu}.
    """
    rng = np.random.default_rng(seed)
    xymin = (0.0, 0.0, 0.0)
    dxy = (dx, dx, dx)
    pts = block_particles((0, 0, 0), tuple(cells), xymin, dxy, (npc, npc, npc), jitter, rng)
    n = pts.shape[0]
    vp = dx ** 3 / npc ** 3
    scene = Scene(
        xyelem=tuple(grid), xymin=xymin, dxy=dxy, idimc=(1, 1, 1), npxye=(npc, npc, npc),
        dt=dt, mtol=mtol, gravity=tuple(gravity),
        iprop=np.array([4], dtype=np.int32), mat_prop=np.array([[c0, gamma, mu]]),
        coord=pts, vel=np.zeros((n, 3)), mass=np.full(n, rho * vp), vol0=np.full(n, vp),
        matid=np.zeros(n, dtype=np.int32), scheme=scheme, name=name)
    nn = scene.xynodec
    for axis, comp in ((0, BC_U), (1, BC_V), (2, BC_W)):
        nodes = np.concatenate([face_nodes(nn, axis, 0), face_nodes(nn, axis, nn[axis] - 1)])
        scene.bcs.append((comp, nodes, np.zeros(nodes.shape[0])))
    return scene


def hydrostatic_column(cells=(8, 8, 20), dx=4.0e-3, head=4, npc=2, c0=30.0, gamma=7.0, mu=1.0e-3, rho=1000.0,
                       g=9.81, dt=5.0e-6):
    """A Tait-fluid column at rest in its hydrostatic state: it fills the box
    laterally (slip walls on every face, `head` empty cell layers above it),
    and each particle starts at the pressure p = rho g (H - z) of its depth,
    with J = (1 + gamma p / (rho c0^2))^(-1/gamma) (the Tait equation of state
    solved for J), F = J^(1/3) I, Cauchy stress -p I, mass rho V / J and
    vol0 = V / J for the lattice volume V = dx^3 / npc^3 (so that the rest
    density m / vol0 is rho and the current volume J vol0 is V).  Returns
    (scene, F (n, 3, 3), stress (n, 6), vol (n), H)."""
    s = dam_break(grid=(cells[0], cells[1], cells[2] + head), dx=dx, cells=cells, npc=npc, c0=c0, gamma=gamma,
                  mu=mu, rho=rho, dt=dt, gravity=(0.0, 0.0, -g), name="hydrostatic_column")
    H = cells[2] * dx
    p = rho * g * (H - s.coord[:, 2])
    J = (1.0 + gamma * p / (rho * c0 * c0)) ** (-1.0 / gamma)
    V = dx ** 3 / npc ** 3
    s.mass[:] = rho * V / J
    s.vol0[:] = V / J
    F = np.zeros((s.num, 3, 3))
    for i in range(3):
        F[:, i, i] = J ** (1.0 / 3.0)
    stress = np.zeros((s.num, 6))
    stress[:, :3] = -p[:, None]
    vol = s.vol0 * np.linalg.det(F)
    return s, F, stress, vol, H


@dataclass
class Batch:
    """Independent scenes packed into one grid (see ``pack_scenes``)."""
    scene: Scene             # the packed scene run by one context
    scenes: list             # the individual scenes, in their own coordinates
    cell_offset: np.ndarray  # (n_scenes, 3) int: cell offset of each scene inside the packed grid
    begin: np.ndarray        # (n_scenes,) first particle of each scene in the packed arrays
    end: np.ndarray          # (n_scenes,) one past the last particle

    def local(self, i, coord):
        """Packed coordinates of scene i's particles -> the scene's own coordinates."""
        s = self.scenes[i]
        return coord - (np.asarray(self.cell_offset[i], dtype=np.float64) * np.asarray(s.dxy))[None, :]


def batch_scenes(n_scenes=256, n_min=1.0e3, n_max=1.0e5, sizes=(32, 40, 48, 56, 64), dx=1.0e-2, npc=2,
                 e_min=1.0e5, e_max=1.0e7, nu_min=0.2, nu_max=0.45, rho=1000.0, dt=1.0e-5, vel_sigma=0.5,
                 gravity=(0.0, 0.0, -9.81), scheme=PIC, seed=12349):
    """The batched workload: independent elastic blocks resting on a fixed floor.

    Scene i: a grid of g^3 cells (g drawn from ``sizes``), a block of about
    N_i particles at npc^3 per cell with N_i log-uniform in [n_min, n_max],
    E log-uniform in [e_min, e_max], nu uniform in [nu_min, nu_max], seeded
    N(0, vel_sigma^2) velocities, the bottom face (k = 0) fixed.  The block
    sits on the floor at a random (x, y) position at least 2 cells from the
    scene's sides.
    """
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_scenes):
        g = int(rng.choice(sizes))
        n_target = float(np.exp(rng.uniform(np.log(n_min), np.log(n_max))))
        cells = max(1.0, n_target / npc ** 3)
        side = max(1, int(round(cells ** (1.0 / 3.0))))
        bz = max(1, int(round(cells / (side * side))))
        b = (min(side, g - 4), min(side, g - 4), min(bz, g - 4))
        lo = (int(rng.integers(2, g - 2 - b[0] + 1)), int(rng.integers(2, g - 2 - b[1] + 1)), 0)
        hi = tuple(lo[d] + b[d] for d in range(3))
        dxy = (dx, dx, dx)
        pts = block_particles(lo, hi, (0.0, 0.0, 0.0), dxy, (npc, npc, npc), 0.1, rng)
        n = pts.shape[0]
        vp = dx ** 3 / npc ** 3
        E = float(np.exp(rng.uniform(np.log(e_min), np.log(e_max))))
        nu = float(rng.uniform(nu_min, nu_max))
        s = Scene(xyelem=(g, g, g), xymin=(0.0, 0.0, 0.0), dxy=dxy, idimc=(1, 1, 1), npxye=(npc, npc, npc),
                  dt=dt, mtol=1.0e-12, gravity=tuple(gravity), iprop=np.array([0], dtype=np.int32),
                  mat_prop=np.array([[E, nu, 0.0]]), coord=pts, vel=rng.normal(0.0, vel_sigma, size=(n, 3)),
                  mass=np.full(n, rho * vp), vol0=np.full(n, vp), matid=np.zeros(n, dtype=np.int32),
                  scheme=scheme, name=f"batch_scene_{i}")
        nodes = face_nodes(s.xynodec, 2, 0)
        for comp in (BC_U, BC_V, BC_W):
            s.bcs.append((comp, nodes, np.zeros(nodes.shape[0])))
        out.append(s)
    return out


def pack_scenes(scenes, gap=2):
    """Pack independent scenes (same dx, dt, gravity, scheme, linear shape
    functions) into one grid so that one context advances all of them with
    one launch per kernel.  Scenes are placed by shelf packing (rows along x,
    rows of rows along y, layers along z) with ``gap`` empty cells between
    neighbours, so no control point is shared and no scene's particles can
    reach another's nodes.  Each scene gets its own material (matid = scene
    index).  Particle-shifting sums are global in a context, so batched runs
    use shifting off."""
    s0 = scenes[0]
    for s in scenes:
        assert s.dxy == s0.dxy and s.dt == s0.dt and s.gravity == s0.gravity and s.scheme == s0.scheme
        assert tuple(s.idimc) == (1, 1, 1)
    ext = np.array([s.xyelem for s in scenes], dtype=np.int64) + gap
    order = np.argsort(-ext.max(axis=1), kind="stable")
    side = int(np.ceil(1.15 * float((ext.prod(axis=1)).sum()) ** (1.0 / 3.0)))
    offs = np.zeros((len(scenes), 3), dtype=np.int64)
    x = y = z = 0
    row_h = layer_h = 0
    width = depth = 0
    for i in order:
        ex, ey, ez = ext[i]
        if x + ex > side and x > 0:            # next row
            x, y = 0, y + row_h
            row_h = 0
        if y + ey > side and y > 0:            # next layer
            x, y, z = 0, 0, z + layer_h
            row_h = layer_h = 0
        offs[i] = (x, y, z)
        x += ex
        row_h = max(row_h, ey)
        layer_h = max(layer_h, ez)
        width, depth = max(width, x), max(depth, y + row_h)
    height = z + layer_h
    grid = (int(width), int(depth), int(height))
    nn = (grid[0] + 1, grid[1] + 1, grid[2] + 1)
    coords, vels, mass, vol0, matid = [], [], [], [], []
    begin, end = [], []
    bcs = {BC_U: [], BC_V: [], BC_W: []}
    n0 = 0
    for i, s in enumerate(scenes):
        shift = offs[i] * np.asarray(s.dxy)
        coords.append(s.coord + shift[None, :])
        vels.append(s.vel)
        mass.append(s.mass)
        vol0.append(s.vol0)
        matid.append(np.full(s.num, i, dtype=np.int32))
        begin.append(n0)
        n0 += s.num
        end.append(n0)
        snx, sny, _ = s.xynodec
        for comp, nodes, vals in s.bcs:
            i_, j_, k_ = nodes % snx, (nodes // snx) % sny, nodes // (snx * sny)
            g = (i_ + offs[i][0]) + nn[0] * ((j_ + offs[i][1]) + nn[1] * (k_ + offs[i][2]))
            bcs[comp].append((g.astype(np.int32), vals))
    packed = Scene(xyelem=grid, xymin=s0.xymin, dxy=s0.dxy, idimc=(1, 1, 1), npxye=s0.npxye, dt=s0.dt,
                   mtol=s0.mtol, gravity=s0.gravity,
                   iprop=np.concatenate([s.iprop[:1] for s in scenes]).astype(np.int32),
                   mat_prop=np.concatenate([s.mat_prop[:1] for s in scenes]),
                   coord=np.concatenate(coords), vel=np.concatenate(vels), mass=np.concatenate(mass),
                   vol0=np.concatenate(vol0), matid=np.concatenate(matid), scheme=s0.scheme,
                   name=f"batch_of_{len(scenes)}")
    for comp in (BC_U, BC_V, BC_W):
        if bcs[comp]:
            packed.bcs.append((comp, np.concatenate([b[0] for b in bcs[comp]]),
                               np.concatenate([b[1] for b in bcs[comp]])))
    return Batch(scene=packed, scenes=list(scenes), cell_offset=offs, begin=np.array(begin), end=np.array(end))


# ---------------------------------------------------------------- decks
SCHEME_NAMES = ("PIC", "FLIP", "TPIC", "APIC")


def write_reference_decks(s: Scene, directory: str, rstflag: int = 0, nsteps: int = 100, rho: float = 1000.0):
    """Write a scene as the reference's input decks for one rank, in the
    formats its readers take: the parameter deck of datain_para
    (work/src_solid/explicit/datain_para.cpp:28-84), the grid deck of
    InputParaGriddata (module/data_io.cpp:31-125) with the u / v / w
    boundary lists of BCInput (module/bc.cpp:9-28), and the particle deck
    of InputPointData (module/solid/solid_data_io.cpp:13-36; it carries no
    velocity).  Returns the three paths (para.txt, grid0.txt, point0.txt)."""
    import os

    os.makedirs(directory, exist_ok=True)
    r = repr
    xymax = [s.xymin[i] + s.dxy[i] * s.xyelem[i] for i in range(3)]
    para = os.path.join(directory, "para.txt")
    with open(para, "w") as f:
        f.write("--- mapping scheme, restart flag, load steps ---\n")
        f.write(f"{SCHEME_NAMES[s.scheme]} {rstflag} 1\n")
        f.write("--- first step, last step, output interval ---\n")
        f.write(f"0 {nsteps} {nsteps}\n")
        f.write("--- dt, mtol ---\n")
        f.write(f"{r(float(s.dt))} {r(float(s.mtol))}\n")
        f.write("--- xyminw ---\n" + " ".join(r(float(v)) for v in s.xymin) + "\n")
        f.write("--- xymaxw ---\n" + " ".join(r(float(v)) for v in xymax) + "\n")
        f.write("--- xyelemw ---\n" + " ".join(str(int(v)) for v in s.xyelem) + "\n")
        f.write("--- idimc ---\n" + " ".join(str(int(v)) for v in s.idimc) + "\n")
        f.write("--- npxye ---\n" + " ".join(str(int(v)) for v in s.npxye) + "\n")
        f.write("--- rho, nmat, npropmax ---\n")
        f.write(f"{r(float(rho))} {len(s.iprop)} 3\n")
        for k in range(len(s.iprop)):
            f.write(f"--- material {k}: iprop, nprop ---\n{int(s.iprop[k])} 3\n")
            f.write(" ".join(r(float(v)) for v in s.mat_prop[k]) + "\n")
        f.write("--- body force ---\n" + " ".join(r(float(v)) for v in s.gravity) + "\n")
    grid = os.path.join(directory, "grid0.txt")
    nel, nn, nc = s.xyelem, [v + 1 for v in s.xyelem], s.xynodec
    with open(grid, "w") as f:
        f.write("0     --- rank ---\n")
        f.write(f"{nel[0] * nel[1] * nel[2]} {nel[0]} {nel[1]} {nel[2]}     --- elements ---\n")
        f.write(f"{nn[0] * nn[1] * nn[2]} {nn[0]} {nn[1]} {nn[2]}     --- nodes ---\n")
        f.write(f"{nc[0] * nc[1] * nc[2]} {nc[0]} {nc[1]} {nc[2]}     --- control points ---\n")
        f.write("0 0 0     --- rank position ---\n")
        f.write(" ".join(r(float(v)) for v in s.xymin) + "     --- xymin ---\n")
        f.write(" ".join(r(float(v)) for v in xymax) + "     --- xymax ---\n")
        f.write("0 0 0     --- first element ---\n")
        f.write(f"{nel[0] - 1} {nel[1] - 1} {nel[2] - 1}     --- last element ---\n")
        f.write("0     --- overlapped ranks ---\n")
        lists = {BC_U: ([], []), BC_V: ([], []), BC_W: ([], [])}
        for comp, nodes, vals in s.bcs:
            lists[comp][0].extend(int(n) for n in nodes)
            lists[comp][1].extend(float(v) for v in vals)
        for comp in (BC_U, BC_V, BC_W):
            nodes, vals = lists[comp]
            f.write(f"{len(nodes)}     --- boundary nodes, component {comp} ---\n")
            for n, v in zip(nodes, vals):
                f.write(f"{n} {r(v)}\n")
    point = os.path.join(directory, "point0.txt")
    with open(point, "w") as f:
        f.write(f"{s.num}     --- number of solid material points ---\n")
        for x in s.coord:
            f.write(" ".join(r(float(v)) for v in x) + "\n")
        for p in range(s.num):
            f.write(f"{p} {int(s.matid[p])} 0 {r(float(s.mass[p]))} {r(float(s.vol0[p]))}\n")
    return para, grid, point
