"""Generate the golden fixtures in tests/golden/ from the reference itself.

Runs the reference's own compiled translation units (oracle/_ref/libmpmref.so,
built by oracle/build_ref.sh from the reference checkout) on small seeded
scenes and stores inputs and outputs as compressed .npz files.  The reference
checkout exists only in the development container, so the fixtures are
committed and this script is re-run only when a case is added:

    oracle/build_ref.sh <reference checkout> && python tests/golden/make_golden.py
    python tests/golden/make_golden.py --hyperelastic     # only models 2 and 3
    python tests/golden/make_golden.py --affine           # only the TPIC / APIC cases
    python tests/golden/make_golden.py --io               # only the deck / restart fixtures (tests/golden/io)
    python tests/golden/make_golden.py --fbar             # only the F-bar cases
    python tests/golden/make_golden.py --fluid            # only the stabilized fluid assembly
    python tests/golden/make_golden.py --implicit2        # only the quadratic / StVK / Mooney-Rivlin implicit cases
    python tests/golden/make_golden.py --fluid-newton     # only the stabilized fluid Newton loop
    python tests/golden/make_golden.py --fluid-step       # only whole stabilized fluid time steps
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "hpc-mpm-code_gb300"))

from mpm_gb300 import scenes  # noqa: E402
from oracle import ref  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def scene_arrays(s):
    d = {"xyelem": np.array(s.xyelem), "xymin": np.array(s.xymin), "dxy": np.array(s.dxy),
         "idimc": np.array(s.idimc), "npxye": np.array(s.npxye), "dt": np.array(s.dt), "mtol": np.array(s.mtol),
         "gravity": np.array(s.gravity), "iprop": s.iprop, "mat_prop": s.mat_prop, "coord": s.coord, "vel": s.vel,
         "mass": s.mass, "vol0": s.vol0, "matid": s.matid, "scheme": np.array(s.scheme)}
    for i, (comp, nodes, vals) in enumerate(s.bcs):
        d[f"bc{i}_comp"] = np.array(comp)
        d[f"bc{i}_nodes"] = nodes
        d[f"bc{i}_vals"] = vals
    d["nbc"] = np.array(len(s.bcs))
    return d


def explicit_case(name, scene, nsteps, facl=1.0, fbar=False):
    r = ref.RefSolid(scene, fbar=fbar)
    r.p2g(facl)
    out = {f"p2g_{k}": r.nodal(k) for k in ("nmass", "nvof", "nmome", "nforce", "nvel", "naccel", "nvol")}
    r = ref.RefSolid(scene, fbar=fbar)
    r.steps(1, facl)
    out.update({f"step1_{k}": v for k, v in r.particles().items()})
    if scene.scheme >= scenes.TPIC:
        out["step1_affine"] = r.affine()
    if fbar:
        out["step1_Fbar"], out["step1_Jbar"] = r.fbar()
    r.steps(nsteps - 1, facl)
    out.update({f"stepN_{k}": v for k, v in r.particles().items()})
    if scene.scheme >= scenes.TPIC:
        out["stepN_affine"] = r.affine()
    if fbar:
        out["stepN_Fbar"], out["stepN_Jbar"] = r.fbar()
        out["fbar"] = np.array(1)
    out["nsteps"] = np.array(nsteps)
    out["facl"] = np.array(facl)
    np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **scene_arrays(scene), **out)
    print("wrote", name, scene.num, "particles")


def implicit_case(name, scene, nr_flag, nsteps):
    r = ref.RefSolid(scene, implicit=True, nr_flag=nr_flag)
    r.assemble()
    matrow, matcol, amat, adiag, b = r.matrix()
    rng = np.random.default_rng(7)
    x = rng.normal(size=r.nodec * 3)
    y = r.matvec(x)
    xs, it = r.solve()
    out = {"matrow": matrow, "matcolid": matcol, "amat": amat, "adiag": adiag, "b_rhs": b, "mv_x": x, "mv_y": y,
           "solve_x": xs, "solve_iters": np.array(it)}
    r = ref.RefSolid(scene, implicit=True, nr_flag=nr_flag)
    r.implicit_steps(nsteps)
    out.update({f"stepN_{k}": v for k, v in r.particles().items()})
    out["nsteps"] = np.array(nsteps)
    out["nr_flag"] = np.array(int(nr_flag))
    np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **scene_arrays(scene), **out)
    print("wrote", name, scene.num, "particles", r.nmat, "blocks")


def hyperelastic_cases():
    """St.Venant-Kirchhoff (model 2) and Mooney-Rivlin (model 3) blocks with a
    random initial velocity; their own generator so that adding them leaves
    the earlier fixtures untouched."""
    rng = np.random.default_rng(20261204)
    s = scenes.elastic_block(grid=(10, 10, 10), cell_lo=(2, 2, 0), cell_hi=(8, 8, 6), iprop=2, seed=105,
                             E=5.0e5, scheme=scenes.FLIP)
    s.vel[:] = rng.normal(0.0, 0.3, size=s.vel.shape)
    explicit_case("explicit_stvk", s, nsteps=10)
    # Mooney-Rivlin: c1 + c2 = mu / 2 and the bulk modulus of E = 1e6, nu = 0.3
    s = scenes.elastic_block(grid=(10, 10, 10), cell_lo=(2, 2, 0), cell_hi=(8, 8, 6), iprop=3, seed=106)
    s.mat_prop[:] = [[1.5e5, 0.42e5, 8.33e5]]
    s.vel[:] = rng.normal(0.0, 0.3, size=s.vel.shape)
    explicit_case("explicit_mooney_rivlin", s, nsteps=10)


def implicit_extra_cases():
    """Implicit solids beyond linear shape functions and models 0 / 1: a
    beam with the shape orders of the reference's own solid case
    (data/generate/solid/input.txt: FLIP, Neo-Hookean, idimc 2 1 2, Newton),
    a St.Venant-Kirchhoff cantilever (linear shapes, Newton) and a
    Mooney-Rivlin cantilever on quadratic B-splines in every direction
    (Newton); each with a random initial velocity so that the first system
    already carries stress."""
    rng = np.random.default_rng(20261210)
    s = scenes.cantilever(grid=(10, 4, 8), cells=(6, 2, 4), cell_lo=(0, 1, 2), iprop=1, idimc=(2, 1, 2),
                          scheme=scenes.FLIP, seed=131)
    s.vel[:] = rng.normal(0.0, 0.05, size=s.vel.shape)
    implicit_case("implicit_beam_quadratic", s, nr_flag=True, nsteps=3)
    s = scenes.cantilever(grid=(10, 8, 8), cells=(6, 4, 4), cell_lo=(0, 2, 2), iprop=2, seed=132)
    s.vel[:] = rng.normal(0.0, 0.05, size=s.vel.shape)
    implicit_case("implicit_stvk", s, nr_flag=True, nsteps=3)
    # Mooney-Rivlin: c1, c2 and the bulk modulus of E = 1e7, nu = 0.3 (c1 + c2 = mu / 2)
    s = scenes.cantilever(grid=(8, 6, 6), cells=(5, 3, 3), cell_lo=(0, 1, 1), iprop=3, idimc=(2, 2, 2), seed=133)
    s.mat_prop[:] = [[1.5e6, 0.42e6, 8.33e6]]
    s.vel[:] = rng.normal(0.0, 0.05, size=s.vel.shape)
    implicit_case("implicit_mooney_rivlin", s, nr_flag=True, nsteps=3)


def affine_cases():
    """TPIC and APIC (MapScheme 2 and 3) with linear and with quadratic
    B-spline shape functions: a block with a random and a rotating velocity
    field, so that the affine matrices are far from zero."""
    rng = np.random.default_rng(20261205)
    for scheme, nm in ((scenes.TPIC, "tpic"), (scenes.APIC, "apic")):
        s = scenes.elastic_block(grid=(10, 10, 8), cell_lo=(2, 2, 0), cell_hi=(7, 7, 5), scheme=scheme,
                                 dt=1.0e-5, seed=107 + scheme)
        c = s.coord.mean(axis=0)
        s.vel[:] = rng.normal(0.0, 0.2, size=s.vel.shape) + 20.0 * np.cross([0.0, 0.0, 1.0], s.coord - c)
        explicit_case(f"explicit_{nm}", s, nsteps=25)
        s = scenes.elastic_block(grid=(10, 6, 10), cell_lo=(2, 1, 0), cell_hi=(8, 5, 5), idimc=(2, 1, 2),
                                 seed=109 + scheme, scheme=scheme)
        c = s.coord.mean(axis=0)
        s.vel[:] = rng.normal(0.0, 0.2, size=s.vel.shape) + 20.0 * np.cross([0.0, 1.0, 0.0], s.coord - c)
        explicit_case(f"explicit_{nm}_quadratic", s, nsteps=10)


def fbar_cases():
    """The F-bar projection (Fbar_flag on; fbar_projection.cpp restated in
    the harness on the reference's members): a linear elastic PIC block and
    a Neo-Hookean FLIP block with a random initial velocity."""
    rng = np.random.default_rng(20261207)
    s = scenes.elastic_block(grid=(10, 10, 8), cell_lo=(2, 2, 0), cell_hi=(7, 7, 5), iprop=0, E=5.0e5, dt=1.0e-5,
                             seed=121)
    s.vel[:] = rng.normal(0.0, 0.3, size=s.vel.shape)
    explicit_case("explicit_fbar_linear", s, nsteps=20, fbar=True)
    s = scenes.elastic_block(grid=(10, 10, 8), cell_lo=(2, 2, 0), cell_hi=(7, 7, 5), iprop=1, E=5.0e5, dt=1.0e-5,
                             seed=122, scheme=scenes.FLIP)
    s.vel[:] = rng.normal(0.0, 0.3, size=s.vel.shape)
    explicit_case("explicit_fbar_neohookean", s, nsteps=20, fbar=True)


def io_cases():
    """The reference's on-disk formats: decks written by
    scenes.write_reference_decks for a small APIC block with a fixed bottom,
    parsed by the reference's own readers (io.npz: parsed_*); a TPIC and an
    APIC restart written by the reference's RestartOutput after 10 steps;
    the APIC restart read back by the reference's RestartInput and run 10
    more steps (io.npz: cont_*)."""
    d = os.path.join(OUT, "io")
    os.makedirs(d, exist_ok=True)
    rng = np.random.default_rng(20261206)
    out = {}
    for scheme, nm in ((scenes.TPIC, "tpic"), (scenes.APIC, "apic")):
        s = scenes.elastic_block(grid=(8, 8, 8), cell_lo=(2, 2, 0), cell_hi=(6, 6, 4), scheme=scheme, dt=1.0e-5,
                                 seed=111 + scheme)
        c = s.coord.mean(axis=0)
        s.vel[:] = rng.normal(0.0, 0.2, size=s.vel.shape) + 20.0 * np.cross([0.0, 0.0, 1.0], s.coord - c)
        if scheme == scenes.APIC:
            para, grid, point = scenes.write_reference_decks(s, d, rstflag=1, nsteps=10)
            parsed = ref.read_decks(grid, point)
            out.update({f"parsed_{k}": v for k, v in parsed.items()})
        r = ref.RefSolid(s)
        r.steps(10)
        r.restart_output(os.path.join(d, f"restart_{nm}"))
        if scheme == scenes.APIC:
            r = ref.RefSolid(s)
            r.restart_input(os.path.join(d, f"restart_{nm}"))
            r.steps(10)
            out.update({f"cont_{k}": v for k, v in r.particles().items()})
            out["cont_affine"] = r.affine()
            out["cont_nsteps"] = np.array(10)
    np.savez_compressed(os.path.join(d, "io.npz"), **out)
    print("wrote", d, sorted(os.listdir(d)))


def ns_inputs(seed=11, xyelem=(6, 5, 4), dx=0.1, ppd=2):
    """Seeded particles (ppd^3 per cell, jittered, in all but the outer cell
    layer) and a nodal Newton state for one stabilized-fluid system; the
    velocity is zero on the lower-x third of the nodes so that the
    zero-velocity branch of the element size (he) is taken there."""
    rng = np.random.default_rng(seed)
    xyelem = np.asarray(xyelem)
    nnc = xyelem + 1
    N = int(np.prod(nnc))
    pts = []
    for k in range(1, xyelem[2] - 1):
        for j in range(1, xyelem[1] - 1):
            for i in range(1, xyelem[0] - 1):
                for c in np.ndindex(ppd, ppd, ppd):
                    pts.append((np.array([i, j, k]) + (np.array(c) + 0.5 + rng.uniform(-0.3, 0.3, 3)) / ppd) * dx)
    x = np.array(pts)
    n = len(x)
    vol = np.full(n, dx ** 3 / ppd ** 3) * rng.uniform(0.9, 1.1, n)
    mass = 1000.0 * vol
    nvel = rng.normal(0.0, 0.5, (3, N))
    ix = np.arange(N) % nnc[0]
    nvel[:, ix <= nnc[0] // 3] = 0.0
    naccel = rng.normal(0.0, 2.0, (3, N))
    ndispl = rng.normal(0.0, 1e-3 * dx, (3, N))
    npres = rng.normal(0.0, 50.0, N)
    nmass = rng.uniform(0.0, 0.2, N)
    return dict(xyelem=xyelem, xymin=np.zeros(3), dxy=np.full(3, dx), x=x, mass=mass, vol=vol,
                nvel=nvel.ravel(), naccel=naccel.ravel(), ndispl=ndispl.ravel(), npres=npres, nmass=nmass,
                rho=1000.0, rmu=1.0e-3 * 50, dt=2.0e-3, beta=0.25, gamma=0.5, gravity=np.array([0.0, 0.0, -9.8]),
                facl=0.8, mtol=1.0e-12)


def fluid_case(name="ns_assemble"):
    """One Newton system of the reference's StabilizedMPM::SolveNS."""
    c = ns_inputs()
    r = ref.RefFluid(c["xyelem"], c["xymin"], c["dxy"], c["dt"], c["mtol"], c["gravity"], c["x"], c["mass"],
                     c["vol"], c["rho"], c["rmu"], c["beta"], c["gamma"])
    out = r.assemble(c["nvel"], c["naccel"], c["ndispl"], c["npres"], c["nmass"], c["facl"])
    np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **c, **out)


def ns_box_inputs(xyelem=(6, 5, 4), dx=0.01, ppd=2, seed=3, amp=0.05):
    """A fluid box filled with particles (every cell, ppd^3 per cell with
    +-0.1 spacing jitter, rho = 1000), the nodal mass of their linear P2G, a
    smooth velocity field that vanishes on the walls, zero acceleration;
    no-slip walls (u = v = w = 0) on the sides and bottom, p = 0 on the top
    face.  Newmark beta = 1/4, gamma = 1/2, dt = 2e-3 s, gravity -9.8 m/s^2."""
    rng = np.random.default_rng(seed)
    xyelem = np.array(xyelem)
    nnc = xyelem + 1
    N = int(np.prod(nnc))
    pts = []
    for k in range(xyelem[2]):
        for j in range(xyelem[1]):
            for i in range(xyelem[0]):
                for c in range(ppd ** 3):
                    a, b, d = c % ppd, (c // ppd) % ppd, c // ppd ** 2
                    off = (np.array([a, b, d]) + 0.5) / ppd + rng.uniform(-0.1, 0.1, 3) / ppd
                    pts.append((np.array([i, j, k]) + off) * dx)
    x = np.array(pts)
    n = len(x)
    vol = np.full(n, dx ** 3 / ppd ** 3)
    mass = 1000.0 * vol
    cell = np.floor(x / dx).astype(int)
    nmass = np.zeros(N)
    for q in range(8):
        i, j, k = q & 1, (q >> 1) & 1, q >> 2
        w = np.ones(n)
        for d, o in enumerate((i, j, k)):
            w *= 1.0 - np.abs(x[:, d] - dx * (cell[:, d] + o)) / dx
        nid = (cell[:, 0] + i) + nnc[0] * ((cell[:, 1] + j) + nnc[1] * (cell[:, 2] + k))
        np.add.at(nmass, nid, w * mass)
    ix = np.arange(N) % nnc[0]
    iy = (np.arange(N) // nnc[0]) % nnc[1]
    iz = np.arange(N) // (nnc[0] * nnc[1])
    X, Y, Z = ix / xyelem[0], iy / xyelem[1], iz / xyelem[2]
    nvel = np.zeros((3, N))
    s3 = np.sin(np.pi * X) * np.sin(np.pi * Y) * np.sin(np.pi * Z)
    nvel[0] = amp * s3 * np.cos(np.pi * Y)
    nvel[1] = -amp * s3 * np.cos(np.pi * X)
    nvel[2] = 0.3 * amp * np.sin(np.pi * X) * np.sin(np.pi * Y) * np.sin(2 * np.pi * Z)
    wall = np.nonzero((ix == 0) | (ix == xyelem[0]) | (iy == 0) | (iy == xyelem[1]) | (iz == 0))[0]
    top = np.nonzero(iz == xyelem[2])[0]
    return dict(xyelem=xyelem, xymin=np.zeros(3), dxy=np.full(3, dx), x=x, mass=mass, vol=vol, nvel=nvel.ravel(),
                naccel=np.zeros(3 * N), nmass=nmass, rho=1000.0, rmu=1.0e-3, dt=2.0e-3, beta=0.25, gamma=0.5,
                gravity=np.array([0.0, 0.0, -9.8]), facl=1.0, mtol=1.0e-12, bc_wall=wall.astype(np.int32),
                bc_top=top.astype(np.int32))


def fluid_newton_case(name="ns_solve"):
    """SolveNS on the filled box: the reference's Newton loop with GPBiCGSafe
    post-iterated to ||b - A x|| <= 1e-10 ||b|| (ref_harness.cpp, ref_ns_solve)."""
    c = ns_box_inputs()
    r = ref.RefFluid(c["xyelem"], c["xymin"], c["dxy"], c["dt"], c["mtol"], c["gravity"], c["x"], c["mass"],
                     c["vol"], c["rho"], c["rmu"], c["beta"], c["gamma"])
    wall, top = c["bc_wall"], c["bc_top"]
    bcs = [(wall, np.zeros(len(wall)))] * 3 + [(top, np.zeros(len(top)))]
    nd, npres, newton, krylov = r.solve(c["nvel"], c["naccel"], c["nmass"], c["facl"], bcs, rtol=1.0e-10)
    np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **c, ndispl=nd, npres=npres, newton=np.array(newton),
                        krylov=np.array(krylov), rtol=np.array(1.0e-10))
    print("wrote", name, len(c["mass"]), "particles,", newton, "Newton iterations,", krylov, "Krylov iterations")


def ns_particle_kinematics(x, dx, xyelem, amp=0.05, seed=5):
    """Particle velocities from the smooth field of ns_box_inputs evaluated at
    the particles, and small seeded accelerations (the FLIP update reads them)."""
    rng = np.random.default_rng(seed)
    X, Y, Z = (x[:, d] / (dx * xyelem[d]) for d in range(3))
    s3 = np.sin(np.pi * X) * np.sin(np.pi * Y) * np.sin(np.pi * Z)
    v = np.stack([amp * s3 * np.cos(np.pi * Y), -amp * s3 * np.cos(np.pi * X),
                  0.3 * amp * np.sin(np.pi * X) * np.sin(np.pi * Y) * np.sin(2 * np.pi * Z)], axis=1)
    a = rng.normal(0.0, 0.1, x.shape)
    return v, a


def fluid_lid_case(name="ns_step_lid", nsteps=2):
    """Whole time steps of the reference's fluid loop with non-zero boundary
    values and a load factor below one: the filled box of ns_box_inputs as a
    lid-driven cavity (no-slip sides and bottom, the top face moving at
    u = 0.04 m/s, the pressure fixed to 5 Pa at one top corner node),
    facl = 0.6, FLIP; the particle state after nsteps and the nodal fields of
    the first Particle2Node."""
    c = ns_box_inputs()
    c["facl"] = 0.6
    xyelem = np.asarray(c["xyelem"])
    nnc = xyelem + 1
    N = int(np.prod(nnc))
    iz = np.arange(N) // (nnc[0] * nnc[1])
    top = np.nonzero(iz == xyelem[2])[0]
    wall = np.setdiff1d(c["bc_wall"], top)
    u_nodes = np.concatenate([wall, top]).astype(np.int32)
    u_vals = np.concatenate([np.zeros(len(wall)), np.full(len(top), 0.04)])
    vw_nodes = u_nodes
    corner = np.array([top[-1]], dtype=np.int32)
    bcs = [(u_nodes, u_vals), (vw_nodes, np.zeros(len(vw_nodes))), (vw_nodes, np.zeros(len(vw_nodes))),
           (corner, np.array([5.0]))]
    vel, acc = ns_particle_kinematics(c["x"], c["dxy"][0], c["xyelem"], seed=8)
    r = ref.RefFluid(c["xyelem"], c["xymin"], c["dxy"], c["dt"], c["mtol"], c["gravity"], c["x"], c["mass"], c["vol"],
                     c["rho"], c["rmu"], c["beta"], c["gamma"])
    nodal, part, newton, krylov = r.run(vel, acc, 1, c["facl"], bcs, nsteps, rtol=1.0e-10)
    out = {k: v for k, v in c.items() if k not in ("bc_wall", "bc_top")}
    out.update(vel=vel, accel=acc, nsteps=np.array(nsteps), bc_u_nodes=u_nodes, bc_u_vals=u_vals,
               bc_vw_nodes=vw_nodes, bc_p_nodes=corner, bc_p_vals=np.array([5.0]))
    out.update({f"p2g_{f}": v for f, v in nodal.items()})
    out.update({f"s_{f}": v for f, v in part.items()})
    np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **out)
    print(name, nsteps, "steps:", newton, "Newton,", krylov, "Krylov iterations")


def fluid_step_case(name="ns_step", nsteps=3):
    """Whole time steps of the reference's fluid loop (MeshPointLinklist,
    Particle2Node, SolveNS with the linear systems solved to 1e-10 as in
    --fluid-newton, Node2Particle) on the filled box of ns_box_inputs, PIC and
    FLIP: the nodal fields of the first Particle2Node and the particle state
    (x, v, a, pres) after one step and after nsteps."""
    c = ns_box_inputs()
    wall, top = c["bc_wall"], c["bc_top"]
    bcs = [(wall, np.zeros(len(wall)))] * 3 + [(top, np.zeros(len(top)))]
    vel, acc = ns_particle_kinematics(c["x"], c["dxy"][0], c["xyelem"])
    out = dict(c, vel=vel, accel=acc, nsteps=np.array(nsteps))
    for scheme, tag in ((0, "pic"), (1, "flip")):
        for k in (1, nsteps):
            r = ref.RefFluid(c["xyelem"], c["xymin"], c["dxy"], c["dt"], c["mtol"], c["gravity"], c["x"],
                             c["mass"], c["vol"], c["rho"], c["rmu"], c["beta"], c["gamma"])
            nodal, part, newton, krylov = r.run(vel, acc, scheme, c["facl"], bcs, k, rtol=1.0e-10)
            if k == 1:
                out.update({f"{tag}_p2g_{f}": v for f, v in nodal.items()})
            out.update({f"{tag}_s{k}_{f}": v for f, v in part.items()})
            out[f"{tag}_s{k}_newton"] = np.array(newton)
            print(name, tag, k, "steps:", newton, "Newton,", krylov, "Krylov iterations")
    np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **out)


def main():
    if not ref.available():
        raise SystemExit("oracle/_ref/libmpmref.so missing: run oracle/build_ref.sh <reference checkout> first")
    if "--hyperelastic" in sys.argv[1:]:
        hyperelastic_cases()
        return
    if "--affine" in sys.argv[1:]:
        affine_cases()
        return
    if "--io" in sys.argv[1:]:
        io_cases()
        return
    if "--fluid" in sys.argv[1:]:
        fluid_case()
        return
    if "--fluid-newton" in sys.argv[1:]:
        fluid_newton_case()
        return
    if "--fluid-step" in sys.argv[1:]:
        fluid_step_case()
        fluid_lid_case()
        return
    if "--implicit2" in sys.argv[1:]:
        implicit_extra_cases()
        return
    if "--fbar" in sys.argv[1:]:
        fbar_cases()
        return
    rng = np.random.default_rng(20261203)
    # small elastic block, fixed bottom, PIC and FLIP, random initial velocity
    for scheme, nm in ((scenes.PIC, "explicit_pic"), (scenes.FLIP, "explicit_flip")):
        s = scenes.elastic_block(grid=(10, 10, 8), cell_lo=(2, 2, 0), cell_hi=(7, 7, 5), scheme=scheme,
                                 dt=1.0e-5, seed=101 + scheme)
        s.vel[:] = rng.normal(0.0, 0.3, size=s.vel.shape)
        explicit_case(nm, s, nsteps=25)
    # quadratic B-spline shape functions in x and z (idimc 2 1 2, like the reference's beam deck)
    s = scenes.elastic_block(grid=(10, 6, 10), cell_lo=(2, 1, 0), cell_hi=(8, 5, 5), idimc=(2, 1, 2), seed=103,
                             scheme=scenes.FLIP)
    s.vel[:] = rng.normal(0.0, 0.2, size=s.vel.shape)
    explicit_case("explicit_quadratic", s, nsteps=10)
    # load ramp factor below one and a Neo-Hookean block
    s = scenes.elastic_block(grid=(10, 10, 10), cell_lo=(2, 2, 0), cell_hi=(8, 8, 6), iprop=1, seed=104,
                             E=5.0e5)
    s.vel[:] = rng.normal(0.0, 0.2, size=s.vel.shape)
    explicit_case("explicit_neohookean", s, nsteps=10, facl=0.5)
    # implicit solid: linear elastic single solve per step, and Neo-Hookean Newton
    s = scenes.cantilever(grid=(10, 8, 8), cells=(6, 4, 4), cell_lo=(0, 2, 2), iprop=0)
    implicit_case("implicit_linear", s, nr_flag=False, nsteps=3)
    s = scenes.cantilever(grid=(10, 8, 8), cells=(6, 4, 4), cell_lo=(0, 2, 2), iprop=1)
    implicit_case("implicit_neohookean", s, nr_flag=True, nsteps=3)
    hyperelastic_cases()
    affine_cases()
    io_cases()
    fbar_cases()
    fluid_case()
    implicit_extra_cases()
    fluid_newton_case()
    fluid_step_case()
    fluid_lid_case()


if __name__ == "__main__":
    main()
