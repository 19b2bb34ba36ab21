"""ORACLE (test infrastructure only): numpy restatement of one Newton system
of the reference's stabilized incompressible fluid MPM on linear shape
functions.  Only tests and fixture scripts import this module.

Follows, step for step:
  StabilizedMPM::MakNSStabCoeff     module/fluid/MPM/solve_ns_mpm.cpp:64-135 (VMS branch)
  PredictNewmarkBetaVelAndAccel     module/nonlinear_time_integration.cpp:58-70
  NewmarkBetaParaSet                module/nonlinear_time_integration.cpp:42-56
  ImplicitDsfCorr                   module/material_point.cpp:127-172 (alpha_f = 1)
  StabilizedMPM::AssembleNSSystem   module/fluid/MPM/solve_ns_mpm.cpp:137-320
  ComputeNRLumpedMat                module/material_point.h:67-71
  AddInertialForceToRHS             module/material_point.h:74-85
The matrix is returned as a 27-point block stencil [27][16][nodec]: slot
s = (dx+1) + 3(dy+1) + 9(dz+1) of the column node's offset from the row node,
entry k = row_var * 4 + col_var over (u, v, w, p) -- the block_id order of
CrsMat (module/solver/crsmat.cpp:73-75).  Pinned against the reference's own
compiled AssembleNSSystem by tests/golden/ns_assemble.npz.
"""
import numpy as np


def newmark(dt, beta, gamma):
    """nb_para of NewmarkBetaParaSet (nonlinear_time_integration.cpp:42-56)."""
    return np.array([gamma / (beta * dt), gamma / beta - 1.0, dt / 2.0 * (gamma / beta - 2.0),
                     1.0 / (beta * dt * dt), 1.0 / (beta * dt), 1.0 / (2.0 * beta) - 1.0])


def _shape(x, xmin, dx, cell, nnc):
    """Linear MakSf (module/shape_function.cpp:28-110) of points x (n,3) in the
    given cells: weights (n,8), gradients (n,8,3), node ids (n,8); node q =
    i + 2j + 4k sits at cell + (i, j, k)."""
    n = x.shape[0]
    w = np.empty((n, 3, 2))
    dw = np.empty((n, 3, 2))
    for d in range(3):
        for k in range(2):
            xy = xmin[d] + dx[d] * (cell[:, d] + k)
            w[:, d, k] = 1.0 - np.abs(x[:, d] - xy) / dx[d]
            dw[:, d, k] = (-1.0 if k == 0 else 1.0) / dx[d]
    W = np.empty((n, 8))
    D = np.empty((n, 8, 3))
    nid = np.empty((n, 8), dtype=np.int64)
    for k in range(2):
        for j in range(2):
            for i in range(2):
                q = i + 2 * j + 4 * k
                W[:, q] = w[:, 0, i] * w[:, 1, j] * w[:, 2, k]
                D[:, q, 0] = dw[:, 0, i] * w[:, 1, j] * w[:, 2, k]
                D[:, q, 1] = w[:, 0, i] * dw[:, 1, j] * w[:, 2, k]
                D[:, q, 2] = w[:, 0, i] * w[:, 1, j] * dw[:, 2, k]
                nid[:, q] = (cell[:, 0] + i) + nnc[0] * ((cell[:, 1] + j) + nnc[1] * (cell[:, 2] + k))
    return W, D, nid


def ns_assemble(xyelem, xymin, dxy, rho, rmu, dt, beta, gamma, gravity, facl, mtol,
                x, mass, vol, nvel, naccel, ndispl, npres, nmass):
    """One Newton system of SolveNS on the nodal state (component-major
    nvel/naccel/ndispl of 3*nodec; npres, nmass of nodec) and particles
    x (n,3), mass, vol.  Returns tau1, tau2, stencil [27][16][nodec], b (4*nodec)."""
    xyelem = np.asarray(xyelem)
    xmin = np.asarray(xymin, dtype=np.float64)
    dx = np.asarray(dxy, dtype=np.float64)
    nnc = xyelem + 1
    N = int(np.prod(nnc))
    x = np.asarray(x, dtype=np.float64)
    n = x.shape[0]
    cell = np.floor((x - xmin) / dx).astype(np.int64)   # MeshPointLinklist (material_point.cpp:59-65)
    nb = newmark(dt, beta, gamma)
    nv = np.asarray(nvel).reshape(3, N)
    na = np.asarray(naccel).reshape(3, N)
    nd = np.asarray(ndispl).reshape(3, N)
    vel_k = nb[0] * nd - nb[1] * nv - nb[2] * na
    acc_k = nb[3] * nd - nb[4] * nv - nb[5] * na
    # ---- MakNSStabCoeff: velocity and gradients at the element centre ----
    xc = xmin + dx * (cell + 0.5)
    Wc, Dc, nid = _shape(xc, xmin, dx, cell, nnc)
    uc = np.einsum("nq,rnq->nr", Wc, nv[:, nid])
    uvw = np.sum(uc * uc, axis=1)
    udsf = np.sum(np.abs(np.einsum("nr,nqr->nq", uc, Dc)), axis=1)
    with np.errstate(divide="ignore", invalid="ignore"):
        he = np.where(udsf < mtol, dx[0] * np.cbrt(6.0 / np.pi), 2.0 * np.sqrt(uvw) / udsf)
    t1 = rho / dt
    t2 = 2.0 * rho * np.sqrt(uvw) / he
    t3 = 4.0 * rmu / (he * he)
    tau1 = 1.0 / (t1 + t2 + t3)
    tau2 = (he * he) / (4.0 * tau1)
    # ---- AssembleNSSystem ----
    W, D, nid = _shape(x, xmin, dx, cell, nnc)
    Fd = np.einsum("nqc,rnq->nrc", D, nd[:, nid]) + np.eye(3)   # ComputeDeltaDefGrad, alpha_f = 1
    D = np.einsum("nqi,nij->nqj", D, np.linalg.inv(Fd))          # ImplicitDsfCorr
    f = np.asarray(gravity, dtype=np.float64) * facl
    pres_k = np.einsum("nq,nq->n", W, npres[nid])
    accel_k = np.einsum("nq,rnq->nr", W, acc_k[:, nid])
    gp = np.einsum("nqc,nq->nc", D, npres[nid])
    gv = np.einsum("nqc,rnq->nrc", D, vel_k[:, nid])             # gv[r][c] = d vel_r / d x_c
    dev = rmu * (gv + np.transpose(gv, (0, 2, 1)))
    V = vol[:, None, None]
    m = mass[:, None, None]
    T1 = tau1[:, None, None]
    T2 = tau2[:, None, None]
    a = D[:, :, None, :]     # row node (test function)
    b = D[:, None, :, :]     # column node (trial function)
    Ni = W[:, :, None]
    Nj = W[:, None, :]
    ab = np.sum(a * b, axis=3)
    K = np.zeros((n, 8, 8, 4, 4))
    for r in range(3):
        for c in range(3):
            K[..., r, c] = nb[0] * (V * rmu * (a[..., c] * b[..., r] + (ab if r == c else 0.0))
                                    + V * T2 * a[..., r] * b[..., c])
        K[..., r, 3] = -V * a[..., r] * Nj
        K[..., 3, r] = nb[0] * V * Ni * b[..., r] + nb[3] * m * a[..., r] * Nj * T1
    K[..., 3, 3] = V * ab * T1
    emd = nb[3] * W * mass[:, None]
    for q in range(8):
        for r in range(3):
            K[:, q, q, r, r] += emd[:, q]
    off = np.array([[i, j, k] for k in range(2) for j in range(2) for i in range(2)])
    d = off[None, :, :] - off[:, None, :]
    slot = (d[..., 0] + 1) + 3 * (d[..., 1] + 1) + 9 * (d[..., 2] + 1)     # [qa][qb]
    stencil = np.zeros(27 * 16 * N)
    idx = ((slot[None, :, :, None] * 16 + np.arange(16)[None, None, None, :]) * N
           + nid[:, :, None, None])
    np.add.at(stencil, np.broadcast_to(idx, (n, 8, 8, 16)).ravel(), K.reshape(n, 8, 8, 16).ravel())
    divv = gv[:, 0, 0] + gv[:, 1, 1] + gv[:, 2, 2]
    Vn = vol[:, None]
    rhs = np.zeros((n, 8, 4))
    for r in range(3):
        rhs[..., r] = (Vn * np.einsum("nqc,nc->nq", D, dev[:, r, :]) - W * mass[:, None] * f[r]
                       - Vn * D[..., r] * pres_k[:, None] + Vn * tau2[:, None] * D[..., r] * divv[:, None])
    rhs[..., 3] = (Vn * W * divv[:, None]
                   + tau1[:, None] * mass[:, None] * np.einsum("nqc,nc->nq", D, accel_k - f)
                   + tau1[:, None] * Vn * np.einsum("nqc,nc->nq", D, gp))
    bvec = np.zeros(4 * N)
    for r in range(4):
        np.add.at(bvec, r * N + nid.ravel(), -rhs[..., r].ravel())
    bvec[:3 * N] -= (np.asarray(nmass)[None, :] * acc_k).ravel()   # AddInertialForceToRHS
    return tau1, tau2, stencil.reshape(27, 16, N), bvec


def stencil_matrix(stencil, nnc):
    """The [27][16][nodec] stencil as a scipy CSR matrix of 4 nodec rows
    (row m nodec + i, column c nodec + j for entry k = 4 m + c of the block
    between row node i and its neighbour j in slot s)."""
    import scipy.sparse as sp

    nx, ny, nz = (int(v) for v in nnc)
    N = nx * ny * nz
    st = np.asarray(stencil).reshape(27, 16, N)
    n = np.arange(N)
    i, j, k = n % nx, (n // nx) % ny, n // (nx * ny)
    rows, cols, vals = [], [], []
    for s in range(27):
        ii, jj, kk = i + s % 3 - 1, j + (s // 3) % 3 - 1, k + s // 9 - 1
        ok = (ii >= 0) & (jj >= 0) & (kk >= 0) & (ii < nx) & (jj < ny) & (kk < nz)
        col = ii + nx * (jj + ny * kk)
        for e in range(16):
            m, c = divmod(e, 4)
            v = st[s, e]
            sel = ok & (v != 0.0)
            rows.append(m * N + n[sel])
            cols.append(c * N + col[sel])
            vals.append(v[sel])
    return sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(4 * N, 4 * N))


def ns_solve(xyelem, xymin, dxy, rho, rmu, dt, beta, gamma, gravity, facl, mtol, x, mass, vol, nvel, naccel,
             nmass, bcs, max_newton=100):
    """SolveNS (module/fluid/MPM/solve_ns_mpm.cpp:28-62) with each linear
    system solved exactly (sparse direct solve): BCNRSet
    (stabilized_mpm.h:56-63: u, v, w lists set the displacement to value dt
    facl, the p list the pressure to value facl), ns_assemble, the solve on
    the rows with a diagonal above mtol that carry no BC (the scaled Krylov
    solve of the reference leaves the increment of every other row at zero),
    UpdateNRIncrement and CheckNRConvergence (solver.cpp:484-593) on the
    physical residual with the BC rows of b zeroed.  bcs: four
    (nodes, values) pairs for u, v, w, p.  Returns ndispl (3 nodec),
    npres (nodec), the Newton iterations and each iteration's residual."""
    import scipy.sparse.linalg as spl

    nnc = np.asarray(xyelem) + 1
    N = int(np.prod(nnc))
    ndispl = np.zeros(3 * N)
    npres = np.zeros(N)
    bc = np.zeros(4 * N, dtype=bool)
    for comp, (nodes, _) in enumerate(bcs):
        bc[comp * N + np.asarray(nodes, dtype=np.int64)] = True
    r0r = 0.0
    hist = []
    for it in range(max_newton):
        for comp in range(3):
            nodes, vals = bcs[comp]
            ndispl[comp * N + np.asarray(nodes, dtype=np.int64)] = np.asarray(vals) * dt * facl
        nodes, vals = bcs[3]
        npres[np.asarray(nodes, dtype=np.int64)] = np.asarray(vals) * facl
        _, _, st, b = ns_assemble(xyelem, xymin, dxy, rho, rmu, dt, beta, gamma, gravity, facl, mtol, x, mass, vol,
                                  nvel, naccel, ndispl, npres, nmass)
        A = stencil_matrix(st, nnc)
        dg = np.abs(A.diagonal())
        active = dg >= mtol
        bb = np.where(bc, 0.0, b)
        free = active & ~bc
        xl = np.zeros(4 * N)
        idx = np.nonzero(free)[0]
        xl[idx] = spl.spsolve(A[idx][:, idx].tocsc(), bb[idx])
        ndispl += xl[:3 * N]
        npres += xl[3 * N:]
        Ax = A @ xl
        Ax[bc] = 0.0
        r = bb - np.where(dg > mtol, Ax, 0.0)
        rkr = float(np.sqrt(r @ r))
        idof = float(np.count_nonzero(dg > mtol))
        rabs = 0.0 if idof <= 1e-30 else float(np.sqrt((r @ r) / idof))
        hist.append(rkr)
        if it == 0:
            r0r = rkr
        rref = rkr / r0r if r0r > 1e-30 else 0.0
        if rref < 1e-6 or r0r < 1e-6 or rabs < 1e-8:
            break
    return ndispl, npres, it + 1, np.array(hist)


# ---------------------------------------------------------------- time step
def nodal_volume(xyelem, xymin, dxy, npxye):
    """MakNodalVol (module/mesh.cpp:160-202) for linear shape functions: every
    element's npxye Gaussian points (GaussianDistribution, mesh.cpp:12-52) add
    N volp to their nodes; the sum factorises over the axes."""
    xyelem = np.asarray(xyelem)
    nnc = xyelem + 1
    offs = {1: [0.0], 2: [-0.25, 0.25], 3: [-1.0 / 3.0, 0.0, 1.0 / 3.0], 4: [-0.375, -0.125, 0.125, 0.375],
            5: [-0.4, -0.2, 0.0, 0.2, 0.4], 6: [-5 / 12, -3 / 12, -1 / 12, 1 / 12, 3 / 12, 5 / 12]}
    w = []
    for d in range(3):
        s = np.zeros(nnc[d])
        for e in range(xyelem[d]):
            xe = xymin[d] + dxy[d] * (e + 0.5)
            for o in offs.get(int(npxye[d]), [0.0] * int(npxye[d])):
                xp = xe + o * dxy[d]
                for k in range(2):
                    s[e + k] += 1.0 - abs(xp - (xymin[d] + dxy[d] * (e + k))) / dxy[d]
        w.append(s)
    volp = float(np.prod(dxy)) / float(np.prod(npxye))
    return (w[0][None, None, :] * w[1][None, :, None] * w[2][:, None, None]).ravel() * volp


def _cells(x, xyelem, xymin, dxy):
    """The element of each point (the last element holds the upper wall, as MeshPointLinklist)."""
    c = np.floor((x - np.asarray(xymin)) / np.asarray(dxy)).astype(np.int64)
    return np.minimum(np.maximum(c, 0), np.asarray(xyelem) - 1)


def ns_p2g(xyelem, xymin, dxy, mtol, facl, x, mass, vol, vel, accel, bcs):
    """StabilizedMPM::Particle2Node (module/fluid/MPM/var_trans_fluid.cpp:17-80)
    for PIC / FLIP: nmass, nvof, nmome = sum N m v, nforce = sum N m a
    (StandardVarP2G, VelP2G, AccelP2G), nvel = nmome / nmass and
    naccel = nforce / nmass where nmass > mtol, then BCSetVal (value facl) on
    nvel and BCSetZero on naccel for the u, v, w lists.  Returns nmass, nvof,
    nvel, naccel (component-major)."""
    nnc = np.asarray(xyelem) + 1
    N = int(np.prod(nnc))
    W, _, nid = _shape(x, xymin, dxy, _cells(x, xyelem, xymin, dxy), nnc)
    nmass = np.zeros(N)
    nvof = np.zeros(N)
    nmome = np.zeros(3 * N)
    nforce = np.zeros(3 * N)
    np.add.at(nmass, nid, W * mass[:, None])
    np.add.at(nvof, nid, W * vol[:, None])
    for c in range(3):
        np.add.at(nmome, c * N + nid, W * (mass * vel[:, c])[:, None])
        np.add.at(nforce, c * N + nid, W * (mass * accel[:, c])[:, None])
    ok = nmass > mtol
    nvel = np.zeros(3 * N)
    naccel = np.zeros(3 * N)
    for c in range(3):
        nvel[c * N:(c + 1) * N][ok] = nmome[c * N:(c + 1) * N][ok] / nmass[ok]
        naccel[c * N:(c + 1) * N][ok] = nforce[c * N:(c + 1) * N][ok] / nmass[ok]
    for c in range(3):
        nodes, vals = bcs[c]
        nodes = np.asarray(nodes, dtype=np.int64)
        nvel[c * N + nodes] = np.asarray(vals) * facl
        naccel[c * N + nodes] = 0.0
    return nmass, nvof, nvel, naccel


def ns_g2p(xyelem, xymin, dxy, dt, beta, gamma, mtol, scheme, x, vol, vel, accel, nvel, naccel, ndispl, npres, nvof,
           nvol):
    """StabilizedMPM::Node2Particle (var_trans_fluid.cpp:82-135) for PIC (0) and
    FLIP (1): PredictNewmarkBetaVelAndAccel + CommitNodalKinematics
    (module/nonlinear_time_integration.cpp:58-77), the pressure, displacement,
    acceleration and (PIC) velocity gathers, DeltaCorrectionParticleShifting
    (module/material_point.cpp:174-228, at the positions of the step's start)
    and CommitParticleKinematics (nonlinear_time_integration.cpp:79-96).
    Returns x, vel, accel (n, 3) and pres (n)."""
    nnc = np.asarray(xyelem) + 1
    N = int(np.prod(nnc))
    nb = newmark(dt, beta, gamma)
    nvel_k = nb[0] * ndispl - nb[1] * nvel - nb[2] * naccel
    naccel_k = nb[3] * ndispl - nb[4] * nvel - nb[5] * naccel
    W, D, nid = _shape(x, xymin, dxy, _cells(x, xyelem, xymin, dxy), nnc)
    pres = (W * npres[nid]).sum(axis=1)
    disp = np.stack([(W * ndispl[c * N + nid]).sum(axis=1) for c in range(3)], axis=1)
    acc = np.stack([(W * naccel_k[c * N + nid]).sum(axis=1) for c in range(3)], axis=1)
    if scheme == 1:
        v = vel + dt * ((1.0 - gamma) * accel + gamma * acc)
    else:
        v = np.stack([(W * nvel_k[c * N + nid]).sum(axis=1) for c in range(3)], axis=1)
    nei = np.maximum(0.0, -nvol + nvof)
    eu = float((nei * nei).sum())
    geup = (D * nei[nid][:, :, None]).sum(axis=1) * (2.0 * vol)[:, None]
    gd = float((geup * geup).sum())
    b0 = 0.0 if gd < mtol else eu / gd
    return x + disp - b0 * geup, v, acc, pres


def ns_step(xyelem, xymin, dxy, npxye, rho, rmu, dt, beta, gamma, gravity, facl, mtol, scheme, x, mass, vol, vel,
            accel, bcs, nsteps=1):
    """nsteps time steps of work/src_fluid/MPM/main.cpp:45-68 (Particle2Node,
    SolveNS with exact linear solves, Node2Particle).  Returns the nodal
    fields of the first Particle2Node and the particle state (x, v, a, pres)."""
    nvol = nodal_volume(xyelem, xymin, dxy, npxye)
    first = None
    pres = np.zeros(len(mass))
    for _ in range(nsteps):
        nmass, nvof, nvel, naccel = ns_p2g(xyelem, xymin, dxy, mtol, facl, x, mass, vol, vel, accel, bcs)
        if first is None:
            first = dict(nmass=nmass, nvof=nvof, nvel=nvel, naccel=naccel)
        nd, npres, _, _ = ns_solve(xyelem, xymin, dxy, rho, rmu, dt, beta, gamma, gravity, facl, mtol, x, mass, vol,
                                   nvel, naccel, nmass, bcs)
        x, vel, accel, pres = ns_g2p(xyelem, xymin, dxy, dt, beta, gamma, mtol, scheme, x, vol, vel, accel, nvel,
                                     naccel, nd, npres, nvof, nvol)
    return first, dict(x=x, v=vel, a=accel, pres=pres)
