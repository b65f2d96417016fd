"""Pure-torch FP64 D3Q19 step used as an autograd checker for the adjoint.

TEST INFRASTRUCTURE ONLY.  Pull streaming with halfway bounce-back and
periodic wrap, Zou-He velocity inlet on face 1X (per-site u_x) and density
outlet on face X1, TRT, BGK or regularized collision with forcing -- the
physics of jyulb/isothermal.pyx:1112-1326 and jyulb/D3Q19.pyx:655-940 -- written with
differentiable tensor operations so that torch autograd yields reference
gradients of the plane-velocity loss.
"""
from __future__ import annotations

import numpy as np
import torch

CI = [-1, -1, -1, -1, -1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 1]
CJ = [-1, 0, 0, 0, 1, -1, -1, -1, 0, 0, 0, 1, 1, 1, -1, 0, 0, 0, 1]
CK = [0, -1, 0, 1, 0, -1, 0, 1, -1, 0, 1, -1, 0, 1, 0, -1, 0, 1, 0]
NNZ = [abs(a) + abs(b) + abs(c) for a, b, c in zip(CI, CJ, CK)]
W = [1 / 3 if n == 0 else (1 / 18 if n == 1 else 1 / 36) for n in NNZ]


def solid_source(phase, periodic, zsym=False):
    """(19, nx, ny, nz) bool: the upstream site x - c_q is solid (sites
    outside a non-periodic face count as solid; across a symmetric z face the
    upstream site is the mirror image of the boundary layer's)."""
    nx, ny, nz = phase.shape
    I, J, K = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing='ij')
    out = np.zeros((19, nx, ny, nz), bool)
    for q in range(19):
        bad = np.zeros(phase.shape, bool)
        src = []
        for ax, (c, n, X) in enumerate(zip((CI[q], CJ[q], CK[q]), (nx, ny, nz), (I, J, K))):
            s = X - c
            if ax == 2 and zsym:
                s = np.clip(s, 0, n - 1)  # the halo mirrors the adjacent layer
            elif periodic[ax]:
                s = s % n
            else:
                bad |= (s < 0) | (s >= n)
                s = np.clip(s, 0, n - 1)
            src.append(s)
        out[q] = bad | (phase[src[0], src[1], src[2]] == 0)
    return torch.from_numpy(out)


def _zmirror(q):
    return next(p for p in range(19) if (CI[p], CJ[p], CK[p]) == (CI[q], CJ[q], -CK[q]))


def stream(f, solid, zsym=False):
    g = []
    for q in range(19):
        moved = torch.roll(f[q], shifts=(CI[q], CJ[q], CK[q]), dims=(0, 1, 2))
        if zsym and CK[q] != 0:
            # pulled across a symmetric z face: the mirrored population of the
            # mirrored (boundary-layer) site
            mir = torch.roll(f[_zmirror(q)], shifts=(CI[q], CJ[q], 0), dims=(0, 1, 2))
            plane = 0 if CK[q] > 0 else -1
            moved = moved.clone()
            moved[:, :, plane] = mir[:, :, plane]
        g.append(torch.where(solid[q], f[18 - q], moved))
    return torch.stack(g)


def zh_plane(gp, face, jx, jy, jz):
    """Zou-He unknowns on a face plane (jyulb/bcs.pyx:487-562), gp: list of 19 (ny,nz)."""
    g = list(gp)
    if face == 0:
        t = g[11] + g[12] + g[13] - g[5] - g[6] - g[7]
        u = g[7] + g[10] + g[13] - g[5] - g[8] - g[11]
        g[14] = g[4] + jx / 6 + 0.5 * t - 0.5 * jy
        g[18] = g[0] + jx / 6 - 0.5 * t + 0.5 * jy
        g[15] = g[3] + jx / 6 + 0.5 * u - 0.5 * jz
        g[17] = g[1] + jx / 6 - 0.5 * u + 0.5 * jz
        g[16] = g[2] + jx / 3
    else:
        t = g[11] + g[12] + g[13] - g[5] - g[6] - g[7]
        u = g[7] + g[10] + g[13] - g[5] - g[8] - g[11]
        g[0] = g[18] - jx / 6 + 0.5 * t - 0.5 * jy
        g[4] = g[14] - jx / 6 - 0.5 * t + 0.5 * jy
        g[1] = g[17] - jx / 6 + 0.5 * u - 0.5 * jz
        g[3] = g[15] - jx / 6 - 0.5 * u + 0.5 * jz
        g[2] = g[16] - jx / 3
    return g


def apply_zou_he(g, uin, rho_out):
    zero = [q for q in range(19) if CI[q] == 0]
    # inlet 1X: fixed velocity (uin, 0, 0)
    p = [g[q][0] for q in range(19)]
    S = sum(p[q] for q in zero) + 2 * sum(p[q] for q in range(19) if CI[q] == -1)
    rho_bc = S / (1.0 - uin)
    p = zh_plane(p, 0, rho_bc * uin, torch.zeros_like(uin), torch.zeros_like(uin))
    # outlet X1: fixed density, zero tangential velocity
    o = [g[q][-1] for q in range(19)]
    S = sum(o[q] for q in zero) + 2 * sum(o[q] for q in range(19) if CI[q] == 1)
    z = torch.zeros_like(S)
    o = zh_plane(o, 1, S - rho_out, z, z)
    out = []
    for q in range(19):
        out.append(torch.cat([p[q][None], g[q][1:-1], o[q][None]], dim=0))
    return torch.stack(out)


def collide(g, a, we, wo):
    C = torch.tensor([CI, CJ, CK], dtype=g.dtype, device=g.device)  # (3,19)
    w = torch.tensor(W, dtype=g.dtype, device=g.device)
    rho = g.sum(0)
    j = torch.einsum('aq,qxyz->axyz', C, g)
    u = j / rho + 0.5 * a[:, None, None, None]
    s = rho * u
    c1, c2 = 1 - 0.5 * wo, 1 - 0.5 * we
    c3, c4 = 1 - 0.5 * (we + wo), 0.5 * (we - wo)
    H0 = we * rho
    H1 = wo * s + c1 * rho * a[:, None, None, None]
    H2 = we * torch.einsum('axyz,bxyz->abxyz', s, s) / rho + c2 * (
        torch.einsum('a,bxyz->abxyz', a, s) + torch.einsum('b,axyz->abxyz', a, s))
    cc = torch.einsum('aq,bq->abq', C, C) - torch.eye(3, dtype=g.dtype, device=g.device)[:, :, None] / 3
    P = w[:, None, None, None] * (H0[None] + 3 * torch.einsum('aq,axyz->qxyz', C, H1)
                                  + 4.5 * torch.einsum('abq,abxyz->qxyz', cc, H2))
    opp = torch.arange(18, -1, -1)
    relax = c3 * g - c4 * g[opp]
    relax = torch.cat([relax[:9], ((1 - we) * g[9])[None], relax[10:]])
    return relax + P, rho, u


def collide_reg(g, a, we):
    """Regularized collision (jyulb/D3Q19.pyx:859-940): f* = P(H) with H0 = rho,
    H1 = j + rho a, H2 = (1 - we)(Pi - rho I/3) + we s s / rho + c2 (a s + s a)."""
    C = torch.tensor([CI, CJ, CK], dtype=g.dtype, device=g.device)
    w = torch.tensor(W, dtype=g.dtype, device=g.device)
    rho = g.sum(0)
    j = torch.einsum('aq,qxyz->axyz', C, g)
    Pi = torch.einsum('aq,bq,qxyz->abxyz', C, C, g)
    ab = a[:, None, None, None]
    s = j + 0.5 * rho * ab
    u = s / rho
    c2 = 1 - 0.5 * we
    eye = torch.eye(3, dtype=g.dtype, device=g.device)
    H0 = rho
    H1 = j + rho * ab
    H2 = (1 - we) * (Pi - eye[:, :, None, None, None] * rho / 3) + we * torch.einsum('axyz,bxyz->abxyz', s, s) / rho \
        + c2 * (torch.einsum('a,bxyz->abxyz', a, s) + torch.einsum('b,axyz->abxyz', a, s))
    cc = torch.einsum('aq,bq->abq', C, C) - eye[:, :, None] / 3
    f = w[:, None, None, None] * (H0[None] + 3 * torch.einsum('aq,axyz->qxyz', C, H1)
                                  + 4.5 * torch.einsum('abq,abxyz->qxyz', cc, H2))
    return f, rho, u


def run(phase, tau, g, uin, steps, magic=None, scheme='TRT', rho_out=1.0, periodic=(False, False, True),
        zsym=False):
    """Returns the stored velocity of the last step, (3, nx, ny, nz).  zsym:
    both z faces symmetric."""
    solid = solid_source(phase, periodic, zsym)
    fluid = torch.from_numpy(phase != 0)
    we = 1.0 / tau
    if scheme == 'TRT':
        wo = 1.0 / (magic / (tau - 0.5) + 0.5) if magic else 8.0 * (2.0 - we) / (8.0 - we)
    else:
        wo = we
    w = torch.tensor(W, dtype=torch.float64)
    f = w[:, None, None, None].expand(19, *phase.shape).clone()
    u = None
    for _ in range(steps):
        gs = stream(f, solid, zsym)
        gs = apply_zou_he(gs, uin, rho_out)
        f, rho, u = collide_reg(gs, g, we) if scheme == 'REG' else collide(gs, g, we, wo)
        f = torch.where(fluid[None], f, w[:, None, None, None].expand_as(f))
    return u


# ---------------------------------------------------------------------------
# General form: Zou-He data on any fixed face from den / vel node fields (as
# Solver.evolve reads them, jyulb/isothermal.pyx:476-502), and moving solids
# with Ladd's term 6 w_q rho_prev (c_q . u_wall) (jyulb/isothermal.pyx:1112-1248)
# ---------------------------------------------------------------------------
WALL, PERIODIC, FIXED_DEN, FIXED_VEL = 0, 1, 2, 3
CAX = (CI, CJ, CK)


def zh_assign(g, fc, jx, jy, jz):
    """Zou-He unknowns of face fc (0..5 = 1X, X1, 1Y, Y1, 1Z, Z1) from the
    known populations and the boundary momentum (jyulb/bcs.pyx:487-716);
    g: list of 19 plane tensors, returned updated."""
    g = list(g)
    s6, s3, h = 1.0 / 6.0, 1.0 / 3.0, 0.5
    if fc == 0:
        t = g[11] + g[12] + g[13] - g[5] - g[6] - g[7]
        g[14] = g[4] + s6 * jx + h * t - h * jy
        g[18] = g[0] + s6 * jx - h * t + h * jy
        t = g[7] + g[10] + g[13] - g[5] - g[8] - g[11]
        g[15] = g[3] + s6 * jx + h * t - h * jz
        g[17] = g[1] + s6 * jx - h * t + h * jz
        g[16] = g[2] + s3 * jx
    elif fc == 1:
        t = g[11] + g[12] + g[13] - g[5] - g[6] - g[7]
        g[0] = g[18] - s6 * jx + h * t - h * jy
        g[4] = g[14] - s6 * jx - h * t + h * jy
        t = g[7] + g[10] + g[13] - g[5] - g[8] - g[11]
        g[1] = g[17] - s6 * jx + h * t - h * jz
        g[3] = g[15] - s6 * jx - h * t + h * jz
        g[2] = g[16] - s3 * jx
    elif fc == 2:
        t = g[15] + g[16] + g[17] - g[1] - g[2] - g[3]
        g[4] = g[14] + s6 * jy + h * t - h * jx
        g[18] = g[0] + s6 * jy - h * t + h * jx
        t = g[17] + g[10] + g[3] - g[15] - g[8] - g[1]
        g[11] = g[7] + s6 * jy + h * t - h * jz
        g[13] = g[5] + s6 * jy - h * t + h * jz
        g[12] = g[6] + s3 * jy
    elif fc == 3:
        t = g[15] + g[16] + g[17] - g[1] - g[2] - g[3]
        g[0] = g[18] - s6 * jy + h * t - h * jx
        g[14] = g[4] - s6 * jy - h * t + h * jx
        t = g[17] + g[10] + g[3] - g[15] - g[8] - g[1]
        g[5] = g[13] - s6 * jy + h * t - h * jz
        g[7] = g[11] - s6 * jy - h * t + h * jz
        g[6] = g[12] - s3 * jy
    elif fc == 4:
        t = g[18] + g[16] + g[14] - g[4] - g[2] - g[0]
        g[3] = g[15] + s6 * jz + h * t - h * jx
        g[17] = g[1] + s6 * jz - h * t + h * jx
        t = g[18] + g[12] + g[4] - g[14] - g[6] - g[0]
        g[7] = g[11] + s6 * jz + h * t - h * jy
        g[13] = g[5] + s6 * jz - h * t + h * jy
        g[10] = g[8] + s3 * jz
    else:
        t = g[18] + g[16] + g[14] - g[4] - g[2] - g[0]
        g[1] = g[17] - s6 * jz + h * t - h * jx
        g[15] = g[3] - s6 * jz - h * t + h * jx
        t = g[18] + g[12] + g[4] - g[14] - g[6] - g[0]
        g[5] = g[13] - s6 * jz + h * t - h * jy
        g[11] = g[7] - s6 * jz - h * t + h * jy
        g[8] = g[10] - s3 * jz
    return g


def refreshed_faces(bc):
    """Faces whose data the solver reads from den / vel: the fixed faces; Z1
    only when bc[Z1] is FIXED_DEN or bc[1Z] is FIXED_VEL
    (jyulb/isothermal.pyx:500)."""
    out = set()
    for f in range(6):
        r = bc[f] in (FIXED_DEN, FIXED_VEL)
        if f == 5:
            r = bc[5] == FIXED_DEN or bc[4] == FIXED_VEL
        if r:
            out.add(f)
    return out


def apply_faces(g, bc, den, vel):
    """Zou-He on every fixed face in face order; den (nx,ny,nz), vel
    (nx,ny,nz,3) tensors give the face data."""
    ref = refreshed_faces(bc)
    for fc in range(6):
        if bc[fc] not in (FIXED_DEN, FIXED_VEL):
            continue
        ax, high = fc >> 1, fc & 1
        idx = [slice(None)] * 3
        idx[ax] = -1 if high else 0
        idx = tuple(idx)
        p = [g[q][idx] for q in range(19)]
        if fc in ref:
            d = den[idx]
            v = [vel[idx + (c,)] for c in range(3)]
        else:
            d = torch.ones_like(p[0])
            v = [torch.zeros_like(p[0])] * 3
        leaving = 1 if high else -1  # normal component of the known outgoing populations
        S = sum(p[q] for q in range(19) if CAX[ax][q] == 0) + 2 * sum(p[q] for q in range(19)
                                                                   if CAX[ax][q] == leaving)
        if bc[fc] == FIXED_VEL:
            rho = S / (1.0 + v[ax]) if high else S / (1.0 - v[ax])
            j = [rho * v[c] for c in range(3)]
        else:
            j = [d * v[c] for c in range(3)]
            j[ax] = (S - d) if high else (d - S)
        p = zh_assign(p, fc, *j)
        g = g.clone()
        for q in range(19):
            g[q][idx] = p[q]
    return g


def moving_links(phase, solid_vel, periodic):
    """(19, nx, ny, nz): c_q . u_wall of the solid upstream site x - c_q inside
    the box (0 where the upstream site is fluid, outside, or immobile)."""
    nx, ny, nz = phase.shape
    I, J, K = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing='ij')
    out = np.zeros((19, nx, ny, nz))
    for q in range(19):
        inside = np.ones(phase.shape, bool)
        src = []
        for ax, (c, n, X) in enumerate(zip((CI[q], CJ[q], CK[q]), (nx, ny, nz), (I, J, K))):
            s = X - c
            if periodic[ax]:
                s = s % n
            else:
                inside &= (s >= 0) & (s < n)
                s = np.clip(s, 0, n - 1)
            src.append(s)
        u = solid_vel[src[0], src[1], src[2]]
        proj = CI[q] * u[..., 0] + CJ[q] * u[..., 1] + CK[q] * u[..., 2]
        out[q] = np.where(inside & (phase[src[0], src[1], src[2]] == 0), proj, 0.0)
    return torch.from_numpy(out)


def run_fields(phase, tau, g, den, vel, steps, bc, magic=None, scheme='TRT', solid_vel=None, f0=None):
    """The stored velocity of the last step, (3, nx, ny, nz), of a domain
    whose fixed faces read den / vel (tensors), whose solids move with
    solid_vel (nx, ny, nz, 3) (numpy, or None), and whose first step takes
    den as the previous-step density of Ladd's term.  It starts from the
    post-collision populations f0 (19, nx, ny, nz), else from rest; next to a
    moving solid the solver's initial state is not rest (its velocity-gradient
    term sees the wall velocity), so f0 comes from the solver's own set-up."""
    periodic = tuple(bc[2 * a] == PERIODIC for a in range(3))
    solid = solid_source(phase, periodic)
    lw = moving_links(phase, solid_vel, periodic) if solid_vel is not None else None
    fluid = torch.from_numpy(phase != 0)
    we = 1.0 / tau
    if scheme == 'TRT':
        wo = 1.0 / (magic / (tau - 0.5) + 0.5) if magic else 8.0 * (2.0 - we) / (8.0 - we)
    else:
        wo = we
    w = torch.tensor(W, dtype=torch.float64)
    f = torch.as_tensor(f0, dtype=torch.float64).clone() if f0 is not None else \
        w[:, None, None, None].expand(19, *phase.shape).clone()
    # the first step's previous-step density comes from den, as Solver.evolve
    # reads it
    rho_prev = den if den is not None else torch.ones(phase.shape, dtype=torch.float64)
    u = None
    for _ in range(steps):
        gs = stream(f, solid)
        if lw is not None:
            ladd = torch.stack([6.0 * W[q] * rho_prev * lw[q] for q in range(19)])
            gs = gs + torch.where(solid, ladd, torch.zeros_like(ladd))
        gs = apply_faces(gs, bc, den, vel)
        f, rho, u = collide_reg(gs, g, we) if scheme == 'REG' else collide(gs, g, we, wo)
        rho_prev = rho
        f = torch.where(fluid[None], f, w[:, None, None, None].expand_as(f))
    return u
