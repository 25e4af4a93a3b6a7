"""FP64 PyTorch transcription of the scheme for one block (test infrastructure).

TEST INFRASTRUCTURE ONLY: the checker of the hand-written reverse kernels.  Torch
autograd through this transcription gives the reference gradient that
``pyhype_gb300.adjoint`` must reproduce; the product never imports it.

It restates the residual and RK stepping of the reference's FP64 path for a single
block whose sides are Reflection, OutletDirichlet or copy sides (no inter-block
halos), Roe, HLLL or HLLE flux, any of the four limiters, conservative or primitive
reconstruction, in the reference's operation order so that every value (and hence
every min/max/branch selection) equals the CUDA path's:

    ghosts + reflection           pyhype/blocks/ghost.py:149-216, boundary_conditions/funcs.py:28-43
    interface averages            pyhype/blocks/quad_block.py:181-218
    Green-Gauss gradient          pyhype/gradients/greengauss.py:110-155
    high-order term               pyhype/blocks/base.py:261-289
    limiter                       pyhype/limiters/base.py:47-221, limiters/limiters.py:25-62
    face / boundary states        pyhype/fvm/SecondOrderMUSCL.py:106-126, fvm/base.py:255-325
    Roe flux + Harten fix         pyhype/flux/Roe.py:175-304, flux/base.py:119-146,
                                  flux/eigen_system.py:150-252, states/primitive.py:223-320
    HLLL / HLLE                   pyhype/flux/HLLL.py:25-103, flux/HLLE.py:22-47 (the norm
                                  as an exactly rounded FMA chain, as numpy/OpenBLAS)
    dUdt                          pyhype/fvm/base.py:108-190
    RK stages                     pyhype/time_marching/explicit_runge_kutta.py:47-89

Selections follow the CUDA path's conventions, which are also the subgradients the
reverse kernels take: ordered comparisons treat -0.0 as below +0.0, min/max keep the
first of equal operands, ``torch.where`` routes the gradient to the selected branch.
"""
from __future__ import annotations

import numpy as np
import torch

E, W, N, S = 0, 1, 2, 3
REFLECT, OUTLET, COPY, NEIGHBOR = "Reflection", "OutletDirichlet", "copy", "neighbor"


class _Sqrt(torch.autograd.Function):
    """Correctly rounded square root (numpy's, as the reference and the GPU compute it;
    torch's vectorised CPU sqrt is off by one ulp for a few inputs)."""

    @staticmethod
    def forward(ctx, x):
        y = torch.from_numpy(np.sqrt(x.detach().cpu().numpy())).to(x.device)
        ctx.save_for_backward(y)
        return y

    @staticmethod
    def backward(ctx, g):
        (y,) = ctx.saved_tensors
        return g * (0.5 / y)


sqrt = _Sqrt.apply


def vlt(a, b):
    """a < b with -0.0 ordered below +0.0 (the CUDA path's integer-key comparison)."""
    return (a < b) | ((a == b) & torch.signbit(a) & ~torch.signbit(b))


class Geometry:
    """Geometry planes of one block as (ny, nx) / (ny, nx+1) / (ny+1, nx) tensors,
    formed with the same expressions as the device problem's planes."""

    def __init__(self, g, device="cpu"):
        t = lambda a: torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device=device)
        self.nx, self.ny = g.nx, g.ny
        self.cart = bool(g.is_cartesian)
        self.A = t(g.A)
        self.ia = t(1.0 / g.A)
        self.hx = [t(getattr(g, f"q{s}_x") - g.xc) for s in "EWNS"]
        self.hy = [t(getattr(g, f"q{s}_y") - g.yc) for s in "EWNS"]
        self.vL, self.vLC, self.vLS = t(g.v_L), t(g.v_L * (1 * g.v_cos)), t(g.v_L * (1 * g.v_sin))
        self.vc, self.vs = t(g.v_cos), t(g.v_sin)
        self.hL, self.hLC, self.hLS = t(g.h_L), t(g.h_L * (1 * g.h_cos)), t(g.h_L * (1 * g.h_sin))
        self.hc, self.hs = t(g.h_cos), t(g.h_sin)


# ---- state algebra ------------------------------------------------------------------
def cons_to_prim(U, gm1):
    rho = U[0]
    u = U[1] / rho
    v = U[2] / rho
    Ek = 0.5 * (u * u + v * v)
    ek = rho * Ek
    return torch.stack([rho, u, v, gm1 * (U[3] - ek)])


def rotate(q, c, s):
    u, v = q[1], q[2]
    return torch.stack([q[0], u * c + v * s, v * c - u * s, q[3]])


def unrotate(q, c, s):
    u, v = q[1], q[2]
    return torch.stack([q[0], u * c - v * s, v * c + u * s, q[3]])


def rotate90(q):
    return torch.stack([q[0], q[2], -q[1], q[3]])


def unrotate90(q):
    return torch.stack([q[0], -q[2], q[1], q[3]])


def reflect(q, c, s):
    r = rotate(q, c, s)
    r = torch.stack([r[0], -r[1], r[2], r[3]])
    return unrotate(r, c, s)


SLOPE_CAP = 1e30  # the slope cap of the CUDA path and the C oracle (psi is exactly 1 beyond ~1e17)


def psi(lim, s):
    if lim == "BarthJespersen":
        return torch.where(vlt(s, torch.ones_like(s)), s, torch.ones_like(s))
    if lim in ("VanAlbada", "Venkatakrishnan"):
        cap = torch.full_like(s, SLOPE_CAP)
        s = torch.where(vlt(cap, s), cap, s)
    if lim == "VanAlbada":
        s2 = s * s
        return (s2 + s) / (s2 + 1)
    if lim == "VanLeer":
        return (torch.abs(s) + s) / (s + 1)
    s2 = s * s
    return (s2 + 2 * s) / (s2 + s + 2)


# ---- Roe flux ----------------------------------------------------------------------
def roe_flux(L, R, g, gm, k):
    sqL, sqR = sqrt(L[0]), sqrt(R[0])
    inv = 1.0 / (sqL + sqR)
    Q0 = sqrt(L[0] * R[0])
    Q1 = (L[1] * sqL + R[1] * sqR) * inv
    Q2 = (L[2] * sqL + R[2] * sqR) * inv
    Q3 = (L[3] * sqL + R[3] * sqR) * inv
    aR = sqrt(g * R[3] / R[0])
    aL = sqrt(g * L[3] / L[0])
    aQ = sqrt(g * Q3 / Q0)
    Lm, Lp = Q1 - aQ, Q1 + aQ
    tp = 2 * ((R[1] - aR) - (L[1] - aL))
    tm = 2 * ((R[1] + aR) - (L[1] + aL))
    tp = torch.where(tp > 0, tp, torch.full_like(tp, 1e-8))
    tm = torch.where(tm > 0, tm, torch.full_like(tm, 1e-8))
    Lm = torch.where(torch.abs(Lm) < tp, 0.5 * ((Lm * Lm) / tp + tp), Lm)
    Lp = torch.where(torch.abs(Lp) < tm, 0.5 * ((Lp * Lp) / tm + tm), Lp)
    Ek = 0.5 * (Q1 * Q1 + Q2 * Q2)
    H = gm * Q3 / Q0 + Ek
    ua = Q1 * aQ
    ia = 1.0 / aQ
    one_a2 = ia * ia
    h = 0.5 * one_a2
    r2a = 0.5 * Q0 * ia
    d0, d1, d2, d3 = R[0] - L[0], R[1] - L[1], R[2] - L[2], R[3] - L[3]
    y0 = (-r2a) * d1 + h * d3
    y1 = d0 + (-one_a2) * d3
    y2 = d2
    y3 = r2a * d1 + h * d3
    z0, z1, z2, z3 = torch.abs(Lm) * y0, torch.abs(Q1) * y1, torch.abs(Q1) * y2, torch.abs(Lp) * y3
    r0 = (z0 + z1) + z3
    r1 = (Lm * z0 + Q1 * z1) + Lp * z3
    r2 = ((Q2 * z0 + Q2 * z1) + z2) + Q2 * z3
    r3 = (((H - ua) * z0 + Ek * z1) + Q2 * z2) + (H + ua) * z3

    def phys(Wv):
        ek = 0.5 * Wv[0] * (Wv[1] * Wv[1] + Wv[2] * Wv[2])
        ru = Wv[0] * Wv[1]
        return ru, ru * Wv[1] + Wv[3], ru * Wv[2], Wv[1] * (k * Wv[3] + ek + Wv[3])

    FL, FR = phys(L), phys(R)
    return torch.stack([0.5 * (FL[0] + FR[0]) - 0.5 * r0, 0.5 * (FL[1] + FR[1]) - 0.5 * r1,
                        0.5 * (FL[2] + FR[2]) - 0.5 * r2, 0.5 * (FL[3] + FR[3]) - 0.5 * r3])


# ---- HLLL and HLLE fluxes -------------------------------------------------------------
def _two_prod(a, b):
    """a * b = p + e exactly (Dekker's product with Veltkamp's split, float64 arrays)."""
    p = a * b
    c = 134217729.0  # 2^27 + 1
    t = c * a
    ah = t - (t - a)
    al = a - ah
    t = c * b
    bh = t - (t - b)
    bl = b - bh
    e = ((ah * bh - p) + ah * bl + al * bh) + al * bl
    return p, e


def _fma(a, b, c):
    """Correctly rounded a * b + c, elementwise: the exact product's two parts and c
    summed once with correct rounding (math.fsum)."""
    import math

    p, e = _two_prod(a, b)
    out = np.empty_like(p)
    pf, ef, cf, of = p.ravel(), e.ravel(), np.broadcast_to(c, p.shape).ravel(), out.ravel()
    for i in range(pf.size):
        of[i] = math.fsum((pf[i], ef[i], cf[i]))
    return out


class _Norm4(torch.autograd.Function):
    """numpy.linalg.norm of a 4-vector as the reference environment evaluates it (the
    square root of a sequential fused multiply-add dot product, OpenBLAS), over the
    leading dimension; derivative x / |x|, 0 at a zero vector."""

    @staticmethod
    def forward(ctx, x):
        xn = x.detach().cpu().numpy()
        r = _fma(xn[0], xn[0], np.zeros_like(xn[0]))
        for k in (1, 2, 3):
            r = _fma(xn[k], xn[k], r)
        n = torch.from_numpy(np.sqrt(r)).to(x.device)
        ctx.save_for_backward(x, n)
        return n

    @staticmethod
    def backward(ctx, g):
        x, n = ctx.saved_tensors
        safe = torch.where(n > 0, n, torch.ones_like(n))
        return torch.where(n > 0, g / safe, torch.zeros_like(n)) * x


norm4 = _Norm4.apply


def _vmax(a, b):
    """max keeping the first operand on ties (the CUDA path's selection)."""
    return torch.where(vlt(a, b), b, a)


def _vmin(a, b):
    return torch.where(vlt(b, a), b, a)


def _hll_bounds(L, R, g):
    """Roe u and a~ and the Harten-corrected bounds L+ = max(u_R + a_R, u~ + a~),
    L- = min(u_L - a_L, u~ - a~) (pyhype/flux/HLLL.py:28-37, HLLE.py:25-33)."""
    sqL, sqR = sqrt(L[0]), sqrt(R[0])
    inv = 1.0 / (sqL + sqR)
    Q0 = sqrt(L[0] * R[0])
    Q1 = (L[1] * sqL + R[1] * sqR) * inv
    Q3 = (L[3] * sqL + R[3] * sqR) * inv
    aL = sqrt(g * L[3] / L[0])
    aR = sqrt(g * R[3] / R[0])
    aQ = sqrt(g * Q3 / Q0)
    slowL, fastL = L[1] - aL, L[1] + aL
    slowR, fastR = R[1] - aR, R[1] + aR
    rs, rf = Q1 - aQ, Q1 + aQ
    tp = 2 * (slowR - slowL)
    tm = 2 * (fastR - fastL)
    tp = torch.where(tp > 0, tp, torch.full_like(tp, 1e-8))
    tm = torch.where(tm > 0, tm, torch.full_like(tm, 1e-8))
    rs = torch.where(torch.abs(rs) < tp, 0.5 * ((rs * rs) / tp + tp), rs)
    rf = torch.where(torch.abs(rf) < tm, 0.5 * ((rf * rf) / tm + tm), rf)
    return Q1, aQ, _vmax(fastR, rf), _vmin(slowL, rs)


def _cons_flux(Wv, gm1):
    """ConservativeState of a primitive state and PrimitiveState.F(U=...)
    (pyhype/states/primitive.py:203-209)."""
    ek = 0.5 * Wv[0] * (Wv[1] * Wv[1] + Wv[2] * Wv[2])
    U = torch.stack([Wv[0], Wv[0] * Wv[1], Wv[0] * Wv[2], Wv[3] / gm1 + ek])
    F = torch.stack([U[1], U[1] * Wv[1] + Wv[3], U[1] * Wv[2], Wv[1] * (U[3] + Wv[3])])
    return U, F


def hlll_flux(L, R, g, gm1):
    """FluxHLLL (pyhype/flux/HLLL.py:25-103, its JIT branch order)."""
    u, aQ, Lp, Lm = _hll_bounds(L, R, g)
    UL, FL = _cons_flux(L, gm1)
    UR, FR = _cons_flux(R, gm1)
    mid = (Lm < 0) & (Lp > 0)
    # the middle branch with its denominators made safe where it is not taken (the
    # gradient of an unselected torch.where branch must stay finite)
    Lms = torch.where(mid, Lm, -torch.ones_like(Lm))
    Lps = torch.where(mid, Lp, torch.ones_like(Lp))
    dU = UR - UL
    r = (FR - FL) - u * dU
    kk = aQ * norm4(dU)
    den_k = torch.where(kk < 1e-16, kk + 1e-14, kk)
    alpha = _vmax(torch.zeros_like(kk), 1 - norm4(r) / den_k)
    sc = Lms * Lps * (1 - alpha * (1 - _vmax(u / Lms, u / Lps)))
    F = (Lps * FL - Lms * FR + sc * dU) / (Lps - Lms)
    return torch.where(Lm >= 0, FL, torch.where(Lp <= 0, FR, F))


def hlle_flux(L, R, g, gm1):
    """FluxHLLE (pyhype/flux/HLLE.py:22-47): F_R where L+ <= 0, else F_L where L- >= 0."""
    _, _, Lp, Lm = _hll_bounds(L, R, g)
    UL, FL = _cons_flux(L, gm1)
    UR, FR = _cons_flux(R, gm1)
    mid = (Lm < 0) & (Lp > 0)
    Lms = torch.where(mid, Lm, -torch.ones_like(Lm))
    Lps = torch.where(mid, Lp, torch.ones_like(Lp))
    F = (Lps * FL - Lms * FR + Lms * Lps * (UR - UL)) / (Lps - Lms)
    return torch.where(Lp <= 0, FR, torch.where(Lm >= 0, FL, F))


# ---- residual ------------------------------------------------------------------------
class Scheme:
    """dUdt of one block and its RK steps.  ``sides`` maps E/W/N/S to Reflection,
    OutletDirichlet or copy."""

    def __init__(self, geo: Geometry, gamma: float, gm1: float, limiter="Venkatakrishnan",
                 recon="ConservativeState", sides=None, flux="Roe"):
        self.geo = geo
        self.g, self.gm1 = gamma, gm1
        self.gm = gamma / (gamma - 1.0)
        self.k = 1.0 / (gamma - 1.0)
        self.lim = limiter
        self.prim = recon == "PrimitiveState"
        self.sides = sides or {s: REFLECT for s in "EWNS"}
        if flux not in ("Roe", "HLLL", "HLLE"):
            raise ValueError(f"flux {flux}")
        self.flux = flux

    def riemann(self, L, R):
        if self.flux == "HLLL":
            return hlll_flux(L, R, self.g, self.gm1)
        if self.flux == "HLLE":
            return hlle_flux(L, R, self.g, self.gm1)
        return roe_flux(L, R, self.g, self.gm, self.k)

    def to_recon(self, U):
        return cons_to_prim(U, self.gm1) if self.prim else U

    def recon_to_prim(self, R):
        return R if self.prim else cons_to_prim(R, self.gm1)

    def _bcs(self, side):
        G = self.geo
        if side == "E":
            return G.vc[:, -1], G.vs[:, -1]
        if side == "W":
            return G.vc[:, 0], G.vs[:, 0]
        if side == "N":
            return G.hc[-1, :], G.hs[-1, :]
        return G.hc[0, :], G.hs[0, :]

    def ghost(self, U, side, halo=None):
        """Conservative ghost values along one side (shape (4, n)); an inter-block side
        takes the neighbour's cells from ``halo``."""
        if self.sides[side] == NEIGHBOR:
            return halo[side]
        own = {"E": U[:, :, -1], "W": U[:, :, 0], "N": U[:, -1, :], "S": U[:, 0, :]}[side]
        if self.sides[side] == REFLECT:
            return reflect(own, *self._bcs(side))
        return own

    def residual(self, U, halo=None):
        """U: (4, ny, nx) conservative; returns dUdt (4, ny, nx).  ``halo`` maps the
        inter-block sides to the neighbour cells next to them (4, n)."""
        G = self.geo
        ny, nx = G.ny, G.nx
        Wr = self.to_recon(U)
        gE, gW = self.to_recon(self.ghost(U, "E", halo)), self.to_recon(self.ghost(U, "W", halo))
        gN, gS = self.to_recon(self.ghost(U, "N", halo)), self.to_recon(self.ghost(U, "S", halo))
        # padded stencil in reconstruction variables
        we = torch.cat([gW[:, :, None], Wr[:, :, :-1]], dim=2)
        ea = torch.cat([Wr[:, :, 1:], gE[:, :, None]], dim=2)
        so = torch.cat([gS[:, None, :], Wr[:, :-1, :]], dim=1)
        no = torch.cat([Wr[:, 1:, :], gN[:, None, :]], dim=1)
        LcE, LcW, LcN, LcS = G.vLC[:, 1:], G.vLC[:, :-1], G.hLC[1:, :], G.hLC[:-1, :]
        LsE, LsW, LsN, LsS = G.vLS[:, 1:], G.vLS[:, :-1], G.hLS[1:, :], G.hLS[:-1, :]
        faces = [[None] * 4 for _ in range(4)]
        for v in range(4):
            w0 = Wr[v]
            ie, iw = 0.5 * (w0 + ea[v]), 0.5 * (we[v] + w0)
            in_, is_ = 0.5 * (w0 + no[v]), 0.5 * (so[v] + w0)
            gx = (ie * LcE + iw * (-LcW) + in_ * LcN + is_ * (-LcS)) * G.ia
            gy = (ie * LsE + iw * (-LsW) + in_ * LsN + is_ * (-LsS)) * G.ia
            mx, mn = w0, w0
            for nb in (we[v], ea[v], so[v], no[v]):
                mx = torch.where(vlt(mx, nb), nb, mx)
                mn = torch.where(vlt(nb, mn), nb, mn)
            dmax, dmin = mx - w0, mn - w0
            hot, ph = [], None
            for s in range(4):
                h = gx * G.hx[s] + gy * G.hy[s]
                hot.append(h)
                davg = (w0 + h) - w0
                pos, neg = davg > 0, davg < 0
                nz = pos | neg
                q = torch.where(pos, dmax, dmin) / torch.where(nz, davg, torch.ones_like(davg))
                sl = torch.where(nz, q, torch.ones_like(q))
                p = psi(self.lim, sl)
                ph = p if s == 0 else torch.where(vlt(p, ph), p, ph)
            ph = torch.where(ph < 0, torch.zeros_like(ph), ph)
            for s in range(4):
                faces[s][v] = w0 + ph * hot[s]
        fE, fW, fN, fS = (torch.stack(faces[s]) for s in range(4))

        def to_face(q, kind, c=None, s=None):
            if kind == "v":
                q = q if G.cart else rotate(q, c, s)
            else:
                q = rotate90(q) if G.cart else rotate(q, c, s)
            return self.recon_to_prim(q)

        # interior face states
        eL = to_face(fE, "v", G.vc[:, 1:], G.vs[:, 1:])     # left state of faces 1..nx
        wR = to_face(fW, "v", G.vc[:, :-1], G.vs[:, :-1])   # right state of faces 0..nx-1
        nL = to_face(fN, "h", G.hc[1:, :], G.hs[1:, :])     # left state of faces 1..ny
        sR = to_face(fS, "h", G.hc[:-1, :], G.hs[:-1, :])   # right state of faces 0..ny-1

        # block-boundary outside states
        def outside(side, own_face, ghost_recon):
            kind = self.sides[side]
            if kind in (COPY, NEIGHBOR):
                return ghost_recon
            if kind == REFLECT:
                return reflect(own_face, *self._bcs(side))
            return own_face

        oW = to_face(outside("W", fW[:, :, 0], gW), "v", G.vc[:, 0], G.vs[:, 0])
        oE = to_face(outside("E", fE[:, :, -1], gE), "v", G.vc[:, -1], G.vs[:, -1])
        oS = to_face(outside("S", fS[:, 0, :], gS), "h", G.hc[0, :], G.hs[0, :])
        oN = to_face(outside("N", fN[:, -1, :], gN), "h", G.hc[-1, :], G.hs[-1, :])
        vLs = torch.cat([oW[:, :, None], eL], dim=2)
        vRs = torch.cat([wR, oE[:, :, None]], dim=2)
        hLs = torch.cat([oS[:, None, :], nL], dim=1)
        hRs = torch.cat([sR, oN[:, None, :]], dim=1)
        Fv = self.riemann(vLs, vRs)
        if not G.cart:
            Fv = unrotate(Fv, G.vc, G.vs)
        Fh = self.riemann(hLs, hRs)
        Fh = unrotate90(Fh) if G.cart else unrotate(Fh, G.hc, G.hs)
        Iv = G.vL * (2 * Fv)
        Ih = G.hL * (2 * Fh)
        return 0.5 * (((Iv[:, :, :-1] - Iv[:, :, 1:]) + Ih[:, :-1, :]) - Ih[:, 1:, :]) / G.A

    def step(self, U, dt, a):
        """One explicit RK step with Butcher rows a (the reference's summation order:
        each stage state is U + (dt*a0)*k0 + (dt*a1)*k1 + ..., zero terms skipped)."""
        S = len(a)
        ks = []
        Y = U
        for s in range(S):
            ks.append(self.residual(Y))
            if s + 1 < S:
                Y = U
                for q in range(s + 1):
                    if a[s][q] != 0.0:
                        Y = Y + (dt * a[s][q]) * ks[q]
        out = U
        for q in range(S):
            if a[S - 1][q] != 0.0:
                out = out + (dt * a[S - 1][q]) * ks[q]
        return out

    def side_pressure(self, U, side="N"):
        G = self.geo
        if side == "N":
            cells, L = U[:, -1, :], G.hL[-1, :]
        elif side == "S":
            cells, L = U[:, 0, :], G.hL[0, :]
        elif side == "E":
            cells, L = U[:, :, -1], G.vL[:, -1]
        else:
            cells, L = U[:, :, 0], G.vL[:, 0]
        p = cons_to_prim(cells, self.gm1)[3]
        return torch.sum(p * L)

    def objective(self, U0, dts, a, side="N"):
        """J = sum_n dt_n * P(U^{n+1}) at the given dt schedule."""
        U = U0
        J = U0.new_zeros(())
        for dt in dts:
            U = self.step(U, float(dt), a)
            J = J + float(dt) * self.side_pressure(U, side)
        return J


class MultiBlockScheme:
    """dUdt of a multiblock problem (``pyhype_gb300.problem.Problem``) with inter-block
    halos: each block's ghost row next to a neighbour is the neighbour's adjacent cells
    (pyhype/blocks/ghost.py:187-216)."""

    KIND = {0: NEIGHBOR, 1: COPY, 2: REFLECT, 3: OUTLET}

    def __init__(self, problem, gamma: float, gm1: float, limiter="Venkatakrishnan", recon="ConservativeState",
                 flux="Roe"):
        self.P = problem
        self.blocks = []
        for b in range(problem.nblocks):
            B = problem.blocks[b]
            kinds = {}
            for si, s in enumerate("EWNS"):
                k = int(B.side_kind[si])
                if k not in self.KIND:
                    raise ValueError("the transcription covers neighbour, copy, reflection and outlet sides")
                kinds[s] = self.KIND[k]
            sch = Scheme(Geometry(problem.block_geometry[b]), gamma, gm1, limiter, recon, kinds, flux)
            self.blocks.append((B.cell_offset, B.nx, B.ny, [int(B.neighbor[si]) for si in range(4)], sch))

    def residual(self, U):
        """U: (4, ncell) SoA planes; returns dUdt in the same layout."""
        views = [U[:, off:off + nx * ny].reshape(4, ny, nx) for off, nx, ny, _, _ in self.blocks]
        out = []
        for b, (off, nx, ny, nbr, sch) in enumerate(self.blocks):
            halo = {}
            for si, s in enumerate("EWNS"):
                if sch.sides[s] != NEIGHBOR:
                    continue
                V = views[nbr[si]]
                halo[s] = {"E": V[:, :, 0], "W": V[:, :, -1], "N": V[:, 0, :], "S": V[:, -1, :]}[s]
            out.append(sch.residual(views[b], halo).reshape(4, -1))
        return torch.cat(out, dim=1)
