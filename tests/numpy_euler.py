"""Independent numpy restatement of the reference's 3D Euler sample
(sample/3d_hllc/3d_hllc.fmr:30-216): MUSCL-Hancock with the TVD slope
limiter, HLLC fluxes in x, y and z (the y and z fluxes through the YZX / ZXY
cycles of the momentum), and the update U - dt*div(F, G, H).

Test infrastructure only.  It is written from the .fmr text, not from this
repository's generator: no import of formura_gb300.generator, no Orthotope
Machine, no manifest rules.  Each expression keeps the program's operation
order (left-associative, as written), so every value is rounded the same way
as in the C that Formura emits for the program; constants follow the
program's definitions, evaluated in binary64 in the program's order, as
the emitted C does.

Positions: a value at the half-integer position q + 1/2 along an axis is
stored at index q (the face between cells q and q + 1); the grid is periodic.
"""
from __future__ import annotations

from fractions import Fraction

import numpy as np


def _min(a, b):                      # min = fun(a, b) if a > b then b else a
    return np.where(a > b, b, a)


def _max(a, b):                      # max = fun(a, b) if a > b then a else b
    return np.where(a > b, a, b)


def _fwd(a, ax):                     # value one cell ahead along ax
    return np.roll(a, -1, ax)


def _bwd(a, ax):                     # value one cell behind along ax
    return np.roll(a, 1, ax)


# momentum cycles (3d_hllc.fmr:43-44, 137-149): the flux along y sees
# (v, w, u), along z (w, u, v); the inverse is the cycle applied twice
CYCLES = {0: lambda m: m, 1: lambda m: (m[1], m[2], m[0]), 2: lambda m: (m[2], m[0], m[1])}


def _inv(ax):
    c = CYCLES[ax]
    return lambda m: c(c(m))


class Euler3D:
    """Constants of 3d_hllc.fmr:22-28 (gamma 7/5, beta 1, max_signal_speed
    4) with the Courant number and box of the run.  Formura folds no
    constant expression: dt = C_cfl*min3(dx,dy,dz)/max_signal_speed and
    gamma1 = gamma - 1.0 are evaluated in binary64 in the emitted C, in that
    order, with dx = length/N the rational rounded once."""

    def __init__(self, shape, length, c_cfl=0.8, gamma=7.0 / 5.0, beta=1.0, max_signal_speed=4.0):
        self.dx = [float(Fraction(str(l)) / n) for l, n in zip(length, shape)]
        mn = _min(np.float64(self.dx[0]), np.float64(self.dx[1]))
        mn = _min(mn, np.float64(self.dx[2]))
        self.dt = float((c_cfl * mn) / max_signal_speed)
        self.half_dt = 0.5 * self.dt
        self.gamma = gamma
        self.gamma1 = gamma - 1.0
        self.beta = beta

    # -- 3d_hllc.fmr:70-80 --------------------------------------------------
    def primitive(self, rho, m, e):
        V = tuple(mi / rho for mi in m)
        norm2 = (V[0] * V[0] + V[1] * V[1]) + V[2] * V[2]
        p = self.gamma1 * (e - (0.5 * rho) * norm2)
        return V, p

    @staticmethod
    def flux_x(rho, V, p, e):
        u = V[0]
        fm = ((rho * V[0]) * u + p, (rho * V[1]) * u + 0.0, (rho * V[2]) * u + 0.0)
        return rho * u, fm, (e + p) * u

    # -- 3d_hllc.fmr:162-172 ------------------------------------------------
    def flux_from_u(self, U, ax):
        rho, m, e = U
        V, p = self.primitive(rho, CYCLES[ax](m), e)
        fr, fm, fe = self.flux_x(rho, V, p, e)
        return fr, _inv(ax)(fm), fe

    # -- 3d_hllc.fmr:82-86, 97-118 -------------------------------------------
    def hllc(self, UL, UR, ax):
        rho_L, mL, e_L = UL
        rho_R, mR, e_R = UR
        mL, mR = CYCLES[ax](mL), CYCLES[ax](mR)
        V_L, p_L = self.primitive(rho_L, mL, e_L)
        V_R, p_R = self.primitive(rho_R, mR, e_R)
        u_L, u_R = V_L[0], V_R[0]
        c_f = _max(np.sqrt(self.gamma * p_L / rho_L), np.sqrt(self.gamma * p_R / rho_R))
        S_L = _min(u_L, u_R) - c_f
        S_R = _max(u_L, u_R) + c_f
        den = rho_L * (S_L - u_L) - rho_R * (S_R - u_R)
        S_M = ((p_R - p_L) + (rho_L * u_L) * (S_L - u_L) - (rho_R * u_R) * (S_R - u_R)) / den
        p_st = ((rho_L * p_R) * (S_L - u_L) - (rho_R * p_L) * (S_R - u_R)
                + (((rho_L * rho_R) * (S_R - u_R)) * (S_L - u_L)) * (u_L - u_R)) / den

        def star(S, rho, V, e, p):
            u = V[0]
            rho_st = rho * (S - u) / (S - S_M)
            V_st = (S_M, V[1], V[2])
            e_st = (((S - u) * e - p * u) + p_st * S_M) / (S - S_M)
            return rho_st, tuple(rho_st * v for v in V_st), e_st

        UstL = star(S_L, rho_L, V_L, e_L, p_L)
        UstR = star(S_R, rho_R, V_R, e_R, p_R)
        FL = self.flux_x(rho_L, V_L, p_L, e_L)
        FR = self.flux_x(rho_R, V_R, p_R, e_R)
        aL, aR = _min(S_L, 0.0), _max(S_R, 0.0)

        def comb(fl, fr_, sl, sr, ul, ur):
            return np.where(S_M > 0, fl + aL * (sl - ul), fr_ + aR * (sr - ur))

        Frho = comb(FL[0], FR[0], UstL[0], UstR[0], rho_L, rho_R)
        Fm = tuple(comb(FL[1][i], FR[1][i], UstL[1][i], UstR[1][i], mL[i], mR[i]) for i in range(3))
        Fe = comb(FL[2], FR[2], UstL[2], UstR[2], e_L, e_R)
        return Frho, _inv(ax)(Fm), Fe

    # -- 3d_hllc.fmr:151-158 --------------------------------------------------
    def tvd_muscl(self, q, ax):
        dq = _fwd(q, ax) - q                    # DU at q + 1/2
        ob, of = _bwd(dq, ax), dq               # DU at q - 1/2 and q + 1/2
        dp = _max(_max(0.0, _min(self.beta * ob, of)), _min(ob, self.beta * of))
        dn = _min(_min(0.0, _max(self.beta * ob, of)), _max(ob, self.beta * of))
        delta = np.where(of > 0, dp, dn)
        return q + 0.5 * delta, q - 0.5 * delta     # (UR, UL)

    # -- 3d_hllc.fmr:178-201, 203-216 -----------------------------------------
    def step(self, rho, m, e):
        """One step from (rho, (rhou, rhov, rhow), e); returns the same tuple."""
        comps = [rho, m[0], m[1], m[2], e]

        def pack(c):
            return c[0], (c[1], c[2], c[3]), c[4]

        def unpack(U):
            return [U[0], U[1][0], U[1][1], U[1][2], U[2]]

        URs, ULs = [], []
        for ax in range(3):
            ur, ul = zip(*(self.tvd_muscl(c, ax) for c in comps))
            URs.append(list(ur))
            ULs.append(list(ul))
        div = None
        for ax in range(3):
            FL = unpack(self.flux_from_u(pack(ULs[ax]), ax))
            FR = unpack(self.flux_from_u(pack(URs[ax]), ax))
            t = [(r - l) / self.dx[ax] for r, l in zip(FR, FL)]
            div = t if div is None else [a + b for a, b in zip(div, t)]
        fluxes = []
        for ax in range(3):
            ulbar = [u - self.half_dt * d for u, d in zip(ULs[ax], div)]
            urbar = [u - self.half_dt * d for u, d in zip(URs[ax], div)]
            U_L = urbar                                  # at q + 1/2: URbar(q)
            U_R = [_fwd(u, ax) for u in ulbar]           # ULbar(q + 1)
            fluxes.append(unpack(self.hllc(pack(U_L), pack(U_R), ax)))
        total = None
        for ax in range(3):
            t = [(f - _bwd(f, ax)) / self.dx[ax] for f in fluxes[ax]]
            total = t if total is None else [a + b for a, b in zip(total, t)]
        out = [u - self.dt * d for u, d in zip(comps, total)]
        return out[0], (out[1], out[2], out[3]), out[4]
