"""Independent numpy restatement of the reference's 3D MHD sample
(sample/mhd_3d_hlld/mhd_3d_hlld.fmr:16-283): MUSCL-Hancock with the TVD
limiter, HLLD fluxes (Miyoshi-Kusano) with the GLM divergence cleaning of
the normal field (normal_B, flux_normal_B) in x, y and z through the YZX /
ZXY cycles, the update U - dt*div(F, G, H), and psi damped by
exp(-dt*c_h/c_r).

Test infrastructure only, written from the .fmr text like numpy_euler.py
(no import of formura_gb300.generator); every expression keeps the
program's operation order, and the constants are evaluated in binary64 in
the program's order, as the emitted C does.  exp comes from the C library
(math.exp), as in the emitted C.
"""
from __future__ import annotations

import math
from fractions import Fraction

import numpy as np

from numpy_euler import CYCLES, _bwd, _fwd, _inv, _max, _min


def _sign(x):                       # sign = fun(x) if x > 0 then 1 else (if x < 0 then -1 else 0)
    return np.where(x > 0, 1.0, np.where(x < 0, -1.0, 0.0))


def _cdot3(a, b):                   # cdot = fun(A, B) sum(A*B)
    return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]


class MHD3D:
    """Constants of mhd_3d_hlld.fmr:25-34."""

    def __init__(self, shape, length, c_cfl=0.3, max_signal_speed=3.0, gamma=5.0 / 3.0, c_r=0.18,
                 epsilon=1.0e-40, beta=1.0):
        self.dx = [float(Fraction(str(l)) / n) for l, n in zip(length, shape)]
        mn = _min(np.float64(self.dx[0]), np.float64(self.dx[1]))
        mn = _min(mn, np.float64(self.dx[2]))
        self.dt = float((c_cfl * mn) / max_signal_speed)
        self.half_dt = 0.5 * self.dt
        self.gamma = gamma
        self.gamma1 = gamma - 1.0
        self.c_h = max_signal_speed
        self.c_r = c_r
        self.eps = epsilon
        self.beta = beta
        self.damp = math.exp(((-self.dt) * self.c_h) / self.c_r)

    # -- mhd_3d_hlld.fmr:84-98 -------------------------------------------------
    def primitive(self, rho, m, bt, e, bx):
        sqB = (bx * bx + bt[0] * bt[0]) + bt[1] * bt[1]
        V = tuple(mi / rho for mi in m)
        p = self.gamma1 * ((e - (0.5 * rho) * _cdot3(V, V)) - 0.5 * sqB)
        return V, p, p + 0.5 * sqB

    @staticmethod
    def flux_x(rho, V, bt, pT, e, bx):
        u = V[0]
        B = (bx, bt[0], bt[1])
        add = (pT, 0.0, 0.0)
        fm = tuple(((rho * V[i]) * u + add[i]) - bx * B[i] for i in range(3))
        fbt = (bt[0] * u - bx * V[1], bt[1] * u - bx * V[2])
        return rho * u, fm, fbt, (e + pT) * u - bx * _cdot3(V, B)

    # -- mhd_3d_hlld.fmr:106-172 --------------------------------------------
    def hlld(self, L, R, bx):
        rho_L, mL, btL, e_L = L
        rho_R, mR, btR, e_R = R
        V_L, p_L, pT_L = self.primitive(rho_L, mL, btL, e_L, bx)
        V_R, p_R, pT_R = self.primitive(rho_R, mR, btR, e_R, bx)
        u_L, u_R = V_L[0], V_R[0]

        def cfast(rho, p, bt):
            gpb2 = self.gamma * p + ((bx * bx + bt[0] * bt[0]) + bt[1] * bt[1])
            return np.sqrt((gpb2 + np.sqrt(gpb2 * gpb2 - ((4.0 * self.gamma) * p) * (bx * bx))) / (2.0 * rho))

        c_f = _max(cfast(rho_L, p_L, btL), cfast(rho_R, p_R, btR))
        S_L = _min(u_L, u_R) - c_f
        S_R = _max(u_L, u_R) + c_f
        den = rho_L * (S_L - u_L) - rho_R * (S_R - u_R)
        S_M = ((pT_R - pT_L) + (rho_L * u_L) * (S_L - u_L) - (rho_R * u_R) * (S_R - u_R)) / den
        p_st = ((rho_L * pT_R) * (S_L - u_L) - (rho_R * pT_L) * (S_R - u_R)
                + (((rho_L * rho_R) * (S_R - u_R)) * (S_L - u_L)) * (u_L - u_R)) / den

        def star(S, rho, V, bt, e, pT):
            u = V[0]
            rho_st = rho * (S - u) / (S - S_M)
            cd = (rho * (S - u)) * (S - S_M) - bx * bx
            big = np.abs(cd) > self.eps
            vf = np.where(big, bx * (S_M - u) / cd, 0.0)
            Vt_st = (V[1] - bt[0] * vf, V[2] - bt[1] * vf)
            V_st = (S_M, Vt_st[0], Vt_st[1])
            bf = np.where(big, (rho * ((S - u) * (S - u)) - bx * bx) / cd, 0.0)
            bt_st = (bt[0] * bf, bt[1] * bf)
            e_st = ((((S - u) * e - pT * u) + p_st * S_M)
                    + bx * (_cdot3(V, (bx, bt[0], bt[1])) - _cdot3(V_st, (bx, bt_st[0], bt_st[1])))) / (S - S_M)
            return rho_st, V_st, bt_st, e_st

        rL, VsL, btsL, esL = star(S_L, rho_L, V_L, btL, e_L, pT_L)
        rR, VsR, btsR, esR = star(S_R, rho_R, V_R, btR, e_R, pT_R)
        # state_star_star (mhd_3d_hlld.fmr:156-169)
        sL, sR = np.sqrt(rL), np.sqrt(rR)
        sg = _sign(bx)
        Vt_ss = tuple((((VsL[1 + i] * sL) + (VsR[1 + i] * sR)) + (btsR[i] - btsL[i]) * sg) / (sL + sR)
                      for i in range(2))
        V_ss = (S_M, Vt_ss[0], Vt_ss[1])
        srr = np.sqrt(rL * rR)
        bt_ss = tuple((((sL * btsR[i]) + (sR * btsL[i])) + (srr * (VsR[1 + i] - VsL[1 + i])) * sg) / (sL + sR)
                      for i in range(2))
        VB_ss = _cdot3(V_ss, (bx, bt_ss[0], bt_ss[1]))
        e_ssL = esL - (sL * (_cdot3(VsL, (bx, btsL[0], btsL[1])) - VB_ss)) * sg
        e_ssR = esR + (sR * (_cdot3(VsR, (bx, btsR[0], btsR[1])) - VB_ss)) * sg

        def U7(rho, m, bt, e):
            return [rho, m[0], m[1], m[2], bt[0], bt[1], e]

        UL, UR = U7(rho_L, mL, btL, e_L), U7(rho_R, mR, btR, e_R)
        UsL = U7(rL, tuple(rL * v for v in VsL), btsL, esL)
        UsR = U7(rR, tuple(rR * v for v in VsR), btsR, esR)
        UssL = U7(rL, tuple(rL * v for v in V_ss), bt_ss, e_ssL)
        UssR = U7(rR, tuple(rR * v for v in V_ss), bt_ss, e_ssR)
        FLt = self.flux_x(rho_L, V_L, btL, pT_L, e_L, bx)
        FRt = self.flux_x(rho_R, V_R, btR, pT_R, e_R, bx)
        FL, FR = U7(FLt[0], FLt[1], FLt[2], FLt[3]), U7(FRt[0], FRt[1], FRt[2], FRt[3])
        # star_speed (mhd_3d_hlld.fmr:135-138)
        S_stL = S_M - np.abs(bx) / sL
        S_stR = S_M + np.abs(bx) / sR
        aL, aR = _min(S_L, 0.0), _max(S_R, 0.0)
        bL, bR = _min(S_stL, 0.0), _max(S_stR, 0.0)
        out = []
        for i in range(7):
            fl = (FL[i] + aL * (UsL[i] - UL[i])) + bL * (UssL[i] - UsL[i])
            fr = (FR[i] + aR * (UsR[i] - UR[i])) + bR * (UssR[i] - UsR[i])
            out.append(np.where(S_M > 0, fl, fr))
        return out      # rho, m (3, cycled), bt (2), e

    # -- mhd_3d_hlld.fmr:190-201 ----------------------------------------------
    def flux_1d(self, UL, UR, ax):
        c, inv = CYCLES[ax], _inv(ax)
        rho_L, mL, BL, e_L, psi_L = UL
        rho_R, mR, BR, e_R, psi_R = UR
        cbL, cbR = c(BL), c(BR)
        bnL, btL = cbL[0], (cbL[1], cbL[2])
        bnR, btR = cbR[0], (cbR[1], cbR[2])
        bn = 0.5 * (bnL + bnR) - (0.5 / self.c_h) * (psi_R - psi_L)
        psi = 0.5 * (psi_L + psi_R) - (0.5 * self.c_h) * (bnR - bnL)
        f = self.hlld((rho_L, c(mL), btL, e_L), (rho_R, c(mR), btR, e_R), bn)
        fpsi = bn * (self.c_h * self.c_h)
        return f[0], inv((f[1], f[2], f[3])), inv((psi, f[4], f[5])), f[6], fpsi

    # -- mhd_3d_hlld.fmr:213-228 ----------------------------------------------
    def flux_from_u(self, U, ax):
        c, inv = CYCLES[ax], _inv(ax)
        rho, m, B, e, psi = U
        cb = c(B)
        bn, bt = cb[0], (cb[1], cb[2])
        V, p, pT = self.primitive(rho, c(m), bt, e, bn)
        fr, fm, fbt, fe = self.flux_x(rho, V, bt, pT, e, bn)
        return fr, inv(fm), inv((psi, fbt[0], fbt[1])), fe, bn * (self.c_h * self.c_h)

    def tvd_muscl(self, q, ax):
        dq = _fwd(q, ax) - q
        ob, of = _bwd(dq, ax), dq
        dp = _max(_max(0.0, _min(self.beta * ob, of)), _min(ob, self.beta * of))
        dn = _min(_min(0.0, _max(self.beta * ob, of)), _max(ob, self.beta * of))
        delta = np.where(of > 0, dp, dn)
        return q + 0.5 * delta, q - 0.5 * delta

    def step(self, comps):
        """One step of the 9 components (rho, rhou, rhov, rhow, B_x, B_y,
        B_z, e, psi); returns them in the same order."""
        def pack(c):
            return c[0], (c[1], c[2], c[3]), (c[4], c[5], c[6]), c[7], c[8]

        def unpack(U):
            return [U[0], U[1][0], U[1][1], U[1][2], U[2][0], U[2][1], U[2][2], U[3], U[4]]

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
            fluxes.append(unpack(self.flux_1d(pack(urbar), pack([_fwd(u, ax) for u in ulbar]), ax)))
        total = None
        for ax in range(3):
            t = [(f - _bwd(f, ax)) / self.dx[ax] for f in fluxes[ax]]
            total = t if total is None else [a + b for a, b in zip(total, t)]
        out = [u - self.dt * d for u, d in zip(comps, total)]
        out[8] = out[8] * self.damp
        return out
