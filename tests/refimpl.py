"""Second, independent restatement of the reference path in vectorised numpy.

Test infrastructure only.  Written separately from the C oracle (different
structure: whole-array masks that replay each reference loop in statement
order, ordered np.add.at scatters instead of per-edge loops) so that the two
transcriptions check each other bit for bit.  Every routine cites the
reference lines it restates.  Arrays use the (entity, level) layout of
fesom2_gb300.mesh; level numbers are 1-based as in the Fortran.
"""
from __future__ import annotations

import math

import numpy as np

R_EARTH = 6367500.0
EPS_AB = 0.1
FLUX_EPS = 1e-16
BIG = 1e3


class Ref:
    def __init__(self, m):
        self.m = m
        self.L1 = m.nl - 1
        self.nl = m.nl
        self.lev = np.arange(1, m.nl)[None, :]        # layer numbers 1..nl-1
        self.levI = np.arange(1, m.nl + 1)[None, :]   # interface numbers 1..nl
        e = m.edges.astype(np.int64)
        self.n1, self.n2 = e[:, 0], e[:, 1]
        self.el1 = m.edge_tri[:, 0].astype(np.int64)
        el2 = m.edge_tri[:, 1].astype(np.int64)
        self.has2 = el2 >= 0
        self.e2 = np.maximum(el2, 0)
        self.nl1 = (m.nlevels[self.el1] - 1)[:, None]
        self.nu1 = m.ulevels[self.el1][:, None]
        self.nl2 = np.where(self.has2, m.nlevels[self.e2] - 1, 0)[:, None]
        self.nu2 = np.where(self.has2, m.ulevels[self.e2], 0)[:, None]
        # scatter range (oce_adv_tra_driver.F90:142-156)
        self.s_nl12 = np.maximum(self.nl1, self.nl2)
        self.s_nu12 = np.where(self.nu2 > 0, np.minimum(self.nu1, self.nu2), self.nu1)
        self.smask = (self.lev >= self.s_nu12) & (self.lev <= self.s_nl12)
        # flux segments A..E (oce_adv_tra_hor.F90:159-250)
        fnl12 = np.minimum(self.nl1, self.nl2)
        fnu12 = np.maximum(self.nu1, self.nu2)
        L = self.lev
        self.segs = [((L >= self.nu1) & (L <= fnu12 - 1), 1),
                     ((self.nu2 > 0) & (L >= self.nu2) & (L <= fnu12 - 1), 2),
                     ((L >= fnu12) & (L <= fnl12), 3),
                     ((L >= fnl12 + 1) & (L <= self.nl1), 1),
                     ((L >= fnl12 + 1) & (L <= self.nl2), 2)]
        self.nzmin = m.ulevels_nod2D[:, None]
        self.nzmax = m.nlevels_nod2D[:, None]
        self.wet = (self.lev >= self.nzmin) & (self.lev <= self.nzmax - 1)
        # ordered scatter rows: per edge (n1, +), (n2, -)
        self.sc_rows = np.stack([self.n1, self.n2], axis=1).reshape(-1)
        # node -> element slots in nod_in_elem2D order
        ptr = m.nod_in_elem2D_ptr
        self.nie_num = np.diff(ptr)
        self.nie_max = int(self.nie_num.max())
        self.nie = np.full((m.nod2D, self.nie_max), -1, np.int64)
        rows = np.repeat(np.arange(m.nod2D), self.nie_num)
        cols = np.arange(ptr[-1]) - np.repeat(ptr[:-1], self.nie_num)
        self.nie[rows, cols] = m.nod_in_elem2D

    # -------------------------------------------------------------------------
    def _scatter(self, F, mask, sign2=-1.0, init=None):
        """Reference edge scatter, ascending edges: node(1) += F, node(2) -= F."""
        N2 = self.m.nod2D
        acc = np.zeros((N2, self.L1)) if init is None else init.copy()
        Fm = np.where(mask, F, 0.0)
        vals = np.stack([Fm, sign2 * Fm], axis=1).reshape(-1, self.L1)
        np.add.at(acc, self.sc_rows, vals)
        return acc

    def vflux(self, vel, which):
        m = self.m
        h1 = m.helem[self.el1]
        h2 = m.helem[self.e2]
        ecd = m.edge_cross_dxdy
        v1 = (-(vel[self.el1, :, 1] * ecd[:, 0:1]) + vel[self.el1, :, 0] * ecd[:, 1:2]) * h1
        v2 = (vel[self.e2, :, 1] * ecd[:, 2:3] - vel[self.e2, :, 0] * ecd[:, 3:4]) * h2
        return {1: v1, 2: v2, 3: v1 + v2}[which]

    # ---- oce_ale_tracer.F90:1526-1689 (diff_part_hor_redi) ---------------------
    def diff_part_hor_redi(self, dt, Ki, trxy, del_ttf, slope=None, trz=None):
        """Edge fluxes Kh (grad T [+ S T_z with Redi]) of the segments A..E, scattered in
        ascending edge order; slope (nod2D, nl-1, 3), trz (nod2D, nl) for Redi = .true."""
        m = self.m
        Kh = (Ki[self.n1] + Ki[self.n2]) / 2.0
        ecd = m.edge_cross_dxdy
        dX1, dY1 = ecd[:, 0:1], ecd[:, 1:2]
        dX2 = np.where(self.has2[:, None], ecd[:, 2:3], 0.0)
        dY2 = np.where(self.has2[:, None], ecd[:, 3:4], 0.0)
        h1, h2 = m.helem[self.el1], m.helem[self.e2]
        t1, t2 = trxy[self.el1], trxy[self.e2]
        if slope is None:
            F = lambda Tx, Ty: (Kh * Tx, Kh * Ty)
        else:
            L1 = self.L1
            # vertical gradient at mid-layer of both edge nodes (:1586-1588)
            Tz1 = 0.5 * (trz[self.n1][:, :L1] + trz[self.n1][:, 1:L1 + 1])
            Tz2 = 0.5 * (trz[self.n2][:, :L1] + trz[self.n2][:, 1:L1 + 1])
            sx = (Tz1 * slope[self.n1][:, :, 0] + Tz2 * slope[self.n2][:, :, 0]) / 2.0
            sy = (Tz1 * slope[self.n1][:, :, 1] + Tz2 * slope[self.n2][:, :, 1]) / 2.0
            F = lambda Tx, Ty: (Kh * (Tx + sx), Kh * (Ty + sy))
        Fx1, Fy1 = F(t1[:, :, 0], t1[:, :, 1])
        Fx2, Fy2 = F(t2[:, :, 0], t2[:, :, 1])
        c1 = (-dX1 * Fy1 + dY1 * Fx1) * h1
        c2 = (dX2 * Fy2 - dY2 * Fx2) * h2
        Tx = 0.5 * (t1[:, :, 0] + t2[:, :, 0])
        Ty = 0.5 * (t1[:, :, 1] + t2[:, :, 1])
        Fx3, Fy3 = F(Tx, Ty)
        c3 = ((dX2 - dX1) * Fy3 - (dY2 - dY1) * Fx3) * ((h1 + h2) / 2.0)
        c = np.zeros_like(Kh)
        for mask, typ in self.segs:
            c = np.where(mask, {1: c1, 2: c2, 3: c3}[typ], c)
        rhs1, rhs2 = 0.0 + c, 0.0 - c
        av = m.areasvol[:, :-1]
        v1 = np.where(self.smask, rhs1 * dt / av[self.n1], 0.0)
        v2 = np.where(self.smask, rhs2 * dt / av[self.n2], 0.0)
        vals = np.stack([v1, v2], axis=1).reshape(-1, self.L1)
        out = del_ttf.copy()
        np.add.at(out, self.sc_rows, vals)
        return out

    # ---- oce_ale_tracer.F90:841-902 (diff_ver_part_expl_ale) ----------------
    def diff_ver_part_expl_ale(self, dt, Kv, flux, T, del_ttf):
        m = self.m
        N2, L1 = m.nod2D, self.L1
        nl1 = (m.nlevels_nod2D - 1)[:, None]
        ul1 = m.ulevels_nod2D[:, None]
        lev = self.lev
        vd = np.zeros((N2, L1 + 2))  # vd[:, nz], nz 1-based
        Tm = np.concatenate([np.zeros((N2, 1)), T[:, :-1]], axis=1)   # T(nz-1)
        zm = np.concatenate([np.ones((N2, 1)), m.Z_3d_n[:, :-1]], axis=1)
        with np.errstate(divide="ignore", invalid="ignore"):
            zinv1 = 1.0 / (zm - m.Z_3d_n)
            inner = Kv[:, :L1] * (Tm - T) * zinv1 * m.area[:, :L1]
        vdl = np.where((lev >= ul1 + 1) & (lev <= nl1), inner, 0.0)
        vdl = np.where(lev == ul1, (np.zeros(N2) if flux is None else flux)[:, None], vdl)
        vd[:, 1:L1 + 1] = vdl
        vnext = vd[:, 2:L1 + 2]
        zb = m.zbar_3d_n
        av = m.areasvol[:, :L1]
        with np.errstate(divide="ignore", invalid="ignore"):
            mid = (vdl - vnext) / (zb[:, :L1] - zb[:, 1:L1 + 1]) * dt / av
            bot = (vdl / (zb[:, :L1] - zb[:, 1:L1 + 1])) * dt / av
        out = del_ttf.copy()
        out = np.where((lev >= ul1) & (lev <= nl1 - 1), out + mid, out)
        out = np.where(lev == nl1, out + bot, out)
        return out

    # ---- oce_tracer_mod.F90:147-188 -----------------------------------------
    def tr_xy(self, T):
        m = self.m
        en = m.elem2D_nodes.astype(np.int64)
        gs = m.gradient_sca
        out = np.zeros((m.elem2D, self.L1, 2))
        Ta, Tb, Tc = T[en[:, 0]], T[en[:, 1]], T[en[:, 2]]
        for c in range(2):
            s = 0.0 + gs[:, 3 * c + 0:3 * c + 1] * Ta
            s = s + gs[:, 3 * c + 1:3 * c + 2] * Tb
            s = s + gs[:, 3 * c + 2:3 * c + 3] * Tc
            out[:, :, c] = s
        wet = (self.lev >= m.ulevels[:, None]) & (self.lev <= m.nlevels[:, None] - 1)
        return np.where(wet[:, :, None], out, 0.0)

    def node_mean(self, trxy):
        """fill_up_dn_grad node means (oce_muscl_adv.F90:388-405) for every node-level."""
        m = self.m
        N2 = m.nod2D
        tvol = np.zeros((N2, self.L1))
        tx = np.zeros((N2, self.L1))
        ty = np.zeros((N2, self.L1))
        for k in range(self.nie_max):
            el = self.nie[:, k]
            has = el >= 0
            elc = np.maximum(el, 0)
            wetk = has[:, None] & ~((m.nlevels[elc][:, None] - 1 < self.lev) | (self.lev < m.ulevels[elc][:, None]))
            ea = m.elem_area[elc][:, None]
            tvol = np.where(wetk, tvol + ea, tvol)
            tx = np.where(wetk, tx + trxy[elc, :, 0] * ea, tx)
            ty = np.where(wetk, ty + trxy[elc, :, 1] * ea, ty)
        with np.errstate(divide="ignore", invalid="ignore"):
            return tx / tvol, ty / tvol

    def fill_up_dn_grad(self, trxy, updn):
        """edge_up_dn_grad (oce_muscl_adv.F90:356-525), loops replayed in order."""
        m = self.m
        E = m.edge2D
        gx, gy = self.node_mean(trxy)
        G = np.zeros((E, self.L1, 4))
        up, dn = updn[:, 0].astype(np.int64), updn[:, 1].astype(np.int64)
        inner = ((up >= 0) & (dn >= 0))[:, None]
        L = self.lev
        nzmin = np.maximum(m.ulevels_nod2D_max[self.n1], m.ulevels_nod2D_max[self.n2])[:, None]
        nzmax = np.minimum(m.nlevels_nod2D_min[self.n1], m.nlevels_nod2D_min[self.n2])[:, None]
        for side, node, (ix, iy) in ((0, self.n1, (0, 2)), (1, self.n2, (1, 3))):
            ul = m.ulevels_nod2D[node][:, None]
            nlv = m.nlevels_nod2D[node][:, None]
            mx, my = gx[node], gy[node]
            tri = np.maximum(up if side == 0 else dn, 0)
            # inner edges: [ul, nzmin-1] mean, [nzmin, nzmax-1] triangle, [nzmax, nl-1] mean
            a = inner & (L >= ul) & (L <= nzmin - 1)
            G[:, :, ix] = np.where(a, mx, G[:, :, ix]); G[:, :, iy] = np.where(a, my, G[:, :, iy])
            b = inner & (L >= nzmin) & (L <= nzmax - 1)
            G[:, :, ix] = np.where(b, trxy[tri, :, 0], G[:, :, ix]); G[:, :, iy] = np.where(b, trxy[tri, :, 1], G[:, :, iy])
            c = inner & (L >= nzmax) & (L <= nlv - 1)
            G[:, :, ix] = np.where(c, mx, G[:, :, ix]); G[:, :, iy] = np.where(c, my, G[:, :, iy])
            d = ~inner & (L >= ul) & (L <= nlv - 1)
            G[:, :, ix] = np.where(d, mx, G[:, :, ix]); G[:, :, iy] = np.where(d, my, G[:, :, iy])
        return G

    # ---- oce_adv_tra_hor.F90 ------------------------------------------------
    def hor_upw1(self, vel, T, flux):
        T1, T2 = T[self.n1], T[self.n2]
        for mask, which in self.segs:
            vf = self.vflux(vel, which)
            val = -(0.5 * (T1 * (vf + np.abs(vf)) + T2 * (vf - np.abs(vf)))) - flux
            flux = np.where(mask, val, flux)
        return flux

    def hor_ho(self, vel, T, num_ord, flux, G, nbl, use_clo):
        m = self.m
        T1, T2 = T[self.n1], T[self.n2]
        el1c = m.elem_cos[self.el1]
        a = R_EARTH * el1c
        a = np.where(self.has2, 0.5 * (a + R_EARTH * m.elem_cos[self.e2]), a)[:, None]
        ex, ey = m.edge_dxdy[:, 0:1], m.edge_dxdy[:, 1:2]
        L = self.lev
        clo1 = np.where((nbl[self.n1][:, None] - L) >= 0, 1.0, 0.0)
        clo2 = np.where((nbl[self.n2][:, None] - L) >= 0, 1.0, 0.0)
        B2 = 2.0 * (T2 - T1) + ex * a * G[:, :, 1] + ey * R_EARTH * G[:, :, 3]
        B1 = 2.0 * (T2 - T1) + ex * a * G[:, :, 0] + ey * R_EARTH * G[:, :, 2]
        if use_clo:
            Tm2 = T2 - B2 / 6.0 * clo2
            Tm1 = T1 + B1 / 6.0 * clo1
        else:
            Tm2 = T2 - B2 / 6.0
            Tm1 = T1 + B1 / 6.0
        for mask, which in self.segs:
            vf = self.vflux(vel, which)
            cHO = (vf + np.abs(vf)) * Tm1 + (vf - np.abs(vf)) * Tm2
            val = -(0.5 * (1.0 - num_ord) * cHO) - vf * num_ord * 0.5 * (Tm1 + Tm2) - flux
            flux = np.where(mask, val, flux)
        return flux

    # ---- oce_adv_tra_ver.F90:244-434 ----------------------------------------
    def _col(self, A, nz):
        """A(nz) per node for a per-node level array nz (1-based), clipped."""
        return np.take_along_axis(A, np.clip(nz - 1, 0, A.shape[1] - 1), axis=1)

    def ver_upw1(self, W, T, flux):
        m = self.m
        N2 = m.nod2D
        I = self.levI
        Tp = np.concatenate([T, np.zeros((N2, 1))], axis=1)           # T(nz), nz = 1..nl
        Tm = np.concatenate([np.zeros((N2, 1)), T], axis=1)           # T(nz-1)
        A = m.area
        s = I == self.nzmin
        flux = np.where(s, -(W * Tp * A) - flux, flux)
        b = I == self.nzmax
        flux = np.where(b, 0.0 - flux, flux)
        i = (I >= self.nzmin + 1) & (I <= self.nzmax - 1)
        flux = np.where(i, -(0.5 * (Tp * (W + np.abs(W)) + Tm * (W - np.abs(W))) * A) - flux, flux)
        return flux

    def ver_qr4c(self, W, T, num_ord, flux):
        m = self.m
        N2 = m.nod2D
        I = self.levI
        z = np.zeros((N2, 1))
        T0 = np.concatenate([T, z], axis=1)
        Tm1 = np.concatenate([z, T], axis=1)
        Tm2 = np.concatenate([z, z, T[:, :-1]], axis=1)
        Tp1 = np.concatenate([T[:, 1:], z, z], axis=1)
        Zn = m.Z_3d_n
        Z0 = np.concatenate([Zn, z], axis=1)
        Zm1 = np.concatenate([z, Zn], axis=1)
        Zm2 = np.concatenate([z, z, Zn[:, :-1]], axis=1)
        Zp1 = np.concatenate([Zn[:, 1:], z, z], axis=1)
        A = m.area
        flux = np.where(I == self.nzmin, -(T0 * W * A) - flux, flux)
        cen = -(0.5 * (Tm1 + T0) * W * A)
        flux = np.where(I == self.nzmin + 1, cen - flux, flux)
        flux = np.where(I == self.nzmax - 1, cen - flux, flux)
        flux = np.where(I == self.nzmax, 0.0 - flux, flux)
        with np.errstate(divide="ignore", invalid="ignore"):
            qc = (Tm1 - T0) / (Zm1 - Z0)
            qu = (T0 - Tp1) / (Z0 - Zp1)
            qd = (Tm2 - Tm1) / (Zm2 - Zm1)
            t1 = T0 + (2 * qc + qu) * (m.zbar_3d_n - Z0) / 3.0
            t2 = Tm1 + (2 * qc + qd) * (m.zbar_3d_n - Zm1) / 3.0
            Tmean = (W + np.abs(W)) * t1 + (W - np.abs(W)) * t2
            val = (-(0.5 * (1.0 - num_ord) * Tmean) - num_ord * (0.5 * (t1 + t2)) * W) * A - flux
        i = (I >= self.nzmin + 2) & (I <= self.nzmax - 2)
        return np.where(i, val, flux)

    # ---- oce_adv_tra_fct.F90:72-512 -----------------------------------------
    def fct(self, dt, T, LO, adf_h, adf_v):
        m = self.m
        N2, L1 = m.nod2D, self.L1
        wet = self.wet
        fmax = np.where(wet, np.maximum(LO, T), 0.0)
        fmin = np.where(wet, np.minimum(LO, T), 0.0)
        en = m.elem2D_nodes.astype(np.int64)
        ewet = (self.lev >= m.ulevels[:, None]) & (self.lev <= m.nlevels[:, None] - 1)
        aux1 = np.where(ewet, np.maximum(np.maximum(fmax[en[:, 0]], fmax[en[:, 1]]), fmax[en[:, 2]]), -BIG)
        aux2 = np.where(ewet, np.minimum(np.minimum(fmin[en[:, 0]], fmin[en[:, 1]]), fmin[en[:, 2]]), BIG)
        tmax = aux1[self.nie[:, 0]]
        tmin = aux2[self.nie[:, 0]]
        for k in range(1, self.nie_max):
            el = self.nie[:, k]
            has = (el >= 0)[:, None]
            tmax = np.where(has, np.maximum(tmax, aux1[np.maximum(el, 0)]), tmax)
            tmin = np.where(has, np.minimum(tmin, aux2[np.maximum(el, 0)]), tmin)
        L = self.lev
        up_ = np.concatenate([tmax[:, :1], tmax[:, :-1]], axis=1)     # tvert(nz-1)
        dn_ = np.concatenate([tmax[:, 1:], tmax[:, -1:]], axis=1)     # tvert(nz+1)
        upm = np.concatenate([tmin[:, :1], tmin[:, :-1]], axis=1)
        dnm = np.concatenate([tmin[:, 1:], tmin[:, -1:]], axis=1)
        bmax = np.where(L == self.nzmin, tmax - LO, 0.0)
        bmin = np.where(L == self.nzmin, tmin - LO, 0.0)
        i = (L >= self.nzmin + 1) & (L <= self.nzmax - 2)
        bmax = np.where(i, np.maximum(np.maximum(up_, tmax), dn_) - LO, bmax)
        bmin = np.where(i, np.minimum(np.minimum(upm, tmin), dnm) - LO, bmin)
        b = L == self.nzmax - 1
        bmax = np.where(b, tmax - LO, bmax)
        bmin = np.where(b, tmin - LO, bmin)
        # b1
        v0, v1 = adf_v[:, :L1], adf_v[:, 1:]
        P = np.where(wet, 0.0 + (np.maximum(0.0, v0) + np.maximum(0.0, -v1)), 0.0)
        Mn = np.where(wet, 0.0 + (np.minimum(0.0, v0) + np.minimum(0.0, -v1)), 0.0)
        Fm = np.where(self.smask, adf_h, 0.0)
        for acc, f1, f2 in ((P, np.maximum(0.0, Fm), np.maximum(0.0, -Fm)),
                            (Mn, np.minimum(0.0, Fm), np.minimum(0.0, -Fm))):
            vals = np.stack([f1, f2], axis=1).reshape(-1, L1)
            np.add.at(acc, self.sc_rows, vals)
        av = m.areasvol[:, :L1]
        hn = m.hnode_new
        with np.errstate(divide="ignore", invalid="ignore"):
            Rp = np.where(wet, np.minimum(1.0, bmax / (P * dt / av / hn + FLUX_EPS)), 0.0)
            Rm = np.where(wet, np.minimum(1.0, bmin / (Mn * dt / av / hn - FLUX_EPS)), 0.0)
        # b3 vertical
        I = self.levI
        Rp_I = np.concatenate([Rp, np.zeros((N2, 1))], axis=1)
        Rm_I = np.concatenate([Rm, np.zeros((N2, 1))], axis=1)
        Rp_Im = np.concatenate([np.zeros((N2, 1)), Rp], axis=1)
        Rm_Im = np.concatenate([np.zeros((N2, 1)), Rm], axis=1)
        pos = adf_v >= 0.0
        ae_s = np.where(pos, np.minimum(1.0, Rp_I), np.minimum(1.0, Rm_I))
        ae_i = np.where(pos, np.minimum(np.minimum(1.0, Rm_Im), Rp_I), np.minimum(np.minimum(1.0, Rp_Im), Rm_I))
        adf_v = np.where(I == self.nzmin, ae_s * adf_v, adf_v)
        adf_v = np.where((I >= self.nzmin + 1) & (I <= self.nzmax - 1), ae_i * adf_v, adf_v)
        # b3 horizontal
        pos = adf_h >= 0.0
        ae = np.where(pos, np.minimum(np.minimum(1.0, Rp[self.n1]), Rm[self.n2]),
                      np.minimum(np.minimum(1.0, Rm[self.n1]), Rp[self.n2]))
        adf_h = np.where(self.smask, ae * adf_h, adf_h)
        return adf_h, adf_v, {"tvert_max": tmax, "tvert_min": tmin}

    # ---- oce_adv_tra_driver.F90 ----------------------------------------------
    def adv_tra(self, dt, vel, W, WE, T, TAB, hor, ver, lim, ph, pv, G, nbl, WI=None, wsplit=False):
        m = self.m
        N2, L1, nl = m.nod2D, self.L1, self.nl
        wet = self.wet
        E = m.edge2D
        av = m.areasvol[:, :L1]
        aux = {}
        if lim == "FCT":
            fh = self.hor_upw1(vel, T, np.zeros((E, L1)))
            LOs = self._scatter(fh, self.smask)
            fv = self.ver_upw1(WE, T, np.zeros((N2, nl)))
            LO = np.where(wet, (T * m.hnode + (LOs + (fv[:, :L1] - fv[:, 1:])) * dt / av) / m.hnode_new, LOs)
            if wsplit:
                LO = vert_impl(m, dt, WI, LO)
                fv = self.ver_upw1(W, T, np.zeros((N2, nl)))
            flux_h, flux_v = fh, fv
            pw = W
        else:
            flux_h, flux_v = np.zeros((E, L1)), np.zeros((N2, nl))
            pw = WE
        if hor == "MUSCL":
            flux_h = self.hor_ho(vel, TAB, ph, flux_h, G, nbl, True)
        elif hor == "MFCT":
            flux_h = self.hor_ho(vel, TAB, ph, flux_h, G, nbl, False)
        else:
            flux_h = self.hor_upw1(vel, TAB, flux_h)
        if ver == "QR4C":
            flux_v = self.ver_qr4c(pw, TAB, pv, flux_v)
        elif ver == "CDIFF":
            flux_v = ver_cdiff(m, pw, TAB, flux_v)
        elif ver == "PPM":
            flux_v = ver_ppm(m, dt, pw, TAB, flux_v)
        else:
            flux_v = self.ver_upw1(pw, TAB, flux_v)
        dv = np.zeros((N2, L1))
        if lim == "FCT":
            flux_h, flux_v, aux = self.fct(dt, T, LO, flux_h, flux_v)
            aux["LO"] = LO
            dv = np.where(wet, dv - T * m.hnode + LO * m.hnode_new, dv)
        dv = np.where(wet, dv + (flux_v[:, :L1] - flux_v[:, 1:]) * dt / av, dv)
        Fm = np.where(self.smask, flux_h, 0.0)
        vals = np.stack([Fm * dt / av[self.n1], -(Fm * dt / av[self.n2])], axis=1).reshape(-1, L1)
        dh = np.zeros((N2, L1))
        # the reference subtracts at node 2: dttf_h = dttf_h - flux*dt/areasvol (same value as adding the negation)
        np.add.at(dh, self.sc_rows, vals)
        return dh, dv, aux

    # ---- oce_ale_tracer.F90:907-1435 ------------------------------------------
    def vdiff(self, dt, Kv, bc, T):
        m = self.m
        N2, nl = m.nod2D, self.nl
        T = T.copy()
        hn = m.hnode_new
        ar, av = m.area, m.areasvol
        nzmin = m.ulevels_nod2D.astype(np.int64)
        nzmax = m.nlevels_nod2D.astype(np.int64)
        rows = np.arange(N2)
        H = lambda k: hn[rows, np.clip(k - 1, 0, nl - 2)]
        g = lambda A, k: A[rows, np.clip(k - 1, 0, A.shape[1] - 1)]
        # Z_n bottom-up
        Zn = np.zeros((N2, nl + 1))
        zb = m.zbar_n_bot.copy()
        Zn[rows, nzmax - 1] = zb + H(nzmax - 1) / 2.0
        for k in range(nl, 0, -1):   # nz = nzmax-1 .. nzmin+1
            act = (k <= nzmax - 1) & (k >= nzmin + 1)
            zb = np.where(act, zb + H(k), zb)
            Zn[rows, np.clip(k - 1, 0, nl)] = np.where(act, zb + H(k - 1) / 2.0, Zn[rows, np.clip(k - 1, 0, nl)])
        ZN = lambda k: Zn[rows, np.clip(k, 0, nl)]
        a = np.zeros((N2, nl + 1)); b = np.zeros((N2, nl + 1)); c = np.zeros((N2, nl + 1)); tr = np.zeros((N2, nl + 1))
        nz = nzmin
        zinv2 = 1.0 / (ZN(nz) - ZN(nz + 1))
        zinv = 1.0 * dt
        c[rows, nz] = -(g(Kv, nz + 1) * zinv2 * zinv * g(ar, nz + 1) / g(av, nz))
        b[rows, nz] = -c[rows, nz] + H(nz)
        zinv1 = zinv2
        for k in range(1, nl + 1):
            act = (k >= nzmin + 1) & (k <= nzmax - 2)
            z2 = 1.0 / (ZN(np.full(N2, k)) - ZN(np.full(N2, k + 1)))
            kk = np.full(N2, k)
            av_ = g(av, kk)
            ak = -(g(Kv, kk) * zinv1 * zinv * (g(ar, kk) / av_))
            ck = -(g(Kv, kk + 1) * z2 * zinv * g(ar, kk + 1) / av_)
            a[:, k] = np.where(act, ak, a[:, k])
            c[:, k] = np.where(act, ck, c[:, k])
            b[:, k] = np.where(act, -ak - ck + H(kk), b[:, k])
            zinv1 = np.where(act, z2, zinv1)
        nz = nzmax - 1
        ak = -(g(Kv, nz) * zinv1 * zinv * (g(ar, nz) / g(av, nz)))
        a[rows, nz] = ak
        c[rows, nz] = 0.0
        b[rows, nz] = -ak + H(nz)
        Tv = lambda k: T[rows, np.clip(k - 1, 0, nl - 2)]
        nz = nzmin
        tr[rows, nz] = -((b[rows, nz] - H(nz)) * Tv(nz)) - c[rows, nz] * Tv(nz + 1)
        for k in range(1, nl + 1):
            act = (k >= nzmin + 1) & (k <= nzmax - 2)
            kk = np.full(N2, k)
            val = -(a[:, k] * Tv(kk - 1)) - (b[:, k] - H(kk)) * Tv(kk) - c[:, k] * Tv(kk + 1)
            tr[:, k] = np.where(act, val, tr[:, k])
        nz = nzmax - 1
        tr[rows, nz] = -(a[rows, nz] * Tv(nz - 1)) - (b[rows, nz] - H(nz)) * Tv(nz)
        tr[rows, nzmin] = tr[rows, nzmin] + bc
        cp = np.zeros((N2, nl + 1)); tp = np.zeros((N2, nl + 1))
        cp[rows, nzmin] = c[rows, nzmin] / b[rows, nzmin]
        tp[rows, nzmin] = tr[rows, nzmin] / b[rows, nzmin]
        for k in range(1, nl + 1):
            act = (k >= nzmin + 1) & (k <= nzmax - 1)
            with np.errstate(divide="ignore", invalid="ignore"):
                mm = b[:, k] - cp[:, k - 1] * a[:, k]
                cp[:, k] = np.where(act, c[:, k] / mm, cp[:, k])
                tp[:, k] = np.where(act, (tr[:, k] - tp[:, k - 1] * a[:, k]) / mm, tp[:, k])
        tr[rows, nzmax - 1] = tp[rows, nzmax - 1]
        for k in range(nl, 0, -1):
            act = (k <= nzmax - 2) & (k >= nzmin)
            tr[:, k] = np.where(act, tp[:, k] - cp[:, k] * tr[:, np.minimum(k + 1, nl)], tr[:, k])
        for k in range(1, nl):
            act = (k >= nzmin) & (k <= nzmax - 1)
            T[:, k - 1] = np.where(act, T[:, k - 1] + tr[:, k], T[:, k - 1])
        return T

    # ---- whole per-tracer body ----------------------------------------------------
    def tracer_step(self, forcing, T, Told, updn, nbl, hor="MUSCL", ver="QR4C", lim="FCT", ph=0.0, pv=1.0,
                    wsplit=False):
        m = self.m
        dt = forcing.dt
        TAB = -((0.5 + EPS_AB) * Told) + (1.5 + EPS_AB) * T
        Told_new = T.copy()
        G = self.fill_up_dn_grad(self.tr_xy(T), updn)
        dh, dv, _ = self.adv_tra(dt, forcing.uv, forcing.w, forcing.w_e, T, TAB, hor, ver, lim, ph, pv, G, nbl,
                                 WI=forcing.w_i, wsplit=wsplit)
        wet = self.wet
        dl = 0.0 + dh + dv
        dl = np.where(wet, dl + T * (m.hnode - m.hnode_new), dl)
        Tn = np.where(wet, T + dl / m.hnode_new, T)
        if wsplit and lim != "FCT":
            Tn = vdiff_wimpl(m, dt, forcing.Kv, forcing.bc_surface, forcing.w_i, Tn)
        else:
            Tn = self.vdiff(dt, forcing.Kv, forcing.bc_surface, Tn)
        return Tn, Told_new


# ---------------------------------------------------------------------------
# Redi = .true. (isoneutral diffusion with the tapered neutral slopes as input)
# ---------------------------------------------------------------------------
def tr_z(m, T):
    """tracer_gradient_z (oce_tracer_mod.F90:192-232) as (nod2D, nl); 0 outside the columns."""
    N2, nl = m.nod2D, m.nl
    out = np.zeros((N2, nl))
    lev = np.arange(1, nl + 1)[None, :]
    dz = 0.5 * (m.hnode[:, :-1] + m.hnode[:, 1:])            # interfaces 2 .. nl-1
    g = (T[:, :-1] - T[:, 1:]) / np.where(dz != 0.0, dz, 1.0)
    inner = (lev[:, 1:nl - 1] >= m.ulevels_nod2D[:, None] + 1) & (lev[:, 1:nl - 1] <= m.nlevels_nod2D[:, None] - 1)
    out[:, 1:nl - 1] = np.where(inner, g, 0.0)
    return out


def _depths_bottom_up(m, h, n, top, bottom_interface):
    """zbar(k), z(k) of column n from the layer thicknesses h, accumulated upward from zbar_n_bot
    (zbar at bottom_interface; z of the layer above it at its half thickness)."""
    zbar = {bottom_interface: m.zbar_n_bot[n]}
    z = {bottom_interface - 1: zbar[bottom_interface] + h[n, bottom_interface - 2] / 2.0}
    for k in range(bottom_interface - 1, top, -1):
        zbar[k] = zbar[k + 1] + h[n, k - 1]
        z[k - 1] = zbar[k] + h[n, k - 2] / 2.0
    return zbar, z


def redi_vexpl(m, dt, Ki, slope, trxy, del_ttf):
    """diff_ver_part_redi_expl (oce_ale_tracer.F90:1439-1518), column by column."""
    out = del_ttf.copy()
    for n in range(m.nod2D):
        nl1, ul1 = int(m.nlevels_nod2D[n]) - 1, int(m.ulevels_nod2D[n])
        els = m.nod_in_elem2D[m.nod_in_elem2D_ptr[n]:m.nod_in_elem2D_ptr[n + 1]]
        gxy = {}
        for nz in range(ul1, nl1 + 1):
            tx = ty = 0.0
            for el in els:
                if m.ulevels[el] <= nz <= m.nlevels[el] - 1:
                    tx = tx + trxy[el, nz - 1, 0] * m.elem_area[el]
                    ty = ty + trxy[el, nz - 1, 1] * m.elem_area[el]
            av = m.areasvol[n, nz - 1]
            gxy[nz] = (tx / 3.0 / av, ty / 3.0 / av)
        zbar, z = _depths_bottom_up(m, m.hnode, n, ul1, nl1 + 1)
        proj = lambda k: slope[n, k - 1, 0] * gxy[k][0] + slope[n, k - 1, 1] * gxy[k][1]
        vd = {k: 0.0 for k in range(ul1, nl1 + 2)}
        for nz in range(ul1 + 1, nl1 + 1):
            v = (z[nz - 1] - zbar[nz]) * proj(nz - 1) * Ki[n, nz - 2]
            v = v + (zbar[nz] - z[nz]) * proj(nz) * Ki[n, nz - 1]
            vd[nz] = v / (z[nz - 1] - z[nz]) * m.area[n, nz - 1]
        for nz in range(ul1, nl1 + 1):
            out[n, nz - 1] = out[n, nz - 1] + (vd[nz] - vd[nz + 1]) * dt / m.areasvol[n, nz - 1]
    return out


def redi_k33(m, Kv, Ki, slope):
    """Kv + Ty of diff_ver_part_impl_ale with Redi (oce_ale_tracer.F90:1099-1204) per interface,
    (nod2D, nl): the diffusivity K_33 = Kv + Kd s^2 that the implicit solve uses."""
    K = Kv.copy()
    for n in range(m.nod2D):
        nzmax, nzmin = int(m.nlevels_nod2D[n]), int(m.ulevels_nod2D[n])
        zbar, Z = _depths_bottom_up(m, m.hnode_new, n, nzmin, nzmax)
        for nz in range(nzmin + 1, nzmax):
            zinv = 1.0 / (Z[nz - 1] - Z[nz])
            sa, sb = slope[n, nz - 2, 2], slope[n, nz - 1, 2]
            Ty = (zbar[nz] - Z[nz]) * zinv * (sa * sa) * Ki[n, nz - 2] + \
                (Z[nz - 1] - zbar[nz]) * zinv * (sb * sb) * Ki[n, nz - 1]
            K[n, nz - 1] = Kv[n, nz - 1] + Ty
    return K


# ---------------------------------------------------------------------------
# column routines as plain loops (small meshes): vertical schemes CDIFF and PPM,
# implicit advection by the w_i part of a split vertical velocity
# ---------------------------------------------------------------------------
def ver_cdiff(m, W, T, flux):
    """adv_tra_ver_cdiff (oce_adv_tra_ver.F90:635-695); flux (nod2D, nl) updated and returned."""
    flux = flux.copy()
    for n in range(m.nod2D):
        nzmax = int(m.nlevels_nod2D[n]) - 1
        nzmin = int(m.ulevels_nod2D[n])
        tvert = {nzmin: -(W[n, nzmin - 1] * T[n, nzmin - 1] * m.area[n, nzmin - 1]), nzmax + 1: 0.0}
        for nz in range(nzmin + 1, nzmax + 1):
            tv = 0.5 * (T[n, nz - 2] + T[n, nz - 1])
            tvert[nz] = -(tv * W[n, nz - 1] * m.area[n, nz - 1])
        for nz in range(nzmin, nzmax + 1):
            flux[n, nz - 1] = tvert[nz] - flux[n, nz - 1]
    return flux


def _sign1(x):
    return -1.0 if math.copysign(1.0, x) < 0 else 1.0


def ver_ppm(m, dt, W, T, flux):
    """adv_tra_vert_ppm (oce_adv_tra_ver.F90:438-631)."""
    flux = flux.copy()
    for n in range(m.nod2D):
        nzmax = int(m.nlevels_nod2D[n])
        nzmin = int(m.ulevels_nod2D[n])
        t = lambda k: T[n, k - 1]
        h = lambda k: m.hnode_new[n, k - 1]
        w = lambda k: W[n, k - 1]
        tv = {}
        tv[nzmin] = t(nzmin)
        tv[nzmin + 1] = 0.5 * (t(nzmin) + t(nzmin + 1))
        tv[nzmax - 1] = 0.5 * (t(nzmax - 2) + t(nzmax - 1))
        tv[nzmax] = t(nzmax - 1)
        for nz in range(nzmin + 1, nzmax - 2):
            a0, a1, a2, a3 = h(nz - 1), h(nz), h(nz + 1), h(nz + 2)
            dj = a1 / (a0 + a1 + a2) * ((2.0 * a0 + a1) / (a2 + a1) * (t(nz + 1) - t(nz))
                                        + (a1 + 2.0 * a2) / (a0 + a1) * (t(nz) - t(nz - 1)))
            dj1 = a2 / (a1 + a2 + a3) * ((2.0 * a1 + a2) / (a3 + a2) * (t(nz + 2) - t(nz + 1))
                                         + (a2 + 2.0 * a3) / (a1 + a2) * (t(nz + 1) - t(nz)))
            if (t(nz + 1) - t(nz)) * (t(nz) - t(nz - 1)) > 0.0:
                dj = min(abs(dj), 2.0 * abs(t(nz + 1) - t(nz)), 2.0 * abs(t(nz) - t(nz - 1))) * _sign1(dj)
            else:
                dj = 0.0
            if (t(nz + 2) - t(nz + 1)) * (t(nz + 1) - t(nz)) > 0.0:
                dj1 = min(abs(dj1), 2.0 * abs(t(nz + 2) - t(nz + 1)), 2.0 * abs(t(nz + 1) - t(nz))) * _sign1(dj1)
            else:
                dj1 = 0.0
            tv[nz + 1] = (t(nz) + a1 / (a1 + a2) * (t(nz + 1) - t(nz))
                          + 1.0 / (a0 + a1 + a2 + a3)
                          * ((2.0 * a2 * a1) / (a1 + a2) * ((a0 + a1) / (2.0 * a1 + a2) - (a3 + a2) / (2.0 * a2 + a1))
                             * (t(nz + 1) - t(nz))
                             - a1 * (a0 + a1) / (2.0 * a1 + a2) * dj1
                             + a2 * (a2 + a3) / (a1 + 2.0 * a2) * dj))
        tvert = {k: 0.0 for k in range(1, nzmax + 1)}
        for nz in range(nzmin, nzmax):
            if w(nz) <= 0.0 and w(nz + 1) >= 0.0:
                continue
            aL, aR = tv[nz], tv[nz + 1]
            if (aR - t(nz)) * (t(nz) - aL) <= 0.0:
                aL = aR = t(nz)
            if (aR - aL) * (t(nz) - 0.5 * (aL + aR)) > (aR - aL) * (aR - aL) / 6.0:
                aL = 3.0 * t(nz) - 2.0 * aR
            if (aR - aL) * (t(nz) - 0.5 * (aR + aL)) < -((aR - aL) * (aR - aL) / 6.0):
                aR = 3.0 * t(nz) - 2.0 * aL
            dz = m.hnode[n, nz - 1]
            aj = 6.0 * (t(nz) - 0.5 * (aL + aR))
            if w(nz) > 0.0:
                x = min(w(nz) * dt / dz, 1.0)
                v = -aL - 0.5 * x * (aR - aL + (1.0 - 2.0 / 3.0 * x) * aj)
                tvert[nz] = v * m.area[n, nz - 1] * w(nz)
            if w(nz + 1) < 0.0:
                x = min(-(w(nz + 1) * dt / dz), 1.0)
                v = -aR + 0.5 * x * (aR - aL - (1.0 - 2.0 / 3.0 * x) * aj)
                tvert[nz + 1] = v * m.area[n, nz] * w(nz + 1)
        tvert[nzmin] = -(tv[nzmin] * w(nzmin) * m.area[n, nzmin - 1])
        tvert[nzmax] = 0.0
        for nz in range(nzmin, nzmax + 1):
            flux[n, nz - 1] = tvert[nz] - flux[n, nz - 1]
    return flux


def _thomas(a, b, c, tr, lo, hi):
    cp, tp = {}, {}
    cp[lo] = c[lo] / b[lo]
    tp[lo] = tr[lo] / b[lo]
    for nz in range(lo + 1, hi + 1):
        mm = b[nz] - cp[nz - 1] * a[nz]
        cp[nz] = c[nz] / mm
        tp[nz] = (tr[nz] - tp[nz - 1] * a[nz]) / mm
    x = {hi: tp[hi]}
    for nz in range(hi - 1, lo - 1, -1):
        x[nz] = tp[nz] - cp[nz] * x[nz + 1]
    return x


def vert_impl(m, dt, W, T):
    """adv_tra_vert_impl (oce_adv_tra_ver.F90:90-240) on a copy of T."""
    T = T.copy()
    for n in range(m.nod2D):
        nzmax = int(m.nlevels_nod2D[n])
        nzmin = int(m.ulevels_nod2D[n])
        hn = lambda k: m.hnode_new[n, k - 1]
        ar = lambda k: m.area[n, k - 1]
        av = lambda k: m.areasvol[n, k - 1]
        w = lambda k: W[n, k - 1]
        a, b, c, tr = {}, {}, {}, {}
        zinv = 1.0 * dt
        nz = nzmin
        a[nz] = 0.0
        v = zinv * ar(nz) / av(nz)
        b[nz] = hn(nz) + w(nz) * v
        v = zinv * ar(nz + 1) / av(nz)
        b[nz] = b[nz] - min(0.0, w(nz + 1)) * v
        c[nz] = -(max(0.0, w(nz + 1)) * v)
        for nz in range(nzmin + 1, nzmax - 1):
            v = zinv * ar(nz) / av(nz)
            a[nz] = min(0.0, w(nz)) * v
            b[nz] = hn(nz) + max(0.0, w(nz)) * v
            v = zinv * ar(nz + 1) / av(nz)
            b[nz] = b[nz] - min(0.0, w(nz + 1)) * v
            c[nz] = -(max(0.0, w(nz + 1)) * v)
        nz = nzmax - 1
        v = zinv * ar(nz) / av(nz)
        a[nz] = min(0.0, w(nz)) * v
        b[nz] = hn(nz) + max(0.0, w(nz)) * v
        c[nz] = 0.0
        t = lambda k: T[n, k - 1]
        tr[nzmin] = -((b[nzmin] - hn(nzmin)) * t(nzmin)) - c[nzmin] * t(nzmin + 1)
        for nz in range(nzmin + 1, nzmax - 1):
            tr[nz] = -(a[nz] * t(nz - 1)) - (b[nz] - hn(nz)) * t(nz) - c[nz] * t(nz + 1)
        nz = nzmax - 1
        tr[nz] = -(a[nz] * t(nz - 1)) - (b[nz] - hn(nz)) * t(nz)
        x = _thomas(a, b, c, tr, nzmin, nzmax - 1)
        for nz in range(nzmin, nzmax):
            T[n, nz - 1] = T[n, nz - 1] + x[nz]
    return T


def vdiff_wimpl(m, dt, Kv, bc, WI, T):
    """diff_ver_part_impl_ale (oce_ale_tracer.F90:907-1435) with do_wimpl, on a copy of T."""
    T = T.copy()
    for n in range(m.nod2D):
        nzmax = int(m.nlevels_nod2D[n])
        nzmin = int(m.ulevels_nod2D[n])
        hn = lambda k: m.hnode_new[n, k - 1]
        ar = lambda k: m.area[n, k - 1]
        av = lambda k: m.areasvol[n, k - 1]
        kv = lambda k: Kv[n, k - 1]
        wi = lambda k: WI[n, k - 1]
        zbar, Z = {}, {}
        zbar[nzmax] = m.zbar_n_bot[n]
        Z[nzmax - 1] = zbar[nzmax] + hn(nzmax - 1) / 2.0
        for nz in range(nzmax - 1, nzmin, -1):
            zbar[nz] = zbar[nz + 1] + hn(nz)
            Z[nz - 1] = zbar[nz] + hn(nz - 1) / 2.0
        a, b, c, tr = {}, {}, {}, {}
        nz = nzmin
        zinv2 = 1.0 / (Z[nz] - Z[nz + 1])
        zinv = 1.0 * dt
        a[nz] = 0.0
        c[nz] = -(kv(nz + 1) * zinv2 * zinv * ar(nz + 1) / av(nz))
        b[nz] = -c[nz] + hn(nz)
        v = zinv * (ar(nz) / av(nz))
        b[nz] = b[nz] + wi(nz) * v
        v = zinv * ar(nz + 1) / av(nz)
        b[nz] = b[nz] - min(0.0, wi(nz + 1)) * v
        c[nz] = c[nz] - max(0.0, wi(nz + 1)) * v
        zinv1 = zinv2
        for nz in range(nzmin + 1, nzmax - 1):
            zinv2 = 1.0 / (Z[nz] - Z[nz + 1])
            a[nz] = -(kv(nz) * zinv1 * zinv * (ar(nz) / av(nz)))
            c[nz] = -(kv(nz + 1) * zinv2 * zinv * ar(nz + 1) / av(nz))
            b[nz] = -a[nz] - c[nz] + hn(nz)
            zinv1 = zinv2
            v = zinv * (ar(nz) / av(nz))
            a[nz] = a[nz] + min(0.0, wi(nz)) * v
            b[nz] = b[nz] + max(0.0, wi(nz)) * v
            v = zinv * ar(nz + 1) / av(nz)
            b[nz] = b[nz] - min(0.0, wi(nz + 1)) * v
            c[nz] = c[nz] - max(0.0, wi(nz + 1)) * v
        nz = nzmax - 1
        a[nz] = -(kv(nz) * zinv1 * zinv * (ar(nz) / av(nz)))
        c[nz] = 0.0
        b[nz] = -a[nz] + hn(nz)
        v = zinv * (ar(nz) / av(nz))
        a[nz] = a[nz] + min(0.0, wi(nz)) * v
        b[nz] = b[nz] + max(0.0, wi(nz)) * v
        t = lambda k: T[n, k - 1]
        tr[nzmin] = -((b[nzmin] - hn(nzmin)) * t(nzmin)) - c[nzmin] * t(nzmin + 1)
        for nz in range(nzmin + 1, nzmax - 1):
            tr[nz] = -(a[nz] * t(nz - 1)) - (b[nz] - hn(nz)) * t(nz) - c[nz] * t(nz + 1)
        nz = nzmax - 1
        tr[nz] = -(a[nz] * t(nz - 1)) - (b[nz] - hn(nz)) * t(nz)
        tr[nzmin] = tr[nzmin] + (0.0 if bc is None else bc[n])
        x = _thomas(a, b, c, tr, nzmin, nzmax - 1)
        for nz in range(nzmin, nzmax):
            T[n, nz - 1] = T[n, nz - 1] + x[nz]
    return T
