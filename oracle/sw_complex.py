"""TEST INFRASTRUCTURE ONLY -- never imported by the product.

Array restatement of the sw app's (h, u) RK4 step, generic in the element
type so that it also runs on complex numbers.  Its purpose is the
complex-step derivative (Squire & Trapp 1998; Martins, Sturdza & Alonso
2003): for a real-analytic F and tiny eps, Im F(x + i eps v) / eps equals the
directional derivative J v to working precision, with no subtractive
cancellation.  That gives an exact reference tangent of the reference
algorithm on the CPU, against which the hand-written adjoint is checked by
the dot-product identity <w, J v> = <J^T w, v>.

The step follows the reference task sequence (tracers are passive in the sw
app and left out; pin_u and FCT are not involved):
  diagnostics   apps/sw/tasks/solve.cc:11-107   (restated in oracle.c:48-97)
  tendencies    apps/sw/tasks/solve.cc:169-234  (oracle.c:100-138)
  del2 momentum oracle test term (sw_extra.c), off when nu = 0
  RK4 stages    apps/sw/run.cc:13-70            (oracle.c sw_advance)
Connectivity is read the reference's way (Mesh.crs): cells and vertices of an
edge in ascending id order (the transposed cell->edge / edge->vertex lists),
the kite areas of a vertex paired with its transposed vertex->cell list.
Only analytic operations (+, -, *, /) touch the state, so the complex step is
exact.  The real part agrees with oracle.c to rounding (summation order
differs)."""
import numpy as np


def _smax(a, b):
    """(a < b) ? b : a on the real parts (the reference's max), carrying the chosen value."""
    return np.where(np.real(a) < np.real(b), b, a)


def _smin(a, b):
    """(b < a) ? b : a on the real parts (the reference's min)."""
    return np.where(np.real(b) < np.real(a), b, a)


class SwComplex:
    def __init__(self, mesh, L, gravity=9.80616, nu=0.0, bottomDepth=None, fct=None, T=0,
                 hmix=False, kappa=0.0, centred=False):
        """fct: the FCT statics (edge signs, advection stencils, del2 scaling), or None;
        centred: the sw app's centred tracer flux even when statics are given."""
        f = mesh.fields
        crs = mesh.crs()
        self.nC, self.nE, self.nV, self.L = mesh.nCells, mesh.nEdges, mesh.nVertices, L
        self.g, self.nu = gravity, nu
        eo, ei = crs["e2c"]
        assert np.all(np.diff(eo) == 2), "every edge needs two cells"
        self.c1, self.c2 = ei[eo[:-1]], ei[eo[:-1] + 1]
        vo, vi = crs["e2v"]
        self.v1, self.v2 = vi[vo[:-1]], vi[vo[:-1] + 1]
        co, ci = crs["c2e"]
        self.c2e_c = np.repeat(np.arange(self.nC), np.diff(co))
        self.c2e_e = ci
        self.c2e_sgn = np.where(self.c1[ci] == self.c2e_c, 1.0, -1.0)  # sw_extra.c divergence sign
        ao, ai = crs["v2c"]
        assert np.all(np.diff(ao) == 3)
        self.vc = ai.reshape(self.nV, 3)
        po, pi = crs["v2e"]
        self.v2e_v = np.repeat(np.arange(self.nV), np.diff(po))
        self.v2e_e = pi
        qo, qi = crs["e2e"]
        cnt = np.diff(qo)
        self.ee_e = np.repeat(np.arange(self.nE), cnt)
        self.ee_o = qi
        slot = np.arange(qi.size) - np.repeat(qo[:-1], cnt)
        self.ee_w = f["weightsOnEdge"][self.ee_e, slot]
        self.dc, self.dv = f["dcEdge"][:, None], f["dvEdge"][:, None]
        self.area = f["areaCell"][:, None]
        self.atri = f["areaTriangle"][:, None]
        self.kite = f["kiteAreasOnVertex"]
        self.fv = f["fVertex"][:, None]
        self.bd = (np.zeros(self.nC) if bottomDepth is None else np.asarray(bottomDepth, float))[:, None]
        # tracers: FCT advection (apps/ocean/tasks/solve.cc:99-326) and del2 mixing (:328-366),
        # thickness-weighted RK of apps/sw/tasks/solve.cc:162, 300-302, 337, 354
        self.T, self.hmix, self.kappa, self.fct = T, hmix, kappa, fct is not None and not centred
        self.c2c_c = np.repeat(np.arange(self.nC), np.diff(crs["c2c"][0]))
        self.c2c_n = crs["c2c"][1]
        slot_e = np.arange(ci.size) - np.repeat(co[:-1], np.diff(co))
        if fct is not None:
            self.esgn = fct["edgeSignOnCell"][self.c2e_c, slot_e][:, None, None]
            na = fct["nAdvCellsForEdge"]
            ea = np.repeat(np.arange(self.nE), na)
            sa = np.arange(na.sum()) - np.repeat(np.cumsum(na) - na, na)
            self.adv_e, self.adv_c = ea, fct["advCellsForEdge"][ea, sa]
            self.adv_c1 = fct["advCoef"][ea, sa][:, None, None]
            self.adv_c3 = (fct["advCoef_3rd"][ea, sa] * 0.25)[:, None, None]
            self.mask = fct["highOrderAdvMask"][:, :L].astype(float)[:, :, None]
            self.msd = fct["meshScalingDel2"][:, None, None]
        else:
            self.esgn = np.where(self.c1[ci] == self.c2e_c, -1.0, 1.0)[:, None, None]
            self.msd = np.ones((self.nE, 1, 1))

    def _scatter(self, n, idx, vals):
        out = np.zeros((n, self.L), vals.dtype)
        np.add.at(out, idx, vals)
        return out

    def diagnostics(self, h, u):
        """h_edge, ke, pv_edge, vorticity of (h, u) (apps/sw/tasks/solve.cc:11-107)."""
        he = 0.5 * (h[self.c1] + h[self.c2])
        circ = self._scatter(self.nV, self.v2, self.dc * u) - self._scatter(self.nV, self.v1, self.dc * u)
        vort = circ / self.atri
        w = (0.25 * self.dc * self.dv)[self.c2e_e]
        ke = self._scatter(self.nC, self.c2e_c, w * u[self.c2e_e] ** 2) / self.area
        hv = (h[self.vc] * self.kite[:, :, None]).sum(axis=1) / self.atri
        pvv = (self.fv + vort) / hv
        pve = self._scatter(self.nE, self.v2e_e, 0.5 * pvv[self.v2e_v])
        return he, ke, pve, vort

    def tendencies(self, h, u):
        """(tend_h, tend_u) of a stage state (apps/sw/tasks/solve.cc:169-234 + del2)."""
        he, ke, pve, vort = self.diagnostics(h, u)
        flux = u * self.dv * he
        tend_h = (self._scatter(self.nC, self.c2, flux) - self._scatter(self.nC, self.c1, flux)) / self.area
        e, o = self.ee_e, self.ee_o
        q = self._scatter(self.nE, e, self.ee_w[:, None] * u[o] * (0.5 * (pve[e] + pve[o])) * he[o])
        c1, c2 = self.c1, self.c2
        tend_u = q - (ke[c2] - ke[c1] + self.g * (h[c2] + self.bd[c2] - h[c1] - self.bd[c1])) / self.dc
        if self.nu != 0.0:
            div = self._scatter(self.nC, self.c2e_c,
                                self.c2e_sgn[:, None] * self.dv[self.c2e_e] * u[self.c2e_e]) / self.area
            tend_u = tend_u + self.nu * ((div[c2] - div[c1]) / self.dc - (vort[self.v2] - vort[self.v1]) / self.dv)
        return tend_h, tend_u

    def tracer_tendency(self, h, u, tr, dt, hE=None, ocean=False):
        """Tracer mass tendency [nC][L][T] of a stage state (FCT of apps/ocean/tasks/
        solve.cc:99-326 on the thickness flux, plus del2 mixing of :328-366).  sw: the
        edge thickness is the cells' mean and, without FCT, the centred flux advects;
        ocean (apps/ocean/run.cc:20-42): the given layerThicknessEdge hE, and
        without FCT nothing advects."""
        c1, c2 = self.c1, self.c2
        he = 0.5 * (h[c1] + h[c2]) if hE is None else hE
        ntf = (u * he)[:, :, None]                                     # normal thickness flux
        dv = self.dv[:, :, None]
        ce, ee = self.c2e_c, self.c2e_e
        sgn_area = self.esgn / self.area[ce][:, :, None]
        if self.fct:
            # provisional thickness and its inverse
            hprov = h + self._scatter(self.nC, ce, (dt * self.dv[ee] * self.esgn[:, :, 0] / self.area[ce])
                                      * (u * he)[ee])
            hpi = (1.0 / hprov)[:, :, None]
            lo = dv * (_smax(0.0, ntf) * tr[c1] + _smin(0.0, ntf) * tr[c2])
            f = ntf[self.adv_e]
            sg = np.where(np.real(f) < 0, -1.0, np.where(np.real(f) > 0, 1.0, 0.0))
            wf = f * self.mask[self.adv_e] * (self.adv_c1 + self.adv_c3 * sg)
            ho = np.zeros(lo.shape, np.result_type(lo, wf))
            np.add.at(ho, self.adv_e, tr[self.adv_c] * wf)
            ho = ho + (1.0 - self.mask) * (dv * 0.5) * ntf * (tr[c1] + tr[c2])
            ho = ho - lo
            # bounds over the cell and its neighbours, taken in the cell->cell list's order
            trmax, trmin = tr.copy(), tr.copy()
            nn = self.c2c_n
            cnt = np.bincount(self.c2c_c, minlength=self.nC)
            start = np.concatenate([[0], np.cumsum(cnt)[:-1]])
            for j in range(cnt.max()):
                sel = cnt > j
                cells = np.nonzero(sel)[0]
                nb = nn[start[sel] + j]
                trmax[cells] = _smax(trmax[cells], tr[nb])
                trmin[cells] = _smin(trmin[cells], tr[nb])
            tend_lo = self._scatter3(ce, sgn_area * lo[ee])
            fin = self._scatter3(ce, _smax(0.0, sgn_area * ho[ee]))
            fout = self._scatter3(ce, _smin(0.0, sgn_area * ho[ee]))
            upw = (tr * h[:, :, None] + dt * tend_lo) * hpi
            tmax_new = upw + dt * fin * hpi
            tmin_new = upw + dt * fout * hpi
            eps = 1.e-10
            rp = _smin(1.0, _smax(0.0, (trmax - upw) / (tmax_new - upw + eps)))
            rm = _smin(1.0, _smax(0.0, (upw - trmin) / (upw - tmin_new + eps)))
            hol = _smax(0.0, ho) * _smin(rm[c1], rp[c2]) + _smin(0.0, ho) * _smin(rp[c1], rm[c2])
            np.add.at(tend_lo, ce, sgn_area * hol[ee])
            tend = tend_lo
        elif not ocean:  # centred flux (apps/sw/tasks/solve.cc:237-270)
            flux = dv * ntf * (0.5 * (tr[c1] + tr[c2]))
            tend = self._scatter3(c2, flux / self.area[c2][:, :, None]) - \
                self._scatter3(c1, flux / self.area[c1][:, :, None])
        else:
            tend = np.zeros(tr.shape, np.result_type(tr, u, he))
        if self.hmix:
            rho = self.msd * self.kappa * dv / self.dc[:, :, None]
            fl = he[:, :, None] * (tr[c2] - tr[c1]) * rho
            tend = tend - self._scatter3(ce, sgn_area * fl[ee])
        return tend

    def _scatter3(self, idx, vals):
        out = np.zeros((self.nC, self.L, self.T), vals.dtype)
        np.add.at(out, idx, vals)
        return out

    def step(self, h, u, dt, nsteps=1, tr=None):
        """nsteps RK4 steps (apps/sw/run.cc:13-70); h (nC, L), u (nE, L), tr (nC, L, T) or None."""
        h = np.asarray(h).reshape(self.nC, self.L)
        u = np.asarray(u).reshape(self.nE, self.L)
        if tr is not None:
            tr = np.asarray(tr).reshape(self.nC, self.L, self.T)
        w = (dt / 6, dt / 3, dt / 3, dt / 6)
        sub = (dt / 2, dt / 2, dt)
        for _ in range(nsteps):
            hp, up, tp = h, u, tr
            hn, un = h.copy(), u.copy()
            qn = None if tr is None else tr * h[:, :, None]
            for rk in range(4):
                th, tu = self.tendencies(hp, up)
                tq = None if tr is None else self.tracer_tendency(hp, up, tp, dt)
                if rk < 3:
                    hp, up = h + sub[rk] * th, u + sub[rk] * tu
                    if tr is not None:
                        tp = (h[:, :, None] * tr + sub[rk] * tq) / hp[:, :, None]
                hn, un = hn + w[rk] * th, un + w[rk] * tu
                if tr is not None:
                    qn = qn + w[rk] * tq
            h, u = hn, un
            if tr is not None:
                tr = qn / hn[:, :, None]
        return (h, u) if tr is None else (h, u, tr)

    def jvp_tracers(self, h, u, tr, vh, vu, vt, dt, nsteps, eps=1e-30):
        """Directional derivative of (h_N, u_N, tr_N) along (vh, vu, vt) by the complex step;
        every max / min / sign of the FCT limiter is decided on the real parts, so this is the
        derivative on the branch the real step takes."""
        hc = np.asarray(h, complex).reshape(self.nC, self.L) + 1j * eps * np.asarray(vh).reshape(self.nC, self.L)
        uc = np.asarray(u, complex).reshape(self.nE, self.L) + 1j * eps * np.asarray(vu).reshape(self.nE, self.L)
        tc = (np.asarray(tr, complex).reshape(self.nC, self.L, self.T)
              + 1j * eps * np.asarray(vt).reshape(self.nC, self.L, self.T))
        hN, uN, tN = self.step(hc, uc, dt, nsteps, tr=tc)
        return hN.imag / eps, uN.imag / eps, tN.imag / eps

    def ocean_step(self, h, hE, u, tr, dt, nsteps=1):
        """nsteps RK4 steps of the ocean app's tracers (apps/ocean/run.cc:10-50): thickness,
        edge thickness and velocity prescribed; tr_s = tr0 + w_sub T_{s-1}, tr_new =
        tr0 + sum w T_s (apps/ocean/tasks/solve.cc:368-399, no thickness weighting)."""
        h = np.asarray(h).reshape(self.nC, self.L)
        hE = np.asarray(hE).reshape(self.nE, self.L)
        u = np.asarray(u).reshape(self.nE, self.L)
        tr = np.asarray(tr).reshape(self.nC, self.L, self.T)
        w = (dt / 6, dt / 3, dt / 3, dt / 6)
        sub = (dt / 2, dt / 2, dt)
        for _ in range(nsteps):
            tp, tn = tr, tr.copy()
            for rk in range(4):
                tq = self.tracer_tendency(h, u, tp, dt, hE=hE, ocean=True)
                tn = tn + w[rk] * tq
                if rk < 3:
                    tp = tr + sub[rk] * tq
            tr = tn
        return tr

    def ocean_jvp(self, h, hE, u, tr, vt, dt, nsteps, eps=1e-30):
        """Directional derivative of the ocean app's final tracers along vt (complex step,
        limiter branches decided on the real parts)."""
        tc = (np.asarray(tr, complex).reshape(self.nC, self.L, self.T)
              + 1j * eps * np.asarray(vt).reshape(self.nC, self.L, self.T))
        return self.ocean_step(h, hE, u, tc, dt, nsteps).imag / eps

    def jvp(self, h, u, vh, vu, dt, nsteps, eps=1e-30):
        """Directional derivative of (h_N, u_N) along (vh, vu) by the complex step."""
        hc = np.asarray(h, complex).reshape(self.nC, self.L) + 1j * eps * np.asarray(vh).reshape(self.nC, self.L)
        uc = np.asarray(u, complex).reshape(self.nE, self.L) + 1j * eps * np.asarray(vu).reshape(self.nE, self.L)
        hN, uN = self.step(hc, uc, dt, nsteps)
        return hN.imag / eps, uN.imag / eps
