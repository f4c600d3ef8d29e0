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


class SwComplex:
    def __init__(self, mesh, L, gravity=9.80616, nu=0.0, bottomDepth=None):
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

    def step(self, h, u, dt, nsteps=1):
        """nsteps RK4 steps (apps/sw/run.cc:13-70); h (nC, L), u (nE, L)."""
        h = np.asarray(h).reshape(self.nC, self.L)
        u = np.asarray(u).reshape(self.nE, self.L)
        w = (dt / 6, dt / 3, dt / 3, dt / 6)
        sub = (dt / 2, dt / 2, dt)
        for _ in range(nsteps):
            hp, up = h, u
            hn, un = h.copy(), u.copy()
            for rk in range(4):
                th, tu = self.tendencies(hp, up)
                if rk < 3:
                    hp, up = h + sub[rk] * th, u + sub[rk] * tu
                hn, un = hn + w[rk] * th, un + w[rk] * tu
            h, u = hn, un
        return h, u

    def jvp(self, h, u, vh, vu, dt, nsteps, eps=1e-30):
        """Directional derivative of (h_N, u_N) along (vh, vu) by the complex step."""
        hc = np.asarray(h, complex).reshape(self.nC, self.L) + 1j * eps * np.asarray(vh).reshape(self.nC, self.L)
        uc = np.asarray(u, complex).reshape(self.nE, self.L) + 1j * eps * np.asarray(vu).reshape(self.nE, self.L)
        hN, uN = self.step(hc, uc, dt, nsteps)
        return hN.imag / eps, uN.imag / eps
