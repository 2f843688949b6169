"""Second, independent restatement of the reference step in numpy/scipy.

Test infrastructure: it cross-checks the C oracle (oracle/ls_oracle.c) on tiny
grids. Arrays here are the padded single-rank arrays of the reference: shape
(I+1, J, K), voxel (i, j, k) at [i, j, k], the extra plane at [I]. Linear
systems are assembled as scipy.sparse matrices and solved directly.

Citations are to src/Simulation.cpp (S.cpp) and src/main.cpp of the reference.
"""
import math

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

AIR, PORE, ROCK, SULPHIDE, PRECIPITATE = 1, 2, 3, 4, 5
# neighbour order of the reference: i+1, i-1, j+1, j-1, k+1, k-1
DIRS = [(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)]


def _cpow(a, b):
    # C pow semantics through the platform libm (numpy's SIMD power differs by an ulp)
    try:
        return math.pow(a, b)
    except ValueError:
        return math.nan
    except OverflowError:
        return math.inf


cpow = np.vectorize(_cpow, otypes=[np.float64])


def smin(a, b):
    """std::min(a, b) elementwise: (b < a) ? b : a."""
    return np.where(b < a, b, a)


def smax(a, b):
    """std::max(a, b) elementwise: (a < b) ? b : a."""
    return np.where(a < b, b, a)


class Twin:
    def __init__(self, labels, params):
        labels = np.asarray(labels)
        I, J, K = labels.shape
        self.I, self.J, self.K = I, J, K
        self.p = params
        z = lambda dt=np.float64: np.zeros((I + 1, J, K), dtype=dt)
        self.label = z(np.int64)
        self.label[:I] = labels
        self.frac = z(np.float32)
        self.perm, self.visc, self.P, self.conc, self.acid = z(), z(), z(), z(), z()
        self.fx, self.fy, self.fz = z(), z(), z()
        self.sat, self.pc, self.kr, self.precip = z(), z(), z(), z()

    # shifted views -----------------------------------------------------------
    def _nb(self, arr, d):
        """arr at the neighbour in direction d for every voxel of the unpadded domain, and
        the validity mask (neighbour inside the global domain)."""
        I, J, K = self.I, self.J, self.K
        di, dj, dk = DIRS[d]
        a = arr[:I]
        out = np.zeros_like(a)
        valid = np.zeros((I, J, K), dtype=bool)
        si = slice(max(0, -di), I - max(0, di))
        sj = slice(max(0, -dj), J - max(0, dj))
        sk = slice(max(0, -dk), K - max(0, dk))
        ti = slice(max(0, di), I - max(0, -di))
        tj = slice(max(0, dj), J - max(0, -dj))
        tk = slice(max(0, dk), K - max(0, -dk))
        out[si, sj, sk] = a[ti, tj, tk]
        valid[si, sj, sk] = True
        return out, valid

    # initialisation ----------------------------------------------------------
    def init_all(self):
        I = self.I
        for f in (self.P, self.conc, self.fx, self.fy, self.fz, self.sat, self.pc, self.kr,
                  self.precip):
            f[:] = 0.0
        lab = self.label[:I]
        self.frac[:I] = np.where(lab == SULPHIDE, 1.0, 0.0).astype(np.float32)   # S.cpp:254-278
        self.sat[:I] = np.where((lab == PORE) | (lab == SULPHIDE), 0.1, 0.0)     # S.cpp:1573-1590
        self.acid[:I] = 0.0                                                     # S.cpp:285-310
        self.props()
        return int((lab == SULPHIDE).sum())

    def props(self):
        """updateRelativePermeability, updateCapillaryPressure, initProperties."""
        p, I = self.p, self.I
        lab = self.label[:I]
        s = self.sat[:I]
        m = 1.0 - (1.0 / p.vg_n)
        active = (lab == PORE) | (lab == SULPHIDE)
        with np.errstate(all="ignore"):
            Se = (s - p.s_res) / (1.0 - p.s_res)
            Sk = smax(0.0, smin(1.0, Se))
            term1 = 1.0 - cpow(1.0 - cpow(Sk, 1.0 / m), m)
            kr = np.where(Sk <= 0.0, 0.0, np.sqrt(Sk) * term1 * term1)       # S.cpp:1643-1657
            Sc = smax(1e-6, smin(1.0, Se))
            pcv = np.where(Sc >= 1.0, 0.0,
                           (1.0 / p.vg_alpha) * cpow(cpow(Sc, -1.0 / m) - 1.0, 1.0 / p.vg_n))
        self.kr[:I] = np.where(active, kr, 0.0)
        self.pc[:I] = np.where(active, pcv, 0.0)
        lkr, lkp = math.log10(1.0e-18), math.log10(1.0e-12)                     # S.cpp:187-248
        pf = smax(0.0, smin(1.0, self.precip[:I]))
        f = self.frac[:I].astype(np.float64)
        Kint = np.full(lab.shape, 1.0e-18)
        Kint = np.where(lab == AIR, 1.0e-12, Kint)
        Kint = np.where(lab == PORE, cpow(10.0, (pf * lkr) + ((1.0 - pf) * lkp)), Kint)
        Kint = np.where(lab == SULPHIDE, cpow(10.0, (f * lkr) + ((1.0 - f) * lkp)), Kint)
        self.visc[:I] = np.where(lab == AIR, 1.8e-5, 1.0e-3)
        self.perm[:I] = Kint * smax(self.kr[:I], 1e-15)

    # pressure ----------------------------------------------------------------
    def pressure_system(self, t):
        """setupPressureEqns (S.cpp:658-798) as a sparse matrix and right-hand side."""
        p, I, J, K = self.p, self.I, self.J, self.K
        N = I * J * K
        idx = np.arange(N).reshape(I, J, K)
        lab = self.label[:I]
        eff = p.top_pressure * (t / 3600.0) + 1e-6 if t < 3600.0 else p.top_pressure
        rows, cols, vals = [], [], []
        b = np.zeros(N)
        ident = (lab == AIR) | (lab == ROCK) | (lab == SULPHIDE) | (lab == PRECIPITATE)
        surf = np.zeros(lab.shape, bool)
        for d in range(6):
            nl, v = self._nb(self.label, d)
            surf |= v & (nl != AIR)
        rows.append(idx[ident]); cols.append(idx[ident]); vals.append(np.ones(ident.sum()))
        b_air = np.where((lab == AIR) & surf, 0.0 + eff, 0.0)
        b += np.where(ident, b_air, 0.0).ravel()
        pore = lab == PORE
        diag = np.zeros(lab.shape)
        src = np.zeros(lab.shape)
        Ks = smax(self.perm[:I], 1e-25)
        for d in range(6):
            nl, v = self._nb(self.label, d)
            nK, _ = self._nb(self.perm, d)
            nidx, _ = self._nb(np.concatenate([idx, idx[:1]]), d)
            use = pore & v
            Kn = np.where(nl == AIR, 1.0e-9, nK)
            src = np.where(use & (nl == AIR), src - p.evaporative_flux * p.dx, src)
            Knn = smax(Kn, 1e-25)
            with np.errstate(all="ignore"):
                c = ((2.0 * Ks * Knn) / (Ks + Knn)) / self.visc[:I]
            rows.append(idx[use]); cols.append(nidx[use]); vals.append(c[use])
            diag = np.where(use, diag - c, diag)
        diag = np.where(np.abs(diag) < 1e-16, 1e-16, diag)
        rows.append(idx[pore]); cols.append(idx[pore]); vals.append(diag[pore])
        b += np.where(pore, 0.0 + src, 0.0).ravel()
        A = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                          shape=(N, N))
        return A, b

    def _solve_into(self, field, A, b):
        """Direct solve; the solution lands one i-plane up (compat shift) or in place.
        Rows with no entries keep the value their initial guess held."""
        I, J, K = self.I, self.J, self.K
        N = I * J * K
        off = J * K if self.p.compat_shift else 0
        flat = field.reshape(-1)
        x0 = flat[off:off + N].copy()
        empty = np.diff(A.indptr) == 0
        if empty.any():
            keep = ~empty
            # move the fixed unknowns to the right-hand side
            Ak = A[keep][:, keep]
            bk = b[keep] - A[keep][:, empty] @ x0[empty]
            x = x0.copy()
            x[keep] = spla.spsolve(Ak.tocsc(), bk)
        else:
            x = spla.spsolve(A.tocsc(), b)
        flat[off:off + N] = x
        return x

    def pressure(self, t):
        A, b = self.pressure_system(t)
        return self._solve_into(self.P, A, b)

    # flux / saturation ---------------------------------------------------------
    def flux(self):
        """calculateFlux, S.cpp:866-953 (np=1)."""
        p, I, J, K = self.p, self.I, self.J, self.K
        dx = p.dx

        def grad(f):
            a = f  # padded: slot I exists
            g = np.empty((3, I, J, K))
            # i axis (slots 0..I available)
            gi = np.empty((I, J, K))
            gi[0] = (a[1] - a[0]) / dx
            if I > 1:
                gi[I - 1] = (a[I - 1] - a[I - 2]) / dx
            gi[1:I - 1] = (a[2:I] - a[0:I - 2]) / (2.0 * dx)
            u = a[:I]
            gj = np.empty((I, J, K))
            gj[:, 0] = (u[:, 1] - u[:, 0]) / dx
            gj[:, J - 1] = (u[:, J - 1] - u[:, J - 2]) / dx
            gj[:, 1:J - 1] = (u[:, 2:] - u[:, :J - 2]) / (2.0 * dx)
            gk = np.empty((I, J, K))
            gk[:, :, 0] = (u[:, :, 1] - u[:, :, 0]) / dx
            gk[:, :, K - 1] = (u[:, :, K - 1] - u[:, :, K - 2]) / dx
            gk[:, :, 1:K - 1] = (u[:, :, 2:] - u[:, :, :K - 2]) / (2.0 * dx)
            g[0], g[1], g[2] = gi, gj, gk
            return g

        gP = grad(self.P)
        gC = grad(self.pc)
        mcg = p.max_cap_grad
        gC = smax(-mcg, smin(mcg, gC))
        T = self.perm[:I] / self.visc[:I]
        rho_g = 1000.0 * 9.81
        self.fx[:I] = -T * ((gP[0] - gC[0]) - rho_g)
        self.fy[:I] = -T * (gP[1] - gC[1])
        self.fz[:I] = -T * (gP[2] - gC[2])

    def _div_evap(self):
        p, I = self.p, self.I
        lab = self.label[:I]
        q = []
        for d, f in enumerate((self.fx, self.fx, self.fy, self.fy, self.fz, self.fz)):
            nf, v = self._nb(f, d)
            q.append(np.where(v, (f[:I] + nf) / 2.0, 0.0))
        div = ((q[0] - q[1]) + (q[2] - q[3]) + (q[4] - q[5])) / p.dx
        air = np.zeros(lab.shape, dtype=np.int64)
        for d in range(6):
            nl, v = self._nb(self.label, d)
            air += (v & (nl == AIR))
        evap = np.where(lab == PORE, (air * p.evaporative_flux) / p.dx, 0.0)
        return div, evap, air

    def saturation(self, dt):
        """updateSaturation, S.cpp:1672-1856; inactive voxels end as 0.0."""
        p, I = self.p, self.I
        lab = self.label[:I]
        active = ~((lab == AIR) | (lab == ROCK) | (lab == SULPHIDE) | (lab == PRECIPITATE))
        div, evap, _ = self._div_evap()
        tot = np.abs(div) + evap
        mx = 0.0
        for v in tot[active].ravel():      # max with the reference's NaN behaviour
            if v > mx:
                mx = v
        dt_safe = (0.1 * p.porosity) / mx if mx > 1e-20 else dt
        calc = np.ceil(dt / dt_safe)
        if np.isinf(calc) or np.isnan(calc) or calc > 1000:
            n = 1000
        elif calc > 1.0:
            n = int(calc)
        else:
            n = 1
        dt_sub = dt / n
        c = dt_sub / p.porosity
        s = self.sat[:I].copy()
        for _ in range(n):
            s = smax(0.0, smin(1.0, s - c * (div + evap)))
        new = np.zeros_like(self.sat)
        new[:I] = np.where(active, s, 0.0)
        self.sat[:] = new
        return {"max_rate": mx, "num_steps": n, "dt_sub": dt_sub}

    def surface(self):
        """handleSurfaceEffects, S.cpp:2063-2103."""
        I = self.I
        lab = self.label[:I]
        nearair = np.zeros(lab.shape, bool)
        for d in range(6):
            nl, v = self._nb(self.label, d)
            nearair |= v & (nl == AIR)
        hit = (lab == PORE) & (self.sat[:I] > 0.0) & nearair
        self.conc[:I][hit] = 1.0
        self.label[:I][hit] = PRECIPITATE

    # transport -------------------------------------------------------------------
    def transport_system(self, dt, which):
        """setupConcentrationEqns, active part S.cpp:1129-1232."""
        p, I, J, K = self.p, self.I, self.J, self.K
        N = I * J * K
        field = self.acid if which else self.conc
        idx = np.arange(N).reshape(I, J, K)
        lab = self.label[:I]
        inv_dt = 1.0 / dt
        f = field[:I]
        diag = np.where(lab == PRECIPITATE, 1.0, inv_dt)
        b = np.where(lab == PRECIPITATE, 0.0 + f, 0.0 + f * inv_dt)
        rows, cols, vals = [], [], []
        qself = {0: self.fx, 2: self.fy, 4: self.fz}
        for d in range(6):
            nl, v = self._nb(self.label, d)
            nidx, _ = self._nb(np.concatenate([idx, idx[:1]]), d)
            nfield, _ = self._nb(field, d)
            # Rock rows: exchange with Pore neighbours only
            rock = (lab == ROCK) & v & (nl == PORE)
            diag = np.where(rock, diag + p.alpha_transfer, diag)
            rows.append(idx[rock]); cols.append(nidx[rock]); vals.append(np.full(rock.sum(), -p.alpha_transfer))
            other = (lab != ROCK) & (lab != PRECIPITATE) & v
            ex = other & (nl == ROCK)
            diag = np.where(ex, diag + p.alpha_transfer, diag)
            rows.append(idx[ex]); cols.append(nidx[ex]); vals.append(np.full(ex.sum(), -p.alpha_transfer))
            lk = other & (nl != ROCK)
            if d % 2 == 0:
                qf = qself[d][:I]
            else:
                src = {1: self.fx, 3: self.fy, 5: self.fz}[d]
                nq, _ = self._nb(src, d)
                qf = -nq
            aq = np.where((nl == PRECIPITATE) | (nl == SULPHIDE), 0.0, qf)
            Deff = np.where(nl == PORE, p.D * p.Dpore_fac, p.D)
            dc = -Deff / (p.dx * p.dx)
            cn = dc.copy()
            cs = -dc
            adv = aq / p.dx
            cs = np.where(adv > 0, cs + adv, cs)
            cn = np.where(adv > 0, cn, cn - adv)
            rows.append(idx[lk]); cols.append(nidx[lk]); vals.append((p.theta * cn)[lk])
            diag = np.where(lk, diag + p.theta * cs, diag)
            b = np.where(lk, b + (1.0 - p.theta) * (-(cs * f + cn * nfield)), b)
        rows.append(idx.ravel()); cols.append(idx.ravel()); vals.append(diag.ravel())
        A = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                          shape=(N, N))
        return A, b.ravel()

    def transport(self, dt):
        for which in (0, 1):
            A, b = self.transport_system(dt, which)
            self._solve_into(self.acid if which else self.conc, A, b)
        solid = (self.label[:self.I] == ROCK) | (self.label[:self.I] == PRECIPITATE)
        for f in (self.fx, self.fy, self.fz):
            f[:self.I][solid] = 0.0

    def precipitation(self):
        """handlePrecipitation, S.cpp:2114-2165."""
        p, I = self.p, self.I
        lab = self.label[:I]
        c = self.conc[:I]
        hit = (lab == PORE) & (c > p.c_sat)
        excess = c - p.c_sat
        if p.use_instant_precipitation:
            self.label[:I][hit] = PRECIPITATE
        else:
            add = (excess * (p.porosity * self.sat[:I])) / p.solid_density
            newp = np.where(hit, self.precip[:I] + add * p.time_scalar, self.precip[:I])
            self.precip[:I] = newp
            self.label[:I][hit & (newp > 0.90)] = PRECIPITATE
        self.conc[:I][hit] = p.c_sat

    # dissolution: the sequential sweep, written as plain loops -------------------
    def dissolve(self, dt):
        """updateFrac, S.cpp:315-617."""
        p, I, J, K = self.p, self.I, self.J, self.K
        lab, acid, frac = self.label, self.acid, self.frac

        def sflux(i, j, k):
            if 0 <= i < I and 0 <= j < J and 0 <= k < K and lab[i, j, k] in (PORE, ROCK):
                k_trans = p.D / p.dx
                k_eff = 1.0 / ((1.0 / k_trans) + (1.0 / p.kreac))
                return k_eff * acid[i, j, k]
            return 0.0

        mx = 0.0
        for k in range(K):
            for j in range(J):
                for i in range(I):
                    if lab[i, j, k] == SULPHIDE:
                        fs = 0.0
                        for (a, b_, c) in DIRS:
                            fs += sflux(i + a, j + b_, k + c)
                        fr = (fs * (p.dx * p.dx)) / (p.dx * p.dx * p.dx)
                        if fr > mx:
                            mx = fr
        eff = mx * p.time_scalar
        dt_safe = 0.1 / eff if eff > 1e-20 else dt
        calc = np.ceil(dt / dt_safe)
        n = 1000 if calc > 1000 else (int(calc) if calc > 1.0 else 1)
        dt_sub = dt / n
        leached = 0
        for _ in range(n):
            for k in range(K):
                for j in range(J):
                    for i in range(I):
                        if lab[i, j, k] >= SULPHIDE and frac[i, j, k] > 0.0:
                            f = [sflux(i + a, j + b_, k + c) for (a, b_, c) in DIRS]
                            fs = f[0] + f[1] + f[2] + f[3] + f[4] + f[5]
                            fl = (fs * (p.dx * p.dx) * dt_sub) / (p.dx * p.dx * p.dx)
                            frac[i, j, k] = np.float32(np.float64(frac[i, j, k]) - fl * p.time_scalar)
                            if fs > 0.0:
                                for q, (a, b_, c) in enumerate(DIRS):
                                    ii, jj, kk = i + a, j + b_, k + c
                                    if 0 <= ii < I and 0 <= jj < J and 0 <= kk < K:
                                        acid[ii, jj, kk] -= fl * (f[q] / fs)
                            if np.float64(frac[i, j, k]) <= 1e-4:
                                frac[i, j, k] = 0.0
                                if lab[i, j, k] == SULPHIDE:
                                    lab[i, j, k] = PORE
                                    self.precip[i, j, k] = 0.0
                                    self.conc[i, j, k] = p.c_sat
                                    leached += 1
        return leached, {"max_rate": mx, "num_steps": n, "dt_sub": dt_sub}

    def step(self, t, dt):
        """One attempt of main.cpp:303-432 with explicit saturation (direct solves)."""
        self.props()
        self.pressure(t)
        self.flux()
        self.saturation(dt)
        self.surface()
        self.transport(dt)
        self.precipitation()
        return self.dissolve(dt)[0]
