"""numpy restatement of the igrid TVD-RK3 LES step, periodic in z, with the (dynamic)
Smagorinsky model.

TEST INFRASTRUCTURE ONLY: the tests and the CPU-baseline leg of ``bench.py`` use it as the
checker; the library never calls it.

Configuration restated (src/incompressible/igrid.F90 with PeriodicInZ, Fourier x/y,
staggered CD06 z, rotational advection, slip-wall BC codes so the viscous z term is
d2dz2_C2C / d2dz2_E2E, no stratification, Coriolis, forcing, turbines or wall model):
  * TVD_RK3 (igrid.F90:1105-1174), compute_deltaT (1374-1403), populate_rhs (1793-1912),
    addNonLinearTerm_Rot (1497-1570), addViscousTerm (1914-1959), project_and_prep
    (1961-1991), interp_PrimitiveVars (1423-1463), compute_duidxj (2553-2684),
    dealiasFields (1020-1037), init sequence (625-648), wrapup_timestep (2067-2072).
  * spectral with fixOddball = .false. (igrid.F90:489-493): k1, k2 with the oddball sign
    flipped; kabs_sq = k1^2 + k2^2; 3-D dealiasing mask for periodic z (spectral.F90:
    777-811) applied through z transforms (314-363).
  * sgs: getTauSGS / getRHS_SGS (sgsmod_igrid.F90:157-265), Smagorinsky kernel and Sij
    (smagorinsky.F90:39-67, eddyViscosity.F90:1-117), deltaLES for periodic z, standard
    dynamic procedure with planar averages (standardDynamicProcedure.F90:74-244).  The
    test filter is the x-y sharp cutoff of spectral.F90:1333-1367 at (2/3)(pi/dx)/deltaRatio;
    the reference refuses it for periodic-z problems (GracefulExit 1233), so the dynamic
    procedure in this configuration is pinned by this restatement alone.
Arrays are Fortran-shaped (i, j, k); C fields have nz planes, E fields nz+1 (plane nz+1 =
plane 1).  FFTs are numpy's standing in for FFTW; the z operators are the C oracle's.
"""
import numpy as np

from oracle import oracle as C
from oracle.spectral_oracle import GetWaveNums, getmodCD06stagg  # noqa: F401


def _sz(f, nz, dz, op):
    """Periodic staggered CD06 z operator on a real or complex (i, j, k) array."""
    if np.iscomplexobj(f):
        return C.stagg(np.ascontiguousarray(f.real), nz, dz, op, periodic=True) + \
            1j * C.stagg(np.ascontiguousarray(f.imag), nz, dz, op, periodic=True)
    return C.stagg(f, nz, dz, op, periodic=True)


class LesOracle:
    def __init__(self, nx, ny, nz, Lx, Ly, Lz, Re=1000.0, CFL=0.5, dynamic=True, Csgs=0.17, deltaRatio=2.0,
                 DynProcFreq=1, dealiasFact=2.0 / 3.0, t_DivergenceCheck=10, useSGS=True, isInviscid=False,
                 SGSModelID=0):
        self.nx, self.ny, self.nz = nx, ny, nz
        self.dx, self.dy, self.dz = Lx / nx, Ly / ny, Lz / nz
        self.Re, self.CFL = Re, CFL
        self.dynamic, self.useSGS, self.isInviscid = dynamic, useSGS, isInviscid
        self.DynProcFreq, self.t_DivergenceCheck = DynProcFreq, t_DivergenceCheck
        nxh = nx // 2 + 1
        k1 = GetWaveNums(nx, self.dx)
        k2 = GetWaveNums(ny, self.dy)
        k3 = GetWaveNums(nz, self.dz)
        k1[nx // 2] = -k1[nx // 2]
        k2[ny // 2] = -k2[ny // 2]
        k3[nz // 2] = -k3[nz // 2]
        self.k1, self.k2, self.k3 = k1[:nxh], k2, k3
        K1, K2 = self.k1[:, None, None], self.k2[None, :, None]
        self.kabs_sq = K1 ** 2 + K2 ** 2
        pi = np.pi
        kdx, kdy, kdz = dealiasFact * pi / self.dx, dealiasFact * pi / self.dy, dealiasFact * pi / self.dz
        G = np.ones((nxh, ny, nz))
        G[np.abs(self.k1) >= kdx, :, :] = 0.0
        G[:, np.abs(self.k2) >= kdy, :] = 0.0
        G[:, :, np.abs(self.k3) >= kdz] = 0.0
        self.Gdealias = G
        kfx = ((2.0 / 3.0) * pi / self.dx) / deltaRatio
        kfy = ((2.0 / 3.0) * pi / self.dy) / deltaRatio
        self.GTestFilt = ((np.abs(self.k1)[:, None] < kfx) & (np.abs(self.k2)[None, :] < kfy)).astype(float)[:, :, None]
        self.deltaRat = deltaRatio
        deltaLES = (1.5 * self.dx * 1.5 * self.dy * 1.5 * self.dz) ** (1.0 / 3.0)
        self.cmodel_global = (Csgs * deltaLES) ** 2
        self.SGSModelID = SGSModelID
        assert SGSModelID == 0 or not dynamic, "sigma / AMD with constant coefficients only"
        if SGSModelID == 2:  # AMD.F90:1-14
            self.camd = (Csgs * self.dx * np.sqrt(1.0 / 12.0), Csgs * self.dy * np.sqrt(1.0 / 12.0),
                         Csgs * self.dz * (1.0 / np.sqrt(10.0)))
            self.cmodel_global = 1.0
        self.meanfact = 1.0 / (float(nx) * float(ny))
        # Poisson (PadePoisson.F90:76-128): raw wavenumbers, CD06-stagg modified k3
        k1r = GetWaveNums(nx, self.dx)[:nxh]
        k2r = GetWaveNums(ny, self.dy)
        k3m = getmodCD06stagg(GetWaveNums(nz, self.dz), self.dz)
        kr = (k1r[:, None, None] ** 2 + k2r[None, :, None] ** 2) + k3m[None, None, :] ** 2
        with np.errstate(divide="ignore"):
            self.kradsq_inv = np.where(kr <= 1e-14, 0.0, 1.0 / kr)
        self.step = 0
        self.mstep = 0
        self.tsim = 0.0
        self.newTimeStep = True
        self.lambda1d = np.zeros(nz)

    # ---------------------------------------------------------------- spectral helpers
    def fft(self, f):
        return np.fft.fft(np.fft.rfft(f, axis=0), axis=1)

    def ifft(self, fh):
        return np.fft.irfft(np.fft.ifft(fh, axis=1), n=self.nx, axis=0)

    def ik1(self, fh):
        return 1j * self.k1[:, None, None] * fh

    def ik2(self, fh):
        return 1j * self.k2[None, :, None] * fh

    def dealias(self, fh):
        return np.fft.ifft(np.fft.fft(fh, axis=2) * self.Gdealias, axis=2)

    def dealias_edge(self, fh):
        g = self.dealias(fh[:, :, : self.nz])
        return np.concatenate([g, g[:, :, :1]], axis=2)

    def sz(self, f, op):
        return _sz(f, self.nz, self.dz, op)

    def test_filter_r2r(self, f):
        return self.ifft(self.fft(f) * self.GTestFilt)

    # ---------------------------------------------------------------- Poisson
    def projection(self, uh, vh, wh):
        K1, K2 = self.k1[:, None, None], self.k2[None, :, None]
        f = self.sz(wh, "ddz_E2C") + 1j * (K1 * uh + K2 * vh)
        p = np.fft.ifft(-self.kradsq_inv * np.fft.fft(f, axis=2), axis=2)
        return uh - 1j * K1 * p, vh - 1j * K2 * p, wh - self.sz(p, "ddz_C2E")

    def divergence(self, uh, vh, wh):
        K1, K2 = self.k1[:, None, None], self.k2[None, :, None]
        return self.ifft(self.sz(wh, "ddz_E2C") + 1j * K1 * uh + 1j * K2 * vh)

    def divergence_check_fix(self, uh, vh, wh):
        div = self.divergence(uh, vh, wh)
        if div.max() > 1e-13:
            uh, vh, wh = self.projection(uh, vh, wh)
            div = self.divergence(uh, vh, wh)
            if div.max() > 1e-10:
                uh, vh, wh = self.projection(uh, vh, wh)
        return uh, vh, wh

    # ---------------------------------------------------------------- igrid pieces
    def init_fields(self, u, v, w):
        """igrid.F90:625-648 with physical u, v (nz planes) and w (nz+1 planes)."""
        uh, vh, wh = self.fft(u), self.fft(v), self.fft(w)
        uh, vh, wh = self.dealias(uh), self.dealias(vh), self.dealias_edge(wh)
        uh, vh, wh = self.projection(uh, vh, wh)
        self.uhat, self.vhat, self.what = uh, vh, wh
        self._prep_physical()

    def _prep_physical(self):
        self.u, self.v, self.w = self.ifft(self.uhat), self.ifft(self.vhat), self.ifft(self.what)
        # interp_PrimitiveVars
        self.whatC = self.sz(self.what, "InterpZ_E2C")
        self.wC = self.ifft(self.whatC)
        self.uEhat = self.sz(self.uhat, "InterpZ_C2E")
        self.uE = self.ifft(self.uEhat)
        self.vEhat = self.sz(self.vhat, "InterpZ_C2E")
        self.vE = self.ifft(self.vEhat)
        self.compute_duidxj()

    def compute_duidxj(self):
        uh, vh, wh = self.uhat, self.vhat, self.what
        C_ = [None] * 9
        E_ = [None] * 9
        C_[0] = self.ifft(self.ik1(uh)); E_[0] = self.ifft(self.ik1(self.uEhat))
        C_[1] = self.ifft(self.ik2(uh)); E_[1] = self.ifft(self.ik2(self.uEhat))
        C_[3] = self.ifft(self.ik1(vh)); E_[3] = self.ifft(self.ik1(self.vEhat))
        C_[4] = self.ifft(self.ik2(vh)); E_[4] = self.ifft(self.ik2(self.vEhat))
        C_[6] = self.ifft(self.ik1(self.whatC)); E_[6] = self.ifft(self.ik1(wh))
        C_[7] = self.ifft(self.ik2(self.whatC)); E_[7] = self.ifft(self.ik2(wh))
        dwdzH = self.sz(wh, "ddz_E2C")
        C_[8] = self.ifft(dwdzH)
        E_[8] = self.ifft(self.sz(dwdzH, "InterpZ_C2E"))
        self.d2wdz2hatE = self.sz(wh, "d2dz2_E2E")
        dudzEH = self.sz(uh, "ddz_C2E")
        E_[2] = self.ifft(dudzEH)
        self.d2udz2hatC = self.sz(uh, "d2dz2_C2C")
        C_[2] = self.ifft(self.sz(dudzEH, "InterpZ_E2C"))
        dvdzEH = self.sz(vh, "ddz_C2E")
        E_[5] = self.ifft(dvdzEH)
        self.d2vdz2hatC = self.sz(vh, "d2dz2_C2C")
        C_[5] = self.ifft(self.sz(dvdzEH, "InterpZ_E2C"))
        self.duidxjC, self.duidxjE = C_, E_

    def compute_deltaT(self):
        rb1 = np.abs((1.0 / self.dx) * self.u) + np.abs((1.0 / self.dy) * self.v)
        rb1 = rb1 + np.abs((1.0 / self.dz) * self.wC)
        dt = self.CFL / rb1.max()
        if not self.isInviscid:
            dt = min(dt, self.CFL * self.Re * min(self.dx, self.dy, self.dz) ** 2)
        self.dt = dt
        return dt

    @staticmethod
    def sij(d):
        return [d[0], 0.5 * (d[1] + d[3]), 0.5 * (d[2] + d[6]), d[4], 0.5 * (d[5] + d[7]), d[8]]

    @staticmethod
    def smag_kernel(S):
        s = S[0] * S[0]
        s = s + 2.0 * (S[1] * S[1])
        s = s + 2.0 * (S[2] * S[2])
        s = s + S[3] * S[3]
        s = s + 2.0 * (S[4] * S[4])
        s = s + S[5] * S[5]
        return np.sqrt(2.0 * s)

    @staticmethod
    def sigma_kernel(d):
        """sigma.F90:30-95, in the reference's operation order."""
        G11 = d[0] * d[0] + d[3] * d[3] + d[6] * d[6]
        G12 = d[0] * d[1] + d[3] * d[4] + d[6] * d[7]
        G13 = d[0] * d[2] + d[3] * d[5] + d[6] * d[8]
        G22 = d[1] * d[1] + d[4] * d[4] + d[7] * d[7]
        G23 = d[1] * d[2] + d[4] * d[5] + d[7] * d[8]
        G33 = d[2] * d[2] + d[5] * d[5] + d[8] * d[8]
        I1 = G11 + G22 + G33
        I1sq = I1 * I1
        I1cu = I1sq * I1
        I2 = -(G11 * G11) - G22 * G22 - G33 * G33
        I2 = I2 - 2.0 * G12 * G12 - 2.0 * G13 * G13
        I2 = I2 - 2.0 * G23 * G23
        I2 = I2 + I1sq
        I2 = 0.5 * I2
        I3 = G11 * (G22 * G33 - G23 * G23)
        I3 = I3 + G12 * (G13 * G23 - G12 * G33)
        I3 = I3 + G13 * (G12 * G23 - G22 * G13)
        a1 = np.maximum(I1sq / 9.0 - I2 / 3.0, 0.0)
        a2 = I1cu / 27.0 - I1 * I2 / 6.0 + I3 / 2.0
        a1s = np.sqrt(a1)
        t = a2 / (a1 * a1s + 1e-13)
        t = np.maximum(np.minimum(t, 1.0), -1.0)
        a3 = (1.0 / 3.0) * np.arccos(t)
        s1sq = np.maximum(I1 / 3.0 + 2.0 * a1s * np.cos(a3), 0.0)
        s1 = np.sqrt(s1sq)
        s2 = np.sqrt(np.maximum((-2.0) * a1s * np.cos(np.pi / 3.0 + a3) + I1 / 3.0, 0.0))
        s3 = np.sqrt(np.maximum((-2.0) * a1s * np.cos(np.pi / 3.0 - a3) + I1 / 3.0, 0.0))
        return s3 * (s1 - s2) * (s2 - s3) / (s1sq + 1e-15)

    @staticmethod
    def amd_kernel(d, S, camd):
        """AMD.F90:23-72, in the reference's operation order."""
        cx, cy, cz = camd

        def dot(r, q):
            return ((d[3 * r] * cx) * (d[3 * q] * cx) + (d[3 * r + 1] * cy) * (d[3 * q + 1] * cy)
                    + (d[3 * r + 2] * cz) * (d[3 * q + 2] * cz))

        num = dot(0, 0) * S[0]
        num = num + dot(1, 1) * S[3]
        num = num + dot(2, 2) * S[5]
        num = num + 2.0 * dot(0, 1) * S[1]
        num = num + 2.0 * dot(0, 2) * S[2]
        num = num + 2.0 * dot(1, 2) * S[4]
        den = d[0] * d[0]
        for i in range(1, 9):
            den = den + d[i] * d[i]
        return np.maximum(-num / (den + 1e-32), 0.0)

    def dynamic_procedure(self, SC, Dsgs):
        """DoStandardDynamicProcedure (standardDynamicProcedure.F90:74-165) -> lambda(z)."""
        Sf = [self.test_filter_r2r(s) for s in SC]
        Df = self.smag_kernel(Sf)
        dr2 = self.deltaRat * self.deltaRat
        M = [self.test_filter_r2r(Dsgs * SC[i]) - dr2 * Df * Sf[i] for i in range(6)]
        G = self.GTestFilt
        uf = [self.ifft(self.uhat * G), self.ifft(self.vhat * G), self.ifft(self.whatC * G)]
        u, v, w = self.u, self.v, self.wC
        prods = [(u, u, 0, 0), (u, v, 0, 1), (u, w, 0, 2), (v, v, 1, 1), (v, w, 1, 2), (w, w, 2, 2)]
        Lij = [self.test_filter_r2r(a * b) - uf[i] * uf[j] for a, b, i, j in prods]
        num = Lij[0] * M[0]
        for i in range(1, 6):
            num = num + Lij[i] * M[i]
        num = num + Lij[1] * M[1] + Lij[2] * M[2] + Lij[4] * M[4]
        den = M[0] * M[0]
        for i in range(1, 6):
            den = den + M[i] * M[i]
        den = den + M[1] * M[1] + M[2] * M[2] + M[4] * M[4]
        den = 2.0 * den
        nm = np.maximum(num.sum(axis=(0, 1)) * self.meanfact, 0.0)
        self.lambda1d = nm / (den.sum(axis=(0, 1)) * self.meanfact + 1e-18)

    def scalar_sgs_rhs(self, T, That, dT, dTdzE, Trhs, Pr=1.0, dynamic=False, fields=None):
        """getRHS_SGS_Scalar / getQjSGS (sgsmod_igrid.F90:268-335) and, when dynamic,
        DoStandardDynamicProcedureScalar (standardDynamicProcedure.F90:1-71) with
        planarAverage_and_TakeRatio (221-244).  fields: the LES state to use, a dict with u, v,
        wC, uhat, vhat, whatC (spectral at the cells), duidxjC (9 arrays), nuC, nuE; dT the
        three cell gradients of T.  Returns (Trhs, Beta(z) or None)."""
        F = fields
        beta = None
        if dynamic:
            SC = self.sij(F["duidxjC"])
            Dsgs = self.smag_kernel(SC)                       # |S| (the Smagorinsky kernel)
            Sf = [self.test_filter_r2r(s) for s in SC]
            Df = self.smag_kernel(Sf)                         # |S| of the filtered strain
            G = self.GTestFilt
            uf = [self.ifft(F["uhat"] * G), self.ifft(F["vhat"] * G), self.ifft(F["whatC"] * G)]
            dr2 = self.deltaRat * self.deltaRat
            dTf = [self.test_filter_r2r(g) for g in dT]                                     # step 1
            R = [self.test_filter_r2r(Dsgs * dT[i]) - dr2 * Df * dTf[i] for i in range(3)]    # step 3
            Tf = self.ifft(That * G)                                                          # step 4
            U = [F["u"], F["v"], F["wC"]]
            Pf = [self.test_filter_r2r(U[i] * T) - uf[i] * Tf for i in range(3)]              # step 5
            num = R[0] * Pf[0] + R[1] * Pf[1] + R[2] * Pf[2]
            den = R[0] * R[0] + R[1] * R[1] + R[2] * R[2]
            nm = np.maximum(num.sum(axis=(0, 1)) * self.meanfact, 0.0)
            beta = nm / (den.sum(axis=(0, 1)) * self.meanfact + 1e-18)
            kC = Dsgs * beta[None, None, :]
            kE = self.sz(kC, "InterpZ_C2E")                   # interpolate_kappaSGS
        else:
            kC, kE = F["nuC"] / Pr, F["nuE"] / Pr
        q1, q2, q3 = -kC * dT[0], -kC * dT[1], -kE * dTdzE
        Trhs = Trhs - self.ik1(self.fft(q1))
        Trhs = Trhs - self.ik2(self.fft(q2))
        Trhs = Trhs - self.sz(self.fft(q3), "ddz_E2C")
        return Trhs, beta

    def sgs_rhs(self, urhs, vrhs, wrhs):
        SC = self.sij(self.duidxjC)
        SE = self.sij(self.duidxjE)
        if self.SGSModelID == 1:
            nuC = self.sigma_kernel(self.duidxjC)
        elif self.SGSModelID == 2:
            nuC = self.amd_kernel(self.duidxjC, SC, self.camd)
        else:
            nuC = self.smag_kernel(SC)
        if self.dynamic:
            if self.newTimeStep:
                Dsgs = nuC.copy()
                if self.mstep % self.DynProcFreq == 0:
                    self.dynamic_procedure(SC, Dsgs)
            nuC = self.lambda1d[None, None, :] * nuC
            nuE = self.sz(nuC, "InterpZ_C2E")
        else:
            nuC = self.cmodel_global * nuC
            nuE = np.maximum(self.sz(nuC, "InterpZ_C2E"), 0.0)
        t11, t12, t22, t33 = -2.0 * nuC * SC[0], -2.0 * nuC * SC[1], -2.0 * nuC * SC[3], -2.0 * nuC * SC[5]
        t13, t23 = -2.0 * nuE * SE[2], -2.0 * nuE * SE[4]
        if self.newTimeStep:
            self.mstep += 1
        urhs = urhs - self.ik1(self.fft(t11))
        vrhs = vrhs - self.ik2(self.fft(t22))
        wrhs = wrhs - self.sz(self.fft(t33), "ddz_C2E")
        c = self.fft(t12)
        vrhs = vrhs - self.ik1(c)
        urhs = urhs - self.ik2(c)
        c = self.fft(t13)
        urhs = urhs - self.sz(c, "ddz_E2C")
        wrhs = wrhs - self.ik1(c)
        c = self.fft(t23)
        vrhs = vrhs - self.sz(c, "ddz_E2C")
        wrhs = wrhs - self.ik2(c)
        return urhs, vrhs, wrhs

    def populate_rhs(self):
        dC, dE = self.duidxjC, self.duidxjE
        dudy, dvdx = dC[1], dC[3]
        dwdx, dwdy, dudz, dvdz = dE[6], dE[7], dE[2], dE[5]
        fT1C = self.fft((dvdx - dudy) * self.v)
        fT2E = self.fft((dwdx - dudz) * self.w)
        urhs = self.sz(fT2E, "InterpZ_E2C") + fT1C
        fT1C = self.fft((dudy - dvdx) * self.u)
        fT2E = self.fft((dwdy - dvdz) * self.w)
        vrhs = self.sz(fT2E, "InterpZ_E2C") + fT1C
        wrhs = self.fft((dudz - dwdx) * self.uE + (dvdz - dwdy) * self.vE)
        if not self.isInviscid:
            r = 1.0 / self.Re
            urhs = urhs + r * (-self.kabs_sq * self.uhat + self.d2udz2hatC)
            vrhs = vrhs + r * (-self.kabs_sq * self.vhat + self.d2vdz2hatC)
            wrhs = wrhs + r * (-self.kabs_sq * self.what + self.d2wdz2hatE)
        if self.useSGS:
            urhs, vrhs, wrhs = self.sgs_rhs(urhs, vrhs, wrhs)
        return urhs, vrhs, wrhs

    def project_and_prep(self):
        self.uhat, self.vhat = self.dealias(self.uhat), self.dealias(self.vhat)
        self.what = self.dealias_edge(self.what)
        self.uhat, self.vhat, self.what = self.projection(self.uhat, self.vhat, self.what)
        if self.step % self.t_DivergenceCheck == 0:
            self.uhat, self.vhat, self.what = self.divergence_check_fix(self.uhat, self.vhat, self.what)
        self._prep_physical()

    def tvd_rk3(self, dt=None):
        """One time step; returns dt."""
        dt = self.compute_deltaT() if dt is None else dt
        self.dt = dt
        u0, v0, w0 = self.uhat, self.vhat, self.what
        ur, vr, wr = self.populate_rhs()
        self.newTimeStep = False
        u1, v1, w1 = u0 + dt * ur, v0 + dt * vr, w0 + dt * wr
        self.uhat, self.vhat, self.what = u1, v1, w1
        self.project_and_prep()
        u1, v1, w1 = self.uhat, self.vhat, self.what
        ur, vr, wr = self.populate_rhs()
        u1 = (3.0 / 4.0) * u0 + (1.0 / 4.0) * u1 + (1.0 / 4.0) * dt * ur
        v1 = (3.0 / 4.0) * v0 + (1.0 / 4.0) * v1 + (1.0 / 4.0) * dt * vr
        w1 = (3.0 / 4.0) * w0 + (1.0 / 4.0) * w1 + (1.0 / 4.0) * dt * wr
        self.uhat, self.vhat, self.what = u1, v1, w1
        self.project_and_prep()
        u1, v1, w1 = self.uhat, self.vhat, self.what
        ur, vr, wr = self.populate_rhs()
        self.uhat = (1.0 / 3.0) * u0 + (2.0 / 3.0) * u1 + (2.0 / 3.0) * dt * ur
        self.vhat = (1.0 / 3.0) * v0 + (2.0 / 3.0) * v1 + (2.0 / 3.0) * dt * vr
        self.what = (1.0 / 3.0) * w0 + (2.0 / 3.0) * w1 + (2.0 / 3.0) * dt * wr
        self.project_and_prep()
        self.step += 1
        self.tsim += dt
        self.newTimeStep = True
        return dt
