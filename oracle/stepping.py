"""CPU ORACLE -- test infrastructure only.

NumPy restatement of PyQuake3D's dense quasi-dynamic stepping, used by the
tests as the checker for the GPU stepper and by bench.py's CPU-baseline leg.
Nothing in the product path imports this module.

Followed line by line (reference file:line):
  * initial state from a per-cell table  src/QDsim_gpu.py:714-770 (read_parameter)
  * right-hand side                      src/QDsim_gpu.py:772-828 (derivative)
  * Dormand-Prince 5(4) attempt          src/QDsim_gpu.py:1266-1397
  * step control and state update        src/QDsim_gpu.py:1029-1122 (simu_forward)
  * pore-pressure dilatancy (optional)   src/QDsim_gpu.py:332-349 (set-up), 611-626
                                         (Calc_Pmatrix), 628-671 (Calc_P_implicit, after
                                         every accepted step, 1119-1120)

Quirks kept on purpose: the traction product K.(V - Vpl) and the slip rate in
the aging law are frozen at the step start; 7 right-hand-side evaluations per
attempt; the error norm is the max relative difference of the 5th- and
4th-order solutions over (psi, tau1, tau2, sigma) with a 1e-10 floor;
RelTol = 1e-4.  Where the reference calls sys.exit (dt < 1e-15 or more than 20
rejections) this raises :class:`StepFailure`.
"""
from __future__ import annotations

import numpy as np

# Dormand-Prince tableau (src/QDsim_gpu.py:1268-1300)
B21 = .2
B31, B32 = 3. / 40, 9. / 40.
B41, B42, B43 = 44. / 45., -56. / 15, 32. / 9
B51, B52, B53, B54 = 19372. / 6561., -25360 / 2187., 64448. / 6561., -212. / 729.
B61, B62, B63, B64, B65 = 9017. / 3168., -355. / 33., -46732. / 5247., 49. / 176., -5103. / 18656.
B71, B73, B74, B75, B76 = 35. / 384., 500. / 1113., 125. / 192., -2187. / 6784., 11. / 84.
B81, B83, B84, B85, B86, B87 = 5179. / 57600., 7571. / 16695., 393. / 640., -92097. / 339200., 187. / 2100., 1. / 40.

REL_TOL = 1e-4


class StepFailure(RuntimeError):
    """dt fell below 1e-15 or more than 20 attempts were rejected."""


def _safe_exp(x, m=700):
    return np.exp(np.clip(x, -m, m))


def _safe_cosh(x, m=700):
    x = np.clip(x, -m, m)
    return (np.exp(x) + np.exp(-x)) / 2


def _safe_sinh(x, m=700):
    x = np.clip(x, -m, m)
    return (np.exp(x) - np.exp(-x)) / 2


class DenseStepper:
    """State and stepping of one dense simulation.

    K: dict with the six N x N operators 'A1s','A2s','Bs','A1d','A2d','Bd'
    (row = receiver, column = source).  table: (N, 10) per-cell table.
    """

    def __init__(self, K, table, *, mu, density, V0=1e-6, Vpl=1e-9, fix_Tn=False, dilatancy=None):
        """dilatancy: None, or dict with the parameter-file values 'Dilatancy
        coefficient', 'Hydraulic diffusivity', 'Actively shearing zone
        thickness', 'Effective compressibility', 'Constant porepressure' and
        'Initial porepressure' (MPa)."""
        self.K = K
        self.mu = float(mu)
        self.Cs = np.sqrt(self.mu / float(density))
        self.V0 = float(V0)
        self.Vpl_con = float(Vpl)
        self.fix_Tn = bool(fix_Tn)
        N = table.shape[0]
        self.P = np.zeros(N)
        self.dPdt0 = np.zeros(N)
        self.Ifdila = dilatancy is not None
        if self.Ifdila:
            self._setup_dilatancy(dilatancy, N)
        self.slipvC = np.ones(N) * self.Vpl_con
        self.time = 0.0
        self._read_parameter(table)
        self.slip1 = np.zeros(N)
        self.slip2 = np.zeros(N)
        self.slip = np.zeros(N)

    # src/QDsim_gpu.py:332-349, 161-165
    def _setup_dilatancy(self, d, N):
        self.DilatancyC = float(d["Dilatancy coefficient"])
        self.Chyd = float(d["Hydraulic diffusivity"])
        self.hs = float(d["Actively shearing zone thickness"])
        self.EPermeability = float(d["Effective compressibility"])
        c = 1e-2
        num = 60
        self.P0 = float(d["Constant porepressure"]) * 1e6
        self.P = np.ones(N) * float(d["Initial porepressure"]) * 1e6
        yp = np.logspace(start=-3, stop=10, num=num, base=10)
        self.zp = np.log(1 + yp / c)
        self.Parr = np.ones([N, num]) * float(d["Initial porepressure"]) * 1e6
        self.Pmatrix = np.zeros([num, num])
        self._calc_pmatrix()

    # src/QDsim_gpu.py:611-626
    def _calc_pmatrix(self):
        K = len(self.zp)
        z = self.zp
        c = self.Chyd
        dz = np.diff(self.zp)
        for i in range(K - 1):
            if i == 0:
                self.Pmatrix[0, 0] = c * (np.exp(-(2 * z[0] - dz[0] / 2)) + np.exp(-(2 * z[0] + dz[0] / 2))) / (dz[0] * dz[0])
                self.Pmatrix[0, 1] = -c * (np.exp(-(2 * z[0] - dz[0] / 2)) + np.exp(-(2 * z[0] + dz[0] / 2))) / (dz[0] * dz[0])
            else:
                self.Pmatrix[i, i] = c * (np.exp(-(2 * z[i] - dz[i] / 2)) + np.exp(-(2 * z[i] + dz[i] / 2))) / (dz[i] * dz[i])
                self.Pmatrix[i, i + 1] = -c * np.exp(-(2 * z[i] + dz[i] / 2)) / (dz[i] * dz[i])
                self.Pmatrix[i, i - 1] = -c * np.exp(-(2 * z[i] - dz[i] / 2)) / (dz[i] * dz[i])

    # src/QDsim_gpu.py:628-671: one implicit step of the fault-normal pore
    # pressure diffusion per cell, flux from the dilatant state evolution
    def calc_p_implicit(self, dt):
        from scipy.linalg import lu_factor, lu_solve
        e, h, beta, c_hyd, dc, z = self.DilatancyC, self.hs, self.EPermeability, self.Chyd, self.dc, self.zp
        dz = np.diff(z)
        K = len(z)
        dt = float(dt)
        M = self.Pmatrix[:-1, :-1] * dt + np.eye(K - 1)
        lu, piv = lu_factor(M)
        theta = self.dc / self.V0 * np.exp((self.state - self.f0) / self.b)
        dthetadt = 1.0 - self.slipv * theta / dc
        g = -e * h / (2.0 * beta * c_hyd * theta) * dthetadt
        for i in range(self.Tno.shape[0]):
            b = np.copy(self.Parr[i, :-1])
            b[0] = b[0] - 2.0 * c_hyd * np.exp(-(z[0] - dz[0] / 2)) * g[i] * dt / dz[0]
            b[-1] = b[-1] + dt / (dz[-1] * dz[-1]) * c_hyd * np.exp(-(z[-2] - dz[-1] / 2)) * self.P0
            x = lu_solve((lu, piv), b)
            self.Parr[i, :-1] = np.copy(x)
            term1 = -np.exp(-(z[0] - dz[0] / 2)) * (self.Parr[i, 0] - self.Parr[i, 1] + 2 * dz[0] * g[i] * np.exp(z[0]))
            term2 = np.exp(-(z[0] + dz[0] / 2)) * (self.Parr[i, 1] - self.Parr[i, 0])
            self.dPdt0[i] = c_hyd * np.exp(-z[0]) * (term1 + term2) / dz[0] ** 2
            self.P[i] = self.Parr[i, 0]

    # src/QDsim_gpu.py:714-770
    def _read_parameter(self, values):
        self.rake = values[:, 0].copy()
        self.a = values[:, 1].copy()
        self.b = values[:, 2].copy()
        self.dc = values[:, 3].copy()
        self.f0 = values[:, 4].copy()
        self.Tno = values[:, 6].copy()
        self.slipv = values[:, 7].copy()
        self.shear_loading = values[:, 8].copy()
        self.normal_loading = values[:, 9].copy()
        x = np.cos(self.rake)
        y = np.sin(self.rake)
        self.slipv1 = self.slipv * x + 1e-16
        self.slipv2 = self.slipv * y + 1e-16
        self.Tt = (self.Tno - self.P * 1e-6) * self.a * np.arcsinh(
            self.slipv / (2.0 * self.V0) * np.exp((self.f0 + self.b * np.log(self.V0 / self.slipvC)) / self.a))
        self.Tt1o = self.Tt * x
        self.Tt2o = self.Tt * y
        self.fric = self.Tt / (self.Tno - self.P * 1e-6)
        self.state = np.log(np.sinh(self.Tt / (self.Tno - self.P * 1e-6) / self.a) * 2.0 * self.V0 / self.slipv) * self.a
        self.maxslipv0 = np.max(self.slipv)
        self.rake0 = np.copy(self.rake)

    # src/QDsim_gpu.py:772-828
    def derivative(self, Tno, Tt1o, Tt2o, state):
        Tno = Tno * 1e6
        Tt1o = Tt1o * 1e6
        Tt2o = Tt2o * 1e6
        P = self.P
        dPdt = self.dPdt0
        V0, a, b, dc, f0 = self.V0, self.a, self.b, self.dc, self.f0
        dV1dtau = 2 * V0 / (a * (Tno - P)) * _safe_exp(-state / a) * _safe_cosh(Tt1o / (a * (Tno - P)))
        dV2dtau = 2 * V0 / (a * (Tno - P)) * _safe_exp(-state / a) * _safe_cosh(Tt2o / (a * (Tno - P)))
        dV1dsigma = -2 * V0 * Tt1o / (a * (Tno - P) ** 2) * _safe_exp(-state / a) * _safe_cosh(Tt1o / (a * (Tno - P)))
        dV2dsigma = -2 * V0 * Tt2o / (a * (Tno - P) ** 2) * _safe_exp(-state / a) * _safe_cosh(Tt2o / (a * (Tno - P)))
        dV1dstate = -2 * V0 / a * _safe_exp(-state / a) * _safe_sinh(Tt1o / (a * (Tno - P)))
        dV2dstate = -2 * V0 / a * _safe_exp(-state / a) * _safe_sinh(Tt2o / (a * (Tno - P)))
        dstatedt = b / dc * (V0 * _safe_exp((f0 - state) / b) - self.slipv)
        eta = self.mu / (2.0 * self.Cs)
        dtau1dt = (-self.AdotV1 + self.shear_loading - eta * (dV1dsigma * (self.dsigmadt - dPdt) + dV1dstate * dstatedt)) / (1.0 + eta * dV1dtau)
        dtau2dt = (-self.AdotV2 + self.shear_loading - eta * (dV2dsigma * (self.dsigmadt - dPdt) + dV2dstate * dstatedt)) / (1.0 + eta * dV2dtau)
        return dstatedt, self.dsigmadt / 1e6, dtau1dt / 1e6, dtau2dt / 1e6

    # src/QDsim_gpu.py:1266-1397
    def rk_attempt_raw(self, h):
        """The seven stages; returns the 5th-order candidate and the two raw
        error maxima (before the 1e-10 floor) over this object's cells."""
        d = self.derivative
        Tno, Tt1o, Tt2o, state = self.Tno, self.Tt1o, self.Tt2o, self.state
        s1, n1, t1, u1 = d(Tno, Tt1o, Tt2o, state)
        s2, n2, t2, u2 = d(Tno + h * B21 * n1, Tt1o + h * B21 * t1, Tt2o + h * B21 * u1, state + h * B21 * s1)
        s3, n3, t3, u3 = d(Tno + h * (B31 * n1 + B32 * n2), Tt1o + h * (B31 * t1 + B32 * t2),
                           Tt2o + h * (B31 * u1 + B32 * u2), state + h * (B31 * s1 + B32 * s2))
        s4, n4, t4, u4 = d(Tno + h * (B41 * n1 + B42 * n2 + B43 * n3), Tt1o + h * (B41 * t1 + B42 * t2 + B43 * t3),
                           Tt2o + h * (B41 * u1 + B42 * u2 + B43 * u3), state + h * (B41 * s1 + B42 * s2 + B43 * s3))
        s5, n5, t5, u5 = d(Tno + h * (B51 * n1 + B52 * n2 + B53 * n3 + B54 * n4),
                           Tt1o + h * (B51 * t1 + B52 * t2 + B53 * t3 + B54 * t4),
                           Tt2o + h * (B51 * u1 + B52 * u2 + B53 * u3 + B54 * u4),
                           state + h * (B51 * s1 + B52 * s2 + B53 * s3 + B54 * s4))
        s6, n6, t6, u6 = d(Tno + h * (B61 * n1 + B62 * n2 + B63 * n3 + B64 * n4 + B65 * n5),
                           Tt1o + h * (B61 * t1 + B62 * t2 + B63 * t3 + B64 * t4 + B65 * t5),
                           Tt2o + h * (B61 * u1 + B62 * u2 + B63 * u3 + B64 * u4 + B65 * u5),
                           state + h * (B61 * s1 + B62 * s2 + B63 * s3 + B64 * s4 + B65 * s5))
        Tno_y = Tno + h * (B71 * n1 + B73 * n3 + B74 * n4 + B75 * n5 + B76 * n6)
        Tt1o_y = Tt1o + h * (B71 * t1 + B73 * t3 + B74 * t4 + B75 * t5 + B76 * t6)
        Tt2o_y = Tt2o + h * (B71 * u1 + B73 * u3 + B74 * u4 + B75 * u5 + B76 * u6)
        state_y = state + h * (B71 * s1 + B73 * s3 + B74 * s4 + B75 * s5 + B76 * s6)
        s7, n7, t7, u7 = d(Tno_y, Tt1o_y, Tt2o_y, state_y)
        Tno_8 = Tno + h * (B81 * n1 + B83 * n3 + B84 * n4 + B85 * n5 + B86 * n6 + B87 * n7)
        Tt1o_8 = Tt1o + h * (B81 * t1 + B83 * t3 + B84 * t4 + B85 * t5 + B86 * t6 + B87 * t7)
        Tt2o_8 = Tt2o + h * (B81 * u1 + B83 * u3 + B84 * u4 + B85 * u5 + B86 * u6 + B87 * u7)
        state_8 = state + h * (B81 * s1 + B83 * s3 + B84 * s4 + B85 * s5 + B86 * s6 + B87 * s7)
        m1 = np.max(np.abs(np.abs(state_8 - state_y) / state_8))
        e2a = np.max(np.abs(np.abs(Tt1o_8 - Tt1o_y) / Tt1o_8))
        e2b = np.max(np.abs(np.abs(Tt2o_8 - Tt2o_y) / Tt2o_8))
        e2c = np.max(np.abs(np.abs(Tno_8 - Tno_y) / Tno_8))
        return Tno_y, Tt1o_y, Tt2o_y, state_y, m1, max(e2a, e2b, e2c)

    @staticmethod
    def step_control(h, m1, m2):
        """(c1, c2, hn1, hn2) from the raw error maxima."""
        err1 = m1 + 1e-10
        err2 = m2 + 1e-10
        c1 = err1 / REL_TOL
        c2 = err2 / REL_TOL
        hn1 = h * 0.9 * (REL_TOL / err1) ** 0.2
        hn2 = h * 0.9 * (REL_TOL / err2) ** 0.2
        return c1, c2, hn1, hn2

    def rk_attempt(self, h):
        Tno_y, Tt1o_y, Tt2o_y, state_y, m1, m2 = self.rk_attempt_raw(h)
        return (Tno_y, Tt1o_y, Tt2o_y, state_y) + self.step_control(h, m1, m2)

    def traction_rates(self):
        """K.(V - Vpl) once per accepted step (src/QDsim_gpu.py:1033-1042)."""
        K = self.K
        v1 = self.slipv1 - self.Vpl_con * np.cos(self.rake0)
        v2 = self.slipv2 - self.Vpl_con * np.sin(self.rake0)
        if self.fix_Tn:
            self.dsigmadt = self.normal_loading
        else:
            self.dsigmadt = np.dot(K['Bs'], v1) + np.dot(K['Bd'], v2) + self.normal_loading
        self.AdotV1 = np.dot(K['A1s'], v1) + np.dot(K['A1d'], v2)
        self.AdotV2 = np.dot(K['A2s'], v1) + np.dot(K['A2d'], v2)

    # src/QDsim_gpu.py:1029-1122
    def simu_forward(self, dttry, force=False):
        """One accepted step; returns (h, dtnext, attempts).

        ``force=True`` takes the step with h = dttry whatever its error (replay
        of a prescribed step sequence, used to compare arithmetic precisions on
        identical steps; not a reference feature)."""
        nrjct = 0
        h = dttry
        self.traction_rates()
        while True:
            Tno_y, Tt1o_y, Tt2o_y, state_y, c1, c2, hn1, hn2 = self.rk_attempt(h)
            if force or (max(c1, c2) < 1.0 and not (np.isnan(c1) or np.isnan(c2))):
                dtnext = min(hn1, hn2)
                dtnext = min(1.5 * h, dtnext)
                break
            nrjct += 1
            dtnext = min(hn1, hn2)
            h = max(0.5 * h, dtnext)
            if h < 1.e-15 or nrjct > 20:
                raise StepFailure("dt is too small")
        self.accept(h, Tno_y, Tt1o_y, Tt2o_y, state_y)
        if self.Ifdila:
            self.calc_p_implicit(h)
        return h, dtnext, nrjct + 1

    def accept(self, h, Tno_y, Tt1o_y, Tt2o_y, state_y):
        """State update of an accepted step (src/QDsim_gpu.py:1077-1113)."""
        self.time = self.time + h
        self.Tno, self.Tt1o, self.Tt2o, self.state = Tno_y, Tt1o_y, Tt2o_y, state_y
        self.Tt = np.sqrt(self.Tt1o * self.Tt1o + self.Tt2o * self.Tt2o)
        self.slipv1 = (2.0 * self.V0) * np.exp(-self.state / self.a) * np.sinh(self.Tt1o / self.Tno / self.a)
        self.slipv2 = (2.0 * self.V0) * np.exp(-self.state / self.a) * np.sinh(self.Tt2o / self.Tno / self.a)
        self.slipv = np.sqrt(self.slipv1 * self.slipv1 + self.slipv2 * self.slipv2)
        self.rake = np.arctan2(self.slipv2, self.slipv1)
        self.slipv[self.slipv < 1e-30] = 1e-30
        self.maxslipv0 = np.max(self.slipv)
        self.slip1 = self.slip1 + self.slipv1 * h
        self.slip2 = self.slip2 + self.slipv2 * h
        self.slip = np.sqrt(self.slip1 * self.slip1 + self.slip2 * self.slip2)
        self.fric = self.Tt / (self.Tno - self.P * 1e-6)

    def run(self, nsteps, dt0=1e-3):
        """The reference main loop (src/main_gpu.py:112-118): dttry = dtnext.
        Returns rows (h, time, attempts)."""
        dttry = dt0
        hist = []
        for _ in range(nsteps):
            h, dttry, att = self.simu_forward(dttry)
            hist.append((h, self.time, att))
        return np.array(hist)

    def replay(self, hs):
        """Take the given step sizes, one attempt each, no step control."""
        for h in hs:
            self.simu_forward(float(h), force=True)
