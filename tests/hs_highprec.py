"""40-digit evaluation (mpmath) of the free-surface correction strain of one
triangular dislocation -- test infrastructure: the yardstick for the
ill-conditioned half-space cases.  The harmonic displacement of an angular
dislocation (published formulas, as in src/DH_greenfunction.py:313-400) is
differentiated numerically at 40 digits; the side set-up, configurations and
sum over sides follow src/TDstressFS_C.cpp:1489-1931."""
from __future__ import annotations

import numpy as np


def fsc_strain(P1, P2, P3, Ss, Ds, Ts, x, nu=0.25, dps=40):
    import mpmath as mp
    mp.mp.dps = dps

    def disp(y1, y2, y3, beta, b, a):
        s, c = mp.sin(beta), mp.cos(beta)
        ct = 1 / mp.tan(beta)
        n1, n2 = 1 - 2 * nu, 1 - nu
        K = 1 / (4 * mp.pi * (1 - nu))
        y3b = y3 + 2 * a
        z1b = y1 * c + y3b * s
        z3b = -y1 * s + y3b * c
        rb = mp.sqrt(y1 * y1 + y2 * y2 + y3b * y3b)
        rb2, rb3 = rb * rb, rb * rb * rb
        P, Q, h, W, ar = rb + y3b, rb + z3b, y3b - a, rb * c + y3b, a / rb
        Fib = 2 * mp.atan(-y2 / (-(rb + y3b) / mp.tan(beta / 2) + y1))
        lP, lQ = mp.log(P), mp.log(Q)
        b1, b2, b3 = b
        u1 = b1 * K * (-2 * n2 * n1 * Fib * ct * ct + n1 * y2 / P * ((n1 - ar) * ct - y1 / P * (nu + ar))
                       + n1 * y2 * c * ct / Q * (c + ar) + a * y2 * h * ct / rb3
                       + y2 * h / (rb * P) * (-n1 * ct + y1 / P * (2 * nu + ar) + a * y1 / rb2)
                       + y2 * h / (rb * Q) * (c / Q * (W * (n1 * c - ar) * ct + 2 * n2 * (rb * s - y1) * c)
                                              - a * y3b * c * ct / rb2))
        u2 = b1 * K * (n1 * ((2 * n2 * ct * ct - nu) * lP - (2 * n2 * ct * ct + n1) * c * lQ)
                       - n1 / P * (y1 * ct * (n1 - ar) + nu * y3b - a + y2 * y2 / P * (nu + ar))
                       - n1 * z1b * ct / Q * (c + ar) - a * y1 * h * ct / rb3
                       + h / P * (-2 * nu + (n1 * y1 * ct - a) / rb + y2 * y2 / (rb * P) * (2 * nu + ar)
                                  + a * y2 * y2 / rb3)
                       + h / Q * (c * c - (n1 * z1b * ct + a * c) / rb + a * y3b * z1b * ct / rb3
                                  - (y2 * y2 * c * c - a * z1b * ct / rb * W) / (rb * Q)))
        u3 = b1 * K * (2 * n2 * (n1 * Fib * ct + y2 / P * (2 * nu + ar) - y2 * c / Q * (c + ar))
                       + y2 * h / rb * (2 * nu / P + a / rb2)
                       + y2 * h * c / (rb * Q) * (n1 - W / Q * (c + ar) - a * y3b / rb2))
        u1 += b2 * K * (n1 * ((2 * n2 * ct * ct + nu) * lP - (2 * n2 * ct * ct + 1) * c * lQ)
                        + n1 / P * (-n1 * y1 * ct + nu * y3b - a + a * y1 * ct / rb + y1 * y1 / P * (nu + ar))
                        - n1 * ct / Q * (z1b * c - a * (rb * s - y1) / (rb * c)) - a * y1 * h * ct / rb3
                        + h / P * (2 * nu + (n1 * y1 * ct + a) / rb - y1 * y1 / (rb * P) * (2 * nu + ar)
                                   - a * y1 * y1 / rb3)
                        + h * ct / Q * (-c * s + a * y1 * y3b / (rb3 * c)
                                        + (rb * s - y1) / rb * (2 * n2 * c - W / Q * (1 + a / (rb * c)))))
        u2 += b2 * K * (2 * n2 * n1 * Fib * ct * ct + n1 * y2 / P * (-(n1 - ar) * ct + y1 / P * (nu + ar))
                        - n1 * y2 * ct / Q * (1 + a / (rb * c)) - a * y2 * h * ct / rb3
                        + y2 * h / (rb * P) * (n1 * ct - 2 * nu * y1 / P - a * y1 / rb * (1 / rb + 1 / P))
                        + y2 * h * ct / (rb * Q) * (-2 * n2 * c + W / Q * (1 + a / (rb * c)) + a * y3b / (rb2 * c)))
        u3 += b2 * K * (-2 * n2 * n1 * ct * (lP - c * lQ) - 2 * n2 * y1 / P * (2 * nu + ar)
                        + 2 * n2 * z1b / Q * (c + ar) + h / rb * (n1 * ct - 2 * nu * y1 / P - a * y1 / rb2)
                        - h / Q * (c * s + W * ct / rb * (2 * n2 * c - W / Q)
                                   + a / rb * (s - y3b * z1b / rb2 - z1b * W / (rb * Q))))
        u1 += b3 * K * (n1 * (y2 / P * (1 + ar) - y2 * c / Q * (c + ar)) - y2 * h / rb * (a / rb2 + 1 / P)
                        + y2 * h * c / (rb * Q) * (W / Q * (c + ar) + a * y3b / rb2))
        u2 += b3 * K * (n1 * (-s * lQ - y1 / P * (1 + ar) + z1b / Q * (c + ar)) + y1 * h / rb * (a / rb2 + 1 / P)
                        - h / Q * (s * (c - ar) + z1b / rb * (1 + a * y3b / rb2)
                                   - (y2 * y2 * c * s - a * z1b / rb * W) / (rb * Q)))
        u3 += b3 * K * (2 * n2 * Fib + 2 * n2 * y2 * s / Q * (c + ar)
                        + y2 * h * s / (rb * Q) * (1 + W / Q * (c + ar) + a * y3b / rb2))
        return [u1, u2, u3]

    def strain_local(y, beta, b, a):
        J = [[mp.diff(lambda t, i=i, k=k: disp(*(y[:k] + [t] + y[k + 1:]), beta, b, a)[i], y[k]) for k in range(3)]
             for i in range(3)]
        return [J[0][0], J[1][1], J[2][2], (J[0][1] + J[1][0]) / 2, (J[0][2] + J[2][0]) / 2, (J[1][2] + J[2][1]) / 2]

    def side(PA, PB, B, x):
        sv = [PB[i] - PA[i] for i in range(3)]
        beta = mp.acos(-sv[2] / mp.sqrt(sum(v * v for v in sv)))
        if abs(beta) < 1e-4 or abs(mp.pi - beta) < 1e-4:
            return [mp.mpf(0)] * 6
        hl = mp.sqrt(sv[0] ** 2 + sv[1] ** 2)
        e1 = [sv[0] / hl, sv[1] / hl, 0]
        e2 = [e1[1], -e1[0], 0]
        e3 = [0, 0, -1]
        E = [e1, e2, e3]
        d = [x[i] - PA[i] for i in range(3)]
        yA = [sum(d[j] * E[k][j] for j in range(3)) for k in range(3)]
        yAB = [sum(sv[j] * E[k][j] for j in range(3)) for k in range(3)]
        bv = [sum(B[j] * E[k][j] for j in range(3)) for k in range(3)]
        yB = [yA[k] - yAB[k] for k in range(3)]
        if beta * yA[0] >= 0:
            br = [-bv[0], -bv[1], bv[2]]
            eA = strain_local([-yA[0], -yA[1], yA[2]], mp.pi - beta, br, -PA[2])
            eB = strain_local([-yB[0], -yB[1], yB[2]], mp.pi - beta, br, -PB[2])
            for e_ in (eA, eB):
                e_[4], e_[5] = -e_[4], -e_[5]
        else:
            eA = strain_local(yA, beta, bv, -PA[2])
            eB = strain_local(yB, beta, bv, -PB[2])
        l = [eB[i] - eA[i] for i in range(6)]
        T = mp.matrix([[l[0], l[3], l[4]], [l[3], l[1], l[5]], [l[4], l[5], l[2]]])
        A = mp.matrix([[e1[0], e2[0], e3[0]], [e1[1], e2[1], e3[1]], [e1[2], e2[2], e3[2]]])
        O = A * T * A.T
        return [O[0, 0], O[1, 1], O[2, 2], O[0, 1], O[0, 2], O[1, 2]]

    P1, P2, P3, x = ([mp.mpf(float(v)) for v in p] for p in (P1, P2, P3, x))
    u = [P2[i] - P1[i] for i in range(3)]
    v = [P3[i] - P1[i] for i in range(3)]
    n = [u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2], u[0] * v[1] - u[1] * v[0]]
    nl = mp.sqrt(sum(t * t for t in n))
    n = [t / nl for t in n]
    st = [-n[1], n[0], mp.mpf(0)]
    sl = mp.sqrt(st[0] ** 2 + st[1] ** 2)
    st = [t / sl for t in st]
    dp = [n[1] * st[2] - n[2] * st[1], n[2] * st[0] - n[0] * st[2], n[0] * st[1] - n[1] * st[0]]
    B = [n[i] * Ts + st[i] * Ss + dp[i] * Ds for i in range(3)]
    out = [mp.mpf(0)] * 6
    for a_, b_ in ((P1, P2), (P2, P3), (P3, P1)):
        f = side(a_, b_, B, x)
        out = [out[i] + f[i] for i in range(6)]
    return np.array([float(t) for t in out])
