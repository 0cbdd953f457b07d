"""Restatement of the reference's Method of Moving Asymptotes (MethodOfMovingAsymptotes.hh) in
numpy, the oracle of the GPU optimiser (test infrastructure only; imported by tests/).

Problem (MethodOfMovingAsymptotes.hh:21-27):
    min f_0(x) + a0 z + sum_i (c_i y_i + d_i y_i^2 / 2)
    s.t. f_i(x) - a_i z - y_i <= 0, xmin <= x <= xmax, y >= 0, z >= 0
with a = 0, c = 1000, d = 1, a0 = 1. Each step builds the convex MMA approximation around the
current iterate (asymptotes :73-95, bounds :96-99, p and q :127-134) and solves it with the
primal-dual interior-point method of the Subproblem (:240-465); GCMMA adds the inner loop of
conservative approximations (:107-123, :137-156, :184-187).
"""
import numpy as np

RAA0, ALBEFA, MOVE, ASYINIT = 1e-5, 0.1, 0.5, 0.5
GAMMA = (0.7, 1.2, 1.0)


class MMA:
    def __init__(self, numVars, numConstr, xmin, xmax, f, df_dx, max_inner=1000):
        self.n, self.m = int(numVars), int(numConstr)
        self.xmin = np.asarray(xmin, dtype=np.float64).copy()
        self.xmax = np.asarray(xmax, dtype=np.float64).copy()
        self.xdiff = self.xmax - self.xmin
        self.f, self.df_dx = f, df_dx
        self.a = np.zeros(self.m)
        self.c = np.full(self.m, 1000.0)
        self.d = np.ones(self.m)
        self.a0 = 1.0
        self.outer_iter = 0
        self.inner_iter = 0
        self.hist = []
        self.enableInner = False
        self.max_inner = max_inner
        self.l = np.zeros(self.n)
        self.u = np.zeros(self.n)

    def enableGCMMA(self, enable):
        self.enableInner = bool(enable)

    def setInitialVar(self, x0):
        self._push(np.asarray(x0, dtype=np.float64).copy())

    def _push(self, x):
        self.hist.insert(0, x)
        del self.hist[3:]

    def getOptimalVar(self):
        return self.hist[0].copy()

    # g_i(x) = sum_j p_ij / (u_j - x_j) + q_ij / (x_j - l_j)   (:159-183)
    def _g(self, ux, xl, rows):
        return np.array([np.sum(self.p[i] / ux + self.q[i] / xl) for i in rows])

    def step(self):
        if not self.hist:
            raise RuntimeError("Must specify an initial value")
        self.outer_iter += 1
        x = self.hist[0]
        if self.outer_iter <= 2:
            self.l = x - ASYINIT * self.xdiff
            self.u = x + ASYINIT * self.xdiff
        else:
            x1, x2 = self.hist[1], self.hist[2]
            zzz = (x - x1) * (x1 - x2)
            gam = np.where(zzz > 0, GAMMA[1], GAMMA[0])
            self.l = np.maximum(np.minimum(x - gam * (x1 - self.l), x - 0.01 * self.xdiff), x - 10 * self.xdiff)
            self.u = np.minimum(np.maximum(x + gam * (self.u - x1), x + 0.01 * self.xdiff), x + 10 * self.xdiff)
        self.alpha = np.maximum(np.maximum(self.xmin, self.l + ALBEFA * (x - self.l)), x - MOVE * self.xdiff)
        self.beta = np.minimum(np.minimum(self.xmax, self.u - ALBEFA * (self.u - x)), x + MOVE * self.xdiff)
        self.f_cur = np.asarray(self.f(x), dtype=np.float64).reshape(self.m + 1)
        df = np.asarray(self.df_dx(x), dtype=np.float64).reshape(self.m + 1, self.n)
        self.dfp, self.dfm = np.maximum(df, 0.0), np.maximum(-df, 0.0)
        ux, xl = self.u - x, x - self.l
        if self.enableInner:
            self.inner_iter = 0
            while True:
                self.rho = self._next_rho(x)
                self._pq(ux, xl, self.rho[:, None] / self.xdiff[None, :])
                self.r = self.f_cur - self._g(ux, xl, range(self.m + 1))
                xin = self._subsolve()
                self.x_inner = xin
                self.inner_iter += 1
                uxi, xli = self.u - xin, xin - self.l
                self.diff_f_subf = np.asarray(self.f(xin), dtype=np.float64).reshape(self.m + 1) - \
                    (self._g(uxi, xli, range(self.m + 1)) + self.r)
                if self.diff_f_subf.max() < 0 or self.inner_iter >= self.max_inner:
                    break
            self._push(xin)
            self.inner_iter = 0
        else:
            self._pq(ux, xl, np.broadcast_to(RAA0 / self.xdiff, (self.m + 1, self.n)))
            self.r = self.f_cur - self._g(ux, xl, range(self.m + 1))
            self._push(self._subsolve())

    def _pq(self, ux, xl, rho_over):
        self.p = (ux ** 2)[None, :] * (1.001 * self.dfp + 0.001 * self.dfm + rho_over)
        self.q = (xl ** 2)[None, :] * (0.001 * self.dfp + 1.001 * self.dfm + rho_over)

    def _next_rho(self, x):
        if self.inner_iter == 0:
            return np.maximum(0.1 / self.n * ((self.dfp + self.dfm) @ self.xdiff), 1e-6)
        xin = self.x_inner
        uxi, xli = self.u - xin, xin - self.l
        dd = np.sum((self.u - self.l) * (xin - x) ** 2 / (uxi * xli * self.xdiff))
        out = self.rho.copy()
        for i in range(self.m + 1):
            delta = self.diff_f_subf[i] / dd
            if not delta < 0:
                out[i] = min(1.1 * (self.rho[i] + delta), 10 * self.rho[i])
        return out

    # ---- primal-dual interior point (Subproblem, :240-465) ----
    def _subsolve(self):
        m, n = self.m, self.n
        al, be, u, l = self.alpha, self.beta, self.u, self.l
        P0, Pm, Q0, Qm = self.p[0], self.p[1:], self.q[0], self.q[1:]
        S = {}
        S["x"] = 0.5 * (al + be)
        S["xi"] = np.maximum(1.0 / (S["x"] - al), 1.0)
        S["eta"] = np.maximum(1.0 / (be - S["x"]), 1.0)
        S["y"], S["z"], S["zeta"] = np.ones(m), 1.0, 1.0
        S["lam"], S["s"] = np.ones(m), np.ones(m)
        S["mu"] = np.maximum(self.c / 2, 1.0)
        a, c, d, a0, r = self.a, self.c, self.d, self.a0, self.r[1:]

        def derived():
            x, lam = S["x"], S["lam"]
            ux, xl = u - x, x - l
            plam = P0 + Pm.T @ lam
            qlam = Q0 + Qm.T @ lam
            dpsi = plam / ux ** 2 - qlam / xl ** 2
            g = np.array([np.sum(Pm[i] / ux + Qm[i] / xl) for i in range(m)])
            return ux, xl, plam, qlam, dpsi, g

        def eqs(eps, dpsi, g):
            x, xi, eta = S["x"], S["xi"], S["eta"]
            return [dpsi - xi + eta, xi * (x - al) - eps, eta * (be - x) - eps,
                    c + d * S["y"] - S["lam"] - S["mu"], np.array([a0 - S["zeta"] - S["lam"] @ a]),
                    g - a * S["z"] - S["y"] + S["s"] + r, S["mu"] * S["y"] - eps,
                    np.array([S["zeta"] * S["z"] - eps]), S["lam"] * S["s"] - eps]

        def sqres(eps, dpsi, g):
            return sum(float(np.sum(e ** 2)) for e in eqs(eps, dpsi, g))

        def kkt_inf(eps, dpsi, g):
            return max(float(np.max(np.abs(e))) for e in eqs(eps, dpsi, g))

        def move(step, D):
            for k in ("x", "xi", "eta", "y", "lam", "mu", "s"):
                S[k] = S[k] + step * D[k]
            S["z"] += step * D["z"]
            S["zeta"] += step * D["zeta"]

        ux, xl, plam, qlam, dpsi, g = derived()
        eps = 1.0
        while eps > 1e-7:
            res_old = None
            for it in range(10):
                x, xi, eta, y, lam, mu, s, z, zeta = (S[k] for k in ("x", "xi", "eta", "y", "lam", "mu", "s", "z",
                                                                    "zeta"))
                dx = dpsi - eps / (x - al) + eps / (be - x)
                Dx = 2 * plam / (ux * ux ** 2) + 2 * qlam / (xl * xl ** 2) + xi / (x - al) + eta / (be - x)
                G = Pm / ux[None, :] ** 2 - Qm / xl[None, :] ** 2
                Dy = d + mu / y
                dy = c + d * y - lam - eps / y
                M = np.zeros((m + 1, m + 1))
                M[:m, :m] = (G / Dx[None, :]) @ G.T
                M[:m, :m] += np.diag(s / lam + 1.0 / Dy)
                M[:m, m] = a
                M[m, :m] = a
                M[m, m] = -zeta / z
                rhs = np.zeros(m + 1)
                rhs[:m] = g - a * z - y + r + eps / lam + dy / Dy - G @ (dx / Dx)
                rhs[m] = a0 - lam @ a - eps / z
                sol = np.linalg.solve(M, rhs)
                D = {"lam": sol[:m], "z": sol[m]}
                D["x"] = -(dx + G.T @ D["lam"]) / Dx
                D["xi"] = -xi + eps / (x - al) - xi * D["x"] / (x - al)
                D["eta"] = -eta + eps / (be - x) + eta * D["x"] / (be - x)
                D["y"] = D["lam"] / Dy - dy / Dy
                D["mu"] = (eps - mu * D["y"]) / y - mu
                D["zeta"] = (eps - zeta * D["z"]) / z - zeta
                D["s"] = (eps - s * D["lam"]) / lam - s
                if it == 0:
                    res_old = sqres(eps, dpsi, g)
                # step keeping the KKT positivity constraints (:378-390)
                mc = min(np.min(D["x"] / (x - al)), np.min(D["x"] / (x - be)), np.min(D["xi"] / xi),
                         np.min(D["eta"] / eta), np.min(D["y"] / y), D["z"] / z, np.min(D["s"] / s),
                         np.min(D["mu"] / mu), D["zeta"] / zeta, np.min(D["lam"] / lam))
                step = 1.0 / max(-1.01 * mc, 1.0)
                move(step, D)
                ux, xl, plam, qlam, dpsi, g = derived()
                res = sqres(eps, dpsi, g)
                while res > res_old:
                    step /= 2
                    move(-step, D)
                    ux, xl, plam, qlam, dpsi, g = derived()
                    res = sqres(eps, dpsi, g)
                res_old = res
                if kkt_inf(eps, dpsi, g) <= 0.9 * eps:
                    break
            eps *= 0.1
        return S["x"].copy()
