"""Generate the golden fixtures of tests/golden/.

* k0_exact_nu0.3.json -- the Q1 element stiffness of a unit voxel for E = 1,
  nu = 3/10, integrated EXACTLY with sympy (polynomial integration over
  [0, 1]^3 of eps_i : C : eps_j), independent of the Gauss-quadrature code of
  the oracle and of the library.
* oracle_small.npz -- oracle outputs on a small seeded cantilever (8x4x4,
  2 coarsenings): applyK of a seeded field, one smoothing sweep per level, the
  FP64 MG-PCG solution, its iteration count and compliance, the compliance
  gradient. Regression anchor of the oracle itself.
* cantilever_256x128x128_oracle.json -- the oracle's FULL FP64 MG-PCG solve of
  the 256x128x128 cantilever (5 coarsenings, tol 1e-8): iterations, final
  relative residual and compliance. Regenerate with ``--full`` (about 1.5
  minutes on 8 cores).
* lbl_128_oracle.json -- oracle FP64 MG-PCG solves of the 128^3 layer-by-layer
  workload (rho U[0.1,1] seed 0, base fixed, gravity -y, 5 coarsenings, zero
  guess, tol 1e-8, 2+2 sweeps) at build heights 1, 16, 64 and 128: per height the
  iteration count, the relative residual and f.u (the evaluator's per-height
  compliance). Regenerate with ``--lbl`` (about 2 minutes on 8 cores).

Run from the repository root:  python tests/golden/make_golden.py   (``--full`` and ``--lbl``
only redo the large solves).
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def exact_k0(nu_num=3, nu_den=10):
    import sympy as sp
    x, y, z = sp.symbols("x y z")
    nu = sp.Rational(nu_num, nu_den)
    E = sp.Integer(1)
    lam = E * nu / ((1 + nu) * (1 - 2 * nu))
    mu = E / (2 * (1 + nu))
    X = (x, y, z)
    N = []
    for l in range(8):
        b = [(l >> 2) & 1, (l >> 1) & 1, l & 1]
        f = sp.Integer(1)
        for d in range(3):
            f *= X[d] if b[d] else (1 - X[d])
        N.append(f)
    G = [[sp.diff(N[l], X[d]) for d in range(3)] for l in range(8)]
    K = sp.zeros(24, 24)
    for a in range(8):
        for c in range(3):
            for bb in range(8):
                for d in range(3):
                    dot = sum(G[a][q] * G[bb][q] for q in range(3))
                    ee = sp.Rational(1, 2) * ((dot if c == d else 0) + G[a][d] * G[bb][c])
                    integrand = sp.expand(lam * G[a][c] * G[bb][d] + 2 * mu * ee)
                    K[3 * a + c, 3 * bb + d] = sp.integrate(integrand, (x, 0, 1), (y, 0, 1), (z, 0, 1))
    return [[float(K[i, j]) for j in range(24)] for i in range(24)]


def oracle_small():
    from oracle import pyoracle as po
    from voxelfem_gb300 import workloads as wl
    ne = (8, 4, 4)
    s = po.Sim(ne)
    wl.setup_cantilever(s, ne, 0.3, 0)
    mg = po.MG(s, 2)
    nn = s.nn
    u = np.random.default_rng(7).standard_normal((nn, 3))
    b = s.buildLoadVector()
    mg.updateStiffnessMatrices()
    out = {"u": u, "b": b, "Ku": s.applyK(u)}
    for l in range(mg.numLevels - 1):
        nl = mg.levelNodes(l)
        ul = np.random.default_rng(10 + l).standard_normal((nl, 3))
        bl = np.random.default_rng(20 + l).standard_normal((nl, 3))
        out["smooth_u%d" % l] = ul
        out["smooth_b%d" % l] = bl
        out["smooth_out%d" % l] = mg.smooth(l, ul, bl, True)
    x = mg.preconditionedConjugateGradient(np.zeros_like(b), b, 100, 1e-10, None, 1, 2, False)
    out["x"] = x
    out["iterations"] = np.array(mg.lastIterations)
    out["compliance"] = np.array(0.5 * np.sum(b * x))
    out["grad"] = s.complianceGradient(x)
    return out


def oracle_full():
    import time
    from oracle import pyoracle as po
    from voxelfem_gb300 import workloads as wl
    ne = (256, 128, 128)
    s = po.Sim(ne)
    wl.setup_cantilever(s, ne, 0.01, 0)
    mg = po.MG(s, 5)
    b = s.buildLoadVector()
    t0 = time.time()
    x = mg.preconditionedConjugateGradient(np.zeros_like(b), b, 200, 1e-8, None, 1, 2, False)
    return {"workload": "cantilever 256x128x128 Q1, rho U[0.01,1] seed 0, E0=1, Emin=1e-9, nu=0.3, p=3, "
                        "5 coarsenings, mgIterations=1, mgSmoothingIterations=2, V-cycle, tol 1e-8, x0=0",
            "iterations": int(mg.lastIterations), "relres": float(mg.lastRelativeResidual),
            "compliance": float(0.5 * np.sum(b * x)), "threads": po.num_threads(),
            "seconds": time.time() - t0}


LBL_HEIGHTS = (1, 16, 64, 128)


def oracle_lbl():
    import time
    from oracle import pyoracle as po
    from voxelfem_gb300 import workloads as wl
    ne = (128, 128, 128)
    out = {"workload": "layer-by-layer 128^3 Q1, rho U[0.1,1] seed 0, E0=1, Emin=1e-9, nu=0.3, p=3, base y=0 "
                       "fixed, gravity (0,-1,0), 5 coarsenings, mgIterations=1, mgSmoothingIterations=2, "
                       "V-cycle, tol 1e-8, x0=0",
           "heights": [], "threads": po.num_threads()}
    for h in LBL_HEIGHTS:
        s = po.Sim(ne)
        wl.setup_layer_by_layer(s, ne, 0.1, 0)
        s.setFabricationMaskHeightByLayer(h)
        mg = po.MG(s, 5)
        mg.setFabricationMaskHeightByLayer(h)
        b = s.buildLoadVector()
        t0 = time.time()
        x = mg.preconditionedConjugateGradient(np.zeros_like(b), b, 500, 1e-8, None, 1, 2, False)
        out["heights"].append({"height": h, "iterations": int(mg.lastIterations),
                               "relres": float(mg.lastRelativeResidual), "f_dot_u": float(np.sum(b * x)),
                               "seconds": time.time() - t0})
    return out


def main():
    if "--lbl" in sys.argv:
        with open(os.path.join(HERE, "lbl_128_oracle.json"), "w") as f:
            json.dump(oracle_lbl(), f, indent=1)
        return
    if "--full" in sys.argv:
        full = oracle_full()
        with open(os.path.join(HERE, "cantilever_256x128x128_oracle.json"), "w") as f:
            json.dump(full, f, indent=1)
        return
    k0 = exact_k0()
    with open(os.path.join(HERE, "k0_exact_nu0.3.json"), "w") as f:
        json.dump({"E": 1.0, "nu": 0.3, "h": [1.0, 1.0, 1.0], "K0": k0}, f)
    small = oracle_small()
    np.savez_compressed(os.path.join(HERE, "oracle_small.npz"), **small)


if __name__ == "__main__":
    main()
