"""pyOptimizer (python_bindings/Optimizer.cc:11-23): the Method of Moving Asymptotes with its
vector work on the GPU.

``MMA(numVars, numConstr, xmin, xmax, f, df_dx)``: ``f(x)`` returns the objective followed by the
``numConstr`` constraint values (constraints are ``<= 0``), ``df_dx(x)`` their gradients as a
``(numConstr + 1, numVars)`` array; both receive ``x`` as a numpy array. ``setInitialVar(x0)``,
``step()`` and ``enableGCMMA(enable)`` as in the reference; ``getOptimalVar()`` returns the
current iterate.
"""
import ctypes as C

import numpy as np

from . import _capi
from ._capi import check

_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.POINTER(C.c_double), C.c_int64, C.POINTER(C.c_double))


class MMA:
    def __init__(self, numVars, numConstr, xmin, xmax, f, df_dx):
        self.n, self.m = int(numVars), int(numConstr)
        lo = np.ascontiguousarray(np.asarray(xmin, dtype=np.float64).reshape(-1))
        hi = np.ascontiguousarray(np.asarray(xmax, dtype=np.float64).reshape(-1))
        if lo.size != self.n or hi.size != self.n:
            raise RuntimeError("Invalid input size")
        self._f, self._df = f, df_dx
        self._err = None

        def f_cb(user, x, n, out):
            try:
                xv = np.ctypeslib.as_array(x, shape=(n,)).copy()
                v = np.asarray(self._f(xv), dtype=np.float64).reshape(-1)
                if v.size != self.m + 1:
                    raise RuntimeError("f must return numConstr + 1 values")
                np.ctypeslib.as_array(out, shape=(self.m + 1,))[:] = v
                return 0
            except Exception as e:  # reported after the call returns
                self._err = e
                return 1

        def df_cb(user, x, n, out):
            try:
                xv = np.ctypeslib.as_array(x, shape=(n,)).copy()
                g = np.asarray(self._df(xv), dtype=np.float64)
                if g.size != (self.m + 1) * n:
                    raise RuntimeError("df_dx must return a (numConstr + 1, numVars) array")
                np.ctypeslib.as_array(out, shape=(self.m + 1, n))[:] = g.reshape(self.m + 1, n)
                return 0
            except Exception as e:
                self._err = e
                return 1

        self._fcb, self._dfcb = _FN(f_cb), _FN(df_cb)
        h = C.c_void_p()
        check(_capi.load().vfem_mma_create(self.n, self.m, lo.ctypes.data_as(C.c_void_p),
                                           hi.ctypes.data_as(C.c_void_p), self._fcb, self._dfcb, None, C.byref(h)))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _capi._lib is not None:
            _capi._lib.vfem_mma_destroy(h)
            self._h = None

    def _call(self, fn, *args):
        self._err = None
        rc = fn(self._h, *args)
        if self._err is not None:
            e, self._err = self._err, None
            raise e
        check(rc)

    def setInitialVar(self, x0):
        x = np.ascontiguousarray(np.asarray(x0, dtype=np.float64).reshape(-1))
        if x.size != self.n:
            raise RuntimeError("Invalid input size")
        self._call(_capi.load().vfem_mma_set_initial_var, x.ctypes.data_as(C.c_void_p))

    def enableGCMMA(self, enable):
        self._call(_capi.load().vfem_mma_enable_gcmma, int(bool(enable)))

    def step(self):
        self._call(_capi.load().vfem_mma_step)

    def getOptimalVar(self):
        out = np.empty(self.n)
        self._call(_capi.load().vfem_mma_get_optimal_var, out.ctypes.data_as(C.c_void_p))
        return out
