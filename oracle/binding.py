"""ctypes binding of the CPU oracle (oracle/flof_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU legs of bench.py, never by the product package.

Grids are numpy arrays in the reference layout (source/grid4d.h:92-97):
a Real grid of size (X, Y, Z, T) is an array of shape (T, Z, Y, X); a Vec4
grid has shape (T, Z, Y, X, 4).  Both are C-contiguous, so x is fastest.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")


def build() -> None:
    """Compile liborc32.so / liborc64.so with the Makefile beside this file."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def dims_of(a: np.ndarray) -> tuple[int, int, int, int]:
    """(X, Y, Z, T) of a Real (T,Z,Y,X) or Vec4 (T,Z,Y,X,4) grid."""
    if a.ndim == 5:
        t, z, y, x, _ = a.shape
    else:
        t, z, y, x = a.shape
    return (x, y, z, t)


def ncomp(a: np.ndarray) -> int:
    return 4 if a.ndim == 5 else 1


class Oracle:
    """One precision of the oracle: float32 (reference "fp1") or float64
    (reference "fp2", -DDOUBLEPRECISION)."""

    def __init__(self, double: bool = False):
        self.double = double
        self.dtype = np.float64 if double else np.float32
        name = "liborc64.so" if double else "liborc32.so"
        path = os.path.join(_BUILD, name)
        if not os.path.exists(path):
            build()
        self.lib = ctypes.CDLL(path)
        self.prefix = "orc64_" if double else "orc32_"
        self.R = ctypes.c_double if double else ctypes.c_float
        self._setup()

    # -- plumbing ---------------------------------------------------------
    def _f(self, name):
        return getattr(self.lib, self.prefix + name)

    def _setup(self):
        R = self.R
        P = ctypes.c_void_p
        I = ctypes.c_int
        sig = {
            "interp4": (R, [P, P, I, I, P]),
            "setConst": (None, [P, P, I, P]),
            "addConst": (None, [P, P, I, P]),
            "multConst": (None, [P, P, I, P]),
            "add": (None, [P, P, I, P]),
            "sub": (None, [P, P, I, P]),
            "addScaled": (None, [P, P, I, P, P]),
            "reduce": (R, [P, P, I, I]),
            "setBound": (None, [P, P, I, P, I]),
            "setBoundNeumann": (None, [P, P, I, I]),
            "resample4d": (None, [P, P, P, P, I, P, P]),
            "gridFactor4d": (None, [P, P, P, P, P, P]),
            "interpolateGrid4d": (None, [P, P, P, P, I, P, P, P]),
            "interpolGrid": (None, [P, P, P, P, I]),
            "advect4d": (None, [P, P, P, I, R]),
            "advectCfl4d": (None, [P, R, P, P, I]),
            "calcLsDiff4d": (R, [P, P, P, P, R, I]),
            "gaussianBlur4d": (None, [P, P, I, R, I]),
            "ofAssemble": (None, [P, P, P, P, R, R, P, P, P]),
            "opticalFlow4d": (None, [P, P, P, P, R, R, R, R, R, I, P, P]),
            "cgSolve": (I, [P, P, P, P, R, R, R, I, P, P, P]),
            "expolSweeps": (None, [P, P, P, I]),
            "projectCells": (None, [P, P, P, P, P, P, R, I]),
            "corrVelsOf4d": (None, [P, P, P, P, P, R, R, R, I, P]),
            "opticalFlowMultiscale4d": (R, [P, P, P, P, P, P]),
            "deform4d": (None, [P, P, P, P, P, P, R, R, I]),
            "optRunFrame": (None, [P, P, P, P, P, P, R, R, R, P, P, P, P, R, I, R]),
            "statsReset": (None, []),
            "statsGet": (I, [P, P, P, I]),
            "repeatFrame4d": (None, [P, P, R, R, I]),
            "extrap4dLsSimple": (None, [P, P, I, I]),
            "join": (None, [ctypes.c_longlong, P, P]),
            "setBound3": (None, [P, P, I, P, I]),
            "setBoundNeumann3": (None, [P, P, I, I]),
            "simpleBlurSpecial": (None, [P, P, I, R, I]),
            "loadPlaceGrid4d": (None, [P, P, P, P, I, P, P, I, I, I, R, P, R, I, R, I, R, R]),
            "loadAdvectTimeSlice": (None, [P, P, P, P, P, P, R, R, R, P, P, P, P, R, I, R]),
        }
        for name, (res, args) in sig.items():
            fn = self._f(name)
            fn.restype = res
            fn.argtypes = args

    def _arr(self, a) -> np.ndarray:
        a = np.ascontiguousarray(a, dtype=self.dtype)
        return a

    @staticmethod
    def _p(a: np.ndarray):
        return a.ctypes.data_as(ctypes.c_void_p)

    def _vec(self, v, n=4):
        v = np.asarray(v, dtype=self.dtype).reshape(-1)
        if v.size == 1:
            v = np.full(n, v[0], dtype=self.dtype)
        return np.ascontiguousarray(v)

    @staticmethod
    def _dims(d) -> np.ndarray:
        return np.ascontiguousarray(np.asarray(d, dtype=np.int32))

    # -- interpolation ------------------------------------------------------
    def interp4(self, grid, pos, comp=0):
        g = self._arr(grid)
        d = self._dims(dims_of(g))
        p = self._vec(pos)
        return self._f("interp4")(self._p(d), self._p(g), ncomp(g), comp, self._p(p))

    # -- Grid4d ops (in place on a copy, returned) --------------------------
    def setConst(self, a, v):
        a = self._arr(a).copy()
        self._f("setConst")(self._p(self._dims(dims_of(a))), self._p(a), ncomp(a), self._p(self._vec(v, ncomp(a))))
        return a

    def addConst(self, a, v):
        a = self._arr(a).copy()
        self._f("addConst")(self._p(self._dims(dims_of(a))), self._p(a), ncomp(a), self._p(self._vec(v, ncomp(a))))
        return a

    def multConst(self, a, v):
        a = self._arr(a).copy()
        self._f("multConst")(self._p(self._dims(dims_of(a))), self._p(a), ncomp(a), self._p(self._vec(v, ncomp(a))))
        return a

    def add(self, a, b):
        a = self._arr(a).copy()
        b = self._arr(b)
        self._f("add")(self._p(self._dims(dims_of(a))), self._p(a), ncomp(a), self._p(b))
        return a

    def sub(self, a, b):
        a = self._arr(a).copy()
        b = self._arr(b)
        self._f("sub")(self._p(self._dims(dims_of(a))), self._p(a), ncomp(a), self._p(b))
        return a

    def addScaled(self, a, b, factor):
        a = self._arr(a).copy()
        b = self._arr(b)
        self._f("addScaled")(self._p(self._dims(dims_of(a))), self._p(a), ncomp(a), self._p(b),
                             self._p(self._vec(factor, ncomp(a))))
        return a

    def getMax(self, a):
        a = self._arr(a)
        return self._f("reduce")(self._p(self._dims(dims_of(a))), self._p(a), ncomp(a), 0)

    def getMin(self, a):
        a = self._arr(a)
        return self._f("reduce")(self._p(self._dims(dims_of(a))), self._p(a), ncomp(a), 1)

    def getMaxAbs(self, a):
        a = self._arr(a)
        return self._f("reduce")(self._p(self._dims(dims_of(a))), self._p(a), ncomp(a), 2)

    def setBound(self, a, value, w):
        a = self._arr(a).copy()
        self._f("setBound")(self._p(self._dims(dims_of(a))), self._p(a), ncomp(a),
                            self._p(self._vec(value, ncomp(a))), int(w))
        return a

    def setBoundNeumann(self, a, w):
        a = self._arr(a).copy()
        self._f("setBoundNeumann")(self._p(self._dims(dims_of(a))), self._p(a), ncomp(a), int(w))
        return a

    # -- input conditioning ---------------------------------------------------
    def repeatFrame4d(self, phi, srct, range_=0.0, bnd=0):
        a = self._arr(phi).copy()
        self._f("repeatFrame4d")(self._p(self._dims(dims_of(a))), self._p(a), float(srct),
                                 float(range_), int(bnd))
        return a

    def extrap4dLsSimple(self, phi, distance=4, inside=False):
        a = self._arr(phi).copy()
        self._f("extrap4dLsSimple")(self._p(self._dims(dims_of(a))), self._p(a), int(distance),
                                    1 if inside else 0)
        return a

    # -- 3D grids (arrays of shape (Z, Y, X[, 4])) -------------------------------
    @staticmethod
    def _dims3(a):
        z, y, x = a.shape[:3]
        return np.ascontiguousarray(np.asarray((x, y, z), dtype=np.int32))

    def join(self, a, b):
        a = self._arr(a).copy()
        b = self._arr(b)
        assert a.shape == b.shape
        self._f("join")(a.size, self._p(a), self._p(b))
        return a

    def setBound3(self, a, value, w):
        a = self._arr(a).copy()
        nc = 4 if a.ndim == 4 else 1
        self._f("setBound3")(self._p(self._dims3(a)), self._p(a), nc, self._p(self._vec(value, nc)),
                             int(w))
        return a

    def setBoundNeumann3(self, a, w):
        a = self._arr(a).copy()
        nc = 4 if a.ndim == 4 else 1
        self._f("setBoundNeumann3")(self._p(self._dims3(a)), self._p(a), nc, int(w))
        return a

    def loadPlaceGrid4d(self, dims, slices, offset, scale, fileIdxStart=-1, fileIdxEnd=-1,
                        debugSkipLoad=999999, spread=1.0, overrideSize=-1.0, overrideTimeOff=0.0,
                        overrideGoodRegion=0, loadTimeScale=1.0, rescaleSdfValues=False,
                        sdfIsoOff=0.0, repeatStartFrame=0.0, phi=None):
        """slices: array (nfiles, Z, Y, X), element q = file index fileIdxStart + q.
        phi (optional) is the grid's previous content, kept where the
        partial-load region says so."""
        X, Y, Z, T = dims
        out = np.zeros((T, Z, Y, X), self.dtype) if phi is None else self._arr(phi).copy()
        sl = self._arr(slices)
        nf, sz, sy, sx = sl.shape
        self._f("loadPlaceGrid4d")(
            self._p(self._dims(dims)), self._p(out), self._p(self._dims((sx, sy, sz))), self._p(sl), nf,
            self._p(self._vec(offset)), self._p(self._vec(scale)), int(fileIdxStart), int(fileIdxEnd),
            int(debugSkipLoad), float(spread), self._p(self._vec(overrideSize)), float(overrideTimeOff),
            int(overrideGoodRegion), float(loadTimeScale), 1 if rescaleSdfValues else 0, float(sdfIsoOff),
            float(repeatStartFrame))
        return out

    def loadAdvectTimeSlice(self, defo, dst, phi, time, blendAlpha, loadTimeScale, defoOffset, defoScale,
                            defoFactor, overrideSize=-1.0, overrideTimeOff=0.0, zeroVel=False,
                            defoAniFac=1.0):
        """dst: (Z, Y, X) array, returned updated inside its bnd = 1 box."""
        d = self._arr(defo)
        out = self._arr(dst).copy()
        p = self._arr(phi)
        z, y, x = out.shape
        self._f("loadAdvectTimeSlice")(
            self._p(self._dims(dims_of(d))), self._p(d), self._p(self._dims((x, y, z))), self._p(out),
            self._p(self._dims(dims_of(p))), self._p(p), float(time), float(blendAlpha),
            float(loadTimeScale), self._p(self._vec(defoOffset)), self._p(self._vec(defoScale)),
            self._p(self._vec(defoFactor)), self._p(self._vec(overrideSize)), float(overrideTimeOff),
            1 if zeroVel else 0, float(defoAniFac))
        return out

    def simpleBlurSpecial(self, a, iter_=1, thresh=0.0, bord=0):
        a = self._arr(a).copy()
        self._f("simpleBlurSpecial")(self._p(self._dims3(a)), self._p(a), int(iter_),
                                     float(thresh), int(bord))
        return a

    # -- resampling ----------------------------------------------------------
    def resample4d(self, target_dims, source, fac, off):
        s = self._arr(source)
        nc = ncomp(s)
        X, Y, Z, T = target_dims
        shape = (T, Z, Y, X, 4) if nc == 4 else (T, Z, Y, X)
        t = np.zeros(shape, dtype=self.dtype)
        self._f("resample4d")(self._p(self._dims(target_dims)), self._p(t), self._p(self._dims(dims_of(s))),
                              self._p(s), nc, self._p(self._vec(fac)), self._p(self._vec(off)))
        return t

    def gridFactor4d(self, s1, s2, optSize, scale, off):
        fac = np.zeros(4, dtype=self.dtype)
        o = self._vec(off).copy()
        self._f("gridFactor4d")(self._p(self._vec(s1)), self._p(self._vec(s2)), self._p(self._vec(optSize)),
                                self._p(self._vec(scale)), self._p(fac), self._p(o))
        return fac, o

    def interpolateGrid4d(self, target_dims, source, offset=(0, 0, 0, 0), scale=(1, 1, 1, 1), size=(-1, -1, -1, -1)):
        s = self._arr(source)
        nc = ncomp(s)
        X, Y, Z, T = target_dims
        shape = (T, Z, Y, X, 4) if nc == 4 else (T, Z, Y, X)
        t = np.zeros(shape, dtype=self.dtype)
        self._f("interpolateGrid4d")(self._p(self._dims(target_dims)), self._p(t), self._p(self._dims(dims_of(s))),
                                     self._p(s), nc, self._p(self._vec(offset)), self._p(self._vec(scale)),
                                     self._p(self._vec(size)))
        return t

    def interpolGrid(self, target_dims, source):
        s = self._arr(source)
        nc = ncomp(s)
        X, Y, Z, T = target_dims
        shape = (T, Z, Y, X, 4) if nc == 4 else (T, Z, Y, X)
        t = np.zeros(shape, dtype=self.dtype)
        self._f("interpolGrid")(self._p(self._dims(target_dims)), self._p(t), self._p(self._dims(dims_of(s))),
                                self._p(s), nc)
        return t

    # -- advection -----------------------------------------------------------
    def advect4d(self, vel, grid, dtFac=1.0):
        v = self._arr(vel)
        g = self._arr(grid).copy()
        self._f("advect4d")(self._p(self._dims(dims_of(g))), self._p(v), self._p(g), ncomp(g), dtFac)
        return g

    def advectCfl4d(self, vel, grid, cfl=999.0):
        v = self._arr(vel)
        g = self._arr(grid).copy()
        self._f("advectCfl4d")(self._p(self._dims(dims_of(g))), cfl, self._p(v), self._p(g), ncomp(g))
        return g

    def calcLsDiff4d(self, i0, i1, correction=1.0, bnd=0, want_out=False):
        a = self._arr(i0)
        b = self._arr(i1)
        out = np.zeros_like(a) if want_out else None
        r = self._f("calcLsDiff4d")(self._p(self._dims(dims_of(a))), self._p(a), self._p(b),
                                    self._p(out) if want_out else None, correction, int(bnd))
        return (r, out) if want_out else r

    def gaussianBlur4d(self, a, sigma, iter=1):
        a = self._arr(a).copy()
        self._f("gaussianBlur4d")(self._p(self._dims(dims_of(a))), self._p(a), ncomp(a), sigma, int(iter))
        return a

    # -- optical flow --------------------------------------------------------
    def ofAssemble(self, vel, i0, i1, wSmooth=0.001, wEnergy=0.0001):
        a = self._arr(i0)
        b = self._arr(i1)
        v = self._arr(vel)
        n = int(np.prod(a.shape))
        rhs = np.zeros(n * 4, dtype=self.dtype)
        blockd = np.zeros(n * 16, dtype=self.dtype)
        offd = np.zeros(n * 4, dtype=self.dtype)
        self._f("ofAssemble")(self._p(self._dims(dims_of(a))), self._p(v), self._p(a), self._p(b), wSmooth, wEnergy,
                              self._p(rhs), self._p(blockd), self._p(offd))
        return rhs, blockd, offd

    def opticalFlow4d(self, vel, i0, i1, wSmooth=0.0, wEnergy=0.0, postVelBlur=0.0, cgAccuracy=1e-4,
                      resetBndWidth=-1.0, cgMaxIter=1000):
        v = self._arr(vel).copy()
        a = self._arr(i0)
        b = self._arr(i1)
        it = ctypes.c_int(0)
        res = self.R(0)
        self._f("opticalFlow4d")(self._p(self._dims(dims_of(a))), self._p(v), self._p(a), self._p(b), wSmooth,
                                 wEnergy, postVelBlur, cgAccuracy, resetBndWidth, int(cgMaxIter),
                                 ctypes.byref(it), ctypes.byref(res))
        return v, it.value, res.value

    def cgSolve(self, vel, i0, i1, wSmooth, wEnergy, accuracy, maxIter=1000):
        a = self._arr(i0)
        b = self._arr(i1)
        v = self._arr(vel)
        x = np.zeros(int(np.prod(a.shape)) * 4, dtype=self.dtype)
        it = ctypes.c_int(0)
        res = self.R(0)
        ok = self._f("cgSolve")(self._p(self._dims(dims_of(a))), self._p(v), self._p(a), self._p(b), wSmooth,
                                wEnergy, accuracy, int(maxIter), self._p(x), ctypes.byref(it), ctypes.byref(res))
        return x, it.value, res.value, bool(ok)

    def expolSweeps(self, dst, mark, sweeps):
        d = self._arr(dst).copy()
        m = self._arr(mark)
        self._f("expolSweeps")(self._p(self._dims(dims_of(d))), self._p(d), self._p(m), int(sweeps))
        return d

    def projectCells(self, vel, phiOrg, phiTarget, threshPhi=4.0, maxIter=40):
        v = self._arr(vel)
        a = self._arr(phiOrg)
        b = self._arr(phiTarget)
        dst = np.zeros_like(v)
        mark = np.zeros_like(a)
        self._f("projectCells")(self._p(self._dims(dims_of(a))), self._p(dst), self._p(v), self._p(a), self._p(b),
                                self._p(mark), threshPhi, int(maxIter))
        return dst, mark

    def corrVelsOf4d(self, vel, phiOrg, phiTarget, threshPhi=4.0, postVelBlur=4.0, resetBndWidth=0.1,
                     maxIter=40):
        v = self._arr(vel).copy()
        a = self._arr(phiOrg)
        b = self._arr(phiTarget)
        dst = np.zeros_like(v)
        e = ctypes.c_int(0)
        self._f("corrVelsOf4d")(self._p(self._dims(dims_of(a))), self._p(dst), self._p(v), self._p(a), self._p(b),
                                threshPhi, postVelBlur, resetBndWidth, int(maxIter), ctypes.byref(e))
        return v, dst, e.value

    def opticalFlowMultiscale4d(self, vel, i0, i1, wSmooth=0.0, wEnergy=0.0, level=0, postVelBlur=0.0,
                                cgAccuracy=1e-4, blurType=1, cfl=999.0, orderTime=1, orderSpace=1,
                                resetBndWidth=-1.0, multiStep=1, projSizeThresh=9999, minGridSize=10,
                                doFinalProject=False, cgMaxIter=1000):
        v = self._arr(vel).copy()
        a = self._arr(i0)
        b = self._arr(i1)
        f = np.array([wSmooth, wEnergy, postVelBlur, cgAccuracy, cfl, resetBndWidth], dtype=self.dtype)
        k = np.array([level, blurType, orderTime, orderSpace, multiStep, projSizeThresh, minGridSize,
                      int(bool(doFinalProject)), cgMaxIter], dtype=np.int32)
        self._f("statsReset")()
        err = self._f("opticalFlowMultiscale4d")(self._p(self._dims(dims_of(a))), self._p(v), self._p(a),
                                                 self._p(b), self._p(f), self._p(k))
        return v, err, self.stats()

    def stats(self):
        cap = 256
        it = np.zeros(cap, dtype=np.int32)
        sz = np.zeros(cap, dtype=np.int32)
        rs = np.zeros(cap, dtype=self.dtype)
        n = self._f("statsGet")(self._p(it), self._p(sz), self._p(rs), cap)
        n = min(n, cap)
        return [(int(sz[q]), int(it[q]), float(rs[q])) for q in range(n)]

    # -- apply ---------------------------------------------------------------
    def deform4d(self, vel, velInv, i0, i1, alpha, twoway=1):
        v = self._arr(vel)
        vi = self._arr(velInv) if velInv is not None else v
        a = self._arr(i0)
        b = self._arr(i1)
        out = np.zeros_like(a)
        alphaInv = float(np.asarray(1.0 - alpha, dtype=self.dtype))
        self._f("deform4d")(self._p(self._dims(dims_of(a))), self._p(v), self._p(vi), self._p(a), self._p(b),
                            self._p(out), alpha, alphaInv, int(twoway))
        return out

    def optRunFrame(self, defo, dst, phi, time, blendAlpha, loadTimeScale=1.0, defoOffset=(0, 0, 0, 0),
                    defoScale=(1, 1, 1, 1), defoFactor=(1, 1, 1, 1), overrideSize=(-1, -1, -1, -1),
                    overrideTimeOff=0.0, bordSkip=1, defoAniFac=1.0):
        dfo = self._arr(defo)
        d = self._arr(dst).copy()
        p = self._arr(phi)
        dd = self._dims((d.shape[2], d.shape[1], d.shape[0], 1))
        self._f("optRunFrame")(self._p(self._dims(dims_of(dfo))), self._p(dfo), self._p(dd), self._p(d),
                               self._p(self._dims(dims_of(p))), self._p(p), time, blendAlpha, loadTimeScale,
                               self._p(self._vec(defoOffset)), self._p(self._vec(defoScale)),
                               self._p(self._vec(defoFactor)), self._p(self._vec(overrideSize)),
                               overrideTimeOff, int(bordSkip), defoAniFac)
        return d


_cache: dict = {}


def get(double: bool = False) -> Oracle:
    if double not in _cache:
        _cache[double] = Oracle(double)
    return _cache[double]
