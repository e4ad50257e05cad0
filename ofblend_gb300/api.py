"""The reference's Python call surface for the FlOF path, backed by the CUDA
library.

scenes/flof.py drives the reference through mantaflow's Python bindings:
``Solver(...)`` with ``solv.create(Grid4Real / Grid4Vec4 / RealGrid)``, the
Grid4d methods (source/grid4d.h:205-236) and the plugins
``opticalFlowMultiscale4d``, ``advect4d``, ``calcLsDiff4d``,
``interpolateGrid4d(Vec)``, ``loadAdvectTimeSlice_Opt*`` and helpers from
source/plugin/optflow4d.cpp and source/grid4d.cpp.  This module offers the
same names, keyword arguments and defaults, so a flof.py-shaped driver runs
with a changed import.  Grids live in GPU memory; ``to_numpy`` /
``from_numpy`` move their contents (layout x fastest, arrays shaped
(T, Z, Y, X) or (T, Z, Y, X, 4)).

Errors surface as FlofError (a RuntimeError), as the reference's errMsg
exceptions surface as Python errors.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import _lib
from ._lib import FLOF_REAL, FLOF_VEC4, FlofError, OFParams, SolveStats, check, f4, lib

__all__ = [
    "FlofError", "Context", "context", "Solver", "Grid4Real", "Grid4Vec4", "RealGrid",
    "vec3", "vec4", "Vec3", "Vec4",
    "opticalFlowMultiscale4d", "opticalFlow4d", "corrVelsOf4d", "advect4d", "calcLsDiff4d",
    "gaussianBlur4d",
    "interpolateGrid4d", "interpolateGrid4dVec", "deform4d",
    "loadAdvectTimeSlice_OptInit", "loadAdvectTimeSlice_OptRun",
    "loadAdvectTimeSlice_OptRunTwoway", "loadAdvectTimeSlice_Finish", "last_solve_stats",
    "LevelsetGrid", "repeatFrame4d", "extrap4dLsSimple", "simpleBlurSpecial", "shiftForwGrid4d",
    "uniFileInfo", "getUniFileSize", "readGrid4dUniSlice", "loadPlaceGrid4d", "loadAdvectTimeSlice",
    "opticalFlowMultiscale4d_batch", "Model",
]


# ---------------------------------------------------------------------------
# small vector types (the scenes use vec3 / vec4 / Vec3 / Vec4)
# ---------------------------------------------------------------------------
class vec4:
    def __init__(self, x=0.0, y=None, z=None, t=None):
        if y is None:
            y = z = t = x
        self.x, self.y, self.z, self.t = float(x), float(y), float(z if z is not None else 0.0), \
            float(t if t is not None else 0.0)

    def __iter__(self):
        return iter((self.x, self.y, self.z, self.t))

    def __repr__(self):
        return f"vec4({self.x}, {self.y}, {self.z}, {self.t})"


class vec3(vec4):
    def __init__(self, x=0.0, y=None, z=None):
        if y is None:
            y = z = x
        super().__init__(x, y, z if z is not None else 0.0, 0.0)

    def __iter__(self):
        return iter((self.x, self.y, self.z))

    def __repr__(self):
        return f"vec3({self.x}, {self.y}, {self.z})"


Vec3 = vec3
Vec4 = vec4


# ---------------------------------------------------------------------------
# context
# ---------------------------------------------------------------------------
class Context:
    """One flof_ctx: a CUDA stream plus a device buffer pool on one GPU."""

    def __init__(self, device: int = 0):
        self.lib = _lib.lib()
        h = ctypes.c_void_p()
        check(self.lib.flof_ctx_create(int(device), ctypes.byref(h)))
        self.h = h
        self.device = device

    def synchronize(self):
        check(self.lib.flof_ctx_synchronize(self.h))

    def copies_sync(self):
        """Wait on the host for every asynchronous grid copy of the context."""
        check(self.lib.flof_ctx_copies_sync(self.h))

    def kernel_launches(self) -> int:
        return int(self.lib.flof_ctx_kernel_launches(self.h))

    def set_stream(self, stream_handle: int | None):
        check(self.lib.flof_ctx_set_stream(self.h, ctypes.c_void_p(stream_handle or 0)))

    def trim(self):
        check(self.lib.flof_ctx_trim(self.h))

    def set_option(self, option: int, value: int):
        """flof_ctx_set_option, e.g. _lib.FLOF_OPT_CFL_SYNC."""
        check(self.lib.flof_ctx_set_option(self.h, int(option), int(value)))

    def set_mg_params(self, omega0=0.95, omegac=1.0, lam=0.9, coarse_sweeps=8, max_iter=200):
        """flof_ctx_set_mg_params: the V-cycle of solver="mg" and its
        iteration cap before the plain PCG takes over."""
        check(self.lib.flof_ctx_set_mg_params(self.h, float(omega0), float(omegac), float(lam),
                                              int(coarse_sweeps), int(max_iter)))

    def mg_fallbacks(self) -> int:
        """Solves of solver="mg" that the plain PCG had to finish."""
        return int(self.lib.flof_ctx_mg_fallbacks(self.h))

    def profile(self, enable: bool = True):
        """Start (clearing old records) or stop per-launch event tracing."""
        check(self.lib.flof_ctx_profile(self.h, int(bool(enable))))

    def profile_records(self):
        """[(kernel class, grid X extent, algorithmic bytes, device ms)]."""
        n = ctypes.c_int()
        check(self.lib.flof_ctx_profile_count(self.h, ctypes.byref(n)))
        out = []
        cls, sx, ms = ctypes.c_int(), ctypes.c_int(), ctypes.c_float()
        nb = ctypes.c_double()
        names = {}
        for i in range(n.value):
            check(self.lib.flof_ctx_profile_record(self.h, i, ctypes.byref(cls), ctypes.byref(sx),
                                                   ctypes.byref(nb), ctypes.byref(ms)))
            if cls.value not in names:
                names[cls.value] = self.lib.flof_kernel_class_name(cls.value).decode()
            out.append((names[cls.value], sx.value, nb.value, ms.value))
        return out

    def close(self):
        if getattr(self, "h", None):
            self.lib.flof_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_ctx: Context | None = None


def context() -> Context:
    """The process-wide default context on cuda:0 (created on first use)."""
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


# ---------------------------------------------------------------------------
# grids
# ---------------------------------------------------------------------------
class _Grid:
    ELEM = FLOF_REAL
    NC = 1

    def __init__(self, parent: "Solver" | None = None, dims=None, ctx: Context | None = None,
                 data_ptr: int | None = None, name: str = ""):
        self.ctx = ctx or (parent.ctx if parent is not None else context())
        if dims is None:
            if parent is None:
                raise FlofError(1, "a grid needs a parent solver or explicit dims")
            dims = parent.grid_dims(self._is3d())
        self.dims = tuple(int(a) for a in dims)
        self.name = name
        h = ctypes.c_void_p()
        cd = (ctypes.c_int * 4)(*self.dims)
        L = self.ctx.lib
        if data_ptr is None:
            check(L.flof_grid_create(self.ctx.h, cd, self.ELEM, ctypes.byref(h)))
        else:
            check(L.flof_grid_wrap(self.ctx.h, cd, self.ELEM, ctypes.c_void_p(data_ptr), ctypes.byref(h)))
        self.h = h

    @staticmethod
    def _is3d():
        return False

    # -- sizes ------------------------------------------------------------------
    def getSizeX(self): return self.dims[0]
    def getSizeY(self): return self.dims[1]
    def getSizeZ(self): return self.dims[2]
    def getSizeT(self): return self.dims[3]

    def getSize(self):
        return vec4(*self.dims)

    @property
    def shape(self):
        X, Y, Z, T = self.dims
        return (T, Z, Y, X, 4) if self.NC == 4 else (T, Z, Y, X)

    def data_ptr(self) -> int:
        return int(self.ctx.lib.flof_grid_data(self.h) or 0)

    # -- host transfer ----------------------------------------------------------
    def from_numpy(self, a):
        a = np.ascontiguousarray(a, dtype=np.float32)
        if a.size != int(np.prod(self.shape)):
            raise FlofError(1, f"array of {a.size} floats does not fit grid {self.dims} x {self.NC}")
        check(self.ctx.lib.flof_grid_upload(self.h, a.ctypes.data_as(ctypes.c_void_p)))
        return self

    def to_numpy(self, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty(self.shape, dtype=np.float32)
        check(self.ctx.lib.flof_grid_download(self.h, out.ctypes.data_as(ctypes.c_void_p)))
        return out

    # -- asynchronous host transfers (copy stream of the context) ---------------
    def _host_buf(self, a):
        if not (isinstance(a, np.ndarray) and a.dtype == np.float32 and a.flags.c_contiguous
                and a.size == int(np.prod(self.shape))):
            raise FlofError(1, f"need a C-contiguous float32 array of {int(np.prod(self.shape))} "
                               "floats (pinned for overlap)")
        return a.ctypes.data_as(ctypes.c_void_p)

    def upload_async(self, a):
        """Queue host -> grid on the copy stream; call copy_wait() before
        work that reads the grid.  `a` must stay alive until the copy ends."""
        check(self.ctx.lib.flof_grid_upload_async(self.h, self._host_buf(a)))
        return self

    def download_async(self, out):
        """Queue grid -> host on the copy stream after the work queued so far;
        call copy_wait() before work that writes the grid, and
        Context.copies_sync() before reading `out`."""
        check(self.ctx.lib.flof_grid_download_async(self.h, self._host_buf(out)))
        return out

    def copy_wait(self):
        """The context stream waits (on the device) for this grid's last
        asynchronous copy."""
        check(self.ctx.lib.flof_grid_copy_wait(self.h))
        return self

    # -- Grid4d methods (grid4d.h:205-236) --------------------------------------
    def copyFrom(self, a, copyType=True):
        check(self.ctx.lib.flof_grid_copyFrom(self.h, a.h))
        return self

    def add(self, a):
        check(self.ctx.lib.flof_grid_add(self.h, a.h))

    def sub(self, a):
        check(self.ctx.lib.flof_grid_sub(self.h, a.h))

    def setConst(self, s):
        check(self.ctx.lib.flof_grid_setConst(self.h, f4(s)))

    def addConst(self, s):
        check(self.ctx.lib.flof_grid_addConst(self.h, f4(s)))

    def multConst(self, s):
        check(self.ctx.lib.flof_grid_multConst(self.h, f4(s)))

    def addScaled(self, a, factor):
        check(self.ctx.lib.flof_grid_addScaled(self.h, a.h, f4(factor)))

    def clear(self):
        check(self.ctx.lib.flof_grid_clear(self.h))

    def _reduce(self, fn):
        out = ctypes.c_float()
        check(fn(self.h, ctypes.byref(out)))
        return float(out.value)

    def getMax(self):
        return self._reduce(self.ctx.lib.flof_grid_getMax)

    def getMin(self):
        return self._reduce(self.ctx.lib.flof_grid_getMin)

    def getMaxAbs(self):
        return self._reduce(self.ctx.lib.flof_grid_getMaxAbs)

    getMaxValue = getMax
    getMinValue = getMin
    getMaxAbsValue = getMaxAbs

    def setBound(self, value, boundaryWidth=1):
        check(self.ctx.lib.flof_grid_setBound(self.h, f4(value), int(boundaryWidth)))

    def setBoundNeumann(self, boundaryWidth=1):
        check(self.ctx.lib.flof_grid_setBoundNeumann(self.h, int(boundaryWidth)))

    def join(self, a):
        """LevelsetGrid::join (levelset.cpp:114-118): self = min(self, a)."""
        check(self.ctx.lib.flof_grid_join(self.h, a.h))

    # -- .uni files (fileio.cpp:834-1000) -----------------------------------------
    def load(self, name):
        """Grid4d::load / Grid<T>::load of a .uni file."""
        check(self.ctx.lib.flof_grid_load(self.h, os.fsencode(name)))
        return self

    def save(self, name):
        """Grid4d::save (M4T2) / Grid<Real>::save (MNT2)."""
        check(self.ctx.lib.flof_grid_save(self.h, os.fsencode(name), 0 if self._is3d() else 1))

    def free(self):
        if getattr(self, "h", None) is not None:
            self.ctx.lib.flof_grid_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Grid4Real(_Grid):
    """Grid4d<Real>."""
    ELEM = FLOF_REAL
    NC = 1


class Grid4Vec4(_Grid):
    """Grid4d<Vec4>."""
    ELEM = FLOF_VEC4
    NC = 4


class RealGrid(_Grid):
    """A 3D Grid<Real> (t extent 1), the output of the mode-3 slice lookup.
    Its border methods follow Grid<T> (grid.cpp:462-511): the z planes count
    only when the z extent is above 1."""
    ELEM = FLOF_REAL
    NC = 1

    @staticmethod
    def _is3d():
        return True

    @property
    def shape(self):
        X, Y, Z, _ = self.dims
        return (Z, Y, X)

    def setBound(self, value, boundaryWidth=1):
        check(self.ctx.lib.flof_grid3_setBound(self.h, f4(value), int(boundaryWidth)))

    def setBoundNeumann(self, boundaryWidth=1):
        check(self.ctx.lib.flof_grid3_setBoundNeumann(self.h, int(boundaryWidth)))


LevelsetGrid = RealGrid


class Solver:
    """FluidSolver stand-in: holds the grid size, the 4th dimension and dt
    (source/fluidsolver.h), and creates grids on the GPU."""

    def __init__(self, name="main", gridSize=None, dim=3, fourthDim=-1, ctx: Context | None = None):
        if gridSize is None:
            raise FlofError(1, "Solver needs gridSize")
        self.name = name
        gs = list(gridSize)
        self.gridSize = (int(gs[0]), int(gs[1]), int(gs[2]))
        self.dim = dim
        self.fourthDim = int(fourthDim)
        self.timestep = 1.0
        self.ctx = ctx or context()

    def grid_dims(self, is3d=False):
        X, Y, Z = self.gridSize
        T = 1 if is3d else max(self.fourthDim, 1)
        return (X, Y, Z, T)

    def create(self, cls, name=""):
        return cls(self, name=name)

    def getDt(self):
        return self.timestep

    def step(self):
        pass


# ---------------------------------------------------------------------------
# plugins
# ---------------------------------------------------------------------------
_last_stats: dict | None = None


def last_solve_stats() -> dict | None:
    """The solve record of the last opticalFlowMultiscale4d call."""
    return _last_stats


def _ctx_of(g) -> Context:
    return g.ctx


def _of_params(wSmooth=0.0, wEnergy=0.0, level=0, postVelBlur=0.0, cgAccuracy=1e-04, blurType=1, cfl=999,
               orderTime=1, orderSpace=1, resetBndWidth=-1.0, multiStep=1, projSizeThresh=9999,
               minGridSize=10, doFinalProject=False, cgMaxIter=1000, precision="fp32", warmStart=False,
               solver="pcg"):
    p = OFParams()
    _lib.lib().flof_of_params_default(ctypes.byref(p))
    p.wSmooth, p.wEnergy, p.level = wSmooth, wEnergy, int(level)
    p.postVelBlur, p.cgAccuracy, p.blurType = postVelBlur, cgAccuracy, int(blurType)
    p.cfl, p.orderTime, p.orderSpace = cfl, int(orderTime), int(orderSpace)
    p.resetBndWidth, p.multiStep = resetBndWidth, int(multiStep)
    p.projSizeThresh, p.minGridSize = int(projSizeThresh), int(minGridSize)
    p.doFinalProject, p.cgMaxIter = int(bool(doFinalProject)), int(cgMaxIter)
    prec = {"fp32": _lib.FLOF_PRECISION_FP32, "mixed": _lib.FLOF_PRECISION_MIXED}
    if precision not in prec:
        raise FlofError(1, "precision must be 'fp32' or 'mixed'")
    p.precision = prec[precision]
    p.warmStart = int(bool(warmStart))
    solvers = {"pcg": _lib.FLOF_SOLVER_PCG, "mg": _lib.FLOF_SOLVER_MG}
    if solver not in solvers:
        raise FlofError(1, "solver must be 'pcg' or 'mg'")
    p.solver = solvers[solver]
    return p


def opticalFlowMultiscale4d(vel, i0, i1, rhsT=None, wSmooth=0.0, wEnergy=0.0, level=0, postVelBlur=0.0,
                            cgAccuracy=1e-04, blurType=1, cfl=999, orderTime=1, orderSpace=1,
                            resetBndWidth=-1.0, multiStep=1, projSizeThresh=9999, minGridSize=10,
                            doFinalProject=False, cgMaxIter=1000, precision="fp32", warmStart=False,
                            solver="pcg"):
    """opticalFlowMultiscale4d (optflow4d.cpp:2182-2195); returns the final
    error metric (the reference's template returns it to C++ callers).
    solver="mg" preconditions the CG with a multigrid V-cycle (same stop
    rule; the plain PCG judges and finishes);
    precision="mixed" solves with the BF16-stored gradient and FP64
    iterative refinement; warmStart=True starts the coarsest level from the
    model attached with Model.attach (neither has a reference counterpart)."""
    global _last_stats
    p = _of_params(wSmooth, wEnergy, level, postVelBlur, cgAccuracy, blurType, cfl, orderTime, orderSpace,
                   resetBndWidth, multiStep, projSizeThresh, minGridSize, doFinalProject, cgMaxIter,
                   precision, warmStart, solver)
    err = ctypes.c_float()
    st = SolveStats()
    ctx = _ctx_of(vel)
    check(ctx.lib.flof_opticalFlowMultiscale4d(ctx.h, vel.h, i0.h, i1.h, ctypes.byref(p),
                                               ctypes.byref(err), ctypes.byref(st)))
    _last_stats = st.as_dict()
    return float(err.value)


def opticalFlowMultiscale4d_batch(vels, i0s, i1s, workers=0, **params):
    """Independent opticalFlowMultiscale4d solves (same keyword parameters,
    any sizes) run concurrently on worker streams; returns the error metrics.
    Each result equals the single call's on the same grids."""
    n = len(vels)
    if not (len(i0s) == n and len(i1s) == n):
        raise FlofError(1, "vels, i0s and i1s must have the same length")
    if n == 0:
        return []
    p = _of_params(**params)
    ctx = _ctx_of(vels[0])
    arr = lambda gs: (ctypes.c_void_p * n)(*[g.h.value for g in gs])
    errs = (ctypes.c_float * n)()
    check(ctx.lib.flof_opticalFlowMultiscale4d_batch(ctx.h, n, arr(vels), arr(i0s), arr(i1s), ctypes.byref(p),
                                                     errs, int(workers)))
    return [float(e) for e in errs]


def opticalFlow4d(vel, i0, i1, rhsT=None, wSmooth=0.0, wEnergy=0.0, postVelBlur=0.0, cgAccuracy=1e-04,
                  blurType=1, resetBndWidth=-1.0, cgMaxIter=1000):
    """opticalFlow4d (optflow4d.cpp:2110-2119); returns (iterations, residual)."""
    ctx = _ctx_of(vel)
    it = ctypes.c_int()
    res = ctypes.c_float()
    check(ctx.lib.flof_opticalFlow4d(ctx.h, vel.h, i0.h, i1.h, wSmooth, wEnergy, postVelBlur, cgAccuracy,
                                     int(blurType), resetBndWidth, int(cgMaxIter), ctypes.byref(it),
                                     ctypes.byref(res)))
    return int(it.value), float(res.value)


def corrVelsOf4d(dst, vel, phiOrg, phiCurr, phiTarget, threshPhi=1e10, threshNorm=1e10, postVelBlur=0.0,
                 resetBndWidth=-1.0, maxIter=100):
    """corrVelsOf4d (optflow4d.cpp:2121-2130)."""
    ctx = _ctx_of(vel)
    check(ctx.lib.flof_corrVelsOf4d(ctx.h, dst.h, vel.h, phiOrg.h, phiCurr.h if phiCurr is not None else None,
                                    phiTarget.h, threshPhi, threshNorm, postVelBlur, resetBndWidth,
                                    int(maxIter)))


def gaussianBlur4d(grid, sigma, blurType=1):
    """gaussianBlurGeneric (optflow4d.cpp:160-174) on a Real or Vec4 grid."""
    ctx = _ctx_of(grid)
    check(ctx.lib.flof_gaussianBlur4d(ctx.h, grid.h, float(sigma), int(blurType)))


def advect4d(vel, grid, dtFac=1.0):
    """advect4d (optflow4d.cpp:1292-1306)."""
    ctx = _ctx_of(vel)
    check(ctx.lib.flof_advect4d(ctx.h, vel.h, grid.h, dtFac))


def calcLsDiff4d(i0, i1, out=None, correction=1.0, bnd=0):
    """calcLsDiff4d (optflow4d.cpp:2132-2137)."""
    ctx = _ctx_of(i0)
    r = ctypes.c_float()
    check(ctx.lib.flof_calcLsDiff4d(ctx.h, i0.h, i1.h, out.h if out is not None else None, correction,
                                    int(bnd), ctypes.byref(r)))
    return float(r.value)


def interpolateGrid4d(target, source, offset=None, scale=None, size=None):
    """interpolateGrid4d (grid4d.cpp:539-547)."""
    ctx = _ctx_of(target)
    check(ctx.lib.flof_interpolateGrid4d(ctx.h, target.h, source.h, f4(offset if offset is not None else 0.0),
                                         f4(scale if scale is not None else 1.0),
                                         f4(size if size is not None else -1.0)))


def interpolateGrid4dVec(target, source, offset=None, scale=None, size=None):
    """interpolateGrid4dVec (grid4d.cpp:549-557)."""
    ctx = _ctx_of(target)
    check(ctx.lib.flof_interpolateGrid4dVec(ctx.h, target.h, source.h,
                                            f4(offset if offset is not None else 0.0),
                                            f4(scale if scale is not None else 1.0),
                                            f4(size if size is not None else -1.0)))


def deform4d(out, i0, i1, vel, velInv=None, alpha=1.0, twoway=1):
    """The mode-2 apply of scenes/flof.py deform4d (:591-615) in one call."""
    ctx = _ctx_of(out)
    alphaInv = float(np.float32(1.0 - alpha))
    check(ctx.lib.flof_deform4d(ctx.h, out.h, i0.h, i1.h if i1 is not None else None, vel.h,
                                velInv.h if velInv is not None else None, float(alpha), alphaInv,
                                int(twoway)))


def loadAdvectTimeSlice_OptInit(ID, fname1, useDefoVols=False, doAligned=False, partialLoadFac=0.2,
                                ctx: Context | None = None):
    """loadAdvectTimeSlice_OptInit (optflow4d.cpp:1871-1913).  `fname1` is the
    .uni deformation file (loaded whole into device memory) or a GPU-resident
    Grid4Vec4."""
    if isinstance(fname1, (str, os.PathLike)):
        ctx = ctx or context()
        check(ctx.lib.flof_loadAdvectTimeSlice_OptInitFile(
            ctx.h, int(ID), os.fsencode(fname1), int(bool(useDefoVols)), int(bool(doAligned)),
            float(partialLoadFac)))
        _lats_ctx[int(ID)] = (ctx, None)
        return
    if not isinstance(fname1, Grid4Vec4):
        raise FlofError(1, "loadAdvectTimeSlice_OptInit expects a file name or a Grid4Vec4")
    ctx = fname1.ctx
    check(ctx.lib.flof_loadAdvectTimeSlice_OptInit(ctx.h, int(ID), fname1.h, int(bool(useDefoVols)),
                                                   int(bool(doAligned)), float(partialLoadFac)))
    _lats_ctx[int(ID)] = (ctx, fname1)  # keeps the deformation grid alive until Finish


_lats_ctx: dict = {}


def loadAdvectTimeSlice_OptRun(ID, fname, dst, phi, time, blendAlpha, loadTimeScale, defoOffset, defoScale,
                               defoFactor, overrideSize=None, overrideTimeOff=0.0, debugVel=None,
                               debugVelT=None, zeroVel=False, thirdAlpha=0.0, bordSkip=1, fourthAlpha=0.0,
                               defoAniFac=1.0):
    """loadAdvectTimeSlice_OptRun (optflow4d.cpp:1951-2105); `fname` is
    accepted for call compatibility and ignored (the deformation was bound
    at OptInit)."""
    ctx = dst.ctx
    check(ctx.lib.flof_loadAdvectTimeSlice_OptRun(
        ctx.h, int(ID), dst.h, phi.h, float(time), float(blendAlpha), float(loadTimeScale), f4(defoOffset),
        f4(defoScale), f4(defoFactor), f4(overrideSize if overrideSize is not None else -1.0),
        float(overrideTimeOff), int(bool(zeroVel)), float(thirdAlpha), int(bordSkip), float(fourthAlpha),
        float(defoAniFac)))


def loadAdvectTimeSlice_OptRunTwoway(ID0, ID1, dst, phi0, phi1, time, blendAlpha, loadTimeScale, defoOffset,
                                     defoScale, defoFactor, overrideSize=None, overrideTimeOff=0.0, bordSkip=1,
                                     defoAniFac=1.0):
    """Both directions of a two-way frame and their blend
    (scenes/flof.py:750-755) in one GPU pass."""
    ctx = dst.ctx
    alphaInv = float(np.float32(1.0 - blendAlpha))
    check(ctx.lib.flof_loadAdvectTimeSlice_OptRunTwoway(
        ctx.h, int(ID0), int(ID1), dst.h, phi0.h, phi1.h, float(time), float(blendAlpha), alphaInv,
        float(loadTimeScale), f4(defoOffset), f4(defoScale), f4(defoFactor),
        f4(overrideSize if overrideSize is not None else -1.0), float(overrideTimeOff), int(bordSkip),
        float(defoAniFac)))


def loadAdvectTimeSlice_Finish(ID):
    """loadAdvectTimeSlice_Finish (optflow4d.cpp:1930-1950)."""
    ent = _lats_ctx.pop(int(ID), None)
    if ent is None:
        return
    ctx = ent[0]
    check(ctx.lib.flof_loadAdvectTimeSlice_Finish(ctx.h, int(ID)))


# ---------------------------------------------------------------------------
# input conditioning and output stage (scenes/flof.py postProcessPhiData,
# writeResults and the time-SDF merge)
# ---------------------------------------------------------------------------
def repeatFrame4d(phi, srct, range=0.0, bnd=0):
    """repeatFrame4d (optflow4d.cpp:1254-1266)."""
    check(phi.ctx.lib.flof_repeatFrame4d(phi.h, float(srct), float(range), int(bnd)))


def extrap4dLsSimple(phi, distance=4, inside=False):
    """extrap4dLsSimple (optflow4d.cpp:1332-1406)."""
    check(phi.ctx.lib.flof_extrap4dLsSimple(phi.h, int(distance), 1 if inside else 0))


def simpleBlurSpecial(a, iter=1, thresh=0.0, bord=0):
    """simpleBlurSpecial (test.cpp:116-131) of a 3D RealGrid."""
    check(a.ctx.lib.flof_simpleBlurSpecial(a.h, int(iter), float(thresh), int(bord)))


def shiftForwGrid4d(phi, overrideGoodRegion=0):
    """shiftForwGrid4d (optflow4d.cpp:1596-1616)."""
    check(phi.ctx.lib.flof_shiftForwGrid4d(phi.h, int(overrideGoodRegion)))


# ---------------------------------------------------------------------------
# .uni files, hi-res 4D assembly, non-optimised slice lookup
# ---------------------------------------------------------------------------
def uniFileInfo(name) -> dict:
    """Header of a .uni file: dims (x, y, z, t), 4D flag, grid type, element size."""
    L = lib()
    dims = (ctypes.c_int * 4)()
    is4d, gt, bpe = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    check(L.flof_uni_info(os.fsencode(name), dims, ctypes.byref(is4d), ctypes.byref(gt), ctypes.byref(bpe)))
    return {"dims": tuple(dims), "is4d": bool(is4d.value), "gridType": gt.value,
            "bytesPerElement": bpe.value}


def getUniFileSize(name):
    """getUniFileSize (fileio.cpp:572-604) as a vec3."""
    d = uniFileInfo(name)["dims"]
    return vec3(d[0], d[1], d[2])


def readGrid4dUniSlice(name, t, slice_grid):
    """readGrid4dUni(name, NULL, t, slice) (fileio.cpp:912-990): t slice of a
    4D file into a grid with t extent 1."""
    check(slice_grid.ctx.lib.flof_uni_read_slice(slice_grid.h, os.fsencode(name), int(t)))
    return slice_grid


def loadPlaceGrid4d(fname, phi, offset, scale, fileIdxStart=-1, fileIdxEnd=-1, debugSkipLoad=999999,
                    spread=1.0, overrideSize=None, overrideTimeOff=0.0, overrideGoodRegion=0,
                    loadTimeScale=1.0, rescaleSdfValues=False, sdfIsoOff=0.0, repeatStartFrame=0.0):
    """loadPlaceGrid4d (optflow4d.cpp:1460-1594).  `fname` is a file-name
    pattern with one integer conversion (3D .uni files) or a list of RealGrid
    slices, element q holding file index fileIdxStart + q."""
    L = phi.ctx.lib
    if isinstance(fname, (str, os.PathLike)):
        name, arr, n = os.fsencode(fname), None, 0
    else:
        grids = list(fname)
        arr = (ctypes.c_void_p * len(grids))(*[g.h.value for g in grids])
        name, n = None, len(grids)
    check(L.flof_loadPlaceGrid4d(
        phi.h, name, arr, n, f4(offset), f4(scale), int(fileIdxStart), int(fileIdxEnd), int(debugSkipLoad),
        float(spread), f4(overrideSize if overrideSize is not None else -1.0), float(overrideTimeOff),
        int(overrideGoodRegion), float(loadTimeScale), int(bool(rescaleSdfValues)), float(sdfIsoOff),
        float(repeatStartFrame)))


def loadAdvectTimeSlice(dummyID, fname, dst, phi, time, blendAlpha, loadTimeScale, defoOffset, defoScale,
                        defoFactor, overrideSize=None, overrideTimeOff=0.0, debugVel=None, debugVelT=None,
                        zeroVel=False, thirdAlpha=0.0, bordSkip=1, fourthAlpha=0.0, defoAniFac=1.0):
    """loadAdvectTimeSlice (optflow4d.cpp:1671-1760), the non-optimised twin of
    OptRun.  `fname` is the .uni deformation file or a Grid4Vec4; debugVel /
    debugVelT outputs are not offered (they must be None)."""
    if debugVel is not None or debugVelT is not None:
        raise FlofError(1, "debugVel / debugVelT outputs are not supported")
    ctx = dst.ctx
    if isinstance(fname, (str, os.PathLike)):
        defo, name = None, os.fsencode(fname)
    else:
        defo, name = fname.h, None
    check(ctx.lib.flof_loadAdvectTimeSlice(
        ctx.h, defo, name, dst.h, phi.h, float(time), float(blendAlpha), float(loadTimeScale),
        f4(defoOffset), f4(defoScale), f4(defoFactor), f4(overrideSize if overrideSize is not None else -1.0),
        float(overrideTimeOff), int(bool(zeroVel)), float(defoAniFac)))


# ---------------------------------------------------------------------------
# learned warm start
# ---------------------------------------------------------------------------
class Model:
    """The learned warm start: a 4D convolutional encoder-decoder mapping the
    coarsest-level inputs (i0, i1 on a res^4 grid) of the multiscale solve to
    that level's deformation.  Trained and evaluated on the GPU."""

    def __init__(self, res: int = 16, ctx: Context | None = None, seed: int = 0):
        self.ctx = ctx or context()
        self.res = int(res)
        h = ctypes.c_void_p()
        check(self.ctx.lib.flof_model_create(self.ctx.h, self.res, ctypes.byref(h)))
        self.h = h
        self.init(seed)

    def init(self, seed: int = 0):
        check(self.ctx.lib.flof_model_init(self.h, ctypes.c_ulonglong(int(seed))))

    @property
    def num_params(self) -> int:
        n = ctypes.c_longlong()
        check(self.ctx.lib.flof_model_num_params(self.h, ctypes.byref(n)))
        return int(n.value)

    def get_params(self) -> np.ndarray:
        out = np.empty(self.num_params, np.float32)
        check(self.ctx.lib.flof_model_get_params(self.h, out.ctypes.data_as(ctypes.c_void_p)))
        return out

    def set_params(self, a):
        a = np.ascontiguousarray(a, dtype=np.float32)
        if a.size != self.num_params:
            raise FlofError(1, f"expected {self.num_params} parameters, got {a.size}")
        check(self.ctx.lib.flof_model_set_params(self.h, a.ctypes.data_as(ctypes.c_void_p)))

    def save(self, path):
        np.save(path, self.get_params())

    def load(self, path):
        self.set_params(np.load(path))
        return self

    def predict(self, i0, i1, vel):
        check(self.ctx.lib.flof_model_predict(self.h, i0.h, i1.h, vel.h))
        return vel

    def loss_grad(self, i0, i1, target):
        """(loss, gradient w.r.t. the parameters) of one sample."""
        loss = ctypes.c_double()
        g = np.empty(self.num_params, np.float32)
        check(self.ctx.lib.flof_model_loss_grad(self.h, i0.h, i1.h, target.h, ctypes.byref(loss),
                                                g.ctypes.data_as(ctypes.c_void_p)))
        return float(loss.value), g

    def train_step(self, samples, lr: float = 1e-3) -> float:
        """One Adam step on the mean loss of [(i0, i1, target), ...]."""
        n = len(samples)
        arr = lambda k: (ctypes.c_void_p * n)(*[s[k].h.value for s in samples])
        loss = ctypes.c_double()
        check(self.ctx.lib.flof_model_train_step(self.h, n, arr(0), arr(1), arr(2), float(lr),
                                                 ctypes.byref(loss)))
        return float(loss.value)

    def attach(self):
        """Use this model when opticalFlowMultiscale4d is called with warmStart=True."""
        check(self.ctx.lib.flof_ctx_set_model(self.ctx.h, self.h))

    def detach(self):
        check(self.ctx.lib.flof_ctx_set_model(self.ctx.h, None))

    def free(self):
        if getattr(self, "h", None) is not None:
            self.ctx.lib.flof_model_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass
