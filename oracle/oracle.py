"""ctypes wrapper of the test oracle (TEST INFRASTRUCTURE).

Only tests, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import this
module, and only to check results.  The product path never does.

* ``liboracle.so``: the C restatement in ``pps_oracle.c`` (runs everywhere).
* ``_ref/libppsref.so``: the reference's own CPU solver headers compiled by
  ``make -C oracle ref`` (only where the reference sources are present).

Fields are float64 numpy arrays of shape (n2+2, n1+2, n0+2) -- x fastest -- where
n_d counts the boundary nodes, exactly the reference's guard-padded layout
(iterativeSolverBase.hpp:34-35).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libppsref.so")


def _ref_include() -> str:
    """Where the reference's solverPoissonMPI_CPU/include lies: $REF_INCLUDE, else
    the default of the recipe that compiles it (oracle/Makefile)."""
    if os.environ.get("REF_INCLUDE"):
        return os.environ["REF_INCLUDE"]
    with open(os.path.join(HERE, "Makefile")) as f:
        for line in f:
            if line.startswith("REF_INCLUDE ?="):
                return line.split("?=", 1)[1].strip()
    return ""


REF_INCLUDE = _ref_include()

BICGSTAB, CG, CHEBYSHEV_MAIN = 0, 1, 2
PREC_NONE, PREC_CHEBYSHEV, PREC_BICGSTAB, PREC_CG = 0, 1, 2, 3


class OraGrid(C.Structure):
    _fields_ = [("np", C.c_int * 3), ("ds", C.c_double * 3), ("origin", C.c_double * 3), ("bcs", C.c_int * 6)]


class OraConfig(C.Structure):
    _fields_ = [("krylov", C.c_int), ("precond", C.c_int), ("cheb_degree", C.c_int), ("cheb_eps", C.c_double),
                ("rescale_min", C.c_double), ("rescale_max", C.c_double), ("tol", C.c_double),
                ("maxit", C.c_int), ("threads", C.c_int), ("prec_tol", C.c_double), ("prec_maxit", C.c_int),
                ("prec_inner", C.c_int)]


class OraStats(C.Structure):
    _fields_ = [("iterations", C.c_int), ("err_iter", C.c_double), ("err_true", C.c_double),
                ("norm_b", C.c_double), ("seconds_loop", C.c_double), ("seconds_total", C.c_double),
                ("prec_iterations", C.c_int)]


@dataclass
class Grid:
    """Grid of a single-rank problem: npglobal (boundary nodes included), spacing,
    origin and boundary types x- x+ y- y+ z- z+ (0 Dirichlet, 1 Neumann)."""
    np: tuple
    ds: tuple
    origin: tuple = (0.0, 0.0, 0.0)
    bcs: tuple = (0, 0, 0, 0, 0, 0)

    @property
    def shape(self):
        return (self.np[2] + 2, self.np[1] + 2, self.np[0] + 2)

    def face_shape(self, f):
        d = f // 2
        n = list(self.np)
        rest = [n[a] for a in range(3) if a != d]
        return (rest[1], rest[0])

    def c(self):
        g = OraGrid()
        g.np[:] = list(self.np)
        g.ds[:] = list(self.ds)
        g.origin[:] = list(self.origin)
        g.bcs[:] = list(self.bcs)
        return g

    def unknown_slices(self):
        """numpy slices (z, y, x) selecting the unknowns (indexLimitsSolver_)."""
        sl = []
        for d in (2, 1, 0):
            lo = 1 + (1 if self.bcs[2 * d] == 0 else 0)
            hi = self.np[d] + 1 - (1 if self.bcs[2 * d + 1] == 0 else 0)
            sl.append(slice(lo, hi))
        return tuple(sl)

    def data_slices(self):
        return tuple(slice(1, self.np[d] + 1) for d in (2, 1, 0))


def cube(m, bcs=(0, 0, 0, 0, 0, 0)):
    """Unit cube with m interior unknowns per axis: npglobal = m+2, h = 1/(m+1)."""
    h = 1.0 / (m + 1)
    return Grid(np=(m + 2, m + 2, m + 2), ds=(h, h, h), bcs=tuple(bcs))


@dataclass
class Config:
    krylov: int = BICGSTAB
    precond: int = PREC_CHEBYSHEV
    cheb_degree: int = 11
    cheb_eps: float = 1e-4
    rescale_min: float = 500.0
    rescale_max: float = 1.0 - 1e-4
    tol: float = 1e-10
    maxit: int = 1700
    threads: int = 1
    # PREC_BICGSTAB / PREC_CG: the inner solver's toll_ and maxIteration, and its own
    # preconditioner (PREC_NONE, or PREC_CHEBYSHEV with the fields above)
    prec_tol: float = 1e-6
    prec_maxit: int = 150
    prec_inner: int = PREC_NONE

    def c(self):
        k = OraConfig()
        k.krylov, k.precond, k.cheb_degree = self.krylov, self.precond, self.cheb_degree
        k.cheb_eps, k.rescale_min, k.rescale_max = self.cheb_eps, self.rescale_min, self.rescale_max
        k.tol, k.maxit, k.threads = self.tol, self.maxit, self.threads
        k.prec_tol, k.prec_maxit, k.prec_inner = self.prec_tol, self.prec_maxit, self.prec_inner
        return k


CPU_PRESET = dict(cheb_degree=11, cheb_eps=1e-4, rescale_min=500.0, rescale_max=1.0 - 1e-4)
ALPAKA_PRESET = dict(cheb_degree=24, cheb_eps=0.0, rescale_min=100.0, rescale_max=1.0 - 1e-4)


@dataclass
class Result:
    iterations: int
    err_iter: float
    err_true: float
    norm_b: float
    seconds_loop: float
    seconds_total: float
    history: np.ndarray = field(repr=False, default=None)
    prec_iterations: int = 0


def build(ref: bool | None = None, quiet: bool = True) -> None:
    """Compile liboracle.so, and the reference library when its sources exist here."""
    out = subprocess.DEVNULL if quiet else None
    subprocess.run(["make", "-C", HERE, "all"], check=True, stdout=out)
    if ref is None:
        ref = bool(REF_INCLUDE) and os.path.isdir(REF_INCLUDE)
    if ref:
        subprocess.run(["make", "-C", HERE, "ref", f"REF_INCLUDE={REF_INCLUDE}"], check=True, stdout=out)


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build(ref=False)
        L = C.CDLL(LIB_PATH)
        dp = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
        L.ora_solve.argtypes = [C.POINTER(OraGrid), C.POINTER(OraConfig), dp, dp, C.c_void_p, C.c_void_p,
                                C.POINTER(OraStats)]
        L.ora_solve.restype = C.c_int
        L.ora_solve_stamped.argtypes = [C.POINTER(OraGrid), C.POINTER(OraConfig), dp, dp, C.c_void_p,
                                        C.c_void_p, C.POINTER(OraStats), C.c_void_p]
        L.ora_solve_stamped.restype = C.c_int
        L.ora_eigen_bounds.argtypes = [C.POINTER(OraGrid), C.POINTER(C.c_double)]
        L.ora_cheb_params.argtypes = [C.POINTER(OraGrid), C.POINTER(OraConfig), C.POINTER(C.c_double)]
        L.ora_apply_A.argtypes = [C.POINTER(OraGrid), dp, dp]
        L.ora_cheb_apply.argtypes = [C.POINTER(OraGrid), C.POINTER(OraConfig), dp, dp]
        L.ora_dot.argtypes = [C.POINTER(OraGrid), dp, dp]
        L.ora_dot.restype = C.c_double
        L.ora_set_problem.argtypes = [C.POINTER(OraGrid), C.c_int, dp, dp, C.c_void_p]
        L.ora_exact_solution.argtypes = [C.POINTER(OraGrid), C.c_int, dp]
        _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_PATH)


def ref_lib():
    global _ref
    if _ref is None:
        if not ref_available():
            raise FileNotFoundError("oracle/_ref/libppsref.so is not built (make -C oracle ref)")
        L = C.CDLL(REF_PATH)
        dp = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
        ip = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
        L.ref_solve.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, ip, dp, dp, ip, C.c_double, C.c_double,
                                C.c_double, C.c_double, C.c_int, dp, dp, C.c_void_p, C.POINTER(C.c_int), dp,
                                C.c_void_p]
        L.ref_solve.restype = C.c_int
        L.ref_solve2.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, ip, dp, dp, ip,
                                 C.c_double, C.c_double, C.c_double, C.c_double, C.c_int, dp, dp, C.c_void_p,
                                 C.POINTER(C.c_int), dp, C.c_void_p]
        L.ref_solve2.restype = C.c_int
        L.ref_set_problem.argtypes = [ip, dp, dp, ip, C.c_int, dp, dp]
        L.ref_table.argtypes = [ip, C.c_int]
        _ref = L
    return _ref


def _neumann_ptrs(grid: Grid, neumann):
    if neumann is None:
        return None, None
    arrs = [None if a is None else np.ascontiguousarray(a, np.float64) for a in neumann]
    ptrs = (C.c_void_p * 6)(*[None if a is None else a.ctypes.data for a in arrs])
    return ptrs, arrs


def new_field(grid: Grid) -> np.ndarray:
    return np.zeros(grid.shape, np.float64)


def set_problem(grid: Grid, problem: int, with_neumann: bool = True):
    """Fields x (Dirichlet values set), b (= f at every data node) and Neumann face
    arrays for a built-in manufactured problem (0 reference default, 1 sine product)."""
    x, b = new_field(grid), new_field(grid)
    faces = [np.zeros(grid.face_shape(f)) if (with_neumann and grid.bcs[f] == 1) else None for f in range(6)]
    ptrs, keep = _neumann_ptrs(grid, faces)
    rc = lib().ora_set_problem(C.byref(grid.c()), problem, x, b, ptrs)
    assert rc == 0
    return x, b, faces


def exact_solution(grid: Grid, problem: int) -> np.ndarray:
    u = new_field(grid)
    assert lib().ora_exact_solution(C.byref(grid.c()), problem, u) == 0
    return u


def solve(grid: Grid, cfg: Config, x: np.ndarray, b: np.ndarray, neumann=None) -> Result:
    """Oracle solve, in place on x and b like the reference."""
    assert x.shape == grid.shape and b.shape == grid.shape
    assert x.dtype == np.float64 and b.dtype == np.float64 and x.flags.c_contiguous and b.flags.c_contiguous
    hist = np.full(cfg.maxit + 1, -1.0)
    st = OraStats()
    ptrs, keep = _neumann_ptrs(grid, neumann)
    rc = lib().ora_solve(C.byref(grid.c()), C.byref(cfg.c()), x, b, ptrs, hist.ctypes.data, C.byref(st))
    if rc != 0:
        raise ValueError("oracle rejected the configuration")
    return Result(st.iterations, st.err_iter, st.err_true, st.norm_b, st.seconds_loop, st.seconds_total,
                  hist[: st.iterations + 1].copy(), st.prec_iterations)


def solve_stamped(grid: Grid, cfg: Config, x: np.ndarray, b: np.ndarray):
    """solve() for BiCGSTAB, also returning wall-clock stamps: [call start, end of
    iteration 1, ..., end of the last iteration, call end] (seconds, monotonic)."""
    assert cfg.krylov == BICGSTAB
    assert x.shape == grid.shape and b.shape == grid.shape
    hist = np.full(cfg.maxit + 1, -1.0)
    stamps = np.zeros(cfg.maxit + 2)
    st = OraStats()
    rc = lib().ora_solve_stamped(C.byref(grid.c()), C.byref(cfg.c()), x, b, None, hist.ctypes.data, C.byref(st),
                                 stamps.ctypes.data)
    if rc != 0:
        raise ValueError("oracle rejected the configuration")
    n = st.iterations
    res = Result(n, st.err_iter, st.err_true, st.norm_b, st.seconds_loop, st.seconds_total, hist[: n + 1].copy(),
                 st.prec_iterations)
    return res, stamps[: n + 2].copy()


def ref_solve(grid: Grid, cfg: Config, x: np.ndarray, b: np.ndarray, problem: int = 0, neumann=None) -> Result:
    """The reference's own classes, in place on x and b.  The reference plugin
    evaluates Neumann data from built-in problem `problem`, or looks it up in the
    face arrays `neumann` when they are given.  With an inner solver (PREC_BICGSTAB,
    PREC_CG) its tolerance is an integer multiple of the main one (a template
    argument there), so cfg.prec_tol must equal that multiple times cfg.tol exactly."""
    L = ref_lib()
    hist = np.full(cfg.maxit + 1, -1.0)
    it = C.c_int(0)
    errs = np.zeros(4)
    ptrs, keep = _neumann_ptrs(grid, neumann)
    if neumann is not None:
        problem = 2
    pratio = 0
    if cfg.krylov != CHEBYSHEV_MAIN and cfg.precond in (PREC_BICGSTAB, PREC_CG):
        pratio = int(round(cfg.prec_tol / cfg.tol))
        if float(pratio) * cfg.tol != cfg.prec_tol:
            raise ValueError("prec_tol must be an integer multiple of tol for the reference")
    rc = L.ref_solve2(cfg.krylov, cfg.precond, cfg.cheb_degree, cfg.maxit, cfg.prec_maxit, pratio, cfg.prec_inner,
                      np.array(grid.np, np.int32), np.array(grid.ds, np.float64), np.array(grid.origin, np.float64),
                      np.array(grid.bcs, np.int32), cfg.tol, cfg.cheb_eps, cfg.rescale_min, cfg.rescale_max, problem,
                      x, b, hist.ctypes.data, C.byref(it), errs, ptrs)
    if rc == -2:
        raise KeyError("combination not instantiated in oracle/_ref")
    n = it.value
    return Result(n, errs[0], errs[1], float("nan"), errs[2], errs[3], hist[: n + 1].copy())


def ref_table():
    out = np.zeros(4 * 256, np.int32)
    n = ref_lib().ref_table(out, 256)
    return [tuple(int(v) for v in out[4 * i: 4 * i + 4]) for i in range(n)]


def ref_set_problem(grid: Grid, problem: int):
    x, b = new_field(grid), new_field(grid)
    ref_lib().ref_set_problem(np.array(grid.np, np.int32), np.array(grid.ds, np.float64),
                              np.array(grid.origin, np.float64), np.array(grid.bcs, np.int32), problem, x, b)
    return x, b


def apply_A(grid: Grid, u: np.ndarray) -> np.ndarray:
    out = np.zeros_like(u)
    lib().ora_apply_A(C.byref(grid.c()), np.ascontiguousarray(u), out)
    return out


def cheb_apply(grid: Grid, cfg: Config, B: np.ndarray) -> np.ndarray:
    X = np.zeros_like(B)
    lib().ora_cheb_apply(C.byref(grid.c()), C.byref(cfg.c()), B, X)
    return X


def cheb_params(grid: Grid, cfg: Config):
    out = (C.c_double * 3)()
    lib().ora_cheb_params(C.byref(grid.c()), C.byref(cfg.c()), out)
    return tuple(out)


def eigen_bounds(grid: Grid):
    out = (C.c_double * 2)()
    lib().ora_eigen_bounds(C.byref(grid.c()), out)
    return tuple(out)


def dot(grid: Grid, a: np.ndarray, b: np.ndarray) -> float:
    return lib().ora_dot(C.byref(grid.c()), a, b)
