"""parallelpoissonsolver_gb300 -- GB300-native Poisson solve loop (host-side mirror).

The compute path is ``libpps.so`` (hand-written sm_103a CUDA behind the C ABI in
``include/pps.h``).  This module binds that ABI with ctypes and mirrors the
reference's solver-class protocol (solverPoissonMPI_CPU/include/inputParam.hpp:24-38):

    grid   = BlockGrid(npglobal=(66, 66, 66), ds=(1/65,)*3)
    solver = BiCGSTAB(grid, ChebyshevIteration(degree=11), tolerance=1e-10, max_iteration=1700)
    x, b   = grid.new_field(), grid.new_field()
    solver.set_problem(x, b)          # setProblem  (iterativeSolverBase.hpp:51-55)
    solver(x, b)                      # operator()  (BiCGSTAB.hpp:55-322)
    solver.get_num_iteration_final()  # getters     (iterativeSolverBase.hpp:410-425)

There is no CPU fallback: if libpps.so is missing or no GPU is visible, the
calls raise.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field
from typing import Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libpps.so")

OK, NOT_CONVERGED, BREAKDOWN, NAN_DETECTED, TIMEOUT = 0, 1, 2, 3, 4
ERR_INVALID_ARG, ERR_CUDA, ERR_OUT_OF_MEMORY, ERR_ZERO_RHS, ERR_UNSUPPORTED, ERR_NO_DEVICE = -1, -2, -3, -4, -5, -6
KRYLOV_BICGSTAB, KRYLOV_CG, KRYLOV_FCG, KRYLOV_CHEBYSHEV = 0, 1, 2, 3
PREC_NONE, PREC_CHEBYSHEV, PREC_BICGSTAB, PREC_CG = 0, 1, 2, 3
FORM_PARITY_FP64, FORM_FP64, FORM_MIXED = 0, 1, 2
FORMS = {"parity": FORM_PARITY_FP64, "fp64": FORM_FP64, "mixed": FORM_MIXED}
PRESET_CPU, PRESET_ALPAKA = 0, 1
PROBLEM_REFERENCE_DEFAULT, PROBLEM_SINE = 0, 1
LEARNED_INITIAL_GUESS, LEARNED_PRECONDITIONER, LEARNED_NO_FALLBACK, LEARNED_POST_SMOOTH = 1, 2, 4, 8
# coarsest-level solvers of the learned V-cycle (pps_set_coarse_solver)
COARSE_NETWORK, COARSE_ZERO, COARSE_SMOOTH, COARSE_EXACT = 0, 1, 2, 3

# Every symbol include/pps.h declares.
EXPORTED = [
    "pps_config_default", "pps_create", "pps_destroy", "pps_set_problem", "pps_set_problem_builtin",
    "pps_set_neumann", "pps_solve", "pps_solve_device", "pps_get_stats", "pps_get_history",
    "pps_write_residual_history", "pps_apply_operator", "pps_apply_preconditioner", "pps_device_count",
    "pps_status_string", "pps_last_error", "pps_abi_version", "pps_apply_operator_noalloc",
    "pps_autotune", "pps_get_tuning", "pps_set_tuning",
    "pps_batch_create", "pps_batch_destroy", "pps_batch_set", "pps_batch_get", "pps_batch_field_device",
    "pps_batch_autotune", "pps_batch_tile", "pps_batch_solve",
    "pps_unet_create", "pps_unet_destroy", "pps_unet_param_count", "pps_unet_get_params", "pps_unet_set_params",
    "pps_unet_forward", "pps_unet_gradients", "pps_unet_train_step", "pps_restrict2", "pps_prolong2",
    "pps_set_learned", "pps_unet_set_activation", "pps_set_learned_cycle", "pps_set_coarse_solver",
    "pps_write_solution", "pps_batch_set_wait_limit",
]


class PpsGrid(C.Structure):
    _fields_ = [("npglobal", C.c_int * 3), ("ds", C.c_double * 3), ("origin", C.c_double * 3),
                ("bcs", C.c_int * 6)]


class PpsConfig(C.Structure):
    _fields_ = [("krylov", C.c_int), ("precond", C.c_int), ("cheb_degree", C.c_int), ("cheb_eps", C.c_double),
                ("rescale_min", C.c_double), ("rescale_max", C.c_double), ("tol", C.c_double),
                ("maxit", C.c_int), ("form", C.c_int), ("inner_tol", C.c_double), ("inner_maxit", C.c_int),
                ("max_refinements", C.c_int), ("check_every", C.c_int), ("use_graph", C.c_int),
                ("device", C.c_int), ("precond_tol", C.c_double), ("precond_maxit", C.c_int),
                ("precond_inner", C.c_int)]


class PpsStats(C.Structure):
    _fields_ = [("iterations", C.c_int), ("refinements", C.c_int), ("precond_applications", C.c_int),
                ("err_iter", C.c_double), ("err_true", C.c_double), ("norm_b", C.c_double),
                ("seconds_solve", C.c_double), ("seconds_total", C.c_double), ("seconds_h2d", C.c_double),
                ("seconds_d2h", C.c_double), ("hbm_bytes", C.c_double), ("kernel_launches", C.c_int),
                ("sweep_seconds", C.c_double), ("sweep_launches", C.c_int), ("sweep_bytes", C.c_double),
                ("learned_applications", C.c_int), ("fallback_iteration", C.c_int),
                ("precond_iterations", C.c_int), ("krylov_seconds", C.c_double), ("krylov_launches", C.c_int),
                ("krylov_bytes", C.c_double), ("copy_overlap", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class PpsTuning(C.Structure):
    _fields_ = [("cheb_ty", C.c_int), ("cheb_cx", C.c_int), ("cheb_waves", C.c_int), ("other_ty", C.c_int),
                ("other_waves", C.c_int), ("cheb_us", C.c_double), ("other_us", C.c_double),
                ("cheb_fused", C.c_int), ("fcg_staged", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}

    OPTIONAL = {"cheb_fused": 0, "fcg_staged": 0}   # keys older stored tunings lack

    @classmethod
    def from_dict(cls, d):
        t = cls()
        for k, _ in cls._fields_:
            setattr(t, k, d.get(k, cls.OPTIONAL[k]) if k in cls.OPTIONAL else d[k])
        return t


class PpsBatchStats(C.Structure):
    _fields_ = [("seconds_solve", C.c_double), ("kernel_launches", C.c_int), ("graph_replays", C.c_int),
                ("max_err_true", C.c_double), ("max_iterations", C.c_int), ("sum_iterations", C.c_int),
                ("max_refinements", C.c_int), ("converged", C.c_int), ("unknowns", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class PpsError(RuntimeError):
    def __init__(self, status: int, where: str):
        msg = f"{where}: {status_string(status)}"
        detail = last_error()
        if detail:
            msg += f" ({detail})"
        super().__init__(msg)
        self.status = status


_lib = None


def lib_path() -> str:
    return LIB_PATH


def load(build_if_missing: bool = False):
    """Load libpps.so (raises if it is missing: there is no fallback path)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if build_if_missing:
            from . import build as _b
            _b.build()
        else:
            raise FileNotFoundError(f"{LIB_PATH} is not built; run parallelpoissonsolver_gb300.build.build()")
    L = C.CDLL(LIB_PATH)
    vp = C.c_void_p
    L.pps_config_default.argtypes = [C.POINTER(PpsConfig), C.c_int]
    L.pps_create.argtypes = [C.POINTER(PpsGrid), C.POINTER(PpsConfig), C.POINTER(vp)]
    L.pps_destroy.argtypes = [vp]
    L.pps_set_problem_builtin.argtypes = [vp, C.c_int, vp, vp]
    L.pps_set_neumann.argtypes = [vp, C.c_int, vp]
    L.pps_solve.argtypes = [vp, vp, vp, C.POINTER(PpsStats)]
    L.pps_solve_device.argtypes = [vp, vp, vp, C.POINTER(PpsStats)]
    L.pps_get_stats.argtypes = [vp, C.POINTER(PpsStats)]
    L.pps_get_history.argtypes = [vp, vp, C.c_int, C.POINTER(C.c_int)]
    L.pps_write_residual_history.argtypes = [vp, C.c_char_p]
    L.pps_apply_operator.argtypes = [vp, vp, vp]
    L.pps_apply_preconditioner.argtypes = [vp, vp, vp]
    L.pps_apply_operator_noalloc.argtypes = [C.POINTER(PpsGrid), vp, vp, vp, vp]
    L.pps_autotune.argtypes = [vp, C.POINTER(PpsTuning)]
    L.pps_get_tuning.argtypes = [vp, C.POINTER(PpsTuning)]
    L.pps_set_tuning.argtypes = [vp, C.POINTER(PpsTuning)]
    L.pps_batch_create.argtypes = [C.c_int, C.POINTER(PpsGrid), C.POINTER(PpsConfig), C.POINTER(vp)]
    L.pps_batch_destroy.argtypes = [vp]
    L.pps_batch_set.argtypes = [vp, C.c_int, vp, vp]
    L.pps_batch_get.argtypes = [vp, C.c_int, vp, C.POINTER(PpsStats)]
    L.pps_batch_field_device.argtypes = [vp, C.c_int, C.POINTER(vp), C.POINTER(vp)]
    L.pps_batch_autotune.argtypes = [vp]
    L.pps_batch_set_wait_limit.argtypes = [vp, C.c_double]
    L.pps_batch_tile.argtypes = [vp, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.pps_batch_solve.argtypes = [vp, C.POINTER(PpsBatchStats)]
    L.pps_unet_create.argtypes = [C.c_int, C.c_int, C.c_int, C.c_ulonglong, C.c_int, C.POINTER(vp)]
    L.pps_unet_destroy.argtypes = [vp]
    L.pps_unet_param_count.argtypes = [vp]
    L.pps_unet_get_params.argtypes = [vp, vp]
    L.pps_unet_set_params.argtypes = [vp, vp]
    L.pps_unet_forward.argtypes = [vp, C.c_int, C.c_int, C.c_int, vp, vp, C.c_int]
    L.pps_unet_gradients.argtypes = [vp, C.c_int, C.c_int, C.c_int, vp, vp, vp, C.POINTER(C.c_double)]
    L.pps_unet_train_step.argtypes = [vp, C.c_int, C.c_int, C.c_int, vp, vp, C.c_float, C.POINTER(C.c_double)]
    L.pps_restrict2.argtypes = [C.c_int, C.c_int, C.c_int, vp, vp]
    L.pps_set_learned.argtypes = [vp, vp, C.c_int, C.c_double, C.c_int]
    L.pps_set_learned_cycle.argtypes = [vp, C.c_int, C.c_int, C.c_double]
    L.pps_set_coarse_solver.argtypes = [vp, C.c_int]
    L.pps_write_solution.argtypes = [C.POINTER(PpsGrid), vp, C.c_int, C.c_char_p, vp]
    L.pps_unet_set_activation.argtypes = [vp, C.c_int]
    L.pps_prolong2.argtypes = [C.c_int, C.c_int, C.c_int, vp, vp]
    L.pps_status_string.restype = C.c_char_p
    L.pps_status_string.argtypes = [C.c_int]
    L.pps_last_error.restype = C.c_char_p
    for name in EXPORTED:
        fn = getattr(L, name)
        if name not in ("pps_status_string", "pps_last_error"):
            fn.restype = C.c_int
    _lib = L
    return L


def status_string(st: int) -> str:
    try:
        return load().pps_status_string(st).decode()
    except Exception:
        return f"status {st}"


def last_error() -> str:
    try:
        return load().pps_last_error().decode()
    except Exception:
        return ""


def device_count() -> int:
    return int(load().pps_device_count())


@dataclass
class BlockGrid:
    """Single-rank BlockGrid (blockGrid.hpp:15-36): npglobal counts boundary nodes."""
    npglobal: Sequence[int]
    ds: Sequence[float]
    origin: Sequence[float] = (0.0, 0.0, 0.0)
    bcs: Sequence[int] = (0, 0, 0, 0, 0, 0)

    @classmethod
    def cube(cls, m: int, bcs=(0, 0, 0, 0, 0, 0)):
        """Unit cube with m unknowns per axis (npglobal = m+2, ds = 1/(m+1))."""
        h = 1.0 / (m + 1)
        return cls(npglobal=(m + 2,) * 3, ds=(h,) * 3, bcs=tuple(bcs))

    @property
    def shape(self):
        n = self.npglobal
        return (n[2] + 2, n[1] + 2, n[0] + 2)

    def new_field(self) -> np.ndarray:
        return np.zeros(self.shape, np.float64)

    def unknowns(self):
        sl = []
        for d in (2, 1, 0):
            lo = 1 + (1 if self.bcs[2 * d] == 0 else 0)
            hi = self.npglobal[d] + 1 - (1 if self.bcs[2 * d + 1] == 0 else 0)
            sl.append(slice(lo, hi))
        return tuple(sl)

    def n_unknowns(self) -> int:
        return int(np.prod([s.stop - s.start for s in self.unknowns()]))

    def c(self) -> PpsGrid:
        g = PpsGrid()
        g.npglobal[:] = [int(v) for v in self.npglobal]
        g.ds[:] = [float(v) for v in self.ds]
        g.origin[:] = [float(v) for v in self.origin]
        g.bcs[:] = [int(v) for v in self.bcs]
        return g


@dataclass
class ChebyshevIteration:
    """Chebyshev-polynomial preconditioner (chebyshevIteration.hpp:15-156)."""
    degree: int = 11
    epsilon: float = 1e-4
    rescale_eig_min: float = 500.0
    rescale_eig_max: float = 1.0 - 1e-4

    @classmethod
    def alpaka_preset(cls):
        return cls(degree=24, epsilon=0.0, rescale_eig_min=100.0)


@dataclass
class NoneSolver:
    """Identity preconditioner (noneSolver.hpp:15-27)."""


@dataclass
class BiCGSTABPreconditioner:
    """An inner BiCGSTAB solve as the preconditioner: the BiCGSTAB class with
    isMainLoop false (BiCGSTAB.hpp:55-322, CPU/include/inputParam.hpp:30).  From X = 0
    it iterates on B / ||B|| until ||r|| < tolerance or max_iteration iterations,
    itself preconditioned by `preconditioner` (NoneSolver or ChebyshevIteration).
    Defaults: the CPU preset (tollPreconditionerSolver 1e4 x 1e-10, 150 iterations)."""
    tolerance: float = 1e4 * 1e-10
    max_iteration: int = 150
    preconditioner: object = field(default_factory=NoneSolver)

    kind = PREC_BICGSTAB


@dataclass
class BaseCGPreconditioner:
    """An inner CG solve as the preconditioner: the BaseCG class with isMainLoop
    false (baseCG.hpp:44-260, CPU/include/inputParam.hpp:29, there preconditioned by
    the Chebyshev iteration)."""
    tolerance: float = 1e4 * 1e-10
    max_iteration: int = 150
    preconditioner: object = field(default_factory=ChebyshevIteration)

    kind = PREC_CG


def _ptr(a: np.ndarray) -> int:
    if a.dtype != np.float64 or not a.flags.c_contiguous:
        raise TypeError("fields must be C-contiguous float64 arrays")
    return a.ctypes.data


class Solver:
    """One libpps solver handle (the reference's solver object)."""

    krylov = KRYLOV_BICGSTAB

    def __init__(self, grid: BlockGrid, preconditioner=None, tolerance: float = 1e-8, max_iteration: int = 1700,
                 form: str | int = "fp64", inner_tol: float = 3e-3, inner_maxit: int = 100000,
                 max_refinements: int = 12, check_every: int = 0, use_graph: bool = True, device: int = 0):
        self.grid = grid
        L = load()
        cfg = PpsConfig()
        L.pps_config_default(C.byref(cfg), PRESET_CPU)
        if preconditioner is None:
            preconditioner = self.default_preconditioner()
        cfg.krylov = self.krylov

        def chebyshev(p):
            cfg.cheb_degree = p.degree
            cfg.cheb_eps = p.epsilon
            cfg.rescale_min = p.rescale_eig_min
            cfg.rescale_max = p.rescale_eig_max

        if isinstance(preconditioner, NoneSolver):
            cfg.precond = PREC_NONE
        elif isinstance(preconditioner, (BiCGSTABPreconditioner, BaseCGPreconditioner)):
            cfg.precond = preconditioner.kind
            cfg.precond_tol = float(preconditioner.tolerance)
            cfg.precond_maxit = int(preconditioner.max_iteration)
            inner = preconditioner.preconditioner
            if isinstance(inner, ChebyshevIteration):
                cfg.precond_inner = PREC_CHEBYSHEV
                chebyshev(inner)
            elif isinstance(inner, NoneSolver) or inner is None:
                cfg.precond_inner = PREC_NONE
            else:
                raise TypeError("an inner solver is preconditioned by NoneSolver or ChebyshevIteration")
        else:
            cfg.precond = PREC_CHEBYSHEV
            chebyshev(preconditioner)
        cfg.tol = float(tolerance)
        cfg.maxit = int(max_iteration)
        cfg.form = FORMS[form] if isinstance(form, str) else int(form)
        cfg.inner_tol = float(inner_tol)
        cfg.inner_maxit = int(inner_maxit)
        cfg.max_refinements = int(max_refinements)
        cfg.check_every = int(check_every)
        cfg.use_graph = 1 if use_graph else 0
        cfg.device = int(device)
        self.config = cfg
        h = C.c_void_p()
        st = L.pps_create(C.byref(grid.c()), C.byref(cfg), C.byref(h))
        if st != OK:
            raise PpsError(st, "pps_create")
        self._h = h
        self._stats = PpsStats()
        self.last_status = OK

    @staticmethod
    def default_preconditioner():
        return ChebyshevIteration()

    def close(self):
        if getattr(self, "_h", None):
            load().pps_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # setProblem (iterativeSolverBase.hpp:51-55)
    def set_problem(self, x: np.ndarray, b: np.ndarray, problem: int = PROBLEM_REFERENCE_DEFAULT):
        st = load().pps_set_problem_builtin(self._h, problem, _ptr(x), _ptr(b))
        if st != OK:
            raise PpsError(st, "pps_set_problem_builtin")

    def set_neumann(self, face: int, values: np.ndarray):
        v = np.ascontiguousarray(values, np.float64)
        st = load().pps_set_neumann(self._h, face, v.ctypes.data)
        if st != OK:
            raise PpsError(st, "pps_set_neumann")

    # operator()(x, b, A) (BiCGSTAB.hpp:55-322)
    def __call__(self, x: np.ndarray, b: np.ndarray, raise_on_error: bool = True) -> int:
        assert x.shape == self.grid.shape and b.shape == self.grid.shape
        st = load().pps_solve(self._h, _ptr(x), _ptr(b), C.byref(self._stats))
        self.last_status = st
        if st < 0 and raise_on_error:
            raise PpsError(st, "pps_solve")
        return st

    solve = __call__

    def solve_device(self, x_ptr: int, b_ptr: int, raise_on_error: bool = True) -> int:
        st = load().pps_solve_device(self._h, C.c_void_p(x_ptr), C.c_void_p(b_ptr), C.byref(self._stats))
        self.last_status = st
        if st < 0 and raise_on_error:
            raise PpsError(st, "pps_solve_device")
        return st

    # getters (iterativeSolverBase.hpp:410-425)
    def stats(self) -> dict:
        return self._stats.as_dict()

    def get_num_iteration_final(self) -> int:
        return self._stats.iterations

    def get_error_from_iteration(self) -> float:
        return self._stats.err_iter

    def get_error_compute_operator(self) -> float:
        return self._stats.err_true

    def get_duration_solver(self) -> float:
        return self._stats.seconds_solve

    def history(self) -> np.ndarray:
        n = C.c_int(0)
        load().pps_get_history(self._h, None, 0, C.byref(n))
        out = np.zeros(max(n.value, 1))
        load().pps_get_history(self._h, out.ctypes.data, n.value, C.byref(n))
        return out[: n.value]

    def write_residual_history(self, path: str):
        st = load().pps_write_residual_history(self._h, path.encode())
        if st != OK:
            raise PpsError(st, "pps_write_residual_history")

    def set_learned(self, net, coarsen: int = 0, gain: float = 1.0,
                    flags: int = LEARNED_INITIAL_GUESS | LEARNED_PRECONDITIONER):
        """Attach a trained UNet (pps_set_learned); net=None detaches.  The solver keeps
        a reference so the network outlives its use."""
        st = load().pps_set_learned(self._h, net.handle if net is not None else None, int(coarsen), float(gain),
                                    int(flags))
        if st != OK:
            raise PpsError(st, "pps_set_learned")
        self._net = net

    def set_learned_cycle(self, fine_degree: int, coarse_degree: int = 0, ratio: float = 8.0):
        """Multigrid form of the learned preconditioner (pps_set_learned_cycle): a
        V-cycle with Chebyshev smoothers of these degrees on [lambda_max/ratio,
        lambda_max] of every level and the network on the coarsest; fine_degree 0
        keeps the two-grid cycle around the solver's own Chebyshev preconditioner."""
        st = load().pps_set_learned_cycle(self._h, int(fine_degree), int(coarse_degree), float(ratio))
        if st != OK:
            raise PpsError(st, "pps_set_learned_cycle")

    def set_coarse_solver(self, kind: int):
        """Coarsest-level solver of the learned V-cycle (pps_set_coarse_solver):
        COARSE_NETWORK (the attached U-Net), COARSE_ZERO (no correction there),
        COARSE_SMOOTH (the coarse smoother) or COARSE_EXACT (tensor-product
        eigen-solve), to measure what the network earns."""
        st = load().pps_set_coarse_solver(self._h, int(kind))
        if st != OK:
            raise PpsError(st, "pps_set_coarse_solver")

    def tuning_key(self) -> str:
        n = self.grid.npglobal
        return f"{n[0]}x{n[1]}x{n[2]}:form{self.config.form}"

    def autotune(self, cache: Optional[str] = None) -> dict:
        """Pick the tile shapes of the z-marching kernels for this grid (pps_autotune).
        With `cache`, a JSON table keyed by grid and form is read first and updated
        after a new measurement, so a grid is tuned once per machine."""
        import json
        key = self.tuning_key()
        table = {}
        if cache and os.path.exists(cache):
            with open(cache) as f:
                table = json.load(f)
            if key in table:
                self.set_tuning(table[key])
                return table[key]
        t = PpsTuning()
        st = load().pps_autotune(self._h, C.byref(t))
        if st != OK:
            raise PpsError(st, "pps_autotune")
        d = t.as_dict()
        if cache:
            table[key] = d
            tmp = cache + ".tmp"
            with open(tmp, "w") as f:
                json.dump(table, f, indent=1, sort_keys=True)
            os.replace(tmp, cache)
        return d

    def tuning(self) -> dict:
        t = PpsTuning()
        load().pps_get_tuning(self._h, C.byref(t))
        return t.as_dict()

    def set_tuning(self, d: dict):
        st = load().pps_set_tuning(self._h, C.byref(PpsTuning.from_dict(d)))
        if st != OK:
            raise PpsError(st, "pps_set_tuning")

    def apply_operator(self, u: np.ndarray, out: Optional[np.ndarray] = None) -> np.ndarray:
        out = np.zeros_like(u) if out is None else out
        st = load().pps_apply_operator(self._h, _ptr(np.ascontiguousarray(u)), _ptr(out))
        if st != OK:
            raise PpsError(st, "pps_apply_operator")
        return out

    def apply_preconditioner(self, B: np.ndarray, X: Optional[np.ndarray] = None) -> np.ndarray:
        X = np.zeros_like(B) if X is None else X
        st = load().pps_apply_preconditioner(self._h, _ptr(np.ascontiguousarray(B)), _ptr(X))
        if st != OK:
            raise PpsError(st, "pps_apply_preconditioner")
        return X


class BiCGSTAB(Solver):
    """Right-preconditioned BiCGSTAB main loop (BiCGSTAB.hpp:14-335)."""
    krylov = KRYLOV_BICGSTAB


class BaseCG(Solver):
    """Preconditioned CG main loop (baseCG.hpp:14-269)."""
    krylov = KRYLOV_CG


class FlexibleCG(Solver):
    """Flexible CG: BaseCG's loop with a Polak-Ribiere beta, so the preconditioner may
    change between applications (no reference counterpart; FP64 and MIXED forms)."""
    krylov = KRYLOV_FCG


class ChebyshevSolver(Solver):
    """The Chebyshev iteration as the main solver: ChebyshevIteration with isMainLoop
    true (chebyshevIteration.hpp:48-140, chebyshevIterationAlpaka.hpp:320-587).  The
    `preconditioner` argument carries the polynomial's parameters; by default degree
    24 with the eigenvalue bounds unscaled (rescale 1, epsilon 0), as the reference
    asks for this use (ALP/include/inputParam.hpp:21).  One application of the
    polynomial to the adjusted b overwrites x; get_error_compute_operator() is the
    absolute ||b - A x||."""
    krylov = KRYLOV_CHEBYSHEV

    @staticmethod
    def default_preconditioner():
        return ChebyshevIteration(degree=24, epsilon=0.0, rescale_eig_min=1.0, rescale_eig_max=1.0)


class Batch:
    """Many independent Dirichlet grids solved together (pps_batch_*), MIXED form.
    method "vcycle": flexible CG with a multigrid V-cycle per problem, the whole solve
    one persistent launch replayed as a CUDA graph (cubes, edge c * 2^k, c <= 32);
    method "bicgstab": the reference's BiCGSTAB + Chebyshev per problem, one launch
    per phase over all problems, the inner iteration replayed as a CUDA graph."""

    def __init__(self, grids: Sequence[BlockGrid], preconditioner: Optional[ChebyshevIteration] = None,
                 tolerance: float = 1e-10, inner_tol: float = 3e-3, inner_maxit: int = 5000,
                 max_refinements: int = 12, check_every: int = 8, use_graph: bool = True, device: int = 0,
                 method: str = "bicgstab"):
        L = load()
        self.grids = list(grids)
        prec = preconditioner or ChebyshevIteration()
        cfg = PpsConfig()
        L.pps_config_default(C.byref(cfg), PRESET_CPU)
        cfg.cheb_degree, cfg.cheb_eps = prec.degree, prec.epsilon
        cfg.rescale_min, cfg.rescale_max = prec.rescale_eig_min, prec.rescale_eig_max
        cfg.form = FORM_MIXED
        cfg.tol, cfg.inner_tol, cfg.inner_maxit = float(tolerance), float(inner_tol), int(inner_maxit)
        cfg.max_refinements, cfg.check_every = int(max_refinements), int(check_every)
        cfg.use_graph, cfg.device = (1 if use_graph else 0), int(device)
        if method not in ("bicgstab", "vcycle"):
            raise ValueError("method: 'bicgstab' or 'vcycle'")
        self.method = method
        if method == "vcycle":
            cfg.krylov = KRYLOV_FCG
        arr = (PpsGrid * len(self.grids))(*[g.c() for g in self.grids])
        h = C.c_void_p()
        st = L.pps_batch_create(len(self.grids), arr, C.byref(cfg), C.byref(h))
        if st != OK:
            raise PpsError(st, "pps_batch_create")
        self._h = h
        self._stats = PpsBatchStats()

    def close(self):
        if getattr(self, "_h", None):
            load().pps_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set(self, p: int, x: np.ndarray, b: np.ndarray):
        st = load().pps_batch_set(self._h, p, _ptr(x), _ptr(b))
        if st != OK:
            raise PpsError(st, "pps_batch_set")

    def get(self, p: int, x: Optional[np.ndarray] = None):
        x = self.grids[p].new_field() if x is None else x
        ps = PpsStats()
        st = load().pps_batch_get(self._h, p, _ptr(x), C.byref(ps))
        if st != OK:
            raise PpsError(st, "pps_batch_get")
        return x, ps.as_dict()

    def field_device(self, p: int):
        xd, bd = C.c_void_p(), C.c_void_p()
        load().pps_batch_field_device(self._h, p, C.byref(xd), C.byref(bd))
        return xd.value, bd.value

    def autotune(self):
        st = load().pps_batch_autotune(self._h)
        if st != OK:
            raise PpsError(st, "pps_batch_autotune")
        out = []
        for p in range(len(self.grids)):
            cx, kc = C.c_int(), C.c_int()
            load().pps_batch_tile(self._h, p, C.byref(cx), C.byref(kc))
            out.append((cx.value, kc.value))
        return out

    def set_wait_limit(self, seconds: float):
        """Persistent batches: the longest a grid-barrier wait may take before the
        solve stops with TIMEOUT (pps_batch_set_wait_limit)."""
        st = load().pps_batch_set_wait_limit(self._h, float(seconds))
        if st != OK:
            raise PpsError(st, "pps_batch_set_wait_limit")

    def solve(self, raise_on_error: bool = True) -> int:
        st = load().pps_batch_solve(self._h, C.byref(self._stats))
        if st < 0 and raise_on_error:
            raise PpsError(st, "pps_batch_solve")
        return st

    def stats(self) -> dict:
        return self._stats.as_dict()


class UNet:
    """The learned preconditioner's 3-D U-Net (pps_unet_*): 3 levels, c1/c2/c3
    channels, 3x3x3 kernels, BF16 weights/activations, FP32 accumulation, trained by
    the library's own forward/backward kernels.  Arrays are device pointers of dense
    FP32 [nz][ny][nx] fields; extents must be multiples of 4."""

    def __init__(self, channels=(16, 32, 64), seed: int = 0, device: int = 0, linear: bool = False):
        h = C.c_void_p()
        st = load().pps_unet_create(channels[0], channels[1], channels[2], seed, device, C.byref(h))
        if st != OK:
            raise PpsError(st, "pps_unet_create")
        self._h = h
        self.channels = tuple(channels)
        self.linear = bool(linear)
        load().pps_unet_set_activation(h, int(self.linear))

    def close(self):
        if getattr(self, "_h", None):
            load().pps_unet_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def param_count(self) -> int:
        return int(load().pps_unet_param_count(self._h))

    def get_params(self) -> np.ndarray:
        out = np.zeros(self.param_count(), np.float32)
        st = load().pps_unet_get_params(self._h, out.ctypes.data)
        if st != OK:
            raise PpsError(st, "pps_unet_get_params")
        return out

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == self.param_count()
        st = load().pps_unet_set_params(self._h, p.ctypes.data)
        if st != OK:
            raise PpsError(st, "pps_unet_set_params")

    def forward(self, shape, in_ptr: int, out_ptr: int, normalize: bool = True):
        nz, ny, nx = shape
        st = load().pps_unet_forward(self._h, nx, ny, nz, C.c_void_p(in_ptr), C.c_void_p(out_ptr), int(normalize))
        if st != OK:
            raise PpsError(st, "pps_unet_forward")

    def gradients(self, shape, in_ptr: int, target_ptr: int):
        nz, ny, nx = shape
        g = np.zeros(self.param_count(), np.float32)
        loss = C.c_double(0)
        st = load().pps_unet_gradients(self._h, nx, ny, nz, C.c_void_p(in_ptr), C.c_void_p(target_ptr),
                                       g.ctypes.data, C.byref(loss))
        if st != OK:
            raise PpsError(st, "pps_unet_gradients")
        return loss.value, g

    def train_step(self, shape, in_ptr: int, target_ptr: int, lr: float) -> float:
        nz, ny, nx = shape
        loss = C.c_double(0)
        st = load().pps_unet_train_step(self._h, nx, ny, nz, C.c_void_p(in_ptr), C.c_void_p(target_ptr),
                                        C.c_float(lr), C.byref(loss))
        if st != OK:
            raise PpsError(st, "pps_unet_train_step")
        return loss.value

    def save(self, path: str):
        np.savez(path, params=self.get_params(), channels=np.array(self.channels), linear=np.array(int(self.linear)))

    @classmethod
    def load_file(cls, path: str, device: int = 0):
        d = np.load(path)
        net = cls(tuple(int(c) for c in d["channels"]), device=device, linear=bool(int(d["linear"])) if "linear" in d else False)
        net.set_params(d["params"])
        return net


def restrict2(coarse_shape, fine_ptr: int, coarse_ptr: int):
    nz, ny, nx = coarse_shape
    st = load().pps_restrict2(nx, ny, nz, C.c_void_p(fine_ptr), C.c_void_p(coarse_ptr))
    if st != OK:
        raise PpsError(st, "pps_restrict2")


def prolong2(coarse_shape, coarse_ptr: int, fine_ptr: int):
    nz, ny, nx = coarse_shape
    st = load().pps_prolong2(nx, ny, nz, C.c_void_p(coarse_ptr), C.c_void_p(fine_ptr))
    if st != OK:
        raise PpsError(st, "pps_prolong2")


def apply_operator_noalloc(grid: BlockGrid, u_ptr: int, out_ptr: int, energy_ptr: int, stream: int = 0) -> int:
    """pps_apply_operator_noalloc on device pointers: out = A u at the unknowns and
    energy = sum u*(A u), with no device allocation (see include/pps.h)."""
    return int(load().pps_apply_operator_noalloc(C.byref(grid.c()), C.c_void_p(u_ptr), C.c_void_p(out_ptr),
                                                 C.c_void_p(energy_ptr), C.c_void_p(stream or None)))


def write_solution(grid: BlockGrid, x, path: str, rank: int = 0, stream: int = 0):
    """solution.dat (pps_write_solution): the rank's guard-padded field at byte offset
    rank * G * 8 of `path`.  x: a float64 numpy field, or a device pointer (int)."""
    if isinstance(x, np.ndarray):
        if x.shape != grid.shape or x.dtype != np.float64 or not x.flags.c_contiguous:
            raise ValueError("x must be a C-contiguous float64 field of the grid's shape")
        ptr = x.ctypes.data
    else:
        ptr = int(x)
    st = load().pps_write_solution(C.byref(grid.c()), ptr, int(rank), path.encode(), stream or None)
    if st != OK:
        raise PpsError(st, "pps_write_solution")


def check_solution(grid: BlockGrid, x: np.ndarray, exact: np.ndarray):
    """checkSolutionLocalGlobal (iterativeSolverBase.hpp:283-408) at one rank:
    (block average |x-u|, point max |x-u|) over the data nodes."""
    d = tuple(slice(1, n + 1) for n in (grid.npglobal[2], grid.npglobal[1], grid.npglobal[0]))
    err = np.abs(x[d] - exact[d])
    return float(err.sum() / err.size), float(err.max())
