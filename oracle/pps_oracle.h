/*
 * pps_oracle.h -- CPU restatement of the reference solve loop (TEST INFRASTRUCTURE).
 *
 * This is the oracle: tests, the smoke check and the CPU-baseline leg of bench.py
 * call it to check results.  The product (libpps) never links or calls it.
 *
 * It restates, in the reference's exact floating-point expression order, the
 * single-rank path of solverPoissonMPI_CPU:
 *   BlockGrid index limits / eigenvalue bounds   include/blockGrid.hpp:184-222, 301-340
 *   MatrixFreeOperatorA                          include/matrixFreeOperatorA.hpp:22-39
 *   ChebyshevIteration (preconditioner mode)     include/chebyshevIteration.hpp:19-34, 48-140
 *   ChebyshevIteration (main solver, isMainLoop)  include/chebyshevIteration.hpp:48-140
 *   BiCGSTAB main loop                           include/BiCGSTAB.hpp:55-322
 *   BiCGSTAB as a preconditioner (isMainLoop false, communicationOFF)
 *                                                include/BiCGSTAB.hpp:55-322, inputParam.hpp:30
 *   BaseCG main loop                             include/baseCG.hpp:44-260
 *   BaseCG as a preconditioner (isMainLoop false, communicationOFF)
 *                                                include/baseCG.hpp:44-260, inputParam.hpp:29
 *   NoneSolver                                   include/noneSolver.hpp:15-27
 *   normalisation / true residual / BC handling  include/iterativeSolverBase.hpp:62-234, 236-280, 429-534
 *
 * Parity is pinned: tests/test_oracle.py checks this port bit-for-bit against the
 * reference's own CPU solver compiled from its headers (oracle/Makefile -> oracle/_ref)
 * and against the committed fixtures in tests/golden/ that the reference produced.
 *
 * Arrays are guard-padded fields of (n0+2)(n1+2)(n2+2) doubles, x fastest, where
 * n_d = npglobal_d counts the boundary nodes (iterativeSolverBase.hpp:34-35).
 * Build with -ffp-contract=off so that no multiply-add is fused (the reference is
 * built for x86-64 without FMA, so every product and sum is rounded separately).
 */
#ifndef PPS_ORACLE_H
#define PPS_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int np[3];          /* npglobal per axis, boundary nodes included            */
    double ds[3];       /* grid spacing                                           */
    double origin[3];   /* coordinate of data index 1                             */
    int bcs[6];         /* x- x+ y- y+ z- z+ : 0 Dirichlet, 1 Neumann             */
} ora_grid;

enum { ORA_BICGSTAB = 0, ORA_CG = 1, ORA_CHEBYSHEV_MAIN = 2 };
enum { ORA_PREC_NONE = 0, ORA_PREC_CHEBYSHEV = 1, ORA_PREC_BICGSTAB = 2, ORA_PREC_CG = 3 };

typedef struct {
    int krylov;           /* ORA_BICGSTAB / ORA_CG / ORA_CHEBYSHEV_MAIN              */
    int precond;          /* ORA_PREC_NONE / _CHEBYSHEV / _BICGSTAB / _CG           */
    int cheb_degree;      /* Chebyshev maxIteration (chebyshevMax)                  */
    double cheb_eps;      /* epsilon                                                */
    double rescale_min;   /* rescaleEigMin                                          */
    double rescale_max;   /* rescaleEigMax                                          */
    double tol;           /* tolerance * tollScalingFactor                          */
    int maxit;            /* maxIteration of the Krylov loop                        */
    int threads;          /* OpenMP threads for element-wise passes (sums stay serial) */
    /* ORA_PREC_BICGSTAB / ORA_PREC_CG: the inner solver object's toll_, maxIteration
     * and its own preconditioner (ORA_PREC_NONE or ORA_PREC_CHEBYSHEV with the fields
     * above). */
    double prec_tol;
    int prec_maxit;
    int prec_inner;
} ora_config;

typedef struct {
    int iterations;       /* getNumIterationFinal                                   */
    double err_iter;      /* getErrorFromIteration (recursive, normalised)          */
    double err_true;      /* getErrorComputeOperator (true, normalised)             */
    double norm_b;        /* ||b_adj|| over the unknowns                            */
    double seconds_loop;  /* wall time of the Krylov loop (getDurationSolver)       */
    double seconds_total; /* wall time of the whole call                            */
    int prec_iterations;  /* inner solver: iterations, summed over applications      */
} ora_stats;

/* Full solve in place on x (in/out) and b (scaled and unscaled in place, as the
 * reference does).  ORA_CHEBYSHEV_MAIN applies the polynomial of degree cheb_degree
 * (always Chebyshev, `precond` is not used), leaves b untouched and reports the
 * absolute true residual in err_iter and err_true.  neumann[f] (f = 2*dir + side)
 * holds du/d(dir) at the data nodes of Neumann face f, laid out with the lower
 * remaining axis fastest; NULL entries mean zero flux.  history needs maxit+1
 * doubles (may be NULL).
 * Returns 0, or -1 on an invalid argument. */
int ora_solve(const ora_grid* g, const ora_config* c, double* x, double* b,
              const double* const* neumann, double* history, ora_stats* st);

/* ora_solve for the BiCGSTAB main solver, also writing wall-clock stamps (seconds
 * on CLOCK_MONOTONIC): stamps[0] when the call starts, stamps[i] when iteration i
 * ends (1 <= i <= iterations), stamps[iterations + 1] when the call returns.
 * stamps needs maxit+2 doubles; history is required.  The benchmark's reference
 * arm times one complete solve in chunks with them. */
int ora_solve_stamped(const ora_grid* g, const ora_config* c, double* x, double* b,
                      const double* const* neumann, double* history, ora_stats* st, double* stamps);

/* Building blocks, exposed for kernel-level parity tests. */
void ora_eigen_bounds(const ora_grid* g, double out[2]);                 /* eigenValuesGlobal_ */
void ora_cheb_params(const ora_grid* g, const ora_config* c, double out[3]); /* theta, delta, sigma */
/* out[p] = A(u)[p] at the unknowns; other entries untouched. */
void ora_apply_A(const ora_grid* g, const double* u, double* out);
/* One preconditioner application X = Cheb(B) (chebyshevIteration.hpp:48-140, not main loop). */
void ora_cheb_apply(const ora_grid* g, const ora_config* c, double* B, double* X);
/* Sequential dot over the unknowns in k,j,i order. */
double ora_dot(const ora_grid* g, const double* a, const double* b);
/* Problem set-up from the built-in manufactured solutions (setProblem,
 * iterativeSolverBase.hpp:51-55, 537-603): problem 0 = the reference default
 * u = sin x + cos y + 3 sin z + x^2 y z + x^2 + 10 with f = lap u; problem 1 = the
 * sine product u = sin(pi x) sin(pi y) sin(pi z) with f = -3 pi^2 u.
 * Also fills neumann face arrays (if non-NULL pointers are given) with du/d(dir). */
int ora_set_problem(const ora_grid* g, int problem, double* x, double* b, double* const* neumann);
/* Exact solution at every data node (for error checks); ghosts untouched. */
int ora_exact_solution(const ora_grid* g, int problem, double* u);

#ifdef __cplusplus
}
#endif
#endif
