/*
 * Project-written driver that compiles the reference's OWN CPU solver headers
 * (solverPoissonMPI_CPU/include, read where they lie; nothing is copied) into
 * oracle/_ref/libppsref.so for the test oracle.  It replaces the reference's
 * src/main.cpp (CPU/src/main.cpp:19-134) at one rank: build a BlockGrid, a
 * CommunicatorMPI, the problem plugin and the operator, construct the solver
 * type that include/inputParam.hpp:24-38 composes, and call operator()(x, b, A).
 *
 * Template arguments are compile-time in the reference, so a table of
 * instantiations covers the Chebyshev degrees and iteration caps the tests use.
 * The only change around the reference classes is in RefSolver below: the
 * residual-history array is re-allocated one entry longer, because the reference
 * writes history[maxIteration] when it stops at the cap (BiCGSTAB.hpp:275-281,
 * iterativeSolverBase.hpp:43), one past its allocation.
 */
#include <algorithm>
#include <array>
#include <chrono>
#include <iostream>
#include <sstream>

#include "ref_setup.hpp"

#include "blockGrid.hpp"
#include "communicationMPI.hpp"
#include "matrixFreeOperatorA.hpp"
#include "solvers.hpp"

namespace {

using NoneP = NoneSolver<3, T_data, 10000, 150>;
template <int DEG>
using ChebP = ChebyshevIteration<3, T_data, 10000, DEG, false, false, NoneP>;

template <class Base, int MAXIT>
struct RefSolver : Base {
    RefSolver(const BlockGrid<3, T_data>& g, const ExactSolutionAndBCs<3, T_data>& e, CommunicatorMPI<3, T_data>& c)
        : Base(g, e, c)
    {
        delete[] this->errorFromIterationHistory_;
        this->errorFromIterationHistory_ = new T_data[MAXIT + 1];
        for (int i = 0; i <= MAXIT; i++) this->errorFromIterationHistory_[i] = -1.0;
    }
    const T_data* history() const { return this->errorFromIterationHistory_; }
};

struct RefArgs {
    int np[3];
    double ds[3], origin[3];
    int bcs[6];
    double tol, eps, rescale_min, rescale_max;
    int problem;
};

struct RefOut {
    int iterations;
    double err_iter, err_true, seconds_loop, seconds_call;
};

template <class S, int MAXIT>
int run(const RefArgs* a, double* x, double* b, double* hist, RefOut* out)
{
    tollScalingFactor = a->tol;    /* with tolerance == 1: toll_ = 1.0 * tol */
    epsilon = a->eps;
    rescaleEigMin = a->rescale_min;
    rescaleEigMax = a->rescale_max;
    ppsOracleProblem = a->problem;
    for (int q = 0; q < 3; q++) {
        ppsOracleNp[q] = a->np[q];
        ppsOracleDs[q] = a->ds[q];
        ppsOracleOrigin[q] = a->origin[q];
    }

    const std::array<int, 3> nranks = {1, 1, 1};
    const std::array<int, 3> npg = {a->np[0], a->np[1], a->np[2]};
    const std::array<T_data, 3> ds = {a->ds[0], a->ds[1], a->ds[2]};
    const std::array<T_data, 3> origin = {a->origin[0], a->origin[1], a->origin[2]};
    const std::array<int, 3> guards = {1, 1, 1};
    const std::array<int, 6> bcs = {a->bcs[0], a->bcs[1], a->bcs[2], a->bcs[3], a->bcs[4], a->bcs[5]};
    const std::array<T_data, 6> bcsValue = {0, 0, 0, 0, 0, 0};

    std::ostringstream sink;
    std::streambuf* saved = std::cout.rdbuf(sink.rdbuf());   /* the reference prints progress */
    {
        BlockGrid<3, T_data> grid(nranks, 0, npg, ds, origin, guards, bcs, bcsValue);
        CommunicatorMPI<3, T_data> comm(grid);
        ExactSolutionAndBCs<3, T_data> exact;
        MatrixFreeOperatorA<3, T_data> opA(grid);
        auto* solver = new RefSolver<S, MAXIT>(grid, exact, comm);
        const auto t0 = std::chrono::high_resolution_clock::now();
        (*solver)(x, b, opA);
        const auto t1 = std::chrono::high_resolution_clock::now();
        out->iterations = solver->getNumIterationFinal();
        out->err_iter = solver->getErrorFromIteration();
        out->err_true = solver->getErrorComputeOperator();
        out->seconds_loop = out->iterations > 0 ? solver->getDurationSolver().count() : 0.0;
        out->seconds_call = std::chrono::duration<double>(t1 - t0).count();
        if (hist)
            for (int i = 0; i <= out->iterations && i <= MAXIT; i++) hist[i] = solver->history()[i];
        delete solver;
    }
    std::cout.rdbuf(saved);
    return 0;
}

typedef int (*run_fn)(const RefArgs*, double*, double*, double*, RefOut*);

/* (krylov, precond, degree, maxit) as in the oracle's enums; for precond 2 or 3 (a
 * BiCGSTAB or BaseCG object as the preconditioner, isMainLoop false) also its
 * maxIteration (pmaxit), its
 * tolerance template argument (pratio: toll_ = pratio * tollScalingFactor, i.e.
 * pratio times the main tolerance) and its own preconditioner (pinner 0 none, 1
 * Chebyshev of `degree`).  krylov 2 is ChebyshevIteration as the main solver. */
struct Entry {
    int krylov, precond, degree, maxit;
    int pmaxit, pratio, pinner;
    run_fn fn;
};

template <int MAXIT, class P>
using BiCG = BiCGSTAB<3, T_data, 1, MAXIT, true, true, P>;
template <int MAXIT, class P>
using CG = BaseCG<3, T_data, 1, MAXIT, true, true, P>;
/* inputParam.hpp:30: BiCGSTAB<..., isbiCGMainLoop2 (false), communicationOFF, T_NoneSolver> */
template <int PRATIO, int PMAXIT, class P>
using BiCGPrec = BiCGSTAB<3, T_data, PRATIO, PMAXIT, false, false, P>;
/* inputParam.hpp:29: BaseCG<..., isbiCGMainLoop2 (false), communicationOFF, T_Preconditioner2> */
template <int PRATIO, int PMAXIT, class P>
using CGPrec = BaseCG<3, T_data, PRATIO, PMAXIT, false, false, P>;
/* ALP/include/inputParam.hpp:37: the Chebyshev iteration as the main solver */
template <int DEG>
using ChebMain = ChebyshevIteration<3, T_data, 10000, DEG, true, true, NoneP>;

#define BICG_CHEB(DEG, MAXIT) {0, 1, DEG, MAXIT, 0, 0, 0, &run<BiCG<MAXIT, ChebP<DEG>>, MAXIT>}
#define BICG_NONE(MAXIT) {0, 0, 0, MAXIT, 0, 0, 0, &run<BiCG<MAXIT, NoneP>, MAXIT>}
#define CG_CHEB(DEG, MAXIT) {1, 1, DEG, MAXIT, 0, 0, 0, &run<CG<MAXIT, ChebP<DEG>>, MAXIT>}
#define CG_NONE(MAXIT) {1, 0, 0, MAXIT, 0, 0, 0, &run<CG<MAXIT, NoneP>, MAXIT>}
#define BICG_BICG(MAXIT, PR, PM) {0, 2, 0, MAXIT, PM, PR, 0, &run<BiCG<MAXIT, BiCGPrec<PR, PM, NoneP>>, MAXIT>}
#define BICG_BICG_CHEB(MAXIT, PR, PM, DEG) \
    {0, 2, DEG, MAXIT, PM, PR, 1, &run<BiCG<MAXIT, BiCGPrec<PR, PM, ChebP<DEG>>>, MAXIT>}
#define CG_BICG(MAXIT, PR, PM) {1, 2, 0, MAXIT, PM, PR, 0, &run<CG<MAXIT, BiCGPrec<PR, PM, NoneP>>, MAXIT>}
#define BICG_CGP_CHEB(MAXIT, PR, PM, DEG) \
    {0, 3, DEG, MAXIT, PM, PR, 1, &run<BiCG<MAXIT, CGPrec<PR, PM, ChebP<DEG>>>, MAXIT>}
#define BICG_CGP(MAXIT, PR, PM) {0, 3, 0, MAXIT, PM, PR, 0, &run<BiCG<MAXIT, CGPrec<PR, PM, NoneP>>, MAXIT>}
#define CHEB_MAIN(DEG) {2, 1, DEG, DEG, 0, 0, 0, &run<ChebMain<DEG>, DEG>}

const Entry kTable[] = {
    BICG_CHEB(1, 1700), BICG_CHEB(2, 1700), BICG_CHEB(3, 1700), BICG_CHEB(4, 1700),
    BICG_CHEB(5, 1700), BICG_CHEB(11, 1700), BICG_CHEB(24, 1700),
    BICG_CHEB(11, 3), BICG_CHEB(24, 3), BICG_CHEB(11, 20000), BICG_CHEB(24, 1000),
    BICG_NONE(1700), BICG_NONE(20000),
    CG_CHEB(2, 1700), CG_CHEB(11, 1700), CG_CHEB(11, 20000), CG_NONE(1700), CG_NONE(20000),
    BICG_BICG(1700, 100, 150), BICG_BICG(1700, 100, 3), BICG_BICG(1700, 100000000, 500),
    BICG_BICG_CHEB(1700, 100, 150, 11), CG_BICG(1700, 100, 150),
    BICG_CGP_CHEB(1700, 100, 150, 11), BICG_CGP(1700, 100, 150), BICG_CGP_CHEB(1700, 100, 3, 11),
    CHEB_MAIN(1), CHEB_MAIN(2), CHEB_MAIN(3), CHEB_MAIN(4), CHEB_MAIN(11), CHEB_MAIN(24), CHEB_MAIN(80),
};

}  // namespace

extern "C" {

/* Solve in place with the reference's classes.  `problem` selects what the
 * plugin evaluates for Neumann data (2: the tabulated `faces`).  pmaxit, pratio and
 * pinner select the inner BiCGSTAB of precond 2 (see Entry).  Returns 0, or -2 when
 * the combination was not instantiated. */
int ref_solve2(int krylov, int precond, int degree, int maxit, int pmaxit, int pratio, int pinner, const int* np,
               const double* ds, const double* origin, const int* bcs, double tol, double eps, double rescale_min,
               double rescale_max, int problem, double* x, double* b, double* hist, int* iterations,
               double* errs /* err_iter, err_true, seconds_loop, seconds_call */, const double* const* faces)
{
    for (int f = 0; f < 6; f++) ppsOracleFaces[f] = faces ? faces[f] : nullptr;
    RefArgs a;
    for (int d = 0; d < 3; d++) { a.np[d] = np[d]; a.ds[d] = ds[d]; a.origin[d] = origin[d]; }
    for (int f = 0; f < 6; f++) a.bcs[f] = bcs[f];
    a.tol = tol; a.eps = eps; a.rescale_min = rescale_min; a.rescale_max = rescale_max; a.problem = problem;
    for (const Entry& e : kTable) {
        bool match;
        if (krylov == 2) {
            match = e.krylov == 2 && e.degree == degree;
        } else {
            const bool nested = precond == 2 || precond == 3;
            match = e.krylov == krylov && e.precond == precond && e.maxit == maxit &&
                    (precond == 0 || (nested && pinner == 0) || e.degree == degree);
            if (nested) match = match && e.pmaxit == pmaxit && e.pratio == pratio && e.pinner == pinner;
        }
        if (match) {
            RefOut o;
            /* the Chebyshev main loop keeps no history; its degree may exceed the caller's maxit */
            int rc = e.fn(&a, x, b, krylov == 2 ? nullptr : hist, &o);
            *iterations = o.iterations;
            errs[0] = o.err_iter; errs[1] = o.err_true; errs[2] = o.seconds_loop; errs[3] = o.seconds_call;
            return rc;
        }
    }
    return -2;
}

int ref_solve(int krylov, int precond, int degree, int maxit, const int* np, const double* ds,
              const double* origin, const int* bcs, double tol, double eps, double rescale_min,
              double rescale_max, int problem, double* x, double* b, double* hist, int* iterations,
              double* errs, const double* const* faces)
{
    return ref_solve2(krylov, precond, degree, maxit, 0, 0, 0, np, ds, origin, bcs, tol, eps, rescale_min,
                      rescale_max, problem, x, b, hist, iterations, errs, faces);
}

/* The instantiated (krylov, precond, degree, maxit) combinations, 4 ints each. */
int ref_table(int* out, int cap)
{
    const int n = (int)(sizeof(kTable) / sizeof(kTable[0]));
    for (int i = 0; i < n && i < cap; i++) {
        out[4 * i] = kTable[i].krylov; out[4 * i + 1] = kTable[i].precond;
        out[4 * i + 2] = kTable[i].degree; out[4 * i + 3] = kTable[i].maxit;
    }
    return n;
}

/* setProblem through the reference's own IterativeSolverBase
 * (iterativeSolverBase.hpp:51-55), for checking the built-in problem set-up. */
int ref_set_problem(const int* np, const double* ds, const double* origin, const int* bcs, int problem,
                    double* x, double* b)
{
    ppsOracleProblem = problem;
    const std::array<int, 3> nranks = {1, 1, 1};
    const std::array<int, 3> npg = {np[0], np[1], np[2]};
    const std::array<T_data, 3> d = {ds[0], ds[1], ds[2]};
    const std::array<T_data, 3> o = {origin[0], origin[1], origin[2]};
    const std::array<int, 3> guards = {1, 1, 1};
    const std::array<int, 6> bc = {bcs[0], bcs[1], bcs[2], bcs[3], bcs[4], bcs[5]};
    const std::array<T_data, 6> bcsValue = {0, 0, 0, 0, 0, 0};
    BlockGrid<3, T_data> grid(nranks, 0, npg, d, o, guards, bc, bcsValue);
    CommunicatorMPI<3, T_data> comm(grid);
    ExactSolutionAndBCs<3, T_data> exact;
    NoneP s(grid, exact, comm);
    s.setProblem(x, b);
    return 0;
}

}  // extern "C"
