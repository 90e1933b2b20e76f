// pps_solver.hpp -- header-only C++ shim that puts libpps behind the reference's
// solver-class protocol, so the reference driver (solverPoissonMPI_CPU/src/main.cpp)
// switches to the GPU by changing only its T_Solver alias (include/inputParam.hpp:33):
//
//   #define PPS_USE_REFERENCE_SETUP        // take epsilon/rescaleEig*/tollScalingFactor
//   #include "pps_solver.hpp"              //   from the reference's solverSetup.hpp
//   using T_Preconditioner2 = pps::ChebyshevIteration<DIM,T_data,tollPreconditionerSolver,
//                                                     chebyshevMax,false,false,T_NoneSolver>;
//   using T_Solver = pps::BiCGSTAB<DIM,T_data,tollMainSolver,iterMaxMainSolver,true,true,
//                                  T_Preconditioner2>;
//
// Constructor, setProblem, operator()(x, b, A), the getters and
// checkSolutionLocalGlobal keep the reference's signatures and meaning
// (BiCGSTAB.hpp:18-55, iterativeSolverBase.hpp:51-55, 283-425).  The grid must be a
// single rank (nranks 1x1x1): libpps runs one domain on one GPU.
//
// The other compositions of inputParam.hpp read the same way:
//   pps::BiCGSTAB<..., true, true, pps::BiCGSTAB<..., false, false, T_NoneSolver>>
//       an inner BiCGSTAB solve as the preconditioner (CPU/include/inputParam.hpp:30);
//   pps::BiCGSTAB<..., true, true, pps::BaseCG<..., false, false, T_Preconditioner2>>
//       an inner CG solve preconditioned by Chebyshev (inputParam.hpp:29);
//   pps::ChebyshevIteration<..., chebyshevMax, true, true, T_NoneSolver>
//       the Chebyshev iteration as the main solver (ALP/include/inputParam.hpp:37).
#ifndef PPS_SOLVER_HPP
#define PPS_SOLVER_HPP

#include <array>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <type_traits>

#include "pps.h"

namespace pps {

// The form every shim solver is created with (PPS_FORM_FP64 unless changed).
inline int& default_form()
{
    static int form = PPS_FORM_FP64;
    return form;
}

struct ChebyshevParams {
    double epsilon = 1e-4;
    double rescale_min = 500.0;
    double rescale_max = 1.0 - 1e-4;
    double toll_scaling = 1e-10;
};

inline ChebyshevParams setup_params()
{
    ChebyshevParams p;
#ifdef PPS_USE_REFERENCE_SETUP
    p.epsilon = epsilon;
    p.rescale_min = rescaleEigMin;
    p.rescale_max = rescaleEigMax;
    p.toll_scaling = tollScalingFactor;
#endif
    return p;
}

// Preconditioner tags: they carry the reference's template arguments only.
template <int DIM, typename T_data, int tolerance, int maxIteration>
struct NoneSolver {
    static constexpr int precond = PPS_PREC_NONE;
    static constexpr int degree = 0;
};

template <int DIM, typename T_data, int tolerance, int maxIteration, bool isMainLoop, bool communicationON,
          typename T_Preconditioner>
struct ChebyshevTag {
    static constexpr int precond = PPS_PREC_CHEBYSHEV;
    static constexpr int degree = maxIteration;
};

template <class Exact>
struct ProblemTrampoline {
    static double f(double x, double y, double z, void* c) { return static_cast<const Exact*>(c)->setFieldB(x, y, z); }
    static double u(double x, double y, double z, void* c)
    {
        return static_cast<const Exact*>(c)->trueSolutionFxyz(x, y, z);
    }
    static double du(double x, double y, double z, int d, void* c)
    {
        return static_cast<const Exact*>(c)->trueSolutionDdir(x, y, z, d);
    }
};

inline void check(pps_status st, const char* where)
{
    if (st < 0) throw std::runtime_error(std::string(where) + ": " + pps_status_string(st) + " " + pps_last_error());
}

template <int DIM, typename T_data, int tolerance, int maxIteration, bool isMainLoop, bool communicationON,
          typename T_Preconditioner, int KRYLOV>
class KrylovSolver {
    static_assert(DIM == 3, "libpps solves 3-D grids");
    static_assert(sizeof(T_data) == sizeof(double), "fields are double precision");

public:
    // As the T_Preconditioner of another solver (isMainLoop false): an inner solve
    // of this kind, tolerance and cap, preconditioned by its own T_Preconditioner.
    static constexpr int precond = KRYLOV == PPS_KRYLOV_CG ? PPS_PREC_CG : PPS_PREC_BICGSTAB;
    static constexpr int degree = T_Preconditioner::degree;
    static constexpr int inner_precond = T_Preconditioner::precond;
    static constexpr int inner_tolerance = tolerance;
    static constexpr int inner_maxit = maxIteration;

    template <class BlockGridT, class ExactT, class CommT>
    KrylovSolver(const BlockGridT& grid, const ExactT& exact, CommT&)
        : exact_(&exact), f_(&ProblemTrampoline<ExactT>::f), u_(&ProblemTrampoline<ExactT>::u),
          du_(&ProblemTrampoline<ExactT>::du)
    {
        const auto nr = grid.getNranks();
        if (nr[0] * nr[1] * nr[2] != 1) throw std::runtime_error("libpps runs a single domain (nranks 1x1x1)");
        pps_grid g;
        const auto np = grid.getNpglobal();
        const auto ds = grid.getDs();
        const auto o = grid.getOrigin();
        const auto bc = grid.getBcsType();
        for (int d = 0; d < 3; d++) {
            g.npglobal[d] = np[d];
            g.ds[d] = ds[d];
            g.origin[d] = o[d];
        }
        for (int q = 0; q < 6; q++) g.bcs[q] = bc[q];
        const ChebyshevParams p = setup_params();
        pps_config c;
        check(pps_config_default(&c, PPS_PRESET_CPU), "pps_config_default");
        c.krylov = KRYLOV;
        if constexpr (KRYLOV == PPS_KRYLOV_CHEBYSHEV) {
            c.precond = PPS_PREC_CHEBYSHEV;
            c.cheb_degree = maxIteration;   // chebyshevMax
        } else {
            c.precond = T_Preconditioner::precond;
            c.cheb_degree = T_Preconditioner::degree > 0 ? T_Preconditioner::degree : 1;
            if constexpr (T_Preconditioner::precond == PPS_PREC_BICGSTAB || T_Preconditioner::precond == PPS_PREC_CG) {
                static_assert(T_Preconditioner::inner_precond == PPS_PREC_NONE ||
                                  T_Preconditioner::inner_precond == PPS_PREC_CHEBYSHEV,
                              "an inner solver is preconditioned by NoneSolver or ChebyshevIteration");
                c.precond_tol = static_cast<double>(T_Preconditioner::inner_tolerance) * p.toll_scaling;
                c.precond_maxit = T_Preconditioner::inner_maxit;
                c.precond_inner = T_Preconditioner::inner_precond;
                nested_ = true;
            }
        }
        c.cheb_eps = p.epsilon;
        c.rescale_min = p.rescale_min;
        c.rescale_max = p.rescale_max;
        c.tol = static_cast<double>(tolerance) * p.toll_scaling;   // BiCGSTAB.hpp:22
        c.maxit = maxIteration;
        c.form = default_form();
        npdata_ = {np[0], np[1], np[2]};
        ds_ = {ds[0], ds[1], ds[2]};
        origin_ = {o[0], o[1], o[2]};
        check(pps_create(&g, &c, &s_), "pps_create");
    }
    ~KrylovSolver()
    {
        if (s_) pps_destroy(s_);
    }
    KrylovSolver(const KrylovSolver&) = delete;
    KrylovSolver& operator=(const KrylovSolver&) = delete;

    // setProblem (iterativeSolverBase.hpp:51-55)
    void setProblem(T_data fieldX[], T_data fieldB[])
    {
        pps_problem p{f_, u_, du_, const_cast<void*>(exact_)};
        check(pps_set_problem(s_, &p, fieldX, fieldB), "pps_set_problem");
    }

    // operator()(x, b, A) (BiCGSTAB.hpp:55) and the alpaka form operator()(x, b).
    template <class OperatorA>
    void operator()(T_data fieldX[], T_data fieldB[], OperatorA&)
    {
        (*this)(fieldX, fieldB);
    }
    void operator()(T_data fieldX[], T_data fieldB[])
    {
        pps_status st = pps_solve(s_, fieldX, fieldB, &stats_);
        check(st, "pps_solve");
        status_ = st;
    }

    int getNumIterationFinal() const { return stats_.iterations; }
    T_data getErrorFromIteration() const { return stats_.err_iter; }
    T_data getErrorComputeOperator() const { return stats_.err_true; }
    std::chrono::duration<double> getDurationSolver() const
    {
        return std::chrono::duration<double>(stats_.seconds_solve);
    }
    // numIterationPreconditionerFinal_: the inner solver's iterations, summed
    // (BiCGstabAlpaka.hpp:214,290), or else the preconditioner applications
    int getNumIterationPreconditionerFinal() const
    {
        return nested_ ? stats_.precond_iterations : stats_.precond_applications;
    }
    pps_status lastStatus() const { return status_; }
    const pps_stats& stats() const { return stats_; }
    pps_solver* handle() const { return s_; }

    void writeResidualHistory(const char* path = "residualHistory.txt") const
    {
        check(pps_write_residual_history(s_, path), "pps_write_residual_history");
    }

    // checkSolutionLocalGlobal at one rank (iterativeSolverBase.hpp:283-408)
    template <class ExactT = void>
    T_data checkSolutionLocalGlobal(T_data fieldX[]) const
    {
        using Tr = double (*)(double, double, double, void*);
        Tr u = u_;
        const long sj = npdata_[0] + 2, sk = sj * (npdata_[1] + 2);
        double errSum = 0, errMax = -1;
        long count = 0;
        for (int k = 1; k <= npdata_[2]; k++)
            for (int j = 1; j <= npdata_[1]; j++)
                for (int i = 1; i <= npdata_[0]; i++) {
                    const double x = origin_[0] + (i - 1) * ds_[0];
                    const double y = origin_[1] + (j - 1) * ds_[1];
                    const double z = origin_[2] + (k - 1) * ds_[2];
                    const double e = std::abs(fieldX[i + sj * j + sk * k] - u(x, y, z, const_cast<void*>(exact_)));
                    errSum += e;
                    if (e > errMax) errMax = e;
                    count++;
                }
        std::printf("Max error local block avg %g in rank 0\nMax error local point %g in rank 0\n",
                    errSum / (double)count, errMax);
        return errSum;
    }

private:
    const void* exact_;
    double (*f_)(double, double, double, void*);
    double (*u_)(double, double, double, void*);
    double (*du_)(double, double, double, int, void*);
    pps_solver* s_ = nullptr;
    pps_stats stats_{};
    pps_status status_ = PPS_OK;
    std::array<int, 3> npdata_{};
    std::array<double, 3> ds_{}, origin_{};
    bool nested_ = false;
};

// BiCGSTAB<DIM, T_data, tolerance, maxIteration, isMainLoop, communicationON, T_Preconditioner>
template <int DIM, typename T_data, int tolerance, int maxIteration, bool isMainLoop, bool communicationON,
          typename T_Preconditioner>
using BiCGSTAB = KrylovSolver<DIM, T_data, tolerance, maxIteration, isMainLoop, communicationON, T_Preconditioner,
                              PPS_KRYLOV_BICGSTAB>;

// BaseCG<DIM, T_data, tolerance, maxIteration, isMainLoop, communicationON, T_Preconditioner>
template <int DIM, typename T_data, int tolerance, int maxIteration, bool isMainLoop, bool communicationON,
          typename T_Preconditioner>
using BaseCG = KrylovSolver<DIM, T_data, tolerance, maxIteration, isMainLoop, communicationON, T_Preconditioner,
                            PPS_KRYLOV_CG>;

// ChebyshevIteration<DIM, T_data, tolerance, maxIteration, isMainLoop, communicationON,
// T_Preconditioner>: a preconditioner tag (isMainLoop false), or the Chebyshev
// iteration as the main solver (isMainLoop true), degree maxIteration.
template <int DIM, typename T_data, int tolerance, int maxIteration, bool isMainLoop, bool communicationON,
          typename T_Preconditioner>
using ChebyshevIteration = typename std::conditional<
    isMainLoop,
    KrylovSolver<DIM, T_data, tolerance, maxIteration, isMainLoop, communicationON, T_Preconditioner,
                 PPS_KRYLOV_CHEBYSHEV>,
    ChebyshevTag<DIM, T_data, tolerance, maxIteration, isMainLoop, communicationON, T_Preconditioner>>::type;

}  // namespace pps

#endif
