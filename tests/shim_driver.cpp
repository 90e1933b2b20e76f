// The reference driver's call sequence (solverPoissonMPI_CPU/src/main.cpp:83-127) on
// the libpps C++ shim, with project-written stand-ins for the reference's BlockGrid,
// ExactSolutionAndBCs (its default manufactured solution, solverSetup.hpp:45-100),
// CommunicatorMPI and MatrixFreeOperatorA.  tests/test_gpu_dropin.py builds and runs
// it on the GPU where the reference's own main.cpp is not available to compile.
//
//   shim_driver <m> <form: parity|fp64|mixed> <solution.dat>
//
// prints the line main.cpp prints after the solve (iterations and both errors, here
// with 17 significant digits) and writes x with pps_write_solution.
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "pps_solver.hpp"

constexpr int DIM = 3;
using T_data = double;

struct BlockGridStandIn {
    std::array<int, 3> np;
    std::array<double, 3> ds;
    std::array<int, 3> getNranks() const { return {1, 1, 1}; }
    std::array<int, 3> getNpglobal() const { return np; }
    std::array<double, 3> getDs() const { return ds; }
    std::array<double, 3> getOrigin() const { return {0, 0, 0}; }
    std::array<int, 6> getBcsType() const { return {0, 0, 0, 0, 0, 0}; }
    long getNtotLocalGuards() const { return (long)(np[0] + 2) * (np[1] + 2) * (np[2] + 2); }
};

struct ExactStandIn {   // u = sin x + cos y + 3 sin z + x^2 y z + x^2 + 10, f = lap u
    double setFieldB(double x, double y, double z) const { return -std::sin(x) - std::cos(y) - 3 * std::sin(z) + 2 * y * z + 2; }
    double trueSolutionFxyz(double x, double y, double z) const
    {
        return std::sin(x) + std::cos(y) + 3 * std::sin(z) + x * x * y * z + x * x + 10;
    }
    double trueSolutionDdir(double x, double y, double z, int dir) const
    {
        if (dir == 0) return std::cos(x) + 2 * x * y * z + 2 * x;
        if (dir == 1) return -std::sin(y) + x * x * z;
        return 3 * std::cos(z) + x * x * y;
    }
};
struct CommStandIn {};
struct OperatorStandIn {};

// the CPU preset's composition (inputParam.hpp:33, solverSetup.hpp:27-40)
using T_NoneSolver = pps::NoneSolver<DIM, T_data, 10000, 150>;
using T_Preconditioner2 = pps::ChebyshevIteration<DIM, T_data, 10000, 11, false, false, T_NoneSolver>;
using T_Solver = pps::BiCGSTAB<DIM, T_data, 100, 1700, true, true, T_Preconditioner2>;

int main(int argc, char** argv)
{
    if (argc < 4) {
        std::fprintf(stderr, "usage: shim_driver m parity|fp64|mixed solution.dat\n");
        return 2;
    }
    const int m = std::atoi(argv[1]);
    if (std::strcmp(argv[2], "parity") == 0) pps::default_form() = PPS_FORM_PARITY_FP64;
    else if (std::strcmp(argv[2], "mixed") == 0) pps::default_form() = PPS_FORM_MIXED;
    BlockGridStandIn blockGrid{{m + 2, m + 2, m + 2}, {1.0 / (m + 1), 1.0 / (m + 1), 1.0 / (m + 1)}};
    ExactStandIn exactSolutionAndBCs;
    CommStandIn communicator;
    OperatorStandIn operatorA;
    T_Solver solver(blockGrid, exactSolutionAndBCs, communicator);
    std::vector<T_data> fieldX((size_t)blockGrid.getNtotLocalGuards(), 0.0), fieldB(fieldX.size(), 0.0);
    solver.setProblem(fieldX.data(), fieldB.data());
    solver(fieldX.data(), fieldB.data(), operatorA);
    std::printf("Iterative solver finished with iter: %d error from algo %.17g error r=b-Ax %.17g\n",
                solver.getNumIterationFinal(), solver.getErrorFromIteration(), solver.getErrorComputeOperator());
    solver.checkSolutionLocalGlobal(fieldX.data());
    pps_grid g{{m + 2, m + 2, m + 2}, {blockGrid.ds[0], blockGrid.ds[1], blockGrid.ds[2]}, {0, 0, 0}, {0, 0, 0, 0, 0, 0}};
    pps::check(pps_write_solution(&g, fieldX.data(), 0, argv[3], nullptr), "pps_write_solution");
    return 0;
}
