/*
 * Project-written configuration header that builds the reference's own driver,
 * solverPoissonMPI_CPU/src/main.cpp (compiled unchanged, where it lies), against
 * libpps.  TEST INFRASTRUCTURE: `make -C oracle dropin` uses it; libpps never does.
 *
 * The reference configures a build by editing include/inputParam.hpp (the solver
 * composition by type alias, inputParam.hpp:24-38, and the grid constants); this
 * header takes its place on the include path with the names main.cpp reads.  The
 * one change a maintainer makes to switch to the GPU is the composition: the
 * aliases name the pps:: shim (include/pps_solver.hpp) instead of the reference's
 * CPU classes.  The grid is one a single rank runs: 64^3 unknowns on the unit cube
 * (npglobal 66, spacing 1/65), Dirichlet data on every face from the reference's
 * default manufactured solution (solverSetup.hpp:45-100).
 *
 * PPS_FORM=parity|fp64|mixed in the environment picks the shim's form (FP64 by
 * default; parity reproduces the reference bit for bit).
 */
#ifndef PARAM_HPP
#define PARAM_HPP

#include <array>
#include <cmath>
#include <cstdlib>
#include <cstring>

#include "solvers.hpp"   // the reference's classes: main.cpp's other headers expect them

#define PPS_USE_REFERENCE_SETUP   // epsilon, rescaleEig*, tollScalingFactor from solverSetup.hpp
#include "pps_solver.hpp"

constexpr int DIM = 3;

constexpr bool ischebyshevMainLoop = false;
constexpr bool isbiCGMainLoop1 = true;
constexpr bool isbiCGMainLoop2 = false;
constexpr bool communicationON = true;
constexpr bool communicationOFF = false;

using T_NoneSolver = pps::NoneSolver<DIM, T_data, tollPreconditionerSolver, iterMaxPreconditioner>;
using T_Preconditioner2 = pps::ChebyshevIteration<DIM, T_data, tollPreconditionerSolver, chebyshevMax,
                                                  ischebyshevMainLoop, communicationOFF, T_NoneSolver>;
using T_Solver = pps::BiCGSTAB<DIM, T_data, tollMainSolver, iterMaxMainSolver, isbiCGMainLoop1, communicationON,
                               T_Preconditioner2>;

constexpr std::array<int, 3> npglobal = {66, 66, 66};
constexpr std::array<T_data, 3> ds = {1.0 / 65, 1.0 / 65, 1.0 / 65};
constexpr std::array<T_data, 3> origin = {0, 0, 0};
constexpr std::array<int, 3> guards = {1, 1, 1};
constexpr std::array<int, 6> bcsType = {0, 0, 0, 0, 0, 0};
const std::array<T_data, 6> bcsValue = {0, 0, 0, 0, 0, 0};

// the shim's form, chosen before main() constructs the solver
inline const int pps_dropin_form = [] {
    const char* f = std::getenv("PPS_FORM");
    if (f && std::strcmp(f, "parity") == 0) pps::default_form() = PPS_FORM_PARITY_FP64;
    else if (f && std::strcmp(f, "mixed") == 0) pps::default_form() = PPS_FORM_MIXED;
    return pps::default_form();
}();

#endif
