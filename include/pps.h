/*
 * pps.h -- C ABI of libpps, the GB300-native (sm_103a) Poisson solve loop.
 *
 * libpps is a drop-in for the solve path of lucak17/ParallelPoissonSolver
 * (solverPoissonMPI_CPU / solverPoissonMPI_alpaka): a right-preconditioned
 * BiCGSTAB (or CG) with a Chebyshev-polynomial preconditioner on the 7-point
 * Laplacian, Dirichlet/Neumann boundary handling and Krylov reductions, on one
 * GPU as a single domain.  The reference has no C ABI: its boundary is the
 * solver-class protocol composed in include/inputParam.hpp:24-38.  Each entry
 * point below names the reference member it replaces.  include/pps_solver.hpp
 * wraps this ABI back into that class protocol.
 *
 * Conventions
 *   - Fields are caller-owned arrays of (n0+2)(n1+2)(n2+2) doubles, x fastest,
 *     where n_d = npglobal_d counts the boundary nodes and one guard layer pads
 *     each side (iterativeSolverBase.hpp:34-35; CPU/src/main.cpp:86-89).
 *   - The equation is A u = b with A the positive-sign 7-point Laplacian
 *     (matrixFreeOperatorA.hpp:22-39): for -lap u = f pass b = -f.
 *   - Every call returns a pps_status; nothing calls exit() (the reference exits
 *     on a bad configuration, CPU/src/main.cpp:51-55).
 *   - One solver handle owns one CUDA stream and its device buffers; a handle is
 *     not thread-safe, distinct handles are independent.
 */
#ifndef PPS_H
#define PPS_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PPS_ABI_VERSION 3

typedef enum {
    PPS_OK = 0,
    PPS_NOT_CONVERGED = 1,      /* stopped at maxit; the reference stops silently       */
    PPS_BREAKDOWN = 2,          /* a Krylov denominator became zero or non-finite        */
    PPS_NAN_DETECTED = 3,       /* the residual norm became NaN/Inf                      */
    PPS_TIMEOUT = 4,            /* a bounded device-side wait gave up                    */
    PPS_ERR_INVALID_ARG = -1,
    PPS_ERR_CUDA = -2,
    PPS_ERR_OUT_OF_MEMORY = -3,
    PPS_ERR_ZERO_RHS = -4,      /* ||b_adj|| == 0: the normalisation divides by zero     */
    PPS_ERR_UNSUPPORTED = -5,
    PPS_ERR_NO_DEVICE = -6
} pps_status;

/* BlockGrid at one rank (blockGrid.hpp:15-36): npglobal, ds, origin, bcsType. */
typedef struct {
    int npglobal[3];            /* grid points per axis, boundary nodes included (>= 3)  */
    double ds[3];               /* spacing                                                */
    double origin[3];           /* coordinate of the first data node                     */
    int bcs[6];                 /* x- x+ y- y+ z- z+ : 0 Dirichlet, 1 Neumann            */
} pps_grid;

/* Main solvers (T_Solver): BiCGSTAB (BiCGSTAB.hpp), CG (baseCG.hpp), flexible CG
 * (no reference counterpart: BaseCG with a Polak-Ribiere beta, for preconditioners
 * that change between applications, FP64 and MIXED forms, Dirichlet grids only),
 * and the Chebyshev iteration as the main solver (ChebyshevIteration with
 * isMainLoop true, chebyshevIteration.hpp:48-140, chebyshevIterationAlpaka.hpp:
 * 320-587): the polynomial of degree cheb_degree applied once to the adjusted b,
 * overwriting x at the unknowns, with no convergence test (`precond` is not used;
 * the reference asks for rescale_min = rescale_max = 1 in this use,
 * ALP/include/inputParam.hpp:21). */
typedef enum {
    PPS_KRYLOV_BICGSTAB = 0,
    PPS_KRYLOV_CG = 1,
    PPS_KRYLOV_FCG = 2,
    PPS_KRYLOV_CHEBYSHEV = 3
} pps_krylov;
/* Preconditioners (T_Preconditioner): none (noneSolver.hpp), the Chebyshev
 * polynomial (chebyshevIteration.hpp, isMainLoop false), or an inner solve from
 * X = 0 on B / ||B|| to precond_tol or precond_maxit iterations, itself
 * preconditioned by precond_inner: BiCGSTAB (BiCGSTAB.hpp with isMainLoop false,
 * CPU/include/inputParam.hpp:30, ALP/include/inputParam.hpp:31-33) or CG (baseCG.hpp
 * with isMainLoop false, CPU/include/inputParam.hpp:29). */
typedef enum { PPS_PREC_NONE = 0, PPS_PREC_CHEBYSHEV = 1, PPS_PREC_BICGSTAB = 2, PPS_PREC_CG = 3 } pps_precond;

typedef enum {
    /* FP64 with the reference's expression order and serial reductions: results are
     * bit-identical to the reference CPU solver at one rank. Slow; for validation. */
    PPS_FORM_PARITY_FP64 = 0,
    /* Plain FP64: fused kernels, deterministic tree reductions, scalars on device. */
    PPS_FORM_FP64 = 1,
    /* FP32 stencil, smoother and Krylov vectors with FP64-accurate inner products,
     * wrapped in FP64 iterative refinement on the FP64 true residual. */
    PPS_FORM_MIXED = 2
} pps_form;

/* Compile-time parameters of the reference, made runtime (solverSetup.hpp:22-40,
 * inputParam.hpp:24-38; alpaka preset ALP/include/solverSetup.hpp:52-72). */
typedef struct {
    int krylov;                 /* pps_krylov (T_Solver)                                   */
    int precond;                /* pps_precond (T_Preconditioner)                          */
    int cheb_degree;            /* chebyshevMax                                             */
    double cheb_eps;            /* epsilon                                                  */
    double rescale_min;         /* rescaleEigMin                                            */
    double rescale_max;         /* rescaleEigMax                                            */
    double tol;                 /* tolerance * tollScalingFactor (on ||r||/||b_adj||)       */
    int maxit;                  /* maxIteration of the Krylov loop                          */
    int form;                   /* pps_form                                                 */
    double inner_tol;           /* MIXED: relative residual reduction per refinement        */
    int inner_maxit;            /* MIXED: iteration cap of one inner solve                  */
    int max_refinements;        /* MIXED: cap on outer refinement steps                     */
    int check_every;            /* iterations between host polls of the device stop flag;
                                   0 = automatic.  Results do not depend on it.             */
    int use_graph;              /* replay the iteration as a CUDA graph (fast forms)        */
    int device;                 /* CUDA device ordinal                                      */
    /* PPS_PREC_BICGSTAB, PPS_PREC_CG: the inner solver's toll_ (tollPreconditionerSolver *
     * tollScalingFactor, on its ||r||/||B||, 0 < precond_tol < 1), maxIteration
     * (iterMaxPreconditioner) and its own preconditioner (PPS_PREC_NONE, or
     * PPS_PREC_CHEBYSHEV with the cheb_* fields above). */
    double precond_tol;
    int precond_maxit;
    int precond_inner;
} pps_config;

typedef enum { PPS_PRESET_CPU = 0, PPS_PRESET_ALPAKA = 1 } pps_preset;

typedef struct {
    int iterations;             /* getNumIterationFinal (MIXED: inner iterations, summed)   */
    int refinements;            /* MIXED: outer refinement steps taken                      */
    int precond_applications;
    double err_iter;            /* getErrorFromIteration: recursive ||r||/||b_adj||         */
    double err_true;            /* getErrorComputeOperator: true FP64 ||b-Ax||/||b_adj||   */
    double norm_b;              /* ||b_adj|| over the unknowns                              */
    double seconds_solve;       /* device time from set-up to the final residual           */
    double seconds_total;       /* host wall time of the call                               */
    double seconds_h2d;         /* host->device copies inside the call                      */
    double seconds_d2h;
    double hbm_bytes;           /* algorithmic bytes of every kernel the solve launched     */
    int kernel_launches;        /* launches of libpps kernels inside the call               */
    double sweep_seconds;       /* device time of the Chebyshev sweeps (event-timed)        */
    int sweep_launches;         /* sweeps launched                                          */
    double sweep_bytes;         /* algorithmic bytes of those sweeps                        */
    int learned_applications;   /* network corrections applied (pps_set_learned)           */
    int fallback_iteration;     /* iteration at which the learned preconditioner was dropped, -1 none */
    int precond_iterations;     /* inner solver: its iterations summed over the
                                   applications (numIterationPreconditionerFinal_,
                                   BiCGstabAlpaka.hpp:214,290)                              */
    double krylov_seconds;      /* flexible CG: device time of its direction + stencil and
                                   x, r update kernels (event-timed, use_graph 0 only)      */
    int krylov_launches;        /* those kernels launched                                   */
    double krylov_bytes;        /* their algorithmic bytes                                  */
    int copy_overlap;           /* pps_solve, MIXED form on pinned arrays: bit 0, b was
                                   uploaded first and the solve started on it while x
                                   uploaded; bit 1, x held a non-zero entry and the solve
                                   restarted on it; bit 2, x's copy out overlapped the
                                   final residual check.  seconds_h2d is then b's upload,
                                   seconds_d2h what remained of x's copy out              */
} pps_stats;

typedef struct pps_solver pps_solver;

/* Problem plugin, the ExactSolutionAndBCs class (solverSetup.hpp:94-161). */
typedef struct {
    double (*field_b)(double x, double y, double z, void* ctx);              /* setFieldB        */
    double (*solution)(double x, double y, double z, void* ctx);             /* trueSolutionFxyz */
    double (*solution_ddir)(double x, double y, double z, int dir, void* ctx); /* trueSolutionDdir */
    void* ctx;
} pps_problem;

typedef enum { PPS_PROBLEM_REFERENCE_DEFAULT = 0, PPS_PROBLEM_SINE = 1 } pps_builtin_problem;

/* Defaults of the reference presets: CPU (n=11, eps=1e-4, rescale 500, tol 1e-8,
 * maxit 1700; inner BiCGSTAB preconditioner tol 1e-6, maxit 150) or alpaka (n=24,
 * eps=0, rescale 100, tol 1e-10, maxit 1000; inner tol 1e-2, maxit 500). */
pps_status pps_config_default(pps_config* cfg, int preset);

/* Solver constructor (BiCGSTAB.hpp:18-39 with the ChebyshevIteration member,
 * chebyshevIteration.hpp:19-34): validates, computes the eigenvalue bounds
 * (blockGrid.hpp:301-340) and allocates every device buffer. */
pps_status pps_create(const pps_grid* grid, const pps_config* cfg, pps_solver** out);
pps_status pps_destroy(pps_solver* s);

/* setProblem (iterativeSolverBase.hpp:51-55): Dirichlet nodes of x from
 * plugin->solution, b from plugin->field_b at every data node, and the Neumann
 * face data from plugin->solution_ddir (kept in the solver for the solves). */
pps_status pps_set_problem(pps_solver* s, const pps_problem* plugin, double* x, double* b);
pps_status pps_set_problem_builtin(pps_solver* s, int builtin_problem, double* x, double* b);
/* Neumann data of face f (2*dir+side) at its data nodes, lower remaining axis fastest. */
pps_status pps_set_neumann(pps_solver* s, int face, const double* values);

/* operator()(x, b, A) (BiCGSTAB.hpp:55-322, BiCGstabAlpaka.hpp:68-475): solves in
 * place on host arrays; x is in/out (Dirichlet nodes hold the boundary values),
 * b is input (PARITY form: scaled and unscaled in place exactly like the reference).
 * Returns PPS_OK, PPS_NOT_CONVERGED, PPS_BREAKDOWN or an error.
 * PPS_KRYLOV_CHEBYSHEV: iterations = cheb_degree, err_iter = err_true = the
 * absolute ||b - A x|| (the reference does not normalise in this use), history one
 * entry holding it; PPS_OK when it is below tol * norm_b, else PPS_NOT_CONVERGED.
 * The MIXED form applies the polynomial in FP32 to the FP64 residual up to
 * max_refinements + 1 times, stopping at tol (iterations: degree x passes).
 * On page-locked arrays the MIXED Krylov solves (Dirichlet faces) upload b first
 * and start on it as if x were zero while x uploads on a second stream; a non-zero
 * x restarts the solve on it, so the result is the same either way.  x is copied out
 * after each refinement, the last copy overlapping the final residual check
 * (pps_stats.copy_overlap); on an error x may hold an intermediate iterate. */
pps_status pps_solve(pps_solver* s, double* x, double* b, pps_stats* stats);
/* The same with device pointers (fields already resident in HBM).  The solver's
 * stream is non-blocking: work that writes x_dev or b_dev on another stream must be
 * complete before the call (the call returns with the solve finished). */
pps_status pps_solve_device(pps_solver* s, double* x_dev, double* b_dev, pps_stats* stats);

/* Getters (iterativeSolverBase.hpp:410-425; iterativeSolverBaseAlpaka.hpp:599-640). */
pps_status pps_get_stats(const pps_solver* s, pps_stats* stats);
/* Residual history: entry 0 is the initial true residual, entry i the recursive
 * residual after iteration i (errorFromIterationHistory_).  *count <= cap. */
pps_status pps_get_history(const pps_solver* s, double* out, int cap, int* count);
/* residualHistory.txt writer (iterativeSolverBaseAlpaka.hpp:620-638). */
pps_status pps_write_residual_history(const pps_solver* s, const char* path);
/* solution.dat writer (the alpaka driver's MPI-IO dump, ALP/src/main.cpp:135-146):
 * the rank's whole guard-padded field x ((n0+2)(n1+2)(n2+2) doubles, memory order)
 * at byte offset rank * G * 8 of `path`, which is created if missing and not
 * truncated otherwise.  x may be host or device memory; a device field is copied
 * on `stream` (a cudaStream_t, NULL = legacy default), after the work queued there. */
pps_status pps_write_solution(const pps_grid* grid, const double* x, int rank, const char* path, void* stream);

/* Building blocks, on host arrays of the field layout.
 * out = A u at the unknowns (MatrixFreeOperatorA::operator(), FP64). */
pps_status pps_apply_operator(pps_solver* s, const double* u, double* out);
/* X = M^{-1} B: one preconditioner application (ChebyshevIteration::operator()
 * in preconditioner mode, chebyshevIteration.hpp:48-140), in the solver's form;
 * with a network attached by pps_set_learned as preconditioner, the learned cycle
 * that flexible CG applies. */
pps_status pps_apply_preconditioner(pps_solver* s, const double* B, double* X);

/* Tile shapes of the z-marching kernels (fast forms).  A tile is (32*cx) x ty
 * columns; each thread walks along z; `waves` sets the grid to about
 * waves x 152 SMs x resident blocks.  cheb_* apply to the Chebyshev kernels and to
 * the Krylov stencil kernels that run on the same tiles (flexible CG's direction
 * update, BiCGSTAB's and CG's stencil + dots, the learned cycle's last
 * prolongation), other_* to the remaining Krylov update/stencil kernels.  cheb_cx 4
 * selects the x-vectorised FP32 kernels (one float4 per thread, the default where
 * npglobal[0] + 2 is a multiple of 4; FP64 fields and other rows run cx 1 tiles of
 * the same size).  cheb_us: the sweep's time per launch; other_us: the
 * stencil+dot kernel's. */
typedef struct {
    int cheb_ty, cheb_cx, cheb_waves;
    int other_ty, other_waves;
    double cheb_us, other_us;
    int cheb_fused;             /* 1: Chebyshev applications of degree 4 or 5 on Dirichlet grids
                                   run all their steps in one temporally blocked pass
                                   (bit-identical); 0 (default): one launch per step */
    int fcg_staged;             /* 1: flexible CG's direction kernel on the cx 4 tiles
                                   stages its inputs in shared memory by TMA (bit-identical;
                                   slower on GB300 at 512^3); 0 (default): it loads them
                                   itself */
} pps_tuning;

/* Autotuner (no reference counterpart; the reference fixes its launch shapes,
 * ALP/include/alpakaHelper.hpp:122-140): times every candidate shape on this
 * solver's grid and buffers, applies the fastest and returns it.  The Chebyshev
 * tiles are scored by the sweep's time, weighted by the Chebyshev launches per
 * Krylov stencil launch of an iteration (cheb_degree - 2, or the learned cycle's
 * fine degree - 2), plus that of the method's Krylov stencil kernel on the same
 * tiles; the other tiles by the stencil+dot kernel.
 * Candidates: ty 2/4/8, cx 1/2/4 (4: FP32 only), waves 1/2/4/8. */
pps_status pps_autotune(pps_solver* s, pps_tuning* out);
pps_status pps_get_tuning(const pps_solver* s, pps_tuning* out);
/* Applies a stored tuning (e.g. from a table persisted by the caller). */
pps_status pps_set_tuning(pps_solver* s, const pps_tuning* t);

/* ---- Batches: many independent Dirichlet grids solved together ----
 * No reference counterpart (the reference solves one grid per run).  Two methods,
 * both in the MIXED form (FP32 inner iterations, FP64 true residual and refinement):
 *   krylov PPS_KRYLOV_FCG: flexible CG with a multigrid V-cycle per problem (cubes
 *     with equal spacings, edge m = c * 2^k, k >= 1, c <= 32), the whole solve ONE
 *     persistent cooperative launch replayed as a CUDA graph: a fixed program of
 *     phases per round spread over every block as (problem, tile) items, phases
 *     separated by a grid barrier whose wait is bounded (pps_batch_set_wait_limit);
 *     a wait that runs out ends the solve with PPS_TIMEOUT;
 *   krylov PPS_KRYLOV_BICGSTAB: the reference's BiCGSTAB + Chebyshev per problem,
 *     one launch per loop phase over all problems, the inner iteration replayed as
 *     a CUDA graph, per-problem tile shapes from the autotuner.
 * Fields live in device pools owned by the batch (pps_batch_set/get copy them,
 * pps_batch_field_device exposes them). */
typedef struct pps_batch pps_batch;

typedef struct {
    double seconds_solve;       /* device time of the whole batched solve                  */
    int kernel_launches;
    int graph_replays;
    double max_err_true;        /* max over problems of the FP64 ||b-Ax||/||b_adj||        */
    int max_iterations;         /* max over problems of the inner iterations               */
    int sum_iterations;
    int max_refinements;
    int converged;              /* problems that reached tol                               */
    double unknowns;            /* sum of the problems' unknowns                           */
} pps_batch_stats;

/* cfg: form PPS_FORM_MIXED; krylov PPS_KRYLOV_FCG (persistent V-cycle) or BiCGSTAB with
 * Chebyshev degree >= 4; grids all-Dirichlet. */
pps_status pps_batch_create(int nprob, const pps_grid* grids, const pps_config* cfg, pps_batch** out);
pps_status pps_batch_destroy(pps_batch* batch);
pps_status pps_batch_set(pps_batch* batch, int p, const double* x, const double* b);
pps_status pps_batch_get(pps_batch* batch, int p, double* x, pps_stats* stats);
pps_status pps_batch_field_device(pps_batch* batch, int p, double** x_dev, double** b_dev);
/* Times the batched sweep for every grid shape in the batch over candidate tiles
 * (columns per thread 1/2, z-chunk 8..128, and the x-vectorised float4 tiles where
 * npglobal[0] + 2 is a multiple of 4) and keeps the fastest per shape. */
pps_status pps_batch_autotune(pps_batch* batch);
/* The Chebyshev kernels' tile of problem p: cx 1, 2, or 4 (float4 per thread). */
pps_status pps_batch_tile(const pps_batch* batch, int p, int* cx, int* kchunk);
/* Solves every problem to cfg->tol (FP64 true residual).  PPS_NOT_CONVERGED if any
 * problem stopped short. */
pps_status pps_batch_solve(pps_batch* batch, pps_batch_stats* stats);
/* Persistent batches (krylov PPS_KRYLOV_FCG): how long a block may wait at a grid
 * barrier for the others before the solve stops with PPS_TIMEOUT (default 5 s; a
 * healthy barrier completes in microseconds). */
pps_status pps_batch_set_wait_limit(pps_batch* batch, double seconds);

/* ---- Learned preconditioner: a 3-D convolutional U-Net ----
 * No reference counterpart.  3 levels with c1/c2/c3 channels (16/32/64), 3x3x3
 * kernels, BF16 weights and activations with FP32 accumulation on the tensor cores,
 * trained by the project's own forward/backward kernels and Adam.  Arrays are dense
 * FP32 [nz][ny][nx] device arrays (extents multiples of 4); the parameter vector is,
 * per layer, W[27][cin][cout] (tap = kz*9 + ky*3 + kx) then b[cout]. */
typedef struct pps_unet pps_unet;
pps_status pps_unet_create(int c1, int c2, int c3, unsigned long long seed, int device, pps_unet** out);
pps_status pps_unet_destroy(pps_unet* net);
int pps_unet_param_count(const pps_unet* net);
/* Activation of the hidden layers: 0 ReLU (default), 1 identity (the network is then
 * a learned linear operator with the U-Net's multigrid structure). */
pps_status pps_unet_set_activation(pps_unet* net, int linear);
pps_status pps_unet_get_params(const pps_unet* net, float* out);
pps_status pps_unet_set_params(pps_unet* net, const float* in);
/* normalize = 1: the input is scaled to unit RMS and the output scaled back.
 * The network's calls run on its own non-blocking stream and return with their work
 * finished; device inputs written on another stream must be complete before the call. */
pps_status pps_unet_forward(pps_unet* net, int nx, int ny, int nz, const float* in_dev, float* out_dev,
                            int normalize);
/* MSE loss of the (unnormalised) output against target, and its gradient (host array
 * of pps_unet_param_count floats). */
pps_status pps_unet_gradients(pps_unet* net, int nx, int ny, int nz, const float* in_dev, const float* target_dev,
                              float* grads, double* loss);
/* One Adam step (beta1 0.9, beta2 0.999, gradient clipped to global norm 1) on the
 * MSE loss of one sample. */
pps_status pps_unet_train_step(pps_unet* net, int nx, int ny, int nz, const float* in_dev, const float* target_dev,
                               float lr, double* loss);
/* Attaches a trained U-Net to a solver (FP64 or MIXED form, Dirichlet grid whose
 * unknown extents are multiples of 4*2^coarsen, at most 65535 along y and z).  flags:
 *   PPS_LEARNED_INITIAL_GUESS   x += gain * P^k N(R^k b) before the solve;
 *   PPS_LEARNED_PRECONDITIONER  inside flexible CG, z = Cheb(r) followed by
 *                               z += gain * P^k N(R^k (r - A z)); the solve falls back
 *                               to the plain preconditioner for good (restarting the
 *                               recurrence) as soon as the per-iteration reduction of
 *                               ||r||, the geometric mean over the last 4 iterations,
 *                               is worse than 0.5.
 * R, P: 2x restriction/prolongation, applied `coarsen` (0..8) times; N: the network with
 * unit-RMS input scaling.  net = NULL detaches.  The network must outlive its use. */
#define PPS_LEARNED_INITIAL_GUESS 1
#define PPS_LEARNED_PRECONDITIONER 2
#define PPS_LEARNED_NO_FALLBACK 4     /* keep the network for the whole solve (measurements) */
#define PPS_LEARNED_POST_SMOOTH 8     /* z += Cheb(r - A z) after the correction (two-grid cycle) */
pps_status pps_set_learned(pps_solver* s, pps_unet* net, int coarsen, double gain, int flags);

/* Multigrid form of the learned preconditioner (no reference counterpart).  With
 * fine_degree >= 2 and coarsen >= 1, each application is a V-cycle over the levels
 * 0..coarsen whose coarsest solver is the network: Chebyshev smoothing on
 * [lambda_max/ratio, lambda_max] of the solver's operator, full-weighting restriction
 * of the residual, on each coarse level l a Jacobi-scaled Chebyshev smoother on
 * [2/ratio, 2] of D^-1 A_l (A_l: the 7-point operator with spacings 2^l ds, whose
 * upper wall lies one fine spacing above the last unknown, as the coarsening of an
 * even grid places it; D = -diag A_l), trilinear prolongation of the correction and
 * post-smoothing (on the solver's grid with PPS_LEARNED_POST_SMOOTH).  The network
 * should be trained for the coarsest level's operator.
 * Degrees count as cheb_degree does (the recurrence's output is s_{n-2}):
 * fine_degree on the solver's grid, coarse_degree on levels 1..coarsen-1 (0: no
 * smoothing there).  fine_degree = 0 (the default) keeps the two-grid cycle around
 * the solver's own Chebyshev preconditioner. */
pps_status pps_set_learned_cycle(pps_solver* s, int fine_degree, int coarse_degree, double ratio);

/* Coarsest-level solver of the learned multigrid V-cycle (pps_set_learned_cycle).
 * No counterpart in the reference: it measures what the network earns in the cycle
 * by putting plain alternatives in its place, with everything else unchanged:
 *   PPS_COARSE_NETWORK  the attached U-Net (the default);
 *   PPS_COARSE_ZERO     no correction on the coarsest level;
 *   PPS_COARSE_SMOOTH   the coarse levels' Jacobi-scaled Chebyshev smoother
 *                       (coarse_degree >= 2 of pps_set_learned_cycle);
 *   PPS_COARSE_EXACT    the level operator's exact inverse by a tensor-product
 *                       eigen-solve (at most 32 unknowns per axis on that level).
 * The network stays attached (it holds the cycle's level count and settings);
 * pps_set_learned resets the choice to PPS_COARSE_NETWORK. */
enum { PPS_COARSE_NETWORK = 0, PPS_COARSE_ZERO = 1, PPS_COARSE_SMOOTH = 2, PPS_COARSE_EXACT = 3 };
pps_status pps_set_coarse_solver(pps_solver* s, int kind);

/* 2x grid transfers of dense unknown arrays (coarse extents nx, ny, nz; the fine
 * grid has twice as many unknowns per axis, coarse unknown i on fine unknown 2i+1):
 * full-weighting restriction and trilinear prolongation (its transpose / 8).
 * ny and nz are at most 32767. */
pps_status pps_restrict2(int nx, int ny, int nz, const float* fine_dev, float* coarse_dev);
pps_status pps_prolong2(int nx, int ny, int nz, const float* coarse_dev, float* fine_dev);

/* Operator apply that allocates nothing.  No counterpart in the reference: it is for
 * callers that cannot call cudaMalloc -- loops that forbid allocation after
 * start-up, plugins whose host framework owns all device memory, applications
 * whose device-memory budget is fixed when they start -- and so cannot create a
 * pps_solver.
 *
 * On device pointers of the field layout: out_dev = A u at the unknowns (the FP64
 * form's kernel; every other entry of out_dev is left as it was) and
 * *energy_dev = sum of u*(A u) over the unknowns.  u_dev, out_dev and energy_dev
 * must not overlap (an in-place call is rejected with PPS_ERR_INVALID_ARG).  Work
 * is queued on `stream` (a cudaStream_t; NULL = the legacy default stream); the
 * call does not wait.
 *
 * Its reduction scratch is a file-scope __device__ array of
 * 512 + 32*PPS_NOALLOC_MAX_BLOCKS bytes (about 512 KiB) that every GPU which loads
 * the library holds until the process exits.  Grids whose launch needs more than
 * PPS_NOALLOC_MAX_BLOCKS thread blocks are rejected with PPS_ERR_INVALID_ARG.
 * The first call on each device looks up the array's device address with that
 * device current and keeps it; make that first call before any stream capture,
 * and do not use the entry point across a cudaDeviceReset.  All calls
 * share the one array, so calls that overlap on the GPU (other streams, other
 * threads) race: serialise them. */
#define PPS_NOALLOC_MAX_BLOCKS 16384
pps_status pps_apply_operator_noalloc(const pps_grid* grid, const double* u_dev, double* out_dev,
                                      double* energy_dev, void* stream);

/* Number of CUDA devices visible to the library (0 without a GPU). */
int pps_device_count(void);
const char* pps_status_string(pps_status st);
/* Message of the last error on this thread ("" if none). */
const char* pps_last_error(void);
int pps_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif
