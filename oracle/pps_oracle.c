/*
 * pps_oracle.c -- CPU restatement of the reference solve loop (TEST INFRASTRUCTURE).
 *
 * The oracle: only tests, the smoke check and bench.py's CPU-baseline leg call it,
 * always to check results.  See pps_oracle.h for the reference files each part follows.
 *
 * Every arithmetic expression below keeps the reference's operand order so that,
 * compiled with -ffp-contract=off, each result is bit-identical to the reference's
 * CPU solver at one rank.  Element-wise passes may run on several OpenMP threads
 * (each output point is computed independently, so threading cannot change a bit);
 * every reduction is a single serial sum in the reference's k,j,i loop order.
 */
#include "pps_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* blockGrid.hpp / solverSetup.hpp:70 */
static const double ORA_PI = 3.141592653589793;

typedef struct {
    int n[3];
    long gx, gy, gz, sj, sk, ntot;
    int lo[3], hi[3];        /* indexLimitsSolver_: unknowns are lo <= i < hi */
    int dlo[3], dhi[3];      /* indexLimitsData_:   data nodes 1 <= i < n+1   */
    double ds[3], origin[3];
    int bcs[6];
    int nthreads;
    double* stamps;          /* main loop: wall clock at the end of each iteration */
} grid_t;

static int make_grid(const ora_grid* g, int threads, grid_t* G)
{
    for (int d = 0; d < 3; d++) {
        if (g->np[d] < 1 || !(g->ds[d] > 0.0)) return -1;
        G->n[d] = g->np[d];
        G->ds[d] = g->ds[d];
        G->origin[d] = g->origin[d];
    }
    for (int f = 0; f < 6; f++) {
        if (g->bcs[f] != 0 && g->bcs[f] != 1) return -1;
        G->bcs[f] = g->bcs[f];
    }
    G->gx = g->np[0] + 2; G->gy = g->np[1] + 2; G->gz = g->np[2] + 2;
    G->sj = G->gx; G->sk = G->gx * G->gy; G->ntot = G->sk * G->gz;
    /* calculateIndexLimitsData (blockGrid.hpp:184-206) and ...Solver (:208-222),
     * single rank so every face is a physical boundary. */
    for (int d = 0; d < 3; d++) {
        G->dlo[d] = 1; G->dhi[d] = g->np[d] + 1;
        G->lo[d] = G->dlo[d] + (g->bcs[2 * d] == 0 ? 1 : 0);
        G->hi[d] = G->dhi[d] - (g->bcs[2 * d + 1] == 0 ? 1 : 0);
    }
    G->nthreads = threads > 0 ? threads : 1;
    G->stamps = NULL;
    return 0;
}

static double now_s(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* MatrixFreeOperatorA::operator() for DIM==3 (matrixFreeOperatorA.hpp:34-38). */
static inline double opA(const grid_t* G, const double* d, long c)
{
    const long sj = G->sj, sk = G->sk;
    return (d[c - 1] - 2 * d[c] + d[c + 1]) / (G->ds[0] * G->ds[0])
         + (d[c - sj] - 2 * d[c] + d[c + sj]) / (G->ds[1] * G->ds[1])
         + (d[c - sk] - 2 * d[c] + d[c + sk]) / (G->ds[2] * G->ds[2]);
}

#define FOR_UNKNOWNS_PAR(G, body)                                                   \
    do {                                                                            \
        _Pragma("omp parallel for schedule(static) num_threads(G->nthreads) if(G->nthreads > 1)") \
        for (int k = G->lo[2]; k < G->hi[2]; k++)                                   \
            for (int j = G->lo[1]; j < G->hi[1]; j++)                               \
                for (int i = G->lo[0]; i < G->hi[0]; i++) {                         \
                    const long c = i + G->sj * j + G->sk * k;                       \
                    body;                                                           \
                }                                                                   \
    } while (0)

#define FOR_ALL_PAR(G, body)                                                        \
    do {                                                                            \
        _Pragma("omp parallel for schedule(static) num_threads(G->nthreads) if(G->nthreads > 1)") \
        for (long c = 0; c < G->ntot; c++) { body; }                                \
    } while (0)

/* Serial sum over the unknowns in the reference's loop order. */
static double dot_serial(const grid_t* G, const double* a, const double* b)
{
    double s = 0.0;
    for (int k = G->lo[2]; k < G->hi[2]; k++)
        for (int j = G->lo[1]; j < G->hi[1]; j++)
            for (int i = G->lo[0]; i < G->hi[0]; i++) {
                const long c = i + G->sj * j + G->sk * k;
                s += a[c] * b[c];
            }
    return s;
}

/* Two serial sums that the reference accumulates in one loop (pSum1, pSum2). */
static void dot2_serial(const grid_t* G, const double* a1, const double* b1, const double* a2,
                        const double* b2, double* s1, double* s2)
{
    double p1 = 0.0, p2 = 0.0;
    for (int k = G->lo[2]; k < G->hi[2]; k++)
        for (int j = G->lo[1]; j < G->hi[1]; j++)
            for (int i = G->lo[0]; i < G->hi[0]; i++) {
                const long c = i + G->sj * j + G->sk * k;
                p1 += a1[c] * b1[c];
                p2 += a2[c] * b2[c];
            }
    *s1 = p1;
    *s2 = p2;
}

/* Face iteration helper: the data-node plane of face f (iterativeSolverBase.hpp:65-78). */
typedef struct { int lo[3], hi[3]; int dir, side; } face_t;

static face_t face_range(const grid_t* G, int f)
{
    face_t F;
    F.dir = f / 2; F.side = f % 2;
    for (int d = 0; d < 3; d++) { F.lo[d] = G->dlo[d]; F.hi[d] = G->dhi[d]; }
    if (F.side == 0) F.hi[F.dir] = F.lo[F.dir] + 1;
    else             F.lo[F.dir] = F.hi[F.dir] - 1;
    return F;
}

/* Index of a data node inside a face array (lower remaining axis fastest). */
static long face_index(const grid_t* G, int dir, int i, int j, int k)
{
    if (dir == 0) return (long)(j - 1) + (long)G->n[1] * (k - 1);
    if (dir == 1) return (long)(i - 1) + (long)G->n[0] * (k - 1);
    return (long)(i - 1) + (long)G->n[0] * (j - 1);
}

/* resetNeumanBCs (iterativeSolverBase.hpp:62-169), orderNeumanBcs == 2.
 * field_data: the isMainLoop && fieldData branch that adds the boundary flux. */
static void reset_neumann(const grid_t* G, double* field, int field_data,
                          const double* const* neumann, double normb)
{
    for (int f = 0; f < 6; f++) {
        if (G->bcs[f] != 1) continue;
        face_t F = face_range(G, f);
        const int dir = F.dir;
        const long step = dir == 0 ? 1 : (dir == 1 ? G->sj : G->sk);
        const double* gface = neumann ? neumann[f] : NULL;
        for (int k = F.lo[2]; k < F.hi[2]; k++)
            for (int j = F.lo[1]; j < F.hi[1]; j++)
                for (int i = F.lo[0]; i < F.hi[0]; i++) {
                    const long c = i + G->sj * j + G->sk * k;
                    long ghost, mirror;
                    if (F.side == 0) { ghost = c - step; mirror = c + step; }
                    else             { ghost = c + step; mirror = c - step; }
                    if (field_data) {
                        const double gv = gface ? gface[face_index(G, dir, i, j, k)] : 0.0;
                        if (F.side == 0)
                            field[ghost] = field[mirror] - 2 * G->ds[dir] * gv / normb;
                        else
                            field[ghost] = field[mirror] + 2 * G->ds[dir] * gv / normb;
                    } else {
                        field[ghost] = field[mirror];
                    }
                }
    }
}

/* adjustFieldBForDirichletNeumanBCs (iterativeSolverBase.hpp:429-534). */
static void adjust_b(const grid_t* G, const double* x, double* b, const double* const* neumann)
{
    for (int dir = 0; dir < 3; dir++) {
        for (int side = 0; side < 2; side++) {
            const int f = 2 * dir + side;
            face_t F = face_range(G, f);
            const long step = dir == 0 ? 1 : (dir == 1 ? G->sj : G->sk);
            const double* gface = neumann ? neumann[f] : NULL;
            for (int k = F.lo[2]; k < F.hi[2]; k++)
                for (int j = F.lo[1]; j < F.hi[1]; j++)
                    for (int i = F.lo[0]; i < F.hi[0]; i++) {
                        const long c = i + G->sj * j + G->sk * k;
                        if (G->bcs[f] == 0) {
                            const long cb = side == 0 ? c + step : c - step;
                            b[cb] -= x[c] / (G->ds[dir] * G->ds[dir]);
                        } else {
                            const double gv = gface ? gface[face_index(G, dir, i, j, k)] : 0.0;
                            if (side == 0) b[c] += 2 * gv / G->ds[dir];
                            else           b[c] -= 2 * gv / G->ds[dir];
                        }
                    }
        }
    }
}

/* normalizeProblemToFieldBNorm<true,...> (iterativeSolverBase.hpp:171-234). */
static double normalize(const grid_t* G, double* x, double* b, const double* const* neumann)
{
    double* bt = (double*)malloc(sizeof(double) * (size_t)G->ntot);
    memcpy(bt, b, sizeof(double) * (size_t)G->ntot);
    adjust_b(G, x, bt, neumann);
    double s = dot_serial(G, bt, bt);
    free(bt);
    const double normb = sqrt(s);
    FOR_ALL_PAR(G, { x[c] /= normb; b[c] /= normb; });
    return normb;
}

/* computeErrorOperatorA<true,...> (iterativeSolverBase.hpp:236-280). */
static double true_residual(const grid_t* G, double* x, const double* b, double* r,
                            const double* const* neumann, double normb)
{
    reset_neumann(G, x, 1, neumann, normb);
    FOR_UNKNOWNS_PAR(G, { r[c] = b[c] - opA(G, x, c); });
    return sqrt(dot_serial(G, r, r));
}

/* computeEigenvalues, global part (blockGrid.hpp:322-339). */
void ora_eigen_bounds(const ora_grid* g, double out[2])
{
    double eigMin = 0, eigMax = 0;
    for (int i = 0; i < 3; i++) {
        int ni = g->np[i];
        if (g->bcs[2 * i] == 0) ni -= 1;
        if (g->bcs[2 * i + 1] == 0) ni -= 1;
        const double dsi = g->ds[i];
        const double emin = 4 * sin(1 * ORA_PI / 2 / (ni + 1)) * sin(1 * ORA_PI / 2 / (ni + 1)) / (dsi * dsi);
        const double emax = 4 * sin(ni * ORA_PI / 2 / (ni + 1)) * sin(ni * ORA_PI / 2 / (ni + 1)) / (dsi * dsi);
        eigMin += emin;
        eigMax += emax;
    }
    out[0] = eigMin;
    out[1] = eigMax;
}

/* ChebyshevIteration constructor (chebyshevIteration.hpp:22-26). */
void ora_cheb_params(const ora_grid* g, const ora_config* c, double out[3])
{
    double e[2];
    ora_eigen_bounds(g, e);
    const double theta = (e[0] * c->rescale_min + e[1] * c->rescale_max) * 0.5 * (1.0 + c->cheb_eps);
    const double delta = (e[0] * c->rescale_min - e[1] * c->rescale_max) * 0.5;
    out[0] = theta;
    out[1] = delta;
    out[2] = theta / delta;
}

typedef struct {
    double theta, delta, sigma;
    int degree;
    double *Y, *Z, *W;   /* persistent buffers, boundary rows stay zero */
} cheb_t;

static int cheb_init(cheb_t* C, const grid_t* G, const ora_grid* g, const ora_config* c)
{
    double p[3];
    ora_cheb_params(g, c, p);
    C->theta = p[0]; C->delta = p[1]; C->sigma = p[2];
    C->degree = c->cheb_degree;
    C->Y = (double*)calloc((size_t)G->ntot, sizeof(double));
    C->Z = (double*)calloc((size_t)G->ntot, sizeof(double));
    C->W = (double*)calloc((size_t)G->ntot, sizeof(double));
    return (C->Y && C->Z && C->W) ? 0 : -1;
}

static void cheb_free(cheb_t* C)
{
    free(C->Y); free(C->Z); free(C->W);
}

/* ChebyshevIteration::operator() with isMainLoop == false, communicationOFF
 * (chebyshevIteration.hpp:48-140). Returns X = -W, where W ends up holding s_{n-2}. */
static void cheb_apply(const grid_t* G, cheb_t* C, double* B, double* X)
{
    const double theta = C->theta, delta = C->delta, sigma = C->sigma;
    double rhoOld = 1 / sigma;
    double rhoCurr = 1 / (2 * sigma - rhoOld);
    reset_neumann(G, B, 0, NULL, 1.0);
    {
        double* Y = C->Y; double* Z = C->Z;
        const double rc = rhoCurr;
        FOR_UNKNOWNS_PAR(G, {
            Z[c] = B[c] / theta;
            Y[c] = 2 * rc / delta * (2 * B[c] + opA(G, B, c) / theta);
        });
    }
    for (int it = 2; it <= C->degree; it++) {
        rhoOld = rhoCurr;
        rhoCurr = 1 / (2 * sigma - rhoOld);
        reset_neumann(G, C->Y, 0, NULL, 1.0);
        {
            double* Y = C->Y; double* Z = C->Z; double* W = C->W;
            const double rc = rhoCurr, ro = rhoOld;
            FOR_UNKNOWNS_PAR(G, {
                W[c] = rc * (2 * sigma * Y[c] + 2 / delta * (B[c] + opA(G, Y, c)) - ro * Z[c]);
            });
        }
        /* std::swap(fieldZ,fieldY); std::swap(fieldW,fieldY); */
        double* t = C->Z; C->Z = C->Y; C->Y = t;
        t = C->W; C->W = C->Y; C->Y = t;
    }
    {
        double* W = C->W;
        FOR_UNKNOWNS_PAR(G, { X[c] = (-1) * W[c]; });
    }
}

/* The seven work fields of one BiCGSTAB object (BiCGSTAB.hpp:23-37). */
typedef struct {
    double *pk, *rk, *r0, *Mpk, *AMpk, *zk, *Azk;
} bicg_t;

static int bicg_alloc(bicg_t* W, const grid_t* G)
{
    const size_t nb = sizeof(double) * (size_t)G->ntot;
    W->pk = (double*)calloc(1, nb); W->rk = (double*)calloc(1, nb); W->r0 = (double*)calloc(1, nb);
    W->Mpk = (double*)calloc(1, nb); W->AMpk = (double*)calloc(1, nb);
    W->zk = (double*)calloc(1, nb); W->Azk = (double*)calloc(1, nb);
    return (W->pk && W->rk && W->r0 && W->Mpk && W->AMpk && W->zk && W->Azk) ? 0 : -1;
}

static void bicg_free(bicg_t* W)
{
    free(W->pk); free(W->rk); free(W->r0); free(W->Mpk); free(W->AMpk); free(W->zk); free(W->Azk);
}

/* A preconditioner object: the T_Preconditioner template argument of a solver
 * (inputParam.hpp:24-33).  Kinds ORA_PREC_BICGSTAB and ORA_PREC_CG are a BiCGSTAB or
 * BaseCG object with isMainLoop == false and communicationOFF, whose own
 * preconditioner is `inner` (the CG one uses pk, rk, AMpk as Apk and zk of W). */
typedef struct prec_s prec_t;
struct prec_s {
    int kind;
    cheb_t C;            /* ORA_PREC_CHEBYSHEV */
    bicg_t W;            /* inner solver: its work fields */
    prec_t* inner;       /* inner solver: its preconditioner (none or Chebyshev) */
    double toll;         /* inner solver: toll_ (tolerance * tollScalingFactor) */
    int maxit;           /* inner solver: maxIteration */
    long iterations;     /* inner solver: iterations, summed over applications */
};

static void precond_apply(const grid_t* G, prec_t* P, double* B, double* X);

/* The iteration loop of BiCGSTAB::operator() (BiCGSTAB.hpp:131-292).  On entry rk,
 * pk and r0 hold the initial residual and x the initial iterate; P is the solver's
 * preconditioner.  hist (main loop only) receives the recursive norms. */
static int bicgstab_loop(const grid_t* G, prec_t* P, bicg_t* W, double* x, double toll, int maxit,
                         double* hist, double* err_iter)
{
    double* pk = W->pk; double* rk = W->rk; double* r0 = W->r0; double* Mpk = W->Mpk;
    double* AMpk = W->AMpk; double* zk = W->zk; double* Azk = W->Azk;
    double alphak = 1, betak = 1, omegak = 1, rho0 = 1, rho1 = 1;
    double pSum1, pSum2;
    int iter = 0;
    while (iter < maxit) {
        precond_apply(G, P, pk, Mpk);
        reset_neumann(G, Mpk, 0, NULL, 1.0);
        FOR_UNKNOWNS_PAR(G, { AMpk[c] = opA(G, Mpk, c); });
        pSum2 = dot_serial(G, r0, AMpk);
        alphak = rho0 / pSum2;
        {
            const double a = alphak;
            FOR_UNKNOWNS_PAR(G, { rk[c] = rk[c] - a * AMpk[c]; });
        }
        precond_apply(G, P, rk, zk);
        reset_neumann(G, zk, 0, NULL, 1.0);
        FOR_UNKNOWNS_PAR(G, { Azk[c] = opA(G, zk, c); });
        dot2_serial(G, rk, Azk, Azk, Azk, &pSum1, &pSum2);
        omegak = pSum1 / pSum2;
        {
            const double a = alphak, w = omegak;
            FOR_ALL_PAR(G, { x[c] = x[c] + a * Mpk[c] + w * zk[c]; });
            FOR_UNKNOWNS_PAR(G, { rk[c] = rk[c] - w * Azk[c]; });
        }
        dot2_serial(G, r0, rk, rk, rk, &pSum1, &pSum2);
        *err_iter = sqrt(pSum2);
        rho1 = pSum1;
        betak = rho1 / rho0 * alphak / omegak;
        rho0 = rho1;
        {
            const double be = betak, w = omegak;
            FOR_UNKNOWNS_PAR(G, { pk[c] = rk[c] + be * (pk[c] - w * AMpk[c]); });
        }
        iter++;
        if (hist) hist[iter] = *err_iter;
        if (hist && G->stamps) G->stamps[iter] = now_s();
        if (*err_iter < toll) break;
    }
    return iter;
}

static void zero_work(const grid_t* G, bicg_t* W)
{
    const size_t nb = sizeof(double) * (size_t)G->ntot;
    memset(W->pk, 0, nb); memset(W->rk, 0, nb); memset(W->r0, 0, nb); memset(W->Mpk, 0, nb);
    memset(W->AMpk, 0, nb); memset(W->zk, 0, nb); memset(W->Azk, 0, nb);
}

/* BiCGSTAB::operator() as a preconditioner: isMainLoop == false, communicationOFF
 * (BiCGSTAB.hpp:55-322).  X = 0; B is normalised in place by its own norm over the
 * unknowns (normalizeProblemToFieldBNorm<false>, iterativeSolverBase.hpp:171-234, no
 * boundary adjustment); the loop runs to toll on that system; X and B are scaled
 * back at the end, so B comes back as (B / n) * n. */
static void bicg_precond(const grid_t* G, prec_t* P, double* B, double* X)
{
    bicg_t* W = &P->W;
    zero_work(G, W);                                              /* :60-66 */
    memset(X, 0, sizeof(double) * (size_t)G->ntot);              /* :94-97 */
    const double normb = sqrt(dot_serial(G, B, B));
    FOR_ALL_PAR(G, { X[c] /= normb; B[c] /= normb; });
    /* computeErrorOperatorA<false,...>: resetNeumanBCs<false,true> is the mirror copy */
    reset_neumann(G, X, 0, NULL, 1.0);
    {
        double* rk = W->rk;
        FOR_UNKNOWNS_PAR(G, { rk[c] = B[c] - opA(G, X, c); });
    }
    const double errC = sqrt(dot_serial(G, W->rk, W->rk));
    if (errC < P->toll) return;          /* :117-121: X and B stay normalised */
    const size_t nb = sizeof(double) * (size_t)G->ntot;
    memcpy(W->pk, W->rk, nb);
    memcpy(W->r0, W->rk, nb);
    double err = 0;
    P->iterations += bicgstab_loop(G, P->inner, W, X, P->toll, P->maxit, NULL, &err);
    reset_neumann(G, X, 0, NULL, 1.0);
    FOR_ALL_PAR(G, { X[c] *= normb; B[c] *= normb; });
}

/* The iteration loop of BaseCG::operator() (baseCG.hpp:115-228).  On entry rk holds
 * the initial residual, zk its preconditioned value and pk = zk.  orderNeumanBcs ==
 * 2, so the reference skips its Neumann resets inside this loop (baseCG.hpp:123-124,
 * 237-238). */
static int cg_loop(const grid_t* G, prec_t* P, double* pk, double* rk, double* Apk, double* zk, double* x,
                   double toll, int maxit, double* hist, double* err_iter)
{
    double alphak = 1, betak = 1, pSum1, pSum2, pSumRk;
    int iter = 0;
    while (iter < maxit) {
        FOR_UNKNOWNS_PAR(G, { Apk[c] = opA(G, pk, c); });
        dot2_serial(G, rk, zk, pk, Apk, &pSum1, &pSum2);
        alphak = pSum1 / pSum2;
        {
            const double a = alphak;
            FOR_UNKNOWNS_PAR(G, {
                x[c] = x[c] + a * pk[c];
                rk[c] = rk[c] - a * Apk[c];
            });
        }
        precond_apply(G, P, rk, zk);
        dot2_serial(G, rk, zk, rk, rk, &pSum2, &pSumRk);
        betak = pSum2 / pSum1;
        *err_iter = sqrt(pSumRk);
        {
            const double be = betak;
            FOR_UNKNOWNS_PAR(G, { pk[c] = zk[c] + be * pk[c]; });
        }
        iter++;
        if (hist) hist[iter] = *err_iter;
        if (*err_iter < toll) break;
    }
    return iter;
}

/* BaseCG::operator() as a preconditioner: isMainLoop == false, communicationOFF
 * (baseCG.hpp:44-260, composed at inputParam.hpp:29).  As bicg_precond, except
 * that z = M r and p = z start the loop and X gets no Neumann reset at the end. */
static void cg_precond(const grid_t* G, prec_t* P, double* B, double* X)
{
    bicg_t* W = &P->W;
    const size_t nb = sizeof(double) * (size_t)G->ntot;
    memset(W->pk, 0, nb); memset(W->rk, 0, nb); memset(W->AMpk, 0, nb); memset(W->zk, 0, nb);  /* :49-52 */
    memset(X, 0, nb);                                                                           /* :81-84 */
    const double normb = sqrt(dot_serial(G, B, B));
    FOR_ALL_PAR(G, { X[c] /= normb; B[c] /= normb; });
    reset_neumann(G, X, 0, NULL, 1.0);
    {
        double* rk = W->rk;
        FOR_UNKNOWNS_PAR(G, { rk[c] = B[c] - opA(G, X, c); });
    }
    const double errC = sqrt(dot_serial(G, W->rk, W->rk));
    if (errC < P->toll) return;          /* :104-108: X and B stay normalised */
    precond_apply(G, P->inner, W->rk, W->zk);
    memcpy(W->pk, W->zk, nb);
    double err = 0;
    P->iterations += cg_loop(G, P->inner, W->pk, W->rk, W->AMpk, W->zk, X, P->toll, P->maxit, NULL, &err);
    FOR_ALL_PAR(G, { X[c] *= normb; B[c] *= normb; });
}

static void precond_apply(const grid_t* G, prec_t* P, double* B, double* X)
{
    if (P->kind == ORA_PREC_CHEBYSHEV) cheb_apply(G, &P->C, B, X);
    else if (P->kind == ORA_PREC_BICGSTAB) bicg_precond(G, P, B, X);
    else if (P->kind == ORA_PREC_CG) cg_precond(G, P, B, X);
    else memcpy(X, B, sizeof(double) * (size_t)G->ntot);   /* NoneSolver */
}

/* BiCGSTAB::operator() main loop (BiCGSTAB.hpp:55-322). */
static int solve_bicgstab(const grid_t* G, const ora_config* cf, prec_t* P, double* x, double* b,
                          const double* const* neumann, double* hist, ora_stats* st)
{
    bicg_t W;
    if (bicg_alloc(&W, G) != 0) { bicg_free(&W); return -1; }
    const size_t nb = sizeof(double) * (size_t)G->ntot;
    const double toll = cf->tol;

    reset_neumann(G, x, 1, neumann, 1.0);              /* normFieldB_ is 1 here */
    const double normb = normalize(G, x, b, neumann);
    st->norm_b = normb;
    st->err_true = true_residual(G, x, b, W.rk, neumann, normb);
    if (hist) hist[0] = st->err_true;
    st->err_iter = -1.0;
    st->iterations = 0;
    st->seconds_loop = 0.0;
    if (st->err_true < toll) {
        /* The reference returns here without undoing the normalisation. */
        bicg_free(&W);
        return 0;
    }
    memcpy(W.pk, W.rk, nb);
    memcpy(W.r0, W.rk, nb);
    const double t0 = now_s();
    st->iterations = bicgstab_loop(G, P, &W, x, toll, cf->maxit, hist, &st->err_iter);
    reset_neumann(G, x, 1, neumann, normb);
    st->seconds_loop = now_s() - t0;
    st->err_true = true_residual(G, x, b, W.rk, neumann, normb);
    FOR_ALL_PAR(G, { x[c] *= normb; b[c] *= normb; });
    bicg_free(&W);
    return 0;
}

/* BaseCG::operator() main loop (baseCG.hpp:44-260). */
static int solve_cg(const grid_t* G, const ora_config* cf, prec_t* P, double* x, double* b,
                    const double* const* neumann, double* hist, ora_stats* st)
{
    const size_t nb = sizeof(double) * (size_t)G->ntot;
    double* pk = (double*)calloc(1, nb);
    double* rk = (double*)calloc(1, nb);
    double* Apk = (double*)calloc(1, nb);
    double* zk = (double*)calloc(1, nb);
    if (!pk || !rk || !Apk || !zk) { free(pk); free(rk); free(Apk); free(zk); return -1; }
    const double toll = cf->tol;

    reset_neumann(G, x, 1, neumann, 1.0);
    const double normb = normalize(G, x, b, neumann);
    st->norm_b = normb;
    st->err_true = true_residual(G, x, b, rk, neumann, normb);
    if (hist) hist[0] = st->err_true;
    st->err_iter = -1.0;
    st->iterations = 0;
    st->seconds_loop = 0.0;
    if (st->err_true < toll) goto out;

    precond_apply(G, P, rk, zk);
    memcpy(pk, zk, nb);
    {
        const double t0 = now_s();
        st->iterations = cg_loop(G, P, pk, rk, Apk, zk, x, toll, cf->maxit, hist, &st->err_iter);
        st->seconds_loop = now_s() - t0;
    }
    st->err_true = true_residual(G, x, b, rk, neumann, normb);
    FOR_ALL_PAR(G, { x[c] *= normb; b[c] *= normb; });
out:
    free(pk); free(rk); free(Apk); free(zk);
    return 0;
}

/* ChebyshevIteration::operator() as the main solver: isMainLoop == true
 * (chebyshevIteration.hpp:48-140).  A copy of b is adjusted for the boundary data
 * and the polynomial of degree maxIteration is applied to it, overwriting x at the
 * unknowns (the initial guess is not used); there is no convergence test and no
 * normalisation (normFieldB_ stays 1), so both errors are the absolute true
 * residual ||b - A x||.  norm_b is reported for the caller only. */
static int solve_cheb_main(const grid_t* G, const ora_config* cf, cheb_t* C, double* x, double* b,
                           const double* const* neumann, ora_stats* st)
{
    const size_t nb = sizeof(double) * (size_t)G->ntot;
    double* bt = (double*)malloc(nb);
    double* r = (double*)calloc(1, nb);
    if (!bt || !r) { free(bt); free(r); return -1; }
    memcpy(bt, b, nb);
    adjust_b(G, x, bt, neumann);
    st->norm_b = sqrt(dot_serial(G, bt, bt));
    const double t0 = now_s();
    cheb_apply(G, C, bt, x);
    st->seconds_loop = now_s() - t0;
    st->err_true = true_residual(G, x, b, r, neumann, 1.0);
    st->err_iter = st->err_true;
    st->iterations = cf->cheb_degree;
    free(bt);
    free(r);
    return 0;
}

static int prec_init(prec_t* P, int kind, const grid_t* G, const ora_grid* g, const ora_config* c)
{
    memset(P, 0, sizeof(*P));
    P->kind = kind;
    if (kind == ORA_PREC_CHEBYSHEV) return cheb_init(&P->C, G, g, c);
    return 0;
}

static void prec_free(prec_t* P)
{
    if (P->kind == ORA_PREC_CHEBYSHEV) cheb_free(&P->C);
    if (P->kind == ORA_PREC_BICGSTAB || P->kind == ORA_PREC_CG) bicg_free(&P->W);
}

static int solve_impl(const ora_grid* g, const ora_config* c, double* x, double* b,
                      const double* const* neumann, double* history, ora_stats* st, double* stamps)
{
    grid_t G;
    if (!g || !c || !x || !b || !st) return -1;
    if (make_grid(g, c->threads, &G) != 0) return -1;
    G.stamps = stamps;
    if (c->maxit < 0 || c->cheb_degree < 1) return -1;
    if (c->krylov != ORA_BICGSTAB && c->krylov != ORA_CG && c->krylov != ORA_CHEBYSHEV_MAIN) return -1;
    if (c->precond < ORA_PREC_NONE || c->precond > ORA_PREC_CG) return -1;
    const int nested = c->precond == ORA_PREC_BICGSTAB || c->precond == ORA_PREC_CG;
    if (nested &&
        (c->prec_maxit < 0 || (c->prec_inner != ORA_PREC_NONE && c->prec_inner != ORA_PREC_CHEBYSHEV)))
        return -1;
    const double t0 = now_s();
    int rc = 0;
    memset(st, 0, sizeof(*st));
    if (c->krylov == ORA_CHEBYSHEV_MAIN) {
        cheb_t C;
        if (cheb_init(&C, &G, g, c) != 0) { cheb_free(&C); return -1; }
        rc = solve_cheb_main(&G, c, &C, x, b, neumann, st);
        cheb_free(&C);
        st->seconds_total = now_s() - t0;
        return rc;
    }
    prec_t P, Pin;
    const int kind = c->precond;
    if (prec_init(&P, kind, &G, g, c) != 0) { prec_free(&P); return -1; }
    if (nested) {
        if (prec_init(&Pin, c->prec_inner, &G, g, c) != 0 || bicg_alloc(&P.W, &G) != 0) {
            prec_free(&Pin); prec_free(&P); return -1;
        }
        P.inner = &Pin;
        P.toll = c->prec_tol;
        P.maxit = c->prec_maxit;
    }
    rc = c->krylov == ORA_BICGSTAB ? solve_bicgstab(&G, c, &P, x, b, neumann, history, st)
                                   : solve_cg(&G, c, &P, x, b, neumann, history, st);
    st->prec_iterations = (int)P.iterations;
    if (nested) prec_free(&Pin);
    prec_free(&P);
    st->seconds_total = now_s() - t0;
    return rc;
}

int ora_solve(const ora_grid* g, const ora_config* c, double* x, double* b,
              const double* const* neumann, double* history, ora_stats* st)
{
    return solve_impl(g, c, x, b, neumann, history, st, NULL);
}

int ora_solve_stamped(const ora_grid* g, const ora_config* c, double* x, double* b,
                      const double* const* neumann, double* history, ora_stats* st, double* stamps)
{
    if (!stamps || !history || c == NULL || c->krylov != ORA_BICGSTAB) return -1;
    stamps[0] = now_s();
    const int rc = solve_impl(g, c, x, b, neumann, history, st, stamps);
    if (rc == 0) stamps[st->iterations + 1] = now_s();
    return rc;
}

void ora_apply_A(const ora_grid* g, const double* u, double* out)
{
    grid_t Gs;
    if (make_grid(g, 1, &Gs) != 0) return;
    const grid_t* G = &Gs;
    FOR_UNKNOWNS_PAR(G, { out[c] = opA(G, u, c); });
}

void ora_cheb_apply(const ora_grid* g, const ora_config* c, double* B, double* X)
{
    grid_t G;
    cheb_t C;
    if (make_grid(g, c->threads, &G) != 0) return;
    if (cheb_init(&C, &G, g, c) != 0) return;
    cheb_apply(&G, &C, B, X);
    cheb_free(&C);
}

double ora_dot(const ora_grid* g, const double* a, const double* b)
{
    grid_t G;
    if (make_grid(g, 1, &G) != 0) return NAN;
    return dot_serial(&G, a, b);
}

/* ---- built-in manufactured problems (solverSetup.hpp:94-161 for problem 0) ---- */

static double prob_f(int p, double x, double y, double z)
{
    if (p == 0) return -sin(x) - cos(y) - 3 * sin(z) + 2 * y * z + 2;
    return -3 * ORA_PI * ORA_PI * sin(ORA_PI * x) * sin(ORA_PI * y) * sin(ORA_PI * z);
}

static double prob_u(int p, double x, double y, double z)
{
    if (p == 0) return sin(x) + cos(y) + 3 * sin(z) + x * x * y * z + x * x + 10;
    return sin(ORA_PI * x) * sin(ORA_PI * y) * sin(ORA_PI * z);
}

static double prob_du(int p, int dir, double x, double y, double z)
{
    if (p == 0) {
        if (dir == 0) return cos(x) + 2 * x * y * z + 2 * x;
        if (dir == 1) return -sin(y) + x * x * z;
        return 3 * cos(z) + x * x * y;
    }
    if (dir == 0) return ORA_PI * cos(ORA_PI * x) * sin(ORA_PI * y) * sin(ORA_PI * z);
    if (dir == 1) return ORA_PI * sin(ORA_PI * x) * cos(ORA_PI * y) * sin(ORA_PI * z);
    return ORA_PI * sin(ORA_PI * x) * sin(ORA_PI * y) * cos(ORA_PI * z);
}

/* Coordinates of data node (i,j,k) at rank location 0 (iterativeSolverBase.hpp:547-549). */
static void coords(const grid_t* G, int i, int j, int k, double* x, double* y, double* z)
{
    *x = G->origin[0] + (i - G->dlo[0]) * G->ds[0] + 0 * (G->n[0]) * G->ds[0];
    *y = G->origin[1] + (j - G->dlo[1]) * G->ds[1] + 0 * (G->n[1]) * G->ds[1];
    *z = G->origin[2] + (k - G->dlo[2]) * G->ds[2] + 0 * (G->n[2]) * G->ds[2];
}

int ora_set_problem(const ora_grid* g, int problem, double* x, double* b, double* const* neumann)
{
    grid_t G;
    if (make_grid(g, 1, &G) != 0 || (problem != 0 && problem != 1)) return -1;
    /* applyDirichletBCsFromFunction (iterativeSolverBase.hpp:557-603) */
    for (int f = 0; f < 6; f++) {
        if (G.bcs[f] != 0) continue;
        face_t F = face_range(&G, f);
        for (int k = F.lo[2]; k < F.hi[2]; k++)
            for (int j = F.lo[1]; j < F.hi[1]; j++)
                for (int i = F.lo[0]; i < F.hi[0]; i++) {
                    double cx, cy, cz;
                    coords(&G, i, j, k, &cx, &cy, &cz);
                    x[i + G.sj * j + G.sk * k] = prob_u(problem, cx, cy, cz);
                }
    }
    /* setFieldValuefromFunction (iterativeSolverBase.hpp:537-555) */
    for (int k = G.dlo[2]; k < G.dhi[2]; k++)
        for (int j = G.dlo[1]; j < G.dhi[1]; j++)
            for (int i = G.dlo[0]; i < G.dhi[0]; i++) {
                double cx, cy, cz;
                coords(&G, i, j, k, &cx, &cy, &cz);
                b[i + G.sj * j + G.sk * k] = prob_f(problem, cx, cy, cz);
            }
    if (neumann) {
        for (int f = 0; f < 6; f++) {
            if (G.bcs[f] != 1 || !neumann[f]) continue;
            face_t F = face_range(&G, f);
            for (int k = F.lo[2]; k < F.hi[2]; k++)
                for (int j = F.lo[1]; j < F.hi[1]; j++)
                    for (int i = F.lo[0]; i < F.hi[0]; i++) {
                        double cx, cy, cz;
                        coords(&G, i, j, k, &cx, &cy, &cz);
                        neumann[f][face_index(&G, F.dir, i, j, k)] = prob_du(problem, F.dir, cx, cy, cz);
                    }
        }
    }
    return 0;
}

int ora_exact_solution(const ora_grid* g, int problem, double* u)
{
    grid_t G;
    if (make_grid(g, 1, &G) != 0 || (problem != 0 && problem != 1)) return -1;
    for (int k = G.dlo[2]; k < G.dhi[2]; k++)
        for (int j = G.dlo[1]; j < G.dhi[1]; j++)
            for (int i = G.dlo[0]; i < G.dhi[0]; i++) {
                double cx, cy, cz;
                coords(&G, i, j, k, &cx, &cy, &cz);
                u[i + G.sj * j + G.sk * k] = prob_u(problem, cx, cy, cz);
            }
    return 0;
}
