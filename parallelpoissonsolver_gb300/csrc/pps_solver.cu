// Solver objects and the C ABI of libpps (include/pps.h).
//
// One pps_solver is the GPU counterpart of one reference solver object
// (BiCGSTAB<...,ChebyshevIteration<...>> composed in inputParam.hpp:33): it owns
// its device work fields, the Chebyshev parameters, a CUDA stream and the
// device-resident Krylov scalars.  Three forms share the same object:
//   PARITY_FP64  host-driven loop over the par_* kernels, scalars on the host in
//                the reference's order, serial device sums -> bit-identical.
//   FP64         device-driven loop over the fast kernels (scalars on device,
//                optional CUDA-graph replay, host polls a stop flag).
//   MIXED        FP64 iterative refinement: FP64 true residual on the device,
//                inner BiCGSTAB/CG with FP32 fields and FP64-accurate dots.
#include "../../include/pps.h"
#include "pps_internal.h"
#include "pps_unet_internal.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <type_traits>
#include <functional>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <sys/types.h>
#include <vector>

using namespace pps;

namespace {

thread_local std::string g_last_error;

void set_error(const std::string& m) { g_last_error = m; }

struct CudaFail {
    cudaError_t err;
};

#define CK(call)                                                                              \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess) {                                                              \
            set_error(std::string(#call) + ": " + cudaGetErrorString(e_));                    \
            throw CudaFail{e_};                                                               \
        }                                                                                     \
    } while (0)

const double kPi = 3.141592653589793;

// Built-in manufactured problems (the reference default of solverSetup.hpp:98-160,
// and the sine product used for the 64^3 eigenvector case).
double builtin_f(double x, double y, double z, void* ctx)
{
    const int p = *(const int*)ctx;
    if (p == 0) return -sin(x) - cos(y) - 3 * sin(z) + 2 * y * z + 2;
    return -3 * kPi * kPi * sin(kPi * x) * sin(kPi * y) * sin(kPi * z);
}
double builtin_u(double x, double y, double z, void* ctx)
{
    const int p = *(const int*)ctx;
    if (p == 0) return sin(x) + cos(y) + 3 * sin(z) + x * x * y * z + x * x + 10;
    return sin(kPi * x) * sin(kPi * y) * sin(kPi * z);
}
double builtin_du(double x, double y, double z, int dir, void* ctx)
{
    const int p = *(const int*)ctx;
    if (p == 0) {
        if (dir == 0) return cos(x) + 2 * x * y * z + 2 * x;
        if (dir == 1) return -sin(y) + x * x * z;
        return 3 * cos(z) + x * x * y;
    }
    if (dir == 0) return kPi * cos(kPi * x) * sin(kPi * y) * sin(kPi * z);
    if (dir == 1) return kPi * sin(kPi * x) * cos(kPi * y) * sin(kPi * z);
    return kPi * sin(kPi * x) * sin(kPi * y) * cos(kPi * z);
}

template <typename T>
struct Fields {
    T *p = nullptr, *r = nullptr, *r0 = nullptr, *Mp = nullptr, *AMp = nullptr, *z = nullptr, *Az = nullptr;
    T *Y = nullptr, *Z = nullptr, *W = nullptr, *e = nullptr;
};

}  // namespace

struct pps_solver {
    pps_grid grid;
    pps_config cfg;
    Geo geo;
    Shape shape;        // z-marching kernels other than the Chebyshev ones
    Shape shape_cheb;   // Chebyshev s1 and sweep kernels
    pps_tuning tuning;
    int device = 0;
    cudaStream_t stream = nullptr;
    double eig[2] = {0, 0};
    double theta = 0, delta = 0, sigma = 0;
    long long n_unknowns = 0;

    double* d_x = nullptr;   // device copies of the caller's fields (host-array path)
    double* d_b = nullptr;
    double* d_bt = nullptr;  // parity: adjusted b
    double* d_dot = nullptr; // parity: serial sums
    Fields<double> f64;
    Fields<float> f32;
    DevState* d_st = nullptr;
    DevState* h_st = nullptr;  // pinned
    bool state_mapped = false; // h_st and h_st_in are device-addressable at their host addresses
    bool xnz_mapped = false;   // h_xnz likewise
    double* d_hist = nullptr;
    int hist_cap = 0;
    double* d_partials = nullptr;
    unsigned* d_counter = nullptr;
    double* h_dot = nullptr;   // pinned
    double* d_cells = nullptr; // FP64 form: cells of canonical sums (3 per cell)

    double* d_faces[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    bool has_neumann = false;

    std::vector<double> history;
    pps_stats stats;
    double cheb_rho_curr_first = 0;

    // Parity-form Chebyshev buffers rotate like the reference's member pointers.
    double *pY = nullptr, *pZ = nullptr, *pW = nullptr;

    // The preconditioner the solve applies at this moment: cfg.precond, or, inside
    // the inner solve of PPS_PREC_BICGSTAB / PPS_PREC_CG, cfg.precond_inner.
    int prec_kind = PPS_PREC_CHEBYSHEV;
    // PPS_PREC_BICGSTAB / PPS_PREC_CG: the inner solver's work fields (in the form's precision)
    // and its own Krylov scalars; inner iterations summed over the applications.
    Fields<double> in64;
    Fields<float> in32;
    DevState* d_st_in = nullptr;
    DevState* h_st_in = nullptr;   // pinned
    long long prec_iters = 0;

    // graph cache
    cudaGraphExec_t gexec = nullptr;
    const void* g_key_x = nullptr;
    const void* g_key_b = nullptr;
    int g_iters = 0;
    int g_form = -1;
    double g_bytes = 0;
    int g_launches = 0;
    double g_sweep_bytes = 0;
    int g_sweep_launches = 0;
    bool g_learned = false;   // captured with the learned preconditioner active
    int g_learned_apps = 0;

    // learned preconditioner / initial guess (pps_set_learned)
    pps_unet* net = nullptr;
    int net_coarsen = 0;
    float net_gain = 1.0f;
    int net_flags = 0;
    bool net_active = false;          // preconditioner in use in the current solve (fallback clears it)
    std::vector<float*> dn;           // dense levels 0..k of the network correction (residual, correction); level 0 only for k = 0
    std::vector<float*> dn_e;
    int learned_apps = 0;
    int fallback_iter = -1;
    // multigrid form of the learned cycle (pps_set_learned_cycle): smoother degrees
    // of the fine and the coarse levels (fine 0: the two-grid cycle), interval ratio;
    // dt: residuals of levels 1..k-1; cY, cZ, cW: Chebyshev buffers of those levels
    int cyc_fine = 0, cyc_coarse = 0;
    double cyc_ratio = 8.0;
    std::vector<float*> dt;
    float *cY = nullptr, *cZ = nullptr, *cW = nullptr;
    // coarsest-level solver of the cycle (pps_set_coarse_solver); d_exact: the
    // eigen-solve's matrices for PPS_COARSE_EXACT
    int coarse_kind = PPS_COARSE_NETWORK;
    float* d_exact = nullptr;

    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // pps_solve on pinned host arrays, MIXED form: b is uploaded first and the solve
    // starts on it as if x were zero, while x uploads on copy_stream and
    // k_flag_nonzero tests it (ev_x: x resident, *h_xnz valid).  spec_x: that test is
    // still unread; the solve reads or writes x only after it (a non-zero x restarts
    // the solve on it).  out_host: after each update of x, copy_stream copies it to
    // this host array (ev_out: done); out_current: the last such copy holds the final x.
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev_h0 = nullptr, ev_b = nullptr, ev_x = nullptr, ev_upd = nullptr, ev_out = nullptr;
    int* d_xnz = nullptr;
    int* h_xnz = nullptr;   // pinned
    bool spec_x = false;
    bool spec_restarted = false;
    double* out_host = nullptr;
    bool out_issued = false;
    bool out_current = false;
    std::vector<cudaEvent_t> sweep_ev;   // pairs, profiling of sweeps
    std::vector<cudaEvent_t> krylov_ev;  // pairs, profiling of flexible CG's direction + update kernels
    int krylov_ev_used = 0;
    double krylov_bytes_acc = 0;
    int krylov_launch_acc = 0;
    int sweep_ev_used = 0;
    double bytes_acc = 0;
    int launches_acc = 0;
    double sweep_bytes_acc = 0;
    int sweep_launch_acc = 0;
};

namespace {

Faces faces_of(const pps_solver* s)
{
    Faces f;
    for (int i = 0; i < 6; i++) f.g[i] = s->d_faces[i];
    return f;
}

RedCtx red(pps_solver* s, int kind)
{
    RedCtx rc;
    rc.partials = s->d_partials;
    rc.counter = s->d_counter;
    rc.st = s->d_st;
    rc.hist = s->d_hist;
    rc.kind = kind;
    return rc;
}

// The sums of the reference methods (BiCGSTAB, CG, their start and the true
// residual) in the FP64 form are canonical: one partial per fixed cell of the grid,
// summed in a fixed tree, so the iterates, the iteration count and the residual
// history depend on the grid and the data alone -- not on the tiles pps_autotune
// picks nor on the GPU's SM count.  The other forms keep the block reduction.
RedCtx red_c(pps_solver* s, int kind)
{
    RedCtx rc = red(s, kind);
    rc.cells = s->d_cells;
    return rc;
}

// A(u) = cc*u + c_d*(pairs) with c_d = 1/h_d^2  (matrixFreeOperatorA.hpp:34-38)
Coef op_coef_ds(const double ds[3])
{
    Coef c;
    const double ix = 1.0 / (ds[0] * ds[0]), iy = 1.0 / (ds[1] * ds[1]), iz = 1.0 / (ds[2] * ds[2]);
    c.cc = -2.0 * (ix + iy + iz);
    c.cx = ix;
    c.cy = iy;
    c.cz = iz;
    c.cb = 0;
    c.cw = 0;
    c.scale = 1.0;
    return c;
}

Coef op_coef(const Geo& g)
{
    return op_coef_ds(g.ds);
}

long long face_count(const pps_solver* s, int f)
{
    const int d = f / 2;
    const int* n = s->grid.npglobal;
    if (d == 0) return (long long)n[1] * n[2];
    if (d == 1) return (long long)n[0] * n[2];
    return (long long)n[0] * n[1];
}

template <typename T>
void alloc_fields(Fields<T>& F, long long ntot, bool with_e, bool with_cheb = true)
{
    T** all[] = {&F.p, &F.r, &F.r0, &F.Mp, &F.AMp, &F.z, &F.Az, &F.Y, &F.Z, &F.W};
    for (T** q : all) {
        if (!with_cheb && (q == &F.Y || q == &F.Z || q == &F.W)) continue;
        CK(cudaMalloc((void**)q, sizeof(T) * (size_t)ntot));
        CK(cudaMemset(*q, 0, sizeof(T) * (size_t)ntot));
    }
    if (with_e) {
        CK(cudaMalloc((void**)&F.e, sizeof(T) * (size_t)ntot));
        CK(cudaMemset(F.e, 0, sizeof(T) * (size_t)ntot));
    }
}

template <typename T>
void free_fields(Fields<T>& F)
{
    T* all[] = {F.p, F.r, F.r0, F.Mp, F.AMp, F.z, F.Az, F.Y, F.Z, F.W, F.e};
    for (T* q : all)
        if (q) cudaFree(q);
    F = Fields<T>();
}

template <typename T>
void zero_fields(Fields<T>& F, long long ntot, cudaStream_t st)
{
    T* all[] = {F.p, F.r, F.r0, F.Mp, F.AMp, F.z, F.Az};
    for (T* q : all) CK(cudaMemsetAsync(q, 0, sizeof(T) * (size_t)ntot, st));
}

void free_all(pps_solver* s)
{
    if (s->gexec) cudaGraphExecDestroy(s->gexec);
    free_fields(s->f64);
    free_fields(s->f32);
    free_fields(s->in64);
    free_fields(s->in32);
    void* ptrs[] = {s->d_x, s->d_b, s->d_bt, s->d_dot, s->d_st, s->d_hist, s->d_partials, s->d_counter, s->d_st_in,
                    s->d_cells};
    for (void* q : ptrs)
        if (q) cudaFree(q);
    if (s->h_st_in) cudaFreeHost(s->h_st_in);
    for (int i = 0; i < 6; i++)
        if (s->d_faces[i]) cudaFree(s->d_faces[i]);
    if (s->h_st) cudaFreeHost(s->h_st);
    if (s->h_dot) cudaFreeHost(s->h_dot);
    for (float* q : s->dn) cudaFree(q);
    for (float* q : s->dn_e) cudaFree(q);
    for (float* q : s->dt) cudaFree(q);
    for (float* q : {s->cY, s->cZ, s->cW, s->d_exact}) cudaFree(q);
    for (cudaEvent_t e : s->sweep_ev) cudaEventDestroy(e);
    for (cudaEvent_t e : s->krylov_ev) cudaEventDestroy(e);
    if (s->ev0) cudaEventDestroy(s->ev0);
    if (s->ev1) cudaEventDestroy(s->ev1);
    for (cudaEvent_t e : {s->ev_h0, s->ev_b, s->ev_x, s->ev_upd, s->ev_out})
        if (e) cudaEventDestroy(e);
    if (s->d_xnz) cudaFree(s->d_xnz);
    if (s->h_xnz) cudaFreeHost(s->h_xnz);
    if (s->copy_stream) cudaStreamDestroy(s->copy_stream);
    if (s->stream) cudaStreamDestroy(s->stream);
}

// ---------------------------------------------------------------------------
// PARITY form: the reference's loop with the par_* kernels
// ---------------------------------------------------------------------------

double par_dot(pps_solver* s, const double* a, const double* b)
{
    seq_dot2(s->geo, a, b, nullptr, nullptr, s->d_dot, s->stream);
    CK(cudaMemcpyAsync(s->h_dot, s->d_dot, 2 * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return s->h_dot[0];
}

void par_dot2(pps_solver* s, const double* a1, const double* b1, const double* a2, const double* b2, double* o1,
              double* o2)
{
    seq_dot2(s->geo, a1, b1, a2, b2, s->d_dot, s->stream);
    CK(cudaMemcpyAsync(s->h_dot, s->d_dot, 2 * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    *o1 = s->h_dot[0];
    *o2 = s->h_dot[1];
}

void par_neumann_helper(pps_solver* s, double* f)
{
    if (s->has_neumann) neumann_fill<double>(s->geo, f, faces_of(s), 0, 1.0, s->stream);
}

// While the inner solve of PPS_PREC_BICGSTAB / PPS_PREC_CG runs, the kernels and the
// host polls use its own Krylov scalars, and the preconditioner applied inside it
// is the inner solver's (precond_inner).  Restored when the scope ends.
struct InnerScope {
    pps_solver* s;
    DevState* d;
    DevState* h;
    int kind;
    explicit InnerScope(pps_solver* s_) : s(s_), d(s_->d_st), h(s_->h_st), kind(s_->prec_kind)
    {
        s->d_st = s->d_st_in;
        s->h_st = s->h_st_in;
        s->prec_kind = s->cfg.precond_inner;
    }
    ~InnerScope()
    {
        s->d_st = d;
        s->h_st = h;
        s->prec_kind = kind;
    }
};

void par_bicgstab_precond(pps_solver* s, double* B, double* X);
void par_cg_precond(pps_solver* s, double* B, double* X);

// The preconditioner s->prec_kind names, applied X = M^{-1} B: NoneSolver's copy
// (noneSolver.hpp:23-26), ChebyshevIteration::operator() in preconditioner mode
// (chebyshevIteration.hpp:48-140), or the inner BiCGSTAB solve.
void par_precond(pps_solver* s, double* B, double* X)
{
    const Geo& g = s->geo;
    if (s->prec_kind == PPS_PREC_BICGSTAB) {
        par_bicgstab_precond(s, B, X);
        return;
    }
    if (s->prec_kind == PPS_PREC_CG) {
        par_cg_precond(s, B, X);
        return;
    }
    if (s->prec_kind == PPS_PREC_NONE) {
        CK(cudaMemcpyAsync(X, B, sizeof(double) * (size_t)g.ntot, cudaMemcpyDeviceToDevice, s->stream));
        return;
    }
    const double sigma = s->sigma, delta = s->delta, theta = s->theta;
    double rhoOld = 1 / sigma;
    double rhoCurr = 1 / (2 * sigma - rhoOld);
    par_neumann_helper(s, B);
    par_cheb_s01(g, B, s->pY, s->pZ, theta, 2 * rhoCurr / delta, s->stream);
    for (int it = 2; it <= s->cfg.cheb_degree; it++) {
        rhoOld = rhoCurr;
        rhoCurr = 1 / (2 * sigma - rhoOld);
        par_neumann_helper(s, s->pY);
        par_cheb_sweep(g, s->pY, B, s->pZ, s->pW, rhoCurr, 2 * sigma, 2 / delta, rhoOld, s->stream);
        std::swap(s->pZ, s->pY);
        std::swap(s->pW, s->pY);
    }
    par_neg(g, s->pW, X, s->stream);
}

double par_true_residual(pps_solver* s, double* x, double* b, double* r, double normb)
{
    if (s->has_neumann) neumann_fill<double>(s->geo, x, faces_of(s), 1, normb, s->stream);
    par_residual(s->geo, x, b, r, s->stream);
    return std::sqrt(par_dot(s, r, r));
}

// The iteration loop of BiCGSTAB::operator() (BiCGSTAB.hpp:131-292) with the
// preconditioner s->prec_kind names.  On entry F.r, F.p and F.r0 hold the initial
// residual.  `main` records the history and counts the applications.
int par_bicgstab_loop(pps_solver* s, Fields<double>& F, double* x, double toll, int maxit, bool main,
                      double* err_iter)
{
    const Geo& g = s->geo;
    cudaStream_t st = s->stream;
    double rho0 = 1, rho1 = 1, alphak = 1, omegak = 1, betak = 1, s1 = 0, s2 = 0;
    int iter = 0;
    while (iter < maxit) {
        par_precond(s, F.p, F.Mp);
        par_neumann_helper(s, F.Mp);
        par_stencil(g, F.Mp, F.AMp, st);
        s2 = par_dot(s, F.r0, F.AMp);
        alphak = rho0 / s2;
        par_axpy(g, F.r, F.AMp, alphak, st);
        par_precond(s, F.r, F.z);
        par_neumann_helper(s, F.z);
        if (main) s->stats.precond_applications += 2;
        par_stencil(g, F.z, F.Az, st);
        par_dot2(s, F.r, F.Az, F.Az, F.Az, &s1, &s2);
        omegak = s1 / s2;
        par_update_x_all(g, x, F.Mp, F.z, alphak, omegak, st);
        par_axpy(g, F.r, F.Az, omegak, st);
        par_dot2(s, F.r0, F.r, F.r, F.r, &s1, &s2);
        *err_iter = std::sqrt(s2);
        rho1 = s1;
        betak = rho1 / rho0 * alphak / omegak;
        rho0 = rho1;
        par_update_p(g, F.p, F.r, F.AMp, betak, omegak, st);
        iter++;
        if (main) s->history.push_back(*err_iter);
        if (*err_iter < toll) break;
    }
    return iter;
}

// BiCGSTAB::operator() as a preconditioner: isMainLoop false, communicationOFF
// (BiCGSTAB.hpp:55-322).  X = 0; B is normalised in place by its own norm over the
// unknowns (normalizeProblemToFieldBNorm<false>, iterativeSolverBase.hpp:171-234,
// without boundary adjustment); the loop runs to precond_tol on that system with
// precond_inner as its preconditioner; X and B are scaled back at the end, so B
// returns as (B / n) * n like the reference's.
void par_bicgstab_precond(pps_solver* s, double* B, double* X)
{
    const Geo& g = s->geo;
    Fields<double>& W = s->in64;
    cudaStream_t st = s->stream;
    const size_t fb = sizeof(double) * (size_t)g.ntot;
    zero_fields(W, g.ntot, st);                   // BiCGSTAB.hpp:60-66
    CK(cudaMemsetAsync(X, 0, fb, st));            // :94-97
    const double normb = std::sqrt(par_dot(s, B, B));
    par_scale_all(g, X, B, normb, 1, st);
    par_neumann_helper(s, X);                     // resetNeumanBCs<false,true>: the mirror copy
    par_residual(g, X, B, W.r, st);
    const double errC = std::sqrt(par_dot(s, W.r, W.r));
    if (errC < s->cfg.precond_tol) return;        // :117-121: X and B stay normalised
    CK(cudaMemcpyAsync(W.p, W.r, fb, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(W.r0, W.r, fb, cudaMemcpyDeviceToDevice, st));
    double err = 0;
    {
        InnerScope in(s);
        s->prec_iters += par_bicgstab_loop(s, W, X, s->cfg.precond_tol, s->cfg.precond_maxit, false, &err);
    }
    par_neumann_helper(s, X);
    par_scale_all(g, X, B, normb, 0, st);
}

// The iteration loop of BaseCG::operator() (baseCG.hpp:115-228) with the
// preconditioner s->prec_kind names.  On entry F.r holds the initial residual, F.z
// its preconditioned value and F.p = F.z; F.AMp serves as Apk.  orderNeumanBcs == 2,
// so the loop makes no Neumann resets (baseCG.hpp:123-124, 237-238).
int par_cg_loop(pps_solver* s, Fields<double>& F, double* x, double toll, int maxit, bool main, double* err_iter)
{
    const Geo& g = s->geo;
    cudaStream_t st = s->stream;
    double* zk = F.z;
    double* Apk = F.AMp;
    double alphak = 1, betak = 1, pSum1 = 0, pSum2 = 0, pSumRk = 0;
    int iter = 0;
    while (iter < maxit) {
        par_stencil(g, F.p, Apk, st);
        par_dot2(s, F.r, zk, F.p, Apk, &pSum1, &pSum2);
        alphak = pSum1 / pSum2;
        par_update_x(g, x, F.p, alphak, st);
        par_axpy(g, F.r, Apk, alphak, st);
        par_precond(s, F.r, zk);
        if (main) s->stats.precond_applications++;
        par_dot2(s, F.r, zk, F.r, F.r, &pSum2, &pSumRk);
        betak = pSum2 / pSum1;
        *err_iter = std::sqrt(pSumRk);
        par_update_p_cg(g, F.p, zk, betak, st);
        iter++;
        if (main) s->history.push_back(*err_iter);
        if (*err_iter < toll) break;
    }
    return iter;
}

// BaseCG::operator() as a preconditioner: isMainLoop false, communicationOFF
// (baseCG.hpp:44-260): as par_bicgstab_precond, except that z = M r and p = z start
// the loop and X gets no Neumann reset at the end (orderNeumanBcs == 2).
void par_cg_precond(pps_solver* s, double* B, double* X)
{
    const Geo& g = s->geo;
    Fields<double>& W = s->in64;
    cudaStream_t st = s->stream;
    const size_t fb = sizeof(double) * (size_t)g.ntot;
    zero_fields(W, g.ntot, st);                   // baseCG.hpp:49-52
    CK(cudaMemsetAsync(X, 0, fb, st));            // :81-84
    const double normb = std::sqrt(par_dot(s, B, B));
    par_scale_all(g, X, B, normb, 1, st);
    par_neumann_helper(s, X);
    par_residual(g, X, B, W.r, st);
    const double errC = std::sqrt(par_dot(s, W.r, W.r));
    if (errC < s->cfg.precond_tol) return;        // :104-108: X and B stay normalised
    double err = 0;
    {
        InnerScope in(s);
        par_precond(s, W.r, W.z);
        CK(cudaMemcpyAsync(W.p, W.z, fb, cudaMemcpyDeviceToDevice, st));
        s->prec_iters += par_cg_loop(s, W, X, s->cfg.precond_tol, s->cfg.precond_maxit, false, &err);
    }
    par_scale_all(g, X, B, normb, 0, st);
}

pps_status solve_parity(pps_solver* s, double* x, double* b)
{
    const Geo& g = s->geo;
    Fields<double>& F = s->f64;
    cudaStream_t st = s->stream;
    pps_stats& S = s->stats;
    const double toll = s->cfg.tol;
    zero_fields(F, g.ntot, st);
    s->history.assign(1, -1.0);

    if (s->has_neumann) neumann_fill<double>(g, x, faces_of(s), 1, 1.0, st);
    // normalizeProblemToFieldBNorm (iterativeSolverBase.hpp:171-234)
    par_adjust_b(g, b, x, faces_of(s), s->d_bt, st);
    const double normb = std::sqrt(par_dot(s, s->d_bt, s->d_bt));
    S.norm_b = normb;
    if (!(normb > 0.0)) return PPS_ERR_ZERO_RHS;
    par_scale_all(g, x, b, normb, 1, st);
    double errC = par_true_residual(s, x, b, F.r, normb);
    S.err_true = errC;
    S.err_iter = -1.0;
    s->history[0] = errC;
    S.iterations = 0;
    if (errC < toll) return PPS_OK;   // the reference returns here, x and b still scaled

    CK(cudaMemcpyAsync(F.p, F.r, sizeof(double) * (size_t)g.ntot, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(F.r0, F.r, sizeof(double) * (size_t)g.ntot, cudaMemcpyDeviceToDevice, st));
    int iter = 0;
    if (s->cfg.krylov == PPS_KRYLOV_CG) {
        // BaseCG::operator() (baseCG.hpp:109-228)
        par_precond(s, F.r, F.z);
        S.precond_applications++;
        CK(cudaMemcpyAsync(F.p, F.z, sizeof(double) * (size_t)g.ntot, cudaMemcpyDeviceToDevice, st));
        iter = par_cg_loop(s, F, x, toll, s->cfg.maxit, true, &S.err_iter);
    } else {
        // BiCGSTAB::operator() (BiCGSTAB.hpp:131-292)
        iter = par_bicgstab_loop(s, F, x, toll, s->cfg.maxit, true, &S.err_iter);
        if (s->has_neumann) neumann_fill<double>(g, x, faces_of(s), 1, normb, st);
    }
    S.iterations = iter;
    S.err_true = par_true_residual(s, x, b, F.r, normb);
    par_scale_all(g, x, b, normb, 0, st);
    return iter >= s->cfg.maxit && !(S.err_iter < toll) ? PPS_NOT_CONVERGED : PPS_OK;
}

// ---------------------------------------------------------------------------
// FP64 and MIXED forms: device-driven loops over the fast kernels
// ---------------------------------------------------------------------------

template <typename T>
double bytes_of(long long n, int words)
{
    return (double)n * words * sizeof(T);
}

// A Chebyshev polynomial in the reference's form (chebyshevIteration.hpp:22-26,
// 48-140): interval parameters theta, delta, sigma = theta/delta and degree n;
// the output is -s_{n-2}.
struct ChebP {
    double theta, delta, sigma;
    int n;
};

ChebP cheb_of(const pps_solver* s)
{
    return ChebP{s->theta, s->delta, s->sigma, s->cfg.cheb_degree};
}

// The same recurrence as a smoother on [lambda_max / ratio, lambda_max] of the
// operator with spacings ds (lambda_max = sum_d 4 / ds_d^2, the bound the
// sine formula approaches): the high-frequency part of the spectrum only.
ChebP smoother_of(const double ds[3], double ratio, int n)
{
    double lmax = 0;
    for (int d = 0; d < 3; d++) lmax += 4.0 / (ds[d] * ds[d]);
    const double lo = lmax / ratio;
    ChebP p;
    p.theta = (lo + lmax) * 0.5;
    p.delta = (lo - lmax) * 0.5;
    p.sigma = p.theta / p.delta;
    p.n = n;
    return p;
}

// Pre-folded Chebyshev coefficients for the fast kernels (a: the operator's).
Coef cheb_s01_coef(const Coef& a, const ChebP& p, double rhoCurr)
{
    const double t = 2 * rhoCurr / p.delta;   // Y = t*(2B + A(B)/theta)
    Coef c;
    c.cc = t * (2.0 + a.cc / p.theta);
    c.cx = t * a.cx / p.theta;
    c.cy = t * a.cy / p.theta;
    c.cz = t * a.cz / p.theta;
    c.cb = 0;
    c.cw = 0;
    c.scale = 1.0;
    return c;
}

Coef cheb_sweep_coef(const Coef& a, const ChebP& p, double rhoCurr, double rhoOld, double scale)
{
    const double tod = 2.0 / p.delta;   // W = rc*(2 sigma Y + 2/delta (B + A Y) - ro Z)
    Coef c;
    c.cc = rhoCurr * (2.0 * p.sigma + tod * a.cc);
    c.cx = rhoCurr * tod * a.cx;
    c.cy = rhoCurr * tod * a.cy;
    c.cz = rhoCurr * tod * a.cz;
    c.cb = rhoCurr * tod;
    c.cw = -rhoCurr * rhoOld;
    c.scale = scale;
    return c;
}

struct Launcher {
    pps_solver* s;
    bool profile;
    double bytes = 0;
    int launches = 0;
};

// One preconditioner application X = M^{-1} B in storage type T.  The two last
// sweeps of the reference are dead (its output is s_{n-2}, chebyshevIteration.hpp:
// 114-125), so sweeps run for i = 2..n-2 and the last one writes X = -s_{n-2}.
template <typename T>
void fast_cheb(pps_solver* s, Fields<T>& F, T* B, T* X, Launcher& L, const ChebP& p);

template <typename T>
void fast_inner_precond(pps_solver* s, T* B, T* X, Launcher& L, bool cg);

// The preconditioner s->prec_kind names: the identity, the Chebyshev polynomial,
// or the inner BiCGSTAB solve.
template <typename T>
void fast_precond(pps_solver* s, Fields<T>& F, T* B, T* X, Launcher& L)
{
    const Geo& g = s->geo;
    if (s->prec_kind == PPS_PREC_NONE) {
        CK(cudaMemcpyAsync(X, B, sizeof(T) * (size_t)g.ntot, cudaMemcpyDeviceToDevice, s->stream));
        L.bytes += bytes_of<T>(g.ntot, 2);
        return;
    }
    if (s->prec_kind == PPS_PREC_BICGSTAB || s->prec_kind == PPS_PREC_CG) {
        fast_inner_precond<T>(s, B, X, L, s->prec_kind == PPS_PREC_CG);
        return;
    }
    fast_cheb<T>(s, F, B, X, L, cheb_of(s));
}

// X = -s_{n-2} of the Chebyshev recurrence p on B (the preconditioner, or a smoother).
template <typename T>
void fast_cheb(pps_solver* s, Fields<T>& F, T* B, T* X, Launcher& L, const ChebP& p)
{
    const Geo& g = s->geo;
    cudaStream_t st = s->stream;
    const long long N = s->n_unknowns;
    const int* done = &s->d_st->done;
    if (s->has_neumann) {
        neumann_fill<T>(g, B, faces_of(s), 0, 1.0, st);
        L.launches += 2;
    }
    const Coef a = op_coef(g);
    const int n = p.n;
    const double sigma = p.sigma;
    double rhoOld = 1 / sigma;
    double rhoCurr = 1 / (2 * sigma - rhoOld);
    if (n == 1) {
        fill_field<T>(X, g.ntot, (T)(-0.0), st);
        L.bytes += bytes_of<T>(g.ntot, 1);
        L.launches++;
        return;
    }
    if (n == 2) {
        fast_scale_copy<T>(g, s->shape, B, X, -1.0 / p.theta, done, st);
        L.bytes += bytes_of<T>(N, 2);
        L.launches++;
        return;
    }
    const Shape& shc = s->shape_cheb;
    Coef c01 = cheb_s01_coef(a, p, rhoCurr);
    if (n == 3) {
        c01.scale = -1.0;
        fast_cheb_s01<T>(g, shc, B, X, c01, done, st);
        L.bytes += bytes_of<T>(N, 2);
        L.launches++;
        return;
    }
    if (!s->has_neumann && s->tuning.cheb_fused && (n == 4 || n == 5)) {
        // all n-2 steps in one temporally blocked pass: B read once, X written once
        Coef cs[3];
        cs[0] = c01;
        for (int it = 2; it <= n - 2; it++) {
            rhoOld = rhoCurr;
            rhoCurr = 1 / (2 * sigma - rhoOld);
            Coef c = cheb_sweep_coef(a, p, rhoCurr, rhoOld, it == n - 2 ? -1.0 : 1.0);
            if (it == 2) {
                c.cb += c.cw / p.theta;
                c.cw = 0.0;
            }
            cs[it - 1] = c;
        }
        const bool prof = L.profile && s->sweep_ev_used + 2 <= (int)s->sweep_ev.size();
        if (prof) CK(cudaEventRecord(s->sweep_ev[s->sweep_ev_used], st));
        fast_cheb_fused<T>(g, n - 2, B, X, cs, done, st);
        if (prof) {
            CK(cudaEventRecord(s->sweep_ev[s->sweep_ev_used + 1], st));
            s->sweep_ev_used += 2;
        }
        L.bytes += bytes_of<T>(N, 2);
        L.launches++;
        s->sweep_bytes_acc += bytes_of<T>(N, 2);
        s->sweep_launch_acc++;
        return;
    }
    T* Y = F.Y;
    T* Z = F.Z;
    T* W = F.W;
    fast_cheb_s01<T>(g, shc, B, Y, c01, done, st);
    L.bytes += bytes_of<T>(N, 2);
    L.launches++;
    const bool prof = L.profile && s->sweep_ev_used + 2 <= (int)s->sweep_ev.size();
    if (prof) CK(cudaEventRecord(s->sweep_ev[s->sweep_ev_used], st));
    for (int it = 2; it <= n - 2; it++) {
        rhoOld = rhoCurr;
        rhoCurr = 1 / (2 * sigma - rhoOld);
        if (s->has_neumann) {
            neumann_fill<T>(g, Y, faces_of(s), 0, 1.0, st);
            L.launches += 2;
        }
        const bool last = (it == n - 2);
        Coef c = cheb_sweep_coef(a, p, rhoCurr, rhoOld, last ? -1.0 : 1.0);
        const bool first = (it == 2);
        if (first) {
            // Z = s0 = B/theta: fold it into the B coefficient instead of storing s0
            c.cb += c.cw / p.theta;
            c.cw = 0.0;
        }
        fast_cheb_sweep<T>(g, shc, Y, B, first ? nullptr : Z, last ? X : W, c, done, st);
        const int words = first ? 3 : 4;
        L.bytes += bytes_of<T>(N, words);
        L.launches++;
        s->sweep_bytes_acc += bytes_of<T>(N, words);
        s->sweep_launch_acc++;
        if (!last) {
            T* t = Z;   // (Y, Z, W) <- (W, Y, Z)
            Z = Y;
            Y = W;
            W = t;
        }
    }
    if (prof) {
        CK(cudaEventRecord(s->sweep_ev[s->sweep_ev_used + 1], st));
        s->sweep_ev_used += 2;
    }
}

unet::Dims dense_dims(const pps_solver* s, int level)
{
    const Geo& g = s->geo;
    const int f = 1 << level;
    return unet::Dims{(g.hi[2] - g.lo[2]) / f, (g.hi[1] - g.lo[1]) / f, (g.hi[0] - g.lo[0]) / f};
}

unet::DLevel level_op(const pps_solver* s, int l);
void dense_cheb(pps_solver* s, int l, const float* B, float* X, bool acc);

// The coarsest level's correction z_k from its residual r_k: the network (gain
// N(r_k)), or the alternative pps_set_coarse_solver chose.
void coarse_solve(pps_solver* s, int k, const float* r, float* z)
{
    const unet::Dims dc = dense_dims(s, k);
    switch (s->coarse_kind) {
    case PPS_COARSE_ZERO:
        unet::level_zero(dc, z, s->stream);
        break;
    case PPS_COARSE_SMOOTH:
        dense_cheb(s, k, r, z, false);
        break;
    case PPS_COARSE_EXACT:
        unet::level_exact(dc, s->d_exact, r, z, s->stream);
        break;
    default:
        if (pps_internal_unet_apply(s->net, dc.W, dc.H, dc.D, r, z, s->net_gain, s->stream) != PPS_OK)
            throw CudaFail{cudaErrorUnknown};
    }
}

// X += gain P^k N(R^k (r - A z)) at the unknowns (R^k r when z is null).  For
// coarsen k >= 1 the first restriction reads the solver fields and the last
// prolongation adds into X, so no fine-grid dense array exists; levels 1..k are
// dense arrays dn[l] (restricted residual) and dn_e[l] (correction).
template <typename T>
void learned_coarse_correction(pps_solver* s, const T* r, const T* z, T* X)
{
    const Geo& g = s->geo;
    cudaStream_t st = s->stream;
    const int k = s->net_coarsen;
    if (k == 0) {
        if (z) unet::field_residual_dense<T>(g, r, z, s->dn[0], st);
        else unet::field_to_dense<T>(g, r, s->dn[0], st);
    } else {
        unet::field_residual_restrict<T>(g, r, z, dense_dims(s, 1), s->dn[1], st);
        for (int l = 1; l < k; l++) unet::restrict2(dense_dims(s, l + 1), s->dn[(size_t)l], s->dn[(size_t)l + 1], st);
    }
    coarse_solve(s, k, s->dn[(size_t)k], s->dn_e[(size_t)k]);
    if (k == 0) {
        unet::dense_to_field<T>(g, s->dn_e[0], X, 1.0f, 1, st);
    } else {
        for (int l = k; l > 1; l--) unet::prolong2(dense_dims(s, l), s->dn_e[(size_t)l], s->dn_e[(size_t)l - 1], st);
        unet::prolong_add_field<T>(g, s->shape_cheb, dense_dims(s, 1), s->dn_e[1], X, st);
    }
    s->learned_apps++;
}

// Operator of coarse level l (2^l times the solver's spacing, the upper wall one
// fine spacing above the last unknown of each axis).
unet::DLevel level_op(const pps_solver* s, int l)
{
    unet::DLevel L;
    for (int d = 0; d < 3; d++) {
        const double h = s->geo.ds[d], H = h * (double)(1 << l);
        L.ih2[d] = (float)(1.0 / (H * H));
        L.last_m[d] = (float)(2.0 / (H * (H + h)));
        L.last_c[d] = (float)(-2.0 / (H * h));
    }
    return L;
}

// out = b - A_l z on coarse level l.
void dense_residual(pps_solver* s, int l, const float* b, const float* z, float* out)
{
    unet::level_residual(dense_dims(s, l), level_op(s, l), z, b, out, s->stream);
}

// X (+)= -s_{n-2} on coarse level l: the preconditioner's Chebyshev recurrence applied
// to the Jacobi-scaled operator D^-1 A_l (D = -diag A_l), whose spectrum lies in
// (0, 2]; smoothing interval [2/ratio, 2].  The scaling absorbs the larger diagonal
// of the unknowns next to the upper wall.
void dense_cheb(pps_solver* s, int l, const float* B, float* X, bool acc)
{
    const unet::DLevel L = level_op(s, l);
    const unet::Dims d = dense_dims(s, l);
    cudaStream_t st = s->stream;
    const int n = s->cyc_coarse;
    const double hi = 2.0, lo = 2.0 / s->cyc_ratio;
    const double theta = 0.5 * (lo + hi), delta = 0.5 * (lo - hi), sigma = theta / delta;
    const float y0 = (float)(1.0 / theta);
    if (n == 2) {
        unet::level_cheb(d, L, nullptr, B, nullptr, X, unet::LCoef{1.0f, 0.0f, 0.0f, 0.0f, -1.0f, y0}, true, acc, st);
        return;
    }
    double rhoOld = 1 / sigma;
    double rhoCurr = 1 / (2 * sigma - rhoOld);
    // s1 = rho1 (2 sigma s0 + 2/delta D^-1 (B + A s0)), s0 = D^-1 B / theta
    const float t1 = (float)(rhoCurr * 2.0 / delta);
    const unet::LCoef c1{(float)(rhoCurr * 2.0 * sigma), t1, t1, 0.0f, n == 3 ? -1.0f : 1.0f, y0};
    if (n == 3) {
        unet::level_cheb(d, L, nullptr, B, nullptr, X, c1, true, acc, st);
        return;
    }
    float *Y = s->cY, *Z = s->cZ, *W = s->cW;
    unet::level_cheb(d, L, nullptr, B, nullptr, Y, c1, true, false, st);
    for (int it = 2; it <= n - 2; it++) {
        rhoOld = rhoCurr;
        rhoCurr = 1 / (2 * sigma - rhoOld);
        const bool last = (it == n - 2), first = (it == 2);
        const double t = rhoCurr * 2.0 / delta;
        double cb = t, cz = -rhoCurr * rhoOld;
        if (first) {   // Z = s0 = D^-1 B / theta: fold it into the B term
            cb += cz / theta;
            cz = 0.0;
        }
        const unet::LCoef c{(float)(rhoCurr * 2.0 * sigma), (float)cb, (float)t, (float)cz, last ? -1.0f : 1.0f, y0};
        unet::level_cheb(d, L, Y, B, first ? nullptr : Z, last ? X : W, c, false, last && acc, st);
        if (!last) {
            float* tmp = Z;
            Z = Y;
            Y = W;
            W = tmp;
        }
    }
}

// The multigrid form of the learned cycle, a V-cycle over levels 0..k whose
// coarsest solver is the network:
//   level 0 (solver fields): X = S_0 B;  r_1 = R (B - A X)
//   level l = 1..k-1:        z_l = S_l r_l;  r_{l+1} = R (r_l - A_l z_l)
//   level k:                 z_k = gain N(r_k)
//   level l = k-1..1:        z_l += P z_{l+1};  z_l += S_l (r_l - A_l z_l)
//   level 0:                 X += P z_1;  [X += S_0 (B - A X)]
// S_l: Chebyshev smoothers on the high-frequency end of each level's spectrum;
// dn[l] holds r_l, dn_e[l] holds z_l.  With `dots` (flexible CG: X = z, B = r) the
// last prolongation also sums z.r and z.Ap when it can; returns whether it did.
template <typename T>
bool learned_vcycle(pps_solver* s, Fields<T>& F, T* B, T* X, Launcher& L, const T* Ap = nullptr,
                    const RedCtx* dots = nullptr)
{
    const Geo& g = s->geo;
    cudaStream_t st = s->stream;
    const int k = s->net_coarsen;
    const ChebP pf = smoother_of(g.ds, s->cyc_ratio, s->cyc_fine);
    fast_cheb<T>(s, F, B, X, L, pf);
    unet::field_residual_restrict<T>(g, B, X, dense_dims(s, 1), s->dn[1], st);
    for (int l = 1; l < k; l++) {
        if (s->cyc_coarse > 0) {
            dense_cheb(s, l, s->dn[(size_t)l], s->dn_e[(size_t)l], false);
            const unet::Dims dl = dense_dims(s, l);
            if ((long long)dl.W * dl.H * dl.D <= (1LL << 21)) {
                // up to 128^3 the fused residual + restriction wins (the levels are
                // L2-resident and launch-bound); above, its 3 x 3 window's recomputed
                // points cost more than the stored residual's extra pass
                unet::level_residual_restrict(dense_dims(s, l + 1), level_op(s, l), s->dn_e[(size_t)l],
                                              s->dn[(size_t)l], s->dn[(size_t)l + 1], st);
            } else {
                dense_residual(s, l, s->dn[(size_t)l], s->dn_e[(size_t)l], s->dt[(size_t)l]);
                unet::restrict2(dense_dims(s, l + 1), s->dt[(size_t)l], s->dn[(size_t)l + 1], st);
            }
        } else {
            unet::restrict2(dense_dims(s, l + 1), s->dn[(size_t)l], s->dn[(size_t)l + 1], st);
        }
    }
    coarse_solve(s, k, s->dn[(size_t)k], s->dn_e[(size_t)k]);
    for (int l = k - 1; l >= 1; l--) {
        if (s->cyc_coarse > 0) {
            unet::prolong2_add(dense_dims(s, l + 1), s->dn_e[(size_t)l + 1], s->dn_e[(size_t)l], st);
            dense_residual(s, l, s->dn[(size_t)l], s->dn_e[(size_t)l], s->dt[(size_t)l]);
            dense_cheb(s, l, s->dt[(size_t)l], s->dn_e[(size_t)l], true);
        } else {
            unet::prolong2(dense_dims(s, l + 1), s->dn_e[(size_t)l + 1], s->dn_e[(size_t)l], st);
        }
    }
    const bool post = (s->net_flags & PPS_LEARNED_POST_SMOOTH) != 0;
    const bool summed = unet::prolong_add_field<T>(g, s->shape_cheb, dense_dims(s, 1), s->dn_e[1], X, st, B, Ap,
                                                   post ? nullptr : dots);
    if (post) {
        unet::field_residual<T>(g, s->shape, B, X, F.r0, st);
        fast_cheb<T>(s, F, F.r0, F.Mp, L, pf);
        unet::field_axpy<T>(g, s->shape, X, F.Mp, st);
    }
    s->learned_apps++;
    return summed;
}

// Preconditioner of the flexible-CG loop: the Chebyshev polynomial (or identity),
// or, while the learned preconditioner is active, a cycle whose coarse solver is
// the network: the two-grid cycle around the solver's own preconditioner
//   z = Cheb(r);  z += gain P^k N(R^k (r - A z));  [z += Cheb(r - A z)]
// or the multigrid V-cycle of learned_vcycle.
// With `dots` (flexible CG) the V-cycle may finish the z.r, z.Ap reduction itself:
// the return value says whether it did.
template <typename T>
bool precond_any(pps_solver* s, Fields<T>& F, T* B, T* X, Launcher& L, const T* Ap = nullptr,
                 const RedCtx* dots = nullptr)
{
    if (s->net && s->net_active && s->cyc_fine > 0 && s->net_coarsen >= 1)
        return learned_vcycle<T>(s, F, B, X, L, Ap, dots);
    fast_precond<T>(s, F, B, X, L);
    if (!(s->net && s->net_active)) return false;
    learned_coarse_correction<T>(s, B, X, X);
    if (s->net_flags & PPS_LEARNED_POST_SMOOTH) {
        // post-smoothing through the fields flexible CG leaves free (r0, Mp)
        const Geo& g = s->geo;
        unet::field_residual<T>(g, s->shape, B, X, F.r0, s->stream);
        fast_precond<T>(s, F, F.r0, F.Mp, L);
        unet::field_axpy<T>(g, s->shape, X, F.Mp, s->stream);
    }
    return false;
}

// One application of the preconditioner the flexible-CG iterations use (with the
// learned cycle when a network is attached as preconditioner).
template <typename T>
void precond_once(pps_solver* s, Fields<T>& F, T* B, T* X, Launcher& L)
{
    const bool keep = s->net_active;
    s->net_active = s->net && (s->net_flags & PPS_LEARNED_PRECONDITIONER);
    precond_any<T>(s, F, B, X, L);
    s->net_active = keep;
}

// Learned initial guess: x += gain P^k N(R^k b) at the unknowns.
void learned_initial_guess(pps_solver* s, double* x, const double* b)
{
    learned_coarse_correction<double>(s, b, nullptr, x);
}

// One BiCGSTAB iteration (BiCGSTAB.hpp:133-272) on the fast kernels; xacc is the
// field the corrections accumulate in (x itself for FP64, the FP32 correction for MIXED).
template <typename T>
void fast_bicgstab_iteration(pps_solver* s, Fields<T>& F, T* xacc, Launcher& L)
{
    const Geo& g = s->geo;
    const Shape& sh = s->shape;
    cudaStream_t st = s->stream;
    const long long N = s->n_unknowns;
    const Coef a = op_coef(g);
    fast_precond<T>(s, F, F.p, F.Mp, L);
    if (s->has_neumann) neumann_fill<T>(g, F.Mp, faces_of(s), 0, 1.0, st);
    // the stencils run on the Chebyshev tiles (x-vectorised for FP32); the updates
    // are flat 16-byte vector passes on Dirichlet grids
    fast_stencil_dot<T>(g, s->shape_cheb, F.Mp, F.r0, F.AMp, a, red_c(s, FIN_ALPHA), st);
    fast_axpy_alpha<T>(g, sh, F.r, F.AMp, s->d_st, st);
    fast_precond<T>(s, F, F.r, F.z, L);
    if (s->has_neumann) neumann_fill<T>(g, F.z, faces_of(s), 0, 1.0, st);
    fast_stencil_dot2<T>(g, s->shape_cheb, F.z, F.r, F.Az, a, red_c(s, FIN_OMEGA), st);
    fast_update_xr<T>(g, sh, xacc, F.Mp, F.z, F.r, F.Az, F.r0, red_c(s, FIN_CONV), st);
    fast_update_p<T>(g, sh, F.p, F.r, F.AMp, s->d_st, st);
    L.bytes += bytes_of<T>(N, 3 + 3 + 3 + 8 + 4);
    L.launches += s->d_cells ? 8 : 5;
}

template <typename T>
Fields<T>& inner_fields(pps_solver* s);
template <>
Fields<double>& inner_fields<double>(pps_solver* s)
{
    return s->in64;
}
template <>
Fields<float>& inner_fields<float>(pps_solver* s)
{
    return s->in32;
}

void read_state(pps_solver* s);

template <typename T>
void fast_cg_iteration(pps_solver* s, Fields<T>& F, T* xacc, Launcher& L);

// BiCGSTAB or CG as the preconditioner (BiCGSTAB.hpp:55-322, baseCG.hpp:44-260 with
// isMainLoop false): X = 0, then iterations on B with their own Krylov scalars, to
// ||r|| < precond_tol ||B|| or precond_maxit iterations, preconditioned by
// precond_inner.  The reference normalises B to unit norm first; the iteration is
// invariant under that scaling, so the fast forms leave B unchanged.  The host
// polls the inner stop flag every few iterations (an inner solve cannot sit inside
// a captured graph, so the outer loop runs without one).
template <typename T>
void fast_inner_precond(pps_solver* s, T* B, T* X, Launcher& L, bool cg)
{
    const Geo& g = s->geo;
    cudaStream_t st = s->stream;
    Fields<T>& W = inner_fields<T>(s);
    fill_field<T>(X, g.ntot, (T)0, st);
    L.bytes += bytes_of<T>(g.ntot, 1);
    if (s->cfg.precond_maxit < 1) return;
    InnerScope in(s);
    // FIN_RES0 with tol_relative: the stop target becomes precond_tol * ||B||
    state_init(s->d_st, s->d_hist, s->cfg.precond_maxit, 0.0, s->cfg.precond_tol, 1, 1, 1.0, 0, st);
    fast_bicg_start<T>(g, s->shape, B, W.r, W.r0, W.p, red_c(s, FIN_RES0), st);
    L.bytes += bytes_of<T>(s->n_unknowns, 4);
    if (cg) {
        // z = M r, p = z (baseCG.hpp:110-112)
        fast_precond<T>(s, W, W.r, W.z, L);
        CK(cudaMemcpyAsync(W.p, W.z, sizeof(T) * (size_t)g.ntot, cudaMemcpyDeviceToDevice, st));
    }
    const int poll = 4;
    for (;;) {
        for (int q = 0; q < poll; q++) {
            if (cg) fast_cg_iteration<T>(s, W, X, L);
            else fast_bicgstab_iteration<T>(s, W, X, L);
        }
        read_state(s);
        if (s->h_st->done) break;
    }
    s->prec_iters += s->h_st->iter;
    // BiCGSTAB ends with resetNeumanBCs<false,true> on X, the mirror copy; CG with
    // orderNeumanBcs == 2 does not
    if (!cg && s->has_neumann) neumann_fill<T>(g, X, faces_of(s), 0, 1.0, st);
}

// One CG iteration (baseCG.hpp:115-228). The caller applied z = M^{-1} r and p = z.
template <typename T>
void fast_cg_iteration(pps_solver* s, Fields<T>& F, T* xacc, Launcher& L)
{
    const Geo& g = s->geo;
    const Shape& sh = s->shape;
    cudaStream_t st = s->stream;
    const long long N = s->n_unknowns;
    const Coef a = op_coef(g);
    fast_cg_stencil_dot<T>(g, sh, F.p, F.r, F.z, F.AMp, a, red_c(s, FIN_CG_ALPHA), st);
    fast_cg_update_xr<T>(g, sh, xacc, F.p, F.r, F.AMp, s->d_st, st);
    fast_precond<T>(s, F, F.r, F.z, L);
    fast_cg_dot_rz<T>(g, sh, F.r, F.z, red_c(s, FIN_CG_CONV), st);
    fast_cg_update_p<T>(g, sh, F.p, F.z, s->d_st, st);
    L.bytes += bytes_of<T>(N, 4 + 6 + 2 + 3);
    L.launches += s->d_cells ? 6 : 4;
}

bool aligned16(const void* p)
{
    return ((uintptr_t)p & 15u) == 0;
}

// One flexible-CG iteration: CG with the Polak-Ribiere beta = z_new.(r_new - r_old) /
// (z_old.r_old), so the preconditioner may change from one application to the next.
// With r_new - r_old = -alpha Ap no old residual is kept; the direction update
// p = z + beta p rides on the stencil kernel, which writes the new direction into
// the other of the fields p and Az (swapped here after every iteration).
template <typename T>
void fast_fcg_iteration(pps_solver* s, Fields<T>& F, T* xacc, Launcher& L)
{
    const Geo& g = s->geo;
    const Shape& sh = s->shape;
    cudaStream_t st = s->stream;
    const long long N = s->n_unknowns;
    const Coef a = op_coef(g);
    // the direction/stencil kernel runs on the Chebyshev tiles (x-vectorised for FP32)
    const bool prof = L.profile && s->krylov_ev_used + 2 <= (int)s->krylov_ev.size();
    if (prof) CK(cudaEventRecord(s->krylov_ev[s->krylov_ev_used], st));
    fast_fcg_p_stencil<T>(g, s->shape_cheb, F.z, F.p, F.Az, F.AMp, a, red(s, FIN_FCG_ALPHA), st,
                          s->tuning.fcg_staged != 0);
    std::swap(F.p, F.Az);
    const bool flat = aligned16(xacc) && aligned16(F.p) && aligned16(F.r) && aligned16(F.AMp) && aligned16(F.z);
    if (flat) fast_fcg_update_xr_flat<T>(g, sh, xacc, F.p, F.r, F.AMp, red(s, FIN_FCG_RES), st);
    else fast_fcg_update_xr<T>(g, sh, xacc, F.p, F.r, F.AMp, red(s, FIN_FCG_RES), st);
    if (prof) {   // z, p_in read, p_out, Ap written; x, r read and written, p, Ap read
        CK(cudaEventRecord(s->krylov_ev[s->krylov_ev_used + 1], st));
        s->krylov_ev_used += 2;
        s->krylov_bytes_acc += bytes_of<T>(N, 4 + 6);
        s->krylov_launch_acc += 2;
    }
    const RedCtx conv = red(s, FIN_FCG_CONV);
    if (precond_any<T>(s, F, F.r, F.z, L, F.AMp, &conv)) {   // the V-cycle summed z.r, z.Ap
        L.bytes += bytes_of<T>(N, 4 + 6 + 2);
        L.launches += 2;
        return;
    }
    if (flat) fast_fcg_dot_flat<T>(g, sh, F.r, F.z, F.AMp, conv, st);
    else fast_fcg_dot<T>(g, sh, F.r, F.z, F.AMp, conv, st);
    L.bytes += bytes_of<T>(N, 4 + 6 + 3);
    L.launches += 3;
}

// Flexible-CG (re)start after z = M r: rho0 = z.r and beta = 0, so the next
// iteration's direction is z.
template <typename T>
void fcg_setup(pps_solver* s, Fields<T>& F, Launcher& L)
{
    fast_fcg_dot<T>(s->geo, s->shape, F.r, F.z, nullptr, red(s, FIN_FCG_SETUP), s->stream);
    L.bytes += bytes_of<T>(s->n_unknowns, 2);
    L.launches += 1;
}

template <typename T>
void fast_iteration(pps_solver* s, Fields<T>& F, T* xacc, Launcher& L)
{
    if (s->cfg.krylov == PPS_KRYLOV_CG) fast_cg_iteration<T>(s, F, xacc, L);
    else if (s->cfg.krylov == PPS_KRYLOV_FCG) fast_fcg_iteration<T>(s, F, xacc, L);
    else fast_bicgstab_iteration<T>(s, F, xacc, L);
}

void read_state(pps_solver* s)
{
    if (s->state_mapped) state_out(s->d_st, s->h_st, s->stream);
    else CK(cudaMemcpyAsync(s->h_st, s->d_st, sizeof(DevState), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
}

// Status of a solve restarted on the uploaded x (internal; never returned to callers)
constexpr pps_status kRestartOnX = (pps_status)1000;

// Ends a speculative start (pps_solve): when x's upload and test are done (or, with
// wait, once they are), the solver's stream is ordered after them and the result is
// read: true when x held a non-zero entry, so the work done on x = 0 is void.  False
// while they are still running (no wait) or when no start was speculative.
bool x_was_nonzero(pps_solver* s, bool wait)
{
    if (!s->spec_x) return false;
    if (wait) {
        CK(cudaEventSynchronize(s->ev_x));
    } else {
        const cudaError_t e = cudaEventQuery(s->ev_x);
        if (e == cudaErrorNotReady) return false;
        CK(e);
    }
    CK(cudaStreamWaitEvent(s->stream, s->ev_x, 0));
    s->spec_x = false;
    return *(volatile int*)s->h_xnz != 0;
}

// After an update of x on the solver's stream: copy x to the caller's pinned array on
// copy_stream, overlapping whatever the solve does next (a final residual check)
void copy_out(pps_solver* s, const double* x)
{
    if (!s->out_host) return;
    CK(cudaEventRecord(s->ev_upd, s->stream));
    CK(cudaStreamWaitEvent(s->copy_stream, s->ev_upd, 0));
    CK(cudaMemcpyAsync(s->out_host, x, sizeof(double) * (size_t)s->geo.ntot, cudaMemcpyDeviceToHost, s->copy_stream));
    CK(cudaEventRecord(s->ev_out, s->copy_stream));
    s->out_issued = true;
    s->out_current = true;
}

// Before the solver's stream writes x again: the copy out of its previous value ends first
void before_x_update(pps_solver* s)
{
    if (s->out_issued) CK(cudaStreamWaitEvent(s->stream, s->ev_out, 0));
    s->out_current = false;
}

int auto_check_every(const pps_solver* s, int elem_size)
{
    if (s->cfg.check_every > 0) return s->cfg.check_every;
    // Estimated iteration time against a ~0.4 ms polling period.
    const int n = std::max(s->cfg.cheb_degree, 4);
    const double bytes = (double)s->n_unknowns * elem_size * (2.0 * (3 + 4 * (n - 3)) + 21);
    const double t_iter = bytes / 5.0e12 + 25 * 3e-6;
    int c = (int)(4e-4 / t_iter);
    return std::max(1, std::min(c, 16));
}

// Runs Krylov iterations until the device stop flag is set. With use_graph, a
// chunk of `chunk` iterations is captured once and replayed.
template <typename T>
pps_status run_iterations(pps_solver* s, Fields<T>& F, T* xacc, int form, Launcher& L)
{
    // with the learned preconditioner the host looks at the residual every two
    // iterations (the fallback rule), otherwise at the automatic polling interval
    int chunk = s->net && s->net_active ? 2 : auto_check_every(s, (int)sizeof(T));
    // flexible CG swaps its direction fields every iteration: a captured chunk must
    // hold an even number of iterations to leave them where the capture found them
    if (s->cfg.krylov == PPS_KRYLOV_FCG) chunk += chunk & 1;
    // the inner BiCGSTAB preconditioner is host-polled: no graph, and every outer
    // iteration is followed by a poll so that no inner solve runs after the stop
    const bool inner = s->cfg.precond == PPS_PREC_BICGSTAB || s->cfg.precond == PPS_PREC_CG;
    if (inner) chunk = 1;
    const bool graph = s->cfg.use_graph != 0 && !L.profile && !inner;
    std::vector<std::pair<int, double>> errs;   // (iteration, residual norm) seen by the fallback rule
    // inside the iterations the learned cycle's kernels return at once after the stop
    // test (a converged iteration skips its preconditioner)
    unet::set_stop_flag(&s->d_st->done);
    struct ClearStop {
        ~ClearStop() { unet::set_stop_flag(nullptr); }
    } clear_stop;
    for (;;) {
        const bool learned = s->net && s->net_active;
        if (graph) {
            if (!(s->gexec && s->g_key_x == xacc && s->g_form == form && s->g_iters == chunk &&
                  s->g_learned == learned)) {
                if (s->gexec) {
                    cudaGraphExecDestroy(s->gexec);
                    s->gexec = nullptr;
                }
                cudaGraph_t gr = nullptr;
                Launcher LG{s, false};
                const double sb = s->sweep_bytes_acc;
                const int sl = s->sweep_launch_acc;
                const int la = s->learned_apps;
                const int c0 = launches_counter();
                {
                    CK(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
                    CaptureGuard cap(s->stream);   // an error below ends the capture
                    for (int q = 0; q < chunk; q++) fast_iteration<T>(s, F, xacc, LG);
                    CK(cap.end(&gr));
                }
                LG.launches = launches_counter() - c0;
                launches_counter_add(-LG.launches);
                const cudaError_t ie = cudaGraphInstantiate(&s->gexec, gr, 0);
                cudaGraphDestroy(gr);
                if (ie != cudaSuccess) s->gexec = nullptr;
                CK(ie);
                s->g_key_x = xacc;
                s->g_form = form;
                s->g_iters = chunk;
                s->g_bytes = LG.bytes;
                s->g_launches = LG.launches;
                s->g_sweep_bytes = s->sweep_bytes_acc - sb;
                s->g_sweep_launches = s->sweep_launch_acc - sl;
                s->sweep_bytes_acc = sb;
                s->sweep_launch_acc = sl;
                s->g_learned = learned;
                s->g_learned_apps = s->learned_apps - la;
                s->learned_apps = la;
            }
            CK(cudaGraphLaunch(s->gexec, s->stream));
            L.bytes += s->g_bytes;
            launches_counter_add(s->g_launches);
            s->sweep_bytes_acc += s->g_sweep_bytes;
            s->sweep_launch_acc += s->g_sweep_launches;
            s->learned_apps += s->g_learned_apps;
        } else {
            for (int q = 0; q < chunk; q++) fast_iteration<T>(s, F, xacc, L);
        }
        read_state(s);
        if (x_was_nonzero(s, false)) return kRestartOnX;
        if (s->h_st->done) break;
        if (learned) {
            // fall back to the plain preconditioner when the per-iteration reduction,
            // the geometric mean over at least the last 4 iterations, is worse than 0.5
            const double e = s->h_st->err;
            const int it = s->h_st->iter;
            errs.emplace_back(it, e);
            int back = -1;   // the latest sample at least 4 iterations old
            for (int q = (int)errs.size() - 1; q >= 0; q--)
                if (it - errs[(size_t)q].first >= 4) {
                    back = q;
                    break;
                }
            if (!(s->net_flags & PPS_LEARNED_NO_FALLBACK) && back >= 0 &&
                std::pow(e / errs[(size_t)back].second, 1.0 / (double)(it - errs[(size_t)back].first)) > 0.5) {
                s->net_active = false;
                s->fallback_iter = s->h_st->iter;
                // restart the flexible-CG recurrence on the plain preconditioner: z = M r, p = z
                precond_any<T>(s, F, F.r, F.z, L);
                fcg_setup<T>(s, F, L);
            }
        }
    }
    return (pps_status)s->h_st->status;
}

void pull_history(pps_solver* s, int n_iter, bool append)
{
    const int n = std::min(n_iter + 1, s->hist_cap);
    std::vector<double> h((size_t)std::max(n, 0));
    if (n > 0) {
        CK(cudaMemcpyAsync(h.data(), s->d_hist, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
    }
    if (!append) s->history.clear();
    const size_t start = append && !s->history.empty() ? 1 : 0;
    for (size_t i = start; i < h.size(); i++) s->history.push_back(h[i]);
}

// True when x is +-0 everywhere (guard layers included): then A x = 0 and, on a
// Dirichlet grid, b_adj = b, so the first residual needs no FP64 stencil.
bool field_is_zero(pps_solver* s, const double* x)
{
    if (((uintptr_t)x & 15u) != 0) return false;
    if (s->xnz_mapped) {   // one pass of integer ORs; the flag is stored through its mapping
        *(volatile int*)s->h_xnz = 0;
        flag_nonzero(s->geo.ntot, x, s->h_xnz, s->stream);
        CK(cudaStreamSynchronize(s->stream));
        return *(volatile int*)s->h_xnz == 0;
    }
    state_init(s->d_st, s->d_hist, 0, 0.0, 0.0, 0, 0, 1.0, 0, s->stream);
    fast_count_nonzero(s->geo, s->shape, x, red(s, FIN_STORE), s->stream);
    read_state(s);
    return s->h_st->sums[0] == 0.0;
}

double norm_badj(pps_solver* s, const double* x, const double* b, bool x_zero = false)
{
    state_init(s->d_st, s->d_hist, 0, 0.0, 0.0, 0, 0, 1.0, 0, s->stream);
    fast_norm_badj(s->geo, s->shape, b, x, faces_of(s), red_c(s, FIN_NORMB), s->stream, x_zero);
    read_state(s);
    return s->h_st->normb;
}

// FP64 form: the reference algorithm on the unscaled system. Scaling commutes with
// every step, so rho0 = ||b_adj||^2 and tol_abs = tol*||b_adj|| reproduce the
// normalised iteration (rho0 = 1, BiCGSTAB.hpp:127) without two scaling passes.
pps_status solve_fp64(pps_solver* s, double* x, const double* b)
{
    const Geo& g = s->geo;
    Fields<double>& F = s->f64;
    cudaStream_t st = s->stream;
    pps_stats& S = s->stats;
    Launcher L{s, s->cfg.use_graph == 0};
    if (s->has_neumann) neumann_fill<double>(g, x, faces_of(s), 1, 1.0, st);
    const bool x0_zero = !s->has_neumann && field_is_zero(s, x);
    const double normb = norm_badj(s, x, b, x0_zero);
    S.norm_b = normb;
    if (!(normb > 0.0)) return PPS_ERR_ZERO_RHS;
    s->net_active = s->net && (s->net_flags & PPS_LEARNED_PRECONDITIONER) && s->cfg.krylov == PPS_KRYLOV_FCG;
    s->learned_apps = 0;
    s->fallback_iter = -1;
    const bool guess = s->net && (s->net_flags & PPS_LEARNED_INITIAL_GUESS);
    if (guess) learned_initial_guess(s, x, b);
    const bool x_zero = x0_zero && !guess;
    const Coef a = op_coef(g);
    state_init(s->d_st, s->d_hist, s->cfg.maxit, s->cfg.tol * normb, 0.0, 0, 0, 1.0 / normb, s->hist_cap, st);
    // BiCGSTAB and CG start from r0 = p = r; flexible CG needs r alone (its first
    // direction is the preconditioned residual)
    const bool fcg = s->cfg.krylov == PPS_KRYLOV_FCG;
    fast_residual<double>(g, s->shape, x, b, F.r, fcg ? nullptr : F.r0, fcg ? nullptr : F.p, a,
                          fcg ? red(s, FIN_RES0) : red_c(s, FIN_RES0), st, x_zero);
    L.bytes += bytes_of<double>(s->n_unknowns, 5) + bytes_of<double>(s->n_unknowns, 1) * 2;
    pps_status rc = PPS_OK;
    read_state(s);
    if (!s->h_st->done) {
        if (s->cfg.krylov == PPS_KRYLOV_CG) {
            precond_any<double>(s, F, F.r, F.z, L);
            CK(cudaMemcpyAsync(F.p, F.z, sizeof(double) * (size_t)g.ntot, cudaMemcpyDeviceToDevice, st));
        } else if (s->cfg.krylov == PPS_KRYLOV_FCG) {
            precond_any<double>(s, F, F.r, F.z, L);
            fcg_setup<double>(s, F, L);
        }
        rc = run_iterations<double>(s, F, x, PPS_FORM_FP64, L);
    } else {
        rc = (pps_status)s->h_st->status;
    }
    S.iterations = s->h_st->iter;
    S.err_iter = s->h_st->iter > 0 ? s->h_st->err / normb : -1.0;
    pull_history(s, S.iterations, false);
    S.precond_applications += S.iterations * (s->cfg.krylov == PPS_KRYLOV_BICGSTAB ? 2 : 1);
    // final true residual (computeErrorOperatorA after the loop, BiCGSTAB.hpp:305-308)
    if (s->has_neumann) neumann_fill<double>(g, x, faces_of(s), 1, 1.0, st);
    fast_residual<double>(g, s->shape, x, b, F.Az, nullptr, nullptr, a, red_c(s, FIN_STORE), st);
    read_state(s);
    S.err_true = std::sqrt(s->h_st->sums[0]) / normb;
    S.hbm_bytes += L.bytes;
    return rc;
}

// MIXED form: FP64 iterative refinement around an FP32 inner solve.
// One pass of the MIXED solve.  Under a speculative start (spec_x) it runs on x = 0
// and, where it would next read or write x (or return), first reads the test of the
// uploaded x: a non-zero x returns kRestartOnX with x untouched.
pps_status solve_mixed_pass(pps_solver* s, double* x, const double* b)
{
    const Geo& g = s->geo;
    Fields<float>& F = s->f32;
    cudaStream_t st = s->stream;
    pps_stats& S = s->stats;
    Launcher L{s, s->cfg.use_graph == 0};
    if (s->has_neumann) {
        before_x_update(s);
        neumann_fill<double>(g, x, faces_of(s), 1, 1.0, st);
    }
    const bool x0_zero = s->spec_x || (!s->has_neumann && field_is_zero(s, x));
    const double normb = norm_badj(s, x, b, x0_zero);
    S.norm_b = normb;
    if (!(normb > 0.0)) return x_was_nonzero(s, true) ? kRestartOnX : PPS_ERR_ZERO_RHS;
    s->net_active = s->net && (s->net_flags & PPS_LEARNED_PRECONDITIONER) && s->cfg.krylov == PPS_KRYLOV_FCG;
    s->learned_apps = 0;
    s->fallback_iter = -1;
    const bool guess = s->net && (s->net_flags & PPS_LEARNED_INITIAL_GUESS);
    if (guess) {
        before_x_update(s);
        learned_initial_guess(s, x, b);
    }
    const bool x_zero = x0_zero && !guess;
    const Coef a = op_coef(g);
    const double tol_abs = s->cfg.tol * normb;
    s->history.clear();
    int total_iter = 0;
    pps_status rc = PPS_NOT_CONVERGED;
    double err_outer = 0;
    for (int ref = 0; ref <= s->cfg.max_refinements; ref++) {
        const int remaining = s->cfg.maxit - total_iter;
        // FIN_RES0 stops when the FP64 residual meets tol_abs; otherwise it sets the
        // inner target max(inner_tol, 0.3*tol_abs/err0)*err0 on the device.
        state_init(s->d_st, s->d_hist, std::max(1, std::min(s->cfg.inner_maxit, remaining)), tol_abs,
                   s->cfg.inner_tol, 1, 1, 1.0 / normb, s->hist_cap, st);
        const bool fcg = s->cfg.krylov == PPS_KRYLOV_FCG;   // r alone (see solve_fp64)
        fast_residual<float>(g, s->shape, x, b, F.r, fcg ? nullptr : F.r0, fcg ? nullptr : F.p, a, red(s, FIN_RES0),
                             st, ref == 0 && x_zero);
        L.bytes += bytes_of<double>(s->n_unknowns, 2) + bytes_of<float>(s->n_unknowns, 3);
        read_state(s);
        err_outer = s->h_st->err0;
        if (s->history.empty()) s->history.push_back(err_outer / normb);
        else s->history.back() = err_outer / normb;   // true residual replaces the recursive estimate
        if (err_outer < tol_abs) {
            if (x_was_nonzero(s, true)) return kRestartOnX;
            rc = PPS_OK;
            break;
        }
        if (ref == s->cfg.max_refinements || remaining <= 0) {
            if (x_was_nonzero(s, true)) return kRestartOnX;
            break;
        }
        fill_field<float>(F.e, g.ntot, 0.0f, st);
        if (s->cfg.krylov == PPS_KRYLOV_CG) {
            precond_any<float>(s, F, F.r, F.z, L);
            CK(cudaMemcpyAsync(F.p, F.z, sizeof(float) * (size_t)g.ntot, cudaMemcpyDeviceToDevice, st));
        } else if (s->cfg.krylov == PPS_KRYLOV_FCG) {
            precond_any<float>(s, F, F.r, F.z, L);
            fcg_setup<float>(s, F, L);
        }
        pps_status irc = run_iterations<float>(s, F, F.e, PPS_FORM_MIXED, L);
        if (irc == kRestartOnX || x_was_nonzero(s, true)) return kRestartOnX;
        const int it = s->h_st->iter;
        total_iter += it;
        pull_history(s, it, true);
        S.precond_applications += it * (s->cfg.krylov == PPS_KRYLOV_BICGSTAB ? 2 : 1);
        S.err_iter = s->h_st->err / normb;
        // e started at zero and the updates add multiples of fields that are zero off
        // the unknowns on Dirichlet grids
        before_x_update(s);
        fast_add_correction(g, s->shape, x, F.e, s->d_st, st, true);
        L.bytes += bytes_of<double>(s->n_unknowns, 2) + bytes_of<float>(s->n_unknowns, 1);
        if (s->has_neumann) neumann_fill<double>(g, x, faces_of(s), 1, 1.0, st);
        copy_out(s, x);   // overlaps the residual check that follows
        S.refinements++;
        if (irc == PPS_NAN_DETECTED) {
            rc = irc;
            break;
        }
    }
    S.iterations = total_iter;
    S.err_true = err_outer / normb;
    S.hbm_bytes += L.bytes;
    return rc;
}

pps_status solve_mixed(pps_solver* s, double* x, const double* b)
{
    const pps_status rc = solve_mixed_pass(s, x, b);
    if (rc != kRestartOnX) return rc;
    // the uploaded x held a non-zero entry: the pass on x = 0 is void, solve from x
    s->spec_restarted = true;
    s->stats.precond_applications = 0;
    s->stats.refinements = 0;
    return solve_mixed_pass(s, x, b);
}

// ChebyshevIteration::operator() as the main solver (chebyshevIteration.hpp:48-140
// with isMainLoop true; chebyshevIterationAlpaka.hpp:320-587): bt = a copy of b
// adjusted for the boundary data (its boundary nodes hold b's values, adjusted where
// a face's neighbour plane reaches them; the stencil of the first step reads them),
// X = -s_{n-2}(bt) at the unknowns (the initial guess is overwritten), then the true
// residual with normFieldB_ = 1, reported absolute.  PARITY and FP64 apply the polynomial once, as the reference does;
// MIXED applies it in FP32, first to bt and then, up to max_refinements times, to
// the FP64 residual, until ||b - A x|| < tol ||b_adj||.
pps_status solve_cheb_main(pps_solver* s, double* x, const double* b)
{
    s->learned_apps = 0;
    s->fallback_iter = -1;
    s->net_active = false;
    const Geo& g = s->geo;
    cudaStream_t st = s->stream;
    pps_stats& S = s->stats;
    const size_t fb = sizeof(double) * (size_t)g.ntot;
    const int n = s->cfg.cheb_degree;
    double* bt = s->d_bt;
    CK(cudaMemcpyAsync(bt, b, fb, cudaMemcpyDeviceToDevice, st));
    par_adjust_b_data(g, b, x, faces_of(s), bt, st);
    s->history.clear();
    double err = 0;
    int passes = 1;
    pps_status rc = PPS_OK;
    if (s->cfg.form == PPS_FORM_PARITY_FP64) {
        S.norm_b = std::sqrt(par_dot(s, bt, bt));
        CK(cudaMemsetAsync(s->pW, 0, fb, st));   // a new object's W (the output at degree 1)
        par_precond(s, bt, x);
        err = par_true_residual(s, x, const_cast<double*>(b), s->f64.r, 1.0);
    } else {
        S.norm_b = norm_badj(s, x, b);
        state_init(s->d_st, s->d_hist, 0, 0.0, 0.0, 0, 0, 1.0, 0, st);
        Launcher L{s, s->cfg.use_graph == 0};
        const Coef a = op_coef(g);
        if (s->cfg.form == PPS_FORM_FP64) {
            Fields<double>& F = s->f64;
            double* X = n == 1 ? F.z : x;   // degree 1 fills the whole output field
            fast_cheb<double>(s, F, bt, X, L, cheb_of(s));
            if (n == 1) fast_scale_copy<double>(g, s->shape, F.z, x, 1.0, nullptr, st);
            if (s->has_neumann) neumann_fill<double>(g, x, faces_of(s), 1, 1.0, st);
            fast_residual<double>(g, s->shape, x, b, F.Az, nullptr, nullptr, a, red(s, FIN_STORE), st);
            read_state(s);
            err = std::sqrt(s->h_st->sums[0]);
        } else {
            Fields<float>& F = s->f32;
            const double tol_abs = s->cfg.tol * S.norm_b;
            cast_field_f32(bt, F.p, g.ntot, st);
            fast_cheb<float>(s, F, F.p, F.e, L, cheb_of(s));
            fast_scale_copy<double>(g, s->shape, b, x, 0.0, nullptr, st);   // x = 0 at the unknowns
            for (;;) {
                fast_add_correction(g, s->shape, x, F.e, s->d_st, st);
                if (s->has_neumann) neumann_fill<double>(g, x, faces_of(s), 1, 1.0, st);
                fast_residual<float>(g, s->shape, x, b, F.r, nullptr, nullptr, a, red(s, FIN_STORE), st);
                read_state(s);
                err = std::sqrt(s->h_st->sums[0]);
                if (!std::isfinite(err)) {
                    rc = PPS_NAN_DETECTED;
                    break;
                }
                if (err < tol_abs || passes > s->cfg.max_refinements) break;
                s->history.push_back(err);
                fast_cheb<float>(s, F, F.r, F.e, L, cheb_of(s));
                passes++;
            }
            S.refinements = passes - 1;
        }
        S.hbm_bytes += L.bytes;
    }
    s->history.push_back(err);
    S.iterations = n * passes;
    S.precond_applications = passes;
    S.err_iter = err;
    S.err_true = err;
    if (rc != PPS_OK) return rc;
    return err < s->cfg.tol * S.norm_b ? PPS_OK : PPS_NOT_CONVERGED;
}

// ---------------------------------------------------------------------------
// Autotuner: tile shapes of the z-marching kernels, timed on the solver's grid
// ---------------------------------------------------------------------------

const int kTys[] = {2, 4, 8};
const int kCxs[] = {1, 2, 4};
const int kWaves[] = {1, 2, 4, 8};

int resident_blocks(int ty)
{
    const int threads = 32 * ty;
    return std::min(32, 2048 / threads);
}

Shape tuned_shape(const Geo& g, int ty, int cx, int waves)
{
    return make_shape(g, ty, waves * sm_count() * resident_blocks(ty), cx);
}

unsigned max_candidate_blocks(const Geo& g)
{
    unsigned m = 0;
    for (int ty : kTys)
        for (int cx : kCxs)
            for (int w : kWaves) m = std::max(m, tuned_shape(g, ty, cx, w).nblocks());
    return m;
}

template <typename T>
double time_launches(pps_solver* s, int reps, const std::function<void()>& launch)
{
    launch();   // warm-up
    CK(cudaEventRecord(s->ev0, s->stream));
    for (int r = 0; r < reps; r++) launch();
    CK(cudaEventRecord(s->ev1, s->stream));
    CK(cudaEventSynchronize(s->ev1));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, s->ev0, s->ev1));
    return 1e3 * ms / reps;
}

template <typename T>
void autotune_fields(pps_solver* s, Fields<T>& F, pps_tuning* best)
{
    const Geo& g = s->geo;
    const long long N = s->n_unknowns;
    const int reps = N > (1LL << 24) ? 5 : 20;
    state_init(s->d_st, s->d_hist, 1, 0.0, 0.0, 0, 0, 1.0, 0, s->stream);
    const Coef c = cheb_sweep_coef(op_coef(g), cheb_of(s), 0.5, 0.5, 1.0);
    const Coef a = op_coef(g);
    // The Chebyshev tiles also carry the Krylov stencil kernel of the method (flexible
    // CG's direction update + stencil, BiCGSTAB's and CG's stencil + dots), whose
    // reads of two fields with their y halo make it the more shape-sensitive one: a
    // candidate is scored by the sweep's time, weighted by the Chebyshev launches per
    // stencil launch of an iteration, plus that kernel's.
    const bool fcg = s->cfg.krylov == PPS_KRYLOV_FCG;
    if (fcg) {   // a non-zero beta, so the direction kernel reads p as well as z
        const double beta = 0.5;
        CK(cudaMemcpyAsync(&s->d_st->beta, &beta, sizeof(double), cudaMemcpyHostToDevice, s->stream));
        CK(cudaStreamSynchronize(s->stream));
    }
    // Chebyshev launches per launch of the Krylov stencil kernel in one iteration: the
    // reference method's two applications of degree n (s1 and n - 3 sweeps each) per two
    // stencil kernels; flexible CG's smoother (the V-cycle's fine degree, or the
    // polynomial) per direction kernel
    const int n = s->cfg.cheb_degree;
    double weight = std::max(1, n - 2);
    if (fcg && s->cyc_fine > 0) weight = std::max(1, s->cyc_fine - 2);
    double best_us = 1e30;
    for (int ty : kTys)
        for (int cx : kCxs)
            for (int w : kWaves) {
                if (cx == 4 && !std::is_same<T, float>::value) continue;   // FP64 runs one-column tiles
                const Shape sh = tuned_shape(g, ty, cx, w);
                const double us = time_launches<T>(s, reps, [&]() {
                    fast_cheb_sweep<T>(g, sh, F.Y, F.r, F.Z, F.W, c, &s->d_st->done, s->stream);
                });
                const double ks = time_launches<T>(s, reps, [&]() {
                    if (fcg)
                        fast_fcg_p_stencil<T>(g, sh, F.z, F.p, F.Az, F.AMp, a, red(s, FIN_STORE), s->stream,
                                              best->fcg_staged != 0);
                    else fast_stencil_dot2<T>(g, sh, F.z, F.r, F.Az, a, red_c(s, FIN_STORE), s->stream);
                });
                if (weight * us + ks < best_us) {
                    best_us = weight * us + ks;
                    best->cheb_ty = ty;
                    best->cheb_cx = cx;
                    best->cheb_waves = w;
                    best->cheb_us = us;
                }
            }
    best_us = 1e30;
    for (int ty : kTys)
        for (int w : kWaves) {
            const Shape sh = tuned_shape(g, ty, 1, w);
            const double us = time_launches<T>(s, reps, [&]() {
                state_init(s->d_st, s->d_hist, 1, 0.0, 0.0, 0, 0, 1.0, 0, s->stream);
                fast_stencil_dot2<T>(g, sh, F.z, F.r, F.Az, a, red_c(s, FIN_STORE), s->stream);
            });
            if (us < best_us) {
                best_us = us;
                best->other_ty = ty;
                best->other_waves = w;
                best->other_us = us;
            }
        }
}

void apply_tuning(pps_solver* s, const pps_tuning& t)
{
    s->tuning = t;
    s->shape_cheb = tuned_shape(s->geo, t.cheb_ty, t.cheb_cx, t.cheb_waves);
    s->shape = tuned_shape(s->geo, t.other_ty, 1, t.other_waves);
    if (s->gexec) {   // captured launches carry the old shapes
        cudaGraphExecDestroy(s->gexec);
        s->gexec = nullptr;
    }
}

bool tuning_valid(const pps_tuning* t)
{
    auto in = [](int v, const int* a, int n) {
        for (int i = 0; i < n; i++)
            if (a[i] == v) return true;
        return false;
    };
    return in(t->cheb_ty, kTys, 3) && in(t->cheb_cx, kCxs, 3) && in(t->cheb_waves, kWaves, 4) &&
           in(t->other_ty, kTys, 3) && in(t->other_waves, kWaves, 4) && (t->cheb_fused == 0 || t->cheb_fused == 1) &&
           (t->fcg_staged == 0 || t->fcg_staged == 1);
}

pps_status validate(const pps_grid* g, const pps_config* c)
{
    if (!g || !c) return PPS_ERR_INVALID_ARG;
    for (int d = 0; d < 3; d++) {
        if (g->npglobal[d] < 3) { set_error("npglobal must be >= 3 on every axis"); return PPS_ERR_INVALID_ARG; }
        if (!(g->ds[d] > 0.0) || !std::isfinite(g->ds[d])) { set_error("ds must be positive"); return PPS_ERR_INVALID_ARG; }
    }
    const double G = (double)(g->npglobal[0] + 2) * (g->npglobal[1] + 2) * (g->npglobal[2] + 2);
    if (G > 4.0e9) { set_error("grid too large for the 32-bit plane indexing"); return PPS_ERR_INVALID_ARG; }
    for (int f = 0; f < 6; f++)
        if (g->bcs[f] != 0 && g->bcs[f] != 1) { set_error("bcs must be 0 (Dirichlet) or 1 (Neumann)"); return PPS_ERR_INVALID_ARG; }
    if (c->krylov != PPS_KRYLOV_BICGSTAB && c->krylov != PPS_KRYLOV_CG && c->krylov != PPS_KRYLOV_FCG &&
        c->krylov != PPS_KRYLOV_CHEBYSHEV) { set_error("unknown krylov"); return PPS_ERR_INVALID_ARG; }
    if (c->krylov == PPS_KRYLOV_CHEBYSHEV && (c->cheb_degree < 1 || c->cheb_degree > 10000)) { set_error("cheb_degree out of range"); return PPS_ERR_INVALID_ARG; }
    if (c->krylov == PPS_KRYLOV_FCG && c->form == PPS_FORM_PARITY_FP64) { set_error("flexible CG has no reference counterpart, so no PARITY form"); return PPS_ERR_UNSUPPORTED; }
    if (c->krylov == PPS_KRYLOV_FCG)
        for (int f = 0; f < 6; f++)
            if (g->bcs[f] != 0) { set_error("flexible CG takes Dirichlet grids only"); return PPS_ERR_UNSUPPORTED; }
    const bool chebmain = c->krylov == PPS_KRYLOV_CHEBYSHEV;
    const bool nested = !chebmain && (c->precond == PPS_PREC_BICGSTAB || c->precond == PPS_PREC_CG);
    if (!chebmain && c->precond != PPS_PREC_NONE && c->precond != PPS_PREC_CHEBYSHEV && !nested) { set_error("unknown precond"); return PPS_ERR_INVALID_ARG; }
    if (nested) {
        if (!(c->precond_tol > 0.0 && c->precond_tol < 1.0)) { set_error("an inner-solver preconditioner needs 0 < precond_tol < 1"); return PPS_ERR_INVALID_ARG; }
        if (c->precond_maxit < 0 || c->precond_maxit > 100000000) { set_error("precond_maxit out of range"); return PPS_ERR_INVALID_ARG; }
        if (c->precond_inner != PPS_PREC_NONE && c->precond_inner != PPS_PREC_CHEBYSHEV) { set_error("precond_inner must be none or Chebyshev"); return PPS_ERR_INVALID_ARG; }
    }
    const bool uses_cheb = !chebmain && (c->precond == PPS_PREC_CHEBYSHEV ||
                                         (nested && c->precond_inner == PPS_PREC_CHEBYSHEV));
    if (uses_cheb && (c->cheb_degree < 1 || c->cheb_degree > 10000)) { set_error("cheb_degree out of range"); return PPS_ERR_INVALID_ARG; }
    if (c->maxit < 0 || c->maxit > 100000000) { set_error("maxit out of range"); return PPS_ERR_INVALID_ARG; }
    if (!(c->tol >= 0.0)) { set_error("tol must be >= 0"); return PPS_ERR_INVALID_ARG; }
    if (c->form < PPS_FORM_PARITY_FP64 || c->form > PPS_FORM_MIXED) { set_error("unknown form"); return PPS_ERR_INVALID_ARG; }
    if (c->form == PPS_FORM_MIXED && (!(c->inner_tol > 0.0 && c->inner_tol < 1.0) || c->inner_maxit < 1 || c->max_refinements < 1)) {
        set_error("mixed form needs 0 < inner_tol < 1, inner_maxit >= 1, max_refinements >= 1");
        return PPS_ERR_INVALID_ARG;
    }
    return PPS_OK;
}

void coords(const pps_solver* s, int i, int j, int k, double* x, double* y, double* z)
{
    // iterativeSolverBase.hpp:547-549 at rank location 0
    const double* o = s->grid.origin;
    const double* d = s->grid.ds;
    *x = o[0] + (i - 1) * d[0] + 0 * (s->grid.npglobal[0]) * d[0];
    *y = o[1] + (j - 1) * d[1] + 0 * (s->grid.npglobal[1]) * d[1];
    *z = o[2] + (k - 1) * d[2] + 0 * (s->grid.npglobal[2]) * d[2];
}

template <typename Fn>
pps_status guarded(Fn&& fn)
{
    const unsigned long long f0 = launch_failures();
    try {
        const pps_status rc = fn();
        return rc >= 0 && launch_failures() != f0 ? PPS_ERR_CUDA : rc;
    } catch (const CudaFail&) {
        return PPS_ERR_CUDA;
    } catch (const std::bad_alloc&) {
        set_error("host allocation failed");
        return PPS_ERR_OUT_OF_MEMORY;
    }
}

pps_status solve_core(pps_solver* s, double* x_dev, double* b_dev)
{
    pps_stats& S = s->stats;
    const double h2d = S.seconds_h2d, d2h = S.seconds_d2h;
    std::memset(&S, 0, sizeof(S));
    S.seconds_h2d = h2d;
    S.seconds_d2h = d2h;
    s->sweep_ev_used = 0;
    s->sweep_bytes_acc = 0;
    s->sweep_launch_acc = 0;
    s->krylov_ev_used = 0;
    s->krylov_bytes_acc = 0;
    s->krylov_launch_acc = 0;
    launches_counter_reset();
    s->prec_kind = s->cfg.krylov == PPS_KRYLOV_CHEBYSHEV ? (int)PPS_PREC_CHEBYSHEV : s->cfg.precond;
    s->prec_iters = 0;
    CK(cudaEventRecord(s->ev0, s->stream));
    pps_status rc;
    if (s->cfg.krylov == PPS_KRYLOV_CHEBYSHEV) rc = solve_cheb_main(s, x_dev, b_dev);
    else if (s->cfg.form == PPS_FORM_PARITY_FP64) rc = solve_parity(s, x_dev, b_dev);
    else if (s->cfg.form == PPS_FORM_FP64) rc = solve_fp64(s, x_dev, b_dev);
    else rc = solve_mixed(s, x_dev, b_dev);
    CK(cudaEventRecord(s->ev1, s->stream));
    CK(cudaEventSynchronize(s->ev1));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, s->ev0, s->ev1));
    S.seconds_solve = ms * 1e-3;
    S.kernel_launches = launches_counter();
    // sweep timing from event pairs
    double sw = 0;
    for (int q = 0; q + 1 < s->sweep_ev_used; q += 2) {
        float m = 0;
        CK(cudaEventElapsedTime(&m, s->sweep_ev[q], s->sweep_ev[q + 1]));
        sw += m * 1e-3;
    }
    S.sweep_seconds = sw;
    S.sweep_launches = s->sweep_launch_acc;
    S.sweep_bytes = s->sweep_bytes_acc;
    double kt = 0;
    for (int q = 0; q + 1 < s->krylov_ev_used; q += 2) {
        float m = 0;
        CK(cudaEventElapsedTime(&m, s->krylov_ev[q], s->krylov_ev[q + 1]));
        kt += m * 1e-3;
    }
    S.krylov_seconds = kt;
    S.krylov_launches = s->krylov_launch_acc;
    S.krylov_bytes = s->krylov_bytes_acc;
    S.learned_applications = s->learned_apps;
    S.fallback_iteration = s->fallback_iter;
    S.precond_iterations = (int)std::min<long long>(s->prec_iters, INT32_MAX);
    return rc;
}

}  // namespace

extern "C" {

pps_status pps_config_default(pps_config* c, int preset)
{
    if (!c) return PPS_ERR_INVALID_ARG;
    std::memset(c, 0, sizeof(*c));
    c->krylov = PPS_KRYLOV_BICGSTAB;
    c->precond = PPS_PREC_CHEBYSHEV;
    if (preset == PPS_PRESET_ALPAKA) {
        // ALP/include/solverSetup.hpp:52-72
        c->cheb_degree = 24;
        c->cheb_eps = 0.0;
        c->rescale_min = 100.0;
        c->rescale_max = 1.0 - 1e-4;
        c->tol = 1.0 * 1e-10;
        c->maxit = 1000;
        c->precond_tol = (double)100000000 * 1e-10;   // tollMainSolver * 1e8 * tollScalingFactor
        c->precond_maxit = 500;
    } else if (preset == PPS_PRESET_CPU) {
        // CPU/include/solverSetup.hpp:22-40
        c->cheb_degree = 11;
        c->cheb_eps = 1e-4;
        c->rescale_min = 500.0;
        c->rescale_max = 1.0 - 1e-4;
        c->tol = (double)100 * 1e-10;
        c->maxit = 1700;
        c->precond_tol = (double)10000 * 1e-10;   // tollPreconditionerSolver * tollScalingFactor
        c->precond_maxit = 150;                    // iterMaxPreconditioner
    } else {
        return PPS_ERR_INVALID_ARG;
    }
    c->form = PPS_FORM_FP64;
    c->inner_tol = 3e-3;
    c->inner_maxit = 100000;
    c->max_refinements = 12;
    c->check_every = 0;
    c->use_graph = 1;
    c->device = 0;
    c->precond_inner = PPS_PREC_NONE;
    return PPS_OK;
}

pps_status pps_create(const pps_grid* grid, const pps_config* cfg, pps_solver** out)
{
    if (!out) return PPS_ERR_INVALID_ARG;
    *out = nullptr;
    pps_status v = validate(grid, cfg);
    if (v != PPS_OK) return v;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        set_error("no CUDA device");
        return PPS_ERR_NO_DEVICE;
    }
    if (cfg->device < 0 || cfg->device >= ndev) {
        set_error("device ordinal out of range");
        return PPS_ERR_INVALID_ARG;
    }
    pps_solver* s = new (std::nothrow) pps_solver();
    if (!s) return PPS_ERR_OUT_OF_MEMORY;
    s->grid = *grid;
    s->cfg = *cfg;
    pps_status rc = guarded([&]() -> pps_status {
        CK(cudaSetDevice(cfg->device));
        s->device = cfg->device;
        Geo& g = s->geo;
        for (int d = 0; d < 3; d++) {
            g.n[d] = grid->npglobal[d];
            g.ds[d] = grid->ds[d];
            g.lo[d] = 1 + (grid->bcs[2 * d] == 0 ? 1 : 0);
            g.hi[d] = grid->npglobal[d] + 1 - (grid->bcs[2 * d + 1] == 0 ? 1 : 0);
        }
        for (int f = 0; f < 6; f++) {
            g.bcs[f] = grid->bcs[f];
            if (grid->bcs[f] == 1) s->has_neumann = true;
        }
        g.sj = grid->npglobal[0] + 2;
        g.sk = g.sj * (grid->npglobal[1] + 2);
        g.ntot = g.sk * (grid->npglobal[2] + 2);
        s->n_unknowns = (long long)(g.hi[0] - g.lo[0]) * (g.hi[1] - g.lo[1]) * (g.hi[2] - g.lo[2]);
        s->shape = make_shape(g, 8, sm_count() * 8 * 4);
        // the Chebyshev kernels default to the x-vectorised FP32 tiles where the row
        // stride allows them (FP64 fields run the scalar tiles of the same size)
        const int cx0 = g.sj % 4 == 0 ? 4 : 1;
        s->shape_cheb = make_shape(g, 8, sm_count() * 8 * 4, cx0);
        s->tuning.cheb_ty = 8;
        s->tuning.cheb_cx = cx0;
        s->tuning.cheb_waves = 4;
        s->tuning.other_ty = 8;
        s->tuning.other_waves = 4;
        s->tuning.cheb_us = 0.0;
        s->tuning.other_us = 0.0;
        s->tuning.cheb_fused = 0;
        s->tuning.fcg_staged = 0;
        // computeEigenvalues, global bounds (blockGrid.hpp:322-339)
        double eigMin = 0, eigMax = 0;
        for (int i = 0; i < 3; i++) {
            int ni = grid->npglobal[i];
            if (grid->bcs[2 * i] == 0) ni -= 1;
            if (grid->bcs[2 * i + 1] == 0) ni -= 1;
            const double dsi = grid->ds[i];
            eigMin += 4 * sin(1 * kPi / 2 / (ni + 1)) * sin(1 * kPi / 2 / (ni + 1)) / (dsi * dsi);
            eigMax += 4 * sin(ni * kPi / 2 / (ni + 1)) * sin(ni * kPi / 2 / (ni + 1)) / (dsi * dsi);
        }
        s->eig[0] = eigMin;
        s->eig[1] = eigMax;
        // ChebyshevIteration constructor (chebyshevIteration.hpp:22-26)
        s->theta = (eigMin * cfg->rescale_min + eigMax * cfg->rescale_max) * 0.5 * (1.0 + cfg->cheb_eps);
        s->delta = (eigMin * cfg->rescale_min - eigMax * cfg->rescale_max) * 0.5;
        s->sigma = s->theta / s->delta;

        CK(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
        CK(cudaStreamCreateWithFlags(&s->copy_stream, cudaStreamNonBlocking));
        CK(cudaEventCreate(&s->ev0));
        CK(cudaEventCreate(&s->ev1));
        CK(cudaEventCreate(&s->ev_h0));
        CK(cudaEventCreate(&s->ev_b));
        for (cudaEvent_t* e : {&s->ev_x, &s->ev_upd, &s->ev_out}) CK(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
        CK(cudaMalloc((void**)&s->d_xnz, sizeof(int)));
        CK(cudaMallocHost((void**)&s->h_xnz, sizeof(int)));
        const size_t fb = sizeof(double) * (size_t)g.ntot;
        CK(cudaMalloc((void**)&s->d_x, fb));
        CK(cudaMalloc((void**)&s->d_b, fb));
        if (cfg->form == PPS_FORM_MIXED) {
            alloc_fields<float>(s->f32, g.ntot, true);
        } else {
            alloc_fields<double>(s->f64, g.ntot, false);
        }
        if (cfg->form == PPS_FORM_PARITY_FP64 || cfg->krylov == PPS_KRYLOV_CHEBYSHEV) {
            CK(cudaMalloc((void**)&s->d_bt, fb));
            CK(cudaMemset(s->d_bt, 0, fb));
        }
        if (cfg->form == PPS_FORM_PARITY_FP64) {
            s->pY = s->f64.Y;
            s->pZ = s->f64.Z;
            s->pW = s->f64.W;
        }
        if (cfg->krylov != PPS_KRYLOV_CHEBYSHEV && (cfg->precond == PPS_PREC_BICGSTAB || cfg->precond == PPS_PREC_CG)) {
            // the inner solver's fields; its Chebyshev buffers only where the fast
            // forms apply a Chebyshev polynomial inside it (PARITY uses pY, pZ, pW)
            const bool cheb_in = cfg->precond_inner == PPS_PREC_CHEBYSHEV && cfg->form != PPS_FORM_PARITY_FP64;
            if (cfg->form == PPS_FORM_MIXED) alloc_fields<float>(s->in32, g.ntot, false, cheb_in);
            else alloc_fields<double>(s->in64, g.ntot, false, cheb_in);
            CK(cudaMalloc((void**)&s->d_st_in, sizeof(DevState)));
            CK(cudaMemset(s->d_st_in, 0, sizeof(DevState)));
            CK(cudaMallocHost((void**)&s->h_st_in, sizeof(DevState)));
        }
        CK(cudaMalloc((void**)&s->d_dot, 4 * sizeof(double)));
        CK(cudaMalloc((void**)&s->d_st, sizeof(DevState)));
        CK(cudaMemset(s->d_st, 0, sizeof(DevState)));
        CK(cudaMallocHost((void**)&s->h_st, sizeof(DevState)));
        CK(cudaMallocHost((void**)&s->h_dot, 4 * sizeof(double)));
        {   // the host polls read the Krylov scalars through the mapping of h_st (read_state)
            bool mapped = true;
            for (DevState* h : {s->h_st, s->h_st_in}) {
                if (!h) continue;
                void* dp = nullptr;
                mapped = mapped && cudaHostGetDevicePointer(&dp, h, 0) == cudaSuccess && dp == (void*)h;
            }
            void* dp = nullptr;
            s->xnz_mapped = cudaHostGetDevicePointer(&dp, s->h_xnz, 0) == cudaSuccess && dp == (void*)s->h_xnz;
            cudaGetLastError();
            s->state_mapped = mapped;
        }
        s->hist_cap = cfg->maxit + 2;
        CK(cudaMalloc((void**)&s->d_hist, sizeof(double) * (size_t)s->hist_cap));
        const unsigned nb = std::max(max_candidate_blocks(g), 128u);   // 128: the canonical sums' blocks
        CK(cudaMalloc((void**)&s->d_partials, sizeof(double) * 4 * (size_t)nb));
        if (cfg->form == PPS_FORM_FP64)
            CK(cudaMalloc((void**)&s->d_cells, sizeof(double) * 3 * (size_t)canon_cells(g)));
        CK(cudaMalloc((void**)&s->d_counter, sizeof(unsigned)));
        CK(cudaMemset(s->d_counter, 0, sizeof(unsigned)));
        for (int f = 0; f < 6; f++) {
            if (grid->bcs[f] != 1) continue;
            const long long m = face_count(s, f);
            CK(cudaMalloc((void**)&s->d_faces[f], sizeof(double) * (size_t)m));
            CK(cudaMemset(s->d_faces[f], 0, sizeof(double) * (size_t)m));
        }
        if (cfg->use_graph == 0) {
            const int pairs = 2 * (cfg->maxit + 2) + 64;
            s->sweep_ev.resize((size_t)std::min(pairs, 20000) * 2);
            for (auto& e : s->sweep_ev) CK(cudaEventCreate(&e));
            s->krylov_ev.resize((size_t)std::min(cfg->maxit + 2, 2000) * 2);
            for (auto& e : s->krylov_ev) CK(cudaEventCreate(&e));
        }
        // the zero fills above ran on the legacy stream, which the handle's non-blocking
        // stream does not wait for: finish them before the handle is used
        CK(cudaDeviceSynchronize());
        std::memset(&s->stats, 0, sizeof(s->stats));
        return PPS_OK;
    });
    if (rc != PPS_OK) {
        free_all(s);
        delete s;
        return rc == PPS_ERR_CUDA ? PPS_ERR_OUT_OF_MEMORY : rc;
    }
    *out = s;
    return PPS_OK;
}

pps_status pps_destroy(pps_solver* s)
{
    if (!s) return PPS_ERR_INVALID_ARG;
    cudaSetDevice(s->device);
    cudaStreamSynchronize(s->stream);
    cudaStreamSynchronize(s->copy_stream);
    free_all(s);
    delete s;
    return PPS_OK;
}

pps_status pps_set_problem(pps_solver* s, const pps_problem* p, double* x, double* b)
{
    if (!s || !p || !x || !b || !p->field_b || !p->solution) return PPS_ERR_INVALID_ARG;
    const int* n = s->grid.npglobal;
    const long long sj = n[0] + 2, sk = sj * (n[1] + 2);
    // applyDirichletBCsFromFunction (iterativeSolverBase.hpp:557-603)
    for (int f = 0; f < 6; f++) {
        if (s->grid.bcs[f] != 0) continue;
        const int d = f / 2, side = f % 2;
        int lo[3] = {1, 1, 1}, hi[3] = {n[0] + 1, n[1] + 1, n[2] + 1};
        if (side == 0) hi[d] = lo[d] + 1;
        else lo[d] = hi[d] - 1;
        for (int k = lo[2]; k < hi[2]; k++)
            for (int j = lo[1]; j < hi[1]; j++)
                for (int i = lo[0]; i < hi[0]; i++) {
                    double cx, cy, cz;
                    coords(s, i, j, k, &cx, &cy, &cz);
                    x[i + sj * j + sk * k] = p->solution(cx, cy, cz, p->ctx);
                }
    }
    // setFieldValuefromFunction (iterativeSolverBase.hpp:537-555)
    for (int k = 1; k <= n[2]; k++)
        for (int j = 1; j <= n[1]; j++)
            for (int i = 1; i <= n[0]; i++) {
                double cx, cy, cz;
                coords(s, i, j, k, &cx, &cy, &cz);
                b[i + sj * j + sk * k] = p->field_b(cx, cy, cz, p->ctx);
            }
    // Neumann face data from trueSolutionDdir
    if (s->has_neumann) {
        if (!p->solution_ddir) return PPS_ERR_INVALID_ARG;
        for (int f = 0; f < 6; f++) {
            if (s->grid.bcs[f] != 1) continue;
            const int d = f / 2, side = f % 2;
            const int a0 = d == 0 ? 1 : 0, a1 = d == 2 ? 1 : 2;
            std::vector<double> vals((size_t)face_count(s, f));
            for (int ib = 1; ib <= n[a1]; ib++)
                for (int ia = 1; ia <= n[a0]; ia++) {
                    int idx[3];
                    idx[d] = side == 0 ? 1 : n[d];
                    idx[a0] = ia;
                    idx[a1] = ib;
                    double cx, cy, cz;
                    coords(s, idx[0], idx[1], idx[2], &cx, &cy, &cz);
                    vals[(size_t)(ia - 1) + (size_t)n[a0] * (ib - 1)] = p->solution_ddir(cx, cy, cz, d, p->ctx);
                }
            pps_status rc = pps_set_neumann(s, f, vals.data());
            if (rc != PPS_OK) return rc;
        }
    }
    return PPS_OK;
}

pps_status pps_set_problem_builtin(pps_solver* s, int which, double* x, double* b)
{
    if (which != PPS_PROBLEM_REFERENCE_DEFAULT && which != PPS_PROBLEM_SINE) return PPS_ERR_INVALID_ARG;
    static const int ids[2] = {0, 1};
    pps_problem p;
    p.field_b = builtin_f;
    p.solution = builtin_u;
    p.solution_ddir = builtin_du;
    p.ctx = (void*)&ids[which];
    return pps_set_problem(s, &p, x, b);
}

pps_status pps_set_neumann(pps_solver* s, int face, const double* values)
{
    if (!s || face < 0 || face > 5 || !values) return PPS_ERR_INVALID_ARG;
    if (s->grid.bcs[face] != 1) {
        set_error("face is not a Neumann face");
        return PPS_ERR_INVALID_ARG;
    }
    return guarded([&]() -> pps_status {
        CK(cudaSetDevice(s->device));
        CK(cudaMemcpyAsync(s->d_faces[face], values, sizeof(double) * (size_t)face_count(s, face),
                           cudaMemcpyHostToDevice, s->stream));
        CK(cudaStreamSynchronize(s->stream));
        return PPS_OK;
    });
}

// A host array the copy engines and kernels reach directly (page-locked, registered)
bool is_pinned(const void* p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

pps_status pps_solve(pps_solver* s, double* x, double* b, pps_stats* stats)
{
    if (!s || !x || !b) return PPS_ERR_INVALID_ARG;
    const auto t0 = std::chrono::steady_clock::now();
    pps_status rc = guarded([&]() -> pps_status {
        CK(cudaSetDevice(s->device));
        const size_t fb = sizeof(double) * (size_t)s->geo.ntot;
        // copy_stream's work on the caller's arrays ends before the call returns, an
        // error included
        struct Drain {
            pps_solver* s;
            ~Drain()
            {
                cudaStreamSynchronize(s->copy_stream);
                s->spec_x = false;
                s->out_host = nullptr;
                s->out_issued = s->out_current = false;
            }
        } drain{s};
        s->spec_restarted = false;
        // MIXED form on pinned arrays (Dirichlet faces, no learned initial guess): b
        // first, then the solve on it as if x were zero while x uploads behind it, and
        // x's copy out overlapping the final residual check.  The link carries one
        // array at a time at the same rate whichever engine drives it, so the gain is
        // the copies hidden behind device work.
        const bool overlap = s->cfg.form == PPS_FORM_MIXED && s->cfg.krylov != PPS_KRYLOV_CHEBYSHEV &&
                             !s->has_neumann && !(s->net && (s->net_flags & PPS_LEARNED_INITIAL_GUESS)) &&
                             is_pinned(x) && is_pinned(b);
        const auto a = std::chrono::steady_clock::now();
        if (overlap) {
            CK(cudaEventRecord(s->ev_h0, s->stream));
            CK(cudaMemcpyAsync(s->d_b, b, fb, cudaMemcpyHostToDevice, s->stream));
            CK(cudaEventRecord(s->ev_b, s->stream));
            CK(cudaStreamWaitEvent(s->copy_stream, s->ev_b, 0));   // x follows b on the link
            CK(cudaMemcpyAsync(s->d_x, x, fb, cudaMemcpyHostToDevice, s->copy_stream));
            if (s->xnz_mapped) {   // the test's flag stored through its mapping
                *(volatile int*)s->h_xnz = 0;
                flag_nonzero(s->geo.ntot, s->d_x, s->h_xnz, s->copy_stream);
            } else {
                CK(cudaMemsetAsync(s->d_xnz, 0, sizeof(int), s->copy_stream));
                flag_nonzero(s->geo.ntot, s->d_x, s->d_xnz, s->copy_stream);
                CK(cudaMemcpyAsync(s->h_xnz, s->d_xnz, sizeof(int), cudaMemcpyDeviceToHost, s->copy_stream));
            }
            CK(cudaEventRecord(s->ev_x, s->copy_stream));
            s->spec_x = true;
            s->out_host = x;
            s->stats.seconds_h2d = 0;
        } else {
            CK(cudaMemcpyAsync(s->d_x, x, fb, cudaMemcpyHostToDevice, s->stream));
            CK(cudaMemcpyAsync(s->d_b, b, fb, cudaMemcpyHostToDevice, s->stream));
            CK(cudaStreamSynchronize(s->stream));
            s->stats.seconds_h2d = std::chrono::duration<double>(std::chrono::steady_clock::now() - a).count();
        }
        s->stats.seconds_d2h = 0;
        pps_status r = solve_core(s, s->d_x, s->d_b);
        if (overlap) s->stats.kernel_launches += 1;   // the test of x, launched before the count restarted
        if (r < 0) return r;
        const auto c = std::chrono::steady_clock::now();
        if (!(overlap && s->out_current)) {
            if (s->out_issued) CK(cudaStreamWaitEvent(s->stream, s->ev_out, 0));
            CK(cudaMemcpyAsync(x, s->d_x, fb, cudaMemcpyDeviceToHost, s->stream));
        }
        if (s->cfg.form == PPS_FORM_PARITY_FP64)
            CK(cudaMemcpyAsync(b, s->d_b, fb, cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
        CK(cudaStreamSynchronize(s->copy_stream));
        s->stats.seconds_d2h = std::chrono::duration<double>(std::chrono::steady_clock::now() - c).count();
        if (overlap) {
            float ms = 0;
            CK(cudaEventElapsedTime(&ms, s->ev_h0, s->ev_b));
            s->stats.seconds_h2d = ms * 1e-3;
            s->stats.copy_overlap = 1 | (s->spec_restarted ? 2 : 0) | (s->out_current ? 4 : 0);
        }
        return r;
    });
    s->stats.seconds_total = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (stats) *stats = s->stats;
    return rc;
}

pps_status pps_solve_device(pps_solver* s, double* x_dev, double* b_dev, pps_stats* stats)
{
    if (!s || !x_dev || !b_dev) return PPS_ERR_INVALID_ARG;
    const auto t0 = std::chrono::steady_clock::now();
    pps_status rc = guarded([&]() -> pps_status {
        CK(cudaSetDevice(s->device));
        s->stats.seconds_h2d = 0;
        s->stats.seconds_d2h = 0;
        return solve_core(s, x_dev, b_dev);
    });
    s->stats.seconds_total = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (stats) *stats = s->stats;
    return rc;
}

pps_status pps_get_stats(const pps_solver* s, pps_stats* stats)
{
    if (!s || !stats) return PPS_ERR_INVALID_ARG;
    *stats = s->stats;
    return PPS_OK;
}

pps_status pps_get_history(const pps_solver* s, double* out, int cap, int* count)
{
    if (!s || !count || cap < 0 || (cap > 0 && !out)) return PPS_ERR_INVALID_ARG;
    const int n = (int)std::min<size_t>(s->history.size(), (size_t)cap);
    for (int i = 0; i < n; i++) out[i] = s->history[(size_t)i];
    *count = (int)s->history.size();
    return PPS_OK;
}

pps_status pps_write_residual_history(const pps_solver* s, const char* path)
{
    // Format of iterativeSolverBaseAlpaka.hpp:620-638: solver time, iterations,
    // preconditioner iterations (an inner solver's, summed; otherwise the number of
    // applications), then one residual per line.
    if (!s || !path) return PPS_ERR_INVALID_ARG;
    FILE* f = fopen(path, "w");
    if (!f) {
        set_error(std::string("cannot open ") + path);
        return PPS_ERR_INVALID_ARG;
    }
    const bool nested = s->cfg.krylov != PPS_KRYLOV_CHEBYSHEV &&
                        (s->cfg.precond == PPS_PREC_BICGSTAB || s->cfg.precond == PPS_PREC_CG);
    fprintf(f, "%.17g\n%d\n%d\n", s->stats.seconds_solve, s->stats.iterations,
            nested ? s->stats.precond_iterations : s->stats.precond_applications);
    for (double v : s->history) fprintf(f, "%.17g\n", v);
    fclose(f);
    return PPS_OK;
}

pps_status pps_write_solution(const pps_grid* grid, const double* x, int rank, const char* path, void* stream)
{
    // solution.dat of the alpaka driver (ALP/src/main.cpp:135-146): the rank's whole
    // guard-padded field, raw doubles in memory order, at byte offset rank * G * 8 of
    // the file, which is created if missing and otherwise not truncated
    // (MPI_MODE_CREATE | MPI_MODE_WRONLY), so the ranks' blocks can share one file.
    if (!grid || !x || !path || rank < 0) return PPS_ERR_INVALID_ARG;
    for (int d = 0; d < 3; d++)
        if (grid->npglobal[d] < 1) {
            set_error("npglobal must be >= 1");
            return PPS_ERR_INVALID_ARG;
        }
    const long long G = (long long)(grid->npglobal[0] + 2) * (grid->npglobal[1] + 2) * (grid->npglobal[2] + 2);
    cudaPointerAttributes at{};
    const bool on_device = cudaPointerGetAttributes(&at, x) == cudaSuccess && at.type == cudaMemoryTypeDevice;
    cudaGetLastError();   // a host pointer unknown to CUDA is not an error here
    FILE* f = fopen(path, "r+b");
    if (!f) f = fopen(path, "wb");
    if (!f) {
        set_error(std::string("cannot open ") + path);
        return PPS_ERR_INVALID_ARG;
    }
    pps_status rc = PPS_OK;
    if (fseeko(f, (off_t)rank * (off_t)G * (off_t)sizeof(double), SEEK_SET) != 0) {
        set_error(std::string("cannot seek in ") + path);
        rc = PPS_ERR_INVALID_ARG;
    } else if (!on_device) {
        if (fwrite(x, sizeof(double), (size_t)G, f) != (size_t)G) {
            set_error(std::string("short write to ") + path);
            rc = PPS_ERR_INVALID_ARG;
        }
    } else {
        // device field: staged through pinned chunks, copied on the caller's stream so
        // they follow the work that produced x
        rc = guarded([&]() -> pps_status {
            CK(cudaSetDevice(at.device));
            cudaStream_t st = (cudaStream_t)stream;
            const long long chunk = std::min<long long>(G, 8LL << 20);
            double* stage = nullptr;
            CK(cudaMallocHost((void**)&stage, sizeof(double) * (size_t)chunk));
            pps_status r = PPS_OK;
            for (long long off = 0; off < G && r == PPS_OK; off += chunk) {
                const long long n = std::min(chunk, G - off);
                cudaError_t e = cudaMemcpyAsync(stage, x + off, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, st);
                if (e == cudaSuccess) e = cudaStreamSynchronize(st);
                if (e != cudaSuccess) {
                    set_error(std::string("copying the solution: ") + cudaGetErrorString(e));
                    r = PPS_ERR_CUDA;
                } else if (fwrite(stage, sizeof(double), (size_t)n, f) != (size_t)n) {
                    set_error(std::string("short write to ") + path);
                    r = PPS_ERR_INVALID_ARG;
                }
            }
            cudaFreeHost(stage);
            return r;
        });
    }
    if (fclose(f) != 0 && rc == PPS_OK) {
        set_error(std::string("cannot close ") + path);
        rc = PPS_ERR_INVALID_ARG;
    }
    return rc;
}

pps_status pps_apply_operator(pps_solver* s, const double* u, double* out)
{
    if (!s || !u || !out) return PPS_ERR_INVALID_ARG;
    return guarded([&]() -> pps_status {
        CK(cudaSetDevice(s->device));
        const size_t fb = sizeof(double) * (size_t)s->geo.ntot;
        CK(cudaMemcpyAsync(s->d_x, u, fb, cudaMemcpyHostToDevice, s->stream));
        CK(cudaMemcpyAsync(s->d_b, out, fb, cudaMemcpyHostToDevice, s->stream));
        if (s->cfg.form == PPS_FORM_PARITY_FP64) {
            par_stencil(s->geo, s->d_x, s->d_b, s->stream);
        } else {
            state_init(s->d_st, s->d_hist, 0, 0.0, 0.0, 0, 0, 1.0, 0, s->stream);
            // A u = b - (b - A u): use the residual kernel with b = 0 and negate via a second pass
            double* tmp = s->cfg.form == PPS_FORM_MIXED ? nullptr : s->f64.Az;
            if (tmp) {
                CK(cudaMemsetAsync(tmp, 0, fb, s->stream));
                fast_stencil_dot<double>(s->geo, s->shape, s->d_x, tmp, s->d_b, op_coef(s->geo),
                                         red(s, FIN_STORE), s->stream);
            } else {
                float* t32 = s->f32.Az;
                float* u32 = s->f32.Y;
                float* o32 = s->f32.W;
                // FP32 operator on the rounded input
                std::vector<float> hu((size_t)s->geo.ntot), ho((size_t)s->geo.ntot);
                for (long long q = 0; q < s->geo.ntot; q++) hu[(size_t)q] = (float)u[q];
                CK(cudaMemcpyAsync(u32, hu.data(), sizeof(float) * (size_t)s->geo.ntot, cudaMemcpyHostToDevice, s->stream));
                CK(cudaMemsetAsync(t32, 0, sizeof(float) * (size_t)s->geo.ntot, s->stream));
                CK(cudaMemsetAsync(o32, 0, sizeof(float) * (size_t)s->geo.ntot, s->stream));
                fast_stencil_dot<float>(s->geo, s->shape, u32, t32, o32, op_coef(s->geo), red(s, FIN_STORE), s->stream);
                CK(cudaMemcpyAsync(ho.data(), o32, sizeof(float) * (size_t)s->geo.ntot, cudaMemcpyDeviceToHost, s->stream));
                CK(cudaStreamSynchronize(s->stream));
                const long long sj = s->geo.sj, sk = s->geo.sk;
                for (int k = s->geo.lo[2]; k < s->geo.hi[2]; k++)
                    for (int j = s->geo.lo[1]; j < s->geo.hi[1]; j++)
                        for (int i = s->geo.lo[0]; i < s->geo.hi[0]; i++) {
                            const long long c = i + sj * j + sk * k;
                            out[c] = (double)ho[(size_t)c];
                        }
                return PPS_OK;
            }
        }
        CK(cudaMemcpyAsync(out, s->d_b, fb, cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
        return PPS_OK;
    });
}

pps_status pps_apply_preconditioner(pps_solver* s, const double* B, double* X)
{
    if (!s || !B || !X) return PPS_ERR_INVALID_ARG;
    return guarded([&]() -> pps_status {
        CK(cudaSetDevice(s->device));
        const Geo& g = s->geo;
        const size_t fb = sizeof(double) * (size_t)g.ntot;
        s->prec_kind = s->cfg.krylov == PPS_KRYLOV_CHEBYSHEV ? (int)PPS_PREC_CHEBYSHEV : s->cfg.precond;
        if (s->cfg.form == PPS_FORM_PARITY_FP64) {
            CK(cudaMemcpyAsync(s->d_b, B, fb, cudaMemcpyHostToDevice, s->stream));
            CK(cudaMemcpyAsync(s->d_x, X, fb, cudaMemcpyHostToDevice, s->stream));
            par_precond(s, s->d_b, s->d_x);
            CK(cudaMemcpyAsync(X, s->d_x, fb, cudaMemcpyDeviceToHost, s->stream));
            CK(cudaStreamSynchronize(s->stream));
            return PPS_OK;
        }
        state_init(s->d_st, s->d_hist, 0, 0.0, 0.0, 0, 0, 1.0, 0, s->stream);
        Launcher L{s, false};
        // B and X pass through the solver's own r and z, whole (boundary nodes and
        // guards included, as the caller gave them); afterwards those entries are
        // zeroed again, the state the solves expect of their work fields.
        if (s->cfg.form == PPS_FORM_FP64) {
            CK(cudaMemcpyAsync(s->f64.r, B, fb, cudaMemcpyHostToDevice, s->stream));
            CK(cudaMemcpyAsync(s->f64.z, X, fb, cudaMemcpyHostToDevice, s->stream));
            precond_once<double>(s, s->f64, s->f64.r, s->f64.z, L);
            CK(cudaMemcpyAsync(X, s->f64.z, fb, cudaMemcpyDeviceToHost, s->stream));
            zero_off_unknowns<double>(g, s->f64.r, s->stream);
            zero_off_unknowns<double>(g, s->f64.z, s->stream);
            CK(cudaStreamSynchronize(s->stream));
            return PPS_OK;
        }
        std::vector<float> hb((size_t)g.ntot), hx((size_t)g.ntot);
        for (long long q = 0; q < g.ntot; q++) {
            hb[(size_t)q] = (float)B[q];
            hx[(size_t)q] = (float)X[q];
        }
        CK(cudaMemcpyAsync(s->f32.r, hb.data(), sizeof(float) * (size_t)g.ntot, cudaMemcpyHostToDevice, s->stream));
        CK(cudaMemcpyAsync(s->f32.z, hx.data(), sizeof(float) * (size_t)g.ntot, cudaMemcpyHostToDevice, s->stream));
        precond_once<float>(s, s->f32, s->f32.r, s->f32.z, L);
        CK(cudaMemcpyAsync(hx.data(), s->f32.z, sizeof(float) * (size_t)g.ntot, cudaMemcpyDeviceToHost, s->stream));
        zero_off_unknowns<float>(g, s->f32.r, s->stream);
        zero_off_unknowns<float>(g, s->f32.z, s->stream);
        CK(cudaStreamSynchronize(s->stream));
        for (long long q = 0; q < g.ntot; q++) X[q] = (double)hx[(size_t)q];
        return PPS_OK;
    });
}

pps_status pps_autotune(pps_solver* s, pps_tuning* out)
{
    if (!s) return PPS_ERR_INVALID_ARG;
    if (s->cfg.form == PPS_FORM_PARITY_FP64) {
        set_error("the PARITY form has no tunable tile shapes");
        return PPS_ERR_UNSUPPORTED;
    }
    return guarded([&]() -> pps_status {
        CK(cudaSetDevice(s->device));
        pps_tuning t = s->tuning;
        if (s->cfg.form == PPS_FORM_MIXED) autotune_fields<float>(s, s->f32, &t);
        else autotune_fields<double>(s, s->f64, &t);
        CK(cudaStreamSynchronize(s->stream));
        apply_tuning(s, t);
        if (out) *out = t;
        return PPS_OK;
    });
}

pps_status pps_set_learned(pps_solver* s, pps_unet* net, int coarsen, double gain, int flags)
{
    if (!s) return PPS_ERR_INVALID_ARG;
    return guarded([&]() -> pps_status {
        CK(cudaSetDevice(s->device));
        if (s->gexec) {   // a captured iteration holds the old buffers and settings
            cudaGraphExecDestroy(s->gexec);
            s->gexec = nullptr;
        }
        for (float* q : s->dn) cudaFree(q);
        for (float* q : s->dn_e) cudaFree(q);
        for (float* q : s->dt) cudaFree(q);
        for (float* q : {s->cY, s->cZ, s->cW, s->d_exact}) cudaFree(q);
        s->dn.clear();
        s->dn_e.clear();
        s->dt.clear();
        s->cY = s->cZ = s->cW = s->d_exact = nullptr;
        s->coarse_kind = PPS_COARSE_NETWORK;
        s->net = nullptr;
        if (!net) return PPS_OK;   // detach
        if (s->cfg.form == PPS_FORM_PARITY_FP64) {
            set_error("the learned preconditioner has no reference counterpart, so no PARITY form");
            return PPS_ERR_UNSUPPORTED;
        }
        if (s->has_neumann) {
            set_error("the learned preconditioner takes Dirichlet grids only");
            return PPS_ERR_UNSUPPORTED;
        }
        if (coarsen < 0 || coarsen > 8 || !(gain > 0.0) || (flags & ~15) != 0 || (flags & 3) == 0) {
            set_error("coarsen 0..8, gain > 0, flags must include PPS_LEARNED_INITIAL_GUESS or _PRECONDITIONER");
            return PPS_ERR_INVALID_ARG;
        }
        const Geo& g = s->geo;
        const int need = 4 << coarsen;
        for (int d = 0; d < 3; d++)
            if ((g.hi[d] - g.lo[d]) % need != 0) {
                set_error("the unknown extents must be multiples of 4 * 2^coarsen for the U-Net");
                return PPS_ERR_INVALID_ARG;
            }
        if (g.hi[1] - g.lo[1] > 65535 || g.hi[2] - g.lo[2] > 65535) {
            set_error("the learned preconditioner takes at most 65535 unknowns along y and z");
            return PPS_ERR_INVALID_ARG;
        }
        s->net = net;
        s->net_coarsen = coarsen;
        s->net_gain = (float)gain;
        s->net_flags = flags;
        // dense levels 1..coarsen (level 0 too when the network runs on the fine grid)
        for (int l = 0; l <= coarsen; l++) {
            float *a = nullptr, *e = nullptr;
            if (l > 0 || coarsen == 0) {
                const unet::Dims d = dense_dims(s, l);
                const size_t n = (size_t)d.D * d.H * d.W;
                CK(cudaMalloc((void**)&a, sizeof(float) * n));
                CK(cudaMalloc((void**)&e, sizeof(float) * n));
            }
            s->dn.push_back(a);
            s->dn_e.push_back(e);
        }
        // residuals of the intermediate levels 1..coarsen-1 and the Chebyshev buffers
        // of the multigrid cycle (sized for level 1)
        for (int l = 0; l < coarsen; l++) {
            float* t = nullptr;
            if (l > 0) {
                const unet::Dims d = dense_dims(s, l);
                CK(cudaMalloc((void**)&t, sizeof(float) * (size_t)d.D * d.H * d.W));
            }
            s->dt.push_back(t);
        }
        if (coarsen >= 2) {
            const unet::Dims d = dense_dims(s, 1);
            const size_t n = (size_t)d.D * d.H * d.W;
            CK(cudaMalloc((void**)&s->cY, sizeof(float) * n));
            CK(cudaMalloc((void**)&s->cZ, sizeof(float) * n));
            CK(cudaMalloc((void**)&s->cW, sizeof(float) * n));
        }
        return PPS_OK;
    });
}

pps_status pps_set_learned_cycle(pps_solver* s, int fine_degree, int coarse_degree, double ratio)
{
    if (!s) return PPS_ERR_INVALID_ARG;
    const bool fine_ok = fine_degree == 0 || (fine_degree >= 2 && fine_degree <= 64);
    const bool coarse_ok = coarse_degree == 0 || (coarse_degree >= 2 && coarse_degree <= 64);
    if (!fine_ok || !coarse_ok || !(ratio > 1.0)) {
        set_error("smoother degrees 0 or 2..64, ratio > 1");
        return PPS_ERR_INVALID_ARG;
    }
    s->cyc_fine = fine_degree;
    s->cyc_coarse = coarse_degree;
    s->cyc_ratio = ratio;
    if (s->gexec) {   // a captured iteration holds the old cycle
        cudaGraphExecDestroy(s->gexec);
        s->gexec = nullptr;
    }
    return PPS_OK;
}

pps_status pps_set_coarse_solver(pps_solver* s, int kind)
{
    if (!s) return PPS_ERR_INVALID_ARG;
    return guarded([&]() -> pps_status {
        if (kind < PPS_COARSE_NETWORK || kind > PPS_COARSE_EXACT) {
            set_error("coarse solver: PPS_COARSE_NETWORK, _ZERO, _SMOOTH or _EXACT");
            return PPS_ERR_INVALID_ARG;
        }
        if (kind != PPS_COARSE_NETWORK && !s->net) {
            set_error("attach the network (pps_set_learned) before choosing its coarse-level alternative");
            return PPS_ERR_INVALID_ARG;
        }
        if (kind == PPS_COARSE_SMOOTH && s->cyc_coarse < 2) {
            set_error("PPS_COARSE_SMOOTH needs coarse_degree >= 2 (pps_set_learned_cycle)");
            return PPS_ERR_INVALID_ARG;
        }
        CK(cudaSetDevice(s->device));
        if (kind == PPS_COARSE_EXACT && !s->d_exact) {
            const int k = s->net_coarsen;
            std::vector<float> mats;
            if (!unet::level_exact_data(dense_dims(s, k), level_op(s, k), mats)) {
                set_error("PPS_COARSE_EXACT takes at most 32 unknowns per axis on the coarsest level");
                return PPS_ERR_INVALID_ARG;
            }
            CK(unet::level_exact_prepare());
            CK(cudaMalloc((void**)&s->d_exact, sizeof(float) * mats.size()));
            CK(cudaMemcpyAsync(s->d_exact, mats.data(), sizeof(float) * mats.size(), cudaMemcpyHostToDevice,
                               s->stream));
            CK(cudaStreamSynchronize(s->stream));
        }
        s->coarse_kind = kind;
        if (s->gexec) {   // a captured iteration holds the old coarse solver
            cudaGraphExecDestroy(s->gexec);
            s->gexec = nullptr;
        }
        return PPS_OK;
    });
}

pps_status pps_get_tuning(const pps_solver* s, pps_tuning* out)
{
    if (!s || !out) return PPS_ERR_INVALID_ARG;
    *out = s->tuning;
    return PPS_OK;
}

pps_status pps_set_tuning(pps_solver* s, const pps_tuning* t)
{
    if (!s || !t) return PPS_ERR_INVALID_ARG;
    if (!tuning_valid(t)) {
        set_error("tuning outside the candidate set (ty 2/4/8, cx 1/2, waves 1/2/4/8)");
        return PPS_ERR_INVALID_ARG;
    }
    apply_tuning(s, *t);
    return PPS_OK;
}

int pps_device_count(void)
{
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) return 0;
    return n;
}

const char* pps_status_string(pps_status st)
{
    switch (st) {
    case PPS_OK: return "ok";
    case PPS_NOT_CONVERGED: return "not converged (iteration cap reached)";
    case PPS_BREAKDOWN: return "Krylov breakdown";
    case PPS_NAN_DETECTED: return "NaN/Inf in the residual";
    case PPS_TIMEOUT: return "device wait timed out";
    case PPS_ERR_INVALID_ARG: return "invalid argument";
    case PPS_ERR_CUDA: return "CUDA error";
    case PPS_ERR_OUT_OF_MEMORY: return "out of memory";
    case PPS_ERR_ZERO_RHS: return "zero right-hand side";
    case PPS_ERR_UNSUPPORTED: return "unsupported";
    case PPS_ERR_NO_DEVICE: return "no CUDA device";
    }
    return "unknown status";
}

const char* pps_last_error(void) { return g_last_error.c_str(); }

void pps_internal_set_error(const char* msg) { set_error(msg ? msg : ""); }

int pps_abi_version(void) { return PPS_ABI_VERSION; }

}  // extern "C"
