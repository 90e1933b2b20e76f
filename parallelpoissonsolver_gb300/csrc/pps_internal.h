// Internal declarations shared by the kernel and solver translation units of libpps.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/pps.h"

// Records the message pps_last_error() returns on this thread.
extern "C" void pps_internal_set_error(const char* msg);

namespace pps {

// Programmatic dependent launch.  Kernels go onto the stream with
// cudaLaunchAttributeProgrammaticStreamSerialization, so the next kernel's blocks
// can be dispatched while the current one drains instead of after it completed.
// Every kernel of the library begins with pdl_enter(): it lets the next kernel
// launch (griddepcontrol.launch_dependents) and then waits until the kernel before
// it has completed with its memory visible (griddepcontrol.wait), before touching
// any global memory.  The wait is transitive along the stream, and it returns at
// once when the kernel was launched without the attribute.
#ifdef __CUDACC__
__device__ __forceinline__ void pdl_enter()
{
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    asm volatile("griddepcontrol.wait;" ::: "memory");
}
#endif
// Kernel launches that failed on this thread.  A failed launch leaves no sticky CUDA
// error for a later synchronisation to report, so the entry points compare this count
// before and after their work and return PPS_ERR_CUDA when it grew.
unsigned long long launch_failures();
void note_launch_failure(cudaError_t e);

template <typename... KArgs, typename... Args>
inline void launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, Args&&... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const cudaError_t e = cudaLaunchKernelEx(&cfg, kernel, static_cast<Args&&>(args)...);
    if (e != cudaSuccess) note_launch_failure(e);
}

// Ends a stream capture that an error left open, dropping the partial graph, so the
// stream does not stay in capture mode and fail every later call on it.  end()
// closes the capture normally.
struct CaptureGuard {
    cudaStream_t stream;
    bool open = true;
    explicit CaptureGuard(cudaStream_t s) : stream(s) {}
    CaptureGuard(const CaptureGuard&) = delete;
    CaptureGuard& operator=(const CaptureGuard&) = delete;
    cudaError_t end(cudaGraph_t* g)
    {
        open = false;
        return cudaStreamEndCapture(stream, g);
    }
    ~CaptureGuard()
    {
        if (!open) return;
        cudaGraph_t g = nullptr;
        cudaStreamEndCapture(stream, &g);
        if (g) cudaGraphDestroy(g);
    }
};

// Cooperative launch (every block resident at once, so blocks may wait on one another
// through a grid barrier); no programmatic dependent launch: the kernel starts after
// the one before it has completed.
template <typename... KArgs, typename... Args>
inline void launch_coop(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, Args&&... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const cudaError_t e = cudaLaunchKernelEx(&cfg, kernel, static_cast<Args&&>(args)...);
    if (e != cudaSuccess) note_launch_failure(e);
}

// Geometry of one single-rank grid in the guard-padded field layout
// (iterativeSolverBase.hpp:34-35): index = i + sj*j + sk*k with
// 0 <= i < n0+2 etc.; data nodes are 1..n, unknowns lo..hi-1 (blockGrid.hpp:184-222).
struct Geo {
    int n[3];
    int lo[3], hi[3];
    long long sj, sk, ntot;
    double ds[3];
    int bcs[6];
};

// Launch shape of the z-marching kernels: tiles of (32 x ty) columns in (i, j),
// each thread walks kchunk planes along k.
struct Shape {
    int ty;
    int cx;           // columns per thread along x (tile width 32*cx); Chebyshev kernels only;
                      // 4: the x-vectorised FP32 tiles (one float4 per thread, aligned to x = 0)
    int ntx, nty, nchunks, kchunk;
    unsigned nblocks() const { return (unsigned)ntx * (unsigned)nty * (unsigned)nchunks; }
};

// Device-resident Krylov scalars: the recurrences run on the device so an
// iteration needs no host round trip (the alpaka reference copies scalars to the
// host three times per iteration, BiCGstabAlpaka.hpp:254-255,343-344,395-396).
struct DevState {
    double rho0;      // rho_k (BiCGSTAB.hpp:127,259) or r.z (CG)
    double alpha, omega, beta;
    double err;       // recursive residual norm (unscaled system)
    double err0;      // initial true residual norm of this (inner) solve
    double tol_abs;   // stop when err < tol_abs
    double hist_scale;// history entries are err * hist_scale (1/||b_adj||)
    double normb;     // ||b_adj||
    double sums[4];   // raw reduction results of the last reduction kernel
    int iter;         // iterations completed
    int maxit;
    int done;         // 1: converged / stopped; every iteration kernel then returns at once
    int status;       // pps_status of the stop
    int rho0_from_r;  // 1: rho0 = <r0,r0> at start (inner solves); 0: rho0 = normb^2
    int tol_relative; // 1: refinement inner solve: stop at tol_abs, else reduce by max(tol_rel, 0.3*tol_abs/err0)
    double tol_rel;
    int hist_cap;
    int pad_;
};

enum FinKind : int {
    FIN_NONE = 0,
    FIN_NORMB = 1,      // normb = sqrt(sum0)
    FIN_RES0 = 2,       // initial residual: err0, hist[0], rho0, early stop
    FIN_ALPHA = 3,      // BiCGSTAB alpha = rho0 / sum0
    FIN_OMEGA = 4,      // BiCGSTAB omega = sum0 / sum1
    FIN_CONV = 5,       // BiCGSTAB err, beta, rho0 update, iteration count, stop test
    FIN_CG_ALPHA = 6,   // CG alpha = rz / pAp
    FIN_CG_CONV = 7,    // CG beta = rz_new / rz, err, stop test
    FIN_STORE = 8,      // only store sums[] (used by tests and true residuals)
    FIN_FCG_CONV = 9,   // flexible CG: Polak-Ribiere beta = -alpha z.Ap / rho0, rho0 = z.r
    FIN_FCG_ALPHA = 10, // flexible CG: alpha = rho0 / pAp
    FIN_FCG_SETUP = 11, // flexible CG (re)start: rho0 = z.r, beta = 0 (the next p is z)
    FIN_FCG_RES = 12    // flexible CG: err = ||r|| after the x, r update, iteration count, stop test
};

struct RedCtx {
    double* partials;   // nblocks * 4 doubles
    unsigned* counter;  // zero between launches; the last block resets it
    DevState* st;
    double* hist;
    int kind;
    // Canonical sums (FP64 form): when cells is set, a kernel launched on the
    // canonical shape (canon_shape) stores one partial per cell -- 32 consecutive
    // columns of one row over one canonical z chunk, summed by the thread along z in
    // plane order and over the warp's lanes by a fixed shuffle tree -- at
    // cells[q * cell_n + cell], cell = (chunk * cell_ny + row) * cell_ntx + tile;
    // k_canon_finalize then sums the cells in a fixed tree.  The result depends on
    // the grid alone, not on the tile shape the autotuner picked or the SM count.
    double* cells = nullptr;
    int cell_ntx = 0, cell_ny = 0;
    long long cell_n = 0;
};

// Chebyshev coefficients of one sweep in pre-folded form (the alpaka kernels fold
// the same way, kernelsAlpakaChebyshev.hpp:147-152,234-241):
//   out = cc*u + cx*(u[i-1]+u[i+1]) + cy*(...) + cz*(...) + cb*B + cw*Z
struct Coef {
    double cc, cx, cy, cz, cb, cw, scale;
};

// Neumann face data on the device: values of du/d(dir) per face (NULL if none).
struct Faces {
    const double* g[6];
};

// ---- batches of independent grids (pps_batch_kernels.cuh, pps_batch.cu) ----

// One problem of a batch: its geometry, the offset of its field in every pooled
// array, its tile shape and its range of launch blocks.
struct BProb {
    Geo g;
    long long off;
    unsigned first_block, nblocks;
    int ntx, nty, nchunks, kchunk, cx;
};

struct BatchDev {
    const BProb* prob;
    const unsigned* blk2prob;   // launch block -> problem
    int nprob;
    unsigned total_blocks;
};

// Per-problem state: the inner Krylov scalars plus the refinement bookkeeping.
struct BState {
    DevState s;
    double tol_rel_outer;   // tolerance on ||r||/||b_adj||
    double tol_outer;       // tol_rel_outer * ||b_adj||
    double err_outer;       // last FP64 true residual norm
    int finished;           // 1: converged (or failed); every kernel skips the problem
    int refinements;
    int total_iters;
    int outer_status;
};

void b_refine_init(const BatchDev& B, BState* bst, int inner_maxit, double inner_tol, cudaStream_t s);
void b_refine_end(const BatchDev& B, BState* bst, cudaStream_t s);
void b_norm_badj(const BatchDev& B, const double* b, const double* x, double* part, unsigned* cnt, BState* bst,
                 cudaStream_t s);
void b_residual(const BatchDev& B, const double* x, const double* b, float* r, float* r0, float* p, double* part,
                unsigned* cnt, BState* bst, cudaStream_t s);
void b_zero(const BatchDev& B, float* e, const BState* bst, cudaStream_t s);
void b_add_correction(const BatchDev& B, double* x, const float* e, const BState* bst, cudaStream_t s);
void b_cheb_s01(const BatchDev& B, const float* Bf, float* Y, const void* coef, int cstride, int ci,
                const BState* bst, cudaStream_t s);
void b_cheb_sweep(const BatchDev& B, const float* Y, const float* Bf, const float* Z, float* W, const void* coef,
                  int cstride, int ci, const BState* bst, cudaStream_t s);
void b_stencil_dot(const BatchDev& B, const float* u, const float* w, float* Au, int nsums, double* part,
                   unsigned* cnt, BState* bst, cudaStream_t s);
void b_axpy_alpha(const BatchDev& B, float* r, const float* v, const BState* bst, cudaStream_t s);
void b_update_xr(const BatchDev& B, float* x, const float* Mp, const float* z, float* r, const float* Az,
                 const float* r0, double* part, unsigned* cnt, BState* bst, cudaStream_t s);
void b_update_p(const BatchDev& B, float* p, const float* r, const float* AMp, const BState* bst, cudaStream_t s);
// Casts n pre-folded coefficient sets to the device layout of the float kernels.
void b_cast_coef(const struct Coef* in, void* out, size_t n);
size_t b_coef_size();

// ---- launch wrappers (pps_kernels.cu) ----
Shape make_shape(const Geo& g, int ty, int target_blocks, int cx = 1);
// Streaming multiprocessors of the current device (cudaDevAttrMultiProcessorCount,
// cached per device): launch grids are sized in waves of it.
int sm_count();
// Canonical shape of canonical sums (RedCtx::cells) and the number of cells per sum.
Shape canon_shape(const Geo& g, int ty);
long long canon_cells(const Geo& g);

// Parity (bit-exact FP64) kernels.
void par_stencil(const Geo& g, const double* u, double* out, cudaStream_t s);
void par_residual(const Geo& g, const double* x, const double* b, double* r, cudaStream_t s);
void par_adjust_b(const Geo& g, const double* b, const double* x, Faces f, double* bt, cudaStream_t s);
// The same at every data node the reference's face loops reach (boundary nodes too).
void par_adjust_b_data(const Geo& g, const double* b, const double* x, Faces f, double* bt, cudaStream_t s);
void par_cheb_s01(const Geo& g, const double* B, double* Y, double* Z, double theta, double t2rd, cudaStream_t s);
void par_cheb_sweep(const Geo& g, const double* Y, const double* B, const double* Z, double* W, double rc,
                    double two_sigma, double two_over_delta, double ro, cudaStream_t s);
void par_neg(const Geo& g, const double* W, double* X, cudaStream_t s);
void par_axpy(const Geo& g, double* r, const double* v, double a, cudaStream_t s);
void par_update_x_all(const Geo& g, double* x, const double* Mp, const double* z, double a, double w, cudaStream_t s);
void par_update_x(const Geo& g, double* x, const double* p, double a, cudaStream_t s);
void par_update_p(const Geo& g, double* p, const double* r, const double* AMp, double beta, double omega, cudaStream_t s);
void par_update_p_cg(const Geo& g, double* p, const double* z, double beta, cudaStream_t s);
void par_scale_all(const Geo& g, double* x, double* b, double v, int divide, cudaStream_t s);
void seq_dot2(const Geo& g, const double* a1, const double* b1, const double* a2, const double* b2, double* out,
              cudaStream_t s);

// Neumann ghost fill (iterativeSolverBase.hpp:62-169): field_mode adds the flux term.
template <typename T>
void neumann_fill(const Geo& g, T* field, Faces f, int field_mode, double normb, cudaStream_t s);

// Fast kernels, T = float or double storage.
// Y = s1 (pre-folded coefficients; scale -1 gives X = -s1 directly).
template <typename T>
void fast_cheb_s01(const Geo& g, const Shape& sh, const T* B, T* Y, const Coef& cy, const int* done, cudaStream_t s);
// One sweep; Z == nullptr for the first sweep (s0 folded into the B coefficient).
// s1..s_nsteps of the Chebyshev recurrence in one pass (nsteps 2 or 3): c[0] makes
// s1 from B, c[t-1] step t (the last one's scale is the output's -1); X = the last
// step.  Bit-identical to fast_cheb_s01 + fast_cheb_sweep launches.  Dirichlet only.
template <typename T>
void fast_cheb_fused(const Geo& g, int nsteps, const T* B, T* X, const Coef* c, const int* done, cudaStream_t s);
template <typename T>
void fast_cheb_sweep(const Geo& g, const Shape& sh, const T* Y, const T* B, const T* Z, T* W, const Coef& c,
                     const int* done, cudaStream_t s);
template <typename T>
void fast_scale_copy(const Geo& g, const Shape& sh, const T* B, T* X, double a, const int* done, cudaStream_t s);
template <typename T>
void fast_stencil_dot(const Geo& g, const Shape& sh, const T* u, const T* r0, T* Au, const Coef& a,
                      RedCtx rc, cudaStream_t s);
template <typename T>
void fast_stencil_dot2(const Geo& g, const Shape& sh, const T* u, const T* r, T* Au, const Coef& a,
                       RedCtx rc, cudaStream_t s);
template <typename T>
void fast_axpy_alpha(const Geo& g, const Shape& sh, T* r, const T* v, const DevState* st, cudaStream_t s);
template <typename T>
void fast_update_xr(const Geo& g, const Shape& sh, T* x, const T* Mp, const T* z, T* r, const T* Az,
                    const T* r0, RedCtx rc, cudaStream_t s);
template <typename T>
void fast_update_p(const Geo& g, const Shape& sh, T* p, const T* r, const T* AMp, const DevState* st,
                   cudaStream_t s);
// CG pieces (baseCG.hpp:115-228).
template <typename T>
void fast_cg_stencil_dot(const Geo& g, const Shape& sh, const T* p, const T* r, const T* z, T* Ap,
                         const Coef& a, RedCtx rc, cudaStream_t s);
template <typename T>
void fast_cg_update_xr(const Geo& g, const Shape& sh, T* x, const T* p, T* r, const T* Ap, const DevState* st,
                       cudaStream_t s);
template <typename T>
void fast_cg_dot_rz(const Geo& g, const Shape& sh, const T* r, const T* z, RedCtx rc, cudaStream_t s);
template <typename T>
void fast_cg_update_p(const Geo& g, const Shape& sh, T* p, const T* z, const DevState* st, cudaStream_t s);
// Flexible CG (no reference counterpart; BaseCG's loop with a Polak-Ribiere beta).
template <typename T>
void fast_fcg_update_xr(const Geo& g, const Shape& sh, T* x, const T* p, T* r, const T* Ap, RedCtx rc,
                        cudaStream_t s);
template <typename T>
void fast_fcg_dot(const Geo& g, const Shape& sh, const T* r, const T* z, const T* Ap, RedCtx rc, cudaStream_t s);
template <typename T>
void fast_fcg_p_stencil(const Geo& g, const Shape& sh, const T* z, const T* pin, T* pout, T* Ap, const Coef& a,
                        RedCtx rc, cudaStream_t s, bool staged);
// The same updates and sums over the whole padded array in 16-byte vectors (fields
// zero on the guard cells, 16-byte aligned).
template <typename T>
void fast_fcg_update_xr_flat(const Geo& g, const Shape& sh, T* x, const T* p, T* r, const T* Ap, RedCtx rc,
                             cudaStream_t s);
template <typename T>
void fast_fcg_dot_flat(const Geo& g, const Shape& sh, const T* r, const T* z, const T* Ap, RedCtx rc, cudaStream_t s);

// FP64 true residual r = b - A x written as TR (also into r0 and p when given),
// with sum r^2 in FP64.
template <typename TR>
void fast_residual(const Geo& g, const Shape& sh, const double* x, const double* b, TR* r, TR* r0, TR* p,
                   const Coef& a, RedCtx rc, cudaStream_t s, bool x_zero = false);
// Number of entries of a whole FP64 field that are not +-0 (into sums[0]).
void fast_count_nonzero(const Geo& g, const Shape& sh, const double* x, RedCtx rc, cudaStream_t s);
// *flag = 1 when an entry of the n doubles at x (16-byte aligned) is not +-0
void flag_nonzero(long long n, const double* x, int* flag, cudaStream_t s);
// *h_mapped = *d, h_mapped a page-locked host DevState whose device address equals its
// host address, stored by a kernel (no copy engine)
void state_out(const DevState* d, DevState* h_mapped, cudaStream_t s);
// ||b_adj||^2 over the unknowns, b_adj formed on the fly (FP64).
void fast_norm_badj(const Geo& g, const Shape& sh, const double* b, const double* x, Faces f, RedCtx rc,
                    cudaStream_t s, bool x_zero = false);
// x += e at the unknowns (FP64 += FP32).  e_zero_off: e is +-0 off the unknowns,
// which lets Dirichlet grids run the flat vector form.
void fast_add_correction(const Geo& g, const Shape& sh, double* x, const float* e, const DevState* st,
                         cudaStream_t s, bool e_zero_off = false);
// Start of an inner BiCGSTAB solve from X = 0: r = r0 = p = B at the unknowns, sum B^2.
template <typename T>
void fast_bicg_start(const Geo& g, const Shape& sh, const T* B, T* r, T* r0, T* p, RedCtx rc, cudaStream_t s);
// out = (float)in over a whole field.
void cast_field_f32(const double* in, float* out, long long n, cudaStream_t s);
template <typename T>
void fill_field(T* p, long long n, T v, cudaStream_t s);
// Zero the boundary nodes and guard layers of a padded field.
template <typename T>
void zero_off_unknowns(const Geo& g, T* p, cudaStream_t s);
// Scalar state helpers.
void state_init(DevState* st, double* hist, int maxit, double tol_abs, double tol_rel, int tol_relative,
                int rho0_from_r, double hist_scale, int hist_cap, cudaStream_t s);

int launches_counter_reset();
int launches_counter();
void launches_counter_add(int d);

// Batched solves in one persistent launch (flexible CG + multigrid V-cycle per problem,
// FP64 refinement; csrc/pps_bvcycle.cu).  The pools are the batch's level-0 fields
// (guard-padded, per-problem offsets); the plan owns its coarse levels.
struct BvcPlan;
struct BvcPools {
    double* x;
    const double* b;
    float *r, *z, *pa, *pb, *ap, *e, *y1, *y2, *t0;
};
bool bvc_create(BvcPlan** out, int nprob, const Geo* geo, const long long* off, const BvcPools& pools, double tol,
                double inner_tol, int inner_maxit, int max_refinements, cudaStream_t s, std::string& err);
void bvc_destroy(BvcPlan* plan);
void bvc_set_wait_limit(BvcPlan* plan, double seconds);
pps_status bvc_solve(BvcPlan* plan, cudaStream_t s, cudaEvent_t ev0, cudaEvent_t ev1, pps_batch_stats* stats,
                     std::string& err);
void bvc_result(const BvcPlan* plan, int q, pps_stats* st);

}  // namespace pps
