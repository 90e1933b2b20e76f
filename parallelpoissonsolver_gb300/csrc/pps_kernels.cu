// CUDA kernels of libpps for sm_103a (GB300).
//
// Two families:
//   * par_*  : the reference's FP64 arithmetic in its exact operand order, every
//              operation an explicitly rounded intrinsic (no FMA contraction), so
//              results are bit-identical to the reference CPU solver.  Reductions
//              are serial sums in the reference's k,j,i loop order (seq_dot2).
//   * fast_* : z-marching stencil kernels with pre-folded coefficients and FMA,
//              templated on the storage type (double, or float for the mixed form),
//              fused with their dot products.  Reductions are deterministic: a fixed
//              shuffle tree per block, block partials in global memory, and the last
//              block to finish sums the partials in block order and advances the
//              Krylov scalars on the device (no host round trip).
#include "pps_internal.h"
#include "pps_reduce.cuh"

#include <algorithm>
#include <initializer_list>
#include <type_traits>

#include <cuda.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>

namespace pps {

// launches issued by this thread (each solve runs on its calling thread)
static thread_local int g_launches = 0;
int launches_counter_reset() { int v = g_launches; g_launches = 0; return v; }
int launches_counter() { return g_launches; }
void launches_counter_add(int d) { g_launches += d; }
static thread_local unsigned long long g_launch_failures = 0;
unsigned long long launch_failures() { return g_launch_failures; }
void note_launch_failure(cudaError_t e)
{
    ++g_launch_failures;
    const char* what = cudaGetErrorString(e);
    char msg[160];
    snprintf(msg, sizeof(msg), "kernel launch failed: %s", what ? what : "unknown error");
    pps_internal_set_error(msg);
}
#define PPS_COUNT_LAUNCH() (++g_launches)

// ---------------------------------------------------------------------------
// Parity kernels (FP64, exact reference expression order)
// ---------------------------------------------------------------------------

struct Lin {
    int ux, uy, uz;
    long long n;
};

__host__ __device__ inline Lin unknown_box(const Geo& g)
{
    Lin L;
    L.ux = g.hi[0] - g.lo[0];
    L.uy = g.hi[1] - g.lo[1];
    L.uz = g.hi[2] - g.lo[2];
    L.n = (long long)L.ux * L.uy * L.uz;
    return L;
}

__device__ __forceinline__ long long lin_to_index(const Geo& g, const Lin& L, long long t)
{
    const int i = g.lo[0] + (int)(t % L.ux);
    const long long q = t / L.ux;
    const int j = g.lo[1] + (int)(q % L.uy);
    const int k = g.lo[2] + (int)(q / L.uy);
    return i + g.sj * j + g.sk * k;
}

// (d[c-1] - 2*d[c] + d[c+1])/(h0*h0) + ... (matrixFreeOperatorA.hpp:34-38)
__device__ __forceinline__ double opA_exact(const double* __restrict__ d, long long c, long long sj, long long sk,
                                            double h2x, double h2y, double h2z)
{
    const double two_c = __dmul_rn(2.0, d[c]);
    const double tx = __ddiv_rn(__dadd_rn(__dsub_rn(d[c - 1], two_c), d[c + 1]), h2x);
    const double ty = __ddiv_rn(__dadd_rn(__dsub_rn(d[c - sj], two_c), d[c + sj]), h2y);
    const double tz = __ddiv_rn(__dadd_rn(__dsub_rn(d[c - sk], two_c), d[c + sk]), h2z);
    return __dadd_rn(__dadd_rn(tx, ty), tz);
}

#define PAR_LOOP(g, L)                                                                          \
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < L.n;             \
         t += (long long)gridDim.x * blockDim.x)

static inline unsigned par_blocks(long long n)
{
    long long b = (n + 255) / 256;
    if (b > sm_count() * 64LL) b = sm_count() * 64LL;
    if (b < 1) b = 1;
    return (unsigned)b;
}

__global__ void k_par_stencil(Geo g, const double* __restrict__ u, double* __restrict__ out, double h2x,
                              double h2y, double h2z)
{
    pdl_enter();
    const Lin L = unknown_box(g);
    PAR_LOOP(g, L)
    {
        const long long c = lin_to_index(g, L, t);
        out[c] = opA_exact(u, c, g.sj, g.sk, h2x, h2y, h2z);
    }
}

__global__ void k_par_residual(Geo g, const double* __restrict__ x, const double* __restrict__ b,
                               double* __restrict__ r, double h2x, double h2y, double h2z)
{
    pdl_enter();
    const Lin L = unknown_box(g);
    PAR_LOOP(g, L)
    {
        const long long c = lin_to_index(g, L, t);
        r[c] = __dsub_rn(b[c], opA_exact(x, c, g.sj, g.sk, h2x, h2y, h2z));
    }
}

// b_adj at the unknowns (adjustFieldBForDirichletNeumanBCs, iterativeSolverBase.hpp:429-534):
// the same subtractions/additions applied to one point in the reference's face order.
__device__ __forceinline__ double badj_exact(const Geo& g, const double* __restrict__ b,
                                             const double* __restrict__ x, const Faces& f, long long c, int i,
                                             int j, int k)
{
    double v = b[c];
    const int idx[3] = {i, j, k};
    const long long step[3] = {1, g.sj, g.sk};
    for (int d = 0; d < 3; d++) {
        const double h2 = __dmul_rn(g.ds[d], g.ds[d]);
        // low face
        if (g.bcs[2 * d] == 0) {
            if (idx[d] == 2) v = __dsub_rn(v, __ddiv_rn(x[c - step[d]], h2));
        } else if (idx[d] == 1 && f.g[2 * d]) {
            long long fi;
            if (d == 0) fi = (long long)(j - 1) + (long long)g.n[1] * (k - 1);
            else if (d == 1) fi = (long long)(i - 1) + (long long)g.n[0] * (k - 1);
            else fi = (long long)(i - 1) + (long long)g.n[0] * (j - 1);
            v = __dadd_rn(v, __ddiv_rn(__dmul_rn(2.0, f.g[2 * d][fi]), g.ds[d]));
        }
        // high face
        if (g.bcs[2 * d + 1] == 0) {
            if (idx[d] == g.n[d] - 1) v = __dsub_rn(v, __ddiv_rn(x[c + step[d]], h2));
        } else if (idx[d] == g.n[d] && f.g[2 * d + 1]) {
            long long fi;
            if (d == 0) fi = (long long)(j - 1) + (long long)g.n[1] * (k - 1);
            else if (d == 1) fi = (long long)(i - 1) + (long long)g.n[0] * (k - 1);
            else fi = (long long)(i - 1) + (long long)g.n[0] * (j - 1);
            v = __dsub_rn(v, __ddiv_rn(__dmul_rn(2.0, f.g[2 * d + 1][fi]), g.ds[d]));
        }
    }
    return v;
}

__global__ void k_par_adjust_b(Geo g, const double* __restrict__ b, const double* __restrict__ x, Faces f,
                               double* __restrict__ bt)
{
    pdl_enter();
    const Lin L = unknown_box(g);
    PAR_LOOP(g, L)
    {
        const int i = g.lo[0] + (int)(t % L.ux);
        const long long q = t / L.ux;
        const int j = g.lo[1] + (int)(q % L.uy);
        const int k = g.lo[2] + (int)(q / L.uy);
        const long long c = i + g.sj * j + g.sk * k;
        bt[c] = badj_exact(g, b, x, f, c, i, j, k);
    }
}

// The same adjustment at every data node it reaches, boundary nodes included: the
// reference adjusts a full copy of b face by face, and the plane next to one face
// holds boundary nodes of the others (iterativeSolverBase.hpp:429-534).  The
// Chebyshev main solver reads them through the stencil of its first step.
__global__ void k_par_adjust_b_data(Geo g, const double* __restrict__ b, const double* __restrict__ x, Faces f,
                                    double* __restrict__ bt)
{
    pdl_enter();
    const long long nx = g.n[0], ny = g.n[1], n = nx * ny * (long long)g.n[2];
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x) {
        const int i = 1 + (int)(t % nx);
        const long long q = t / nx;
        const int j = 1 + (int)(q % ny);
        const int k = 1 + (int)(q / ny);
        const long long c = i + g.sj * j + g.sk * k;
        bt[c] = badj_exact(g, b, x, f, c, i, j, k);
    }
}

// Z = B/theta; Y = 2*rho/delta * (2*B + A(B)/theta)   (chebyshevIteration.hpp:79-90)
__global__ void k_par_cheb_s01(Geo g, const double* __restrict__ B, double* __restrict__ Y, double* __restrict__ Z,
                               double theta, double t2rd, double h2x, double h2y, double h2z)
{
    pdl_enter();
    const Lin L = unknown_box(g);
    PAR_LOOP(g, L)
    {
        const long long c = lin_to_index(g, L, t);
        Z[c] = __ddiv_rn(B[c], theta);
        const double ab = opA_exact(B, c, g.sj, g.sk, h2x, h2y, h2z);
        Y[c] = __dmul_rn(t2rd, __dadd_rn(__dmul_rn(2.0, B[c]), __ddiv_rn(ab, theta)));
    }
}

// W = rho*(2*sigma*Y + 2/delta*(B + A(Y)) - rhoOld*Z)   (chebyshevIteration.hpp:110)
__global__ void k_par_cheb_sweep(Geo g, const double* __restrict__ Y, const double* __restrict__ B,
                                 const double* __restrict__ Z, double* __restrict__ W, double rc, double two_sigma,
                                 double two_over_delta, double ro, double h2x, double h2y, double h2z)
{
    pdl_enter();
    const Lin L = unknown_box(g);
    PAR_LOOP(g, L)
    {
        const long long c = lin_to_index(g, L, t);
        const double ay = opA_exact(Y, c, g.sj, g.sk, h2x, h2y, h2z);
        const double t1 = __dmul_rn(two_sigma, Y[c]);
        const double t2 = __dmul_rn(two_over_delta, __dadd_rn(B[c], ay));
        W[c] = __dmul_rn(rc, __dsub_rn(__dadd_rn(t1, t2), __dmul_rn(ro, Z[c])));
    }
}

__global__ void k_par_neg(Geo g, const double* __restrict__ W, double* __restrict__ X)
{
    pdl_enter();
    const Lin L = unknown_box(g);
    PAR_LOOP(g, L)
    {
        const long long c = lin_to_index(g, L, t);
        X[c] = __dmul_rn(-1.0, W[c]);
    }
}

__global__ void k_par_axpy(Geo g, double* __restrict__ r, const double* __restrict__ v, double a)
{
    pdl_enter();
    const Lin L = unknown_box(g);
    PAR_LOOP(g, L)
    {
        const long long c = lin_to_index(g, L, t);
        r[c] = __dsub_rn(r[c], __dmul_rn(a, v[c]));
    }
}

// x = x + a*Mp + w*z over every point of the field (BiCGSTAB.hpp:227-230)
__global__ void k_par_update_x_all(long long n, double* __restrict__ x, const double* __restrict__ Mp,
                                   const double* __restrict__ z, double a, double w)
{
    pdl_enter();
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x)
        x[c] = __dadd_rn(__dadd_rn(x[c], __dmul_rn(a, Mp[c])), __dmul_rn(w, z[c]));
}

__global__ void k_par_update_x(Geo g, double* __restrict__ x, const double* __restrict__ p, double a)
{
    pdl_enter();
    const Lin L = unknown_box(g);
    PAR_LOOP(g, L)
    {
        const long long c = lin_to_index(g, L, t);
        x[c] = __dadd_rn(x[c], __dmul_rn(a, p[c]));
    }
}

// p = r + beta*(p - omega*AMp)   (BiCGSTAB.hpp:269)
__global__ void k_par_update_p(Geo g, double* __restrict__ p, const double* __restrict__ r,
                               const double* __restrict__ AMp, double beta, double omega)
{
    pdl_enter();
    const Lin L = unknown_box(g);
    PAR_LOOP(g, L)
    {
        const long long c = lin_to_index(g, L, t);
        p[c] = __dadd_rn(r[c], __dmul_rn(beta, __dsub_rn(p[c], __dmul_rn(omega, AMp[c]))));
    }
}

// p = z + beta*p   (baseCG.hpp:204)
__global__ void k_par_update_p_cg(Geo g, double* __restrict__ p, const double* __restrict__ z, double beta)
{
    pdl_enter();
    const Lin L = unknown_box(g);
    PAR_LOOP(g, L)
    {
        const long long c = lin_to_index(g, L, t);
        p[c] = __dadd_rn(z[c], __dmul_rn(beta, p[c]));
    }
}

__global__ void k_par_scale_all(long long n, double* __restrict__ x, double* __restrict__ b, double v, int divide)
{
    pdl_enter();
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
        if (divide) {
            x[c] = __ddiv_rn(x[c], v);
            b[c] = __ddiv_rn(b[c], v);
        } else {
            x[c] = __dmul_rn(x[c], v);
            b[c] = __dmul_rn(b[c], v);
        }
    }
}

// Serial sums s1 = sum a1*b1, s2 = sum a2*b2 over the unknowns in k,j,i order.
// One block: all threads form products of a chunk into shared memory, then one
// thread adds them in order, exactly as the reference's loop does.
constexpr int SEQ_THREADS = 512;
constexpr int SEQ_CHUNK = 2048;

__global__ void __launch_bounds__(SEQ_THREADS) k_seq_dot2(Geo g, const double* __restrict__ a1,
                                                          const double* __restrict__ b1, const double* __restrict__ a2,
                                                          const double* __restrict__ b2, double* __restrict__ out)
{
    pdl_enter();
    __shared__ double p1[SEQ_CHUNK];
    __shared__ double p2[SEQ_CHUNK];
    const Lin L = unknown_box(g);
    double s1 = 0.0, s2 = 0.0;
    const bool two = (a2 != nullptr);
    for (long long base = 0; base < L.n; base += SEQ_CHUNK) {
        const int m = (int)((L.n - base) < SEQ_CHUNK ? (L.n - base) : SEQ_CHUNK);
        for (int q = threadIdx.x; q < m; q += blockDim.x) {
            const long long c = lin_to_index(g, L, base + q);
            p1[q] = __dmul_rn(a1[c], b1[c]);
            if (two) p2[q] = __dmul_rn(a2[c], b2[c]);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            if (two) {
                for (int q = 0; q < m; q++) {
                    s1 = __dadd_rn(s1, p1[q]);
                    s2 = __dadd_rn(s2, p2[q]);
                }
            } else {
                for (int q = 0; q < m; q++) s1 = __dadd_rn(s1, p1[q]);
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = s1;
        out[1] = s2;
    }
}

void par_stencil(const Geo& g, const double* u, double* out, cudaStream_t s)
{
    launch_pdl(k_par_stencil, par_blocks(unknown_box(g).n), 256, 0, s, g, u, out, g.ds[0] * g.ds[0], g.ds[1] * g.ds[1],
                                                                 g.ds[2] * g.ds[2]);
    PPS_COUNT_LAUNCH();
}
void par_residual(const Geo& g, const double* x, const double* b, double* r, cudaStream_t s)
{
    launch_pdl(k_par_residual, par_blocks(unknown_box(g).n), 256, 0, s, g, x, b, r, g.ds[0] * g.ds[0], g.ds[1] * g.ds[1],
                                                                  g.ds[2] * g.ds[2]);
    PPS_COUNT_LAUNCH();
}
void par_adjust_b(const Geo& g, const double* b, const double* x, Faces f, double* bt, cudaStream_t s)
{
    launch_pdl(k_par_adjust_b, par_blocks(unknown_box(g).n), 256, 0, s, g, b, x, f, bt);
    PPS_COUNT_LAUNCH();
}
void par_adjust_b_data(const Geo& g, const double* b, const double* x, Faces f, double* bt, cudaStream_t s)
{
    launch_pdl(k_par_adjust_b_data, par_blocks((long long)g.n[0] * g.n[1] * g.n[2]), 256, 0, s, g, b, x, f, bt);
    PPS_COUNT_LAUNCH();
}
void par_cheb_s01(const Geo& g, const double* B, double* Y, double* Z, double theta, double t2rd, cudaStream_t s)
{
    launch_pdl(k_par_cheb_s01, par_blocks(unknown_box(g).n), 256, 0, s, g, B, Y, Z, theta, t2rd, g.ds[0] * g.ds[0],
                                                                  g.ds[1] * g.ds[1], g.ds[2] * g.ds[2]);
    PPS_COUNT_LAUNCH();
}
void par_cheb_sweep(const Geo& g, const double* Y, const double* B, const double* Z, double* W, double rc,
                    double two_sigma, double two_over_delta, double ro, cudaStream_t s)
{
    launch_pdl(k_par_cheb_sweep, par_blocks(unknown_box(g).n), 256, 0, s, g, Y, B, Z, W, rc, two_sigma, two_over_delta, ro,
                                                                    g.ds[0] * g.ds[0], g.ds[1] * g.ds[1],
                                                                    g.ds[2] * g.ds[2]);
    PPS_COUNT_LAUNCH();
}
void par_neg(const Geo& g, const double* W, double* X, cudaStream_t s)
{
    launch_pdl(k_par_neg, par_blocks(unknown_box(g).n), 256, 0, s, g, W, X);
    PPS_COUNT_LAUNCH();
}
void par_axpy(const Geo& g, double* r, const double* v, double a, cudaStream_t s)
{
    launch_pdl(k_par_axpy, par_blocks(unknown_box(g).n), 256, 0, s, g, r, v, a);
    PPS_COUNT_LAUNCH();
}
void par_update_x_all(const Geo& g, double* x, const double* Mp, const double* z, double a, double w, cudaStream_t s)
{
    launch_pdl(k_par_update_x_all, par_blocks(g.ntot), 256, 0, s, g.ntot, x, Mp, z, a, w);
    PPS_COUNT_LAUNCH();
}
void par_update_x(const Geo& g, double* x, const double* p, double a, cudaStream_t s)
{
    launch_pdl(k_par_update_x, par_blocks(unknown_box(g).n), 256, 0, s, g, x, p, a);
    PPS_COUNT_LAUNCH();
}
void par_update_p(const Geo& g, double* p, const double* r, const double* AMp, double beta, double omega, cudaStream_t s)
{
    launch_pdl(k_par_update_p, par_blocks(unknown_box(g).n), 256, 0, s, g, p, r, AMp, beta, omega);
    PPS_COUNT_LAUNCH();
}
void par_update_p_cg(const Geo& g, double* p, const double* z, double beta, cudaStream_t s)
{
    launch_pdl(k_par_update_p_cg, par_blocks(unknown_box(g).n), 256, 0, s, g, p, z, beta);
    PPS_COUNT_LAUNCH();
}
void par_scale_all(const Geo& g, double* x, double* b, double v, int divide, cudaStream_t s)
{
    launch_pdl(k_par_scale_all, par_blocks(g.ntot), 256, 0, s, g.ntot, x, b, v, divide);
    PPS_COUNT_LAUNCH();
}
void seq_dot2(const Geo& g, const double* a1, const double* b1, const double* a2, const double* b2, double* out,
              cudaStream_t s)
{
    launch_pdl(k_seq_dot2, 1, SEQ_THREADS, 0, s, g, a1, b1, a2, b2, out);
    PPS_COUNT_LAUNCH();
}

// ---------------------------------------------------------------------------
// Neumann ghost fill (both families; the arithmetic matches the reference order)
// ---------------------------------------------------------------------------

template <typename T>
__global__ void k_neumann_fill(Geo g, T* __restrict__ field, Faces f, int face, int field_mode, double normb)
{
    pdl_enter();
    const int dir = face / 2, side = face % 2;
    const int a0 = dir == 0 ? 1 : 0;          // first remaining axis
    const int a1 = dir == 2 ? 1 : 2;          // second remaining axis
    const int na = g.n[a0], nb = g.n[a1];
    const long long step = dir == 0 ? 1 : (dir == 1 ? g.sj : g.sk);
    const long long stride[3] = {1, g.sj, g.sk};
    const long long total = (long long)na * nb;
    const double* gf = f.g[face];
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
        const int ia = 1 + (int)(t % na);
        const int ib = 1 + (int)(t / na);
        const int inode = side == 0 ? 1 : g.n[dir];
        const long long c = inode * stride[dir] + ia * stride[a0] + ib * stride[a1];
        const long long ghost = side == 0 ? c - step : c + step;
        const long long mirror = side == 0 ? c + step : c - step;
        if (field_mode) {
            const double gv = gf ? gf[t] : 0.0;
            const double term = __ddiv_rn(__dmul_rn(__dmul_rn(2.0, g.ds[dir]), gv), normb);
            const double m = (double)field[mirror];
            field[ghost] = (T)(side == 0 ? __dsub_rn(m, term) : __dadd_rn(m, term));
        } else {
            field[ghost] = field[mirror];
        }
    }
}

template <typename T>
void neumann_fill(const Geo& g, T* field, Faces f, int field_mode, double normb, cudaStream_t s)
{
    for (int face = 0; face < 6; face++) {
        if (g.bcs[face] != 1) continue;
        const int dir = face / 2;
        const long long total = (long long)g.n[dir == 0 ? 1 : 0] * g.n[dir == 2 ? 1 : 2];
        unsigned blocks = (unsigned)((total + 255) / 256);
        if (blocks > 1024) blocks = 1024;
        launch_pdl(k_neumann_fill<T>, blocks, 256, 0, s, g, field, f, face, field_mode, normb);
        PPS_COUNT_LAUNCH();
    }
}
template void neumann_fill<double>(const Geo&, double*, Faces, int, double, cudaStream_t);
template void neumann_fill<float>(const Geo&, float*, Faces, int, double, cudaStream_t);

// ---------------------------------------------------------------------------
// Fast kernels
// ---------------------------------------------------------------------------

int sm_count()
{
    static int cached[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) dev = 0;
    int n = __atomic_load_n(&cached[dev], __ATOMIC_RELAXED);
    if (n <= 0) {
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 148;
        __atomic_store_n(&cached[dev], n, __ATOMIC_RELAXED);
    }
    return n;
}

Shape make_shape(const Geo& g, int ty, int target_blocks, int cx)
{
    Shape sh;
    sh.ty = ty;
    sh.cx = cx;
    const int ux = g.hi[0] - g.lo[0], uy = g.hi[1] - g.lo[1], uz = g.hi[2] - g.lo[2];
    // cx = 4: the x-vectorised tiles start at x = 0 (16-byte aligned float4), so they
    // must reach hi[0] from there
    sh.ntx = cx == 4 ? (g.hi[0] + 127) / 128 : (ux + 32 * cx - 1) / (32 * cx);
    sh.nty = (uy + ty - 1) / ty;
    const long long tiles = (long long)sh.ntx * sh.nty;
    long long chunks = (target_blocks + tiles - 1) / tiles;
    if (chunks < 1) chunks = 1;
    if (chunks > uz) chunks = uz;
    sh.kchunk = (int)((uz + chunks - 1) / chunks);
    sh.nchunks = (uz + sh.kchunk - 1) / sh.kchunk;
    return sh;
}

// Canonical launch shape of the FP64 form's reduction kernels: one-column tiles of
// 32 x ty and a z chunk fixed by the grid alone, so that the cells of canonical sums
// (RedCtx::cells) are the same whatever ty the autotuner picked.  ty does not enter
// the cells: each warp stores its own.
Shape canon_shape(const Geo& g, int ty)
{
    Shape sh;
    sh.ty = ty;
    sh.cx = 1;
    const int ux = g.hi[0] - g.lo[0], uy = g.hi[1] - g.lo[1], uz = g.hi[2] - g.lo[2];
    sh.ntx = (ux + 31) / 32;
    sh.nty = (uy + ty - 1) / ty;
    sh.kchunk = std::min(64, std::max(4, (uz + 15) / 16));
    sh.nchunks = (uz + sh.kchunk - 1) / sh.kchunk;
    return sh;
}

long long canon_cells(const Geo& g)
{
    const Shape sh = canon_shape(g, 8);
    return (long long)sh.ntx * (g.hi[1] - g.lo[1]) * sh.nchunks;
}

// The context and shape of one canonical launch.
static void canon_launch(const Geo& g, Shape& sh, RedCtx& rc)
{
    sh = canon_shape(g, sh.ty);
    rc.cell_ntx = sh.ntx;
    rc.cell_ny = g.hi[1] - g.lo[1];
    rc.cell_n = (long long)sh.ntx * rc.cell_ny * sh.nchunks;
}

// Sum of the cells of a canonical launch in a fixed tree, then the finalizer.
// Block b of CANON_BLOCKS sums cells [b*per, (b+1)*per) (thread t the ones at t +
// 256 m, in order; then the warps' shuffle trees and the eight warps in order); the
// last block to finish sums the CANON_BLOCKS partials the same way.  Launched with
// CANON_BLOCKS x 256 threads after the kernel that stored the cells; `done` is that
// kernel's early-exit flag (null if it always runs).
static constexpr int CANON_BLOCKS = 128;
template <int NS>
__global__ void __launch_bounds__(256) k_canon_finalize(RedCtx rc, const int* done)
{
    pdl_enter();
    EARLY_EXIT(done);
    __shared__ double sm[8][NS];
    __shared__ int is_last;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const long long n = rc.cell_n;
    const long long per = (n + CANON_BLOCKS - 1) / CANON_BLOCKS;
    const long long c0 = (long long)blockIdx.x * per, c1 = min(n, c0 + per);
    double acc[NS];
#pragma unroll
    for (int q = 0; q < NS; q++) acc[q] = 0.0;
    for (long long c = c0 + tid; c < c1; c += 256) {
#pragma unroll
        for (int q = 0; q < NS; q++) acc[q] += rc.cells[q * n + c];
    }
#pragma unroll
    for (int q = 0; q < NS; q++) {
        const double w = warp_sum(acc[q]);
        if (lane == 0) sm[warp][q] = w;
    }
    __syncthreads();
    if (tid == 0) {
#pragma unroll
        for (int q = 0; q < NS; q++) {
            double t = 0.0;
            for (int w = 0; w < 8; w++) t += sm[w][q];
            rc.partials[(size_t)blockIdx.x * 4 + q] = t;
        }
        __threadfence();
        is_last = atomicAdd(rc.counter, 1u) == CANON_BLOCKS - 1;
    }
    __syncthreads();
    if (!is_last) return;
    __threadfence();
#pragma unroll
    for (int q = 0; q < NS; q++) acc[q] = tid < CANON_BLOCKS ? __ldcg(&rc.partials[(size_t)tid * 4 + q]) : 0.0;
    __syncthreads();
#pragma unroll
    for (int q = 0; q < NS; q++) {
        const double w = warp_sum(acc[q]);
        if (lane == 0) sm[warp][q] = w;
    }
    __syncthreads();
    if (tid == 0) {
        double tot[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
        for (int q = 0; q < NS; q++) {
            double t = 0.0;
            for (int w = 0; w < 8; w++) t += sm[w][q];
            tot[q] = t;
        }
        finalize(rc, tot);
        __threadfence();
        *rc.counter = 0u;
    }
}

// Equal weights on the three axes (equal spacings): the FP64 kernels then sum the six
// neighbours on the integer pipe.
static inline bool iso_coef(const Coef& c) { return c.cx == c.cy && c.cx == c.cz; }

template <int NS>
static void canon_finalize(const RedCtx& rc, const int* done, cudaStream_t s)
{
    launch_pdl(k_canon_finalize<NS>, CANON_BLOCKS, 256, 0, s, rc, done);
    PPS_COUNT_LAUNCH();
}

struct Col {
    int i, j, k0, k1;
    long long c;
    bool active;
};

__device__ __forceinline__ Col column(const Geo& g, const Shape& sh)
{
    Col q;
    const int bx = blockIdx.x % sh.ntx;
    const int by = blockIdx.x / sh.ntx;
    q.i = g.lo[0] + bx * 32 + threadIdx.x;
    q.j = g.lo[1] + by * sh.ty + threadIdx.y;
    q.k0 = g.lo[2] + blockIdx.y * sh.kchunk;
    q.k1 = min(q.k0 + sh.kchunk, g.hi[2]);
    q.active = q.i < g.hi[0] && q.j < g.hi[1];
    q.c = q.i + g.sj * q.j + g.sk * q.k0;
    return q;
}

static inline dim3 grid_of(const Shape& sh) { return dim3((unsigned)(sh.ntx * sh.nty), (unsigned)sh.nchunks, 1); }
static inline dim3 block_of(const Shape& sh) { return dim3(32, (unsigned)sh.ty, 1); }


// Chebyshev coefficients cast to the storage type on the host (no FP64 work
// in the FP32 kernels; GB300 issues FP64 at 1/64 of the FP32 rate).
template <typename T>
struct CT {
    T cc, cx, cy, cz, cb, cw;
};

template <typename T>
static CT<T> cast_coef(const Coef& c)
{
    CT<T> o;
    o.cc = (T)(c.cc * c.scale);
    o.cx = (T)(c.cx * c.scale);
    o.cy = (T)(c.cy * c.scale);
    o.cz = (T)(c.cz * c.scale);
    o.cb = (T)(c.cb * c.scale);
    o.cw = (T)(c.cw * c.scale);
    return o;
}

// First column of this thread in a tile of (32*CX) x ty columns; the thread's
// other columns sit 32, 64, ... further along x.
__device__ __forceinline__ Col column_cx(const Geo& g, const Shape& sh, int cxw)
{
    Col q;
    const int bx = blockIdx.x % sh.ntx;
    const int by = blockIdx.x / sh.ntx;
    q.i = g.lo[0] + bx * 32 * cxw + threadIdx.x;
    q.j = g.lo[1] + by * sh.ty + threadIdx.y;
    q.k0 = g.lo[2] + blockIdx.y * sh.kchunk;
    q.k1 = min(q.k0 + sh.kchunk, g.hi[2]);
    q.active = q.j < g.hi[1];
    q.c = q.i + g.sj * q.j + g.sk * q.k0;
    return q;
}

// s1 of the preconditioner (chebyshevIteration.hpp:79-90) in pre-folded form:
//   Y = cc*B + cx*(Bx pair) + cy*(By pair) + cz*(Bz pair)
// s0 = B/theta is never stored: the first sweep folds it into its B coefficient.
// With the output scale -1 folded into the coefficients this also writes X = -s1
// directly (degree 3).
template <typename T, int CX>
__global__ void __launch_bounds__(256) k_cheb_s01(Geo g, Shape sh, const T* __restrict__ B, T* __restrict__ Y,
                                                  CT<T> cf, const int* done)
{
    pdl_enter();
    EARLY_EXIT(done);
    const Col q = column_cx(g, sh, CX);
    if (!q.active) return;
    const long long sj = g.sj, sk = g.sk;
    bool on[CX];
    T bm[CX], bc[CX];
#pragma unroll
    for (int u = 0; u < CX; u++) {
        on[u] = q.i + 32 * u < g.hi[0];
        const long long c = q.c + 32 * u;
        bm[u] = on[u] ? B[c - sk] : T(0);
        bc[u] = on[u] ? B[c] : T(0);
    }
    long long c0 = q.c;
#pragma unroll 2
    for (int k = q.k0; k < q.k1; k++) {
#pragma unroll
        for (int u = 0; u < CX; u++) {
            if (!on[u]) continue;
            const long long c = c0 + 32 * u;
            const T bp = B[c + sk];
            const T sx = B[c - 1] + B[c + 1];
            const T sy = B[c - sj] + B[c + sj];
            T y = cf.cc * bc[u];
            y = fmx(cf.cx, sx, y);
            y = fmx(cf.cy, sy, y);
            y = fmx(cf.cz, bm[u] + bp, y);
            Y[c] = y;
            bm[u] = bc[u];
            bc[u] = bp;
        }
        c0 += sk;
    }
}

// One sweep (chebyshevIteration.hpp:110) in pre-folded form:
//   W = cc*Y + cx*(Yx pair) + cy*(Yy pair) + cz*(Yz pair) + cb*B [+ cw*Z]
// HAS_Z = false for the first sweep, whose Z = s0 = B/theta is folded into cb.
template <typename T, int CX, bool HAS_Z>
__global__ void __launch_bounds__(256) k_cheb_sweep(Geo g, Shape sh, const T* __restrict__ Y,
                                                    const T* __restrict__ B, const T* __restrict__ Z,
                                                    T* __restrict__ W, CT<T> cf, const int* done)
{
    pdl_enter();
    EARLY_EXIT(done);
    const Col q = column_cx(g, sh, CX);
    if (!q.active) return;
    const long long sj = g.sj, sk = g.sk;
    bool on[CX];
    T ym[CX], yc[CX];
#pragma unroll
    for (int u = 0; u < CX; u++) {
        on[u] = q.i + 32 * u < g.hi[0];
        const long long c = q.c + 32 * u;
        ym[u] = on[u] ? Y[c - sk] : T(0);
        yc[u] = on[u] ? Y[c] : T(0);
    }
    long long c0 = q.c;
#pragma unroll 2
    for (int k = q.k0; k < q.k1; k++) {
#pragma unroll
        for (int u = 0; u < CX; u++) {
            if (!on[u]) continue;
            const long long c = c0 + 32 * u;
            const T yp = Y[c + sk];
            const T sx = Y[c - 1] + Y[c + 1];
            const T sy = Y[c - sj] + Y[c + sj];
            T w = cf.cc * yc[u];
            w = fmx(cf.cx, sx, w);
            w = fmx(cf.cy, sy, w);
            w = fmx(cf.cz, ym[u] + yp, w);
            w = fmx(cf.cb, B[c], w);
            if (HAS_Z) w = fmx(cf.cw, Z[c], w);
            W[c] = w;
            ym[u] = yc[u];
            yc[u] = yp;
        }
        c0 += sk;
    }
}

// The FP32 Chebyshev kernels vectorised along x: a thread owns four consecutive x
// points (one float4), a warp 128, a block 128 x ty columns, tiles aligned to x = 0
// so that every float4 starts on a 16-byte boundary (the row stride is a multiple
// of 4 floats).  The x neighbours of a float4 come from the neighbouring lanes by
// shuffle (lanes 0 and 31 load the one outside the warp); the y and z neighbours
// are float4 loads, z kept in registers as the thread marches along z.  Points off
// the unknowns are computed on whatever the field holds there and not stored.  The
// arithmetic per point is that of k_cheb_s01 / k_cheb_sweep in the same order, so
// the results are bit-identical; a sweep moves 4x fewer, 4x wider requests.
struct Col4 {
    int i0, j, k0, k1;   // first x of the float4, row, planes [k0, k1)
    long long c;         // field index of (i0, j, k0)
    bool act;            // the float4 holds an unknown
};

__device__ __forceinline__ Col4 column4(const Geo& g, const Shape& sh)
{
    Col4 q;
    const int bx = blockIdx.x % sh.ntx, by = blockIdx.x / sh.ntx;
    q.i0 = bx * 128 + threadIdx.x * 4;
    q.j = g.lo[1] + by * sh.ty + threadIdx.y;
    q.k0 = g.lo[2] + blockIdx.y * sh.kchunk;
    q.k1 = min(q.k0 + sh.kchunk, g.hi[2]);
    q.act = q.i0 < g.hi[0] && q.i0 + 4 > g.lo[0];
    q.c = q.i0 + g.sj * q.j + g.sk * q.k0;
    return q;
}

__device__ __forceinline__ float4 ld4(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ float4 add4(float4 a, float4 b)
{
    return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w);
}

// One thread's march of k_cheb_v4 along z: the float4 at x = i0 (a multiple of 4)
// of the row whose plane-k0 index is c, planes [k0, k1).  MODE 0: W = s1 of U
// (k_cheb_s01); 1: a sweep without Z; 2: a sweep with Z.  Every lane of the warp must
// call it (the x neighbours come by shuffle); lanes whose float4 holds no unknown
// compute on zeros and store nothing.
template <int MODE>
__device__ __forceinline__ void cheb_v4_march(const Geo& g, int i0, int k0, int k1, long long c,
                                              const float* __restrict__ U, const float* __restrict__ B,
                                              const float* __restrict__ Z, float* __restrict__ W, const CT<float>& cf)
{
    const bool act = i0 < g.hi[0] && i0 + 4 > g.lo[0];
    const int lane = threadIdx.x;
    const bool m0 = i0 >= g.lo[0] && i0 < g.hi[0], m1 = i0 + 1 >= g.lo[0] && i0 + 1 < g.hi[0];
    const bool m2 = i0 + 2 >= g.lo[0] && i0 + 2 < g.hi[0], m3 = i0 + 3 >= g.lo[0] && i0 + 3 < g.hi[0];
    const bool all4 = m0 && m1 && m2 && m3;
    const long long sj = g.sj, sk = g.sk;
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    float4 um = act ? ld4(U + c - sk) : zero, uc = act ? ld4(U + c) : zero;
#pragma unroll 2
    for (int k = k0; k < k1; k++) {
        const float4 up = act ? ld4(U + c + sk) : zero;
        const float4 uy = act ? add4(ld4(U + c - sj), ld4(U + c + sj)) : zero;
        const float4 bv = (MODE >= 1 && act) ? ld4(B + c) : zero;
        const float4 zv = (MODE == 2 && act) ? ld4(Z + c) : zero;
        float left = __shfl_up_sync(0xffffffffu, uc.w, 1), right = __shfl_down_sync(0xffffffffu, uc.x, 1);
        if (lane == 0) left = act ? U[c - 1] : 0.f;
        if (lane == 31) right = act && i0 + 4 < sj ? U[c + 4] : 0.f;
        float4 w;
        w.x = fmx(cf.cz, um.x + up.x, fmx(cf.cy, uy.x, fmx(cf.cx, left + uc.y, cf.cc * uc.x)));
        w.y = fmx(cf.cz, um.y + up.y, fmx(cf.cy, uy.y, fmx(cf.cx, uc.x + uc.z, cf.cc * uc.y)));
        w.z = fmx(cf.cz, um.z + up.z, fmx(cf.cy, uy.z, fmx(cf.cx, uc.y + uc.w, cf.cc * uc.z)));
        w.w = fmx(cf.cz, um.w + up.w, fmx(cf.cy, uy.w, fmx(cf.cx, uc.z + right, cf.cc * uc.w)));
        if (MODE >= 1) {
            w.x = fmx(cf.cb, bv.x, w.x);
            w.y = fmx(cf.cb, bv.y, w.y);
            w.z = fmx(cf.cb, bv.z, w.z);
            w.w = fmx(cf.cb, bv.w, w.w);
        }
        if (MODE == 2) {
            w.x = fmx(cf.cw, zv.x, w.x);
            w.y = fmx(cf.cw, zv.y, w.y);
            w.z = fmx(cf.cw, zv.z, w.z);
            w.w = fmx(cf.cw, zv.w, w.w);
        }
        if (act) {
            if (all4) {
                *reinterpret_cast<float4*>(W + c) = w;
            } else {
                if (m0) W[c] = w.x;
                if (m1) W[c + 1] = w.y;
                if (m2) W[c + 2] = w.z;
                if (m3) W[c + 3] = w.w;
            }
        }
        um = uc;
        uc = up;
        c += sk;
    }
}

template <int MODE>
__global__ void __launch_bounds__(256) k_cheb_v4(Geo g, Shape sh, const float* __restrict__ U,
                                                 const float* __restrict__ B, const float* __restrict__ Z,
                                                 float* __restrict__ W, CT<float> cf, const int* done)
{
    pdl_enter();
    EARLY_EXIT(done);
    const Col4 q = column4(g, sh);
    if (q.j >= g.hi[1]) return;   // a warp shares its row, so its lanes leave together
    cheb_v4_march<MODE>(g, q.i0, q.k0, q.k1, q.c, U, B, Z, W, cf);
}

// The vectorised kernels take FP32 fields whose rows start on 16-byte boundaries.
template <typename T>
static bool v4_ok(const Geo& g, const void* a, const void* b, const void* c, const void* d)
{
    if (!std::is_same<T, float>::value || g.sj % 4 != 0) return false;
    for (const void* p : {a, b, c, d})
        if (p && ((uintptr_t)p & 15u) != 0) return false;
    return true;
}

// Several Chebyshev steps in one pass (temporal blocking).  The steps s1..s_NS of
// the recurrence above (s1 from B, then sweeps; the last writes X = -s_NS) run as a
// wavefront along z over a tile of 32 x 16 columns: when B plane j is loaded, step t
// computes its plane j - 2t from planes of step t-1 (B for t = 1) that earlier
// iterations left in shared memory, so one barrier per plane orders everything.
// Step t covers the tile plus a halo of NS - t columns (the halo of B is NS), so the
// tile's outputs need no other block's work; step values off the unknowns are zero,
// as the guard cells of the unfused work fields are, and B is read as stored, its
// guard layer included.  The arithmetic is the unfused kernels' (same coefficients,
// same operand order), so the result is bit-identical to k_cheb_s01 followed by
// NS - 1 k_cheb_sweep launches.  Dirichlet grids only.
template <typename T>
struct ChebStages {
    CT<T> c[4];   // c[0]: s1 from B; c[t-1]: step t (c[NS-1] carries the -1 of the output)
};

constexpr int FUSE_TX = 32, FUSE_TY = 16;

template <int NS>
struct FuseDims {
    // step t (0: B) covers (32 + 2h) x (16 + 2h) columns, h = NS - t
    __host__ __device__ static constexpr int w(int t) { return FUSE_TX + 2 * (NS - t); }
    __host__ __device__ static constexpr int h(int t) { return FUSE_TY + 2 * (NS - t); }
    __host__ __device__ static constexpr int sz(int t) { return w(t) * h(t); }
    // ring depths: B is read back to plane j - 2NS (the last step's B term) and written
    // at j; step t (1 <= t < NS) is written at j - 2t and read back to j - 2t - 3
    // (step t+1's stencil) and j - 2t - 4 (step t+2's Z term)
    __host__ __device__ static constexpr int depth(int t) { return t == 0 ? 2 * NS + 1 : (t + 2 <= NS ? 5 : 4); }
    __host__ __device__ static constexpr int off(int t) { return t == 0 ? 0 : off(t - 1) + depth(t - 1) * sz(t - 1); }
    __host__ __device__ static constexpr int total() { return off(NS); }
};

template <typename T, int NS>
__global__ void __launch_bounds__(256) k_cheb_fused(Geo g, int ntx, int kchunk, const T* __restrict__ B,
                                                    T* __restrict__ X, ChebStages<T> cs, const int* done)
{
    pdl_enter();
    EARLY_EXIT(done);
    typedef FuseDims<NS> FD;
    constexpr int NT = 256;
    constexpr int NB = (FD::sz(0) + NT - 1) / NT;                 // B items per thread
    constexpr int NI = (FD::sz(1) + NT - 1) / NT;                 // step items per thread (the widest step)
    constexpr int NO = (FUSE_TX * FUSE_TY + NT - 1) / NT;         // output items per thread
    extern __shared__ __align__(16) unsigned char fuse_smem[];
    T* sm = reinterpret_cast<T*>(fuse_smem);
    const int tid = threadIdx.x + FUSE_TX * threadIdx.y;
    const int i0 = g.lo[0] + (blockIdx.x % ntx) * FUSE_TX;
    const int j0 = g.lo[1] + (blockIdx.x / ntx) * FUSE_TY;
    const int kb = g.lo[2] + blockIdx.y * kchunk;
    const int ke = min(kb + kchunk, g.hi[2]);
    const int base = kb - NS;   // first B plane; ring slots count planes from here
    const long long sk = g.sk;

    // Everything that does not depend on the plane is set up once per thread: the
    // B items' global column offsets, and for every step item its neighbour indices
    // in the previous step's region, in B's region and in step t-2's region.
    long long bofs[NB];
    bool bxy[NB];
#pragma unroll
    for (int r = 0; r < NB; r++) {
        const int q = tid + NT * r;
        const int a = q % FD::w(0), b = q / FD::w(0);
        const int i = i0 - NS + a, j = j0 - NS + b;
        bxy[r] = q < FD::sz(0) && i >= g.lo[0] - 1 && i <= g.hi[0] && j >= g.lo[1] - 1 && j <= g.hi[1];
        bofs[r] = bxy[r] ? (long long)i + g.sj * j : 0;
    }
    int ie[NS][NI], ib[NS][NI], iz[NS][NI];
    bool ixy[NS][NI];
    long long xofs[NO];
#pragma unroll
    for (int t = 1; t <= NS; t++) {
        const int wi = t < NS ? FD::w(t) : FUSE_TX;
        const int npos = t < NS ? FD::sz(t) : FUSE_TX * FUSE_TY;
        const int hal = NS - t;
#pragma unroll
        for (int r = 0; r < NI; r++) {
            const int q = tid + NT * r;
            const int a = q % wi, b = q / wi;
            const int i = i0 - hal + a, j = j0 - hal + b;
            ixy[t - 1][r] = q < npos && i >= g.lo[0] && i < g.hi[0] && j >= g.lo[1] && j < g.hi[1];
            ie[t - 1][r] = (b + 1) * FD::w(t - 1) + (a + 1);
            ib[t - 1][r] = (b + t) * FD::w(0) + (a + t);
            iz[t - 1][r] = t >= 3 ? (b + 2) * FD::w(t >= 3 ? t - 2 : 0) + (a + 2) : 0;
            if (t == NS && r < NO) xofs[r] = (long long)i + g.sj * j;
        }
    }
    auto plane_of = [&](int t, int p) -> T* { return sm + FD::off(t) + ((p - base) % FD::depth(t)) * FD::sz(t); };

    // B plane jp+1 is fetched into registers while the steps of iteration jp run, so
    // the global-memory latency overlaps the shared-memory work
    T breg[NB];
    auto fetch = [&](int jp) {
        const bool zs = jp >= g.lo[2] - 1 && jp <= g.hi[2];
        const long long zo = sk * jp;
#pragma unroll
        for (int r = 0; r < NB; r++) breg[r] = (bxy[r] && zs) ? B[bofs[r] + zo] : T(0);
    };
    fetch(base);
    for (int jp = base; jp < ke + 2 * NS; jp++) {
        if (jp < ke + NS) {
            T* dst = plane_of(0, jp);
#pragma unroll
            for (int r = 0; r < NB; r++) {
                const int q = tid + NT * r;
                if (q < FD::sz(0)) dst[q] = breg[r];
            }
            if (jp + 1 < ke + NS) fetch(jp + 1);
        }
#pragma unroll
        for (int t = 1; t <= NS; t++) {
            const int p = jp - 2 * t;   // plane of step t; its inputs were written by earlier iterations
            if (p >= kb - (NS - t) && p < ke + (NS - t)) {
                const CT<T> cf = cs.c[t - 1];
                const int wp = FD::w(t - 1);
                const T* ym = plane_of(t - 1, p - 1);
                const T* yc = plane_of(t - 1, p);
                const T* yp = plane_of(t - 1, p + 1);
                const T* bb = plane_of(0, p);
                const T* zz = plane_of(t >= 3 ? t - 2 : 0, p);
                T* out = plane_of(t < NS ? t : 0, p);
                const bool zin = p >= g.lo[2] && p < g.hi[2];
                const int npos = t < NS ? FD::sz(t) : FUSE_TX * FUSE_TY;
#pragma unroll
                for (int r = 0; r < NI; r++) {
                    const int q = tid + NT * r;
                    if (q >= npos) continue;
                    T v = T(0);
                    if (ixy[t - 1][r] && zin) {
                        const int e = ie[t - 1][r];
                        const T sx = yc[e - 1] + yc[e + 1];
                        const T sy = yc[e - wp] + yc[e + wp];
                        T w = cf.cc * yc[e];
                        w = fmx(cf.cx, sx, w);
                        w = fmx(cf.cy, sy, w);
                        w = fmx(cf.cz, ym[e] + yp[e], w);
                        if (t >= 2) w = fmx(cf.cb, bb[ib[t - 1][r]], w);
                        if (t >= 3) w = fmx(cf.cw, zz[iz[t - 1][r]], w);
                        v = w;
                    }
                    if (t < NS) out[q] = v;
                    else if (r < NO && p >= kb && p < ke && ixy[t - 1][r]) X[xofs[r] + sk * p] = v;
                }
            }
        }
        __syncthreads();
    }
}

template <typename T>
__global__ void __launch_bounds__(256) k_scale_copy(Geo g, Shape sh, const T* __restrict__ B, T* __restrict__ X, T a,
                                                    const int* done)
{
    pdl_enter();
    EARLY_EXIT(done);
    const Col q = column(g, sh);
    if (!q.active) return;
    long long c = q.c;
#pragma unroll 4
    for (int k = q.k0; k < q.k1; k++) {
        X[c] = a * B[c];
        c += g.sk;
    }
}

// Au = A(u); sum r0*Au   (BiCGSTAB.hpp:142-164, BiCGstab1Kernel)
template <typename T>
__global__ void __launch_bounds__(256) k_stencil_dot(Geo g, Shape sh, const T* __restrict__ u,
                                                     const T* __restrict__ r0, T* __restrict__ Au, Coef cf, RedCtx rc)
{
    pdl_enter();
    EARLY_EXIT(&rc.st->done);
    const Col q = column(g, sh);
    Acc<T> acc;
    if (q.active) {
        const T cc = (T)cf.cc, cx = (T)cf.cx, cy = (T)cf.cy, cz = (T)cf.cz;
        const long long sj = g.sj, sk = g.sk;
        long long c = q.c;
        T um = u[c - sk], uc = u[c];
#pragma unroll 4
        for (int k = q.k0; k < q.k1; k++) {
            const T up = u[c + sk];
            const T sx = u[c - 1] + u[c + 1];
            const T sy = u[c - sj] + u[c + sj];
            T a = cc * uc;
            a = fmx(cx, sx, a);
            a = fmx(cy, sy, a);
            a = fmx(cz, um + up, a);
            Au[c] = a;
            acc.add(r0[c], a);
            um = uc;
            uc = up;
            c += sk;
        }
    }
    double v[1] = {acc.value()};
    reduce_emit<1>(v, rc, sh);
}

// Au = A(u); sum r*Au, sum Au*Au   (BiCGSTAB.hpp:189-225, BiCGstab2Kernel)
template <typename T>
__global__ void __launch_bounds__(256) k_stencil_dot2(Geo g, Shape sh, const T* __restrict__ u,
                                                      const T* __restrict__ r, T* __restrict__ Au, Coef cf, RedCtx rc)
{
    pdl_enter();
    EARLY_EXIT(&rc.st->done);
    const Col q = column(g, sh);
    Acc<T> a1, a2;
    if (q.active) {
        const T cc = (T)cf.cc, cx = (T)cf.cx, cy = (T)cf.cy, cz = (T)cf.cz;
        const long long sj = g.sj, sk = g.sk;
        long long c = q.c;
        T um = u[c - sk], uc = u[c];
#pragma unroll 4
        for (int k = q.k0; k < q.k1; k++) {
            const T up = u[c + sk];
            const T sx = u[c - 1] + u[c + 1];
            const T sy = u[c - sj] + u[c + sj];
            T a = cc * uc;
            a = fmx(cx, sx, a);
            a = fmx(cy, sy, a);
            a = fmx(cz, um + up, a);
            Au[c] = a;
            a1.add(r[c], a);
            a2.add(a, a);
            um = uc;
            uc = up;
            c += sk;
        }
    }
    double v[2] = {a1.value(), a2.value()};
    reduce_emit<2>(v, rc, sh);
}

// r -= alpha*v   (BiCGSTAB.hpp:167-178)
template <typename T>
__global__ void __launch_bounds__(256) k_axpy_alpha(Geo g, Shape sh, T* __restrict__ r, const T* __restrict__ v,
                                                    const DevState* st)
{
    pdl_enter();
    EARLY_EXIT(&st->done);
    const Col q = column(g, sh);
    if (!q.active) return;
    const T a = (T)st->alpha;
    long long c = q.c;
#pragma unroll 4
    for (int k = q.k0; k < q.k1; k++) {
        r[c] = fmx(-a, v[c], r[c]);
        c += g.sk;
    }
}

// x += alpha*Mp + omega*z; r -= omega*Az; sums r0*r, r*r   (BiCGSTAB.hpp:227-257)
template <typename T>
__global__ void __launch_bounds__(256) k_update_xr(Geo g, Shape sh, T* __restrict__ x, const T* __restrict__ Mp,
                                                   const T* __restrict__ z, T* __restrict__ r,
                                                   const T* __restrict__ Az, const T* __restrict__ r0, RedCtx rc)
{
    pdl_enter();
    EARLY_EXIT(&rc.st->done);
    const Col q = column(g, sh);
    Acc<T> a1, a2;
    if (q.active) {
        const T a = (T)rc.st->alpha, w = (T)rc.st->omega;
        long long c = q.c;
#pragma unroll 4
        for (int k = q.k0; k < q.k1; k++) {
            x[c] = fmx(w, z[c], fmx(a, Mp[c], x[c]));
            const T rn = fmx(-w, Az[c], r[c]);
            r[c] = rn;
            a1.add(r0[c], rn);
            a2.add(rn, rn);
            c += g.sk;
        }
    }
    double v[2] = {a1.value(), a2.value()};
    reduce_emit<2>(v, rc, sh);
}

// p = r + beta*(p - omega*AMp)   (BiCGSTAB.hpp:261-272)
template <typename T>
__global__ void __launch_bounds__(256) k_update_p(Geo g, Shape sh, T* __restrict__ p, const T* __restrict__ r,
                                                  const T* __restrict__ AMp, const DevState* st)
{
    pdl_enter();
    EARLY_EXIT(&st->done);
    const Col q = column(g, sh);
    if (!q.active) return;
    const T be = (T)st->beta, w = (T)st->omega;
    long long c = q.c;
#pragma unroll 4
    for (int k = q.k0; k < q.k1; k++) {
        p[c] = fmx(be, fmx(-w, AMp[c], p[c]), r[c]);
        c += g.sk;
    }
}

// CG: Ap = A(p); sums r*z, p*Ap   (baseCG.hpp:126-150)
template <typename T>
__global__ void __launch_bounds__(256) k_cg_stencil_dot(Geo g, Shape sh, const T* __restrict__ p,
                                                        const T* __restrict__ r, const T* __restrict__ z,
                                                        T* __restrict__ Ap, Coef cf, RedCtx rc)
{
    pdl_enter();
    EARLY_EXIT(&rc.st->done);
    const Col q = column(g, sh);
    Acc<T> a1, a2;
    if (q.active) {
        const T cc = (T)cf.cc, cx = (T)cf.cx, cy = (T)cf.cy, cz = (T)cf.cz;
        const long long sj = g.sj, sk = g.sk;
        long long c = q.c;
        T um = p[c - sk], uc = p[c];
#pragma unroll 4
        for (int k = q.k0; k < q.k1; k++) {
            const T up = p[c + sk];
            const T sx = p[c - 1] + p[c + 1];
            const T sy = p[c - sj] + p[c + sj];
            T a = cc * uc;
            a = fmx(cx, sx, a);
            a = fmx(cy, sy, a);
            a = fmx(cz, um + up, a);
            Ap[c] = a;
            a1.add(r[c], z[c]);
            a2.add(uc, a);
            um = uc;
            uc = up;
            c += sk;
        }
    }
    double v[2] = {a1.value(), a2.value()};
    reduce_emit<2>(v, rc, sh);
}

// CG: x += alpha*p; r -= alpha*Ap   (baseCG.hpp:154-165)
template <typename T>
__global__ void __launch_bounds__(256) k_cg_update_xr(Geo g, Shape sh, T* __restrict__ x, const T* __restrict__ p,
                                                      T* __restrict__ r, const T* __restrict__ Ap, const DevState* st)
{
    pdl_enter();
    EARLY_EXIT(&st->done);
    const Col q = column(g, sh);
    if (!q.active) return;
    const T a = (T)st->alpha;
    long long c = q.c;
#pragma unroll 4
    for (int k = q.k0; k < q.k1; k++) {
        x[c] = fmx(a, p[c], x[c]);
        r[c] = fmx(-a, Ap[c], r[c]);
        c += g.sk;
    }
}

// CG: sums r*z, r*r   (baseCG.hpp:169-194)
template <typename T>
__global__ void __launch_bounds__(256) k_cg_dot_rz(Geo g, Shape sh, const T* __restrict__ r, const T* __restrict__ z,
                                                   RedCtx rc)
{
    pdl_enter();
    EARLY_EXIT(&rc.st->done);
    const Col q = column(g, sh);
    Acc<T> a1, a2;
    if (q.active) {
        long long c = q.c;
#pragma unroll 4
        for (int k = q.k0; k < q.k1; k++) {
            const T rv = r[c];
            a1.add(rv, z[c]);
            a2.add(rv, rv);
            c += g.sk;
        }
    }
    double v[2] = {a1.value(), a2.value()};
    reduce_emit<2>(v, rc, sh);
}

// CG: p = z + beta*p   (baseCG.hpp:197-207)
template <typename T>
__global__ void __launch_bounds__(256) k_cg_update_p(Geo g, Shape sh, T* __restrict__ p, const T* __restrict__ z,
                                                     const DevState* st)
{
    pdl_enter();
    EARLY_EXIT(&st->done);
    const Col q = column(g, sh);
    if (!q.active) return;
    const T be = (T)st->beta;
    long long c = q.c;
#pragma unroll 4
    for (int k = q.k0; k < q.k1; k++) {
        p[c] = fmx(be, p[c], z[c]);
        c += g.sk;
    }
}

// FCG: p_out = z + beta*p_in (z itself when beta = 0, the (re)start); Ap = A p_out;
// sums p_out.Ap.  The direction update rides on the stencil: each thread forms
// p_out at the 7 points from z and p_in, so p_in and p_out must be distinct fields.
template <typename T>
__global__ void __launch_bounds__(256) k_fcg_p_stencil(Geo g, Shape sh, const T* __restrict__ z,
                                                       const T* __restrict__ pin, T* __restrict__ pout,
                                                       T* __restrict__ Ap, Coef cf, RedCtx rc)
{
    pdl_enter();
    EARLY_EXIT(&rc.st->done);
    const Col q = column(g, sh);
    Acc<T> a1;
    if (q.active) {
        const T cc = (T)cf.cc, cx = (T)cf.cx, cy = (T)cf.cy, cz = (T)cf.cz;
        const bool restart = rc.st->beta == 0.0;
        const T be = (T)rc.st->beta;
        const long long sj = g.sj, sk = g.sk;
        auto pv = [&](long long c) -> T { return restart ? z[c] : fmx(be, pin[c], z[c]); };
        long long c = q.c;
        T um = pv(c - sk), uc = pv(c);
#pragma unroll 2
        for (int k = q.k0; k < q.k1; k++) {
            const T up = pv(c + sk);
            const T sx = pv(c - 1) + pv(c + 1);
            const T sy = pv(c - sj) + pv(c + sj);
            T a = cc * uc;
            a = fmx(cx, sx, a);
            a = fmx(cy, sy, a);
            a = fmx(cz, um + up, a);
            pout[c] = uc;
            Ap[c] = a;
            a1.add(uc, a);
            um = uc;
            uc = up;
            c += sk;
        }
    }
    double v[1] = {a1.value()};
    reduce_finalize<1>(v, rc);
}

// k_fcg_p_stencil on the x-vectorised FP32 tiles of k_cheb_v4: p = z + beta p_in
// formed at every tap (from float4 loads, the x neighbours by shuffle), Ap, and
// sum p.Ap over the unknowns.  The per-point arithmetic is k_fcg_p_stencil's; the
// sum visits the points in another order.
__global__ void __launch_bounds__(256) k_fcg_p_stencil_v4(Geo g, Shape sh, const float* __restrict__ z,
                                                          const float* __restrict__ pin, float* __restrict__ pout,
                                                          float* __restrict__ Ap, Coef cf, RedCtx rc)
{
    pdl_enter();
    EARLY_EXIT(&rc.st->done);
    const Col4 q = column4(g, sh);
    Acc<float> a1;
    if (q.j < g.hi[1]) {   // a warp shares its row: the shuffles below see all 32 lanes
        const bool act = q.act;
        const int lane = threadIdx.x;
        const bool m0 = q.i0 >= g.lo[0] && q.i0 < g.hi[0], m1 = q.i0 + 1 >= g.lo[0] && q.i0 + 1 < g.hi[0];
        const bool m2 = q.i0 + 2 >= g.lo[0] && q.i0 + 2 < g.hi[0], m3 = q.i0 + 3 >= g.lo[0] && q.i0 + 3 < g.hi[0];
        const bool all4 = m0 && m1 && m2 && m3;
        const float cc = (float)cf.cc, cx = (float)cf.cx, cy = (float)cf.cy, cz = (float)cf.cz;
        const bool restart = rc.st->beta == 0.0;
        const float be = (float)rc.st->beta;
        const long long sj = g.sj, sk = g.sk;
        const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
        auto pv4 = [&](long long c) -> float4 {
            if (!act) return zero;
            const float4 zv = ld4(z + c);
            if (restart) return zv;
            const float4 pv = ld4(pin + c);
            return make_float4(fmx(be, pv.x, zv.x), fmx(be, pv.y, zv.y), fmx(be, pv.z, zv.z), fmx(be, pv.w, zv.w));
        };
        auto pv1 = [&](long long c) -> float { return restart ? z[c] : fmx(be, pin[c], z[c]); };
        long long c = q.c;
        float4 um = pv4(c - sk), uc = pv4(c);
#pragma unroll 1
        for (int k = q.k0; k < q.k1; k++) {
            const float4 up = pv4(c + sk);
            const float4 uy = add4(pv4(c - sj), pv4(c + sj));
            float left = __shfl_up_sync(0xffffffffu, uc.w, 1), right = __shfl_down_sync(0xffffffffu, uc.x, 1);
            if (lane == 0) left = act ? pv1(c - 1) : 0.f;
            if (lane == 31) right = act && q.i0 + 4 < sj ? pv1(c + 4) : 0.f;
            float4 a;
            a.x = fmx(cz, um.x + up.x, fmx(cy, uy.x, fmx(cx, left + uc.y, cc * uc.x)));
            a.y = fmx(cz, um.y + up.y, fmx(cy, uy.y, fmx(cx, uc.x + uc.z, cc * uc.y)));
            a.z = fmx(cz, um.z + up.z, fmx(cy, uy.z, fmx(cx, uc.y + uc.w, cc * uc.z)));
            a.w = fmx(cz, um.w + up.w, fmx(cy, uy.w, fmx(cx, uc.z + right, cc * uc.w)));
            if (act) {
                if (all4) {
                    *reinterpret_cast<float4*>(pout + c) = uc;
                    *reinterpret_cast<float4*>(Ap + c) = a;
                } else {
                    if (m0) { pout[c] = uc.x; Ap[c] = a.x; }
                    if (m1) { pout[c + 1] = uc.y; Ap[c + 1] = a.y; }
                    if (m2) { pout[c + 2] = uc.z; Ap[c + 2] = a.z; }
                    if (m3) { pout[c + 3] = uc.w; Ap[c + 3] = a.w; }
                }
                if (m0) a1.add(uc.x, a.x);
                if (m1) a1.add(uc.y, a.y);
                if (m2) a1.add(uc.z, a.z);
                if (m3) a1.add(uc.w, a.w);
            }
            um = uc;
            uc = up;
            c += sk;
        }
    }
    double v[1] = {a1.value()};
    reduce_finalize<1>(v, rc);
}

// ---- bulk-copy staging (cp.async.bulk into shared memory, mbarrier completion) ----

__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
// one arrival that also announces the bytes the phase's bulk copies will deliver
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity)
{
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// one box of a tiled tensor map (coordinates x, y, z in elements; x * 4 bytes a multiple
// of 16) into this CTA's shared memory (128-byte aligned), completing on the mbarrier;
// the parts of the box outside the tensor arrive as zeros
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int zc,
                                            unsigned long long* bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smem_addr(dst)),
        "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(zc), "r"(smem_addr(bar))
        : "memory");
}
__device__ __forceinline__ unsigned long long globaltimer_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

constexpr int STAGE_ROW = 136;   // floats per staged row: x0 - 4 .. x0 + 131 (128 columns and their x halo)
constexpr int STAGES = 4;        // planes in the ring
constexpr unsigned long long STAGE_WAIT_NS = 2000000000ull;   // 2 s: a wait this long means a lost copy

// floats of one staged box (ty + 2 rows), rounded up to 128 bytes (TMA destinations)
__host__ __device__ constexpr int stage_box_floats(int ty) { return ((ty + 2) * STAGE_ROW + 31) / 32 * 32; }
static size_t stage_smem_bytes(int ty)
{
    return sizeof(float) * (size_t)STAGES * 2 * stage_box_floats(ty) + sizeof(unsigned long long) * STAGES;
}

// k_fcg_p_stencil_v4 with its inputs staged by TMA.  One thread copies, for each
// plane of the block's z range and the plane on either side, the tile's rows of z (and
// of p_in unless beta = 0) with the x and y halo into a ring of STAGES shared-memory slots,
// each completing on its own mbarrier; the block computes from shared memory while the
// next planes are in flight, so the loads' latency no longer sits in the registers of
// the computing threads.  Tiles, per-point arithmetic and per-thread sums are
// k_fcg_p_stencil_v4's, so every output and the block sums are bit-identical to it.
// A wait is bounded (STAGE_WAIT_NS by %globaltimer); one that runs out ends the solve
// with PPS_TIMEOUT (state done) and the block runs to its end on whatever arrived.
// The boxes come from tiled tensor maps over the padded fields (one copy per field and
// plane, 136 x (ty + 2) floats); box parts outside the field arrive as zeros, which is
// what the guard cells the register-marching kernel reads there hold.
__global__ void __launch_bounds__(256) k_fcg_p_stencil_staged(Geo g, Shape sh, const __grid_constant__ CUtensorMap tz,
                                                              const __grid_constant__ CUtensorMap tp,
                                                              float* __restrict__ pout, float* __restrict__ Ap, Coef cf,
                                                              RedCtx rc)
{
    pdl_enter();
    EARLY_EXIT(&rc.st->done);
    extern __shared__ __align__(128) unsigned char stage_raw[];
    const int ty = blockDim.y, box = stage_box_floats(ty);
    float* stage = reinterpret_cast<float*>(stage_raw);
    unsigned long long* bars =
        reinterpret_cast<unsigned long long*>(stage_raw + sizeof(float) * (size_t)STAGES * 2 * box);
    const int lane = threadIdx.x, wrow = threadIdx.y;
    const Col4 q = column4(g, sh);
    const int bx = blockIdx.x % sh.ntx, by = blockIdx.x / sh.ntx;
    const int x0 = bx * 128, ylo = g.lo[1] + by * ty;
    const int k0 = q.k0, k1 = q.k1, kbase = k0 - 1;
    const int xs = x0 - 4;                              // staged rows: x0 - 4 .. x0 + 131 of rows ylo - 1 .. ylo + ty
    const bool restart = rc.st->beta == 0.0;
    const int nf = restart ? 1 : 2;
    const unsigned plane_bytes = (unsigned)(nf * (ty + 2) * STAGE_ROW) * 4u;   // whole boxes, zeros included
    if (wrow == 0 && lane == 0) {
        for (int b = 0; b < STAGES; b++) mbar_init(&bars[b], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    auto slot_of = [&](int kk) { return (kk - kbase) % STAGES; };
    auto at = [&](int kk, int f, int rr) { return stage + (size_t)(slot_of(kk) * 2 + f) * box + rr * STAGE_ROW; };
    // thread 0: plane kk's box of z (and of p_in) into its slot (kk <= k1, the last plane any thread reads)
    auto issue = [&](int kk) {
        if (wrow != 0 || lane != 0 || kk > k1) return;
        unsigned long long* bar = &bars[slot_of(kk)];
        mbar_arrive_expect_tx(bar, plane_bytes);
        tma_load_3d(at(kk, 0, 0), &tz, xs, ylo - 1, kk, bar);
        if (!restart) tma_load_3d(at(kk, 1, 0), &tp, xs, ylo - 1, kk, bar);
    };
    bool lost = false;
    auto wait_plane = [&](int kk) {
        unsigned long long* bar = &bars[slot_of(kk)];
        const unsigned parity = (unsigned)((kk - kbase) / STAGES) & 1u;
        if (mbar_try_wait(bar, parity)) return;
        const unsigned long long t0 = globaltimer_ns();
        while (!mbar_try_wait(bar, parity)) {
            if (globaltimer_ns() - t0 > STAGE_WAIT_NS) {
                lost = true;
                return;
            }
        }
    };
    for (int kk = kbase; kk < kbase + STAGES; kk++) issue(kk);

    Acc<float> a1;
    const bool live = q.j < g.hi[1];   // a warp shares its row
    const bool act = live && q.act;
    const bool m0 = q.i0 >= g.lo[0] && q.i0 < g.hi[0], m1 = q.i0 + 1 >= g.lo[0] && q.i0 + 1 < g.hi[0];
    const bool m2 = q.i0 + 2 >= g.lo[0] && q.i0 + 2 < g.hi[0], m3 = q.i0 + 3 >= g.lo[0] && q.i0 + 3 < g.hi[0];
    const bool all4 = m0 && m1 && m2 && m3;
    const float cc = (float)cf.cc, cx = (float)cf.cx, cy = (float)cf.cy, cz = (float)cf.cz;
    const float be = (float)rc.st->beta;
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    const int xo = q.i0 - xs;   // the thread's float4 in a staged row (4 * lane + 4)
    const int rr0 = wrow + 1;   // the thread's row in the staged rows
    auto pv4 = [&](int kk, int rr) -> float4 {
        if (!act) return zero;
        const float4 zv = *reinterpret_cast<const float4*>(at(kk, 0, rr) + xo);
        if (restart) return zv;
        const float4 pv = *reinterpret_cast<const float4*>(at(kk, 1, rr) + xo);
        return make_float4(fmx(be, pv.x, zv.x), fmx(be, pv.y, zv.y), fmx(be, pv.z, zv.z), fmx(be, pv.w, zv.w));
    };
    auto pv1 = [&](int kk, int o) -> float {   // o: offset in the staged row
        const float zv = at(kk, 0, rr0)[o];
        return restart ? zv : fmx(be, at(kk, 1, rr0)[o], zv);
    };
    wait_plane(kbase);
    float4 um = pv4(kbase, rr0);
    wait_plane(k0);
    float4 uc = pv4(k0, rr0);
    __syncthreads();       // plane kbase's slot is free
    issue(kbase + STAGES);
    long long c = q.c;
#pragma unroll 1
    for (int k = k0; k < k1; k++) {
        wait_plane(k + 1);
        const float4 up = pv4(k + 1, rr0);
        const float4 uy = add4(pv4(k, rr0 - 1), pv4(k, rr0 + 1));
        float left = __shfl_up_sync(0xffffffffu, uc.w, 1), right = __shfl_down_sync(0xffffffffu, uc.x, 1);
        if (lane == 0) left = act ? pv1(k, xo - 1) : 0.f;
        if (lane == 31) right = act && q.i0 + 4 < g.sj ? pv1(k, xo + 4) : 0.f;
        float4 a;
        a.x = fmx(cz, um.x + up.x, fmx(cy, uy.x, fmx(cx, left + uc.y, cc * uc.x)));
        a.y = fmx(cz, um.y + up.y, fmx(cy, uy.y, fmx(cx, uc.x + uc.z, cc * uc.y)));
        a.z = fmx(cz, um.z + up.z, fmx(cy, uy.z, fmx(cx, uc.y + uc.w, cc * uc.z)));
        a.w = fmx(cz, um.w + up.w, fmx(cy, uy.w, fmx(cx, uc.z + right, cc * uc.w)));
        if (act) {
            if (all4) {
                *reinterpret_cast<float4*>(pout + c) = uc;
                *reinterpret_cast<float4*>(Ap + c) = a;
            } else {
                if (m0) { pout[c] = uc.x; Ap[c] = a.x; }
                if (m1) { pout[c + 1] = uc.y; Ap[c + 1] = a.y; }
                if (m2) { pout[c + 2] = uc.z; Ap[c + 2] = a.z; }
                if (m3) { pout[c + 3] = uc.w; Ap[c + 3] = a.w; }
            }
            if (m0) a1.add(uc.x, a.x);
            if (m1) a1.add(uc.y, a.y);
            if (m2) a1.add(uc.z, a.z);
            if (m3) a1.add(uc.w, a.w);
        }
        um = uc;
        uc = up;
        c += g.sk;
        __syncthreads();   // plane k's slot is free
        issue(k + STAGES);
    }
    if (lost) {
        rc.st->status = PPS_TIMEOUT;
        rc.st->done = 1;
    }
    double v[1] = {a1.value()};
    reduce_finalize<1>(v, rc);
}

// FCG: x += alpha*p; r -= alpha*Ap; sum r.r (the convergence test, before the
// preconditioner, which a converged iteration then skips)
template <typename T>
__global__ void __launch_bounds__(256) k_fcg_update_xr(Geo g, Shape sh, T* __restrict__ x, const T* __restrict__ p,
                                                       T* __restrict__ r, const T* __restrict__ Ap, RedCtx rc)
{
    pdl_enter();
    EARLY_EXIT(&rc.st->done);
    const Col q = column(g, sh);
    Acc<T> rr;
    if (q.active) {
        const T a = (T)rc.st->alpha;
        long long c = q.c;
#pragma unroll 4
        for (int k = q.k0; k < q.k1; k++) {
            x[c] = fmx(a, p[c], x[c]);
            const T rn = fmx(-a, Ap[c], r[c]);
            r[c] = rn;
            rr.add(rn, rn);
            c += g.sk;
        }
    }
    double v[1] = {rr.value()};
    reduce_finalize<1>(v, rc);
}

// FCG: sums z.r, z.Ap, r.r after the (possibly nonlinear) preconditioner; with
// r_new - r_old = -alpha Ap the Polak-Ribiere numerator is -alpha z.Ap
template <typename T>
__global__ void __launch_bounds__(256) k_fcg_dot(Geo g, Shape sh, const T* __restrict__ r, const T* __restrict__ z,
                                                 const T* __restrict__ Ap, RedCtx rc)
{
    pdl_enter();
    EARLY_EXIT(&rc.st->done);
    const Col q = column(g, sh);
    Acc<T> a1, a2, a3;
    if (q.active) {
        long long c = q.c;
#pragma unroll 4
        for (int k = q.k0; k < q.k1; k++) {
            const T rv = r[c], zv = z[c];
            a1.add(zv, rv);
            if (Ap) a2.add(zv, Ap[c]);
            a3.add(rv, rv);
            c += g.sk;
        }
    }
    double v[3] = {a1.value(), a2.value(), a3.value()};
    reduce_finalize<3>(v, rc);
}

// Flexible CG over the whole padded array in 16-byte vectors.  Every flexible-CG
// work field is zero on the guard cells (allocated zeroed, written only at the
// unknowns, Dirichlet grids only), so x += alpha*0 leaves the guard cells of x as
// they are and they add nothing to the sums.  The caller checks 16-byte alignment.
template <typename T>
struct Vec16;
template <>
struct Vec16<float> {
    typedef float4 type;
    static constexpr int n = 4;
    __device__ static float& at(float4& v, int i) { return (&v.x)[i]; }
};
template <>
struct Vec16<double> {
    typedef double2 type;
    static constexpr int n = 2;
    __device__ static double& at(double2& v, int i) { return (&v.x)[i]; }
};

template <typename T>
__global__ void __launch_bounds__(256) k_fcg_update_xr_flat(long long n, T* __restrict__ x, const T* __restrict__ p,
                                                            T* __restrict__ r, const T* __restrict__ Ap, RedCtx rc)
{
    pdl_enter();
    EARLY_EXIT(&rc.st->done);
    typedef Vec16<T> VT;
    typedef typename VT::type V;
    const T a = (T)rc.st->alpha;
    Acc<T> rr;
    const long long nv = n / VT::n, stride = (long long)gridDim.x * blockDim.x;
    const long long t0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    for (long long i = t0; i < nv; i += stride) {
        V xv = reinterpret_cast<const V*>(x)[i], rv = reinterpret_cast<const V*>(r)[i];
        V pv = reinterpret_cast<const V*>(p)[i], av = reinterpret_cast<const V*>(Ap)[i];
#pragma unroll
        for (int e = 0; e < VT::n; e++) {
            VT::at(xv, e) = fmx(a, VT::at(pv, e), VT::at(xv, e));
            VT::at(rv, e) = fmx(-a, VT::at(av, e), VT::at(rv, e));
            rr.add(VT::at(rv, e), VT::at(rv, e));
        }
        reinterpret_cast<V*>(x)[i] = xv;
        reinterpret_cast<V*>(r)[i] = rv;
    }
    for (long long i = nv * VT::n + t0; i < n; i += stride) {
        x[i] = fmx(a, p[i], x[i]);
        const T rn = fmx(-a, Ap[i], r[i]);
        r[i] = rn;
        rr.add(rn, rn);
    }
    double v[1] = {rr.value()};
    reduce_finalize<1>(v, rc);
}

template <typename T>
__global__ void __launch_bounds__(256) k_fcg_dot_flat(long long n, const T* __restrict__ r, const T* __restrict__ z,
                                                      const T* __restrict__ Ap, RedCtx rc)
{
    pdl_enter();
    EARLY_EXIT(&rc.st->done);
    typedef Vec16<T> VT;
    typedef typename VT::type V;
    Acc<T> a1, a2, a3;
    const long long nv = n / VT::n, stride = (long long)gridDim.x * blockDim.x;
    const long long t0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    for (long long i = t0; i < nv; i += stride) {
        V rv = reinterpret_cast<const V*>(r)[i], zv = reinterpret_cast<const V*>(z)[i];
        V av;
        if (Ap) av = reinterpret_cast<const V*>(Ap)[i];
#pragma unroll
        for (int e = 0; e < VT::n; e++) {
            a1.add(VT::at(zv, e), VT::at(rv, e));
            if (Ap) a2.add(VT::at(zv, e), VT::at(av, e));
            a3.add(VT::at(rv, e), VT::at(rv, e));
        }
    }
    for (long long i = nv * VT::n + t0; i < n; i += stride) {
        a1.add(z[i], r[i]);
        if (Ap) a2.add(z[i], Ap[i]);
        a3.add(r[i], r[i]);
    }
    double v[3] = {a1.value(), a2.value(), a3.value()};
    reduce_finalize<3>(v, rc);
}

// The BiCGSTAB updates in the same flat form (Dirichlet grids: r, r0, Mp, z, Az,
// AMp and p are zero off the unknowns, so the guard cells of x and p keep their
// values and add nothing to the sums; the reference itself updates x over every
// cell, BiCGSTAB.hpp:227-230).
// x += alpha Mp + omega z; r -= omega Az; sums r0.r, r.r   (BiCGSTAB.hpp:227-257)
template <typename T>
__global__ void __launch_bounds__(256) k_update_xr_flat(long long n, T* __restrict__ x, const T* __restrict__ Mp,
                                                        const T* __restrict__ z, T* __restrict__ r,
                                                        const T* __restrict__ Az, const T* __restrict__ r0, RedCtx rc)
{
    pdl_enter();
    EARLY_EXIT(&rc.st->done);
    typedef Vec16<T> VT;
    typedef typename VT::type V;
    const T a = (T)rc.st->alpha, w = (T)rc.st->omega;
    Acc<T> a1, a2;
    const long long nv = n / VT::n, stride = (long long)gridDim.x * blockDim.x;
    const long long t0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    for (long long i = t0; i < nv; i += stride) {
        V xv = reinterpret_cast<const V*>(x)[i], mv = reinterpret_cast<const V*>(Mp)[i];
        V zv = reinterpret_cast<const V*>(z)[i], rv = reinterpret_cast<const V*>(r)[i];
        V av = reinterpret_cast<const V*>(Az)[i], ov = reinterpret_cast<const V*>(r0)[i];
#pragma unroll
        for (int e = 0; e < VT::n; e++) {
            VT::at(xv, e) = fmx(w, VT::at(zv, e), fmx(a, VT::at(mv, e), VT::at(xv, e)));
            const T rn = fmx(-w, VT::at(av, e), VT::at(rv, e));
            VT::at(rv, e) = rn;
            a1.add(VT::at(ov, e), rn);
            a2.add(rn, rn);
        }
        reinterpret_cast<V*>(x)[i] = xv;
        reinterpret_cast<V*>(r)[i] = rv;
    }
    for (long long i = nv * VT::n + t0; i < n; i += stride) {
        x[i] = fmx(w, z[i], fmx(a, Mp[i], x[i]));
        const T rn = fmx(-w, Az[i], r[i]);
        r[i] = rn;
        a1.add(r0[i], rn);
        a2.add(rn, rn);
    }
    double v[2] = {a1.value(), a2.value()};
    reduce_finalize<2>(v, rc);
}

// p = r + beta (p - omega AMp)   (BiCGSTAB.hpp:261-272)
template <typename T>
__global__ void __launch_bounds__(256) k_update_p_flat(long long n, T* __restrict__ p, const T* __restrict__ r,
                                                       const T* __restrict__ AMp, const DevState* st)
{
    pdl_enter();
    EARLY_EXIT(&st->done);
    typedef Vec16<T> VT;
    typedef typename VT::type V;
    const T be = (T)st->beta, w = (T)st->omega;
    const long long nv = n / VT::n, stride = (long long)gridDim.x * blockDim.x;
    const long long t0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    for (long long i = t0; i < nv; i += stride) {
        V pv = reinterpret_cast<const V*>(p)[i], rv = reinterpret_cast<const V*>(r)[i];
        V av = reinterpret_cast<const V*>(AMp)[i];
#pragma unroll
        for (int e = 0; e < VT::n; e++) VT::at(pv, e) = fmx(be, fmx(-w, VT::at(av, e), VT::at(pv, e)), VT::at(rv, e));
        reinterpret_cast<V*>(p)[i] = pv;
    }
    for (long long i = nv * VT::n + t0; i < n; i += stride) p[i] = fmx(be, fmx(-w, AMp[i], p[i]), r[i]);
}

// r -= alpha v   (BiCGSTAB.hpp:167-178)
template <typename T>
__global__ void __launch_bounds__(256) k_axpy_alpha_flat(long long n, T* __restrict__ r, const T* __restrict__ v,
                                                         const DevState* st)
{
    pdl_enter();
    EARLY_EXIT(&st->done);
    typedef Vec16<T> VT;
    typedef typename VT::type V;
    const T a = (T)st->alpha;
    const long long nv = n / VT::n, stride = (long long)gridDim.x * blockDim.x;
    const long long t0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    for (long long i = t0; i < nv; i += stride) {
        V rv = reinterpret_cast<const V*>(r)[i], vv = reinterpret_cast<const V*>(v)[i];
#pragma unroll
        for (int e = 0; e < VT::n; e++) VT::at(rv, e) = fmx(-a, VT::at(vv, e), VT::at(rv, e));
        reinterpret_cast<V*>(r)[i] = rv;
    }
    for (long long i = nv * VT::n + t0; i < n; i += stride) r[i] = fmx(-a, v[i], r[i]);
}

// The BiCGSTAB stencils on the x-vectorised FP32 tiles: Au = A u and, NS = 1, sum
// w.Au (k_stencil_dot, w = r0) or, NS = 2, sums w.Au and Au.Au (k_stencil_dot2,
// w = r); per point the arithmetic of the one-column kernels, the sums in another
// order.
template <int NS>
__global__ void __launch_bounds__(256) k_stencil_dots_v4(Geo g, Shape sh, const float* __restrict__ u,
                                                         const float* __restrict__ wv, float* __restrict__ Au,
                                                         Coef cf, RedCtx rc)
{
    pdl_enter();
    EARLY_EXIT(&rc.st->done);
    const Col4 q = column4(g, sh);
    Acc<float> a1, a2;
    if (q.j < g.hi[1]) {   // a warp shares its row: the shuffles below see all 32 lanes
        const bool act = q.act;
        const int lane = threadIdx.x;
        const bool m0 = q.i0 >= g.lo[0] && q.i0 < g.hi[0], m1 = q.i0 + 1 >= g.lo[0] && q.i0 + 1 < g.hi[0];
        const bool m2 = q.i0 + 2 >= g.lo[0] && q.i0 + 2 < g.hi[0], m3 = q.i0 + 3 >= g.lo[0] && q.i0 + 3 < g.hi[0];
        const bool all4 = m0 && m1 && m2 && m3;
        const float cc = (float)cf.cc, cx = (float)cf.cx, cy = (float)cf.cy, cz = (float)cf.cz;
        const long long sj = g.sj, sk = g.sk;
        const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
        long long c = q.c;
        float4 um = act ? ld4(u + c - sk) : zero, uc = act ? ld4(u + c) : zero;
#pragma unroll 1
        for (int k = q.k0; k < q.k1; k++) {
            const float4 up = act ? ld4(u + c + sk) : zero;
            const float4 uy = act ? add4(ld4(u + c - sj), ld4(u + c + sj)) : zero;
            float left = __shfl_up_sync(0xffffffffu, uc.w, 1), right = __shfl_down_sync(0xffffffffu, uc.x, 1);
            if (lane == 0) left = act ? u[c - 1] : 0.f;
            if (lane == 31) right = act && q.i0 + 4 < sj ? u[c + 4] : 0.f;
            float4 a;
            a.x = fmx(cz, um.x + up.x, fmx(cy, uy.x, fmx(cx, left + uc.y, cc * uc.x)));
            a.y = fmx(cz, um.y + up.y, fmx(cy, uy.y, fmx(cx, uc.x + uc.z, cc * uc.y)));
            a.z = fmx(cz, um.z + up.z, fmx(cy, uy.z, fmx(cx, uc.y + uc.w, cc * uc.z)));
            a.w = fmx(cz, um.w + up.w, fmx(cy, uy.w, fmx(cx, uc.z + right, cc * uc.w)));
            if (act) {
                const float4 w4 = ld4(wv + c);
                if (all4) {
                    *reinterpret_cast<float4*>(Au + c) = a;
                } else {
                    if (m0) Au[c] = a.x;
                    if (m1) Au[c + 1] = a.y;
                    if (m2) Au[c + 2] = a.z;
                    if (m3) Au[c + 3] = a.w;
                }
                if (m0) {
                    a1.add(w4.x, a.x);
                    if (NS == 2) a2.add(a.x, a.x);
                }
                if (m1) {
                    a1.add(w4.y, a.y);
                    if (NS == 2) a2.add(a.y, a.y);
                }
                if (m2) {
                    a1.add(w4.z, a.z);
                    if (NS == 2) a2.add(a.z, a.z);
                }
                if (m3) {
                    a1.add(w4.w, a.w);
                    if (NS == 2) a2.add(a.w, a.w);
                }
            }
            um = uc;
            uc = up;
            c += sk;
        }
    }
    if (NS == 1) {
        double v[1] = {a1.value()};
        reduce_finalize<1>(v, rc);
    } else {
        double v[2] = {a1.value(), a2.value()};
        reduce_finalize<2>(v, rc);
    }
}

// r = b - A x in FP64 (computeErrorOperatorA, iterativeSolverBase.hpp:236-280),
// stored as TR; optional copies into r0 and p (BiCGSTAB.hpp:125-126); sum r^2.
// A double as m * 2^(e - 1075) with |m| < 2^53 (subnormals: e = 1, no hidden bit).
struct MI {
    long long m;
    int e;
};
__device__ __forceinline__ MI msplit(double v)
{
    const long long u = __double_as_longlong(v);
    const int ex = (int)(u >> 52) & 0x7ff;
    const long long mag = (u & 0xFFFFFFFFFFFFFll) | ((long long)(ex != 0) << 52);
    const long long sgn = u >> 63;   // 0 or -1
    MI r;
    r.m = (mag ^ sgn) - sgn;
    r.e = ex + (ex == 0);
    return r;
}
// m * 2^(e - E) for E >= e, rounded toward minus infinity (one arithmetic shift)
__device__ __forceinline__ long long malign(const MI& a, int E)
{
    return a.m >> min(E - a.e, 63);
}

// FP64 kernels on equal spacings (cx = cy = cz): GB300 issues FP64 at 1/64 of the
// FP32 rate, so the plain FP64 stencil (three pair sums and four multiply-adds) is
// bound by the FP64 pipe, not by HBM.  With one weight for the six neighbours their
// sum moves to the integer pipe: each value as m * 2^(e-1075) (msplit), aligned to
// the largest exponent E by an arithmetic shift, summed exactly in int64
// (|sum| < 6 * 2^53), converted once, and scaled by 2^(E-1075) in the exponent bits.
// The shifts drop at most one unit of 2^(E-1075) per value, the rounding FP64
// additions of the same values have anyway.  INT_CONVERT: the conversion too runs
// on the integer pipe (scaled_i2d), for kernels whose FP64 pipe is the bound.
// Returns false when a value is Inf/NaN
// (E = 2047) or the scaling would leave the normal range (E < 53 or E > 2000); the
// caller then adds in FP64.
// S * 2^(E-1075) as a double for 0 < |S| < 2^56 and 53 <= E <= 2000, on the integer
// pipe (the int64 -> FP64 conversion instruction issues on the FP64 pipe): the
// leading one of |S| moves to bit 52, the bits below are rounded half away from
// zero (|S| >= 2^53 only), and the exponent field is written directly (p + E - 52
// lies in [1, 2004], so the result is normal).
__device__ __forceinline__ double scaled_i2d(long long S, int E)
{
    const unsigned long long sg = (unsigned long long)S & 0x8000000000000000ull;
    const unsigned long long a = S < 0 ? 0ull - (unsigned long long)S : (unsigned long long)S;
    int p = 63 - __clzll((long long)a);
    unsigned long long mant;
    if (p > 52) {
        mant = ((a >> (p - 53)) + 1ull) >> 1;
        if (mant >> 53) {
            mant >>= 1;
            p++;
        }
    } else {
        mant = a << (52 - p);
    }
    return __longlong_as_double((long long)(sg | ((unsigned long long)(p + E - 52) << 52) | (mant & 0xFFFFFFFFFFFFFull)));
}

template <bool INT_CONVERT>
__device__ __forceinline__ bool nsum6(const MI& a, const MI& b, const MI& c, const MI& d, const MI& e, const MI& f,
                                      double& out)
{
    const int E = max(max(max(a.e, b.e), max(c.e, d.e)), max(e.e, f.e));
    if (E < 53 || E > 2000) return false;
    const long long S = malign(a, E) + malign(b, E) + malign(c, E) + malign(d, E) + malign(e, E) + malign(f, E);
    if (S == 0) {
        out = 0.0;
        return true;
    }
    if (INT_CONVERT) out = scaled_i2d(S, E);
    else out = __longlong_as_double(__double_as_longlong(__ll2double_rn(S)) + ((long long)(E - 1075) << 52));
    return true;
}

// The Chebyshev steps of the FP64 form on equal spacings (one column per thread, z
// kept in registers with its integer split):
//   MODE 0: W = cc U + cx (sum of U's six neighbours)               (s1, U = B)
//   MODE 1: W = cc U + cx (six-neighbour sum) + cb B                 (first sweep)
//   MODE 2: W = cc U + cx (six-neighbour sum) + cb B + cw Z          (later sweeps)
// with the coefficients of k_cheb_s01 / k_cheb_sweep: 3, 4 or 5 FP64 operations per
// unknown instead of 8 or 9.
template <int MODE>
__global__ void __launch_bounds__(256) k_cheb_iso64(Geo g, Shape sh, const double* __restrict__ U,
                                                    const double* __restrict__ B, const double* __restrict__ Z,
                                                    double* __restrict__ W, CT<double> cf, const int* done)
{
    pdl_enter();
    EARLY_EXIT(done);
    const Col q = column(g, sh);
    if (!q.active) return;
    const long long sj = g.sj, sk = g.sk;
    long long c = q.c;
    double um = U[c - sk], uc = U[c];
    MI mm = msplit(um), mc = msplit(uc);
#pragma unroll 2
    for (int k = q.k0; k < q.k1; k++) {
        const double up = U[c + sk];
        const double xw = U[c - 1], xe = U[c + 1], ys = U[c - sj], yn = U[c + sj];
        const MI mp = msplit(up);
        double s6, w;
        if (nsum6<true>(msplit(xw), msplit(xe), msplit(ys), msplit(yn), mm, mp, s6)) {
            w = fmx(cf.cx, s6, cf.cc * uc);
        } else {
            w = cf.cc * uc;
            w = fmx(cf.cx, xw + xe, w);
            w = fmx(cf.cy, ys + yn, w);
            w = fmx(cf.cz, um + up, w);
        }
        if (MODE >= 1) w = fmx(cf.cb, B[c], w);
        if (MODE == 2) w = fmx(cf.cw, Z[c], w);
        W[c] = w;
        um = uc;
        uc = up;
        mm = mc;
        mc = mp;
        c += sk;
    }
}

// Au = A u with the six-neighbour sum on the integer pipe (equal spacings), and
// NS = 1: sum w.Au (k_stencil_dot, w = r0); NS = 2: sums w.Au, Au.Au (k_stencil_dot2,
// w = r).  Three FP64 operations per unknown for A u instead of seven.
template <int NS>
__global__ void __launch_bounds__(256, 4) k_stencil_dots_iso64(Geo g, Shape sh, const double* __restrict__ u,
                                                            const double* __restrict__ w, double* __restrict__ Au,
                                                            Coef cf, RedCtx rc)
{
    pdl_enter();
    EARLY_EXIT(&rc.st->done);
    const Col q = column(g, sh);
    Acc<double> a1, a2;
    if (q.active) {
        const long long sj = g.sj, sk = g.sk;
        long long c = q.c;
        double um = u[c - sk], uc = u[c];
        MI mm = msplit(um), mc = msplit(uc);
#pragma unroll 2
        for (int k = q.k0; k < q.k1; k++) {
            const double up = u[c + sk];
            const double xw = u[c - 1], xe = u[c + 1], ys = u[c - sj], yn = u[c + sj];
            const MI mp = msplit(up);
            double s6, a;
            if (nsum6<true>(msplit(xw), msplit(xe), msplit(ys), msplit(yn), mm, mp, s6)) {
                a = fmx(cf.cx, s6, cf.cc * uc);
            } else {
                a = cf.cc * uc;
                a = fmx(cf.cx, xw + xe, a);
                a = fmx(cf.cy, ys + yn, a);
                a = fmx(cf.cz, um + up, a);
            }
            Au[c] = a;
            a1.add(w[c], a);
            if (NS == 2) a2.add(a, a);
            um = uc;
            uc = up;
            mm = mc;
            mc = mp;
            c += sk;
        }
    }
    double v[NS];
    v[0] = a1.value();
    if (NS == 2) v[NS - 1] = a2.value();
    reduce_emit<NS>(v, rc, sh);
}

// Counts the entries of a whole field (guard layers included) whose bit pattern is
// not +-0, in 16-byte vectors.
__global__ void __launch_bounds__(256) k_count_nonzero(long long n, const double* __restrict__ x, RedCtx rc)
{
    pdl_enter();
    double cnt = 0.0;
    const long long nv = n / 2, stride = (long long)gridDim.x * blockDim.x;
    const long long t0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const longlong2* xv = reinterpret_cast<const longlong2*>(x);
    long long i = t0;
    for (; i + 3 * stride < nv; i += 4 * stride) {   // four loads in flight per thread
        longlong2 v[4];
#pragma unroll
        for (int u = 0; u < 4; u++) v[u] = xv[i + u * stride];
#pragma unroll
        for (int u = 0; u < 4; u++) cnt += ((unsigned long long)v[u].x << 1 != 0ull) + ((unsigned long long)v[u].y << 1 != 0ull);
    }
    for (; i < nv; i += stride) {
        const longlong2 v = xv[i];
        cnt += ((unsigned long long)v.x << 1 != 0ull) + ((unsigned long long)v.y << 1 != 0ull);
    }
    for (long long i = nv * 2 + t0; i < n; i += stride) cnt += ((unsigned long long)__double_as_longlong(x[i]) << 1) != 0ull;
    double v[1] = {cnt};
    reduce_finalize<1>(v, rc);
}

// Sets *flag to 1 when some entry of a whole field (guard layers included) is not
// +-0.  It runs on a second stream while the solve works on b, so it takes no
// reduction state of the solver: one block-wide OR and a plain store of 1.
__global__ void __launch_bounds__(256) k_flag_nonzero(long long n, const double* __restrict__ x, int* __restrict__ flag)
{
    pdl_enter();
    const long long nv = n / 2, stride = (long long)gridDim.x * blockDim.x;
    const long long t0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const longlong2* xv = reinterpret_cast<const longlong2*>(x);
    unsigned long long bits = 0;
    long long i = t0;
    for (; i + 3 * stride < nv; i += 4 * stride) {   // four loads in flight per thread
        longlong2 v[4];
#pragma unroll
        for (int u = 0; u < 4; u++) v[u] = xv[i + u * stride];
#pragma unroll
        for (int u = 0; u < 4; u++) bits |= ((unsigned long long)v[u].x << 1) | ((unsigned long long)v[u].y << 1);
    }
    for (; i < nv; i += stride) {
        const longlong2 v = xv[i];
        bits |= ((unsigned long long)v.x << 1) | ((unsigned long long)v.y << 1);
    }
    for (long long j = nv * 2 + t0; j < n; j += stride) bits |= (unsigned long long)__double_as_longlong(x[j]) << 1;
    if (__syncthreads_or(bits != 0ull) && threadIdx.x == 0) *flag = 1;
}

// ISO: equal spacings on the three axes, so the six neighbours share one weight
// (GB300 runs FP64 at 1/64 of the FP32 rate, and this kernel is bound by it).  The
// sum of squares of the stored value accumulates in double-float for TR = float.
template <typename TR, bool ISO, bool XZERO>
__global__ void __launch_bounds__(256) k_residual(Geo g, Shape sh, const double* __restrict__ x,
                                                  const double* __restrict__ b, TR* __restrict__ r,
                                                  TR* __restrict__ r0, TR* __restrict__ p, Coef cf, RedCtx rc)
{
    pdl_enter();
    const Col q = column(g, sh);
    Acc<TR> acc;
    if (XZERO && q.active) {   // x = 0 on every point the stencil reads: r = b
        const long long sk = g.sk;
        long long c = q.c;
        int k = q.k0;
        auto put = [&](long long cc, double bv) {
            const TR rs = (TR)bv;
            r[cc] = rs;
            if (r0) r0[cc] = rs;
            if (p) p[cc] = rs;
            acc.add(rs, rs);
        };
        for (; k + 4 <= q.k1; k += 4, c += 4 * sk) {   // four planes' loads in flight, summed in plane order
            double bv[4];
#pragma unroll
            for (int u = 0; u < 4; u++) bv[u] = b[c + u * sk];
#pragma unroll
            for (int u = 0; u < 4; u++) put(c + u * sk, bv[u]);
        }
        for (; k < q.k1; k++, c += sk) put(c, b[c]);
    } else if (ISO && q.active) {
        // Equal spacings: A x = cx (sum of the six neighbours - 6 x).  The seven values
        // are aligned to the largest one's exponent as 53-bit integers, so the second
        // difference is exact in int64 on the integer pipe; one conversion and one FMA
        // remain on the FP64 pipe (instead of eight operations).  Dropping the smaller
        // values' low bits (an arithmetic shift) costs at most 2^-53 of the largest per
        // value, the rounding the FP64 stencil has anyway.
        const long long sj = g.sj, sk = g.sk;
        long long c = q.c;
        MI um = msplit(x[c - sk]), uc = msplit(x[c]);
        for (int k = q.k0; k < q.k1; k++) {
            const MI up = msplit(x[c + sk]);
            const MI w = msplit(x[c - 1]), e = msplit(x[c + 1]), sv = msplit(x[c - sj]), nv = msplit(x[c + sj]);
            const int E = max(max(max(um.e, uc.e), max(up.e, w.e)), max(max(e.e, sv.e), nv.e));
            double rv;
            if (E == 2047) {   // an Inf or NaN: let FP64 arithmetic propagate it
                rv = b[c] - cf.cx * (x[c - 1] + x[c + 1] + x[c - sj] + x[c + sj] + x[c - sk] + x[c + sk] - 6.0 * x[c]);
            } else {
                const long long D = malign(w, E) + malign(e, E) + malign(sv, E) + malign(nv, E) + malign(um, E) +
                                    malign(up, E) - 6 * malign(uc, E);
                // A x = cx * D * 2^(E - 1075); below 2^-1022 it is far under b's rounding.
                // The power of two goes into the exponent bits of D on the integer pipe
                // (exact: D converts to a normal double and the sum stays normal).
                const double Dd = __ll2double_rn(D);
                if (E >= 53 && E <= 2000) {
                    const double Ds = D != 0 ? __longlong_as_double(__double_as_longlong(Dd) + ((long long)(E - 1075) << 52))
                                             : 0.0;
                    rv = fmx(-cf.cx, Ds, b[c]);
                } else if (E > 2000) {
                    // magnitudes near the top of the range: cx * D first, then the power of
                    // two 2^(E-1075) (a normal double), so nothing overflows while A x is
                    // finite, and D = 0 gives b exactly
                    rv = fmx(-(cf.cx * Dd), __longlong_as_double((long long)(E - 52) << 52), b[c]);
                } else {
                    rv = b[c];   // every value below 2^-1022: A x is far under b's rounding
                }
            }
            const TR rs = (TR)rv;
            r[c] = rs;
            if (r0) r0[c] = rs;
            if (p) p[c] = rs;
            acc.add(rs, rs);
            um = uc;
            uc = up;
            c += sk;
        }
    } else if (q.active) {
        const long long sj = g.sj, sk = g.sk;
        long long c = q.c;
        double um = x[c - sk], uc = x[c];
        for (int k = q.k0; k < q.k1; k++) {
            const double up = x[c + sk];
            const double sx = x[c - 1] + x[c + 1];
            const double sy = x[c - sj] + x[c + sj];
            double a;
            {
                a = cf.cc * uc;
                a = fmx(cf.cx, sx, a);
                a = fmx(cf.cy, sy, a);
                a = fmx(cf.cz, um + up, a);
            }
            const double rv = b[c] - a;
            const TR rs = (TR)rv;
            r[c] = rs;
            if (r0) r0[c] = rs;
            if (p) p[c] = rs;
            acc.add(rs, rs);
            um = uc;
            uc = up;
            c += sk;
        }
    }
    double v[1] = {acc.value()};
    reduce_emit<1>(v, rc, sh);
}

// sum b_adj^2 over the unknowns (normalizeProblemToFieldBNorm, iterativeSolverBase.hpp:171-234);
// XZERO: Dirichlet grid with x = 0 everywhere, so b_adj = b
template <bool XZERO>
__global__ void __launch_bounds__(256) k_norm_badj(Geo g, Shape sh, const double* __restrict__ b,
                                                   const double* __restrict__ x, Faces f, RedCtx rc)
{
    pdl_enter();
    const Col q = column(g, sh);
    double s = 0.0;
    if (XZERO && q.active) {   // four planes' loads in flight, summed in plane order
        const long long sk = g.sk;
        long long c = q.c;
        int k = q.k0;
        for (; k + 4 <= q.k1; k += 4, c += 4 * sk) {
            double v[4];
#pragma unroll
            for (int u = 0; u < 4; u++) v[u] = b[c + u * sk];
#pragma unroll
            for (int u = 0; u < 4; u++) s = fmx(v[u], v[u], s);
        }
        for (; k < q.k1; k++, c += sk) s = fmx(b[c], b[c], s);
    } else if (q.active) {
        long long c = q.c;
        for (int k = q.k0; k < q.k1; k++) {
            const double v = badj_exact(g, b, x, f, c, q.i, q.j, k);
            s = fmx(v, v, s);
            c += g.sk;
        }
    }
    double v[1] = {s};
    reduce_emit<1>(v, rc, sh);
}

__global__ void __launch_bounds__(256) k_add_correction(Geo g, Shape sh, double* __restrict__ x,
                                                        const float* __restrict__ e)
{
    pdl_enter();
    const Col q = column(g, sh);
    if (!q.active) return;
    const long long sk = g.sk;
    long long c = q.c;
    int k = q.k0;
    for (; k + 4 <= q.k1; k += 4, c += 4 * sk) {   // four planes' loads in flight
        double xv[4];
        float ev[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            xv[u] = x[c + u * sk];
            ev[u] = e[c + u * sk];
        }
#pragma unroll
        for (int u = 0; u < 4; u++) x[c + u * sk] = xv[u] + (double)ev[u];
    }
    for (; k < q.k1; k++, c += sk) x[c] += (double)e[c];
}

// The same over the whole padded array in 16-byte vectors, for corrections that are
// +-0 off the unknowns (Dirichlet grids): x changes only where e is non-zero, so
// the boundary nodes and guards keep their bits.
__global__ void __launch_bounds__(256) k_add_correction_flat(long long n, double* __restrict__ x,
                                                             const float* __restrict__ e)
{
    pdl_enter();
    const long long nv = n / 2, stride = (long long)gridDim.x * blockDim.x;
    const long long t0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double2* xv = reinterpret_cast<double2*>(x);
    const float2* ev = reinterpret_cast<const float2*>(e);
    long long i = t0;
    for (; i + stride < nv; i += 2 * stride) {   // two vectors of each in flight per thread
        double2 a = xv[i], b = xv[i + stride];
        const float2 ea = ev[i], eb = ev[i + stride];
        if (ea.x != 0.0f) a.x += (double)ea.x;
        if (ea.y != 0.0f) a.y += (double)ea.y;
        if (eb.x != 0.0f) b.x += (double)eb.x;
        if (eb.y != 0.0f) b.y += (double)eb.y;
        xv[i] = a;
        xv[i + stride] = b;
    }
    for (; i < nv; i += stride) {
        double2 a = xv[i];
        const float2 ea = ev[i];
        if (ea.x != 0.0f) a.x += (double)ea.x;
        if (ea.y != 0.0f) a.y += (double)ea.y;
        xv[i] = a;
    }
    for (long long q = nv * 2 + t0; q < n; q += stride)
        if (e[q] != 0.0f) x[q] += (double)e[q];
}

// Start of an inner BiCGSTAB solve from X = 0 (BiCGSTAB.hpp:94-126 with isMainLoop
// false): the residual of the zero iterate is B, so r = r0 = p = B at the unknowns,
// and sum B^2 feeds FIN_RES0 (||B|| is the normalisation and the initial residual).
template <typename T>
__global__ void __launch_bounds__(256) k_bicg_start(Geo g, Shape sh, const T* __restrict__ B, T* __restrict__ r,
                                                    T* __restrict__ r0, T* __restrict__ p, RedCtx rc)
{
    pdl_enter();
    EARLY_EXIT(&rc.st->done);
    const Col q = column(g, sh);
    Acc<T> a;
    if (q.active) {
        long long c = q.c;
#pragma unroll 4
        for (int k = q.k0; k < q.k1; k++) {
            const T v = B[c];
            r[c] = v;
            r0[c] = v;
            p[c] = v;
            a.add(v, v);
            c += g.sk;
        }
    }
    double v[1] = {a.value()};
    reduce_emit<1>(v, rc, sh);
}

__global__ void k_cast_f32(const double* __restrict__ in, float* __restrict__ out, long long n)
{
    pdl_enter();
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x)
        out[c] = (float)in[c];
}

template <typename T>
__global__ void k_fill(T* p, long long n, T v)
{
    pdl_enter();
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x)
        p[c] = v;
}

// Zero every entry of a padded field that is not an unknown (boundary nodes and
// guard layers), the state the solver's work fields keep between solves.
template <typename T>
__global__ void k_zero_off_unknowns(Geo g, T* p)
{
    pdl_enter();
    const long long nj = g.sk / g.sj;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < g.ntot;
         c += (long long)gridDim.x * blockDim.x) {
        const long long i = c % g.sj, j = (c / g.sj) % nj, k = c / g.sk;
        const bool unknown = i >= g.lo[0] && i < g.hi[0] && j >= g.lo[1] && j < g.hi[1] && k >= g.lo[2] && k < g.hi[2];
        if (!unknown) p[c] = (T)0;
    }
}

__global__ void k_state_init(DevState* st, double* hist, int maxit, double tol_abs, double tol_rel, int tol_relative,
                             int rho0_from_r, double hist_scale, int hist_cap)
{
    pdl_enter();
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        st->rho0 = 1.0;
        st->alpha = st->omega = st->beta = 1.0;
        st->err = -1.0;
        st->err0 = -1.0;
        st->tol_abs = tol_abs;
        st->tol_rel = tol_rel;
        st->tol_relative = tol_relative;
        st->rho0_from_r = rho0_from_r;
        st->hist_scale = hist_scale;
        st->hist_cap = hist_cap;
        st->iter = 0;
        st->maxit = maxit;
        st->done = 0;
        st->status = 0;
        for (int q = 0; q < 4; q++) st->sums[q] = 0.0;
    }
}

// ---- wrappers ----

template <typename T>
void fast_cheb_s01(const Geo& g, const Shape& sh, const T* B, T* Y, const Coef& cy, const int* done, cudaStream_t s)
{
    const CT<T> c = cast_coef<T>(cy);
    if (sh.cx == 4) {
        if constexpr (std::is_same<T, float>::value) {
            if (v4_ok<T>(g, B, Y, nullptr, nullptr)) {
                launch_pdl(k_cheb_v4<0>, grid_of(sh), block_of(sh), 0, s, g, sh, B, nullptr, nullptr, Y, c, done);
                PPS_COUNT_LAUNCH();
                return;
            }
        }
        fast_cheb_s01<T>(g, make_shape(g, sh.ty, (int)sh.nblocks(), 1), B, Y, cy, done, s);   // scalar tiles
        return;
    }
    if constexpr (std::is_same<T, double>::value) {
        if (iso_coef(cy)) {   // equal spacings: the neighbour sum on the integer pipe
            const Shape c1 = sh.cx == 1 ? sh : make_shape(g, sh.ty, (int)sh.nblocks(), 1);
            launch_pdl(k_cheb_iso64<0>, grid_of(c1), block_of(c1), 0, s, g, c1, B, nullptr, nullptr, Y, c, done);
            PPS_COUNT_LAUNCH();
            return;
        }
    }
    if (sh.cx == 2) launch_pdl(k_cheb_s01<T, 2>, grid_of(sh), block_of(sh), 0, s, g, sh, B, Y, c, done);
    else launch_pdl(k_cheb_s01<T, 1>, grid_of(sh), block_of(sh), 0, s, g, sh, B, Y, c, done);
    PPS_COUNT_LAUNCH();
}
template <typename T>
void fast_cheb_sweep(const Geo& g, const Shape& sh, const T* Y, const T* B, const T* Z, T* W, const Coef& cf,
                     const int* done, cudaStream_t s)
{
    const CT<T> c = cast_coef<T>(cf);
    if (sh.cx == 4) {
        if constexpr (std::is_same<T, float>::value) {
            if (v4_ok<T>(g, Y, B, Z, W)) {
                if (Z) launch_pdl(k_cheb_v4<2>, grid_of(sh), block_of(sh), 0, s, g, sh, Y, B, Z, W, c, done);
                else launch_pdl(k_cheb_v4<1>, grid_of(sh), block_of(sh), 0, s, g, sh, Y, B, Z, W, c, done);
                PPS_COUNT_LAUNCH();
                return;
            }
        }
        fast_cheb_sweep<T>(g, make_shape(g, sh.ty, (int)sh.nblocks(), 1), Y, B, Z, W, cf, done, s);   // scalar tiles
        return;
    }
    if constexpr (std::is_same<T, double>::value) {
        if (iso_coef(cf)) {   // equal spacings: the neighbour sum on the integer pipe
            const Shape c1 = sh.cx == 1 ? sh : make_shape(g, sh.ty, (int)sh.nblocks(), 1);
            if (Z) launch_pdl(k_cheb_iso64<2>, grid_of(c1), block_of(c1), 0, s, g, c1, Y, B, Z, W, c, done);
            else launch_pdl(k_cheb_iso64<1>, grid_of(c1), block_of(c1), 0, s, g, c1, Y, B, Z, W, c, done);
            PPS_COUNT_LAUNCH();
            return;
        }
    }
    if (Z) {
        if (sh.cx == 2) launch_pdl(k_cheb_sweep<T, 2, true>, grid_of(sh), block_of(sh), 0, s, g, sh, Y, B, Z, W, c, done);
        else launch_pdl(k_cheb_sweep<T, 1, true>, grid_of(sh), block_of(sh), 0, s, g, sh, Y, B, Z, W, c, done);
    } else {
        if (sh.cx == 2) launch_pdl(k_cheb_sweep<T, 2, false>, grid_of(sh), block_of(sh), 0, s, g, sh, Y, B, Z, W, c, done);
        else launch_pdl(k_cheb_sweep<T, 1, false>, grid_of(sh), block_of(sh), 0, s, g, sh, Y, B, Z, W, c, done);
    }
    PPS_COUNT_LAUNCH();
}
template <typename T>
void fast_cheb_fused(const Geo& g, int nsteps, const T* B, T* X, const Coef* c, const int* done, cudaStream_t s)
{
    ChebStages<T> cs;
    for (int t = 0; t < nsteps && t < 4; t++) cs.c[t] = cast_coef<T>(c[t]);
    const int ux = g.hi[0] - g.lo[0], uy = g.hi[1] - g.lo[1], uz = g.hi[2] - g.lo[2];
    const int ntx = (ux + FUSE_TX - 1) / FUSE_TX, nty = (uy + FUSE_TY - 1) / FUSE_TY;
    const long long tiles = (long long)ntx * nty;
    // z chunks: about 8 blocks per SM, each chunk at most 128 planes (the wavefront
    // re-reads 2*nsteps planes per chunk)
    long long chunks = std::max((sm_count() * 8LL + tiles - 1) / tiles, (long long)((uz + 127) / 128));
    chunks = std::max(1LL, std::min(chunks, (long long)uz));
    const int kchunk = (int)((uz + chunks - 1) / chunks);
    const dim3 grid((unsigned)tiles, (unsigned)((uz + kchunk - 1) / kchunk));
    const dim3 block(FUSE_TX, 256 / FUSE_TX);
    // the dynamic shared-memory opt-in, once per device and instantiation (a host call)
    static unsigned long long attr_set = 0;
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 64 && !(attr_set & (1ull << dev))) {
        cudaFuncSetAttribute(k_cheb_fused<T, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(sizeof(T) * FuseDims<2>::total()));
        cudaFuncSetAttribute(k_cheb_fused<T, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(sizeof(T) * FuseDims<3>::total()));
        attr_set |= 1ull << dev;
    }
    if (nsteps == 2)
        launch_pdl(k_cheb_fused<T, 2>, grid, block, sizeof(T) * FuseDims<2>::total(), s, g, ntx, kchunk, B, X, cs, done);
    else
        launch_pdl(k_cheb_fused<T, 3>, grid, block, sizeof(T) * FuseDims<3>::total(), s, g, ntx, kchunk, B, X, cs, done);
    PPS_COUNT_LAUNCH();
}
template <typename T>
void fast_scale_copy(const Geo& g, const Shape& sh, const T* B, T* X, double a, const int* done, cudaStream_t s)
{
    launch_pdl(k_scale_copy<T>, grid_of(sh), block_of(sh), 0, s, g, sh, B, X, (T)a, done);
    PPS_COUNT_LAUNCH();
}
template <typename T>
void fast_stencil_dot(const Geo& g, const Shape& sh, const T* u, const T* r0, T* Au, const Coef& a, RedCtx rc,
                      cudaStream_t s)
{
    if constexpr (std::is_same<T, double>::value) {
        if (iso_coef(a)) {   // equal spacings: the neighbour sum on the integer pipe
            Shape c = sh.cx == 1 ? sh : make_shape(g, sh.ty, (int)sh.nblocks(), 1);
            if (rc.cells) canon_launch(g, c, rc);
            launch_pdl(k_stencil_dots_iso64<1>, grid_of(c), block_of(c), 0, s, g, c, u, r0, Au, a, rc);
            PPS_COUNT_LAUNCH();
            if (rc.cells) canon_finalize<1>(rc, &rc.st->done, s);
            return;
        }
    }
    if (rc.cells) {   // canonical sums: one-column kernel on the canonical shape
        Shape c = sh;
        canon_launch(g, c, rc);
        launch_pdl(k_stencil_dot<T>, grid_of(c), block_of(c), 0, s, g, c, u, r0, Au, a, rc);
        PPS_COUNT_LAUNCH();
        canon_finalize<1>(rc, &rc.st->done, s);
        return;
    }
    if (sh.cx != 1) {   // the Chebyshev tiles: x-vectorised FP32, else the one-column tiles
        if constexpr (std::is_same<T, float>::value) {
            if (sh.cx == 4 && v4_ok<T>(g, u, r0, Au, nullptr)) {
                launch_pdl(k_stencil_dots_v4<1>, grid_of(sh), block_of(sh), 0, s, g, sh, u, r0, Au, a, rc);
                PPS_COUNT_LAUNCH();
                return;
            }
        }
        fast_stencil_dot<T>(g, make_shape(g, sh.ty, (int)sh.nblocks(), 1), u, r0, Au, a, rc, s);
        return;
    }
    launch_pdl(k_stencil_dot<T>, grid_of(sh), block_of(sh), 0, s, g, sh, u, r0, Au, a, rc);
    PPS_COUNT_LAUNCH();
}
template <typename T>
void fast_stencil_dot2(const Geo& g, const Shape& sh, const T* u, const T* r, T* Au, const Coef& a, RedCtx rc,
                       cudaStream_t s)
{
    if constexpr (std::is_same<T, double>::value) {
        if (iso_coef(a)) {   // equal spacings: the neighbour sum on the integer pipe
            Shape c = sh.cx == 1 ? sh : make_shape(g, sh.ty, (int)sh.nblocks(), 1);
            if (rc.cells) canon_launch(g, c, rc);
            launch_pdl(k_stencil_dots_iso64<2>, grid_of(c), block_of(c), 0, s, g, c, u, r, Au, a, rc);
            PPS_COUNT_LAUNCH();
            if (rc.cells) canon_finalize<2>(rc, &rc.st->done, s);
            return;
        }
    }
    if (rc.cells) {
        Shape c = sh;
        canon_launch(g, c, rc);
        launch_pdl(k_stencil_dot2<T>, grid_of(c), block_of(c), 0, s, g, c, u, r, Au, a, rc);
        PPS_COUNT_LAUNCH();
        canon_finalize<2>(rc, &rc.st->done, s);
        return;
    }
    if (sh.cx != 1) {
        if constexpr (std::is_same<T, float>::value) {
            if (sh.cx == 4 && v4_ok<T>(g, u, r, Au, nullptr)) {
                launch_pdl(k_stencil_dots_v4<2>, grid_of(sh), block_of(sh), 0, s, g, sh, u, r, Au, a, rc);
                PPS_COUNT_LAUNCH();
                return;
            }
        }
        fast_stencil_dot2<T>(g, make_shape(g, sh.ty, (int)sh.nblocks(), 1), u, r, Au, a, rc, s);
        return;
    }
    launch_pdl(k_stencil_dot2<T>, grid_of(sh), block_of(sh), 0, s, g, sh, u, r, Au, a, rc);
    PPS_COUNT_LAUNCH();
}
// Dirichlet grids with 16-byte aligned fields: the flat vector forms of the updates.
static bool flat_ok(const Geo& g, std::initializer_list<const void*> ptrs)
{
    for (int f = 0; f < 6; f++)
        if (g.bcs[f] != 0) return false;
    for (const void* p : ptrs)
        if (((uintptr_t)p & 15u) != 0) return false;
    return true;
}
template <typename T>
void fast_axpy_alpha(const Geo& g, const Shape& sh, T* r, const T* v, const DevState* st, cudaStream_t s)
{
    if (flat_ok(g, {r, v})) {
        launch_pdl(k_axpy_alpha_flat<T>, sh.nblocks(), 32 * sh.ty, 0, s, g.ntot, r, v, st);
        PPS_COUNT_LAUNCH();
        return;
    }
    launch_pdl(k_axpy_alpha<T>, grid_of(sh), block_of(sh), 0, s, g, sh, r, v, st);
    PPS_COUNT_LAUNCH();
}
template <typename T>
void fast_update_xr(const Geo& g, const Shape& sh, T* x, const T* Mp, const T* z, T* r, const T* Az, const T* r0,
                    RedCtx rc, cudaStream_t s)
{
    if (rc.cells) {
        Shape c = sh;
        canon_launch(g, c, rc);
        launch_pdl(k_update_xr<T>, grid_of(c), block_of(c), 0, s, g, c, x, Mp, z, r, Az, r0, rc);
        PPS_COUNT_LAUNCH();
        canon_finalize<2>(rc, &rc.st->done, s);
        return;
    }
    if (flat_ok(g, {x, Mp, z, r, Az, r0})) {
        launch_pdl(k_update_xr_flat<T>, sh.nblocks(), 32 * sh.ty, 0, s, g.ntot, x, Mp, z, r, Az, r0, rc);
        PPS_COUNT_LAUNCH();
        return;
    }
    launch_pdl(k_update_xr<T>, grid_of(sh), block_of(sh), 0, s, g, sh, x, Mp, z, r, Az, r0, rc);
    PPS_COUNT_LAUNCH();
}
template <typename T>
void fast_update_p(const Geo& g, const Shape& sh, T* p, const T* r, const T* AMp, const DevState* st, cudaStream_t s)
{
    if (flat_ok(g, {p, r, AMp})) {
        launch_pdl(k_update_p_flat<T>, sh.nblocks(), 32 * sh.ty, 0, s, g.ntot, p, r, AMp, st);
        PPS_COUNT_LAUNCH();
        return;
    }
    launch_pdl(k_update_p<T>, grid_of(sh), block_of(sh), 0, s, g, sh, p, r, AMp, st);
    PPS_COUNT_LAUNCH();
}
template <typename T>
void fast_cg_stencil_dot(const Geo& g, const Shape& sh, const T* p, const T* r, const T* z, T* Ap, const Coef& a,
                         RedCtx rc, cudaStream_t s)
{
    if (rc.cells) {
        Shape c = sh;
        canon_launch(g, c, rc);
        launch_pdl(k_cg_stencil_dot<T>, grid_of(c), block_of(c), 0, s, g, c, p, r, z, Ap, a, rc);
        PPS_COUNT_LAUNCH();
        canon_finalize<2>(rc, &rc.st->done, s);
        return;
    }
    launch_pdl(k_cg_stencil_dot<T>, grid_of(sh), block_of(sh), 0, s, g, sh, p, r, z, Ap, a, rc);
    PPS_COUNT_LAUNCH();
}
template <typename T>
void fast_cg_update_xr(const Geo& g, const Shape& sh, T* x, const T* p, T* r, const T* Ap, const DevState* st,
                       cudaStream_t s)
{
    launch_pdl(k_cg_update_xr<T>, grid_of(sh), block_of(sh), 0, s, g, sh, x, p, r, Ap, st);
    PPS_COUNT_LAUNCH();
}
template <typename T>
void fast_cg_dot_rz(const Geo& g, const Shape& sh, const T* r, const T* z, RedCtx rc, cudaStream_t s)
{
    if (rc.cells) {
        Shape c = sh;
        canon_launch(g, c, rc);
        launch_pdl(k_cg_dot_rz<T>, grid_of(c), block_of(c), 0, s, g, c, r, z, rc);
        PPS_COUNT_LAUNCH();
        canon_finalize<2>(rc, &rc.st->done, s);
        return;
    }
    launch_pdl(k_cg_dot_rz<T>, grid_of(sh), block_of(sh), 0, s, g, sh, r, z, rc);
    PPS_COUNT_LAUNCH();
}
template <typename T>
void fast_cg_update_p(const Geo& g, const Shape& sh, T* p, const T* z, const DevState* st, cudaStream_t s)
{
    launch_pdl(k_cg_update_p<T>, grid_of(sh), block_of(sh), 0, s, g, sh, p, z, st);
    PPS_COUNT_LAUNCH();
}
template <typename T>
void fast_fcg_update_xr(const Geo& g, const Shape& sh, T* x, const T* p, T* r, const T* Ap, RedCtx rc,
                        cudaStream_t s)
{
    launch_pdl(k_fcg_update_xr<T>, grid_of(sh), block_of(sh), 0, s, g, sh, x, p, r, Ap, rc);
    PPS_COUNT_LAUNCH();
}
template <typename T>
void fast_fcg_dot(const Geo& g, const Shape& sh, const T* r, const T* z, const T* Ap, RedCtx rc, cudaStream_t s)
{
    launch_pdl(k_fcg_dot<T>, grid_of(sh), block_of(sh), 0, s, g, sh, r, z, Ap, rc);
    PPS_COUNT_LAUNCH();
}
template <typename T>
void fast_fcg_update_xr_flat(const Geo& g, const Shape& sh, T* x, const T* p, T* r, const T* Ap, RedCtx rc,
                             cudaStream_t s)
{
    launch_pdl(k_fcg_update_xr_flat<T>, sh.nblocks(), 32 * sh.ty, 0, s, g.ntot, x, p, r, Ap, rc);
    PPS_COUNT_LAUNCH();
}
template <typename T>
void fast_fcg_dot_flat(const Geo& g, const Shape& sh, const T* r, const T* z, const T* Ap, RedCtx rc, cudaStream_t s)
{
    launch_pdl(k_fcg_dot_flat<T>, sh.nblocks(), 32 * sh.ty, 0, s, g.ntot, r, z, Ap, rc);
    PPS_COUNT_LAUNCH();
}
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// the driver's tensor-map encoder, fetched through the runtime (no link to the driver library)
static EncodeTiledFn encode_tiled()
{
    static const EncodeTiledFn fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            return (EncodeTiledFn) nullptr;
        }
        return (EncodeTiledFn)p;
    }();
    return fn;
}

// A tiled map over a padded FP32 field (x, y, z = row, plane, field extents) whose
// boxes are STAGE_ROW x rows x 1; parts of a box outside the field read as zeros.
// False where the encoder is missing or refuses (the caller then takes another kernel).
static bool field_map(CUtensorMap* m, const float* base, const Geo& g, int rows)
{
    const EncodeTiledFn fn = encode_tiled();
    if (!fn || ((uintptr_t)base & 15u) != 0 || g.sj % 4 != 0 || rows > 256) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)g.sj, (cuuint64_t)(g.sk / g.sj), (cuuint64_t)(g.ntot / g.sk)};
    const cuuint64_t strides[2] = {(cuuint64_t)g.sj * 4u, (cuuint64_t)g.sk * 4u};
    const cuuint32_t boxd[3] = {(cuuint32_t)STAGE_ROW, (cuuint32_t)rows, 1u};
    const cuuint32_t es[3] = {1u, 1u, 1u};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(base), dims, strides, boxd, es,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <typename T>
void fast_fcg_p_stencil(const Geo& g, const Shape& sh, const T* z, const T* pin, T* pout, T* Ap, const Coef& a,
                        RedCtx rc, cudaStream_t s, bool staged)
{
    if (sh.cx != 1) {   // the Chebyshev tiles: x-vectorised FP32, else the one-column tiles
        if constexpr (std::is_same<T, float>::value) {
            if (sh.cx == 4 && v4_ok<T>(g, z, pin, pout, Ap)) {
                CUtensorMap mz, mp;
                if (staged && field_map(&mz, z, g, sh.ty + 2) && field_map(&mp, pin, g, sh.ty + 2)) {
                    const size_t smem = stage_smem_bytes(sh.ty);
                    static int attr_set = 0;   // bytes the attribute allows
                    if (smem > 48 * 1024 && attr_set < (int)smem) {
                        cudaFuncSetAttribute(k_fcg_p_stencil_staged, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
                        attr_set = (int)smem;
                    }
                    launch_pdl(k_fcg_p_stencil_staged, grid_of(sh), block_of(sh), smem, s, g, sh, mz, mp, pout, Ap,
                               a, rc);
                } else {
                    launch_pdl(k_fcg_p_stencil_v4, grid_of(sh), block_of(sh), 0, s, g, sh, z, pin, pout, Ap, a, rc);
                }
                PPS_COUNT_LAUNCH();
                return;
            }
        }
        fast_fcg_p_stencil<T>(g, make_shape(g, sh.ty, (int)sh.nblocks(), 1), z, pin, pout, Ap, a, rc, s, staged);
        return;
    }
    launch_pdl(k_fcg_p_stencil<T>, grid_of(sh), block_of(sh), 0, s, g, sh, z, pin, pout, Ap, a, rc);
    PPS_COUNT_LAUNCH();
}
void flag_nonzero(long long n, const double* x, int* flag, cudaStream_t s)
{
    launch_pdl(k_flag_nonzero, sm_count() * 4, 256, 0, s, n, x, flag);
    PPS_COUNT_LAUNCH();
}
void fast_count_nonzero(const Geo& g, const Shape& sh, const double* x, RedCtx rc, cudaStream_t s)
{
    launch_pdl(k_count_nonzero, sh.nblocks(), 32 * sh.ty, 0, s, g.ntot, x, rc);
    PPS_COUNT_LAUNCH();
}
template <typename TR>
void fast_residual(const Geo& g, const Shape& sh, const double* x, const double* b, TR* r, TR* r0, TR* p,
                   const Coef& a, RedCtx rc, cudaStream_t s, bool x_zero)
{
    Shape c = sh;
    if (rc.cells) canon_launch(g, c, rc);
    if (x_zero)
        launch_pdl(k_residual<TR, true, true>, grid_of(c), block_of(c), 0, s, g, c, x, b, r, r0, p, a, rc);
    else if (a.cx == a.cy && a.cx == a.cz)
        launch_pdl(k_residual<TR, true, false>, grid_of(c), block_of(c), 0, s, g, c, x, b, r, r0, p, a, rc);
    else
        launch_pdl(k_residual<TR, false, false>, grid_of(c), block_of(c), 0, s, g, c, x, b, r, r0, p, a, rc);
    PPS_COUNT_LAUNCH();
    if (rc.cells) canon_finalize<1>(rc, nullptr, s);
}
void fast_norm_badj(const Geo& g, const Shape& sh, const double* b, const double* x, Faces f, RedCtx rc,
                    cudaStream_t s, bool x_zero)
{
    Shape c = sh;
    if (rc.cells) canon_launch(g, c, rc);
    if (x_zero) launch_pdl(k_norm_badj<true>, grid_of(c), block_of(c), 0, s, g, c, b, x, f, rc);
    else launch_pdl(k_norm_badj<false>, grid_of(c), block_of(c), 0, s, g, c, b, x, f, rc);
    PPS_COUNT_LAUNCH();
    if (rc.cells) canon_finalize<1>(rc, nullptr, s);
}
void fast_add_correction(const Geo& g, const Shape& sh, double* x, const float* e, const DevState*, cudaStream_t s,
                         bool e_zero_off)
{
    if (e_zero_off && flat_ok(g, {x}) && ((uintptr_t)e & 7u) == 0) {
        launch_pdl(k_add_correction_flat, sh.nblocks(), 32 * sh.ty, 0, s, g.ntot, x, e);
    } else {
        launch_pdl(k_add_correction, grid_of(sh), block_of(sh), 0, s, g, sh, x, e);
    }
    PPS_COUNT_LAUNCH();
}
template <typename T>
void fast_bicg_start(const Geo& g, const Shape& sh, const T* B, T* r, T* r0, T* p, RedCtx rc, cudaStream_t s)
{
    Shape c = sh;
    if (rc.cells) canon_launch(g, c, rc);
    launch_pdl(k_bicg_start<T>, grid_of(c), block_of(c), 0, s, g, c, B, r, r0, p, rc);
    PPS_COUNT_LAUNCH();
    if (rc.cells) canon_finalize<1>(rc, &rc.st->done, s);
}
void cast_field_f32(const double* in, float* out, long long n, cudaStream_t s)
{
    const long long blocks = std::min<long long>((n + 255) / 256, sm_count() * 16LL);
    launch_pdl(k_cast_f32, (unsigned)std::max<long long>(blocks, 1), 256, 0, s, in, out, n);
    PPS_COUNT_LAUNCH();
}
template <typename T>
void fill_field(T* p, long long n, T v, cudaStream_t s)
{
    launch_pdl(k_fill<T>, par_blocks(n), 256, 0, s, p, n, v);
    PPS_COUNT_LAUNCH();
}
template <typename T>
void zero_off_unknowns(const Geo& g, T* p, cudaStream_t s)
{
    launch_pdl(k_zero_off_unknowns<T>, par_blocks(g.ntot), 256, 0, s, g, p);
    PPS_COUNT_LAUNCH();
}
// The Krylov scalars to their page-locked host copy, stored by one warp through the
// mapping of that memory: a host poll that needs no copy engine, so it never queues
// behind a bulk copy of a field that another stream has in flight.
__global__ void __launch_bounds__(32) k_state_out(const DevState* __restrict__ d, DevState* __restrict__ h)
{
    pdl_enter();
    constexpr int n = (int)(sizeof(DevState) / sizeof(unsigned long long));
    const unsigned long long* src = reinterpret_cast<const unsigned long long*>(d);
    unsigned long long* dst = reinterpret_cast<unsigned long long*>(h);
    for (int i = threadIdx.x; i < n; i += 32) dst[i] = src[i];
}

void state_out(const DevState* d, DevState* h_mapped, cudaStream_t s)
{
    static_assert(sizeof(DevState) % sizeof(unsigned long long) == 0, "DevState is copied in 8-byte words");
    launch_pdl(k_state_out, 1, 32, 0, s, d, h_mapped);
    PPS_COUNT_LAUNCH();
}

void state_init(DevState* st, double* hist, int maxit, double tol_abs, double tol_rel, int tol_relative,
                int rho0_from_r, double hist_scale, int hist_cap, cudaStream_t s)
{
    launch_pdl(k_state_init, 1, 32, 0, s, st, hist, maxit, tol_abs, tol_rel, tol_relative, rho0_from_r, hist_scale, hist_cap);
    PPS_COUNT_LAUNCH();
}

#include "pps_batch_kernels.cuh"

#define PPS_INST(T)                                                                                              \
    template void fast_cheb_s01<T>(const Geo&, const Shape&, const T*, T*, const Coef&, const int*,               \
                                   cudaStream_t);                                                                \
    template void fast_cheb_sweep<T>(const Geo&, const Shape&, const T*, const T*, const T*, T*, const Coef&,    \
                                     const int*, cudaStream_t);                                                  \
    template void fast_scale_copy<T>(const Geo&, const Shape&, const T*, T*, double, const int*, cudaStream_t); \
    template void fast_stencil_dot<T>(const Geo&, const Shape&, const T*, const T*, T*, const Coef&, RedCtx,     \
                                      cudaStream_t);                                                             \
    template void fast_stencil_dot2<T>(const Geo&, const Shape&, const T*, const T*, T*, const Coef&, RedCtx,    \
                                       cudaStream_t);                                                            \
    template void fast_axpy_alpha<T>(const Geo&, const Shape&, T*, const T*, const DevState*, cudaStream_t);     \
    template void fast_update_xr<T>(const Geo&, const Shape&, T*, const T*, const T*, T*, const T*, const T*,    \
                                    RedCtx, cudaStream_t);                                                       \
    template void fast_update_p<T>(const Geo&, const Shape&, T*, const T*, const T*, const DevState*,            \
                                   cudaStream_t);                                                                \
    template void fast_cg_stencil_dot<T>(const Geo&, const Shape&, const T*, const T*, const T*, T*,             \
                                         const Coef&, RedCtx, cudaStream_t);                                     \
    template void fast_cg_update_xr<T>(const Geo&, const Shape&, T*, const T*, T*, const T*, const DevState*,    \
                                       cudaStream_t);                                                            \
    template void fast_cg_dot_rz<T>(const Geo&, const Shape&, const T*, const T*, RedCtx, cudaStream_t);         \
    template void fast_cg_update_p<T>(const Geo&, const Shape&, T*, const T*, const DevState*, cudaStream_t);    \
    template void fast_fcg_update_xr<T>(const Geo&, const Shape&, T*, const T*, T*, const T*, RedCtx,            \
                                        cudaStream_t);                                                           \
    template void fast_fcg_dot<T>(const Geo&, const Shape&, const T*, const T*, const T*, RedCtx, cudaStream_t); \
    template void fast_fcg_p_stencil<T>(const Geo&, const Shape&, const T*, const T*, T*, T*, const Coef&,       \
                                        RedCtx, cudaStream_t, bool);                                             \
    template void fast_cheb_fused<T>(const Geo&, int, const T*, T*, const Coef*, const int*, cudaStream_t);      \
    template void fast_fcg_update_xr_flat<T>(const Geo&, const Shape&, T*, const T*, T*, const T*, RedCtx,       \
                                             cudaStream_t);                                                      \
    template void fast_fcg_dot_flat<T>(const Geo&, const Shape&, const T*, const T*, const T*, RedCtx,          \
                                       cudaStream_t);                                                            \
    template void fast_residual<T>(const Geo&, const Shape&, const double*, const double*, T*, T*, T*,           \
                                   const Coef&, RedCtx, cudaStream_t, bool);                                     \
    template void fill_field<T>(T*, long long, T, cudaStream_t);                                                  \
    template void zero_off_unknowns<T>(const Geo&, T*, cudaStream_t);                                             \
    template void fast_bicg_start<T>(const Geo&, const Shape&, const T*, T*, T*, T*, RedCtx, cudaStream_t);

PPS_INST(double)
PPS_INST(float)

}  // namespace pps
