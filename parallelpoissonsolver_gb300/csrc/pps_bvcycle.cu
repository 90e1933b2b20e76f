// Batched solves in ONE persistent launch: flexible CG with a multigrid V-cycle per
// problem, FP32 inner iterations inside FP64 iterative refinement.
//
// No reference counterpart (the reference solves one grid per run).  The batch's
// problems are cubes of uneven size (Dirichlet walls, equal spacings).  One
// cooperative kernel (every block resident) runs the whole solve: a fixed program of
// phases per round, all problems advancing together, each phase spread over every
// block as (problem, tile) work items, phases separated by a grid barrier whose wait
// is bounded in time (a wait that runs out sets an error flag, every block returns,
// and the solve reports PPS_TIMEOUT).  The launch, with the state reset before it, is
// captured once as a CUDA graph and replayed.
//
// A round for one problem is either an FCG iteration or a refinement step:
//   A  FCG: p = z + beta p_old, Ap = A p, sum p.Ap -> alpha   | refine: x += e, e = 0
//   B  FCG: e += alpha p, r -= alpha Ap, sum r.r -> stop test | refine: r = b - A x
//      in FP64, ||r|| -> outer stop test, inner target
//   V-cycle z = M r (skipped once the inner solve has converged):
//      level 0: Chebyshev(5) on [lmax/8, lmax]; residual; full-weighting restriction
//      levels 1..k-1: Jacobi-scaled Chebyshev(4) on [2/8, 2] of D^-1 A_l, residual,
//      restriction; level k (at most 32 unknowns per axis): exact inverse by a
//      tensor-product eigen-solve; back up: trilinear prolongation, residual,
//      Jacobi-scaled Chebyshev(4) post-smoothing; level 0: z += P z_1
//   P0 sums z.r, z.Ap -> beta (Polak-Ribiere, -alpha z.Ap / rho), rho = z.r
// The coarse operators are the learned V-cycle's (level l: spacing 2^l h, the upper
// wall one fine spacing above the last unknown).  Reductions are per problem and
// deterministic: one partial per work item, summed in item order by the problem's
// last item, which then advances that problem's scalars.
#include "../../include/pps.h"
#include "pps_internal.h"
#include "pps_reduce.cuh"
#include "pps_unet_internal.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <string>
#include <vector>

namespace pps {
namespace bvc {

constexpr int MAXLEV = 6;          // levels 0..5
constexpr int NT = 256;            // threads per block: 32 x 8 columns of a tile
constexpr int EX_MAX = 32;         // coarsest level: at most 32 unknowns per axis
constexpr double RATIO = 8.0;      // smoothing interval [lmax/RATIO, lmax]

struct Prob {
    int m, k;                      // unknowns per axis on level 0; coarsest level
    long long off;                 // pooled offset of the level-0 guard-padded fields
    long long coff[MAXLEV];        // pooled offset of level l >= 1 (dense n_l^3)
    int n[MAXLEV];                 // unknowns per axis on level l
    int kz[MAXLEV];                // planes per work item on level l
    int ntx[MAXLEV], nty[MAXLEV], nch[MAXLEV];
    double ih2;                    // 1/h^2 (FP64 residual)
    float fcc[3], fcn[3], fcb[3], fcz[3];   // fine Chebyshev steps: W = cc Y + cn sum(Y nbrs) + cb B + cz Z
    float lih2[MAXLEV], lastm[MAXLEV], lastc[MAXLEV];   // level operators (l >= 1)
    long long mats;                // offset of the coarsest level's eigen-solve matrices
};

struct State {
    double normb, tol_outer, err_outer, target, err;
    double rho, alpha, beta;
    int mode;                      // 0: refinement step next, 1: FCG iteration
    int done, status, skip, par;
    int inner_it, total_it, refinements;
};

struct Barrier {
    unsigned count, gen;
    int error, pad;
};

enum : int { PH_NORM = 0, PH_A, PH_B, PH_C1, PH_C2, PH_C3, PH_R0, PH_RS, PH_D1, PH_D2, PH_DR, PH_EX, PH_UP, PH_UR,
             PH_U1, PH_U2, PH_P0 };

struct Phase {
    int type, level;
};

struct Dev {
    const Prob* prob;
    int nprob;
    const long long* toff;         // toff[l * (nprob + 1) + q]: first work item of problem q on level l
    const Phase* phases;
    int nphases;
    State* st;
    double* x;
    const double* b;
    float *r, *z, *pa, *pb, *ap, *e, *y1, *y2, *t0;   // level 0 (guard-padded)
    float *cr, *cz, *ct, *cc1;                        // levels >= 1 (dense)
    const float* mats;
    double* partials;
    unsigned* counters;
    Barrier* bar;
    int* unfinished;
    double tol, inner_tol;
    int inner_maxit, max_refinements, max_rounds;
    float jt, ja1, jb1, ja2, jb2, jc2;   // coarse Jacobi-Chebyshev constants (ph_jcheb)
    unsigned long long limit_ns;
};

__device__ __forceinline__ unsigned long long now_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Grid barrier of the resident blocks.  Thread 0 of each block reads the generation,
// arrives on the counter, and waits for the generation to change; the last block to
// arrive resets the counter and advances the generation.  The wait gives up after
// limit_ns (or as soon as another block gave up): it then sets the error flag and
// every block returns.  Returns false after an error.
__device__ bool grid_barrier(const Dev& D)
{
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned* gen = &D.bar->gen;
        volatile int* err = &D.bar->error;
        const unsigned g = *gen;
        __threadfence();
        if (atomicAdd(&D.bar->count, 1u) == gridDim.x - 1) {
            D.bar->count = 0u;
            __threadfence();
            atomicAdd(&D.bar->gen, 1u);
        } else {
            const unsigned long long t0 = now_ns();
            while (*gen == g) {
                if (*err != 0 || now_ns() - t0 > D.limit_ns) {
                    atomicExch(&D.bar->error, 1);
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
        ok = (*err == 0);
    }
    __syncthreads();
    return ok != 0;
}

// ---- work items ----

struct Item {
    int q;
    int i, j, k0, k1;              // this thread's column (0-based unknown indices) and planes
    bool on;                       // the column lies inside the level
    long long item;                // item index within the phase
};

__device__ __forceinline__ int find_problem(const long long* row, int nprob, long long item)
{
    int lo = 0, hi = nprob - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (row[mid] <= item) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ Item decode(const Dev& D, int lev, long long item)
{
    Item it;
    const long long* row = D.toff + (long long)lev * (D.nprob + 1);
    it.q = find_problem(row, D.nprob, item);
    it.item = item;
    const Prob& P = D.prob[it.q];
    const long long t = item - row[it.q];
    const int ntx = P.ntx[lev], nty = P.nty[lev];
    const int bx = (int)(t % ntx), by = (int)((t / ntx) % nty), ch = (int)(t / ((long long)ntx * nty));
    const int n = P.n[lev];
    it.i = bx * 32 + (int)(threadIdx.x & 31);
    it.j = by * 8 + (int)(threadIdx.x >> 5);
    it.k0 = ch * P.kz[lev];
    it.k1 = min(it.k0 + P.kz[lev], n);
    it.on = it.i < n && it.j < n;
    return it;
}

// Block sum of NS partials in a fixed order (warp trees, then the eight warps in
// order), stored as this item's partial; the problem's last item sums its items'
// partials in item order (thread t the ones at t + 256 m, then the same block tree)
// and returns true to thread 0 with the totals.
template <int NS>
__device__ bool item_reduce(const Dev& D, const Item& it, long long first, long long count, double (&v)[NS],
                            double (&tot)[2])
{
    __shared__ double sm[8][2];
    __shared__ int last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int s = 0; s < NS; s++) {
        const double w = warp_sum(v[s]);
        if (lane == 0) sm[warp][s] = w;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int s = 0; s < NS; s++) {
            double t = 0.0;
            for (int w = 0; w < 8; w++) t += sm[w][s];
            D.partials[it.item * 2 + s] = t;
        }
        __threadfence();
        last = atomicAdd(&D.counters[it.q], 1u) == (unsigned)(count - 1);
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double acc[NS];
#pragma unroll
    for (int s = 0; s < NS; s++) acc[s] = 0.0;
    for (long long c = first + threadIdx.x; c < first + count; c += NT) {
#pragma unroll
        for (int s = 0; s < NS; s++) acc[s] += __ldcg(&D.partials[c * 2 + s]);
    }
    __syncthreads();
#pragma unroll
    for (int s = 0; s < NS; s++) {
        const double w = warp_sum(acc[s]);
        if (lane == 0) sm[warp][s] = w;
    }
    __syncthreads();
    bool mine = false;
    if (threadIdx.x == 0) {
        tot[0] = tot[1] = 0.0;
#pragma unroll
        for (int s = 0; s < NS; s++) {
            double t = 0.0;
            for (int w = 0; w < 8; w++) t += sm[w][s];
            tot[s] = t;
        }
        D.counters[it.q] = 0u;
        mine = true;
    }
    __syncthreads();
    return mine;
}

__device__ void finish(const Dev& D, State& S, int status)
{
    S.done = 1;
    S.status = status;
    atomicSub(D.unfinished, 1);
}

// The problem's scalars after a reduction phase (thread 0 of its last item).
__device__ void advance(const Dev& D, int q, int type, const double (&tot)[2])
{
    State& S = D.st[q];
    switch (type) {
    case PH_NORM:
        S.normb = sqrt(tot[0]);
        S.tol_outer = D.tol * S.normb;
        S.mode = 0;
        S.skip = 0;
        if (!(S.normb > 0.0)) finish(D, S, PPS_ERR_ZERO_RHS);
        else if (!isfinite(S.normb)) finish(D, S, PPS_NAN_DETECTED);
        break;
    case PH_A:   // FCG: alpha = rho / p.Ap; the new direction becomes p_old
        S.alpha = S.rho / tot[0];
        S.par ^= 1;
        if (!isfinite(S.alpha)) finish(D, S, PPS_BREAKDOWN);
        break;
    case PH_B:
        if (S.mode == 1) {   // FCG: recursive residual norm, inner stop test
            S.err = sqrt(tot[0]);
            S.inner_it++;
            S.total_it++;
            if (!isfinite(S.err)) {
                finish(D, S, PPS_NAN_DETECTED);
            } else if (S.err < S.target || S.inner_it >= D.inner_maxit) {
                S.skip = 1;    // converged inner solve: no V-cycle; a refinement step next
                S.mode = 0;
            }
        } else {             // refinement: FP64 true residual, outer stop test
            S.err_outer = sqrt(tot[0]);
            if (!isfinite(S.err_outer)) {
                finish(D, S, PPS_NAN_DETECTED);
            } else if (S.err_outer <= S.tol_outer) {
                finish(D, S, PPS_OK);
            } else if (S.refinements >= D.max_refinements) {
                finish(D, S, PPS_NOT_CONVERGED);
            } else {
                S.refinements++;
                S.target = fmax(D.inner_tol, 0.3 * S.tol_outer / S.err_outer) * S.err_outer;
                S.inner_it = 0;
                S.skip = 0;
            }
        }
        break;
    case PH_P0:
        if (S.mode == 0) {   // after a refinement step: the FCG recurrence (re)starts
            S.rho = tot[0];
            S.beta = 0.0;
            S.mode = 1;
        } else {             // Polak-Ribiere: beta = z_new.(r_new - r_old) / rho, r_new - r_old = -alpha Ap
            S.beta = -S.alpha * tot[1] / S.rho;
            S.rho = tot[0];
        }
        if (!isfinite(S.beta) || !isfinite(S.rho)) finish(D, S, PPS_BREAKDOWN);
        break;
    default:
        break;
    }
}

// ---- level 0: guard-padded fields, one column per thread ----

__device__ __forceinline__ long long idx0(const Prob& P, int i, int j, int k)
{
    const long long sj = P.m + 4, sk = sj * sj;
    return P.off + (i + 2) + sj * (j + 2) + sk * (k + 2);
}

// sum of the six neighbours of c (guard and boundary cells of the work fields are 0)
__device__ __forceinline__ float nsum(const float* f, long long c, long long sj, long long sk)
{
    return ((f[c - 1] + f[c + 1]) + (f[c - sj] + f[c + sj])) + (f[c - sk] + f[c + sk]);
}

// ---- levels >= 1: dense n^3, the upper wall one fine spacing above the last unknown ----

__device__ __forceinline__ float lvl_apply(const float* u, long long base, int n, int i, int j, int k, float ih2,
                                           float lm, float lc, float uc)
{
    const long long sj = n, sk = (long long)n * n;
    const long long c = base + i + sj * j + sk * k;
    float a = 0.f;
    const int t[3] = {i, j, k};
    const long long s[3] = {1, sj, sk};
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const float um = t[d] > 0 ? u[c - s[d]] : 0.f;
        if (t[d] < n - 1) a += ih2 * ((um + u[c + s[d]]) - 2.f * uc);
        else a += lm * um + lc * uc;
    }
    return a;
}

__device__ __forceinline__ float lvl_dinv(int n, int i, int j, int k, float ih2, float lc)
{
    float d = 0.f;
    d += i < n - 1 ? 2.f * ih2 : -lc;
    d += j < n - 1 ? 2.f * ih2 : -lc;
    d += k < n - 1 ? 2.f * ih2 : -lc;
    return 1.f / d;
}

// ---- phase bodies ----

// ||b_adj||^2: b minus the Dirichlet nodes' contributions (x on the boundary nodes)
__device__ void ph_norm(const Dev& D, const Item& it, double& acc)
{
    const Prob& P = D.prob[it.q];
    if (!it.on) return;
    const long long sj = P.m + 4, sk = sj * sj;
    const int m = P.m;
    for (int k = it.k0; k < it.k1; k++) {
        const long long c = idx0(P, it.i, it.j, k);
        double bd = 0.0;
        if (it.i == 0) bd += D.x[c - 1];
        if (it.i == m - 1) bd += D.x[c + 1];
        if (it.j == 0) bd += D.x[c - sj];
        if (it.j == m - 1) bd += D.x[c + sj];
        if (k == 0) bd += D.x[c - sk];
        if (k == m - 1) bd += D.x[c + sk];
        const double v = D.b[c] - bd * P.ih2;
        acc = fma(v, v, acc);
    }
}

// FCG direction: p_out = z + beta p_in at the point and its six neighbours (so p_in
// and p_out are distinct fields), Ap = A p_out, sum p_out.Ap
__device__ void ph_a_fcg(const Dev& D, const Item& it, Acc<float>& acc)
{
    const Prob& P = D.prob[it.q];
    const State& S = D.st[it.q];
    if (!it.on) return;
    const long long sj = P.m + 4, sk = sj * sj;
    const float* pin = S.par ? D.pb : D.pa;
    float* pout = S.par ? D.pa : D.pb;
    const float be = (float)S.beta, ih2 = (float)P.ih2;
    // z and p_in of the planes below and above are carried along the march; the sums
    // keep nsum's operand order
    long long c = idx0(P, it.i, it.j, it.k0);
    float zm = D.z[c - sk], zc = D.z[c], qm = 0.f, qc = 0.f;
    if (be != 0.f) {
        qm = pin[c - sk];
        qc = pin[c];
    }
    for (int k = it.k0; k < it.k1; k++, c += sk) {
        const float zp = D.z[c + sk];
        const float zs = ((D.z[c - 1] + D.z[c + 1]) + (D.z[c - sj] + D.z[c + sj])) + (zm + zp);
        float pc, ps, qp = 0.f;
        if (be == 0.f) {
            pc = zc;
            ps = zs;
        } else {
            qp = pin[c + sk];
            pc = fmaf(be, qc, zc);
            ps = fmaf(be, ((pin[c - 1] + pin[c + 1]) + (pin[c - sj] + pin[c + sj])) + (qm + qp), zs);
        }
        const float a = (ps - 6.f * pc) * ih2;
        pout[c] = pc;
        D.ap[c] = a;
        acc.add(pc, a);
        zm = zc;
        zc = zp;
        qm = qc;
        qc = qp;
    }
}

__device__ void ph_a_refine(const Dev& D, const Item& it)
{
    const Prob& P = D.prob[it.q];
    if (!it.on) return;
    for (int k = it.k0; k < it.k1; k++) {
        const long long c = idx0(P, it.i, it.j, k);
        const float ev = D.e[c];
        if (ev != 0.f) D.x[c] += (double)ev;
        D.e[c] = 0.f;
    }
}

__device__ void ph_b_fcg(const Dev& D, const Item& it, Acc<float>& acc)
{
    const Prob& P = D.prob[it.q];
    const State& S = D.st[it.q];
    if (!it.on) return;
    const float* p = S.par ? D.pb : D.pa;   // the direction phase A wrote (its parity flipped since)
    const float al = (float)S.alpha;
    for (int k = it.k0; k < it.k1; k++) {
        const long long c = idx0(P, it.i, it.j, k);
        D.e[c] = fmaf(al, p[c], D.e[c]);
        const float rn = fmaf(-al, D.ap[c], D.r[c]);
        D.r[c] = rn;
        acc.add(rn, rn);
    }
}

// refinement residual r = b - A x in FP64, stored in FP32; sum of its FP64 squares
__device__ void ph_b_refine(const Dev& D, const Item& it, double& acc)
{
    const Prob& P = D.prob[it.q];
    if (!it.on) return;
    const long long sj = P.m + 4, sk = sj * sj;
    const double* x = D.x;
    long long c = idx0(P, it.i, it.j, it.k0);
    double xm = x[c - sk], xc = x[c];   // the planes below and above carried along the march
    for (int k = it.k0; k < it.k1; k++, c += sk) {
        const double xp = x[c + sk];
        const double s6 = ((x[c - 1] + x[c + 1]) + (x[c - sj] + x[c + sj])) + (xm + xp);
        const double rv = D.b[c] - (s6 - 6.0 * xc) * P.ih2;
        D.r[c] = (float)rv;
        acc = fma(rv, rv, acc);
        xm = xc;
        xc = xp;
    }
}

// fine Chebyshev step t: W = cc Y + cn sum(Y nbrs) + cb B + cz Z
// (t = 0: Y = r -> y1; t = 1: Y = y1 -> y2; t = 2: Y = y2, Z = y1 -> z)
__device__ void ph_cheb0(const Dev& D, const Item& it, int t)
{
    const Prob& P = D.prob[it.q];
    if (!it.on) return;
    const long long sj = P.m + 4, sk = sj * sj;
    const float* Y = t == 0 ? D.r : (t == 1 ? D.y1 : D.y2);
    float* W = t == 0 ? D.y1 : (t == 1 ? D.y2 : D.z);
    const float cc = P.fcc[t], cn = P.fcn[t], cb = P.fcb[t], cz = P.fcz[t];
    long long c = idx0(P, it.i, it.j, it.k0);
    float ym = Y[c - sk], yc = Y[c];   // the planes below and above carried along the march
    for (int k = it.k0; k < it.k1; k++, c += sk) {
        const float yp = Y[c + sk];
        float w = fmaf(cn, ((Y[c - 1] + Y[c + 1]) + (Y[c - sj] + Y[c + sj])) + (ym + yp), cc * yc);
        if (t > 0) w = fmaf(cb, D.r[c], w);
        if (t == 2) w = fmaf(cz, D.y1[c], w);
        W[c] = w;
        ym = yc;
        yc = yp;
    }
}

// fine residual t0 = r - A z
__device__ void ph_r0(const Dev& D, const Item& it)
{
    const Prob& P = D.prob[it.q];
    if (!it.on) return;
    const long long sj = P.m + 4, sk = sj * sj;
    const float ih2 = (float)P.ih2;
    long long c = idx0(P, it.i, it.j, it.k0);
    float zm = D.z[c - sk], zc = D.z[c];   // the planes below and above carried along the march
    for (int k = it.k0; k < it.k1; k++, c += sk) {
        const float zp = D.z[c + sk];
        D.t0[c] = D.r[c] - ((((D.z[c - 1] + D.z[c + 1]) + (D.z[c - sj] + D.z[c + sj])) + (zm + zp)) - 6.f * zc) * ih2;
        zm = zc;
        zc = zp;
    }
}

// full-weighting restriction onto level lc (its unknown c on the finer level's 2c+1),
// from t0 (lc = 1) or the finer level's residual ct
__device__ void ph_restrict(const Dev& D, const Item& it, int lc)
{
    const Prob& P = D.prob[it.q];
    if (!it.on) return;
    const int nf = P.n[lc - 1];
    const float w[3] = {0.25f, 0.5f, 0.25f};
    for (int k = it.k0; k < it.k1; k++) {
        float s = 0.f;
        for (int a = 0; a < 3; a++) {
            const int fk = 2 * k + a;
            if (fk >= nf) continue;
            for (int bb = 0; bb < 3; bb++) {
                const int fj = 2 * it.j + bb;
                if (fj >= nf) continue;
                float row = 0.f;
                for (int cc = 0; cc < 3; cc++) {
                    const int fi = 2 * it.i + cc;
                    if (fi >= nf) continue;
                    const float v = lc == 1 ? D.t0[idx0(P, fi, fj, fk)]
                                            : D.ct[P.coff[lc - 1] + fi + (long long)nf * (fj + (long long)nf * fk)];
                    row = fmaf(w[cc], v, row);
                }
                s = fmaf(w[bb] * w[a], row, s);
            }
        }
        const int n = P.n[lc];
        D.cr[P.coff[lc] + it.i + (long long)n * (it.j + (long long)n * k)] = s;
    }
}

// Jacobi-scaled Chebyshev on level l, on the interval [2/RATIO, 2] of D^-1 A_l:
//   s0 = D^-1 b / theta;  s1 = a1 s0 + b1 D^-1 (b + A s0);
//   X = -(a2 s1 + b2 D^-1 (b + A s1) - c2 s0)
// step 1 writes s1 (cc1); step 2 writes X into z (up: adds it).  b is r_l (down leg)
// or t_l (up leg).
__device__ void ph_jcheb(const Dev& D, const Item& it, int l, int step, bool up)
{
    const Prob& P = D.prob[it.q];
    if (!it.on) return;
    const int n = P.n[l];
    const long long base = P.coff[l];
    const float* bsrc = up ? D.ct : D.cr;
    const float ih2 = P.lih2[l], lm = P.lastm[l], lc = P.lastc[l];
    const long long sj = n, sk = (long long)n * n;
    for (int k = it.k0; k < it.k1; k++) {
        const long long c = base + it.i + sj * it.j + sk * k;
        const float dinv = lvl_dinv(n, it.i, it.j, k, ih2, lc);
        const float bv = bsrc[c];
        const float s0 = dinv * bv * D.jt;
        if (step == 1) {
            // A s0 needs s0 at the neighbours: D^-1 b / theta there
            float as0 = 0.f;
            const int t[3] = {it.i, it.j, k};
            const long long s[3] = {1, sj, sk};
            for (int d = 0; d < 3; d++) {
                int ti[3] = {it.i, it.j, k};
                float um = 0.f;
                if (t[d] > 0) {
                    ti[d] = t[d] - 1;
                    um = lvl_dinv(n, ti[0], ti[1], ti[2], ih2, lc) * bsrc[c - s[d]] * D.jt;
                }
                if (t[d] < n - 1) {
                    ti[d] = t[d] + 1;
                    const float upv = lvl_dinv(n, ti[0], ti[1], ti[2], ih2, lc) * bsrc[c + s[d]] * D.jt;
                    as0 += ih2 * ((um + upv) - 2.f * s0);
                } else {
                    as0 += lm * um + lc * s0;
                }
            }
            D.cc1[c] = fmaf(D.ja1, s0, D.jb1 * dinv * (bv + as0));
        } else {
            const float s1 = D.cc1[c];
            const float as1 = lvl_apply(D.cc1, base, n, it.i, it.j, k, ih2, lm, lc, s1);
            const float X = -(fmaf(D.ja2, s1, D.jb2 * dinv * (bv + as1)) - D.jc2 * s0);
            D.cz[c] = up ? D.cz[c] + X : X;
        }
    }
}

// t_l = r_l - A_l z_l
__device__ void ph_lres(const Dev& D, const Item& it, int l)
{
    const Prob& P = D.prob[it.q];
    if (!it.on) return;
    const int n = P.n[l];
    const long long base = P.coff[l];
    for (int k = it.k0; k < it.k1; k++) {
        const long long c = base + it.i + (long long)n * (it.j + (long long)n * k);
        D.ct[c] = D.cr[c] - lvl_apply(D.cz, base, n, it.i, it.j, k, P.lih2[l], P.lastm[l], P.lastc[l], D.cz[c]);
    }
}

// trilinear prolongation weights of fine unknown f from the coarse line: f = 2c+1
// takes z_c; f = 2c takes (z_{c-1} + z_c) / 2 (z_{-1} = 0, the wall)
__device__ __forceinline__ int pro_taps(int f, int nc, int (&c)[2], float (&w)[2])
{
    if (f & 1) {
        c[0] = f >> 1;
        w[0] = 1.f;
        return c[0] < nc ? 1 : 0;
    }
    const int hc = f >> 1;
    int n = 0;
    if (hc - 1 >= 0) {
        c[n] = hc - 1;
        w[n++] = 0.5f;
    }
    if (hc < nc) {
        c[n] = hc;
        w[n++] = 0.5f;
    }
    return n;
}

__device__ __forceinline__ float prolong_at(const float* zc, long long base, int nc, int fi, int fj, int fk)
{
    int ci[2], cj[2], ck[2];
    float wi[2], wj[2], wk[2];
    const int ni = pro_taps(fi, nc, ci, wi), nj = pro_taps(fj, nc, cj, wj), nk = pro_taps(fk, nc, ck, wk);
    float s = 0.f;
    for (int a = 0; a < nk; a++)
        for (int bb = 0; bb < nj; bb++) {
            float row = 0.f;
            for (int cc = 0; cc < ni; cc++)
                row = fmaf(wi[cc], zc[base + ci[cc] + (long long)nc * (cj[bb] + (long long)nc * ck[a])], row);
            s = fmaf(wk[a] * wj[bb], row, s);
        }
    return s;
}

// z_l += P z_{l+1} on level l >= 1
__device__ void ph_up(const Dev& D, const Item& it, int l)
{
    const Prob& P = D.prob[it.q];
    if (!it.on) return;
    const int n = P.n[l], nc = P.n[l + 1];
    for (int k = it.k0; k < it.k1; k++) {
        const long long c = P.coff[l] + it.i + (long long)n * (it.j + (long long)n * k);
        D.cz[c] += prolong_at(D.cz, P.coff[l + 1], nc, it.i, it.j, k);
    }
}

// level 0: z += P z_1, then sums z.r and z.Ap
__device__ void ph_p0(const Dev& D, const Item& it, Acc<float>& a1, Acc<float>& a2)
{
    const Prob& P = D.prob[it.q];
    if (!it.on) return;
    const int nc = P.n[1];
    for (int k = it.k0; k < it.k1; k++) {
        const long long c = idx0(P, it.i, it.j, k);
        const float zv = D.z[c] + prolong_at(D.cz, P.coff[1], nc, it.i, it.j, k);
        D.z[c] = zv;
        a1.add(zv, D.r[c]);
        a2.add(zv, D.ap[c]);
    }
}

// z_k = A_k^-1 r_k on the coarsest level, the whole level in shared memory (one block):
// passes along x, y, z with V^-1, the eigenvalue division, passes with V
// (matrices as unet::level_exact_data lays them out)
__device__ void ph_exact(const Dev& D, int q, float* sm)
{
    const Prob& P = D.prob[q];
    const int n = P.n[P.k];
    const long long tot = (long long)n * n * n;
    float* cube = sm;
    float* M = sm + tot;
    const int nm = 6 * n * n + 3 * n;
    const float* src = D.mats + P.mats;
    for (int i = threadIdx.x; i < nm; i += NT) M[i] = src[i];
    const long long base = P.coff[P.k];
    for (long long i = threadIdx.x; i < tot; i += NT) cube[i] = D.cr[base + i];
    __syncthreads();
    for (int pass = 0; pass < 7; pass++) {
        if (pass == 3) {
            const float* lam = M + 6 * n * n;
            for (long long i = threadIdx.x; i < tot; i += NT) {
                const int xi = (int)(i % n), yi = (int)((i / n) % n), zi = (int)(i / ((long long)n * n));
                cube[i] = cube[i] / (lam[xi] + lam[n + yi] + lam[2 * n + zi]);
            }
        } else {
            const int axis = pass < 3 ? pass : pass - 4;
            const float* Mat = M + (pass < 3 ? axis : 3 + axis) * n * n;
            const long long stride = axis == 0 ? 1 : (axis == 1 ? n : (long long)n * n);
            float v[EX_MAX];
            for (int t = threadIdx.x; t < n * n; t += NT) {
                long long b0;
                if (axis == 0) b0 = (long long)t * n;
                else if (axis == 1) b0 = (t % n) + (long long)(t / n) * n * n;
                else b0 = t;
                for (int mm = 0; mm < n; mm++) v[mm] = cube[b0 + mm * stride];
                for (int i = 0; i < n; i++) {
                    float acc = 0.f;
                    for (int mm = 0; mm < n; mm++) acc = fmaf(Mat[i * n + mm], v[mm], acc);
                    cube[b0 + i * stride] = acc;
                }
            }
        }
        __syncthreads();
    }
    for (long long i = threadIdx.x; i < tot; i += NT) D.cz[base + i] = cube[i];
    __syncthreads();
}

// Is problem q part of this phase?  (uniform over a block)
__device__ __forceinline__ bool takes_part(const Dev& D, const Phase& ph, int q)
{
    const State& S = D.st[q];
    if (S.done) return false;
    if (ph.type == PH_NORM || ph.type == PH_A || ph.type == PH_B) return true;
    if (S.skip) return false;
    const int k = D.prob[q].k;
    switch (ph.type) {
    case PH_RS:
        return ph.level + 1 <= k;
    case PH_D1: case PH_D2: case PH_DR: case PH_UP: case PH_UR: case PH_U1: case PH_U2:
        return ph.level < k;
    default:
        return true;
    }
}

// The level whose work items a phase covers.
__device__ __forceinline__ int item_level(const Phase& ph)
{
    switch (ph.type) {
    case PH_RS:
        return ph.level + 1;
    case PH_D1: case PH_D2: case PH_DR: case PH_UP: case PH_UR: case PH_U1: case PH_U2:
        return ph.level;
    default:
        return 0;
    }
}

__device__ void run_phase(const Dev& D, const Phase& ph, float* sm)
{
    if (ph.type == PH_EX) {
        for (int q = blockIdx.x; q < D.nprob; q += gridDim.x)
            if (takes_part(D, ph, q)) ph_exact(D, q, sm);
        return;
    }
    const int lev = item_level(ph);
    const long long* row = D.toff + (long long)lev * (D.nprob + 1);
    const long long total = row[D.nprob];
    for (long long item = blockIdx.x; item < total; item += gridDim.x) {
        const Item it = decode(D, lev, item);
        if (!takes_part(D, ph, it.q)) continue;
        const State& S = D.st[it.q];
        const long long first = row[it.q], count = row[it.q + 1] - row[it.q];
        double tot[2];
        switch (ph.type) {
        case PH_NORM: {
            double v[1] = {0.0};
            ph_norm(D, it, v[0]);
            if (item_reduce<1>(D, it, first, count, v, tot)) advance(D, it.q, PH_NORM, tot);
            break;
        }
        case PH_A:
            if (S.mode == 1) {
                Acc<float> a;
                ph_a_fcg(D, it, a);
                double v[1] = {a.value()};
                if (item_reduce<1>(D, it, first, count, v, tot)) advance(D, it.q, PH_A, tot);
            } else {
                ph_a_refine(D, it);
            }
            break;
        case PH_B:
            if (S.mode == 1) {
                Acc<float> a;
                ph_b_fcg(D, it, a);
                double v[1] = {a.value()};
                if (item_reduce<1>(D, it, first, count, v, tot)) advance(D, it.q, PH_B, tot);
            } else {
                double v[1] = {0.0};
                ph_b_refine(D, it, v[0]);
                if (item_reduce<1>(D, it, first, count, v, tot)) advance(D, it.q, PH_B, tot);
            }
            break;
        case PH_C1: ph_cheb0(D, it, 0); break;
        case PH_C2: ph_cheb0(D, it, 1); break;
        case PH_C3: ph_cheb0(D, it, 2); break;
        case PH_R0: ph_r0(D, it); break;
        case PH_RS: ph_restrict(D, it, ph.level + 1); break;
        case PH_D1: ph_jcheb(D, it, ph.level, 1, false); break;
        case PH_D2: ph_jcheb(D, it, ph.level, 2, false); break;
        case PH_DR: ph_lres(D, it, ph.level); break;
        case PH_UR: ph_lres(D, it, ph.level); break;
        case PH_UP: ph_up(D, it, ph.level); break;
        case PH_U1: ph_jcheb(D, it, ph.level, 1, true); break;
        case PH_U2: ph_jcheb(D, it, ph.level, 2, true); break;
        case PH_P0: {
            Acc<float> a1, a2;
            ph_p0(D, it, a1, a2);
            double v[2] = {a1.value(), a2.value()};
            if (item_reduce<2>(D, it, first, count, v, tot)) advance(D, it.q, PH_P0, tot);
            break;
        }
        default:
            break;
        }
    }
}

// The persistent solve: the norm phase, then rounds of the phase program until every
// problem has finished (or max_rounds), a grid barrier after every phase.  All blocks
// read `unfinished` after the same barrier, so they leave the loop together.
__global__ void __launch_bounds__(NT, 6) k_bvc_solve(Dev D)
{
    pdl_enter();
    extern __shared__ float sm_ex[];
    run_phase(D, Phase{PH_NORM, 0}, sm_ex);
    if (!grid_barrier(D)) return;
    for (int round = 0; round < D.max_rounds; round++) {
        for (int p = 0; p < D.nphases; p++) {
            run_phase(D, D.phases[p], sm_ex);
            if (!grid_barrier(D)) return;
        }
        if (*(volatile int*)D.unfinished == 0) break;
    }
}

// Initial state of every problem (one thread per problem), counters and barrier.
__global__ void k_bvc_init(Dev D)
{
    pdl_enter();
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q == 0) {
        D.bar->count = 0u;
        D.bar->gen = 0u;
        D.bar->error = 0;
        *D.unfinished = D.nprob;
    }
    if (q < D.nprob) {
        State s;
        memset(&s, 0, sizeof(s));
        D.st[q] = s;
        D.counters[q] = 0u;
    }
}

// ---- host ----

struct Plan {
    int nprob = 0;
    std::vector<Prob> prob;        // in the caller's order
    std::vector<int> slot;         // problem -> its row in the device table (largest first)
    std::vector<long long> toff;
    std::vector<Phase> phases;
    int maxk = 0;
    size_t ex_smem = 0;
    long long max_items = 0;
    Prob* dprob = nullptr;
    long long* dtoff = nullptr;
    Phase* dphases = nullptr;
    State* dst = nullptr;
    float *cr = nullptr, *cz = nullptr, *ct = nullptr, *cc1 = nullptr;
    float* dmats = nullptr;
    double* partials = nullptr;
    unsigned* counters = nullptr;
    Barrier* bar = nullptr;
    int* unfinished = nullptr;
    Dev D{};
    int grid = 0;
    double limit_s = 5.0;
    cudaGraphExec_t gexec = nullptr;
    std::vector<State> hst;
};

void free_plan(Plan* p)
{
    if (p->gexec) cudaGraphExecDestroy(p->gexec);
    void* ptrs[] = {p->dprob, p->dtoff, p->dphases, p->dst, p->cr, p->cz, p->ct, p->cc1, p->dmats, p->partials,
                    p->counters, p->bar, p->unfinished};
    for (void* q : ptrs)
        if (q) cudaFree(q);
}

// Chebyshev coefficients of the fine smoother (degree 5 on [lmax/RATIO, lmax] with
// lmax = 12/h^2, the preconditioner's recurrence, output X = -s3) in the form
// W = cc Y + cn sum(Y nbrs) + cb B + cz Z, A Y = (sum(Y nbrs) - 6 Y) / h^2:
//   s1 = (2 rho1 / delta) (2 B + A B / theta)
//   s2 = rho2 (2 sigma s1 + 2/delta (B + A s1)) - rho2 rho1 s0,  s0 = B / theta
//   X  = -(rho3 (2 sigma s2 + 2/delta (B + A s2)) - rho3 rho2 s1)
void fine_coefs(Prob& P, double h)
{
    const double ih2 = 1.0 / (h * h), hi = 12.0 * ih2, lo = hi / RATIO;
    const double theta = 0.5 * (lo + hi), delta = 0.5 * (lo - hi), sigma = theta / delta;
    const double rho0 = 1.0 / sigma, rho1 = 1.0 / (2.0 * sigma - rho0), rho2 = 1.0 / (2.0 * sigma - rho1),
                 rho3 = 1.0 / (2.0 * sigma - rho2);
    const double cy[3] = {4.0 * rho1 / delta, 2.0 * rho2 * sigma, -2.0 * rho3 * sigma};
    const double ca[3] = {2.0 * rho1 / (delta * theta), 2.0 * rho2 / delta, -2.0 * rho3 / delta};
    const double cb[3] = {0.0, 2.0 * rho2 / delta - rho2 * rho1 / theta, -2.0 * rho3 / delta};
    const double cz[3] = {0.0, 0.0, rho3 * rho2};
    for (int t = 0; t < 3; t++) {
        P.fcc[t] = (float)(cy[t] - 6.0 * ca[t] * ih2);
        P.fcn[t] = (float)(ca[t] * ih2);
        P.fcb[t] = (float)cb[t];
        P.fcz[t] = (float)cz[t];
    }
}

}  // namespace bvc

using namespace bvc;

#define VK(call)                                                                                   \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess) {                                                                   \
            err = std::string(#call) + ": " + cudaGetErrorString(e_);                              \
            return fail();                                                                         \
        }                                                                                          \
    } while (0)

bool bvc_create(BvcPlan** out, int nprob, const Geo* geo, const long long* off, const BvcPools& pools, double tol,
                double inner_tol, int inner_maxit, int max_refinements, cudaStream_t s, std::string& err)
{
    *out = nullptr;
    Plan* P = new Plan();
    auto fail = [&]() {
        free_plan(P);
        delete P;
        return false;
    };
    P->nprob = nprob;
    P->prob.resize((size_t)nprob);
    long long cpool = 0;
    std::map<int, long long> mats_of;   // edge -> offset of its eigen-solve matrices
    std::vector<float> mats;
    for (int q = 0; q < nprob; q++) {
        const Geo& g = geo[q];
        const int m = g.n[0] - 2;
        if (g.n[1] != g.n[0] || g.n[2] != g.n[0] || g.ds[1] != g.ds[0] || g.ds[2] != g.ds[0]) {
            err = "the persistent V-cycle batch takes cubes with equal spacings";
            return fail();
        }
        Prob& pr = P->prob[(size_t)q];
        std::memset(&pr, 0, sizeof(pr));
        pr.m = m;
        pr.off = off[q];
        int k = 0, n = m;
        while (n > 16 && n % 2 == 0 && k + 1 < MAXLEV) {
            n /= 2;
            k++;
        }
        if (k < 1 || n > EX_MAX) {
            err = "the persistent V-cycle batch needs edges m = c * 2^k with k >= 1 and c <= 32 (m = " +
                  std::to_string(m) + ")";
            return fail();
        }
        pr.k = k;
        const double h = g.ds[0];
        pr.ih2 = 1.0 / (h * h);
        fine_coefs(pr, h);
        for (int l = 0; l <= k; l++) {
            const int nl = m >> l;
            pr.n[l] = nl;
            // planes per item: up to 128 on the solver's grid, where an item's fixed costs
            // (locating its problem, the block sum) are worth amortising over long columns
            // (256 problems of the batched workload: 119.9 ms with 16, 112.8 ms with 128);
            // 16 on the coarse levels
            pr.kz[l] = std::min(nl, l == 0 ? 128 : 16);
            pr.ntx[l] = (nl + 31) / 32;
            pr.nty[l] = (nl + 7) / 8;
            pr.nch[l] = (nl + pr.kz[l] - 1) / pr.kz[l];
            if (l >= 1) {
                const double H = h * (double)(1 << l);
                pr.lih2[l] = (float)(1.0 / (H * H));
                pr.lastm[l] = (float)(2.0 / (H * (H + h)));
                pr.lastc[l] = (float)(-2.0 / (H * h));
                pr.coff[l] = cpool;
                cpool += ((long long)nl * nl * nl + 31) / 32 * 32;
            }
        }
        auto it = mats_of.find(m);
        if (it == mats_of.end()) {
            unet::DLevel L;
            for (int d = 0; d < 3; d++) {
                L.ih2[d] = pr.lih2[k];
                L.last_m[d] = pr.lastm[k];
                L.last_c[d] = pr.lastc[k];
            }
            std::vector<float> mk;
            if (!unet::level_exact_data(unet::Dims{n, n, n}, L, mk)) {
                err = "coarsest level too large for the exact solve";
                return fail();
            }
            it = mats_of.emplace(m, (long long)mats.size()).first;
            mats.insert(mats.end(), mk.begin(), mk.end());
        }
        pr.mats = it->second;
        P->maxk = std::max(P->maxk, k);
        P->ex_smem = std::max(P->ex_smem, sizeof(float) * ((size_t)n * n * n + 6 * (size_t)n * n + 3 * (size_t)n));
    }
    // item order: largest problems first, so their items are handed out first
    std::vector<int> order((size_t)nprob);
    for (int q = 0; q < nprob; q++) order[(size_t)q] = q;
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int b) { return P->prob[(size_t)a].m > P->prob[(size_t)b].m; });
    std::vector<Prob> table((size_t)nprob);
    P->slot.resize((size_t)nprob);
    for (int t = 0; t < nprob; t++) {
        table[(size_t)t] = P->prob[(size_t)order[(size_t)t]];
        P->slot[(size_t)order[(size_t)t]] = t;
    }
    P->toff.assign((size_t)MAXLEV * (nprob + 1), 0);
    for (int l = 0; l < MAXLEV; l++) {
        long long acc = 0;
        for (int t = 0; t < nprob; t++) {
            P->toff[(size_t)l * (nprob + 1) + t] = acc;
            const Prob& pr = table[(size_t)t];
            if (l <= pr.k) acc += (long long)pr.ntx[l] * pr.nty[l] * pr.nch[l];
        }
        P->toff[(size_t)l * (nprob + 1) + nprob] = acc;
        P->max_items = std::max(P->max_items, acc);
    }
    // the phase program of one round
    auto add = [&](int type, int level) { P->phases.push_back(Phase{type, level}); };
    add(PH_A, 0);
    add(PH_B, 0);
    add(PH_C1, 0);
    add(PH_C2, 0);
    add(PH_C3, 0);
    add(PH_R0, 0);
    add(PH_RS, 0);
    for (int l = 1; l < P->maxk; l++) {
        add(PH_D1, l);
        add(PH_D2, l);
        add(PH_DR, l);
        add(PH_RS, l);
    }
    add(PH_EX, 0);
    for (int l = P->maxk - 1; l >= 1; l--) {
        add(PH_UP, l);
        add(PH_UR, l);
        add(PH_U1, l);
        add(PH_U2, l);
    }
    add(PH_P0, 0);

    const size_t cbytes = sizeof(float) * (size_t)std::max(cpool, 32LL);
    VK(cudaMalloc((void**)&P->dprob, sizeof(Prob) * (size_t)nprob));
    VK(cudaMalloc((void**)&P->dtoff, sizeof(long long) * P->toff.size()));
    VK(cudaMalloc((void**)&P->dphases, sizeof(Phase) * P->phases.size()));
    VK(cudaMalloc((void**)&P->dst, sizeof(State) * (size_t)nprob));
    for (float** f : {&P->cr, &P->cz, &P->ct, &P->cc1}) {
        VK(cudaMalloc((void**)f, cbytes));
        VK(cudaMemsetAsync(*f, 0, cbytes, s));
    }
    VK(cudaMalloc((void**)&P->dmats, sizeof(float) * std::max<size_t>(mats.size(), 1)));
    VK(cudaMalloc((void**)&P->partials, sizeof(double) * 2 * (size_t)std::max<long long>(P->max_items, 1)));
    VK(cudaMalloc((void**)&P->counters, sizeof(unsigned) * (size_t)nprob));
    VK(cudaMalloc((void**)&P->bar, sizeof(Barrier)));
    VK(cudaMalloc((void**)&P->unfinished, sizeof(int)));
    VK(cudaMemcpyAsync(P->dprob, table.data(), sizeof(Prob) * (size_t)nprob, cudaMemcpyHostToDevice, s));
    VK(cudaMemcpyAsync(P->dtoff, P->toff.data(), sizeof(long long) * P->toff.size(), cudaMemcpyHostToDevice, s));
    VK(cudaMemcpyAsync(P->dphases, P->phases.data(), sizeof(Phase) * P->phases.size(), cudaMemcpyHostToDevice, s));
    if (!mats.empty())
        VK(cudaMemcpyAsync(P->dmats, mats.data(), sizeof(float) * mats.size(), cudaMemcpyHostToDevice, s));
    VK(cudaStreamSynchronize(s));

    // coarse Jacobi-Chebyshev constants on [2/RATIO, 2] (degree 4, output -s2)
    const double lo = 2.0 / RATIO, hi = 2.0, theta = 0.5 * (lo + hi), delta = 0.5 * (lo - hi), sigma = theta / delta;
    const double rho0 = 1.0 / sigma, rho1 = 1.0 / (2.0 * sigma - rho0), rho2 = 1.0 / (2.0 * sigma - rho1);
    Dev& D = P->D;
    D.prob = P->dprob;
    D.nprob = nprob;
    D.toff = P->dtoff;
    D.phases = P->dphases;
    D.nphases = (int)P->phases.size();
    D.st = P->dst;
    D.x = pools.x;
    D.b = pools.b;
    D.r = pools.r;
    D.z = pools.z;
    D.pa = pools.pa;
    D.pb = pools.pb;
    D.ap = pools.ap;
    D.e = pools.e;
    D.y1 = pools.y1;
    D.y2 = pools.y2;
    D.t0 = pools.t0;
    D.cr = P->cr;
    D.cz = P->cz;
    D.ct = P->ct;
    D.cc1 = P->cc1;
    D.mats = P->dmats;
    D.partials = P->partials;
    D.counters = P->counters;
    D.bar = P->bar;
    D.unfinished = P->unfinished;
    D.tol = tol;
    D.inner_tol = inner_tol;
    D.inner_maxit = inner_maxit;
    D.max_refinements = max_refinements;
    // a round is one FCG iteration or refinement step of every unfinished problem
    D.max_rounds = (int)std::min<long long>(2000, (long long)(max_refinements + 1) * (inner_maxit + 2));
    D.jt = (float)(1.0 / theta);
    D.ja1 = (float)(2.0 * rho1 * sigma);
    D.jb1 = (float)(2.0 * rho1 / delta);
    D.ja2 = (float)(2.0 * rho2 * sigma);
    D.jb2 = (float)(2.0 * rho2 / delta);
    D.jc2 = (float)(rho2 * rho1);
    // one resident wave: the grid barrier needs every block resident
    VK(cudaFuncSetAttribute(k_bvc_solve, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)P->ex_smem));
    int per_sm = 0;
    VK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bvc_solve, NT, P->ex_smem));
    if (per_sm < 1) {
        err = "the persistent kernel does not fit on an SM";
        return fail();
    }
    P->grid = per_sm * sm_count();
    P->hst.resize((size_t)nprob);
    *out = reinterpret_cast<BvcPlan*>(P);
    return true;
}

void bvc_destroy(BvcPlan* plan)
{
    if (!plan) return;
    Plan* P = reinterpret_cast<Plan*>(plan);
    free_plan(P);
    delete P;
}

void bvc_set_wait_limit(BvcPlan* plan, double seconds)
{
    Plan* P = reinterpret_cast<Plan*>(plan);
    P->limit_s = seconds;
    if (P->gexec) {   // the captured launch holds the old limit
        cudaGraphExecDestroy(P->gexec);
        P->gexec = nullptr;
    }
}

// Runs the persistent solve (replaying the captured graph), then reads the states.
// PPS_TIMEOUT when a barrier wait ran out; else the first failing problem's status
// (PPS_NOT_CONVERGED for one stopped short), or PPS_OK.
pps_status bvc_solve(BvcPlan* plan, cudaStream_t s, cudaEvent_t ev0, cudaEvent_t ev1, pps_batch_stats* stats,
                     std::string& err)
{
    Plan* P = reinterpret_cast<Plan*>(plan);
    auto ck = [&](cudaError_t e, const char* what) {
        if (e != cudaSuccess) err = std::string(what) + ": " + cudaGetErrorString(e);
        return e == cudaSuccess;
    };
    P->D.limit_ns = (unsigned long long)(P->limit_s * 1e9);
    if (!P->gexec) {
        cudaGraph_t gr = nullptr;
        if (!ck(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture"))
            return PPS_ERR_CUDA;
        {
            CaptureGuard cap(s);
            launch_pdl(k_bvc_init, (unsigned)((P->nprob + 255) / 256), 256, 0, s, P->D);
            launch_coop(k_bvc_solve, (unsigned)P->grid, NT, P->ex_smem, s, P->D);
            if (!ck(cap.end(&gr), "cudaStreamEndCapture")) return PPS_ERR_CUDA;
        }
        const cudaError_t ie = cudaGraphInstantiate(&P->gexec, gr, 0);
        cudaGraphDestroy(gr);
        if (ie != cudaSuccess) P->gexec = nullptr;
        if (!ck(ie, "cudaGraphInstantiate")) return PPS_ERR_CUDA;
    }
    if (!ck(cudaEventRecord(ev0, s), "cudaEventRecord")) return PPS_ERR_CUDA;
    if (!ck(cudaGraphLaunch(P->gexec, s), "cudaGraphLaunch")) return PPS_ERR_CUDA;
    if (!ck(cudaEventRecord(ev1, s), "cudaEventRecord")) return PPS_ERR_CUDA;
    if (!ck(cudaEventSynchronize(ev1), "cudaEventSynchronize")) return PPS_ERR_CUDA;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ev0, ev1);
    std::vector<State> table((size_t)P->nprob);
    Barrier bar{};
    if (!ck(cudaMemcpyAsync(table.data(), P->dst, sizeof(State) * table.size(), cudaMemcpyDeviceToHost, s),
            "cudaMemcpyAsync") ||
        !ck(cudaMemcpyAsync(&bar, P->bar, sizeof(Barrier), cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync") ||
        !ck(cudaStreamSynchronize(s), "cudaStreamSynchronize"))
        return PPS_ERR_CUDA;
    for (int q = 0; q < P->nprob; q++) P->hst[(size_t)q] = table[(size_t)P->slot[(size_t)q]];
    pps_batch_stats& S = *stats;
    std::memset(&S, 0, sizeof(S));
    S.seconds_solve = ms * 1e-3;
    S.kernel_launches = 2;
    S.graph_replays = 1;
    pps_status rc = PPS_OK;
    for (int q = 0; q < P->nprob; q++) {
        const State& st = P->hst[(size_t)q];
        const double e = st.normb > 0 ? st.err_outer / st.normb : 0.0;
        S.max_err_true = std::max(S.max_err_true, e);
        S.max_iterations = std::max(S.max_iterations, st.total_it);
        S.sum_iterations += st.total_it;
        S.max_refinements = std::max(S.max_refinements, st.refinements);
        const double m = (double)P->prob[(size_t)q].m;
        S.unknowns += m * m * m;
        if (st.done && st.status == PPS_OK) S.converged++;
        else if (rc == PPS_OK) rc = st.done && st.status != PPS_OK ? (pps_status)st.status : PPS_NOT_CONVERGED;
    }
    if (bar.error != 0) {
        err = "a grid barrier of the persistent batched solve waited longer than its limit";
        return PPS_TIMEOUT;
    }
    return rc;
}

void bvc_result(const BvcPlan* plan, int q, pps_stats* st)
{
    const Plan* P = reinterpret_cast<const Plan*>(plan);
    const State& s = P->hst[(size_t)q];
    st->iterations = s.total_it;
    st->refinements = s.refinements;
    st->norm_b = s.normb;
    st->err_true = s.normb > 0 ? s.err_outer / s.normb : -1.0;
    st->err_iter = s.normb > 0 ? s.err / s.normb : -1.0;
}

}  // namespace pps
