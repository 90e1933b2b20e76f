// Batched kernels: many independent grids of uneven size in one launch per phase.
// Included by pps_kernels.cu (same translation unit: shares Acc, finalize, CT).
//
// Every field of every problem lives in one pooled array at the problem's offset.
// A launch has one thread block per (problem, tile, z-chunk) work item; the
// block -> problem table `blk2prob` maps a block to its problem, whose own tile
// shape (columns per thread cx, z-chunk) the autotuner picked for its grid size.
// Reductions are per problem: block partials in launch order, a per-problem
// completion counter, and the problem's last block sums its partials in block
// order and advances that problem's scalars.  A problem whose stop flag is set is
// skipped by every block of every later launch.

struct BCol {
    int p;
    const BProb* P;
    int i, j, k0, k1, cx;
    long long c;     // pooled index of (i, j, k0)
    bool active;
};

__device__ __forceinline__ BCol bcolumn(const BatchDev& B)
{
    BCol q;
    q.p = B.blk2prob[blockIdx.x];
    q.P = &B.prob[q.p];
    const BProb& P = *q.P;
    const unsigned local = blockIdx.x - P.first_block;
    const unsigned tiles = (unsigned)P.ntx * (unsigned)P.nty;
    const unsigned tile = local % tiles, chunk = local / tiles;
    const int bx = (int)(tile % (unsigned)P.ntx), by = (int)(tile / (unsigned)P.ntx);
    q.cx = P.cx;
    // cx 4: the x-vectorised Chebyshev tiles, a float4 per thread from x = 0
    q.i = P.cx == 4 ? bx * 128 + threadIdx.x * 4 : P.g.lo[0] + bx * 32 * P.cx + threadIdx.x;
    q.j = P.g.lo[1] + by * (int)blockDim.y + threadIdx.y;
    q.k0 = P.g.lo[2] + (int)chunk * P.kchunk;
    q.k1 = min(q.k0 + P.kchunk, P.g.hi[2]);
    q.active = q.j < P.g.hi[1];
    q.c = P.off + q.i + P.g.sj * q.j + P.g.sk * q.k0;
    return q;
}

// Per-problem reduction of NS sums; the problem's last block finalizes its state.
template <int NS>
__device__ __forceinline__ void breduce_finalize(double (&v)[NS], const BatchDev& B, const BCol& q,
                                                 double* partials, unsigned* counters, BState* bst, int kind)
{
    __shared__ double sm[32][NS];
    __shared__ int is_last;
    const int tid = threadIdx.x + blockDim.x * threadIdx.y;
    const int nthr = blockDim.x * blockDim.y;
    const int lane = tid & 31, warp = tid >> 5, nwarp = (nthr + 31) >> 5;
#pragma unroll
    for (int s = 0; s < NS; s++) {
        const double w = warp_sum(v[s]);
        if (lane == 0) sm[warp][s] = w;
    }
    __syncthreads();
    if (tid == 0) {
#pragma unroll
        for (int s = 0; s < NS; s++) {
            double t = 0.0;
            for (int w = 0; w < nwarp; w++) t += sm[w][s];
            partials[(size_t)blockIdx.x * 4 + s] = t;
        }
        __threadfence();
        const unsigned ticket = atomicAdd(&counters[q.p], 1u);
        is_last = (ticket == q.P->nblocks - 1);
    }
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    double acc[NS];
#pragma unroll
    for (int s = 0; s < NS; s++) acc[s] = 0.0;
    const unsigned b0 = q.P->first_block, nb = q.P->nblocks;
    for (unsigned b = tid; b < nb; b += nthr) {
#pragma unroll
        for (int s = 0; s < NS; s++) acc[s] += __ldcg(&partials[(size_t)(b0 + b) * 4 + s]);
    }
    __syncthreads();
#pragma unroll
    for (int s = 0; s < NS; s++) {
        const double w = warp_sum(acc[s]);
        if (lane == 0) sm[warp][s] = w;
    }
    __syncthreads();
    if (tid == 0) {
        double tot[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
        for (int s = 0; s < NS; s++) {
            double t = 0.0;
            for (int w = 0; w < nwarp; w++) t += sm[w][s];
            tot[s] = t;
        }
        BState* b = &bst[q.p];
        RedCtx rc;
        rc.partials = partials;
        rc.counter = &counters[q.p];
        rc.st = &b->s;
        rc.hist = nullptr;
        rc.kind = kind;
        if (kind == FIN_NORMB) {
            b->s.normb = sqrt(tot[0]);
            b->tol_outer = b->tol_rel_outer * b->s.normb;
        } else {
            finalize(rc, tot);
            if (kind == FIN_RES0) {
                b->err_outer = b->s.err0;
                if (b->s.done) {   // the FP64 residual meets the tolerance (or is not finite)
                    b->finished = 1;
                    b->outer_status = b->s.status;
                }
            }
        }
        __threadfence();
        counters[q.p] = 0u;
    }
}

#define BSKIP_INNER(bst, q) \
    if (*(volatile const int*)&(bst)[(q).p].s.done) return;
#define BSKIP_FINISHED(bst, q) \
    if (*(volatile const int*)&(bst)[(q).p].finished) return;

// Set-up of one refinement step: the inner scalars restart, the outer tolerance
// is restored as the first stop test.
__global__ void bk_refine_init(int nprob, BState* bst, int inner_maxit, double inner_tol)
{
    pdl_enter();
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nprob) return;
    BState& b = bst[p];
    DevState& s = b.s;
    s.rho0 = 1.0;
    s.alpha = s.omega = s.beta = 1.0;
    s.err = -1.0;
    s.err0 = -1.0;
    s.tol_abs = b.tol_outer;
    s.tol_rel = inner_tol;
    s.tol_relative = 1;
    s.rho0_from_r = 1;
    s.hist_scale = 1.0;
    s.hist_cap = 0;
    s.iter = 0;
    s.maxit = inner_maxit;
    s.done = b.finished ? 1 : 0;
    s.status = 0;
}

// End of a refinement step: count the inner iterations of every problem that ran.
__global__ void bk_refine_end(int nprob, BState* bst)
{
    pdl_enter();
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nprob) return;
    BState& b = bst[p];
    if (b.finished) return;
    b.total_iters += b.s.iter;
    b.refinements += 1;
}

// ||b_adj||^2 per problem (Dirichlet values moved to the right-hand side).
__global__ void __launch_bounds__(256) bk_norm_badj(BatchDev B, const double* __restrict__ b,
                                                    const double* __restrict__ x, double* partials,
                                                    unsigned* counters, BState* bst)
{
    pdl_enter();
    const BCol q = bcolumn(B);
    const Geo& g = q.P->g;
    double s = 0.0;
    Faces none;
    for (int f = 0; f < 6; f++) none.g[f] = nullptr;
    if (q.active) {
        for (int u = 0; u < q.cx; u++) {
            const int i = q.i + 32 * u;
            if (i >= g.hi[0]) break;
            long long c = q.c + 32 * u;
            for (int k = q.k0; k < q.k1; k++) {
                // badj_exact indexes relative to the problem's base
                const double v = badj_exact(g, b + q.P->off, x + q.P->off, none, c - q.P->off, i, q.j, k);
                s = fmx(v, v, s);
                c += g.sk;
            }
        }
    }
    double v[1] = {s};
    breduce_finalize<1>(v, B, q, partials, counters, bst, FIN_NORMB);
}

// FP64 true residual r = b - A x per problem, stored in FP32 r, r0 and p.
__global__ void __launch_bounds__(256) bk_residual(BatchDev B, const double* __restrict__ x,
                                                   const double* __restrict__ b, float* __restrict__ r,
                                                   float* __restrict__ r0, float* __restrict__ p,
                                                   double* partials, unsigned* counters, BState* bst)
{
    pdl_enter();
    const BCol q = bcolumn(B);
    BSKIP_FINISHED(bst, q);
    const Geo& g = q.P->g;
    const double ix = 1.0 / (g.ds[0] * g.ds[0]), iy = 1.0 / (g.ds[1] * g.ds[1]), iz = 1.0 / (g.ds[2] * g.ds[2]);
    const double cc = -2.0 * (ix + iy + iz);
    double s = 0.0;
    if (q.active) {
        for (int u = 0; u < q.cx; u++) {
            if (q.i + 32 * u >= g.hi[0]) break;
            long long c = q.c + 32 * u;
            double um = x[c - g.sk], uc = x[c];
            for (int k = q.k0; k < q.k1; k++) {
                const double up = x[c + g.sk];
                double a = cc * uc;
                a = fmx(ix, x[c - 1] + x[c + 1], a);
                a = fmx(iy, x[c - g.sj] + x[c + g.sj], a);
                a = fmx(iz, um + up, a);
                const double rv = b[c] - a;
                const float rs = (float)rv;
                r[c] = rs;
                r0[c] = rs;
                p[c] = rs;
                s = fmx(rv, rv, s);
                um = uc;
                uc = up;
                c += g.sk;
            }
        }
    }
    double v[1] = {s};
    breduce_finalize<1>(v, B, q, partials, counters, bst, FIN_RES0);
}

__global__ void __launch_bounds__(256) bk_zero(BatchDev B, float* __restrict__ e, const BState* bst)
{
    pdl_enter();
    const BCol q = bcolumn(B);
    BSKIP_FINISHED(bst, q);
    if (!q.active) return;
    for (int u = 0; u < q.cx; u++) {
        if (q.i + 32 * u >= q.P->g.hi[0]) break;
        long long c = q.c + 32 * u;
        for (int k = q.k0; k < q.k1; k++, c += q.P->g.sk) e[c] = 0.0f;
    }
}

// x += e per problem that ran this refinement step.
__global__ void __launch_bounds__(256) bk_add_correction(BatchDev B, double* __restrict__ x,
                                                         const float* __restrict__ e, const BState* bst)
{
    pdl_enter();
    const BCol q = bcolumn(B);
    BSKIP_FINISHED(bst, q);
    if (!q.active) return;
    for (int u = 0; u < q.cx; u++) {
        if (q.i + 32 * u >= q.P->g.hi[0]) break;
        long long c = q.c + 32 * u;
        for (int k = q.k0; k < q.k1; k++, c += q.P->g.sk) x[c] += (double)e[c];
    }
}

// Chebyshev s1 (coefficients per problem: coef[p * cstride + ci]).
__global__ void __launch_bounds__(256) bk_cheb_s01(BatchDev B, const float* __restrict__ Bf, float* __restrict__ Y,
                                                   const CT<float>* __restrict__ coef, int cstride, int ci,
                                                   const BState* bst)
{
    pdl_enter();
    const BCol q = bcolumn(B);
    BSKIP_INNER(bst, q);
    if (!q.active) return;
    const CT<float> cf = coef[(size_t)q.p * cstride + ci];
    const Geo& g = q.P->g;
    if (q.cx == 4) {   // the block's rows are whole warps: all lanes reach the shuffles
        cheb_v4_march<0>(g, q.i, q.k0, q.k1, q.c, Bf, nullptr, nullptr, Y, cf);
        return;
    }
    const long long sj = g.sj, sk = g.sk;
    for (int u = 0; u < q.cx; u++) {
        if (q.i + 32 * u >= g.hi[0]) break;
        long long c = q.c + 32 * u;
        float bm = Bf[c - sk], bc = Bf[c];
#pragma unroll 2
        for (int k = q.k0; k < q.k1; k++) {
            const float bp = Bf[c + sk];
            float y = cf.cc * bc;
            y = fmx(cf.cx, Bf[c - 1] + Bf[c + 1], y);
            y = fmx(cf.cy, Bf[c - sj] + Bf[c + sj], y);
            y = fmx(cf.cz, bm + bp, y);
            Y[c] = y;
            bm = bc;
            bc = bp;
            c += sk;
        }
    }
}

template <bool HAS_Z>
__global__ void __launch_bounds__(256) bk_cheb_sweep(BatchDev B, const float* __restrict__ Y,
                                                     const float* __restrict__ Bf, const float* __restrict__ Z,
                                                     float* __restrict__ W, const CT<float>* __restrict__ coef,
                                                     int cstride, int ci, const BState* bst)
{
    pdl_enter();
    const BCol q = bcolumn(B);
    BSKIP_INNER(bst, q);
    if (!q.active) return;
    const CT<float> cf = coef[(size_t)q.p * cstride + ci];
    const Geo& g = q.P->g;
    if (q.cx == 4) {
        cheb_v4_march<HAS_Z ? 2 : 1>(g, q.i, q.k0, q.k1, q.c, Y, Bf, Z, W, cf);
        return;
    }
    const long long sj = g.sj, sk = g.sk;
    for (int u = 0; u < q.cx; u++) {
        if (q.i + 32 * u >= g.hi[0]) break;
        long long c = q.c + 32 * u;
        float ym = Y[c - sk], yc = Y[c];
#pragma unroll 2
        for (int k = q.k0; k < q.k1; k++) {
            const float yp = Y[c + sk];
            float w = cf.cc * yc;
            w = fmx(cf.cx, Y[c - 1] + Y[c + 1], w);
            w = fmx(cf.cy, Y[c - sj] + Y[c + sj], w);
            w = fmx(cf.cz, ym + yp, w);
            w = fmx(cf.cb, Bf[c], w);
            if (HAS_Z) w = fmx(cf.cw, Z[c], w);
            W[c] = w;
            ym = yc;
            yc = yp;
            c += sk;
        }
    }
}

// NS = 1: Au and sum r0*Au (FIN_ALPHA); NS = 2: Au, sum r*Au and Au*Au (FIN_OMEGA).
template <int NS>
__global__ void __launch_bounds__(256) bk_stencil_dot(BatchDev B, const float* __restrict__ u,
                                                      const float* __restrict__ w, float* __restrict__ Au,
                                                      double* partials, unsigned* counters, BState* bst)
{
    pdl_enter();
    const BCol q = bcolumn(B);
    BSKIP_INNER(bst, q);
    const Geo& g = q.P->g;
    const float ix = (float)(1.0 / (g.ds[0] * g.ds[0])), iy = (float)(1.0 / (g.ds[1] * g.ds[1])),
                iz = (float)(1.0 / (g.ds[2] * g.ds[2]));
    const float cc = (float)(-2.0 * (1.0 / (g.ds[0] * g.ds[0]) + 1.0 / (g.ds[1] * g.ds[1]) +
                                    1.0 / (g.ds[2] * g.ds[2])));
    Acc<float> a1, a2;
    if (q.active) {
        const long long sj = g.sj, sk = g.sk;
        for (int uu = 0; uu < q.cx; uu++) {
            if (q.i + 32 * uu >= g.hi[0]) break;
            long long c = q.c + 32 * uu;
            float um = u[c - sk], uc = u[c];
#pragma unroll 2
            for (int k = q.k0; k < q.k1; k++) {
                const float up = u[c + sk];
                float a = cc * uc;
                a = fmx(ix, u[c - 1] + u[c + 1], a);
                a = fmx(iy, u[c - sj] + u[c + sj], a);
                a = fmx(iz, um + up, a);
                Au[c] = a;
                a1.add(w[c], a);
                if (NS == 2) a2.add(a, a);
                um = uc;
                uc = up;
                c += sk;
            }
        }
    }
    double v[NS];
    v[0] = a1.value();
    if (NS == 2) v[NS - 1] = a2.value();
    breduce_finalize<NS>(v, B, q, partials, counters, bst, NS == 1 ? FIN_ALPHA : FIN_OMEGA);
}

__global__ void __launch_bounds__(256) bk_axpy_alpha(BatchDev B, float* __restrict__ r, const float* __restrict__ v,
                                                     const BState* bst)
{
    pdl_enter();
    const BCol q = bcolumn(B);
    BSKIP_INNER(bst, q);
    if (!q.active) return;
    const float a = (float)bst[q.p].s.alpha;
    for (int u = 0; u < q.cx; u++) {
        if (q.i + 32 * u >= q.P->g.hi[0]) break;
        long long c = q.c + 32 * u;
#pragma unroll 4
        for (int k = q.k0; k < q.k1; k++, c += q.P->g.sk) r[c] = fmx(-a, v[c], r[c]);
    }
}

__global__ void __launch_bounds__(256) bk_update_xr(BatchDev B, float* __restrict__ x, const float* __restrict__ Mp,
                                                    const float* __restrict__ z, float* __restrict__ r,
                                                    const float* __restrict__ Az, const float* __restrict__ r0,
                                                    double* partials, unsigned* counters, BState* bst)
{
    pdl_enter();
    const BCol q = bcolumn(B);
    BSKIP_INNER(bst, q);
    Acc<float> a1, a2;
    if (q.active) {
        const float a = (float)bst[q.p].s.alpha, w = (float)bst[q.p].s.omega;
        for (int u = 0; u < q.cx; u++) {
            if (q.i + 32 * u >= q.P->g.hi[0]) break;
            long long c = q.c + 32 * u;
#pragma unroll 2
            for (int k = q.k0; k < q.k1; k++, c += q.P->g.sk) {
                x[c] = fmx(w, z[c], fmx(a, Mp[c], x[c]));
                const float rn = fmx(-w, Az[c], r[c]);
                r[c] = rn;
                a1.add(r0[c], rn);
                a2.add(rn, rn);
            }
        }
    }
    double v[2] = {a1.value(), a2.value()};
    breduce_finalize<2>(v, B, q, partials, counters, bst, FIN_CONV);
}

__global__ void __launch_bounds__(256) bk_update_p(BatchDev B, float* __restrict__ p, const float* __restrict__ r,
                                                   const float* __restrict__ AMp, const BState* bst)
{
    pdl_enter();
    const BCol q = bcolumn(B);
    BSKIP_INNER(bst, q);
    if (!q.active) return;
    const float be = (float)bst[q.p].s.beta, w = (float)bst[q.p].s.omega;
    for (int u = 0; u < q.cx; u++) {
        if (q.i + 32 * u >= q.P->g.hi[0]) break;
        long long c = q.c + 32 * u;
#pragma unroll 4
        for (int k = q.k0; k < q.k1; k++, c += q.P->g.sk) p[c] = fmx(be, fmx(-w, AMp[c], p[c]), r[c]);
    }
}

// ---- batched launch wrappers ----

static inline unsigned bgrid(const BatchDev& B) { return B.total_blocks; }

void b_refine_init(const BatchDev& B, BState* bst, int inner_maxit, double inner_tol, cudaStream_t s)
{
    launch_pdl(bk_refine_init, (B.nprob + 127) / 128, 128, 0, s, B.nprob, bst, inner_maxit, inner_tol);
    PPS_COUNT_LAUNCH();
}
void b_refine_end(const BatchDev& B, BState* bst, cudaStream_t s)
{
    launch_pdl(bk_refine_end, (B.nprob + 127) / 128, 128, 0, s, B.nprob, bst);
    PPS_COUNT_LAUNCH();
}
void b_norm_badj(const BatchDev& B, const double* b, const double* x, double* part, unsigned* cnt, BState* bst,
                 cudaStream_t s)
{
    launch_pdl(bk_norm_badj, bgrid(B), dim3(32, 8), 0, s, B, b, x, part, cnt, bst);
    PPS_COUNT_LAUNCH();
}
void b_residual(const BatchDev& B, const double* x, const double* b, float* r, float* r0, float* p, double* part,
                unsigned* cnt, BState* bst, cudaStream_t s)
{
    launch_pdl(bk_residual, bgrid(B), dim3(32, 8), 0, s, B, x, b, r, r0, p, part, cnt, bst);
    PPS_COUNT_LAUNCH();
}
void b_zero(const BatchDev& B, float* e, const BState* bst, cudaStream_t s)
{
    launch_pdl(bk_zero, bgrid(B), dim3(32, 8), 0, s, B, e, bst);
    PPS_COUNT_LAUNCH();
}
void b_add_correction(const BatchDev& B, double* x, const float* e, const BState* bst, cudaStream_t s)
{
    launch_pdl(bk_add_correction, bgrid(B), dim3(32, 8), 0, s, B, x, e, bst);
    PPS_COUNT_LAUNCH();
}
void b_cheb_s01(const BatchDev& B, const float* Bf, float* Y, const void* coef, int cstride, int ci,
                const BState* bst, cudaStream_t s)
{
    launch_pdl(bk_cheb_s01, bgrid(B), dim3(32, 8), 0, s, B, Bf, Y, (const CT<float>*)coef, cstride, ci, bst);
    PPS_COUNT_LAUNCH();
}
void b_cheb_sweep(const BatchDev& B, const float* Y, const float* Bf, const float* Z, float* W, const void* coef,
                  int cstride, int ci, const BState* bst, cudaStream_t s)
{
    if (Z) launch_pdl(bk_cheb_sweep<true>, bgrid(B), dim3(32, 8), 0, s, B, Y, Bf, Z, W, (const CT<float>*)coef, cstride, ci, bst);
    else launch_pdl(bk_cheb_sweep<false>, bgrid(B), dim3(32, 8), 0, s, B, Y, Bf, Z, W, (const CT<float>*)coef, cstride, ci, bst);
    PPS_COUNT_LAUNCH();
}
void b_stencil_dot(const BatchDev& B, const float* u, const float* w, float* Au, int nsums, double* part,
                   unsigned* cnt, BState* bst, cudaStream_t s)
{
    if (nsums == 1) launch_pdl(bk_stencil_dot<1>, bgrid(B), dim3(32, 8), 0, s, B, u, w, Au, part, cnt, bst);
    else launch_pdl(bk_stencil_dot<2>, bgrid(B), dim3(32, 8), 0, s, B, u, w, Au, part, cnt, bst);
    PPS_COUNT_LAUNCH();
}
void b_axpy_alpha(const BatchDev& B, float* r, const float* v, const BState* bst, cudaStream_t s)
{
    launch_pdl(bk_axpy_alpha, bgrid(B), dim3(32, 8), 0, s, B, r, v, bst);
    PPS_COUNT_LAUNCH();
}
void b_update_xr(const BatchDev& B, float* x, const float* Mp, const float* z, float* r, const float* Az,
                 const float* r0, double* part, unsigned* cnt, BState* bst, cudaStream_t s)
{
    launch_pdl(bk_update_xr, bgrid(B), dim3(32, 8), 0, s, B, x, Mp, z, r, Az, r0, part, cnt, bst);
    PPS_COUNT_LAUNCH();
}
void b_update_p(const BatchDev& B, float* p, const float* r, const float* AMp, const BState* bst, cudaStream_t s)
{
    launch_pdl(bk_update_p, bgrid(B), dim3(32, 8), 0, s, B, p, r, AMp, bst);
    PPS_COUNT_LAUNCH();
}
void b_cast_coef(const Coef* in, void* out, size_t n)
{
    CT<float>* o = (CT<float>*)out;
    for (size_t i = 0; i < n; i++) o[i] = cast_coef<float>(in[i]);
}
size_t b_coef_size() { return sizeof(CT<float>); }
