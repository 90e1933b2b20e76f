// Batched solves: many independent Dirichlet grids of uneven size solved together.
//
// No reference counterpart (the reference solves one block-decomposed grid per
// run).  Each problem is the reference's solve -- BiCGSTAB with the Chebyshev
// preconditioner on its own grid and its own eigenvalue bounds -- in the MIXED form:
// FP32 inner iterations with FP64-accurate dots, FP64 true residual and refinement.
// Every phase of the loop is ONE launch over all problems (one block per
// (problem, tile, z-chunk) item, per-problem tile shapes from the autotuner); the
// inner iteration is captured once as a CUDA graph and replayed until every
// problem's stop flag is set.
#include "../../include/pps.h"
#include "pps_internal.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <new>
#include <numeric>
#include <string>
#include <vector>

using namespace pps;

namespace {

struct Fail {};

#define BK(call)                                                                              \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess) {                                                              \
            pps_internal_set_error((std::string(#call) + ": " + cudaGetErrorString(e_)).c_str()); \
            throw Fail{};                                                                     \
        }                                                                                     \
    } while (0)

const double kPi = 3.141592653589793;

// Tiles of one grid shape: columns per thread and planes per z-chunk of every
// kernel, and, where the rows allow it, the x-vectorised float4 tiles (v4, with their
// own z-chunk) that the Chebyshev kernels then run on.
struct SizeTile {
    int cx = 1;
    int kchunk = 32;
    bool v4 = false;
    int kchunk4 = 32;
};

const int kKchunks[] = {8, 16, 32, 64, 128};

}  // namespace

struct pps_batch {
    int nprob = 0;
    std::vector<pps_grid> grids;
    pps_config cfg;
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::vector<Geo> geo;
    std::vector<long long> off;      // pooled offset of each problem's field
    long long pool = 0;
    std::map<long long, SizeTile> tiles;   // keyed by unknown count of a grid shape
    std::vector<double> theta, delta, sigma;
    // device
    double *x = nullptr, *b = nullptr;
    float *p = nullptr, *r = nullptr, *r0 = nullptr, *Mp = nullptr, *AMp = nullptr, *z = nullptr, *Az = nullptr;
    float *Y = nullptr, *Z = nullptr, *W = nullptr, *e = nullptr;
    BProb* dprob = nullptr;
    unsigned* dblk = nullptr;
    unsigned blk_cap = 0;
    // the Chebyshev kernels' table (v4 tiles where chosen)
    BProb* dprob4 = nullptr;
    unsigned* dblk4 = nullptr;
    unsigned blk_cap4 = 0;
    double* partials = nullptr;
    unsigned* counters = nullptr;
    BState* dst = nullptr;
    BState* hst = nullptr;
    void* coef = nullptr;
    int cstride = 0;
    BatchDev B;
    BatchDev B4;
    cudaGraphExec_t gexec = nullptr;
    int g_iters = 0;
    int g_launches = 0;
    pps_batch_stats stats;
    BvcPlan* vc = nullptr;   // krylov FCG: the persistent V-cycle solve
};

namespace {

long long key_of(const Geo& g)
{
    // shape key: unknown extents packed
    return ((long long)(g.hi[0] - g.lo[0]) << 40) | ((long long)(g.hi[1] - g.lo[1]) << 20) |
           (long long)(g.hi[2] - g.lo[2]);
}

// The problem's tile for the Chebyshev kernels (cheb) or for the others.  v4 tiles
// start at x = 0 and must reach hi[0]; they need a row stride of whole float4s.
BProb make_prob(const Geo& g, long long off, const SizeTile& t, bool cheb)
{
    BProb P;
    P.g = g;
    P.off = off;
    const bool v4 = cheb && t.v4 && g.sj % 4 == 0 && off % 4 == 0;
    P.cx = v4 ? 4 : t.cx;
    const int ux = g.hi[0] - g.lo[0], uy = g.hi[1] - g.lo[1], uz = g.hi[2] - g.lo[2];
    P.ntx = v4 ? (g.hi[0] + 127) / 128 : (ux + 32 * t.cx - 1) / (32 * t.cx);
    P.nty = (uy + 7) / 8;
    P.kchunk = std::min(v4 ? t.kchunk4 : t.kchunk, uz);
    P.nchunks = (uz + P.kchunk - 1) / P.kchunk;
    P.nblocks = (unsigned)P.ntx * P.nty * P.nchunks;
    P.first_block = 0;
    return P;
}

// Builds the problem table and the block -> problem map for the problems in
// `which` (biggest first, so the longest items start first), uploads them: the
// table of every kernel, or (cheb) the Chebyshev kernels' own.
BatchDev build_table(pps_batch* s, const std::vector<int>& which, bool cheb = false)
{
    BProb*& dprob = cheb ? s->dprob4 : s->dprob;
    unsigned*& dblk = cheb ? s->dblk4 : s->dblk;
    unsigned& cap = cheb ? s->blk_cap4 : s->blk_cap;
    const BatchDev& previous = cheb ? s->B4 : s->B;
    std::vector<int> order = which;
    std::stable_sort(order.begin(), order.end(), [&](int a, int c) {
        const long long na = (long long)(s->geo[a].hi[0] - s->geo[a].lo[0]) * (s->geo[a].hi[1] - s->geo[a].lo[1]) *
                             (s->geo[a].hi[2] - s->geo[a].lo[2]);
        const long long nc = (long long)(s->geo[c].hi[0] - s->geo[c].lo[0]) * (s->geo[c].hi[1] - s->geo[c].lo[1]) *
                             (s->geo[c].hi[2] - s->geo[c].lo[2]);
        return na > nc;
    });
    std::vector<BProb> hp((size_t)s->nprob);
    std::vector<unsigned> blk;
    for (int p = 0; p < s->nprob; p++)
        hp[(size_t)p] = make_prob(s->geo[(size_t)p], s->off[(size_t)p], s->tiles[key_of(s->geo[(size_t)p])], cheb);
    for (int p : order) {
        BProb& P = hp[(size_t)p];
        P.first_block = (unsigned)blk.size();
        for (unsigned q = 0; q < P.nblocks; q++) blk.push_back((unsigned)p);
    }
    if (blk.size() > cap) {
        if (s->gexec) {   // a captured graph holds the old table pointers
            cudaGraphExecDestroy(s->gexec);
            s->gexec = nullptr;
        }
        if (dblk) cudaFree(dblk);
        cap = (unsigned)blk.size();
        BK(cudaMalloc((void**)&dblk, sizeof(unsigned) * cap));
        if (!cheb) {   // block partials of the reductions (the Chebyshev kernels reduce nothing)
            if (s->partials) cudaFree(s->partials);
            BK(cudaMalloc((void**)&s->partials, sizeof(double) * 4 * (size_t)cap));
        }
    }
    BK(cudaMemcpyAsync(dprob, hp.data(), sizeof(BProb) * hp.size(), cudaMemcpyHostToDevice, s->stream));
    BK(cudaMemcpyAsync(dblk, blk.data(), sizeof(unsigned) * blk.size(), cudaMemcpyHostToDevice, s->stream));
    BK(cudaStreamSynchronize(s->stream));
    BatchDev B;
    B.prob = dprob;
    B.blk2prob = dblk;
    B.nprob = s->nprob;
    B.total_blocks = (unsigned)blk.size();
    if (s->gexec && B.total_blocks != previous.total_blocks) {   // the graph was captured for another table
        cudaGraphExecDestroy(s->gexec);
        s->gexec = nullptr;
    }
    return B;
}

// Pre-folded Chebyshev coefficients of problem p (same algebra as the single-grid
// path): index 0 = s1, index it-1 = sweep it for it = 2..n-2 (s0 folded into the
// first sweep, output scale -1 on the last).
void coefs_of(const pps_batch* s, int p, Coef* out)
{
    const Geo& g = s->geo[(size_t)p];
    const double ix = 1.0 / (g.ds[0] * g.ds[0]), iy = 1.0 / (g.ds[1] * g.ds[1]), iz = 1.0 / (g.ds[2] * g.ds[2]);
    const double acc = -2.0 * (ix + iy + iz);
    const double theta = s->theta[(size_t)p], delta = s->delta[(size_t)p], sigma = s->sigma[(size_t)p];
    const int n = s->cfg.cheb_degree;
    double rhoOld = 1 / sigma;
    double rhoCurr = 1 / (2 * sigma - rhoOld);
    const double t = 2 * rhoCurr / delta;
    Coef c0{t * (2.0 + acc / theta), t * ix / theta, t * iy / theta, t * iz / theta, 0.0, 0.0, 1.0};
    out[0] = c0;
    for (int it = 2; it <= n - 2; it++) {
        rhoOld = rhoCurr;
        rhoCurr = 1 / (2 * sigma - rhoOld);
        const double tod = 2.0 / delta;
        Coef c{rhoCurr * (2.0 * sigma + tod * acc), rhoCurr * tod * ix, rhoCurr * tod * iy, rhoCurr * tod * iz,
               rhoCurr * tod, -rhoCurr * rhoOld, it == n - 2 ? -1.0 : 1.0};
        if (it == 2) {
            c.cb += c.cw / theta;
            c.cw = 0.0;
        }
        out[it - 1] = c;
    }
}

// Chebyshev preconditioner X = M^{-1} Bf for every active problem.
void b_precond(pps_batch* s, const BatchDev& B, const float* Bf, float* X)
{
    const int n = s->cfg.cheb_degree;
    float* Y = s->Y;
    float* Z = s->Z;
    float* W = s->W;
    const BatchDev& B4 = s->B4;   // the Chebyshev kernels' tiles (B: the others')
    (void)B;
    b_cheb_s01(B4, Bf, Y, s->coef, s->cstride, 0, s->dst, s->stream);
    for (int it = 2; it <= n - 2; it++) {
        const bool last = it == n - 2;
        b_cheb_sweep(B4, Y, Bf, it == 2 ? nullptr : Z, last ? X : W, s->coef, s->cstride, it - 1, s->dst, s->stream);
        if (!last) {
            float* t = Z;
            Z = Y;
            Y = W;
            W = t;
        }
    }
}

void b_iteration(pps_batch* s, const BatchDev& B)
{
    cudaStream_t st = s->stream;
    b_precond(s, B, s->p, s->Mp);
    b_stencil_dot(B, s->Mp, s->r0, s->AMp, 1, s->partials, s->counters, s->dst, st);
    b_axpy_alpha(B, s->r, s->AMp, s->dst, st);
    b_precond(s, B, s->r, s->z);
    b_stencil_dot(B, s->z, s->r, s->Az, 2, s->partials, s->counters, s->dst, st);
    b_update_xr(B, s->e, s->Mp, s->z, s->r, s->Az, s->r0, s->partials, s->counters, s->dst, st);
    b_update_p(B, s->p, s->r, s->AMp, s->dst, st);
}

void read_states(pps_batch* s)
{
    BK(cudaMemcpyAsync(s->hst, s->dst, sizeof(BState) * (size_t)s->nprob, cudaMemcpyDeviceToHost, s->stream));
    BK(cudaStreamSynchronize(s->stream));
}

bool any_inner_active(const pps_batch* s)
{
    for (int p = 0; p < s->nprob; p++)
        if (!s->hst[p].s.done) return true;
    return false;
}

bool any_unfinished(const pps_batch* s)
{
    for (int p = 0; p < s->nprob; p++)
        if (!s->hst[p].finished) return true;
    return false;
}

void free_batch(pps_batch* s)
{
    if (s->vc) bvc_destroy(s->vc);
    if (s->gexec) cudaGraphExecDestroy(s->gexec);
    void* ptrs[] = {s->x, s->b, s->p, s->r, s->r0, s->Mp, s->AMp, s->z, s->Az, s->Y, s->Z, s->W, s->e,
                    s->dprob, s->dblk, s->dprob4, s->dblk4, s->partials, s->counters, s->dst, s->coef};
    for (void* q : ptrs)
        if (q) cudaFree(q);
    if (s->hst) cudaFreeHost(s->hst);
    if (s->ev0) cudaEventDestroy(s->ev0);
    if (s->ev1) cudaEventDestroy(s->ev1);
    if (s->stream) cudaStreamDestroy(s->stream);
}

template <typename Fn>
pps_status bguard(Fn&& fn)
{
    const unsigned long long f0 = launch_failures();
    try {
        const pps_status rc = fn();
        return rc >= 0 && launch_failures() != f0 ? PPS_ERR_CUDA : rc;
    } catch (const Fail&) {
        return PPS_ERR_CUDA;
    } catch (const std::bad_alloc&) {
        pps_internal_set_error("host allocation failed");
        return PPS_ERR_OUT_OF_MEMORY;
    }
}

pps_status run_batch(pps_batch* s)
{
    cudaStream_t st = s->stream;
    std::vector<int> all((size_t)s->nprob);
    std::iota(all.begin(), all.end(), 0);
    s->B = build_table(s, all);
    s->B4 = build_table(s, all, true);
    const BatchDev& B = s->B;
    std::vector<BState> init((size_t)s->nprob);
    std::memset(init.data(), 0, sizeof(BState) * init.size());
    for (auto& q : init) {
        q.tol_rel_outer = s->cfg.tol;
        q.s.done = 0;
    }
    BK(cudaMemcpyAsync(s->dst, init.data(), sizeof(BState) * init.size(), cudaMemcpyHostToDevice, st));
    BK(cudaMemsetAsync(s->counters, 0, sizeof(unsigned) * (size_t)s->nprob, st));
    const int l0 = launches_counter();
    BK(cudaEventRecord(s->ev0, st));
    b_norm_badj(B, s->b, s->x, s->partials, s->counters, s->dst, st);
    read_states(s);
    bool zero_rhs = false;
    for (int p = 0; p < s->nprob; p++) {
        if (!(s->hst[p].s.normb > 0.0)) {
            zero_rhs = true;
        }
    }
    if (zero_rhs) return PPS_ERR_ZERO_RHS;
    const int chunk = std::max(1, s->cfg.check_every > 0 ? s->cfg.check_every : 8);
    int replays = 0;
    for (int ref = 0; ref <= s->cfg.max_refinements; ref++) {
        b_refine_init(B, s->dst, s->cfg.inner_maxit, s->cfg.inner_tol, st);
        b_residual(B, s->x, s->b, s->r, s->r0, s->p, s->partials, s->counters, s->dst, st);
        read_states(s);
        if (!any_unfinished(s) || ref == s->cfg.max_refinements) break;
        b_zero(B, s->e, s->dst, st);
        if (s->cfg.use_graph) {
            if (!s->gexec || s->g_iters != chunk) {
                if (s->gexec) cudaGraphExecDestroy(s->gexec);
                s->gexec = nullptr;
                cudaGraph_t gr = nullptr;
                const int c0 = launches_counter();
                {
                    BK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
                    CaptureGuard cap(st);   // an error below ends the capture
                    for (int q = 0; q < chunk; q++) b_iteration(s, B);
                    BK(cap.end(&gr));
                }
                s->g_launches = launches_counter() - c0;
                launches_counter_add(-s->g_launches);
                const cudaError_t ie = cudaGraphInstantiate(&s->gexec, gr, 0);
                cudaGraphDestroy(gr);
                if (ie != cudaSuccess) s->gexec = nullptr;
                BK(ie);
                s->g_iters = chunk;
            }
        }
        for (;;) {
            if (s->cfg.use_graph) {
                BK(cudaGraphLaunch(s->gexec, st));
                launches_counter_add(s->g_launches);
                replays++;
            } else {
                for (int q = 0; q < chunk; q++) b_iteration(s, B);
            }
            read_states(s);
            if (!any_inner_active(s)) break;
        }
        b_refine_end(B, s->dst, st);
        b_add_correction(B, s->x, s->e, s->dst, st);
    }
    BK(cudaEventRecord(s->ev1, st));
    BK(cudaEventSynchronize(s->ev1));
    read_states(s);
    float ms = 0;
    BK(cudaEventElapsedTime(&ms, s->ev0, s->ev1));
    pps_batch_stats& S = s->stats;
    std::memset(&S, 0, sizeof(S));
    S.seconds_solve = ms * 1e-3;
    S.kernel_launches = launches_counter() - l0;
    S.graph_replays = replays;
    S.max_err_true = 0;
    for (int p = 0; p < s->nprob; p++) {
        const BState& q = s->hst[p];
        const double e = q.err_outer / q.s.normb;
        S.max_err_true = std::max(S.max_err_true, e);
        S.max_iterations = std::max(S.max_iterations, q.total_iters);
        S.sum_iterations += q.total_iters;
        S.max_refinements = std::max(S.max_refinements, q.refinements);
        if (q.finished && q.outer_status == 0 && e < s->cfg.tol) S.converged++;
    }
    S.unknowns = 0;
    for (int p = 0; p < s->nprob; p++) {
        const Geo& g = s->geo[(size_t)p];
        S.unknowns += (double)(g.hi[0] - g.lo[0]) * (g.hi[1] - g.lo[1]) * (g.hi[2] - g.lo[2]);
    }
    return S.converged == s->nprob ? PPS_OK : PPS_NOT_CONVERGED;
}

// Times the batched sweep kernel over the problems of one grid shape for every
// candidate tile and keeps the fastest.
void tune_shape(pps_batch* s, long long key, const std::vector<int>& which)
{
    const int n = s->cfg.cheb_degree;
    (void)n;
    float best = 1e30f;
    SizeTile best_t;
    std::vector<BState> init((size_t)s->nprob);
    std::memset(init.data(), 0, sizeof(BState) * init.size());
    BK(cudaMemcpyAsync(s->dst, init.data(), sizeof(BState) * init.size(), cudaMemcpyHostToDevice, s->stream));
    const Geo& g0 = s->geo[(size_t)which[0]];
    const bool v4_ok = g0.sj % 4 == 0;
    float best4 = 1e30f;
    int best_kc4 = 32;
    // the one-column tiles (cx 1, 2) for every kernel, then the v4 tiles for the
    // Chebyshev kernels (kept when they beat the best one-column tile on the sweep)
    for (int cx : {1, 2, 4}) {
        if (cx == 4 && !v4_ok) break;
        for (int kc : kKchunks) {
            SizeTile t = best_t;
            if (cx == 4) {
                t.v4 = true;
                t.kchunk4 = kc;
            } else {
                t.cx = cx;
                t.kchunk = kc;
                t.v4 = false;
            }
            s->tiles[key] = t;
            const BatchDev B = build_table(s, which, true);
            s->B4 = B;
            auto launch = [&]() {
                b_cheb_sweep(B, s->Y, s->r, s->Z, s->W, s->coef, s->cstride, std::min(2, s->cstride - 1), s->dst,
                             s->stream);
            };
            launch();
            BK(cudaEventRecord(s->ev0, s->stream));
            const int reps = 10;
            for (int q = 0; q < reps; q++) launch();
            BK(cudaEventRecord(s->ev1, s->stream));
            BK(cudaEventSynchronize(s->ev1));
            float ms = 0;
            BK(cudaEventElapsedTime(&ms, s->ev0, s->ev1));
            if (cx == 4) {
                if (ms < best4) {
                    best4 = ms;
                    best_kc4 = kc;
                }
            } else if (ms < best) {
                best = ms;
                best_t = t;
            }
        }
    }
    best_t.v4 = best4 < best;
    best_t.kchunk4 = best_kc4;
    s->tiles[key] = best_t;
}

}  // namespace

extern "C" {

pps_status pps_batch_create(int nprob, const pps_grid* grids, const pps_config* cfg, pps_batch** out)
{
    if (!out || !grids || !cfg || nprob < 1) return PPS_ERR_INVALID_ARG;
    *out = nullptr;
    const bool vcycle = cfg->krylov == PPS_KRYLOV_FCG;
    if (cfg->form != PPS_FORM_MIXED ||
        (!vcycle && (cfg->krylov != PPS_KRYLOV_BICGSTAB || cfg->precond != PPS_PREC_CHEBYSHEV || cfg->cheb_degree < 4))) {
        pps_internal_set_error("batches run the MIXED form: flexible CG with the multigrid V-cycle in one persistent "
                               "launch, or BiCGSTAB + Chebyshev (degree >= 4)");
        return PPS_ERR_UNSUPPORTED;
    }
    if (!(cfg->tol > 0.0) || !(cfg->inner_tol > 0.0 && cfg->inner_tol < 1.0) || cfg->inner_maxit < 1 ||
        cfg->max_refinements < 1) {
        pps_internal_set_error("invalid tolerance or refinement settings");
        return PPS_ERR_INVALID_ARG;
    }
    for (int p = 0; p < nprob; p++) {
        const pps_grid& g = grids[p];
        for (int d = 0; d < 3; d++)
            if (g.npglobal[d] < 3 || !(g.ds[d] > 0.0)) {
                pps_internal_set_error("every grid needs npglobal >= 3 and ds > 0");
                return PPS_ERR_INVALID_ARG;
            }
        for (int f = 0; f < 6; f++)
            if (g.bcs[f] != 0) {
                pps_internal_set_error("batches take Dirichlet grids only");
                return PPS_ERR_UNSUPPORTED;
            }
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        pps_internal_set_error("no CUDA device");
        return PPS_ERR_NO_DEVICE;
    }
    pps_batch* s = new (std::nothrow) pps_batch();
    if (!s) return PPS_ERR_OUT_OF_MEMORY;
    s->nprob = nprob;
    s->grids.assign(grids, grids + nprob);
    s->cfg = *cfg;
    pps_status rc = bguard([&]() -> pps_status {
        BK(cudaSetDevice(cfg->device));
        s->device = cfg->device;
        BK(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
        BK(cudaEventCreate(&s->ev0));
        BK(cudaEventCreate(&s->ev1));
        s->geo.resize((size_t)nprob);
        s->off.resize((size_t)nprob);
        s->theta.resize((size_t)nprob);
        s->delta.resize((size_t)nprob);
        s->sigma.resize((size_t)nprob);
        long long pool = 0;
        for (int p = 0; p < nprob; p++) {
            const pps_grid& gr = grids[p];
            Geo& g = s->geo[(size_t)p];
            for (int d = 0; d < 3; d++) {
                g.n[d] = gr.npglobal[d];
                g.ds[d] = gr.ds[d];
                g.lo[d] = 2;
                g.hi[d] = gr.npglobal[d];
            }
            for (int f = 0; f < 6; f++) g.bcs[f] = 0;
            g.sj = gr.npglobal[0] + 2;
            g.sk = g.sj * (gr.npglobal[1] + 2);
            g.ntot = g.sk * (gr.npglobal[2] + 2);
            s->off[(size_t)p] = pool;
            pool += (g.ntot + 31) / 32 * 32;   // 256-byte aligned starts for the FP64 pools
            // eigenvalue bounds and Chebyshev parameters of this grid (blockGrid.hpp:322-339,
            // chebyshevIteration.hpp:22-26)
            double eigMin = 0, eigMax = 0;
            for (int i = 0; i < 3; i++) {
                const int ni = gr.npglobal[i] - 2;
                eigMin += 4 * sin(1 * kPi / 2 / (ni + 1)) * sin(1 * kPi / 2 / (ni + 1)) / (gr.ds[i] * gr.ds[i]);
                eigMax += 4 * sin(ni * kPi / 2 / (ni + 1)) * sin(ni * kPi / 2 / (ni + 1)) / (gr.ds[i] * gr.ds[i]);
            }
            const double th = (eigMin * cfg->rescale_min + eigMax * cfg->rescale_max) * 0.5 * (1.0 + cfg->cheb_eps);
            const double de = (eigMin * cfg->rescale_min - eigMax * cfg->rescale_max) * 0.5;
            s->theta[(size_t)p] = th;
            s->delta[(size_t)p] = de;
            s->sigma[(size_t)p] = th / de;
            s->tiles[key_of(g)] = SizeTile();
        }
        s->pool = pool;
        BK(cudaMalloc((void**)&s->x, sizeof(double) * (size_t)pool));
        BK(cudaMalloc((void**)&s->b, sizeof(double) * (size_t)pool));
        BK(cudaMemsetAsync(s->x, 0, sizeof(double) * (size_t)pool, s->stream));
        BK(cudaMemsetAsync(s->b, 0, sizeof(double) * (size_t)pool, s->stream));
        float** f32[] = {&s->p, &s->r, &s->r0, &s->Mp, &s->AMp, &s->z, &s->Az, &s->Y, &s->Z, &s->W, &s->e};
        for (float** q : f32) {
            BK(cudaMalloc((void**)q, sizeof(float) * (size_t)pool));
            BK(cudaMemsetAsync(*q, 0, sizeof(float) * (size_t)pool, s->stream));
        }
        BK(cudaMalloc((void**)&s->dprob, sizeof(BProb) * (size_t)nprob));
        BK(cudaMalloc((void**)&s->dprob4, sizeof(BProb) * (size_t)nprob));
        BK(cudaMalloc((void**)&s->counters, sizeof(unsigned) * (size_t)nprob));
        BK(cudaMemsetAsync(s->counters, 0, sizeof(unsigned) * (size_t)nprob, s->stream));
        BK(cudaMalloc((void**)&s->dst, sizeof(BState) * (size_t)nprob));
        BK(cudaMallocHost((void**)&s->hst, sizeof(BState) * (size_t)nprob));
        if (vcycle) {   // flexible CG + V-cycle in one persistent launch (pps_bvcycle.cu)
            const BvcPools pools{s->x, s->b, s->r, s->z, s->p, s->r0, s->AMp, s->e, s->Y, s->Z, s->W};
            std::string err;
            if (!bvc_create(&s->vc, nprob, s->geo.data(), s->off.data(), pools, cfg->tol, cfg->inner_tol,
                            cfg->inner_maxit, cfg->max_refinements, s->stream, err)) {
                pps_internal_set_error(err.c_str());
                return err.find("cuda") != std::string::npos ? PPS_ERR_CUDA : PPS_ERR_UNSUPPORTED;
            }
            return PPS_OK;
        }
        s->cstride = cfg->cheb_degree - 2;
        std::vector<Coef> hc((size_t)nprob * s->cstride);
        for (int p = 0; p < nprob; p++) coefs_of(s, p, &hc[(size_t)p * s->cstride]);
        std::vector<unsigned char> dev(hc.size() * b_coef_size());
        b_cast_coef(hc.data(), dev.data(), hc.size());
        BK(cudaMalloc(&s->coef, dev.size()));
        BK(cudaMemcpyAsync(s->coef, dev.data(), dev.size(), cudaMemcpyHostToDevice, s->stream));
        BK(cudaStreamSynchronize(s->stream));
        return PPS_OK;
    });
    if (rc != PPS_OK) {
        free_batch(s);
        delete s;
        return rc;
    }
    *out = s;
    return PPS_OK;
}

pps_status pps_batch_destroy(pps_batch* s)
{
    if (!s) return PPS_ERR_INVALID_ARG;
    cudaSetDevice(s->device);
    cudaStreamSynchronize(s->stream);
    free_batch(s);
    delete s;
    return PPS_OK;
}

pps_status pps_batch_field_device(pps_batch* s, int p, double** x_dev, double** b_dev)
{
    if (!s || p < 0 || p >= s->nprob) return PPS_ERR_INVALID_ARG;
    if (x_dev) *x_dev = s->x + s->off[(size_t)p];
    if (b_dev) *b_dev = s->b + s->off[(size_t)p];
    return PPS_OK;
}

pps_status pps_batch_set(pps_batch* s, int p, const double* x, const double* b)
{
    if (!s || p < 0 || p >= s->nprob || !x || !b) return PPS_ERR_INVALID_ARG;
    return bguard([&]() -> pps_status {
        BK(cudaSetDevice(s->device));
        const size_t n = (size_t)s->geo[(size_t)p].ntot;
        BK(cudaMemcpyAsync(s->x + s->off[(size_t)p], x, sizeof(double) * n, cudaMemcpyHostToDevice, s->stream));
        BK(cudaMemcpyAsync(s->b + s->off[(size_t)p], b, sizeof(double) * n, cudaMemcpyHostToDevice, s->stream));
        BK(cudaStreamSynchronize(s->stream));
        return PPS_OK;
    });
}

pps_status pps_batch_get(pps_batch* s, int p, double* x, pps_stats* st)
{
    if (!s || p < 0 || p >= s->nprob) return PPS_ERR_INVALID_ARG;
    return bguard([&]() -> pps_status {
        BK(cudaSetDevice(s->device));
        if (x) {
            const size_t n = (size_t)s->geo[(size_t)p].ntot;
            BK(cudaMemcpyAsync(x, s->x + s->off[(size_t)p], sizeof(double) * n, cudaMemcpyDeviceToHost, s->stream));
            BK(cudaStreamSynchronize(s->stream));
        }
        if (st && s->vc) {
            std::memset(st, 0, sizeof(*st));
            bvc_result(s->vc, p, st);
            st->seconds_solve = s->stats.seconds_solve;
        } else if (st) {
            std::memset(st, 0, sizeof(*st));
            const BState& q = s->hst[p];
            st->iterations = q.total_iters;
            st->refinements = q.refinements;
            st->norm_b = q.s.normb;
            st->err_true = q.s.normb > 0 ? q.err_outer / q.s.normb : -1.0;
            st->seconds_solve = s->stats.seconds_solve;
        }
        return PPS_OK;
    });
}

pps_status pps_batch_solve(pps_batch* s, pps_batch_stats* stats)
{
    if (!s) return PPS_ERR_INVALID_ARG;
    pps_status rc = bguard([&]() -> pps_status {
        BK(cudaSetDevice(s->device));
        if (s->vc) {
            std::string err;
            const pps_status r = bvc_solve(s->vc, s->stream, s->ev0, s->ev1, &s->stats, err);
            if (!err.empty()) pps_internal_set_error(err.c_str());
            return r;
        }
        return run_batch(s);
    });
    if (stats) *stats = s->stats;
    return rc;
}

pps_status pps_batch_set_wait_limit(pps_batch* s, double seconds)
{
    if (!s || !(seconds > 0.0) || !std::isfinite(seconds)) return PPS_ERR_INVALID_ARG;
    if (!s->vc) {
        pps_internal_set_error("only the persistent (flexible CG) batch waits on a grid barrier");
        return PPS_ERR_UNSUPPORTED;
    }
    bvc_set_wait_limit(s->vc, seconds);
    return PPS_OK;
}

pps_status pps_batch_autotune(pps_batch* s)
{
    if (!s) return PPS_ERR_INVALID_ARG;
    if (s->vc) return PPS_OK;   // the persistent solve's work items have a fixed shape
    return bguard([&]() -> pps_status {
        BK(cudaSetDevice(s->device));
        std::map<long long, std::vector<int>> groups;
        for (int p = 0; p < s->nprob; p++) groups[key_of(s->geo[(size_t)p])].push_back(p);
        for (auto& kv : groups) tune_shape(s, kv.first, kv.second);
        if (s->gexec) {
            cudaGraphExecDestroy(s->gexec);
            s->gexec = nullptr;
        }
        return PPS_OK;
    });
}

pps_status pps_batch_tile(const pps_batch* s, int p, int* cx, int* kchunk)
{
    if (!s || p < 0 || p >= s->nprob) return PPS_ERR_INVALID_ARG;
    auto it = s->tiles.find(key_of(s->geo[(size_t)p]));
    if (it == s->tiles.end()) return PPS_ERR_INVALID_ARG;
    const bool v4 = it->second.v4 && s->geo[(size_t)p].sj % 4 == 0;   // the Chebyshev kernels' tile
    if (cx) *cx = v4 ? 4 : it->second.cx;
    if (kchunk) *kchunk = v4 ? it->second.kchunk4 : it->second.kchunk;
    return PPS_OK;
}

}  // extern "C"
