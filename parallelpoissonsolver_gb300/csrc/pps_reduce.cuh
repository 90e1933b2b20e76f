// Device-side reductions shared by the solver kernels and the learned cycle's
// transfer kernels: exact-product accumulators, the deterministic block/grid
// reduction whose last block advances the Krylov scalars (finalize), and the
// early exit of kernels launched after the stop flag was set.
#pragma once
#include "pps_internal.h"

#include <cuda_runtime.h>
#include <math.h>

namespace pps {

// Fused multiply-add for either storage type.
__device__ __forceinline__ float fmx(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fmx(double a, double b, double c) { return __fma_rn(a, b, c); }

// Accumulator of exact products: FP64 FMA for double data; for float data a
// double-float pair (Dekker/Knuth error-free product and sum in FP32), so the
// inner products of the mixed form are FP64-accurate without FP64 arithmetic
// per point (GB300 runs FP64 at 1/64 of the FP32 rate).
template <typename T>
struct Acc;
template <>
struct Acc<double> {
    double s = 0.0;
    __device__ __forceinline__ void add(double a, double b) { s = fmx(a, b, s); }
    __device__ __forceinline__ double value() const { return s; }
};
template <>
struct Acc<float> {
    float hi = 0.f, lo = 0.f;
    __device__ __forceinline__ void add(float a, float b)
    {
        const float p = __fmul_rn(a, b);
        const float e = __fmaf_rn(a, b, -p);
        const float s = __fadd_rn(hi, p);
        const float bb = __fsub_rn(s, hi);
        const float t = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(p, bb));
        hi = s;
        lo = __fadd_rn(lo, __fadd_rn(t, e));
    }
    __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

static __device__ void finalize(const RedCtx& rc, const double* tot)
{
    DevState* st = rc.st;
    for (int q = 0; q < 4; q++) st->sums[q] = tot[q];
    switch (rc.kind) {
    case FIN_NORMB:
        st->normb = sqrt(tot[0]);
        break;
    case FIN_RES0: {
        const double e0 = sqrt(tot[0]);
        st->err0 = e0;
        st->err = e0;
        if (rc.hist && st->hist_cap > 0) rc.hist[0] = e0 * st->hist_scale;
        st->rho0 = st->rho0_from_r ? tot[0] : st->normb * st->normb;
        st->iter = 0;
        if (!(e0 == e0) || isinf(e0)) {
            st->status = 3;
            st->done = 1;
        } else if (e0 < st->tol_abs) {
            st->status = 0;
            st->done = 1;
        } else {
            st->done = 0;
            st->status = 0;
            // inner solve of a refinement step: reduce by tol_rel, or less if enough
            if (st->tol_relative) st->tol_abs = fmax(st->tol_rel, 0.3 * st->tol_abs / e0) * e0;
        }
        break;
    }
    case FIN_ALPHA: {
        const double a = st->rho0 / tot[0];
        st->alpha = a;
        if (!isfinite(a)) {
            st->status = 2;
            st->done = 1;
        }
        break;
    }
    case FIN_OMEGA: {
        const double w = tot[0] / tot[1];
        st->omega = w;
        if (!isfinite(w) || w == 0.0) {
            st->status = 2;
            st->done = 1;
        }
        break;
    }
    case FIN_CONV: {
        const double err = sqrt(tot[1]);
        const double rho1 = tot[0];
        st->err = err;
        st->beta = rho1 / st->rho0 * st->alpha / st->omega;
        st->rho0 = rho1;
        st->iter += 1;
        if (rc.hist && st->iter < st->hist_cap) rc.hist[st->iter] = err * st->hist_scale;
        if (!isfinite(err)) {
            st->status = 3;
            st->done = 1;
        } else if (err < st->tol_abs) {
            st->status = 0;
            st->done = 1;
        } else if (st->iter >= st->maxit) {
            st->status = 1;
            st->done = 1;
        } else if (!isfinite(st->beta)) {
            st->status = 2;
            st->done = 1;
        }
        break;
    }
    case FIN_CG_ALPHA: {
        st->rho0 = tot[0];                    // r.z
        st->alpha = tot[0] / tot[1];          // r.z / p.Ap
        if (!isfinite(st->alpha)) {
            st->status = 2;
            st->done = 1;
        }
        break;
    }
    case FIN_CG_CONV: {
        const double err = sqrt(tot[1]);
        st->err = err;
        st->beta = tot[0] / st->rho0;         // r_new.z_new / r.z
        st->iter += 1;
        if (rc.hist && st->iter < st->hist_cap) rc.hist[st->iter] = err * st->hist_scale;
        if (!isfinite(err)) {
            st->status = 3;
            st->done = 1;
        } else if (err < st->tol_abs) {
            st->status = 0;
            st->done = 1;
        } else if (st->iter >= st->maxit) {
            st->status = 1;
            st->done = 1;
        }
        break;
    }
    case FIN_FCG_ALPHA: {
        st->alpha = st->rho0 / tot[0];        // z.r / p.Ap
        if (!isfinite(st->alpha)) {
            st->status = 2;
            st->done = 1;
        }
        break;
    }
    case FIN_FCG_SETUP: {
        st->rho0 = tot[0];                    // z.r
        st->beta = 0.0;
        break;
    }
    case FIN_FCG_RES: {
        // flexible CG after x, r: the recursive residual norm and the stop test
        const double err = sqrt(tot[0]);
        st->err = err;
        st->iter += 1;
        if (rc.hist && st->iter < st->hist_cap) rc.hist[st->iter] = err * st->hist_scale;
        if (!isfinite(err)) {
            st->status = 3;
            st->done = 1;
        } else if (err < st->tol_abs) {
            st->status = 0;
            st->done = 1;
        } else if (st->iter >= st->maxit) {
            st->status = 1;
            st->done = 1;
        }
        break;
    }
    case FIN_FCG_CONV: {
        // flexible CG, Polak-Ribiere: beta = z_new.(r_new - r_old) / (z_old.r_old)
        // with r_new - r_old = -alpha Ap
        st->beta = -st->alpha * tot[1] / st->rho0;
        st->rho0 = tot[0];
        if (!isfinite(st->beta)) {
            st->status = 2;
            st->done = 1;
        }
        break;
    }
    default:
        break;
    }
}

// Block reduction of NS partial sums, then the last block reduces all block
// partials in block order and runs the finalizer.  Every thread of every block
// must call this (inactive threads pass zeros).
template <int NS>
__device__ __forceinline__ void reduce_finalize(double (&v)[NS], const RedCtx& rc)
{
    __shared__ double sm[32][NS];
    __shared__ int is_last;
    const int tid = threadIdx.x + blockDim.x * threadIdx.y;
    const int nthr = blockDim.x * blockDim.y;
    const int lane = tid & 31, warp = tid >> 5, nwarp = (nthr + 31) >> 5;
    const unsigned nblocks = gridDim.x * gridDim.y;
    const unsigned bid = blockIdx.x + gridDim.x * blockIdx.y;
#pragma unroll
    for (int q = 0; q < NS; q++) {
        const double w = warp_sum(v[q]);
        if (lane == 0) sm[warp][q] = w;
    }
    __syncthreads();
    if (tid == 0) {
#pragma unroll
        for (int q = 0; q < NS; q++) {
            double s = 0.0;
            for (int w = 0; w < nwarp; w++) s += sm[w][q];
            rc.partials[(size_t)bid * 4 + q] = s;
        }
        __threadfence();
        const unsigned ticket = atomicAdd(rc.counter, 1u);
        is_last = (ticket == nblocks - 1);
    }
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    double acc[NS];
#pragma unroll
    for (int q = 0; q < NS; q++) acc[q] = 0.0;
    for (unsigned b = tid; b < nblocks; b += nthr) {
#pragma unroll
        for (int q = 0; q < NS; q++) acc[q] += __ldcg(&rc.partials[(size_t)b * 4 + q]);
    }
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
            double s = 0.0;
            for (int w = 0; w < nwarp; w++) s += sm[w][q];
            tot[q] = s;
        }
        finalize(rc, tot);
        __threadfence();
        *rc.counter = 0u;
    }
}

// The end of a z-marching kernel on the one-column tiles: the deterministic block
// reduction above, or, with canonical sums, one partial per warp stored as its cell
// (every lane calls it; rows past the last unknown own no cell).
template <int NS>
__device__ __forceinline__ void reduce_emit(double (&v)[NS], const RedCtx& rc, const Shape& sh)
{
    if (rc.cells == nullptr) {
        reduce_finalize<NS>(v, rc);
        return;
    }
    const int bx = blockIdx.x % sh.ntx;
    const int row = (blockIdx.x / sh.ntx) * sh.ty + threadIdx.y;
    double w[NS];
#pragma unroll
    for (int q = 0; q < NS; q++) w[q] = warp_sum(v[q]);
    if (row < rc.cell_ny && threadIdx.x == 0) {
        const long long cell = ((long long)blockIdx.y * rc.cell_ny + row) * rc.cell_ntx + bx;
#pragma unroll
        for (int q = 0; q < NS; q++) rc.cells[q * rc.cell_n + cell] = w[q];
    }
}

#define EARLY_EXIT(done)                                      \
    if (done != nullptr && *(volatile const int*)(done) != 0) return;

}  // namespace pps
