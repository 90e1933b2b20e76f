// Kernels of the learned preconditioner: a 3-D convolutional U-Net with BF16 weights
// and activations and FP32 accumulation, plus the grid-transfer kernels that move a
// solver field to the network's grid and back.  No reference counterpart.
//
// Activations are channels-last: act[((z*H + y)*W + x)*ld + c0 + c], BF16, where a
// tensor may occupy a channel slot [c0, c0+C) of a wider buffer (the U-Net's skip
// concatenations).  Convolutions are 3x3x3, zero-padded, stride 1, as implicit
// GEMMs on the tensor cores: M = voxels, N = output channels, K = 27 taps x input
// channels, 16x16x16 BF16 fragments with FP32 accumulators.
#include "pps_unet_internal.h"
#include "pps_reduce.cuh"

#include <algorithm>
#include <cmath>
#include <type_traits>

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <mma.h>

namespace pps {
namespace unet {

// The stop flag the forward and transfer kernels check on entry: a solver sets it to
// its device stop flag while it runs the learned cycle, so a cycle launched (or
// replayed) after the iteration converged costs no more than its launches.
static thread_local const int* g_stop = nullptr;
void set_stop_flag(const int* done) { g_stop = done; }

using namespace nvcuda;
typedef __nv_bfloat16 bf16;

constexpr int TILE_V = 64;   // voxels (along x) per conv block: 4 warps x 16

// ---------------------------------------------------------------------------
// Convolution, forward: Y[v][co] = act(bias[co] + sum_tap sum_ci X[v+off(tap)][ci] W[tap][ci][co])
// Cin, Cout multiples of 16.  One block: one 16 x 16 output fragment (16 consecutive
// voxels in (z, y, x) order, 16 output channels).  The K = 27 * Cin/16 steps of
// 16 x 16 x 16 are dealt round-robin to the NW warps, so each warp's dependent chain
// is 1/NW of K (the grids are small: at 16^3 and below latency, not the tensor pipe,
// is the limit; the deep layers run 54-162 steps on 16-64 blocks).  Each warp stages
// its A tile in its own shared slot (warp-level sync only) and prefetches the next
// step's A tile and weight fragment into registers while the current step's
// multiply-add runs; the NW partial fragments are summed at the end.
// ---------------------------------------------------------------------------
constexpr int CONV_V = 16;   // voxels per block

template <bool RELU, bool OUT_F32, int NW>
__global__ void __launch_bounds__(32 * NW) k_conv(Dims d, const bf16* __restrict__ X, int ldx, int cx0, int Cin,
                                                  const bf16* __restrict__ Wt, const float* __restrict__ bias,
                                                  void* __restrict__ Yv, int ldy, int cy0, int Cout,
                                                  const int* __restrict__ stop, ConvIO io)
{
    pdl_enter();
    if (stop && *(volatile const int*)stop) return;
    __shared__ __align__(32) bf16 sA[NW][CONV_V * 16];
    __shared__ __align__(32) float sC[NW][16 * 16];
    const long long nvox = (long long)d.D * d.H * d.W;
    const long long v0 = (long long)blockIdx.x * CONV_V;
    const int co0 = blockIdx.y * 16;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // this lane's voxel row of the A tile and its 8-channel half
    const int va = lane >> 1, ha = lane & 1;
    const long long lva = v0 + va;
    const bool va_in = lva < nvox;
    const int xa = (int)(lva % d.W), ya = (int)((lva / d.W) % d.H), za = (int)(lva / ((long long)d.W * d.H));
    const int csteps = Cin / 16, ksteps = 27 * csteps;
    const float in_sc = io.dense_in && io.rms ? (*io.rms > 0.0f ? 1.0f / *io.rms : 0.0f) : 1.0f;
    const int Hc = d.H / 2, Wc = d.W / 2;
    auto load_a = [&](int t) -> uint4 {
        const int tap = t / csteps, c0 = (t - tap * csteps) * 16;
        const int zz = za + tap / 9 - 1, yy = ya + (tap / 3) % 3 - 1, xx = xa + tap % 3 - 1;
        uint4 val = make_uint4(0, 0, 0, 0);
        if (va_in && zz >= 0 && zz < d.D && yy >= 0 && yy < d.H && xx >= 0 && xx < d.W) {
            const long long vox = ((long long)zz * d.H + yy) * d.W + xx;
            if (io.dense_in) {   // channel 0 of the first 16 (Cin = 16): the scaled dense input
                if (ha == 0) val.x = (unsigned)__bfloat16_as_ushort(__float2bfloat16(io.dense_in[vox] * in_sc));
            } else if (c0 < io.c_up) {   // the upsampled channels, read at the coarse voxel
                const long long cv = ((long long)(zz >> 1) * Hc + (yy >> 1)) * Wc + (xx >> 1);
                val = *reinterpret_cast<const uint4*>(io.up + cv * io.ld_up + c0 + 8 * ha);
            } else {
                val = *reinterpret_cast<const uint4*>(X + vox * ldx + cx0 + c0 + 8 * ha);
            }
        }
        return val;
    };
    auto w_at = [&](int t) {
        const int tap = t / csteps, c0 = (t - tap * csteps) * 16;
        return Wt + ((long long)tap * Cin + c0) * Cout + co0;
    };
    wmma::fragment<wmma::accumulator, 16, 16, 16, float> acc;
    wmma::fill_fragment(acc, 0.0f);
    wmma::fragment<wmma::matrix_b, 16, 16, 16, bf16, wmma::row_major> bcur, bnext;
    int t = warp;
    uint4 next = t < ksteps ? load_a(t) : make_uint4(0, 0, 0, 0);
    if (t < ksteps) wmma::load_matrix_sync(bnext, w_at(t), Cout);
    for (; t < ksteps; t += NW) {
        *reinterpret_cast<uint4*>(&sA[warp][va * 16 + 8 * ha]) = next;
        bcur = bnext;
        __syncwarp();
        if (t + NW < ksteps) {
            next = load_a(t + NW);
            wmma::load_matrix_sync(bnext, w_at(t + NW), Cout);
        }
        wmma::fragment<wmma::matrix_a, 16, 16, 16, bf16, wmma::row_major> a;
        wmma::load_matrix_sync(a, sA[warp], 16);
        wmma::mma_sync(acc, a, bcur, acc);
        __syncwarp();
    }
    wmma::store_matrix_sync(sC[warp], acc, 16, wmma::mem_row_major);
    __syncthreads();
    for (int q = threadIdx.x; q < CONV_V * 16; q += 32 * NW) {
        const int v = q >> 4, co = q & 15;
        if (v0 + v >= nvox) continue;
        float val = 0.0f;
#pragma unroll
        for (int w = 0; w < NW; w++) val += sC[w][q];
        val += bias ? bias[co0 + co] : 0.0f;
        if (RELU) val = fmaxf(val, 0.0f);
        if (io.dense_out) {   // channel 0 only, scaled back
            if (co0 + co == 0) io.dense_out[v0 + v] = val * ((io.rms ? *io.rms : 1.0f) * io.gain);
            continue;
        }
        const long long o = (v0 + v) * ldy + cy0 + co0 + co;
        if (OUT_F32) reinterpret_cast<float*>(Yv)[o] = val;
        else reinterpret_cast<bf16*>(Yv)[o] = __float2bfloat16(val);
    }
}

template <int NW>
static void conv_nw(const dim3& grid, const Dims& d, const bf16* X, int ldx, int cx0, int Cin, const bf16* W,
                    const float* bias, void* Y, int ldy, int cy0, int Cout, bool relu, bool out_f32, cudaStream_t s,
                    const ConvIO& io)
{
    const dim3 block(32 * NW);
    if (out_f32) {
        if (relu) launch_pdl(k_conv<true, true, NW>, grid, block, 0, s, d, X, ldx, cx0, Cin, W, bias, Y, ldy, cy0, Cout, g_stop, io);
        else launch_pdl(k_conv<false, true, NW>, grid, block, 0, s, d, X, ldx, cx0, Cin, W, bias, Y, ldy, cy0, Cout, g_stop, io);
    } else {
        if (relu) launch_pdl(k_conv<true, false, NW>, grid, block, 0, s, d, X, ldx, cx0, Cin, W, bias, Y, ldy, cy0, Cout, g_stop, io);
        else launch_pdl(k_conv<false, false, NW>, grid, block, 0, s, d, X, ldx, cx0, Cin, W, bias, Y, ldy, cy0, Cout, g_stop, io);
    }
}

void conv(const Dims& d, const bf16* X, int ldx, int cx0, int Cin, const bf16* W, const float* bias, void* Y, int ldy,
          int cy0, int Cout, bool relu, bool out_f32, cudaStream_t s, const ConvIO& io)
{
    const dim3 grid((unsigned)(((long long)d.D * d.H * d.W + CONV_V - 1) / CONV_V), (unsigned)(Cout / 16));
    // warps per block: enough that each warp's chain of K steps stays short
    const int ksteps = 27 * (Cin / 16);
    if (ksteps >= 64) conv_nw<16>(grid, d, X, ldx, cx0, Cin, W, bias, Y, ldy, cy0, Cout, relu, out_f32, s, io);
    else conv_nw<8>(grid, d, X, ldx, cx0, Cin, W, bias, Y, ldy, cy0, Cout, relu, out_f32, s, io);
    launches_counter_add(1);
}

// ---------------------------------------------------------------------------
// Weight gradient: dW[tap][ci][co] += sum_v X[v+off(tap)][ci] * dY[v][co]
// One block per (tap, z-plane): a GEMM with K = the plane's voxels, accumulated in
// fragments and added to the FP32 gradient with atomics.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_conv_wgrad(Dims d, const bf16* __restrict__ X, int ldx, int cx0, int Cin,
                                                    const bf16* __restrict__ G, int ldg, int cg0, int Cout,
                                                    float* __restrict__ dW)
{
    pdl_enter();
    __shared__ __align__(32) bf16 sX[TILE_V * 96];    // 64 voxels x Cin   (col-major A: ci x v)
    __shared__ __align__(32) bf16 sG[TILE_V * 96];    // 64 voxels x Cout  (row-major B: v x co)
    __shared__ __align__(32) float sC[96 * 96 / 4];   // staging of one warp's fragments
    const int tap = blockIdx.x % 27;
    const int z = blockIdx.x / 27;
    const int dz = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
    const int tid = threadIdx.x, warp = tid >> 5;
    const int mi = Cin / 16, ni = Cout / 16, nf = mi * ni;   // fragment pairs, split over warps
    wmma::fragment<wmma::accumulator, 16, 16, 16, float> acc[9];
#pragma unroll
    for (int f = 0; f < 9; f++) wmma::fill_fragment(acc[f], 0.0f);
    const int zz = z + dz;
    const bool plane_ok = zz >= 0 && zz < d.D;
    if (plane_ok) {
        const int ntx = (d.W + TILE_V - 1) / TILE_V;
        for (int y = 0; y < d.H; y++) {
            const int yy = y + dy;
            const bool row_ok = yy >= 0 && yy < d.H;
            if (!row_ok) continue;
            for (int xt = 0; xt < ntx; xt++) {
                const int x0 = xt * TILE_V;
                for (int q = tid; q < TILE_V * Cin / 8; q += 128) {
                    const int v = q / (Cin / 8), c8 = q % (Cin / 8);
                    const int xx = x0 + v + dx;
                    uint4 val = make_uint4(0, 0, 0, 0);
                    if (x0 + v < d.W && xx >= 0 && xx < d.W)
                        val = *reinterpret_cast<const uint4*>(X + ((long long)(zz * d.H + yy) * d.W + xx) * ldx + cx0 + 8 * c8);
                    *reinterpret_cast<uint4*>(&sX[v * 96 + 8 * c8]) = val;
                }
                for (int q = tid; q < TILE_V * Cout / 8; q += 128) {
                    const int v = q / (Cout / 8), c8 = q % (Cout / 8);
                    uint4 val = make_uint4(0, 0, 0, 0);
                    if (x0 + v < d.W)
                        val = *reinterpret_cast<const uint4*>(G + ((long long)(z * d.H + y) * d.W + x0 + v) * ldg + cg0 + 8 * c8);
                    *reinterpret_cast<uint4*>(&sG[v * 96 + 8 * c8]) = val;
                }
                __syncthreads();
                for (int k = 0; k < TILE_V; k += 16) {
#pragma unroll
                    for (int f = 0; f < 9; f++) {
                        const int pair = warp + 4 * f;
                        if (pair < nf) {
                            const int m = pair / ni, n = pair % ni;
                            wmma::fragment<wmma::matrix_a, 16, 16, 16, bf16, wmma::col_major> a;
                            wmma::fragment<wmma::matrix_b, 16, 16, 16, bf16, wmma::row_major> b;
                            wmma::load_matrix_sync(a, sX + k * 96 + m * 16, 96);
                            wmma::load_matrix_sync(b, sG + k * 96 + n * 16, 96);
                            wmma::mma_sync(acc[f], a, b, acc[f]);
                        }
                    }
                }
                __syncthreads();
            }
        }
    }
    // accumulate into dW[tap][ci][co], one warp at a time through the staging tile
    for (int w = 0; w < 4; w++) {
        if (warp == w) {
#pragma unroll
            for (int f = 0; f < 9; f++) {
                const int pair = warp + 4 * f;
                if (pair < nf) {
                    const int m = pair / ni, n = pair % ni;
                    wmma::store_matrix_sync(sC, acc[f], 16, wmma::mem_row_major);
                    __syncwarp();
                    for (int q = tid & 31; q < 256; q += 32) {
                        const int r = q / 16, c = q % 16;
                        const float v = sC[q];
                        if (v != 0.0f) atomicAdd(&dW[((long long)tap * Cin + m * 16 + r) * Cout + n * 16 + c], v);
                    }
                    __syncwarp();
                }
            }
        }
        __syncthreads();
    }
}

void conv_wgrad(const Dims& d, const bf16* X, int ldx, int cx0, int Cin, const bf16* G, int ldg, int cg0, int Cout,
                float* dW, cudaStream_t s)
{
    launch_pdl(k_conv_wgrad, (unsigned)(27 * d.D), 128, 0, s, d, X, ldx, cx0, Cin, G, ldg, cg0, Cout, dW);
    launches_counter_add(1);
}

// db[co] += sum_v G[v][co]
__global__ void k_bias_grad(long long nv, const bf16* __restrict__ G, int ldg, int cg0, int Cout, float* __restrict__ db)
{
    pdl_enter();
    __shared__ float s[96];
    for (int c = threadIdx.x; c < Cout; c += blockDim.x) s[c] = 0.0f;
    __syncthreads();
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < nv * Cout;
         q += (long long)gridDim.x * blockDim.x) {
        const long long v = q / Cout;
        const int c = (int)(q % Cout);
        atomicAdd(&s[c], __bfloat162float(G[v * ldg + cg0 + c]));
    }
    __syncthreads();
    for (int c = threadIdx.x; c < Cout; c += blockDim.x) atomicAdd(&db[c], s[c]);
}

void bias_grad(long long nv, const bf16* G, int ldg, int cg0, int Cout, float* db, cudaStream_t s)
{
    long long blocks = (nv * Cout + 255) / 256;
    if (blocks > 1024) blocks = 1024;
    launch_pdl(k_bias_grad, (unsigned)blocks, 256, 0, s, nv, G, ldg, cg0, Cout, db);
    launches_counter_add(1);
}

// G[v][c] *= (Y[v][c] > 0): ReLU backward through the layer's own output.
__global__ void k_relu_bwd(long long nv, bf16* __restrict__ G, int ldg, int cg0, const bf16* __restrict__ Y, int ldy,
                           int cy0, int C)
{
    pdl_enter();
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < nv * C; q += (long long)gridDim.x * blockDim.x) {
        const long long v = q / C;
        const int c = (int)(q % C);
        if (!(__bfloat162float(Y[v * ldy + cy0 + c]) > 0.0f)) G[v * ldg + cg0 + c] = __float2bfloat16(0.0f);
    }
}

static unsigned eblocks(long long n)
{
    long long b = (n + 255) / 256;
    if (b > sm_count() * 32LL) b = sm_count() * 32LL;
    if (b < 1) b = 1;
    return (unsigned)b;
}

void relu_bwd(long long nv, bf16* G, int ldg, int cg0, const bf16* Y, int ldy, int cy0, int C, cudaStream_t s)
{
    launch_pdl(k_relu_bwd, eblocks(nv * C), 256, 0, s, nv, G, ldg, cg0, Y, ldy, cy0, C);
    launches_counter_add(1);
}

// 2x average pooling: out (D/2,H/2,W/2) dense C channels <- in slot of ldi
__global__ void k_pool2(Dims dout, const bf16* __restrict__ in, int ldi, int ci0, bf16* __restrict__ out, int C, const int* __restrict__ stop)
{
    pdl_enter();
    if (stop && *(volatile const int*)stop) return;
    const long long n = (long long)dout.D * dout.H * dout.W * C;
    const int Hi = dout.H * 2, Wi = dout.W * 2;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(q % C);
        const long long v = q / C;
        const int x = (int)(v % dout.W), y = (int)((v / dout.W) % dout.H), z = (int)(v / ((long long)dout.W * dout.H));
        float s = 0.0f;
        for (int o = 0; o < 8; o++) {
            const int zz = 2 * z + (o >> 2), yy = 2 * y + ((o >> 1) & 1), xx = 2 * x + (o & 1);
            s += __bfloat162float(in[((long long)(zz * Hi + yy) * Wi + xx) * ldi + ci0 + c]);
        }
        out[q] = __float2bfloat16(0.125f * s);
    }
}

void pool2(const Dims& dout, const bf16* in, int ldi, int ci0, bf16* out, int C, cudaStream_t s)
{
    launch_pdl(k_pool2, eblocks((long long)dout.D * dout.H * dout.W * C), 256, 0, s, dout, in, ldi, ci0, out, C, g_stop);
    launches_counter_add(1);
}

// pooling backward: gin slot (fine) += g_out/8 at each of the 8 children
__global__ void k_pool2_bwd(Dims dout, const bf16* __restrict__ gout, bf16* __restrict__ gin, int ldi, int ci0, int C)
{
    pdl_enter();
    const int Hi = dout.H * 2, Wi = dout.W * 2;
    const long long n = (long long)dout.D * 8 * dout.H * dout.W * C;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(q % C);
        const long long vf = q / C;
        const int xx = (int)(vf % Wi), yy = (int)((vf / Wi) % Hi), zz = (int)(vf / ((long long)Wi * Hi));
        const long long vc = ((long long)(zz / 2) * dout.H + yy / 2) * dout.W + xx / 2;
        bf16* p = gin + vf * ldi + ci0 + c;
        *p = __float2bfloat16(__bfloat162float(*p) + 0.125f * __bfloat162float(gout[vc * C + c]));
    }
}

void pool2_bwd(const Dims& dout, const bf16* gout, bf16* gin, int ldi, int ci0, int C, cudaStream_t s)
{
    launch_pdl(k_pool2_bwd, eblocks((long long)dout.D * 8 * dout.H * dout.W * C), 256, 0, s, dout, gout, gin, ldi, ci0, C);
    launches_counter_add(1);
}

// nearest 2x upsampling: out slot (fine) <- in dense (coarse)
__global__ void k_up2(Dims dfine, const bf16* __restrict__ in, int C, bf16* __restrict__ out, int ldo, int co0, const int* __restrict__ stop)
{
    pdl_enter();
    if (stop && *(volatile const int*)stop) return;
    const long long n = (long long)dfine.D * dfine.H * dfine.W * C;
    const int Hc = dfine.H / 2, Wc = dfine.W / 2;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(q % C);
        const long long v = q / C;
        const int x = (int)(v % dfine.W), y = (int)((v / dfine.W) % dfine.H), z = (int)(v / ((long long)dfine.W * dfine.H));
        out[v * ldo + co0 + c] = in[((long long)(z / 2) * Hc + y / 2) * Wc * C + (long long)(x / 2) * C + c];
    }
}

void up2(const Dims& dfine, const bf16* in, int C, bf16* out, int ldo, int co0, cudaStream_t s)
{
    launch_pdl(k_up2, eblocks((long long)dfine.D * dfine.H * dfine.W * C), 256, 0, s, dfine, in, C, out, ldo, co0, g_stop);
    launches_counter_add(1);
}

// upsampling backward: gin (coarse dense) = sum of the 8 children of gout's slot
__global__ void k_up2_bwd(Dims dcoarse, const bf16* __restrict__ gout, int ldo, int co0, bf16* __restrict__ gin, int C)
{
    pdl_enter();
    const long long n = (long long)dcoarse.D * dcoarse.H * dcoarse.W * C;
    const int Hf = dcoarse.H * 2, Wf = dcoarse.W * 2;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(q % C);
        const long long v = q / C;
        const int x = (int)(v % dcoarse.W), y = (int)((v / dcoarse.W) % dcoarse.H),
                  z = (int)(v / ((long long)dcoarse.W * dcoarse.H));
        float s = 0.0f;
        for (int o = 0; o < 8; o++) {
            const int zz = 2 * z + (o >> 2), yy = 2 * y + ((o >> 1) & 1), xx = 2 * x + (o & 1);
            s += __bfloat162float(gout[((long long)(zz * Hf + yy) * Wf + xx) * ldo + co0 + c]);
        }
        gin[q] = __float2bfloat16(s);
    }
}

void up2_bwd(const Dims& dcoarse, const bf16* gout, int ldo, int co0, bf16* gin, int C, cudaStream_t s)
{
    launch_pdl(k_up2_bwd, eblocks((long long)dcoarse.D * dcoarse.H * dcoarse.W * C), 256, 0, s, dcoarse, gout, ldo, co0, gin, C);
    launches_counter_add(1);
}

// Wf[tap'][co][ci] = W[26-tap][ci][co]: the weights of the backward-data convolution.
__global__ void k_flip(const bf16* __restrict__ W, bf16* __restrict__ Wf, int Cin, int Cout)
{
    pdl_enter();
    const int n = 27 * Cin * Cout;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        const int co = q % Cout, ci = (q / Cout) % Cin, tap = q / (Cout * Cin);
        Wf[((long long)(26 - tap) * Cout + co) * Cin + ci] = W[q];
    }
}

void flip(const bf16* W, bf16* Wf, int Cin, int Cout, cudaStream_t s)
{
    launch_pdl(k_flip, (27 * Cin * Cout + 255) / 256, 256, 0, s, W, Wf, Cin, Cout);
    launches_counter_add(1);
}

// MSE on channel 0 of an FP32 output slab [v][ld]: loss += sum (o - t)^2 / n,
// gradient G[v][0] = 2 (o - t) / n, other channels 0.
__global__ void k_mse(long long nv, const float* __restrict__ out, int ldo, const float* __restrict__ t,
                      bf16* __restrict__ G, int ldg, double* loss)
{
    pdl_enter();
    double s = 0.0;
    const float inv = (float)(1.0 / (double)nv);
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nv; v += (long long)gridDim.x * blockDim.x) {
        const float e = out[v * ldo] - t[v];
        s += (double)e * (double)e;
        G[v * ldg] = __float2bfloat16(2.0f * e * inv);
        for (int c = 1; c < ldg; c++) G[v * ldg + c] = __float2bfloat16(0.0f);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, s / (double)nv);
}

void mse(long long nv, const float* out, int ldo, const float* t, bf16* G, int ldg, double* loss, cudaStream_t s)
{
    launch_pdl(k_mse, eblocks(nv), 256, 0, s, nv, out, ldo, t, G, ldg, loss);
    launches_counter_add(1);
}

// Adam on FP32 master parameters; refreshes the BF16 copy of the weights.  The
// gradient is first scaled by min(1, max_norm / ||g||) (global-norm clipping), with
// ||g|| = (*g_rms) * sqrt(n) from k_rms.
__global__ void k_adam(long long n, float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, bf16* __restrict__ pb, float lr, float b1, float b2, float eps, float c1,
                       float c2, const float* g_rms, float max_norm)
{
    pdl_enter();
    float clip = 1.0f;
    if (g_rms) {
        const float norm = *g_rms * sqrtf((float)n);
        if (norm > max_norm && norm > 0.0f) clip = max_norm / norm;
    }
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        const float gq = g[q] * clip;
        const float mq = b1 * m[q] + (1.0f - b1) * gq;
        const float vq = b2 * v[q] + (1.0f - b2) * gq * gq;
        m[q] = mq;
        v[q] = vq;
        const float upd = lr * (mq / c1) / (sqrtf(vq / c2) + eps);
        const float pn = p[q] - upd;
        p[q] = pn;
        if (pb) pb[q] = __float2bfloat16(pn);
    }
}

void adam(long long n, float* p, const float* g, float* m, float* v, bf16* pb, float lr, float b1, float b2, float eps,
          int step, const float* g_rms, float max_norm, cudaStream_t s)
{
    const float c1 = 1.0f - powf(b1, (float)step), c2 = 1.0f - powf(b2, (float)step);
    launch_pdl(k_adam, eblocks(n), 256, 0, s, n, p, g, m, v, pb, lr, b1, b2, eps, c1, c2, g_rms, max_norm);
    launches_counter_add(1);
}

__global__ void k_f32_to_bf16(long long n, const float* __restrict__ a, bf16* __restrict__ b)
{
    pdl_enter();
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x)
        b[q] = __float2bfloat16(a[q]);
}

void f32_to_bf16(long long n, const float* a, bf16* b, cudaStream_t s)
{
    launch_pdl(k_f32_to_bf16, eblocks(n), 256, 0, s, n, a, b);
    launches_counter_add(1);
}

// Dense FP32 input [v] -> channel 0 of a BF16 activation [v][ld], scaled by 1/(*rms)
// (rms == nullptr: scale 1); the other channels zero.
__global__ void k_dense_to_act(long long nv, const float* __restrict__ in, const float* rms, bf16* __restrict__ act, int ld, const int* __restrict__ stop)
{
    pdl_enter();
    if (stop && *(volatile const int*)stop) return;
    const float sc = rms ? (*rms > 0.0f ? 1.0f / *rms : 0.0f) : 1.0f;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nv; v += (long long)gridDim.x * blockDim.x) {
        act[v * ld] = __float2bfloat16(in[v] * sc);
        for (int c = 1; c < ld; c++) act[v * ld + c] = __float2bfloat16(0.0f);
    }
}

void dense_to_act(long long nv, const float* in, const float* rms, bf16* act, int ld, cudaStream_t s)
{
    launch_pdl(k_dense_to_act, eblocks(nv), 256, 0, s, nv, in, rms, act, ld, g_stop);
    launches_counter_add(1);
}

// channel 0 of an FP32 output slab -> dense FP32, times (*rms) * gain
__global__ void k_out_to_dense(long long nv, const float* __restrict__ out, int ld, const float* rms, float gain,
                               float* __restrict__ dense, const int* __restrict__ stop)
{
    pdl_enter();
    if (stop && *(volatile const int*)stop) return;
    const float sc = (rms ? *rms : 1.0f) * gain;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nv; v += (long long)gridDim.x * blockDim.x)
        dense[v] = out[v * ld] * sc;
}

void out_to_dense(long long nv, const float* out, int ld, const float* rms, float gain, float* dense, cudaStream_t s)
{
    launch_pdl(k_out_to_dense, eblocks(nv), 256, 0, s, nv, out, ld, rms, gain, dense, g_stop);
    launches_counter_add(1);
}

// rms of a dense FP32 array into *rms (single block, deterministic)
__global__ void k_rms(long long n, const float* __restrict__ a, float* rms, const int* __restrict__ stop)
{
    pdl_enter();
    if (stop && *(volatile const int*)stop) return;
    __shared__ double sm[32];
    double s = 0.0;
    for (long long q = threadIdx.x; q < n; q += blockDim.x) s += (double)a[q] * (double)a[q];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += sm[w];
        *rms = (float)sqrt(t / (double)(n > 0 ? n : 1));
    }
}

void rms(long long n, const float* a, float* out, cudaStream_t s)
{
    launch_pdl(k_rms, 1, 1024, 0, s, n, a, out, g_stop);
    launches_counter_add(1);
}

// ---------------------------------------------------------------------------
// Grid transfers between a solver field (guard-padded layout, Dirichlet unknowns
// 2..n-1 per axis) and dense [z][y][x] arrays of its unknowns.
// ---------------------------------------------------------------------------

// The transfer kernels below run one thread per unknown (or per coarse column)
// on a 3-D grid: x along threadIdx/blockIdx.x, y on blockIdx.y, z on blockIdx.z,
// so no thread divides to find its indices.  Extents along y and z are at most
// 65535 (checked when the learned preconditioner is attached).
static dim3 field_grid(int ux, int uy, int uz, int bx) { return dim3((unsigned)((ux + bx - 1) / bx), (unsigned)uy, (unsigned)uz); }

__device__ __forceinline__ long long field_at(const Geo& g, int i, int j, int k)
{
    return (g.lo[0] + i) + g.sj * (long long)(g.lo[1] + j) + g.sk * (long long)(g.lo[2] + k);
}

// dense = field unknowns (type T -> float)
template <typename T>
__global__ void k_field_to_dense(Geo g, const T* __restrict__ f, float* __restrict__ dense, const int* __restrict__ stop)
{
    pdl_enter();
    if (stop && *(volatile const int*)stop) return;
    const int ux = g.hi[0] - g.lo[0], uy = g.hi[1] - g.lo[1];
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, k = blockIdx.z;
    if (i >= ux) return;
    dense[((long long)k * uy + j) * ux + i] = (float)f[field_at(g, i, j, k)];
}

// field unknowns (+)= scale * dense
template <typename T>
__global__ void k_dense_to_field(Geo g, const float* __restrict__ dense, T* __restrict__ f, float scale, int add, const int* __restrict__ stop)
{
    pdl_enter();
    if (stop && *(volatile const int*)stop) return;
    const int ux = g.hi[0] - g.lo[0], uy = g.hi[1] - g.lo[1];
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, k = blockIdx.z;
    if (i >= ux) return;
    const long long c = field_at(g, i, j, k);
    const T v = (T)(scale * dense[((long long)k * uy + j) * ux + i]);
    f[c] = add ? f[c] + v : v;
}

template <typename T>
void field_to_dense(const Geo& g, const T* f, float* dense, cudaStream_t s)
{
    launch_pdl(k_field_to_dense<T>, field_grid(g.hi[0] - g.lo[0], g.hi[1] - g.lo[1], g.hi[2] - g.lo[2], 128), 128, 0, s,
        g, f, dense, g_stop);
    launches_counter_add(1);
}

template <typename T>
void dense_to_field(const Geo& g, const float* dense, T* f, float scale, int add, cudaStream_t s)
{
    launch_pdl(k_dense_to_field<T>, field_grid(g.hi[0] - g.lo[0], g.hi[1] - g.lo[1], g.hi[2] - g.lo[2], 128), 128, 0, s,
        g, dense, f, scale, add, g_stop);
    launches_counter_add(1);
}

template void field_to_dense<float>(const Geo&, const float*, float*, cudaStream_t);
template void field_to_dense<double>(const Geo&, const double*, float*, cudaStream_t);
template void dense_to_field<float>(const Geo&, const float*, float*, float, int, cudaStream_t);
template void dense_to_field<double>(const Geo&, const float*, double*, float, int, cudaStream_t);

// ---------------------------------------------------------------------------
// Transfers fused with the solver fields.  The fast fields keep their guard
// cells (the Dirichlet boundary nodes) at zero, so the 7-point stencil reads them
// unconditionally.
// ---------------------------------------------------------------------------

template <typename T>
struct StencilW {
    T ix, iy, iz, diag;   // 1/h^2 per axis and the centre weight -2 (ix + iy + iz)
};
template <typename T>
static StencilW<T> stencil_w(const Geo& g)
{
    StencilW<T> w;
    const double ix = 1.0 / (g.ds[0] * g.ds[0]), iy = 1.0 / (g.ds[1] * g.ds[1]), iz = 1.0 / (g.ds[2] * g.ds[2]);
    w.ix = (T)ix;
    w.iy = (T)iy;
    w.iz = (T)iz;
    w.diag = (T)(-2.0 * (ix + iy + iz));
    return w;
}

template <typename T>
__device__ __forceinline__ T residual_at(const Geo& g, const T* __restrict__ r, const T* __restrict__ z, long long c,
                                         const StencilW<T>& w)
{
    T a = w.diag * z[c];
    a += w.ix * (z[c - 1] + z[c + 1]);
    a += w.iy * (z[c - g.sj] + z[c + g.sj]);
    a += w.iz * (z[c - g.sk] + z[c + g.sk]);
    return r[c] - a;
}

// dense = r - A z at the unknowns.
template <typename T>
__global__ void k_field_residual_dense(Geo g, const T* __restrict__ r, const T* __restrict__ z, StencilW<T> w,
                                       float* __restrict__ dense, const int* __restrict__ stop)
{
    pdl_enter();
    if (stop && *(volatile const int*)stop) return;
    const int ux = g.hi[0] - g.lo[0], uy = g.hi[1] - g.lo[1];
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, k = blockIdx.z;
    if (i >= ux) return;
    dense[((long long)k * uy + j) * ux + i] = (float)residual_at<T>(g, r, z, field_at(g, i, j, k), w);
}

// The field kernels below march along z over the column tiles of a Shape (32 x ty
// columns per block, kchunk planes per thread, one column per thread), like the
// solver's own z-marching kernels.
struct ZCol {
    int i, j, k0, k1;   // column (i, j) of unknowns, planes [k0, k1)
    long long c;        // field index of (i, j, k0)
    bool active;
};

__device__ __forceinline__ ZCol zcolumn(const Geo& g, const Shape& sh)
{
    ZCol q;
    const int bx = blockIdx.x % sh.ntx, by = blockIdx.x / sh.ntx;
    q.i = g.lo[0] + bx * 32 + threadIdx.x;
    q.j = g.lo[1] + by * sh.ty + threadIdx.y;
    q.k0 = g.lo[2] + blockIdx.y * sh.kchunk;
    q.k1 = min(q.k0 + sh.kchunk, g.hi[2]);
    q.active = q.i < g.hi[0] && q.j < g.hi[1];
    q.c = q.i + g.sj * q.j + g.sk * q.k0;
    return q;
}

static dim3 zgrid(const Shape& sh) { return dim3((unsigned)(sh.ntx * sh.nty), (unsigned)sh.nchunks, 1); }
static dim3 zblock(const Shape& sh) { return dim3(32, (unsigned)sh.ty, 1); }

// out = r - A z at the unknowns (z planes k-1, k, k+1 kept in registers).
template <typename T>
__global__ void __launch_bounds__(256) k_field_residual(Geo g, Shape sh, const T* __restrict__ r,
                                                        const T* __restrict__ z, StencilW<T> w, T* __restrict__ out, const int* __restrict__ stop)
{
    pdl_enter();
    if (stop && *(volatile const int*)stop) return;
    const ZCol q = zcolumn(g, sh);
    if (!q.active) return;
    const long long sj = g.sj, sk = g.sk;
    long long c = q.c;
    T zm = z[c - sk], zc = z[c];
    for (int k = q.k0; k < q.k1; k++, c += sk) {
        const T zp = z[c + sk];
        T a = w.diag * zc;
        a += w.ix * (z[c - 1] + z[c + 1]);
        a += w.iy * (z[c - sj] + z[c + sj]);
        a += w.iz * (zm + zp);
        out[c] = r[c] - a;
        zm = zc;
        zc = zp;
    }
}

// x += y at the unknowns.
template <typename T>
__global__ void __launch_bounds__(256) k_field_axpy(Geo g, Shape sh, T* __restrict__ x, const T* __restrict__ y, const int* __restrict__ stop)
{
    pdl_enter();
    if (stop && *(volatile const int*)stop) return;
    const ZCol q = zcolumn(g, sh);
    if (!q.active) return;
    long long c = q.c;
    for (int k = q.k0; k < q.k1; k++, c += g.sk) x[c] += y[c];
}

// Full-weighting restriction (the weights of k_restrict: 1/4, 1/2, 1/4 per axis
// over fine 2c, 2c+1, 2c+2) of the residual r - A z of the solver fields, straight
// into the coarse dense array; with HAS_Z false the restricted field is r itself.
// One thread per coarse (x, y) column walks `zc` coarse planes, keeping the three z
// planes of its 3 x 3 fine points in registers: per pair of fine planes it loads
// 9 z, 9 r and the 12 in-plane neighbours, and each fine value is read from DRAM
// once (the fine-grid residual is never stored).
template <typename T, bool HAS_Z>
__global__ void __launch_bounds__(128) k_field_residual_restrict(Geo g, const T* __restrict__ r,
                                                                 const T* __restrict__ z, StencilW<T> w, Dims dc,
                                                                 int zc, float* __restrict__ coarse, const int* __restrict__ stop)
{
    pdl_enter();
    if (stop && *(volatile const int*)stop) return;
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= dc.W || y >= dc.H) return;
    const int z0 = blockIdx.z * zc, z1 = min(dc.D, z0 + zc);
    if (z0 >= z1) return;
    const int uz = 2 * dc.D;
    // the third fine column / row lies on the boundary node for the last coarse column / row
    const bool on_x2 = 2 * x + 2 < 2 * dc.W, on_y2 = 2 * y + 2 < 2 * dc.H;
    const long long sj = g.sj;
    const T wt[3] = {(T)0.25, (T)0.5, (T)0.25};
    T zm[3][3], zcn[3][3], zp[3][3];   // z at fine planes f-1, f, f+1 of the 3 x 3 fine points

    auto load_plane = [&](int k, T (&pl)[3][3]) {
        const long long c = field_at(g, 2 * x, 2 * y, k);
#pragma unroll
        for (int b = 0; b < 3; b++)
#pragma unroll
            for (int a = 0; a < 3; a++) pl[b][a] = z[c + b * sj + a];
    };
    // weighted 3 x 3 sum of the residual on fine plane f (zcn holds plane f)
    auto plane_sum = [&](int f) -> T {
        const long long c = field_at(g, 2 * x, 2 * y, f);
        T acc = (T)0;
#pragma unroll
        for (int b = 0; b < 3; b++) {
            if (b == 2 && !on_y2) continue;
#pragma unroll
            for (int a = 0; a < 3; a++) {
                if (a == 2 && !on_x2) continue;
                const long long o = c + b * sj + a;
                T res = r[o];
                if (HAS_Z) {
                    const T left = a > 0 ? zcn[b][a - 1] : z[o - 1];
                    const T right = a < 2 ? zcn[b][a + 1] : z[o + 1];
                    const T down = b > 0 ? zcn[b - 1][a] : z[o - sj];
                    const T up = b < 2 ? zcn[b + 1][a] : z[o + sj];
                    T av = w.diag * zcn[b][a];
                    av += w.ix * (left + right);
                    av += w.iy * (down + up);
                    av += w.iz * (zm[b][a] + zp[b][a]);
                    res -= av;
                }
                acc += wt[b] * wt[a] * res;
            }
        }
        return acc;
    };
    auto shift = [&](int knext) {
#pragma unroll
        for (int b = 0; b < 3; b++)
#pragma unroll
            for (int a = 0; a < 3; a++) {
                zm[b][a] = zcn[b][a];
                zcn[b][a] = zp[b][a];
            }
        if (HAS_Z) load_plane(knext, zp);
    };

    const int f0 = 2 * z0;   // < uz
    if (HAS_Z) {
        load_plane(f0 - 1, zm);
        load_plane(f0, zcn);
        load_plane(f0 + 1, zp);
    }
    T prev = plane_sum(f0);
    long long out = ((long long)z0 * dc.H + y) * dc.W + x;
    const long long cstride = (long long)dc.H * dc.W;
    for (int cz = z0; cz < z1; cz++, out += cstride) {
        shift(2 * cz + 2);                     // now at plane 2cz+1; plane 2cz+2 <= uz is in the field
        const T mid = plane_sum(2 * cz + 1);
        T next = (T)0;
        if (2 * cz + 2 < uz) {
            shift(2 * cz + 3);                 // 2cz+3 <= uz
            next = plane_sum(2 * cz + 2);
        }
        coarse[out] = (float)(wt[0] * prev + wt[1] * mid + wt[2] * next);
        prev = next;
    }
}

// field unknowns += trilinear prolongation of a coarse dense array with half the
// unknowns per axis (the weights of k_prolong: fine i takes coarse (i-1)/2 when i
// is odd, the mean of coarse i/2-1 and i/2 otherwise, zero beyond the grid).
// Each thread marches its column along z and interpolates every coarse plane in
// (x, y) once (4 loads), so a fine point costs about 2 coarse loads.
template <typename T>
__global__ void __launch_bounds__(256) k_prolong_add_field(Geo g, Shape sh, Dims dc, const float* __restrict__ coarse,
                                                           T* __restrict__ f, const int* __restrict__ stop)
{
    pdl_enter();
    if (stop && *(volatile const int*)stop) return;
    const ZCol q = zcolumn(g, sh);
    if (!q.active) return;
    const int ii = q.i - g.lo[0], jj = q.j - g.lo[1];
    int xa, xb, ya, yb;   // coarse indices along x and y
    float wxa, wxb, wya, wyb;
    if (ii & 1) {
        xa = xb = ii >> 1;
        wxa = 1.0f;
        wxb = 0.0f;
    } else {
        xa = (ii >> 1) - 1;
        xb = ii >> 1;
        wxa = xa >= 0 ? 0.5f : 0.0f;
        wxb = 0.5f;
        if (xa < 0) xa = xb;
    }
    if (jj & 1) {
        ya = yb = jj >> 1;
        wya = 1.0f;
        wyb = 0.0f;
    } else {
        ya = (jj >> 1) - 1;
        yb = jj >> 1;
        wya = ya >= 0 ? 0.5f : 0.0f;
        wyb = 0.5f;
        if (ya < 0) ya = yb;
    }
    const long long plane = (long long)dc.H * dc.W;
    const long long oaa = (long long)ya * dc.W + xa, oab = (long long)ya * dc.W + xb;
    const long long oba = (long long)yb * dc.W + xa, obb = (long long)yb * dc.W + xb;
    auto interp = [&](int cz) -> float {   // bilinear value of coarse plane cz at this column
        const float* p = coarse + (long long)cz * plane;
        return wya * (wxa * p[oaa] + wxb * p[oab]) + wyb * (wxa * p[oba] + wxb * p[obb]);
    };
    const long long sk = g.sk;
    const int kk1 = q.k1 - g.lo[2];
    int kk = q.k0 - g.lo[2];
    int cz = kk >> 1;
    float vm = cz >= 1 ? interp(cz - 1) : 0.0f;   // coarse planes cz-1 and cz
    float v0 = interp(cz);
    long long c = q.c;
    if (kk & 1) {   // odd first plane: coarse plane cz alone
        f[c] += (T)v0;
        c += sk;
        kk++;
        vm = v0;
        cz++;
        v0 = cz < dc.D ? interp(cz) : 0.0f;
    }
    // plane pairs (2cz, 2cz+1): the mean of coarse planes cz-1, cz, then cz alone
    for (; kk + 1 < kk1; kk += 2, c += 2 * sk) {
        const float vn = cz + 1 < dc.D ? interp(cz + 1) : 0.0f;
        const T f0 = f[c], f1 = f[c + sk];
        f[c] = f0 + (T)(0.5f * (vm + v0));
        f[c + sk] = f1 + (T)v0;
        vm = v0;
        v0 = vn;
        cz++;
    }
    if (kk < kk1) f[c] += (T)(0.5f * (vm + v0));   // a last even plane
}

// One thread's column of k_prolong_add_field_v4: fine x points i0..i0+3 (those
// that are unknowns) of row j, planes k0..k1-1.
template <bool DOTS>
__device__ __forceinline__ void prolong_v4_column(const Geo& g, const Dims& dc, const float* __restrict__ coarse,
                                                  float* __restrict__ f, const float* __restrict__ r,
                                                  const float* __restrict__ Ap, int i0, int j, int k0, int k1,
                                                  Acc<float>& zr, Acc<float>& zap)
{
    const bool m0 = i0 >= g.lo[0] && i0 < g.hi[0], m1 = i0 + 1 >= g.lo[0] && i0 + 1 < g.hi[0];
    const bool m2 = i0 + 2 >= g.lo[0] && i0 + 2 < g.hi[0], m3 = i0 + 3 >= g.lo[0] && i0 + 3 < g.hi[0];
    const bool all4 = m0 && m1 && m2 && m3;
    const int ii0 = i0 - g.lo[0];
    const bool odd0 = (ii0 & 1) != 0;
    const int X0 = (ii0 - 1) >> 1;   // floor((ii0 - 1) / 2): the lowest coarse column the points use
    const int jj = j - g.lo[1];
    int ya, yb;
    float wya, wyb;
    if (jj & 1) {
        ya = yb = jj >> 1;
        wya = 1.0f;
        wyb = 0.0f;
    } else {
        ya = (jj >> 1) - 1;
        yb = jj >> 1;
        wya = ya >= 0 ? 0.5f : 0.0f;
        wyb = 0.5f;
        if (ya < 0) ya = yb;
    }
    const long long plane = (long long)dc.H * dc.W;
    const long long ra = (long long)ya * dc.W, rb = (long long)yb * dc.W;
    auto load3 = [&](int cz, float (&v)[3]) {   // coarse columns X0..X0+2 of plane cz, interpolated in y
        const float* p = coarse + (long long)cz * plane;
#pragma unroll
        for (int q = 0; q < 3; q++) {
            const int X = X0 + q;
            v[q] = X >= 0 && X < dc.W ? wya * p[ra + X] + wyb * p[rb + X] : 0.0f;
        }
    };
    // x interpolation at the four points: odd fine columns take one coarse column,
    // even ones the mean of two (fine ii: odd -> (ii-1)/2, even -> ii/2-1, ii/2)
    auto xi = [&](const float (&v)[3]) -> float4 {
        if (odd0) return make_float4(v[0], 0.5f * (v[0] + v[1]), v[1], 0.5f * (v[1] + v[2]));
        return make_float4(0.5f * (v[0] + v[1]), v[1], 0.5f * (v[1] + v[2]), v[2]);
    };
    auto add = [&](long long c, float4 v) {
        if (all4) {
            float4 q = *reinterpret_cast<const float4*>(f + c);
            q.x += v.x;
            q.y += v.y;
            q.z += v.z;
            q.w += v.w;
            *reinterpret_cast<float4*>(f + c) = q;
            if (DOTS) {
                const float4 rv = *reinterpret_cast<const float4*>(r + c);
                const float4 av = *reinterpret_cast<const float4*>(Ap + c);
                zr.add(q.x, rv.x);
                zap.add(q.x, av.x);
                zr.add(q.y, rv.y);
                zap.add(q.y, av.y);
                zr.add(q.z, rv.z);
                zap.add(q.z, av.z);
                zr.add(q.w, rv.w);
                zap.add(q.w, av.w);
            }
        } else {
            const bool m[4] = {m0, m1, m2, m3};
            const float vv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
            for (int e = 0; e < 4; e++)
                if (m[e]) {
                    const float q = f[c + e] + vv[e];
                    f[c + e] = q;
                    if (DOTS) {
                        zr.add(q, r[c + e]);
                        zap.add(q, Ap[c + e]);
                    }
                }
        }
    };
    const long long sk = g.sk;
    const int kk1 = k1 - g.lo[2];
    int kk = k0 - g.lo[2];
    int cz = kk >> 1;
    float vm[3] = {0.0f, 0.0f, 0.0f}, v0[3];
    if (cz >= 1) load3(cz - 1, vm);
    load3(cz, v0);
    float4 xm = xi(vm), x0 = xi(v0);
    long long c = i0 + g.sj * (long long)j + sk * (long long)k0;
    if (kk & 1) {   // odd first plane: coarse plane cz alone
        add(c, x0);
        c += sk;
        kk++;
        xm = x0;
        cz++;
        if (cz < dc.D) {
            load3(cz, v0);
            x0 = xi(v0);
        } else {
            x0 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
    }
    for (; kk + 1 < kk1; kk += 2, c += 2 * sk) {
        float4 xn = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (cz + 1 < dc.D) {
            float vn[3];
            load3(cz + 1, vn);
            xn = xi(vn);
        }
        const float4 xa = make_float4(0.5f * (xm.x + x0.x), 0.5f * (xm.y + x0.y), 0.5f * (xm.z + x0.z), 0.5f * (xm.w + x0.w));
        if (all4) {
            // both fine planes' loads before either store: f is written in place, so
            // the compiler cannot move the second plane's loads above the first
            // plane's store, and the pair would cost two round trips to memory
            float4 q0 = *reinterpret_cast<const float4*>(f + c), q1 = *reinterpret_cast<const float4*>(f + c + sk);
            float4 r0, r1, a0, a1;
            if (DOTS) {
                r0 = *reinterpret_cast<const float4*>(r + c);
                r1 = *reinterpret_cast<const float4*>(r + c + sk);
                a0 = *reinterpret_cast<const float4*>(Ap + c);
                a1 = *reinterpret_cast<const float4*>(Ap + c + sk);
            }
            q0 = make_float4(q0.x + xa.x, q0.y + xa.y, q0.z + xa.z, q0.w + xa.w);
            q1 = make_float4(q1.x + x0.x, q1.y + x0.y, q1.z + x0.z, q1.w + x0.w);
            *reinterpret_cast<float4*>(f + c) = q0;
            *reinterpret_cast<float4*>(f + c + sk) = q1;
            if (DOTS) {   // plane order, element order: the sums of add()
                zr.add(q0.x, r0.x);
                zap.add(q0.x, a0.x);
                zr.add(q0.y, r0.y);
                zap.add(q0.y, a0.y);
                zr.add(q0.z, r0.z);
                zap.add(q0.z, a0.z);
                zr.add(q0.w, r0.w);
                zap.add(q0.w, a0.w);
                zr.add(q1.x, r1.x);
                zap.add(q1.x, a1.x);
                zr.add(q1.y, r1.y);
                zap.add(q1.y, a1.y);
                zr.add(q1.z, r1.z);
                zap.add(q1.z, a1.z);
                zr.add(q1.w, r1.w);
                zap.add(q1.w, a1.w);
            }
        } else {
            add(c, xa);
            add(c + sk, x0);
        }
        xm = x0;
        x0 = xn;
        cz++;
    }
    if (kk < kk1)   // a last even plane
        add(c, make_float4(0.5f * (xm.x + x0.x), 0.5f * (xm.y + x0.y), 0.5f * (xm.z + x0.z), 0.5f * (xm.w + x0.w)));
}


// k_prolong_add_field on x-vectorised FP32 tiles: a thread owns four consecutive x
// points of the field (one float4, tiles aligned to x = 0 as the solver's
// vectorised Chebyshev tiles).  The four points need at most three consecutive
// coarse x columns, X0..X0+2: per coarse plane the thread interpolates those in y
// (6 loads), then each point in x, and adds the two fine planes the coarse plane
// covers with float4 read-modify-writes.  The weights are k_prolong_add_field's
// (interpolated in y first, so the rounding differs from it).
// DOTS: f is flexible CG's z = M r, finished here, so the kernel also sums z.r and
// z.Ap over the unknowns (the FIN_FCG_CONV reduction) while z is in registers.
template <bool DOTS>
__global__ void __launch_bounds__(256) k_prolong_add_field_v4(Geo g, Shape sh, Dims dc, const float* __restrict__ coarse,
                                                              float* __restrict__ f, const int* __restrict__ stop,
                                                              const float* __restrict__ r, const float* __restrict__ Ap,
                                                              RedCtx rc)
{
    pdl_enter();
    if (stop && *(volatile const int*)stop) return;
    const int bx = blockIdx.x % sh.ntx, by = blockIdx.x / sh.ntx;
    const int i0 = bx * 128 + threadIdx.x * 4;
    const int j = g.lo[1] + by * sh.ty + threadIdx.y;
    const int k0 = g.lo[2] + blockIdx.y * sh.kchunk, k1 = min(k0 + sh.kchunk, g.hi[2]);
    Acc<float> zr, zap;
    if (!(j >= g.hi[1] || i0 >= g.hi[0] || i0 + 4 <= g.lo[0]))
        prolong_v4_column<DOTS>(g, dc, coarse, f, r, Ap, i0, j, k0, k1, zr, zap);
    if (DOTS) {
        double v[2] = {zr.value(), zap.value()};
        reduce_finalize<2>(v, rc);
    }
}

template <typename T>
void field_residual_dense(const Geo& g, const T* r, const T* z, float* dense, cudaStream_t s)
{
    launch_pdl(k_field_residual_dense<T>, field_grid(g.hi[0] - g.lo[0], g.hi[1] - g.lo[1], g.hi[2] - g.lo[2], 128), 128, 0, s,
        g, r, z, stencil_w<T>(g), dense, g_stop);
    launches_counter_add(1);
}
template <typename T>
void field_residual(const Geo& g, const Shape& sh, const T* r, const T* z, T* out, cudaStream_t s)
{
    launch_pdl(k_field_residual<T>, zgrid(sh), zblock(sh), 0, s, g, sh, r, z, stencil_w<T>(g), out, g_stop);
    launches_counter_add(1);
}
template <typename T>
void field_axpy(const Geo& g, const Shape& sh, T* x, const T* y, cudaStream_t s)
{
    launch_pdl(k_field_axpy<T>, zgrid(sh), zblock(sh), 0, s, g, sh, x, y, g_stop);
    launches_counter_add(1);
}
template <typename T>
void field_residual_restrict(const Geo& g, const T* r, const T* z, const Dims& dc, float* coarse, cudaStream_t s)
{
    const int zc = 8;
    const dim3 block(32, 4);
    const dim3 grid((unsigned)((dc.W + 31) / 32), (unsigned)((dc.H + 3) / 4), (unsigned)((dc.D + zc - 1) / zc));
    if (z) launch_pdl(k_field_residual_restrict<T, true>, grid, block, 0, s, g, r, z, stencil_w<T>(g), dc, zc, coarse, g_stop);
    else launch_pdl(k_field_residual_restrict<T, false>, grid, block, 0, s, g, r, z, stencil_w<T>(g), dc, zc, coarse, g_stop);
    launches_counter_add(1);
}
template <typename T>
bool prolong_add_field(const Geo& g, const Shape& sh, const Dims& dc, const float* coarse, T* f, cudaStream_t s,
                       const T* r, const T* Ap, const RedCtx* dots)
{
    if (sh.cx == 4) {   // the x-vectorised tiles (FP32 rows on 16-byte boundaries), else one column per thread
        if constexpr (std::is_same<T, float>::value) {
            auto a16 = [](const void* p) { return ((uintptr_t)p & 15u) == 0; };
            if (g.sj % 4 == 0 && a16(f)) {
                if (dots && r && Ap && a16(r) && a16(Ap))
                    launch_pdl(k_prolong_add_field_v4<true>, zgrid(sh), zblock(sh), 0, s, g, sh, dc, coarse, f, g_stop, r, Ap,
                                                                                 *dots);
                else
                    launch_pdl(k_prolong_add_field_v4<false>, zgrid(sh), zblock(sh), 0, s, g, sh, dc, coarse, f, g_stop,
                                                                                  nullptr, nullptr, RedCtx{});
                launches_counter_add(1);
                return dots && r && Ap && a16(r) && a16(Ap);
            }
        }
        return prolong_add_field<T>(g, make_shape(g, sh.ty, (int)sh.nblocks(), 1), dc, coarse, f, s);
    }
    if (sh.cx != 1)   // two-column Chebyshev tiles: the kernel below covers 32 columns per tile
        return prolong_add_field<T>(g, make_shape(g, sh.ty, (int)sh.nblocks(), 1), dc, coarse, f, s);
    launch_pdl(k_prolong_add_field<T>, zgrid(sh), zblock(sh), 0, s, g, sh, dc, coarse, f, g_stop);
    launches_counter_add(1);
    return false;
}
template void field_residual_dense<float>(const Geo&, const float*, const float*, float*, cudaStream_t);
template void field_residual_dense<double>(const Geo&, const double*, const double*, float*, cudaStream_t);
template void field_residual<float>(const Geo&, const Shape&, const float*, const float*, float*, cudaStream_t);
template void field_residual<double>(const Geo&, const Shape&, const double*, const double*, double*, cudaStream_t);
template void field_axpy<float>(const Geo&, const Shape&, float*, const float*, cudaStream_t);
template void field_axpy<double>(const Geo&, const Shape&, double*, const double*, cudaStream_t);
template void field_residual_restrict<float>(const Geo&, const float*, const float*, const Dims&, float*, cudaStream_t);
template void field_residual_restrict<double>(const Geo&, const double*, const double*, const Dims&, float*,
                                              cudaStream_t);
template bool prolong_add_field<float>(const Geo&, const Shape&, const Dims&, const float*, float*, cudaStream_t,
                                       const float*, const float*, const RedCtx*);
template bool prolong_add_field<double>(const Geo&, const Shape&, const Dims&, const float*, double*, cudaStream_t,
                                        const double*, const double*, const RedCtx*);

// ---------------------------------------------------------------------------
// Coarse levels of the learned multigrid cycle: dense [z][y][x] arrays with the
// Dirichlet zero beyond the array edges.
// ---------------------------------------------------------------------------

// -diag(A) at a point whose last-unknown flags along x, y, z are lx, ly, lz
__device__ __forceinline__ float level_negdiag(const DLevel& L, bool lx, bool ly, bool lz)
{
    return (lx ? -L.last_c[0] : 2.0f * L.ih2[0]) + (ly ? -L.last_c[1] : 2.0f * L.ih2[1]) +
           (lz ? -L.last_c[2] : 2.0f * L.ih2[2]);
}

// One pass over a coarse level, z-marching:
//   RESID:  W = B - A Y
//   CHEB:   W (+)= scale (cy Y + D^-1 (cb B + ca A Y) + cz Z)     (HASZ: with Z)
// with D = -diag(A).  FIRST: Y is not read; its values are D^-1 B / theta (the
// recurrence's starting term), formed at each of the 7 points on the fly.  A
// column's coefficients (and D^-1 of its own and neighbouring points) are fixed
// except on the last plane, which is peeled off the plane loop.
template <bool CHEB, bool FIRST, bool HASZ, bool ACC>
__global__ void __launch_bounds__(256) k_level_pass(Dims d, DLevel L, int kchunk, const float* __restrict__ Y,
                                                    const float* __restrict__ B, const float* __restrict__ Z,
                                                    float* __restrict__ W, LCoef c, const int* __restrict__ stop)
{
    pdl_enter();
    if (stop && *(volatile const int*)stop) return;
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= d.W || y >= d.H) return;
    const int z0 = blockIdx.z * kchunk, z1 = min(d.D, z0 + kchunk);
    const long long sy = d.W, sz = (long long)d.W * d.H;
    const bool hx0 = x > 0, hx1 = x + 1 < d.W, hy0 = y > 0, hy1 = y + 1 < d.H;
    const bool lx = x == d.W - 1, ly = y == d.H - 1;
    // neighbour weights of this column (zero where the neighbour is the wall)
    const float wxm = hx0 ? (lx ? L.last_m[0] : L.ih2[0]) : 0.0f, wxp = hx1 ? L.ih2[0] : 0.0f;
    const float wym = hy0 ? (ly ? L.last_m[1] : L.ih2[1]) : 0.0f, wyp = hy1 ? L.ih2[1] : 0.0f;
    // per plane kind e (0: inside, 1: the last plane): -diag, D^-1, and for FIRST the
    // starting-term scales of the neighbours (D^-1/theta at each of them)
    float ndg[2], di[2], fc[2], fxm[2], fxp[2], fym[2], fyp[2];
#pragma unroll
    for (int e = 0; e < 2; e++) {
        ndg[e] = level_negdiag(L, lx, ly, e);
        di[e] = 1.0f / ndg[e];
        if (FIRST) {
            fc[e] = c.y0 * di[e];
            fxm[e] = hx0 ? c.y0 / level_negdiag(L, false, ly, e) : 0.0f;
            fxp[e] = hx1 ? c.y0 / level_negdiag(L, x + 1 == d.W - 1, ly, e) : 0.0f;
            fym[e] = hy0 ? c.y0 / level_negdiag(L, lx, false, e) : 0.0f;
            fyp[e] = hy1 ? c.y0 / level_negdiag(L, lx, y + 1 == d.H - 1, e) : 0.0f;
        }
    }
    const float* S = FIRST ? B : Y;   // the stencil's field
    // the value of the stencil's field at column offset q on plane kind e
    auto val = [&](long long q, float f) -> float { return FIRST ? S[q] * f : S[q]; };
    long long q = (long long)z0 * sz + (long long)y * sy + x;
    const int zlast = d.D - 1;
    float ym = z0 > 0 ? val(q - sz, fc[0]) : 0.0f;
    float yc = val(q, z0 == zlast ? fc[1] : fc[0]);
    auto point = [&](int e, float yp) {
        // in-plane neighbours: the stencil field is read directly (the weights above
        // hold the wall); FIRST scales each by its own D^-1/theta
        const float xm = hx0 ? val(q - 1, fxm[e]) : 0.0f;
        const float xp = hx1 ? val(q + 1, fxp[e]) : 0.0f;
        const float ymn = hy0 ? val(q - sy, fym[e]) : 0.0f;
        const float ypn = hy1 ? val(q + sy, fyp[e]) : 0.0f;
        const float wzm = e ? L.last_m[2] : L.ih2[2];
        const float wzp = e ? 0.0f : L.ih2[2];
        float ay = -ndg[e] * yc;
        ay = fmaf(wxm, xm, ay);
        ay = fmaf(wxp, xp, ay);
        ay = fmaf(wym, ymn, ay);
        ay = fmaf(wyp, ypn, ay);
        ay = fmaf(wzm, ym, ay);
        ay = fmaf(wzp, yp, ay);
        const float b = B[q];
        float v;
        if (CHEB) {
            v = fmaf(c.cb, b, c.ca * ay) * di[e];
            v = fmaf(c.cy, yc, v);
            if (HASZ) v = fmaf(c.cz, Z[q], v);
            v *= c.scale;
        } else {
            v = b - ay;
        }
        if (ACC) v += W[q];
        W[q] = v;
    };
    const int zend = min(z1, zlast);   // planes before the last one
    int z = z0;
#pragma unroll 2
    for (; z < zend; z++) {
        const float yp = val(q + sz, z + 1 == zlast ? fc[1] : fc[0]);
        point(0, yp);
        ym = yc;
        yc = yp;
        q += sz;
    }
    if (z < z1) point(1, 0.0f);   // the last plane: upper wall one fine spacing above
}

static void level_launch(const Dims& d, int& kchunk, dim3& grid, int waves = 4)
{
    // 32 x 8 columns per block, z split into chunks for about `waves` waves of 8
    // blocks per SM (one wave left the 256^3 level at under half the HBM rate; the
    // first Chebyshev step, whose columns start with ten divisions, keeps one)
    const int tx = (d.W + 31) / 32, ty = (d.H + 7) / 8;
    long long chunks = (sm_count() * 8LL * waves + (long long)tx * ty - 1) / ((long long)tx * ty);
    if (chunks < 1) chunks = 1;
    if (chunks > d.D) chunks = d.D;
    kchunk = (int)((d.D + chunks - 1) / chunks);
    grid = dim3((unsigned)tx, (unsigned)ty, (unsigned)((d.D + kchunk - 1) / kchunk));
}

// W = B - A_l Y on level l (k_level_pass's residual, the same arithmetic per point)
// restricted by full weighting to level l+1 in the same pass, so the level-l
// residual is never stored (restrict2 of it, summed plane by plane).  A thread owns
// a coarse (x, y) column and marches a chunk of coarse planes; on each fine plane
// it forms the residual at the 3 x 3 fine points its coarse point weights, from Y
// of that window on three planes held in registers plus the ring around it.
__global__ void __launch_bounds__(128) k_level_residual_restrict(Dims dc, DLevel L, int zc, const float* __restrict__ Y,
                                                                 const float* __restrict__ B,
                                                                 float* __restrict__ coarse, const int* __restrict__ stop)
{
    pdl_enter();
    if (stop && *(volatile const int*)stop) return;
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= dc.W || y >= dc.H) return;
    const int z0 = blockIdx.z * zc, z1 = min(dc.D, z0 + zc);
    if (z0 >= z1) return;
    const int Wf = 2 * dc.W, Hf = 2 * dc.H, Df = 2 * dc.D;
    const long long sy = Wf, sz = (long long)Wf * Hf;
    const bool in_a2 = 2 * x + 2 < Wf, in_b2 = 2 * y + 2 < Hf;   // the window's third fine column / row exists
    const float wt[3] = {0.25f, 0.5f, 0.25f};
    float ym[3][3], yc[3][3], yp[3][3];   // Y on fine planes f-1, f, f+1 of the window (0 beyond the grid)
    const long long base = (long long)(2 * y) * sy + 2 * x;

    auto load_plane = [&](int f, float (&pl)[3][3]) {
        const bool in = f >= 0 && f < Df;
        const long long o = (long long)f * sz + base;
#pragma unroll
        for (int b = 0; b < 3; b++)
#pragma unroll
            for (int a = 0; a < 3; a++)
                pl[b][a] = in && (a < 2 || in_a2) && (b < 2 || in_b2) ? Y[o + b * sy + a] : 0.0f;
    };
    // the window's weighted residual sum on fine plane f (yc holds plane f)
    auto plane_sum = [&](int f) -> float {
        const bool lz = f == Df - 1;
        const float wzm = lz ? L.last_m[2] : L.ih2[2], wzp = lz ? 0.0f : L.ih2[2];
        const long long o = (long long)f * sz + base;
        float acc = 0.0f;
#pragma unroll
        for (int b = 0; b < 3; b++) {
            if (b == 2 && !in_b2) continue;
            const int yy = 2 * y + b;
            const bool ly = yy == Hf - 1;
            const float wym = yy > 0 ? (ly ? L.last_m[1] : L.ih2[1]) : 0.0f, wyp = ly ? 0.0f : L.ih2[1];
#pragma unroll
            for (int a = 0; a < 3; a++) {
                if (a == 2 && !in_a2) continue;
                const int xx = 2 * x + a;
                const bool lx = xx == Wf - 1;
                const float wxm = xx > 0 ? (lx ? L.last_m[0] : L.ih2[0]) : 0.0f, wxp = lx ? 0.0f : L.ih2[0];
                const long long q = o + b * sy + a;
                const float left = a > 0 ? yc[b][a - 1] : (xx > 0 ? Y[q - 1] : 0.0f);
                const float right = a < 2 ? yc[b][a + 1] : (xx + 1 < Wf ? Y[q + 1] : 0.0f);
                const float down = b > 0 ? yc[b - 1][a] : (yy > 0 ? Y[q - sy] : 0.0f);
                const float up = b < 2 ? yc[b + 1][a] : (yy + 1 < Hf ? Y[q + sy] : 0.0f);
                float ay = -level_negdiag(L, lx, ly, lz) * yc[b][a];
                ay = fmaf(wxm, left, ay);
                ay = fmaf(wxp, right, ay);
                ay = fmaf(wym, down, ay);
                ay = fmaf(wyp, up, ay);
                ay = fmaf(wzm, ym[b][a], ay);
                ay = fmaf(wzp, yp[b][a], ay);
                acc += wt[b] * wt[a] * (B[q] - ay);
            }
        }
        return acc;
    };
    auto shift = [&](int fnext) {
#pragma unroll
        for (int b = 0; b < 3; b++)
#pragma unroll
            for (int a = 0; a < 3; a++) {
                ym[b][a] = yc[b][a];
                yc[b][a] = yp[b][a];
            }
        load_plane(fnext, yp);
    };

    const int f0 = 2 * z0;
    load_plane(f0 - 1, ym);
    load_plane(f0, yc);
    load_plane(f0 + 1, yp);
    float prev = plane_sum(f0);
    long long out = ((long long)z0 * dc.H + y) * dc.W + x;
    const long long cstride = (long long)dc.H * dc.W;
    for (int cz = z0; cz < z1; cz++, out += cstride) {
        shift(2 * cz + 2);   // yc: plane 2cz+1
        const float mid = plane_sum(2 * cz + 1);
        float next = 0.0f;
        if (2 * cz + 2 < Df) {
            shift(2 * cz + 3);   // yc: plane 2cz+2
            next = plane_sum(2 * cz + 2);
        }
        coarse[out] = wt[0] * prev + wt[1] * mid + wt[2] * next;
        prev = next;
    }
}

void level_residual_restrict(const Dims& dc, const DLevel& L, const float* Y, const float* B, float* coarse,
                             cudaStream_t s)
{
    // 32 x 4 coarse columns per block; z split into chunks for about two waves of
    // eight blocks per SM
    const int tx = (dc.W + 31) / 32, ty = (dc.H + 3) / 4;
    long long chunks = (sm_count() * 8LL * 2 + (long long)tx * ty - 1) / ((long long)tx * ty);
    chunks = std::max(1LL, std::min(chunks, (long long)dc.D));
    const int zc = (int)((dc.D + chunks - 1) / chunks);
    const dim3 grid((unsigned)tx, (unsigned)ty, (unsigned)((dc.D + zc - 1) / zc));
    launch_pdl(k_level_residual_restrict, grid, dim3(32, 4), 0, s, dc, L, zc, Y, B, coarse, g_stop);
    launches_counter_add(1);
}

// Exact coarse-level solve.  Each axis's 1-D level operator A_a (tridiagonal, the
// wall gap in its last row) is diagonalisable, A_a = V_a diag(lam_a) V_a^-1, so the
// level operator A = A_x + A_y + A_z (each acting along its axis) has the inverse
// (V_z V_y V_x) diag(1 / (lam_x + lam_y + lam_z)) (V_z^-1 V_y^-1 V_x^-1).  One block
// holds the level in shared memory; each pass transforms every line along one axis,
// a thread per line (the line is read into registers first, so the pass is in place).
__device__ void exact_pass(float* cube, const float* M, int n_a, int stride, int W, int H, int D, int axis)
{
    float v[LEVEL_EXACT_MAX];
    const int lines = W * H * D / n_a;
    for (int t = threadIdx.x; t < lines; t += blockDim.x) {
        int base;
        if (axis == 0) base = t * W;                                     // lines along x: (y, z)
        else if (axis == 1) base = (t % W) + (t / W) * W * H;             // along y: (x, z)
        else base = t;                                                   // along z: (x, y)
        for (int m = 0; m < n_a; m++) v[m] = cube[base + m * stride];
        for (int i = 0; i < n_a; i++) {
            float acc = 0.f;
            for (int m = 0; m < n_a; m++) acc = fmaf(M[i * n_a + m], v[m], acc);
            cube[base + i * stride] = acc;
        }
    }
}

__global__ void __launch_bounds__(512) k_level_exact(Dims d, const float* __restrict__ mats,
                                                     const float* __restrict__ r, float* __restrict__ z,
                                                     const int* done)
{
    pdl_enter();
    EARLY_EXIT(done);
    extern __shared__ float sm[];
    const int W = d.W, H = d.H, D = d.D, n = W * H * D;
    const int nm = 2 * (W * W + H * H + D * D) + W + H + D;
    float* cube = sm;
    float* M = sm + n;
    for (int i = threadIdx.x; i < nm; i += blockDim.x) M[i] = mats[i];
    for (int i = threadIdx.x; i < n; i += blockDim.x) cube[i] = r[i];
    __syncthreads();
    const float* Vix = M;
    const float* Viy = Vix + W * W;
    const float* Viz = Viy + H * H;
    const float* Vx = Viz + D * D;
    const float* Vy = Vx + W * W;
    const float* Vz = Vy + H * H;
    const float* lx = Vz + D * D;
    const float* ly = lx + W;
    const float* lz = ly + H;
    exact_pass(cube, Vix, W, 1, W, H, D, 0);
    __syncthreads();
    exact_pass(cube, Viy, H, W, W, H, D, 1);
    __syncthreads();
    exact_pass(cube, Viz, D, W * H, W, H, D, 2);
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int x = i % W, y = (i / W) % H, zz = i / (W * H);
        cube[i] = cube[i] / (lx[x] + ly[y] + lz[zz]);
    }
    __syncthreads();
    exact_pass(cube, Vx, W, 1, W, H, D, 0);
    __syncthreads();
    exact_pass(cube, Vy, H, W, W, H, D, 1);
    __syncthreads();
    exact_pass(cube, Vz, D, W * H, W, H, D, 2);
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) z[i] = cube[i];
}

void level_exact(const Dims& d, const float* mats, const float* r, float* z, cudaStream_t s)
{
    const size_t smem = sizeof(float) * ((size_t)d.W * d.H * d.D + 2 * (d.W * d.W + d.H * d.H + d.D * d.D) + d.W +
                                         d.H + d.D);
    launch_pdl(k_level_exact, 1, 512, smem, s, d, mats, r, z, g_stop);
    launches_counter_add(1);
}

// Symmetric eigen-solve by cyclic Jacobi rotations (n <= 32, double): S = Q diag(w) Q^T.
static void jacobi_eigen(int n, std::vector<double>& S, std::vector<double>& Q, std::vector<double>& w)
{
    Q.assign((size_t)n * n, 0.0);
    for (int i = 0; i < n; i++) Q[(size_t)i * n + i] = 1.0;
    for (int sweep = 0; sweep < 100; sweep++) {
        double off = 0.0, diag = 0.0;
        for (int i = 0; i < n; i++)
            for (int j = 0; j < n; j++) (i == j ? diag : off) += S[(size_t)i * n + j] * S[(size_t)i * n + j];
        if (off <= 1e-30 * diag) break;
        for (int p = 0; p < n - 1; p++)
            for (int q = p + 1; q < n; q++) {
                const double apq = S[(size_t)p * n + q];
                if (apq == 0.0) continue;
                const double app = S[(size_t)p * n + p], aqq = S[(size_t)q * n + q];
                const double theta = (aqq - app) / (2.0 * apq);
                const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                const double c = 1.0 / std::sqrt(t * t + 1.0), sn = t * c;
                for (int k = 0; k < n; k++) {   // S <- J^T S J, rows then columns
                    const double skp = S[(size_t)k * n + p], skq = S[(size_t)k * n + q];
                    S[(size_t)k * n + p] = c * skp - sn * skq;
                    S[(size_t)k * n + q] = sn * skp + c * skq;
                }
                for (int k = 0; k < n; k++) {
                    const double spk = S[(size_t)p * n + k], sqk = S[(size_t)q * n + k];
                    S[(size_t)p * n + k] = c * spk - sn * sqk;
                    S[(size_t)q * n + k] = sn * spk + c * sqk;
                }
                for (int k = 0; k < n; k++) {   // Q <- Q J
                    const double qkp = Q[(size_t)k * n + p], qkq = Q[(size_t)k * n + q];
                    Q[(size_t)k * n + p] = c * qkp - sn * qkq;
                    Q[(size_t)k * n + q] = sn * qkp + c * qkq;
                }
            }
    }
    w.resize(n);
    for (int i = 0; i < n; i++) w[i] = S[(size_t)i * n + i];
}

cudaError_t level_exact_prepare()
{
    // the largest level (32^3) needs 150 KiB of shared memory
    return cudaFuncSetAttribute(k_level_exact, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
}

bool level_exact_data(const Dims& d, const DLevel& L, std::vector<float>& mats)
{
    const int ext[3] = {d.W, d.H, d.D};
    for (int a = 0; a < 3; a++)
        if (ext[a] < 1 || ext[a] > LEVEL_EXACT_MAX) return false;
    std::vector<float> vinv, v, lam;
    for (int a = 0; a < 3; a++) {
        const int n = ext[a];
        // the 1-D operator: diagonal -2/H^2 (last: -2/(H h)), upper 1/H^2, lower 1/H^2
        // (last row: 2/(H (H+h))).  With d_0 = 1, d_{i+1} = d_i sqrt(lower_i / upper_i)
        // it is D S D^-1 with S symmetric (off-diagonals sqrt(upper * lower)).
        std::vector<double> diag(n), up(n > 1 ? n - 1 : 0), lo(n > 1 ? n - 1 : 0);
        for (int i = 0; i < n; i++) diag[i] = -2.0 * L.ih2[a];
        diag[n - 1] = L.last_c[a];
        for (int i = 0; i + 1 < n; i++) {
            up[i] = L.ih2[a];
            lo[i] = (i + 1 == n - 1) ? L.last_m[a] : L.ih2[a];
        }
        std::vector<double> dsc(n, 1.0);
        for (int i = 0; i + 1 < n; i++) dsc[i + 1] = dsc[i] * std::sqrt(lo[i] / up[i]);
        std::vector<double> S((size_t)n * n, 0.0), Q, w;
        for (int i = 0; i < n; i++) S[(size_t)i * n + i] = diag[i];
        for (int i = 0; i + 1 < n; i++) S[(size_t)i * n + i + 1] = S[(size_t)(i + 1) * n + i] = std::sqrt(up[i] * lo[i]);
        jacobi_eigen(n, S, Q, w);
        // V = D Q, V^-1 = Q^T D^-1
        for (int i = 0; i < n; i++)
            for (int j = 0; j < n; j++) vinv.push_back((float)(Q[(size_t)j * n + i] / dsc[j]));
        for (int i = 0; i < n; i++)
            for (int j = 0; j < n; j++) v.push_back((float)(dsc[i] * Q[(size_t)i * n + j]));
        for (int i = 0; i < n; i++) lam.push_back((float)w[i]);
    }
    mats.clear();
    mats.insert(mats.end(), vinv.begin(), vinv.end());
    mats.insert(mats.end(), v.begin(), v.end());
    mats.insert(mats.end(), lam.begin(), lam.end());
    return true;
}

__global__ void k_level_zero(long long n, float* __restrict__ z, const int* done)
{
    pdl_enter();
    EARLY_EXIT(done);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        z[i] = 0.f;
}

void level_zero(const Dims& d, float* z, cudaStream_t s)
{
    const long long n = (long long)d.W * d.H * d.D;
    launch_pdl(k_level_zero, eblocks(n), 256, 0, s, n, z, g_stop);
    launches_counter_add(1);
}

void level_residual(const Dims& d, const DLevel& L, const float* Y, const float* B, float* W, cudaStream_t s)
{
    int kchunk;
    dim3 grid;
    level_launch(d, kchunk, grid);
    launch_pdl(k_level_pass<false, false, false, false>, grid, dim3(32, 8), 0, s, d, L, kchunk, Y, B, nullptr, W, LCoef{}, g_stop);
    launches_counter_add(1);
}

void level_cheb(const Dims& d, const DLevel& L, const float* Y, const float* B, const float* Z, float* W,
                const LCoef& c, bool first, bool acc, cudaStream_t s)
{
    int kchunk;
    dim3 grid;
    level_launch(d, kchunk, grid, first ? 1 : 4);
    const dim3 blk(32, 8);
    if (first) {
        if (acc) launch_pdl(k_level_pass<true, true, false, true>, grid, blk, 0, s, d, L, kchunk, Y, B, Z, W, c, g_stop);
        else launch_pdl(k_level_pass<true, true, false, false>, grid, blk, 0, s, d, L, kchunk, Y, B, Z, W, c, g_stop);
    } else if (Z) {
        if (acc) launch_pdl(k_level_pass<true, false, true, true>, grid, blk, 0, s, d, L, kchunk, Y, B, Z, W, c, g_stop);
        else launch_pdl(k_level_pass<true, false, true, false>, grid, blk, 0, s, d, L, kchunk, Y, B, Z, W, c, g_stop);
    } else {
        if (acc) launch_pdl(k_level_pass<true, false, false, true>, grid, blk, 0, s, d, L, kchunk, Y, B, Z, W, c, g_stop);
        else launch_pdl(k_level_pass<true, false, false, false>, grid, blk, 0, s, d, L, kchunk, Y, B, Z, W, c, g_stop);
    }
    launches_counter_add(1);
}

// Full-weighting restriction of dense unknown arrays, fine (2m) -> coarse (m) per
// axis: coarse unknown I sits on fine unknown 2I+1 (0-based), weights 1/4,1/2,1/4
// per axis; fine values beyond the grid are the Dirichlet zero.
__global__ void k_restrict(Dims dc, const float* __restrict__ fine, float* __restrict__ coarse, const int* __restrict__ stop)
{
    pdl_enter();
    if (stop && *(volatile const int*)stop) return;
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, z = blockIdx.z;
    if (x >= dc.W) return;
    const int Wf = dc.W * 2, Hf = dc.H * 2, Df = dc.D * 2;
    const float w1[3] = {0.25f, 0.5f, 0.25f};
    float s = 0.0f;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const int zz = 2 * z + a;
        if (zz >= Df) continue;
#pragma unroll
        for (int b = 0; b < 3; b++) {
            const int yy = 2 * y + b;
            if (yy >= Hf) continue;
#pragma unroll
            for (int c = 0; c < 3; c++) {
                const int xx = 2 * x + c;
                if (xx >= Wf) continue;
                s += w1[a] * w1[b] * w1[c] * fine[((long long)zz * Hf + yy) * Wf + xx];
            }
        }
    }
    coarse[((long long)z * dc.H + y) * dc.W + x] = s;
}

void restrict2(const Dims& dc, const float* fine, float* coarse, cudaStream_t s)
{
    launch_pdl(k_restrict, field_grid(dc.W, dc.H, dc.D, 128), 128, 0, s, dc, fine, coarse, g_stop);
    launches_counter_add(1);
}

// Trilinear prolongation, coarse (m) -> fine (2m): fine unknown i takes coarse
// (i-1)/2 exactly when i is odd (0-based), the mean of its two coarse neighbours
// otherwise (zero beyond the grid); the transpose of k_restrict up to a factor 8.
// One thread per fine (x, y) column marches along z: it interpolates each coarse
// plane of its chunk in (x, y) once (4 loads) and writes the two fine planes that
// plane covers (2cz: the mean with the plane below, 2cz+1: the plane itself), so a
// fine point costs about two coarse loads and one (ADD: two) fine accesses.
template <bool ADD>
__global__ void __launch_bounds__(256) k_prolong_z(Dims dc, int ntx, int cchunk, const float* __restrict__ coarse,
                                                   float* __restrict__ fine, const int* __restrict__ stop)
{
    pdl_enter();
    if (stop && *(volatile const int*)stop) return;
    const int Wf = 2 * dc.W, Hf = 2 * dc.H;
    const int x = (int)(blockIdx.x % ntx) * 32 + threadIdx.x;
    const int y = (int)(blockIdx.x / ntx) * blockDim.y + threadIdx.y;
    if (x >= Wf || y >= Hf) return;
    const int cz0 = blockIdx.y * cchunk, cz1 = min(dc.D, cz0 + cchunk);
    if (cz0 >= cz1) return;
    int xa, xb, ya, yb;   // coarse indices along x and y
    float wxa, wxb, wya, wyb;
    if (x & 1) {
        xa = xb = x >> 1;
        wxa = 1.0f;
        wxb = 0.0f;
    } else {
        xa = (x >> 1) - 1;
        xb = x >> 1;
        wxa = xa >= 0 ? 0.5f : 0.0f;
        wxb = 0.5f;
        if (xa < 0) xa = xb;
    }
    if (y & 1) {
        ya = yb = y >> 1;
        wya = 1.0f;
        wyb = 0.0f;
    } else {
        ya = (y >> 1) - 1;
        yb = y >> 1;
        wya = ya >= 0 ? 0.5f : 0.0f;
        wyb = 0.5f;
        if (ya < 0) ya = yb;
    }
    const long long plane = (long long)dc.H * dc.W;
    const long long oaa = (long long)ya * dc.W + xa, oab = (long long)ya * dc.W + xb;
    const long long oba = (long long)yb * dc.W + xa, obb = (long long)yb * dc.W + xb;
    auto interp = [&](int cz) -> float {   // bilinear value of coarse plane cz at this column
        const float* p = coarse + (long long)cz * plane;
        return wya * (wxa * p[oaa] + wxb * p[oab]) + wyb * (wxa * p[oba] + wxb * p[obb]);
    };
    const long long fplane = (long long)Hf * Wf;
    long long q = (2LL * cz0 * Hf + y) * Wf + x;
    float vm = cz0 >= 1 ? interp(cz0 - 1) : 0.0f;
    for (int cz = cz0; cz < cz1; cz++, q += 2 * fplane) {
        const float v = interp(cz);
        const float e = 0.5f * (vm + v);
        if (ADD) {
            fine[q] += e;
            fine[q + fplane] += v;
        } else {
            fine[q] = e;
            fine[q + fplane] = v;
        }
        vm = v;
    }
}

template <bool ADD>
static void prolong_z(const Dims& dc, const float* coarse, float* fine, cudaStream_t s)
{
    const int ty = 8;
    const int ntx = (2 * dc.W + 31) / 32, nty = (2 * dc.H + ty - 1) / ty;
    const long long tiles = (long long)ntx * nty;
    long long chunks = (sm_count() * 8LL * 4 + tiles - 1) / tiles;
    chunks = std::max(1LL, std::min<long long>(chunks, dc.D));
    const int cchunk = (int)((dc.D + chunks - 1) / chunks);
    const unsigned nch = (unsigned)((dc.D + cchunk - 1) / cchunk);
    launch_pdl(k_prolong_z<ADD>, dim3((unsigned)tiles, nch), dim3(32, ty), 0, s, dc, ntx, cchunk, coarse, fine, g_stop);
    launches_counter_add(1);
}

void prolong2(const Dims& dc, const float* coarse, float* fine, cudaStream_t s)
{
    prolong_z<false>(dc, coarse, fine, s);
}

void prolong2_add(const Dims& dc, const float* coarse, float* fine, cudaStream_t s)
{
    prolong_z<true>(dc, coarse, fine, s);
}

}  // namespace unet
}  // namespace pps
