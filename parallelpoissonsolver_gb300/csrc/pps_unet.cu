// The learned preconditioner's network: a 3-level 3-D convolutional U-Net
// (channels c1/c2/c3, 3x3x3 kernels, BF16 weights and activations, FP32
// accumulation), trained and run by the project's own kernels
// (pps_unet_kernels.cu).  No reference counterpart.
//
//   x0 --conv0,relu--> e1a --conv1,relu--> e1 ----------------------------(skip)--+
//                                           |pool                                 |
//             p1 --conv2,relu--> e2a --conv3,relu--> e2 -------------(skip)--+     |
//                                                     |pool                  |     |
//                        p2 --conv4,relu--> e3a --conv5,relu--> e3 --up--> [e3|e2] |
//                                                       conv6,relu -> d2a -> conv7,relu -> d2
//                                                                          --up--> [d2|e1]
//                                                       conv8,relu -> d1a -> conv9,relu -> d1
//                                                       conv10 (linear, 1 channel) -> out
//
// Input and output are one channel; the input is scaled to unit RMS and the output
// scaled back by the same factor, so the map is positively homogeneous like A^-1.
#include "../../include/pps.h"
#include "pps_unet_internal.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <random>
#include <string>
#include <vector>

using namespace pps;
using namespace pps::unet;

namespace {

struct UFail {};

#define UK(call)                                                                              \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess) {                                                              \
            pps_internal_set_error((std::string(#call) + ": " + cudaGetErrorString(e_)).c_str()); \
            throw UFail{};                                                                    \
        }                                                                                     \
    } while (0)

struct Layer {
    int cin, cout;         // real channels
    int cin_p, cout_p;     // padded to multiples of 16
    bool relu;
    size_t w, b;           // offsets of W [27][cin_p][cout_p] and b [cout_p] in the padded arrays
    size_t rw, rb;         // offsets in the real (unpadded) flat parameter vector
};

int pad16(int c) { return (c + 15) / 16 * 16; }

struct Acts {
    Dims s1{0, 0, 0}, s2{0, 0, 0}, s3{0, 0, 0};   // grid of each level
    bf16 *x0 = nullptr, *e1a = nullptr, *cat1 = nullptr, *d1a = nullptr, *d1 = nullptr;
    bf16 *p1 = nullptr, *e2a = nullptr, *cat2 = nullptr, *d2a = nullptr, *d2 = nullptr;
    bf16 *p2 = nullptr, *e3a = nullptr, *e3 = nullptr;
    float* out = nullptr;
    // gradients
    bf16 *g_out = nullptr, *g_d1 = nullptr, *g_d1a = nullptr, *g_cat1 = nullptr, *g_d2 = nullptr, *g_d2a = nullptr,
         *g_cat2 = nullptr, *g_e3 = nullptr, *g_e3a = nullptr, *g_p2 = nullptr, *g_e2a = nullptr, *g_p1 = nullptr,
         *g_e1a = nullptr;
    bool grads = false;
};

}  // namespace

struct pps_unet {
    int c1, c2, c3;
    int linear = 0;        // 1: identity activations (a learned linear multigrid-like operator)
    int device = 0;
    cudaStream_t stream = nullptr;
    std::vector<Layer> L;
    size_t npad = 0, nreal = 0;
    float *P = nullptr, *G = nullptr, *M = nullptr, *V = nullptr;   // FP32 master, grads, Adam moments
    bf16* PB = nullptr;    // BF16 copy of the padded parameters
    bf16* WF = nullptr;    // flipped weights of one layer (backward data)
    float* dtmp = nullptr; // device scalar: rms of the input
    double* dloss = nullptr;
    int step = 0;
    Acts A;
};

namespace {

void free_acts(Acts& A)
{
    bf16* b[] = {A.x0, A.e1a, A.cat1, A.d1a, A.d1, A.p1, A.e2a, A.cat2, A.d2a, A.d2, A.p2, A.e3a, A.e3,
                 A.g_out, A.g_d1, A.g_d1a, A.g_cat1, A.g_d2, A.g_d2a, A.g_cat2, A.g_e3, A.g_e3a, A.g_p2,
                 A.g_e2a, A.g_p1, A.g_e1a};
    for (bf16* q : b)
        if (q) cudaFree(q);
    if (A.out) cudaFree(A.out);
    A = Acts();
}

// Zeroed on `s`, the stream whose kernels use the buffer next (the legacy stream's
// fills are not ordered with the library's non-blocking streams).
bf16* balloc(long long n, cudaStream_t s)
{
    bf16* p = nullptr;
    UK(cudaMalloc((void**)&p, sizeof(bf16) * (size_t)n));
    UK(cudaMemsetAsync(p, 0, sizeof(bf16) * (size_t)n, s));
    return p;
}

void ensure_acts(pps_unet* u, int nx, int ny, int nz, bool grads)
{
    Acts& A = u->A;
    if (A.s1.W == nx && A.s1.H == ny && A.s1.D == nz && (A.grads || !grads)) return;
    free_acts(A);
    A.s1 = Dims{nz, ny, nx};
    A.s2 = Dims{nz / 2, ny / 2, nx / 2};
    A.s3 = Dims{nz / 4, ny / 4, nx / 4};
    const long long v1 = (long long)nx * ny * nz, v2 = v1 / 8, v3 = v2 / 8;
    const int c1 = u->c1, c2 = u->c2, c3 = u->c3;
    A.x0 = balloc(v1 * 16, u->stream);
    A.e1a = balloc(v1 * c1, u->stream);
    A.cat1 = balloc(v1 * (c2 + c1), u->stream);
    A.d1a = balloc(v1 * c1, u->stream);
    A.d1 = balloc(v1 * c1, u->stream);
    A.p1 = balloc(v2 * c1, u->stream);
    A.e2a = balloc(v2 * c2, u->stream);
    A.cat2 = balloc(v2 * (c3 + c2), u->stream);
    A.d2a = balloc(v2 * c2, u->stream);
    A.d2 = balloc(v2 * c2, u->stream);
    A.p2 = balloc(v3 * c2, u->stream);
    A.e3a = balloc(v3 * c3, u->stream);
    A.e3 = balloc(v3 * c3, u->stream);
    UK(cudaMalloc((void**)&A.out, sizeof(float) * (size_t)v1 * 16));
    if (grads) {
        A.g_out = balloc(v1 * 16, u->stream);
        A.g_d1 = balloc(v1 * c1, u->stream);
        A.g_d1a = balloc(v1 * c1, u->stream);
        A.g_cat1 = balloc(v1 * (c2 + c1), u->stream);
        A.g_d2 = balloc(v2 * c2, u->stream);
        A.g_d2a = balloc(v2 * c2, u->stream);
        A.g_cat2 = balloc(v2 * (c3 + c2), u->stream);
        A.g_e3 = balloc(v3 * c3, u->stream);
        A.g_e3a = balloc(v3 * c3, u->stream);
        A.g_p2 = balloc(v3 * c2, u->stream);
        A.g_e2a = balloc(v2 * c2, u->stream);
        A.g_p1 = balloc(v2 * c1, u->stream);
        A.g_e1a = balloc(v1 * c1, u->stream);
        A.grads = true;
    }
}

const bf16* Wb(const pps_unet* u, int l) { return u->PB + u->L[(size_t)l].w; }
const float* Bf(const pps_unet* u, int l) { return u->P + u->L[(size_t)l].b; }

// The forward pass.  With `dense_out` (inference) the glue kernels fold into the
// convolutions next to them: the first reads the dense input scaled by 1/(*rms_dev),
// the two after an upsampling read the coarse tensor for the upsampled channels, and
// the last writes channel 0 times (*rms_dev) * gain into dense_out (the same values;
// A.x0, the upsampled slots of A.cat1/A.cat2 and A.out are then not written).
// Without it (training) every activation is stored for the backward pass.
void forward(pps_unet* u, const float* in, const float* rms_dev, float* dense_out = nullptr, float gain = 1.0f)
{
    Acts& A = u->A;
    cudaStream_t s = u->stream;
    const int c1 = u->c1, c2 = u->c2, c3 = u->c3;
    const long long v1 = (long long)A.s1.D * A.s1.H * A.s1.W;
    const bool R = !u->linear;
    const bool infer = dense_out != nullptr;
    ConvIO first, up2io, up1io, last;
    if (infer) {
        first.dense_in = in;
        first.rms = rms_dev;
        up2io.up = A.e3;
        up2io.ld_up = c3;
        up2io.c_up = c3;
        up1io.up = A.d2;
        up1io.ld_up = c2;
        up1io.c_up = c2;
        last.dense_out = dense_out;
        last.rms = rms_dev;
        last.gain = gain;
    } else {
        dense_to_act(v1, in, rms_dev, A.x0, 16, s);
    }
    conv(A.s1, A.x0, 16, 0, 16, Wb(u, 0), Bf(u, 0), A.e1a, c1, 0, c1, R, false, s, first);
    conv(A.s1, A.e1a, c1, 0, c1, Wb(u, 1), Bf(u, 1), A.cat1, c2 + c1, c2, c1, R, false, s);
    pool2(A.s2, A.cat1, c2 + c1, c2, A.p1, c1, s);
    conv(A.s2, A.p1, c1, 0, c1, Wb(u, 2), Bf(u, 2), A.e2a, c2, 0, c2, R, false, s);
    conv(A.s2, A.e2a, c2, 0, c2, Wb(u, 3), Bf(u, 3), A.cat2, c3 + c2, c3, c2, R, false, s);
    pool2(A.s3, A.cat2, c3 + c2, c3, A.p2, c2, s);
    conv(A.s3, A.p2, c2, 0, c2, Wb(u, 4), Bf(u, 4), A.e3a, c3, 0, c3, R, false, s);
    conv(A.s3, A.e3a, c3, 0, c3, Wb(u, 5), Bf(u, 5), A.e3, c3, 0, c3, R, false, s);
    if (!infer) up2(A.s2, A.e3, c3, A.cat2, c3 + c2, 0, s);
    conv(A.s2, A.cat2, c3 + c2, 0, c3 + c2, Wb(u, 6), Bf(u, 6), A.d2a, c2, 0, c2, R, false, s, up2io);
    conv(A.s2, A.d2a, c2, 0, c2, Wb(u, 7), Bf(u, 7), A.d2, c2, 0, c2, R, false, s);
    if (!infer) up2(A.s1, A.d2, c2, A.cat1, c2 + c1, 0, s);
    conv(A.s1, A.cat1, c2 + c1, 0, c2 + c1, Wb(u, 8), Bf(u, 8), A.d1a, c1, 0, c1, R, false, s, up1io);
    conv(A.s1, A.d1a, c1, 0, c1, Wb(u, 9), Bf(u, 9), A.d1, c1, 0, c1, R, false, s);
    conv(A.s1, A.d1, c1, 0, c1, Wb(u, 10), Bf(u, 10), A.out, 16, 0, 16, false, true, s, last);
}

// gradient of layer l: weights/bias from (X, G), then the data gradient Gin = conv(G, flip(W_l))
void layer_bwd(pps_unet* u, int l, const Dims& d, const bf16* X, int ldx, int cx0, const bf16* Gv, int ldg, int cg0,
               bf16* Gin, int ldgi, int cgi0)
{
    const Layer& Ly = u->L[(size_t)l];
    cudaStream_t s = u->stream;
    const long long nv = (long long)d.D * d.H * d.W;
    conv_wgrad(d, X, ldx, cx0, Ly.cin_p, Gv, ldg, cg0, Ly.cout_p, u->G + Ly.w, s);
    bias_grad(nv, Gv, ldg, cg0, Ly.cout_p, u->G + Ly.b, s);
    if (Gin) {
        flip(u->PB + Ly.w, u->WF, Ly.cin_p, Ly.cout_p, s);
        conv(d, Gv, ldg, cg0, Ly.cout_p, u->WF, nullptr, Gin, ldgi, cgi0, Ly.cin_p, false, false, s);
    }
}

void backward(pps_unet* u)
{
    Acts& A = u->A;
    cudaStream_t s = u->stream;
    const int c1 = u->c1, c2 = u->c2, c3 = u->c3;
    const long long v1 = (long long)A.s1.D * A.s1.H * A.s1.W, v2 = v1 / 8, v3 = v2 / 8;
    UK(cudaMemsetAsync(u->G, 0, sizeof(float) * u->npad, s));
    // out <- d1
    layer_bwd(u, 10, A.s1, A.d1, c1, 0, A.g_out, 16, 0, A.g_d1, c1, 0);
    if (!u->linear) relu_bwd(v1, A.g_d1, c1, 0, A.d1, c1, 0, c1, s);
    layer_bwd(u, 9, A.s1, A.d1a, c1, 0, A.g_d1, c1, 0, A.g_d1a, c1, 0);
    if (!u->linear) relu_bwd(v1, A.g_d1a, c1, 0, A.d1a, c1, 0, c1, s);
    layer_bwd(u, 8, A.s1, A.cat1, c2 + c1, 0, A.g_d1a, c1, 0, A.g_cat1, c2 + c1, 0);
    // up slot of cat1 -> d2
    up2_bwd(A.s2, A.g_cat1, c2 + c1, 0, A.g_d2, c2, s);
    if (!u->linear) relu_bwd(v2, A.g_d2, c2, 0, A.d2, c2, 0, c2, s);
    layer_bwd(u, 7, A.s2, A.d2a, c2, 0, A.g_d2, c2, 0, A.g_d2a, c2, 0);
    if (!u->linear) relu_bwd(v2, A.g_d2a, c2, 0, A.d2a, c2, 0, c2, s);
    layer_bwd(u, 6, A.s2, A.cat2, c3 + c2, 0, A.g_d2a, c2, 0, A.g_cat2, c3 + c2, 0);
    // up slot of cat2 -> e3
    up2_bwd(A.s3, A.g_cat2, c3 + c2, 0, A.g_e3, c3, s);
    if (!u->linear) relu_bwd(v3, A.g_e3, c3, 0, A.e3, c3, 0, c3, s);
    layer_bwd(u, 5, A.s3, A.e3a, c3, 0, A.g_e3, c3, 0, A.g_e3a, c3, 0);
    if (!u->linear) relu_bwd(v3, A.g_e3a, c3, 0, A.e3a, c3, 0, c3, s);
    layer_bwd(u, 4, A.s3, A.p2, c2, 0, A.g_e3a, c3, 0, A.g_p2, c2, 0);
    // pooling -> skip slot of cat2 (adds to the skip gradient of conv6)
    pool2_bwd(A.s3, A.g_p2, A.g_cat2, c3 + c2, c3, c2, s);
    if (!u->linear) relu_bwd(v2, A.g_cat2, c3 + c2, c3, A.cat2, c3 + c2, c3, c2, s);
    layer_bwd(u, 3, A.s2, A.e2a, c2, 0, A.g_cat2, c3 + c2, c3, A.g_e2a, c2, 0);
    if (!u->linear) relu_bwd(v2, A.g_e2a, c2, 0, A.e2a, c2, 0, c2, s);
    layer_bwd(u, 2, A.s2, A.p1, c1, 0, A.g_e2a, c2, 0, A.g_p1, c1, 0);
    pool2_bwd(A.s2, A.g_p1, A.g_cat1, c2 + c1, c2, c1, s);
    if (!u->linear) relu_bwd(v1, A.g_cat1, c2 + c1, c2, A.cat1, c2 + c1, c2, c1, s);
    layer_bwd(u, 1, A.s1, A.e1a, c1, 0, A.g_cat1, c2 + c1, c2, A.g_e1a, c1, 0);
    if (!u->linear) relu_bwd(v1, A.g_e1a, c1, 0, A.e1a, c1, 0, c1, s);
    layer_bwd(u, 0, A.s1, A.x0, 16, 0, A.g_e1a, c1, 0, nullptr, 0, 0);
}

pps_status check_dims(int nx, int ny, int nz)
{
    if (nx < 4 || ny < 4 || nz < 4 || nx % 4 || ny % 4 || nz % 4) {
        pps_internal_set_error("the U-Net needs every extent to be a multiple of 4 (two 2x poolings)");
        return PPS_ERR_INVALID_ARG;
    }
    return PPS_OK;
}

template <typename Fn>
pps_status uguard(Fn&& fn)
{
    const unsigned long long f0 = pps::launch_failures();
    try {
        const pps_status rc = fn();
        return rc >= 0 && pps::launch_failures() != f0 ? PPS_ERR_CUDA : rc;
    } catch (const UFail&) {
        return PPS_ERR_CUDA;
    } catch (const std::bad_alloc&) {
        pps_internal_set_error("host allocation failed");
        return PPS_ERR_OUT_OF_MEMORY;
    }
}

}  // namespace

// internal: run the forward pass on the U-Net's stream-independent buffers (used
// by the solver's learned preconditioner).  in/out dense [nz][ny][nx] FP32.
pps_status pps_internal_unet_apply(pps_unet* u, int nx, int ny, int nz, const float* in, float* out, float gain,
                                   cudaStream_t s)
{
    if (check_dims(nx, ny, nz) != PPS_OK) return PPS_ERR_INVALID_ARG;
    return uguard([&]() -> pps_status {
        cudaStream_t saved = u->stream;
        u->stream = s;
        ensure_acts(u, nx, ny, nz, false);
        const long long nv = (long long)nx * ny * nz;
        rms(nv, in, u->dtmp, s);
        forward(u, in, u->dtmp, out, gain);
        u->stream = saved;
        return PPS_OK;
    });
}

extern "C" {

pps_status pps_unet_create(int c1, int c2, int c3, unsigned long long seed, int device, pps_unet** out)
{
    if (!out || c1 < 16 || c2 < 16 || c3 < 16 || c1 % 16 || c2 % 16 || c3 % 16 || c3 + c2 > 96 || c2 + c1 > 96) {
        pps_internal_set_error("U-Net channels must be multiples of 16 with c3+c2 <= 96");
        return PPS_ERR_INVALID_ARG;
    }
    *out = nullptr;
    pps_unet* u = new (std::nothrow) pps_unet();
    if (!u) return PPS_ERR_OUT_OF_MEMORY;
    u->c1 = c1;
    u->c2 = c2;
    u->c3 = c3;
    const int spec[11][3] = {{1, c1, 1},  {c1, c1, 1}, {c1, c2, 1}, {c2, c2, 1},      {c2, c3, 1}, {c3, c3, 1},
                             {c3 + c2, c2, 1}, {c2, c2, 1}, {c2 + c1, c1, 1}, {c1, c1, 1}, {c1, 1, 0}};
    size_t off = 0, roff = 0;
    for (auto& sp : spec) {
        Layer l;
        l.cin = sp[0];
        l.cout = sp[1];
        l.relu = sp[2] != 0;
        l.cin_p = pad16(l.cin);
        l.cout_p = pad16(l.cout);
        l.w = off;
        off += (size_t)27 * l.cin_p * l.cout_p;
        l.b = off;
        off += (size_t)l.cout_p;
        l.rw = roff;
        roff += (size_t)27 * l.cin * l.cout;
        l.rb = roff;
        roff += (size_t)l.cout;
        u->L.push_back(l);
    }
    u->npad = off;
    u->nreal = roff;
    pps_status rc = uguard([&]() -> pps_status {
        UK(cudaSetDevice(device));
        u->device = device;
        UK(cudaStreamCreateWithFlags(&u->stream, cudaStreamNonBlocking));
        float** f[] = {&u->P, &u->G, &u->M, &u->V};
        for (float** q : f) {
            UK(cudaMalloc((void**)q, sizeof(float) * u->npad));
            UK(cudaMemsetAsync(*q, 0, sizeof(float) * u->npad, u->stream));
        }
        UK(cudaMalloc((void**)&u->PB, sizeof(bf16) * u->npad));
        UK(cudaMalloc((void**)&u->WF, sizeof(bf16) * 27 * 96 * 96));
        UK(cudaMalloc((void**)&u->dtmp, sizeof(float) * 4));
        UK(cudaMalloc((void**)&u->dloss, sizeof(double)));
        // He initialisation of the real weights, zero biases
        std::vector<float> h(u->npad, 0.0f);
        std::mt19937_64 rng(seed);
        for (const Layer& l : u->L) {
            std::normal_distribution<float> nd(0.0f, std::sqrt(2.0f / (27.0f * l.cin)));
            for (int t = 0; t < 27; t++)
                for (int ci = 0; ci < l.cin; ci++)
                    for (int co = 0; co < l.cout; co++)
                        h[l.w + ((size_t)t * l.cin_p + ci) * l.cout_p + co] = nd(rng) * (l.relu ? 1.0f : 0.1f);
        }
        UK(cudaMemcpyAsync(u->P, h.data(), sizeof(float) * u->npad, cudaMemcpyHostToDevice, u->stream));
        f32_to_bf16((long long)u->npad, u->P, u->PB, u->stream);
        UK(cudaStreamSynchronize(u->stream));
        return PPS_OK;
    });
    if (rc != PPS_OK) {
        pps_unet_destroy(u);
        return rc;
    }
    *out = u;
    return PPS_OK;
}

pps_status pps_unet_destroy(pps_unet* u)
{
    if (!u) return PPS_ERR_INVALID_ARG;
    cudaSetDevice(u->device);
    if (u->stream) cudaStreamSynchronize(u->stream);
    free_acts(u->A);
    void* p[] = {u->P, u->G, u->M, u->V, u->PB, u->WF, u->dtmp, u->dloss};
    for (void* q : p)
        if (q) cudaFree(q);
    if (u->stream) cudaStreamDestroy(u->stream);
    delete u;
    return PPS_OK;
}

int pps_unet_param_count(const pps_unet* u) { return u ? (int)u->nreal : -1; }

pps_status pps_unet_set_activation(pps_unet* u, int linear)
{
    if (!u || (linear != 0 && linear != 1)) return PPS_ERR_INVALID_ARG;
    u->linear = linear;
    return PPS_OK;
}

// Flat real-parameter layout: per layer W[27][cin][cout] (tap = kz*9+ky*3+kx) then b[cout].
static void pack(const pps_unet* u, const std::vector<float>& padded, float* real)
{
    for (const Layer& l : u->L) {
        for (int t = 0; t < 27; t++)
            for (int ci = 0; ci < l.cin; ci++)
                for (int co = 0; co < l.cout; co++)
                    real[l.rw + ((size_t)t * l.cin + ci) * l.cout + co] = padded[l.w + ((size_t)t * l.cin_p + ci) * l.cout_p + co];
        for (int co = 0; co < l.cout; co++) real[l.rb + co] = padded[l.b + co];
    }
}

pps_status pps_unet_get_params(const pps_unet* u, float* out)
{
    if (!u || !out) return PPS_ERR_INVALID_ARG;
    return uguard([&]() -> pps_status {
        UK(cudaSetDevice(u->device));
        std::vector<float> h(u->npad);
        UK(cudaMemcpyAsync(h.data(), u->P, sizeof(float) * u->npad, cudaMemcpyDeviceToHost, u->stream));
        UK(cudaStreamSynchronize(u->stream));
        pack(u, h, out);
        return PPS_OK;
    });
}

pps_status pps_unet_set_params(pps_unet* u, const float* in)
{
    if (!u || !in) return PPS_ERR_INVALID_ARG;
    return uguard([&]() -> pps_status {
        UK(cudaSetDevice(u->device));
        std::vector<float> h(u->npad, 0.0f);
        for (const Layer& l : u->L) {
            for (int t = 0; t < 27; t++)
                for (int ci = 0; ci < l.cin; ci++)
                    for (int co = 0; co < l.cout; co++)
                        h[l.w + ((size_t)t * l.cin_p + ci) * l.cout_p + co] = in[l.rw + ((size_t)t * l.cin + ci) * l.cout + co];
            for (int co = 0; co < l.cout; co++) h[l.b + co] = in[l.rb + co];
        }
        UK(cudaMemcpyAsync(u->P, h.data(), sizeof(float) * u->npad, cudaMemcpyHostToDevice, u->stream));
        UK(cudaMemsetAsync(u->M, 0, sizeof(float) * u->npad, u->stream));
        UK(cudaMemsetAsync(u->V, 0, sizeof(float) * u->npad, u->stream));
        u->step = 0;
        f32_to_bf16((long long)u->npad, u->P, u->PB, u->stream);
        UK(cudaStreamSynchronize(u->stream));
        return PPS_OK;
    });
}

pps_status pps_unet_forward(pps_unet* u, int nx, int ny, int nz, const float* in_dev, float* out_dev, int normalize)
{
    if (!u || !in_dev || !out_dev) return PPS_ERR_INVALID_ARG;
    if (check_dims(nx, ny, nz) != PPS_OK) return PPS_ERR_INVALID_ARG;
    return uguard([&]() -> pps_status {
        UK(cudaSetDevice(u->device));
        ensure_acts(u, nx, ny, nz, false);
        const long long nv = (long long)nx * ny * nz;
        const float* r = nullptr;
        if (normalize) {
            rms(nv, in_dev, u->dtmp, u->stream);
            r = u->dtmp;
        }
        forward(u, in_dev, r, out_dev, 1.0f);
        UK(cudaStreamSynchronize(u->stream));
        return PPS_OK;
    });
}

static pps_status loss_and_grads(pps_unet* u, int nx, int ny, int nz, const float* in, const float* target,
                                 double* loss)
{
    ensure_acts(u, nx, ny, nz, true);
    const long long nv = (long long)nx * ny * nz;
    forward(u, in, nullptr);
    UK(cudaMemsetAsync(u->dloss, 0, sizeof(double), u->stream));
    mse(nv, u->A.out, 16, target, u->A.g_out, 16, u->dloss, u->stream);
    backward(u);
    UK(cudaMemcpyAsync(loss, u->dloss, sizeof(double), cudaMemcpyDeviceToHost, u->stream));
    UK(cudaStreamSynchronize(u->stream));
    return PPS_OK;
}

pps_status pps_unet_gradients(pps_unet* u, int nx, int ny, int nz, const float* in_dev, const float* target_dev,
                              float* grads, double* loss)
{
    if (!u || !in_dev || !target_dev || !grads || !loss) return PPS_ERR_INVALID_ARG;
    if (check_dims(nx, ny, nz) != PPS_OK) return PPS_ERR_INVALID_ARG;
    return uguard([&]() -> pps_status {
        UK(cudaSetDevice(u->device));
        pps_status rc = loss_and_grads(u, nx, ny, nz, in_dev, target_dev, loss);
        if (rc != PPS_OK) return rc;
        std::vector<float> h(u->npad);
        UK(cudaMemcpyAsync(h.data(), u->G, sizeof(float) * u->npad, cudaMemcpyDeviceToHost, u->stream));
        UK(cudaStreamSynchronize(u->stream));
        pack(u, h, grads);
        return PPS_OK;
    });
}

pps_status pps_unet_train_step(pps_unet* u, int nx, int ny, int nz, const float* in_dev, const float* target_dev,
                               float lr, double* loss)
{
    if (!u || !in_dev || !target_dev || !loss || !(lr > 0.0f)) return PPS_ERR_INVALID_ARG;
    if (check_dims(nx, ny, nz) != PPS_OK) return PPS_ERR_INVALID_ARG;
    return uguard([&]() -> pps_status {
        UK(cudaSetDevice(u->device));
        pps_status rc = loss_and_grads(u, nx, ny, nz, in_dev, target_dev, loss);
        if (rc != PPS_OK) return rc;
        u->step += 1;
        rms((long long)u->npad, u->G, u->dtmp + 1, u->stream);   // global-norm clipping at 1
        adam((long long)u->npad, u->P, u->G, u->M, u->V, u->PB, lr, 0.9f, 0.999f, 1e-8f, u->step, u->dtmp + 1, 1.0f,
             u->stream);
        UK(cudaStreamSynchronize(u->stream));
        return PPS_OK;
    });
}

pps_status pps_restrict2(int nx, int ny, int nz, const float* fine_dev, float* coarse_dev)
{
    if (nx < 1 || ny < 1 || nz < 1 || ny > 32767 || nz > 32767 || !fine_dev || !coarse_dev) return PPS_ERR_INVALID_ARG;
    restrict2(Dims{nz, ny, nx}, fine_dev, coarse_dev, 0);
    return cudaGetLastError() == cudaSuccess && cudaDeviceSynchronize() == cudaSuccess ? PPS_OK : PPS_ERR_CUDA;
}

pps_status pps_prolong2(int nx, int ny, int nz, const float* coarse_dev, float* fine_dev)
{
    if (nx < 1 || ny < 1 || nz < 1 || ny > 32767 || nz > 32767 || !fine_dev || !coarse_dev) return PPS_ERR_INVALID_ARG;
    prolong2(Dims{nz, ny, nx}, coarse_dev, fine_dev, 0);
    return cudaGetLastError() == cudaSuccess && cudaDeviceSynchronize() == cudaSuccess ? PPS_OK : PPS_ERR_CUDA;
}

}  // extern "C"
