// Internal declarations of the learned preconditioner (U-Net) kernels.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <vector>

#include "../../include/pps.h"
#include "pps_internal.h"

namespace pps {
namespace unet {

struct Dims {
    int D, H, W;   // z, y, x extents of an activation grid
};

// Device stop flag that the forward and transfer kernels check on entry (a set flag
// makes them return at once); null (the default) while training or outside a solve.
void set_stop_flag(const int* done);

typedef __nv_bfloat16 bf16;

// Optional sources and sink of a convolution that replace the glue kernels of the
// inference pass (each gives the values the glue kernel would have stored):
//   dense_in: the input is a dense FP32 field scaled by 1/(*rms) (rms null: 1) in
//             channel 0 of 16, zeros elsewhere (dense_to_act);
//   up:       input channels [0, c_up) are the nearest 2x upsampling of `up`
//             (coarse grid, leading dimension ld_up; up2);
//   dense_out: channel 0 of the FP32 output, times (*rms) (rms null: 1) * gain, into
//             a dense field instead of Y (out_to_dense).
struct ConvIO {
    const float* dense_in = nullptr;
    const bf16* up = nullptr;
    int ld_up = 0, c_up = 0;
    float* dense_out = nullptr;
    const float* rms = nullptr;
    float gain = 1.0f;
};

// 3x3x3 zero-padded convolution on tensor cores (Cin, Cout multiples of 16).
void conv(const Dims& d, const bf16* X, int ldx, int cx0, int Cin, const bf16* W, const float* bias, void* Y, int ldy,
          int cy0, int Cout, bool relu, bool out_f32, cudaStream_t s, const ConvIO& io = ConvIO());
void conv_wgrad(const Dims& d, const bf16* X, int ldx, int cx0, int Cin, const bf16* G, int ldg, int cg0, int Cout,
                float* dW, cudaStream_t s);
void bias_grad(long long nv, const bf16* G, int ldg, int cg0, int Cout, float* db, cudaStream_t s);
void relu_bwd(long long nv, bf16* G, int ldg, int cg0, const bf16* Y, int ldy, int cy0, int C, cudaStream_t s);
void pool2(const Dims& dout, const bf16* in, int ldi, int ci0, bf16* out, int C, cudaStream_t s);
void pool2_bwd(const Dims& dout, const bf16* gout, bf16* gin, int ldi, int ci0, int C, cudaStream_t s);
void up2(const Dims& dfine, const bf16* in, int C, bf16* out, int ldo, int co0, cudaStream_t s);
void up2_bwd(const Dims& dcoarse, const bf16* gout, int ldo, int co0, bf16* gin, int C, cudaStream_t s);
void flip(const bf16* W, bf16* Wf, int Cin, int Cout, cudaStream_t s);
void mse(long long nv, const float* out, int ldo, const float* t, bf16* G, int ldg, double* loss, cudaStream_t s);
void adam(long long n, float* p, const float* g, float* m, float* v, bf16* pb, float lr, float b1, float b2, float eps,
          int step, const float* g_rms, float max_norm, cudaStream_t s);
void f32_to_bf16(long long n, const float* a, bf16* b, cudaStream_t s);
void dense_to_act(long long nv, const float* in, const float* rms, bf16* act, int ld, cudaStream_t s);
void out_to_dense(long long nv, const float* out, int ld, const float* rms, float gain, float* dense, cudaStream_t s);
void rms(long long n, const float* a, float* out, cudaStream_t s);

// Solver field (guard-padded, Dirichlet unknowns) <-> dense unknown arrays.
template <typename T>
void field_to_dense(const Geo& g, const T* f, float* dense, cudaStream_t s);
template <typename T>
void dense_to_field(const Geo& g, const float* dense, T* f, float scale, int add, cudaStream_t s);
// Transfers fused with the solver fields (Dirichlet unknowns of Geo g, guard cells
// zero): dense = r - A z; out = r - A z; x += y; coarse = R(r - A z) (R r when z is
// null) with the full weighting of restrict2; f += the trilinear prolongation of
// `coarse` (prolong2's weights).  Shape: the z-marching column tiles (cx = 1).
template <typename T>
void field_residual_dense(const Geo& g, const T* r, const T* z, float* dense, cudaStream_t s);
template <typename T>
void field_residual(const Geo& g, const Shape& sh, const T* r, const T* z, T* out, cudaStream_t s);
template <typename T>
void field_axpy(const Geo& g, const Shape& sh, T* x, const T* y, cudaStream_t s);
template <typename T>
void field_residual_restrict(const Geo& g, const T* r, const T* z, const Dims& dc, float* coarse, cudaStream_t s);
// f += P coarse at the unknowns.  With `dots` (flexible CG's z = M r finished by this
// prolongation) the FP32 float4 kernel also runs the z.r, z.Ap reduction `dots`
// describes over the unknowns and the call returns true; otherwise (FP64, unaligned
// rows, no `dots`) it returns false and the caller sums them.
template <typename T>
bool prolong_add_field(const Geo& g, const Shape& sh, const Dims& dc, const float* coarse, T* f, cudaStream_t s,
                       const T* r = nullptr, const T* Ap = nullptr, const RedCtx* dots = nullptr);
// 2x full-weighting restriction and trilinear prolongation of dense unknown arrays
// (prolong2_add: fine += P coarse).
void restrict2(const Dims& dc, const float* fine, float* coarse, cudaStream_t s);
void prolong2(const Dims& dc, const float* coarse, float* fine, cudaStream_t s);
void prolong2_add(const Dims& dc, const float* coarse, float* fine, cudaStream_t s);

// Coarse levels of the learned multigrid cycle.  Level l of an even fine grid puts
// its unknown c on the fine position 2^l (c+1) h: spacing H = 2^l h, the lower wall
// H below the first unknown, the upper wall only h above the last one.  The level
// operator is the 7-point second difference with that gap on the upper side: at the
// last unknown of an axis the lower neighbour weighs 2/(H (H+h)) and the centre
// -2/(H h) (the non-uniform three-point formula, wall value 0).
struct DLevel {
    float ih2[3];      // 1/H_d^2
    float last_m[3];   // 2/(H_d (H_d + h_d))
    float last_c[3];   // -2/(H_d h_d)
};
// Jacobi-scaled Chebyshev step coefficients, D = -diag(A):
// W (+)= scale (cy Y + D^-1 (cb B + ca A Y) + cz Z); y0 = 1/theta scales D^-1 B into
// the starting term when `first`.
struct LCoef {
    float cy, cb, ca, cz, scale, y0;
};
// W = B - A Y on the level
void level_residual(const Dims& d, const DLevel& L, const float* Y, const float* B, float* W, cudaStream_t s);
// R (B - A_l Y): level l's residual restricted to level l+1 (dims dc) in one pass
void level_residual_restrict(const Dims& dc, const DLevel& L, const float* Y, const float* B, float* coarse,
                             cudaStream_t s);
void level_cheb(const Dims& d, const DLevel& L, const float* Y, const float* B, const float* Z, float* W,
                const LCoef& c, bool first, bool acc, cudaStream_t s);
// Exact solve z = A_l^-1 r on a coarse level of at most LEVEL_EXACT_MAX unknowns per
// axis.  mats holds, per axis x, y, z of extents n_a, the 1-D level operator's
// eigenvector matrix V_a (n_a x n_a, row-major), its inverse and its eigenvalues:
// [Vx^-1, Vy^-1, Vz^-1, Vx, Vy, Vz, lam_x, lam_y, lam_z] (level_exact_data builds it).
constexpr int LEVEL_EXACT_MAX = 32;
void level_exact(const Dims& d, const float* mats, const float* r, float* z, cudaStream_t s);
// Host: mats of level_exact for level operator L on dims d (double eigen-solve,
// stored as float).  Returns false when an axis is longer than LEVEL_EXACT_MAX.
bool level_exact_data(const Dims& d, const DLevel& L, std::vector<float>& mats);
// Lets k_level_exact use the shared memory of a 32^3 level (current device).
cudaError_t level_exact_prepare();
// z = 0 on a dense level (the zero coarse correction)
void level_zero(const Dims& d, float* z, cudaStream_t s);

}  // namespace unet
}  // namespace pps

struct pps_unet;
// Forward pass of the network on dense [nz][ny][nx] FP32 arrays on stream s:
// out = gain * rms(in) * N(in / rms(in)).
pps_status pps_internal_unet_apply(pps_unet* u, int nx, int ny, int nz, const float* in, float* out, float gain,
                                   cudaStream_t s);
