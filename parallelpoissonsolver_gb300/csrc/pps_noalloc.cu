// pps_apply_operator_noalloc: the FP64 operator apply + energy reduction for
// callers that cannot allocate device memory.
//
// Who needs it: code that must not call cudaMalloc -- a real-time loop that
// forbids allocation after start-up, a plugin running inside a framework that owns
// all device memory through its own pool, or an application whose device-memory
// budget is fixed when it starts.  Those callers own their input and output
// buffers but cannot create a pps_solver, whose constructor allocates the work
// fields.
//
// The scratch array's device address is looked up on a device's first call and
// kept for the life of the process; cudaDeviceReset on that device invalidates it,
// so the entry point must not be used across a device reset.
//
// The kernel is k_stencil_dot<double> (the FP64 form's stencil + dot kernel).
// Its reduction scratch -- the scalar block, the block-completion counter and
// the per-block partial sums -- lives in the file-scope array below instead of
// in buffers a solver allocates.  The array exists once per GPU that loads the
// library and stays resident until the process exits.
#include "../../include/pps.h"
#include "pps_internal.h"

#include <cuda_runtime.h>

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <mutex>
#include <string>

using namespace pps;

namespace {

// Scratch layout: [0, 256) DevState, [256, 512) completion counter,
// [512, 512 + 32*PPS_NOALLOC_MAX_BLOCKS) block partials (4 doubles per block).
constexpr size_t kStateOffset = 0;
constexpr size_t kCounterOffset = 256;
constexpr size_t kPartialsOffset = 512;
constexpr size_t kScratchBytes = kPartialsOffset + (size_t)PPS_NOALLOC_MAX_BLOCKS * 4 * sizeof(double);
static_assert(sizeof(DevState) <= kCounterOffset - kStateOffset, "DevState must fit its slot");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned char* g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch array on the current device; looked up once per
// device (cudaGetSymbolAddress with that device current).
cudaError_t scratch_address(int dev, unsigned char** out)
{
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_ptr[dev]) {
        unsigned char* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress((void**)&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return cudaSuccess;
}

pps_status fail(pps_status st, const std::string& msg)
{
    pps_internal_set_error(msg.c_str());
    return st;
}

}  // namespace

extern "C" pps_status pps_apply_operator_noalloc(const pps_grid* grid, const double* u_dev, double* out_dev,
                                                 double* energy_dev, void* stream)
{
    if (!grid || !u_dev || !out_dev || !energy_dev)
        return fail(PPS_ERR_INVALID_ARG, "pps_apply_operator_noalloc: null argument");
    // Each thread reads u around its points while others write out, so an in-place
    // call (or any overlap, or energy inside either field) would read overwritten
    // values: rejected below, once the field size is known.
    Geo g;
    for (int d = 0; d < 3; d++) {
        if (grid->npglobal[d] < 3) return fail(PPS_ERR_INVALID_ARG, "npglobal must be >= 3 on every axis");
        if (!(grid->ds[d] > 0.0) || !std::isfinite(grid->ds[d]))
            return fail(PPS_ERR_INVALID_ARG, "ds must be positive");
        g.n[d] = grid->npglobal[d];
        g.ds[d] = grid->ds[d];
        g.lo[d] = 1 + (grid->bcs[2 * d] == 0 ? 1 : 0);
        g.hi[d] = grid->npglobal[d] + 1 - (grid->bcs[2 * d + 1] == 0 ? 1 : 0);
    }
    for (int f = 0; f < 6; f++) {
        if (grid->bcs[f] != 0 && grid->bcs[f] != 1)
            return fail(PPS_ERR_INVALID_ARG, "bcs must be 0 (Dirichlet) or 1 (Neumann)");
        g.bcs[f] = grid->bcs[f];
    }
    g.sj = grid->npglobal[0] + 2;
    g.sk = g.sj * (grid->npglobal[1] + 2);
    g.ntot = g.sk * (grid->npglobal[2] + 2);
    const Shape sh = make_shape(g, 8, sm_count() * 8 * 4);
    if (sh.nblocks() > (unsigned)PPS_NOALLOC_MAX_BLOCKS)
        return fail(PPS_ERR_INVALID_ARG, "pps_apply_operator_noalloc: the grid needs " +
                                             std::to_string(sh.nblocks()) + " blocks of partial sums; the "
                                             "static scratch holds " + std::to_string(PPS_NOALLOC_MAX_BLOCKS));
    {
        const uintptr_t nb = (uintptr_t)g.ntot * sizeof(double);
        const uintptr_t u0 = (uintptr_t)u_dev, o0 = (uintptr_t)out_dev, e0 = (uintptr_t)energy_dev;
        auto overlap = [](uintptr_t a, uintptr_t na, uintptr_t b, uintptr_t nb2) { return a < b + nb2 && b < a + na; };
        if (overlap(u0, nb, o0, nb) || overlap(e0, sizeof(double), u0, nb) || overlap(e0, sizeof(double), o0, nb))
            return fail(PPS_ERR_INVALID_ARG, "pps_apply_operator_noalloc: u, out and energy must not overlap");
    }

    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return fail(PPS_ERR_NO_DEVICE, "pps_apply_operator_noalloc: no usable current CUDA device");
    unsigned char* base = nullptr;
    cudaError_t e = scratch_address(dev, &base);
    if (e != cudaSuccess)
        return fail(PPS_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));

    cudaStream_t s = (cudaStream_t)stream;
    DevState* st = (DevState*)(base + kStateOffset);
    unsigned* counter = (unsigned*)(base + kCounterOffset);
    double* partials = (double*)(base + kPartialsOffset);
    // The array keeps the previous call's contents: reset the scalar block (done = 0)
    // and the completion counter, which the kernel needs at zero.
    const unsigned long long failures = launch_failures();
    state_init(st, nullptr, 0, 0.0, 0.0, 0, 0, 1.0, 0, s);
    e = cudaMemsetAsync(counter, 0, sizeof(unsigned), s);
    if (e != cudaSuccess) return fail(PPS_ERR_CUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));

    RedCtx rc;
    rc.partials = partials;
    rc.counter = counter;
    rc.st = st;
    rc.hist = nullptr;
    rc.kind = FIN_STORE;
    Coef a;
    const double ix = 1.0 / (g.ds[0] * g.ds[0]), iy = 1.0 / (g.ds[1] * g.ds[1]), iz = 1.0 / (g.ds[2] * g.ds[2]);
    a.cc = -2.0 * (ix + iy + iz);
    a.cx = ix;
    a.cy = iy;
    a.cz = iz;
    a.cb = a.cw = 0.0;
    a.scale = 1.0;
    // out = A u at the unknowns; sum u * (A u) over the unknowns into st->sums[0]
    fast_stencil_dot<double>(g, sh, u_dev, u_dev, out_dev, a, rc, s);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(PPS_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
    if (launch_failures() != failures) return PPS_ERR_CUDA;   // the message is set already
    e = cudaMemcpyAsync(energy_dev, &st->sums[0], sizeof(double), cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return fail(PPS_ERR_CUDA, std::string("cudaMemcpyAsync: ") + cudaGetErrorString(e));
    return PPS_OK;
}
