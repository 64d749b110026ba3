// noalloc.cu -- pd_apply_operator_noalloc: the system operator without any
// device allocation.
//
// Some callers cannot call cudaMalloc: a host application that owns every
// device allocation (its own pool or arena) and hands libraries only pointers
// into it, or code that must not allocate inside a time-critical loop.  This
// entry point applies the operator described by a pd_operator_view to
// vectors the caller provides, using for its reduction scratch only a fixed
// array in this library's static device memory.
//
// The scratch holds one FP64 partial sum per thread block (at most
// kNoAllocMaxBlocks blocks) and the blocks' arrival counter, ~33 KB on every
// GPU that loads the library, kept until the process exits.  Every call
// shares it and it keeps the last call's contents; the counter, which must
// start at zero, is cleared on the call's stream before each launch.  Calls
// whose launches overlap on the GPU race on the shared scratch.
//
// The scratch's device address is resolved once per device ordinal, in the
// runtime's primary context, and kept: after cudaDeviceReset, or from a
// context other than the primary one, the kept address is not valid.  The
// view's arrays must live on the current device (checked per call).
#include <mutex>
#include <string>

#include "pd_gb300.h"
#include "pd_kernels.h"

namespace pdgb {
void set_handleless_error(const std::string& msg);   // capi.cpp

namespace {

constexpr int kNoAllocMaxBlocks = 4096;
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_partials[kNoAllocMaxBlocks];
static __device__ __align__(256) unsigned int g_noalloc_counter[64];

// In host code the array names are host-side stand-ins, not device
// addresses; the device addresses are looked up once per device.
struct DeviceScratch {
    double* partials = nullptr;
    unsigned int* counter = nullptr;
    bool ready = false;
};
DeviceScratch g_scratch[kNoAllocMaxDevices];
std::mutex g_scratch_mutex;

// Set-up on the first call on the current device: resolve the scratch's
// device addresses with that device current.
cudaError_t scratch_for_current_device(DeviceScratch* out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kNoAllocMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    DeviceScratch& s = g_scratch[dev];
    if (!s.ready) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_partials);
        if (e != cudaSuccess) return e;
        s.partials = (double*)p;
        e = cudaGetSymbolAddress(&p, g_noalloc_counter);
        if (e != cudaSuccess) return e;
        s.counter = (unsigned int*)p;
        s.ready = true;
    }
    *out = s;
    return cudaSuccess;
}

pd_status reject(const std::string& msg)
{
    set_handleless_error("pd_apply_operator_noalloc: " + msg);
    return PD_ERR_INVALID_ARGUMENT;
}

}  // namespace
}  // namespace pdgb

extern "C" pd_status pd_apply_operator_noalloc(const pd_operator_view* v, const void* d_x, void* d_y,
                                               double* d_dot, void* stream)
{
    using namespace pdgb;
    if (!v) return reject("view is NULL");
    if (v->n < 0) return reject("n < 0");
    const int lanes = v->lanes_per_particle;
    if (lanes != 4 && lanes != 8 && lanes != 16 && lanes != 32) return reject("lanes_per_particle must be 4, 8, 16 or 32");
    if (v->precision != PD_PRECISION_MIXED && v->precision != PD_PRECISION_FP64) return reject("unknown precision");
    if (v->blocks < 0 || v->blocks > kNoAllocMaxBlocks)
        return reject("blocks must be 0 (automatic) or at most 4096, the size of the static scratch");
    const bool fp64 = v->precision == PD_PRECISION_FP64;
    if (v->n > 0) {
        if (!d_x || !d_y || !v->activity || !v->row_ptr || !v->bond_count || !v->bond_slot)
            return reject("a required device pointer is NULL");
        if (fp64 ? (!v->jac || !v->jac_diag) : (!v->ref_pos || !v->disp || !v->pos_cell || !v->inv_d0))
            return reject("the view lacks the arrays of its precision mode");
    }
    DeviceScratch scratch;
    cudaError_t e = scratch_for_current_device(&scratch);
    if (e != cudaSuccess) {
        set_handleless_error(std::string("pd_apply_operator_noalloc: scratch set-up: ") + cudaGetErrorString(e));
        cudaGetLastError();
        return PD_ERR_CUDA;
    }
    if (v->n > 0) {   // the view's arrays must be on the current device (the scratch is per device)
        int dev = 0;
        cudaPointerAttributes attr{};
        if (cudaGetDevice(&dev) == cudaSuccess && cudaPointerGetAttributes(&attr, v->row_ptr) == cudaSuccess &&
            attr.type == cudaMemoryTypeDevice && attr.device != dev)
            return reject("the view's arrays are on device " + std::to_string(attr.device) + ", the current device is " +
                          std::to_string(dev));
        cudaGetLastError();
    }
    StepParams P{};
    P.n = v->n;
    P.mass = v->mass;
    P.t2 = v->t2;
    P.bond_coeff = v->bond_coeff;
    for (int k = 0; k < 3; ++k) P.sphere_c_local[k] = v->sphere_center_local[k];
    P.sphere_k = v->sphere_stiffness;
    DeviceState S{};
    S.n = v->n;
    S.act = const_cast<uint8_t*>(v->activity);
    S.row_ptr = const_cast<int*>(v->row_ptr);
    S.cnt = const_cast<int*>(v->bond_count);
    S.col = const_cast<int*>(v->bond_slot);
    S.X32 = (float4*)const_cast<void*>(v->ref_pos);
    S.u32 = (float4*)const_cast<void*>(v->disp);
    S.xs4 = (float4*)const_cast<void*>(v->pos_cell);
    S.inv_d0 = const_cast<float*>(v->inv_d0);
    P.sup = v->supercell_size;
    P.inv_sup = v->supercell_size > 0 ? 1.0 / v->supercell_size : 0.0;
    S.jac = const_cast<double*>(v->jac);
    S.jdiag = const_cast<double*>(v->jac_diag);
    int grid = v->blocks;
    if (grid == 0) {
        const long long rows_per_block = kBlock / lanes;
        long long g = ((long long)v->n + rows_per_block - 1) / rows_per_block;
        grid = (int)(g < 1 ? 1 : (g > kNoAllocMaxBlocks ? kNoAllocMaxBlocks : g));
    }
    cudaStream_t st = (cudaStream_t)stream;
    e = cudaMemsetAsync(scratch.counter, 0, sizeof(unsigned int), st);
    if (e == cudaSuccess) {
        ReduceSlot slot{scratch.partials, scratch.counter};
        launch_operator(fp64, P, S, lanes, grid, d_x, d_y, slot, d_dot, st);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) {
        set_handleless_error(std::string("pd_apply_operator_noalloc: ") + cudaGetErrorString(e));
        return PD_ERR_CUDA;
    }
    return PD_OK;
}
