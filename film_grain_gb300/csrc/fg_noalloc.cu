// fg_noalloc.cu -- a pixel-wise render that allocates no device memory.
//
// Some callers cannot let a library allocate GPU memory: a host application that budgets all device
// memory itself and hands plug-ins only the buffers it owns, or a real-time preview loop that cannot
// afford cudaMalloc/cudaFree (which can block on the device and take driver locks) in the middle of
// a frame.  fg_render_pixelwise_noalloc serves them: the caller passes the lambda plane and the
// output plane (device memory); the kernel's scratch -- the per-input-pixel cell table, the device
// copy of the offsets and the diagnostic counters -- lives in one file-scope __device__ array of
// fixed size, so nothing is allocated at call time.  The array exists on every GPU that loads this
// library, from load until process exit.
//
// The host side only ever uses the array through the device address that cudaGetSymbolAddress
// returns for the current device (the symbol itself is a host-side stand-in, not a device address).
// That address is looked up on the first call made on each device and cached together with the
// unique ID of the CUDA context it belongs to; when the device's context is later destroyed and
// recreated (cudaDeviceReset, or another context made current), the ID changes and the next call
// looks the address up again instead of using a stale one.
#include <mutex>
#include <string>

#include <cuda.h>
#include <cuda_runtime.h>

#include "../../include/film_grain_gb300.h"
#include "fg_host.h"
#include "fg_internal.h"
#include "fg_kernels.cuh"

namespace fg {

constexpr size_t kNaCellsBytes = (size_t)FG_NOALLOC_MAX_INPUT_PIXELS * sizeof(CellParam);
constexpr size_t kNaOffsBytes = (size_t)FG_NOALLOC_MAX_SAMPLES * 2 * sizeof(float);
constexpr size_t kNaDiagBytes = kPwDiagWords * sizeof(unsigned long long);
constexpr size_t kNaScratchBytes = kNaCellsBytes + kNaOffsBytes + kNaDiagBytes;

// The shared scratch of every fg_render_pixelwise_noalloc call on a device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNaScratchBytes];

struct NoallocSlot {
    unsigned long long ctx_id;  // context the address belongs to (0: unknown, look up on every call)
    unsigned char *ptr;
};
static std::mutex g_noalloc_mu;
static NoallocSlot g_noalloc_slot[128];  // per device ordinal

// Unique ID of the calling thread's current CUDA context (0 when there is none or the driver
// entry points are unavailable).  The driver functions are reached through the runtime, so the
// library needs no link against the driver library.
static unsigned long long current_context_id() {
    typedef CUresult (*GetCurrentFn)(CUcontext *);
    typedef CUresult (*GetIdFn)(CUcontext, unsigned long long *);
    static GetCurrentFn get_current = nullptr;
    static GetIdFn get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<GetCurrentFn>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<GetIdFn>(f);
        cudaGetLastError();
    });
    if (!get_current || !get_id) return 0;
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (get_current(&ctx) != CUDA_SUCCESS || !ctx) return 0;
    if (get_id(ctx, &id) != CUDA_SUCCESS) return 0;
    return id;
}

// Device address of the scratch array on the current device and context, looked up once per
// device (again after its context changes).
static fg_status noalloc_scratch(unsigned char **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_error(e, "cudaGetDevice");
    if (dev < 0 || dev >= 128) return set_error(FG_ERR_UNSUPPORTED, "device ordinal out of range");
    const unsigned long long id = current_context_id();
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    NoallocSlot &slot = g_noalloc_slot[dev];
    if (!slot.ptr || id == 0 || slot.ctx_id != id) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_error(e, "cudaGetSymbolAddress of the scratch array");
        slot.ptr = static_cast<unsigned char *>(p);
        slot.ctx_id = id ? id : current_context_id();  // the lookup made the device's context current
    }
    *out = slot.ptr;
    return FG_OK;
}

}  // namespace fg

using namespace fg;

extern "C" FG_API fg_status fg_render_pixelwise_noalloc(const float *d_lambda, const fg_params *params,
                                                        const fg_derived *derived, const float *offsets_input,
                                                        float *d_out, void *stream) {
    fg_status st = check_render_args(params, derived);
    if (st != FG_OK) return st;
    if (!d_lambda || !offsets_input || !d_out) return set_error(FG_ERR_INVALID, "null buffer");
    const long long n_in = derived->input_width * derived->input_height;
    if (n_in > (long long)FG_NOALLOC_MAX_INPUT_PIXELS)
        return set_error(FG_ERR_UNSUPPORTED,
                         "input plane has " + std::to_string(n_in) + " pixels; the allocation-free render takes at most " +
                             std::to_string(FG_NOALLOC_MAX_INPUT_PIXELS));
    if (params->n_samples > FG_NOALLOC_MAX_SAMPLES)
        return set_error(FG_ERR_UNSUPPORTED, "n_samples " + std::to_string(params->n_samples) +
                                                 " exceeds the allocation-free render's maximum of " +
                                                 std::to_string(FG_NOALLOC_MAX_SAMPLES));
    if (!is_device_ptr(d_lambda) || !is_device_ptr(d_out))
        return set_error(FG_ERR_INVALID, "lambda and out must be device memory");
    if (is_device_ptr(offsets_input)) return set_error(FG_ERR_INVALID, "offsets_input must be host memory");
    unsigned char *scratch = nullptr;
    st = noalloc_scratch(&scratch);
    if (st != FG_OK) return st;
    CellParam *cells = reinterpret_cast<CellParam *>(scratch);
    float *offs = reinterpret_cast<float *>(scratch + kNaCellsBytes);
    unsigned long long *diag = reinterpret_cast<unsigned long long *>(scratch + kNaCellsBytes + kNaOffsBytes);
    cudaStream_t s = (cudaStream_t)stream;
    // The array keeps the previous call's contents: the offsets are overwritten here, the cell table
    // by the cell-parameter kernel, and the counters must start at zero.
    cudaError_t e = cudaMemcpyAsync(offs, offsets_input, sizeof(float) * 2 * params->n_samples,
                                    cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return cuda_error(e, "offsets H2D");
    e = cudaMemsetAsync(diag, 0, kNaDiagBytes, s);
    if (e != cudaSuccess) return cuda_error(e, "clear counters");
    st = enqueue_pixelwise(d_lambda, *params, *derived, offsets_input, offs, d_out, cells, diag, nullptr, s,
                           /*may_allocate=*/false);
    if (st == FG_OK) clear_error();
    return st;
}
