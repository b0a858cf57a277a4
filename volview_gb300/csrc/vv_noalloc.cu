// vv_noalloc.cu — the a-trous denoiser on caller-provided device buffers,
// without allocating any device memory.
//
// Some callers cannot allocate device memory when they want a denoised image:
// a host application whose per-frame callback runs under a device-memory
// budget fixed at start-up (an allocation there can fail or stall the frame),
// or a process where another runtime owns every device allocation and hands
// out only buffers it manages. This entry point takes the accumulation images
// and the output from the caller and keeps its scratch images (the a-trous
// ping and pong and the guides) in a file-scope __device__ array instead.
//
// The array holds four images of NOALLOC_MAX_PIXELS pixels (512 x 512
// RGBA32F: ping, pong and the two edge-stopping guides, 4 x 4 MiB), and every
// device that loads the library keeps it until the process exits. Every call shares it: calls whose work overlaps on the GPU
// (different streams, or different host threads on one device) race on it.
// Each call overwrites every pixel of the scratch it uses before reading it,
// so nothing needs clearing between calls.
//
// The array exists once per CUDA context that loaded the library's module, so
// its device address is looked up once per context (the first call made with
// that context current; make it before any stream capture). A device reset
// while the library is loaded is not supported: the reset context's handle
// may come back with the array at another address.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/volpt.h"
#include "vv_kernels.h"

namespace vv {

// Largest image, in pixels, the allocation-free denoiser accepts.
constexpr size_t NOALLOC_MAX_PIXELS = 512 * 512;

// Ping and pong of the a-trous passes (denoise.comp bindings 20-21), then the
// per-pixel guides the passes read.
static __device__ __align__(256) float4 g_atrous_scratch[4 * NOALLOC_MAX_PIXELS];

// Device addresses of g_atrous_scratch, looked up once per CUDA context (a
// caller may run on a context of its own rather than the device's primary
// one, and each context holds its own copy of the array). In host code the
// array's name is only a host-side stand-in, never a device address.
struct ScratchEntry {
    int device;
    CUcontext context;
    float4* addr;
};
static std::mutex g_scratch_mutex;
static ScratchEntry g_scratch_addr[64] = {};
static int g_scratch_used = 0;
typedef CUresult (*CtxGetCurrent)(CUcontext*);

static cudaError_t scratch_for_current_context(float4** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    static CtxGetCurrent get_current = nullptr;
    if (!get_current) {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult found;
        e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000, cudaEnableDefault, &found);
        if (e != cudaSuccess) return e;
        if (found != cudaDriverEntryPointSuccess || !fn) return cudaErrorSymbolNotFound;
        get_current = (CtxGetCurrent)fn;
    }
    CUcontext ctx = nullptr;
    if (get_current(&ctx) != CUDA_SUCCESS) return cudaErrorDeviceUninitialized;
    for (int i = 0; ctx && i < g_scratch_used; i++) {
        if (g_scratch_addr[i].device == dev && g_scratch_addr[i].context == ctx) {
            *out = g_scratch_addr[i].addr;
            return cudaSuccess;
        }
    }
    // No context yet on this thread: the lookup itself makes the runtime's
    // (primary) context current, which is then the one the address belongs to.
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_atrous_scratch);
    if (e != cudaSuccess) return e;
    if (!ctx && (get_current(&ctx) != CUDA_SUCCESS || !ctx)) return cudaErrorDeviceUninitialized;
    if (g_scratch_used < 64) g_scratch_addr[g_scratch_used++] = {dev, ctx, (float4*)p};
    *out = (float4*)p;
    return cudaSuccess;
}

vv_status internal_fail(vv_status s, const std::string& msg);

}  // namespace vv

using namespace vv;

extern "C" vv_status vv_denoise_atrous_noalloc(const float* accum, const float* albedo, const float* normal,
                                               uint16_t* hdr, uint32_t width, uint32_t height, uint32_t samples,
                                               void* stream) {
    if (!accum || !albedo || !normal || !hdr) return internal_fail(VV_ERR_ARG, "null buffer");
    // The kernels read the images as float4 and write the output as 4 halves:
    // a sub-view that is not aligned to that would fault on the device.
    if (((uintptr_t)accum | (uintptr_t)albedo | (uintptr_t)normal) % 16 != 0 || (uintptr_t)hdr % 8 != 0)
        return internal_fail(VV_ERR_ARG, "accum, albedo and normal must be 16-byte aligned, hdr 8-byte aligned");
    if (width == 0 || height == 0 || samples == 0) return internal_fail(VV_ERR_ARG, "empty image or no samples");
    if ((size_t)width * height > NOALLOC_MAX_PIXELS)
        return internal_fail(VV_ERR_LIMIT, "the allocation-free denoiser takes at most " +
                                               std::to_string(NOALLOC_MAX_PIXELS) + " pixels (512 x 512); got " +
                                               std::to_string((size_t)width * height));
    // An error some earlier work left on this thread is reported as such, not
    // as a failure of this call's launches.
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return internal_fail(VV_ERR_CUDA, std::string("pending CUDA error before the call: ") + cudaGetErrorString(e));
    float4* scratch = nullptr;
    e = scratch_for_current_context(&scratch);
    if (e != cudaSuccess) return internal_fail(VV_ERR_CUDA, std::string("scratch address: ") + cudaGetErrorString(e));
    PostArgs a;
    memset(&a, 0, sizeof(a));
    a.u.path[0] = samples;  // samples() of denoise.comp is path.x + path.z
    a.width = width;
    a.height = height;
    a.accum = (const float4*)accum;
    a.albedo = (const float4*)albedo;
    a.normal = (const float4*)normal;
    a.ping = scratch;
    a.pong = scratch + NOALLOC_MAX_PIXELS;
    a.guide_nd = scratch + 2 * NOALLOC_MAX_PIXELS;
    a.guide_alb = scratch + 3 * NOALLOC_MAX_PIXELS;
    a.hdr = (ushort4*)hdr;
    int launches = 0;
    e = launch_denoise(a, (cudaStream_t)stream, &launches);
    if (e != cudaSuccess) return internal_fail(VV_ERR_CUDA, std::string("denoise launch: ") + cudaGetErrorString(e));
    return VV_OK;
}
