// hs_noalloc.cu -- an MSM entry point that allocates no device memory.
//
// Some callers cannot allocate device memory on the call path: code that runs
// under a memory pool or allocator that must not be bypassed, processes whose
// device memory is fully reserved ahead of time, and real-time or graph-driven
// callers that must not hit cudaMalloc/cudaFree (they synchronise the device).
// For them hs_msm_device_noalloc runs the same device pipeline as
// hs_msm_device, but every scratch buffer it needs is carved from one
// file-scope device array of fixed size, reserved when the library's module is
// loaded on a device and held until the process exits.
#include <cuda_runtime.h>

#include <mutex>

#include "hs_internal.h"

namespace hs {

// 64 MiB of scratch per device.  In host code `g_noalloc_scratch` is only a
// stand-in symbol; its device address comes from cudaGetSymbolAddress below.
constexpr size_t NOALLOC_SCRATCH_BYTES = size_t(64) << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

constexpr int NOALLOC_MAX_DEVICES = 64;
static std::once_flag g_noalloc_once[NOALLOC_MAX_DEVICES];
static void *g_noalloc_ptr[NOALLOC_MAX_DEVICES];
static cudaError_t g_noalloc_err[NOALLOC_MAX_DEVICES];

// once per device, with that device current: the device address of the scratch array
static cudaError_t noalloc_scratch(int device, void **ptr)
{
    if (device < 0 || device >= NOALLOC_MAX_DEVICES)
        return cudaErrorInvalidDevice;
    std::call_once(g_noalloc_once[device], [device] {
        g_noalloc_err[device] = cudaGetSymbolAddress(&g_noalloc_ptr[device], g_noalloc_scratch);
        if (g_noalloc_err[device] != cudaSuccess) {
            g_noalloc_ptr[device] = nullptr;
            cudaGetLastError();
        }
    });
    *ptr = g_noalloc_ptr[device];
    return g_noalloc_err[device];
}

}  // namespace hs

using namespace hs;

extern "C" {

size_t hs_msm_noalloc_scratch_bytes(void) { return NOALLOC_SCRATCH_BYTES; }

int hs_msm_device_noalloc(int curve, const void *d_scalars, const void *d_points, size_t n, void *d_out, int out_fmt,
                          void *stream)
{
    if ((curve != HS_HELIOS && curve != HS_SELENE) || out_fmt < HS_FMT_JACOBIAN51 || out_fmt > HS_FMT_COMPRESSED ||
        !d_out || (n && (!d_scalars || !d_points)))
        return HS_EINVAL;
    if (n == 0 || n > HS_NOALLOC_MAX_POINTS)
        return HS_ERANGE;
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess) {
        cudaGetLastError();
        return HS_ECUDA;
    }
    void *scratch = nullptr;
    if (noalloc_scratch(device, &scratch) != cudaSuccess || !scratch)
        return HS_ECUDA;
    // A stack context over the caller's stream: direct launches (no graph cache,
    // which would allocate), no profiling events, the scratch array as arena.
    Context ctx;
    ctx.device = device;
    ctx.stream = static_cast<cudaStream_t>(stream);
    ctx.use_graphs = false;
    if (cudaDeviceGetAttribute(&ctx.sm_count, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
        sort_smem_attrs(device) != cudaSuccess) {
        cudaGetLastError();
        return HS_ECUDA;
    }
    const size_t sizes[1] = {n};
    BatchPlan p = make_batch_plan(ctx, curve, sizes, 1);
    p.global_sort = true;  // the smaller workspace: the fixed scratch array bounds it
    if (batch_bytes(p) > NOALLOC_SCRATCH_BYTES)
        return HS_ERANGE;
    ctx.arena.base = static_cast<char *>(scratch);
    ctx.arena.cap = NOALLOC_SCRATCH_BYTES;
    ctx.arena.off = 0;
    BatchBuffers b;
    const bool ok = carve(ctx.arena, p, b);
    ctx.arena.base = nullptr;  // the arena does not own the scratch: keep its destructor path inert
    ctx.arena.cap = 0;
    if (!ok)
        return HS_ERANGE;
    b.scalars = static_cast<const uint32_t *>(d_scalars);
    b.points = static_cast<const uint4 *>(d_points);
    // every buffer that must start at zero (bucket counters, heavy-bucket counter)
    // is cleared by the launch sequence itself; the descriptors are rewritten here
    cudaError_t e = cudaMemcpyAsync(b.desc, p.msms.data(), p.msms.size() * sizeof(MsmDesc),
                                    cudaMemcpyHostToDevice, ctx.stream);
    if (e == cudaSuccess)
        e = launch_batch(ctx, p, b, d_out, out_fmt);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return HS_ECUDA;
    }
    return HS_OK;
}

}  // extern "C"
