// hs_noalloc.cu -- an MSM entry point that allocates no device memory.
//
// Some callers cannot allocate device memory on the call path: code that runs
// under a memory pool or allocator that must not be bypassed, processes whose
// device memory is fully reserved ahead of time, and latency-critical callers
// that must not reach cudaMalloc/cudaFree (both can synchronise the device).
// For them hs_msm_device_noalloc runs the same device pipeline as
// hs_msm_device, but every scratch buffer it needs is carved from one
// file-scope device array of fixed size.
//
// When the array is reserved: with CUDA's lazy module loading (the default),
// the array of a device is reserved on the first call on that device, when
// cudaGetSymbolAddress loads this file's module; with CUDA_MODULE_LOADING=EAGER
// it is reserved when the library loads.  Either way it is held until the
// process exits.  A caller that reserves its device memory up front should
// make one call first.
#include <cuda_runtime.h>

#include <mutex>

#include "hs_internal.h"

namespace hs {

// 64 MiB of scratch per device.  In host code `g_noalloc_scratch` is only a
// stand-in symbol; its device address comes from cudaGetSymbolAddress below.
constexpr size_t NOALLOC_SCRATCH_BYTES = size_t(64) << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

constexpr int NOALLOC_MAX_DEVICES = 64;
static std::mutex g_noalloc_mu;
static void *g_noalloc_ptr[NOALLOC_MAX_DEVICES];

// With `device` current: the device address of the scratch array, looked up
// once per device.  A failed lookup is not cached, so a later call retries it.
static cudaError_t noalloc_scratch(int device, void **ptr)
{
    if (device < 0 || device >= NOALLOC_MAX_DEVICES)
        return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[device]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return e != cudaSuccess ? e : cudaErrorInvalidSymbol;
        g_noalloc_ptr[device] = p;
    }
    *ptr = g_noalloc_ptr[device];
    return cudaSuccess;
}

// The MSM descriptor reaches the device as a kernel argument, so the upload is
// ordered on the caller's stream like every other step and reads no host
// buffer after the call returns.
__global__ void k_put_desc(MsmDesc d, MsmDesc *out)
{
    if (blockIdx.x == 0 && threadIdx.x == 0)
        *out = d;
}

// a failure this call caused: its text for hs_last_error(NULL), the error cleared
static int noalloc_fail(cudaError_t e, const char *what)
{
    set_thread_error(std::string("hs_msm_device_noalloc: ") + what + ": " + cudaGetErrorString(e));
    cudaGetLastError();
    return HS_ECUDA;
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
    // An error left pending by the caller's own earlier work is not ours to
    // clear: refuse, and leave it for the caller to read.
    cudaError_t e = cudaPeekAtLastError();
    if (e != cudaSuccess) {
        set_thread_error(std::string("hs_msm_device_noalloc: a CUDA error was already pending: ") +
                         cudaGetErrorString(e));
        return HS_ECUDA;
    }
    int device = 0;
    if ((e = cudaGetDevice(&device)) != cudaSuccess)
        return noalloc_fail(e, "cudaGetDevice");
    void *scratch = nullptr;
    if ((e = noalloc_scratch(device, &scratch)) != cudaSuccess)
        return noalloc_fail(e, "scratch array address");
    // A stack context over the caller's stream: direct launches (no graph cache,
    // which would allocate), no profiling events, the scratch array as arena.
    Context ctx;
    ctx.device = device;
    ctx.stream = static_cast<cudaStream_t>(stream);
    ctx.use_graphs = false;
    ctx.ba_rounds[0] = ctx.ba_rounds[1] = 0;  // the entries' XYZZ accumulation: the smallest workspace
    if ((e = cudaDeviceGetAttribute(&ctx.sm_count, cudaDevAttrMultiProcessorCount, device)) != cudaSuccess)
        return noalloc_fail(e, "device attribute");
    if ((e = sort_smem_attrs(device)) != cudaSuccess)
        return noalloc_fail(e, "kernel attribute");
    const size_t sizes[1] = {n};
    BatchPlan p = make_batch_plan(ctx, curve, sizes, 1);
    p.global_sort = true;  // the smaller workspace: the fixed scratch array bounds it
    if (batch_bytes(p) > NOALLOC_SCRATCH_BYTES) {
        set_thread_error("hs_msm_device_noalloc: the workspace does not fit the scratch array");
        return HS_ERANGE;
    }
    ctx.arena.base = static_cast<char *>(scratch);
    ctx.arena.cap = NOALLOC_SCRATCH_BYTES;
    ctx.arena.off = 0;
    BatchBuffers b;
    const bool ok = carve(ctx.arena, p, b);
    ctx.arena.base = nullptr;  // the arena does not own the scratch: keep its destructor path inert
    ctx.arena.cap = 0;
    if (!ok) {
        set_thread_error("hs_msm_device_noalloc: the workspace does not fit the scratch array");
        return HS_ERANGE;
    }
    b.scalars = static_cast<const uint32_t *>(d_scalars);
    b.points = static_cast<const uint4 *>(d_points);
    // every buffer that must start at zero (bucket counters, heavy-bucket counter)
    // is cleared by the launch sequence itself; the descriptor is rewritten here
    k_put_desc<<<1, 32, 0, ctx.stream>>>(p.msms[0], b.desc);
    if ((e = cudaGetLastError()) != cudaSuccess)
        return noalloc_fail(e, "descriptor write");
    if ((e = launch_batch(ctx, p, b, d_out, out_fmt)) != cudaSuccess)
        return noalloc_fail(e, "MSM launch");
    return HS_OK;
}

}  // extern "C"
