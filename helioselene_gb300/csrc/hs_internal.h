// hs_internal.h -- host-side runtime shared by the translation units of the library.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/helioselene_gb300.h"

namespace hs {

// Grow-only device arena.  A call reserves what it needs up front (reserve may
// reallocate, which synchronises the device), then carves buffers with take().
struct DeviceArena {
    char *base = nullptr;
    size_t cap = 0;
    size_t off = 0;
    cudaError_t reserve(size_t bytes);
    void *take(size_t bytes);
    void reset() { off = 0; }
    void release();
};

struct WindowRule {
    size_t n_min, n_max;
    int c;
};

struct Context {
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    DeviceArena arena;
    std::mutex mu;
    std::string last_error;
    uint64_t launches = 0;
    std::vector<WindowRule> rules[2];
    // instrumentation (hs_profile_*)
    bool profile = false;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> prof_events;
    uint64_t prof_entries = 0;
    double prof_ms = 0.0;
    uint64_t prof_launches = 0;
};

// events around the dominant kernel when profiling is on
void prof_begin(Context &ctx, cudaEvent_t *ev);
void prof_end(Context &ctx, cudaEvent_t ev0, uint64_t entries);

// Pippenger plan for one MSM of n points with c-bit signed windows.
struct MsmPlan {
    int curve = 0;
    uint32_t n = 0;
    int c = 0;           // window bits
    uint32_t W = 0;      // windows = ceil(257 / c)
    uint32_t B = 0;      // buckets per window = 2^(c-1)
    uint32_t NB = 0;     // W * B
    uint32_t L = 0;      // max entries per accumulation segment
    uint32_t max_entries = 0;
    uint32_t max_segs = 0;
    uint32_t hist_blocks = 0;  // blocks of the segment-length histogram
    uint32_t m0 = 0;     // buckets per thread in the bucket reduction
};

// Device buffers of one MSM (all carved from the arena).
struct MsmBuffers {
    const uint32_t *scalars = nullptr;  // n * 8 words
    const uint4 *points = nullptr;      // n * 4 uint4 (affine x || y)
    uint32_t *counts = nullptr;         // NB + 1 (later reused as fill cursors)
    uint32_t *offsets = nullptr;        // NB + 1, exclusive scan of counts
    uint32_t *seg_off = nullptr;        // NB + 1, exclusive scan of segment counts
    uint32_t *scan_tmp = nullptr;       // per-block partials of the scan
    uint32_t *sorted = nullptr;         // max_entries: point index | sign << 31
    uint4 *segs = nullptr;              // max_segs: (start, length, destination slot, 0), longest first
    uint32_t *len_hist = nullptr;       // (L+1) x hist blocks: segment-length histogram, then its scan
    uint32_t *len_scan = nullptr;       // exclusive scan of len_hist (+1 total)
    uint4 *seg_sum = nullptr;           // max_segs XYZZ sums (8 uint4 each)
    uint32_t *heavy = nullptr;          // NB heavy-bucket list
    uint32_t *heavy_n = nullptr;        // 1 counter
    uint4 *redA = nullptr;              // W * (B / m0) weighted group sums
    uint4 *redR = nullptr;              // W window sums
    uint32_t *out_jac = nullptr;        // 24 words: canonical Jacobian X, Y, Z
};

MsmPlan make_plan(const Context &ctx, int curve, size_t n);
size_t plan_bytes(const MsmPlan &p);
void carve(DeviceArena &a, const MsmPlan &p, MsmBuffers &b);

// curve-independent launches (hs_runtime.cu)
cudaError_t launch_sort(Context &ctx, const MsmPlan &p, const MsmBuffers &b);

// per-curve entry points (hs_curve_helios.cu / hs_curve_selene.cu)
struct CurveOps {
    // buckets -> window sums -> canonical Jacobian in b.out_jac (after launch_sort)
    cudaError_t (*msm_tail)(Context &ctx, const MsmPlan &p, const MsmBuffers &b);
    // jac51 / affine51 / affine input -> device affine (n * 64 bytes); scalars of
    // identity points are left alone (the accumulator skips (0,0) bases)
    cudaError_t (*to_affine)(Context &ctx, const void *d_in, int fmt, size_t n, uint4 *d_out, void *scratch);
    size_t (*to_affine_scratch)(size_t n);
    // count canonical Jacobians (24 words each) -> out_fmt
    cudaError_t (*format_out)(Context &ctx, const uint32_t *d_jac, size_t count, int out_fmt, void *d_out);
    cudaError_t (*map_to_curve)(Context &ctx, const void *d_u, size_t n, uint4 *d_out);
    // any point format -> canonical Jacobian, 24 words per point
    cudaError_t (*to_jac24)(Context &ctx, const void *d_in, int fmt, size_t n, uint32_t *d_out);
    // element-wise field op over n 32-byte values (validation hook)
    cudaError_t (*field_op)(Context &ctx, int op, const void *d_a, const void *d_b, size_t n, void *d_out);
};
extern const CurveOps helios_ops;
extern const CurveOps selene_ops;
const CurveOps &curve_ops(int curve);

size_t fmt_bytes(int fmt);

#define HS_LAUNCH_CHECK(ctx)                                 \
    do {                                                     \
        (ctx).launches++;                                    \
        cudaError_t e__ = cudaGetLastError();                \
        if (e__ != cudaSuccess)                              \
            return e__;                                      \
    } while (0)

}  // namespace hs
