// hs_internal.h -- host-side runtime shared by the translation units of the library.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
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
    // When set, the arena is allocated and freed in the order of this stream
    // (stream-ordered allocator), so growing it does not synchronise the device
    // and stall the work of other streams.
    cudaStream_t ordered = nullptr;
    cudaError_t reserve(size_t bytes);
    void *take(size_t bytes);
    void reset() { off = 0; }
    void release();
};

// A size class's window width and, when ba_rounds >= 0, its batch-affine
// rounds (a plan takes the rounds of the class holding most of its entries).
struct WindowRule {
    size_t n_min, n_max;
    int c;
    int ba_rounds = -1;
};

// A captured launch sequence, replayed when the same batch shape runs again on
// the same buffers.
struct GraphEntry {
    std::vector<uint64_t> key;
    cudaGraphExec_t exec = nullptr;
    uint64_t kernels = 0;
    void *d_desc = nullptr;  // the batch descriptors, uploaded once at capture
};

// the library's batch-affine default for a curve's plans: one round on
// Helios, two on Selene (Context: the kinds of plans that take their own
// until hs_context_set_batch_affine sets the curve)
constexpr uint32_t BA_DEFAULT_ROUNDS[2] = {1, 2};
constexpr uint64_t BA_DEFAULT_MIN_ENTRIES = uint64_t(1) << 21;

struct Context {
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;   // the stream every launch goes to
    cudaStream_t stream2 = nullptr;  // second curve group of a mixed batch, lower window half of a split MSM
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;  // fork/join of the two streams (created with stream2)
    // host-input path (created with stream2): inputs arrive on the device's link
    // stream, the bases are converted on stream3
    cudaStream_t stream3 = nullptr;
    cudaEvent_t ev_sc = nullptr;   // scalars on the device
    cudaEvent_t ev_rec[2] = {};    // input records on the device (per part)
    cudaEvent_t ev_pts[2] = {};    // affine bases ready (per part)
    bool use_graphs = true;
    // the device reads pageable host memory directly (cudaDevAttrPageableMemoryAccess):
    // host inputs in pageable memory are then pulled by a copy kernel (h2d_async)
    bool pageable_access = false;
    // set while a launch sequence of host inputs is being captured: waits on the
    // input events (recorded outside the capture) become external event waits
    bool capturing_host = false;
    size_t split_min = size_t(1) << 18;  // single MSMs this large run as two window halves (0: never)
    // Batch-affine accumulation per curve: rounds (0: off) for plans of at
    // least ba_min_entries entries.  Measured at n = 2^20 on GB300
    // (accumulation per MSM, ms): Selene 2.54 -> 2.29 with one round, 2.27
    // with two; Helios 1.55 -> 1.56 with one.  For a Helios and a Selene MSM
    // side by side on two streams, back to back (the throughput form): 4.78
    // ms per pair with one round on Helios and two on Selene, 5.07 with one on
    // both, 5.06 with none on Helios: one curve's memory-bound rounds overlap
    // the other's multiply-bound work.
    uint32_t ba_rounds[2] = {BA_DEFAULT_ROUNDS[0], BA_DEFAULT_ROUNDS[1]};
    uint64_t ba_min_entries[2] = {BA_DEFAULT_MIN_ENTRIES, BA_DEFAULT_MIN_ENTRIES};
    // Until hs_context_set_batch_affine sets a curve, two kinds of plans take
    // their own rounds, because there a curve's MSMs run mostly alone, where
    // the round pays on Selene only:
    // - fixed-base commitments (4096 over 2^20 generators on GB300: Helios 617
    //   commitments/s without a round, 568 with; Selene 397 without, 427 with);
    // - single MSMs from host buffers, whose accumulation is pipelined with
    //   the link (a Helios and a Selene call of 2^20 points from two host
    //   threads: 6.06 ms per pair with one round on both, 5.91 ms without one
    //   on Helios).
    bool ba_set[2] = {false, false};
    uint32_t fixed_ba_rounds[2] = {0, 1};
    uint32_t host_ba_rounds[2] = {0, 1};
    std::vector<GraphEntry> graphs;
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

// One MSM inside a batch (device-visible; every MSM of a batch is on the same curve).
// Its points and scalars sit at [pt_off, pt_off + n) of the batch's concatenated
// arrays; its W x B buckets at [bucket_base, bucket_base + W*B) of the batch's
// bucket space; its W * (B/m0) reduction groups at group_base; its W window
// sums at win_base.
// buckets per level-1 reduction group (k_reduce_groups), and groups per
// level-2 chunk (k_window_chunks)
constexpr uint32_t RED_GROUP = 8;
constexpr uint32_t RED_CHUNK = 256;

// A fixed-base MSM (fixed = 1) reads its bases from a table of window
// multiples 2^(c k) G_i stored at index i*W + k: every window then adds into
// the same B buckets, so it reduces Wr = 1 window and needs no Horner step.
// With fixed = 2 its points are rows of such a table named by an index list
// (BatchBuffers::pt_idx): point pt_off + j of the batch is generator
// pt_idx[pt_off + j] of the table.
struct MsmDesc {
    uint32_t pt_off, n;
    uint32_t c, W, B;
    uint32_t bucket_base;
    uint32_t group_base, m0, log2m0, T;  // T = B / m0 groups per window
    uint32_t win_base;
    uint32_t fixed;   // 1: bases from a window-multiple table, 2: table rows named by BatchBuffers::pt_idx
    uint32_t Wr;      // windows that are reduced and combined (W, or 1 for fixed-base)
    uint32_t w_lo;    // first window this descriptor emits (a window-split half starts above 0)
    uint32_t w_cnt;   // windows emitted: [w_lo, w_lo + w_cnt)
    uint32_t shift;   // doublings applied after the Horner step (c * w_lo for an upper half)
    uint32_t chunk_base;  // first level-2 reduction chunk (Wr * max(1, T / RED_CHUNK) per MSM)
    uint32_t slices;      // counting sort: point slices per emitted window (one block each)
    uint32_t sblk_base;   // first counting-sort block of this MSM (w_cnt * slices blocks)
    uint32_t cnt_base;    // first per-block bucket count of this MSM
    uint32_t dig_base;    // first signed digit of this MSM (w_cnt x n, window-major)
};

// counting sort in shared memory: buckets per window it handles, threads per block
constexpr uint32_t SORT_SMEM_MAX_B = 32768;
constexpr int SORT_THREADS = 1024;
constexpr uint32_t SORT_MIN_POINTS_PER_BLOCK = 8192;  // below this average per block: the global-atomic sort

// A run of MSMs sharing one window width (one templated recode launch).
struct WindowClass {
    int c;
    uint32_t first, count;       // MSM indices
    uint32_t pt_begin, pt_end;   // concatenated point range
};

// Pippenger plan for a batch of MSMs on one curve (a single MSM is a batch of one).
struct BatchPlan {
    int curve = 0;
    std::vector<MsmDesc> msms;
    std::vector<WindowClass> classes;
    uint32_t M = 0;             // MSMs
    uint32_t n_total = 0;       // points
    uint32_t NB = 0;            // buckets (all MSMs, all windows)
    uint32_t G = 0;             // reduction groups
    uint32_t WS = 0;            // window sums
    uint32_t CH = 0;            // level-2 reduction chunks
    uint32_t max_T = 1;         // largest groups-per-window of the batch
    uint32_t max_nbk = 1;       // largest chunks-per-window of the batch
    uint32_t max_B = 1;         // largest buckets-per-window of the batch
    uint32_t sort_blocks = 0;   // counting-sort blocks (shared-memory path)
    uint64_t cnt_len = 0;       // per-block bucket counts (shared-memory path)
    bool global_sort = false;   // keep the global-atomic sort (no digit and count buffers)
    bool smem_sort() const { return !global_sort && max_B <= SORT_SMEM_MAX_B; }
    uint32_t L = 0;             // max entries per accumulation segment
    uint32_t max_entries = 0;
    uint32_t max_segs = 0;
    uint32_t hist_blocks = 0;   // blocks of the segment-length histogram
    // > 0: host inputs arrive in two parts, points below and above counting-sort
    // slice part_slice (one MSM, shared-memory sort).  Every bucket then has
    // its own segments per part, in two longest-first lists; a bucket's first
    // part-1 segment continues the sum of its first part-0 segment.
    uint32_t part_slice = 0;
    uint64_t entries_bound = 0; // sum n_i * W_i
    // the algorithmic count of (point, window) entries: n_i * ceil(256/c_i) per
    // MSM (the full windows of a 256-bit scalar, not the carry window), the
    // unit of the pinned work figure that instrumentation reports
    uint64_t entries_pinned = 0;
    // Batch-affine accumulation (ba_rounds > 0): rounds of pairwise affine
    // additions halve every bucket's list before the XYZZ fold, whose segments
    // (L, max_segs, hist_blocks above) then cut the last round's lists.
    uint32_t ba_rounds = 0;      // 0: the XYZZ accumulation of the entries (else: entries padded per bucket)
    uint64_t ba_items[3] = {};   // bound on the outputs of round r (index r-1)
    uint32_t ba_blocks[3] = {};  // blocks of round r's kernels (BA_K * BA_BT outputs each)
};

// batch-affine rounds: outputs per thread and threads per block of a round (one
// shared inversion per block), and the rounds at most
constexpr uint32_t BA_PLAN_K = 16;
constexpr uint32_t BA_PLAN_BT = 128;
constexpr uint32_t BA_MAX_ROUNDS = 3;

// Device buffers of one batch (carved from the arena).
struct BatchBuffers {
    const uint32_t *scalars = nullptr;  // n_total * 8 words
    const uint4 *points = nullptr;      // n_total * 4 uint4 (affine x || y), or a window-multiple table
    const uint32_t *pt_idx = nullptr;   // n_total table generators of the MSMs with fixed = 2
    MsmDesc *desc = nullptr;            // M descriptors
    uint32_t *counts = nullptr;         // NB + 1 (later reused as fill cursors)
    uint32_t *offsets = nullptr;        // NB + 1, exclusive scan of counts
    uint32_t *seg_off = nullptr;        // NB + 1, exclusive scan of segment counts
    uint32_t *scan_tmp = nullptr;       // per-block partials of the scans
    uint32_t *len_hist = nullptr;       // (L+1) x hist_blocks segment-length histogram
    uint32_t *len_scan = nullptr;       // its exclusive scan (+1 total)
    uint32_t *sorted = nullptr;         // max_entries: point index | sign << 31
    uint4 *segs = nullptr;              // max_segs: (start, length, destination slot, 0), longest first
    uint4 *seg_sum = nullptr;           // max_segs XYZZ sums (8 uint4 each)
    uint32_t *heavy = nullptr;          // NB heavy-bucket list
    uint32_t *heavy_n = nullptr;        // 1 counter
    uint4 *redA = nullptr;              // G group (acc, run) pairs
    uint4 *redC = nullptr;              // CH chunk (sum, run) pairs
    uint32_t *sort_cnt = nullptr;       // cnt_len per-block bucket counts, then offsets
    uint32_t *digits = nullptr;         // max_entries signed digits (|d| | sign << 31, 0 = none)
    uint4 *redS = nullptr;              // WS window sums
    uint32_t *out_jac = nullptr;        // M x 24 words: canonical Jacobian X, Y, Z
    uint32_t *counts0 = nullptr;        // NB part-0 entry counts (plans with part_slice)
    // batch-affine rounds (plans with ba_rounds): round r's list of bucket k is
    // [offsets[k] >> r, offsets[k+1] >> r) of its level
    uint4 *ba_lvl[2] = {};              // round outputs, affine (4 uint4 each): odd rounds [0], even [1]
    uint4 *ba_pre = nullptr;            // round-1 bound of outputs: exclusive prefix products (2 uint4 each)
    uint4 *ba_co = nullptr;             // per thread: product of the other threads' totals of its block
    uint4 *ba_tot = nullptr;            // per block: product of its denominators
    uint4 *ba_inv = nullptr;            // per block: its inverse
    // host inputs: the accumulation of part j waits for ready[j] (null: bases resident)
    cudaEvent_t ready[2] = {nullptr, nullptr};
};

// index of the MSM owning element x of a batch: the largest m with key(m) <= x
template <class KeyFn>
__device__ __forceinline__ uint32_t find_msm(uint32_t M, uint32_t x, KeyFn key)
{
    uint32_t lo = 0, hi = M - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (key(mid) <= x)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

int choose_window(const Context &ctx, int curve, size_t n);
// base_rounds >= 0: the batch-affine rounds in place of the curve's setting
// (a window rule that names rounds still wins)
BatchPlan make_batch_plan(const Context &ctx, int curve, const size_t *sizes, uint32_t M, int base_rounds = -1);
// count fixed-base MSMs of n table generators each (window c), scalars back to back
BatchPlan make_fixed_plan(int curve, size_t n, int c, uint32_t count);
// M MSMs over rows of one window-multiple table (window c) named by index lists
// (fixed = 2): sizes[i] generators each, scalars and indices back to back
BatchPlan make_indexed_plan(const Context &ctx, int curve, const size_t *sizes, uint32_t M, int c);
// one MSM of n points restricted to windows [w_lo, w_lo + w_cnt) of width c
BatchPlan make_window_plan(int curve, size_t n, int c, uint32_t w_lo, uint32_t w_cnt);
// switch a plan to batch-affine accumulation with `rounds` rounds (0 or a plan
// below min_entries: left as it is)
void plan_batch_affine(BatchPlan &p, uint32_t rounds, uint64_t min_entries);
size_t batch_bytes(const BatchPlan &p);
bool carve(DeviceArena &a, const BatchPlan &p, BatchBuffers &b);

// curve-independent launches (hs_runtime.cu): descriptor upload, recode, sort, segments
cudaError_t launch_sort(Context &ctx, const BatchPlan &p, const BatchBuffers &b);

// per-curve entry points (hs_curve_helios.cu / hs_curve_selene.cu)
struct CurveOps {
    // buckets -> window sums -> canonical Jacobians in b.out_jac (after launch_sort)
    cudaError_t (*msm_tail)(Context &ctx, const BatchPlan &p, const BatchBuffers &b);
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
    // window-multiple table: table[i*W + k] = 2^(c k) * gens[i] (affine), tmp holds n*W XYZZ points
    cudaError_t (*fixed_table)(Context &ctx, const uint4 *d_gens, size_t n, int c, int W, uint4 *d_tmp,
                               uint4 *d_table);
    // out[i] = a[i] + b[i] for count canonical Jacobians (24 words each)
    cudaError_t (*join)(Context &ctx, const uint32_t *d_a, const uint32_t *d_b, size_t count, uint32_t *d_out);
    // 32-byte encodings -> canonical affine; invalid ones give (0, 0), d_valid[i] = 0
    // (d_valid may be null) and a count in *d_bad (not cleared here)
    cudaError_t (*decompress)(Context &ctx, const void *d_in, size_t n, uint4 *d_out, uint8_t *d_valid,
                              uint32_t *d_bad);
    // out[i] = s_i P_i as canonical Jacobians (24 words), points canonical affine
    cudaError_t (*scalar_mul)(Context &ctx, const void *d_scalars, const uint4 *d_points, size_t n, uint32_t *d_out);
};
extern const CurveOps helios_ops;
extern const CurveOps selene_ops;
const CurveOps &curve_ops(int curve);

size_t fmt_bytes(int fmt);
size_t align256(size_t b);

// One piece of a gathered host-to-device copy (pull_list): a device that reads
// pageable host memory (Context::pageable_access) copies the pieces with one
// kernel, reading the list and the sources where they lie in host memory.
struct PullChunk {
    const uint8_t *src;
    uint8_t *dst;
    uint64_t bytes;
};
constexpr size_t PULL_CHUNK_BYTES = size_t(256) << 10;  // a block copies one piece at a time

// A caller's buffer is read on the CPU at its first and last byte before a copy
// kernel reads it: a bad pointer, or a buffer shorter than its count where the
// memory past it is unmapped, then fails on the host -- as a copy-engine copy
// from pageable memory, which the CPU stages, would -- and not on the device.
inline void touch_host_range(const void *p, size_t bytes)
{
    if (!bytes)
        return;
    const volatile uint8_t *b = static_cast<const volatile uint8_t *>(p);
    (void)b[0];
    (void)b[bytes - 1];
}

// append a copy of `bytes` from src to dst, cut into pieces of at most PULL_CHUNK_BYTES
inline void pull_add(std::vector<PullChunk> &list, void *dst, const void *src, size_t bytes)
{
    touch_host_range(src, bytes);
    for (size_t o = 0; o < bytes; o += PULL_CHUNK_BYTES)
        list.push_back({static_cast<const uint8_t *>(src) + o, static_cast<uint8_t *>(dst) + o,
                        std::min(PULL_CHUNK_BYTES, bytes - o)});
}

// one kernel copying every piece of `list` (host memory the device reads, left
// untouched until the stream has passed the kernel) on stream s
cudaError_t pull_list(Context &ctx, const PullChunk *list, size_t count, cudaStream_t s);

// make `dev` current for a scope
struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev)
    {
        cudaGetDevice(&prev);
        if (prev != dev)
            cudaSetDevice(dev);
    }
    ~DeviceGuard()
    {
        if (prev >= 0)
            cudaSetDevice(prev);
    }
};

// batch execution helpers shared with the serving loop (hs_runtime.cu)
int reserve_batch(Context &ctx, const BatchPlan &p, size_t extra_bytes, BatchBuffers &b, void **extra);
int execute_batch(Context &ctx, const BatchPlan &p, const BatchBuffers &b, void *d_out, int out_fmt);
// recode, sort, accumulate, reduce, combine and format one batch with direct launches
cudaError_t sort_smem_attrs(int device);
cudaError_t launch_batch(Context &ctx, const BatchPlan &p, const BatchBuffers &b, void *d_out, int out_fmt);
void drop_graphs(Context &ctx);
int fail(Context &ctx, cudaError_t e, const char *what);
// the calling thread's error text, read by hs_last_error(NULL)
void set_thread_error(const std::string &what);
int fail_msg(Context &ctx, int code, const char *what);

#define HS_LAUNCH_CHECK(ctx)                                 \
    do {                                                     \
        (ctx).launches++;                                    \
        cudaError_t e__ = cudaGetLastError();                \
        if (e__ != cudaSuccess)                              \
            return e__;                                      \
    } while (0)

}  // namespace hs
