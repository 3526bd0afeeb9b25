// hs_runtime.cu -- context, workspace, signed-digit recode + counting sort, and the C ABI.
//
// The recode follows encode_signed_wbit (helios/src/x64/helios_msm_vartime.cpp:127-162)
// with one difference: W = ceil(257/c) windows, so the carry out of the last
// full window is kept (the reference drops it when 256 % c == 0, i.e. c = 8).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>

#include "hs_internal.h"

struct hs_context {
    hs::Context c;
};

struct hs_fixed_base {
    int curve = 0;
    int device = 0;
    int c = 0;
    int W = 0;
    size_t n_user = 0;  // generators given
    size_t n_gen = 0;   // + H when present
    bool has_H = false;
    uint4 *d_table = nullptr;
};

namespace hs {

// ---------------------------------------------------------------------------
// arena
// ---------------------------------------------------------------------------
cudaError_t DeviceArena::reserve(size_t bytes)
{
    off = 0;
    if (bytes <= cap)
        return cudaSuccess;
    if (base) {
        cudaError_t e = ordered ? cudaFreeAsync(base, ordered) : cudaFree(base);
        base = nullptr;
        cap = 0;
        if (e != cudaSuccess)
            return e;
    }
    size_t want = bytes + bytes / 8;
    cudaError_t e = ordered ? cudaMallocAsync(reinterpret_cast<void **>(&base), want, ordered)
                            : cudaMalloc(reinterpret_cast<void **>(&base), want);
    if (e != cudaSuccess) {
        cudaGetLastError();
        base = nullptr;
        return e;
    }
    cap = want;
    return cudaSuccess;
}

void *DeviceArena::take(size_t bytes)
{
    size_t o = (off + 255) & ~size_t(255);
    if (o + bytes > cap)
        return nullptr;
    off = o + bytes;
    return base + o;
}

void DeviceArena::release()
{
    if (base) {
        if (ordered) {
            cudaFreeAsync(base, ordered);
            cudaStreamSynchronize(ordered);
        } else {
            cudaFree(base);
        }
    }
    base = nullptr;
    cap = off = 0;
}

size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

size_t fmt_bytes(int fmt)
{
    switch (fmt) {
    case HS_FMT_JACOBIAN51:
        return 120;
    case HS_FMT_AFFINE51:
        return 80;
    case HS_FMT_AFFINE:
        return 64;
    case HS_FMT_COMPRESSED:
        return 32;
    default:
        return 0;
    }
}

const CurveOps &curve_ops(int curve) { return curve == HS_SELENE ? selene_ops : helios_ops; }

// ---------------------------------------------------------------------------
// planning
// ---------------------------------------------------------------------------
static constexpr uint32_t SEG_HIST_THREADS = 256;

static int model_window(size_t n)
{
    // cost ~ W(c) * (n * madd + 2^(c-1) * 2 adds), madd ~ 10 M, add ~ 14 M.  A
    // first guess only: the autotuner (helioselene_gb300.autotune) measures each
    // size class on the device and installs rules that override it.  On GB300 at
    // n = 2^20 the measured optimum agrees (c = 16: 16 full windows plus a
    // carry window that is almost empty).
    // Below c = 8 the model's work saving does not pay on the GPU: small MSMs are
    // latency-bound, and c = 8 (32 full windows, the top one with 7 used bits)
    // measured fastest from 512 to 4096 points on both curves.
    int best = 8;
    double best_cost = 1e300;
    for (int c = 8; c <= 20; c++) {
        const double W = (257 + c - 1) / c;
        const double cost = W * (10.0 * (double)n + 28.0 * (double)(1u << (c - 1)));
        if (cost < best_cost) {
            best_cost = cost;
            best = c;
        }
    }
    return best;
}

int choose_window(const Context &ctx, int curve, size_t n)
{
    int c = 0;
    for (const WindowRule &r : ctx.rules[curve == HS_SELENE ? 1 : 0])
        if (n >= r.n_min && n <= r.n_max)
            c = r.c;
    if (c < 4 || c > 20)
        c = model_window(n);
    return c;
}

// Shared-memory counting sort: MSM m's emitted windows are each cut into
// `slices` point ranges, one block per (window, slice).  A block counts its
// bucket keys in shared memory and writes one row of counts; a bucket's rows
// are Q = slices (or w_cnt * slices for a fixed-base MSM, whose windows share
// its B buckets) and its columns the MSM's buckets, so cnt_base + q * Bm + col.
static void plan_sort(BatchPlan &p)
{
    uint64_t blk = 0, cnt = 0, dig = 0;
    p.max_B = 1;
    for (MsmDesc &d : p.msms) {
        d.dig_base = (uint32_t)dig;
        dig += (uint64_t)d.w_cnt * d.n;
        d.slices = (uint32_t)std::min<uint64_t>(64, std::max<uint64_t>(1, ((uint64_t)d.n + 131071) / 131072));
        d.sblk_base = (uint32_t)blk;
        d.cnt_base = (uint32_t)cnt;
        blk += (uint64_t)d.w_cnt * d.slices;
        const uint64_t Bm = d.fixed ? d.B : (uint64_t)d.w_cnt * d.B;
        const uint64_t Q = d.fixed ? (uint64_t)d.w_cnt * d.slices : d.slices;
        cnt += Bm * Q;
        p.max_B = std::max(p.max_B, d.B);
    }
    p.sort_blocks = (uint32_t)blk;
    p.cnt_len = cnt;
    // a block clears and writes a whole row of B counts: worth it only when its
    // slice holds thousands of points (many small MSMs keep the global atomics)
    if (dig < (uint64_t)SORT_MIN_POINTS_PER_BLOCK * std::max<uint64_t>(1, blk))
        p.global_sort = true;
}

// level-2 reduction chunks: chunk_base per MSM and the plan totals
static void plan_chunks(BatchPlan &p)
{
    uint64_t ch = 0;
    p.max_T = 1;
    p.max_nbk = 1;
    for (MsmDesc &d : p.msms) {
        const uint32_t nbk = d.T > RED_CHUNK ? d.T / RED_CHUNK : 1;
        d.chunk_base = (uint32_t)ch;
        ch += (uint64_t)d.Wr * nbk;
        p.max_T = std::max(p.max_T, d.T);
        p.max_nbk = std::max(p.max_nbk, nbk);
    }
    p.CH = (uint32_t)ch;
}

// Buckets per level-1 group for a plan of nb buckets.  A group is one thread's
// chain of 2 m0 additions and the groups are level 1's parallelism: 8 for one
// large MSM, fewer for small plans (latency-bound, so shorter chains on more
// threads win), more once there are millions of buckets, so that level 2 --
// latency-bound, a scan per window -- has fewer groups to combine.
static uint32_t group_size(uint64_t nb)
{
    if (nb >= (1ull << 22))
        return 4 * RED_GROUP;
    if (nb >= (1ull << 21))
        return 2 * RED_GROUP;
    if (nb >= (1ull << 18))
        return RED_GROUP;
    return nb >= (1ull << 16) ? RED_GROUP / 2 : RED_GROUP / 4;
}

// Entries per accumulation segment at most.  A large plan keeps about two
// buckets' worth (one segment per bucket, few merges: the accumulation is
// throughput-bound).  A plan too small to fill the device is latency-bound --
// its longest segment sets the time -- so the cap shrinks with the entry count
// (about 65536 segments' worth), down to 8 and to a quarter of the mean bucket,
// at the price of more, short merges (shorter segments made the merges of the
// largest buckets outlast the accumulation).
static uint32_t seg_cap(uint64_t ent, uint64_t nb)
{
    const uint64_t avg = nb ? (ent + nb - 1) / nb : 1;
    const uint64_t big = std::max<uint64_t>(16, std::min<uint64_t>(128, 2 * avg));
    const uint64_t least = std::max<uint64_t>(8, avg / 4);  // at most ~4 segments per typical bucket
    return (uint32_t)std::min<uint64_t>(big, std::max<uint64_t>(least, ent / 65536));
}

BatchPlan make_batch_plan(const Context &ctx, int curve, const size_t *sizes, uint32_t M, int base_rounds)
{
    BatchPlan p;
    p.curve = curve;
    p.M = M;
    p.msms.resize(M);
    uint64_t nb_all = 0;
    std::vector<int> cs(M);
    for (uint32_t i = 0; i < M; i++) {
        cs[i] = choose_window(ctx, curve, sizes[i] ? sizes[i] : 1);
        nb_all += (uint64_t)((257 + cs[i] - 1) / cs[i]) << (cs[i] - 1);
    }
    const uint32_t gsz = group_size(nb_all);
    uint64_t pt = 0, nb = 0, g = 0, ws = 0, ent = 0;
    for (uint32_t i = 0; i < M; i++) {
        MsmDesc &d = p.msms[i];
        const size_t n = sizes[i];
        const int c = cs[i];
        d.pt_off = (uint32_t)pt;
        d.n = (uint32_t)n;
        d.c = (uint32_t)c;
        d.W = (uint32_t)((257 + c - 1) / c);
        d.B = 1u << (c - 1);
        d.m0 = std::min<uint32_t>(gsz, d.B);
        d.log2m0 = 0;
        while ((1u << d.log2m0) < d.m0)
            d.log2m0++;
        d.T = d.B / d.m0;
        d.bucket_base = (uint32_t)nb;
        d.group_base = (uint32_t)g;
        d.win_base = (uint32_t)ws;
        d.fixed = 0;
        d.Wr = d.W;
        d.w_lo = 0;
        d.w_cnt = d.W;
        d.shift = 0;
        pt += n;
        nb += (uint64_t)d.W * d.B;
        g += (uint64_t)d.W * d.T;
        ws += d.W;
        ent += (uint64_t)n * d.W;
        p.entries_pinned += (uint64_t)n * (uint64_t)((256 + c - 1) / c);
    }
    p.n_total = (uint32_t)pt;
    p.NB = (uint32_t)nb;
    p.G = (uint32_t)g;
    p.WS = (uint32_t)ws;
    p.entries_bound = ent;
    p.max_entries = (uint32_t)std::max<uint64_t>(1, ent);
    p.L = seg_cap(ent, nb);
    p.max_segs = (uint32_t)(std::min<uint64_t>(ent, nb) + ent / p.L + 1);
    p.hist_blocks = (p.NB + SEG_HIST_THREADS - 1) / SEG_HIST_THREADS;
    plan_chunks(p);
    plan_sort(p);
    // batch-affine rounds: those of the size class (window rule) holding most of
    // the plan's entries when that rule names some, else the curve's setting
    const auto &rules = ctx.rules[curve == HS_SELENE ? 1 : 0];
    int rounds = base_rounds >= 0 ? base_rounds : (int)ctx.ba_rounds[curve == HS_SELENE];
    if (!rules.empty()) {
        std::vector<uint64_t> by_rule(rules.size(), 0);
        for (uint32_t i = 0; i < M; i++) {
            int hit = -1;
            for (size_t k = 0; k < rules.size(); k++)
                if (sizes[i] >= rules[k].n_min && sizes[i] <= rules[k].n_max)
                    hit = (int)k;  // the last matching rule wins, as in choose_window
            if (hit >= 0)
                by_rule[hit] += (uint64_t)sizes[i] * p.msms[i].W;
        }
        const size_t top = (size_t)(std::max_element(by_rule.begin(), by_rule.end()) - by_rule.begin());
        if (by_rule[top] && rules[top].ba_rounds >= 0)
            rounds = rules[top].ba_rounds;
    }
    plan_batch_affine(p, (uint32_t)rounds, ctx.ba_min_entries[curve == HS_SELENE]);
    return p;
}

BatchPlan make_fixed_plan(int curve, size_t n, int c, uint32_t count)
{
    BatchPlan p;
    p.curve = curve;
    p.M = count;
    p.msms.resize(count);
    const uint32_t W = (uint32_t)((257 + c - 1) / c), B = 1u << (c - 1);
    const uint32_t m0 = std::min<uint32_t>(group_size((uint64_t)count * B), B);
    uint32_t log2m0 = 0;
    while ((1u << log2m0) < m0)
        log2m0++;
    for (uint32_t j = 0; j < count; j++) {
        MsmDesc &d = p.msms[j];
        d.pt_off = (uint32_t)(j * n);
        d.n = (uint32_t)n;
        d.c = (uint32_t)c;
        d.W = W;
        d.B = B;
        d.m0 = m0;
        d.log2m0 = log2m0;
        d.T = B / m0;
        d.bucket_base = j * B;
        d.group_base = j * d.T;
        d.win_base = j;
        d.fixed = 1;
        d.Wr = 1;
        d.w_lo = 0;
        d.w_cnt = W;
        d.shift = 0;
    }
    const uint64_t ent = (uint64_t)count * n * W;
    p.entries_pinned = (uint64_t)count * n * (uint64_t)((256 + c - 1) / c);
    p.n_total = (uint32_t)(count * n);
    p.NB = count * B;
    p.G = count * (B / m0);
    p.WS = count;
    p.entries_bound = ent;
    p.max_entries = (uint32_t)std::max<uint64_t>(1, ent);
    p.L = seg_cap(ent, p.NB);
    p.max_segs = (uint32_t)(std::min<uint64_t>(ent, p.NB) + ent / p.L + 1);
    p.hist_blocks = (p.NB + SEG_HIST_THREADS - 1) / SEG_HIST_THREADS;
    plan_chunks(p);
    plan_sort(p);
    return p;
}

BatchPlan make_indexed_plan(const Context &ctx, int curve, const size_t *sizes, uint32_t M, int c)
{
    BatchPlan p;
    p.curve = curve;
    p.M = M;
    p.msms.resize(M);
    const uint32_t W = (uint32_t)((257 + c - 1) / c), B = 1u << (c - 1);
    const uint32_t m0 = std::min<uint32_t>(group_size((uint64_t)M * B), B);
    uint32_t log2m0 = 0;
    while ((1u << log2m0) < m0)
        log2m0++;
    uint64_t pt = 0;
    for (uint32_t j = 0; j < M; j++) {
        MsmDesc &d = p.msms[j];
        d.pt_off = (uint32_t)pt;
        d.n = (uint32_t)sizes[j];
        d.c = (uint32_t)c;
        d.W = W;
        d.B = B;
        d.m0 = m0;
        d.log2m0 = log2m0;
        d.T = B / m0;
        d.bucket_base = j * B;
        d.group_base = j * d.T;
        d.win_base = j;
        d.fixed = 2;
        d.Wr = 1;
        d.w_lo = 0;
        d.w_cnt = W;
        d.shift = 0;
        pt += sizes[j];
    }
    const uint64_t ent = pt * W;
    p.entries_pinned = pt * (uint64_t)((256 + c - 1) / c);
    p.n_total = (uint32_t)pt;
    p.NB = M * B;
    p.G = M * (B / m0);
    p.WS = M;
    p.entries_bound = ent;
    p.max_entries = (uint32_t)std::max<uint64_t>(1, ent);
    p.L = seg_cap(ent, p.NB);
    p.max_segs = (uint32_t)(std::min<uint64_t>(ent, p.NB) + ent / p.L + 1);
    p.hist_blocks = (p.NB + SEG_HIST_THREADS - 1) / SEG_HIST_THREADS;
    plan_chunks(p);
    plan_sort(p);
    const int cv = curve == HS_SELENE;
    plan_batch_affine(p, ctx.ba_rounds[cv], ctx.ba_min_entries[cv]);
    return p;
}

BatchPlan make_window_plan(int curve, size_t n, int c, uint32_t w_lo, uint32_t w_cnt)
{
    BatchPlan p;
    p.curve = curve;
    p.M = 1;
    p.msms.resize(1);
    MsmDesc &d = p.msms[0];
    d.pt_off = 0;
    d.n = (uint32_t)n;
    d.c = (uint32_t)c;
    d.W = (uint32_t)((257 + c - 1) / c);
    d.B = 1u << (c - 1);
    d.m0 = std::min<uint32_t>(group_size((uint64_t)w_cnt * d.B), d.B);
    d.log2m0 = 0;
    while ((1u << d.log2m0) < d.m0)
        d.log2m0++;
    d.T = d.B / d.m0;
    d.bucket_base = 0;
    d.group_base = 0;
    d.win_base = 0;
    d.fixed = 0;
    d.Wr = w_cnt;
    d.w_lo = w_lo;
    d.w_cnt = w_cnt;
    d.shift = (uint32_t)c * w_lo;
    const uint64_t ent = (uint64_t)n * w_cnt;
    {
        const uint32_t full = (uint32_t)((256 + c - 1) / c);  // windows below the carry window
        const uint32_t hi = std::min(full, w_lo + w_cnt);
        p.entries_pinned = hi > w_lo ? (uint64_t)n * (hi - w_lo) : 0;
    }
    p.n_total = (uint32_t)n;
    p.NB = w_cnt * d.B;
    p.G = w_cnt * d.T;
    p.WS = w_cnt;
    p.entries_bound = ent;
    p.max_entries = (uint32_t)std::max<uint64_t>(1, ent);
    p.L = seg_cap(ent, p.NB);
    p.max_segs = (uint32_t)(std::min<uint64_t>(ent, p.NB) + ent / p.L + 1);
    p.hist_blocks = (p.NB + SEG_HIST_THREADS - 1) / SEG_HIST_THREADS;
    plan_chunks(p);
    plan_sort(p);
    return p;
}

// Batch-affine rounds: every bucket's entry list is padded to a multiple of
// 2^R (at most NB (2^R - 1) padding entries), so round r's lists are the
// padded offsets shifted right by r and need no scan; the fold's segments cut
// the last round's lists with the cap of an entry count that size.
void plan_batch_affine(BatchPlan &p, uint32_t rounds, uint64_t min_entries)
{
    rounds = std::min<uint32_t>(rounds, BA_MAX_ROUNDS);
    const uint64_t padded = (uint64_t)p.max_entries + (uint64_t)p.NB * ((1u << rounds) - 1);
    if (rounds == 0 || p.entries_bound < min_entries || p.part_slice || padded >= 0x80000000ull)
        return;
    p.ba_rounds = rounds;
    p.max_entries = (uint32_t)padded;
    const uint64_t per_block = (uint64_t)BA_PLAN_K * BA_PLAN_BT;
    for (uint32_t r = 1; r <= rounds; r++) {
        p.ba_items[r - 1] = (padded >> r) + 1;
        p.ba_blocks[r - 1] = (uint32_t)((p.ba_items[r - 1] + per_block - 1) / per_block);
    }
    const uint64_t ent = p.ba_items[rounds - 1];
    p.L = seg_cap(ent, p.NB);
    p.max_segs = (uint32_t)(std::min<uint64_t>(ent, p.NB) + ent / p.L + 1);
}

static constexpr int SCAN_THREADS = 1024;
static constexpr int SCAN_ITEMS = 4;
static constexpr uint32_t SCAN_BLOCK = SCAN_THREADS * SCAN_ITEMS;

static uint32_t scan_blocks(uint32_t NB) { return (NB + SCAN_BLOCK - 1) / SCAN_BLOCK; }

static size_t hist_len(const BatchPlan &p) { return (size_t)(p.L + 1) * p.hist_blocks * (p.part_slice ? 2 : 1); }

// entry lists of a plan: one per bucket, or with batch-affine rounds and host
// inputs in two parts, one per (part, bucket): list NB*part + bucket
static uint32_t list_count(const BatchPlan &p) { return (p.ba_rounds && p.part_slice) ? 2 * p.NB : p.NB; }

size_t batch_bytes(const BatchPlan &p)
{
    size_t b = 0;
    const size_t nh = hist_len(p);
    b += align256((size_t)p.M * sizeof(MsmDesc));
    const size_t nl = list_count(p);
    b += align256((size_t)(p.NB + 1) * 4);                                                 // counts
    b += 2 * align256((nl + 1) * 4);                                                       // offsets, seg_off
    b += align256((size_t)2 * scan_blocks((uint32_t)std::max<size_t>(nl, nh)) * 4 + 64);   // scan partials
    b += 2 * align256((nh + 1) * 4);                                                       // length histogram + scan
    b += align256((size_t)p.max_entries * 4);                                              // sorted
    b += align256((size_t)p.max_segs * 16);                                                // segs
    b += align256((size_t)p.max_segs * 128);                                               // seg_sum
    b += align256((size_t)p.NB * 4) + 256;                                                 // heavy list + counter
    b += align256((size_t)std::max<uint32_t>(1, p.G) * 256);                               // group (acc, run) pairs
    b += align256((size_t)std::max<uint32_t>(1, p.CH) * 256);                              // chunk (sum, run) pairs
    b += p.smem_sort() ? align256((size_t)std::max<uint64_t>(1, p.cnt_len) * 4) : 0;         // per-block counts
    b += p.smem_sort() ? align256((size_t)p.max_entries * 4) : 0;                            // signed digits
    b += align256((size_t)std::max<uint32_t>(1, p.WS) * 128);                              // window sums
    b += align256((size_t)std::max<uint32_t>(1, p.M) * 96);                                // results
    b += p.part_slice ? align256((size_t)(p.NB + 1) * 4) : 0;                                // part-0 counts
    if (p.ba_rounds) {
        b += align256((size_t)p.ba_items[0] * 64);                                            // odd rounds
        b += p.ba_rounds > 1 ? align256((size_t)p.ba_items[1] * 64) : 0;                      // even rounds
        b += align256((size_t)p.ba_items[0] * 32);                                            // prefixes
        b += align256((size_t)p.ba_blocks[0] * BA_PLAN_BT * 32);                              // co-products
        b += 2 * align256((size_t)p.ba_blocks[0] * 32);                                       // totals, inverses
        b += 8 * 256;
    }
    return b + 16 * 256;
}

bool carve(DeviceArena &a, const BatchPlan &p, BatchBuffers &b)
{
    const size_t nh = hist_len(p);
    b.desc = (MsmDesc *)a.take((size_t)p.M * sizeof(MsmDesc));
    const size_t nl = list_count(p);
    b.counts = (uint32_t *)a.take((size_t)(p.NB + 1) * 4);
    b.offsets = (uint32_t *)a.take((nl + 1) * 4);
    b.seg_off = (uint32_t *)a.take((nl + 1) * 4);
    b.scan_tmp = (uint32_t *)a.take((size_t)2 * scan_blocks((uint32_t)std::max<size_t>(nl, nh)) * 4 + 64);
    b.len_hist = (uint32_t *)a.take((nh + 1) * 4);
    b.len_scan = (uint32_t *)a.take((nh + 1) * 4);
    b.sorted = (uint32_t *)a.take((size_t)p.max_entries * 4);
    b.segs = (uint4 *)a.take((size_t)p.max_segs * 16);
    b.seg_sum = (uint4 *)a.take((size_t)p.max_segs * 128);
    b.heavy = (uint32_t *)a.take((size_t)p.NB * 4);
    b.heavy_n = (uint32_t *)a.take(4);
    b.redA = (uint4 *)a.take((size_t)std::max<uint32_t>(1, p.G) * 256);
    b.redC = (uint4 *)a.take((size_t)std::max<uint32_t>(1, p.CH) * 256);
    b.sort_cnt = p.smem_sort() ? (uint32_t *)a.take((size_t)std::max<uint64_t>(1, p.cnt_len) * 4) : nullptr;
    b.digits = p.smem_sort() ? (uint32_t *)a.take((size_t)p.max_entries * 4) : nullptr;
    b.redS = (uint4 *)a.take((size_t)std::max<uint32_t>(1, p.WS) * 128);
    b.out_jac = (uint32_t *)a.take((size_t)std::max<uint32_t>(1, p.M) * 96);
    b.counts0 = p.part_slice ? (uint32_t *)a.take((size_t)(p.NB + 1) * 4) : nullptr;
    bool ba_ok = true;
    if (p.ba_rounds) {
        ba_ok = ba_ok && (b.ba_lvl[0] = (uint4 *)a.take((size_t)p.ba_items[0] * 64));
        if (p.ba_rounds > 1)
            ba_ok = ba_ok && (b.ba_lvl[1] = (uint4 *)a.take((size_t)p.ba_items[1] * 64));
        ba_ok = ba_ok && (b.ba_pre = (uint4 *)a.take((size_t)p.ba_items[0] * 32));
        ba_ok = ba_ok && (b.ba_co = (uint4 *)a.take((size_t)p.ba_blocks[0] * BA_PLAN_BT * 32));
        ba_ok = ba_ok && (b.ba_tot = (uint4 *)a.take((size_t)p.ba_blocks[0] * 32));
        ba_ok = ba_ok && (b.ba_inv = (uint4 *)a.take((size_t)p.ba_blocks[0] * 32));
    }
    return b.desc && b.counts && b.offsets && b.seg_off && b.scan_tmp && b.len_hist && b.len_scan && b.sorted &&
           b.segs && b.seg_sum && b.heavy && b.heavy_n && b.redA && b.redC && b.redS && b.out_jac &&
           ((b.sort_cnt && b.digits) || !p.smem_sort()) && (b.counts0 || !p.part_slice) && ba_ok;
}

// ---------------------------------------------------------------------------
// 1. signed-digit recode and counting sort
// ---------------------------------------------------------------------------
template <int CB>
__device__ __forceinline__ uint32_t window_bits(const uint32_t s[8], int k)
{
    const int o = k * CB;
    const int wi = o >> 5, sh = o & 31;
    const uint32_t lo = (wi < 8) ? s[wi] : 0u;
    const uint32_t hi = (wi + 1 < 8) ? s[wi + 1] : 0u;
    return __funnelshift_r(lo, hi, sh) & ((1u << CB) - 1u);
}

// Digits in [-2^(c-1), 2^(c-1)) except the top one, which keeps the final
// carry and is at most 2^(c-1) because W*c >= 257.  count pass: histogram of
// bucket keys; scatter pass: place "index | sign" at offsets[key] + running fill.
// Normal MSMs: window k uses buckets bucket_base + k*B + ..., entries name the
// point (pbase = i, pstep = 0).  Fixed-base MSMs: every window uses the same B
// buckets (wstep = 0), entries name table row g*W + k (pstep = 1) of generator
// g = i - pt_off, or g = pt_idx[i] for an indexed MSM.
// The digits are always computed from window 0 (the carries run upward), but
// only windows [w_lo, w_lo + w_cnt) are emitted (a window-split half).
template <int CB, bool SCATTER>
__device__ __forceinline__ void recode_one(const uint32_t s[8], uint32_t pbase, uint32_t pstep, uint32_t wstep,
                                           uint32_t bucket_base, uint32_t w_lo, uint32_t w_cnt,
                                           uint32_t *__restrict__ counts, const uint32_t *__restrict__ offsets,
                                           uint32_t *__restrict__ sorted)
{
    constexpr int W = (257 + CB - 1) / CB;
    constexpr uint32_t B = 1u << (CB - 1);
    uint32_t carry = 0;
#pragma unroll
    for (int k = 0; k < W; k++) {
        const uint32_t v = window_bits<CB>(s, k) + carry;
        uint32_t mag;
        bool neg = false;
        if (k < W - 1 && v >= B) {
            mag = (1u << CB) - v;  // digit v - 2^c < 0
            neg = mag != 0;
            carry = 1;
        } else {
            mag = v;
            carry = 0;
        }
        if (mag != 0 && (uint32_t)k - w_lo < w_cnt) {
            const uint32_t kb = bucket_base + ((uint32_t)k - w_lo) * wstep + mag - 1u;
            if (!SCATTER) {
                atomicAdd(counts + kb, 1u);
            } else {
                const uint32_t pos = offsets[kb] + atomicAdd(counts + kb, 1u);
                sorted[pos] = (pbase + (uint32_t)k * pstep) | (neg ? 0x80000000u : 0u);
            }
        }
    }
}

// One thread per point of the batch; the window width is per MSM.
// table generator of batch point i of a fixed-base MSM
__device__ __forceinline__ uint32_t table_gen(const MsmDesc &d, const uint32_t *__restrict__ pt_idx, uint32_t i)
{
    return d.fixed == 2 ? __ldg(pt_idx + i) : i - d.pt_off;
}

template <bool SCATTER>
__global__ void k_recode(const uint4 *__restrict__ scalars, uint32_t n_total, const MsmDesc *__restrict__ desc,
                         uint32_t M, uint32_t *__restrict__ counts, const uint32_t *__restrict__ offsets,
                         uint32_t *__restrict__ sorted, const uint32_t *__restrict__ pt_idx)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_total)
        return;
    const uint32_t m = find_msm(M, i, [&](uint32_t k) { return desc[k].pt_off; });
    const uint32_t c = desc[m].c, base = desc[m].bucket_base;
    const bool fixed = desc[m].fixed != 0;
    const uint32_t pbase = fixed && SCATTER ? table_gen(desc[m], pt_idx, i) * desc[m].W : i;
    const uint32_t pstep = fixed ? 1u : 0u;
    const uint32_t wstep = fixed ? 0u : desc[m].B;
    const uint32_t w_lo = desc[m].w_lo, w_cnt = desc[m].w_cnt;
    const uint4 a = __ldg(scalars + 2 * (size_t)i), b = __ldg(scalars + 2 * (size_t)i + 1);
    const uint32_t s[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
    switch (c) {
#define HS_CASE(v)                                                       \
    case v:                                                              \
        recode_one<v, SCATTER>(s, pbase, pstep, wstep, base, w_lo, w_cnt, counts, offsets, sorted); \
        break;
        HS_CASE(4)
        HS_CASE(5)
        HS_CASE(6)
        HS_CASE(7)
        HS_CASE(8)
        HS_CASE(9)
        HS_CASE(10)
        HS_CASE(11)
        HS_CASE(12)
        HS_CASE(13)
        HS_CASE(14)
        HS_CASE(15)
        HS_CASE(16)
        HS_CASE(17)
        HS_CASE(18)
        HS_CASE(19)
        HS_CASE(20)
#undef HS_CASE
    default:
        break;
    }
}

// ---------------------------------------------------------------------------
// counting sort in shared memory (window widths up to 16): one block per
// (emitted window, point slice).  Bucket keys of one window fit a block's
// shared memory, so the per-entry atomics are shared-memory atomics; only one
// row of counts per block goes to global memory.
//   k_digits       every scalar's signed digits, window-major, in one pass
//   k_sort_count   count the block's keys, write its row of counts
//   k_sort_totals  per bucket: the sum of its rows -> counts (then the scan)
//   k_sort_offsets per bucket: each row's first slot, offsets + earlier rows
//   k_sort_scatter place "index | sign" at the row's slot + running fill
// ---------------------------------------------------------------------------
struct SortBlock {
    uint32_t m, k_abs, q, col, lo, hi;  // MSM, window, count row, first column, point range
};

__device__ __forceinline__ SortBlock sort_block(const MsmDesc *__restrict__ desc, uint32_t M, uint32_t blk)
{
    SortBlock sb;
    sb.m = find_msm(M, blk, [&](uint32_t k) { return desc[k].sblk_base; });
    const MsmDesc &d = desc[sb.m];
    const uint32_t local = blk - d.sblk_base;
    const uint32_t k = local / d.slices, s = local % d.slices;
    sb.k_abs = d.w_lo + k;
    sb.q = d.fixed ? k * d.slices + s : s;
    sb.col = d.fixed ? 0u : k * d.B;
    const uint32_t per = (d.n + d.slices - 1) / d.slices;
    sb.lo = d.pt_off + min(d.n, s * per);
    sb.hi = d.pt_off + min(d.n, (s + 1) * per);
    return sb;
}

__device__ __forceinline__ void load_scalar(const uint4 *__restrict__ scalars, uint32_t i, uint32_t s[8])
{
    const uint4 a = __ldg(scalars + 2 * (size_t)i), b = __ldg(scalars + 2 * (size_t)i + 1);
    s[0] = a.x; s[1] = a.y; s[2] = a.z; s[3] = a.w;
    s[4] = b.x; s[5] = b.y; s[6] = b.z; s[7] = b.w;
}

// all emitted signed digits of one scalar, window-major per MSM (the rule of
// recode_one: the carry runs up from window 0, the top window keeps it)
template <int CB>
__device__ __forceinline__ void digits_one(const uint32_t s[8], uint32_t w_lo, uint32_t w_cnt, uint32_t *__restrict__ out,
                                           uint32_t stride)
{
    constexpr int W = (257 + CB - 1) / CB;
    constexpr uint32_t B = 1u << (CB - 1);
    uint32_t carry = 0;
#pragma unroll
    for (int k = 0; k < W; k++) {
        const uint32_t v = window_bits<CB>(s, k) + carry;
        uint32_t mag, neg = 0;
        if (k < W - 1 && v >= B) {
            mag = (1u << CB) - v;
            neg = mag != 0 ? 1u : 0u;
            carry = 1;
        } else {
            mag = v;
            carry = 0;
        }
        if ((uint32_t)k - w_lo < w_cnt)
            out[(size_t)((uint32_t)k - w_lo) * stride] = mag | (neg << 31);
    }
}

__global__ void k_digits(const uint4 *__restrict__ scalars, uint32_t n_total, const MsmDesc *__restrict__ desc,
                         uint32_t M, uint32_t *__restrict__ digits)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_total)
        return;
    const uint32_t m = find_msm(M, i, [&](uint32_t k) { return desc[k].pt_off; });
    const MsmDesc &d = desc[m];
    uint32_t s[8];
    load_scalar(scalars, i, s);
    uint32_t *out = digits + d.dig_base + (i - d.pt_off);
    switch (d.c) {
#define HS_CASE(v)                                            \
    case v:                                                   \
        digits_one<v>(s, d.w_lo, d.w_cnt, out, d.n);          \
        break;
        HS_CASE(4)
        HS_CASE(5)
        HS_CASE(6)
        HS_CASE(7)
        HS_CASE(8)
        HS_CASE(9)
        HS_CASE(10)
        HS_CASE(11)
        HS_CASE(12)
        HS_CASE(13)
        HS_CASE(14)
        HS_CASE(15)
        HS_CASE(16)
#undef HS_CASE
    default:
        break;
    }
}

__global__ void __launch_bounds__(SORT_THREADS) k_sort_count(const uint32_t *__restrict__ digits,
                                                           const MsmDesc *__restrict__ desc, uint32_t M,
                                                           uint32_t *__restrict__ cnt)
{
    extern __shared__ uint32_t hist[];
    const SortBlock sb = sort_block(desc, M, blockIdx.x);
    const MsmDesc &d = desc[sb.m];
    for (uint32_t j = threadIdx.x; j < d.B; j += blockDim.x)
        hist[j] = 0;
    __syncthreads();
    const uint32_t *dg = digits + d.dig_base + (size_t)(sb.k_abs - d.w_lo) * d.n;
    // four independent loads in flight per thread, then their atomics
    const uint32_t step = blockDim.x;
    uint32_t i = sb.lo + threadIdx.x;
    for (; i + 3 * step < sb.hi; i += 4 * step) {
        uint32_t v[4];
#pragma unroll
        for (int u = 0; u < 4; u++)
            v[u] = __ldg(dg + (i + u * step - d.pt_off)) & 0x7fffffffu;
#pragma unroll
        for (int u = 0; u < 4; u++)
            if (v[u])
                atomicAdd(hist + v[u] - 1, 1u);
    }
    for (; i < sb.hi; i += step) {
        const uint32_t mag = __ldg(dg + (i - d.pt_off)) & 0x7fffffffu;
        if (mag)
            atomicAdd(hist + mag - 1, 1u);
    }
    __syncthreads();
    const uint64_t Bm = d.fixed ? d.B : (uint64_t)d.w_cnt * d.B;
    uint32_t *row = cnt + d.cnt_base + (uint64_t)sb.q * Bm + sb.col;
    for (uint32_t j = threadIdx.x; j < d.B; j += blockDim.x)
        row[j] = hist[j];
}

// one thread per bucket of the batch: total over its rows (mode 0), or turn the
// rows into first slots from offsets (mode 1; with offsets1, the rows from
// qsplit on -- part 1 of host inputs -- start at offsets1[bucket], their own list)
template <int MODE>
__global__ void k_sort_rows(const MsmDesc *__restrict__ desc, uint32_t M, uint32_t NB, uint32_t *__restrict__ cnt,
                            uint32_t *__restrict__ counts, const uint32_t *__restrict__ offsets, uint32_t qsplit,
                            uint32_t *__restrict__ counts0, const uint32_t *__restrict__ offsets1)
{
    const uint32_t kb = blockIdx.x * blockDim.x + threadIdx.x;
    if (kb >= NB)
        return;
    const uint32_t m = find_msm(M, kb, [&](uint32_t k) { return desc[k].bucket_base; });
    const MsmDesc &d = desc[m];
    const uint32_t lb = kb - d.bucket_base;
    const uint64_t Bm = d.fixed ? d.B : (uint64_t)d.w_cnt * d.B;
    const uint32_t Q = d.fixed ? d.w_cnt * d.slices : d.slices;
    uint32_t *col = cnt + d.cnt_base + lb;
    uint32_t run = MODE == 0 ? 0u : offsets[kb];
    uint32_t c0 = 0;  // entries of the rows below qsplit (host inputs in two parts)
    for (uint32_t q0 = 0; q0 < Q; q0 += 8) {  // eight loads in flight, then their sums
        uint32_t v[8];
#pragma unroll
        for (int u = 0; u < 8; u++)
            v[u] = q0 + u < Q ? col[(uint64_t)(q0 + u) * Bm] : 0u;
#pragma unroll
        for (int u = 0; u < 8; u++) {
            if (MODE == 1 && offsets1 && q0 + u == qsplit)
                run = offsets1[kb];
            if (MODE == 1 && q0 + u < Q)
                col[(uint64_t)(q0 + u) * Bm] = run;
            if (MODE == 0 && q0 + u == qsplit)
                c0 = run;
            run += v[u];
        }
    }
    if (MODE == 0) {
        counts[kb] = run;
        if (counts0)
            counts0[kb] = qsplit < Q ? c0 : run;
    }
}

__global__ void __launch_bounds__(SORT_THREADS) k_sort_scatter(const uint32_t *__restrict__ digits,
                                                             const MsmDesc *__restrict__ desc, uint32_t M,
                                                             const uint32_t *__restrict__ cnt,
                                                             uint32_t *__restrict__ sorted,
                                                             const uint32_t *__restrict__ pt_idx)
{
    extern __shared__ uint32_t slot[];
    const SortBlock sb = sort_block(desc, M, blockIdx.x);
    const MsmDesc &d = desc[sb.m];
    const uint64_t Bm = d.fixed ? d.B : (uint64_t)d.w_cnt * d.B;
    const uint32_t *row = cnt + d.cnt_base + (uint64_t)sb.q * Bm + sb.col;
    for (uint32_t j = threadIdx.x; j < d.B; j += blockDim.x)
        slot[j] = row[j];
    __syncthreads();
    const uint32_t *dg = digits + d.dig_base + (size_t)(sb.k_abs - d.w_lo) * d.n;
    const uint32_t step = blockDim.x;
    uint32_t i = sb.lo + threadIdx.x;
    for (; i + 3 * step < sb.hi; i += 4 * step) {
        uint32_t dv[4];
#pragma unroll
        for (int u = 0; u < 4; u++)
            dv[u] = __ldg(dg + (i + u * step - d.pt_off));
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const uint32_t mag = dv[u] & 0x7fffffffu;
            if (mag) {
                const uint32_t ii = i + u * step;
                const uint32_t pos = atomicAdd(slot + mag - 1, 1u);
                const uint32_t v = d.fixed ? table_gen(d, pt_idx, ii) * d.W + sb.k_abs : ii;
                sorted[pos] = v | (dv[u] & 0x80000000u);
            }
        }
    }
    for (; i < sb.hi; i += step) {
        const uint32_t dv = __ldg(dg + (i - d.pt_off)), mag = dv & 0x7fffffffu;
        if (mag) {
            const uint32_t pos = atomicAdd(slot + mag - 1, 1u);
            const uint32_t v = d.fixed ? table_gen(d, pt_idx, i) * d.W + sb.k_abs : i;
            sorted[pos] = v | (dv & 0x80000000u);
        }
    }
}

// exclusive scan of (count, ceil(count / L)) pairs, three phases
__device__ __forceinline__ uint2 warp_incl_scan(uint2 v)
{
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t x = __shfl_up_sync(0xffffffffu, v.x, d);
        const uint32_t y = __shfl_up_sync(0xffffffffu, v.y, d);
        if (lane >= d) {
            v.x += x;
            v.y += y;
        }
    }
    return v;
}

// block-wide exclusive scan of one pair per thread; returns the prefix, sets *total
__device__ __forceinline__ uint2 block_excl_scan(uint2 v, uint2 *total)
{
    __shared__ uint2 warp_tot[SCAN_THREADS / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint2 inc = warp_incl_scan(v);
    __syncthreads();
    if (lane == 31)
        warp_tot[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        uint2 t = (lane < (int)(blockDim.x >> 5)) ? warp_tot[lane] : make_uint2(0, 0);
        const uint2 ti = warp_incl_scan(t);
        warp_tot[lane] = make_uint2(ti.x - t.x, ti.y - t.y);  // exclusive warp prefix
        if (lane == 31)
            *total = ti;
    }
    __syncthreads();
    const uint2 wp = warp_tot[warp];
    return make_uint2(wp.x + inc.x - v.x, wp.y + inc.y - v.y);
}

// destination slots of a bucket of c entries, c0 of them in part 0 of host
// inputs in two parts: its segments per part, less one when both parts have
// some (the first part-1 segment continues the first part-0 segment's sum)
__device__ __forceinline__ uint32_t part_slots(uint32_t c, uint32_t c0, uint32_t L)
{
    const uint32_t c1 = c - c0;
    return (c0 + L - 1) / L + (c1 + L - 1) / L - ((c0 && c1) ? 1u : 0u);
}

// pad: counts rounded up to a multiple of pad + 1 (a power of two) first.
// split_nb > 0 (batch-affine plans of host inputs in two parts): the n =
// 2 split_nb lists are bucket k's part-0 entries (list k) and part-1 entries
// (list split_nb + k), each padded, and bucket k's segment slots -- over the
// last round's lists, 2^shift times shorter -- are counted at list k.
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_a(const uint32_t *__restrict__ counts, uint32_t NB, uint32_t L,
                                                        uint32_t *__restrict__ offsets, uint32_t *__restrict__ seg_off,
                                                        uint32_t *__restrict__ tmp, const uint32_t *__restrict__ counts0,
                                                        uint32_t pad, uint32_t split_nb, uint32_t shift)
{
    __shared__ uint2 tot;
    const uint32_t base = blockIdx.x * SCAN_BLOCK + threadIdx.x * SCAN_ITEMS;
    uint32_t c[SCAN_ITEMS], s[SCAN_ITEMS];
    uint2 v = make_uint2(0, 0);
#pragma unroll
    for (int j = 0; j < SCAN_ITEMS; j++) {
        const uint32_t idx = base + j;
        if (split_nb) {
            const uint32_t k = idx < split_nb ? idx : idx - split_nb;
            const uint32_t c0 = idx < NB ? (counts0[k] + pad) & ~pad : 0u;
            const uint32_t c1 = idx < NB ? (counts[k] - counts0[k] + pad) & ~pad : 0u;
            c[j] = idx < split_nb ? c0 : c1;
            s[j] = idx < split_nb ? part_slots((c0 + c1) >> shift, c0 >> shift, L) : 0u;
        } else {
            c[j] = idx < NB ? (counts[idx] + pad) & ~pad : 0u;
            s[j] = counts0 ? (idx < NB ? part_slots(c[j], counts0[idx], L) : 0u) : (c[j] + L - 1) / L;
        }
        v.x += c[j];
        v.y += s[j];
    }
    uint2 pre = block_excl_scan(v, &tot);
#pragma unroll
    for (int j = 0; j < SCAN_ITEMS; j++) {
        const uint32_t idx = base + j;
        if (idx < NB) {
            offsets[idx] = pre.x;
            if (seg_off)
                seg_off[idx] = pre.y;
        }
        pre.x += c[j];
        pre.y += s[j];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        tmp[2 * blockIdx.x] = tot.x;
        tmp[2 * blockIdx.x + 1] = tot.y;
    }
}

// scan of the block partials, in chunks of SCAN_BLOCK with a running carry
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_b(uint32_t *__restrict__ tmp, uint32_t nblocks,
                                                        uint32_t *__restrict__ off_total,
                                                        uint32_t *__restrict__ seg_total)
{
    __shared__ uint2 tot;
    uint2 carry = make_uint2(0, 0);
    for (uint32_t chunk = 0; chunk < nblocks; chunk += SCAN_BLOCK) {
        const uint32_t base = chunk + threadIdx.x * SCAN_ITEMS;
        uint2 it[SCAN_ITEMS];
        uint2 v = make_uint2(0, 0);
#pragma unroll
        for (int j = 0; j < SCAN_ITEMS; j++) {
            const uint32_t idx = base + j;
            it[j] = idx < nblocks ? make_uint2(tmp[2 * idx], tmp[2 * idx + 1]) : make_uint2(0, 0);
            v.x += it[j].x;
            v.y += it[j].y;
        }
        uint2 pre = block_excl_scan(v, &tot);
        pre.x += carry.x;
        pre.y += carry.y;
#pragma unroll
        for (int j = 0; j < SCAN_ITEMS; j++) {
            const uint32_t idx = base + j;
            if (idx < nblocks) {
                tmp[2 * idx] = pre.x;
                tmp[2 * idx + 1] = pre.y;
            }
            pre.x += it[j].x;
            pre.y += it[j].y;
        }
        __syncthreads();
        carry.x += tot.x;
        carry.y += tot.y;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        *off_total = carry.x;
        if (seg_total)
            *seg_total = carry.y;
    }
}

__global__ void k_scan_c(uint32_t *__restrict__ offsets, uint32_t *__restrict__ seg_off, uint32_t NB,
                         const uint32_t *__restrict__ tmp)
{
    const uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= NB)
        return;
    const uint32_t blk = idx / SCAN_BLOCK;
    offsets[idx] += tmp[2 * blk];
    if (seg_off)
        seg_off[idx] += tmp[2 * blk + 1];
}

// Segments (<= L entries of one bucket) are emitted longest first so that the
// 32 lanes of a warp in k_accumulate get equal work: a per-block histogram of
// segment lengths, a scan over (length descending, block), and a scatter
// through block-local cursors.  Each descriptor carries its destination slot
// seg_off[bucket] + j, so a bucket's partial sums stay contiguous.
// shift: the lists segmented are the entry lists shifted right by it (the last
// batch-affine round's, 2^shift times shorter; offsets are multiples of 2^shift)
// A bucket's list, or its two part lists: [start0, start0 + c0) and [start1,
// start1 + c1).  One list (counts0 null): c1 = 0.  Host inputs in two parts:
// the part-0 entries come first in the bucket's list (counts0), or with
// offsets1 (batch-affine plans) each part has its own list, bucket kb's part-1
// list starting at offsets1[kb].
struct PartLists {
    uint32_t start0, c0, start1, c1;
};

__device__ __forceinline__ PartLists part_lists(const uint32_t *__restrict__ offsets,
                                                const uint32_t *__restrict__ offsets1,
                                                const uint32_t *__restrict__ counts0, uint32_t kb, uint32_t shift)
{
    PartLists l;
    l.start0 = offsets[kb] >> shift;
    const uint32_t cnt = (offsets[kb + 1] >> shift) - l.start0;
    if (offsets1) {
        l.c0 = cnt;
        l.start1 = offsets1[kb] >> shift;
        l.c1 = (offsets1[kb + 1] >> shift) - l.start1;
    } else {
        l.c0 = counts0 ? counts0[kb] : cnt;
        l.start1 = l.start0 + l.c0;
        l.c1 = cnt - l.c0;
    }
    return l;
}

__global__ void __launch_bounds__(SEG_HIST_THREADS) k_seg_hist(const uint32_t *__restrict__ offsets, uint32_t NB,
                                                              uint32_t L, uint32_t nblk, uint32_t *__restrict__ hist,
                                                              const uint32_t *__restrict__ counts0, uint32_t shift,
                                                              const uint32_t *__restrict__ offsets1)
{
    extern __shared__ uint32_t h[];
    const uint32_t parts = (counts0 || offsets1) ? 2u : 1u;
    for (uint32_t i = threadIdx.x; i < parts * (L + 1); i += blockDim.x)
        h[i] = 0;
    __syncthreads();
    const uint32_t kb = blockIdx.x * blockDim.x + threadIdx.x;
    if (kb < NB) {
        const PartLists pl = part_lists(offsets, offsets1, counts0, kb, shift);
        for (uint32_t part = 0; part < parts; part++) {
            const uint32_t c = part ? pl.c1 : pl.c0;
            const uint32_t nfull = c / L, rem = c % L;
            if (nfull)
                atomicAdd(&h[part * (L + 1) + L], nfull);
            if (rem)
                atomicAdd(&h[part * (L + 1) + rem], 1u);
        }
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < parts * (L + 1); i += blockDim.x) {
        const uint32_t part = i / (L + 1), len = i % (L + 1);
        hist[(size_t)(part * (L + 1) + L - len) * nblk + blockIdx.x] = h[i];
    }
}

// one part's segments of a bucket: entries [start, start + cnt) cut into
// pieces of L (then the remainder); piece j goes to slot first (j = 0) or
// rest + j - 1, the first one continuing the stored sum when resume is set
__device__ __forceinline__ void emit_segments(uint32_t *cur, uint32_t L, uint32_t start, uint32_t cnt, uint32_t first,
                                              uint32_t rest, uint32_t resume, uint4 *__restrict__ segs)
{
    const uint32_t nfull = cnt / L, rem = cnt % L;
    if (nfull) {
        const uint32_t p = atomicAdd(&cur[L], nfull);
        for (uint32_t j = 0; j < nfull; j++)
            segs[p + j] = make_uint4(start + j * L, L, j ? rest + j - 1 : first, j ? 0u : resume);
    }
    if (rem) {
        const uint32_t p = atomicAdd(&cur[rem], 1u);
        segs[p] = make_uint4(start + nfull * L, rem, nfull ? rest + nfull - 1 : first, nfull ? 0u : resume);
    }
}

__global__ void __launch_bounds__(SEG_HIST_THREADS) k_seg_scatter(const uint32_t *__restrict__ offsets,
                                                                 const uint32_t *__restrict__ seg_off, uint32_t NB,
                                                                 uint32_t L, uint32_t nblk,
                                                                 const uint32_t *__restrict__ hist_scan,
                                                                 uint4 *__restrict__ segs,
                                                                 const uint32_t *__restrict__ counts0, uint32_t shift,
                                                                 const uint32_t *__restrict__ offsets1)
{
    extern __shared__ uint32_t cur[];
    const uint32_t parts = (counts0 || offsets1) ? 2u : 1u;
    for (uint32_t i = threadIdx.x; i < parts * (L + 1); i += blockDim.x) {
        const uint32_t part = i / (L + 1), len = i % (L + 1);
        cur[i] = hist_scan[(size_t)(part * (L + 1) + L - len) * nblk + blockIdx.x];
    }
    __syncthreads();
    const uint32_t kb = blockIdx.x * blockDim.x + threadIdx.x;
    if (kb >= NB)
        return;
    const PartLists pl = part_lists(offsets, offsets1, counts0, kb, shift);
    const uint32_t dest = seg_off[kb];
    emit_segments(cur, L, pl.start0, pl.c0, dest, dest + 1, 0u, segs);
    if (parts == 1)
        return;
    const uint32_t s0 = (pl.c0 + L - 1) / L;
    if (s0)
        emit_segments(cur + (L + 1), L, pl.start1, pl.c1, dest, dest + s0, 1u, segs);
    else
        emit_segments(cur + (L + 1), L, pl.start1, pl.c1, dest, dest + 1, 0u, segs);
}

static cudaError_t launch_scan(Context &ctx, const uint32_t *in, uint32_t n, uint32_t L, uint32_t *out,
                               uint32_t *out2, uint32_t *tmp, const uint32_t *counts0 = nullptr, uint32_t pad = 0,
                               uint32_t split_nb = 0, uint32_t shift = 0)
{
    cudaStream_t st = ctx.stream;
    const uint32_t nblk = std::max<uint32_t>(1, scan_blocks(n));
    k_scan_a<<<nblk, SCAN_THREADS, 0, st>>>(in, n, L, out, out2, tmp, counts0, pad, split_nb, shift);
    HS_LAUNCH_CHECK(ctx);
    k_scan_b<<<1, SCAN_THREADS, 0, st>>>(tmp, nblk, out + n, out2 ? out2 + n : nullptr);
    HS_LAUNCH_CHECK(ctx);
    if (n) {
        k_scan_c<<<(n + 255) / 256, 256, 0, st>>>(out, out2, n, tmp);
        HS_LAUNCH_CHECK(ctx);
    }
    return cudaSuccess;
}

// recode + counting sort + segments of a whole batch (descriptors already on the device)
// the sort kernels' shared-memory opt-in, once per device (outside any capture:
// contexts set it when they are created)
cudaError_t sort_smem_attrs(int device)
{
    static std::once_flag once[64];
    static cudaError_t err[64];
    if (device < 0 || device >= 64)
        return cudaErrorInvalidDevice;
    std::call_once(once[device], [device] {
        int prev = 0;
        cudaGetDevice(&prev);
        cudaSetDevice(device);
        cudaError_t a = cudaFuncSetAttribute(k_sort_count, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)(SORT_SMEM_MAX_B * 4));
        cudaError_t b = cudaFuncSetAttribute(k_sort_scatter, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)(SORT_SMEM_MAX_B * 4));
        cudaSetDevice(prev);
        err[device] = a != cudaSuccess ? a : b;
    });
    return err[device];
}

cudaError_t launch_sort(Context &ctx, const BatchPlan &p, const BatchBuffers &b)
{
    cudaStream_t st = ctx.stream;
    cudaError_t e;
    if ((e = cudaMemsetAsync(b.counts, 0, (size_t)(p.NB + 1) * 4, st)) != cudaSuccess)
        return e;
    const uint4 *sc = reinterpret_cast<const uint4 *>(b.scalars);
    // batch-affine plans: every bucket's list padded to a multiple of 2^R with
    // PAD_ENTRY (the identity), and the fold's segments counted on lists 2^R
    // times shorter
    const uint32_t pad = p.ba_rounds ? (1u << p.ba_rounds) - 1 : 0u;
    const uint32_t seg_L = p.L << p.ba_rounds;
    if (p.ba_rounds && (e = cudaMemsetAsync(b.sorted, 0xff, (size_t)p.max_entries * 4, st)) != cudaSuccess)
        return e;
    // batch-affine rounds over host inputs in two parts: each part's entries of
    // a bucket form their own padded list (list NB*part + bucket)
    const bool split_lists = p.ba_rounds && p.part_slice;
    if (p.smem_sort()) {
        if ((e = sort_smem_attrs(ctx.device)) != cudaSuccess)
            return e;
        const size_t smem = (size_t)p.max_B * 4;
        const unsigned tb = (p.NB + 255) / 256;
        if (p.n_total) {
            k_digits<<<(p.n_total + 255) / 256, 256, 0, st>>>(sc, p.n_total, b.desc, p.M, b.digits);
            HS_LAUNCH_CHECK(ctx);
        }
        k_sort_count<<<p.sort_blocks, SORT_THREADS, smem, st>>>(b.digits, b.desc, p.M, b.sort_cnt);
        HS_LAUNCH_CHECK(ctx);
        const uint32_t *c0 = p.part_slice ? b.counts0 : nullptr;
        k_sort_rows<0><<<tb, 256, 0, st>>>(b.desc, p.M, p.NB, b.sort_cnt, b.counts, nullptr, p.part_slice,
                                           p.part_slice ? b.counts0 : nullptr, nullptr);
        HS_LAUNCH_CHECK(ctx);
        if (split_lists) {  // a list per (part, bucket), each padded; segment slots on the last round's lists
            if ((e = launch_scan(ctx, b.counts, 2 * p.NB, p.L, b.offsets, b.seg_off, b.scan_tmp, c0, pad, p.NB,
                                 p.ba_rounds)) != cudaSuccess)
                return e;
        } else if ((e = launch_scan(ctx, b.counts, p.NB, seg_L, b.offsets, b.seg_off, b.scan_tmp, c0, pad)) !=
                   cudaSuccess) {
            return e;
        }
        k_sort_rows<1><<<tb, 256, 0, st>>>(b.desc, p.M, p.NB, b.sort_cnt, nullptr, b.offsets, p.part_slice, nullptr,
                                           split_lists ? b.offsets + p.NB : nullptr);
        HS_LAUNCH_CHECK(ctx);
        k_sort_scatter<<<p.sort_blocks, SORT_THREADS, smem, st>>>(b.digits, b.desc, p.M, b.sort_cnt, b.sorted,
                                                                  b.pt_idx);
        HS_LAUNCH_CHECK(ctx);
    } else {
        const unsigned rblocks = (p.n_total + 255) / 256;
        if (p.n_total) {
            k_recode<false><<<rblocks, 256, 0, st>>>(sc, p.n_total, b.desc, p.M, b.counts, b.offsets, b.sorted,
                                                      b.pt_idx);
            HS_LAUNCH_CHECK(ctx);
        }
        if ((e = launch_scan(ctx, b.counts, p.NB, seg_L, b.offsets, b.seg_off, b.scan_tmp, nullptr, pad)) !=
            cudaSuccess)
            return e;
        if ((e = cudaMemsetAsync(b.counts, 0, (size_t)(p.NB + 1) * 4, st)) != cudaSuccess)
            return e;
        if (p.n_total) {
            k_recode<true><<<rblocks, 256, 0, st>>>(sc, p.n_total, b.desc, p.M, b.counts, b.offsets, b.sorted,
                                                     b.pt_idx);
            HS_LAUNCH_CHECK(ctx);
        }
    }
    // segments, longest first
    const uint32_t nh = (uint32_t)hist_len(p);
    const uint32_t *c0 = (p.part_slice && p.smem_sort() && !split_lists) ? b.counts0 : nullptr;
    const uint32_t *off1 = split_lists ? b.offsets + p.NB : nullptr;
    const size_t hsm = (size_t)(p.L + 1) * 4 * ((c0 || off1) ? 2 : 1);
    k_seg_hist<<<p.hist_blocks, SEG_HIST_THREADS, hsm, st>>>(b.offsets, p.NB, p.L, p.hist_blocks, b.len_hist, c0,
                                                             p.ba_rounds, off1);
    HS_LAUNCH_CHECK(ctx);
    if ((e = launch_scan(ctx, b.len_hist, nh, 1u, b.len_scan, nullptr, b.scan_tmp)) != cudaSuccess)
        return e;
    k_seg_scatter<<<p.hist_blocks, SEG_HIST_THREADS, hsm, st>>>(b.offsets, b.seg_off, p.NB, p.L, p.hist_blocks,
                                                                 b.len_scan, b.segs, c0, p.ba_rounds, off1);
    HS_LAUNCH_CHECK(ctx);
    return cudaSuccess;
}

// ---------------------------------------------------------------------------
// instrumentation
// ---------------------------------------------------------------------------
void prof_begin(Context &ctx, cudaEvent_t *ev)
{
    *ev = nullptr;
    if (!ctx.profile)
        return;
    if (cudaEventCreate(ev) != cudaSuccess) {
        *ev = nullptr;
        return;
    }
    cudaEventRecord(*ev, ctx.stream);
}

void prof_end(Context &ctx, cudaEvent_t ev0, uint64_t entries)
{
    if (!ev0)
        return;
    cudaEvent_t ev1;
    if (cudaEventCreate(&ev1) != cudaSuccess)
        return;
    cudaEventRecord(ev1, ctx.stream);
    ctx.prof_events.emplace_back(ev0, ev1);
    ctx.prof_entries += entries;
    ctx.prof_launches++;
}

// Probes of the integer-multiply pipe, 8 independent chains per thread:
// MODE 0 alternates mad.lo / mad.hi (one 32x32->64 product = 2 IMAD-equivalents
// per pair), MODE 1 is mad.lo alone, MODE 2 mad.hi alone; k_imad_wide_peak runs
// mad.wide.u32 chains (the whole product in one instruction).  The ceiling is
// the faster of the two product forms.
template <int MODE>
__global__ void k_imad_peak(uint32_t seed, int iters, uint32_t *out)
{
    uint32_t a[8], b = seed ^ (threadIdx.x * 0x9e3779b9u) ^ blockIdx.x;
#pragma unroll
    for (int k = 0; k < 8; k++)
        a[k] = b + (uint32_t)k * 0x85ebca6bu;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < 8; k++) {
            if (MODE != 2)
                asm volatile("mad.lo.u32 %0, %0, %1, %2;" : "+r"(a[k]) : "r"(b), "r"((uint32_t)k));
            if (MODE != 1)
                asm volatile("mad.hi.u32 %0, %0, %1, %0;" : "+r"(a[k]) : "r"(b));
        }
    }
    uint32_t r = 0;
#pragma unroll
    for (int k = 0; k < 8; k++)
        r ^= a[k];
    if (r == 0x12345678u)
        out[blockIdx.x * blockDim.x + threadIdx.x] = r;
}

__global__ void k_imad_wide_peak(uint32_t seed, int iters, uint32_t *out)
{
    uint64_t acc[8];
    uint32_t a = seed ^ (threadIdx.x * 0x9e3779b9u) ^ blockIdx.x, b = a * 0x85ebca6bu + 1u;
#pragma unroll
    for (int k = 0; k < 8; k++)
        acc[k] = (uint64_t)(a + (uint32_t)k) << 7;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < 8; k++) {
            // acc = lo32(acc) * b + acc: one full product per step, each chain depending on itself
            asm volatile("mad.wide.u32 %0, %1, %2, %0;" : "+l"(acc[k]) : "r"((uint32_t)acc[k]), "r"(b));
        }
    }
    uint64_t r = 0;
#pragma unroll
    for (int k = 0; k < 8; k++)
        r ^= acc[k];
    if ((uint32_t)r == 0x12345678u)
        out[blockIdx.x * blockDim.x + threadIdx.x] = (uint32_t)(r >> 32);
}

// ---------------------------------------------------------------------------
// host helpers for the C ABI
// ---------------------------------------------------------------------------
int fail(Context &ctx, cudaError_t e, const char *what)
{
    ctx.last_error = std::string(what) + ": " + cudaGetErrorString(e);
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? HS_ENOMEM : HS_ECUDA;
}

int fail_msg(Context &ctx, int code, const char *what)
{
    ctx.last_error = what;
    return code;
}

#define HS_CU(call, what)                        \
    do {                                         \
        cudaError_t e_ = (call);                 \
        if (e_ != cudaSuccess)                   \
            return fail(ctx, e_, what);          \
    } while (0)

static void identity_out(int curve, int out_fmt, void *out)
{
    (void)curve;
    std::memset(out, 0, fmt_bytes(out_fmt));
    if (out_fmt == HS_FMT_JACOBIAN51) {
        uint64_t *o = static_cast<uint64_t *>(out);
        o[0] = 1;  // X = 1
        o[5] = 1;  // Y = 1, Z = 0 (helios/include/helios_ops.h:45-50)
    }
}

static bool valid_curve(int c) { return c == HS_HELIOS || c == HS_SELENE; }
static bool valid_in_fmt(int f) { return f == HS_FMT_JACOBIAN51 || f == HS_FMT_AFFINE51 || f == HS_FMT_AFFINE; }
// point inputs of the MSM forms: also the 32-byte encoding, decoded on the device
static bool valid_pt_fmt(int f) { return valid_in_fmt(f) || f == HS_FMT_COMPRESSED; }

// after a stream synchronise: the invalid-encoding count that to_affine left in
// the first word of its scratch
static int check_decoded(Context &ctx, const void *d_scratch)
{
    uint32_t bad = 0;
    HS_CU(cudaMemcpy(&bad, d_scratch, sizeof(bad), cudaMemcpyDeviceToHost), "decode check");
    if (bad)
        return fail_msg(ctx, HS_EINVAL, "invalid point encoding");
    return HS_OK;
}
static bool valid_out_fmt(int f) { return f >= HS_FMT_JACOBIAN51 && f <= HS_FMT_COMPRESSED; }

// Reserve the arena for one batch plus extra_bytes of call-specific staging
// (one reservation: a later reserve could move the arena).
int reserve_batch(Context &ctx, const BatchPlan &p, size_t extra_bytes, BatchBuffers &b, void **extra)
{
    HS_CU(ctx.arena.reserve(batch_bytes(p) + align256(extra_bytes) + 1024), "workspace allocation");
    if (!carve(ctx.arena, p, b))
        return fail_msg(ctx, HS_ENOMEM, "workspace carve");
    if (extra) {
        *extra = extra_bytes ? ctx.arena.take(extra_bytes) : nullptr;
        if (extra_bytes && !*extra)
            return fail_msg(ctx, HS_ENOMEM, "workspace carve");
    }
    return HS_OK;
}

cudaError_t launch_batch(Context &ctx, const BatchPlan &p, const BatchBuffers &b, void *d_out, int out_fmt)
{
    cudaError_t e;
    if ((e = launch_sort(ctx, p, b)) != cudaSuccess)
        return e;
    const CurveOps &ops = curve_ops(p.curve);
    if ((e = ops.msm_tail(ctx, p, b)) != cudaSuccess)
        return e;
    return ops.format_out(ctx, b.out_jac, p.M, out_fmt, d_out);
}

// Run a batch plan whose inputs are in b.scalars / b.points (device, concatenated),
// results (M records of out_fmt) to d_out.  The descriptors are uploaded every
// time; the launch sequence is captured once per (shape, buffers) and replayed.
int execute_batch(Context &ctx, const BatchPlan &p, const BatchBuffers &b, void *d_out, int out_fmt)
{
    cudaStream_t st = ctx.stream;
    if (!ctx.use_graphs || ctx.profile) {
        HS_CU(cudaMemcpyAsync(b.desc, p.msms.data(), (size_t)p.M * sizeof(MsmDesc), cudaMemcpyHostToDevice, st),
              "descriptor upload");
        HS_CU(launch_batch(ctx, p, b, d_out, out_fmt), "MSM launch");
        return HS_OK;
    }
    std::vector<uint64_t> key;
    key.reserve(12 + 2 * p.M);
    key.push_back((uint64_t)p.curve);
    key.push_back((uint64_t)p.M);
    key.push_back((uint64_t)out_fmt);
    key.push_back((uint64_t)(uintptr_t)ctx.arena.base);
    key.push_back((uint64_t)ctx.arena.cap);
    key.push_back((uint64_t)(uintptr_t)b.scalars);
    key.push_back((uint64_t)(uintptr_t)b.points);
    key.push_back((uint64_t)(uintptr_t)d_out);
    key.push_back((uint64_t)(uintptr_t)st);
    key.push_back((uint64_t)(uintptr_t)b.counts);
    key.push_back((uint64_t)p.ba_rounds);
    for (const MsmDesc &d : p.msms) {
        key.push_back(((uint64_t)d.n << 16) | ((uint64_t)d.fixed << 8) | d.c);
        key.push_back(d.pt_off);
    }
    for (GraphEntry &g : ctx.graphs) {
        if (g.key == key) {
            HS_CU(cudaGraphLaunch(g.exec, st), "graph launch");
            ctx.launches += g.kernels;
            return HS_OK;
        }
    }
    // The descriptors of a captured shape live in a buffer owned by the graph:
    // uploaded once here, so a replay needs no host copy (a pageable copy
    // would synchronise the stream).
    GraphEntry ent;
    HS_CU(cudaMalloc(&ent.d_desc, (size_t)p.M * sizeof(MsmDesc)), "descriptor allocation");
    cudaError_t ue = cudaMemcpy(ent.d_desc, p.msms.data(), (size_t)p.M * sizeof(MsmDesc), cudaMemcpyHostToDevice);
    if (ue != cudaSuccess) {
        cudaFree(ent.d_desc);
        return fail(ctx, ue, "descriptor upload");
    }
    BatchBuffers bg = b;
    bg.desc = (MsmDesc *)ent.d_desc;
    cudaGraph_t graph = nullptr;
    const uint64_t before = ctx.launches;
    cudaError_t ce = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
    cudaError_t le = ce == cudaSuccess ? launch_batch(ctx, p, bg, d_out, out_fmt) : ce;
    if (ce == cudaSuccess)
        ce = cudaStreamEndCapture(st, &graph);
    if (le != cudaSuccess || ce != cudaSuccess) {
        if (graph)
            cudaGraphDestroy(graph);
        cudaFree(ent.d_desc);
        return fail(ctx, le != cudaSuccess ? le : ce, "graph capture");
    }
    cudaGraphExec_t exec = nullptr;
    cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ie != cudaSuccess) {
        cudaFree(ent.d_desc);
        return fail(ctx, ie, "graph instantiate");
    }
    ent.key = std::move(key);
    ent.exec = exec;
    ent.kernels = ctx.launches - before;
    if (ctx.graphs.size() >= 64) {
        cudaStreamSynchronize(st);
        cudaGraphExecDestroy(ctx.graphs.front().exec);
        cudaFree(ctx.graphs.front().d_desc);
        ctx.graphs.erase(ctx.graphs.begin());
    }
    ctx.graphs.push_back(std::move(ent));
    HS_CU(cudaGraphLaunch(exec, st), "graph launch");
    return HS_OK;
}

// ---------------------------------------------------------------------------
// window-split MSM: the upper windows on the context stream, the lower windows
// on a second, lower-priority stream, joined by one point addition.  The upper
// half carries the long Horner chain (its extra c*w_lo doublings), so it starts
// first and its chain runs while the lower half is still accumulating.
// ---------------------------------------------------------------------------
// the second stream gets the greatest priority: the upper window half goes there
static cudaError_t ensure_stream2(Context &ctx)
{
    cudaError_t e = cudaSuccess;
    if (!ctx.stream2) {
        int least = 0, greatest = 0;
        if ((e = cudaDeviceGetStreamPriorityRange(&least, &greatest)) != cudaSuccess)
            return e;
        if ((e = cudaStreamCreateWithPriority(&ctx.stream2, cudaStreamNonBlocking, greatest)) != cudaSuccess)
            return e;
    }
    if (!ctx.ev_fork && (e = cudaEventCreateWithFlags(&ctx.ev_fork, cudaEventDisableTiming)) != cudaSuccess)
        return e;
    if (!ctx.ev_join && (e = cudaEventCreateWithFlags(&ctx.ev_join, cudaEventDisableTiming)) != cudaSuccess)
        return e;
    if (!ctx.stream3) {
        int least = 0, greatest = 0;
        if ((e = cudaDeviceGetStreamPriorityRange(&least, &greatest)) != cudaSuccess)
            return e;
        if ((e = cudaStreamCreateWithPriority(&ctx.stream3, cudaStreamNonBlocking, greatest)) != cudaSuccess)
            return e;
    }
    for (cudaEvent_t *ev : {&ctx.ev_sc, &ctx.ev_rec[0], &ctx.ev_rec[1], &ctx.ev_pts[0], &ctx.ev_pts[1]})
        if (!*ev && (e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming)) != cudaSuccess)
            return e;
    return e;
}

// The host-to-device input copies of every context on a device go to one
// stream, in the order the calls issue them (one call's copies back to back
// under the mutex).  Calls from several host threads then receive their inputs
// one after another at the link's full rate, so the first can start computing
// while the next is still arriving, instead of all of them sharing the link and
// all starting late.  The streams live as long as the process.
struct LinkStream {
    std::mutex mu;
    cudaStream_t s = nullptr;
};

static cudaError_t link_stream(int device, LinkStream **out)
{
    static std::mutex reg_mu;
    static std::vector<LinkStream *> reg;
    std::lock_guard<std::mutex> lk(reg_mu);
    if (device < 0)
        return cudaErrorInvalidDevice;
    if (reg.size() <= (size_t)device)
        reg.resize((size_t)device + 1, nullptr);
    if (!reg[device]) {
        LinkStream *ls = new (std::nothrow) LinkStream();
        if (!ls)
            return cudaErrorMemoryAllocation;
        // the greatest priority: the copy kernels of pageable inputs (h2d_async)
        // then take SM slots ahead of the compute kernels waiting for them
        int least = 0, greatest = 0;
        cudaDeviceGetStreamPriorityRange(&least, &greatest);
        const cudaError_t e = cudaStreamCreateWithPriority(&ls->s, cudaStreamNonBlocking, greatest);
        if (e != cudaSuccess) {
            delete ls;
            return e;
        }
        reg[device] = ls;
    }
    *out = reg[device];
    return cudaSuccess;
}

// Host-to-device copies from pageable host memory.  A copy-engine copy from
// pageable memory returns only once its data has been staged: it holds the
// calling thread for the whole transfer (after draining the stream), so the
// launches queued behind it -- and other threads' copies on the shared link
// stream -- start late.  On a device that reads pageable host memory directly
// (cudaDevAttrPageableMemoryAccess: Grace-class hosts, where the GPU reaches
// system memory through the host's page tables) a copy kernel reading the
// caller's pages is stream-ordered and returns at once, like a copy from pinned
// memory, and runs at the same link rate (about 209 GB/s on GB300 for both, and
// for copy-engine copies from pinned memory).  Pinned, registered, managed and
// device memory keep the copy engine.
constexpr int PULL_DEPTH = 8;
constexpr int PULL_BLOCK_DIV = 4;

template <class Word>
__global__ void __launch_bounds__(256) k_pull(const Word *__restrict__ src, Word *__restrict__ dst, size_t words,
                                              const uint8_t *__restrict__ src_tail, uint8_t *__restrict__ dst_tail,
                                              uint32_t tail)
{
    const size_t T = (size_t)gridDim.x * blockDim.x;
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    // PULL_DEPTH loads in flight per thread: the link's latency is microseconds
    for (; i + (PULL_DEPTH - 1) * T < words; i += PULL_DEPTH * T) {
        Word v[PULL_DEPTH];
#pragma unroll
        for (int k = 0; k < PULL_DEPTH; k++)
            v[k] = src[i + k * T];
#pragma unroll
        for (int k = 0; k < PULL_DEPTH; k++)
            dst[i + k * T] = v[k];
    }
    for (; i < words; i += T)
        dst[i] = src[i];
    if (blockIdx.x == 0 && threadIdx.x < tail)
        dst_tail[threadIdx.x] = src_tail[threadIdx.x];
}

template <class Word>
static void launch_pull(Context &ctx, void *dst, const void *src, size_t bytes, cudaStream_t s)
{
    const size_t words = bytes / sizeof(Word);
    const uint32_t tail = (uint32_t)(bytes % sizeof(Word));
    // A quarter as many blocks as SMs keep about 1.2 MB of 16-byte loads in
    // flight and leave the other SM slots to the compute kernels running beside
    // the copy.  On GB300, a Helios and a Selene call of 2^20 points from two
    // threads took per pair: 6.99 ms with 152 blocks of four loads, 6.30 with
    // 76, 6.08 with 38; 6.06 with 38 blocks of eight loads, 6.25 with 19 and
    // 6.72 with 9 (fewer SMs do not fill the link); 5.90 from pinned buffers by
    // the copy engine, and 6.70 from pageable ones by the copy engine.
    const size_t per_block = 256 * PULL_DEPTH;
    const unsigned blocks = (unsigned)std::max<size_t>(
        1, std::min<size_t>((size_t)std::max(1, ctx.sm_count / PULL_BLOCK_DIV), (words + per_block - 1) / per_block));
    k_pull<Word><<<blocks, 256, 0, s>>>(static_cast<const Word *>(src), static_cast<Word *>(dst), words,
                                        static_cast<const uint8_t *>(src) + words * sizeof(Word),
                                        static_cast<uint8_t *>(dst) + words * sizeof(Word), tail);
    ctx.launches++;
}

// true when p is ordinary pageable host memory (not pinned, registered, managed
// or device); a pointer the runtime cannot classify keeps the copy engine
static bool is_pageable(const void *p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeUnregistered;
}

// A block copies one piece of a gathered copy in `Word`s, then the ragged tail
template <class Word>
__device__ __forceinline__ void pull_piece(const uint8_t *__restrict__ src, uint8_t *__restrict__ dst, size_t bytes)
{
    const size_t words = bytes / sizeof(Word);
    const Word *s = reinterpret_cast<const Word *>(src);
    Word *d = reinterpret_cast<Word *>(dst);
    const size_t T = blockDim.x;
    size_t i = threadIdx.x;
    for (; i + (PULL_DEPTH - 1) * T < words; i += PULL_DEPTH * T) {
        Word v[PULL_DEPTH];
#pragma unroll
        for (int k = 0; k < PULL_DEPTH; k++)
            v[k] = s[i + k * T];
#pragma unroll
        for (int k = 0; k < PULL_DEPTH; k++)
            d[i + k * T] = v[k];
    }
    for (; i < words; i += T)
        d[i] = s[i];
    const size_t done = words * sizeof(Word);
    if (threadIdx.x < bytes - done)
        dst[done + threadIdx.x] = src[done + threadIdx.x];
}

// the pieces of a gathered copy, one block per piece at a time; the list and
// the sources are read where they lie in host memory
__global__ void __launch_bounds__(256) k_pull_list(const PullChunk *__restrict__ list, uint32_t count)
{
    for (uint32_t c = blockIdx.x; c < count; c += gridDim.x) {
        const PullChunk ch = list[c];
        const uintptr_t al = reinterpret_cast<uintptr_t>(ch.src) | reinterpret_cast<uintptr_t>(ch.dst);
        if (al % 16 == 0)
            pull_piece<uint4>(ch.src, ch.dst, ch.bytes);
        else if (al % 8 == 0)
            pull_piece<uint2>(ch.src, ch.dst, ch.bytes);
        else if (al % 4 == 0)
            pull_piece<uint32_t>(ch.src, ch.dst, ch.bytes);
        else
            pull_piece<uint8_t>(ch.src, ch.dst, ch.bytes);
    }
}

cudaError_t pull_list(Context &ctx, const PullChunk *list, size_t count, cudaStream_t s)
{
    if (!count)
        return cudaSuccess;
    if (count >= 0xffffffffull)
        return cudaErrorInvalidValue;
    const unsigned blocks =
        (unsigned)std::max<size_t>(1, std::min<size_t>((size_t)std::max(1, ctx.sm_count / PULL_BLOCK_DIV), count));
    k_pull_list<<<blocks, 256, 0, s>>>(list, (uint32_t)count);
    ctx.launches++;
    return cudaGetLastError();
}

// drains a stream on scope exit unless cleared
struct LinkDrain {
    cudaStream_t s;
    ~LinkDrain()
    {
        if (s)
            cudaStreamSynchronize(s);
    }
};

static cudaError_t h2d_async(Context &ctx, void *dst, const void *src, size_t bytes, cudaStream_t s)
{
    if (!bytes)
        return cudaSuccess;
    if (!ctx.pageable_access || !is_pageable(src))
        return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s);
    touch_host_range(src, bytes);
    const uintptr_t al = reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src);
    if (al % 16 == 0)
        launch_pull<uint4>(ctx, dst, src, bytes, s);
    else if (al % 8 == 0)
        launch_pull<uint2>(ctx, dst, src, bytes, s);
    else if (al % 4 == 0)
        launch_pull<uint32_t>(ctx, dst, src, bytes, s);
    else
        launch_pull<uint8_t>(ctx, dst, src, bytes, s);
    return cudaGetLastError();
}

struct SplitPlan {
    BatchPlan hi, lo;
};

static SplitPlan make_split(const Context &ctx, int curve, size_t n, int base_rounds = -1)
{
    const int c = choose_window(ctx, curve, n);
    const uint32_t W = (uint32_t)((257 + c - 1) / c);
    const uint32_t h = W / 2;
    SplitPlan sp{make_window_plan(curve, n, c, h, W - h), make_window_plan(curve, n, c, 0, h)};
    const int k = curve == HS_SELENE;
    const uint32_t rounds = base_rounds >= 0 ? (uint32_t)base_rounds : ctx.ba_rounds[k];
    plan_batch_affine(sp.hi, rounds, ctx.ba_min_entries[k]);
    plan_batch_affine(sp.lo, rounds, ctx.ba_min_entries[k]);
    return sp;
}

static size_t split_bytes(const SplitPlan &s) { return batch_bytes(s.hi) + batch_bytes(s.lo) + 2048; }

static cudaError_t launch_split(Context &ctx, const SplitPlan &s, const BatchBuffers &bh, const BatchBuffers &bl,
                                uint32_t *d_final, void *d_out, int out_fmt)
{
    const CurveOps &ops = curve_ops(s.hi.curve);
    cudaStream_t a = ctx.stream, b = ctx.stream2;
    cudaError_t e;
    if ((e = cudaEventRecord(ctx.ev_fork, a)) != cudaSuccess || (e = cudaStreamWaitEvent(b, ctx.ev_fork, 0)) != cudaSuccess)
        return e;
    ctx.stream = b;  // upper half on the high-priority stream
    e = launch_sort(ctx, s.hi, bh);
    if (e == cudaSuccess)
        e = ops.msm_tail(ctx, s.hi, bh);
    ctx.stream = a;
    if (e != cudaSuccess)
        return e;
    if ((e = launch_sort(ctx, s.lo, bl)) != cudaSuccess || (e = ops.msm_tail(ctx, s.lo, bl)) != cudaSuccess)
        return e;
    if ((e = cudaEventRecord(ctx.ev_join, b)) != cudaSuccess || (e = cudaStreamWaitEvent(a, ctx.ev_join, 0)) != cudaSuccess)
        return e;
    if ((e = ops.join(ctx, bh.out_jac, bl.out_jac, 1, d_final)) != cudaSuccess)
        return e;
    return ops.format_out(ctx, d_final, 1, out_fmt, d_out);
}

// buffers: both halves carved after one reservation made by the caller
static int execute_split(Context &ctx, const SplitPlan &s, const void *d_scalars, const void *d_points, void *d_out,
                         int out_fmt)
{
    HS_CU(ensure_stream2(ctx), "stream creation");
    BatchBuffers bh, bl;
    if (!carve(ctx.arena, s.hi, bh) || !carve(ctx.arena, s.lo, bl))
        return fail_msg(ctx, HS_ENOMEM, "workspace carve");
    uint32_t *d_final = (uint32_t *)ctx.arena.take(96);
    if (!d_final)
        return fail_msg(ctx, HS_ENOMEM, "workspace carve");
    bh.scalars = bl.scalars = static_cast<const uint32_t *>(d_scalars);
    bh.points = bl.points = static_cast<const uint4 *>(d_points);
    cudaStream_t st = ctx.stream;
    if (!ctx.use_graphs || ctx.profile) {
        HS_CU(cudaMemcpyAsync(bh.desc, s.hi.msms.data(), sizeof(MsmDesc), cudaMemcpyHostToDevice, st), "descriptors");
        HS_CU(cudaMemcpyAsync(bl.desc, s.lo.msms.data(), sizeof(MsmDesc), cudaMemcpyHostToDevice, st), "descriptors");
        HS_CU(launch_split(ctx, s, bh, bl, d_final, d_out, out_fmt), "split MSM launch");
        return HS_OK;
    }
    std::vector<uint64_t> key = {0x5350u, (uint64_t)s.hi.curve, (uint64_t)s.hi.msms[0].n, (uint64_t)s.hi.msms[0].c,
                                 (uint64_t)out_fmt, (uint64_t)(uintptr_t)ctx.arena.base, (uint64_t)ctx.arena.cap,
                                 (uint64_t)(uintptr_t)bh.counts, (uint64_t)(uintptr_t)d_scalars,
                                 (uint64_t)(uintptr_t)d_points, (uint64_t)(uintptr_t)d_out, (uint64_t)(uintptr_t)st,
                                 (uint64_t)s.hi.ba_rounds, (uint64_t)s.lo.ba_rounds};
    for (GraphEntry &g : ctx.graphs) {
        if (g.key == key) {
            HS_CU(cudaGraphLaunch(g.exec, st), "graph launch");
            ctx.launches += g.kernels;
            return HS_OK;
        }
    }
    GraphEntry ent;
    HS_CU(cudaMalloc(&ent.d_desc, 2 * sizeof(MsmDesc)), "descriptor allocation");
    const MsmDesc both[2] = {s.hi.msms[0], s.lo.msms[0]};
    cudaError_t ue = cudaMemcpy(ent.d_desc, both, sizeof(both), cudaMemcpyHostToDevice);
    if (ue != cudaSuccess) {
        cudaFree(ent.d_desc);
        return fail(ctx, ue, "descriptor upload");
    }
    bh.desc = (MsmDesc *)ent.d_desc;
    bl.desc = (MsmDesc *)ent.d_desc + 1;
    cudaGraph_t graph = nullptr;
    const uint64_t before = ctx.launches;
    cudaError_t ce = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
    cudaError_t le = ce == cudaSuccess ? launch_split(ctx, s, bh, bl, d_final, d_out, out_fmt) : ce;
    if (ce == cudaSuccess)
        ce = cudaStreamEndCapture(st, &graph);
    if (le != cudaSuccess || ce != cudaSuccess) {
        if (graph)
            cudaGraphDestroy(graph);
        cudaFree(ent.d_desc);
        return fail(ctx, le != cudaSuccess ? le : ce, "graph capture");
    }
    cudaGraphExec_t exec = nullptr;
    // the captured stream priorities stay on the kernel nodes: the upper half is scheduled first
    cudaError_t ie = cudaGraphInstantiateWithFlags(&exec, graph, cudaGraphInstantiateFlagUseNodePriority);
    cudaGraphDestroy(graph);
    if (ie != cudaSuccess) {
        cudaFree(ent.d_desc);
        return fail(ctx, ie, "graph instantiate");
    }
    ent.key = std::move(key);
    ent.exec = exec;
    ent.kernels = ctx.launches - before;
    if (ctx.graphs.size() >= 64) {
        cudaStreamSynchronize(st);
        cudaGraphExecDestroy(ctx.graphs.front().exec);
        cudaFree(ctx.graphs.front().d_desc);
        ctx.graphs.erase(ctx.graphs.begin());
    }
    ctx.graphs.push_back(std::move(ent));
    HS_CU(cudaGraphLaunch(exec, st), "graph launch");
    return HS_OK;
}

void drop_graphs(Context &ctx)
{
    if (!ctx.graphs.empty() && ctx.stream)
        cudaStreamSynchronize(ctx.stream);
    for (GraphEntry &g : ctx.graphs) {
        cudaGraphExecDestroy(g.exec);
        cudaFree(g.d_desc);
    }
    ctx.graphs.clear();
}

}  // namespace hs

using namespace hs;

// ===========================================================================
// C ABI
// ===========================================================================
namespace hs {
static thread_local std::string g_tls_error;
void set_thread_error(const std::string &what) { g_tls_error = what; }
}  // namespace hs

extern "C" {

int hs_abi_version(void) { return 1; }

const char *hs_strerror(int s)
{
    switch (s) {
    case HS_OK:
        return "ok";
    case HS_EINVAL:
        return "invalid argument";
    case HS_ENOMEM:
        return "out of memory";
    case HS_ECUDA:
        return "CUDA error";
    case HS_ETIMEDOUT:
        return "timed out";
    case HS_EBUSY:
        return "busy";
    case HS_ERANGE:
        return "size out of range";
    default:
        return "unknown status";
    }
}

int hs_context_create(hs_context **out, int device)
{
    if (!out)
        return HS_EINVAL;
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || device < 0 || device >= count) {
        g_tls_error = std::string("no such CUDA device: ") + (e != cudaSuccess ? cudaGetErrorString(e) : "index");
        cudaGetLastError();
        return e != cudaSuccess ? HS_ECUDA : HS_EINVAL;
    }
    hs_context *h = new (std::nothrow) hs_context();
    if (!h)
        return HS_ENOMEM;
    Context &ctx = h->c;
    ctx.device = device;
    DeviceGuard g(device);
    e = cudaStreamCreateWithFlags(&ctx.stream, cudaStreamNonBlocking);
    if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(&ctx.sm_count, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) {
        int pma = 0;
        e = cudaDeviceGetAttribute(&pma, cudaDevAttrPageableMemoryAccess, device);
        ctx.pageable_access = pma == 1;
    }
    if (e == cudaSuccess)
        e = sort_smem_attrs(device);
    if (e != cudaSuccess) {
        g_tls_error = std::string("context creation: ") + cudaGetErrorString(e);
        cudaGetLastError();
        delete h;
        return HS_ECUDA;
    }
    *out = h;
    return HS_OK;
}

void hs_context_destroy(hs_context *h)
{
    if (!h)
        return;
    {
        DeviceGuard g(h->c.device);
        // every stream that may still use the workspace finishes first
        cudaStreamSynchronize(h->c.stream);
        if (h->c.stream2)
            cudaStreamSynchronize(h->c.stream2);
        if (h->c.stream3)
            cudaStreamSynchronize(h->c.stream3);
        drop_graphs(h->c);
        h->c.arena.release();
        cudaStreamDestroy(h->c.stream);
        if (h->c.stream2)
            cudaStreamDestroy(h->c.stream2);
        if (h->c.ev_fork)
            cudaEventDestroy(h->c.ev_fork);
        if (h->c.ev_join)
            cudaEventDestroy(h->c.ev_join);
        if (h->c.stream3)
            cudaStreamDestroy(h->c.stream3);
        for (cudaEvent_t ev : {h->c.ev_sc, h->c.ev_rec[0], h->c.ev_rec[1], h->c.ev_pts[0], h->c.ev_pts[1]})
            if (ev)
                cudaEventDestroy(ev);
    }
    delete h;
}

const char *hs_last_error(const hs_context *h) { return h ? h->c.last_error.c_str() : g_tls_error.c_str(); }

uint64_t hs_context_launches(const hs_context *h) { return h ? h->c.launches : 0; }

void *hs_context_stream(hs_context *h) { return h ? (void *)h->c.stream : nullptr; }

int hs_context_set_window(hs_context *h, int curve, size_t n_min, size_t n_max, int window)
{
    return hs_context_set_rule(h, curve, n_min, n_max, window, -1);
}

int hs_context_set_rule(hs_context *h, int curve, size_t n_min, size_t n_max, int window, int ba_rounds)
{
    if (!h || !valid_curve(curve) || n_min > n_max || (window != 0 && (window < 4 || window > 20)) ||
        ba_rounds < -1 || ba_rounds > (int)BA_MAX_ROUNDS)
        return HS_EINVAL;
    std::lock_guard<std::mutex> lk(h->c.mu);
    auto &rules = h->c.rules[curve == HS_SELENE ? 1 : 0];
    if (window == 0) {
        rules.clear();
        return HS_OK;
    }
    WindowRule r{n_min, n_max, window};
    r.ba_rounds = ba_rounds;
    rules.push_back(r);
    return HS_OK;
}

int hs_context_set_graphs(hs_context *h, int on)
{
    if (!h)
        return HS_EINVAL;
    std::lock_guard<std::mutex> lk(h->c.mu);
    DeviceGuard g(h->c.device);
    h->c.use_graphs = on != 0;
    if (!on)
        drop_graphs(h->c);
    return HS_OK;
}

int hs_context_set_priority(hs_context *h, int high)
{
    if (!h)
        return HS_EINVAL;
    Context &ctx = h->c;
    std::lock_guard<std::mutex> lk(ctx.mu);
    DeviceGuard g(ctx.device);
    int least = 0, greatest = 0;
    HS_CU(cudaDeviceGetStreamPriorityRange(&least, &greatest), "stream priorities");
    cudaStream_t s = nullptr;
    HS_CU(cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, high ? greatest : least), "stream creation");
    HS_CU(cudaStreamSynchronize(ctx.stream), "stream drain");
    drop_graphs(ctx);  // captured sequences are keyed by the stream they were captured on
    cudaStreamDestroy(ctx.stream);
    ctx.stream = s;
    return HS_OK;
}

int hs_context_set_split(hs_context *h, size_t min_points)
{
    if (!h)
        return HS_EINVAL;
    std::lock_guard<std::mutex> lk(h->c.mu);
    h->c.split_min = min_points;
    return HS_OK;
}

int hs_context_set_batch_affine(hs_context *h, int curve, int rounds, size_t min_entries)
{
    if (!h || !valid_curve(curve) || rounds < -1 || rounds > (int)BA_MAX_ROUNDS)
        return HS_EINVAL;
    Context &ctx = h->c;
    std::lock_guard<std::mutex> lk(ctx.mu);
    DeviceGuard g(ctx.device);
    drop_graphs(ctx);
    const int k = curve == HS_SELENE;
    if (rounds < 0) {  // the library's defaults
        ctx.ba_rounds[k] = BA_DEFAULT_ROUNDS[k];
        ctx.ba_min_entries[k] = BA_DEFAULT_MIN_ENTRIES;
        ctx.ba_set[k] = false;
        return HS_OK;
    }
    ctx.ba_rounds[k] = (uint32_t)rounds;
    ctx.ba_min_entries[k] = min_entries;
    ctx.ba_set[k] = true;
    return HS_OK;
}

// one launch sequence indexes its (point, window) entries with 31 bits
static bool entries_fit(const Context &ctx, int curve, size_t n)
{
    const int c = choose_window(ctx, curve, n);
    return (uint64_t)n * (uint64_t)((257 + c - 1) / c) < 0x80000000ull;
}

int hs_msm_device(hs_context *h, int curve, const void *d_scalars, const void *d_points, size_t n, void *d_out,
                  int out_fmt)
{
    if (!h || !valid_curve(curve) || !valid_out_fmt(out_fmt) || !d_out || (n && (!d_scalars || !d_points)))
        return HS_EINVAL;
    if (n >= 0x80000000ull)
        return HS_ERANGE;
    Context &ctx = h->c;
    std::lock_guard<std::mutex> lk(ctx.mu);
    if (!entries_fit(ctx, curve, n))
        return fail_msg(ctx, HS_ERANGE, "n x windows exceeds one launch sequence: sum partial MSMs of smaller slices");
    DeviceGuard g(ctx.device);
    if (n == 0) {
        unsigned char idb[128];
        identity_out(curve, out_fmt, idb);
        HS_CU(cudaMemcpyAsync(d_out, idb, fmt_bytes(out_fmt), cudaMemcpyHostToDevice, ctx.stream), "copy");
        HS_CU(cudaStreamSynchronize(ctx.stream), "sync");
        return HS_OK;
    }
    if (ctx.split_min && n >= ctx.split_min) {
        const SplitPlan s = make_split(ctx, curve, n);
        HS_CU(ctx.arena.reserve(split_bytes(s)), "workspace allocation");
        return execute_split(ctx, s, d_scalars, d_points, d_out, out_fmt);
    }
    const size_t sizes[1] = {n};
    const BatchPlan p = make_batch_plan(ctx, curve, sizes, 1);
    BatchBuffers b;
    int rc = reserve_batch(ctx, p, 0, b, nullptr);
    if (rc != HS_OK)
        return rc;
    b.scalars = static_cast<const uint32_t *>(d_scalars);
    b.points = static_cast<const uint4 *>(d_points);
    return execute_batch(ctx, p, b, d_out, out_fmt);
}

// Host inputs in two parts split at counting-sort slice `slice`: each bucket
// may get one more segment descriptor (its part-1 entries).
static void plan_parts(BatchPlan &p, uint32_t slice)
{
    p.part_slice = slice;
    if (p.ba_rounds) {
        // each part's list of a bucket padded apart: up to NB (2^R - 1) more
        // padding entries; the last round's 2 NB lists cut into segments of L
        const uint64_t padded = (uint64_t)p.max_entries + (uint64_t)p.NB * ((1u << p.ba_rounds) - 1);
        p.max_entries = (uint32_t)padded;
        const uint64_t per_block = (uint64_t)BA_PLAN_K * BA_PLAN_BT;
        for (uint32_t r = 1; r <= p.ba_rounds; r++) {
            p.ba_items[r - 1] = (padded >> r) + 1;
            p.ba_blocks[r - 1] = (uint32_t)((p.ba_items[r - 1] + per_block - 1) / per_block);
        }
        const uint64_t ent = p.ba_items[p.ba_rounds - 1];
        p.max_segs = (uint32_t)std::min<uint64_t>(0xffffffffull, std::min<uint64_t>(ent, 2ull * p.NB) + ent / p.L + 1);
        return;
    }
    const uint64_t more = std::min<uint64_t>(p.entries_bound, p.NB);
    p.max_segs = (uint32_t)std::min<uint64_t>(0xffffffffull, (uint64_t)p.max_segs + more);
}

// Stage host inputs (scalars and points in any format) and run one MSM of
// n_total terms whose first `lead` terms come from (lead_scalar, lead_point).
static int msm_host(Context &ctx, int curve, const uint8_t *lead_scalar, const void *lead_point, const uint8_t *scalars,
                    const void *points, int point_fmt, size_t n, void *out, int out_fmt)
{
    const size_t lead = lead_scalar ? 1 : 0;
    const size_t total = n + lead;
    if (total == 0) {
        identity_out(curve, out_fmt, out);
        return HS_OK;
    }
    if (total >= 0x80000000ull || !entries_fit(ctx, curve, total))
        return fail_msg(ctx, HS_ERANGE, "n x windows exceeds one launch sequence: sum partial MSMs of smaller slices");
    DeviceGuard g(ctx.device);
    const size_t pb = fmt_bytes(point_fmt);
    const CurveOps &ops = curve_ops(curve);
    const bool split = ctx.split_min && total >= ctx.split_min;
    const int k = curve == HS_SELENE;
    const int base_rounds = ctx.ba_set[k] ? -1 : (int)ctx.host_ba_rounds[k];
    SplitPlan s;
    BatchPlan p;
    if (split)
        s = make_split(ctx, curve, total, base_rounds);
    else {
        const size_t sizes[1] = {total};
        p = make_batch_plan(ctx, curve, sizes, 1, base_rounds);
    }
    // Bases spanning several counting-sort slices arrive in two parts, split at a
    // slice boundary: the entries of a bucket come in slice order, so each part's
    // entries of a bucket are contiguous and get their own segments, and the
    // accumulation of part 0 runs while part 1 is still on the link.
    const MsmDesc &d0 = split ? s.lo.msms[0] : p.msms[0];
    // (a batch-affine plan gives each part's entries of a bucket their own list,
    // so that each part's rounds pair only entries that have arrived)
    const auto padded_fits = [](const BatchPlan &q) {
        return !q.ba_rounds || (uint64_t)q.max_entries + (uint64_t)q.NB * ((1u << q.ba_rounds) - 1) < 0x80000000ull;
    };
    const bool two = point_fmt != HS_FMT_COMPRESSED && d0.slices >= 2 &&
                     (split ? (s.hi.smem_sort() && s.lo.smem_sort() && padded_fits(s.hi) && padded_fits(s.lo))
                            : (p.smem_sort() && padded_fits(p)));
    size_t bound[3] = {0, total, total};
    if (two) {
        const uint32_t cut = d0.slices / 2;
        if (split) {
            plan_parts(s.hi, cut);
            plan_parts(s.lo, cut);
        } else {
            plan_parts(p, cut);
        }
        bound[1] = std::min<size_t>(total, (size_t)((total + d0.slices - 1) / d0.slices) * cut);
    }
    const int nparts = two ? 2 : 1;
    const size_t need_in = align256(total * 32) + align256(total * 64) +
                           (point_fmt == HS_FMT_AFFINE ? 0 : align256(total * pb)) +
                           align256(ops.to_affine_scratch(total)) + 256;
    HS_CU(ctx.arena.reserve(need_in + (split ? split_bytes(s) : batch_bytes(p)) + 2048), "workspace allocation");
    uint8_t *d_sc = (uint8_t *)ctx.arena.take(need_in);
    if (!d_sc)
        return fail_msg(ctx, HS_ENOMEM, "workspace carve");
    uint8_t *d_pts = d_sc + align256(total * 32);
    uint8_t *d_raw = point_fmt == HS_FMT_AFFINE ? d_pts : d_pts + align256(total * 64);
    uint8_t *d_scratch = (point_fmt == HS_FMT_AFFINE ? d_pts + align256(total * 64) : d_raw + align256(total * pb));
    uint8_t *d_out = d_scratch + align256(ops.to_affine_scratch(total));
    // Inputs go to the device's link stream, the scalars first: the counting
    // sort needs only them, so it runs while the bases arrive; each part of the
    // bases is converted on the third stream as soon as it is in, and each
    // accumulation launch waits for its part.
    HS_CU(ensure_stream2(ctx), "stream creation");
    LinkStream *link = nullptr;
    HS_CU(link_stream(ctx.device, &link), "stream creation");
    cudaStream_t st = ctx.stream, s2 = ctx.stream2, s3 = ctx.stream3;
    // a copy kernel may still be reading the caller's pages when the call fails
    // part way: the link stream drains before such a return
    LinkDrain drain{link->s};
    HS_CU(cudaEventRecord(ctx.ev_fork, st), "event");  // earlier work on the buffers comes first
    {
        std::lock_guard<std::mutex> lk(link->mu);
        cudaStream_t cs = link->s;
        HS_CU(cudaStreamWaitEvent(cs, ctx.ev_fork, 0), "stream wait");
        if (lead)
            HS_CU(h2d_async(ctx, d_sc, lead_scalar, 32, cs), "H2D scalars");
        if (n)
            HS_CU(h2d_async(ctx, d_sc + 32 * lead, scalars, n * 32, cs), "H2D scalars");
        HS_CU(cudaEventRecord(ctx.ev_sc, cs), "event");
        for (int j = 0; j < nparts; j++) {
            // point g of the MSM: the lead term at 0, then points[g - lead]
            size_t g = bound[j];
            if (lead && g == 0 && bound[j + 1] > 0) {
                HS_CU(h2d_async(ctx, d_raw, lead_point, pb, cs), "H2D points");
                g = 1;
            }
            if (bound[j + 1] > g)
                HS_CU(h2d_async(ctx, d_raw + pb * g, static_cast<const uint8_t *>(points) + pb * (g - lead),
                                pb * (bound[j + 1] - g), cs),
                      "H2D points");
            HS_CU(cudaEventRecord(ctx.ev_rec[j], cs), "event");
        }
    }
    cudaEvent_t ready[2] = {nullptr, nullptr};
    for (int j = 0; j < nparts; j++) {
        ready[j] = ctx.ev_rec[j];
        if (point_fmt == HS_FMT_AFFINE)  // copied in place, nothing to convert
            continue;
        HS_CU(cudaStreamWaitEvent(s3, ctx.ev_rec[j], 0), "stream wait");
        ctx.stream = s3;
        const cudaError_t ce = ops.to_affine(ctx, d_raw + pb * bound[j], point_fmt, bound[j + 1] - bound[j],
                                             (uint4 *)d_pts + 4 * bound[j], d_scratch);
        ctx.stream = st;
        HS_CU(ce, "input conversion");
        HS_CU(cudaEventRecord(ctx.ev_pts[j], s3), "event");
        ready[j] = ctx.ev_pts[j];
    }
    // The device work of the call -- sorts, accumulations, reductions, combine,
    // join and output format -- is one captured launch sequence per call shape,
    // replayed: a call then costs its copies, the input conversion and one graph
    // launch instead of dozens of kernel launches.  Its waits on the input events
    // (recorded above, outside the sequence) are external event waits.
    BatchBuffers bh, bl, b;
    uint32_t *d_final = nullptr;
    if (split) {
        if (!carve(ctx.arena, s.hi, bh) || !carve(ctx.arena, s.lo, bl) || !(d_final = (uint32_t *)ctx.arena.take(96)))
            return fail_msg(ctx, HS_ENOMEM, "workspace carve");
        bh.scalars = bl.scalars = (const uint32_t *)d_sc;
        bh.points = bl.points = (const uint4 *)d_pts;
        for (int j = 0; j < 2; j++)
            bh.ready[j] = bl.ready[j] = ready[j];
    } else {
        if (!carve(ctx.arena, p, b))
            return fail_msg(ctx, HS_ENOMEM, "workspace carve");
        b.scalars = (const uint32_t *)d_sc;
        b.points = (const uint4 *)d_pts;
        b.ready[0] = ready[0];
        b.ready[1] = ready[1];
    }
    auto device_work = [&](MsmDesc *desc_hi, MsmDesc *desc_lo) -> cudaError_t {
        cudaError_t e;
        const unsigned wflags = ctx.capturing_host ? cudaEventWaitExternal : 0;
        if ((e = cudaStreamWaitEvent(st, ctx.ev_sc, wflags)) != cudaSuccess)
            return e;
        if (split) {
            BatchBuffers h = bh, l = bl;
            h.desc = desc_hi;
            l.desc = desc_lo;
            if ((e = launch_sort(ctx, s.hi, h)) != cudaSuccess || (e = launch_sort(ctx, s.lo, l)) != cudaSuccess)
                return e;
            // upper half on the second stream once both sorts are in (the accumulations
            // wait for the bases)
            if ((e = cudaEventRecord(ctx.ev_fork, st)) != cudaSuccess ||
                (e = cudaStreamWaitEvent(s2, ctx.ev_fork, 0)) != cudaSuccess)
                return e;
            ctx.stream = s2;
            e = ops.msm_tail(ctx, s.hi, h);
            ctx.stream = st;
            if (e != cudaSuccess)
                return e;
            if ((e = cudaEventRecord(ctx.ev_join, s2)) != cudaSuccess || (e = ops.msm_tail(ctx, s.lo, l)) != cudaSuccess ||
                (e = cudaStreamWaitEvent(st, ctx.ev_join, 0)) != cudaSuccess)
                return e;
            if ((e = ops.join(ctx, h.out_jac, l.out_jac, 1, d_final)) != cudaSuccess)
                return e;
            return ops.format_out(ctx, d_final, 1, out_fmt, d_out);
        }
        BatchBuffers one = b;
        one.desc = desc_hi;
        if ((e = launch_sort(ctx, p, one)) != cudaSuccess || (e = ops.msm_tail(ctx, p, one)) != cudaSuccess)
            return e;
        return ops.format_out(ctx, one.out_jac, 1, out_fmt, d_out);
    };
    if (!ctx.use_graphs || ctx.profile) {
        if (split) {
            HS_CU(cudaMemcpyAsync(bh.desc, s.hi.msms.data(), sizeof(MsmDesc), cudaMemcpyHostToDevice, st), "descriptors");
            HS_CU(cudaMemcpyAsync(bl.desc, s.lo.msms.data(), sizeof(MsmDesc), cudaMemcpyHostToDevice, st), "descriptors");
            HS_CU(device_work(bh.desc, bl.desc), "MSM launch");
        } else {
            HS_CU(cudaMemcpyAsync(b.desc, p.msms.data(), sizeof(MsmDesc), cudaMemcpyHostToDevice, st), "descriptors");
            HS_CU(device_work(b.desc, nullptr), "MSM launch");
        }
    } else {
        const BatchPlan &p0 = split ? s.hi : p;
        std::vector<uint64_t> key = {0x484f5354u, (uint64_t)curve, (uint64_t)total, (uint64_t)out_fmt,
                                     (uint64_t)split, (uint64_t)nparts, (uint64_t)bound[1], (uint64_t)p0.msms[0].c,
                                     (uint64_t)p0.ba_rounds, (uint64_t)(split ? s.lo.ba_rounds : 0),
                                     (uint64_t)(uintptr_t)ctx.arena.base, (uint64_t)ctx.arena.cap,
                                     (uint64_t)(uintptr_t)d_sc, (uint64_t)(uintptr_t)d_out, (uint64_t)(uintptr_t)st,
                                     (uint64_t)(uintptr_t)s2, (uint64_t)(uintptr_t)ready[0],
                                     (uint64_t)(uintptr_t)ready[1]};
        GraphEntry *hit = nullptr;
        for (GraphEntry &g : ctx.graphs)
            if (g.key == key)
                hit = &g;
        if (!hit) {
            // descriptors in a buffer owned by the graph, uploaded once here
            GraphEntry ent;
            HS_CU(cudaMalloc(&ent.d_desc, 2 * sizeof(MsmDesc)), "descriptor allocation");
            const MsmDesc both[2] = {p0.msms[0], split ? s.lo.msms[0] : p0.msms[0]};
            cudaError_t ue = cudaMemcpy(ent.d_desc, both, sizeof(both), cudaMemcpyHostToDevice);
            if (ue != cudaSuccess) {
                cudaFree(ent.d_desc);
                return fail(ctx, ue, "descriptor upload");
            }
            cudaGraph_t graph = nullptr;
            const uint64_t before = ctx.launches;
            cudaError_t ce = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
            ctx.capturing_host = true;
            cudaError_t le = ce == cudaSuccess ? device_work((MsmDesc *)ent.d_desc, (MsmDesc *)ent.d_desc + 1) : ce;
            ctx.capturing_host = false;
            if (ce == cudaSuccess)
                ce = cudaStreamEndCapture(st, &graph);
            cudaGraphExec_t exec = nullptr;
            cudaError_t ie = (le == cudaSuccess && ce == cudaSuccess)
                                 ? cudaGraphInstantiateWithFlags(&exec, graph, cudaGraphInstantiateFlagUseNodePriority)
                                 : cudaSuccess;
            if (graph)
                cudaGraphDestroy(graph);
            if (le != cudaSuccess || ce != cudaSuccess || ie != cudaSuccess) {
                cudaFree(ent.d_desc);
                return fail(ctx, le != cudaSuccess ? le : (ce != cudaSuccess ? ce : ie), "graph capture");
            }
            ent.key = std::move(key);
            ent.exec = exec;
            ent.kernels = ctx.launches - before;
            if (ctx.graphs.size() >= 64) {
                cudaStreamSynchronize(st);
                cudaGraphExecDestroy(ctx.graphs.front().exec);
                cudaFree(ctx.graphs.front().d_desc);
                ctx.graphs.erase(ctx.graphs.begin());
            }
            ctx.graphs.push_back(std::move(ent));
            hit = &ctx.graphs.back();
            ctx.launches = before;  // counted again at the launch below
        }
        HS_CU(cudaGraphLaunch(hit->exec, st), "graph launch");
        ctx.launches += hit->kernels;
    }
    HS_CU(cudaMemcpyAsync(out, d_out, fmt_bytes(out_fmt), cudaMemcpyDeviceToHost, st), "D2H result");
    HS_CU(cudaStreamSynchronize(st), "MSM");
    drain.s = nullptr;  // the launch sequence waited for every input copy
    if (point_fmt == HS_FMT_COMPRESSED)
        return check_decoded(ctx, d_scratch);
    return HS_OK;
}

int hs_msm(hs_context *h, int curve, const uint8_t *scalars, const void *points, int point_fmt, size_t n, void *out,
           int out_fmt)
{
    if (!h || !valid_curve(curve) || !valid_pt_fmt(point_fmt) || !valid_out_fmt(out_fmt) || !out ||
        (n && (!scalars || !points)))
        return HS_EINVAL;
    Context &ctx = h->c;
    std::lock_guard<std::mutex> lk(ctx.mu);
    return msm_host(ctx, curve, nullptr, nullptr, scalars, points, point_fmt, n, out, out_fmt);
}

int hs_pedersen(hs_context *h, int curve, const uint8_t blinding[32], const void *H, const uint8_t *values,
                const void *generators, int point_fmt, size_t n, void *out, int out_fmt)
{
    if (!h || !valid_curve(curve) || !valid_pt_fmt(point_fmt) || !valid_out_fmt(out_fmt) || !out || !blinding ||
        !H || (n && (!values || !generators)))
        return HS_EINVAL;
    Context &ctx = h->c;
    std::lock_guard<std::mutex> lk(ctx.mu);
    return msm_host(ctx, curve, blinding, H, values, generators, point_fmt, n, out, out_fmt);
}

int hs_batch_to_affine(hs_context *h, int curve, const void *in, size_t n, void *out, int out_fmt)
{
    if (!h || !valid_curve(curve) || (out_fmt != HS_FMT_AFFINE && out_fmt != HS_FMT_AFFINE51) ||
        (n && (!in || !out)))
        return HS_EINVAL;
    if (n == 0)
        return HS_OK;
    Context &ctx = h->c;
    std::lock_guard<std::mutex> lk(ctx.mu);
    DeviceGuard g(ctx.device);
    const CurveOps &ops = curve_ops(curve);
    HS_CU(ctx.arena.reserve(align256(n * 120) + align256(n * 64) + align256(ops.to_affine_scratch(n)) +
                            align256(n * 80) + 1024),
          "workspace allocation");
    void *d_in = ctx.arena.take(n * 120);
    uint4 *d_aff = (uint4 *)ctx.arena.take(n * 64);
    void *d_scr = ctx.arena.take(ops.to_affine_scratch(n));
    void *d_o51 = ctx.arena.take(n * 80);
    cudaStream_t st = ctx.stream;
    HS_CU(cudaMemcpyAsync(d_in, in, n * 120, cudaMemcpyHostToDevice, st), "H2D");
    HS_CU(ops.to_affine(ctx, d_in, HS_FMT_JACOBIAN51, n, d_aff, d_scr), "batch to affine");
    if (out_fmt == HS_FMT_AFFINE) {
        HS_CU(cudaMemcpyAsync(out, d_aff, n * 64, cudaMemcpyDeviceToHost, st), "D2H");
    } else {
        // affine -> canonical Jacobian with Z = 1 -> radix-2^51 (x, y) pairs
        uint32_t *d_j = (uint32_t *)d_in;  // n*120 bytes >= n*96
        HS_CU(ops.to_jac24(ctx, d_aff, HS_FMT_AFFINE, n, d_j), "affine pack");
        HS_CU(ops.format_out(ctx, d_j, n, HS_FMT_AFFINE51, d_o51), "affine pack");
        HS_CU(cudaMemcpyAsync(out, d_o51, n * 80, cudaMemcpyDeviceToHost, st), "D2H");
    }
    HS_CU(cudaStreamSynchronize(st), "batch to affine");
    return HS_OK;
}

int hs_compress(hs_context *h, int curve, const void *in, int in_fmt, size_t n, uint8_t *out)
{
    if (!h || !valid_curve(curve) || !valid_in_fmt(in_fmt) || (n && (!in || !out)))
        return HS_EINVAL;
    if (n == 0)
        return HS_OK;
    Context &ctx = h->c;
    std::lock_guard<std::mutex> lk(ctx.mu);
    DeviceGuard g(ctx.device);
    const CurveOps &ops = curve_ops(curve);
    const size_t pb = fmt_bytes(in_fmt);
    HS_CU(ctx.arena.reserve(align256(n * pb) + align256(n * 96) + align256(n * 32) + 1024), "workspace allocation");
    void *d_in = ctx.arena.take(n * pb);
    uint32_t *d_j = (uint32_t *)ctx.arena.take(n * 96);
    void *d_o = ctx.arena.take(n * 32);
    cudaStream_t st = ctx.stream;
    HS_CU(cudaMemcpyAsync(d_in, in, n * pb, cudaMemcpyHostToDevice, st), "H2D");
    HS_CU(ops.to_jac24(ctx, d_in, in_fmt, n, d_j), "unpack");
    HS_CU(ops.format_out(ctx, d_j, n, HS_FMT_COMPRESSED, d_o), "compress");
    HS_CU(cudaMemcpyAsync(out, d_o, n * 32, cudaMemcpyDeviceToHost, st), "D2H");
    HS_CU(cudaStreamSynchronize(st), "compress");
    return HS_OK;
}

int hs_decompress(hs_context *h, int curve, const uint8_t *in, size_t n, void *out, int out_fmt, uint8_t *valid)
{
    if (!h || !valid_curve(curve) || (n && (!in || !out)) ||
        (out_fmt != HS_FMT_AFFINE && out_fmt != HS_FMT_AFFINE51 && out_fmt != HS_FMT_JACOBIAN51))
        return HS_EINVAL;
    if (n == 0)
        return HS_OK;
    Context &ctx = h->c;
    std::lock_guard<std::mutex> lk(ctx.mu);
    DeviceGuard g(ctx.device);
    const CurveOps &ops = curve_ops(curve);
    const size_t ob = fmt_bytes(out_fmt);
    HS_CU(ctx.arena.reserve(align256(n * 32) + align256(n * 64) + align256(n * 96) + align256(n * ob) + align256(n) +
                            2048),
          "workspace allocation");
    uint8_t *d_in = (uint8_t *)ctx.arena.take(n * 32);
    uint4 *d_aff = (uint4 *)ctx.arena.take(n * 64);
    uint32_t *d_j = (uint32_t *)ctx.arena.take(n * 96);
    uint8_t *d_o = (uint8_t *)ctx.arena.take(n * ob);
    uint8_t *d_valid = (uint8_t *)ctx.arena.take(n);
    uint32_t *d_bad = (uint32_t *)ctx.arena.take(256);
    if (!d_in || !d_aff || !d_j || !d_o || !d_valid || !d_bad)
        return fail_msg(ctx, HS_ENOMEM, "workspace carve");
    cudaStream_t st = ctx.stream;
    HS_CU(cudaMemcpyAsync(d_in, in, n * 32, cudaMemcpyHostToDevice, st), "H2D");
    HS_CU(cudaMemsetAsync(d_bad, 0, sizeof(uint32_t), st), "memset");
    HS_CU(ops.decompress(ctx, d_in, n, d_aff, d_valid, d_bad), "decompress");
    const void *src = d_aff;
    if (out_fmt != HS_FMT_AFFINE) {
        // canonical Jacobian with Z = 1 (identity for invalid entries), then the radix-2^51 record
        HS_CU(ops.to_jac24(ctx, d_aff, HS_FMT_AFFINE, n, d_j), "decompress");
        HS_CU(ops.format_out(ctx, d_j, n, out_fmt, d_o), "decompress");
        src = d_o;
    }
    HS_CU(cudaMemcpyAsync(out, src, n * ob, cudaMemcpyDeviceToHost, st), "D2H");
    if (valid)
        HS_CU(cudaMemcpyAsync(valid, d_valid, n, cudaMemcpyDeviceToHost, st), "D2H");
    uint32_t bad = 0;
    HS_CU(cudaMemcpyAsync(&bad, d_bad, sizeof(bad), cudaMemcpyDeviceToHost, st), "D2H");
    HS_CU(cudaStreamSynchronize(st), "decompress");
    if (bad)
        return fail_msg(ctx, HS_EINVAL, "invalid point encoding");
    return HS_OK;
}

int hs_decompress_device(hs_context *h, int curve, const void *d_in, size_t n, void *d_out, uint8_t *d_valid)
{
    if (!h || !valid_curve(curve) || (n && (!d_in || !d_out || !d_valid)))
        return HS_EINVAL;
    if (n == 0)
        return HS_OK;
    Context &ctx = h->c;
    std::lock_guard<std::mutex> lk(ctx.mu);
    DeviceGuard g(ctx.device);
    HS_CU(ctx.arena.reserve(1024), "workspace allocation");
    uint32_t *d_bad = (uint32_t *)ctx.arena.take(256);
    if (!d_bad)
        return fail_msg(ctx, HS_ENOMEM, "workspace carve");
    HS_CU(cudaMemsetAsync(d_bad, 0, sizeof(uint32_t), ctx.stream), "memset");
    HS_CU(curve_ops(curve).decompress(ctx, d_in, n, static_cast<uint4 *>(d_out), d_valid, d_bad), "decompress");
    return HS_OK;
}

int hs_map_to_curve_device(hs_context *h, int curve, const void *d_u, size_t n, void *d_out_affine)
{
    if (!h || !valid_curve(curve) || (n && (!d_u || !d_out_affine)))
        return HS_EINVAL;
    Context &ctx = h->c;
    std::lock_guard<std::mutex> lk(ctx.mu);
    DeviceGuard g(ctx.device);
    HS_CU(curve_ops(curve).map_to_curve(ctx, d_u, n, (uint4 *)d_out_affine), "map to curve");
    return HS_OK;
}

int hs_map_to_curve(hs_context *h, int curve, const uint8_t *u, size_t n, void *out, int out_fmt)
{
    if (!h || !valid_curve(curve) || (out_fmt != HS_FMT_AFFINE && out_fmt != HS_FMT_COMPRESSED &&
                                      out_fmt != HS_FMT_JACOBIAN51) ||
        (n && (!u || !out)))
        return HS_EINVAL;
    if (n == 0)
        return HS_OK;
    Context &ctx = h->c;
    std::lock_guard<std::mutex> lk(ctx.mu);
    DeviceGuard g(ctx.device);
    const CurveOps &ops = curve_ops(curve);
    HS_CU(ctx.arena.reserve(align256(n * 32) + align256(n * 64) + align256(n * 96) + align256(n * 120) + 1024),
          "workspace allocation");
    void *d_u = ctx.arena.take(n * 32);
    uint4 *d_aff = (uint4 *)ctx.arena.take(n * 64);
    uint32_t *d_j = (uint32_t *)ctx.arena.take(n * 96);
    void *d_o = ctx.arena.take(n * 120);
    cudaStream_t st = ctx.stream;
    HS_CU(cudaMemcpyAsync(d_u, u, n * 32, cudaMemcpyHostToDevice, st), "H2D");
    HS_CU(ops.map_to_curve(ctx, d_u, n, d_aff), "map to curve");
    if (out_fmt == HS_FMT_AFFINE) {
        HS_CU(cudaMemcpyAsync(out, d_aff, n * 64, cudaMemcpyDeviceToHost, st), "D2H");
    } else {
        HS_CU(ops.to_jac24(ctx, d_aff, HS_FMT_AFFINE, n, d_j), "pack");
        HS_CU(ops.format_out(ctx, d_j, n, out_fmt, d_o), "format");
        HS_CU(cudaMemcpyAsync(out, d_o, n * fmt_bytes(out_fmt), cudaMemcpyDeviceToHost, st), "D2H");
    }
    HS_CU(cudaStreamSynchronize(st), "map to curve");
    return HS_OK;
}

int hs_scalar_mul_device(hs_context *h, int curve, const void *d_scalars, const void *d_points, size_t n, void *d_out,
                         int out_fmt)
{
    if (!h || !valid_curve(curve) || !valid_out_fmt(out_fmt) || (n && (!d_scalars || !d_points || !d_out)))
        return HS_EINVAL;
    if (n == 0)
        return HS_OK;
    Context &ctx = h->c;
    std::lock_guard<std::mutex> lk(ctx.mu);
    DeviceGuard g(ctx.device);
    const CurveOps &ops = curve_ops(curve);
    HS_CU(ctx.arena.reserve(align256(n * 96) + 1024), "workspace allocation");
    uint32_t *d_j = (uint32_t *)ctx.arena.take(n * 96);
    if (!d_j)
        return fail_msg(ctx, HS_ENOMEM, "workspace carve");
    HS_CU(ops.scalar_mul(ctx, d_scalars, static_cast<const uint4 *>(d_points), n, d_j), "scalar multiplication");
    HS_CU(ops.format_out(ctx, d_j, n, out_fmt, d_out), "format");
    return HS_OK;
}

int hs_scalar_mul(hs_context *h, int curve, const uint8_t *scalars, const void *points, int point_fmt, size_t n,
                  void *out, int out_fmt)
{
    if (!h || !valid_curve(curve) || !valid_pt_fmt(point_fmt) || !valid_out_fmt(out_fmt) ||
        (n && (!scalars || !points || !out)))
        return HS_EINVAL;
    if (n == 0)
        return HS_OK;
    Context &ctx = h->c;
    std::lock_guard<std::mutex> lk(ctx.mu);
    DeviceGuard g(ctx.device);
    const CurveOps &ops = curve_ops(curve);
    const size_t pb = fmt_bytes(point_fmt), ob = fmt_bytes(out_fmt);
    HS_CU(ctx.arena.reserve(align256(n * 32) + align256(n * pb) + align256(n * 64) +
                            align256(ops.to_affine_scratch(n)) + align256(n * 96) + align256(n * ob) + 2048),
          "workspace allocation");
    uint8_t *d_sc = (uint8_t *)ctx.arena.take(n * 32);
    uint8_t *d_raw = (uint8_t *)ctx.arena.take(n * pb);
    uint4 *d_aff = (uint4 *)ctx.arena.take(n * 64);
    void *d_scr = ctx.arena.take(ops.to_affine_scratch(n));
    uint32_t *d_j = (uint32_t *)ctx.arena.take(n * 96);
    void *d_o = ctx.arena.take(n * ob);
    if (!d_sc || !d_raw || !d_aff || !d_scr || !d_j || !d_o)
        return fail_msg(ctx, HS_ENOMEM, "workspace carve");
    cudaStream_t st = ctx.stream;
    HS_CU(cudaMemcpyAsync(d_sc, scalars, n * 32, cudaMemcpyHostToDevice, st), "H2D scalars");
    HS_CU(cudaMemcpyAsync(d_raw, points, n * pb, cudaMemcpyHostToDevice, st), "H2D points");
    if (point_fmt == HS_FMT_AFFINE)
        HS_CU(cudaMemcpyAsync(d_aff, d_raw, n * 64, cudaMemcpyDeviceToDevice, st), "copy");
    else
        HS_CU(ops.to_affine(ctx, d_raw, point_fmt, n, d_aff, d_scr), "input conversion");
    HS_CU(ops.scalar_mul(ctx, d_sc, d_aff, n, d_j), "scalar multiplication");
    HS_CU(ops.format_out(ctx, d_j, n, out_fmt, d_o), "format");
    HS_CU(cudaMemcpyAsync(out, d_o, n * ob, cudaMemcpyDeviceToHost, st), "D2H");
    HS_CU(cudaStreamSynchronize(st), "scalar multiplication");
    if (point_fmt == HS_FMT_COMPRESSED)
        return check_decoded(ctx, d_scr);
    return HS_OK;
}

int hs_field_op(hs_context *h, int field, int op, const uint8_t *a, const uint8_t *b, size_t n, uint8_t *out)
{
    const bool binary = op == 0 || op == 2 || op == 3 || op == 7 || op == 8;
    if (!h || !valid_curve(field) || op < 0 || op > 10 || (n && (!a || !out || (binary && !b))))
        return HS_EINVAL;
    if (n == 0)
        return HS_OK;
    Context &ctx = h->c;
    std::lock_guard<std::mutex> lk(ctx.mu);
    DeviceGuard g(ctx.device);
    HS_CU(ctx.arena.reserve(3 * align256(n * 32) + 1024), "workspace allocation");
    void *da = ctx.arena.take(n * 32), *db = ctx.arena.take(n * 32), *dout = ctx.arena.take(n * 32);
    cudaStream_t st = ctx.stream;
    HS_CU(cudaMemcpyAsync(da, a, n * 32, cudaMemcpyHostToDevice, st), "H2D");
    if (binary)
        HS_CU(cudaMemcpyAsync(db, b, n * 32, cudaMemcpyHostToDevice, st), "H2D");
    HS_CU(curve_ops(field).field_op(ctx, op, da, db, n, dout), "field op");
    HS_CU(cudaMemcpyAsync(out, dout, n * 32, cudaMemcpyDeviceToHost, st), "D2H");
    HS_CU(cudaStreamSynchronize(st), "field op");
    return HS_OK;
}

int hs_msm_batch_device(hs_context *h, int curve, const size_t *sizes, size_t count, const void *d_scalars,
                        const void *d_points, void *d_out, int out_fmt)
{
    if (!h || !valid_curve(curve) || !valid_out_fmt(out_fmt) || (count && (!sizes || !d_out)))
        return HS_EINVAL;
    if (count == 0)
        return HS_OK;
    if (count >= 0x1000000ull)
        return HS_ERANGE;
    uint64_t total = 0;
    for (size_t i = 0; i < count; i++)
        total += sizes[i];
    if (total >= 0x80000000ull)
        return HS_ERANGE;
    if (total && (!d_scalars || !d_points))
        return HS_EINVAL;
    Context &ctx = h->c;
    std::lock_guard<std::mutex> lk(ctx.mu);
    DeviceGuard g(ctx.device);
    const BatchPlan p = make_batch_plan(ctx, curve, sizes, (uint32_t)count);
    if ((uint64_t)p.NB >= 0x80000000ull || p.entries_bound >= 0x80000000ull)
        return fail_msg(ctx, HS_ERANGE, "batch too large for one launch sequence");
    BatchBuffers b;
    int rc = reserve_batch(ctx, p, 0, b, nullptr);
    if (rc != HS_OK)
        return rc;
    b.scalars = static_cast<const uint32_t *>(d_scalars);
    b.points = static_cast<const uint4 *>(d_points);
    return execute_batch(ctx, p, b, d_out, out_fmt);
}

// Host-buffer batch of MSMs on either curve: the MSMs are grouped by curve,
// each group is staged into concatenated device arrays and runs as one batch;
// the Selene group runs on a second stream concurrently with the Helios group.
int hs_msm_batch(hs_context *h, const hs_msm_desc *descs, size_t count, int point_fmt, int out_fmt)
{
    if (!h || (count && !descs) || !valid_pt_fmt(point_fmt) || !valid_out_fmt(out_fmt))
        return HS_EINVAL;
    for (size_t i = 0; i < count; i++)
        if (!valid_curve(descs[i].curve) || !descs[i].out || (descs[i].n && (!descs[i].scalars || !descs[i].points)))
            return HS_EINVAL;
    if (count == 0)
        return HS_OK;
    Context &ctx = h->c;
    std::lock_guard<std::mutex> lk(ctx.mu);
    DeviceGuard g(ctx.device);
    const size_t pb = fmt_bytes(point_fmt), ob = fmt_bytes(out_fmt);
    std::vector<size_t> idx[2];
    std::vector<size_t> sizes[2];
    size_t totals[2] = {0, 0};
    for (size_t i = 0; i < count; i++) {
        const int k = descs[i].curve == HS_SELENE ? 1 : 0;
        idx[k].push_back(i);
        sizes[k].push_back(descs[i].n);
        totals[k] += descs[i].n;
    }
    if (totals[0] >= 0x80000000ull || totals[1] >= 0x80000000ull)
        return fail_msg(ctx, HS_ERANGE, "batch too large");
    BatchPlan plans[2];
    size_t bytes = 1024, stage[2] = {0, 0};
    for (int k = 0; k < 2; k++) {
        if (idx[k].empty())
            continue;
        plans[k] = make_batch_plan(ctx, k, sizes[k].data(), (uint32_t)idx[k].size());
        if (plans[k].entries_bound >= 0x80000000ull)
            return fail_msg(ctx, HS_ERANGE, "batch too large for one launch sequence");
        const size_t t = std::max<size_t>(1, totals[k]);
        stage[k] = align256(t * 32) + align256(t * 64) + (point_fmt == HS_FMT_AFFINE ? 0 : align256(t * pb)) +
                   align256(curve_ops(k).to_affine_scratch(t)) + align256(idx[k].size() * ob);
        bytes += batch_bytes(plans[k]) + stage[k] + 1024;
    }
    HS_CU(ctx.arena.reserve(bytes), "workspace allocation");
    BatchBuffers bufs[2];
    uint8_t *st_base[2] = {nullptr, nullptr};
    for (int k = 0; k < 2; k++) {
        if (idx[k].empty())
            continue;
        if (!carve(ctx.arena, plans[k], bufs[k]) || !(st_base[k] = (uint8_t *)ctx.arena.take(stage[k])))
            return fail_msg(ctx, HS_ENOMEM, "workspace carve");
    }
    HS_CU(ensure_stream2(ctx), "stream creation");
    LinkStream *link = nullptr;
    HS_CU(link_stream(ctx.device, &link), "stream creation");
    cudaStream_t s1 = ctx.stream, s3 = ctx.stream3;
    // On a device that reads pageable host memory, each group's input copies are
    // one gathered copy kernel (pull_list) instead of two driver-staged copies
    // per MSM; the lists are read by the device, so they outlive the drain below.
    std::vector<PullChunk> pulls[2];
    LinkDrain drain{link->s};  // drained before an early return (copy kernels may read the caller's pages)
    // per curve group: inputs on the device, bases converted; and the join
    cudaEvent_t ev_rec[2] = {}, ev_pts[2] = {}, ev_done = nullptr;
    struct EvGuard {
        cudaEvent_t *e[5];
        ~EvGuard()
        {
            for (cudaEvent_t *p : e)
                if (*p)
                    cudaEventDestroy(*p);
        }
    } evg{{&ev_rec[0], &ev_rec[1], &ev_pts[0], &ev_pts[1], &ev_done}};
    for (cudaEvent_t *p : evg.e)
        HS_CU(cudaEventCreateWithFlags(p, cudaEventDisableTiming), "event");
    // The group with more work (a Selene point costs about 1.6 Helios points)
    // is staged first on the device's link stream: its computation starts while
    // the other group's inputs are still arriving.
    const int first = totals[1] * 8 >= totals[0] * 5 ? 1 : 0;
    const int order[2] = {first, 1 - first};
    uint8_t *d_out[2] = {nullptr, nullptr};
    uint8_t *d_raw_k[2] = {nullptr, nullptr};
    uint8_t *d_scr_k[2] = {nullptr, nullptr};
    for (int k = 0; k < 2; k++) {
        if (idx[k].empty())
            continue;
        const size_t t = std::max<size_t>(1, totals[k]);
        uint8_t *d_sc = st_base[k];
        uint8_t *d_pts = d_sc + align256(t * 32);
        d_raw_k[k] = point_fmt == HS_FMT_AFFINE ? d_pts : d_pts + align256(t * 64);
        d_scr_k[k] = point_fmt == HS_FMT_AFFINE ? d_pts + align256(t * 64) : d_raw_k[k] + align256(t * pb);
        d_out[k] = d_scr_k[k] + align256(curve_ops(k).to_affine_scratch(t));
        bufs[k].scalars = (const uint32_t *)d_sc;
        bufs[k].points = (const uint4 *)d_pts;
    }
    HS_CU(cudaEventRecord(ctx.ev_fork, s1), "event");  // earlier work on the buffers comes first
    {
        std::lock_guard<std::mutex> lk(link->mu);
        cudaStream_t cs = link->s;
        HS_CU(cudaStreamWaitEvent(cs, ctx.ev_fork, 0), "stream wait");
        for (int k : order) {
            if (idx[k].empty())
                continue;
            // One copy kernel when the group's first inputs are pageable, or when the
            // group has more than 16 MSMs (two copy-engine copies each would cost more
            // host time than one launch); else the copy engine, which leaves the SMs
            // to the other group's work.  Either reads any host memory.  For the
            // 1024-MSM batched stream from host arrays on GB300: 61.9 ms per call
            // with the copy engine staging pageable arrays and 47.1 ms with it from
            // pinned ones; with the copy kernel 45.0-46.1 ms from pageable arrays
            // and 45.0 ms from pinned ones.
            bool pull = false;
            for (size_t j = 0; j < idx[k].size(); j++)
                if (descs[idx[k][j]].n) {
                    pull = ctx.pageable_access && (idx[k].size() > 16 || is_pageable(descs[idx[k][j]].scalars));
                    break;
                }
            size_t off = 0;
            for (size_t j = 0; j < idx[k].size(); j++) {
                const hs_msm_desc &d = descs[idx[k][j]];
                if (d.n && pull) {
                    pull_add(pulls[k], (uint8_t *)bufs[k].scalars + 32 * off, d.scalars, d.n * 32);
                    pull_add(pulls[k], d_raw_k[k] + pb * off, d.points, d.n * pb);
                } else if (d.n) {
                    HS_CU(cudaMemcpyAsync((uint8_t *)bufs[k].scalars + 32 * off, d.scalars, d.n * 32,
                                          cudaMemcpyHostToDevice, cs),
                          "H2D");
                    HS_CU(cudaMemcpyAsync(d_raw_k[k] + pb * off, d.points, d.n * pb, cudaMemcpyHostToDevice, cs),
                          "H2D");
                }
                off += d.n;
            }
            HS_CU(pull_list(ctx, pulls[k].data(), pulls[k].size(), cs), "H2D");
            HS_CU(cudaEventRecord(ev_rec[k], cs), "event");
        }
    }
    for (int k : order) {
        if (idx[k].empty())
            continue;
        HS_CU(cudaStreamWaitEvent(s3, ev_rec[k], 0), "stream wait");
        if (point_fmt != HS_FMT_AFFINE && totals[k]) {
            ctx.stream = s3;
            const cudaError_t ce = curve_ops(k).to_affine(ctx, d_raw_k[k], point_fmt, totals[k],
                                                          (uint4 *)bufs[k].points, d_scr_k[k]);
            ctx.stream = s1;
            HS_CU(ce, "conversion");
        }
        HS_CU(cudaEventRecord(ev_pts[k], s3), "event");
    }
    // Helios group on the first stream, Selene group on the second, each after its inputs
    int rc = HS_OK;
    if (!idx[0].empty()) {
        HS_CU(cudaStreamWaitEvent(s1, ev_pts[0], 0), "stream wait");
        rc = execute_batch(ctx, plans[0], bufs[0], d_out[0], out_fmt);
    }
    if (rc == HS_OK && !idx[1].empty()) {
        HS_CU(cudaStreamWaitEvent(ctx.stream2, ev_pts[1], 0), "stream wait");
        ctx.stream = ctx.stream2;
        rc = execute_batch(ctx, plans[1], bufs[1], d_out[1], out_fmt);
        ctx.stream = s1;
        HS_CU(cudaEventRecord(ev_done, ctx.stream2), "event");
        HS_CU(cudaStreamWaitEvent(s1, ev_done, 0), "stream wait");
    }
    if (rc != HS_OK)
        return rc;
    std::vector<uint8_t> host_out[2];
    for (int k = 0; k < 2; k++) {
        if (idx[k].empty())
            continue;
        host_out[k].resize(idx[k].size() * ob);
        HS_CU(cudaMemcpyAsync(host_out[k].data(), d_out[k], host_out[k].size(), cudaMemcpyDeviceToHost, s1), "D2H");
    }
    HS_CU(cudaStreamSynchronize(s1), "MSM batch");
    drain.s = nullptr;  // both groups waited for their input copies
    if (point_fmt == HS_FMT_COMPRESSED)
        for (int k = 0; k < 2; k++)
            if (!idx[k].empty() && totals[k] && (rc = check_decoded(ctx, d_scr_k[k])) != HS_OK)
                return rc;
    for (int k = 0; k < 2; k++)
        for (size_t j = 0; j < idx[k].size(); j++)
            std::memcpy(descs[idx[k][j]].out, host_out[k].data() + j * ob, ob);
    return HS_OK;
}

int hs_profile_enable(hs_context *h, int on)
{
    if (!h)
        return HS_EINVAL;
    std::lock_guard<std::mutex> lk(h->c.mu);
    h->c.profile = on != 0;
    return HS_OK;
}

int hs_profile_read(hs_context *h, double *ms, uint64_t *launches, uint64_t *entries, int reset)
{
    if (!h)
        return HS_EINVAL;
    Context &ctx = h->c;
    std::lock_guard<std::mutex> lk(ctx.mu);
    DeviceGuard g(ctx.device);
    HS_CU(cudaStreamSynchronize(ctx.stream), "profile sync");
    for (auto &pr : ctx.prof_events) {
        float t = 0.f;
        if (cudaEventElapsedTime(&t, pr.first, pr.second) == cudaSuccess)
            ctx.prof_ms += t;
        cudaEventDestroy(pr.first);
        cudaEventDestroy(pr.second);
    }
    ctx.prof_events.clear();
    if (ms)
        *ms = ctx.prof_ms;
    if (launches)
        *launches = ctx.prof_launches;
    if (entries)
        *entries = ctx.prof_entries;
    if (reset) {
        ctx.prof_ms = 0.0;
        ctx.prof_launches = 0;
        ctx.prof_entries = 0;
    }
    return HS_OK;
}

// instructions per second of probe `probe`: 0 mad.lo/mad.hi pairs, 1 mad.wide.u32,
// 2 mad.lo alone, 3 mad.hi alone (8 chains x iters per thread)
static int imad_probe(Context &ctx, int probe, double *instr_per_s)
{
    const int threads = 256, blocks = ctx.sm_count * 8, iters = 4096;
    const size_t out_bytes = (size_t)blocks * threads * sizeof(uint32_t);
    HS_CU(ctx.arena.reserve(out_bytes + 256), "workspace allocation");
    uint32_t *d = (uint32_t *)ctx.arena.take(out_bytes);
    if (!d)
        return fail_msg(ctx, HS_ENOMEM, "workspace carve");
    cudaEvent_t e0, e1;
    HS_CU(cudaEventCreate(&e0), "event");
    HS_CU(cudaEventCreate(&e1), "event");
    auto launch = [&](uint32_t seed, int it) {
        switch (probe) {
        case 0: k_imad_peak<0><<<blocks, threads, 0, ctx.stream>>>(seed, it, d); break;
        case 1: k_imad_wide_peak<<<blocks, threads, 0, ctx.stream>>>(seed, it, d); break;
        case 2: k_imad_peak<1><<<blocks, threads, 0, ctx.stream>>>(seed, it, d); break;
        default: k_imad_peak<2><<<blocks, threads, 0, ctx.stream>>>(seed, it, d); break;
        }
        ctx.launches++;
    };
    launch(1u, 64);  // warm-up
    float best = 1e30f;
    for (int rep = 0; rep < 5; rep++) {
        cudaEventRecord(e0, ctx.stream);
        launch((uint32_t)rep, iters);
        cudaEventRecord(e1, ctx.stream);
        const cudaError_t se = cudaEventSynchronize(e1);
        if (se != cudaSuccess) {
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            return fail(ctx, se, "imad probe");
        }
        float t = 0.f;
        cudaEventElapsedTime(&t, e0, e1);
        best = std::min(best, t);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    HS_CU(cudaGetLastError(), "imad probe");
    const double per_iter = probe == 0 ? 16.0 : 8.0;  // instructions per chain step of the 8 chains
    *instr_per_s = (double)blocks * threads * iters * per_iter / (best * 1e-3);
    return HS_OK;
}

int hs_measure_imad_peak(hs_context *h, double *imad_per_s)
{
    if (!h || !imad_per_s)
        return HS_EINVAL;
    Context &ctx = h->c;
    std::lock_guard<std::mutex> lk(ctx.mu);
    DeviceGuard g(ctx.device);
    double pair = 0.0, wide = 0.0;
    int rc = imad_probe(ctx, 0, &pair);
    if (rc == HS_OK)
        rc = imad_probe(ctx, 1, &wide);
    if (rc != HS_OK)
        return rc;
    // a lo/hi pair is one product (2 IMAD-eq); a wide instruction is one product
    *imad_per_s = std::max(pair, 2.0 * wide);
    return HS_OK;
}

int hs_measure_imad_rates(hs_context *h, double rates[4])
{
    if (!h || !rates)
        return HS_EINVAL;
    Context &ctx = h->c;
    std::lock_guard<std::mutex> lk(ctx.mu);
    DeviceGuard g(ctx.device);
    for (int probe = 0; probe < 4; probe++) {
        const int rc = imad_probe(ctx, probe, &rates[probe]);
        if (rc != HS_OK)
            return rc;
    }
    return HS_OK;
}

// ---- fixed-base commitments ----
static int fixed_window(size_t n)
{
    // one reduction window: cost ~ W(c) * n * madd + 2^(c-1) * 2 adds
    int best = 8;
    double best_cost = 1e300;
    for (int c = 6; c <= 20; c++) {
        const double W = (257 + c - 1) / c;
        const double cost = W * 10.0 * (double)n + 28.0 * (double)(1u << (c - 1));
        if (cost < best_cost) {
            best_cost = cost;
            best = c;
        }
    }
    return best;
}

int hs_fixed_base_create(hs_context *h, int curve, const void *generators, int point_fmt, size_t n, const void *H,
                         int window, hs_fixed_base **out)
{
    if (!h || !out || !valid_curve(curve) || !valid_pt_fmt(point_fmt) || (n && !generators) ||
        (window != 0 && (window < 4 || window > 20)))
        return HS_EINVAL;
    *out = nullptr;
    const size_t n_gen = n + (H ? 1 : 0);
    if (n_gen == 0)
        return HS_EINVAL;
    const int c = window ? window : fixed_window(n_gen);
    const int W = (257 + c - 1) / c;
    if (n_gen * (size_t)W >= 0x80000000ull)
        return HS_ERANGE;
    Context &ctx = h->c;
    std::lock_guard<std::mutex> lk(ctx.mu);
    DeviceGuard g(ctx.device);
    const CurveOps &ops = curve_ops(curve);
    const size_t pb = fmt_bytes(point_fmt);
    const size_t m = n_gen * (size_t)W;
    HS_CU(ctx.arena.reserve(align256(n_gen * pb) + align256(n_gen * 64) + align256(ops.to_affine_scratch(n_gen)) +
                            align256(m * 160) + 1024),
          "workspace allocation");
    uint8_t *d_raw = (uint8_t *)ctx.arena.take(n_gen * pb);
    uint4 *d_gens = (uint4 *)ctx.arena.take(n_gen * 64);
    void *d_scr = ctx.arena.take(ops.to_affine_scratch(n_gen));
    uint4 *d_tmp = (uint4 *)ctx.arena.take(m * 160);
    if (!d_raw || !d_gens || !d_scr || !d_tmp)
        return fail_msg(ctx, HS_ENOMEM, "workspace carve");
    hs_fixed_base *fb = new (std::nothrow) hs_fixed_base();
    if (!fb)
        return HS_ENOMEM;
    fb->curve = curve;
    fb->device = ctx.device;
    fb->c = c;
    fb->W = W;
    fb->n_user = n;
    fb->n_gen = n_gen;
    fb->has_H = H != nullptr;
    cudaError_t e = cudaMalloc((void **)&fb->d_table, m * 64);
    if (e != cudaSuccess) {
        delete fb;
        return fail(ctx, e, "fixed-base table allocation");
    }
    cudaStream_t st = ctx.stream;
    auto bail = [&](cudaError_t err, const char *what) {
        cudaFree(fb->d_table);
        delete fb;
        return fail(ctx, err, what);
    };
    if (n && (e = cudaMemcpyAsync(d_raw, generators, n * pb, cudaMemcpyHostToDevice, st)) != cudaSuccess)
        return bail(e, "H2D generators");
    if (H && (e = cudaMemcpyAsync(d_raw + n * pb, H, pb, cudaMemcpyHostToDevice, st)) != cudaSuccess)
        return bail(e, "H2D H");
    if (point_fmt != HS_FMT_AFFINE) {
        if ((e = ops.to_affine(ctx, d_raw, point_fmt, n_gen, d_gens, d_scr)) != cudaSuccess)
            return bail(e, "generator conversion");
    } else if ((e = cudaMemcpyAsync(d_gens, d_raw, n_gen * 64, cudaMemcpyDeviceToDevice, st)) != cudaSuccess) {
        return bail(e, "generator copy");
    }
    if ((e = ops.fixed_table(ctx, d_gens, n_gen, c, W, d_tmp, fb->d_table)) != cudaSuccess)
        return bail(e, "window table");
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess)
        return bail(e, "window table");
    if (point_fmt == HS_FMT_COMPRESSED && n_gen) {
        uint32_t bad = 0;
        if ((e = cudaMemcpy(&bad, d_scr, sizeof(bad), cudaMemcpyDeviceToHost)) != cudaSuccess)
            return bail(e, "decode check");
        if (bad) {
            cudaFree(fb->d_table);
            delete fb;
            return fail_msg(ctx, HS_EINVAL, "invalid point encoding");
        }
    }
    *out = fb;
    return HS_OK;
}

// a chunk of `count` commitments, with the curve's bucket accumulation form
static BatchPlan fixed_plan(const Context &ctx, const hs_fixed_base *fb, uint32_t count)
{
    BatchPlan p = make_fixed_plan(fb->curve, fb->n_gen, fb->c, count);
    const int k = fb->curve == HS_SELENE ? 1 : 0;
    plan_batch_affine(p, ctx.ba_set[k] ? ctx.ba_rounds[k] : ctx.fixed_ba_rounds[k], ctx.ba_min_entries[k]);
    return p;
}

// Run count fixed-base commitments whose scalars are at d_scalars (count x n_gen
// x 32 bytes on the device) in chunks bounded by the entry count; results to d_out.
static int fixed_commit_chunks(Context &ctx, const hs_fixed_base *fb, const uint8_t *d_scalars, size_t count,
                               uint8_t *d_out, int out_fmt)
{
    const uint64_t per = (uint64_t)fb->n_gen * fb->W;
    const size_t chunk = (size_t)std::max<uint64_t>(1, std::min<uint64_t>(count, (1ull << 29) / per));
    const BatchPlan big = fixed_plan(ctx, fb, (uint32_t)chunk);
    const bool aff = out_fmt == HS_FMT_AFFINE;
    // affine results: Jacobian first, then one shared inversion per 16 commitments
    const size_t extra = aff ? align256(count * 120) + align256(count * 32) : 0;
    HS_CU(ctx.arena.reserve(batch_bytes(big) + extra + 2048), "workspace allocation");
    const size_t ob = aff ? 120 : fmt_bytes(out_fmt);
    uint8_t *d_jac = nullptr;
    void *d_scr = nullptr;
    for (size_t j0 = 0; j0 < count; j0 += chunk) {
        const size_t cnt = std::min(chunk, count - j0);
        const BatchPlan p = fixed_plan(ctx, fb, (uint32_t)cnt);
        ctx.arena.reset();
        if (aff) {  // results and scratch live at the front of the arena, below the batch workspace
            d_jac = (uint8_t *)ctx.arena.take(count * 120);
            d_scr = ctx.arena.take(count * 32);
        }
        BatchBuffers b;
        if (!carve(ctx.arena, p, b))
            return fail_msg(ctx, HS_ENOMEM, "workspace carve");
        b.scalars = (const uint32_t *)(d_scalars + 32 * fb->n_gen * j0);
        b.points = fb->d_table;
        const int rc = execute_batch(ctx, p, b, (aff ? d_jac : d_out) + ob * j0, aff ? HS_FMT_JACOBIAN51 : out_fmt);
        if (rc != HS_OK)
            return rc;
    }
    if (aff)
        HS_CU(curve_ops(fb->curve).to_affine(ctx, d_jac, HS_FMT_JACOBIAN51, count, (uint4 *)d_out, d_scr),
              "batch to affine");
    return HS_OK;
}

int hs_fixed_base_commit_device(hs_context *h, const hs_fixed_base *fb, const void *d_scalars, size_t count,
                                void *d_out, int out_fmt)
{
    if (!h || !fb || !valid_out_fmt(out_fmt) || (count && (!d_scalars || !d_out)))
        return HS_EINVAL;
    if (count == 0)
        return HS_OK;
    if ((uint64_t)count * fb->n_gen >= 0x80000000ull)
        return HS_ERANGE;
    Context &ctx = h->c;
    if (ctx.device != fb->device)
        return HS_EINVAL;
    std::lock_guard<std::mutex> lk(ctx.mu);
    DeviceGuard g(ctx.device);
    return fixed_commit_chunks(ctx, fb, (const uint8_t *)d_scalars, count, (uint8_t *)d_out, out_fmt);
}

int hs_fixed_base_commit(hs_context *h, const hs_fixed_base *fb, const uint8_t *values, const uint8_t *blindings,
                         size_t count, void *out, int out_fmt)
{
    if (!h || !fb || !valid_out_fmt(out_fmt) || (count && (!out || (fb->n_user && !values))) ||
        (blindings && !fb->has_H))
        return HS_EINVAL;
    if (count == 0)
        return HS_OK;
    Context &ctx = h->c;
    if (ctx.device != fb->device)
        return HS_EINVAL;
    std::lock_guard<std::mutex> lk(ctx.mu);
    DeviceGuard g(ctx.device);
    const CurveOps &ops = curve_ops(fb->curve);
    const uint64_t per = (uint64_t)fb->n_gen * fb->W;
    const size_t chunk = (size_t)std::max<uint64_t>(1, std::min<uint64_t>(count, (1ull << 29) / per));
    const size_t ob = fmt_bytes(out_fmt);
    // staging for one chunk: scalars in the device layout, Jacobian results, formatted results
    const size_t sc_bytes = align256(chunk * fb->n_gen * 32);
    const size_t extra = sc_bytes + align256(chunk * 120) + align256(chunk * ob) + align256(chunk * 32) + 256;
    std::vector<uint8_t> host(count * ob);
    for (size_t j0 = 0; j0 < count; j0 += chunk) {
        const size_t cnt = std::min(chunk, count - j0);
        const BatchPlan big = fixed_plan(ctx, fb, (uint32_t)chunk);
        HS_CU(ctx.arena.reserve(batch_bytes(big) + align256(extra) + 1024), "workspace allocation");
        const BatchPlan p = fixed_plan(ctx, fb, (uint32_t)cnt);
        BatchBuffers b;
        if (!carve(ctx.arena, p, b))
            return fail_msg(ctx, HS_ENOMEM, "workspace carve");
        uint8_t *d_sc = (uint8_t *)ctx.arena.take(sc_bytes);
        uint8_t *d_jac = (uint8_t *)ctx.arena.take(align256(chunk * 120));
        uint8_t *d_fmt = (uint8_t *)ctx.arena.take(align256(chunk * ob));
        void *d_scr = ctx.arena.take(align256(chunk * 32));
        if (!d_sc || !d_jac || !d_fmt || !d_scr)
            return fail_msg(ctx, HS_ENOMEM, "workspace carve");
        cudaStream_t st = ctx.stream;
        const size_t g = fb->n_gen;
        if (fb->n_user)
            HS_CU(cudaMemcpy2DAsync(d_sc, g * 32, values + j0 * fb->n_user * 32, fb->n_user * 32, fb->n_user * 32,
                                    cnt, cudaMemcpyHostToDevice, st),
                  "H2D values");
        if (fb->has_H) {
            if (blindings)
                HS_CU(cudaMemcpy2DAsync(d_sc + fb->n_user * 32, g * 32, blindings + j0 * 32, 32, 32, cnt,
                                        cudaMemcpyHostToDevice, st),
                      "H2D blindings");
            else
                HS_CU(cudaMemset2DAsync(d_sc + fb->n_user * 32, g * 32, 0, 32, cnt, st), "zero blindings");
        }
        b.scalars = (const uint32_t *)d_sc;
        b.points = fb->d_table;
        const bool aff = out_fmt == HS_FMT_AFFINE;
        int rc = execute_batch(ctx, p, b, aff ? d_jac : d_fmt, aff ? HS_FMT_JACOBIAN51 : out_fmt);
        if (rc != HS_OK)
            return rc;
        if (aff)  // normalise all results with one shared inversion per 16 (Montgomery's trick)
            HS_CU(ops.to_affine(ctx, d_jac, HS_FMT_JACOBIAN51, cnt, (uint4 *)d_fmt, d_scr), "batch to affine");
        HS_CU(cudaMemcpyAsync(host.data() + j0 * ob, d_fmt, cnt * ob, cudaMemcpyDeviceToHost, st), "D2H");
        HS_CU(cudaStreamSynchronize(st), "fixed-base commit");
    }
    std::memcpy(out, host.data(), host.size());
    return HS_OK;
}

int hs_fixed_base_info(const hs_fixed_base *fb, int *window, size_t *table_bytes)
{
    if (!fb)
        return HS_EINVAL;
    if (window)
        *window = fb->c;
    if (table_bytes)
        *table_bytes = fb->n_gen * (size_t)fb->W * 64;
    return HS_OK;
}

void hs_fixed_base_destroy(hs_fixed_base *fb)
{
    if (!fb)
        return;
    {
        DeviceGuard g(fb->device);
        cudaDeviceSynchronize();
        cudaFree(fb->d_table);
    }
    delete fb;
}

// ---- reference-signature drop-ins on a process-wide context ----
static hs_context *g_ctx = nullptr;
static std::once_flag g_ctx_once;
static int g_ctx_rc = HS_OK;

static hs_context *global_ctx()
{
    std::call_once(g_ctx_once, [] { g_ctx_rc = hs_context_create(&g_ctx, 0); });
    if (g_ctx_rc != HS_OK || !g_ctx) {
        std::fprintf(stderr, "helioselene_gb300: cannot create the device context (%s: %s)\n",
                     hs_strerror(g_ctx_rc), hs_last_error(nullptr));
        std::abort();
    }
    return g_ctx;
}

static void must(int rc, const char *what)
{
    if (rc != HS_OK) {
        std::fprintf(stderr, "helioselene_gb300: %s failed (%s: %s)\n", what, hs_strerror(rc),
                     hs_last_error(g_ctx));
        std::abort();
    }
}

void hs_helios_msm_vartime(hs_jacobian51 *result, const unsigned char *scalars, const hs_jacobian51 *points, size_t n)
{
    if (n == 0 || !scalars || !points) {
        identity_out(HS_HELIOS, HS_FMT_JACOBIAN51, result);
        return;
    }
    must(hs_msm(global_ctx(), HS_HELIOS, scalars, points, HS_FMT_JACOBIAN51, n, result, HS_FMT_JACOBIAN51),
         "helios MSM");
}

void hs_selene_msm_vartime(hs_jacobian51 *result, const unsigned char *scalars, const hs_jacobian51 *points, size_t n)
{
    if (n == 0 || !scalars || !points) {
        identity_out(HS_SELENE, HS_FMT_JACOBIAN51, result);
        return;
    }
    must(hs_msm(global_ctx(), HS_SELENE, scalars, points, HS_FMT_JACOBIAN51, n, result, HS_FMT_JACOBIAN51),
         "selene MSM");
}

void hs_helios_scalarmult_vartime(hs_jacobian51 *result, const unsigned char scalar[32], const hs_jacobian51 *p)
{
    must(hs_scalar_mul(global_ctx(), HS_HELIOS, scalar, p, HS_FMT_JACOBIAN51, 1, result, HS_FMT_JACOBIAN51),
         "helios scalar multiplication");
}

void hs_selene_scalarmult_vartime(hs_jacobian51 *result, const unsigned char scalar[32], const hs_jacobian51 *p)
{
    must(hs_scalar_mul(global_ctx(), HS_SELENE, scalar, p, HS_FMT_JACOBIAN51, 1, result, HS_FMT_JACOBIAN51),
         "selene scalar multiplication");
}

void hs_helios_pedersen_commit(hs_jacobian51 *result, const unsigned char *blinding, const hs_jacobian51 *H,
                               const unsigned char *values, const hs_jacobian51 *generators, size_t n)
{
    must(hs_pedersen(global_ctx(), HS_HELIOS, blinding, H, values, generators, HS_FMT_JACOBIAN51, n, result,
                     HS_FMT_JACOBIAN51),
         "helios Pedersen commitment");
}

void hs_selene_pedersen_commit(hs_jacobian51 *result, const unsigned char *blinding, const hs_jacobian51 *H,
                               const unsigned char *values, const hs_jacobian51 *generators, size_t n)
{
    must(hs_pedersen(global_ctx(), HS_SELENE, blinding, H, values, generators, HS_FMT_JACOBIAN51, n, result,
                     HS_FMT_JACOBIAN51),
         "selene Pedersen commitment");
}

void hs_helios_batch_to_affine(hs_affine51 *out, const hs_jacobian51 *points, size_t n)
{
    must(hs_batch_to_affine(global_ctx(), HS_HELIOS, points, n, out, HS_FMT_AFFINE51), "helios batch to affine");
}

void hs_selene_batch_to_affine(hs_affine51 *out, const hs_jacobian51 *points, size_t n)
{
    must(hs_batch_to_affine(global_ctx(), HS_SELENE, points, n, out, HS_FMT_AFFINE51), "selene batch to affine");
}

}  // extern "C"
