// hs_serving.cu -- continuous-batching request loop for MSMs (hs_server_*).
//
// The reference has no serving layer; this is the GB300 form of "many
// independent public-data MSMs arriving over time" (FCMP++ alternates Helios
// and Selene layers).  One scheduler thread owns `slots` execution slots
// (stream + workspace each).  Each pass it (1) retires slots whose completion
// event fired, copying results out and waking waiters; (2) while a slot is
// free and requests are queued, takes the oldest request's curve, collects up
// to the caps of queued requests of that curve (FIFO), checks the batch's
// workspace against the HBM budget, stages scalars / fresh bases, and launches
// the batched MSM pipeline on that slot.  A curve's resident pool is also kept
// as a table of window multiples 2^(c k) P_i (built once by
// hs_server_set_pool): a request whose bases all come from the pool is a
// fixed-base MSM over the table rows its indices name (one reduced window, no
// Horner chain), batched with other such requests.  A request with fresh bases
// is a variable-base MSM whose pooled bases are gathered into its batch on the
// device.  A batch holds one curve and one of the two forms.
// All waits are host-side and bounded.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "hs_internal.h"

namespace hs {

// Pooled bases of a batch: request r's pool indices are src[seg[r].y, seg[r].y +
// seg[r].z) and its bases go to out[seg[r].x ...].  Entry p belongs to the last
// request whose first index is <= p (requests without pooled bases share the
// next one's start and lose the search).
__global__ void k_gather_pool(const uint4 *__restrict__ pool, const uint32_t *__restrict__ src,
                              const uint4 *__restrict__ seg, uint32_t nseg, uint32_t count, uint4 *__restrict__ out)
{
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= count)
        return;
    const uint32_t r = find_msm(nseg, p, [&](uint32_t k) { return seg[k].y; });
    const uint4 *s = pool + 4 * (size_t)src[p];
    uint4 *d = out + 4 * ((size_t)seg[r].x + (p - seg[r].y));
    d[0] = s[0];
    d[1] = s[1];
    d[2] = s[2];
    d[3] = s[3];
}

using Clock = std::chrono::steady_clock;

// one launch sequence indexes its (point, window) entries with 31 bits
constexpr uint64_t BATCH_ENTRIES_MAX = 0x7fffffffull;

struct ReqState {
    hs_request req;
    size_t n = 0;
    bool table = false;    // pooled bases only, computed over the pool's window table
    uint64_t entries = 0;  // n x windows under the slots' window rules at submission
    Clock::time_point submitted;
    double latency_ms = 0.0;
    int status = 1;  // 1 = pending, else HS_OK / error
};

struct Slot {
    Context ctx;
    cudaEvent_t done = nullptr;
    bool busy = false;
    int curve = 0;
    size_t bytes = 0;
    std::vector<uint64_t> tickets;
    uint8_t *pinned_out = nullptr;
    size_t pinned_cap = 0;
    std::vector<uint4> h_seg;  // per request: (first point, first pool index, pool count); kept until retire
    // the batch's input copies as one gathered copy (pull_list, devices that read
    // pageable host memory); read by the device, so kept until retire
    std::vector<PullChunk> h_pull;
};

struct Pool {
    uint4 *d = nullptr;      // affine bases (pools without a table)
    uint4 *table = nullptr;  // n * W window multiples, affine: row i*W + k = 2^(c k) P_i
    int c = 0;
    uint32_t W = 0;
    size_t n = 0;
    uint64_t gen = 0;  // bumped by every replacement
    int window = -1;   // for the next replacement: table width, 0 = no table, -1 = POOL_WINDOW_AUTO
};

// width of a pool's window-multiple table unless set: for requests of a few
// hundred to a few hundred thousand pooled bases, c = 12 (22 rows per base)
// takes fewer (point, window) entries than the variable-base windows of
// requests up to ~2^17 bases and reduces 2048 buckets per request
constexpr int POOL_WINDOW_AUTO = 12;

struct Server {
    hs_server_config cfg{};
    std::vector<std::unique_ptr<Slot>> slots;
    Pool pools[2];
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<uint64_t> queue;
    std::unordered_map<uint64_t, ReqState> reqs;
    uint64_t next_ticket = 1;
    size_t in_flight = 0;
    bool stop = false;
    hs_server_stats stats{};
    std::thread thr;
    std::string last_error;
};

// whether a request runs over its curve's pool table
static bool table_form(const Server &S, const hs_request &q)
{
    return S.pools[q.curve].table && q.n_pool && !q.n_fresh;
}

// (point, window) entries of a request under the slots' window rules, or the
// pool table's windows
static uint64_t request_entries(const Server &S, const hs_request &q)
{
    const size_t n = q.n_pool + q.n_fresh;
    if (table_form(S, q))
        return (uint64_t)n * S.pools[q.curve].W;
    const int c = choose_window(S.slots[0]->ctx, q.curve, n ? n : 1);
    return (uint64_t)n * (uint64_t)((257 + c - 1) / c);
}

static size_t batch_stage_bytes(size_t total, size_t total_pool, size_t msms, size_t ob)
{
    return align256(std::max<size_t>(1, total) * 32) + align256(std::max<size_t>(1, total) * 64) +
           align256(std::max<size_t>(1, total_pool) * 4) + align256(std::max<size_t>(1, msms) * 16) +
           align256(std::max<size_t>(1, msms) * ob);
}

static void finish_launch(Server &S, Slot &s, std::vector<uint64_t> &batch, int curve, size_t bytes)
{
    s.busy = true;
    s.curve = curve;
    s.bytes = bytes;
    s.tickets = batch;
    S.in_flight += bytes;
    S.stats.peak_bytes = std::max<uint64_t>(S.stats.peak_bytes, S.in_flight);
    S.stats.batches++;
    S.stats.max_batch_msms = std::max<uint64_t>(S.stats.max_batch_msms, batch.size());
}

static bool fail_requests(Server &S, Slot &s, const std::vector<uint64_t> &batch, int code)
{
    for (uint64_t t : batch) {
        ReqState &r = S.reqs[t];
        r.status = code;
        S.stats.failed++;
    }
    S.last_error = s.ctx.last_error;
    S.cv_done.notify_all();
    return true;
}

// a batch that fails after its copies were issued: the slot's stream drains
// first (a copy kernel may still be reading the requests' buffers, which their
// callers may free once told of the failure)
static bool fail_staged(Server &S, Slot &s, const std::vector<uint64_t> &batch, int code)
{
    cudaStreamSynchronize(s.ctx.stream);
    cudaGetLastError();
    return fail_requests(S, s, batch, code);
}

static bool ensure_pinned_out(Slot &s, size_t bytes)
{
    if (s.pinned_cap >= bytes)
        return true;
    if (s.pinned_out)
        cudaFreeHost(s.pinned_out);
    s.pinned_cap = std::max<size_t>(bytes, 1024 * 120);
    if (cudaMallocHost((void **)&s.pinned_out, s.pinned_cap) != cudaSuccess) {
        s.pinned_out = nullptr;
        s.pinned_cap = 0;
        cudaGetLastError();
        return false;
    }
    return true;
}

// A batch of pool-only requests: fixed-base MSMs over the rows of the curve's
// pool table that their indices name.  Called with the server lock held;
// false = deferred (budget).
static bool launch_table(Server &S, Slot &s, std::vector<uint64_t> &batch, int curve)
{
    const Pool &pool = S.pools[curve];
    const size_t ob = fmt_bytes(S.cfg.out_fmt);
    const uint32_t M = (uint32_t)batch.size();
    std::vector<size_t> sizes(M);
    size_t tp = 0;
    for (uint32_t j = 0; j < M; j++) {
        sizes[j] = S.reqs[batch[j]].req.n_pool;
        tp += sizes[j];
    }
    Context &ctx = s.ctx;
    const BatchPlan p = make_indexed_plan(ctx, curve, sizes.data(), M, pool.c);
    if (p.entries_bound > BATCH_ENTRIES_MAX)
        return fail_requests(S, s, batch, HS_ERANGE);
    // staging: scalars, indices, M results
    const size_t extra = align256(std::max<size_t>(1, tp) * 32) + align256(std::max<size_t>(1, tp) * 4) +
                         align256((size_t)M * ob);
    const size_t bytes = batch_bytes(p) + extra + 2048;
    if (S.in_flight > 0 && S.in_flight + bytes > S.cfg.hbm_budget) {
        S.stats.deferred++;
        return false;
    }
    BatchBuffers b;
    void *ext = nullptr;
    if (reserve_batch(ctx, p, extra, b, &ext) != HS_OK)
        return fail_requests(S, s, batch, HS_ENOMEM);
    uint8_t *d_sc = (uint8_t *)ext;
    uint32_t *d_idx = (uint32_t *)(d_sc + align256(std::max<size_t>(1, tp) * 32));
    uint8_t *d_out = (uint8_t *)d_idx + align256(std::max<size_t>(1, tp) * 4);
    if (!ensure_pinned_out(s, (size_t)M * ob))
        return fail_requests(S, s, batch, HS_ENOMEM);
    cudaStream_t st = ctx.stream;
    cudaError_t e = cudaSuccess;
    size_t off = 0;
    s.h_pull.clear();
    for (uint64_t t : batch) {
        const hs_request &q = S.reqs[t].req;
        if (ctx.pageable_access) {
            pull_add(s.h_pull, d_sc + 32 * off, q.scalars, 32 * q.n_pool);
            pull_add(s.h_pull, d_idx + off, q.pool_idx, 4 * q.n_pool);
        } else {
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(d_sc + 32 * off, q.scalars, 32 * q.n_pool, cudaMemcpyHostToDevice, st);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(d_idx + off, q.pool_idx, 4 * q.n_pool, cudaMemcpyHostToDevice, st);
        }
        off += q.n_pool;
    }
    if (e == cudaSuccess)
        e = pull_list(ctx, s.h_pull.data(), s.h_pull.size(), st);
    if (e != cudaSuccess) {
        ctx.last_error = std::string("staging: ") + cudaGetErrorString(e);
        return fail_staged(S, s, batch, HS_ECUDA);
    }
    b.scalars = (const uint32_t *)d_sc;
    b.points = pool.table;
    b.pt_idx = d_idx;
    if (execute_batch(ctx, p, b, d_out, S.cfg.out_fmt) != HS_OK)
        return fail_staged(S, s, batch, HS_ECUDA);
    e = cudaMemcpyAsync(s.pinned_out, d_out, (size_t)M * ob, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess)
        e = cudaEventRecord(s.done, st);
    if (e != cudaSuccess) {
        ctx.last_error = std::string("result copy: ") + cudaGetErrorString(e);
        return fail_staged(S, s, batch, HS_ECUDA);
    }
    finish_launch(S, s, batch, curve, bytes);
    return true;
}

// launch one batch on slot s; called with the server lock held; false = deferred (budget)
static bool launch(Server &S, Slot &s, std::vector<uint64_t> &batch, int curve)
{
    if (S.reqs[batch.front()].table)
        return launch_table(S, s, batch, curve);
    const size_t ob = fmt_bytes(S.cfg.out_fmt);
    std::vector<size_t> sizes;
    size_t total = 0, total_pool = 0;
    for (uint64_t t : batch) {
        const ReqState &r = S.reqs[t];
        sizes.push_back(r.n);
        total += r.n;
        total_pool += r.req.n_pool;
    }
    Context &ctx = s.ctx;
    const BatchPlan p = make_batch_plan(ctx, curve, sizes.data(), (uint32_t)sizes.size());
    if (p.entries_bound > BATCH_ENTRIES_MAX) {  // window rules changed since submission
        for (uint64_t t : batch) {
            S.reqs[t].status = HS_ERANGE;
            S.stats.failed++;
        }
        S.cv_done.notify_all();
        return true;
    }
    const size_t extra = batch_stage_bytes(total, total_pool, batch.size(), ob);
    const size_t bytes = batch_bytes(p) + extra + 2048;
    if (S.in_flight > 0 && S.in_flight + bytes > S.cfg.hbm_budget) {
        S.stats.deferred++;
        return false;
    }
    auto fail_batch = [&](int code) { return fail_requests(S, s, batch, code); };
    BatchBuffers b;
    void *ext = nullptr;
    if (reserve_batch(ctx, p, extra, b, &ext) != HS_OK)
        return fail_batch(HS_ENOMEM);
    uint8_t *d_sc = (uint8_t *)ext;
    uint8_t *d_pts = d_sc + align256(std::max<size_t>(1, total) * 32);
    uint32_t *d_src = (uint32_t *)(d_pts + align256(std::max<size_t>(1, total) * 64));
    uint4 *d_seg = (uint4 *)((uint8_t *)d_src + align256(std::max<size_t>(1, total_pool) * 4));
    uint8_t *d_out = (uint8_t *)d_seg + align256(std::max<size_t>(1, batch.size()) * 16);
    if (!ensure_pinned_out(s, batch.size() * ob))
        return fail_batch(HS_ENOMEM);
    cudaStream_t st = ctx.stream;
    // per request: its scalars, fresh bases and pool indices copied straight from
    // the caller's buffers, plus one table row; the pooled bases are gathered on
    // the device
    // (on a device that reads pageable host memory, all of them as one gathered
    // copy: the scheduler then issues one launch instead of staging each copy
    // through the driver, which holds it -- and the server lock -- per copy)
    s.h_seg.clear();
    s.h_pull.clear();
    size_t off = 0, poff = 0;
    cudaError_t e = cudaSuccess;
    for (uint64_t t : batch) {
        const hs_request &q = S.reqs[t].req;
        const size_t n = q.n_pool + q.n_fresh;
        if (ctx.pageable_access) {
            pull_add(s.h_pull, d_sc + 32 * off, q.scalars, 32 * n);
            pull_add(s.h_pull, d_pts + 64 * (off + q.n_pool), q.fresh_points, 64 * q.n_fresh);
            pull_add(s.h_pull, d_src + poff, q.pool_idx, 4 * q.n_pool);
        } else {
            if (n && e == cudaSuccess)
                e = cudaMemcpyAsync(d_sc + 32 * off, q.scalars, 32 * n, cudaMemcpyHostToDevice, st);
            if (q.n_fresh && e == cudaSuccess)
                e = cudaMemcpyAsync(d_pts + 64 * (off + q.n_pool), q.fresh_points, 64 * q.n_fresh,
                                    cudaMemcpyHostToDevice, st);
            if (q.n_pool && e == cudaSuccess)
                e = cudaMemcpyAsync(d_src + poff, q.pool_idx, 4 * q.n_pool, cudaMemcpyHostToDevice, st);
        }
        s.h_seg.push_back(make_uint4((uint32_t)off, (uint32_t)poff, (uint32_t)q.n_pool, 0u));
        off += n;
        poff += q.n_pool;
    }
    if (total_pool && ctx.pageable_access)
        pull_add(s.h_pull, d_seg, s.h_seg.data(), 16 * s.h_seg.size());
    if (e == cudaSuccess)
        e = pull_list(ctx, s.h_pull.data(), s.h_pull.size(), st);
    if (total_pool && e == cudaSuccess) {
        if (!ctx.pageable_access)
            e = cudaMemcpyAsync(d_seg, s.h_seg.data(), 16 * s.h_seg.size(), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) {
            k_gather_pool<<<(unsigned)((total_pool + 255) / 256), 256, 0, st>>>(
                S.pools[curve].d, d_src, d_seg, (uint32_t)s.h_seg.size(), (uint32_t)total_pool, (uint4 *)d_pts);
            ctx.launches++;
            e = cudaGetLastError();
        }
    }
    if (e != cudaSuccess) {
        ctx.last_error = std::string("staging: ") + cudaGetErrorString(e);
        return fail_staged(S, s, batch, HS_ECUDA);
    }
    b.scalars = (const uint32_t *)d_sc;
    b.points = (const uint4 *)d_pts;
    if (execute_batch(ctx, p, b, d_out, S.cfg.out_fmt) != HS_OK)
        return fail_staged(S, s, batch, HS_ECUDA);
    e = cudaMemcpyAsync(s.pinned_out, d_out, batch.size() * ob, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess)
        e = cudaEventRecord(s.done, st);
    if (e != cudaSuccess) {
        ctx.last_error = std::string("result copy: ") + cudaGetErrorString(e);
        return fail_staged(S, s, batch, HS_ECUDA);
    }
    finish_launch(S, s, batch, curve, bytes);
    return true;
}

static void retire(Server &S, Slot &s, cudaError_t status)
{
    const size_t ob = fmt_bytes(S.cfg.out_fmt);
    const auto now = Clock::now();
    for (size_t j = 0; j < s.tickets.size(); j++) {
        auto it = S.reqs.find(s.tickets[j]);
        if (it == S.reqs.end())
            continue;
        ReqState &r = it->second;
        if (status == cudaSuccess) {
            std::memcpy(r.req.out, s.pinned_out + j * ob, ob);
            r.status = HS_OK;
            S.stats.completed++;
        } else {
            r.status = HS_ECUDA;
            S.stats.failed++;
        }
        r.latency_ms = std::chrono::duration<double, std::milli>(now - r.submitted).count();
    }
    if (status != cudaSuccess)
        S.last_error = std::string("batch: ") + cudaGetErrorString(status);
    S.in_flight -= s.bytes;
    s.bytes = 0;
    s.busy = false;
    s.tickets.clear();
    S.cv_done.notify_all();
}

static void scheduler(Server *Sp)
{
    Server &S = *Sp;
    cudaSetDevice(S.cfg.device);
    std::unique_lock<std::mutex> lk(S.mu);
    while (true) {
        bool progress = false;
        for (auto &sp : S.slots) {
            Slot &s = *sp;
            if (!s.busy)
                continue;
            const cudaError_t q = cudaEventQuery(s.done);
            if (q == cudaErrorNotReady)
                continue;
            if (q != cudaSuccess)
                cudaGetLastError();
            retire(S, s, q);
            progress = true;
        }
        if (S.stop) {
            bool any = false;
            for (auto &sp : S.slots)
                any = any || sp->busy;
            if (!any)
                break;
        }
        while (!S.stop && !S.queue.empty()) {
            Slot *free_slot = nullptr;
            for (auto &sp : S.slots)
                if (!sp->busy) {
                    free_slot = sp.get();
                    break;
                }
            if (!free_slot)
                break;
            // the oldest request decides the curve and the form (pool table or
            // not); take queued requests of both, FIFO, up to the caps
            const int curve = S.reqs[S.queue.front()].req.curve;
            const bool form = S.reqs[S.queue.front()].table;
            std::vector<uint64_t> batch;
            size_t pts = 0;
            uint64_t ent = 0;
            std::deque<uint64_t> rest;
            while (!S.queue.empty()) {
                const uint64_t t = S.queue.front();
                S.queue.pop_front();
                const ReqState &r = S.reqs[t];
                if (r.req.curve == curve && r.table == form && batch.size() < S.cfg.max_batch_msms &&
                    (batch.empty() || (pts + r.n <= S.cfg.max_batch_points && ent + r.entries <= BATCH_ENTRIES_MAX))) {
                    batch.push_back(t);
                    pts += r.n;
                    ent += r.entries;
                } else {
                    rest.push_back(t);
                }
            }
            S.queue.swap(rest);
            if (!launch(S, *free_slot, batch, curve)) {
                // over budget: put the batch back at the front and wait for a completion
                for (auto it = batch.rbegin(); it != batch.rend(); ++it)
                    S.queue.push_front(*it);
                break;
            }
            progress = true;
        }
        if (!progress) {
            bool busy = false;
            for (auto &sp : S.slots)
                busy = busy || sp->busy;
            // poll the device every 50 us while batches are in flight, otherwise sleep until work arrives
            S.cv_work.wait_for(lk, busy ? std::chrono::microseconds(50) : std::chrono::milliseconds(20));
        }
    }
    // fail what is still queued
    for (uint64_t t : S.queue) {
        S.reqs[t].status = HS_EBUSY;
        S.stats.failed++;
    }
    S.queue.clear();
    S.cv_done.notify_all();
}

}  // namespace hs

using namespace hs;

struct hs_server {
    Server s;
};

extern "C" {

int hs_server_create(hs_server **out, const hs_server_config *cfg)
{
    if (!out || !cfg)
        return HS_EINVAL;
    *out = nullptr;
    if (cfg->out_fmt < HS_FMT_JACOBIAN51 || cfg->out_fmt > HS_FMT_COMPRESSED || cfg->slots < 0 || cfg->slots > 16)
        return HS_EINVAL;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || cfg->device < 0 || cfg->device >= count) {
        cudaGetLastError();
        return HS_EINVAL;
    }
    std::unique_ptr<hs_server> h(new (std::nothrow) hs_server());
    if (!h)
        return HS_ENOMEM;
    Server &S = h->s;
    S.cfg = *cfg;
    if (S.cfg.slots == 0)
        S.cfg.slots = 4;
    if (S.cfg.max_batch_points == 0)
        S.cfg.max_batch_points = size_t(1) << 22;
    if (S.cfg.max_batch_msms == 0)
        S.cfg.max_batch_msms = 1024;
    DeviceGuard g(S.cfg.device);
    if (S.cfg.hbm_budget == 0) {
        size_t fr = 0, tot = 0;
        if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
            cudaGetLastError();
            return HS_ECUDA;
        }
        S.cfg.hbm_budget = fr / 2;
    }
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, S.cfg.device);
    if (sort_smem_attrs(S.cfg.device) != cudaSuccess) {
        cudaGetLastError();
        return HS_ECUDA;
    }
    int pools = 0, pageable = 0;
    cudaDeviceGetAttribute(&pools, cudaDevAttrMemoryPoolsSupported, S.cfg.device);
    cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, S.cfg.device);
    for (int i = 0; i < S.cfg.slots; i++) {
        auto sl = std::make_unique<Slot>();
        sl->ctx.device = S.cfg.device;
        sl->ctx.sm_count = sms;
        sl->ctx.pageable_access = pageable == 1;
        sl->ctx.use_graphs = false;  // request shapes rarely repeat
        if (cudaStreamCreateWithFlags(&sl->ctx.stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&sl->done, cudaEventDisableTiming) != cudaSuccess) {
            cudaGetLastError();
            return HS_ECUDA;
        }
        // a slot's workspace grows in its own stream's order: a larger batch on
        // one slot does not stall the batches in flight on the others
        if (pools)
            sl->ctx.arena.ordered = sl->ctx.stream;
        S.slots.push_back(std::move(sl));
    }
    S.thr = std::thread(scheduler, &S);
    *out = h.release();
    return HS_OK;
}

int hs_server_set_pool(hs_server *h, int curve, const void *pts, size_t n)
{
    if (!h || (curve != HS_HELIOS && curve != HS_SELENE) || (n && !pts) || n >= 0x80000000ull)
        return HS_EINVAL;
    Server &S = h->s;
    std::lock_guard<std::mutex> lk(S.mu);
    for (auto &sp : S.slots)
        if (sp->busy || !S.queue.empty())
            return HS_EBUSY;  // replace pools only while idle
    DeviceGuard g(S.cfg.device);
    Pool &p = S.pools[curve];
    if (p.d)
        cudaFree(p.d);
    if (p.table)
        cudaFree(p.table);
    p.d = p.table = nullptr;
    p.n = 0;
    p.c = 0;
    p.W = 0;
    p.gen++;
    if (!n)
        return HS_OK;
    if (cudaMalloc((void **)&p.d, n * 64) != cudaSuccess) {
        cudaGetLastError();
        p.d = nullptr;
        return HS_ENOMEM;
    }
    if (cudaMemcpy(p.d, pts, n * 64, cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaGetLastError();
        return HS_ECUDA;
    }
    const int c = p.window < 0 ? POOL_WINDOW_AUTO : p.window;
    if (c) {
        // the table of window multiples, built with the first slot's context
        // (idle: pools are replaced only while nothing is queued or in flight)
        const uint32_t W = (uint32_t)((257 + c - 1) / c);
        const size_t m = n * W;
        if (m >= 0x80000000ull)
            return HS_ERANGE;
        Context &ctx = S.slots[0]->ctx;
        if (cudaMalloc((void **)&p.table, m * 64) != cudaSuccess) {
            cudaGetLastError();
            p.table = nullptr;
            return HS_ENOMEM;
        }
        cudaError_t e = ctx.arena.reserve(align256(m * 160) + 1024);
        uint4 *d_tmp = e == cudaSuccess ? (uint4 *)ctx.arena.take(m * 160) : nullptr;
        if (e == cudaSuccess && !d_tmp)
            e = cudaErrorMemoryAllocation;
        if (e == cudaSuccess)
            e = curve_ops(curve).fixed_table(ctx, p.d, n, c, (int)W, d_tmp, p.table);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(ctx.stream);
        ctx.arena.release();  // the build's scratch is not kept as the slot's workspace
        if (e != cudaSuccess) {
            cudaGetLastError();
            cudaFree(p.table);
            p.table = nullptr;
            S.last_error = std::string("pool table: ") + cudaGetErrorString(e);
            return e == cudaErrorMemoryAllocation ? HS_ENOMEM : HS_ECUDA;
        }
        p.c = c;
        p.W = W;
    }
    p.n = n;
    return HS_OK;
}

int hs_server_set_pool_window(hs_server *h, int curve, int window)
{
    if (!h || (curve != HS_HELIOS && curve != HS_SELENE) || (window != 0 && (window < 4 || window > 16)))
        return HS_EINVAL;
    Server &S = h->s;
    std::lock_guard<std::mutex> lk(S.mu);
    S.pools[curve].window = window;
    return HS_OK;
}

int hs_server_set_window(hs_server *h, int curve, size_t n_min, size_t n_max, int window)
{
    if (!h || (curve != HS_HELIOS && curve != HS_SELENE) || n_min > n_max ||
        (window != 0 && (window < 4 || window > 20)))
        return HS_EINVAL;
    Server &S = h->s;
    std::lock_guard<std::mutex> lk(S.mu);  // batches are planned under this lock
    for (auto &sp : S.slots) {
        auto &rules = sp->ctx.rules[curve == HS_SELENE ? 1 : 0];
        if (window == 0)
            rules.clear();
        else
            rules.push_back(WindowRule{n_min, n_max, window});
    }
    return HS_OK;
}

int hs_server_submit(hs_server *h, const hs_request *req, uint64_t *ticket)
{
    if (!h || !req || !ticket || (req->curve != HS_HELIOS && req->curve != HS_SELENE) || !req->out)
        return HS_EINVAL;
    const size_t n = req->n_pool + req->n_fresh;
    if ((n && !req->scalars) || (req->n_pool && !req->pool_idx) || (req->n_fresh && !req->fresh_points))
        return HS_EINVAL;
    Server &S = h->s;
    if (n > S.cfg.max_batch_points)
        return HS_ERANGE;
    // the indices are checked without the lock (the scheduler keeps running),
    // against the pool size of a generation that is still current when queued
    std::unique_lock<std::mutex> lk(S.mu);
    if (S.stop)
        return HS_EBUSY;
    while (req->n_pool) {
        const Pool &p = S.pools[req->curve];
        const size_t pool_n = p.n;
        const uint64_t gen = p.gen;
        lk.unlock();
        for (size_t j = 0; j < req->n_pool; j++)
            if (req->pool_idx[j] >= pool_n)
                return HS_EINVAL;
        lk.lock();
        if (S.stop)
            return HS_EBUSY;
        if (S.pools[req->curve].gen == gen)
            break;
    }
    const uint64_t entries = request_entries(S, *req);
    if (entries > BATCH_ENTRIES_MAX)
        return HS_ERANGE;
    const uint64_t t = S.next_ticket++;
    ReqState &r = S.reqs[t];
    r.req = *req;
    r.n = n;
    r.table = table_form(S, *req);
    r.entries = entries;
    r.submitted = Clock::now();
    S.queue.push_back(t);
    S.stats.submitted++;
    *ticket = t;
    S.cv_work.notify_one();
    return HS_OK;
}

int hs_server_wait(hs_server *h, uint64_t ticket, int timeout_ms, double *latency_ms)
{
    if (!h)
        return HS_EINVAL;
    Server &S = h->s;
    std::unique_lock<std::mutex> lk(S.mu);
    auto it = S.reqs.find(ticket);
    if (it == S.reqs.end())
        return HS_EINVAL;
    const auto deadline = Clock::now() + std::chrono::milliseconds(std::max(0, timeout_ms));
    while (it->second.status == 1) {
        if (S.cv_done.wait_until(lk, deadline) == std::cv_status::timeout && it->second.status == 1)
            return HS_ETIMEDOUT;
        it = S.reqs.find(ticket);
        if (it == S.reqs.end())
            return HS_EINVAL;
    }
    const int st = it->second.status;
    if (latency_ms)
        *latency_ms = it->second.latency_ms;
    S.reqs.erase(it);
    return st;
}

int hs_server_get_stats(hs_server *h, hs_server_stats *st)
{
    if (!h || !st)
        return HS_EINVAL;
    std::lock_guard<std::mutex> lk(h->s.mu);
    *st = h->s.stats;
    return HS_OK;
}

void hs_server_destroy(hs_server *h)
{
    if (!h)
        return;
    Server &S = h->s;
    {
        std::lock_guard<std::mutex> lk(S.mu);
        S.stop = true;
        S.cv_work.notify_all();
    }
    if (S.thr.joinable())
        S.thr.join();
    {
        DeviceGuard g(S.cfg.device);
        for (auto &sp : S.slots) {
            Slot &s = *sp;
            cudaStreamSynchronize(s.ctx.stream);
            drop_graphs(s.ctx);
            s.ctx.arena.release();
            cudaStreamDestroy(s.ctx.stream);
            cudaEventDestroy(s.done);
            if (s.pinned_out)
                cudaFreeHost(s.pinned_out);
        }
        for (Pool &p : S.pools) {
            if (p.d)
                cudaFree(p.d);
            if (p.table)
                cudaFree(p.table);
        }
    }
    delete h;
}

}  // extern "C"
