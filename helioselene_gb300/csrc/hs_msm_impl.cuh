// hs_msm_impl.cuh -- curve-templated device kernels of the MSM path.
//
// Pipeline of one MSM (n points, c-bit signed windows, W = ceil(257/c) windows,
// B = 2^(c-1) buckets per window), following the reference Pippenger
// (helios/src/x64/helios_msm_vartime.cpp:265-388) but laid out for the GPU:
//   1. recode + counting sort (hs_runtime.cu): every (point, window) with a
//      nonzero digit becomes one entry "point index | sign" placed
//      contiguously per bucket;
//   2. k_accumulate: buckets are cut into segments of at most L entries, one
//      thread sums one segment of affine bases into an XYZZ point;
//   3. k_merge_light / k_merge_heavy: buckets with several segments are folded
//      (sequentially when few, by a block-wide tree when many);
//   4. k_reduce_groups / k_window_chunks / k_window_sum: per window
//      S = sum_j (j+1) B_j by running sums over groups of 8 buckets, then
//      suffix scans and trees over the groups (no scalar multiples);
//   5. k_combine: Horner over the windows, S = 2^c S + S_k (the reference's
//      per-window doublings, :285-289) on one warp, result as canonical Jacobian.
#pragma once

#include "hs_curve.cuh"
#include "hs_internal.h"

namespace hs {

// ---------------------------------------------------------------------------
// memory helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ void load_affine(const uint4 *__restrict__ pts, uint32_t idx, Fe &x, Fe &y)
{
    const uint4 *p = pts + 4 * (size_t)idx;
    uint4 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2), d = __ldg(p + 3);
    x.w[0] = a.x; x.w[1] = a.y; x.w[2] = a.z; x.w[3] = a.w;
    x.w[4] = b.x; x.w[5] = b.y; x.w[6] = b.z; x.w[7] = b.w;
    y.w[0] = c.x; y.w[1] = c.y; y.w[2] = c.z; y.w[3] = c.w;
    y.w[4] = d.x; y.w[5] = d.y; y.w[6] = d.z; y.w[7] = d.w;
}

__device__ __forceinline__ void store_fe(uint4 *o, const Fe &f)
{
    o[0] = make_uint4(f.w[0], f.w[1], f.w[2], f.w[3]);
    o[1] = make_uint4(f.w[4], f.w[5], f.w[6], f.w[7]);
}

__device__ __forceinline__ Fe load_fe(const uint4 *o)
{
    Fe f;
    uint4 a = o[0], b = o[1];
    f.w[0] = a.x; f.w[1] = a.y; f.w[2] = a.z; f.w[3] = a.w;
    f.w[4] = b.x; f.w[5] = b.y; f.w[6] = b.z; f.w[7] = b.w;
    return f;
}

__device__ __forceinline__ void store_xyzz(uint4 *o, const Xyzz &p)
{
    store_fe(o, p.X);
    store_fe(o + 2, p.Y);
    store_fe(o + 4, p.ZZ);
    store_fe(o + 6, p.ZZZ);
}

__device__ __forceinline__ Xyzz load_xyzz(const uint4 *o)
{
    Xyzz p;
    p.X = load_fe(o);
    p.Y = load_fe(o + 2);
    p.ZZ = load_fe(o + 4);
    p.ZZZ = load_fe(o + 6);
    return p;
}

// ---------------------------------------------------------------------------
// 2. bucket accumulation: one thread per segment of <= L entries (segments come
//    longest first, so the lanes of a warp do equal work).  The launch takes the
//    descriptors [*seg_lo, *seg_hi) (device values: one list, or one part of
//    host inputs in two parts); with RESUME, a descriptor with d.w set
//    continues the sum stored in its slot by the earlier part.
// ---------------------------------------------------------------------------
template <class C, bool RESUME>
__global__ void __launch_bounds__(128) k_accumulate(const uint4 *__restrict__ segs, const uint32_t *__restrict__ seg_lo,
                                                   const uint32_t *__restrict__ seg_hi,
                                                   const uint32_t *__restrict__ sorted, const uint4 *__restrict__ pts,
                                                   uint4 *__restrict__ seg_sum)
{
    using G = Group<C>;
    using F = typename C::F;
    const uint32_t S0 = *seg_lo, S = *seg_hi;
    for (uint32_t s = S0 + blockIdx.x * blockDim.x + threadIdx.x; s < S; s += gridDim.x * blockDim.x) {
        const uint4 d = segs[s];  // start, length, destination slot, continue
        Xyzz acc = (RESUME && d.w) ? load_xyzz(seg_sum + 8 * (size_t)d.z) : G::inf();
        for (uint32_t i = 0; i < d.y; i++) {
            const uint32_t e = __ldg(sorted + d.x + i);
            Fe x, y;
            load_affine(pts, e & 0x7fffffffu, x, y);
            if (F::is_exact_zero(x) && F::is_exact_zero(y))
                continue;  // identity base (the reference's Z == 0 input) contributes nothing
            if (e >> 31)
                y = F::neg(y);
            G::add_affine(acc, x, y);
        }
        store_xyzz(seg_sum + 8 * (size_t)d.z, acc);
    }
}

// ---------------------------------------------------------------------------
// 2'. batch-affine bucket accumulation (plans with ba_rounds = R > 0)
// ---------------------------------------------------------------------------
// Every bucket's entry list is padded to a multiple of 2^R (padding entries are
// PAD_ENTRY, the identity), so the lists of every round start at even
// positions.  Round r then adds the items of the previous level in flat pairs:
// output q = item 2q + item 2q+1 (round 1: entries, later: affine sums), by
//     lambda = (y_b - y_a) / (x_b - x_a)   (doubling: (3 x_a^2 - 3) / (2 y_a)),
//     x = lambda^2 - x_a - x_b,  y = lambda (x_a - x) - y_a,
// and bucket k's round-r list is [off_k >> r, off_{k+1} >> r) with no scan:
// a round is a pure stream over the level, every warp reading 32 consecutive
// pairs.  The divisions of a round share inversions by Montgomery's trick
// (fp/include/fp_batch_invert.h:61-114 applied across a wave of additions):
//   k_ba_pairs   lane l of warp tile w takes outputs w*32K + l + 32k (k < K):
//                denominators, their running product (each output's exclusive
//                prefix is stored), then a product tree over the block's
//                threads; the block total goes out and each thread keeps its
//                co-product (the product of the other threads' totals);
//   k_ba_invert  one inversion per block total (BA_K * BA_BT additions);
//   k_ba_finish  1/T_t = inv(block) * co-product, then each output walks back:
//                1/d = (1/prefix through d) * (prefix before d), and the sum.
// Pairs with equal x double (d = 2 y_a) or cancel (the identity, d = 1); an
// identity operand (affine (0,0), or a padding entry) takes d = 1 and the
// other operand is copied.  The last round's sums are folded into XYZZ bucket
// sums by k_accumulate_level.
constexpr int BA_K = (int)BA_PLAN_K;    // outputs per thread
constexpr int BA_BT = (int)BA_PLAN_BT;  // threads per block: one shared inversion per BA_K * BA_BT outputs
constexpr uint32_t PAD_ENTRY = 0xffffffffu;

enum BaKind : int { BA_ADD, BA_DBL, BA_COPY_A, BA_COPY_B, BA_ZERO };

__device__ __forceinline__ Fe ba_ld(const uint4 *p)
{
    const uint4 a = __ldg(p), b = __ldg(p + 1);
    Fe f;
    f.w[0] = a.x; f.w[1] = a.y; f.w[2] = a.z; f.w[3] = a.w;
    f.w[4] = b.x; f.w[5] = b.y; f.w[6] = b.z; f.w[7] = b.w;
    return f;
}

// Where item i of a round's input lives: round 1 reads entry i (point index |
// sign << 31; PAD_ENTRY is the identity, src null), later rounds the previous
// level's affine sum i.
template <bool FIRST>
__device__ __forceinline__ const uint4 *ba_src(uint32_t e, const uint4 *__restrict__ pts,
                                              const uint4 *__restrict__ lvl, uint32_t i, bool &neg)
{
    if (FIRST) {
        neg = (e >> 31) != 0;
        return e == PAD_ENTRY ? nullptr : pts + 4 * (size_t)(e & 0x7fffffffu);
    }
    neg = false;
    return lvl + 4 * (size_t)i;
}

// y of an item (negated for a negative round-1 digit; the identity left (0,0))
template <class C>
__device__ __forceinline__ Fe ba_load_y(const uint4 *src, bool neg, const Fe &x)
{
    using F = typename C::F;
    const Fe y = ba_ld(src + 2);
    return (neg && !(F::is_exact_zero(x) && F::is_exact_zero(y))) ? F::neg(y) : y;
}

// Kind and denominator of output q (items 2q and 2q+1).  With FULL every
// coordinate is loaded (for the sum); without, a y coordinate only when the
// case needs it (identity check, equal x).
template <class C, bool FIRST, bool FULL>
__device__ __forceinline__ int ba_item(const uint32_t *__restrict__ sorted, const uint4 *__restrict__ pts,
                                       const uint4 *__restrict__ lvl, uint32_t q, Fe &xa, Fe &ya, Fe &xb, Fe &yb,
                                       Fe &d)
{
    using F = typename C::F;
    uint32_t ea = 0, eb = 0;
    if (FIRST) {
        const uint2 e = __ldg(reinterpret_cast<const uint2 *>(sorted) + q);
        ea = e.x;
        eb = e.y;
    }
    bool na, nb;
    const uint4 *sa = ba_src<FIRST>(ea, pts, lvl, 2 * q, na);
    const uint4 *sb = ba_src<FIRST>(eb, pts, lvl, 2 * q + 1, nb);
    d = F::one();
    xa = sa ? ba_ld(sa) : F::zero();
    xb = sb ? ba_ld(sb) : F::zero();
    const bool xa0 = F::is_exact_zero(xa), xb0 = F::is_exact_zero(xb);
    ya = (sa && (FULL || xa0)) ? ba_load_y<C>(sa, na, xa) : F::zero();
    yb = (sb && (FULL || xb0)) ? ba_load_y<C>(sb, nb, xb) : F::zero();
    if (xb0 && F::is_exact_zero(yb))
        return BA_COPY_A;  // b is the identity
    if (xa0 && F::is_exact_zero(ya))
        return BA_COPY_B;  // a is the identity
    const Fe dx = F::sub(xb, xa);
    if (F::is_zero(dx)) {
        if (!FULL) {
            ya = ba_load_y<C>(sa, na, xa);
            yb = ba_load_y<C>(sb, nb, xb);
        }
        if (!F::is_zero(F::sub(yb, ya)) || F::is_zero(ya))
            return BA_ZERO;  // b = -a (or a point of order 2, which doubles to the identity)
        d = F::dbl(ya);  // b = a: double
        return BA_DBL;
    }
    d = dx;
    return BA_ADD;
}

// first output of this thread's warp tile, plus its lane (outputs base + 32 k),
// in a launch over outputs [E0, E)
__device__ __forceinline__ uint64_t ba_tile_base(uint32_t E0)
{
    const uint64_t tile = (uint64_t)blockIdx.x * (BA_BT / 32) + (threadIdx.x >> 5);
    return E0 + tile * 32 * BA_K + (threadIdx.x & 31);
}

// A launch covers round r's outputs [*lo >> r, *hi >> r) (lo null: from 0):
// the whole level, or the lists of one part of host inputs in two parts.
__device__ __forceinline__ uint32_t ba_first(const uint32_t *lo, uint32_t r) { return lo ? __ldg(lo) >> r : 0u; }

template <class C, bool FIRST>
__global__ void __launch_bounds__(BA_BT) k_ba_pairs(const uint32_t *__restrict__ lo, const uint32_t *__restrict__ hi,
                                                   uint32_t r, const uint32_t *__restrict__ sorted,
                                                   const uint4 *__restrict__ pts, const uint4 *__restrict__ lvl,
                                                   uint4 *__restrict__ pre, uint4 *__restrict__ co,
                                                   uint4 *__restrict__ tot)
{
    using F = typename C::F;
    __shared__ Fe tree[2 * BA_BT];
    __shared__ Fe cop[2 * BA_BT];
    const uint32_t E0 = ba_first(lo, r), E = __ldg(hi) >> r;  // outputs of this launch
    const uint32_t t = threadIdx.x;
    if (E0 + (uint64_t)blockIdx.x * BA_BT * BA_K >= E)
        return;  // the whole block is past the launch's outputs
    const uint64_t base = ba_tile_base(E0);
    Fe run = F::one();
    bool any = false;
#pragma unroll 1
    for (int k = 0; k < BA_K; k++) {
        const uint64_t q = base + 32 * (uint64_t)k;
        if (q >= E)
            break;
        Fe xa, ya, xb, yb, d;
        const int kind = ba_item<C, FIRST, false>(sorted, pts, lvl, (uint32_t)q, xa, ya, xb, yb, d);
        if (kind == BA_ADD || kind == BA_DBL) {
            store_fe(pre + 2 * q, run);  // exclusive prefix of this output (1 for the first)
            run = any ? F::mul(run, d) : d;
            any = true;
        }
    }
    // product tree over the block's thread totals (leaf t at BA_BT + t)
    tree[BA_BT + t] = run;
    __syncthreads();
    for (uint32_t s2 = BA_BT / 2; s2 >= 1; s2 >>= 1) {
        if (t < s2)
            tree[s2 + t] = F::mul(tree[2 * (s2 + t)], tree[2 * (s2 + t) + 1]);
        __syncthreads();
    }
    // co-products top-down: cop[node] = product of all leaves outside node's subtree
    if (t == 0)
        cop[1] = F::one();
    __syncthreads();
    for (uint32_t s2 = 1; s2 < BA_BT; s2 <<= 1) {
        if (t < s2) {
            const uint32_t nd = s2 + t;
            const Fe c = cop[nd];
            cop[2 * nd] = F::mul(c, tree[2 * nd + 1]);
            cop[2 * nd + 1] = F::mul(c, tree[2 * nd]);
        }
        __syncthreads();
    }
    store_fe(co + 2 * ((size_t)blockIdx.x * BA_BT + t), cop[BA_BT + t]);
    if (t == 0)
        store_fe(tot + 2 * (size_t)blockIdx.x, tree[1]);
}

// one inversion per block total (a block total is never zero: every factor is)
template <class C>
__global__ void k_ba_invert(const uint32_t *__restrict__ lo, const uint32_t *__restrict__ hi, uint32_t r,
                            const uint4 *__restrict__ tot, uint4 *__restrict__ inv)
{
    using F = typename C::F;
    const uint32_t E0 = ba_first(lo, r), E = __ldg(hi) >> r;
    const uint32_t nblk = (uint32_t)(((uint64_t)(E - E0) + BA_BT * BA_K - 1) / (BA_BT * BA_K));
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nblk)
        return;
    store_fe(inv + 2 * (size_t)i, F::inv(load_fe(tot + 2 * (size_t)i)));
}

template <class C, bool FIRST>
__global__ void __launch_bounds__(BA_BT) k_ba_finish(const uint32_t *__restrict__ lo, const uint32_t *__restrict__ hi,
                                                    uint32_t r, const uint32_t *__restrict__ sorted,
                                                    const uint4 *__restrict__ pts, const uint4 *__restrict__ lvl,
                                                    const uint4 *__restrict__ pre, const uint4 *__restrict__ co,
                                                    const uint4 *__restrict__ inv, uint4 *__restrict__ out)
{
    using F = typename C::F;
    const uint32_t E0 = ba_first(lo, r), E = __ldg(hi) >> r;
    const uint64_t base = ba_tile_base(E0);
    if (base >= E)
        return;
    // 1 / (this thread's total)
    Fe inv_run = F::mul(load_fe(inv + 2 * (size_t)blockIdx.x),
                        load_fe(co + 2 * ((size_t)blockIdx.x * BA_BT + threadIdx.x)));
    const int kmax = (int)((E - 1 - base) / 32) < BA_K - 1 ? (int)((E - 1 - base) / 32) : BA_K - 1;
#pragma unroll 1
    for (int k = kmax; k >= 0; k--) {
        const uint64_t q = base + 32 * (uint64_t)k;
        Fe xa, ya, xb, yb, d;
        const int kind = ba_item<C, FIRST, true>(sorted, pts, lvl, (uint32_t)q, xa, ya, xb, yb, d);
        Fe x3, y3;
        if (kind == BA_ADD || kind == BA_DBL) {
            const Fe inv_d = F::mul(inv_run, load_fe(pre + 2 * q));
            inv_run = F::mul(inv_run, d);
            Fe num;
            if (kind == BA_ADD) {
                num = F::sub(yb, ya);
            } else {
                const Fe t = F::sub(F::sqr(xa), F::one());
                num = F::add(F::dbl(t), t);  // 3 x^2 + a, a = -3
                xb = xa;
            }
            const Fe lam = F::mul(num, inv_d);
            x3 = F::sub(F::sub(F::sqr(lam), xa), xb);
            y3 = F::sub(F::mul(lam, F::sub(xa, x3)), ya);
        } else if (kind == BA_COPY_A) {
            x3 = xa;
            y3 = ya;
        } else if (kind == BA_COPY_B) {
            x3 = xb;
            y3 = yb;
        } else {
            x3 = F::zero();
            y3 = F::zero();
        }
        uint4 *dst = out + 4 * q;
        store_fe(dst, x3);
        store_fe(dst + 2, y3);
    }
}

// The batch-affine rounds' last sums, folded per segment into XYZZ bucket sums
// (segments of a bucket's list in the last level buffer, longest first, as in
// k_accumulate; the items are affine points, (0,0) the identity).  With
// RESUME (part 1 of host inputs in two parts), a descriptor with d.w set
// continues the sum stored in its slot by part 0.
template <class C, bool RESUME>
__global__ void __launch_bounds__(128) k_accumulate_level(const uint4 *__restrict__ segs,
                                                         const uint32_t *__restrict__ seg_lo,
                                                         const uint32_t *__restrict__ seg_hi,
                                                         const uint4 *__restrict__ lvl, uint4 *__restrict__ seg_sum)
{
    using G = Group<C>;
    using F = typename C::F;
    const uint32_t S0 = *seg_lo, S = *seg_hi;
    for (uint32_t s = S0 + blockIdx.x * blockDim.x + threadIdx.x; s < S; s += gridDim.x * blockDim.x) {
        const uint4 d = segs[s];  // start, length, destination slot, continue
        Xyzz acc = (RESUME && d.w) ? load_xyzz(seg_sum + 8 * (size_t)d.z) : G::inf();
        for (uint32_t i = 0; i < d.y; i++) {
            Fe x, y;
            load_affine(lvl, d.x + i, x, y);
            if (F::is_exact_zero(x) && F::is_exact_zero(y))
                continue;
            G::add_affine(acc, x, y);
        }
        store_xyzz(seg_sum + 8 * (size_t)d.z, acc);
    }
}

// Out-of-line point operations for the latency-bound level-2 reduction kernels
// (k_window_chunks, k_window_sum): with about one warp per scheduler their
// inlined copies overflow the instruction cache, while one shared body stays
// resident (a call costs a few dozen instructions next to the ~2000 of an
// addition).  The points cross the call by value.  A form that passed them by
// address (the caller's local memory, result stored after both operands were
// read) gave wrong sums on this toolchain for sm_103a, in every MSM, while
// this form has passed every parity test; the l2_add / l2_dbl wrappers keep
// the call sites in the by-address shape.
template <class C>
__device__ __noinline__ Xyzz l2_addv(const Xyzz a, const Xyzz b)
{
    return Group<C>::add(a, b);
}
template <class C>
__device__ __noinline__ Xyzz l2_dblv(const Xyzz a)
{
    return Group<C>::dbl(a);
}
template <class C>
__device__ __forceinline__ void l2_add(Xyzz *r, const Xyzz *a, const Xyzz *b)
{
    *r = l2_addv<C>(*a, *b);
}
template <class C>
__device__ __forceinline__ void l2_dbl(Xyzz *r, const Xyzz *a)
{
    *r = l2_dblv<C>(*a);
}

// ---------------------------------------------------------------------------
// 3. folding buckets that were cut into several segments
// ---------------------------------------------------------------------------
template <class C>
__global__ void k_merge_light(const uint32_t *__restrict__ seg_off, uint32_t NB, uint4 *__restrict__ seg_sum,
                              uint32_t *__restrict__ heavy, uint32_t *__restrict__ heavy_n, uint32_t heavy_min)
{
    using G = Group<C>;
    const uint32_t kb = blockIdx.x * blockDim.x + threadIdx.x;
    if (kb >= NB)
        return;
    const uint32_t s0 = seg_off[kb], ns = seg_off[kb + 1] - s0;
    if (ns < 2)
        return;
    if (ns > heavy_min) {
        heavy[atomicAdd(heavy_n, 1u)] = kb;
        return;
    }
    Xyzz acc = load_xyzz(seg_sum + 8 * (size_t)s0);
    for (uint32_t j = 1; j < ns; j++)
        acc = G::add(acc, load_xyzz(seg_sum + 8 * (size_t)(s0 + j)));
    store_xyzz(seg_sum + 8 * (size_t)s0, acc);
}

constexpr int HEAVY_THREADS = 128;

template <class C>
__global__ void __launch_bounds__(HEAVY_THREADS) k_merge_heavy(const uint32_t *__restrict__ seg_off,
                                                              const uint32_t *__restrict__ heavy,
                                                              const uint32_t *__restrict__ heavy_n,
                                                              uint4 *__restrict__ seg_sum)
{
    using G = Group<C>;
    __shared__ uint4 sh[HEAVY_THREADS * 8];
    const uint32_t cnt = *heavy_n;
    for (uint32_t h = blockIdx.x; h < cnt; h += gridDim.x) {
        const uint32_t kb = heavy[h];
        const uint32_t s0 = seg_off[kb], ns = seg_off[kb + 1] - s0;
        Xyzz acc = G::inf();
        for (uint32_t j = threadIdx.x; j < ns; j += HEAVY_THREADS)
            acc = G::add(acc, load_xyzz(seg_sum + 8 * (size_t)(s0 + j)));
        store_xyzz(sh + 8 * threadIdx.x, acc);
        __syncthreads();
        // the tree spans only the threads that hold a segment (a power of two)
        uint32_t width = 1;
        while (width < ns && width < HEAVY_THREADS)
            width <<= 1;
        for (uint32_t stride = width / 2; stride > 0; stride >>= 1) {
            if (threadIdx.x < stride) {
                Xyzz a = load_xyzz(sh + 8 * threadIdx.x);
                Xyzz b = load_xyzz(sh + 8 * (threadIdx.x + stride));
                store_xyzz(sh + 8 * threadIdx.x, G::add(a, b));
            }
            __syncthreads();
        }
        if (threadIdx.x == 0)
            store_xyzz(seg_sum + 8 * (size_t)s0, load_xyzz(sh));
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// 4. bucket reduction: S = sum_j (j+1) B_j per window, in two levels
// ---------------------------------------------------------------------------
// Level 1, k_reduce_groups: thread (k, t) owns the m0 buckets [t m0, (t+1) m0)
// of window k and runs the reference's top-down running sum over them
// (helios_msm_vartime.cpp:334-361), giving
//     run_t = sum_j B_j,   acc_t = sum_j (j - t m0 + 1) B_j,
// so that S = sum_t acc_t + m0 sum_t t run_t.
template <class C>
__global__ void __launch_bounds__(128, 4) k_reduce_groups(const uint32_t *__restrict__ seg_off,
                                                      const uint4 *__restrict__ seg_sum,
                                                      const MsmDesc *__restrict__ desc, uint32_t M, uint32_t G,
                                                      uint4 *__restrict__ out)
{
    using G_ = Group<C>;
    const uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= G)
        return;
    const uint32_t mi = find_msm(M, gid, [&](uint32_t k) { return desc[k].group_base; });
    const MsmDesc d = desc[mi];
    const uint32_t local = gid - d.group_base;
    const uint32_t k = local / d.T, t = local % d.T;
    const uint32_t m = d.m0;
    Xyzz run = G_::inf(), acc = G_::inf();
    for (int j = (int)((t + 1) * m) - 1; j >= (int)(t * m); j--) {
        const uint32_t kb = d.bucket_base + k * d.B + (uint32_t)j;
        const uint32_t s0 = seg_off[kb];
        if (seg_off[kb + 1] != s0)
            run = G_::add(run, load_xyzz(seg_sum + 8 * (size_t)s0));
        acc = G_::add(acc, run);
    }
    store_xyzz(out + 16 * (size_t)gid, acc);
    store_xyzz(out + 16 * (size_t)gid + 8, run);
}

// Level 2 spreads each window's T groups over chunks of up to RED_CHUNK groups,
// one block per chunk (k_window_chunks), then adds the chunks of a window
// (k_window_sum).  Both use one identity: for points x_0..x_{m-1},
//     sum_i i x_i = sum_{i >= 1} X_i,   X_i = sum_{j >= i} x_j,
// where the suffix sums X_i come from a scan over the threads of a block.
// Chunk b of window k (groups from t0 = b RED_CHUNK) yields
//     C_b = sum_t acc_t + m0 sum_t (t - t0) run_t,     R_b = sum_t run_t,
// and the window sum is S = sum_b C_b + m0 RED_CHUNK sum_b b R_b.  Each step
// is a short running sum, a log-depth scan or tree, and log2 of a power of two
// doublings: no scalar multiples by group index.
// Shared-memory points are stored word-group-major (uint4 c of thread i at
// c * N + i), so a warp's 16-byte accesses to one uint4 of consecutive threads
// fall in distinct banks.
__device__ __forceinline__ void st_fe_soa(uint4 *sh, uint32_t c, uint32_t i, uint32_t N, const Fe &f)
{
    sh[(2 * c) * N + i] = make_uint4(f.w[0], f.w[1], f.w[2], f.w[3]);
    sh[(2 * c + 1) * N + i] = make_uint4(f.w[4], f.w[5], f.w[6], f.w[7]);
}

__device__ __forceinline__ Fe ld_fe_soa(const uint4 *sh, uint32_t c, uint32_t i, uint32_t N)
{
    const uint4 a = sh[(2 * c) * N + i], b = sh[(2 * c + 1) * N + i];
    Fe f;
    f.w[0] = a.x; f.w[1] = a.y; f.w[2] = a.z; f.w[3] = a.w;
    f.w[4] = b.x; f.w[5] = b.y; f.w[6] = b.z; f.w[7] = b.w;
    return f;
}

__device__ __forceinline__ void st_soa(uint4 *sh, uint32_t i, uint32_t N, const Xyzz &p)
{
    st_fe_soa(sh, 0, i, N, p.X);
    st_fe_soa(sh, 1, i, N, p.Y);
    st_fe_soa(sh, 2, i, N, p.ZZ);
    st_fe_soa(sh, 3, i, N, p.ZZZ);
}

__device__ __forceinline__ Xyzz ld_soa(const uint4 *sh, uint32_t i, uint32_t N)
{
    Xyzz p;
    p.X = ld_fe_soa(sh, 0, i, N);
    p.Y = ld_fe_soa(sh, 1, i, N);
    p.ZZ = ld_fe_soa(sh, 2, i, N);
    p.ZZZ = ld_fe_soa(sh, 3, i, N);
    return p;
}

// inclusive suffix scan of r over the first nt threads (sh holds N points)
template <class C>
__device__ __forceinline__ Xyzz block_suffix_scan(uint4 *sh, uint32_t N, Xyzz r, uint32_t i, uint32_t nt)
{
    using G = Group<C>;
    st_soa(sh, i, N, r);
    __syncthreads();
    for (uint32_t dl = 1; dl < nt; dl <<= 1) {
        Xyzz o = G::inf();
        const bool take = i + dl < nt;
        if (take)
            o = ld_soa(sh, i + dl, N);
        __syncthreads();
        if (take) {
            l2_add<C>(&r, &r, &o);
            st_soa(sh, i, N, r);
        }
        __syncthreads();
    }
    return r;
}

// sum of v over the first nt (a power of two) threads, result at index 0
template <class C>
__device__ __forceinline__ void block_tree_sum(uint4 *sh, uint32_t N, const Xyzz &v, uint32_t i, uint32_t nt)
{
    using G = Group<C>;
    __syncthreads();
    st_soa(sh, i, N, v);
    __syncthreads();
    for (uint32_t stride = nt / 2; stride > 0; stride >>= 1) {
        if (i < stride) {
            Xyzz x = ld_soa(sh, i, N), y = ld_soa(sh, i + stride, N);
            l2_add<C>(&x, &x, &y);
            st_soa(sh, i, N, x);
        }
        __syncthreads();
    }
}

// k_window_chunks: thread i of a chunk first runs a top-down running sum over
// its q consecutive groups (lo = t0 + i q):
//     r_i = sum run_t,  w_i = sum (t - lo) run_t,  a_i = sum acc_t,
// then the block scans r (X_i = sum_{j >= i} r_j) and thread i contributes
//     a_i + m0 (w_i + q X_i [i >= 1]),
// which sums to C_b; X_0 is R_b.  q = 4 groups per thread keeps both the
// sequential part and the scans' extra work small; in a plan of few windows
// (latency-bound) a window of at most 64 groups takes one per thread, so that
// only the scan is serial.
constexpr uint32_t RED_CHUNK_Q = 4;
constexpr uint32_t RED_CHUNK_THREADS = RED_CHUNK / RED_CHUNK_Q;

// DIRECT: every window of the batch is one chunk (T <= RED_CHUNK), so C_b is
// already the window sum and goes straight to S (k_window_sum is skipped).
template <class C, bool DIRECT>
__global__ void __launch_bounds__(RED_CHUNK_THREADS) k_window_chunks(const uint4 *__restrict__ in,
                                                                    const MsmDesc *__restrict__ desc, uint32_t M,
                                                                    uint4 *__restrict__ outC, int wide)
{
    using G = Group<C>;
    __shared__ uint4 sh[RED_CHUNK_THREADS * 8];
    const uint32_t ch = blockIdx.x, i = threadIdx.x;
    const uint32_t mi = find_msm(M, ch, [&](uint32_t k) { return desc[k].chunk_base; });
    const MsmDesc d = desc[mi];
    const uint32_t nbk = d.T > RED_CHUNK ? d.T / RED_CHUNK : 1;
    const uint32_t nt = d.T < RED_CHUNK ? d.T : RED_CHUNK;
    // groups per thread: RED_CHUNK_Q, or (wide: a plan of few windows, so
    // latency-bound) as few as fill the block, the scan taking the rest
    const uint32_t q = wide ? (nt > RED_CHUNK_THREADS ? nt / RED_CHUNK_THREADS : 1)
                            : (nt < RED_CHUNK_Q ? nt : RED_CHUNK_Q);
    const uint32_t P = nt / q;
    const uint32_t local = ch - d.chunk_base;
    const uint32_t k = local / nbk, b = local % nbk;
    Xyzz a = G::inf(), r = G::inf(), w = G::inf();
    if (i < P) {
        const size_t lo = (size_t)d.group_base + (size_t)k * d.T + (size_t)b * RED_CHUNK + (size_t)i * q;
        for (int u = (int)q - 1; u >= 0; u--) {
            Xyzz t = load_xyzz(in + 16 * (lo + u));
            l2_add<C>(&a, &a, &t);
            t = load_xyzz(in + 16 * (lo + u) + 8);
            l2_add<C>(&r, &r, &t);
            if (u > 0)
                l2_add<C>(&w, &w, &r);
        }
    }
    r = block_suffix_scan<C>(sh, RED_CHUNK_THREADS, r, i, P);
    Xyzz v = (i >= 1 && i < P) ? r : G::inf();
    for (uint32_t m = q; m > 1; m >>= 1)
        l2_dbl<C>(&v, &v);
    l2_add<C>(&v, &v, &w);
    for (uint32_t m = d.m0; m > 1; m >>= 1)
        l2_dbl<C>(&v, &v);
    l2_add<C>(&v, &v, &a);
    block_tree_sum<C>(sh, RED_CHUNK_THREADS, v, i, P);
    if (i == 0) {
        if (DIRECT) {
            store_xyzz(outC + 8 * (size_t)ch, ld_soa(sh, 0, RED_CHUNK_THREADS));
        } else {
            store_xyzz(outC + 16 * (size_t)ch, ld_soa(sh, 0, RED_CHUNK_THREADS));
            store_xyzz(outC + 16 * (size_t)ch + 8, r);  // thread 0's suffix sum is the chunk's run total
        }
    }
}

template <class C>
__global__ void __launch_bounds__(RED_CHUNK) k_window_sum(const uint4 *__restrict__ inC,
                                                         const MsmDesc *__restrict__ desc, uint32_t M,
                                                         uint4 *__restrict__ S)
{
    using G = Group<C>;
    __shared__ uint4 sh[RED_CHUNK * 8];
    const uint32_t s = blockIdx.x, i = threadIdx.x;
    const uint32_t mi = find_msm(M, s, [&](uint32_t k) { return desc[k].win_base; });
    const MsmDesc d = desc[mi];
    const uint32_t nbk = d.T > RED_CHUNK ? d.T / RED_CHUNK : 1;
    Xyzz cb = G::inf(), r = G::inf();
    if (i < nbk) {
        const size_t c = (size_t)d.chunk_base + (size_t)(s - d.win_base) * nbk + i;
        cb = load_xyzz(inC + 16 * c);
        r = load_xyzz(inC + 16 * c + 8);
    }
    r = block_suffix_scan<C>(sh, RED_CHUNK, r, i, nbk);
    Xyzz v = (i >= 1 && i < nbk) ? r : G::inf();
    for (uint32_t m = d.m0 * RED_CHUNK; m > 1 && nbk > 1; m >>= 1)
        l2_dbl<C>(&v, &v);
    l2_add<C>(&v, &v, &cb);
    block_tree_sum<C>(sh, RED_CHUNK, v, i, nbk);
    if (i == 0)
        store_xyzz(S + 8 * (size_t)s, ld_soa(sh, 0, RED_CHUNK));
}

// ---------------------------------------------------------------------------
// 5. window combination (Horner) -> canonical Jacobian
// ---------------------------------------------------------------------------
template <class C>
__device__ void store_jacobian_canon(uint32_t *out, const Xyzz &p)
{
    using G = Group<C>;
    using F = typename C::F;
    Fe X, Y, Z;
    G::to_jacobian(X, Y, Z, p);
    X = F::canon(X);
    Y = F::canon(Y);
    Z = F::canon(Z);
#pragma unroll
    for (int i = 0; i < 8; i++) {
        out[i] = X.w[i];
        out[8 + i] = Y.w[i];
        out[16 + i] = Z.w[i];
    }
}

// Lane-sliced field elements for the Horner chain.  The chain's 256
// doublings are sequential, so its time is the latency of one doubling.  In
// eight 32-bit limbs a product is about 180 multiply instructions of serial
// carry chains on one warp, bound by one scheduler's multiply pipe (about 525
// cycles on F_p, 870 on F_q).  Here an element is spread over a warp: lane
// l < 10 holds limb l of a radix-2^26 form (lanes 10..31 hold 0).  A product
// is formed column-wise -- lane l sums a_i b_(l-i) in a 64-bit register --
// then one carry step moves bits 26..51 of every column up one lane and bits
// 52.. up two, and the columns at and above 2^260 are folded back: on F_p by
// 2^260 == 608 (and 2^520 == 608^2); on F_q by a table of 2^(26(10+h)) mod q,
// then the two limbs that carried past 2^260 by 2^260 mod q = 32 gamma.
// Products come out with limbs below 2^27 (below 2^26 + 2^20 on F_p).
// Additions are limb-wise; a subtraction adds Z or 2Z, multiples of m whose
// limbs (Z: in [2^28, 1.25 * 2^28]) exceed every limb of the subtrahend.
// A product's inputs must keep every column below 2^64: with limbs below
// 2^30.1 and 2^29.8, ten products stay below 2^63.2.  Every function is
// called by all 32 lanes of a warp.
constexpr unsigned LF_ALL = 0xffffffffu;
constexpr uint64_t LF_M26 = (1ull << 26) - 1;

// Z = 129 p and 129 q in radix-2^26 limbs
static __constant__ uint32_t LF_Z[2][10] = {
    {0x13fff66du, 0x13fffffbu, 0x13fffffbu, 0x13fffffbu, 0x13fffffbu, 0x13fffffbu, 0x13fffffbu, 0x13fffffbu,
     0x13fffffbu, 0x101ffffbu},
    {0x110b971fu, 0x1002ebbfu, 0x1178fc9eu, 0x1221a868u, 0x137f3b8au, 0x13fffff3u, 0x13fffffbu, 0x13fffffbu,
     0x13fffffbu, 0x101ffffbu}};
// row h: 2^(26 (10 + h)) mod q in radix-2^26 limbs (row 0: 2^260 mod q = 32 gamma)
static __constant__ uint32_t LF_RQ[11][10] = {
            {0x3070c20u, 0x16c6c36u, 0x14f2292u, 0x1a44d4au, 0x01010fau, 0x0000002u, 0x0000000u, 0x0000000u, 0x0000000u, 0x0000000u},
            {0x0000000u, 0x3070c20u, 0x16c6c36u, 0x14f2292u, 0x1a44d4au, 0x01010fau, 0x0000002u, 0x0000000u, 0x0000000u, 0x0000000u},
            {0x0000000u, 0x0000000u, 0x3070c20u, 0x16c6c36u, 0x14f2292u, 0x1a44d4au, 0x01010fau, 0x0000002u, 0x0000000u, 0x0000000u},
            {0x0000000u, 0x0000000u, 0x0000000u, 0x3070c20u, 0x16c6c36u, 0x14f2292u, 0x1a44d4au, 0x01010fau, 0x0000002u, 0x0000000u},
            {0x0000000u, 0x0000000u, 0x0000000u, 0x0000000u, 0x3070c20u, 0x16c6c36u, 0x14f2292u, 0x1a44d4au, 0x01010fau, 0x0000002u},
            {0x20e1840u, 0x2d8d86du, 0x29e4524u, 0x3489a94u, 0x02021f4u, 0x3070c24u, 0x16c6c36u, 0x14f2292u, 0x1a44d4au, 0x01010fau},
            {0x09eb42du, 0x1f359fcu, 0x23798c8u, 0x17660e7u, 0x2f5edcbu, 0x0408471u, 0x3070c24u, 0x16c6c36u, 0x14f2292u, 0x0044d4au},
            {0x3a1550au, 0x24f5d25u, 0x36b84ebu, 0x121f2c1u, 0x1a54480u, 0x2fe99a7u, 0x0408471u, 0x3070c24u, 0x16c6c36u, 0x00f2292u},
            {0x2cb966bu, 0x248f1a0u, 0x0cf0f2fu, 0x10edbc3u, 0x1fe917eu, 0x1c3c66fu, 0x2fe99a7u, 0x0408471u, 0x3070c24u, 0x00c6c36u},
            {0x25f57d8u, 0x2f3ea03u, 0x1679a21u, 0x0c9df95u, 0x1650e8du, 0x2179bd1u, 0x1c3c66fu, 0x2fe99a7u, 0x0408471u, 0x0070c24u},
            {0x01fa542u, 0x0c733b9u, 0x04912c4u, 0x3c483d4u, 0x331e04fu, 0x1734323u, 0x2179bd1u, 0x1c3c66fu, 0x2fe99a7u, 0x0008471u},
};

template <class F>
struct LaneField {
    static constexpr bool FQ = F::Params::NC != 1;

    // this lane's constants, read once per thread
    struct Regs {
        uint32_t z, z2;   // limb `lane` of Z and 2Z (0 on lanes >= 10)
        uint32_t r[11];   // F_q: limb `lane` of row h of the fold table
        uint32_t k0, k1;  // F_q: limbs lane and lane - 1 of 2^260 mod q
    };
    __device__ __forceinline__ static Regs regs(int lane)
    {
        Regs g;
        const bool in = lane < 10;
        g.z = in ? LF_Z[FQ ? 1 : 0][in ? lane : 0] : 0u;
        g.z2 = 2 * g.z;
#pragma unroll
        for (int h = 0; h < 11; h++)
            g.r[h] = in ? LF_RQ[h][in ? lane : 0] : 0u;
        g.k0 = lane < 6 ? LF_RQ[0][lane < 6 ? lane : 0] : 0u;
        g.k1 = (lane >= 1 && lane <= 6) ? LF_RQ[0][(lane >= 1 && lane <= 6) ? lane - 1 : 0] : 0u;
        return g;
    }

    // bits 26..51 of every lane's value up one lane, bits 52.. up two
    __device__ __forceinline__ static uint64_t split_carry(uint64_t c, int lane)
    {
        const uint32_t u1 = __shfl_up_sync(LF_ALL, (uint32_t)(c >> 26) & (uint32_t)LF_M26, 1);
        const uint32_t u2 = __shfl_up_sync(LF_ALL, (uint32_t)(c >> 52), 2);
        return (c & LF_M26) + (lane >= 1 ? u1 : 0u) + (lane >= 2 ? u2 : 0u);
    }

    __device__ __forceinline__ static uint32_t mul(uint32_t a, uint32_t b, int lane, const Regs &g)
    {
        // columns: lane l gets sum_i a_i b_(l-i); b's index wraps to lanes >= 22
        // when l < i, which hold 0, as do lanes >= 10
        uint64_t c0 = 0, c1 = 0;
#pragma unroll
        for (int i = 0; i < 10; i += 2) {
            const uint32_t a0 = __shfl_sync(LF_ALL, a, i), a1 = __shfl_sync(LF_ALL, a, i + 1);
            const uint32_t b0 = __shfl_sync(LF_ALL, b, (lane - i) & 31);
            const uint32_t b1 = __shfl_sync(LF_ALL, b, (lane - i - 1) & 31);
            c0 += (uint64_t)a0 * b0;
            c1 += (uint64_t)a1 * b1;
        }
        // 19 columns below 2^63.2 -> lanes 0..20 below 2^27.1 (lane 20 below 2^12)
        const uint32_t cur = (uint32_t)split_carry(c0 + c1, lane);
        if constexpr (!FQ) {
            const uint32_t hi = __shfl_sync(LF_ALL, cur, (lane + 10) & 31);
            const uint32_t top = __shfl_sync(LF_ALL, cur, 20);
            // below 2^37
            const uint64_t d =
                lane < 10 ? (uint64_t)cur + 608ull * hi + (lane == 0 ? 369664ull * top : 0ull) : 0ull;
            // one carry step, the excess of limb 9 folded into limb 0
            const uint32_t e = (uint32_t)(d >> 26);
            const uint32_t up = __shfl_up_sync(LF_ALL, e, 1);
            const uint32_t e9 = __shfl_sync(LF_ALL, e, 9);
            return lane < 10 ? (uint32_t)(d & LF_M26) + (lane ? up : 608u * e9) : 0u;
        } else {
            // columns 10..20 times their table rows (below 2^55)
            uint64_t d = lane < 10 ? (uint64_t)cur : 0ull;
#pragma unroll
            for (int h = 0; h < 11; h++)
                d += (uint64_t)__shfl_sync(LF_ALL, cur, 10 + h) * g.r[h];
            // lanes 0..9 below 2^27, the carries past 2^260 at lanes 10 and 11
            const uint32_t c = (uint32_t)split_carry(d, lane);
            const uint32_t h10 = __shfl_sync(LF_ALL, c, 10), h11 = __shfl_sync(LF_ALL, c, 11);
            const uint64_t e = lane < 10 ? (uint64_t)c + (uint64_t)h10 * g.k0 + (uint64_t)h11 * g.k1 : 0ull;
            // one more carry step; limb 9 keeps its excess (below 2^27 + 2)
            const uint32_t u1 = __shfl_up_sync(LF_ALL, (uint32_t)(e >> 26) & (uint32_t)LF_M26, 1);
            const uint32_t u2 = __shfl_up_sync(LF_ALL, (uint32_t)(e >> 52), 2);
            const uint32_t in = (lane >= 1 ? u1 : 0u) + (lane >= 2 ? u2 : 0u);
            return lane < 9 ? (uint32_t)(e & LF_M26) + in : (lane == 9 ? (uint32_t)e + in : 0u);
        }
    }

    // a - b + Z (zk = g.z) or + 2Z (zk = g.z2): b's limbs must not exceed zk's
    __device__ __forceinline__ static uint32_t sub(uint32_t a, uint32_t b, uint32_t zk) { return a + zk - b; }

    // eight 32-bit limbs (any value below 2^256) -> this lane's limb
    __device__ __forceinline__ static uint32_t from_fe(const Fe &a, int lane)
    {
        uint32_t v = 0;
#pragma unroll
        for (int l = 0; l < 10; l++) {
            const int bit = 26 * l, w = bit >> 5, off = bit & 31;
            uint64_t x = a.w[w];
            if (w + 1 < 8)
                x |= (uint64_t)a.w[w + 1] << 32;
            const uint32_t limb = (uint32_t)((x >> off) & LF_M26);
            v = lane == l ? limb : v;
        }
        return v;
    }

    // -> eight 32-bit limbs, weakly reduced (below 2^256), the same on every lane
    __device__ __forceinline__ static Fe to_fe(uint32_t v, int lane)
    {
        // every lane gathers the limbs (below 2^32), then carries exactly in
        // registers: limbs 0..8 below 2^26, limb 9 keeps the excess
        uint32_t L[10];
#pragma unroll
        for (int l = 0; l < 10; l++)
            L[l] = __shfl_sync(LF_ALL, v, l);
#pragma unroll
        for (int l = 0; l < 9; l++) {
            L[l + 1] += L[l] >> 26;
            L[l] &= (uint32_t)LF_M26;
        }
        // pack bits 26 l .. of limb l (limb 9 may reach bit 266)
        uint32_t t[16];
#pragma unroll
        for (int k = 0; k < 16; k++)
            t[k] = 0;
#pragma unroll
        for (int l = 0; l < 10; l++) {
            const int bit = 26 * l, w = bit >> 5, off = bit & 31;
            const uint64_t x = (uint64_t)L[l] << off;
            t[w] |= (uint32_t)x;
            t[w + 1] |= (uint32_t)(x >> 32);
        }
        return F::reduce_wide(t);
    }
};

// The Horner chain on one block of four warps (one per scheduler), the
// operands in a shared slot file, one slot per field element (lane l reads
// word l).  A stage of the doubling or addition formula puts its independent
// products on different warps; the linear steps are done by the warp that
// needs their result, in registers.  The running total is double-buffered:
// set s holds X, Y = YA - YB, ZZ, ZZZ, and a doubling or addition writes set
// s ^ 1.  Limb bounds: products are below 2^27; X, a difference, below
// 2^29.6; the other product inputs below are sums of at most four products
// plus Z or 2Z, each below 2^30.1 where the other operand is below 2^29.8.
enum LaneSlot : int {
    LX, LYA, LYB, LZZ, LZZZ,  // running total, set 0 (set 1: + LSET)
    LSET = 5,
    LV = 10, LM, LW, LS, LM2,                 // doubling
    LX2, LY2, LZZ2, LZZZ2,                    // addend
    LU1, LU2, LS1, LS2, LZ12, LZZZ12, LPP, LRR, LPPP, LQ,  // addition
    LNSLOTS
};

template <class C>
struct LaneHorner {
    using F = typename C::F;
    using LF = LaneField<F>;
    uint32_t (*sl)[32];
    int lane, warp;
    typename LF::Regs g;
    uint32_t z, z2;  // this lane's limbs of Z and 2Z

    __device__ __forceinline__ uint32_t ld(int slot) const { return sl[slot][lane]; }
    __device__ __forceinline__ void st(int slot, uint32_t v) const { sl[slot][lane] = v; }

    // set s -> set s ^ 1 (the total is not the identity)
    __device__ void dbl(int s)
    {
        const int o = s * LSET, n = (s ^ 1) * LSET;
        if (warp == 0) {
            const uint32_t y = LF::sub(ld(o + LYA), ld(o + LYB), z);
            st(LV, LF::mul(y + y, y + y, lane, g));  // V = U^2, U = 2Y
        } else if (warp == 1) {
            const uint32_t x = ld(o + LX), zz = ld(o + LZZ);
            const uint32_t t = LF::mul(LF::sub(x, zz, z), x + zz, lane, g);  // (X - ZZ)(X + ZZ)
            st(LM, t + t + t);                                            // M = 3(X^2 - ZZ^2), a = -3
        }
        __syncthreads();
        if (warp == 0) {
            const uint32_t y = LF::sub(ld(o + LYA), ld(o + LYB), z);
            st(LW, LF::mul(y + y, ld(LV), lane, g));  // W = U V
        } else if (warp == 1) {
            st(LS, LF::mul(ld(o + LX), ld(LV), lane, g));  // S = X V
        } else if (warp == 2) {
            const uint32_t m = ld(LM);
            st(LM2, LF::mul(m, m, lane, g));  // M^2
        } else {
            st(n + LZZ, LF::mul(ld(LV), ld(o + LZZ), lane, g));  // ZZ' = V ZZ
        }
        __syncthreads();
        if (warp == 0) {
            const uint32_t sv = ld(LS);
            const uint32_t xn = LF::sub(ld(LM2), sv + sv, z);  // X' = M^2 - 2S
            st(n + LX, xn);
            st(n + LYA, LF::mul(ld(LM), LF::sub(sv, xn, z2), lane, g));  // M (S - X')
        } else if (warp == 1) {
            st(n + LZZZ, LF::mul(ld(LW), ld(o + LZZZ), lane, g));  // ZZZ' = W ZZZ
        } else if (warp == 2) {
            const uint32_t y = LF::sub(ld(o + LYA), ld(o + LYB), z);
            st(n + LYB, LF::mul(ld(LW), y, lane, g));  // W Y; Y' = M (S - X') - W Y
        }
        __syncthreads();
    }

    // set s += addend slots (neither is the identity): 0 -> the sum in set s ^ 1,
    // 1 -> the operands are equal (the caller doubles), 2 -> they cancel
    __device__ int add(int s, int *flag)
    {
        const int o = s * LSET, n = (s ^ 1) * LSET;
        if (warp == 0) {
            st(LU1, LF::mul(ld(o + LX), ld(LZZ2), lane, g));
        } else if (warp == 1) {
            st(LU2, LF::mul(ld(LX2), ld(o + LZZ), lane, g));
        } else if (warp == 2) {
            const uint32_t y = LF::sub(ld(o + LYA), ld(o + LYB), z);
            st(LS1, LF::mul(y, ld(LZZZ2), lane, g));
        } else {
            st(LS2, LF::mul(ld(LY2), ld(o + LZZZ), lane, g));
        }
        __syncthreads();
        // P = U2 - U1, R = S2 - S1: their squares and ZZ1 ZZ2, ZZZ1 ZZZ2 while
        // warp 3 also tests P and R for zero (rare: then the products go unused)
        const uint32_t pv = LF::sub(ld(LU2), ld(LU1), z), rv = LF::sub(ld(LS2), ld(LS1), z);
        if (warp == 0) {
            st(LPP, LF::mul(pv, pv, lane, g));
        } else if (warp == 1) {
            st(LRR, LF::mul(rv, rv, lane, g));
        } else if (warp == 2) {
            st(LZ12, LF::mul(ld(o + LZZ), ld(LZZ2), lane, g));
        } else {
            st(LZZZ12, LF::mul(ld(o + LZZZ), ld(LZZZ2), lane, g));
            const int f = F::is_zero(LF::to_fe(pv, lane)) ? (F::is_zero(LF::to_fe(rv, lane)) ? 1 : 2) : 0;
            if (lane == 0)
                *flag = f;
        }
        __syncthreads();
        const int f = *flag;
        if (f)
            return f;
        if (warp == 0)
            st(LPPP, LF::mul(pv, ld(LPP), lane, g));
        else if (warp == 1)
            st(LQ, LF::mul(ld(LU1), ld(LPP), lane, g));
        else if (warp == 2)
            st(n + LZZ, LF::mul(ld(LZ12), ld(LPP), lane, g));
        __syncthreads();
        if (warp == 0) {
            const uint32_t q = ld(LQ), ppp = ld(LPPP), rr = ld(LRR);
            st(n + LX, LF::sub(rr, ppp + q + q, z2));                               // X' = R^2 - PPP - 2Q
            st(n + LYA, LF::mul(rv, LF::sub(q + q + q + ppp, rr, z), lane, g));  // R (Q - X') = R (3Q + PPP - R^2)
        } else if (warp == 1) {
            st(n + LYB, LF::mul(ld(LS1), ld(LPPP), lane, g));  // S1 PPP
        } else if (warp == 2) {
            st(n + LZZZ, LF::mul(ld(LZZZ12), ld(LPPP), lane, g));  // ZZZ' = ZZZ12 PPP
        }
        __syncthreads();
        return 0;
    }
};

// one block of four warps per MSM of the batch
template <class C>
__global__ void __launch_bounds__(128) k_combine(const uint4 *__restrict__ S, const MsmDesc *__restrict__ desc,
                                                uint32_t *__restrict__ out)
{
    using F = typename C::F;
    using LF = LaneField<F>;
    __shared__ uint32_t sl[LNSLOTS][32];
    __shared__ int add_flag;
    const MsmDesc d = desc[blockIdx.x];
    const uint4 *Sm = S + 8 * (size_t)d.win_base;
    if (d.Wr == 1 && d.shift == 0) {  // one window (fixed base): nothing to combine
        if (threadIdx.x == 0)
            store_jacobian_canon<C>(out + 24 * (size_t)blockIdx.x, load_xyzz(Sm));
        return;
    }
    LaneHorner<C> h;
    h.sl = sl;
    h.lane = threadIdx.x & 31;
    h.warp = threadIdx.x >> 5;
    h.g = LF::regs(h.lane);
    h.z = h.g.z;
    h.z2 = h.g.z2;
    // words 10..31 of every slot stay 0
    for (int i = threadIdx.x; i < LNSLOTS * 32; i += blockDim.x)
        (&sl[0][0])[i] = 0;
    __syncthreads();
    // Load window sum k into the addend slots (warp w converts coordinate w);
    // false when it is the identity.  Every thread reads its ZZ to decide.
    auto load_addend = [&](int k) -> bool {
        const uint4 *p = Sm + 8 * (size_t)k;
        if (F::is_exact_zero(load_fe(p + 4)))
            return false;
        h.st(LX2 + h.warp, LF::from_fe(load_fe(p + 2 * h.warp), h.lane));  // LX2, LY2, LZZ2, LZZZ2
        __syncthreads();
        return true;
    };
    // copy the addend into set s as the total
    auto take_addend = [&](int s) {
        const int o = s * LSET;
        if (h.warp == 0) {
            h.st(o + LX, h.ld(LX2));
            h.st(o + LYA, h.ld(LY2));
            h.st(o + LYB, 0u);
            h.st(o + LZZ, h.ld(LZZ2));
            h.st(o + LZZZ, h.ld(LZZZ2));
        }
        __syncthreads();
    };
    int s = 0;
    bool ident = true;
    for (int k = (int)d.Wr - 1; k >= 0; k--) {
        if (!ident && k < (int)d.Wr - 1)
            for (uint32_t i = 0; i < d.c; i++) {
                h.dbl(s);
                s ^= 1;
            }
        if (!load_addend(k))
            continue;
        if (ident) {
            take_addend(s);
            ident = false;
            continue;
        }
        const int r = h.add(s, &add_flag);
        if (r == 0) {
            s ^= 1;
        } else if (r == 1) {  // equal operands: double
            h.dbl(s);
            s ^= 1;
        } else {  // they cancel
            ident = true;
        }
        __syncthreads();  // the addend slots are reused by the next window
    }
    if (!ident)
        for (uint32_t i = 0; i < d.shift; i++) {  // upper window-split half: times 2^(c w_lo)
            h.dbl(s);
            s ^= 1;
        }
    if (h.warp == 0) {
        Xyzz t = Group<C>::inf();
        if (!ident) {
            const int o = s * LSET;
            t.X = LF::to_fe(h.ld(o + LX), h.lane);
            t.Y = LF::to_fe(LF::sub(h.ld(o + LYA), h.ld(o + LYB), h.z), h.lane);
            t.ZZ = LF::to_fe(h.ld(o + LZZ), h.lane);
            t.ZZZ = LF::to_fe(h.ld(o + LZZZ), h.lane);
        }
        if (h.lane == 0)
            store_jacobian_canon<C>(out + 24 * (size_t)blockIdx.x, t);
    }
}

// Point operations on groups of eight lanes (four groups per warp): the
// independent products of a formula stage run on different lanes of the group,
// each in eight 32-bit limbs, so an addition is 4 product stages and a
// doubling 3, against 14 and 9 products in sequence on one thread; the linear
// steps are done by the group's lane 0.  Each group keeps its points and
// temporaries in its own shared slot file and synchronises only its own lanes,
// so groups may take different branches.  The formulas are Group's (add-2008-s,
// dbl-2008-s-1 with a = -3), complete.
enum GroupSlot : int {
    GRUN = 0, GACC = 4, GTMP = 8,  // points: X, Y, ZZ, ZZZ at base + 0..3
    GU = 12, GV, GW, GS, GM, GM2, GT, GA, GB, GD, GYA, GYB, GXN, GZZN, GZZZN,
    GU1, GU2, GS1, GS2, GZ12, GZZZ12, GP, GR, GPP, GRR, GPPP, GQ,
    GNSLOTS
};

struct GroupSlots {
    Fe f[GNSLOTS];
    int flag;
};

template <class C>
struct Group8 {
    using F = typename C::F;
    GroupSlots *sf;
    int gl;          // lane within the group
    unsigned gmask;  // the group's lanes in the warp

    __device__ __forceinline__ void sync() const { __syncwarp(gmask); }

    // slot lists packed six bits per lane: lane k's slot is bits 6k..6k+5
    __device__ __forceinline__ static constexpr uint64_t pk(int s0, int s1 = 0, int s2 = 0, int s3 = 0, int s4 = 0,
                                                           int s5 = 0)
    {
        return (uint64_t)s0 | (uint64_t)s1 << 6 | (uint64_t)s2 << 12 | (uint64_t)s3 << 18 | (uint64_t)s4 << 24 |
               (uint64_t)s5 << 30;
    }

    // lanes gl < width: f[d[gl]] = f[a[gl]] * f[b[gl]]
    __device__ __forceinline__ void products(int width, uint64_t a, uint64_t b, uint64_t d) const
    {
        sync();
        if (gl < width) {
            const int sh = 6 * gl;
            const Fe x = sf->f[(a >> sh) & 63], y = sf->f[(b >> sh) & 63];
            sf->f[(d >> sh) & 63] = F::mul(x, y);
        }
        sync();
    }

    __device__ __forceinline__ bool is_inf(int base) const { return F::is_exact_zero(sf->f[base + 2]); }

    __device__ __forceinline__ void set_inf(int base) const
    {
        sync();
        if (gl < 4)
            sf->f[base + gl] = F::zero();
        sync();
    }

    __device__ __forceinline__ void copy(int dst, int src) const
    {
        sync();
        if (gl < 4)
            sf->f[dst + gl] = sf->f[src + gl];
        sync();
    }

    // p = 2p (p at base)
    __device__ void dbl(int base) const
    {
        sync();
        if (is_inf(base))
            return;
        const int X = base, Y = base + 1, ZZ = base + 2, ZZZ = base + 3;
        if (gl == 0) {
            sf->f[GU] = F::dbl(sf->f[Y]);
            sf->f[GA] = F::sub(sf->f[X], sf->f[ZZ]);
            sf->f[GB] = F::add(sf->f[X], sf->f[ZZ]);
        }
        products(2, pk(GU, GA), pk(GU, GB), pk(GV, GT));  // V = U^2, T = (X - ZZ)(X + ZZ)
        if (gl == 0) {
            const Fe t = sf->f[GT];
            sf->f[GM] = F::add(F::dbl(t), t);  // M = 3(X^2 - ZZ^2), a = -3
        }
        // W = U V, S = X V, M^2, ZZ' = V ZZ
        products(4, pk(GU, X, GM, GV), pk(GV, GV, GM, ZZ), pk(GW, GS, GM2, GZZN));
        if (gl == 0) {
            const Fe xn = F::sub(sf->f[GM2], F::dbl(sf->f[GS]));
            sf->f[GXN] = xn;
            sf->f[GD] = F::sub(sf->f[GS], xn);
        }
        products(3, pk(GM, GW, GW), pk(GD, ZZZ, Y), pk(GYA, GZZZN, GYB));  // M (S - X'), W ZZZ, W Y
        if (gl == 0) {
            sf->f[X] = sf->f[GXN];
            sf->f[Y] = F::sub(sf->f[GYA], sf->f[GYB]);
            sf->f[ZZ] = sf->f[GZZN];
            sf->f[ZZZ] = sf->f[GZZZN];
            if (F::is_zero(sf->f[ZZ]))  // y = 0: no such point on a prime-order curve, kept complete
                sf->f[X] = sf->f[Y] = sf->f[ZZ] = sf->f[ZZZ] = F::zero();
        }
        sync();
    }

    // p += q (p at dst, q at src)
    __device__ void add(int dst, int src) const
    {
        sync();
        if (is_inf(src))
            return;
        if (is_inf(dst)) {
            copy(dst, src);
            return;
        }
        const int X1 = dst, Y1 = dst + 1, ZZ1 = dst + 2, ZZZ1 = dst + 3;
        const int X2 = src, Y2 = src + 1, ZZ2 = src + 2, ZZZ2 = src + 3;
        products(6, pk(X1, X2, Y1, Y2, ZZ1, ZZZ1), pk(ZZ2, ZZ1, ZZZ2, ZZZ1, ZZ2, ZZZ2),
                 pk(GU1, GU2, GS1, GS2, GZ12, GZZZ12));
        if (gl == 0) {
            sf->f[GP] = F::sub(sf->f[GU2], sf->f[GU1]);
            sf->f[GR] = F::sub(sf->f[GS2], sf->f[GS1]);
            sf->flag = F::is_zero(sf->f[GP]) ? (F::is_zero(sf->f[GR]) ? 1 : 2) : 0;
        }
        sync();
        const int flag = sf->flag;
        if (flag == 1) {  // equal points: double
            dbl(dst);
            return;
        }
        if (flag == 2) {  // opposite points
            set_inf(dst);
            return;
        }
        products(2, pk(GP, GR), pk(GP, GR), pk(GPP, GRR));
        products(3, pk(GP, GU1, GZ12), pk(GPP, GPP, GPP), pk(GPPP, GQ, GZZN));
        if (gl == 0) {
            const Fe xn = F::sub(F::sub(sf->f[GRR], sf->f[GPPP]), F::dbl(sf->f[GQ]));
            sf->f[GXN] = xn;
            sf->f[GD] = F::sub(sf->f[GQ], xn);
        }
        products(3, pk(GR, GS1, GZZZ12), pk(GD, GPPP, GPPP), pk(GYA, GYB, GZZZN));
        if (gl == 0) {
            sf->f[X1] = sf->f[GXN];
            sf->f[Y1] = F::sub(sf->f[GYA], sf->f[GYB]);
            sf->f[ZZ1] = sf->f[GZZN];
            sf->f[ZZZ1] = sf->f[GZZZN];
        }
        sync();
    }

    // p = 2 (x, y) for the affine point at src (x, y at src, src + 1), into dst
    // (mdbl-2008-s-1, M = 3 x^2 - 3)
    __device__ void dbl_affine(int dst, int src) const
    {
        sync();
        if (gl == 0)
            sf->f[GU] = F::dbl(sf->f[src + 1]);
        products(2, pk(GU, src), pk(GU, src), pk(GV, GT));  // V = U^2, x^2
        if (gl == 0) {
            const Fe t = F::sub(sf->f[GT], F::one());
            sf->f[GM] = F::add(F::dbl(t), t);
        }
        products(3, pk(GU, src, GM), pk(GV, GV, GM), pk(GW, GS, GM2));  // W = U V, S = x V, M^2
        if (gl == 0) {
            const Fe xn = F::sub(sf->f[GM2], F::dbl(sf->f[GS]));
            sf->f[GXN] = xn;
            sf->f[GD] = F::sub(sf->f[GS], xn);
        }
        products(2, pk(GM, GW), pk(GD, src + 1), pk(GYA, GYB));  // M (S - X'), W y
        if (gl == 0) {
            if (F::is_zero(sf->f[GV])) {  // y = 0: no such point on a prime-order curve, kept complete
                sf->f[dst] = sf->f[dst + 1] = sf->f[dst + 2] = sf->f[dst + 3] = F::zero();
            } else {
                sf->f[dst] = sf->f[GXN];
                sf->f[dst + 1] = F::sub(sf->f[GYA], sf->f[GYB]);
                sf->f[dst + 2] = sf->f[GV];
                sf->f[dst + 3] = sf->f[GW];
            }
        }
        sync();
    }

    // p += (x, y), the affine point at src (never the identity): madd-2008-s
    __device__ void madd(int dst, int src) const
    {
        sync();
        if (is_inf(dst)) {
            if (gl < 4)
                sf->f[dst + gl] = gl < 2 ? sf->f[src + gl] : F::one();
            sync();
            return;
        }
        const int X1 = dst, Y1 = dst + 1, ZZ1 = dst + 2, ZZZ1 = dst + 3;
        products(2, pk(src, src + 1), pk(ZZ1, ZZZ1), pk(GU2, GS2));  // U2 = x ZZ1, S2 = y ZZZ1
        if (gl == 0) {
            sf->f[GP] = F::sub(sf->f[GU2], sf->f[X1]);
            sf->f[GR] = F::sub(sf->f[GS2], sf->f[Y1]);
            sf->flag = F::is_zero(sf->f[GP]) ? (F::is_zero(sf->f[GR]) ? 1 : 2) : 0;
        }
        sync();
        const int flag = sf->flag;
        if (flag == 1) {  // same point: double
            dbl_affine(dst, src);
            return;
        }
        if (flag == 2) {  // opposite points
            set_inf(dst);
            return;
        }
        products(2, pk(GP, GR), pk(GP, GR), pk(GPP, GRR));
        products(3, pk(GP, X1, ZZ1), pk(GPP, GPP, GPP), pk(GPPP, GQ, GZZN));  // PPP, Q = X1 PP, ZZ1 PP
        if (gl == 0) {
            const Fe xn = F::sub(F::sub(sf->f[GRR], sf->f[GPPP]), F::dbl(sf->f[GQ]));
            sf->f[GXN] = xn;
            sf->f[GD] = F::sub(sf->f[GQ], xn);
        }
        products(3, pk(GR, Y1, ZZZ1), pk(GD, GPPP, GPPP), pk(GYA, GYB, GZZZN));  // R (Q - X'), Y1 PPP, ZZZ1 PPP
        if (gl == 0) {
            sf->f[X1] = sf->f[GXN];
            sf->f[Y1] = F::sub(sf->f[GYA], sf->f[GYB]);
            sf->f[ZZ1] = sf->f[GZZN];
            sf->f[ZZZ1] = sf->f[GZZZN];
        }
        sync();
    }
};

// Window sums of a plan of few windows of at most WG_MAX_B buckets, where the
// two-level reduction's chains of one-thread additions set the time: one block
// of WG_GROUPS eight-lane groups per window, group g taking the q = B / groups
// buckets [g q, (g + 1) q):
//     run_g = sum_j B_j,   acc_g = sum_j (j - g q + 1) B_j   (top-down running sum),
// then S = sum_g acc_g + q sum_{g >= 1} R_g with R_g = sum_{h >= g} run_h (a
// suffix scan over the groups), q R_g by doublings, and a tree sum.
constexpr int WG_GROUPS = 32;
constexpr uint32_t WG_MAX_B = 256;

template <class C>
__global__ void __launch_bounds__(WG_GROUPS * 8) k_window_groups(const uint32_t *__restrict__ seg_off,
                                                                const uint4 *__restrict__ seg_sum,
                                                                const MsmDesc *__restrict__ desc, uint32_t M,
                                                                uint4 *__restrict__ S)
{
    __shared__ GroupSlots sl[WG_GROUPS];
    const uint32_t s = blockIdx.x;
    const uint32_t mi = find_msm(M, s, [&](uint32_t k) { return desc[k].win_base; });
    const MsmDesc d = desc[mi];
    const uint32_t k = s - d.win_base;
    const uint32_t g = threadIdx.x >> 3;
    Group8<C> op;
    op.sf = &sl[g];
    op.gl = (int)(threadIdx.x & 7);
    op.gmask = 0xffu << (8 * (g & 3));
    const uint32_t nga = d.B < (uint32_t)WG_GROUPS ? d.B : (uint32_t)WG_GROUPS;  // B is a power of two
    const uint32_t q = d.B / nga;
    const bool active = g < nga;
    op.set_inf(GRUN);
    op.set_inf(GACC);
    if (active) {
        for (int j = (int)((g + 1) * q) - 1; j >= (int)(g * q); j--) {
            const uint32_t kb = d.bucket_base + k * d.B + (uint32_t)j;
            const uint32_t s0 = seg_off[kb];
            if (seg_off[kb + 1] != s0) {
                op.sync();
                if (op.gl < 4)
                    op.sf->f[GTMP + op.gl] = load_fe(seg_sum + 8 * (size_t)s0 + 2 * op.gl);
                op.add(GRUN, GTMP);
            }
            op.add(GACC, GRUN);
        }
    }
    __syncthreads();
    for (uint32_t dl = 1; dl < nga; dl <<= 1) {  // R_g
        const bool take = active && g + dl < nga;
        if (take && op.gl < 4)
            op.sf->f[GTMP + op.gl] = sl[g + dl].f[GRUN + op.gl];
        __syncthreads();
        if (take)
            op.add(GRUN, GTMP);
        __syncthreads();
    }
    if (active) {  // v_g = q R_g [g >= 1] + acc_g, in GRUN
        if (g >= 1) {
            for (uint32_t m = q; m > 1; m >>= 1)
                op.dbl(GRUN);
        } else {
            op.set_inf(GRUN);
        }
        op.add(GRUN, GACC);
    }
    __syncthreads();
    for (uint32_t st = nga / 2; st > 0; st >>= 1) {
        if (g < st) {
            if (op.gl < 4)
                op.sf->f[GTMP + op.gl] = sl[g + st].f[GRUN + op.gl];
            op.add(GRUN, GTMP);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        Xyzz t;
        t.X = sl[0].f[GRUN];
        t.Y = sl[0].f[GRUN + 1];
        t.ZZ = sl[0].f[GRUN + 2];
        t.ZZZ = sl[0].f[GRUN + 3];
        store_xyzz(S + 8 * (size_t)s, t);
    }
}

// Bucket accumulation and merges of small plans on eight-lane groups (a mixed
// addition is 4 product stages against 10 products on one thread): one group
// per segment, then one group per bucket of 2..8 segments (more go to the
// heavy-bucket list as in k_merge_light).  About 3.7 times the instructions
// per entry of the one-thread form, so only for plans of at most
// ACC_GROUPS_MAX_ENTRIES entries.
constexpr uint64_t ACC_GROUPS_MAX_ENTRIES = 98304;

template <class C>
__global__ void __launch_bounds__(256) k_accumulate_groups(const uint4 *__restrict__ segs,
                                                          const uint32_t *__restrict__ seg_lo,
                                                          const uint32_t *__restrict__ seg_hi,
                                                          const uint32_t *__restrict__ sorted,
                                                          const uint4 *__restrict__ pts, uint4 *__restrict__ seg_sum)
{
    using F = typename C::F;
    __shared__ GroupSlots sl[32];
    const uint32_t g = threadIdx.x >> 3;
    Group8<C> op;
    op.sf = &sl[g];
    op.gl = (int)(threadIdx.x & 7);
    op.gmask = 0xffu << (8 * (g & 3));
    const uint32_t S0 = *seg_lo, S = *seg_hi;
    for (uint32_t s = S0 + blockIdx.x * 32 + g; s < S; s += gridDim.x * 32) {
        const uint4 d = segs[s];  // start, length, destination slot
        op.set_inf(GRUN);
        for (uint32_t i = 0; i < d.y; i++) {
            const uint32_t e = __ldg(sorted + d.x + i);
            Fe x, y;
            load_affine(pts, e & 0x7fffffffu, x, y);
            if (F::is_exact_zero(x) && F::is_exact_zero(y))
                continue;  // identity base
            op.sync();
            if (op.gl == 0)
                op.sf->f[GTMP] = x;
            else if (op.gl == 1)
                op.sf->f[GTMP + 1] = (e >> 31) ? F::neg(y) : y;
            op.madd(GRUN, GTMP);
        }
        op.sync();
        if (op.gl < 4)
            store_fe(seg_sum + 8 * (size_t)d.z + 2 * op.gl, op.sf->f[GRUN + op.gl]);
    }
}

template <class C>
__global__ void __launch_bounds__(256) k_merge_groups(const uint32_t *__restrict__ seg_off, uint32_t NB,
                                                     uint4 *__restrict__ seg_sum, uint32_t *__restrict__ heavy,
                                                     uint32_t *__restrict__ heavy_n, uint32_t heavy_min)
{
    __shared__ GroupSlots sl[32];
    const uint32_t g = threadIdx.x >> 3;
    Group8<C> op;
    op.sf = &sl[g];
    op.gl = (int)(threadIdx.x & 7);
    op.gmask = 0xffu << (8 * (g & 3));
    for (uint32_t kb = blockIdx.x * 32 + g; kb < NB; kb += gridDim.x * 32) {
        const uint32_t s0 = seg_off[kb], ns = seg_off[kb + 1] - s0;
        if (ns < 2)
            continue;
        if (ns > heavy_min) {
            if (op.gl == 0)
                heavy[atomicAdd(heavy_n, 1u)] = kb;
            continue;
        }
        op.sync();
        if (op.gl < 4)
            op.sf->f[GRUN + op.gl] = load_fe(seg_sum + 8 * (size_t)s0 + 2 * op.gl);
        for (uint32_t j = 1; j < ns; j++) {
            op.sync();
            if (op.gl < 4)
                op.sf->f[GTMP + op.gl] = load_fe(seg_sum + 8 * (size_t)(s0 + j) + 2 * op.gl);
            op.add(GRUN, GTMP);
        }
        op.sync();
        if (op.gl < 4)
            store_fe(seg_sum + 8 * (size_t)s0 + 2 * op.gl, op.sf->f[GRUN + op.gl]);
    }
}

template <class C>
cudaError_t msm_tail(Context &ctx, const BatchPlan &p, const BatchBuffers &b)
{
    cudaStream_t st = ctx.stream;
    // a small plan: accumulation and merges on eight-lane groups
    const bool small = !p.ba_rounds && !p.part_slice && p.entries_bound <= ACC_GROUPS_MAX_ENTRIES;
    // 2. accumulate: a grid of short blocks (up to 32 per SM, several waves), each
    //    thread taking segments at a stride of the grid.  Segments come longest
    //    first, so every block gets a like mix of long and short ones; blocks end
    //    wave by wave, so kernels of other streams (another MSM's tail) get SM
    //    slots while this one runs.  Threads past the device-side count exit.
    if (p.ba_rounds) {
        // Host inputs in two parts: bucket k's part-j entries form list NB*j + k
        // (offsets has 2 NB + 1 entries), so each part's lists are one range of
        // every level; its rounds and its fold run once that part is in, and
        // the first part-1 segment of a bucket continues its part-0 sum.
        const int parts = p.part_slice ? 2 : 1;
        const size_t nh = (size_t)(p.L + 1) * p.hist_blocks * (p.part_slice ? 2 : 1);
        const uint32_t *bound[3] = {b.len_scan, b.len_scan + (p.part_slice ? nh / 2 : nh), b.len_scan + nh};
        const uint4 *last = b.ba_lvl[(p.ba_rounds - 1) & 1];
        for (int j = 0; j < parts; j++) {
            if (b.ready[j]) {  // host inputs: this part of the bases arrives on another stream
                const cudaError_t e =
                    cudaStreamWaitEvent(st, b.ready[j], ctx.capturing_host ? cudaEventWaitExternal : 0);
                if (e != cudaSuccess)
                    return e;
            }
            cudaEvent_t ev0 = nullptr;
            prof_begin(ctx, &ev0);
            const uint32_t *lo = j ? b.offsets + p.NB : nullptr;
            const uint32_t *hi = b.offsets + (size_t)p.NB * (j + 1);
            for (uint32_t r = 1; r <= p.ba_rounds; r++) {
                const uint4 *in_lvl = r == 1 ? nullptr : b.ba_lvl[(r - 2) & 1];
                uint4 *out_lvl = b.ba_lvl[(r - 1) & 1];
                const uint32_t blocks = std::max<uint32_t>(1, p.ba_blocks[r - 1]);
                if (r == 1)
                    k_ba_pairs<C, true><<<blocks, BA_BT, 0, st>>>(lo, hi, r, b.sorted, b.points, in_lvl, b.ba_pre,
                                                                  b.ba_co, b.ba_tot);
                else
                    k_ba_pairs<C, false><<<blocks, BA_BT, 0, st>>>(lo, hi, r, b.sorted, b.points, in_lvl, b.ba_pre,
                                                                   b.ba_co, b.ba_tot);
                HS_LAUNCH_CHECK(ctx);
                k_ba_invert<C><<<(blocks + 63) / 64, 64, 0, st>>>(lo, hi, r, b.ba_tot, b.ba_inv);
                HS_LAUNCH_CHECK(ctx);
                if (r == 1)
                    k_ba_finish<C, true><<<blocks, BA_BT, 0, st>>>(lo, hi, r, b.sorted, b.points, in_lvl, b.ba_pre,
                                                                   b.ba_co, b.ba_inv, out_lvl);
                else
                    k_ba_finish<C, false><<<blocks, BA_BT, 0, st>>>(lo, hi, r, b.sorted, b.points, in_lvl,
                                                                    b.ba_pre, b.ba_co, b.ba_inv, out_lvl);
                HS_LAUNCH_CHECK(ctx);
            }
            const int threads = 128;
            const uint64_t want = (p.max_segs + threads - 1) / threads;
            const int blocks = (int)std::max<uint64_t>(1, std::min<uint64_t>(want, (uint64_t)ctx.sm_count * 32));
            if (j == 0)
                k_accumulate_level<C, false><<<blocks, threads, 0, st>>>(b.segs, bound[0], bound[1], last, b.seg_sum);
            else
                k_accumulate_level<C, true><<<blocks, threads, 0, st>>>(b.segs, bound[1], bound[2], last, b.seg_sum);
            HS_LAUNCH_CHECK(ctx);
            prof_end(ctx, ev0, j == 0 ? p.entries_pinned : 0);
        }
    } else if (small) {
        const uint64_t want = (p.max_segs + 31) / 32;
        const int blocks = (int)std::max<uint64_t>(1, std::min<uint64_t>(want, (uint64_t)ctx.sm_count * 8));
        const size_t nh = (size_t)(p.L + 1) * p.hist_blocks;
        cudaEvent_t ev0 = nullptr;
        prof_begin(ctx, &ev0);
        k_accumulate_groups<C><<<blocks, 256, 0, st>>>(b.segs, b.len_scan, b.len_scan + nh, b.sorted, b.points,
                                                       b.seg_sum);
        HS_LAUNCH_CHECK(ctx);
        prof_end(ctx, ev0, p.entries_pinned);
    } else {
        const int threads = 128;
        const uint64_t want = (p.max_segs + threads - 1) / threads;
        const int blocks = (int)std::max<uint64_t>(1, std::min<uint64_t>(want, (uint64_t)ctx.sm_count * 32));
        // the segment lists: [0, total), or per part [0, P1) and [P1, total) with P1
        // the scan position where the part-1 histogram starts
        const size_t nh = (size_t)(p.L + 1) * p.hist_blocks * (p.part_slice ? 2 : 1);
        const int parts = p.part_slice ? 2 : 1;
        const uint32_t *bound[3] = {b.len_scan, b.len_scan + (p.part_slice ? nh / 2 : nh), b.len_scan + nh};
        for (int j = 0; j < parts; j++) {
            if (b.ready[j]) {  // host inputs: this part of the bases arrives on another stream
                const cudaError_t e = cudaStreamWaitEvent(st, b.ready[j], ctx.capturing_host ? cudaEventWaitExternal : 0);
                if (e != cudaSuccess)
                    return e;
            }
            cudaEvent_t ev0 = nullptr;
            prof_begin(ctx, &ev0);
            if (j == 0)
                k_accumulate<C, false><<<blocks, threads, 0, st>>>(b.segs, bound[0], bound[1], b.sorted, b.points,
                                                                   b.seg_sum);
            else
                k_accumulate<C, true><<<blocks, threads, 0, st>>>(b.segs, bound[1], bound[2], b.sorted, b.points,
                                                                  b.seg_sum);
            HS_LAUNCH_CHECK(ctx);
            prof_end(ctx, ev0, j == 0 ? p.entries_pinned : 0);
        }
    }
    // 3. merge multi-segment buckets
    {
        cudaError_t e = cudaMemsetAsync(b.heavy_n, 0, sizeof(uint32_t), st);
        if (e != cudaSuccess)
            return e;
        const int threads = 256;
        if (small) {
            const unsigned mb = (unsigned)std::max<uint32_t>(1, std::min<uint32_t>((p.NB + 31) / 32,
                                                                                   (uint32_t)ctx.sm_count * 8));
            k_merge_groups<C><<<mb, 256, 0, st>>>(b.seg_off, p.NB, b.seg_sum, b.heavy, b.heavy_n, 8);
        } else {
            k_merge_light<C><<<(p.NB + threads - 1) / threads, threads, 0, st>>>(b.seg_off, p.NB, b.seg_sum,
                                                                               b.heavy, b.heavy_n, 8);
        }
        HS_LAUNCH_CHECK(ctx);
        k_merge_heavy<C><<<ctx.sm_count, HEAVY_THREADS, 0, st>>>(b.seg_off, b.heavy, b.heavy_n, b.seg_sum);
        HS_LAUNCH_CHECK(ctx);
    }
    // 4. bucket reduction: group running sums, then one block per window; a
    //    plan of few windows of at most WG_MAX_B buckets reduces each window on
    //    one block of eight-lane groups
    if (p.max_B <= WG_MAX_B && p.WS <= 4u * (uint32_t)ctx.sm_count) {
        k_window_groups<C><<<p.WS, WG_GROUPS * 8, 0, st>>>(b.seg_off, b.seg_sum, b.desc, p.M, b.redS);
        HS_LAUNCH_CHECK(ctx);
    } else {
        const int threads = 128;
        k_reduce_groups<C><<<(p.G + threads - 1) / threads, threads, 0, st>>>(b.seg_off, b.seg_sum, b.desc, p.M,
                                                                            p.G, b.redA);
        HS_LAUNCH_CHECK(ctx);
        // A plan of few chunks (one or a few MSMs) is latency-bound, and so are
        // windows of at most 16 groups: one thread per group up to
        // RED_CHUNK_THREADS groups.  Many chunks of more groups (a batch of larger
        // MSMs) fill the device, and RED_CHUNK_Q groups per thread keep the scans'
        // extra work small.  (Measured: 256 FCMP++ verifications, 16 groups per
        // window, 51k -> 65k per second one group per thread; 1024 MSMs of
        // 64..65536 points 1.5% faster with four.)
        const int wide = p.CH <= 4u * (uint32_t)ctx.sm_count || p.max_T <= 16;
        const uint32_t t2 =
            std::max<uint32_t>(32, std::min<uint32_t>(RED_CHUNK_THREADS, wide ? p.max_T : p.max_T / RED_CHUNK_Q));
        if (p.max_nbk == 1) {  // one chunk per window: chunk index == window slot
            k_window_chunks<C, true><<<p.CH, t2, 0, st>>>(b.redA, b.desc, p.M, b.redS, wide);
            HS_LAUNCH_CHECK(ctx);
        } else {
            k_window_chunks<C, false><<<p.CH, t2, 0, st>>>(b.redA, b.desc, p.M, b.redC, wide);
            HS_LAUNCH_CHECK(ctx);
            const uint32_t t3 = std::max<uint32_t>(32, std::min<uint32_t>(RED_CHUNK, p.max_nbk));
            k_window_sum<C><<<p.WS, t3, 0, st>>>(b.redC, b.desc, p.M, b.redS);
            HS_LAUNCH_CHECK(ctx);
        }
    }
    // 5. Horner over windows, one block of four warps per MSM
    k_combine<C><<<p.M, 128, 0, st>>>(b.redS, b.desc, b.out_jac);
    HS_LAUNCH_CHECK(ctx);
    return cudaSuccess;
}

// ---------------------------------------------------------------------------
// input conversion: radix-2^51 limbs -> 8 x 32-bit words (weakly reduced)
// ---------------------------------------------------------------------------
template <class C>
__device__ Fe fe_from_51(const uint64_t *l)
{
    using F = typename C::F;
    // sum l_i * 2^(51 i) into five 64-bit words (limbs may exceed 51 bits)
    unsigned __int128 acc = 0;
    uint64_t w[5];
    // word j covers bits [64j, 64j+64)
    unsigned __int128 v0 = (unsigned __int128)l[0];
    unsigned __int128 v1 = (unsigned __int128)l[1] << 51;  // bits 51..115
    unsigned __int128 v2 = (unsigned __int128)l[2] << 38;  // 102 = 64 + 38
    unsigned __int128 v3 = (unsigned __int128)l[3] << 25;  // 153 = 128 + 25
    unsigned __int128 v4 = (unsigned __int128)l[4] << 12;  // 204 = 192 + 12
    acc = (unsigned __int128)(uint64_t)v0 + (uint64_t)v1;
    w[0] = (uint64_t)acc;
    acc = (acc >> 64) + (uint64_t)(v0 >> 64) + (uint64_t)(v1 >> 64) + (uint64_t)v2;
    w[1] = (uint64_t)acc;
    acc = (acc >> 64) + (uint64_t)(v2 >> 64) + (uint64_t)v3;
    w[2] = (uint64_t)acc;
    acc = (acc >> 64) + (uint64_t)(v3 >> 64) + (uint64_t)v4;
    w[3] = (uint64_t)acc;
    acc = (acc >> 64) + (uint64_t)(v4 >> 64);
    w[4] = (uint64_t)acc;  // < 2^13
    Fe r;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        r.w[2 * i] = (uint32_t)w[i];
        r.w[2 * i + 1] = (uint32_t)(w[i] >> 32);
    }
    // fold w[4] * 2^256 == w[4] * c, one bit at a time (w[4] is tiny, usually 0)
    uint64_t top = w[4];
    Fe c1 = F::zero();
    F::add_c_masked(c1, 0xffffffffu);  // c1 = c = 2^256 mod m
    while (top) {
        if (top & 1)
            r = F::add(r, c1);
        c1 = F::dbl(c1);
        top >>= 1;
    }
    return r;
}

template <class C>
__device__ void fe_to_51(uint64_t *l, const Fe &canon)
{
    uint64_t w[4];
#pragma unroll
    for (int i = 0; i < 4; i++)
        w[i] = (uint64_t)canon.w[2 * i] | ((uint64_t)canon.w[2 * i + 1] << 32);
    const uint64_t M51 = (1ull << 51) - 1;
    l[0] = w[0] & M51;
    l[1] = ((w[0] >> 51) | (w[1] << 13)) & M51;
    l[2] = ((w[1] >> 38) | (w[2] << 26)) & M51;
    l[3] = ((w[2] >> 25) | (w[3] << 39)) & M51;
    l[4] = (w[3] >> 12) & M51;
}

// batch Jacobian -> affine: each thread owns a chunk, multiplies the Z values
// that are neither 0 nor 1 (Montgomery's trick, fp/include/fp_batch_invert.h:61-114),
// inverts the chunk product once and walks back.  Identity (Z == 0) -> (0,0).
constexpr int AFF_CHUNK = 16;

template <class C>
__global__ void k_jac_to_affine(const uint64_t *__restrict__ in, int fmt, size_t n, uint4 *__restrict__ out,
                                uint4 *__restrict__ scratch)
{
    using F = typename C::F;
    // thread t takes points t, t + T, t + 2T, ... (T threads in the grid, at most
    // AFF_CHUNK points each): a warp reads consecutive records
    const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    const size_t T = (size_t)gridDim.x * blockDim.x;
    if (t >= n)
        return;
    const size_t cnt = (n - t + T - 1) / T;
    const size_t stride = (fmt == HS_FMT_JACOBIAN51) ? 15 : (fmt == HS_FMT_AFFINE51 ? 10 : 8);
    // pass 1: prefix products of the Z values that need inverting
    Fe run = F::one();
    bool any = false;
    for (size_t j = 0; j < cnt; j++) {
        const size_t i = t + j * T;
        Fe z;
        if (fmt == HS_FMT_JACOBIAN51) {
            z = fe_from_51<C>(in + stride * i + 10);
            Fe zc = F::canon(z);
            bool is0 = F::is_exact_zero(zc);
            Fe one = F::one();
            bool is1 = true;
#pragma unroll
            for (int k = 0; k < 8; k++)
                is1 = is1 && (zc.w[k] == one.w[k]);
            if (!is0 && !is1) {
                run = F::mul(run, z);
                any = true;
            }
        }
        store_fe(scratch + 2 * i, run);
    }
    Fe inv = any ? F::inv(run) : F::one();
    // pass 2: walk back
    for (size_t j = cnt; j-- > 0;) {
        const size_t i = t + j * T;
        Fe x, y;
        if (fmt == HS_FMT_JACOBIAN51) {
            x = fe_from_51<C>(in + stride * i);
            y = fe_from_51<C>(in + stride * i + 5);
        } else if (fmt == HS_FMT_AFFINE51) {
            x = fe_from_51<C>(in + stride * i);
            y = fe_from_51<C>(in + stride * i + 5);
        } else {
            const uint4 *src = reinterpret_cast<const uint4 *>(in) + 4 * i;
            x = load_fe(src);
            y = load_fe(src + 2);
        }
        bool ident = false;
        if (fmt == HS_FMT_JACOBIAN51) {
            Fe z = fe_from_51<C>(in + stride * i + 10);
            Fe zc = F::canon(z);
            bool is0 = F::is_exact_zero(zc);
            Fe one = F::one();
            bool is1 = true;
#pragma unroll
            for (int k = 0; k < 8; k++)
                is1 = is1 && (zc.w[k] == one.w[k]);
            if (is0) {
                ident = true;
            } else if (!is1) {
                Fe prev = (j > 0) ? load_fe(scratch + 2 * (i - T)) : F::one();
                Fe zi = F::mul(inv, prev);  // 1/z
                inv = F::mul(inv, z);
                Fe zi2 = F::sqr(zi);
                x = F::mul(x, zi2);
                y = F::mul(y, F::mul(zi2, zi));
            }
        } else {
            Fe xc = F::canon(x), yc = F::canon(y);
            ident = F::is_exact_zero(xc) && F::is_exact_zero(yc);
        }
        if (ident) {
            x = F::zero();
            y = F::zero();
        }
        store_fe(out + 4 * i, F::canon(x));
        store_fe(out + 4 * i + 2, F::canon(y));
    }
}

template <class C>
cudaError_t decompress(Context &ctx, const void *d_in, size_t n, uint4 *d_out, uint8_t *d_valid, uint32_t *d_bad);

// HS_FMT_COMPRESSED input decodes on the device; the count of invalid
// encodings is left in the first word of scratch for the caller to check.
template <class C>
cudaError_t to_affine(Context &ctx, const void *d_in, int fmt, size_t n, uint4 *d_out, void *scratch)
{
    if (n == 0)
        return cudaSuccess;
    if (fmt == HS_FMT_COMPRESSED) {
        cudaError_t e = cudaMemsetAsync(scratch, 0, sizeof(uint32_t), ctx.stream);
        if (e != cudaSuccess)
            return e;
        return decompress<C>(ctx, d_in, n, d_out, nullptr, static_cast<uint32_t *>(scratch));
    }
    const size_t chunks = (n + AFF_CHUNK - 1) / AFF_CHUNK;
    const int threads = 128;
    k_jac_to_affine<C><<<(unsigned)((chunks + threads - 1) / threads), threads, 0, ctx.stream>>>(
        reinterpret_cast<const uint64_t *>(d_in), fmt, n, d_out, reinterpret_cast<uint4 *>(scratch));
    HS_LAUNCH_CHECK(ctx);
    return cudaSuccess;
}

inline size_t to_affine_scratch(size_t n) { return n * 32; }

// ---------------------------------------------------------------------------
// output formatting of canonical Jacobians (24 words each)
// ---------------------------------------------------------------------------
template <class C>
__global__ void k_format_out(const uint32_t *__restrict__ jac, size_t count, int fmt, void *__restrict__ out)
{
    using F = typename C::F;
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= count)
        return;
    Fe X, Y, Z;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        X.w[k] = jac[24 * i + k];
        Y.w[k] = jac[24 * i + 8 + k];
        Z.w[k] = jac[24 * i + 16 + k];
    }
    const bool ident = F::is_zero(Z);
    if (fmt == HS_FMT_JACOBIAN51) {
        uint64_t *o = reinterpret_cast<uint64_t *>(out) + 15 * i;
        fe_to_51<C>(o, F::canon(X));
        fe_to_51<C>(o + 5, F::canon(Y));
        fe_to_51<C>(o + 10, F::canon(Z));
        return;
    }
    Fe x = F::zero(), y = F::zero();
    Fe zc = F::canon(Z);
    bool z_one = zc.w[0] == 1u;
#pragma unroll
    for (int k = 1; k < 8; k++)
        z_one = z_one && zc.w[k] == 0u;
    if (z_one) {
        x = F::canon(X);
        y = F::canon(Y);
    } else if (!ident) {
        Fe zi = F::inv(Z);
        Fe zi2 = F::sqr(zi);
        x = F::canon(F::mul(X, zi2));
        y = F::canon(F::mul(Y, F::mul(zi2, zi)));
    }
    if (fmt == HS_FMT_AFFINE51) {
        uint64_t *o = reinterpret_cast<uint64_t *>(out) + 10 * i;
        fe_to_51<C>(o, x);
        fe_to_51<C>(o + 5, y);
    } else if (fmt == HS_FMT_AFFINE) {
        uint4 *o = reinterpret_cast<uint4 *>(out) + 4 * i;
        store_fe(o, x);
        store_fe(o + 2, y);
    } else {  // compressed: x with parity of y in bit 255
        uint32_t *o = reinterpret_cast<uint32_t *>(out) + 8 * i;
#pragma unroll
        for (int k = 0; k < 8; k++)
            o[k] = x.w[k];
        if (!ident)
            o[7] |= (y.w[0] & 1u) << 31;
    }
}

template <class C>
cudaError_t format_out(Context &ctx, const uint32_t *d_jac, size_t count, int out_fmt, void *d_out)
{
    if (count == 0)
        return cudaSuccess;
    const int threads = 64;
    k_format_out<C><<<(unsigned)((count + threads - 1) / threads), threads, 0, ctx.stream>>>(d_jac, count, out_fmt,
                                                                                           d_out);
    HS_LAUNCH_CHECK(ctx);
    return cudaSuccess;
}

// ---------------------------------------------------------------------------
// simplified SWU map (RFC 9380 6.6.2) as the reference computes it
// (helios/src/x64/helios_map_to_curve.cpp:98-198): output affine, Z = 1.
// ---------------------------------------------------------------------------
template <class C>
__device__ bool fsqrt(Fe &r, const Fe &a);

template <>
__device__ inline bool fsqrt<HeliosCurve>(Fe &r, const Fe &a)
{
    // p = 5 (mod 8): x = a^((p+3)/8); if x^2 = -a multiply by sqrt(-1) = 2^((p-1)/4)
    const uint32_t e[8] = {0xfffffffeu, 0xffffffffu, 0xffffffffu, 0xffffffffu,
                           0xffffffffu, 0xffffffffu, 0xffffffffu, 0x0fffffffu};
    const Fe sqrtm1 = {{0x4a0ea0b0u, 0xc4ee1b27u, 0xad2fe478u, 0x2f431806u,
                        0x3dfbd7a7u, 0x2b4d0099u, 0x4fc1df0bu, 0x2b832480u}};
    Fe x = Fp::pow(a, e);
    Fe x2 = Fp::sqr(x);
    if (!Fp::eq(x2, a)) {
        if (!Fp::eq(x2, Fp::neg(a)))
            return false;
        x = Fp::mul(x, sqrtm1);
    }
    r = x;
    return true;
}

template <>
__device__ inline bool fsqrt<SeleneCurve>(Fe &r, const Fe &a)
{
    // q = 3 (mod 4): x = a^((q+1)/4)
    const uint32_t e[8] = {0x9e49f1e8u, 0x1badb49cu, 0x2dd95ad6u, 0xefdfde0bu,
                           0xffffffffu, 0xffffffffu, 0xffffffffu, 0x1fffffffu};
    Fe x = Fq::pow(a, e);
    if (!Fq::eq(Fq::sqr(x), a))
        return false;
    r = x;
    return true;
}

template <class C>
__global__ void k_map_to_curve(const uint4 *__restrict__ u, size_t n, uint4 *__restrict__ out)
{
    using F = typename C::F;
    using G = Group<C>;
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    Fe uu = load_fe(u + 2 * i);
    uu.w[7] &= 0x7fffffffu;  // fp_frombytes masks bit 255
    const Fe A = F::neg(F::from_u32(3));
    const Fe Z = (C::SSWU_Z < 0) ? F::neg(F::from_u32((uint32_t)(-C::SSWU_Z))) : F::from_u32((uint32_t)C::SSWU_Z);
    const Fe B = G::b();
    Fe u2 = F::sqr(uu);
    Fe Zu2 = F::mul(Z, u2);
    Fe den = F::add(F::sqr(Zu2), Zu2);
    Fe x1;
    if (F::is_zero(den)) {
        x1 = F::mul(B, F::inv(F::mul(Z, A)));  // B / (Z A)
    } else {
        // x1 = (-B/A) (1 + 1/den) = -B (den + 1) / (A den)
        Fe num = F::neg(F::mul(B, F::add(den, F::one())));
        x1 = F::mul(num, F::inv(F::mul(A, den)));
    }
    Fe gx1 = F::add(F::sub(F::mul(F::sqr(x1), x1), F::add(F::dbl(x1), x1)), B);
    Fe x, y;
    if (fsqrt<C>(y, gx1)) {
        x = x1;
    } else {
        x = F::mul(Zu2, x1);
        Fe gx2 = F::add(F::sub(F::mul(F::sqr(x), x), F::add(F::dbl(x), x)), B);
        fsqrt<C>(y, gx2);
    }
    y = F::canon(y);
    Fe uc = F::canon(uu);
    if ((uc.w[0] & 1u) != (y.w[0] & 1u))
        y = F::canon(F::neg(y));
    store_fe(out + 4 * i, F::canon(x));
    store_fe(out + 4 * i + 2, y);
}

template <class C>
cudaError_t map_to_curve(Context &ctx, const void *d_u, size_t n, uint4 *d_out)
{
    if (n == 0)
        return cudaSuccess;
    const int threads = 64;
    k_map_to_curve<C><<<(unsigned)((n + threads - 1) / threads), threads, 0, ctx.stream>>>(
        reinterpret_cast<const uint4 *>(d_u), n, d_out);
    HS_LAUNCH_CHECK(ctx);
    return cudaSuccess;
}

// ---------------------------------------------------------------------------
// point decoding (helios/src/x64/helios_frombytes.cpp:59-109, selene twin):
// bit 255 is the parity of y; x must be canonical (the reference re-encodes and
// compares); y = sqrt(x^3 - 3x + b), negated when its parity differs.  An
// invalid encoding (x >= m, or no square root: this includes the 32 zero bytes
// of the identity's encoding) gives (0, 0), valid[i] = 0 and one count in *bad.
// ---------------------------------------------------------------------------
template <class C>
__global__ void k_decompress(const uint4 *__restrict__ in, size_t n, uint4 *__restrict__ out,
                             uint8_t *__restrict__ valid, uint32_t *__restrict__ bad)
{
    using F = typename C::F;
    using G = Group<C>;
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    Fe x = load_fe(in + 2 * i);
    const uint32_t parity = x.w[7] >> 31;
    x.w[7] &= 0x7fffffffu;
    const Fe xc = F::canon(x);
    bool ok = true;
#pragma unroll
    for (int k = 0; k < 8; k++)
        ok = ok && (xc.w[k] == x.w[k]);
    Fe y = F::zero();
    if (ok) {
        const Fe rhs = F::add(F::sub(F::mul(F::sqr(x), x), F::add(F::dbl(x), x)), G::b());
        ok = fsqrt<C>(y, rhs);
    }
    if (ok) {
        y = F::canon(y);
        if ((y.w[0] & 1u) != parity)
            y = F::canon(F::neg(y));
    } else {
        x = F::zero();
        y = F::zero();
        atomicAdd(bad, 1u);
    }
    store_fe(out + 4 * i, x);
    store_fe(out + 4 * i + 2, y);
    if (valid)
        valid[i] = ok ? 1 : 0;
}

template <class C>
cudaError_t decompress(Context &ctx, const void *d_in, size_t n, uint4 *d_out, uint8_t *d_valid, uint32_t *d_bad)
{
    if (n == 0)
        return cudaSuccess;
    const int threads = 64;
    k_decompress<C><<<(unsigned)((n + threads - 1) / threads), threads, 0, ctx.stream>>>(
        reinterpret_cast<const uint4 *>(d_in), n, d_out, d_valid, d_bad);
    HS_LAUNCH_CHECK(ctx);
    return cudaSuccess;
}

// any input format -> canonical Jacobian (24 words); affine inputs get Z = 1,
// the affine identity (0,0) becomes (1:1:0)
template <class C>
__global__ void k_to_jac24(const uint64_t *__restrict__ in, int fmt, size_t n, uint32_t *__restrict__ out)
{
    using F = typename C::F;
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    Fe X, Y, Z;
    if (fmt == HS_FMT_JACOBIAN51) {
        X = fe_from_51<C>(in + 15 * i);
        Y = fe_from_51<C>(in + 15 * i + 5);
        Z = fe_from_51<C>(in + 15 * i + 10);
    } else {
        if (fmt == HS_FMT_AFFINE51) {
            X = fe_from_51<C>(in + 10 * i);
            Y = fe_from_51<C>(in + 10 * i + 5);
        } else {
            const uint4 *src = reinterpret_cast<const uint4 *>(in) + 4 * i;
            X = load_fe(src);
            Y = load_fe(src + 2);
        }
        const bool ident = F::is_zero(X) && F::is_zero(Y);
        Z = ident ? F::zero() : F::one();
        if (ident) {
            X = F::one();
            Y = F::one();
        }
    }
    X = F::canon(X);
    Y = F::canon(Y);
    Z = F::canon(Z);
#pragma unroll
    for (int k = 0; k < 8; k++) {
        out[24 * i + k] = X.w[k];
        out[24 * i + 8 + k] = Y.w[k];
        out[24 * i + 16 + k] = Z.w[k];
    }
}

template <class C>
cudaError_t to_jac24(Context &ctx, const void *d_in, int fmt, size_t n, uint32_t *d_out)
{
    if (n == 0)
        return cudaSuccess;
    const int threads = 128;
    k_to_jac24<C><<<(unsigned)((n + threads - 1) / threads), threads, 0, ctx.stream>>>(
        reinterpret_cast<const uint64_t *>(d_in), fmt, n, d_out);
    HS_LAUNCH_CHECK(ctx);
    return cudaSuccess;
}

template <class C>
__global__ void k_field_op(int op, const uint4 *__restrict__ a, const uint4 *__restrict__ b, size_t n,
                           uint4 *__restrict__ out)
{
    using F = typename C::F;
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const Fe x = load_fe(a + 2 * i);
    const Fe y = (op == 2 || op == 3 || op == 0) ? load_fe(b + 2 * i) : F::zero();
    Fe r;
    switch (op) {
    case 0: r = F::mul(x, y); break;
    case 1: r = F::sqr(x); break;
    case 2: r = F::add(x, y); break;
    case 3: r = F::sub(x, y); break;
    case 4: r = x; break;
    case 5: r = F::inv(x); break;
    default: r = F::neg(x); break;
    }
    store_fe(out + 2 * i, F::canon(r));
}

// The lane-sliced field of the Horner chain, one warp per element: op 7
// a*b, 8 (a - b)(a + b) (a subtraction's bound), 9 a^(2^32) by 32 squarings
// (repeated products of products), 10 the conversion in and out.
template <class C>
__global__ void k_field_lane_op(int op, const uint4 *__restrict__ a, const uint4 *__restrict__ b, size_t n,
                                uint4 *__restrict__ out)
{
    using F = typename C::F;
    using LF = LaneField<F>;
    const size_t i = blockIdx.x * (size_t)(blockDim.x / 32) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (i >= n)  // whole warps leave together
        return;
    const typename LF::Regs g = LF::regs(lane);
    const uint32_t x = LF::from_fe(load_fe(a + 2 * i), lane);
    const uint32_t y = op == 7 || op == 8 ? LF::from_fe(load_fe(b + 2 * i), lane) : 0u;
    uint32_t r;
    switch (op) {
    case 7: r = LF::mul(x, y, lane, g); break;
    case 8: r = LF::mul(LF::sub(x, y, g.z), x + y, lane, g); break;
    case 9:
        r = x;
        for (int k = 0; k < 32; k++)
            r = LF::mul(r, r, lane, g);
        break;
    default: r = x; break;
    }
    const Fe f = LF::to_fe(r, lane);
    if (lane == 0)
        store_fe(out + 2 * i, F::canon(f));
}

template <class C>
cudaError_t field_op(Context &ctx, int op, const void *d_a, const void *d_b, size_t n, void *d_out)
{
    if (n == 0)
        return cudaSuccess;
    const int threads = 128;
    if (op >= 7) {
        k_field_lane_op<C><<<(unsigned)((n + 3) / 4), threads, 0, ctx.stream>>>(op, (const uint4 *)d_a,
                                                                               (const uint4 *)d_b, n, (uint4 *)d_out);
        HS_LAUNCH_CHECK(ctx);
        return cudaSuccess;
    }
    k_field_op<C><<<(unsigned)((n + threads - 1) / threads), threads, 0, ctx.stream>>>(
        op, (const uint4 *)d_a, (const uint4 *)d_b, n, (uint4 *)d_out);
    HS_LAUNCH_CHECK(ctx);
    return cudaSuccess;
}

// ---------------------------------------------------------------------------
// fixed-base window tables: table[i*W + k] = 2^(c k) * G_i, affine
// ---------------------------------------------------------------------------
template <class C>
__global__ void k_fb_expand(const uint4 *__restrict__ gens, size_t n, int c, int W, uint4 *__restrict__ tmp)
{
    using G = Group<C>;
    using F = typename C::F;
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    Fe x, y;
    load_affine(gens, (uint32_t)i, x, y);
    Xyzz acc = (F::is_exact_zero(x) && F::is_exact_zero(y)) ? G::inf() : G::from_affine(x, y);
    for (int k = 0; k < W; k++) {
        store_xyzz(tmp + 8 * ((size_t)i * W + k), acc);
        if (k + 1 < W)
            for (int d = 0; d < c; d++)
                acc = G::dbl(acc);
    }
}

// XYZZ -> affine in chunks of 16 with one inversion per chunk (Montgomery's
// trick on ZZ*ZZZ); identity -> (0,0)
template <class C>
__global__ void k_fb_normalize(const uint4 *__restrict__ tmp, size_t m, uint4 *__restrict__ table,
                               uint4 *__restrict__ prefix)
{
    using G = Group<C>;
    using F = typename C::F;
    const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    const size_t lo = t * AFF_CHUNK;
    if (lo >= m)
        return;
    const size_t hi = lo + AFF_CHUNK < m ? lo + AFF_CHUNK : m;
    Fe run = F::one();
    for (size_t i = lo; i < hi; i++) {
        const Xyzz p = load_xyzz(tmp + 8 * i);
        if (!G::is_inf(p))
            run = F::mul(run, F::mul(p.ZZ, p.ZZZ));
        store_fe(prefix + 2 * i, run);
    }
    Fe inv = F::inv(run);
    for (size_t i = hi; i-- > lo;) {
        const Xyzz p = load_xyzz(tmp + 8 * i);
        Fe x = F::zero(), y = F::zero();
        if (!G::is_inf(p)) {
            const Fe z = F::mul(p.ZZ, p.ZZZ);
            const Fe prev = (i > lo) ? load_fe(prefix + 2 * (i - 1)) : F::one();
            const Fe zi = F::mul(inv, prev);  // 1 / (ZZ ZZZ)
            inv = F::mul(inv, z);
            x = F::canon(F::mul(p.X, F::mul(p.ZZZ, zi)));
            y = F::canon(F::mul(p.Y, F::mul(p.ZZ, zi)));
        }
        store_fe(table + 4 * i, x);
        store_fe(table + 4 * i + 2, y);
    }
}

template <class C>
cudaError_t fixed_table(Context &ctx, const uint4 *d_gens, size_t n, int c, int W, uint4 *d_tmp, uint4 *d_table)
{
    if (n == 0)
        return cudaSuccess;
    const size_t m = n * (size_t)W;
    uint4 *prefix = d_tmp + 8 * m;  // tmp holds m XYZZ points then m prefix products
    k_fb_expand<C><<<(unsigned)((n + 127) / 128), 128, 0, ctx.stream>>>(d_gens, n, c, W, d_tmp);
    HS_LAUNCH_CHECK(ctx);
    const size_t chunks = (m + AFF_CHUNK - 1) / AFF_CHUNK;
    k_fb_normalize<C><<<(unsigned)((chunks + 127) / 128), 128, 0, ctx.stream>>>(d_tmp, m, d_table, prefix);
    HS_LAUNCH_CHECK(ctx);
    return cudaSuccess;
}

// out = a + b over canonical Jacobians (the two halves of a window-split MSM)
template <class C>
__device__ Xyzz xyzz_from_jac24(const uint32_t *j)
{
    using F = typename C::F;
    using G = Group<C>;
    Fe X, Y, Z;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        X.w[k] = j[k];
        Y.w[k] = j[8 + k];
        Z.w[k] = j[16 + k];
    }
    if (F::is_zero(Z))
        return G::inf();
    Xyzz p;
    p.X = X;
    p.Y = Y;
    p.ZZ = F::sqr(Z);
    p.ZZZ = F::mul(p.ZZ, Z);
    return p;
}

template <class C>
__global__ void k_join(const uint32_t *__restrict__ a, const uint32_t *__restrict__ b, size_t count,
                       uint32_t *__restrict__ out)
{
    using G = Group<C>;
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= count)
        return;
    store_jacobian_canon<C>(out + 24 * i, G::add(xyzz_from_jac24<C>(a + 24 * i), xyzz_from_jac24<C>(b + 24 * i)));
}

template <class C>
cudaError_t join(Context &ctx, const uint32_t *d_a, const uint32_t *d_b, size_t count, uint32_t *d_out)
{
    if (count == 0)
        return cudaSuccess;
    const int threads = 64;
    k_join<C><<<(unsigned)((count + threads - 1) / threads), threads, 0, ctx.stream>>>(d_a, d_b, count, d_out);
    HS_LAUNCH_CHECK(ctx);
    return cudaSuccess;
}

// ---------------------------------------------------------------------------
// independent variable-time scalar multiplications s_i * P_i
// (helios/include/helios_scalarmult_vartime.h:39-57, the n = 1 case of the MSM)
// ---------------------------------------------------------------------------
// One thread per pair: signed 4-bit digits d_0..d_64 in [-8, 8] (the recode of
// the MSM with c = 4, carry kept), a table of P..8P in XYZZ, then from the top
// digit four doublings and one addition of +-|d| P per digit.
template <class C>
__global__ void __launch_bounds__(128) k_scalar_mul(const uint4 *__restrict__ scalars, const uint4 *__restrict__ pts,
                                                   size_t n, uint32_t *__restrict__ out)
{
    using G = Group<C>;
    using F = typename C::F;
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    Fe x, y;
    load_affine(pts, (uint32_t)i, x, y);
    Xyzz Q = G::inf();
    if (!(F::is_exact_zero(x) && F::is_exact_zero(y))) {
        const uint4 sa = __ldg(scalars + 2 * i), sb = __ldg(scalars + 2 * i + 1);
        const uint32_t s[8] = {sa.x, sa.y, sa.z, sa.w, sb.x, sb.y, sb.z, sb.w};
        int8_t d[65];
        uint32_t carry = 0;
#pragma unroll
        for (int k = 0; k < 65; k++) {
            const uint32_t v = (k < 64 ? (s[k >> 3] >> (4 * (k & 7))) & 15u : 0u) + carry;
            if (k < 64 && v >= 8u) {
                d[k] = (int8_t)((int)v - 16);
                carry = 1;
            } else {
                d[k] = (int8_t)v;
                carry = 0;
            }
        }
        Xyzz T[8];
        T[0] = G::from_affine(x, y);
        T[1] = G::dbl(T[0]);
        for (int j = 2; j < 8; j++) {
            T[j] = T[j - 1];
            G::add_affine(T[j], x, y);
        }
        for (int k = 64; k >= 0; k--) {
            if (k < 64)
                for (int b = 0; b < 4; b++)
                    Q = G::dbl(Q);
            const int dk = d[k];
            if (dk != 0)
                Q = G::add(Q, dk > 0 ? T[dk - 1] : G::neg(T[-dk - 1]));
        }
    }
    store_jacobian_canon<C>(out + 24 * i, Q);
}

template <class C>
cudaError_t scalar_mul(Context &ctx, const void *d_scalars, const uint4 *d_points, size_t n, uint32_t *d_out)
{
    if (n == 0)
        return cudaSuccess;
    const int threads = 128;
    k_scalar_mul<C><<<(unsigned)((n + threads - 1) / threads), threads, 0, ctx.stream>>>(
        static_cast<const uint4 *>(d_scalars), d_points, n, d_out);
    HS_LAUNCH_CHECK(ctx);
    return cudaSuccess;
}

template <class C>
CurveOps make_ops()
{
    return CurveOps{&msm_tail<C>, &to_affine<C>, &to_affine_scratch, &format_out<C>, &map_to_curve<C>,
                    &to_jac24<C>, &field_op<C>,  &fixed_table<C>,    &join<C>,       &decompress<C>,
                    &scalar_mul<C>};
}

}  // namespace hs
