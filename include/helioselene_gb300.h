/*
 * helioselene_gb300.h -- C ABI of the GB300 variable-time MSM for the
 * Helios/Selene curve cycle.
 *
 * Drop-in boundary for helioselene's public-data MSM path.  Every entry point
 * takes plain pointers and sizes; nothing here exposes CUDA or any framework
 * type.  The library computes on one CUDA device and never falls back to
 * the CPU: if the device work fails, the call returns an error status (or,
 * for the void-returning reference-signature entry points, prints the
 * reason and aborts).
 *
 * Point formats (per point, little endian):
 *   HS_FMT_JACOBIAN51  120 bytes: X[5], Y[5], Z[5] uint64 radix-2^51 limbs,
 *                      the layout of helios_jacobian / selene_jacobian on
 *                      64-bit hosts (helios/include/helios.h:41-46,
 *                      fp/include/fp.h:42-46).  Limbs may be non-canonical;
 *                      Z may be anything; Z == 0 is the identity.
 *   HS_FMT_AFFINE51     80 bytes: x[5], y[5] radix-2^51 limbs
 *                      (helios_affine, helios/include/helios.h:48-52);
 *                      (0,0) is the identity.
 *   HS_FMT_AFFINE       64 bytes: x || y as 32-byte little-endian integers;
 *                      64 zero bytes are the identity.  The device-resident
 *                      layout.
 *   HS_FMT_COMPRESSED   32 bytes: the reference serialization (x with the
 *                      parity of y in bit 255; identity = 32 zero bytes,
 *                      helios/src/x64/helios_tobytes.cpp:42-66).  Output only.
 * Scalars are 32-byte little-endian integers; any 256-bit value is accepted
 * and the result is the exact sum (the reference additionally drops a
 * recode carry for 864 <= n < 2592, helios/src/x64/helios_msm_vartime.cpp:
 * 127-162 and 248-263; this library does not reproduce that defect).
 */
#ifndef HELIOSELENE_GB300_H
#define HELIOSELENE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define HS_OK 0
#define HS_EINVAL (-1)    /* bad argument (null pointer with n > 0, unknown format/curve) */
#define HS_ENOMEM (-2)    /* device or pinned-host allocation refused */
#define HS_ECUDA (-3)     /* a CUDA call failed; hs_last_error() has the text */
#define HS_ETIMEDOUT (-4) /* a bounded device wait ran out */
#define HS_EBUSY (-5)     /* serving queue full / admission refused */
#define HS_ERANGE (-6)    /* size beyond a documented maximum */

/* ---- curves and formats ---- */
#define HS_HELIOS 0
#define HS_SELENE 1

#define HS_FMT_JACOBIAN51 0
#define HS_FMT_AFFINE51 1
#define HS_FMT_AFFINE 2
#define HS_FMT_COMPRESSED 3

/* The reference's point structs on 64-bit hosts (helios/include/helios.h:41-52,
 * selene/include/selene.h:41-52). */
typedef struct hs_jacobian51 {
    uint64_t X[5];
    uint64_t Y[5];
    uint64_t Z[5];
} hs_jacobian51;

typedef struct hs_affine51 {
    uint64_t x[5];
    uint64_t y[5];
} hs_affine51;

typedef struct hs_context hs_context;

/* ---- context ----
 * A context owns one CUDA stream, a grow-only device workspace and pinned
 * staging buffers on one device.  Calls on one context are serialised by an
 * internal lock; use one context per host thread for concurrency. */
int hs_context_create(hs_context **ctx, int device);
void hs_context_destroy(hs_context *ctx);
/* last error text of this context (or of the calling thread when ctx is NULL) */
const char *hs_last_error(const hs_context *ctx);
const char *hs_strerror(int status);
/* kernels launched on this context since creation (instrumentation) */
uint64_t hs_context_launches(const hs_context *ctx);
/* the context's cudaStream_t, as an opaque pointer */
void *hs_context_stream(hs_context *ctx);
/* Bucket accumulation form of one curve's plans of at least min_entries
 * (point, window) entries: `rounds` (1..3) rounds of pairwise affine
 * additions, each round sharing one field inversion per 2048 additions
 * (Montgomery's trick, fp/include/fp_batch_invert.h:61-114, across a wave of
 * bucket additions), then an XYZZ fold of what is left; 0 keeps the XYZZ mixed
 * additions of every entry (helios/src/x64/helios_msm_vartime.cpp:296-325 is
 * the bucket loop both replace).  Results are identical either way.  Default:
 * one round on Helios and two on Selene, from 2^21 entries, except in two
 * kinds of plans where a curve's MSMs mostly run alone: fixed-base commitments
 * and single MSMs from host buffers take no round on Helios and one on
 * Selene, until this call sets the curve.  rounds = -1 restores the defaults.  Host-input calls
 * send their bases in two parts either way: with rounds, each part's entries
 * of a bucket form their own list, whose rounds run once that part is in. */
int hs_context_set_batch_affine(hs_context *ctx, int curve, int rounds, size_t min_entries);
/* set the Pippenger window width for one curve; 0 restores the built-in
 * cost model (the autotuner writes this) */
int hs_context_set_window(hs_context *ctx, int curve, size_t n_min, size_t n_max, int window);
/* the same, with the batch-affine rounds (0..3) of plans whose entries lie
 * mostly in this size class (-1: the curve's setting, hs_context_set_batch_affine);
 * the autotuner writes both */
int hs_context_set_rule(hs_context *ctx, int curve, size_t n_min, size_t n_max, int window, int ba_rounds);
/* capture launch sequences as CUDA graphs and replay them for repeated shapes
 * (on by default); off launches every kernel directly */
int hs_context_set_graphs(hs_context *ctx, int on);
/* single MSMs of at least min_points run as two window halves on two streams
 * joined by one addition, so the long doubling chain of the upper half overlaps
 * the accumulation of the lower half (default 2^18; 0 turns the split off, for
 * callers that already overlap several MSMs on the device) */
int hs_context_set_split(hs_context *ctx, size_t min_points);
/* replace the context stream by one of the greatest (high != 0) or the default
 * (high == 0) priority: when several contexts share a device, the blocks of a
 * high-priority context are scheduled first, so its MSMs finish first and the
 * others fill the SMs its latency-bound tail leaves idle.  The stream handle
 * (hs_context_stream) changes. */
int hs_context_set_priority(hs_context *ctx, int high);

/* ---- MSM: sum of scalars[i] * points[i] ----
 * Replaces helios_msm_vartime / selene_msm_vartime
 * (helios/include/helios_msm_vartime.h:45-71, selene/include/selene_msm_vartime.h)
 * and HeliosPoint/SelenePoint::multi_scalar_mul (include/helioselene_point.h:166-167,
 * src/api_point.cpp:98-116, 202-220).
 * Host buffers.  out: one point in out_fmt (JACOBIAN51 or COMPRESSED or AFFINE).
 * n == 0 gives the identity, as in the reference (helios_msm_vartime.cpp:402-406).
 * One call handles n x W(c) < 2^31 (point, window) entries, about 126M points
 * at c = 16; beyond that it returns HS_ERANGE and the caller sums the results
 * of slices (they add as points).
 * The host-to-device copies of every context on a device go through one copy
 * stream in call order; the scalars go first, and bases of more than 2^17
 * points go in two parts whose first is accumulated while the second is in
 * transit.  Pinned host memory is copied by the copy engine.  Pageable memory
 * (an ordinary array) is read by a copy kernel where the device reads pageable
 * host memory (Grace-class hosts), which keeps the copies asynchronous too;
 * elsewhere the copy engine stages it, which holds the calling thread for each
 * copy.  hs_msm_batch gathers a curve group's copies into one copy kernel
 * there when they come from pageable memory or the group has more than 16
 * MSMs. */
int hs_msm(hs_context *ctx, int curve, const uint8_t *scalars, const void *points, int point_fmt, size_t n,
           void *out, int out_fmt);

/* Same on device-resident data: d_scalars n*32 bytes, d_points n*64 bytes
 * (HS_FMT_AFFINE), d_out one point in out_fmt, all device pointers; runs on
 * the context stream and does not synchronise. */
int hs_msm_device(hs_context *ctx, int curve, const void *d_scalars, const void *d_points, size_t n, void *d_out,
                  int out_fmt);

/* ---- Pedersen commitment r*H + sum values[i] * generators[i] ----
 * Replaces helios_pedersen_commit / selene_pedersen_commit
 * (helios/include/helios_pedersen.h:55-86) and HeliosPoint::pedersen_commit
 * (include/helioselene_point.h:170-174, src/api_point.cpp:118-144).
 * H and generators use point_fmt; one MSM of n+1 terms. */
int hs_pedersen(hs_context *ctx, int curve, const uint8_t blinding[32], const void *H, const uint8_t *values,
                const void *generators, int point_fmt, size_t n, void *out, int out_fmt);

/* ---- batch Jacobian -> affine with one shared inversion per chunk ----
 * Replaces helios_batch_to_affine / selene_batch_to_affine
 * (helios/include/helios_batch_affine.h:55-98): identity -> (0,0).
 * in: n points in HS_FMT_JACOBIAN51; out: n points in HS_FMT_AFFINE51 or HS_FMT_AFFINE. */
int hs_batch_to_affine(hs_context *ctx, int curve, const void *in, size_t n, void *out, int out_fmt);

/* ---- serialization of n points (the reference's to_bytes, helios_tobytes.cpp:42-66) ----
 * in: n points in in_fmt (JACOBIAN51, AFFINE51 or AFFINE); out: n*32 bytes. */
int hs_compress(hs_context *ctx, int curve, const void *in, int in_fmt, size_t n, uint8_t *out);

/* ---- independent variable-time scalar multiplications: out[i] = scalars[i] * points[i] ----
 * Replaces helios_scalarmult_vartime / selene_scalarmult_vartime
 * (helios/include/helios_scalarmult_vartime.h:39-57), batched: one thread per
 * pair, any 32-byte scalar.  points in point_fmt (any input form); out n
 * records of out_fmt. */
int hs_scalar_mul(hs_context *ctx, int curve, const uint8_t *scalars, const void *points, int point_fmt, size_t n,
                  void *out, int out_fmt);
/* device form: d_scalars n*32 bytes, d_points n*64 bytes (HS_FMT_AFFINE), d_out n
 * records of out_fmt; on the context stream, does not synchronise */
int hs_scalar_mul_device(hs_context *ctx, int curve, const void *d_scalars, const void *d_points, size_t n, void *d_out,
                         int out_fmt);

/* ---- decoding of n 32-byte encodings (helios/src/x64/helios_frombytes.cpp:59-109,
 * selene twin; HeliosPoint::from_bytes, src/api_point.cpp:58-64) ----
 * out: n points in HS_FMT_AFFINE, HS_FMT_AFFINE51 or HS_FMT_JACOBIAN51; valid:
 * n bytes (1 = decoded) or NULL.  An encoding the reference rejects (x not
 * canonical, no square root; this includes the identity's 32 zero bytes) is
 * written as the identity with valid[i] = 0, and the call returns HS_EINVAL.
 * The MSM forms (hs_msm, hs_pedersen, hs_msm_batch, hs_fixed_base_create) also
 * take point_fmt = HS_FMT_COMPRESSED, decode on the device and return HS_EINVAL
 * when any input point is invalid. */
int hs_decompress(hs_context *ctx, int curve, const uint8_t *in, size_t n, void *out, int out_fmt, uint8_t *valid);
/* device form: d_in n*32 bytes -> d_out n*64 bytes (HS_FMT_AFFINE), d_valid n
 * bytes; on the context stream, does not synchronise */
int hs_decompress_device(hs_context *ctx, int curve, const void *d_in, size_t n, void *d_out, uint8_t *d_valid);

/* ---- simplified SWU map of n field elements (helios/src/x64/helios_map_to_curve.cpp:98-198,
 * selene twin); u: n*32 bytes (bit 255 ignored); out: n points in out_fmt ----
 * Used to derive bases / generators (HeliosPoint::map_to_curve, api_point.cpp:146-151). */
int hs_map_to_curve(hs_context *ctx, int curve, const uint8_t *u, size_t n, void *out, int out_fmt);
int hs_map_to_curve_device(hs_context *ctx, int curve, const void *d_u, size_t n, void *d_out_affine);

/* ---- batched MSMs: many independent MSMs of uneven size, either curve ----
 * One fused launch sequence over all of them (captured in a CUDA graph and
 * replayed when the same shape is submitted again).  descs[i] names MSM i;
 * all pointers are host pointers; outputs are written in out_fmt. */
typedef struct hs_msm_desc {
    int curve;
    size_t n;
    const uint8_t *scalars;
    const void *points; /* point_fmt of the call */
    void *out;
} hs_msm_desc;
int hs_msm_batch(hs_context *ctx, const hs_msm_desc *descs, size_t count, int point_fmt, int out_fmt);

/* Batched MSMs on device-resident data, all on one curve: MSM i has sizes[i]
 * points whose scalars (32 bytes each) and HS_FMT_AFFINE points (64 bytes each)
 * follow those of MSM i-1 in d_scalars / d_points; d_out receives count
 * records of out_fmt.  One launch sequence serves the whole batch: recode and
 * counting sort over all MSMs' buckets, one accumulation launch, reductions
 * indexed by MSM, and one warp per MSM for the window combination.  Window
 * widths come from the context's rules (hs_context_set_window) or the cost
 * model, per MSM size.  Runs on the context stream; does not synchronise. */
int hs_msm_batch_device(hs_context *ctx, int curve, const size_t *sizes, size_t count, const void *d_scalars,
                        const void *d_points, void *d_out, int out_fmt);

/* ---- fixed-base commitments over a resident generator set ----
 * Pedersen-style r*H + sum v_i G_i (helios/include/helios_pedersen.h:55-86) for
 * many commitments over the same generators.  hs_fixed_base_create uploads the
 * n generators (and H, appended as generator n when given), then precomputes on
 * the device, for window width c, the table 2^(c k) G_i for every window k
 * (the vartime counterpart of the reference's per-base multiple tables,
 * helios/include/helios_scalarmult_fixed.h:54-63, helios_msm_fixed.h:60-155).
 * A commitment then adds every (generator, window) digit into one set of
 * 2^(c-1) buckets: one bucket reduction, no per-window doublings.  window 0
 * picks c from the generator count.  The table stays resident until destroy. */
typedef struct hs_fixed_base hs_fixed_base;
int hs_fixed_base_create(hs_context *ctx, int curve, const void *generators, int point_fmt, size_t n, const void *H,
                         int window, hs_fixed_base **fb);
/* values: count x n scalars (32 bytes each, commitment-major); blindings:
 * count scalars or NULL (then r = 0; required NULL when created without H);
 * out: count records of out_fmt (HS_FMT_AFFINE outputs are normalised with
 * one shared inversion per 16 commitments). */
int hs_fixed_base_commit(hs_context *ctx, const hs_fixed_base *fb, const uint8_t *values, const uint8_t *blindings,
                         size_t count, void *out, int out_fmt);
/* device variant: d_scalars holds count x g scalars, g = n (+1 with H, the
 * blinding last in each commitment); d_out count records; does not synchronise */
int hs_fixed_base_commit_device(hs_context *ctx, const hs_fixed_base *fb, const void *d_scalars, size_t count,
                                void *d_out, int out_fmt);
/* window width and device bytes of the table */
int hs_fixed_base_info(const hs_fixed_base *fb, int *window, size_t *table_bytes);
void hs_fixed_base_destroy(hs_fixed_base *fb);

/* ---- serving: continuous batching of MSM requests ----
 * A server owns `slots` CUDA streams, each with its own workspace, a request
 * queue and one scheduler thread.  Requests that arrive while others are on
 * the GPU are admitted as soon as a slot and enough of the HBM budget are
 * free: the scheduler groups queued requests by curve (up to the batch caps),
 * gathers their pool bases on the device, and runs each group as one batched
 * launch sequence (the hs_msm_batch_device pipeline) on a free slot, so
 * batches overlap on the device.  Completion is detected with CUDA events and
 * bounded host waits only.  A request's buffers (scalars, indices, fresh
 * points, out) must stay valid until hs_server_wait has returned for it;
 * a batch's copies from them run asynchronously (on a device that reads
 * pageable host memory, as one gathered copy kernel; elsewhere page-locked
 * buffers keep the copy engine's copies asynchronous).  Results are the
 * same whichever requests share a batch: with HS_FMT_COMPRESSED or
 * HS_FMT_AFFINE the bytes are identical alone and in the mix (a Jacobian
 * result is the same point, its Z depends on the summation order). */
typedef struct hs_server hs_server;

typedef struct hs_server_config {
    int device;
    int slots;               /* batches in flight at once, 1..16; 0 selects 4 */
    size_t hbm_budget;       /* device bytes the in-flight batches may hold; 0 selects half the free memory */
    size_t max_batch_points; /* points per launched batch; 0 selects 2^22 */
    size_t max_batch_msms;   /* requests per launched batch; 0 selects 1024 */
    int out_fmt;             /* result format of every request */
} hs_server_config;

typedef struct hs_request {
    int curve;
    size_t n_pool;            /* leading bases taken from the curve's resident pool */
    const uint32_t *pool_idx; /* n_pool indices into that pool */
    size_t n_fresh;           /* trailing bases given with the request */
    const void *fresh_points; /* n_fresh HS_FMT_AFFINE points */
    const uint8_t *scalars;   /* (n_pool + n_fresh) * 32 bytes */
    void *out;                /* one out_fmt record, written before the request completes */
} hs_request;

typedef struct hs_server_stats {
    uint64_t submitted, completed, failed, batches, max_batch_msms;
    uint64_t peak_bytes;   /* peak device workspace held by in-flight batches */
    uint64_t deferred;     /* launches postponed by the HBM budget */
} hs_server_stats;

int hs_server_create(hs_server **srv, const hs_server_config *cfg);
/* upload (replace) the resident base pool of one curve: n HS_FMT_AFFINE points.
 * Unless the curve's pool window is 0, the pool is also expanded once into a
 * resident table of window multiples 2^(c k) P_i (n * ceil(257/c) affine
 * points, 64 bytes each; a scratch of 160 bytes per table point while it is
 * built): a request whose bases all come from the pool is then a fixed-base
 * MSM over that table (one reduced window, no doubling chain), batched with
 * other such requests; requests with fresh bases gather their pooled bases
 * into a variable-base batch.  Only while nothing is queued or in flight
 * (HS_EBUSY otherwise). */
int hs_server_set_pool(hs_server *srv, int curve, const void *affine_points, size_t n);
/* window width c of the curve's pool table from the next hs_server_set_pool:
 * 4..16, or 0 for no table (every request's pooled bases are gathered into
 * its batch as variable bases).  The default is 12. */
int hs_server_set_pool_window(hs_server *srv, int curve, int window);
/* window rule for the batches of every slot, as hs_context_set_window (window 0
 * clears the curve's rules); applies to batches planned after the call */
int hs_server_set_window(hs_server *srv, int curve, size_t n_min, size_t n_max, int window);
/* queue a request; HS_ERANGE if it alone exceeds the batch caps or the budget,
 * or its n x windows reaches 2^31 (batches are also formed below that bound) */
int hs_server_submit(hs_server *srv, const hs_request *req, uint64_t *ticket);
/* wait up to timeout_ms for a request: HS_OK (result written, latency from
 * submit to completion in *latency_ms), HS_ETIMEDOUT, or the failure status */
int hs_server_wait(hs_server *srv, uint64_t ticket, int timeout_ms, double *latency_ms);
int hs_server_get_stats(hs_server *srv, hs_server_stats *st);
/* stops the scheduler after the in-flight batches finish; queued requests fail */
void hs_server_destroy(hs_server *srv);

/* ---- drop-in entry points with the reference's exact signatures ----
 * Same arguments and meaning as helios_msm_vartime / selene_msm_vartime
 * (helios/include/helios_msm_vartime.h:45-49) and the dispatch-table slots
 * helioselene_dispatch_table::{helios,selene}_msm_vartime
 * (include/helioselene_dispatch.h:49-57).  They use a process-wide context on
 * device 0 (created on first use, thread-safe).  The reference returns void;
 * on a device failure these print the error and abort -- there is no CPU
 * fallback. */
void hs_helios_msm_vartime(hs_jacobian51 *result, const unsigned char *scalars, const hs_jacobian51 *points,
                           size_t n);
void hs_selene_msm_vartime(hs_jacobian51 *result, const unsigned char *scalars, const hs_jacobian51 *points,
                           size_t n);
/* exact signature of helios_scalarmult_vartime / selene_scalarmult_vartime
 * (helios/include/helios_scalarmult_vartime.h:39-57); aborts on a device failure */
void hs_helios_scalarmult_vartime(hs_jacobian51 *result, const unsigned char scalar[32], const hs_jacobian51 *p);
void hs_selene_scalarmult_vartime(hs_jacobian51 *result, const unsigned char scalar[32], const hs_jacobian51 *p);
void hs_helios_pedersen_commit(hs_jacobian51 *result, const unsigned char *blinding, const hs_jacobian51 *H,
                               const unsigned char *values, const hs_jacobian51 *generators, size_t n);
void hs_selene_pedersen_commit(hs_jacobian51 *result, const unsigned char *blinding, const hs_jacobian51 *H,
                               const unsigned char *values, const hs_jacobian51 *generators, size_t n);
void hs_helios_batch_to_affine(hs_affine51 *out, const hs_jacobian51 *points, size_t n);
void hs_selene_batch_to_affine(hs_affine51 *out, const hs_jacobian51 *points, size_t n);

/* ---- instrumentation ----
 * With profiling on, the context records CUDA events around its bucket
 * accumulation launches (the dominant kernel).  hs_profile_read synchronises
 * the context stream and returns the summed device time and launch count
 * since the last reset, plus the algorithmic (point, window) entry count of the
 * profiled MSMs: n x ceil(256/c) per MSM (the full windows of a 256-bit
 * scalar), the unit of the pinned work figure. */
int hs_profile_enable(hs_context *ctx, int on);
int hs_profile_read(hs_context *ctx, double *accumulate_ms, uint64_t *accumulate_launches, uint64_t *entries,
                    int reset);
/* Integer multiply throughput of this device: kernels of independent
 * mad.lo/mad.hi chains and of independent mad.wide.u32 chains on every SM,
 * timed with CUDA events.  Returns the faster, in IMAD-equivalents per second
 * (a 32x32->64 product counts as 2, in either form). */
int hs_measure_imad_peak(hs_context *ctx, double *imad_per_s);
/* The probes behind hs_measure_imad_peak, in instructions per second over the
 * whole device: rates[0] mad.lo/mad.hi alternating (each instruction is one
 * IMAD-equivalent), rates[1] mad.wide.u32 (each is one 32x32->64 product, two
 * IMAD-equivalents), rates[2] mad.lo alone, rates[3] mad.hi alone.  Divide by
 * the SM count and clock for rates per SM per cycle. */
int hs_measure_imad_rates(hs_context *ctx, double rates[4]);

/* Field arithmetic on the device, for validation of the field layer:
 * field HS_HELIOS selects F_p (2^255-19), HS_SELENE selects F_q (2^255-gamma).
 * op: 0 mul, 1 square, 2 add, 3 sub, 4 canonical reduce, 5 invert (0 -> 0), 6 negate;
 * the lane-sliced form of the window combination: 7 mul, 8 (a - b)(a + b),
 * 9 a^(2^32) by repeated squaring, 10 conversion in and out (canonical reduce).
 * a, b, out: n little-endian 32-byte values in host memory (b unused for unary ops);
 * inputs may be any 256-bit value, outputs are canonical. */
int hs_field_op(hs_context *ctx, int field, int op, const uint8_t *a, const uint8_t *b, size_t n, uint8_t *out);

/* ---- MSM without device allocation ----
 * For callers that cannot allocate device memory while they run: code under
 * an allocator or memory pool that must not be bypassed, processes whose
 * device memory is reserved up front, and latency-critical callers that must
 * not reach cudaMalloc / cudaFree (both can synchronise the device).  This
 * entry point has no counterpart in the reference.
 * Same computation and arguments as hs_msm_device, but every scratch buffer
 * comes from one fixed array of hs_msm_noalloc_scratch_bytes() (64 MiB) in
 * device memory.  Under CUDA's default lazy module loading a device's array
 * is reserved by the first call on that device (at library load under
 * CUDA_MODULE_LOADING=EAGER) and held until the process exits: a caller that
 * reserves its device memory up front should make one call first.
 * It needs no context: it runs on the current device and on `stream` (a
 * cudaStream_t, NULL for the default stream), and writes its descriptor with a
 * kernel on that stream, so it does not synchronise.  n must be
 * 1 .. HS_NOALLOC_MAX_POINTS; larger sizes, and any size whose workspace would
 * not fit the array, return HS_ERANGE.
 * Errors: a CUDA error already pending on the calling thread is left in place
 * and the call returns HS_ECUDA; a failure of the call itself is cleared and
 * described by hs_last_error(NULL).
 * All calls on a device share the one array and find the previous call's
 * contents in it (each call clears what it needs cleared): calls whose work
 * overlaps on the GPU -- on different streams, or from different threads --
 * race and corrupt each other's results; run them one after another. */
#define HS_NOALLOC_MAX_POINTS 262144
int hs_msm_device_noalloc(int curve, const void *d_scalars, const void *d_points, size_t n, void *d_out, int out_fmt,
                          void *stream);
size_t hs_msm_noalloc_scratch_bytes(void);

/* ---- library info ---- */
int hs_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif /* HELIOSELENE_GB300_H */
