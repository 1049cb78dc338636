/*
 * rsbd8g.h - C ABI of the GB300 (sm_103a) stable LSD radix sort.
 *
 * A device-resident drop-in for the sorting entry points of the Radixsortbidi8
 * library (header Radixsortbidi8.hpp, namespace rsbd8).  Every entry point takes
 * plain device pointers and sizes; no C++ or CUDA type crosses this boundary.
 * The C++ template facade in rsbd8.hpp maps the reference's template
 * parameters (key type, sortingmode, sortingdirection, member pointer or
 * type+offset indirection) onto rsbd8g_desc and calls these functions.
 *
 * Semantics are those of the reference: a stable sort by the filtered key of the
 * selected sortingmode, ascending or descending, with ties in input order
 * (forward) or reversed (reverse order), where the reference honours it.
 *
 * Stream use: every call is ordered on the given stream (NULL = the legacy
 * default stream).  The allocating forms (rsbd8g_radixsort, rsbd8g_radixsortcopy)
 * block until the sort is complete, as the reference's functions do, and report
 * device-side errors.  The noalloc forms only enqueue work; call
 * rsbd8g_scratch_status() to wait and read the device-side status word.
 */
#ifndef RSBD8G_H
#define RSBD8G_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define RSBD8G_API __attribute__((visibility("default")))
#else
#define RSBD8G_API
#endif

/* an opaque CUDA stream handle; pass a cudaStream_t (or CUstream) here */
typedef struct CUstream_st *rsbd8g_stream;

typedef enum rsbd8g_status {
    RSBD8G_OK = 0,
    RSBD8G_ERR_BAD_ARG = 1,      /* null pointer, aliasing, bad mode/direction/key size, scratch too small */
    RSBD8G_ERR_NO_MEMORY = 2,    /* device allocation failed (the reference returns false here) */
    RSBD8G_ERR_CUDA = 3,         /* a CUDA runtime call failed */
    RSBD8G_ERR_TIMEOUT = 4,      /* a bounded device-side wait ran out (the look-back of the scatter) */
    RSBD8G_ERR_DEVICE_FAULT = 5, /* the device flagged an internal inconsistency */
    RSBD8G_ERR_TOO_LARGE = 6,    /* count beyond the supported range */
    RSBD8G_ERR_BUSY = 7          /* serving: admission refused, the memory budget is exhausted */
} rsbd8g_status;

/* what std::is_signed_v / std::is_floating_point_v report for the key type:
 * enumerations, bool and classes are RSBD8G_KIND_UNSIGNED, as in the reference.
 * 16-byte keys (two little-endian 64-bit words, 16-byte aligned arrays): UNSIGNED / SIGNED for
 * 128-bit integers, FLOAT for a 128-bit float word with the sign in bit 127 (IEEE binary128, the
 * reference's test128 with the floating-point flag), and RSBD8G_KIND_X87 for x87 extended
 * precision in 16-byte storage (64-bit significand, then sign and 15-bit exponent; the upper
 * 48 bits are padding, ignored by the order and moved with the element: the reference's
 * longdoubletest128, and long double on x86-64) */
enum { RSBD8G_KIND_UNSIGNED = 0, RSBD8G_KIND_SIGNED = 1, RSBD8G_KIND_FLOAT = 2, RSBD8G_KIND_X87 = 3 };

/* rsbd8::sortingmode values (Radixsortbidi8.hpp:212-250) */
enum {
    RSBD8G_MODE_FORCEUNSIGNED = 0, RSBD8G_MODE_SPECIALSIGNED = 0,
    RSBD8G_MODE_FORCETIEREDABSSIGNED = 1, RSBD8G_MODE_FORCESIGNED = 2,
    RSBD8G_MODE_FORCEABSSIGNED = 3, RSBD8G_MODE_SPECIALFLOATINGP = 4,
    RSBD8G_MODE_FORCETIEREDABSFLOATINGP = 5, RSBD8G_MODE_FORCEFLOATINGP = 6,
    RSBD8G_MODE_FORCEABSFLOATINGP = 7, RSBD8G_MODE_SPECIALUNSIGNED = 7,
    RSBD8G_MODE_NATIVE = 64, RSBD8G_MODE_NATIVEABS = 65, RSBD8G_MODE_NATIVETIEREDABS = 66
};

/* rsbd8::sortingdirection values (Radixsortbidi8.hpp:252-265) */
enum {
    RSBD8G_ASCFWDORDER = 0, RSBD8G_DSCFWDORDER = 1,
    RSBD8G_ASCREVORDER = 2, RSBD8G_DSCREVORDER = 3
};

/* indirection kinds */
enum {
    RSBD8G_DIRECT = 0,      /* the arrays hold the keys themselves */
    RSBD8G_MEMBER = 1,      /* the arrays hold object pointers; the key is at byte offset1 of each object
                               (member object pointer or type+offset form) */
    RSBD8G_MEMBER2 = 2,     /* second level: the object holds a pointer at byte offset1, and the key
                               sits at byte offset2 behind that pointer */
    RSBD8G_KEYED = 3        /* rsbd8g_radixsortcopy_keyed only: the keys come in a separate array */
};

/* diagnostics only: tile 1 of every scatter pass never publishes its look-back state, so
 * the tiles after it run into the bounded device-side wait (200 ms) and the call reports
 * RSBD8G_ERR_TIMEOUT with the output undefined; the device stays usable */
#define RSBD8G_FLAG_DIAG_STALL 1u
/* diagnostics only: the allocating forms act as if their device allocation failed (the one
 * failure the reference reports, as a false return): RSBD8G_ERR_NO_MEMORY, arrays untouched */
#define RSBD8G_FLAG_DIAG_NOMEM 2u
/* the caller states that every array of the call -- in the pointer-table segmented form also every
 * array the tables point to -- is device memory (cudaMalloc, a CUDA memory pool).  The scatter
 * passes then prefetch each tile into L2 with a bulk copy before loading it.  The plain forms and
 * the contiguous segmented form find this out themselves (cudaPointerGetAttributes); the
 * pointer-table form prefetches only with this flag.  Managed and host memory are read with plain
 * loads alone. */
#define RSBD8G_FLAG_DEVICE_ARRAYS 4u

typedef struct rsbd8g_desc {
    uint32_t key_bytes;     /* 1, 2, 4, 8 or 16 (x87 keys: not in the segmented and serving entry points) */
    uint32_t key_kind;      /* RSBD8G_KIND_* */
    uint32_t mode;          /* rsbd8::sortingmode value */
    uint32_t direction;     /* rsbd8::sortingdirection value */
    uint32_t indirection;   /* RSBD8G_DIRECT / RSBD8G_MEMBER / RSBD8G_MEMBER2 */
    uint32_t flags;         /* 0, or RSBD8G_FLAG_* */
    int64_t offset1;        /* RSBD8G_MEMBER*: byte offset of the key (or second pointer) in each object */
    int64_t offset2;        /* RSBD8G_MEMBER2: byte offset of the key behind the second pointer */
} rsbd8g_desc;

/* Scratch bytes the noalloc forms need for `count` elements (the index counts,
 * look-back state and, for indirection, the gathered keys).  The ping-pong
 * buffer of `count` elements is separate, as in the reference.
 * Replaces: rsbd8::allocatearray sizing (Radixsortbidi8.hpp:59928). */
RSBD8G_API rsbd8g_status rsbd8g_scratch_bytes(const rsbd8g_desc *desc, size_t count, size_t *bytes);

/* Sort `count` elements of `input` into `output` (input is not written).
 * Allocates its scratch and buffer on the stream, blocks until done.
 * Replaces: rsbd8::radixsortcopy (Radixsortbidi8.hpp:60476, single-part :60536;
 * member pointer :61242; type+offset :61359-61739). */
RSBD8G_API rsbd8g_status rsbd8g_radixsortcopy(const rsbd8g_desc *desc, size_t count,
                                              const void *input, void *output, rsbd8g_stream stream);

/* Sort the `count` 8-byte values of `input` (object pointers) into `output` by the keys in
 * `keys` (count raw keys of desc->key_bytes each, same index), with desc->indirection ==
 * RSBD8G_KEYED.  Allocates, blocks until done.  The C++ facade uses it for getter
 * indirection, whose keys it evaluates on the host.
 * Replaces: rsbd8::radixsortcopy<&V::getter, ...> (Radixsortbidi8.hpp:61242 with a member
 * function pointer; the getter call itself is splitget, Radixsortbidi8.hpp:2405-2719). */
RSBD8G_API rsbd8g_status rsbd8g_radixsortcopy_keyed(const rsbd8g_desc *desc, size_t count, const void *keys,
                                                    const void *input, void *output, rsbd8g_stream stream);

/* The noalloc forms of rsbd8g_radixsortcopy_keyed (desc->indirection == RSBD8G_KEYED): `keys`
 * (count raw keys, device-accessible) are read, not written; scratch as sized by
 * rsbd8g_scratch_bytes for this descriptor; buffer of count 8-byte values.  Stream-ordered.
 * The C++ facade's noalloc getter forms use them.
 * Replaces: rsbd8::radixsortcopynoalloc / radixsortnoalloc with a getter member function
 * (Radixsortbidi8.hpp:60983, :61018). */
RSBD8G_API rsbd8g_status rsbd8g_radixsortcopynoalloc_keyed(const rsbd8g_desc *desc, size_t count, const void *keys,
                                                           void *scratch, size_t scratch_bytes, const void *input,
                                                           void *output, void *buffer, rsbd8g_stream stream);
RSBD8G_API rsbd8g_status rsbd8g_radixsortnoalloc_keyed(const rsbd8g_desc *desc, size_t count, const void *keys,
                                                       void *scratch, size_t scratch_bytes, void *input, void *buffer,
                                                       int movetobuffer, rsbd8g_stream stream);

/* Sort `count` elements of `input` in place.  Allocates, blocks until done.
 * Replaces: rsbd8::radixsort (Radixsortbidi8.hpp:60398). */
RSBD8G_API rsbd8g_status rsbd8g_radixsort(const rsbd8g_desc *desc, size_t count, void *input,
                                          rsbd8g_stream stream);

/* Sort into `output` with caller-provided `buffer` (count elements) and `scratch`
 * (rsbd8g_scratch_bytes, any content: the call clears what it needs).
 * Stream-ordered: returns after enqueueing.
 * Replaces: rsbd8::radixsortcopynoalloc (Radixsortbidi8.hpp:60129; indirect :60983);
 * the reference's allowedthreads / pfuturesplaceholder have no GPU meaning and
 * `scratch` takes the place of pzeroedindices. */
RSBD8G_API rsbd8g_status rsbd8g_radixsortcopynoalloc(const rsbd8g_desc *desc, size_t count,
                                                     void *scratch, size_t scratch_bytes,
                                                     const void *input, void *output, void *buffer,
                                                     rsbd8g_stream stream);

/* In-place sort of `input` using `buffer` (count elements); the result lands in
 * `input`, or in `buffer` when movetobuffer is non-zero (the other array then
 * holds garbage).  Stream-ordered.
 * Replaces: rsbd8::radixsortnoalloc (Radixsortbidi8.hpp:60163; indirect :61018). */
RSBD8G_API rsbd8g_status rsbd8g_radixsortnoalloc(const rsbd8g_desc *desc, size_t count,
                                                 void *scratch, size_t scratch_bytes,
                                                 void *input, void *buffer, int movetobuffer,
                                                 rsbd8g_stream stream);

/* The plain-key copy sort (as rsbd8g_radixsortcopy, direct keys only) without any device
 * allocation.  It has no counterpart in the reference: it exists for callers that must not
 * call cudaMalloc -- plugins whose host framework owns all device memory through its own
 * allocator or a fixed budget, latency-critical paths that cannot take cudaMalloc's implicit
 * synchronisation, or callers that are only handed an input and an output buffer.
 * The scratch and the ping-pong buffer live in one 64 MiB array in the library's device memory
 * (one per GPU, kept until the process exits), so `count` is limited to what fits there:
 * rsbd8g_scratch_bytes(count) + count * key_bytes rounded up to 256 bytes must not exceed
 * 64 MiB -- about 63.1 M one-byte, 30.9 M two-byte, 15.5 M four-byte or 7.45 M eight-byte
 * keys.  Larger counts return RSBD8G_ERR_TOO_LARGE without touching the device.
 * The first call on a device looks up the array's device address (once per device), so make
 * that first call before capturing the stream into a CUDA graph.  Every call reuses the same
 * array and clears the parts that must start at zero; calls whose work overlaps on the GPU
 * (other streams, other host threads) race on it, so order them.  Stream-ordered like the
 * noalloc forms: the return value only says whether the work was enqueued.  A failure on the
 * device (a bounded wait that ran out) sets a status word inside the array and leaves the
 * output undefined; no CUDA error reports it, so a stream synchronisation alone does not see
 * it -- read it with rsbd8g_static_status before the next call on the device clears it. */
RSBD8G_API rsbd8g_status rsbd8g_radixsortcopy_static(const rsbd8g_desc *desc, size_t count,
                                                     const void *input, void *output, rsbd8g_stream stream);

/* Wait for `stream`, then read and clear the device-side status word that the last
 * rsbd8g_radixsortcopy_static call on the current device left in the library's array:
 * RSBD8G_OK, RSBD8G_ERR_TIMEOUT (a bounded device-side wait ran out; that call's output is
 * undefined) or RSBD8G_ERR_DEVICE_FAULT.  Pass the stream the sort was enqueued on.  Allocates
 * nothing.  No counterpart in the reference (its functions report no device state). */
RSBD8G_API rsbd8g_status rsbd8g_static_status(rsbd8g_stream stream);

/* ---- merges of sorted runs, and arrays larger than the device ------------------------------
 * rsbd8g_merge_runs: stable merge of `nruns` runs that lie back to back in `input` (device
 * memory), each sorted by `desc` (direct keys), into `output`; run r holds run_counts[r] elements
 * (run_counts is a host array).  On equal filtered keys the earlier run goes first, or the later
 * run when the direction has reverse order and the mode honours it (as in the sort).  Two runs
 * merge straight into `output`; more runs take `buffer` (as many elements as the runs together;
 * it may be null for two runs).  Stream-ordered; allocates nothing.
 * Replaces: the merges of the halves and thirds that the reference's threads sort
 * (mergehalvesmtc / mergehalvesmain, Radixsortbidi8.hpp:54437, :54815; mergethirdsmtc /
 * mergethirdsmain, :55369, :56014): with run_counts {count / 2, count - count / 2} or
 * {count / 3, (count + 1) / 3, the rest} it merges the same parts into the same order. */
RSBD8G_API rsbd8g_status rsbd8g_merge_runs(const rsbd8g_desc *desc, size_t nruns, const size_t *run_counts,
                                           const void *input, void *output, void *buffer, rsbd8g_stream stream);

/* Sort `count` keys held in HOST memory (input and output host arrays; pinned memory copies
 * fastest), with the semantics of rsbd8g_radixsortcopy, using at most `device_bytes` of device
 * memory (0: nine tenths of the free memory).  An array whose in-place sort (array, ping-pong
 * buffer, scratch) fits that budget is sorted in one piece; a larger one is sorted in chunks that
 * fit, kept as sorted runs in a host buffer, and merged block by block on the device.  Allocates
 * (device memory within the budget, a host buffer of `count` keys), blocks until done.  Direct keys.
 * Replaces: rsbd8::radixsortcopy (Radixsortbidi8.hpp:60476) for arrays that do not fit the GPU;
 * the split into parts sorted apart and merged is the reference's own multithreaded scheme
 * (Radixsortbidi8.hpp:55100-55160). */
RSBD8G_API rsbd8g_status rsbd8g_radixsortcopy_chunked(const rsbd8g_desc *desc, size_t count, const void *input,
                                                      void *output, size_t device_bytes, rsbd8g_stream stream);

/* ---- batched (segmented) sort -------------------------------------------------------------
 * Many independent arrays of uneven sizes in one stream-ordered call: segment s is elements
 * [offsets[s], offsets[s+1]) of `input` (offsets: a device array of nsegs + 1 non-decreasing
 * uint64 values from 0 to total), sorted on its own, with the semantics of rsbd8g_radixsortcopy
 * for desc (direct keys), into the same range of `output`.  Segments of at most the small
 * cutoff are sorted whole in shared memory; larger ones run the onesweep passes, all of them
 * in the same launches.  No host synchronisation happens inside, so the call can be captured
 * into a CUDA graph and replayed.  Each segment must hold fewer than 2^30 keys (a device-side
 * fault flag otherwise, read with rsbd8g_scratch_status).
 * No counterpart in the reference (its callers loop over rsbd8::radixsortcopy per array). */
typedef struct rsbd8g_segtuning {
    uint32_t small_variant;   /* shape of the small-segment block sort: 0, 1 or 2 (threads x items of the block sort, per key size) */
    uint32_t small_cutoff;    /* largest segment sorted whole in shared memory (0 = the shape's capacity) */
    uint32_t large_variant;   /* tile of the large segments' onesweep passes: 0 or 1 (keys per thread, per key size) */
    uint32_t reserved;
} rsbd8g_segtuning;

RSBD8G_API rsbd8g_status rsbd8g_segmented_scratch_bytes(const rsbd8g_desc *desc, size_t total, size_t nsegs,
                                                        const rsbd8g_segtuning *tuning, size_t *bytes);
RSBD8G_API rsbd8g_status rsbd8g_segmented_sortcopy(const rsbd8g_desc *desc, size_t total, size_t nsegs,
                                                   const uint64_t *offsets, void *scratch, size_t scratch_bytes,
                                                   const void *input, void *output, void *buffer,
                                                   const rsbd8g_segtuning *tuning, rsbd8g_stream stream);

/* The same for segments that live in separate device arrays: segment s is input_ptrs[s] ->
 * output_ptrs[s], using buffer_ptrs[s] (each a device pointer, stored in device arrays of nsegs
 * uint64 values); offsets (nsegs + 1 prefix sums of the lengths) only give the lengths.
 * The serving loop launches its coalesced batches through this form. */
RSBD8G_API rsbd8g_status rsbd8g_segmented_sortcopy_ptrs(const rsbd8g_desc *desc, size_t total, size_t nsegs,
                                                        const uint64_t *offsets, const uint64_t *input_ptrs,
                                                        const uint64_t *output_ptrs, const uint64_t *buffer_ptrs,
                                                        void *scratch, size_t scratch_bytes,
                                                        const rsbd8g_segtuning *tuning, rsbd8g_stream stream);

/* The pointer-table form with a direction per segment: `directions` is a device array of nsegs
 * bytes, each the sortingdirection value (0..3) of its segment; desc->direction is not used.  The
 * other fields of desc (key type, mode, flags) hold for every segment.  The serving loop coalesces
 * requests that differ only in direction through this form.  No counterpart in the reference. */
RSBD8G_API rsbd8g_status rsbd8g_segmented_sortcopy_ptrs_dirs(const rsbd8g_desc *desc, size_t total, size_t nsegs,
                                                             const uint64_t *offsets, const uint64_t *input_ptrs,
                                                             const uint64_t *output_ptrs, const uint64_t *buffer_ptrs,
                                                             const uint8_t *directions, void *scratch,
                                                             size_t scratch_bytes, const rsbd8g_segtuning *tuning,
                                                             rsbd8g_stream stream);

/* ---- serving loop -------------------------------------------------------------------------
 * Continuous batching of sort requests on the current device.  rsbd8g_server_create allocates
 * the whole device-memory budget once (buffers, scratch and tables of in-flight batches come out
 * of it) and starts a dispatcher thread.  rsbd8g_server_submit queues one request (device input
 * and output arrays of `count` keys, direct keys only, < 2^30 keys) from any host thread and
 * returns at once; the dispatcher admits pending requests in arrival order while the budget and
 * the `max_inflight` batch slots allow, coalesces admitted requests of the same key type, mode and
 * flags (directions may differ) into one batched launch on its own stream, and retires batches as
 * they finish, so requests arriving while others run are admitted and overlap on the device.  The
 * server's streams are not ordered after any stream of the caller: the input must already hold
 * its keys when it is submitted (the work that wrote it has finished), and neither array may be
 * used by other work until the request is done.  A request that can never fit the budget is
 * refused (RSBD8G_ERR_BUSY).  Times are seconds on a steady host clock.
 * No counterpart in the reference. */
typedef struct rsbd8g_server rsbd8g_server;

typedef struct rsbd8g_request_info {
    rsbd8g_status status;
    uint32_t reserved;
    uint64_t count;
    double submit_s, start_s, done_s;   /* submitted, launched in a batch, batch finished on the device */
} rsbd8g_request_info;

typedef struct rsbd8g_server_counters {
    uint64_t submitted, completed, keys_completed, batches, max_coalesced, max_inflight_batches, pending;
    uint64_t arena_used, budget;
} rsbd8g_server_counters;

RSBD8G_API rsbd8g_status rsbd8g_server_create(size_t budget_bytes, uint32_t max_inflight, rsbd8g_server **server);
RSBD8G_API rsbd8g_status rsbd8g_server_submit(rsbd8g_server *server, const rsbd8g_desc *desc, size_t count,
                                              const void *input, void *output, uint64_t *request_id);
/* wait up to timeout_s for one request; returns its status (RSBD8G_ERR_TIMEOUT if still running) */
RSBD8G_API rsbd8g_status rsbd8g_server_wait(rsbd8g_server *server, uint64_t request_id, double timeout_s,
                                            rsbd8g_request_info *info);
/* wait until nothing is pending or in flight */
RSBD8G_API rsbd8g_status rsbd8g_server_drain(rsbd8g_server *server, double timeout_s);
RSBD8G_API rsbd8g_status rsbd8g_server_stats(rsbd8g_server *server, rsbd8g_server_counters *stats);
/* finish the batches in flight, stop the dispatcher, free the budget */
RSBD8G_API rsbd8g_status rsbd8g_server_destroy(rsbd8g_server *server);

/* Wait for the stream, then read and clear the device-side status word of a
 * scratch area used by a noalloc or segmented call (RSBD8G_OK, RSBD8G_ERR_TIMEOUT, ...). */
RSBD8G_API rsbd8g_status rsbd8g_scratch_status(void *scratch, rsbd8g_stream stream);

/* Human-readable name of a status code. */
RSBD8G_API const char *rsbd8g_status_string(rsbd8g_status status);

/* ---- launch profiling (measurement support; no counterpart in the reference) ---------- */

/* The plain sorts compute their plan in the histogram launch, so PLAN records only the segmented
 * sort's plan launch. The copy forms fold the copy step into the last digit pass, so COPY records the
 * in-place forms' copy launch and the segmented sort's. */
enum {
    RSBD8G_KERNEL_MEMSET = 0, RSBD8G_KERNEL_HISTOGRAM = 1, RSBD8G_KERNEL_PLAN = 2,
    RSBD8G_KERNEL_ONESWEEP = 3, RSBD8G_KERNEL_COPY = 4, RSBD8G_KERNEL_SEGMENTED = 5, RSBD8G_KERNEL_MERGE = 6
};

typedef struct rsbd8g_launch_record {
    uint32_t kernel;      /* RSBD8G_KERNEL_* */
    uint32_t key_bytes;
    uint32_t pass;        /* digit index of an onesweep launch */
    uint32_t reserved;
    uint64_t count;       /* elements of the sort the launch belongs to */
    double ms;            /* device time between CUDA events recorded around the launch on its stream */
} rsbd8g_launch_record;

/* While enabled, every kernel launch of the library (outside stream capture) is bracketed
 * by CUDA events on the stream it is launched on. */
RSBD8G_API rsbd8g_status rsbd8g_profile_enable(int enable);

/* Wait for the recorded events, copy up to `capacity` records (oldest first), report the
 * number recorded in *count, and forget them. */
RSBD8G_API rsbd8g_status rsbd8g_profile_collect(rsbd8g_launch_record *records, size_t capacity, size_t *count);

/* Library version: major * 10000 + minor * 100 + patch. */
RSBD8G_API int rsbd8g_version(void);

/* The architecture the library's kernels were compiled for, as the CUDA runtime reports it for
 * the loaded module on the current device (cudaFuncAttributes::binaryVersion: 103 for sm_103a).
 * Needs a device.  No counterpart in the reference. */
RSBD8G_API rsbd8g_status rsbd8g_binary_version(int *version);

/* Load and set up, on the current device, every kernel that sorts with this descriptor's key type,
 * mode and indirection can launch, at any count (and, for direct keys, the segmented sort's).
 * The CUDA runtime loads each kernel at its first use, which can hold the calling thread for tens
 * of milliseconds; a latency-sensitive caller prepares its descriptors once ahead of its first
 * sorts.  Optional: every entry point works without it.  rsbd8g_server_create prepares every key
 * type and mode the server accepts.  Allocates nothing.  No counterpart in the reference. */
RSBD8G_API rsbd8g_status rsbd8g_prepare(const rsbd8g_desc *desc);

#ifdef __cplusplus
}
#endif
#endif /* RSBD8G_H */
