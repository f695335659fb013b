/*
 * C ABI of the GB300 hash-join engine (libhjgb300.so).
 *
 * This is the flat, FFI-friendly form of the contest entry points of
 * eleanalt/hash-join-optimizer.  Plain pointers and sizes only; no C++ or torch
 * types cross it.  The C++ `Contest::execute(const Plan&, void*)` of
 * include/plan.h is a thin wrapper over `hj_execute`.
 *
 *   reference interface (file:line in eleanalt/hash-join-optimizer)   replaced by
 *   Contest::build_context()            include/plan.h:400, src/execute.cpp:610   hj_context_create
 *   Contest::destroy_context(void*)     include/plan.h:401, src/execute.cpp:614   hj_context_destroy
 *   Contest::execute(const Plan&,void*) include/plan.h:403, src/execute.cpp:598   hj_execute + hj_result_*
 *   UnchainedHash::build_insert/finalize_build
 *                                       include/unchained.h:155-217               hj_table_build
 *   UnchainedHash::probe(key, cb)       include/unchained.h:220-246               hj_table_probe
 *   PartitionedDirectoryHash::build/probe
 *                                       include/partitioned_directory_hash.h:86-215 hj_table_build / hj_table_probe
 *   Table::to_columnar / ColumnInserter src/build_table.cpp:657-882, plan.h:212-396 hj_pages_from_* (host)
 *
 * Errors: every entry point returns an HJ_* status.  The classes mirror the
 * exceptions the reference throws: HJ_ERR_RUNTIME <-> std::runtime_error
 * ("Join key isn't of type int32_t", src/execute.cpp:81,130), HJ_ERR_OUT_OF_RANGE
 * <-> std::out_of_range (StrRef field overflow, include/value_t.h:36-47).
 * hj_last_error() gives the message of the last failure on a context.
 *
 * Threading: a context is used by one host thread at a time, as the contest
 * harness calls execute() (tests/read_sql.cpp:1434-1447).  All device work of a
 * context runs in order on the context's CUDA stream.
 */
#ifndef HJ_API_H
#define HJ_API_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HJ_PAGE_SIZE 8192

enum hj_status {
    HJ_OK                = 0,
    HJ_ERR_INVALID       = 1, /* malformed plan or argument                     */
    HJ_ERR_RUNTIME       = 2, /* std::runtime_error class                       */
    HJ_ERR_OUT_OF_RANGE  = 3, /* std::out_of_range class (StrRef overflow)      */
    HJ_ERR_CUDA          = 4, /* a CUDA runtime call failed                     */
    HJ_ERR_NO_DEVICE     = 5, /* no usable CUDA device                          */
    HJ_ERR_CAPACITY      = 6, /* caller buffer too small; size needed returned  */
    HJ_ERR_DEVICE_STATUS = 7, /* a kernel reported an error in its status word  */
    HJ_ERR_NOMEM         = 8  /* device or pinned host allocation failed        */
};

/* DataType enumerators in the order of `enum class DataType`. */
enum hj_dtype { HJ_INT32 = 0, HJ_INT64 = 1, HJ_FP64 = 2, HJ_VARCHAR = 3 };

/* NodeType enumerators in the order of `enum class NodeType`. */
enum hj_node_kind { HJ_NODE_JOIN = 0, HJ_NODE_SCAN = 1 };

/* One input column: `num_pages` pointers to 8192-byte pages in host memory. */
typedef struct hj_column_desc {
    int32_t            type;      /* hj_dtype */
    uint64_t           num_pages;
    const void* const* pages;
} hj_column_desc;

/* One input table.  `resident` = 0: the pages above are host pages, uploaded
 * per call.  Otherwise it is a handle from hj_table_upload() and the table is
 * read from HBM (columns/num_columns are then ignored). */
typedef struct hj_table_desc {
    uint64_t              num_rows;
    uint32_t              num_columns;
    const hj_column_desc* columns;
    uint64_t              resident;
} hj_table_desc;

/* One (column index, DataType) entry of PlanNode::output_attrs. */
typedef struct hj_attr {
    uint64_t index;
    int32_t  type;
} hj_attr;

/* PlanNode.  kind = HJ_NODE_SCAN uses base_table_id; kind = HJ_NODE_JOIN uses
 * build_left/left/right/left_attr/right_attr with the meaning of JoinNode. */
/* A scan predicate on an INT32 column of the scanned table: the reference's
 * Comparison (include/statement.h:53-184 with src/statement.cpp:46-67 and
 * include/inner_column.h:172-326), which its table loader applies before
 * execute() (src/build_table.cpp:321-325).  A row passes when its bitmap bit is
 * set and `value OP literal` holds (a NULL never compares true); IS_NULL /
 * IS_NOT_NULL test the bitmap; the literal is cast to int32 as the reference
 * does.  The filters of one scan are combined with AND (LogicalOperation AND).
 * Operator numbers follow Comparison::Op; LIKE / NOT LIKE are not INT32
 * operators and are rejected. */
enum { HJ_CMP_EQ = 0, HJ_CMP_NEQ = 1, HJ_CMP_LT = 2, HJ_CMP_GT = 3, HJ_CMP_LEQ = 4, HJ_CMP_GEQ = 5,
       HJ_CMP_IS_NULL = 8, HJ_CMP_IS_NOT_NULL = 9 };
#define HJ_MAX_SCAN_FILTERS 4
typedef struct hj_filter {
    uint64_t column; /* column index in the scanned table */
    int32_t  op;     /* HJ_CMP_* */
    int32_t  pad;
    int64_t  value;  /* the literal */
} hj_filter;

typedef struct hj_node_desc {
    int32_t          kind;
    int32_t          build_left;
    uint64_t         base_table_id;
    uint64_t         left;
    uint64_t         right;
    uint64_t         left_attr;
    uint64_t         right_attr;
    uint32_t         num_attrs;
    const hj_attr*   attrs;
    /* scan nodes only: rows of the base table that pass all filters (none = all
     * rows).  The passing rows are compacted in order before the scan's first
     * use; with option "fuse_filters" = 1 a filtered probe side is instead read
     * raw and its predicate evaluated inside the probe's first pass. */
    uint32_t         num_filters;
    const hj_filter* filters;
} hj_node_desc;

typedef struct hj_plan_desc {
    uint32_t             num_nodes;
    const hj_node_desc*  nodes;
    uint32_t             num_inputs;
    const hj_table_desc* inputs;
    uint64_t             root;
} hj_plan_desc;

typedef struct hj_context    hj_context;
typedef struct hj_result     hj_result;
typedef struct hj_hash_table hj_hash_table;

/* ---- context (Contest::build_context / destroy_context) ------------------ */

/* Creates a context on CUDA device `device` (-1 = current device).  Returns
 * NULL when no device is usable; hj_last_error(NULL) then says why. */
hj_context* hj_context_create(int device);
void        hj_context_destroy(hj_context* ctx);
/* Message of the last failed call on `ctx` (or of the last failed create). */
const char* hj_last_error(const hj_context* ctx);
/* Library version string. */
const char* hj_version(void);
/* The cudaStream_t all device work of the context runs on (for callers that
 * order their own work or CUDA events against it). */
void* hj_context_stream(hj_context* ctx);

/* Engine tunables.  Names: "dir_bits" (-1 = next_pow2 of the build tuples, as
 * UnchainedHash::choose_directory_size, capped at 2^dir_cap_bits words),
 * "dir_cap_bits" (default 23: automatic directories of hj_execute stay within
 * 64 MB, cache resident; results do not depend on it), "radix_bits" (partition fan-out of the
 * build, 0..12), "probe_group" (output rows per thread of the match writer,
 * so a probe key's matches spread over count / probe_group threads: 1, 2, 4,
 * 8, 16 or 32; default 4), "light_max" (a bucket of several keys with at most
 * this many tuples is compared by the probing thread itself; larger ones by a
 * warp or block per hit), "timing" (1: record per-phase device times of
 * each hj_execute, read with hj_result_phase_ms), "host_access" (1, default:
 * where the GPU can read and write pageable host memory, it moves input and
 * result pages itself; 0: host threads stage them through pinned memory),
 * "table_cache" (1: a join whose build side is a whole resident base column
 * keeps the table built over it in HBM for later plans; 0, default: every
 * execute builds its own), "fuse_filters" (1: a filtered scan on the probe
 * side of a join is evaluated inside the probe instead of compacted first;
 * 0, default: compaction, which reads only the predicate columns of the
 * rejected rows and measured faster at 10% selectivity).
 * hj_get_option("host_access_capable") reports whether the device can. */
int hj_set_option(hj_context* ctx, const char* name, int64_t value);
int hj_get_option(const hj_context* ctx, const char* name, int64_t* value);

/* ---- resident base tables (HBM) ------------------------------------------ */

/* Uploads a host table once and keeps its pages in HBM; returns a handle for
 * hj_table_desc.resident.  hj_table_release frees it. */
int hj_table_upload(hj_context* ctx, const hj_table_desc* table, uint64_t* handle);
int hj_table_release(hj_context* ctx, uint64_t handle);
/* Binary table files in the reference's cache format (DumpTable,
 * include/table.h:128-211; Table::from_cache, src/build_table.cpp:147-203):
 * hj_table_dump writes a host table (at most 16 columns); hj_table_load maps a
 * file and uploads it as a resident table (handle as from hj_table_upload).
 * Files written by either side load on the other. */
int hj_table_dump(const hj_table_desc* table, const char* path);
int hj_table_load(hj_context* ctx, const char* path, uint64_t* handle);
/* Decodes every column of a resident table once and keeps the decoded form in
 * HBM, so later plans skip the per-call decode (no counterpart in the
 * reference: its tables are host-resident and decoded per execute). */
int hj_table_prepare(hj_context* ctx, uint64_t handle);

/* ---- query execution (Contest::execute) ---------------------------------- */

/* Runs the plan.  On success *out holds the root's columns as pages in HBM;
 * fetch them with hj_result_copy_pages, free with hj_result_free. */
int hj_execute(hj_context* ctx, const hj_plan_desc* plan, hj_result** out);

int hj_result_shape(const hj_result* res, uint64_t* num_rows, uint32_t* num_columns);
int hj_result_column(const hj_result* res, uint32_t col, int32_t* type, uint64_t* num_pages);
/* Copies the pages of column `col` to host memory: page i goes to dst_pages[i]
 * (8192 bytes each; no alignment needed). */
int hj_result_copy_pages(hj_context* ctx, const hj_result* res, uint32_t col,
                         void* const* dst_pages);
/* Same, into one contiguous host buffer of num_pages * 8192 bytes. */
int hj_result_copy_contiguous(hj_context* ctx, const hj_result* res, uint32_t col, void* dst);
/* Page-locks (pins) a host range for transfers, or releases it
 * (cudaHostRegister / cudaHostUnregister, for callers without CUDA bindings).
 * Input pages and result buffers in page-locked memory move through the copy
 * engines, one copy per run of consecutive pages, without occupying SMs, and
 * uploads of one plan overlap result downloads of another in the other
 * direction of the link; pageable memory takes the GPU-gather or staged path. */
int hj_host_register(void* ptr, uint64_t bytes);
int hj_host_unregister(void* ptr);
/* Kernel-side statistics of the last hj_execute on this result: number of
 * build tuples, probe tuples and output rows summed over all joins. */
int  hj_result_stats(const hj_result* res, uint64_t* build_tuples, uint64_t* probe_tuples,
                     uint64_t* output_rows);
/* Device milliseconds of one phase of the hj_execute that made `res` (option
 * "timing" = 1): "upload", "decode", "build", "probe" (count kernels),
 * "probe_sync" (match-count readback), "probe_write" (match emission),
 * "materialize", "total".
 * Phase "launches" gives the number of kernels that hj_execute launched. */
int  hj_result_phase_ms(const hj_result* res, const char* phase, double* ms);
/* Counters of the hj_execute that made `res`, summed over its joins (no
 * counterpart in the reference; they size the roofline of a run):
 * "dir_words" (directory words of the built tables, 2^b + 1 each),
 * "table_tuples" (tuples inserted, i.e. non-NULL build keys), "joins",
 * "launches" (kernels launched).  HJ_ERR_INVALID for another name. */
int  hj_result_counter(const hj_result* res, const char* name, uint64_t* value);
void hj_result_free(hj_result* res);

/* ---- hash table on device columns (UnchainedHash semantics) -------------- */

/* Builds the unchained table over device keys.  keys: int32[n] in HBM;
 * valid: validity bitmap in HBM (bit i%32 of word i/32 set = row i non-NULL) or
 * NULL when every row is valid.  NULL rows are not inserted.  dir_bits < 0 sizes
 * the directory as UnchainedHash does: next_pow2(#inserted), i.e. the same
 * directory words for the same key multiset. */
int hj_table_build(hj_context* ctx, const int32_t* keys, const uint32_t* valid, uint64_t n,
                   int32_t dir_bits, hj_hash_table** out);
/* Device pointers of the built table: directory (2^dir_bits + 1 words of
 * (first tuple << 16 | 16-bit Bloom tag)), tuple keys and build row ids in
 * adjacency-array order. */
int hj_table_info(const hj_hash_table* t, uint32_t* dir_bits, uint64_t* num_tuples,
                  const uint64_t** dir, const int32_t** tuple_keys, const uint32_t** tuple_rows);
/* Probes the table with device keys (NULL rows never match) and writes every
 * match as (probe row, build row) into caller buffers in HBM.  If more than
 * `capacity` matches exist nothing is written, *num_matches is set to the
 * count and HJ_ERR_CAPACITY is returned. */
int hj_table_probe(hj_context* ctx, const hj_hash_table* t, const int32_t* keys,
                   const uint32_t* valid, uint64_t n, uint32_t* out_probe_rows,
                   uint32_t* out_build_rows, uint64_t capacity, uint64_t* num_matches);
void hj_table_free(hj_hash_table* t);

/* ---- allocation-free probe -------------------------------------------------
 * No counterpart in the reference.  Same matches as hj_table_probe, for callers
 * that cannot allocate device memory during the call: engines that hand all
 * device memory to their own sub-allocator under a fixed budget, embedders
 * whose CUDA memory pool must not grow after start-up, and latency-critical
 * paths that cannot afford an allocation.  Every temporary comes from one array of
 * HJ_NOALLOC_SCRATCH_BYTES inside the library image, which each GPU that loads
 * the library holds until the process exits; the call itself allocates
 * nothing.  At most HJ_NOALLOC_MAX_PROBE_ROWS probe rows per call (more:
 * HJ_ERR_INVALID with a message naming the limit).  The first call on a device
 * looks up the array's device address and should come before any stream
 * capture.  The address is looked up in the device's primary context (the
 * one the CUDA runtime uses) and kept for the life of the process: calls from
 * a non-primary driver-API context, or after cudaDeviceReset on that device,
 * are not supported.  All calls share the array: calls whose GPU work overlaps
 * race, so the caller serialises them. */
#define HJ_NOALLOC_MAX_PROBE_ROWS 65536u
#define HJ_NOALLOC_SCRATCH_BYTES (6u << 20)
int hj_table_probe_noalloc(hj_context* ctx, const hj_hash_table* t, const int32_t* keys,
                           const uint32_t* valid, uint64_t n, uint32_t* out_probe_rows,
                           uint32_t* out_build_rows, uint64_t capacity, uint64_t* num_matches);

/* ---- batched independent joins ----------------------------------------------
 * Many independent INT32 join chains in one call: instance i joins its
 * relations R0 x R1 x ... x Rm-1 (2 <= m <= 8) on one key (R0 probes R1, the
 * result probes R2, ...).  Every relation is (key, payload) INT32 columns in
 * HBM without NULLs.  Per instance the call returns the result row count and a
 * checksum: the sum mod 2^64 over the result rows of a 64-bit fingerprint
 * folded over (key, payload of R0, ..., payload of Rm-1).
 *   mode HJ_BATCH_PERSISTENT: all relations of all instances radix-partitioned
 *     together on the key (partitions of ~2^batch_part_log2 build rows), then
 *     per (instance, partition) the build relations become shared-memory
 *     tables and R0's rows run through the whole chain -- persistent kernels
 *     over device-side work queues, the whole batch launched as one CUDA graph
 *     (options batch_part_log2, batch_load_pct, batch_graph).  Instances with
 *     a partition too large for shared memory (heavy duplicate keys) are
 *     recomputed with the plain path; *recomputed (may be NULL) counts them.
 *   mode HJ_BATCH_PLAIN: the instances one after another through the regular
 *     build / probe (options dir_bits, radix_bits, dir_cap_bits, probe_group,
 *     light_max) -- the one-query-at-a-time comparison.
 * Synchronous.  No counterpart in the reference (its execute() runs one plan). */
typedef struct hj_batch_relation {
    const int32_t* keys;
    const int32_t* payload;
    uint64_t       rows;
} hj_batch_relation;
typedef struct hj_batch_instance {
    uint32_t                 num_relations;
    const hj_batch_relation* relations;
} hj_batch_instance;
enum { HJ_BATCH_PERSISTENT = 0, HJ_BATCH_PLAIN = 1 };
int hj_batch_execute(hj_context* ctx, const hj_batch_instance* instances, uint32_t n, int32_t mode,
                     uint64_t* rows, uint64_t* checksums, uint32_t* recomputed);
/* Synthetic relation of a batch instance, generated in HBM from (seed,
 * instance, relation), enqueued on the context stream (hj_context_stream).
 * Build relations (relation >= 1): `rows` <= build_rows distinct keys in
 * [0, 2 build_rows).  Relation 0 (probe): `rows` keys, each one of R1's keys
 * with probability match_q24 / 2^24, else a key R1 does not hold.  Payloads
 * are uniform 32-bit values. */
int hj_batch_generate(hj_context* ctx, uint64_t seed, uint32_t instance, uint32_t relation,
                      uint64_t build_rows, uint32_t match_q24, uint64_t rows, int32_t* keys,
                      int32_t* payload);

/* ---- serving -----------------------------------------------------------------
 * A request loop over plans.  Clients submit plans from any thread and wait
 * on tickets; the server runs up to `slots` plans at once, each on its own
 * CUDA stream and host thread sharing ctx's resident tables (and, with option
 * "table_cache", the tables built over them), so concurrent plans overlap on
 * the GPU.  Admission is first come, first served against an HBM budget: a
 * plan starts when a slot is free and its estimated working memory (tables,
 * probe lists, row ids and pages, from its inputs' row counts) fits beside the
 * running ones; one plan larger than the budget runs alone.  Plans read their
 * inputs while they run: resident handles, or host pages that must stay valid
 * until the plan's wait returns.  Results are freed with hj_result_free and
 * read with ctx (hj_result_copy_*).  Destroy the server before ctx; it first
 * runs the queued plans.  No counterpart in the reference. */
typedef struct hj_server hj_server;
typedef struct hj_server_options {
    uint64_t hbm_budget_bytes; /* working memory of the running plans (estimated) */
    uint32_t slots;            /* plans running at once, 1..256 */
} hj_server_options;
typedef struct hj_request_stats {
    double   queue_ms;   /* submit -> start */
    double   service_ms; /* start -> result in HBM */
    double   latency_ms; /* submit -> result in HBM */
    uint64_t est_bytes;  /* the admission estimate */
} hj_request_stats;
hj_server* hj_server_create(hj_context* ctx, const hj_server_options* opt);
int        hj_server_submit(hj_server* srv, const hj_plan_desc* plan, uint64_t* ticket);
/* Blocks until the plan ran; returns its status (message into err when not
 * NULL) and on success its result. */
int        hj_server_wait(hj_server* srv, uint64_t ticket, hj_result** out, hj_request_stats* stats,
                          char* err, uint32_t err_cap);
int        hj_server_info(hj_server* srv, uint64_t* queued, uint64_t* running, uint64_t* running_bytes,
                          uint64_t* peak_bytes);
void       hj_server_destroy(hj_server* srv);

/* ---- host page writers (Table::to_columnar / ColumnInserter packing) ----- */

/* INT32 column of n rows into pages: valid (one byte per row, 0 = NULL) may be
 * NULL for "all valid".  With out == NULL only *num_pages is computed. */
int hj_pages_from_int32(const int32_t* values, const uint8_t* valid, uint64_t n, void* out,
                        uint64_t capacity_pages, uint64_t* num_pages);
/* VARCHAR column: string i is bytes[offsets[i] .. offsets[i+1]); valid as above. */
int hj_pages_from_strings(const uint8_t* bytes, const uint64_t* offsets, const uint8_t* valid,
                          uint64_t n, void* out, uint64_t capacity_pages, uint64_t* num_pages);

#ifdef __cplusplus
}
#endif

#endif /* HJ_API_H */
