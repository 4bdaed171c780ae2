/*
 * multians_gb300 -- C ABI of the GB300 (sm_103a) MULTIANS tANS decoder.
 *
 * Plain pointers and sizes only.  Device pointers are CUDA device memory of
 * the current device; `stream` is a cudaStream_t passed as void* (NULL =
 * legacy default stream).  Every entry point returns a mans_status code.
 *
 * Data formats are the reference's own:
 *   stream units  uint32, in CUHDInputBuffer order (the encoder's units
 *                 reversed; src/multians_input_buffer.cc:29); units past
 *                 n_units are treated as the zero padding
 *                 (src/multians_input_buffer.cc:23)
 *   table         L uint32 words, each a CUHDCodetableItem
 *                 {u16 next_state, u8 symbol, u8 min_num_bits}
 *                 (include/cuhd_codetable.h:20-24)
 *   output        n_out uint8 symbols in decode order, i.e. reversed like
 *                 the reference GPU decoder's output (src/main.cc:119-123)
 */
#ifndef MULTIANS_GB300_H_
#define MULTIANS_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    MANS_OK = 0,
    MANS_ERR_ARG = 1,          /* bad argument (sizes, L, first_state ...) */
    MANS_ERR_CUDA = 2,         /* a CUDA runtime call failed */
    MANS_ERR_AUX_SMALL = 3,    /* decoder memory smaller than needed */
    MANS_ERR_TABLE = 4,        /* table entry outside the decodable form */
    MANS_ERR_SYNC = 5,         /* a sync walk ran past its slots */
    MANS_ERR_NOMEM = 6,        /* allocation failed */
    MANS_ERR_BUSY = 7,         /* serving queue full / budget exhausted */
    MANS_ERR_NOT_FOUND = 8     /* unknown request / handle */
} mans_status;

/* Device-side status bits (mans_aux_status). */
#define MANS_DEV_BAD_TABLE      0x1u   /* invalid table entry seen */
#define MANS_DEV_SYNC_OVERFLOW  0x2u   /* a walk needed more slots */
#define MANS_DEV_DEGENERATE     0x4u   /* single-symbol table: filled */
#define MANS_DEV_COUNT_MISMATCH 0x8u   /* final pass disagreed with scan */
#define MANS_DEV_SCAN_TIMEOUT   0x10u  /* a bounded device wait gave up */

/* The mans_status a decode with these device bits returns
 * (MANS_DEV_DEGENERATE alone is success: the output is filled). */
int mans_status_code(uint32_t dev_status);

/* Launch geometry of one decode.  Zero fields are chosen by the built-in
 * autotuner from (L, units, output size); flags are copied through. */
typedef struct {
    uint32_t block_units;     /* units per output block (final pass) */
    uint32_t region_blocks;   /* blocks per sync region */
    uint32_t walk_slots;      /* regions a sync walk may cross */
    uint32_t threads;         /* threads per CTA */
    uint32_t flags;           /* MANS_DECODE_* */
    uint32_t capture_bytes;   /* symbol capture bytes per region (0: none) */
} mans_cfg;

/* Output order.  By default the output is in decode order, reversed like
 * the reference's (src/main.cc:119-123: the caller reverses on the host).
 * With MANS_DECODE_SOURCE_ORDER the final pass writes the i-th decoded
 * symbol to out[n_out - 1 - i]: a full decode is then the source symbols
 * in order and no host reversal is needed (CUHDOutputBuffer::reverse,
 * src/multians_output_buffer.cc:27-29, fused into the write). */
#define MANS_DECODE_SOURCE_ORDER 0x1u

/* Symbol capture.  When the stream has at least two bits per symbol on
 * average (few zero-bit codewords), L <= 4096 and at least 16 Mi units (64
 * MiB compressed; below that the capture's fixed cost outweighs what it
 * saves), or when capture_bytes is given, the planner gives every sync
 * region capture_bytes of workspace: the sync passes, which decode each
 * region once from a guessed state anyway, keep the symbols they decode
 * there, and the final pass copies every block whose owning trajectory was
 * captured instead of decoding it a second time.  MANS_DECODE_NO_CAPTURE
 * turns this off (smaller workspace, every block decoded in the final
 * pass); the output is identical either way. */
#define MANS_DECODE_NO_CAPTURE 0x2u
/* Capture whenever bits per symbol and L allow it, whatever the stream's
 * length (measured on the 4096-stream batch workload, where every stream is
 * short, capture lost: the capturing G pass holds fewer warps per SM). */
#define MANS_DECODE_CAPTURE 0x4u

/* Plan from the analytic model even where the measured table has an
 * entry (see mans_plan). */
#define MANS_PLAN_MODEL 0x8u

/* Start anywhere: first_bit gives the decode's start as a bit offset from
 * the least significant bit of the first unit, 0 .. 127, instead of the
 * reference's count of valid bits in unit 0 (the start at bit
 * 32 - first_bit).  A decode can then begin at any bit of a stream whose
 * units it addresses from the 16-byte aligned unit at most 3 units before
 * the start: a segment of a multi-table stream (multians_gb300/segments.py).
 * Honoured by mans_decode, mans_decode_sync, the batch descriptors' flags
 * and mans_trajectory_query. */
#define MANS_DECODE_START_OFFSET 0x10u

/* Seeded merge walks.  The walk pass lasts as long as its longest merge
 * walk, one dependent chain of table lookups.  With seeds, a warp whose
 * last walk is still running after two of its windows puts its idle lanes
 * to decoding from guessed states at the blocks ahead of that walk; where
 * the walk's trajectory meets one of theirs it continues from that lane's
 * position.  The planner turns seeds on where that was measured to pay
 * (1 to 4.5 bits per symbol; to 7 at L >= 4096); MANS_DECODE_SEEDS turns them on and
 * MANS_DECODE_NO_SEEDS off whatever the stream.  The output is identical
 * either way.  Plain decodes only (batches walk without seeds). */
#define MANS_DECODE_SEEDS 0x20u
#define MANS_DECODE_NO_SEEDS 0x40u

/* Fills `out` with the geometry the decoder uses for this call: the built-in
 * autotuner, keyed on the table size L and the compression ratio (bits per
 * symbol = 32 n_units / n_out).  Where the hint fixes no geometry and no
 * capture, units per block, the shortest region (in mean merge distances)
 * and symbol capture (from 16 Mi units on, where it pays at all) come from
 * the table the tuning tool measured on GB300 (mans_tune_lookup;
 * multians_gb300/tune.py writes it), the rest from the model; elsewhere,
 * or with MANS_PLAN_MODEL, all from the model.  The
 * reference takes these as fixed caller arguments (subsequence size and
 * threads per block, include/cuhd_gpu_decoder.h:24-35) and leaves its
 * CUHDUtil::optimal_subsequence_size (src/multians_util.cc:74-86) unused. */
int mans_plan(size_t n_units, size_t n_out, uint32_t L, const mans_cfg* hint,
              mans_cfg* out);

/* One measured table entry: the decode it was measured on (L, bits per
 * symbol, large = 256 MiB of symbols rather than 16 MiB) and the choice the
 * sweep kept, with its decoded GB/s next to the model's plan's. */
typedef struct {
    uint32_t L;
    float bits_per_symbol;
    uint32_t large;
    uint32_t block_units;
    float meet_mult;          /* shortest region in mean merge distances */
    uint32_t capture;
    float gbps;
    float model_gbps;
} mans_tune_entry;

/* The table entry mans_plan uses for a decode of n_out symbols at this L and
 * bits per symbol: returns 1 and fills `out`, or 0 where the table has none
 * (then the model plans). */
int mans_tune_lookup(uint32_t L, double bits_per_symbol, uint64_t n_out, mans_tune_entry* out);

/* The plan mans_plan makes from a table entry with these values (what the
 * tuning sweep times for each candidate). */
int mans_plan_tuned(size_t n_units, size_t n_out, uint32_t L, uint32_t block_units,
                    double meet_mult, int capture, mans_cfg* out);

/* Bytes of decoder memory ("aux") a decode with this geometry needs.
 * Replaces CUHDGPUDecoderMemory's sizing by (num_units, subsequence size,
 * threads) in src/multians_gpu_decoder_memory.cc:13-50. */
size_t mans_aux_size(size_t n_units, const mans_cfg* cfg);

/* Worst-case aux bytes over every geometry mans_plan can pick for n_units
 * units without symbol capture (what CUHDGPUDecoderMemory::allocate
 * reserves).  A decode given this much always runs: when the plan's capture
 * does not fit it decodes without (capture slices scale with the output
 * size, which this call does not see). */
size_t mans_aux_size_max(size_t n_units);

/* Aux bytes that every plan mans_plan can pick for n_units units fits,
 * symbol capture included, whatever the output size and table size (what
 * CUHDGPUDecoderMemory::allocate reserves, so that its decode never needs
 * more memory). */
size_t mans_aux_size_max_any(size_t n_units);

/* Decodes one stream; asynchronous on `stream`.  Replaces
 * cuhd::CUHDGPUDecoder::decode (include/cuhd_gpu_decoder.h:24-35,
 * src/multians_gpu_decoder.cu:575-687): same inputs (units, table, initial
 * state and bit, number of states), same output.  Allocates nothing.
 * cfg may be NULL (autotuned).  Argument errors return immediately; data
 * errors are reported through mans_aux_status. */
int mans_decode(const uint32_t* d_units, size_t n_units,
                uint8_t* d_out, size_t n_out,
                const uint32_t* d_table, uint32_t L,
                uint32_t first_state, uint32_t first_bit,
                void* d_aux, size_t aux_bytes,
                const mans_cfg* cfg, void* stream);

/* Waits for `stream` and returns the device status bits of the last decode
 * that used d_aux (0 = clean). */
int mans_aux_status(const void* d_aux, void* stream, uint32_t* status_out);

/* What the synchronisation of the last decode in d_aux cost, beside the
 * decode's own bytes.  The reference's counterpart is its phase-2 seam
 * passes (src/multians_gpu_decoder.cu:363-466, 617-656), which re-decode
 * subsequences until every seam agrees; here merge walks re-decode units
 * past each region's end until two trajectories meet.  Pass the arguments
 * of that decode (cfg as given to mans_decode, the workspace size it saw);
 * the call waits for `stream` and reads the workspace back. */
typedef struct {
    uint64_t regions;          /* regions of the plan the decode ran with */
    uint64_t blocks;           /* blocks of that plan */
    uint64_t walks;            /* merge walks (regions that have a successor) */
    uint64_t open_walks;       /* walks the decode pass left to the walk pass */
    uint64_t walk_units;       /* units the merge walks decoded a second time */
    uint64_t walk_max_units;   /* units of the longest walk */
    uint64_t walk_blocks;      /* block starts the walks crossed (walk records) */
    uint64_t metadata_bytes;   /* block records, walk records, per-region values and
                                  walk jobs written by the sync passes */
    uint64_t fallback_warps;   /* symbol capture: warps the final pass decoded */
    uint32_t unmerged;         /* walks that reached the stream end without merging
                                  (or ran out of walk slots: MANS_DEV_SYNC_OVERFLOW,
                                  counted to the stream end) */
    uint32_t seeded_walks;     /* walks finished with seeds (MANS_DECODE_SEEDS) */
} mans_sync_stats;

int mans_sync_stats_get(const void* d_aux, size_t aux_bytes, size_t n_units, size_t n_out,
                        uint32_t L, const mans_cfg* cfg, void* stream,
                        mans_sync_stats* out);

/* Trajectory query: where the decode of (units, first_state, first_bit)
 * stands at given bit positions.  For each position q (bits from the start
 * of the units, unit i holding positions 32 i .. 32 i + 31, read LSB first
 * as the decoder reads them) the decode's first codeword at or after q: its
 * bit position, the decoder state there and the number of symbols decoded
 * before it (found = 0 if the decode does not reach q).  Runs the sync
 * passes of a decode (no output) and one short decode per position from
 * the owner record of its block.  This is what splitting one stream over
 * several GPUs needs (multians_gb300/shard.py): a slice's exit state and
 * symbol count, and where two starts of a slice meet; the reference's
 * sync-point array holds the same facts per subsequence
 * (include/cuhd_subsequence_sync_point.h, src/multians_gpu_decoder.cu
 * :335-353).  n_out_hint: the expected symbol count, used for planning only
 * (0: 8 per unit).  flags: MANS_DECODE_START_OFFSET or 0.  d_aux:
 * mans_trajectory_aux_size bytes, 256-byte
 * aligned.  At most 1024 positions.  Synchronous on `stream`; a
 * single-symbol table returns MANS_ERR_TABLE. */
typedef struct {
    uint64_t pos;      /* bit position of the first codeword at or after q */
    uint32_t state;    /* decoder state there, in [L, 2L) */
    uint32_t found;
    uint64_t count;    /* symbols decoded before it */
} mans_point;

size_t mans_trajectory_aux_size(size_t n_units, size_t n_out_hint, uint32_t L, uint32_t nq);
int mans_trajectory_query(const uint32_t* d_units, size_t n_units, const uint32_t* d_table,
                          uint32_t L, uint32_t first_state, uint32_t first_bit, uint32_t flags,
                          size_t n_out_hint, void* d_aux, size_t aux_bytes,
                          const uint64_t* h_pos, uint32_t nq, mans_point* h_out, void* stream,
                          uint32_t* dev_status);

/* Synchronous decode: mans_decode, then the status check; on a sync-walk
 * overflow it re-plans with four times longer regions and decodes again.
 * hint may be NULL. */
int mans_decode_sync(const uint32_t* d_units, size_t n_units,
                     uint8_t* d_out, size_t n_out,
                     const uint32_t* d_table, uint32_t L,
                     uint32_t first_state, uint32_t first_bit,
                     void* d_aux, size_t aux_bytes, const mans_cfg* hint,
                     void* stream, uint32_t* status_out);

/* Workspace and table management for callers that do not hold device
 * memory of their own (the reference's CUHDGPUDecoderMemory::allocate /
 * free, src/multians_gpu_decoder_memory.cc:21-50, and
 * CUHDGPUCodetable's cpy_host_to_device, include/cuhd_gpu_memory_buffer.hxx:
 * 36-61).  mans_aux_alloc plans the decode of (n_units, n_out, L) (hint may
 * be NULL) and allocates exactly the workspace that plan needs, symbol
 * capture included; *bytes receives its size.  mans_table_upload checks a
 * host table (mans_table_check) and copies it to new device memory;
 * single-symbol tables are accepted (the decode fills the output). */
int mans_aux_alloc(size_t n_units, size_t n_out, uint32_t L, const mans_cfg* hint,
                   void** d_aux, size_t* bytes);
int mans_aux_free(void* d_aux);
int mans_table_upload(const uint32_t* h_table, uint32_t L, uint32_t** d_table);
int mans_table_free(uint32_t* d_table);

/* Host-side table check: 0 if every entry decodes inside [L, 2L) and
 * zero-bit entries strictly decrease the state, 1 if the table holds a
 * single symbol (all entries are zero-bit self loops), -1 otherwise. */
int mans_table_check(const uint32_t* h_table, uint32_t L);

/* Per-kernel timing of decodes (no counterpart in the reference, which
 * times whole decodes with cudaEvents in src/multians_util.cc:20-63).
 * mans_timing_enable(n) makes the next n decodes record CUDA events around
 * each of their kernels on the decode stream (n = 0 turns it off);
 * mans_timing_collect waits for them and returns the summed milliseconds
 * per kernel (prep, sync, scan, final) and how many decodes were timed. */
int mans_timing_enable(int max_decodes);
int mans_timing_collect(float* ms_per_kernel, int n_kernels, int* n_decodes);

/* Number of kernels launched by the last decode on this thread. */
uint32_t mans_last_launch_count(void);

/* ---- Batched decode of many independent streams --------------------------
 * No single counterpart in the reference, which decodes one stream per
 * CUHDGPUDecoder::decode call (src/main.cc:111-116); this decodes a whole
 * list of streams, each with its own table, in one launch of each kernel
 * (a work list spans the streams).  mans_batch_create plans every stream,
 * uploads the stream parameters and work list once, and uses the caller's
 * device workspace when given (mans_batch_workspace_size bytes) or
 * allocates its own.  mans_batch_decode enqueues the decode on `stream`
 * (nothing allocated, no host synchronisation); mans_batch_graph_decode
 * captures that into a CUDA graph on first use (on a private stream) and
 * replays it on `stream`.  Every stream gets its own device status word
 * (mans_batch_status: OR over the batch and, if per_stream != NULL, one
 * word per stream). */
typedef struct {
    const uint32_t* d_units;  /* 16-byte aligned */
    uint64_t n_units;
    uint8_t* d_out;
    uint64_t n_out;
    const uint32_t* d_table;
    uint32_t L;
    uint32_t first_state;
    uint32_t first_bit;
    uint32_t flags;           /* MANS_DECODE_* */
} mans_stream_desc;

typedef struct mans_batch mans_batch;

int mans_batch_workspace_size(const mans_stream_desc* streams, uint32_t n, const mans_cfg* hint,
                              size_t* bytes);
int mans_batch_create(const mans_stream_desc* streams, uint32_t n, const mans_cfg* hint,
                      void* d_workspace, size_t workspace_bytes, mans_batch** out);
/* Split layout, for callers that keep every stream's decode workspace
 * next to its own buffers: a small per-launch header
 * (mans_batch_header_size bytes at d_header) plus one slice per stream
 * (mans_batch_slice_size bytes, 16-byte aligned, at d_slices[i]).  The
 * parameters are uploaded asynchronously on `stream`; the host images stay
 * in the batch object until mans_batch_destroy. */
int mans_batch_slice_size(const mans_stream_desc* stream, const mans_cfg* hint, size_t* bytes);
int mans_batch_header_size(const mans_stream_desc* streams, uint32_t n, const mans_cfg* hint,
                           size_t* bytes);
int mans_batch_create_split(const mans_stream_desc* streams, uint32_t n, const mans_cfg* hint,
                            void* d_header, size_t header_bytes, void* const* d_slices,
                            void* stream, mans_batch** out);
int mans_batch_decode(mans_batch* b, void* stream);
int mans_batch_graph_decode(mans_batch* b, void* stream);
int mans_batch_status(mans_batch* b, void* stream, uint32_t* or_status, uint32_t* per_stream);
/* Synchronous: re-decodes every stream whose sync walks ran out of slots
 * (MANS_DEV_SYNC_OVERFLOW) with longer regions inside that stream's own
 * workspace slice, and updates its status.  Allocates nothing. */
int mans_batch_fixup(mans_batch* b, void* stream, uint32_t* n_redone);
int mans_batch_destroy(mans_batch* b);

/* One call for a batch: plan, decode (in d_workspace when given, else in
 * memory it allocates and frees), wait, re-decode streams whose walks ran
 * out of slots, and report the OR of the device status bits (and, if
 * per_stream != NULL, each stream's).  Synchronous on `stream`. */
int mans_decode_batch(const mans_stream_desc* streams, uint32_t n, const mans_cfg* hint,
                      void* d_workspace, size_t workspace_bytes, void* stream,
                      uint32_t* or_status, uint32_t* per_stream);

/* A loop of plain decodes, the way a C caller decodes many streams one at
 * a time with the reference's call (src/main.cc:111-116 decodes one stream
 * per CUHDGPUDecoder::decode): mans_decode of streams[i] with the cached
 * plan plans[i] (from mans_plan; the descriptor's MANS_DECODE_SOURCE_ORDER
 * is added) in workspace d_aux[i] of aux_bytes[i] bytes, i = 0 .. n-1, in
 * order on `stream`, asynchronous.  events may be NULL, else n cudaEvent_t
 * handles (as void*; NULL entries skipped), events[i] recorded after
 * stream i's decode.  Stops at the first error and returns it.
 * mans_last_launch_count then gives the kernels of the whole loop. */
int mans_decode_loop(const mans_stream_desc* streams, uint32_t n, const mans_cfg* plans,
                     void* const* d_aux, const size_t* aux_bytes, void* stream,
                     void* const* events);

/* Serving loop.  No counterpart in the reference, whose decode is one
 * blocking call on the default stream (include/cuhd_gpu_decoder.h:22-36).
 * A server owns one device range of budget_bytes (default 16 GiB, capped at
 * creation by the free device memory less 1 GiB), a worker thread and
 * max_inflight CUDA streams (one more for small requests, below).  Tables
 * are added once and stay resident.
 * mans_server_submit queues requests and returns at once.  The worker admits
 * queued requests in arrival order while each one's device memory (units,
 * output, decode workspace) fits the range, copies host inputs in on a copy
 * stream, and launches everything admitted since the previous launch as one
 * batch on a free stream; host outputs are copied back behind the batch on
 * the same stream.  Small requests (n_out <= small_bytes) have one more
 * stream of their own, at the device's highest stream priority: they are
 * batched there, apart from the larger requests, so that a small request
 * does not wait for a batch of large ones to decode and copy back.  A
 * request whose memory could never fit is completed
 * with MANS_ERR_NOMEM; bad arguments with MANS_ERR_ARG.
 * mans_server_poll returns completions (waiting up to wait_us for one).
 * Host buffers should be page-locked (cudaHostAlloc / cudaHostRegister):
 * pageable inputs are staged synchronously, pageable outputs are copied
 * after the batch completes.  Buffers must stay valid until completion. */
typedef struct mans_server mans_server;

typedef struct {
    uint64_t budget_bytes;    /* device memory the server may hold; 0 = 16 GiB */
    uint32_t max_inflight;    /* batches on the GPU at once, besides the
                                 small-request stream's; 0 = 2 */
    uint32_t max_batch;       /* requests per launch; 0 = 4096 */
    uint32_t small_bytes;     /* requests with n_out at most this are batched on
                                 the small-request stream; 0 = 1 MiB,
                                 UINT32_MAX = no small-request stream */
    uint32_t reserved;
} mans_server_cfg;

#define MANS_REQ_DEVICE_IO 0x1u     /* units / out are caller-owned device memory */
#define MANS_REQ_SOURCE_ORDER 0x2u  /* output in source order (MANS_DECODE_SOURCE_ORDER) */
#define MANS_REQ_CONTAINER 0x4u     /* units points at a host container of n_units
                                       bytes; table, n_out, first_state / first_bit
                                       come from it (out must hold n_symbols); its
                                       table is added as by mans_server_add_table
                                       (identical tables shared, kept until destroy) */
#define MANS_REQ_NO_CAPTURE 0x8u    /* decode without symbol capture (MANS_DECODE_NO_CAPTURE) */

typedef struct {
    const uint32_t* units;    /* CUHDInputBuffer order; 16-byte aligned if device */
    uint64_t n_units;
    uint8_t* out;             /* n_out symbols, decode order */
    uint64_t n_out;
    uint32_t table;           /* id from mans_server_add_table */
    uint32_t first_state;
    uint32_t first_bit;
    uint32_t flags;           /* MANS_REQ_* */
    uint64_t tag;             /* echoed in the completion */
    uint64_t arrival_ns;      /* mans_server_now_ns clock; 0 = time of submit */
} mans_request;

typedef struct {
    uint64_t tag;
    int32_t status;           /* mans_status */
    uint32_t dev_status;      /* MANS_DEV_* bits */
    uint64_t arrival_ns;
    uint64_t admit_ns;        /* device memory granted, input copy queued */
    uint64_t done_ns;         /* output in place */
    uint64_t batch;           /* sequence number of the launch (0 if none) */
} mans_completion;

typedef struct {
    uint64_t submitted, completed, failed;
    uint64_t batches, kernel_launches, streams_redone;
    uint64_t bytes_in, bytes_out;
    uint64_t range_bytes, range_peak, range_in_use;
    uint64_t admission_waits;  /* times the oldest queued request waited for memory */
    uint64_t largest_batch;
} mans_server_stats;

int mans_server_create(const mans_server_cfg* cfg, mans_server** out);
/* Copies an L-word decoder table to the device; it stays until destroy. */
int mans_server_add_table(mans_server* s, const uint32_t* host_table, uint32_t L, uint32_t* id);
int mans_server_submit(mans_server* s, const mans_request* reqs, size_t n);
int mans_server_poll(mans_server* s, mans_completion* out, size_t cap, size_t* n_out,
                     uint32_t wait_us);
int mans_server_stats_get(mans_server* s, mans_server_stats* out);
/* The clock of arrival_ns / done_ns (CLOCK_MONOTONIC, nanoseconds). */
uint64_t mans_server_now_ns(void);
/* Finishes the batches in flight, drops requests not yet launched (no
 * completion; their input copies end before it returns), joins the worker
 * and frees everything. */
int mans_server_destroy(mans_server* s);

/* Host-side data preparation (the reference's ANSTableGenerator +
 * ANSEncoder path, src/ans_table_generator.cc, src/ans_encoder.cc, as C
 * calls).  mans_host_gen_symbols: n seeded symbols
 * min(255, floor(-ln(U) / lambda)), U = ((x >> 11) + 1) * 2^-53, x from
 * mt19937_64(seed).  mans_host_max_units: the unit capacity (padding
 * included) mans_host_encode needs for these symbols.  mans_host_encode:
 * builds the L-state table from the symbol counts
 * (generate_distribution_from_buffer with `table_seed`, generate_table,
 * generate_encoder_table, get_decoder_table) and encodes; writes the L
 * decoder words, the units in CUHDInputBuffer order plus 4 zero units, the
 * unit count and the first bit / first state.  sym must be readable one
 * byte past n (the encoder looks one symbol ahead). */
int mans_host_gen_symbols(uint64_t seed, double lambda, uint8_t* out, size_t n);
size_t mans_host_max_units(const uint8_t* sym, size_t n, uint32_t L, uint32_t table_seed);
int mans_host_encode(const uint8_t* sym, size_t n, uint32_t L, uint32_t table_seed,
                     uint32_t* dec_table, uint32_t* units, size_t cap, size_t* n_units,
                     uint32_t* first_bit, uint32_t* first_state);

/* GPU encoder: the reference's table build and ANSEncoder::encode
 * (src/ans_table_generator.cc:61-314, src/ans_encoder.cc:13-97) with the
 * counting and the encoding on the device.  The units equal the host
 * encoder's (mans_host_encode) bit for bit, in CUHDInputBuffer order with
 * four zero units of padding; the byte after the last symbol is taken as 0
 * (mans_host_encode reads it from the zero padding it adds).  L must be a
 * power of two <= 8192.
 *   mans_histogram          byte counts of d_sym into d_hist[256] (async)
 *   mans_host_encode_tables tables from those counts: the L-word decoder
 *                           table and the encoder table blob
 *                           (mans_encode_blob_words words)
 *   mans_encode             encodes n bytes (d_sym 16-byte aligned) into
 *                           d_units (mans_encode_max_units words); workspace
 *                           mans_encode_aux_size bytes; chunk_hint 0 = plan
 *                           (async)
 *   mans_encode_result      n_units, first_bit, first_state (synchronous);
 *                           MANS_ERR_SYNC: merges ran out of slots, retry
 *                           with a larger chunk_hint */
size_t mans_encode_blob_words(uint32_t L);
int mans_histogram(const uint8_t* d_sym, size_t n, uint64_t* d_hist, void* stream);
int mans_host_encode_tables(const uint64_t* hist, uint32_t L, uint32_t table_seed,
                            uint32_t* dec_table, uint32_t* enc_blob);
size_t mans_encode_max_units(size_t n, uint32_t L);
size_t mans_encode_aux_size(size_t n, uint32_t chunk_hint);
int mans_encode(const uint8_t* d_sym, size_t n, const uint32_t* d_enc_blob, uint32_t L,
                uint32_t* d_units, size_t cap_units, void* d_aux, size_t aux_bytes,
                uint32_t chunk_hint, void* stream);
int mans_encode_result(const void* d_aux, void* stream, uint64_t* n_units, uint32_t* first_bit,
                       uint32_t* first_state, uint32_t* dev_status);
/* mans_encode + mans_encode_result, re-planning with 4x longer chunks while
 * the merges outrun their slots (workspace: mans_encode_aux_size(n, 0)). */
int mans_encode_sync(const uint8_t* d_sym, size_t n, const uint32_t* d_enc_blob, uint32_t L,
                     uint32_t* d_units, size_t cap_units, void* d_aux, size_t aux_bytes,
                     void* stream, uint64_t* n_units, uint32_t* first_bit,
                     uint32_t* first_state);

/* Stream container: one buffer holding a 64-byte header (magic, symbol and
 * unit counts, L, first state and bit, a header checksum), the L-word
 * decoder table and the units in CUHDInputBuffer order (no padding).  The
 * reference passes these as separate arguments (src/main.cc:111-116).
 * mans_container_parse checks the header and bounds and reports where the
 * table and units start; it does not read the payload. */
typedef struct {
    uint64_t n_symbols, n_units;
    uint32_t L, first_state, first_bit, reserved;
    uint64_t table_offset, units_offset;   /* bytes from the buffer start */
} mans_container_info;

size_t mans_container_size(uint64_t n_units, uint32_t L);
int mans_container_write(void* buf, size_t cap, const uint32_t* units, uint64_t n_units,
                         uint64_t n_symbols, const uint32_t* table, uint32_t L,
                         uint32_t first_state, uint32_t first_bit, size_t* size);
int mans_container_parse(const void* buf, size_t size, mans_container_info* info);

/* Decode that allocates nothing.  No counterpart in the reference: its
 * decode needs caller-allocated CUHDGPUDecoderMemory.  For callers that may
 * not allocate device memory when they decode (inside a host application's
 * own memory pool, on a path that must not stall behind cudaMalloc/cudaFree,
 * or when device memory is already exhausted): the workspace is a 32 MiB
 * device array inside this library (mans_noalloc_scratch_bytes), held by
 * every GPU that loads the library until exit.  Same arguments and result
 * as mans_decode_sync (arguments are checked first: MANS_ERR_ARG).  A stream
 * is accepted when a plan of it fits the array (the planner's, else without
 * symbol capture, else with fewer walk slots: about 28 million units at 6
 * bits/symbol, 7.7 million at 0.67 bits/symbol, L = 1024); larger ones get
 * MANS_ERR_AUX_SMALL before any GPU work.  All calls on a device share the
 * array: calls that overlap on the GPU race, so serialise them.  The first
 * call on a device looks up the array's address (again after the device's
 * context is re-created) and should come before any stream capture; under
 * lazy module loading that first call is also what reserves the array, so
 * a caller that relies on it once memory is exhausted makes one call early.
 * Synchronous on `stream`. */
int mans_decode_noalloc(const uint32_t* d_units, size_t n_units, uint8_t* d_out, size_t n_out,
                        const uint32_t* d_table, uint32_t L, uint32_t first_state,
                        uint32_t first_bit, void* stream, uint32_t* status_out);
size_t mans_noalloc_scratch_bytes(void);

/* Library version string. */
const char* mans_version(void);

#ifdef __cplusplus
}
#endif

#endif /* MULTIANS_GB300_H_ */
