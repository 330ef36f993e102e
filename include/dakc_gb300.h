/*
 * dakc_gb300.h -- C ABI of the GB300 k-mer counting engine.
 *
 * A drop-in for DAKC's k-mer counting entry point: DAKC's counter is the
 * constructor
 *     kmercounter(char* read_chunk, std::vector<kmer_t>& vectordbg)
 * (dakc/src/kcounter/kcounter.hpp:84-99), which parses a NUL-terminated chunk
 * of fixed-width read lines, counts every k-mer (k = KMERLEN, line width =
 * READLEN, both compile-time there: dakc/src/common/common.hpp:34-40) and
 * leaves the per-PE sorted (kmer, count) table in the public member lightdbg
 * (kcounter.cpp:385-414).  dk_count takes the same read buffer, k and line
 * width at run time and returns the globally sorted table -- the merge of all
 * PEs' lightdbg tables -- in one call on one GPU.
 *
 * Convention (bit-exact with the reference):
 *   - base codes C=0, A=1, T=2, G=3, upper or lower case
 *     (char2base, common.hpp:72-92);
 *   - a k-mer is packed MSB-first into the low 2k bits of a uint64
 *     (set_kmer_fast/update_kmer_fast, kcounter_funcs.cpp:25-38);
 *   - forward strand only, no canonical form;
 *   - a line is line_width bytes followed by one terminator byte that is never
 *     examined (the last terminator may be missing); 'M'/'m' ends the line;
 *     any other non-ACGT byte splits it; a run of L bases yields L-k+1 k-mers
 *     (read_till_buf_max, kcounter_funcs.cpp:69-111, including its rule that
 *     the last run is emitted only when it starts before line_width-1);
 *   - parsing stops before the first line (after line 0) whose first byte is
 *     NUL, as the reference stops at rchunk[read_idx] == '\0' (one PE).
 *
 * All entry points return 0 (DK_OK) or a negative DK_ERR_* status; nothing
 * throws across this boundary.  No call takes torch or C++ types.
 */
#ifndef DAKC_GB300_H
#define DAKC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DK_ABI_VERSION 1

/* status codes */
#define DK_OK 0
#define DK_ERR_INVALID_ARG (-1)     /* bad k, line width, sizes or pointers        */
#define DK_ERR_OOM (-2)             /* device or host allocation failed            */
#define DK_ERR_COUNT_OVERFLOW (-3)  /* a count does not fit 32 bits                */
#define DK_ERR_CUDA (-4)            /* a CUDA call failed (see dk_last_error_string)*/
#define DK_ERR_TIMEOUT (-5)         /* a bounded device or host wait ran out       */
#define DK_ERR_ADMISSION (-6)       /* job larger than the context's memory budget */
#define DK_ERR_PENDING (-7)         /* dk_poll: the job has not finished yet        */
#define DK_ERR_NOT_FOUND (-8)       /* unknown ticket                              */
#define DK_ERR_CANCELLED (-9)       /* job cancelled before it ran                 */
#define DK_ERR_NO_DEVICE (-10)      /* no CUDA device / engine not built for it    */

/* per-bucket count variants */
#define DK_VARIANT_AUTO 0  /* picked per workload                                 */
#define DK_VARIANT_SORT 1  /* partition + shared-memory sort + run-length reduce  */
#define DK_VARIANT_HASH 2  /* partition + shared-memory hash aggregation          */

/* k-mer conventions */
#define DK_CONV_DAKC 0     /* DAKC's rules, above                                  */
#define DK_CONV_PAKMAN 1   /* PakMan*'s: every byte b of a read is the 2-bit code
                              (b >> 1) & 7 OR'ed into the shifted window (A=0 C=1
                              T=2 G=3; other bytes give 4..7 as PakMan* computes
                              them, char_to_el / kmer_shift, pakman_star/includes/
                              distribute_kmers.h), nothing splits a run, a read
                              ends at '\n' (padding), and a k-mer ends at each
                              position from the k-th (Sliding_window,
                              pakman_star/src/kmer_counting.cpp:283-341).        */

/* where dk_count leaves the table */
#define DK_RESIDENT_HOST 0   /* kmers/counts are host arrays owned by the context  */
#define DK_RESIDENT_DEVICE 1 /* kmers/counts are device pointers owned by the ctx  */

typedef struct dk_ctx dk_ctx;

typedef struct {
  int device;          /* CUDA device ordinal                                    */
  int reserved0;
  uint64_t mem_budget; /* device bytes the context may hold; 0 = 80% of free    */
  uint64_t flags;      /* DK_FLAG_* bits, 0 by default                           */
} dk_config;

/* dk_config.flags: a host table is normally copied out group by group, while
 * the rest of the count runs, only when the input holds at least 64 Mi k-mers;
 * with this flag every host table is (the same table, other timing) */
#define DK_FLAG_STREAM_ALL 1ull
/* Pageable host reads are normally read in place by the device where it
 * accesses pageable memory through the host's page tables (Grace: coherent
 * chip-to-chip access), chunk by chunk like page-locked reads; with this flag
 * they are staged through page-locked slots by host threads instead */
#define DK_FLAG_STAGE_PAGEABLE 2ull
/* Batch waves (dk_count_batch, serving) run their partition levels, bin
 * count, tree offsets and compact as one launch of a CUDA graph whose level
 * loop is a conditional node; with this flag the host drives them launch by
 * launch, as for dk_count (the same tables) */
#define DK_FLAG_NO_GRAPH 4ull
/* Size the wave graph's buffers at their minimum, so that a wave whose
 * levels outgrow them is counted again with the host-driven tail (tests the
 * fallback; tables are the same) */
#define DK_FLAG_GRAPH_MIN_BUFFERS 8ull

typedef struct {
  int line_width;  /* READLEN: bytes per line before the terminator (>= 1)      */
  int k;           /* KMERLEN: 1..32                                            */
  int convention;  /* DK_CONV_DAKC or DK_CONV_PAKMAN                             */
  int variant;     /* DK_VARIANT_*                                               */
  int residency;   /* DK_RESIDENT_*                                              */
  int l1_bits;     /* tuning: level-1 partition bits, 0 = automatic (<= 12)     */
  int bin_target;  /* tuning: target keys per bin, 0 = automatic (<= 6000)      */
  int reserved;
} dk_input_desc;

typedef struct {
  uint64_t* kmers;   /* n distinct k-mers, ascending                           */
  uint32_t* counts;  /* occurrences of kmers[i]                                */
  uint64_t n;        /* distinct k-mers (DAKC's global_distinct_kmers)         */
  uint64_t n_kmers;  /* k-mer occurrences (DAKC's global_kmers)                */
  int on_device;     /* 1 when kmers/counts are device pointers                */
  int variant_used;  /* DK_VARIANT_SORT or DK_VARIANT_HASH                     */
  uint64_t handle;   /* owner token, pass back to dk_table_free                */
} dk_table;

/* timings of the last dk_count/dk_count_device on a context (CUDA events on
 * the context's stream) */
typedef struct {
  double ms_device;     /* first kernel to table complete in device memory     */
  double ms_h2d;        /* host -> device copy of the reads (dk_count only)    */
  double ms_d2h;        /* device -> host copy of the table (host residency)   */
  double ms_wall;       /* host wall time of the whole call                    */
  double ms_stage[8];   /* extract+count, scatter, partition, bin count,
                           output, hash, reserved, reserved                    */
  uint64_t n_kmers, n_distinct, n_lines;
  uint64_t kernel_launches;  /* engine kernels launched by the call            */
  uint64_t dev_bytes_peak;   /* device bytes held by the context               */
  int variant_used;
  int partition_levels;
  uint64_t n_bins;
  /* CUDA-event time of the main kernels (ms, summed over launches):
     [0] extract+count  [1] extract+scatter  [2] partition histogram
     [3] partition scatter  [4] bin count  [5] compact
     [6] batch waves' graphs (partition levels, bin count, tree offsets and
         compact of a wave in one CUDA graph launch)
     [7] everything else (scans, classify, tree offsets) */
  double ms_kernel[8];
  uint64_t launches_kernel[8];
  uint64_t n_partitioned;  /* keys moved by partition levels below level 1    */
  uint64_t n_waves;        /* dk_count_batch: memory-bounded waves run         */
  uint64_t n_bins_resorted; /* hash variant: bins the hash pass handed to sorting
                               (too many distinct keys or a long probe run)      */
  uint64_t n_bins_big;      /* hash variant: nodes larger than a bin that hold one
                               hot k-mer, counted whole by one hash bin          */
  uint64_t n_bins_retried;  /* of those, bins with too many distinct keys, which
                               were partitioned further                          */
  uint64_t n_groups;        /* groups of level-1 buckets counted one after another */
  uint64_t table_streamed;  /* 1: the host table was copied out group by group
                               while the count ran; 0: after it               */
  uint64_t upload_chunks;   /* chunks the reads were uploaded in, each counted as
                               it landed (0: one upload before the count)     */
  uint64_t n_bins_packed;   /* hash variant: bins counted in a packed table (one
                               64-bit word per distinct k-mer)                 */
  uint64_t n_bins_fallback; /* of the final bins, those the packed table could not
                               hold (counted by the general bin kernel)        */
  uint64_t upload_in_place; /* 1: pageable reads were read in place by the device
                               (no page-locked staging)                        */
  uint64_t graph_waves;     /* batch waves whose tail ran as one graph launch   */
  uint64_t graph_builds;    /* wave graphs built (and instantiated) by the call */
  uint64_t graph_retries;   /* waves counted again with the host-driven tail (a
                               level outgrew the graph's buffers, or a big bin
                               had to be re-partitioned)                       */
} dk_stats;

/* One read set of a batch (dk_count_batch). */
typedef struct {
  const char* text;  /* host pointer (pinned or pageable)                       */
  uint64_t nbytes;
} dk_job;

/* --- context ---------------------------------------------------------- */
int dk_create(const dk_config* cfg, dk_ctx** out);
int dk_destroy(dk_ctx* ctx);
const char* dk_strerror(int status);
const char* dk_last_error_string(dk_ctx* ctx);
int dk_abi_version(void);

/* --- plain count ------------------------------------------------------ */
/* Replaces kmercounter(read_chunk, vectordbg) + reading lightdbg
 * (kcounter.hpp:84-99, kcounter.cpp:385-414): `text` is a host buffer of
 * nbytes (pinned or pageable; borrowed for the call).  On success *out holds
 * the sorted table; release it with dk_table_free. */
int dk_count(dk_ctx* ctx, const char* text, uint64_t nbytes, const dk_input_desc* desc,
             dk_table* out);

/* Same, with the reads already in device memory (d_text: device pointer). */
int dk_count_device(dk_ctx* ctx, const char* d_text, uint64_t nbytes, const dk_input_desc* desc,
                    dk_table* out);

int dk_table_free(dk_ctx* ctx, dk_table* t);
int dk_last_stats(dk_ctx* ctx, dk_stats* out);

/* --- batched count ----------------------------------------------------- */
/* Count njobs independent read sets (same line width and k) in one pipeline:
 * the reference would run one kmercounter per set (kcounter.hpp:84-99); here
 * every set is its own level-1 partition of one launch sequence, processed in
 * waves sized to the context's memory budget (up to 4,096 sets per wave).
 * outs[j] receives job j's sorted table, host- or device-resident as
 * desc->residency asks (tables of one wave share one allocation, each must
 * still be released with dk_table_free; device-resident tables are never
 * copied back).  Per-job tables equal dk_count's on that job's text. */
int dk_count_batch(dk_ctx* ctx, const dk_job* jobs, int njobs, const dk_input_desc* desc,
                   dk_table* outs);

/* --- reads in other layouts ------------------------------------------- */
#define DK_FORMAT_LINES 0  /* one read per line, any length                      */
#define DK_FORMAT_FASTQ 1  /* 4-line records; the reads are line 2 of each
                              (syngen/fq2txtmaker.sh:12)                          */
#define DK_FORMAT_FASTA 2  /* from the first '>': header line, sequence line, ...
                              (pakman_star/src/kmer_counting.cpp:283-300)         */
/* Count reads given in `format` (host buffer): they are laid out on the GPU
 * as fixed-width lines -- width desc->line_width, or the longest read when it
 * is 0 -- padded as the reference's conversion pads them (DAKC convention:
 * 'M', with spaces turned into 'M' for FASTQ, syngen/fq2txtmaker.sh:12-18;
 * PakMan* convention: '\n', where its reader ends a read), and counted as
 * dk_count counts those lines.  *line_width (optional) receives the width. */
int dk_count_format(dk_ctx* ctx, const char* text, uint64_t nbytes, int format,
                    const dk_input_desc* desc, dk_table* out, int* line_width);

/* Number of lines dk_count will parse for this buffer under the framing rules
 * above (host-side, no GPU work); negative status for a malformed size. */
int64_t dk_num_lines(const char* text, uint64_t nbytes, int line_width);

/* Page-locked host memory for read buffers (dk_count then copies it with one
 * DMA instead of staging it).  Replaces the reference's malloc'd read chunk
 * (dakc/src/fqreader/fqreader.cpp:59). */
int dk_host_alloc(uint64_t nbytes, void** out);
int dk_host_free(void* p);

/* --- autotuning --------------------------------------------------------- */
/* The partition's level-1 fan-out, the keys per bin and the per-bin count
 * variant decide how fast a count runs; their best values depend on the
 * input's size and k-mer spectrum.  dk_autotune counts `text` (host buffer,
 * as for dk_count) under a small set of choices -- level-1 bits around the
 * automatic rule, three bin sizes, both variants -- and keeps the fastest in
 * the context for inputs of the same shape (line width, k, and size class
 * ceil(log2(lines * (line_width - k + 1)))).  Later dk_count /
 * dk_count_device calls whose desc leaves l1_bits = 0, bin_target = 0 and
 * variant = DK_VARIANT_AUTO use it.  Every choice gives the same table; only
 * the time differs.  No counterpart in the reference (its bucket sizes are
 * compile-time constants, common.hpp:36-44). */
typedef struct {
  int l1_bits;       /* chosen level-1 partition bits                          */
  int bin_target;    /* chosen target keys per bin                             */
  int variant;       /* chosen DK_VARIANT_SORT or DK_VARIANT_HASH              */
  int candidates;    /* parameter sets timed                                   */
  double ms_device;  /* device time of the chosen set                          */
  double ms_auto;    /* device time of the automatic choice                    */
} dk_tune;

int dk_autotune(dk_ctx* ctx, const char* text, uint64_t nbytes, const dk_input_desc* desc,
                dk_tune* out);
/* forget every tuned choice of the context */
int dk_autotune_reset(dk_ctx* ctx);

/* --- operations on finished tables --------------------------------------
 * `t` is a table the library returned (host- or device-resident); kernels
 * read it where it lies.  No counterpart in DAKC, which stops at the table;
 * these are the consumers of the table in PakMan*, the reference's second
 * implementation of the path. */

/* hist[c] = distinct k-mers whose count is c, for c < num_buckets (hist: host
 * array of num_buckets); *min_bucket (optional) = PakMan*'s cut-off, the
 * first minimum of hist[1 .. num_buckets-1] (pakman_star/src/
 * kmer_histogram.cpp:72-123); 0 when num_buckets == 1. */
int dk_table_histogram(dk_ctx* ctx, const dk_table* t, uint32_t num_buckets, uint64_t* hist,
                       uint32_t* min_bucket);
/* *out = the k-mers of t whose count is >= min_count, in order, with the same
 * residency (a new table: release both with dk_table_free); out->n_kmers is
 * the sum of the kept counts.  PakMan* keeps count >= min_bucket
 * (kmer_histogram.cpp:123-130). */
int dk_table_filter(dk_ctx* ctx, const dk_table* t, uint32_t min_count, dk_table* out);
/* counts[i] = count of queries[i] in t, 0 when absent (host arrays of n). */
int dk_table_lookup(dk_ctx* ctx, const dk_table* t, const uint64_t* queries, uint64_t n,
                    uint32_t* counts);
/* The table as t->n packed 12-byte records {uint64 k-mer; uint32 count}, the
 * layout of PakMan*'s KmerPairs (pakman_star/includes/distribute_kmers.h:
 * 690-696); `out` (host or device, 4-byte aligned) holds 12 * t->n bytes. */
int dk_table_pairs(dk_ctx* ctx, const dk_table* t, void* out);

/* --- serving ----------------------------------------------------------- */
/* A request loop over `workers` engine workers (each with its own CUDA
 * stream, device arenas and 1/workers of the context's memory budget).  Jobs
 * are admitted by an estimate of their device memory, queue, and are
 * coalesced into batched launches (dk_count_batch) by whichever worker frees
 * up first, so work of jobs that arrive while others run overlaps on the
 * device.  A job's table is host-resident, or stays in device memory when
 * its descriptor asks for DK_RESIDENT_DEVICE (valid until dk_serve_stop).
 * No counterpart in the reference (one kmercounter per run). */
typedef struct {
  double queued_us;  /* submit -> start of its batch                      */
  double run_us;     /* start of its batch -> its table ready               */
  int batch_jobs;    /* jobs in the batch it ran in                       */
  int worker;
} dk_job_info;

int dk_serve_start(dk_ctx* ctx, int workers, int max_batch_jobs);
/* text is borrowed until dk_poll / dk_wait returns anything but
 * DK_ERR_PENDING or DK_ERR_TIMEOUT for the job */
int dk_submit(dk_ctx* ctx, const char* text, uint64_t nbytes, const dk_input_desc* desc,
              uint64_t* ticket);
/* DK_ERR_PENDING while queued or running; otherwise the job's status, with
 * its table in *out (release with dk_table_free; out NULL releases it) */
int dk_poll(dk_ctx* ctx, uint64_t ticket, dk_table* out, dk_job_info* info);
int dk_wait(dk_ctx* ctx, uint64_t ticket, int timeout_ms, dk_table* out, dk_job_info* info);
/* a queued job is dropped at once; a running one stays DK_ERR_PENDING (its
 * text still read) until its batch ends, then polls as DK_ERR_CANCELLED */
int dk_cancel(dk_ctx* ctx, uint64_t ticket);
int dk_serve_stop(dk_ctx* ctx);  /* finishes queued jobs, joins the workers */

/* --- counting without any allocation ------------------------------------
 * No counterpart in the reference: DAKC always allocates its buffers.
 *
 * For callers that cannot allocate memory at the point where they need a
 * count -- code running inside a memory allocator's callback, latency-bound
 * serving or real-time loops that must not take the allocator's locks or its
 * device-wide synchronisation, or programs that own all device memory
 * through their own pool.  dk_count needs a context whose work buffers are
 * allocated on demand; this call needs none.  The caller passes the reads
 * (d_text, device memory), the output table (d_kmers / d_counts, device
 * memory, at least `capacity` entries) and d_summary (device memory, 3
 * uint64: distinct k-mers, k-mer occurrences, status 0 = ok).  The call is
 * asynchronous on `stream` (a cudaStream_t, NULL for the default stream) on
 * the current device and allocates nothing: its scratch is one fixed array
 * of 12,288 uint64 (96 KB) inside the library, which every device that
 * loads the library holds until the process exits.
 *   - Inputs whose k-mer upper bound, lines * (line_width - k + 1), exceeds
 *     12,288 are rejected with DK_ERR_ADMISSION before any launch;
 *     capacity must be at least that bound (else DK_ERR_INVALID_ARG).
 *   - Every call on a device shares that scratch array (it keeps the last
 *     call's contents; each call writes all it reads).  Calls that overlap
 *     on the GPU race on it: issue them on one stream, or order them.
 *   - The first call on a device does a one-time set-up with that device
 *     current (it looks up the scratch array's device address and sets the
 *     kernel's shared-memory limit); make that first call before any stream
 *     capture on that device.  After a device reset, use a new process.
 * Results equal dk_count's table for the same reads. */
int dk_count_small_noalloc(const char* d_text, uint64_t nbytes, int line_width, int k,
                           uint64_t* d_kmers, uint32_t* d_counts, uint64_t capacity,
                           uint64_t* d_summary, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* DAKC_GB300_H */
