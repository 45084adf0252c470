/*
 * seismic_gb300 -- C ABI of the GB300 (sm_103a) all-pairs normalised
 * cross-correlation library (libseismic_gb300.so).
 *
 * Two groups of entry points:
 *
 *  1. Drop-in symbols with the exact names, argument lists and meaning of the
 *     reference's ctypes boundary, so the reference's correlation_lib.py can
 *     load this library instead of its own:
 *       correlationCPP   Correlation_in_OMP/correlation_c.cpp:210-213
 *                        (ctypes argtypes Correlation_in_OMP/correlation_lib.py:88-92)
 *       correlationCUDA  Correlation_in_CUDA/correlation_cuda.cu:530-533
 *                        (ctypes argtypes Correlation_in_CUDA/correlation_lib.py:77-80)
 *       initialiseCUDA   Correlation_in_CUDA/correlation_cuda.cu:509
 *                        (Correlation_in_CUDA/correlation_lib.py:101-106)
 *     They return void like the originals; a failure is reported on stderr
 *     and through seismic_last_error().  `events_reversed`, `num_threads` and
 *     `chunk_size` are accepted and ignored (the reversed spectrum is the
 *     conjugate of the forward one; the GPU schedules its own work).
 *
 *  2. Native entry points returning an int status (SEISMIC_OK == 0), taking
 *     explicit sizes and strides, with channels, device-resident buffers and
 *     caller-provided streams.  They have no counterpart in the reference's
 *     ABI beyond the computation itself (correlation_c.cpp:58-137,251-293),
 *     whose semantics they keep.
 *
 * Semantics shared by all entry points (reference: correlation_c.cpp):
 *  - pairs (i, j >= i) of the upper triangle including the diagonal, packed
 *    row-major at index i*N - i*(i-1)/2 + (j-i) (:269), 64-bit;
 *  - lags d = 1-shift .. shift, series value at lag d = sum_k x_i[k] x_j[k-d]
 *    (circular of size paddedSize), first strict maximum above 0 / minimum
 *    below 0 in increasing d, else value 0 and lag 0 (:102-111).  A
 *    paddedSize that is not a power of two is accepted where it holds the
 *    lag window (paddedSize >= event_length + shift: the circular series is
 *    then the linear one, computed at the next power of two);
 *  - coefficient = peak / (paddedSize * |x_i| * |x_j|), norms in FP64
 *    (:115,:127); with C > 1 channels, the mean over channels of the
 *    per-channel normalised series;
 *  - histograms count every pair before thresholding: last bin for
 *    |coef| >= 1, else int(|coef| / float(1.0/n_classes_hist)) (:116-117,
 *    :128-129), accumulated into the caller's arrays;
 *  - threshold: coef > threshold (max) / coef < -threshold (min) are kept,
 *    others become 0 with lag 0 (:119-136);
 *  - a pair with a zero-norm event (all channels) reports 0 / 0 and is
 *    counted in no histogram bin (the reference divides by zero there).
 */
#ifndef SEISMIC_GB300_H
#define SEISMIC_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define SEISMIC_OK 0
#define SEISMIC_ERR_INVALID_ARGUMENT 1
#define SEISMIC_ERR_UNSUPPORTED_SIZE 2
#define SEISMIC_ERR_OUT_OF_MEMORY 3
#define SEISMIC_ERR_CUDA 4
#define SEISMIC_ERR_NO_DEVICE 5
#define SEISMIC_ERR_WORKSPACE_TOO_SMALL 6

/* ---- computation forms -------------------------------------------------- */
#define SEISMIC_FORM_FP32 0 /* FP32 spectra, FP32 products, FP32 inverse FFT */
/* FP16 (resp. BF16) spectra scaled by 1/norm, pointwise conj-products in
 * FP16 (BF16) accumulated over channels in FP32, FP32 inverse FFT and scan. */
#define SEISMIC_FORM_FP16_SPECTRA 1
#define SEISMIC_FORM_BF16_SPECTRA 3
/* Time-domain lag sums on the tensor cores (tcgen05), BF16 hi+lo split of the
 * samples scaled by 1/norm, three products (hi*hi + hi*lo + lo*hi)
 * accumulated in FP32; linear
 * correlation (padded_size is not used); needs 2*shift <= 512 and the
 * per-event lag strip to fit in shared memory (event_length up to ~1500 at
 * 2*shift = 256). */
#define SEISMIC_FORM_LAGGEMM_BF16X3 2
/* The same lag sums with one FP16 product (samples scaled by 1/norm, then
 * rounded to FP16; FP32 accumulation): a third of the tensor-core work of the
 * three-product form, coefficient errors up to ~1e-3 (typically ~1e-4).
 * Same limits on shift and event_length.  Also a serving form. */
#define SEISMIC_FORM_LAGGEMM_FP16 4

#define SEISMIC_ERR_DEVICE_TIMEOUT 7 /* a kernel's bounded wait ran out; results invalid */

/* ---- drop-in symbols (reference ABI) ----------------------------------- */

/* Replaces correlationCPP, Correlation_in_OMP/correlation_c.cpp:210-213. */
void correlationCPP(float *events, float *events_reversed, int n_events, int event_length, int shift,
                    int paddedSize, int num_threads, int chunk_size, float threshold,
                    int n_classes_hist, float *xcorr_vals_pos, int *xcorr_lags_pos,
                    float *xcorr_vals_neg, int *xcorr_lags_neg, int *max_hist, int *min_hist);

/* Replaces correlationCUDA, Correlation_in_CUDA/correlation_cuda.cu:530-533
 * (OpenMP-path semantics: below-threshold outputs are written as 0). */
void correlationCUDA(float *events, float *events_reversed, int n_events, int event_length, int shift,
                     int paddedSize, int num_threads, float threshold, float *xcorr_vals_pos,
                     int *xcorr_lags_pos, float *xcorr_vals_neg, int *xcorr_lags_neg);

/* Replaces initialiseCUDA, Correlation_in_CUDA/correlation_cuda.cu:509-527:
 * creates the context and loads the kernels so the first call is not
 * charged for it. */
void initialiseCUDA(void);

/* ---- errors ------------------------------------------------------------ */

/* Status of the calling thread's last call into this library. */
int seismic_last_error(void);
/* Human-readable message for the calling thread's last error ("" if none). */
const char *seismic_last_error_message(void);
const char *seismic_status_string(int status);

/* ---- native entry points ------------------------------------------------ */

/* Padded FFT size used when a native call passes padded_size = 0: the
 * smallest power of two >= event_length + shift (exact linear correlation
 * over the whole lag window).  Supported: up to 16384 (the plain transform),
 * and beyond, up to 2^24, where shift <= 1792 (the FFT forms then run the
 * overlap-save form, the same linear correlation).  Returns 0 otherwise.
 * Batched catalogs and the entry points given precomputed spectra take the
 * plain sizes only (batched: up to 8192). */
int seismic_resolve_padded_size(int event_length, int shift);

/* Device workspace (bytes) seismic_xcorr_device needs for these sizes
 * (padded_size 0 = seismic_resolve_padded_size); 0 if the sizes are
 * unsupported for the form. */
size_t seismic_xcorr_workspace_bytes(long long n_events, int n_channels, int event_length, int shift,
                                     int padded_size, int form);

/* The transform seismic_xcorr_device / seismic_xcorr_host run for these
 * sizes in an FFT form: *transform_size = padded_size and *blocks = 0 for
 * the plain form (one size-P transform per event), or, for a short lag
 * window, the overlap-save form: *blocks frames of *transform_size points
 * per event, each covering *block_length samples plus `shift` on either
 * side, whose correlations sum to the same linear correlation at fewer
 * FLOPs per pair.  padded_size 0 = seismic_resolve_padded_size.  No
 * counterpart in the reference (always one size-P transform,
 * correlation_c.cpp:39-45). */
int seismic_fft_plan(int event_length, int shift, int padded_size, int n_channels, int form, int *transform_size,
                     int *blocks, int *block_length);

/* Returns SEISMIC_OK, or SEISMIC_ERR_DEVICE_TIMEOUT if a kernel of this
 * library gave up a bounded wait since the last check (and clears the flag).
 * Synchronises the current device.  Allocates nothing (no stream, no
 * buffer), so callers of seismic_xcorr_device_noalloc may use it. */
int seismic_check_device_error(void);

/* All-pairs correlation of device-resident events.
 *   d_events: element (e, c, s) at d_events[e*event_stride + c*channel_stride + s],
 *             s < event_length (samples beyond are treated as zero);
 *   outputs:  device arrays of n_events*(n_events+1)/2 entries (packed triangle);
 *   d_max_hist/d_min_hist: device int[n_classes_hist], accumulated into, or
 *             NULL with n_classes_hist == 0;
 *   workspace: device buffer of seismic_xcorr_workspace_bytes(), 256-byte
 *             aligned (as cudaMalloc returns), or NULL (the library then uses
 *             its own cached allocation);
 *   stream:   a cudaStream_t (NULL = legacy default stream).
 * Asynchronous with respect to the host.  Returns a SEISMIC_* status. */
int seismic_xcorr_device(const float *d_events, long long n_events, int n_channels, int event_length,
                         long long event_stride, long long channel_stride, int padded_size, int shift,
                         float threshold, int n_classes_hist, int form, float *d_vals_pos,
                         int *d_lags_pos, float *d_vals_neg, int *d_lags_neg, int *d_max_hist,
                         int *d_min_hist, void *workspace, size_t workspace_bytes, void *stream);

/* seismic_xcorr_device in two halves over the caller's workspace: stages = 1
 * runs the per-event transforms into the workspace (kernel (a): spectra and
 * FP64 norms, or the lag-GEMM form's sample planes), stages = 2 the pairs
 * from it (kernel (b)), 3 both.  The workspace must stay untouched between
 * the two calls, which take the same arguments; reusing one stage-1 result
 * for several stage-2 calls (other thresholds or histogram sizes) is
 * allowed.  The output pointers are not read by stage 1.  No counterpart in
 * the reference, whose correlationCPP (correlation_c.cpp:210) runs both in
 * one call. */
int seismic_xcorr_device_stages(const float *d_events, long long n_events, int n_channels, int event_length,
                                long long event_stride, long long channel_stride, int padded_size, int shift,
                                float threshold, int n_classes_hist, int form, float *d_vals_pos, int *d_lags_pos,
                                float *d_vals_neg, int *d_lags_neg, int *d_max_hist, int *d_min_hist,
                                void *workspace, size_t workspace_bytes, void *stream, int stages);

/* Same computation from host memory (pinned or pageable) into host memory,
 * synchronous: copies events in, runs, copies the packed outputs back and
 * adds the histograms into max_hist/min_hist (may be NULL if
 * n_classes_hist == 0).  Host events use the strides of seismic_xcorr_device
 * with event_stride == n_channels * channel_stride. */
int seismic_xcorr_host(const float *events, long long n_events, int n_channels, int event_length,
                       long long event_stride, long long channel_stride, int padded_size, int shift,
                       float threshold, int n_classes_hist, int form, float *vals_pos, int *lags_pos,
                       float *vals_neg, int *lags_neg, int *max_hist, int *min_hist);

/* Kernel (a) alone: packed half spectra and FP64 norms of every (event,
 * channel) row.  d_spectra: n_events*n_channels rows of padded_size/2
 * float2 (slot 0 = (Re X[0], Re X[P/2]), slot k = X[k]); d_norms: room for
 * rows = n_events*n_channels doubles (the norms) followed by rows float
 * pairs (1/norm computed in FP64, kept as hi + lo floats; 0 for a zero
 * row): 16*rows bytes.  prescale != 0 scales each row by 1/norm (0 for a zero row), the
 * form the multichannel mean uses. */
int seismic_spectra_device(const float *d_events, long long n_events, int n_channels, int event_length,
                           long long event_stride, long long channel_stride, int padded_size, int prescale,
                           void *d_spectra, double *d_norms, void *stream);

/* Kernel (b) alone: all pairs of the upper triangle from spectra made by
 * seismic_spectra_device with the same padded_size (prescale must be set
 * when n_channels > 1).  Outputs and histograms as seismic_xcorr_device. */
int seismic_pairs_device(const void *d_spectra, const double *d_norms, long long n_events, int n_channels,
                         int padded_size, int prescaled, int shift, float threshold, int n_classes_hist,
                         int form, float *d_vals_pos, int *d_lags_pos, float *d_vals_neg, int *d_lags_neg,
                         int *d_max_hist, int *d_min_hist, void *stream);

/* seismic_pairs_device restricted to the work items [couple_begin,
 * couple_end) of seismic_pair_couples(n_events, padded_size, n_channels):
 * disjoint ranges on different GPUs (or streams) together cover the whole
 * triangle with no exchange, each writing only its own pairs of the shared
 * packed output layout.  Replaces the row partition of the reference's
 * multi-GPU variant (Correlation_in_MultiCUDA/correlation_multicuda.cu:157-203). */
int seismic_pairs_device_range(const void *d_spectra, const double *d_norms, long long n_events, int n_channels,
                               int padded_size, int prescaled, int shift, float threshold, int n_classes_hist,
                               long long couple_begin, long long couple_end, float *d_vals_pos, int *d_lags_pos,
                               float *d_vals_neg, int *d_lags_neg, int *d_max_hist, int *d_min_hist, void *stream);
/* Number of work items of the pair kernel on the triangle of n_events at
 * this padded size and channel count: couples (two pairs each) in the
 * direct-load form, blocks of TI x TJ events in the staged form (the name
 * keeps the first meaning).  Only ranges of this count are meaningful. */
long long seismic_pair_couples(long long n_events, int padded_size, int n_channels);

/* seismic_xcorr_device for callers that cannot allocate device memory.
 * No counterpart in the reference: it exists for callers that must not call
 * cudaMalloc/cudaFree -- a host framework that has reserved nearly all of
 * the GPU's memory for its own pool, a process under a fixed device-memory
 * quota, or a latency-critical loop that cannot afford an allocation's
 * implicit synchronisation.  Arguments and results are those of
 * seismic_xcorr_device (FP32 form, no workspace argument), always through
 * the plain size-P transform (where seismic_xcorr_device takes the
 * overlap-save form of a short lag window, the two agree to the parity
 * bar: 1e-5 on coefficients, lags up to FP32 ties); the scratch for
 * the spectra and norms is one fixed array of seismic_noalloc_scratch_bytes()
 * (64 MiB) inside this library, reserved on every device that uses it until
 * the process exits.  Catalogs needing more than that
 * (n_events*n_channels*(padded_size*4 + 16) bytes, 256-byte rounded per part)
 * are rejected with SEISMIC_ERR_WORKSPACE_TOO_SMALL.  The first call on a
 * device sets that device up, so make it before any stream capture.  All
 * calls share the scratch: calls that overlap on the GPU (other streams or
 * threads) race and must be serialised by the caller.  The call allocates
 * nothing: no cudaMalloc, no cudaFree, no allocating library routine.  It
 * returns once the kernels are queued; a kernel whose bounded wait ran out
 * leaves the device error flag set, which seismic_check_device_error()
 * (allocation-free as well) reads and clears after the caller has
 * synchronised. */
int seismic_xcorr_device_noalloc(const float *d_events, long long n_events, int n_channels, int event_length,
                                 long long event_stride, long long channel_stride, int padded_size, int shift,
                                 float threshold, int n_classes_hist, float *d_vals_pos, int *d_lags_pos,
                                 float *d_vals_neg, int *d_lags_neg, int *d_max_hist, int *d_min_hist,
                                 void *stream);

/* Size in bytes of the fixed scratch used by seismic_xcorr_device_noalloc.
 * No counterpart in the reference. */
size_t seismic_noalloc_scratch_bytes(void);

/* ---- batched form -------------------------------------------------------
 * Many independent station catalogs (uneven N, L, channels) correlated by
 * one persistent pair kernel (plus one spectra kernel) replayed from a
 * captured CUDA graph.  No counterpart in the reference ABI, which handles
 * one catalog per call (correlation_c.cpp:210); per catalog the semantics
 * are those of seismic_xcorr_device in the FP32 form, at the padded size
 * seismic_resolve_padded_size(event_length, shift). */
typedef struct seismic_catalog {
  const float *events; /* device; element (e, c, s) at e*event_stride + c*channel_stride + s */
  long long n_events;
  int n_channels;
  int event_length;
  long long event_stride;
  long long channel_stride;
  int shift;
  float threshold;
  int n_classes_hist; /* 0: no histograms */
  float *vals_pos;    /* device outputs, n_events*(n_events+1)/2 each */
  int *lags_pos;
  float *vals_neg;
  int *lags_neg;
  int *max_hist; /* device int[n_classes_hist], accumulated into, or NULL */
  int *min_hist;
} seismic_catalog;

typedef struct seismic_batch seismic_batch; /* opaque plan */

#define SEISMIC_BATCH_NO_GRAPH 1 /* flag: launch directly instead of replaying a graph */
/* flag: one persistent pair launch per transform size on parallel graph
 * branches, instead of the default single launch over all sizes */
#define SEISMIC_BATCH_PER_SIZE 2

/* Plans the batch (work lists sorted by cost, tuned tile sizes from the
 * autotuner cache), allocates its workspace and captures the CUDA graph.
 * The catalog buffers are bound to the plan; their contents may change
 * between runs. */
int seismic_batch_create(const seismic_catalog *catalogs, int n_catalogs, int flags, seismic_batch **out);
/* Runs the whole batch on `stream` (asynchronous). */
int seismic_batch_run(seismic_batch *batch, void *stream);
int seismic_batch_destroy(seismic_batch *batch);
/* Total pairs of all catalogs, kernels launched per run. */
long long seismic_batch_pairs(const seismic_batch *batch);
int seismic_batch_kernels_per_run(const seismic_batch *batch);

/* ---- autotuner ---------------------------------------------------------
 * Times the pair kernel for padded size P and n_channels over its tile
 * sizes, CTAs per SM and batched item sizes on the current device and stores
 * the fastest in the cache file (cache_path, else $SEISMIC_TUNE_CACHE, else
 * ~/.cache/seismic_gb300/tune.txt).  Later plans of this process and of
 * processes reading that file use it.  No counterpart in the reference. */
int seismic_autotune(int padded_size, int n_channels, const char *cache_path);
/* The parameters currently used for (P, n_channels). */
int seismic_tuning(int padded_size, int n_channels, int *tile, int *ctas_per_sm, int *item_groups);
/* The TMA-staged form's CTA shape the autotuner cached for exactly
 * (padded_size, n_channels spectrum rows per event): FFT warps per CTA (12,
 * or 99 for the widest CTA that keeps 128 registers a thread) and spectral
 * chunks per ring slot; both 0 when nothing is cached (the built-in rule
 * applies).  No counterpart in the reference. */
int seismic_tuning_staged(int padded_size, int n_channels, int *staged_warps, int *chunks_per_slot);

/* ---- serving loop --------------------------------------------------------
 * A catalog kept resident on the device as packed half spectra (FP32 or
 * FP16, form SEISMIC_FORM_FP32 / SEISMIC_FORM_FP16_SPECTRA) plus FP64 norms;
 * query requests of up to max_query_events events are correlated against a
 * contiguous catalog subset [subset_begin, subset_end) with continuous
 * batching: requests are admitted in arrival order as soon as one of n_slots
 * slots (CUDA streams) and enough of the hbm_budget_bytes pool are free
 * (a request that does not fit lets later, smaller ones go first), and
 * admitted requests run concurrently on the device.  No counterpart in the
 * reference (which correlates one catalog with itself per call). */
typedef struct seismic_server seismic_server;

/* catalog: host float32 [n_catalog][n_channels][event_length].  hbm_budget
 * 0 = room for n_slots requests of max_query_events against the whole
 * catalog.  topk: matches reported per query event (0..64). */
int seismic_server_create(const float *catalog, long long n_catalog, int n_channels, int event_length, int shift,
                          float threshold, int form, int n_slots, size_t hbm_budget_bytes, int max_query_events,
                          int topk, seismic_server **out);
/* Enqueues a request and returns at once with a ticket.  query: host float32
 * [n_query][n_channels][event_length], read when the request is admitted.
 * Outputs (host, any may be NULL; pinned memory keeps the copies
 * asynchronous): vals/lags [n_query][subset size] row-major, top-K values and
 * catalog indices [n_query][topk] (largest max-coefficient, ties to the lower
 * index).  All buffers must stay valid until seismic_server_wait returns. */
int seismic_server_submit(seismic_server *server, const float *query, int n_query, long long subset_begin,
                          long long subset_end, float *vals_pos, int *lags_pos, float *vals_neg, int *lags_neg,
                          float *topk_vals, long long *topk_index, long long *ticket);
/* The same for query events of query_length samples (1 .. event_length):
 * query is host float32 [n_query][n_channels][query_length], zero-padded to
 * the catalog's event_length on the device (norms are of the given samples). */
int seismic_server_submit_len(seismic_server *server, const float *query, int n_query, int query_length,
                              long long subset_begin, long long subset_end, float *vals_pos, int *lags_pos,
                              float *vals_neg, int *lags_neg, float *topk_vals, long long *topk_index,
                              long long *ticket);
/* Blocks until the ticket's results are in host memory; latency_ms (may be
 * NULL) = submit -> completion. */
int seismic_server_wait(seismic_server *server, long long ticket, double *latency_ms);
int seismic_server_stats(seismic_server *server, long long *completed, long long *pairs, int *in_flight,
                         int *pending);
/* Waits for every admitted and pending request, then frees everything. */
int seismic_server_destroy(seismic_server *server);

/* ---- consumers of the packed outputs --------------------------------------
 *
 * Sparse output.  Replaces the host-side sparsification of the reference's
 * driver (Correlation_in_OMP/test_c.py:43-55: each packed array becomes a
 * 1 x N(N+1)/2 scipy CSR matrix of its nonzeros, saved with save_npz), on the
 * device and in one pass over the outputs.  Keeps, in packed order, every pair
 * with d_vals_pos > threshold (index, value, lag into the *_pos arrays) and
 * every pair with d_vals_neg < -threshold (into the *_neg arrays).  Applied to
 * outputs computed with threshold 0 it gives exactly the entries the
 * reference's matrices hold after a run with `threshold` (the pair kernel
 * thresholds with the same strict comparisons).  Writes at most `capacity`
 * entries per side and the full counts to d_counts[0] (positive side) and
 * d_counts[1] (negative side); capacity 0 only counts.  `workspace` holds
 * seismic_compact_workspace_bytes(n_pairs) bytes.  Stream-ordered. */
size_t seismic_compact_workspace_bytes(long long n_pairs);
int seismic_compact_pairs_device(const float *d_vals_pos, const int *d_lags_pos, const float *d_vals_neg,
                                 const int *d_lags_neg, long long n_pairs, float threshold, long long capacity,
                                 long long *d_index_pos, float *d_value_pos, int *d_lag_pos,
                                 long long *d_index_neg, float *d_value_neg, int *d_lag_neg,
                                 long long *d_counts, void *workspace, size_t workspace_bytes, void *stream);

/* Histograms of stored coefficients, accumulated into d_max_hist / d_min_hist
 * with the rule of Correlation_in_OMP/correlation_c.cpp:116-117, :128-129
 * (last bin for |v| >= 1, else int(|v| / float(1.0 / n_classes_hist))).  On
 * outputs computed with threshold 0 it equals the pair kernel's own
 * histograms, except that pairs with a zero-norm event (stored as 0) count in
 * bin 0; it lets a threshold be chosen after the correlation has run. */
int seismic_histogram_device(const float *d_vals_pos, const float *d_vals_neg, long long n_pairs,
                             int n_classes_hist, int *d_max_hist, int *d_min_hist, void *stream);

/* Number of kernels this library has launched in this process. */
unsigned long long seismic_launch_count(void);

/* Releases the library's cached device buffers on the current device. */
int seismic_release_cached_memory(void);

#ifdef __cplusplus
}
#endif

#endif /* SEISMIC_GB300_H */
