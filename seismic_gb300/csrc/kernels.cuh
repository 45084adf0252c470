// Kernel declarations and launch helpers shared by the C-ABI layer.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <cuda_runtime.h>

namespace seismic {

constexpr int kMaxP = 16384;  // largest padded size of the plain transform (one 512-thread FFT group a CTA)
constexpr int kMinP = 64;     // smallest
constexpr int kMaxBatchP = 8192;          // batched launches (256-thread CTAs)
constexpr int kMaxPadded = 1 << 24;       // beyond kMaxP: the overlap-save form only
constexpr int kMaxBlockShift = 7 * 4096 / 16;  // its widest lag window: frames of Q = 4096, blocks >= Q / 8

// A padded size that is not a power of two but holds the whole lag window
// (padded >= event_length + shift) gives the reference's size-padded
// circular correlation without aliasing, i.e. the linear correlation, which
// any larger transform gives too: such a size runs at the next power of
// two.  Others come back unchanged (an aliasing non-power-of-two size stays
// unsupported).
inline int effective_padded(int padded, int event_length, int shift) {
  if (padded <= 0 || (padded & (padded - 1)) == 0) return padded;
  if ((long long)event_length + shift > padded) return padded;
  long long p = kMinP;
  while (p < padded) p <<= 1;
  return p <= kMaxPadded ? (int)p : padded;
}

// Layout of the packed half spectrum of one (event, channel) row:
//   slot 0      = (Re X[0], Re X[P/2])   (both bins are real for real input)
//   slot k>0    = X[k],  k = 1 .. P/2-1
// Rows are [event][channel], each P/2 float2 = 4P bytes (16-byte aligned).

struct SpectraArgs {
  const float *events;     // time series, element (e, c, s) at events[e*ev_stride + c*ch_stride + s]
  long long n_events;
  int n_channels;
  int length;              // L samples used (zero beyond)
  long long ev_stride;     // elements
  long long ch_stride;     // elements
  int prescale;            // 1: spectra scaled by 1/norm (0 if norm == 0); 0: unscaled
  int stype;               // spectrum storage: 0 float2, 1 half2 (FP16), 2 bfloat162 (BF16)
  void *spectra;           // out [n_events*n_channels][P/2] of stype
  double *norms;           // out [n_events*n_channels], FP64 L2 norms
  float2 *inv_norms;       // out [n_events*n_channels], FP64 1/norm as hi + lo floats (0 for 0)
  const float2 *twiddles;  // twiddle_table()
  // Overlap-save frames (blocks > 0, block_spectra_kernel): per (event,
  // channel) row, `blocks` pairs of size-P transforms.  Frame b covers
  // samples o_b .. o_b + P - 1, o_b = b * block_len - block_shift; the A
  // frame keeps samples b * block_len .. + block_len - 1 (zero elsewhere),
  // the W frame all of them.  A spectra go to `spectra`, W spectra to
  // `spectra_w`, both [n_events*n_channels][blocks][P/2]; a null pointer
  // leaves that set out (a serving catalog keeps only W, queries only A).
  int blocks;
  int block_len;
  int block_shift;
  void *spectra_w;
};

// Overlap-save plan of a short lag window (block_plan, api.cu): the
// correlation at lags 1-shift .. shift of events of L samples is the sum
// over nb blocks of B samples of size-Q circular correlations of an A frame
// (the block) with a W frame (the block widened by `shift` on both sides),
// exact while B + 2 shift <= Q; the Q-point transforms then replace the
// size-P one.  nb == 0: no plan (the plain size-P form).
struct BlockPlan {
  int Q = 0;       // frame (FFT) size
  int B = 0;       // block length
  int nb = 0;      // blocks per (event, channel) row
};
BlockPlan block_plan(int length, int shift, int P, int n_channels, int stype);
cudaError_t launch_block_spectra(int Q, const SpectraArgs &a, cudaStream_t s);

// A norms buffer holds `rows` FP64 norms followed by `rows` inverse norms
// 1/norm, each computed in FP64 and stored as an unevaluated float pair
// hi + lo (hi = the float nearest to it, lo = the float nearest to the
// rest): 48 significant bits (fewer for norms above ~2^102, whose lo part
// falls into FP32's subnormal range), from which the final normalisation of every
// form is computed at FP64-equivalent accuracy without FP64 instructions in
// the FFT pair loop (compensated_scale below).
inline size_t norms_buffer_bytes(long long rows) { return ((size_t)rows * 16 + 255) / 256 * 256; }
__host__ __device__ inline float2 *inverse_norms_of(double *norms, long long rows) {
  return reinterpret_cast<float2 *>(norms + rows);
}
__host__ __device__ inline const float2 *inverse_norms_of(const double *norms, long long rows) {
  return reinterpret_cast<const float2 *>(norms + rows);
}
// FP64 value -> (hi, lo) float pair.
__host__ __device__ inline float2 split_double(double v) {
  const float hi = (float)v;
  return make_float2(hi, (float)(v - (double)hi));
}

struct PairArgs {
  const void *spectra;     // [n_events*n_channels][P/2] of stype
  int stype;               // 0 float2, 1 half2, 2 bfloat162
  const double *norms;     // [n_events*n_channels]
  const float2 *inv_norms;    // [n_events*n_channels], see SpectraArgs
  const float2 *inv_norms_q;  // rectangle mode: the queries' inverse norms
  long long n_events;
  int n_channels;
  int shift;               // lags d = 1-shift .. shift
  int prescaled;           // spectra were scaled by 1/norm (multichannel mean)
  float threshold;
  int n_hist;              // 0 disables histograms
  float delta_hist;        // float(1.0 / n_hist)
  float *vals_pos;
  int *lags_pos;
  float *vals_neg;
  int *lags_neg;
  int *max_hist;           // device, accumulated into
  int *min_hist;
  // work range in couples (pairs of pairs), for chunked or sharded launches
  long long couple_begin;
  long long couple_end;
  int tile;                // events per tile side
  const float2 *twiddles;  // twiddle_table()
  // Rectangle mode (rect != 0): pairs (query q, catalog event col_begin + j)
  // for q < n_query, j < n_cols, instead of the upper triangle.  The query
  // spectra / norms are separate; `spectra` / `norms` are the catalog's;
  // outputs are [n_query][n_cols] row-major; couples are ordered in chunks of
  // `tile` couple-columns times all queries (catalog spectra reused across
  // queries from L1).
  int rect;
  const void *spectra_q;
  const double *norms_q;
  long long n_query;
  long long col_begin;
  long long n_cols;
  // Staged form (staged_core.cuh) only: tile columns per L2 band of the
  // triangle walk, the shared-memory ring depth, and the device error flag
  // set when a bounded wait runs out.
  int band_tiles;
  int ring;
  int *error_flag;
  // Overlap-save form (staged form only): i-side spectra that differ from the
  // j-side ones (the A frames; `spectra` holds the W frames), and spectrum
  // rows per event (n_channels * blocks; 0 = n_channels).
  const void *spectra_i;
  int spec_channels;
  // Staged form: a CTA shape forced by the autotuner while it times the
  // candidates (FFT warps per CTA, chunks per ring slot; 0 = not forced).
  int staged_warps;
  int staged_ru;
  // Staged form, set by its launch: i and j events per work item (TI, TJ;
  // see StagedGeom), ceil(2^16 / (TJ / 2)) so that a group's item row is
  // (group * item_magic) >> 16, and the bytes of one ring slot.
  int item_i;
  int item_j;
  unsigned item_magic;
  unsigned unit_bytes;
  // Poll limit of the staged form's producer waits (0: the built-in limit,
  // seconds of back-off).  Set from SEISMIC_DEVICE_WAIT_POLLS: a few polls
  // make the waits run out on a healthy GPU, which is how the abort path and
  // its error status are tested.
  unsigned wait_limit;
  // Nonzero (SEISMIC_DEVICE_WAIT_PROBE): the producer's first wait is on a
  // barrier nothing ever completes, so it runs out after wait_limit polls
  // -- the deterministic way for a test to take the abort path.
  int wait_probe;
};

// SEISMIC_DEVICE_WAIT_PROBE set to a nonzero value.
inline int device_wait_probe() {
  const char *e = getenv("SEISMIC_DEVICE_WAIT_PROBE");
  return (e && atoi(e) != 0) ? 1 : 0;
}

// Spectrum rows per event of the pair launch `a` (channels x blocks).
__host__ __device__ inline int spectrum_rows(const PairArgs &a) {
  return a.spec_channels > 0 ? a.spec_channels : a.n_channels;
}

// SEISMIC_DEVICE_WAIT_POLLS (1 .. 2^30), else 0.
inline unsigned device_wait_polls() {
  const char *e = getenv("SEISMIC_DEVICE_WAIT_POLLS");
  if (!e) return 0;
  const long long v = atoll(e);
  return (v >= 1 && v <= (1LL << 30)) ? (unsigned)v : 0u;
}

// Tile rows per L2 band of the triangle walk (PairArgs::band_tiles) so
// that the spectra of one band's events take about 48 MB of L2
// (SEISMIC_L2_BAND_MB sets another size, 1 .. 4096 MB).
inline int l2_band_tiles(long long n_channels, int P, int elem_bytes, int tile) {
  long long band_mb = 48;
  if (const char *env = getenv("SEISMIC_L2_BAND_MB")) {
    const long long v = atoll(env);
    if (v >= 1 && v <= 4096) band_mb = v;
  }
  const long long ev_bytes = n_channels * (P / 2) * (long long)elem_bytes;
  const long long band_events = (band_mb << 20) / (ev_bytes > 0 ? ev_bytes : 1);
  return (int)(band_events / tile > 1 ? band_events / tile : 1);
}

// Row bands of the triangle walk (band_tile, pair_core.cuh): the number of bands, and the first tile index and
// first tile row of band k (k == bands: the totals).
__host__ __device__ __forceinline__ long long band_count(long long nb, long long band) {
  if (band <= 0 || band > nb) band = nb;
  return nb > 0 ? (nb + band - 1) / band : 0;
}
__host__ __device__ __forceinline__ long long band_first_tile(long long k, long long nb, long long band) {
  if (band <= 0 || band > nb) band = nb;
  long long r0 = k * band < nb ? k * band : nb;
  // tiles in rows 0 .. r0 - 1 of the upper triangle
  return r0 * nb - r0 * (r0 - 1) / 2;
}

// ---- staged pair form (staged_core.cuh): spectra staged into shared memory
// by TMA (P = 512 .. 4096).  Work items are TI events i x TJ consecutive j
// (staged_core.cuh, StagedGeom).
bool staged_supported(int P, const PairArgs &a);
// The staged form can run at all (not disabled by SEISMIC_PAIR_KERNEL=direct,
// and the driver's tensor-map encoder is available).
bool staged_enabled();
long long staged_items_total(int P, const PairArgs &a);  // triangle or rectangle
// Triangle walk of the staged form: events per tile side and work items per tile.
void staged_tiling(int P, const PairArgs &a, long long *tile_side, long long *items_per_tile);
// Launches items [a.couple_begin, a.couple_end) of the staged decomposition.
cudaError_t launch_pairs_staged(int P, const PairArgs &a, int sm_count, cudaStream_t s);

// Pair-form dispatch (api.cu): the staged form where staged_supported, else
// the direct form with a.tile.  pair_work_total is the item count of the
// form launch_pair_work runs for `a`; ctas_per_sm (0 = occupancy maximum)
// applies to the direct form.
long long pair_work_total(int P, const PairArgs &a);
cudaError_t launch_pair_work(int P, const PairArgs &a, int sm_count, int ctas_per_sm, cudaStream_t s);
// Couples covering a rectangle of n_query x n_cols pairs with chunk width `tile`.
long long rect_couples_total(long long n_query, long long n_cols, int tile);

// Number of two-pair work items ("couples") covering the upper triangle of
// n_events with square tiles of `tile` events.
long long pair_couples_total(long long n_events, int tile);
int pair_tile_for(int P);

cudaError_t launch_spectra(int P, const SpectraArgs &a, cudaStream_t s);
cudaError_t launch_pairs(int P, const PairArgs &a, int grid_ctas, cudaStream_t s);
int pair_ctas_per_sm(int P);
cudaError_t init_twiddles(cudaStream_t s);
// Device address of the twiddle table exp(+2 pi i k / kMaxP) of the current
// device (valid after init_twiddles on that device).
const float2 *twiddle_table();

bool supported_padded_size(int P);

// ---- batched form: many independent catalogs in one persistent launch
struct BatchCatalog {  // device-resident descriptor of one catalog
  SpectraArgs spec;    // its events -> spectra, norms
  PairArgs pairs;      // its spectra -> packed outputs (couple range unused)
  int P;               // padded size of this catalog
};
struct BatchItem {     // a contiguous range of work of one catalog
  int cat;
  long long begin, end;  // spectra: row-pair indices; pairs: couple indices
};
cudaError_t launch_batched_spectra(const BatchCatalog *cats, const BatchItem *items, long long n_items, int grid,
                                   cudaStream_t s);
// Persistent pair launch over the items of the catalogs of one size P.
cudaError_t launch_batched_pairs(int P, const BatchCatalog *cats, const BatchItem *items, long long n_items,
                                 unsigned long long *counter, int grid, int max_hist, cudaStream_t s);
// Also sets the kernel's shared-memory attribute: call before any capture.
int batched_pairs_ctas_per_sm(int P, int max_hist);
// One persistent launch over the items of every size (batched_pair_kernel_mixed).
cudaError_t launch_batched_pairs_mixed(const BatchCatalog *cats, const BatchItem *items, long long n_items,
                                       unsigned long long *counter, int grid, int max_hist, cudaStream_t s);
int batched_mixed_ctas_per_sm(int max_hist);  // sets the attribute too: before any capture
int groups_per_cta(int P);  // 256 / (P / 32), at least 1

// Device context for entry points in other translation units (api.cu).
int device_context(int *sm_count, const float2 **twiddles, int **error_flag);

// ---- autotuner cache (autotune.cu): tuned pair-kernel parameters per (P, C)
struct TuneEntry {
  int tile;          // events per tile side
  int ctas_per_sm;   // 0 = occupancy maximum
  int item_groups;   // couples per batched work item, in units of groups per CTA
  int staged_warps;  // staged form: FFT warps per CTA (0: the built-in rule)
  int staged_ru;     // staged form, FP32 spectra: chunks per ring slot (0: the built-in rule)
};
TuneEntry tune_lookup(int P, int n_channels);
// The staged form's tuned CTA shape for exactly (P, spectrum rows), if any.
bool tune_staged_lookup(int P, int spec_rows, int *warps, int *ru);

// ---- lag-GEMM form (laggemm.cu): time-domain lag sums on tcgen05 tensor cores
struct LagPlan {
  bool ok;
  int lp, nt, wt, wpad, jp, nbuf, nm, strip_bytes, xs_len, jc, stages, smem, kgroup;
};
// Lag forms: SEISMIC_FORM_LAGGEMM_BF16X3 (BF16 hi + lo planes, three
// products) and SEISMIC_FORM_LAGGEMM_FP16 (one FP16 plane, one product).
int lag_planes(int form);
LagPlan lag_plan(long long n_events, int n_channels, int length, int shift, int n_hist, int nhl = 2);
size_t lag_workspace_bytes(long long n_events, int n_channels, int length, int nhl = 2);
// Prep (planes + FP64 norms) of n events into a workspace of lag_workspace_bytes.
cudaError_t lag_prepare(const float *events, long long n, int C, int length, long long ev_stride,
                        long long ch_stride, int form, void *ws, cudaStream_t s);
cudaError_t launch_lag_gemm(const float *events, long long n, int C, int length, long long ev_stride,
                            long long ch_stride, int shift, float threshold, int n_hist, float *vp, int *lp,
                            float *vn, int *ln, int *hmax, int *hmin, void *ws, int *error_flag, int sm_count,
                            cudaStream_t s, int *launches, int form);
// The triangle's A-side blocks of 128 events, the first event row of block b
// (n for b past the end), and a launch over blocks [blk_begin, blk_end) of
// events already prepared in ws: it writes the packed outputs of rows
// lag_block_row(blk_begin) .. lag_block_row(blk_end) - 1, a contiguous range.
long long lag_blocks(long long n);
long long lag_block_row(long long b, long long n);
cudaError_t launch_lag_blocks(const void *ws, long long n, int C, int length, int shift, float threshold,
                              int n_hist, float *vp, int *lp, float *vn, int *ln, int *hmax, int *hmin,
                              int *error_flag, int sm_count, cudaStream_t s, int form, long long blk_begin,
                              long long blk_end);
// Rectangle: queries (prepared in q_ws) x catalog events col_begin ..
// col_begin + n_cols - 1 (prepared in cat_ws); outputs [n_query][n_cols].
cudaError_t launch_lag_rect(const void *cat_ws, long long n_cat, const void *q_ws, long long n_query, int C,
                            int length, int shift, long long col_begin, long long n_cols, float threshold, int form,
                            float *vp, int *lp, float *vn, int *ln, int *error_flag, int sm_count, cudaStream_t s);
// Device address of the kernels' error flag (set when a bounded wait runs out).
int *device_error_flag();

// Raises the dynamic shared-memory limit of kernel `func` to at least `bytes`
// on the CURRENT device.  The attribute is per device context, so the
// setting is remembered per (kernel, device) under a lock: a second GPU in
// the same process gets its own cudaFuncSetAttribute.  Not a stream
// operation; the first call for a device should come before any capture.
cudaError_t ensure_dynamic_smem(const void *func, int bytes);
// Occupancy of the direct pair form at size P on the current device, cached
// per device (api.cu).
int pair_ctas_per_sm_cached(int P);

// Status plumbing shared by the entry points of every translation unit
// (defined in api.cu): set the calling thread's status / message.
int report_status(int status, const char *message);
int report_cuda(cudaError_t e, const char *what);
void note_launches(unsigned n);
// plain_only: the padded size must be one of the plain transform (the caller
// runs no overlap-save form).
int check_xcorr_args(long long n_events, int n_channels, int event_length, int padded, int shift, int n_hist,
                     int form, bool plain_only = false);

}  // namespace seismic
