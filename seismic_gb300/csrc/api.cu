// C ABI of libseismic_gb300.so: drop-in reference symbols and native entry
// points (declared in include/seismic_gb300.h).
//
// Host-side flow of one correlation (replacing correlationCUDA,
// Correlation_in_CUDA/correlation_cuda.cu:530-673, and correlationCPP,
// Correlation_in_OMP/correlation_c.cpp:210-298):
//   H2D of the L valid samples of every event row (one 2-D copy)
//   kernel (a) spectra_kernel : packed half spectra + FP64 norms
//   kernel (b) pair_kernel    : all pairs of the upper triangle
//   D2H of the four packed outputs and the histograms.
#include <atomic>
#include <cstdarg>
#include <map>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/seismic_gb300.h"
#include "kernels.cuh"

namespace seismic {

// ------------------------------------------------------------------ errors
static thread_local int tl_status = SEISMIC_OK;
static thread_local char tl_message[512] = {0};

static int set_status(int status, const char *fmt, ...) {
  tl_status = status;
  if (status == SEISMIC_OK) {
    tl_message[0] = 0;
    return status;
  }
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(tl_message, sizeof(tl_message), fmt, ap);
  va_end(ap);
  return status;
}

static int cuda_status(cudaError_t e, const char *what) {
  if (e == cudaSuccess) return SEISMIC_OK;
  if (e == cudaErrorMemoryAllocation)
    return set_status(SEISMIC_ERR_OUT_OF_MEMORY, "%s: %s", what, cudaGetErrorString(e));
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver)
    return set_status(SEISMIC_ERR_NO_DEVICE, "%s: %s", what, cudaGetErrorString(e));
  return set_status(SEISMIC_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define SEISMIC_TRY(expr, what)                          \
  do {                                                   \
    cudaError_t e__ = (expr);                            \
    if (e__ != cudaSuccess) return cuda_status(e__, what); \
  } while (0)

static std::atomic<unsigned long long> g_launches{0};

// ----------------------------------------------------------- device state
struct DeviceState {
  bool ready = false;
  int sm_count = 0;
  const float2 *twiddles = nullptr;
  int *error_flag = nullptr;  // set by kernels whose bounded waits ran out
  cudaStream_t stream = nullptr;
  cudaStream_t copy_stream = nullptr;  // device-to-host copies of the host entry point (made on first use)
  // grow-only cached buffers used when the caller passes none
  void *ws = nullptr;
  size_t ws_bytes = 0;
  void *io = nullptr;  // events + outputs + histograms for the host entry point
  size_t io_bytes = 0;
};

static std::mutex g_mutex;
static std::vector<DeviceState> g_devices;

// Pair launches per host call: the device-to-host copy of each chunk's
// outputs overlaps the next chunk's kernel.
constexpr int kHostChunks = 8;
// SEISMIC_HOST_CHUNKS (1 .. 64) overrides the chunk count.
static int host_chunks() {
  if (const char *e = getenv("SEISMIC_HOST_CHUNKS")) {
    const int v = atoi(e);
    if (v >= 1 && v <= 64) return v;
  }
  return kHostChunks;
}

// Packed index of pair (i, i): where row i of the upper triangle starts.
static long long packed_row_start(long long i, long long n) { return i * n - i * (i - 1) / 2; }

static int ensure_device(int *dev_out, DeviceState **st_out) {
  int dev = 0;
  SEISMIC_TRY(cudaGetDevice(&dev), "cudaGetDevice");
  std::lock_guard<std::mutex> lock(g_mutex);
  if ((int)g_devices.size() <= dev) g_devices.resize(dev + 1);
  DeviceState &st = g_devices[dev];
  if (!st.ready) {
    SEISMIC_TRY(cudaDeviceGetAttribute(&st.sm_count, cudaDevAttrMultiProcessorCount, dev),
                "cudaDeviceGetAttribute");
    SEISMIC_TRY(cudaStreamCreateWithFlags(&st.stream, cudaStreamNonBlocking), "cudaStreamCreate");
    SEISMIC_TRY(init_twiddles(st.stream), "twiddle init");
    g_launches.fetch_add(1);
    SEISMIC_TRY(cudaStreamSynchronize(st.stream), "twiddle init sync");
    st.twiddles = twiddle_table();
    if (!st.twiddles) return set_status(SEISMIC_ERR_CUDA, "twiddle table address");
    st.error_flag = device_error_flag();
    if (!st.error_flag) return set_status(SEISMIC_ERR_CUDA, "device error flag address");
    st.ready = true;
  }
  *dev_out = dev;
  *st_out = &st;
  return SEISMIC_OK;
}

static int grow(void **ptr, size_t *have, size_t need, const char *what) {
  if (*have >= need && *ptr) return SEISMIC_OK;
  if (*ptr) {
    cudaFree(*ptr);
    *ptr = nullptr;
    *have = 0;
  }
  SEISMIC_TRY(cudaMalloc(ptr, need), what);
  *have = need;
  return SEISMIC_OK;
}

static size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

// Spectrum storage of an FFT form: 0 float2, 1 half2, 2 bfloat162.
static int form_stype(int form) {
  return form == SEISMIC_FORM_FP16_SPECTRA ? 1 : (form == SEISMIC_FORM_BF16_SPECTRA ? 2 : 0);
}
static size_t spectra_bytes(long long rows, int P, int stype = 0) {
  return align256((size_t)rows * (size_t)(P / 2) * (stype ? 4 : 8));
}
static size_t norms_bytes(long long rows) { return norms_buffer_bytes(rows); }

// Overlap-save plan of a short lag window (declared in kernels.cuh).  The
// pair cost of a transform size is its inverse FFT plus the conj-products
// of every spectrum row, 2.5 Q log2 Q + 6 C nb (Q/2) flop per pair; a block
// form is chosen when it costs under 3/4 of the plain size-P form, and
// always (the cheapest Q) for a padded size beyond the plain transform's
// kMaxP, which has no other form.  Only where the plain form has no circular
// aliasing (L + shift <= P), so both compute the same linear correlation,
// and only for the sizes of the staged pair form (it has no direct-load
// twin).  SEISMIC_BLOCK_FORM=off keeps the plain form (padded sizes up to
// kMaxP).
BlockPlan block_plan(int length, int shift, int P, int n_channels, int stype) {
  BlockPlan best;
  const char *env = getenv("SEISMIC_BLOCK_FORM");
  if ((env && strcmp(env, "off") == 0) || !staged_enabled()) return best;
  // FP32 and FP16 spectra (BF16's 8-bit mantissa, summed over the frames,
  // would pass its 1e-3 coefficient bar)
  if (stype < 0 || stype > 1 || shift < 1 || (long long)length + shift > P) return best;
  auto cost = [&](int q, int nb) {
    return 2.5 * q * (31 - __builtin_clz((unsigned)q)) + 6.0 * n_channels * nb * (q / 2);
  };
  double best_cost = P > kMaxP ? 1e300 : 0.75 * cost(P, 1);
  for (int q = 512; q <= 4096 && q < P; q <<= 1) {
    const int b = q - 2 * shift;  // B + 2 shift <= Q
    if (b < q / 8) continue;      // blocks too short to pay for their frames
    const int nb = (length + b - 1) / b;
    const double c = cost(q, nb);
    if (c < best_cost) {
      best_cost = c;
      best.Q = q;
      best.B = b;
      best.nb = nb;
    }
  }
  return best;
}

// Workspace layout of an FFT form on one catalog: plain size-P spectra + norms,
// or the overlap-save A frames, W frames + norms.
struct FftJob {
  int P = 0;          // transform size of the pair kernel (Q in the overlap-save form)
  int stype = 0;
  int C = 1;
  int L = 0;
  int shift = 0;
  BlockPlan bp;       // bp.nb == 0: plain
  long long n = 0;
  size_t spec_b = 0;  // one spectra array (plain or A), 256-byte aligned
  int prescale = 0;
  int spec_rows() const { return bp.nb ? C * bp.nb : C; }
  size_t total() const { return (bp.nb ? 2 : 1) * spec_b + norms_bytes(n * C); }
  void *spectra(void *ws) const { return ws; }  // plain, or A frames
  void *spectra_w(void *ws) const { return bp.nb ? static_cast<char *>(ws) + spec_b : nullptr; }
  double *norms(void *ws) const {
    return reinterpret_cast<double *>(static_cast<char *>(ws) + (bp.nb ? 2 : 1) * spec_b);
  }
};

static FftJob fft_job(long long n, int C, int L, int shift, int P, int stype) {
  FftJob j;
  j.n = n;
  j.C = C;
  j.L = L;
  j.shift = shift;
  j.stype = stype;
  j.bp = block_plan(L, shift, P, C, stype);
  j.P = j.bp.nb ? j.bp.Q : P;
  j.spec_b = spectra_bytes(n * C * (j.bp.nb ? j.bp.nb : 1), j.P, stype);
  // half-precision spectra are always scaled by 1/norm (keeps |X| <= sqrt(L))
  j.prescale = (C > 1 || stype != 0) ? 1 : 0;
  return j;
}

static bool is_lag_form(int form) {
  return form == SEISMIC_FORM_LAGGEMM_BF16X3 || form == SEISMIC_FORM_LAGGEMM_FP16;
}

// A padded size the FFT forms run: a power of two up to kMaxP (the plain
// transform), or beyond it up to kMaxPadded where the overlap-save form
// takes the lag window (unless plain_only: entry points given plain spectra).
static bool fft_size_ok(int padded, int event_length, int shift, int n_channels, int form, bool plain_only) {
  if (supported_padded_size(padded)) return true;
  if (plain_only || padded <= kMaxP || padded > kMaxPadded || (padded & (padded - 1)) != 0) return false;
  return block_plan(event_length, shift, padded, n_channels, form_stype(form)).nb > 0;
}

static int validate(long long n_events, int n_channels, int event_length, int padded, int shift,
                    int n_hist, int form, bool plain_only = false) {
  if (n_events < 1) return set_status(SEISMIC_ERR_INVALID_ARGUMENT, "n_events must be >= 1 (got %lld)", n_events);
  if (n_channels < 1) return set_status(SEISMIC_ERR_INVALID_ARGUMENT, "n_channels must be >= 1");
  if (event_length < 1) return set_status(SEISMIC_ERR_INVALID_ARGUMENT, "event_length must be >= 1");
  if (is_lag_form(form) ? (padded < kMinP || padded > kMaxPadded || (padded & (padded - 1)) != 0)
                        : !fft_size_ok(padded, event_length, shift, n_channels, form, plain_only))
    return set_status(SEISMIC_ERR_UNSUPPORTED_SIZE,
                      plain_only ? "paddedSize %d unsupported (power of two in [64, 16384], or any size >= "
                                   "event_length + shift up to 16384)"
                                 : "paddedSize %d unsupported (power of two in [64, 16384], or any size >= "
                                   "event_length + shift; larger ones where the overlap-save form takes the lag "
                                   "window: shift <= 1792, FP32 or FP16 spectra)",
                      padded);
  if (event_length > padded)
    return set_status(SEISMIC_ERR_INVALID_ARGUMENT, "event_length %d exceeds paddedSize %d", event_length, padded);
  if (shift < 0) return set_status(SEISMIC_ERR_INVALID_ARGUMENT, "shift must be >= 0");
  if (n_hist < 0) return set_status(SEISMIC_ERR_INVALID_ARGUMENT, "n_classes_hist must be >= 0");
  if (form != SEISMIC_FORM_FP32 && !is_lag_form(form) && form != SEISMIC_FORM_FP16_SPECTRA &&
      form != SEISMIC_FORM_BF16_SPECTRA)
    return set_status(SEISMIC_ERR_INVALID_ARGUMENT, "unknown form %d", form);
  if (is_lag_form(form)) {
    if (shift < 1 || 2 * shift > 512)
      return set_status(SEISMIC_ERR_UNSUPPORTED_SIZE, "lag-GEMM form needs 1 <= shift <= 256 (got %d)", shift);
    if (!lag_plan(n_events, n_channels, event_length, shift, n_hist, lag_planes(form)).ok)
      return set_status(SEISMIC_ERR_UNSUPPORTED_SIZE,
                        "lag-GEMM form: event_length %d with shift %d does not fit in shared memory", event_length,
                        shift);
  }
  // lag indices must fit in int32 alongside the sentinel values
  if (shift > (1 << 29)) return set_status(SEISMIC_ERR_INVALID_ARGUMENT, "shift too large");
  return SEISMIC_OK;
}

static int run_spectra(const DeviceState &st, const float *d_events, long long n, int C, int L, long long ev_stride,
                       long long ch_stride, int P, int prescale, void *spectra, double *norms, cudaStream_t stream,
                       int stype = 0) {
  SpectraArgs sa{};
  sa.stype = stype;
  sa.events = d_events;
  sa.n_events = n;
  sa.n_channels = C;
  sa.length = L;
  sa.ev_stride = ev_stride;
  sa.ch_stride = ch_stride;
  sa.prescale = prescale;
  sa.spectra = spectra;
  sa.norms = norms;
  sa.inv_norms = inverse_norms_of(norms, n * C);
  sa.twiddles = st.twiddles;
  SEISMIC_TRY(launch_spectra(P, sa, stream), "spectra kernel launch");
  g_launches.fetch_add(1);
  return SEISMIC_OK;
}

static int run_pairs(const DeviceState &st, const void *spectra, const double *norms, long long n, int C, int P,
                     int prescaled, int shift, float thr, int n_hist, float *vp, int *lp, float *vn, int *ln,
                     int *hmax, int *hmin, cudaStream_t stream, int stype = 0, long long range_begin = 0,
                     long long range_end = -1, const void *spectra_i = nullptr, int spec_rows = 0) {
  PairArgs pa{};  // zero: triangle mode, no query spectra
  pa.spectra = spectra;
  pa.spectra_i = spectra_i;
  pa.spec_channels = spec_rows;
  pa.stype = stype;
  pa.norms = norms;
  pa.inv_norms = inverse_norms_of(norms, n * C);
  pa.n_events = n;
  pa.n_channels = C;
  pa.shift = shift;
  pa.prescaled = prescaled;
  pa.threshold = thr;
  pa.n_hist = n_hist;
  pa.delta_hist = n_hist > 0 ? (float)(1.0 / n_hist) : 0.f;
  pa.vals_pos = vp;
  pa.lags_pos = lp;
  pa.vals_neg = vn;
  pa.lags_neg = ln;
  pa.max_hist = hmax;
  pa.min_hist = hmin;
  const TuneEntry tune = tune_lookup(P, C);  // autotuner cache, else built-in defaults
  pa.tile = tune.tile;
  pa.twiddles = st.twiddles;
  pa.error_flag = st.error_flag;
  const long long total = pair_work_total(P, pa);
  pa.couple_begin = range_begin < 0 ? 0 : (range_begin > total ? total : range_begin);
  pa.couple_end = (range_end < 0 || range_end > total) ? total : range_end;
  if (pa.couple_end <= pa.couple_begin) return SEISMIC_OK;
  SEISMIC_TRY(launch_pair_work(P, pa, st.sm_count, tune.ctas_per_sm, stream), "pair kernel launch");
  g_launches.fetch_add(1);
  return SEISMIC_OK;
}

long long pair_work_total(int P, const PairArgs &a) {
  if (staged_supported(P, a)) return staged_items_total(P, a);
  return a.rect ? rect_couples_total(a.n_query, a.n_cols, a.tile) : pair_couples_total(a.n_events, a.tile);
}

cudaError_t launch_pair_work(int P, const PairArgs &a, int sm_count, int ctas_per_sm, cudaStream_t stream) {
  if (a.couple_end <= a.couple_begin) return cudaSuccess;
  if (staged_supported(P, a)) return launch_pairs_staged(P, a, sm_count, stream);
  if (a.spectra_i) return cudaErrorNotSupported;  // overlap-save frames: staged form only
  PairArgs d = a;  // direct form: L2 row bands of tiles (triangle mode)
  if (!d.rect && d.band_tiles == 0) d.band_tiles = l2_band_tiles(d.n_channels, P, d.stype ? 4 : 8, d.tile);
  const int occ = pair_ctas_per_sm_cached(P);
  const int ctas = (ctas_per_sm > 0 && ctas_per_sm < occ) ? ctas_per_sm : occ;
  const int NG = groups_per_cta(P);
  long long want = (d.couple_end - d.couple_begin + NG - 1) / NG;
  long long grid = (long long)sm_count * ctas;
  if (want < grid) grid = want;
  if (grid < 1) grid = 1;
  return launch_pairs(P, d, (int)grid, stream);
}

cudaError_t ensure_dynamic_smem(const void *func, int bytes) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  static std::mutex m;
  static std::map<std::pair<const void *, int>, int> done;  // (kernel, device) -> bytes set
  std::lock_guard<std::mutex> lock(m);
  auto it = done.find({func, dev});
  if (it != done.end() && it->second >= bytes) return cudaSuccess;
  e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess) done[{func, dev}] = bytes;
  return e;
}

int pair_ctas_per_sm_cached(int P) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) dev = 0;
  static std::mutex m;
  static std::map<std::pair<int, int>, int> cache;  // (device, P) -> CTAs per SM
  {
    std::lock_guard<std::mutex> lock(m);
    auto it = cache.find({dev, P});
    if (it != cache.end()) return it->second;
  }
  const int n = pair_ctas_per_sm(P);  // sets the kernel attribute on this device
  std::lock_guard<std::mutex> lock(m);
  cache[{dev, P}] = n;
  return n;
}

// Row bands of the pair form launch_pair_work runs on the triangle of these
// spectra: tile side, work items per tile, tiles per side and tile rows per
// band, computed as the kernels compute them.
struct PairBandPlan {
  long long tile_side, items_per_tile, nb, band;
};
static PairBandPlan pair_band_plan(int P, const void *spectra, int stype, long long n, int C,
                                   const void *spectra_i = nullptr, int spec_rows = 0) {
  PairArgs a{};
  a.spectra = spectra;
  a.spectra_i = spectra_i;
  a.spec_channels = spec_rows;
  a.stype = stype;
  a.n_events = n;
  a.n_channels = C;
  a.tile = tune_lookup(P, C).tile;
  PairBandPlan b{};
  if (staged_supported(P, a)) {
    staged_tiling(P, a, &b.tile_side, &b.items_per_tile);
  } else {
    b.tile_side = a.tile;
    b.items_per_tile = (long long)a.tile * a.tile / 2;
  }
  b.nb = (n + b.tile_side - 1) / b.tile_side;
  b.band = l2_band_tiles(spectrum_rows(a), P, stype ? 4 : 8, (int)b.tile_side);
  return b;
}
// First event row of band k (n past the last band).
static long long band_row(const PairBandPlan &b, long long k, long long n) {
  const long long band = (b.band <= 0 || b.band > b.nb) ? b.nb : b.band;
  const long long r = k * band * b.tile_side;
  return r < n ? r : n;
}

// Kernel (a) of an FFT job: plain spectra, or the overlap-save frames.
static int run_fft_spectra(const DeviceState &st, const FftJob &job, const float *d_events, long long ev_stride,
                           long long ch_stride, void *ws, cudaStream_t stream) {
  if (!job.bp.nb)
    return run_spectra(st, d_events, job.n, job.C, job.L, ev_stride, ch_stride, job.P, job.prescale,
                       job.spectra(ws), job.norms(ws), stream, job.stype);
  SpectraArgs sa{};
  sa.events = d_events;
  sa.n_events = job.n;
  sa.n_channels = job.C;
  sa.length = job.L;
  sa.ev_stride = ev_stride;
  sa.ch_stride = ch_stride;
  sa.prescale = job.prescale;
  sa.stype = job.stype;
  sa.spectra = job.spectra(ws);
  sa.spectra_w = job.spectra_w(ws);
  sa.norms = job.norms(ws);
  sa.inv_norms = inverse_norms_of(sa.norms, job.n * job.C);
  sa.twiddles = st.twiddles;
  sa.blocks = job.bp.nb;
  sa.block_len = job.bp.B;
  sa.block_shift = job.shift;
  SEISMIC_TRY(launch_block_spectra(job.P, sa, stream), "overlap-save spectra kernel launch");
  g_launches.fetch_add(1);
  return SEISMIC_OK;
}

// Kernel (b) of an FFT job over work items [range_begin, range_end).
static int run_fft_pairs(const DeviceState &st, const FftJob &job, void *ws, float thr, int n_hist, float *vp,
                         int *lp, float *vn, int *ln, int *hmax, int *hmin, cudaStream_t stream,
                         long long range_begin = 0, long long range_end = -1) {
  if (!job.bp.nb)
    return run_pairs(st, job.spectra(ws), job.norms(ws), job.n, job.C, job.P, job.prescale, job.shift, thr, n_hist,
                     vp, lp, vn, ln, hmax, hmin, stream, job.stype, range_begin, range_end);
  // the W frames are the j side (TMA-staged columns), the A frames row i
  return run_pairs(st, job.spectra_w(ws), job.norms(ws), job.n, job.C, job.P, job.prescale, job.shift, thr, n_hist,
                   vp, lp, vn, ln, hmax, hmin, stream, job.stype, range_begin, range_end, job.spectra(ws),
                   job.spec_rows());
}

static PairBandPlan job_band_plan(const FftJob &job, void *ws) {
  return job.bp.nb ? pair_band_plan(job.P, job.spectra_w(ws), job.stype, job.n, job.C, job.spectra(ws),
                                    job.spec_rows())
                   : pair_band_plan(job.P, job.spectra(ws), job.stype, job.n, job.C);
}

int device_context(int *sm_count, const float2 **twiddles, int **error_flag) {
  int dev;
  DeviceState *st;
  const int s = ensure_device(&dev, &st);
  if (s) return s;
  *sm_count = st->sm_count;
  *twiddles = st->twiddles;
  *error_flag = st->error_flag;
  return SEISMIC_OK;
}

// Used by entry points defined in other translation units.
int report_status(int status, const char *message) { return set_status(status, "%s", message); }
int report_cuda(cudaError_t e, const char *what) { return cuda_status(e, what); }
void note_launches(unsigned n) { g_launches.fetch_add(n); }
int check_xcorr_args(long long n_events, int n_channels, int event_length, int padded, int shift, int n_hist,
                     int form, bool plain_only) {
  return validate(n_events, n_channels, event_length, padded, shift, n_hist, form, plain_only);
}

// Core: spectra + pairs on `stream`; buffers all on device.
// stages: 1 = the per-event transforms into ws (spectra + norms, or the
// lag form's planes + norms), 2 = the pairs from ws, 3 = both.
static int run_xcorr(const DeviceState &st, const float *d_events, long long n, int C, int L, long long ev_stride,
                     long long ch_stride, int P, int shift, float thr, int n_hist, float *vp, int *lp, float *vn,
                     int *ln, int *hmax, int *hmin, void *ws, cudaStream_t stream, int form = SEISMIC_FORM_FP32,
                     int stages = 3) {
  if (is_lag_form(form)) {
    if (stages == 3) {
      int launched = 0;
      cudaError_t e = launch_lag_gemm(d_events, n, C, L, ev_stride, ch_stride, shift, thr, n_hist, vp, lp, vn, ln,
                                      hmax, hmin, ws, st.error_flag, st.sm_count, stream, &launched, form);
      g_launches.fetch_add(launched);
      SEISMIC_TRY(e, "lag-GEMM launch");
      return SEISMIC_OK;
    }
    if (stages & 1) {
      SEISMIC_TRY(lag_prepare(d_events, n, C, L, ev_stride, ch_stride, form, ws, stream), "lag-GEMM prep");
      g_launches.fetch_add(1);
    }
    if (stages & 2) {
      SEISMIC_TRY(launch_lag_blocks(ws, n, C, L, shift, thr, n_hist, vp, lp, vn, ln, hmax, hmin, st.error_flag,
                                    st.sm_count, stream, form, 0, lag_blocks(n)),
                  "lag-GEMM launch");
      g_launches.fetch_add(1);
    }
    return SEISMIC_OK;
  }
  const FftJob job = fft_job(n, C, L, shift, P, form_stype(form));
  if (stages & 1) {
    const int s = run_fft_spectra(st, job, d_events, ev_stride, ch_stride, ws, stream);
    if (s) return s;
  }
  if (stages & 2) return run_fft_pairs(st, job, ws, thr, n_hist, vp, lp, vn, ln, hmax, hmin, stream);
  return SEISMIC_OK;
}

}  // namespace seismic

using namespace seismic;

extern "C" {

int seismic_last_error(void) { return tl_status; }
const char *seismic_last_error_message(void) { return tl_message; }

const char *seismic_status_string(int status) {
  switch (status) {
    case SEISMIC_OK: return "ok";
    case SEISMIC_ERR_INVALID_ARGUMENT: return "invalid argument";
    case SEISMIC_ERR_UNSUPPORTED_SIZE: return "unsupported size";
    case SEISMIC_ERR_OUT_OF_MEMORY: return "out of device memory";
    case SEISMIC_ERR_CUDA: return "CUDA error";
    case SEISMIC_ERR_NO_DEVICE: return "no CUDA device";
    case SEISMIC_ERR_WORKSPACE_TOO_SMALL: return "workspace too small";
    case SEISMIC_ERR_DEVICE_TIMEOUT: return "device wait timed out";
    default: return "unknown status";
  }
}

unsigned long long seismic_launch_count(void) { return g_launches.load(); }

int seismic_resolve_padded_size(int event_length, int shift) {
  if (event_length < 1 || shift < 0) return 0;
  long long need = (long long)event_length + shift;
  long long p = kMinP;
  while (p < need) p <<= 1;
  if (p <= kMaxP) return (int)p;
  return (p <= kMaxPadded && shift <= kMaxBlockShift) ? (int)p : 0;  // the overlap-save form's sizes
}

size_t seismic_xcorr_workspace_bytes(long long n_events, int n_channels, int event_length, int shift,
                                     int padded_size, int form) {
  if (n_events < 1 || n_channels < 1 || event_length < 1) return 0;
  if (is_lag_form(form)) {
    if (!lag_plan(n_events, n_channels, event_length, shift, 0, lag_planes(form)).ok) return 0;
    return lag_workspace_bytes(n_events, n_channels, event_length, lag_planes(form));
  }
  if (padded_size == 0) padded_size = seismic_resolve_padded_size(event_length, shift);
  padded_size = effective_padded(padded_size, event_length, shift);
  if (!fft_size_ok(padded_size, event_length, shift, n_channels, form, false)) return 0;
  return fft_job(n_events, n_channels, event_length, shift, padded_size, form_stype(form)).total();
}

int seismic_fft_plan(int event_length, int shift, int padded_size, int n_channels, int form, int *transform_size,
                     int *blocks, int *block_length) {
  set_status(SEISMIC_OK, "");
  if (padded_size == 0) padded_size = seismic_resolve_padded_size(event_length, shift);
  padded_size = effective_padded(padded_size, event_length, shift);
  int s = validate(1, n_channels, event_length, padded_size, shift, 0, form);
  if (s) return s;
  if (is_lag_form(form)) return set_status(SEISMIC_ERR_INVALID_ARGUMENT, "lag-GEMM forms use no transform");
  const BlockPlan bp = block_plan(event_length, shift, padded_size, n_channels, form_stype(form));
  if (transform_size) *transform_size = bp.nb ? bp.Q : padded_size;
  if (blocks) *blocks = bp.nb;
  if (block_length) *block_length = bp.nb ? bp.B : event_length;
  return SEISMIC_OK;
}

int seismic_check_device_error(void) {
  // Allocation-free (usable by callers of seismic_xcorr_device_noalloc): no
  // stream, no buffer, only the flag's symbol address and two small copies.
  set_status(SEISMIC_OK, "");
  int *flag_addr = device_error_flag();
  if (!flag_addr) return set_status(SEISMIC_ERR_CUDA, "device error flag address");
  SEISMIC_TRY(cudaDeviceSynchronize(), "device synchronise");
  int flag = 0;
  SEISMIC_TRY(cudaMemcpy(&flag, flag_addr, sizeof(int), cudaMemcpyDeviceToHost), "error flag read");
  if (flag) {
    const int zero = 0;
    SEISMIC_TRY(cudaMemcpy(flag_addr, &zero, sizeof(int), cudaMemcpyHostToDevice), "error flag clear");
    return set_status(SEISMIC_ERR_DEVICE_TIMEOUT, "a kernel gave up a bounded wait; its results are invalid");
  }
  return SEISMIC_OK;
}

int seismic_xcorr_device(const float *d_events, long long n_events, int n_channels, int event_length,
                         long long event_stride, long long channel_stride, int padded_size, int shift,
                         float threshold, int n_classes_hist, int form, float *d_vals_pos, int *d_lags_pos,
                         float *d_vals_neg, int *d_lags_neg, int *d_max_hist, int *d_min_hist, void *workspace,
                         size_t workspace_bytes, void *stream) {
  return seismic_xcorr_device_stages(d_events, n_events, n_channels, event_length, event_stride, channel_stride,
                                     padded_size, shift, threshold, n_classes_hist, form, d_vals_pos, d_lags_pos,
                                     d_vals_neg, d_lags_neg, d_max_hist, d_min_hist, workspace, workspace_bytes,
                                     stream, 3);
}

int seismic_xcorr_device_stages(const float *d_events, long long n_events, int n_channels, int event_length,
                                long long event_stride, long long channel_stride, int padded_size, int shift,
                                float threshold, int n_classes_hist, int form, float *d_vals_pos, int *d_lags_pos,
                                float *d_vals_neg, int *d_lags_neg, int *d_max_hist, int *d_min_hist,
                                void *workspace, size_t workspace_bytes, void *stream, int stages) {
  set_status(SEISMIC_OK, "");
  if (stages < 1 || stages > 3) return set_status(SEISMIC_ERR_INVALID_ARGUMENT, "stages must be 1, 2 or 3");
  if (stages != 3 && !workspace)
    return set_status(SEISMIC_ERR_INVALID_ARGUMENT, "running one stage needs the caller's workspace");
  if (padded_size == 0) padded_size = seismic_resolve_padded_size(event_length, shift);
  padded_size = effective_padded(padded_size, event_length, shift);
  int s = validate(n_events, n_channels, event_length, padded_size, shift, n_classes_hist, form);
  if (s) return s;
  if (!d_events || !d_vals_pos || !d_lags_pos || !d_vals_neg || !d_lags_neg)
    return set_status(SEISMIC_ERR_INVALID_ARGUMENT, "null buffer");
  if (n_classes_hist > 0 && (!d_max_hist || !d_min_hist))
    return set_status(SEISMIC_ERR_INVALID_ARGUMENT, "null histogram buffer");
  int dev;
  DeviceState *st;
  if ((s = ensure_device(&dev, &st))) return s;
  const size_t need = seismic_xcorr_workspace_bytes(n_events, n_channels, event_length, shift, padded_size, form);
  if (workspace) {
    if (workspace_bytes < need)
      return set_status(SEISMIC_ERR_WORKSPACE_TOO_SMALL, "workspace %zu < %zu bytes", workspace_bytes, need);
    if (reinterpret_cast<uintptr_t>(workspace) & 255u)  // TMA sources and 16-byte loads inside it
      return set_status(SEISMIC_ERR_INVALID_ARGUMENT, "workspace must be 256-byte aligned");
  } else {
    std::lock_guard<std::mutex> lock(g_mutex);
    if ((s = grow(&st->ws, &st->ws_bytes, need, "workspace allocation"))) return s;
    workspace = st->ws;
  }
  return run_xcorr(*st, d_events, n_events, n_channels, event_length, event_stride, channel_stride, padded_size,
                   shift, threshold, n_classes_hist, d_vals_pos, d_lags_pos, d_vals_neg, d_lags_neg, d_max_hist,
                   d_min_hist, workspace, (cudaStream_t)stream, form, stages);
}

int seismic_spectra_device(const float *d_events, long long n_events, int n_channels, int event_length,
                           long long event_stride, long long channel_stride, int padded_size, int prescale,
                           void *d_spectra, double *d_norms, void *stream) {
  set_status(SEISMIC_OK, "");
  int s = validate(n_events, n_channels, event_length, padded_size, 0, 0, SEISMIC_FORM_FP32, true);
  if (s) return s;
  if (!d_events || !d_spectra || !d_norms) return set_status(SEISMIC_ERR_INVALID_ARGUMENT, "null buffer");
  int dev;
  DeviceState *st;
  if ((s = ensure_device(&dev, &st))) return s;
  return run_spectra(*st, d_events, n_events, n_channels, event_length, event_stride, channel_stride, padded_size,
                     prescale ? 1 : 0, reinterpret_cast<float2 *>(d_spectra), d_norms, (cudaStream_t)stream);
}

int seismic_pairs_device(const void *d_spectra, const double *d_norms, long long n_events, int n_channels,
                         int padded_size, int prescaled, int shift, float threshold, int n_classes_hist, int form,
                         float *d_vals_pos, int *d_lags_pos, float *d_vals_neg, int *d_lags_neg, int *d_max_hist,
                         int *d_min_hist, void *stream) {
  set_status(SEISMIC_OK, "");
  int s = validate(n_events, n_channels, 1, padded_size, shift, n_classes_hist, form, true);
  if (s) return s;
  if (!d_spectra || !d_norms || !d_vals_pos || !d_lags_pos || !d_vals_neg || !d_lags_neg)
    return set_status(SEISMIC_ERR_INVALID_ARGUMENT, "null buffer");
  if (n_classes_hist > 0 && (!d_max_hist || !d_min_hist))
    return set_status(SEISMIC_ERR_INVALID_ARGUMENT, "null histogram buffer");
  if (form != SEISMIC_FORM_FP32)
    return set_status(SEISMIC_ERR_INVALID_ARGUMENT, "seismic_pairs_device pairs FP32 spectra (form 0)");
  if (reinterpret_cast<uintptr_t>(d_spectra) & 15u)
    return set_status(SEISMIC_ERR_INVALID_ARGUMENT, "spectra must be 16-byte aligned");
  if (n_channels > 1 && !prescaled)
    return set_status(SEISMIC_ERR_INVALID_ARGUMENT, "multichannel spectra must be prescaled");
  int dev;
  DeviceState *st;
  if ((s = ensure_device(&dev, &st))) return s;
  return run_pairs(*st, reinterpret_cast<const float2 *>(d_spectra), d_norms, n_events, n_channels, padded_size,
                   prescaled ? 1 : 0, shift, threshold, n_classes_hist, d_vals_pos, d_lags_pos, d_vals_neg,
                   d_lags_neg, d_max_hist, d_min_hist, (cudaStream_t)stream);
}

long long seismic_pair_couples(long long n_events, int padded_size, int n_channels) {
  if (n_events < 1 || n_channels < 1 || !supported_padded_size(padded_size)) return 0;
  PairArgs pa{};  // FP32 spectra at an aligned address, triangle mode
  pa.n_events = n_events;
  pa.n_channels = n_channels;
  pa.tile = tune_lookup(padded_size, n_channels).tile;
  return pair_work_total(padded_size, pa);
}

int seismic_pairs_device_range(const void *d_spectra, const double *d_norms, long long n_events, int n_channels,
                               int padded_size, int prescaled, int shift, float threshold, int n_classes_hist,
                               long long couple_begin, long long couple_end, float *d_vals_pos, int *d_lags_pos,
                               float *d_vals_neg, int *d_lags_neg, int *d_max_hist, int *d_min_hist, void *stream) {
  set_status(SEISMIC_OK, "");
  int s = validate(n_events, n_channels, 1, padded_size, shift, n_classes_hist, SEISMIC_FORM_FP32, true);
  if (s) return s;
  if (!d_spectra || !d_norms || !d_vals_pos || !d_lags_pos || !d_vals_neg || !d_lags_neg)
    return set_status(SEISMIC_ERR_INVALID_ARGUMENT, "null buffer");
  if (n_classes_hist > 0 && (!d_max_hist || !d_min_hist))
    return set_status(SEISMIC_ERR_INVALID_ARGUMENT, "null histogram buffer");
  if (n_channels > 1 && !prescaled)
    return set_status(SEISMIC_ERR_INVALID_ARGUMENT, "multichannel spectra must be prescaled");
  if (couple_begin < 0 || couple_end < couple_begin)
    return set_status(SEISMIC_ERR_INVALID_ARGUMENT, "bad couple range");
  if (reinterpret_cast<uintptr_t>(d_spectra) & 15u)
    return set_status(SEISMIC_ERR_INVALID_ARGUMENT, "spectra must be 16-byte aligned");
  int dev;
  DeviceState *st;
  if ((s = ensure_device(&dev, &st))) return s;
  return run_pairs(*st, d_spectra, d_norms, n_events, n_channels, padded_size, prescaled ? 1 : 0, shift, threshold,
                   n_classes_hist, d_vals_pos, d_lags_pos, d_vals_neg, d_lags_neg, d_max_hist, d_min_hist,
                   (cudaStream_t)stream, 0, couple_begin, couple_end);
}

int seismic_xcorr_host(const float *events, long long n_events, int n_channels, int event_length,
                       long long event_stride, long long channel_stride, int padded_size, int shift,
                       float threshold, int n_classes_hist, int form, float *vals_pos, int *lags_pos,
                       float *vals_neg, int *lags_neg, int *max_hist, int *min_hist) {
  set_status(SEISMIC_OK, "");
  if (padded_size == 0) padded_size = seismic_resolve_padded_size(event_length, shift);
  padded_size = effective_padded(padded_size, event_length, shift);
  int s = validate(n_events, n_channels, event_length, padded_size, shift, n_classes_hist, form);
  if (s) return s;
  if (!events || !vals_pos || !lags_pos || !vals_neg || !lags_neg)
    return set_status(SEISMIC_ERR_INVALID_ARGUMENT, "null buffer");
  if (n_classes_hist > 0 && (!max_hist || !min_hist))
    return set_status(SEISMIC_ERR_INVALID_ARGUMENT, "null histogram buffer");
  if (event_stride != (long long)n_channels * channel_stride || channel_stride < event_length)
    return set_status(SEISMIC_ERR_INVALID_ARGUMENT,
                      "host events need event_stride == n_channels*channel_stride >= n_channels*event_length");
  int dev;
  DeviceState *st;
  if ((s = ensure_device(&dev, &st))) return s;

  const long long rows = n_events * n_channels;
  const long long npairs = n_events * (n_events + 1) / 2;
  const size_t ev_b = align256((size_t)rows * event_length * sizeof(float));
  const size_t out_b = align256((size_t)npairs * 4);
  const size_t hist_b = align256((size_t)2 * (n_classes_hist > 0 ? n_classes_hist : 1) * sizeof(int));
  const size_t ws_b = seismic_xcorr_workspace_bytes(n_events, n_channels, event_length, shift, padded_size, form);
  const size_t total = ev_b + 4 * out_b + hist_b + ws_b;

  std::lock_guard<std::mutex> lock(g_mutex);  // the cached io buffer is shared
  if ((s = grow(&st->io, &st->io_bytes, total, "device buffers for the host call"))) return s;
  char *base = reinterpret_cast<char *>(st->io);
  float *d_ev = reinterpret_cast<float *>(base);
  float *d_vp = reinterpret_cast<float *>(base + ev_b);
  int *d_lp = reinterpret_cast<int *>(base + ev_b + out_b);
  float *d_vn = reinterpret_cast<float *>(base + ev_b + 2 * out_b);
  int *d_ln = reinterpret_cast<int *>(base + ev_b + 3 * out_b);
  int *d_hist = reinterpret_cast<int *>(base + ev_b + 4 * out_b);
  void *d_ws = base + ev_b + 4 * out_b + hist_b;
  cudaStream_t stream = st->stream;

  SEISMIC_TRY(cudaMemcpy2DAsync(d_ev, (size_t)event_length * sizeof(float), events,
                                (size_t)channel_stride * sizeof(float), (size_t)event_length * sizeof(float),
                                (size_t)rows, cudaMemcpyHostToDevice, stream),
              "events H2D");
  if (n_classes_hist > 0)
    SEISMIC_TRY(cudaMemsetAsync(d_hist, 0, 2 * (size_t)n_classes_hist * sizeof(int), stream), "hist clear");
  int *d_hmax = d_hist, *d_hmin = d_hist + (n_classes_hist > 0 ? n_classes_hist : 0);
  if (is_lag_form(form)) {
    // the lag-GEMM walks the triangle by blocks of rows, whose packed outputs
    // are contiguous: launch it in chunks and copy each chunk's outputs back
    // on a second stream while the next chunk runs
    if (!st->copy_stream)
      SEISMIC_TRY(cudaStreamCreateWithFlags(&st->copy_stream, cudaStreamNonBlocking), "copy stream");
    SEISMIC_TRY(lag_prepare(d_ev, n_events, n_channels, event_length, (long long)n_channels * event_length,
                            event_length, form, d_ws, stream),
                "lag-GEMM prep");
    g_launches.fetch_add(1);
    const long long nblk = lag_blocks(n_events);
    const int chunks = (int)(nblk < host_chunks() ? nblk : host_chunks());
    float *hv[2] = {vals_pos, vals_neg};
    int *hl[2] = {lags_pos, lags_neg};
    float *dv[2] = {d_vp, d_vn};
    int *dl[2] = {d_lp, d_ln};
    std::vector<cudaEvent_t> done(chunks, nullptr);
    int status = SEISMIC_OK;
    long long b0 = 0;
    for (int k = 0; k < chunks && status == SEISMIC_OK; ++k) {
      // chunk k ends where the rows so far hold about (k + 1) / chunks of the pairs
      const long long target = npairs * (k + 1) / chunks;
      long long b1 = b0 + 1;
      while (b1 < nblk && packed_row_start(lag_block_row(b1, n_events), n_events) < target) ++b1;
      if (k == chunks - 1) b1 = nblk;
      const long long p0 = packed_row_start(lag_block_row(b0, n_events), n_events);
      const long long p1 = packed_row_start(lag_block_row(b1, n_events), n_events);
      cudaError_t e = launch_lag_blocks(d_ws, n_events, n_channels, event_length, shift, threshold, n_classes_hist,
                                        d_vp, d_lp, d_vn, d_ln, d_hmax, d_hmin, st->error_flag, st->sm_count,
                                        stream, form, b0, b1);
      if (e == cudaSuccess) {
        g_launches.fetch_add(1);
        e = cudaEventCreateWithFlags(&done[k], cudaEventDisableTiming);
      }
      if (e == cudaSuccess) e = cudaEventRecord(done[k], stream);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(st->copy_stream, done[k], 0);
      for (int o = 0; o < 2 && e == cudaSuccess && p1 > p0; ++o) {
        e = cudaMemcpyAsync(hv[o] + p0, dv[o] + p0, (size_t)(p1 - p0) * 4, cudaMemcpyDeviceToHost, st->copy_stream);
        if (e == cudaSuccess)
          e = cudaMemcpyAsync(hl[o] + p0, dl[o] + p0, (size_t)(p1 - p0) * 4, cudaMemcpyDeviceToHost,
                              st->copy_stream);
      }
      if (e != cudaSuccess) status = cuda_status(e, "lag-GEMM chunk");
      if (b1 >= nblk) break;
      b0 = b1;
    }
    const cudaError_t es = cudaStreamSynchronize(st->copy_stream);
    for (cudaEvent_t ev : done)
      if (ev) cudaEventDestroy(ev);
    if (status) return status;
    SEISMIC_TRY(es, "copy stream sync");
  } else {
    // FFT forms: the pair kernels walk the triangle in L2 row bands, whose
    // outputs are contiguous packed rows: launch them in chunks of bands
    // and copy each chunk back on a second stream while the next one runs
    const FftJob job = fft_job(n_events, n_channels, event_length, shift, padded_size, form_stype(form));
    s = run_fft_spectra(*st, job, d_ev, (long long)n_channels * event_length, event_length, d_ws, stream);
    if (s) return s;
    const PairBandPlan bp = job_band_plan(job, d_ws);
    const long long bands = band_count(bp.nb, bp.band);
    const int chunks = (int)(bands < host_chunks() ? bands : host_chunks());
    if (!st->copy_stream)
      SEISMIC_TRY(cudaStreamCreateWithFlags(&st->copy_stream, cudaStreamNonBlocking), "copy stream");
    std::vector<cudaEvent_t> done(chunks > 0 ? chunks : 0, nullptr);
    int status = SEISMIC_OK;
    long long k0 = 0;
    for (int k = 0; k < chunks && status == SEISMIC_OK; ++k) {
      // chunk k ends at the first band boundary holding >= (k + 1) / chunks of the pairs
      const long long target = npairs * (k + 1) / chunks;
      long long k1 = k0 + 1;
      while (k1 < bands && packed_row_start(band_row(bp, k1, n_events), n_events) < target) ++k1;
      if (k == chunks - 1) k1 = bands;
      const long long r0 = band_row(bp, k0, n_events), r1 = band_row(bp, k1, n_events);
      const long long p0 = packed_row_start(r0, n_events), p1 = packed_row_start(r1, n_events);
      s = run_fft_pairs(*st, job, d_ws, threshold, n_classes_hist, d_vp, d_lp, d_vn, d_ln, d_hmax, d_hmin, stream,
                        band_first_tile(k0, bp.nb, bp.band) * bp.items_per_tile,
                        band_first_tile(k1, bp.nb, bp.band) * bp.items_per_tile);
      if (s) {
        status = s;
        break;
      }
      cudaError_t e = cudaEventCreateWithFlags(&done[k], cudaEventDisableTiming);
      if (e == cudaSuccess) e = cudaEventRecord(done[k], stream);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(st->copy_stream, done[k], 0);
      float *hv[2] = {vals_pos, vals_neg};
      int *hl[2] = {lags_pos, lags_neg};
      float *dv[2] = {d_vp, d_vn};
      int *dl[2] = {d_lp, d_ln};
      for (int o = 0; o < 2 && e == cudaSuccess && p1 > p0; ++o) {
        e = cudaMemcpyAsync(hv[o] + p0, dv[o] + p0, (size_t)(p1 - p0) * 4, cudaMemcpyDeviceToHost, st->copy_stream);
        if (e == cudaSuccess)
          e = cudaMemcpyAsync(hl[o] + p0, dl[o] + p0, (size_t)(p1 - p0) * 4, cudaMemcpyDeviceToHost,
                              st->copy_stream);
      }
      if (e != cudaSuccess) status = cuda_status(e, "pair chunk copy");
      if (k1 >= bands) break;
      k0 = k1;
    }
    const cudaError_t es = cudaStreamSynchronize(st->copy_stream);
    for (cudaEvent_t ev : done)
      if (ev) cudaEventDestroy(ev);
    if (status) return status;
    SEISMIC_TRY(es, "copy stream sync");
  }
  std::vector<int> h(n_classes_hist > 0 ? 2 * (size_t)n_classes_hist : 0);
  if (n_classes_hist > 0)
    SEISMIC_TRY(cudaMemcpyAsync(h.data(), d_hist, h.size() * sizeof(int), cudaMemcpyDeviceToHost, stream),
                "hist D2H");
  SEISMIC_TRY(cudaStreamSynchronize(stream), "host call sync");
  {  // every form's kernels raise this flag when a bounded wait runs out
    int flag = 0;
    SEISMIC_TRY(cudaMemcpy(&flag, st->error_flag, sizeof(int), cudaMemcpyDeviceToHost), "error flag read");
    if (flag) {
      const int zero = 0;
      cudaMemcpy(st->error_flag, &zero, sizeof(int), cudaMemcpyHostToDevice);
      return set_status(SEISMIC_ERR_DEVICE_TIMEOUT, "a kernel gave up a bounded wait; results invalid");
    }
  }
  for (int k = 0; k < n_classes_hist; ++k) {
    max_hist[k] += h[k];
    min_hist[k] += h[n_classes_hist + k];
  }
  return SEISMIC_OK;
}

int seismic_release_cached_memory(void) {
  set_status(SEISMIC_OK, "");
  int dev = 0;
  SEISMIC_TRY(cudaGetDevice(&dev), "cudaGetDevice");
  std::lock_guard<std::mutex> lock(g_mutex);
  if ((int)g_devices.size() > dev) {
    DeviceState &st = g_devices[dev];
    if (st.ws) cudaFree(st.ws);
    if (st.io) cudaFree(st.io);
    st.ws = st.io = nullptr;
    st.ws_bytes = st.io_bytes = 0;
  }
  return SEISMIC_OK;
}

// ----------------------------------------------------- reference symbols
static void report_legacy(const char *fn, int status) {
  if (status != SEISMIC_OK) fprintf(stderr, "seismic_gb300 %s: %s\n", fn, tl_message);
}

void correlationCPP(float *events, float *events_reversed, int n_events, int event_length, int shift,
                    int paddedSize, int num_threads, int chunk_size, float threshold, int n_classes_hist,
                    float *xcorr_vals_pos, int *xcorr_lags_pos, float *xcorr_vals_neg, int *xcorr_lags_neg,
                    int *max_hist, int *min_hist) {
  (void)events_reversed;
  (void)num_threads;
  (void)chunk_size;
  if (n_classes_hist < 1) {
    set_status(SEISMIC_ERR_INVALID_ARGUMENT, "n_classes_hist must be >= 1");
    report_legacy("correlationCPP", tl_status);
    return;
  }
  const int s = seismic_xcorr_host(events, n_events, 1, event_length, paddedSize, paddedSize, paddedSize, shift,
                                   threshold, n_classes_hist, SEISMIC_FORM_FP32, xcorr_vals_pos, xcorr_lags_pos,
                                   xcorr_vals_neg, xcorr_lags_neg, max_hist, min_hist);
  report_legacy("correlationCPP", s);
}

void correlationCUDA(float *events, float *events_reversed, int n_events, int event_length, int shift,
                     int paddedSize, int num_threads, float threshold, float *xcorr_vals_pos, int *xcorr_lags_pos,
                     float *xcorr_vals_neg, int *xcorr_lags_neg) {
  (void)events_reversed;
  (void)num_threads;
  const int s = seismic_xcorr_host(events, n_events, 1, event_length, paddedSize, paddedSize, paddedSize, shift,
                                   threshold, 0, SEISMIC_FORM_FP32, xcorr_vals_pos, xcorr_lags_pos, xcorr_vals_neg,
                                   xcorr_lags_neg, nullptr, nullptr);
  report_legacy("correlationCUDA", s);
}

void initialiseCUDA(void) {
  set_status(SEISMIC_OK, "");
  int dev;
  DeviceState *st;
  const int s = ensure_device(&dev, &st);
  if (s == SEISMIC_OK) {
    for (int P = kMinP; P <= kMaxP; P <<= 1) pair_ctas_per_sm(P);  // loads the kernels
  }
  report_legacy("initialiseCUDA", s);
}

}  // extern "C"
