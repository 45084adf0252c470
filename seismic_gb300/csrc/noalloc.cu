// seismic_xcorr_device_noalloc: the all-pairs correlation of
// seismic_xcorr_device for callers that cannot allocate device memory.
//
// Some callers must not call cudaMalloc/cudaFree at all: a host framework
// that has already reserved (nearly) all of the GPU's memory for its own pool
// and forbids other allocations, a process running under a fixed device
// memory quota, or a latency-critical loop where an allocation's implicit
// device synchronisation and unpredictable cost are not acceptable.  Such a
// caller still owns its inputs and outputs, but cannot hand this library a
// workspace or let it grow one.  This entry point therefore takes its
// scratch (the packed spectra and FP64 norms that kernel (a) produces and
// kernel (b) reads) from one file-scope __device__ array of fixed size,
// kNoAllocScratchBytes (64 MiB), reserved when this module is loaded on a
// device and held until the process exits.
//
// Rules for callers:
//  * The first call on each device sets up that device (looks up the
//    scratch array's device address and fills the twiddle table); make that
//    first call before any stream capture on the device.
//  * All calls on a device share the one scratch array, and each call
//    overwrites it completely before reading it, so nothing carries over
//    between calls; but calls whose work overlaps on the GPU (different
//    streams, or host threads racing) corrupt each other's scratch.
//    Serialise them, e.g. on one stream.
//  * Catalogs whose spectra + norms exceed the scratch are rejected with
//    SEISMIC_ERR_WORKSPACE_TOO_SMALL before anything is launched.
//  * The call returns once the kernels are queued.  A kernel whose bounded
//    wait ran out leaves the device error flag set (its outputs are then
//    invalid); after synchronising the stream, seismic_check_device_error()
//    reads and clears that flag, and it allocates nothing either.
//  * Launch shapes come from the same autotuner cache as seismic_xcorr_device
//    (a host-side lookup), so both entry points run the same kernels.
#include <cstdio>
#include <mutex>

#include "../../include/seismic_gb300.h"
#include "kernels.cuh"

namespace seismic {

constexpr size_t kNoAllocScratchBytes = (size_t)64 << 20;  // SEISMIC_NOALLOC_SCRATCH_BYTES

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {

constexpr int kMaxDevices = 64;

struct NoAllocDevice {
  bool ready = false;
  unsigned char *scratch = nullptr;  // device address of g_noalloc_scratch
  const float2 *twiddles = nullptr;
  int *error_flag = nullptr;  // device flag set by a bounded wait that ran out
  int sm_count = 0;
};

std::mutex g_noalloc_mutex;
NoAllocDevice g_noalloc_devices[kMaxDevices];

size_t round256(size_t v) { return (v + 255) & ~(size_t)255; }

// Once per device, with that device current.  Uses no allocating call.
int noalloc_setup(NoAllocDevice **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return report_cuda(e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) return report_status(SEISMIC_ERR_NO_DEVICE, "device index out of range");
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  NoAllocDevice &d = g_noalloc_devices[dev];
  if (!d.ready) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return report_cuda(e, "cudaGetSymbolAddress(no-alloc scratch)");
    e = cudaDeviceGetAttribute(&d.sm_count, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return report_cuda(e, "cudaDeviceGetAttribute");
    e = init_twiddles(0);
    if (e == cudaSuccess) e = cudaStreamSynchronize(0);
    if (e != cudaSuccess) return report_cuda(e, "twiddle init");
    note_launches(1);
    d.twiddles = twiddle_table();
    if (!d.twiddles) return report_status(SEISMIC_ERR_CUDA, "twiddle table address");
    d.error_flag = device_error_flag();
    if (!d.error_flag) return report_status(SEISMIC_ERR_CUDA, "device error flag address");
    d.scratch = static_cast<unsigned char *>(p);
    d.ready = true;
  }
  *out = &d;
  return SEISMIC_OK;
}

}  // namespace
}  // namespace seismic

using namespace seismic;

extern "C" size_t seismic_noalloc_scratch_bytes(void) { return kNoAllocScratchBytes; }

extern "C" int seismic_xcorr_device_noalloc(const float *d_events, long long n_events, int n_channels,
                                            int event_length, long long event_stride, long long channel_stride,
                                            int padded_size, int shift, float threshold, int n_classes_hist,
                                            float *d_vals_pos, int *d_lags_pos, float *d_vals_neg,
                                            int *d_lags_neg, int *d_max_hist, int *d_min_hist, void *stream) {
  report_status(SEISMIC_OK, "");
  if (padded_size == 0) padded_size = seismic_resolve_padded_size(event_length, shift);
  padded_size = effective_padded(padded_size, event_length, shift);
  int s = check_xcorr_args(n_events, n_channels, event_length, padded_size, shift, n_classes_hist,
                           SEISMIC_FORM_FP32, true);
  if (s) return s;
  if (!d_events || !d_vals_pos || !d_lags_pos || !d_vals_neg || !d_lags_neg)
    return report_status(SEISMIC_ERR_INVALID_ARGUMENT, "null buffer");
  if (n_classes_hist > 0 && (!d_max_hist || !d_min_hist))
    return report_status(SEISMIC_ERR_INVALID_ARGUMENT, "null histogram buffer");

  const long long rows = n_events * n_channels;
  const size_t spec_b = round256((size_t)rows * (size_t)(padded_size / 2) * sizeof(float2));
  const size_t norm_b = norms_buffer_bytes(rows);  // FP64 norms + FP64 inverse norms
  if (spec_b + norm_b > kNoAllocScratchBytes) {
    char msg[200];
    snprintf(msg, sizeof(msg),
             "catalog needs %zu bytes of scratch (n_events*n_channels*(padded_size*4 + 16)); "
             "the no-alloc entry point has %zu",
             spec_b + norm_b, kNoAllocScratchBytes);
    return report_status(SEISMIC_ERR_WORKSPACE_TOO_SMALL, msg);
  }

  NoAllocDevice *d = nullptr;
  if ((s = noalloc_setup(&d))) return s;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  float2 *spectra = reinterpret_cast<float2 *>(d->scratch);
  double *norms = reinterpret_cast<double *>(d->scratch + spec_b);
  const int prescale = n_channels > 1 ? 1 : 0;

  SpectraArgs sa{};
  sa.events = d_events;
  sa.n_events = n_events;
  sa.n_channels = n_channels;
  sa.length = event_length;
  sa.ev_stride = event_stride;
  sa.ch_stride = channel_stride;
  sa.prescale = prescale;
  sa.stype = 0;  // FP32 spectra
  sa.spectra = spectra;
  sa.norms = norms;
  sa.inv_norms = inverse_norms_of(norms, rows);
  sa.twiddles = d->twiddles;
  cudaError_t e = launch_spectra(padded_size, sa, st);
  if (e != cudaSuccess) return report_cuda(e, "spectra kernel launch");
  note_launches(1);

  PairArgs pa{};
  pa.spectra = spectra;
  pa.norms = norms;
  pa.inv_norms = inverse_norms_of(norms, rows);
  pa.n_events = n_events;
  pa.n_channels = n_channels;
  pa.shift = shift;
  pa.prescaled = prescale;
  pa.stype = 0;
  pa.threshold = threshold;
  pa.n_hist = n_classes_hist;
  pa.delta_hist = n_classes_hist > 0 ? (float)(1.0 / n_classes_hist) : 0.f;
  pa.vals_pos = d_vals_pos;
  pa.lags_pos = d_lags_pos;
  pa.vals_neg = d_vals_neg;
  pa.lags_neg = d_lags_neg;
  pa.max_hist = d_max_hist;
  pa.min_hist = d_min_hist;
  const TuneEntry tune = tune_lookup(padded_size, n_channels);  // host-side cache, as seismic_xcorr_device
  pa.tile = tune.tile;
  pa.twiddles = d->twiddles;
  pa.error_flag = d->error_flag;
  pa.couple_begin = 0;
  pa.couple_end = pair_work_total(padded_size, pa);
  e = launch_pair_work(padded_size, pa, d->sm_count, tune.ctas_per_sm, st);
  if (e != cudaSuccess) return report_cuda(e, "pair kernel launch");
  note_launches(1);
  return SEISMIC_OK;
}
