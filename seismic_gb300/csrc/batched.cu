// Batched form: many independent station catalogs of uneven N, L and channel
// count, correlated by persistent launches replayed from one captured CUDA
// graph.
//
// Planning (seismic_batch_create) is done once on the host:
//  * per catalog: padded size P = smallest power of two >= L + shift (exact
//    linear correlation over the catalog's whole lag window), tile size from
//    the autotuner (tune_lookup), a slice of one workspace allocation for its
//    spectra and FP64 norms, and a BatchCatalog descriptor in device memory;
//  * spectra work: one item per CTA's worth of row pairs (NG(P) of them),
//    all catalogs in one launch (batched_spectra_kernel switches on P);
//  * pair work: items of item_groups * NG(P) couples of every catalog, all
//    sizes in one list sorted by decreasing cost (couples * (P log2 P +
//    products)), handed out by an atomic counter to ONE persistent launch of
//    batched_pair_kernel_mixed, which switches on each item's P;
//  * the graph: counter reset -> spectra -> pairs (two kernels per run).
//  * With SEISMIC_BATCH_PER_SIZE (flag), the pair work runs instead as one
//    persistent batched_pair_kernel<P> per size present, on fork/join
//    branches of the graph (largest total work first).
// seismic_batch_run only replays the graph: one host call, no allocation.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <vector>

#include "../../include/seismic_gb300.h"
#include "kernels.cuh"

namespace {
struct SizeClass {
  int P = 0;
  long long n_items = 0;
  size_t item_offset = 0;  // into d_pair_items
  int grid = 0;
  double work = 0.0;
  cudaStream_t branch = nullptr;
  cudaEvent_t done = nullptr;
};
}  // namespace

struct seismic_batch {
  int device = 0;
  bool use_graph = true;
  bool per_size = false;   // one pair launch per transform size instead of one mixed launch
  long long n_pair_items = 0;
  int mixed_grid = 0;
  seismic::BatchCatalog *d_cats = nullptr;
  seismic::BatchItem *d_spec_items = nullptr;
  seismic::BatchItem *d_pair_items = nullptr;
  long long n_spec_items = 0;
  unsigned long long *d_counters = nullptr;  // one per size class
  void *d_ws = nullptr;
  int spec_grid = 0, max_hist = 0;
  long long total_pairs = 0;
  std::vector<SizeClass> classes;
  cudaEvent_t fork = nullptr;
  cudaStream_t capture_stream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

namespace seismic {
namespace {

int enqueue(seismic_batch *b, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(b->d_counters, 0, sizeof(unsigned long long) * b->classes.size(), s);
  if (e == cudaSuccess) e = launch_batched_spectra(b->d_cats, b->d_spec_items, b->n_spec_items, b->spec_grid, s);
  if (!b->per_size) {
    if (e == cudaSuccess)
      e = launch_batched_pairs_mixed(b->d_cats, b->d_pair_items, b->n_pair_items, b->d_counters, b->mixed_grid,
                                     b->max_hist, s);
    return e == cudaSuccess ? SEISMIC_OK : report_cuda(e, "batched launch");
  }
  if (e == cudaSuccess) e = cudaEventRecord(b->fork, s);
  for (size_t k = 0; e == cudaSuccess && k < b->classes.size(); ++k) {
    SizeClass &c = b->classes[k];
    e = cudaStreamWaitEvent(c.branch, b->fork, 0);
    if (e == cudaSuccess)
      e = launch_batched_pairs(c.P, b->d_cats, b->d_pair_items + c.item_offset, c.n_items, b->d_counters + k,
                               c.grid, b->max_hist, c.branch);
    if (e == cudaSuccess) e = cudaEventRecord(c.done, c.branch);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, c.done, 0);
  }
  return e == cudaSuccess ? SEISMIC_OK : report_cuda(e, "batched launch");
}

void release(seismic_batch *b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  if (b->capture_stream) cudaStreamDestroy(b->capture_stream);
  for (auto &c : b->classes) {
    if (c.branch) cudaStreamDestroy(c.branch);
    if (c.done) cudaEventDestroy(c.done);
  }
  if (b->fork) cudaEventDestroy(b->fork);
  cudaFree(b->d_cats);
  cudaFree(b->d_spec_items);
  cudaFree(b->d_pair_items);
  cudaFree(b->d_counters);
  cudaFree(b->d_ws);
  delete b;
}

}  // namespace
}  // namespace seismic

using namespace seismic;

extern "C" int seismic_batch_create(const seismic_catalog *catalogs, int n_catalogs, int flags,
                                    seismic_batch **out) {
  report_status(SEISMIC_OK, "");
  if (!out) return report_status(SEISMIC_ERR_INVALID_ARGUMENT, "null output handle");
  *out = nullptr;
  if (!catalogs || n_catalogs < 1) return report_status(SEISMIC_ERR_INVALID_ARGUMENT, "no catalogs");
  int sm_count = 0;
  const float2 *tw = nullptr;
  int *err_flag = nullptr;
  int s = device_context(&sm_count, &tw, &err_flag);
  if (s) return s;

  std::vector<BatchCatalog> cats(n_catalogs);
  std::vector<int> item_groups(n_catalogs);
  std::vector<size_t> ws_off(n_catalogs), spec_bytes(n_catalogs);
  size_t ws_total = 0;
  int max_hist = 0;
  long long total_pairs = 0;
  for (int k = 0; k < n_catalogs; ++k) {
    const seismic_catalog &c = catalogs[k];
    const int P = seismic_resolve_padded_size(c.event_length, c.shift);
    s = check_xcorr_args(c.n_events, c.n_channels, c.event_length, P, c.shift, c.n_classes_hist, SEISMIC_FORM_FP32,
                         true);
    if (s) return s;
    if (P > kMaxBatchP)
      return report_status(SEISMIC_ERR_UNSUPPORTED_SIZE,
                           "batched catalogs: padded size up to 8192 (event_length + shift <= 8192)");
    if (!c.events || !c.vals_pos || !c.lags_pos || !c.vals_neg || !c.lags_neg ||
        (c.n_classes_hist > 0 && (!c.max_hist || !c.min_hist)))
      return report_status(SEISMIC_ERR_INVALID_ARGUMENT, "catalog with a null buffer");
    const long long rows = c.n_events * c.n_channels;
    ws_off[k] = ws_total;
    spec_bytes[k] = ((size_t)rows * (P / 2) * sizeof(float2) + 255) / 256 * 256;
    ws_total += spec_bytes[k] + norms_buffer_bytes(rows);
    max_hist = std::max(max_hist, c.n_classes_hist);
    total_pairs += c.n_events * (c.n_events + 1) / 2;
    cats[k].P = P;
  }

  seismic_batch *b = new seismic_batch();
  b->use_graph = !(flags & SEISMIC_BATCH_NO_GRAPH);
  b->per_size = (flags & SEISMIC_BATCH_PER_SIZE) != 0;
  b->total_pairs = total_pairs;
  b->max_hist = max_hist;
  cudaGetDevice(&b->device);
  cudaError_t e = cudaMalloc(&b->d_ws, ws_total ? ws_total : 256);
  if (e != cudaSuccess) {
    release(b);
    return report_cuda(e, "batch workspace");
  }

  std::vector<BatchItem> spec_items;
  std::map<int, std::vector<std::pair<double, BatchItem>>> by_size;
  for (int k = 0; k < n_catalogs; ++k) {
    const seismic_catalog &c = catalogs[k];
    const int P = cats[k].P;
    const int C = c.n_channels;
    const long long rows = c.n_events * C;
    const TuneEntry te = tune_lookup(P, C);
    char *ws = static_cast<char *>(b->d_ws) + ws_off[k];
    double *norms = reinterpret_cast<double *>(ws + spec_bytes[k]);
    const int prescale = C > 1 ? 1 : 0;
    SpectraArgs &sa = cats[k].spec;
    std::memset(&sa, 0, sizeof(sa));
    sa.events = c.events;
    sa.n_events = c.n_events;
    sa.n_channels = C;
    sa.length = c.event_length;
    sa.ev_stride = c.event_stride;
    sa.ch_stride = c.channel_stride;
    sa.prescale = prescale;
    sa.stype = 0;
    sa.spectra = ws;
    sa.norms = norms;
    sa.inv_norms = inverse_norms_of(norms, rows);
    sa.twiddles = tw;
    PairArgs &pa = cats[k].pairs;
    std::memset(&pa, 0, sizeof(pa));
    pa.spectra = ws;
    pa.stype = 0;
    pa.norms = norms;
    pa.inv_norms = inverse_norms_of(norms, rows);
    pa.n_events = c.n_events;
    pa.n_channels = C;
    pa.shift = c.shift;
    pa.prescaled = prescale;
    pa.threshold = c.threshold;
    pa.n_hist = c.n_classes_hist;
    pa.delta_hist = c.n_classes_hist > 0 ? (float)(1.0 / c.n_classes_hist) : 0.f;
    pa.vals_pos = c.vals_pos;
    pa.lags_pos = c.lags_pos;
    pa.vals_neg = c.vals_neg;
    pa.lags_neg = c.lags_neg;
    pa.max_hist = c.max_hist;
    pa.min_hist = c.min_hist;
    pa.tile = te.tile;
    pa.band_tiles = l2_band_tiles(C, P, 8, te.tile);  // L2 row bands, as the single-catalog launch
    pa.twiddles = tw;
    pa.couple_begin = 0;
    pa.couple_end = pair_couples_total(c.n_events, te.tile);

    const int ng = groups_per_cta(P);
    const long long row_pairs = (rows + 1) / 2;
    for (long long r = 0; r < row_pairs; r += ng) spec_items.push_back({k, r, std::min(r + ng, row_pairs)});
    const long long chunk = (long long)ng * std::max(1, te.item_groups);
    const double per_couple = 2.5 * P * std::log2((double)P) + 12.0 * C * (P / 2 + 1);
    for (long long w = 0; w < pa.couple_end; w += chunk) {
      const long long end = std::min(w + chunk, pa.couple_end);
      by_size[P].push_back({per_couple * (double)(end - w), BatchItem{k, w, end}});
    }
  }

  // per size: items largest first; sizes ordered by total work (largest first)
  std::vector<BatchItem> pair_items;
  if (!b->per_size) {  // one list over every size, largest first, one counter
    std::vector<std::pair<double, BatchItem>> all;
    for (auto &kv : by_size) all.insert(all.end(), kv.second.begin(), kv.second.end());
    std::stable_sort(all.begin(), all.end(), [](const auto &x, const auto &y) { return x.first > y.first; });
    for (auto &it : all) pair_items.push_back(it.second);
    SizeClass sc;  // one class: the counter and the item count
    sc.n_items = (long long)pair_items.size();
    b->classes.push_back(sc);
    b->n_pair_items = (long long)pair_items.size();
    b->mixed_grid = sm_count * batched_mixed_ctas_per_sm(max_hist);  // also sets the kernel attribute
    by_size.clear();
  }
  for (auto &kv : by_size) {
    auto &v = kv.second;
    std::stable_sort(v.begin(), v.end(), [](const auto &x, const auto &y) { return x.first > y.first; });
    SizeClass sc;
    sc.P = kv.first;
    sc.item_offset = pair_items.size();
    sc.n_items = (long long)v.size();
    for (auto &it : v) {
      sc.work += it.first;
      pair_items.push_back(it.second);
    }
    sc.grid = sm_count * batched_pairs_ctas_per_sm(sc.P, max_hist);  // also sets the kernel attribute
    b->classes.push_back(sc);
  }
  std::stable_sort(b->classes.begin(), b->classes.end(),
                   [](const SizeClass &x, const SizeClass &y) { return x.work > y.work; });

  b->n_spec_items = (long long)spec_items.size();
  e = cudaMalloc(&b->d_cats, sizeof(BatchCatalog) * cats.size());
  if (e == cudaSuccess) e = cudaMalloc(&b->d_spec_items, sizeof(BatchItem) * std::max<size_t>(1, spec_items.size()));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_pair_items, sizeof(BatchItem) * std::max<size_t>(1, pair_items.size()));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_counters, sizeof(unsigned long long) * b->classes.size());
  if (e == cudaSuccess)
    e = cudaMemcpy(b->d_cats, cats.data(), sizeof(BatchCatalog) * cats.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && !spec_items.empty())
    e = cudaMemcpy(b->d_spec_items, spec_items.data(), sizeof(BatchItem) * spec_items.size(),
                   cudaMemcpyHostToDevice);
  if (e == cudaSuccess && !pair_items.empty())
    e = cudaMemcpy(b->d_pair_items, pair_items.data(), sizeof(BatchItem) * pair_items.size(),
                   cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
  for (auto &c : b->classes) {
    if (!b->per_size) break;  // branches only for per-size launches
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c.branch, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c.done, cudaEventDisableTiming);
  }
  if (e != cudaSuccess) {
    release(b);
    return report_cuda(e, "batch descriptors");
  }
  b->spec_grid = (int)std::max(1LL, std::min<long long>(b->n_spec_items, (long long)sm_count * 3));
  // sets the spectra kernel's shared-memory attribute before any capture
  e = launch_batched_spectra(b->d_cats, b->d_spec_items, 0, 1, nullptr);
  if (e != cudaSuccess) {
    release(b);
    return report_cuda(e, "batched spectra set-up");
  }

  if (b->use_graph) {
    e = cudaStreamCreateWithFlags(&b->capture_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamBeginCapture(b->capture_stream, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      s = enqueue(b, b->capture_stream);
      cudaGraph_t g = nullptr;
      const cudaError_t e2 = cudaStreamEndCapture(b->capture_stream, &g);
      b->graph = g;
      if (s) {
        release(b);
        return s;
      }
      e = e2;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, b->graph, 0);
    if (e != cudaSuccess) {
      release(b);
      return report_cuda(e, "batch graph capture");
    }
  }
  *out = b;
  return SEISMIC_OK;
}

extern "C" int seismic_batch_run(seismic_batch *b, void *stream) {
  report_status(SEISMIC_OK, "");
  if (!b) return report_status(SEISMIC_ERR_INVALID_ARGUMENT, "null batch");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (b->use_graph) {
    const cudaError_t e = cudaGraphLaunch(b->exec, s);
    if (e != cudaSuccess) return report_cuda(e, "batch graph launch");
  } else {
    const int st = enqueue(b, s);
    if (st) return st;
  }
  note_launches((unsigned)seismic_batch_kernels_per_run(b));
  return SEISMIC_OK;
}

extern "C" int seismic_batch_destroy(seismic_batch *b) {
  report_status(SEISMIC_OK, "");
  if (b) release(b);
  return SEISMIC_OK;
}

extern "C" long long seismic_batch_pairs(const seismic_batch *b) { return b ? b->total_pairs : 0; }
extern "C" int seismic_batch_kernels_per_run(const seismic_batch *b) {
  if (!b) return 0;
  return b->per_size ? 1 + (int)b->classes.size() : 2;
}
