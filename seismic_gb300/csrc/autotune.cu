// Autotuner for the pair kernel.
//
// For a transform size P and C spectrum rows per event (channels, times the
// frames of the overlap-save form) it times, on the current device, on a
// synthetic catalog sized so one launch takes ~10-50 ms:
//  * the direct-load form over tile sizes (events per tile side: how many
//    couples share one event's spectrum in L1) and CTAs per SM;
//  * the TMA-staged form (P = 512 .. 4096) over its CTA shapes: FFT warps
//    per CTA (12, or the widest that keeps 128 registers a thread), which
//    sets the pairs per work item, and spectral chunks per ring slot;
//  * the batched kernel over work-item sizes (couples per item, in units of
//    the CTA's groups).
// The fastest parameters go into an in-process table (used by every later
// launch in this process) and into a text cache file, one line per (P, C):
//   P=<P> C=<C> tile=<t> ctas=<k> item=<g> us=<time> gpu=<name> warps=<w> ru=<r>
// Lookups of the direct-form and batched parameters fall back to (P, any C),
// then to built-in defaults; the staged shape is used for the exact (P, C)
// only.
#include <sys/stat.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/seismic_gb300.h"
#include "kernels.cuh"

namespace seismic {
namespace {

struct Entry {
  int P, C;
  TuneEntry t;
  double us;
  std::string gpu;
};

std::mutex g_tune_mutex;
std::vector<Entry> g_table;
bool g_loaded = false;

std::string default_cache_path() {
  const char *env = getenv("SEISMIC_TUNE_CACHE");
  if (env && *env) return env;
  const char *home = getenv("HOME");
  return std::string(home ? home : ".") + "/.cache/seismic_gb300/tune.txt";
}

void load_file(const std::string &path) {
  FILE *f = fopen(path.c_str(), "r");
  if (!f) return;
  char line[512];
  while (fgets(line, sizeof(line), f)) {
    Entry e{};
    char gpu[256] = {0};
    e.t.ctas_per_sm = 0;
    if (sscanf(line, "P=%d C=%d tile=%d ctas=%d item=%d us=%lf gpu=%255s", &e.P, &e.C, &e.t.tile,
               &e.t.ctas_per_sm, &e.t.item_groups, &e.us, gpu) >= 5) {
      if (e.t.tile < 2 || e.t.tile > 64 || (e.t.tile & 1) || e.t.item_groups < 1) continue;
      const char *w = strstr(line, " warps=");
      const char *r = strstr(line, " ru=");
      e.t.staged_warps = w ? atoi(w + 7) : 0;
      e.t.staged_ru = r ? atoi(r + 4) : 0;
      e.gpu = gpu;
      bool replaced = false;
      for (auto &x : g_table)
        if (x.P == e.P && x.C == e.C) {
          x = e;
          replaced = true;
        }
      if (!replaced) g_table.push_back(e);
    }
  }
  fclose(f);
}

void ensure_loaded() {
  if (!g_loaded) {
    load_file(default_cache_path());
    g_loaded = true;
  }
}

bool write_file(const std::string &path) {
  const size_t slash = path.find_last_of('/');
  if (slash != std::string::npos) {
    const std::string dir = path.substr(0, slash);
    for (size_t p = 1; p <= dir.size(); ++p)  // create missing parent directories
      if (p == dir.size() || dir[p] == '/') mkdir(dir.substr(0, p).c_str(), 0755);
  }
  FILE *f = fopen(path.c_str(), "w");
  if (!f) return false;
  for (const auto &e : g_table)
    fprintf(f, "P=%d C=%d tile=%d ctas=%d item=%d us=%.1f gpu=%s warps=%d ru=%d\n", e.P, e.C, e.t.tile,
            e.t.ctas_per_sm, e.t.item_groups, e.us, e.gpu.empty() ? "unknown" : e.gpu.c_str(), e.t.staged_warps,
            e.t.staged_ru);
  fclose(f);
  return true;
}

}  // namespace

TuneEntry tune_lookup(int P, int n_channels) {
  std::lock_guard<std::mutex> lock(g_tune_mutex);
  ensure_loaded();
  const Entry *any = nullptr;
  for (const auto &e : g_table) {
    if (e.P != P) continue;
    if (e.C == n_channels) return e.t;
    if (!any) any = &e;
  }
  if (any) return any->t;
  TuneEntry d{};
  d.tile = pair_tile_for(P);
  d.ctas_per_sm = 0;
  d.item_groups = 16;
  return d;
}

bool tune_staged_lookup(int P, int spec_rows, int *warps, int *ru) {
  std::lock_guard<std::mutex> lock(g_tune_mutex);
  ensure_loaded();
  for (const auto &e : g_table) {
    if (e.P == P && e.C == spec_rows && e.t.staged_warps > 0) {
      *warps = e.t.staged_warps;
      *ru = e.t.staged_ru;
      return true;
    }
  }
  return false;
}

}  // namespace seismic

using namespace seismic;

static __global__ void tune_fill_kernel(float *x, long long n, unsigned seed) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    unsigned h = (unsigned)i * 2654435761u ^ seed;
    h ^= h >> 13;
    h *= 0x5bd1e995u;
    h ^= h >> 15;
    x[i] = (float)(h & 0xffffff) / 16777216.0f - 0.5f;
  }
}

extern "C" int seismic_tuning(int padded_size, int n_channels, int *tile, int *ctas_per_sm, int *item_groups) {
  report_status(SEISMIC_OK, "");
  if (!supported_padded_size(padded_size) || n_channels < 1)
    return report_status(SEISMIC_ERR_UNSUPPORTED_SIZE, "unsupported padded size or channel count");
  const TuneEntry t = tune_lookup(padded_size, n_channels);
  if (tile) *tile = t.tile;
  if (ctas_per_sm) *ctas_per_sm = t.ctas_per_sm;
  if (item_groups) *item_groups = t.item_groups;
  return SEISMIC_OK;
}

extern "C" int seismic_tuning_staged(int padded_size, int n_channels, int *staged_warps, int *chunks_per_slot) {
  report_status(SEISMIC_OK, "");
  if (!supported_padded_size(padded_size) || n_channels < 1)
    return report_status(SEISMIC_ERR_UNSUPPORTED_SIZE, "unsupported padded size or channel count");
  int w = 0, ru = 0;
  if (!tune_staged_lookup(padded_size, n_channels, &w, &ru)) w = ru = 0;
  if (staged_warps) *staged_warps = w;
  if (chunks_per_slot) *chunks_per_slot = ru;
  return SEISMIC_OK;
}

extern "C" int seismic_autotune(int padded_size, int n_channels, const char *cache_path) {
  report_status(SEISMIC_OK, "");
  const int P = padded_size, C = n_channels;
  if (!supported_padded_size(P) || C < 1 || C > 16)
    return report_status(SEISMIC_ERR_UNSUPPORTED_SIZE, "unsupported padded size or channel count");
  int sm_count = 0;
  const float2 *tw = nullptr;
  int *err_flag = nullptr;
  int s = device_context(&sm_count, &tw, &err_flag);
  if (s) return s;

  // synthetic catalog: ~4e9 flop-units of pair work per launch
  const double unit = 2.5 * P * std::log2((double)P) + 6.0 * C * (P / 2 + 1);
  long long n = (long long)std::sqrt(2.0 * 4e9 / unit);
  n = std::max(64LL, std::min(4096LL, n));
  const int L = P / 2;
  const long long rows = n * C, npairs = n * (n + 1) / 2;
  float *ev = nullptr, *vp = nullptr, *vn = nullptr;
  int *lp = nullptr, *ln = nullptr;
  void *spec = nullptr;
  double *norms = nullptr;
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaMalloc(&ev, sizeof(float) * rows * L);
  if (e == cudaSuccess) e = cudaMalloc(&spec, sizeof(float2) * rows * (P / 2));
  if (e == cudaSuccess) e = cudaMalloc(&norms, norms_buffer_bytes(rows));
  if (e == cudaSuccess) e = cudaMalloc(&vp, sizeof(float) * npairs);
  if (e == cudaSuccess) e = cudaMalloc(&vn, sizeof(float) * npairs);
  if (e == cudaSuccess) e = cudaMalloc(&lp, sizeof(int) * npairs);
  if (e == cudaSuccess) e = cudaMalloc(&ln, sizeof(int) * npairs);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  auto cleanup = [&]() {
    cudaFree(ev);
    cudaFree(spec);
    cudaFree(norms);
    cudaFree(vp);
    cudaFree(vn);
    cudaFree(lp);
    cudaFree(ln);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (st) cudaStreamDestroy(st);
  };
  if (e != cudaSuccess) {
    cleanup();
    return report_cuda(e, "autotune buffers");
  }
  tune_fill_kernel<<<sm_count * 4, 256, 0, st>>>(ev, rows * L, 12345u);
  SpectraArgs sa;
  std::memset(&sa, 0, sizeof(sa));
  sa.events = ev;
  sa.n_events = n;
  sa.n_channels = C;
  sa.length = L;
  sa.ev_stride = (long long)C * L;
  sa.ch_stride = L;
  sa.prescale = C > 1;
  sa.stype = 0;
  sa.spectra = spec;
  sa.norms = norms;
  sa.inv_norms = inverse_norms_of(norms, rows);
  sa.twiddles = tw;
  e = launch_spectra(P, sa, st);
  note_launches(2);

  PairArgs pa;
  std::memset(&pa, 0, sizeof(pa));
  pa.spectra = spec;
  pa.stype = 0;
  pa.norms = norms;
  pa.inv_norms = inverse_norms_of(norms, rows);
  pa.n_events = n;
  pa.n_channels = C;
  pa.shift = P / 2;
  pa.prescaled = C > 1;
  pa.threshold = 0.f;
  pa.n_hist = 0;
  pa.vals_pos = vp;
  pa.lags_pos = lp;
  pa.vals_neg = vn;
  pa.lags_neg = ln;
  pa.twiddles = tw;

  auto time_pairs = [&](int tile, int ctas) -> double {
    pa.tile = tile;
    pa.couple_begin = 0;
    pa.couple_end = pair_couples_total(n, tile);
    const int ng = groups_per_cta(P);
    long long grid = (long long)sm_count * ctas;
    grid = std::min(grid, (pa.couple_end + ng - 1) / ng);
    double best = 1e30;
    for (int rep = 0; rep < 3; ++rep) {
      cudaEventRecord(e0, st);
      if (launch_pairs(P, pa, (int)grid, st) != cudaSuccess) return 1e30;
      cudaEventRecord(e1, st);
      if (cudaEventSynchronize(e1) != cudaSuccess) return 1e30;
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      best = std::min(best, (double)ms * 1e3);
    }
    note_launches(3);
    return best;
  };

  const int max_ctas = std::max(1, pair_ctas_per_sm(P));
  TuneEntry bestT{pair_tile_for(P), 0, 16, 0, 0};
  double best_us = 1e30;
  const int tiles[] = {2, 4, 8, 16};
  for (int tile : tiles) {
    for (int ctas = 1; ctas <= max_ctas; ++ctas) {
      const double us = time_pairs(tile, ctas);
      if (us < best_us) {
        best_us = us;
        bestT.tile = tile;
        bestT.ctas_per_sm = ctas;
      }
    }
  }

  // the staged form's CTA shape (FFT warps per CTA x chunks per ring slot)
  if (P >= 512 && P <= 4096 && staged_enabled()) {
    const int shapes[4][2] = {{12, 4}, {12, 2}, {99, 4}, {99, 2}};  // 99: the widest CTA of this P
    double best_staged = 1e30;
    for (const auto &sh : shapes) {
      PairArgs sa2 = pa;
      sa2.staged_warps = sh[0];
      sa2.staged_ru = sh[1];
      sa2.tile = bestT.tile;
      sa2.error_flag = err_flag;
      sa2.couple_begin = 0;
      sa2.couple_end = pair_work_total(P, sa2);
      double best = 1e30;
      for (int rep = 0; rep < 3; ++rep) {
        cudaEventRecord(e0, st);
        if (launch_pair_work(P, sa2, sm_count, 0, st) != cudaSuccess) break;
        cudaEventRecord(e1, st);
        if (cudaEventSynchronize(e1) != cudaSuccess) break;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        best = std::min(best, (double)ms * 1e3);
      }
      note_launches(3);
      if (best < best_staged) {
        best_staged = best;
        bestT.staged_warps = sh[0] == 12 ? 12 : 99;
        bestT.staged_ru = sh[1];
      }
    }
  }

  // batched work-item size, on a one-catalog batch of the same data
  {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    ensure_loaded();
  }
  const int items[] = {4, 16, 64};
  double best_item_us = 1e30;
  for (int ig : items) {
    {
      std::lock_guard<std::mutex> lock(g_tune_mutex);
      bool found = false;
      for (auto &x : g_table)
        if (x.P == P && x.C == C) {
          x.t = bestT;
          x.t.item_groups = ig;
          found = true;
        }
      if (!found) {
        Entry en{P, C, bestT, best_us, ""};
        en.t.item_groups = ig;
        g_table.push_back(en);
      }
    }
    seismic_catalog cat;
    std::memset(&cat, 0, sizeof(cat));
    cat.events = ev;
    cat.n_events = n;
    cat.n_channels = C;
    cat.event_length = L;
    cat.event_stride = (long long)C * L;
    cat.channel_stride = L;
    cat.shift = P / 2;
    cat.vals_pos = vp;
    cat.lags_pos = lp;
    cat.vals_neg = vn;
    cat.lags_neg = ln;
    seismic_batch *b = nullptr;
    if (seismic_batch_create(&cat, 1, SEISMIC_BATCH_NO_GRAPH, &b) != SEISMIC_OK) continue;
    double bu = 1e30;
    for (int rep = 0; rep < 3; ++rep) {
      cudaEventRecord(e0, st);
      seismic_batch_run(b, st);
      cudaEventRecord(e1, st);
      cudaEventSynchronize(e1);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      bu = std::min(bu, (double)ms * 1e3);
    }
    seismic_batch_destroy(b);
    if (bu < best_item_us) {
      best_item_us = bu;
      bestT.item_groups = ig;
    }
  }
  cleanup();
  e = cudaGetLastError();
  if (e != cudaSuccess) return report_cuda(e, "autotune");

  char name[256] = "unknown";
  cudaDeviceProp prop;
  int dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess && cudaGetDeviceProperties(&prop, dev) == cudaSuccess) {
    snprintf(name, sizeof(name), "%s", prop.name);
    for (char *c = name; *c; ++c)
      if (*c == ' ') *c = '_';
  }
  std::lock_guard<std::mutex> lock(g_tune_mutex);
  for (auto &x : g_table)
    if (x.P == P && x.C == C) {
      x.t = bestT;
      x.us = best_us;
      x.gpu = name;
    }
  const std::string path = cache_path && *cache_path ? cache_path : default_cache_path();
  if (!write_file(path)) return report_status(SEISMIC_ERR_INVALID_ARGUMENT, "cannot write the tuning cache file");
  return SEISMIC_OK;
}
