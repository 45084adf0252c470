// Serving loop: a catalog kept resident on the device (spectra + FP64
// norms), query requests correlated against it with continuous batching.
//
//  * seismic_server_create computes the catalog's packed half spectra (FP32
//    or FP16) and FP64 norms once and keeps them; the time-domain catalog is
//    not kept.  It reserves the device memory pool (the HBM budget) from which
//    in-flight requests take their buffers.
//  * seismic_server_submit only enqueues (host-side, O(1)) and returns a
//    ticket.  A dispatcher thread admits pending requests in arrival order as
//    soon as a slot (a CUDA stream) and enough pool memory are free -- a
//    request that does not fit lets later, smaller ones go first -- and
//    enqueues its whole pipeline on the slot's stream:
//      H2D query events -> spectra kernel (query rows) -> rectangular pair
//      kernel (queries x catalog subset) -> top-K kernel -> D2H outputs ->
//      host callback (completion time, frees slot + memory).
//    Requests in different slots run concurrently on the device.
//  * The rectangular pair kernel is persistent (one CTA per SM, nearly all
//    of an SM's shared memory), so two of them interleave only at CTA
//    boundaries, and a kernel launched behind one would take every SM the
//    first one frees -- including the SMs the first request's own top-K
//    kernel needs, which would then wait for the whole second kernel.  So
//    the pair kernels of admitted requests run in admission order (each
//    waits on the previous one's completion event), on all but `spare_sms`
//    SMs; the other stages of every request in flight (H2D, query
//    transform, top-K, D2H) run beside them on the spare SMs and the copy
//    engines.  A request finishes one pair-kernel time after the one ahead
//    of it, and the device never idles between requests.
//  * seismic_server_wait blocks until a ticket completes and returns its
//    latency (submit -> results in host memory).
// Results do not depend on what else is in flight: every request has its own
// buffers and the kernels are deterministic.
#include <chrono>
#include <cstdlib>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/seismic_gb300.h"
#include "kernels.cuh"

namespace seismic {

// ------------------------------------------------------------- top-K kernel
// One CTA per query row: the K largest values of vals[row][0..n) (ties to the
// smaller column), as (value, catalog index = col_begin + column).
constexpr int kTopKMax = 64;
constexpr int kTopKThreads = 256;

__global__ void __launch_bounds__(kTopKThreads)
    topk_kernel(const float *__restrict__ vals, long long n, int k, long long col_begin, float *__restrict__ out_v,
                long long *__restrict__ out_i) {
  const long long row = blockIdx.x;
  const float *v = vals + row * n;
  // per-thread sorted list (descending value, ascending index)
  float lv[kTopKMax];
  long long li[kTopKMax];
  int cnt = 0;
  for (int q = 0; q < kTopKMax; ++q) {
    lv[q] = -INFINITY;
    li[q] = LLONG_MAX;
  }
  for (long long j = threadIdx.x; j < n; j += blockDim.x) {
    const float x = v[j];
    if (cnt == k && !(x > lv[k - 1])) continue;  // later columns lose ties
    int pos = (cnt < k) ? cnt : k - 1;
    while (pos > 0 && x > lv[pos - 1]) {
      lv[pos] = lv[pos - 1];
      li[pos] = li[pos - 1];
      --pos;
    }
    lv[pos] = x;
    li[pos] = j;
    if (cnt < k) ++cnt;
  }
  // K rounds of a block-wide arg-max over the list heads
  __shared__ float s_v[kTopKThreads / 32];
  __shared__ long long s_i[kTopKThreads / 32];
  __shared__ int s_t[kTopKThreads / 32];
  int head = 0;
  for (int r = 0; r < k; ++r) {
    float bv = head < cnt ? lv[head] : -INFINITY;
    long long bi = head < cnt ? li[head] : LLONG_MAX;
    int bt = threadIdx.x;
    for (int o = 16; o > 0; o >>= 1) {
      const float ov = __shfl_xor_sync(0xffffffffu, bv, o);
      const long long oi = __shfl_xor_sync(0xffffffffu, bi, o);
      const int ot = __shfl_xor_sync(0xffffffffu, bt, o);
      if (ov > bv || (ov == bv && oi < bi)) {
        bv = ov;
        bi = oi;
        bt = ot;
      }
    }
    if ((threadIdx.x & 31) == 0) {
      s_v[threadIdx.x / 32] = bv;
      s_i[threadIdx.x / 32] = bi;
      s_t[threadIdx.x / 32] = bt;
    }
    __syncthreads();
    float wv = s_v[0];
    long long wi = s_i[0];
    int wt = s_t[0];
    for (int w = 1; w < kTopKThreads / 32; ++w)
      if (s_v[w] > wv || (s_v[w] == wv && s_i[w] < wi)) {
        wv = s_v[w];
        wi = s_i[w];
        wt = s_t[w];
      }
    if (threadIdx.x == 0) {
      out_v[row * k + r] = wi == LLONG_MAX ? 0.f : wv;
      out_i[row * k + r] = wi == LLONG_MAX ? -1 : col_begin + wi;
    }
    if (threadIdx.x == wt) ++head;
    __syncthreads();
  }
}

}  // namespace seismic

using namespace seismic;

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
  long long ticket = 0;
  const float *query = nullptr;
  int n_query = 0;
  int query_length = 0;  // samples per query row (<= the catalog's L; zero-padded)
  long long col_begin = 0, n_cols = 0;
  float *vp = nullptr, *vn = nullptr;
  int *lp = nullptr, *ln = nullptr;
  float *topk_v = nullptr;
  long long *topk_i = nullptr;
  size_t bytes = 0;      // pool bytes it needs
  size_t pool_off = 0;   // where it got them
  int slot = -1;
  Clock::time_point submitted, finished;
  bool done = false;
  int status = SEISMIC_OK;
  struct seismic_server *server = nullptr;
};

}  // namespace

struct seismic_server {
  // catalog
  long long n_cat = 0;
  int C = 0, L = 0, P = 0, shift = 0, stype = 0, prescale = 0, topk = 16;
  // FFT forms: the overlap-save plan of the lag window (nb == 0: plain size-P
  // transforms).  With a plan the catalog keeps its W frames and each request
  // transforms its queries into A frames; PT is the pair kernel's size.
  BlockPlan bp;
  int PT = 0;
  float threshold = 0.f;
  void *cat_spectra = nullptr;
  double *cat_norms = nullptr;
  // lag forms (SEISMIC_FORM_LAGGEMM_*): the catalog's 16-bit planes + norms
  int lag_form = 0;
  void *cat_lag = nullptr;
  int sm_count = 0;
  const float2 *tw = nullptr;
  int *error_flag = nullptr;  // device flag set by a bounded wait that ran out
  int max_query = 64;
  // A request joins others already on the device only when at least this
  // many requests wait (counting it).  Default 1: admitted whenever a slot
  // and pool memory are free (continuous batching);
  // SEISMIC_SERVER_OVERLAP_BACKLOG=2 holds a lone arrival until the device
  // is idle.
  int overlap_backlog = 1;
  // SMs the pair kernels leave to the other stages of requests in flight
  // (SEISMIC_SERVER_SPARE_SMS, default 2).
  int spare_sms = 2;
  // completion of each slot's pair kernel, and the most recent one enqueued
  // (the next pair kernel waits on it); dispatcher thread only
  std::vector<cudaEvent_t> pair_done;
  cudaEvent_t last_pair = nullptr;
  // pool
  char *pool = nullptr;
  size_t pool_bytes = 0;
  std::map<size_t, size_t> free_list;  // offset -> size
  // slots
  std::vector<cudaStream_t> streams;
  std::vector<bool> slot_busy;
  // requests
  std::mutex mu;
  std::condition_variable cv_dispatch, cv_done;
  std::deque<Request *> pending;
  std::unordered_map<long long, Request *> by_ticket;
  long long next_ticket = 1;
  bool stopping = false;
  std::thread dispatcher;
  long long completed = 0, pairs_done = 0;
};

namespace {

size_t round256(size_t v) { return (v + 255) & ~(size_t)255; }

// Bytes of the per-request transforms of the queries: spectra + norms, or the
// lag form's planes + norms.
// Bytes of one (plain or A-frame) spectra array of `rows` event rows.
size_t spectra_rows_bytes(const seismic_server *s, size_t rows) {
  return round256(rows * (size_t)(s->bp.nb ? s->bp.nb : 1) * (s->PT / 2) * (s->stype ? 4 : 8));
}

size_t query_prep_bytes(const seismic_server *s, int nq) {
  const size_t rows = (size_t)nq * s->C;
  if (s->lag_form) return round256(lag_workspace_bytes(nq, s->C, s->L, lag_planes(s->lag_form)));
  return spectra_rows_bytes(s, rows) + norms_buffer_bytes((long long)rows);
}

// Kernel (a) of `n` events into `spectra` (plain) or, with a plan, into the A
// frames (`spectra`) and / or the W frames (`spectra_w`).
cudaError_t server_spectra(const seismic_server *s, const float *events, long long n, void *spectra,
                           void *spectra_w, double *norms, cudaStream_t st) {
  SpectraArgs sa{};
  sa.events = events;
  sa.n_events = n;
  sa.n_channels = s->C;
  sa.length = s->L;
  sa.ev_stride = (long long)s->C * s->L;
  sa.ch_stride = s->L;
  sa.prescale = s->prescale;
  sa.stype = s->stype;
  sa.spectra = spectra;
  sa.spectra_w = spectra_w;
  sa.norms = norms;
  sa.inv_norms = inverse_norms_of(norms, n * s->C);
  sa.twiddles = s->tw;
  if (!s->bp.nb) return launch_spectra(s->P, sa, st);
  sa.blocks = s->bp.nb;
  sa.block_len = s->bp.B;
  sa.block_shift = s->shift;
  return launch_block_spectra(s->PT, sa, st);
}

size_t request_bytes(const seismic_server *s, int nq, long long ncols) {
  const size_t rows = (size_t)nq * s->C;
  size_t b = round256(rows * s->L * sizeof(float));                             // query events
  b += query_prep_bytes(s, nq);                                                 // query spectra / planes
  b += 4 * round256((size_t)nq * ncols * 4);                                    // outputs
  b += round256((size_t)nq * s->topk * 4) + round256((size_t)nq * s->topk * 8);  // top-K
  return b;
}

bool pool_alloc(seismic_server *s, size_t bytes, size_t *off) {
  for (auto it = s->free_list.begin(); it != s->free_list.end(); ++it) {
    if (it->second >= bytes) {
      *off = it->first;
      const size_t rest = it->second - bytes;
      const size_t rest_off = it->first + bytes;
      s->free_list.erase(it);
      if (rest) s->free_list[rest_off] = rest;
      return true;
    }
  }
  return false;
}

void pool_free(seismic_server *s, size_t off, size_t bytes) {
  auto it = s->free_list.emplace(off, bytes).first;
  auto nx = std::next(it);
  if (nx != s->free_list.end() && it->first + it->second == nx->first) {  // merge right
    it->second += nx->second;
    s->free_list.erase(nx);
  }
  if (it != s->free_list.begin()) {  // merge left
    auto pv = std::prev(it);
    if (pv->first + pv->second == it->first) {
      pv->second += it->second;
      s->free_list.erase(it);
    }
  }
}

void CUDART_CB on_complete(void *p) {
  Request *r = static_cast<Request *>(p);
  seismic_server *s = r->server;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    r->finished = Clock::now();
    r->done = true;
    s->slot_busy[r->slot] = false;
    pool_free(s, r->pool_off, r->bytes);
    s->completed += 1;
    s->pairs_done += (long long)r->n_query * r->n_cols;
  }
  s->cv_done.notify_all();
  s->cv_dispatch.notify_one();
}

// SMs the pair kernels of requests run on.
int pair_sms(const seismic_server *s) {
  const int n = s->sm_count - s->spare_sms;
  return n > 0 ? n : 1;
}

// Enqueue the whole pipeline of `r` on its slot's stream (dispatcher thread).
int launch_request(seismic_server *s, Request *r) {
  cudaStream_t st = s->streams[r->slot];
  const int nq = r->n_query;
  const size_t rows = (size_t)nq * s->C;
  char *base = s->pool + r->pool_off;
  float *q_ev = reinterpret_cast<float *>(base);
  base += round256(rows * s->L * sizeof(float));
  void *q_spec = base;  // spectra, or the lag form's planes
  double *q_norm = reinterpret_cast<double *>(base + (s->lag_form ? 0 : spectra_rows_bytes(s, rows)));
  base += query_prep_bytes(s, nq);
  const size_t ob = round256((size_t)nq * r->n_cols * 4);
  float *d_vp = reinterpret_cast<float *>(base);
  int *d_lp = reinterpret_cast<int *>(base + ob);
  float *d_vn = reinterpret_cast<float *>(base + 2 * ob);
  int *d_ln = reinterpret_cast<int *>(base + 3 * ob);
  base += 4 * ob;
  float *d_tv = reinterpret_cast<float *>(base);
  long long *d_ti = reinterpret_cast<long long *>(base + round256((size_t)nq * s->topk * 4));

  // queries of the catalog's length in one copy; shorter ones zero-padded
  // to it (a pitched copy of query_length samples per row)
  cudaError_t e;
  if (r->query_length == s->L) {
    e = cudaMemcpyAsync(q_ev, r->query, rows * s->L * sizeof(float), cudaMemcpyHostToDevice, st);
  } else {
    e = cudaMemsetAsync(q_ev, 0, rows * s->L * sizeof(float), st);
    if (e == cudaSuccess)
      e = cudaMemcpy2DAsync(q_ev, (size_t)s->L * sizeof(float), r->query, (size_t)r->query_length * sizeof(float),
                            (size_t)r->query_length * sizeof(float), rows, cudaMemcpyHostToDevice, st);
  }
  if (s->lag_form) {  // time-domain lag sums on the tensor cores
    if (e == cudaSuccess)
      e = lag_prepare(q_ev, nq, s->C, s->L, (long long)s->C * s->L, s->L, s->lag_form, q_spec, st);
    if (e == cudaSuccess && s->last_pair) e = cudaStreamWaitEvent(st, s->last_pair, 0);
    if (e == cudaSuccess)
      e = launch_lag_rect(s->cat_lag, s->n_cat, q_spec, nq, s->C, s->L, s->shift, r->col_begin, r->n_cols,
                          s->threshold, s->lag_form, d_vp, d_lp, d_vn, d_ln, s->error_flag, pair_sms(s), st);
    note_launches(2);
  } else {
  // the queries' spectra (the A frames with an overlap-save plan)
  if (e == cudaSuccess) e = server_spectra(s, q_ev, nq, q_spec, nullptr, q_norm, st);
  PairArgs pa{};
  pa.rect = 1;
  pa.spectra = s->cat_spectra;
  pa.norms = s->cat_norms;
  pa.inv_norms = inverse_norms_of(s->cat_norms, s->n_cat * s->C);
  pa.spectra_q = q_spec;
  pa.norms_q = q_norm;
  pa.inv_norms_q = inverse_norms_of(q_norm, (long long)rows);
  pa.stype = s->stype;
  pa.n_query = nq;
  pa.col_begin = r->col_begin;
  pa.n_cols = r->n_cols;
  pa.n_events = s->n_cat;
  pa.n_channels = s->C;
  pa.shift = s->shift;
  pa.prescaled = s->prescale;
  pa.threshold = s->threshold;
  pa.vals_pos = d_vp;
  pa.lags_pos = d_lp;
  pa.vals_neg = d_vn;
  pa.lags_neg = d_ln;
  pa.tile = 8;
  pa.twiddles = s->tw;
  pa.error_flag = s->error_flag;
  pa.couple_begin = 0;
  pa.spec_channels = s->bp.nb ? s->C * s->bp.nb : 0;  // catalog W frames (j), query A frames (i)
  pa.couple_end = pair_work_total(s->PT, pa);
  if (e == cudaSuccess && s->last_pair) e = cudaStreamWaitEvent(st, s->last_pair, 0);
  if (e == cudaSuccess) e = launch_pair_work(s->PT, pa, pair_sms(s), 0, st);
  }
  if (e == cudaSuccess) e = cudaEventRecord(s->pair_done[r->slot], st);
  if (e == cudaSuccess) s->last_pair = s->pair_done[r->slot];
  if (e == cudaSuccess && s->topk > 0) {
    topk_kernel<<<nq, kTopKThreads, 0, st>>>(d_vp, r->n_cols, s->topk, r->col_begin, d_tv, d_ti);
    e = cudaGetLastError();
  }
  const size_t nbytes = (size_t)nq * r->n_cols * 4;
  if (e == cudaSuccess && r->vp) e = cudaMemcpyAsync(r->vp, d_vp, nbytes, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && r->lp) e = cudaMemcpyAsync(r->lp, d_lp, nbytes, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && r->vn) e = cudaMemcpyAsync(r->vn, d_vn, nbytes, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && r->ln) e = cudaMemcpyAsync(r->ln, d_ln, nbytes, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && r->topk_v && s->topk > 0)
    e = cudaMemcpyAsync(r->topk_v, d_tv, (size_t)nq * s->topk * 4, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && r->topk_i && s->topk > 0)
    e = cudaMemcpyAsync(r->topk_i, d_ti, (size_t)nq * s->topk * 8, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaLaunchHostFunc(st, on_complete, r);
  note_launches(s->topk > 0 ? 3 : 2);
  return e == cudaSuccess ? SEISMIC_OK : SEISMIC_ERR_CUDA;
}

void dispatcher_main(seismic_server *s, int device) {
  cudaSetDevice(device);
  std::unique_lock<std::mutex> lk(s->mu);
  std::vector<Request *> admitted;
  while (!s->stopping) {
    // admit in arrival order; a request that does not fit lets later ones try
    admitted.clear();
    for (auto it = s->pending.begin(); it != s->pending.end();) {
      int slot = -1, busy = 0;
      for (size_t k = 0; k < s->slot_busy.size(); ++k) {
        if (s->slot_busy[k])
          ++busy;
        else if (slot < 0)
          slot = (int)k;
      }
      if (slot < 0) break;
      if (busy > 0 && (long long)s->pending.size() < s->overlap_backlog) break;  // wait for the device
      Request *r = *it;
      size_t off = 0;
      if (!pool_alloc(s, r->bytes, &off)) {
        ++it;
        continue;
      }
      r->pool_off = off;
      r->slot = slot;
      s->slot_busy[slot] = true;
      it = s->pending.erase(it);
      admitted.push_back(r);
    }
    if (admitted.empty()) {
      s->cv_dispatch.wait_for(lk, std::chrono::milliseconds(50));
      continue;
    }
    // enqueue outside the lock: completion callbacks of other requests take it
    lk.unlock();
    for (Request *r : admitted) {
      const int st = launch_request(s, r);
      if (st != SEISMIC_OK) {  // nothing will call back: finish it here
        std::lock_guard<std::mutex> g(s->mu);
        r->status = st;
        r->finished = Clock::now();
        r->done = true;
        s->slot_busy[r->slot] = false;
        pool_free(s, r->pool_off, r->bytes);
        s->cv_done.notify_all();
      }
    }
    lk.lock();
  }
}

}  // namespace

extern "C" int seismic_server_create(const float *catalog, long long n_catalog, int n_channels, int event_length,
                                     int shift, float threshold, int form, int n_slots, size_t hbm_budget_bytes,
                                     int max_query_events, int topk, seismic_server **out) {
  report_status(SEISMIC_OK, "");
  if (!out) return report_status(SEISMIC_ERR_INVALID_ARGUMENT, "null output handle");
  *out = nullptr;
  const bool lag = form == SEISMIC_FORM_LAGGEMM_BF16X3 || form == SEISMIC_FORM_LAGGEMM_FP16;
  if (form != SEISMIC_FORM_FP32 && form != SEISMIC_FORM_FP16_SPECTRA && !lag)
    return report_status(SEISMIC_ERR_INVALID_ARGUMENT, "server forms: FP32 or FP16 spectra, or a lag-GEMM form");
  const int P = seismic_resolve_padded_size(event_length, shift);
  int s0 = check_xcorr_args(n_catalog, n_channels, event_length, P, shift, 0, lag ? form : SEISMIC_FORM_FP32);
  if (s0) return s0;
  if (!catalog) return report_status(SEISMIC_ERR_INVALID_ARGUMENT, "null catalog");
  if (n_slots < 1 || n_slots > 64 || max_query_events < 1 || topk < 0 || topk > kTopKMax)
    return report_status(SEISMIC_ERR_INVALID_ARGUMENT, "bad slot / query / top-K limits");
  int sm = 0;
  const float2 *tw = nullptr;
  int *ef = nullptr;
  if ((s0 = device_context(&sm, &tw, &ef))) return s0;

  seismic_server *s = new seismic_server();
  s->n_cat = n_catalog;
  s->C = n_channels;
  s->L = event_length;
  s->P = P;
  s->shift = shift;
  s->threshold = threshold;
  s->stype = form == SEISMIC_FORM_FP16_SPECTRA ? 1 : 0;
  s->lag_form = lag ? form : 0;
  s->prescale = (n_channels > 1 || s->stype) ? 1 : 0;
  if (!lag) s->bp = block_plan(event_length, shift, P, n_channels, s->stype);
  s->PT = s->bp.nb ? s->bp.Q : P;
  s->topk = topk;
  s->sm_count = sm;
  s->tw = tw;
  s->error_flag = ef;
  s->max_query = max_query_events;
  if (const char *env = getenv("SEISMIC_SERVER_OVERLAP_BACKLOG")) {
    const int v = atoi(env);
    if (v >= 1) s->overlap_backlog = v;
  }
  if (const char *env = getenv("SEISMIC_SERVER_SPARE_SMS")) {
    const int v = atoi(env);
    if (v >= 0 && v < sm) s->spare_sms = v;
  }
  const long long rows = n_catalog * n_channels;
  float *d_cat = nullptr;
  cudaError_t e = cudaSuccess;
  if (lag) {
    e = cudaMalloc(&s->cat_lag, lag_workspace_bytes(n_catalog, n_channels, event_length, lag_planes(form)));
  } else {
    e = cudaMalloc(&s->cat_spectra, spectra_rows_bytes(s, (size_t)rows));
    if (e == cudaSuccess) e = cudaMalloc(&s->cat_norms, norms_buffer_bytes(rows));
  }
  if (e == cudaSuccess) e = cudaMalloc(&d_cat, (size_t)rows * event_length * sizeof(float));
  if (e == cudaSuccess)
    e = cudaMemcpy(d_cat, catalog, (size_t)rows * event_length * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && lag) {
    e = lag_prepare(d_cat, n_catalog, n_channels, event_length, (long long)n_channels * event_length,
                    event_length, form, s->cat_lag, nullptr);
    note_launches(1);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
  } else if (e == cudaSuccess) {
    // the catalog's spectra (the W frames with an overlap-save plan)
    e = s->bp.nb ? server_spectra(s, d_cat, n_catalog, nullptr, s->cat_spectra, s->cat_norms, nullptr)
                 : server_spectra(s, d_cat, n_catalog, s->cat_spectra, nullptr, s->cat_norms, nullptr);
    note_launches(1);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
  }
  cudaFree(d_cat);  // only the spectra and norms stay resident
  // the pool: the HBM budget for in-flight requests (default: room for n_slots
  // requests of max_query_events events against the whole catalog)
  // (a request that needs more than the whole budget is refused at submit)
  const size_t per_req = request_bytes(s, max_query_events, n_catalog);
  s->pool_bytes = hbm_budget_bytes ? round256(hbm_budget_bytes) : per_req * (size_t)n_slots;
  if (e == cudaSuccess) e = cudaMalloc(&s->pool, s->pool_bytes);
  if (e != cudaSuccess) {
    cudaFree(s->cat_spectra);
    cudaFree(s->cat_norms);
    cudaFree(s->cat_lag);
    cudaFree(s->pool);
    delete s;
    return report_cuda(e, "server set-up");
  }
  s->free_list[0] = s->pool_bytes;
  s->streams.resize(n_slots);
  s->pair_done.resize(n_slots);
  s->slot_busy.assign(n_slots, false);
  for (auto &st : s->streams) cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  for (auto &ev : s->pair_done) cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
  // make sure the pair kernel's attributes are set before concurrent use
  pair_ctas_per_sm(P);
  int dev = 0;
  cudaGetDevice(&dev);
  s->dispatcher = std::thread(dispatcher_main, s, dev);
  *out = s;
  return SEISMIC_OK;
}

extern "C" int seismic_server_submit(seismic_server *s, const float *query, int n_query, long long subset_begin,
                                     long long subset_end, float *vals_pos, int *lags_pos, float *vals_neg,
                                     int *lags_neg, float *topk_vals, long long *topk_index, long long *ticket) {
  if (!s) return report_status(SEISMIC_ERR_INVALID_ARGUMENT, "null server");
  return seismic_server_submit_len(s, query, n_query, s->L, subset_begin, subset_end, vals_pos, lags_pos, vals_neg,
                                   lags_neg, topk_vals, topk_index, ticket);
}

extern "C" int seismic_server_submit_len(seismic_server *s, const float *query, int n_query, int query_length,
                                         long long subset_begin, long long subset_end, float *vals_pos,
                                         int *lags_pos, float *vals_neg, int *lags_neg, float *topk_vals,
                                         long long *topk_index, long long *ticket) {
  report_status(SEISMIC_OK, "");
  if (!s || !query || !ticket) return report_status(SEISMIC_ERR_INVALID_ARGUMENT, "null argument");
  if (n_query < 1 || n_query > s->max_query)
    return report_status(SEISMIC_ERR_INVALID_ARGUMENT, "query size outside 1..max_query_events");
  if (query_length < 1 || query_length > s->L)
    return report_status(SEISMIC_ERR_INVALID_ARGUMENT, "query length outside 1..the catalog's event_length");
  if (subset_begin < 0 || subset_end > s->n_cat || subset_end <= subset_begin)
    return report_status(SEISMIC_ERR_INVALID_ARGUMENT, "catalog subset out of range");
  Request *r = new Request();
  r->query = query;
  r->n_query = n_query;
  r->query_length = query_length;
  r->col_begin = subset_begin;
  r->n_cols = subset_end - subset_begin;
  r->vp = vals_pos;
  r->lp = lags_pos;
  r->vn = vals_neg;
  r->ln = lags_neg;
  r->topk_v = topk_vals;
  r->topk_i = topk_index;
  r->server = s;
  r->bytes = request_bytes(s, n_query, r->n_cols);
  if (r->bytes > s->pool_bytes) {
    delete r;
    return report_status(SEISMIC_ERR_OUT_OF_MEMORY, "request larger than the server's HBM budget");
  }
  r->submitted = Clock::now();
  {
    std::lock_guard<std::mutex> lk(s->mu);
    r->ticket = s->next_ticket++;
    s->by_ticket[r->ticket] = r;
    s->pending.push_back(r);
  }
  s->cv_dispatch.notify_one();
  *ticket = r->ticket;
  return SEISMIC_OK;
}

extern "C" int seismic_server_wait(seismic_server *s, long long ticket, double *latency_ms) {
  report_status(SEISMIC_OK, "");
  if (!s) return report_status(SEISMIC_ERR_INVALID_ARGUMENT, "null server");
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->by_ticket.find(ticket);
  if (it == s->by_ticket.end()) return report_status(SEISMIC_ERR_INVALID_ARGUMENT, "unknown ticket");
  Request *r = it->second;
  s->cv_done.wait(lk, [&] { return r->done; });
  const int st = r->status;
  if (latency_ms) latency_ms[0] = std::chrono::duration<double, std::milli>(r->finished - r->submitted).count();
  s->by_ticket.erase(it);
  delete r;
  if (st != SEISMIC_OK) return report_status(st, "request failed on the device");
  return SEISMIC_OK;
}

extern "C" int seismic_server_stats(seismic_server *s, long long *completed, long long *pairs, int *in_flight,
                                    int *pending) {
  if (!s) return report_status(SEISMIC_ERR_INVALID_ARGUMENT, "null server");
  std::lock_guard<std::mutex> lk(s->mu);
  if (completed) *completed = s->completed;
  if (pairs) *pairs = s->pairs_done;
  int busy = 0;
  for (bool b : s->slot_busy) busy += b ? 1 : 0;
  if (in_flight) *in_flight = busy;
  if (pending) *pending = (int)s->pending.size();
  return SEISMIC_OK;
}

extern "C" int seismic_server_destroy(seismic_server *s) {
  report_status(SEISMIC_OK, "");
  if (!s) return SEISMIC_OK;
  {
    std::unique_lock<std::mutex> lk(s->mu);
    // let admitted and pending work finish
    s->cv_done.wait(lk, [&] {
      bool busy = false;
      for (bool b : s->slot_busy) busy |= b;
      return !busy && s->pending.empty();
    });
    s->stopping = true;
  }
  s->cv_dispatch.notify_all();
  if (s->dispatcher.joinable()) s->dispatcher.join();
  for (auto &st : s->streams) cudaStreamDestroy(st);
  for (auto &ev : s->pair_done) cudaEventDestroy(ev);
  for (auto &kv : s->by_ticket) delete kv.second;
  cudaFree(s->cat_spectra);
  cudaFree(s->cat_norms);
  cudaFree(s->cat_lag);
  cudaFree(s->pool);
  delete s;
  return SEISMIC_OK;
}
