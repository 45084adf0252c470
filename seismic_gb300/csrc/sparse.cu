// Consumers of the packed outputs: on-device compaction of the pairs above a
// threshold (the reference's sparse output), and a standalone histogram of
// stored coefficients.
//
// The reference thresholds inside the pair loop and then stores each packed
// array as a 1 x N(N+1)/2 CSR matrix of its nonzeros
// (Correlation_in_OMP/test_c.py:43-55, scipy csr_matrix + save_npz).  Here the
// pair kernel can run once with threshold 0; seismic_histogram_device bins the
// stored coefficients with the pair kernel's rule (Correlation_in_OMP/
// correlation_c.cpp:116-117, :128-129) so a threshold can be chosen, and
// seismic_compact_pairs_device keeps, in packed order, the pairs whose
// coefficient passes it (vals_pos > thr, vals_neg < -thr) -- the entries the
// reference's CSR matrices hold after a run with that threshold -- so only
// those cross PCIe.
//
// Compaction is two passes over blocks of kCompactBlock pairs: count per
// block, one exclusive scan of the block counts, then a write pass that ranks
// each kept pair inside its block with warp ballots.  Output order is the
// packed order; every pass is HBM-bound (algorithmic bytes: 8 B per pair read
// twice for the values, plus the kept pairs' lags and outputs).
#include <cstdint>

#include "../../include/seismic_gb300.h"
#include "kernels.cuh"

namespace seismic {

int report_status(int status, const char *message);
int report_cuda(cudaError_t e, const char *what);
void note_launches(unsigned n);

constexpr int kCompactThreads = 256;
constexpr int kCompactPerThread = 16;
constexpr int kCompactBlock = kCompactThreads * kCompactPerThread;  // pairs per block
constexpr int kHistSmemMax = 4096;

__device__ __forceinline__ int sparse_hist_bin(float v, float delta, int n_hist) {
  if (v >= 1.0f) return n_hist - 1;
  int b = (int)(v / delta);
  return b > n_hist - 1 ? n_hist - 1 : (b < 0 ? 0 : b);
}

__global__ void __launch_bounds__(kCompactThreads) compact_count_kernel(const float *__restrict__ vp,
                                                                          const float *__restrict__ vn,
                                                                          long long n, float thr, long long nb,
                                                                          long long *__restrict__ counts) {
  for (long long b = blockIdx.x; b < nb; b += gridDim.x) {
    int cp = 0, cn = 0;
#pragma unroll 4
    for (int k = 0; k < kCompactPerThread; ++k) {
      const long long e = b * kCompactBlock + k * kCompactThreads + threadIdx.x;
      if (e < n) {
        cp += __ldg(vp + e) > thr;
        cn += __ldg(vn + e) < -thr;
      }
    }
    const int sp = __reduce_add_sync(0xffffffffu, (unsigned)cp);
    const int sn = __reduce_add_sync(0xffffffffu, (unsigned)cn);
    __shared__ int s_p[kCompactThreads / 32], s_n[kCompactThreads / 32];
    if ((threadIdx.x & 31) == 0) {
      s_p[threadIdx.x >> 5] = sp;
      s_n[threadIdx.x >> 5] = sn;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      long long tp = 0, tn = 0;
      for (int w = 0; w < kCompactThreads / 32; ++w) {
        tp += s_p[w];
        tn += s_n[w];
      }
      counts[b] = tp;
      counts[nb + b] = tn;
    }
    __syncthreads();
  }
}

// Exclusive scan of the 2 nb block counts in place (one CTA); totals to out[0..1].
__global__ void __launch_bounds__(1024) compact_scan_kernel(long long *__restrict__ counts, long long nb,
                                                            long long *__restrict__ totals) {
  __shared__ long long s[1024];
  for (int side = 0; side < 2; ++side) {
    long long *c = counts + side * nb;
    const long long per = (nb + blockDim.x - 1) / blockDim.x;
    const long long b0 = threadIdx.x * per, b1 = b0 + per < nb ? b0 + per : nb;
    long long local = 0;
    for (long long b = b0; b < b1; ++b) local += c[b];
    s[threadIdx.x] = local;
    __syncthreads();
    for (int off = 1; off < (int)blockDim.x; off <<= 1) {  // inclusive Hillis-Steele scan
      const long long add = threadIdx.x >= (unsigned)off ? s[threadIdx.x - off] : 0;
      __syncthreads();
      s[threadIdx.x] += add;
      __syncthreads();
    }
    long long run = s[threadIdx.x] - local;  // exclusive prefix of this thread's segment
    for (long long b = b0; b < b1; ++b) {
      const long long v = c[b];
      c[b] = run;
      run += v;
    }
    if (threadIdx.x == blockDim.x - 1) totals[side] = s[threadIdx.x];
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kCompactThreads) compact_write_kernel(
    const float *__restrict__ vp, const int *__restrict__ lp, const float *__restrict__ vn,
    const int *__restrict__ ln, long long n, float thr, long long nb, const long long *__restrict__ offsets,
    long long capacity, long long *__restrict__ idx_p, float *__restrict__ val_p, int *__restrict__ lag_p,
    long long *__restrict__ idx_n, float *__restrict__ val_n, int *__restrict__ lag_n) {
  __shared__ int s_p[kCompactThreads / 32], s_n[kCompactThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned below = (1u << lane) - 1u;
  for (long long b = blockIdx.x; b < nb; b += gridDim.x) {
    long long op = offsets[b], on = offsets[nb + b];
    for (int k = 0; k < kCompactPerThread; ++k) {
      const long long e = b * kCompactBlock + k * kCompactThreads + threadIdx.x;
      float a = 0.f, c = 0.f;
      if (e < n) {
        a = __ldg(vp + e);
        c = __ldg(vn + e);
      }
      const bool kp = e < n && a > thr, kn = e < n && c < -thr;
      const unsigned bp = __ballot_sync(0xffffffffu, kp), bn = __ballot_sync(0xffffffffu, kn);
      if (lane == 0) {
        s_p[warp] = __popc(bp);
        s_n[warp] = __popc(bn);
      }
      __syncthreads();
      int wp = 0, wn = 0, tp = 0, tn = 0;
#pragma unroll
      for (int w = 0; w < kCompactThreads / 32; ++w) {
        if (w < warp) {
          wp += s_p[w];
          wn += s_n[w];
        }
        tp += s_p[w];
        tn += s_n[w];
      }
      if (kp) {
        const long long o = op + wp + __popc(bp & below);
        if (o < capacity) {
          idx_p[o] = e;
          val_p[o] = a;
          lag_p[o] = __ldg(lp + e);
        }
      }
      if (kn) {
        const long long o = on + wn + __popc(bn & below);
        if (o < capacity) {
          idx_n[o] = e;
          val_n[o] = c;
          lag_n[o] = __ldg(ln + e);
        }
      }
      op += tp;
      on += tn;
      __syncthreads();  // s_p / s_n are reused by the next k
    }
  }
}

__global__ void __launch_bounds__(256) histogram_kernel(const float *__restrict__ vp, const float *__restrict__ vn,
                                                         long long n, int n_hist, float delta, int *hmax,
                                                         int *hmin) {
  extern __shared__ int s_hist[];
  const bool smem = n_hist <= kHistSmemMax;
  if (smem)
    for (int h = threadIdx.x; h < 2 * n_hist; h += blockDim.x) s_hist[h] = 0;
  __syncthreads();
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const int hp = sparse_hist_bin(__ldg(vp + e), delta, n_hist);
    const int hn = sparse_hist_bin(-__ldg(vn + e), delta, n_hist);
    if (smem) {
      atomicAdd(&s_hist[hp], 1);
      atomicAdd(&s_hist[n_hist + hn], 1);
    } else {
      atomicAdd(&hmax[hp], 1);
      atomicAdd(&hmin[hn], 1);
    }
  }
  __syncthreads();
  if (smem) {
    for (int h = threadIdx.x; h < n_hist; h += blockDim.x) {
      if (s_hist[h]) atomicAdd(&hmax[h], s_hist[h]);
      if (s_hist[n_hist + h]) atomicAdd(&hmin[h], s_hist[n_hist + h]);
    }
  }
}

}  // namespace seismic

using namespace seismic;

extern "C" {

size_t seismic_compact_workspace_bytes(long long n_pairs) {
  if (n_pairs < 0) return 0;
  const long long nb = (n_pairs + kCompactBlock - 1) / kCompactBlock;
  return (size_t)(2 * nb + 2) * sizeof(long long);
}

int seismic_compact_pairs_device(const float *d_vals_pos, const int *d_lags_pos, const float *d_vals_neg,
                                 const int *d_lags_neg, long long n_pairs, float threshold, long long capacity,
                                 long long *d_index_pos, float *d_value_pos, int *d_lag_pos,
                                 long long *d_index_neg, float *d_value_neg, int *d_lag_neg,
                                 long long *d_counts, void *workspace, size_t workspace_bytes, void *stream) {
  report_status(SEISMIC_OK, "");
  if (n_pairs < 0 || capacity < 0 || !(threshold >= 0.f))
    return report_status(SEISMIC_ERR_INVALID_ARGUMENT, "n_pairs, capacity and threshold must be >= 0");
  if (!d_vals_pos || !d_lags_pos || !d_vals_neg || !d_lags_neg || !d_counts || !workspace)
    return report_status(SEISMIC_ERR_INVALID_ARGUMENT, "null buffer");
  if (capacity > 0 && (!d_index_pos || !d_value_pos || !d_lag_pos || !d_index_neg || !d_value_neg || !d_lag_neg))
    return report_status(SEISMIC_ERR_INVALID_ARGUMENT, "null output buffer with capacity > 0");
  if (workspace_bytes < seismic_compact_workspace_bytes(n_pairs))
    return report_status(SEISMIC_ERR_WORKSPACE_TOO_SMALL, "compaction workspace too small");
  int sm = 0;
  const float2 *tw;
  int *ef;
  int s = device_context(&sm, &tw, &ef);
  if (s) return s;
  cudaStream_t st = (cudaStream_t)stream;
  const long long nb = (n_pairs + kCompactBlock - 1) / kCompactBlock;
  long long *counts = static_cast<long long *>(workspace);
  if (nb == 0) {
    cudaError_t e = cudaMemsetAsync(d_counts, 0, 2 * sizeof(long long), st);
    return e == cudaSuccess ? SEISMIC_OK : report_cuda(e, "compaction count clear");
  }
  const int grid = (int)(nb < (long long)sm * 8 ? nb : (long long)sm * 8);
  compact_count_kernel<<<grid, kCompactThreads, 0, st>>>(d_vals_pos, d_vals_neg, n_pairs, threshold, nb, counts);
  compact_scan_kernel<<<1, 1024, 0, st>>>(counts, nb, d_counts);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess && capacity > 0) {
    compact_write_kernel<<<grid, kCompactThreads, 0, st>>>(d_vals_pos, d_lags_pos, d_vals_neg, d_lags_neg, n_pairs,
                                                           threshold, nb, counts, capacity, d_index_pos,
                                                           d_value_pos, d_lag_pos, d_index_neg, d_value_neg,
                                                           d_lag_neg);
    e = cudaGetLastError();
    note_launches(1);
  }
  if (e != cudaSuccess) return report_cuda(e, "compaction launch");
  note_launches(2);
  return SEISMIC_OK;
}

int seismic_histogram_device(const float *d_vals_pos, const float *d_vals_neg, long long n_pairs,
                             int n_classes_hist, int *d_max_hist, int *d_min_hist, void *stream) {
  report_status(SEISMIC_OK, "");
  if (n_pairs < 0 || n_classes_hist < 1)
    return report_status(SEISMIC_ERR_INVALID_ARGUMENT, "n_pairs must be >= 0 and n_classes_hist >= 1");
  if (!d_vals_pos || !d_vals_neg || !d_max_hist || !d_min_hist)
    return report_status(SEISMIC_ERR_INVALID_ARGUMENT, "null buffer");
  if (n_pairs == 0) return SEISMIC_OK;
  int sm = 0;
  const float2 *tw;
  int *ef;
  int s = device_context(&sm, &tw, &ef);
  if (s) return s;
  const long long want = (n_pairs + 255) / 256;
  const int grid = (int)(want < (long long)sm * 8 ? want : (long long)sm * 8);
  const size_t smem = n_classes_hist <= kHistSmemMax ? (size_t)2 * n_classes_hist * sizeof(int) : 0;
  histogram_kernel<<<grid, 256, smem, (cudaStream_t)stream>>>(d_vals_pos, d_vals_neg, n_pairs, n_classes_hist,
                                                             (float)(1.0 / n_classes_hist), d_max_hist, d_min_hist);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return report_cuda(e, "histogram launch");
  note_launches(1);
  return SEISMIC_OK;
}

}  // extern "C"
