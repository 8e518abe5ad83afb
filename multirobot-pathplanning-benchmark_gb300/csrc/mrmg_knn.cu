// mrmg_knn.cu -- per-mode k nearest neighbours under the reference's metrics
// (PRM get_neighbors, planners/prm/prm_graph.py:389-549: batch_config_dist of
// one query against the mode's node array, then argpartition + argsort;
// RRT nearest / near, planners/rrtstar_base.py:1228-1337).
//
// Exact path (any metric): warp per query, FP64 distances with the reference's
// operation order, per-lane top-k lists, warp merge by (distance, index).
//
// Tensor-core path (euclidean with D <= 29, max_euclidean with <= 4 agents of
// <= 7 coordinates): the squared distances |q|^2 + |x|^2 - 2 q.x come from a
// tcgen05 GEMM on split-BF16 operands (x = x_hi + x_lo, products
// q_hi.x_hi + q_hi.x_lo + q_lo.x_hi, the |x|^2 term folded into the K
// dimension), accumulated in FP32 in tensor memory; the epilogue keeps each
// query's 16 smallest values per node chunk.  A merge kernel certifies that
// every true k-nearest node is among the kept candidates (a node whose
// approximate value exceeds the k-th approximate value plus twice the error
// bound cannot be in the true top k) and re-ranks them with the exact FP64
// distances; an uncertified query is rerun on the exact path.
#include <algorithm>
#include <cstring>
#include <vector>

#include <cuda_bf16.h>

#include "mrmg_bulk.cuh"
#include "mrmg_internal.cuh"

namespace mrmg {

constexpr int kKnnMaxK = 64;
constexpr int kKeep = 16;          // candidates kept per query per node chunk
constexpr int kTileM = 128;        // queries per tile (TMEM lanes)
constexpr int kRowBytes = 128;     // one SW128 row: 64 bf16
constexpr int kStagesB = 3;        // node-tile buffers in flight per candidate CTA

// ---------------------------------------------------------------------------
// Exact FP64 k-NN: warp per query
// ---------------------------------------------------------------------------
namespace {

// Distances are >= 0 (or +inf), so their IEEE bit patterns order like the
// values: lists compare int64 keys on the integer pipe instead of FP64
// comparisons (GB300 runs FP64 at a small fraction of its FP32/INT rate).
__device__ __forceinline__ long long dkey(double d) { return __double_as_longlong(d); }

template <int KM>
__device__ __forceinline__ void topk_insert(long long (&td)[KM], long long (&ti)[KM], int k, long long d, long long id) {
  // lists hold (distance key, index) ascending; equal distances keep the lower index
  if (!(d < td[k - 1])) return;
#pragma unroll
  for (int i = KM - 1; i > 0; i--) {
    if (i < k) {
      if (d < td[i - 1]) { td[i] = td[i - 1]; ti[i] = ti[i - 1]; }
      else if (d < td[i]) { td[i] = d; ti[i] = id; }
    }
  }
  if (d < td[0]) { td[0] = d; ti[0] = id; }
}

// lexicographic warp argmin over (distance key, id); returns the winning lane
__device__ __forceinline__ int warp_argmin(long long d, long long id) {
  int lane = threadIdx.x & 31;
  long long bd = d;
  long long bi = id;
  int bl = lane;
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    const long long od = __shfl_xor_sync(MRMG_FULL, bd, o);
    const long long oi = __shfl_xor_sync(MRMG_FULL, bi, o);
    const int ol = __shfl_xor_sync(MRMG_FULL, bl, o);
    if (od < bd || (od == bd && oi < bi) || (od == bd && oi == bi && ol < bl)) { bd = od; bi = oi; bl = ol; }
  }
  return bl;
}

template <int KM>
__global__ void knn_exact_kernel(const double* __restrict__ qs, long long Q, const int* __restrict__ q_mode,
                                 const long long* __restrict__ q_list, long long n_list,
                                 const double* __restrict__ nodes, const long long* __restrict__ mode_beg,
                                 const long long* __restrict__ mode_end, SliceTab t, int metric, int k,
                                 long long* __restrict__ out_idx, double* __restrict__ out_dist) {
  const int lane = threadIdx.x & 31;
  const long long warp = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const long long nwarps = (long long)gridDim.x * (blockDim.x >> 5);
  const int D = t.D;
  const long long total = q_list ? n_list : Q;
  for (long long w = warp; w < total; w += nwarps) {
    const long long q = q_list ? q_list[w] : w;
    const int m = q_mode[q];
    const long long s = mode_beg[m], e = mode_end[m];
    long long td[KM];
    long long ti[KM];
#pragma unroll
    for (int i = 0; i < KM; i++) { td[i] = 0x7ff0000000000000ll; ti[i] = -1; }
    const double* qq = qs + q * D;
    for (long long x = s + lane; x < e; x += 32) {
      const double* xx = nodes + x * D;
      auto dfun = [&](int j) { return __dsub_rn(qq[j], xx[j]); };
      topk_insert<KM>(td, ti, k, dkey(dist_of(t, metric, dfun)), x - s);
    }
    // merge the 32 sorted lane lists
    int head = 0;
    for (int r = 0; r < k; r++) {
      long long hd = 0x7ff0000000000000ll;
      long long hi = 0x7fffffffffffffffll;
#pragma unroll
      for (int i = 0; i < KM; i++)
        if (i == head && i < k) { hd = td[i]; hi = ti[i]; }
      if (hi < 0) hi = 0x7fffffffffffffffll;
      const int win = warp_argmin(hd, hi);
      const long long wd = __shfl_sync(MRMG_FULL, hd, win);
      const long long wi = __shfl_sync(MRMG_FULL, hi, win);
      if (lane == 0) {
        out_idx[q * k + r] = wi == 0x7fffffffffffffffll ? -1 : wi;
        out_dist[q * k + r] = wi == 0x7fffffffffffffffll ? __longlong_as_double(0x7ff0000000000000ll)
                                                         : __longlong_as_double(wd);
      }
      if (lane == win) head++;
    }
  }
}

// ---------------------------------------------------------------------------
// Radius decision (d <= r' as the reference's FP64 distance decides it) with
// an FP32 pre-test for the euclidean and max-over-agents metrics: the FP32
// sum of squared coordinate differences (per agent, then the maximum) lies
// within 2.4e-6 (|q| + |x|)^2 of the exact squared distance (each FP32
// coordinate difference within 2^-23 (|q_j| + |x_j|) of the exact one, the
// sum of 28 squares within 28 * 2^-24 of its value), so a node more than
// 7.7e-6 (|q| + |x|)^2 (three times that) plus 2^-20 r'^2 (the rounding of
// r'^2 and of these sums) inside or outside r'^2 is decided without FP64;
// the rest, and every other metric, take the FP64 distance.  GB300 issues
// FP64 at a small fraction of its FP32 rate, and a warp instruction costs the
// same with one active lane as with 32, so this keeps the sparse re-checks
// of radius queries off the FP64 pipe.
// ---------------------------------------------------------------------------
struct RadiusTest {
  double rp;     // r' = radius + eps (FP64)
  float lo, hi;  // (r')^2 (1 -+ 2^-20) in FP32
};

__device__ __forceinline__ RadiusTest radius_test(double rp) {
  RadiusTest r;
  r.rp = rp;
  const float r2 = (float)(rp * rp);
  r.lo = r2 * (1.f - 9.5367431640625e-7f);
  r.hi = r2 * (1.f + 9.5367431640625e-7f);
  return r;
}

// q32 / x32: FP32 copies (rounded to nearest) of the FP64 rows qq / xx
__device__ __forceinline__ bool within_radius(const float* __restrict__ q32, const float* __restrict__ x32,
                                              const double* __restrict__ qq, const double* __restrict__ xx,
                                              const SliceTab& t, int metric, const RadiusTest& r) {
  if (!(r.rp >= 0.0)) return false;   // distances are >= 0; NaN selects nothing
  if (metric == MRMG_METRIC_EUCLIDEAN || metric == MRMG_METRIC_MAX_EUCLIDEAN) {
    float qn = 0.f, xn = 0.f, m = 0.f;
    if (metric == MRMG_METRIC_EUCLIDEAN) {
      for (int k = 0; k < t.end_all; k++) {
        const float qf = q32[k], xf = x32[k], d = qf - xf;
        m = fmaf(d, d, m);
        qn = fmaf(qf, qf, qn);
        xn = fmaf(xf, xf, xn);
      }
    } else {
      for (int a = 0; a < t.A; a++) {
        float sa = 0.f;
        for (int k = t.s[a]; k < t.e[a]; k++) {
          const float qf = q32[k], xf = x32[k], d = qf - xf;
          sa = fmaf(d, d, sa);
          qn = fmaf(qf, qf, qn);
          xn = fmaf(xf, xf, xn);
        }
        m = fmaxf(m, sa);
      }
    }
    const float e = sqrtf(qn) + sqrtf(xn);
    const float bnd = 7.7e-6f * e * e;
    if (m < r.lo - bnd) return true;
    if (m > r.hi + bnd) return false;
  }
  auto dfun = [&](int j) { return __dsub_rn(qq[j], xx[j]); };
  return dist_of(t, metric, dfun) <= r.rp;
}

__global__ void f64_to_f32_kernel(const double* __restrict__ src, float* __restrict__ dst, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    dst[i] = (float)src[i];
}

// ---------------------------------------------------------------------------
// Node-parallel exact FP64 paths for small query batches: work items are
// (query, chunk of kSplitNodes nodes) pairs, so one query spreads over the
// whole GPU instead of one warp.
// ---------------------------------------------------------------------------
constexpr int kSplitNodes = 256;

// index q of the range [off[q], off[q + 1]) holding f (off ascending, off[0] = 0 <= f < off[Q])
__device__ __forceinline__ long long owner_of(const long long* __restrict__ off, long long Q, long long f) {
  long long lo = 0, hi = Q;
  while (hi - lo > 1) {
    const long long mid = (lo + hi) >> 1;
    if (off[mid] <= f) lo = mid; else hi = mid;
  }
  return lo;
}

// warp per item: the chunk's k best (distance key, mode-local index), ascending
// (queries are listed entries: query qmap[l] for list entry l, or l itself
// when qmap is NULL; q_mode is per list entry)
template <int KM>
__global__ void knn_split_kernel(const double* __restrict__ qs, const long long* __restrict__ qmap, long long Q,
                                 const int* __restrict__ q_mode, const long long* __restrict__ ioff,
                                 const double* __restrict__ nodes,
                                 const long long* __restrict__ mode_beg, const long long* __restrict__ mode_end,
                                 SliceTab t, int metric, int k, long long* __restrict__ cand_key,
                                 long long* __restrict__ cand_idx) {
  const int lane = threadIdx.x & 31;
  const long long warp = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const long long nwarps = (long long)gridDim.x * (blockDim.x >> 5);
  const long long n_items = ioff[Q];
  for (long long it = warp; it < n_items; it += nwarps) {
    const long long l = owner_of(ioff, Q, it);
    const int m = q_mode[l];
    const long long b = mode_beg[m];
    const long long s = b + (it - ioff[l]) * kSplitNodes;
    const long long e = s + kSplitNodes < mode_end[m] ? s + kSplitNodes : mode_end[m];
    long long td[KM];
    long long ti[KM];
#pragma unroll
    for (int i = 0; i < KM; i++) { td[i] = 0x7ff0000000000000ll; ti[i] = -1; }
    const double* qq = qs + (qmap ? qmap[l] : l) * t.D;
    for (long long x = s + lane; x < e; x += 32) {
      const double* xx = nodes + x * t.D;
      auto dfun = [&](int j) { return __dsub_rn(qq[j], xx[j]); };
      topk_insert<KM>(td, ti, k, dkey(dist_of(t, metric, dfun)), x - b);
    }
    int head = 0;
    for (int r = 0; r < k; r++) {
      long long hd = 0x7ff0000000000000ll;
      long long hi = 0x7fffffffffffffffll;
#pragma unroll
      for (int i = 0; i < KM; i++)
        if (i == head && i < k) { hd = td[i]; hi = ti[i]; }
      if (hi < 0) hi = 0x7fffffffffffffffll;
      const int win = warp_argmin(hd, hi);
      const long long wd = __shfl_sync(MRMG_FULL, hd, win);
      const long long wi = __shfl_sync(MRMG_FULL, hi, win);
      if (lane == 0) {
        cand_key[it * k + r] = wd;
        cand_idx[it * k + r] = wi == 0x7fffffffffffffffll ? -1 : wi;
      }
      if (lane == win) head++;
    }
  }
}

// warp per query: lane l takes the query's items l, l + 32, ... whole and in
// order (each item's list is sorted and later items hold higher indices, so
// equal distances still arrive in index order), then the lanes merge
template <int KM>
__global__ void knn_split_merge_kernel(const long long* __restrict__ qmap, long long Q,
                                       const long long* __restrict__ ioff, int k,
                                       const long long* __restrict__ cand_key, const long long* __restrict__ cand_idx,
                                       long long* __restrict__ out_idx, double* __restrict__ out_dist) {
  const int lane = threadIdx.x & 31;
  const long long warp = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const long long nwarps = (long long)gridDim.x * (blockDim.x >> 5);
  for (long long l = warp; l < Q; l += nwarps) {
    const long long q = qmap ? qmap[l] : l;
    long long td[KM];
    long long ti[KM];
#pragma unroll
    for (int i = 0; i < KM; i++) { td[i] = 0x7ff0000000000000ll; ti[i] = -1; }
    for (long long it = ioff[l] + lane; it < ioff[l + 1]; it += 32)
      for (int r = 0; r < k; r++) {
        const long long id = cand_idx[it * k + r];
        const long long d = cand_key[it * k + r];
        if (id < 0 || !(d < td[k - 1])) break;   // sorted: nothing further enters
        topk_insert<KM>(td, ti, k, d, id);
      }
    int head = 0;
    for (int r = 0; r < k; r++) {
      long long hd = 0x7ff0000000000000ll;
      long long hi = 0x7fffffffffffffffll;
#pragma unroll
      for (int i = 0; i < KM; i++)
        if (i == head && i < k) { hd = td[i]; hi = ti[i]; }
      if (hi < 0) hi = 0x7fffffffffffffffll;
      const int win = warp_argmin(hd, hi);
      const long long wd = __shfl_sync(MRMG_FULL, hd, win);
      const long long wi = __shfl_sync(MRMG_FULL, hi, win);
      if (lane == 0) {
        out_idx[q * k + r] = wi == 0x7fffffffffffffffll ? -1 : wi;
        out_dist[q * k + r] = wi == 0x7fffffffffffffffll ? __longlong_as_double(0x7ff0000000000000ll)
                                                         : __longlong_as_double(wd);
      }
      if (lane == win) head++;
    }
  }
}

// ---------------------------------------------------------------------------
// Node-parallel k-NN with an FP32 candidate pass (euclidean, max over
// agents): per (query, 256-node chunk) item the k smallest FP32 squared
// distances of the FP32 node copy (direct coordinate differences; per agent,
// then the maximum), the item's (k+1)-th smallest value (the first node left
// out) and the band 7.7e-6 (|q| + max |x|)^2 that bounds the FP32 values'
// error (the radius pre-test's bound).  The merge re-ranks in FP64 only the
// candidates within tau = (k-th FP32 value + 2 band)(1 + 2^-20) and
// certifies that every left-out node lies above tau (then its FP64 distance
// exceeds the k-th); a query that fails is rerun on the FP64 kernels.
// ---------------------------------------------------------------------------
constexpr int kSplitWarps = 4;

template <int KM>
__global__ void knn_split32_kernel(const double* __restrict__ qs, const long long* __restrict__ qmap, long long Q,
                                   const int* __restrict__ q_mode, const long long* __restrict__ ioff,
                                   const float* __restrict__ nodes32, const long long* __restrict__ mode_beg,
                                   const long long* __restrict__ mode_end, SliceTab t, int metric, int k,
                                   float* __restrict__ cand_key, int* __restrict__ cand_idx,
                                   float* __restrict__ item_next, float* __restrict__ item_band) {
  __shared__ float s_q[kSplitWarps][64];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const long long warp = (long long)blockIdx.x * kSplitWarps + wib;
  const long long nwarps = (long long)gridDim.x * kSplitWarps;
  const long long n_items = ioff[Q];
  const float INF = __int_as_float(0x7f800000);
  float* q32 = s_q[wib];
  long long cur = -1;
  float qn = 0.f;
  for (long long it = warp; it < n_items; it += nwarps) {
    const long long l = owner_of(ioff, Q, it);
    const long long q = qmap ? qmap[l] : l;
    if (q != cur) {   // the query in FP32 (and |q|^2), once per query in this warp
      __syncwarp();
      for (int j = lane; j < t.D; j += 32) q32[j] = (float)qs[q * t.D + j];
      __syncwarp();
      float a = 0.f;
      for (int j = 0; j < t.D; j++) a = fmaf(q32[j], q32[j], a);
      qn = a;
      cur = q;
    }
    const int m = q_mode[l];
    const long long b = mode_beg[m];
    const long long s = b + (it - ioff[l]) * kSplitNodes;
    const long long e = s + kSplitNodes < mode_end[m] ? s + kSplitNodes : mode_end[m];
    float td[KM];
    int ti[KM];
#pragma unroll
    for (int i = 0; i < KM; i++) { td[i] = INF; ti[i] = 0x7fffffff; }
    float xmax = 0.f;
    for (long long x = s + lane; x < e; x += 32) {
      const float* xx = nodes32 + x * t.D;
      float v = 0.f, xn = 0.f;
      if (metric == MRMG_METRIC_EUCLIDEAN) {
        for (int j = 0; j < t.end_all; j++) {
          const float d = q32[j] - xx[j];
          v = fmaf(d, d, v);
          xn = fmaf(xx[j], xx[j], xn);
        }
      } else {
        for (int a = 0; a < t.A; a++) {
          float sa = 0.f;
          for (int j = t.s[a]; j < t.e[a]; j++) {
            const float d = q32[j] - xx[j];
            sa = fmaf(d, d, sa);
            xn = fmaf(xx[j], xx[j], xn);
          }
          v = fmaxf(v, sa);
        }
      }
      xmax = fmaxf(xmax, xn);
      if (v != v) v = INF;   // NaN coordinates: never a candidate here, the FP64 check decides
      const int id = (int)(x - b);
      if (v < td[KM - 1]) {   // nodes arrive in index order: equal values keep the lower index first
#pragma unroll
        for (int i = KM - 1; i > 0; i--) {
          if (v < td[i - 1]) { td[i] = td[i - 1]; ti[i] = ti[i - 1]; }
          else if (v < td[i]) { td[i] = v; ti[i] = id; }
        }
        if (v < td[0]) { td[0] = v; ti[0] = id; }
      }
    }
    // the item's k smallest (value, index), then the (k+1)-th value
    int head = 0;
    for (int r = 0; r <= k; r++) {
      float hv = INF;
      int hi = 0x7fffffff;
#pragma unroll
      for (int i = 0; i < KM; i++)
        if (i == head) { hv = td[i]; hi = ti[i]; }
      float bv = hv;
      int bi = hi, bl = lane;
#pragma unroll
      for (int o = 16; o; o >>= 1) {
        const float ov = __shfl_xor_sync(MRMG_FULL, bv, o);
        const int oi = __shfl_xor_sync(MRMG_FULL, bi, o);
        const int ol = __shfl_xor_sync(MRMG_FULL, bl, o);
        if (ov < bv || (ov == bv && (oi < bi || (oi == bi && ol < bl)))) { bv = ov; bi = oi; bl = ol; }
      }
      if (r < k) {
        if (lane == 0) {
          cand_key[it * k + r] = bv;
          cand_idx[it * k + r] = bv == INF ? -1 : bi;
        }
        if (lane == bl) head++;
      } else if (lane == 0) {
        item_next[it] = bv;
      }
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) xmax = fmaxf(xmax, __shfl_xor_sync(MRMG_FULL, xmax, o));
    if (lane == 0) {
      const float ee = sqrtf(qn) + sqrtf(xmax);
      item_band[it] = 7.7e-6f * ee * ee;
    }
  }
}

// merge of the FP32 candidates: warp per query
constexpr int kSplitGather = 512;   // candidates within tau re-ranked per query (more: rerun)

template <int KM>
__global__ void knn_split32_merge_kernel(const double* __restrict__ qs, const long long* __restrict__ qmap,
                                         long long Q, const int* __restrict__ q_mode,
                                         const long long* __restrict__ ioff, const double* __restrict__ nodes,
                                         const long long* __restrict__ mode_beg,
                                         const long long* __restrict__ mode_end, SliceTab t, int metric, int k,
                                         const float* __restrict__ cand_key, const int* __restrict__ cand_idx,
                                         const float* __restrict__ item_next, const float* __restrict__ item_band,
                                         long long* __restrict__ out_idx, double* __restrict__ out_dist,
                                         long long* __restrict__ fallback, int* __restrict__ n_fallback) {
  __shared__ int s_id[kSplitWarps][kSplitGather];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const long long warp = (long long)blockIdx.x * kSplitWarps + wib;
  const long long nwarps = (long long)gridDim.x * kSplitWarps;
  const float INF = __int_as_float(0x7f800000);
  int* sid = s_id[wib];
  for (long long l = warp; l < Q; l += nwarps) {
    const long long q = qmap ? qmap[l] : l;
    const int m = q_mode[l];
    const long long M = mode_end[m] - mode_beg[m];
    const long long i0 = ioff[l], i1 = ioff[l + 1];
    // the k-th smallest FP32 value over the items' sorted lists, and the band
    float band = 0.f;
    for (long long it = i0 + lane; it < i1; it += 32) band = fmaxf(band, item_band[it]);
#pragma unroll
    for (int o = 16; o; o >>= 1) band = fmaxf(band, __shfl_xor_sync(MRMG_FULL, band, o));
    float kth = INF;
    {
      // lane l owns items l, l + 32, ..., (up to 16 each: 512 items, modes
      // of up to 131,072 nodes; larger ones rerun) with a head position per item
      int heads[16];
#pragma unroll
      for (int j = 0; j < 16; j++) heads[j] = 0;
      const long long n_it = i1 - i0;
      bool ok = n_it <= 512;
      if (__any_sync(MRMG_FULL, !ok)) {
        if (lane == 0) { const int slot = atomicAdd(n_fallback, 1); fallback[slot] = l; }
        continue;
      }
      for (int r = 0; r < k; r++) {
        float bv = INF;
        int bj = -1;
#pragma unroll
        for (int j = 0; j < 16; j++) {
          const long long it = i0 + lane + 32 * j;
          if (it < i1 && heads[j] < k) {
            const float v = cand_key[it * k + heads[j]];
            if (v < bv) { bv = v; bj = j; }
          }
        }
        float wv = bv;
#pragma unroll
        for (int o = 16; o; o >>= 1) wv = fminf(wv, __shfl_xor_sync(MRMG_FULL, wv, o));
        kth = wv;
        if (wv == INF) break;
        const unsigned who = __ballot_sync(MRMG_FULL, bv == wv);
        if (lane == __ffs(who) - 1) {
#pragma unroll
          for (int j = 0; j < 16; j++)
            if (j == bj) heads[j]++;
        }
      }
    }
    const float tau = kth == INF ? INF : (kth + 2.f * band) * (1.f + 9.5367431640625e-7f);
    // certificate: every left-out node of every item lies above tau (with
    // fewer than k finite values: every node of the mode is a candidate)
    bool unsafe = false;
    if (kth != INF)
      for (long long it = i0 + lane; it < i1; it += 32) unsafe |= !(item_next[it] > tau);
    // gather the finite candidates within tau, in item order
    int mine = 0;
    for (long long it = i0 + lane; it < i1; it += 32)
      for (int r = 0; r < k && cand_key[it * k + r] <= tau && cand_key[it * k + r] < INF; r++) mine++;
    int incl = mine;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(MRMG_FULL, incl, o);
      if (lane >= o) incl += y;
    }
    const int ncand = __shfl_sync(MRMG_FULL, incl, 31);
    unsafe |= ncand > kSplitGather || (kth == INF && ncand != M);
    if (__any_sync(MRMG_FULL, unsafe)) {
      if (lane == 0) { const int slot = atomicAdd(n_fallback, 1); fallback[slot] = l; }
      continue;
    }
    int w = incl - mine;
    for (long long it = i0 + lane; it < i1; it += 32)
      for (int r = 0; r < k && cand_key[it * k + r] <= tau && cand_key[it * k + r] < INF; r++)
        sid[w++] = cand_idx[it * k + r];
    __syncwarp();
    // FP64 re-rank, one candidate per lane; (distance, index) order
    long long td[KM];
    long long ti[KM];
#pragma unroll
    for (int i = 0; i < KM; i++) { td[i] = 0x7ff0000000000000ll; ti[i] = 0x7fffffffffffffffll; }
    const double* qq = qs + q * t.D;
    const double* xb = nodes + mode_beg[m] * t.D;
    for (int x = lane; x < ncand; x += 32) {
      const long long id = sid[x];
      const double* xx = xb + id * t.D;
      auto dfun = [&](int jj) { return __dsub_rn(qq[jj], xx[jj]); };
      const long long d = dkey(dist_of(t, metric, dfun));
      if (d < td[k - 1] || (d == td[k - 1] && id < ti[k - 1])) {
#pragma unroll
        for (int i = KM - 1; i > 0; i--) {
          if (i < k) {
            const bool before = d < td[i - 1] || (d == td[i - 1] && id < ti[i - 1]);
            const bool here = d < td[i] || (d == td[i] && id < ti[i]);
            if (before) { td[i] = td[i - 1]; ti[i] = ti[i - 1]; }
            else if (here) { td[i] = d; ti[i] = id; }
          }
        }
        if (d < td[0] || (d == td[0] && id < ti[0])) { td[0] = d; ti[0] = id; }
      }
    }
    int head = 0;
    for (int r = 0; r < k; r++) {
      long long hd = 0x7ff0000000000000ll;
      long long hi = 0x7fffffffffffffffll;
#pragma unroll
      for (int i = 0; i < KM; i++)
        if (i == head) { hd = td[i]; hi = ti[i]; }
      const int win = warp_argmin(hd, hi);
      const long long wd = __shfl_sync(MRMG_FULL, hd, win);
      const long long wi = __shfl_sync(MRMG_FULL, hi, win);
      if (lane == 0) {
        out_idx[q * k + r] = wi == 0x7fffffffffffffffll ? -1 : wi;
        out_dist[q * k + r] = wi == 0x7fffffffffffffffll ? __longlong_as_double(0x7ff0000000000000ll)
                                                         : __longlong_as_double(wd);
      }
      if (lane == win) head++;
    }
    __syncwarp();
  }
}

// radius, exact: warp per (query, bitmap word), lane = node of the word
__global__ void near_split_kernel(const double* __restrict__ qs, const float* __restrict__ qs32, long long Q,
                                  const int* __restrict__ q_mode, const double* __restrict__ nodes,
                                  const float* __restrict__ nodes32, const long long* __restrict__ mode_beg,
                                  const long long* __restrict__ mode_end, SliceTab t, int metric,
                                  const double* __restrict__ rp, const long long* __restrict__ woff,
                                  unsigned* __restrict__ bits, unsigned long long* __restrict__ counts) {
  const int lane = threadIdx.x & 31;
  const long long warp = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const long long nwarps = (long long)gridDim.x * (blockDim.x >> 5);
  const long long total = woff[Q];
  for (long long f = warp; f < total; f += nwarps) {
    const long long q = owner_of(woff, Q, f);
    const int m = q_mode[q];
    const long long id = (f - woff[q]) * 32 + lane;
    bool in = false;
    if (id < mode_end[m] - mode_beg[m]) {
      const long long x = mode_beg[m] + id;
      in = within_radius(qs32 + q * t.D, nodes32 + x * t.D, qs + q * t.D, nodes + x * t.D, t, metric,
                         radius_test(rp[q]));
    }
    const unsigned mk = __ballot_sync(MRMG_FULL, in);
    if (lane == 0) {
      bits[f] = mk;
      if (mk) atomicAdd(counts + q, (unsigned long long)__popc(mk));
    }
  }
}

}  // namespace

cudaError_t knn_exact(const double* qs, long long Q, const int* q_mode, const long long* q_list, long long n_list,
                      const double* nodes, const long long* mode_beg, const long long* mode_end, const SliceTab& t,
                      int metric, int k, long long* out_idx, double* out_dist, int num_sms, cudaStream_t st) {
  const long long total = q_list ? n_list : Q;
  if (total <= 0) return cudaSuccess;
  const int warps = 4;
  const int grid = (int)std::min<long long>((total + warps - 1) / warps, (long long)num_sms * 16);
  if (k <= 16)
    knn_exact_kernel<16><<<grid, warps * 32, 0, st>>>(qs, Q, q_mode, q_list, n_list, nodes, mode_beg, mode_end, t,
                                                      metric, k, out_idx, out_dist);
  else
    knn_exact_kernel<kKnnMaxK><<<grid, warps * 32, 0, st>>>(qs, Q, q_mode, q_list, n_list, nodes, mode_beg, mode_end,
                                                            t, metric, k, out_idx, out_dist);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// tcgen05 / TMA / mbarrier helpers (inline PTX)
// ---------------------------------------------------------------------------
namespace {

__device__ __forceinline__ void tmem_alloc(uint32_t* dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(dst_smem)), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// D[tmem] (+)= A[smem] * B[smem]^T, kind::f16 (BF16 in, FP32 accumulate), one thread
__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(bar))
               : "memory");
}

// 32 lanes x 32 consecutive FP32 columns of TMEM (warp-wide)
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%"
      "28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

// shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 bytes apart; `addr` may carry a K offset inside the 128-byte row
__device__ __forceinline__ uint64_t sw128_desc(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFF) >> 4);
  d |= (uint64_t)1 << 16;            // leading byte offset (unused for a single 128-byte K span)
  d |= (uint64_t)(1024 >> 4) << 32;  // stride byte offset: next 8-row group
  d |= (uint64_t)1 << 46;            // descriptor version
  d |= (uint64_t)2 << 61;            // 128-byte swizzle
  return d;
}

// instruction descriptor, kind::f16: FP32 accumulator, BF16 A and B, both K-major
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// byte offset of element (row, col) (bf16) in a SW128 K-major tile
__host__ __device__ __forceinline__ uint32_t sw128_off(int row, int col) {
  const uint32_t lin = (uint32_t)row * kRowBytes + (uint32_t)col * 2;
  const uint32_t chunk = (lin >> 4) & 7, r8 = (lin >> 7) & 7;
  return (lin & ~0x70u) | ((chunk ^ r8) << 4);
}

}  // namespace

// ---------------------------------------------------------------------------
// Self-test GEMM for the descriptor encodings: C[128 x N] = A[128 x 64] *
// B[N x 64]^T with A, B given row-major BF16 in global memory (one CTA).
// ---------------------------------------------------------------------------
namespace {
__global__ void umma_selftest_kernel(const __nv_bfloat16* A, const __nv_bfloat16* B, int N, float* C, int* err) {
  extern __shared__ __align__(1024) unsigned char sm_raw[];
  unsigned char* base = (unsigned char*)(((uintptr_t)sm_raw + 1023) & ~(uintptr_t)1023);
  unsigned char* sa = base;                       // 16 KB
  unsigned char* sb = base + kTileM * kRowBytes;  // N * 128 B
  __shared__ uint64_t bar;
  __shared__ uint32_t tbase;
  const int tid = threadIdx.x, warp = tid >> 5;
  for (int i = tid; i < kTileM * 64; i += blockDim.x) *(__nv_bfloat16*)(sa + sw128_off(i / 64, i % 64)) = A[i];
  for (int i = tid; i < N * 64; i += blockDim.x) *(__nv_bfloat16*)(sb + sw128_off(i / 64, i % 64)) = B[i];
  if (tid == 0) {
    mbar_init(&bar, 1);
    fence_barrier_init();
  }
  fence_async_smem();
  if (warp == 0) tmem_alloc(&tbase, 256);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tm = tbase;
  if (tid == 0) {
    const uint32_t idesc = idesc_bf16(kTileM, N);
    for (int s = 0; s < 4; s++)
      umma_bf16(tm, sw128_desc(su32(sa) + 32 * s), sw128_desc(su32(sb) + 32 * s), idesc, s > 0);
    umma_commit(&bar);
  }
  const bool ok = mbar_wait(&bar, 0);
  tc_fence_after();
  if (!ok) {
    if (tid == 0) atomicOr(err, E_TIMEOUT);
  } else {
    for (int c0 = 0; c0 < N; c0 += 32) {
      float v[32];
      tmem_ld32(tm + ((uint32_t)(32 * warp) << 16) + c0, v);
      for (int i = 0; i < 32; i++) C[(32 * warp + (tid & 31)) * N + c0 + i] = v[i];
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) tmem_dealloc(tm, 256);
}
}  // namespace

cudaError_t umma_selftest(const void* A, const void* B, int N, float* C, int* err, cudaStream_t st) {
  const size_t smem = 1024 + (size_t)(kTileM + N) * kRowBytes;
  cudaFuncSetAttribute(umma_selftest_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  umma_selftest_kernel<<<1, 128, smem, st>>>((const __nv_bfloat16*)A, (const __nv_bfloat16*)B, N, C, err);
  return cudaGetLastError();
}

}  // namespace mrmg

// ===========================================================================
// Tensor-core candidate path
// ===========================================================================
namespace mrmg {

// node-store formats
enum : int { KNN_FMT_EUCL = 0, KNN_FMT_AGENT = 1 };
constexpr int kNtEucl = 128, kNtAgent = 64;

struct KnnItem {          // one CTA: a query tile of one mode against a chunk of its node tiles
  int mode, q0, qn;       // queries qorder[q0 .. q0+qn)
  int tile0, tile1;       // node tiles [tile0, tile1) of the mode (mode-local tile index)
  int chunk;              // chunk slot of this item in the candidate lists
  int pad;
};

struct KnnStoreDev {
  int fmt, NT, D, A;
  int agent_s[4], agent_e[4];
  const unsigned char* tiles;     // packed SW128 tiles
  const long long* mode_beg;      // first row of each mode in the node buffer (device)
  const long long* mode_end;      // one past its last row
  const int* mode_tile0;          // first global tile of each mode (mode_beg / NT)
  const float* mode_xmax;         // max |x| of each mode (for the error bound)
};

namespace {

__device__ __forceinline__ void put_bf16(unsigned char* row_base_tile, int row, int col, float v) {
  *(__nv_bfloat16*)(row_base_tile + sw128_off(row, col)) = __float2bfloat16_rn(v);
}

// split x into bf16 hi + lo (both as floats)
__device__ __forceinline__ void split2(double x, float* hi, float* lo) {
  const float xf = (float)x;
  const float h = __bfloat162float(__float2bfloat16_rn(xf));
  *hi = h;
  *lo = __bfloat162float(__float2bfloat16_rn((float)(x - (double)h)));
}

// packs the rows of global tiles [tile_lo, tile_hi): a row past its mode's
// last node is padding.  `mode` >= 0 names the tiles' mode, else each tile's
// mode is found from the (ascending) first tiles.
__global__ void knn_pack_kernel(const double* __restrict__ nodes, KnnStoreDev st, int n_modes, int mode,
                                long long tile_lo, long long tile_hi, unsigned char* __restrict__ tiles,
                                float* __restrict__ xmax_out) {
  const long long rows = (tile_hi - tile_lo) * st.NT;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < rows;
       g += (long long)gridDim.x * blockDim.x) {
    const long long tile = tile_lo + g / st.NT;
    const int row = (int)(g % st.NT);
    int m = mode;
    if (m < 0) {
      m = 0;
      while (m + 1 < n_modes && st.mode_tile0[m + 1] <= tile) m++;
    }
    const long long local = (tile - st.mode_tile0[m]) * st.NT + row;
    const long long node = st.mode_beg[m] + local;
    unsigned char* t = tiles + tile * (long long)st.NT * kRowBytes;
    for (int c = 0; c < 64; c++) put_bf16(t, row, c, 0.f);
    if (node >= st.mode_end[m]) {     // padding row: a huge |x|^2 term, never selected
      if (st.fmt == KNN_FMT_EUCL) put_bf16(t, row, st.D, 1.0e30f);
      else for (int a = 0; a < st.A; a++) put_bf16(t, row, 16 * a + 2 * (st.agent_e[a] - st.agent_s[a]), 1.0e30f);
      continue;
    }
    const double* x = nodes + node * st.D;
    double n2 = 0.0;
    if (st.fmt == KNN_FMT_EUCL) {
      for (int j = 0; j < st.D; j++) {
        float h, l;
        split2(x[j], &h, &l);
        put_bf16(t, row, j, h);
        put_bf16(t, row, st.D + 3 + j, l);
        n2 += x[j] * x[j];
      }
      const float a1 = __bfloat162float(__float2bfloat16_rn((float)n2));
      const double r1 = n2 - (double)a1;
      const float a2 = __bfloat162float(__float2bfloat16_rn((float)r1));
      const float a3 = (float)(r1 - (double)a2);
      put_bf16(t, row, st.D, a1);
      put_bf16(t, row, st.D + 1, a2);
      put_bf16(t, row, st.D + 2, a3);
    } else {
      for (int a = 0; a < st.A; a++) {
        const int s = st.agent_s[a], d = st.agent_e[a] - s;
        double na = 0.0;
        for (int j = 0; j < d; j++) {
          float h, l;
          split2(x[s + j], &h, &l);
          put_bf16(t, row, 16 * a + j, h);
          put_bf16(t, row, 16 * a + d + j, l);
          na += x[s + j] * x[s + j];
        }
        const float a1 = __bfloat162float(__float2bfloat16_rn((float)na));
        put_bf16(t, row, 16 * a + 2 * d, a1);
        put_bf16(t, row, 16 * a + 2 * d + 1, (float)(na - (double)a1));
        n2 += na;
      }
    }
    atomicMax((int*)&xmax_out[m], __float_as_int((float)sqrt(n2) * 1.000001f));   // non-negative floats order as ints
  }
}

// Per-thread kept list: kKeep packed keys in ascending order.  A key is the
// FP32 bit pattern of a non-negative approximate squared distance with its
// low bits (`imask`) replaced by the node's index within the item's node
// chunk, so unsigned key order is distance order (the distance truncated to
// the remaining mantissa bits, ties to the lower index) and one unsigned
// min/max pair per slot inserts distance and index together, branch-free.
// The key's distance lies in [lower, upper]: its bits with the index bits
// cleared, and with them all set.  An empty slot holds kKeyEmpty: FLT_MAX's
// bits, whose index field (all ones) no node of a chunk has (a chunk holds
// fewer than imask + 1 nodes).
constexpr unsigned kKeyEmpty = 0x7f7fffffu;

__device__ __forceinline__ void key_insert(unsigned (&kk)[kKeep], unsigned key) {
#pragma unroll
  for (int i = kKeep - 1; i > 0; i--) kk[i] = min(kk[i], max(kk[i - 1], key));
  kk[0] = min(kk[0], key);
}

__device__ __forceinline__ float key_lower(unsigned key, unsigned imask) { return __uint_as_float(key & ~imask); }
__device__ __forceinline__ float key_upper(unsigned key, unsigned imask) { return __uint_as_float(key | imask); }

// Column groups of the epilogue: warp w reads TMEM lanes 32*(w%4) (the lane
// quadrant its warp rank allows) and the w/4-th slice of each tile's columns,
// so every query row is scanned by kSplit threads with their own kept lists,
// merged through shared memory at the end.
// Marks of a 32-column chunk (bit i: v[i] > t, or v[i] < t): four
// independent partial masks, so the compare-and-or chain is 8 steps deep
// instead of 32 (a warp per TMEM lane quadrant leaves few warps per scheduler
// to hide a long chain).
template <bool GT>
__device__ __forceinline__ unsigned mark32(const float (&v)[32], float t) {
  unsigned p[4] = {0u, 0u, 0u, 0u};
#pragma unroll
  for (int i = 0; i < 8; i++)
#pragma unroll
    for (int g = 0; g < 4; g++) p[g] |= (unsigned)(GT ? v[8 * g + i] > t : v[8 * g + i] < t) << (8 * g + i);
  return (p[0] | p[1]) | (p[2] | p[3]);
}

// One 32-column chunk of a query row, `mk` marking the columns whose
// distance may lie under the row's threshold: the chunk's values go to this
// thread's column of `cand` (column-major over the CTA's threads, so stores
// and dynamically indexed reloads are bank-conflict free) and only the marked
// ones become keys and meet the kept list: the warp runs as many insert steps
// as its busiest lane needs, instead of one per column whenever any lane
// inserts.  `lcol0` is the chunk-local index of the first column.  A marked
// value whose key does not beat the 16th (earlier inserts of the chunk may
// have lowered it) is dropped after one compare; a NaN distance is never
// marked, an infinite one makes a key above every kept key.
template <bool FROM_DOT>
__device__ __forceinline__ void keep_marked(unsigned (&kk)[kKeep], const float (&v)[32], unsigned mk, float qn,
                                            float* cand, int lcol0, unsigned imask) {
  const int nth = blockDim.x;
#pragma unroll
  for (int i = 0; i < 32; i++) cand[i * nth] = v[i];
  while (mk) {
    const int i = __ffs(mk) - 1;
    mk &= mk - 1;
    const float d = FROM_DOT ? fmaf(-2.f, cand[i * nth], qn) : cand[i * nth];
    const unsigned key = (__float_as_uint(fmaxf(d, 0.f)) & ~imask) | (unsigned)(lcol0 + i);
    if (key < kk[kKeep - 1]) key_insert(kk, key);
  }
}

// Radius mode: each thread's 32 columns of a chunk are 32 consecutive
// mode-local nodes starting on a multiple of 32, so the chunk's verdicts are
// one whole word of the query's candidate bitmap, written by exactly this
// thread (no atomics, no list capacity).
struct RadOut {
  unsigned* bits;                   // word w of query q at bits[woff[q] + w]
  const long long* woff;            // [Q + 1]
  const float* rad2;                // per query: (radius + eps)^2 rounded up (or -1)
};

template <bool FROM_DOT>
__device__ __forceinline__ void rad_chunk(const float (&v)[32], float qn, float tau, long long qid, int col0,
                                          const RadOut& ro) {
  if (qid < 0) return;
  unsigned m = 0;
#pragma unroll
  for (int i = 0; i < 32; i++) {
    const float d = FROM_DOT ? fmaf(-2.f, v[i], qn) : v[i];
    if (d <= tau) m |= 1u << i;
  }
  ro.bits[ro.woff[qid] + (col0 >> 5)] = m;
}

template <int FMT> struct TcSplit { static constexpr int S = FMT == KNN_FMT_EUCL ? 1 : 2; };

template <int FMT, bool RAD>
__global__ void __launch_bounds__(128 * TcSplit<FMT>::S, 1) knn_tc_kernel(KnnStoreDev st, const double* __restrict__ qs,
                                                        const int* __restrict__ qorder, const KnnItem* __restrict__ items,
                                                        int chunks_max, float* __restrict__ cand_d,
                                                        int* __restrict__ cand_i, float* __restrict__ cand_b,
                                                        unsigned* __restrict__ g_thr, float* __restrict__ q_eps,
                                                        int* __restrict__ err, RadOut ro, unsigned imask) {
  constexpr int NT = FMT == KNN_FMT_EUCL ? kNtEucl : kNtAgent;
  constexpr uint32_t BT = NT * kRowBytes;   // bytes per node tile
  constexpr int S = TcSplit<FMT>::S, NCOL = NT / S;
  static_assert(NCOL % 32 == 0, "column slice is whole 32-column loads");
  // tensor-memory columns: two accumulator buffers of one node tile each
  // (euclidean: 2 x 128 = 256, so two CTAs share an SM's 512 columns;
  // per-agent blocks: 2 x 4 x 64 = 512, one CTA per SM)
  constexpr uint32_t kTm = FMT == KNN_FMT_EUCL ? 2 * NT : 512;
  extern __shared__ __align__(1024) unsigned char sm_raw[];
  unsigned char* base = (unsigned char*)(((uintptr_t)sm_raw + 1023) & ~(uintptr_t)1023);
  unsigned char* sA1 = base;
  unsigned char* sA2 = base + kTileM * kRowBytes;
  unsigned char* sB0 = base + 2 * kTileM * kRowBytes;   // kStagesB node-tile buffers
  // per-thread candidate column: [32][blockDim] values after the operand buffers
  float* cand = (float*)(sB0 + kStagesB * (size_t)BT) + threadIdx.x;
  __shared__ uint64_t bar_load[kStagesB], bar_mma[2];
  __shared__ uint32_t tbase;
  __shared__ int s_fail;
  __shared__ float s_qn[kTileM], s_qna[4][kTileM];
  __shared__ float s_tau[RAD ? kTileM : 1];
  __shared__ long long s_qid[kTileM];
  __shared__ float s_bound[RAD ? 1 : kTileM];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int row = tid & (kTileM - 1), slice = tid / kTileM;
  const KnnItem it = items[blockIdx.x];
  const int D = st.D;

  if (tid == 0) {
    for (int b = 0; b < kStagesB; b++) mbar_init(&bar_load[b], 1);
    mbar_init(&bar_mma[0], 1); mbar_init(&bar_mma[1], 1);
    s_fail = 0;
    fence_barrier_init();
  }
  if (warp == 0) tmem_alloc(&tbase, kTm);

  // ---- the query tile: A1 = [q_hi | -1/2 ... | q_hi], A2 = [q_lo]; one thread per row
  float qn = 0.f, qna[4] = {0.f, 0.f, 0.f, 0.f};
  long long qid = -1;
  if (tid < kTileM) {
    const int r = tid;
    for (int c = 0; c < 64; c++) {
      *(__nv_bfloat16*)(sA1 + sw128_off(r, c)) = __float2bfloat16_rn(0.f);
      *(__nv_bfloat16*)(sA2 + sw128_off(r, c)) = __float2bfloat16_rn(0.f);
    }
    if (r < it.qn) {
      qid = qorder[it.q0 + r];
      const double* q = qs + qid * D;
      if (FMT == KNN_FMT_EUCL) {
        double n2 = 0.0;
        for (int j = 0; j < D; j++) {
          float h, l;
          split2(q[j], &h, &l);
          *(__nv_bfloat16*)(sA1 + sw128_off(r, j)) = __float2bfloat16_rn(h);
          *(__nv_bfloat16*)(sA1 + sw128_off(r, D + 3 + j)) = __float2bfloat16_rn(h);
          *(__nv_bfloat16*)(sA2 + sw128_off(r, j)) = __float2bfloat16_rn(l);
          n2 += q[j] * q[j];
        }
        for (int c = 0; c < 3; c++) *(__nv_bfloat16*)(sA1 + sw128_off(r, D + c)) = __float2bfloat16_rn(-0.5f);
        qn = (float)n2;
      } else {
        for (int a = 0; a < st.A; a++) {
          const int s = st.agent_s[a], d = st.agent_e[a] - s;
          double na = 0.0;
          for (int j = 0; j < d; j++) {
            float h, l;
            split2(q[s + j], &h, &l);
            *(__nv_bfloat16*)(sA1 + sw128_off(r, 16 * a + j)) = __float2bfloat16_rn(h);
            *(__nv_bfloat16*)(sA1 + sw128_off(r, 16 * a + d + j)) = __float2bfloat16_rn(h);
            *(__nv_bfloat16*)(sA2 + sw128_off(r, 16 * a + j)) = __float2bfloat16_rn(l);
            na += q[s + j] * q[s + j];
          }
          *(__nv_bfloat16*)(sA1 + sw128_off(r, 16 * a + 2 * d)) = __float2bfloat16_rn(-0.5f);
          *(__nv_bfloat16*)(sA1 + sw128_off(r, 16 * a + 2 * d + 1)) = __float2bfloat16_rn(-0.5f);
          qna[a] = (float)na;
          qn += (float)na;
        }
      }
      // error bound of the approximate squared distance (split-BF16 operands,
      // FP32 accumulation), per query; stored once per query
      const float es = sqrtf(qn) + st.mode_xmax[it.mode];
      const float eps = 1.2e-4f * es * es + 1e-30f;
      if (!RAD && it.chunk == 0) q_eps[qid] = eps;
      if (RAD) s_tau[r] = ro.rad2[qid] < 0.f ? -__int_as_float(0x7f800000) : ro.rad2[qid] + 1.0001f * eps;
    }
    s_qid[r] = qid;
    s_qn[r] = qn;
    for (int a = 0; a < 4; a++) s_qna[a][r] = qna[a];
  }
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tm = tbase;
  const int T = it.tile1 - it.tile0;
  qn = s_qn[row];
  const unsigned char* gtiles = st.tiles + (long long)(st.mode_tile0[it.mode] + it.tile0) * BT;
  const uint32_t idesc = idesc_bf16(kTileM, NT);

  auto issue_load = [&](int t) {
    unsigned char* dst = sB0 + (t % kStagesB) * BT;
    mbar_expect_tx(&bar_load[t % kStagesB], BT);
    bulk_g2s(dst, gtiles + (long long)t * BT, BT, &bar_load[t % kStagesB]);
  };
  auto issue_mma = [&](int t) {
    const uint32_t a1 = su32(sA1), a2 = su32(sA2), b = su32(sB0 + (t % kStagesB) * BT);
    const uint32_t dcol = tm + (uint32_t)((t & 1) * (kTm / 2));
    if (FMT == KNN_FMT_EUCL) {
      for (int s = 0; s < 4; s++) umma_bf16(dcol, sw128_desc(a1 + 32 * s), sw128_desc(b + 32 * s), idesc, s > 0);
      const int s2 = (D + 15) / 16;
      for (int s = 0; s < s2; s++) umma_bf16(dcol, sw128_desc(a2 + 32 * s), sw128_desc(b + 32 * s), idesc, 1);
    } else {
      for (int a = 0; a < st.A; a++) {
        umma_bf16(dcol + 64 * a, sw128_desc(a1 + 32 * a), sw128_desc(b + 32 * a), idesc, 0);
        umma_bf16(dcol + 64 * a, sw128_desc(a2 + 32 * a), sw128_desc(b + 32 * a), idesc, 1);
      }
    }
    umma_commit(&bar_mma[t & 1]);
  };

  if (tid == 0 && T > 0) {
    for (int t = 0; t < kStagesB && t < T; t++) issue_load(t);
    if (mbar_wait(&bar_load[0], 0)) issue_mma(0);
    else s_fail = 1;
  }

  unsigned kk[kKeep];
#pragma unroll
  for (int i = 0; i < kKeep; i++) kk[i] = kKeyEmpty;
  // Threshold shared by the CTAs that scan other node chunks of the same
  // query: g_thr[q] holds the smallest 16th-kept value any of them has
  // published (FP32 bits of a non-negative value, so unsigned order is value
  // order): the upper end of its 16th key's distance, so 16 nodes lie at or
  // below it.  A row filters with min(lower end of its own 16th key, shared),
  // read one tile ahead (a node the filter drops may tie the 16th key's
  // truncated distance: the list may then miss it, which the bound covers);
  // `bound` is the smallest shared threshold this row has filtered with: every
  // node of the chunk left out of the list lies at or above min(bound, lower
  // end of the 16th key).
  const long long qrow = RAD ? -1 : s_qid[row];
  float gcur = __int_as_float(0x7f800000), gnext = gcur, bound = gcur, published = gcur;

  for (int t = 0; t < T; t++) {
    if (tid == 0 && t + 1 < T && !s_fail) {
      if (mbar_wait(&bar_load[(t + 1) % kStagesB], ((t + 1) / kStagesB) & 1)) issue_mma(t + 1);
      else s_fail = 1;
    }
    const bool done = mbar_wait(&bar_mma[t & 1], (t >> 1) & 1);
    if (!done) s_fail = 1;
    tc_fence_after();
    if (tid == 0 && t + kStagesB < T && done) issue_load(t + kStagesB);   // tile t's MMAs have read its buffer
    if (!RAD && qrow >= 0) gnext = __uint_as_float(*(volatile const unsigned*)&g_thr[qrow]);
    if (done) {
      const int lcol = t * NT;   // chunk-local index of the tile's first node
      const uint32_t lane_base = tm + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)((t & 1) * (kTm / 2));
      if (FMT == KNN_FMT_EUCL) {
#pragma unroll 1
        for (int c0 = slice * NCOL; c0 < slice * NCOL + NCOL; c0 += 32) {
          float v[32];
          tmem_ld32(lane_base + c0, v);
          if (RAD) {
            rad_chunk<true>(v, qn, s_tau[row], s_qid[row], (it.tile0 + t) * NT + c0, ro);
          } else if (qrow >= 0) {   // a padding row of a partial query tile keeps no list
            // marks: the dot products against the row's threshold in dot
            // space, (qn - thr) / 2, lowered by a margin that covers the FP32
            // rounding of both forms, so an unmarked column's distance
            // qn - 2 v lies at or above thr
            const float thr = fminf(key_lower(kk[kKeep - 1], imask), gcur);
            const float thd = 0.5f * (qn - thr) - 1e-6f * (fabsf(qn) + fabsf(thr));
            const unsigned mk = mark32<true>(v, thd);
            if (mk) keep_marked<true>(kk, v, mk, qn, cand, lcol + c0, imask);
          }
        }
      } else {
#pragma unroll 1
        for (int c0 = slice * NCOL; c0 < slice * NCOL + NCOL; c0 += 32) {
          float m[32];
#pragma unroll
          for (int i = 0; i < 32; i++) m[i] = -__int_as_float(0x7f800000);
          for (int a = 0; a < st.A; a++) {
            float v[32];
            tmem_ld32(lane_base + 64 * a + c0, v);
            const float qa = s_qna[a][row];
#pragma unroll
            for (int i = 0; i < 32; i++) m[i] = fmaxf(m[i], fmaf(-2.f, v[i], qa));
          }
          if (RAD) {
            rad_chunk<false>(m, 0.f, s_tau[row], s_qid[row], (it.tile0 + t) * NT + c0, ro);
          } else if (qrow >= 0) {
            const float thr = fminf(key_lower(kk[kKeep - 1], imask), gcur);
            const unsigned mk = mark32<false>(m, thr);
            if (mk) keep_marked<false>(kk, m, mk, 0.f, cand, lcol + c0, imask);
          }
        }
      }
    }
    if (!RAD && qrow >= 0) {
      bound = fminf(bound, gcur);
      const float up = key_upper(kk[kKeep - 1], imask);
      if (up < published) {   // publish a better 16th value
        published = up;
        atomicMin(&g_thr[qrow], __float_as_uint(fmaxf(published, 0.f)));
      }
      gcur = fminf(gcur, gnext);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (s_fail) break;
  }
  if (s_fail && tid == 0) atomicOr(err, E_TIMEOUT);
  (void)lane;
  // merge the slices' lists into slice 0's; every MMA has completed, so the
  // operand buffers are free (skipped after a timeout: copies may be in flight)
  if (!RAD && !s_fail) {
    unsigned* mk = (unsigned*)base;
    if (slice > 0) {
#pragma unroll
      for (int i = 0; i < kKeep; i++) mk[((size_t)(slice - 1) * kKeep + i) * kTileM + row] = kk[i];
      if (S > 1) s_bound[row] = bound;   // (S <= 2)
    }
    __syncthreads();
    if (slice == 0) {
      for (int o = 0; o < S - 1; o++)
        for (int i = 0; i < kKeep; i++) {
          const unsigned key = mk[((size_t)o * kKeep + i) * kTileM + row];
          if (key >= kk[kKeep - 1]) break;   // each list is sorted
          key_insert(kk, key);
        }
      if (S > 1) bound = fminf(bound, s_bound[row]);
    }
  }
  // the lists leave as (lower end of the distance, mode-local node index),
  // an empty slot as (inf, -1)
  if (!RAD && qid >= 0) {
    float* od = cand_d + ((size_t)qid * chunks_max + it.chunk) * kKeep;
    int* oi = cand_i + ((size_t)qid * chunks_max + it.chunk) * kKeep;
    const float INF = __int_as_float(0x7f800000);
#pragma unroll
    for (int i = 0; i < kKeep; i++) {
      const bool empty = (kk[i] & imask) == imask;
      od[i] = empty ? INF : key_lower(kk[i], imask);
      oi[i] = empty ? -1 : it.tile0 * NT + (int)(kk[i] & imask);
    }
    const bool e15 = (kk[kKeep - 1] & imask) == imask;
    cand_b[(size_t)qid * chunks_max + it.chunk] = fminf(bound, e15 ? INF : key_lower(kk[kKeep - 1], imask));
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) tmem_dealloc(tm, kTm);
}

constexpr int kMergeWarps = 4;   // warps per merge CTA

// ---------------------------------------------------------------------------
// merge: certify the kept candidates and re-rank them in exact FP64
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(32 * kMergeWarps, 4) knn_merge_kernel(const double* __restrict__ qs, long long Q, const int* __restrict__ q_mode,
                                 const double* __restrict__ nodes, const long long* __restrict__ mode_beg,
                                 const long long* __restrict__ mode_end, const int* __restrict__ mode_chunks, int chunks_max, const float* __restrict__ cand_d,
                                 const int* __restrict__ cand_i, const float* __restrict__ cand_b,
                                 const float* __restrict__ q_eps, SliceTab t,
                                 int metric, int k, long long* __restrict__ out_idx, double* __restrict__ out_dist,
                                 long long* __restrict__ fallback, int* __restrict__ n_fallback, unsigned imask) {
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const long long warp = (long long)blockIdx.x * (blockDim.x >> 5) + wib;
  const long long nwarps = (long long)gridDim.x * (blockDim.x >> 5);
  const float INF = __int_as_float(0x7f800000);
  const double DINF = __longlong_as_double(0x7ff0000000000000ll);
  // per warp: the query's candidate lists (<= 64 x 16 approximate distances)
  // and the gathered ids within tau
  __shared__ float s_cd[kMergeWarps][64 * kKeep];
  __shared__ int s_id[kMergeWarps][64 * kKeep];
  float* sv = s_cd[wib];
  int* sid = s_id[wib];
  for (long long q = warp; q < Q; q += nwarps) {
    const int m = q_mode[q];
    const long long M = mode_end[m] - mode_beg[m];
    const int C = mode_chunks[m];
    if (M == 0 || C == 0) {
      for (int r = lane; r < k; r += 32) { out_idx[q * k + r] = -1; out_dist[q * k + r] = DINF; }
      continue;
    }
    // lane l holds chunks l and l + 32 (C <= 64); the lists are staged in
    // shared memory with coalesced loads, so the rounds below do not wait on
    // global memory
    const float* cd = cand_d + (size_t)q * chunks_max * kKeep;
    const int* ci = cand_i + (size_t)q * chunks_max * kKeep;
    __syncwarp();
    for (int x = lane; x < C * kKeep; x += 32) sv[x] = cd[x];
    __syncwarp();
    int h0 = 0, h1 = 0;
    const int c0 = lane, c1 = lane + 32;
    // The lists hold the lower ends of their keys' distances (sorted; an
    // empty slot is inf), so a kept distance lies in [v, v | imask].  An
    // upper bound of the k-th smallest approximate value: k rounds of a warp
    // argmin over list heads, each head at its upper end.
    auto upper = [&](float v) { return v == INF ? INF : __uint_as_float(__float_as_uint(v) | imask); };
    float kth = INF;
    for (int r = 0; r < k; r++) {
      const float v0 = (c0 < C && h0 < kKeep) ? upper(sv[c0 * kKeep + h0]) : INF;
      const float v1 = (c1 < C && h1 < kKeep) ? upper(sv[c1 * kKeep + h1]) : INF;
      float v = fminf(v0, v1);
      float b = v;
#pragma unroll
      for (int o = 16; o; o >>= 1) b = fminf(b, __shfl_xor_sync(MRMG_FULL, b, o));
      kth = b;
      const unsigned who = __ballot_sync(MRMG_FULL, v == b);
      if (b == INF) break;
      if (lane == __ffs(who) - 1) { if (v0 <= v1) h0++; else h1++; }
    }
    const float tau = kth == INF ? INF : kth + 2.f * q_eps[q];
    // certified when every chunk's bound (all its nodes left out of its list
    // lie at or above it) is above tau
    bool unsafe = false;
    const float* cb = cand_b + (size_t)q * chunks_max;
    if (c0 < C) unsafe |= !(cb[c0] > tau);
    if (c1 < C) unsafe |= !(cb[c1] > tau);
    if (__any_sync(MRMG_FULL, unsafe)) {
      if (lane == 0) { const int s = atomicAdd(n_fallback, 1); fallback[s] = q; }
      continue;
    }
    // exact FP64 re-rank of every candidate within tau
    long long td[16];
    long long tix[16];
#pragma unroll
    for (int i = 0; i < 16; i++) { td[i] = 0x7ff0000000000000ll; tix[i] = -1; }
    const double* qq = qs + q * t.D;
    // gather the candidates within tau (a sorted prefix of each list) into
    // one warp-wide list, then compute their FP64 distances one per lane
    int n0 = 0, n1 = 0;
    if (c0 < C) while (n0 < kKeep && sv[c0 * kKeep + n0] <= tau) n0++;
    if (c1 < C) while (n1 < kKeep && sv[c1 * kKeep + n1] <= tau) n1++;
    int mine = n0 + n1, incl = mine;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(MRMG_FULL, incl, o);
      if (lane >= o) incl += y;
    }
    const int ncand = __shfl_sync(MRMG_FULL, incl, 31);
    int w = incl - mine;
    for (int j = 0; j < n0; j++) sid[w++] = ci[c0 * kKeep + j];
    for (int j = 0; j < n1; j++) sid[w++] = ci[c1 * kKeep + j];
    __syncwarp();
    for (int x = lane; x < ncand; x += 32) {
      const int id = sid[x];
      if (id < 0 || id >= M) continue;
      const double* xx = nodes + (mode_beg[m] + id) * t.D;
      auto dfun = [&](int jj) { return __dsub_rn(qq[jj], xx[jj]); };
      topk_insert<16>(td, tix, k < 16 ? k : 16, dkey(dist_of(t, metric, dfun)), id);
    }
    int head = 0;
    for (int r = 0; r < k; r++) {
      long long hd = 0x7ff0000000000000ll;
      long long hi = 0x7fffffffffffffffll;
#pragma unroll
      for (int i = 0; i < 16; i++)
        if (i == head) { hd = td[i]; hi = tix[i] < 0 ? 0x7fffffffffffffffll : tix[i]; }
      const int win = warp_argmin(hd, hi);
      const long long wd = __shfl_sync(MRMG_FULL, hd, win);
      const long long wi = __shfl_sync(MRMG_FULL, hi, win);
      if (lane == 0) {
        out_idx[q * k + r] = wi == 0x7fffffffffffffffll ? -1 : wi;
        out_dist[q * k + r] = wi == 0x7fffffffffffffffll ? DINF : __longlong_as_double(wd);
      }
      if (lane == win) head++;
    }
  }
}

// ---------------------------------------------------------------------------
// radius queries: exact re-check of the candidate bitmap, scan, ordered emit
// ---------------------------------------------------------------------------
constexpr int kNearWarps = 4;

// Each warp takes a query and walks its bitmap 32 words (1024 nodes) at a
// time: the set bits are listed in shared memory and spread over the lanes for
// the FP64 distance, so a dense word does not serialise one lane.  Bits whose
// exact distance exceeds the query's r' (or past the mode's nodes) are cleared.
constexpr int kNearStage = 48;   // results per query staged in order by the exact pass

__global__ void near_exact_kernel(const double* __restrict__ qs, const float* __restrict__ qs32, long long Q,
                                  const int* __restrict__ q_mode, const double* __restrict__ nodes,
                                  const float* __restrict__ nodes32, const long long* __restrict__ mode_beg,
                                  const long long* __restrict__ mode_end, SliceTab t,
                                  int metric, const double* __restrict__ rp, const long long* __restrict__ woff,
                                  unsigned* __restrict__ bits, long long* __restrict__ counts,
                                  int* __restrict__ stage) {
  __shared__ int s_list[kNearWarps][1024];
  __shared__ unsigned s_res[kNearWarps][32];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const long long warp = (long long)blockIdx.x * kNearWarps + wib;
  const long long nwarps = (long long)gridDim.x * kNearWarps;
  int* list = s_list[wib];
  for (long long q = warp; q < Q; q += nwarps) {
    const int m = q_mode[q];
    const long long M = mode_end[m] - mode_beg[m];
    const double* xb = nodes + mode_beg[m] * t.D;
    const float* xb32 = nodes32 + mode_beg[m] * t.D;
    const double* qq = qs + q * t.D;
    const float* qq32 = qs32 + q * t.D;
    const long long w0 = woff[q], W = woff[q + 1] - w0;
    const RadiusTest rt = radius_test(rp[q]);
    long long cnt = 0;
    for (long long base = 0; base < W; base += 32) {
      const long long w = base + lane;
      const unsigned mk = w < W ? bits[w0 + w] : 0u;
      const int c = __popc(mk);
      int incl = c;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(MRMG_FULL, incl, o);
        if (lane >= o) incl += y;
      }
      const int n = __shfl_sync(MRMG_FULL, incl, 31);
      if (n == 0) continue;
      int pos = incl - c;
      unsigned mm = mk;
      while (mm) {
        const int b = __ffs(mm) - 1;
        mm &= mm - 1;
        list[pos++] = lane * 32 + b;
      }
      s_res[wib][lane] = 0u;
      __syncwarp();
      for (int x = lane; x < n; x += 32) {
        const int loc = list[x];
        const long long id = base * 32 + loc;
        if (id >= M) continue;
        if (within_radius(qq32, xb32 + id * t.D, qq, xb + id * t.D, t, metric, rt))
          atomicOr(&s_res[wib][loc >> 5], 1u << (loc & 31));
      }
      __syncwarp();
      const unsigned res = s_res[wib][lane];
      if (w < W) bits[w0 + w] = res;
      // stage the first kNearStage results of the query in ascending order
      const int rc = __popc(res);
      int ri = rc;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(MRMG_FULL, ri, o);
        if (lane >= o) ri += y;
      }
      long long sp = cnt + ri - rc;
      unsigned rm = res;
      while (rm && sp < kNearStage) {
        const int b = __ffs(rm) - 1;
        rm &= rm - 1;
        stage[q * kNearStage + sp++] = (int)((base + lane) * 32 + b);
      }
      cnt += __shfl_sync(MRMG_FULL, ri, 31);
      __syncwarp();
    }
    if (lane == 0) counts[q] = cnt;   // the same in every lane
  }
}

// exclusive scan of the per-query counts into offsets[Q + 1] (one block; the
// query counts of a planner batch are thousands, not millions)
__global__ void near_scan_kernel(const long long* __restrict__ counts, long long Q, long long* __restrict__ offs_user,
                                 long long* __restrict__ offs, long long* __restrict__ total) {
  __shared__ long long s[1024];
  const int tid = threadIdx.x;
  const long long per = (Q + 1023) / 1024;
  const long long lo = tid * per < Q ? tid * per : Q, hi = lo + per < Q ? lo + per : Q;
  long long sum = 0;
  for (long long i = lo; i < hi; i++) sum += counts[i];
  s[tid] = sum;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    const long long y = tid >= o ? s[tid - o] : 0;
    __syncthreads();
    s[tid] += y;
    __syncthreads();
  }
  long long run = s[tid] - sum;
  for (long long i = lo; i < hi; i++) {
    offs[i] = run;
    if (offs_user) offs_user[i] = run;
    run += counts[i];
  }
  if (tid == 1023) {
    offs[Q] = s[1023];
    if (offs_user) offs_user[Q] = s[1023];
    *total = s[1023];
  }
}

// ascending mode-local indices, written from offsets[q]; positions at or
// past `cap` are skipped (their distances follow in near_dist_kernel)
__global__ void near_emit_kernel(long long Q, const long long* __restrict__ woff, const unsigned* __restrict__ bits,
                                 const int* __restrict__ stage, const long long* __restrict__ offs, long long cap,
                                 long long* __restrict__ out_idx) {
  __shared__ int s_list[kNearWarps][1024];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const long long warp = (long long)blockIdx.x * kNearWarps + wib;
  const long long nwarps = (long long)gridDim.x * kNearWarps;
  int* list = s_list[wib];
  for (long long q = warp; q < Q; q += nwarps) {
    long long o = offs[q];
    const long long nq = offs[q + 1] - o;
    if (o >= cap || nq == 0) continue;
    if (stage && nq <= kNearStage) {   // staged by the exact pass
      for (int x = lane; x < nq && o + x < cap; x += 32) out_idx[o + x] = stage[q * kNearStage + x];
      continue;
    }
    const long long w0 = woff[q], W = woff[q + 1] - w0;
    for (long long base = 0; base < W && o < cap; base += 32) {
      const long long w = base + lane;
      const unsigned mk = w < W ? bits[w0 + w] : 0u;
      const int c = __popc(mk);
      int incl = c;
#pragma unroll
      for (int sh = 1; sh < 32; sh <<= 1) {
        const int y = __shfl_up_sync(MRMG_FULL, incl, sh);
        if (lane >= sh) incl += y;
      }
      const int n = __shfl_sync(MRMG_FULL, incl, 31);
      if (n == 0) continue;
      int pos = incl - c;
      unsigned mm = mk;
      while (mm) {
        const int b = __ffs(mm) - 1;
        mm &= mm - 1;
        list[pos++] = lane * 32 + b;
      }
      __syncwarp();
      for (int x = lane; x < n; x += 32) {
        const long long p = o + x;
        if (p >= cap) break;
        out_idx[p] = base * 32 + list[x];
      }
      o += n;
      __syncwarp();
    }
  }
}

// FP64 distance of every written neighbour, a thread per output position (all
// lanes busy on the FP64 pipe); the total comes from the scan on the device
__global__ void near_dist_kernel(const double* __restrict__ qs, long long Q, const int* __restrict__ q_mode,
                                 const double* __restrict__ nodes, const long long* __restrict__ mode_beg, SliceTab t,
                                 int metric, const long long* __restrict__ offs, long long cap,
                                 const long long* __restrict__ out_idx, double* __restrict__ out_dist) {
  const long long total = offs[Q] < cap ? offs[Q] : cap;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < total;
       p += (long long)gridDim.x * blockDim.x) {
    const long long q = owner_of(offs, Q, p);
    const double* qq = qs + q * t.D;
    const double* xx = nodes + (mode_beg[q_mode[q]] + out_idx[p]) * t.D;
    auto dfun = [&](int j) { return __dsub_rn(qq[j], xx[j]); };
    out_dist[p] = dist_of(t, metric, dfun);
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// host side: node store and query launch
// ---------------------------------------------------------------------------
// The store owns its nodes: FP64 rows grouped by mode, each mode in a
// segment with room to grow (a multiple of the tile height), and on the
// tensor-core path the split-BF16 tiles of the same rows at the same
// positions.  Appending copies the new rows and packs only the tiles they
// touch; a full segment doubles (every segment is moved once to a new layout).
struct KnnStore {
  KnnStoreDev dev{};                      // tile-kernel view (tensor-core path)
  bool tc = false;
  SliceTab slices{};
  int metric = 0;
  int n_modes = 0;
  int D = 0;
  int NT = 64;                            // rows per tile = capacity granule
  std::vector<long long> beg, cnt, cap;   // per mode: first row, rows, capacity
  std::vector<int> mode_tiles;            // per mode: tiles holding its rows
  double* nodes = nullptr;                // [cap_total, D]
  float* nodes32 = nullptr;               // [cap_total, D] FP32 copy (radius pre-tests)
  unsigned char* tiles = nullptr;         // [cap_total / NT] tiles (tensor-core path)
  void* meta = nullptr;                   // device: beg, end, tile0, xmax per mode
  long long* d_beg = nullptr;
  long long* d_end = nullptr;
  int* d_tile0 = nullptr;
  float* d_xmax = nullptr;
  long long cap_total = 0;
  std::vector<long long> h_meta;          // staging for the beg / end upload
  std::vector<int> h_tile0;
  int* d_qmode = nullptr;                 // exact path: uploaded query modes
  long long qmode_cap = 0;
  int path = 0;                           // 0 auto, 1 tensor core where supported, 2 node-parallel exact
};

bool knn_tc_supported(const SliceTab& t, int metric) {
  if (metric == MRMG_METRIC_EUCLIDEAN) return t.end_all == t.D && t.D >= 1 && 2 * t.D + 3 <= 64;
  if (metric == MRMG_METRIC_MAX_EUCLIDEAN) {
    if (t.A < 1 || t.A > 4) return false;
    for (int i = 0; i < t.A; i++)
      if (t.e[i] - t.s[i] < 1 || 2 * (t.e[i] - t.s[i]) + 2 > 16) return false;
    return true;
  }
  return false;
}

static size_t al1k(size_t x) { return (x + 1023) & ~(size_t)1023; }

static void set_dev_view(KnnStore* s) {
  KnnStoreDev& d = s->dev;
  d.NT = s->NT;
  d.D = s->D;
  d.A = s->slices.A;
  for (int i = 0; i < 4; i++) {
    d.agent_s[i] = i < s->slices.A ? s->slices.s[i] : 0;
    d.agent_e[i] = i < s->slices.A ? s->slices.e[i] : 0;
  }
  d.tiles = s->tiles;
  d.mode_beg = s->d_beg;
  d.mode_end = s->d_end;
  d.mode_tile0 = s->d_tile0;
  d.mode_xmax = s->d_xmax;
}

static cudaError_t upload_meta(KnnStore* s, cudaStream_t st) {
  const int n = s->n_modes;
  s->h_meta.resize(2 * (size_t)std::max(n, 1));
  s->h_tile0.resize(std::max(n, 1));
  for (int m = 0; m < n; m++) {
    s->h_meta[m] = s->beg[m];
    s->h_meta[n + m] = s->beg[m] + s->cnt[m];
    s->h_tile0[m] = (int)(s->beg[m] / s->NT);
  }
  if (n == 0) return cudaSuccess;
  // beg and end sit back to back on the device
  cudaError_t e = cudaMemcpyAsync(s->d_beg, s->h_meta.data(), sizeof(long long) * 2 * n, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(s->d_tile0, s->h_tile0.data(), sizeof(int) * n, cudaMemcpyHostToDevice, st);
  return e;
}

// new buffers for `n_new` modes with capacities `cap_new` (rows, multiples of
// NT); the old modes' rows, tiles and norm bounds move over
static cudaError_t relayout(KnnStore* s, int n_new, const std::vector<long long>& cap_new, cudaStream_t st) {
  // every host allocation happens here, before the device buffers change
  // hands: a host allocation failure leaves the store as it was
  s->cnt.reserve(n_new);
  s->mode_tiles.reserve(n_new);
  s->cap.reserve(n_new);
  s->h_meta.reserve(2 * (size_t)std::max(n_new, 1));
  s->h_tile0.reserve(std::max(n_new, 1));
  std::vector<long long> beg_new(n_new, 0);
  long long total = 0;
  for (int m = 0; m < n_new; m++) { beg_new[m] = total; total += cap_new[m]; }
  double* nodes = nullptr;
  float* nodes32 = nullptr;
  unsigned char* tiles = nullptr;
  void* meta = nullptr;
  const size_t b_l = al1k(sizeof(long long) * std::max(n_new, 1));
  const size_t b_i = al1k(sizeof(int) * std::max(n_new, 1));
  cudaError_t e = cudaMalloc(&nodes, sizeof(double) * std::max<long long>(total, 1) * std::max(s->D, 1));
  if (e == cudaSuccess) e = cudaMalloc(&nodes32, sizeof(float) * std::max<long long>(total, 1) * std::max(s->D, 1));
  if (e == cudaSuccess && s->tc) e = cudaMalloc(&tiles, (size_t)std::max<long long>(total, s->NT) * kRowBytes);
  if (e == cudaSuccess) e = cudaMalloc(&meta, 2 * b_l + 2 * b_i);
  if (e != cudaSuccess) {
    if (nodes) cudaFree(nodes);
    if (nodes32) cudaFree(nodes32);
    if (tiles) cudaFree(tiles);
    return e;
  }
  long long* d_beg = (long long*)meta;
  long long* d_end = d_beg + (n_new > 0 ? n_new : 1);    // beg and end back to back
  int* d_tile0 = (int*)((unsigned char*)meta + 2 * b_l);
  float* d_xmax = (float*)((unsigned char*)meta + 2 * b_l + b_i);
  e = cudaMemsetAsync(d_xmax, 0, sizeof(float) * std::max(n_new, 1), st);
  for (int m = 0; m < s->n_modes && e == cudaSuccess; m++) {
    if (s->cnt[m] == 0) continue;
    e = cudaMemcpyAsync(nodes + beg_new[m] * s->D, s->nodes + s->beg[m] * s->D, sizeof(double) * s->cnt[m] * s->D,
                        cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(nodes32 + beg_new[m] * s->D, s->nodes32 + s->beg[m] * s->D,
                          sizeof(float) * s->cnt[m] * s->D, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess && s->tc)
      e = cudaMemcpyAsync(tiles + beg_new[m] * kRowBytes, s->tiles + s->beg[m] * kRowBytes,
                          (size_t)s->mode_tiles[m] * s->NT * kRowBytes, cudaMemcpyDeviceToDevice, st);
  }
  if (e == cudaSuccess && s->n_modes > 0 && s->d_xmax)
    e = cudaMemcpyAsync(d_xmax, s->d_xmax, sizeof(float) * std::min(s->n_modes, n_new), cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);   // the old buffers are read until here
  if (e != cudaSuccess) {
    cudaFree(nodes);
    cudaFree(nodes32);
    if (tiles) cudaFree(tiles);
    cudaFree(meta);
    return e;
  }
  if (s->nodes) cudaFree(s->nodes);
  if (s->nodes32) cudaFree(s->nodes32);
  if (s->tiles) cudaFree(s->tiles);
  if (s->meta) cudaFree(s->meta);
  s->nodes = nodes;
  s->nodes32 = nodes32;
  s->tiles = tiles;
  s->meta = meta;
  s->d_beg = d_beg;
  s->d_end = d_end;
  s->d_tile0 = d_tile0;
  s->d_xmax = d_xmax;
  s->cnt.resize(n_new, 0);
  s->mode_tiles.resize(n_new, 0);
  s->beg.swap(beg_new);
  s->cap.assign(cap_new.begin(), cap_new.end());
  s->n_modes = n_new;
  s->cap_total = total;
  set_dev_view(s);
  return upload_meta(s, st);
}

static long long round_up(long long x, long long g) { return (x + g - 1) / g * g; }

// FP32 copy of n values (rounded to nearest)
static cudaError_t to_f32(const double* src, float* dst, long long n, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const int grid = (int)std::min<long long>((n + 255) / 256, 4096);
  f64_to_f32_kernel<<<grid, 256, 0, st>>>(src, dst, n);
  return cudaGetLastError();
}

static cudaError_t pack_tiles(KnnStore* s, int mode, long long tile_lo, long long tile_hi, cudaStream_t st) {
  if (!s->tc || tile_hi <= tile_lo) return cudaSuccess;
  const long long rows = (tile_hi - tile_lo) * s->NT;
  const int grid = (int)std::min<long long>((rows + 255) / 256, 4096);
  knn_pack_kernel<<<grid, 256, 0, st>>>(s->nodes, s->dev, s->n_modes, mode, tile_lo, tile_hi, s->tiles, s->d_xmax);
  return cudaGetLastError();
}

cudaError_t knn_store_build(KnnStore* s, const double* d_nodes, long long M, const long long* h_mode_off, int n_modes,
                            const SliceTab& t, int metric, int D, cudaStream_t st) {
  s->slices = t;
  s->metric = metric;
  s->D = D;
  s->tc = knn_tc_supported(t, metric);
  const int fmt = metric == MRMG_METRIC_EUCLIDEAN ? KNN_FMT_EUCL : KNN_FMT_AGENT;
  s->NT = s->tc ? (fmt == KNN_FMT_EUCL ? kNtEucl : kNtAgent) : 64;
  s->dev.fmt = fmt;
  std::vector<long long> cap(n_modes, 0);
  for (int m = 0; m < n_modes; m++) {
    const long long c = h_mode_off[m + 1] - h_mode_off[m];
    cap[m] = c > 0 ? round_up(c + c / 4, s->NT) : 0;   // a quarter to grow into
  }
  cudaError_t e = relayout(s, n_modes, cap, st);
  if (e != cudaSuccess) return e;
  for (int m = 0; m < n_modes && e == cudaSuccess; m++) {
    const long long c = h_mode_off[m + 1] - h_mode_off[m];
    s->cnt[m] = c;
    s->mode_tiles[m] = (int)((c + s->NT - 1) / s->NT);
    if (c > 0)
      e = cudaMemcpyAsync(s->nodes + s->beg[m] * D, d_nodes + h_mode_off[m] * D, sizeof(double) * c * D,
                          cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess) e = to_f32(s->nodes + s->beg[m] * D, s->nodes32 + s->beg[m] * D, c * D, st);
  }
  if (e == cudaSuccess) e = upload_meta(s, st);
  if (e == cudaSuccess) e = pack_tiles(s, -1, 0, s->cap_total / s->NT, st);
  return e;
}

cudaError_t knn_store_append(KnnStore* s, int mode, const double* rows, long long n, cudaStream_t st) {
  cudaError_t e = cudaSuccess;
  if (mode >= s->n_modes || s->cnt[mode] + n > s->cap[mode]) {
    std::vector<long long> cap = s->cap;
    cap.resize(std::max(s->n_modes, mode + 1), 0);
    const long long need = (mode < s->n_modes ? s->cnt[mode] : 0) + n;
    if (need > cap[mode]) cap[mode] = round_up(std::max(need, 2 * cap[mode]), s->NT);
    e = relayout(s, (int)cap.size(), cap, st);
    if (e != cudaSuccess) return e;
  }
  if (n == 0) return cudaSuccess;
  const long long old = s->cnt[mode];
  // rows may be host or device memory
  e = cudaMemcpyAsync(s->nodes + (s->beg[mode] + old) * s->D, rows, sizeof(double) * n * s->D, cudaMemcpyDefault, st);
  if (e == cudaSuccess)
    e = to_f32(s->nodes + (s->beg[mode] + old) * s->D, s->nodes32 + (s->beg[mode] + old) * s->D, n * s->D, st);
  if (e != cudaSuccess) return e;
  s->cnt[mode] = old + n;
  s->mode_tiles[mode] = (int)((old + n + s->NT - 1) / s->NT);
  s->h_meta[s->n_modes + mode] = s->beg[mode] + old + n;
  e = cudaMemcpyAsync(s->d_end + mode, &s->h_meta[s->n_modes + mode], sizeof(long long), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return e;
  const long long t0 = s->beg[mode] / s->NT;
  return pack_tiles(s, mode, t0 + old / s->NT, t0 + s->mode_tiles[mode], st);
}

// removal by moving the mode's last node into the freed slot (the order
// SingleTree.remove_node leaves, rrtstar_base.py:278-289); repacks the two
// tiles involved
cudaError_t knn_store_remove(KnnStore* s, int mode, long long idx, cudaStream_t st) {
  const long long last = s->cnt[mode] - 1;
  cudaError_t e = cudaSuccess;
  if (idx != last) {
    e = cudaMemcpyAsync(s->nodes + (s->beg[mode] + idx) * s->D, s->nodes + (s->beg[mode] + last) * s->D,
                        sizeof(double) * s->D, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(s->nodes32 + (s->beg[mode] + idx) * s->D, s->nodes32 + (s->beg[mode] + last) * s->D,
                          sizeof(float) * s->D, cudaMemcpyDeviceToDevice, st);
  }
  if (e != cudaSuccess) return e;
  s->cnt[mode] = last;
  s->mode_tiles[mode] = (int)((last + s->NT - 1) / s->NT);
  s->h_meta[s->n_modes + mode] = s->beg[mode] + last;
  e = cudaMemcpyAsync(s->d_end + mode, &s->h_meta[s->n_modes + mode], sizeof(long long), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return e;
  // the tile of the old last row (that row becomes padding) unless the mode
  // no longer uses it, and the tile of idx when it is another one
  const long long t0 = s->beg[mode] / s->NT;
  const long long t_last = last / s->NT, t_idx = idx / s->NT;
  if (t_last < s->mode_tiles[mode]) e = pack_tiles(s, mode, t0 + t_last, t0 + t_last + 1, st);
  if (e == cudaSuccess && idx != last && t_idx != t_last) e = pack_tiles(s, mode, t0 + t_idx, t0 + t_idx + 1, st);
  return e;
}

long long knn_store_count(const KnnStore* s, int mode) { return mode < s->n_modes ? s->cnt[mode] : 0; }
int knn_store_modes(const KnnStore* s) { return s->n_modes; }
bool knn_store_tc(const KnnStore* s) { return s->tc; }
void knn_store_set_path(KnnStore* s, int path) { s->path = path; }

void knn_store_free(KnnStore* s) {
  if (s->nodes) cudaFree(s->nodes);
  if (s->nodes32) cudaFree(s->nodes32);
  s->nodes32 = nullptr;
  if (s->tiles) cudaFree(s->tiles);
  if (s->meta) cudaFree(s->meta);
  if (s->d_qmode) cudaFree(s->d_qmode);
  s->nodes = nullptr;
  s->tiles = nullptr;
  s->meta = nullptr;
  s->d_qmode = nullptr;
}

// scratch for one query launch, owned by the caller (the ABI layer)
struct KnnScratch {
  void* block = nullptr;    // device scratch
  size_t bytes = 0;
  void* host = nullptr;     // pinned staging: the per-call tables go up in one copy
  size_t host_bytes = 0;
};

// queries grouped by mode (order), and work items: query tiles x node-tile
// chunks, about three waves of CTAs, at most 64 chunks per mode
constexpr int kMaxChunkTiles = 128;   // node tiles per chunk when the lists allow it (14 index bits)

struct ItemPlan {
  std::vector<int> order, qcount, qstart, mode_chunks;
  std::vector<KnnItem> items;
  int chunks_max = 1;
  int tpc = 1;              // node tiles per chunk
};

// the index field of the candidate keys: the low bits of a key hold a node's
// index within its chunk (tpc * NT nodes), all ones marks an empty slot
static unsigned key_index_mask(const ItemPlan& pl, int NT) {
  const long long n = (long long)pl.tpc * NT;   // a chunk's nodes: indices 0 .. n - 1 < mask
  unsigned b = 1;
  while ((1ll << b) <= n) b++;
  return (unsigned)((1ll << b) - 1);
}

static void plan_items(const KnnStore* s, const int* h_q_mode, long long Q, int num_sms, ItemPlan* pl) {
  const int n_modes = s->n_modes;
  pl->order.assign(Q, 0);
  pl->qcount.assign(n_modes, 0);
  pl->qstart.assign(n_modes + 1, 0);
  for (long long q = 0; q < Q; q++) pl->qcount[h_q_mode[q]]++;
  for (int m = 0; m < n_modes; m++) pl->qstart[m + 1] = pl->qstart[m] + pl->qcount[m];
  {
    std::vector<int> fill(pl->qstart.begin(), pl->qstart.end() - 1);
    for (long long q = 0; q < Q; q++) pl->order[fill[h_q_mode[q]]++] = (int)q;
  }
  long long units = 0;
  for (int m = 0; m < n_modes; m++) units += (long long)((pl->qcount[m] + kTileM - 1) / kTileM) * s->mode_tiles[m];
  const long long target = std::max(1, 3 * num_sms);
  // at most kMaxChunkTiles node tiles per chunk (unless the 64-list limit
  // below needs more): a chunk's node index fills the low bits of the
  // candidate keys, so this keeps at least 9 of their 23 mantissa bits
  int tpc = (int)std::min<long long>(kMaxChunkTiles, std::max<long long>(1, (units + target - 1) / target));
  int chunks_max = 1;
  for (int m = 0; m < n_modes; m++) chunks_max = std::max(chunks_max, (s->mode_tiles[m] + tpc - 1) / tpc);
  while (chunks_max > 64) {   // at most 64 candidate lists per query
    tpc *= 2;
    chunks_max = 1;
    for (int m = 0; m < n_modes; m++) chunks_max = std::max(chunks_max, (s->mode_tiles[m] + tpc - 1) / tpc);
  }
  pl->chunks_max = chunks_max;
  pl->tpc = tpc;
  pl->items.clear();
  pl->mode_chunks.assign(n_modes, 0);
  for (int m = 0; m < n_modes; m++) {
    if (pl->qcount[m] == 0 || s->mode_tiles[m] == 0) continue;
    const int nch = (s->mode_tiles[m] + tpc - 1) / tpc;
    pl->mode_chunks[m] = nch;
    for (int q0 = 0; q0 < pl->qcount[m]; q0 += kTileM)
      for (int c = 0; c < nch; c++) {
        KnnItem it;
        it.mode = m;
        it.q0 = pl->qstart[m] + q0;
        it.qn = std::min(kTileM, pl->qcount[m] - q0);
        it.tile0 = c * tpc;
        it.tile1 = std::min(s->mode_tiles[m], (c + 1) * tpc);
        it.chunk = c;
        it.pad = 0;
        pl->items.push_back(it);
      }
  }
  // longest items first (CTAs start in index order: the short ones fill the
  // tail of the last wave); the outputs do not depend on the order
  std::stable_sort(pl->items.begin(), pl->items.end(), [](const KnnItem& a, const KnnItem& b) {
    return (long long)(a.tile1 - a.tile0) * a.qn > (long long)(b.tile1 - b.tile0) * b.qn;
  });
}

// Shared memory of a candidate CTA.  The euclidean kernel takes 256 tensor-
// memory columns and about 97 KB (three node-tile buffers), so two CTAs share an SM (a third does not
// fit in shared memory, so no CTA waits for columns); the per-agent kernel
// takes all 512 columns and is held to one CTA per SM by asking for at least
// 120 KB, so two CTAs never wait on each other for the columns.
static size_t tc_smem_bytes(const KnnStore* s) {
  const int NT = s->dev.NT;
  const bool eucl = s->dev.fmt == KNN_FMT_EUCL;
  const int nthreads = 128 * (eucl ? TcSplit<KNN_FMT_EUCL>::S : TcSplit<KNN_FMT_AGENT>::S);
  const size_t need = 1024 + 2 * (size_t)kTileM * kRowBytes + kStagesB * (size_t)NT * kRowBytes +
                      32 * sizeof(float) * (size_t)nthreads;
  return eucl ? need : std::max<size_t>(need, 120 * 1024);
}

// the attribute is per function: raise it once, to the opt-in limit less the
// kernel's static shared memory
template <int FMT, bool RAD>
static void raise_smem_limit() {
  static bool done = false;
  if (done) return;
  int dev = 0, optin = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  cudaFuncAttributes fa;
  if (cudaFuncGetAttributes(&fa, knn_tc_kernel<FMT, RAD>) == cudaSuccess)
    cudaFuncSetAttribute(knn_tc_kernel<FMT, RAD>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         optin - (int)fa.sharedSizeBytes);
  cudaGetLastError();
  done = true;
}

static cudaError_t knn_split_query(KnnStore* s, KnnScratch* scr, const double* d_qs, long long Q, const int* h_q_mode,
                                   int k, long long* d_idx, double* d_dist, int num_sms, cudaStream_t st,
                                   const long long* h_list = nullptr, long long n_list = 0);

cudaError_t knn_query(KnnStore* s, const double* d_qs, long long Q, const int* h_q_mode, int k, long long* d_idx,
                      double* d_dist, KnnScratch* scr, int num_sms, int* n_fallback_out, cudaStream_t st) {
  const int n_modes = s->n_modes;
  ItemPlan pl;
  plan_items(s, h_q_mode, Q, num_sms, &pl);
  // the keys' index field must stay within the 23 mantissa bits: a chunk of
  // 2^23 nodes or more (a mode of over 500 million nodes) goes to the exact
  // node-parallel kernels instead
  const unsigned imask = key_index_mask(pl, s->dev.NT);
  *n_fallback_out = 0;
  if (imask > 0x7fffffu) return knn_split_query(s, scr, d_qs, Q, h_q_mode, k, d_idx, d_dist, num_sms, st);
  const std::vector<int>& order = pl.order;
  const std::vector<KnnItem>& items = pl.items;
  const std::vector<int>& mode_chunks = pl.mode_chunks;
  const int chunks_max = pl.chunks_max;
  // scratch: order, q_mode, items, mode_chunks, cand lists, eps, fallback list, counters
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  const size_t b_order = al(sizeof(int) * std::max<long long>(Q, 1));
  const size_t b_qmode = b_order;
  const size_t b_items = al(sizeof(KnnItem) * std::max<size_t>(items.size(), 1));
  const size_t b_mch = al(sizeof(int) * std::max(n_modes, 1));
  const size_t b_g = al(sizeof(unsigned) * std::max<long long>(Q, 1));
  const size_t b_cd = al(sizeof(float) * std::max<long long>(Q, 1) * chunks_max * kKeep);
  const size_t b_ci = b_cd;
  const size_t b_cb = al(sizeof(float) * std::max<long long>(Q, 1) * chunks_max);
  const size_t b_eps = al(sizeof(float) * std::max<long long>(Q, 1));
  const size_t b_fb = al(sizeof(long long) * std::max<long long>(Q, 1));
  const size_t b_ctr = 256;
  const size_t need = b_order + b_qmode + b_items + b_mch + b_g + b_cd + b_ci + b_cb + b_eps + b_fb + b_ctr;
  if (scr->bytes < need) {
    if (scr->block) cudaFree(scr->block);
    scr->block = nullptr;
    cudaError_t e = cudaMalloc(&scr->block, need);
    if (e != cudaSuccess) { scr->bytes = 0; return e; }
    scr->bytes = need;
  }
  unsigned char* p = (unsigned char*)scr->block;
  int* d_order = (int*)p; p += b_order;
  int* d_qmode = (int*)p; p += b_qmode;
  KnnItem* d_items = (KnnItem*)p; p += b_items;
  int* d_mch = (int*)p; p += b_mch;
  unsigned* d_g = (unsigned*)p; p += b_g;
  float* d_cd = (float*)p; p += b_cd;
  int* d_ci = (int*)p; p += b_ci;
  float* d_cb = (float*)p; p += b_cb;
  float* d_eps = (float*)p; p += b_eps;
  long long* d_fb = (long long*)p; p += b_fb;
  int* d_ctr = (int*)p;   // [0] fallback count, [1] error bits
  // order, query modes, items, chunk counts and the shared thresholds' start
  // values sit back to back in the device block: stage them in pinned memory
  // with the same layout, one copy
  const size_t b_up = b_order + b_qmode + b_items + b_mch + b_g;
  if (scr->host_bytes < b_up + 256) {
    if (scr->host) cudaFreeHost(scr->host);
    scr->host = nullptr;
    scr->host_bytes = 0;
    cudaError_t e = cudaMallocHost(&scr->host, b_up + 256);
    if (e != cudaSuccess) return e;
    scr->host_bytes = b_up + 256;
  }
  unsigned char* hp = (unsigned char*)scr->host;
  std::memcpy(hp, order.data(), sizeof(int) * Q);
  std::memcpy(hp + b_order, h_q_mode, sizeof(int) * Q);
  if (!items.empty()) std::memcpy(hp + b_order + b_qmode, items.data(), sizeof(KnnItem) * items.size());
  std::memcpy(hp + b_order + b_qmode + b_items, mode_chunks.data(), sizeof(int) * n_modes);
  std::memset(hp + b_order + b_qmode + b_items + b_mch, 0x7f, b_g);   // 0x7f7f7f7f: a huge FP32 threshold
  int* h_ctr = (int*)(hp + b_up);
  cudaError_t e = cudaMemcpyAsync(d_order, hp, b_up, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(d_ctr, 0, 256, st);
  if (e != cudaSuccess) return e;
  const size_t smem = tc_smem_bytes(s);
  raise_smem_limit<KNN_FMT_EUCL, false>();
  raise_smem_limit<KNN_FMT_AGENT, false>();
  if (!items.empty()) {
    if (s->dev.fmt == KNN_FMT_EUCL) {
      knn_tc_kernel<KNN_FMT_EUCL, false><<<(int)items.size(), 128 * TcSplit<KNN_FMT_EUCL>::S, smem, st>>>(s->dev, d_qs, d_order, d_items, chunks_max,
                                                                         d_cd, d_ci, d_cb, d_g, d_eps, d_ctr + 1, RadOut{}, imask);
    } else {
      knn_tc_kernel<KNN_FMT_AGENT, false><<<(int)items.size(), 128 * TcSplit<KNN_FMT_AGENT>::S, smem, st>>>(s->dev, d_qs, d_order, d_items, chunks_max,
                                                                          d_cd, d_ci, d_cb, d_g, d_eps, d_ctr + 1, RadOut{}, imask);
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  const int mgrid = (int)std::min<long long>((Q + 3) / 4, (long long)num_sms * 16);
  knn_merge_kernel<<<std::max(mgrid, 1), 32 * kMergeWarps, 0, st>>>(d_qs, Q, d_qmode, s->nodes, s->d_beg, s->d_end, d_mch, chunks_max,
                                                       d_cd, d_ci, d_cb, d_eps, s->slices, s->metric, k, d_idx, d_dist, d_fb,
                                                       d_ctr, imask);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  e = cudaMemcpyAsync(h_ctr, d_ctr, sizeof(int) * 2, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return e;
  *n_fallback_out = h_ctr[0];
  if (h_ctr[1]) return cudaErrorLaunchTimeout;
  if (h_ctr[0] > 0) {   // uncertified queries: node-parallel exact (the list leaves the scratch first)
    std::vector<long long> fb(h_ctr[0]);
    e = cudaMemcpyAsync(fb.data(), d_fb, sizeof(long long) * fb.size(), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e == cudaSuccess)
      e = knn_split_query(s, scr, d_qs, Q, h_q_mode, k, d_idx, d_dist, num_sms, st, fb.data(), (long long)fb.size());
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// FP64 work (node rows x coordinates) below which a batch takes the
// node-parallel exact path even where the tensor-core path applies: about
// 150,000 distances in 28-D, some 10 us of the GPU's FP64 rate, less than the
// tensor-core path's per-tile setup for a handful of queries
constexpr long long kSmallWork = 1ll << 22;

static long long batch_work(const KnnStore* s, const int* h_q_mode, long long Q) {
  if (s->path == 1) return kSmallWork + 1;
  if (s->path == 2) return 0;
  long long w = 0;
  for (long long q = 0; q < Q; q++) w += s->cnt[h_q_mode[q]];
  return w * std::max(s->D, 1);
}

// pinned + device scratch of at least the given sizes
static cudaError_t scratch_reserve(KnnScratch* scr, size_t dev_bytes, size_t host_bytes) {
  if (scr->bytes < dev_bytes) {
    if (scr->block) cudaFree(scr->block);
    scr->block = nullptr;
    scr->bytes = 0;
    cudaError_t e = cudaMalloc(&scr->block, dev_bytes);
    if (e != cudaSuccess) return e;
    scr->bytes = dev_bytes;
  }
  if (scr->host_bytes < host_bytes) {
    if (scr->host) cudaFreeHost(scr->host);
    scr->host = nullptr;
    scr->host_bytes = 0;
    cudaError_t e = cudaMallocHost(&scr->host, host_bytes);
    if (e != cudaSuccess) return e;
    scr->host_bytes = host_bytes;
  }
  return cudaSuccess;
}

// node-parallel exact k nearest: items (query, 256-node chunk), then a merge;
// with `h_list` only the listed queries (n_list of them) are answered
static cudaError_t knn_split_query(KnnStore* s, KnnScratch* scr, const double* d_qs, long long Q, const int* h_q_mode,
                                   int k, long long* d_idx, double* d_dist, int num_sms, cudaStream_t st,
                                   const long long* h_list, long long n_list) {
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  const long long L = h_list ? n_list : Q;
  const size_t b_qm = al(sizeof(int) * std::max<long long>(L, 1)), b_off = al(sizeof(long long) * (L + 1));
  const size_t b_map = h_list ? al(sizeof(long long) * std::max<long long>(L, 1)) : 0;
  const size_t b_up = b_qm + b_off + b_map;
  cudaError_t e = scratch_reserve(scr, 0, b_up);
  if (e != cudaSuccess) return e;
  unsigned char* hp = (unsigned char*)scr->host;
  int* hqm = (int*)hp;
  for (long long l = 0; l < L; l++) hqm[l] = h_q_mode[h_list ? h_list[l] : l];
  long long* ioff = (long long*)(hp + b_qm);
  ioff[0] = 0;
  for (long long l = 0; l < L; l++) ioff[l + 1] = ioff[l] + (s->cnt[hqm[l]] + kSplitNodes - 1) / kSplitNodes;
  if (h_list) std::memcpy(hp + b_qm + b_off, h_list, sizeof(long long) * L);
  const long long n_items = ioff[L];
  const size_t b_cand = al(sizeof(long long) * std::max<long long>(n_items, 1) * k);
  e = scratch_reserve(scr, b_up + 2 * b_cand, 0);
  if (e != cudaSuccess) return e;
  unsigned char* p = (unsigned char*)scr->block;
  const int* d_qm = (const int*)p;
  const long long* d_ioff = (const long long*)(p + b_qm);
  const long long* d_map = h_list ? (const long long*)(p + b_qm + b_off) : nullptr;
  long long* d_ck = (long long*)(p + b_up);
  long long* d_ci = (long long*)(p + b_up + b_cand);
  e = cudaMemcpyAsync(p, hp, b_up, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return e;
  if (n_items > 0) {
    const int grid = (int)std::min<long long>((n_items + 3) / 4, (long long)num_sms * 16);
    if (k <= 16)
      knn_split_kernel<16><<<grid, 128, 0, st>>>(d_qs, d_map, L, d_qm, d_ioff, s->nodes, s->d_beg, s->d_end,
                                                 s->slices, s->metric, k, d_ck, d_ci);
    else
      knn_split_kernel<kKnnMaxK><<<grid, 128, 0, st>>>(d_qs, d_map, L, d_qm, d_ioff, s->nodes, s->d_beg, s->d_end,
                                                       s->slices, s->metric, k, d_ck, d_ci);
  }
  const int mgrid = (int)std::max<long long>(1, std::min<long long>((L + 3) / 4, (long long)num_sms * 16));
  if (k <= 16)
    knn_split_merge_kernel<16><<<mgrid, 128, 0, st>>>(d_map, L, d_ioff, k, d_ck, d_ci, d_idx, d_dist);
  else
    knn_split_merge_kernel<kKnnMaxK><<<mgrid, 128, 0, st>>>(d_map, L, d_ioff, k, d_ck, d_ci, d_idx, d_dist);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);   // the pinned tables are reused by the next call
  return e;
}

// node-parallel k nearest with the FP32 candidate pass (euclidean and max
// over agents, k <= 31): candidates, certified FP64 re-rank, and the FP64
// kernels for the queries whose certificate fails
static cudaError_t knn_split32_query(KnnStore* s, KnnScratch* scr, const double* d_qs, long long Q,
                                     const int* h_q_mode, int k, long long* d_idx, double* d_dist, int num_sms,
                                     int* n_fallback, cudaStream_t st) {
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  const size_t b_qm = al(sizeof(int) * std::max<long long>(Q, 1)), b_off = al(sizeof(long long) * (Q + 1));
  const size_t b_up = b_qm + b_off;
  cudaError_t e = scratch_reserve(scr, 0, b_up + 256);
  if (e != cudaSuccess) return e;
  unsigned char* hp = (unsigned char*)scr->host;
  std::memcpy(hp, h_q_mode, sizeof(int) * Q);
  long long* ioff = (long long*)(hp + b_qm);
  ioff[0] = 0;
  for (long long q = 0; q < Q; q++) ioff[q + 1] = ioff[q] + (s->cnt[h_q_mode[q]] + kSplitNodes - 1) / kSplitNodes;
  const long long n_items = ioff[Q];
  const size_t b_ck = al(sizeof(float) * std::max<long long>(n_items, 1) * k);
  const size_t b_it = al(sizeof(float) * std::max<long long>(n_items, 1));
  const size_t b_fb = al(sizeof(long long) * std::max<long long>(Q, 1));
  e = scratch_reserve(scr, b_up + 2 * b_ck + 2 * b_it + b_fb + 256, 0);
  if (e != cudaSuccess) return e;
  unsigned char* p = (unsigned char*)scr->block;
  const int* d_qm = (const int*)p;
  const long long* d_ioff = (const long long*)(p + b_qm);
  float* d_ck = (float*)(p + b_up);
  int* d_ci = (int*)(p + b_up + b_ck);
  float* d_next = (float*)(p + b_up + 2 * b_ck);
  float* d_band = (float*)(p + b_up + 2 * b_ck + b_it);
  long long* d_fb = (long long*)(p + b_up + 2 * b_ck + 2 * b_it);
  int* d_ctr = (int*)(p + b_up + 2 * b_ck + 2 * b_it + b_fb);
  int* h_ctr = (int*)(hp + b_up);
  e = cudaMemcpyAsync(p, hp, b_up, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(d_ctr, 0, sizeof(int), st);
  if (e != cudaSuccess) return e;
  const int grid = (int)std::max<long long>(1, std::min<long long>((n_items + kSplitWarps - 1) / kSplitWarps,
                                                                    (long long)num_sms * 16));
  const int mgrid = (int)std::max<long long>(1, std::min<long long>((Q + kSplitWarps - 1) / kSplitWarps,
                                                                     (long long)num_sms * 16));
  if (k <= 15) {
    if (n_items > 0)
      knn_split32_kernel<16><<<grid, 32 * kSplitWarps, 0, st>>>(d_qs, nullptr, Q, d_qm, d_ioff, s->nodes32, s->d_beg,
                                                                s->d_end, s->slices, s->metric, k, d_ck, d_ci, d_next,
                                                                d_band);
    knn_split32_merge_kernel<16><<<mgrid, 32 * kSplitWarps, 0, st>>>(d_qs, nullptr, Q, d_qm, d_ioff, s->nodes, s->d_beg,
                                                                     s->d_end, s->slices, s->metric, k, d_ck, d_ci,
                                                                     d_next, d_band, d_idx, d_dist, d_fb, d_ctr);
  } else {
    if (n_items > 0)
      knn_split32_kernel<32><<<grid, 32 * kSplitWarps, 0, st>>>(d_qs, nullptr, Q, d_qm, d_ioff, s->nodes32, s->d_beg,
                                                                s->d_end, s->slices, s->metric, k, d_ck, d_ci, d_next,
                                                                d_band);
    knn_split32_merge_kernel<32><<<mgrid, 32 * kSplitWarps, 0, st>>>(d_qs, nullptr, Q, d_qm, d_ioff, s->nodes, s->d_beg,
                                                                     s->d_end, s->slices, s->metric, k, d_ck, d_ci,
                                                                     d_next, d_band, d_idx, d_dist, d_fb, d_ctr);
  }
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(h_ctr, d_ctr, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return e;
  *n_fallback = h_ctr[0];
  if (h_ctr[0] > 0) {   // uncertified: the FP64 kernels (the list leaves the scratch first)
    std::vector<long long> fb(h_ctr[0]);
    e = cudaMemcpyAsync(fb.data(), d_fb, sizeof(long long) * fb.size(), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e == cudaSuccess)
      e = knn_split_query(s, scr, d_qs, Q, h_q_mode, k, d_idx, d_dist, num_sms, st, fb.data(), (long long)fb.size());
  }
  return e;
}

// k nearest on the store: the node-parallel exact path for small batches,
// the tensor-core path for its formats and k <= 16, else the exact
// warp-per-query kernel
cudaError_t knn_store_query(KnnStore* s, KnnScratch* scr, const double* d_qs, long long Q, const int* h_q_mode, int k,
                            long long* d_idx, double* d_dist, int num_sms, int* used_tc, int* n_fallback,
                            cudaStream_t st) {
  *used_tc = 0;
  *n_fallback = 0;
  const bool small = batch_work(s, h_q_mode, Q) <= kSmallWork;
  if (small || (!(s->tc && k <= 16) && Q < 2048)) {
    // (the candidate kernel stages the query in 64 floats of shared memory)
    if ((s->metric == MRMG_METRIC_EUCLIDEAN || s->metric == MRMG_METRIC_MAX_EUCLIDEAN) && k <= 31 && s->D <= 64)
      return knn_split32_query(s, scr, d_qs, Q, h_q_mode, k, d_idx, d_dist, num_sms, n_fallback, st);
    return knn_split_query(s, scr, d_qs, Q, h_q_mode, k, d_idx, d_dist, num_sms, st);
  }
  if (s->tc && k <= 16) {
    *used_tc = 1;
    cudaError_t e = knn_query(s, d_qs, Q, h_q_mode, k, d_idx, d_dist, scr, num_sms, n_fallback, st);
    return e;
  }
  if (s->qmode_cap < Q) {
    if (s->d_qmode) cudaFree(s->d_qmode);
    s->d_qmode = nullptr;
    s->qmode_cap = 0;
    cudaError_t e = cudaMalloc(&s->d_qmode, sizeof(int) * Q);
    if (e != cudaSuccess) return e;
    s->qmode_cap = Q;
  }
  cudaError_t e = cudaMemcpyAsync(s->d_qmode, h_q_mode, sizeof(int) * Q, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = knn_exact(d_qs, Q, s->d_qmode, nullptr, 0, s->nodes, s->d_beg, s->d_end, s->slices, s->metric, k, d_idx, d_dist,
                  num_sms, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return e;
}

// ---------------------------------------------------------------------------
// radius queries (host)
// ---------------------------------------------------------------------------
struct NearState {
  KnnScratch scr;
  // the last query, kept for near_fetch
  const double* qs = nullptr;
  long long Q = 0;
  const double* nodes = nullptr;
  const long long* mode_beg = nullptr;
  SliceTab t{};
  int metric = 0;
  const int* qmode = nullptr;
  const long long* woff = nullptr;
  const unsigned* bits = nullptr;
  const int* stage = nullptr;
  const long long* offs = nullptr;
  long long total = 0;
};

NearState* near_state_new() { return new NearState(); }
void near_state_delete(NearState* ns) {
  if (!ns) return;
  if (ns->scr.block) cudaFree(ns->scr.block);
  if (ns->scr.host) cudaFreeHost(ns->scr.host);
  delete ns;
}

static int near_grid(long long Q, int num_sms) {
  return (int)std::max<long long>(1, std::min<long long>((Q + kNearWarps - 1) / kNearWarps, (long long)num_sms * 16));
}

// f32 value >= x^2 (x >= 0 finite), +inf for +inf, -1 for x < 0 or NaN (nothing within)
static float rad2_up(double x) {
  if (!(x >= 0.0)) return -1.f;
  const double x2 = x * x;
  if (x2 > 3.0e38) return __builtin_huge_valf();
  const float f = (float)x2;
  return (double)f >= x2 ? f : std::nextafter(f, __builtin_huge_valf());
}

cudaError_t near_query(NearState* ns, KnnStore* s, const double* d_qs, long long Q, const int* h_q_mode,
                       const double* h_radius, double add_eps, long long* d_offsets, long long* d_idx, double* d_dist,
                       long long cap, int num_sms, long long* total_out, cudaStream_t st) {
  const int n_modes = s->n_modes;
  const bool small = batch_work(s, h_q_mode, Q) <= kSmallWork;
  KnnStore* tc = s->tc && !small ? s : nullptr;   // else every node is checked in FP64, node-parallel
  const double* nodes = s->nodes;
  const SliceTab& t = s->slices;
  const int metric = s->metric;
  // words of each query's bitmap: whole node tiles on the tensor-core path
  // (every word is written by the candidate kernel), else ceil(M / 32)
  std::vector<long long> words(n_modes);
  for (int m = 0; m < n_modes; m++)
    words[m] = tc ? (long long)s->mode_tiles[m] * s->NT / 32 : (s->cnt[m] + 31) / 32;
  ItemPlan pl;
  if (tc) plan_items(tc, h_q_mode, Q, num_sms, &pl);
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  const size_t b_order = al(sizeof(int) * std::max<long long>(Q, 1));
  const size_t b_qmode = b_order;
  const size_t b_items = al(sizeof(KnnItem) * std::max<size_t>(pl.items.size(), 1));
  const size_t b_woff = al(sizeof(long long) * (Q + 1));
  const size_t b_rp = al(sizeof(double) * std::max<long long>(Q, 1));
  const size_t b_rad2 = al(sizeof(float) * std::max<long long>(Q, 1));
  const size_t b_up = b_order + b_qmode + b_items + b_woff + b_rp + b_rad2;
  // host tables
  if (ns->scr.host_bytes < b_up + 256) {
    if (ns->scr.host) cudaFreeHost(ns->scr.host);
    ns->scr.host = nullptr;
    ns->scr.host_bytes = 0;
    cudaError_t e = cudaMallocHost(&ns->scr.host, b_up + 256);
    if (e != cudaSuccess) return e;
    ns->scr.host_bytes = b_up + 256;
  }
  unsigned char* hp = (unsigned char*)ns->scr.host;
  long long* h_woff = (long long*)(hp + b_order + b_qmode + b_items);
  double* h_rp = (double*)(hp + b_order + b_qmode + b_items + b_woff);
  float* h_rad2 = (float*)(hp + b_order + b_qmode + b_items + b_woff + b_rp);
  h_woff[0] = 0;
  for (long long q = 0; q < Q; q++) {
    h_woff[q + 1] = h_woff[q] + words[h_q_mode[q]];
    h_rp[q] = h_radius[q] + add_eps;     // the reference's r += eps, in FP64
    h_rad2[q] = rad2_up(h_rp[q]);
  }
  const long long Wtot = h_woff[Q];
  if (tc) std::memcpy(hp, pl.order.data(), sizeof(int) * Q);
  std::memcpy(hp + b_order, h_q_mode, sizeof(int) * Q);
  if (!pl.items.empty()) std::memcpy(hp + b_order + b_qmode, pl.items.data(), sizeof(KnnItem) * pl.items.size());
  long long* h_ctr = (long long*)(hp + b_up);
  // device: the uploaded tables, then bitmap, counts, offsets, counters
  const size_t b_bits = al(sizeof(unsigned) * std::max<long long>(Wtot, 1));
  const size_t b_cnt = al(sizeof(long long) * std::max<long long>(Q, 1));
  const size_t b_offs = al(sizeof(long long) * (Q + 1));
  const size_t b_q32 = al(sizeof(float) * std::max<long long>(Q, 1) * std::max(s->D, 1));
  const size_t b_stage = al(sizeof(int) * std::max<long long>(Q, 1) * kNearStage);
  const size_t need = b_up + b_bits + b_cnt + b_offs + 256 + b_q32 + b_stage;
  if (ns->scr.bytes < need) {
    if (ns->scr.block) cudaFree(ns->scr.block);
    ns->scr.block = nullptr;
    ns->scr.bytes = 0;
    cudaError_t e = cudaMalloc(&ns->scr.block, need);
    if (e != cudaSuccess) return e;
    ns->scr.bytes = need;
  }
  unsigned char* p = (unsigned char*)ns->scr.block;
  int* d_order = (int*)p;
  int* d_qmode = (int*)(p + b_order);
  KnnItem* d_items = (KnnItem*)(p + b_order + b_qmode);
  long long* d_woff = (long long*)(p + b_order + b_qmode + b_items);
  double* d_rp = (double*)(p + b_order + b_qmode + b_items + b_woff);
  float* d_rad2 = (float*)(p + b_order + b_qmode + b_items + b_woff + b_rp);
  unsigned* d_bits = (unsigned*)(p + b_up);
  long long* d_cnt = (long long*)(p + b_up + b_bits);
  long long* d_offs = (long long*)(p + b_up + b_bits + b_cnt);
  long long* d_ctr = (long long*)(p + b_up + b_bits + b_cnt + b_offs);   // [0] total, [1] error bits
  float* d_q32 = (float*)(p + b_up + b_bits + b_cnt + b_offs + 256);
  int* d_stage = (int*)(p + b_up + b_bits + b_cnt + b_offs + 256 + b_q32);
  cudaError_t e = cudaMemcpyAsync(p, hp, b_up, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(d_ctr, 0, 256, st);
  if (e == cudaSuccess) e = to_f32(d_qs, d_q32, Q * s->D, st);
  if (e != cudaSuccess) return e;
  if (tc && !pl.items.empty()) {
    const size_t smem = tc_smem_bytes(tc);
    const RadOut ro{d_bits, d_woff, d_rad2};
    if (s->dev.fmt == KNN_FMT_EUCL) {
      raise_smem_limit<KNN_FMT_EUCL, true>();
      knn_tc_kernel<KNN_FMT_EUCL, true><<<(int)pl.items.size(), 128 * TcSplit<KNN_FMT_EUCL>::S, smem, st>>>(
          tc->dev, d_qs, d_order, d_items, pl.chunks_max, nullptr, nullptr, nullptr, nullptr, nullptr,
          (int*)(d_ctr + 1), ro, 0u);
    } else {
      raise_smem_limit<KNN_FMT_AGENT, true>();
      knn_tc_kernel<KNN_FMT_AGENT, true><<<(int)pl.items.size(), 128 * TcSplit<KNN_FMT_AGENT>::S, smem, st>>>(
          tc->dev, d_qs, d_order, d_items, pl.chunks_max, nullptr, nullptr, nullptr, nullptr, nullptr,
          (int*)(d_ctr + 1), ro, 0u);
    }
  }
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const int grid = near_grid(Q, num_sms);
  if (tc) {
    near_exact_kernel<<<grid, 32 * kNearWarps, 0, st>>>(d_qs, d_q32, Q, d_qmode, nodes, s->nodes32, s->d_beg,
                                                        s->d_end, t, metric, d_rp, d_woff, d_bits, d_cnt, d_stage);
  } else {
    e = cudaMemsetAsync(d_cnt, 0, sizeof(long long) * Q, st);
    if (e != cudaSuccess) return e;
    if (Wtot > 0) {
      const int g2 = (int)std::min<long long>((Wtot + 3) / 4, (long long)num_sms * 16);
      near_split_kernel<<<g2, 128, 0, st>>>(d_qs, d_q32, Q, d_qmode, nodes, s->nodes32, s->d_beg, s->d_end, t, metric,
                                            d_rp, d_woff, d_bits, (unsigned long long*)d_cnt);
    }
  }
  near_scan_kernel<<<1, 1024, 0, st>>>(d_cnt, Q, d_offsets, d_offs, d_ctr);
  if (cap > 0) {
    near_emit_kernel<<<grid, 32 * kNearWarps, 0, st>>>(Q, d_woff, d_bits, tc ? d_stage : nullptr, d_offs, cap, d_idx);
    if (d_dist)
      near_dist_kernel<<<num_sms * 4, 256, 0, st>>>(d_qs, Q, d_qmode, nodes, s->d_beg, t, metric, d_offs, cap, d_idx,
                                                    d_dist);
  }
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(h_ctr, d_ctr, 2 * sizeof(long long), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return e;
  if (h_ctr[1]) return cudaErrorLaunchTimeout;
  ns->qs = d_qs;
  ns->Q = Q;
  ns->nodes = nodes;
  ns->mode_beg = s->d_beg;
  ns->t = t;
  ns->metric = metric;
  ns->qmode = d_qmode;
  ns->woff = d_woff;
  ns->bits = d_bits;
  ns->stage = tc ? d_stage : nullptr;
  ns->offs = d_offs;
  ns->total = h_ctr[0];
  *total_out = h_ctr[0];
  return cudaSuccess;
}

cudaError_t near_fetch(NearState* ns, long long* d_idx, double* d_dist, long long cap, int num_sms, cudaStream_t st) {
  if (ns->Q == 0 || cap <= 0) return cudaSuccess;
  near_emit_kernel<<<near_grid(ns->Q, num_sms), 32 * kNearWarps, 0, st>>>(ns->Q, ns->woff, ns->bits, ns->stage,
                                                                            ns->offs, cap, d_idx);
  if (d_dist)
    near_dist_kernel<<<num_sms * 4, 256, 0, st>>>(ns->qs, ns->Q, ns->qmode, ns->nodes, ns->mode_beg, ns->t,
                                                  ns->metric, ns->offs, cap, d_idx, d_dist);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return e;
}

long long near_last_total(const NearState* ns) { return ns->total; }

KnnStore* knn_store_new() { return new KnnStore(); }
void knn_store_delete(KnnStore* s) {
  if (s) { knn_store_free(s); delete s; }
}
KnnScratch* knn_scratch_new() { return new KnnScratch(); }
void knn_scratch_delete(KnnScratch* s) {
  if (s) {
    if (s->block) cudaFree(s->block);
    if (s->host) cudaFreeHost(s->host);
    delete s;
  }
}

}  // namespace mrmg
