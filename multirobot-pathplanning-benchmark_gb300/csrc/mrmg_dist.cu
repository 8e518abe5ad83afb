// mrmg_dist.cu -- configuration distances and costs
// (problems/core/configuration.py): batch_config_dist / NpConfiguration._batch_dist
// (:303-349), compute_sliced_euclidean_dists (:101-126), the sum / max /
// max+w*sum / abs-max reductions (:129-219) and batch_config_cost (:437-510).
//
// Every value is the FP64 result of the reference's own operation sequence
// (sequential sums of d*d without fusion, IEEE sqrt, strict '>' maxima), so
// outputs are bit-identical to the reference.  These kernels are bound by the
// FP64 pipe on GB300 (a few FP64 operations per output byte), not by HBM.
#include "mrmg_internal.cuh"

namespace mrmg {

namespace {

constexpr int kQTile = 16;        // queries per CTA (shared memory)
constexpr int kMaxTileD = 128;    // coordinates staged per query

// out[q, m] = dist(queries[q] - nodes[m])
__global__ void dist_matrix_kernel(const double* __restrict__ qs, long long Q, const double* __restrict__ nodes,
                                   long long M, SliceTab t, int metric, double* __restrict__ out) {
  __shared__ double sq[kQTile * kMaxTileD];
  const int D = t.D;
  const long long q0 = (long long)blockIdx.y * kQTile;
  const int nq = (int)min((long long)kQTile, Q - q0);
  const bool staged = D <= kMaxTileD;
  if (staged)
    for (int i = threadIdx.x; i < nq * D; i += blockDim.x) sq[i] = qs[q0 * D + i];
  __syncthreads();
  for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < M; m += (long long)gridDim.x * blockDim.x) {
    const double* x = nodes + m * D;
    for (int j = 0; j < nq; j++) {
      const double* qq = staged ? sq + j * D : qs + (q0 + j) * D;
      auto d = [&](int k) { return __dsub_rn(qq[k], x[k]); };
      out[(q0 + j) * M + m] = dist_of(t, metric, d);
    }
  }
}

// _batch_config_cost_impl on diff rows; mode 0: starts[0] - ends[m],
// 1: starts[m] - ends[m], 2: starts[m+1] - starts[m] (path form)
__global__ void cost_kernel(const double* __restrict__ a, const double* __restrict__ b, long long M, SliceTab t,
                            int cmetric, int red, double w, int mode, double* __restrict__ out) {
  const int D = t.D;
  for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < M; m += (long long)gridDim.x * blockDim.x) {
    const double* x;
    const double* y;
    if (mode == 0) { x = a; y = b + m * D; }
    else if (mode == 1) { x = a + m * D; y = b + m * D; }
    else { x = a + (m + 1) * D; y = a + m * D; }
    double mx = 0.0, sm = 0.0;
    for (int i = 0; i < t.A; i++) {
      double v;
      if (cmetric == MRMG_COST_EUCLIDEAN) {
        double acc = 0.0;
        for (int k = t.s[i]; k < t.e[i]; k++) { double d = __dsub_rn(x[k], y[k]); acc = __dadd_rn(acc, __dmul_rn(d, d)); }
        v = sqrt(acc);
      } else {
        // np.max(np.abs(diff[:, s:e])): exact; a NaN anywhere propagates
        v = fabs(__dsub_rn(x[t.s[i]], y[t.s[i]]));
        for (int k = t.s[i] + 1; k < t.e[i]; k++) { double d = fabs(__dsub_rn(x[k], y[k])); if (d > v || d != d) v = d; }
      }
      if (red == MRMG_REDUCE_MAX) {              // compute_max_sum_reduction (:150-171)
        if (i == 0) { mx = v; sm = v; }
        else { if (v > mx) mx = v; sm = __dadd_rn(sm, v); }
      } else {                                   // compute_sum_reduction (:129-147)
        sm = __dadd_rn(sm, v);
      }
    }
    out[m] = red == MRMG_REDUCE_MAX ? __dadd_rn(mx, __dmul_rn(w, sm)) : sm;
  }
}

int grid_for(long long n, int threads, int cap) {
  long long g = (n + threads - 1) / threads;
  if (g < 1) g = 1;
  return (int)(g < cap ? g : cap);
}

}  // namespace

cudaError_t dist_matrix(const double* qs, long long Q, const double* nodes, long long M, const SliceTab& t, int metric,
                        double* out, int num_sms, cudaStream_t st) {
  if (Q == 0 || M == 0) return cudaSuccess;
  const int threads = 256;
  long long qtiles = (Q + kQTile - 1) / kQTile;
  int gx = grid_for(M, threads, num_sms * 8);
  if (qtiles > 65535) return cudaErrorInvalidValue;
  dim3 grid(gx, (unsigned)qtiles);
  dist_matrix_kernel<<<grid, threads, 0, st>>>(qs, Q, nodes, M, t, metric, out);
  return cudaGetLastError();
}

cudaError_t batch_cost(const double* a, const double* b, long long M, const SliceTab& t, int cmetric, int red, double w,
                       int mode, double* out, int num_sms, cudaStream_t st) {
  if (M <= 0) return cudaSuccess;
  cost_kernel<<<grid_for(M, 256, num_sms * 16), 256, 0, st>>>(a, b, M, t, cmetric, red, w, mode, out);
  return cudaGetLastError();
}

}  // namespace mrmg
