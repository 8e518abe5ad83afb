// mrmg_abstract.cu -- collision kernels for abstract point-agent scenes
// (problems/abstract_env.py: Sphere :41-58, Rectangle :61-109,
// AbstractEnvironment.is_collision_free :255-276, is_edge_collision_free
// :301-354).
//
// Two passes per call:
//  pass 1  FP32 classification of every configuration against a band that
//          bounds the FP32 error: definitely colliding, definitely free, or
//          pending.  An item with a definite collision is decided; an item
//          whose only doubt is a pending configuration is queued.
//  pass 2  the queued items again, with each pending configuration decided
//          by the exact FP64 restatement of the reference's arithmetic.
#include "mrmg_internal.cuh"

namespace mrmg {
namespace {

template <typename T>
__device__ __forceinline__ double ld(const void* p, long long i) {
  return (double)((const T*)p)[i];
}

__device__ __forceinline__ double ldq(const void* p, int dtype, long long i) {
  return dtype == MRMG_F32 ? ld<float>(p, i) : ld<double>(p, i);
}

// ---------------------------------------------------------------------------
// FP32 classification of one configuration; coordinates come from `acc(k)`.
// ---------------------------------------------------------------------------
template <class Acc>
__device__ uint8_t classify32(const AbstractDev& s, Acc acc) {
  float qf[kMaxAgents * kMaxAgentDim];
  float qmax = 0.f;
  bool bad = false;
  for (int k = 0; k < s.D; k++) {
    double v = acc(k);
    bad |= !(fabs(v) <= 1e30);            // NaN, inf or huge: exact path decides
    float f = (float)v;
    qf[k] = f;
    qmax = fmaxf(qmax, fabsf(f));
  }
  if (bad) return V_PENDING;
  const float delta = s.delta_k * (qmax + s.omax);
  bool unc = false;
  const int A = s.A, dim = s.dim;
  // agent - agent  (abstract_env.py:261-268)
  for (int i = 0; i < A; i++)
    for (int j = i + 1; j < A; j++) {
      const float* a = qf + s.agent_off[i];
      const float* b = qf + s.agent_off[j];
      float ss = 0.f;
      for (int k = 0; k < dim; k++) { float d = a[k] - b[k]; ss = fmaf(d, d, ss); }
      float thr = s.pair_thr32[i * A + j];
      float hi = thr + 2.f * delta, lo = thr - 2.f * delta;
      if (!(ss > hi * hi)) {
        if (lo > 0.f && ss < lo * lo) return V_COLLIDE;
        unc = true;
      }
    }
  // agent - obstacle  (abstract_env.py:270-274)
  for (int i = 0; i < A; i++) {
    const float* c = qf + s.agent_off[i];
    const float r = s.r32[i];
    const float rhi = r + delta, rlo = r - delta;
    for (int b = 0; b < s.nb; b++) {
      const float* lo = s.box_lo32 + b * dim;
      const float* hi = s.box_hi32 + b * dim;
      float ss = 0.f;
      for (int k = 0; k < dim; k++) {
        float v = fminf(fmaxf(c[k], lo[k]), hi[k]) - c[k];
        ss = fmaf(v, v, ss);
      }
      if (!(ss > rhi * rhi)) {
        if (rlo > 0.f && ss < rlo * rlo) return V_COLLIDE;
        unc = true;
      }
    }
    for (int o = 0; o < s.ns; o++) {
      const float* p = s.sph_pos32 + o * dim;
      float ss = 0.f;
      for (int k = 0; k < dim; k++) { float d = p[k] - c[k]; ss = fmaf(d, d, ss); }
      float thr = s.sph_thr32[o * A + i];
      float hi = thr + 2.f * delta, lo = thr - 2.f * delta;
      if (!(ss > hi * hi)) {
        if (lo > 0.f && ss < lo * lo) return V_COLLIDE;
        unc = true;
      }
    }
  }
  return unc ? V_PENDING : V_FREE;
}

// ---------------------------------------------------------------------------
// Exact FP64 restatement (same operation order as the reference).
// np.linalg.norm -> sqrt of a fused multiply-add chain from 0 (OpenBLAS ddot);
// np.sum of the squared clip residuals -> numpy pairwise order.
// ---------------------------------------------------------------------------
template <class Acc>
__device__ bool exact_free(const AbstractDev& s, Acc acc) {
  const int A = s.A, dim = s.dim;
  double d[kMaxAgentDim];
  for (int i = 0; i < A; i++)
    for (int j = i + 1; j < A; j++) {
      double ss = 0.0;
      for (int k = 0; k < dim; k++) {
        double t = __dsub_rn(acc(s.agent_off[i] + k), acc(s.agent_off[j] + k));
        ss = __fma_rn(t, t, ss);
      }
      if (sqrt(ss) < s.pair_thr[i * A + j]) return false;
    }
  for (int i = 0; i < A; i++) {
    const int off = s.agent_off[i];
    for (int b = 0; b < s.nb; b++) {
      const double* lo = s.box_lo + b * dim;
      const double* hi = s.box_hi + b * dim;
      for (int k = 0; k < dim; k++) {
        double c = acc(off + k);
        double v = c > lo[k] ? c : lo[k];
        v = v < hi[k] ? v : hi[k];
        double e = __dsub_rn(v, c);
        d[k] = __dmul_rn(e, e);
      }
      if (np_sum_dyn(d, dim) <= s.r2[i]) return false;
    }
    for (int o = 0; o < s.ns; o++) {
      const double* p = s.sph_pos + o * dim;
      double ss = 0.0;
      for (int k = 0; k < dim; k++) {
        double t = __dsub_rn(p[k], acc(off + k));
        ss = __fma_rn(t, t, ss);
      }
      if (sqrt(ss) < s.sph_thr[o * A + i]) return false;
    }
  }
  return true;
}

// ---------------------------------------------------------------------------
// Configurations: one thread per configuration.
// ---------------------------------------------------------------------------
__global__ void configs_pass1(AbstractDev s, const void* q, int dtype, long long n, uint8_t* out,
                              int* ctr, long long* pend) {
  const int D = s.D;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    auto acc = [&](int k) { return ldq(q, dtype, i * D + k); };
    uint8_t v = classify32(s, acc);
    out[i] = v;
    if (v == V_PENDING) {
      int slot = atomicAdd(&ctr[kCtrPending], 1);
      pend[slot] = i;
    }
  }
}

__global__ void configs_pass2(AbstractDev s, const void* q, int dtype, uint8_t* out, const int* ctr,
                              const long long* pend) {
  const int D = s.D;
  const int np = ctr[kCtrPending];
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < np; k += gridDim.x * blockDim.x) {
    long long i = pend[k];
    auto acc = [&](int j) { return ldq(q, dtype, i * D + j); };
    out[i] = exact_free(s, acc) ? 1 : 0;
  }
}

// ---------------------------------------------------------------------------
// Edges: one warp per edge; the lanes check consecutive chunks of the
// reference's binary-search order, with a warp vote after each chunk.
// ---------------------------------------------------------------------------
template <bool RESOLVE>
__global__ void edges_kernel(AbstractDev s, const void* q1, const void* q2, int dtype, long long n,
                             double res, int incl, const long long* Np, long long N_start,
                             long long N_max, uint8_t* out, int* ctr, long long* pend) {
  extern __shared__ double sm_ab[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int D = s.D;
  double* wq1 = sm_ab + (size_t)wib * 2 * D;
  double* wdir = wq1 + D;
  const unsigned lt_mask = (1u << lane) - 1u;

  while (true) {
    long long e;
    {
      long long k = 0;
      if (lane == 0) k = atomicAdd(&ctr[RESOLVE ? kCtrQueue2 : kCtrQueue], 1);
      k = __shfl_sync(MRMG_FULL, k, 0);
      if (RESOLVE) {
        if (k >= ctr[kCtrPending]) break;
        e = pend[k];
      } else {
        if (k >= n) break;
        e = k;
      }
    }
    // endpoints (NpConfiguration stores float64) and N
    double mloc = -1.0;
    bool nan0 = false;
    for (int k = lane; k < D; k += 32) {
      double a = ldq(q1, dtype, e * D + k), b = ldq(q2, dtype, e * D + k);
      wq1[k] = a;
      wdir[k] = b;
      double v = fabs(__dsub_rn(a, b));
      if (k == 0) nan0 = (v != v);
      mloc = fmax(mloc, v);
    }
    long long N;
    bool bad = false;
    if (Np) {
      N = Np[e];
      bad = N < 1;
    } else {
      // config_dist(q1, q2, "max") / resolution  (abstract_env.py:321-323)
      double m = warp_max_d(mloc);
      nan0 = __any_sync(MRMG_FULL, nan0);
      double t = __ddiv_rn(m, res);
      if (nan0 || !(t < 9.0e15)) bad = true;
      N = bad ? 2 : (long long)t + 1;
      if (N < 2) N = 2;
    }
    if (bad) {
      if (lane == 0) { atomicOr(&ctr[kCtrErr], E_BAD_INPUT); out[e] = 0; }
      __syncwarp();
      continue;
    }
    if (N_start > N) {   // the reference asserts (abstract_env.py:325-326)
      if (lane == 0) { atomicOr(&ctr[kCtrErr], E_N_START); out[e] = 0; }
      __syncwarp();
      continue;
    }
    const long long nmax = (N_max < 0 || N_max > N) ? N : N_max;
    const double denom = (double)(N - 1);
    __syncwarp();
    for (int k = lane; k < D; k += 32) wdir[k] = __ddiv_rn(__dsub_rn(wdir[k], wq1[k]), denom);
    __syncwarp();

    BfsChunker ch;
    ch.init(N);
    long long v;
    unsigned m;
    long long pos0;
    bool coll = false, pending = false;
    while (ch.next(lane, &v, &m, &pos0)) {
      if (pos0 >= nmax) break;
      long long my_pos = pos0 + __popc(m & lt_mask);
      bool active = v >= 0 && my_pos >= N_start && my_pos < nmax && (incl || (v != 0 && v != N - 1));
      uint8_t code = V_FREE;
      if (active) {
        const double di = (double)v;
        auto acc = [&](int k) { return __dadd_rn(wq1[k], __dmul_rn(wdir[k], di)); };
        code = classify32(s, acc);
        if (RESOLVE && code == V_PENDING) code = exact_free(s, acc) ? V_FREE : V_COLLIDE;
      }
      if (__any_sync(MRMG_FULL, code == V_COLLIDE)) { coll = true; break; }
      pending |= __any_sync(MRMG_FULL, code == V_PENDING);
    }
    if (lane == 0) {
      uint8_t r = coll ? V_COLLIDE : (pending ? V_PENDING : V_FREE);
      out[e] = r;
      if (!RESOLVE && r == V_PENDING) {
        int slot = atomicAdd(&ctr[kCtrPending], 1);
        pend[slot] = e;
      }
    }
    __syncwarp();
  }
}

}  // namespace

cudaError_t abstract_configs(const AbstractDev& s, const void* q, int dtype, long long n,
                             uint8_t* out, const CallScratch& sc, const LaunchShape& ls,
                             cudaStream_t st) {
  int threads = 256;
  long long want = (n + threads - 1) / threads;
  int grid = (int)(want < (long long)ls.num_sms * 8 ? (want > 0 ? want : 1) : (long long)ls.num_sms * 8);
  configs_pass1<<<grid, threads, 0, st>>>(s, q, dtype, n, out, sc.ctr, sc.pend);
  configs_pass2<<<ls.num_sms, 128, 0, st>>>(s, q, dtype, out, sc.ctr, sc.pend);
  return cudaGetLastError();
}

cudaError_t abstract_edges(const AbstractDev& s, const void* q1, const void* q2, int dtype,
                           long long n, double res, int incl, const long long* Np,
                           long long N_start, long long N_max, uint8_t* out,
                           const CallScratch& sc, const LaunchShape& ls, cudaStream_t st) {
  const int warps = 8;
  size_t smem = (size_t)warps * 2 * s.D * sizeof(double);
  long long want = (n + warps - 1) / warps;
  int grid = (int)(want < (long long)ls.num_sms * 8 ? (want > 0 ? want : 1) : (long long)ls.num_sms * 8);
  edges_kernel<false><<<grid, warps * 32, smem, st>>>(s, q1, q2, dtype, n, res, incl, Np, N_start,
                                                      N_max, out, sc.ctr, sc.pend);
  edges_kernel<true><<<ls.num_sms, warps * 32, smem, st>>>(s, q1, q2, dtype, n, res, incl, Np,
                                                           N_start, N_max, out, sc.ctr, sc.pend);
  return cudaGetLastError();
}

}  // namespace mrmg
