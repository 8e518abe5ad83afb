// mrmg_abstract.cu -- collision kernels for abstract point-agent scenes
// (problems/abstract_env.py: Sphere :41-58, Rectangle :61-109,
// AbstractEnvironment.is_collision_free :255-276, is_edge_collision_free
// :301-354).
//
// Every configuration is first classified in FP32 against a band that
// bounds the FP32 error: definitely colliding, definitely free, or pending.
// A pending configuration is decided by the exact FP64 restatement of the
// reference's arithmetic: at once, by the warp that met it (configurations
// and edge batches up to kFlatMaxEdges: one launch per call), or, for larger
// edge batches, in a second pass over the queued edges.
//
// The FP64 pipe of this part is narrow and issues a warp instruction at the
// same cost whatever the number of active lanes, so FP64 work is kept off
// long dependent chains: edge positions are interpolated in double-float
// FP32, step counts come from an FP32 quotient with an integer-distance
// certificate, and a pending configuration is decided by a whole warp at
// once, one agent pair, box or sphere test per lane.
#include <algorithm>

#include "mrmg_bulk.cuh"
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
// FP32 classification of one configuration qf[D] whose coordinates lie within
// 2^-24 |q| of the exact ones (plus `extra`, a distance), qmax = max |qf|.
// ---------------------------------------------------------------------------
__device__ uint8_t classify_core(const AbstractDev& s, const float* qf, float qmax, float extra) {
  const float delta = s.delta_k * (qmax + s.omax) + extra;
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
    int b = 0;
    // two boxes per step (independent chains; any definite collision decides,
    // so the order of the tests does not change the result)
    for (; b + 1 < s.nb; b += 2) {
      const float* lo0 = s.box_lo32 + b * dim;
      const float* hi0 = s.box_hi32 + b * dim;
      const float* lo1 = lo0 + dim;
      const float* hi1 = hi0 + dim;
      float ss0 = 0.f, ss1 = 0.f;
      for (int k = 0; k < dim; k++) {
        const float v0 = fminf(fmaxf(c[k], lo0[k]), hi0[k]) - c[k];
        const float v1 = fminf(fmaxf(c[k], lo1[k]), hi1[k]) - c[k];
        ss0 = fmaf(v0, v0, ss0);
        ss1 = fmaf(v1, v1, ss1);
      }
      if (!(ss0 > rhi * rhi)) {
        if (rlo > 0.f && ss0 < rlo * rlo) return V_COLLIDE;
        unc = true;
      }
      if (!(ss1 > rhi * rhi)) {
        if (rlo > 0.f && ss1 < rlo * rlo) return V_COLLIDE;
        unc = true;
      }
    }
    for (; b < s.nb; b++) {
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

// A configuration given as FP32 values x(k) (rounded once from the exact
// coordinates); NaN, inf or huge coordinates leave it pending (the exact
// path decides).
template <class Acc>
__device__ uint8_t classify32(const AbstractDev& s, Acc x, float extra) {
  float qf[kMaxAgents * kMaxAgentDim];
  float qmax = 0.f;
  bool bad = false;
  for (int k = 0; k < s.D; k++) {
    const float f = x(k);
    bad |= !(fabsf(f) <= 1e30f);
    qf[k] = f;
    qmax = fmaxf(qmax, fabsf(f));
  }
  return bad ? V_PENDING : classify_core(s, qf, qmax, extra);
}

// The same classification with the agent dimension known at compile time:
// each agent's coordinates are fetched into registers when a test needs them
// (x(k) is a cheap load or interpolation), so no per-thread array is indexed
// at run time (such arrays live in local memory).  Thresholds, band and test
// order are those of classify_core.
template <int DIM, class Acc>
__device__ uint8_t classify_dim(const AbstractDev& s, Acc x, float extra) {
  float qmax = 0.f;
  bool bad = false;
  for (int k = 0; k < s.D; k++) {
    const float f = x(k);
    bad |= !(fabsf(f) <= 1e30f);
    qmax = fmaxf(qmax, fabsf(f));
  }
  if (bad) return V_PENDING;
  const float delta = s.delta_k * (qmax + s.omax) + extra;
  bool unc = false;
  const int A = s.A;
  // agent - agent  (abstract_env.py:261-268)
  for (int i = 0; i < A; i++) {
    float a[DIM];
#pragma unroll
    for (int k = 0; k < DIM; k++) a[k] = x(s.agent_off[i] + k);
    for (int j = i + 1; j < A; j++) {
      float ss = 0.f;
#pragma unroll
      for (int k = 0; k < DIM; k++) {
        const float d = a[k] - x(s.agent_off[j] + k);
        ss = fmaf(d, d, ss);
      }
      const float thr = s.pair_thr32[i * A + j];
      const float hi = thr + 2.f * delta, lo = thr - 2.f * delta;
      if (!(ss > hi * hi)) {
        if (lo > 0.f && ss < lo * lo) return V_COLLIDE;
        unc = true;
      }
    }
  }
  // agent - obstacle  (abstract_env.py:270-274)
  for (int i = 0; i < A; i++) {
    float c[DIM];
#pragma unroll
    for (int k = 0; k < DIM; k++) c[k] = x(s.agent_off[i] + k);
    const float r = s.r32[i];
    const float rhi = r + delta, rlo = r - delta;
    int b = 0;
    for (; b + 1 < s.nb; b += 2) {
      const float* lo0 = s.box_lo32 + b * DIM;
      const float* hi0 = s.box_hi32 + b * DIM;
      float ss0 = 0.f, ss1 = 0.f;
#pragma unroll
      for (int k = 0; k < DIM; k++) {
        const float v0 = fminf(fmaxf(c[k], lo0[k]), hi0[k]) - c[k];
        const float v1 = fminf(fmaxf(c[k], lo0[DIM + k]), hi0[DIM + k]) - c[k];
        ss0 = fmaf(v0, v0, ss0);
        ss1 = fmaf(v1, v1, ss1);
      }
      if (!(ss0 > rhi * rhi)) {
        if (rlo > 0.f && ss0 < rlo * rlo) return V_COLLIDE;
        unc = true;
      }
      if (!(ss1 > rhi * rhi)) {
        if (rlo > 0.f && ss1 < rlo * rlo) return V_COLLIDE;
        unc = true;
      }
    }
    for (; b < s.nb; b++) {
      const float* lo = s.box_lo32 + b * DIM;
      const float* hi = s.box_hi32 + b * DIM;
      float ss = 0.f;
#pragma unroll
      for (int k = 0; k < DIM; k++) {
        const float v = fminf(fmaxf(c[k], lo[k]), hi[k]) - c[k];
        ss = fmaf(v, v, ss);
      }
      if (!(ss > rhi * rhi)) {
        if (rlo > 0.f && ss < rlo * rlo) return V_COLLIDE;
        unc = true;
      }
    }
    for (int o = 0; o < s.ns; o++) {
      const float* p = s.sph_pos32 + o * DIM;
      float ss = 0.f;
#pragma unroll
      for (int k = 0; k < DIM; k++) {
        const float d = p[k] - c[k];
        ss = fmaf(d, d, ss);
      }
      const float thr = s.sph_thr32[o * A + i];
      const float hi = thr + 2.f * delta, lo = thr - 2.f * delta;
      if (!(ss > hi * hi)) {
        if (lo > 0.f && ss < lo * lo) return V_COLLIDE;
        unc = true;
      }
    }
  }
  return unc ? V_PENDING : V_FREE;
}

// DIM > 0: the compile-time form; 0: any agent dimension
template <int DIM, class Acc>
__device__ __forceinline__ uint8_t classify_any(const AbstractDev& s, Acc x, float extra) {
  if constexpr (DIM == 0) return classify32(s, x, extra);
  else return classify_dim<DIM>(s, x, extra);
}

// ---------------------------------------------------------------------------
// Exact FP64 restatement of one configuration (same operation order as the
// reference), evaluated by all lanes of a warp together: lane t takes test t,
// t + 32, ... of the agent pairs, then the agent-box and agent-sphere tests.
// acc(k) is coordinate k in FP64.  np.linalg.norm -> sqrt of a fused
// multiply-add chain from 0 (OpenBLAS ddot); np.sum of the squared clip
// residuals -> numpy pairwise order.  Each test is the one the reference's
// loops make, so "any test collides" is their verdict.  Warp-uniform.
// ---------------------------------------------------------------------------
template <class Acc>
__device__ bool exact_free_warp(const AbstractDev& s, Acc acc, int lane) {
  const int A = s.A, dim = s.dim;
  const int n_pair = A * (A - 1) / 2, n_box = A * s.nb, n_all = n_pair + n_box + A * s.ns;
  for (int t0 = 0; t0 < n_all; t0 += 32) {
    const int t = t0 + lane;
    bool hit = false;
    if (t < n_pair) {
      int i = 0, r = t;
      while (r >= A - 1 - i) { r -= A - 1 - i; i++; }
      const int j = i + 1 + r;
      double ss = 0.0;
      for (int k = 0; k < dim; k++) {
        const double d = __dsub_rn(acc(s.agent_off[i] + k), acc(s.agent_off[j] + k));
        ss = __fma_rn(d, d, ss);
      }
      hit = sqrt(ss) < s.pair_thr[i * A + j];
    } else if (t < n_pair + n_box) {
      const int i = (t - n_pair) / s.nb, b = t - n_pair - i * s.nb;
      const int off = s.agent_off[i];
      const double* lo = s.box_lo + b * dim;
      const double* hi = s.box_hi + b * dim;
      double d[kMaxAgentDim];
      for (int k = 0; k < dim; k++) {
        const double c = acc(off + k);
        double v = c > lo[k] ? c : lo[k];
        v = v < hi[k] ? v : hi[k];
        const double e = __dsub_rn(v, c);
        d[k] = __dmul_rn(e, e);
      }
      hit = np_sum_dyn(d, dim) <= s.r2[i];
    } else if (t < n_all) {
      const int u = t - n_pair - n_box;
      const int i = u / s.ns, o = u - i * s.ns;
      const int off = s.agent_off[i];
      const double* p = s.sph_pos + o * dim;
      double ss = 0.0;
      if (s.sph_batch_form) {
        // Sphere.batch_collides_with_sphere (abstract_env.py:51-55):
        // np.linalg.norm(pos - centers, axis=1) = sqrt(add.reduce(d * d))
        double d2[kMaxAgentDim];
        for (int k = 0; k < dim; k++) {
          const double d = __dsub_rn(p[k], acc(off + k));
          d2[k] = __dmul_rn(d, d);
        }
        ss = np_sum_dyn(d2, dim);
      } else {
        // Sphere.collides_with_sphere (:44-47): the norm of one vector (ddot)
        for (int k = 0; k < dim; k++) {
          const double d = __dsub_rn(p[k], acc(off + k));
          ss = __fma_rn(d, d, ss);
        }
      }
      hit = sqrt(ss) < s.sph_thr[o * A + i];
    }
    if (__any_sync(MRMG_FULL, hit)) return false;
  }
  return true;
}

// ---------------------------------------------------------------------------
// The FP32 tables of the bulk pass, staged once per CTA in shared memory when
// they fit in kTabSmem bytes, so that the classification loop reads no global
// memory.  Every table holds 4-byte elements; each starts on 16 bytes.
// ---------------------------------------------------------------------------
constexpr size_t kTabSmem = 16384;

// bytes of the staged tables, 0 when they are read from global memory
__host__ __device__ inline size_t tab_bytes(const AbstractDev& s) {
  size_t off[8];
  abstract_table_layout(s, off);
  return off[7] <= kTabSmem ? off[7] : 0;
}

template <typename T>
__device__ __forceinline__ void stage_copy(T* dst, const T* src, size_t n) {
  for (size_t i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src[i];
}

// The scene with its FP32 tables in shared memory at `sm` (tab_bytes(s)
// bytes, abstract_table_layout): one bulk asynchronous copy of the scene's
// table image, or loads when it has none (or the copy timed out).  Every
// thread calls it; a __syncthreads() must follow.
__device__ AbstractDev staged_view(const AbstractDev& s, unsigned char* sm) {
  __shared__ __align__(8) uint64_t stage_bar;
  AbstractDev t = s;
  const size_t tb = tab_bytes(s);
  if (tb == 0) return t;
  size_t off[8];
  abstract_table_layout(s, off);
  t.agent_off = (const int*)(sm + off[0]);
  t.r32 = (const float*)(sm + off[1]);
  t.pair_thr32 = (const float*)(sm + off[2]);
  t.box_lo32 = (const float*)(sm + off[3]);
  t.box_hi32 = (const float*)(sm + off[4]);
  t.sph_pos32 = (const float*)(sm + off[5]);
  t.sph_thr32 = (const float*)(sm + off[6]);
  const bool bulk = s.img && bulk_ok(sm, s.img, tb);
  if (bulk && stage_bulk(sm, s.img, (uint32_t)tb, &stage_bar)) return t;
  stage_copy((int*)t.agent_off, s.agent_off, (size_t)s.A);
  stage_copy((float*)t.r32, s.r32, (size_t)s.A);
  stage_copy((float*)t.pair_thr32, s.pair_thr32, (size_t)s.A * s.A);
  stage_copy((float*)t.box_lo32, s.box_lo32, (size_t)s.nb * s.dim);
  stage_copy((float*)t.box_hi32, s.box_hi32, (size_t)s.nb * s.dim);
  stage_copy((float*)t.sph_pos32, s.sph_pos32, (size_t)s.ns * s.dim);
  stage_copy((float*)t.sph_thr32, s.sph_thr32, (size_t)s.ns * s.A);
  if (bulk) stage_bulk_drain(&stage_bar);
  return t;
}

// ---------------------------------------------------------------------------
// Edges: one warp per edge; the lanes check consecutive chunks of the
// reference's binary-search order, with a warp vote after each chunk.
//
// Positions q1 + (q2 - q1) * i / (N - 1) are formed in double-float FP32
// (interp_df: q1 and q2 - q1 as hi + lo pairs, ~44 significant bits) and
// rounded once, so each coordinate lies within 2^-24 |q| + 2^-42 (|q1| + |q2|)
// of the reference's FP64 position; `extra` = 2^-30 * max(|q1| + |q2|) * dim
// covers the second term (with a wide margin) in every distance, agent pairs
// included.  Pass 2 decides a pending position from the reference's own FP64
// arithmetic, q1 + ((q2 - q1) / (N - 1)) * i.
//
// Shared memory per warp: the double-float endpoints ah, al, dh, dl [D]
// (floats) and, in pass 2, q1 and the FP64 direction [D] (doubles).
// ---------------------------------------------------------------------------
constexpr size_t edge_warp_bytes(int D, bool resolve) { return (size_t)D * (resolve ? 32 : 16); }

template <bool RESOLVE>
__global__ void edges_kernel(AbstractDev s, const void* q1, const void* q2, int dtype, long long n,
                             double res, int incl, const long long* Np, long long N_start,
                             long long N_max, uint8_t* out, int* ctr, long long* pend) {
  extern __shared__ __align__(16) double sm_ab[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int D = s.D;
  // pass 1 classifies from staged tables (pass 2 is rare and reads them in place)
  const size_t tb = RESOLVE ? 0 : tab_bytes(s);
  const AbstractDev cs = RESOLVE ? s : staged_view(s, (unsigned char*)sm_ab);
  if (!RESOLVE) __syncthreads();
  unsigned char* wbase = (unsigned char*)sm_ab + tb + (size_t)wib * edge_warp_bytes(D, RESOLVE);
  double* w64a = (double*)wbase;                 // pass 2 only
  double* w64d = w64a + D;
  float* wah = (float*)(wbase + (RESOLVE ? (size_t)16 * D : 0));
  float* wal = wah + D;
  float* wdh = wal + D;
  float* wdl = wdh + D;
  const float res32 = (float)res;
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
    // endpoints as double-float: a = q1 and d = q2 - q1 (exact for FP32
    // endpoints; for FP64 ones d is the reference's FP64 difference, split)
    float mloc = 0.f, emax = 0.f;
    bool nanf = false;
    for (int k = lane; k < D; k += 32) {
      float a_h, a_l = 0.f, d_h, d_l;
      if (dtype == MRMG_F32) {
        const float a = ((const float*)q1)[e * D + k], b = ((const float*)q2)[e * D + k];
        a_h = a;
        two_sum(b, -a, &d_h, &d_l);
      } else {
        const double a = ((const double*)q1)[e * D + k], b = ((const double*)q2)[e * D + k];
        const double d = __dsub_rn(b, a);
        a_h = (float)a;
        a_l = (float)__dsub_rn(a, (double)a_h);
        d_h = (float)d;
        d_l = (float)__dsub_rn(d, (double)d_h);
      }
      wah[k] = a_h; wal[k] = a_l; wdh[k] = d_h; wdl[k] = d_l;
      nanf |= d_h != d_h;
      mloc = fmaxf(mloc, fabsf(d_h));
      emax = fmaxf(emax, fabsf(a_h) + fabsf(__fadd_rn(a_h, d_h)));
    }
    long long N = 2;
    bool bad = false;
    if (Np) {
      N = Np[e];
      bad = N < 1;
    } else {
      const float m32 = warp_max(mloc);
      const bool anynan = __any_sync(MRMG_FULL, nanf);
      if (!steps_fp32(m32, anynan, res32, &N)) {
        // config_dist(q1, q2, "max") / resolution in FP64 (abstract_env.py:321-323)
        double mx = -1.0;
        bool nan0 = false;
        for (int k = lane; k < D; k += 32) {
          const double v = fabs(__dsub_rn(ldq(q1, dtype, e * D + k), ldq(q2, dtype, e * D + k)));
          if (k == 0) nan0 = (v != v);
          mx = fmax(mx, v);
        }
        const double m = warp_max_d(mx);
        nan0 = __any_sync(MRMG_FULL, nan0);
        const double t = __ddiv_rn(m, res);
        if (nan0 || !(t < 9.0e15)) bad = true;
        N = bad ? 2 : (long long)t + 1;
        if (N < 2) N = 2;
      }
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
    // positions are exact FP32 integers up to 2^24; beyond, pass 1 leaves
    // the edge to pass 2, which interpolates those in FP64
    const bool df_ok = N <= (1ll << 24);
    const float nm1 = df_ok ? (float)(int)(N - 1) : 1.f;
    const float rn = __frcp_rn(nm1);
    const float extra = ldexpf(warp_max(emax) * (float)s.dim, -30);
    bool have64 = false;
    auto load64 = [&]() {   // the reference's q1 and (q2 - q1) / (N - 1), once per edge
      const double denom = (double)(N - 1);
      for (int k = lane; k < D; k += 32) {
        const double a = ldq(q1, dtype, e * D + k), b = ldq(q2, dtype, e * D + k);
        w64a[k] = a;
        w64d[k] = __ddiv_rn(__dsub_rn(b, a), denom);
      }
      __syncwarp();
      have64 = true;
    };
    __syncwarp();
    if (RESOLVE && !df_ok) load64();

    bool coll = false, pending = false;
    if (!RESOLVE && !df_ok) {
      pending = true;
    } else {
      BfsChunker ch;
      ch.init(N);
      long long v;
      unsigned m;
      long long pos0;
      while (ch.next(lane, &v, &m, &pos0)) {
        if (pos0 >= nmax) break;
        const long long my_pos = pos0 + __popc(m & lt_mask);
        const bool active = v >= 0 && my_pos >= N_start && my_pos < nmax && (incl || (v != 0 && v != N - 1));
        uint8_t code = V_FREE;
        if (active) {
          if (df_ok) {
            const float fi = (float)(int)v;
            auto x = [&](int k) {
              float h, l;
              interp_df(wah[k], wal[k], wdh[k], wdl[k], fi, nm1, rn, &h, &l);
              return __fadd_rn(h, l);
            };
            code = classify32(cs, x, extra);
          } else {
            const double di = (double)v;
            auto x = [&](int k) { return (float)__dadd_rn(w64a[k], __dmul_rn(w64d[k], di)); };
            code = classify32(cs, x, 0.f);
          }
        }
        if (RESOLVE) {
          unsigned pm = __ballot_sync(MRMG_FULL, code == V_PENDING);
          if (pm && !have64) load64();
          while (pm) {
            const int src = __ffs(pm) - 1;
            pm &= pm - 1;
            const double di = (double)__shfl_sync(MRMG_FULL, v, src);
            auto acc = [&](int k) { return __dadd_rn(w64a[k], __dmul_rn(w64d[k], di)); };
            const bool ok = exact_free_warp(s, acc, lane);
            if (lane == src) code = ok ? V_FREE : V_COLLIDE;
          }
        }
        if (__any_sync(MRMG_FULL, code == V_COLLIDE)) { coll = true; break; }
        if (!RESOLVE) pending |= __any_sync(MRMG_FULL, code == V_PENDING);
      }
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

// ---------------------------------------------------------------------------
// Single-launch forms.  A pending classification is decided at once by the
// warp that met it (the lanes' pending items are taken one by one, each by
// the whole warp with the exact FP64 restatement), so no second pass, no
// pending list and no counter reset are needed: one launch per call.
// ctr may be NULL (no statistics, and no error bits: the host-pointer calls
// validate step counts on the host before launching).
// ---------------------------------------------------------------------------
template <int DIM>
__global__ void __launch_bounds__(256) configs_fused_kernel(AbstractDev s, const void* q, int dtype, long long n,
                                                            uint8_t* out, int* ctr) {
  extern __shared__ __align__(16) double sm_cfg[];
  const AbstractDev cs = staged_view(s, (unsigned char*)sm_cfg);
  __syncthreads();
  const int D = s.D;
  const int lane = threadIdx.x & 31;
  double* wq = (double*)((unsigned char*)sm_cfg + tab_bytes(s)) + (size_t)(threadIdx.x >> 5) * D;
  int npend = 0;
  for (long long i0 = blockIdx.x * (long long)blockDim.x; i0 < n; i0 += (long long)gridDim.x * blockDim.x) {
    const long long i = i0 + threadIdx.x;
    uint8_t v = V_FREE;
    if (i < n) {
      auto x = [&](int k) {
        return dtype == MRMG_F32 ? ((const float*)q)[i * D + k] : (float)((const double*)q)[i * D + k];
      };
      v = classify_any<DIM>(cs, x, 0.f);
    }
    unsigned pm = __ballot_sync(MRMG_FULL, v == V_PENDING);
    npend += __popc(pm);
    while (pm) {
      const int src = __ffs(pm) - 1;
      pm &= pm - 1;
      const long long j = __shfl_sync(MRMG_FULL, i, src);
      // the configuration's coordinates into the warp's shared area once
      // (the inputs may sit in host memory mapped for the device)
      for (int k = lane; k < D; k += 32) wq[k] = ldq(q, dtype, j * D + k);
      __syncwarp();
      auto acc = [&](int k) { return wq[k]; };
      const bool ok = exact_free_warp(s, acc, lane);
      if (lane == src) v = ok ? V_FREE : V_COLLIDE;
      __syncwarp();
    }
    if (i < n) out[i] = v;
  }
  if (ctr && lane == 0 && npend) atomicAdd(&ctr[kCtrPending], npend);
}

// Edges, flat: each CTA takes `epc` edges at a time; its warps compute the
// edges' step counts and double-float endpoints, then every thread takes
// (edge, BFS position) items of the group, so the positions of an edge are
// checked side by side instead of chunk after chunk by one warp.  A position
// of an edge already seen to collide is skipped.
constexpr int kFlatMaxEpc = 8;

template <int DIM>
__global__ void __launch_bounds__(256) edges_flat_kernel(AbstractDev s, const void* q1, const void* q2, int dtype,
                                                         long long n, double res, int incl, const long long* Np,
                                                         long long N_start, long long N_max, uint8_t* out, int* ctr,
                                                         int epc, uint8_t* cta_err) {
  extern __shared__ __align__(16) double sm_ab[];
  const AbstractDev cs = staged_view(s, (unsigned char*)sm_ab);
  __shared__ int s_err;   // error bits of this CTA when reported per CTA (cta_err)
  __shared__ long long sN[kFlatMaxEpc];
  __shared__ int soff[kFlatMaxEpc + 1];
  __shared__ float sext[kFlatMaxEpc];
  __shared__ int sst[kFlatMaxEpc];   // bit 0 collides, bit 1 decided already (error, or positions beyond FP32)
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int D = s.D;
  float* eah = (float*)((unsigned char*)sm_ab + tab_bytes(s));   // [epc][D] x 4 arrays
  float* eal = eah + kFlatMaxEpc * D;
  float* edh = eal + kFlatMaxEpc * D;
  float* edl = edh + kFlatMaxEpc * D;
  // the reference's FP64 q1 and (q2 - q1) / (N - 1) of each edge, for the exact path
  double* e64a = (double*)(edl + kFlatMaxEpc * D);
  double* e64d = e64a + kFlatMaxEpc * D;
  const float res32 = (float)res;
  int npend = 0;
  if (threadIdx.x == 0) s_err = 0;
  __syncthreads();
  for (long long e0 = (long long)blockIdx.x * epc; e0 < n; e0 += (long long)gridDim.x * epc) {
    const int ne = (int)min((long long)epc, n - e0);
    // ---- per edge: endpoints as double-float, N, error checks
    for (int w = wib; w < ne; w += nw) {
      const long long e = e0 + w;
      float mloc = 0.f, emax = 0.f;
      bool nanf = false;
      for (int k = lane; k < D; k += 32) {
        float a_h, a_l = 0.f, d_h, d_l;
        if (dtype == MRMG_F32) {
          const float a = ((const float*)q1)[e * D + k], b = ((const float*)q2)[e * D + k];
          a_h = a;
          two_sum(b, -a, &d_h, &d_l);
        } else {
          const double a = ((const double*)q1)[e * D + k], b = ((const double*)q2)[e * D + k];
          const double d = __dsub_rn(b, a);
          a_h = (float)a;
          a_l = (float)__dsub_rn(a, (double)a_h);
          d_h = (float)d;
          d_l = (float)__dsub_rn(d, (double)d_h);
        }
        eah[w * D + k] = a_h; eal[w * D + k] = a_l; edh[w * D + k] = d_h; edl[w * D + k] = d_l;
        nanf |= d_h != d_h;
        mloc = fmaxf(mloc, fabsf(d_h));
        emax = fmaxf(emax, fabsf(a_h) + fabsf(__fadd_rn(a_h, d_h)));
      }
      long long N = 2;
      bool bad = false;
      if (Np) {
        N = Np[e];
        bad = N < 1;
      } else {
        const float m32 = warp_max(mloc);
        const bool anynan = __any_sync(MRMG_FULL, nanf);
        if (!steps_fp32(m32, anynan, res32, &N)) {
          // config_dist(q1, q2, "max") / resolution in FP64 (abstract_env.py:321-323)
          double mx = -1.0;
          bool nan0 = false;
          for (int k = lane; k < D; k += 32) {
            const double v = fabs(__dsub_rn(ldq(q1, dtype, e * D + k), ldq(q2, dtype, e * D + k)));
            if (k == 0) nan0 = (v != v);
            mx = fmax(mx, v);
          }
          const double m = warp_max_d(mx);
          nan0 = __any_sync(MRMG_FULL, nan0);
          const double t = __ddiv_rn(m, res);
          if (nan0 || !(t < 9.0e15)) bad = true;
          N = bad ? 2 : (long long)t + 1;
          if (N < 2) N = 2;
        }
      }
      const float ext = ldexpf(warp_max(emax) * (float)s.dim, -30);
      {
        const double denom = (double)(N - 1);
        for (int k = lane; k < D; k += 32) {
          const double a = ldq(q1, dtype, e * D + k), b = ldq(q2, dtype, e * D + k);
          e64a[w * D + k] = a;
          e64d[w * D + k] = __ddiv_rn(__dsub_rn(b, a), denom);
        }
      }
      if (lane == 0) {
        sN[w] = N;
        sext[w] = ext;
        sst[w] = 0;
        if (bad || N_start > N) {   // the reference raises / asserts (abstract_env.py:321-326)
          if (ctr) atomicOr(&ctr[kCtrErr], bad ? E_BAD_INPUT : E_N_START);
          else atomicOr(&s_err, bad ? E_BAD_INPUT : E_N_START);
          out[e] = 0;
          sst[w] = 2;
        }
      }
    }
    __syncthreads();
    if (wib == 0) {   // item offsets: an inclusive scan over the group's edges (ne <= 8)
      int cnt = 0;
      if (lane < ne) {
        const long long N = sN[lane];
        const long long nmax = (N_max < 0 || N_max > N) ? N : N_max;
        if (!(sst[lane] & 2) && nmax > N_start) cnt = (int)(nmax - N_start);
      }
      int inc = cnt;
#pragma unroll
      for (int o = 1; o < kFlatMaxEpc; o <<= 1) {
        const int y = __shfl_up_sync(MRMG_FULL, inc, o);
        if (lane >= o) inc += y;
      }
      if (lane < ne) soff[lane + 1] = inc;
      if (lane == 0) soff[0] = 0;
    }
    __syncthreads();
    const int total = soff[ne];
    for (int t0 = 0; t0 < total; t0 += blockDim.x) {
      const int t = t0 + threadIdx.x;
      int w = 0;
      long long iv = -1, N = 2;
      uint8_t code = V_FREE;
      if (t < total) {
        while (t >= soff[w + 1]) w++;
        N = sN[w];
        iv = N <= (1ll << 24) ? (long long)bfs_at32((int)N, (int)(N_start + (t - soff[w])))
                              : bfs_at(N, N_start + (t - soff[w]));
        const bool skip = (!incl && (iv == 0 || iv == N - 1)) || (*(volatile int*)&sst[w] & 1);
        if (skip) {
          iv = -1;
        } else if (N <= (1ll << 24)) {
          const float nm1 = (float)(int)(N - 1), rn = __frcp_rn(nm1), fi = (float)(int)iv;
          const float* ah = eah + w * D; const float* al = eal + w * D;
          const float* dh = edh + w * D; const float* dl = edl + w * D;
          auto x = [&](int k) {
            float h, l;
            interp_df(ah[k], al[k], dh[k], dl[k], fi, nm1, rn, &h, &l);
            return __fadd_rn(h, l);
          };
          code = classify_any<DIM>(cs, x, sext[w]);
        } else {
          code = V_PENDING;   // positions beyond exact FP32 integers: FP64 at once
        }
      }
      // pending positions: the reference's FP64 position q1 + ((q2 - q1) / (N - 1)) * i, decided by the warp
      unsigned pm = __ballot_sync(MRMG_FULL, code == V_PENDING);
      npend += __popc(pm);
      while (pm) {
        const int src = __ffs(pm) - 1;
        pm &= pm - 1;
        const int ws = __shfl_sync(MRMG_FULL, w, src);
        const double di = (double)__shfl_sync(MRMG_FULL, iv, src);
        const double* a64 = e64a + ws * D;
        const double* d64 = e64d + ws * D;
        auto acc = [&](int k) { return __dadd_rn(a64[k], __dmul_rn(d64[k], di)); };
        const bool ok = exact_free_warp(s, acc, lane);
        if (lane == src) code = ok ? V_FREE : V_COLLIDE;
      }
      if (t < total && code == V_COLLIDE) atomicOr(&sst[w], 1);
    }
    __syncthreads();
    if (threadIdx.x < ne && !(sst[threadIdx.x] & 2)) out[e0 + threadIdx.x] = (sst[threadIdx.x] & 1) ? V_COLLIDE : V_FREE;
    __syncthreads();
  }
  if (ctr && lane == 0 && npend) atomicAdd(&ctr[kCtrPending], npend);
  if (cta_err && threadIdx.x == 0) cta_err[blockIdx.x] = (uint8_t)s_err;   // after the loop's last barrier
}

}  // namespace

// the fused kernels, compiled for agent dimensions 2 and 3 and for any
static void launch_configs_fused(const AbstractDev& s, int grid, int threads, cudaStream_t st, const void* q,
                                 int dtype, long long n, uint8_t* out, int* ctr) {
  const size_t sm = tab_bytes(s) + (size_t)(threads / 32) * s.D * sizeof(double);   // tables, per-warp coordinates
  if (s.dim == 2) configs_fused_kernel<2><<<grid, threads, sm, st>>>(s, q, dtype, n, out, ctr);
  else if (s.dim == 3) configs_fused_kernel<3><<<grid, threads, sm, st>>>(s, q, dtype, n, out, ctr);
  else configs_fused_kernel<0><<<grid, threads, sm, st>>>(s, q, dtype, n, out, ctr);
}

static size_t flat_smem(const AbstractDev& s) { return tab_bytes(s) + (size_t)kFlatMaxEpc * s.D * 32; }

static void launch_edges_flat(const AbstractDev& s, int grid, cudaStream_t st, const void* q1, const void* q2,
                              int dtype, long long n, double res, int incl, const long long* Np, long long N_start,
                              long long N_max, uint8_t* out, int* ctr, int epc, uint8_t* cta_err) {
  const size_t sm = flat_smem(s);
  if (s.dim == 2)
    edges_flat_kernel<2><<<grid, 256, sm, st>>>(s, q1, q2, dtype, n, res, incl, Np, N_start, N_max, out, ctr, epc,
                                                cta_err);
  else if (s.dim == 3)
    edges_flat_kernel<3><<<grid, 256, sm, st>>>(s, q1, q2, dtype, n, res, incl, Np, N_start, N_max, out, ctr, epc,
                                                cta_err);
  else
    edges_flat_kernel<0><<<grid, 256, sm, st>>>(s, q1, q2, dtype, n, res, incl, Np, N_start, N_max, out, ctr, epc,
                                                cta_err);
}

cudaError_t abstract_configs(const AbstractDev& s, const void* q, int dtype, long long n,
                             uint8_t* out, const CallScratch& sc, const LaunchShape& ls,
                             cudaStream_t st) {
  // 128-thread CTAs: a batch of a few thousand configurations spreads over
  // more SMs (each thread's chain is latency-bound, not issue-bound)
  const int threads = 128;
  const long long want = (n + threads - 1) / threads;
  const int grid = (int)std::max(1ll, std::min(want, (long long)ls.num_sms * 16));
  launch_configs_fused(s, grid, threads, st, q, dtype, n, out, sc.ctr);
  return cudaGetLastError();
}

// edges per CTA of the flat kernel: enough CTAs to fill the GPU
static int flat_epc(long long n, int num_sms) {
  const long long per = (n + (long long)num_sms * 4 - 1) / ((long long)num_sms * 4);
  return (int)std::max(1ll, std::min((long long)kFlatMaxEpc, per));
}


cudaError_t abstract_configs_mapped(const AbstractDev& s, const void* q, int dtype, long long n, uint8_t* out,
                                    int num_sms, cudaStream_t st) {
  const int threads = 128;
  const long long want = (n + threads - 1) / threads;
  const int grid = (int)std::max(1ll, std::min(want, (long long)num_sms * 16));
  launch_configs_fused(s, grid, threads, st, q, dtype, n, out, nullptr);
  return cudaGetLastError();
}

cudaError_t abstract_edges_mapped(const AbstractDev& s, const void* q1, const void* q2, int dtype, long long n,
                                  double res, int incl, const long long* Np, long long N_start, long long N_max,
                                  uint8_t* out, uint8_t* cta_err, int num_sms, cudaStream_t st, int* grid_out) {
  const int epc = flat_epc(n, num_sms);
  const long long want = (n + epc - 1) / epc;
  const int grid = (int)std::max(1ll, std::min(want, (long long)num_sms * 8));
  *grid_out = grid;
  launch_edges_flat(s, grid, st, q1, q2, dtype, n, res, incl, Np, N_start, N_max, out, nullptr, epc, cta_err);
  return cudaGetLastError();
}

int abstract_prepare(const AbstractDev& s) {
  // the kernels' limits go to the device maximum once (see allow_max_smem)
  if (allow_max_smem(edges_flat_kernel<0>) != cudaSuccess || allow_max_smem(edges_flat_kernel<2>) != cudaSuccess ||
      allow_max_smem(edges_flat_kernel<3>) != cudaSuccess)
    return -1;
  int dev = 0, optin = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
    return -1;
  return flat_smem(s) + 1024 <= (size_t)optin ? 0 : -1;
}

cudaError_t abstract_edges(const AbstractDev& s, const void* q1, const void* q2, int dtype,
                           long long n, double res, int incl, const long long* Np,
                           long long N_start, long long N_max, uint8_t* out,
                           const CallScratch& sc, const LaunchShape& ls, cudaStream_t st) {
  if (n <= kFlatMaxEdges) {
    const int epc = flat_epc(n, ls.num_sms);
    const long long want = (n + epc - 1) / epc;
    const int grid = (int)std::min(want, (long long)ls.num_sms * 8);
    launch_edges_flat(s, grid, st, q1, q2, dtype, n, res, incl, Np, N_start, N_max, out, sc.ctr, epc, nullptr);
    return cudaGetLastError();
  }
  const int warps = 8;
  const size_t smem1 = tab_bytes(s) + (size_t)warps * edge_warp_bytes(s.D, false);
  const size_t smem2 = (size_t)warps * edge_warp_bytes(s.D, true);
  cudaError_t e = cudaSuccess;
  if (smem1 > 48 * 1024)
    e = cudaFuncSetAttribute(edges_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem1);
  if (e == cudaSuccess && smem2 > 48 * 1024)
    e = cudaFuncSetAttribute(edges_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem2);
  if (e != cudaSuccess) return e;
  long long want = (n + warps - 1) / warps;
  int grid = (int)(want < (long long)ls.num_sms * 8 ? (want > 0 ? want : 1) : (long long)ls.num_sms * 8);
  edges_kernel<false><<<grid, warps * 32, smem1, st>>>(s, q1, q2, dtype, n, res, incl, Np, N_start,
                                                       N_max, out, sc.ctr, sc.pend);
  edges_kernel<true><<<ls.num_sms, warps * 32, smem2, st>>>(s, q1, q2, dtype, n, res, incl, Np,
                                                            N_start, N_max, out, sc.ctr, sc.pend);
  return cudaGetLastError();
}

unsigned int abstract_stage_timeouts() {
  unsigned int v = 0;
  if (cudaMemcpyFromSymbol(&v, g_stage_timeouts, sizeof v) != cudaSuccess) return 0;
  return v;
}

}  // namespace mrmg
