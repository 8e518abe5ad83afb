// mrmg_common.cuh -- device helpers shared by every kernel of the library.
//
// Exactness rule: every FP64 expression that must reproduce the reference's
// IEEE results is written with explicit round-to-nearest intrinsics
// (__dadd_rn, __dmul_rn, __fma_rn ...), so nvcc's multiply-add contraction can
// never change a rounding.  FP32 code paths are free to contract: their error
// is covered by the re-check band.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/mrmg_gb300.h"

#define MRMG_FULL 0xffffffffu

namespace mrmg {

// ---------------------------------------------------------------------------
// Deterministic FP64 sine / cosine.
// Cody & Waite argument reduction by pi/2 with a three-part split constant,
// then the Taylor series of sin and cos on [-pi/4, pi/4] (coefficients
// (-1)^n/(2n+1)! and (-1)^n/(2n)!, correctly rounded), Horner's rule with
// separate multiplies and adds.  Every step is an IEEE-rounded operation, so
// host and device evaluate the same bits.  |x| >= 2^30 or non-finite -> NaN.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void sincos_exact(double x, double* sn, double* cs) {
  const double TWO_OVER_PI = 0x1.45f306dc9c883p-1;
  const double P1 = 0x1.921fb54400000p+0, P2 = 0x1.0b4611a600000p-34, P3 = 0x1.3198a2e037073p-69;
  if (!(fabs(x) < 0x1p30)) {
    *sn = __longlong_as_double(0x7ff8000000000000ll);
    *cs = *sn;
    return;
  }
  const double S[9] = {-0x1.5555555555555p-3, 0x1.1111111111111p-7, -0x1.a01a01a01a01ap-13,
                       0x1.71de3a556c734p-19, -0x1.ae64567f544e4p-26, 0x1.6124613a86d09p-33,
                       -0x1.ae7f3e733b81fp-41, 0x1.952c77030ad4ap-49, -0x1.2f49b46814157p-57};
  const double C[9] = {-0x1.0000000000000p-1, 0x1.5555555555555p-5, -0x1.6c16c16c16c17p-10,
                       0x1.a01a01a01a01ap-16, -0x1.27e4fb7789f5cp-22, 0x1.1eed8eff8d898p-29,
                       -0x1.93974a8c07c9dp-37, 0x1.ae7f3e733b81fp-45, -0x1.6827863b97d97p-53};
  double k = rint(__dmul_rn(x, TWO_OVER_PI));
  double r = __dsub_rn(x, __dmul_rn(k, P1));
  r = __dsub_rn(r, __dmul_rn(k, P2));
  r = __dsub_rn(r, __dmul_rn(k, P3));
  double r2 = __dmul_rn(r, r);
  double ps = S[8];
#pragma unroll
  for (int i = 7; i >= 0; i--) ps = __dadd_rn(__dmul_rn(ps, r2), S[i]);
  double sr = __dadd_rn(r, __dmul_rn(__dmul_rn(r, r2), ps));
  double pc = C[8];
#pragma unroll
  for (int i = 7; i >= 0; i--) pc = __dadd_rn(__dmul_rn(pc, r2), C[i]);
  double cr = __dadd_rn(1.0, __dmul_rn(r2, pc));
  long long q = ((long long)k) & 3;
  if (q == 0) { *sn = sr; *cs = cr; }
  else if (q == 1) { *sn = cr; *cs = -sr; }
  else if (q == 2) { *sn = -sr; *cs = -cr; }
  else { *sn = -cr; *cs = sr; }
}

// FP64 -> FP32 angle for the bulk path: reduce to [-pi, pi] in FP64 (two-part
// 2*pi), then round.  Returns false when |x| is too large for the reduction
// (the configuration is then re-checked in FP64).
__device__ __forceinline__ bool reduce_angle_f32(double x, float* out) {
  const double INV_2PI = 0x1.45f306dc9c883p-3;
  const double TP1 = 0x1.921fb54400000p+2, TP2 = 0x1.0b4611a600000p-32;
  if (x != x) { *out = (float)x; return true; }   // NaN stays NaN: never collides
  if (!(fabs(x) < 0x1p20)) { *out = 0.f; return false; }
  double k = rint(x * INV_2PI);
  double r = fma(-k, TP1, x);
  r = fma(-k, TP2, r);
  *out = (float)r;
  return true;
}

// ---------------------------------------------------------------------------
// Double-float (hi + lo FP32 pair) helpers for the FP32 bulk path.  The
// intrinsics keep nvcc from fusing the error-free transforms.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void two_sum(float a, float b, float* s, float* e) {
  const float t = __fadd_rn(a, b);
  const float bb = __fsub_rn(t, a);
  *e = __fadd_rn(__fsub_rn(a, __fsub_rn(t, bb)), __fsub_rn(b, bb));
  *s = t;
}

// Angle h + l reduced to [-pi, pi] with one final rounding to FP32
// (2*pi = C1 + C2, C1 = fl32(2*pi); k*C1 split exactly with an FMA, h - k*C1
// exact by Sterbenz).  False when |h| >= 2^14 (the exact path decides).
__device__ __forceinline__ bool reduce_df(float h, float l, float* out) {
  if (h != h || l != l) { *out = __fadd_rn(h, l); return true; }   // NaN never collides
  if (!(fabsf(h) < 16384.f)) { *out = 0.f; return false; }
  const float C1 = 0x1.921fb6p+2f, C2 = -0x1.777a5cp-23f, INV = 0x1.45f306p-3f;
  const float k = rintf(__fmul_rn(h, INV));
  const float p1h = __fmul_rn(k, C1);
  const float p1l = fmaf(k, C1, -p1h);
  const float sh = __fsub_rn(h, p1h);
  const float t = fmaf(-k, C2, __fsub_rn(l, p1l));
  *out = __fadd_rn(sh, t);
  return true;
}

// theta = a + d * (i / nm1) for double-float a = (ah, al), d = (dh, dl);
// rn ~ 1 / nm1.  Result (h, l) carries ~44 significant bits.
__device__ __forceinline__ void interp_df(float ah, float al, float dh, float dl, float fi, float nm1, float rn,
                                          float* h, float* l) {
  const float th = __fmul_rn(fi, rn);
  const float tl = __fmul_rn(fmaf(-th, nm1, fi), rn);
  const float ph = __fmul_rn(dh, th);
  float pl = fmaf(dh, th, -ph);
  pl = fmaf(dh, tl, fmaf(dl, th, pl));
  float sh, sl;
  two_sum(ah, ph, &sh, &sl);
  *h = sh;
  *l = __fadd_rn(__fadd_rn(sl, pl), al);
}

// np.sum of up to 15 float64 values in numpy's pairwise order.
template <int N>
__device__ __forceinline__ double np_sum_small(const double* a) {
  static_assert(N >= 1 && N <= 15, "dims 1..15");
  if (N < 8) {
    double r = 0.0;
#pragma unroll
    for (int i = 0; i < N; i++) r = __dadd_rn(r, a[i]);
    return r;
  } else {
    double res = __dadd_rn(__dadd_rn(__dadd_rn(a[0], a[1]), __dadd_rn(a[2], a[3])),
                           __dadd_rn(__dadd_rn(a[4], a[5]), __dadd_rn(a[6], a[7])));
#pragma unroll
    for (int i = 8; i < N; i++) res = __dadd_rn(res, a[i]);
    return res;
  }
}

// runtime-dim variant (dims 1..15)
__device__ __forceinline__ double np_sum_dyn(const double* a, int n) {
  if (n < 8) {
    double r = 0.0;
    for (int i = 0; i < n; i++) r = __dadd_rn(r, a[i]);
    return r;
  }
  double res = __dadd_rn(__dadd_rn(__dadd_rn(a[0], a[1]), __dadd_rn(a[2], a[3])),
                         __dadd_rn(__dadd_rn(a[4], a[5]), __dadd_rn(a[6], a[7])));
  for (int i = 8; i < n; i++) res = __dadd_rn(res, a[i]);
  return res;
}

// ---------------------------------------------------------------------------
// generate_binary_search_indices (problems/planning_env.py:34-51) without a
// table: the reference's BFS over midpoint intervals visits the midpoint tree
// level by level, left to right.  Node `slot` of level `level` is reached by
// following the slot's bits (MSB first, 0 = left half, 1 = right half); it
// exists iff its interval is non-empty.  Returns the node's index or -1.
// ---------------------------------------------------------------------------
__device__ __forceinline__ long long bfs_node(long long N, int level, long long slot) {
  long long s = 0, e = N - 1;
  for (int b = level - 1; b >= 0; b--) {
    if (s > e) return -1;
    long long mid = (s + e) >> 1;
    if ((slot >> b) & 1) s = mid + 1;
    else e = mid - 1;
  }
  if (s > e) return -1;
  return (s + e) >> 1;
}

// Position p of the BFS order directly.  Every level of the midpoint tree is
// full except possibly the last (interval sizes on one level differ by at
// most one), so positions below 2^L - 1 map to (level, slot) in closed form;
// on the last level the r-th present node is found by descending the tree,
// where a subtree rooted at depth d with interval size s has
// s - (2^(L-d) - 1) nodes on level L.  O(log N), no table.
__device__ __forceinline__ long long bfs_at(long long N, long long p) {
  const int L = 63 - __clzll(N + 1);          // 2^L - 1 <= N
  const long long full = (1ll << L) - 1;
  if (p < full) {
    const int lv = 63 - __clzll(p + 1);
    return bfs_node(N, lv, p + 1 - (1ll << lv));
  }
  long long r = p - full, a = 0, b = N - 1;
  for (int d = 0; d < L; d++) {
    const long long m = (a + b) >> 1;
    const long long cnt = (m - a) - ((1ll << (L - d - 1)) - 1);
    if (r < cnt) b = m - 1;
    else { r -= cnt; a = m + 1; }
  }
  return a;
}

// bfs_at in 32-bit arithmetic, for N <= 2^24 (the FP32 edge paths)
__device__ __forceinline__ int bfs_at32(int N, int p) {
  const int L = 31 - __clz(N + 1);
  const int full = (1 << L) - 1;
  if (p < full) {
    const int lv = 31 - __clz(p + 1);
    const int slot = p + 1 - (1 << lv);
    int s = 0, e = N - 1;
    for (int b = lv - 1; b >= 0; b--) {
      const int mid = (s + e) >> 1;
      if ((slot >> b) & 1) s = mid + 1;
      else e = mid - 1;
    }
    return (s + e) >> 1;   // levels above the last are full: the node exists
  }
  int r = p - full, a = 0, b = N - 1;
  for (int d = 0; d < L; d++) {
    const int m = (a + b) >> 1;
    const int cnt = (m - a) - ((1 << (L - d - 1)) - 1);
    if (r < cnt) b = m - 1;
    else { r -= cnt; a = m + 1; }
  }
  return a;
}

// Warp-uniform iterator over the BFS order in chunks of up to 32 slots of one
// level.  next() returns, per lane, the index held by that lane's slot (or -1
// where the slot is empty), the ballot of non-empty slots and the BFS position
// of the chunk's first element; lane j's element sits at BFS position
// pos0 + popc(mask & lanemask_lt(j)).  All lanes must call next() together.
struct BfsChunker {
  long long N;
  int level;
  long long slot;      // next slot to scan at `level`
  long long emitted;   // BFS positions handed out so far
  __device__ void init(long long n) { N = n; level = 0; slot = 0; emitted = 0; }
  __device__ bool next(int lane, long long* my_idx, unsigned* mask, long long* pos0) {
    while (emitted < N) {
      if (level > 62) return false;   // unreachable for a correct midpoint tree; never loop forever
      long long lvl_slots = 1ll << level;
      if (slot >= lvl_slots) { level++; slot = 0; continue; }
      long long sl = slot + lane;
      long long v = (sl < lvl_slots) ? bfs_node(N, level, sl) : -1;
      unsigned m = __ballot_sync(MRMG_FULL, v >= 0);
      slot += 32;
      if (!m) continue;
      *my_idx = v;
      *mask = m;
      *pos0 = emitted;
      emitted += __popc(m);
      return true;
    }
    return false;
  }
};

__device__ __forceinline__ float warp_min(float v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v = fminf(v, __shfl_xor_sync(MRMG_FULL, v, o));
  return v;
}

__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v = fmaxf(v, __shfl_xor_sync(MRMG_FULL, v, o));
  return v;
}

__device__ __forceinline__ double warp_max_d(double v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v = fmax(v, __shfl_xor_sync(MRMG_FULL, v, o));
  return v;
}

// Step count N = max(2, int(m / res) + 1) of an edge from FP32 values, when
// that is certain (abstract_env.py:321-323).  m32 = fl32(m), m the FP64
// max |q2 - q1| (for FP32 endpoints the FP64 difference is exact), res32 =
// fl32(res): with both normal, t32 = m32 / res32 lies within a relative
// 4 * 2^-24 of the FP64 quotient, so when t32 is farther than
// 4.8e-7 * max(t32, 1) from an integer both have the same integer part.
// False when that is not shown (the caller divides in FP64).
__device__ __forceinline__ bool steps_fp32(float m32, bool anynan, float res32, long long* N) {
  if (anynan || !(res32 >= 0x1p-60f) || !(m32 >= 0x1p-60f)) return false;
  const float t32 = __fdiv_rn(m32, res32);
  if (!(t32 < 4194304.f)) return false;
  const float fl = floorf(t32);
  const float fr = t32 - fl;
  const float tol = 4.8e-7f * fmaxf(t32, 1.f);
  if (!(fr > tol && fr < 1.f - tol)) return false;
  *N = max(2, (int)fl + 1);   // through int32: fl < 2^22
  return true;
}

// Per-item verdict codes written by the FP32 pass.
enum : uint8_t { V_COLLIDE = 0, V_FREE = 1, V_PENDING = 2 };

// Device-side error bits (ored into the call's status word).
enum : int { E_BAD_INPUT = 1, E_N_START = 2, E_TIMEOUT = 4 };

}  // namespace mrmg
