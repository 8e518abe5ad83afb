// mrmg_pen.cu -- smoothed path-penetration cost of sphere-arm paths and its
// gradient through forward kinematics.
//
// There is no counterpart in the reference; the consumer is path shortcutting
// and repair (robot_mode_shortcut, planners/shortcutting.py:87-244).  For a
// path w[0..T-1] (each a full joint vector):
//
//   cost = sum_t sum_pairs softplus(beta (margin - d)) / (beta scale)
//        + smooth_w * sum_t |w[t+1] - w[t]|^2
//
// over every sphere-box pair (d = box signed distance of the centre minus the
// radius) and every pair of spheres on different robots (d = centre distance
// minus both radii).  With beta = 1 this is softplus(margin - d) / scale.
//
// One CTA per segment of 32 consecutive waypoints of one path, one waypoint per
// lane: forward kinematics runs per segment (warp r walks robot r's chain for
// its 32 waypoints) and is recomputed, not stored, when the gradient is asked
// for.  The gradient of a joint angle theta_k follows the geometric Jacobian:
// with o, z the origin and z axis of frame k-1 and g_s = dcost/dc_s,
//   dcost/dtheta_k = z . sum_{s beyond joint k} (c_s - o) x g_s
//                  = z . (M - o x G),  M = sum c_s x g_s,  G = sum g_s,
// accumulated from the tip back.  FP32 throughout; per-lane sums are
// compensated and segment totals are added in FP64 in a fixed order, so the
// cost and gradient are deterministic (no atomics: with the gradient, each
// inter-robot pair is evaluated from both sides).
#include <algorithm>

#include "mrmg_internal.cuh"

namespace mrmg {
namespace {

constexpr int kSeg = 32;   // waypoints per CTA

__host__ __device__ inline size_t al4(size_t n) { return (n + 3) & ~(size_t)3; }

// shared memory layout, in floats (every region a multiple of 16 bytes).
// The gradient regions cover the Sg spheres and Rg robots whose gradients
// the launch computes (all of them, or one group of robots of a scene too
// large for one CTA's shared memory).
struct PenLayout {
  size_t C, G, OZ, W, QG, sph, box, task, br, part, total;
  __host__ __device__ PenLayout(int S, int B, int D, bool grad, int warps, int Sg, int Rg) {
    size_t o = 0;
    C = o;   o += (size_t)S * 3 * kSeg;                          // sphere centres [S*3][32]
    G = o;   o += grad ? (size_t)Sg * 3 * kSeg : 0;              // dcost/dcentre  [Sg*3][32]
    OZ = o;  o += grad ? (size_t)Rg * kMaxLinks * 6 * kSeg : 0;  // frame origin, z axis [Rg][L][6][32]
    W = o;   o += al4((size_t)(kSeg + 2) * D);                   // waypoints t0-1 .. t0+32
    QG = o;  o += grad ? al4((size_t)kSeg * D) : 0;              // obstacle gradient [32][D]
    sph = o; o += (size_t)S * 4;
    box = o; o += (size_t)B * 8;
    task = o; o += (size_t)S * 4;                               // at most S tasks (int4)
    br = o;  o += al4((size_t)S);                               // beta log2(e) radius
    part = o; o += (size_t)warps * kSeg * 2;
    total = o;
  }
};

__host__ __device__ inline int pen_first_sphere(const PenDev& pd, int R, int r) { return r < R ? pd.lk[r][0] : pd.S; }

// MUFU approximations (PTX): 2^x, log2, sqrt, 1/sqrt, 1/x
__device__ __forceinline__ float ex2a(float x) { float y; asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x)); return y; }
__device__ __forceinline__ float lg2a(float x) { float y; asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x)); return y; }
__device__ __forceinline__ float sqrta(float x) { float y; asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x)); return y; }
__device__ __forceinline__ float rsqa(float x) { float y; asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x)); return y; }
__device__ __forceinline__ float rcpa(float x) { float y; asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x)); return y; }

// Pair terms in base-2 units.  With x2 = beta log2(e) (margin - d) and
// e = 2^-|x2|:  softplus(beta (margin - d)) = ln 2 * (max(x2, 0) + log2(1 + e))
// and sigmoid(beta (margin - d)) = 1 / (1 + e) for x2 >= 0, e / (1 + e) else.
// K folds the constant part: x2 = K - beta log2(e) * (distance).
//
// A task's two spheres are evaluated together in packed FP32x2 arithmetic
// (.x = first sphere, .y = second): one add / multiply / FMA instruction does
// both; min/max, abs and the special functions stay per component.
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 bc2(float v) { return make_float2(v, v); }

struct PairAcc2 {
  float2 ps;           // sums of max(x2, 0) + log2(1 + e)
  float2 gx, gy, gz;   // dcost / dcentre
};

// softplus (base 2) of x2 into ps; sigmoid-based dterm/d(distance) into w
template <bool COST, bool GRAD>
__device__ __forceinline__ void term2(float2 x2, float inv_scale, float2& ps, float2& w) {
  const float2 e = make_float2(ex2a(-fabsf(x2.x)), ex2a(-fabsf(x2.y)));
  const float2 ope = add2(e, bc2(1.f));
  if (COST)
    ps = add2(ps, add2(make_float2(fmaxf(x2.x, 0.f), fmaxf(x2.y, 0.f)), make_float2(lg2a(ope.x), lg2a(ope.y))));
  if (GRAD) {
    const float2 r = make_float2(rcpa(ope.x), rcpa(ope.y));
    const float2 er = mul2(e, r);
    w = mul2(make_float2(x2.x >= 0.f ? r.x : er.x, x2.y >= 0.f ? r.y : er.y), bc2(-inv_scale));
  }
}

template <bool COST, bool GRAD>
__device__ __forceinline__ void box_pair2(float2 cx, float2 cy, float2 cz, const float4& bc, const float4& bh,
                                          float2 nbl, float2 K, float inv_scale, PairAcc2& acc) {
  const float2 dx = add2(cx, bc2(-bc.x)), dy = add2(cy, bc2(-bc.y)), dz = add2(cz, bc2(-bc.z));
  const float2 ax = make_float2(fabsf(dx.x) - bh.x, fabsf(dx.y) - bh.x);
  const float2 ay = make_float2(fabsf(dy.x) - bh.y, fabsf(dy.y) - bh.y);
  const float2 az = make_float2(fabsf(dz.x) - bh.z, fabsf(dz.y) - bh.z);
  const float2 ux = make_float2(fmaxf(ax.x, 0.f), fmaxf(ax.y, 0.f));
  const float2 uy = make_float2(fmaxf(ay.x, 0.f), fmaxf(ay.y, 0.f));
  const float2 uz = make_float2(fmaxf(az.x, 0.f), fmaxf(az.y, 0.f));
  const float2 u2 = fma2(ux, ux, fma2(uy, uy, mul2(uz, uz)));
  const float2 mx = make_float2(fmaxf(ax.x, fmaxf(ay.x, az.x)), fmaxf(ax.y, fmaxf(ay.y, az.y)));
  float2 w;
  if (!GRAD) {
    // signed distance of the box: |max(q, 0)| + min(max_k q_k, 0)
    const float2 sdf = add2(make_float2(sqrta(u2.x), sqrta(u2.y)), make_float2(fminf(mx.x, 0.f), fminf(mx.y, 0.f)));
    term2<COST, false>(fma2(nbl, sdf, K), inv_scale, acc.ps, w);
  } else {
    const float2 inv = make_float2(rsqa(fmaxf(u2.x, 1e-30f)), rsqa(fmaxf(u2.y, 1e-30f)));
    const float2 ui = mul2(u2, inv);
    const bool ox = mx.x > 0.f, oy = mx.y > 0.f;
    const float2 sdf = make_float2(ox ? ui.x : mx.x, oy ? ui.y : mx.y);
    term2<COST, true>(fma2(nbl, sdf, K), inv_scale, acc.ps, w);
    // d(distance)/dc: the unit vector of max(q, 0) outside, the axis of the
    // largest q inside; both with the signs of c - centre
    float2 sx = mul2(ux, inv), sy = mul2(uy, inv), sz = mul2(uz, inv);
    if (!ox) {
      const bool bx = ax.x >= ay.x && ax.x >= az.x, by = !bx && ay.x >= az.x;
      sx.x = bx ? 1.f : 0.f; sy.x = by ? 1.f : 0.f; sz.x = (!bx && !by) ? 1.f : 0.f;
    }
    if (!oy) {
      const bool bx = ax.y >= ay.y && ax.y >= az.y, by = !bx && ay.y >= az.y;
      sx.y = bx ? 1.f : 0.f; sy.y = by ? 1.f : 0.f; sz.y = (!bx && !by) ? 1.f : 0.f;
    }
    acc.gx = fma2(w, make_float2(copysignf(sx.x, dx.x), copysignf(sx.y, dx.y)), acc.gx);
    acc.gy = fma2(w, make_float2(copysignf(sy.x, dy.x), copysignf(sy.y, dy.y)), acc.gy);
    acc.gz = fma2(w, make_float2(copysignf(sz.x, dz.x), copysignf(sz.y, dz.y)), acc.gz);
  }
}

template <bool COST, bool GRAD>
__device__ __forceinline__ void sphere_pair2(float2 cx, float2 cy, float2 cz, float jx, float jy, float jz, float2 nbl,
                                             float2 K, float inv_scale, PairAcc2& acc) {
  const float2 vx = add2(cx, bc2(-jx)), vy = add2(cy, bc2(-jy)), vz = add2(cz, bc2(-jz));
  const float2 d2 = fma2(vx, vx, fma2(vy, vy, mul2(vz, vz)));
  float2 w;
  if (!GRAD) {
    term2<COST, false>(fma2(nbl, make_float2(sqrta(d2.x), sqrta(d2.y)), K), inv_scale, acc.ps, w);
  } else {
    const float2 inv = make_float2(rsqa(fmaxf(d2.x, 1e-30f)), rsqa(fmaxf(d2.y, 1e-30f)));
    term2<COST, true>(fma2(nbl, mul2(d2, inv), K), inv_scale, acc.ps, w);
    const float2 f = mul2(w, inv);
    acc.gx = fma2(f, vx, acc.gx);
    acc.gy = fma2(f, vy, acc.gy);
    acc.gz = fma2(f, vz, acc.gz);
  }
}

__device__ __forceinline__ void acc2(float& h, float& l, float v) {
  float s, e;
  two_sum(h, v, &s, &e);
  h = s;
  l += e;
}

// the cost kernel fits two 16-warp CTAs per SM (shared memory allows it when
// the registers stay at 64); the gradient kernel holds twice the tables
template <bool COST, bool GRAD>
__global__ void __launch_bounds__(512, GRAD ? 1 : 2)
    pen_kernel(ArmDev a, PenDev pd, PenParams pp, const float* __restrict__ paths, int T, int nseg,
               const float* __restrict__ gout, double* __restrict__ seg_cost, float* __restrict__ wp_cost,
               float* __restrict__ grad, int gr0, int gr1) {
  extern __shared__ __align__(16) float smf[];
  const int S = pd.S, B = pd.B, R = a.R, D = a.D;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, NW = blockDim.x >> 5;
  const long long p = blockIdx.x / nseg;
  const int seg = blockIdx.x - (int)(p * nseg);
  const int t0 = seg * kSeg;
  // the gradient of this launch: robots [gr0, gr1), their spheres [s_lo, s_hi)
  // and joints [j_lo, j_hi) (robots' joints are contiguous in robot order)
  const int s_lo = pen_first_sphere(pd, R, gr0), s_hi = pen_first_sphere(pd, R, gr1);
  const int j_lo = a.q_off[gr0], j_hi = gr1 < R ? a.q_off[gr1] : D;
  const PenLayout L(S, B, D, GRAD, NW, s_hi - s_lo, gr1 - gr0);
  float* C = smf + L.C;
  float* Gs = smf + L.G;
  float* OZ = smf + L.OZ;
  float* W = smf + L.W;
  float* QG = smf + L.QG;
  float4* sph = (float4*)(smf + L.sph);
  float4* box = (float4*)(smf + L.box);
  int4* tasks = (int4*)(smf + L.task);
  float* br = smf + L.br;
  const int NTK = pd.NTK;
  float* part = smf + L.part;

  // ---- stage tables and the segment's waypoints (rows t0-1 .. t0+32)
  for (int i = tid; i < S; i += blockDim.x) {
    sph[i] = pd.sph[i];
    br[i] = pp.beta * 1.4426950408889634f * pd.sph[i].w;
  }
  for (int i = tid; i < NTK; i += blockDim.x) tasks[i] = pd.task[i];
  for (int i = tid; i < 2 * B; i += blockDim.x) box[i] = pd.box[i];
  {
    const float* src = paths + (size_t)p * T * D;
    const int n = (kSeg + 2) * D;
    for (int i = tid; i < n; i += blockDim.x) {
      const int t = t0 - 1 + i / D;
      W[i] = (t >= 0 && t < T) ? src[(long long)(t0 - 1) * D + i] : 0.f;
    }
  }
  if (GRAD)
    for (int i = tid; i < kSeg * D; i += blockDim.x) QG[i] = 0.f;
  __syncthreads();

  // ---- forward kinematics: warp r walks robot r's chain, lane = waypoint
  if (warp < R) {
    const int r = warp;
    const float* q = W + (lane + 1) * D;
    int jo = a.q_off[r];
    float m[9], o[3];
    {
      const float4 b0 = a.base32[3 * r], b1 = a.base32[3 * r + 1], b2 = a.base32[3 * r + 2];
      if (a.base_kind[r] == 1) {
        float sn, cs;
        sincosf(a.off32 ? q[jo + 2] + a.off32[jo + 2].x : q[jo + 2], &sn, &cs);
        m[0] = cs * b0.x - sn * b1.x; m[1] = cs * b0.y - sn * b1.y; m[2] = cs * b0.z - sn * b1.z;
        m[3] = sn * b0.x + cs * b1.x; m[4] = sn * b0.y + cs * b1.y; m[5] = sn * b0.z + cs * b1.z;
        m[6] = b2.x; m[7] = b2.y; m[8] = b2.z;
        o[0] = q[jo] + (cs * b0.w - sn * b1.w);
        o[1] = q[jo + 1] + (sn * b0.w + cs * b1.w);
        o[2] = b2.w;
        jo += 3;
      } else {
        m[0] = b0.x; m[1] = b0.y; m[2] = b0.z; m[3] = b1.x; m[4] = b1.y; m[5] = b1.z;
        m[6] = b2.x; m[7] = b2.y; m[8] = b2.z;
        o[0] = b0.w; o[1] = b1.w; o[2] = b2.w;
      }
    }
    const int nl = a.nl[r];
    for (int k = 0; k <= nl; k++) {
      if (k > 0) {
        if (GRAD && r >= gr0 && r < gr1) {
          float* oz = OZ + (size_t)(((r - gr0) * kMaxLinks + (k - 1)) * 6) * kSeg + lane;
          oz[0] = o[0]; oz[kSeg] = o[1]; oz[2 * kSeg] = o[2];
          oz[3 * kSeg] = m[2]; oz[4 * kSeg] = m[5]; oz[5 * kSeg] = m[8];
        }
        const float4 h = a.dh32[r * kMaxLinks + k - 1];   // a, d, cos(alpha), sin(alpha)
        float sn, cs;
        sincosf(a.off32 ? q[jo + k - 1] + a.off32[jo + k - 1].x : q[jo + k - 1], &sn, &cs);
        const float sca = sn * h.z, cca = cs * h.z, ssa = sn * h.w, csa = cs * h.w;
        const float ac = h.x * cs, as = h.x * sn;
#pragma unroll
        for (int i = 0; i < 3; i++) {
          const float r0 = m[3 * i], r1 = m[3 * i + 1], r2 = m[3 * i + 2];
          m[3 * i] = r0 * cs + r1 * sn;
          m[3 * i + 1] = (r1 * cca - r0 * sca) + r2 * h.w;
          m[3 * i + 2] = (r0 * ssa - r1 * csa) + r2 * h.z;
          o[i] += (r0 * ac + r1 * as) + r2 * h.y;
        }
      }
      for (int s = pd.lk[r][k]; s < pd.lk[r][k + 1]; s++) {
        const float4 l = sph[s];
#pragma unroll
        for (int i = 0; i < 3; i++)
          C[(3 * s + i) * kSeg + lane] = o[i] + ((m[3 * i] * l.x + m[3 * i + 1] * l.y) + m[3 * i + 2] * l.z);
      }
    }
  }
  __syncthreads();

  // ---- pair terms.  A task is one or two spheres of one robot, lane =
  // waypoint; its warp evaluates them against every box and every sphere of
  // the other robots.  With the gradient, each inter-robot pair is evaluated
  // from both sides, so a task owns its spheres' gradients outright (no
  // atomics, a fixed summation order); the cost counts each pair once (the
  // partners on later robots).  Tasks are dealt zig-zag over the warps.
  const float bl = pp.beta * 1.4426950408889634f;   // beta log2(e)
  const float blm = bl * pp.margin;
  float acc_h = 0.f, acc_l = 0.f;
  for (int base = 0; base < NTK; base += NW) {
    const int tk = ((base / NW) & 1) ? base + NW - 1 - warp : base + warp;
    if (tk >= NTK) continue;
    const int4 task = tasks[tk];   // sphere, second sphere (-1: none), robot's first sphere, next robot's first
    if (GRAD && !COST && (task.x < s_lo || task.x >= s_hi)) continue;   // another group's robot
    const bool two = task.y >= 0;
    const int i0 = task.x, i1 = two ? task.y : task.x;
    const float2 cx = make_float2(C[(3 * i0) * kSeg + lane], C[(3 * i1) * kSeg + lane]);
    const float2 cy = make_float2(C[(3 * i0 + 1) * kSeg + lane], C[(3 * i1 + 1) * kSeg + lane]);
    const float2 cz = make_float2(C[(3 * i0 + 2) * kSeg + lane], C[(3 * i1 + 2) * kSeg + lane]);
    const float2 K = make_float2(fmaf(bl, sph[i0].w, blm), fmaf(bl, sph[i1].w, blm));
    const float2 nbl = bc2(-bl);
    PairAcc2 a{bc2(0.f), bc2(0.f), bc2(0.f), bc2(0.f)};
#pragma unroll 2
    for (int b = 0; b < B; b++)
      box_pair2<COST, GRAD>(cx, cy, cz, box[2 * b], box[2 * b + 1], nbl, K, pp.inv_scale, a);
#pragma unroll 2
    for (int j = task.w; j < S; j++)
      sphere_pair2<COST, GRAD>(cx, cy, cz, C[(3 * j) * kSeg + lane], C[(3 * j + 1) * kSeg + lane],
                               C[(3 * j + 2) * kSeg + lane], nbl, add2(K, bc2(br[j])), pp.inv_scale, a);
    if (GRAD) {
#pragma unroll 2
      for (int j = 0; j < task.z; j++)
        sphere_pair2<false, true>(cx, cy, cz, C[(3 * j) * kSeg + lane], C[(3 * j + 1) * kSeg + lane],
                                  C[(3 * j + 2) * kSeg + lane], nbl, add2(K, bc2(br[j])), pp.inv_scale, a);
      const int g0 = i0 - s_lo, g1 = i1 - s_lo;
      Gs[(3 * g0) * kSeg + lane] = a.gx.x;
      Gs[(3 * g0 + 1) * kSeg + lane] = a.gy.x;
      Gs[(3 * g0 + 2) * kSeg + lane] = a.gz.x;
      if (two) {
        Gs[(3 * g1) * kSeg + lane] = a.gx.y;
        Gs[(3 * g1 + 1) * kSeg + lane] = a.gy.y;
        Gs[(3 * g1 + 2) * kSeg + lane] = a.gz.y;
      }
    }
    if (COST) acc2(acc_h, acc_l, two ? a.ps.x + a.ps.y : a.ps.x);
  }
  if (COST) {
    part[warp * kSeg + lane] = acc_h;
    part[(NW + warp) * kSeg + lane] = acc_l;
  }
  __syncthreads();

  const int t = t0 + lane;
  if (COST && warp == 0) {
    double c = 0.0;
    for (int w = 0; w < NW; w++) c += (double)part[w * kSeg + lane] + (double)part[(NW + w) * kSeg + lane];
    c *= 0.69314718055994531 * (double)pp.inv_beta * (double)pp.inv_scale;   // ln 2 / (beta scale)
    if (t + 1 < T) {
      const float* w0 = W + (lane + 1) * D;
      const float* w1 = W + (lane + 2) * D;
      float sh = 0.f, sl = 0.f;
      for (int k = 0; k < D; k++) {
        const float dv = w1[k] - w0[k];
        acc2(sh, sl, dv * dv);
      }
      c += (double)pp.smooth_w * ((double)sh + (double)sl);
    }
    if (t >= T) c = 0.0;
    if (wp_cost && t < T) wp_cost[(size_t)p * T + t] = (float)c;
#pragma unroll
    for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(MRMG_FULL, c, o);
    if (lane == 0 && seg_cost) seg_cost[(size_t)p * nseg + seg] = c;
  }

  if (GRAD) {
    // ---- joint gradients from the sphere gradients, tip to base
    if (warp >= gr0 && warp < gr1) {
      const int r = warp;
      const int nl = a.nl[r];
      int jo = a.q_off[r] + (a.base_kind[r] == 1 ? 3 : 0);
      float G0 = 0.f, G1 = 0.f, G2 = 0.f, M0 = 0.f, M1 = 0.f, M2 = 0.f;
      float* qg = QG + lane * D;
      for (int k = nl; k >= 0; k--) {
        for (int s = pd.lk[r][k]; s < pd.lk[r][k + 1]; s++) {
          const float c0 = C[(3 * s) * kSeg + lane], c1 = C[(3 * s + 1) * kSeg + lane], c2 = C[(3 * s + 2) * kSeg + lane];
          const int sg = s - s_lo;
          const float g0 = Gs[(3 * sg) * kSeg + lane], g1 = Gs[(3 * sg + 1) * kSeg + lane], g2 = Gs[(3 * sg + 2) * kSeg + lane];
          G0 += g0; G1 += g1; G2 += g2;
          M0 += c1 * g2 - c2 * g1;
          M1 += c2 * g0 - c0 * g2;
          M2 += c0 * g1 - c1 * g0;
        }
        if (k == 0) break;
        const float* oz = OZ + (size_t)(((r - gr0) * kMaxLinks + (k - 1)) * 6) * kSeg + lane;
        const float o0 = oz[0], o1 = oz[kSeg], o2 = oz[2 * kSeg];
        const float z0 = oz[3 * kSeg], z1 = oz[4 * kSeg], z2 = oz[5 * kSeg];
        const float v0 = M0 - (o1 * G2 - o2 * G1), v1 = M1 - (o2 * G0 - o0 * G2), v2 = M2 - (o0 * G1 - o1 * G0);
        qg[jo + k - 1] = z0 * v0 + z1 * v1 + z2 * v2;
      }
      if (a.base_kind[r] == 1) {
        const int b0 = a.q_off[r];
        const float x = W[(lane + 1) * D + b0], y = W[(lane + 1) * D + b0 + 1];
        qg[b0] = G0;
        qg[b0 + 1] = G1;
        qg[b0 + 2] = M2 - (x * G1 - y * G0);
      }
    }
    __syncthreads();
    // ---- add the smoothness gradient, scale by dL/dcost, write coalesced
    const float go = gout ? gout[p] : 1.f;
    const float sw2 = 2.f * pp.smooth_w;
    const int n = kSeg * D;
    float* dst = grad + ((size_t)p * T + t0) * D;
    for (int i = tid; i < n; i += blockDim.x) {
      const int tt = t0 + i / D;
      if (tt >= T) break;
      const int j = i - (i / D) * D;
      if (j < j_lo || j >= j_hi) continue;   // another group's joint
      const float wc = W[i + D];
      float gsm = 0.f;
      if (tt > 0) gsm += sw2 * (wc - W[i]);
      if (tt + 1 < T) gsm -= sw2 * (W[i + 2 * D] - wc);
      dst[i] = go * (QG[i] + gsm);
    }
  }
}

__global__ void pen_sum_kernel(const double* __restrict__ seg, long long P, int nseg, double* __restrict__ cost) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < P; p += (long long)gridDim.x * blockDim.x) {
    double c = 0.0;
    for (int s = 0; s < nseg; s++) c += seg[p * nseg + s];
    cost[p] = c;
  }
}

template <bool COST, bool GRAD>
cudaError_t launch_one(const ArmDev& a, const PenDev& pd, const PenParams& pp, const float* paths, long long P, int T,
                       int nseg, const float* gout, double* seg, float* wp, float* grad, int warps, int gr0, int gr1,
                       cudaStream_t st) {
  const PenLayout L(pd.S, pd.B, a.D, GRAD, warps, pen_first_sphere(pd, a.R, gr1) - pen_first_sphere(pd, a.R, gr0),
                    gr1 - gr0);
  const size_t smem = L.total * sizeof(float);
  cudaError_t e = cudaFuncSetAttribute(pen_kernel<COST, GRAD>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  pen_kernel<COST, GRAD><<<(unsigned)(P * nseg), warps * 32, smem, st>>>(a, pd, pp, paths, T, nseg, gout, seg, wp, grad,
                                                                          gr0, gr1);
  return cudaGetLastError();
}

}  // namespace

size_t pen_smem_bytes(const ArmDev& a, const PenDev& pd, int grad, int warps, int gr0, int gr1) {
  return PenLayout(pd.S, pd.B, a.D, grad != 0, warps, pen_first_sphere(pd, a.R, gr1) - pen_first_sphere(pd, a.R, gr0),
                   gr1 - gr0).total * sizeof(float);
}

int pen_grad_groups(const ArmDev& a, const PenDev& pd, int warps, size_t smem_max, int* bounds) {
  // joints must be contiguous in robot order for the groups' joint ranges
  int jo = 0;
  for (int r = 0; r < a.R; r++) {
    if (a.q_off[r] != jo) return a.R == 1 || pen_smem_bytes(a, pd, 1, warps, 0, a.R) <= smem_max ? 1 : 0;
    jo += (a.base_kind[r] == 1 ? 3 : 0) + a.nl[r];
  }
  if (jo != a.D) return pen_smem_bytes(a, pd, 1, warps, 0, a.R) <= smem_max ? 1 : 0;
  // fewest groups of consecutive robots (balanced by count) whose gradient regions fit
  for (int ng = 1; ng <= a.R; ng++) {
    bool ok = true;
    for (int g = 0; g <= ng; g++) bounds[g] = g * a.R / ng;
    for (int g = 0; g < ng && ok; g++) ok = pen_smem_bytes(a, pd, 1, warps, bounds[g], bounds[g + 1]) <= smem_max;
    if (ok) return ng;
  }
  return 0;
}

cudaError_t pen_launch(const ArmDev& a, const PenDev& pd, const PenParams& pp, const float* paths, long long P, int T,
                       const float* gout, double* seg, double* cost, float* wp_cost, float* grad, int warps,
                       int n_groups, const int* bounds, cudaStream_t st) {
  if (P <= 0) return cudaSuccess;
  const int nseg = (T + kSeg - 1) / kSeg;
  const bool want_cost = cost || wp_cost;
  cudaError_t e = cudaSuccess;
  if (grad && n_groups <= 1) {
    if (want_cost) e = launch_one<true, true>(a, pd, pp, paths, P, T, nseg, gout, seg, wp_cost, grad, warps, 0, a.R, st);
    else e = launch_one<false, true>(a, pd, pp, paths, P, T, nseg, gout, nullptr, nullptr, grad, warps, 0, a.R, st);
  } else {
    if (want_cost || !grad)
      e = launch_one<true, false>(a, pd, pp, paths, P, T, nseg, gout, seg, wp_cost, nullptr, warps, 0, a.R, st);
    for (int g = 0; grad && g < n_groups && e == cudaSuccess; g++)
      e = launch_one<false, true>(a, pd, pp, paths, P, T, nseg, gout, nullptr, nullptr, grad, warps, bounds[g],
                                  bounds[g + 1], st);
  }
  if (e != cudaSuccess || !cost) return e;
  const int blocks = (int)std::min<long long>((P + 255) / 256, 4096);
  pen_sum_kernel<<<blocks, 256, 0, st>>>(seg, P, nseg, cost);
  return cudaGetLastError();
}

}  // namespace mrmg
