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

// shared memory layout, in floats (every region a multiple of 16 bytes)
struct PenLayout {
  size_t C, G, OZ, W, QG, sph, box, task, br, part, total;
  __host__ __device__ PenLayout(int S, int B, int R, int D, bool grad, int warps) {
    size_t o = 0;
    C = o;   o += (size_t)S * 3 * kSeg;                         // sphere centres [S*3][32]
    G = o;   o += grad ? (size_t)S * 3 * kSeg : 0;              // dcost/dcentre  [S*3][32]
    OZ = o;  o += grad ? (size_t)R * kMaxLinks * 6 * kSeg : 0;  // frame origin, z axis [R][L][6][32]
    W = o;   o += al4((size_t)(kSeg + 2) * D);                  // waypoints t0-1 .. t0+32
    QG = o;  o += grad ? al4((size_t)kSeg * D) : 0;             // obstacle gradient [32][D]
    sph = o; o += (size_t)S * 4;
    box = o; o += (size_t)B * 8;
    task = o; o += (size_t)S * 4;                              // at most S tasks (int4)
    br = o;  o += al4((size_t)S);                              // beta log2(e) radius
    part = o; o += (size_t)warps * kSeg * 2;
    total = o;
  }
};

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
struct PairAcc {
  float ps;            // sum of max(x2, 0) + log2(1 + e)
  float gx, gy, gz;    // dcost / dcentre
};

template <bool COST, bool GRAD>
__device__ __forceinline__ void box_pair(float cx, float cy, float cz, const float4& bc, const float4& bh, float bl,
                                         float K, float inv_scale, PairAcc& acc) {
  const float dx = cx - bc.x, dy = cy - bc.y, dz = cz - bc.z;
  const float ax = fabsf(dx) - bh.x, ay = fabsf(dy) - bh.y, az = fabsf(dz) - bh.z;
  const float ux = fmaxf(ax, 0.f), uy = fmaxf(ay, 0.f), uz = fmaxf(az, 0.f);
  const float u2 = fmaf(ux, ux, fmaf(uy, uy, uz * uz));
  const float mx = fmaxf(ax, fmaxf(ay, az));
  if (!GRAD) {
    // signed distance of the box: |max(q, 0)| + min(max_k q_k, 0)
    const float x2 = fmaf(-bl, sqrta(u2) + fminf(mx, 0.f), K);
    const float e = ex2a(-fabsf(x2));
    acc.ps += fmaxf(x2, 0.f) + lg2a(1.f + e);
  } else {
    const float inv = rsqa(fmaxf(u2, 1e-30f));
    const bool outside = mx > 0.f;
    const float x2 = fmaf(-bl, outside ? u2 * inv : mx, K);
    const float e = ex2a(-fabsf(x2));
    if (COST) acc.ps += fmaxf(x2, 0.f) + lg2a(1.f + e);
    const float r = rcpa(1.f + e);
    const float w = -(x2 >= 0.f ? r : e * r) * inv_scale;   // dterm / d(distance)
    // d(distance)/dc: the unit vector of max(q, 0) outside, the axis of the
    // largest q inside; both with the signs of c - centre
    float sx, sy, sz;
    if (outside) {
      sx = ux * inv; sy = uy * inv; sz = uz * inv;
    } else {
      const bool bx = ax >= ay && ax >= az, by = !bx && ay >= az;
      sx = bx ? 1.f : 0.f; sy = by ? 1.f : 0.f; sz = (!bx && !by) ? 1.f : 0.f;
    }
    acc.gx = fmaf(w, copysignf(sx, dx), acc.gx);
    acc.gy = fmaf(w, copysignf(sy, dy), acc.gy);
    acc.gz = fmaf(w, copysignf(sz, dz), acc.gz);
  }
}

template <bool COST, bool GRAD>
__device__ __forceinline__ void sphere_pair(float cx, float cy, float cz, float jx, float jy, float jz, float bl, float K,
                                            float inv_scale, PairAcc& acc) {
  const float vx = cx - jx, vy = cy - jy, vz = cz - jz;
  const float d2 = fmaf(vx, vx, fmaf(vy, vy, vz * vz));
  if (!GRAD) {
    const float x2 = fmaf(-bl, sqrta(d2), K);
    const float e = ex2a(-fabsf(x2));
    acc.ps += fmaxf(x2, 0.f) + lg2a(1.f + e);
  } else {
    const float inv = rsqa(fmaxf(d2, 1e-30f));
    const float x2 = fmaf(-bl, d2 * inv, K);
    const float e = ex2a(-fabsf(x2));
    if (COST) acc.ps += fmaxf(x2, 0.f) + lg2a(1.f + e);
    const float r = rcpa(1.f + e);
    const float f = -(x2 >= 0.f ? r : e * r) * inv_scale * inv;
    acc.gx = fmaf(f, vx, acc.gx);
    acc.gy = fmaf(f, vy, acc.gy);
    acc.gz = fmaf(f, vz, acc.gz);
  }
}

__device__ __forceinline__ void acc2(float& h, float& l, float v) {
  float s, e;
  two_sum(h, v, &s, &e);
  h = s;
  l += e;
}

template <bool COST, bool GRAD>
__global__ void __launch_bounds__(512, 1)
    pen_kernel(ArmDev a, PenDev pd, PenParams pp, const float* __restrict__ paths, int T, int nseg,
               const float* __restrict__ gout, double* __restrict__ seg_cost, float* __restrict__ wp_cost,
               float* __restrict__ grad) {
  extern __shared__ __align__(16) float smf[];
  const int S = pd.S, B = pd.B, R = a.R, D = a.D;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, NW = blockDim.x >> 5;
  const long long p = blockIdx.x / nseg;
  const int seg = blockIdx.x - (int)(p * nseg);
  const int t0 = seg * kSeg;
  const PenLayout L(S, B, R, D, GRAD, NW);
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
        sincosf(q[jo + 2], &sn, &cs);
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
        if (GRAD) {
          float* oz = OZ + (size_t)((r * kMaxLinks + (k - 1)) * 6) * kSeg + lane;
          oz[0] = o[0]; oz[kSeg] = o[1]; oz[2 * kSeg] = o[2];
          oz[3 * kSeg] = m[2]; oz[4 * kSeg] = m[5]; oz[5 * kSeg] = m[8];
        }
        const float4 h = a.dh32[r * kMaxLinks + k - 1];   // a, d, cos(alpha), sin(alpha)
        float sn, cs;
        sincosf(q[jo + k - 1], &sn, &cs);
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
    const bool two = task.y >= 0;
    const int i0 = task.x, i1 = two ? task.y : task.x;
    const float c0x = C[(3 * i0) * kSeg + lane], c0y = C[(3 * i0 + 1) * kSeg + lane], c0z = C[(3 * i0 + 2) * kSeg + lane];
    const float c1x = C[(3 * i1) * kSeg + lane], c1y = C[(3 * i1 + 1) * kSeg + lane], c1z = C[(3 * i1 + 2) * kSeg + lane];
    const float K0 = fmaf(bl, sph[i0].w, blm), K1 = fmaf(bl, sph[i1].w, blm);
    PairAcc a0{0.f, 0.f, 0.f, 0.f}, a1{0.f, 0.f, 0.f, 0.f};
#pragma unroll 2
    for (int b = 0; b < B; b++) {
      const float4 bc = box[2 * b], bh = box[2 * b + 1];
      box_pair<COST, GRAD>(c0x, c0y, c0z, bc, bh, bl, K0, pp.inv_scale, a0);
      box_pair<COST, GRAD>(c1x, c1y, c1z, bc, bh, bl, K1, pp.inv_scale, a1);
    }
#pragma unroll 2
    for (int j = task.w; j < S; j++) {
      const float jx = C[(3 * j) * kSeg + lane], jy = C[(3 * j + 1) * kSeg + lane], jz = C[(3 * j + 2) * kSeg + lane];
      const float bj = br[j];
      sphere_pair<COST, GRAD>(c0x, c0y, c0z, jx, jy, jz, bl, K0 + bj, pp.inv_scale, a0);
      sphere_pair<COST, GRAD>(c1x, c1y, c1z, jx, jy, jz, bl, K1 + bj, pp.inv_scale, a1);
    }
    if (GRAD) {
#pragma unroll 2
      for (int j = 0; j < task.z; j++) {
        const float jx = C[(3 * j) * kSeg + lane], jy = C[(3 * j + 1) * kSeg + lane], jz = C[(3 * j + 2) * kSeg + lane];
        const float bj = br[j];
        sphere_pair<false, true>(c0x, c0y, c0z, jx, jy, jz, bl, K0 + bj, pp.inv_scale, a0);
        sphere_pair<false, true>(c1x, c1y, c1z, jx, jy, jz, bl, K1 + bj, pp.inv_scale, a1);
      }
      Gs[(3 * i0) * kSeg + lane] = a0.gx;
      Gs[(3 * i0 + 1) * kSeg + lane] = a0.gy;
      Gs[(3 * i0 + 2) * kSeg + lane] = a0.gz;
      if (two) {
        Gs[(3 * i1) * kSeg + lane] = a1.gx;
        Gs[(3 * i1 + 1) * kSeg + lane] = a1.gy;
        Gs[(3 * i1 + 2) * kSeg + lane] = a1.gz;
      }
    }
    if (COST) acc2(acc_h, acc_l, two ? a0.ps + a1.ps : a0.ps);
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
    if (warp < R) {
      const int r = warp;
      const int nl = a.nl[r];
      int jo = a.q_off[r] + (a.base_kind[r] == 1 ? 3 : 0);
      float G0 = 0.f, G1 = 0.f, G2 = 0.f, M0 = 0.f, M1 = 0.f, M2 = 0.f;
      float* qg = QG + lane * D;
      for (int k = nl; k >= 0; k--) {
        for (int s = pd.lk[r][k]; s < pd.lk[r][k + 1]; s++) {
          const float c0 = C[(3 * s) * kSeg + lane], c1 = C[(3 * s + 1) * kSeg + lane], c2 = C[(3 * s + 2) * kSeg + lane];
          const float g0 = Gs[(3 * s) * kSeg + lane], g1 = Gs[(3 * s + 1) * kSeg + lane], g2 = Gs[(3 * s + 2) * kSeg + lane];
          G0 += g0; G1 += g1; G2 += g2;
          M0 += c1 * g2 - c2 * g1;
          M1 += c2 * g0 - c0 * g2;
          M2 += c0 * g1 - c1 * g0;
        }
        if (k == 0) break;
        const float* oz = OZ + (size_t)((r * kMaxLinks + (k - 1)) * 6) * kSeg + lane;
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
                       int nseg, const float* gout, double* seg, float* wp, float* grad, int warps, cudaStream_t st) {
  const size_t smem = pen_smem_bytes(pd.S, pd.B, a.R, a.D, GRAD, warps);
  cudaError_t e = cudaFuncSetAttribute(pen_kernel<COST, GRAD>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  pen_kernel<COST, GRAD><<<(unsigned)(P * nseg), warps * 32, smem, st>>>(a, pd, pp, paths, T, nseg, gout, seg, wp, grad);
  return cudaGetLastError();
}

}  // namespace

size_t pen_smem_bytes(int S, int B, int R, int D, int grad, int warps) {
  return PenLayout(S, B, R, D, grad != 0, warps).total * sizeof(float);
}

cudaError_t pen_launch(const ArmDev& a, const PenDev& pd, const PenParams& pp, const float* paths, long long P, int T,
                       const float* gout, double* seg, double* cost, float* wp_cost, float* grad, int warps,
                       cudaStream_t st) {
  if (P <= 0) return cudaSuccess;
  const int nseg = (T + kSeg - 1) / kSeg;
  const bool want_cost = cost || wp_cost;
  cudaError_t e;
  if (want_cost && grad) e = launch_one<true, true>(a, pd, pp, paths, P, T, nseg, gout, seg, wp_cost, grad, warps, st);
  else if (grad) e = launch_one<false, true>(a, pd, pp, paths, P, T, nseg, gout, nullptr, nullptr, grad, warps, st);
  else e = launch_one<true, false>(a, pd, pp, paths, P, T, nseg, gout, seg, wp_cost, nullptr, warps, st);
  if (e != cudaSuccess || !cost) return e;
  const int blocks = (int)std::min<long long>((P + 255) / 256, 4096);
  pen_sum_kernel<<<blocks, 256, 0, st>>>(seg, P, nseg, cost);
  return cudaGetLastError();
}

}  // namespace mrmg
