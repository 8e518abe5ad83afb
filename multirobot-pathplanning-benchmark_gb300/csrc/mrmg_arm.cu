// mrmg_arm.cu -- collision kernels for sphere-arm scenes: batched forward
// kinematics of DH arms carrying collision spheres, sphere-box and
// sphere-sphere (different robots) tests, configuration and edge checks.
//
// Mapping: one warp evaluates one configuration.  Lane l owns sphere groups
// g = l, l+32, ... (a group = up to SPG spheres of one robot link); it runs
// the robot's kinematic chain up to that link with the joint transforms in
// registers, then tests its spheres against every box (box tables in shared
// memory, broadcast reads).  Inter-robot group pairs are dealt round-robin to
// the lanes and read their spheres from the warp's shared sphere table.  A
// warp vote after every box and every pair round stops the configuration at
// its first certain collision.
//
// Exactness: the bulk runs in FP32 against per-sphere thresholds widened and
// narrowed by the band delta, which bounds |FP32 centre - FP64 centre|.  A
// test inside the band is pending; pass 2 recomputes the chain in FP64 with
// the operation order of the CPU restatement and decides each pending test
// exactly (Rectangle.collides_with_sphere, problems/abstract_env.py:69-84;
// agent-agent norm rule, abstract_env.py:261-268).
#include <algorithm>
#include <cstdio>

#include "mrmg_bulk.cuh"
#include "mrmg_internal.cuh"

namespace mrmg {
namespace {

constexpr float kFar = 1.0e15f;

__device__ __forceinline__ double ldq(const void* p, int dtype, long long i) {
  return dtype == MRMG_F32 ? (double)((const float*)p)[i] : ((const double*)p)[i];
}

// Shared-memory image of the scene (per CTA) --------------------------------
struct ArmSmem {
  float4* box;      // [B*2]
  float4* base;     // [R*3]
  float4* dh;       // [R*8]
  float4* sph;      // [G*SPG]
  float4* band;     // [G*SPG]
  int* grp;         // [G]
  float4* gbs;      // [G] group bounds
  uint32_t* pairs;  // [NP]
  uint32_t prismatic[3];
};

__host__ __device__ inline size_t table_bytes(const ArmDev& s) {
  size_t off[9];
  arm_table_layout(s, off);
  return off[8];
}

// per-warp FP32 work area: joint cos/sin, planar translations, sphere table
constexpr int kNearBlock = 512;   // at most this many group pairs compacted per block of the pair rounds

__host__ __device__ inline int near_block(const ArmDev& s) { return s.NP < kNearBlock ? (s.NP > 0 ? s.NP : 1) : kNearBlock; }


// the per-warp list holds the near (group, box) items of one box block, then
// the near group pairs of one pair block
__host__ __device__ inline int list_cap(const ArmDev& s) {
  return near_block(s) > s.G * s.box_block ? near_block(s) : s.G * s.box_block;
}

__host__ __device__ inline size_t warp32_bytes(const ArmDev& s) {
  return align16(sizeof(float2) * s.D) + align16(sizeof(float) * s.D) +
         align16(sizeof(float4) * s.G * s.SPG) + align16(sizeof(float) * s.G * s.SPG) +
         align16(sizeof(float4) * s.G) + align16(sizeof(uint32_t) * list_cap(s));
}

// per-warp FP64 work area for pass 2: joint values, cos/sin, sphere centres
__host__ __device__ inline size_t warp64_bytes(const ArmDev& s) {
  return align16(sizeof(double) * s.D) + align16(sizeof(double) * 2 * s.D) +
         align16(sizeof(double) * 3 * s.G * s.SPG);
}

// The FP32 tables into shared memory at `base` (arm_table_layout): one bulk
// asynchronous copy of the scene's table image, or loads when the scene has
// none (or the copy timed out).  Every thread calls it; a __syncthreads()
// must follow.
__device__ void stage_tables(const ArmDev& s, unsigned char* base, ArmSmem* t) {
  __shared__ __align__(8) uint64_t stage_bar;
  size_t off[9];
  arm_table_layout(s, off);
  t->box = (float4*)(base + off[0]);
  t->base = (float4*)(base + off[1]);
  t->dh = (float4*)(base + off[2]);
  t->sph = (float4*)(base + off[3]);
  t->band = (float4*)(base + off[4]);
  t->grp = (int*)(base + off[5]);
  t->gbs = (float4*)(base + off[6]);
  t->pairs = (uint32_t*)(base + off[7]);
  t->prismatic[0] = s.prismatic[0];
  t->prismatic[1] = s.prismatic[1];
  t->prismatic[2] = s.prismatic[2];
  const bool bulk = s.img && bulk_ok(base, s.img, off[8]);
  if (bulk && stage_bulk(base, s.img, (uint32_t)off[8], &stage_bar)) return;
  for (int i = threadIdx.x; i < s.B * 2; i += blockDim.x) t->box[i] = s.box32[i];
  for (int i = threadIdx.x; i < s.R * 3; i += blockDim.x) t->base[i] = s.base32[i];
  for (int i = threadIdx.x; i < s.R * kMaxLinks; i += blockDim.x) t->dh[i] = s.dh32[i];
  for (int i = threadIdx.x; i < s.G * s.SPG; i += blockDim.x) {
    t->sph[i] = s.sph32[i];
    t->band[i] = s.band32[i];
  }
  for (int i = threadIdx.x; i < s.G; i += blockDim.x) {
    t->grp[i] = s.grp[i];
    t->gbs[i] = s.gbs32[i];
  }
  for (int i = threadIdx.x; i < s.NP; i += blockDim.x) t->pairs[i] = s.pairs[i];
  if (bulk) stage_bulk_drain(&stage_bar);
}

__device__ __forceinline__ bool is_prismatic(const ArmSmem& t, int j) {
  return (t.prismatic[j >> 5] >> (j & 31)) & 1u;
}

// Joint angle with the scene's fixed offset: theta = q + offset.  FP32 path:
// the double-float angle (h, l) plus the offset's hi + lo, one error-free sum
// (the result keeps ~44 bits, the reduction then rounds once); FP64 path: one
// IEEE addition, as the CPU restatement does.
__device__ __forceinline__ void add_offset_df(const ArmDev& s, int j, float* h, float* l) {
  if (!s.off32) return;
  const float2 o = s.off32[j];
  float sh, se;
  two_sum(*h, o.x, &sh, &se);
  *h = sh;
  *l = __fadd_rn(__fadd_rn(se, *l), o.y);
}
__device__ __forceinline__ double add_offset64(const ArmDev& s, int j, double th) {
  return s.off64 ? __dadd_rn(th, s.off64[j]) : th;
}

// ---------------------------------------------------------------------------
// FP32 forward kinematics of one group: world frame of (robot r, link k).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void chain32(const ArmDev& s, const ArmSmem& t, const float2* wcs,
                                        const float* wqv, int r, int k, float R[9], float p[3]) {
  const float4 b0 = t.base[r * 3 + 0], b1 = t.base[r * 3 + 1], b2 = t.base[r * 3 + 2];
  int joff = s.q_off[r];
  if (s.base_kind[r] == 1) {
    const float x = wqv[joff], y = wqv[joff + 1];
    const float2 cs = wcs[joff + 2];
    const float c = cs.x, sn = cs.y;
    // Rz(theta) * mount
    R[0] = c * b0.x - sn * b1.x; R[1] = c * b0.y - sn * b1.y; R[2] = c * b0.z - sn * b1.z;
    R[3] = sn * b0.x + c * b1.x; R[4] = sn * b0.y + c * b1.y; R[5] = sn * b0.z + c * b1.z;
    R[6] = b2.x; R[7] = b2.y; R[8] = b2.z;
    p[0] = x + (c * b0.w - sn * b1.w);
    p[1] = y + (sn * b0.w + c * b1.w);
    p[2] = b2.w;
    joff += 3;
  } else {
    R[0] = b0.x; R[1] = b0.y; R[2] = b0.z; p[0] = b0.w;
    R[3] = b1.x; R[4] = b1.y; R[5] = b1.z; p[1] = b1.w;
    R[6] = b2.x; R[7] = b2.y; R[8] = b2.z; p[2] = b2.w;
  }
  for (int j = 0; j < k; j++) {
    const float2 cs = wcs[joff + j];
    const float4 h = t.dh[r * kMaxLinks + j];
    const float c = cs.x, sn = cs.y;
    const float sca = sn * h.z, cca = c * h.z, ssa = sn * h.w, csa = c * h.w;
    const float ac = h.x * c, as = h.x * sn;
#pragma unroll
    for (int i = 0; i < 3; i++) {
      const float r0 = R[3 * i], r1 = R[3 * i + 1], r2 = R[3 * i + 2];
      R[3 * i] = r0 * c + r1 * sn;
      R[3 * i + 1] = r1 * cca - r0 * sca + r2 * h.w;
      R[3 * i + 2] = r0 * ssa - r1 * csa + r2 * h.z;
      p[i] = p[i] + (r0 * ac + r1 * as + r2 * h.y);
    }
  }
}

// ---------------------------------------------------------------------------
// Exact FP64 chain: identical operation order to the CPU restatement.
// ---------------------------------------------------------------------------
__device__ void chain64(const ArmDev& s, const double* wth, const double* wcs, int r, int k,
                        double R[9], double p[3]) {
  const double* bp = s.base64 + r * 12;
  int jo = s.q_off[r];
  if (s.base_kind[r] == 1) {
    const double x = wth[jo], y = wth[jo + 1];
    const double cs = wcs[2 * (jo + 2)], sn = wcs[2 * (jo + 2) + 1];
#pragma unroll
    for (int j = 0; j < 3; j++) {
      R[j] = __dsub_rn(__dmul_rn(cs, bp[j]), __dmul_rn(sn, bp[3 + j]));
      R[3 + j] = __dadd_rn(__dmul_rn(sn, bp[j]), __dmul_rn(cs, bp[3 + j]));
      R[6 + j] = bp[6 + j];
    }
    p[0] = __dadd_rn(x, __dsub_rn(__dmul_rn(cs, bp[9]), __dmul_rn(sn, bp[10])));
    p[1] = __dadd_rn(y, __dadd_rn(__dmul_rn(sn, bp[9]), __dmul_rn(cs, bp[10])));
    p[2] = bp[11];
    jo += 3;
  } else {
#pragma unroll
    for (int i = 0; i < 9; i++) R[i] = bp[i];
    p[0] = bp[9]; p[1] = bp[10]; p[2] = bp[11];
  }
  for (int j = 0; j < k; j++) {
    const double* h = s.dh64 + (r * kMaxLinks + j) * 4;
    const double cs = wcs[2 * (jo + j)], sn = wcs[2 * (jo + j) + 1];
    const double ad = h[0], dd = h[1], ca = h[2], sa = h[3];
    const double sca = __dmul_rn(sn, ca), cca = __dmul_rn(cs, ca);
    const double ssa = __dmul_rn(sn, sa), csa = __dmul_rn(cs, sa);
    const double ac = __dmul_rn(ad, cs), as = __dmul_rn(ad, sn);
#pragma unroll
    for (int i = 0; i < 3; i++) {
      const double r0 = R[3 * i], r1 = R[3 * i + 1], r2 = R[3 * i + 2];
      R[3 * i] = __dadd_rn(__dmul_rn(r0, cs), __dmul_rn(r1, sn));
      R[3 * i + 1] = __dadd_rn(__dsub_rn(__dmul_rn(r1, cca), __dmul_rn(r0, sca)), __dmul_rn(r2, sa));
      R[3 * i + 2] = __dadd_rn(__dsub_rn(__dmul_rn(r0, ssa), __dmul_rn(r1, csa)), __dmul_rn(r2, ca));
      p[i] = __dadd_rn(p[i], __dadd_rn(__dadd_rn(__dmul_rn(r0, ac), __dmul_rn(r1, as)), __dmul_rn(r2, dd)));
    }
  }
}

// exact sphere-box test (numpy order for 3 coordinates)
__device__ __forceinline__ bool exact_box_hit(const double* c, const double* bx, double r2) {
  double sq[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    double v = c[k] > bx[k] ? c[k] : bx[k];
    v = v < bx[3 + k] ? v : bx[3 + k];
    double e = __dsub_rn(v, c[k]);
    sq[k] = __dmul_rn(e, e);
  }
  return __dadd_rn(__dadd_rn(sq[0], sq[1]), sq[2]) <= r2;
}

// exact sphere-sphere test: sqrt(ddot) < ra + rb
__device__ __forceinline__ bool exact_pair_hit(const double* a, const double* b, double ra, double rb) {
  double ss = 0.0;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    double d = __dsub_rn(a[k], b[k]);
    ss = __fma_rn(d, d, ss);
  }
  return sqrt(ss) < __dadd_rn(ra, rb);
}

// every test of the configuration in FP64 (pass 2, when an angle or a planar
// translation is outside the FP32 path's range)
__device__ __forceinline__ bool group_in_mask(const ArmDev& s, int g) {
  return (s.robot_mask >> (s.grp[g] & 0xff)) & 1u;
}

__device__ bool exact_all_collide(const ArmDev& s, const double* wc64, int lane) {
  bool hit = false;
  const int slots = s.G * s.SPG;
  for (int sl = lane; sl < slots && !hit; sl += 32) {
    if (s.sph64[(size_t)sl * 5 + 3] < 0.0 || !group_in_mask(s, sl / s.SPG)) continue;
    for (int b = 0; b < s.B && !hit; b++)
      hit |= exact_box_hit(wc64 + (size_t)sl * 3, s.box64 + (size_t)b * 6, s.sph64[(size_t)sl * 5 + 4]);
  }
  for (int pi = lane; pi < s.NP && !hit; pi += 32) {
    const uint32_t pr = s.pairs[pi];
    const int ga = pr & 0xffff, gb = pr >> 16;
    if (!group_in_mask(s, ga) || !group_in_mask(s, gb)) continue;
    for (int v = 0; v < s.SPG && !hit; v++) {
      const int sa = ga * s.SPG + v;
      if (s.sph64[(size_t)sa * 5 + 3] < 0.0) continue;
      for (int w = 0; w < s.SPG && !hit; w++) {
        const int sb = gb * s.SPG + w;
        if (s.sph64[(size_t)sb * 5 + 3] < 0.0) continue;
        hit |= exact_pair_hit(wc64 + (size_t)sa * 3, wc64 + (size_t)sb * 3, s.sph64[(size_t)sa * 5 + 3],
                              s.sph64[(size_t)sb * 5 + 3]);
      }
    }
  }
  return __any_sync(MRMG_FULL, hit);
}

// ---------------------------------------------------------------------------
// Joint sources.  A source gives joint j of the configuration under test as a
// double-float (pass 1, FP32 arithmetic only) and as the exact FP64 value the
// reference computes (pass 2).  Every lane asks only for its own joints
// j = lane + 32 u; their per-edge data live in that lane's registers.
// ---------------------------------------------------------------------------
constexpr int kJPL = (kMaxArmDof + 31) / 32;

struct CfgSource {          // a stored configuration row
  const void* q;
  int dtype;
  long long row;
  int D;
  __device__ void df(int j, float* h, float* l) const {
    if (dtype == MRMG_F32) {
      *h = ((const float*)q)[row * D + j];
      *l = 0.f;
    } else {
      const double x = ((const double*)q)[row * D + j];
      *h = (float)x;
      *l = (float)__dsub_rn(x, (double)*h);
    }
  }
  __device__ double f64(int j) const { return ldq(q, dtype, row * D + j); }
};

struct EdgeSourceDF {       // pass 1: q1 + (q2 - q1) * i / (N - 1) in double-float
  float ah[kJPL], al[kJPL], dh[kJPL], dl[kJPL];
  float fi, nm1, rn;
  __device__ void df(int j, float* h, float* l) const {
    const int u = j >> 5;
    float a0 = 0.f, a1 = 0.f, d0 = 0.f, d1 = 0.f;
#pragma unroll
    for (int w = 0; w < kJPL; w++)
      if (w == u) { a0 = ah[w]; a1 = al[w]; d0 = dh[w]; d1 = dl[w]; }
    interp_df(a0, a1, d0, d1, fi, nm1, rn, h, l);
  }
  __device__ double f64(int) const { return 0.0; }
};

struct EdgeSource64 {       // pass 2: q1 + dir * i exactly as the reference (FP64)
  double a1[kJPL], dir[kJPL];
  double di;
  __device__ double f64(int j) const {
    const int u = j >> 5;
    double a = 0.0, d = 0.0;
#pragma unroll
    for (int w = 0; w < kJPL; w++)
      if (w == u) { a = a1[w]; d = dir[w]; }
    return __dadd_rn(a, __dmul_rn(d, di));
  }
  __device__ void df(int j, float* h, float* l) const {
    const double x = f64(j);
    *h = (float)x;
    *l = (float)__dsub_rn(x, (double)*h);
  }
};

// the warp's pair-filter norms s = |c|^2 - 2 r'^2, group bounds (world centre,
// radius) and near group-pair list, stored right after its sphere table
__device__ __forceinline__ float* wss_of(const ArmDev& s, float4* wsph) {
  return (float*)((unsigned char*)wsph + align16(sizeof(float4) * s.G * s.SPG));
}
__device__ __forceinline__ float4* wgb_of(const ArmDev& s, float4* wsph) {
  return (float4*)((unsigned char*)wss_of(s, wsph) + align16(sizeof(float) * s.G * s.SPG));
}
__device__ __forceinline__ uint32_t* wnear_of(const ArmDev& s, float4* wsph) {
  return (uint32_t*)((unsigned char*)wgb_of(s, wsph) + align16(sizeof(float4) * s.G));
}

// ---------------------------------------------------------------------------
// Warp evaluation of one configuration.
// Returns V_COLLIDE, V_FREE, or (pass 1 only) V_PENDING; warp-uniform.
// ---------------------------------------------------------------------------
// BOXES selects the box phase: BOX_EACH tests box by box with an early exit
// at the first colliding box (stored configurations); BOX_BLOCKS compacts
// the near (group, box) items of blocks of boxes (positions of surviving
// edges, mostly free: every box is scanned); BOX_HEAD_BLOCKS tests the
// first s.box_head boxes (the tuned order puts the likeliest hits first) box
// by box and the rest in blocks (first positions of edges: most collide early,
// the survivors scan everything).
enum : int { BOX_EACH = 0, BOX_BLOCKS = 1, BOX_HEAD_BLOCKS = 2 };

template <int GPL, int SPG, bool RESOLVE, int BOXES = BOX_EACH, class Src>
__device__ uint8_t eval_config(const ArmDev& s, const ArmSmem& t, float2* wcs, float* wqv,
                               float4* wsph, double* w64, int lane, const Src& src, bool full,
                               bool accum = false) {
  __syncwarp();
  bool hit_any = false;   // full evaluation: remember a collision instead of stopping
  // --- joint preprocessing: FP32 cos/sin of angles reduced to [-pi, pi]
  bool ok = true;
  for (int j = lane; j < s.D; j += 32) {
    float h, l;
    src.df(j, &h, &l);
    if (is_prismatic(t, j)) {
      wqv[j] = __fadd_rn(h, l);
      ok &= fabsf(h) <= s.xy_max;
      wcs[j] = make_float2(1.f, 0.f);
    } else {
      float a;
      add_offset_df(s, j, &h, &l);
      ok &= reduce_df(h, l, &a);
      float sn, cs;
      sincosf(a, &sn, &cs);
      wcs[j] = make_float2(cs, sn);
      wqv[j] = a;
    }
  }
  // --- exact FP64 chain for pass 2 (joint values, cos/sin, centres)
  double* wth64 = w64;
  double* wcs64 = w64 + ((s.D + 1) & ~1);
  double* wc64 = wcs64 + 2 * s.D;
  if constexpr (RESOLVE) {
    for (int j = lane; j < s.D; j += 32) {
      const double th = src.f64(j);
      wth64[j] = th;
      double sn, cs;
      sincos_exact(add_offset64(s, j, th), &sn, &cs);
      wcs64[2 * j] = cs;
      wcs64[2 * j + 1] = sn;
    }
  }
  const bool all_ok = __all_sync(MRMG_FULL, ok);
  if (!RESOLVE && !all_ok) return V_PENDING;
  __syncwarp();
  if constexpr (RESOLVE) {
#pragma unroll
    for (int u = 0; u < GPL; u++) {
      const int g = lane + 32 * u;
      if (g < s.G) {
        const int gi = t.grp[g];
        double R[9], p[3];
        chain64(s, wth64, wcs64, gi & 0xff, gi >> 8, R, p);
        for (int v = 0; v < SPG; v++) {
          const double* l = s.sph64 + (size_t)(g * SPG + v) * 5;
          double* c = wc64 + (size_t)(g * SPG + v) * 3;
#pragma unroll
          for (int i = 0; i < 3; i++)
            c[i] = __dadd_rn(p[i], __dadd_rn(__dadd_rn(__dmul_rn(R[3 * i], l[0]), __dmul_rn(R[3 * i + 1], l[1])),
                                             __dmul_rn(R[3 * i + 2], l[2])));
        }
      }
    }
    __syncwarp();
    if (!all_ok) return exact_all_collide(s, wc64, lane) ? V_COLLIDE : V_FREE;
  }

  // --- FP32 chain + sphere centres (and group bound centres) of the owned groups
  float cx[GPL][SPG], cy[GPL][SPG], cz[GPL][SPG], rh[GPL][SPG];   // per-box phase only
  float gb[GPL][4];
#pragma unroll
  for (int u = 0; u < GPL; u++) {
    const int g = lane + 32 * u;
    if (g < s.G) {
      const int gi = t.grp[g];
      float R[9], p[3];
      chain32(s, t, wcs, wqv, gi & 0xff, gi >> 8, R, p);
      const float4 lb = t.gbs[g];
      gb[u][0] = p[0] + (R[0] * lb.x + R[1] * lb.y + R[2] * lb.z);
      gb[u][1] = p[1] + (R[3] * lb.x + R[4] * lb.y + R[5] * lb.z);
      gb[u][2] = p[2] + (R[6] * lb.x + R[7] * lb.y + R[8] * lb.z);
      // a robot outside the call's mask: its bound never reaches a box or
      // another group, so none of its spheres is tested
      gb[u][3] = ((s.robot_mask >> (gi & 0xff)) & 1u) ? lb.w : -1.f;
#pragma unroll
      for (int v = 0; v < SPG; v++) {
        const float4 l = t.sph[g * SPG + v];
        const float4 bd = t.band[g * SPG + v];
        float x = p[0] + (R[0] * l.x + R[1] * l.y + R[2] * l.z);
        float y = p[1] + (R[3] * l.x + R[4] * l.y + R[5] * l.z);
        float z = p[2] + (R[6] * l.x + R[7] * l.y + R[8] * l.z);
        if (bd.y < 0.f) { x = kFar * (float)(g + 1); y = x; z = 0.f; }   // padding slot
        if constexpr (BOXES != BOX_BLOCKS) { cx[u][v] = x; cy[u][v] = y; cz[u][v] = z; rh[u][v] = bd.y; }
        wsph[g * SPG + v] = make_float4(x, y, z, bd.z);
      }
    } else {
      if constexpr (BOXES != BOX_BLOCKS) {
#pragma unroll
        for (int v = 0; v < SPG; v++) {
          cx[u][v] = kFar * (float)(200 + lane); cy[u][v] = cx[u][v]; cz[u][v] = 0.f; rh[u][v] = -1.f;
        }
      }
      gb[u][0] = kFar * (float)(200 + lane); gb[u][1] = gb[u][0]; gb[u][2] = 0.f; gb[u][3] = -1.f;
    }
  }
  __syncwarp();

  bool unc = false;
  const int b_each = BOXES == BOX_EACH ? s.B : (BOXES == BOX_HEAD_BLOCKS ? min(s.B, s.box_head) : 0);
  {
    // --- spheres against boxes, box by box: all of them, or the head
    for (int b = 0; b < b_each; b++) {
      const float4 bc = t.box[2 * b], bh = t.box[2 * b + 1];
      float umin = 3.0e38f;
#pragma unroll
      for (int u = 0; u < GPL; u++) {
        // the group's bound first: its spheres are tested only if it reaches the box
        const float gx = fmaxf(fabsf(gb[u][0] - bc.x) - bh.x, 0.f);
        const float gy = fmaxf(fabsf(gb[u][1] - bc.y) - bh.y, 0.f);
        const float gz = fmaxf(fabsf(gb[u][2] - bc.z) - bh.z, 0.f);
        if (fmaf(gz, gz, fmaf(gy, gy, fmaf(gx, gx, -gb[u][3]))) <= 0.f) {
#pragma unroll
          for (int v = 0; v < SPG; v++) {
            const float ex = fmaxf(fabsf(cx[u][v] - bc.x) - bh.x, 0.f);
            const float ey = fmaxf(fabsf(cy[u][v] - bc.y) - bh.y, 0.f);
            const float ez = fmaxf(fabsf(cz[u][v] - bc.z) - bh.z, 0.f);
            umin = fminf(umin, fmaf(ez, ez, fmaf(ey, ey, fmaf(ex, ex, -rh[u][v]))));
          }
        }
      }
      if (__any_sync(MRMG_FULL, umin <= 0.f)) {
        bool coll = false;
        if (umin <= 0.f) {
#pragma unroll
          for (int u = 0; u < GPL; u++)
#pragma unroll
            for (int v = 0; v < SPG; v++) {
              const int g = lane + 32 * u;
              const float ex = fmaxf(fabsf(cx[u][v] - bc.x) - bh.x, 0.f);
              const float ey = fmaxf(fabsf(cy[u][v] - bc.y) - bh.y, 0.f);
              const float ez = fmaxf(fabsf(cz[u][v] - bc.z) - bh.z, 0.f);
              const float ss = fmaf(ez, ez, fmaf(ey, ey, ex * ex));
              if (ss <= rh[u][v]) {
                const float4 bd = t.band[g * SPG + v];
                if (ss < bd.x) coll = true;
                else if (RESOLVE) {
                  const int slot = g * SPG + v;
                  coll |= exact_box_hit(wc64 + (size_t)slot * 3, s.box64 + (size_t)b * 6, s.sph64[(size_t)slot * 5 + 4]);
                } else {
                  unc = true;
                }
              }
            }
        }
        if (__any_sync(MRMG_FULL, coll)) {
          if (!full) return V_COLLIDE;
          hit_any = true;
        }
      }
    }
  }

  // --- spheres against boxes in blocks.  Per block, every lane tests its
  // groups' bounds against each box and the (group, box) pairs whose bound
  // reaches the box are compacted into the warp's list; then each lane takes
  // one listed pair and tests the group's spheres (centres from the warp's
  // sphere table), so the sphere tests run with the lanes full.  A collision
  // ends the configuration after its block (early exit).
  if constexpr (BOXES != BOX_EACH) {
    uint32_t* witem = wnear_of(s, wsph);
    const unsigned ltb = (1u << lane) - 1u;
    // BOX_BLOCKS: blocks of 1, 1, 2, 4, ... up to s.box_block boxes from the
    // first box; BOX_HEAD_BLOCKS: blocks of s.box_block after the per-box head
    const int bmax = s.box_block;
    int bs = BOXES == BOX_BLOCKS ? 1 : bmax;
    // phase B with `accum` (full evaluation: every box is scanned anyway)
    // lists the items of consecutive blocks together and tests them when the
    // next block could overflow the list, instead of a mostly empty round of
    // item tests per block
    int nacc = 0;
    for (int b0 = b_each; b0 < s.B; b0 += bs, bs = (BOXES == BOX_BLOCKS && b0 <= 1) ? 1 : min(2 * bs, bmax)) {
      const int b1 = min(s.B, b0 + bs);
      int nit = BOXES == BOX_BLOCKS ? nacc : 0;
      int b = b0;
      if constexpr (BOXES == BOX_BLOCKS) {
        // phase B: two boxes per packed FP32x2 instruction (same values as
        // the scalar test below)
        for (; b + 1 < b1; b += 2) {
          const float4 c0 = t.box[2 * b], h0 = t.box[2 * b + 1], c1 = t.box[2 * b + 2], h1 = t.box[2 * b + 3];
#pragma unroll
          for (int u = 0; u < GPL; u++) {
            const float2 dx = __fadd2_rn(make_float2(gb[u][0], gb[u][0]), make_float2(-c0.x, -c1.x));
            const float2 dy = __fadd2_rn(make_float2(gb[u][1], gb[u][1]), make_float2(-c0.y, -c1.y));
            const float2 dz = __fadd2_rn(make_float2(gb[u][2], gb[u][2]), make_float2(-c0.z, -c1.z));
            const float2 ox = __fadd2_rn(make_float2(fabsf(dx.x), fabsf(dx.y)), make_float2(-h0.x, -h1.x));
            const float2 oy = __fadd2_rn(make_float2(fabsf(dy.x), fabsf(dy.y)), make_float2(-h0.y, -h1.y));
            const float2 oz = __fadd2_rn(make_float2(fabsf(dz.x), fabsf(dz.y)), make_float2(-h0.z, -h1.z));
            const float2 gx = make_float2(fmaxf(ox.x, 0.f), fmaxf(ox.y, 0.f));
            const float2 gy = make_float2(fmaxf(oy.x, 0.f), fmaxf(oy.y, 0.f));
            const float2 gz = make_float2(fmaxf(oz.x, 0.f), fmaxf(oz.y, 0.f));
            const float nr2 = -gb[u][3];
            const float2 q2 = __ffma2_rn(gz, gz, __ffma2_rn(gy, gy, __ffma2_rn(gx, gx, make_float2(nr2, nr2))));
            const bool n0 = q2.x <= 0.f, n1 = q2.y <= 0.f;
            const unsigned m0 = __ballot_sync(MRMG_FULL, n0);
            if (n0) witem[nit + __popc(m0 & ltb)] = (uint32_t)(lane + 32 * u) | ((uint32_t)b << 16);
            nit += __popc(m0);
            const unsigned m1 = __ballot_sync(MRMG_FULL, n1);
            if (n1) witem[nit + __popc(m1 & ltb)] = (uint32_t)(lane + 32 * u) | ((uint32_t)(b + 1) << 16);
            nit += __popc(m1);
          }
        }
      }
      for (; b < b1; b++) {
        const float4 bc = t.box[2 * b], bh = t.box[2 * b + 1];
#pragma unroll
        for (int u = 0; u < GPL; u++) {
          const float gx = fmaxf(fabsf(gb[u][0] - bc.x) - bh.x, 0.f);
          const float gy = fmaxf(fabsf(gb[u][1] - bc.y) - bh.y, 0.f);
          const float gz = fmaxf(fabsf(gb[u][2] - bc.z) - bh.z, 0.f);
          const bool nr = fmaf(gz, gz, fmaf(gy, gy, fmaf(gx, gx, -gb[u][3]))) <= 0.f;
          const unsigned m = __ballot_sync(MRMG_FULL, nr);
          if (nr) witem[nit + __popc(m & ltb)] = (uint32_t)(lane + 32 * u) | ((uint32_t)b << 16);
          nit += __popc(m);
        }
      }
      if constexpr (BOXES == BOX_BLOCKS) {
        const int nbs = b0 + bs <= 1 ? 1 : min(2 * bs, bmax);   // the next block's size
        if (accum && b1 < s.B && nit + s.G * nbs <= (int)list_cap(s)) {
          nacc = nit;
          continue;
        }
        nacc = 0;
      }
      __syncwarp();
      for (int base = 0; base < nit; base += 32) {
        bool coll = false;
        if (base + lane < nit) {
          const uint32_t it = witem[base + lane];
          const int g = it & 0xffff, b = it >> 16;
          const float4 bc = t.box[2 * b], bh = t.box[2 * b + 1];
          // phase B: two spheres per packed FP32x2 instruction (each element
          // rounds as the scalar instruction would: the same ss values)
          constexpr int Q2 = BOXES == BOX_BLOCKS ? SPG / 2 : 0;
          float ssp[2 * Q2 > 0 ? 2 * Q2 : 1];
#pragma unroll
          for (int v2 = 0; v2 < Q2; v2++) {
            const float4 c0 = wsph[g * SPG + 2 * v2], c1 = wsph[g * SPG + 2 * v2 + 1];
            const float2 dx = __fadd2_rn(make_float2(c0.x, c1.x), make_float2(-bc.x, -bc.x));
            const float2 dy = __fadd2_rn(make_float2(c0.y, c1.y), make_float2(-bc.y, -bc.y));
            const float2 dz = __fadd2_rn(make_float2(c0.z, c1.z), make_float2(-bc.z, -bc.z));
            const float2 ox = __fadd2_rn(make_float2(fabsf(dx.x), fabsf(dx.y)), make_float2(-bh.x, -bh.x));
            const float2 oy = __fadd2_rn(make_float2(fabsf(dy.x), fabsf(dy.y)), make_float2(-bh.y, -bh.y));
            const float2 oz = __fadd2_rn(make_float2(fabsf(dz.x), fabsf(dz.y)), make_float2(-bh.z, -bh.z));
            const float2 ex = make_float2(fmaxf(ox.x, 0.f), fmaxf(ox.y, 0.f));
            const float2 ey = make_float2(fmaxf(oy.x, 0.f), fmaxf(oy.y, 0.f));
            const float2 ez = make_float2(fmaxf(oz.x, 0.f), fmaxf(oz.y, 0.f));
            const float2 s2 = __ffma2_rn(ez, ez, __ffma2_rn(ey, ey, __fmul2_rn(ex, ex)));
            ssp[2 * v2] = s2.x;
            ssp[2 * v2 + 1] = s2.y;
          }
#pragma unroll
          for (int v = 0; v < SPG; v++) {
            const float4 c = wsph[g * SPG + v];
            const float4 bd = t.band[g * SPG + v];
            float ss;
            if (v < 2 * Q2) {
              ss = ssp[v];
            } else {
              const float ex = fmaxf(fabsf(c.x - bc.x) - bh.x, 0.f);
              const float ey = fmaxf(fabsf(c.y - bc.y) - bh.y, 0.f);
              const float ez = fmaxf(fabsf(c.z - bc.z) - bh.z, 0.f);
              ss = fmaf(ez, ez, fmaf(ey, ey, ex * ex));
            }
            if (ss <= bd.y) {
              if (ss < bd.x) coll = true;
              else if (RESOLVE) {
                const int slot = g * SPG + v;
                coll |= exact_box_hit(wc64 + (size_t)slot * 3, s.box64 + (size_t)b * 6, s.sph64[(size_t)slot * 5 + 4]);
              } else {
                unc = true;
              }
            }
          }
        }
        if (__any_sync(MRMG_FULL, coll)) {
          if (!full) return V_COLLIDE;
          hit_any = true;
        }
      }
      __syncwarp();   // the next block rewrites the list
    }
  }

  // --- spheres of different robots.  Filter: since (r_a + r_b)^2 <= 2 r_a^2 +
  // 2 r_b^2 (equal for equal radii), |a - b|^2 - (r_a + r_b)^2 >= s_a + s_b - 2 a.b
  // with s = |c|^2 - 2 r^2 per sphere (r = radius + delta): three products
  // per pair.  Pairs with a filter value within its FP32 error bound go to the
  // direct test below, which decides exactly as before.
  // Group pairs whose bounds are apart (|g_a - g_b| > R_a + R_b; each R holds
  // 4 delta, 2 delta more than the band needs) cannot hold a flagged sphere
  // pair: they are dropped first and the rest are compacted, so the sphere
  // pairs run in dense rounds.
  const float d4 = 4.f * s.delta;
  float* wss = wss_of(s, wsph);
  float4* wgb = wgb_of(s, wsph);
  uint32_t* wnear = wnear_of(s, wsph);
#pragma unroll
  for (int u = 0; u < GPL; u++) {
    const int g = lane + 32 * u;
    if (g < s.G) {
#pragma unroll
      for (int v = 0; v < SPG; v++) {
        const float4 c = wsph[g * SPG + v];
        wss[g * SPG + v] = fmaf(c.x, c.x, fmaf(c.y, c.y, fmaf(c.z, c.z, -2.f * c.w * c.w)));
      }
      wgb[g] = make_float4(gb[u][0], gb[u][1], gb[u][2], gb[u][3] >= 0.f ? sqrtf(gb[u][3]) : -1.0e30f);
    }
  }
  __syncwarp();
  const unsigned lt = (1u << lane) - 1u;
  const int nblk = near_block(s);
  for (int blk = 0; blk < s.NP; blk += nblk) {
  const int blk_end = min(s.NP, blk + nblk);
  int nnear = 0;
  for (int base = blk; base < blk_end; base += 32) {
    const int pi = base + lane;
    bool near = false;
    uint32_t pr = 0;
    if (pi < blk_end) {
      pr = t.pairs[pi];
      const float4 ga = wgb[pr & 0xffff], gq = wgb[pr >> 16];
      const float dx = ga.x - gq.x, dy = ga.y - gq.y, dz = ga.z - gq.z;
      const float rr = ga.w + gq.w;
      near = rr > 0.f && fmaf(dz, dz, fmaf(dy, dy, dx * dx)) <= rr * rr;
    }
    const unsigned m = __ballot_sync(MRMG_FULL, near);
    if (near) wnear[nnear + __popc(m & lt)] = pr;
    nnear += __popc(m);
  }
  __syncwarp();
  for (int base = 0; base < nnear; base += 32) {
    const int pi = base + lane;
    float umin = 3.0e38f;
    uint32_t pr = 0;
    if (pi < nnear) {
      pr = wnear[pi];
      const int sa0 = (pr & 0xffff) * SPG, sb0 = (pr >> 16) * SPG;
      // phase B: group a's spheres two at a time in packed FP32x2 registers
      // (each packed FMA / add rounds its two elements exactly as the scalar
      // instruction would, so the filter values are the scalar ones); the
      // first positions keep scalar code, which fits their register budget
      constexpr int P2 = BOXES == BOX_BLOCKS ? SPG / 2 : 0;
      float2 ax[P2 > 0 ? P2 : 1], ay[P2 > 0 ? P2 : 1], az[P2 > 0 ? P2 : 1], aw[P2 > 0 ? P2 : 1];
#pragma unroll
      for (int v = 0; v < P2; v++) {
        const float4 c0 = wsph[sa0 + 2 * v], c1 = wsph[sa0 + 2 * v + 1];
        ax[v] = make_float2(-2.f * c0.x, -2.f * c1.x);
        ay[v] = make_float2(-2.f * c0.y, -2.f * c1.y);
        az[v] = make_float2(-2.f * c0.z, -2.f * c1.z);
        aw[v] = make_float2(wss[sa0 + 2 * v], wss[sa0 + 2 * v + 1]);
      }
      float4 a[SPG - 2 * P2 > 0 ? SPG - 2 * P2 : 1];   // the spheres not packed: (-2 x, -2 y, -2 z, s)
#pragma unroll
      for (int v = 2 * P2; v < SPG; v++) {
        const float4 c = wsph[sa0 + v];
        a[v - 2 * P2] = make_float4(-2.f * c.x, -2.f * c.y, -2.f * c.z, wss[sa0 + v]);
      }
#pragma unroll
      for (int w = 0; w < SPG; w++) {
        const float4 bq = wsph[sb0 + w];
        const float sb = wss[sb0 + w];
        const float2 bx = make_float2(bq.x, bq.x), by = make_float2(bq.y, bq.y), bz = make_float2(bq.z, bq.z);
        const float2 sb2 = make_float2(sb, sb);
#pragma unroll
        for (int v = 0; v < P2; v++) {
          const float2 f = __ffma2_rn(ax[v], bx, __ffma2_rn(ay[v], by, __ffma2_rn(az[v], bz, __fadd2_rn(aw[v], sb2))));
          umin = fminf(umin, fminf(f.x, f.y));
        }
#pragma unroll
        for (int v = 0; v < SPG - 2 * P2; v++)
          umin = fminf(umin, fmaf(a[v].x, bq.x, fmaf(a[v].y, bq.y, fmaf(a[v].z, bq.z, a[v].w + sb))));
      }
    }
    if (__any_sync(MRMG_FULL, umin <= s.pair_eps)) {
      bool coll = false;
      if (umin <= 0.f) {
        const int ga = pr & 0xffff, gb = pr >> 16;
        for (int w = 0; w < SPG; w++) {
          const float4 bq = wsph[gb * SPG + w];
          for (int v = 0; v < SPG; v++) {
            const float4 aq = wsph[ga * SPG + v];
            const float dx = aq.x - bq.x, dy = aq.y - bq.y, dz = aq.z - bq.z;
            const float W = aq.w + bq.w;
            const float ss = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
            if (ss <= W * W) {
              const float Wl = W - d4;
              if (Wl > 0.f && ss < Wl * Wl) coll = true;
              else if (RESOLVE) {
                const int sa = ga * SPG + v, sb = gb * SPG + w;
                coll |= exact_pair_hit(wc64 + (size_t)sa * 3, wc64 + (size_t)sb * 3,
                                       s.sph64[(size_t)sa * 5 + 3], s.sph64[(size_t)sb * 5 + 3]);
              } else {
                unc = true;
              }
            }
          }
        }
      }
      if (__any_sync(MRMG_FULL, coll)) {
        if (!full) return V_COLLIDE;
        hit_any = true;
      }
    }
  }
  __syncwarp();   // the next block rewrites the near list
  }
  if (hit_any) return V_COLLIDE;
  if (RESOLVE) return V_FREE;
  return __any_sync(MRMG_FULL, unc) ? V_PENDING : V_FREE;
}

__device__ __forceinline__ void warp_areas(const ArmDev& s, unsigned char* smem_base, size_t tbytes,
                                           int wib, bool with64, float2** wcs, float** wqv,
                                           float4** wsph, double** w64) {
  size_t per = warp32_bytes(s) + (with64 ? warp64_bytes(s) : 0);
  unsigned char* p = smem_base + tbytes + per * wib;
  *wcs = (float2*)p; p += align16(sizeof(float2) * s.D);
  *wqv = (float*)p; p += align16(sizeof(float) * s.D);
  *wsph = (float4*)p; p += align16(sizeof(float4) * s.G * s.SPG);
  // pair-filter norms, group bounds, near group pairs (after wsph, see wss_of)
  p += align16(sizeof(float) * s.G * s.SPG) + align16(sizeof(float4) * s.G) + align16(sizeof(uint32_t) * list_cap(s));
  *w64 = (double*)p;
}

// ---------------------------------------------------------------------------
// Configurations (warp per configuration, configurations taken from a work
// queue in chunks of s.cfg_chunk).
// ---------------------------------------------------------------------------

template <int GPL, int SPG, bool RESOLVE>
__global__ void __launch_bounds__(256, RESOLVE ? 1 : (GPL == 1 ? 4 : (GPL == 2 ? 2 : 1))) arm_configs_kernel(ArmDev s, const void* q, int dtype, long long n,
                                                          uint8_t* out, int* ctr, long long* pend, int full) {
  if (RESOLVE && ctr[kCtrPending] == 0) return;   // nothing was left undecided
  extern __shared__ __align__(16) unsigned char smem_arm[];
  ArmSmem t;
  stage_tables(s, smem_arm, &t);
  __syncthreads();
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  float2* wcs; float* wqv; float4* wsph; double* w64;
  warp_areas(s, smem_arm, table_bytes(s), wib, RESOLVE, &wcs, &wqv, &wsph, &w64);
  const int D = s.D;
  while (true) {
    long long k0 = 0;
    if (lane == 0) k0 = atomicAdd(&ctr[RESOLVE ? kCtrQueue2 : kCtrQueue], RESOLVE ? 1 : s.cfg_chunk);
    k0 = __shfl_sync(MRMG_FULL, k0, 0);
    const long long lim = RESOLVE ? (long long)ctr[kCtrPending] : n;
    if (k0 >= lim) break;
    const int cnt = RESOLVE ? 1 : (int)min((long long)s.cfg_chunk, lim - k0);
    for (int c = 0; c < cnt; c++) {
      const long long i = RESOLVE ? pend[k0] : k0 + c;
      const CfgSource src{q, dtype, i, D};
      uint8_t v = eval_config<GPL, SPG, RESOLVE>(s, t, wcs, wqv, wsph, w64, lane, src, full != 0);
      if (lane == 0) {
        out[i] = v;
        if (!RESOLVE && v == V_PENDING) {
          int slot = atomicAdd(&ctr[kCtrPending], 1);
          pend[slot] = i;
        }
      }
      __syncwarp();
    }
  }
}

// ---------------------------------------------------------------------------
// Edges.
//   phase A  warp per edge (work queue): N, then the first BFS position of
//            generate_binary_search_indices(N) that is checked; most edges of a
//            cluttered scene stop here.  Survivors are appended to a list with
//            their remaining position range.
//   phase B  the survivors' remaining positions, position-major (all
//            survivors' next position, then the one after, ...), dealt to every
//            warp in blocks of 32; a collision marks the edge dead and its
//            remaining positions are skipped.  Long free edges no longer run on
//            one warp.
//   finalize survivors' verdicts (last CTA of the last phase-B launch);
//            undecided ones join the FP64 pending list.
//   pass 2   (RESOLVE) warp per pending edge, the reference's order, exact.
// ---------------------------------------------------------------------------

// this lane's joints of edge e as double-floats: a = q1, d = q2 - q1
__device__ __forceinline__ void load_edge(const void* q1, const void* q2, int dtype, long long e, int D, int lane,
                                          EdgeSourceDF* sdf, float* mloc, bool* nanf) {
  *mloc = 0.f;
  *nanf = false;
#pragma unroll
  for (int u = 0; u < kJPL; u++) {
    const int j = lane + 32 * u;
    sdf->ah[u] = 0.f; sdf->al[u] = 0.f; sdf->dh[u] = 0.f; sdf->dl[u] = 0.f;
    if (j < D) {
      if (dtype == MRMG_F32) {
        const float a = ((const float*)q1)[e * D + j], b = ((const float*)q2)[e * D + j];
        sdf->ah[u] = a;
        two_sum(b, -a, &sdf->dh[u], &sdf->dl[u]);           // q2 - q1 exactly
      } else {
        const double a = ((const double*)q1)[e * D + j], b = ((const double*)q2)[e * D + j];
        const double d = __dsub_rn(b, a);
        sdf->ah[u] = (float)a;
        sdf->al[u] = (float)__dsub_rn(a, (double)sdf->ah[u]);
        sdf->dh[u] = (float)d;
        sdf->dl[u] = (float)__dsub_rn(d, (double)sdf->dh[u]);
      }
      *nanf |= sdf->dh[u] != sdf->dh[u];
      *mloc = fmaxf(*mloc, fabsf(sdf->dh[u]));
    }
  }
}

// N of edge e: given, or max(2, int(max|q1 - q2| / res) + 1) -- FP32 with an
// integer-distance certificate, else FP64 (abstract_env.py:321-323).
// Returns false on a non-finite edge length (int() of nan/inf raises).
__device__ __forceinline__ bool edge_N(const void* q1, const void* q2, int dtype, long long e, int D, int lane,
                                       double res, float res32, const long long* Np, float mloc, bool nanf,
                                       bool allow_fast, long long* N_out) {
  if (Np) {
    *N_out = Np[e];
    return *N_out >= 0;
  }
  if (allow_fast) {
    const float m32 = warp_max(mloc);
    const bool anynan = __any_sync(MRMG_FULL, nanf);
    if (steps_fp32(m32, anynan, res32, N_out)) return true;
  }
  double mx = -1.0;
  bool nan0 = false;
#pragma unroll
  for (int u = 0; u < kJPL; u++) {
    const int j = lane + 32 * u;
    if (j < D) {
      const double v = fabs(__dsub_rn(ldq(q1, dtype, e * D + j), ldq(q2, dtype, e * D + j)));
      if (j == 0) nan0 = (v != v);
      mx = fmax(mx, v);
    }
  }
  const double m = warp_max_d(mx);
  nan0 = __any_sync(MRMG_FULL, nan0);
  const double tq = __ddiv_rn(m, res);
  if (nan0 || !(tq < 9.0e15)) return false;
  *N_out = max(2ll, (long long)tq + 1);
  return true;
}

template <int GPL, int SPG, bool RESOLVE>
__global__ void __launch_bounds__(256, RESOLVE ? 1 : (GPL == 1 ? 4 : (GPL == 2 ? 2 : 1))) arm_edges_kernel(ArmDev s, const void* q1, const void* q2, int dtype,
                                                        long long n, double res, int incl,
                                                        const long long* Np, long long N_start,
                                                        long long N_max, uint8_t* out, int* ctr,
                                                        long long* pend, SurvivorEdge* surv, int full) {
  if (RESOLVE && ctr[kCtrPending] == 0) return;   // nothing was left undecided
  extern __shared__ __align__(16) unsigned char smem_arm[];
  ArmSmem t;
  stage_tables(s, smem_arm, &t);
  __syncthreads();
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  float2* wcs; float* wqv; float4* wsph; double* w64;
  warp_areas(s, smem_arm, table_bytes(s), wib, RESOLVE, &wcs, &wqv, &wsph, &w64);
  const int D = s.D;
  const float res32 = (float)res;
  const unsigned lt_mask = (1u << lane) - 1u;
  long long stat_cfg = 0;

  // edges (phase A) or pending edges (pass 2) through a work queue: the cost
  // per edge is uneven (a free first configuration is a full evaluation)
  while (true) {
    long long k = 0;
    if (lane == 0) k = atomicAdd(&ctr[RESOLVE ? kCtrQueue2 : kCtrQueue], 1);
    k = __shfl_sync(MRMG_FULL, k, 0);
    long long e;
    if (RESOLVE) {
      if (k >= ctr[kCtrPending]) break;
      e = pend[k];
    } else {
      if (k >= n) break;
      e = k;
    }
    EdgeSourceDF sdf;
    float mloc;
    bool nanf;
    load_edge(q1, q2, dtype, e, D, lane, &sdf, &mloc, &nanf);
    long long N = 0;
    const bool good = edge_N(q1, q2, dtype, e, D, lane, res, res32, Np, mloc, nanf, !RESOLVE, &N);
    if (!good || N_start > N) {
      if (lane == 0) { atomicOr(&ctr[kCtrErr], !good ? E_BAD_INPUT : E_N_START); out[e] = 0; }
      __syncwarp();
      continue;
    }
    const long long nmax = (N_max < 0 || N_max > N) ? N : N_max;

    if constexpr (!RESOLVE) {
      // ---- phase A: the first checked position
      uint8_t r = V_FREE;
      if (N > (1ll << 24)) {
        r = V_PENDING;                      // indices beyond exact FP32 integers: exact pass
      } else {
        long long p = N_start, iv = -1;
        for (; p < nmax; p++) {
          const long long c = bfs_at(N, p);
          if (incl || (c != 0 && c != N - 1)) { iv = c; break; }
        }
        if (iv >= 0) {
          // N <= 2^24 here: int32 -> FP32 conversions (the 64-bit ones issue
          // on the FP64 pipe, which is narrow on this part)
          sdf.nm1 = (float)(int)(N - 1);
          sdf.rn = __frcp_rn(sdf.nm1);
          sdf.fi = (float)(int)iv;
          stat_cfg++;
          const uint8_t code = eval_config<GPL, SPG, false, BOX_HEAD_BLOCKS>(s, t, wcs, wqv, wsph, w64, lane, sdf,
                                                                          full != 0);
          if (code == V_COLLIDE && !full) {
            r = V_COLLIDE;
          } else if (p + 1 < nmax) {
            if (lane == 0) {
              const int slot = atomicAdd(&ctr[kCtrL1], 1);
              SurvivorEdge sv;
              sv.e = e; sv.N = (int)N; sv.p_next = (int)(p + 1); sv.nmax = (int)nmax;
              sv.dead = code == V_COLLIDE; sv.pend = code == V_PENDING; sv.pad = 0;
              surv[slot] = sv;
              atomicMax(&ctr[kCtrMaxJ], (int)(nmax - p - 1));
            }
            __syncwarp();
            continue;                       // phase B decides (its last launch finalizes)
          } else {
            r = code;
          }
        }
      }
      if (lane == 0) {
        out[e] = r;
        if (r == V_PENDING) {
          const int slot = atomicAdd(&ctr[kCtrPending], 1);
          pend[slot] = e;
        }
      }
      __syncwarp();
    } else {
      // ---- pass 2: the reference's order, one configuration at a time, FP64 where pending
      EdgeSource64 s64;
      const double denom = (double)(N - 1);
#pragma unroll
      for (int u = 0; u < kJPL; u++) {
        const int j = lane + 32 * u;
        s64.a1[u] = 0.0; s64.dir[u] = 0.0;
        if (j < D) {
          const double a = ldq(q1, dtype, e * D + j), b = ldq(q2, dtype, e * D + j);
          s64.a1[u] = a;
          s64.dir[u] = __ddiv_rn(__dsub_rn(b, a), denom);   // (q2 - q1) / (N - 1)
        }
      }
      BfsChunker ch;
      ch.init(N);
      long long v;
      unsigned m;
      long long pos0;
      bool coll = false;
      while (!coll && ch.next(lane, &v, &m, &pos0)) {
        if (pos0 >= nmax) break;
        const long long my_pos = pos0 + __popc(m & lt_mask);
        const bool active = v >= 0 && my_pos >= N_start && my_pos < nmax && (incl || (v != 0 && v != N - 1));
        unsigned act = __ballot_sync(MRMG_FULL, active);
        while (act) {
          const int srcl = __ffs(act) - 1;
          act &= act - 1;
          s64.di = (double)__shfl_sync(MRMG_FULL, v, srcl);
          if (eval_config<GPL, SPG, true>(s, t, wcs, wqv, wsph, w64, lane, s64, false) == V_COLLIDE) {
            coll = true;
            break;
          }
        }
      }
      if (lane == 0) out[e] = coll ? V_COLLIDE : V_FREE;
      __syncwarp();
    }
  }
  if (lane == 0 && !RESOLVE) atomicAdd((unsigned long long*)&ctr[kCtrStat0], (unsigned long long)stat_cfg);
}

// survivors' verdicts; undecided ones join the FP64 pending list.  Run by
// one CTA (thread stride) after every phase-B configuration has finished.
__device__ void finalize_survivors(int* ctr, const SurvivorEdge* surv, uint8_t* out, long long* pend) {
  const int nsv = *(volatile int*)&ctr[kCtrL1];
  const volatile SurvivorEdge* vs = surv;
  for (int l = threadIdx.x; l < nsv; l += blockDim.x) {
    const long long e = vs[l].e;
    const uint8_t r = vs[l].dead ? V_COLLIDE : (vs[l].pend ? V_PENDING : V_FREE);
    out[e] = r;
    if (r == V_PENDING) {
      const int slot = atomicAdd(&ctr[kCtrPending], 1);
      pend[slot] = e;
    }
  }
}

// positions p_next + j, j in [j_lo, j_hi), of every survivor (j_hi < 0: to the end)
template <int GPL, int SPG>
__global__ void __launch_bounds__(256, GPL == 1 ? 3 : (GPL == 2 ? 2 : 1)) arm_edges_phase_b(ArmDev s, const void* q1, const void* q2, int dtype,
                                                         int incl, int* ctr, SurvivorEdge* surv, int full,
                                                         int j_lo, int j_hi, uint8_t* out, long long* pend) {
  // the last launch (j_hi < 0) also finalizes: its last CTA to finish sets the
  // survivors' verdicts (or CTA 0, when the launch has no positions left)
  const bool fin = j_hi < 0;
  const int nsv = ctr[kCtrL1];
  const long long maxj = j_hi < 0 ? (long long)ctr[kCtrMaxJ] : min((long long)j_hi, (long long)ctr[kCtrMaxJ]);
  const long long first = (long long)nsv * j_lo;
  const long long total = (long long)nsv * maxj;
  if (total <= first) {
    if (fin && blockIdx.x == 0) finalize_survivors(ctr, surv, out, pend);
    return;
  }
  extern __shared__ __align__(16) unsigned char smem_arm[];
  ArmSmem t;
  stage_tables(s, smem_arm, &t);
  __syncthreads();
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  float2* wcs; float* wqv; float4* wsph; double* w64;
  warp_areas(s, smem_arm, table_bytes(s), wib, false, &wcs, &wqv, &wsph, &w64);
  const int D = s.D;
  long long stat_cfg = 0;
  volatile SurvivorEdge* vsurv = surv;
  // static interleave, no shared counter: warp w takes items w, w + W, w + 2W,
  // ... (32 per round, one per lane); items are position-major, so every
  // warp walks its share in BFS-position order and the expensive items (the
  // configurations of long free edges) spread over all warps
  const long long W = (long long)gridDim.x * (blockDim.x >> 5);
  const long long wg = (long long)blockIdx.x * (blockDim.x >> 5) + wib;
  for (long long k0 = 0; first + wg + W * k0 < total; k0 += 32) {
    const long long id = first + wg + W * (k0 + lane);
    int l = 0;
    long long iv = -1;
    if (id < total) {
      l = (int)(id % nsv);
      const long long j = id / nsv;
      const long long p = __ldg(&surv[l].p_next) + j;
      if (p < __ldg(&surv[l].nmax) && (full || !vsurv[l].dead)) {
        const long long N = __ldg(&surv[l].N);
        const long long c = bfs_at(N, p);
        if (incl || (c != 0 && c != N - 1)) iv = c;
      }
    }
    unsigned act = __ballot_sync(MRMG_FULL, iv >= 0);
    while (act) {
      const int srcl = __ffs(act) - 1;
      act &= act - 1;
      const int ls = __shfl_sync(MRMG_FULL, l, srcl);
      const long long is = __shfl_sync(MRMG_FULL, iv, srcl);
      int dead = (lane == 0 && !full) ? vsurv[ls].dead : 0;   // read once, decide warp-uniformly
      if (__shfl_sync(MRMG_FULL, dead, 0)) continue;          // another warp found its collision
      const long long e = __ldg(&surv[ls].e);
      const int N = __ldg(&surv[ls].N);
      EdgeSourceDF sdf;
      float mloc;
      bool nanf;
      load_edge(q1, q2, dtype, e, D, lane, &sdf, &mloc, &nanf);
      sdf.nm1 = (float)(N - 1);
      sdf.rn = __frcp_rn(sdf.nm1);
      sdf.fi = (float)(int)is;   // survivors have N <= 2^24
      stat_cfg++;
      const uint8_t code = eval_config<GPL, SPG, false, BOX_BLOCKS>(s, t, wcs, wqv, wsph, w64, lane, sdf, full != 0,
                                                                    full != 0 || j_lo > 0);
      if (lane == 0) {
        if (code == V_COLLIDE) vsurv[ls].dead = 1;
        else if (code == V_PENDING) vsurv[ls].pend = 1;
      }
    }
  }
  if (lane == 0) atomicAdd((unsigned long long*)&ctr[kCtrStat0], (unsigned long long)stat_cfg);
  if (fin) {
    __shared__ int s_last;
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      s_last = atomicAdd(&ctr[kCtrDoneB], 1) == (int)gridDim.x - 1;
    }
    __syncthreads();
    if (s_last) {
      __threadfence();
      finalize_survivors(ctr, surv, out, pend);
    }
  }
}



// ---------------------------------------------------------------------------
// Small synchronous batches (a planner's single is_collision_free /
// is_edge_collision_free call, or a few): one launch that reads its inputs
// from mapped pinned host memory and writes its hits there.  Items are the
// configurations, or every (edge, position) pair of the edges' checked
// position ranges, laid out edge by edge (offsets and step counts computed on
// the host).  Warp w takes items w, w + W, ...; a configuration the FP32 pass
// leaves pending is decided at once in FP64 by the same warp (the reference's
// interpolation q1 + ((q2 - q1) / (N - 1)) * i for edge positions).  A
// collision sets the edge's device flag to the call's epoch and its host hit
// byte; positions of an edge already seen to collide are skipped.
// ---------------------------------------------------------------------------
template <int GPL, int SPG>
__global__ void __launch_bounds__(128, 1) arm_small_kernel(ArmDev s, SmallBatch b) {
  extern __shared__ __align__(16) unsigned char smem_arm[];
  __shared__ int s_stat[2];
  ArmSmem t;
  stage_tables(s, smem_arm, &t);
  if (threadIdx.x < 2) s_stat[threadIdx.x] = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  float2* wcs; float* wqv; float4* wsph; double* w64;
  warp_areas(s, smem_arm, table_bytes(s), wib, true, &wcs, &wqv, &wsph, &w64);
  const int D = s.D;
  const int W = (int)(gridDim.x * (blockDim.x >> 5));
  int stat_cfg = 0, stat_pend = 0;
  volatile unsigned* flags = b.flags;
  for (int it = (int)(blockIdx.x * (blockDim.x >> 5)) + wib; it < b.items; it += W) {
    if (!b.edges) {
      const CfgSource src{b.q1, b.dtype, (long long)it, D};
      uint8_t code = eval_config<GPL, SPG, false>(s, t, wcs, wqv, wsph, w64, lane, src, false);
      stat_cfg++;
      if (code == V_PENDING) {
        stat_pend++;
        code = eval_config<GPL, SPG, true>(s, t, wcs, wqv, wsph, w64, lane, src, false);
      }
      if (lane == 0 && code == V_COLLIDE) b.hit[it] = 1;
      __syncwarp();
      continue;
    }
    // the edge holding item `it`: the last e with off[e] <= it
    int lo = 0, hi = b.n - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (b.off[mid] <= it) lo = mid;
      else hi = mid - 1;
    }
    const int e = lo;
    const long long N = b.N[e];
    const long long iv = bfs_at(N, b.N_start + (it - b.off[e]));
    if (!b.incl && (iv == 0 || iv == N - 1)) continue;
    if (flags[e] == b.epoch) continue;                      // another position already collides
    EdgeSourceDF sdf;
    float mloc;
    bool nanf;
    load_edge(b.q1, b.q2, b.dtype, e, D, lane, &sdf, &mloc, &nanf);
    sdf.nm1 = (float)(int)(N - 1);                          // N <= 2^24 on this path
    sdf.rn = __frcp_rn(sdf.nm1);
    sdf.fi = (float)(int)iv;
    uint8_t code = eval_config<GPL, SPG, false, BOX_BLOCKS>(s, t, wcs, wqv, wsph, w64, lane, sdf, false);
    stat_cfg++;
    if (code == V_PENDING) {
      stat_pend++;
      EdgeSource64 s64;
      const double denom = (double)(N - 1);
#pragma unroll
      for (int u = 0; u < kJPL; u++) {
        const int j = lane + 32 * u;
        s64.a1[u] = 0.0; s64.dir[u] = 0.0;
        if (j < D) {
          const double a = ldq(b.q1, b.dtype, (long long)e * D + j), c = ldq(b.q2, b.dtype, (long long)e * D + j);
          s64.a1[u] = a;
          s64.dir[u] = __ddiv_rn(__dsub_rn(c, a), denom);   // (q2 - q1) / (N - 1)
        }
      }
      s64.di = (double)iv;
      code = eval_config<GPL, SPG, true>(s, t, wcs, wqv, wsph, w64, lane, s64, false);
    }
    if (lane == 0 && code == V_COLLIDE) {
      flags[e] = b.epoch;
      b.hit[e] = 1;
    }
    __syncwarp();
  }
  if (lane == 0 && stat_cfg) {
    atomicAdd(&s_stat[0], stat_cfg);
    if (stat_pend) atomicAdd(&s_stat[1], stat_pend);
  }
  __syncthreads();
  if (threadIdx.x < 2) b.stats[2 * blockIdx.x + threadIdx.x] = s_stat[threadIdx.x];
}

// sphere centres for the error-bound check: warp per configuration
__global__ void arm_centers_kernel(ArmDev s, const void* q, int dtype, long long n, float* c32, double* c64) {
  extern __shared__ __align__(16) unsigned char smem_arm[];
  ArmSmem t;
  stage_tables(s, smem_arm, &t);
  __syncthreads();
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  float2* wcs; float* wqv; float4* wsph; double* w64;
  warp_areas(s, smem_arm, table_bytes(s), wib, true, &wcs, &wqv, &wsph, &w64);
  const int D = s.D;
  const int nw = gridDim.x * (blockDim.x >> 5);
  for (long long i = blockIdx.x * (blockDim.x >> 5) + wib; i < n; i += nw) {
    for (int j = lane; j < D; j += 32) {
      const double th = ldq(q, dtype, i * D + j);
      if (is_prismatic(t, j)) { wqv[j] = (float)th; wcs[j] = make_float2(1.f, 0.f); }
      else {
        float a;
        reduce_angle_f32(add_offset64(s, j, th), &a);
        float sn, cs;
        sincosf(a, &sn, &cs);
        wcs[j] = make_float2(cs, sn);
      }
      w64[j] = th;
      double sn, cs;
      sincos_exact(add_offset64(s, j, th), &sn, &cs);
      w64[((D + 1) & ~1) + 2 * j] = cs;
      w64[((D + 1) & ~1) + 2 * j + 1] = sn;
    }
    __syncwarp();
    for (int g = lane; g < s.G; g += 32) {
      const int gi = t.grp[g];
      float R[9], p[3];
      chain32(s, t, wcs, wqv, gi & 0xff, gi >> 8, R, p);
      double Rd[9], pd[3];
      chain64(s, w64, w64 + ((D + 1) & ~1), gi & 0xff, gi >> 8, Rd, pd);
      for (int v = 0; v < s.SPG; v++) {
        const int slot = g * s.SPG + v;
        const double* l = s.sph64 + (size_t)slot * 5;
        if (l[3] < 0.0) continue;
        const long long sid = slot;   // output is per slot; the host maps slots to spheres
        const float4 lf = t.sph[slot];
        if (c32) {
          c32[(i * s.G * s.SPG + sid) * 3 + 0] = p[0] + (R[0] * lf.x + R[1] * lf.y + R[2] * lf.z);
          c32[(i * s.G * s.SPG + sid) * 3 + 1] = p[1] + (R[3] * lf.x + R[4] * lf.y + R[5] * lf.z);
          c32[(i * s.G * s.SPG + sid) * 3 + 2] = p[2] + (R[6] * lf.x + R[7] * lf.y + R[8] * lf.z);
        }
        if (c64) {
          for (int k = 0; k < 3; k++)
            c64[(i * s.G * s.SPG + sid) * 3 + k] =
                __dadd_rn(pd[k], __dadd_rn(__dadd_rn(__dmul_rn(Rd[3 * k], l[0]), __dmul_rn(Rd[3 * k + 1], l[1])),
                                           __dmul_rn(Rd[3 * k + 2], l[2])));
        }
      }
    }
    __syncwarp();
  }
}

// Total penetration depth of each configuration (FP64 sphere centres): the
// sum over every sphere-box pair of the radius minus the signed distance of
// the centre to the box (outside: the Euclidean distance; inside: minus the
// distance to the nearest face), and over every pair of spheres on different
// robots of the two radii minus the centre distance, where positive.  Each
// overlap is rounded to a multiple of 2^-40 m and the multiples are summed as
// 64-bit integers, so the total does not depend on the order of the sum.
constexpr double kPenUnit = 0x1p40;

__device__ __forceinline__ long long overlap_units(double ov) {
  return ov > 0.0 ? __double2ll_rn(__dmul_rn(ov, kPenUnit)) : 0ll;
}

__device__ __forceinline__ double box_overlap64(const double* c, const double* bx, double r) {
  double g2 = 0.0, dmax = -1.0e300;
  bool outside = false;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const double d = fmax(__dsub_rn(bx[k], c[k]), __dsub_rn(c[k], bx[3 + k]));
    dmax = fmax(dmax, d);
    if (d > 0.0) {
      g2 = __dadd_rn(g2, __dmul_rn(d, d));
      outside = true;
    }
  }
  return __dsub_rn(r, outside ? __dsqrt_rn(g2) : dmax);
}

__global__ void arm_penetration_kernel(ArmDev s, const void* q, int dtype, long long n, double* out) {
  extern __shared__ __align__(16) unsigned char smem_arm[];
  ArmSmem t;
  stage_tables(s, smem_arm, &t);
  __syncthreads();
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  float2* wcs; float* wqv; float4* wsph; double* w64;
  warp_areas(s, smem_arm, table_bytes(s), wib, true, &wcs, &wqv, &wsph, &w64);
  const int D = s.D, SPG = s.SPG;
  double* wcs64 = w64 + ((D + 1) & ~1);
  double* wc64 = wcs64 + 2 * D;
  const long long nbox = (long long)s.G * SPG * s.B, npair = (long long)s.NP * SPG * SPG;
  const int nw = gridDim.x * (blockDim.x >> 5);
  for (long long i = blockIdx.x * (blockDim.x >> 5) + wib; i < n; i += nw) {
    for (int j = lane; j < D; j += 32) {
      const double th = ldq(q, dtype, i * D + j);
      w64[j] = th;
      double sn, cs;
      sincos_exact(add_offset64(s, j, th), &sn, &cs);
      wcs64[2 * j] = cs;
      wcs64[2 * j + 1] = sn;
    }
    __syncwarp();
    for (int g = lane; g < s.G; g += 32) {
      const int gi = t.grp[g];
      double R[9], p[3];
      chain64(s, w64, wcs64, gi & 0xff, gi >> 8, R, p);
      for (int v = 0; v < SPG; v++) {
        const double* l = s.sph64 + (size_t)(g * SPG + v) * 5;
        double* c = wc64 + (size_t)(g * SPG + v) * 3;
        for (int k = 0; k < 3; k++)
          c[k] = __dadd_rn(p[k], __dadd_rn(__dadd_rn(__dmul_rn(R[3 * k], l[0]), __dmul_rn(R[3 * k + 1], l[1])),
                                           __dmul_rn(R[3 * k + 2], l[2])));
      }
    }
    __syncwarp();
    long long acc = 0;
    for (long long u = lane; u < nbox; u += 32) {
      const int slot = (int)(u / s.B), b = (int)(u % s.B);
      const double r = s.sph64[(size_t)slot * 5 + 3];
      if (r < 0.0) continue;
      acc += overlap_units(box_overlap64(wc64 + 3 * slot, s.box64 + 6 * (size_t)b, r));
    }
    for (long long u = lane; u < npair; u += 32) {
      const int pi = (int)(u / (SPG * SPG)), a = (int)((u / SPG) % SPG), bb = (int)(u % SPG);
      const uint32_t pr = s.pairs[pi];
      const int sa = (int)(pr & 0xffffu) * SPG + a, sb = (int)(pr >> 16) * SPG + bb;
      const double ra = s.sph64[(size_t)sa * 5 + 3], rb = s.sph64[(size_t)sb * 5 + 3];
      if (ra < 0.0 || rb < 0.0) continue;
      const double* ca = wc64 + 3 * sa;
      const double* cb = wc64 + 3 * sb;
      const double dx = __dsub_rn(ca[0], cb[0]), dy = __dsub_rn(ca[1], cb[1]), dz = __dsub_rn(ca[2], cb[2]);
      const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
      acc += overlap_units(__dsub_rn(__dadd_rn(ra, rb), __dsqrt_rn(d2)));
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(MRMG_FULL, acc, off);
    if (lane == 0) out[i] = __dmul_rn(__ll2double_rn(acc), 0x1p-40);
    __syncwarp();
  }
}

// Test-order calibration: for each sample configuration, the set of boxes
// that any sphere touches (FP32, within the re-check band) as a bitmask
// hits[i * words + b / 32].  Verdicts never depend on the order; the order
// decides how soon a colliding configuration stops.
__global__ void arm_box_hits_kernel(ArmDev s, const void* q, int dtype, long long n, uint32_t* hits, int words) {
  extern __shared__ __align__(16) unsigned char smem_arm[];
  ArmSmem t;
  stage_tables(s, smem_arm, &t);
  __syncthreads();
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  float2* wcs; float* wqv; float4* wsph; double* w64;
  warp_areas(s, smem_arm, table_bytes(s), wib, false, &wcs, &wqv, &wsph, &w64);
  const int D = s.D;
  const int nw = gridDim.x * (blockDim.x >> 5);
  for (long long i = blockIdx.x * (blockDim.x >> 5) + wib; i < n; i += nw) {
    const CfgSource src{q, dtype, i, D};
    for (int j = lane; j < D; j += 32) {
      float h, l;
      src.df(j, &h, &l);
      if (is_prismatic(t, j)) { wqv[j] = __fadd_rn(h, l); wcs[j] = make_float2(1.f, 0.f); }
      else {
        float a;
        add_offset_df(s, j, &h, &l);
        reduce_df(h, l, &a);
        float sn, cs;
        sincosf(a, &sn, &cs);
        wcs[j] = make_float2(cs, sn);
      }
    }
    __syncwarp();
    for (int w = 0; w < words; w++) {
      uint32_t bits = 0;
      for (int g = lane; g < s.G; g += 32) {
        const int gi = t.grp[g];
        float R[9], p[3];
        chain32(s, t, wcs, wqv, gi & 0xff, gi >> 8, R, p);
        for (int v = 0; v < s.SPG; v++) {
          const float4 lf = t.sph[g * s.SPG + v];
          const float4 bd = t.band[g * s.SPG + v];
          if (bd.y < 0.f) continue;
          const float x = p[0] + (R[0] * lf.x + R[1] * lf.y + R[2] * lf.z);
          const float y = p[1] + (R[3] * lf.x + R[4] * lf.y + R[5] * lf.z);
          const float z = p[2] + (R[6] * lf.x + R[7] * lf.y + R[8] * lf.z);
          for (int b = 32 * w; b < min(s.B, 32 * w + 32); b++) {
            const float4 bc = t.box[2 * b], bh = t.box[2 * b + 1];
            const float ex = fmaxf(fabsf(x - bc.x) - bh.x, 0.f);
            const float ey = fmaxf(fabsf(y - bc.y) - bh.y, 0.f);
            const float ez = fmaxf(fabsf(z - bc.z) - bh.z, 0.f);
            if (fmaf(ez, ez, fmaf(ey, ey, ex * ex)) <= bd.y) bits |= 1u << (b - 32 * w);
          }
        }
      }
#pragma unroll
      for (int o = 16; o; o >>= 1) bits |= __shfl_xor_sync(MRMG_FULL, bits, o);
      if (lane == 0) hits[i * words + w] = bits;
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------
// dispatch over the compiled (groups per lane, spheres per group) variants
// ---------------------------------------------------------------------------
template <bool RESOLVE>
cudaError_t launch_configs(const ArmDev& s, int gpl, const void* q, int dtype, long long n, uint8_t* out,
                           const CallScratch& sc, int grid, int warps, size_t smem, int full, cudaStream_t st) {
#define MRMG_ARM_CFG(G_, S_)                                                                       \
  if (gpl == G_ && s.SPG == S_) {                                                                  \
    auto k = arm_configs_kernel<G_, S_, RESOLVE>;                                                  \
    k<<<grid, warps * 32, smem, st>>>(s, q, dtype, n, out, sc.ctr, sc.pend, full);                 \
    return cudaGetLastError();                                                                     \
  }
  MRMG_ARM_CFG(1, 6)
  MRMG_ARM_CFG(2, 5)
  MRMG_ARM_CFG(4, 8)
#undef MRMG_ARM_CFG
  return cudaErrorInvalidValue;
}

template <bool RESOLVE>
cudaError_t launch_edges(const ArmDev& s, int gpl, const void* q1, const void* q2, int dtype, long long n,
                         double res, int incl, const long long* Np, long long N_start, long long N_max,
                         uint8_t* out, const CallScratch& sc, int grid, int warps, size_t smem, int full,
                         cudaStream_t st) {
#define MRMG_ARM_EDGE(G_, S_)                                                                      \
  if (gpl == G_ && s.SPG == S_) {                                                                  \
    auto k = arm_edges_kernel<G_, S_, RESOLVE>;                                                    \
    k<<<grid, warps * 32, smem, st>>>(s, q1, q2, dtype, n, res, incl, Np, N_start, N_max, out,     \
                                      sc.ctr, sc.pend, sc.surv, full);                             \
    return cudaGetLastError();                                                                     \
  }
  MRMG_ARM_EDGE(1, 6)
  MRMG_ARM_EDGE(2, 5)
  MRMG_ARM_EDGE(4, 8)
#undef MRMG_ARM_EDGE
  return cudaErrorInvalidValue;
}

// resident CTAs per SM of the phase-B kernel (its register budget differs
// from phase A's), cached per variant and shape
template <int G_, int S_>
int phase_b_occupancy(int warps, size_t smem) {
  static int cached[9] = {0};
  static size_t cached_smem[9] = {0};
  if (warps < 1 || warps > 8) return 1;
  if (cached[warps] == 0 || cached_smem[warps] != smem) {
    int blocks = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, arm_edges_phase_b<G_, S_>, warps * 32, smem) !=
            cudaSuccess || blocks < 1)
      blocks = 1;
    cudaGetLastError();
    cached[warps] = blocks;
    cached_smem[warps] = smem;
  }
  return cached[warps];
}

cudaError_t launch_phase_b(const ArmDev& s, int gpl, const void* q1, const void* q2, int dtype, int incl,
                           const CallScratch& sc, int grid, int warps, size_t smem, int full, int j_lo, int j_hi,
                           uint8_t* out, int num_sms, cudaStream_t st) {
#define MRMG_ARM_PB(G_, S_)                                                                        \
  if (gpl == G_ && s.SPG == S_) {                                                                  \
    grid = std::min(grid, num_sms * phase_b_occupancy<G_, S_>(warps, smem));                       \
    arm_edges_phase_b<G_, S_><<<grid, warps * 32, smem, st>>>(s, q1, q2, dtype, incl, sc.ctr, sc.surv, full, \
                                                              j_lo, j_hi, out, sc.pend);           \
    return cudaGetLastError();                                                                     \
  }
  MRMG_ARM_PB(1, 6)
  MRMG_ARM_PB(2, 5)
  MRMG_ARM_PB(4, 8)
#undef MRMG_ARM_PB
  return cudaErrorInvalidValue;
}

}  // namespace

int arm_supported_spg(int idx) {
  static const int v[] = {6, 5, 8, -1};
  return idx >= 0 && idx < 4 ? v[idx] : -1;
}

int arm_gpl_for_spg(int spg) { return spg == 6 ? 1 : spg == 5 ? 2 : spg == 8 ? 4 : 0; }

static size_t smem_pass(const ArmDev& s, int warps, bool with64) {
  return table_bytes(s) + (size_t)warps * (warp32_bytes(s) + (with64 ? warp64_bytes(s) : 0));
}

// Raises the dynamic shared-memory limit of every kernel of the scene's
// variant (at scene creation, so that later calls can be captured in a
// graph) and returns the resident CTAs per SM of the first-pass edge kernel.
bool arm_tuning_fits(const ArmDev& s) {
  int dev = 0, optin = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
    return false;
  const size_t lim = (size_t)optin - 64;   // static shared memory of the kernels
  return smem_pass(s, 8, false) <= lim && smem_pass(s, 4, true) <= lim && smem_pass(s, 2, true) <= lim;
}

int arm_prepare(const ArmDev& s, int warps) {
  const int gpl = arm_gpl_for_spg(s.SPG);
  int blocks = 0;
  cudaError_t err = cudaErrorInvalidValue;
#define MRMG_PREP(G_, S_)                                                                          \
  if (gpl == G_ && s.SPG == S_) {                                                                  \
    allow_max_smem(arm_edges_kernel<G_, S_, false>);                                               \
    allow_max_smem(arm_edges_kernel<G_, S_, true>);                                                \
    allow_max_smem(arm_configs_kernel<G_, S_, false>);                                             \
    allow_max_smem(arm_configs_kernel<G_, S_, true>);                                              \
    allow_max_smem(arm_edges_phase_b<G_, S_>);                                                     \
    allow_max_smem(arm_small_kernel<G_, S_>);                                                      \
    err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, arm_edges_kernel<G_, S_, false>, warps * 32, \
                                                        smem_pass(s, warps, false));              \
  }
  MRMG_PREP(1, 6)
  MRMG_PREP(2, 5)
  MRMG_PREP(4, 8)
#undef MRMG_PREP
  allow_max_smem(arm_centers_kernel);
  allow_max_smem(arm_box_hits_kernel);
  allow_max_smem(arm_penetration_kernel);
  if (err != cudaSuccess || blocks < 1) return 1;
  return blocks;
}

cudaError_t arm_configs(const ArmDev& s, const void* q, int dtype, long long n, uint8_t* out,
                        const CallScratch& sc, const LaunchShape& ls, int full, cudaStream_t st) {
  const int gpl = arm_gpl_for_spg(s.SPG);
  const size_t smem1 = smem_pass(s, ls.warps, false);
  long long want = (n + (long long)ls.warps * s.cfg_chunk - 1) / ((long long)ls.warps * s.cfg_chunk);
  int grid = (int)std::max(1ll, std::min(want, (long long)ls.ctas));
  cudaError_t e = launch_configs<false>(s, gpl, q, dtype, n, out, sc, grid, ls.warps, smem1, full, st);
  if (e != cudaSuccess) return e;
  const int w2 = 2;
  return launch_configs<true>(s, gpl, q, dtype, n, out, sc, ls.num_sms, w2, smem_pass(s, w2, true), 0, st);
}

cudaError_t arm_edges(const ArmDev& s, const void* q1, const void* q2, int dtype, long long n,
                      double res, int incl, const long long* Np, long long N_start,
                      long long N_max, uint8_t* out, const CallScratch& sc,
                      const LaunchShape& ls, int full, cudaStream_t st) {
  const int gpl = arm_gpl_for_spg(s.SPG);
  const size_t smem1 = smem_pass(s, ls.warps, false);
  long long want = (n + ls.warps - 1) / ls.warps;
  int grid = (int)std::max(1ll, std::min(want, (long long)ls.ctas));
  cudaError_t e = launch_edges<false>(s, gpl, q1, q2, dtype, n, res, incl, Np, N_start, N_max, out, sc,
                                      grid, ls.warps, smem1, full, st);
  if (e != cudaSuccess) return e;
  // B1: the next s.phase_b1 positions of every survivor (kills most colliding
  // survivors); B2: everything left, spread over all warps
  e = launch_phase_b(s, gpl, q1, q2, dtype, incl, sc, ls.ctas, ls.warps, smem1, full, 0, s.phase_b1, out, ls.num_sms,
                     st);
  if (e != cudaSuccess) return e;
  // B2 finalizes the survivors' verdicts in its last CTA
  e = launch_phase_b(s, gpl, q1, q2, dtype, incl, sc, ls.ctas, ls.warps, smem1, full, s.phase_b1, -1, out, ls.num_sms,
                     st);
  if (e != cudaSuccess) return e;
  const int w2 = 2;
  return launch_edges<true>(s, gpl, q1, q2, dtype, n, res, incl, Np, N_start, N_max, out, sc, ls.num_sms,
                            w2, smem_pass(s, w2, true), 0, st);
}

bool arm_small_ok(const ArmDev& s) {
  // four warps with FP32 and FP64 work areas within the 227 KB a CTA can use
  return arm_gpl_for_spg(s.SPG) > 0 && smem_pass(s, kSmallWarps, true) + 64 <= (size_t)227 * 1024;   // + static shared memory
}

cudaError_t arm_small(const ArmDev& s, const SmallBatch& b, int num_sms, cudaStream_t st, int* grid_out) {
  *grid_out = 0;
  if (b.items <= 0) return cudaSuccess;
  const int gpl = arm_gpl_for_spg(s.SPG);
  const int warps = kSmallWarps;
  const size_t smem = smem_pass(s, warps, true);
  const int grid = (int)std::max(1ll, std::min({(long long)(b.items + warps - 1) / warps, (long long)num_sms * 4,
                                                (long long)kSmallMaxCtas}));
  *grid_out = grid;
#define MRMG_ARM_SMALL(G_, S_)                                                                     \
  if (gpl == G_ && s.SPG == S_) {                                                                  \
    arm_small_kernel<G_, S_><<<grid, warps * 32, smem, st>>>(s, b);                                \
    return cudaGetLastError();                                                                     \
  }
  MRMG_ARM_SMALL(1, 6)
  MRMG_ARM_SMALL(2, 5)
  MRMG_ARM_SMALL(4, 8)
#undef MRMG_ARM_SMALL
  return cudaErrorInvalidValue;
}

cudaError_t arm_box_hits(const ArmDev& s, const void* q, int dtype, long long n, uint32_t* hits, int words,
                         cudaStream_t st) {
  const int warps = 4;
  size_t smem = smem_pass(s, warps, false);
  cudaFuncSetAttribute(arm_box_hits_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  long long want = (n + warps - 1) / warps;
  int grid = (int)std::max(1ll, std::min(want, 4096ll));
  arm_box_hits_kernel<<<grid, warps * 32, smem, st>>>(s, q, dtype, n, hits, words);
  return cudaGetLastError();
}

cudaError_t arm_penetration(const ArmDev& s, const void* q, int dtype, long long n, double* out, int num_sms,
                            cudaStream_t st) {
  const int warps = 4;
  const size_t smem = smem_pass(s, warps, true);
  const long long want = (n + warps - 1) / warps;
  const int grid = (int)std::max(1ll, std::min(want, (long long)num_sms * 8));
  arm_penetration_kernel<<<grid, warps * 32, smem, st>>>(s, q, dtype, n, out);
  return cudaGetLastError();
}

cudaError_t arm_centers(const ArmDev& s, const void* q, int dtype, long long n, float* c32, double* c64,
                        cudaStream_t st) {
  const int warps = 4;
  size_t smem = smem_pass(s, warps, true);
  long long want = (n + warps - 1) / warps;
  int grid = (int)std::max(1ll, std::min(want, 4096ll));
  arm_centers_kernel<<<grid, warps * 32, smem, st>>>(s, q, dtype, n, c32, c64);
  return cudaGetLastError();
}

unsigned int arm_stage_timeouts() {
  unsigned int v = 0;
  if (cudaMemcpyFromSymbol(&v, g_stage_timeouts, sizeof v) != cudaSuccess) return 0;
  return v;
}

}  // namespace mrmg
