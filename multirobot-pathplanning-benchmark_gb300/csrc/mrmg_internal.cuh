// mrmg_internal.cuh -- scene tables as the kernels see them, and the host-side
// launchers each translation unit provides to the C ABI layer (mrmg_api.cu).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "mrmg_common.cuh"

namespace mrmg {

constexpr int kMaxRobots = 16;
constexpr int kMaxLinks = 8;
constexpr int kMaxArmDof = 96;
constexpr int kMaxAgents = 16;
constexpr int kMaxAgentDim = 15;

// ---------------------------------------------------------------------------
// Abstract point-agent scene (problems/abstract_env.py:112-131).
// ---------------------------------------------------------------------------
struct AbstractDev {
  int A, dim, D, nb, ns;
  const int* agent_off;                         // [A]
  // exact FP64 tables
  const double *pair_thr, *r2, *box_lo, *box_hi, *sph_pos, *sph_thr;
  // FP32 copies for the bulk pass
  const float *r32, *pair_thr32, *box_lo32, *box_hi32, *sph_pos32, *sph_thr32;
  float omax;       // max |coordinate| / threshold of any obstacle or agent radius
  float delta_k;    // FP32 band per unit magnitude: 8 * dim * 2^-24
  const void* img;  // the FP32 tables in their shared-memory layout (tab_bytes), one bulk copy; NULL: staged by loads
  int sph_batch_form;   // per call: Sphere obstacles in the axis=1 norm form (rounded squares,
                        // numpy sum, sqrt) of Sphere.batch_collides_with_sphere, not the ddot form
};

// shared-memory layout of the FP32 abstract tables (and of AbstractDev::img):
// agent offsets, radii, pair thresholds, box lo, box hi, sphere centres,
// sphere thresholds, each padded to 16 bytes; off[7] = total
__host__ __device__ inline size_t abstract_tab_pad(size_t n) { return (n * 4 + 15) & ~(size_t)15; }
__host__ __device__ inline void abstract_table_layout(const AbstractDev& s, size_t off[8]) {
  const size_t A = s.A, dim = s.dim, nb = s.nb, ns = s.ns;
  const size_t len[7] = {A, A, A * A, nb * dim, nb * dim, ns * dim, ns * A};
  size_t p = 0;
  for (int k = 0; k < 7; k++) {
    off[k] = p;
    p += abstract_tab_pad(len[k]);
  }
  off[7] = p;
}

// ---------------------------------------------------------------------------
// Sphere-arm scene.  Spheres are packed into groups of SPG slots; a group
// holds spheres of one (robot, link) frame.  Padding slots never collide.
// ---------------------------------------------------------------------------
struct ArmDev {
  int R, D, G, SPG, B, NP;
  float delta;      // FP32 re-check band (metres)
  float xy_max;     // planar base |x|,|y| beyond this -> exact path
  float pair_eps;   // FP32 error bound (m^2) of the pair filter s_a + s_b - 2 a.b
  int q_off[kMaxRobots], base_kind[kMaxRobots], nl[kMaxRobots];
  uint32_t prismatic[3];   // bit j: joint j is a planar-base translation
  uint32_t robot_mask;     // bit r: robot r's spheres take part (per call; all robots by default)
  // exact FP64 tables (global memory)
  const double* base64;    // [R*12]
  const double* dh64;      // [R*8*4]  a, d, cos(alpha), sin(alpha)
  const double* sph64;     // [G*SPG*5] local xyz, radius, radius^2 (radius < 0: padding)
  const double* box64;     // [B*6]    lo xyz, hi xyz
  // FP32 tables (staged into shared memory)
  const float4* base32;    // [R*3]    rows (r0, r1, r2, p_i)
  const float4* dh32;      // [R*8]    a, d, cos(alpha), sin(alpha)
  const float4* sph32;     // [G*SPG]  local xyz, radius
  const float4* band32;    // [G*SPG]  rlo^2, rhi^2, r + delta, r - delta  (padding: -1,-1,0,0)
  const float4* box32;     // [B*2]    centre xyz, half extents xyz
  const int* grp;          // [G]      robot | link << 8
  const float4* gbs32;     // [G]      group bound: local centre xyz, radius^2 (radius covers every
                           //          sphere of the group plus 4 delta; padding groups: -1)
  const uint32_t* pairs;   // [NP]     group a | group b << 16 (different robots)
  // fixed joint-angle offsets (imported general chains): revolute joint j
  // turns by q[j] + offset[j]; NULL when the scene has none
  const float2* off32;     // [D]      offset as FP32 hi + lo
  const double* off64;     // [D]
  // the FP32 tables above, in their shared-memory layout (arm_table_layout),
  // staged by one bulk asynchronous copy; NULL: staged by loads
  const void* img;
  // launch tuning (never changes a verdict): boxes per compacted block of
  // the block box phases (the obstacle tile), boxes tested one by one before
  // the blocks on first positions, configurations a warp takes from the
  // work queue at a time, positions per survivor in the first phase-B launch
  int box_block, box_head, cfg_chunk, phase_b1;
};

constexpr int kMaxBoxBlock = 32, kMaxBoxHead = 64, kMaxCfgChunk = 32, kMaxPhaseB1 = 64;

__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

// byte offsets of the FP32 arm tables in shared memory (and in ArmDev::img):
// boxes, base rows, DH rows, spheres, sphere bands, group ids, group bounds,
// group pairs; off[8] = total
__host__ __device__ inline void arm_table_layout(const ArmDev& s, size_t off[9]) {
  size_t p = 0;
  off[0] = p; p += align16(sizeof(float4) * s.B * 2);
  off[1] = p; p += align16(sizeof(float4) * s.R * 3);
  off[2] = p; p += align16(sizeof(float4) * s.R * kMaxLinks);
  off[3] = p; p += align16(sizeof(float4) * s.G * s.SPG);
  off[4] = p; p += align16(sizeof(float4) * s.G * s.SPG);
  off[5] = p; p += align16(sizeof(int) * s.G);
  off[6] = p; p += align16(sizeof(float4) * s.G);
  off[7] = p; p += align16(sizeof(uint32_t) * s.NP);
  off[8] = p;
}

// ---------------------------------------------------------------------------
// Path-penetration cost tables of an arm scene: the real spheres (padding
// dropped) grouped by robot, then by frame, so the spheres of other robots
// are [0, first of robot) and [first of next robot, S); boxes in input order.
// ---------------------------------------------------------------------------
struct PenDev {
  int S, B, NTK;
  const float4* sph;     // [S]  local xyz, radius
  const int4* task;      // [NTK] sphere, second sphere of the same robot (-1: none),
                         //       the robot's first sphere, the next robot's first sphere
  const float4* box;     // [2B] centre xyz, half extents xyz
  int lk[kMaxRobots][kMaxLinks + 2];   // spheres of (robot r, frame k): [lk[r][k], lk[r][k+1])
};

// cost of one pair with signed distance d: softplus(beta (margin - d)) / (beta scale)
struct PenParams {
  float margin, inv_scale, beta, inv_beta, smooth_w;
};

// per-call scratch counters (device): [0] work queue, [1] pending count,
// [2] error bits, [3] pass-two queue, [4..5] configurations evaluated (64-bit),
// [6] surviving edges, [7] longest remaining position range, [8..9] phase-B
// queue (64-bit), [10] finished CTAs of the last phase-B launch
constexpr int kCtrQueue = 0, kCtrPending = 1, kCtrErr = 2, kCtrQueue2 = 3, kCtrStat0 = 4;
constexpr int kCtrL1 = 6, kCtrMaxJ = 7, kCtrQueueB = 8;
constexpr int kCtrDoneB = 10;   // CTAs of the last phase-B launch that have finished
constexpr int kNumCtr = 16;

// an edge that survived its first checked configuration: its remaining
// BFS positions [p_next, nmax) are dealt to all warps
struct SurvivorEdge {
  long long e;
  int N, p_next, nmax;
  int dead;      // a remaining configuration collides
  int pend;      // a configuration needs the exact FP64 pass
  int pad;
};

struct CallScratch {
  int* ctr;             // [kNumCtr]
  long long* pend;      // pending item list
  SurvivorEdge* surv;   // surviving edges (arm edge checks)
  long long pend_cap;
};

struct LaunchShape {
  int ctas, warps;   // persistent grid
  int num_sms;
};

// one small synchronous batch (arm_small): inputs, hits and statistics in
// mapped pinned host memory, per-edge flags in device memory
constexpr int kSmallWarps = 4;   // warps per CTA of the small-batch kernel
constexpr int kSmallMaxCtas = 2048;
struct SmallBatch {
  int n;                 // configurations or edges
  int items;             // configurations, or the edges' position ranges summed
  int edges;             // 0: configurations, 1: edges
  int dtype, incl;
  long long N_start;
  const int* off;        // [n + 1] first item of each edge
  const int* N;          // [n]     step count of each edge (<= 2^24)
  const void* q1;        // [n, D]  configurations, or the edges' first endpoints
  const void* q2;        // [n, D]  the edges' second endpoints
  uint8_t* hit;          // [n]     set to 1 on a collision (zeroed by the caller)
  int* stats;            // [2 * CTAs] per CTA: configurations evaluated, FP64 decisions
  unsigned* flags;       // [n]     device: edge e collides in this call iff flags[e] == epoch
  unsigned epoch;
};

// Raises a kernel's dynamic shared-memory limit to the device's opt-in
// maximum less the kernel's static shared memory.  The limit is per kernel
// and process-wide: setting it once to the maximum means one scene's set-up
// never lowers it under another scene's launches.
template <class K>
inline cudaError_t allow_max_smem(K kernel) {
  int dev = 0, optin = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  cudaFuncAttributes fa{};
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, kernel);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 optin - (int)fa.sharedSizeBytes);
  return e;
}

// total penetration depth per configuration (FP64; see arm_penetration_kernel)
cudaError_t arm_penetration(const ArmDev& s, const void* q, int dtype, long long n, double* out, int num_sms,
                            cudaStream_t st);

// the serving batcher's gather of host request arrays (mrmg_serving_gather)
cudaError_t serving_gather(const void* table, int max_src, int D, long long ccap, long long ecap, float* q1,
                           float* q2, long long* N, int* err, cudaStream_t st);

// whether every arm kernel's shared memory fits a CTA with this tuning
bool arm_tuning_fits(const ArmDev& s);

// table-staging copies that timed out in each translation unit's kernels
unsigned int arm_stage_timeouts();
unsigned int abstract_stage_timeouts();

struct SliceTab {
  int A, D, end_all;
  int s[64], e[64];
};

// FP64 distance of one difference row d(k) = a[k] - b[k] with the reference's
// operation order (NpConfiguration._batch_dist, core/configuration.py:303-329:
// sequential unfused sums of d*d, IEEE sqrt, strict '>' maxima)
template <class Diff>
__device__ __forceinline__ double dist_of(const SliceTab& t, int metric, Diff d) {
  if (metric == MRMG_METRIC_EUCLIDEAN) {
    double acc = 0.0;
    for (int k = 0; k < t.end_all; k++) { double v = d(k); acc = __dadd_rn(acc, __dmul_rn(v, v)); }
    return sqrt(acc);
  }
  if (metric == MRMG_METRIC_MAX) {
    double m = fabs(d(0));
    for (int k = 1; k < t.D; k++) { double v = fabs(d(k)); if (v > m) m = v; }
    return m;
  }
  double red = 0.0;
  for (int i = 0; i < t.A; i++) {
    double acc = 0.0;
    for (int k = t.s[i]; k < t.e[i]; k++) { double v = d(k); acc = __dadd_rn(acc, __dmul_rn(v, v)); }
    const double r = sqrt(acc);
    if (metric == MRMG_METRIC_SUM_EUCLIDEAN) red = __dadd_rn(red, r);
    else if (i == 0 || r > red) red = r;
  }
  return red;
}

// host launchers ------------------------------------------------------------
cudaError_t abstract_configs(const AbstractDev& s, const void* q, int dtype, long long n,
                             uint8_t* out, const CallScratch& sc, const LaunchShape& ls,
                             cudaStream_t st);
// edges per call up to which the abstract edge check runs the flat single-launch kernel
constexpr long long kFlatMaxEdges = 65536;
cudaError_t abstract_edges(const AbstractDev& s, const void* q1, const void* q2, int dtype,
                           long long n, double res, int incl, const long long* Np,
                           long long N_start, long long N_max, uint8_t* out,
                           const CallScratch& sc, const LaunchShape& ls, cudaStream_t st);
int abstract_prepare(const AbstractDev& s);   // kernel attributes, once per scene (before any capture)
// single launches on caller-visible (e.g. mapped host) buffers, no counters;
// the edge kernel reports its error bits per CTA in cta_err[grid] (plain stores)
cudaError_t abstract_configs_mapped(const AbstractDev& s, const void* q, int dtype, long long n, uint8_t* out,
                                    int num_sms, cudaStream_t st);
cudaError_t abstract_edges_mapped(const AbstractDev& s, const void* q1, const void* q2, int dtype, long long n,
                                  double res, int incl, const long long* Np, long long N_start, long long N_max,
                                  uint8_t* out, uint8_t* cta_err, int num_sms, cudaStream_t st, int* grid_out);

cudaError_t arm_configs(const ArmDev& s, const void* q, int dtype, long long n, uint8_t* out,
                        const CallScratch& sc, const LaunchShape& ls, int full, cudaStream_t st);
cudaError_t arm_edges(const ArmDev& s, const void* q1, const void* q2, int dtype, long long n,
                      double res, int incl, const long long* Np, long long N_start,
                      long long N_max, uint8_t* out, const CallScratch& sc,
                      const LaunchShape& ls, int full, cudaStream_t st);
bool arm_small_ok(const ArmDev& s);   // the single-launch kernel fits the scene's shared memory
cudaError_t arm_small(const ArmDev& s, const SmallBatch& b, int num_sms, cudaStream_t st, int* grid_out);
cudaError_t arm_box_hits(const ArmDev& s, const void* q, int dtype, long long n, uint32_t* hits, int words,
                         cudaStream_t st);
cudaError_t arm_centers(const ArmDev& s, const void* q, int dtype, long long n, float* c32,
                        double* c64, cudaStream_t st);
int arm_prepare(const ArmDev& s, int warps);
int arm_supported_spg(int idx);   // list of compiled SPG values, -1 at end
int arm_gpl_for_spg(int spg);

// shared memory of a penetration launch whose gradient covers robots [gr0, gr1)
size_t pen_smem_bytes(const ArmDev& a, const PenDev& pd, int grad, int warps, int gr0, int gr1);
// splits the robots into the fewest groups of consecutive robots whose
// gradient launches fit in smem_max bytes: bounds[0..n] (n returned; 0 when
// none fits)
int pen_grad_groups(const ArmDev& a, const PenDev& pd, int warps, size_t smem_max, int* bounds);
cudaError_t pen_launch(const ArmDev& a, const PenDev& pd, const PenParams& pp, const float* paths, long long P, int T,
                       const float* gout, double* seg, double* cost, float* wp_cost, float* grad, int warps,
                       int n_groups, const int* bounds, cudaStream_t st);

cudaError_t binary_indices(long long N, long long* out, cudaStream_t st, int chunked);


cudaError_t knn_exact(const double* qs, long long Q, const int* q_mode, const long long* q_list, long long n_list,
                      const double* nodes, const long long* mode_beg, const long long* mode_end, const SliceTab& t,
                      int metric, int k, long long* out_idx, double* out_dist, int num_sms, cudaStream_t st);
struct KnnStore;
struct KnnScratch;
bool knn_tc_supported(const SliceTab& t, int metric);
cudaError_t knn_store_build(KnnStore* s, const double* d_nodes, long long M, const long long* h_mode_off, int n_modes,
                            const SliceTab& t, int metric, int D, cudaStream_t st);
cudaError_t knn_store_append(KnnStore* s, int mode, const double* rows, long long n, cudaStream_t st);
cudaError_t knn_store_remove(KnnStore* s, int mode, long long idx, cudaStream_t st);
long long knn_store_count(const KnnStore* s, int mode);
int knn_store_modes(const KnnStore* s);
bool knn_store_tc(const KnnStore* s);
void knn_store_set_path(KnnStore* s, int path);
void knn_store_free(KnnStore* s);
cudaError_t knn_store_query(KnnStore* s, KnnScratch* scr, const double* d_qs, long long Q, const int* h_q_mode, int k,
                            long long* d_idx, double* d_dist, int num_sms, int* used_tc, int* n_fallback,
                            cudaStream_t st);
KnnStore* knn_store_new();
void knn_store_delete(KnnStore* s);
KnnScratch* knn_scratch_new();
void knn_scratch_delete(KnnScratch* s);
struct NearState;
NearState* near_state_new();
void near_state_delete(NearState* ns);
cudaError_t near_query(NearState* ns, KnnStore* s, const double* d_qs, long long Q, const int* h_q_mode,
                       const double* h_radius, double add_eps, long long* d_offsets, long long* d_idx, double* d_dist,
                       long long cap, int num_sms, long long* total_out, cudaStream_t st);
cudaError_t near_fetch(NearState* ns, long long* d_idx, double* d_dist, long long cap, int num_sms, cudaStream_t st);
long long near_last_total(const NearState* ns);
cudaError_t umma_selftest(const void* A, const void* B, int N, float* C, int* err, cudaStream_t st);

cudaError_t dist_matrix(const double* qs, long long Q, const double* nodes, long long M, const SliceTab& t, int metric,
                        double* out, int num_sms, cudaStream_t st);
cudaError_t batch_cost(const double* a, const double* b, long long M, const SliceTab& t, int cmetric, int red, double w,
                       int mode, double* out, int num_sms, cudaStream_t st);

}  // namespace mrmg
