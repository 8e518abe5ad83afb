// mrmg_api.cu -- the C ABI: scene handles, per-handle scratch, status codes.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <mutex>
#include <new>
#include <numeric>
#include <string>
#include <vector>

#include <cuda.h>

#include "mrmg_bulk.cuh"
#include "mrmg_internal.cuh"

using namespace mrmg;

namespace {

thread_local std::string g_last_error;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  try {
    g_last_error = buf;
  } catch (...) {
    g_last_error.clear();
  }
  return code;
}

int cuda_fail(cudaError_t e, const char* where) {
  return fail(MRMG_ERR_CUDA, "%s: %s", where, cudaGetErrorString(e));
}

// The handler of the entry points whose host allocations grow with their
// inputs (function-try-blocks): no C++ exception unwinds through the C ABI.
int host_fail() {
  try {
    throw;
  } catch (const std::bad_alloc&) {
    return fail(MRMG_ERR_HOST, "host memory allocation failed");
  } catch (const std::exception& ex) {
    return fail(MRMG_ERR_HOST, "host exception: %s", ex.what());
  } catch (...) {
    return fail(MRMG_ERR_HOST, "unknown host exception");
  }
}

// One device allocation holding every table of a scene.
struct DevBlock {
  std::vector<unsigned char> host;
  std::vector<std::pair<size_t, void**>> fixups;
  template <typename T>
  void add(const T* data, size_t count, const T** dst) {
    size_t off = (host.size() + 255) & ~(size_t)255;
    host.resize(off + sizeof(T) * std::max<size_t>(count, 1));
    if (count) std::memcpy(host.data() + off, data, sizeof(T) * count);
    fixups.push_back({off, (void**)dst});
  }
  cudaError_t upload(void** dev) {
    cudaError_t e = cudaMalloc(dev, host.size());
    if (e != cudaSuccess) return e;
    e = cudaMemcpy(*dev, host.data(), host.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return e;
    for (auto& f : fixups) *f.second = (unsigned char*)*dev + f.first;
    return cudaSuccess;
  }
};

}  // namespace

// creation inputs of an arm scene that per-mode tables are built from
struct ArmSrc {
  int S = 0, B = 0, SPG = 0, G = 0;
  double delta = 0.0;
  std::vector<double> local, radius, box_lo, box_hi;
  std::vector<int> slot_sphere, grp;
};

// one complete set of sphere- and box-dependent tables: the device views in
// `d` / `pd` and host copies of the box tables (their test order can be tuned)
struct ArmTables {
  ArmDev d{};
  PenDev pd{};
  std::vector<float4> box32_host;
  std::vector<double> box64_host;
  // host data kept until the upload
  std::vector<float4> sph32, band32, gbs, pen_sph, pen_box;
  std::vector<double> sph64;
  std::vector<int4> pen_task;
};

// work-queue counters are 32-bit: keep every batch well below 2^31
constexpr long long kMaxBatch = (1ll << 31) - (1ll << 26);

struct mrmg_scene {
  int kind = 0;   // 0 abstract, 1 arm
  int q_dim = 0;
  AbstractDev ab{};
  ArmDev arm{};
  void* d_tables = nullptr;
  int* d_ctr = nullptr;
  long long* d_pend = nullptr;
  SurvivorEdge* d_surv = nullptr;
  long long pend_cap = 0;
  int* h_ctr = nullptr;       // pinned mirror of the counters
  int ctas = 0, warps = 0;    // persistent launch shape (0 = automatic)
  int occ_ctas_per_sm = 0;    // resident CTAs per SM of the first pass (8 warps)
  int num_sms = 0;
  int device = 0;
  double band = 0.0;
  int64_t n_pairs_groups = 0;
  std::vector<int> slot_to_sphere;   // arm: slot -> input sphere index (-1 padding)
  PenDev pen{};                      // arm: path-penetration cost tables
  double* d_pen_seg = nullptr;       // per-segment cost scratch
  long long pen_seg_cap = 0;
  // arm: the table sets -- the scene as created, and one per mode when modes
  // are declared; `arm` / `pen` are copies of the current set's views
  ArmTables base;
  std::vector<ArmTables> modes;
  int cur_mode = -1;
  void* d_mode_tables = nullptr;
  std::vector<void*> imgs;    // table images (bulk-staged copies of the FP32 tables)
  void* d_offsets = nullptr;          // arm: fixed joint-angle offsets (FP32 hi/lo pairs, FP64)
  ArmSrc src;
  ArmTables& tabs() { return cur_mode < 0 ? base : modes[cur_mode]; }
  // host-pointer calls: the scene's own stream and one staging buffer (pinned
  // host image + device copy) holding a call's counters, hits and inputs
  cudaStream_t own_stream = nullptr;
  unsigned char* h_stage = nullptr;   // mapped pinned host memory
  unsigned char* m_stage = nullptr;   // its device address
  unsigned char* d_stage = nullptr;   // device memory of the same size
  size_t stage_cap = 0;
  unsigned* d_small_flags = nullptr;  // single-launch path: per-edge "collides in call epoch" flags
  unsigned small_epoch = 0;
  // the device reads pageable host memory coherently (a CPU-GPU link with
  // address translation): host-pointer calls hand the caller's input arrays
  // to the kernels instead of staging them
  bool pageable = false;
};

namespace {

int init_common(mrmg_scene* sc) {
  cudaError_t e = cudaGetDevice(&sc->device);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  e = cudaDeviceGetAttribute(&sc->num_sms, cudaDevAttrMultiProcessorCount, sc->device);
  if (e != cudaSuccess) return cuda_fail(e, "cudaDeviceGetAttribute");
  int pg = 0;
  if (cudaDeviceGetAttribute(&pg, cudaDevAttrPageableMemoryAccess, sc->device) != cudaSuccess) pg = 0;
  const char* stage = std::getenv("MRMG_STAGE_HOST_INPUTS");   // "1": always stage host inputs
  sc->pageable = pg != 0 && !(stage && stage[0] == '1');
  e = cudaMalloc(&sc->d_ctr, sizeof(int) * kNumCtr);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(counters)");
  e = cudaMallocHost(&sc->h_ctr, sizeof(int) * kNumCtr);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMallocHost");
  return MRMG_OK;
}

int ensure_pending(mrmg_scene* sc, long long n, cudaStream_t st) {
  if (n <= sc->pend_cap) return MRMG_OK;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  cudaStreamIsCapturing(st, &cap);
  if (cap != cudaStreamCaptureStatusNone)
    return fail(MRMG_ERR_ARG, "scratch for %lld items must be reserved before stream capture", n);
  long long cap_new = std::max(n, 2 * sc->pend_cap);
  long long* p = nullptr;
  SurvivorEdge* sv = nullptr;
  cudaError_t e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
  e = cudaMalloc(&p, sizeof(long long) * cap_new);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(pending)");
  if (sc->kind == 1) {
    e = cudaMalloc(&sv, sizeof(SurvivorEdge) * cap_new);
    if (e != cudaSuccess) { cudaFree(p); return cuda_fail(e, "cudaMalloc(survivors)"); }
  }
  if (sc->d_pend) cudaFree(sc->d_pend);
  if (sc->d_surv) cudaFree(sc->d_surv);
  sc->d_pend = p;
  sc->d_surv = sv;
  sc->pend_cap = cap_new;
  return MRMG_OK;
}

LaunchShape shape(mrmg_scene* sc) {
  LaunchShape ls;
  ls.num_sms = sc->num_sms;
  ls.warps = sc->warps > 0 ? sc->warps : 8;
  if (sc->ctas > 0) ls.ctas = sc->ctas;
  else if (sc->kind == 1) ls.ctas = sc->num_sms * std::max(1, sc->occ_ctas_per_sm * 8 / ls.warps);
  else ls.ctas = sc->num_sms * 8;
  return ls;
}

// the scene's stream and mapped staging buffer (host-pointer calls, below)
int ensure_stage(mrmg_scene* sc, size_t bytes);
constexpr size_t kStageHead = 16 * 1024;   // per-CTA statistics / error bytes at the head of the mapped buffer

int finish_call(mrmg_scene* sc, cudaStream_t st, int flags) {
  cudaError_t e = cudaMemcpyAsync(sc->h_ctr, sc->d_ctr, sizeof(int) * kNumCtr, cudaMemcpyDeviceToHost, st);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(status)");
  if (flags & MRMG_FLAG_ASYNC) return MRMG_OK;
  e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "kernel execution");
  int err = sc->h_ctr[kCtrErr];
  if (err & E_N_START) return fail(MRMG_ERR_N_START, "N_start > N for at least one edge");
  if (err & E_BAD_INPUT) return fail(MRMG_ERR_ARG, "non-finite or out-of-range edge length (int() of nan/inf)");
  if (err & E_TIMEOUT) return fail(MRMG_ERR_TIMEOUT, "a bounded device wait ran out");
  return MRMG_OK;
}

float f32_up(double x) {   // FP32 value >= x
  float f = (float)x;
  if ((double)f < x) f = nextafterf(f, INFINITY);
  return f;
}
float f32_down(double x) {
  float f = (float)x;
  if ((double)f > x) f = nextafterf(f, -INFINITY);
  return f;
}

// Slot tables of one sphere set: slots whose sphere is off (or absent) are
// padding, and each group bound covers the group's spheres that are on: the
// centre of their local offsets and a radius over |offset - centre| + r,
// widened by 4 delta (FP32 error of the group centre and of each sphere
// centre, plus rounding of the bound test); a group with none is never near.
void sphere_tables(const ArmSrc& a, const std::vector<char>& on, ArmTables* t) {
  const int NS = a.G * a.SPG;
  t->sph32.assign(NS, make_float4(0.f, 0.f, 0.f, 0.f));
  t->band32.assign(NS, make_float4(-1.f, -1.f, 0.f, 0.f));
  t->sph64.assign((size_t)NS * 5, 0.0);
  t->gbs.assign(a.G, make_float4(0.f, 0.f, 0.f, -1.f));
  auto live = [&](int sl) { const int i = a.slot_sphere[sl]; return i >= 0 && on[i] ? i : -1; };
  for (int sl = 0; sl < NS; sl++) {
    const int i = live(sl);
    if (i < 0) { t->sph64[(size_t)sl * 5 + 3] = -1.0; continue; }
    const double* l = &a.local[3 * i];
    const double r = a.radius[i];
    t->sph32[sl] = make_float4((float)l[0], (float)l[1], (float)l[2], (float)r);
    const double rhi = r + a.delta, rlo = r - a.delta;
    t->band32[sl] = make_float4(rlo > 0 ? f32_down(rlo * rlo * (1.0 - 1e-6)) : -1.f, f32_up(rhi * rhi * (1.0 + 1e-6)),
                                f32_up(r + a.delta), f32_down(r - a.delta));
    for (int k = 0; k < 3; k++) t->sph64[(size_t)sl * 5 + k] = l[k];
    t->sph64[(size_t)sl * 5 + 3] = r;
    t->sph64[(size_t)sl * 5 + 4] = r * r;
  }
  for (int g = 0; g < a.G; g++) {
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    int cnt = 0;
    for (int v = 0; v < a.SPG; v++) {
      const int i = live(g * a.SPG + v);
      if (i < 0) continue;
      cnt++;
      for (int k = 0; k < 3; k++) {
        lo[k] = std::min(lo[k], a.local[3 * i + k]);
        hi[k] = std::max(hi[k], a.local[3 * i + k]);
      }
    }
    if (!cnt) continue;
    double c[3], rad = 0.0;
    for (int k = 0; k < 3; k++) c[k] = 0.5 * (lo[k] + hi[k]);
    for (int v = 0; v < a.SPG; v++) {
      const int i = live(g * a.SPG + v);
      if (i < 0) continue;
      double d2 = 0.0;
      for (int k = 0; k < 3; k++) d2 += (a.local[3 * i + k] - c[k]) * (a.local[3 * i + k] - c[k]);
      rad = std::max(rad, std::sqrt(d2) + a.radius[i]);
    }
    rad += 4.0 * a.delta;
    t->gbs[g] = make_float4((float)c[0], (float)c[1], (float)c[2], f32_up(rad * rad * (1.0 + 1e-6)));
  }
}

// box tables of a box set, larger boxes first (earlier certain collisions;
// verdicts do not depend on the order): FP32 centre / half extent (the band
// absorbs their rounding, |box| < 1e6 m) and FP64 lo / hi
void box_tables(const ArmSrc& a, std::vector<int> boxes, ArmTables* t) {
  auto vol = [&](int b) {
    double v = 1.0;
    for (int k = 0; k < 3; k++) v *= std::max(0.0, a.box_hi[3 * b + k] - a.box_lo[3 * b + k]);
    return v;
  };
  std::stable_sort(boxes.begin(), boxes.end(), [&](int x, int y) { return vol(x) > vol(y); });
  const int B = (int)boxes.size();
  t->box32_host.assign(2 * (size_t)B, make_float4(0.f, 0.f, 0.f, 0.f));
  t->box64_host.assign(6 * (size_t)B, 0.0);
  for (int bi = 0; bi < B; bi++) {
    const double* lo = &a.box_lo[3 * boxes[bi]];
    const double* hi = &a.box_hi[3 * boxes[bi]];
    t->box32_host[2 * bi] = make_float4((float)(0.5 * (lo[0] + hi[0])), (float)(0.5 * (lo[1] + hi[1])),
                                        (float)(0.5 * (lo[2] + hi[2])), 0.f);
    t->box32_host[2 * bi + 1] = make_float4((float)(0.5 * (hi[0] - lo[0])), (float)(0.5 * (hi[1] - lo[1])),
                                            (float)(0.5 * (hi[2] - lo[2])), 0.f);
    for (int k = 0; k < 3; k++) { t->box64_host[6 * (size_t)bi + k] = lo[k]; t->box64_host[6 * (size_t)bi + 3 + k] = hi[k]; }
  }
  t->d.B = B;
}

// penetration-cost tables: the set's spheres in slot order (robot, then
// frame), tasks of two consecutive spheres of one robot, boxes in the given order
void pen_tables(const ArmSrc& a, int R, const std::vector<char>& on, const std::vector<int>& boxes, ArmTables* t) {
  PenDev& pd = t->pd;
  int cnt[kMaxRobots][kMaxLinks + 1] = {};
  t->pen_sph.clear();
  t->pen_task.clear();
  for (int sl = 0; sl < a.G * a.SPG; sl++) {
    const int i = a.slot_sphere[sl];
    if (i < 0 || !on[i]) continue;
    const int r = a.grp[sl / a.SPG] & 0xff, k = a.grp[sl / a.SPG] >> 8;
    cnt[r][k]++;
    t->pen_sph.push_back(make_float4((float)a.local[3 * i], (float)a.local[3 * i + 1], (float)a.local[3 * i + 2],
                                     (float)a.radius[i]));
  }
  int acc = 0;
  for (int r = 0; r < kMaxRobots; r++) {
    for (int k = 0; k <= kMaxLinks; k++) { pd.lk[r][k] = acc; acc += cnt[r][k]; }
    pd.lk[r][kMaxLinks + 1] = acc;
  }
  for (int r = 0; r < R; r++) {
    const int s0 = pd.lk[r][0], s1 = pd.lk[r][kMaxLinks + 1];
    for (int i = s0; i < s1; i += 2) t->pen_task.push_back(make_int4(i, i + 1 < s1 ? i + 1 : -1, s0, s1));
  }
  t->pen_box.assign(2 * boxes.size(), make_float4(0.f, 0.f, 0.f, 0.f));
  for (size_t j = 0; j < boxes.size(); j++) {
    const double* lo = &a.box_lo[3 * boxes[j]];
    const double* hi = &a.box_hi[3 * boxes[j]];
    t->pen_box[2 * j] = make_float4((float)(0.5 * (lo[0] + hi[0])), (float)(0.5 * (lo[1] + hi[1])),
                                    (float)(0.5 * (lo[2] + hi[2])), 0.f);
    t->pen_box[2 * j + 1] = make_float4((float)(0.5 * (hi[0] - lo[0])), (float)(0.5 * (hi[1] - lo[1])),
                                        (float)(0.5 * (hi[2] - lo[2])), 0.f);
  }
  pd.S = (int)t->pen_sph.size();
  pd.B = (int)boxes.size();
  pd.NTK = (int)t->pen_task.size();
}

// The FP32 arm tables of view `v` copied into one device buffer in their
// shared-memory layout (arm_table_layout), so that a kernel stages them with
// one bulk asynchronous copy; v->img stays NULL (loads) when they are too large.
cudaError_t build_arm_image(std::vector<void*>* owned, ArmDev* v) {
  size_t off[9];
  arm_table_layout(*v, off);
  v->img = nullptr;
  if (off[8] == 0 || off[8] > kStageMaxBytes) return cudaSuccess;
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, off[8]);
  if (e != cudaSuccess) return e;
  owned->push_back(p);
  unsigned char* b = (unsigned char*)p;
  e = cudaMemset(p, 0, off[8]);
  const size_t SL = (size_t)v->G * v->SPG;
  const void* src[8] = {v->box32, v->base32, v->dh32, v->sph32, v->band32, v->grp, v->gbs32, v->pairs};
  const size_t bytes[8] = {sizeof(float4) * 2 * v->B, sizeof(float4) * 3 * v->R, sizeof(float4) * kMaxLinks * v->R,
                           sizeof(float4) * SL, sizeof(float4) * SL, sizeof(int) * v->G, sizeof(float4) * v->G,
                           sizeof(uint32_t) * v->NP};
  for (int k = 0; k < 8 && e == cudaSuccess; k++)
    if (bytes[k]) e = cudaMemcpy(b + off[k], src[k], bytes[k], cudaMemcpyDeviceToDevice);
  if (e == cudaSuccess) v->img = p;
  return e;
}

// registers a table set's arrays with the upload block
void add_tables(DevBlock& blk, ArmTables* t) {
  blk.add(t->sph64.data(), t->sph64.size(), &t->d.sph64);
  blk.add(t->box64_host.data(), t->box64_host.size(), &t->d.box64);
  blk.add(t->sph32.data(), t->sph32.size(), &t->d.sph32);
  blk.add(t->band32.data(), t->band32.size(), &t->d.band32);
  blk.add(t->box32_host.data(), t->box32_host.size(), &t->d.box32);
  blk.add(t->gbs.data(), t->gbs.size(), &t->d.gbs32);
  blk.add(t->pen_sph.data(), t->pen_sph.size(), &t->pd.sph);
  blk.add(t->pen_task.data(), t->pen_task.size(), &t->pd.task);
  blk.add(t->pen_box.data(), t->pen_box.size(), &t->pd.box);
}

// drops the host copies needed only for the upload
void trim_tables(ArmTables* t) {
  for (auto* v : {&t->sph32, &t->band32, &t->gbs, &t->pen_sph, &t->pen_box}) std::vector<float4>().swap(*v);
  std::vector<double>().swap(t->sph64);
  std::vector<int4>().swap(t->pen_task);
}

}  // namespace

extern "C" {

const char* mrmg_version(void) { return "mrmg_gb300 0.1 (sm_103a)"; }
const char* mrmg_last_error(void) { return g_last_error.c_str(); }

int mrmg_abstract_scene_create(int32_t n_agents, int32_t dim, int32_t q_dim, const int64_t* h_agent_offsets,
                               const double* h_agent_radius, const double* h_pair_threshold,
                               const double* h_agent_radius_sq, int32_t n_boxes, const double* h_box_lo,
                               const double* h_box_hi, int32_t n_spheres, const double* h_sphere_pos,
                               const double* h_sphere_radius, const double* h_sphere_threshold,
                               mrmg_scene** out) try {
  if (!out) return fail(MRMG_ERR_ARG, "out is NULL");
  *out = nullptr;
  if (n_agents < 1 || n_agents > kMaxAgents) return fail(MRMG_ERR_UNSUPPORTED, "agents must be 1..%d", kMaxAgents);
  if (dim < 1 || dim > kMaxAgentDim) return fail(MRMG_ERR_UNSUPPORTED, "agent dimension must be 1..%d", kMaxAgentDim);
  if (n_boxes < 0 || n_spheres < 0 || n_boxes > 4096 || n_spheres > 4096) return fail(MRMG_ERR_ARG, "obstacle counts");
  if (q_dim < 1 || q_dim > kMaxAgents * kMaxAgentDim) return fail(MRMG_ERR_UNSUPPORTED, "q_dim out of range");
  for (int i = 0; i < n_agents; i++)
    if (h_agent_offsets[i] < 0 || h_agent_offsets[i] + dim > q_dim) return fail(MRMG_ERR_ARG, "agent slice outside q");
  mrmg_scene* sc = new mrmg_scene();
  sc->kind = 0;
  sc->q_dim = q_dim;
  int rc = init_common(sc);
  if (rc) { mrmg_scene_destroy(sc); return rc; }

  const int A = n_agents;
  std::vector<int> off(A);
  std::vector<float> r32(A), pthr32(A * A), lo32(n_boxes * dim), hi32(n_boxes * dim), sp32(n_spheres * dim),
      sthr32(n_spheres * A);
  double omax = 0.0;
  for (int i = 0; i < A; i++) {
    off[i] = (int)h_agent_offsets[i];
    r32[i] = (float)h_agent_radius[i];
    omax = std::max(omax, std::fabs(h_agent_radius[i]));
  }
  for (int i = 0; i < A * A; i++) { pthr32[i] = (float)h_pair_threshold[i]; omax = std::max(omax, std::fabs(h_pair_threshold[i])); }
  for (int i = 0; i < n_boxes * dim; i++) {
    lo32[i] = (float)h_box_lo[i];
    hi32[i] = (float)h_box_hi[i];
    omax = std::max(omax, std::max(std::fabs(h_box_lo[i]), std::fabs(h_box_hi[i])));
  }
  for (int i = 0; i < n_spheres * dim; i++) { sp32[i] = (float)h_sphere_pos[i]; omax = std::max(omax, std::fabs(h_sphere_pos[i])); }
  for (int i = 0; i < n_spheres * A; i++) { sthr32[i] = (float)h_sphere_threshold[i]; omax = std::max(omax, std::fabs(h_sphere_threshold[i])); }
  if (!(omax < 1e30)) { mrmg_scene_destroy(sc); return fail(MRMG_ERR_ARG, "non-finite or huge scene values"); }

  AbstractDev& d = sc->ab;
  d.A = A; d.dim = dim; d.D = q_dim; d.nb = n_boxes; d.ns = n_spheres;
  d.omax = f32_up(omax * (1.0 + 1e-6) + 1e-30);
  d.delta_k = (float)(8.0 * dim * std::ldexp(1.0, -24));
  DevBlock blk;
  blk.add(off.data(), off.size(), &d.agent_off);
  blk.add(h_pair_threshold, (size_t)A * A, &d.pair_thr);
  blk.add(h_agent_radius_sq, (size_t)A, &d.r2);
  blk.add(h_box_lo, (size_t)n_boxes * dim, &d.box_lo);
  blk.add(h_box_hi, (size_t)n_boxes * dim, &d.box_hi);
  blk.add(h_sphere_pos, (size_t)n_spheres * dim, &d.sph_pos);
  blk.add(h_sphere_threshold, (size_t)n_spheres * A, &d.sph_thr);
  blk.add(r32.data(), r32.size(), &d.r32);
  blk.add(pthr32.data(), pthr32.size(), &d.pair_thr32);
  blk.add(lo32.data(), lo32.size(), &d.box_lo32);
  blk.add(hi32.data(), hi32.size(), &d.box_hi32);
  blk.add(sp32.data(), sp32.size(), &d.sph_pos32);
  blk.add(sthr32.data(), sthr32.size(), &d.sph_thr32);
  // the same FP32 tables in their shared-memory layout, staged by one bulk copy
  std::vector<unsigned char> img;
  const unsigned char* d_img = nullptr;
  {
    size_t lay[8];
    abstract_table_layout(d, lay);
    img.assign(lay[7], 0);
    auto put = [&](int k, const void* src, size_t bytes) { if (bytes) std::memcpy(img.data() + lay[k], src, bytes); };
    put(0, off.data(), sizeof(int) * A);
    put(1, r32.data(), sizeof(float) * r32.size());
    put(2, pthr32.data(), sizeof(float) * pthr32.size());
    put(3, lo32.data(), sizeof(float) * lo32.size());
    put(4, hi32.data(), sizeof(float) * hi32.size());
    put(5, sp32.data(), sizeof(float) * sp32.size());
    put(6, sthr32.data(), sizeof(float) * sthr32.size());
    blk.add(img.data(), img.size(), &d_img);
  }
  cudaError_t e = blk.upload(&sc->d_tables);
  if (e != cudaSuccess) { mrmg_scene_destroy(sc); return cuda_fail(e, "upload abstract scene"); }
  d.img = (img.empty() || img.size() > kStageMaxBytes) ? nullptr : d_img;
  if (abstract_prepare(sc->ab)) { mrmg_scene_destroy(sc); return fail(MRMG_ERR_UNSUPPORTED, "scene too large"); }
  sc->band = d.delta_k * d.omax;
  *out = sc;
  return MRMG_OK;
} catch (...) {
  return host_fail();
}

int mrmg_arm_scene_create(int32_t R, int32_t D, const int32_t* h_q_offset, const int32_t* h_base_kind,
                          const double* h_base_pose, const int32_t* h_n_links, const double* h_dh, int32_t S,
                          const int32_t* h_sphere_robot, const int32_t* h_sphere_link, const double* h_sphere_local,
                          const double* h_sphere_radius, int32_t B, const double* h_box_lo, const double* h_box_hi,
                          double band, mrmg_scene** out) try {
  if (!out) return fail(MRMG_ERR_ARG, "out is NULL");
  *out = nullptr;
  if (R < 1 || R > kMaxRobots) return fail(MRMG_ERR_UNSUPPORTED, "robots must be 1..%d", kMaxRobots);
  if (D < 1 || D > kMaxArmDof) return fail(MRMG_ERR_UNSUPPORTED, "q_dim must be 1..%d", kMaxArmDof);
  if (S < 1 || S > 1024 || B < 0 || B > 1024) return fail(MRMG_ERR_UNSUPPORTED, "sphere / box counts");
  uint32_t prism[3] = {0, 0, 0};
  std::vector<int> used(D, 0);
  for (int r = 0; r < R; r++) {
    if (h_n_links[r] < 0 || h_n_links[r] > kMaxLinks) return fail(MRMG_ERR_UNSUPPORTED, "links per robot 0..%d", kMaxLinks);
    if (h_base_kind[r] != 0 && h_base_kind[r] != 1) return fail(MRMG_ERR_ARG, "base kind must be 0 or 1");
    int dof = h_n_links[r] + (h_base_kind[r] == 1 ? 3 : 0);
    if (h_q_offset[r] < 0 || h_q_offset[r] + dof > D) return fail(MRMG_ERR_ARG, "robot %d joints outside q", r);
    for (int j = 0; j < dof; j++) used[h_q_offset[r] + j]++;
    if (h_base_kind[r] == 1) {
      prism[h_q_offset[r] >> 5] |= 1u << (h_q_offset[r] & 31);
      prism[(h_q_offset[r] + 1) >> 5] |= 1u << ((h_q_offset[r] + 1) & 31);
    }
  }
  for (int j = 0; j < D; j++)
    if (used[j] > 1) return fail(MRMG_ERR_ARG, "joint %d shared by two robots", j);
  for (int i = 0; i < S; i++) {
    int r = h_sphere_robot[i];
    if (r < 0 || r >= R || h_sphere_link[i] < 0 || h_sphere_link[i] > h_n_links[r])
      return fail(MRMG_ERR_ARG, "sphere %d: bad robot/link", i);
    if (!(h_sphere_radius[i] >= 0.0) || !(h_sphere_radius[i] < 1e6)) return fail(MRMG_ERR_ARG, "sphere %d radius", i);
  }

  // pack spheres into groups (robot, link) of SPG slots for the cheapest
  // compiled variant that fits in 32 * groups-per-lane groups
  std::vector<std::vector<int>> by_frame(R * (kMaxLinks + 1));
  for (int i = 0; i < S; i++) by_frame[h_sphere_robot[i] * (kMaxLinks + 1) + h_sphere_link[i]].push_back(i);
  int best_spg = -1, best_cost = 1 << 30, best_G = 0;
  for (int vi = 0; arm_supported_spg(vi) > 0; vi++) {
    int spg = arm_supported_spg(vi), gpl = arm_gpl_for_spg(spg);
    int G = 0;
    for (auto& f : by_frame) G += ((int)f.size() + spg - 1) / spg;
    if (G > 32 * gpl) continue;
    int cost = gpl * spg;
    if (cost < best_cost) { best_cost = cost; best_spg = spg; best_G = G; }
  }
  if (best_spg < 0) return fail(MRMG_ERR_UNSUPPORTED, "too many sphere groups for the compiled variants");
  const int SPG = best_spg, G = best_G;
  std::vector<int> grp;            // robot | link << 8
  std::vector<int> grp_robot;
  std::vector<int> slot_sphere;    // slot -> sphere or -1
  for (int r = 0; r < R; r++)
    for (int k = 0; k <= kMaxLinks; k++) {
      auto& f = by_frame[r * (kMaxLinks + 1) + k];
      for (size_t s0 = 0; s0 < f.size(); s0 += SPG) {
        grp.push_back(r | (k << 8));
        grp_robot.push_back(r);
        for (int v = 0; v < SPG; v++) slot_sphere.push_back(s0 + v < f.size() ? f[s0 + v] : -1);
      }
    }
  // inter-robot group pairs
  std::vector<uint32_t> pairs;
  for (int a = 0; a < G; a++)
    for (int b = a + 1; b < G; b++)
      if (grp_robot[a] != grp_robot[b]) pairs.push_back((uint32_t)a | ((uint32_t)b << 16));

  // FP32 band: bounds |FP32 centre - FP64 centre|: 16 (L+1) 2^-24 times the
  // largest reach (base translation magnitude + link lengths + sphere offsets),
  // plus 4 2^-24 times the largest box coordinate (the box tables' rounding)
  double max_box = 0.0;
  for (int i = 0; i < 3 * B; i++) max_box = std::max(max_box, std::max(std::fabs(h_box_lo[i]), std::fabs(h_box_hi[i])));
  if (!(max_box < 1e6)) return fail(MRMG_ERR_ARG, "box coordinates must be finite and < 1e6");
  const double xy_max = std::max(8.0, 2.0 * max_box);
  double reach_max = 0.0;
  int lmax = 0;
  for (int r = 0; r < R; r++) {
    const double* bp = h_base_pose + r * 12;
    double reach = 0.0;
    if (h_base_kind[r] == 1) reach += xy_max * std::sqrt(2.0) + std::fabs(bp[11]);
    reach += std::sqrt(bp[9] * bp[9] + bp[10] * bp[10] + bp[11] * bp[11]);
    for (int k = 0; k < h_n_links[r]; k++) {
      const double* h = h_dh + (r * kMaxLinks + k) * 4;
      reach += std::fabs(h[0]) + std::fabs(h[1]);
    }
    double loc = 0.0;
    for (int i = 0; i < S; i++)
      if (h_sphere_robot[i] == r) {
        const double* l = h_sphere_local + 3 * i;
        loc = std::max(loc, std::sqrt(l[0] * l[0] + l[1] * l[1] + l[2] * l[2]));
      }
    reach += loc;
    reach_max = std::max(reach_max, reach);
    lmax = std::max(lmax, h_n_links[r] + (h_base_kind[r] == 1 ? 1 : 0));
  }
  double delta = 16.0 * (lmax + 1) * std::ldexp(1.0, -24) * reach_max + 4.0 * std::ldexp(1.0, -24) * max_box;
  if (band > delta) delta = band;
  if (!(delta < 1.0)) return fail(MRMG_ERR_ARG, "kinematic reach too large for the FP32 path");

  mrmg_scene* sc = new mrmg_scene();
  sc->kind = 1;
  sc->q_dim = D;
  int rc = init_common(sc);
  if (rc) { mrmg_scene_destroy(sc); return rc; }
  ArmDev& d = sc->arm;
  d.R = R; d.D = D; d.G = G; d.SPG = SPG; d.B = B; d.NP = (int)pairs.size();
  d.delta = f32_up(delta);
  d.xy_max = (float)xy_max;
  {
    // |centre| <= cmax for every configuration the FP32 path accepts (planar
    // bases are limited to |x|, |y| <= xy_max); the pair filter's FP32 value
    // s_a + s_b - 2 a.b (s = |c|^2 - 2 r^2) and the direct FP32
    // |a - b|^2 - (r_a + r_b)^2 each lie within 24 * 2^-24 * (2 cmax^2 +
    // 4 rmax^2) / 2 of their exact values (a generous multiple of the
    // rounding of their products and sums)
    double rmax = 0.0;
    for (int i = 0; i < S; i++) rmax = std::max(rmax, h_sphere_radius[i]);
    rmax += delta;
    const double cmax = reach_max + rmax;
    d.pair_eps = f32_up(24.0 * std::ldexp(1.0, -24) * (2.0 * cmax * cmax + 4.0 * rmax * rmax));
  }
  for (int r = 0; r < R; r++) { d.q_off[r] = h_q_offset[r]; d.base_kind[r] = h_base_kind[r]; d.nl[r] = h_n_links[r]; }
  d.prismatic[0] = prism[0]; d.prismatic[1] = prism[1]; d.prismatic[2] = prism[2];
  d.robot_mask = R >= 32 ? 0xffffffffu : ((1u << R) - 1u);
  d.box_block = 8; d.box_head = 8; d.cfg_chunk = 4; d.phase_b1 = 3;

  std::vector<float4> base32(R * 3), dh32(R * kMaxLinks);
  for (int r = 0; r < R; r++) {
    const double* bp = h_base_pose + r * 12;
    for (int i = 0; i < 3; i++) base32[r * 3 + i] = make_float4((float)bp[3 * i], (float)bp[3 * i + 1], (float)bp[3 * i + 2], (float)bp[9 + i]);
    for (int k = 0; k < kMaxLinks; k++) {
      const double* h = h_dh + (r * kMaxLinks + k) * 4;
      dh32[r * kMaxLinks + k] = make_float4((float)h[0], (float)h[1], (float)h[2], (float)h[3]);
    }
  }
  // the creation inputs the sphere / box tables (and later per-mode tables) come from
  ArmSrc& a = sc->src;
  a.S = S; a.B = B; a.SPG = SPG; a.G = G; a.delta = delta;
  a.local.assign(h_sphere_local, h_sphere_local + 3 * (size_t)S);
  a.radius.assign(h_sphere_radius, h_sphere_radius + S);
  a.box_lo.assign(h_box_lo, h_box_lo + 3 * (size_t)B);
  a.box_hi.assign(h_box_hi, h_box_hi + 3 * (size_t)B);
  a.slot_sphere = slot_sphere;
  a.grp = grp;
  std::vector<char> all_on(S, 1);
  std::vector<int> all_boxes(B);
  std::iota(all_boxes.begin(), all_boxes.end(), 0);
  ArmTables& t = sc->base;
  sphere_tables(a, all_on, &t);
  box_tables(a, all_boxes, &t);
  pen_tables(a, R, all_on, all_boxes, &t);
  DevBlock blk;
  blk.add(h_base_pose, (size_t)R * 12, &d.base64);
  blk.add(h_dh, (size_t)R * kMaxLinks * 4, &d.dh64);
  blk.add(base32.data(), base32.size(), &d.base32);
  blk.add(dh32.data(), dh32.size(), &d.dh32);
  blk.add(grp.data(), grp.size(), &d.grp);
  blk.add(pairs.data(), pairs.size(), &d.pairs);
  add_tables(blk, &t);
  cudaError_t e = blk.upload(&sc->d_tables);
  if (e != cudaSuccess) { mrmg_scene_destroy(sc); return cuda_fail(e, "upload arm scene"); }
  // the base set's view: the shared tables plus its own
  {
    ArmDev v = d;
    v.sph64 = t.d.sph64; v.box64 = t.d.box64; v.sph32 = t.d.sph32; v.band32 = t.d.band32;
    v.box32 = t.d.box32; v.gbs32 = t.d.gbs32; v.B = t.d.B;
    e = build_arm_image(&sc->imgs, &v);
    if (e != cudaSuccess) { mrmg_scene_destroy(sc); return cuda_fail(e, "arm table image"); }
    t.d = v;
    sc->arm = v;
    sc->pen = t.pd;
  }
  trim_tables(&t);
  sc->band = d.delta;
  sc->occ_ctas_per_sm = arm_prepare(d, 8);
  sc->n_pairs_groups = (int64_t)pairs.size();
  sc->slot_to_sphere = slot_sphere;
  *out = sc;
  return MRMG_OK;
} catch (...) {
  return host_fail();
}

int mrmg_arm_scene_set_modes(mrmg_scene* sc, int32_t n_modes, const int32_t* h_sphere_attach,
                             const int64_t* h_mode_box_off, const int32_t* h_mode_boxes,
                             const int64_t* h_mode_attach_off, const int32_t* h_mode_attach) try {
  if (!sc || sc->kind != 1) return fail(MRMG_ERR_ARG, "arm scene required");
  if (!sc->modes.empty()) return fail(MRMG_ERR_ARG, "the scene's modes are already set");
  if (n_modes < 1 || n_modes > (1 << 16)) return fail(MRMG_ERR_ARG, "modes must be 1..65536");
  if (!h_mode_box_off || !h_mode_attach_off) return fail(MRMG_ERR_ARG, "NULL offsets");
  const ArmSrc& a = sc->src;
  if (h_sphere_attach)
    for (int i = 0; i < a.S; i++)
      if (h_sphere_attach[i] < -1) return fail(MRMG_ERR_ARG, "sphere %d: attachment id must be >= -1", i);
  for (const int64_t* off : {h_mode_box_off, h_mode_attach_off}) {
    if (off[0] != 0) return fail(MRMG_ERR_ARG, "mode offsets must start at 0");
    for (int m = 0; m < n_modes; m++)
      if (off[m + 1] < off[m]) return fail(MRMG_ERR_ARG, "mode offsets must not decrease");
  }
  if ((h_mode_box_off[n_modes] > 0 && !h_mode_boxes) || (h_mode_attach_off[n_modes] > 0 && !h_mode_attach))
    return fail(MRMG_ERR_ARG, "NULL mode lists");
  sc->modes.assign(n_modes, ArmTables());
  DevBlock blk;
  for (int m = 0; m < n_modes; m++) {
    std::vector<int> boxes;
    std::vector<char> seen(a.B, 0);
    for (int64_t j = h_mode_box_off[m]; j < h_mode_box_off[m + 1]; j++) {
      const int b = h_mode_boxes[j];
      if (b < 0 || b >= a.B || seen[b]) { sc->modes.clear(); return fail(MRMG_ERR_ARG, "mode %d: bad or repeated box %d", m, b); }
      seen[b] = 1;
      boxes.push_back(b);
    }
    std::vector<char> on(a.S, 1);
    if (h_sphere_attach)
      for (int i = 0; i < a.S; i++) {
        if (h_sphere_attach[i] < 0) continue;
        on[i] = 0;
        for (int64_t j = h_mode_attach_off[m]; j < h_mode_attach_off[m + 1]; j++)
          if (h_mode_attach[j] == h_sphere_attach[i]) on[i] = 1;
      }
    ArmTables* t = &sc->modes[m];
    sphere_tables(a, on, t);
    box_tables(a, boxes, t);
    pen_tables(a, sc->arm.R, on, boxes, t);
    add_tables(blk, t);
  }
  cudaError_t e = blk.upload(&sc->d_mode_tables);
  if (e != cudaSuccess) { sc->modes.clear(); return cuda_fail(e, "upload mode tables"); }
  for (int m = 0; m < n_modes; m++) {
    ArmTables& t = sc->modes[m];
    ArmDev v = sc->base.d;
    v.sph64 = t.d.sph64; v.box64 = t.d.box64; v.sph32 = t.d.sph32; v.band32 = t.d.band32;
    v.box32 = t.d.box32; v.gbs32 = t.d.gbs32; v.B = t.d.B;
    e = build_arm_image(&sc->imgs, &v);
    if (e != cudaSuccess) throw std::bad_alloc();
    t.d = v;
    trim_tables(&t);
  }
  return MRMG_OK;
} catch (...) {
  // the scene keeps working as created, without modes
  if (sc) {
    sc->modes.clear();
    if (sc->d_mode_tables) cudaFree(sc->d_mode_tables);
    sc->d_mode_tables = nullptr;
  }
  return host_fail();
}

int mrmg_arm_scene_set_joint_offsets(mrmg_scene* sc, const double* h_offsets) try {
  if (!sc || sc->kind != 1) return fail(MRMG_ERR_ARG, "arm scene required");
  const int D = sc->q_dim;
  std::vector<float2> o32(D);
  std::vector<double> o64(D, 0.0);
  bool any = false;
  for (int j = 0; j < D; j++) {
    const double o = h_offsets ? h_offsets[j] : 0.0;
    if (!std::isfinite(o) || std::fabs(o) > 64.0) return fail(MRMG_ERR_ARG, "joint offset %d must be finite, |o| <= 64", j);
    const bool pris = (sc->arm.prismatic[j >> 5] >> (j & 31)) & 1u;
    if (pris && o != 0.0) return fail(MRMG_ERR_ARG, "joint %d is a planar-base translation: no angle offset", j);
    o64[j] = o;
    const float hi = (float)o;
    o32[j] = make_float2(hi, (float)(o - (double)hi));
    any |= o != 0.0;
  }
  void* blk = nullptr;
  if (any) {
    const size_t b32 = (sizeof(float2) * D + 255) & ~(size_t)255;
    cudaError_t e = cudaMalloc(&blk, b32 + sizeof(double) * D);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(joint offsets)");
    e = cudaMemcpy(blk, o32.data(), sizeof(float2) * D, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy((unsigned char*)blk + b32, o64.data(), sizeof(double) * D, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) { cudaFree(blk); return cuda_fail(e, "upload joint offsets"); }
  }
  cudaError_t e = cudaDeviceSynchronize();   // no call in flight reads the old offsets
  if (e != cudaSuccess) { if (blk) cudaFree(blk); return cuda_fail(e, "cudaDeviceSynchronize"); }
  if (sc->d_offsets) cudaFree(sc->d_offsets);
  sc->d_offsets = blk;
  const float2* p32 = any ? (const float2*)blk : nullptr;
  const double* p64 = any ? (const double*)((unsigned char*)blk + ((sizeof(float2) * D + 255) & ~(size_t)255)) : nullptr;
  sc->base.d.off32 = p32; sc->base.d.off64 = p64;
  for (auto& m : sc->modes) { m.d.off32 = p32; m.d.off64 = p64; }
  sc->arm.off32 = p32; sc->arm.off64 = p64;
  return MRMG_OK;
} catch (...) {
  return host_fail();
}

int mrmg_scene_set_mode(mrmg_scene* sc, int32_t mode) {
  if (!sc || sc->kind != 1) return fail(MRMG_ERR_ARG, "arm scene required");
  if (mode < -1 || mode >= (int)sc->modes.size()) return fail(MRMG_ERR_ARG, "mode %d out of range", mode);
  sc->cur_mode = mode;
  sc->arm = sc->tabs().d;
  sc->pen = sc->tabs().pd;
  return MRMG_OK;
}

int mrmg_scene_destroy(mrmg_scene* sc) {
  if (!sc) return MRMG_OK;
  if (sc->d_tables) cudaFree(sc->d_tables);
  if (sc->d_mode_tables) cudaFree(sc->d_mode_tables);
  if (sc->d_offsets) cudaFree(sc->d_offsets);
  for (void* p : sc->imgs) cudaFree(p);
  if (sc->d_ctr) cudaFree(sc->d_ctr);
  if (sc->d_pend) cudaFree(sc->d_pend);
  if (sc->d_surv) cudaFree(sc->d_surv);
  if (sc->d_pen_seg) cudaFree(sc->d_pen_seg);
  if (sc->h_ctr) cudaFreeHost(sc->h_ctr);
  if (sc->own_stream) cudaStreamSynchronize(sc->own_stream);
  if (sc->h_stage) cudaFreeHost(sc->h_stage);
  if (sc->d_stage) cudaFree(sc->d_stage);
  if (sc->d_small_flags) cudaFree(sc->d_small_flags);
  if (sc->own_stream) cudaStreamDestroy(sc->own_stream);
  delete sc;
  return MRMG_OK;
}

int mrmg_scene_set_tuning(mrmg_scene* sc, int32_t box_block, int32_t box_head, int32_t cfg_chunk,
                          int32_t phase_b1) try {
  if (!sc || sc->kind != 1) return fail(MRMG_ERR_ARG, "arm scene required");
  if (box_block < 0 || box_block > kMaxBoxBlock || box_head < 0 || box_head > kMaxBoxHead || cfg_chunk < 0 ||
      cfg_chunk > kMaxCfgChunk || phase_b1 < 0 || phase_b1 > kMaxPhaseB1)
    return fail(MRMG_ERR_ARG, "tuning out of range (box_block <= %d, box_head <= %d, cfg_chunk <= %d, phase_b1 <= %d)",
                kMaxBoxBlock, kMaxBoxHead, kMaxCfgChunk, kMaxPhaseB1);
  ArmDev v = sc->arm;
  v.box_block = box_block ? box_block : 8;
  v.box_head = box_head;
  v.cfg_chunk = cfg_chunk ? cfg_chunk : 4;
  v.phase_b1 = phase_b1 ? phase_b1 : 3;
  if (!arm_tuning_fits(v)) return fail(MRMG_ERR_UNSUPPORTED, "box_block %d needs more shared memory than a CTA has", v.box_block);
  cudaError_t e = cudaDeviceSynchronize();   // no call in flight reads the old shape
  if (e != cudaSuccess) return cuda_fail(e, "cudaDeviceSynchronize");
  auto apply = [&](ArmDev& d) { d.box_block = v.box_block; d.box_head = v.box_head; d.cfg_chunk = v.cfg_chunk; d.phase_b1 = v.phase_b1; };
  apply(sc->base.d);
  for (auto& m : sc->modes) apply(m.d);
  apply(sc->arm);
  sc->occ_ctas_per_sm = arm_prepare(sc->base.d, 8);
  return MRMG_OK;
} catch (...) {
  return host_fail();
}

int mrmg_scene_get_tuning(const mrmg_scene* sc, int32_t* out4) {
  if (!sc || sc->kind != 1 || !out4) return fail(MRMG_ERR_ARG, "arm scene and out4 required");
  out4[0] = sc->arm.box_block; out4[1] = sc->arm.box_head; out4[2] = sc->arm.cfg_chunk; out4[3] = sc->arm.phase_b1;
  return MRMG_OK;
}

int mrmg_host_access(int32_t* out) {
  if (!out) return fail(MRMG_ERR_ARG, "NULL argument");
  int dev = 0, v = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccess, dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaDeviceGetAttribute(pageable memory access)");
  const char* force = std::getenv("MRMG_STAGE_HOST_INPUTS");
  *out = (v && !(force && force[0] == '1')) ? 1 : 0;
  return MRMG_OK;
}

int mrmg_serving_gather(const void* h_table, int32_t max_src, int32_t q_dim, int64_t ccap, int64_t ecap, float* d_q1,
                        float* d_q2, int64_t* d_N, int32_t* d_err, void* stream) {
  if (!h_table || !d_q1 || !d_q2 || !d_N || !d_err) return fail(MRMG_ERR_ARG, "mrmg_serving_gather: NULL argument");
  if (max_src < 0 || max_src > 65534 || q_dim < 1 || ccap < 0 || ecap < 0)
    return fail(MRMG_ERR_ARG, "mrmg_serving_gather: max_src 0..65534, q_dim >= 1, capacities >= 0");
  const cudaError_t e = serving_gather(h_table, max_src, q_dim, ccap, ecap, d_q1, d_q2, (long long*)d_N, d_err,
                                       (cudaStream_t)stream);
  return e == cudaSuccess ? MRMG_OK : cuda_fail(e, "launch serving gather");
}

int mrmg_table_stage_timeouts(uint32_t* out) {
  if (!out) return fail(MRMG_ERR_ARG, "NULL argument");
  *out = arm_stage_timeouts() + abstract_stage_timeouts();
  return MRMG_OK;
}

int mrmg_scene_info(const mrmg_scene* sc, int64_t* out7, double* out_band) {
  if (!sc || !out7) return fail(MRMG_ERR_ARG, "NULL argument");
  LaunchShape ls = shape(const_cast<mrmg_scene*>(sc));
  out7[0] = sc->kind;
  out7[1] = sc->q_dim;
  out7[2] = sc->kind == 1 ? sc->arm.SPG : 0;
  out7[3] = sc->kind == 1 ? sc->arm.G : 0;
  out7[4] = sc->n_pairs_groups;
  out7[5] = ls.ctas;
  out7[6] = ls.warps;
  if (out_band) *out_band = sc->band;
  return MRMG_OK;
}

int mrmg_scene_set_launch(mrmg_scene* sc, int32_t ctas, int32_t warps) {
  if (!sc || ctas < 0 || warps < 0 || warps > 8) return fail(MRMG_ERR_ARG, "launch shape");
  sc->ctas = ctas;
  sc->warps = warps;
  return MRMG_OK;
}

int mrmg_arm_slot_map(const mrmg_scene* sc, int32_t* out, int64_t cap) {
  if (!sc || sc->kind != 1 || !out) return fail(MRMG_ERR_ARG, "arm scene required");
  if (cap < (int64_t)sc->slot_to_sphere.size()) return fail(MRMG_ERR_ARG, "capacity too small");
  for (size_t i = 0; i < sc->slot_to_sphere.size(); i++) out[i] = sc->slot_to_sphere[i];
  return (int)sc->slot_to_sphere.size();
}

int mrmg_arm_scene_tune_order(mrmg_scene* sc, const void* d_q, int32_t dtype, int64_t n, int32_t* h_order_out,
                              void* stream) try {
  if (!sc || sc->kind != 1) return fail(MRMG_ERR_ARG, "arm scene required");
  if (n < 1 || (dtype != MRMG_F32 && dtype != MRMG_F64) || !d_q) return fail(MRMG_ERR_ARG, "samples / dtype");
  const int B = sc->arm.B;
  if (B < 2) return MRMG_OK;
  const int words = (B + 31) / 32;
  cudaStream_t st = (cudaStream_t)stream;
  std::vector<uint32_t> hits((size_t)words * n);   // host first: nothing to free if it throws
  uint32_t* d_hits = nullptr;
  cudaError_t e = cudaMalloc(&d_hits, sizeof(uint32_t) * words * n);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(hits)");
  e = arm_box_hits(sc->arm, d_q, dtype, n, d_hits, words, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(hits.data(), d_hits, sizeof(uint32_t) * words * n, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(d_hits);
  if (e != cudaSuccess) return cuda_fail(e, "box hit calibration");
  // greedy cover: next the box that touches most samples not yet touched by
  // the boxes before it; then the rest by how many samples they touch
  std::vector<char> covered(n, 0), used(B, 0);
  std::vector<int> order;
  auto hit = [&](long long i, int b) { return (hits[i * words + b / 32] >> (b % 32)) & 1u; };
  while ((int)order.size() < B) {
    int best = -1;
    long long best_cnt = -1, best_tot = -1;
    for (int b = 0; b < B; b++) {
      if (used[b]) continue;
      long long cnt = 0, tot = 0;
      for (long long i = 0; i < n; i++) {
        const unsigned h = hit(i, b);
        tot += h;
        cnt += h && !covered[i];
      }
      if (cnt > best_cnt || (cnt == best_cnt && tot > best_tot)) { best = b; best_cnt = cnt; best_tot = tot; }
    }
    used[best] = 1;
    order.push_back(best);
    for (long long i = 0; i < n; i++)
      if (hit(i, best)) covered[i] = 1;
  }
  std::vector<float4> b32(2 * B);
  std::vector<double> b64(6 * (size_t)B);
  for (int k = 0; k < B; k++) {
    b32[2 * k] = sc->tabs().box32_host[2 * order[k]];
    b32[2 * k + 1] = sc->tabs().box32_host[2 * order[k] + 1];
    for (int c = 0; c < 6; c++) b64[6 * (size_t)k + c] = sc->tabs().box64_host[6 * (size_t)order[k] + c];
  }
  e = cudaMemcpy((void*)sc->arm.box32, b32.data(), sizeof(float4) * 2 * B, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy((void*)sc->arm.box64, b64.data(), sizeof(double) * 6 * B, cudaMemcpyHostToDevice);
  // the table image starts with the boxes (arm_table_layout)
  if (e == cudaSuccess && sc->arm.img)
    e = cudaMemcpy((void*)sc->arm.img, b32.data(), sizeof(float4) * 2 * B, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(e, "upload box order");
  sc->tabs().box32_host = b32;
  sc->tabs().box64_host = b64;
  if (h_order_out)
    for (int k = 0; k < B; k++) h_order_out[k] = order[k];
  return MRMG_OK;
} catch (...) {
  return host_fail();
}

int mrmg_is_collision_free_batch(mrmg_scene* sc, const void* d_q, int32_t dtype, int64_t n, uint8_t* d_out,
                                 void* stream, int32_t flags) {
  if (!sc) return fail(MRMG_ERR_ARG, "scene is NULL");
  if (n < 0 || (dtype != MRMG_F32 && dtype != MRMG_F64)) return fail(MRMG_ERR_ARG, "n / dtype");
  if (n > kMaxBatch) return fail(MRMG_ERR_ARG, "batch of %lld exceeds %lld items; split it", (long long)n, kMaxBatch);
  if (n == 0) return MRMG_OK;
  if (!d_q || !d_out) return fail(MRMG_ERR_ARG, "NULL device pointer");
  cudaStream_t st = (cudaStream_t)stream;
  AbstractDev ab = sc->ab;
  ab.sph_batch_form = (flags & MRMG_FLAG_BATCH_FORM) ? 1 : 0;
  int rc = ensure_pending(sc, n, st);   // also reserves the scratch of later captured calls
  if (rc) return rc;
  if (sc->kind == 0 && !(flags & MRMG_FLAG_ASYNC)) {
    // synchronous abstract call: the fused kernel alone (pending
    // configurations are decided inline), no counter round trip
    cudaError_t e = abstract_configs_mapped(ab, d_q, dtype, n, d_out, sc->num_sms, st);
    if (e != cudaSuccess) return cuda_fail(e, "launch configs");
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "kernel execution");
    std::memset(sc->h_ctr, 0, sizeof(int) * kNumCtr);
    return MRMG_OK;
  }
  cudaError_t e = cudaMemsetAsync(sc->d_ctr, 0, sizeof(int) * kNumCtr, st);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync");
  CallScratch cs{sc->d_ctr, sc->d_pend, sc->d_surv, sc->pend_cap};
  LaunchShape ls = shape(sc);
  e = sc->kind == 0 ? abstract_configs(ab, d_q, dtype, n, d_out, cs, ls, st)
                    : arm_configs(sc->arm, d_q, dtype, n, d_out, cs, ls, (flags & MRMG_FLAG_FULL_EVAL) ? 1 : 0, st);
  if (e != cudaSuccess) return cuda_fail(e, "launch configs");
  return finish_call(sc, st, flags);
}

int mrmg_is_collision_free_batch_robots(mrmg_scene* sc, const void* d_q, int32_t dtype, int64_t n,
                                        uint32_t robot_mask, uint8_t* d_out, void* stream, int32_t flags) {
  if (!sc) return fail(MRMG_ERR_ARG, "scene is NULL");
  if (sc->kind != 1) return fail(MRMG_ERR_UNSUPPORTED, "per-robot checks need an arm scene");
  const uint32_t all = sc->arm.R >= 32 ? 0xffffffffu : ((1u << sc->arm.R) - 1u);
  if (!(robot_mask & all) || (robot_mask & ~all)) return fail(MRMG_ERR_ARG, "robot mask must select robots of the scene");
  if (n < 0 || (dtype != MRMG_F32 && dtype != MRMG_F64)) return fail(MRMG_ERR_ARG, "n / dtype");
  if (n > kMaxBatch) return fail(MRMG_ERR_ARG, "batch of %lld exceeds %lld items; split it", (long long)n, kMaxBatch);
  if (n == 0) return MRMG_OK;
  if (!d_q || !d_out) return fail(MRMG_ERR_ARG, "NULL device pointer");
  cudaStream_t st = (cudaStream_t)stream;
  int rc = ensure_pending(sc, n, st);
  if (rc) return rc;
  cudaError_t e = cudaMemsetAsync(sc->d_ctr, 0, sizeof(int) * kNumCtr, st);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync");
  CallScratch cs{sc->d_ctr, sc->d_pend, sc->d_surv, sc->pend_cap};
  ArmDev a = sc->arm;
  a.robot_mask = robot_mask;
  e = arm_configs(a, d_q, dtype, n, d_out, cs, shape(sc), (flags & MRMG_FLAG_FULL_EVAL) ? 1 : 0, st);
  if (e != cudaSuccess) return cuda_fail(e, "launch configs");
  return finish_call(sc, st, flags);
}

int mrmg_is_edge_collision_free_batch(mrmg_scene* sc, const void* d_q1, const void* d_q2, int32_t dtype, int64_t n,
                                      double resolution, int32_t include_endpoints, const int64_t* d_N,
                                      int64_t N_start, int64_t N_max, uint8_t* d_out, void* stream, int32_t flags) {
  if (!sc) return fail(MRMG_ERR_ARG, "scene is NULL");
  if (n < 0 || (dtype != MRMG_F32 && dtype != MRMG_F64)) return fail(MRMG_ERR_ARG, "n / dtype");
  if (!d_N && !(resolution > 0.0)) return fail(MRMG_ERR_ARG, "resolution must be > 0");
  if (N_start < 0) return fail(MRMG_ERR_ARG, "N_start must be >= 0");
  if (n > kMaxBatch) return fail(MRMG_ERR_ARG, "batch of %lld exceeds %lld items; split it", (long long)n, kMaxBatch);
  if (n == 0) return MRMG_OK;
  if (!d_q1 || !d_q2 || !d_out) return fail(MRMG_ERR_ARG, "NULL device pointer");
  cudaStream_t st = (cudaStream_t)stream;
  int rc = ensure_pending(sc, n, st);   // also reserves the scratch of later captured calls
  if (rc) return rc;
  if (sc->kind == 0 && n <= kFlatMaxEdges && !(flags & MRMG_FLAG_ASYNC)) {
    // synchronous abstract call: the flat edge kernel alone, its error bits
    // per CTA in the mapped buffer's head, no counter round trip
    rc = ensure_stage(sc, kStageHead);
    if (rc) return rc;
    int grid = 0;
    cudaError_t e = abstract_edges_mapped(sc->ab, d_q1, d_q2, dtype, n, resolution, include_endpoints,
                                          (const long long*)d_N, N_start, N_max, d_out, sc->m_stage, sc->num_sms, st,
                                          &grid);
    if (e != cudaSuccess) return cuda_fail(e, "launch edges");
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "kernel execution");
    int bits = 0;
    for (int c = 0; c < grid; c++) bits |= sc->h_stage[c];
    std::memset(sc->h_ctr, 0, sizeof(int) * kNumCtr);
    sc->h_ctr[kCtrErr] = bits;
    return bits ? mrmg_status_from_error_bits(bits) : MRMG_OK;
  }
  cudaError_t e = cudaMemsetAsync(sc->d_ctr, 0, sizeof(int) * kNumCtr, st);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync");
  CallScratch cs{sc->d_ctr, sc->d_pend, sc->d_surv, sc->pend_cap};
  LaunchShape ls = shape(sc);
  e = sc->kind == 0
          ? abstract_edges(sc->ab, d_q1, d_q2, dtype, n, resolution, include_endpoints, (const long long*)d_N,
                           N_start, N_max, d_out, cs, ls, st)
          : arm_edges(sc->arm, d_q1, d_q2, dtype, n, resolution, include_endpoints, (const long long*)d_N, N_start,
                      N_max, d_out, cs, ls, (flags & MRMG_FLAG_FULL_EVAL) ? 1 : 0, st);
  if (e != cudaSuccess) return cuda_fail(e, "launch edges");
  return finish_call(sc, st, flags);
}

int mrmg_scene_error_word(mrmg_scene* sc, void** d_err) {
  if (!sc || !d_err) return fail(MRMG_ERR_ARG, "NULL argument");
  *d_err = sc->d_ctr + kCtrErr;
  return MRMG_OK;
}

int mrmg_scene_reserve(mrmg_scene* sc, int64_t n, void* stream) {
  if (!sc || n < 0) return fail(MRMG_ERR_ARG, "scene / n");
  return ensure_pending(sc, n, (cudaStream_t)stream);
}

int mrmg_status_from_error_bits(int32_t bits) {
  if (bits & E_N_START) return fail(MRMG_ERR_N_START, "N_start > N for at least one edge");
  if (bits & E_BAD_INPUT)
    return fail(MRMG_ERR_ARG, "bad input: a non-finite or out-of-range edge length (int() of nan/inf), or a gather row "
                "outside its step's capacity");
  if (bits & E_TIMEOUT) return fail(MRMG_ERR_TIMEOUT, "a bounded device wait ran out");
  return MRMG_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Host-pointer calls (the planners' one-at-a-time pattern).
//
// Small arm batches run one kernel launch that reads its inputs straight from
// a mapped pinned staging buffer and writes its hits and statistics back into
// it (zero-copy over the CPU-GPU link), so a call is: inputs written into the
// buffer, one launch, one wait on the scene's own stream.  Everything else is
// staged: the inputs cross to the device in one copy, the batched kernels run,
// and the verdicts and counters come back in one copy each.
// ---------------------------------------------------------------------------
namespace {

constexpr long long kSmallEdges = 256;      // edges per call on the single-launch path
constexpr long long kSmallItems = 1 << 16;  // (edge, position) items on that path
constexpr long long kSmallConfigs = 4096;   // configurations per call on that path
constexpr size_t kStageStats = kStageHead;

size_t pad16(size_t x) { return (x + 15) & ~(size_t)15; }

int ensure_stage(mrmg_scene* sc, size_t bytes) {
  if (!sc->own_stream) {
    cudaError_t e = cudaStreamCreateWithFlags(&sc->own_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamCreate");
  }
  if (!sc->d_small_flags) {
    cudaError_t e = cudaMalloc(&sc->d_small_flags, sizeof(unsigned) * kSmallConfigs);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(edge flags)");
    e = cudaMemset(sc->d_small_flags, 0, sizeof(unsigned) * kSmallConfigs);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemset(edge flags)");
  }
  if (bytes <= sc->stage_cap) return MRMG_OK;
  const size_t cap = std::max(bytes, std::max((size_t)65536, 2 * sc->stage_cap));
  cudaError_t e = cudaStreamSynchronize(sc->own_stream);
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
  if (sc->h_stage) cudaFreeHost(sc->h_stage);
  if (sc->d_stage) cudaFree(sc->d_stage);
  sc->h_stage = nullptr;
  sc->m_stage = nullptr;
  sc->d_stage = nullptr;
  sc->stage_cap = 0;
  e = cudaHostAlloc((void**)&sc->h_stage, cap, cudaHostAllocMapped);
  if (e != cudaSuccess) return cuda_fail(e, "cudaHostAlloc(staging)");
  e = cudaHostGetDevicePointer((void**)&sc->m_stage, sc->h_stage, 0);
  if (e == cudaSuccess) e = cudaMalloc(&sc->d_stage, cap);
  if (e != cudaSuccess) {
    cudaFreeHost(sc->h_stage);
    sc->h_stage = nullptr;
    sc->m_stage = nullptr;
    return cuda_fail(e, "staging buffers");
  }
  sc->stage_cap = cap;
  return MRMG_OK;
}

// the next call's flag epoch (flags of earlier calls never match it); the
// flags are cleared when the 32-bit epoch wraps
int next_epoch(mrmg_scene* sc, unsigned* ep) {
  if (++sc->small_epoch == 0) {
    cudaError_t e = cudaMemsetAsync(sc->d_small_flags, 0, sizeof(unsigned) * kSmallConfigs, sc->own_stream);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(edge flags)");
    sc->small_epoch = 1;
  }
  *ep = sc->small_epoch;
  return MRMG_OK;
}

// N of one edge as the reference computes it (abstract_env.py:321-323):
// max(2, int(max_k |q1_k - q2_k| / resolution) + 1); false when int() would
// raise (NaN in the first coordinate, an infinite or huge quotient)
bool host_edge_N(const void* q1, const void* q2, int dtype, long long e, int D, double res, long long* N) {
  double m = 0.0;
  bool nan0 = false;
  for (int k = 0; k < D; k++) {
    const double a = dtype == MRMG_F32 ? (double)((const float*)q1)[e * D + k] : ((const double*)q1)[e * D + k];
    const double b = dtype == MRMG_F32 ? (double)((const float*)q2)[e * D + k] : ((const double*)q2)[e * D + k];
    const double v = std::fabs(a - b);
    if (k == 0) {
      m = v;
      nan0 = v != v;
    } else if (v > m) {
      m = v;
    }
  }
  const double t = m / res;
  if (nan0 || !(t < 9.0e15)) return false;
  *N = std::max(2ll, (long long)t + 1);
  return true;
}

// launch the single-launch kernel on the mapped buffer, wait, and fill the
// scene's statistics from the per-CTA slots
int run_small(mrmg_scene* sc, const ArmDev& a, SmallBatch& b) {
  int grid = 0;
  cudaError_t e = arm_small(a, b, sc->num_sms, sc->own_stream, &grid);
  if (e != cudaSuccess) return cuda_fail(e, "launch small batch");
  e = cudaStreamSynchronize(sc->own_stream);
  if (e != cudaSuccess) return cuda_fail(e, "kernel execution");
  const int* st = (const int*)sc->h_stage;
  long long cfg = 0, pend = 0;
  for (int c = 0; c < grid; c++) {
    cfg += st[2 * c];
    pend += st[2 * c + 1];
  }
  std::memset(sc->h_ctr, 0, sizeof(int) * kNumCtr);
  sc->h_ctr[kCtrPending] = (int)pend;
  std::memcpy(sc->h_ctr + kCtrStat0, &cfg, sizeof(cfg));
  return MRMG_OK;
}

}  // namespace

extern "C" {

int mrmg_is_collision_free_host(mrmg_scene* sc, const void* h_q, int32_t dtype, int64_t n, uint32_t robot_mask,
                                uint8_t* h_out, int32_t flags) try {
  if (!sc) return fail(MRMG_ERR_ARG, "scene is NULL");
  if (n < 0 || (dtype != MRMG_F32 && dtype != MRMG_F64)) return fail(MRMG_ERR_ARG, "n / dtype");
  if (n > kMaxBatch) return fail(MRMG_ERR_ARG, "batch of %lld exceeds %lld items; split it", (long long)n, kMaxBatch);
  if (robot_mask && sc->kind != 1) return fail(MRMG_ERR_UNSUPPORTED, "per-robot checks need an arm scene");
  if (sc->kind == 1) {
    const uint32_t all = sc->arm.R >= 32 ? 0xffffffffu : ((1u << sc->arm.R) - 1u);
    if (robot_mask & ~all) return fail(MRMG_ERR_ARG, "robot mask must select robots of the scene");
  }
  if (n == 0) return MRMG_OK;
  if (!h_q || !h_out) return fail(MRMG_ERR_ARG, "NULL host pointer");
  const size_t es = dtype == MRMG_F32 ? 4 : 8;
  const size_t qbytes = (size_t)n * sc->q_dim * es;
  const size_t o_hit = kStageStats, o_q = o_hit + pad16((size_t)n), total = o_q + pad16(qbytes);
  int rc = ensure_stage(sc, total);
  if (rc) return rc;
  unsigned char* H = sc->h_stage;
  ArmDev a = sc->arm;
  if (robot_mask) a.robot_mask = robot_mask;
  std::memset(H + o_hit, 0, (size_t)n);
  // the inputs as the kernels read them: the caller's array itself where the
  // device reads pageable host memory, else a copy in the mapped buffer
  const void* in_q = h_q;
  if (!sc->pageable) {
    std::memcpy(H + o_q, h_q, qbytes);
    in_q = sc->m_stage + o_q;
  }
  if (sc->kind == 0 && n <= kSmallConfigs) {
    // one launch, verdicts written straight into the mapped buffer
    AbstractDev ab = sc->ab;
    ab.sph_batch_form = (flags & MRMG_FLAG_BATCH_FORM) ? 1 : 0;
    cudaError_t e = abstract_configs_mapped(ab, in_q, dtype, n, sc->m_stage + o_hit, sc->num_sms,
                                            sc->own_stream);
    if (e != cudaSuccess) return cuda_fail(e, "launch configs");
    e = cudaStreamSynchronize(sc->own_stream);
    if (e != cudaSuccess) return cuda_fail(e, "kernel execution");
    std::memcpy(h_out, H + o_hit, (size_t)n);
    return MRMG_OK;
  }
  if (sc->kind == 1 && n <= kSmallConfigs && !(flags & MRMG_FLAG_FULL_EVAL) && arm_small_ok(a)) {
    SmallBatch b{};
    b.n = (int)n; b.items = (int)n; b.edges = 0; b.dtype = dtype; b.incl = 0; b.N_start = 0;
    b.q1 = in_q; b.hit = sc->m_stage + o_hit; b.stats = (int*)sc->m_stage;
    b.flags = sc->d_small_flags;
    rc = next_epoch(sc, &b.epoch);
    if (rc) return rc;
    rc = run_small(sc, a, b);
    if (rc) return rc;
    for (long long i = 0; i < n; i++) h_out[i] = H[o_hit + i] ? 0 : 1;
    return MRMG_OK;
  }
  cudaStream_t st = sc->own_stream;
  unsigned char* Dv = sc->d_stage;
  // the kernels read the caller's array in place where the device reads
  // pageable host memory, else one copy of the mapped buffer's input
  const void* k_q = h_q;
  cudaError_t e = cudaSuccess;
  if (!sc->pageable) {
    e = cudaMemcpyAsync(Dv + o_q, H + o_q, qbytes, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(inputs)");
    k_q = Dv + o_q;
  }
  rc = ensure_pending(sc, n, st);
  if (rc) return rc;
  e = cudaMemsetAsync(sc->d_ctr, 0, sizeof(int) * kNumCtr, st);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync");
  CallScratch cs{sc->d_ctr, sc->d_pend, sc->d_surv, sc->pend_cap};
  LaunchShape ls = shape(sc);
  if (sc->kind == 0) {
    AbstractDev ab = sc->ab;
    ab.sph_batch_form = (flags & MRMG_FLAG_BATCH_FORM) ? 1 : 0;
    e = abstract_configs(ab, k_q, dtype, n, Dv + o_hit, cs, ls, st);
  } else {
    e = arm_configs(a, k_q, dtype, n, Dv + o_hit, cs, ls, (flags & MRMG_FLAG_FULL_EVAL) ? 1 : 0, st);
  }
  if (e != cudaSuccess) return cuda_fail(e, "launch configs");
  e = cudaMemcpyAsync(H + o_hit, Dv + o_hit, (size_t)n, cudaMemcpyDeviceToHost, st);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(verdicts)");
  rc = finish_call(sc, st, 0);
  std::memcpy(h_out, H + o_hit, (size_t)n);
  return rc;
} catch (...) {
  return host_fail();
}

int mrmg_is_edge_collision_free_host(mrmg_scene* sc, const void* h_q1, const void* h_q2, int32_t dtype, int64_t n,
                                     double resolution, int32_t include_endpoints, const int64_t* h_N,
                                     int64_t N_start, int64_t N_max, uint8_t* h_out, int32_t flags) try {
  if (!sc) return fail(MRMG_ERR_ARG, "scene is NULL");
  if (n < 0 || (dtype != MRMG_F32 && dtype != MRMG_F64)) return fail(MRMG_ERR_ARG, "n / dtype");
  if (!h_N && !(resolution > 0.0)) return fail(MRMG_ERR_ARG, "resolution must be > 0");
  if (N_start < 0) return fail(MRMG_ERR_ARG, "N_start must be >= 0");
  if (n > kMaxBatch) return fail(MRMG_ERR_ARG, "batch of %lld exceeds %lld items; split it", (long long)n, kMaxBatch);
  if (n == 0) return MRMG_OK;
  if (!h_q1 || !h_q2 || !h_out) return fail(MRMG_ERR_ARG, "NULL host pointer");
  const int D = sc->q_dim;
  const size_t es = dtype == MRMG_F32 ? 4 : 8;
  const size_t qbytes = (size_t)n * D * es;
  const size_t o_hit = kStageStats, o_off = o_hit + pad16((size_t)n), o_N32 = o_off + pad16(4 * ((size_t)n + 1)),
               o_N64 = o_N32 + pad16(4 * (size_t)n), o_q1 = o_N64 + pad16(8 * (size_t)n),
               o_q2 = o_q1 + pad16(qbytes), total = o_q2 + pad16(qbytes);
  int rc = ensure_stage(sc, total);
  if (rc) return rc;
  unsigned char* H = sc->h_stage;
  std::memset(H + o_hit, 0, (size_t)n);
  const void* in_q1 = h_q1;
  const void* in_q2 = h_q2;
  const long long* in_N = (const long long*)h_N;
  if (!sc->pageable) {   // copies in the mapped buffer (see the configurations above)
    std::memcpy(H + o_q1, h_q1, qbytes);
    std::memcpy(H + o_q2, h_q2, qbytes);
    if (h_N) std::memcpy(H + o_N64, h_N, 8 * (size_t)n);
    in_q1 = sc->m_stage + o_q1;
    in_q2 = sc->m_stage + o_q2;
    in_N = h_N ? (const long long*)(sc->m_stage + o_N64) : nullptr;
  }
  // the single-launch path: arm scenes, few edges, every N known and valid
  bool small = sc->kind == 1 && n <= kSmallEdges && !(flags & MRMG_FLAG_FULL_EVAL) && arm_small_ok(sc->arm);
  long long items = 0;
  if (small) {
    int* off = (int*)(H + o_off);
    int* N32 = (int*)(H + o_N32);
    for (long long e = 0; e < n && small; e++) {
      long long N = 0;
      if (h_N) {
        N = h_N[e];
        small = N >= 2;
      } else {
        small = host_edge_N(h_q1, h_q2, dtype, e, D, resolution, &N);
      }
      small = small && N_start <= N && N <= (1ll << 24);
      const long long nmax = (N_max < 0 || N_max > N) ? N : N_max;
      off[e] = (int)items;
      N32[e] = (int)N;
      if (nmax > N_start) items += nmax - N_start;
      small = small && items <= kSmallItems;
    }
    off[n] = (int)items;
  }
  if (sc->kind == 0 && n <= kFlatMaxEdges) {
    // abstract scenes: the flat edge kernel on the mapped buffer; its error
    // bits come back per CTA in the head of the buffer
    int grid = 0;
    cudaError_t e = abstract_edges_mapped(sc->ab, in_q1, in_q2, dtype, n, resolution, include_endpoints, in_N,
                                          N_start, N_max, sc->m_stage + o_hit, sc->m_stage, sc->num_sms,
                                          sc->own_stream, &grid);
    if (e != cudaSuccess) return cuda_fail(e, "launch edges");
    e = cudaStreamSynchronize(sc->own_stream);
    if (e != cudaSuccess) return cuda_fail(e, "kernel execution");
    int bits = 0;
    for (int c = 0; c < grid; c++) bits |= H[c];
    std::memset(sc->h_ctr, 0, sizeof(int) * kNumCtr);
    sc->h_ctr[kCtrErr] = bits;
    std::memcpy(h_out, H + o_hit, (size_t)n);
    return bits ? mrmg_status_from_error_bits(bits) : MRMG_OK;
  }
  if (small) {
    SmallBatch b{};
    b.n = (int)n; b.items = (int)items; b.edges = 1; b.dtype = dtype; b.incl = include_endpoints ? 1 : 0;
    b.N_start = N_start;
    b.off = (const int*)(sc->m_stage + o_off); b.N = (const int*)(sc->m_stage + o_N32);
    b.q1 = in_q1; b.q2 = in_q2; b.hit = sc->m_stage + o_hit;
    b.stats = (int*)sc->m_stage;
    b.flags = sc->d_small_flags;
    rc = next_epoch(sc, &b.epoch);
    if (rc) return rc;
    rc = run_small(sc, sc->arm, b);
    if (rc) return rc;
    for (long long i = 0; i < n; i++) h_out[i] = H[o_hit + i] ? 0 : 1;
    return MRMG_OK;
  }
  cudaStream_t st = sc->own_stream;
  unsigned char* Dv = sc->d_stage;
  cudaError_t e = cudaSuccess;
  // the kernels' inputs: where the device reads pageable host memory, the
  // caller's arrays themselves (no staging copy); else one copy of the
  // mapped buffer's inputs
  const void* k_q1 = h_q1;
  const void* k_q2 = h_q2;
  const long long* dN = (const long long*)h_N;
  if (!sc->pageable) {
    e = cudaMemcpyAsync(Dv + o_N64, H + o_N64, total - o_N64, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(inputs)");
    k_q1 = Dv + o_q1;
    k_q2 = Dv + o_q2;
    dN = h_N ? (const long long*)(Dv + o_N64) : nullptr;
  }
  rc = ensure_pending(sc, n, st);
  if (rc) return rc;
  e = cudaMemsetAsync(sc->d_ctr, 0, sizeof(int) * kNumCtr, st);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync");
  CallScratch cs{sc->d_ctr, sc->d_pend, sc->d_surv, sc->pend_cap};
  LaunchShape ls = shape(sc);
  e = sc->kind == 0
          ? abstract_edges(sc->ab, k_q1, k_q2, dtype, n, resolution, include_endpoints, dN, N_start, N_max,
                           Dv + o_hit, cs, ls, st)
          : arm_edges(sc->arm, k_q1, k_q2, dtype, n, resolution, include_endpoints, dN, N_start, N_max,
                      Dv + o_hit, cs, ls, (flags & MRMG_FLAG_FULL_EVAL) ? 1 : 0, st);
  if (e != cudaSuccess) return cuda_fail(e, "launch edges");
  e = cudaMemcpyAsync(H + o_hit, Dv + o_hit, (size_t)n, cudaMemcpyDeviceToHost, st);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(verdicts)");
  rc = finish_call(sc, st, 0);
  std::memcpy(h_out, H + o_hit, (size_t)n);
  return rc;
} catch (...) {
  return host_fail();
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Edge checks without allocation.
//
// Some callers cannot call cudaMalloc at the moment they check edges: a
// planner step being recorded into a CUDA graph (allocation is not a
// capturable operation), a real-time control loop that forbids allocation
// after start-up, or a process whose memory pool already owns the device.
// The regular entry point grows the scene's scratch with cudaMalloc when a
// larger batch arrives; this one takes its scratch from the fixed device
// array below instead, so a call never allocates or frees.
//
// The array is sized for MRMG_NOALLOC_MAX_EDGES edges: 256 bytes of
// counters, 8 bytes per edge for the FP64 pending list and 32 bytes per edge
// for the survivor list (16,384 edges -> 640 KiB + 256 B).  Every GPU that
// loads the library holds it until the process exits.  All calls share it
// and it keeps the last call's contents; each call clears its counters
// before use.  Calls that overlap on the GPU (other streams, threads or
// scenes) race on it and must be serialised by the caller.  A call also
// writes the scene's counter words and their pinned host mirror (the error
// word and the statistics), as the regular entry point does: two calls on one
// scene that overlap on the GPU race there too, whichever entry points they
// use.
// ---------------------------------------------------------------------------
namespace {

constexpr size_t kNoAllocCtrBytes = 256;
constexpr size_t kNoAllocPendBytes = sizeof(long long) * MRMG_NOALLOC_MAX_EDGES;
constexpr size_t kNoAllocSurvBytes = sizeof(SurvivorEdge) * MRMG_NOALLOC_MAX_EDGES;
static_assert(sizeof(int) * kNumCtr <= kNoAllocCtrBytes, "counters fit");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocCtrBytes + kNoAllocPendBytes + kNoAllocSurvBytes];

// Host code only has a stand-in for g_noalloc_scratch; its device address is
// looked up with that device current and cached per device, together with
// the id of the CUDA context it belongs to.  A new context on the device
// (after cudaDeviceReset, for instance) reloads the module at another
// address, so a changed context id triggers a fresh lookup.  The context id
// comes from the driver (cuCtxGetCurrent / cuCtxGetId, resolved through the
// runtime's entry-point query, so the library does not link libcuda).
struct NoAllocSlot {
  unsigned long long ctx;   // 0: unknown
  void* addr;
};
std::mutex g_noalloc_mu;
NoAllocSlot g_noalloc_slot[256] = {};

using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

// id of the calling thread's current context; false when unavailable
bool current_context_id(unsigned long long* id) {
  static CtxGetCurrentFn get_cur = nullptr;
  static CtxGetIdFn get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_cur = (CtxGetCurrentFn)f;
    f = nullptr;
    q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = (CtxGetIdFn)f;
  });
  if (!get_cur || !get_id) return false;
  CUcontext c = nullptr;
  if (get_cur(&c) != CUDA_SUCCESS || !c) return false;
  return get_id(c, id) == CUDA_SUCCESS && *id != 0;
}

int noalloc_scratch(unsigned char** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev < 0 || dev >= 256) return fail(MRMG_ERR_UNSUPPORTED, "device index %d", dev);
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  NoAllocSlot& slot = g_noalloc_slot[dev];
  unsigned long long ctx = 0;
  if (slot.addr && slot.ctx && current_context_id(&ctx) && ctx == slot.ctx) {
    *out = (unsigned char*)slot.addr;
    return MRMG_OK;
  }
  void* p = nullptr;
  e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(no-allocation scratch)");
  if (!current_context_id(&ctx)) ctx = 0;   // unknown context: look the address up on every call
  slot.ctx = ctx;
  slot.addr = p;
  *out = (unsigned char*)p;
  return MRMG_OK;
}

}  // namespace

extern "C" {

int mrmg_is_edge_collision_free_batch_noalloc(mrmg_scene* sc, const void* d_q1, const void* d_q2, int32_t dtype,
                                              int64_t n, double resolution, int32_t include_endpoints,
                                              const int64_t* d_N, int64_t N_start, int64_t N_max, uint8_t* d_out,
                                              void* stream, int32_t flags) {
  if (!sc) return fail(MRMG_ERR_ARG, "scene is NULL");
  if (n < 0 || (dtype != MRMG_F32 && dtype != MRMG_F64)) return fail(MRMG_ERR_ARG, "n / dtype");
  if (n > MRMG_NOALLOC_MAX_EDGES)
    return fail(MRMG_ERR_ARG, "batch of %lld edges exceeds the no-allocation limit of %d edges per call",
                (long long)n, (int)MRMG_NOALLOC_MAX_EDGES);
  if (!d_N && !(resolution > 0.0)) return fail(MRMG_ERR_ARG, "resolution must be > 0");
  if (N_start < 0) return fail(MRMG_ERR_ARG, "N_start must be >= 0");
  if (n == 0) return MRMG_OK;
  if (!d_q1 || !d_q2 || !d_out) return fail(MRMG_ERR_ARG, "NULL device pointer");
  unsigned char* base = nullptr;
  int rc = noalloc_scratch(&base);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  CallScratch cs{(int*)base, (long long*)(base + kNoAllocCtrBytes),
                 (SurvivorEdge*)(base + kNoAllocCtrBytes + kNoAllocPendBytes), (long long)MRMG_NOALLOC_MAX_EDGES};
  cudaError_t e = cudaMemsetAsync(cs.ctr, 0, sizeof(int) * kNumCtr, st);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync");
  LaunchShape ls = shape(sc);
  e = sc->kind == 0
          ? abstract_edges(sc->ab, d_q1, d_q2, dtype, n, resolution, include_endpoints, (const long long*)d_N,
                           N_start, N_max, d_out, cs, ls, st)
          : arm_edges(sc->arm, d_q1, d_q2, dtype, n, resolution, include_endpoints, (const long long*)d_N, N_start,
                      N_max, d_out, cs, ls, (flags & MRMG_FLAG_FULL_EVAL) ? 1 : 0, st);
  if (e != cudaSuccess) return cuda_fail(e, "launch edges");
  // status: the counters are copied into the scene's own counter words (so the
  // word of mrmg_scene_error_word and mrmg_last_call_stats describe this call,
  // also when it was recorded into a graph), then to their pinned mirror
  e = cudaMemcpyAsync(sc->d_ctr, cs.ctr, sizeof(int) * kNumCtr, cudaMemcpyDeviceToDevice, st);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(counters)");
  e = cudaMemcpyAsync(sc->h_ctr, sc->d_ctr, sizeof(int) * kNumCtr, cudaMemcpyDeviceToHost, st);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(status)");
  if (flags & MRMG_FLAG_ASYNC) return MRMG_OK;
  e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "kernel execution");
  return mrmg_status_from_error_bits(sc->h_ctr[kCtrErr]);
}

int mrmg_last_call_stats(const mrmg_scene* sc, int64_t* out4) {
  if (!sc || !out4) return fail(MRMG_ERR_ARG, "NULL argument");
  out4[0] = sc->h_ctr[kCtrPending];
  out4[1] = sc->h_ctr[kCtrErr];
  long long cfg;
  std::memcpy(&cfg, sc->h_ctr + kCtrStat0, sizeof(cfg));
  out4[2] = cfg;
  out4[3] = 0;
  return MRMG_OK;
}

int mrmg_arm_sphere_centers(mrmg_scene* sc, const void* d_q, int32_t dtype, int64_t n, float* d_c32, double* d_c64,
                            void* stream) {
  if (!sc || sc->kind != 1) return fail(MRMG_ERR_ARG, "arm scene required");
  if (n < 0 || (dtype != MRMG_F32 && dtype != MRMG_F64)) return fail(MRMG_ERR_ARG, "n / dtype");
  if (n == 0) return MRMG_OK;
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = arm_centers(sc->arm, d_q, dtype, n, d_c32, d_c64, st);
  if (e != cudaSuccess) return cuda_fail(e, "launch centers");
  e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "centers kernel");
  return MRMG_OK;
}

int mrmg_arm_total_penetration(mrmg_scene* sc, const void* d_q, int32_t dtype, int64_t n, double* d_out,
                               void* stream) {
  if (!sc || sc->kind != 1) return fail(MRMG_ERR_ARG, "arm scene required");
  if (n < 0 || (dtype != MRMG_F32 && dtype != MRMG_F64)) return fail(MRMG_ERR_ARG, "n / dtype");
  if (n > kMaxBatch) return fail(MRMG_ERR_ARG, "batch of %lld exceeds %lld items; split it", (long long)n, kMaxBatch);
  if (n == 0) return MRMG_OK;
  if (!d_q || !d_out) return fail(MRMG_ERR_ARG, "NULL device pointer");
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = arm_penetration(sc->arm, d_q, dtype, n, d_out, sc->num_sms, st);
  if (e != cudaSuccess) return cuda_fail(e, "launch total penetration");
  e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "total penetration kernel");
  return MRMG_OK;
}

int mrmg_path_penetration(mrmg_scene* sc, const float* d_paths, int64_t P, int32_t T, const double* h_params,
                          const float* d_grad_cost, double* d_cost, float* d_wp_cost, float* d_grad,
                          int32_t warps_per_cta, void* stream, int32_t flags) {
  if (!sc || sc->kind != 1) return fail(MRMG_ERR_ARG, "arm scene required");
  if (!h_params) return fail(MRMG_ERR_ARG, "params is NULL");
  if (P < 0 || T < 1) return fail(MRMG_ERR_ARG, "need n_paths >= 0 and n_waypoints >= 1");
  if (!d_cost && !d_wp_cost && !d_grad) return fail(MRMG_ERR_ARG, "no output requested");
  if (P > 0 && !d_paths) return fail(MRMG_ERR_ARG, "paths is NULL");
  const double margin = h_params[0], scale = h_params[1], beta = h_params[2], smooth = h_params[3];
  if (!std::isfinite(margin) || !(scale > 0.0) || !std::isfinite(scale) || !(beta > 0.0) || !std::isfinite(beta) ||
      !(smooth >= 0.0) || !std::isfinite(smooth))
    return fail(MRMG_ERR_ARG, "params: finite margin, scale > 0, beta > 0, smooth weight >= 0");
  const long long nseg = (T + 31) / 32;
  if (P * nseg >= (1ll << 31)) return fail(MRMG_ERR_ARG, "too many path segments for one call");
  int warps = warps_per_cta > 0 ? warps_per_cta : 16;
  if (warps < sc->arm.R) warps = sc->arm.R;
  if (warps > 16) return fail(MRMG_ERR_UNSUPPORTED, "warps per CTA must be <= 16 (and >= robots)");
  int smem_max = 0;
  cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, sc->device);
  const size_t smem = pen_smem_bytes(sc->arm, sc->pen, 0, warps, 0, sc->arm.R);
  if (smem > (size_t)smem_max)
    return fail(MRMG_ERR_UNSUPPORTED, "scene too large for the penetration kernel (%zu B shared memory > %d)", smem,
                smem_max);
  // the gradient runs in one launch, or per group of robots when one CTA's
  // shared memory cannot hold every sphere's gradient
  int bounds[kMaxRobots + 1] = {0};
  int n_groups = 1;
  if (d_grad) {
    n_groups = pen_grad_groups(sc->arm, sc->pen, warps, (size_t)smem_max, bounds);
    if (n_groups < 1)
      return fail(MRMG_ERR_UNSUPPORTED, "scene too large for the penetration gradient kernel (one robot's gradient "
                  "needs more than %d B of shared memory)", smem_max);
  }
  if (P == 0) return MRMG_OK;
  cudaStream_t st = (cudaStream_t)stream;
  if (d_cost && P * nseg > sc->pen_seg_cap) {
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(st, &cap);
    if (cap != cudaStreamCaptureStatusNone)
      return fail(MRMG_ERR_ARG, "penetration scratch must be sized by an uncaptured call of at least this size first");
    if (sc->d_pen_seg) cudaFree(sc->d_pen_seg);
    sc->d_pen_seg = nullptr;
    sc->pen_seg_cap = 0;
    cudaError_t e = cudaMalloc(&sc->d_pen_seg, sizeof(double) * P * nseg);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(penetration scratch)");
    sc->pen_seg_cap = P * nseg;
  }
  PenParams pp;
  pp.margin = (float)margin;
  pp.inv_scale = (float)(1.0 / scale);
  pp.beta = (float)beta;
  pp.inv_beta = (float)(1.0 / beta);
  pp.smooth_w = (float)smooth;
  cudaError_t e = pen_launch(sc->arm, sc->pen, pp, d_paths, P, T, d_grad_cost, sc->d_pen_seg, d_cost, d_wp_cost,
                             d_grad, warps, n_groups, bounds, st);
  if (e != cudaSuccess) return cuda_fail(e, "launch penetration cost");
  if (flags & MRMG_FLAG_ASYNC) return MRMG_OK;
  e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "penetration kernel");
  return MRMG_OK;
}

int mrmg_penetration_info(const mrmg_scene* sc, int64_t* out4) {
  if (!sc || sc->kind != 1 || !out4) return fail(MRMG_ERR_ARG, "arm scene and out4 required");
  out4[0] = sc->pen.S;
  out4[1] = sc->pen.B;
  out4[2] = (int64_t)pen_smem_bytes(sc->arm, sc->pen, 0, 16, 0, sc->arm.R);
  out4[3] = (int64_t)pen_smem_bytes(sc->arm, sc->pen, 1, 16, 0, sc->arm.R);
  return MRMG_OK;
}

static int device_sms() {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  }
  return sms;
}

static int make_slices(const int64_t* h_slices, int32_t A, int32_t D, SliceTab* t) {
  if (D < 1 || A < 1 || A > 64 || !h_slices) return fail(MRMG_ERR_ARG, "slices: 1..64 agents, D >= 1");
  t->A = A;
  t->D = D;
  for (int i = 0; i < A; i++) {
    int64_t s = h_slices[2 * i], e = h_slices[2 * i + 1];
    if (s < 0 || e < s || e > D) return fail(MRMG_ERR_ARG, "agent slice %d outside [0, D]", i);
    t->s[i] = (int)s;
    t->e[i] = (int)e;
  }
  t->end_all = t->e[A - 1];
  return MRMG_OK;
}

static int sync_unless_async(cudaStream_t st, int32_t flags, const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, what);
  if (flags & MRMG_FLAG_ASYNC) return MRMG_OK;
  e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, what);
  return MRMG_OK;
}

int mrmg_config_dist_matrix(const double* d_queries, int64_t Q, const double* d_nodes, int64_t M, int32_t D,
                            const int64_t* h_slices, int32_t A, int32_t metric, double* d_out, void* stream,
                            int32_t flags) {
  if (Q < 0 || M < 0 || metric < 0 || metric > 3) return fail(MRMG_ERR_ARG, "Q / M / metric");
  SliceTab t;
  int rc = make_slices(h_slices, A, D, &t);
  if (rc) return rc;
  if (Q == 0 || M == 0) return MRMG_OK;
  if (!d_queries || !d_nodes || !d_out) return fail(MRMG_ERR_ARG, "NULL device pointer");
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = dist_matrix(d_queries, Q, d_nodes, M, t, metric, d_out, device_sms(), st);
  if (e != cudaSuccess) return cuda_fail(e, "launch distance matrix");
  return sync_unless_async(st, flags, "distance matrix");
}

int mrmg_batch_config_cost(const double* d_starts, const double* d_ends, int64_t M, int32_t D, const int64_t* h_slices,
                           int32_t A, int32_t cost_metric, int32_t reduction, double w, int32_t mode, double* d_out,
                           void* stream, int32_t flags) {
  if (M < 0 || mode < 0 || mode > 2) return fail(MRMG_ERR_ARG, "M / mode");
  if (cost_metric != MRMG_COST_EUCLIDEAN && cost_metric != MRMG_COST_MAX) return fail(MRMG_ERR_ARG, "cost metric");
  if (reduction != MRMG_REDUCE_MAX && reduction != MRMG_REDUCE_SUM) return fail(MRMG_ERR_ARG, "reduction");
  SliceTab t;
  int rc = make_slices(h_slices, A, D, &t);
  if (rc) return rc;
  for (int i = 0; i < A; i++)
    if (cost_metric == MRMG_COST_MAX && t.e[i] == t.s[i]) return fail(MRMG_ERR_ARG, "empty agent slice");
  if (M == 0) return MRMG_OK;
  if (!d_starts || (mode != 2 && !d_ends) || !d_out) return fail(MRMG_ERR_ARG, "NULL device pointer");
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = batch_cost(d_starts, d_ends, M, t, cost_metric, reduction, w, mode, d_out, device_sms(), st);
  if (e != cudaSuccess) return cuda_fail(e, "launch cost");
  return sync_unless_async(st, flags, "cost");
}

int mrmg_knn_exact(const double* d_queries, int64_t Q, const int32_t* d_query_mode, const double* d_nodes,
                   const int64_t* d_mode_offsets, int32_t D, const int64_t* h_slices, int32_t A, int32_t metric,
                   int32_t k, int64_t* d_idx, double* d_dist, void* stream, int32_t flags) {
  if (Q < 0 || metric < 0 || metric > 3 || k < 1 || k > 64) return fail(MRMG_ERR_ARG, "Q / metric / k (1..64)");
  SliceTab t;
  int rc = make_slices(h_slices, A, D, &t);
  if (rc) return rc;
  if (Q == 0) return MRMG_OK;
  if (!d_queries || !d_query_mode || !d_nodes || !d_mode_offsets || !d_idx || !d_dist)
    return fail(MRMG_ERR_ARG, "NULL device pointer");
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = knn_exact(d_queries, Q, d_query_mode, nullptr, 0, d_nodes, (const long long*)d_mode_offsets,
                            (const long long*)d_mode_offsets + 1, t, metric, k, (long long*)d_idx, d_dist,
                            device_sms(), st);
  if (e != cudaSuccess) return cuda_fail(e, "launch knn");
  return sync_unless_async(st, flags, "knn");
}

}  // extern "C"

struct mrmg_node_store {
  KnnStore* store = nullptr;         // owned nodes (+ tensor-core tiles)
  KnnScratch* scratch = nullptr;
  NearState* near = nullptr;         // radius queries: scratch and the last result
  bool near_valid = false;
  int D = 0;
  long long last_fallback = 0;
  // device copies of host-resident queries: one for k-NN calls, one for
  // radius calls (kept for mrmg_near_fetch)
  double* qbuf[2] = {nullptr, nullptr};
  long long qcap[2] = {0, 0};
};

// queries in host memory are copied to the store's staging buffer `which`
// (the copy is stream-ordered; pageable sources are staged by the CUDA driver
// before the call returns); device pointers pass through
static cudaError_t stage_queries(mrmg_node_store* s, int which, const double* q, long long Q, const double** out,
                                 cudaStream_t st) {
  cudaPointerAttributes at;
  cudaError_t e = cudaPointerGetAttributes(&at, q);
  if (e != cudaSuccess) {
    cudaGetLastError();
    at.type = cudaMemoryTypeUnregistered;
  }
  if (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) {
    *out = q;
    return cudaSuccess;
  }
  const long long n = Q * (long long)s->D;
  if (s->qcap[which] < n) {
    const long long cap = std::max(n, 2 * s->qcap[which]);
    if (s->qbuf[which]) cudaFree(s->qbuf[which]);
    s->qbuf[which] = nullptr;
    s->qcap[which] = 0;
    e = cudaMalloc(&s->qbuf[which], sizeof(double) * cap);
    if (e != cudaSuccess) return e;
    s->qcap[which] = cap;
  }
  e = cudaMemcpyAsync(s->qbuf[which], q, sizeof(double) * n, cudaMemcpyHostToDevice, st);
  *out = s->qbuf[which];
  return e;
}

extern "C" {

int mrmg_node_store_create(const double* d_nodes, int64_t M, int32_t D, const int64_t* h_mode_offsets,
                           int32_t n_modes, const int64_t* h_slices, int32_t A, int32_t metric,
                           mrmg_node_store** out, void* stream) try {
  if (!out) return fail(MRMG_ERR_ARG, "out is NULL");
  *out = nullptr;
  if (M < 0 || n_modes < 1 || n_modes > MRMG_MAX_STORE_MODES || metric < 0 || metric > 3 || !h_mode_offsets)
    return fail(MRMG_ERR_ARG, "M / modes (1..%d) / metric", (int)MRMG_MAX_STORE_MODES);
  if (h_mode_offsets[0] != 0 || h_mode_offsets[n_modes] != M) return fail(MRMG_ERR_ARG, "mode offsets must span [0, M]");
  for (int m = 0; m < n_modes; m++)
    if (h_mode_offsets[m + 1] < h_mode_offsets[m]) return fail(MRMG_ERR_ARG, "mode offsets must not decrease");
  if (M > 0 && !d_nodes) return fail(MRMG_ERR_ARG, "NULL nodes");
  SliceTab t;
  int rc = make_slices(h_slices, A, D, &t);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  mrmg_node_store* s = new mrmg_node_store();
  cudaError_t e = cudaSuccess;
  try {
    s->D = D;
    s->scratch = knn_scratch_new();
    s->near = near_state_new();
    s->store = knn_store_new();
    e = knn_store_build(s->store, d_nodes, M, (const long long*)h_mode_offsets, n_modes, t, metric, D, st);
  } catch (...) {
    mrmg_node_store_destroy(s);
    throw;
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) { mrmg_node_store_destroy(s); return cuda_fail(e, "node store"); }
  *out = s;
  return MRMG_OK;
} catch (...) {
  return host_fail();
}

int mrmg_node_store_destroy(mrmg_node_store* s) {
  if (!s) return MRMG_OK;
  knn_store_delete(s->store);
  knn_scratch_delete(s->scratch);
  near_state_delete(s->near);
  for (double* b : s->qbuf)
    if (b) cudaFree(b);
  delete s;
  return MRMG_OK;
}

int mrmg_node_store_append(mrmg_node_store* s, int32_t mode, const double* rows, int64_t n, void* stream) try {
  if (!s) return fail(MRMG_ERR_ARG, "store is NULL");
  if (mode < 0 || n < 0) return fail(MRMG_ERR_ARG, "mode / n must be >= 0");
  if (mode >= MRMG_MAX_STORE_MODES) return fail(MRMG_ERR_ARG, "mode %d: a store holds < %d modes", mode,
                                                 (int)MRMG_MAX_STORE_MODES);
  if (n > 0 && !rows) return fail(MRMG_ERR_ARG, "NULL rows");
  if (knn_store_count(s->store, mode) + n > (1ll << 31) - 1) return fail(MRMG_ERR_ARG, "a mode holds < 2^31 nodes");
  cudaStream_t st = (cudaStream_t)stream;
  s->near_valid = false;
  cudaError_t e = knn_store_append(s->store, mode, rows, n, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return e == cudaSuccess ? MRMG_OK : cuda_fail(e, "node store append");
} catch (...) {
  return host_fail();
}

int mrmg_node_store_remove(mrmg_node_store* s, int32_t mode, int64_t idx, void* stream) {
  if (!s) return fail(MRMG_ERR_ARG, "store is NULL");
  if (mode < 0 || mode >= knn_store_modes(s->store)) return fail(MRMG_ERR_ARG, "mode out of range");
  if (idx < 0 || idx >= knn_store_count(s->store, mode)) return fail(MRMG_ERR_ARG, "index out of range");
  cudaStream_t st = (cudaStream_t)stream;
  s->near_valid = false;
  cudaError_t e = knn_store_remove(s->store, mode, idx, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return e == cudaSuccess ? MRMG_OK : cuda_fail(e, "node store remove");
}

int mrmg_node_store_set_path(mrmg_node_store* s, int32_t path) {
  if (!s) return fail(MRMG_ERR_ARG, "store is NULL");
  if (path < 0 || path > 2) return fail(MRMG_ERR_ARG, "path: 0 auto, 1 tensor core, 2 exact");
  knn_store_set_path(s->store, path);
  return MRMG_OK;
}

int mrmg_node_store_info(const mrmg_node_store* s, int32_t mode, int64_t* out3) {
  if (!s || !out3) return fail(MRMG_ERR_ARG, "NULL pointer");
  out3[0] = knn_store_modes(s->store);
  out3[1] = mode >= 0 ? knn_store_count(s->store, mode) : 0;
  out3[2] = knn_store_tc(s->store) ? 1 : 0;
  return MRMG_OK;
}

static int check_query_modes(const mrmg_node_store* s, const int32_t* h_query_mode, long long Q) {
  const int n = knn_store_modes(s->store);
  for (long long q = 0; q < Q; q++)
    if (h_query_mode[q] < 0 || h_query_mode[q] >= n) return fail(MRMG_ERR_ARG, "query %lld: mode out of range", q);
  return MRMG_OK;
}

int mrmg_knn(mrmg_node_store* s, const double* d_queries, int64_t Q, const int32_t* h_query_mode, int32_t k,
             int64_t* d_idx, double* d_dist, int64_t* out_stats2, void* stream) try {
  if (!s) return fail(MRMG_ERR_ARG, "store is NULL");
  if (Q < 0 || k < 1 || k > 64) return fail(MRMG_ERR_ARG, "Q / k (1..64)");
  if (Q == 0) return MRMG_OK;
  if (!d_queries || !h_query_mode || !d_idx || !d_dist) return fail(MRMG_ERR_ARG, "NULL pointer");
  int rc = check_query_modes(s, h_query_mode, Q);
  if (rc) return rc;
  int used_tc = 0, nfb = 0;
  const double* dq = nullptr;
  cudaError_t e = stage_queries(s, 0, d_queries, Q, &dq, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "knn query copy");
  e = knn_store_query(s->store, s->scratch, dq, Q, h_query_mode, k, (long long*)d_idx, d_dist, device_sms(), &used_tc,
                      &nfb, (cudaStream_t)stream);
  if (e == cudaErrorLaunchTimeout) return fail(MRMG_ERR_TIMEOUT, "a bounded tensor-core pipeline wait ran out");
  if (e != cudaSuccess) return cuda_fail(e, "knn");
  s->last_fallback = nfb;
  if (out_stats2) { out_stats2[0] = used_tc; out_stats2[1] = nfb; }
  return MRMG_OK;
} catch (...) {
  return host_fail();
}

int mrmg_near(mrmg_node_store* s, const double* d_queries, int64_t Q, const int32_t* h_query_mode,
              const double* h_radius, double add_eps, int64_t* d_offsets, int64_t* d_idx, double* d_dist, int64_t cap,
              int64_t* out_total, void* stream) try {
  if (!s) return fail(MRMG_ERR_ARG, "store is NULL");
  if (Q < 0 || cap < 0) return fail(MRMG_ERR_ARG, "Q / cap must be >= 0");
  if (!d_offsets || !out_total) return fail(MRMG_ERR_ARG, "NULL offsets / total");
  if (Q > 0 && (!d_queries || !h_query_mode || !h_radius)) return fail(MRMG_ERR_ARG, "NULL pointer");
  if (cap > 0 && !d_idx) return fail(MRMG_ERR_ARG, "NULL index output with cap > 0");
  if (!(add_eps >= 0.0)) return fail(MRMG_ERR_ARG, "add_eps must be >= 0");
  int rc = check_query_modes(s, h_query_mode, Q);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  s->near_valid = false;
  *out_total = 0;
  if (Q == 0) {
    cudaError_t e = cudaMemsetAsync(d_offsets, 0, sizeof(int64_t), st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return e == cudaSuccess ? MRMG_OK : cuda_fail(e, "near");
  }
  long long total = 0;
  const double* dq = nullptr;
  cudaError_t e = stage_queries(s, 1, d_queries, Q, &dq, st);
  if (e != cudaSuccess) return cuda_fail(e, "near query copy");
  e = near_query(s->near, s->store, dq, Q, h_query_mode, h_radius, add_eps, (long long*)d_offsets, (long long*)d_idx,
                 d_dist, cap, device_sms(), &total, st);
  if (e == cudaErrorLaunchTimeout) return fail(MRMG_ERR_TIMEOUT, "a bounded tensor-core pipeline wait ran out");
  if (e != cudaSuccess) return cuda_fail(e, "near");
  s->near_valid = true;
  *out_total = total;
  return MRMG_OK;
} catch (...) {
  return host_fail();
}

int mrmg_near_fetch(mrmg_node_store* s, int64_t* d_idx, double* d_dist, int64_t cap, void* stream) try {
  if (!s) return fail(MRMG_ERR_ARG, "store is NULL");
  if (!s->near_valid) return fail(MRMG_ERR_ARG, "no radius query to fetch");
  if (cap < near_last_total(s->near)) return fail(MRMG_ERR_ARG, "cap %lld < total %lld", (long long)cap,
                                                    near_last_total(s->near));
  if (cap > 0 && !d_idx) return fail(MRMG_ERR_ARG, "NULL index output");
  cudaError_t e = near_fetch(s->near, (long long*)d_idx, d_dist, cap, device_sms(), (cudaStream_t)stream);
  return e == cudaSuccess ? MRMG_OK : cuda_fail(e, "near fetch");
} catch (...) {
  return host_fail();
}

int mrmg_selftest_umma(const void* d_a, const void* d_b, int32_t n, float* d_c, void* stream) {
  if (n < 32 || n > 256 || n % 32) return fail(MRMG_ERR_ARG, "n must be 32..256, a multiple of 32");
  cudaStream_t st = (cudaStream_t)stream;
  int* d_err = nullptr;
  cudaError_t e = cudaMalloc(&d_err, sizeof(int));
  if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc");
  cudaMemsetAsync(d_err, 0, sizeof(int), st);
  e = umma_selftest(d_a, d_b, n, d_c, d_err, st);
  int h_err = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h_err, d_err, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(d_err);
  if (e != cudaSuccess) return cuda_fail(e, "umma self-test");
  return mrmg_status_from_error_bits(h_err);
}

int mrmg_binary_search_indices(int64_t N, int64_t* d_out, int32_t chunked, void* stream) {
  if (N < 0 || (N > 0 && !d_out)) return fail(MRMG_ERR_ARG, "N / out");
  if (N == 0) return MRMG_OK;
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = binary_indices(N, (long long*)d_out, st, chunked);
  if (e != cudaSuccess) return cuda_fail(e, "launch binary indices");
  e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "binary indices kernel");
  return MRMG_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
namespace mrmg {
namespace {
// position-parallel form (bfs_at), the one the edge kernels use to deal
// positions to warps
__global__ void binary_indices_kernel(long long N, long long* out) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < N; p += (long long)gridDim.x * blockDim.x)
    out[p] = bfs_at(N, p);
}

// warp-chunked form (BfsChunker), the one the sequential edge walks use
__global__ void binary_indices_chunked_kernel(long long N, long long* out) {
  const int lane = threadIdx.x & 31;
  BfsChunker ch;
  ch.init(N);
  long long v;
  unsigned m;
  long long pos0;
  while (ch.next(lane, &v, &m, &pos0)) {
    if (v >= 0) out[pos0 + __popc(m & ((1u << lane) - 1u))] = v;
  }
}
}  // namespace
cudaError_t binary_indices(long long N, long long* out, cudaStream_t st, int chunked) {
  if (chunked) binary_indices_chunked_kernel<<<1, 32, 0, st>>>(N, out);
  else binary_indices_kernel<<<(int)std::min<long long>((N + 255) / 256, 1024), 256, 0, st>>>(N, out);
  return cudaGetLastError();
}
}  // namespace mrmg
