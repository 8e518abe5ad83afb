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

#include "mrmg_internal.cuh"

namespace mrmg {

constexpr int kKnnMaxK = 64;
constexpr int kKeep = 16;          // candidates kept per query per node chunk
constexpr int kTileM = 128;        // queries per tile (TMEM lanes)
constexpr int kRowBytes = 128;     // one SW128 row: 64 bf16
constexpr long long kWaitSpins = 1ll << 22;

// ---------------------------------------------------------------------------
// Exact FP64 k-NN: warp per query
// ---------------------------------------------------------------------------
namespace {

template <int KM>
__device__ __forceinline__ void topk_insert(double (&td)[KM], long long (&ti)[KM], int k, double d, long long id) {
  // lists hold (distance, index) ascending; equal distances keep the lower index
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

// lexicographic warp argmin over (d, id); returns the winning lane
__device__ __forceinline__ int warp_argmin(double d, long long id) {
  int lane = threadIdx.x & 31;
  double bd = d;
  long long bi = id;
  int bl = lane;
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    const double od = __shfl_xor_sync(MRMG_FULL, bd, o);
    const long long oi = __shfl_xor_sync(MRMG_FULL, bi, o);
    const int ol = __shfl_xor_sync(MRMG_FULL, bl, o);
    if (od < bd || (od == bd && oi < bi) || (od == bd && oi == bi && ol < bl)) { bd = od; bi = oi; bl = ol; }
  }
  return bl;
}

template <int KM>
__global__ void knn_exact_kernel(const double* __restrict__ qs, long long Q, const int* __restrict__ q_mode,
                                 const long long* __restrict__ q_list, long long n_list,
                                 const double* __restrict__ nodes, const long long* __restrict__ mode_off, SliceTab t,
                                 int metric, int k, long long* __restrict__ out_idx, double* __restrict__ out_dist) {
  const int lane = threadIdx.x & 31;
  const long long warp = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const long long nwarps = (long long)gridDim.x * (blockDim.x >> 5);
  const int D = t.D;
  const long long total = q_list ? n_list : Q;
  for (long long w = warp; w < total; w += nwarps) {
    const long long q = q_list ? q_list[w] : w;
    const int m = q_mode[q];
    const long long s = mode_off[m], e = mode_off[m + 1];
    double td[KM];
    long long ti[KM];
#pragma unroll
    for (int i = 0; i < KM; i++) { td[i] = __longlong_as_double(0x7ff0000000000000ll); ti[i] = -1; }
    const double* qq = qs + q * D;
    for (long long x = s + lane; x < e; x += 32) {
      const double* xx = nodes + x * D;
      auto dfun = [&](int j) { return __dsub_rn(qq[j], xx[j]); };
      topk_insert<KM>(td, ti, k, dist_of(t, metric, dfun), x - s);
    }
    // merge the 32 sorted lane lists
    int head = 0;
    for (int r = 0; r < k; r++) {
      double hd = __longlong_as_double(0x7ff0000000000000ll);
      long long hi = 0x7fffffffffffffffll;
#pragma unroll
      for (int i = 0; i < KM; i++)
        if (i == head && i < k) { hd = td[i]; hi = ti[i]; }
      if (hi < 0) hi = 0x7fffffffffffffffll;
      const int win = warp_argmin(hd, hi);
      const double wd = __shfl_sync(MRMG_FULL, hd, win);
      const long long wi = __shfl_sync(MRMG_FULL, hi, win);
      if (lane == 0) {
        out_idx[q * k + r] = wi == 0x7fffffffffffffffll ? -1 : wi;
        out_dist[q * k + r] = wi == 0x7fffffffffffffffll ? __longlong_as_double(0x7ff0000000000000ll) : wd;
      }
      if (lane == win) head++;
    }
  }
}

}  // namespace

cudaError_t knn_exact(const double* qs, long long Q, const int* q_mode, const long long* q_list, long long n_list,
                      const double* nodes, const long long* mode_off, const SliceTab& t, int metric, int k,
                      long long* out_idx, double* out_dist, int num_sms, cudaStream_t st) {
  const long long total = q_list ? n_list : Q;
  if (total <= 0) return cudaSuccess;
  const int warps = 4;
  const int grid = (int)std::min<long long>((total + warps - 1) / warps, (long long)num_sms * 16);
  if (k <= 16)
    knn_exact_kernel<16><<<grid, warps * 32, 0, st>>>(qs, Q, q_mode, q_list, n_list, nodes, mode_off, t, metric, k,
                                                      out_idx, out_dist);
  else
    knn_exact_kernel<kKnnMaxK><<<grid, warps * 32, 0, st>>>(qs, Q, q_mode, q_list, n_list, nodes, mode_off, t, metric,
                                                            k, out_idx, out_dist);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// tcgen05 / TMA / mbarrier helpers (inline PTX)
// ---------------------------------------------------------------------------
namespace {

__device__ __forceinline__ uint32_t su32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(su32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait: false when the barrier did not complete within the limit
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  for (long long i = 0; i < kWaitSpins; i++) {
    if (mbar_try_wait(bar, parity)) return true;
    if (i > 32) __nanosleep(128);
  }
  return false;
}
// bulk asynchronous copy (TMA, non-tensor) global -> shared, completing on `bar`
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(su32(dst)),
               "l"(src), "r"(bytes), "r"(su32(bar))
               : "memory");
}
__device__ __forceinline__ void fence_barrier_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

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
