// mrmg_serving.cu -- the serving batcher's input gather: the device reads
// every planner instance's request arrays straight from host memory (where
// the device reads pageable host memory coherently, as GB300 does over its
// host link) into the step's device buffers, so a step needs no host-side
// packing pass and no staging copy.
#include <cstdint>

#include "mrmg_internal.cuh"

namespace mrmg {
namespace {

// one source array of the step (table row, 32 bytes)
struct GatherEntry {
  const void* src;      // host address of a C-contiguous array
  long long rows;       // rows of D floats (kinds 0-2) or int64 step counts (kind 3)
  long long dst_row;    // first destination row within its region
  int kind;             // 0 configurations, 1 edge starts, 2 edge ends, 3 edge step counts
  int pad;
};

// table: int64 {n_src, n_configs, n_edges, 0}, then n_src GatherEntry rows.
// Grid: x = chunks, y = one row per source plus a last row that writes the
// step counts of the configurations (3) and of the unused slots (2).
__global__ void serving_gather_kernel(const long long* __restrict__ table, int max_src, int D, long long ccap,
                                      long long ecap, float* __restrict__ q1, float* __restrict__ q2,
                                      long long* __restrict__ N, int* __restrict__ err) {
  const long long n_src = table[0], nc = table[1], ne = table[2];
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long t0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y;
  if (y == (int)gridDim.y - 1) {
    if (nc > ccap || ne > ecap || n_src > max_src || nc < 0 || ne < 0 || n_src < 0) {
      if (t0 == 0) atomicOr(err, E_BAD_INPUT);
      return;
    }
    for (long long i = t0; i < ccap + ecap; i += stride)
      if (i < ccap) N[i] = i < nc ? 3 : 2;
      else if (i >= ccap + ne) N[i] = 2;
    return;
  }
  if (y >= n_src || y >= max_src) return;
  const GatherEntry e = ((const GatherEntry*)(table + 4))[y];
  const long long cap = e.kind == 0 ? ccap : ecap;
  if (e.rows <= 0) return;
  if (e.kind < 0 || e.kind > 3 || e.dst_row < 0 || e.dst_row + e.rows > cap || !e.src) {
    if (t0 == 0) atomicOr(err, E_BAD_INPUT);
    return;
  }
  if (e.kind == 3) {
    const long long* s = (const long long*)e.src;
    long long* d = N + ccap + e.dst_row;
    for (long long i = t0; i < e.rows; i += stride) d[i] = s[i];
    return;
  }
  float* d1 = (e.kind == 2 ? q2 : q1) + (e.kind == 0 ? e.dst_row : ccap + e.dst_row) * D;
  float* d2 = e.kind == 0 ? q2 + e.dst_row * D : nullptr;   // a configuration is the edge q -> q
  const float* s = (const float*)e.src;
  const long long cnt = e.rows * D;
  const bool vec = (((uintptr_t)s | (uintptr_t)d1 | (uintptr_t)(d2 ? d2 : d1)) & 15) == 0;
  long long done = 0;
  if (vec) {
    const long long n4 = cnt >> 2;
    const float4* s4 = (const float4*)s;
    float4* a4 = (float4*)d1;
    float4* b4 = (float4*)d2;
    for (long long i = t0; i < n4; i += stride) {
      const float4 v = s4[i];
      a4[i] = v;
      if (d2) b4[i] = v;
    }
    done = n4 << 2;
  }
  for (long long i = done + t0; i < cnt; i += stride) {
    const float v = s[i];
    d1[i] = v;
    if (d2) d2[i] = v;
  }
}

}  // namespace

cudaError_t serving_gather(const void* table, int max_src, int D, long long ccap, long long ecap, float* q1,
                           float* q2, long long* N, int* err, cudaStream_t st) {
  const dim3 grid(64, (unsigned)max_src + 1);
  serving_gather_kernel<<<grid, 256, 0, st>>>((const long long*)table, max_src, D, ccap, ecap, q1, q2, N, err);
  return cudaGetLastError();
}

}  // namespace mrmg
