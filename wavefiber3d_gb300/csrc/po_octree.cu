// po_octree.cu -- device octree of the PO engine.
//
// Replaces util/tree.h:289-715 (build_octree_kernel, recursive CUDA dynamic
// parallelism, one 256-thread block per node, 8^d blocks even for empty
// nodes) and the host passes of compareMie/sphere.cu:255-328.
//
// The reference splits every node at the float centre of its box, counts
// points per octant with warp ballots and scatters them stably.  The final
// order is therefore the points sorted by their octant path (root digit
// first), ties kept in input order.  Here that order is produced directly:
//   1. k_keys: every point walks its path with the same float box arithmetic
//      (tree.h:116-120, :672-687) and records one 3-bit octant digit per level;
//   2. a stable LSD radix sort of (key, index) with 8-bit digits;
//   3. the active nodes of every level are the distinct key prefixes; they are
//      found by flagging prefix changes and compacting with a device scan,
//      leaves first, then each coarser level from the one below it.
// Octant digit o = 4*(z < cz) + 2*(y < cy) + (x >= cx), which is the order
// of tree.h:379-414.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <vector>

#include "po_common.cuh"
#include "po_internal.h"

namespace wavepo {

namespace {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 8;  // per thread
constexpr int kSortTile = kSortThreads * kSortItems;
constexpr int kScanThreads = 1024;

__global__ void k_keys(const float *__restrict__ x, const float *__restrict__ y, const float *__restrict__ z,
                       int64_t n, float3 bmin, float3 bmax, int depth, uint32_t *__restrict__ keys,
                       int32_t *__restrict__ idx) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  float px = x[i], py = y[i], pz = z[i];
  float mnx = bmin.x, mny = bmin.y, mnz = bmin.z, mxx = bmax.x, mxy = bmax.y, mxz = bmax.z;
  uint32_t key = 0;
  for (int l = 0; l < depth; ++l) {
    float cx = 0.5f * (mnx + mxx), cy = 0.5f * (mny + mxy), cz = 0.5f * (mnz + mxz);
    bool hx = !(px < cx), ly = py < cy, lz = pz < cz;
    uint32_t o = (lz ? 4u : 0u) | (ly ? 2u : 0u) | (hx ? 1u : 0u);
    key = (key << 3) | o;
    if (hx) mnx = cx; else mxx = cx;
    if (ly) mxy = cy; else mny = cy;
    if (lz) mxz = cz; else mnz = cz;
  }
  keys[i] = key;
  idx[i] = (int32_t)i;
}

// ---- stable LSD radix sort (8-bit digits) ----------------------------------
__global__ void k_digit_hist(const uint32_t *__restrict__ keys, int64_t n, int shift, int nblocks,
                             int32_t *__restrict__ hist) {
  __shared__ int32_t h[256];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) h[i] = 0;
  __syncthreads();
  int64_t base = (int64_t)blockIdx.x * kSortTile;
  for (int k = threadIdx.x; k < kSortTile; k += blockDim.x) {
    int64_t i = base + k;
    if (i < n) atomicAdd(&h[(keys[i] >> shift) & 255u], 1);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < 256; d += blockDim.x) hist[(int64_t)d * nblocks + blockIdx.x] = h[d];
}

// Each warp owns 256 consecutive items of the tile (8 rounds of 32); items are
// ranked in (warp, round, lane) order, which is input order: the sort is stable.
__global__ void k_digit_scatter(const uint32_t *__restrict__ kin, const int32_t *__restrict__ vin, int64_t n,
                                int shift, int nblocks, const int32_t *__restrict__ offs,
                                uint32_t *__restrict__ kout, int32_t *__restrict__ vout) {
  __shared__ int32_t wcnt[kSortThreads / 32][256];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int i = threadIdx.x; i < (kSortThreads / 32) * 256; i += blockDim.x) (&wcnt[0][0])[i] = 0;
  __syncthreads();
  const int64_t wbase = (int64_t)blockIdx.x * kSortTile + (int64_t)warp * 32 * kSortItems;
  const unsigned lt = (1u << lane) - 1u;
  // pass 1: per-warp digit counts
  for (int r = 0; r < kSortItems; ++r) {
    int64_t i = wbase + r * 32 + lane;
    bool ok = i < n;
    uint32_t d = ok ? ((kin[i] >> shift) & 255u) : 256u;
    unsigned peers = __match_any_sync(0xffffffffu, d);
    if (ok && (peers & lt) == 0) wcnt[warp][d] += __popc(peers);
    __syncwarp();
  }
  __syncthreads();
  // exclusive scan over warps for every digit, plus the global offset
  for (int d = threadIdx.x; d < 256; d += blockDim.x) {
    int32_t run = offs[(int64_t)d * nblocks + blockIdx.x];
    for (int w = 0; w < kSortThreads / 32; ++w) {
      int32_t c = wcnt[w][d];
      wcnt[w][d] = run;
      run += c;
    }
  }
  __syncthreads();
  // pass 2: ranks and scatter
  for (int r = 0; r < kSortItems; ++r) {
    int64_t i = wbase + r * 32 + lane;
    bool ok = i < n;
    uint32_t k = ok ? kin[i] : 0u;
    uint32_t d = ok ? ((k >> shift) & 255u) : 256u;
    unsigned peers = __match_any_sync(0xffffffffu, d);
    if (ok) {
      int32_t dst = wcnt[warp][d] + __popc(peers & lt);
      kout[dst] = k;
      vout[dst] = vin[i];
    }
    __syncwarp();
    if (ok && (peers & lt) == 0) wcnt[warp][d] += __popc(peers);
    __syncwarp();
  }
}

// ---- device-wide exclusive scan of int32 (three phases) -------------------
__device__ __forceinline__ int32_t block_exclusive_scan(int32_t v, int32_t *sm, int32_t *total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int32_t x = v;
  for (int o = 1; o < 32; o <<= 1) {
    int32_t t = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += t;
  }
  if (lane == 31) sm[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int32_t w = lane < nw ? sm[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      int32_t t = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += t;
    }
    if (lane < nw) sm[lane] = w;
  }
  __syncthreads();
  int32_t pre = (warp > 0 ? sm[warp - 1] : 0) + x - v;
  if (total) *total = sm[nw - 1];
  __syncthreads();
  return pre;
}

// sums of tiles of kScanThreads*4 elements; `count` may live on the device
__global__ void k_scan_reduce(const int32_t *__restrict__ in, const int64_t *count_dev, int64_t count_host,
                              int32_t *__restrict__ sums) {
  __shared__ int32_t sm[32];
  int64_t n = count_dev ? *count_dev : count_host;
  int64_t base = (int64_t)blockIdx.x * kScanThreads * 4;
  int32_t s = 0;
  for (int k = 0; k < 4; ++k) {
    int64_t i = base + (int64_t)k * kScanThreads + threadIdx.x;
    if (i < n) s += in[i];
  }
  int32_t tot;
  block_exclusive_scan(s, sm, &tot);
  if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ void k_scan_sums(int32_t *sums, int nb) {
  __shared__ int32_t sm[32];
  int32_t carry = 0;
  for (int base = 0; base < nb; base += blockDim.x) {
    int i = base + threadIdx.x;
    int32_t v = i < nb ? sums[i] : 0, tot;
    int32_t p = block_exclusive_scan(v, sm, &tot);
    if (i < nb) sums[i] = p + carry;
    carry += tot;
  }
}

__global__ void k_scan_final(const int32_t *__restrict__ in, const int64_t *count_dev, int64_t count_host,
                             const int32_t *__restrict__ sums, int32_t *__restrict__ out) {
  __shared__ int32_t sm[32];
  int64_t n = count_dev ? *count_dev : count_host;
  int64_t base = (int64_t)blockIdx.x * kScanThreads * 4;
  // thread t owns 4 consecutive elements base + 4t .. 4t+3
  int32_t v[4], s = 0;
  for (int k = 0; k < 4; ++k) {
    int64_t i = base + 4 * threadIdx.x + k;
    v[k] = i < n ? in[i] : 0;
    s += v[k];
  }
  int32_t pre = block_exclusive_scan(s, sm, nullptr) + sums[blockIdx.x];
  for (int k = 0; k < 4; ++k) {
    int64_t i = base + 4 * threadIdx.x + k;
    if (i < n) out[i] = pre;
    pre += v[k];
  }
}

po_status exclusive_scan(const int32_t *in, int32_t *out, int64_t cap, const int64_t *count_dev, int32_t *sums,
                         cudaStream_t st) {
  int64_t nb = (cap + kScanThreads * 4 - 1) / (kScanThreads * 4);
  if (nb == 0) return PO_OK;
  k_scan_reduce<<<(unsigned)nb, kScanThreads, 0, st>>>(in, count_dev, cap, sums);
  k_scan_sums<<<1, kScanThreads, 0, st>>>(sums, (int)nb);
  k_scan_final<<<(unsigned)nb, kScanThreads, 0, st>>>(in, count_dev, cap, sums, out);
  count_launch(); count_launch(); count_launch();
  PO_CUDA(cudaGetLastError());
  return PO_OK;
}

// ---- node extraction --------------------------------------------------------
// leaves: flag[i] = 1 where the full key changes
__global__ void k_leaf_flags(const uint32_t *__restrict__ keys, int64_t n, int32_t *__restrict__ flag) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) flag[i] = (i == 0 || keys[i] != keys[i - 1]) ? 1 : 0;
}

__global__ void k_leaf_emit(const uint32_t *__restrict__ keys, int64_t n, const int32_t *__restrict__ flag,
                            const int32_t *__restrict__ pos, int32_t *__restrict__ begin,
                            uint32_t *__restrict__ prefix, int64_t *__restrict__ count) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n && flag[i]) {
    begin[pos[i]] = (int32_t)i;
    prefix[pos[i]] = keys[i];
  }
  if (i == n - 1) {
    int64_t c = (int64_t)pos[i] + flag[i];
    *count = c;
    begin[c] = (int32_t)n;
  }
}

// coarser level from the level below: flag[j] = 1 where prefix>>3 changes
__global__ void k_level_flags(const uint32_t *__restrict__ cpre, const int64_t *__restrict__ ccount,
                              int32_t *__restrict__ flag) {
  int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (j >= *ccount) return;
  flag[j] = (j == 0 || (cpre[j] >> 3) != (cpre[j - 1] >> 3)) ? 1 : 0;
}

__global__ void k_level_emit(const uint32_t *__restrict__ cpre, const int32_t *__restrict__ cbegin,
                             const int64_t *__restrict__ ccount, const int32_t *__restrict__ flag,
                             const int32_t *__restrict__ pos, int32_t *__restrict__ cparent,
                             int32_t *__restrict__ begin, uint32_t *__restrict__ prefix,
                             int32_t *__restrict__ child, int64_t *__restrict__ count, int64_t n) {
  int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  int64_t cc = *ccount;
  if (j >= cc) return;
  int32_t q = pos[j] + flag[j] - 1;  // parent index
  cparent[j] = q;
  child[(int64_t)q * 8 + (cpre[j] & 7u)] = (int32_t)j;
  if (flag[j]) {
    begin[q] = cbegin[j];
    prefix[q] = cpre[j] >> 3;
  }
  if (j == cc - 1) {
    *count = (int64_t)q + 1;
    begin[q + 1] = (int32_t)n;
  }
}

__global__ void k_fill_i32(int32_t *p, int64_t count, int32_t v) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < count) p[i] = v;
}

__global__ void k_root_empty(int32_t *begin, uint32_t *prefix, int64_t *count) {
  begin[0] = 0;
  begin[1] = 0;
  prefix[0] = 0;
  *count = 1;
}

__global__ void k_heap_ranges(const uint32_t *__restrict__ keys, int64_t n, int depth, int level,
                              int64_t level_off, int64_t level_count, int32_t *__restrict__ out) {
  int64_t id = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (id >= level_count) return;
  int sh = 3 * (depth - level);
  uint64_t lo = (uint64_t)id << sh, hi = (uint64_t)(id + 1) << sh;
  auto lower = [&](uint64_t v) {
    int64_t a = 0, b = n;
    while (a < b) {
      int64_t m = (a + b) >> 1;
      if ((uint64_t)keys[m] < v) a = m + 1; else b = m;
    }
    return a;
  };
  out[2 * (level_off + id)] = (int32_t)lower(lo);
  out[2 * (level_off + id) + 1] = (int32_t)lower(hi);
}

__global__ void k_gather7(int64_t n, const int32_t *__restrict__ perm, const float *s0, const float *s1,
                          const float *s2, const float *s3, const float *s4, const float *s5, const float *s6,
                          float *d0, float *d1, float *d2, float *d3, float *d4, float *d5, float *d6) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  int32_t p = perm[i];
  d0[i] = s0[p]; d1[i] = s1[p]; d2[i] = s2[p]; d3[i] = s3[p];
  d4[i] = s4[p]; d5[i] = s5[p]; d6[i] = s6[p];
}

inline size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

struct Carver {
  char *p;
  size_t left;
  bool ok = true;
  template <typename T>
  T *take(int64_t count) {
    size_t b = align256(sizeof(T) * (size_t)(count > 0 ? count : 1));
    if (b > left) { ok = false; return nullptr; }
    T *r = (T *)p;
    p += b;
    left -= b;
    return r;
  }
};

int64_t level_capacity(int64_t n, int l);

int64_t level_capacity(int64_t n, int l) {
  int64_t c = 1;
  for (int i = 0; i < l && c < n; ++i) c *= 8;
  if (c > n) c = n;
  return c < 1 ? 1 : c;
}

}  // namespace

// Layout of the octree workspace; with a null base it only measures.
struct OctreeLayout {
  uint32_t *ka, *kb;
  int32_t *va, *vb, *flag, *pos, *hist, *offs, *sums;
  int64_t *counts;
  OctreeLevel level[PO_MAX_DEPTH + 1];
  size_t bytes;
  bool ok;
};

OctreeLayout carve_octree(void *ws, size_t ws_bytes, int64_t n, int depth) {
  OctreeLayout L;
  Carver cv{(char *)ws, ws ? ws_bytes : (size_t)-1};
  const int64_t nn = n > 0 ? n : 1;
  const int64_t nb = (nn + kSortTile - 1) / kSortTile;
  L.ka = cv.take<uint32_t>(nn);
  L.kb = cv.take<uint32_t>(nn);
  L.va = cv.take<int32_t>(nn);
  L.vb = cv.take<int32_t>(nn);
  L.flag = cv.take<int32_t>(nn);
  L.pos = cv.take<int32_t>(nn);
  L.hist = cv.take<int32_t>(256 * nb);
  L.offs = cv.take<int32_t>(256 * nb);
  // block sums of the device scan: the largest scanned array is max(n, 256 * nb)
  L.sums = cv.take<int32_t>((std::max(nn, 256 * nb) + kScanThreads * 4 - 1) / (kScanThreads * 4) + 1);
  L.counts = cv.take<int64_t>(PO_MAX_DEPTH + 1);
  for (int l = 0; l <= depth; ++l) {
    int64_t c = level_capacity(nn, l);
    L.level[l].begin = cv.take<int32_t>(c + 1);
    L.level[l].parent = cv.take<int32_t>(c);
    L.level[l].prefix = cv.take<uint32_t>(c);
    L.level[l].child = l < depth ? cv.take<int32_t>(c * 8) : nullptr;
    L.level[l].count = 0;
  }
  L.ok = cv.ok;
  L.bytes = (size_t)(cv.p - (char *)ws);
  return L;
}

size_t octree_workspace_bytes(int64_t n, int depth) { return carve_octree(nullptr, 0, n, depth).bytes + 256; }

po_status build_octree(const float *x, const float *y, const float *z, int64_t n, const float box_min[3],
                       const float box_max[3], int depth, void *ws, size_t ws_bytes, OctreeBuffers *out,
                       cudaStream_t st) {
  if (depth < 0 || depth > PO_MAX_DEPTH) return fail(PO_ERR_INVALID_ARGUMENT, "octree depth out of range");
  if (n < 0 || n > INT32_MAX - 1) return fail(PO_ERR_INVALID_ARGUMENT, "point count out of range");
  if (!ws) return fail(PO_ERR_INVALID_ARGUMENT, "null octree workspace");
  OctreeLayout lay = carve_octree(ws, ws_bytes, n, depth);
  if (!lay.ok) return fail(PO_ERR_INVALID_ARGUMENT, "octree workspace too small");
  int64_t nn = n > 0 ? n : 1;
  int64_t nb = (nn + kSortTile - 1) / kSortTile;
  uint32_t *ka = lay.ka, *kb = lay.kb;
  int32_t *va = lay.va, *vb = lay.vb, *flag = lay.flag, *pos = lay.pos, *hist = lay.hist, *offs = lay.offs;
  int32_t *sums = lay.sums;
  int64_t *counts = lay.counts;
  OctreeBuffers t;
  t.depth = depth;
  t.n = n;
  for (int l = 0; l <= depth; ++l) t.level[l] = lay.level[l];

  const int T = 256;
  if (n > 0) {
    float3 bmin = make_float3(box_min[0], box_min[1], box_min[2]);
    float3 bmax = make_float3(box_max[0], box_max[1], box_max[2]);
    k_keys<<<(unsigned)((n + T - 1) / T), T, 0, st>>>(x, y, z, n, bmin, bmax, depth, ka, va);
    count_launch();
    // radix passes over 3*depth key bits
    int bits = 3 * depth;
    for (int shift = 0; shift < bits; shift += 8) {
      k_digit_hist<<<(unsigned)nb, kSortThreads, 0, st>>>(ka, n, shift, (int)nb, hist);
      count_launch();
      PO_TRY(exclusive_scan(hist, offs, 256 * nb, nullptr, sums, st));
      k_digit_scatter<<<(unsigned)nb, kSortThreads, 0, st>>>(ka, va, n, shift, (int)nb, offs, kb, vb);
      count_launch();
      std::swap(ka, kb);
      std::swap(va, vb);
    }
    // leaves
    OctreeLevel &L = t.level[depth];
    k_leaf_flags<<<(unsigned)((n + T - 1) / T), T, 0, st>>>(ka, n, flag);
    count_launch();
    PO_TRY(exclusive_scan(flag, pos, n, nullptr, sums, st));
    k_leaf_emit<<<(unsigned)((n + T - 1) / T), T, 0, st>>>(ka, n, flag, pos, L.begin, L.prefix, counts + depth);
    count_launch();
    for (int l = depth - 1; l >= 0; --l) {
      OctreeLevel &C = t.level[l + 1], &P = t.level[l];
      int64_t ccap = level_capacity(nn, l + 1), pcap = level_capacity(nn, l);
      unsigned g = (unsigned)((ccap + T - 1) / T);
      k_fill_i32<<<(unsigned)((pcap * 8 + T - 1) / T), T, 0, st>>>(P.child, pcap * 8, -1);
      k_level_flags<<<g, T, 0, st>>>(C.prefix, counts + l + 1, flag);
      PO_TRY(exclusive_scan(flag, pos, ccap, counts + l + 1, sums, st));
      k_level_emit<<<g, T, 0, st>>>(C.prefix, C.begin, counts + l + 1, flag, pos, C.parent, P.begin, P.prefix,
                                    P.child, counts + l, n);
      count_launch(); count_launch(); count_launch();
    }
  } else {
    // no points: a single empty root; deeper levels are empty
    k_root_empty<<<1, 1, 0, st>>>(t.level[0].begin, t.level[0].prefix, counts);
    count_launch();
    PO_CUDA(cudaMemsetAsync(counts + 1, 0, sizeof(int64_t) * depth, st));
    if (depth > 0) {
      k_fill_i32<<<1, 8, 0, st>>>(t.level[0].child, 8, -1);
      count_launch();
    }
  }
  PO_CUDA(cudaGetLastError());
  int64_t hc[PO_MAX_DEPTH + 1];
  PO_CUDA(cudaMemcpyAsync(hc, counts, sizeof(int64_t) * (depth + 1), cudaMemcpyDeviceToHost, st));
  PO_CUDA(cudaStreamSynchronize(st));
  for (int l = 0; l <= depth; ++l) t.level[l].count = hc[l];
  t.perm = va;
  t.keys = ka;
  *out = t;
  return PO_OK;
}

po_status octree_heap_ranges(const OctreeBuffers &t, int32_t *heap_range, cudaStream_t st) {
  int64_t off = 0, cnt = 1;
  const int T = 256;
  for (int l = 0; l <= t.depth; ++l) {
    k_heap_ranges<<<(unsigned)((cnt + T - 1) / T), T, 0, st>>>(t.keys, t.n, t.depth, l, off, cnt, heap_range);
    count_launch();
    off += cnt;
    cnt *= 8;
  }
  PO_CUDA(cudaGetLastError());
  return PO_OK;
}

po_status gather_points(int64_t n, const int32_t *perm, const float *const src[7], float *const dst[7],
                        cudaStream_t st) {
  if (n <= 0) return PO_OK;
  const int T = 256;
  k_gather7<<<(unsigned)((n + T - 1) / T), T, 0, st>>>(n, perm, src[0], src[1], src[2], src[3], src[4], src[5],
                                                      src[6], dst[0], dst[1], dst[2], dst[3], dst[4], dst[5], dst[6]);
  count_launch();
  PO_CUDA(cudaGetLastError());
  return PO_OK;
}

}  // namespace wavepo
