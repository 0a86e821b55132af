// po_geometry.cu -- fiber height field -> surface samples (one per quad).
//
// Replaces util/geometry.h:3-75 (full ring) and util/geometry.h:76-179 (ring
// segment [startindex, endindex], the variant fibersim/treePO.cu:132 calls).
// The height field is float32 [2][numel][numelvert]: plane 0 holds x, plane 1
// holds y of vertex (j, i) at j*numelvert + i (j around the ring, i along the
// axis), z_i = i*unitz - period/2.  Quad (i, j) has the vertices
//   p1 = (j, i), p2 = (j+1 mod numel, i), p3 = (j, i'), p4 = (j+1 mod numel, i')
// with i' = i+1, except on the last axial row where i' = i but p3/p4 still take
// z_{i+1} (geometry.h:100-103,135-150).  The sample is the vertex average, the
// area 0.5(|(p2-p1)x(p3-p1)| + |(p4-p2)x(p3-p2)|), the normal the normalised
// sum of both cross products; output index i*(end-start+1) + (j-start).
//
// Every float operation is written with an explicit rounding intrinsic in the
// reference's evaluation order (products and sums rounded separately, no
// fused multiply-add), so the samples equal the reference's host code bit for
// bit.  A vertex at the origin (x == y == 0) is an error in the reference
// (geometry.h:110-114, exit(1)); here it raises a device flag and the call
// returns PO_ERR_INVALID_ARGUMENT.
//
// Layout: the height field is axial-contiguous (i fastest) and the samples are
// ring-contiguous (j fastest), so each CTA stages a 33 x 33 vertex tile in
// shared memory (coalesced along i), then writes its 32 x 32 samples coalesced
// along j.
#include <cuda_runtime.h>

#include "po_internal.h"
#include "po_kernels.h"

namespace wavepo {

namespace {

constexpr int kTile = 32;
constexpr int kRows = 8;  // threadIdx.y extent

struct V3 {
  float x, y, z;
};

__device__ __forceinline__ V3 sub3(V3 a, V3 b) { return {__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z)}; }
__device__ __forceinline__ V3 add3(V3 a, V3 b) { return {__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z)}; }
// util/util.h:339-345 component order
__device__ __forceinline__ V3 cross3(V3 a, V3 b) {
  return {__fsub_rn(__fmul_rn(a.y, b.z), __fmul_rn(b.y, a.z)), __fsub_rn(__fmul_rn(a.z, b.x), __fmul_rn(b.z, a.x)),
          __fsub_rn(__fmul_rn(b.y, a.x), __fmul_rn(a.y, b.x))};
}
__device__ __forceinline__ float norm3(V3 a) {
  return __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(a.x, a.x), __fmul_rn(a.y, a.y)), __fmul_rn(a.z, a.z)));
}

__global__ void __launch_bounds__(kTile * kRows) k_height_field(const float *__restrict__ hx, const float *__restrict__ hy,
                                                              int numel, int numelvert, float unitz, float half_period,
                                                              int ring_begin, int ring_end, float *__restrict__ px,
                                                              float *__restrict__ py, float *__restrict__ pz,
                                                              float *__restrict__ nx, float *__restrict__ ny,
                                                              float *__restrict__ nz, float *__restrict__ area,
                                                              int *__restrict__ err) {
  __shared__ float sx[kTile + 1][kTile + 1];
  __shared__ float sy[kTile + 1][kTile + 1];
  const int j0 = ring_begin + blockIdx.x * kTile;  // first ring column of the tile
  const int i0 = blockIdx.y * kTile;               // first axial row of the tile
  const int jlast = ring_end + 1;                  // last column any quad of this call reads
  // stage vertices (column j0+jj, row i0+ii), coalesced along ii
  for (int jj = threadIdx.y; jj <= kTile; jj += kRows) {
    int j = j0 + jj;
    if (j > jlast) break;
    int col = j < numel ? j : 0;
    for (int ii = threadIdx.x; ii <= kTile; ii += kTile) {
      int i = i0 + ii;
      if (i >= numelvert) continue;
      int64_t v = (int64_t)col * numelvert + i;
      sx[jj][ii] = hx[v];
      sy[jj][ii] = hy[v];
    }
  }
  __syncthreads();
  const int ncol = ring_end - ring_begin + 1;
  const int jj = threadIdx.x;
  const int j = j0 + jj;
  if (j > ring_end) return;
  int bad = 0;
  for (int ii = threadIdx.y; ii < kTile; ii += kRows) {
    int i = i0 + ii;
    if (i >= numelvert) break;
    int in = i < numelvert - 1 ? ii + 1 : ii;
    float z = __fsub_rn(__fmul_rn((float)i, unitz), half_period);
    float zn = __fsub_rn(__fmul_rn((float)(i + 1), unitz), half_period);
    V3 p1 = {sx[jj][ii], sy[jj][ii], z};
    V3 p2 = {sx[jj + 1][ii], sy[jj + 1][ii], z};
    V3 p3 = {sx[jj][in], sy[jj][in], zn};
    V3 p4 = {sx[jj + 1][in], sy[jj + 1][in], zn};
    bad |= (p1.x == 0.f && p1.y == 0.f) | (p2.x == 0.f && p2.y == 0.f) | (p3.x == 0.f && p3.y == 0.f) |
           (p4.x == 0.f && p4.y == 0.f);
    V3 a1 = cross3(sub3(p2, p1), sub3(p3, p1));
    V3 a2 = cross3(sub3(p4, p2), sub3(p3, p2));
    float n1 = norm3(a1), n2 = norm3(a2);
    V3 s = add3(a1, a2);
    float ns = norm3(s);
    int64_t o = (int64_t)i * ncol + (j - ring_begin);
    px[o] = __fmul_rn(__fadd_rn(__fadd_rn(__fadd_rn(p1.x, p2.x), p3.x), p4.x), 0.25f);
    py[o] = __fmul_rn(__fadd_rn(__fadd_rn(__fadd_rn(p1.y, p2.y), p3.y), p4.y), 0.25f);
    pz[o] = __fmul_rn(__fadd_rn(__fadd_rn(__fadd_rn(p1.z, p2.z), p3.z), p4.z), 0.25f);
    area[o] = __fmul_rn(__fadd_rn(n1, n2), 0.5f);
    nx[o] = __fdiv_rn(s.x, ns);
    ny[o] = __fdiv_rn(s.y, ns);
    nz[o] = __fdiv_rn(s.z, ns);
  }
  if (bad) atomicOr(err, 1);
}

}  // namespace

po_status launch_height_field(const float *height, int numel, int numelvert, float period, float unitz, int ring_begin,
                              int ring_end, float *const out[7], int *err, cudaStream_t st) {
  const int ncol = ring_end - ring_begin + 1;
  dim3 grid((unsigned)((ncol + kTile - 1) / kTile), (unsigned)((numelvert + kTile - 1) / kTile));
  k_height_field<<<grid, dim3(kTile, kRows), 0, st>>>(height, height + (int64_t)numel * numelvert, numel, numelvert,
                                                     unitz, period * 0.5f, ring_begin, ring_end, out[0], out[1],
                                                     out[2], out[3], out[4], out[5], out[6], err);
  count_launch();
  PO_CUDA(cudaGetLastError());
  return PO_OK;
}

}  // namespace wavepo

using namespace wavepo;

extern "C" po_status po_height_field_points(const float *height, int numel, int numelvert, float period, float unitz,
                                            int ring_begin, int ring_end, float *x, float *y, float *z, float *nx,
                                            float *ny, float *nz, float *area, void *stream) {
  if (!height || !x || !y || !z || !nx || !ny || !nz || !area) return fail(PO_ERR_INVALID_ARGUMENT, "null pointer");
  if (numel < 2 || numelvert < 1) return fail(PO_ERR_INVALID_ARGUMENT, "numel must be >= 2 and numelvert >= 1");
  if (ring_begin < 0 || ring_end < ring_begin || ring_end >= numel)
    return fail(PO_ERR_INVALID_ARGUMENT, "ring range must satisfy 0 <= begin <= end < numel");
  if ((int64_t)numel * numelvert > (int64_t)1 << 30) return fail(PO_ERR_INVALID_ARGUMENT, "height field too large");
  if (!(unitz > 0) || !std::isfinite(period)) return fail(PO_ERR_INVALID_ARGUMENT, "unitz must be > 0");
  cudaStream_t st = (cudaStream_t)stream;
  int *err = nullptr;
  PO_CUDA(cudaMallocAsync((void **)&err, sizeof(int), st));
  cudaError_t e = cudaMemsetAsync(err, 0, sizeof(int), st);
  float *out[7] = {x, y, z, nx, ny, nz, area};
  po_status s = e == cudaSuccess ? launch_height_field(height, numel, numelvert, period, unitz, ring_begin, ring_end,
                                                       out, err, st)
                                 : cuda_fail(e, "cudaMemsetAsync");
  int h_err = 0;
  if (s == PO_OK) {
    e = cudaMemcpyAsync(&h_err, err, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) s = cuda_fail(e, "height field status read");
  }
  cudaFreeAsync(err, st);
  if (s == PO_OK && h_err) return fail(PO_ERR_INVALID_ARGUMENT, "height field has a vertex at the origin (x == y == 0)");
  return s;
}
