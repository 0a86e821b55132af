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

// ---------------------------------------------------------------- adjoint
// d(sample)/d(vertex xy) of one quad by forward mode in FP64: 8 tangents,
// (x, y) of p1, p2, p3, p4.
struct D8 {
  double v, d[8];
};
__device__ __forceinline__ D8 c8(double v) {
  D8 r;
  r.v = v;
#pragma unroll
  for (int i = 0; i < 8; ++i) r.d[i] = 0.0;
  return r;
}
__device__ __forceinline__ D8 var8(double v, int i) {
  D8 r = c8(v);
  r.d[i] = 1.0;
  return r;
}
__device__ __forceinline__ D8 operator+(const D8 &a, const D8 &b) {
  D8 r;
  r.v = a.v + b.v;
#pragma unroll
  for (int i = 0; i < 8; ++i) r.d[i] = a.d[i] + b.d[i];
  return r;
}
__device__ __forceinline__ D8 operator-(const D8 &a, const D8 &b) {
  D8 r;
  r.v = a.v - b.v;
#pragma unroll
  for (int i = 0; i < 8; ++i) r.d[i] = a.d[i] - b.d[i];
  return r;
}
__device__ __forceinline__ D8 operator*(const D8 &a, const D8 &b) {
  D8 r;
  r.v = a.v * b.v;
#pragma unroll
  for (int i = 0; i < 8; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
  return r;
}
__device__ __forceinline__ D8 scale8(const D8 &a, double s) {
  D8 r;
  r.v = a.v * s;
#pragma unroll
  for (int i = 0; i < 8; ++i) r.d[i] = a.d[i] * s;
  return r;
}
__device__ __forceinline__ D8 sqrt8(const D8 &a) {
  D8 r;
  r.v = sqrt(a.v);
  const double f = r.v > 0 ? 0.5 / r.v : 0.0;
#pragma unroll
  for (int i = 0; i < 8; ++i) r.d[i] = a.d[i] * f;
  return r;
}
__device__ __forceinline__ D8 div8(const D8 &a, const D8 &b) {
  D8 r;
  const double ib = 1.0 / b.v;
  r.v = a.v * ib;
#pragma unroll
  for (int i = 0; i < 8; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) * ib;
  return r;
}
struct V8 {
  D8 x, y, z;
};
__device__ __forceinline__ V8 sub8(const V8 &a, const V8 &b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ V8 cross8(const V8 &a, const V8 &b) {
  return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, b.y * a.x - a.y * b.x};
}
__device__ __forceinline__ D8 norm8(const V8 &a) { return sqrt8(a.x * a.x + a.y * a.y + a.z * a.z); }

// One thread per quad: gh[2][numel][numelvert] (double, zeroed) += J^T g.
__global__ void k_height_field_adjoint(const float *__restrict__ hx, const float *__restrict__ hy, int numel,
                                       int numelvert, float unitz, float half_period, int ring_begin, int ring_end,
                                       const float *__restrict__ gs, int64_t n, double *__restrict__ ghx,
                                       double *__restrict__ ghy) {
  const int ncol = ring_end - ring_begin + 1;
  const int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (o >= n) return;
  const int i = (int)(o / ncol), j = ring_begin + (int)(o % ncol);
  const int pj = j < numel - 1 ? j + 1 : 0, zi = i < numelvert - 1 ? i + 1 : i;
  const int64_t v[4] = {(int64_t)j * numelvert + i, (int64_t)pj * numelvert + i, (int64_t)j * numelvert + zi,
                        (int64_t)pj * numelvert + zi};
  const double z = (double)__fsub_rn(__fmul_rn((float)i, unitz), half_period);
  const double zn = (double)__fsub_rn(__fmul_rn((float)(i + 1), unitz), half_period);
  V8 p[4];
  for (int q = 0; q < 4; ++q)
    p[q] = {var8(hx[v[q]], 2 * q), var8(hy[v[q]], 2 * q + 1), c8(q < 2 ? z : zn)};
  const V8 a1 = cross8(sub8(p[1], p[0]), sub8(p[2], p[0]));
  const V8 a2 = cross8(sub8(p[3], p[1]), sub8(p[2], p[1]));
  const V8 sm = {a1.x + a2.x, a1.y + a2.y, a1.z + a2.z};
  const D8 ns = norm8(sm);
  const D8 area = scale8(norm8(a1) + norm8(a2), 0.5);
  const D8 nrm[3] = {div8(sm.x, ns), div8(sm.y, ns), div8(sm.z, ns)};
  const double g[7] = {gs[o], gs[n + o], gs[2 * n + o], gs[3 * n + o], gs[4 * n + o], gs[5 * n + o], gs[6 * n + o]};
  double acc[8];
#pragma unroll
  for (int t = 0; t < 8; ++t) {
    // x = mean of the vertex x (tangent 2q), y = mean of the vertex y (2q+1); z has no xy dependence
    acc[t] = 0.25 * ((t & 1) ? g[1] : g[0]) + g[3] * nrm[0].d[t] + g[4] * nrm[1].d[t] + g[5] * nrm[2].d[t] +
             g[6] * area.d[t];
  }
  for (int q = 0; q < 4; ++q) {
    atomicAdd(ghx + v[q], acc[2 * q]);
    atomicAdd(ghy + v[q], acc[2 * q + 1]);
  }
}

__global__ void k_narrow_f64(const double *__restrict__ in, float *__restrict__ out, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] = (float)in[i];
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

extern "C" po_status po_height_field_adjoint(const float *height, int numel, int numelvert, float period, float unitz,
                                             int ring_begin, int ring_end, const float *grad_samples,
                                             float *grad_height, void *stream) {
  if (!height || !grad_samples || !grad_height) return fail(PO_ERR_INVALID_ARGUMENT, "null pointer");
  if (numel < 2 || numelvert < 1) return fail(PO_ERR_INVALID_ARGUMENT, "numel must be >= 2 and numelvert >= 1");
  if (ring_begin < 0 || ring_end < ring_begin || ring_end >= numel)
    return fail(PO_ERR_INVALID_ARGUMENT, "ring range must satisfy 0 <= begin <= end < numel");
  if ((int64_t)numel * numelvert > (int64_t)1 << 30) return fail(PO_ERR_INVALID_ARGUMENT, "height field too large");
  if (!(unitz > 0) || !std::isfinite(period)) return fail(PO_ERR_INVALID_ARGUMENT, "unitz must be > 0");
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t nv = 2 * (int64_t)numel * numelvert;
  const int64_t n = (int64_t)(ring_end - ring_begin + 1) * numelvert;
  double *acc = nullptr;
  PO_CUDA(cudaMallocAsync((void **)&acc, sizeof(double) * nv, st));
  po_status s = PO_OK;
  cudaError_t e = cudaMemsetAsync(acc, 0, sizeof(double) * nv, st);
  if (e != cudaSuccess) s = cuda_fail(e, "cudaMemsetAsync");
  if (s == PO_OK) {
    k_height_field_adjoint<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(
        height, height + (int64_t)numel * numelvert, numel, numelvert, unitz, period * 0.5f, ring_begin, ring_end,
        grad_samples, n, acc, acc + (int64_t)numel * numelvert);
    count_launch();
    k_narrow_f64<<<(unsigned)((nv + 255) / 256), 256, 0, st>>>(acc, grad_height, nv);
    count_launch();
    e = cudaGetLastError();
    if (e != cudaSuccess) s = cuda_fail(e, "height field adjoint launch");
  }
  cudaFreeAsync(acc, st);
  return s;
}
