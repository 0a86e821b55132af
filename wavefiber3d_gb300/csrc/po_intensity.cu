// po_intensity.cu -- transverse projection and far-field intensity.
//
// Replaces util/fields.h:172-204 (computeintensity):
//   E_perp = E - (E.s) s, H_perp = H - (H.s) s,
//   E' = E_perp - Z0 s x H_perp,  I = |E'|^2.
// The root pattern may be supersampled by integer factors (mt, mp) when the
// first tree level needs a finer grid than the output; the output sample
// (i, k) is then root sample (mt*i, mp*k), which is the same direction.
#include <cuda_runtime.h>

#include "po_common.cuh"
#include "po_internal.h"
#include "po_kernels.h"

namespace wavepo {

template <typename V, typename T>
__device__ __forceinline__ float intensity_at(const V *f, int64_t cstride, int64_t idx, const double s[3], T z0) {
  T sx = (T)s[0], sy = (T)s[1], sz = (T)s[2];
  V E[3], H[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    E[c] = f[c * cstride + idx];
    H[c] = f[(3 + c) * cstride + idx];
  }
  T der = E[0].x * sx + E[1].x * sy + E[2].x * sz, dei = E[0].y * sx + E[1].y * sy + E[2].y * sz;
  T dhr = H[0].x * sx + H[1].x * sy + H[2].x * sz, dhi = H[0].y * sx + H[1].y * sy + H[2].y * sz;
  T ss[3] = {sx, sy, sz};
  T er[3], ei[3], hr[3], hi[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    er[c] = E[c].x - der * ss[c];
    ei[c] = E[c].y - dei * ss[c];
    hr[c] = H[c].x - dhr * ss[c];
    hi[c] = H[c].y - dhi * ss[c];
  }
  // E' = E - Z0 (s x H) written as fields.h:290-292
  T xr = er[0] - (hr[2] * sy - hr[1] * sz) * z0, xi = ei[0] - (hi[2] * sy - hi[1] * sz) * z0;
  T yr = er[1] + (hr[2] * sx - hr[0] * sz) * z0, yi = ei[1] + (hi[2] * sx - hi[0] * sz) * z0;
  T zr = er[2] - (hr[1] * sx - hr[0] * sy) * z0, zi = ei[2] - (hi[1] * sx - hi[0] * sy) * z0;
  return (float)(xr * xr + xi * xi + yr * yr + yi * yi + zr * zr + zi * zi);
}

// Output directions of an n_theta x n_phi grid (grid_direction rounded to float),
// built once per context: dirs[d] = (s_x, s_y, s_z, 0).
__global__ void k_out_dirs(int nth, int nph, float4 *__restrict__ dirs) {
  const int64_t d = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (d >= (int64_t)nth * nph) return;
  double s[3];
  grid_direction((int)(d / nph), (int)(d % nph), nth, nph, s);
  dirs[d] = make_float4((float)s[0], (float)s[1], (float)s[2], 0.f);
}

po_status launch_out_dirs(int nth, int nph, float4 *dirs, cudaStream_t st) {
  const int64_t nd = (int64_t)nth * nph;
  if (nd <= 0) return PO_OK;
  k_out_dirs<<<(unsigned)((nd + 255) / 256), 256, 0, st>>>(nth, nph, dirs);
  count_launch();
  PO_CUDA(cudaGetLastError());
  return PO_OK;
}

__global__ void k_intensity_f32(const float2 *__restrict__ fields, int n_slots, int T, int Phi, int nth, int nph,
                                int mt, int mp, const float4 *__restrict__ dirs, float z0, float *__restrict__ out) {
  int64_t d = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  int slot = blockIdx.y;
  int64_t nd = (int64_t)nth * nph;
  if (d >= nd) return;
  int it = (int)(d / nph), ip = (int)(d % nph);
  double s[3];  // the context's direction table, or (no table) grid_direction itself
  if (dirs) {
    const float4 sv = __ldg(dirs + d);
    s[0] = sv.x, s[1] = sv.y, s[2] = sv.z;
  } else {
    grid_direction(it, ip, nth, nph, s);
  }
  int64_t cstride = (int64_t)T * Phi;
  const float2 *f = fields + (int64_t)slot * 6 * cstride;
  int64_t idx = (int64_t)(it * mt) * Phi + (int64_t)ip * mp;
  out[(int64_t)slot * nd + d] = intensity_at<float2, float>(f, cstride, idx, s, z0);
}

__global__ void k_intensity_f64(const double2 *__restrict__ fields, int n_slots, int nth, int nph, double z0,
                                float *__restrict__ out) {
  int64_t d = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  int slot = blockIdx.y;
  int64_t nd = (int64_t)nth * nph;
  if (d >= nd) return;
  double s[3];
  grid_direction((int)(d / nph), (int)(d % nph), nth, nph, s);
  const double2 *f = fields + (int64_t)slot * 6 * nd;
  out[(int64_t)slot * nd + d] = intensity_at<double2, double>(f, nd, d, s, z0);
}

po_status launch_intensity_f32(const float2 *fields, int n_slots, int T, int Phi, int nth, int nph, int mt, int mp,
                               const float4 *dirs, float *out, cudaStream_t st) {
  int64_t nd = (int64_t)nth * nph;
  if (nd <= 0 || n_slots <= 0) return PO_OK;
  dim3 grid((unsigned)((nd + 255) / 256), (unsigned)n_slots);
  k_intensity_f32<<<grid, 256, 0, st>>>(fields, n_slots, T, Phi, nth, nph, mt, mp, dirs, (float)z0_host(), out);
  count_launch();
  PO_CUDA(cudaGetLastError());
  return PO_OK;
}

po_status launch_intensity_f64(const double2 *fields, int n_slots, int nth, int nph, float *out, cudaStream_t st) {
  int64_t nd = (int64_t)nth * nph;
  if (nd <= 0 || n_slots <= 0) return PO_OK;
  dim3 grid((unsigned)((nd + 255) / 256), (unsigned)n_slots);
  k_intensity_f64<<<grid, 256, 0, st>>>(fields, n_slots, nth, nph, z0_host(), out);
  count_launch();
  PO_CUDA(cudaGetLastError());
  return PO_OK;
}

// util/fields.h:206-234 (average_cpu): box average of a fine pattern onto a
// coarse grid, phi first, then theta, with the reference's integer ratios
// r = n_in / n_out (integer division, so only the first r*n_out samples of each
// axis take part) and its float evaluation order:
//   row(i', j) = sum_k in[i'][j*rp + k] / rp,  out(i, j) = sum_k row(i*rt + k, j) / rt.
__global__ void k_average(const float *__restrict__ in, int nth_in, int nph_in, float *__restrict__ out, int nth_out,
                          int nph_out, int rt, int rp) {
  int64_t d = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  int64_t nd = (int64_t)nth_out * nph_out;
  if (d >= nd) return;
  const float *src = in + (int64_t)blockIdx.y * nth_in * nph_in;
  int i = (int)(d / nph_out), j = (int)(d % nph_out);
  float acc = 0.f;
  for (int kt = 0; kt < rt; ++kt) {
    const float *row = src + (int64_t)(i * rt + kt) * nph_in + (int64_t)j * rp;
    float s = 0.f;
    for (int kp = 0; kp < rp; ++kp) s = __fadd_rn(s, __fdiv_rn(row[kp], (float)rp));
    acc = __fadd_rn(acc, __fdiv_rn(s, (float)rt));
  }
  out[(int64_t)blockIdx.y * nd + d] = acc;
}

}  // namespace wavepo

using namespace wavepo;

extern "C" po_status po_average_pattern(const float *in, int nth_in, int nph_in, float *out, int nth_out,
                                        int nph_out, int n_patterns, void *stream) {
  if (!in || !out) return fail(PO_ERR_INVALID_ARGUMENT, "null pointer");
  if (nth_out <= 0 || nph_out <= 0 || n_patterns < 0 || n_patterns > 65535)
    return fail(PO_ERR_INVALID_ARGUMENT, "output grid must be positive and n_patterns in [0, 65535]");
  if (nth_in < nth_out || nph_in < nph_out)
    return fail(PO_ERR_INVALID_ARGUMENT, "the input grid must be at least as fine as the output grid");
  if (n_patterns == 0) return PO_OK;
  const int rt = nth_in / nth_out, rp = nph_in / nph_out;
  const int64_t nd = (int64_t)nth_out * nph_out;
  dim3 grid((unsigned)((nd + 255) / 256), (unsigned)n_patterns);
  k_average<<<grid, 256, 0, (cudaStream_t)stream>>>(in, nth_in, nph_in, out, nth_out, nph_out, rt, rp);
  count_launch();
  PO_CUDA(cudaGetLastError());
  return PO_OK;
}
