// po_adjoint.cu -- gradient of far-field intensity with respect to the surface
// samples (positions, normals, areas).
//
// The forward map of the engine is F = T(C(x, n, a)): tangent-plane currents
// C per point (util/tangentplane.h:19-80), leaf or depth-0 far-field sums
// F(s) = sum_p exp(i k s.(x_p - c)) C_p (util/fields.h:2-50), then the linear
// tree aggregation T, and the intensity I = |E - Z0 s x H|^2 of the
// transverse projection (util/fields.h:172-204).  For a scalar loss with
// dL/dI given on the output grid, dL = 2 Re sum G^H dF with
//   G(s) = dL/dI(s) [E'; Z0 s x E'],   E' = P(s) F(s)            (root adjoint)
// at the root; the aggregation passes its exact transpose down to the leaves
// (po_interp_mma.cu); at a leaf (or the whole cloud at depth 0)
//   A_p   = sum_s G(s) exp(-i k s.(x_p - c)),
//   A_p^a = sum_s s_a G(s) exp(-i k s.(x_p - c))   (a = x, y, z)
// and
//   dL/dx_p,a += -2 k Im(A_p^a^H C_p)          (phase of the far-field sum)
//   dL/dq     += 2 Re(A_p^H dC_p/dq)            (q in x, y, z, n, area)
// The Jacobian dC_p/dq of the tangent-plane model is taken in forward mode
// (dual numbers with 7 tangents) per point and pattern, in the precision of
// the back-projection (FP32, or FP64 for the FP64 chain).  Only the root
// fields of the forward pass are kept; nothing of the intermediate levels is
// stored, because the transposed aggregation is linear.
#include <cuda_runtime.h>

#include "po_common.cuh"
#include "po_dual.cuh"
#include "po_internal.h"
#include "po_kernels.h"

namespace wavepo {

// Per-point Jacobians: forward-mode duals (po_dual.cuh), all 7 tangents.

// ------------------------------------------------------------ root adjoint
// G at the sampled root points (output sample (i, k) = root (mt*i, mp*k));
// every other root sample gets 0.  fields/G: [slot][6][T][Phi].
template <typename V, typename R>
__global__ void k_intensity_adjoint(const V *__restrict__ fields, const float *__restrict__ dl_di, int T, int Phi,
                                    int nth, int nph, int mt, int mp, const float4 *__restrict__ dirs, R z0,
                                    V *__restrict__ G) {
  const int64_t cstride = (int64_t)T * Phi;
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int slot = blockIdx.y;
  if (e >= cstride) return;
  const int it = (int)(e / Phi), ip = (int)(e % Phi);
  const V *f = fields + (int64_t)slot * 6 * cstride;
  V *g = G + (int64_t)slot * 6 * cstride;
  const bool sampled = (it % mt == 0) && (ip % mp == 0) && it / mt < nth && ip / mp < nph;
  if (!sampled) {
#pragma unroll
    for (int c = 0; c < 6; ++c) g[c * cstride + e] = V{0, 0};
    return;
  }
  const int i = it / mt, k = ip / mp;
  // FP32 chain: the context's output-direction table (grid_direction rounded to
  // float); FP64 chain (dirs == nullptr): the directions in FP64
  double sd[3];
  if (dirs) {
    const float4 sv = __ldg(dirs + (int64_t)i * nph + k);
    sd[0] = sv.x, sd[1] = sv.y, sd[2] = sv.z;
  } else {
    grid_direction(i, k, nth, nph, sd);
  }
  const R s[3] = {(R)sd[0], (R)sd[1], (R)sd[2]};
  V E[3], H[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    E[c] = f[c * cstride + e];
    H[c] = f[(3 + c) * cstride + e];
  }
  // E' = (E - (E.s) s) - Z0 s x (H - (H.s) s) = (E - (E.s) s) - Z0 s x H
  const R der = E[0].x * s[0] + E[1].x * s[1] + E[2].x * s[2];
  const R dei = E[0].y * s[0] + E[1].y * s[1] + E[2].y * s[2];
  R er[3], ei[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    er[c] = E[c].x - der * s[c];
    ei[c] = E[c].y - dei * s[c];
  }
  const R xr[3] = {s[1] * H[2].x - s[2] * H[1].x, s[2] * H[0].x - s[0] * H[2].x, s[0] * H[1].x - s[1] * H[0].x};
  const R xi[3] = {s[1] * H[2].y - s[2] * H[1].y, s[2] * H[0].y - s[0] * H[2].y, s[0] * H[1].y - s[1] * H[0].y};
  R pr[3], pi[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    pr[c] = er[c] - z0 * xr[c];
    pi[c] = ei[c] - z0 * xi[c];
  }
  const R w = (R)dl_di[((int64_t)slot * nth + i) * nph + k];
  // G_E = w E' ; G_H = w Z0 (s x E')
  g[0 * cstride + e] = V{w * pr[0], w * pi[0]};
  g[1 * cstride + e] = V{w * pr[1], w * pi[1]};
  g[2 * cstride + e] = V{w * pr[2], w * pi[2]};
  const R wz = w * z0;
  g[3 * cstride + e] = V{wz * (s[1] * pr[2] - s[2] * pr[1]), wz * (s[1] * pi[2] - s[2] * pi[1])};
  g[4 * cstride + e] = V{wz * (s[2] * pr[0] - s[0] * pr[2]), wz * (s[2] * pi[0] - s[0] * pi[2])};
  g[5 * cstride + e] = V{wz * (s[0] * pr[1] - s[1] * pr[0]), wz * (s[0] * pi[1] - s[1] * pi[0])};
}

po_status launch_intensity_adjoint_f32(const float2 *fields, const float *dl_di, int n_slots, int T, int Phi, int nth,
                                       int nph, int mt, int mp, const float4 *dirs, float2 *G, cudaStream_t st) {
  const int64_t cs = (int64_t)T * Phi;
  if (cs <= 0 || n_slots <= 0) return PO_OK;
  dim3 grid((unsigned)((cs + 255) / 256), (unsigned)n_slots);
  k_intensity_adjoint<float2, float><<<grid, 256, 0, st>>>(fields, dl_di, T, Phi, nth, nph, mt, mp, dirs,
                                                          (float)z0_host(), G);
  count_launch();
  PO_CUDA(cudaGetLastError());
  return PO_OK;
}

po_status launch_intensity_adjoint_f64(const double2 *fields, const float *dl_di, int n_slots, int nth, int nph,
                                       double2 *G, cudaStream_t st) {
  const int64_t cs = (int64_t)nth * nph;
  if (cs <= 0 || n_slots <= 0) return PO_OK;
  dim3 grid((unsigned)((cs + 255) / 256), (unsigned)n_slots);
  k_intensity_adjoint<double2, double><<<grid, 256, 0, st>>>(fields, dl_di, nth, nph, nth, nph, 1, 1, nullptr,
                                                            z0_host(), G);
  count_launch();
  PO_CUDA(cudaGetLastError());
  return PO_OK;
}

// ------------------------------------------------------- point adjoint
// CUDA-core back-projection of the FP64 chain (the FP32 chain runs the
// tensor-core kernel of po_adjoint_mma.cu).
// One warp per (node, 32-point chunk); 4 warps per CTA.  A node's points are
// [begin[node], begin[node+1]); its adjoint pattern is
// G[slot][node * node_stride][6][ndir] about centre[3 * node * center_stride]
// (node_stride = center_stride = 0 lets all chunks of a depth-0 sum share one
// pattern and centre).  Every slot of the launch is accumulated into the
// point's 7 gradients in registers and added to grad[7][n] once.
constexpr int kAdjWarps = 4;
constexpr int kAdjTile = 32;  // directions staged per step

template <typename R>
struct AdjVec;
template <>
struct AdjVec<float> {
  using V = float2;
};
template <>
struct AdjVec<double> {
  using V = double2;
};

__device__ __forceinline__ void phase_exp(float ph, float *sn, float *cs) { sincos_small(ph, sn, cs); }
__device__ __forceinline__ void phase_exp(double ph, double *sn, double *cs) { sincos(ph, sn, cs); }

template <typename R>
__global__ void __launch_bounds__(32 * kAdjWarps) k_point_adjoint(
    const float *__restrict__ x, const float *__restrict__ y, const float *__restrict__ z,
    const float *__restrict__ nx, const float *__restrict__ ny, const float *__restrict__ nz,
    const float *__restrict__ area, const int32_t *__restrict__ begin, int64_t n_nodes,
    const double *__restrict__ center, int center_stride, const typename AdjVec<R>::V *__restrict__ G,
    int64_t node_stride, int64_t slot_stride, const float4 *__restrict__ dirs, const double *__restrict__ dirs_d,
    int ndir, const SlotParams<double> *__restrict__ slots, int n_lambda, int Gc, int64_t n,
    double *__restrict__ grad) {
  using V = typename AdjVec<R>::V;
  __shared__ V s_g[kAdjWarps][6][kAdjTile];
  __shared__ R s_d[kAdjWarps][kAdjTile][3];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t node = (int64_t)blockIdx.x * kAdjWarps + warp;
  if (node >= n_nodes) return;
  const int b = begin[node], e = begin[node + 1];
  const double *ctr = center + 3 * node * center_stride;
  const double cx_ = ctr[0], cy_ = ctr[1], cz_ = ctr[2];
  for (int c0 = b; c0 < e; c0 += 32) {
    const int p = c0 + lane;
    const bool ok = p < e;
    const float px = ok ? x[p] : 0.f, py = ok ? y[p] : 0.f, pz = ok ? z[p] : 0.f;
    double gacc[kNT];
#pragma unroll
    for (int i = 0; i < kNT; ++i) gacc[i] = 0.0;
    for (int lam = 0; lam < n_lambda; ++lam) {
      const double k0 = slots[lam * Gc].k0d;
      const R ux = (R)(k0 * ((double)px - cx_)), uy = (R)(k0 * ((double)py - cy_)), uz = (R)(k0 * ((double)pz - cz_));
      for (int g = 0; g < Gc; ++g) {
        const int slot = lam * Gc + g;
        const V *gp = G + slot * slot_stride + node * node_stride;
        R ar[4][6], ai[4][6];
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int c = 0; c < 6; ++c) ar[a][c] = ai[a][c] = (R)0;
        for (int d0 = 0; d0 < ndir; d0 += kAdjTile) {
          __syncwarp();
          const int d = d0 + lane;
          if (dirs_d) {  // FP64 directions
#pragma unroll
            for (int a = 0; a < 3; ++a) s_d[warp][lane][a] = d < ndir ? (R)dirs_d[3 * (int64_t)d + a] : (R)0;
          } else {
            const float4 f = d < ndir ? dirs[d] : make_float4(0.f, 0.f, 0.f, 0.f);
            s_d[warp][lane][0] = (R)f.x;
            s_d[warp][lane][1] = (R)f.y;
            s_d[warp][lane][2] = (R)f.z;
          }
#pragma unroll
          for (int c = 0; c < 6; ++c) s_g[warp][c][lane] = d < ndir ? gp[(int64_t)c * ndir + d] : V{0, 0};
          __syncwarp();
          const int cnt = ndir - d0 < kAdjTile ? ndir - d0 : kAdjTile;
          for (int q = 0; q < cnt; ++q) {
            const R sx = s_d[warp][q][0], sy = s_d[warp][q][1], sz = s_d[warp][q][2];
            const R ph = -(ux * sx + uy * sy + uz * sz);
            R sn, cs;
            phase_exp(ph, &sn, &cs);
            const R w[4] = {(R)1, sx, sy, sz};
#pragma unroll
            for (int c = 0; c < 6; ++c) {
              const V gv = s_g[warp][c][q];
              const R tr = gv.x * cs - gv.y * sn, ti = gv.x * sn + gv.y * cs;
#pragma unroll
              for (int a = 0; a < 4; ++a) {
                ar[a][c] += w[a] * tr;
                ai[a][c] += w[a] * ti;
              }
            }
          }
        }
        if (!ok) continue;
        const int sel[kNT] = {0, 1, 2, 3, 4, 5, 6};
        CDual<R> C[6];
        tangent_plane_jvp<R, kNT>(slots[slot], px, py, pz, nx[p], ny[p], nz[p], area[p], sel, C);
#pragma unroll
        for (int i = 0; i < kNT; ++i) {
          double s = 0.0;
#pragma unroll
          for (int c = 0; c < 6; ++c) s += (double)ar[0][c] * C[c].re.d[i] + (double)ai[0][c] * C[c].im.d[i];
          gacc[i] += 2.0 * s;
        }
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          double im = 0.0;  // Im(sum_c conj(A^a_c) C_c)
#pragma unroll
          for (int c = 0; c < 6; ++c) im += (double)ar[a + 1][c] * C[c].im.v - (double)ai[a + 1][c] * C[c].re.v;
          gacc[a] += -2.0 * k0 * im;
        }
      }
    }
    if (ok) {
#pragma unroll
      for (int i = 0; i < kNT; ++i) grad[(int64_t)i * n + p] += gacc[i];
    }
  }
}

template <typename R>
static po_status launch_point_adjoint_t(const float *const g[7], const int32_t *begin, int64_t n_nodes,
                                        const double *center, int center_stride, const void *G, int64_t node_stride,
                                        int64_t slot_stride, const float4 *dirs, const double *dirs_d, int ndir,
                                        const SlotParams<double> *slots, int n_lambda, int Gc, int64_t n,
                                        double *grad, cudaStream_t st) {
  if (n_nodes <= 0 || n_lambda <= 0 || Gc <= 0) return PO_OK;
  const int64_t blocks = (n_nodes + kAdjWarps - 1) / kAdjWarps;
  if (blocks > 2147483647LL) return fail(PO_ERR_UNSUPPORTED, "too many nodes for one launch");
  k_point_adjoint<R><<<(unsigned)blocks, 32 * kAdjWarps, 0, st>>>(
      g[0], g[1], g[2], g[3], g[4], g[5], g[6], begin, n_nodes, center, center_stride,
      (const typename AdjVec<R>::V *)G, node_stride, slot_stride, dirs, dirs_d, ndir, slots, n_lambda, Gc, n, grad);
  count_launch();
  PO_CUDA(cudaGetLastError());
  return PO_OK;
}

po_status launch_point_adjoint_f64(const float *const g[7], const int32_t *begin, int64_t n_nodes,
                                   const double *center, int center_stride, const double2 *G, int64_t node_stride,
                                   int64_t slot_stride, const double *dirs_d, int ndir, const SlotParams<double> *slots,
                                   int n_lambda, int Gc, int64_t n, double *grad, cudaStream_t st) {
  return launch_point_adjoint_t<double>(g, begin, n_nodes, center, center_stride, G, node_stride, slot_stride,
                                        nullptr, dirs_d, ndir, slots, n_lambda, Gc, n, grad, st);
}

// chunk starts 0, chunk, 2 chunk, ... n (the depth-0 adjoint treats every
// chunk of points as a node)
__global__ void k_chunk_begin(int32_t *begin, int64_t nchunk, int64_t n, int chunk) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i <= nchunk) begin[i] = (int32_t)(i * chunk < n ? i * chunk : n);
}

po_status launch_chunk_begin(int32_t *begin, int64_t n, int chunk, cudaStream_t st) {
  const int64_t nchunk = (n + chunk - 1) / chunk;
  k_chunk_begin<<<(unsigned)((nchunk + 256) / 256), 256, 0, st>>>(begin, nchunk, n, chunk);
  count_launch();
  PO_CUDA(cudaGetLastError());
  return PO_OK;
}

// grad_out[k][perm[i]] = (float) grad_sorted[k][i]  (perm = NULL: identity)
__global__ void k_scatter_grad(const double *__restrict__ gs, const int32_t *__restrict__ perm, int64_t n,
                               float *__restrict__ out) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t dst = perm ? perm[i] : i;
#pragma unroll
  for (int k = 0; k < kNT; ++k) out[(int64_t)k * n + dst] = (float)gs[(int64_t)k * n + i];
}

po_status launch_scatter_grad(const double *grad_sorted, const int32_t *perm, int64_t n, float *out, cudaStream_t st) {
  if (n <= 0) return PO_OK;
  k_scatter_grad<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(grad_sorted, perm, n, out);
  count_launch();
  PO_CUDA(cudaGetLastError());
  return PO_OK;
}

}  // namespace wavepo
