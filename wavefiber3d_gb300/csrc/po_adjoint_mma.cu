// po_adjoint_mma.cu -- back-projection of the leaf adjoint patterns onto the
// points as a split-precision tensor-core contraction (FP32 gradient chain).
//
// For one leaf and one slot (the transpose of the leaf sum of po_leaf_mma.cu,
// util/fields.h:2-50):
//   A^a_c(p) = sum_d w_a(d) G_c(d) exp(-i s_d.u_p),  w = (1, s_x, s_y, s_z),
// a complex product of the phase matrix (points x directions) with the 24
// weighted adjoint columns (a, c).  As one real GEMM with K = 2 x directions:
//   A[p][2d] = cos(-s_d.u_p), A[p][2d+1] = sin(-s_d.u_p)
//   B[2d][2j] = Re W, B[2d][2j+1] = Im W, B[2d+1][2j] = -Im W, B[2d+1][2j+1] = Re W
// with W = w_a G_c and complex column j = 4 c + a, so that lane quad position
// tq of the D fragment holds A^{a=tq}_c for all six components.  A is
// generated in registers in fragment order; B is built per chunk of
// directions in shared memory; both are split into bf16 hi + lo and
// multiplied as hi*hi + hi*lo + lo*hi with FP32 accumulation.
//
// The gradients then follow as in the CUDA-core kernel (po_adjoint.cu):
//   dL/dq_i += 2 Re(A^0^H dC/dq_i),  dL/dx_a += -2 k Im(A^a^H C)
// with the tangent-plane Jacobian dC/dq split over the four lanes of a quad:
// lane tq carries the tangents sel[tq] = {nx, ny}, {x, nz}, {y, area}, {z},
// so the phase term of coordinate a-1 lands in the lane that holds A^a, and
// every (gradient, point) pair has exactly one owner.
#include <cuda_runtime.h>

#include "po_common.cuh"
#include "po_dual.cuh"
#include "po_internal.h"
#include "po_kernels.h"

namespace wavepo {

namespace {

constexpr int kPaDirs = 128;                // directions per chunk (16 k-steps of 8)
constexpr int kPaWarps = 8;                 // one 16-point tile per warp
constexpr int kPaPts = kPaWarps * 16;       // points per pass of a CTA
constexpr int kPaNT = 6;                    // n-tiles: 6 components x 4 weights = 24 complex columns
constexpr size_t kPaSmem = sizeof(uint4) * (kPaDirs / 8) * kPaNT * 32 + sizeof(float2) * 6 * kPaDirs +
                           sizeof(float4) * kPaDirs;

// (cos, sin) of -s.u split into hi / lo bf16 pairs (an A-fragment register).
// REDUCE: Cody-Waite reduction to [-pi, pi] first; without it the hardware
// sine / cosine take the argument directly, which the kernel allows only when
// every |u| of the warp is <= kAdjFastPhase (absolute error <= ~2e-6 there).
constexpr float kAdjFastPhase = 16.f;
template <bool REDUCE>
__device__ __forceinline__ void adj_phase_frag(float4 s, float ux, float uy, float uz, uint32_t &hi, uint32_t &lo) {
  float sn, cs;
  const float ph = -fmaf(s.x, ux, fmaf(s.y, uy, s.z * uz));
  if (REDUCE)
    sincos_small(ph, &sn, &cs);
  else
    __sincosf(ph, &sn, &cs);
  split_bf16x2(cs, sn, hi, lo);
}

// The Jacobian is taken once per (point, slot), outside the direction loop:
// a call keeps its registers out of the tensor-core loop's budget.
__device__ __noinline__ void jvp_two_tangents(const SlotParams<double> &P, float px, float py, float pz, float qx,
                                              float qy, float qz, float area, const int (&sel)[2],
                                              CDual<float, 2> out[6]) {
  tangent_plane_jvp<float, 2>(P, px, py, pz, qx, qy, qz, area, sel, out);
}

}  // namespace

// CTA: one node, 8 warps; warp w owns points p0 + 16 w + (g, g + 8) of each
// pass of 128 points.  G[slot][node * node_stride][6][ndir] about
// centre[3 * node * center_stride]; gradients are added to grad[7][n].
__global__ void __launch_bounds__(32 * kPaWarps, 2) k_point_adjoint_mma(
    const float *__restrict__ x, const float *__restrict__ y, const float *__restrict__ z,
    const float *__restrict__ nx, const float *__restrict__ ny, const float *__restrict__ nz,
    const float *__restrict__ area, const int32_t *__restrict__ begin, const double *__restrict__ center,
    int center_stride, const float2 *__restrict__ G, int64_t node_stride, int64_t slot_stride,
    const float4 *__restrict__ dirs, int ndir, const SlotParams<double> *__restrict__ slots, int n_lambda, int Gc,
    int64_t n, double *__restrict__ grad) {
  extern __shared__ uint4 smem_pa[];
  uint4 *s_b = smem_pa;                                        // [kPaDirs/8][kPaNT][32]
  float2 *s_g = (float2 *)(s_b + (kPaDirs / 8) * kPaNT * 32);  // [6][kPaDirs]
  float4 *s_s = (float4 *)(s_g + 6 * kPaDirs);                 // [kPaDirs]
  const int64_t node = blockIdx.x;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, tq = lane & 3;
  const int b = begin[node], e = begin[node + 1];
  const double *ctr = center + 3 * node * center_stride;
  const double cx_ = ctr[0], cy_ = ctr[1], cz_ = ctr[2];
  // this lane's tangents (global 0..6 = x, y, z, nx, ny, nz, area; -1 unused)
  const int sel[2] = {tq == 0 ? 3 : tq - 1, tq == 0 ? 4 : tq == 1 ? 5 : tq == 2 ? 6 : -1};
  for (int p0 = b; p0 < e; p0 += kPaPts) {
    int pp[2];
    bool ok[2];
    float px[2], py[2], pz[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      pp[h] = p0 + warp * 16 + g + 8 * h;
      ok[h] = pp[h] < e;
      px[h] = ok[h] ? x[pp[h]] : 0.f;
      py[h] = ok[h] ? y[pp[h]] : 0.f;
      pz[h] = ok[h] ? z[pp[h]] : 0.f;
    }
    const bool warp_active = p0 + warp * 16 < e;
    double gacc[2][2] = {{0.0, 0.0}, {0.0, 0.0}};  // [row h][tangent slot]
    for (int lam = 0; lam < n_lambda; ++lam) {
      const double k0 = slots[lam * Gc].k0d;
      float ux[2], uy[2], uz[2];
      bool big = false;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        ux[h] = (float)(k0 * ((double)px[h] - cx_));
        uy[h] = (float)(k0 * ((double)py[h] - cy_));
        uz[h] = (float)(k0 * ((double)pz[h] - cz_));
        big |= ok[h] && !(ux[h] * ux[h] + uy[h] * uy[h] + uz[h] * uz[h] <= kAdjFastPhase * kAdjFastPhase);
      }
      const bool reduce = __any_sync(0xffffffffu, big);
      for (int gs = 0; gs < Gc; ++gs) {
        const int slot = lam * Gc + gs;
        const float2 *gp = G + slot * slot_stride + node * node_stride;
        float acc[kPaNT][4];
#pragma unroll
        for (int nt = 0; nt < kPaNT; ++nt) acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.f;
        for (int d0 = 0; d0 < ndir; d0 += kPaDirs) {
          const int cnt = ndir - d0 < kPaDirs ? ndir - d0 : kPaDirs;
          const int ksn = (cnt + 7) / 8;
          __syncthreads();
          for (int q = threadIdx.x; q < 6 * kPaDirs; q += blockDim.x) {
            const int c = q / kPaDirs, dq = q - c * kPaDirs;
            s_g[q] = dq < cnt ? gp[(int64_t)c * ndir + d0 + dq] : make_float2(0.f, 0.f);
          }
          for (int q = threadIdx.x; q < kPaDirs; q += blockDim.x)
            s_s[q] = q < cnt ? __ldg(dirs + d0 + q) : make_float4(0.f, 0.f, 0.f, 0.f);
          __syncthreads();
          // B fragments: lane ln of n-tile nt (component c = nt) holds direction rows
          // ks*8 + (ln & 3) and + 4 of real column n = ln >> 2 (weight a = n >> 1)
          for (int idx = threadIdx.x; idx < ksn * kPaNT * 32; idx += blockDim.x) {
            const int ln = idx & 31, nt = (idx >> 5) % kPaNT, ks = (idx >> 5) / kPaNT;
            const int nn = ln >> 2, a = nn >> 1, part = nn & 1;
            float v[4];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
              const int dl = ks * 8 + (ln & 3) + 4 * h;
              const float4 s = s_s[dl];
              const float w = a == 0 ? 1.f : a == 1 ? s.x : a == 2 ? s.y : s.z;
              const float2 gv = s_g[nt * kPaDirs + dl];
              const float wr = w * gv.x, wi = w * gv.y;
              v[2 * h] = part ? wi : wr;       // cos row
              v[2 * h + 1] = part ? wr : -wi;  // sin row
            }
            uint32_t h0, l0, h1, l1;
            split_bf16x2(v[0], v[1], h0, l0);
            split_bf16x2(v[2], v[3], h1, l1);
            s_b[idx] = make_uint4(h0, h1, l0, l1);
          }
          __syncthreads();
          if (!warp_active) continue;
          for (int ks = 0; ks < ksn; ++ks) {
            const float4 sa = s_s[ks * 8 + tq], sb = s_s[ks * 8 + tq + 4];
            uint32_t ahi[4], alo[4];
            if (reduce) {
              adj_phase_frag<true>(sa, ux[0], uy[0], uz[0], ahi[0], alo[0]);  // row g, direction tq
              adj_phase_frag<true>(sa, ux[1], uy[1], uz[1], ahi[1], alo[1]);  // row g + 8
              adj_phase_frag<true>(sb, ux[0], uy[0], uz[0], ahi[2], alo[2]);  // row g, direction tq + 4
              adj_phase_frag<true>(sb, ux[1], uy[1], uz[1], ahi[3], alo[3]);
            } else {
              adj_phase_frag<false>(sa, ux[0], uy[0], uz[0], ahi[0], alo[0]);
              adj_phase_frag<false>(sa, ux[1], uy[1], uz[1], ahi[1], alo[1]);
              adj_phase_frag<false>(sb, ux[0], uy[0], uz[0], ahi[2], alo[2]);
              adj_phase_frag<false>(sb, ux[1], uy[1], uz[1], ahi[3], alo[3]);
            }
            uint4 bv[kPaNT];
#pragma unroll
            for (int nt = 0; nt < kPaNT; ++nt) bv[nt] = s_b[(ks * kPaNT + nt) * 32 + lane];
#pragma unroll
            for (int nt = 0; nt < kPaNT; ++nt) {
              const uint32_t bh[2] = {bv[nt].x, bv[nt].y};
              mma_bf16(acc[nt], ahi, bh);
            }
#pragma unroll
            for (int nt = 0; nt < kPaNT; ++nt) {
              const uint32_t bl[2] = {bv[nt].z, bv[nt].w};
              mma_bf16(acc[nt], ahi, bl);
            }
#pragma unroll
            for (int nt = 0; nt < kPaNT; ++nt) {
              const uint32_t bh[2] = {bv[nt].x, bv[nt].y};
              mma_bf16(acc[nt], alo, bh);
            }
          }
        }
        if (!warp_active) continue;
        // contraction with the currents and their Jacobian, rows g and g + 8
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          float a0r[6], a0i[6];  // A^0 of this row, from lane (g, 0)
#pragma unroll
          for (int c = 0; c < 6; ++c) {
            a0r[c] = __shfl_sync(0xffffffffu, acc[c][2 * h], lane & ~3);
            a0i[c] = __shfl_sync(0xffffffffu, acc[c][2 * h + 1], lane & ~3);
          }
          if (!ok[h]) continue;
          const int p = pp[h];
          CDual<float, 2> C[6];
          jvp_two_tangents(slots[slot], px[h], py[h], pz[h], nx[p], ny[p], nz[p], area[p], sel, C);
#pragma unroll
          for (int k = 0; k < 2; ++k) {
            float t = 0.f;
#pragma unroll
            for (int c = 0; c < 6; ++c) t += a0r[c] * C[c].re.d[k] + a0i[c] * C[c].im.d[k];
            gacc[h][k] += 2.0 * (double)t;
          }
          if (tq >= 1) {  // phase term of coordinate tq - 1: Im(sum_c conj(A^a_c) C_c)
            float im = 0.f;
#pragma unroll
            for (int c = 0; c < 6; ++c) im += acc[c][2 * h] * C[c].im.v - acc[c][2 * h + 1] * C[c].re.v;
            gacc[h][0] += -2.0 * k0 * (double)im;
          }
        }
      }
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      if (!ok[h]) continue;
#pragma unroll
      for (int k = 0; k < 2; ++k)
        if (sel[k] >= 0) grad[(int64_t)sel[k] * n + pp[h]] += gacc[h][k];
    }
  }
}

po_status init_point_adjoint_mma_attributes() {
  PO_CUDA(cudaFuncSetAttribute(k_point_adjoint_mma, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kPaSmem));
  return PO_OK;
}

po_status launch_point_adjoint_mma(const float *const g[7], const int32_t *begin, int64_t n_nodes,
                                   const double *center, int center_stride, const float2 *G, int64_t node_stride,
                                   int64_t slot_stride, const float4 *dirs, int ndir,
                                   const SlotParams<double> *slots, int n_lambda, int Gc, int64_t n, double *grad,
                                   cudaStream_t st) {
  if (n_nodes <= 0 || n_lambda <= 0 || Gc <= 0) return PO_OK;
  if (n_nodes > 2147483647LL) return fail(PO_ERR_UNSUPPORTED, "too many nodes for one launch");
  k_point_adjoint_mma<<<(unsigned)n_nodes, 32 * kPaWarps, kPaSmem, st>>>(
      g[0], g[1], g[2], g[3], g[4], g[5], g[6], begin, center, center_stride, G, node_stride, slot_stride, dirs, ndir,
      slots, n_lambda, Gc, n, grad);
  count_launch();
  PO_CUDA(cudaGetLastError());
  return PO_OK;
}

}  // namespace wavepo
