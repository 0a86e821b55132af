// po_leaf_mma.cu -- leaf far-field sums as a split-precision tensor-core
// contraction (PO_PREC_SPLIT_BF16).
//
// Replaces the same reference code as k_leaf (util/fields.h:2-50 with the
// per-leaf reduce of compareMie/sphere.cu:603-658, currents of
// util/tangentplane.h:84 fused).  For one leaf and one wavelength
//   F[d][j] = sum_p exp(i s_d.u_p) C_p[j],   j = (slot, component)
// is a complex product of the phase matrix (directions x points) with the
// currents (points x 6G).  As one real GEMM with K = 2 x points:
//   A[d][2p] = cos(s_d.u_p), A[d][2p+1] = sin(s_d.u_p)
//   B[2p][2j] = Re C, B[2p][2j+1] = Im C, B[2p+1][2j] = -Im C, B[2p+1][2j+1] = Re C
// so that D[d][2j] = Re F, D[d][2j+1] = Im F.  A is generated in registers,
// directly in the mma.sync fragment layout, from FP32 phases (the leaf-local
// argument is small: k times the leaf half-diagonal) after a Cody-Waite
// reduction; B is built once per point chunk in shared memory.  Both are split
// into bf16 hi + lo and multiplied as hi*hi + hi*lo + lo*hi with FP32
// accumulation: the phase generation is shared by all slots of a wavelength.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>

#include "po_common.cuh"
#include "po_internal.h"
#include "po_kernels.h"
#include "po_rows_block.cuh"

namespace wavepo {

namespace {

// (cos, sin) of the phase of direction s and point u, split into hi/lo pairs.
// REDUCE: Cody-Waite reduction to [-pi, pi] first; without it the hardware
// sine / cosine take the argument directly, which the caller allows only for
// |phase| <= kLeafFastPhase (absolute error <= ~2e-6 there, below the ~1.5e-5
// of the split operands).
constexpr float kLeafFastPhase = 16.f;
template <bool REDUCE>
__device__ __forceinline__ void phase_frag(float sx, float sy, float sz, float4 u, uint32_t &hi, uint32_t &lo) {
  float sn, cs;
  const float ph = fmaf(sx, u.x, fmaf(sy, u.y, sz * u.z));
  if (REDUCE)
    sincos_small(ph, &sn, &cs);
  else
    __sincosf(ph, &sn, &cs);
  split_bf16x2(cs, sn, hi, lo);
}

constexpr int kPC = 128;  // points per chunk (16 k-steps of 16 = 8 points x cos/sin)

}  // namespace

// CTA: one (leaf, wavelength) and GC slots g0.. of the wavelength (NT n-tiles
// of 8 real columns = 2 x 6 GC), 4 warps over the 16-direction row tiles.
// Dynamic shared memory: s_u[kPC] float4, s_cur[kPC][6 GC] float2,
// s_b[kPC/8][NT][32] uint4 (B fragments {hi0, hi1, lo0, lo1}).
// Fused phi pass of the level above (fz.mid set): once the leaf's patterns
// are complete, the CTA re-reads them (L2) and writes the packed mirror-pair
// sums and differences of its 6 GC patterns (rows_block<1>, the φ-matrix
// fragments staged in s_b), which removes the separate row pass of that level.
struct LeafRowFusion {
  const uint4 *B;  // phi matrix fragments of the level above (one n-tile group)
  uint4 *mid;      // packed output (nullptr: no fusion)
  int KS, nq, Rc, Pc, Pp;
};
// The fused phi pass of one CTA (its own register allocation: kept out of the
// contraction loop's).
__device__ __noinline__ void leaf_rows_epilogue(const float2 *out, uint4 *s_b, const LeafRowFusion fz, int64_t lam,
                                                int64_t leaf, int64_t n_leaves, int Gtot, int g0, int GC) {
  for (int e = threadIdx.x; e < fz.nq * fz.KS * 32; e += blockDim.x) s_b[e] = fz.B[e];
  __syncthreads();
  const int Rc2 = fz.Rc + (fz.Rc & 1), warp = threadIdx.x >> 5;
  for (int s2 = 0; s2 < GC; ++s2) {
    const int64_t lo = ((lam * Gtot + g0 + s2) * n_leaves + leaf) * 6 * Rc2, hi = lo + 6 * Rc2;
    for (int64_t blk = lo / 8 + warp; blk * 8 < hi; blk += 4)
      rows_block<1, true>(blk, lo, hi, out, fz.mid, fz.Rc, Rc2, fz.Pc, fz.Pp, fz.KS, s_b, 0, fz.nq, 0);
  }
}

template <int GC>
__global__ void __launch_bounds__(128, 5) k_leaf_mma(
    const float *__restrict__ x, const float *__restrict__ y, const float *__restrict__ z,
    const float *__restrict__ nx, const float *__restrict__ ny, const float *__restrict__ nz,
    const float *__restrict__ area, const int32_t *__restrict__ leaf_begin, const double *__restrict__ leaf_center,
    const SlotParams<float> *__restrict__ slots, const float4 *__restrict__ dirs, int ndir, int64_t n_leaves,
    int Gtot, int g0, float2 *__restrict__ out, LeafRowFusion fz) {
  constexpr int NC = 6 * GC;            // complex columns
  constexpr int NT = (2 * NC + 7) / 8;  // n-tiles of 8 real columns
  extern __shared__ uint4 smem_leaf[];
  uint4 *s_b = smem_leaf;                                        // [kPC/8][NT][32]
  float4 *s_u = (float4 *)(s_b + (kPC / 8) * NT * 32);           // [kPC]
  float2 *s_cur = (float2 *)(s_u + kPC);                         // [kPC][NC]
  const int64_t leaf = blockIdx.x;
  const int lam = blockIdx.y;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, tq = lane & 3;
  const int b = leaf_begin[leaf], e = leaf_begin[leaf + 1];
  const double cxd = leaf_center[3 * leaf], cyd = leaf_center[3 * leaf + 1], czd = leaf_center[3 * leaf + 2];
  const SlotParams<float> *sl = slots + (int64_t)lam * Gtot + g0;
  const double k0 = sl[0].k0d;
  const int64_t slot_stride = n_leaves * 6 * (int64_t)ndir;
  float2 *obase = out + ((int64_t)lam * Gtot + g0) * slot_stride + leaf * 6 * (int64_t)ndir;
  const int MT = (ndir + 15) / 16;
  for (int c0 = b; c0 < e || (c0 == b && b == e); c0 += kPC) {
    const int cnt = max(0, min(kPC, e - c0));
    const bool first = (c0 == b);
    __syncthreads();
    bool big = false;  // a phase |s.u| <= |u| of this chunk may exceed kLeafFastPhase
    for (int q = threadIdx.x; q < kPC; q += blockDim.x) {
      if (q < cnt) {
        const int p = c0 + q;
        const float px = x[p], py = y[p], pz = z[p];
        const float4 u = make_float4((float)(k0 * ((double)px - cxd)), (float)(k0 * ((double)py - cyd)),
                                     (float)(k0 * ((double)pz - czd)), 0.f);
        s_u[q] = u;
        big |= !(u.x * u.x + u.y * u.y + u.z * u.z <= kLeafFastPhase * kLeafFastPhase);
        const float qx = nx[p], qy = ny[p], qz = nz[p], ar = area[p];
#pragma unroll
        for (int s2 = 0; s2 < GC; ++s2) {
          cx<float> c[6];
          tangent_plane<float>(sl[s2], px, py, pz, qx, qy, qz, ar, c);
#pragma unroll
          for (int k = 0; k < 6; ++k) s_cur[q * NC + s2 * 6 + k] = make_float2(c[k].re, c[k].im);
        }
      } else {
        s_u[q] = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int k = 0; k < NC; ++k) s_cur[q * NC + k] = make_float2(0.f, 0.f);
      }
    }
    const bool reduce = __syncthreads_or(big) != 0;
    const int ksteps = (cnt + 7) / 8;
    // B fragments: lane ln of n-tile nt holds rows k = 2tq', 2tq'+1 (point tq') and
    // 2tq'+8, 2tq'+9 (point tq'+4) of real column n = nt*8 + g'
    for (int idx = threadIdx.x; idx < ksteps * NT * 32; idx += blockDim.x) {
      const int ln = idx & 31, nt = (idx >> 5) % NT, ks = (idx >> 5) / NT;
      const int n = nt * 8 + (ln >> 2), j = n >> 1, part = n & 1;
      const int p0 = ks * 8 + (ln & 3);
      float v[4];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const float2 cv = j < NC ? s_cur[(p0 + 4 * h) * NC + j] : make_float2(0.f, 0.f);
        v[2 * h] = part ? cv.y : cv.x;       // cos row
        v[2 * h + 1] = part ? cv.x : -cv.y;  // sin row
      }
      uint32_t h0, l0, h1, l1;
      split_bf16x2(v[0], v[1], h0, l0);
      split_bf16x2(v[2], v[3], h1, l1);
      s_b[idx] = make_uint4(h0, h1, l0, l1);
    }
    __syncthreads();
    for (int mt = warp; mt < MT; mt += 4) {
      const int d0 = mt * 16 + g, d1 = d0 + 8;
      const float4 s0 = __ldg(dirs + min(d0, ndir - 1)), s1 = __ldg(dirs + min(d1, ndir - 1));
      float acc[NT][4];
#pragma unroll
      for (int nt = 0; nt < NT; ++nt) acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.f;
      for (int ks = 0; ks < ksteps; ++ks) {
        const float4 ua = s_u[ks * 8 + tq], ub = s_u[ks * 8 + tq + 4];
        uint32_t ahi[4], alo[4];
        if (reduce) {
          phase_frag<true>(s0.x, s0.y, s0.z, ua, ahi[0], alo[0]);
          phase_frag<true>(s1.x, s1.y, s1.z, ua, ahi[1], alo[1]);
          phase_frag<true>(s0.x, s0.y, s0.z, ub, ahi[2], alo[2]);
          phase_frag<true>(s1.x, s1.y, s1.z, ub, ahi[3], alo[3]);
        } else {
          phase_frag<false>(s0.x, s0.y, s0.z, ua, ahi[0], alo[0]);
          phase_frag<false>(s1.x, s1.y, s1.z, ua, ahi[1], alo[1]);
          phase_frag<false>(s0.x, s0.y, s0.z, ub, ahi[2], alo[2]);
          phase_frag<false>(s1.x, s1.y, s1.z, ub, ahi[3], alo[3]);
        }
        uint4 bv[NT];
#pragma unroll
        for (int nt = 0; nt < NT; ++nt) bv[nt] = s_b[(ks * NT + nt) * 32 + lane];
#pragma unroll
        for (int nt = 0; nt < NT; ++nt) {
          const uint32_t bhi[2] = {bv[nt].x, bv[nt].y};
          mma_bf16(acc[nt], ahi, bhi);
        }
#pragma unroll
        for (int nt = 0; nt < NT; ++nt) {
          const uint32_t blo[2] = {bv[nt].z, bv[nt].w};
          mma_bf16(acc[nt], ahi, blo);
        }
#pragma unroll
        for (int nt = 0; nt < NT; ++nt) {
          const uint32_t bhi[2] = {bv[nt].x, bv[nt].y};
          mma_bf16(acc[nt], alo, bhi);
        }
      }
      // D fragment: (d0, d1) = Re/Im of complex column nt*4+tq at direction d0; (d2, d3) at d1
#pragma unroll
      for (int nt = 0; nt < NT; ++nt) {
        const int j = nt * 4 + tq;
        if (j >= NC) continue;
        float2 *o = obase + (int64_t)(j / 6) * slot_stride + (int64_t)(j % 6) * ndir;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int d = h ? d1 : d0;
          if (d >= ndir) continue;
          float2 v = make_float2(acc[nt][2 * h], acc[nt][2 * h + 1]);
          if (!first) {
            const float2 w = o[d];
            v.x += w.x;
            v.y += w.y;
          }
          o[d] = v;
        }
      }
    }
    if (cnt == 0) break;  // an empty leaf (root of an empty cloud) was written as zeros
  }
  if (fz.mid) {
    __syncthreads();  // the leaf's patterns are written (read back through L2); s_b is free
    leaf_rows_epilogue(out, s_b, fz, lam, leaf, n_leaves, Gtot, g0, GC);
  }
}

template <int GC>
static size_t leaf_mma_smem() {
  constexpr int NT = (12 * GC + 7) / 8;
  return sizeof(uint4) * (kPC / 8) * NT * 32 + sizeof(float4) * kPC + sizeof(float2) * kPC * 6 * GC;
}

po_status init_leaf_mma_attributes() {
  PO_CUDA(cudaFuncSetAttribute(k_leaf_mma<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)leaf_mma_smem<1>()));
  PO_CUDA(cudaFuncSetAttribute(k_leaf_mma<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)leaf_mma_smem<2>()));
  PO_CUDA(cudaFuncSetAttribute(k_leaf_mma<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)leaf_mma_smem<3>()));
  PO_CUDA(cudaFuncSetAttribute(k_leaf_mma<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)leaf_mma_smem<4>()));
  return PO_OK;
}

// Whether the phi pass from a leaf grid of Rc x Pc to Pp parent columns can run
// fused in the leaf kernel: one n-tile group, fragments within s_b (GC = 1).
bool leaf_row_fusion_fits(int Pc, int Pp, int Kp) {
  const int NTt = ((Pp + 1) / 2 + 3) / 4, KS = Kp / 16;
  return NTt <= kRowNG && Kp >= Pc && Kp % 16 == 0 && NTt * KS * 32 <= (kPC / 8) * ((12 + 7) / 8) * 32;
}

po_status launch_leaf_mma(const float *const g[7], const int32_t *leaf_begin, const double *leaf_center,
                          int64_t n_leaves, const SlotParams<float> *slots_dev, int n_lambda, int G,
                          const float4 *dirs, int ndir, float2 *out, cudaStream_t st, const uint32_t *fuse_B,
                          uint4 *fuse_mid, int Rc, int Pc, int Pp, int Kp) {
  if (n_leaves <= 0 || n_lambda <= 0) return PO_OK;
  LeafRowFusion fz{nullptr, nullptr, 0, 0, 0, 0, 0};
  if (fuse_mid) {
    if (!leaf_row_fusion_fits(Pc, Pp, Kp) || (int64_t)Rc * Pc != ndir)
      return fail(PO_ERR_INTERNAL, "leaf/phi-pass fusion does not fit");
    fz = LeafRowFusion{(const uint4 *)fuse_B, fuse_mid, Kp / 16, ((Pp + 1) / 2 + 3) / 4, Rc, Pc, Pp};
  }
  if (n_lambda > 65535) return fail(PO_ERR_UNSUPPORTED, "too many wavelengths for one launch");
  dim3 grid((unsigned)n_leaves, (unsigned)n_lambda);
  // slots of a wavelength share its phases; groups of up to 4 per launch
  for (int g0 = 0; g0 < G; g0 += 4) {
    const int gc = std::min(4, G - g0);
#define PO_LEAF_MMA(GG)                                                                                          \
  k_leaf_mma<GG><<<grid, 128, leaf_mma_smem<GG>(), st>>>(g[0], g[1], g[2], g[3], g[4], g[5], g[6], leaf_begin, \
                                                        leaf_center, slots_dev, dirs, ndir, n_leaves, G, g0, out, fz)
    switch (gc) {
      case 1: PO_LEAF_MMA(1); break;
      case 2: PO_LEAF_MMA(2); break;
      case 3: PO_LEAF_MMA(3); break;
      default: PO_LEAF_MMA(4); break;
    }
#undef PO_LEAF_MMA
    count_launch();
  }
  PO_CUDA(cudaGetLastError());
  return PO_OK;
}

}  // namespace wavepo
