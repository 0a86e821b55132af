// po_rows_block.cuh -- one warp's block of 8 output rows of the phi pass on the
// tensor cores (split-bf16 mma.sync), shared by the row-pass kernel
// (po_interp_mma.cu) and the leaf kernel's fused epilogue (po_leaf_mma.cu).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "po_common.cuh"

namespace wavepo {

// One warp per block of 8 rows; n-tiles in groups of kRowNG (accumulators in
// registers); the B fragments come from shared memory when they fit.
// PACK (forward pass feeding k_theta_warp): the phi matrix is in mirror-pair
// column order (build_phi_matrix), rows are indexed over patterns of Rc2 = Rc
// rounded up to even rows (row Rc of an odd Rc is a zero row), and the output
// is S = h_j + h_j', D = h_j - h_j' (j' = j + H, H = ceil(Pp/2) pairs; an odd
// Pp has one phantom column j' = Pp, a zero column of the phi matrix) split
// into bf16 hi + lo in row pairs: per pattern [Rc2/2][H][re, im] uint4 {S hi
// pair, S lo pair, D hi pair, D lo pair}, each pair holding rows 2 tp (low
// half) and 2 tp + 1.
// Lane g and lane g^1 (4 apart) hold the two rows of a pair; the even lane
// stores the real parts, the odd lane the imaginary parts.
// PACK == 2 (forward pass feeding the tcgen05 theta pass, po_theta_tc.cu): the
// same sums and differences as four bf16 matrices (S hi, S lo, D hi, D lo) per
// child, whose six component patterns share one column space, in chunks of 16
// rows, [Rr/16][matrix][npad/8][2][8][8]: core matrices of 8 columns x 8 rows
// (16 B per column row); element (column n = comp Pp + 2j + part, row t) of
// matrix m at byte
// (t/16) 128 npad + m 32 npad + (n/8) 256 + ((t/8)%2) 128 + (n%8) 16 + (t%8) 2.
// Patterns have Rr rows (rows Rc .. Rr-1 are zero); the 32 lanes of a warp
// store one whole core matrix per matrix and n-tile.
constexpr int kRowNG = 8;

// Rows blk*8 .. blk*8+7 of the output, of which [row_lo, row_hi) are this
// caller's (the others are neither read nor written; in the packed layouts
// row_lo and row_hi are even, so that no row pair is split).  B: the phi
// matrix fragments of n-tile group ng (nq tiles, KS k-steps).  COHERENT: the
// input was written earlier by the same kernel, so it is read through L2
// (ld.global.cg), never through the read-only path.
template <int PACK, bool COHERENT>
__device__ __forceinline__ void rows_block(int64_t blk, int64_t row_lo, int64_t row_hi, const float2 *src,
                                           void *__restrict__ dst_, int Rc, int Rc2, int Pc, int Pp, int KS,
                                           const uint4 *B, int ng, int nq, int npad) {
  const int lane = threadIdx.x & 31, g = lane >> 2, tq = lane & 3;
  const int half = (Pp + 1) / 2;  // PACK == 2: Pp is even
  const int64_t r = blk * 8 + g;
  const bool rok = r >= row_lo && r < row_hi;
  int64_t srow = r;
  bool in_ok = rok;
  if (PACK) {
    const int64_t pattern = r / Rc2;
    const int t = (int)(r - pattern * Rc2);
    srow = pattern * Rc + t;
    in_ok = rok && t < Rc;
  }
  const float2 *in = src + (in_ok ? srow : 0) * (int64_t)Pc;
  auto load_in = [&](int ks, float2 (&v)[4]) {
    const int k0 = ks * 16 + 2 * tq;
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int k = k0 + (u & 1) + (u >> 1) * 8;
      v[u] = (in_ok && k < Pc) ? (COHERENT ? __ldcg(in + k) : in[k]) : make_float2(0.f, 0.f);
    }
  };
  float acc[kRowNG][4];
#pragma unroll
  for (int q = 0; q < kRowNG; ++q) acc[q][0] = acc[q][1] = acc[q][2] = acc[q][3] = 0.f;
  float2 vn[4];
  load_in(0, vn);
  for (int ks = 0; ks < KS; ++ks) {
    const float2 v[4] = {vn[0], vn[1], vn[2], vn[3]};
    if (ks + 1 < KS) load_in(ks + 1, vn);
    uint32_t ahi[4], alo[4];
    split_bf16x2(v[0].x, v[1].x, ahi[0], alo[0]);  // row g (real parts), k0, k0+1
    split_bf16x2(v[0].y, v[1].y, ahi[1], alo[1]);  // row g+8 (imaginary parts)
    split_bf16x2(v[2].x, v[3].x, ahi[2], alo[2]);  // row g, k0+8, k0+9
    split_bf16x2(v[2].y, v[3].y, ahi[3], alo[3]);
    if (nq == kRowNG) {  // full group: n-tiles in pairs, two independent accumulators per product
#pragma unroll
      for (int q = 0; q < kRowNG; q += 2) {
        const uint4 b0 = B[((size_t)q * KS + ks) * 32 + lane], b1 = B[((size_t)(q + 1) * KS + ks) * 32 + lane];
        const uint32_t h0[2] = {b0.x, b0.y}, l0[2] = {b0.z, b0.w}, h1[2] = {b1.x, b1.y}, l1[2] = {b1.z, b1.w};
        mma_bf16(acc[q], ahi, h0);
        mma_bf16(acc[q + 1], ahi, h1);
        mma_bf16(acc[q], ahi, l0);
        mma_bf16(acc[q + 1], ahi, l1);
        mma_bf16(acc[q], alo, h0);
        mma_bf16(acc[q + 1], alo, h1);
      }
    } else {
#pragma unroll
      for (int q = 0; q < kRowNG; ++q) {
        if (q >= nq) break;
        const uint4 bv = B[((size_t)q * KS + ks) * 32 + lane];
        const uint32_t bhi[2] = {bv.x, bv.y}, blo[2] = {bv.z, bv.w};
        mma_bf16(acc[q], ahi, bhi);
        mma_bf16(acc[q], ahi, blo);
        mma_bf16(acc[q], alo, bhi);
      }
    }
  }
  if (PACK == 2) {
    const bool odd = g & 1;
    const int64_t pattern = r / Rc2;
    const int t0 = (int)(r - pattern * Rc2) & ~1;  // the pair's first row
    // the six component patterns of a child share one column space
    const int64_t group = pattern / 6;
    const int col0 = (int)(pattern - group * 6) * Pp;
    uint8_t *base = (uint8_t *)dst_ + (size_t)group * 8 * npad * Rc2;
    const size_t mat = (size_t)npad * 32;  // matrix stride inside a 16-row chunk
#pragma unroll
    for (int q = 0; q < kRowNG; ++q) {
      if (q >= nq) break;
      const float sr = acc[q][0] + acc[q][1], dr = acc[q][0] - acc[q][1];
      const float si = acc[q][2] + acc[q][3], di = acc[q][2] - acc[q][3];
      const float xs = __shfl_xor_sync(0xffffffffu, odd ? sr : si, 4);
      const float xd = __shfl_xor_sync(0xffffffffu, odd ? dr : di, 4);
      const float s0 = odd ? xs : sr, s1 = odd ? si : xs;
      const float d0 = odd ? xd : dr, d1 = odd ? di : xd;
      const int j = (ng + q) * 4 + tq;
      uint32_t sh, sl, dh, dl;
      split_bf16x2(s0, s1, sh, sl);
      split_bf16x2(d0, d1, dh, dl);
      if (rok && j < half) {
        const int n = col0 + 2 * j + (odd ? 1 : 0);
        const size_t off = (size_t)(t0 >> 4) * 128 * npad + (size_t)(n >> 3) * 256 + ((t0 >> 3) & 1) * 128 +
                           (n & 7) * 16 + (t0 & 7) * 2;
        *(uint32_t *)(base + off) = sh;
        *(uint32_t *)(base + mat + off) = sl;
        *(uint32_t *)(base + 2 * mat + off) = dh;
        *(uint32_t *)(base + 3 * mat + off) = dl;
      }
    }
  } else if (PACK == 1) {
    uint4 *dst = (uint4 *)dst_;
    const bool odd = g & 1;
    const int64_t pair_row = r >> 1;  // = pattern * Rc2/2 + t/2, Rc2 even
#pragma unroll
    for (int q = 0; q < kRowNG; ++q) {
      if (q >= nq) break;
      // acc: {re j, re j', im j, im j'} of this lane's row
      const float sr = acc[q][0] + acc[q][1], dr = acc[q][0] - acc[q][1];
      const float si = acc[q][2] + acc[q][3], di = acc[q][2] - acc[q][3];
      // even lane (row t) keeps the real parts and sends its imaginary ones
      const float xs = __shfl_xor_sync(0xffffffffu, odd ? sr : si, 4);
      const float xd = __shfl_xor_sync(0xffffffffu, odd ? dr : di, 4);
      const float s0 = odd ? xs : sr, s1 = odd ? si : xs;  // rows t, t+1 of this lane's part
      const float d0 = odd ? xd : dr, d1 = odd ? di : xd;
      const int j = (ng + q) * 4 + tq;
      uint32_t sh, sl, dh, dl;
      split_bf16x2(s0, s1, sh, sl);
      split_bf16x2(d0, d1, dh, dl);
      if (rok && j < half) dst[(pair_row * half + j) * 2 + (odd ? 1 : 0)] = make_uint4(sh, sl, dh, dl);
    }
  } else if (rok) {
    float2 *out = (float2 *)dst_ + r * (int64_t)Pp;
#pragma unroll
    for (int q = 0; q < kRowNG; ++q) {
      const int j = (ng + q) * 8 + 2 * tq;
      if (j < Pp) out[j] = make_float2(acc[q][0], acc[q][2]);
      if (j + 1 < Pp) out[j + 1] = make_float2(acc[q][1], acc[q][3]);
    }
  }
}

}  // namespace wavepo
