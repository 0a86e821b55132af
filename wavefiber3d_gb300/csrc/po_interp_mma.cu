// po_interp_mma.cu -- theta interpolation + translation + child sum as a
// split-precision tensor-core product.
//
// The theta half of util/interpolation.h:47-77 (FFT along theta, zero pad with
// the Nyquist split, inverse FFT, scale 1/n) is one fixed linear map per tree
// level: out[t'] = sum_t K_n(t'/Tp - t/Tc) x[t] with the real trigonometric
// kernel
//   K_n(v) = (1/n) [1 + 2 sum_{k=1}^{n/2-1} cos(2 pi k v) + cos(pi n v)]   (n even)
//   K_n(v) = (1/n) sin(pi n v) / sin(pi v)                                 (n odd).
// With the double cover stored as rows 0..n_theta (see k_interp_cols), a
// parent column j is A h_j + B h_{j+Phi/2}: a GEMM with K = 2 Rc whose
// operands are the level's constant matrix [A | B] and the child's stored
// half columns.  Both are split into bf16 hi + lo parts and multiplied as
// hi*hi + hi*lo + lo*hi with FP32 accumulation (mma.sync m16n8k16), which
// keeps ~16 bits of every operand.  The epilogue multiplies each child's
// result by exp(i k s.(c_child - c_parent)) and sums the children into the
// parent in shared memory.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "po_common.cuh"
#include "po_internal.h"
#include "po_kernels.h"

namespace wavepo {

// ------------------------------------------------------------ host side
static double trig_kernel(int n, double v) {
  double f = v - std::nearbyint(v);
  if (std::fabs(f) < 1e-15) return 1.0;
  double x = 2.0 * kPi * v;
  if (n % 2) return std::sin(0.5 * n * x) / (n * std::sin(0.5 * x));
  // even n: Dirichlet sum up to n/2-1 plus the split Nyquist cosine
  double d = std::sin(0.5 * (n - 1) * x) / std::sin(0.5 * x);
  return (d + std::cos(0.5 * n * x)) / n;
}

static uint16_t bf16_rne(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  if ((u & 0x7f800000u) == 0x7f800000u) return (uint16_t)(u >> 16);
  uint32_t r = u + 0x7fffu + ((u >> 16) & 1u);
  return (uint16_t)(r >> 16);
}
static float bf16_to_f(uint16_t h) {
  uint32_t u = (uint32_t)h << 16;
  float f;
  std::memcpy(&f, &u, 4);
  return f;
}

// A operand of one level in mma.sync fragment order:
//   [mtile][kstep][lane] { hi[4] b32, lo[4] b32 }  (32 bytes per lane)
// Rows: parent rows t' < Rp.  Columns (K): own half column rows 0..Rc-1, then
// (mirror) the partner half column rows 0..Rc-1.
size_t theta_matrix_words(int Rp, int Kp) { return (size_t)((Rp + 15) / 16) * (Kp / 16) * 32 * 8; }

// dense M (rows x Kp, row-major) -> A fragments (split hi + lo bf16)
static void a_fragments(const std::vector<double> &M, int rows, int Kp, std::vector<uint32_t> &out) {
  const int MT = (rows + 15) / 16, KS = Kp / 16;
  out.assign(theta_matrix_words(rows, Kp), 0u);
  for (int mt = 0; mt < MT; ++mt)
    for (int ks = 0; ks < KS; ++ks)
      for (int lane = 0; lane < 32; ++lane) {
        const int g = lane >> 2, tq = lane & 3;
        const int rr[4] = {mt * 16 + g, mt * 16 + g + 8, mt * 16 + g, mt * 16 + g + 8};
        const int cc[4] = {ks * 16 + 2 * tq, ks * 16 + 2 * tq, ks * 16 + 2 * tq + 8, ks * 16 + 2 * tq + 8};
        uint32_t *dst = &out[(((size_t)mt * KS + ks) * 32 + lane) * 8];
        for (int q = 0; q < 4; ++q) {
          uint16_t h[2], l[2];
          for (int e = 0; e < 2; ++e) {
            int r = rr[q], c = cc[q] + e;
            double v = (r < rows && c < Kp) ? M[(size_t)r * Kp + c] : 0.0;
            h[e] = bf16_rne((float)v);
            l[e] = bf16_rne((float)(v - (double)bf16_to_f(h[e])));
          }
          dst[q] = (uint32_t)h[0] | ((uint32_t)h[1] << 16);
          dst[4 + q] = (uint32_t)l[0] | ((uint32_t)l[1] << 16);
        }
      }
}

// theta interpolation of one level: parent row r from the child's own half
// column (rows t < Rc) and, mirrored, its partner half column (rows s)
static double theta_own(int Tc, int Tp, int r, int t) { return trig_kernel(Tc, (double)r / Tp - (double)t / Tc); }
static double theta_partner(int Tc, int Tp, int r, int s) {
  return trig_kernel(Tc, (double)r / Tp - (double)(Tc - s) / Tc);
}

void build_theta_matrix(int Tc, int Tp, int Rc, int Rp, int mirror, int Kp, std::vector<uint32_t> &out) {
  const int nth_c = Tc / 2;
  std::vector<double> M((size_t)Rp * Kp, 0.0);
  for (int r = 0; r < Rp; ++r) {
    for (int t = 0; t < Rc; ++t) M[(size_t)r * Kp + t] = theta_own(Tc, Tp, r, t);
    if (mirror)
      for (int s = 1; s < nth_c; ++s) M[(size_t)r * Kp + Rc + s] = theta_partner(Tc, Tp, r, s);
  }
  a_fragments(M, Rp, Kp, out);
}

// Transpose of the mirrored theta map (double cover only): child row t of a
// half column pair from the parent's own column (K = r < Rp) and its partner
// (K = Rp + r):  [A_own^T | A_partner^T], rows t < Rc.
void build_theta_matrix_adj(int Tc, int Tp, int Rc, int Rp, int Kp, std::vector<uint32_t> &out) {
  const int nth_c = Tc / 2;
  std::vector<double> M((size_t)Rc * Kp, 0.0);
  for (int t = 0; t < Rc; ++t)
    for (int r = 0; r < Rp; ++r) {
      M[(size_t)t * Kp + r] = theta_own(Tc, Tp, r, t);
      if (t >= 1 && t < nth_c) M[(size_t)t * Kp + Rp + r] = theta_partner(Tc, Tp, r, t);
    }
  a_fragments(M, Rc, Kp, out);
}

// ---------------------------------------------------------- device side
__device__ __forceinline__ void mma_bf16(float *d, const uint32_t *a, const uint32_t *b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ void split_bf16x2(float x0, float x1, uint32_t &hi, uint32_t &lo) {
  __nv_bfloat16 h0 = __float2bfloat16_rn(x0), h1 = __float2bfloat16_rn(x1);
  __nv_bfloat16 l0 = __float2bfloat16_rn(x0 - __bfloat162float(h0));
  __nv_bfloat16 l1 = __float2bfloat16_rn(x1 - __bfloat162float(h1));
  hi = (uint32_t)__bfloat16_as_ushort(h0) | ((uint32_t)__bfloat16_as_ushort(h1) << 16);
  lo = (uint32_t)__bfloat16_as_ushort(l0) | ((uint32_t)__bfloat16_as_ushort(l1) << 16);
}

// CTA: one (parent node, component, slot) and NCC complex columns (NCC/2
// mirror pairs).  4 warps; warp w owns the 16-row tiles w, w+4, ...
// B operand (child half columns) is staged per child in fragment order:
//   Bf[kstep][ntile][lane] = {hi0, hi1, lo0, lo1}  (n = 2*column + re/im)
template <int NCC>
__global__ void __launch_bounds__(128) k_interp_cols_mma(
    const float2 *__restrict__ mid, float2 *__restrict__ parent, const int32_t *__restrict__ child_table,
    int64_t n_parent, int64_t n_child, int phi, int Rc, int Rp, int Kp, int mirror,
    const uint4 *__restrict__ Afrag, const float4 *__restrict__ trans, int G, float scale_unused) {
  constexpr int NT = NCC / 4;  // n-tiles of 8 (re, im interleaved)
  constexpr int NP = NCC + 1;  // padded row stride of the staged tiles (no bank conflicts)
  extern __shared__ uint4 smem_u4[];
  const int KS = Kp / 16, MT = (Rp + 15) / 16;
  uint4 *Bf = smem_u4;                                       // [KS][NT][32]
  float2 *tile = (float2 *)(Bf + (size_t)KS * NT * 32);      // [Rc][NP]
  float2 *acc = tile + (size_t)Rc * NP;                      // [Rp][NP]
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, tq = lane & 3;
  const int TW = mirror ? NCC / 2 : NCC;
  const int span = mirror ? phi / 2 : phi;
  const int ntile = (span + TW - 1) / TW;
  const int j0 = (int)(blockIdx.x % ntile) * TW;
  const int64_t pc = blockIdx.x / ntile;
  const int64_t p = pc / 6;
  const int comp = (int)(pc % 6);
  const int slot = blockIdx.z, lam = slot / G;
  auto col_of = [&](int q) { return mirror ? (q < TW ? j0 + q : j0 + (q - TW) + phi / 2) : j0 + q; };
  auto ok_of = [&](int q) { return (mirror ? j0 + (q < TW ? q : q - TW) : j0 + q) < span; };
  auto partner_of = [&](int q) { return mirror ? (q < TW ? q + TW : q - TW) : q; };
  for (int e = threadIdx.x; e < Rp * NCC; e += blockDim.x) acc[(e / NCC) * NP + e % NCC] = make_float2(0.f, 0.f);
  const float4 *tr = trans + (int64_t)lam * Rp * phi;
  for (int o = 0; o < 8; ++o) {
    const int32_t c = child_table[p * 8 + o];
    if (c < 0) continue;
    __syncthreads();
    const float2 *m = mid + (((int64_t)slot * n_child + c) * 6 + comp) * (int64_t)Rc * phi;
    for (int e = threadIdx.x; e < Rc * NCC; e += blockDim.x) {
      int t = e / NCC, q = e - t * NCC;
      tile[t * NP + q] = ok_of(q) ? m[(int64_t)t * phi + col_of(q)] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    // B fragments: rows kk of the stacked operand [own half; partner half]
    for (int e = threadIdx.x; e < KS * NT * 32; e += blockDim.x) {
      const int ln = e & 31, nt = (e >> 5) % NT, ks = (e >> 5) / NT;
      const int n = nt * 8 + (ln >> 2), q = n >> 1, part = n & 1;
      const int kb = ks * 16 + 2 * (ln & 3);
      float v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int kk = kb + (u & 1) + (u >> 1) * 8;
        float2 x = make_float2(0.f, 0.f);
        if (kk < Rc) x = tile[kk * NP + q];
        else if (mirror && kk < 2 * Rc) x = tile[(kk - Rc) * NP + partner_of(q)];
        v[u] = part ? x.y : x.x;
      }
      uint32_t h0, l0, h1, l1;
      split_bf16x2(v[0], v[1], h0, l0);
      split_bf16x2(v[2], v[3], h1, l1);
      Bf[e] = make_uint4(h0, h1, l0, l1);
    }
    __syncthreads();
    const float sgx = (o & 1) ? 1.f : -1.f, sgy = (o & 2) ? -1.f : 1.f, sgz = (o & 4) ? -1.f : 1.f;
    for (int mt = warp; mt < MT; mt += 4) {
      float d[NT][4];
#pragma unroll
      for (int nt = 0; nt < NT; ++nt) d[nt][0] = d[nt][1] = d[nt][2] = d[nt][3] = 0.f;
      const uint4 *ap = Afrag + ((size_t)mt * KS) * 64 + lane * 2;
      uint4 nh = __ldg(ap), nl = __ldg(ap + 1);  // A fragments of the next k-step in flight
      for (int ks = 0; ks < KS; ++ks) {
        const uint4 ah = nh, al = nl;
        if (ks + 1 < KS) {
          nh = __ldg(ap + (size_t)(ks + 1) * 64);
          nl = __ldg(ap + (size_t)(ks + 1) * 64 + 1);
        }
        const uint32_t a_hi[4] = {ah.x, ah.y, ah.z, ah.w}, a_lo[4] = {al.x, al.y, al.z, al.w};
#pragma unroll
        for (int nt = 0; nt < NT; ++nt) {
          const uint4 b = Bf[((size_t)ks * NT + nt) * 32 + lane];
          const uint32_t b_hi[2] = {b.x, b.y}, b_lo[2] = {b.z, b.w};
          mma_bf16(d[nt], a_hi, b_hi);
          mma_bf16(d[nt], a_hi, b_lo);
          mma_bf16(d[nt], a_lo, b_hi);
        }
      }
      // epilogue: rows r0 = mt*16+g (d0,d1) and r0+8 (d2,d3); complex column q = nt*4+tq
#pragma unroll
      for (int nt = 0; nt < NT; ++nt) {
        const int q = nt * 4 + tq;
        if (!ok_of(q)) continue;
        const int j = col_of(q);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int r = mt * 16 + g + 8 * h;
          if (r >= Rp) continue;
          const float4 rr = tr[(int64_t)r * phi + j];
          float sn, cs;
          sincos_small(fmaf(sgx, rr.x, fmaf(sgy, rr.y, sgz * rr.z)), &sn, &cs);
          const float vr = d[nt][2 * h], vi = d[nt][2 * h + 1];
          float2 a = acc[r * NP + q];
          a.x += vr * cs - vi * sn;
          a.y += vr * sn + vi * cs;
          acc[r * NP + q] = a;
        }
      }
    }
  }
  __syncthreads();
  float2 *out = parent + (((int64_t)slot * n_parent + p) * 6 + comp) * (int64_t)Rp * phi;
  for (int e = threadIdx.x; e < Rp * NCC; e += blockDim.x) {
    int t = e / NCC, q = e - t * NCC;
    if (ok_of(q)) out[(int64_t)t * phi + col_of(q)] = acc[t * NP + q];
  }
}

// Register-accumulator variant (double cover): CTA of W warps, warp w owns
// the 16-row tiles w, w+W, ... (at most MTPW of them) and keeps its part of
// the parent tile in registers across the children, so shared memory holds
// only the staged child tile and its B fragments.  That leaves room for 16
// columns per CTA (half the A traffic of 8) at the upper levels.
template <int NCC, int MTPW>
__global__ void __launch_bounds__(256) k_interp_cols_reg(
    const float2 *__restrict__ mid, float2 *__restrict__ parent, const int32_t *__restrict__ child_table,
    int64_t n_parent, int64_t n_child, int phi, int Rc, int Rp, int Kp, const uint4 *__restrict__ Afrag,
    const float4 *__restrict__ trans, int G) {
  constexpr int NT = NCC / 4;
  constexpr int NP = NCC + 1;
  constexpr int TW = NCC / 2;
  extern __shared__ uint4 smem_u4[];
  const int KS = Kp / 16, MT = (Rp + 15) / 16;
  const int W = blockDim.x >> 5;
  uint4 *Bf = smem_u4;                                   // [KS][NT][32]
  float2 *tile = (float2 *)(Bf + (size_t)KS * NT * 32);  // [Rc][NP]
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, tq = lane & 3;
  const int span = phi / 2;
  const int ntile = (span + TW - 1) / TW;
  const int j0 = (int)(blockIdx.x % ntile) * TW;
  const int64_t pc = blockIdx.x / ntile;
  const int64_t p = pc / 6;
  const int comp = (int)(pc % 6);
  const int slot = blockIdx.z, lam = slot / G;
  auto col_of = [&](int q) { return q < TW ? j0 + q : j0 + (q - TW) + span; };
  auto ok_of = [&](int q) { return j0 + (q < TW ? q : q - TW) < span; };
  auto partner_of = [&](int q) { return q < TW ? q + TW : q - TW; };
  float acc[MTPW][NT][4];
#pragma unroll
  for (int i = 0; i < MTPW; ++i)
#pragma unroll
    for (int nt = 0; nt < NT; ++nt) acc[i][nt][0] = acc[i][nt][1] = acc[i][nt][2] = acc[i][nt][3] = 0.f;
  const float4 *tr = trans + (int64_t)lam * Rp * phi;
  for (int o = 0; o < 8; ++o) {
    const int32_t c = child_table[p * 8 + o];
    if (c < 0) continue;
    __syncthreads();
    const float2 *m = mid + (((int64_t)slot * n_child + c) * 6 + comp) * (int64_t)Rc * phi;
    for (int e = threadIdx.x; e < Rc * NCC; e += blockDim.x) {
      const int t = e / NCC, q = e - t * NCC;
      tile[t * NP + q] = ok_of(q) ? m[(int64_t)t * phi + col_of(q)] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    for (int e = threadIdx.x; e < KS * NT * 32; e += blockDim.x) {
      const int ln = e & 31, nt = (e >> 5) % NT, ks = (e >> 5) / NT;
      const int n = nt * 8 + (ln >> 2), q = n >> 1, part = n & 1;
      const int kb = ks * 16 + 2 * (ln & 3);
      float v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int kk = kb + (u & 1) + (u >> 1) * 8;
        float2 x = make_float2(0.f, 0.f);
        if (kk < Rc) x = tile[kk * NP + q];
        else if (kk < 2 * Rc) x = tile[(kk - Rc) * NP + partner_of(q)];
        v[u] = part ? x.y : x.x;
      }
      uint32_t h0, l0, h1, l1;
      split_bf16x2(v[0], v[1], h0, l0);
      split_bf16x2(v[2], v[3], h1, l1);
      Bf[e] = make_uint4(h0, h1, l0, l1);
    }
    __syncthreads();
    const float sgx = (o & 1) ? 1.f : -1.f, sgy = (o & 2) ? -1.f : 1.f, sgz = (o & 4) ? -1.f : 1.f;
#pragma unroll
    for (int i = 0; i < MTPW; ++i) {
      const int mt = warp + i * W;
      if (mt >= MT) break;
      float d[NT][4];
#pragma unroll
      for (int nt = 0; nt < NT; ++nt) d[nt][0] = d[nt][1] = d[nt][2] = d[nt][3] = 0.f;
      const uint4 *ap = Afrag + ((size_t)mt * KS) * 64 + lane * 2;
      uint4 nh = __ldg(ap), nl = __ldg(ap + 1);
      for (int ks = 0; ks < KS; ++ks) {
        const uint4 ah = nh, al = nl;
        if (ks + 1 < KS) {
          nh = __ldg(ap + (size_t)(ks + 1) * 64);
          nl = __ldg(ap + (size_t)(ks + 1) * 64 + 1);
        }
        const uint32_t a_hi[4] = {ah.x, ah.y, ah.z, ah.w}, a_lo[4] = {al.x, al.y, al.z, al.w};
#pragma unroll
        for (int nt = 0; nt < NT; ++nt) {
          const uint4 b = Bf[((size_t)ks * NT + nt) * 32 + lane];
          const uint32_t b_hi[2] = {b.x, b.y}, b_lo[2] = {b.z, b.w};
          mma_bf16(d[nt], a_hi, b_hi);
          mma_bf16(d[nt], a_hi, b_lo);
          mma_bf16(d[nt], a_lo, b_hi);
        }
      }
#pragma unroll
      for (int nt = 0; nt < NT; ++nt) {
        const int q = nt * 4 + tq;
        if (!ok_of(q)) continue;
        const int j = col_of(q);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int r = mt * 16 + g + 8 * h;
          if (r >= Rp) continue;
          const float4 rr = __ldg(tr + (int64_t)r * phi + j);
          float sn, cs;
          sincos_small(fmaf(sgx, rr.x, fmaf(sgy, rr.y, sgz * rr.z)), &sn, &cs);
          const float vr = d[nt][2 * h], vi = d[nt][2 * h + 1];
          acc[i][nt][2 * h] += vr * cs - vi * sn;
          acc[i][nt][2 * h + 1] += vr * sn + vi * cs;
        }
      }
    }
  }
  float2 *out = parent + (((int64_t)slot * n_parent + p) * 6 + comp) * (int64_t)Rp * phi;
#pragma unroll
  for (int i = 0; i < MTPW; ++i) {
    const int mt = warp + i * W;
    if (mt >= MT) break;
#pragma unroll
    for (int nt = 0; nt < NT; ++nt) {
      const int q = nt * 4 + tq;
      if (!ok_of(q)) continue;
      const int j = col_of(q);
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int r = mt * 16 + g + 8 * h;
        if (r < Rp) out[(int64_t)r * phi + j] = make_float2(acc[i][nt][2 * h], acc[i][nt][2 * h + 1]);
      }
    }
  }
}

static size_t cols_reg_smem(int ncc, int Rc, int Kp) {
  return sizeof(uint4) * (size_t)(Kp / 16) * (ncc / 4) * 32 + sizeof(float2) * (size_t)Rc * (ncc + 1);
}

template <int NCC>
static po_status launch_cols_reg(dim3 grid, int W, int mtpw, size_t smem, const float2 *mid, float2 *parent,
                                 const int32_t *child_table, int64_t n_parent, int64_t n_child, int phi, int Rc,
                                 int Rp, int Kp, const uint4 *A, const float4 *trans, int G, cudaStream_t st) {
  switch (mtpw) {
#define PO_REG(M)                                                                                               \
  case M:                                                                                                      \
    k_interp_cols_reg<NCC, M><<<grid, 32 * W, smem, st>>>(mid, parent, child_table, n_parent, n_child, phi, Rc, \
                                                          Rp, Kp, A, trans, G);                                 \
    break;
    PO_REG(1) PO_REG(2) PO_REG(3) PO_REG(4) PO_REG(5) PO_REG(6)
#undef PO_REG
    default: return fail(PO_ERR_UNSUPPORTED, "angular grid too large for the register theta pass");
  }
  return PO_OK;
}

static size_t cols_mma_smem(int ncc, int Rc, int Rp, int Kp) {
  return sizeof(uint4) * (size_t)(Kp / 16) * (ncc / 4) * 32 +
         sizeof(float2) * ((size_t)Rc * (ncc + 1) + (size_t)Rp * (ncc + 1));
}

po_status launch_interp_cols_mma(const float2 *mid, float2 *parent, const int32_t *child_table, int64_t n_parent,
                                 int64_t n_child, int phi, int Rc, int Rp, int Kp, int mirror, const uint32_t *Afrag,
                                 const float4 *trans, int n_slots, int G, int tile, cudaStream_t st) {
  if (n_parent <= 0 || n_slots <= 0) return PO_OK;
  if (Kp % 16 || Kp < (mirror ? 2 * Rc : Rc)) return fail(PO_ERR_INTERNAL, "theta matrix K padding");
  // large parent grids (the root): register accumulators and 16 columns per CTA
  // (half the A traffic); smaller grids: the shared-memory kernel with 8 columns
  // (per-level launch lists of the headline workload: 3.4 vs 5.5 ms at the root,
  // 4.8-9.0 vs 7.1-13.7 ms below it)
  if (mirror && phi % 2 == 0 && tile == 0 && (Rp + 15) / 16 >= 16) {
    const int MT = (Rp + 15) / 16;
    const int mtpw = (MT + 7) / 8;
    const int W = (MT + mtpw - 1) / mtpw;
    int ncc = (phi / 2 > 4 && cols_reg_smem(16, Rc, Kp) <= 96 * 1024) ? 16 : 8;
    const size_t smem = cols_reg_smem(ncc, Rc, Kp);
    if (mtpw <= 6 && smem <= 227 * 1024) {
      const int TW = ncc / 2;
      const int64_t gx = (int64_t)((phi / 2 + TW - 1) / TW) * n_parent * 6;
      if (gx > 2147483647LL || n_slots > 65535) return fail(PO_ERR_UNSUPPORTED, "too many nodes for one launch");
      dim3 grid((unsigned)gx, 1u, (unsigned)n_slots);
      const uint4 *A = (const uint4 *)Afrag;
      if (ncc == 16)
        PO_TRY(launch_cols_reg<16>(grid, W, mtpw, smem, mid, parent, child_table, n_parent, n_child, phi, Rc, Rp, Kp,
                                   A, trans, G, st));
      else
        PO_TRY(launch_cols_reg<8>(grid, W, mtpw, smem, mid, parent, child_table, n_parent, n_child, phi, Rc, Rp, Kp, A,
                                  trans, G, st));
      count_launch();
      PO_CUDA(cudaGetLastError());
      return PO_OK;
    }
  }
  int ncc = 8;
  if (tile == 16 && cols_mma_smem(16, Rc, Rp, Kp) <= 227 * 1024 && (mirror ? phi / 2 : phi) > 4) ncc = 16;
  const size_t smem = cols_mma_smem(ncc, Rc, Rp, Kp);
  if (smem > 227 * 1024) return fail(PO_ERR_UNSUPPORTED, "angular grid too large for the tensor-core interpolation");
  const int TW = mirror ? ncc / 2 : ncc;
  const int span = mirror ? phi / 2 : phi;
  int64_t gx = (int64_t)((span + TW - 1) / TW) * n_parent * 6;
  if (gx > 2147483647LL || n_slots > 65535) return fail(PO_ERR_UNSUPPORTED, "too many nodes for one launch");
  dim3 grid((unsigned)gx, 1u, (unsigned)n_slots);
  if (ncc == 16) {
    k_interp_cols_mma<16><<<grid, 128, smem, st>>>(mid, parent, child_table, n_parent, n_child, phi, Rc, Rp, Kp,
                                                   mirror, (const uint4 *)Afrag, trans, G, 0.f);
  } else {
    k_interp_cols_mma<8><<<grid, 128, smem, st>>>(mid, parent, child_table, n_parent, n_child, phi, Rc, Rp, Kp,
                                                  mirror, (const uint4 *)Afrag, trans, G, 0.f);
  }
  count_launch();
  PO_CUDA(cudaGetLastError());
  return PO_OK;
}

// ----------------------------------------------- transposed theta pass
// Adjoint of k_interp_cols_mma for one child: its parent's adjoint pattern
// times exp(-i k s.(c_child - c_parent)) on the parent grid, then the
// transposed mirrored theta map [A_own^T | A_partner^T] (rows t < Rc, K over
// the parent's own and partner half columns).  Every child writes its own
// output, so there is no reduction.  CTA: one (child, component, slot) and
// NCC complex columns (NCC/2 mirror pairs), 4 warps over the 16-row tiles.
template <int NCC>
__global__ void __launch_bounds__(128) k_interp_cols_adj_mma(
    const float2 *__restrict__ parent_adj, float2 *__restrict__ mid_adj, const int32_t *__restrict__ child_parent,
    const uint32_t *__restrict__ child_prefix, int64_t n_parent, int64_t n_child, int phi, int Rc, int Rp, int Kp,
    const uint4 *__restrict__ Afrag, const float4 *__restrict__ trans, int G) {
  constexpr int NT = NCC / 4;
  constexpr int TW = NCC / 2;
  constexpr int NP = NCC + 1;  // padded row stride of the staged tile
  extern __shared__ uint4 smem_u4[];
  const int KS = Kp / 16, MT = (Rc + 15) / 16;
  uint4 *Bf = smem_u4;                                   // [KS][NT][32]
  float2 *tile = (float2 *)(Bf + (size_t)KS * NT * 32);  // [Rp][NP]
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, tq = lane & 3;
  const int span = phi / 2;
  const int ntile = (span + TW - 1) / TW;
  const int j0 = (int)(blockIdx.x % ntile) * TW;
  const int64_t cc = blockIdx.x / ntile;
  const int64_t c = cc / 6;
  const int comp = (int)(cc % 6);
  const int slot = blockIdx.z, lam = slot / G;
  auto col_of = [&](int q) { return q < TW ? j0 + q : j0 + (q - TW) + phi / 2; };
  auto ok_of = [&](int q) { return j0 + (q < TW ? q : q - TW) < span; };
  auto partner_of = [&](int q) { return q < TW ? q + TW : q - TW; };
  const int64_t p = child_parent[c];
  const int o = (int)(child_prefix[c] & 7u);
  const float sgx = (o & 1) ? 1.f : -1.f, sgy = (o & 2) ? -1.f : 1.f, sgz = (o & 4) ? -1.f : 1.f;
  const float4 *tr = trans + (int64_t)lam * Rp * phi;
  const float2 *src = parent_adj + (((int64_t)slot * n_parent + p) * 6 + comp) * (int64_t)Rp * phi;
  for (int e = threadIdx.x; e < Rp * NCC; e += blockDim.x) {
    const int r = e / NCC, q = e - r * NCC;
    float2 v = make_float2(0.f, 0.f);
    if (ok_of(q)) {
      const int j = col_of(q);
      const float2 a = src[(int64_t)r * phi + j];
      const float4 rr = tr[(int64_t)r * phi + j];
      float sn, cs;
      sincos_small(fmaf(sgx, rr.x, fmaf(sgy, rr.y, sgz * rr.z)), &sn, &cs);
      v = make_float2(a.x * cs + a.y * sn, a.y * cs - a.x * sn);  // a * exp(-i ph)
    }
    tile[r * NP + q] = v;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < KS * NT * 32; e += blockDim.x) {
    const int ln = e & 31, nt = (e >> 5) % NT, ks = (e >> 5) / NT;
    const int n = nt * 8 + (ln >> 2), q = n >> 1, part = n & 1;
    const int kb = ks * 16 + 2 * (ln & 3);
    float v[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int kk = kb + (u & 1) + (u >> 1) * 8;
      float2 x = make_float2(0.f, 0.f);
      if (kk < Rp) x = tile[kk * NP + q];
      else if (kk < 2 * Rp) x = tile[(kk - Rp) * NP + partner_of(q)];
      v[u] = part ? x.y : x.x;
    }
    uint32_t h0, l0, h1, l1;
    split_bf16x2(v[0], v[1], h0, l0);
    split_bf16x2(v[2], v[3], h1, l1);
    Bf[e] = make_uint4(h0, h1, l0, l1);
  }
  __syncthreads();
  float2 *dst = mid_adj + (((int64_t)slot * n_child + c) * 6 + comp) * (int64_t)Rc * phi;
  for (int mt = warp; mt < MT; mt += 4) {
    float d[NT][4];
#pragma unroll
    for (int nt = 0; nt < NT; ++nt) d[nt][0] = d[nt][1] = d[nt][2] = d[nt][3] = 0.f;
    const uint4 *ap = Afrag + ((size_t)mt * KS) * 64 + lane * 2;
    uint4 nh = __ldg(ap), nl = __ldg(ap + 1);
    for (int ks = 0; ks < KS; ++ks) {
      const uint4 ah = nh, al = nl;
      if (ks + 1 < KS) {
        nh = __ldg(ap + (size_t)(ks + 1) * 64);
        nl = __ldg(ap + (size_t)(ks + 1) * 64 + 1);
      }
      const uint32_t a_hi[4] = {ah.x, ah.y, ah.z, ah.w}, a_lo[4] = {al.x, al.y, al.z, al.w};
#pragma unroll
      for (int nt = 0; nt < NT; ++nt) {
        const uint4 b = Bf[((size_t)ks * NT + nt) * 32 + lane];
        const uint32_t b_hi[2] = {b.x, b.y}, b_lo[2] = {b.z, b.w};
        mma_bf16(d[nt], a_hi, b_hi);
        mma_bf16(d[nt], a_hi, b_lo);
        mma_bf16(d[nt], a_lo, b_hi);
      }
    }
#pragma unroll
    for (int nt = 0; nt < NT; ++nt) {
      const int q = nt * 4 + tq;
      if (!ok_of(q)) continue;
      const int j = col_of(q);
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int t = mt * 16 + g + 8 * h;
        if (t < Rc) dst[(int64_t)t * phi + j] = make_float2(d[nt][2 * h], d[nt][2 * h + 1]);
      }
    }
  }
}

static size_t cols_adj_smem(int ncc, int Rp, int Kp) {
  return sizeof(uint4) * (size_t)(Kp / 16) * (ncc / 4) * 32 + sizeof(float2) * (size_t)Rp * (ncc + 1);
}

po_status launch_interp_cols_adj_mma(const float2 *parent_adj, float2 *mid_adj, const int32_t *child_parent,
                                     const uint32_t *child_prefix, int64_t n_parent, int64_t n_child, int phi, int Rc,
                                     int Rp, int Kp, const uint32_t *Afrag, const float4 *trans, int n_slots, int G,
                                     cudaStream_t st) {
  if (n_child <= 0 || n_slots <= 0) return PO_OK;
  if (Kp % 16 || Kp < 2 * Rp) return fail(PO_ERR_INTERNAL, "adjoint theta matrix K padding");
  if (phi % 2) return fail(PO_ERR_INTERNAL, "mirrored storage needs an even phi grid");
  int ncc = 16;
  if (cols_adj_smem(ncc, Rp, Kp) > 100 * 1024 || phi / 2 <= 4) ncc = 8;
  const size_t smem = cols_adj_smem(ncc, Rp, Kp);
  if (smem > 227 * 1024) return fail(PO_ERR_UNSUPPORTED, "angular grid too large for the adjoint theta pass");
  const int TW = ncc / 2;
  int64_t gx = (int64_t)((phi / 2 + TW - 1) / TW) * n_child * 6;
  if (gx > 2147483647LL || n_slots > 65535) return fail(PO_ERR_UNSUPPORTED, "too many nodes for one launch");
  dim3 grid((unsigned)gx, 1u, (unsigned)n_slots);
  if (ncc == 16) {
    k_interp_cols_adj_mma<16><<<grid, 128, smem, st>>>(parent_adj, mid_adj, child_parent, child_prefix, n_parent,
                                                       n_child, phi, Rc, Rp, Kp, (const uint4 *)Afrag, trans, G);
  } else {
    k_interp_cols_adj_mma<8><<<grid, 128, smem, st>>>(parent_adj, mid_adj, child_parent, child_prefix, n_parent,
                                                      n_child, phi, Rc, Rp, Kp, (const uint4 *)Afrag, trans, G);
  }
  count_launch();
  PO_CUDA(cudaGetLastError());
  return PO_OK;
}

// ---------------------------------------------------------------- row pass
// The phi half of interpFFT (interpolation.h:17-45) is out[r][j'] =
// sum_j K_{Phi_c}(j'/Phi_p - j/Phi_c) in[r][j] for every stored row r.  As a
// GEMM the A operand stacks 8 complex rows as 16 real rows (real parts in
// rows 0-7, imaginary parts in rows 8-15), so a lane's A fragment is two
// contiguous 16-byte loads of one input row and its D fragment is two
// complex outputs of one output row.  B = the level's phi matrix, transposed,
// in fragment order  Bm[ntile][kstep][lane] = {hi0, hi1, lo0, lo1}.
size_t phi_matrix_words(int Pp, int Kp) { return (size_t)((Pp + 7) / 8) * (Kp / 16) * 32 * 4; }

// B operand of the row kernel for out[n] = sum_k W(n, k) in[k], n < Pout, k < Kin
template <typename F>
static void b_fragments(int Pout, int Kin, int Kp, F W, std::vector<uint32_t> &out) {
  const int NTt = (Pout + 7) / 8, KS = Kp / 16;
  out.assign(phi_matrix_words(Pout, Kp), 0u);
  for (int nt = 0; nt < NTt; ++nt)
    for (int ks = 0; ks < KS; ++ks)
      for (int lane = 0; lane < 32; ++lane) {
        const int n = nt * 8 + (lane >> 2), kb = ks * 16 + 2 * (lane & 3);
        const int ks4[4] = {kb, kb + 1, kb + 8, kb + 9};
        uint16_t h[4], l[4];
        for (int u = 0; u < 4; ++u) {
          double v = (n < Pout && ks4[u] < Kin) ? W(n, ks4[u]) : 0.0;
          h[u] = bf16_rne((float)v);
          l[u] = bf16_rne((float)(v - (double)bf16_to_f(h[u])));
        }
        uint32_t *dst = &out[(((size_t)nt * KS + ks) * 32 + lane) * 4];
        dst[0] = (uint32_t)h[0] | ((uint32_t)h[1] << 16);
        dst[1] = (uint32_t)h[2] | ((uint32_t)h[3] << 16);
        dst[2] = (uint32_t)l[0] | ((uint32_t)l[1] << 16);
        dst[3] = (uint32_t)l[2] | ((uint32_t)l[3] << 16);
      }
}

void build_phi_matrix(int Pc, int Pp, int Kp, std::vector<uint32_t> &out) {
  b_fragments(Pp, Pc, Kp, [&](int n, int k) { return trig_kernel(Pc, (double)n / Pp - (double)k / Pc); }, out);
}

// transpose of the phi map: child column j (< Pc) from parent columns j' (< Pp)
void build_phi_matrix_adj(int Pc, int Pp, int Kp, std::vector<uint32_t> &out) {
  b_fragments(Pc, Pp, Kp, [&](int j, int jp) { return trig_kernel(Pc, (double)jp / Pp - (double)j / Pc); }, out);
}

// One warp per block of 8 rows; n-tiles in groups of kRowNG (accumulators in
// registers); the B fragments come from shared memory when they fit.
constexpr int kRowNG = 8;
__global__ void __launch_bounds__(128) k_interp_rows_mma(const float2 *__restrict__ src, float2 *__restrict__ dst,
                                                         int64_t nrows, int Pc, int Pp, int Kp,
                                                         const uint4 *__restrict__ Bm, int b_in_smem) {
  extern __shared__ uint4 bsm[];
  const int KS = Kp / 16, NTt = (Pp + 7) / 8;
  if (b_in_smem) {
    for (int e = threadIdx.x; e < NTt * KS * 32; e += blockDim.x) bsm[e] = Bm[e];
    __syncthreads();
  }
  const uint4 *B = b_in_smem ? bsm : Bm;
  const int lane = threadIdx.x & 31, g = lane >> 2, tq = lane & 3;
  const int64_t nblk = (nrows + 7) / 8;
  for (int64_t blk = (int64_t)blockIdx.x * 4 + (threadIdx.x >> 5); blk < nblk; blk += (int64_t)gridDim.x * 4) {
    const int64_t r = blk * 8 + g;
    const bool rok = r < nrows;
    const float2 *in = src + (rok ? r : 0) * (int64_t)Pc;
    float2 *out = dst + (rok ? r : 0) * (int64_t)Pp;
    for (int ng = 0; ng < NTt; ng += kRowNG) {
      float acc[kRowNG][4];
#pragma unroll
      for (int q = 0; q < kRowNG; ++q) acc[q][0] = acc[q][1] = acc[q][2] = acc[q][3] = 0.f;
      for (int ks = 0; ks < KS; ++ks) {
        const int k0 = ks * 16 + 2 * tq;
        float2 v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int k = k0 + (u & 1) + (u >> 1) * 8;
          v[u] = (rok && k < Pc) ? in[k] : make_float2(0.f, 0.f);
        }
        uint32_t ahi[4], alo[4];
        split_bf16x2(v[0].x, v[1].x, ahi[0], alo[0]);  // row g (real parts), k0, k0+1
        split_bf16x2(v[0].y, v[1].y, ahi[1], alo[1]);  // row g+8 (imaginary parts)
        split_bf16x2(v[2].x, v[3].x, ahi[2], alo[2]);  // row g, k0+8, k0+9
        split_bf16x2(v[2].y, v[3].y, ahi[3], alo[3]);
#pragma unroll
        for (int q = 0; q < kRowNG; ++q) {
          const int nt = ng + q;
          if (nt >= NTt) break;
          const uint4 bv = B[((size_t)nt * KS + ks) * 32 + lane];
          const uint32_t bhi[2] = {bv.x, bv.y}, blo[2] = {bv.z, bv.w};
          mma_bf16(acc[q], ahi, bhi);
          mma_bf16(acc[q], ahi, blo);
          mma_bf16(acc[q], alo, bhi);
        }
      }
      if (rok) {
#pragma unroll
        for (int q = 0; q < kRowNG; ++q) {
          const int j = (ng + q) * 8 + 2 * tq;
          if (j < Pp) out[j] = make_float2(acc[q][0], acc[q][2]);
          if (j + 1 < Pp) out[j + 1] = make_float2(acc[q][1], acc[q][3]);
        }
      }
    }
  }
}

po_status launch_interp_rows_mma(const float2 *src, float2 *dst, int64_t nrows, int Pc, int Pp, int Kp,
                                 const uint32_t *Bm, int sm_count, cudaStream_t st) {
  if (nrows <= 0) return PO_OK;
  if (Kp % 16 || Kp < Pc) return fail(PO_ERR_INTERNAL, "phi matrix K padding");
  const size_t bbytes = sizeof(uint32_t) * phi_matrix_words(Pp, Kp);
  const bool b_smem = bbytes <= 48 * 1024;
  const size_t smem = b_smem ? bbytes : 0;
  int64_t blocks = ((nrows + 7) / 8 + 3) / 4;
  const int64_t cap = (int64_t)sm_count * 16;
  if (blocks > cap) blocks = cap;
  k_interp_rows_mma<<<(unsigned)blocks, 128, smem, st>>>(src, dst, nrows, Pc, Pp, Kp, (const uint4 *)Bm,
                                                         b_smem ? 1 : 0);
  count_launch();
  PO_CUDA(cudaGetLastError());
  return PO_OK;
}

// Opt-in shared-memory limit of every kernel here, set once per device (the
// launchers pick their shared-memory size at run time and must not change
// function attributes while a stream is being captured).
po_status init_interp_mma_attributes(int max_smem) {
  PO_CUDA(cudaFuncSetAttribute(k_interp_cols_mma<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem));
  PO_CUDA(cudaFuncSetAttribute(k_interp_cols_mma<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem));
  PO_CUDA(cudaFuncSetAttribute(k_interp_cols_adj_mma<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem));
  PO_CUDA(cudaFuncSetAttribute(k_interp_cols_adj_mma<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem));
  PO_CUDA(cudaFuncSetAttribute(k_interp_rows_mma, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem));
#define PO_REG_ATTR(N, M) \
  PO_CUDA(cudaFuncSetAttribute(k_interp_cols_reg<N, M>, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem));
  PO_REG_ATTR(8, 1) PO_REG_ATTR(8, 2) PO_REG_ATTR(8, 3) PO_REG_ATTR(8, 4) PO_REG_ATTR(8, 5) PO_REG_ATTR(8, 6)
  PO_REG_ATTR(16, 1) PO_REG_ATTR(16, 2) PO_REG_ATTR(16, 3) PO_REG_ATTR(16, 4) PO_REG_ATTR(16, 5) PO_REG_ATTR(16, 6)
#undef PO_REG_ATTR
  return PO_OK;
}

}  // namespace wavepo
