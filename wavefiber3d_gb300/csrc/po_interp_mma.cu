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
// parent column j is A_own h_j + A_partner h_{j+Phi/2} and column j+Phi/2 is
// A_own h_{j+Phi/2} + A_partner h_j: two GEMMs with K = Rc over the child's
// stored half columns.  Operands are split into bf16 hi + lo parts and
// multiplied as hi*hi + hi*lo + lo*hi with FP32 accumulation (mma.sync
// m16n8k16), which keeps ~16 bits of every operand.  The row (phi) pass writes
// its output already split, in row pairs, so the theta pass loads B fragments
// straight from global memory.  The epilogue multiplies each child's result by
// exp(i k s.(c_child - c_parent)) and sums the children in registers.
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

// Forward theta matrices of one level (double cover), K = rows t < Rc of one
// half column, padded to 16:  A_own[r][t] and A_partner[r][s] (s >= 1).
// Layout [mtile][kstep][u][lane] uint4 with u = own hi, own lo, partner hi,
// partner lo (a lane's four a-registers), so a warp's shared-memory reads of
// one u are 512 contiguous bytes.
size_t theta_pair_words(int Rp, int Kp) { return (size_t)((Rp + 15) / 16) * (Kp / 16) * 4 * 32 * 4; }

void build_theta_matrix(int Tc, int Tp, int Rc, int Rp, int Kp, std::vector<uint32_t> &out) {
  const int nth_c = Tc / 2;
  std::vector<double> Mo((size_t)Rp * Kp, 0.0), Mp((size_t)Rp * Kp, 0.0);
  for (int r = 0; r < Rp; ++r) {
    for (int t = 0; t < Rc; ++t) Mo[(size_t)r * Kp + t] = theta_own(Tc, Tp, r, t);
    for (int s = 1; s < nth_c; ++s) Mp[(size_t)r * Kp + s] = theta_partner(Tc, Tp, r, s);
  }
  std::vector<uint32_t> fo, fp;
  a_fragments(Mo, Rp, Kp, fo);
  a_fragments(Mp, Rp, Kp, fp);
  const int MT = (Rp + 15) / 16, KS = Kp / 16;
  out.assign(theta_pair_words(Rp, Kp), 0u);
  for (int mt = 0; mt < MT; ++mt)
    for (int ks = 0; ks < KS; ++ks)
      for (int lane = 0; lane < 32; ++lane) {
        const uint32_t *so = &fo[(((size_t)mt * KS + ks) * 32 + lane) * 8];
        const uint32_t *sp = &fp[(((size_t)mt * KS + ks) * 32 + lane) * 8];
        const uint32_t *src[4] = {so, so + 4, sp, sp + 4};
        for (int u = 0; u < 4; ++u)
          std::memcpy(&out[((((size_t)mt * KS + ks) * 4 + u) * 32 + lane) * 4], src[u], 16);
      }
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
// (not volatile: a pure function of its operands, so the scheduler may
// interleave independent accumulators)
__device__ __forceinline__ void mma_bf16(float *d, const uint32_t *a, const uint32_t *b) {
  asm(
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

// Theta pass as warp tasks (double cover).  A warp owns one (slot, parent,
// component) and TW = 2 NT own columns j0.. with their partners j0+Phi/2..,
// for the CTA's 16-row tiles mt0 .. mt0+MTW-1 (blockIdx.y selects them).
// mid (from k_interp_rows_mma<true>): per (slot, child, component) rows in
// pairs, [Rc2/2][phi] x {re, im} x {hi pair, lo pair} -- exactly a lane's B
// registers.  The CTA stages its slice of the theta matrices in shared memory
// once; after that warps run independently: B fragments of the next k-step
// (or next child) are loaded while the current one multiplies, and the
// parent tile accumulates in registers across the children.
template <int NT, int MTW>
__global__ void __launch_bounds__(256, 2) k_theta_warp(const uint2 *__restrict__ mid, float2 *__restrict__ parent,
                                                    const int32_t *__restrict__ child_table, int64_t n_parent,
                                                    int64_t n_child, int phi, int Rch, int Rp, int KS, int MT,
                                                    const uint4 *__restrict__ Afrag, const float4 *__restrict__ trans,
                                                    int G, int n_ct, int64_t n_task) {
  constexpr int NO = NT / 2;  // own n-tiles; n-tile NO + i holds the partners of n-tile i
  constexpr int TW = 4 * NO;  // own complex columns per warp
  extern __shared__ uint4 sA[];  // [MTW][KS][4][32]
  const int mt0 = blockIdx.y * MTW;
  const int nmt = MT - mt0 < MTW ? MT - mt0 : MTW;
  {
    // tiles past MT (last group) are zero, so the k-loop below needs no guard
    const uint4 *src = Afrag + (size_t)mt0 * KS * 128;
    const int n = nmt * KS * 128;
    for (int e = threadIdx.x; e < MTW * KS * 128; e += blockDim.x)
      sA[e] = e < n ? __ldg(src + e) : make_uint4(0u, 0u, 0u, 0u);
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, tq = lane & 3;
  const int64_t task = (int64_t)blockIdx.x * (blockDim.x >> 5) + warp;
  if (task >= n_task) return;
  const int ct = (int)(task % n_ct);
  int64_t rest = task / n_ct;
  const int comp = (int)(rest % 6);
  rest /= 6;
  const int64_t p = rest % n_parent;
  const int slot = (int)(rest / n_parent), lam = slot / G;
  const int span = phi / 2, j0 = ct * TW, part = g & 1;
  const int64_t pat = (int64_t)Rch * phi * 2;  // uint2 words of one child pattern component
  const uint2 *mbase = mid + ((int64_t)slot * n_child * 6 + comp) * pat;
  const int32_t cl = lane < 8 ? child_table[p * 8 + lane] : -1;
  unsigned rem = __ballot_sync(0xffffffffu, cl >= 0);  // children present (bits 0..7)
  // B operand of k-step ks of one child: n-tile nt, k rows 2 tq, 2 tq + 1 (pair tq) and + 8 (pair tq + 4)
  auto load_b = [&](const uint2 *m, int ks, uint32_t (&h)[NT][2], uint32_t (&l)[NT][2]) {
#pragma unroll
    for (int nt = 0; nt < NT; ++nt) {
      const int q = (nt % NO) * 4 + (g >> 1);
      const bool ok = j0 + q < span;
      const int col = j0 + q + (nt < NO ? 0 : span);
#pragma unroll
      for (int hh = 0; hh < 2; ++hh) {
        const int tp = ks * 8 + tq + 4 * hh;
        uint2 u = make_uint2(0u, 0u);
        if (ok && tp < Rch) u = __ldg(m + ((int64_t)tp * phi + col) * 2 + part);
        h[nt][hh] = u.x;
        l[nt][hh] = u.y;
      }
    }
  };
  auto child_ptr = [&](int o) { return mbase + (int64_t)__shfl_sync(0xffffffffu, cl, o) * 6 * pat; };
  float acc[MTW][NT][4];
#pragma unroll
  for (int i = 0; i < MTW; ++i)
#pragma unroll
    for (int nt = 0; nt < NT; ++nt) acc[i][nt][0] = acc[i][nt][1] = acc[i][nt][2] = acc[i][nt][3] = 0.f;
  const float4 *tr = trans + (int64_t)lam * Rp * phi;
  bool more = rem != 0;
  int o = more ? __ffs(rem) - 1 : 0;
  rem &= rem - 1;
  const uint2 *m = child_ptr(o);
  uint32_t nh[NT][2] = {}, nl[NT][2] = {};
  if (more) load_b(m, 0, nh, nl);
  while (more) {
    float d[MTW][NT][4];
#pragma unroll
    for (int i = 0; i < MTW; ++i)
#pragma unroll
      for (int nt = 0; nt < NT; ++nt) d[i][nt][0] = d[i][nt][1] = d[i][nt][2] = d[i][nt][3] = 0.f;
    int o_next = o;
    const uint2 *m_next = m;
    for (int ks = 0; ks < KS; ++ks) {
      uint32_t bh[NT][2], bl[NT][2];
#pragma unroll
      for (int nt = 0; nt < NT; ++nt) {
        bh[nt][0] = nh[nt][0];
        bh[nt][1] = nh[nt][1];
        bl[nt][0] = nl[nt][0];
        bl[nt][1] = nl[nt][1];
      }
      if (ks + 1 < KS) {
        load_b(m, ks + 1, nh, nl);
      } else if (rem) {
        o_next = __ffs(rem) - 1;
        m_next = child_ptr(o_next);
        load_b(m_next, 0, nh, nl);
      }
      // one basic block: MTW x NT independent accumulators, each product
      // term issued across all of them before the next
#pragma unroll
      for (int i = 0; i < MTW; ++i) {
        const uint4 *a = sA + (size_t)(i * KS + ks) * 128 + lane;
        const uint4 oh = a[0], ol = a[32], ph = a[64], pl = a[96];
        const uint32_t aoh[4] = {oh.x, oh.y, oh.z, oh.w}, aol[4] = {ol.x, ol.y, ol.z, ol.w};
        const uint32_t aph[4] = {ph.x, ph.y, ph.z, ph.w}, apl[4] = {pl.x, pl.y, pl.z, pl.w};
#pragma unroll
        for (int nt = 0; nt < NT; ++nt) {
          const int nx = nt < NO ? nt + NO : nt - NO;  // partner n-tile
          const uint32_t bsh[2] = {bh[nt][0], bh[nt][1]}, bsl[2] = {bl[nt][0], bl[nt][1]};
          const uint32_t bxh[2] = {bh[nx][0], bh[nx][1]}, bxl[2] = {bl[nx][0], bl[nx][1]};
          mma_bf16(d[i][nt], aoh, bsh);
          mma_bf16(d[i][nt], aph, bxh);
          mma_bf16(d[i][nt], aoh, bsl);
          mma_bf16(d[i][nt], aph, bxl);
          mma_bf16(d[i][nt], aol, bsh);
          mma_bf16(d[i][nt], apl, bxh);
        }
      }
    }
    // translation of child octant o and the child sum.  Rows >= Rp (zero
    // rows of A) and columns past the half span (zero B) hold exact zeros, so
    // every element runs unguarded with its table index clamped in range:
    // one basic block of independent chains.
    const float sgx = (o & 1) ? 1.f : -1.f, sgy = (o & 2) ? -1.f : 1.f, sgz = (o & 4) ? -1.f : 1.f;
#pragma unroll
    for (int i = 0; i < MTW; ++i) {
#pragma unroll
      for (int nt = 0; nt < NT; ++nt) {
        const int q = (nt % NO) * 4 + tq;
        const int j = (j0 + q < span ? j0 + q : span - 1) + (nt < NO ? 0 : span);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int r0 = (mt0 + i) * 16 + g + 8 * h;
          const int r = r0 < Rp ? r0 : Rp - 1;
          const float4 rr = __ldg(tr + (int64_t)r * phi + j);
          float sn, cs;
          sincos_small(fmaf(sgx, rr.x, fmaf(sgy, rr.y, sgz * rr.z)), &sn, &cs);
          const float vr = d[i][nt][2 * h], vi = d[i][nt][2 * h + 1];
          acc[i][nt][2 * h] += vr * cs - vi * sn;
          acc[i][nt][2 * h + 1] += vr * sn + vi * cs;
        }
      }
    }
    more = rem != 0;
    if (more) {
      o = o_next;
      m = m_next;
      rem &= rem - 1;
    }
  }
  float2 *out = parent + (((int64_t)slot * n_parent + p) * 6 + comp) * (int64_t)Rp * phi;
#pragma unroll
  for (int i = 0; i < MTW; ++i) {
    if (i >= nmt) break;
#pragma unroll
    for (int nt = 0; nt < NT; ++nt) {
      const int q = (nt % NO) * 4 + tq;
      if (j0 + q >= span) continue;
      const int j = j0 + q + (nt < NO ? 0 : span);
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int r = (mt0 + i) * 16 + g + 8 * h;
        if (r < Rp) out[(int64_t)r * phi + j] = make_float2(acc[i][nt][2 * h], acc[i][nt][2 * h + 1]);
      }
    }
  }
}

template <int NT, int MTW>
static void launch_theta_warp(dim3 grid, size_t smem, const uint2 *mid, float2 *parent, const int32_t *child_table,
                              int64_t n_parent, int64_t n_child, int phi, int Rch, int Rp, int KS, int MT,
                              const uint4 *A, const float4 *trans, int G, int n_ct, int64_t n_task, cudaStream_t st) {
  k_theta_warp<NT, MTW><<<grid, 256, smem, st>>>(mid, parent, child_table, n_parent, n_child, phi, Rch, Rp, KS, MT, A,
                                                 trans, G, n_ct, n_task);
}

po_status launch_interp_cols_mma(const uint2 *mid, float2 *parent, const int32_t *child_table, int64_t n_parent,
                                 int64_t n_child, int phi, int Rc, int Rp, int Kp, const uint32_t *Afrag,
                                 const float4 *trans, int n_slots, int G, int tile, cudaStream_t st) {
  if (n_parent <= 0 || n_slots <= 0) return PO_OK;
  const int Rc2 = Rc + (Rc & 1);
  if (Kp % 16 || Kp < Rc2) return fail(PO_ERR_INTERNAL, "theta matrix K padding");
  if (phi % 2) return fail(PO_ERR_INTERNAL, "mirrored storage needs an even phi grid");
  const int KS = Kp / 16, MT = (Rp + 15) / 16;
  const int NT = tile == 16 ? 4 : 2;
  // 16-row tiles per warp: up to 4 (measured on the headline workload: caps of
  // 1 / 2 / 4 tiles gave 23.5 / 18.4 / 15.1 ms for the theta passes of a solve)
  const int cap = NT == 4 ? 2 : 4;
  const int nmg = (MT + cap - 1) / cap;
  const int MTW = (MT + nmg - 1) / nmg;
  const size_t smem = sizeof(uint4) * (size_t)MTW * KS * 128;
  if (smem > 227 * 1024) return fail(PO_ERR_UNSUPPORTED, "angular grid too large for the tensor-core interpolation");
  const int TW = 2 * NT;
  const int n_ct = (phi / 2 + TW - 1) / TW;
  const int64_t n_task = (int64_t)n_slots * n_parent * 6 * n_ct;
  const int64_t gx = (n_task + 7) / 8;
  if (gx > 2147483647LL || nmg > 65535) return fail(PO_ERR_UNSUPPORTED, "too many nodes for one launch");
  dim3 grid((unsigned)gx, (unsigned)nmg, 1u);
  const uint4 *A = (const uint4 *)Afrag;
#define PO_TW(N, M)                                                                                                 \
  if (NT == N && MTW == M) {                                                                                       \
    launch_theta_warp<N, M>(grid, smem, mid, parent, child_table, n_parent, n_child, phi, Rc2 / 2, Rp, KS, MT, A, \
                            trans, G, n_ct, n_task, st);                                                            \
  } else
  PO_TW(2, 1) PO_TW(2, 2) PO_TW(2, 3) PO_TW(2, 4) PO_TW(4, 1) PO_TW(4, 2) {
    return fail(PO_ERR_INTERNAL, "theta pass variant");
  }
#undef PO_TW
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
// PACK (forward pass feeding k_theta_warp): rows are indexed over patterns of
// Rc2 = Rc rounded up to even rows (row Rc of an odd Rc is a zero row), and the
// output is split into bf16 hi + lo and stored in row pairs: per pattern
// [Rc2/2][Pp] uint4 {re hi pair, re lo pair, im hi pair, im lo pair}, each pair
// holding rows 2 tp (low half) and 2 tp + 1.  Lane g and lane g^1 (4 apart)
// hold the two rows of a pair and swap one column each, so every lane stores
// one 16-byte word.
constexpr int kRowNG = 8;
template <bool PACK>
__global__ void __launch_bounds__(128) k_interp_rows_mma(const float2 *__restrict__ src, void *__restrict__ dst_,
                                                         int64_t nrows, int Rc, int Pc, int Pp, int Kp,
                                                         const uint4 *__restrict__ Bm, int b_in_smem) {
  extern __shared__ uint4 bsm[];
  const int KS = Kp / 16, NTt = (Pp + 7) / 8;
  if (b_in_smem) {
    for (int e = threadIdx.x; e < NTt * KS * 32; e += blockDim.x) bsm[e] = Bm[e];
    __syncthreads();
  }
  const uint4 *B = b_in_smem ? bsm : Bm;
  const int lane = threadIdx.x & 31, g = lane >> 2, tq = lane & 3;
  const int Rc2 = Rc + (Rc & 1);
  const int64_t nblk = (nrows + 7) / 8;
  for (int64_t blk = (int64_t)blockIdx.x * 4 + (threadIdx.x >> 5); blk < nblk; blk += (int64_t)gridDim.x * 4) {
    const int64_t r = blk * 8 + g;
    const bool rok = r < nrows;
    int64_t srow = r;
    bool in_ok = rok;
    if (PACK) {
      const int64_t pattern = r / Rc2;
      const int t = (int)(r - pattern * Rc2);
      srow = pattern * Rc + t;
      in_ok = rok && t < Rc;
    }
    const float2 *in = src + (in_ok ? srow : 0) * (int64_t)Pc;
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
          v[u] = (in_ok && k < Pc) ? in[k] : make_float2(0.f, 0.f);
        }
        uint32_t ahi[4], alo[4];
        split_bf16x2(v[0].x, v[1].x, ahi[0], alo[0]);  // row g (real parts), k0, k0+1
        split_bf16x2(v[0].y, v[1].y, ahi[1], alo[1]);  // row g+8 (imaginary parts)
        split_bf16x2(v[2].x, v[3].x, ahi[2], alo[2]);  // row g, k0+8, k0+9
        split_bf16x2(v[2].y, v[3].y, ahi[3], alo[3]);
        if (ng + kRowNG <= NTt) {  // full group: one basic block, 8 independent accumulators
          uint4 bv[kRowNG];
#pragma unroll
          for (int q = 0; q < kRowNG; ++q) bv[q] = B[((size_t)(ng + q) * KS + ks) * 32 + lane];
#pragma unroll
          for (int q = 0; q < kRowNG; ++q) {
            const uint32_t bhi[2] = {bv[q].x, bv[q].y};
            mma_bf16(acc[q], ahi, bhi);
          }
#pragma unroll
          for (int q = 0; q < kRowNG; ++q) {
            const uint32_t blo[2] = {bv[q].z, bv[q].w};
            mma_bf16(acc[q], ahi, blo);
          }
#pragma unroll
          for (int q = 0; q < kRowNG; ++q) {
            const uint32_t bhi[2] = {bv[q].x, bv[q].y};
            mma_bf16(acc[q], alo, bhi);
          }
        } else {
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
      }
      if (PACK) {
        uint4 *dst = (uint4 *)dst_;
        const bool odd = g & 1;
        const int64_t pair_row = r >> 1;  // = pattern * Rc2/2 + t/2, Rc2 even
#pragma unroll
        for (int q = 0; q < kRowNG; ++q) {
          if (ng + q >= NTt) break;
          // even g keeps column j (rows t, t+1 from the neighbour), odd g keeps j+1
          const float sr = odd ? acc[q][0] : acc[q][1], si = odd ? acc[q][2] : acc[q][3];
          const float rr = __shfl_xor_sync(0xffffffffu, sr, 4), ri = __shfl_xor_sync(0xffffffffu, si, 4);
          const float r0 = odd ? rr : acc[q][0], i0 = odd ? ri : acc[q][2];  // row t (even)
          const float r1 = odd ? acc[q][1] : rr, i1 = odd ? acc[q][3] : ri;  // row t+1
          const int j = (ng + q) * 8 + 2 * tq + (odd ? 1 : 0);
          uint32_t hr, lr, hi, li;
          split_bf16x2(r0, r1, hr, lr);
          split_bf16x2(i0, i1, hi, li);
          if (rok && j < Pp) dst[pair_row * Pp + j] = make_uint4(hr, lr, hi, li);
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
  }
}

static po_status launch_rows(bool pack, const float2 *src, void *dst, int64_t nrows, int Rc, int Pc, int Pp, int Kp,
                             const uint32_t *Bm, int sm_count, cudaStream_t st) {
  if (nrows <= 0) return PO_OK;
  if (Kp % 16 || Kp < Pc) return fail(PO_ERR_INTERNAL, "phi matrix K padding");
  const size_t bbytes = sizeof(uint32_t) * phi_matrix_words(Pp, Kp);
  const bool b_smem = bbytes <= 48 * 1024;
  const size_t smem = b_smem ? bbytes : 0;
  int64_t blocks = ((nrows + 7) / 8 + 3) / 4;
  const int64_t cap = (int64_t)sm_count * 16;
  if (blocks > cap) blocks = cap;
  if (pack)
    k_interp_rows_mma<true><<<(unsigned)blocks, 128, smem, st>>>(src, dst, nrows, Rc, Pc, Pp, Kp, (const uint4 *)Bm,
                                                                 b_smem ? 1 : 0);
  else
    k_interp_rows_mma<false><<<(unsigned)blocks, 128, smem, st>>>(src, dst, nrows, Rc, Pc, Pp, Kp,
                                                                  (const uint4 *)Bm, b_smem ? 1 : 0);
  count_launch();
  PO_CUDA(cudaGetLastError());
  return PO_OK;
}

po_status launch_interp_rows_mma(const float2 *src, float2 *dst, int64_t nrows, int Pc, int Pp, int Kp,
                                 const uint32_t *Bm, int sm_count, cudaStream_t st) {
  return launch_rows(false, src, dst, nrows, 0, Pc, Pp, Kp, Bm, sm_count, st);
}

po_status launch_interp_rows_packed(const float2 *src, uint2 *dst, int64_t n_patterns, int Rc, int Pc, int Pp,
                                    int Kp, const uint32_t *Bm, int sm_count, cudaStream_t st) {
  const int64_t nrows = n_patterns * (int64_t)(Rc + (Rc & 1));
  return launch_rows(true, src, dst, nrows, Rc, Pc, Pp, Kp, Bm, sm_count, st);
}

// Opt-in shared-memory limit of every kernel here, set once per device (the
// launchers pick their shared-memory size at run time and must not change
// function attributes while a stream is being captured).
po_status init_interp_mma_attributes(int max_smem) {
  PO_CUDA(cudaFuncSetAttribute(k_interp_cols_adj_mma<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem));
  PO_CUDA(cudaFuncSetAttribute(k_interp_cols_adj_mma<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem));
  PO_CUDA(cudaFuncSetAttribute(k_interp_rows_mma<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem));
  PO_CUDA(cudaFuncSetAttribute(k_interp_rows_mma<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem));
#define PO_TW_ATTR(N, M) \
  PO_CUDA(cudaFuncSetAttribute(k_theta_warp<N, M>, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem));
  PO_TW_ATTR(2, 1) PO_TW_ATTR(2, 2) PO_TW_ATTR(2, 3) PO_TW_ATTR(2, 4)
  PO_TW_ATTR(4, 1) PO_TW_ATTR(4, 2)
#undef PO_TW_ATTR
  return PO_OK;
}

}  // namespace wavepo
