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
// parent column j is A_own h_j + A_partner h_j' and its mirror j' = j + Phi/2
// is A_own h_j' + A_partner h_j.  In sums and differences S = h_j + h_j',
// D = h_j - h_j' this is two GEMMs with K = Rc instead of four:
//   U = A_plus S,  V = A_minus D,  A_plus/minus = (A_own +- A_partner) / 2,
//   Y_j = U + V,  Y_j' = U - V.
// The row (phi) pass orders its output columns as (j, j') pairs and writes S
// and D, already split into bf16 hi + lo parts in row pairs, so the theta pass
// loads B fragments straight from global memory.  Products are hi*hi + hi*lo
// + lo*hi with FP32 accumulation (mma.sync m16n8k16), which keeps ~16 bits of
// every operand.  The epilogue multiplies each child's result by
// exp(i k s.(c_child - c_parent)) and sums the children in registers.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "po_common.cuh"
#include "po_internal.h"
#include "po_kernels.h"
#include "po_rows_block.cuh"

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
// half column, padded to 16:  A_plus/minus[r][t] = (A_own[r][t] +- A_partner[r][t]) / 2
// with A_partner[r][s] nonzero for 1 <= s < Tc/2.  Layout [mtile][kstep][u][lane]
// uint4 with u = plus hi, plus lo, minus hi, minus lo (a lane's four a-registers),
// so a warp's shared-memory reads of one u are 512 contiguous bytes.
size_t theta_pair_words(int Rp, int Kp) { return (size_t)((Rp + 15) / 16) * (Kp / 16) * 4 * 32 * 4; }

// A_plus / A_minus of one level as dense FP64 [Rp][ld] (columns t < Rc).
// Without the mirror (the reference's pi-periodic theta, all T rows stored) the
// partner term vanishes and A_plus = A_minus = A_own / 2, so that
// Y_j = U + V = A_own h_j and Y_j' = U - V = A_own h_j' with the same kernels.
void theta_plus_minus(int Tc, int Tp, int Rc, int Rp, int ld, std::vector<double> &Mplus,
                      std::vector<double> &Mminus, bool mirror) {
  const int nth_c = mirror ? Tc / 2 : 0;
  Mplus.assign((size_t)Rp * ld, 0.0);
  Mminus.assign((size_t)Rp * ld, 0.0);
  for (int r = 0; r < Rp; ++r)
    for (int t = 0; t < Rc; ++t) {
      const double own = theta_own(Tc, Tp, r, t);
      const double partner = (t >= 1 && t < nth_c) ? theta_partner(Tc, Tp, r, t) : 0.0;
      Mplus[(size_t)r * ld + t] = 0.5 * (own + partner);
      Mminus[(size_t)r * ld + t] = 0.5 * (own - partner);
    }
}

void build_theta_matrix(int Tc, int Tp, int Rc, int Rp, int Kp, std::vector<uint32_t> &out, bool mirror) {
  std::vector<double> Mplus, Mminus;
  theta_plus_minus(Tc, Tp, Rc, Rp, Kp, Mplus, Mminus, mirror);
  std::vector<uint32_t> fp, fm;
  a_fragments(Mplus, Rp, Kp, fp);
  a_fragments(Mminus, Rp, Kp, fm);
  const int MT = (Rp + 15) / 16, KS = Kp / 16;
  out.assign(theta_pair_words(Rp, Kp), 0u);
  for (int mt = 0; mt < MT; ++mt)
    for (int ks = 0; ks < KS; ++ks)
      for (int lane = 0; lane < 32; ++lane) {
        const uint32_t *sp = &fp[(((size_t)mt * KS + ks) * 32 + lane) * 8];
        const uint32_t *sm = &fm[(((size_t)mt * KS + ks) * 32 + lane) * 8];
        const uint32_t *src[4] = {sp, sp + 4, sm, sm + 4};
        for (int u = 0; u < 4; ++u)
          std::memcpy(&out[((((size_t)mt * KS + ks) * 4 + u) * 32 + lane) * 4], src[u], 16);
      }
}

// Transposed theta matrices of one level (double cover), rows t < Rc of the
// child, K = parent rows r < Rp padded to 16:  A_plus/minus^T[t][r] =
// (A_own[r][t] +- A_partner[r][t]) / 2, in the layout of build_theta_matrix
// ([mtile][kstep][u][lane] uint4, u = plus hi, plus lo, minus hi, minus lo).
void build_theta_matrix_adj(int Tc, int Tp, int Rc, int Rp, int Kp, std::vector<uint32_t> &out) {
  const int nth_c = Tc / 2;
  std::vector<double> Mplus((size_t)Rc * Kp, 0.0), Mminus((size_t)Rc * Kp, 0.0);
  for (int t = 0; t < Rc; ++t)
    for (int r = 0; r < Rp; ++r) {
      const double own = theta_own(Tc, Tp, r, t);
      const double partner = (t >= 1 && t < nth_c) ? theta_partner(Tc, Tp, r, t) : 0.0;
      Mplus[(size_t)t * Kp + r] = 0.5 * (own + partner);
      Mminus[(size_t)t * Kp + r] = 0.5 * (own - partner);
    }
  std::vector<uint32_t> fp, fm;
  a_fragments(Mplus, Rc, Kp, fp);
  a_fragments(Mminus, Rc, Kp, fm);
  const int MT = (Rc + 15) / 16, KS = Kp / 16;
  out.assign(theta_pair_words(Rc, Kp), 0u);
  for (int mt = 0; mt < MT; ++mt)
    for (int ks = 0; ks < KS; ++ks)
      for (int lane = 0; lane < 32; ++lane) {
        const uint32_t *sp = &fp[(((size_t)mt * KS + ks) * 32 + lane) * 8];
        const uint32_t *sm = &fm[(((size_t)mt * KS + ks) * 32 + lane) * 8];
        const uint32_t *src[4] = {sp, sp + 4, sm, sm + 4};
        for (int u = 0; u < 4; ++u)
          std::memcpy(&out[((((size_t)mt * KS + ks) * 4 + u) * 32 + lane) * 4], src[u], 16);
      }
}

// ---------------------------------------------------------- device side
// Theta pass as warp tasks (double cover).  A warp owns one (slot, parent,
// component) and TW = 4 NPT column pairs (j, j + Phi/2), j = j0.., for the
// CTA's 16-row tiles mt0 .. mt0+MTW-1 (blockIdx.y selects them).
// ODD (reference theta mode, odd parent phi grid): the pairs are (j, j + H),
// H = (Phi + 1)/2, whose partner is not at phi + pi: its translation phase
// comes from its own table entry, and the phantom partner Phi is not stored.
// mid (from k_interp_rows_mma<1>): per (slot, child, component)
// [Rc2/2][(Phi+1)/2][re, im] uint4 {S hi pair, S lo pair, D hi pair, D lo pair} --
// a lane's B registers for the S and the D n-tile in one 16-byte load.  The
// CTA stages its slice of the theta matrices in shared memory once; after
// that warps run independently: B fragments of the next k-step (or next
// child) are loaded while the current one multiplies, and the parent tile
// accumulates in registers across the children.
template <int NPT, int MTW, bool ODD>
__global__ void __launch_bounds__(256, (NPT == 1 && MTW <= 2) ? 3 : 2) k_theta_warp(const uint4 *__restrict__ mid, float2 *__restrict__ parent,
                                                       const int32_t *__restrict__ child_table, int64_t n_parent,
                                                       int64_t n_child, int phi, int Rch, int Rp, int KS, int MT,
                                                       const uint4 *__restrict__ Afrag,
                                                       const float4 *__restrict__ trans, int G, int n_ct,
                                                       int64_t n_task) {
  constexpr int TW = 4 * NPT;    // column pairs per warp
  extern __shared__ uint4 sA[];  // [MTW][KS][4][32]
  // blockIdx.x = task CTA * groups + row-tile group: the groups of the same tasks run side by side
  // and read each child's mid from L2 instead of streaming it from DRAM once per group
  const int nmg = (MT + MTW - 1) / MTW;
  const int mt0 = (int)(blockIdx.x % nmg) * MTW;
  const int64_t cta = blockIdx.x / nmg;
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
  const int64_t task = cta * (blockDim.x >> 5) + warp;
  if (task >= n_task) return;
  const int ct = (int)(task % n_ct);
  int64_t rest = task / n_ct;
  const int comp = (int)(rest % 6);
  rest /= 6;
  const int64_t p = rest % n_parent;
  const int slot = (int)(rest / n_parent), lam = slot / G;
  const int span = (phi + 1) / 2, j0 = ct * TW, part = g & 1;
  const int64_t pat = (int64_t)Rch * span * 2;  // uint4 words of one child pattern component
  const uint4 *mbase = mid + ((int64_t)slot * n_child * 6 + comp) * pat;
  const int32_t cl = lane < 8 ? child_table[p * 8 + lane] : -1;
  unsigned rem = __ballot_sync(0xffffffffu, cl >= 0);  // children present (bits 0..7)
  // B operand of k-step ks of one child: pair tile pt, k rows 2 tq, 2 tq + 1 (pair tq) and + 8 (pair tq + 4)
  auto load_b = [&](const uint4 *m, int ks, uint4 (&b)[NPT][2]) {
#pragma unroll
    for (int pt = 0; pt < NPT; ++pt) {
      const int col = j0 + pt * 4 + (g >> 1);
#pragma unroll
      for (int hh = 0; hh < 2; ++hh) {
        const int tp = ks * 8 + tq + 4 * hh;
        uint4 u = make_uint4(0u, 0u, 0u, 0u);
        if (col < span && tp < Rch) u = __ldg(m + ((int64_t)tp * span + col) * 2 + part);
        b[pt][hh] = u;
      }
    }
  };
  auto child_ptr = [&](int o) { return mbase + (int64_t)__shfl_sync(0xffffffffu, cl, o) * 6 * pat; };
  float acc[MTW][NPT][2][4];  // [..][j / j'][re, im of rows g and g + 8]
#pragma unroll
  for (int i = 0; i < MTW; ++i)
#pragma unroll
    for (int pt = 0; pt < NPT; ++pt)
#pragma unroll
      for (int w = 0; w < 2; ++w) acc[i][pt][w][0] = acc[i][pt][w][1] = acc[i][pt][w][2] = acc[i][pt][w][3] = 0.f;
  const float4 *tr = trans + (int64_t)lam * Rp * phi;
  bool more = rem != 0;
  int o = more ? __ffs(rem) - 1 : 0;
  rem &= rem - 1;
  const uint4 *m = child_ptr(o);
  uint4 nb[NPT][2] = {};
  if (more) load_b(m, 0, nb);
  while (more) {
    float d[MTW][NPT][2][4];  // [..][U, V][..]
#pragma unroll
    for (int i = 0; i < MTW; ++i)
#pragma unroll
      for (int pt = 0; pt < NPT; ++pt)
#pragma unroll
        for (int w = 0; w < 2; ++w) d[i][pt][w][0] = d[i][pt][w][1] = d[i][pt][w][2] = d[i][pt][w][3] = 0.f;
    int o_next = o;
    const uint4 *m_next = m;
    for (int ks = 0; ks < KS; ++ks) {
      uint4 b[NPT][2];
#pragma unroll
      for (int pt = 0; pt < NPT; ++pt) {
        b[pt][0] = nb[pt][0];
        b[pt][1] = nb[pt][1];
      }
      if (ks + 1 < KS) {
        load_b(m, ks + 1, nb);
      } else if (rem) {
        o_next = __ffs(rem) - 1;
        m_next = child_ptr(o_next);
        load_b(m_next, 0, nb);
      }
      // one basic block: MTW x NPT x 2 independent accumulators
#pragma unroll
      for (int i = 0; i < MTW; ++i) {
        const uint4 *a = sA + (size_t)(i * KS + ks) * 128 + lane;
        const uint4 ph = a[0], pl = a[32], mh = a[64], ml = a[96];
        const uint32_t aph[4] = {ph.x, ph.y, ph.z, ph.w}, apl[4] = {pl.x, pl.y, pl.z, pl.w};
        const uint32_t amh[4] = {mh.x, mh.y, mh.z, mh.w}, aml[4] = {ml.x, ml.y, ml.z, ml.w};
#pragma unroll
        for (int pt = 0; pt < NPT; ++pt) {
          const uint32_t sh[2] = {b[pt][0].x, b[pt][1].x}, sl[2] = {b[pt][0].y, b[pt][1].y};
          const uint32_t dh[2] = {b[pt][0].z, b[pt][1].z}, dl[2] = {b[pt][0].w, b[pt][1].w};
          mma_bf16(d[i][pt][0], aph, sh);
          mma_bf16(d[i][pt][1], amh, dh);
          mma_bf16(d[i][pt][0], aph, sl);
          mma_bf16(d[i][pt][1], amh, dl);
          mma_bf16(d[i][pt][0], apl, sh);
          mma_bf16(d[i][pt][1], aml, dh);
        }
      }
    }
    // Y_j = U + V, Y_j' = U - V; translation of child octant o and the child
    // sum.  Rows >= Rp (zero rows of A) and columns past the half span (zero
    // B) hold exact zeros, so every element runs unguarded with its table
    // index clamped in range: one basic block of independent chains.
    const float sgx = (o & 1) ? 1.f : -1.f, sgy = (o & 2) ? -1.f : 1.f, sgz = (o & 4) ? -1.f : 1.f;
#pragma unroll
    for (int i = 0; i < MTW; ++i) {
#pragma unroll
      for (int pt = 0; pt < NPT; ++pt) {
        const int jq = j0 + pt * 4 + tq;
        const int jc = jq < span ? jq : span - 1;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int r0 = (mt0 + i) * 16 + g + 8 * h;
          const int r = r0 < Rp ? r0 : Rp - 1;
          const float ur = d[i][pt][0][2 * h], ui = d[i][pt][0][2 * h + 1];
          const float vr = d[i][pt][1][2 * h], vi = d[i][pt][1][2 * h + 1];
          // phi_{j+Phi/2} = phi_j + pi: the mirror column's x and y phases are
          // the negatives of column j's, so one table entry serves both
          const float4 rr = __ldg(tr + (int64_t)r * phi + jc);
          const float pxy = fmaf(sgx, rr.x, sgy * rr.y), pz = sgz * rr.z;
          float pxm = -pxy;
          if (ODD) {  // the partner's own entry (same row: same z phase)
            const int jm = jc + span < phi ? jc + span : phi - 1;
            const float4 rm = __ldg(tr + (int64_t)r * phi + jm);
            pxm = fmaf(sgx, rm.x, sgy * rm.y);
          }
#pragma unroll
          for (int w = 0; w < 2; ++w) {
            // each table phase is reduced to [-pi, pi], so |pz +- pxy| <= 3 pi:
            // the hardware sine / cosine need no further reduction (abs. error ~1e-6)
            float sn, cs;
            __sincosf(pz + (w ? pxm : pxy), &sn, &cs);
            const float yr = w ? ur - vr : ur + vr, yi = w ? ui - vi : ui + vi;
            acc[i][pt][w][2 * h] += yr * cs - yi * sn;
            acc[i][pt][w][2 * h + 1] += yr * sn + yi * cs;
          }
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
    for (int pt = 0; pt < NPT; ++pt) {
      const int jq = j0 + pt * 4 + tq;
      if (jq >= span) continue;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int r = (mt0 + i) * 16 + g + 8 * h;
        if (r >= Rp) continue;
#pragma unroll
        for (int w = 0; w < 2; ++w)
          if (!ODD || jq + w * span < phi)
            out[(int64_t)r * phi + jq + w * span] = make_float2(acc[i][pt][w][2 * h], acc[i][pt][w][2 * h + 1]);
      }
    }
  }
}

template <int NPT, int MTW, bool ODD>
static void launch_theta_warp(dim3 grid, size_t smem, const uint4 *mid, float2 *parent, const int32_t *child_table,
                              int64_t n_parent, int64_t n_child, int phi, int Rch, int Rp, int KS, int MT,
                              const uint4 *A, const float4 *trans, int G, int n_ct, int64_t n_task, cudaStream_t st) {
  k_theta_warp<NPT, MTW, ODD><<<grid, 256, smem, st>>>(mid, parent, child_table, n_parent, n_child, phi, Rch, Rp, KS,
                                                       MT, A, trans, G, n_ct, n_task);
}

po_status launch_interp_cols_mma(const uint4 *mid, float2 *parent, const int32_t *child_table, int64_t n_parent,
                                 int64_t n_child, int phi, int Rc, int Rp, int Kp, const uint32_t *Afrag,
                                 const float4 *trans, int n_slots, int G, int tile, cudaStream_t st) {
  if (n_parent <= 0 || n_slots <= 0) return PO_OK;
  const int Rc2 = Rc + (Rc & 1);
  if (Kp % 16 || Kp < Rc2) return fail(PO_ERR_INTERNAL, "theta matrix K padding");
  const bool odd = phi % 2 != 0;  // reference theta mode only (no mirrored rows)
  const int KS = Kp / 16, MT = (Rp + 15) / 16;
  const int NPT = tile == 16 && !odd ? 2 : 1;
  // 16-row tiles per warp: up to 4 (register budget of the accumulators), and
  // few enough that the CTA's matrix slice (2 KB per tile and k-step) leaves
  // room for two CTAs per SM; a single tile may use the whole opt-in limit
  const size_t tile_bytes = sizeof(uint4) * (size_t)KS * 128;
  int cap = NPT == 2 ? 2 : 4;
  while (cap > 1 && (size_t)cap * tile_bytes > 113 * 1024) --cap;
  if (tile_bytes > 227 * 1024)
    return fail(PO_ERR_UNSUPPORTED, "angular grid too large for the tensor-core interpolation");
  const int nmg = (MT + cap - 1) / cap;
  const int MTW = (MT + nmg - 1) / nmg;
  const size_t smem = (size_t)MTW * tile_bytes;
  const int TW = 4 * NPT;
  const int n_ct = ((phi + 1) / 2 + TW - 1) / TW;
  const int64_t n_task = (int64_t)n_slots * n_parent * 6 * n_ct;
  const int64_t gx = (n_task + 7) / 8 * nmg;
  if (gx > 2147483647LL) return fail(PO_ERR_UNSUPPORTED, "too many nodes for one launch");
  dim3 grid((unsigned)gx, 1u, 1u);
  const uint4 *A = (const uint4 *)Afrag;
#define PO_TW(N, M, O)                                                                                             \
  if (NPT == N && MTW == M && odd == O) {                                                                         \
    launch_theta_warp<N, M, O>(grid, smem, mid, parent, child_table, n_parent, n_child, phi, Rc2 / 2, Rp, KS, MT, \
                               A, trans, G, n_ct, n_task, st);                                                     \
  } else
  PO_TW(1, 1, false) PO_TW(1, 2, false) PO_TW(1, 3, false) PO_TW(1, 4, false) PO_TW(2, 1, false) PO_TW(2, 2, false)
  PO_TW(1, 1, true) PO_TW(1, 2, true) PO_TW(1, 3, true) PO_TW(1, 4, true) {
    return fail(PO_ERR_INTERNAL, "theta pass variant");
  }
#undef PO_TW
  count_launch();
  PO_CUDA(cudaGetLastError());
  return PO_OK;
}

// ----------------------------------------------- transposed theta pass
// Adjoint of k_theta_warp for the children of one parent.  With
// X_j = P_j exp(-i k s.(c_child - c_parent)) on the parent grid (P: the
// parent's adjoint pattern) and S' = X_j + X_j', D' = X_j - X_j':
//   U' = A_plus^T S',  V' = A_minus^T D',  mid_j = U' + V',  mid_j' = U' - V'.
// A warp owns one (slot, parent, component) and 4 column pairs j = j0.., for
// the CTA's 16-row tiles of the children (blockIdx.y), and writes every child
// of the parent in turn: the parent's pattern and translation entries are
// read from L2 for the first child and from L1 after it.  The CTA stages its
// slice of the transposed matrices in shared memory.  B fragments (K = parent
// rows) are generated in registers: the lanes of a column's real and
// imaginary parts (g even / odd) each rotate two of the four rows and swap
// halves, so every phasor is evaluated once per child.
template <int MTW>
__global__ void __launch_bounds__(256, 2) k_theta_adj_warp(
    const float2 *__restrict__ parent_adj, float2 *__restrict__ mid_adj, const int32_t *__restrict__ child_table,
    int64_t n_parent, int64_t n_child, int phi, int Rc, int Rp, int KS, int MT, const uint4 *__restrict__ Afrag,
    const float4 *__restrict__ trans, int G, int n_ct, int64_t n_task) {
  extern __shared__ uint4 sA[];  // [MTW][KS][4][32]
  // blockIdx.x = task CTA * groups + row-tile group (groups of a task side by side: the parent's
  // pattern is read from L2 once per task)
  const int nmg = (MT + MTW - 1) / MTW;
  const int mt0 = (int)(blockIdx.x % nmg) * MTW;
  const int64_t cta = blockIdx.x / nmg;
  const int nmt = MT - mt0 < MTW ? MT - mt0 : MTW;
  {
    const uint4 *src = Afrag + (size_t)mt0 * KS * 128;
    const int n = nmt * KS * 128;
    for (int e = threadIdx.x; e < MTW * KS * 128; e += blockDim.x)
      sA[e] = e < n ? __ldg(src + e) : make_uint4(0u, 0u, 0u, 0u);
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, tq = lane & 3;
  const int64_t task = cta * (blockDim.x >> 5) + warp;
  if (task >= n_task) return;
  const int ct = (int)(task % n_ct);
  int64_t rest = task / n_ct;
  const int comp = (int)(rest % 6);
  rest /= 6;
  const int64_t p = rest % n_parent;
  const int slot = (int)(rest / n_parent), lam = slot / G;
  const int span = phi / 2, j0 = ct * 4;
  const bool odd = g & 1;
  const float4 *tr = trans + (int64_t)lam * Rp * phi;
  const float2 *src = parent_adj + (((int64_t)slot * n_parent + p) * 6 + comp) * (int64_t)Rp * phi;
  const int jq = j0 + (g >> 1);  // this lane's column pair (B n-index g)
  const bool jok = jq < span;
  const int jo = j0 + tq;  // the D fragment's column pair
  const int32_t cl = lane < 8 ? child_table[p * 8 + lane] : -1;
  unsigned rem = __ballot_sync(0xffffffffu, cl >= 0);  // children present (bits 0..7)
  while (rem) {
    const int o = __ffs(rem) - 1;
    rem &= rem - 1;
    const int64_t c = __shfl_sync(0xffffffffu, cl, o);
    const float sgx = (o & 1) ? 1.f : -1.f, sgy = (o & 2) ? -1.f : 1.f, sgz = (o & 4) ? -1.f : 1.f;
    // S', D' of parent row r for column pair jq (zero outside the grid)
    auto rotated = [&](int r, float2 &S, float2 &D) {
      S = D = make_float2(0.f, 0.f);
      if (!jok || r >= Rp) return;
      const float2 a = src[(int64_t)r * phi + jq], b = src[(int64_t)r * phi + jq + span];
      const float4 rr = __ldg(tr + (int64_t)r * phi + jq);
      const float pxy = fmaf(sgx, rr.x, sgy * rr.y), pz = sgz * rr.z;
      float s1, c1, s2, c2;  // |pz +- pxy| <= 3 pi (table phases reduced to [-pi, pi])
      __sincosf(pz + pxy, &s1, &c1);  // column j
      __sincosf(pz - pxy, &s2, &c2);  // its mirror (x and y phases negated)
      const float xr = a.x * c1 + a.y * s1, xi = a.y * c1 - a.x * s1;  // a exp(-i ph_j)
      const float yr = b.x * c2 + b.y * s2, yi = b.y * c2 - b.x * s2;
      S = make_float2(xr + yr, xi + yi);
      D = make_float2(xr - yr, xi - yi);
    };
    float d[MTW][2][4];
#pragma unroll
    for (int i = 0; i < MTW; ++i)
#pragma unroll
      for (int w = 0; w < 2; ++w) d[i][w][0] = d[i][w][1] = d[i][w][2] = d[i][w][3] = 0.f;
    for (int ks = 0; ks < KS; ++ks) {
      // even lane: rows 2tq, 2tq+8 (keeps real parts); odd lane: rows 2tq+1, 2tq+9 (imaginary)
      const int r0 = ks * 16 + 2 * tq + (odd ? 1 : 0);
      float2 S0, D0, S1, D1;
      rotated(r0, S0, D0);
      rotated(r0 + 8, S1, D1);
      const float xs0 = __shfl_xor_sync(0xffffffffu, odd ? S0.x : S0.y, 4);
      const float xd0 = __shfl_xor_sync(0xffffffffu, odd ? D0.x : D0.y, 4);
      const float xs1 = __shfl_xor_sync(0xffffffffu, odd ? S1.x : S1.y, 4);
      const float xd1 = __shfl_xor_sync(0xffffffffu, odd ? D1.x : D1.y, 4);
      // pairs (row 2tq, row 2tq+1) and (2tq+8, 2tq+9) of this lane's part
      const float sa = odd ? xs0 : S0.x, sb = odd ? S0.y : xs0, sc = odd ? xs1 : S1.x, sd = odd ? S1.y : xs1;
      const float da = odd ? xd0 : D0.x, db = odd ? D0.y : xd0, dc = odd ? xd1 : D1.x, dd = odd ? D1.y : xd1;
      uint32_t sh[2], sl[2], dh[2], dl[2];
      split_bf16x2(sa, sb, sh[0], sl[0]);
      split_bf16x2(sc, sd, sh[1], sl[1]);
      split_bf16x2(da, db, dh[0], dl[0]);
      split_bf16x2(dc, dd, dh[1], dl[1]);
#pragma unroll
      for (int i = 0; i < MTW; ++i) {
        const uint4 *a = sA + (size_t)(i * KS + ks) * 128 + lane;
        const uint4 ph = a[0], pl = a[32], mh = a[64], ml = a[96];
        const uint32_t aph[4] = {ph.x, ph.y, ph.z, ph.w}, apl[4] = {pl.x, pl.y, pl.z, pl.w};
        const uint32_t amh[4] = {mh.x, mh.y, mh.z, mh.w}, aml[4] = {ml.x, ml.y, ml.z, ml.w};
        mma_bf16(d[i][0], aph, sh);
        mma_bf16(d[i][1], amh, dh);
        mma_bf16(d[i][0], aph, sl);
        mma_bf16(d[i][1], amh, dl);
        mma_bf16(d[i][0], apl, sh);
        mma_bf16(d[i][1], aml, dh);
      }
    }
    // D fragment: rows t = tile*16 + g (+8), complex column pair j0 + tq
    if (jo >= span) continue;
    float2 *dst = mid_adj + (((int64_t)slot * n_child + c) * 6 + comp) * (int64_t)Rc * phi;
#pragma unroll
    for (int i = 0; i < MTW; ++i) {
      if (i >= nmt) break;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int t = (mt0 + i) * 16 + g + 8 * h;
        if (t >= Rc) continue;
        const float ur = d[i][0][2 * h], ui = d[i][0][2 * h + 1], vr = d[i][1][2 * h], vi = d[i][1][2 * h + 1];
        dst[(int64_t)t * phi + jo] = make_float2(ur + vr, ui + vi);
        dst[(int64_t)t * phi + jo + span] = make_float2(ur - vr, ui - vi);
      }
    }
  }
}

po_status launch_interp_cols_adj_mma(const float2 *parent_adj, float2 *mid_adj, const int32_t *child_table,
                                     int64_t n_parent, int64_t n_child, int phi, int Rc, int Rp, int Kp,
                                     const uint32_t *Afrag, const float4 *trans, int n_slots, int G,
                                     cudaStream_t st) {
  if (n_parent <= 0 || n_slots <= 0) return PO_OK;
  if (Kp % 16 || Kp < Rp) return fail(PO_ERR_INTERNAL, "adjoint theta matrix K padding");
  if (phi % 2) return fail(PO_ERR_INTERNAL, "mirrored storage needs an even phi grid");
  const int KS = Kp / 16, MT = (Rc + 15) / 16;
  const size_t tile_bytes = sizeof(uint4) * (size_t)KS * 128;
  int cap = 4;
  while (cap > 1 && (size_t)cap * tile_bytes > 113 * 1024) --cap;
  if (tile_bytes > 227 * 1024) return fail(PO_ERR_UNSUPPORTED, "angular grid too large for the adjoint theta pass");
  const int nmg = (MT + cap - 1) / cap;
  const int MTW = (MT + nmg - 1) / nmg;
  const size_t smem = (size_t)MTW * tile_bytes;
  const int n_ct = (phi / 2 + 3) / 4;
  const int64_t n_task = (int64_t)n_slots * n_parent * 6 * n_ct;
  const int64_t gx = (n_task + 7) / 8 * nmg;
  if (gx > 2147483647LL) return fail(PO_ERR_UNSUPPORTED, "too many nodes for one launch");
  dim3 grid((unsigned)gx, 1u, 1u);
  const uint4 *A = (const uint4 *)Afrag;
  switch (MTW) {
#define PO_TA(M)                                                                                          \
  case M:                                                                                                \
    k_theta_adj_warp<M><<<grid, 256, smem, st>>>(parent_adj, mid_adj, child_table, n_parent, n_child,   \
                                                 phi, Rc, Rp, KS, MT, A, trans, G, n_ct, n_task);      \
    break;
    PO_TA(1) PO_TA(2) PO_TA(3) PO_TA(4)
#undef PO_TA
    default: return fail(PO_ERR_INTERNAL, "adjoint theta pass variant");
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

// Forward phi matrix in mirror-pair column order (the packed row pass):
// n-tile nt, slot 2q + w holds parent column nt*4 + q + w H (H = ceil(Pp/2)
// pairs), so a lane's D fragment holds a column and its partner for two rows.
// An odd Pp (reference theta mode, where the columns of a level need not pair
// up as phi and phi + pi) leaves one phantom partner, column Pp: a zero column.
void build_phi_matrix(int Pc, int Pp, int Kp, std::vector<uint32_t> &out) {
  const int half = (Pp + 1) / 2, NTt = (half + 3) / 4;
  b_fragments(NTt * 8, Pc, Kp,
              [&](int n, int k) {
                const int j = (n >> 3) * 4 + ((n & 7) >> 1);
                const int col = j + (n & 1) * half;
                if (j >= half || col >= Pp) return 0.0;
                return trig_kernel(Pc, (double)col / Pp - (double)k / Pc);
              },
              out);
}

// phi map as the B operand of the tcgen05 row pass (po_rows_tc.cu): per N tile
// of ntn columns (column n = 2 jl + w: pair j = nt ntn/2 + jl, w = 0 for
// parent column j and 1 for j + Pp/2) and per 16-row K chunk, the bf16 hi and
// lo matrices [ntn/8][2][8][8] (K-major core matrices), zero beyond Pc rows and
// Pp/2 pairs; one tile is Kc/16 chunks of 64 ntn bytes.
void build_phi_tc(int Pc, int Pp, int Kc, int ntn, int n_nt, std::vector<uint16_t> &out) {
  const int half = Pp / 2, KC = Kc / 16;
  const size_t chunk = (size_t)2 * ntn * 16, tile = (size_t)KC * chunk;
  out.assign(tile * n_nt, 0);
  for (int nt = 0; nt < n_nt; ++nt)
    for (int n = 0; n < ntn; ++n) {
      const int j = nt * (ntn / 2) + (n >> 1);
      if (j >= half) continue;
      const int col = j + (n & 1) * half;
      for (int k = 0; k < Pc; ++k) {
        const double v = trig_kernel(Pc, (double)col / Pp - (double)k / Pc);
        const uint16_t h = bf16_rne((float)v), l = bf16_rne((float)(v - (double)bf16_to_f(h)));
        const size_t base = nt * tile + (size_t)(k / 16) * chunk;
        const size_t in_mat = ((size_t)(n / 8) * 2 + (k % 16) / 8) * 64 + (n % 8) * 8 + (k % 8);
        out[base + in_mat] = h;
        out[base + (size_t)ntn * 16 + in_mat] = l;
      }
    }
}

// transpose of the phi map: child column j (< Pc) from parent columns j' (< Pp)
void build_phi_matrix_adj(int Pc, int Pp, int Kp, std::vector<uint32_t> &out) {
  b_fragments(Pc, Pp, Kp, [&](int j, int jp) { return trig_kernel(Pc, (double)jp / Pp - (double)j / Pc); }, out);
}

// blockIdx.y selects a group of kRowNG n-tiles (output columns); its slice of
// the phi matrix is staged in shared memory when it fits (b_in_smem), and
// every warp runs over blocks of 8 rows with the next k-step's input loads in
// flight while the current one multiplies (rows_block, po_rows_block.cuh).
template <int PACK>
__global__ void __launch_bounds__(128, 6) k_interp_rows_mma(const float2 *__restrict__ src, void *__restrict__ dst_,
                                                         int64_t nrows, int Rc, int Pc, int Pp, int Kp,
                                                         const uint4 *__restrict__ Bm, int b_in_smem, int Rr,
                                                         int npad) {
  extern __shared__ uint4 bsm[];
  const int KS = Kp / 16, NTt = PACK ? ((Pp + 1) / 2 + 3) / 4 : (Pp + 7) / 8;
  const int ng = blockIdx.y * kRowNG;
  const int nq = NTt - ng < kRowNG ? NTt - ng : kRowNG;  // n-tiles in this group
  const uint4 *Bg = Bm + (size_t)ng * KS * 32;
  if (b_in_smem) {
    for (int e = threadIdx.x; e < nq * KS * 32; e += blockDim.x) bsm[e] = Bg[e];
    __syncthreads();
  }
  const uint4 *B = b_in_smem ? bsm : Bg;
  const int Rc2 = PACK == 2 ? Rr : Rc + (Rc & 1);
  const int64_t nblk = (nrows + 7) / 8;
  for (int64_t blk = (int64_t)blockIdx.x * 4 + (threadIdx.x >> 5); blk < nblk; blk += (int64_t)gridDim.x * 4)
    rows_block<PACK, false>(blk, 0, nrows, src, dst_, Rc, Rc2, Pc, Pp, KS, B, ng, nq, npad);
}

// Packed row pass (k_theta_warp's operand) for narrow child grids, Pc <= 32
// (two k-steps) and at most NG n-tiles of 4 mirror pairs: the same products
// and output as rows_block<1, false>, but each warp keeps the whole input of
// its next block of 8 rows in flight (both k-steps, statically indexed
// ping-pong registers) while the current block multiplies, so that a warp has
// about 2 KB of loads outstanding instead of one k-step.
template <int NG>
__global__ void __launch_bounds__(128, 5) k_rows_mma_narrow(const float2 *__restrict__ src,
                                                                          uint4 *__restrict__ dst, int64_t nrows,
                                                                          int Rc, int Pc, int Pp,
                                                                          const uint4 *__restrict__ Bm) {
  constexpr int KS = 2;
  __shared__ uint4 bsm[NG * KS * 32];
  const int half = (Pp + 1) / 2, nq = (half + 3) / 4;
  for (int e = threadIdx.x; e < NG * KS * 32; e += blockDim.x)
    bsm[e] = e < nq * KS * 32 ? Bm[e] : make_uint4(0u, 0u, 0u, 0u);
  __syncthreads();
  const int lane = threadIdx.x & 31, g = lane >> 2, tq = lane & 3;
  const bool odd = g & 1;
  const int Rc2 = Rc + (Rc & 1);
  const int64_t nblk = (nrows + 7) / 8, stride = (int64_t)gridDim.x * 4;
  auto load = [&](int64_t blk, float2 (&v)[KS][4]) {
    const int64_t r = blk * 8 + g;
    const int64_t pattern = r / Rc2;
    const int t = (int)(r - pattern * Rc2);
    const bool ok = blk < nblk && r < nrows && t < Rc;
    const float2 *in = src + (ok ? pattern * Rc + t : 0) * (int64_t)Pc;
#pragma unroll
    for (int ks = 0; ks < KS; ++ks)
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int k = ks * 16 + 2 * tq + (u & 1) + (u >> 1) * 8;
        v[ks][u] = (ok && k < Pc) ? __ldg(in + k) : make_float2(0.f, 0.f);
      }
  };
  auto block = [&](int64_t blk, const float2 (&v)[KS][4]) {
    float acc[NG][4];
#pragma unroll
    for (int q = 0; q < NG; ++q) acc[q][0] = acc[q][1] = acc[q][2] = acc[q][3] = 0.f;
#pragma unroll
    for (int ks = 0; ks < KS; ++ks) {
      uint32_t ahi[4], alo[4];
      split_bf16x2(v[ks][0].x, v[ks][1].x, ahi[0], alo[0]);  // row g (real parts), k0, k0+1
      split_bf16x2(v[ks][0].y, v[ks][1].y, ahi[1], alo[1]);  // row g+8 (imaginary parts)
      split_bf16x2(v[ks][2].x, v[ks][3].x, ahi[2], alo[2]);  // row g, k0+8, k0+9
      split_bf16x2(v[ks][2].y, v[ks][3].y, ahi[3], alo[3]);
#pragma unroll
      for (int q = 0; q < NG; ++q) {
        const uint4 bv = bsm[(q * KS + ks) * 32 + lane];  // zero for the n-tiles past nq
        const uint32_t bhi[2] = {bv.x, bv.y}, blo[2] = {bv.z, bv.w};
        mma_bf16(acc[q], ahi, bhi);
        mma_bf16(acc[q], ahi, blo);
        mma_bf16(acc[q], alo, bhi);
      }
    }
    const int64_t r = blk * 8 + g, pair_row = r >> 1;
    const bool rok = r < nrows;
#pragma unroll
    for (int q = 0; q < NG; ++q) {
      const float sr = acc[q][0] + acc[q][1], dr = acc[q][0] - acc[q][1];
      const float si = acc[q][2] + acc[q][3], di = acc[q][2] - acc[q][3];
      const float xs = __shfl_xor_sync(0xffffffffu, odd ? sr : si, 4);
      const float xd = __shfl_xor_sync(0xffffffffu, odd ? dr : di, 4);
      const float s0 = odd ? xs : sr, s1 = odd ? si : xs;
      const float d0 = odd ? xd : dr, d1 = odd ? di : xd;
      const int j = q * 4 + tq;
      uint32_t sh, sl, dh, dl;
      split_bf16x2(s0, s1, sh, sl);
      split_bf16x2(d0, d1, dh, dl);
      if (rok && j < half) dst[(pair_row * half + j) * 2 + (odd ? 1 : 0)] = make_uint4(sh, sl, dh, dl);
    }
  };
  // every lane of a warp walks the same blocks (the epilogue shuffles need the whole warp)
  int64_t blk = (int64_t)blockIdx.x * 4 + (threadIdx.x >> 5);
  float2 va[KS][4], vb[KS][4];
  load(blk, va);
  for (; blk < nblk; blk += 2 * stride) {
    load(blk + stride, vb);
    block(blk, va);
    if (blk + stride >= nblk) break;
    load(blk + 2 * stride, va);
    block(blk + stride, vb);
  }
}

static po_status launch_rows(int pack, const float2 *src, void *dst, int64_t nrows, int Rc, int Pc, int Pp, int Kp,
                             const uint32_t *Bm, int sm_count, cudaStream_t st, int Rr = 0, int npad = 0) {
  if (nrows <= 0) return PO_OK;
  if (Kp % 16 || Kp < Pc) return fail(PO_ERR_INTERNAL, "phi matrix K padding");
  const int NTt = pack ? ((Pp + 1) / 2 + 3) / 4 : (Pp + 7) / 8;
  const int ngroups = (NTt + kRowNG - 1) / kRowNG;
  const size_t bbytes = sizeof(uint4) * (size_t)kRowNG * (Kp / 16) * 32;
  const bool b_smem = bbytes <= 128 * 1024;
  const size_t smem = b_smem ? bbytes : 0;
  int64_t blocks = ((nrows + 7) / 8 + 3) / 4;
  const int64_t cap = (int64_t)sm_count * 16 / ngroups + 1;
  if (blocks > cap) blocks = cap;
  if (ngroups > 65535) return fail(PO_ERR_UNSUPPORTED, "angular grid too large for the row pass");
  dim3 grid((unsigned)blocks, (unsigned)ngroups);
  if (pack == 1 && Kp == 32 && NTt <= 8) {
    // narrow child grid: whole blocks in flight (k_rows_mma_narrow), grid of
    // resident CTAs (5 per SM), each warp walking many blocks
    const int64_t nb = std::min<int64_t>(((nrows + 7) / 8 + 3) / 4, (int64_t)sm_count * 5);
    if (NTt <= 4)
      k_rows_mma_narrow<4><<<(unsigned)nb, 128, 0, st>>>(src, (uint4 *)dst, nrows, Rc, Pc, Pp, (const uint4 *)Bm);
    else
      k_rows_mma_narrow<8><<<(unsigned)nb, 128, 0, st>>>(src, (uint4 *)dst, nrows, Rc, Pc, Pp, (const uint4 *)Bm);
  } else if (pack == 2)
    k_interp_rows_mma<2><<<grid, 128, smem, st>>>(src, dst, nrows, Rc, Pc, Pp, Kp, (const uint4 *)Bm,
                                                  b_smem ? 1 : 0, Rr, npad);
  else if (pack == 1)
    k_interp_rows_mma<1><<<grid, 128, smem, st>>>(src, dst, nrows, Rc, Pc, Pp, Kp, (const uint4 *)Bm,
                                                  b_smem ? 1 : 0, 0, 0);
  else
    k_interp_rows_mma<0><<<grid, 128, smem, st>>>(src, dst, nrows, Rc, Pc, Pp, Kp, (const uint4 *)Bm,
                                                  b_smem ? 1 : 0, 0, 0);
  count_launch();
  PO_CUDA(cudaGetLastError());
  return PO_OK;
}

po_status launch_interp_rows_mma(const float2 *src, float2 *dst, int64_t nrows, int Pc, int Pp, int Kp,
                                 const uint32_t *Bm, int sm_count, cudaStream_t st) {
  return launch_rows(0, src, dst, nrows, 0, Pc, Pp, Kp, Bm, sm_count, st);
}

po_status launch_interp_rows_packed(const float2 *src, uint4 *dst, int64_t n_patterns, int Rc, int Pc, int Pp,
                                    int Kp, const uint32_t *Bm, int sm_count, cudaStream_t st) {
  const int64_t nrows = n_patterns * (int64_t)(Rc + (Rc & 1));
  return launch_rows(1, src, dst, nrows, Rc, Pc, Pp, Kp, Bm, sm_count, st);
}

po_status launch_interp_rows_core(const float2 *src, uint8_t *dst, int64_t n_patterns, int Rc, int Rr, int npad,
                                  int Pc, int Pp, int Kp, const uint32_t *Bm, int sm_count, cudaStream_t st) {
  if (Rr % 16 || Rr < Rc || npad % 8 || npad < 6 * Pp || n_patterns % 6 || Pp % 2)
    return fail(PO_ERR_INTERNAL, "core-matrix row pass padding");
  return launch_rows(2, src, dst, n_patterns * (int64_t)Rr, Rc, Pc, Pp, Kp, Bm, sm_count, st, Rr, npad);
}

// Opt-in shared-memory limit of every kernel here, set once per device (the
// launchers pick their shared-memory size at run time and must not change
// function attributes while a stream is being captured).
po_status init_interp_mma_attributes(int max_smem) {
  PO_CUDA(cudaFuncSetAttribute(k_theta_adj_warp<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem));
  PO_CUDA(cudaFuncSetAttribute(k_theta_adj_warp<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem));
  PO_CUDA(cudaFuncSetAttribute(k_theta_adj_warp<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem));
  PO_CUDA(cudaFuncSetAttribute(k_theta_adj_warp<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem));
  PO_CUDA(cudaFuncSetAttribute(k_interp_rows_mma<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem));
  PO_CUDA(cudaFuncSetAttribute(k_interp_rows_mma<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem));
  PO_CUDA(cudaFuncSetAttribute(k_interp_rows_mma<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem));
#define PO_TW_ATTR(N, M, O) \
  PO_CUDA(cudaFuncSetAttribute(k_theta_warp<N, M, O>, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem));
  PO_TW_ATTR(1, 1, false) PO_TW_ATTR(1, 2, false) PO_TW_ATTR(1, 3, false) PO_TW_ATTR(1, 4, false)
  PO_TW_ATTR(2, 1, false) PO_TW_ATTR(2, 2, false)
  PO_TW_ATTR(1, 1, true) PO_TW_ATTR(1, 2, true) PO_TW_ATTR(1, 3, true) PO_TW_ATTR(1, 4, true)
#undef PO_TW_ATTR
  return PO_OK;
}

}  // namespace wavepo
