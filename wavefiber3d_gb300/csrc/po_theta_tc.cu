// po_theta_tc.cu -- theta pass + translation + child sum on the 5th-generation
// tensor cores (tcgen05, accumulators in tensor memory) for the tree levels
// whose parent rows fill 128-row tiles.
//
// Same contraction as k_theta_warp (po_interp_mma.cu; util/interpolation.h:47-77,
// util/fields.h:92-103 and :153-169): for every child of a parent,
//   U = A_plus S,  V = A_minus D,  Y_j = U + V,  Y_j' = U - V,
// rotated by the child's translation phasor and summed over the children.
//
// The six component patterns of a child share one column space (packed pair
// P = comp Phi/2 + j, real columns 2 P and 2 P + 1), so that a level's columns
// are padded to whole chunks once per child instead of once per component.
// One CTA owns one (slot, parent), kTcPairs packed column pairs (N = 128 real
// columns of S and D) and one 128-row tile of the parent, and runs as three
// roles:
//  * copy warp (one thread): streams K chunks of 16 child rows -- the chunk of
//    the four split theta matrices (A_plus hi, lo, A_minus hi, lo; 16 KB) and
//    of the child's four split operands (S hi, lo, D hi, lo; 16 KB) -- with
//    bulk copies (cp.async.bulk) into a ring of shared-memory stages, each
//    completing the stage's "full" mbarrier by transaction bytes;
//  * MMA warp (one thread): issues the products (hi*hi + hi*lo + lo*hi per
//    matrix pair: 6 tcgen05.mma of 128 x 128 x 16 per chunk) into one of two
//    U/V accumulator pairs in tensor memory (one per child parity), commits
//    each chunk to the stage's "empty" mbarrier and a child's last chunk to
//    the accumulator's "full" mbarrier;
//  * 16 epilogue warps (warp w reads tensor-memory lanes 32 (w % 4) .., i.e.
//    one parent row per thread, and 16 column pairs per warpgroup): read a
//    finished child's U and V (tcgen05.ld), rotate and accumulate them in
//    registers and release the accumulator pair, while the next child's
//    products run into the other pair.
// The child's phasor at (row, column j) is e^{i (sz z + sx x + sy y)} and at
// the mirror column e^{i (sz z - sx x - sy y)}, with the octant's signs s and
// the reduced phases (x, y, z) of the translation table.  Once per CTA the
// epilogue warps stage (x, y) per (row, pair) and e^{i z} per row; a child
// then costs one sincos per (row, pair), and the row's z phasor turns the
// accumulator twice per task, since the children run in octant order (the
// positive z sign first).  (Staging e^{i (x + y)} and
// e^{i (x - y)} instead, which removes that sincos, needs twice the table
// space, leaves room for one stage less and measured slower.)
//
// Operand layouts (bf16, K-major, no swizzle; core matrices of 8 rows x 16 B):
// a chunk of one matrix is [rows / 8][2][8][8] (row block, k8 block, row,
// k), i.e. leading-dimension offset 128 B, stride offset 256 B.  The theta
// matrices are stored as [tile][chunk][matrix][128 / 8][2][8][8]
// (build_theta_tc); the row pass writes each child's six packed component
// patterns as [chunk][matrix][npad / 8][2][8][8] (launch_rows_tc,
// launch_interp_rows_core), so that one CTA's share of a chunk is one
// contiguous 4-KB run per matrix.
//
// Every wait is bounded in time: on a timeout the kernel records error word 1
// and every role stops (`withhold`, a self-test switch, leaves the first
// stage unfilled so that this path runs).  Operand runs outside their buffers (checked once per
// CTA) record error word 2 and nothing is copied.  Before the CTA exits, the
// copy and MMA threads wait for the last phase of every barrier they armed, so
// that no copy or commit arrive outlives the CTA.
#include <cuda_runtime.h>

#include <cstring>
#include <vector>

#include "po_common.cuh"
#include "po_internal.h"
#include "po_kernels.h"
#include "po_tc_common.cuh"

namespace wavepo {

namespace {

using namespace tc;

constexpr int kTcKC = 16;                                 // K (child rows) per chunk
constexpr int kTcPairs = 64;                              // column pairs per CTA
constexpr int kTcN = 2 * kTcPairs;                        // real columns per product
constexpr int kTcEpiWarps = kTcPairs / 4;                 // 4 warps per 16 pairs
constexpr int kTcCopyWarp = kTcEpiWarps, kTcMmaWarp = kTcEpiWarps + 1;
constexpr int kTcThreads = 32 * (kTcEpiWarps + 2);
constexpr int kAStage = 4 * 128 * kTcKC * 2;              // 16 KB
constexpr int kBStage = 4 * kTcN * kTcKC * 2;             // 16 KB
constexpr uint32_t kTcTmemCols = 4 * kTcN;                // (U, V) x 2 children = 512 columns

constexpr int kTcLd = 129;  // float2 per pair (or output row) in the staged tables: 128 rows + 1 (bank spread)

// shared-memory plan; after the last child the output tile [128 rows][kTcLd]
// of (j, j') pairs is transposed through the stage and table space (the
// barriers behind it stay live)
struct TcPlan {
  static constexpr int stages = 4;
  static constexpr int table = kTcPairs * kTcLd * 8;     // (x, y) per (pair, row)
  static constexpr int table_off = stages * (kAStage + kBStage);
  static constexpr int pz_off = table_off + table;        // e^{i z} per row
  static constexpr int bar_off = pz_off + 128 * 8;
  static constexpr int smem = bar_off + 128;              // + mbarriers, TMEM slot, abort flag
  static_assert(128 * kTcLd * 8 <= pz_off, "output transpose overlaps the live tables");
};
static_assert(TcPlan::smem + 128 <= 227 * 1024, "shared memory (dynamic + the static child table)");

}  // namespace

// A operand of one level for the tcgen05 pass: the theta matrices A_plus,
// A_minus over K = child rows padded to Kr (a multiple of 16), split into
// bf16 hi + lo, Kr KB per 128-row tile.
size_t theta_tc_bytes(int Rp, int Kr) {
  const int MT = (Rp + 127) / 128;
  return (size_t)MT * Kr * 1024;
}

static uint16_t bf16_bits(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  if ((u & 0x7f800000u) == 0x7f800000u) return (uint16_t)(u >> 16);
  return (uint16_t)((u + 0x7fffu + ((u >> 16) & 1u)) >> 16);
}
static float bf16_val(uint16_t h) {
  uint32_t u = (uint32_t)h << 16;
  float f;
  std::memcpy(&f, &u, 4);
  return f;
}

// Mplus / Mminus: [Rp][ld] (theta_plus_minus), columns >= Rc are zero padding
void build_theta_tc(const std::vector<double> &Mplus, const std::vector<double> &Mminus, int Rp, int Rc, int ld,
                    int Kr, std::vector<uint16_t> &out) {
  out.assign(theta_tc_bytes(Rp, Kr) / 2, 0);
  const size_t tile = (size_t)Kr * 512, chunk = kAStage / 2, matrix = 128 * kTcKC;  // in bf16 elements
  for (int r = 0; r < Rp; ++r)
    for (int k = 0; k < Rc; ++k)
      for (int pm = 0; pm < 2; ++pm) {
        const double v = (pm ? Mminus : Mplus)[(size_t)r * ld + k];
        const uint16_t h = bf16_bits((float)v);
        const uint16_t l = bf16_bits((float)(v - (double)bf16_val(h)));
        const int rr = r % 128, kk = k % kTcKC;
        const size_t base = (size_t)(r / 128) * tile + (size_t)(k / kTcKC) * chunk;
        const size_t in_mat = ((size_t)(rr / 8) * 2 + kk / 8) * 64 + (rr % 8) * 8 + (kk % 8);
        out[base + (size_t)(2 * pm) * matrix + in_mat] = h;
        out[base + (size_t)(2 * pm + 1) * matrix + in_mat] = l;
      }
}

// grid.x = task * MT + tile (task = (slot, parent, packed column chunk)), kTcThreads threads
__global__ void __launch_bounds__(kTcThreads, 1) k_theta_tc(
    const uint8_t *__restrict__ mid, float2 *__restrict__ parent, const int32_t *__restrict__ child_table,
    int64_t n_parent, int64_t n_child, int phi, int Kr, int Npad, int Rp, const uint8_t *__restrict__ Atc,
    const float4 *__restrict__ trans, int G, int n_nc, int64_t n_task, int *__restrict__ err, size_t mid_bytes,
    size_t atc_bytes, int withhold) {
  using Plan = TcPlan;
  constexpr int NST = Plan::stages;
  extern __shared__ __align__(128) uint8_t smem_tc[];
  uint8_t *sA = smem_tc;                                     // [NST][kAStage]
  uint8_t *sB = smem_tc + NST * kAStage;                     // [NST][kBStage]
  float2 *sT = (float2 *)(smem_tc + Plan::table_off);        // [kTcPairs][kTcLd]
  float2 *sPz = (float2 *)(smem_tc + Plan::pz_off);          // [128]
  uint64_t *full = (uint64_t *)(smem_tc + Plan::bar_off), *empty = full + NST, *accf = empty + NST,
           *acce = accf + 2;
  uint32_t *tmem_slot = (uint32_t *)(acce + 2);
  volatile int *abort_flag = (volatile int *)(tmem_slot + 1);
  __shared__ int32_t s_child[8];

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int MT = (Rp + 127) / 128, KC = Kr / kTcKC;
  const int mtile = (int)(blockIdx.x % MT);
  const int64_t task = blockIdx.x / MT;
  if (task >= n_task) return;
  const int nc = (int)(task % n_nc);
  const int64_t rest = task / n_nc;
  const int64_t p = rest % n_parent;
  const int slot = (int)(rest / n_parent), lam = slot / G;
  const int span = phi / 2, npairs = 6 * span;  // packed pairs of one child

  if (tid < 8) s_child[tid] = child_table[p * 8 + tid];
  if (tid == 0) {
    for (int b = 0; b < NST; ++b) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&full[b])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&empty[b])));
    }
    for (int b = 0; b < 2; ++b) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&accf[b])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(&acce[b])), "r"(kTcEpiWarps * 32));
    }
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tmem_slot)),
                 "r"(kTcTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = *tmem_slot;
  int kids[8], nkids = 0;
#pragma unroll
  for (int o = 0; o < 8; ++o)
    if (s_child[o] >= 0) kids[nkids++] = o;
  const int nsteps = nkids * KC;
  const size_t pat = (size_t)8 * Npad * Kr;  // bytes of one child's six packed patterns (4 matrices)

  if (warp == kTcCopyWarp) {
    // ---- copy role ----
    if (lane == 0) {
      int last_load[NST];
#pragma unroll
      for (int b = 0; b < NST; ++b) last_load[b] = -1;
      bool ok = (size_t)(mtile + 1) * Kr * 1024 <= atc_bytes;
      for (int i = 0; i < nkids; ++i) {
        const int64_t ch = s_child[kids[i]];
        ok = ok && ch < n_child && (((size_t)slot * n_child + ch) + 1) * pat <= mid_bytes;
      }
      if (!ok) {
        atomicExch(err, 2);
        *abort_flag = 1;
      }
      const uint8_t *abase = Atc + (size_t)mtile * Kr * 1024;
      const size_t col_off = (size_t)nc * (kTcN / 8) * 256;
      constexpr uint32_t bmat = kTcN / 8 * 256;  // bytes of one matrix's share of a chunk
      int ci = 0, kc = -1;  // child and K chunk of step t (no division on this thread's path)
      for (int t = 0; t < nsteps && ok; ++t) {
        if (++kc == KC) {
          kc = 0;
          ++ci;
        }
        const int b = t % NST;
        if (t >= NST && !mbar_wait(smem_addr(&empty[b]), ((t / NST) - 1) & 1, abort_flag)) {
          ok = false;
          break;
        }
        if (withhold && t == 0) continue;  // self-test: stage 0 never filled, its consumers give up
        const uint32_t fb = smem_addr(&full[b]);
        mbar_expect_tx(fb, kAStage + 4 * bmat);
        bulk_copy(smem_addr(sA + b * kAStage), abase + (size_t)kc * kAStage, kAStage, fb);
        const uint8_t *cb = mid + ((size_t)slot * n_child + s_child[kids[ci]]) * pat + (size_t)kc * 128 * Npad +
                            col_off;
#pragma unroll
        for (int m = 0; m < 4; ++m)
          bulk_copy(smem_addr(sB + b * kBStage + m * bmat), cb + (size_t)m * 32 * Npad, bmat, fb);
        last_load[b] = t;
      }
      if (!ok && !*abort_flag) {
        *abort_flag = 1;
        atomicCAS(err, 0, 1);
      }
      // every copy lands before the CTA exits
      for (int b = 0; b < NST; ++b)
        if (last_load[b] >= 0) (void)mbar_wait(smem_addr(&full[b]), (last_load[b] / NST) & 1, nullptr);
    }
    __syncwarp();
  } else if (warp == kTcMmaWarp) {
    // ---- MMA role ----
    if (lane == 0) {
      // D f32, A and B bf16, both K-major, N = kTcN, M = 128
      const uint32_t idesc =
          (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kTcN >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
      const uint64_t ad0 = tc_desc(smem_addr(sA)), bd0 = tc_desc(smem_addr(sB));
      constexpr uint64_t mA = (kAStage / 4) >> 4, mB = (kBStage / 4) >> 4;  // one matrix, in descriptor units
      bool ok = true;
      int committed = 0;
      int ci = 0, kc = -1;  // child and K chunk of step s (no division on the issuing path)
      for (int s = 0; s < nsteps; ++s) {
        if (++kc == KC) {
          kc = 0;
          ++ci;
        }
        const int b = s % NST;
        if (kc == 0 && ci >= 2 && !mbar_wait(smem_addr(&acce[ci & 1]), ((ci >> 1) - 1) & 1, abort_flag)) {
          ok = false;
          break;
        }
        if (!mbar_wait(smem_addr(&full[b]), (s / NST) & 1, abort_flag)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint32_t dU = tmem + (uint32_t)((ci & 1) * 2 * kTcN), dV = dU + kTcN;
        const uint64_t ad = ad0 + (uint64_t)b * (kAStage >> 4), bd = bd0 + (uint64_t)b * (kBStage >> 4);
        const uint32_t first = kc == 0 ? 0u : 1u;
        tc_mma(dU, ad, bd, idesc, first);                        // A+ hi * S hi
        tc_mma(dV, ad + 2 * mA, bd + 2 * mB, idesc, first);      // A- hi * D hi
        tc_mma(dU, ad, bd + mB, idesc, 1u);                      // A+ hi * S lo
        tc_mma(dV, ad + 2 * mA, bd + 3 * mB, idesc, 1u);         // A- hi * D lo
        tc_mma(dU, ad + mA, bd, idesc, 1u);                      // A+ lo * S hi
        tc_mma(dV, ad + 3 * mA, bd + 2 * mB, idesc, 1u);         // A- lo * D hi
        tc_commit(smem_addr(&empty[b]));
        if (kc == KC - 1) tc_commit(smem_addr(&accf[ci & 1]));
        committed = s + 1;
      }
      if (!ok && !*abort_flag) {
        *abort_flag = 1;
        atomicCAS(err, 0, 1);
      }
      // every commit arrive lands before the CTA exits (only the latest phase
      // of each barrier is waited on)
      for (int b = 0; b < NST; ++b) {
        const int ls = committed - 1 - (((committed - 1 - b) % NST) + NST) % NST;
        if (ls >= 0) (void)mbar_wait(smem_addr(&empty[b]), (ls / NST) & 1, nullptr);
      }
      const int done_kids = committed / KC;
      for (int ci = done_kids - 2 > 0 ? done_kids - 2 : 0; ci < done_kids; ++ci)
        (void)mbar_wait(smem_addr(&accf[ci & 1]), (ci >> 1) & 1, nullptr);
    }
    __syncwarp();
  } else {
    // ---- epilogue role: thread = parent row, warpgroup = 16 column pairs ----
    const int wg = warp >> 2, quarter = warp & 3, rl = quarter * 32 + lane;
    {
      // thread = one pair (lanes: consecutive pairs, contiguous in the table)
      // and 16 rows, loaded 8 at a time
      const float4 *tr = trans + (int64_t)lam * Rp * phi;
      const int pl = tid & (kTcPairs - 1);
      const int pp = nc * kTcPairs + pl < npairs ? nc * kTcPairs + pl : npairs - 1;
      const int jq = pp % span;  // the pair's column within its component
#pragma unroll
      for (int half = 0; half < 2; ++half) {
        float4 v[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const int row = (tid / kTcPairs) + 8 * (8 * half + i);
          const int rr = mtile * 128 + row < Rp ? mtile * 128 + row : Rp - 1;
          v[i] = __ldg(tr + (int64_t)rr * phi + jq);
        }
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const int row = (tid / kTcPairs) + 8 * (8 * half + i);
          sT[pl * kTcLd + row] = make_float2(v[i].x, v[i].y);
          if (pl == 0) {
            float sz, cz;
            sincosf(v[i].z, &sz, &cz);
            sPz[row] = make_float2(cz, sz);
          }
        }
      }
      asm volatile("bar.sync 1, %0;" ::"r"(kTcEpiWarps * 32));
    }
    float acc[16][2][2];
#pragma unroll
    for (int q = 0; q < 16; ++q) acc[q][0][0] = acc[q][0][1] = acc[q][1][0] = acc[q][1][1] = 0.f;
    const float2 ez = sPz[rl];
    // The z phasor e^{+-i z} depends on the row only (this thread's) and on
    // the child's z sign; the children come in octant order, those with the
    // positive z sign (o < 4) first.  So the accumulator collects sum Y e over
    // the positive children, is turned by e^{2 i z} once before the first
    // negative child, and by e^{-i z} once at the end:
    // e^{-iz} (e^{2iz} S+ + S-) = e^{iz} S+ + e^{-iz} S-.
    auto turn = [&](float cr, float ci_) {
#pragma unroll
      for (int q = 0; q < 16; ++q)
#pragma unroll
        for (int w = 0; w < 2; ++w) {
          const float ar = acc[q][w][0], ai = acc[q][w][1];
          acc[q][w][0] = ar * cr - ai * ci_;
          acc[q][w][1] = ar * ci_ + ai * cr;
        }
    };
    bool turned = false;
    bool ok = true;
    for (int ci = 0; ci < nkids && ok; ++ci) {
      const int b = ci & 1;
      ok = __all_sync(0xffffffffu, mbar_wait(smem_addr(&accf[b]), (ci >> 1) & 1, abort_flag)) != 0;
      if (!ok) break;
      asm volatile("tcgen05.fence::after_thread_sync;");
      const int o = kids[ci];
      if ((o & 4) && !turned) {
        turn(ez.x * ez.x - ez.y * ez.y, 2.f * ez.x * ez.y);
        turned = true;
      }
      // octant signs: x + for o & 1, y + for !(o & 2)
      const bool px = (o & 1) != 0, py = (o & 2) == 0;
      const float sgx = px ? 1.f : -1.f, sgy = py ? 1.f : -1.f;
      const uint32_t ta = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(b * 2 * kTcN + 32 * wg);
#pragma unroll
      for (int h = 0; h < 4; ++h) {  // 4 column pairs at a time
        uint32_t u[8], v[8];
        tmem_ld8x2(ta + 8 * h, ta + kTcN + 8 * h, u, v);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int pl = 16 * wg + 4 * h + q;
          // e^{i (sx x + sy y)}; reduced phases: |sx x + sy y| <= 2 pi
          float er, ei;
          const float2 xy = sT[pl * kTcLd + rl];
          __sincosf(fmaf(sgx, xy.x, sgy * xy.y), &ei, &er);
          // column j: e;  mirror column: conj(e) (the z phasor is applied by turn)
          const float ur = __uint_as_float(u[2 * q]), ui = __uint_as_float(u[2 * q + 1]);
          const float vr = __uint_as_float(v[2 * q]), vi = __uint_as_float(v[2 * q + 1]);
          const float y1r = ur + vr, y1i = ui + vi, y2r = ur - vr, y2i = ui - vi;
          acc[4 * h + q][0][0] += y1r * er - y1i * ei;
          acc[4 * h + q][0][1] += y1r * ei + y1i * er;
          acc[4 * h + q][1][0] += y2r * er + y2i * ei;
          acc[4 * h + q][1][1] += y2i * er - y2r * ei;
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;");
      mbar_arrive(smem_addr(&acce[b]));
    }
    if (turned)
      turn(ez.x, -ez.y);
    else
      turn(ez.x, ez.y);
    if (!ok) {
      *abort_flag = 1;
      if (lane == 0) atomicCAS(err, 0, 1);
    }
    // all epilogue warps agree (ok everywhere) before the stage space is reused
    uint32_t all_ok;
    asm volatile("{\n.reg .pred p, q;\nsetp.ne.u32 q, %1, 0;\nbar.red.and.pred p, 1, %2, q;\nselp.u32 %0, 1, 0, p;\n}\n"
                 : "=r"(all_ok)
                 : "r"(ok ? 1u : 0u), "r"(kTcEpiWarps * 32)
                 : "memory");
    if (all_ok) {
      // transpose through shared memory: row rl, pairs (16 wg + q) and 64 + (16 wg + q)
      float2 *sO = (float2 *)smem_tc;  // [128][kTcLd]
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        sO[rl * kTcLd + 16 * wg + q] = make_float2(acc[q][0][0], acc[q][0][1]);
        sO[rl * kTcLd + kTcPairs + 16 * wg + q] = make_float2(acc[q][1][0], acc[q][1][1]);
      }
      asm volatile("bar.sync 1, %0;" ::"r"(kTcEpiWarps * 32));
      // warp w stores rows w, w + 16, ...: 64 consecutive packed pairs of j,
      // then of j' (a chunk's pairs may belong to several components)
      float2 *out = parent + ((int64_t)slot * n_parent + p) * 6 * (int64_t)Rp * phi;
      int64_t pofs[2];  // per lane half k & 1: component offset + column of the pair
      bool pok[2];
#pragma unroll
      for (int k = 0; k < 2; ++k) {
        const int pp = nc * kTcPairs + 32 * k + lane, comp = pp / span;
        pok[k] = pp < npairs;
        pofs[k] = (int64_t)comp * Rp * phi + (pp - comp * span);
      }
      for (int row = warp; row < 128; row += kTcEpiWarps) {
        const int rg = mtile * 128 + row;
        if (rg >= Rp) break;
#pragma unroll
        for (int k = 0; k < 4; ++k)
          if (pok[k & 1])
            out[pofs[k & 1] + (int64_t)rg * phi + (k >> 1) * span] = sO[row * kTcLd + (k >> 1) * kTcPairs +
                                                                         32 * (k & 1) + lane];
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();  // every role done
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcTmemCols));
  }
}

po_status init_theta_tc_attributes() {
  PO_CUDA(cudaFuncSetAttribute(k_theta_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, TcPlan::smem));
  return PO_OK;
}

// Columns of the core-matrix child operands: the six packed component patterns
// of a child (6 x 2 x Phi/2 real columns) rounded up to whole column chunks of
// the CTA.
int theta_tc_npad(int phi) { return (6 * phi + kTcN - 1) / kTcN * kTcN; }

po_status launch_theta_tc(const uint8_t *mid, float2 *parent, const int32_t *child_table, int64_t n_parent,
                          int64_t n_child, int phi, int Kr, int Rp, const uint8_t *Atc, const float4 *trans,
                          int n_slots, int G, int *err, size_t mid_bytes, size_t atc_bytes, cudaStream_t st,
                          int withhold) {
  if (n_parent <= 0 || n_slots <= 0) return PO_OK;
  if (phi % 2 || Kr % kTcKC || Kr <= 0) return fail(PO_ERR_INTERNAL, "tcgen05 theta pass: grid");
  const int MT = (Rp + 127) / 128, n_nc = (6 * (phi / 2) + kTcPairs - 1) / kTcPairs;
  const int64_t n_task = (int64_t)n_slots * n_parent * n_nc;
  const int64_t gx = n_task * MT;
  if (gx > 2147483647LL) return fail(PO_ERR_UNSUPPORTED, "too many nodes for one launch");
  k_theta_tc<<<(unsigned)gx, kTcThreads, TcPlan::smem, st>>>(mid, parent, child_table, n_parent, n_child, phi, Kr,
                                                         theta_tc_npad(phi), Rp, Atc, trans, G, n_nc, n_task, err,
                                                         mid_bytes, atc_bytes, withhold);
  count_launch();
  PO_CUDA(cudaGetLastError());
  return PO_OK;
}

}  // namespace wavepo
