// po_leaf_tc.cu -- leaf far-field sums on the 5th-generation tensor cores
// (tcgen05, accumulators in tensor memory) for launches with many patterns
// per wavelength (incidences x polarisations).
//
// Replaces the same reference code as k_leaf_mma (util/fields.h:2-50 with the
// per-leaf reduce of compareMie/sphere.cu:603-658, currents of
// util/tangentplane.h:84 and fields.h:123,147).  For one leaf and one
// wavelength
//   F_j(d) = sum_p exp(i s_d.u_p) C_pj,   u_p = k (x_p - c_leaf),
// j = (slot, component) over all G slots of the launch, is computed as two
// real GEMMs with the points as K:
//   D1 = Acos B,  D2 = Asin B,   Acos[d][p] = cos(s_d.u_p), Asin = sin,
//   B[p][2j] = Re C_pj, B[p][2j+1] = Im C_pj,
//   Re F_j = D1[2j] - D2[2j+1],  Im F_j = D1[2j+1] + D2[2j],
// every operand split into bf16 hi + lo and multiplied as hi*hi + hi*lo +
// lo*hi with FP32 accumulation (6 tcgen05.mma of 128 x 128 x 16 per chunk of
// 16 points).  The phase matrix is generated once per (leaf, wavelength)
// and serves every column tile of 64 complex columns (leaves of at most
// kLtRes chunks), where the warp-level kernel regenerates it for every 4
// slots.
//
// Two kernels:
//  * k_leaf_tc_operands: per chunk of 16 points of a leaf (leaves padded to
//    whole chunks), the currents of all G slots split into bf16 hi + lo in the
//    UMMA K-major core-matrix layout, one contiguous 8-KB block per column
//    tile, and the chunk's scaled offsets u = k (x - c) (zero for padding);
//  * k_leaf_tc: one CTA per (leaf, wavelength) walking (direction tile m,
//    column tile n, point chunk k) with four roles (a depth-0 solve is one
//    leaf of all points, its direction tiles spread over msplit CTAs) --
//      - 4 producer warps (thread = direction row): cos and sin of the
//        chunk's phases, split, stored in the core-matrix A layout.  The
//        phases do not depend on the column tile, so for a leaf of at most
//        kLtRes chunks the chunks of direction tile m are made once and serve
//        all column tiles; larger leaves remake them for every (m, n) through
//        the slots as a ring;
//      - a copy thread: one bulk copy (cp.async.bulk) of the 8-KB B block of
//        every (n, k) step into a 3-stage ring;
//      - an MMA thread: the 6 products per step into D1 / D2 in tensor memory
//        (256 columns), releasing a phase slot after its last column tile;
//      - 8 epilogue warps (thread = TMEM lane = direction, two warps per lane
//        quarter on alternate 16-column blocks): combine D1 and D2 into the
//        64 complex columns of the tile and store them (consecutive
//        directions per warp: 256-B runs).
//    Two CTAs per SM (104 KB of shared memory each), so that one CTA's
//    epilogue overlaps the other's products.
// Every wait is bounded in time (error word 1) and aborts the other roles;
// the copy and MMA threads wait for their last copy / commit before the CTA
// exits.  `withhold` (a self-test switch) leaves the first stage's copy
// unissued so that the timeout path runs.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>

#include "po_common.cuh"
#include "po_internal.h"
#include "po_kernels.h"
#include "po_tc_common.cuh"

namespace wavepo {

namespace {

using namespace tc;

constexpr int kLtKC = 16;                          // points per chunk
constexpr int kLtN = 128;                          // real columns per tile (64 complex)
constexpr int kLtAStage = 4 * 128 * kLtKC * 2;     // Acos hi, lo, Asin hi, lo of one chunk: 16 KB
constexpr int kLtBBlock = 2 * kLtN * kLtKC * 2;    // B hi, lo of one (chunk, column tile): 8 KB
constexpr int kLtBStages = 3;
constexpr int kLtEpiWarps = 8, kLtProdWarps = 4;
constexpr int kLtProd0 = kLtEpiWarps;              // warps 8..11: thread = direction row
constexpr int kLtMmaWarp = kLtEpiWarps + kLtProdWarps, kLtCopyWarp = kLtMmaWarp + 1;
constexpr int kLtThreads = 32 * (kLtCopyWarp + 1);
// Shared-memory and tensor-memory plan of one variant: ABUF direction tiles of
// RES phase chunks in flight, ACC accumulator tiles (D1, D2) in tensor memory;
// CTAS resident CTAs per SM.
template <int ABUF, int RES, int ACC>
struct LtPlan {
  static constexpr int res = RES, abuf = ABUF, acc = ACC;
  static constexpr int slots = ABUF * RES;
  static constexpr uint32_t tmem_cols = ACC * 2 * kLtN;
  static constexpr int bar_off = slots * kLtAStage + kLtBStages * kLtBBlock;
  static constexpr int smem = bar_off + 512;
  static constexpr int ctas = ACC == 1 ? 2 : 1;
};
// Two CTAs per SM, one direction tile of up to 5 resident chunks each (62% of
// the fiber segment's leaf work; its leaves have 1-8 chunks): measured as fast
// as a plan of one CTA per SM with two direction tiles of 6 chunks and two
// accumulator tiles in flight (51.5 against 61.7 ms per fiber wavelength),
// because the epilogue, not the phase generation, bounds the kernel.
using LtMain = LtPlan<1, 5, 1>;
static_assert(2 * (LtMain::smem + 1024) <= 228 * 1024, "shared memory");
constexpr float kLtFastPhase = 16.f;               // |s.u| below this: no range reduction (as k_leaf_mma)

// byte of element (row r, k < 16) in one 128-row (or 128-column) K-major
// operand of 16 K values: core matrices of 8 rows x 16 B, K-adjacent at 128 B,
// row groups at 256 B
__host__ __device__ __forceinline__ uint32_t core_off(int r, int k) {
  return (uint32_t)((((r >> 3) * 2 + (k >> 3)) * 128) + (r & 7) * 16 + (k & 7) * 2);
}

}  // namespace

int leaf_tc_col_tiles(int G) { return (12 * std::min(G, kLeafTcMaxSlots) + kLtN - 1) / kLtN; }
size_t leaf_tc_block_bytes() { return kLtBBlock; }

// grid (n_chunks, n_lambda), 256 threads.  bop[lam][chunk][tile] 8-KB blocks,
// uop[lam][chunk][16] float4.
__global__ void __launch_bounds__(256) k_leaf_tc_operands(
    const float *__restrict__ x, const float *__restrict__ y, const float *__restrict__ z,
    const float *__restrict__ nx, const float *__restrict__ ny, const float *__restrict__ nz,
    const float *__restrict__ area, const int32_t *__restrict__ leaf_begin, const int32_t *__restrict__ kc0,
    const int32_t *__restrict__ chunk_leaf, const double *__restrict__ leaf_center,
    const SlotParams<float> *__restrict__ slots, int Gtot, int g0, int G, int NT, int64_t n_chunks,
    uint8_t *__restrict__ bop, float4 *__restrict__ uop) {
  extern __shared__ __align__(16) uint8_t smem_lo[];  // [NT][kLtBBlock]
  const int64_t kc = blockIdx.x;
  const int lam = blockIdx.y;
  const int leaf = chunk_leaf[kc];
  const int p0 = leaf_begin[leaf] + (int)(kc - kc0[leaf]) * kLtKC, pe = leaf_begin[leaf + 1];
  const SlotParams<float> *sl = slots + (int64_t)lam * Gtot + g0;
  const int words = NT * kLtBBlock / 16;
  uint4 *s4 = (uint4 *)smem_lo;
  for (int i = threadIdx.x; i < words; i += blockDim.x) s4[i] = make_uint4(0u, 0u, 0u, 0u);
  if (threadIdx.x < kLtKC) {  // lanes 0..15 of warp 0
    const int p = p0 + threadIdx.x;
    float4 u = make_float4(0.f, 0.f, 0.f, 0.f);
    if (p < pe) {
      const double k0 = sl[0].k0d;
      u = make_float4((float)(k0 * ((double)x[p] - leaf_center[3 * leaf])),
                      (float)(k0 * ((double)y[p] - leaf_center[3 * leaf + 1])),
                      (float)(k0 * ((double)z[p] - leaf_center[3 * leaf + 2])), 0.f);
    }
    // w = 1 on every point of a chunk where some |s.u| <= |u| may exceed the fast-phase range
    const bool big = !(u.x * u.x + u.y * u.y + u.z * u.z <= kLtFastPhase * kLtFastPhase);
    u.w = __any_sync(0x0000ffffu, big) ? 1.f : 0.f;
    uop[((int64_t)lam * n_chunks + kc) * kLtKC + threadIdx.x] = u;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < kLtKC * G; e += blockDim.x) {
    const int k = e % kLtKC, s = e / kLtKC, p = p0 + k;
    if (p >= pe) continue;
    cx<float> c[6];
    tangent_plane<float>(sl[s], x[p], y[p], z[p], nx[p], ny[p], nz[p], area[p], c);
#pragma unroll
    for (int q = 0; q < 6; ++q) {
#pragma unroll
      for (int part = 0; part < 2; ++part) {
        const float v = part ? c[q].im : c[q].re;
        const __nv_bfloat16 h = __float2bfloat16_rn(v);
        const __nv_bfloat16 l = __float2bfloat16_rn(v - __bfloat162float(h));
        const int n = 12 * s + 2 * q + part, t = n / kLtN, nn = n % kLtN;
        uint8_t *blk = smem_lo + (size_t)t * kLtBBlock;
        *(__nv_bfloat16 *)(blk + core_off(nn, k)) = h;
        *(__nv_bfloat16 *)(blk + kLtBBlock / 2 + core_off(nn, k)) = l;
      }
    }
  }
  __syncthreads();
  uint4 *dst = (uint4 *)(bop + ((size_t)lam * n_chunks + kc) * (size_t)NT * kLtBBlock);
  for (int i = threadIdx.x; i < words; i += blockDim.x) dst[i] = s4[i];
}

// grid (n_leaves, n_lambda), kLtThreads threads, P::smem bytes.
//
// Work order: direction tiles m, column tiles n, chunks kc.  A leaf of at
// most kLtRes chunks ("resident") has the phase chunks of direction tile m
// generated once into A slots (m & 1) kLtRes + kc and multiplied with every
// column tile before the slots are released (the phases do not depend on the
// column); a larger leaf regenerates them for every (m, n, kc) step through the
// slots as a ring.  A slot fill is counted per slot, so that each wait knows
// its phase: resident fill index m >> 1, ring fill index g / kLtASlots for
// production g.  Accumulators: two tiles (D1, D2) in tensor memory, tile t in
// buffer t & 1, so that the epilogue of one tile overlaps the products of the
// next.
template <class P>
__global__ void __launch_bounds__(kLtThreads, P::ctas) k_leaf_tc(
    const uint8_t *__restrict__ bop, const float4 *__restrict__ uop, const int32_t *__restrict__ kc0,
    int64_t n_chunks, const float4 *__restrict__ dirs, int ndir, int64_t n_leaves, int Gtot, int g0, int G, int NT,
    float2 *__restrict__ out, int *__restrict__ err, int withhold, int msplit) {
  extern __shared__ __align__(1024) uint8_t smem_lt[];
  constexpr int kLtRes = P::res, kLtASlots = P::slots, kAcc = P::acc;
  uint8_t *sA = smem_lt;                                   // [kLtASlots][kLtAStage]
  uint8_t *sB = smem_lt + kLtASlots * kLtAStage;           // [kLtBStages][kLtBBlock]
  uint64_t *afull = (uint64_t *)(smem_lt + P::bar_off), *aempty = afull + kLtASlots, *bfull = aempty + kLtASlots,
           *bempty = bfull + kLtBStages, *accf = bempty + kLtBStages, *acce = accf + kAcc;
  uint32_t *tmem_slot = (uint32_t *)(acce + kAcc);
  volatile int *abort_flag = (volatile int *)(tmem_slot + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // CTA = (leaf, direction tiles m0, m0 + msplit, ...): msplit > 1 spreads
  // one large leaf (the whole point set of a depth-0 solve) over many CTAs
  const int64_t leaf = blockIdx.x / msplit;
  const int m0 = (int)(blockIdx.x % msplit);
  const int lam = blockIdx.y;
  const int c0 = kc0[leaf], KCl = kc0[leaf + 1] - c0;
  const int MT = (ndir + 127) / 128;
  const int MTl = m0 < MT ? (MT - m0 + msplit - 1) / msplit : 0;  // direction tiles of this CTA
  const int ntiles = MTl * NT;
  const bool resident = KCl <= kLtRes;
  if (tid == 0) {
    for (int q = 0; q < kLtASlots; ++q) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(&afull[q])), "r"(32 * kLtProdWarps));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&aempty[q])));
    }
    for (int q = 0; q < kLtBStages; ++q) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&bfull[q])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&bempty[q])));
    }
    for (int q = 0; q < kAcc; ++q) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&accf[q])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(&acce[q])), "r"(32 * kLtEpiWarps));
    }
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  if (warp == kLtMmaWarp) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tmem_slot)),
                 "r"(P::tmem_cols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = *tmem_slot;
  const int64_t slot_stride = n_leaves * 6 * (int64_t)ndir;
  float2 *obase = out + ((int64_t)lam * Gtot + g0) * slot_stride + leaf * 6 * (int64_t)ndir;

  if (warp == kLtCopyWarp) {
    // ---- copy role: the B block of every (m, n, kc) step ----
    if (lane == 0 && KCl > 0) {
      bool ok = true;
      int64_t step = 0, last[kLtBStages];
#pragma unroll
      for (int q = 0; q < kLtBStages; ++q) last[q] = -1;
      const uint8_t *bl = bop + ((size_t)lam * n_chunks + c0) * (size_t)NT * kLtBBlock;
      for (int t = 0; t < ntiles && ok; ++t) {
        const int n = t % NT;
        for (int kc = 0; kc < KCl; ++kc, ++step) {
          const int q = (int)(step % kLtBStages);
          if (step >= kLtBStages &&
              !mbar_wait(smem_addr(&bempty[q]), (uint32_t)(((step / kLtBStages) - 1) & 1), abort_flag)) {
            ok = false;
            break;
          }
          if (withhold && step == 0) continue;  // self-test: stage 0 never filled, its consumers give up
          mbar_expect_tx(smem_addr(&bfull[q]), kLtBBlock);
          bulk_copy(smem_addr(sB + q * kLtBBlock), bl + ((size_t)kc * NT + n) * kLtBBlock, kLtBBlock,
                    smem_addr(&bfull[q]));
          last[q] = step;
        }
      }
      if (!ok && !*abort_flag) {
        *abort_flag = 1;
        atomicCAS(err, 0, 1);
      }
      // every copy lands before the CTA exits
      for (int q = 0; q < kLtBStages; ++q)
        if (last[q] >= 0) (void)mbar_wait(smem_addr(&bfull[q]), (uint32_t)((last[q] / kLtBStages) & 1), nullptr);
    }
    __syncwarp();
  } else if (warp == kLtMmaWarp) {
    // ---- MMA role ----
    if (lane == 0 && KCl > 0) {
      // D f32, A and B bf16, both K-major, N = kLtN, M = 128
      const uint32_t idesc =
          (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kLtN >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
      const uint64_t ad0 = tc_desc(smem_addr(sA)), bd0 = tc_desc(smem_addr(sB));
      constexpr uint64_t mA = (kLtAStage / 4) >> 4, mB = (kLtBBlock / 2) >> 4;  // one matrix, descriptor units
      bool ok = true;
      int64_t step = 0, g = 0, bcommitted = 0;
      int alast[kLtASlots];  // fill index of each A slot's latest release
#pragma unroll
      for (int q = 0; q < kLtASlots; ++q) alast[q] = -1;
      int tiles_done = 0;
      for (int t = 0; t < ntiles && ok; ++t) {
        const int m = t / NT, n = t % NT, buf = t % kAcc;  // m: this CTA's tile index
        if (t >= kAcc && !mbar_wait(smem_addr(&acce[buf]), (uint32_t)(((t / kAcc) - 1) & 1), abort_flag)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint32_t d1 = tmem + (uint32_t)(buf * 2 * kLtN), d2 = d1 + kLtN;
        for (int kc = 0; kc < KCl; ++kc, ++step) {
          const int slot = resident ? (m % P::abuf) * kLtRes + kc : (int)(g % kLtASlots);
          const int fill = resident ? m / P::abuf : (int)(g / kLtASlots);
          const int q = (int)(step % kLtBStages);
          if (!mbar_wait(smem_addr(&afull[slot]), (uint32_t)(fill & 1), abort_flag) ||
              !mbar_wait(smem_addr(&bfull[q]), (uint32_t)((step / kLtBStages) & 1), abort_flag)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;");
          const uint64_t ad = ad0 + (uint64_t)slot * (kLtAStage >> 4), bd = bd0 + (uint64_t)q * (kLtBBlock >> 4);
          const uint32_t first = kc == 0 ? 0u : 1u;
          tc_mma(d1, ad, bd, idesc, first);               // Acos hi * B hi
          tc_mma(d2, ad + 2 * mA, bd, idesc, first);      // Asin hi * B hi
          tc_mma(d1, ad, bd + mB, idesc, 1u);             // Acos hi * B lo
          tc_mma(d2, ad + 2 * mA, bd + mB, idesc, 1u);    // Asin hi * B lo
          tc_mma(d1, ad + mA, bd, idesc, 1u);             // Acos lo * B hi
          tc_mma(d2, ad + 3 * mA, bd, idesc, 1u);         // Asin lo * B hi
          tc_commit(smem_addr(&bempty[q]));
          bcommitted = step + 1;
          if (!resident || n == NT - 1) {  // the slot's last use
            tc_commit(smem_addr(&aempty[slot]));
            alast[slot] = fill;
          }
          if (!resident) ++g;
        }
        if (!ok) break;
        tc_commit(smem_addr(&accf[buf]));
        tiles_done = t + 1;
      }
      if (!ok && !*abort_flag) {
        *abort_flag = 1;
        atomicCAS(err, 0, 1);
      }
      // every commit arrive lands before the CTA exits (latest phase of each barrier)
      for (int q = 0; q < kLtBStages; ++q) {
        const int64_t ls = bcommitted - 1 - (((bcommitted - 1 - q) % kLtBStages) + kLtBStages) % kLtBStages;
        if (ls >= 0) (void)mbar_wait(smem_addr(&bempty[q]), (uint32_t)((ls / kLtBStages) & 1), nullptr);
      }
      for (int q = 0; q < kLtASlots; ++q)
        if (alast[q] >= 0) (void)mbar_wait(smem_addr(&aempty[q]), (uint32_t)(alast[q] & 1), nullptr);
      for (int t = tiles_done - kAcc > 0 ? tiles_done - kAcc : 0; t < tiles_done; ++t)
        (void)mbar_wait(smem_addr(&accf[t % kAcc]), (uint32_t)((t / kAcc) & 1), nullptr);
    }
    __syncwarp();
  } else if (warp >= kLtProd0) {
    // ---- producer role: thread = direction row of the tile ----
    const int r = tid - 32 * kLtProd0;
    bool ok = true;
    int64_t g = 0;
    const float4 *ul = uop + ((int64_t)lam * n_chunks + c0) * kLtKC;
    // phases of the 16 points of chunk kc for direction sd into A slot `slot`
    auto produce = [&](const float4 &sd, int kc, int slot) {
      const float4 *uc = ul + kc * kLtKC;
      const bool big = __ldg(uc).w != 0.f;  // the same for every thread: no divergence
      uint8_t *st = sA + slot * kLtAStage;
#pragma unroll
      for (int kb = 0; kb < 2; ++kb) {  // points 8 kb .. 8 kb + 7
        float4 uu[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) uu[i] = __ldg(uc + 8 * kb + i);
        uint32_t ch[4], cl[4], sh[4], sl[4];
#pragma unroll
        for (int w = 0; w < 4; ++w) {
          float sn[2], cs[2];
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const float4 u = uu[2 * w + h];
            const float ph = fmaf(sd.x, u.x, fmaf(sd.y, u.y, sd.z * u.z));
            if (big)
              sincos_small(ph, &sn[h], &cs[h]);
            else
              __sincosf(ph, &sn[h], &cs[h]);
          }
          split_bf16x2(cs[0], cs[1], ch[w], cl[w]);
          split_bf16x2(sn[0], sn[1], sh[w], sl[w]);
        }
        const uint32_t o = core_off(r, 8 * kb);
        *(uint4 *)(st + o) = make_uint4(ch[0], ch[1], ch[2], ch[3]);
        *(uint4 *)(st + 4096 + o) = make_uint4(cl[0], cl[1], cl[2], cl[3]);
        *(uint4 *)(st + 8192 + o) = make_uint4(sh[0], sh[1], sh[2], sh[3]);
        *(uint4 *)(st + 12288 + o) = make_uint4(sl[0], sl[1], sl[2], sl[3]);
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      mbar_arrive(smem_addr(&afull[slot]));
    };
    for (int m = 0; m < MTl && ok && KCl > 0; ++m) {  // this CTA's tile index
      const float4 sd = __ldg(dirs + min((m0 + m * msplit) * 128 + r, ndir - 1));
      const int nrep = resident ? 1 : NT;  // a resident tile's chunks serve every column tile
      for (int rep = 0; rep < nrep && ok; ++rep)
        for (int kc = 0; kc < KCl; ++kc) {
          const int slot = resident ? (m % P::abuf) * kLtRes + kc : (int)(g % kLtASlots);
          const int fill = resident ? m / P::abuf : (int)(g / kLtASlots);
          if (fill >= 1 && !mbar_wait(smem_addr(&aempty[slot]), (uint32_t)((fill - 1) & 1), abort_flag)) {
            ok = false;
            break;
          }
          produce(sd, kc, slot);
          if (!resident) ++g;
        }
    }
    if (!ok) *abort_flag = 1;
  } else {
    // ---- epilogue role: thread = tensor-memory lane = direction of the tile;
    // the two warps of a lane quarter take alternate 16-column blocks ----
    const int quarter = warp & 3, eh = warp >> 2, r = 32 * quarter + lane;
    bool ok = true;
    for (int t = 0; t < ntiles && ok; ++t) {
      const int m = m0 + (t / NT) * msplit, n = t % NT, d = m * 128 + r, buf = t % kAcc;
      const uint32_t ta = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(buf * 2 * kLtN);
      if (KCl > 0) {
        ok = __all_sync(0xffffffffu, mbar_wait(smem_addr(&accf[buf]), (uint32_t)((t / kAcc) & 1), abort_flag)) != 0;
        if (!ok) break;
        asm volatile("tcgen05.fence::after_thread_sync;");
      }
#pragma unroll 1
      for (int b = eh; b < kLtN / 16; b += kLtEpiWarps / 4) {
        uint32_t v[16], w[16];
        if (KCl > 0) {
          tmem_ld16x2(ta + 16 * b, ta + kLtN + 16 * b, v, w);
        } else {
#pragma unroll
          for (int q = 0; q < 16; ++q) v[q] = w[q] = 0u;
        }
        if (d >= ndir) continue;
        // complex column j = 6 slot + component, walked without divisions
        const int j0 = n * (kLtN / 2) + 8 * b, nj = min(8, 6 * G - j0);
        int comp = j0 % 6;
        float2 *po = obase + (int64_t)(j0 / 6) * slot_stride + (int64_t)comp * ndir + d;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          if (q >= nj) break;
          const float re = __uint_as_float(v[2 * q]) - __uint_as_float(w[2 * q + 1]);
          const float im = __uint_as_float(v[2 * q + 1]) + __uint_as_float(w[2 * q]);
          *po = make_float2(re, im);
          po += ndir;
          if (++comp == 6) {
            comp = 0;
            po += slot_stride - 6 * (int64_t)ndir;
          }
        }
      }
      if (KCl > 0) {
        asm volatile("tcgen05.fence::before_thread_sync;");
        mbar_arrive(smem_addr(&acce[buf]));
      }
    }
    if (!ok) {
      *abort_flag = 1;
      if (lane == 0) atomicCAS(err, 0, 1);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();  // every role done
  if (warp == kLtMmaWarp) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(P::tmem_cols));
  }
}

po_status init_leaf_tc_attributes() {
  PO_CUDA(cudaFuncSetAttribute(k_leaf_tc<LtMain>, cudaFuncAttributeMaxDynamicSharedMemorySize, LtMain::smem));
  PO_CUDA(cudaFuncSetAttribute(k_leaf_tc<LtMain>, cudaFuncAttributePreferredSharedMemoryCarveout,
                               (int)cudaSharedmemCarveoutMaxShared));
  PO_CUDA(cudaFuncSetAttribute(k_leaf_tc_operands, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               leaf_tc_col_tiles(kLeafTcMaxSlots) * kLtBBlock));
  return PO_OK;
}

po_status launch_leaf_tc(const float *const g[7], const int32_t *leaf_begin, const int32_t *kc0,
                         const int32_t *chunk_leaf, int64_t n_chunks, const double *leaf_center, int64_t n_leaves,
                         const SlotParams<float> *slots_dev, int n_lambda, int Gtot, int g0, int G,
                         const float4 *dirs, int ndir, uint8_t *bop, size_t bop_bytes, float4 *uop,
                         size_t uop_bytes, float2 *out, int *err, cudaStream_t st, int group, int withhold,
                         int msplit) {
  if (n_leaves <= 0 || n_lambda <= 0 || G <= 0) return PO_OK;
  if (group < 8 || group > kLeafTcMaxSlots || group % 8 != 0)
    return fail(PO_ERR_INTERNAL, "tcgen05 leaf: slots per pass");
  if (n_chunks <= 0 || n_lambda > 65535 || msplit < 1 || n_leaves * msplit > 2147483647LL ||
      n_chunks > 2147483647LL)
    return fail(PO_ERR_INTERNAL, "tcgen05 leaf: launch shape");
  if ((size_t)n_lambda * n_chunks * leaf_tc_col_tiles(std::min(G, group)) * kLtBBlock > bop_bytes ||
      (size_t)n_lambda * n_chunks * kLtKC * sizeof(float4) > uop_bytes)
    return fail(PO_ERR_INTERNAL, "tcgen05 leaf: operand buffers");
  // slots in groups of at most `group` (kLeafTcMaxSlots = 6 column tiles); the
  // operand buffers are reused group after group in stream order
  for (int gs = 0; gs < G; gs += group) {
    const int gc = std::min(group, G - gs), NT = leaf_tc_col_tiles(gc);
    k_leaf_tc_operands<<<dim3((unsigned)n_chunks, (unsigned)n_lambda), 256, NT * kLtBBlock, st>>>(
        g[0], g[1], g[2], g[3], g[4], g[5], g[6], leaf_begin, kc0, chunk_leaf, leaf_center, slots_dev, Gtot,
        g0 + gs, gc, NT, n_chunks, bop, uop);
    count_launch();
    k_leaf_tc<LtMain><<<dim3((unsigned)(n_leaves * msplit), (unsigned)n_lambda), kLtThreads, LtMain::smem, st>>>(
        bop, uop, kc0, n_chunks, dirs, ndir, n_leaves, Gtot, g0 + gs, gc, NT, out, err, withhold, msplit);
    count_launch();
  }
  PO_CUDA(cudaGetLastError());
  return PO_OK;
}

}  // namespace wavepo
