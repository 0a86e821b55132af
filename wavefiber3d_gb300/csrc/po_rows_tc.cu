// po_rows_tc.cu -- phi pass on the 5th-generation tensor cores (tcgen05,
// accumulators in tensor memory) for the levels whose theta pass runs on
// tcgen05 (po_theta_tc.cu), writing its core-matrix operand layout.
//
// Same map as k_interp_rows_mma<2> (the phi half of interpFFT,
// util/interpolation.h:17-45): every child row h (Pc columns) becomes Pp
// parent columns, h'_n = sum_k Phi[k][n] h_k, and each mirror pair
// (j, j + Pp/2) is stored as S = h'_j + h'_j', D = h'_j - h'_j', split into
// bf16 hi + lo.  As a GEMM: M = 128 rows = 64 complex rows with their real
// and imaginary parts interleaved (row 2i, 2i + 1), K = Pc, N = one tile of
// the parent columns in pair order (column 2 jl + w).
//
// CTA (persistent over blocks of 64 output rows, one N tile): 9 warps.
//  * MMA warp (one thread): bulk-copies the whole phi tile of its N tile into
//    shared memory once, then per 16-row K chunk issues hi*hi + hi*lo + lo*hi
//    (3 tcgen05.mma of 128 x ntn x 16) into one of two accumulators in tensor
//    memory (one per row block parity) and commits the chunk's stage and,
//    after the last chunk, the accumulator;
//  * 4 converter warps (8 with the wide tiles, two groups on alternate K
//    chunks): load the FP32 rows of each K chunk (16-byte loads, one or two
//    of the group's chunks ahead into a statically indexed ring of registers,
//    by the length of the K loop),
//    split them into bf16 hi + lo and store them in the core-matrix A layout
//    of a 4-stage ring (padding rows of the output patterns and columns past
//    Pc are zero);
//  * 4 or 8 epilogue warps (tensor-memory lane = M row = one part of one
//    complex row; for tiles wider than 128 columns the two warps of a lane
//    quarter take alternate 16-column blocks and read two blocks per wait;
//    narrower tiles keep 4 warps, so that two CTAs fit an SM, and one block
//    per wait): store the four bf16 values of every pair at their place in
//    the theta pass's operand layout.
// Every wait is bounded in time (error word 1); the phi tile and the output
// must lie inside their buffers (checked on the host); the MMA thread waits
// for its last commit arrives before the CTA exits.
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

// EW epilogue warps (4, or 8 = two per tensor-memory lane quarter for wide
// tiles); converter warps in groups of 4 that take alternate K chunks (two
// groups with the wide tiles, one CTA per SM: twice the loads in flight)
template <int EW>
struct RtWarps {
  static constexpr int cvt = EW == 8 ? 8 : 4;
  static constexpr int groups = cvt / 4;
  static constexpr int ctl = EW + cvt;  // the phi-tile / MMA warp
  static constexpr int threads = 32 * (ctl + 1);
};
constexpr int kRtStages = 4;
constexpr int kRtAStage = 2 * 128 * 16 * 2;  // bf16 hi + lo of 128 rows x 16: 8 KB
constexpr int kRtMaxSmem = 216 * 1024;

__host__ __device__ inline int rows_tc_smem(int KC, int ntn) { return KC * 64 * ntn + kRtStages * kRtAStage + 128; }

__device__ __forceinline__ uint32_t a_off(int m, int k) {  // byte of (row m, k < 16) in one A matrix
  return (uint32_t)((((m >> 3) * 2 + (k >> 3)) * 128) + (m & 7) * 16 + (k & 7) * 2);
}

}  // namespace

// N tiling of the pass from Pc to Pp columns: the fewest tiles whose phi tile
// (Kc x ntn, hi + lo) fits shared memory next to the A ring, ntn <= 256
// columns (a multiple of 16) per tile.  False when Pp is odd or Pc is odd
// (16-byte row loads) or no tiling fits.
bool rows_tc_plan(int Pc, int Pp, int &ntn, int &n_nt) {
  if (Pc <= 0 || Pp <= 0 || (Pc & 1) || (Pp & 1)) return false;
  const int half = Pp / 2, KC = (Pc + 15) / 16;
  for (n_nt = 1; n_nt <= 16; ++n_nt) {
    ntn = (2 * ((half + n_nt - 1) / n_nt) + 15) / 16 * 16;
    if (ntn <= 256 && rows_tc_smem(KC, ntn) <= kRtMaxSmem) return true;
  }
  return false;
}

// NB: converter register buffers (chunks of 4 x 16 B per thread)
template <int EW, int NB>
__global__ void __launch_bounds__(RtWarps<EW>::threads, EW == 4 ? 2 : 1) k_rows_tc(
    const float2 *__restrict__ src, uint8_t *__restrict__ dst, int64_t n_rows_out, int Rc, int Rr, int Pc, int KC,
    int half, int npad, int ntn, int n_nt, const uint8_t *__restrict__ Bt, uint32_t tcols, int *__restrict__ err) {
  extern __shared__ __align__(128) uint8_t smem_rt[];
  const int b_bytes = KC * 64 * ntn;
  uint8_t *sB = smem_rt, *sA = smem_rt + b_bytes;
  uint64_t *bfull = (uint64_t *)(sA + kRtStages * kRtAStage), *afull = bfull + 1, *aempty = afull + kRtStages,
           *accf = aempty + kRtStages, *acce = accf + 2;
  uint32_t *tmem_slot = (uint32_t *)(acce + 2);
  volatile int *abort_flag = (volatile int *)(tmem_slot + 1);
  constexpr int kRtEpiWarps = EW, kRtCtlWarp = RtWarps<EW>::ctl, NH = EW / 4;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nt = (int)(blockIdx.x % n_nt);
  const int64_t rb0 = blockIdx.x / n_nt, rb_step = gridDim.x / n_nt;
  const int64_t n_rb = (n_rows_out + 63) / 64;
  const int n_it = rb0 < n_rb ? (int)((n_rb - 1 - rb0) / rb_step + 1) : 0;  // row blocks of this CTA
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bfull)));
    for (int s = 0; s < kRtStages; ++s) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(&afull[s])), "r"(32 * 4));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&aempty[s])));
    }
    for (int b = 0; b < 2; ++b) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&accf[b])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(&acce[b])), "r"(32 * kRtEpiWarps));
    }
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tmem_slot)),
                 "r"(tcols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = *tmem_slot;

  if (warp == kRtCtlWarp) {
    // ---- phi tile + MMA role ----
    if (lane == 0 && n_it > 0) {
      bool ok = true;
      mbar_expect_tx(smem_addr(bfull), (uint32_t)b_bytes);
      bulk_copy(smem_addr(sB), Bt + (size_t)nt * b_bytes, (uint32_t)b_bytes, smem_addr(bfull));
      if (!mbar_wait(smem_addr(bfull), 0, abort_flag)) ok = false;
      asm volatile("tcgen05.fence::after_thread_sync;");
      // D f32, A and B bf16, both K-major, N = ntn, M = 128
      const uint32_t idesc =
          (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(ntn >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
      const uint64_t ad0 = tc_desc(smem_addr(sA)), bd0 = tc_desc(smem_addr(sB));
      int64_t g = 0, committed = 0;
      int done_it = 0;
      for (int it = 0; it < n_it && ok; ++it) {
        const int buf = it & 1;
        if (it >= 2 && !mbar_wait(smem_addr(&acce[buf]), ((it >> 1) - 1) & 1, abort_flag)) {
          ok = false;
          break;
        }
        const uint32_t d = tmem + (uint32_t)(buf * ntn);
        for (int kc = 0; kc < KC; ++kc, ++g) {
          const int s = (int)(g % kRtStages);
          if (!mbar_wait(smem_addr(&afull[s]), (uint32_t)((g / kRtStages) & 1), abort_flag)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;");
          const uint64_t ad = ad0 + (uint64_t)s * (kRtAStage >> 4);
          const uint64_t bd = bd0 + (uint64_t)kc * ((64 * ntn) >> 4);
          tc_mma(d, ad, bd, idesc, kc > 0 ? 1u : 0u);                      // hi * hi
          tc_mma(d, ad, bd + (uint64_t)(2 * ntn), idesc, 1u);              // hi * lo (B lo at +32 ntn B)
          tc_mma(d, ad + (uint64_t)(4096 >> 4), bd, idesc, 1u);            // lo * hi (A lo at +4 KB)
          tc_commit(smem_addr(&aempty[s]));
          committed = g + 1;
        }
        if (!ok) break;
        tc_commit(smem_addr(&accf[buf]));
        done_it = it + 1;
      }
      if (!ok && !*abort_flag) {
        *abort_flag = 1;
        atomicCAS(err, 0, 1);
      }
      // every commit arrive lands before the CTA exits (latest phase of each barrier)
      for (int s = 0; s < kRtStages; ++s) {
        const int64_t ls = committed - 1 - (((committed - 1 - s) % kRtStages) + kRtStages) % kRtStages;
        if (ls >= 0) (void)mbar_wait(smem_addr(&aempty[s]), (uint32_t)((ls / kRtStages) & 1), nullptr);
      }
      for (int it = done_it - 2 > 0 ? done_it - 2 : 0; it < done_it; ++it)
        (void)mbar_wait(smem_addr(&accf[it & 1]), (uint32_t)((it >> 1) & 1), nullptr);
      (void)mbar_wait(smem_addr(bfull), 0, nullptr);
    }
    __syncwarp();
  } else if (warp >= kRtEpiWarps) {
    // ---- converter role: FP32 rows -> split bf16 A chunks ----
    // group grp of 4 warps converts chunks grp, grp + NG, ...
    constexpr int NG = RtWarps<EW>::groups;
    const int grp = (tid - 32 * kRtEpiWarps) >> 7, ct = (tid - 32 * kRtEpiWarps) & 127;
    const int64_t n_chunks = (int64_t)n_it * KC;
    const int64_t n_local = n_chunks > grp ? (n_chunks - grp + NG - 1) / NG : 0;
    // source rows of this thread's two output rows (i and i + 32) of row block
    // it: one division per row block, cached across its chunks
    int64_t row_it = -1, srow[2];
    bool rowok[2];
    auto rows_of = [&](int it) {
      const int64_t r0 = (rb0 + it * rb_step) * 64 + (ct >> 2);
      int64_t pattern = r0 / Rr;
      int t = (int)(r0 - pattern * Rr);
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        if (h) {
          t += 32;
          while (t >= Rr) {
            t -= Rr;
            ++pattern;
          }
        }
        rowok[h] = r0 + 32 * h < n_rows_out && t < Rc;
        srow[h] = pattern * Rc + t;
      }
      row_it = it;
    };
    auto load_chunk = [&](int64_t gg, float4 (&v)[4]) {
#pragma unroll
      for (int pass = 0; pass < 4; ++pass) v[pass] = make_float4(0.f, 0.f, 0.f, 0.f);
      if (gg >= n_chunks) return;
      const int it = (int)(gg / KC), kc = (int)(gg - (int64_t)it * KC);
      if (it != row_it) rows_of(it);
#pragma unroll
      for (int pass = 0; pass < 4; ++pass) {
        const int k = kc * 16 + 2 * ((ct & 3) + 4 * (pass >> 1));
        if (rowok[pass & 1] && k < Pc) v[pass] = __ldg((const float4 *)(src + srow[pass & 1] * (int64_t)Pc + k));
      }
    };
    // a ring of kRtBufs register buffers, statically indexed (the loop over a
    // ring turn is unrolled): kRtBufs - 1 chunks are loading while one is
    // converted, and no buffer is copied, so no load is waited for early
    constexpr int kRtBufs = NB;
    float4 v[kRtBufs][4];
#pragma unroll
    for (int b = 0; b < kRtBufs - 1; ++b) load_chunk(grp + (int64_t)NG * b, v[b]);
    bool ok = true;
    for (int64_t i0 = 0; i0 < n_local && ok; i0 += kRtBufs) {
#pragma unroll
      for (int b = 0; b < kRtBufs; ++b) {
        const int64_t il = i0 + b, g = grp + (int64_t)NG * il;
        if (il >= n_local) break;
        load_chunk(g + (int64_t)NG * (kRtBufs - 1), v[(b + kRtBufs - 1) % kRtBufs]);
        const int s = (int)(g % kRtStages);
        if (g >= kRtStages &&
            !mbar_wait(smem_addr(&aempty[s]), (uint32_t)(((g / kRtStages) - 1) & 1), abort_flag)) {
          ok = false;
          break;
        }
        uint8_t *st = sA + s * kRtAStage;
#pragma unroll
        for (int pass = 0; pass < 4; ++pass) {
          const int i = (ct >> 2) + 32 * (pass & 1), kk = 2 * ((ct & 3) + 4 * (pass >> 1));
          uint32_t rh, rl, ih, il;
          split_bf16x2(v[b][pass].x, v[b][pass].z, rh, rl);  // real parts of columns k, k + 1
          split_bf16x2(v[b][pass].y, v[b][pass].w, ih, il);  // imaginary parts
          *(uint32_t *)(st + a_off(2 * i, kk)) = rh;
          *(uint32_t *)(st + 4096 + a_off(2 * i, kk)) = rl;
          *(uint32_t *)(st + a_off(2 * i + 1, kk)) = ih;
          *(uint32_t *)(st + 4096 + a_off(2 * i + 1, kk)) = il;
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_arrive(smem_addr(&afull[s]));
      }
    }
    if (!ok) *abort_flag = 1;
  } else {
    // ---- epilogue role: lane = M row (part of one complex row) ----
    const int quarter = warp & 3, wh = warp >> 2;  // lane quarter, column-block parity
    const int m = 32 * quarter + lane, i = m >> 1, part = m & 1;
    bool ok = true;
    for (int it = 0; it < n_it && ok; ++it) {
      const int buf = it & 1;
      ok = __all_sync(0xffffffffu, mbar_wait(smem_addr(&accf[buf]), (uint32_t)((it >> 1) & 1), abort_flag)) != 0;
      if (!ok) break;
      asm volatile("tcgen05.fence::after_thread_sync;");
      const int64_t r = (rb0 + it * rb_step) * 64 + i;
      const bool rok = r < n_rows_out;
      const int64_t pattern = rok ? r / Rr : 0;
      const int t = rok ? (int)(r - pattern * Rr) : 0;
      // the six component patterns of a child share one column space: column
      // n' = comp 2 half + n of child group pattern / 6
      const int64_t group = pattern / 6;
      const int col0 = (int)(pattern - group * 6) * 2 * half;
      uint8_t *pb = dst + group * (int64_t)8 * npad * Rr + (int64_t)(t >> 4) * 128 * npad + ((t >> 3) & 1) * 128 +
                    (t & 7) * 2;
      const int64_t mstride = (int64_t)32 * npad;  // matrix stride inside a 16-row chunk
      const uint32_t ta = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(buf * ntn);
      auto emit = [&](const uint32_t (&v)[16], int c0) {
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const int j = nt * (ntn / 2) + c0 / 2 + q;
          if (!rok || j >= half) continue;
          const float h = __uint_as_float(v[2 * q]), hp = __uint_as_float(v[2 * q + 1]);
          const float sv = h + hp, dv = h - hp;
          const __nv_bfloat16 sh = __float2bfloat16_rn(sv), dh = __float2bfloat16_rn(dv);
          const __nv_bfloat16 sl = __float2bfloat16_rn(sv - __bfloat162float(sh));
          const __nv_bfloat16 dl = __float2bfloat16_rn(dv - __bfloat162float(dh));
          const int n = col0 + 2 * j + part;
          uint8_t *e = pb + (n >> 3) * 256 + (n & 7) * 16;
          *(__nv_bfloat16 *)e = sh;
          *(__nv_bfloat16 *)(e + mstride) = sl;
          *(__nv_bfloat16 *)(e + 2 * mstride) = dh;
          *(__nv_bfloat16 *)(e + 3 * mstride) = dl;
        }
      };
      // this warp's 16-column blocks: wh, wh + NH, ...; two per wait with two
      // warps per lane quarter (one per wait measured faster with one warp)
      const int nblk = ntn / 16;
      for (int b = wh; b < nblk; b += 2 * NH) {
        uint32_t v[16], w[16];
        if (NH == 1) {
          tmem_ld16(ta + 16 * b, v);
          emit(v, 16 * b);
          if (b + 1 < nblk) {
            tmem_ld16(ta + 16 * (b + 1), w);
            emit(w, 16 * (b + 1));
          }
        } else if (b + NH < nblk) {
          tmem_ld16x2(ta + 16 * b, ta + 16 * (b + NH), v, w);
          emit(v, 16 * b);
          emit(w, 16 * (b + NH));
        } else {
          tmem_ld16(ta + 16 * b, v);
          emit(v, 16 * b);
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;");
      mbar_arrive(smem_addr(&acce[buf]));
    }
    if (!ok) {
      *abort_flag = 1;
      if (lane == 0) atomicCAS(err, 0, 1);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(tcols));
  }
}

template <int EW, int NB>
static po_status rows_tc_attributes() {
  PO_CUDA(cudaFuncSetAttribute(k_rows_tc<EW, NB>, cudaFuncAttributeMaxDynamicSharedMemorySize, kRtMaxSmem));
  PO_CUDA(cudaFuncSetAttribute(k_rows_tc<EW, NB>, cudaFuncAttributePreferredSharedMemoryCarveout,
                               (int)cudaSharedmemCarveoutMaxShared));
  return PO_OK;
}

po_status init_rows_tc_attributes() {
  // the whole shared-memory carveout, so that the occupancy query (and the
  // launch) can place two narrow-tile CTAs on an SM
  PO_TRY((rows_tc_attributes<4, 2>()));
  PO_TRY((rows_tc_attributes<4, 3>()));
  PO_TRY((rows_tc_attributes<8, 3>()));
  return PO_OK;
}

po_status launch_rows_tc(const float2 *src, uint8_t *dst, size_t dst_bytes, int64_t n_patterns, int Rc, int Rr,
                         int npad, int Pc, int Pp, const uint8_t *Bt, size_t bt_bytes, int ntn, int n_nt,
                         int sm_count, int *err, cudaStream_t st) {
  if (n_patterns <= 0) return PO_OK;
  const int KC = (Pc + 15) / 16;
  const int64_t n_rows_out = n_patterns * (int64_t)Rr;
  if ((Pc & 1) || (Pp & 1) || Rr % 16 || Rr < Rc || npad % 8 || npad < 6 * Pp || n_patterns % 6 || ntn % 16 ||
      ntn > 256 || n_nt < 1 || (int64_t)n_nt * (ntn / 2) < Pp / 2 || (size_t)n_nt * KC * 64 * ntn > bt_bytes ||
      (size_t)(n_patterns / 6) * 8 * npad * Rr > dst_bytes)
    return fail(PO_ERR_INTERNAL, "tcgen05 row pass: tiling or buffer sizes");
  const int smem = rows_tc_smem(KC, ntn);
  if (smem > kRtMaxSmem) return fail(PO_ERR_INTERNAL, "tcgen05 row pass: shared memory");
  uint32_t tcols = 32;
  while (tcols < (uint32_t)(2 * ntn)) tcols <<= 1;
  // resident CTAs per SM, persistent over row blocks: registers (allocated in
  // units of 8 per thread), shared memory (+1 KB reserved per CTA) and tensor
  // memory
  const bool wide = ntn > 128;
  // converter buffers: deep prefetch pays on long K loops (fiber root, 34
  // chunks: 57.8 -> 47.8 ms per wavelength with 3 buffers instead of 2) and
  // costs on short ones, where the pass is bound by DRAM writes (fiber level
  // 4, 3 chunks: 20.4 ms with 2 buffers, 28.0 with 3).  The wide tiles run two
  // converter groups of 3 buffers (17 warps: 96 registers per thread).
  const int nb = wide ? 3 : KC >= 8 ? 3 : 2;
  cudaFuncAttributes fa;
  if (wide)
    PO_CUDA(cudaFuncGetAttributes(&fa, k_rows_tc<8, 3>));
  else
    PO_CUDA(nb == 3 ? cudaFuncGetAttributes(&fa, k_rows_tc<4, 3>) : cudaFuncGetAttributes(&fa, k_rows_tc<4, 2>));
  const int threads = wide ? RtWarps<8>::threads : RtWarps<4>::threads;
  // registers: each of the 4 SM sub-partitions holds 16K and takes every
  // fourth warp of the resident CTAs (registers allocated 8 per thread)
  const int warps = threads / 32, regs = std::max(8, (fa.numRegs + 7) / 8 * 8);
  int reg_limit = 1;
  for (int c = 2; c <= 8; ++c)
    if ((c * warps + 3) / 4 * 32 * regs <= 16384) reg_limit = c;
  const int smem_limit = 228 * 1024 / (smem + 1024);
  const int per_sm = std::max(1, std::min(std::min(reg_limit, smem_limit), (int)(512 / tcols)));
  const int64_t n_rb = (n_rows_out + 63) / 64;
  const int64_t ctas_per_tile = std::min<int64_t>(n_rb, std::max(1, sm_count * per_sm / n_nt));
  const int64_t grid = ctas_per_tile * n_nt;
  if (grid > 2147483647LL) return fail(PO_ERR_UNSUPPORTED, "row pass grid");
#define PO_RT_LAUNCH(E, N)                                                                                    \
  k_rows_tc<E, N><<<(unsigned)grid, RtWarps<E>::threads, smem, st>>>(src, dst, n_rows_out, Rc, Rr, Pc, KC, Pp / 2, \
                                                                     npad, ntn, n_nt, Bt, tcols, err)
  if (wide) {
    PO_RT_LAUNCH(8, 3);
  } else {
    if (nb == 3) PO_RT_LAUNCH(4, 3); else PO_RT_LAUNCH(4, 2);
  }
#undef PO_RT_LAUNCH
  count_launch();
  PO_CUDA(cudaGetLastError());
  return PO_OK;
}

}  // namespace wavepo
