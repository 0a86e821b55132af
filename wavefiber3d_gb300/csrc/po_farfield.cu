// po_farfield.cu -- surface currents and far-field sums of the PO engine.
//
// Replaces, for the leaf level and for depth 0:
//   util/tangentplane.h:84-92 + util/fields.h:123,:147  (currents, area, prefactors)
//   util/fields.h:2-50 + compareMie/sphere.cu:603-658   (phase * current, reduce per node)
// The reference launches one N-length transform per direction and one
// host-synchronous thrust::reduce per (leaf, direction).  Here one CTA owns a
// leaf (or a direction tile at depth 0), stages the points of the leaf in
// shared memory with their currents computed in the prologue, and every
// thread accumulates whole directions in registers.
//
// Phase arguments.  A leaf pattern is taken about the leaf centre, so its
// phase k s.(x - c) is small (k times the leaf half-diagonal) and float is
// exact enough; the offsets x - c are formed in double.  The depth-0 sum
// splits the phase into k s.(c_t - c) over a tile of 128 points (formed and
// reduced mod 2pi in double) plus the small in-tile part in float, so the
// large part of the argument never passes through float.
#include <cuda_runtime.h>

#include <algorithm>

#include "po_common.cuh"
#include "po_internal.h"
#include "po_kernels.h"

namespace wavepo {

// ---------------------------------------------------------------- currents
template <typename T>
__global__ void k_currents(int64_t n, const float *__restrict__ x, const float *__restrict__ y,
                           const float *__restrict__ z, const float *__restrict__ nx, const float *__restrict__ ny,
                           const float *__restrict__ nz, const float *__restrict__ area,
                           const SlotParams<T> *__restrict__ slots, int n_slots, T *__restrict__ out) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  int s = blockIdx.y;
  if (i >= n || s >= n_slots) return;
  SlotParams<T> P = slots[s];
  cx<T> c[6];
  tangent_plane<T>(P, x[i], y[i], z[i], nx[i], ny[i], nz[i], area ? area[i] : 1.0f, c);
  T *o = out + ((int64_t)s * n + i) * 12;
#pragma unroll
  for (int k = 0; k < 6; ++k) { o[2 * k] = c[k].re; o[2 * k + 1] = c[k].im; }
}

po_status launch_currents_f32(int64_t n, const float *const g[7], const SlotParams<float> *slots_dev, int n_slots,
                              float *out, cudaStream_t st) {
  if (n <= 0 || n_slots <= 0) return PO_OK;
  dim3 grid((unsigned)((n + 255) / 256), (unsigned)n_slots);
  k_currents<float><<<grid, 256, 0, st>>>(n, g[0], g[1], g[2], g[3], g[4], g[5], g[6], slots_dev, n_slots, out);
  count_launch();
  PO_CUDA(cudaGetLastError());
  return PO_OK;
}

po_status launch_currents_f64(int64_t n, const float *const g[7], const SlotParams<double> *slots_dev, int n_slots,
                              double *out, cudaStream_t st) {
  if (n <= 0 || n_slots <= 0) return PO_OK;
  dim3 grid((unsigned)((n + 255) / 256), (unsigned)n_slots);
  k_currents<double><<<grid, 256, 0, st>>>(n, g[0], g[1], g[2], g[3], g[4], g[5], g[6], slots_dev, n_slots, out);
  count_launch();
  PO_CUDA(cudaGetLastError());
  return PO_OK;
}

// ------------------------------------------------------------- leaf sums
// One CTA per (leaf, wavelength).  G slots (incidences x polarisations)
// share the phase of a wavelength.  Output: P[slot][leaf][comp][dir] complex.
// The block holds ceil(ndir / DPT) threads rounded up to a warp (at most
// kLeafMaxThreads; more directions take balanced passes), so no pass runs
// mostly empty direction slots.
constexpr int kLeafMaxThreads = 256;
constexpr int kLeafChunk = 256;

template <int G, int DPT>
__global__ void __launch_bounds__(kLeafMaxThreads) k_leaf(
    const float *__restrict__ x, const float *__restrict__ y, const float *__restrict__ z,
    const float *__restrict__ nx, const float *__restrict__ ny, const float *__restrict__ nz,
    const float *__restrict__ area, const int32_t *__restrict__ leaf_begin, const double *__restrict__ leaf_center,
    const SlotParams<float> *__restrict__ slots, const float4 *__restrict__ dirs, int ndir, int64_t n_leaves,
    int Gtot, int g0, float2 *__restrict__ out) {
  __shared__ float4 s_u[kLeafChunk];
  __shared__ float2 s_cur[kLeafChunk][G * 6];
  const int64_t leaf = blockIdx.x;
  const int lam = blockIdx.y;
  const int b = leaf_begin[leaf], e = leaf_begin[leaf + 1];
  const double cxd = leaf_center[3 * leaf], cyd = leaf_center[3 * leaf + 1], czd = leaf_center[3 * leaf + 2];
  const SlotParams<float> *sl = slots + lam * Gtot + g0;
  const double k0 = sl[0].k0d;
  const int64_t slot_stride = n_leaves * 6 * (int64_t)ndir;
  float2 *obase = out + ((int64_t)lam * Gtot + g0) * slot_stride + leaf * 6 * (int64_t)ndir;
  const int nthr = blockDim.x;
  const int per_pass = nthr * DPT;
  for (int c0 = b; c0 < e; c0 += kLeafChunk) {
    const int cnt = min(kLeafChunk, e - c0);
    __syncthreads();
    for (int q = threadIdx.x; q < cnt; q += nthr) {
      int p = c0 + q;
      float px = x[p], py = y[p], pz = z[p];
      s_u[q] = make_float4((float)(k0 * ((double)px - cxd)), (float)(k0 * ((double)py - cyd)),
                           (float)(k0 * ((double)pz - czd)), 0.f);
      float qx = nx[p], qy = ny[p], qz = nz[p], ar = area[p];
#pragma unroll
      for (int g = 0; g < G; ++g) {
        cx<float> c[6];
        tangent_plane<float>(sl[g], px, py, pz, qx, qy, qz, ar, c);
#pragma unroll
        for (int k = 0; k < 6; ++k) s_cur[q][g * 6 + k] = make_float2(c[k].re, c[k].im);
      }
    }
    __syncthreads();
    const bool first = (c0 == b);
    for (int base = 0; base < ndir; base += per_pass) {
      float sx[DPT], sy[DPT], sz[DPT];
      float ar_[DPT][G * 6], ai_[DPT][G * 6];
#pragma unroll
      for (int q = 0; q < DPT; ++q) {
        int d = base + q * nthr + threadIdx.x;
        float4 sv = d < ndir ? dirs[d] : make_float4(0.f, 0.f, 0.f, 0.f);
        sx[q] = sv.x; sy[q] = sv.y; sz[q] = sv.z;
#pragma unroll
        for (int k = 0; k < G * 6; ++k) { ar_[q][k] = 0.f; ai_[q][k] = 0.f; }
      }
      for (int j = 0; j < cnt; ++j) {
        float4 u = s_u[j];
#pragma unroll
        for (int q = 0; q < DPT; ++q) {
          float ph = fmaf(sx[q], u.x, fmaf(sy[q], u.y, sz[q] * u.z));
          float sn, cs;
          sincos_small(ph, &sn, &cs);
#pragma unroll
          for (int k = 0; k < G * 6; ++k) {
            float2 c = s_cur[j][k];
            ar_[q][k] = fmaf(c.x, cs, fmaf(-c.y, sn, ar_[q][k]));
            ai_[q][k] = fmaf(c.x, sn, fmaf(c.y, cs, ai_[q][k]));
          }
        }
      }
#pragma unroll
      for (int q = 0; q < DPT; ++q) {
        int d = base + q * nthr + threadIdx.x;
        if (d >= ndir) continue;
#pragma unroll
        for (int g = 0; g < G; ++g) {
#pragma unroll
          for (int k = 0; k < 6; ++k) {
            float2 *o = obase + g * slot_stride + (int64_t)k * ndir + d;
            float2 v = make_float2(ar_[q][g * 6 + k], ai_[q][g * 6 + k]);
            if (!first) { float2 w = *o; v.x += w.x; v.y += w.y; }
            *o = v;
          }
        }
      }
    }
  }
  if (b == e) {  // an empty node (only the root of an empty cloud) has a zero pattern
    for (int d = threadIdx.x; d < ndir; d += nthr)
      for (int g = 0; g < G; ++g)
        for (int k = 0; k < 6; ++k) obase[g * slot_stride + (int64_t)k * ndir + d] = make_float2(0.f, 0.f);
  }
}

po_status launch_leaf(const float *const g[7], const int32_t *leaf_begin, const double *leaf_center,
                      int64_t n_leaves, const SlotParams<float> *slots_dev, int n_lambda, int G,
                      const float4 *dirs, int ndir, float2 *out, cudaStream_t st) {
  if (n_leaves <= 0 || n_lambda <= 0) return PO_OK;
  if (n_lambda > 65535) return fail(PO_ERR_UNSUPPORTED, "too many wavelengths for one launch");
  dim3 grid((unsigned)n_leaves, (unsigned)n_lambda);
  // the slots of a wavelength share its phases; they go through the kernel in
  // chunks of at most 4 (register budget of the accumulators)
  for (int g0 = 0; g0 < G; g0 += 4) {
    const int gc = std::min(4, G - g0);
    const int dpt = gc == 1 ? 4 : gc == 2 ? 2 : 1;
    const int passes = (ndir + kLeafMaxThreads * dpt - 1) / (kLeafMaxThreads * dpt);
    const int per_pass = (ndir + passes - 1) / passes;
    const int threads = std::max(64, (per_pass + dpt - 1) / dpt + 31) / 32 * 32;
#define PO_LEAF(GG, DD)                                                                                   \
  k_leaf<GG, DD><<<grid, threads, 0, st>>>(g[0], g[1], g[2], g[3], g[4], g[5], g[6], leaf_begin,         \
                                          leaf_center, slots_dev, dirs, ndir, n_leaves, G, g0, out)
    switch (gc) {
      case 1: PO_LEAF(1, 4); break;
      case 2: PO_LEAF(2, 2); break;
      case 3: PO_LEAF(3, 1); break;
      default: PO_LEAF(4, 1); break;
    }
#undef PO_LEAF
    count_launch();
  }
  PO_CUDA(cudaGetLastError());
  return PO_OK;
}

// ---------------------------------------------------- depth-0 direct sums
constexpr int kDirThreads = 128;
constexpr int kDirDPT = 2;
constexpr int kDirTile = 128;

// tile centres (double) of consecutive groups of kDirTile points: bbox midpoint
__global__ void k_tile_centers(int64_t n, const float *__restrict__ x, const float *__restrict__ y,
                               const float *__restrict__ z, double *__restrict__ ctr) {
  int64_t t = blockIdx.x;
  int64_t b = t * kDirTile, e = min(n, b + kDirTile);
  __shared__ float mn[3][32], mx[3][32];
  float lo[3] = {3.4e38f, 3.4e38f, 3.4e38f}, hi[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
  for (int64_t i = b + threadIdx.x; i < e; i += blockDim.x) {
    float v[3] = {x[i], y[i], z[i]};
    for (int a = 0; a < 3; ++a) { lo[a] = fminf(lo[a], v[a]); hi[a] = fmaxf(hi[a], v[a]); }
  }
  for (int a = 0; a < 3; ++a) {
    for (int o = 16; o > 0; o >>= 1) {
      lo[a] = fminf(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], o));
      hi[a] = fmaxf(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], o));
    }
  }
  int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if ((threadIdx.x & 31) == 0)
    for (int a = 0; a < 3; ++a) { mn[a][w] = lo[a]; mx[a][w] = hi[a]; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int a = 0; a < 3; ++a) {
      float l = mn[a][0], h = mx[a][0];
      for (int q = 1; q < nw; ++q) { l = fminf(l, mn[a][q]); h = fmaxf(h, mx[a][q]); }
      ctr[3 * t + a] = 0.5 * ((double)l + (double)h);
    }
  }
}

// grid: (direction tiles, point splits, wavelengths).  partial[split][slot][comp][dir]
template <int G>
__global__ void __launch_bounds__(kDirThreads) k_direct_f32(
    int64_t n, const float *__restrict__ x, const float *__restrict__ y, const float *__restrict__ z,
    const float2 *__restrict__ cur /* [slot][n][6] */, const double *__restrict__ tile_ctr,
    const double *__restrict__ k_per_lambda, double c0x, double c0y, double c0z, const float4 *__restrict__ dirs,
    const double *__restrict__ dirs_d, int ndir, int tiles_per_split, int n_slots_total, int Gtot, int g0,
    float2 *__restrict__ partial) {
  __shared__ float4 s_u[kDirTile];
  __shared__ float2 s_cur[kDirTile][G * 6];
  const int lam = blockIdx.z, split = blockIdx.y;
  const double k0 = k_per_lambda[lam];
  const int64_t ntiles = (n + kDirTile - 1) / kDirTile;
  const int64_t t0 = (int64_t)split * tiles_per_split, t1 = min(ntiles, t0 + tiles_per_split);
  int dd[kDirDPT];
  float sx[kDirDPT], sy[kDirDPT], sz[kDirDPT];
  double sdx[kDirDPT], sdy[kDirDPT], sdz[kDirDPT];
  float tr[kDirDPT][G * 6], ti[kDirDPT][G * 6];
#pragma unroll
  for (int q = 0; q < kDirDPT; ++q) {
    dd[q] = (blockIdx.x * kDirDPT + q) * kDirThreads + threadIdx.x;
    int d = min(dd[q], ndir - 1);
    float4 sv = dirs[d];
    sx[q] = sv.x; sy[q] = sv.y; sz[q] = sv.z;
    sdx[q] = dirs_d[3 * d]; sdy[q] = dirs_d[3 * d + 1]; sdz[q] = dirs_d[3 * d + 2];
#pragma unroll
    for (int k = 0; k < G * 6; ++k) { tr[q][k] = 0.f; ti[q][k] = 0.f; }
  }
  for (int64_t t = t0; t < t1; ++t) {
    const int64_t pb = t * kDirTile;
    const int cnt = (int)min((int64_t)kDirTile, n - pb);
    const double tcx = tile_ctr[3 * t], tcy = tile_ctr[3 * t + 1], tcz = tile_ctr[3 * t + 2];
    __syncthreads();
    for (int q = threadIdx.x; q < cnt; q += kDirThreads) {
      int64_t p = pb + q;
      s_u[q] = make_float4((float)(k0 * ((double)x[p] - tcx)), (float)(k0 * ((double)y[p] - tcy)),
                           (float)(k0 * ((double)z[p] - tcz)), 0.f);
#pragma unroll
      for (int g = 0; g < G; ++g)
#pragma unroll
        for (int k = 0; k < 6; ++k) s_cur[q][g * 6 + k] = cur[(((int64_t)lam * Gtot + g0 + g) * n + p) * 6 + k];
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < kDirDPT; ++q) {
      float lr[G * 6], li[G * 6];
#pragma unroll
      for (int k = 0; k < G * 6; ++k) { lr[k] = 0.f; li[k] = 0.f; }
      for (int j = 0; j < cnt; ++j) {
        float4 u = s_u[j];
        float ph = fmaf(sx[q], u.x, fmaf(sy[q], u.y, sz[q] * u.z));
        float sn, cs;
        sincos_small(ph, &sn, &cs);
#pragma unroll
        for (int k = 0; k < G * 6; ++k) {
          float2 c = s_cur[j][k];
          lr[k] = fmaf(c.x, cs, fmaf(-c.y, sn, lr[k]));
          li[k] = fmaf(c.x, sn, fmaf(c.y, cs, li[k]));
        }
      }
      // rotate by the tile-centre phase k s.(c_t - c), argument in double
      float2 rot = expi_reduced(k0 * (sdx[q] * (tcx - c0x) + sdy[q] * (tcy - c0y) + sdz[q] * (tcz - c0z)));
#pragma unroll
      for (int k = 0; k < G * 6; ++k) {
        tr[q][k] += lr[k] * rot.x - li[k] * rot.y;
        ti[q][k] += lr[k] * rot.y + li[k] * rot.x;
      }
    }
  }
#pragma unroll
  for (int q = 0; q < kDirDPT; ++q) {
    if (dd[q] >= ndir) continue;
#pragma unroll
    for (int g = 0; g < G; ++g)
#pragma unroll
      for (int k = 0; k < 6; ++k)
        partial[(((int64_t)split * n_slots_total + (int64_t)lam * Gtot + g0 + g) * 6 + k) * ndir + dd[q]] =
            make_float2(tr[q][g * 6 + k], ti[q][g * 6 + k]);
  }
}

// plain FP64 direct sum (the "plain method" denominator): one thread per
// direction per point split.  partial64[split][slot][comp][dir] (double2)
constexpr int kDir64Tile = 64;
__global__ void __launch_bounds__(128) k_direct_f64(
    int64_t n, const float *__restrict__ x, const float *__restrict__ y, const float *__restrict__ z,
    const double2 *__restrict__ cur /* [slot][n][6] */, const double *__restrict__ k_per_lambda, double c0x,
    double c0y, double c0z, const double *__restrict__ dirs_d, int ndir, int64_t pts_per_split, int n_slots_total,
    double2 *__restrict__ partial) {
  __shared__ double s_x[kDir64Tile][3];
  __shared__ double2 s_c[kDir64Tile][6];
  const int lam = blockIdx.z, split = blockIdx.y;
  const int d = blockIdx.x * blockDim.x + threadIdx.x;
  const double k0 = k_per_lambda[lam];
  const int dc = min(d, ndir - 1);
  const double sx = dirs_d[3 * dc], sy = dirs_d[3 * dc + 1], sz = dirs_d[3 * dc + 2];
  double ar[6] = {0, 0, 0, 0, 0, 0}, ai[6] = {0, 0, 0, 0, 0, 0};
  const int64_t p0 = (int64_t)split * pts_per_split, p1 = min(n, p0 + pts_per_split);
  for (int64_t pb = p0; pb < p1; pb += kDir64Tile) {
    const int cnt = (int)min((int64_t)kDir64Tile, p1 - pb);
    __syncthreads();
    for (int q = threadIdx.x; q < cnt; q += blockDim.x) {
      int64_t p = pb + q;
      s_x[q][0] = (double)x[p] - c0x;
      s_x[q][1] = (double)y[p] - c0y;
      s_x[q][2] = (double)z[p] - c0z;
      for (int k = 0; k < 6; ++k) s_c[q][k] = cur[((int64_t)lam * n + p) * 6 + k];
    }
    __syncthreads();
    for (int j = 0; j < cnt; ++j) {
      double ph = k0 * (sx * s_x[j][0] + sy * s_x[j][1] + sz * s_x[j][2]);
      double sn, cs;
      sincos(ph, &sn, &cs);
#pragma unroll
      for (int k = 0; k < 6; ++k) {
        double2 c = s_c[j][k];
        ar[k] += c.x * cs - c.y * sn;
        ai[k] += c.x * sn + c.y * cs;
      }
    }
  }
  if (d < ndir)
    for (int k = 0; k < 6; ++k)
      partial[(((int64_t)split * n_slots_total + lam) * 6 + k) * ndir + d] = make_double2(ar[k], ai[k]);
}

__global__ void k_widen(const float *__restrict__ in, double2 *__restrict__ out, int64_t n) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] = make_double2((double)in[2 * i], (double)in[2 * i + 1]);
}

__global__ void k_narrow(const double2 *__restrict__ in, float2 *__restrict__ out, int64_t n) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] = make_float2((float)in[i].x, (float)in[i].y);
}

po_status launch_widen(const float *in, double2 *out, int64_t n, cudaStream_t st) {
  if (n <= 0) return PO_OK;
  k_widen<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(in, out, n);
  count_launch();
  PO_CUDA(cudaGetLastError());
  return PO_OK;
}

po_status launch_narrow(const double2 *in, float2 *out, int64_t n, cudaStream_t st) {
  if (n <= 0) return PO_OK;
  k_narrow<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(in, out, n);
  count_launch();
  PO_CUDA(cudaGetLastError());
  return PO_OK;
}

template <typename V>
__global__ void k_sum_splits(const V *__restrict__ partial, int nsplit, int64_t per_split, V *__restrict__ out) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= per_split) return;
  V acc = partial[i];
  for (int s = 1; s < nsplit; ++s) {
    V v = partial[(int64_t)s * per_split + i];
    acc.x += v.x;
    acc.y += v.y;
  }
  out[i] = acc;
}

int direct_splits(int64_t n, int ndir, int n_lambda, int sm_count) {
  int64_t ntiles = (n + kDirTile - 1) / kDirTile;
  int64_t dtiles = (ndir + kDirThreads * kDirDPT - 1) / (kDirThreads * kDirDPT);
  int64_t want = (int64_t)sm_count * 8;
  int64_t have = dtiles * n_lambda;
  int64_t s = (want + have - 1) / have;
  if (s < 1) s = 1;
  if (s > ntiles) s = ntiles;
  if (s > 64) s = 64;
  return (int)s;
}

po_status launch_direct_f32(int64_t n, const float *x, const float *y, const float *z, const float2 *cur,
                            double *tile_ctr, const double *k_per_lambda, int n_lambda, int G,
                            const double c0[3], const float4 *dirs, const double *dirs_d, int ndir, int nsplit,
                            float2 *partial, float2 *out, cudaStream_t st) {
  if (n_lambda <= 0 || ndir <= 0) return PO_OK;
  const int S = n_lambda * G;
  if (n <= 0) {
    PO_CUDA(cudaMemsetAsync(out, 0, sizeof(float2) * (size_t)S * 6 * ndir, st));
    return PO_OK;
  }
  int64_t ntiles = (n + kDirTile - 1) / kDirTile;
  k_tile_centers<<<(unsigned)ntiles, 128, 0, st>>>(n, x, y, z, tile_ctr);
  count_launch();
  int tps = (int)((ntiles + nsplit - 1) / nsplit);
  dim3 grid((unsigned)((ndir + kDirThreads * kDirDPT - 1) / (kDirThreads * kDirDPT)), (unsigned)nsplit,
            (unsigned)n_lambda);
  for (int g0 = 0; g0 < G; g0 += 4) {
    const int gc = std::min(4, G - g0);
#define PO_DIR(GG)                                                                                             \
  k_direct_f32<GG><<<grid, kDirThreads, 0, st>>>(n, x, y, z, cur, tile_ctr, k_per_lambda, c0[0], c0[1], c0[2], \
                                                 dirs, dirs_d, ndir, tps, S, G, g0, partial)
    switch (gc) {
      case 1: PO_DIR(1); break;
      case 2: PO_DIR(2); break;
      case 3: PO_DIR(3); break;
      default: PO_DIR(4); break;
    }
#undef PO_DIR
    count_launch();
  }
  int64_t per = (int64_t)S * 6 * ndir;
  k_sum_splits<float2><<<(unsigned)((per + 255) / 256), 256, 0, st>>>(partial, nsplit, per, out);
  count_launch();
  PO_CUDA(cudaGetLastError());
  return PO_OK;
}

po_status launch_direct_f64(int64_t n, const float *x, const float *y, const float *z, const double2 *cur,
                            const double *k_per_lambda, int n_slots, const double c0[3], const double *dirs_d,
                            int ndir, int nsplit, double2 *partial, double2 *out, cudaStream_t st) {
  if (n_slots <= 0 || ndir <= 0) return PO_OK;
  if (n <= 0) {
    PO_CUDA(cudaMemsetAsync(out, 0, sizeof(double2) * (size_t)n_slots * 6 * ndir, st));
    return PO_OK;
  }
  int64_t pps = (n + nsplit - 1) / nsplit;
  dim3 grid((unsigned)((ndir + 127) / 128), (unsigned)nsplit, (unsigned)n_slots);
  k_direct_f64<<<grid, 128, 0, st>>>(n, x, y, z, cur, k_per_lambda, c0[0], c0[1], c0[2], dirs_d, ndir, pps,
                                     n_slots, partial);
  count_launch();
  int64_t per = (int64_t)n_slots * 6 * ndir;
  k_sum_splits<double2><<<(unsigned)((per + 255) / 256), 256, 0, st>>>(partial, nsplit, per, out);
  count_launch();
  PO_CUDA(cudaGetLastError());
  return PO_OK;
}

}  // namespace wavepo
