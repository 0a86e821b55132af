// po_fft.cu -- angular interpolation between tree levels with hand-written
// shared-memory FFTs, fused with the child->parent phase shift and child sum.
//
// Replaces util/interpolation.h:2-93 (cuFFT forward/inverse along phi and
// theta with a host loop of thrust::copy per row for the zero padding, a
// setvalue kernel for the Nyquist split and Scale_by_constant), plus
// util/fields.h:92-103 (translation_compute), :153-169 (sumchildren) and the
// host table factor1 of compareMie/sphere.cu:499-539.  The reference runs
// this chain once per (active child, component, node): 4 cuFFT executions
// and ~2(theta+phi) copy launches each.
//
// Here a level is two kernels over every node, component and wavelength:
//   rows  : every row of every child pattern: FFT_phi_c -> pad -> IFFT_phi_p
//           (one warp per row, Stockham autosort in shared memory);
//   cols  : for a parent and a tile of phi columns, for each active child:
//           tile load (coalesced along phi) -> FFT_theta_c -> pad -> IFFT_theta_p
//           -> times exp(i k s.(c_child - c_parent)) -> sum into the parent.
// The translation argument is taken from a per-(wavelength, level) table of
// the three axis phases k*a_ax*s_ax reduced mod 2pi in double; a child's
// phase is the signed sum of the three (exact up to a multiple of 2pi).
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "po_common.cuh"
#include "po_internal.h"
#include "po_kernels.h"

namespace wavepo {

// -------------------------------------------------------------- FFT plans
int fft_plan(int n, int *radix /*[kMaxStages]*/) {
  int s = 0;
  int m = n;
  const int pref[] = {4, 2, 3, 5, 7};
  for (int r : pref)
    while (m % r == 0 && m > 1) { radix[s++] = r; m /= r; }
  for (int q = 11; m > 1; q += 2)
    while (m % q == 0) { radix[s++] = q; m /= q; }
  return s;
}

FftPlan make_plan(int n, int tw_offset) {
  FftPlan p;
  p.n = n;
  p.tw = tw_offset;
  p.nstages = fft_plan(n, p.radix);
  return p;
}

__global__ void k_twiddles(int n, float2 *out) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  double s, c;
  sincospi(-2.0 * (double)k / (double)n, &s, &c);
  out[k] = make_float2((float)c, (float)s);
}

po_status launch_twiddles(int n, float2 *out, cudaStream_t st) {
  k_twiddles<<<(n + 255) / 256, 256, 0, st>>>(n, out);
  count_launch();
  PO_CUDA(cudaGetLastError());
  return PO_OK;
}

// ------------------------------------------------------- FFT device code
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
// twiddle W_n^k (forward) or its conjugate (inverse)
__device__ __forceinline__ float2 tw(const float2 *W, int k, bool inv) {
  float2 w = W[k];
  return inv ? make_float2(w.x, -w.y) : w;
}

// small DFT in registers, radix R in {3,5,7}: V[r] = sum_q v[q] e^{-+2pi i q r / R}
// (cos, sin) of 2 pi m / R for m = 0..R-1
__device__ __forceinline__ void root_of_unity(int R, int m, float *c, float *s) {
  switch (R * 8 + m) {
    case 3 * 8 + 1: *c = -0.5f; *s = 0.86602540378443865f; return;
    case 3 * 8 + 2: *c = -0.5f; *s = -0.86602540378443865f; return;
    case 5 * 8 + 1: *c = 0.30901699437494742f; *s = 0.95105651629515357f; return;
    case 5 * 8 + 2: *c = -0.80901699437494742f; *s = 0.58778525229247313f; return;
    case 5 * 8 + 3: *c = -0.80901699437494742f; *s = -0.58778525229247313f; return;
    case 5 * 8 + 4: *c = 0.30901699437494742f; *s = -0.95105651629515357f; return;
    case 7 * 8 + 1: *c = 0.62348980185873353f; *s = 0.78183148246802981f; return;
    case 7 * 8 + 2: *c = -0.22252093395631440f; *s = 0.97492791218182361f; return;
    case 7 * 8 + 3: *c = -0.90096886790241912f; *s = 0.43388373911755812f; return;
    case 7 * 8 + 4: *c = -0.90096886790241912f; *s = -0.43388373911755812f; return;
    case 7 * 8 + 5: *c = -0.22252093395631440f; *s = -0.97492791218182361f; return;
    case 7 * 8 + 6: *c = 0.62348980185873353f; *s = -0.78183148246802981f; return;
    default: *c = 1.f; *s = 0.f; return;
  }
}

template <int R>
__device__ __forceinline__ void small_dft(float2 *v, bool inv) {
  const float sg = inv ? 1.f : -1.f;  // forward transform uses e^{-i}
  float2 out[R];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    float2 acc = v[0];
#pragma unroll
    for (int q = 1; q < R; ++q) {
      float c, s;
      root_of_unity(R, (q * r) % R, &c, &s);
      s *= sg;
      acc.x += v[q].x * c - v[q].y * s;
      acc.y += v[q].x * s + v[q].y * c;
    }
    out[r] = acc;
  }
#pragma unroll
  for (int r = 0; r < R; ++r) v[r] = out[r];
}

template <int R>
__device__ __forceinline__ void stage_bfly(const float2 *a, float2 *b, int N, int Ns, const float2 *W, bool inv,
                                           int lane, int nl) {
  const int NR = N / R;
  const int twstep = N / (Ns * R);
  for (int j = lane; j < NR; j += nl) {
    const int jm = j % Ns;
    float2 v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = a[j + r * NR];
    if (Ns > 1) {
#pragma unroll
      for (int r = 1; r < R; ++r) v[r] = cmul(v[r], tw(W, r * jm * twstep, inv));
    }
    if (R == 2) {
      float2 t0 = cadd(v[0], v[1]), t1 = csub(v[0], v[1]);
      v[0] = t0; v[1] = t1;
    } else if (R == 4) {
      float2 s02 = cadd(v[0], v[2]), d02 = csub(v[0], v[2]);
      float2 s13 = cadd(v[1], v[3]), d13 = csub(v[1], v[3]);
      // forward: multiply d13 by -i ; inverse by +i
      float2 jd = inv ? make_float2(-d13.y, d13.x) : make_float2(d13.y, -d13.x);
      v[0] = cadd(s02, s13);
      v[2] = csub(s02, s13);
      v[1] = cadd(d02, jd);
      v[3] = csub(d02, jd);
    } else {
      small_dft<R>(v, inv);
    }
    const int idxD = (j / Ns) * Ns * R + jm;
#pragma unroll
    for (int r = 0; r < R; ++r) b[idxD + r * Ns] = v[r];
  }
}

// element-parallel stage for a large prime radix R
__device__ __forceinline__ void stage_generic(const float2 *a, float2 *b, int N, int Ns, int R, const float2 *W,
                                              bool inv, int lane, int nl) {
  const int NR = N / R;
  const int twstep = N / (Ns * R);
  for (int o = lane; o < N; o += nl) {
    const int jm = o % Ns;
    const int t = o / Ns;
    const int r = t % R;
    const int j = (t / R) * Ns + jm;
    int step = jm * twstep + r * NR;
    if (step >= N) step -= N;
    int idx = 0;
    float2 acc = make_float2(0.f, 0.f);
    for (int q = 0; q < R; ++q) {
      float2 w = tw(W, idx, inv);
      float2 x = a[j + q * NR];
      acc.x += x.x * w.x - x.y * w.y;
      acc.y += x.x * w.y + x.y * w.x;
      idx += step;
      if (idx >= N) idx -= N;
    }
    b[o] = acc;
  }
}

// Full transform of length p.n by `nl` lanes of one warp (sync = __syncwarp).
// Data starts in `a`; returns the buffer holding the result.
__device__ float2 *fft_warp(float2 *a, float2 *b, const FftPlan &p, const float2 *W, bool inv, int lane) {
  int Ns = 1;
  for (int s = 0; s < p.nstages; ++s) {
    const int R = p.radix[s];
    switch (R) {
      case 2: stage_bfly<2>(a, b, p.n, Ns, W, inv, lane, 32); break;
      case 3: stage_bfly<3>(a, b, p.n, Ns, W, inv, lane, 32); break;
      case 4: stage_bfly<4>(a, b, p.n, Ns, W, inv, lane, 32); break;
      case 5: stage_bfly<5>(a, b, p.n, Ns, W, inv, lane, 32); break;
      case 7: stage_bfly<7>(a, b, p.n, Ns, W, inv, lane, 32); break;
      default: stage_generic(a, b, p.n, Ns, R, W, inv, lane, 32); break;
    }
    __syncwarp();
    float2 *t = a;
    a = b;
    b = t;
    Ns *= R;
  }
  return a;
}

// Zero pad of a spectrum X (length n) into Y (length nf), interpolation.h:20-37.
// split: apply the Nyquist halving of setvalue (interpolation.h:2-9).
__device__ __forceinline__ void pad_spectrum(const float2 *X, int n, float2 *Y, int nf, bool split, int lane) {
  const int nyq = (n + 2) / 2;  // ceil((n+1)/2)
  const int sh = nf - n;
  for (int k = lane; k < nf; k += 32) {
    float2 v = make_float2(0.f, 0.f);
    if (k < nyq) v = X[k];
    else if (k >= nyq + sh) v = X[k - sh];
    Y[k] = v;
  }
  __syncwarp();
  if (split && (n % 2 == 0) && lane == 0) {
    float2 t = Y[nyq - 1];
    t.x *= 0.5f;
    t.y *= 0.5f;
    Y[nyq - 1] = t;
    Y[nyq - 1 + sh] = t;
  }
  __syncwarp();
}

// ------------------------------------------------------------- row pass
// rows: src [nrows][n_in] -> dst [nrows][n_out], both complex64.
__global__ void k_interp_rows(const float2 *__restrict__ src, float2 *__restrict__ dst, int64_t nrows, FftPlan pin,
                              FftPlan pout, const float2 *__restrict__ twiddles, float scale) {
  extern __shared__ float2 smem[];
  const int nw = blockDim.x >> 5, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nmax = max(pin.n, pout.n);
  float2 *Win = smem, *Wout = smem + pin.n;
  float2 *bufA = Wout + pout.n + (size_t)w * 2 * nmax, *bufB = bufA + nmax;
  for (int k = threadIdx.x; k < pin.n; k += blockDim.x) Win[k] = twiddles[pin.tw + k];
  for (int k = threadIdx.x; k < pout.n; k += blockDim.x) Wout[k] = twiddles[pout.tw + k];
  __syncthreads();
  for (int64_t row = (int64_t)blockIdx.x * nw + w; row < nrows; row += (int64_t)gridDim.x * nw) {
    const float2 *s = src + row * pin.n;
    for (int k = lane; k < pin.n; k += 32) bufA[k] = s[k];
    __syncwarp();
    float2 *X = fft_warp(bufA, bufB, pin, Win, false, lane);
    float2 *Y = (X == bufA) ? bufB : bufA;
    pad_spectrum(X, pin.n, Y, pout.n, true, lane);  // every row is reached (interpolation.h:34-37)
    float2 *Z = fft_warp(Y, X, pout, Wout, true, lane);
    float2 *d = dst + row * pout.n;
    for (int k = lane; k < pout.n; k += 32) {
      float2 v = Z[k];
      d[k] = make_float2(v.x * scale, v.y * scale);
    }
    __syncwarp();
  }
}

int rows_warps(int nmax, int nin, int nout) {
  size_t tw = sizeof(float2) * (size_t)(nin + nout);
  size_t per = sizeof(float2) * 2 * (size_t)nmax;
  int w = 8;
  while (w > 1 && tw + per * w > 200 * 1024) w >>= 1;
  return w;
}

po_status launch_interp_rows(const float2 *src, float2 *dst, int64_t nrows, const FftPlan &pin, const FftPlan &pout,
                             const float2 *twiddles, float scale, int sm_count, cudaStream_t st) {
  if (nrows <= 0) return PO_OK;
  const int nmax = std::max(pin.n, pout.n);
  const int w = rows_warps(nmax, pin.n, pout.n);
  size_t smem = sizeof(float2) * ((size_t)pin.n + pout.n + (size_t)w * 2 * nmax);
  if (smem > 227 * 1024) return fail(PO_ERR_UNSUPPORTED, "angular grid too large for the shared-memory FFT");
  PO_CUDA(cudaFuncSetAttribute(k_interp_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int64_t blocks = (nrows + w - 1) / w;
  int64_t cap = (int64_t)sm_count * 16;
  if (blocks > cap) blocks = cap;
  k_interp_rows<<<(unsigned)blocks, 32 * w, smem, st>>>(src, dst, nrows, pin, pout, twiddles, scale);
  count_launch();
  PO_CUDA(cudaGetLastError());
  return PO_OK;
}

// ---------------------------------------------------- column pass + sum
// mid   : [slot][child][comp][Tc][Phi] (output of the row pass)
// parent: [slot][node][comp][Tp][Phi]
// trans : [lambda][Tp*Phi] float4 (r_x, r_y, r_z, 0) reduced axis phases
// One warp owns one phi column; a CTA owns `nw` consecutive columns of one
// (parent node, component, slot).
__global__ void k_interp_cols(const float2 *__restrict__ mid, float2 *__restrict__ parent,
                              const int32_t *__restrict__ child_table, int64_t n_parent, int64_t n_child, int phi,
                              FftPlan pin, FftPlan pout, const float2 *__restrict__ twiddles,
                              const float4 *__restrict__ trans, int G, int quirk_reach, float scale, int ncomp) {
  extern __shared__ float2 smem[];
  const int nw = blockDim.x >> 5, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int Tc = pin.n, Tp = pout.n;
  const int nmax = max(Tc, Tp);
  float2 *Win = smem, *Wout = smem + Tc;
  float2 *tile = Wout + Tp;                       // [Tc][nw]
  float2 *acc = tile + (size_t)Tc * nw;           // [nw][Tp]
  float2 *bufA = acc + (size_t)nw * Tp + (size_t)w * 2 * nmax, *bufB = bufA + nmax;
  float2 *myacc = acc + (size_t)w * Tp;
  const int ntile = (phi + nw - 1) / nw;
  const int j0 = (int)(blockIdx.x % ntile) * nw;
  const int64_t pc = blockIdx.x / ntile;  // parent * ncomp + comp
  const int64_t p = pc / ncomp;
  const int comp = (int)(pc % ncomp);
  const int slot = blockIdx.z;
  const int lam = slot / G;
  const int j = j0 + w;
  const bool col_ok = j < phi;
  for (int k = threadIdx.x; k < Tc; k += blockDim.x) Win[k] = twiddles[pin.tw + k];
  for (int k = threadIdx.x; k < Tp; k += blockDim.x) Wout[k] = twiddles[pout.tw + k];
  for (int k = lane; k < Tp; k += 32) myacc[k] = make_float2(0.f, 0.f);
  const bool split = (j < quirk_reach);
  const float4 *tr = trans ? trans + (int64_t)lam * Tp * phi : nullptr;
  // child_table == nullptr: plain interpolation of pattern p (one "child", no phase shift)
  const int nchild_slots = child_table ? 8 : 1;
  for (int o = 0; o < nchild_slots; ++o) {
    const int32_t c = child_table ? child_table[p * 8 + o] : (int32_t)p;
    if (c < 0) continue;
    __syncthreads();
    // coalesced tile load: row t, columns j0..j0+nw
    const float2 *m = mid + (((int64_t)slot * n_child + c) * ncomp + comp) * (int64_t)Tc * phi;
    for (int e = threadIdx.x; e < Tc * nw; e += blockDim.x) {
      int t = e / nw, q = e % nw;
      int jj = j0 + q;
      tile[t * nw + q] = (jj < phi) ? m[(int64_t)t * phi + jj] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    for (int t = lane; t < Tc; t += 32) bufA[t] = tile[t * nw + w];
    __syncwarp();
    float2 *X = fft_warp(bufA, bufB, pin, Win, false, lane);
    float2 *Y = (X == bufA) ? bufB : bufA;
    pad_spectrum(X, Tc, Y, Tp, split, lane);
    float2 *Z = fft_warp(Y, X, pout, Wout, true, lane);
    // child centre - parent centre = (sx*a_x, sy*a_y, sz*a_z) with the octant signs of tree.h:672-687
    const float sgx = (o & 1) ? 1.f : -1.f, sgy = (o & 2) ? -1.f : 1.f, sgz = (o & 4) ? -1.f : 1.f;
    if (col_ok && trans == nullptr) {
      for (int t = lane; t < Tp; t += 32) {
        float2 v = Z[t];
        float2 a = myacc[t];
        a.x += scale * v.x;
        a.y += scale * v.y;
        myacc[t] = a;
      }
    } else if (col_ok) {
      for (int t = lane; t < Tp; t += 32) {
        float4 r = tr[(int64_t)t * phi + j];
        float ph = fmaf(sgx, r.x, fmaf(sgy, r.y, sgz * r.z));
        float sn, cs;
        sincos_small(ph, &sn, &cs);
        float2 v = Z[t];
        float2 a = myacc[t];
        a.x += scale * (v.x * cs - v.y * sn);
        a.y += scale * (v.x * sn + v.y * cs);
        myacc[t] = a;
      }
    }
    __syncwarp();
  }
  __syncthreads();
  float2 *out = parent + (((int64_t)slot * n_parent + p) * ncomp + comp) * (int64_t)Tp * phi;
  for (int e = threadIdx.x; e < Tp * nw; e += blockDim.x) {
    int t = e / nw, q = e % nw;
    int jj = j0 + q;
    if (jj < phi) out[(int64_t)t * phi + jj] = acc[(size_t)q * Tp + t];
  }
}

int cols_warps(int tc, int tp) {
  int nmax = std::max(tc, tp);
  int w = 8;
  while (w > 1) {
    size_t b = sizeof(float2) * ((size_t)tc + tp + (size_t)tc * w + (size_t)w * tp + (size_t)w * 2 * nmax);
    if (b <= 200 * 1024) break;
    w >>= 1;
  }
  return w;
}

po_status launch_interp_cols(const float2 *mid, float2 *parent, const int32_t *child_table, int64_t n_parent,
                             int64_t n_child, int phi, const FftPlan &pin, const FftPlan &pout,
                             const float2 *twiddles, const float4 *trans, int n_slots, int G, int quirk_reach,
                             float scale, int ncomp, cudaStream_t st) {
  if (n_parent <= 0 || n_slots <= 0) return PO_OK;
  const int w = cols_warps(pin.n, pout.n);
  const int nmax = std::max(pin.n, pout.n);
  size_t smem = sizeof(float2) * ((size_t)pin.n + pout.n + (size_t)pin.n * w + (size_t)w * pout.n +
                                  (size_t)w * 2 * nmax);
  if (smem > 227 * 1024) return fail(PO_ERR_UNSUPPORTED, "angular grid too large for the shared-memory FFT");
  PO_CUDA(cudaFuncSetAttribute(k_interp_cols, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int64_t gx = (int64_t)((phi + w - 1) / w) * n_parent * ncomp;
  if (gx > 2147483647LL || n_slots > 65535) return fail(PO_ERR_UNSUPPORTED, "too many nodes for one launch");
  dim3 grid((unsigned)gx, 1u, (unsigned)n_slots);
  k_interp_cols<<<grid, 32 * w, smem, st>>>(mid, parent, child_table, n_parent, n_child, phi, pin, pout, twiddles,
                                            trans, G, quirk_reach, scale, ncomp);
  count_launch();
  PO_CUDA(cudaGetLastError());
  return PO_OK;
}

// ----------------------------------------------------- translation table
// r_a = (k * a_a * s_a) mod 2pi for a = x, y, z and every direction of a
// Tp x Phi grid (theta rows may run into the second cover), per wavelength.
__global__ void k_trans_table(const double *__restrict__ k_per_lambda, int n_lambda, int nth, int Tp, int phi,
                              double ax, double ay, double az, float4 *__restrict__ out) {
  int64_t d = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  int lam = blockIdx.y;
  int64_t nd = (int64_t)Tp * phi;
  if (d >= nd || lam >= n_lambda) return;
  int it = (int)(d / phi), ip = (int)(d % phi);
  double s[3];
  grid_direction(it, ip, nth, phi, s);
  double k = k_per_lambda[lam];
  const double inv2pi = 0.15915494309189533577, p_hi = 6.28318530717958623200, p_lo = 2.44929359829470635445e-16;
  double a[3] = {k * ax * s[0], k * ay * s[1], k * az * s[2]};
  float r[3];
  for (int q = 0; q < 3; ++q) {
    double n = rint(a[q] * inv2pi);
    double v = fma(-n, p_hi, a[q]);
    r[q] = (float)fma(-n, p_lo, v);
  }
  out[(int64_t)lam * nd + d] = make_float4(r[0], r[1], r[2], 0.f);
}

po_status launch_trans_table(const double *k_per_lambda, int n_lambda, int nth, int Tp, int phi, const double a[3],
                             float4 *out, cudaStream_t st) {
  int64_t nd = (int64_t)Tp * phi;
  if (nd <= 0 || n_lambda <= 0) return PO_OK;
  dim3 grid((unsigned)((nd + 255) / 256), (unsigned)n_lambda);
  k_trans_table<<<grid, 256, 0, st>>>(k_per_lambda, n_lambda, nth, Tp, phi, a[0], a[1], a[2], out);
  count_launch();
  PO_CUDA(cudaGetLastError());
  return PO_OK;
}

}  // namespace wavepo
