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

// One Stockham stage of radix R over butterflies j = glane, glane+L, ...
// tab[j] packs the output base idxD = (j/Ns)*Ns*R + j%Ns (low 16 bits) and
// the twiddle base (j%Ns)*N/(Ns*R) (high 16 bits), precomputed per CTA so
// that no integer division runs per butterfly.
template <int R>
__device__ __forceinline__ void stage_bfly(const float2 *a, float2 *b, int N, int Ns, const float2 *W, bool inv,
                                           int glane, int L, const uint32_t *tab) {
  const int NR = N / R;
  for (int j = glane; j < NR; j += L) {
    const uint32_t e = tab[j];
    const int idxD = (int)(e & 0xffffu), twb = (int)(e >> 16);
    float2 v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = a[j + r * NR];
    if (Ns > 1) {
#pragma unroll
      for (int r = 1; r < R; ++r) v[r] = cmul(v[r], tw(W, r * twb, inv));
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
#pragma unroll
    for (int r = 0; r < R; ++r) b[idxD + r * Ns] = v[r];
  }
}

// Number of table entries of a plan (sum over stages of N/R).
__host__ __device__ __forceinline__ int stage_table_size(const FftPlan &p) {
  int t = 0;
  for (int s = 0; s < p.nstages; ++s) t += p.n / p.radix[s];
  return t;
}

// Fills the per-stage butterfly tables of plan p (all threads of the CTA).
__device__ void build_stage_table(const FftPlan &p, uint32_t *tab) {
  int Ns = 1, off = 0;
  for (int s = 0; s < p.nstages; ++s) {
    const int R = p.radix[s], NR = p.n / R, twstep = p.n / (Ns * R);
    for (int j = threadIdx.x; j < NR; j += blockDim.x) {
      const int jm = j % Ns;
      const int idxD = (j / Ns) * Ns * R + jm;
      tab[off + j] = (uint32_t)idxD | ((uint32_t)(jm * twstep) << 16);
    }
    off += NR;
    Ns *= R;
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

// Transform of length p.n by the L lanes of one lane group (glane in [0, L)).
// All groups of a warp run the same plan in lockstep, so a warp-wide
// __syncwarp separates the stages.  Data starts in `a`; returns the buffer
// holding the result.  tab: the plan's stage tables (build_stage_table).
__device__ float2 *fft_group(float2 *a, float2 *b, const FftPlan &p, const float2 *W, bool inv, int glane, int L,
                             const uint32_t *tab) {
  int Ns = 1;
  for (int s = 0; s < p.nstages; ++s) {
    const int R = p.radix[s];
    switch (R) {
      case 2: stage_bfly<2>(a, b, p.n, Ns, W, inv, glane, L, tab); break;
      case 3: stage_bfly<3>(a, b, p.n, Ns, W, inv, glane, L, tab); break;
      case 4: stage_bfly<4>(a, b, p.n, Ns, W, inv, glane, L, tab); break;
      case 5: stage_bfly<5>(a, b, p.n, Ns, W, inv, glane, L, tab); break;
      case 7: stage_bfly<7>(a, b, p.n, Ns, W, inv, glane, L, tab); break;
      default: stage_generic(a, b, p.n, Ns, R, W, inv, glane, L); break;
    }
    tab += p.n / R;
    __syncwarp();
    float2 *t = a;
    a = b;
    b = t;
    Ns *= R;
  }
  return a;
}

// Zero pad of a spectrum X (length n) into Y (length nf), interpolation.h:20-37.
// split: apply the Nyquist halving of setvalue (interpolation.h:2-9).  When
// nf == n both halves land on one bin; the reference then keeps half of it
// (split = true), the exact trigonometric interpolant keeps all of it, which
// callers request by passing split = false for that case.
__device__ __forceinline__ void pad_spectrum(const float2 *X, int n, float2 *Y, int nf, bool split, int glane,
                                             int L) {
  const int nyq = (n + 2) / 2;  // ceil((n+1)/2)
  const int sh = nf - n;
  for (int k = glane; k < nf; k += L) {
    float2 v = make_float2(0.f, 0.f);
    if (k < nyq) v = X[k];
    else if (k >= nyq + sh) v = X[k - sh];
    Y[k] = v;
  }
  __syncwarp();
  if (split && (n % 2 == 0) && glane == 0) {
    float2 t = Y[nyq - 1];
    t.x *= 0.5f;
    t.y *= 0.5f;
    Y[nyq - 1] = t;
    Y[nyq - 1 + sh] = t;
  }
  __syncwarp();
}

// lanes per transform: enough butterflies per lane to amortise a stage
int group_lanes(int nmax) {
  int want = (nmax + 15) / 16, L = 2;
  while (L < want && L < 32) L <<= 1;
  return L;
}

// ------------------------------------------------------------- row pass
// rows: src [nrows][n_in] -> dst [nrows][n_out], both complex64.  A CTA
// processes NG = blockDim/L consecutive rows per iteration (one lane group per
// row); consecutive rows are contiguous, so loads and stores are coalesced
// through shared memory.
__global__ void k_interp_rows(const float2 *__restrict__ src, float2 *__restrict__ dst, int64_t nrows, FftPlan pin,
                              FftPlan pout, const float2 *__restrict__ twiddles, float scale, int L, int ref_nyquist) {
  extern __shared__ float2 smem[];
  const int NG = blockDim.x / L, gid = threadIdx.x / L, glane = threadIdx.x % L;
  const int nin = pin.n, nout = pout.n, nmax = max(nin, nout);
  const int stride = 2 * nmax + 1;  // odd: lane groups start in different banks
  float2 *Win = smem, *Wout = smem + nin;
  float2 *bufs = Wout + nout;
  uint32_t *tin = (uint32_t *)(bufs + (size_t)NG * stride);
  uint32_t *tout = tin + stage_table_size(pin);
  float2 *bufA = bufs + (size_t)gid * stride, *bufB = bufA + nmax;
  for (int k = threadIdx.x; k < nin; k += blockDim.x) Win[k] = twiddles[pin.tw + k];
  for (int k = threadIdx.x; k < nout; k += blockDim.x) Wout[k] = twiddles[pout.tw + k];
  build_stage_table(pin, tin);
  build_stage_table(pout, tout);
  for (int64_t base = (int64_t)blockIdx.x * NG; base < nrows; base += (int64_t)gridDim.x * NG) {
    const int nr = (int)min((int64_t)NG, nrows - base);
    __syncthreads();
    const float2 *s = src + base * nin;
    for (int e = threadIdx.x; e < NG * nin; e += blockDim.x) {
      int g = e / nin, k = e - g * nin;
      bufs[(size_t)g * stride + k] = g < nr ? s[e] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    float2 *X = fft_group(bufA, bufB, pin, Win, false, glane, L, tin);
    float2 *Y = (X == bufA) ? bufB : bufA;
    // every row is reached by the reference's split (interpolation.h:34-37)
    pad_spectrum(X, nin, Y, nout, ref_nyquist || nin != nout, glane, L);
    float2 *Z = fft_group(Y, X, pout, Wout, true, glane, L, tout);
    // the result sits in bufA or bufB of every group (same parity for all)
    const int zoff = (Z == bufA) ? 0 : nmax;
    __syncthreads();
    float2 *d = dst + base * nout;
    for (int e = threadIdx.x; e < nr * nout; e += blockDim.x) {
      int g = e / nout, k = e - g * nout;
      float2 v = bufs[(size_t)g * stride + zoff + k];
      d[e] = make_float2(v.x * scale, v.y * scale);
    }
  }
}

static size_t rows_smem(const FftPlan &pin, const FftPlan &pout, int NG) {
  const int nmax = std::max(pin.n, pout.n);
  return sizeof(float2) * ((size_t)pin.n + pout.n + (size_t)NG * (2 * nmax + 1)) +
         sizeof(uint32_t) * (stage_table_size(pin) + stage_table_size(pout)) + 16;
}

po_status launch_interp_rows(const float2 *src, float2 *dst, int64_t nrows, const FftPlan &pin, const FftPlan &pout,
                             const float2 *twiddles, float scale, int sm_count, int ref_nyquist, cudaStream_t st) {
  if (nrows <= 0) return PO_OK;
  const int nmax = std::max(pin.n, pout.n);
  const int L = group_lanes(nmax);
  int threads = 256;
  while (rows_smem(pin, pout, threads / L) > 72 * 1024 && threads > std::max(32, L)) threads >>= 1;
  const size_t smem = rows_smem(pin, pout, threads / L);
  if (smem > 227 * 1024) return fail(PO_ERR_UNSUPPORTED, "angular grid too large for the shared-memory FFT");
  const int NG = threads / L;
  int64_t blocks = (nrows + NG - 1) / NG;
  int64_t cap = (int64_t)sm_count * 32;
  if (blocks > cap) blocks = cap;
  k_interp_rows<<<(unsigned)blocks, threads, smem, st>>>(src, dst, nrows, pin, pout, twiddles, scale, L, ref_nyquist);
  count_launch();
  PO_CUDA(cudaGetLastError());
  return PO_OK;
}

// ---------------------------------------------------- column pass + sum
// mid   : [slot][child][comp][Rc][Phi]   (row-pass output, Rc stored theta rows)
// parent: [slot][node][comp][Rp][Phi]
// trans : [lambda][Rp*Phi] float4 (r_x, r_y, r_z, 0) reduced axis phases
// Without `mirror`, Rc = Tc and Rp = Tp: whole theta columns are stored.
// With `mirror` (double cover, Phi even), a level stores rows 0..n_theta only
// (Rc = Tc/2 + 1); row t > n_theta of column j is row Tc - t of column
// j + Phi/2 (the same direction), so a CTA takes columns in pairs
// (j, j + Phi/2) and rebuilds both full columns from the two stored halves.
// A CTA owns NG = 2^lgNG columns of one (parent node, component, slot); one
// lane group of L lanes transforms one column.
__global__ void k_interp_cols(const float2 *__restrict__ mid, float2 *__restrict__ parent,
                              const int32_t *__restrict__ child_table, int64_t n_parent, int64_t n_child, int phi,
                              int Rc, int Rp, FftPlan pin, FftPlan pout, const float2 *__restrict__ twiddles,
                              const float4 *__restrict__ trans, int G, int quirk_reach, float scale, int ncomp,
                              int mirror, int L, int lgNG, int ref_nyquist) {
  extern __shared__ float2 smem[];
  const int NG = 1 << lgNG, gid = threadIdx.x / L, glane = threadIdx.x % L;
  const int Tc = pin.n, Tp = pout.n;
  const int nmax = max(Tc, Tp), stride = 2 * nmax + 1, ts = NG + 1;
  float2 *Win = smem, *Wout = smem + Tc;
  float2 *tile = Wout + Tp;                 // [Rc][NG + 1]
  float2 *acc = tile + (size_t)Rc * ts;     // [NG][Rp + 1]
  float2 *bufs = acc + (size_t)NG * (Rp + 1);
  uint32_t *tin = (uint32_t *)(bufs + (size_t)NG * stride);
  uint32_t *tout = tin + stage_table_size(pin);
  float2 *bufA = bufs + (size_t)gid * stride, *bufB = bufA + nmax;
  float2 *myacc = acc + (size_t)gid * (Rp + 1);
  // columns of this CTA
  const int TW = mirror ? NG / 2 : NG;          // distinct column starts per tile
  const int span = mirror ? phi / 2 : phi;      // columns covered by tile starts
  const int ntile = (span + TW - 1) / TW;
  const int j0 = (int)(blockIdx.x % ntile) * TW;
  const int64_t pc = blockIdx.x / ntile;  // parent * ncomp + comp
  const int64_t p = pc / ncomp;
  const int comp = (int)(pc % ncomp);
  const int slot = blockIdx.z;
  const int lam = slot / G;
  // the column this thread's group owns and the column this thread loads/stores
  // in the cooperative tile loops (blockDim is a multiple of NG, so it is fixed)
  const int gl = threadIdx.x & (NG - 1);
  auto col_of = [&](int g) { return mirror ? (g < TW ? j0 + g : j0 + (g - TW) + phi / 2) : j0 + g; };
  auto base_of = [&](int g) { return mirror ? j0 + (g < TW ? g : g - TW) : j0 + g; };
  const int j = col_of(gid);
  const bool ok = base_of(gid) < span;
  const int jl = col_of(gl);
  const bool okl = base_of(gl) < span;
  const int partner = mirror ? (gid < TW ? gid + TW : gid - TW) : gid;
  const int nth_c = Tc / 2;
  const int rstep = blockDim.x >> lgNG;
  for (int k = threadIdx.x; k < Tc; k += blockDim.x) Win[k] = twiddles[pin.tw + k];
  for (int k = threadIdx.x; k < Tp; k += blockDim.x) Wout[k] = twiddles[pout.tw + k];
  build_stage_table(pin, tin);
  build_stage_table(pout, tout);
  for (int k = glane; k < Rp; k += L) myacc[k] = make_float2(0.f, 0.f);
  const bool split = (j < quirk_reach) && (ref_nyquist || Tc != Tp);
  const float4 *tr = trans ? trans + (int64_t)lam * Rp * phi : nullptr;
  // child_table == nullptr: plain interpolation of pattern p (one "child", no phase shift)
  const int nchild_slots = child_table ? 8 : 1;
  for (int o = 0; o < nchild_slots; ++o) {
    const int32_t c = child_table ? child_table[p * 8 + o] : (int32_t)p;
    if (c < 0) continue;
    __syncthreads();
    const float2 *m = mid + (((int64_t)slot * n_child + c) * ncomp + comp) * (int64_t)Rc * phi;
    for (int t = threadIdx.x >> lgNG; t < Rc; t += rstep)
      tile[t * ts + gl] = okl ? m[(int64_t)t * phi + jl] : make_float2(0.f, 0.f);
    __syncthreads();
    if (mirror) {
      for (int t = glane; t < Tc; t += L)
        bufA[t] = t <= nth_c ? tile[t * ts + gid] : tile[(Tc - t) * ts + partner];
    } else {
      for (int t = glane; t < Tc; t += L) bufA[t] = tile[t * ts + gid];
    }
    __syncwarp();
    float2 *X = fft_group(bufA, bufB, pin, Win, false, glane, L, tin);
    float2 *Y = (X == bufA) ? bufB : bufA;
    pad_spectrum(X, Tc, Y, Tp, split, glane, L);
    float2 *Z = fft_group(Y, X, pout, Wout, true, glane, L, tout);
    // child centre - parent centre = (sx*a_x, sy*a_y, sz*a_z) with the octant signs of tree.h:672-687
    const float sgx = (o & 1) ? 1.f : -1.f, sgy = (o & 2) ? -1.f : 1.f, sgz = (o & 4) ? -1.f : 1.f;
    if (ok && tr == nullptr) {
      for (int t = glane; t < Rp; t += L) {
        float2 v = Z[t];
        float2 a = myacc[t];
        a.x += scale * v.x;
        a.y += scale * v.y;
        myacc[t] = a;
      }
    } else if (ok) {
      for (int t = glane; t < Rp; t += L) {
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
  float2 *out = parent + (((int64_t)slot * n_parent + p) * ncomp + comp) * (int64_t)Rp * phi;
  if (okl)
    for (int t = threadIdx.x >> lgNG; t < Rp; t += rstep) out[(int64_t)t * phi + jl] = acc[(size_t)gl * (Rp + 1) + t];
}

static size_t cols_smem(const FftPlan &pin, const FftPlan &pout, int Rc, int Rp, int NG) {
  const int nmax = std::max(pin.n, pout.n);
  return sizeof(float2) * ((size_t)pin.n + pout.n + (size_t)Rc * (NG + 1) + (size_t)NG * (Rp + 1) +
                           (size_t)NG * (2 * nmax + 1)) +
         sizeof(uint32_t) * (stage_table_size(pin) + stage_table_size(pout)) + 16;
}

po_status launch_interp_cols(const float2 *mid, float2 *parent, const int32_t *child_table, int64_t n_parent,
                             int64_t n_child, int phi, int Rc, int Rp, const FftPlan &pin, const FftPlan &pout,
                             const float2 *twiddles, const float4 *trans, int n_slots, int G, int quirk_reach,
                             float scale, int ncomp, int mirror, int ref_nyquist, cudaStream_t st) {
  if (n_parent <= 0 || n_slots <= 0) return PO_OK;
  if (mirror && (phi % 2 != 0 || pin.n % 2 != 0 || pout.n % 2 != 0 || Rc != pin.n / 2 + 1 || Rp != pout.n / 2 + 1))
    return fail(PO_ERR_INTERNAL, "mirrored column pass needs even sizes and half-stored rows");
  if (!mirror && (Rc != pin.n || Rp != pout.n)) return fail(PO_ERR_INTERNAL, "row counts must match the transforms");
  const int nmax = std::max(pin.n, pout.n);
  const int L = group_lanes(nmax);
  int threads = 256;
  // fewer columns per CTA when one tile would mostly hang over the grid edge
  const int span = mirror ? phi / 2 : phi;
  while (threads > 2 * L && (threads / L) / (mirror ? 2 : 1) >= 2 * span) threads >>= 1;
  while (cols_smem(pin, pout, Rc, Rp, threads / L) > 72 * 1024 && threads > std::max(64, 2 * L)) threads >>= 1;
  const int NG = threads / L;
  const size_t smem = cols_smem(pin, pout, Rc, Rp, NG);
  if (smem > 227 * 1024) return fail(PO_ERR_UNSUPPORTED, "angular grid too large for the shared-memory FFT");
  if (mirror && NG < 2) return fail(PO_ERR_UNSUPPORTED, "mirrored column pass needs two lane groups per CTA");
  int lg = 0;
  while ((1 << lg) < NG) ++lg;
  const int TW = mirror ? NG / 2 : NG;
  int64_t gx = (int64_t)((span + TW - 1) / TW) * n_parent * ncomp;
  if (gx > 2147483647LL || n_slots > 65535) return fail(PO_ERR_UNSUPPORTED, "too many nodes for one launch");
  dim3 grid((unsigned)gx, 1u, (unsigned)n_slots);
  k_interp_cols<<<grid, threads, smem, st>>>(mid, parent, child_table, n_parent, n_child, phi, Rc, Rp, pin, pout,
                                             twiddles, trans, G, quirk_reach, scale, ncomp, mirror, L, lg,
                                             ref_nyquist);
  count_launch();
  PO_CUDA(cudaGetLastError());
  return PO_OK;
}

// ----------------------------------------------------- translation table
// Direction factors of one level's grid (the terms of grid_direction):
// trig[it] = (cos th, sin th) for rows it < R, trig[R + ip] = (cos ph, sin ph).
// Built once per context, so the per-solve table below needs no FP64 trig.
__global__ void k_dir_trig(int nth, int R, int phi, double2 *__restrict__ trig) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < R) {
    const double th = -kPi / 2 + kThetaOffset + kPi / nth * e;
    trig[e] = make_double2(cos(th), sin(th));
  } else if (e < R + phi) {
    const double ph = kTwoPi / phi * (e - R);
    trig[e] = make_double2(cos(ph), sin(ph));
  }
}

po_status launch_dir_trig(int nth, int R, int phi, double2 *trig, cudaStream_t st) {
  if (R + phi <= 0) return PO_OK;
  k_dir_trig<<<(unsigned)((R + phi + 255) / 256), 256, 0, st>>>(nth, R, phi, trig);
  count_launch();
  PO_CUDA(cudaGetLastError());
  return PO_OK;
}

// r_a = (k * a_a * s_a) mod 2pi for a = x, y, z and every direction of a
// Tp x Phi grid (theta rows may run into the second cover), per wavelength;
// s = (cos th cos ph, cos th sin ph, sin th) from the level's trig table.
__global__ void k_trans_table(const double *__restrict__ k_per_lambda, int n_lambda, int Rp, int phi,
                              const double2 *__restrict__ trig, double ax, double ay, double az,
                              float4 *__restrict__ out) {
  int64_t d = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  int lam = blockIdx.y;
  int64_t nd = (int64_t)Rp * phi;
  if (d >= nd || lam >= n_lambda) return;
  int it = (int)(d / phi), ip = (int)(d % phi);
  const double2 th = trig[it], ph = trig[Rp + ip];
  const double s[3] = {th.x * ph.x, th.x * ph.y, th.y};
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

po_status launch_trans_table(const double *k_per_lambda, int n_lambda, int Rp, int phi, const double2 *trig,
                             const double a[3], float4 *out, cudaStream_t st) {
  int64_t nd = (int64_t)Rp * phi;
  if (nd <= 0 || n_lambda <= 0) return PO_OK;
  dim3 grid((unsigned)((nd + 255) / 256), (unsigned)n_lambda);
  k_trans_table<<<grid, 256, 0, st>>>(k_per_lambda, n_lambda, Rp, phi, trig, a[0], a[1], a[2], out);
  count_launch();
  PO_CUDA(cudaGetLastError());
  return PO_OK;
}

// opt-in shared-memory limit of the FFT interpolation kernels, set once per device
po_status init_fft_attributes(int max_smem) {
  PO_CUDA(cudaFuncSetAttribute(k_interp_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem));
  PO_CUDA(cudaFuncSetAttribute(k_interp_cols, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem));
  return PO_OK;
}

}  // namespace wavepo
