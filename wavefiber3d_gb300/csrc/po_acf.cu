// po_acf.cu -- spectra and autocorrelations of pattern ensembles on the GPU.
//
// Replaces the statistics of fitting/fittingutil.py:22-74, which the fitting
// notebook (fitting/fitnoise.ipynb) runs on many rough-fiber pattern
// instances:
//   ForwardFFT_shifted(A) = roll(FFT2(roll(A, s)), -s),  s = floor(n/2) per axis
//   InverseFFT_shifted(A) = roll(IFFT2(roll(A, -s)), s)   (unnormalised)
//   ACFfromFT:  F = mean_i |ForwardFFT_shifted(noise_i - mean)|,
//               acf = Re ForwardFFT_shifted(F^2)
// (ACFweightedFT and weightedsum are elementwise combinations around the same
// transform; the Python layer composes them.)
//
// The shifted transform is one DFT per axis with the kernel
//   W[k][m] = exp(-2 pi i ((m + s)(k + s) mod n) / n),
// because roll(A, s)[j] = A[j - s] and roll(R, -s)[k] = R[k + s]; the inverse
// has exp(+2 pi i ((m - s)(k - s) mod n) / n).  The tables
// are built on the device from the exact integer phase ((m+s)(k+s) mod n) with
// FP64 sincospi, and each axis is a tiled complex product (32 x 32 output
// tiles, operands staged in shared memory, FP32 accumulation).  The FFTW
// transform of the reference is unnormalised; so is this one.
#include <cuda_runtime.h>

#include <algorithm>

#include "po_internal.h"
#include "po_kernels.h"

namespace wavepo {

namespace {

constexpr int kDt = 32;  // output tile (batch rows x transform bins)

__global__ void k_dft_table(float2 *__restrict__ W, int n, int inverse) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= (int64_t)n * n) return;
  const int64_t k = e / n, m = e % n, s = inverse ? (n - n / 2) % n : n / 2;
  const int64_t ph = ((m + s) % n) * ((k + s) % n) % n;
  double sn, cs;
  sincospi((inverse ? 2.0 : -2.0) * (double)ph / (double)n, &sn, &cs);
  W[e] = make_float2((float)cs, (float)sn);
}

// out[b][k] = sum_m W[k][m] in[b][m] along one axis.  Element (b, m) of an
// array lives at (b / inner) * outer + (b % inner) * istride + m * mstride.
__global__ void __launch_bounds__(256) k_dft_axis(const float2 *__restrict__ in, float2 *__restrict__ out,
                                                  const float2 *__restrict__ W, int64_t nb, int n, int64_t inner,
                                                  int64_t outer, int64_t istride, int64_t mstride) {
  __shared__ float2 sA[kDt][kDt + 1];  // [b][m]
  __shared__ float2 sW[kDt][kDt + 1];  // [k][m]
  const int64_t b0 = (int64_t)blockIdx.x * kDt;
  const int k0 = blockIdx.y * kDt;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
  auto base = [&](int64_t b) { return (b / inner) * outer + (b % inner) * istride; };
  float2 acc[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) acc[i] = make_float2(0.f, 0.f);
  const bool m_fast = mstride == 1;
  for (int m0 = 0; m0 < n; m0 += kDt) {
    __syncthreads();
    for (int e = threadIdx.x; e < kDt * kDt; e += blockDim.x) {
      // coalesce along whichever index is contiguous in memory
      const int bi = m_fast ? e / kDt : e % kDt, mi = m_fast ? e % kDt : e / kDt;
      const int64_t b = b0 + bi;
      const int m = m0 + mi;
      sA[bi][mi] = (b < nb && m < n) ? in[base(b) + (int64_t)m * mstride] : make_float2(0.f, 0.f);
      const int kk = k0 + e / kDt, mm = m0 + e % kDt;
      sW[e / kDt][e % kDt] = (kk < n && mm < n) ? W[(int64_t)kk * n + mm] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    // thread (tx, ty): bin k = k0 + tx, rows b = b0 + ty + 8 i
#pragma unroll 8
    for (int mi = 0; mi < kDt; ++mi) {
      const float2 w = sW[tx][mi];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const float2 a = sA[ty + 8 * i][mi];
        acc[i].x = fmaf(w.x, a.x, fmaf(-w.y, a.y, acc[i].x));
        acc[i].y = fmaf(w.x, a.y, fmaf(w.y, a.x, acc[i].y));
      }
    }
  }
  const int k = k0 + tx;
  if (k >= n) return;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int64_t b = b0 + ty + 8 * i;
    if (b < nb) out[base(b) + (int64_t)k * mstride] = acc[i];
  }
}

// batch x [nth][nph] complex -> shifted 2-D DFT (phi axis first, then theta)
po_status shifted_fft2(const float2 *in, float2 *out, float2 *tmp, const float2 *Wth, const float2 *Wph, int batch,
                       int nth, int nph, cudaStream_t st) {
  const int64_t plane = (int64_t)nth * nph;
  {  // phi axis: b = item*nth + theta, m = phi
    const int64_t nb = (int64_t)batch * nth;
    dim3 grid((unsigned)((nb + kDt - 1) / kDt), (unsigned)((nph + kDt - 1) / kDt));
    k_dft_axis<<<grid, 256, 0, st>>>(in, tmp, Wph, nb, nph, 1, nph, 0, 1);
    count_launch();
  }
  {  // theta axis: b = item*nph + phi, m = theta
    const int64_t nb = (int64_t)batch * nph;
    dim3 grid((unsigned)((nb + kDt - 1) / kDt), (unsigned)((nth + kDt - 1) / kDt));
    k_dft_axis<<<grid, 256, 0, st>>>(tmp, out, Wth, nb, nth, nph, plane, 1, nph);
    count_launch();
  }
  PO_CUDA(cudaGetLastError());
  return PO_OK;
}

po_status dft_tables(float2 *Wth, float2 *Wph, int nth, int nph, int inverse, cudaStream_t st) {
  k_dft_table<<<(unsigned)(((int64_t)nth * nth + 255) / 256), 256, 0, st>>>(Wth, nth, inverse);
  k_dft_table<<<(unsigned)(((int64_t)nph * nph + 255) / 256), 256, 0, st>>>(Wph, nph, inverse);
  count_launch();
  count_launch();
  PO_CUDA(cudaGetLastError());
  return PO_OK;
}

// mean over instances of real patterns [ni][nd] (fittingutil.py:65 order)
__global__ void k_mean(const float *__restrict__ p, int ni, int64_t nd, float *__restrict__ mean) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= nd) return;
  float s = 0.f;
  for (int i = 0; i < ni; ++i) s += p[(int64_t)i * nd + e] / (float)ni;
  mean[e] = s;
}

// x_i = p_i - mean as complex
__global__ void k_center(const float *__restrict__ p, const float *__restrict__ mean, int64_t nd, int64_t total,
                         float2 *__restrict__ x) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= total) return;
  x[e] = make_float2(p[e] - mean[e % nd], 0.f);
}

// F = sum_i |X_i| / ni (fittingutil.py:69-72); F2 = F^2 as complex
__global__ void k_abs_mean(const float2 *__restrict__ X, int ni, int64_t nd, float *__restrict__ F,
                           float2 *__restrict__ F2) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= nd) return;
  float s = 0.f;
  for (int i = 0; i < ni; ++i) {
    const float2 v = X[(int64_t)i * nd + e];
    s += hypotf(v.x, v.y) / (float)ni;
  }
  F[e] = s;
  F2[e] = make_float2(s * s, 0.f);
}

__global__ void k_real_part(const float2 *__restrict__ z, int64_t n, float *__restrict__ r) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e < n) r[e] = z[e].x;
}

unsigned blocks_for(int64_t n) { return (unsigned)((n + 255) / 256); }

}  // namespace

}  // namespace wavepo

using namespace wavepo;

extern "C" po_status po_shifted_fft2(const float *in, float *out, int batch, int n_theta, int n_phi, int inverse,
                                     void *stream) {
  if (!in || !out) return fail(PO_ERR_INVALID_ARGUMENT, "null pointer");
  if (inverse != 0 && inverse != 1) return fail(PO_ERR_INVALID_ARGUMENT, "inverse must be 0 or 1");
  if (batch < 0 || n_theta <= 0 || n_phi <= 0 || n_theta > 8192 || n_phi > 8192)
    return fail(PO_ERR_INVALID_ARGUMENT, "batch >= 0 and 0 < n_theta, n_phi <= 8192 required");
  if (batch == 0) return PO_OK;
  if ((int64_t)batch * std::max(n_theta, n_phi) > (int64_t)1 << 35)  // grid.x < 2^31
    return fail(PO_ERR_INVALID_ARGUMENT, "batch too large");
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t plane = (int64_t)n_theta * n_phi;
  float2 *scratch = nullptr;
  const size_t words = (size_t)batch * plane + (size_t)n_theta * n_theta + (size_t)n_phi * n_phi;
  PO_CUDA(cudaMallocAsync((void **)&scratch, sizeof(float2) * words, st));
  float2 *tmp = scratch, *Wth = tmp + (size_t)batch * plane, *Wph = Wth + (size_t)n_theta * n_theta;
  po_status s = dft_tables(Wth, Wph, n_theta, n_phi, inverse, st);
  if (s == PO_OK) s = shifted_fft2((const float2 *)in, (float2 *)out, tmp, Wth, Wph, batch, n_theta, n_phi, st);
  cudaFreeAsync(scratch, st);
  return s;
}

extern "C" po_status po_acf_from_patterns(const float *patterns, int n_inst, int n_theta, int n_phi, float *mean,
                                          float *spectrum, float *acf, void *stream) {
  if (!patterns || !mean || !spectrum || !acf) return fail(PO_ERR_INVALID_ARGUMENT, "null pointer");
  if (n_inst <= 0 || n_theta <= 0 || n_phi <= 0 || n_theta > 8192 || n_phi > 8192)
    return fail(PO_ERR_INVALID_ARGUMENT, "n_inst > 0 and 0 < n_theta, n_phi <= 8192 required");
  if ((int64_t)n_inst * std::max(n_theta, n_phi) > (int64_t)1 << 35)
    return fail(PO_ERR_INVALID_ARGUMENT, "too many instances");
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t nd = (int64_t)n_theta * n_phi, total = nd * n_inst;
  float2 *scratch = nullptr;
  const size_t words = 2 * (size_t)total + 2 * (size_t)nd + (size_t)n_theta * n_theta + (size_t)n_phi * n_phi;
  PO_CUDA(cudaMallocAsync((void **)&scratch, sizeof(float2) * words, st));
  float2 *X = scratch, *tmp = X + total, *F2 = tmp + total, *A = F2 + nd;
  float2 *Wth = A + nd, *Wph = Wth + (size_t)n_theta * n_theta;
  po_status s = dft_tables(Wth, Wph, n_theta, n_phi, 0, st);
  if (s == PO_OK) {
    k_mean<<<blocks_for(nd), 256, 0, st>>>(patterns, n_inst, nd, mean);
    k_center<<<blocks_for(total), 256, 0, st>>>(patterns, mean, nd, total, X);
    count_launch();
    count_launch();
    s = shifted_fft2(X, X, tmp, Wth, Wph, n_inst, n_theta, n_phi, st);
  }
  if (s == PO_OK) {
    k_abs_mean<<<blocks_for(nd), 256, 0, st>>>(X, n_inst, nd, spectrum, F2);
    count_launch();
    s = shifted_fft2(F2, A, tmp, Wth, Wph, 1, n_theta, n_phi, st);
  }
  if (s == PO_OK) {
    k_real_part<<<blocks_for(nd), 256, 0, st>>>(A, nd, acf);
    count_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) s = cuda_fail(e, "acf launch");
  }
  cudaFreeAsync(scratch, st);
  return s;
}
