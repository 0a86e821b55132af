// po_common.cuh -- shared device/host helpers of the PO engine.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>

#include "wavepo.h"

namespace wavepo {

// util/util.h:16-19 (as double; the engine rounds to float where it needs to)
constexpr double kC0 = 299792458.0;
constexpr double kMu0 = 4e-7 * 3.14159265358979323846;
constexpr double kEps0 = 8.8541878e-12;
constexpr double kPi = 3.14159265358979323846;
constexpr double kTwoPi = 6.28318530717958647692;
constexpr double kThetaOffset = 1e-10;  // compareMie/sphere.cu:53

inline double z0_host() { return std::sqrt(kMu0 / kEps0); }

// ------------------------------------------------------------------ complex
template <typename T>
struct cx {
  T re, im;
};
template <typename T>
__host__ __device__ __forceinline__ cx<T> mk(T r, T i) { return cx<T>{r, i}; }
template <typename T>
__host__ __device__ __forceinline__ cx<T> operator+(cx<T> a, cx<T> b) { return {a.re + b.re, a.im + b.im}; }
template <typename T>
__host__ __device__ __forceinline__ cx<T> operator-(cx<T> a, cx<T> b) { return {a.re - b.re, a.im - b.im}; }
template <typename T>
__host__ __device__ __forceinline__ cx<T> operator-(cx<T> a) { return {-a.re, -a.im}; }
template <typename T>
__host__ __device__ __forceinline__ cx<T> operator*(cx<T> a, cx<T> b) {
  return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
template <typename T>
__host__ __device__ __forceinline__ cx<T> operator*(cx<T> a, T s) { return {a.re * s, a.im * s}; }
template <typename T>
__host__ __device__ __forceinline__ cx<T> operator*(T s, cx<T> a) { return {a.re * s, a.im * s}; }
template <typename T>
__host__ __device__ __forceinline__ cx<T> cdiv(cx<T> a, cx<T> b) {
  T d = b.re * b.re + b.im * b.im;
  return {(a.re * b.re + a.im * b.im) / d, (a.im * b.re - a.re * b.im) / d};
}
template <typename T>
__host__ __device__ __forceinline__ cx<T> conjg(cx<T> a) { return {a.re, -a.im}; }
template <typename T>
__host__ __device__ __forceinline__ T cabs2(cx<T> a) { return a.re * a.re + a.im * a.im; }

// principal square root
__host__ __device__ __forceinline__ cx<double> csqrt_(cx<double> z) {
  double r = sqrt(z.re * z.re + z.im * z.im);
  double a = sqrt(fmax(0.5 * (r + z.re), 0.0));
  double b = sqrt(fmax(0.5 * (r - z.re), 0.0));
  return {a, z.im < 0 ? -b : b};
}
__host__ __device__ __forceinline__ cx<float> csqrt_(cx<float> z) {
  float r = sqrtf(z.re * z.re + z.im * z.im);
  float a = sqrtf(fmaxf(0.5f * (r + z.re), 0.0f));
  float b = sqrtf(fmaxf(0.5f * (r - z.re), 0.0f));
  return {a, z.im < 0 ? -b : b};
}

// e^{i t} for a possibly large double argument: t is reduced modulo 2 pi in
// double (Cody-Waite style: n = rint(t / 2pi), r = t - n*2pi with 2pi split in
// a head and a tail), then the small remainder is evaluated in float.
__device__ __forceinline__ float2 expi_reduced(double t) {
  const double inv2pi = 0.15915494309189533577;
  const double p_hi = 6.28318530717958623200;   // 2pi rounded to double
  const double p_lo = 2.44929359829470635445e-16;  // 2pi - p_hi
  double n = rint(t * inv2pi);
  double r = fma(-n, p_hi, t);
  r = fma(-n, p_lo, r);
  float s, c;
  sincosf((float)r, &s, &c);
  return make_float2(c, s);
}

// Reduce a float phase of moderate size to [-pi, pi] (two-term Cody-Waite
// split of 2pi) and evaluate e^{i r} with the SFU approximation.
__device__ __forceinline__ void sincos_small(float ph, float *s, float *c) {
  const float inv2pi = 0.159154943091895f;
  float n = rintf(ph * inv2pi);
  float r = fmaf(-n, 6.28318548202514648f, ph);
  r = fmaf(-n, -1.74845553e-7f, r);
  __sincosf(r, s, c);
}

// ------------------------------------------------ split-bf16 tensor products
// mma.sync m16n8k16, bf16 operands, FP32 accumulation.  Not volatile: a pure
// function of its operands, so the scheduler may interleave independent
// accumulators.
__device__ __forceinline__ void mma_bf16(float *d, const uint32_t *a, const uint32_t *b) {
  asm("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// (x0, x1) -> bf16x2 hi = rn(x), lo = rn(x - hi), x0 in the low half (fragment
// order): two packed conversions, the hi parts widened back by shifts.
__device__ __forceinline__ void split_bf16x2(float x0, float x1, uint32_t &hi, uint32_t &lo) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(x0, x1);
  uint32_t hu;
  memcpy(&hu, &h, 4);
  const float h0 = __uint_as_float(hu << 16), h1 = __uint_as_float(hu & 0xffff0000u);
  const __nv_bfloat162 l = __floats2bfloat162_rn(x0 - h0, x1 - h1);
  hi = hu;
  memcpy(&lo, &l, 4);
}

// ------------------------------------------------------------------ vectors
template <typename T>
struct v3 {
  T x, y, z;
};
template <typename T>
__host__ __device__ __forceinline__ T dot3(v3<T> a, v3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <typename T>
__host__ __device__ __forceinline__ v3<T> cross3(v3<T> a, v3<T> b) {
  return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, b.y * a.x - a.y * b.x};
}

// Incident plane wave (compareMie/sphere.cu:559-579).  Computed on the host in
// double and passed to the kernels.
struct Incident {
  double wavedir[3], edir[3], hdir[3];
};
inline Incident make_incident(double theta_i, double phi_i, bool te) {
  Incident in;
  in.wavedir[0] = std::cos(theta_i) * std::cos(phi_i);
  in.wavedir[1] = std::cos(theta_i) * std::sin(phi_i);
  in.wavedir[2] = std::sin(theta_i);
  if (!te) {
    in.edir[0] = -std::sin(theta_i) * std::cos(phi_i);
    in.edir[1] = -std::sin(theta_i) * std::sin(phi_i);
    in.edir[2] = std::cos(theta_i);
    in.hdir[0] = std::sin(phi_i);
    in.hdir[1] = -std::cos(phi_i);
    in.hdir[2] = 0.0;
  } else {
    in.edir[0] = -std::sin(phi_i);
    in.edir[1] = std::cos(phi_i);
    in.edir[2] = 0.0;
    in.hdir[0] = -std::sin(theta_i) * std::cos(phi_i);
    in.hdir[1] = -std::sin(theta_i) * std::sin(phi_i);
    in.hdir[2] = std::cos(theta_i);
  }
  return in;
}

// Everything the tangent-plane model needs for one (lambda, incidence, pol),
// in the precision of the kernel.  `ef`/`hf` fold field_times_area's unit
// scale with the E/H prefactors (fields.h:123-150, sphere.cu:491-494).
template <typename T>
struct SlotParams {
  T wavedir[3], edir[3], hdir[3];
  T eta_re, eta_im;
  T z0, inv_two_sigma2, k0;
  double k0d;          // k0 in double for the incident phase argument
  double wd[3];        // wave direction in double for the incident phase argument
  T ef_re, ef_im, hf_re, hf_im;
  int te;
};

template <typename T>
inline SlotParams<T> make_slot(double lambda_m, double theta_i, double phi_i, bool te, double eta_re,
                               double eta_im, double sigma, double distance, bool scale) {
  Incident in = make_incident(theta_i, phi_i, te);
  SlotParams<T> p;
  for (int a = 0; a < 3; ++a) {
    p.wavedir[a] = (T)in.wavedir[a];
    p.edir[a] = (T)in.edir[a];
    p.hdir[a] = (T)in.hdir[a];
    p.wd[a] = in.wavedir[a];
  }
  p.eta_re = (T)eta_re;
  p.eta_im = (T)eta_im;
  p.z0 = (T)z0_host();
  p.inv_two_sigma2 = (T)(0.5 / (sigma * sigma));
  double k0 = kTwoPi / lambda_m;
  p.k0 = (T)k0;
  p.k0d = k0;
  p.te = te ? 1 : 0;
  if (scale) {
    // Efactor = -i w mu0/(4pi) e^{-i k0 Dis}/Dis ; Hfactor with eps0
    double omega = k0 * kC0;
    double ph = -std::fmod(k0 * distance, kTwoPi);
    double gr = std::cos(ph) / distance, gi = std::sin(ph) / distance;
    double ea = omega * kMu0 / (4 * kPi), ha = omega * kEps0 / (4 * kPi);
    // -i * a * (gr + i gi) = a*gi - i a*gr
    p.ef_re = (T)(ea * gi);
    p.ef_im = (T)(-ea * gr);
    p.hf_re = (T)(ha * gi);
    p.hf_im = (T)(-ha * gr);
  } else {
    p.ef_re = (T)1;
    p.ef_im = (T)0;
    p.hf_re = (T)1;
    p.hf_im = (T)0;
  }
  return p;
}

// util/util.h:365-382
template <typename T>
__device__ __forceinline__ cx<T> cos_internal_angle(cx<T> n, T theta) {
  T s = sin(theta);
  cx<T> q = cdiv(mk<T>(s, 0), n);
  q = cdiv(q * s, n);
  return csqrt_(mk<T>(1 - q.re, -q.im));
}
template <typename T>
__device__ __forceinline__ cx<T> fresnel_rs(T theta, cx<T> n0, cx<T> nt) {
  cx<T> p0 = n0 * cos_internal_angle(n0, theta);
  cx<T> pt = nt * cos_internal_angle(cdiv(nt, n0), theta);
  return cdiv(p0 - pt, p0 + pt);
}
template <typename T>
__device__ __forceinline__ cx<T> fresnel_rp(T theta, cx<T> n0, cx<T> nt) {
  cx<T> q0 = cdiv(cos_internal_angle(n0, theta), n0);
  cx<T> qt = cdiv(cos_internal_angle(nt, theta), nt);
  return cdiv(q0 - qt, q0 + qt);
}

// Tangent-plane currents of one point (util/tangentplane.h:19-80) times area
// and the E/H prefactors.  out[0..2] = J, out[3..5] = M.  Decisions are taken
// in float as the reference takes them.
template <typename T>
__device__ __forceinline__ void tangent_plane(const SlotParams<T> &P, float px, float py, float pz, float qx,
                                              float qy, float qz, float area, cx<T> out[6]) {
  v3<T> kd = {P.wavedir[0], P.wavedir[1], P.wavedir[2]};
  v3<T> nr = {(T)qx, (T)qy, (T)qz};
  T dotvalue = dot3(kd, nr);
  cx<T> Ei[3] = {{0, 0}, {0, 0}, {0, 0}}, Hi[3] = {{0, 0}, {0, 0}, {0, 0}};
  cx<T> Es[3] = {{0, 0}, {0, 0}, {0, 0}}, Hs[3] = {{0, 0}, {0, 0}, {0, 0}};
  float dot_f = (float)dotvalue;
  if (dot_f <= 0.0f) {
    // incident phase exp(-i k0 k.x) with the argument formed in double
    double dd = P.wd[0] * (double)px + P.wd[1] * (double)py + P.wd[2] * (double)pz;
    float2 e = expi_reduced(-P.k0d * dd);
    T beam = exp(-(T)pz * (T)pz * P.inv_two_sigma2);
    cx<T> Ei0 = {beam * (T)e.x, beam * (T)e.y};
    cx<T> Hi0 = Ei0 * ((T)1 / P.z0);
    Ei[0] = Ei0 * P.edir[0]; Ei[1] = Ei0 * P.edir[1]; Ei[2] = Ei0 * P.edir[2];
    Hi[0] = Hi0 * P.hdir[0]; Hi[1] = Hi0 * P.hdir[1]; Hi[2] = Hi0 * P.hdir[2];
    cx<T> eta_in = {1, 0}, eta_out = {P.eta_re, P.eta_im};
    if (fabsf(fabsf(dot_f) - 1.0f) < 1e-10f) {  // tangentplane.h:39-49
      cx<T> R = P.te ? cdiv(eta_out - eta_in, eta_in + eta_out) : cdiv(eta_in - eta_out, eta_in + eta_out);
      for (int c = 0; c < 3; ++c) { Es[c] = Ei[c] * R; Hs[c] = Hi[c] * R; }
    } else {  // tangentplane.h:51-62
      v3<T> rp = cross3(kd, nr);
      T inv = (T)1 / sqrt(dot3(rp, rp));
      rp = {rp.x * inv, rp.y * inv, rp.z * inv};
      cx<T> f = Ei[0] * rp.x + Ei[1] * rp.y + Ei[2] * rp.z;
      cx<T> Eperp[3] = {f * rp.x, f * rp.y, f * rp.z};
      cx<T> Epar[3] = {Ei[0] - Eperp[0], Ei[1] - Eperp[1], Ei[2] - Eperp[2]};
      T iz = (T)1 / P.z0;
      cx<T> Hpar[3] = {(Epar[2] * kd.y - Epar[1] * kd.z) * iz, (Epar[0] * kd.z - Epar[2] * kd.x) * iz,
                       (Epar[1] * kd.x - Epar[0] * kd.y) * iz};
      cx<T> Hperp[3] = {Hi[0] - Hpar[0], Hi[1] - Hpar[1], Hi[2] - Hpar[2]};
      T lphi = acos(fabs(dotvalue));
      cx<T> Rs = fresnel_rs(lphi, eta_in, eta_out);
      cx<T> Rp = fresnel_rp(lphi, eta_in, eta_out);
      for (int c = 0; c < 3; ++c) {
        Es[c] = Eperp[c] * Rs - Epar[c] * Rp;
        Hs[c] = Hpar[c] * Rp - Hperp[c] * Rs;
      }
    }
  }
  // shadowed points: Ei = Hi = 0 so Es = -Ei = 0 (tangentplane.h:64-67)
  cx<T> Et[3], Ht[3];
  for (int c = 0; c < 3; ++c) { Et[c] = Ei[c] + Es[c]; Ht[c] = Hi[c] + Hs[c]; }
  // M = Et x n ; J = n x Ht (tangentplane.h:70-71)
  cx<T> M[3] = {Et[1] * nr.z - Et[2] * nr.y, Et[2] * nr.x - Et[0] * nr.z, Et[0] * nr.y - Et[1] * nr.x};
  cx<T> J[3] = {Ht[2] * nr.y - Ht[1] * nr.z, Ht[0] * nr.z - Ht[2] * nr.x, Ht[1] * nr.x - Ht[0] * nr.y};
  cx<T> ef = {P.ef_re * (T)area, P.ef_im * (T)area}, hf = {P.hf_re * (T)area, P.hf_im * (T)area};
  for (int c = 0; c < 3; ++c) { out[c] = J[c] * ef; out[3 + c] = M[c] * hf; }
}

// Direction of grid sample (it, ip) (compareMie/sphere.cu:370-384); `it` may
// run past n_theta into the second cover of the sphere.
__host__ __device__ __forceinline__ void grid_direction(int it, int ip, int nth, int nph, double s[3]) {
  double th = -kPi / 2 + kThetaOffset + kPi / nth * it;
  double ph = kTwoPi / nph * ip;
  double ct = cos(th), st = sin(th);
  s[0] = ct * cos(ph);
  s[1] = ct * sin(ph);
  s[2] = st;
}

}  // namespace wavepo
