// po_dual.cuh -- forward-mode dual numbers and the differentiated
// tangent-plane model (util/tangentplane.h:19-80, util/util.h:365-382).
//
// Dual<T, N> carries N tangents.  A selector sel[N] names the global tangent
// (0..6 = x, y, z, nx, ny, nz, area) each slot follows, so one point's
// Jacobian can be split over several threads (-1: an unused slot).
#pragma once

#include "po_common.cuh"

namespace wavepo {

constexpr int kNT = 7;  // tangents: x, y, z, nx, ny, nz, area

template <typename T, int N = kNT>
struct Dual {
  T v;
  T d[N];
};

template <typename T, int N>
__device__ __forceinline__ Dual<T, N> dconst(T v) {
  Dual<T, N> r;
  r.v = v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = (T)0;
  return r;
}
// the variable of global tangent gi: derivative 1 in the slot that follows it
template <typename T, int N>
__device__ __forceinline__ Dual<T, N> dvar(T v, int gi, const int (&sel)[N]) {
  Dual<T, N> r = dconst<T, N>(v);
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = sel[i] == gi ? (T)1 : (T)0;
  return r;
}
// f(u) with f(u.v) = fv and f'(u.v) = fp
template <typename T, int N>
__device__ __forceinline__ Dual<T, N> dchain(const Dual<T, N> &u, T fv, T fp) {
  Dual<T, N> r;
  r.v = fv;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = fp * u.d[i];
  return r;
}
template <typename T, int N>
__device__ __forceinline__ Dual<T, N> operator+(const Dual<T, N> &a, const Dual<T, N> &b) {
  Dual<T, N> r;
  r.v = a.v + b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + b.d[i];
  return r;
}
template <typename T, int N>
__device__ __forceinline__ Dual<T, N> operator-(const Dual<T, N> &a, const Dual<T, N> &b) {
  Dual<T, N> r;
  r.v = a.v - b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - b.d[i];
  return r;
}
template <typename T, int N>
__device__ __forceinline__ Dual<T, N> operator-(const Dual<T, N> &a) { return dchain(a, -a.v, (T)-1); }
template <typename T, int N>
__device__ __forceinline__ Dual<T, N> operator*(const Dual<T, N> &a, const Dual<T, N> &b) {
  Dual<T, N> r;
  r.v = a.v * b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
  return r;
}
template <typename T, int N>
__device__ __forceinline__ Dual<T, N> operator*(const Dual<T, N> &a, T s) { return dchain(a, a.v * s, s); }
template <typename T, int N>
__device__ __forceinline__ Dual<T, N> operator/(const Dual<T, N> &a, const Dual<T, N> &b) {
  Dual<T, N> r;
  const T ib = (T)1 / b.v;
  r.v = a.v * ib;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) * ib;
  return r;
}
template <typename T, int N>
__device__ __forceinline__ Dual<T, N> dsqrt(const Dual<T, N> &a) {
  const T s = sqrt(a.v);
  return dchain(a, s, s > (T)0 ? (T)0.5 / s : (T)0);
}
template <typename T, int N>
__device__ __forceinline__ Dual<T, N> dexp(const Dual<T, N> &a) {
  const T e = exp(a.v);
  return dchain(a, e, e);
}
template <typename T, int N>
__device__ __forceinline__ Dual<T, N> dabs(const Dual<T, N> &a) { return a.v < (T)0 ? -a : a; }

template <typename T, int N = kNT>
using CDual = cx<Dual<T, N>>;
template <typename T, int N>
__device__ __forceinline__ CDual<T, N> cd(T re, T im) { return {dconst<T, N>(re), dconst<T, N>(im)}; }
template <typename T, int N>
__device__ __forceinline__ CDual<T, N> operator*(const CDual<T, N> &a, const CDual<T, N> &b) {
  return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
template <typename T, int N>
__device__ __forceinline__ CDual<T, N> operator*(const CDual<T, N> &a, const Dual<T, N> &s) {
  return {a.re * s, a.im * s};
}
template <typename T, int N>
__device__ __forceinline__ CDual<T, N> operator*(const CDual<T, N> &a, T s) { return {a.re * s, a.im * s}; }
template <typename T, int N>
__device__ __forceinline__ CDual<T, N> operator+(const CDual<T, N> &a, const CDual<T, N> &b) {
  return {a.re + b.re, a.im + b.im};
}
template <typename T, int N>
__device__ __forceinline__ CDual<T, N> operator-(const CDual<T, N> &a, const CDual<T, N> &b) {
  return {a.re - b.re, a.im - b.im};
}
template <typename T, int N>
__device__ __forceinline__ CDual<T, N> cddiv(const CDual<T, N> &a, const CDual<T, N> &b) {
  Dual<T, N> d = b.re * b.re + b.im * b.im;
  return {(a.re * b.re + a.im * b.im) / d, (a.im * b.re - a.re * b.im) / d};
}
// principal square root (as csqrt_ of po_common.cuh)
template <typename T, int N>
__device__ __forceinline__ CDual<T, N> cdsqrt(const CDual<T, N> &z) {
  const Dual<T, N> r = dsqrt(z.re * z.re + z.im * z.im);
  const Dual<T, N> ha = (r + z.re) * (T)0.5, hb = (r - z.re) * (T)0.5;
  const Dual<T, N> a = ha.v > (T)0 ? dsqrt(ha) : dconst<T, N>(0);
  const Dual<T, N> b = hb.v > (T)0 ? dsqrt(hb) : dconst<T, N>(0);
  return {a, z.im.v < (T)0 ? -b : b};
}
// util/util.h:365-382, differentiated in terms of x = cos(theta) = |k.n|
// and s2 = sin^2(theta) = 1 - x^2 instead of theta itself.  The reference
// evaluates sqrt(1 - (sin(theta)/n)^2) with theta = acos(x); the values agree,
// but the derivative of acos (-1/sqrt(1 - x^2)) and of sin are singular at
// normal incidence and cancel only analytically: in FP32 their product loses
// about eps/theta^2 of relative accuracy, which near the specular points of a
// surface swamps the normal gradient.  d(s2)/dx = -2x carries no such factor.
// For the incident medium n = 1 the angle cosine is x itself.
template <typename T, int N>
__device__ __forceinline__ CDual<T, N> d_cos_internal(const CDual<T, N> &n, const Dual<T, N> &x, const Dual<T, N> &s2) {
  if (n.re.v == (T)1 && n.im.v == (T)0) return {x, dconst<T, N>(0)};
  CDual<T, N> q = cddiv(CDual<T, N>{s2, dconst<T, N>(0)}, n);
  q = cddiv(q, n);
  return cdsqrt(CDual<T, N>{dconst<T, N>(1) - q.re, -q.im});
}
template <typename T, int N>
__device__ __forceinline__ CDual<T, N> d_rs(const Dual<T, N> &x, const Dual<T, N> &s2, const CDual<T, N> &n0,
                                            const CDual<T, N> &nt) {
  CDual<T, N> p0 = n0 * d_cos_internal(n0, x, s2);
  CDual<T, N> pt = nt * d_cos_internal(cddiv(nt, n0), x, s2);
  return cddiv(p0 - pt, p0 + pt);
}
template <typename T, int N>
__device__ __forceinline__ CDual<T, N> d_rp(const Dual<T, N> &x, const Dual<T, N> &s2, const CDual<T, N> &n0,
                                            const CDual<T, N> &nt) {
  CDual<T, N> q0 = cddiv(d_cos_internal(n0, x, s2), n0);
  CDual<T, N> qt = cddiv(d_cos_internal(nt, x, s2), nt);
  return cddiv(q0 - qt, q0 + qt);
}

// The tangent-plane model of tangent_plane() (po_common.cuh) on dual inputs
// in precision T: the same branches (taken on the float-rounded values, as
// the forward kernels take them), differentiated.  The incident phase value
// k0 w.x is formed and reduced in FP64 whatever T is (its sine and cosine in
// FP64 for T = double, in FP32 of the reduced argument for T = float, as the
// forward kernels take them); its derivative is -k0 w.  out[0..2] = J,
// out[3..5] = M.
template <typename T, int N>
__device__ __forceinline__ void tangent_plane_jvp(const SlotParams<double> &P, float px, float py, float pz, float qx, float qy,
                                  float qz, float area, const int (&sel)[N], CDual<T, N> out[6]) {
  const Dual<T, N> Z = dvar<T, N>(pz, 2, sel);
  const Dual<T, N> nr[3] = {dvar<T, N>(qx, 3, sel), dvar<T, N>(qy, 4, sel), dvar<T, N>(qz, 5, sel)};
  const Dual<T, N> Ar = dvar<T, N>(area, 6, sel);
  const T kd[3] = {(T)P.wavedir[0], (T)P.wavedir[1], (T)P.wavedir[2]};
  const Dual<T, N> dotvalue = nr[0] * kd[0] + nr[1] * kd[1] + nr[2] * kd[2];
  const CDual<T, N> zero = cd<T, N>(0, 0);
  CDual<T, N> Ei[3] = {zero, zero, zero}, Hi[3] = {zero, zero, zero};
  CDual<T, N> Es[3] = {zero, zero, zero}, Hs[3] = {zero, zero, zero};
  const float dot_f = (float)(P.wavedir[0] * qx + P.wavedir[1] * qy + P.wavedir[2] * qz);
  if (dot_f <= 0.0f) {
    // incident phase exp(-i k0 w.x) and beam exp(-z^2 / (2 sigma^2))
    const double argd = -P.k0d * (P.wd[0] * (double)px + P.wd[1] * (double)py + P.wd[2] * (double)pz);
    const double rd = argd - kTwoPi * rint(argd * (1.0 / kTwoPi));
    T snd, csd;
    if constexpr (sizeof(T) == sizeof(double)) {
      sincos(rd, &snd, &csd);
    } else {
      sincosf((float)rd, &snd, &csd);
    }
    Dual<T, N> arg = dconst<T, N>((T)rd);
#pragma unroll
    for (int i = 0; i < N; ++i) arg.d[i] = (sel[i] >= 0 && sel[i] < 3) ? (T)(-P.k0d * P.wd[sel[i]]) : (T)0;
    const CDual<T, N> e = {dchain(arg, csd, -snd), dchain(arg, snd, csd)};
    const Dual<T, N> beam = dexp(-(Z * Z) * (T)P.inv_two_sigma2);
    const CDual<T, N> Ei0 = e * beam;
    const CDual<T, N> Hi0 = Ei0 * (T)(1.0 / P.z0);
    for (int c = 0; c < 3; ++c) {
      Ei[c] = Ei0 * (T)P.edir[c];
      Hi[c] = Hi0 * (T)P.hdir[c];
    }
    const CDual<T, N> eta_in = cd<T, N>(1, 0), eta_out = cd<T, N>((T)P.eta_re, (T)P.eta_im);
    if (fabsf(fabsf(dot_f) - 1.0f) < 1e-10f) {  // tangentplane.h:39-49
      const CDual<T, N> R =
          P.te ? cddiv(eta_out - eta_in, eta_in + eta_out) : cddiv(eta_in - eta_out, eta_in + eta_out);
      for (int c = 0; c < 3; ++c) {
        Es[c] = Ei[c] * R;
        Hs[c] = Hi[c] * R;
      }
    } else {  // tangentplane.h:51-62
      Dual<T, N> rp[3] = {nr[2] * kd[1] - nr[1] * kd[2], nr[0] * kd[2] - nr[2] * kd[0],
                          nr[1] * kd[0] - nr[0] * kd[1]};
      const Dual<T, N> inv = dconst<T, N>(1) / dsqrt(rp[0] * rp[0] + rp[1] * rp[1] + rp[2] * rp[2]);
      for (int c = 0; c < 3; ++c) rp[c] = rp[c] * inv;
      const CDual<T, N> f = Ei[0] * rp[0] + Ei[1] * rp[1] + Ei[2] * rp[2];
      CDual<T, N> Eperp[3], Epar[3], Hpar[3], Hperp[3];
      for (int c = 0; c < 3; ++c) {
        Eperp[c] = f * rp[c];
        Epar[c] = Ei[c] - Eperp[c];
      }
      const T iz = (T)(1.0 / P.z0);
      Hpar[0] = (Epar[2] * kd[1] - Epar[1] * kd[2]) * iz;
      Hpar[1] = (Epar[0] * kd[2] - Epar[2] * kd[0]) * iz;
      Hpar[2] = (Epar[1] * kd[0] - Epar[0] * kd[1]) * iz;
      for (int c = 0; c < 3; ++c) Hperp[c] = Hi[c] - Hpar[c];
      const Dual<T, N> xc = dabs(dotvalue);  // cos of the local angle acos|k.n|
      const Dual<T, N> s2 = dconst<T, N>(1) - xc * xc;
      const CDual<T, N> Rs = d_rs(xc, s2, eta_in, eta_out);
      const CDual<T, N> Rp = d_rp(xc, s2, eta_in, eta_out);
      for (int c = 0; c < 3; ++c) {
        Es[c] = Eperp[c] * Rs - Epar[c] * Rp;
        Hs[c] = Hpar[c] * Rp - Hperp[c] * Rs;
      }
    }
  }
  CDual<T, N> Et[3], Ht[3];
  for (int c = 0; c < 3; ++c) {
    Et[c] = Ei[c] + Es[c];
    Ht[c] = Hi[c] + Hs[c];
  }
  const CDual<T, N> M[3] = {Et[1] * nr[2] - Et[2] * nr[1], Et[2] * nr[0] - Et[0] * nr[2],
                            Et[0] * nr[1] - Et[1] * nr[0]};
  const CDual<T, N> J[3] = {Ht[2] * nr[1] - Ht[1] * nr[2], Ht[0] * nr[2] - Ht[2] * nr[0],
                            Ht[1] * nr[0] - Ht[0] * nr[1]};
  const CDual<T, N> ef = {Ar * (T)P.ef_re, Ar * (T)P.ef_im}, hf = {Ar * (T)P.hf_re, Ar * (T)P.hf_im};
  for (int c = 0; c < 3; ++c) {
    out[c] = J[c] * ef;
    out[3 + c] = M[c] * hf;
  }
}

}  // namespace wavepo
