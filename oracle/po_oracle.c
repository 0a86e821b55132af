/*
 * po_oracle.c -- FP64 CPU restatement of the WaveFiber3d physical-optics (PO)
 * far-field path.  TEST INFRASTRUCTURE ONLY: it is the checker for the CUDA
 * library, it is never linked into the product and never called by it.
 *
 * Every function cites the reference file:line it restates (paths are relative
 * to the WaveFiber3d project root).  Arithmetic is double precision; only the
 * branch decisions of the tangent-plane model are taken on the float-rounded
 * values, because the reference takes them in float (tangentplane.h:29-31,
 * :39-40) and the inputs are float32 arrays.
 *
 * Parity pins for this oracle (tests/test_oracle.py):
 *   - outputs of the reference's own CUDA build run on a GB300 on the same
 *     inputs (tests/golden/ref_*.bin, generated by tests/golden/gen_ref_fixtures.py),
 *   - a Mie-series check on spheres (oracle/mie.py),
 *   - the reference's own tree-vs-direct consistency check (README.md:44).
 */
#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

typedef double complex cdbl;

void po_oracle_intensity_sampled(int nth, int nph, int64_t m, const int64_t *dirs, const double *fields,
                                 double *intensity);

/* util/util.h:16-19 */
static const double ORC_C0 = 299792458.0;
static const double ORC_MU0 = 4e-7 * M_PI;
static const double ORC_EPS0 = 8.8541878e-12;
static double orc_z0(void) { return sqrt(ORC_MU0 / ORC_EPS0); }

double po_oracle_z0(void) { return orc_z0(); }

/* ------------------------------------------------------------------------ */
/* Fresnel coefficients: util/util.h:365-382                                 */
/* ------------------------------------------------------------------------ */
static cdbl cos_internal_angle(cdbl n, double theta) {
  /* util.h:366-368: sqrt(1 - sin(theta)/n*sin(theta)/n) on the principal branch */
  cdbl s = sin(theta) / n;
  return csqrt(1.0 - s * sin(theta) / n);
}

static cdbl fresnel_rs(double theta, cdbl n0, cdbl nt) {
  /* util.h:371-375 */
  cdbl p0 = n0 * cos_internal_angle(n0, theta);
  cdbl pt = nt * cos_internal_angle(nt / n0, theta);
  return (p0 - pt) / (p0 + pt);
}

static cdbl fresnel_rp(double theta, cdbl n0, cdbl nt) {
  /* util.h:378-382 (note: cos_internal_angle(nt, .) and not nt/n0) */
  cdbl q0 = cos_internal_angle(n0, theta) / n0;
  cdbl qt = cos_internal_angle(nt, theta) / nt;
  return (q0 - qt) / (q0 + qt);
}

void po_oracle_fresnel(double theta, double n0re, double n0im, double ntre, double ntim,
                       double *rs_out /*2*/, double *rp_out /*2*/) {
  cdbl n0 = n0re + I * n0im, nt = ntre + I * ntim;
  cdbl rs = fresnel_rs(theta, n0, nt), rp = fresnel_rp(theta, n0, nt);
  rs_out[0] = creal(rs); rs_out[1] = cimag(rs);
  rp_out[0] = creal(rp); rp_out[1] = cimag(rp);
}

/* ------------------------------------------------------------------------ */
/* Incident wave set-up: compareMie/sphere.cu:559-579 (= fibersim/treePO.cu:585-601) */
/* ------------------------------------------------------------------------ */
void po_oracle_incident(double theta_i, double phi_i, int mode_te, double *wavedir,
                        double *edir, double *hdir) {
  wavedir[0] = cos(theta_i) * cos(phi_i);
  wavedir[1] = cos(theta_i) * sin(phi_i);
  wavedir[2] = sin(theta_i);
  if (!mode_te) { /* mode 'M' */
    edir[0] = -sin(theta_i) * cos(phi_i);
    edir[1] = -sin(theta_i) * sin(phi_i);
    edir[2] = cos(theta_i);
    hdir[0] = sin(phi_i);
    hdir[1] = -cos(phi_i);
    hdir[2] = 0.0;
  } else { /* mode 'E' */
    edir[0] = -sin(phi_i);
    edir[1] = cos(phi_i);
    edir[2] = 0.0;
    hdir[0] = -sin(theta_i) * cos(phi_i);
    hdir[1] = -sin(theta_i) * sin(phi_i);
    hdir[2] = cos(theta_i);
  }
}

/* ------------------------------------------------------------------------ */
/* Tangent-plane currents: util/tangentplane.h:19-80                         */
/* ------------------------------------------------------------------------ */
static void cross_rc(const double *a, const cdbl *b, cdbl *r) {
  r[0] = a[1] * b[2] - b[1] * a[2];
  r[1] = a[2] * b[0] - b[2] * a[0];
  r[2] = b[1] * a[0] - a[1] * b[0];
}
static void cross_cr(const cdbl *a, const double *b, cdbl *r) {
  r[0] = a[1] * b[2] - b[1] * a[2];
  r[1] = a[2] * b[0] - b[2] * a[0];
  r[2] = b[1] * a[0] - a[1] * b[0];
}

/* One point: returns J (cur[0..2]) and M (cur[3..5]) before area/prefactor scaling.
 * eta_in = 1 (sphere.cu:581-582 passes comThr(1.0,0.0)), eta_out = eta. */
static void tangent_plane_point(const double *wavedir, const double *edir, const double *hdir,
                                cdbl eta_in, cdbl eta_out, double z0, double sigma, double k0,
                                int mode_te, const double *src, const double *nrm, cdbl *cur) {
  cdbl Ei[3] = {0, 0, 0}, Hi[3] = {0, 0, 0}, Es[3] = {0, 0, 0}, Hs[3] = {0, 0, 0};
  double dotvalue = wavedir[0] * nrm[0] + wavedir[1] * nrm[1] + wavedir[2] * nrm[2];
  float dot_f = (float)dotvalue; /* branch decisions as the float reference takes them */
  if (dot_f <= 0.0f) {                                             /* :31 */
    double dot = wavedir[0] * src[0] + wavedir[1] * src[1] + wavedir[2] * src[2];
    double tmp = src[2];
    double beam = exp(-0.5 * tmp * tmp / (sigma * sigma));           /* :33-34 */
    cdbl Ei0 = beam * cexp(-I * k0 * dot);                             /* :35 */
    cdbl Hi0 = Ei0 / z0;                                               /* :36 */
    for (int c = 0; c < 3; ++c) { Ei[c] = edir[c] * Ei0; Hi[c] = hdir[c] * Hi0; }
    if (fabsf(fabsf(dot_f) - 1.0f) < 1e-10f) {                         /* :39-40 */
      if (!mode_te) {
        cdbl Rs = (eta_in - eta_out) / (eta_in + eta_out);             /* :42 */
        for (int c = 0; c < 3; ++c) { Es[c] = Ei[c] * Rs; Hs[c] = Hi[c] * Rs; }
      } else {
        cdbl Rp = (eta_out - eta_in) / (eta_in + eta_out);             /* :46 */
        for (int c = 0; c < 3; ++c) { Es[c] = Ei[c] * Rp; Hs[c] = Hi[c] * Rp; }
      }
    } else {
      double rpn[3] = {wavedir[1] * nrm[2] - nrm[1] * wavedir[2],
                       wavedir[2] * nrm[0] - nrm[2] * wavedir[0],
                       nrm[1] * wavedir[0] - wavedir[1] * nrm[0]};     /* :51 */
      double nn = sqrt(rpn[0] * rpn[0] + rpn[1] * rpn[1] + rpn[2] * rpn[2]);
      for (int c = 0; c < 3; ++c) rpn[c] /= nn;
      cdbl factor = Ei[0] * rpn[0] + Ei[1] * rpn[1] + Ei[2] * rpn[2]; /* :52 */
      cdbl Ei_perp[3], Ei_par[3], Hi_par[3], Hi_perp[3], kx[3];
      for (int c = 0; c < 3; ++c) { Ei_perp[c] = rpn[c] * factor; Ei_par[c] = Ei[c] - Ei_perp[c]; }
      cross_rc(wavedir, Ei_par, kx);                                   /* :55 */
      for (int c = 0; c < 3; ++c) { Hi_par[c] = kx[c] * (1.0 / z0); Hi_perp[c] = Hi[c] - Hi_par[c]; }
      double localphi = acos(fabs(dotvalue));                          /* :58 */
      cdbl Rs = fresnel_rs(localphi, eta_in, eta_out);                 /* :59 */
      cdbl Rp = fresnel_rp(localphi, eta_in, eta_out);                 /* :60 */
      for (int c = 0; c < 3; ++c) {
        Es[c] = Ei_perp[c] * Rs - Ei_par[c] * Rp;                      /* :61 */
        Hs[c] = Hi_par[c] * Rp - Hi_perp[c] * Rs;                      /* :62 */
      }
    }
  } else {
    /* shadow (:64-67): Ei, Hi were never assigned (value-initialised zero) */
    for (int c = 0; c < 3; ++c) { Es[c] = -Ei[c]; Hs[c] = -Hi[c]; }
  }
  cdbl Et[3], Ht[3], J[3], M[3];
  for (int c = 0; c < 3; ++c) { Et[c] = Ei[c] + Es[c]; Ht[c] = Hi[c] + Hs[c]; } /* :68-69 */
  cross_cr(Et, nrm, M);                                               /* :70 */
  cross_rc(nrm, Ht, J);                                               /* :71 */
  for (int c = 0; c < 3; ++c) { cur[c] = J[c]; cur[3 + c] = M[c]; }   /* :72-77 */
}

/* Prefactors of compareMie/sphere.cu:491-494 (Dis = distance to the observer). */
static void prefactors(double k0, double dis, cdbl *ef, cdbl *hf) {
  double omega = k0 * ORC_C0;
  cdbl g = cexp(-I * k0 * dis) / dis;
  *ef = -I * omega * ORC_MU0 / (4.0 * M_PI) * g;
  *hf = -I * omega * ORC_EPS0 / (4.0 * M_PI) * g;
}

/* Illumination record shared by the oracle entry points. */
typedef struct {
  double lambda_m, theta_i, phi_i, eta_re, eta_im, sigma, dis;
  int mode_te; /* 0 = 'M' (TM), 1 = 'E' (TE) */
} po_oracle_illum;

/* Currents (tangentplane.h:84-92) then field_times_area (fields.h:123) and
 * multiply_current_factor (fields.h:147) when scale != 0.
 * out: n x 6 complex as 12 doubles per point [Jx,Jy,Jz,Mx,My,Mz] (re,im). */
void po_oracle_currents(int64_t n, const float *x, const float *y, const float *z,
                        const float *nx, const float *ny, const float *nz, const float *area,
                        const po_oracle_illum *il, int scale, double *out) {
  double wavedir[3], edir[3], hdir[3];
  po_oracle_incident(il->theta_i, il->phi_i, il->mode_te, wavedir, edir, hdir);
  double k0 = 2.0 * M_PI / il->lambda_m, z0 = orc_z0();
  cdbl ef = 1.0, hf = 1.0;
  if (scale) prefactors(k0, il->dis, &ef, &hf);
  cdbl eta = il->eta_re + I * il->eta_im;
#pragma omp parallel for schedule(static)
  for (int64_t p = 0; p < n; ++p) {
    double src[3] = {x[p], y[p], z[p]}, nrm[3] = {nx[p], ny[p], nz[p]};
    cdbl cur[6];
    tangent_plane_point(wavedir, edir, hdir, 1.0, eta, z0, il->sigma, k0, il->mode_te, src, nrm, cur);
    for (int c = 0; c < 6; ++c) {
      cdbl v = cur[c];
      if (scale) v *= (double)area[p] * (c < 3 ? ef : hf);
      out[p * 12 + 2 * c] = creal(v);
      out[p * 12 + 2 * c + 1] = cimag(v);
    }
  }
}

/* Direction grid: compareMie/sphere.cu:370-384 (theta = elevation). */
static void direction(int it, int ip, int nth, int nph, double *s) {
  double th = -M_PI / 2 + 1e-10 + M_PI / nth * it;
  double ph = 2 * M_PI / nph * ip;
  s[0] = cos(th) * cos(ph);
  s[1] = cos(th) * sin(ph);
  s[2] = sin(th);
}

void po_oracle_direction(int it, int ip, int nth, int nph, double *s) { direction(it, ip, nth, nph, s); }

/* Far field of a set of scaled currents about centre c, on an nth x nph grid:
 * fields.h:2-39 (phase exp(+i k s.(x-c))) summed as by the per-node
 * thrust::reduce of sphere.cu:635-643.  out: [dir][6] complex (12 doubles). */
void po_oracle_far_field(int64_t n, const float *x, const float *y, const float *z,
                         const double *cur, double k0, const double *c, int nth, int nph,
                         double *out) {
  int64_t nd = (int64_t)nth * nph;
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t d = 0; d < nd; ++d) {
    double s[3];
    direction((int)(d / nph), (int)(d % nph), nth, nph, s);
    cdbl acc[6] = {0, 0, 0, 0, 0, 0};
    for (int64_t p = 0; p < n; ++p) {
      double dot = ((double)x[p] - c[0]) * s[0] + ((double)y[p] - c[1]) * s[1] + ((double)z[p] - c[2]) * s[2];
      double ph = k0 * dot;
      cdbl g = cos(ph) + I * sin(ph);
      const double *q = cur + p * 12;
      for (int k = 0; k < 6; ++k) acc[k] += (q[2 * k] + I * q[2 * k + 1]) * g;
    }
    for (int k = 0; k < 6; ++k) {
      out[d * 12 + 2 * k] = creal(acc[k]);
      out[d * 12 + 2 * k + 1] = cimag(acc[k]);
    }
  }
}

/* Projection and intensity: fields.h:172-204.  fields: [dir][6] complex. */
void po_oracle_intensity(int nth, int nph, const double *fields, double *intensity) {
  double z0 = orc_z0();
  int64_t nd = (int64_t)nth * nph;
  for (int64_t d = 0; d < nd; ++d) {
    double s[3];
    direction((int)(d / nph), (int)(d % nph), nth, nph, s);
    const double *f = fields + d * 12;
    cdbl E[3], H[3];
    for (int c = 0; c < 3; ++c) { E[c] = f[2 * c] + I * f[2 * c + 1]; H[c] = f[6 + 2 * c] + I * f[6 + 2 * c + 1]; }
    cdbl de = E[0] * s[0] + E[1] * s[1] + E[2] * s[2];
    for (int c = 0; c < 3; ++c) E[c] -= de * s[c];
    cdbl dh = H[0] * s[0] + H[1] * s[1] + H[2] * s[2];
    for (int c = 0; c < 3; ++c) H[c] -= dh * s[c];
    cdbl ex = E[0] - (H[2] * s[1] - H[1] * s[2]) * z0;     /* :290 */
    cdbl ey = E[1] - (-(H[2] * s[0] - H[0] * s[2])) * z0;  /* :291 */
    cdbl ez = E[2] - (H[1] * s[0] - H[0] * s[1]) * z0;     /* :292 */
    intensity[d] = creal(ex * conj(ex)) + creal(ey * conj(ey)) + creal(ez * conj(ez));
  }
}

/* Whole depth-0 solve for one (lambda, incidence, polarisation): currents,
 * area and prefactor scaling, far-field sum about `center`, intensity.
 * This is the plain FP64 direct sum that the engine is checked against. */
void po_oracle_solve_direct(int64_t n, const float *x, const float *y, const float *z,
                            const float *nx, const float *ny, const float *nz, const float *area,
                            const po_oracle_illum *il, const double *center, int nth, int nph,
                            double *intensity) {
  double *cur = (double *)malloc(sizeof(double) * 12 * (size_t)(n > 0 ? n : 1));
  double *fld = (double *)malloc(sizeof(double) * 12 * (size_t)nth * nph);
  po_oracle_currents(n, x, y, z, nx, ny, nz, area, il, 1, cur);
  po_oracle_far_field(n, x, y, z, cur, 2.0 * M_PI / il->lambda_m, center, nth, nph, fld);
  po_oracle_intensity(nth, nph, fld, intensity);
  free(cur);
  free(fld);
}

/* The depth-0 solve with FP64 samples (positions, normals, areas as double):
 * the same model as po_oracle_solve_direct, for central finite differences
 * whose steps a float32 coordinate could not resolve. */
void po_oracle_solve_direct_d(int64_t n, const double *x, const double *y, const double *z, const double *nx,
                              const double *ny, const double *nz, const double *area, const po_oracle_illum *il,
                              const double *center, int nth, int nph, double *intensity) {
  double wavedir[3], edir[3], hdir[3];
  po_oracle_incident(il->theta_i, il->phi_i, il->mode_te, wavedir, edir, hdir);
  double k0 = 2.0 * M_PI / il->lambda_m, z0 = orc_z0();
  cdbl ef, hf;
  prefactors(k0, il->dis, &ef, &hf);
  cdbl eta = il->eta_re + I * il->eta_im;
  cdbl *cur = (cdbl *)malloc(sizeof(cdbl) * 6 * (size_t)(n > 0 ? n : 1));
  double *fld = (double *)malloc(sizeof(double) * 12 * (size_t)nth * nph);
#pragma omp parallel for schedule(static)
  for (int64_t p = 0; p < n; ++p) {
    double src[3] = {x[p], y[p], z[p]}, nrm[3] = {nx[p], ny[p], nz[p]};
    tangent_plane_point(wavedir, edir, hdir, 1.0, eta, z0, il->sigma, k0, il->mode_te, src, nrm, cur + 6 * p);
    for (int c = 0; c < 6; ++c) cur[6 * p + c] *= area[p] * (c < 3 ? ef : hf);
  }
  int64_t nd = (int64_t)nth * nph;
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t d = 0; d < nd; ++d) {
    double s[3];
    direction((int)(d / nph), (int)(d % nph), nth, nph, s);
    cdbl acc[6] = {0, 0, 0, 0, 0, 0};
    for (int64_t p = 0; p < n; ++p) {
      double ph = k0 * ((x[p] - center[0]) * s[0] + (y[p] - center[1]) * s[1] + (z[p] - center[2]) * s[2]);
      cdbl g = cos(ph) + I * sin(ph);
      for (int k = 0; k < 6; ++k) acc[k] += cur[6 * p + k] * g;
    }
    for (int k = 0; k < 6; ++k) {
      fld[d * 12 + 2 * k] = creal(acc[k]);
      fld[d * 12 + 2 * k + 1] = cimag(acc[k]);
    }
  }
  po_oracle_intensity(nth, nph, fld, intensity);
  free(cur);
  free(fld);
}

/* po_oracle_solve_direct_d on the listed flat direction indices only
 * (intensity out: [m]). */
/* FP64 far field of (x..area) float64 samples at the flat direction indices
 * dirs (the sum of po_oracle_solve_direct_d about the origin, without the
 * intensity): fields [m][6] complex (12 doubles per direction).  per_point
 * != 0 keeps every point's own field instead of the sum: fields [n][m][6]. */
void po_oracle_fields_sampled_d(int64_t n, const double *x, const double *y, const double *z, const double *nx,
                                const double *ny, const double *nz, const double *area, const po_oracle_illum *il,
                                int nth, int nph, int64_t m, const int64_t *dirs, int per_point, double *fld) {
  double wavedir[3], edir[3], hdir[3];
  po_oracle_incident(il->theta_i, il->phi_i, il->mode_te, wavedir, edir, hdir);
  double k0 = 2.0 * M_PI / il->lambda_m, z0 = orc_z0();
  cdbl ef, hf;
  prefactors(k0, il->dis, &ef, &hf);
  cdbl eta = il->eta_re + I * il->eta_im;
  cdbl *cur = (cdbl *)malloc(sizeof(cdbl) * 6 * (size_t)(n > 0 ? n : 1));
#pragma omp parallel for schedule(static)
  for (int64_t p = 0; p < n; ++p) {
    double src[3] = {x[p], y[p], z[p]}, nrm[3] = {nx[p], ny[p], nz[p]};
    tangent_plane_point(wavedir, edir, hdir, 1.0, eta, z0, il->sigma, k0, il->mode_te, src, nrm, cur + 6 * p);
    for (int c = 0; c < 6; ++c) cur[6 * p + c] *= area[p] * (c < 3 ? ef : hf);
  }
  if (per_point) {
#pragma omp parallel for schedule(static)
    for (int64_t q = 0; q < n * m; ++q) {
      int64_t p = q / m, j = q % m;
      double s[3];
      direction((int)(dirs[j] / nph), (int)(dirs[j] % nph), nth, nph, s);
      double ph = k0 * (x[p] * s[0] + y[p] * s[1] + z[p] * s[2]);
      cdbl g = cos(ph) + I * sin(ph);
      for (int k = 0; k < 6; ++k) {
        cdbl v = cur[6 * p + k] * g;
        fld[q * 12 + 2 * k] = creal(v);
        fld[q * 12 + 2 * k + 1] = cimag(v);
      }
    }
  } else {
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t j = 0; j < m; ++j) {
      double s[3];
      direction((int)(dirs[j] / nph), (int)(dirs[j] % nph), nth, nph, s);
      cdbl acc[6] = {0, 0, 0, 0, 0, 0};
      for (int64_t p = 0; p < n; ++p) {
        double ph = k0 * (x[p] * s[0] + y[p] * s[1] + z[p] * s[2]);
        cdbl g = cos(ph) + I * sin(ph);
        for (int k = 0; k < 6; ++k) acc[k] += cur[6 * p + k] * g;
      }
      for (int k = 0; k < 6; ++k) {
        fld[j * 12 + 2 * k] = creal(acc[k]);
        fld[j * 12 + 2 * k + 1] = cimag(acc[k]);
      }
    }
  }
  free(cur);
}

/* Intensity of the FP64 samples at the flat direction indices dirs. */
void po_oracle_solve_sampled_d(int64_t n, const double *x, const double *y, const double *z, const double *nx,
                               const double *ny, const double *nz, const double *area, const po_oracle_illum *il,
                               int nth, int nph, int64_t m, const int64_t *dirs, double *intensity) {
  double *fld = (double *)malloc(sizeof(double) * 12 * (size_t)(m > 0 ? m : 1));
  po_oracle_fields_sampled_d(n, x, y, z, nx, ny, nz, area, il, nth, nph, m, dirs, 0, fld);
  po_oracle_intensity_sampled(nth, nph, m, dirs, fld, intensity);
  free(fld);
}

/* Sampled variant for timing and for large cases: only the listed flat
 * direction indices of the nth x nph grid are evaluated (fields out: [m][6]). */
void po_oracle_far_field_sampled(int64_t n, const float *x, const float *y, const float *z,
                                 const double *cur, double k0, const double *c, int nth, int nph,
                                 int64_t m, const int64_t *dirs, double *out) {
#pragma omp parallel for schedule(dynamic, 4)
  for (int64_t j = 0; j < m; ++j) {
    int64_t d = dirs[j];
    double s[3];
    direction((int)(d / nph), (int)(d % nph), nth, nph, s);
    cdbl acc[6] = {0, 0, 0, 0, 0, 0};
    for (int64_t p = 0; p < n; ++p) {
      double dot = ((double)x[p] - c[0]) * s[0] + ((double)y[p] - c[1]) * s[1] + ((double)z[p] - c[2]) * s[2];
      double ph = k0 * dot;
      cdbl g = cos(ph) + I * sin(ph);
      const double *q = cur + p * 12;
      for (int k = 0; k < 6; ++k) acc[k] += (q[2 * k] + I * q[2 * k + 1]) * g;
    }
    for (int k = 0; k < 6; ++k) {
      out[j * 12 + 2 * k] = creal(acc[k]);
      out[j * 12 + 2 * k + 1] = cimag(acc[k]);
    }
  }
}

/* Intensity of a subset of directions (fields [m][6] at flat indices dirs). */
void po_oracle_intensity_sampled(int nth, int nph, int64_t m, const int64_t *dirs,
                                 const double *fields, double *intensity) {
  double z0 = orc_z0();
  for (int64_t j = 0; j < m; ++j) {
    int64_t d = dirs[j];
    double s[3];
    direction((int)(d / nph), (int)(d % nph), nth, nph, s);
    const double *f = fields + j * 12;
    cdbl E[3], H[3];
    for (int c = 0; c < 3; ++c) { E[c] = f[2 * c] + I * f[2 * c + 1]; H[c] = f[6 + 2 * c] + I * f[6 + 2 * c + 1]; }
    cdbl de = E[0] * s[0] + E[1] * s[1] + E[2] * s[2];
    for (int c = 0; c < 3; ++c) E[c] -= de * s[c];
    cdbl dh = H[0] * s[0] + H[1] * s[1] + H[2] * s[2];
    for (int c = 0; c < 3; ++c) H[c] -= dh * s[c];
    cdbl ex = E[0] - (H[2] * s[1] - H[1] * s[2]) * z0;
    cdbl ey = E[1] + (H[2] * s[0] - H[0] * s[2]) * z0;
    cdbl ez = E[2] - (H[1] * s[0] - H[0] * s[1]) * z0;
    intensity[j] = creal(ex * conj(ex)) + creal(ey * conj(ey)) + creal(ez * conj(ez));
  }
}

/* The transverse field E' = E_perp - Z0 s x H_perp of fields.h:172-204 (the
 * intensity is |E'|^2) at the flat direction indices dirs: out [m][3] complex. */
void po_oracle_project_sampled(int nth, int nph, int64_t m, const int64_t *dirs, const double *fields,
                               double *out) {
  double z0 = orc_z0();
  for (int64_t j = 0; j < m; ++j) {
    int64_t d = dirs[j];
    double s[3];
    direction((int)(d / nph), (int)(d % nph), nth, nph, s);
    const double *f = fields + j * 12;
    cdbl E[3], H[3];
    for (int c = 0; c < 3; ++c) { E[c] = f[2 * c] + I * f[2 * c + 1]; H[c] = f[6 + 2 * c] + I * f[6 + 2 * c + 1]; }
    cdbl de = E[0] * s[0] + E[1] * s[1] + E[2] * s[2];
    for (int c = 0; c < 3; ++c) E[c] -= de * s[c];
    cdbl dh = H[0] * s[0] + H[1] * s[1] + H[2] * s[2];
    for (int c = 0; c < 3; ++c) H[c] -= dh * s[c];
    cdbl e3[3] = {E[0] - (H[2] * s[1] - H[1] * s[2]) * z0, E[1] + (H[2] * s[0] - H[0] * s[2]) * z0,
                  E[2] - (H[1] * s[0] - H[0] * s[1]) * z0};
    for (int c = 0; c < 3; ++c) {
      out[j * 6 + 2 * c] = creal(e3[c]);
      out[j * 6 + 2 * c + 1] = cimag(e3[c]);
    }
  }
}

int po_oracle_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
