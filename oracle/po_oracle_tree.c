/*
 * po_oracle_tree.c -- FP64 CPU restatement of the reference's hierarchical
 * (octree) PO solve.  TEST INFRASTRUCTURE ONLY: the checker for the CUDA
 * library's octree build, FFT angular interpolation and level aggregation.
 *
 *   octree build ............ util/tree.h:289-715 (recursive stable 8-way split)
 *   active node lists ....... compareMie/sphere.cu:255-307
 *   leaf far fields ......... compareMie/sphere.cu:603-658, util/fields.h:2-50
 *   angular interpolation ... util/interpolation.h:2-93 (FFTs restated as DFTs)
 *   translation table ....... compareMie/sphere.cu:499-539, util/fields.h:92-103
 *   child sum ............... util/fields.h:153-169, compareMie/sphere.cu:661-884
 *   intensity ............... util/fields.h:172-204
 *
 * Geometry decisions (octant membership, box centres) are taken in float
 * exactly as the reference does; everything else is double precision.
 */
#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef double complex cdbl;

typedef struct {
  double lambda_m, theta_i, phi_i, eta_re, eta_im, sigma, dis;
  int mode_te;
} po_oracle_illum;

void po_oracle_currents(int64_t n, const float *x, const float *y, const float *z,
                        const float *nx, const float *ny, const float *nz, const float *area,
                        const po_oracle_illum *il, int scale, double *out);
void po_oracle_direction(int it, int ip, int nth, int nph, double *s);
void po_oracle_far_field(int64_t n, const float *x, const float *y, const float *z,
                         const double *cur, double k0, const double *c, int nth, int nph,
                         double *out);
void po_oracle_intensity(int nth, int nph, const double *fields, double *intensity);

/* ------------------------------------------------------------------------ */
/* Octree: util/tree.h                                                       */
/* ------------------------------------------------------------------------ */
typedef struct {
  float mn[3], mx[3];
  int begin, end;
} onode;

static int64_t level_offset(int l) { /* (8^l - 1) / 7, sphere.cu:260 */
  int64_t o = 0, p = 1;
  for (int i = 0; i < l; ++i) { o += p; p *= 8; }
  return o;
}

/* Octant predicate order of tree.h:379-414 / :522-623. */
static int octant_of(const float *p, const float *c) {
  int lo_x = p[0] < c[0], lo_y = p[1] < c[1], lo_z = p[2] < c[2];
  if (lo_x && !lo_y && !lo_z) return 0;
  if (!lo_x && !lo_y && !lo_z) return 1;
  if (lo_x && lo_y && !lo_z) return 2;
  if (!lo_x && lo_y && !lo_z) return 3;
  if (lo_x && !lo_y && lo_z) return 4;
  if (!lo_x && !lo_y && lo_z) return 5;
  if (lo_x && lo_y && lo_z) return 6;
  return 7;
}

/* Child bounding boxes of tree.h:672-687. */
static void child_box(const onode *par, const float *c, int o, onode *ch) {
  const float *mn = par->mn, *mx = par->mx;
  float bx0 = (o & 1) ? c[0] : mn[0], bx1 = (o & 1) ? mx[0] : c[0];
  float by0 = (o & 2) ? mn[1] : c[1], by1 = (o & 2) ? c[1] : mx[1];
  float bz0 = (o & 4) ? mn[2] : c[2], bz1 = (o & 4) ? c[2] : mx[2];
  ch->mn[0] = bx0; ch->mn[1] = by0; ch->mn[2] = bz0;
  ch->mx[0] = bx1; ch->mx[1] = by1; ch->mx[2] = bz1;
}

static void box_center(const onode *nd, float *c) { /* tree.h:116-120 */
  for (int a = 0; a < 3; ++a) c[a] = 0.5f * (nd->mn[a] + nd->mx[a]);
}

static void build_rec(onode *nodes, int level, int64_t id, int depth, float *pts /*n x 3*/,
                      int *perm, float *tmp_pts, int *tmp_perm) {
  onode *nd = &nodes[level_offset(level) + id];
  if (level >= depth) return; /* tree.h:331 */
  float c[3];
  box_center(nd, c);
  int cnt[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int i = nd->begin; i < nd->end; ++i) cnt[octant_of(pts + 3 * i, c)]++;
  int off[8], run = nd->begin;
  for (int o = 0; o < 8; ++o) { off[o] = run; run += cnt[o]; }
  int pos[8];
  memcpy(pos, off, sizeof(pos));
  for (int i = nd->begin; i < nd->end; ++i) { /* stable scatter, tree.h:511-624 */
    int o = octant_of(pts + 3 * i, c);
    int d = pos[o]++;
    memcpy(tmp_pts + 3 * d, pts + 3 * i, 3 * sizeof(float));
    tmp_perm[d] = perm[i];
  }
  memcpy(pts + 3 * nd->begin, tmp_pts + 3 * nd->begin, 3 * sizeof(float) * (nd->end - nd->begin));
  memcpy(perm + nd->begin, tmp_perm + nd->begin, sizeof(int) * (nd->end - nd->begin));
  for (int o = 0; o < 8; ++o) {
    onode *ch = &nodes[level_offset(level + 1) + 8 * id + o];
    child_box(nd, c, o, ch);
    ch->begin = off[o];
    ch->end = off[o] + cnt[o];
  }
  for (int o = 0; o < 8; ++o) build_rec(nodes, level + 1, 8 * id + o, depth, pts, perm, tmp_pts, tmp_perm);
}

/* Builds the full heap of (8^(d+1)-1)/7 nodes.  perm[i] = input index of the
 * point at sorted position i.  node_range[2*h] / [2*h+1] = begin / end of heap
 * node h; node_box[6*h..] = min xyz, max xyz. */
int po_oracle_octree(int n, const float *x, const float *y, const float *z, const float *box_min,
                     const float *box_max, int depth, int *perm, int *node_range, float *node_box) {
  if (depth < 0 || depth > 7) return 1;
  int64_t nn = level_offset(depth + 1);
  onode *nodes = (onode *)calloc((size_t)nn, sizeof(onode));
  float *pts = (float *)malloc(sizeof(float) * 3 * (size_t)(n > 0 ? n : 1));
  float *tpts = (float *)malloc(sizeof(float) * 3 * (size_t)(n > 0 ? n : 1));
  int *tperm = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
  for (int i = 0; i < n; ++i) { pts[3 * i] = x[i]; pts[3 * i + 1] = y[i]; pts[3 * i + 2] = z[i]; perm[i] = i; }
  for (int a = 0; a < 3; ++a) { nodes[0].mn[a] = box_min[a]; nodes[0].mx[a] = box_max[a]; }
  nodes[0].begin = 0;
  nodes[0].end = n;
  build_rec(nodes, 0, 0, depth, pts, perm, tpts, tperm);
  for (int64_t h = 0; h < nn; ++h) {
    if (node_range) { node_range[2 * h] = nodes[h].begin; node_range[2 * h + 1] = nodes[h].end; }
    if (node_box)
      for (int a = 0; a < 3; ++a) { node_box[6 * h + a] = nodes[h].mn[a]; node_box[6 * h + 3 + a] = nodes[h].mx[a]; }
  }
  free(nodes); free(pts); free(tpts); free(tperm);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Angular interpolation: util/interpolation.h:2-93                          */
/* ------------------------------------------------------------------------ */
static void dft(const cdbl *in, cdbl *out, int n, int sign) {
  for (int k = 0; k < n; ++k) {
    cdbl acc = 0;
    for (int j = 0; j < n; ++j) {
      long m = ((long)j * k) % n;
      double a = sign * 2.0 * M_PI * (double)m / n;
      acc += in[j] * (cos(a) + I * sin(a));
    }
    out[k] = acc;
  }
}

/* Zero pad of interpolation.h:20-31 plus the Nyquist split of setvalue
 * (interpolation.h:2-9, :34-37) when `split` is set. */
static void pad_spectrum(const cdbl *X, int n, cdbl *Y, int nf, int split) {
  for (int k = 0; k < nf; ++k) Y[k] = 0;
  int nyq = (int)ceil((n + 1) / 2.0);
  for (int k = 0; k < nyq; ++k) Y[k] = X[k];
  for (int k = nyq; k < n; ++k) Y[k + nf - n] = X[k];
  if ((n % 2 == 0) && split) {
    Y[nyq - 1] = Y[nyq - 1] / 2.0;
    Y[nyq + nf - n - 1] = Y[nyq - 1];
  }
}

/* interpFFT (interpolation.h:11-80): trigonometric upsampling of a
 * th_c x ph_c pattern to th_p x ph_p, phi first, then theta.  With
 * `nyquist_quirk` set, the theta-pass Nyquist split is applied only to the
 * columns the reference's setvalue launch reaches (interpolation.h:66 sizes
 * that launch from the row count th_c, so columns j >= 256*(th_c/256+1) of an
 * even th_c keep the unsplit Nyquist bin). in/out are [theta][phi] complex. */
int po_oracle_interp(int th_c, int ph_c, int th_p, int ph_p, int nyquist_quirk,
                     const double *in /*re,im pairs*/, double *out) {
  if (th_p < th_c || ph_p < ph_c) return 1; /* the reference cannot downsample */
  int nmax = th_p > ph_p ? th_p : ph_p;
  cdbl *mid = (cdbl *)calloc((size_t)th_c * ph_p, sizeof(cdbl));
  cdbl *a = (cdbl *)malloc(sizeof(cdbl) * nmax), *b = (cdbl *)malloc(sizeof(cdbl) * nmax);
  cdbl *c = (cdbl *)malloc(sizeof(cdbl) * nmax);
  for (int t = 0; t < th_c; ++t) {
    for (int j = 0; j < ph_c; ++j) a[j] = in[2 * ((size_t)t * ph_c + j)] + I * in[2 * ((size_t)t * ph_c + j) + 1];
    dft(a, b, ph_c, -1);
    pad_spectrum(b, ph_c, c, ph_p, 1); /* every row is reached (:35) */
    dft(c, a, ph_p, +1);
    for (int j = 0; j < ph_p; ++j) mid[(size_t)t * ph_p + j] = a[j] / (double)ph_c; /* :45 */
  }
  int reach = 256 * (th_c / 256 + 1);
  for (int j = 0; j < ph_p; ++j) {
    for (int t = 0; t < th_c; ++t) a[t] = mid[(size_t)t * ph_p + j];
    dft(a, b, th_c, -1);
    pad_spectrum(b, th_c, c, th_p, nyquist_quirk ? (j < reach) : 1);
    dft(c, a, th_p, +1);
    for (int t = 0; t < th_p; ++t) {
      cdbl v = a[t] / (double)th_c; /* :77 */
      out[2 * ((size_t)t * ph_p + j)] = creal(v);
      out[2 * ((size_t)t * ph_p + j) + 1] = cimag(v);
    }
  }
  free(mid); free(a); free(b); free(c);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Hierarchical solve: compareMie/sphere.cu:212-936                          */
/* ------------------------------------------------------------------------ */
/* nth[l], nph[l] for l = 0..depth (level 0 = output grid).  intensity out:
 * nth[0] x nph[0].  Returns nonzero on an unsupported configuration. */
int po_oracle_solve_tree(int n, const float *x, const float *y, const float *z, const float *nx,
                         const float *ny, const float *nz, const float *area,
                         const po_oracle_illum *il, const float *box_min, const float *box_max,
                         int depth, const int *nth, const int *nph, int nyquist_quirk,
                         double *intensity) {
  for (int l = 0; l < depth; ++l)
    if (nth[l] < nth[l + 1] || nph[l] < nph[l + 1]) return 1;
  int64_t nn = level_offset(depth + 1);
  int *perm = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
  int *rng = (int *)malloc(sizeof(int) * 2 * (size_t)nn);
  float *bx = (float *)malloc(sizeof(float) * 6 * (size_t)nn);
  if (po_oracle_octree(n, x, y, z, box_min, box_max, depth, perm, rng, bx)) return 2;
  /* reordered geometry (tree.h moves points, normals and areas together) */
  float *sx = malloc(sizeof(float) * (size_t)(n > 0 ? n : 1) * 7);
  float *sy = sx + n, *sz = sy + n, *snx = sz + n, *sny = snx + n, *snz = sny + n, *sa = snz + n;
  for (int i = 0; i < n; ++i) {
    int p = perm[i];
    sx[i] = x[p]; sy[i] = y[p]; sz[i] = z[p]; snx[i] = nx[p]; sny[i] = ny[p]; snz[i] = nz[p]; sa[i] = area[p];
  }
  double *cur = (double *)malloc(sizeof(double) * 12 * (size_t)(n > 0 ? n : 1));
  po_oracle_currents(n, sx, sy, sz, snx, sny, snz, sa, il, 1, cur);
  double k0 = 2.0 * M_PI / il->lambda_m;

  /* per level: active (non-empty) heap nodes in heap order (sphere.cu:255-307) */
  int64_t **act = (int64_t **)calloc(depth + 1, sizeof(int64_t *));
  int64_t *nact = (int64_t *)calloc(depth + 1, sizeof(int64_t));
  for (int l = 0; l <= depth; ++l) {
    int64_t o = level_offset(l), cnt = level_offset(l + 1) - o;
    act[l] = (int64_t *)malloc(sizeof(int64_t) * (size_t)cnt);
    for (int64_t h = o; h < o + cnt; ++h)
      if (rng[2 * h] < rng[2 * h + 1] || (l == 0)) act[l][nact[l]++] = h;
  }

  /* leaf far fields (or the depth-0 direct sum) */
  int64_t dl = (int64_t)nth[depth] * nph[depth];
  double *cur_lvl = (double *)calloc((size_t)(nact[depth] * dl * 12 + 12), sizeof(double));
  for (int64_t a = 0; a < nact[depth]; ++a) {
    int64_t h = act[depth][a];
    float cf[3];
    onode tmp;
    memcpy(tmp.mn, bx + 6 * h, 3 * sizeof(float));
    memcpy(tmp.mx, bx + 6 * h + 3, 3 * sizeof(float));
    box_center(&tmp, cf);
    double c[3] = {cf[0], cf[1], cf[2]};
    int b = rng[2 * h], e = rng[2 * h + 1];
    po_oracle_far_field(e - b, sx + b, sy + b, sz + b, cur + 12 * (size_t)b, k0, c, nth[depth], nph[depth],
                        cur_lvl + a * dl * 12);
  }

  for (int l = depth - 1; l >= 0; --l) {
    int thp = nth[l], php = nph[l], thc = nth[l + 1], phc = nph[l + 1];
    int64_t dp = (int64_t)thp * php, dc = (int64_t)thc * phc;
    double *par = (double *)calloc((size_t)(nact[l] * dp * 12), sizeof(double));
    /* translation factors from the first node of the level (sphere.cu:499-539) */
    int64_t h0 = level_offset(l), hc0 = level_offset(l + 1);
    float pc[3];
    onode t0;
    memcpy(t0.mn, bx + 6 * h0, 12);
    memcpy(t0.mx, bx + 6 * h0 + 3, 12);
    box_center(&t0, pc);
    double diff[8][3];
    for (int o = 0; o < 8; ++o) {
      onode tc;
      float cc[3];
      memcpy(tc.mn, bx + 6 * (hc0 + o), 12);
      memcpy(tc.mx, bx + 6 * (hc0 + o) + 3, 12);
      box_center(&tc, cc);
      for (int a = 0; a < 3; ++a) diff[o][a] = (double)cc[a] - (double)pc[a];
    }
    double *cin = (double *)malloc(sizeof(double) * 2 * (size_t)dc);
    double *cout = (double *)malloc(sizeof(double) * 2 * (size_t)dp);
    for (int64_t a = 0; a < nact[l]; ++a) {
      int64_t h = act[l][a];
      int64_t id = h - level_offset(l);
      for (int o = 0; o < 8; ++o) {
        int64_t hc = level_offset(l + 1) + 8 * id + o;
        int64_t ci = -1;
        for (int64_t s = 0; s < nact[l + 1]; ++s)
          if (act[l + 1][s] == hc) { ci = s; break; }
        if (ci < 0) continue;
        for (int comp = 0; comp < 6; ++comp) {
          for (int64_t d = 0; d < dc; ++d) {
            cin[2 * d] = cur_lvl[(ci * dc + d) * 12 + 2 * comp];
            cin[2 * d + 1] = cur_lvl[(ci * dc + d) * 12 + 2 * comp + 1];
          }
          po_oracle_interp(thc, phc, thp, php, nyquist_quirk, cin, cout);
          for (int64_t d = 0; d < dp; ++d) {
            double s[3];
            po_oracle_direction((int)(d / php), (int)(d % php), thp, php, s);
            double ph = k0 * (diff[o][0] * s[0] + diff[o][1] * s[1] + diff[o][2] * s[2]);
            cdbl f = cos(ph) + I * sin(ph);
            cdbl v = (cout[2 * d] + I * cout[2 * d + 1]) * f;
            par[(a * dp + d) * 12 + 2 * comp] += creal(v);
            par[(a * dp + d) * 12 + 2 * comp + 1] += cimag(v);
          }
        }
      }
    }
    free(cin); free(cout); free(cur_lvl);
    cur_lvl = par;
  }
  po_oracle_intensity(nth[0], nph[0], cur_lvl, intensity);
  for (int l = 0; l <= depth; ++l) free(act[l]);
  free(act); free(nact); free(cur_lvl); free(cur); free(sx); free(perm); free(rng); free(bx);
  return 0;
}
