/*
 * po_oracle_geometry.c -- CPU restatement of the fiber height-field sampler.
 * TEST INFRASTRUCTURE ONLY: the checker for po_height_field_points, never
 * linked into the product.
 *
 * Follows util/geometry.h:76-179 (set_sourcepoint over the ring segment
 * [startindex, endindex]; the full-ring form util/geometry.h:3-75 is the
 * segment 0 .. numel-1 with the same output order).  The reference computes in
 * float, so this restatement does too, operation by operation in the
 * reference's order (util/util.h:300-345 for the vector helpers); it is built
 * with -ffp-contract=off so that no multiply-add is fused on any host.
 * Returns 0, or 1 when a vertex lies at the origin (geometry.h:110-114 prints
 * an error and exits there).
 *
 * Also restates util/fields.h:206-234 (average_cpu), the box average of a
 * fine pattern onto a coarse grid, in float and in the reference's order.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>

typedef struct {
  float x, y, z;
} v3;

static v3 sub(v3 a, v3 b) { v3 r = {a.x - b.x, a.y - b.y, a.z - b.z}; return r; }
static v3 add(v3 a, v3 b) { v3 r = {a.x + b.x, a.y + b.y, a.z + b.z}; return r; }
/* util/util.h:339-345 */
static v3 cross(v3 a, v3 b) {
  v3 r = {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, b.y * a.x - a.y * b.x};
  return r;
}
/* util/util.h:306-309 */
static float norm(v3 a) { return sqrtf(a.x * a.x + a.y * a.y + a.z * a.z); }

int po_oracle_height_field(const float *height, int numel, int numelvert, float period, float unitz, int start,
                           int end, float *px, float *py, float *pz, float *nx, float *ny, float *nz, float *area) {
  const float *hx = height, *hy = height + (int64_t)numel * numelvert;
  int bad = 0;
  for (int i = 0; i < numelvert; ++i) {
    /* geometry.h:89-90: float product, then the difference taken in double
       (exact for these operands) and rounded to float once */
    float z = (float)((double)((float)i * unitz) - period * 0.5);
    float zn = (float)((double)((float)(i + 1) * unitz) - period * 0.5);
    int zi = i < numelvert - 1 ? i + 1 : i;
    for (int j = start; j <= end; ++j) {
      int pj = j < numel - 1 ? j + 1 : 0;
      v3 p1 = {hx[(int64_t)j * numelvert + i], hy[(int64_t)j * numelvert + i], z};
      v3 p2 = {hx[(int64_t)pj * numelvert + i], hy[(int64_t)pj * numelvert + i], z};
      v3 p3 = {hx[(int64_t)j * numelvert + zi], hy[(int64_t)j * numelvert + zi], zn};
      v3 p4 = {hx[(int64_t)pj * numelvert + zi], hy[(int64_t)pj * numelvert + zi], zn};
      if ((p1.x == 0 && p1.y == 0) || (p2.x == 0 && p2.y == 0) || (p3.x == 0 && p3.y == 0) ||
          (p4.x == 0 && p4.y == 0))
        bad = 1;
      int64_t o = (int64_t)i * (end - start + 1) + (j - start);
      /* float sums, then /4.0 in double (exact) */
      px[o] = (float)((double)(p1.x + p2.x + p3.x + p4.x) / 4.0);
      py[o] = (float)((double)(p1.y + p2.y + p3.y + p4.y) / 4.0);
      pz[o] = (float)((double)(p1.z + p2.z + p3.z + p4.z) / 4.0);
      v3 a1 = cross(sub(p2, p1), sub(p3, p1));
      v3 a2 = cross(sub(p4, p2), sub(p3, p2));
      area[o] = (float)(0.5 * (double)(norm(a1) + norm(a2)));
      v3 s = add(a1, a2);
      float ns = norm(s); /* util/util.h:312-320 */
      nx[o] = s.x / ns;
      ny[o] = s.y / ns;
      nz[o] = s.z / ns;
    }
  }
  return bad;
}

/* util/fields.h:206-234: ratios by integer division (std::ceil of an int
   quotient), phi pass into a zeroed row buffer, then the theta pass into a
   zeroed output. */
void po_oracle_average(const float *in, int nth_in, int nph_in, float *out, int nth_out, int nph_out) {
  int rp = nph_in / nph_out, rt = nth_in / nth_out;
  float *rows = (float *)calloc((size_t)nth_in * nph_out, sizeof(float));
  for (int i = 0; i < nth_in; ++i)
    for (int j = 0; j < nph_out; ++j)
      for (int k = 0; k < rp; ++k) rows[(size_t)i * nph_out + j] += in[(size_t)i * nph_in + j * rp + k] / (float)rp;
  for (int i = 0; i < nth_out; ++i)
    for (int j = 0; j < nph_out; ++j) {
      out[(size_t)i * nph_out + j] = 0.f;
      for (int k = 0; k < rt; ++k) out[(size_t)i * nph_out + j] += rows[(size_t)(i * rt + k) * nph_out + j] / (float)rt;
    }
  free(rows);
}
