// wavepo_cli.cpp -- drop-in command-line drivers over the C ABI (include/wavepo.h).
//
// Each executable keeps the argv, the relative input paths and the output
// file names of one reference driver, so existing scripts and notebooks run
// unchanged against the GB300 engine:
//
//   wavepo_sphere   LS LE DEPTH            compareMie/sphere.cu:23-25
//       mesh/sphere10um_{,area_,normal_}float.binary -> output/sphere_10um_lambda<i>_T<M|E>_depth<d>.binary
//   wavepo_ellipsoid DEPTH                 compareBEM3d/ellipsoid.cu:23
//       mesh/PO/ellipsoid_3_3_2_{,area_,normal_}float.binary
//       -> output/ellipsoid_lambda0_T<M|E>_depth<d>_kappa0.3.binary
//   wavepo_ellipsoid_simple                compareBEM3d/ellipsoid_simple.cu:384
//       (same mesh) -> output/ellipsoid_TM_kappa0.3.binary (float64, 3600 azimuths at theta = 0)
//   wavepo_treepo   LS LE TI PI FIBER DEPTH R0 R1   fibersim/treePO.cu:27-34
//       mesh/fiber<k>.binary -> output/fiber_<k>_lambda<i>_TM_depth<d>.binary
//
// Every physical constant, preset and grid rule is the driver's own (cited at
// each use).  Inputs are the reference's raw float32 files: SoA points
// [x..., y..., z...], areas, normals [nx..., ny..., nz...] (sphere.cu:94-125)
// or the height field [2][numel][numelvert] (treePO.cu:81-86); outputs are raw
// float32 [n_theta][n_phi] intensities (sphere.cu:929-932), except the FP64
// ring of ellipsoid_simple (float64, ellipsoid_simple.cu:609-611).
//
// Differences from the reference drivers, all on the side of failing loudly:
// a missing or short input file is an error (the reference reads whatever is
// there), the point count of a mesh is taken from the size of its area file
// (the reference hard-codes it; the shipped meshes have exactly that many),
// and CUDA or argument errors return a non-zero exit status instead of exit()
// from inside a helper.  Options after the positional arguments, which the
// reference ignores, select the engine's modes:
//   --theta-mode double|reference   (default double: accurate at the poles)
//   --precision fp32|split_bf16|fp64  --interp tensor|fft
//   --mesh-dir DIR  --output-dir DIR
#include <cuda_runtime.h>
#include <sys/stat.h>

#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "wavepo.h"

namespace {

struct Options {
  int theta_mode = PO_THETA_DOUBLE_COVER;
  int precision = -1;  // -1: the driver's own (FP32 patterns; FP64 for ellipsoid_simple)
  int interp = PO_INTERP_TENSOR;
  std::string mesh_dir = "mesh";
  std::string output_dir = "output";
};

[[noreturn]] void die(const std::string &msg) {
  std::fprintf(stderr, "error: %s\n", msg.c_str());
  std::exit(1);
}

void check(po_status s, const char *what) {
  if (s != PO_OK) die(std::string(what) + ": " + po_status_string(s) + ": " + po_last_error());
}

Options parse_options(int argc, char **argv, int first) {
  Options o;
  for (int i = first; i < argc; ++i) {
    std::string a = argv[i];
    auto val = [&](const char *name) -> std::string {
      if (i + 1 >= argc) die(std::string("missing value after ") + name);
      return argv[++i];
    };
    if (a == "--theta-mode") {
      std::string v = val("--theta-mode");
      if (v == "double") o.theta_mode = PO_THETA_DOUBLE_COVER;
      else if (v == "reference") o.theta_mode = PO_THETA_REFERENCE;
      else die("--theta-mode must be double or reference");
    } else if (a == "--precision") {
      std::string v = val("--precision");
      if (v == "fp32") o.precision = PO_PREC_FP32;
      else if (v == "split_bf16") o.precision = PO_PREC_SPLIT_BF16;
      else if (v == "fp64") o.precision = PO_PREC_FP64;
      else die("--precision must be fp32, split_bf16 or fp64");
    } else if (a == "--interp") {
      std::string v = val("--interp");
      if (v == "tensor") o.interp = PO_INTERP_TENSOR;
      else if (v == "fft") o.interp = PO_INTERP_FFT;
      else die("--interp must be tensor or fft");
    } else if (a == "--mesh-dir") {
      o.mesh_dir = val("--mesh-dir");
    } else if (a == "--output-dir") {
      o.output_dir = val("--output-dir");
    } else {
      die("unknown option " + a);
    }
  }
  return o;
}

int parse_int(const char *s, const char *what) {
  char *end = nullptr;
  long v = std::strtol(s, &end, 10);
  if (!end || *end || end == s) die(std::string(what) + " must be an integer");
  return (int)v;
}

std::vector<float> read_floats(const std::string &path, size_t count) {
  std::ifstream f(path, std::ios::binary);
  if (!f) die("cannot open " + path);
  std::vector<float> v(count);
  f.read((char *)v.data(), (std::streamsize)(count * sizeof(float)));
  if ((size_t)f.gcount() != count * sizeof(float)) die("short read: " + path);
  return v;
}

size_t file_floats(const std::string &path) {
  std::ifstream f(path, std::ios::binary | std::ios::ate);
  if (!f) die("cannot open " + path);
  return (size_t)f.tellg() / sizeof(float);
}

void write_file(const std::string &path, const void *p, size_t bytes) {
  std::ofstream f(path, std::ios::binary);
  if (!f) die("cannot write " + path);
  f.write((const char *)p, (std::streamsize)bytes);
  if (!f) die("write failed: " + path);
}

// SoA mesh of compareMie/sphere.cu:94-125 (prefix_float / _area_float / _normal_float)
struct Mesh {
  int64_t n = 0;
  std::vector<float> p, a, q;  // [3][n], [n], [3][n]
  po_geometry geometry() const {
    po_geometry g{};
    g.n = n;
    g.x = p.data();
    g.y = p.data() + n;
    g.z = p.data() + 2 * n;
    g.nx = q.data();
    g.ny = q.data() + n;
    g.nz = q.data() + 2 * n;
    g.area = a.data();
    g.on_device = 0;
    return g;
  }
};

Mesh read_mesh(const std::string &prefix) {
  Mesh m;
  m.n = (int64_t)file_floats(prefix + "_area_float.binary");
  if (m.n <= 0) die("empty mesh " + prefix);
  m.p = read_floats(prefix + "_float.binary", 3 * (size_t)m.n);
  m.a = read_floats(prefix + "_area_float.binary", (size_t)m.n);
  m.q = read_floats(prefix + "_normal_float.binary", 3 * (size_t)m.n);
  return m;
}

// wavelength of index i: compareMie/sphere.cu:486-488 (float arithmetic)
double reference_lambda(int i) {
  float w = 400.f + (700.f - 400.f) / (float)25 * i;
  w *= 1e-9f;
  return (double)w;
}

po_config make_config(int depth, int nth, int nph, const float bmin[3], const float bmax[3], double theta_extent,
                      double phi_extent, double ratio, const Options &o) {
  po_config cfg;
  check(po_config_init(&cfg, depth, nth, nph, bmin, bmax, theta_extent, phi_extent, ratio, 6.0, 0.4e-6),
        "po_config_init");
  cfg.theta_mode = o.theta_mode;
  cfg.precision = o.precision < 0 ? PO_PREC_FP32 : o.precision;
  cfg.interp_method = o.interp;
  if (cfg.precision == PO_PREC_FP64 && depth != 0) die("--precision fp64 needs depth 0");
  return cfg;
}

// one po_solve over the wavelengths x polarisations of a driver; out is [L][1][P][nth][nph]
std::vector<float> solve(const po_config &cfg, const po_geometry &g, const std::vector<double> &lams,
                         double theta_i, double phi_i, int pol_mask, double eta_re, double eta_im, double sigma) {
  po_ctx *ctx = nullptr;
  check(po_create(&ctx, &cfg), "po_create");
  po_illum il{};
  il.n_lambda = (int)lams.size();
  il.lambda_m = lams.data();
  il.n_inc = 1;
  il.theta_i = &theta_i;
  il.phi_i = &phi_i;
  il.pol_mask = pol_mask;
  il.eta_re = eta_re;
  il.eta_im = eta_im;
  il.sigma = sigma;
  const int npol = ((pol_mask & PO_POL_TM) ? 1 : 0) + ((pol_mask & PO_POL_TE) ? 1 : 0);
  std::vector<float> out(lams.size() * npol * (size_t)cfg.n_theta[0] * cfg.n_phi[0]);
  po_status s = po_solve(ctx, &g, &il, out.data(), 0, nullptr, nullptr);
  po_destroy(ctx);
  check(s, "po_solve");
  return out;
}

void make_dir(const std::string &d) {
  if (mkdir(d.c_str(), 0777) != 0 && errno != EEXIST) die("cannot create " + d);
}

// ------------------------------------------------------------------ sphere
int main_sphere(int argc, char **argv) {
  if (argc < 4) {
    std::fprintf(stderr, "usage: wavepo_sphere LAMBDA_START LAMBDA_END DEPTH [options]\n");
    return 2;
  }
  const int ls = parse_int(argv[1], "LAMBDA_START"), le = parse_int(argv[2], "LAMBDA_END");
  const int depth = parse_int(argv[3], "DEPTH");
  if (depth < 0) die("DEPTH must be >= 0");  // sphere.cu:26 asserts
  Options o = parse_options(argc, argv, 4);
  make_dir(o.output_dir);
  // sphere.cu:35-58: radius 10 um, beam sigma 10000 um, 900 x 1440, box 1.1 r, ratio 1.3
  const float radius = 10e-6f, er = 1.1f;
  const float bmin[3] = {-radius * er, -radius * er, -radius * er}, bmax[3] = {radius * er, radius * er, radius * er};
  po_config cfg = make_config(depth, 900, 1440, bmin, bmax, 2.0 * radius, 2.0 * radius, 1.3, o);
  Mesh m = read_mesh(o.mesh_dir + "/sphere10um");
  std::vector<double> lams;
  for (int i = ls; i < le; ++i) lams.push_back(reference_lambda(i));
  if (lams.empty()) return 0;
  // sphere.cu:541-579: theta_i = phi_i = 0, eta = 1.55, polarisations M then E
  std::vector<float> out = solve(cfg, m.geometry(), lams, 0.0, 0.0, PO_POL_TM | PO_POL_TE, 1.55, 0.0, 10000e-6);
  const size_t nd = 900 * 1440;
  for (size_t l = 0; l < lams.size(); ++l)
    for (int p = 0; p < 2; ++p) {
      // sphere.cu:929-932
      std::string f = o.output_dir + "/sphere_10um_lambda" + std::to_string(ls + (int)l) + "_T" + (p ? "E" : "M") +
                      "_depth" + std::to_string(depth) + ".binary";
      write_file(f, out.data() + (l * 2 + p) * nd, nd * sizeof(float));
    }
  return 0;
}

// ------------------------------------------------------------ ellipsoid (tree)
int main_ellipsoid(int argc, char **argv) {
  if (argc < 2) {
    std::fprintf(stderr, "usage: wavepo_ellipsoid DEPTH [options]\n");
    return 2;
  }
  const int depth = parse_int(argv[1], "DEPTH");
  if (depth < 0) die("DEPTH must be >= 0");
  Options o = parse_options(argc, argv, 2);
  make_dir(o.output_dir);
  // ellipsoid.cu:38-56: box +-10 x +-10 x +-5 um, ratio 3 on a 10 um period / 20 um width
  const float r1 = 10e-6f, r2 = 10e-6f, period = 10e-6f;
  const float bmin[3] = {-r1, -r2, -period * 0.5f}, bmax[3] = {r1, r2, period * 0.5f};
  po_config cfg = make_config(depth, 900, 1440, bmin, bmax, period, 2.0 * std::max(r1, r2), 3.0, o);
  Mesh m = read_mesh(o.mesh_dir + "/PO/ellipsoid_3_3_2");
  // ellipsoid.cu:486-560: 500 nm, eta = 1.55 + 0.3i, theta_i = phi_i = 0, M then E
  std::vector<float> out = solve(cfg, m.geometry(), {(double)(500.f * 1e-9f)}, 0.0, 0.0, PO_POL_TM | PO_POL_TE, 1.55,
                                 0.3, 10000e-6);
  const size_t nd = 900 * 1440;
  for (int p = 0; p < 2; ++p) {
    std::string f = o.output_dir + "/ellipsoid_lambda0_T" + (p ? "E" : "M") + "_depth" + std::to_string(depth) +
                    "_kappa0.3.binary";  // ellipsoid.cu:956
    write_file(f, out.data() + p * nd, nd * sizeof(float));
  }
  return 0;
}

// ------------------------------------------------- ellipsoid_simple (FP64 ring)
int main_ellipsoid_simple(int argc, char **argv) {
  Options o = parse_options(argc, argv, 1);
  make_dir(o.output_dir);
  Mesh m = read_mesh(o.mesh_dir + "/PO/ellipsoid_3_3_2");
  // ellipsoid_simple.cu:396-472: 500 nm, eta = 1.55 + 0.3i, TM, 3600 azimuths on the theta = 0 ring.
  // Row 1 of a 2 x 3600 grid is theta = -pi/2 + 1e-10 + pi/2 = 1e-10, the ring to 1e-10 rad.  The
  // reference evaluates exp(-ik|ob - x|)/|ob - x| at |ob| = 1 m; this is its far-field limit (the
  // two differ by O(k |x|^2 / 2 m), 6e-5 rad for this mesh).
  const float bmin[3] = {-10e-6f, -10e-6f, -5e-6f}, bmax[3] = {10e-6f, 10e-6f, 5e-6f};
  if (o.precision < 0) o.precision = PO_PREC_FP64;  // the driver is the FP64 direct sum
  po_config cfg = make_config(0, 2, 3600, bmin, bmax, 10e-6, 20e-6, 3.0, o);
  std::vector<float> out = solve(cfg, m.geometry(), {500e-9}, 0.0, 0.0, PO_POL_TM, 1.55, 0.3, 10000e-6);
  std::vector<double> ring(3600);
  for (int k = 0; k < 3600; ++k) ring[k] = out[3600 + k];
  write_file(o.output_dir + "/ellipsoid_TM_kappa0.3.binary", ring.data(), ring.size() * sizeof(double));
  return 0;
}

// ------------------------------------------------------------------ treePO
int main_treepo(int argc, char **argv) {
  if (argc < 9) {
    std::fprintf(stderr,
                 "usage: wavepo_treepo LAMBDA_START LAMBDA_END THETA_I PHI_I FIBER DEPTH RING_START RING_END "
                 "[options]\n");
    return 2;
  }
  const int ls = parse_int(argv[1], "LAMBDA_START"), le = parse_int(argv[2], "LAMBDA_END");
  const int ti = parse_int(argv[3], "THETA_I"), pi = parse_int(argv[4], "PHI_I");
  const int fiber = parse_int(argv[5], "FIBER"), depth = parse_int(argv[6], "DEPTH");
  const int r0 = parse_int(argv[7], "RING_START"), r1i = parse_int(argv[8], "RING_END");
  if (fiber < 0 || fiber > 3) die("FIBER must be 0..3");
  if (depth < 0) die("DEPTH must be >= 0");
  Options o = parse_options(argc, argv, 9);
  make_dir(o.output_dir);
  // treePO.cu:44-51 presets
  const float periodv[4] = {20e-6f, 50e-6f, 400e-6f, 400e-6f};
  const float r1v[4] = {20e-6f, 40e-6f, 40e-6f, 40e-6f}, r2v[4] = {20e-6f, 40e-6f, 35e-6f, 35e-6f};
  const float sigv[4] = {10e-6f, 10e-6f, 150e-6f, 150e-6f};
  const int numelv[4] = {3000, 5026, 4420, 4720}, numelvertv[4] = {478, 1000, 8000, 8000};
  const int thetaov[4] = {450, 900, 7200, 7200}, phiov[4] = {880, 1440, 1440, 1440};
  const float period = periodv[fiber], r1 = r1v[fiber], r2 = r2v[fiber];
  const int numel = numelv[fiber], numelvert = numelvertv[fiber];
  const float unitz = period / numelvert;  // treePO.cu:61
  if (r0 < 0 || r1i < r0 || r1i >= numel) die("ring segment out of range");
  std::vector<float> h = read_floats(o.mesh_dir + "/fiber" + std::to_string(fiber) + ".binary",
                                     2 * (size_t)numel * numelvert);
  const int64_t n = (int64_t)(r1i - r0 + 1) * numelvert;
  float *dh = nullptr, *dg = nullptr;
  if (cudaMalloc(&dh, h.size() * sizeof(float)) != cudaSuccess || cudaMalloc(&dg, 7 * n * sizeof(float)) != cudaSuccess)
    die("cudaMalloc failed");
  if (cudaMemcpy(dh, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess)
    die("cudaMemcpy failed");
  // treePO.cu:132 -> util/geometry.h:76-179
  check(po_height_field_points(dh, numel, numelvert, period, unitz, r0, r1i, dg, dg + n, dg + 2 * n, dg + 3 * n,
                               dg + 4 * n, dg + 5 * n, dg + 6 * n, nullptr),
        "po_height_field_points");
  po_geometry g{};
  g.n = n;
  g.x = dg;
  g.y = dg + n;
  g.z = dg + 2 * n;
  g.nx = dg + 3 * n;
  g.ny = dg + 4 * n;
  g.nz = dg + 5 * n;
  g.area = dg + 6 * n;
  g.on_device = 1;
  // treePO.cu:93-98 box, :353-359 grids (ratio 1.2)
  const float er = 1.1f;
  const float bmin[3] = {-r1 * er, -r2 * er, -period * 0.5f * er}, bmax[3] = {r1 * er, r2 * er, period * 0.5f * er};
  po_config cfg = make_config(depth, thetaov[fiber], phiov[fiber], bmin, bmax, period, 2.0 * std::max(r1, r2), 1.2, o);
  std::vector<double> lams;
  for (int i = ls; i < le; ++i) lams.push_back(reference_lambda(i));
  int rc = 0;
  if (!lams.empty()) {
    // treePO.cu:554-565: incidence from the indices (float), eta = 1.55 (sigma = 0 -> kappa = 0), mode M only
    const float thetai = (float)(-M_PI / 2 + 1e-10f + M_PI / 180 * ti);
    const float phii = (float)(2 * M_PI / 360 * pi);
    std::vector<float> out = solve(cfg, g, lams, thetai, phii, PO_POL_TM, 1.55, 0.0, sigv[fiber]);
    const size_t nd = (size_t)thetaov[fiber] * phiov[fiber];
    for (size_t l = 0; l < lams.size(); ++l) {
      std::string f = o.output_dir + "/fiber_" + std::to_string(fiber) + "_lambda" + std::to_string(ls + (int)l) +
                      "_TM_depth" + std::to_string(depth) + ".binary";  // treePO.cu:969
      write_file(f, out.data() + l * nd, nd * sizeof(float));
    }
  }
  cudaFree(dh);
  cudaFree(dg);
  return rc;
}

}  // namespace

int main(int argc, char **argv) {
#if defined(WAVEPO_CLI_SPHERE)
  return main_sphere(argc, argv);
#elif defined(WAVEPO_CLI_ELLIPSOID)
  return main_ellipsoid(argc, argv);
#elif defined(WAVEPO_CLI_ELLIPSOID_SIMPLE)
  return main_ellipsoid_simple(argc, argv);
#elif defined(WAVEPO_CLI_TREEPO)
  return main_treepo(argc, argv);
#else
#error "define one of WAVEPO_CLI_SPHERE, WAVEPO_CLI_ELLIPSOID, WAVEPO_CLI_ELLIPSOID_SIMPLE, WAVEPO_CLI_TREEPO"
#endif
}
