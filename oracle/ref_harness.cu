// ref_harness.cu -- runs the UNMODIFIED WaveFiber3d CUDA path (util/*.h) on
// caller-chosen inputs so that its outputs can be frozen as golden fixtures.
// TEST INFRASTRUCTURE ONLY.  Built on the GPU host by oracle/Makefile from
// reference headers staged into oracle/_ref/src (never committed).
//
// The call sequence restates the driver main() of compareMie/sphere.cu:
//   octree build ........ sphere.cu:212-251 -> util/tree.h:290
//   active lists/centres  sphere.cu:255-328
//   level grids ......... given on the command line (sphere.cu:334-365 rule is
//                         applied by the fixture script)
//   factor1 table ....... sphere.cu:499-539
//   currents ............ sphere.cu:581-585 -> tangentplane.h:84, fields.h:123,:147
//   level loop .......... sphere.cu:592-936 (leaf reduce, copyandinterp,
//                         translation_compute, sumchildren, computeintensity)
// Only the parameters (geometry, box, grids, wavelength, incidence, mode,
// ior, beam sigma) differ from the reference drivers.

#include <cufft.h>
// cuFFT 12+ dropped three result codes that util/helper_cuda.h:141-157 still
// names; give them unused values so the header compiles unmodified.
#define CUFFT_INCOMPLETE_PARAMETER_LIST ((cufftResult)0xA)
#define CUFFT_PARSE_ERROR ((cufftResult)0xC)
#define CUFFT_LICENSE_ERROR ((cufftResult)0xF)
#include <thrust/functional.h>
// CCCL 3 removed thrust::binary_function, which util/util.h:384 derives from.
namespace thrust {
template <typename A1, typename A2, typename R>
struct binary_function {
  typedef A1 first_argument_type;
  typedef A2 second_argument_type;
  typedef R result_type;
};
}  // namespace thrust

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "util/util.h"
#include "util/tangentplane.h"
#include "util/fields.h"
#include "util/interpolation.h"
#include "util/tree.h"
#include "util/geometry.h"

static std::vector<float> read_f32(const char *path, size_t count) {
  std::vector<float> v(count);
  std::ifstream f(path, std::ios::binary);
  if (!f) { fprintf(stderr, "cannot open %s\n", path); exit(2); }
  f.read((char *)v.data(), count * sizeof(float));
  if ((size_t)f.gcount() != count * sizeof(float)) { fprintf(stderr, "short read %s\n", path); exit(2); }
  return v;
}

static void write_bytes(const char *path, const void *p, size_t bytes) {
  std::ofstream f(path, std::ios::binary);
  f.write((const char *)p, bytes);
}

// geometry file: SoA float32 x[n] y[n] z[n] nx[n] ny[n] nz[n] area[n]
struct Geom {
  int n;
  hostFvec x, y, z, nx, ny, nz, a;
};
static Geom load_geom(const char *path, int n) {
  std::vector<float> v = read_f32(path, (size_t)7 * n);
  Geom g;
  g.n = n;
  g.x.assign(v.begin(), v.begin() + n);
  g.y.assign(v.begin() + n, v.begin() + 2 * n);
  g.z.assign(v.begin() + 2 * n, v.begin() + 3 * n);
  g.nx.assign(v.begin() + 3 * n, v.begin() + 4 * n);
  g.ny.assign(v.begin() + 4 * n, v.begin() + 5 * n);
  g.nz.assign(v.begin() + 5 * n, v.begin() + 6 * n);
  g.a.assign(v.begin() + 6 * n, v.begin() + 7 * n);
  return g;
}

// E/H directions of sphere.cu:559-579
static void incident(float thetai, float phii, char mode, Float3 &wavedir, Float3 &Edir, Float3 &Hdir) {
  thrust::get<0>(wavedir) = cos(thetai) * cos(phii);
  thrust::get<1>(wavedir) = cos(thetai) * sin(phii);
  thrust::get<2>(wavedir) = sin(thetai);
  if (mode == 'M') {
    thrust::get<0>(Edir) = -sin(thetai) * cos(phii);
    thrust::get<1>(Edir) = -sin(thetai) * sin(phii);
    thrust::get<2>(Edir) = cos(thetai);
    thrust::get<0>(Hdir) = sin(phii);
    thrust::get<1>(Hdir) = -cos(phii);
    thrust::get<2>(Hdir) = 0;
  } else {
    thrust::get<0>(Edir) = -sin(phii);
    thrust::get<1>(Edir) = cos(phii);
    thrust::get<2>(Edir) = 0;
    thrust::get<0>(Hdir) = -sin(thetai) * cos(phii);
    thrust::get<1>(Hdir) = -sin(thetai) * sin(phii);
    thrust::get<2>(Hdir) = cos(thetai);
  }
}

static void dump_c6(const char *path, const deviceC6vec &cur) {
  hostC6vec h = cur;
  std::vector<float> out(h.size() * 12);
  for (size_t i = 0; i < h.size(); ++i) {
    comFloat6 c = h[i];
    comThr v[6] = {thrust::get<0>(c), thrust::get<1>(c), thrust::get<2>(c),
                   thrust::get<3>(c), thrust::get<4>(c), thrust::get<5>(c)};
    for (int k = 0; k < 6; ++k) { out[i * 12 + 2 * k] = v[k].real(); out[i * 12 + 2 * k + 1] = v[k].imag(); }
  }
  write_bytes(path, out.data(), out.size() * sizeof(float));
}

// currents <geom> <n> <lambda_m> <theta_i> <phi_i> <M|E> <eta_re> <eta_im> <sigma> <out>
static int cmd_currents(char **a) {
  int n = atoi(a[1]);
  Geom g = load_geom(a[0], n);
  float wavelength = atof(a[2]), thetai = atof(a[3]), phii = atof(a[4]);
  char mode = a[5][0];
  comThr eta = comThr((float)atof(a[6]), (float)atof(a[7]));
  float sigma = atof(a[8]);
  float k0 = 2 * M_PI / wavelength;
  deviceFvec x = g.x, y = g.y, z = g.z, nx = g.nx, ny = g.ny, nz = g.nz;
  deviceC6vec cur(n);
  Float3 wavedir, Edir, Hdir;
  incident(thetai, phii, mode, wavedir, Edir, Hdir);
  computeLocalTangentPlane(x, y, z, nx, ny, nz, cur, wavedir, Edir, Hdir, comThr(1.0, 0.0), eta, Z0,
                           cos(thetai), sigma, k0, mode);
  checkCudaErrors(cudaDeviceSynchronize());
  dump_c6(a[9], cur);
  return 0;
}

// interp <in.bin complex64 [thc][phc]> <thc> <phc> <thp> <php> <out>
static int cmd_interp(char **a) {
  int thc = atoi(a[1]), phc = atoi(a[2]), thp = atoi(a[3]), php = atoi(a[4]);
  std::vector<float> in = read_f32(a[0], (size_t)2 * thc * phc);
  int obnum = thp * php;
  // plans exactly as sphere.cu:392-447 with level i+1 = child, i = parent
  cufftHandle pphi, piphi, pth, pith;
  int rank = 1, num[1], inembed[1], onembed[1];
  num[0] = phc; inembed[0] = thc * phc; onembed[0] = thc * phc;
  cufftPlanMany(&pphi, rank, num, inembed, 1, phc, onembed, 1, phc, CUFFT_C2C, thc);
  num[0] = php;
  cufftPlanMany(&piphi, rank, num, inembed, 1, php, onembed, 1, php, CUFFT_C2C, thc);
  inembed[0] = obnum; onembed[0] = obnum; num[0] = thc;
  cufftPlanMany(&pth, rank, num, inembed, php, 1, onembed, 1, thc, CUFFT_C2C, php);
  num[0] = thp;
  cufftPlanMany(&pith, rank, num, inembed, 1, thp, onembed, php, 1, CUFFT_C2C, php);
  hostf2vec hin(thc * phc);
  for (int i = 0; i < thc * phc; ++i) { hin[i].x = in[2 * i]; hin[i].y = in[2 * i + 1]; }
  devicef2vec field = hin, tmp1(obnum), tmp2(obnum);
  copyandinterp(field, 0, thc * phc, tmp1, tmp2, obnum, pphi, piphi, pth, pith, phc, php, thc, thp, thc, php);
  checkCudaErrors(cudaDeviceSynchronize());
  hostf2vec hout = tmp1;
  std::vector<float> out((size_t)2 * obnum);
  for (int i = 0; i < obnum; ++i) { out[2 * i] = hout[i].x; out[2 * i + 1] = hout[i].y; }
  write_bytes(a[5], out.data(), out.size() * sizeof(float));
  return 0;
}

struct Tree {
  std::vector<Octree_node> nodes;
  int max_nodes;
};

// CDP build of util/tree.h:290 exactly as sphere.cu:212-251; geometry arrays
// are reordered in place (x_d0 etc.).
static Tree build_tree(deviceFvec &x0, deviceFvec &y0, deviceFvec &z0, deviceFvec &nx0, deviceFvec &ny0,
                       deviceFvec &nz0, deviceFvec &a0, const float *box, int max_depth) {
  int n = x0.size();
  deviceFvec x1(n), y1(n), z1(n), nx1(n), ny1(n), nz1(n), a1(n);
  Points pinit[2], ninit[2];
  Area ainit[2];
  pinit[0].set(thrust::raw_pointer_cast(&x0[0]), thrust::raw_pointer_cast(&y0[0]), thrust::raw_pointer_cast(&z0[0]));
  pinit[1].set(thrust::raw_pointer_cast(&x1[0]), thrust::raw_pointer_cast(&y1[0]), thrust::raw_pointer_cast(&z1[0]));
  ninit[0].set(thrust::raw_pointer_cast(&nx0[0]), thrust::raw_pointer_cast(&ny0[0]), thrust::raw_pointer_cast(&nz0[0]));
  ninit[1].set(thrust::raw_pointer_cast(&nx1[0]), thrust::raw_pointer_cast(&ny1[0]), thrust::raw_pointer_cast(&nz1[0]));
  ainit[0].set(thrust::raw_pointer_cast(&a0[0]));
  ainit[1].set(thrust::raw_pointer_cast(&a1[0]));
  Points *points, *normals;
  Area *areas;
  checkCudaErrors(cudaMalloc((void **)&points, 2 * sizeof(Points)));
  checkCudaErrors(cudaMemcpy(points, pinit, 2 * sizeof(Points), cudaMemcpyHostToDevice));
  checkCudaErrors(cudaMalloc((void **)&normals, 2 * sizeof(Points)));
  checkCudaErrors(cudaMemcpy(normals, ninit, 2 * sizeof(Points), cudaMemcpyHostToDevice));
  checkCudaErrors(cudaMalloc((void **)&areas, 2 * sizeof(Area)));
  checkCudaErrors(cudaMemcpy(areas, ainit, 2 * sizeof(Area), cudaMemcpyHostToDevice));
  Tree t;
  t.max_nodes = (int)((pow(8, max_depth + 1) - 1) / 7);
  Octree_node root;
  root.set_range(0, n);
  root.set_bounding_box(box[0], box[1], box[2], box[3], box[4], box[5]);
  Octree_node *nodes;
  checkCudaErrors(cudaMalloc((void **)&nodes, t.max_nodes * sizeof(Octree_node)));
  checkCudaErrors(cudaMemcpy(nodes, &root, sizeof(Octree_node), cudaMemcpyHostToDevice));
  // sphere.cu:226 sets the sync depth without checking; under CUDA 12+ dynamic
  // parallelism that limit is unsupported, so the call fails there as well.
  cudaDeviceSetLimit(cudaLimitDevRuntimeSyncDepth, max_depth > 0 ? max_depth : 1);
  cudaGetLastError();
  checkCudaErrors(cudaDeviceSetLimit(cudaLimitDevRuntimePendingLaunchCount, 32768));
  Parameters params(max_depth, 16);
  const int NT = 256;
  build_octree_kernel<NT><<<1, NT, 8 * (NT / 32) * sizeof(int)>>>(nodes, points, normals, areas, params);
  checkCudaErrors(cudaGetLastError());
  checkCudaErrors(cudaDeviceSynchronize());
  t.nodes.resize(t.max_nodes);
  checkCudaErrors(cudaMemcpy(t.nodes.data(), nodes, t.max_nodes * sizeof(Octree_node), cudaMemcpyDeviceToHost));
  cudaFree(nodes); cudaFree(points); cudaFree(normals); cudaFree(areas);
  return t;
}

// octree <geom> <n> <6 box floats> <depth> <out>: reordered SoA geometry then
// (begin,end) of every heap node as int32.
static int cmd_octree(char **a) {
  int n = atoi(a[1]);
  Geom g = load_geom(a[0], n);
  float box[6];
  for (int i = 0; i < 6; ++i) box[i] = atof(a[2 + i]);
  int depth = atoi(a[8]);
  deviceFvec x = g.x, y = g.y, z = g.z, nx = g.nx, ny = g.ny, nz = g.nz, ar = g.a;
  Tree t = build_tree(x, y, z, nx, ny, nz, ar, box, depth);
  std::vector<float> out;
  for (deviceFvec *v : {&x, &y, &z, &nx, &ny, &nz, &ar}) {
    hostFvec h = *v;
    out.insert(out.end(), h.begin(), h.end());
  }
  std::vector<int> rng(2 * t.max_nodes);
  for (int i = 0; i < t.max_nodes; ++i) { rng[2 * i] = t.nodes[i].points_begin(); rng[2 * i + 1] = t.nodes[i].points_end(); }
  std::ofstream f(a[9], std::ios::binary);
  f.write((const char *)out.data(), out.size() * sizeof(float));
  f.write((const char *)rng.data(), rng.size() * sizeof(int));
  return 0;
}

// solve <geom> <n> <6 box floats> <depth> <th0> <ph0> [<th_i> <ph_i> for i=1..depth]
//       <lambda_m> <theta_i> <phi_i> <M|E> <eta_re> <eta_im> <sigma> <out>
// Times of the phases of one solve (ms, CUDA events on the legacy stream,
// which the reference's calls use) and the counts needed to extrapolate the
// capped loops: the leaf loop runs `leaf_dirs_done` of `leaf_dirs` directions
// and each level `children_done[i]` of `children[i]` active children.
struct SolveTiming {
  double tree = 0, setup = 0, leaf = 0, level[16] = {}, intensity = 0;
  int leaf_dirs = 0, leaf_dirs_done = 0, children[16] = {}, children_done[16] = {};
};

static float ev_ms(cudaEvent_t a, cudaEvent_t b) {
  float t = 0;
  cudaEventSynchronize(b);
  cudaEventElapsedTime(&t, a, b);
  return t;
}

static int run_solve(char **a, int max_leaf_dirs, int max_children, SolveTiming *tm, bool skip_root = false);
static int cmd_solve(char **a) { return run_solve(a, 0, 0, nullptr); }

// time <solve arguments> <max leaf directions (0: all)> <max children per level (0: all)> <skip root>
// Prints one line: the measured phase times and the counts of the capped loops.
// skip root = 1 leaves out the root level and the intensity: the reference's
// interpolation only upsamples (util/interpolation.h:29-30 index the padding
// from the size difference), so a level-1 grid finer than the output grid is
// outside what it can run.
static int cmd_time(char **a, int argc) {
  int max_depth = atoi(a[8]);
  const int extra = 9 + 2 * (max_depth + 1) + 8;
  if (argc < extra + 3) { fprintf(stderr, "time: missing caps\n"); return 2; }
  SolveTiming tm;
  const int rc = run_solve(a, atoi(a[extra]), atoi(a[extra + 1]), &tm, atoi(a[extra + 2]) != 0);
  if (rc) return rc;
  printf("{\"tree_ms\": %.4f, \"setup_ms\": %.4f, \"leaf_ms\": %.4f, \"leaf_dirs\": %d, \"leaf_dirs_done\": %d, "
         "\"intensity_ms\": %.4f, \"levels\": [", tm.tree, tm.setup, tm.leaf, tm.leaf_dirs, tm.leaf_dirs_done,
         tm.intensity);
  for (int i = 0; i < max_depth; ++i)
    printf("%s{\"level\": %d, \"ms\": %.4f, \"children\": %d, \"children_done\": %d}", i ? ", " : "", i,
           tm.level[i], tm.children[i], tm.children_done[i]);
  printf("]}\n");
  return 0;
}

static int run_solve(char **a, int max_leaf_dirs, int max_children, SolveTiming *tm, bool skip_root) {
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, 0);
  int n = atoi(a[1]);
  Geom g = load_geom(a[0], n);
  float box[6];
  for (int i = 0; i < 6; ++i) box[i] = atof(a[2 + i]);
  int max_depth = atoi(a[8]);
  std::vector<int> thn(max_depth + 1), phn(max_depth + 1), an(max_depth + 1);
  int k = 9;
  for (int i = 0; i <= max_depth; ++i) { thn[i] = atoi(a[k++]); phn[i] = atoi(a[k++]); an[i] = thn[i] * phn[i]; }
  float wavelength = atof(a[k++]);
  float thetai = atof(a[k++]), phii = atof(a[k++]);
  char mode = a[k++][0];
  float eta_re = atof(a[k++]), eta_im = atof(a[k++]);
  float gaussiansigma = atof(a[k++]);
  const char *outpath = a[k++];
  const float thetastartoffset = 1e-10;
  const float Dis = 1;
  const int NT = 256;
  int thetaonum = thn[0], phionum = phn[0], obnum = an[0];
  int max_nodes = (int)((pow(8, max_depth + 1) - 1) / 7);
  int nonleafnodes = (int)((pow(8, max_depth) - 1) / 7);

  deviceFvec x_d0 = g.x, y_d0 = g.y, z_d0 = g.z, nx_d0 = g.nx, ny_d0 = g.ny, nz_d0 = g.nz, a_d0 = g.a;
  Tree t = build_tree(x_d0, y_d0, z_d0, nx_d0, ny_d0, nz_d0, a_d0, box, max_depth);
  std::vector<Octree_node> &host_nodes = t.nodes;
  cudaEventRecord(e1, 0);
  if (tm) tm->tree = ev_ms(e0, e1);
  cudaEventRecord(e0, 0);

  // active lists, leaf to top (sphere.cu:255-307)
  std::vector<std::vector<int>> nonempty;
  std::vector<int> nonemptynum(max_depth);
  for (int level = max_depth; level > 0; level--) {
    int s = (int)((pow(8, level) - 1) / 7), e = (int)((pow(8, level + 1) - 1) / 7);
    nonempty.push_back(std::vector<int>());
    int cnt = 0;
    for (int i = s; i < e; ++i) {
      Octree_node nd = host_nodes[i];
      bool act = false;
      if (nd.points_begin() < nd.points_end()) {
        if (level == max_depth) act = true;
        else
          for (int c = 0; c < 8; ++c)
            if (host_nodes[e + (i - s) * 8 + c].active) { act = true; break; }
      }
      host_nodes[i].active = act;
      if (act) { nonempty[max_depth - level].push_back(i); cnt++; }
    }
    nonemptynum[max_depth - level] = cnt;
  }
  // per-point leaf centres (sphere.cu:310-328)
  hostFvec cx(n, 0.0), cy(n, 0.0), cz(n, 0.0);
  for (int i = nonleafnodes; i < max_nodes; ++i) {
    float3 c;
    host_nodes[i].bounding_box().compute_center(c);
    for (int j = host_nodes[i].points_begin(); j < host_nodes[i].points_end(); ++j) { cx[j] = c.x; cy[j] = c.y; cz[j] = c.z; }
  }
  deviceFvec cx_d = cx, cy_d = cy, cz_d = cz;
  int anglesum_nonleaf = obnum, maxnum = obnum;
  for (int i = 1; i <= max_depth; ++i) {
    if (i < max_depth) anglesum_nonleaf += an[i];
    int cur = nonemptynum[max_depth - i] * an[i];
    if (cur > maxnum) maxnum = cur;
  }
  hostFvec dirvec(obnum * 3);
  for (int it = 0; it < thetaonum; it++) {
    float th = -M_PI / 2 + thetastartoffset + M_PI / thetaonum * it;
    for (int ip = 0; ip < phionum; ip++) {
      float ph = 2 * M_PI / phionum * ip;
      int d = it * phionum + ip;
      dirvec[d * 3] = cos(th) * cos(ph);
      dirvec[d * 3 + 1] = cos(th) * sin(ph);
      dirvec[d * 3 + 2] = sin(th);
    }
  }
  deviceFvec dirvec_d = dirvec;
  // cuFFT plans (sphere.cu:386-447)
  std::vector<cufftHandle> p_phi(max_depth), p_iphi(max_depth), p_th(max_depth), p_ith(max_depth);
  for (int i = 0; i < max_depth; ++i) {
    int rank = 1, num[1], inembed[1] = {an[i + 1]}, onembed[1] = {an[i + 1]};
    num[0] = phn[i + 1];
    cufftPlanMany(&p_phi[i], rank, num, inembed, 1, phn[i + 1], onembed, 1, phn[i + 1], CUFFT_C2C, thn[i + 1]);
    num[0] = phn[i];
    cufftPlanMany(&p_iphi[i], rank, num, inembed, 1, phn[i], onembed, 1, phn[i], CUFFT_C2C, thn[i + 1]);
    inembed[0] = an[i]; onembed[0] = an[i]; num[0] = thn[i + 1];
    cufftPlanMany(&p_th[i], rank, num, inembed, phn[i], 1, onembed, 1, thn[i + 1], CUFFT_C2C, phn[i]);
    num[0] = thn[i];
    cufftPlanMany(&p_ith[i], rank, num, inembed, 1, thn[i], onembed, phn[i], 1, CUFFT_C2C, phn[i]);
  }
  float6 zero6;
  thrust::get<0>(zero6) = make_cuFloatComplex(0, 0); thrust::get<1>(zero6) = make_cuFloatComplex(0, 0);
  thrust::get<2>(zero6) = make_cuFloatComplex(0, 0); thrust::get<3>(zero6) = make_cuFloatComplex(0, 0);
  thrust::get<4>(zero6) = make_cuFloatComplex(0, 0); thrust::get<5>(zero6) = make_cuFloatComplex(0, 0);
  int num = n > maxnum ? n : maxnum;
  devicef2vec F0[6], F1[6], T1[6];
  for (int c = 0; c < 6; ++c) { F0[c].resize(maxnum); F1[c].resize(num); T1[c].resize(obnum); }
  devicef2vec tmp2(obnum);
  deviceFvec scattering(obnum);

  float k0 = 2 * M_PI / wavelength;
  float omega = k0 * c0;
  comThr Efactor = -cunit * omega * mu0 / (4 * M_PI) * exp(-cunit * k0 * Dis) / Dis;
  comThr Hfactor = -cunit * omega * eps0 / (4 * M_PI) * exp(-cunit * k0 * Dis) / Dis;
  // factor1 (sphere.cu:499-539)
  hostf2vec factor1(8 * anglesum_nonleaf);
  int idx = 0;
  for (int l = 0; l < max_depth; ++l) {
    int so = (int)((pow(8, l) - 1) / 7), inc = (int)((pow(8, l + 1) - 1) / 7);
    float3 mc, cc;
    host_nodes[so].bounding_box().compute_center(mc);
    for (int c = 0; c < 8; ++c) {
      host_nodes[inc + c].bounding_box().compute_center(cc);
      float xd = cc.x - mc.x, yd = cc.y - mc.y, zd = cc.z - mc.z;
      for (int j = 0; j < thn[l]; ++j) {
        float th = -M_PI / 2 + thetastartoffset + M_PI / thn[l] * j;
        for (int kk = 0; kk < phn[l]; ++kk) {
          float ph = 2 * M_PI / phn[l] * kk;
          float dot = xd * (cos(th) * cos(ph)) + yd * (cos(th) * sin(ph)) + zd * sin(th);
          comThr gr = exp(cunit * k0 * dot);
          factor1[idx].x = gr.real();
          factor1[idx].y = gr.imag();
          idx++;
        }
      }
    }
  }
  devicef2vec factor1_d = factor1;

  comThr eta = comThr(eta_re, eta_im);
  Float3 wavedir, Edir, Hdir;
  incident(thetai, phii, mode, wavedir, Edir, Hdir);
  deviceC6vec cur(n);
  computeLocalTangentPlane(x_d0, y_d0, z_d0, nx_d0, ny_d0, nz_d0, cur, wavedir, Edir, Hdir, comThr(1.0, 0.0),
                           eta, Z0, cos(thetai), gaussiansigma, k0, mode);
  field_times_area(cur, a_d0);
  multiply_current_factor(cur, Efactor, Hfactor);

  cudaEventRecord(e1, 0);
  if (tm) tm->setup = ev_ms(e0, e1);
  for (int i = max_depth; i >= 0; i--) {
    if (skip_root && i == 0 && max_depth > 0) break;
    int s = (int)((pow(8, i) - 1) / 7), e = (int)((pow(8, i + 1) - 1) / 7);
    cudaEventRecord(e0, 0);
    if (i == max_depth) {  // sphere.cu:602-658
      int dirs_done = 0;
      for (int it = 0; it < thn[i]; it++) {
        if (max_leaf_dirs > 0 && dirs_done >= max_leaf_dirs) break;
        float th = -M_PI / 2 + thetastartoffset + M_PI / thn[i] * it;
        for (int ip = 0; ip < phn[i]; ip++) {
          if (max_leaf_dirs > 0 && dirs_done >= max_leaf_dirs) break;
          ++dirs_done;
          int dirindex = it * phn[i] + ip;
          float ph = 2 * M_PI / (phn[i]) * ip;
          Float3 dir = Float3(cos(th) * cos(ph), cos(th) * sin(ph), sin(th));
          current_times_green_center(dir, k0, x_d0, y_d0, z_d0, cx_d, cy_d, cz_d, cur, F1[0], F1[1], F1[2], F1[3],
                                     F1[4], F1[5], max_nodes);
          int loopend = (i == 0) ? 1 : (int)nonempty[0].size();
          for (int v = 0; v < loopend; ++v) {
            int nodeindex = (i == 0) ? 0 : nonempty[0][v];
            const Octree_node &nd = host_nodes[nodeindex];
            int b = nd.points_begin(), en = nd.points_end();
            float6 f = thrust::reduce(thrust::device,
                thrust::make_zip_iterator(thrust::make_tuple(F1[0].begin() + b, F1[1].begin() + b, F1[2].begin() + b,
                                                             F1[3].begin() + b, F1[4].begin() + b, F1[5].begin() + b)),
                thrust::make_zip_iterator(thrust::make_tuple(F1[0].begin() + en, F1[1].begin() + en, F1[2].begin() + en,
                                                             F1[3].begin() + en, F1[4].begin() + en, F1[5].begin() + en)),
                zero6, add6());
            int index = v * an[i] + dirindex;
            thrust::fill(thrust::device,
                thrust::make_zip_iterator(thrust::make_tuple(F0[0].begin() + index, F0[1].begin() + index, F0[2].begin() + index,
                                                             F0[3].begin() + index, F0[4].begin() + index, F0[5].begin() + index)),
                thrust::make_zip_iterator(thrust::make_tuple(F0[0].begin() + index + 1, F0[1].begin() + index + 1,
                                                             F0[2].begin() + index + 1, F0[3].begin() + index + 1,
                                                             F0[4].begin() + index + 1, F0[5].begin() + index + 1)),
                f);
          }
        }
      }
      cudaEventRecord(e1, 0);
      if (tm) {
        tm->leaf = ev_ms(e0, e1);
        tm->leaf_dirs = an[i];
        tm->leaf_dirs_done = dirs_done;
      }
    } else {  // sphere.cu:659-884 (ping-pong by parity)
      bool odd = ((max_depth - i) % 2 == 1);
      devicef2vec *dst = odd ? F1 : F0;
      devicef2vec *srcv = odd ? F0 : F1;
      for (int c = 0; c < 6; ++c) thrust::fill(dst[c].begin(), dst[c].end(), zerofloat2);
      int ndn = an[i + 1], ndt = an[i];
      int sofar = 0;
      for (int l = 0; l < i; ++l) sofar += an[l];
      int leveloffset = 8 * sofar;
      int curact = (i > 0) ? (int)nonempty[max_depth - i].size() : 1;
      int kids_total = (int)nonempty[max_depth - i - 1].size(), kids_done = 0;
      for (int v = 0; v < curact; ++v) {
        if (max_children > 0 && kids_done >= max_children) break;
        int nodeindex = (i > 0) ? nonempty[max_depth - i][v] : 0;
        int parentstart = v * ndt;
        const std::vector<int> &childlist = nonempty[max_depth - i - 1];
        for (int c = 0; c < 8; ++c) {
          int truechild = e + (nodeindex - s) * 8 + c;
          for (size_t si = 0; si < childlist.size(); ++si) {
            if (childlist[si] != truechild) continue;
            for (int comp = 0; comp < 6; ++comp)
              copyandinterp(srcv[comp], (int)si, ndn, T1[comp], tmp2, ndt, p_phi[i], p_iphi[i], p_th[i], p_ith[i],
                            phn[i + 1], phn[i], thn[i + 1], thn[i], thn[i + 1], phn[i]);
            ++kids_done;
            translation_compute(T1[0], T1[1], T1[2], T1[3], T1[4], T1[5], factor1_d, 0, ndt, leveloffset + c * ndt);
            int nb = std::ceil(ndt / NT) + 1;
            sumchildren<<<nb, NT>>>(thrust::raw_pointer_cast(T1[0].data()), thrust::raw_pointer_cast(T1[1].data()),
                                    thrust::raw_pointer_cast(T1[2].data()), thrust::raw_pointer_cast(T1[3].data()),
                                    thrust::raw_pointer_cast(T1[4].data()), thrust::raw_pointer_cast(T1[5].data()),
                                    thrust::raw_pointer_cast(dst[0].data()) + parentstart,
                                    thrust::raw_pointer_cast(dst[1].data()) + parentstart,
                                    thrust::raw_pointer_cast(dst[2].data()) + parentstart,
                                    thrust::raw_pointer_cast(dst[3].data()) + parentstart,
                                    thrust::raw_pointer_cast(dst[4].data()) + parentstart,
                                    thrust::raw_pointer_cast(dst[5].data()) + parentstart, ndt);
            break;
          }
        }
      }
      cudaEventRecord(e1, 0);
      if (tm) {
        tm->level[i] = ev_ms(e0, e1);
        tm->children[i] = kids_total;
        tm->children_done[i] = kids_done;
      }
    }
    if (i == 0) {  // sphere.cu:888-932
      cudaEventRecord(e0, 0);
      devicef2vec *fin = ((max_depth - i) % 2 == 1) ? F1 : F0;
      int nb = std::ceil((float)obnum / NT) + 1;
      computeintensity<<<nb, NT>>>(thrust::raw_pointer_cast(scattering.data()), obnum,
                                   thrust::raw_pointer_cast(fin[0].data()), thrust::raw_pointer_cast(fin[1].data()),
                                   thrust::raw_pointer_cast(fin[2].data()), thrust::raw_pointer_cast(fin[3].data()),
                                   thrust::raw_pointer_cast(fin[4].data()), thrust::raw_pointer_cast(fin[5].data()),
                                   thrust::raw_pointer_cast(dirvec_d.data()), Z0);
      checkCudaErrors(cudaGetLastError());
      checkCudaErrors(cudaDeviceSynchronize());
      hostFvec h = scattering;
      cudaEventRecord(e1, 0);
      if (tm) tm->intensity = ev_ms(e0, e1);
      write_bytes(outpath, &h[0], sizeof(float) * obnum);
    }
  }
  for (int i = 0; i < max_depth; ++i) {
    cufftDestroy(p_phi[i]); cufftDestroy(p_iphi[i]); cufftDestroy(p_th[i]); cufftDestroy(p_ith[i]);
  }
  return 0;
}

// util/geometry.h:76-179 (host code): height field -> samples, written as
// float32 [7][n] (x, y, z, nx, ny, nz, area).  Runs without a GPU.
static int cmd_heightfield(char **a) {
  const char *path = a[0];
  int numel = atoi(a[1]), numelvert = atoi(a[2]);
  float period = (float)atof(a[3]), unitz = (float)atof(a[4]);
  int start = atoi(a[5]), end = atoi(a[6]);
  const char *outpath = a[7];
  std::vector<float> h = read_f32(path, (size_t)2 * numel * numelvert);
  int n = (end - start + 1) * numelvert;
  hostFvec x(n), y(n), z(n), area(n), nx(n), ny(n), nz(n);
  set_sourcepoint(0.f, 0.f, period, unitz, x, y, z, area, nx, ny, nz, numel, numelvert, h.data(), start, end);
  std::vector<float> out((size_t)7 * n);
  const hostFvec *cols[7] = {&x, &y, &z, &nx, &ny, &nz, &area};
  for (int k = 0; k < 7; ++k)
    for (int i = 0; i < n; ++i) out[(size_t)k * n + i] = (*cols[k])[i];
  write_bytes(outpath, out.data(), sizeof(float) * out.size());
  return 0;
}

// util/fields.h:206-234 (average_cpu, host code): float32 [nth_in][nph_in]
// -> [nth_out][nph_out].  Runs without a GPU.
static int cmd_average(char **a) {
  const char *path = a[0];
  int nth_in = atoi(a[1]), nph_in = atoi(a[2]), nth_out = atoi(a[3]), nph_out = atoi(a[4]);
  const char *outpath = a[5];
  std::vector<float> v = read_f32(path, (size_t)nth_in * nph_in);
  hostFvec in(v.begin(), v.end()), out((size_t)nth_out * nph_out, 0.f);
  average_cpu(in, out, nth_out, nth_in, nph_out, nph_in);
  std::vector<float> o(out.begin(), out.end());
  write_bytes(outpath, o.data(), sizeof(float) * o.size());
  return 0;
}

int main(int argc, char **argv) {
  if (argc < 2) { fprintf(stderr, "usage: ref_harness currents|interp|octree|solve|heightfield|average ...\n"); return 2; }
  std::string c = argv[1];
  if (c == "currents" && argc >= 12) return cmd_currents(argv + 2);
  if (c == "interp" && argc >= 8) return cmd_interp(argv + 2);
  if (c == "octree" && argc >= 12) return cmd_octree(argv + 2);
  if (c == "solve" && argc >= 12) return cmd_solve(argv + 2);
  if (c == "time" && argc >= 12) return cmd_time(argv + 2, argc - 2);
  if (c == "heightfield" && argc >= 10) return cmd_heightfield(argv + 2);
  if (c == "average" && argc >= 8) return cmd_average(argv + 2);
  fprintf(stderr, "bad arguments\n");
  return 2;
}
