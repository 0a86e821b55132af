// po_solver.cu -- host orchestration of the PO solve and the C ABI.
//
// One call of po_solve does what the reference's driver main() does from the
// octree build to the intensity write (compareMie/sphere.cu:212-936,
// fibersim/treePO.cu:230-961), for every wavelength, incidence and
// polarisation at once:
//   geometry (H2D if host) -> octree (po_octree.cu) -> sorted geometry
//   depth 0 : currents -> direct sum (FP32 tiles or FP64) -> intensity
//   depth d : leaf sums (currents fused) -> for each level: row FFTs, column
//             FFTs + translation + child sum -> intensity of the root
// All work is ordered on the caller's stream; the only host synchronisation
// is the read-back of the per-level node counts after the octree build.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <set>
#include <string>
#include <vector>

#include "po_common.cuh"
#include "po_internal.h"
#include "po_kernels.h"

namespace wavepo {

thread_local int64_t g_launch_count = 0;
static thread_local std::string g_last_error = "";

void set_error(const std::string &msg) { g_last_error = msg; }
po_status fail(po_status s, const std::string &msg) {
  g_last_error = msg;
  return s;
}
po_status cuda_fail(cudaError_t e, const char *what) {
  g_last_error = std::string("CUDA error ") + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ") in " + what;
  return e == cudaErrorMemoryAllocation ? PO_ERR_OUT_OF_MEMORY : PO_ERR_CUDA;
}

namespace {

struct DevBuf {
  void *p = nullptr;
  size_t bytes = 0;
  po_status ensure(size_t b) {
    if (b <= bytes && p) return PO_OK;
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    cudaError_t e = cudaMalloc(&p, b ? b : 256);
    if (e != cudaSuccess) {
      p = nullptr;
      return cuda_fail(e, "cudaMalloc(workspace)");
    }
    bytes = b ? b : 256;
    return PO_OK;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  template <typename T>
  T *as() const { return (T *)p; }
};

__global__ void k_leaf_centers(const uint32_t *__restrict__ prefix, int64_t count, int depth, double3 lo0,
                               double3 hi0, double *__restrict__ out) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= count) return;
  uint32_t key = prefix[i];
  double lo[3] = {lo0.x, lo0.y, lo0.z}, hi[3] = {hi0.x, hi0.y, hi0.z};
  for (int l = 1; l <= depth; ++l) {
    uint32_t o = (key >> (3 * (depth - l))) & 7u;
    double m[3] = {0.5 * (lo[0] + hi[0]), 0.5 * (lo[1] + hi[1]), 0.5 * (lo[2] + hi[2])};
    if (o & 1u) lo[0] = m[0]; else hi[0] = m[0];
    if (o & 2u) hi[1] = m[1]; else lo[1] = m[1];
    if (o & 4u) hi[2] = m[2]; else lo[2] = m[2];
  }
  out[3 * i] = 0.5 * (lo[0] + hi[0]);
  out[3 * i + 1] = 0.5 * (lo[1] + hi[1]);
  out[3 * i + 2] = 0.5 * (lo[2] + hi[2]);
}

std::vector<float4> host_dirs_f4(int T, int Phi, int nth) {
  std::vector<float4> v((size_t)T * Phi);
  for (int it = 0; it < T; ++it)
    for (int ip = 0; ip < Phi; ++ip) {
      double s[3];
      grid_direction(it, ip, nth, Phi, s);
      v[(size_t)it * Phi + ip] = make_float4((float)s[0], (float)s[1], (float)s[2], 0.f);
    }
  return v;
}

std::vector<double> host_dirs_d(int T, int Phi, int nth) {
  std::vector<double> v((size_t)T * Phi * 3);
  for (int it = 0; it < T; ++it)
    for (int ip = 0; ip < Phi; ++ip) grid_direction(it, ip, nth, Phi, &v[((size_t)it * Phi + ip) * 3]);
  return v;
}

int ceil_div(int a, int b) { return (a + b - 1) / b; }

// smallest n' >= n with no prime factor above 7 (and even if requested)
int smooth_at_least(int n, bool even) {
  for (int m = std::max(n, 1);; ++m) {
    if (even && (m % 2)) continue;
    int k = m;
    for (int p : {2, 3, 5, 7})
      while (k % p == 0) k /= p;
    if (k == 1) return m;
  }
}

}  // namespace

// Kernel attributes are per device; set them before the first launch on a
// device (and so before any stream capture of engine launches).
po_status init_device_attributes(int dev) {
  static std::mutex mu;
  static std::set<int> done;
  std::lock_guard<std::mutex> lock(mu);
  if (done.count(dev)) return PO_OK;
  int smem = 0;
  PO_CUDA(cudaDeviceGetAttribute(&smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  PO_TRY(init_interp_mma_attributes(smem));
  PO_TRY(init_fft_attributes(smem));
  PO_TRY(init_leaf_mma_attributes());
  PO_TRY(init_point_adjoint_mma_attributes());
  PO_TRY(init_theta_tc_attributes());
  PO_TRY(init_rows_tc_attributes());
  PO_TRY(init_leaf_tc_attributes());
  done.insert(dev);
  return PO_OK;
}

}  // namespace wavepo

using namespace wavepo;

struct po_ctx {
  po_config cfg;
  int device = 0;
  int sm_count = 152;
  int depth = 0;
  int cover = 2;
  int mt = 1, mp = 1;
  int nth[PO_MAX_DEPTH + 1];  // samples over pi per level (root: output * mt)
  int T[PO_MAX_DEPTH + 1];    // theta transform length per level (cover * nth)
  int R[PO_MAX_DEPTH + 1];    // theta rows stored per level (mirror: nth + 1, else T)
  int Phi[PO_MAX_DEPTH + 1];
  int mirror = 0;             // double cover stored as rows 0..nth (see k_interp_cols)
  bool tensor_theta = false;  // some level interpolates on the tensor cores (po_interp_mma.cu)
  bool tt_level[PO_MAX_DEPTH] = {};  // level l (parent) interpolates on the tensor cores
  size_t amat_off[PO_MAX_DEPTH] = {};
  int amat_kp[PO_MAX_DEPTH] = {};
  size_t bmat_off[PO_MAX_DEPTH] = {};
  int bmat_kp[PO_MAX_DEPTH] = {};
  DevBuf amat, bmat;
  DevBuf dir_trig;  // per level: (cos, sin) of the grid's theta rows, then of its phi columns
  DevBuf out_dirs;  // output grid directions (float4), for the intensity and its adjoint
  // tcgen05 theta pass of the levels with more than 128 parent rows (po_theta_tc.cu)
  bool tc_level[PO_MAX_DEPTH] = {};
  int tc_kr[PO_MAX_DEPTH] = {};       // child rows padded to 16 (the K of its products)
  size_t tc_off[PO_MAX_DEPTH] = {};   // byte offset of the level's theta chunks in tc_amat
  DevBuf tc_amat, tc_err;
  // tcgen05 phi pass feeding those levels (po_rows_tc.cu): phi tiles per level
  bool rt_level[PO_MAX_DEPTH] = {};
  int rt_ntn[PO_MAX_DEPTH] = {}, rt_nnt[PO_MAX_DEPTH] = {};
  size_t rt_off[PO_MAX_DEPTH] = {}, rt_bytes[PO_MAX_DEPTH] = {};
  DevBuf rt_bmat;
  size_t trig_off[PO_MAX_DEPTH] = {};
  // transposed level matrices of the adjoint (built on the first po_grad)
  bool adj_ready = false;
  size_t amat_adj_off[PO_MAX_DEPTH] = {}, bmat_adj_off[PO_MAX_DEPTH] = {};
  int amat_adj_kp[PO_MAX_DEPTH] = {}, bmat_adj_kp[PO_MAX_DEPTH] = {};
  DevBuf amat_adj, bmat_adj, slots64, grad_acc, chunk_begin, center0;
  std::map<int, int> tw_offset;
  DevBuf twiddles;
  DevBuf geom_in, geom_sorted, octree_ws, leaf_ctr, dirs, dirs_d, trans, levelA, levelB, mid, slots, kvals, out,
      cur, partial, tile_ctr;
  // tcgen05 leaf sums (po_leaf_tc.cu): per-leaf chunk bases, chunk -> leaf, operand scratch
  DevBuf leaf_kc0, leaf_chunk, leaf_bop, leaf_uop;
  cudaEvent_t ev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  // per kernel class: [0..1] leaf/direct kernel, then rows and cols per level
  cudaEvent_t kev[2 + 4 * PO_MAX_DEPTH] = {};
};

extern "C" {

const char *po_version(void) { return "wavepo 0.1 (sm_103a)"; }

const char *po_status_string(po_status s) {
  switch (s) {
    case PO_OK: return "ok";
    case PO_ERR_INVALID_ARGUMENT: return "invalid argument";
    case PO_ERR_CUDA: return "CUDA error";
    case PO_ERR_OUT_OF_MEMORY: return "out of device memory";
    case PO_ERR_UNSUPPORTED: return "unsupported configuration";
    case PO_ERR_TIMEOUT: return "device wait timed out";
    case PO_ERR_INTERNAL: return "internal error";
  }
  return "unknown status";
}

const char *po_last_error(void) {
  static thread_local std::string copy;
  copy = g_last_error;
  return copy.c_str();
}

po_status po_config_init(po_config *cfg, int max_depth, int n_theta_out, int n_phi_out, const float box_min[3],
                         const float box_max[3], double theta_extent, double phi_extent, double ratio, double beta,
                         double lambda_min) {
  if (!cfg || !box_min || !box_max) return fail(PO_ERR_INVALID_ARGUMENT, "null argument");
  if (max_depth < 0 || max_depth > PO_MAX_DEPTH) return fail(PO_ERR_INVALID_ARGUMENT, "max_depth out of range");
  if (n_theta_out <= 0 || n_phi_out <= 0) return fail(PO_ERR_INVALID_ARGUMENT, "output grid must be positive");
  if (!(lambda_min > 0) || !(ratio > 0)) return fail(PO_ERR_INVALID_ARGUMENT, "lambda_min and ratio must be > 0");
  std::memset(cfg, 0, sizeof(*cfg));
  cfg->max_depth = max_depth;
  cfg->n_theta[0] = n_theta_out;
  cfg->n_phi[0] = n_phi_out;
  const double kmin = kTwoPi / lambda_min;
  for (int i = 1; i <= max_depth; ++i) {
    // compareMie/sphere.cu:346-350: d is a float
    float dth = (float)(std::pow(0.5, i) * (double)((float)theta_extent * (float)ratio));
    float dph = (float)(std::pow(0.5, i) * (double)((float)phi_extent * (float)ratio));
    double a = kmin * dth, b = kmin * dph;
    cfg->n_theta[i] = (int)std::ceil(a + beta * std::pow(a, 1.0 / 3.0));
    cfg->n_phi[i] = (int)std::ceil(b + beta * std::pow(b, 1.0 / 3.0));
  }
  for (int a = 0; a < 3; ++a) {
    cfg->box_min[a] = box_min[a];
    cfg->box_max[a] = box_max[a];
  }
  cfg->precision = PO_PREC_FP32;
  cfg->theta_mode = PO_THETA_DOUBLE_COVER;
  cfg->nyquist_quirk = 1;
  cfg->distance = 1.0;
  cfg->interp_method = PO_INTERP_TENSOR;
  return PO_OK;
}

// The tcgen05 theta pass works on 128-row tiles of the parent; it serves the
// levels whose rows fill at least 60% of their tiles, the others keep the
// warp-level kernel, whose 16-row tiles waste fewer rows (ellipsoid workload:
// the 109-, 201- and 361-row levels on tcgen05, 64 rows and fewer not; fiber
// workload: every level from 97 rows up).  Its column chunks of 64 mirror
// pairs are padded too, but even the fiber's 97 x 84 level (66% of its
// columns) runs 1.4x faster on tcgen05 than on the warp-level kernel.
static bool theta_on_tcgen05(int rows, int phi) {
  (void)phi;
  return rows * 5 >= 3 * 128 * ((rows + 127) / 128);
}

po_status po_create(po_ctx **out, const po_config *cfg) {
  if (!out || !cfg) return fail(PO_ERR_INVALID_ARGUMENT, "null argument");
  *out = nullptr;
  const int d = cfg->max_depth;
  if (d < 0 || d > PO_MAX_DEPTH) return fail(PO_ERR_INVALID_ARGUMENT, "max_depth out of range");
  for (int l = 0; l <= d; ++l)
    if (cfg->n_theta[l] <= 0 || cfg->n_phi[l] <= 0)
      return fail(PO_ERR_INVALID_ARGUMENT, "every level needs positive n_theta and n_phi");
  for (int l = 1; l < d; ++l)
    if (cfg->n_theta[l] < cfg->n_theta[l + 1] || cfg->n_phi[l] < cfg->n_phi[l + 1])
      return fail(PO_ERR_INVALID_ARGUMENT, "level grids must not grow with depth (the interpolation only upsamples)");
  for (int a = 0; a < 3; ++a)
    if (!(cfg->box_max[a] > cfg->box_min[a])) return fail(PO_ERR_INVALID_ARGUMENT, "empty bounding box");
  if (cfg->precision < 0 || cfg->precision > 3) return fail(PO_ERR_INVALID_ARGUMENT, "unknown precision");
  if (cfg->precision == PO_PREC_FP64 && d != 0)
    return fail(PO_ERR_UNSUPPORTED, "the plain FP64 path is the depth-0 direct sum");
  if (cfg->precision == PO_PREC_SPLIT_FP16)
    return fail(PO_ERR_UNSUPPORTED,
                "split FP16 needs per-tile scaling of the currents (FP16 range); use PO_PREC_SPLIT_BF16");
  if (cfg->theta_mode != PO_THETA_DOUBLE_COVER && cfg->theta_mode != PO_THETA_REFERENCE)
    return fail(PO_ERR_INVALID_ARGUMENT, "unknown theta mode");
  if (!(cfg->distance > 0)) return fail(PO_ERR_INVALID_ARGUMENT, "distance must be > 0");
  if (cfg->interp_method != PO_INTERP_FFT && cfg->interp_method != PO_INTERP_TENSOR)
    return fail(PO_ERR_INVALID_ARGUMENT, "unknown interpolation method");
  if (cfg->interp_tile != 0 && cfg->interp_tile != 8 && cfg->interp_tile != 16)
    return fail(PO_ERR_INVALID_ARGUMENT, "interp_tile must be 0, 8 or 16");
  if (cfg->leaf_kernel < PO_LEAF_AUTO || cfg->leaf_kernel > PO_LEAF_TCGEN05)
    return fail(PO_ERR_INVALID_ARGUMENT, "unknown leaf kernel");
  if (cfg->leaf_kernel != PO_LEAF_AUTO && (cfg->precision != PO_PREC_SPLIT_BF16 || d == 0))
    return fail(PO_ERR_INVALID_ARGUMENT, "the leaf kernel choice applies to split-BF16 tree solves");
  if (cfg->leaf_slots != 0 && (cfg->leaf_slots < 8 || cfg->leaf_slots > kLeafTcMaxSlots || cfg->leaf_slots % 8))
    return fail(PO_ERR_INVALID_ARGUMENT, "leaf_slots must be 0 or a multiple of 8 up to 64");
  int dev = 0;
  PO_CUDA(cudaGetDevice(&dev));
  PO_TRY(init_device_attributes(dev));
  po_ctx *c = new po_ctx();
  c->cfg = *cfg;
  c->device = dev;
  cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, dev);
  c->depth = d;
  c->cover = cfg->theta_mode == PO_THETA_DOUBLE_COVER ? 2 : 1;
  c->mt = c->mp = 1;
  c->mirror = (d >= 1 && c->cover == 2) ? 1 : 0;
  int lvl_th[PO_MAX_DEPTH + 1], lvl_ph[PO_MAX_DEPTH + 1];
  for (int l = 0; l <= d; ++l) {
    lvl_th[l] = cfg->n_theta[l];
    lvl_ph[l] = cfg->n_phi[l];
    // double cover: inner levels are rounded up to FFT-friendly sizes (7-smooth,
    // even in phi so that phi + pi is a grid line); more samples never lower
    // the accuracy of the interpolation
    if (c->mirror && l >= 1) {
      lvl_th[l] = smooth_at_least(lvl_th[l], false);
      lvl_ph[l] = smooth_at_least(lvl_ph[l], true);
    }
  }
  // The root grid is the output grid times (mt, mp), so that the FFT
  // interpolation only upsamples and the output is every mt-th row and mp-th
  // column of the root (sphere.cu's copy of the root pattern).  The matrix
  // passes of the double cover evaluate the trigonometric interpolant at any
  // position, so they evaluate it at the output grid directly: the same values
  // (row r of the output is at r / T on both grids) for 1 / (mt mp) of the
  // root's work.
  const bool direct_root = c->mirror && cfg->interp_method == PO_INTERP_TENSOR && lvl_ph[0] % 2 == 0;
  if (d >= 1 && !direct_root) {
    c->mt = ceil_div(lvl_th[1], lvl_th[0]);
    c->mp = ceil_div(lvl_ph[1], lvl_ph[0]);
    if (c->mirror && (c->mp * lvl_ph[0]) % 2) ++c->mp;
  }
  for (int l = 0; l <= d; ++l) {
    c->nth[l] = l == 0 ? lvl_th[0] * c->mt : lvl_th[l];
    c->Phi[l] = l == 0 ? lvl_ph[0] * c->mp : lvl_ph[l];
    c->T[l] = (d == 0) ? cfg->n_theta[0] : c->cover * c->nth[l];
    c->R[l] = c->mirror ? c->nth[l] + 1 : c->T[l];
  }
  // twiddle tables for every transform length of the level chain
  std::vector<int> lens;
  for (int l = 0; l < d; ++l) {
    lens.push_back(c->Phi[l + 1]);
    lens.push_back(c->Phi[l]);
    lens.push_back(c->T[l + 1]);
    lens.push_back(c->T[l]);
  }
  std::sort(lens.begin(), lens.end());
  lens.erase(std::unique(lens.begin(), lens.end()), lens.end());
  int total = 0;
  for (int n : lens) {
    c->tw_offset[n] = total;
    total += n;
  }
  po_status s = c->twiddles.ensure(sizeof(float2) * (size_t)std::max(total, 1));
  if (s != PO_OK) { po_destroy(c); return s; }
  for (int n : lens) {
    s = launch_twiddles(n, c->twiddles.as<float2>() + c->tw_offset[n], 0);
    if (s != PO_OK) { po_destroy(c); return s; }
  }
  // output-grid directions
  s = c->out_dirs.ensure(sizeof(float4) * std::max<size_t>((size_t)cfg->n_theta[0] * cfg->n_phi[0], 1));
  if (s == PO_OK) s = launch_out_dirs(cfg->n_theta[0], cfg->n_phi[0], c->out_dirs.as<float4>(), 0);
  if (s != PO_OK) { po_destroy(c); return s; }
  // direction factors of every parent level (translation tables)
  {
    size_t n_trig = 0;
    for (int l = 0; l < d; ++l) {
      c->trig_off[l] = n_trig;
      n_trig += (size_t)c->R[l] + c->Phi[l];
    }
    s = c->dir_trig.ensure(sizeof(double2) * std::max<size_t>(n_trig, 1));
    for (int l = 0; l < d && s == PO_OK; ++l)
      s = launch_dir_trig(c->nth[l], c->R[l], c->Phi[l], c->dir_trig.as<double2>() + c->trig_off[l], 0);
    if (s != PO_OK) { po_destroy(c); return s; }
  }
  for (auto &e : c->ev) {
    if (cudaEventCreate(&e) != cudaSuccess) { po_destroy(c); return fail(PO_ERR_CUDA, "cudaEventCreate"); }
  }
  for (auto &e : c->kev) {
    if (cudaEventCreate(&e) != cudaSuccess) { po_destroy(c); return fail(PO_ERR_CUDA, "cudaEventCreate"); }
  }
  // constant theta-interpolation matrices of every level (tensor-core path)
  // Double cover: every level.  Reference theta mode: the levels whose maps are
  // real and column-independent -- not where the Nyquist quirk of
  // interpolation.h:66 reaches a parent column (columns past it keep the
  // unsplit Nyquist bin: a complex, column-dependent map) and not between
  // equal sizes (the reference halves the Nyquist bin there); the other levels
  // keep the FFTs.  An odd parent phi grid pairs column j with j + (Phi+1)/2
  // (one phantom partner) on the warp-level theta pass.
  for (int l = 0; l < d; ++l) {
    if (cfg->interp_method != PO_INTERP_TENSOR) break;
    if (c->mirror) {
      c->tt_level[l] = true;
    } else {
      const bool quirk = cfg->nyquist_quirk && c->T[l + 1] % 2 == 0 && c->Phi[l] > 256 * (c->T[l + 1] / 256 + 1);
      c->tt_level[l] = !quirk && c->T[l + 1] != c->T[l] && c->Phi[l + 1] != c->Phi[l];
    }
    c->tensor_theta = c->tensor_theta || c->tt_level[l];
  }
  if (c->tensor_theta) {
    std::vector<uint32_t> all, one;
    for (int l = 0; l < d; ++l) {
      const int Rc2 = c->R[l + 1] + (c->R[l + 1] & 1);
      c->amat_kp[l] = (Rc2 + 15) / 16 * 16;
      build_theta_matrix(c->T[l + 1], c->T[l], c->R[l + 1], c->R[l], c->amat_kp[l], one, c->mirror != 0);
      c->amat_off[l] = all.size();
      all.insert(all.end(), one.begin(), one.end());
    }
    // theta chunks of the levels on the tcgen05 pass
    {
      std::vector<uint16_t> tall, tone;
      std::vector<double> Mp, Mm;
      for (int l = 0; l < d; ++l) {
        if (!c->tt_level[l] || c->Phi[l] % 2 || !theta_on_tcgen05(c->R[l], c->Phi[l])) continue;
        c->tc_level[l] = true;
        c->tc_kr[l] = (c->R[l + 1] + 15) / 16 * 16;
        theta_plus_minus(c->T[l + 1], c->T[l], c->R[l + 1], c->R[l], c->tc_kr[l], Mp, Mm, c->mirror != 0);
        build_theta_tc(Mp, Mm, c->R[l], c->R[l + 1], c->tc_kr[l], c->tc_kr[l], tone);
        c->tc_off[l] = tall.size() * sizeof(uint16_t);
        tall.insert(tall.end(), tone.begin(), tone.end());
      }
      // the phi pass of those levels on tcgen05 where its phi tile fits shared memory
      std::vector<uint16_t> rall, rone;
      for (int l = 0; l < d; ++l) {
        if (!c->tc_level[l] || !rows_tc_plan(c->Phi[l + 1], c->Phi[l], c->rt_ntn[l], c->rt_nnt[l])) continue;
        c->rt_level[l] = true;
        build_phi_tc(c->Phi[l + 1], c->Phi[l], (c->Phi[l + 1] + 15) / 16 * 16, c->rt_ntn[l], c->rt_nnt[l], rone);
        c->rt_off[l] = rall.size() * sizeof(uint16_t);
        c->rt_bytes[l] = rone.size() * sizeof(uint16_t);
        rall.insert(rall.end(), rone.begin(), rone.end());
      }
      s = c->rt_bmat.ensure(std::max<size_t>(rall.size() * sizeof(uint16_t), 16));
      if (s == PO_OK && !rall.empty() &&
          cudaMemcpy(c->rt_bmat.p, rall.data(), rall.size() * sizeof(uint16_t), cudaMemcpyHostToDevice) != cudaSuccess)
        s = fail(PO_ERR_CUDA, "upload of the tcgen05 phi tiles");
      if (s != PO_OK) { po_destroy(c); return s; }
      s = c->tc_amat.ensure(std::max<size_t>(tall.size() * sizeof(uint16_t), 16));
      if (s == PO_OK) s = c->tc_err.ensure(sizeof(int));
      if (s == PO_OK && !tall.empty() &&
          cudaMemcpy(c->tc_amat.p, tall.data(), tall.size() * sizeof(uint16_t), cudaMemcpyHostToDevice) != cudaSuccess)
        s = fail(PO_ERR_CUDA, "upload of the tcgen05 theta matrices");
      if (s == PO_OK && cudaMemset(c->tc_err.p, 0, sizeof(int)) != cudaSuccess) s = fail(PO_ERR_CUDA, "cudaMemset");
      if (s != PO_OK) { po_destroy(c); return s; }
    }
    s = c->amat.ensure(sizeof(uint32_t) * std::max<size_t>(all.size(), 1));
    if (s == PO_OK && !all.empty() &&
        cudaMemcpy(c->amat.p, all.data(), sizeof(uint32_t) * all.size(), cudaMemcpyHostToDevice) != cudaSuccess)
      s = fail(PO_ERR_CUDA, "upload of the interpolation matrices");
    if (s != PO_OK) { po_destroy(c); return s; }
    // phi matrices (row pass)
    all.clear();
    for (int l = 0; l < d; ++l) {
      c->bmat_kp[l] = (c->Phi[l + 1] + 15) / 16 * 16;
      build_phi_matrix(c->Phi[l + 1], c->Phi[l], c->bmat_kp[l], one);
      c->bmat_off[l] = all.size();
      all.insert(all.end(), one.begin(), one.end());
    }
    s = c->bmat.ensure(sizeof(uint32_t) * std::max<size_t>(all.size(), 1));
    if (s == PO_OK && !all.empty() &&
        cudaMemcpy(c->bmat.p, all.data(), sizeof(uint32_t) * all.size(), cudaMemcpyHostToDevice) != cudaSuccess)
      s = fail(PO_ERR_CUDA, "upload of the interpolation matrices");
    if (s != PO_OK) { po_destroy(c); return s; }
  }
  // error word of the bounded device waits (tcgen05 passes and leaf sums)
  if (!c->tc_err.p) {
    s = c->tc_err.ensure(sizeof(int));
    if (s == PO_OK && cudaMemset(c->tc_err.p, 0, sizeof(int)) != cudaSuccess) s = fail(PO_ERR_CUDA, "cudaMemset");
    if (s != PO_OK) { po_destroy(c); return s; }
  }
  if (cudaDeviceSynchronize() != cudaSuccess) { po_destroy(c); return fail(PO_ERR_CUDA, "set-up kernels failed"); }
  *out = c;
  return PO_OK;
}

po_status po_destroy(po_ctx *c) {
  if (!c) return PO_OK;
  for (DevBuf *b : {&c->twiddles, &c->geom_in, &c->geom_sorted, &c->octree_ws, &c->leaf_ctr, &c->dirs, &c->dirs_d,
                    &c->trans, &c->levelA, &c->levelB, &c->mid, &c->slots, &c->kvals, &c->out, &c->cur, &c->partial,
                    &c->tile_ctr, &c->amat, &c->bmat, &c->amat_adj, &c->bmat_adj, &c->slots64, &c->grad_acc,
                    &c->chunk_begin, &c->center0, &c->dir_trig, &c->out_dirs, &c->tc_amat, &c->tc_err, &c->rt_bmat,
                    &c->leaf_kc0, &c->leaf_chunk, &c->leaf_bop, &c->leaf_uop})
    b->release();
  for (auto &e : c->ev)
    if (e) cudaEventDestroy(e);
  for (auto &e : c->kev)
    if (e) cudaEventDestroy(e);
  delete c;
  return PO_OK;
}

// A contiguous range of pattern slots processed together: either whole
// wavelengths (gc == G) or a run of the slots of one wavelength.
struct SlotChunk {
  int s0, ns;  // first slot, slot count
  int l0, nl;  // first wavelength, wavelength count
  int gc;      // slots per wavelength inside the chunk
};

// Contiguous slot ranges of at most chunk_slots slots: whole wavelengths when
// one fits, else runs of one wavelength's incidences.  The ranges are as even
// as the count allows (64 incidences under a cap of 27: 22 + 21 + 21, not
// 27 + 27 + 10), so that no chunk leaves the upper levels' launches short of
// work; the first range is the largest (the buffers are sized by it).
static std::vector<SlotChunk> plan_chunks(int L, int G, int chunk_slots) {
  std::vector<SlotChunk> v;
  if (chunk_slots >= G) {
    const int cap = chunk_slots / G, n = (L + cap - 1) / cap;  // wavelengths per chunk, chunks
    for (int i = 0, l0 = 0; i < n; ++i) {
      const int nl = (L - l0 + n - i - 1) / (n - i);  // the remaining wavelengths over the remaining chunks
      v.push_back({l0 * G, nl * G, l0, nl, G});
      l0 += nl;
    }
  } else {
    const int n = (G + chunk_slots - 1) / chunk_slots;
    for (int l = 0; l < L; ++l)
      for (int i = 0, g0 = 0; i < n; ++i) {
        const int ns = (G - g0 + n - i - 1) / (n - i);
        v.push_back({l * G + g0, ns, l, 1, ns});
        g0 += ns;
      }
  }
  return v;
}

static int chunk_slot_count(int64_t budget, double bytes_per_slot, int S) {
  if (!(bytes_per_slot > 0)) return S;
  double c = std::floor((double)budget / bytes_per_slot);
  return (int)std::max(1.0, std::min((double)S, c));
}

// Transposed level matrices for the adjoint aggregation (double cover and
// tensor-core interpolation only).
static po_status ensure_adjoint_matrices(po_ctx *c) {
  if (c->adj_ready) return PO_OK;
  const int d = c->depth;
  std::vector<uint32_t> all, one, ball, bone;
  for (int l = 0; l < d; ++l) {
    c->amat_adj_kp[l] = (c->R[l] + 15) / 16 * 16;
    build_theta_matrix_adj(c->T[l + 1], c->T[l], c->R[l + 1], c->R[l], c->amat_adj_kp[l], one);
    c->amat_adj_off[l] = all.size();
    all.insert(all.end(), one.begin(), one.end());
    c->bmat_adj_kp[l] = (c->Phi[l] + 15) / 16 * 16;
    build_phi_matrix_adj(c->Phi[l + 1], c->Phi[l], c->bmat_adj_kp[l], bone);
    c->bmat_adj_off[l] = ball.size();
    ball.insert(ball.end(), bone.begin(), bone.end());
  }
  PO_TRY(c->amat_adj.ensure(sizeof(uint32_t) * std::max<size_t>(all.size(), 1)));
  PO_TRY(c->bmat_adj.ensure(sizeof(uint32_t) * std::max<size_t>(ball.size(), 1)));
  if (!all.empty()) PO_CUDA(cudaMemcpy(c->amat_adj.p, all.data(), sizeof(uint32_t) * all.size(), cudaMemcpyHostToDevice));
  if (!ball.empty())
    PO_CUDA(cudaMemcpy(c->bmat_adj.p, ball.data(), sizeof(uint32_t) * ball.size(), cudaMemcpyHostToDevice));
  c->adj_ready = true;
  return PO_OK;
}

// Adjoint request of po_grad: dL/dI on the output grid and the gradient out
// (both device arrays; NULL for a plain solve).
struct AdjointArgs {
  const float *dl_di = nullptr;  // [S][n_theta][n_phi]
  float *grad = nullptr;         // [7][n]
};

// Everything a solve needs on the device before its patterns are computed:
// built by prepare_solve (allocations, uploads, the octree with its count
// read-back, tables), consumed by enqueue_solve (kernel launches only).
struct SolvePlan {
  int L = 0, G = 0, S = 0;
  int64_t n = 0, nd_out = 0;
  bool fp64 = false, adj = false;
  const float *gin[7] = {};   // input order
  const float *gsc[7] = {};   // octree order
  OctreeBuffers tree;
  int64_t nleaf = 0;
  double c0[3] = {0, 0, 0};
  std::vector<SlotChunk> chunks;
  std::vector<size_t> tr_off;
  int nsplit_max = 1;
  const double *k_lambda = nullptr, *k_slot = nullptr;
  const SlotParams<double> *sp64_dev = nullptr;
  const int32_t *perm_out = nullptr;  // sorted position -> input index of the gradient
  bool leaf_tc = false;               // leaf sums on tcgen05 (po_leaf_tc.cu)
  int leaf_group = kLeafTcMaxSlots;   // slots per pass of the tcgen05 leaf kernel
  int64_t leaf_chunks = 0;            // 16-point chunks over all leaves
};

// Per-kernel-class device times of a solve (CUDA events; requested by a report).
struct SolveTimes {
  double leaf = 0, agg = 0, inten = 0, leafk = 0, rows = 0, cols = 0;
  double rows_l[PO_MAX_DEPTH] = {}, cols_l[PO_MAX_DEPTH] = {};
  double agg_b = 0;
  int n_leaf = 0, n_row = 0, n_col = 0;
  double leaf_pd = 0, rows_b = 0, cols_b = 0;
};

static po_status prepare_solve(po_ctx *c, const po_geometry *g, const po_illum *il, bool adj, cudaStream_t st,
                               SolvePlan &P) {
  const po_config &cfg = c->cfg;
  const int d = c->depth;
  const int64_t n = g->n;
  const int npol = ((il->pol_mask & PO_POL_TM) ? 1 : 0) + ((il->pol_mask & PO_POL_TE) ? 1 : 0);
  const int L = il->n_lambda, I = il->n_inc, G = I * npol, S = L * G;
  const int nth_out = cfg.n_theta[0], nph_out = cfg.n_phi[0];
  const int64_t nd_out = (int64_t)nth_out * nph_out;
  P.L = L;
  P.G = G;
  P.S = S;
  P.n = n;
  P.nd_out = nd_out;
  P.adj = adj;
  P.fp64 = cfg.precision == PO_PREC_FP64;

  int64_t budget = cfg.max_workspace_bytes;
  if (budget <= 0) {
    size_t fr = 0, tot = 0;
    PO_CUDA(cudaMemGetInfo(&fr, &tot));
    budget = (int64_t)(tot / 2);
  }

  // ---- geometry on the device
  if (g->on_device) {
    const float *src[7] = {g->x, g->y, g->z, g->nx, g->ny, g->nz, g->area};
    for (int k = 0; k < 7; ++k) P.gin[k] = src[k];
  } else {
    PO_TRY(c->geom_in.ensure(sizeof(float) * 7 * (size_t)std::max<int64_t>(n, 1)));
    const float *src[7] = {g->x, g->y, g->z, g->nx, g->ny, g->nz, g->area};
    for (int k = 0; k < 7; ++k) {
      float *dst = c->geom_in.as<float>() + (size_t)k * n;
      if (n > 0) PO_CUDA(cudaMemcpyAsync(dst, src[k], sizeof(float) * n, cudaMemcpyHostToDevice, st));
      P.gin[k] = dst;
    }
  }

  // per-slot parameters, slot = (lambda, incidence, polarisation)
  std::vector<double> kl(L), ks(S);
  for (int l = 0; l < L; ++l) kl[l] = kTwoPi / il->lambda_m[l];
  std::vector<SlotParams<float>> sp32;
  std::vector<SlotParams<double>> sp64;
  for (int l = 0; l < L; ++l)
    for (int i = 0; i < I; ++i)
      for (int p = 0; p < 2; ++p) {
        int bit = p == 0 ? PO_POL_TM : PO_POL_TE;
        if (!(il->pol_mask & bit)) continue;
        ks[sp32.size()] = kl[l];
        sp32.push_back(make_slot<float>(il->lambda_m[l], il->theta_i[i], il->phi_i[i], p == 1, il->eta_re,
                                        il->eta_im, il->sigma, cfg.distance, true));
        sp64.push_back(make_slot<double>(il->lambda_m[l], il->theta_i[i], il->phi_i[i], p == 1, il->eta_re,
                                         il->eta_im, il->sigma, cfg.distance, true));
      }
  PO_TRY(c->slots.ensure(std::max(sizeof(SlotParams<float>), sizeof(SlotParams<double>)) * S));
  PO_TRY(c->kvals.ensure(sizeof(double) * (L + S)));
  // the host vectors go out of scope: these copies complete before returning (synchronous)
  PO_CUDA(cudaMemcpyAsync(c->kvals.as<double>(), kl.data(), sizeof(double) * L, cudaMemcpyHostToDevice, st));
  PO_CUDA(cudaMemcpyAsync(c->kvals.as<double>() + L, ks.data(), sizeof(double) * S, cudaMemcpyHostToDevice, st));
  if (P.fp64)
    PO_CUDA(cudaMemcpyAsync(c->slots.p, sp64.data(), sizeof(SlotParams<double>) * S, cudaMemcpyHostToDevice, st));
  else
    PO_CUDA(cudaMemcpyAsync(c->slots.p, sp32.data(), sizeof(SlotParams<float>) * S, cudaMemcpyHostToDevice, st));
  if (adj) {
    PO_TRY(c->slots64.ensure(sizeof(SlotParams<double>) * S));
    PO_CUDA(cudaMemcpyAsync(c->slots64.p, sp64.data(), sizeof(SlotParams<double>) * S, cudaMemcpyHostToDevice, st));
    P.sp64_dev = c->slots64.as<SlotParams<double>>();
    PO_TRY(c->grad_acc.ensure(sizeof(double) * 7 * (size_t)std::max<int64_t>(n, 1)));
    PO_TRY(c->chunk_begin.ensure(sizeof(int32_t) * (size_t)((n + 31) / 32 + 1)));
    PO_TRY(c->center0.ensure(sizeof(double) * 3));
  }
  P.k_lambda = c->kvals.as<double>();
  P.k_slot = P.k_lambda + L;

  // root centre (tree.h:116-120, float box)
  for (int a = 0; a < 3; ++a) P.c0[a] = (double)(0.5f * (cfg.box_min[a] + cfg.box_max[a]));
  if (adj) {
    PO_CUDA(cudaMemcpyAsync(c->center0.p, P.c0, sizeof(P.c0), cudaMemcpyHostToDevice, st));
    // depth-0 point adjoint: the points in chunks (32 for the FP64 chain, 128 =
    // one pass of the tensor-core kernel for the FP32 chain) sharing one pattern
    if (n > 0) PO_TRY(launch_chunk_begin(c->chunk_begin.as<int32_t>(), n, P.fp64 ? 32 : 128, st));
  }

  if (P.fp64) {
    // ---- plain FP64 direct sum (the "plain method"): no tree, no sort
    auto splits = [&](int ns) {
      int64_t tiles = (int64_t)ns * ceil_div((int)nd_out, 128);
      int s = (int)std::max<int64_t>(
          1, std::min<int64_t>(64, (c->sm_count * 8 + tiles - 1) / std::max<int64_t>(1, tiles)));
      return (int)std::min<int64_t>(s, std::max<int64_t>(1, n));
    };
    int cs = chunk_slot_count(budget, 96.0 * (double)(n + nd_out * (1 + splits(1))), S);
    cs = chunk_slot_count(budget, 96.0 * (double)(n + nd_out * (1 + splits(cs))), S);
    P.chunks = plan_chunks(L, G, cs);
    const int ns_max = P.chunks.front().ns;
    P.nsplit_max = splits(std::min(ns_max, P.chunks.back().ns));
    PO_TRY(c->cur.ensure(sizeof(double2) * 6 * (size_t)ns_max * std::max<int64_t>(n, 1)));
    std::vector<double> dd = host_dirs_d(nth_out, nph_out, nth_out);
    PO_TRY(c->dirs_d.ensure(sizeof(double) * dd.size()));
    PO_CUDA(cudaMemcpyAsync(c->dirs_d.p, dd.data(), sizeof(double) * dd.size(), cudaMemcpyHostToDevice, st));
    PO_TRY(c->partial.ensure(sizeof(double2) * 6 * (size_t)ns_max * nd_out * P.nsplit_max));
    PO_TRY(c->levelA.ensure(sizeof(double2) * 6 * (size_t)ns_max * nd_out));
    P.perm_out = nullptr;
    PO_CUDA(cudaStreamSynchronize(st));  // host tables above are released on return
    return PO_OK;
  }

  // ---- octree (depth 0 still sorts the points so that direct-sum tiles are compact)
  const int tdepth = d > 0 ? d : 6;
  size_t wsb = octree_workspace_bytes(n, tdepth);
  PO_TRY(c->octree_ws.ensure(wsb));
  PO_TRY(build_octree(P.gin[0], P.gin[1], P.gin[2], n, cfg.box_min, cfg.box_max, tdepth, c->octree_ws.p, wsb, &P.tree,
                      st));
  PO_TRY(c->geom_sorted.ensure(sizeof(float) * 7 * (size_t)std::max<int64_t>(n, 1)));
  float *gs[7];
  for (int k = 0; k < 7; ++k) gs[k] = c->geom_sorted.as<float>() + (size_t)k * n;
  PO_TRY(gather_points(n, P.tree.perm, P.gin, gs, st));
  for (int k = 0; k < 7; ++k) P.gsc[k] = gs[k];
  P.perm_out = P.tree.perm;
  if (d == 0) {
    std::vector<float4> df = host_dirs_f4(nth_out, nph_out, nth_out);
    std::vector<double> dd = host_dirs_d(nth_out, nph_out, nth_out);
    PO_TRY(c->dirs.ensure(sizeof(float4) * df.size()));
    PO_TRY(c->dirs_d.ensure(sizeof(double) * dd.size()));
    PO_CUDA(cudaMemcpyAsync(c->dirs.p, df.data(), sizeof(float4) * df.size(), cudaMemcpyHostToDevice, st));
    PO_CUDA(cudaMemcpyAsync(c->dirs_d.p, dd.data(), sizeof(double) * dd.size(), cudaMemcpyHostToDevice, st));
    int cs = chunk_slot_count(
        budget, 48.0 * (double)(n + nd_out * (1 + direct_splits(n, (int)nd_out, 1, c->sm_count))), S);
    P.chunks = plan_chunks(L, G, cs);
    const int ns_max = P.chunks.front().ns;
    P.nsplit_max = 1;
    for (const SlotChunk &ch : P.chunks)
      P.nsplit_max = std::max(P.nsplit_max, direct_splits(n, (int)nd_out, ch.nl, c->sm_count));
    PO_TRY(c->cur.ensure(sizeof(float2) * 6 * (size_t)ns_max * std::max<int64_t>(n, 1)));
    PO_TRY(c->tile_ctr.ensure(sizeof(double) * 3 * (size_t)((n + 127) / 128 + 1)));
    PO_TRY(c->partial.ensure(sizeof(float2) * 6 * (size_t)ns_max * nd_out * P.nsplit_max));
    PO_TRY(c->levelA.ensure(sizeof(float2) * 6 * (size_t)ns_max * nd_out));
    if (adj) PO_TRY(c->levelB.ensure(sizeof(float2) * 6 * (size_t)ns_max * nd_out));
    // split BF16: the tcgen05 leaf kernel over one leaf of all points about
    // the box centre (the direct sum's centre), its direction tiles spread
    // over CTAs; tables [kc0: 0, chunks | begin: 0, n] and chunk -> leaf 0
    P.leaf_tc = cfg.precision == PO_PREC_SPLIT_BF16 && n > 0;
    P.leaf_group = cfg.leaf_slots ? cfg.leaf_slots : kLeafTcMaxSlots;
    if (P.leaf_tc) {
      const int64_t nchunks = (n + 15) / 16;
      if (nchunks > 2147483647LL) return fail(PO_ERR_UNSUPPORTED, "too many points for the tcgen05 direct sum");
      const int32_t tab[4] = {0, (int32_t)nchunks, 0, (int32_t)n};
      PO_TRY(c->leaf_kc0.ensure(sizeof(tab)));
      PO_TRY(c->leaf_chunk.ensure(sizeof(int32_t) * (size_t)nchunks));
      PO_TRY(c->leaf_ctr.ensure(sizeof(double) * 3));
      PO_CUDA(cudaMemcpyAsync(c->leaf_kc0.p, tab, sizeof(tab), cudaMemcpyHostToDevice, st));
      PO_CUDA(cudaMemsetAsync(c->leaf_chunk.p, 0, sizeof(int32_t) * (size_t)nchunks, st));
      PO_CUDA(cudaMemcpyAsync(c->leaf_ctr.p, P.c0, sizeof(P.c0), cudaMemcpyHostToDevice, st));
      P.leaf_chunks = nchunks;
      size_t bop = 0;
      int nl_max = 1;
      for (const SlotChunk &ch : P.chunks) {
        bop = std::max(bop, (size_t)ch.nl * nchunks * leaf_tc_col_tiles(std::min(ch.gc, P.leaf_group)) *
                                leaf_tc_block_bytes());
        nl_max = std::max(nl_max, ch.nl);
      }
      PO_TRY(c->leaf_bop.ensure(bop));
      PO_TRY(c->leaf_uop.ensure(sizeof(float4) * 16 * (size_t)nl_max * nchunks));
    }
    PO_CUDA(cudaStreamSynchronize(st));
    return PO_OK;
  }

  // ---- hierarchical solve
  P.nleaf = P.tree.level[d].count;
  PO_TRY(c->leaf_ctr.ensure(sizeof(double) * 3 * (size_t)std::max<int64_t>(P.nleaf, 1)));
  double3 lo = make_double3(cfg.box_min[0], cfg.box_min[1], cfg.box_min[2]);
  double3 hi = make_double3(cfg.box_max[0], cfg.box_max[1], cfg.box_max[2]);
  if (P.nleaf > 0) {
    k_leaf_centers<<<(unsigned)((P.nleaf + 255) / 256), 256, 0, st>>>(P.tree.level[d].prefix, P.nleaf, d, lo, hi,
                                                                       c->leaf_ctr.as<double>());
    count_launch();
  }
  // tcgen05 leaf sums when a wavelength has many patterns: the leaves' points
  // in chunks of 16 (bases computed on the host from the leaf ranges)
  P.leaf_tc = cfg.precision == PO_PREC_SPLIT_BF16 && P.nleaf > 0 &&
              (cfg.leaf_kernel == PO_LEAF_TCGEN05 || (cfg.leaf_kernel == PO_LEAF_AUTO && G >= kLeafTcMinSlots));
  P.leaf_group = cfg.leaf_slots ? cfg.leaf_slots : kLeafTcMaxSlots;
  double leaf_tc_per_slot = 0;
  if (P.leaf_tc) {
    std::vector<int32_t> lb((size_t)P.nleaf + 1);
    PO_CUDA(cudaMemcpyAsync(lb.data(), P.tree.level[d].begin, sizeof(int32_t) * lb.size(), cudaMemcpyDeviceToHost,
                            st));
    PO_CUDA(cudaStreamSynchronize(st));
    std::vector<int32_t> kc0((size_t)P.nleaf + 1);
    int64_t tot = 0;
    for (int64_t l = 0; l < P.nleaf; ++l) {
      kc0[l] = (int32_t)tot;
      tot += (lb[l + 1] - lb[l] + 15) / 16;
    }
    if (tot > 2147483647LL) return fail(PO_ERR_UNSUPPORTED, "too many points for the tcgen05 leaf sums");
    kc0[P.nleaf] = (int32_t)tot;
    std::vector<int32_t> cl((size_t)std::max<int64_t>(tot, 1), 0);
    for (int64_t l = 0; l < P.nleaf; ++l)
      for (int32_t k = kc0[l]; k < kc0[l + 1]; ++k) cl[k] = (int32_t)l;
    PO_TRY(c->leaf_kc0.ensure(sizeof(int32_t) * kc0.size()));
    PO_TRY(c->leaf_chunk.ensure(sizeof(int32_t) * cl.size()));
    PO_CUDA(cudaMemcpy(c->leaf_kc0.p, kc0.data(), sizeof(int32_t) * kc0.size(), cudaMemcpyHostToDevice));
    PO_CUDA(cudaMemcpy(c->leaf_chunk.p, cl.data(), sizeof(int32_t) * cl.size(), cudaMemcpyHostToDevice));
    P.leaf_chunks = tot;
    leaf_tc_per_slot = (double)tot * (double)leaf_tc_block_bytes() * 12.0 / 128.0;
  }
  // pattern buffers per slot: two level buffers + the row-pass output (R + 1
  // rows: the packed tensor-core row pass pads odd row counts to even)
  size_t lvl_max = 0, mid_max = 0;
  for (int l = 0; l <= d; ++l)
    lvl_max = std::max(lvl_max, (size_t)P.tree.level[l].count * 6 * (size_t)c->R[l] * c->Phi[l]);
  for (int l = 0; l < d; ++l) {
    // float2 words per slot and child: 6 components x R + 1 rows x Phi rounded
    // up to even (packed pairs), or 4 bf16 matrices of tc_kr x npad (core matrices of the tcgen05
    // pass, the six components in one column space) = tc_kr x npad float2
    const size_t per = c->tc_level[l] ? (size_t)c->tc_kr[l] * theta_tc_npad(c->Phi[l])
                                      : (size_t)6 * (c->R[l + 1] + 1) * (c->Phi[l] + (c->Phi[l] & 1));
    mid_max = std::max(mid_max, (size_t)P.tree.level[l + 1].count * per);
  }
  P.chunks = plan_chunks(L, G, chunk_slot_count(budget, 8.0 * (2.0 * lvl_max + mid_max) + leaf_tc_per_slot, S));
  const int ns_max = P.chunks.front().ns;
  if (P.leaf_tc) {
    size_t bop = 0;
    int nl_max = 1;
    for (const SlotChunk &ch : P.chunks) {
      bop = std::max(bop, (size_t)ch.nl * P.leaf_chunks * leaf_tc_col_tiles(std::min(ch.gc, P.leaf_group)) *
                              leaf_tc_block_bytes());
      nl_max = std::max(nl_max, ch.nl);
    }
    PO_TRY(c->leaf_bop.ensure(bop));
    PO_TRY(c->leaf_uop.ensure(sizeof(float4) * 16 * (size_t)nl_max * P.leaf_chunks));
  }
  PO_TRY(c->levelA.ensure(sizeof(float2) * lvl_max * ns_max));
  PO_TRY(c->levelB.ensure(sizeof(float2) * lvl_max * ns_max));
  PO_TRY(c->mid.ensure(sizeof(float2) * std::max<size_t>(mid_max * ns_max, 1)));
  // translation tables (per level, per wavelength)
  size_t tr_total = 0;
  P.tr_off.assign(d, 0);
  for (int l = 0; l < d; ++l) {
    P.tr_off[l] = tr_total;
    tr_total += (size_t)L * c->R[l] * c->Phi[l];
  }
  PO_TRY(c->trans.ensure(sizeof(float4) * std::max<size_t>(tr_total, 1)));
  for (int l = 0; l < d; ++l) {
    double a[3];
    for (int q = 0; q < 3; ++q) a[q] = ((double)cfg.box_max[q] - (double)cfg.box_min[q]) / std::ldexp(1.0, l + 2);
    PO_TRY(launch_trans_table(P.k_lambda, L, c->R[l], c->Phi[l], c->dir_trig.as<double2>() + c->trig_off[l], a,
                              c->trans.as<float4>() + P.tr_off[l], st));
  }
  // leaf directions
  std::vector<float4> df = host_dirs_f4(c->R[d], c->Phi[d], c->nth[d]);
  PO_TRY(c->dirs.ensure(sizeof(float4) * df.size()));
  PO_CUDA(cudaMemcpyAsync(c->dirs.p, df.data(), sizeof(float4) * df.size(), cudaMemcpyHostToDevice, st));
  PO_CUDA(cudaStreamSynchronize(st));
  return PO_OK;
}

// Kernel launches of a prepared solve: per slot chunk the leaf (or depth-0)
// sums, the level passes, the intensity into out_dev and, for po_grad, the
// adjoint.  No allocation and no host synchronisation unless `times` asks for
// per-chunk event timing, so this runs inside a stream capture.
static po_status enqueue_solve(po_ctx *c, const SolvePlan &P, float *out_dev, const AdjointArgs *adj,
                               cudaStream_t st, SolveTimes *times) {
  const po_config &cfg = c->cfg;
  const int d = c->depth;
  const int64_t n = P.n, nd_out = P.nd_out;
  const int nth_out = cfg.n_theta[0], nph_out = cfg.n_phi[0];
  auto rec = [&](cudaEvent_t e) -> po_status {
    if (times) PO_CUDA(cudaEventRecord(e, st));
    return PO_OK;
  };
  auto chunk_done = [&](bool tree_levels) -> po_status {
    if (!times) return PO_OK;
    PO_CUDA(cudaEventSynchronize(c->ev[4]));
    float t = 0;
    if (cudaEventElapsedTime(&t, c->kev[0], c->kev[1]) == cudaSuccess) { times->leafk += t; times->leaf += t; }
    if (cudaEventElapsedTime(&t, c->kev[1], c->ev[3]) == cudaSuccess) times->agg += t;
    if (cudaEventElapsedTime(&t, c->ev[3], c->ev[4]) == cudaSuccess) times->inten += t;
    if (tree_levels)
      for (int l = 0; l < d; ++l) {
        if (cudaEventElapsedTime(&t, c->kev[2 + 4 * l], c->kev[3 + 4 * l]) == cudaSuccess) {
          times->rows += t;
          times->rows_l[l] += t;
        }
        if (cudaEventElapsedTime(&t, c->kev[4 + 4 * l], c->kev[5 + 4 * l]) == cudaSuccess) {
          times->cols += t;
          times->cols_l[l] += t;
        }
      }
    cudaGetLastError();
    return PO_OK;
  };
  SolveTimes dummy;
  SolveTimes &T = times ? *times : dummy;
  if (adj && n > 0) PO_CUDA(cudaMemsetAsync(c->grad_acc.p, 0, sizeof(double) * 7 * (size_t)n, st));

  if (P.fp64) {
    for (const SlotChunk &ch : P.chunks) {
      PO_TRY(rec(c->kev[0]));
      PO_TRY(launch_currents_f64(n, P.gin, c->slots.as<SlotParams<double>>() + ch.s0, ch.ns, c->cur.as<double>(), st));
      int64_t tiles = (int64_t)ch.ns * ceil_div((int)nd_out, 128);
      int nsplit = (int)std::max<int64_t>(
          1, std::min<int64_t>(64, (c->sm_count * 8 + tiles - 1) / std::max<int64_t>(1, tiles)));
      nsplit = (int)std::min<int64_t>(std::min(nsplit, P.nsplit_max), std::max<int64_t>(1, n));
      PO_TRY(launch_direct_f64(n, P.gin[0], P.gin[1], P.gin[2], c->cur.as<double2>(), P.k_slot + ch.s0, ch.ns, P.c0,
                               c->dirs_d.as<double>(), (int)nd_out, nsplit, c->partial.as<double2>(),
                               c->levelA.as<double2>(), st));
      PO_TRY(rec(c->kev[1]));
      PO_TRY(rec(c->ev[3]));
      PO_TRY(launch_intensity_f64(c->levelA.as<double2>(), ch.ns, nth_out, nph_out, out_dev + (size_t)ch.s0 * nd_out,
                                  st));
      if (adj) {
        double2 *Gd = c->partial.as<double2>();
        PO_TRY(launch_intensity_adjoint_f64(c->levelA.as<double2>(), adj->dl_di + (size_t)ch.s0 * nd_out, ch.ns,
                                            nth_out, nph_out, Gd, st));
        PO_TRY(launch_point_adjoint_f64(P.gin, c->chunk_begin.as<int32_t>(), (n + 31) / 32, c->center0.as<double>(),
                                        0, Gd, 0, 6 * nd_out, c->dirs_d.as<double>(), (int)nd_out,
                                        P.sp64_dev + ch.s0, ch.nl, ch.gc, n, c->grad_acc.as<double>(), st));
      }
      PO_TRY(rec(c->ev[4]));
      T.n_leaf += 3;
      PO_TRY(chunk_done(false));
    }
    T.leaf_pd = (double)n * nd_out * P.S;
  } else if (d == 0) {
    for (const SlotChunk &ch : P.chunks) {
      PO_TRY(rec(c->kev[0]));
      if (P.leaf_tc) {
        const int32_t *tab = c->leaf_kc0.as<int32_t>();
        PO_TRY(launch_leaf_tc(P.gsc, tab + 2, tab, c->leaf_chunk.as<int32_t>(), P.leaf_chunks, c->leaf_ctr.as<double>(),
                              1, c->slots.as<SlotParams<float>>() + ch.s0, ch.nl, ch.gc, 0, ch.gc,
                              c->dirs.as<float4>(), (int)nd_out, c->leaf_bop.as<uint8_t>(), c->leaf_bop.bytes,
                              c->leaf_uop.as<float4>(), c->leaf_uop.bytes, c->levelA.as<float2>(), c->tc_err.as<int>(),
                              st, P.leaf_group, 0, ceil_div((int)nd_out, 128)));
      } else {
        PO_TRY(launch_currents_f32(n, P.gsc, c->slots.as<SlotParams<float>>() + ch.s0, ch.ns, c->cur.as<float>(),
                                   st));
        int nsplit = direct_splits(n, (int)nd_out, ch.nl, c->sm_count);
        PO_TRY(launch_direct_f32(n, P.gsc[0], P.gsc[1], P.gsc[2], c->cur.as<float2>(), c->tile_ctr.as<double>(),
                                 P.k_lambda + ch.l0, ch.nl, ch.gc, P.c0, c->dirs.as<float4>(), c->dirs_d.as<double>(),
                                 (int)nd_out, nsplit, c->partial.as<float2>(), c->levelA.as<float2>(), st));
      }
      PO_TRY(rec(c->kev[1]));
      PO_TRY(rec(c->ev[3]));
      PO_TRY(launch_intensity_f32(c->levelA.as<float2>(), ch.ns, nth_out, nph_out, nth_out, nph_out, 1, 1,
                                  c->out_dirs.as<float4>(), out_dev + (size_t)ch.s0 * nd_out, st));
      if (adj) {
        float2 *Gf = c->levelB.as<float2>();
        PO_TRY(launch_intensity_adjoint_f32(c->levelA.as<float2>(), adj->dl_di + (size_t)ch.s0 * nd_out, ch.ns,
                                            nth_out, nph_out, nth_out, nph_out, 1, 1, c->out_dirs.as<float4>(), Gf,
                                            st));
        PO_TRY(launch_point_adjoint_mma(P.gsc, c->chunk_begin.as<int32_t>(), (n + 127) / 128, c->center0.as<double>(),
                                        0, Gf, 0, 6 * nd_out, c->dirs.as<float4>(), (int)nd_out, P.sp64_dev + ch.s0,
                                        ch.nl, ch.gc, n, c->grad_acc.as<double>(), st));
      }
      PO_TRY(rec(c->ev[4]));
      T.n_leaf += P.leaf_tc ? 2 * ((ch.gc + P.leaf_group - 1) / P.leaf_group) : 3 + (ch.gc + 3) / 4;
      PO_TRY(chunk_done(false));
    }
    T.leaf_pd = (double)n * nd_out * P.S;
  } else {
    const int refnq = c->cover == 1 ? 1 : 0;
    for (const SlotChunk &ch : P.chunks) {
      const SlotParams<float> *sp = c->slots.as<SlotParams<float>>() + ch.s0;
      PO_TRY(rec(c->kev[0]));
      // the phi pass of the deepest parent level runs in the leaf kernel's epilogue
      // when its packed output fits one n-tile group
      const bool fuse_rows = cfg.precision == PO_PREC_SPLIT_BF16 && !P.leaf_tc && d >= 1 && c->tt_level[d - 1] &&
                             !c->tc_level[d - 1] && leaf_row_fusion_fits(c->Phi[d], c->Phi[d - 1], c->bmat_kp[d - 1]);
      if (P.leaf_tc)
        PO_TRY(launch_leaf_tc(P.gsc, P.tree.level[d].begin, c->leaf_kc0.as<int32_t>(), c->leaf_chunk.as<int32_t>(),
                              P.leaf_chunks, c->leaf_ctr.as<double>(), P.nleaf, sp, ch.nl, ch.gc, 0, ch.gc,
                              c->dirs.as<float4>(), c->R[d] * c->Phi[d], c->leaf_bop.as<uint8_t>(), c->leaf_bop.bytes,
                              c->leaf_uop.as<float4>(), c->leaf_uop.bytes, c->levelA.as<float2>(), c->tc_err.as<int>(),
                              st, P.leaf_group));
      else if (cfg.precision == PO_PREC_SPLIT_BF16)
        PO_TRY(launch_leaf_mma(P.gsc, P.tree.level[d].begin, c->leaf_ctr.as<double>(), P.nleaf, sp, ch.nl, ch.gc,
                               c->dirs.as<float4>(), c->R[d] * c->Phi[d], c->levelA.as<float2>(), st,
                               fuse_rows ? c->bmat.as<uint32_t>() + c->bmat_off[d - 1] : nullptr,
                               fuse_rows ? c->mid.as<uint4>() : nullptr, c->R[d], c->Phi[d], c->Phi[d - 1],
                               d >= 1 ? c->bmat_kp[d - 1] : 0));
      else
        PO_TRY(launch_leaf(P.gsc, P.tree.level[d].begin, c->leaf_ctr.as<double>(), P.nleaf, sp, ch.nl, ch.gc,
                           c->dirs.as<float4>(), c->R[d] * c->Phi[d], c->levelA.as<float2>(), st));
      PO_TRY(rec(c->kev[1]));
      T.n_leaf += P.nleaf <= 0 ? 0 : P.leaf_tc ? 2 * ((ch.gc + P.leaf_group - 1) / P.leaf_group) : (ch.gc + 3) / 4;
      float2 *cur_lvl = c->levelA.as<float2>(), *nxt = c->levelB.as<float2>();
      for (int l = d - 1; l >= 0; --l) {
        const int64_t nc = P.tree.level[l + 1].count, np = P.tree.level[l].count;
        const float4 *trans = c->trans.as<float4>() + P.tr_off[l] + (size_t)ch.l0 * c->R[l] * c->Phi[l];
        int64_t nrows = (int64_t)ch.ns * nc * 6 * c->R[l + 1];
        PO_TRY(rec(c->kev[2 + 4 * l]));
        if (fuse_rows && l == d - 1) {
          // written by the leaf kernel
        } else if (c->rt_level[l]) {
          PO_TRY(launch_rows_tc(cur_lvl, c->mid.as<uint8_t>(), c->mid.bytes, (int64_t)ch.ns * nc * 6, c->R[l + 1],
                                c->tc_kr[l], theta_tc_npad(c->Phi[l]), c->Phi[l + 1], c->Phi[l],
                                c->rt_bmat.as<uint8_t>() + c->rt_off[l], c->rt_bytes[l], c->rt_ntn[l], c->rt_nnt[l],
                                c->sm_count, c->tc_err.as<int>(), st));
        } else if (c->tc_level[l]) {
          PO_TRY(launch_interp_rows_core(cur_lvl, c->mid.as<uint8_t>(), (int64_t)ch.ns * nc * 6, c->R[l + 1],
                                         c->tc_kr[l], theta_tc_npad(c->Phi[l]), c->Phi[l + 1], c->Phi[l],
                                         c->bmat_kp[l], c->bmat.as<uint32_t>() + c->bmat_off[l], c->sm_count, st));
        } else if (c->tt_level[l]) {
          PO_TRY(launch_interp_rows_packed(cur_lvl, c->mid.as<uint4>(), (int64_t)ch.ns * nc * 6, c->R[l + 1],
                                           c->Phi[l + 1], c->Phi[l], c->bmat_kp[l],
                                           c->bmat.as<uint32_t>() + c->bmat_off[l], c->sm_count, st));
        } else {
          FftPlan prow_in = make_plan(c->Phi[l + 1], c->tw_offset[c->Phi[l + 1]]);
          FftPlan prow_out = make_plan(c->Phi[l], c->tw_offset[c->Phi[l]]);
          PO_TRY(launch_interp_rows(cur_lvl, c->mid.as<float2>(), nrows, prow_in, prow_out, c->twiddles.as<float2>(),
                                    1.0f / (float)c->Phi[l + 1], c->sm_count, refnq, st));
        }
        PO_TRY(rec(c->kev[3 + 4 * l]));
        T.rows_b += 8.0 * nrows * (c->Phi[l + 1] + c->Phi[l]);
        T.cols_b += 8.0 * ch.ns * 6 * ((double)nc * c->R[l + 1] * c->Phi[l] + (double)np * c->R[l] * c->Phi[l]);
        T.agg_b += 8.0 * ch.ns * 6 * ((double)nc * c->R[l + 1] * c->Phi[l + 1] + (double)np * c->R[l] * c->Phi[l]);
        if (nrows > 0 && !(fuse_rows && l == d - 1)) ++T.n_row;
        if (np > 0) ++T.n_col;
        PO_TRY(rec(c->kev[4 + 4 * l]));
        if (c->tc_level[l]) {
          PO_TRY(launch_theta_tc(c->mid.as<uint8_t>(), nxt, P.tree.level[l].child, np, nc, c->Phi[l], c->tc_kr[l],
                                 c->R[l], c->tc_amat.as<uint8_t>() + c->tc_off[l], trans, ch.ns, ch.gc,
                                 c->tc_err.as<int>(), c->mid.bytes, c->tc_amat.bytes - c->tc_off[l], st));
        } else if (c->tt_level[l]) {
          PO_TRY(launch_interp_cols_mma(c->mid.as<uint4>(), nxt, P.tree.level[l].child, np, nc, c->Phi[l],
                                        c->R[l + 1], c->R[l], c->amat_kp[l], c->amat.as<uint32_t>() + c->amat_off[l],
                                        trans, ch.ns, ch.gc, cfg.interp_tile, st));
        } else {
          FftPlan pcol_in = make_plan(c->T[l + 1], c->tw_offset[c->T[l + 1]]);
          FftPlan pcol_out = make_plan(c->T[l], c->tw_offset[c->T[l]]);
          int reach = 0x7fffffff;
          if (c->cover == 1 && cfg.nyquist_quirk) reach = 256 * (c->T[l + 1] / 256 + 1);
          PO_TRY(launch_interp_cols(c->mid.as<float2>(), nxt, P.tree.level[l].child, np, nc, c->Phi[l], c->R[l + 1],
                                    c->R[l], pcol_in, pcol_out, c->twiddles.as<float2>(), trans, ch.ns, ch.gc, reach,
                                    1.0f / (float)c->T[l + 1], 6, c->mirror, refnq, st));
        }
        PO_TRY(rec(c->kev[5 + 4 * l]));
        std::swap(cur_lvl, nxt);
      }
      PO_TRY(rec(c->ev[3]));
      PO_TRY(launch_intensity_f32(cur_lvl, ch.ns, c->R[0], c->Phi[0], nth_out, nph_out, c->mt, c->mp,
                                  c->out_dirs.as<float4>(), out_dev + (size_t)ch.s0 * nd_out, st));
      if (adj) {
        // root adjoint, then the transposed aggregation down to the leaves
        PO_TRY(launch_intensity_adjoint_f32(cur_lvl, adj->dl_di + (size_t)ch.s0 * nd_out, ch.ns, c->R[0], c->Phi[0],
                                            nth_out, nph_out, c->mt, c->mp, c->out_dirs.as<float4>(), nxt, st));
        std::swap(cur_lvl, nxt);
        for (int l = 0; l < d; ++l) {
          const int64_t np = P.tree.level[l].count, nc = P.tree.level[l + 1].count;
          const float4 *trans = c->trans.as<float4>() + P.tr_off[l] + (size_t)ch.l0 * c->R[l] * c->Phi[l];
          PO_TRY(launch_interp_cols_adj_mma(cur_lvl, c->mid.as<float2>(), P.tree.level[l].child, np, nc, c->Phi[l],
                                            c->R[l + 1], c->R[l], c->amat_adj_kp[l],
                                            c->amat_adj.as<uint32_t>() + c->amat_adj_off[l], trans, ch.ns, ch.gc, st));
          PO_TRY(launch_interp_rows_mma(c->mid.as<float2>(), nxt, (int64_t)ch.ns * nc * 6 * c->R[l + 1], c->Phi[l],
                                        c->Phi[l + 1], c->bmat_adj_kp[l],
                                        c->bmat_adj.as<uint32_t>() + c->bmat_adj_off[l], c->sm_count, st));
          std::swap(cur_lvl, nxt);
        }
        const int64_t ndl = (int64_t)c->R[d] * c->Phi[d];
        PO_TRY(launch_point_adjoint_mma(P.gsc, P.tree.level[d].begin, P.nleaf, c->leaf_ctr.as<double>(), 1, cur_lvl,
                                        6 * ndl, P.nleaf * 6 * ndl, c->dirs.as<float4>(), (int)ndl, P.sp64_dev + ch.s0,
                                        ch.nl, ch.gc, n, c->grad_acc.as<double>(), st));
      }
      PO_TRY(rec(c->ev[4]));
      PO_TRY(chunk_done(true));
    }
    T.leaf_pd = (double)n * c->R[d] * c->Phi[d] * P.S;
  }
  if (adj) PO_TRY(launch_scatter_grad(c->grad_acc.as<double>(), P.perm_out, n, adj->grad, st));
  return PO_OK;
}

// The error word of the tcgen05 theta pass: nonzero when one of its bounded
// waits gave up (the level's output is then incomplete).  Read after a
// synchronous solve; an asynchronous solve leaves it for the next check.
static po_status check_device_waits(po_ctx *c) {
  if (!c->tc_err.p) return PO_OK;
  int h = 0;
  PO_CUDA(cudaMemcpy(&h, c->tc_err.p, sizeof(int), cudaMemcpyDeviceToHost));
  if (h == 0) return PO_OK;
  PO_CUDA(cudaMemset(c->tc_err.p, 0, sizeof(int)));
  if (h == 2) return fail(PO_ERR_INTERNAL, "tcgen05 pass: operand run outside its buffer");
  return fail(PO_ERR_TIMEOUT, "tcgen05 pass (leaf sums or theta/phi interpolation): a device wait timed out");
}

static po_status solve_impl(po_ctx *c, const po_geometry *g, const po_illum *il, float *intensity, int out_on_device,
                            cudaStream_t st, po_report *rep, const AdjointArgs *adj = nullptr) {
  const int64_t launches0 = g_launch_count;
  PO_CUDA(cudaEventRecord(c->ev[0], st));
  SolvePlan P;
  PO_CUDA(cudaEventRecord(c->ev[1], st));
  PO_TRY(prepare_solve(c, g, il, adj != nullptr, st, P));
  PO_CUDA(cudaEventRecord(c->ev[2], st));
  float *out_dev = intensity;
  if (!out_on_device || !intensity) {
    PO_TRY(c->out.ensure(sizeof(float) * (size_t)P.S * P.nd_out));
    out_dev = c->out.as<float>();
  }
  SolveTimes T;
  PO_TRY(enqueue_solve(c, P, out_dev, adj, st, rep ? &T : nullptr));
  if (intensity && !out_on_device)
    PO_CUDA(cudaMemcpyAsync(intensity, out_dev, sizeof(float) * (size_t)P.S * P.nd_out, cudaMemcpyDeviceToHost, st));
  PO_CUDA(cudaEventRecord(c->ev[5], st));
  if (rep || !out_on_device) {
    PO_CUDA(cudaEventSynchronize(c->ev[5]));
    PO_TRY(check_device_waits(c));
  }
  PO_CUDA(cudaGetLastError());
  if (rep) {
    float t[2];
    cudaEventElapsedTime(&t[0], c->ev[0], c->ev[5]);
    cudaEventElapsedTime(&t[1], c->ev[1], c->ev[2]);
    rep->ms_total = t[0];
    rep->ms_build = t[1];
    rep->ms_leaf = T.leaf;
    rep->ms_aggregate = T.agg;
    rep->ms_intensity = T.inten;
    rep->root_theta = c->nth[0];
    rep->root_phi = c->Phi[0];
    if (!P.fp64) {
      const int tdepth = c->depth > 0 ? c->depth : 6;
      rep->n_leaves = P.tree.level[tdepth].count;
      int64_t tot = 0;
      for (int l = 0; l <= tdepth; ++l) {
        tot += P.tree.level[l].count;
        if (l <= PO_MAX_DEPTH) rep->n_nodes_level[l] = P.tree.level[l].count;
      }
      rep->n_nodes_total = tot;
    }
    int64_t ws = 0;
    for (DevBuf *b : {&c->twiddles, &c->geom_in, &c->geom_sorted, &c->octree_ws, &c->leaf_ctr, &c->dirs, &c->dirs_d,
                      &c->trans, &c->levelA, &c->levelB, &c->mid, &c->slots, &c->kvals, &c->out, &c->cur, &c->partial,
                      &c->tile_ctr, &c->slots64, &c->grad_acc, &c->chunk_begin, &c->amat_adj, &c->bmat_adj,
                      &c->leaf_kc0, &c->leaf_chunk, &c->leaf_bop, &c->leaf_uop})
      ws += (int64_t)b->bytes;
    rep->workspace_bytes = ws;
    rep->kernel_launches = g_launch_count - launches0;
    rep->n_leaf_launches = T.n_leaf;
    rep->n_row_launches = T.n_row;
    rep->n_col_launches = T.n_col;
    rep->n_chunks = (int)P.chunks.size();
    rep->chunk_slots = P.chunks.empty() ? 0 : P.chunks.front().ns;
    rep->leaf_point_dirs = T.leaf_pd;
    rep->rows_bytes = T.rows_b;
    rep->cols_bytes = T.cols_b;
    rep->agg_bytes = T.agg_b;
    rep->ms_leaf_kernel = T.leafk;
    rep->ms_rows = T.rows;
    rep->ms_cols = T.cols;
    for (int l = 0; l < PO_MAX_DEPTH; ++l) {
      rep->ms_rows_level[l] = T.rows_l[l];
      rep->ms_cols_level[l] = T.cols_l[l];
    }
    cudaGetLastError();
  }
  return PO_OK;
}

po_status po_solve(po_ctx *c, const po_geometry *g, const po_illum *il, float *intensity, int out_on_device,
                   void *stream, po_report *rep) {
  if (!c || !g || !il || !intensity) return fail(PO_ERR_INVALID_ARGUMENT, "null argument");
  if (g->n < 0 || g->n > 2000000000LL) return fail(PO_ERR_INVALID_ARGUMENT, "point count out of range");
  if (g->n > 0 && (!g->x || !g->y || !g->z || !g->nx || !g->ny || !g->nz || !g->area))
    return fail(PO_ERR_INVALID_ARGUMENT, "null geometry array");
  if (il->n_lambda <= 0 || !il->lambda_m) return fail(PO_ERR_INVALID_ARGUMENT, "no wavelengths");
  if (il->n_inc <= 0 || !il->theta_i || !il->phi_i) return fail(PO_ERR_INVALID_ARGUMENT, "no incident directions");
  if ((il->pol_mask & (PO_POL_TM | PO_POL_TE)) == 0 || (il->pol_mask & ~(PO_POL_TM | PO_POL_TE)))
    return fail(PO_ERR_INVALID_ARGUMENT, "pol_mask must select TM and/or TE");
  for (int l = 0; l < il->n_lambda; ++l)
    if (!(il->lambda_m[l] > 0) || !std::isfinite(il->lambda_m[l]))
      return fail(PO_ERR_INVALID_ARGUMENT, "wavelengths must be positive");
  if (!(il->sigma > 0)) return fail(PO_ERR_INVALID_ARGUMENT, "beam sigma must be > 0");
  const int npol = ((il->pol_mask & PO_POL_TM) ? 1 : 0) + ((il->pol_mask & PO_POL_TE) ? 1 : 0);
  if ((int64_t)il->n_lambda * il->n_inc * npol > 65535) return fail(PO_ERR_UNSUPPORTED, "too many patterns per call");
  int dev = 0;
  PO_CUDA(cudaGetDevice(&dev));
  if (dev != c->device) return fail(PO_ERR_INVALID_ARGUMENT, "context was created on another device");
  if (rep) std::memset(rep, 0, sizeof(*rep));
  return solve_impl(c, g, il, intensity, out_on_device, (cudaStream_t)stream, rep);
}

po_status po_check(po_ctx *c, void *stream) {
  if (!c) return fail(PO_ERR_INVALID_ARGUMENT, "null argument");
  PO_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
  return check_device_waits(c);
}

// ---------------------------------------------------------------- single steps
po_status po_grad(po_ctx *c, const po_geometry *g, const po_illum *il, const float *dl_di, float *grad,
                  float *intensity, void *stream, po_report *rep) {
  if (!c || !g || !il || !dl_di || !grad) return fail(PO_ERR_INVALID_ARGUMENT, "null argument");
  if (g->n < 0 || g->n > 2000000000LL) return fail(PO_ERR_INVALID_ARGUMENT, "point count out of range");
  if (g->n > 0 && (!g->x || !g->y || !g->z || !g->nx || !g->ny || !g->nz || !g->area))
    return fail(PO_ERR_INVALID_ARGUMENT, "null geometry array");
  if (il->n_lambda <= 0 || !il->lambda_m) return fail(PO_ERR_INVALID_ARGUMENT, "no wavelengths");
  if (il->n_inc <= 0 || !il->theta_i || !il->phi_i) return fail(PO_ERR_INVALID_ARGUMENT, "no incident directions");
  if ((il->pol_mask & (PO_POL_TM | PO_POL_TE)) == 0 || (il->pol_mask & ~(PO_POL_TM | PO_POL_TE)))
    return fail(PO_ERR_INVALID_ARGUMENT, "pol_mask must select TM and/or TE");
  for (int l = 0; l < il->n_lambda; ++l)
    if (!(il->lambda_m[l] > 0) || !std::isfinite(il->lambda_m[l]))
      return fail(PO_ERR_INVALID_ARGUMENT, "wavelengths must be positive");
  if (!(il->sigma > 0)) return fail(PO_ERR_INVALID_ARGUMENT, "beam sigma must be > 0");
  const int npol = ((il->pol_mask & PO_POL_TM) ? 1 : 0) + ((il->pol_mask & PO_POL_TE) ? 1 : 0);
  if ((int64_t)il->n_lambda * il->n_inc * npol > 65535) return fail(PO_ERR_UNSUPPORTED, "too many patterns per call");
  if (c->depth > 0 && !(c->tensor_theta && c->mirror))
    return fail(PO_ERR_UNSUPPORTED, "the adjoint of a tree solve needs double-cover theta and PO_INTERP_TENSOR");
  int dev = 0;
  PO_CUDA(cudaGetDevice(&dev));
  if (dev != c->device) return fail(PO_ERR_INVALID_ARGUMENT, "context was created on another device");
  if (c->depth > 0) PO_TRY(ensure_adjoint_matrices(c));
  if (rep) std::memset(rep, 0, sizeof(*rep));
  AdjointArgs a;
  a.dl_di = dl_di;
  a.grad = grad;
  return solve_impl(c, g, il, intensity, 1, (cudaStream_t)stream, rep, &a);
}

po_status po_tangent_plane_currents(int64_t n, const float *x, const float *y, const float *z, const float *nx,
                                    const float *ny, const float *nz, const float *area, double lambda_m,
                                    double theta_i, double phi_i, int pol, double eta_re, double eta_im, double sigma,
                                    double distance, int scale, float *currents, void *stream) {
  if (n < 0) return fail(PO_ERR_INVALID_ARGUMENT, "negative point count");
  if (n == 0) return PO_OK;
  if (!x || !y || !z || !nx || !ny || !nz || !currents || (scale && !area))
    return fail(PO_ERR_INVALID_ARGUMENT, "null pointer");
  if (pol != PO_POL_TM && pol != PO_POL_TE) return fail(PO_ERR_INVALID_ARGUMENT, "pol must be PO_POL_TM or PO_POL_TE");
  if (!(lambda_m > 0) || !(sigma > 0) || (scale && !(distance > 0)))
    return fail(PO_ERR_INVALID_ARGUMENT, "lambda, sigma and distance must be > 0");
  cudaStream_t st = (cudaStream_t)stream;
  SlotParams<float> p = make_slot<float>(lambda_m, theta_i, phi_i, pol == PO_POL_TE, eta_re, eta_im, sigma,
                                         scale ? distance : 1.0, scale != 0);
  SlotParams<float> *dp = nullptr;
  PO_CUDA(cudaMallocAsync((void **)&dp, sizeof(p), st));
  cudaError_t e = cudaMemcpyAsync(dp, &p, sizeof(p), cudaMemcpyHostToDevice, st);
  const float *g[7] = {x, y, z, nx, ny, nz, scale ? area : nullptr};
  po_status s = e == cudaSuccess ? launch_currents_f32(n, g, dp, 1, currents, st) : cuda_fail(e, "cudaMemcpyAsync");
  cudaFreeAsync(dp, st);
  if (s == PO_OK) PO_CUDA(cudaStreamSynchronize(st));  // the host slot struct goes out of scope
  return s;
}

po_status po_build_octree(int64_t n, const float *x, const float *y, const float *z, const float box_min[3],
                          const float box_max[3], int depth, int32_t *perm, int32_t *heap_range, void *stream) {
  if (n < 0 || (n > 0 && (!x || !y || !z || !perm)) || !box_min || !box_max)
    return fail(PO_ERR_INVALID_ARGUMENT, "null pointer or negative count");
  if (depth < 0 || depth > 7) return fail(PO_ERR_INVALID_ARGUMENT, "depth must be in [0, 7] for the heap layout");
  cudaStream_t st = (cudaStream_t)stream;
  size_t wsb = octree_workspace_bytes(n, depth);
  void *ws = nullptr;
  PO_CUDA(cudaMallocAsync(&ws, wsb, st));
  OctreeBuffers t;
  po_status s = build_octree(x, y, z, n, box_min, box_max, depth, ws, wsb, &t, st);
  if (s == PO_OK && n > 0) {
    cudaError_t e = cudaMemcpyAsync(perm, t.perm, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) s = cuda_fail(e, "cudaMemcpyAsync(perm)");
  }
  if (s == PO_OK && heap_range) s = octree_heap_ranges(t, heap_range, st);
  cudaFreeAsync(ws, st);
  if (s == PO_OK) PO_CUDA(cudaStreamSynchronize(st));
  return s;
}

po_status po_far_field_direct(int64_t n, const float *x, const float *y, const float *z, const float *currents,
                              double k, const double center[3], int n_theta, int n_phi, int precision, float *fields,
                              void *stream) {
  if (n < 0 || n_theta <= 0 || n_phi <= 0 || !center || !fields || (n > 0 && (!x || !y || !z || !currents)))
    return fail(PO_ERR_INVALID_ARGUMENT, "invalid argument");
  if (!(k > 0)) return fail(PO_ERR_INVALID_ARGUMENT, "k must be > 0");
  if (precision != PO_PREC_FP32 && precision != PO_PREC_FP64)
    return fail(PO_ERR_UNSUPPORTED, "direct sum precision must be FP32 or FP64");
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t nd = (int64_t)n_theta * n_phi;
  std::vector<float4> df = host_dirs_f4(n_theta, n_phi, n_theta);
  std::vector<double> dd = host_dirs_d(n_theta, n_phi, n_theta);
  void *bdirs = nullptr, *bdd = nullptr, *bk = nullptr, *bpart = nullptr, *btile = nullptr, *bacc = nullptr;
  po_status s = PO_OK;
  int nsplit = precision == PO_PREC_FP32 ? direct_splits(n, (int)nd, 1, 152) : 8;
  if (n > 0 && nsplit > n) nsplit = (int)n;
  size_t vb = precision == PO_PREC_FP32 ? sizeof(float2) : sizeof(double2);
#define A(ptr, bytes)                                             \
  do {                                                            \
    cudaError_t _e = cudaMallocAsync(&ptr, (bytes), st);          \
    if (_e != cudaSuccess && s == PO_OK) s = cuda_fail(_e, "cudaMallocAsync"); \
  } while (0)
  A(bdirs, sizeof(float4) * df.size());
  A(bdd, sizeof(double) * dd.size());
  A(bk, sizeof(double));
  A(bpart, vb * 6 * nd * nsplit);
  A(btile, sizeof(double) * 3 * ((n + 127) / 128 + 1));
  A(bacc, precision == PO_PREC_FP64 ? sizeof(double2) * 6 * (n > 0 ? n : 1) + sizeof(double2) * 6 * nd : 16);
#undef A
  if (s == PO_OK) {
    cudaMemcpyAsync(bdirs, df.data(), sizeof(float4) * df.size(), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(bdd, dd.data(), sizeof(double) * dd.size(), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(bk, &k, sizeof(double), cudaMemcpyHostToDevice, st);
    if (precision == PO_PREC_FP32) {
      s = launch_direct_f32(n, x, y, z, (const float2 *)currents, (double *)btile, (const double *)bk, 1, 1, center,
                            (const float4 *)bdirs, (const double *)bdd, (int)nd, nsplit, (float2 *)bpart,
                            (float2 *)fields, st);
    } else {
      // widen the float currents, sum in double, narrow the fields
      double2 *cur64 = (double2 *)bacc, *f64 = cur64 + 6 * (n > 0 ? n : 1);
      s = launch_widen(currents, cur64, 6 * n, st);
      if (s == PO_OK)
        s = launch_direct_f64(n, x, y, z, cur64, (const double *)bk, 1, center, (const double *)bdd, (int)nd, nsplit,
                              (double2 *)bpart, f64, st);
      if (s == PO_OK) s = launch_narrow(f64, (float2 *)fields, 6 * nd, st);
    }
  }
  for (void *p : {bdirs, bdd, bk, bpart, btile, bacc})
    if (p) cudaFreeAsync(p, st);
  if (s == PO_OK) PO_CUDA(cudaStreamSynchronize(st));
  return s;
}

po_status po_interp_fft(const float *in, int th_c, int ph_c, float *out, int th_p, int ph_p, int batch, int theta_mode,
                        int nyquist_quirk, void *stream) {
  if (!in || !out || th_c <= 0 || ph_c <= 0 || batch < 0) return fail(PO_ERR_INVALID_ARGUMENT, "invalid argument");
  if (th_p < th_c || ph_p < ph_c) return fail(PO_ERR_INVALID_ARGUMENT, "the interpolation only upsamples");
  if (theta_mode != PO_THETA_DOUBLE_COVER && theta_mode != PO_THETA_REFERENCE)
    return fail(PO_ERR_INVALID_ARGUMENT, "unknown theta mode");
  if (batch == 0) return PO_OK;
  {
    int dev = 0;
    PO_CUDA(cudaGetDevice(&dev));
    PO_TRY(init_device_attributes(dev));
  }
  cudaStream_t st = (cudaStream_t)stream;
  std::vector<int> lens = {ph_c, ph_p, th_c, th_p};
  std::sort(lens.begin(), lens.end());
  lens.erase(std::unique(lens.begin(), lens.end()), lens.end());
  std::map<int, int> off;
  int total = 0;
  for (int n : lens) { off[n] = total; total += n; }
  void *tw = nullptr, *mid = nullptr;
  po_status s = PO_OK;
  cudaError_t e = cudaMallocAsync(&tw, sizeof(float2) * total, st);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMallocAsync(twiddles)");
  e = cudaMallocAsync(&mid, sizeof(float2) * (size_t)batch * th_c * ph_p, st);
  if (e != cudaSuccess) { cudaFreeAsync(tw, st); return cuda_fail(e, "cudaMallocAsync(scratch)"); }
  for (int n : lens)
    if (s == PO_OK) s = launch_twiddles(n, (float2 *)tw + off[n], st);
  int sm = 152, dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, dev);
  if (s == PO_OK)
    s = launch_interp_rows((const float2 *)in, (float2 *)mid, (int64_t)batch * th_c, make_plan(ph_c, off[ph_c]),
                           make_plan(ph_p, off[ph_p]), (const float2 *)tw, 1.0f / (float)ph_c, sm,
                           theta_mode == PO_THETA_REFERENCE ? 1 : 0, st);
  int reach = (theta_mode == PO_THETA_REFERENCE && nyquist_quirk) ? 256 * (th_c / 256 + 1) : 0x7fffffff;
  if (s == PO_OK)
    s = launch_interp_cols((const float2 *)mid, (float2 *)out, nullptr, batch, batch, ph_p, th_c, th_p,
                           make_plan(th_c, off[th_c]), make_plan(th_p, off[th_p]), (const float2 *)tw, nullptr, 1, 1,
                           reach, 1.0f / (float)th_c, 1, 0, theta_mode == PO_THETA_REFERENCE ? 1 : 0, st);
  cudaFreeAsync(mid, st);
  cudaFreeAsync(tw, st);
  if (s == PO_OK) PO_CUDA(cudaStreamSynchronize(st));
  return s;
}

po_status po_compute_intensity(const float *fields, int n_theta, int n_phi, float *intensity, void *stream) {
  if (!fields || !intensity || n_theta <= 0 || n_phi <= 0) return fail(PO_ERR_INVALID_ARGUMENT, "invalid argument");
  return launch_intensity_f32((const float2 *)fields, 1, n_theta, n_phi, n_theta, n_phi, 1, 1, nullptr, intensity,
                              (cudaStream_t)stream);
}


// ------------------------------------------------------------------ batches
struct po_batch {
  std::vector<po_ctx *> ctx;
  std::vector<SolvePlan> plans;
  std::vector<int> branch;  // stream branch of each item
  int n_streams = 1;
  std::vector<cudaStream_t> streams;
  std::vector<cudaEvent_t> joins;
  cudaEvent_t fork = nullptr;
  cudaStream_t cap = nullptr;  // capture origin (the caller's stream may be the legacy default stream)
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int64_t nodes = 0;
  double ms_prepare = 0;
  int device = 0;
};

static void batch_release_graph(po_batch *b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
  b->nodes = 0;
}

po_status po_batch_destroy(po_batch *b) {
  if (!b) return PO_OK;
  batch_release_graph(b);
  for (po_ctx *c : b->ctx) po_destroy(c);
  for (cudaStream_t s : b->streams)
    if (s) cudaStreamDestroy(s);
  for (cudaEvent_t e : b->joins)
    if (e) cudaEventDestroy(e);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->cap) cudaStreamDestroy(b->cap);
  delete b;
  return PO_OK;
}

po_status po_batch_create(po_batch **out, int n_items, const po_config *configs, int n_streams) {
  if (!out || !configs || n_items <= 0) return fail(PO_ERR_INVALID_ARGUMENT, "null argument or empty batch");
  if (n_streams < 1 || n_streams > 64) return fail(PO_ERR_INVALID_ARGUMENT, "n_streams must be in [1, 64]");
  *out = nullptr;
  po_batch *b = new po_batch();
  b->n_streams = n_streams;
  cudaGetDevice(&b->device);
  for (int i = 0; i < n_items; ++i) {
    if (configs[i].precision == PO_PREC_FP64) {
      po_batch_destroy(b);
      return fail(PO_ERR_UNSUPPORTED, "batches run the FP32 / split-BF16 engine (no PO_PREC_FP64 items)");
    }
    po_ctx *c = nullptr;
    po_status s = po_create(&c, &configs[i]);
    if (s != PO_OK) {
      po_batch_destroy(b);
      return s;
    }
    b->ctx.push_back(c);
  }
  b->streams.assign(n_streams, nullptr);
  b->joins.assign(n_streams, nullptr);
  for (int k = 0; k < n_streams; ++k) {
    if (cudaStreamCreateWithFlags(&b->streams[k], cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->joins[k], cudaEventDisableTiming) != cudaSuccess) {
      po_batch_destroy(b);
      return fail(PO_ERR_CUDA, "stream / event creation failed");
    }
  }
  if (cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking) != cudaSuccess) {
    po_batch_destroy(b);
    return fail(PO_ERR_CUDA, "event / stream creation failed");
  }
  *out = b;
  return PO_OK;
}

// Estimated device work of a prepared item (multiply-adds of its leaf sums
// and level GEMMs), for the branch assignment.
static double plan_cost(const po_ctx *c, const SolvePlan &P) {
  const int d = c->depth;
  if (d == 0) return (double)P.S * (double)P.n * (double)P.nd_out;
  double w = (double)P.n * c->R[d] * c->Phi[d];
  for (int l = 0; l < d; ++l)
    w += (double)P.tree.level[l + 1].count * 6.0 * c->R[l + 1] * (double)c->Phi[l] * (c->Phi[l + 1] + 2.0 * c->R[l]);
  return (double)P.S * w;
}

po_status po_batch_prepare(po_batch *b, const po_batch_item *items, void *stream) {
  if (!b || !items) return fail(PO_ERR_INVALID_ARGUMENT, "null argument");
  int dev = 0;
  PO_CUDA(cudaGetDevice(&dev));
  if (dev != b->device) return fail(PO_ERR_INVALID_ARGUMENT, "batch was created on another device");
  const int n = (int)b->ctx.size();
  for (int i = 0; i < n; ++i) {
    const po_batch_item &it = items[i];
    if (!it.geom.on_device) return fail(PO_ERR_INVALID_ARGUMENT, "batch geometry must be device memory");
    if (!it.intensity) return fail(PO_ERR_INVALID_ARGUMENT, "null intensity of a batch item");
    if (it.geom.n < 0 || (it.geom.n > 0 && (!it.geom.x || !it.geom.y || !it.geom.z || !it.geom.nx || !it.geom.ny ||
                                             !it.geom.nz || !it.geom.area)))
      return fail(PO_ERR_INVALID_ARGUMENT, "null geometry array in a batch item");
    const po_illum &il = it.illum;
    if (il.n_lambda <= 0 || !il.lambda_m || il.n_inc <= 0 || !il.theta_i || !il.phi_i || !(il.sigma > 0) ||
        (il.pol_mask & (PO_POL_TM | PO_POL_TE)) == 0 || (il.pol_mask & ~(PO_POL_TM | PO_POL_TE)))
      return fail(PO_ERR_INVALID_ARGUMENT, "invalid illumination in a batch item");
    for (int l = 0; l < il.n_lambda; ++l)
      if (!(il.lambda_m[l] > 0) || !std::isfinite(il.lambda_m[l]))
        return fail(PO_ERR_INVALID_ARGUMENT, "wavelengths must be positive");
  }
  cudaStream_t st = (cudaStream_t)stream;
  batch_release_graph(b);
  const auto t0 = std::chrono::steady_clock::now();
  b->plans.assign(n, SolvePlan());
  for (int i = 0; i < n; ++i) PO_TRY(prepare_solve(b->ctx[i], &items[i].geom, &items[i].illum, false, st, b->plans[i]));
  // branch assignment: longest estimated item first onto the least loaded branch
  std::vector<int> order(n);
  std::vector<double> cost(n);
  for (int i = 0; i < n; ++i) {
    order[i] = i;
    cost[i] = plan_cost(b->ctx[i], b->plans[i]);
  }
  std::sort(order.begin(), order.end(), [&](int a, int c) { return cost[a] > cost[c]; });
  std::vector<double> load(b->n_streams, 0.0);
  b->branch.assign(n, 0);
  std::vector<std::vector<int>> per(b->n_streams);
  for (int i : order) {
    int k = (int)(std::min_element(load.begin(), load.end()) - load.begin());
    b->branch[i] = k;
    load[k] += cost[i];
    per[k].push_back(i);
  }
  // capture on the batch's own stream: fork onto the branches, enqueue, join
  PO_CUDA(cudaStreamSynchronize(st));
  const cudaStream_t cap = b->cap;
  PO_CUDA(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
  po_status s = PO_OK;
  cudaError_t e = cudaEventRecord(b->fork, cap);
  if (e != cudaSuccess) s = cuda_fail(e, "cudaEventRecord(fork)");
  for (int k = 0; k < b->n_streams && s == PO_OK; ++k) {
    e = cudaStreamWaitEvent(b->streams[k], b->fork, 0);
    if (e != cudaSuccess) s = cuda_fail(e, "cudaStreamWaitEvent(fork)");
    for (int i : per[k]) {
      if (s != PO_OK) break;
      s = enqueue_solve(b->ctx[i], b->plans[i], items[i].intensity, nullptr, b->streams[k], nullptr);
    }
    if (s == PO_OK) {
      e = cudaEventRecord(b->joins[k], b->streams[k]);
      if (e != cudaSuccess) s = cuda_fail(e, "cudaEventRecord(join)");
    }
    if (s == PO_OK) {
      e = cudaStreamWaitEvent(cap, b->joins[k], 0);
      if (e != cudaSuccess) s = cuda_fail(e, "cudaStreamWaitEvent(join)");
    }
  }
  cudaGraph_t g = nullptr;
  e = cudaStreamEndCapture(cap, &g);
  if (s != PO_OK) {
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    return s;
  }
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
  b->graph = g;
  e = cudaGraphInstantiate(&b->exec, g, 0);
  if (e != cudaSuccess) {
    batch_release_graph(b);
    return cuda_fail(e, "cudaGraphInstantiate");
  }
  size_t nn = 0;
  if (cudaGraphGetNodes(g, nullptr, &nn) == cudaSuccess) b->nodes = (int64_t)nn;
  PO_CUDA(cudaStreamSynchronize(st));
  b->ms_prepare = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return PO_OK;
}

po_status po_batch_launch(po_batch *b, void *stream) {
  if (!b) return fail(PO_ERR_INVALID_ARGUMENT, "null batch");
  if (!b->exec) return fail(PO_ERR_INVALID_ARGUMENT, "po_batch_prepare has not captured a graph");
  PO_CUDA(cudaGraphLaunch(b->exec, (cudaStream_t)stream));
  return PO_OK;
}

po_status po_batch_check(po_batch *b, void *stream) {
  if (!b) return fail(PO_ERR_INVALID_ARGUMENT, "null batch");
  PO_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
  po_status first = PO_OK;
  std::string msg;
  for (size_t i = 0; i < b->ctx.size(); ++i) {
    const po_status s = check_device_waits(b->ctx[i]);
    if (s != PO_OK && first == PO_OK) {
      first = s;
      msg = "batch item " + std::to_string(i) + ": " + po_last_error();
    }
  }
  return first == PO_OK ? PO_OK : fail(first, msg);
}

po_status po_batch_info(const po_batch *b, int64_t *graph_nodes, int64_t *workspace_bytes, double *ms_prepare) {
  if (!b) return fail(PO_ERR_INVALID_ARGUMENT, "null batch");
  if (graph_nodes) *graph_nodes = b->nodes;
  if (ms_prepare) *ms_prepare = b->ms_prepare;
  if (workspace_bytes) {
    int64_t ws = 0;
    for (const po_ctx *c : b->ctx)
      for (const DevBuf *d : {&c->twiddles, &c->geom_in, &c->geom_sorted, &c->octree_ws, &c->leaf_ctr, &c->dirs,
                              &c->dirs_d, &c->trans, &c->levelA, &c->levelB, &c->mid, &c->slots, &c->kvals, &c->out,
                              &c->cur, &c->partial, &c->tile_ctr, &c->amat, &c->bmat})
        ws += (int64_t)d->bytes;
    *workspace_bytes = ws;
  }
  return PO_OK;
}

}  // extern "C"
