// po_selftest.cu -- self-test of the failure paths of the bounded device
// waits (po_selftest_device_waits).  No counterpart in the reference, which
// reports nothing but exit() (util/helper_cuda.h:583-595).
//
// Each case launches one tcgen05 kernel of the engine on small buffers of its
// own, set up so that the kernel must take a failure path, then reads and
// clears the kernel's error word:
//   1  theta pass (k_theta_tc) told that its theta matrices are 0 bytes long:
//      the per-CTA operand check fails before any copy is issued (word 2);
//   2  theta pass with the first stage's copies withheld: the MMA and
//      epilogue waits give up after their time limit (word 1);
//   3  tcgen05 leaf sums (k_leaf_tc) with the first stage's copy withheld
//      (word 1).
// In every case the roles abort together, the copies already issued land
// before the CTA exits and the tensor memory is released, so the context
// stays usable.  No wait is endless and nothing faults.
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "po_common.cuh"
#include "po_internal.h"
#include "po_kernels.h"

using namespace wavepo;

namespace {

struct Scratch {
  std::vector<void *> bufs;
  ~Scratch() {
    for (void *p : bufs) cudaFree(p);
  }
  po_status alloc(void **p, size_t bytes) {
    *p = nullptr;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(self-test buffer)");
    bufs.push_back(*p);
    return cudaMemset(*p, 0, bytes) == cudaSuccess ? PO_OK : fail(PO_ERR_CUDA, "cudaMemset");
  }
};

po_status theta_case(bool withhold, int *err, cudaStream_t st) {
  Scratch S;
  const int phi = 128, Kr = 16, Rp = 128;
  const size_t mid_bytes = (size_t)8 * theta_tc_npad(phi) * Kr, atc_bytes = theta_tc_bytes(Rp, Kr);
  void *mid, *atc, *trans, *parent, *child;
  PO_TRY(S.alloc(&mid, mid_bytes));
  PO_TRY(S.alloc(&atc, atc_bytes));
  PO_TRY(S.alloc(&trans, sizeof(float4) * Rp * phi));
  PO_TRY(S.alloc(&parent, sizeof(float2) * 6 * Rp * phi));
  PO_TRY(S.alloc(&child, sizeof(int32_t) * 8));
  const int32_t table[8] = {0, -1, -1, -1, -1, -1, -1, -1};
  PO_CUDA(cudaMemcpy(child, table, sizeof(table), cudaMemcpyHostToDevice));
  PO_TRY(launch_theta_tc((const uint8_t *)mid, (float2 *)parent, (const int32_t *)child, 1, 1, phi, Kr, Rp,
                         (const uint8_t *)atc, (const float4 *)trans, 1, 1, err, mid_bytes,
                         withhold ? atc_bytes : 0, st, withhold ? 1 : 0));
  PO_CUDA(cudaStreamSynchronize(st));
  return PO_OK;
}

po_status leaf_case(int *err, cudaStream_t st) {
  Scratch S;
  const int npts = 16, ndir = 128;
  void *pts, *begin, *kc0, *chunk, *ctr, *slot, *dirs, *bop, *uop, *out;
  PO_TRY(S.alloc(&pts, sizeof(float) * 7 * npts));
  PO_TRY(S.alloc(&begin, sizeof(int32_t) * 2));
  PO_TRY(S.alloc(&kc0, sizeof(int32_t) * 2));
  PO_TRY(S.alloc(&chunk, sizeof(int32_t)));
  PO_TRY(S.alloc(&ctr, sizeof(double) * 3));
  PO_TRY(S.alloc(&slot, sizeof(SlotParams<float>)));
  PO_TRY(S.alloc(&dirs, sizeof(float4) * ndir));
  const size_t bop_bytes = leaf_tc_col_tiles(1) * leaf_tc_block_bytes(), uop_bytes = sizeof(float4) * 16;
  PO_TRY(S.alloc(&bop, bop_bytes));
  PO_TRY(S.alloc(&uop, uop_bytes));
  PO_TRY(S.alloc(&out, sizeof(float2) * 6 * ndir));
  // 16 points on a small disc facing -x, lit by a wave along +x
  std::vector<float> g(7 * npts, 0.f);
  for (int i = 0; i < npts; ++i) {
    g[1 * npts + i] = 1e-8f * std::cos(0.4f * i);
    g[2 * npts + i] = 1e-8f * std::sin(0.4f * i);
    g[3 * npts + i] = -1.f;
    g[6 * npts + i] = 1e-16f;
  }
  PO_CUDA(cudaMemcpy(pts, g.data(), sizeof(float) * g.size(), cudaMemcpyHostToDevice));
  const int32_t b[2] = {0, npts}, k[2] = {0, 1};
  PO_CUDA(cudaMemcpy(begin, b, sizeof(b), cudaMemcpyHostToDevice));
  PO_CUDA(cudaMemcpy(kc0, k, sizeof(k), cudaMemcpyHostToDevice));
  const SlotParams<float> sp = make_slot<float>(500e-9, 0.0, 0.0, false, 1.55, 0.0, 1e-2, 1.0, true);
  PO_CUDA(cudaMemcpy(slot, &sp, sizeof(sp), cudaMemcpyHostToDevice));
  std::vector<float4> dv(ndir);
  for (int i = 0; i < ndir; ++i) dv[i] = make_float4(std::cos(0.05f * i), std::sin(0.05f * i), 0.f, 0.f);
  PO_CUDA(cudaMemcpy(dirs, dv.data(), sizeof(float4) * ndir, cudaMemcpyHostToDevice));
  const float *gp[7];
  for (int q = 0; q < 7; ++q) gp[q] = (const float *)pts + q * npts;
  PO_TRY(launch_leaf_tc(gp, (const int32_t *)begin, (const int32_t *)kc0, (const int32_t *)chunk, 1,
                        (const double *)ctr, 1, (const SlotParams<float> *)slot, 1, 1, 0, 1, (const float4 *)dirs,
                        ndir, (uint8_t *)bop, bop_bytes, (float4 *)uop, uop_bytes, (float2 *)out, err, st,
                        kLeafTcMaxSlots, 1));
  PO_CUDA(cudaStreamSynchronize(st));
  return PO_OK;
}

}  // namespace

extern "C" po_status po_selftest_device_waits(int which, void *stream) {
  if (which < 1 || which > 3) return fail(PO_ERR_INVALID_ARGUMENT, "self-test case must be 1, 2 or 3");
  int dev = 0;
  PO_CUDA(cudaGetDevice(&dev));
  PO_TRY(init_device_attributes(dev));
  cudaStream_t st = (cudaStream_t)stream;
  int *err = nullptr;
  PO_CUDA(cudaMalloc(&err, sizeof(int)));
  po_status s = cudaMemset(err, 0, sizeof(int)) == cudaSuccess ? PO_OK : fail(PO_ERR_CUDA, "cudaMemset");
  if (s == PO_OK) s = which == 3 ? leaf_case(err, st) : theta_case(which == 2, err, st);
  int h = 0;
  if (s == PO_OK && cudaMemcpy(&h, err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
    s = fail(PO_ERR_CUDA, "read-back of the error word");
  cudaFree(err);
  if (s != PO_OK) return s;
  if (h == 2) return fail(PO_ERR_INTERNAL, "self-test: operand run outside its buffer (detected, nothing copied)");
  if (h == 1) return fail(PO_ERR_TIMEOUT, "self-test: a device wait timed out (detected, roles aborted)");
  return PO_OK;
}
