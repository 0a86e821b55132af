// po_noalloc.cu -- po_interp_fft_noalloc: the angular interpolation of
// po_interp_fft with its scratch in a fixed device array instead of memory
// taken from an allocator.
//
// Some callers must not allocate or free device memory while they run: host
// applications that own a fixed device-memory budget and forbid library-side
// allocations (plugins inside a renderer or a simulation runtime), and code
// paths that cannot afford an allocator call or its failure.  For them the
// scratch lives in `g_noalloc_scratch`, a file-scope __device__ array of
// PO_NOALLOC_SCRATCH_BYTES that every GPU loading this library holds until the
// process exits.
//
// The array's name is only a host-side stand-in in host code, so its device
// address is looked up once per device with cudaGetSymbolAddress (on the
// first call on that device, with that device current) and cached.  Every
// call shares the array: calls that overlap on the GPU (different streams, or
// different host threads on one device) race on it.  Nothing in it needs to
// start at zero: each call writes its twiddle tables and every scratch element
// it later reads.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>

#include "po_common.cuh"
#include "po_internal.h"
#include "po_kernels.h"

namespace wavepo {
namespace {

static __device__ __align__(256) unsigned char g_noalloc_scratch[PO_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void *g_scratch_dev[kMaxDevices] = {};

// Device address of the scratch array on the current device (set-up on the
// first call per device).
po_status scratch_address(void **out) {
  int dev = 0;
  PO_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return fail(PO_ERR_UNSUPPORTED, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_dev[dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    g_scratch_dev[dev] = p;
  }
  *out = g_scratch_dev[dev];
  return PO_OK;
}

}  // namespace
}  // namespace wavepo

using namespace wavepo;

extern "C" po_status po_interp_fft_noalloc(const float *in, int th_c, int ph_c, float *out, int th_p, int ph_p,
                                           int batch, int theta_mode, int nyquist_quirk, void *stream) {
  if (!in || !out || th_c <= 0 || ph_c <= 0 || batch < 0) return fail(PO_ERR_INVALID_ARGUMENT, "invalid argument");
  if (th_p < th_c || ph_p < ph_c) return fail(PO_ERR_INVALID_ARGUMENT, "the interpolation only upsamples");
  if (theta_mode != PO_THETA_DOUBLE_COVER && theta_mode != PO_THETA_REFERENCE)
    return fail(PO_ERR_INVALID_ARGUMENT, "unknown theta mode");
  // scratch layout: twiddle tables of the distinct lengths, then the row-pass
  // output [batch][th_c][ph_p] complex64 at the next 256-byte boundary
  int lens[4] = {ph_c, ph_p, th_c, th_p};
  std::sort(lens, lens + 4);
  int nl = (int)(std::unique(lens, lens + 4) - lens);
  int off[4], total = 0;
  for (int i = 0; i < nl; ++i) { off[i] = total; total += lens[i]; }
  const size_t tw_bytes = ((sizeof(float2) * (size_t)total + 255) / 256) * 256;
  const size_t mid_bytes = sizeof(float2) * (size_t)batch * (size_t)th_c * (size_t)ph_p;
  if (tw_bytes + mid_bytes > (size_t)PO_NOALLOC_SCRATCH_BYTES)
    return fail(PO_ERR_INVALID_ARGUMENT,
                "po_interp_fft_noalloc: batch*th_c*ph_p*8 bytes plus the twiddle tables exceed the fixed scratch of "
                "PO_NOALLOC_SCRATCH_BYTES; use po_interp_fft or split the batch");
  if (batch == 0) return PO_OK;
  void *base = nullptr;
  {
    int dev = 0;
    PO_CUDA(cudaGetDevice(&dev));
    PO_TRY(init_device_attributes(dev));
  }
  PO_TRY(scratch_address(&base));
  float2 *tw = (float2 *)base;
  float2 *mid = (float2 *)((char *)base + tw_bytes);
  cudaStream_t st = (cudaStream_t)stream;
  auto offset_of = [&](int n) {
    for (int i = 0; i < nl; ++i)
      if (lens[i] == n) return off[i];
    return 0;
  };
  for (int i = 0; i < nl; ++i) PO_TRY(launch_twiddles(lens[i], tw + off[i], st));
  int dev = 0, sm = 152;
  PO_CUDA(cudaGetDevice(&dev));
  cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, dev);
  PO_TRY(launch_interp_rows((const float2 *)in, mid, (int64_t)batch * th_c, make_plan(ph_c, offset_of(ph_c)),
                            make_plan(ph_p, offset_of(ph_p)), tw, 1.0f / (float)ph_c, sm,
                            theta_mode == PO_THETA_REFERENCE ? 1 : 0, st));
  int reach = (theta_mode == PO_THETA_REFERENCE && nyquist_quirk) ? 256 * (th_c / 256 + 1) : 0x7fffffff;
  PO_TRY(launch_interp_cols(mid, (float2 *)out, nullptr, batch, batch, ph_p, th_c, th_p,
                            make_plan(th_c, offset_of(th_c)), make_plan(th_p, offset_of(th_p)), tw, nullptr, 1, 1,
                            reach, 1.0f / (float)th_c, 1, 0, theta_mode == PO_THETA_REFERENCE ? 1 : 0, st));
  return PO_OK;
}
