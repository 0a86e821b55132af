// po_internal.h -- host-side declarations shared by the engine's translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "wavepo.h"

namespace wavepo {

// thread-local last error message (po_last_error)
void set_error(const std::string &msg);
po_status fail(po_status s, const std::string &msg);
po_status cuda_fail(cudaError_t e, const char *what);

#define PO_CUDA(call)                                         \
  do {                                                        \
    cudaError_t _e = (call);                                  \
    if (_e != cudaSuccess) return ::wavepo::cuda_fail(_e, #call); \
  } while (0)

#define PO_TRY(call)                   \
  do {                                 \
    po_status _s = (call);             \
    if (_s != PO_OK) return _s;        \
  } while (0)

// opt-in shared-memory attributes of the engine's kernels on a device (once)
po_status init_device_attributes(int dev);

// counts launches made by the engine (po_report.kernel_launches)
extern thread_local int64_t g_launch_count;
inline void count_launch() { ++g_launch_count; }

// ---------------------------------------------------------------- octree
struct OctreeLevel {
  int64_t count;          // active (non-empty) nodes
  int32_t *begin;         // [count+1] first sorted point of each node (begin[count] = n)
  int32_t *parent;        // [count] index of the parent in the level above (level>0)
  int32_t *child;         // [count*8] index of child octant o in the level below or -1
  uint32_t *prefix;       // [count] octant path (3 bits per level, root first)
};

struct OctreeBuffers {
  int depth = 0;
  int64_t n = 0;
  int32_t *perm = nullptr;        // sorted position -> input index
  uint32_t *keys = nullptr;       // sorted keys
  OctreeLevel level[PO_MAX_DEPTH + 1];
};

// Device scratch needed by build_octree for n points and the given depth.
size_t octree_workspace_bytes(int64_t n, int depth);
// Builds the tree of the reference (float centre comparisons, stable octant
// order).  `ws` must hold octree_workspace_bytes; level arrays are carved
// from it.  Copies the per-level counts to the host (one synchronisation).
po_status build_octree(const float *x, const float *y, const float *z, int64_t n, const float box_min[3],
                       const float box_max[3], int depth, void *ws, size_t ws_bytes, OctreeBuffers *out,
                       cudaStream_t st);
// Fills the (begin, end) of every heap node from the sorted keys.
po_status octree_heap_ranges(const OctreeBuffers &t, int32_t *heap_range, cudaStream_t st);

// gathers SoA float arrays by perm: dst[k][i] = src[k][perm[i]]
po_status gather_points(int64_t n, const int32_t *perm, const float *const src[7], float *const dst[7],
                        cudaStream_t st);

}  // namespace wavepo
