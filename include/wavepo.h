/*
 * wavepo.h -- C ABI of the GB300-native physical-optics (PO) far-field engine.
 *
 * The reference (WaveFiber3d) has no library interface: its PO path is a set
 * of header-only host functions that each driver main() calls in a fixed
 * order (compareMie/sphere.cu:581-936).  Every entry point below states the
 * reference function(s) it replaces.  All of them
 *   - take plain pointers and sizes (no C++ or framework types),
 *   - order their GPU work on the caller's CUDA stream (`stream`, may be NULL
 *     for the legacy default stream),
 *   - report errors through po_status and never exit the process (the
 *     reference calls exit() from checkCudaErrors, util/helper_cuda.h:583-595).
 * Device pointers must be valid on the current CUDA device.
 */
#ifndef WAVEPO_H
#define WAVEPO_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PO_MAX_DEPTH 10

typedef enum po_status {
  PO_OK = 0,
  PO_ERR_INVALID_ARGUMENT = 1,
  PO_ERR_CUDA = 2,
  PO_ERR_OUT_OF_MEMORY = 3,
  PO_ERR_UNSUPPORTED = 4,
  PO_ERR_TIMEOUT = 5,
  PO_ERR_INTERNAL = 6
} po_status;

/* Arithmetic of the far-field sums. */
typedef enum po_precision {
  PO_PREC_FP32 = 0,       /* FP32 sums, FP64 phase arguments where they are large */
  PO_PREC_FP64 = 1,       /* plain FP64 everywhere (depth 0 only) */
  PO_PREC_SPLIT_BF16 = 2, /* leaf sums as tensor-core hi+lo BF16 products, FP32 accumulation
                             (depth 0: the same tcgen05 sum over one leaf of all points) */
  PO_PREC_SPLIT_FP16 = 3  /* reserved: rejected with PO_ERR_UNSUPPORTED (the currents need
                             per-tile scaling to fit the FP16 range) */
} po_precision;

/* How the elevation axis is interpolated between tree levels. */
typedef enum po_theta_mode {
  /* theta sampled over [-pi/2, 3pi/2) (the sphere covered twice), so that the
   * trigonometric interpolation sees a smooth 2pi-periodic function */
  PO_THETA_DOUBLE_COVER = 0,
  /* as util/interpolation.h:48-77: theta over [-pi/2, pi/2) treated as
   * pi-periodic (accurate only when the pattern is small at both poles) */
  PO_THETA_REFERENCE = 1
} po_theta_mode;

/* Which kernel computes the leaf sums of a split-BF16 tree solve. */
typedef enum po_leaf_kernel {
  PO_LEAF_AUTO = 0,    /* tcgen05 from 8 patterns per wavelength, warp-level below */
  PO_LEAF_WARP = 1,    /* warp-level mma.sync, 4 patterns per CTA */
  PO_LEAF_TCGEN05 = 2  /* tcgen05 with tensor-memory accumulators, leaf_slots patterns per pass */
} po_leaf_kernel;

/* Polarisation mask: 'M' (TM) and 'E' (TE) of compareMie/sphere.cu:551-579. */
#define PO_POL_TM 1
#define PO_POL_TE 2

typedef struct po_config {
  int max_depth;                    /* octree depth, 0 = direct sum (sphere.cu:25) */
  int n_theta[PO_MAX_DEPTH + 1];    /* elevation samples over pi per level; [0] = output grid */
  int n_phi[PO_MAX_DEPTH + 1];      /* azimuth samples over 2pi per level; [0] = output grid */
  float box_min[3], box_max[3];     /* root bounding box (sphere.cu:212-216) */
  int precision;                    /* po_precision */
  int theta_mode;                   /* po_theta_mode */
  int nyquist_quirk;                /* PO_THETA_REFERENCE only: split the theta Nyquist bin
                                       only where interpolation.h:66's launch reaches */
  double distance;                  /* observer distance Dis of the prefactors (sphere.cu:46) */
  int interp_method;                /* po_interp_method of the phi and theta passes between levels */
  int64_t max_workspace_bytes;      /* device workspace cap of one solve; the patterns are
                                       processed in chunks of slots that fit (0 = half of
                                       the device's memory) */
  int interp_tile;                  /* complex columns per CTA of the warp-level tensor-core
                                       theta pass (levels with few rows; autotuner knob):
                                       0 = automatic, 8 or 16 */
  int leaf_kernel;                  /* po_leaf_kernel (split BF16 only; autotuner knob) */
  int leaf_slots;                   /* patterns of one wavelength per pass of the tcgen05 leaf
                                       kernel: 0 = 64, else a multiple of 8 up to 64 */
} po_config;

/* How the angular interpolation between tree levels (phi pass, then theta
 * pass with translation and child sum) is computed. */
typedef enum po_interp_method {
  PO_INTERP_FFT = 0,    /* shared-memory batched FFTs (any theta mode) */
  PO_INTERP_TENSOR = 1  /* the level's trigonometric interpolation matrices as split hi+lo
                           BF16 tensor-core products, for both passes: tcgen05 with
                           tensor-memory accumulators on levels whose rows fill 128-row
                           tiles, warp-level mma.sync on the others.  In the reference
                           theta mode two kinds of level keep the FFTs: those where the
                           Nyquist quirk of interpolation.h:66 reaches a parent column (a
                           complex, column-dependent map) and those between equal sizes */
} po_interp_method;

typedef struct po_geometry {
  int64_t n;                        /* number of surface points */
  const float *x, *y, *z;           /* positions (m), SoA (sphere.cu:94-125) */
  const float *nx, *ny, *nz;        /* unit outward normals */
  const float *area;                /* area per point (m^2) */
  int on_device;                    /* 1: device pointers, 0: host pointers */
} po_geometry;

typedef struct po_illum {
  int n_lambda;                     /* wavelengths (m): sphere.cu:486-490 loops over these */
  const double *lambda_m;
  int n_inc;                        /* incident directions (radians, elevation/azimuth as */
  const double *theta_i;            /*   treePO.cu:559-564 and sphere.cu:544-562)          */
  const double *phi_i;
  int pol_mask;                     /* PO_POL_TM | PO_POL_TE */
  double eta_re, eta_im;            /* complex index of refraction of the scatterer */
  double sigma;                     /* Gaussian beam width (m), tangentplane.h:33-34 */
} po_illum;

typedef struct po_report {
  double ms_total;                  /* device time of the whole solve (CUDA events) */
  double ms_build;                  /* octree build */
  double ms_leaf;                   /* leaf / direct far-field sums */
  double ms_aggregate;              /* interpolation + translation + child sums */
  double ms_intensity;              /* projection, intensity, output copy */
  int64_t n_leaves;                 /* active nodes at the deepest level */
  int64_t n_nodes_total;            /* active nodes over all levels */
  int root_theta, root_phi;         /* root grid actually used (output x supersampling) */
  int64_t workspace_bytes;          /* device workspace held by the context */
  int64_t kernel_launches;          /* kernels launched by the solve */
  double ms_leaf_kernel;            /* the leaf (or direct-sum) kernel launches alone */
  double ms_rows;                   /* all row (phi) interpolation launches */
  double ms_cols;                   /* all column (theta) interpolation + child-sum launches */
  int n_leaf_launches, n_row_launches, n_col_launches;
  int n_chunks;                     /* slot chunks the patterns were processed in */
  int chunk_slots;                  /* patterns per chunk (the last may be smaller) */
  double leaf_point_dirs;           /* sum over leaves of points x leaf directions x patterns */
  double rows_bytes, cols_bytes;    /* algorithmic bytes (pattern reads + writes) of the passes */
  double ms_rows_level[PO_MAX_DEPTH];  /* ms_rows and ms_cols split by parent level l = 0..depth-1 */
  double ms_cols_level[PO_MAX_DEPTH];
  double agg_bytes;                 /* algorithmic bytes of the aggregation: per level, the child
                                       patterns read at the child grid + the parent patterns written */
  int64_t n_nodes_level[PO_MAX_DEPTH + 1];  /* active nodes per level (0 = root) */
} po_report;

typedef struct po_ctx po_ctx;

/* ---- configuration helpers --------------------------------------------- */

/* Fills cfg with defaults and the per-level grids of the reference rule
 * n(i) = ceil(k d_i + beta (k d_i)^(1/3)), k = 2 pi / lambda_min,
 * d_i = 0.5^i * extent * ratio (compareMie/sphere.cu:345-352,
 * fibersim/treePO.cu:353-359).  Level 0 is the n_theta_out x n_phi_out grid. */
po_status po_config_init(po_config *cfg, int max_depth, int n_theta_out, int n_phi_out,
                         const float box_min[3], const float box_max[3], double theta_extent,
                         double phi_extent, double ratio, double beta, double lambda_min);

const char *po_status_string(po_status s);
/* Message of the last failing call on this host thread (never NULL). */
const char *po_last_error(void);

/* ---- whole solve (replaces the driver main() of sphere.cu / ellipsoid.cu /
 *      treePO.cu from the octree build to the intensity write, :212-936) --- */

po_status po_create(po_ctx **ctx, const po_config *cfg);
po_status po_destroy(po_ctx *ctx);
/* intensity: [n_lambda][n_inc][n_pol][n_theta[0]][n_phi[0]] float32, host or
 * device memory (out_on_device).  Polarisations in the order TM, TE. */
po_status po_solve(po_ctx *ctx, const po_geometry *geom, const po_illum *illum, float *intensity,
                   int out_on_device, void *stream, po_report *report);

/* No counterpart in the reference (it reports failures only by exit()).
 * Waits for the stream and reports whether a bounded device wait of the
 * context's kernels gave up since the last check (the output of that solve
 * is then incomplete): PO_ERR_TIMEOUT, or PO_ERR_INTERNAL for an operand run
 * outside its buffer; clears the record.  A synchronous solve (report
 * requested or host output) performs this check itself; callers of
 * asynchronous solves call po_check before they trust the output. */
po_status po_check(po_ctx *ctx, void *stream);

/* No counterpart in the reference (it has no gradients).  Gradient of a
 * scalar loss L with respect to every surface sample, given dL/dI on the
 * output grid: dl_di [n_lambda][n_inc][n_pol][n_theta[0]][n_phi[0]] float32
 * (device).  grad (device, float32 [7][n], overwritten) receives dL/dx,
 * dL/dy, dL/dz, dL/dnx, dL/dny, dL/dnz, dL/darea in the input point order;
 * normals are differentiated as given (no renormalisation).  The forward
 * solve is recomputed (intensity, if not NULL, receives it on the device);
 * then the root adjoint, the exact transpose of the tree aggregation (or of
 * the depth-0 sum) and the derivative of the tangent-plane currents give the
 * gradient of the discrete map the engine evaluates.  Needs double-cover
 * theta and PO_INTERP_TENSOR when max_depth > 0 (else PO_ERR_UNSUPPORTED);
 * PO_PREC_FP64 runs the whole chain in FP64 (depth 0).  The gradient is
 * piecewise: the octree assignment and the lit/shadow switch of every point
 * are held fixed. */
po_status po_grad(po_ctx *ctx, const po_geometry *geom, const po_illum *illum, const float *dl_di, float *grad,
                  float *intensity, void *stream, po_report *report);

/* ---- batches of independent solves (no counterpart in the reference) ----
 * Many geometries, each with its own configuration and illumination, run as
 * one CUDA graph: po_batch_prepare builds every octree and table (host
 * synchronisations happen here) and captures the pattern computations of all
 * items into a graph whose branches run concurrently (items spread over
 * n_streams branches, longest estimated first); po_batch_launch replays it on
 * a stream.  Items keep their own workspaces, so a replay recomputes every
 * pattern from the prepared trees (the geometry arrays must not move).
 * Geometry and intensity pointers are device memory. */
typedef struct po_batch po_batch;
typedef struct po_batch_item {
  po_geometry geom;                 /* on_device must be 1 */
  po_illum illum;
  float *intensity;                 /* [n_lambda][n_inc][n_pol][n_theta[0]][n_phi[0]] of its config */
} po_batch_item;
po_status po_batch_create(po_batch **batch, int n_items, const po_config *configs, int n_streams);
po_status po_batch_prepare(po_batch *batch, const po_batch_item *items, void *stream);
po_status po_batch_launch(po_batch *batch, void *stream);
/* po_check for every item of a replayed batch (waits for the stream): the
 * first item whose kernels gave up a bounded wait, or PO_OK. */
po_status po_batch_check(po_batch *batch, void *stream);
/* graph nodes, device workspace of all items, host+device time of the last
 * prepare (ms); any pointer may be NULL */
po_status po_batch_info(const po_batch *batch, int64_t *graph_nodes, int64_t *workspace_bytes, double *ms_prepare);
po_status po_batch_destroy(po_batch *batch);

/* ---- single steps of the path (device pointers) ------------------------ */

/* util/tangentplane.h:84-92 (computeLocalTangentPlane) and, when scale != 0,
 * util/fields.h:123 (field_times_area) and :147 (multiply_current_factor) with
 * the prefactors of compareMie/sphere.cu:491-494.
 * currents: n x [Jx,Jy,Jz,Mx,My,Mz] complex64 (float2 pairs), point-major. */
po_status po_tangent_plane_currents(int64_t n, const float *x, const float *y, const float *z,
                                    const float *nx, const float *ny, const float *nz, const float *area,
                                    double lambda_m, double theta_i, double phi_i, int pol, double eta_re,
                                    double eta_im, double sigma, double distance, int scale, float *currents,
                                    void *stream);

/* util/tree.h:289-715 (build_octree_kernel) + compareMie/sphere.cu:255-307.
 * perm[i] = input index of the point at tree position i (the stable octant
 * order of the reference).  heap_range, if not NULL, receives (begin, end)
 * for every node of the full 8-ary heap of (8^(depth+1)-1)/7 nodes, in the
 * reference's heap order. */
po_status po_build_octree(int64_t n, const float *x, const float *y, const float *z, const float box_min[3],
                          const float box_max[3], int depth, int32_t *perm, int32_t *heap_range, void *stream);

/* current_times_green_center + thrust::reduce over all points
 * (util/fields.h:2-50, compareMie/sphere.cu:603-658 at depth 0):
 * F_c(s) = sum_p exp(+i k s.(x_p - center)) cur_p[c] on an n_theta x n_phi grid.
 * currents: n x 6 complex64 (as above); fields out: [6][n_theta][n_phi] complex64
 * (the reference's separate Ex..Hz arrays).  precision: PO_PREC_FP32 or PO_PREC_FP64. */
po_status po_far_field_direct(int64_t n, const float *x, const float *y, const float *z, const float *currents,
                              double k, const double center[3], int n_theta, int n_phi, int precision,
                              float *fields, void *stream);

/* util/interpolation.h:82-93 (copyandinterp -> interpFFT): trigonometric
 * upsampling of `batch` patterns [th_c][ph_c] -> [th_p][ph_p] (complex64),
 * phi first, then theta, with hand-written shared-memory FFTs.
 * theta_mode PO_THETA_REFERENCE treats theta as pi-periodic exactly as the
 * reference; PO_THETA_DOUBLE_COVER expects th_c / th_p samples over 2pi.
 * Scratch of batch*th_c*ph_p complex64 is taken from the stream-ordered
 * allocator. */
po_status po_interp_fft(const float *in, int th_c, int ph_c, float *out, int th_p, int ph_p, int batch,
                        int theta_mode, int nyquist_quirk, void *stream);

/* No counterpart in the reference.  The interpolation of po_interp_fft for
 * callers that must not allocate or free device memory while they run (host
 * applications that own a fixed device-memory budget, plugins, code paths that
 * cannot afford an allocator call or its failure).  Its scratch is one fixed
 * device array of PO_NOALLOC_SCRATCH_BYTES per GPU that loads this library,
 * held until the process exits; a call needs
 *   batch*th_c*ph_p*8 bytes + the twiddle tables (8 bytes per sample of each
 *   distinct length among th_c, ph_c, th_p, ph_p, rounded up to 256 bytes)
 * and larger requests are rejected with PO_ERR_INVALID_ARGUMENT.  The first
 * call on a device looks up the array's device address (make it before any
 * stream capture).  All calls share the array: calls that overlap on the GPU
 * race.  The looked-up address is cached per device for the life of the
 * process; after a cudaDeviceReset it would be stale, so a process that resets
 * a device must not call this function on it again.  The output is complete
 * in stream order; the call does not synchronise. */
#define PO_NOALLOC_SCRATCH_BYTES (16u << 20)
po_status po_interp_fft_noalloc(const float *in, int th_c, int ph_c, float *out, int th_p, int ph_p, int batch,
                                int theta_mode, int nyquist_quirk, void *stream);

/* util/fields.h:172-204 (computeintensity): projection onto the transverse
 * plane and |E - Z0 s x H|^2.  fields: [6][n_theta][n_phi] complex64. */
po_status po_compute_intensity(const float *fields, int n_theta, int n_phi, float *intensity, void *stream);

/* util/geometry.h:3-75 and :76-179 (set_sourcepoint, full ring and ring
 * segment; the segment form is the one fibersim/treePO.cu:132 calls): a fiber
 * surface given as a quad grid of vertices -> one surface sample per quad.
 * height: device float32 [2][numel][numelvert], plane 0 = x, plane 1 = y of
 * vertex (j, i) at j*numelvert + i (fibersim/treePO.cu:83-86 file layout);
 * z_i = i*unitz - period/2.  Quads i in [0, numelvert), j in
 * [ring_begin, ring_end] (the full ring is 0 .. numel-1); outputs (device,
 * (ring_end-ring_begin+1)*numelvert floats each) at i*(ring_end-ring_begin+1)
 * + (j-ring_begin): vertex average, area 0.5(|a1| + |a2|) of the two triangle
 * cross products, unit normal along a1 + a2.  Results equal the reference's
 * float arithmetic bit for bit.  A vertex at the origin, which the reference
 * rejects with exit(1), returns PO_ERR_INVALID_ARGUMENT.  Synchronises the
 * stream (reads the status flag). */
po_status po_height_field_points(const float *height, int numel, int numelvert, float period, float unitz,
                                 int ring_begin, int ring_end, float *x, float *y, float *z, float *nx, float *ny,
                                 float *nz, float *area, void *stream);

/* No counterpart in the reference.  Adjoint of po_height_field_points:
 * given dL/d(sample) (device float32 [7][n] in the sample order of
 * po_height_field_points: x, y, z, nx, ny, nz, area), writes dL/d(vertex)
 * into grad_height (device float32 [2][numel][numelvert], overwritten;
 * vertices outside the ring segment get 0).  Derivatives are taken in FP64
 * per quad and accumulated with atomics. */
po_status po_height_field_adjoint(const float *height, int numel, int numelvert, float period, float unitz,
                                  int ring_begin, int ring_end, const float *grad_samples, float *grad_height,
                                  void *stream);

/* util/fields.h:206-234 (average_cpu): box average of n_patterns float32
 * patterns [nth_in][nph_in] onto [nth_out][nph_out] (device pointers), phi
 * first, then theta.  As in the reference the ratios are the integer
 * quotients nth_in / nth_out and nph_in / nph_out, so when they do not divide
 * evenly only the first ratio*n_out rows / columns contribute (for the fiber
 * preset 450 x 880 -> 180 x 360: ratios 2 and 2, rows 0..359 and columns
 * 0..719).  Results equal the reference's float arithmetic bit for bit. */
po_status po_average_pattern(const float *in, int nth_in, int nph_in, float *out, int nth_out, int nph_out,
                             int n_patterns, void *stream);

/* fitting/fittingutil.py:22-33 (ForwardFFT_shifted, inverse = 0): for each
 * of `batch` complex64 arrays [n_theta][n_phi] (device), roll by floor(n/2)
 * along both axes, unnormalised forward 2-D DFT (FFTW / numpy sign
 * convention), roll back by -floor(n/2).  inverse = 1 is InverseFFT_shifted
 * (fittingutil.py:35-46): roll by -floor(n/2), unnormalised backward DFT
 * (FFTW_BACKWARD, no 1/n), roll by +floor(n/2).  out may equal in.  FP32
 * accumulation, twiddles exact to FP32 rounding.  Scratch from the
 * stream-ordered allocator. */
po_status po_shifted_fft2(const float *in, float *out, int batch, int n_theta, int n_phi, int inverse,
                          void *stream);

/* fitting/fittingutil.py:67-74 (ACFfromFT) with the mean of :55-65
 * (weightedsum): patterns = n_inst real float32 arrays [n_theta][n_phi]
 * (device, instance-major); outputs (device, [n_theta][n_phi]): the mean over
 * the instances, spectrum = mean_i |ForwardFFT_shifted(pattern_i - mean)| and
 * acf = Re ForwardFFT_shifted(spectrum^2). */
po_status po_acf_from_patterns(const float *patterns, int n_inst, int n_theta, int n_phi, float *mean,
                               float *spectrum, float *acf, void *stream);

/* No counterpart in the reference.  Self-test of the failure handling of the
 * bounded device waits: launches one tcgen05 kernel of the engine on small
 * internal buffers, arranged so that it must fail, and returns the status its
 * error word maps to.  which = 1: the theta pass sees its operand buffer as
 * too small (expected PO_ERR_INTERNAL, no copy issued); 2: the theta pass
 * with its first copy stage withheld (expected PO_ERR_TIMEOUT after the 1-s
 * wait limit); 3: the tcgen05 leaf sums likewise (PO_ERR_TIMEOUT).  PO_OK
 * would mean the failure went undetected.  The CUDA context stays usable. */
po_status po_selftest_device_waits(int which, void *stream);

/* Library build identification (sm arch, version). */
const char *po_version(void);

#ifdef __cplusplus
}
#endif

#endif /* WAVEPO_H */
