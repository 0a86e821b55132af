// po_kernels.h -- kernel launchers shared between the engine's translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "po_common.cuh"
#include "wavepo.h"

namespace wavepo {

constexpr int kMaxStages = 24;

// Stockham FFT plan: radix sequence and offset of the W_n table in the
// engine's twiddle buffer.
struct FftPlan {
  int n = 0;
  int tw = 0;
  int nstages = 0;
  int radix[kMaxStages];
};

int fft_plan(int n, int *radix);
FftPlan make_plan(int n, int tw_offset);
po_status launch_twiddles(int n, float2 *out, cudaStream_t st);

// currents: out[slot][n][6] complex (T pairs)
po_status launch_currents_f32(int64_t n, const float *const g[7], const SlotParams<float> *slots_dev, int n_slots,
                              float *out, cudaStream_t st);
po_status launch_currents_f64(int64_t n, const float *const g[7], const SlotParams<double> *slots_dev, int n_slots,
                              double *out, cudaStream_t st);

// leaf far fields: out[slot][leaf][comp][dir]; slots grouped by wavelength (G per lambda)
po_status launch_leaf(const float *const g[7], const int32_t *leaf_begin, const double *leaf_center,
                      int64_t n_leaves, const SlotParams<float> *slots_dev, int n_lambda, int G,
                      const float4 *dirs, int ndir, float2 *out, cudaStream_t st);

// split hi+lo BF16 tensor-core leaf sums (po_leaf_mma.cu); same layout as launch_leaf
po_status init_leaf_mma_attributes();
// fuse_mid != nullptr: also run the phi pass of the level above (Rc x Pc leaf
// grid to Pp columns, fragments fuse_B with Kp rows) and write its packed
// output there (leaf_row_fusion_fits must hold)
po_status launch_leaf_mma(const float *const g[7], const int32_t *leaf_begin, const double *leaf_center,
                          int64_t n_leaves, const SlotParams<float> *slots_dev, int n_lambda, int G,
                          const float4 *dirs, int ndir, float2 *out, cudaStream_t st, const uint32_t *fuse_B = nullptr,
                          uint4 *fuse_mid = nullptr, int Rc = 0, int Pc = 0, int Pp = 0, int Kp = 0);
bool leaf_row_fusion_fits(int Pc, int Pp, int Kp);

// tcgen05 leaf sums for many patterns per wavelength (po_leaf_tc.cu); same
// output layout as launch_leaf.  The points of every leaf are taken in chunks
// of 16: kc0[leaf] = first chunk of the leaf (kc0[n_leaves] = n_chunks),
// chunk_leaf[chunk] = its leaf.  bop / uop: operand scratch of
// n_lambda x n_chunks x leaf_tc_col_tiles(G) x leaf_tc_block_bytes() and of
// n_lambda x n_chunks x 16 float4.  group: slots per pass (a multiple of 8 up
// to kLeafTcMaxSlots); each pass regenerates the phase operands of every leaf.
constexpr int kLeafTcMaxSlots = 64;  // slots per operand pass (6 column tiles of 64 complex columns)
constexpr int kLeafTcMinSlots = 8;   // fewer patterns per wavelength keep the warp-level kernel
int leaf_tc_col_tiles(int G);
size_t leaf_tc_block_bytes();
po_status init_leaf_tc_attributes();
po_status launch_leaf_tc(const float *const g[7], const int32_t *leaf_begin, const int32_t *kc0,
                         const int32_t *chunk_leaf, int64_t n_chunks, const double *leaf_center, int64_t n_leaves,
                         const SlotParams<float> *slots_dev, int n_lambda, int Gtot, int g0, int G,
                         const float4 *dirs, int ndir, uint8_t *bop, size_t bop_bytes, float4 *uop,
                         size_t uop_bytes, float2 *out, int *err, cudaStream_t st, int group = kLeafTcMaxSlots,
                         int withhold = 0, int msplit = 1);

int direct_splits(int64_t n, int ndir, int n_lambda, int sm_count);
// FP32 depth-0 sum about c0: out[slot][comp][dir]; cur[slot][n][6]
po_status launch_direct_f32(int64_t n, const float *x, const float *y, const float *z, const float2 *cur,
                            double *tile_ctr, const double *k_per_lambda, int n_lambda, int G,
                            const double c0[3], const float4 *dirs, const double *dirs_d, int ndir, int nsplit,
                            float2 *partial, float2 *out, cudaStream_t st);
// FP64 depth-0 sum (k per slot): out[slot][comp][dir]
po_status launch_direct_f64(int64_t n, const float *x, const float *y, const float *z, const double2 *cur,
                            const double *k_per_slot, int n_slots, const double c0[3], const double *dirs_d,
                            int ndir, int nsplit, double2 *partial, double2 *out, cudaStream_t st);

// complex64 <-> complex128 copies of n complex values
po_status launch_widen(const float *in, double2 *out, int64_t n, cudaStream_t st);
po_status launch_narrow(const double2 *in, float2 *out, int64_t n, cudaStream_t st);

// interpolation passes
// ref_nyquist: equal sizes keep the reference's halved Nyquist bin (else exact)
po_status launch_interp_rows(const float2 *src, float2 *dst, int64_t nrows, const FftPlan &pin, const FftPlan &pout,
                             const float2 *twiddles, float scale, int sm_count, int ref_nyquist, cudaStream_t st);
// Rc/Rp: stored theta rows of child/parent patterns (mirror: Tc/2+1, Tp/2+1)
po_status launch_interp_cols(const float2 *mid, float2 *parent, const int32_t *child_table, int64_t n_parent,
                             int64_t n_child, int phi, int Rc, int Rp, const FftPlan &pin, const FftPlan &pout,
                             const float2 *twiddles, const float4 *trans, int n_slots, int G, int quirk_reach,
                             float scale, int ncomp, int mirror, int ref_nyquist, cudaStream_t st);
// tensor-core theta pass (po_interp_mma.cu): double cover, or the reference
// theta mode's real column-independent map (an odd phi pairs column j with
// j + (phi+1)/2).  mid: the packed output of launch_interp_rows_packed; Kp =
// Rc rounded up to even, then to 16.
size_t theta_matrix_words(int Rp, int Kp);
size_t theta_pair_words(int Rp, int Kp);
void build_theta_matrix(int Tc, int Tp, int Rc, int Rp, int Kp, std::vector<uint32_t> &out, bool mirror = true);
po_status launch_interp_cols_mma(const uint4 *mid, float2 *parent, const int32_t *child_table, int64_t n_parent,
                                 int64_t n_child, int phi, int Rc, int Rp, int Kp, const uint32_t *Afrag,
                                 const float4 *trans, int n_slots, int G, int tile, cudaStream_t st);
// tensor-core phi pass (po_interp_mma.cu): float2 rows -> float2 rows, or
// (packed) n_patterns x Rc rows -> mirror-pair sums / differences in split-bf16
// row pairs for the theta pass
size_t phi_matrix_words(int Pp, int Kp);
void build_phi_matrix(int Pc, int Pp, int Kp, std::vector<uint32_t> &out);
po_status launch_interp_rows_mma(const float2 *src, float2 *dst, int64_t nrows, int Pc, int Pp, int Kp,
                                 const uint32_t *Bm, int sm_count, cudaStream_t st);
po_status launch_interp_rows_packed(const float2 *src, uint4 *dst, int64_t n_patterns, int Rc, int Pc, int Pp,
                                    int Kp, const uint32_t *Bm, int sm_count, cudaStream_t st);
// (core) the same sums / differences as four bf16 core-matrix arrays per pattern
// (npad columns x Rr rows, rows Rc.. zero) for the tcgen05 theta pass
po_status launch_interp_rows_core(const float2 *src, uint8_t *dst, int64_t n_patterns, int Rc, int Rr, int npad,
                                  int Pc, int Pp, int Kp, const uint32_t *Bm, int sm_count, cudaStream_t st);
void theta_plus_minus(int Tc, int Tp, int Rc, int Rp, int ld, std::vector<double> &Mplus,
                      std::vector<double> &Mminus, bool mirror = true);
// tcgen05 theta pass for levels with more than 128 parent rows (po_theta_tc.cu)
size_t theta_tc_bytes(int Rp, int Kr);
int theta_tc_npad(int phi);
void build_theta_tc(const std::vector<double> &Mplus, const std::vector<double> &Mminus, int Rp, int Rc, int ld,
                    int Kr, std::vector<uint16_t> &out);
po_status init_theta_tc_attributes();
void build_phi_tc(int Pc, int Pp, int Kc, int ntn, int n_nt, std::vector<uint16_t> &out);
bool rows_tc_plan(int Pc, int Pp, int &ntn, int &n_nt);
po_status init_rows_tc_attributes();
po_status launch_rows_tc(const float2 *src, uint8_t *dst, size_t dst_bytes, int64_t n_patterns, int Rc, int Rr,
                         int npad, int Pc, int Pp, const uint8_t *Bt, size_t bt_bytes, int ntn, int n_nt,
                         int sm_count, int *err, cudaStream_t st);
po_status launch_theta_tc(const uint8_t *mid, float2 *parent, const int32_t *child_table, int64_t n_parent,
                          int64_t n_child, int phi, int Kr, int Rp, const uint8_t *Atc, const float4 *trans,
                          int n_slots, int G, int *err, size_t mid_bytes, size_t atc_bytes, cudaStream_t st,
                          int withhold = 0);
// adjoint (transposed) passes, double cover only (po_interp_mma.cu)
void build_theta_matrix_adj(int Tc, int Tp, int Rc, int Rp, int Kp, std::vector<uint32_t> &out);
void build_phi_matrix_adj(int Pc, int Pp, int Kp, std::vector<uint32_t> &out);
po_status launch_interp_cols_adj_mma(const float2 *parent_adj, float2 *mid_adj, const int32_t *child_table,
                                     int64_t n_parent, int64_t n_child, int phi, int Rc, int Rp, int Kp,
                                     const uint32_t *Afrag, const float4 *trans, int n_slots, int G,
                                     cudaStream_t st);
// direction factors of a level grid (once per context) and the per-solve
// translation phases built from them (po_fft.cu)
po_status launch_dir_trig(int nth, int R, int phi, double2 *trig, cudaStream_t st);
po_status launch_trans_table(const double *k_per_lambda, int n_lambda, int Rp, int phi, const double2 *trig,
                             const double a[3], float4 *out, cudaStream_t st);

// height field [2][numel][numelvert] -> samples of quads (i, j in [ring_begin, ring_end]);
// out = {x, y, z, nx, ny, nz, area}; err |= 1 on a vertex at the origin (po_geometry.cu)
po_status launch_height_field(const float *height, int numel, int numelvert, float period, float unitz, int ring_begin,
                              int ring_end, float *const out[7], int *err, cudaStream_t st);

// adjoint of the intensity and of the far-field sums (po_adjoint.cu)
po_status launch_intensity_adjoint_f32(const float2 *fields, const float *dl_di, int n_slots, int T, int Phi, int nth,
                                       int nph, int mt, int mp, const float4 *dirs, float2 *G, cudaStream_t st);
po_status launch_intensity_adjoint_f64(const double2 *fields, const float *dl_di, int n_slots, int nth, int nph,
                                       double2 *G, cudaStream_t st);
// tensor-core back-projection of the leaf adjoint patterns, FP32 chain (po_adjoint_mma.cu)
po_status init_point_adjoint_mma_attributes();
po_status launch_point_adjoint_mma(const float *const g[7], const int32_t *begin, int64_t n_nodes,
                                   const double *center, int center_stride, const float2 *G, int64_t node_stride,
                                   int64_t slot_stride, const float4 *dirs, int ndir,
                                   const SlotParams<double> *slots, int n_lambda, int Gc, int64_t n, double *grad,
                                   cudaStream_t st);
po_status launch_point_adjoint_f64(const float *const g[7], const int32_t *begin, int64_t n_nodes,
                                   const double *center, int center_stride, const double2 *G, int64_t node_stride,
                                   int64_t slot_stride, const double *dirs_d, int ndir, const SlotParams<double> *slots,
                                   int n_lambda, int Gc, int64_t n, double *grad, cudaStream_t st);
po_status launch_chunk_begin(int32_t *begin, int64_t n, int chunk, cudaStream_t st);
po_status launch_scatter_grad(const double *grad_sorted, const int32_t *perm, int64_t n, float *out, cudaStream_t st);

// once per device: opt-in shared memory of the kernels whose launchers size it at run time
po_status init_interp_mma_attributes(int max_smem);
po_status init_fft_attributes(int max_smem);

// intensity: fields [slot][comp][T][Phi] (root, possibly supersampled by
// (mt, mp)) -> out [slot][nth][nph]
// out_dirs: the context's output-direction table (launch_out_dirs)
po_status launch_out_dirs(int nth, int nph, float4 *dirs, cudaStream_t st);
po_status launch_intensity_f32(const float2 *fields, int n_slots, int T, int Phi, int nth, int nph, int mt, int mp,
                               const float4 *dirs, float *out, cudaStream_t st);
po_status launch_intensity_f64(const double2 *fields, int n_slots, int nth, int nph, float *out, cudaStream_t st);

}  // namespace wavepo
