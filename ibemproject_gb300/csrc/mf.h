// Internal interface of the matrix-free solver (mf.cu) and the learned preconditioner
// (gnn.cu): the sphere system of layout 24 is never stored; its 24 x 24 pair blocks are
// evaluated on the fly inside the products.
//
// Batches: the particles of several independent realisations (segments) are concatenated;
// particle p belongs to segment seg_of[p] and interacts only with particles of that
// segment.  Unknowns of particle p are rows 24p .. 24p + 23 (E_ij | E_ijk, as layout 24).
//
// Scaled system.  With a_p the radius of particle p, mu0 the matrix shear modulus of the
// segment, rho_r = 1 for rows of order 1 (r >= 6) and sigma_c = 1 for columns of order 1,
//   As = Dr A Dc,   Dr = diag(a_s^rho_r / mu0),   Dc = diag(a_h^-sigma_c),
// so that As[(s,r),(h,c)] = (a_s / a_h)^rho_r * B(x / a_h; 1)_rc / mu0 with B the pair block
// of a unit sphere: every entry is O(1) whatever the radii and moduli, which is what the
// FP32 products need.  x = Dc xs and bs = Dr b.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "gen_sphere_common.cuh"
#include "gen_sphere24_f32.cuh"
#include "ibem_internal.h"

namespace ibem {

constexpr int kMfNu = 24;   // unknowns per particle of the matrix-free path
constexpr int kKnn = 16;    // neighbours per particle of the learned preconditioner

struct MfTile {
  int seg, s0, ns, pad;     // one CTA's target particles s0 .. s0 + ns - 1 of segment seg
};

// Stream-ordered scratch: allocations and frees of the solver's temporaries are queued on
// the call's stream (cudaMallocAsync / cudaFreeAsync), so that no call synchronises the
// device to release memory.
inline cudaError_t alloc_async(void** p, size_t bytes, cudaStream_t st) {
  return cudaMallocAsync(p, bytes > 0 ? bytes : 1, st);
}
inline void free_async(void* p, cudaStream_t st) {
  if (p) cudaFreeAsync(p, st);
}

struct MfBatch {
  cudaStream_t st = nullptr;   // stream of the call that owns the batch's buffers
  int nu = 24;                 // unknowns per particle: 24 or 60
  int nseg = 0, num = 0, max_seg = 0;
  int64_t N = 0;
  std::vector<int> seg_begin_h;
  std::vector<ibem_material> mats_h;
  int* seg_begin = nullptr;   // nseg + 1
  int* seg_of = nullptr;      // num
  const double* cen = nullptr;  // caller's, num x 3
  const double* rad = nullptr;  // caller's, num
  const double* axes = nullptr; // caller's, num x 3 (ellipsoids), or nullptr (spheres)
  float4* gh = nullptr;       // centre (high float parts), radius
  float4* gl = nullptr;       // centre (low float parts), 1 / radius
  SphMat* matd = nullptr;     // per segment, physical units
  SphMatF* matf = nullptr;    // per segment, divided by mu0
  SphMat* mats = nullptr;     // per segment, FP64, divided by mu0 (scaled system)
  double* dr = nullptr;       // N: row scaling
  double* dc = nullptr;       // N: column scaling
  MfTile* tiles = nullptr;
  int ntiles = 0;
  int* perm = nullptr;        // num: particles of each realisation in the Morton order of their
                              // centres (position -> particle), used by the split FP64 product
  int hsplit = 1;      // source slices per target tile, FP32 product (autotuned)
  int hsplit_wide = 1; // the same for the double-float and FP64 products (~255 registers)
  // FP32 product (the GMRES operator): tile shape and launch form, picked by the autotuner
  MfTile* tiles_s[3] = {nullptr, nullptr, nullptr};   // tiles of 64, 128 and 256 targets
  int ntiles_s[3] = {0, 0, 0};
  int tshape = 1;             // index of the tile shape (64 << tshape targets per CTA)
  int persist = 0;            // 1: persistent CTAs over a cost-sorted list of (tile, slice)
  int2* work = nullptr;       // that list (persist only)
  int nwork = 0, persist_ctas = 0;
};

// layout-60 products (mf60.cu): FP32 and FP64 (the double-float entry points fall back to
// FP64 there), the realisations' block-Jacobi inverses (Pseg: nseg x 60 x 60) and their
// application
ibem_status mf60_apply_f32(const MfBatch& b, const float* x, float* y, cudaStream_t st, const int* mask, int mask_on);
ibem_status mf60_apply_f64(const MfBatch& b, const double* x, double* y, cudaStream_t st, const int* mask,
                           int mask_on);
ibem_status mf60_block_jacobi(const MfBatch& b, float* Pseg, cudaStream_t st);
ibem_status mf60_precond_apply(const MfBatch& b, const float* Pseg, const float* v, float* z, const int* kdev,
                               int64_t vstride, cudaStream_t st);

// Sets the FP32 product's tile shape (0, 1, 2: 64, 128, 256 targets per CTA), source slices
// and launch form; builds the persistent form's work list.
ibem_status mf_set_f32_shape(MfBatch& b, int tshape, int hsplit, int persist, cudaStream_t st);

// layout 24 (orders 0 and 1) or 60 (orders 0 to 2: block-Jacobi preconditioner only)
ibem_status mf_batch_init(MfBatch& b, const ibem_e3d_batch& in, cudaStream_t st, int layout = 24);
// Source-slice counts of the products for this batch's shape, from the autotuner's table
// (timed on first use of a shape class, then cached for the process).
ibem_status mf_tune(MfBatch& b, cudaStream_t st);
void mf_batch_free(MfBatch& b);

// y = As x (FP32, scaled system); y is overwritten.  With a mask, realisation s takes part
// only when mask[s] == mask_on (its rows of y stay zero otherwise); the same for the others.
ibem_status mf_apply_f32(const MfBatch& b, const float* x, float* y, cudaStream_t st, const int* mask = nullptr,
                         int mask_on = 1);

// Block-sparse preconditioner on the k-nearest-neighbour graph:
//   (P v)_i = D_i v_i + sum_slot Q_(i,slot) v_nbr(i,slot)
struct MfPrecond {
  float* D = nullptr;    // num x 24 x 24 diagonal blocks (row-major)
  float* Q = nullptr;    // num*kKnn x 24 x 24 off-diagonal blocks, or nullptr (block-diagonal)
  int* nbr = nullptr;    // num*kKnn neighbour indices (-1: empty slot)
};
// y = As x (scaled system, the deciding residual); y is overwritten.  In batches whose largest
// realisation has 1,280 particles or more, pairs whose source lies within 4 of its radii of
// the box of the warp's targets are evaluated in FP64 and the others in double-float; below
// that, every pair in FP64.  Targets and sources in Morton order.
ibem_status mf_apply_f64(const MfBatch& b, const double* x, double* y, cudaStream_t st, const int* mask = nullptr,
                         int mask_on = 1);
// the same with every pair in FP64 (the reference for the split)
ibem_status mf_apply_f64_all(const MfBatch& b, const double* x, double* y, cudaStream_t st);
// y = As x in double-float arithmetic (~48 bits, FP32 pipe); y is overwritten
ibem_status mf_apply_df(const MfBatch& b, const double* x, double* y, cudaStream_t st, const int* mask = nullptr,
                        int mask_on = 1);
// P[p] = inverse of the scaled diagonal block As[p, p] (24 x 24, row-major, FP32)
ibem_status mf_block_jacobi(const MfBatch& b, float* P, cudaStream_t st);

// ---- learned preconditioner (gnn.cu) ----
constexpr int kGnnHidden = 64, kGnnLayers = 3, kGnnNodeF = 10, kGnnEdgeF = 7, kGnnOut = 2;
int64_t gnn_param_count();
// k nearest neighbours within each segment (by centre distance, ties to the lower index);
// nbr[p * kKnn + j] = neighbour index or -1
ibem_status gnn_knn(const MfBatch& b, int* nbr, cudaStream_t st);
ibem_status gnn_features(const MfBatch& b, const int* nbr, float* xn, float* ef, cudaStream_t st);
// Neumann blocks of every edge e = (i <- j), B the block-Jacobi inverses:
//   C_e = -B_i As_ij B_j          (first-order term of (As^-1)_ij)
//   T_e =  B_i As_ij B_j As_ji B_i (second-order term of (As^-1)_ii)
// With weights wa (num*kKnn x 2: w_e, alpha_e): D[i] += w_e T_e (D holds B on entry) and
// Q[e] = alpha_e C_e.  With samples r (nrhs x N): u[q][e] = (T_e r_qi, C_e r_qj).
ibem_status gnn_edge_corrections(const MfBatch& b, const int* nbr, const float* B, const float* wa, float* D,
                                 float* Q, int nrhs, const float* r, float* u, cudaStream_t st);
// Edge outputs (w_e, alpha_e) of the network (forward only): num * kKnn x 2
ibem_status gnn_forward_weights(int num, const int* nbr, const float* xn, const float* ef, const float* params,
                                float* wa, cudaStream_t st);
// The neighbour-coupled preconditioner of a batch: block-Jacobi plus the Neumann blocks
// weighted by the network (params) or all weighted 1 (params == nullptr).  D must hold
// the block-Jacobi inverses; Q and nbr are allocated here (freed by the caller).
ibem_status mf_neighbour_precond(const MfBatch& b, const float* params, MfPrecond& pc, cudaStream_t st);

}  // namespace ibem
