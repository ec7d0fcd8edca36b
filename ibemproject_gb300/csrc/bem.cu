// Boundary-element kernels of the 3D elastic iBEM path (FP64).
//
//  bem_hg        classical Q4 BEM H and G with 8x8 Gauss-Legendre quadrature, the singular
//                element split into two degenerate triangles, and the rigid-body diagonal
//                (BEMBuilderElastic3D.cpp:1169-1509, BEMElasticHelper3D.cpp:29-321).
//                One thread per (collocation node, element); the element's 12 traction
//                columns are scattered into node columns with FP64 atomics (the reference
//                accumulates them under `omp critical`, :1432-1454).
//  bem_to_incl   stress and its 1st/2nd gradient at particle centres from unit boundary
//                displacements/tractions (addFluxEquivalent{,FirstOrder,SecondOrder}BEM,
//                :1511-1867).  One thread per (particle, element, derivative tuple W, dof),
//                48 accumulators each; the generated kernel for (order, W, dof) is picked
//                by blockIdx.z.
//  bem_post      boundary part of the stress at sample points (post_stress_BEM,
//                postProcessorElastic3D.cpp:224-365), contracted with U and T at every
//                Gauss point: a per-call quadrature table (point, normal, weight x Jacobian,
//                interpolated U and T per Gauss point) staged through shared memory, one
//                thread per sample point.
#include <algorithm>
#include <cuda_runtime.h>

#include "gen_bem.cuh"
#include "bem_contract.cuh"
#include "ibem_internal.h"
#include "prof.h"

namespace {

__constant__ double kGP[8] = {0.960289856497536,  -0.960289856497536, 0.796666477413627,
                              -0.796666477413627, 0.525532409916329,  -0.525532409916329,
                              0.183434642495650,  -0.183434642495650};
__constant__ double kGW[8] = {0.101228536290376, 0.101228536290376, 0.222381034453374,
                              0.222381034453374, 0.313706645877887, 0.313706645877887,
                              0.362683783378362, 0.362683783378362};

struct Elem {
  double c[12];  // 4 corners x 3
};

// Corner coordinates of element e; false (nothing read) if a node number is outside
// 1..NN, so a bad connectivity table can never address outside the node array.
__device__ __forceinline__ bool load_elem(const double* __restrict__ nodes, int NN, const int* __restrict__ conn,
                                          int e, Elem& el, int* sc) {
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    sc[j] = conn[4 * e + j];
    if (sc[j] < 1 || sc[j] > NN) return false;
  }
#pragma unroll
  for (int j = 0; j < 4; ++j)
#pragma unroll
    for (int k = 0; k < 3; ++k) el.c[3 * j + k] = nodes[3 * (sc[j] - 1) + k];
  return true;
}

// Serendip_func, Normal_Jac, Cartesian (BEMElasticHelper3D.cpp:199-280)
__device__ __forceinline__ void q4_point(const double* c, double xi, double et, double* N,
                                         double* gc, double* nv, double& jac) {
  N[0] = 0.25 * (1 - xi) * (1 - et);
  N[1] = 0.25 * (1 + xi) * (1 - et);
  N[2] = 0.25 * (1 + xi) * (1 + et);
  N[3] = 0.25 * (1 - xi) * (1 + et);
  const double dxi[4] = {-0.25 * (1 - et), 0.25 * (1 - et), 0.25 * (1 + et), -0.25 * (1 + et)};
  const double det[4] = {-0.25 * (1 - xi), -0.25 * (1 + xi), 0.25 * (1 + xi), 0.25 * (1 - xi)};
  double vx[3], ve[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    vx[i] = dxi[0] * c[i] + dxi[1] * c[3 + i] + dxi[2] * c[6 + i] + dxi[3] * c[9 + i];
    ve[i] = det[0] * c[i] + det[1] * c[3 + i] + det[2] * c[6 + i] + det[3] * c[9 + i];
    gc[i] = N[0] * c[i] + N[1] * c[3 + i] + N[2] * c[6 + i] + N[3] * c[9 + i];
  }
  nv[0] = vx[1] * ve[2] - ve[1] * vx[2];
  nv[1] = vx[2] * ve[0] - vx[0] * ve[2];
  nv[2] = vx[0] * ve[1] - vx[1] * ve[0];
  jac = sqrt(nv[0] * nv[0] + nv[1] * nv[1] + nv[2] * nv[2]);
  nv[0] /= jac;
  nv[1] /= jac;
  nv[2] /= jac;
}

// Trans_Tri + Triangle_Coord (BEMElasticHelper3D.cpp:29-191): Gauss point (xb, eb) of the
// square mapped onto triangle `ntr` of the split at corner l_pi; jb its Jacobian.
__device__ __forceinline__ void tri_map(int ntr, int l_pi, double xb, double eb, double& xi,
                                        double& et, double& jb) {
  // corner/mid-side indices of the two triangles for each singular corner
  const int tab[2][4][3] = {{{1, 2, 0}, {2, 3, 1}, {0, 1, 2}, {0, 1, 3}},
                            {{2, 3, 0}, {3, 0, 1}, {3, 0, 2}, {1, 2, 3}}};
  const double xs[4] = {-1, 1, 1, -1};
  const double es[4] = {-1, -1, 1, 1};
  double cx[3], ce[3];
#pragma unroll
  for (int n = 0; n < 3; ++n) {
    cx[n] = xs[tab[ntr][l_pi][n]];
    ce[n] = es[tab[ntr][l_pi][n]];
  }
  const double Nb[3] = {0.25 * (1 + xb) * (1 - eb), 0.25 * (1 + xb) * (1 + eb), 0.5 * (1 - xb)};
  const double dNx[3] = {0.25 * (1 - eb), 0.25 * (1 + eb), -0.5};
  const double dNe[3] = {-0.25 * (1 + xb), 0.25 * (1 + xb), 0.0};
  xi = Nb[0] * cx[0] + Nb[1] * cx[1] + Nb[2] * cx[2];
  et = Nb[0] * ce[0] + Nb[1] * ce[1] + Nb[2] * ce[2];
  const double J00 = dNx[0] * cx[0] + dNx[1] * cx[1] + dNx[2] * cx[2];
  const double J01 = dNx[0] * ce[0] + dNx[1] * ce[1] + dNx[2] * ce[2];
  const double J10 = dNe[0] * cx[0] + dNe[1] * cx[1] + dNe[2] * cx[2];
  const double J11 = dNe[0] * ce[0] + dNe[1] * ce[1] + dNe[2] * ce[2];
  jb = J00 * J11 - J01 * J10;
}

struct KelvinC {
  double cu, c1, ct, c3;  // UK: c/(r) (c1 + r_i r_j);  TK: c2 / r^2, c3 = 1 - 2 nu
};

// Integ3 for one (collocation node, element): dU, dT (3 x 12), BEMBuilderElastic3D.cpp:1169-1353
// The traction part of this element is written to TG, laid out like G (column 12e + 3a + j,
// row 3i + ii; zero for the singular corner); node_gather then sums the columns of the
// elements that share a node in a fixed order, so H is the same bit for bit on every run.
__global__ void __launch_bounds__(128) bem_hg_kernel(const double* __restrict__ nodes, int NN,
                                                     const int* __restrict__ conn, KelvinC kc,
                                                     double* __restrict__ TG, int64_t ldt,
                                                     double* __restrict__ G, int64_t ldg) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int e = blockIdx.y;
  if (i >= NN) return;
  Elem el;
  int sc[4];
  if (!load_elem(nodes, NN, conn, e, el, sc)) return;
  const double xP[3] = {nodes[3 * i], nodes[3 * i + 1], nodes[3 * i + 2]};
  int l_pi = -1;
#pragma unroll
  for (int n = 0; n < 4; ++n)
    if (sc[n] == i + 1) l_pi = n;
  double dU[3][12], dT[3][12];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 12; ++b) { dU[a][b] = 0.0; dT[a][b] = 0.0; }
  const int ntri = l_pi < 0 ? 1 : 2;
  for (int ntr = 0; ntr < ntri; ++ntr)
    for (int mq = 0; mq < 8; ++mq)
      for (int kq = 0; kq < 8; ++kq) {
        const double W = kGW[mq] * kGW[kq];
        double xi = kGP[mq], et = kGP[kq], jb = 1.0;
        if (l_pi >= 0) tri_map(ntr, l_pi, kGP[mq], kGP[kq], xi, et, jb);
        double N[4], gc[3], nv[3], jac;
        q4_point(el.c, xi, et, N, gc, nv, jac);
        jac *= jb;
        const double dx0 = gc[0] - xP[0], dx1 = gc[1] - xP[1], dx2 = gc[2] - xP[2];
        const double r = sqrt(dx0 * dx0 + dx1 * dx1 + dx2 * dx2);
        const double dr[3] = {dx0 / r, dx1 / r, dx2 / r};
        // UK / TK (BEMElasticHelper3D.cpp:269-321)
        const double conr = kc.cu / r;
        const double cth = nv[0] * dr[0] + nv[1] * dr[1] + nv[2] * dr[2];
        const double cr = kc.ct / (r * r);
        const double wj = jac * W;
#pragma unroll
        for (int ii = 0; ii < 3; ++ii)
#pragma unroll
          for (int jj = 0; jj < 3; ++jj) {
            const double U = conr * ((ii == jj ? kc.c1 : 0.0) + dr[ii] * dr[jj]);
            const double T = (ii == jj) ? -cr * (kc.c3 + 3 * dr[ii] * dr[ii]) * cth
                                        : -cr * (3 * dr[ii] * dr[jj] * cth - kc.c3 * (nv[jj] * dr[ii] - nv[ii] * dr[jj]));
#pragma unroll
            for (int n = 0; n < 4; ++n) {
              dU[ii][3 * n + jj] += N[n] * U * wj;
              if (l_pi < 0 || n != l_pi) dT[ii][3 * n + jj] += N[n] * T * wj;
            }
          }
      }
  // G columns of this element, and its traction columns for H (summed per node by node_gather)
#pragma unroll
  for (int ii = 0; ii < 3; ++ii)
#pragma unroll
    for (int k = 0; k < 12; ++k) {
      G[(12 * (int64_t)e + k) * ldg + 3 * i + ii] = dU[ii][k];
      TG[(12 * (int64_t)e + k) * ldt + 3 * i + ii] = (l_pi < 0 || k / 3 != l_pi) ? dT[ii][k] : 0.0;
    }
}

// ---- node incidence: the (element, corner) slots of every node, in increasing order ----
// inc_start[c] .. inc_start[c + 1] - 1 index inc_slot, whose entries are 4e + a for the
// corners a of elements e at node c.  Built with integer atomics, then each node's list is
// sorted, so the order (and every sum over it) does not depend on scheduling.
__global__ void k_inc_count(const int* __restrict__ conn, int NE, int NN, int* __restrict__ cnt) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= 4 * NE) return;
  const int c = conn[id] - 1;
  if (c >= 0 && c < NN) atomicAdd(cnt + c, 1);
}

// exclusive prefix sum of n counts into start[0..n] (one block, sequential chunks)
__global__ void k_inc_scan(const int* __restrict__ cnt, int n, int* __restrict__ start) {
  __shared__ int sh[1024];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < n; base += 1024) {
    const int i = base + threadIdx.x;
    const int v = i < n ? cnt[i] : 0;
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
      const int t = threadIdx.x >= off ? sh[threadIdx.x - off] : 0;
      __syncthreads();
      sh[threadIdx.x] += t;
      __syncthreads();
    }
    if (i < n) start[i] = carry + sh[threadIdx.x] - v;
    __syncthreads();
    if (threadIdx.x == 1023) carry += sh[1023];
    __syncthreads();
  }
  if (threadIdx.x == 0) start[n] = carry;
}

__global__ void k_inc_fill(const int* __restrict__ conn, int NE, int NN, const int* __restrict__ start,
                           int* __restrict__ cursor, int* __restrict__ slot) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= 4 * NE) return;
  const int c = conn[id] - 1;
  if (c < 0 || c >= NN) return;
  slot[start[c] + atomicAdd(cursor + c, 1)] = id;
}

__global__ void k_inc_sort(int NN, const int* __restrict__ start, int* __restrict__ slot) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= NN) return;
  for (int i = start[c] + 1; i < start[c + 1]; ++i) {
    const int v = slot[i];
    int j = i - 1;
    while (j >= start[c] && slot[j] > v) { slot[j + 1] = slot[j]; --j; }
    slot[j + 1] = v;
  }
}

// H[(3c + d) ldh + r] (+)= sum over node c's slots 4e + a, in order, of S[(12e + 3a + d) lds + r]
// for rows r < nrows; the element columns of S are laid out like G.
__global__ void __launch_bounds__(256) k_node_gather(int64_t nrows, int NN, const int* __restrict__ start,
                                                     const int* __restrict__ slot, const double* __restrict__ S,
                                                     int64_t lds, double* __restrict__ H, int64_t ldh, int accumulate) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= nrows) return;
  for (int c = blockIdx.y; c < NN; c += gridDim.y) {
    double acc0 = 0.0, acc1 = 0.0, acc2 = 0.0;
    for (int q = start[c]; q < start[c + 1]; ++q) {
      const int64_t col = 3 * (int64_t)slot[q];   // 12e + 3a
      acc0 += S[col * lds + r];
      acc1 += S[(col + 1) * lds + r];
      acc2 += S[(col + 2) * lds + r];
    }
    double* h = H + 3 * (int64_t)c * ldh + r;
    if (accumulate) {
      h[0] += acc0;
      h[ldh] += acc1;
      h[2 * ldh] += acc2;
    } else {
      h[0] = acc0;
      h[ldh] = acc1;
      h[2 * ldh] = acc2;
    }
  }
}

// Rigid-body diagonal (:1478-1501): H(r, 3i+l) = -sum_c H(r, c) over columns c with c%3 == l.
__global__ void bem_diag_kernel(int NN, double* __restrict__ H, int64_t ldh) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= 3 * NN) return;
  double s0 = 0, s1 = 0, s2 = 0;
  for (int c = 0; c < NN; ++c) {
    s0 += H[(3 * (int64_t)c) * ldh + r];
    s1 += H[(3 * (int64_t)c + 1) * ldh + r];
    s2 += H[(3 * (int64_t)c + 2) * ldh + r];
  }
  const int64_t i = r / 3;
  H[(3 * i) * ldh + r] = -s0;
  H[(3 * i + 1) * ldh + r] = -s1;
  H[(3 * i + 2) * ldh + r] = -s2;
}

// ---- boundary -> inclusion rows ----
typedef void (*StressFn)(double, double, double, double, double, double, const BemMat&, double,
                         double, double*, double*);

template <int ORDER>
__device__ __forceinline__ void stress_dispatch(int f, double x0, double x1, double x2, double n0,
                                                double n1, double n2, const BemMat& bm,
                                                double* su, double* st) {
  const double dl = bm.dlam, dm = bm.dmu;
#define IBEM_S(fn) fn(x0, x1, x2, n0, n1, n2, bm, dl, dm, su, st)
  if (ORDER == 0) {
    switch (f) {
      case 0: IBEM_S(bem_stress_o0_w_n0); break;
      case 1: IBEM_S(bem_stress_o0_w_n1); break;
      default: IBEM_S(bem_stress_o0_w_n2); break;
    }
  } else if (ORDER == 1) {
    switch (f) {
      case 0: IBEM_S(bem_stress_o1_w0_n0); break; case 1: IBEM_S(bem_stress_o1_w0_n1); break;
      case 2: IBEM_S(bem_stress_o1_w0_n2); break; case 3: IBEM_S(bem_stress_o1_w1_n0); break;
      case 4: IBEM_S(bem_stress_o1_w1_n1); break; case 5: IBEM_S(bem_stress_o1_w1_n2); break;
      case 6: IBEM_S(bem_stress_o1_w2_n0); break; case 7: IBEM_S(bem_stress_o1_w2_n1); break;
      default: IBEM_S(bem_stress_o1_w2_n2); break;
    }
  } else {
    switch (f) {
#define IBEM_C2(F, WS, N) case F: IBEM_S(bem_stress_o2_w##WS##_n##N); break;
      IBEM_C2(0, 00, 0) IBEM_C2(1, 00, 1) IBEM_C2(2, 00, 2) IBEM_C2(3, 01, 0) IBEM_C2(4, 01, 1)
      IBEM_C2(5, 01, 2) IBEM_C2(6, 02, 0) IBEM_C2(7, 02, 1) IBEM_C2(8, 02, 2) IBEM_C2(9, 10, 0)
      IBEM_C2(10, 10, 1) IBEM_C2(11, 10, 2) IBEM_C2(12, 11, 0) IBEM_C2(13, 11, 1)
      IBEM_C2(14, 11, 2) IBEM_C2(15, 12, 0) IBEM_C2(16, 12, 1) IBEM_C2(17, 12, 2)
      IBEM_C2(18, 20, 0) IBEM_C2(19, 20, 1) IBEM_C2(20, 20, 2) IBEM_C2(21, 21, 0)
      IBEM_C2(22, 21, 1) IBEM_C2(23, 21, 2) IBEM_C2(24, 22, 0) IBEM_C2(25, 22, 1)
      default: IBEM_S(bem_stress_o2_w22_n2); break;
#undef IBEM_C2
    }
  }
#undef IBEM_S
}

// blockIdx.z = W index * 3 + dof.  Rows of the layout: order 0 -> t; order 1 -> 6 + 3t + w;
// order 2 -> 24 + 9t + 3w + z (layout 78) or 24 + 6t + pairidx(w<=z) (layout 60).
// The displacement part (the H rows) is written per element into UG, laid out like G;
// node_gather sums it per node in a fixed element order (no atomics on matrix entries).
template <int ORDER>
__global__ void __launch_bounds__(128) bem_incl_kernel(
    const double* __restrict__ nodes, int NN, const int* __restrict__ conn, const double* __restrict__ cen,
    int num, BemMat bm, int nu, int compact, double* __restrict__ UG, int64_t ldu,
    double* __restrict__ G, int64_t ldg) {
  const int K = blockIdx.x * blockDim.x + threadIdx.x;
  const int e = blockIdx.y;
  const int f = blockIdx.z;
  if (K >= num) return;
  const int wi = f / 3, n = f % 3;
  const int w = ORDER == 2 ? wi / 3 : wi, z = wi % 3;
  if (ORDER == 2 && compact && z < w) return;
  Elem el;
  int sc[4];
  if (!load_elem(nodes, NN, conn, e, el, sc)) return;
  const double P0 = cen[3 * K], P1 = cen[3 * K + 1], P2 = cen[3 * K + 2];
  double au[6][4], at[6][4];
#pragma unroll
  for (int t = 0; t < 6; ++t)
#pragma unroll
    for (int a = 0; a < 4; ++a) { au[t][a] = 0.0; at[t][a] = 0.0; }
  for (int mq = 0; mq < 8; ++mq)
    for (int kq = 0; kq < 8; ++kq) {
      double N[4], gc[3], nv[3], jac;
      q4_point(el.c, kGP[mq], kGP[kq], N, gc, nv, jac);
      const double wj = kGW[mq] * kGW[kq] * jac;
      double su[18], st[18];
      stress_dispatch<ORDER>(f, gc[0] - P0, gc[1] - P1, gc[2] - P2, nv[0], nv[1], nv[2], bm, su, st);
#pragma unroll
      for (int t = 0; t < 6; ++t) {
        const double vu = su[3 * t + n] * wj, vt = st[3 * t + n] * wj;
#pragma unroll
        for (int a = 0; a < 4; ++a) { au[t][a] += vu * N[a]; at[t][a] += vt * N[a]; }
      }
    }
  const double fac = ORDER == 2 ? 0.5 : 1.0;
  int cidx = 0;  // compact (w<=z) pair index
  if (ORDER == 2 && compact) cidx = (w == 0) ? z : (w == 1 ? 2 + z : 5);
#pragma unroll
  for (int t = 0; t < 6; ++t) {
    int r;
    if (ORDER == 0) r = t;
    else if (ORDER == 1) r = 6 + 3 * t + w;
    else r = compact ? 24 + 6 * t + cidx : 24 + 9 * t + 3 * w + z;
    const int64_t row = (int64_t)nu * K + r;
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      UG[(12 * (int64_t)e + 3 * a + n) * ldu + row] = -fac * au[t][a];   // summed per node by node_gather
      G[(12 * (int64_t)e + 3 * a + n) * ldg + row] = fac * at[t][a];
    }
  }
}

// ---- boundary part of the stress at sample points ----
// Everything at a Gauss point that does not depend on the sample point -- its position, unit
// normal, weight x Jacobian, and U and T interpolated there -- is one record of the
// quadrature table, formed once per call (one thread per (element, Gauss point)); the
// per-point kernel then only evaluates the Kelvin stress kernels and contracts them.
constexpr int kPostQ = 64;        // 8 x 8 Gauss points per element
constexpr int kPostRec = 13;      // x y z, nx ny nz, w*J, u(3), t(3)
constexpr int kPostStage = 128;   // table records per shared-memory stage (13 KB)

__global__ void bem_post_table(const double* __restrict__ nodes, int NN, const int* __restrict__ conn, int NE,
                               const double* __restrict__ U, const double* __restrict__ T,
                               double* __restrict__ tab) {
  const int64_t id = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (id >= (int64_t)NE * kPostQ) return;
  const int e = (int)(id / kPostQ), q = (int)(id % kPostQ), mq = q / 8, kq = q % 8;
  double c[12], u[12], t[12];
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    int node = conn[4 * e + a] - 1;
    if (node < 0 || node >= NN) node = 0;  // out-of-range connectivity: never index outside
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      c[3 * a + d] = nodes[3 * node + d];
      u[3 * a + d] = U[3 * node + d];
    }
  }
#pragma unroll
  for (int k = 0; k < 12; ++k) t[k] = T[12 * (int64_t)e + k];
  double N[4], gc[3], nv[3], jac;
  q4_point(c, kGP[mq], kGP[kq], N, gc, nv, jac);
  double* r = tab + id * kPostRec;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    r[d] = gc[d];
    r[3 + d] = nv[d];
    r[7 + d] = N[0] * u[d] + N[1] * u[3 + d] + N[2] * u[6 + d] + N[3] * u[9 + d];
    r[10 + d] = N[0] * t[d] + N[1] * t[3 + d] + N[2] * t[6 + d] + N[3] * t[9 + d];
  }
  r[6] = kGW[mq] * kGW[kq] * jac;
}

// sums over the staged Gauss points of the stress contracted with their boundary values
// (bem_contract.cuh: ~115 FP64 operations per pair instead of forming the 2 x 18 Kelvin kernels)
// Gauss points [q_begin, q_end) of slice blockIdx.y of gridDim.y (a multiple of kPostStage)
__device__ __forceinline__ void post_slice(int64_t nq, int64_t& qb, int64_t& qe) {
  const int64_t per = ((nq + gridDim.y - 1) / gridDim.y + kPostStage - 1) / kPostStage * kPostStage;
  qb = min(nq, (int64_t)blockIdx.y * per);
  qe = min(nq, qb + per);
}

__global__ void __launch_bounds__(128) bem_post_kernel(const double* __restrict__ pts, int nump,
                                                       const double* __restrict__ tab, int64_t nq, BemPostCoef cf,
                                                       double* __restrict__ part) {
  __shared__ double sq[kPostStage * kPostRec];
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  const bool act = s < nump;
  double P0 = 0, P1 = 0, P2 = 0;
  if (act) { P0 = pts[3 * s]; P1 = pts[3 * s + 1]; P2 = pts[3 * s + 2]; }
  double acc[6] = {0, 0, 0, 0, 0, 0};
  int64_t qb, qe;
  post_slice(nq, qb, qe);
  for (int64_t q0 = qb; q0 < qe; q0 += kPostStage) {
    const int nqs = (int)min((int64_t)kPostStage, qe - q0);
    __syncthreads();
    for (int idx = threadIdx.x; idx < nqs * kPostRec; idx += blockDim.x) sq[idx] = tab[q0 * kPostRec + idx];
    __syncthreads();
    if (!act) continue;
    for (int qq = 0; qq < nqs; ++qq) {
      const double* r = sq + qq * kPostRec;
      double sg[6];
      bem_post_contracted(r[0] - P0, r[1] - P1, r[2] - P2, r[3], r[4], r[5], r[7], r[8], r[9], r[10], r[11], r[12], cf,
                          sg);
      const double wj = r[6];
#pragma unroll
      for (int t = 0; t < 6; ++t) acc[t] += wj * sg[t];
    }
  }
  if (act)
#pragma unroll
    for (int t = 0; t < 6; ++t) part[6 * ((int64_t)blockIdx.y * nump + s) + t] = acc[t];
}

// stress = sum of the slices' partial sums, in slice order (the same result on every run)
__global__ void k_post_reduce(int nump, int nslice, const double* __restrict__ part, double* __restrict__ stress) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= 6 * (int64_t)nump) return;
  double v = 0.0;
  for (int k = 0; k < nslice; ++k) v += part[(int64_t)k * 6 * nump + i];
  stress[i] = v;
}

// double-float records of the Gauss points (one thread each)
__global__ void k_post_df_table(const double* __restrict__ tab, int64_t nq, BemPostCoef cf,
                                ibem::BemPostDF* __restrict__ out) {
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q < nq) out[q] = ibem::bem_post_df_record(tab + q * kPostRec, cf);
}

// the mixed form's boundary sums: double-float contraction (bem_contract.cuh), the records
// staged in shared memory 64 at a time, compensated sums per component
constexpr int kPostStageDF = 64;
__global__ void __launch_bounds__(128) bem_post_kernel_df(const double* __restrict__ pts, int nump,
                                                          const ibem::BemPostDF* __restrict__ tab, int64_t nq,
                                                          ibem::BemPostCoefDF cf, double* __restrict__ part) {
  static_assert(sizeof(ibem::BemPostDF) == 11 * sizeof(float4), "BemPostDF is copied as 11 float4");
  __shared__ __align__(16) ibem::BemPostDF sq[kPostStageDF];
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  const bool act = s < nump;
  ibem::dfloat p[3] = {};
  if (act)
    for (int k = 0; k < 3; ++k) p[k] = ibem::df_make(pts[3 * (int64_t)s + k]);
  ibem::dacc acc[6] = {};
  int64_t qb, qe;
  post_slice(nq, qb, qe);   // slice boundaries are multiples of kPostStage, hence of kPostStageDF
  for (int64_t q0 = qb; q0 < qe; q0 += kPostStageDF) {
    const int nqs = (int)min((int64_t)kPostStageDF, qe - q0);
    __syncthreads();
    {
      const float4* src = reinterpret_cast<const float4*>(tab + q0);
      float4* dst = reinterpret_cast<float4*>(sq);
      for (int i = threadIdx.x; i < nqs * 11; i += blockDim.x) dst[i] = src[i];
    }
    __syncthreads();
    if (!act) continue;
#pragma unroll 1
    for (int qq = 0; qq < nqs; ++qq) ibem::bem_post_contracted_df(p, sq[qq], cf, acc);
  }
  if (act)
#pragma unroll
    for (int t = 0; t < 6; ++t) part[6 * ((int64_t)blockIdx.y * nump + s) + t] = (double)acc[t].s + (double)acc[t].c;
}

}  // namespace

namespace ibem {

// Node incidence lists of the mesh (see k_inc_*), in stream-ordered memory freed by the caller
// with cudaFreeAsync: *start (NN + 1 ints) then the slots (4 NE ints) in one allocation.
static ibem_status node_incidence(const int* conn, int NN, int NE, int** start, int** slot, cudaStream_t st) {
  int* buf = nullptr;
  const size_t n = (size_t)(NN + 1) + 2 * (size_t)NN + 4 * (size_t)NE;
  IBEM_CUDA(cudaMallocAsync((void**)&buf, sizeof(int) * n, st));
  int* s0 = buf;
  int* cnt = s0 + NN + 1;
  int* cur = cnt + NN;
  int* sl = cur + NN;
  IBEM_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int) * 2 * (size_t)NN, st));
  const unsigned g4 = (unsigned)((4 * (int64_t)NE + 255) / 256);
  if (NE > 0) ::ibem::count_launch(), k_inc_count<<<g4, 256, 0, st>>>(conn, NE, NN, cnt);
  ::ibem::count_launch(), k_inc_scan<<<1, 1024, 0, st>>>(cnt, NN, s0);
  if (NE > 0) ::ibem::count_launch(), k_inc_fill<<<g4, 256, 0, st>>>(conn, NE, NN, s0, cur, sl);
  ::ibem::count_launch(), k_inc_sort<<<(NN + 255) / 256, 256, 0, st>>>(NN, s0, sl);
  IBEM_LAUNCH_CHECK("node incidence");
  *start = s0;
  *slot = sl;
  return IBEM_OK;
}

static dim3 gather_grid(int64_t nrows, int NN) {
  return dim3((unsigned)((nrows + 255) / 256), (unsigned)std::min(NN, 65535));
}

ibem_status bem_hg(const double* nodes, int NN, const int* conn, int NE, const ibem_material& m,
                   double* H, int64_t ldh, int64_t hrow0, int64_t hcol0, double* G, int64_t ldg,
                   int64_t grow0, int64_t gcol0, cudaStream_t st) {
  double* Hb = H + hcol0 * ldh + hrow0;
  double* Gb = G + gcol0 * ldg + grow0;
  if (NN <= 0) return IBEM_OK;
  const int64_t ldt = 3 * (int64_t)NN;
  double* TG = nullptr;
  const size_t tg_bytes = sizeof(double) * ldt * 12 * (size_t)(NE > 0 ? NE : 1);
  IBEM_CUDA(cudaMallocAsync((void**)&TG, tg_bytes, st));
  IBEM_CUDA(cudaMemsetAsync(TG, 0, tg_bytes, st));   // an element with bad connectivity adds nothing
  int *start = nullptr, *slot = nullptr;
  ibem_status s = node_incidence(conn, NN, NE, &start, &slot, st);
  if (s) { cudaFreeAsync(TG, st); return s; }
  const double mu = m.E0 / (2 * (1 + m.nu0));
  KelvinC kc;
  kc.cu = 1.0 / (16 * IBEM_PI * mu * (1 - m.nu0));
  kc.c1 = 3 - 4 * m.nu0;
  kc.ct = 1.0 / (8 * IBEM_PI * (1 - m.nu0));
  kc.c3 = 1 - 2 * m.nu0;
  dim3 grid((NN + 127) / 128, NE);
  if (NE > 0) ::ibem::count_launch(), bem_hg_kernel<<<grid, 128, 0, st>>>(nodes, NN, conn, kc, TG, ldt, Gb, ldg);
  ::ibem::count_launch(), k_node_gather<<<gather_grid(ldt, NN), 256, 0, st>>>(ldt, NN, start, slot, TG, ldt, Hb, ldh, 0);
  ::ibem::count_launch(), bem_diag_kernel<<<(3 * NN + 127) / 128, 128, 0, st>>>(NN, Hb, ldh);
  cudaFreeAsync(start, st);
  cudaFreeAsync(TG, st);
  IBEM_LAUNCH_CHECK("bem_hg");
  return IBEM_OK;
}

ibem_status bem_to_incl(const double* nodes, int NN, const int* conn, int NE, const double* cen,
                        int num, const ibem_material& m, int layout, double* H, int64_t ldh,
                        int64_t hcol0, double* G, int64_t ldg, int64_t gcol0, int64_t row0,
                        cudaStream_t st) {
  BemMat bm = bem_mat_init(m.E0, m.nu0, m.E1, m.nu1);
  double* Hb = H + hcol0 * ldh + row0;
  double* Gb = G + gcol0 * ldg + row0;
  const int compact = layout == 60;
  if (NN <= 0 || NE <= 0 || num <= 0) return IBEM_OK;
  const int64_t rows = (int64_t)layout * num;
  double* UG = nullptr;
  const size_t ug_bytes = sizeof(double) * rows * 12 * (size_t)NE;
  IBEM_CUDA(cudaMallocAsync((void**)&UG, ug_bytes, st));
  IBEM_CUDA(cudaMemsetAsync(UG, 0, ug_bytes, st));   // an element with bad connectivity adds nothing
  int *start = nullptr, *slot = nullptr;
  ibem_status s = node_incidence(conn, NN, NE, &start, &slot, st);
  if (s) { cudaFreeAsync(UG, st); return s; }
  dim3 g0((num + 127) / 128, NE, 3), g1((num + 127) / 128, NE, 9), g2((num + 127) / 128, NE, 27);
  ::ibem::count_launch(), bem_incl_kernel<0><<<g0, 128, 0, st>>>(nodes, NN, conn, cen, num, bm, layout, compact, UG, rows, Gb, ldg);
  ::ibem::count_launch(), bem_incl_kernel<1><<<g1, 128, 0, st>>>(nodes, NN, conn, cen, num, bm, layout, compact, UG, rows, Gb, ldg);
  if (layout != 24)
    ::ibem::count_launch(), bem_incl_kernel<2><<<g2, 128, 0, st>>>(nodes, NN, conn, cen, num, bm, layout, compact, UG, rows, Gb, ldg);
  ::ibem::count_launch(), k_node_gather<<<gather_grid(rows, NN), 256, 0, st>>>(rows, NN, start, slot, UG, rows, Hb, ldh, 1);
  cudaFreeAsync(start, st);
  cudaFreeAsync(UG, st);
  IBEM_LAUNCH_CHECK("bem_to_incl");
  return IBEM_OK;
}

ibem_status bem_post(const double* pts, int nump, const double* nodes, int NN, const int* conn,
                     int NE, const ibem_material& m, const double* U, const double* T,
                     double* stress, cudaStream_t st, bool mixed) {
  BemMat bm = bem_mat_init(m.E0, m.nu0, m.E1, m.nu1);
  const BemPostCoef cf = bem_post_coef(bm);
  ProfScope ps(PROF_BEM, st);
  const int64_t nq = (int64_t)NE * kPostQ;
  double* tab = nullptr;
  // source slices of the Gauss points: about 8 CTAs per SM in total, at least one staged
  // chunk each (few sample points would otherwise leave most SMs idle)
  int dev = 0, nsm = 0;
  IBEM_CUDA(cudaGetDevice(&dev));
  IBEM_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const int gx = (nump + 127) / 128;
  const int64_t chunks = (nq + kPostStage - 1) / kPostStage;
  const int nslice = (int)std::max<int64_t>(1, std::min<int64_t>((8 * (int64_t)nsm + gx - 1) / gx, chunks));
  const size_t tab_bytes = (sizeof(double) * kPostRec * (nq > 0 ? nq : 1) + 255) / 256 * 256;
  const size_t df_bytes = mixed ? (sizeof(BemPostDF) * (nq > 0 ? nq : 1) + 255) / 256 * 256 : 0;
  const size_t part_bytes = sizeof(double) * 6 * (size_t)nslice * (size_t)nump;
  IBEM_CUDA(cudaMallocAsync((void**)&tab, tab_bytes + df_bytes + part_bytes, st));
  BemPostDF* tdf = mixed ? reinterpret_cast<BemPostDF*>(reinterpret_cast<char*>(tab) + tab_bytes) : nullptr;
  double* part = reinterpret_cast<double*>(reinterpret_cast<char*>(tab) + tab_bytes + df_bytes);
  const unsigned gq = (unsigned)((nq + 127) / 128);
  const dim3 grid((unsigned)gx, (unsigned)nslice);
  if (nq > 0)
    ::ibem::count_launch(), bem_post_table<<<gq, 128, 0, st>>>(nodes, NN, conn, NE, U, T, tab);
  if (mixed) {
    if (nq > 0) ::ibem::count_launch(), k_post_df_table<<<gq, 128, 0, st>>>(tab, nq, cf, tdf);
    ::ibem::count_launch(), bem_post_kernel_df<<<grid, 128, 0, st>>>(pts, nump, tdf, nq, bem_post_coef_df(cf), part);
  } else {
    ::ibem::count_launch(), bem_post_kernel<<<grid, 128, 0, st>>>(pts, nump, tab, nq, cf, part);
  }
  ::ibem::count_launch(), k_post_reduce<<<(unsigned)((6 * (int64_t)nump + 255) / 256), 256, 0, st>>>(nump, nslice,
                                                                                                   part, stress);
  cudaFreeAsync(tab, st);
  IBEM_LAUNCH_CHECK("bem_post");
  return IBEM_OK;
}

}  // namespace ibem
