// pn_device.cuh -- device kernels of the PN-moment energy march (sm_103a).
//
// One launch advances the classes of one parity by one StaRMAP sub-step (starmap/src/solver.jl:
// 171-196): for every target cell it
//   1. (face cells only) evaluates the ghost values of the neighbouring class that the cell's
//      stencil reads, from the cell's own old values and the neighbour's interior value
//      (apply_boundary_source!/zero!, starmap/src/boundary_conditions.jl:67-102), and stores them;
//   2. forms du = sum_d A_d (u_r - u_l) / h_d over the active axes with the generated sparse
//      stencils (kernel!/matmuldiff!, starmap/src/solver_core.jl:59-69,108-137);
//   3. applies du = ((Q - du) - C u) / S * phi1(-C/S dt) with S = sum_e rho_e s_e and
//      C_l = sum_e rho_e c_{e,l} formed on the fly from the per-step tables (weighted_sum!,
//      pn_solver/pn_problem.jl:213-249; right_hand_side!, solver_core.jl:92-106) and
//   4. writes u + dt du (update!, solver.jl:149-168).
// A ghost value that lies outside the grid along exactly one axis is read by exactly one target
// cell -- the cell at that face of the switched class -- so the thread that owns that cell
// computes it, with no other thread reading or writing it during the launch.  Ghosts along two or
// more axes are read by no stencil and are not maintained.
//
// The plain path (one solve per launch) runs these sub-steps and the density integral with two
// threads per target cell (substep_split_kernel, integrate_split_kernel), each updating the
// moments of half of the cell's degrees, with the same arithmetic per moment.
//
// The adjoint density kernel (integrate_adjoint_densities!, pn_solver/pn_intensities.jl:129-164)
// evaluates du of a tape state for every class (plain right-hand side, no exponential factor) and
// accumulates rho_bar[e] += sum_m lambda_m (s_e du_m + c_{e,l(m)} u_m) dvol dE w, plus the eee
// pullbacks of the intensity integral (integrate_step_and_add_pullback!,
// pn_solver/x_ray_intensities.jl:193-223).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "generated/pn_stencils.cuh"
#include "pn_f32x2.cuh"

namespace pn {

constexpr int MAXE = 4;     // elements per solve
constexpr int MAXR = 8;     // x-ray lines per solve
constexpr int MAXSEG = 16;  // work segments per launch
constexpr int BLOCK = 128;  // threads per block of the batched generic kernels
// threads per block of the plain (one solve per launch) kernels: one solve's sub-step launch has
// only ~4 blocks of 128 per SM on a 2D P11 grid, so 64-thread blocks halve the imbalance between
// SMs with one block more and one block fewer
#ifndef PN_PLAIN_BLOCK
#define PN_PLAIN_BLOCK 64
#endif
constexpr int PBLOCK = PN_PLAIN_BLOCK;

struct Geom {
  int n[3];        // points per axis (ghosts included)
  int px;          // x pitch in elements
  int nm;          // moments
  int pad;
  long long ms;    // moment stride in elements (px * ny * nz)
};

// A contiguous range of blocks working on one target class: either an inner box (cells whose
// stencil needs no ghost) tiled tile_x x (128 / tile_x), or a list of face cells.
struct Seg {
  int cls;
  int kind;        // 0 = box, 1 = face list
  int block0;
  int nblocks;
  int lo[3];
  int ext[3];
  int tiles_x, tiles_y;
  int tile_x;
  int n_face;
  const int* faces;  // packed i | j << 11 | k << 22
};

__host__ __device__ inline int pack_cell(int i, int j, int k) { return i | (j << 11) | (k << 22); }

__host__ __device__ inline int class_parity_d(int c) { return (((c >> 2) & 1) + ((c >> 1) & 1) + (c & 1)) & 1; }

template <class T, int N>
struct SubArgs {
  Geom g[8];
  T* rd[8];                   // read pointer per class (from-classes, own old values, ghosts)
  T* wr[8];                   // write pointer per class (targets)
  const T* rho[8];            // [e][z][y][x] with the class geometry
  const double* bmat[3][8];   // boundary blocks n_f x n_t (row-major)
  const double* beam[8];      // right-x-face source [z][y][m] (classes odd in x)
  int act[3];                 // active axes
  int ne, nr;
  int nseg;
  int adjoint_source;         // add Q on eee moment 0
  T dt;
  double bc;                  // beam energy weight of this step (forward source)
  double scale_g;             // multiplier of the beam source (power of two)
  T s[MAXE];
  T c[MAXE][N + 1];
  // adjoint source on eee moment 0: Q = -sum_r sigma_r ACS NOA ibar_r
  const double* acs;          // [cell][r], eee cells
  const double* noa;          // [cell][e]
  const double* ibar;         // [r] (device)
  int xel[MAXR];
  double sig_src[MAXR];
  static constexpr bool line_src = false;   // Q from acs, noa and ibar per line
  // intensity partial sums of the new eee moment 0 (forward, even sub-step)
  const double* wint;         // [cell][r] = ACS * NOA
  double* partial;            // [block][r]
  // right-hand-side factors of the odd classes, shared by the two half sub-steps of one step
  // (same coefficients, densities and dt): planes 1/S, C_0..C_N, phi1_0..phi1_N per class
  T* cache[8];
  int cache_mode;             // 0 none, 1 compute and store, 2 load
  int pre_ghosts;             // 1: ghost_kernel wrote the face ghosts before this launch
  Seg seg[MAXSEG];
  T tab[Ord<N>::n_tab];       // advection nnz values divided by the grid step
};

template <class T, int N>
struct IntArgs {
  Geom g[8];
  T* u[8];                    // tape state (ghosts rewritten)
  const T* lam[8];            // adjoint state
  const T* rho[8];
  double* rbar[8];            // rho_bar per class [e][z][y][x]
  const double* bmat[3][8];   // forward boundary blocks
  const double* beam[8];
  int act[3];
  int ne, nr;
  int nseg;
  double bc;
  double scale_g;
  double wfac;                // dvol * dE * w
  T s[MAXE];
  T c[MAXE][N + 1];
  const double* acs;
  const double* noa;
  const double* ibar;
  double* acs_bar;
  double* noa_bar;
  int xel[MAXR];
  double coef[MAXR];          // dE * dvol * sigma_r * w   (times ibar_r in the kernel)
  static constexpr bool line_sums = false;   // accumulate acs_bar / noa_bar directly
  int pre_ghosts;             // 1: ghost_kernel wrote the face ghosts before this launch
  Seg seg[MAXSEG];
  T tab[Ord<N>::n_tab];
};

// --------------------------------------------------------------------------------------------
// small helpers
// --------------------------------------------------------------------------------------------
// 1 / n! as the double nearest to it (n! is exact in a double for n <= 18)
__host__ __device__ constexpr double inv_fact(int n) {
  double f = 1.0;
  for (int i = 2; i <= n; ++i) f *= i;
  return 1.0 / f;
}

// sum_{k=0..K} c^k / (k+1)! in Horner form (K FMAs)
template <int K>
__device__ __forceinline__ double phi1_series(double c) {
  double t = inv_fact(K + 1);
#pragma unroll
  for (int k = K - 1; k >= 0; --k) t = fma(t, c, inv_fact(k + 1));
  return t;
}

// FP64 phi1(c) = (e^c - 1) / c, expm1div of solver_core.jl:38-44.  |c| <= 2e-4: the reference's
// own Taylor form.  Above, the series sum_k c^k / (k+1)! truncated after the term K that keeps its
// truncation below ~5e-16 relative on the range of |c| (the same order as the cancellation error
// of the reference's (e^c - 1) / c there): K = 6 below 0.03, 8 below 0.1, 10 below 0.3 (4.3e-15 at
// 0.3), 14 below 0.7; beyond, (exp(c) - 1) / c as the reference.  The factors of the 2D workloads
// reach |c| = 0.27 on half steps and 0.62 on full steps (the high degrees), which before the K = 14
// range paid an FP64 exponential and a division on this GPU's scarce FP64 pipe.  The range is
// chosen on the integer pipe from the high word of c (monotone in |c|; each bound rounds down to
// its high word, by less than 2^-20 relative).
__device__ __forceinline__ double phi1(double c) {
  if (fabs(c) <= 0.0002) return 1.0 + 0.5 * c + 1.0 / 6.0 * (c * c);
  const unsigned hi = (unsigned)__double2hiint(c) & 0x7fffffffu;
  if (hi < 0x3f9eb851u) return phi1_series<6>(c);    // |c| < 0.03
  if (hi < 0x3fb99999u) return phi1_series<8>(c);    // |c| < 0.1
  if (hi < 0x3fd33333u) return phi1_series<10>(c);   // |c| < 0.3
  if (hi < 0x3fe66666u) return phi1_series<14>(c);   // |c| < 0.7
  return (exp(c) - 1.0) / c;
}

// FP32 phi1(c) = (e^c - 1) / c.  |c| <= 1/4: the Taylor series sum_k c^k / (k+1)! to k = 6
// (truncation below 2e-9 relative); otherwise the fast exponential and division (ex2.approx-based
// __expf, __fdividef), whose relative error is ~1e-6 at |c| = 1/4, where e^c - 1 cancels most,
// and smaller beyond.  pn_selftest_phi1 compares it with expm1f(c) / c on the device.
// The Horner steps are written as explicit FMAs so that the scalar form and the two-lane form
// (phi1 of an f2, the tile kernels) round identically.
__device__ __forceinline__ float phi1_series(float c) {
  float t = fmaf(c, 1.0f / 5040.0f, 1.0f / 720.0f);
  t = fmaf(c, t, 1.0f / 120.0f);
  t = fmaf(c, t, 1.0f / 24.0f);
  t = fmaf(c, t, 1.0f / 6.0f);
  t = fmaf(c, t, 0.5f);
  return fmaf(c, t, 1.0f);
}

__device__ __forceinline__ float phi1(float c) {
  if (fabsf(c) <= 0.25f) return phi1_series(c);
  return __fdividef(__expf(c) - 1.0f, c);
}

// both lanes of an f2: the series on both at once, a lane beyond 1/4 by the scalar form
__device__ __forceinline__ f2 phi1(f2 c) {
  f2 t = fma(c, splat(1.0f / 5040.0f), splat(1.0f / 720.0f));
  t = fma(c, t, splat(1.0f / 120.0f));
  t = fma(c, t, splat(1.0f / 24.0f));
  t = fma(c, t, splat(1.0f / 6.0f));
  t = fma(c, t, splat(0.5f));
  t = fma(c, t, splat(1.0f));
  if (fabsf(c.x) > 0.25f) t.x = __fdividef(__expf(c.x) - 1.0f, c.x);
  if (fabsf(c.y) > 0.25f) t.y = __fdividef(__expf(c.y) - 1.0f, c.y);
  return t;
}

// the reference form in FP32, for the self-test
__device__ __forceinline__ float phi1_ref(float c) {
  if (fabsf(c) <= 1e-3f) return 1.0f + c * (0.5f + c * (1.0f / 6.0f));
  return expm1f(c) / c;
}

template <class T>
__device__ __forceinline__ T recip(T x) { return T(1) / x; }


// minimum resident blocks per SM the plain sub-step kernel is compiled for: 5 keeps the FP64 P11
// instances within 96 registers (5 x 4 warps per SM to feed the FP64 pipe, instead of 4 x 4)
#ifndef PN_PLAIN_MINB
#define PN_PLAIN_MINB 5
#endif

// C_l = sum_e rho_e c_{e,l} for the degrees of a class, over the solve's ne elements only
template <class T, int N, unsigned MASK, int NE>
__device__ __forceinline__ void cl_sums_n(const T* rr, const T (*c)[N + 1], T* Cl) {
#pragma unroll
  for (int l = 0; l <= N; ++l) {
    T cc = T(0);
    if ((MASK >> l) & 1u) {
#pragma unroll
      for (int e = 0; e < NE; ++e) cc = fma(rr[e], c[e][l], cc);
    }
    Cl[l] = cc;
  }
}

template <class T, int N, unsigned MASK>
__device__ __forceinline__ void cl_sums(const T* rr, const T (*c)[N + 1], int ne, T* Cl) {
  switch (ne) {
    case 1: cl_sums_n<T, N, MASK, 1>(rr, c, Cl); break;
    case 2: cl_sums_n<T, N, MASK, 2>(rr, c, Cl); break;
    case 3: cl_sums_n<T, N, MASK, 3>(rr, c, Cl); break;
    default: cl_sums_n<T, N, MASK, MAXE>(rr, c, Cl); break;
  }
}

template <int BS = BLOCK>
__device__ __forceinline__ bool locate(const Seg* seg, int nseg, int b, int tid, int& s, int& i, int& j,
                                       int& k) {
  s = 0;
  while (s + 1 < nseg && b >= seg[s + 1].block0) ++s;
  const Seg& g = seg[s];
  const int lb = b - g.block0;
  if (g.kind == 0) {
    const int ty = BS / g.tile_x;
    const int bx = lb % g.tiles_x;
    const int rest = lb / g.tiles_x;
    const int by = rest % g.tiles_y;
    const int bz = rest / g.tiles_y;
    const int li = bx * g.tile_x + tid % g.tile_x;
    const int lj = by * ty + tid / g.tile_x;
    if (li >= g.ext[0] || lj >= g.ext[1] || bz >= g.ext[2]) return false;
    i = g.lo[0] + li;
    j = g.lo[1] + lj;
    k = g.lo[2] + bz;
    return true;
  }
  const int f = lb * BS + tid;
  if (f >= g.n_face) return false;
  const int p = g.faces[f];
  i = p & 2047;
  j = (p >> 11) & 2047;
  k = (p >> 22) & 1023;
  return true;
}

__device__ __forceinline__ long long lin(const Geom& g, int i, int j, int k) {
  return ((long long)k * g.n[1] + j) * g.px + i;
}

__device__ __forceinline__ long long eee_cell(const Geom& g, int i, int j, int k) {
  return ((long long)k * g.n[1] + j) * g.n[0] + i;
}

// rows of a boundary block evaluated together by a face thread
#ifndef PN_GHOST_ROWS
#define PN_GHOST_ROWS 1
#endif

// Ghost of class F = switch(C, d) next to target cell (i,j,k) of class C (C even along d, cell on
// a face along d).  Writes the ghost into F's storage.  `left` selects the face at index 0.
template <class T, int N, int C, int D>
__device__ __forceinline__ void ghost_fill(T* const* rd, const Geom* g, const double* const (*bmat)[8],
                                           const double* const* beam, double bc_scaled, bool source,
                                           int i, int j, int k, bool left) {
  constexpr int F = C ^ (4 >> D);
  constexpr int nt = Ord<N>::n(C);
  constexpr int nf = Ord<N>::n(F);
  if constexpr (nt == 0 || nf == 0) {
    return;
  } else {
    const Geom& gt = g[C];
    const Geom& gf = g[F];
    const T* ut = rd[C] + lin(gt, i, j, k);
    T v[nt];
#pragma unroll
    for (int m = 0; m < nt; ++m) v[m] = ut[m * gt.ms];
    int c[3] = {i, j, k};
    int cg[3] = {i, j, k};
    int ci[3] = {i, j, k};
    if (left) {
      cg[D] = 0;
      ci[D] = 1;
    } else {
      cg[D] = c[D] + 1;
      ci[D] = c[D];
    }
    T* fg = rd[F] + lin(gf, cg[0], cg[1], cg[2]);
    const T* fi = rd[F] + lin(gf, ci[0], ci[1], ci[2]);
    const double* B = bmat[D][F];
    const bool src = source && D == 0 && !left;
    const double* bm = src ? beam[F] + ((long long)k * gf.n[1] + j) * nf : nullptr;
    // PN_GHOST_ROWS rows of B v at a time in FP64: independent dot products in flight, each still
    // summed over q in order, so the values do not depend on the chunking (7 rows measured 10 %
    // slower on the 2D P11 solve than 1: register pressure).  FP32 keeps one row.
    constexpr int RC = sizeof(T) == 8 ? PN_GHOST_ROWS : 1;
#pragma unroll 1
    for (int r0 = 0; r0 < nf; r0 += RC) {
      T bv[RC];
#pragma unroll
      for (int rr = 0; rr < RC; ++rr) bv[rr] = T(0);
#pragma unroll
      for (int q = 0; q < nt; ++q) {
        const T vq = v[q];
#pragma unroll
        for (int rr = 0; rr < RC; ++rr)
          if (r0 + rr < nf) bv[rr] = fma(T(B[(r0 + rr) * nt + q]), vq, bv[rr]);
      }
#pragma unroll
      for (int rr = 0; rr < RC; ++rr) {
        const int r = r0 + rr;
        if (r < nf) {
          const T gval = src ? T(bm[r] * bc_scaled) : T(0);
          const T interior = fi[r * gf.ms];
          const T gh = left ? T(2) * (gval - bv[rr]) - interior : T(2) * (bv[rr] + gval) - interior;
          fg[r * gf.ms] = gh;
        }
      }
    }
  }
}

template <class T, int N, int C>
__device__ __forceinline__ void ghosts_for_cell(T* const* rd, const Geom* g, const int* act,
                                                const double* const (*bmat)[8], const double* const* beam,
                                                double bc_scaled, bool source, int i, int j, int k) {
  const int c3[3] = {i, j, k};
  if (act[0] && !((C >> 2) & 1)) {
    if (c3[0] == 0) ghost_fill<T, N, C, 0>(rd, g, bmat, beam, bc_scaled, source, i, j, k, true);
    if (c3[0] == g[C].n[0] - 1) ghost_fill<T, N, C, 0>(rd, g, bmat, beam, bc_scaled, source, i, j, k, false);
  }
  if (act[1] && !((C >> 1) & 1)) {
    if (c3[1] == 0) ghost_fill<T, N, C, 1>(rd, g, bmat, beam, bc_scaled, source, i, j, k, true);
    if (c3[1] == g[C].n[1] - 1) ghost_fill<T, N, C, 1>(rd, g, bmat, beam, bc_scaled, source, i, j, k, false);
  }
  if (act[2] && !(C & 1)) {
    if (c3[2] == 0) ghost_fill<T, N, C, 2>(rd, g, bmat, beam, bc_scaled, source, i, j, k, true);
    if (c3[2] == g[C].n[2] - 1) ghost_fill<T, N, C, 2>(rd, g, bmat, beam, bc_scaled, source, i, j, k, false);
  }
}

// --------------------------------------------------------------------------------------------
// face ghosts ahead of a launch
// --------------------------------------------------------------------------------------------
// A ghost line: the ghost of F = switch(C, dim) next to face cell `cell` (packed) of target class
// C, on the face at index 0 (`left`) or at the last index along dim.
struct GLine {
  int cls, dim, left, cell;
};

template <class T>
struct GhostArgs {
  Geom g[8];
  T* rd[8];                   // target classes (read) and their switched classes (ghosts written)
  const double* bmat[3][8];
  const double* beam[8];
  double bc_scaled;
  int source;                 // forward problem: beam source on the right x face
  const GLine* lines;
  int n_lines;
};

// Component r of one ghost line: ghost_fill's arithmetic for that component (the same dot product
// over q in the same order), so the values are those the face threads would form.
template <class T, int N, int C, int D>
__device__ __forceinline__ void ghost_component(const GhostArgs<T>& a, int i, int j, int k, bool left, int r) {
  constexpr int F = C ^ (4 >> D);
  constexpr int nt = Ord<N>::n(C);
  constexpr int nf = Ord<N>::n(F);
  if constexpr (nt == 0 || nf == 0 || ((C >> (2 - D)) & 1)) {
    (void)a; (void)i; (void)j; (void)k; (void)left; (void)r;
  } else {
    if (r >= nf) return;
    const Geom& gt = a.g[C];
    const Geom& gf = a.g[F];
    const T* ut = a.rd[C] + lin(gt, i, j, k);
    int cg[3] = {i, j, k};
    int ci[3] = {i, j, k};
    if (left) {
      cg[D] = 0;
      ci[D] = 1;
    } else {
      cg[D] = cg[D] + 1;
    }
    T* fg = a.rd[F] + lin(gf, cg[0], cg[1], cg[2]);
    const T* fi = a.rd[F] + lin(gf, ci[0], ci[1], ci[2]);
    const double* B = a.bmat[D][F];
    T bv = T(0);
#pragma unroll
    for (int q = 0; q < nt; ++q) bv = fma(T(B[r * nt + q]), ut[q * gt.ms], bv);
    const bool src = a.source && D == 0 && !left;
    const T gval = src ? T(a.beam[F][((long long)k * gf.n[1] + j) * nf + r] * a.bc_scaled) : T(0);
    const T interior = fi[r * gf.ms];
    fg[r * gf.ms] = left ? T(2) * (gval - bv) - interior : T(2) * (bv + gval) - interior;
  }
}

template <class T, int N, int C>
__device__ __forceinline__ void ghost_line(const GhostArgs<T>& a, const GLine& gl, int r) {
  const int i = gl.cell & 2047, j = (gl.cell >> 11) & 2047, k = (gl.cell >> 22) & 1023;
  switch (gl.dim) {
    case 0: ghost_component<T, N, C, 0>(a, i, j, k, gl.left != 0, r); break;
    case 1: ghost_component<T, N, C, 1>(a, i, j, k, gl.left != 0, r); break;
    default: ghost_component<T, N, C, 2>(a, i, j, k, gl.left != 0, r); break;
  }
}

// One warp per ghost line, lane r forms component r.  Launched before a sub-step (or density
// integral) whose face cells then skip ghosts_for_cell: the boundary products, which made the face
// threads several times slower than the interior ones and their SMs the last to finish, spread
// over a full grid.
template <class T, int N>
__global__ void __launch_bounds__(256) ghost_kernel(const __grid_constant__ GhostArgs<T> a) {
  const int line = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5);
  const int r = threadIdx.x & 31;
  if (line >= a.n_lines) return;
  const GLine gl = a.lines[line];
  switch (gl.cls) {
    case 0: ghost_line<T, N, 0>(a, gl, r); break;
    case 1: ghost_line<T, N, 1>(a, gl, r); break;
    case 2: ghost_line<T, N, 2>(a, gl, r); break;
    case 3: ghost_line<T, N, 3>(a, gl, r); break;
    case 4: ghost_line<T, N, 4>(a, gl, r); break;
    case 5: ghost_line<T, N, 5>(a, gl, r); break;
    case 6: ghost_line<T, N, 6>(a, gl, r); break;
    default: ghost_line<T, N, 7>(a, gl, r); break;
  }
}

// acc[m] += sum over active axes of A_d[C] (f_r - f_l) / h_d  (sign flipped for the adjoint).
// LIT = false: coefficients from `tab`, already divided by h_d.  LIT = true: the literal closed-form
// coefficient compiled into the stencil, with the difference multiplied by inv_h.
template <class T, int N, int C, int D, bool NEG, bool LIT>
__device__ __forceinline__ void stencil_axis(T* acc, T* const* rd, const Geom* g, int i, int j, int k,
                                             const T* tab, T inv_h) {
  constexpr int F = C ^ (4 >> D);
  constexpr int nf = Ord<N>::n(F);
  if constexpr (nf == 0 || Ord<N>::n(C) == 0) {
    return;
  } else {
    const Geom& gf = g[F];
    int r3[3] = {i, j, k};
    int l3[3] = {i, j, k};
    if ((C >> (2 - D)) & 1) {  // odd target: even neighbour at i (right) and i - 1 (left)
      l3[D] -= 1;
    } else {                   // even target: odd neighbour at i + 1 (right) and i (left)
      r3[D] += 1;
    }
    const T* fr = rd[F] + lin(gf, r3[0], r3[1], r3[2]);
    const T* fl = rd[F] + lin(gf, l3[0], l3[1], l3[2]);
    const long long ms = gf.ms;
    auto diff = [&](int q) -> T {
      const T a = fr[q * ms];
      const T b = fl[q * ms];
      const T d = NEG ? (b - a) : (a - b);
      if constexpr (LIT) return d * inv_h;
      else return d;
    };
    constexpr int off = Ord<N>::off(C, D);
    auto coef = [&](int kk, double lit) -> T {
      if constexpr (LIT) {
        (void)kk;
        return T(lit);
      } else {
        (void)lit;
        return tab[off + kk];
      }
    };
    Adv<N, C, D>::template apply<T>(acc, diff, coef);
  }
}

template <bool LIT, class T, class A>
__device__ __forceinline__ const T* tab_of(const A& a) {
  if constexpr (LIT) return nullptr;
  else return a.tab;
}

template <bool LIT, class T, class A>
__device__ __forceinline__ T invh_of(const A& a, int d) {
  if constexpr (LIT) return a.inv_h[d];
  else return T(1);
}

// Neighbour values of one axis, loaded before any arithmetic so that every load of a cell is in
// flight at once (used when the active axes are known at compile time, DIMS != 0).
template <class T, int N, int C, int D>
struct Nbr {
  static constexpr int F = C ^ (4 >> D);
  static constexpr int nf = Ord<N>::n(F);
  T r[nf > 0 ? nf : 1];
  T l[nf > 0 ? nf : 1];
};

template <class T, int N, int C, int D>
__device__ __forceinline__ void load_nbr(Nbr<T, N, C, D>& v, T* const* rd, const Geom* g, int i, int j, int k) {
  constexpr int F = C ^ (4 >> D);
  constexpr int nf = Ord<N>::n(F);
  if constexpr (nf > 0 && Ord<N>::n(C) > 0) {
    const Geom& gf = g[F];
    int r3[3] = {i, j, k};
    int l3[3] = {i, j, k};
    if ((C >> (2 - D)) & 1) l3[D] -= 1;
    else r3[D] += 1;
    const T* fr = rd[F] + lin(gf, r3[0], r3[1], r3[2]);
    const T* fl = rd[F] + lin(gf, l3[0], l3[1], l3[2]);
    const long long ms = gf.ms;
#pragma unroll
    for (int q = 0; q < nf; ++q) {
      v.r[q] = fr[q * ms];
      v.l[q] = fl[q * ms];
    }
  }
}

template <class T, int N, int C, int D, bool NEG, bool LIT>
__device__ __forceinline__ void apply_nbr(T* acc, const Nbr<T, N, C, D>& v, const T* tab, T inv_h) {
  constexpr int F = C ^ (4 >> D);
  if constexpr (Ord<N>::n(F) > 0 && Ord<N>::n(C) > 0) {
    auto diff = [&](int q) -> T {
      const T d = NEG ? (v.l[q] - v.r[q]) : (v.r[q] - v.l[q]);
      if constexpr (LIT) return d * inv_h;
      else return d;
    };
    constexpr int off = Ord<N>::off(C, D);
    auto coef = [&](int kk, double lit) -> T {
      if constexpr (LIT) {
        (void)kk;
        return T(lit);
      } else {
        (void)lit;
        return tab[off + kk];
      }
    };
    Adv<N, C, D>::template apply<T>(acc, diff, coef);
  }
}

// advection sum of one cell: DIMS == 0 checks the active axes at run time and loads while it
// accumulates; DIMS != 0 (bit d = axis d active) loads every neighbour first
template <class T, int N, int C, bool NEG, bool LIT, int DIMS, class A>
__device__ __forceinline__ void advection_sum(T* acc, const A& a, T* const* rd, int i, int j, int k) {
  const T* tab = tab_of<LIT, T>(a);
  if constexpr (DIMS == 0) {
    if (a.act[0]) stencil_axis<T, N, C, 0, NEG, LIT>(acc, rd, a.g, i, j, k, tab, invh_of<LIT, T>(a, 0));
    if (a.act[1]) stencil_axis<T, N, C, 1, NEG, LIT>(acc, rd, a.g, i, j, k, tab, invh_of<LIT, T>(a, 1));
    if (a.act[2]) stencil_axis<T, N, C, 2, NEG, LIT>(acc, rd, a.g, i, j, k, tab, invh_of<LIT, T>(a, 2));
  } else {
    Nbr<T, N, C, 0> vx;
    Nbr<T, N, C, 1> vy;
    Nbr<T, N, C, 2> vz;
    if constexpr ((DIMS & 1) != 0) load_nbr<T, N, C, 0>(vx, rd, a.g, i, j, k);
    if constexpr ((DIMS & 2) != 0) load_nbr<T, N, C, 1>(vy, rd, a.g, i, j, k);
    if constexpr ((DIMS & 4) != 0) load_nbr<T, N, C, 2>(vz, rd, a.g, i, j, k);
    if constexpr ((DIMS & 1) != 0) apply_nbr<T, N, C, 0, NEG, LIT>(acc, vx, tab, invh_of<LIT, T>(a, 0));
    if constexpr ((DIMS & 2) != 0) apply_nbr<T, N, C, 1, NEG, LIT>(acc, vy, tab, invh_of<LIT, T>(a, 1));
    if constexpr ((DIMS & 4) != 0) apply_nbr<T, N, C, 2, NEG, LIT>(acc, vz, tab, invh_of<LIT, T>(a, 2));
  }
}

// --------------------------------------------------------------------------------------------
// sub-step kernel
// --------------------------------------------------------------------------------------------
template <class T, int N, int C, bool ADJ, bool LIT, class A, int DIMS = 0>
__device__ __forceinline__ void substep_cell(const A& a, int i, int j, int k, bool face, double* part) {
  constexpr int n = Ord<N>::n(C);
  if constexpr (n == 0) {
    return;
  } else {
    T* const* rd = a.rd;
    if (face && !a.pre_ghosts) ghosts_for_cell<T, N, C>(const_cast<T* const*>(rd), a.g, a.act, a.bmat, a.beam,
                                       a.bc * a.scale_g, !ADJ, i, j, k);
    const Geom& gt = a.g[C];
    const long long p = lin(gt, i, j, k);
    T upre[DIMS != 0 ? n : 1];
    if constexpr (DIMS != 0) {
      const T* uo0 = a.rd[C] + p;
#pragma unroll
      for (int m = 0; m < n; ++m) upre[m] = uo0[m * gt.ms];
    }
    T acc[n];
#pragma unroll
    for (int m = 0; m < n; ++m) acc[m] = T(0);
    advection_sum<T, N, C, ADJ, LIT, DIMS>(acc, a, rd, i, j, k);

    constexpr unsigned mask = Ord<N>::deg_mask(C);
    // per degree: C_l and g_l = dt phi1(-C_l dt / S) / S, so that u' = u + g_l (q - A u - C_l u)
    T Cl[N + 1];
    T gl[N + 1];
    if (a.cache_mode == 2) {
      // the first half sub-step of this energy step left the factors of this cell
      const T* cp = a.cache[C] + p;
#pragma unroll
      for (int l = 0; l <= N; ++l) {
        Cl[l] = ((mask >> l) & 1u) ? cp[l * gt.ms] : T(0);
        gl[l] = ((mask >> l) & 1u) ? cp[(1 + N + l) * gt.ms] : T(0);
      }
    } else {
      const T* rho = a.rho[C] + p;
      T rr[MAXE];
      T S = T(0);
#pragma unroll
      for (int e = 0; e < MAXE; ++e) {
        rr[e] = e < a.ne ? rho[e * gt.ms] : T(0);
        S = fma(rr[e], a.s[e], S);
      }
      const T invS = recip(S);
      const T dts = a.dt * invS;
      cl_sums<T, N, mask>(rr, a.c, a.ne, Cl);
#pragma unroll
      for (int l = 0; l <= N; ++l) gl[l] = ((mask >> l) & 1u) ? dts * phi1(-(Cl[l] * dts)) : T(0);
      if (a.cache_mode == 1) {
        T* cp = a.cache[C] + p;
#pragma unroll
        for (int l = 0; l <= N; ++l)
          if ((mask >> l) & 1u) {
            cp[l * gt.ms] = Cl[l];
            cp[(1 + N + l) * gt.ms] = gl[l];
          }
      }
    }
    const T* uo = a.rd[C] + p;
    T* un = a.wr[C] + p;
    T q0 = T(0);
    if constexpr (ADJ && C == 0) {
      if (a.adjoint_source) {
        const long long ce = eee_cell(gt, i, j, k);
        double q = 0.0;
        if constexpr (A::line_src) {
          // per-line source weights acs noa ibar, formed once per adjoint sweep
          for (int r = 0; r < a.nr; ++r) q = fma(-a.sig_src[r], a.wsrc[ce * a.nr + r], q);
        } else {
          for (int r = 0; r < a.nr; ++r)
            q = q - a.sig_src[r] * a.acs[ce * a.nr + r] * a.noa[ce * a.ne + a.xel[r]] * a.ibar[r];
        }
        q0 = T(q);
      }
    }
#pragma unroll
    for (int m = 0; m < n; ++m) {
      const int l = degree_of<N, C>(m);
      T u;
      if constexpr (DIMS != 0) u = upre[m];
      else u = uo[m * gt.ms];
      const T q = (m == 0) ? q0 : T(0);
      const T num = fma(-Cl[l], u, q - acc[m]);   // (q - A u) - C_l u
      const T unew = fma(num, gl[l], u);
      un[m * gt.ms] = unew;
      if constexpr (C == 0 && !ADJ) {
        if (m == 0 && part != nullptr) {
          const long long ce = eee_cell(gt, i, j, k);
#pragma unroll
          for (int r = 0; r < MAXR; ++r)
            if (r < a.nr) part[r] += a.wint[ce * a.nr + r] * double(unew);
        }
      }
    }
  }
}

template <class T, int N, bool ADJ>
__global__ void __launch_bounds__(PBLOCK, PN_PLAIN_MINB * (BLOCK / PBLOCK)) substep_kernel(const __grid_constant__ SubArgs<T, N> a) {
  int s, i, j, k;
  const bool ok = locate<PBLOCK>(a.seg, a.nseg, blockIdx.x, threadIdx.x, s, i, j, k);
  const int cls = a.seg[s].cls;
  const bool face = a.seg[s].kind == 1;
  double part[MAXR];
#pragma unroll
  for (int r = 0; r < MAXR; ++r) part[r] = 0.0;
  double* pp = (a.partial != nullptr) ? part : nullptr;
  if (ok) {
    switch (cls) {
      case 0: substep_cell<T, N, 0, ADJ, false>(a, i, j, k, face, pp); break;
      case 1: substep_cell<T, N, 1, ADJ, false>(a, i, j, k, face, pp); break;
      case 2: substep_cell<T, N, 2, ADJ, false>(a, i, j, k, face, pp); break;
      case 3: substep_cell<T, N, 3, ADJ, false>(a, i, j, k, face, pp); break;
      case 4: substep_cell<T, N, 4, ADJ, false>(a, i, j, k, face, pp); break;
      case 5: substep_cell<T, N, 5, ADJ, false>(a, i, j, k, face, pp); break;
      case 6: substep_cell<T, N, 6, ADJ, false>(a, i, j, k, face, pp); break;
      default: substep_cell<T, N, 7, ADJ, false>(a, i, j, k, face, pp); break;
    }
  }
  if (a.partial != nullptr) {
    // block sum of the intensity partials, fixed order -> deterministic
    __shared__ double red[PBLOCK / 32][MAXR];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int r = 0; r < MAXR; ++r) {
      if (r < a.nr) {
        double v = part[r];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) red[w][r] = v;
      }
    }
    __syncthreads();
    if (threadIdx.x < a.nr) {
      double v = 0.0;
#pragma unroll
      for (int q = 0; q < PBLOCK / 32; ++q) v += red[q][threadIdx.x];
      a.partial[(long long)blockIdx.x * a.nr + threadIdx.x] = v;
    }
  }
}

// --------------------------------------------------------------------------------------------
// plain sub-step with two threads per cell
// --------------------------------------------------------------------------------------------
// One solve's sub-step launch holds about 14 warps per SM (one thread per target cell), and they
// leave the FP64 pipe idle while they wait for their neighbour values.  This form gives every
// target cell two threads in two different warps: half h updates the moments [M0, M1) of its cell
// (h = 0 the lower degrees, h = 1 the rest, split at the degree boundary nearest to half the
// moments), forms the factors of those degrees only, and loads only the neighbour moments that its
// rows couple to.  Each row receives the same products in the same order as in substep_cell, so
// the results are bit-identical to substep_kernel's.

// first moment of the upper half of class C (n when the class has a single degree: the lower
// half then does all of it, so moment 0, with the intensity partials and the adjoint source, is
// always in the lower half)
template <int N, int C>
__host__ __device__ constexpr int split_moment() {
  const int n = Ord<N>::n(C);
  int best = 0, bd = 1 << 30;
  for (int m = 1; m < n; ++m) {
    if (degree_of<N, C>(m) == degree_of<N, C>(m - 1)) continue;
    const int d = 2 * m > n ? 2 * m - n : n - 2 * m;
    if (d < bd) {
      bd = d;
      best = m;
    }
  }
  return best > 0 ? best : n;
}

// degrees of the moments [M0, M1) of class C
template <int N, int C, int M0, int M1>
__host__ __device__ constexpr unsigned range_deg_mask() {
  unsigned msk = 0u;
  for (int m = M0; m < M1; ++m) msk |= 1u << degree_of<N, C>(m);
  return msk;
}

// Accumulators of rows [M0, M1); the other rows go to a sink that nothing reads, so the compiler
// drops their products, and the differences and loads that only they use.
template <class T, int M0, int M1>
struct RowAcc {
  T v[M1 > M0 ? M1 - M0 : 1];
  T sink;
  __device__ __forceinline__ T& operator[](int m) { return (m >= M0 && m < M1) ? v[m - M0] : sink; }
};

// stencil_axis (table coefficients, runtime active axes) over a row range
template <class T, int N, int C, int D, bool NEG, class Acc>
__device__ __forceinline__ void stencil_axis_rows(Acc& acc, T* const* rd, const Geom* g, int i, int j, int k,
                                                  const T* tab) {
  constexpr int F = C ^ (4 >> D);
  constexpr int nf = Ord<N>::n(F);
  if constexpr (nf == 0 || Ord<N>::n(C) == 0) {
    return;
  } else {
    const Geom& gf = g[F];
    int r3[3] = {i, j, k};
    int l3[3] = {i, j, k};
    if ((C >> (2 - D)) & 1) l3[D] -= 1;
    else r3[D] += 1;
    const T* fr = rd[F] + lin(gf, r3[0], r3[1], r3[2]);
    const T* fl = rd[F] + lin(gf, l3[0], l3[1], l3[2]);
    const long long ms = gf.ms;
    auto diff = [&](int q) -> T {
      const T x = fr[q * ms];
      const T y = fl[q * ms];
      return NEG ? (y - x) : (x - y);
    };
    constexpr int off = Ord<N>::off(C, D);
    auto coef = [&](int kk, double lit) -> T {
      (void)lit;
      return tab[off + kk];
    };
    Adv<N, C, D>::template apply<T>(acc, diff, coef);
  }
}

template <class T, int N, int C, bool ADJ, int H>
__device__ __forceinline__ void substep_cell_half(const SubArgs<T, N>& a, int i, int j, int k, double* part) {
  constexpr int n = Ord<N>::n(C);
  constexpr int MS = split_moment<N, C>();
  constexpr int M0 = H == 0 ? 0 : MS;
  constexpr int M1 = H == 0 ? MS : n;
  if constexpr (n == 0 || M1 <= M0) {
    (void)a; (void)i; (void)j; (void)k; (void)part;
  } else {
    const Geom& gt = a.g[C];
    const long long p = lin(gt, i, j, k);
    RowAcc<T, M0, M1> acc;
#pragma unroll
    for (int m = 0; m < M1 - M0; ++m) acc.v[m] = T(0);
    acc.sink = T(0);
    if (a.act[0]) stencil_axis_rows<T, N, C, 0, ADJ>(acc, a.rd, a.g, i, j, k, a.tab);
    if (a.act[1]) stencil_axis_rows<T, N, C, 1, ADJ>(acc, a.rd, a.g, i, j, k, a.tab);
    if (a.act[2]) stencil_axis_rows<T, N, C, 2, ADJ>(acc, a.rd, a.g, i, j, k, a.tab);

    constexpr unsigned mask = range_deg_mask<N, C, M0, M1>();
    T Cl[N + 1];
    T gl[N + 1];
    if (a.cache_mode == 2) {
      const T* cp = a.cache[C] + p;
#pragma unroll
      for (int l = 0; l <= N; ++l) {
        Cl[l] = ((mask >> l) & 1u) ? cp[l * gt.ms] : T(0);
        gl[l] = ((mask >> l) & 1u) ? cp[(1 + N + l) * gt.ms] : T(0);
      }
    } else {
      const T* rho = a.rho[C] + p;
      T rr[MAXE];
      T S = T(0);
#pragma unroll
      for (int e = 0; e < MAXE; ++e) {
        rr[e] = e < a.ne ? rho[e * gt.ms] : T(0);
        S = fma(rr[e], a.s[e], S);
      }
      const T invS = recip(S);
      const T dts = a.dt * invS;
      cl_sums<T, N, mask>(rr, a.c, a.ne, Cl);
#pragma unroll
      for (int l = 0; l <= N; ++l) gl[l] = ((mask >> l) & 1u) ? dts * phi1(-(Cl[l] * dts)) : T(0);
      if (a.cache_mode == 1) {
        T* cp = a.cache[C] + p;
#pragma unroll
        for (int l = 0; l <= N; ++l)
          if ((mask >> l) & 1u) {
            cp[l * gt.ms] = Cl[l];
            cp[(1 + N + l) * gt.ms] = gl[l];
          }
      }
    }
    const T* uo = a.rd[C] + p;
    T* un = a.wr[C] + p;
    T q0 = T(0);
    if constexpr (ADJ && C == 0 && M0 == 0) {
      if (a.adjoint_source) {
        const long long ce = eee_cell(gt, i, j, k);
        double q = 0.0;
        for (int r = 0; r < a.nr; ++r)
          q = q - a.sig_src[r] * a.acs[ce * a.nr + r] * a.noa[ce * a.ne + a.xel[r]] * a.ibar[r];
        q0 = T(q);
      }
    }
#pragma unroll
    for (int m = M0; m < M1; ++m) {
      const int l = degree_of<N, C>(m);
      const T u = uo[m * gt.ms];
      const T q = (m == 0) ? q0 : T(0);
      const T num = fma(-Cl[l], u, q - acc.v[m - M0]);   // (q - A u) - C_l u
      const T unew = fma(num, gl[l], u);
      un[m * gt.ms] = unew;
      if constexpr (C == 0 && !ADJ && M0 == 0) {
        if (m == 0 && part != nullptr) {
          const long long ce = eee_cell(gt, i, j, k);
#pragma unroll
          for (int r = 0; r < MAXR; ++r)
            if (r < a.nr) part[r] += a.wint[ce * a.nr + r] * double(unew);
        }
      }
    }
  }
}

template <class T, int N, bool ADJ, int H>
__device__ __forceinline__ void substep_half_of(const SubArgs<T, N>& a, int cls, int i, int j, int k, double* part) {
  switch (cls) {
    case 0: substep_cell_half<T, N, 0, ADJ, H>(a, i, j, k, part); break;
    case 1: substep_cell_half<T, N, 1, ADJ, H>(a, i, j, k, part); break;
    case 2: substep_cell_half<T, N, 2, ADJ, H>(a, i, j, k, part); break;
    case 3: substep_cell_half<T, N, 3, ADJ, H>(a, i, j, k, part); break;
    case 4: substep_cell_half<T, N, 4, ADJ, H>(a, i, j, k, part); break;
    case 5: substep_cell_half<T, N, 5, ADJ, H>(a, i, j, k, part); break;
    case 6: substep_cell_half<T, N, 6, ADJ, H>(a, i, j, k, part); break;
    default: substep_cell_half<T, N, 7, ADJ, H>(a, i, j, k, part); break;
  }
}

// resident blocks of 2 x PBLOCK threads per SM the split kernel is compiled for (its register cap)
#ifndef PN_SPLIT_MINB
#define PN_SPLIT_MINB 7
#endif

// Same work segments and partial-sum slots as substep_kernel (PBLOCK cells per block); threads
// [0, PBLOCK) are the lower halves of the block's cells, [PBLOCK, 2 PBLOCK) the upper halves.  The
// face ghosts must have been written by ghost_kernel before the launch.
template <class T, int N, bool ADJ>
__global__ void __launch_bounds__(2 * PBLOCK, PN_SPLIT_MINB) substep_split_kernel(const __grid_constant__ SubArgs<T, N> a) {
  const int h = threadIdx.x >= PBLOCK ? 1 : 0;   // warp-uniform
  const int tid = threadIdx.x - h * PBLOCK;
  int s, i, j, k;
  const bool ok = locate<PBLOCK>(a.seg, a.nseg, blockIdx.x, tid, s, i, j, k);
  const int cls = a.seg[s].cls;
  double part[MAXR];
#pragma unroll
  for (int r = 0; r < MAXR; ++r) part[r] = 0.0;
  double* pp = (a.partial != nullptr) ? part : nullptr;
  if (ok) {
    if (h == 0) substep_half_of<T, N, ADJ, 0>(a, cls, i, j, k, pp);
    else substep_half_of<T, N, ADJ, 1>(a, cls, i, j, k, pp);
  }
  if (a.partial != nullptr) {
    // moment 0 is in the lower half: the lower warps' sums, in substep_kernel's order
    __shared__ double red[PBLOCK / 32][MAXR];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (h == 0) {
#pragma unroll
      for (int r = 0; r < MAXR; ++r) {
        if (r < a.nr) {
          double v = part[r];
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
          if (lane == 0) red[w][r] = v;
        }
      }
    }
    __syncthreads();
    if (threadIdx.x < a.nr) {
      double v = 0.0;
#pragma unroll
      for (int q = 0; q < PBLOCK / 32; ++q) v += red[q][threadIdx.x];
      a.partial[(long long)blockIdx.x * a.nr + threadIdx.x] = v;
    }
  }
}

// --------------------------------------------------------------------------------------------
// adjoint density kernel
// --------------------------------------------------------------------------------------------
template <class T, int N, int C, bool LIT, class A, int DIMS = 0>
__device__ __forceinline__ void integrate_cell(const A& a, int i, int j, int k, bool face) {
  constexpr int n = Ord<N>::n(C);
  if constexpr (n == 0) {
    return;
  } else {
    if (face && !a.pre_ghosts) ghosts_for_cell<T, N, C>(a.u, a.g, a.act, a.bmat, a.beam, a.bc * a.scale_g, true, i, j, k);
    const Geom& gt = a.g[C];
    const long long p = lin(gt, i, j, k);
    T upre[DIMS != 0 ? n : 1];
    T lpre[DIMS != 0 ? n : 1];
    if constexpr (DIMS != 0) {
      const T* u0 = a.u[C] + p;
      const T* l0 = a.lam[C] + p;
#pragma unroll
      for (int m = 0; m < n; ++m) {
        upre[m] = u0[m * gt.ms];
        lpre[m] = l0[m * gt.ms];
      }
    }
    T acc[n];
#pragma unroll
    for (int m = 0; m < n; ++m) acc[m] = T(0);
    advection_sum<T, N, C, false, LIT, DIMS>(acc, a, a.u, i, j, k);
    const T* rho = a.rho[C] + p;
    T rr[MAXE];
    T S = T(0);
#pragma unroll
    for (int e = 0; e < MAXE; ++e) {
      rr[e] = e < a.ne ? rho[e * gt.ms] : T(0);
      S = fma(rr[e], a.s[e], S);
    }
    const T invS = recip(S);
    constexpr unsigned mask = Ord<N>::deg_mask(C);
    T Cl[N + 1];
    cl_sums<T, N, mask>(rr, a.c, a.ne, Cl);
    const T* uu = a.u[C] + p;
    const T* la = a.lam[C] + p;
    // P = sum_m lam_m du_m ; R_l = sum_{m: l(m) = l} lam_m u_m
    T P = T(0);
    T R[N + 1];
#pragma unroll
    for (int l = 0; l <= N; ++l) R[l] = T(0);
#pragma unroll
    for (int m = 0; m < n; ++m) {
      const int l = degree_of<N, C>(m);
      T u, lm;
      if constexpr (DIMS != 0) {
        u = upre[m];
        lm = lpre[m];
      } else {
        u = uu[m * gt.ms];
        lm = la[m * gt.ms];
      }
      // P = sum_m lambda_m du_m with du = (-A u - C_l u) / S: the 1/S applied once, below
      P = fma(lm, fma(-Cl[l], u, -acc[m]), P);
      R[l] = fma(lm, u, R[l]);
    }
    P *= invS;
    double* rb = a.rbar[C] + p;
#pragma unroll
    for (int e = 0; e < MAXE; ++e) {
      if (e < a.ne) {
        // this step's increment in the state's precision, accumulated in FP64
        T v = a.s[e] * P;
#pragma unroll
        for (int l = 0; l <= N; ++l)
          if ((mask >> l) & 1u) v = fma(T(a.c[e][l]), R[l], v);
        rb[e * gt.ms] = fma(double(v), a.wfac, rb[e * gt.ms]);
      }
    }
    if constexpr (C == 0) {
      const long long ce = eee_cell(gt, i, j, k);
      const double u0 = double(uu[0]);
      if constexpr (A::line_sums) {
        // W_r(cell) += coef_r u0; acs_bar and noa_bar are formed from W once, after the sweep
        for (int r = 0; r < a.nr; ++r) a.wsum[ce * a.nr + r] = fma(a.coef[r], u0, a.wsum[ce * a.nr + r]);
      } else {
        for (int r = 0; r < a.nr; ++r) {
          const double cr = a.coef[r] * a.ibar[r];
          const int el = a.xel[r];
          a.acs_bar[ce * a.nr + r] += a.noa[ce * a.ne + el] * u0 * cr;
          a.noa_bar[ce * a.ne + el] += a.acs[ce * a.nr + r] * u0 * cr;
        }
      }
    }
  }
}

// The density integral with two threads per cell (the plain path's form, as
// substep_split_kernel): half h forms du for the moments [M0, M1) of its cell and the sums
// R_l of its degrees.  P = sum_m lambda_m du_m is one FMA chain in moment order: the lower half
// runs it over its moments and hands the partial chain, with its R_l, to the upper half through
// shared memory; the upper half continues the chain over its moments and writes rho_bar.  Every
// sum is formed in integrate_cell's order, so rho_bar is bit-identical to a one-thread-per-cell
// evaluation of integrate_cell.
template <class T, int N>
struct IntXchg {
  T P[PBLOCK];
  T R[N + 1][PBLOCK];
};

template <class T, int N, int C, int H>
__device__ __forceinline__ void integrate_cell_half(const IntArgs<T, N>& a, bool ok, int i, int j, int k, int tid,
                                                    IntXchg<T, N>& x) {
  constexpr int n = Ord<N>::n(C);
  constexpr int MS = split_moment<N, C>();
  constexpr int M0 = H == 0 ? 0 : MS;
  constexpr int M1 = H == 0 ? MS : n;
  constexpr bool alone = MS >= n;   // one degree: the lower half does all of it
  if constexpr (n == 0 || M1 <= M0) {
    __syncthreads();
  } else {
    const Geom& gt = a.g[C];
    const long long p = ok ? lin(gt, i, j, k) : 0;
    constexpr unsigned mask = range_deg_mask<N, C, M0, M1>();
    constexpr unsigned cmask = Ord<N>::deg_mask(C);
    T P = T(0);
    T R[N + 1];
#pragma unroll
    for (int l = 0; l <= N; ++l) R[l] = T(0);
    T tm[M1 - M0], lmv[M1 - M0];
    T invS = T(1);
    if (ok) {
      RowAcc<T, M0, M1> acc;
#pragma unroll
      for (int m = 0; m < M1 - M0; ++m) acc.v[m] = T(0);
      acc.sink = T(0);
      if (a.act[0]) stencil_axis_rows<T, N, C, 0, false>(acc, a.u, a.g, i, j, k, a.tab);
      if (a.act[1]) stencil_axis_rows<T, N, C, 1, false>(acc, a.u, a.g, i, j, k, a.tab);
      if (a.act[2]) stencil_axis_rows<T, N, C, 2, false>(acc, a.u, a.g, i, j, k, a.tab);
      const T* rho = a.rho[C] + p;
      T rr[MAXE];
      T S = T(0);
#pragma unroll
      for (int e = 0; e < MAXE; ++e) {
        rr[e] = e < a.ne ? rho[e * gt.ms] : T(0);
        S = fma(rr[e], a.s[e], S);
      }
      invS = recip(S);
      T Cl[N + 1];
      cl_sums<T, N, mask>(rr, a.c, a.ne, Cl);
      const T* uu = a.u[C] + p;
      const T* la = a.lam[C] + p;
#pragma unroll
      for (int m = M0; m < M1; ++m) {
        const int l = degree_of<N, C>(m);
        const T u = uu[m * gt.ms];
        const T lm = la[m * gt.ms];
        tm[m - M0] = fma(-Cl[l], u, -acc.v[m - M0]);
        lmv[m - M0] = lm;
        R[l] = fma(lm, u, R[l]);
      }
      if constexpr (H == 0) {
#pragma unroll
        for (int m = 0; m < M1; ++m) P = fma(lmv[m], tm[m], P);
        if constexpr (!alone) {
          x.P[tid] = P;
#pragma unroll
          for (int l = 0; l <= N; ++l)
            if ((mask >> l) & 1u) x.R[l][tid] = R[l];
        }
      }
      if constexpr (C == 0 && H == 0) {
        const long long ce = eee_cell(gt, i, j, k);
        const double u0 = double(uu[0]);
        for (int r = 0; r < a.nr; ++r) {
          const double cr = a.coef[r] * a.ibar[r];
          const int el = a.xel[r];
          a.acs_bar[ce * a.nr + r] += a.noa[ce * a.ne + el] * u0 * cr;
          a.noa_bar[ce * a.ne + el] += a.acs[ce * a.nr + r] * u0 * cr;
        }
      }
    }
    __syncthreads();
    // the half that finishes: the upper one, or the lower one of a single-degree class
    if (ok && (H == 1 || alone)) {
      if constexpr (H == 1) {
        P = x.P[tid];
#pragma unroll
        for (int m = M0; m < M1; ++m) P = fma(lmv[m - M0], tm[m - M0], P);
#pragma unroll
        for (int l = 0; l <= N; ++l)
          if (((cmask & ~mask) >> l) & 1u) R[l] = x.R[l][tid];
      }
      P *= invS;
      double* rb = a.rbar[C] + p;
#pragma unroll
      for (int e = 0; e < MAXE; ++e) {
        if (e < a.ne) {
          T v = a.s[e] * P;
#pragma unroll
          for (int l = 0; l <= N; ++l)
            if ((cmask >> l) & 1u) v = fma(T(a.c[e][l]), R[l], v);
          rb[e * gt.ms] = fma(double(v), a.wfac, rb[e * gt.ms]);
        }
      }
    }
  }
}

template <class T, int N, int H>
__device__ __forceinline__ void integrate_half_of(const IntArgs<T, N>& a, int cls, bool ok, int i, int j, int k,
                                                  int tid, IntXchg<T, N>& x) {
  switch (cls) {
    case 0: integrate_cell_half<T, N, 0, H>(a, ok, i, j, k, tid, x); break;
    case 1: integrate_cell_half<T, N, 1, H>(a, ok, i, j, k, tid, x); break;
    case 2: integrate_cell_half<T, N, 2, H>(a, ok, i, j, k, tid, x); break;
    case 3: integrate_cell_half<T, N, 3, H>(a, ok, i, j, k, tid, x); break;
    case 4: integrate_cell_half<T, N, 4, H>(a, ok, i, j, k, tid, x); break;
    case 5: integrate_cell_half<T, N, 5, H>(a, ok, i, j, k, tid, x); break;
    case 6: integrate_cell_half<T, N, 6, H>(a, ok, i, j, k, tid, x); break;
    default: integrate_cell_half<T, N, 7, H>(a, ok, i, j, k, tid, x); break;
  }
}

// PBLOCK cells per block, one class per block (the plain path's segments); the face
// ghosts must have been written by ghost_kernel before the launch.  Every thread reaches the one
// __syncthreads of its class's path.
template <class T, int N>
__global__ void __launch_bounds__(2 * PBLOCK, PN_SPLIT_MINB) integrate_split_kernel(const __grid_constant__ IntArgs<T, N> a) {
  __shared__ IntXchg<T, N> x;
  const int h = threadIdx.x >= PBLOCK ? 1 : 0;   // warp-uniform
  const int tid = threadIdx.x - h * PBLOCK;
  int s, i, j, k;
  const bool ok = locate<PBLOCK>(a.seg, a.nseg, blockIdx.x, tid, s, i, j, k);
  const int cls = a.seg[s].cls;   // block-uniform
  if (h == 0) integrate_half_of<T, N, 0>(a, cls, ok, i, j, k, tid, x);
  else integrate_half_of<T, N, 1>(a, cls, ok, i, j, k, tid, x);
}

}  // namespace pn
